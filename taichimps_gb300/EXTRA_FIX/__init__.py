from .base import Fix
from .damping_cundall import FixDampingCundall
from .deform_pressure import FixDeformPressure
from .nve_sphere import FixNVESphere

__all__ = ["Fix", "FixNVESphere", "FixDampingCundall", "FixDeformPressure"]

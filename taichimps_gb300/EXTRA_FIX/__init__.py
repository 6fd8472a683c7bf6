from .base import Fix
from .damping_cundall import FixDampingCundall
from .deform_pressure import FixDeformPressure
from .nve_sphere import FixNVESphere
from .wall_gran import FixWallGran
from .wall_gran_region import FixWallGranRegion

__all__ = ["Fix", "FixNVESphere", "FixDampingCundall", "FixDeformPressure", "FixWallGran", "FixWallGranRegion"]

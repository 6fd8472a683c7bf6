"""
taichimps_gb300: the per-step granular-DEM contact path of taichimps, native
to GB300 (sm_103a CUDA behind a C ABI), behind the reference's own plug-in
API (pair / fix / neighbor / history / compute classes driven by Simulation).
"""

from .adjoint import AdjointRun, stress_curve
from .atom import AtomSystem
from .computes import ComputeContactAtom, Computes
from .contact_history import ContactHistory
from .domain import Domain
from .ensemble import BatchedEngine
from .EXTRA_FIX import (Fix, FixDampingCundall, FixDeformPressure, FixNVESphere, FixWallGran,
                        FixWallGranRegion)
from .GRANULAR import GranHertz, GranHertzHistory, GranHooke, GranHookeHistory, GranularPair, PairGranular
from .neighbor import NeighborList
from .simulation import Simulation

__all__ = ["AdjointRun", "AtomSystem", "BatchedEngine", "ComputeContactAtom", "Computes", "ContactHistory", "Domain", "Fix", "FixDampingCundall",
           "FixDeformPressure", "FixNVESphere", "FixWallGran", "FixWallGranRegion", "GranHertz", "GranHertzHistory", "GranHooke",
           "GranHookeHistory", "GranularPair", "PairGranular", "NeighborList", "Simulation", "stress_curve"]

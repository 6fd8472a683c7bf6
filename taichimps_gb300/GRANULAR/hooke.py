"""pair_style gran/hooke (src/taichimps/GRANULAR/hooke.py:23-173)."""

from __future__ import annotations

from typing import Any

from .base import GranularPair


class _LegacyGran(GranularPair):
    STYLE = 0

    def __init__(self, domain, kn: float, gamman: float, kt: float, gammat: float, xmu: float,
                 dampflag: int = 1, limit_damping: bool = False, float_type: Any = None) -> None:
        super().__init__(domain, float_type=float_type)
        self.kn = float(kn)
        self.gamman = float(gamman)
        self.kt = float(kt)
        self.dampflag = int(dampflag)
        # LAMMPS: "if (dampflag == 0) gammat = 0.0" -- damping is always meff-scaled
        self.gammat = 0.0 if self.dampflag == 0 else float(gammat)
        self.xmu = float(xmu)
        self.limit_damping = 1 if limit_damping else 0
        p = self.params
        p.style = self.STYLE
        p.kn, p.kt, p.gamman, p.gammat, p.xmu = self.kn, self.kt, self.gamman, self.gammat, self.xmu
        p.limit_damping = self.limit_damping


class GranHooke(_LegacyGran):
    """Hookean normal force + viscous tangential damping capped by Coulomb, no history."""

    STYLE = 0

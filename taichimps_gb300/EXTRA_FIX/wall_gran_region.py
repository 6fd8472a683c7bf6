"""
fix wall/gran/region with a cylinder region: granular contact with the curved
side of a cylinder, from inside or outside.

Mirrors taichimps ``FixWallGranRegion`` (src/taichimps/EXTRA_FIX/wall_gran_region.py:33-290):
hooke or hertz normal (the hertz variants scale the stiffness and both
dampings by the contact radius a = sqrt(delta r_i)), mass-scaled damping,
linear_history_classic tangential with history (``*/history`` styles) or the
history-free dashpot with the Coulomb cap; one surface, one history slot per
atom; ``axis_lo``/``axis_hi`` bound which atoms are considered (they are not
end caps).  Runs on the device (tmps_wall_gran, kind 1).
"""

from __future__ import annotations

from typing import Any

from .. import _lib
from .wall_gran import _WallBase


class FixWallGranRegion(_WallBase):
    def __init__(self, domain, axis: int | str = 2, c1: float = 0.0, c2: float = 0.0, radius: float = 1.0,
                 side="in", axis_lo: float | None = None, axis_hi: float | None = None, fstyle: str = "hooke",
                 kn: float = 1e5, gamman: float = 0.0, kt: float | None = None, gammat: float | None = None,
                 xmu: float = 0.0, dampflag: int = 1, history: bool | None = None, limit_damping: bool = False,
                 max_atoms: int = 100000, float_type: Any = None) -> None:
        super().__init__(domain, float_type)
        if isinstance(axis, str):
            axis = {"x": 0, "y": 1, "z": 2}[axis.lower()]
        self.axis = int(axis)
        if self.axis not in (0, 1, 2):
            raise ValueError("axis must be 0, 1 or 2 (or x, y, z)")
        self.c1 = float(c1)
        self.c2 = float(c2)
        self.radius = float(radius)
        if isinstance(side, str):
            self.side = -1 if side.lower() in ("in", "inside", "-1") else 1
        else:
            self.side = -1 if side < 0 else 1
        self.axis_lo = float(axis_lo) if axis_lo is not None else -1e30
        self.axis_hi = float(axis_hi) if axis_hi is not None else 1e30
        self.has_axis_bounds = 1 if (axis_lo is not None or axis_hi is not None) else 0
        self.fstyle = fstyle.lower()
        self.is_hertz = 1 if "hertz" in self.fstyle else 0
        self.kn = float(kn)
        self.gamman = float(gamman)
        self.kt = float(kt) if kt is not None else (2.0 / 7.0 * self.kn)
        self.dampflag = int(dampflag)
        gammat_val = float(gammat) if gammat is not None else (0.5 * self.gamman)
        self.gammat = 0.0 if self.dampflag == 0 else gammat_val
        self.xmu = float(xmu)
        self.limit_damping = 1 if limit_damping else 0
        self.use_history = 1 if (self.fstyle.endswith("history") if history is None else history) else 0
        self._alloc_history(max_atoms)

    def params(self) -> _lib.WallParams:
        p = _lib.WallParams()
        p.kind, p.axis, p.side = 1, self.axis, self.side
        p.history, p.hertz, p.limit_damping = self.use_history, self.is_hertz, self.limit_damping
        p.shear_axis, p.has_axis_bounds = -1, self.has_axis_bounds
        p.c1, p.c2, p.radius = self.c1, self.c2, self.radius
        p.axis_lo, p.axis_hi = self.axis_lo, self.axis_hi
        p.kn, p.kt, p.gamman, p.gammat, p.xmu = self.kn, self.kt, self.gamman, self.gammat, self.xmu
        return p

    def post_force(self, atom, dt: float) -> None:
        if atom.nlocal == 0:
            return
        self._launch(atom, dt, self.params())

"""
fix wall/gran: granular contact with one flat, axis-aligned wall.

Mirrors taichimps ``FixWallGran`` (src/taichimps/EXTRA_FIX/wall_gran.py:39-242):
hooke normal with mass_velocity damping and linear_history_classic tangential
(``history=True``, the ``hooke/history`` style) or the history-free viscous
dashpot with the Coulomb cap (``history=False``, ``hooke``); the wall may
shear in its plane or wiggle along its normal.  The wall is a partner of zero
radius and infinite mass (radsum = Reff = r_i, meff = m_i, moment arm r_i).
The force runs on the device (tmps_wall_gran); the shear history is one slot
per atom, indexed by insertion order so it follows the atoms through the
neighbor build's re-sort.
"""

from __future__ import annotations

import math
from typing import Any

import torch

from .. import _device, _lib
from .base import Fix


class _WallBase(Fix):
    def _alloc_history(self, max_atoms: int) -> None:
        self.max_atoms = int(max_atoms)
        dev = _device.device()
        self.shear = torch.zeros((3, self.max_atoms), dtype=torch.float64, device=dev)
        self.touch = torch.zeros(self.max_atoms, dtype=torch.int32, device=dev)
        self._n_seen = -1

    def reset_history(self, nlocal: int | None = None) -> None:
        self.shear.zero_()
        self.touch.zero_()

    def _launch(self, atom, dt: float, p: _lib.WallParams) -> None:
        n = atom.nlocal
        if n == 0:
            return
        if n > self.max_atoms:
            raise ValueError(f"{type(self).__name__} was built for max_atoms={self.max_atoms}, the system has {n}")
        if n != self._n_seen:
            # a changed atom count renumbers the insertion order: start the wall history afresh
            if self._n_seen >= 0:
                self.reset_history()
            self._n_seen = n
        with _device.timed("wall"):
            rc = _device.lib().tmps_wall_gran(atom.cstruct(), p, float(dt), 1 if self.history_update else 0,
                                              self.shear.data_ptr(), self.touch.data_ptr(), self.max_atoms,
                                              _device.stream())
        _lib.check(rc, "tmps_wall_gran")


class FixWallGran(_WallBase):
    def __init__(self, domain, wall_axis: int, wall_side: int, wall_coord: float, kn: float, gamman: float,
                 kt: float, gammat: float, xmu: float, dampflag: int = 1, history: bool = True,
                 limit_damping: bool = False, shear_axis: int = -1, shear_vel: float = 0.0,
                 wiggle_amplitude: float = 0.0, wiggle_period: float = 0.0, max_atoms: int = 100000,
                 float_type: Any = None) -> None:
        super().__init__(domain, float_type)
        # the reference's argument checks (wall_gran.py:84-93)
        if wall_axis not in (0, 1, 2):
            raise ValueError("wall_axis must be 0, 1 or 2")
        if wall_side not in (-1, 1):
            raise ValueError("wall_side must be -1 (low) or +1 (high)")
        if shear_axis == wall_axis:
            raise ValueError("shear must act in the plane of the wall, not along its normal")
        if wiggle_amplitude != 0.0 and shear_vel != 0.0:
            raise ValueError("cannot wiggle and shear the same wall, as in LAMMPS")
        if wiggle_amplitude != 0.0 and wiggle_period <= 0.0:
            raise ValueError("wiggle needs a positive period")
        self.wall_axis = int(wall_axis)
        self.wall_side = int(wall_side)
        self.wall_coord = float(wall_coord)
        self.kn = float(kn)
        self.gamman = float(gamman)
        self.kt = float(kt)
        self.dampflag = int(dampflag)
        # LAMMPS: "if (dampflag == 0) gammat = 0.0"
        self.gammat = 0.0 if self.dampflag == 0 else float(gammat)
        self.xmu = float(xmu)
        self.limit_damping = 1 if limit_damping else 0
        self.use_history = 1 if history else 0
        self.shear_axis = int(shear_axis)
        self.shear_vel = float(shear_vel)
        self.wiggle_amplitude = float(wiggle_amplitude)
        self.wiggle_period = float(wiggle_period)
        self.elapsed = 0.0
        self._alloc_history(max_atoms)

    def wall_state(self) -> tuple[float, float]:
        """Wall position and normal velocity this step (FixWallGran.post_force, wall_gran.py:230-239)."""
        coord, vwall_n = self.wall_coord, 0.0
        if self.wiggle_amplitude != 0.0:
            omega_w = 2.0 * math.pi / self.wiggle_period
            arg = omega_w * self.elapsed
            coord += self.wiggle_amplitude * (1.0 - math.cos(arg))
            vwall_n = self.wiggle_amplitude * omega_w * math.sin(arg)
        return coord, vwall_n

    def params(self) -> _lib.WallParams:
        coord, vwall_n = self.wall_state()
        p = _lib.WallParams()
        p.kind, p.axis, p.side = 0, self.wall_axis, self.wall_side
        p.history, p.hertz, p.limit_damping = self.use_history, 0, self.limit_damping
        p.shear_axis, p.has_axis_bounds = self.shear_axis, 0
        p.coord, p.vwall_n, p.vwall_s = coord, vwall_n, self.shear_vel
        p.kn, p.kt, p.gamman, p.gammat, p.xmu = self.kn, self.kt, self.gamman, self.gammat, self.xmu
        return p

    def post_force(self, atom, dt: float) -> None:
        if atom.nlocal == 0:
            return
        self._launch(atom, dt, self.params())
        self.elapsed += dt

    def setup(self, nsteps_total: int = 0, dt: float = 0.0) -> None:
        """Restart the clock the wall motion is referenced to."""
        self.elapsed = 0.0

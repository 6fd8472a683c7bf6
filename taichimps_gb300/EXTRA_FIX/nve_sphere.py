"""
fix nve/sphere: velocity-Verlet translation and rotation, I = 0.4 m r^2.

Mirrors taichimps ``FixNVESphere`` (src/taichimps/EXTRA_FIX/nve_sphere.py:34-114);
no wrap per step -- positions are wrapped at reneighboring only.
"""

from __future__ import annotations

from typing import Any

from .. import _device, _lib
from .base import Fix


class FixNVESphere(Fix):
    def __init__(self, domain, float_type: Any = None) -> None:
        super().__init__(domain, float_type=float_type)

    def initial_integrate(self, atom, dt: float) -> None:
        if atom.nlocal == 0:
            return
        with _device.timed("verlet_initial"):
            rc = _device.lib().tmps_verlet_initial(atom.cstruct(), float(dt), _device.stream())
        _lib.check(rc, "tmps_verlet_initial")

    def final_integrate(self, atom, dt: float) -> None:
        if atom.nlocal == 0:
            return
        with _device.timed("verlet_final"):
            rc = _device.lib().tmps_verlet_final(atom.cstruct(), float(dt), _device.stream())
        _lib.check(rc, "tmps_verlet_final")

"""
fix damping/cundall: sign-based local damping of forces and torques.

Mirrors taichimps ``FixDampingCundall`` (src/taichimps/EXTRA_FIX/damping_cundall.py:17-63).
"""

from __future__ import annotations

from typing import Any

from .. import _device, _lib
from .base import Fix


class FixDampingCundall(Fix):
    def __init__(self, domain=None, gamma_lin: float = 0.3, gamma_ang: float = 0.3, float_type: Any = None) -> None:
        super().__init__(domain, float_type)
        self.gamma_lin = float(gamma_lin)
        self.gamma_ang = float(gamma_ang)

    def post_force(self, atom, dt: float) -> None:
        if atom.nlocal == 0:
            return
        with _device.timed("cundall"):
            rc = _device.lib().tmps_damping_cundall(atom.cstruct(), self.gamma_lin, self.gamma_ang,
                                                    _device.stream())
        _lib.check(rc, "tmps_damping_cundall")

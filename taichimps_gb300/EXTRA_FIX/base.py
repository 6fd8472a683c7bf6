"""
Fix protocol (src/taichimps/EXTRA_FIX/base.py:15-57): the hooks Simulation
calls in LAMMPS Verlet order, plus ``history_update``, ``force_reneighbor``
and ``timestep``.
"""

from __future__ import annotations

from abc import ABC
from typing import Any


class Fix(ABC):
    def __init__(self, domain=None, float_type: Any = None) -> None:
        self.domain = domain
        self.float_type = float_type
        self.history_update = True
        self.force_reneighbor = False
        self.timestep: int = 0

    def setup(self, nsteps_total: int = 0, dt: float = 0.0) -> None:
        """Start of a run (LAMMPS Fix::init)."""

    def initial_integrate(self, atom, dt: float) -> None:
        """Start of a step."""

    def post_force(self, atom, dt: float) -> None:
        """After the pair forces."""

    def final_integrate(self, atom, dt: float) -> None:
        """Second half of the step."""

    def end_of_step(self, atom, dt: float) -> None:
        """End of a step."""

    def check_status(self) -> None:
        """Raise for an error a device kernel of this fix recorded (read at sync points)."""

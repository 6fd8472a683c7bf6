"""pair_style gran/hertz/history (src/taichimps/GRANULAR/hertz_history.py:30-193)."""

from __future__ import annotations

from .hooke import _LegacyGran


class GranHertzHistory(_LegacyGran):
    """Hertzian normal force + polyhertz-scaled tangential history."""

    STYLE = 3
    uses_history = True

"""pair_style gran/hertz (src/taichimps/GRANULAR/hertz.py:18-148)."""

from __future__ import annotations

from .hooke import _LegacyGran


class GranHertz(_LegacyGran):
    """Hertzian normal force (polyhertz = sqrt(reff * delta)) without history."""

    STYLE = 2

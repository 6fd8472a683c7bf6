"""pair_style gran/hooke/history (src/taichimps/GRANULAR/hooke_history.py:71-217)."""

from __future__ import annotations

from .hooke import _LegacyGran


class GranHookeHistory(_LegacyGran):
    """Hookean normal force + incremental shear history with Coulomb rescale."""

    STYLE = 1
    uses_history = True

"""
Granular pair styles on the GB300 contact kernel.

Mirrors taichimps ``GranularPair`` (src/taichimps/GRANULAR/base.py:17-38):
``compute(atom, nlist, history, dt, shearupdate=True)`` adds the contact
forces, torques and the pairwise virial into the atom arrays, and advances the
shear history unless ``shearupdate`` is False (the setup force evaluation).
"""

from __future__ import annotations

from abc import ABC
from typing import Any

from .. import _device, _lib


class GranularPair(ABC):
    """Base class; subclasses fill ``self.params`` (a tmps_pair_params)."""

    uses_history = False

    def __init__(self, domain, float_type: Any = None) -> None:
        self.domain = domain
        self.float_type = float_type
        self.params = _lib.PairParams()

    def compute(self, atom, nlist, history, dt: float, shearupdate: bool = True) -> None:
        """Add this step's contact forces into f / torque / virial (atomic_add semantics)."""
        self._launch(atom, nlist, history, dt, shearupdate, accumulate=True)

    def _launch(self, atom, nlist, history, dt: float, shearupdate: bool, accumulate: bool) -> None:
        if atom.nlocal == 0:
            return
        if not nlist.has_built:
            raise RuntimeError("pair compute needs a built neighbor list")
        if history is None:
            if self.uses_history:
                raise ValueError(f"{type(self).__name__} needs a ContactHistory")
            from ..contact_history import ContactHistory
            history = getattr(nlist, "_private_history", None)
            if history is None:
                history = nlist._private_history = ContactHistory(nlist.max_atoms, nlist.max_neighbors_per_atom)
        if self.params.rolling_id:
            history.enable_rolling()
        nl = history.cstruct(nlist)
        with _device.timed("contact"):
            rc = _device.lib().tmps_contact(atom.cstruct(), nl, self.domain.dbox, self.params, float(dt),
                                            1 if shearupdate else 0, 1 if accumulate else 0, _device.stream())
        _lib.check(rc, "tmps_contact")

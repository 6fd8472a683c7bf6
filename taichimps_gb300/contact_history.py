"""
Tangential contact history, stored per full-list slot.

Mirrors taichimps ``ContactHistory`` (src/taichimps/contact_history.py:24-214).
The reference keeps history per half-list pair and carries it across a
rebuild by saving touching contacts keyed by partner tag and looking them up
again (save_state / restore_state).  Here the history lives beside the full
list -- ``shear[3][slots][n]`` in each row atom's own i->j sense (LAMMPS'
both-sided form) and a 64-bit ``touch`` mask per atom -- and the carry-over
is one kernel (tmps_history_remap) run by ``restore_state`` after the build.

``partner`` / ``shear`` present the reference's per-pair view (half list,
insertion order) for code that reads them.
"""

from __future__ import annotations

from typing import Any

import numpy as np
import torch

from . import _device, _lib
from .neighbor import NBR_INDEX_MASK, _Array


class ContactHistory:
    def __init__(self, max_atoms: int, max_neighbors: int = 64, float_type: Any = None) -> None:
        self.max_atoms = int(max_atoms)
        self.max_neighbors = int(max_neighbors)
        self.float_type = float_type
        self.dev = _device.device()
        self.setup_pending = False
        self._shape = None
        self.touch = self.shear = self._touch_alt = self._shear_alt = None
        self._synced_build = -1     # build_count of the list this history belongs to
        self._saved_build = None    # build_count at save_state()
        self._nlist = None

    def _alloc(self, n: int, slots: int) -> None:
        if self._shape == (n, slots):
            return
        self.touch = torch.zeros(n, dtype=torch.int64, device=self.dev)
        self.shear = torch.zeros((3, slots, n), dtype=torch.float64, device=self.dev)
        self._touch_alt = torch.zeros_like(self.touch)
        self._shear_alt = torch.zeros_like(self.shear)
        self._shape = (n, slots)

    def reset(self) -> None:
        if self.touch is not None:
            self.touch.zero_()
            self.shear.zero_()

    def ensure(self, nlist) -> None:
        """Make the history match `nlist`'s current build (fresh zeros if it does not)."""
        self._nlist = nlist
        self._alloc(nlist._n, nlist.slots)
        if self._synced_build != nlist.build_count:
            self.reset()
            self._synced_build = nlist.build_count

    def cstruct(self, nlist) -> _lib.NList:
        self.ensure(nlist)
        return nlist.cstruct(self.touch, self.shear)

    def save_state(self, atom, nlist) -> None:
        """Mark the current contacts for carry-over across the next build."""
        if atom.nlocal == 0 or self.setup_pending:
            return
        if nlist.has_built and self._synced_build == nlist.build_count and self.touch is not None:
            self._saved_build = nlist.build_count
        else:
            self._saved_build = None

    def restore_state(self, atom, nlist) -> None:
        """Carry the saved contacts onto the freshly built list (contact_history.py:147-154)."""
        if atom.nlocal == 0:
            return
        carried = (self._saved_build is not None and nlist.build_count == self._saved_build + 1
                   and self._shape == (nlist._n, nlist.slots))
        if carried:
            L = _device.lib()
            old = nlist.cstruct(self.touch, self.shear, prev=True)
            new = nlist.cstruct(self._touch_alt, self._shear_alt)
            _lib.check(L.tmps_history_remap(old, new, nlist.order.data_ptr(), _device.stream()),
                       "tmps_history_remap")
            self.touch, self._touch_alt = self._touch_alt, self.touch
            self.shear, self._shear_alt = self._shear_alt, self.shear
            self._synced_build = nlist.build_count
        else:
            self._alloc(nlist._n, nlist.slots)
            self.reset()
            self._synced_build = nlist.build_count
        self._saved_build = None
        self.setup_pending = False

    # ------------------------------------------------------ reference views

    def _pairs(self):
        """Half-list view: per pair (i < j insertion order) partner tag and i->j shear."""
        nl = self._nlist
        atom = nl._atom
        n = atom.nlocal
        nbr, nnb = nl.full_rows()
        uid = atom.uid_host()
        tag = atom.buffers.tag.cpu().numpy()
        touch = self.touch.cpu().numpy().view(np.uint64)
        sh = self.shear.cpu().numpy()
        rows = {}
        for p in range(n):
            for k in range(nnb[p]):
                q = nbr[k, p]
                if uid[q] > uid[p]:
                    on = (int(touch[p]) >> k) & 1
                    rows[(int(uid[p]), int(uid[q]))] = (int(tag[q]) if on else -1,
                                                        sh[:, k, p].copy() if on else np.zeros(3))
        keys = sorted(rows)
        partner = np.array([rows[k][0] for k in keys], dtype=np.int32)
        shear = np.array([rows[k][1] for k in keys], dtype=np.float64).reshape(-1, 3)
        return keys, partner, shear

    @property
    def partner(self):
        return _Array(self._pairs()[1])

    @property
    def shear_pairs(self):
        return _Array(self._pairs()[2])

    def touching_by_atom(self, nlist, nlocal: int) -> list[list[tuple[int, np.ndarray]]]:
        """Touching contacts of each atom as (partner tag, shear), both sides (restart form)."""
        self.ensure(nlist)
        atom = nlist._atom
        nbr, nnb = nlist.full_rows()
        uid = atom.uid_host()
        tag = atom.buffers.tag.cpu().numpy()
        touch = self.touch.cpu().numpy().view(np.uint64)
        sh = self.shear.cpu().numpy()
        out: list[list[tuple[int, np.ndarray]]] = [[] for _ in range(nlocal)]
        for p in range(atom.nlocal):
            for k in range(nnb[p]):
                if (int(touch[p]) >> k) & 1 and uid[p] < nlocal:
                    out[uid[p]].append((int(tag[nbr[k, p] & NBR_INDEX_MASK]), sh[:, k, p].copy()))
        return out

    def contacts_by_tag(self, nlist) -> dict[tuple[int, int], np.ndarray]:
        """{(tag_i, tag_j): shear in the i->j sense} for every touching slot (both sides)."""
        out = {}
        for i_rows in [self.touching_by_atom(nlist, nlist._atom.nlocal)]:
            tags = nlist._atom.tag.to_numpy()
            for u, row in enumerate(i_rows):
                for t, s in row:
                    out[(int(tags[u]), t)] = s
        return out

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
        # rolling displacement per slot (contact_history.py:58-59), kept only for a rolling model
        self.rolling_enabled = False
        self.rolling = self._rolling_alt = None
        self._synced_build = -1     # build_count of the list this history belongs to
        self._saved_build = None    # build_count at save_state()
        self._nlist = None
        self._restart = None        # records from load_restart, applied at the next build

    def _alloc(self, n: int, slots: int) -> bool:
        """Arrays for n atoms x slots; True when they were just allocated (touch masks zero).

        A slot's shear (and rolling) entry means something only while its touch bit is set: every
        kernel and view reads it under that bit, and a contact that starts begins from zero whatever
        the entry holds.  So only the touch masks are zeroed; the carry-over targets of a rebuild
        (the *_alt arrays) are allocated at the first rebuild that carries history."""
        if self._shape == (n, slots):
            return False
        self.touch = torch.zeros(n, dtype=torch.int64, device=self.dev)
        self.shear = torch.empty((3, slots, n), dtype=torch.float64, device=self.dev)
        self._touch_alt = self._shear_alt = self._rolling_alt = None
        self.rolling = torch.empty_like(self.shear) if self.rolling_enabled else None
        self._shape = (n, slots)
        return True

    def _carry_targets(self, n: int, slots: int) -> None:
        """The arrays a rebuild's carry-over writes (touch masks and every entry below the new row
        lengths are written by it)."""
        if self._shear_alt is None or tuple(self._shear_alt.shape) != (3, slots, n):
            self._touch_alt = torch.empty(n, dtype=torch.int64, device=self.dev)
            self._shear_alt = torch.empty((3, slots, n), dtype=torch.float64, device=self.dev)
            self._rolling_alt = None
        if self.rolling is not None and self._rolling_alt is None:
            self._rolling_alt = torch.empty_like(self._shear_alt)

    def enable_rolling(self) -> None:
        """Keep a rolling displacement beside the shear (a pair with a rolling model asks for it)."""
        if not self.rolling_enabled:
            self.rolling_enabled = True
            if self.shear is not None:
                # contacts may be touching already: their rolling displacement starts at zero
                self.rolling = torch.zeros_like(self.shear)
                self._rolling_alt = None

    def reset(self) -> None:
        """No touching contacts (the entries behind clear touch bits are not read)."""
        if self.touch is not None:
            self.touch.zero_()

    def ensure(self, nlist) -> None:
        """Make the history match `nlist`'s current build (fresh zeros if it does not)."""
        self._nlist = nlist
        self._alloc(nlist._n, nlist.slots)
        if self._synced_build != nlist.build_count:
            self.reset()
            self._synced_build = nlist.build_count

    def cstruct(self, nlist) -> _lib.NList:
        self.ensure(nlist)
        return nlist.cstruct(self.touch, self.shear, rolling=self.rolling)

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
        if self._restart is not None:
            self._apply_restart(atom, nlist)
            self._saved_build = None
            self.setup_pending = False
            return
        carried = (self._saved_build is not None and nlist.build_count == self._saved_build + 1
                   and self._shape == (nlist._n, nlist.prev_slots))
        if carried:
            L = _device.lib()
            # targets for the carry (new-sized when the list changed its slot count, slots="auto")
            self._carry_targets(nlist._n, nlist.slots)
            old = nlist.cstruct(self.touch, self.shear, prev=True, rolling=self.rolling)
            new = nlist.cstruct(self._touch_alt, self._shear_alt, rolling=self._rolling_alt)
            _lib.check(L.tmps_history_remap(old, new, nlist.order.data_ptr(), _device.stream()),
                       "tmps_history_remap")
            self.touch, self._touch_alt = self._touch_alt, self.touch
            self.shear, self._shear_alt = self._shear_alt, self.shear
            if self.rolling is not None:
                self.rolling, self._rolling_alt = self._rolling_alt, self.rolling
            if nlist.slots != nlist.prev_slots:
                self._shear_alt = self._touch_alt = self._rolling_alt = None
                self._shape = (nlist._n, nlist.slots)
            self._synced_build = nlist.build_count
        else:
            if not self._alloc(nlist._n, nlist.slots):  # fresh arrays are zeros already
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

    def _touching_slots(self, nlist):
        """Every touching slot as arrays (row p, slot k, partner q) in internal order, with uid, tag
        and the shear array on the host."""
        self.ensure(nlist)
        atom = nlist._atom
        nbr, nnb = nlist.full_rows()
        uid = atom.uid_host()
        tag = atom.buffers.tag.cpu().numpy()
        touch = self.touch.cpu().numpy().view(np.uint64)
        sh = self.shear.cpu().numpy()
        S = nbr.shape[0]
        bits = (touch[None, :] >> np.arange(S, dtype=np.uint64)[:, None]) & np.uint64(1)
        live = (bits == 1) & (np.arange(S)[:, None] < nnb[None, :])
        kk, pp = np.nonzero(live)
        order = np.lexsort((kk, uid[pp]))  # by row atom (insertion order), then slot
        kk, pp = kk[order], pp[order]
        qq = nbr[kk, pp]
        return pp, kk, qq, uid, tag, sh

    def touching_by_atom(self, nlist, nlocal: int) -> list[list[tuple[int, np.ndarray]]]:
        """The touching contacts of each local atom as (partner tag, shear), one entry per contact,
        under its lower-index atom in that atom's i->j sense (contact_history.py:155-174): what the
        reference's half list holds, for write_restart to expand into LAMMPS' both-sided records."""
        pp, kk, qq, uid, tag, sh = self._touching_slots(nlist)
        out: list[list[tuple[int, np.ndarray]]] = [[] for _ in range(nlocal)]
        for p, k, q in zip(pp, kk, qq):
            if uid[p] < uid[q] and uid[p] < nlocal:
                out[uid[p]].append((int(tag[q]), sh[:, k, p].copy()))
        return out

    def both_sided_contacts(self, nlist):
        """Every touching contact under both of its atoms, as flat arrays (row atom's insertion index,
        partner tag, values): values are the shear in the row atom's i->j sense, followed by the
        rolling displacement when a rolling model keeps one (3 or 6 per contact).  Rows ascend, each
        row's contacts in slot order -- FixNeighHistory's per-atom records, for write_restart."""
        pp, kk, qq, uid, tag, sh = self._touching_slots(nlist)
        vals = sh[:, kk, pp].T
        if self.rolling is not None:
            vals = np.concatenate([vals, self.rolling.cpu().numpy()[:, kk, pp].T], axis=1)
        return uid[pp].astype(np.int64), tag[qq].astype(np.int32), np.ascontiguousarray(vals)

    def contacts_by_tag(self, nlist) -> dict[tuple[int, int], np.ndarray]:
        """{(tag_i, tag_j): shear in the i->j sense} for every touching slot (both sides)."""
        pp, kk, qq, uid, tag, sh = self._touching_slots(nlist)
        return {(int(tag[p]), int(tag[q])): sh[:, k, p].copy() for p, k, q in zip(pp, kk, qq)}

    def load_restart(self, partner_tags: list, values: list) -> None:
        """Seed the history from a restart file, keyed by partner tag (contact_history.py:176-214,
        the counterpart of FixNeighHistory::unpack_restart).  Entry i belongs to the i-th atom handed
        to AtomSystem.add_particles; each record is in that atom's i->j sense (LAMMPS stores every
        contact under both partners, the second copy negated).  The first neighbor build of the run
        puts the values onto the list: a contact is restored from its lower-index atom's record, as
        the reference's half list does, and its other copy is set to the exact negative."""
        n = min(len(partner_tags), self.max_atoms)
        us, ts, vs = [], [], []
        width = 3
        for i in range(n):
            t = np.asarray(partner_tags[i], dtype=np.int64).reshape(-1)
            m = len(t)
            v = np.asarray(values[i], dtype=np.float64).reshape(m, -1) if m else np.zeros((0, 3))
            width = max(width, v.shape[1])
            us.append(np.full(m, i, dtype=np.int64))
            ts.append(t)
            vs.append(v)
        width = 6 if width >= 6 else 3
        vs = [np.pad(v[:, :width], ((0, 0), (0, max(0, width - v.shape[1])))) for v in vs]
        cat = lambda a, shape: np.concatenate(a) if a else np.zeros(shape)
        self.load_restart_arrays(cat(us, 0), cat(ts, 0), cat(vs, (0, width)))

    def load_restart_arrays(self, rows, partner_tags, values) -> None:
        """load_restart from flat arrays, one entry per stored contact: the atom's position in the
        add_particles order, the partner's tag and the values (shear, then the rolling displacement when
        there are six).  RestartData.neigh_history() gives these arrays for a whole file at once."""
        rows = np.asarray(rows, dtype=np.int64).reshape(-1)
        tags = np.asarray(partner_tags, dtype=np.int64).reshape(-1)
        vals = np.asarray(values, dtype=np.float64).reshape(len(rows), -1) if len(rows) else np.zeros((0, 3))
        keep = rows < self.max_atoms
        rows, tags, vals = rows[keep], tags[keep], vals[keep]
        if len(rows):
            per = np.bincount(rows)
            if per.max() > self.max_neighbors:
                i = int(np.argmax(per))
                raise ValueError(f"atom {i} has {int(per[i])} stored contacts but the history only "
                                 f"has {self.max_neighbors} slots per atom")
        if vals.shape[1] >= 6:
            self.enable_rolling()  # the records carry a rolling displacement: keep it
        self._restart = (rows, tags, vals)
        self.setup_pending = True

    def _apply_restart(self, atom, nlist) -> None:
        """Put loaded restart records onto the freshly built list (see load_restart)."""
        u_file, t_file, v_file = self._restart
        self._restart = None
        self._alloc(nlist._n, nlist.slots)
        self.reset()
        self._synced_build = nlist.build_count
        if len(u_file) == 0 or atom.nlocal == 0:
            return
        nbr, nnb = nlist.full_rows()
        uid = atom.uid_host()
        tag = atom.buffers.tag.cpu().numpy().astype(np.int64)
        S, n = nbr.shape
        kk, pp = np.nonzero(np.arange(S)[:, None] < nnb[None, :])
        qq = nbr[kk, pp]
        own = uid[pp] < uid[qq]
        ko, po, qo = kk[own], pp[own], qq[own]
        # look each owned slot up in the file: key (insertion index, partner tag)
        fkey = (u_file << 32) | t_file
        order = np.argsort(fkey, kind="stable")
        fkey_s = fkey[order]
        skey = (uid[po].astype(np.int64) << 32) | tag[qo]
        at = np.searchsorted(fkey_s, skey)
        hit = (at < len(fkey_s)) & (fkey_s[np.minimum(at, len(fkey_s) - 1)] == skey)
        ko, po, qo, val = ko[hit], po[hit], qo[hit], v_file[order[at[hit]]]
        # the other copy: row q's slot whose partner is p (slots keyed by row * n + partner)
        mkey_all = pp.astype(np.int64) * n + qq
        morder = np.argsort(mkey_all, kind="stable")
        mk = np.searchsorted(mkey_all[morder], qo.astype(np.int64) * n + po)
        km = kk[morder[mk]]
        touch = np.zeros(n, dtype=np.uint64)
        sh = np.zeros((3, S, n))
        np.bitwise_or.at(touch, po, np.left_shift(np.uint64(1), ko.astype(np.uint64)))
        np.bitwise_or.at(touch, qo, np.left_shift(np.uint64(1), km.astype(np.uint64)))
        sh[:, ko, po] = val[:, :3].T
        sh[:, km, qo] = -val[:, :3].T
        self.touch.copy_(torch.from_numpy(touch.view(np.int64)))
        self.shear.copy_(torch.from_numpy(sh))
        if self.rolling is not None and val.shape[1] >= 6:
            rl = np.zeros((3, S, n))
            rl[:, ko, po] = val[:, 3:6].T
            rl[:, km, qo] = -val[:, 3:6].T
            self.rolling.copy_(torch.from_numpy(rl))

"""
Cell-list neighbor list with the skin-displacement rebuild trigger.

Mirrors taichimps ``NeighborList`` (src/taichimps/neighbor.py:16-435).  The
host keeps the reference's decision logic (delay / every / check, decide())
and grid setup (setup_grid, the same float arithmetic); the device does the
binning, the Morton re-sort and the list itself (tmps_nlist_build).

The list is a *full* list (both i->j and j->i), slot-major, so the contact
kernel can run one thread per atom with no atomics.  For code written against
the reference, ``num_neighbors`` / ``neighbors`` / ``npairs`` / ``pair_i`` /
``pair_j`` present the equivalent half list (j > i in insertion order).
"""

from __future__ import annotations

import math
from functools import lru_cache
from typing import Any

import numpy as np
import torch

from . import _device, _lib

NBR_INDEX_MASK = (1 << 27) - 1
MAX_SLOTS = 64


class _Scalar:
    """A 0-d value read as ``x[None]``, like a Taichi scalar field."""

    def __init__(self, get):
        self._get = get

    def __getitem__(self, key):
        return self._get()

    def __int__(self):
        return int(self._get())

    def __index__(self):
        return int(self._get())

    def __eq__(self, other):
        return int(self._get()) == other


@lru_cache(maxsize=16)
def morton_rank(gx: int, gy: int, gz: int) -> np.ndarray:
    """Rank of every linear cell id (cx + cy gx + cz gx gy) along a Morton curve."""
    cx, cy, cz = np.meshgrid(np.arange(gx), np.arange(gy), np.arange(gz), indexing="ij")
    cx, cy, cz = (a.transpose(2, 1, 0).ravel().astype(np.uint64) for a in (cx, cy, cz))

    def spread(v):
        out = np.zeros_like(v)
        for bit in range(21):
            out |= ((v >> np.uint64(bit)) & np.uint64(1)) << np.uint64(3 * bit)
        return out

    code = spread(cx) | (spread(cy) << np.uint64(1)) | (spread(cz) << np.uint64(2))
    order = np.argsort(code, kind="stable")
    rank = np.empty(len(order), dtype=np.int32)
    rank[order] = np.arange(len(order), dtype=np.int32)
    return rank


@lru_cache(maxsize=8)
def _rank_on_device(gx: int, gy: int, gz: int, dev_index: int) -> torch.Tensor:
    """morton_rank on the device, shared by every list with this grid (read only)."""
    return torch.from_numpy(morton_rank(gx, gy, gz)).to(torch.device("cuda", dev_index))


def setup_grid_dims(prd, periodicity, max_cutoff: float, skin: float, max_cells: int):
    """
    NeighborList.setup_grid (neighbor.py:143-189) for an orthogonal box, with the
    perpendicular widths of neighbor.py:122-141 computed as the reference does
    (vol / |b x c| ...), so the grid -- and therefore every cell assignment --
    is the reference's.
    """
    cut = max_cutoff + skin
    if cut <= 0:
        cut = 1.0
    xprd, yprd, zprd = (float(v) for v in prd)
    vol = xprd * yprd * zprd
    # |b x c| of the orthogonal edge vectors as numpy forms it: the cross product's one nonzero
    # component (y z - 0 0 = y z) and norm sqrt(dot) -- the same IEEE operations in plain floats
    widths = [vol / math.sqrt((yprd * zprd) * (yprd * zprd)), vol / math.sqrt((zprd * xprd) * (zprd * xprd)),
              vol / math.sqrt((xprd * yprd) * (xprd * yprd))]
    g = [max(1, int(math.floor(w / cut))) for w in widths]
    for k in range(3):
        if periodicity[k] == 1 and g[k] == 2:
            g[k] = 1
    total = g[0] * g[1] * g[2]
    if total > max_cells:
        factor = (max_cells / total) ** (1.0 / 3.0)
        g = [max(1, int(v * factor)) for v in g]
    csize = [1.0 / g[0], 1.0 / g[1], 1.0 / g[2]]
    return np.array(g, dtype=np.int32), np.array(csize, dtype=np.float64)


class NeighborList:
    def __init__(self, domain, skin: float = 0.001, max_atoms: int = 100000,
                 max_neighbors_per_atom: int = 64, max_neighbors: int | None = None,
                 float_type: Any = None, slots: int | str | None = None) -> None:
        self.domain = domain
        self.skin = float(skin)
        self.max_atoms = int(max_atoms)
        self.max_neighbors_per_atom = int(max_neighbors if max_neighbors is not None else max_neighbors_per_atom)
        self.float_type = float_type
        # Full-list slots per atom.  A full row holds both halves of the
        # reference's half list, so twice its cap, at most one 64-bit touch mask.
        # slots="auto": sized from the longest row of each build (shrunk to
        # 1.25x it plus a margin, grown and rebuilt when a row overflows)
        # instead of a fixed cap; the history follows every change.
        self.auto_slots = slots == "auto"
        if self.auto_slots:
            self.slots = MAX_SLOTS
        else:
            self.slots = int(slots) if slots is not None else min(MAX_SLOTS, 2 * self.max_neighbors_per_atom)
        if not 1 <= self.slots <= MAX_SLOTS:
            raise ValueError(f"slots must be in [1, {MAX_SLOTS}]")
        self.prev_slots = self.slots
        self.max_grid_cells = 200000
        self.delay, self.every, self.check = 0, 1, True
        self.last_build_step = -1
        self.current_step = 0
        self.has_built = False
        self.build_count = 0
        self._check_stamp = 0
        self.grid_dim = np.ones(3, dtype=np.int32)
        self.cell_size = np.ones(3, dtype=np.float64)
        self.dev = _device.device()
        self._n = -1
        self._atom = None
        self.status = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self._status_pending = False
        self.flag = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self._ws = torch.zeros(0, dtype=torch.uint8, device=self.dev)
        self.nbr = self.nnb = self.prev_nbr = self.prev_nnb = None
        self.order = self.cell_of = None
        self._rank_t = None
        self._rank_key = None

    # ------------------------------------------------------------ grid

    def perpendicular_widths(self) -> list[float]:
        xprd, yprd, zprd = (float(v) for v in self.domain.prd)
        a, b, c = np.array([xprd, 0.0, 0.0]), np.array([0.0, yprd, 0.0]), np.array([0.0, 0.0, zprd])
        vol = xprd * yprd * zprd
        return [vol / np.linalg.norm(np.cross(b, c)), vol / np.linalg.norm(np.cross(c, a)),
                vol / np.linalg.norm(np.cross(a, b))]

    def setup_grid(self, max_cutoff: float) -> None:
        g, cs = setup_grid_dims(self.domain.prd, self.domain.periodicity, max_cutoff, self.skin,
                                self.max_grid_cells)
        self.grid_dim, self.cell_size = g, cs
        self.domain.set_grid(g, cs)

    # ---------------------------------------------------------- storage

    @staticmethod
    def fit_slots(longest: int) -> int:
        """Slots for a build whose longest row has `longest` entries: 1.25x plus a margin of 4, a
        multiple of 4, within [8, 64]."""
        want = int(math.ceil(1.25 * longest)) + 4
        return max(8, min(MAX_SLOTS, (want + 3) // 4 * 4))

    def _alloc(self, n: int) -> None:
        if n == self._n:
            return
        S = self.slots
        i32 = dict(dtype=torch.int32, device=self.dev)
        # a row's entries past its length are never read (every reader stops at nnb), so the lists
        # are left unset; the lengths start at zero (an empty previous list for the first carry-over)
        self.nbr = torch.empty((S, n), **i32)
        self.nnb = torch.zeros(n, **i32)
        self.prev_nbr = torch.empty((S, n), **i32)
        self.prev_nnb = torch.zeros(n, **i32)
        self.order = torch.empty(n, **i32)
        self.cell_of = torch.empty(n, **i32)
        self._n = n

    def cstruct(self, touch: torch.Tensor | None, shear: torch.Tensor | None, prev: bool = False,
                rolling: torch.Tensor | None = None) -> _lib.NList:
        s = _lib.NList()
        s.n = self._n
        s.slots = self.prev_slots if prev else self.slots
        s.nbr = (self.prev_nbr if prev else self.nbr).data_ptr()
        s.nnb = (self.prev_nnb if prev else self.nnb).data_ptr()
        s.touch = touch.data_ptr() if touch is not None else None
        s.shear = shear.data_ptr() if shear is not None else None
        s.rolling = rolling.data_ptr() if rolling is not None else None
        return s

    # ------------------------------------------------------------ build

    def build(self, atom, defer_check: bool = False) -> None:
        """NeighborList.build (neighbor.py:414-435): bin, re-sort, list; raise on overflow.
        `defer_check` (a fixed slot count only): return without waiting for the device; the build's
        status (a row past the slot count, a non-finite position) is read and raised by
        check_status() at the caller's next synchronisation.  A row that overflows keeps its first
        `slots` entries, so nothing in between reads past the list."""
        if atom.nlocal == 0:
            return
        self.check_status()  # an earlier deferred build's status first (this one clears the word)
        L = _device.lib()
        self.domain.pull()
        self.setup_grid(2.0 * atom.max_radius)
        n = atom.nlocal
        self._alloc(n)
        key = tuple(int(v) for v in self.grid_dim)
        if key != self._rank_key:
            self._rank_t = _rank_on_device(*key, self.dev.index)
            self._rank_key = key
        ncell = int(np.prod(self.grid_dim))
        wsb = int(L.tmps_nlist_workspace_bytes(n, ncell))
        if self._ws.numel() < wsb:
            self._ws = torch.empty(wsb, dtype=torch.uint8, device=self.dev)  # the build clears what it counts in
        # the list built last time becomes `prev`, for the history carry-over
        self.nbr, self.prev_nbr = self.prev_nbr, self.nbr
        self.nnb, self.prev_nnb = self.prev_nnb, self.nnb
        self.prev_slots = self.slots
        while True:
            if self.nbr.shape[0] < self.slots:
                self.nbr = torch.empty((self.slots, n), dtype=torch.int32, device=self.dev)
            self.status.zero_()
            nl = self.cstruct(None, None)
            src, dst = atom.cstruct(atom.buffers), atom.cstruct(atom.alt_buffers)
            rc = L.tmps_nlist_build(src, dst, self.domain.dbox, ncell, self.skin, self._rank_t.data_ptr(),
                                    self.order.data_ptr(), self.cell_of.data_ptr(), nl, self._ws.data_ptr(),
                                    wsb, self.status.data_ptr(), _device.stream())
            _lib.check(rc, "tmps_nlist_build")
            if defer_check and not self.auto_slots:
                self._status_pending = True
                status = 0
                break
            status = int(self.status.item())
            if not (status & _lib.STATUS_NLIST_OVERFLOW and self.auto_slots and self.slots < MAX_SLOTS):
                break
            # a row overflowed: grow and rebuild from the same (untouched) source buffers
            self.slots = MAX_SLOTS
        atom.swap_buffers()
        self._atom = atom
        if not self._status_pending:
            if status & _lib.STATUS_NONFINITE:
                raise RuntimeError("Neighbor build found a non-finite particle position")
            if self.auto_slots and not status & _lib.STATUS_NLIST_OVERFLOW:
                fit = self.fit_slots(int(self.nnb.max().item()))
                if fit < self.slots:
                    self.nbr = self.nbr[:fit].clone()
                    self.slots = fit
            self._raise_for(status)
        self.has_built = True
        self.build_count += 1
        self.last_build_step = self.current_step

    def _raise_for(self, status: int) -> None:
        if status & _lib.STATUS_NONFINITE:
            raise RuntimeError("Neighbor build found a non-finite particle position")
        if status & _lib.STATUS_NLIST_OVERFLOW:
            raise RuntimeError(
                "Neighbor list overflow: more than "
                f"{self.max_neighbors_per_atom} neighbors for at least one particle. "
                "Increase max_neighbors_per_atom, or reduce the neighbor skin.")

    @property
    def status_pending(self) -> bool:
        """Whether a deferred build's status is still to be read."""
        return self._status_pending

    def check_status(self, status: int | None = None) -> None:
        """Raise for a deferred build's overflow or non-finite position: reads the status word
        (synchronises), or takes `status`, the word as the caller read it with other values."""
        if not self._status_pending:
            return
        self._status_pending = False
        self._raise_for(int(self.status.item()) if status is None else int(status))

    def check_displacement(self, atom, trigger_sq: float, stamp: int) -> None:
        L = _device.lib()
        with _device.timed("skin_check"):
            rc = L.tmps_skin_check(atom.cstruct(), float(trigger_sq), int(stamp), self.flag.data_ptr(),
                                   _device.stream())
        _lib.check(rc, "tmps_skin_check")

    def decide(self, atom, timestep: int | None = None) -> bool:
        """NeighborList.decide (neighbor.py:371-403), same rules and order."""
        if not self.has_built:
            return True
        self.check_status()
        if timestep is not None:
            self.current_step = timestep
        else:
            self.current_step += 1
        since = self.current_step - self.last_build_step
        if since < self.delay:
            return False
        if since % self.every != 0:
            return False
        if not self.check:
            return True
        if atom.nlocal == 0:
            return False
        self._check_stamp += 1
        self.check_displacement(atom, 0.25 * self.skin * self.skin, self._check_stamp)
        return int(self.flag.item()) == self._check_stamp

    def check_and_build(self, atom, timestep: int | None = None) -> bool:
        if self.decide(atom, timestep):
            self.build(atom)
            return True
        return False

    # ------------------------------------------------- reference views

    def full_rows(self):
        """(nbr[S, n] partner internal index, nnb[n]) on the host; entries past a row's length
        read as 0."""
        nbr, nnb = self.nbr.cpu().numpy() & NBR_INDEX_MASK, self.nnb.cpu().numpy()
        nbr[np.arange(nbr.shape[0])[:, None] >= nnb[None, :]] = 0
        return nbr, nnb

    def _half(self):
        atom = self._atom
        n = atom.nlocal
        nbr, nnb = self.full_rows()
        uid = atom.uid_host()
        rows = [[] for _ in range(n)]
        for p in range(n):
            up = uid[p]
            for k in range(nnb[p]):
                uq = uid[nbr[k, p]]
                if uq > up:
                    rows[up].append(int(uq))
        for r in rows:
            r.sort()
        return rows

    @property
    def num_neighbors(self):
        m = self.max_atoms
        out = np.zeros(m, dtype=np.int32)
        if self.has_built:
            for i, r in enumerate(self._half()):
                out[i] = len(r)
        return _Array(out)

    @property
    def neighbors(self):
        out = np.zeros((self.max_atoms, self.max_neighbors_per_atom), dtype=np.int32)
        if self.has_built:
            for i, r in enumerate(self._half()):
                out[i, :len(r)] = r[: self.max_neighbors_per_atom]
        return _Array(out)

    def _pairs(self):
        rows = self._half() if self.has_built else []
        pi = [i for i, r in enumerate(rows) for _ in r]
        pj = [j for r in rows for j in r]
        return np.array(pi, dtype=np.int32), np.array(pj, dtype=np.int32)

    @property
    def npairs(self):
        return _Scalar(lambda: len(self._pairs()[0]))

    @property
    def pair_i(self):
        return _Array(self._pairs()[0])

    @property
    def pair_j(self):
        return _Array(self._pairs()[1])

    def pair_set_tags(self) -> set[tuple[int, int]]:
        """The list as a set of (tag_lo, tag_hi) pairs (each contact once)."""
        atom = self._atom
        nbr, nnb = self.full_rows()
        tag = atom.buffers.tag.cpu().numpy()
        out = set()
        for p in range(atom.nlocal):
            for k in range(nnb[p]):
                a, b = int(tag[p]), int(tag[nbr[k, p]])
                out.add((min(a, b), max(a, b)))
        return out


class _Array(np.ndarray):
    """numpy array with a ``to_numpy()`` method, for reference-style reads."""

    def __new__(cls, a):
        return np.asarray(a).view(cls)

    def to_numpy(self):
        return np.asarray(self)

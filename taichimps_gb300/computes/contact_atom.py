"""
ComputeContactAtom: per-atom contact count (coordination number), LAMMPS
compute contact/atom.

Mirrors taichimps ``ComputeContactAtom`` (src/taichimps/computes/contact_atom.py:15-63):
the same constructor and ``compute(atom, domain, neighbor)`` returning the
counts of the local atoms in insertion order.  The count runs on the GPU over
the full neighbor list (tmps_contact_count); ``reduce`` gives what
``compute reduce`` takes of it (sum, average, min, max).
"""

from __future__ import annotations

import numpy as np
import torch

from .. import _device, _lib


class ComputeContactAtom:
    def __init__(self, max_atoms: int = 2000000) -> None:
        self.max_atoms = int(max_atoms)
        self._count = torch.zeros(0, dtype=torch.int32, device=_device.device())

    def compute(self, atom, domain, neighbor) -> np.ndarray:
        n = atom.nlocal
        if n == 0:
            return np.zeros(0, dtype=np.int32)
        if not neighbor.has_built:
            neighbor.build(atom)
        if self._count.numel() < n:
            self._count = torch.zeros(n, dtype=torch.int32, device=_device.device())
        rc = _device.lib().tmps_contact_count(atom.cstruct(), neighbor.cstruct(None, None), domain.dbox,
                                              self._count.data_ptr(), _device.stream())
        _lib.check(rc, "tmps_contact_count")
        ordered = torch.empty(n, dtype=torch.int32, device=self._count.device)
        ordered[atom.buffers.uid.long()] = self._count[:n]
        return ordered.cpu().numpy()

    @staticmethod
    def reduce(counts: np.ndarray, mode: str = "ave") -> float:
        """compute reduce over the per-atom counts: sum, ave, min or max."""
        c = np.asarray(counts, dtype=np.float64)
        if c.size == 0:
            return 0.0
        return float({"sum": c.sum, "ave": c.mean, "min": c.min, "max": c.max}[mode]())

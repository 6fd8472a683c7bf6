"""
Pressure and virial reductions (src/taichimps/computes/thermo.py:33-215).

``compute_pressure_tensor`` sums the per-atom virial the contact kernel
tallied (plus, with ``kinetic``, sum m v_a v_b) on the device in a fixed order
and divides by the volume: the LAMMPS ``compute pressure`` tensor
[xx, yy, zz, xy, xz, yz].
"""

from __future__ import annotations

import math
from typing import Any

import numpy as np
import torch

from .. import _device, _lib

BOLTZMANN = 1.3806504e-23
MAX_VIRIAL_CHUNKS = 1024


def virial_chunks(nlocal: int) -> int:
    """Chunk count the reference uses for its reduction (thermo.py:28-30)."""
    return int(min(MAX_VIRIAL_CHUNKS, max(64, 2.0 * math.sqrt(max(nlocal, 1)))))


class _DeviceVector:
    def __init__(self, t: torch.Tensor):
        self.t = t

    def to_numpy(self) -> np.ndarray:
        return self.t.detach().cpu().numpy().copy()


class Computes:
    def __init__(self, float_type: Any = None) -> None:
        self.float_type = float_type
        self.dev = _device.device()
        self._vt = torch.zeros(6, dtype=torch.float64, device=self.dev)
        self.virial_tensor = _DeviceVector(self._vt)
        self._ws = torch.zeros(0, dtype=torch.uint8, device=self.dev)

    def compute_virial_kernel(self, nlocal: int, atom, keflag: int, chunks: int | None = None) -> None:
        """Device reduction of the per-atom virial (+ kinetic term) into virial_tensor."""
        L = _device.lib()
        wsb = int(L.tmps_virial_workspace_bytes(atom.nlocal))
        if self._ws.numel() < wsb:
            self._ws = torch.zeros(wsb, dtype=torch.uint8, device=self.dev)
        _lib.check(L.tmps_virial_reduce(atom.cstruct(), int(keflag), self._vt.data_ptr(), self._ws.data_ptr(),
                                        wsb, _device.stream()), "tmps_virial_reduce")

    def compute_pressure_tensor(self, atom, domain, kinetic: bool = True) -> np.ndarray:
        if atom.nlocal == 0:
            return np.zeros(6, dtype=np.float64)
        domain.pull()
        vol = domain.volume
        if vol <= 0.0:
            return np.zeros(6, dtype=np.float64)
        self.compute_virial_kernel(atom.nlocal, atom, 1 if kinetic else 0)
        return self.virial_tensor.to_numpy() / vol

    # Output-only quantities (not on the per-step path).
    def _ke(self, atom) -> tuple[float, float]:
        b = atom.buffers
        v, m = b.vm[:, :3], b.vm[:, 3]
        w, inertia = b.om[:, :3], b.om[:, 3]
        ket = float((0.5 * m * (v * v).sum(dim=1)).sum().item())
        ker = float((0.5 * inertia * (w * w).sum(dim=1)).sum().item())
        return ket, ker

    def ke_trans(self, atom) -> float:
        return 0.0 if atom.nlocal == 0 else self._ke(atom)[0]

    def ke_rot(self, atom) -> float:
        return 0.0 if atom.nlocal == 0 else self._ke(atom)[1]

    def ke_total(self, atom) -> float:
        return 0.0 if atom.nlocal == 0 else sum(self._ke(atom))

    def kinetic_tensor(self, atom) -> np.ndarray:
        if atom.nlocal == 0:
            return np.zeros(6)
        self.compute_virial_kernel(atom.nlocal, _NoVirial(atom), 1)
        return self.virial_tensor.to_numpy()

    def temperature(self, atom) -> float:
        if atom.nlocal == 0:
            return 0.0
        dof = 3.0 * atom.nlocal - 3.0
        if dof <= 0.0:
            return 0.0
        return float(np.sum(self.kinetic_tensor(atom)[:3]) / (dof * BOLTZMANN))


class _NoVirial:
    """An atom view whose per-atom virial pointer is NULL (kinetic term only)."""

    def __init__(self, atom):
        self._atom = atom
        self.nlocal = atom.nlocal

    def cstruct(self):
        s = self._atom.cstruct()
        s.virial = None
        return s

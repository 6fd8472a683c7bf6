"""
Simulation box: host mirror plus a device-resident ``tmps_box``.

Mirrors taichimps ``Domain`` (src/taichimps/domain.py:12-584): the box is held
twice, as host numpy arrays and as a device struct every kernel reads.  A
kernel that changes the box (the pressure servo) leaves the host mirror
stale; reading a box property then raises until ``pull()`` brings it back,
exactly as the reference does (domain.py:93-167).

Only orthogonal boxes are supported on this path: a non-zero tilt raises.
"""

from __future__ import annotations

from typing import Any

import numpy as np

from . import _device, _lib


class Domain:
    def __init__(self, boxlo, boxhi, boundary=("p", "p", "p"), tilt=None, float_type: Any = None) -> None:
        self.float_type = float_type
        self._boxlo = np.array([float(v) for v in boxlo], dtype=np.float64)
        self._boxhi = np.array([float(v) for v in boxhi], dtype=np.float64)
        self._prd = self._boxhi - self._boxlo
        self._periodicity = np.array([1 if b == "p" else 0 for b in boundary], dtype=np.int32)
        self._tilt = np.zeros(3, dtype=np.float64)
        if tilt is not None:
            self._tilt = np.array([float(v) for v in tilt], dtype=np.float64)
            if np.any(self._tilt != 0.0):
                raise NotImplementedError("taichimps_gb300 supports orthogonal boxes only (tilt must be zero)")
        self._h_rate = np.zeros(6, dtype=np.float64)
        self.vremap = False
        self._host_stale = False
        # neighbor grid published with the box (set by NeighborList.build)
        self.grid_dim = np.ones(3, dtype=np.int32)
        self.cell_size = np.ones(3, dtype=np.float64)
        self._dbox = _device.struct_buffer(_lib.Box())
        self._sync()

    # ---------------------------------------------------- host / device

    def mark_device_authoritative(self) -> None:
        self._host_stale = True

    def pull(self) -> None:
        """Bring the host mirror in step with the device (synchronises)."""
        if not self._host_stale:
            return
        self.take_pulled(_device.pull_struct(self._dbox, _lib.Box))

    @property
    def dbox_tensor(self):
        """The device box record's byte buffer."""
        return self._dbox

    def take_pulled(self, b) -> None:
        """Adopt a box record read from the device (the current one) as the host mirror."""
        self._boxlo = np.array(b.lo[:], dtype=np.float64)
        self._boxhi = np.array(b.hi[:], dtype=np.float64)
        self._prd = np.array(b.prd[:], dtype=np.float64)
        self._h_rate = np.array(b.h_rate[:], dtype=np.float64)
        self.vremap = bool(b.vremap)
        self._host_stale = False

    def _fresh(self, name: str) -> None:
        if self._host_stale:
            raise RuntimeError(
                f"Domain.{name} was read while the device holds the current box. "
                "Call domain.pull() first, at a point where synchronising with "
                "the device is acceptable -- not on the per-step path.")

    @property
    def boxlo(self) -> np.ndarray:
        self._fresh("boxlo")
        return self._boxlo

    @property
    def boxhi(self) -> np.ndarray:
        self._fresh("boxhi")
        return self._boxhi

    @property
    def prd(self) -> np.ndarray:
        self._fresh("prd")
        return self._prd

    @property
    def tilt(self) -> np.ndarray:
        self._fresh("tilt")
        return self._tilt

    @property
    def h_rate(self) -> np.ndarray:
        self._fresh("h_rate")
        return self._h_rate

    @property
    def periodicity(self) -> np.ndarray:
        return self._periodicity

    @property
    def triclinic(self) -> bool:
        return False

    @property
    def xy(self) -> float:
        return 0.0

    @property
    def xz(self) -> float:
        return 0.0

    @property
    def yz(self) -> float:
        return 0.0

    def host_box(self) -> _lib.Box:
        """The host mirror as a tmps_box struct (grid fields included)."""
        b = _lib.Box()
        for k in range(3):
            b.lo[k] = float(self._boxlo[k])
            b.hi[k] = float(self._boxhi[k])
            b.prd[k] = float(self._prd[k])
            b.inv_prd[k] = 1.0 / float(self._prd[k]) if self._prd[k] != 0.0 else 0.0
            b.per[k] = int(self._periodicity[k])
            b.g[k] = int(self.grid_dim[k])
            b.csize[k] = float(self.cell_size[k])
            b.hcell[k] = float(self._prd[k]) / float(self.grid_dim[k])
            b.old_lo[k] = float(self._boxlo[k])
            b.old_prd[k] = float(self._prd[k])
        for k in range(6):
            b.h_rate[k] = float(self._h_rate[k])
        b.vremap = 1 if self.vremap else 0
        b.ncell = int(np.prod(self.grid_dim))
        b.remap_pending = 0
        return b

    def _sync(self) -> None:
        """Push the host box to the device (Domain._sync, domain.py:235-254)."""
        self._host_stale = False
        _device.push_struct(self._dbox, self.host_box())

    @property
    def dbox(self) -> int:
        """Device pointer of the tmps_box every kernel reads."""
        return self._dbox.data_ptr()

    @property
    def volume(self) -> float:
        prd = self.prd
        return float(prd[0] * prd[1] * prd[2])

    def set_box(self, boxlo, boxhi, tilt=None) -> None:
        self._boxlo = np.array([float(v) for v in boxlo], dtype=np.float64)
        self._boxhi = np.array([float(v) for v in boxhi], dtype=np.float64)
        self._prd = self._boxhi - self._boxlo
        if tilt is not None and np.any(np.asarray(tilt, dtype=np.float64) != 0.0):
            raise NotImplementedError("taichimps_gb300 supports orthogonal boxes only")
        self._sync()

    def set_tilt(self, tilt) -> None:
        if np.any(np.asarray(tilt, dtype=np.float64) != 0.0):
            raise NotImplementedError("taichimps_gb300 supports orthogonal boxes only")

    def set_box_and_h_rate(self, boxlo, boxhi, tilt, h_rate, vremap: bool) -> None:
        self._boxlo = np.array([float(v) for v in boxlo], dtype=np.float64)
        self._boxhi = np.array([float(v) for v in boxhi], dtype=np.float64)
        self._prd = self._boxhi - self._boxlo
        self._h_rate = np.asarray(h_rate, dtype=np.float64).copy()
        self.vremap = bool(vremap)
        self._sync()

    def set_h_rate(self, h_rate, vremap: bool) -> None:
        self._fresh("h_rate")
        self._h_rate = np.asarray(h_rate, dtype=np.float64).copy()
        self.vremap = bool(vremap)
        self._sync()

    def set_boundary(self, boundary) -> None:
        self._periodicity = np.array([1 if b == "p" else 0 for b in boundary], dtype=np.int32)
        self._sync()

    def set_grid(self, gdim, csize) -> None:
        """Publish the neighbor grid with the box (host mirror must be current)."""
        self._fresh("grid")
        self.grid_dim = np.asarray(gdim, dtype=np.int32).copy()
        self.cell_size = np.asarray(csize, dtype=np.float64).copy()
        self._sync()

    def bounding_box(self):
        return self._boxlo.copy(), self._boxhi.copy()

    @property
    def pbc_x(self) -> bool:
        return bool(self._periodicity[0])

    @property
    def pbc_y(self) -> bool:
        return bool(self._periodicity[1])

    @property
    def pbc_z(self) -> bool:
        return bool(self._periodicity[2])

    def pbc(self, atom) -> None:
        """Wrap positions into the box; under remap v also kick crossing velocities."""
        if atom.nlocal == 0:
            return
        L = _device.lib()
        _lib.check(L.tmps_pbc(atom.cstruct(), self.dbox, _device.stream()), "tmps_pbc")

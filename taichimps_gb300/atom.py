"""
Per-atom state of atom_style sphere, held in device tensors.

Mirrors taichimps ``AtomSystem`` (src/taichimps/atom.py:13-220).  Storage is
internal-order and packed for the kernels (see include/taichimps_gb300.h):
``xr`` = (x, y, z, radius), ``vm`` = (v, mass), ``om`` = (omega, inertia),
``f``/``torque`` component-major.  The neighbor build re-sorts atoms by cell,
so internal order changes; ``uid`` records each slot's insertion index and the
field views below (``atom.x.to_numpy()`` ...) always present insertion order,
padded to ``max_atoms`` rows like the reference's Taichi fields.
"""

from __future__ import annotations

from typing import Any

import numpy as np
import torch

from . import _device, _lib

def _sphere_mass(rad: np.ndarray, dens: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """rmass = (4/3) pi r^3 density and inertia 0.4 m r r (atom.py:110-111), numpy's pow for r^3 as
    in the reference."""
    vol = (4.0 / 3.0) * np.pi * (rad ** 3)
    mass = vol * dens
    inertia = ((0.4 * mass) * rad) * rad
    return mass, inertia


class _Buffers:
    """One complete set of per-atom device arrays (two exist: build permutes A -> B).  `fill`: zeros;
    without it the arrays are left unset (a permutation target, which the build writes in full)."""

    def __init__(self, n: int, dev: torch.device, fill: bool = True) -> None:
        f64 = dict(dtype=torch.float64, device=dev)
        i32 = dict(dtype=torch.int32, device=dev)
        new = torch.zeros if fill else torch.empty
        self.xr = new((n, 4), **f64)
        self.vm = new((n, 4), **f64)
        self.om = new((n, 4), **f64)
        self.f = new((3, n), **f64)
        self.torque = new((3, n), **f64)
        self.virial = new((6, n), **f64)
        self.tag = new(n, **i32)
        self.uid = new(n, **i32)
        self.x0 = new((3, n), **f64)


_EMPTY: dict = {}


def _empty_buffers(dev: torch.device) -> _Buffers:
    """The arrays of an empty system (shared: nothing writes to zero-length arrays)."""
    if dev not in _EMPTY:
        _EMPTY[dev] = _Buffers(0, dev)
    return _EMPTY[dev]


class FieldView:
    """
    Reference-style access to one per-atom quantity in insertion order:
    ``to_numpy()``, ``from_numpy()``, ``fill()``, ``[i]`` and ``[i] = v``.
    """

    def __init__(self, atom: "AtomSystem", name: str, width: int, dtype) -> None:
        self._atom, self._name, self._w, self._dtype = atom, name, width, dtype

    def _internal(self) -> torch.Tensor:
        return self._atom._internal_view(self._name)

    def to_numpy(self) -> np.ndarray:
        a = self._atom
        shape = (a.max_atoms,) if self._w == 1 else (a.max_atoms, self._w)
        if not a.nlocal:
            return np.zeros(shape, dtype=self._dtype)
        if self._name in _lib.FIELD:
            # one kernel writes the rows in insertion order straight into page-locked memory
            shape_n = (a.nlocal,) if self._w == 1 else (a.nlocal, self._w)
            staged = torch.empty(shape_n, dtype=torch.float64, pin_memory=True)
            rc = _device.lib().tmps_atoms_read(a.cstruct(), _lib.FIELD[self._name], a.slot_scratch().data_ptr(),
                                               staged.data_ptr(), _device.stream())
            _lib.check(rc, "tmps_atoms_read")
        else:
            # back to insertion order on the device, then one contiguous copy
            vals = self._internal().detach()
            ordered = torch.empty(vals.shape, dtype=vals.dtype, device=vals.device)
            ordered[a.buffers.uid.long()] = vals
            staged = torch.empty(vals.shape, dtype=vals.dtype, pin_memory=True)
            staged.copy_(ordered, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        host = staged.numpy().astype(self._dtype, copy=False)
        if a.nlocal == a.max_atoms:
            return host
        out = np.zeros(shape, dtype=self._dtype)
        out[:a.nlocal] = host
        return out

    def from_numpy(self, arr) -> None:
        a = self._atom
        arr = np.asarray(arr)
        n = a.nlocal
        vals = arr[:n]
        uid = a.uid_host()
        t = torch.from_numpy(np.ascontiguousarray(vals[uid]).astype(self._dtype)).to(a.device)
        a._assign_internal(self._name, t)

    def fill(self, value: float) -> None:
        a = self._atom
        if a.nlocal:
            v = self._internal()
            a._assign_internal(self._name, torch.full_like(v, value))

    def __getitem__(self, i: int):
        return self.to_numpy()[i]

    def __setitem__(self, i: int, value) -> None:
        full = self.to_numpy()
        full[i] = np.asarray(value, dtype=self._dtype)
        self.from_numpy(full)

    def __array__(self, dtype=None):
        a = self.to_numpy()
        return a if dtype is None else a.astype(dtype)


class AtomSystem:
    def __init__(self, max_atoms: int, float_type: Any = None) -> None:
        self.max_atoms = int(max_atoms)
        self.nlocal = 0
        self.float_type = float_type
        self.device = _device.device()
        self._buf = self._alt = _empty_buffers(self.device)
        # per-atom type and mask on the host; a uniform value stays a scalar until read as an array
        self._type_arr: np.ndarray | None = np.zeros(0, dtype=np.int32)
        self._mask_arr: np.ndarray | None = np.zeros(0, dtype=np.int32)
        self._type_fill = 1
        self._uid_cache: np.ndarray | None = None
        self.x = FieldView(self, "x", 3, np.float64)
        self.v = FieldView(self, "v", 3, np.float64)
        self.f = FieldView(self, "f", 3, np.float64)
        self.omega = FieldView(self, "omega", 3, np.float64)
        self.torque = FieldView(self, "torque", 3, np.float64)
        self.radius = FieldView(self, "radius", 1, np.float64)
        self.rmass = FieldView(self, "rmass", 1, np.float64)
        self.tag = FieldView(self, "tag", 1, np.int32)
        self.virial = FieldView(self, "virial", 6, np.float64)
        self._max_radius, self._max_radius_dev = 0.0, None
        self._pending_inputs = None
        self._slot_of: torch.Tensor | None = None
        self._listeners: list = []

    # ------------------------------------------------------------ views

    def _internal_view(self, name: str) -> torch.Tensor:
        b = self._buf
        return {
            "x": lambda: b.xr[:, :3], "v": lambda: b.vm[:, :3], "omega": lambda: b.om[:, :3],
            "radius": lambda: b.xr[:, 3], "rmass": lambda: b.vm[:, 3],
            "f": lambda: b.f.t(), "torque": lambda: b.torque.t(), "virial": lambda: b.virial.t(),
            "tag": lambda: b.tag,
        }[name]()

    def _assign_internal(self, name: str, t: torch.Tensor) -> None:
        self._internal_view(name).copy_(t)
        if name in ("radius", "rmass"):
            # keep the packed inertia in step (atom.py:110-111, nve_sphere.py:63)
            b = self._buf
            m, r = b.vm[:, 3], b.xr[:, 3]
            b.om[:, 3] = ((0.4 * m) * r) * r
            self.max_radius = float(b.xr[:, 3].max().item()) if self.nlocal else 0.0

    def slot_scratch(self) -> torch.Tensor:
        """int32[n] device scratch of tmps_atoms_read."""
        if self._slot_of is None or self._slot_of.numel() < self.nlocal:
            self._slot_of = torch.empty(max(self.nlocal, 1), dtype=torch.int32, device=self.device)
        return self._slot_of

    def uid_host(self) -> np.ndarray:
        if self._uid_cache is None:
            self._uid_cache = self._buf.uid.cpu().numpy().astype(np.int64)
        return self._uid_cache

    @property
    def buffers(self) -> _Buffers:
        return self._buf

    @property
    def alt_buffers(self) -> _Buffers:
        return self._alt

    def swap_buffers(self) -> None:
        """Called by the neighbor build after permuting into the alternate set."""
        self._buf, self._alt = self._alt, self._buf
        self._uid_cache = None
        for cb in self._listeners:
            cb()

    def cstruct(self, b: _Buffers | None = None) -> _lib.Atoms:
        b = self._buf if b is None else b
        s = _lib.Atoms()
        s.n = self.nlocal
        s.xr, s.vm, s.om = b.xr.data_ptr(), b.vm.data_ptr(), b.om.data_ptr()
        s.f, s.torque, s.virial = b.f.data_ptr(), b.torque.data_ptr(), b.virial.data_ptr()
        s.tag, s.uid, s.x0 = b.tag.data_ptr(), b.uid.data_ptr(), b.x0.data_ptr()
        return s

    # ---------------------------------------------------------- particles

    def add_particles(self, x, radius, density, v=None, omega=None, tag=None, atom_type=1, rmass=None) -> None:
        """Append particles; rmass = 4/3 pi r^3 density (atom.py:55-145).  Arrays may be numpy or
        torch tensors; a pinned host tensor or a CUDA tensor is uploaded without a host copy.
        `rmass` (not in the reference): the masses as given, for a system read back from a restart
        file, which stores them -- recomputing them from a density would round differently."""
        tens = {k: a for k, a in (("x", x), ("v", v), ("omega", omega)) if isinstance(a, torch.Tensor)}
        if (tens and rmass is None and self.nlocal == 0 and "x" in tens
                and all(t.dtype == torch.float64 and t.dim() == 2 and t.shape[1] == 3 for t in tens.values())
                and all(isinstance(a, torch.Tensor) for a in (v, omega) if a is not None)):
            self._add_first_tensors(tens, radius, density, tag, atom_type)
            return
        if isinstance(radius, torch.Tensor):
            radius = radius.detach().cpu().numpy()
        x = x.detach().cpu().numpy() if isinstance(x, torch.Tensor) else x
        v = v.detach().cpu().numpy() if isinstance(v, torch.Tensor) else v
        omega = omega.detach().cpu().numpy() if isinstance(omega, torch.Tensor) else omega
        x_np = np.asarray(x, dtype=np.float64)
        if x_np.ndim == 1:
            x_np = x_np.reshape(1, 3)
        n_new = len(x_np)
        if self.nlocal + n_new > self.max_atoms:
            raise ValueError(f"Exceeded max_atoms capacity: {self.nlocal + n_new} > {self.max_atoms}")
        v_np = np.zeros_like(x_np) if v is None else np.asarray(v, dtype=np.float64).reshape(n_new, 3)
        o_np = np.zeros_like(x_np) if omega is None else np.asarray(omega, dtype=np.float64).reshape(n_new, 3)
        rad = np.asarray(radius, dtype=np.float64)
        if rad.ndim == 0:
            rad = np.full(n_new, float(rad))
        dens = np.full(n_new, float(density)) if np.isscalar(density) else np.asarray(density, dtype=np.float64)
        types = (np.full(n_new, int(atom_type), dtype=np.int32) if np.isscalar(atom_type)
                 else np.asarray(atom_type, dtype=np.int32))
        mass, inertia = _sphere_mass(rad, dens)
        if rmass is not None:
            mass = np.broadcast_to(np.asarray(rmass, dtype=np.float64), rad.shape).copy()
            inertia = ((0.4 * mass) * rad) * rad
        start = self.nlocal
        tags = (np.arange(start + 1, start + n_new + 1, dtype=np.int32) if tag is None
                else np.asarray(tag, dtype=np.int32))

        n = start + n_new
        if start == 0:
            # first particles: upload the inputs, assemble the packed records on the device
            nb = _Buffers(n, self.device)
            dev = self.device

            def up(arr):
                return torch.from_numpy(np.ascontiguousarray(arr)).to(dev)

            nb.xr[:, :3] = up(x_np)
            nb.xr[:, 3] = up(rad)
            nb.vm[:, :3] = up(v_np)
            nb.vm[:, 3] = up(mass)
            if omega is not None:
                nb.om[:, :3] = up(o_np)
            nb.om[:, 3] = up(inertia)
            nb.tag.copy_(up(tags))
            nb.uid.copy_(torch.arange(n, dtype=torch.int32, device=dev))
            self._buf = nb
            self._alt = _Buffers(n, dev, fill=False)
            self.atom_type_host = np.concatenate([self.atom_type_host, types])
            self.mask_host = np.concatenate([self.mask_host, np.ones(n_new, dtype=np.int32)])
            self.nlocal = n
            self._uid_cache = None
            self.max_radius = float(rad.max()) if n else 0.0
            for cb in self._listeners:
                cb()
            return
        old = self._gather_all()
        nb = _Buffers(n, self.device)
        host = {
            "xr": np.zeros((n, 4)), "vm": np.zeros((n, 4)), "om": np.zeros((n, 4)),
            "f": np.zeros((3, n)), "torque": np.zeros((3, n)), "virial": np.zeros((6, n)),
            "tag": np.zeros(n, dtype=np.int32), "uid": np.arange(n, dtype=np.int32),
            "x0": np.zeros((3, n)),
        }
        for k in ("xr", "vm", "om", "tag"):
            host[k][:start] = old[k]
        for k in ("f", "torque", "virial", "x0"):
            host[k][:, :start] = old[k]
        host["xr"][start:, :3] = x_np
        host["xr"][start:, 3] = rad
        host["vm"][start:, :3] = v_np
        host["vm"][start:, 3] = mass
        host["om"][start:, :3] = o_np
        host["om"][start:, 3] = inertia
        host["tag"][start:] = tags
        for k, arr in host.items():
            getattr(nb, k).copy_(torch.from_numpy(np.ascontiguousarray(arr)))
        self._buf = nb
        self._alt = _Buffers(n, self.device)
        self.atom_type_host = np.concatenate([self.atom_type_host, types])
        self.mask_host = np.concatenate([self.mask_host, np.ones(n_new, dtype=np.int32)])
        self.nlocal = n
        self._uid_cache = None
        self.max_radius = float(host["xr"][:, 3].max()) if n else 0.0
        for cb in self._listeners:
            cb()

    def _add_first_tensors(self, tens, radius, density, tag, atom_type) -> None:
        """add_particles into an empty system from float64 [n, 3] tensors (x; v and omega optional):
        the records, masses and moments of inertia are assembled by one kernel (tmps_atoms_assemble)
        that reads page-locked host or device arrays in place, with r^3 rounded once (as numpy's
        r**3 of the array path rounds it) and the products in the reference's order; the largest
        radius stays on the device until something reads it."""
        dev = self.device
        L = _device.lib()
        keep = []  # inputs staged for the kernel, alive until it has run

        def readable(t: torch.Tensor, shape_n3: bool) -> torch.Tensor:
            t = t.detach()
            if t.dtype != torch.float64 or not t.is_contiguous():
                t = t.to(torch.float64).contiguous()
            if not (t.is_cuda or t.is_pinned()):
                t = t.to(dev, non_blocking=False)
            keep.append(t)
            return t

        xt = readable(tens["x"], True)
        n = int(xt.shape[0])
        if n > self.max_atoms:
            raise ValueError(f"Exceeded max_atoms capacity: {n} > {self.max_atoms}")

        def per_atom(val, what):
            """(pointer or None, value for every atom) of a per-atom double or a scalar."""
            if torch.is_tensor(val):
                t = readable(val.reshape(-1), False)
                if t.numel() == 1:
                    return None, float(t.cpu()[0])
                if t.numel() != n:
                    raise ValueError(f"{what}: {t.numel()} values for {n} particles")
                return t.data_ptr(), 0.0
            a = np.asarray(val, dtype=np.float64)
            if a.ndim == 0 or a.size == 1:
                return None, float(a.reshape(-1)[0])
            if a.size != n:
                raise ValueError(f"{what}: {a.size} values for {n} particles")
            t = torch.from_numpy(np.ascontiguousarray(a.reshape(-1))).to(dev)
            keep.append(t)
            return t.data_ptr(), 0.0

        r_ptr, r_val = per_atom(radius, "radius")
        d_ptr, d_val = per_atom(density, "density")
        v_ptr = readable(tens["v"], True).data_ptr() if "v" in tens else None
        w_ptr = readable(tens["omega"], True).data_ptr() if "omega" in tens else None
        tag_ptr = None
        if tag is not None:
            tt = torch.from_numpy(np.ascontiguousarray(np.asarray(tag, dtype=np.int32))).to(dev)
            keep.append(tt)
            tag_ptr = tt.data_ptr()
        types = None if np.isscalar(atom_type) else np.asarray(atom_type, dtype=np.int32)
        nb = _Buffers(n, dev, fill=False)  # the kernel writes every array
        self._buf = nb
        self._alt = _Buffers(n, dev, fill=False)
        self.nlocal = n
        rmax = torch.empty(1, dtype=torch.float64, device=dev)
        rc = L.tmps_atoms_assemble(self.cstruct(nb), xt.data_ptr(), v_ptr, w_ptr, r_ptr, r_val, d_ptr, d_val,
                                   tag_ptr, rmax.data_ptr(), _device.stream())
        if rc != _lib.TMPS_OK:
            # nothing was added: back to the empty system before reporting
            self._buf = self._alt = _empty_buffers(dev)
            self.nlocal = 0
        _lib.check(rc, "tmps_atoms_assemble")
        # page-locked inputs are read in place: held until a synchronisation shows the kernel has run
        self._pending_inputs = keep
        if np.isscalar(atom_type):
            self._type_arr, self._type_fill = None, int(atom_type)
        else:
            self.atom_type_host = types
        self._mask_arr = None
        self._uid_cache = None
        self._max_radius, self._max_radius_dev = 0.0, rmax
        for cb in self._listeners:
            cb()

    @property
    def max_radius(self) -> float:
        """The largest radius (a device value from tmps_atoms_assemble is read on first use)."""
        if self._max_radius_dev is not None:
            self._max_radius = float(self._max_radius_dev.item())
            self._max_radius_dev = None
            self._pending_inputs = None
        return self._max_radius

    @max_radius.setter
    def max_radius(self, value: float) -> None:
        self._max_radius, self._max_radius_dev = float(value), None

    def _gather_all(self) -> dict[str, np.ndarray]:
        """All per-atom arrays in insertion order (host copies)."""
        b = self._buf
        uid = self.uid_host()
        out = {}
        for k in ("xr", "vm", "om", "tag"):
            a = getattr(b, k).cpu().numpy()
            o = np.empty_like(a)
            o[uid] = a
            out[k] = o
        for k in ("f", "torque", "virial", "x0"):
            a = getattr(b, k).cpu().numpy()
            o = np.empty_like(a)
            o[:, uid] = a
            out[k] = o
        return out

    def on_reorder(self, cb) -> None:
        """Register a callback run whenever internal order or size changes."""
        self._listeners.append(cb)

    @property
    def atom_type_host(self) -> np.ndarray:
        if self._type_arr is None:
            self._type_arr = np.full(self.nlocal, self._type_fill, dtype=np.int32)
        return self._type_arr

    @atom_type_host.setter
    def atom_type_host(self, v) -> None:
        self._type_arr = np.asarray(v, dtype=np.int32)

    @property
    def mask_host(self) -> np.ndarray:
        if self._mask_arr is None:
            self._mask_arr = np.ones(self.nlocal, dtype=np.int32)
        return self._mask_arr

    @mask_host.setter
    def mask_host(self, v) -> None:
        self._mask_arr = np.asarray(v, dtype=np.int32)

    @property
    def atom_type(self) -> np.ndarray:
        return self.atom_type_host

    @property
    def mask(self) -> np.ndarray:
        return self.mask_host

    def clear_forces(self) -> None:
        """Zero f, torque and the per-atom virial (atom.py:201-220)."""
        if self.nlocal == 0:
            return
        _lib.check(_device.lib().tmps_clear_forces(self.cstruct(), _device.stream()), "tmps_clear_forces")

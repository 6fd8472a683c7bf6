"""
Particle input and output through the C ABI (tmps_atoms_assemble, tmps_atoms_read): a system built
from page-locked host tensors or device tensors equals one built from numpy arrays (positions,
velocities and radii bit for bit; masses within one ulp of numpy's (4/3 pi) r**3 density, the
reference's expression), and every field read back in insertion order after a neighbor build has
re-sorted the atoms equals the device records reordered on the host.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _system(G, x, r, v, dens=2.5, L=12.0, tensors=None):
    dom = G.Domain(boxlo=[0.0] * 3, boxhi=[L] * 3, boundary=("p", "p", "p"))
    atom = G.AtomSystem(max_atoms=len(x))
    if tensors is None:
        atom.add_particles(x=x, radius=r, density=dens, v=v)
    else:
        atom.add_particles(x=tensors["x"], radius=tensors["radius"], density=dens, v=tensors["v"])
    return dom, atom


def _packing(n, seed, L=12.0):
    rng = np.random.default_rng(seed)
    x = rng.uniform(0.0, L, size=(n, 3))
    r = rng.uniform(0.4, 0.6, size=n)
    v = rng.normal(size=(n, 3))
    return x, r, v


@pytest.mark.parametrize("where", ["pinned", "cuda"])
def test_tensor_input_matches_array_input(gpu, where):
    import torch
    import taichimps_gb300 as G
    n = 5000
    x, r, v = _packing(n, 3)
    _, ref = _system(G, x, r, v)

    def t(a):
        a = torch.from_numpy(np.ascontiguousarray(a))
        return a.pin_memory() if where == "pinned" else a.cuda()

    _, atom = _system(G, x, r, v, tensors={"x": t(x), "radius": t(r), "v": t(v)})
    assert atom.max_radius == r.max()
    for name in ("x", "v", "radius", "omega", "tag"):
        np.testing.assert_array_equal(getattr(atom, name).to_numpy(), getattr(ref, name).to_numpy(), err_msg=name)
    for name in ("f", "torque", "virial"):
        assert not getattr(atom, name).to_numpy().any(), name
    m, m_ref = atom.rmass.to_numpy(), ref.rmass.to_numpy()
    expect = (4.0 / 3.0) * np.pi * (r ** 3) * 2.5
    np.testing.assert_array_equal(m_ref, expect)
    # r^3 rounded once on the device; numpy's pow may round differently within an ulp at most
    ulps = np.abs(m.view(np.int64) - expect.view(np.int64))
    assert ulps.max() <= 1 and np.count_nonzero(ulps) <= n // 1000, (ulps.max(), np.count_nonzero(ulps))
    inertia = atom.buffers.om[:, 3].cpu().numpy()
    mm = atom.buffers.vm[:, 3].cpu().numpy()
    rr = atom.buffers.xr[:, 3].cpu().numpy()
    np.testing.assert_array_equal(inertia, ((0.4 * mm) * rr) * rr)


def test_field_reads_follow_insertion_order(gpu):
    """After a build re-sorts the atoms, each field read back by the kernel equals the device
    records reordered by uid on the host, for the packed and the component-major fields."""
    import torch
    import taichimps_gb300 as G
    n = 3000
    x, r, v = _packing(n, 7)
    dom, atom = _system(G, x, r, v)
    nl = G.NeighborList(domain=dom, skin=0.1, max_atoms=n, max_neighbors_per_atom=32)
    nl.build(atom)
    b = atom.buffers
    uid = b.uid.cpu().numpy()
    assert not np.array_equal(uid, np.arange(n))  # the build did re-sort
    rng = np.random.default_rng(1)
    # give every component-major field distinct values
    for name, rows in (("f", 3), ("torque", 3), ("virial", 6)):
        getattr(b, name).copy_(torch.from_numpy(rng.normal(size=(rows, n))))
    b.om[:, :3] = torch.from_numpy(rng.normal(size=(n, 3))).cuda()
    host = {"x": b.xr[:, :3], "v": b.vm[:, :3], "omega": b.om[:, :3], "radius": b.xr[:, 3], "rmass": b.vm[:, 3],
            "f": b.f.t(), "torque": b.torque.t(), "virial": b.virial.t()}
    for name, dev in host.items():
        vals = dev.cpu().numpy()
        want = np.empty_like(vals)
        want[uid] = vals
        got = getattr(atom, name).to_numpy()
        np.testing.assert_array_equal(got, want, err_msg=name)
    np.testing.assert_array_equal(atom.x.to_numpy(), x)


def test_pageable_input_is_refused(gpu):
    """The entry point takes device or page-locked memory only; a pageable host array is refused
    before any launch."""
    import torch
    import taichimps_gb300 as G
    from taichimps_gb300 import _device, _lib
    x, r, v = _packing(64, 2)
    _, atom = _system(G, x, r, v)
    L = _device.lib()
    pageable = np.ascontiguousarray(x)
    rmax = torch.empty(1, dtype=torch.float64, device="cuda")
    rc = L.tmps_atoms_assemble(atom.cstruct(), pageable.ctypes.data_as(ctypes.c_void_p), None, None, None, 0.5,
                               None, 2.5, None, rmax.data_ptr(), _device.stream())
    assert rc == _lib.TMPS_ERR_BAD_ARG
    out = np.empty((64, 3))
    rc = L.tmps_atoms_read(atom.cstruct(), _lib.FIELD["x"], atom.slot_scratch().data_ptr(),
                           out.ctypes.data_as(ctypes.c_void_p), _device.stream())
    assert rc == _lib.TMPS_ERR_BAD_ARG
    torch.cuda.synchronize()

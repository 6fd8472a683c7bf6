"""
tmps_nlist_build_noalloc: the neighbor build for callers that cannot allocate
device memory (a fixed device arena owned by the host, a step loop that must
not enter the CUDA allocator, a foreign-language host that only passes
registered arrays).  Its scratch is built into the library, so this checks, through the
C ABI, that it gives exactly what tmps_nlist_build gives with a caller-provided
workspace, on two calls in a row (the second reuses the scratch the first
left behind), and that it refuses sizes beyond its fixed limits.

The file is named to run last: if it fails, a run stopped at the first failure
has already run every other test.  It also passes alone in a fresh process.
"""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _system(n_side=16, seed=3):
    import taichimps_gb300 as G
    from taichimps_gb300.packing import make_packing
    p = make_packing(n_side ** 3, 0.9, 1.1, 0.40, seed)
    dom = G.Domain(boxlo=[0.0] * 3, boxhi=[p["L"]] * 3)
    atom = G.AtomSystem(max_atoms=len(p["x"]))
    atom.add_particles(x=p["x"], radius=p["radius"], density=2.5)
    nl = G.NeighborList(domain=dom, skin=0.1, max_atoms=len(p["x"]), max_neighbors_per_atom=16)
    nl.setup_grid(2.0 * atom.max_radius)
    return dom, atom, nl


def _outputs(atom, n, slots):
    """Fresh output buffers for one build call."""
    from taichimps_gb300.atom import _Buffers
    dst = _Buffers(n, atom.device)
    i32 = dict(dtype=torch.int32, device=atom.device)
    return {"dst": dst, "nbr": torch.zeros((slots, n), **i32), "nnb": torch.zeros(n, **i32),
            "order": torch.zeros(n, **i32), "cell_of": torch.zeros(n, **i32), "status": torch.zeros(1, **i32)}


def _nl_struct(o, n, slots):
    from taichimps_gb300 import _lib
    s = _lib.NList()
    s.n, s.slots = n, slots
    s.nbr, s.nnb = o["nbr"].data_ptr(), o["nnb"].data_ptr()
    return s


def _snapshot(o, n):
    nnb = o["nnb"].cpu().numpy()
    nbr = o["nbr"].cpu().numpy()
    rows = [nbr[: nnb[p], p].copy() for p in range(n)]
    d = o["dst"]
    return {"nnb": nnb, "rows": rows, "order": o["order"].cpu().numpy(), "cell_of": o["cell_of"].cpu().numpy(),
            "status": int(o["status"].item()), "xr": d.xr.cpu().numpy(), "vm": d.vm.cpu().numpy(),
            "uid": d.uid.cpu().numpy(), "x0": d.x0.cpu().numpy()}


def _same(a, b):
    for k in ("nnb", "order", "cell_of", "xr", "vm", "uid", "x0"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    assert a["status"] == b["status"] == 0
    for ra, rb in zip(a["rows"], b["rows"]):
        np.testing.assert_array_equal(ra, rb)


def test_noalloc_build_matches_workspace_build_twice(gpu):
    from taichimps_gb300 import _device, _lib
    from taichimps_gb300.neighbor import morton_rank
    L = _lib.load()
    dom, atom, nl = _system()
    n, slots = atom.nlocal, nl.slots
    ncell = int(np.prod(nl.grid_dim))
    rank = torch.from_numpy(morton_rank(*[int(g) for g in nl.grid_dim])).to(atom.device)
    src = atom.cstruct(atom.buffers)
    st = _device.stream()

    ref = _outputs(atom, n, slots)
    wsb = int(L.tmps_nlist_workspace_bytes(n, ncell))
    ws = torch.zeros(wsb, dtype=torch.uint8, device=atom.device)
    rc = L.tmps_nlist_build(src, atom.cstruct(ref["dst"]), dom.dbox, ncell, 0.1, rank.data_ptr(),
                            ref["order"].data_ptr(), ref["cell_of"].data_ptr(), _nl_struct(ref, n, slots),
                            ws.data_ptr(), wsb, ref["status"].data_ptr(), st)
    assert rc == _lib.TMPS_OK
    torch.cuda.synchronize()
    want = _snapshot(ref, n)
    assert want["nnb"].sum() > 0

    for _ in range(2):
        out = _outputs(atom, n, slots)
        rc = L.tmps_nlist_build_noalloc(src, atom.cstruct(out["dst"]), dom.dbox, ncell, 0.1, rank.data_ptr(),
                                        out["order"].data_ptr(), out["cell_of"].data_ptr(),
                                        _nl_struct(out, n, slots), out["status"].data_ptr(), st)
        assert rc == _lib.TMPS_OK
        torch.cuda.synchronize()
        _same(_snapshot(out, n), want)


def test_noalloc_build_replays_as_a_graph(gpu):
    """After a first direct call (which looks the built-in scratch up), the build can be captured into
    a CUDA graph -- no allocation happens inside it -- and the replay gives the workspace build's output."""
    from taichimps_gb300 import _device, _lib
    from taichimps_gb300.neighbor import morton_rank
    L = _lib.load()
    dom, atom, nl = _system(seed=5)
    n, slots = atom.nlocal, nl.slots
    ncell = int(np.prod(nl.grid_dim))
    rank = torch.from_numpy(morton_rank(*[int(g) for g in nl.grid_dim])).to(atom.device)
    src = atom.cstruct(atom.buffers)
    ref = _outputs(atom, n, slots)
    wsb = int(L.tmps_nlist_workspace_bytes(n, ncell))
    ws = torch.zeros(wsb, dtype=torch.uint8, device=atom.device)
    rc = L.tmps_nlist_build(src, atom.cstruct(ref["dst"]), dom.dbox, ncell, 0.1, rank.data_ptr(),
                            ref["order"].data_ptr(), ref["cell_of"].data_ptr(), _nl_struct(ref, n, slots),
                            ws.data_ptr(), wsb, ref["status"].data_ptr(), _device.stream())
    assert rc == _lib.TMPS_OK
    torch.cuda.synchronize()
    want = _snapshot(ref, n)

    def call(o):
        return L.tmps_nlist_build_noalloc(src, atom.cstruct(o["dst"]), dom.dbox, ncell, 0.1, rank.data_ptr(),
                                          o["order"].data_ptr(), o["cell_of"].data_ptr(), _nl_struct(o, n, slots),
                                          o["status"].data_ptr(), _device.stream())

    first = _outputs(atom, n, slots)
    assert call(first) == _lib.TMPS_OK
    torch.cuda.synchronize()
    out = _outputs(atom, n, slots)
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.graph(g, stream=side):
        rc = call(out)
    torch.cuda.current_stream().wait_stream(side)
    assert rc == _lib.TMPS_OK
    g.replay()
    torch.cuda.synchronize()
    _same(_snapshot(out, n), want)


def test_noalloc_build_refuses_sizes_beyond_its_scratch(gpu):
    """Checked on the host before anything is launched."""
    from taichimps_gb300 import _device, _lib
    L = _lib.load()
    dom, atom, nl = _system(n_side=4)
    n, slots = atom.nlocal, nl.slots
    out = _outputs(atom, n, slots)
    rank = torch.zeros(_lib.NOALLOC_MAX_CELLS + 1, dtype=torch.int32, device=atom.device)
    rc = L.tmps_nlist_build_noalloc(atom.cstruct(), atom.cstruct(out["dst"]), dom.dbox,
                                    _lib.NOALLOC_MAX_CELLS + 1, 0.1, rank.data_ptr(), out["order"].data_ptr(),
                                    out["cell_of"].data_ptr(), _nl_struct(out, n, slots), out["status"].data_ptr(),
                                    _device.stream())
    assert rc == _lib.TMPS_ERR_TOO_LARGE
    big = atom.cstruct()
    big.n = _lib.NOALLOC_MAX_ATOMS + 1
    bdst = atom.cstruct(out["dst"])
    bdst.n = big.n
    bnl = _nl_struct(out, big.n, slots)
    rc = L.tmps_nlist_build_noalloc(big, bdst, dom.dbox, 8, 0.1, rank.data_ptr(), out["order"].data_ptr(),
                                    out["cell_of"].data_ptr(), bnl, out["status"].data_ptr(), _device.stream())
    assert rc == _lib.TMPS_ERR_TOO_LARGE

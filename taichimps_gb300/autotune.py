"""
Launch-shape autotuner for batched runs.

No reference counterpart (the reference runs one system per process and
leaves launch geometry to Taichi).

Each step kernel of a batched run covers every instance in one grid, and an
instance's launch shape (tmps_fused_shape: 32-atom groups per warp of the
update kernel A and of the contact kernel C) sets how many blocks it owns.
The default shape gives a small system one group per warp, so a batch of many
small systems needs many block waves, each block paying its fixed latency
(instance descriptor, engine record, partial sums) for few atoms; more groups
per warp amortise that latency and, in C, put several groups in flight
together (up to kLive), until the last instance's warps run too long.  Where
the balance lies depends on the sizes, the contact density and the GPU, so it
is measured.

The measurement runs A alone and C alone over the batch's current state, once
per candidate shape, with everything the kernel writes -- positions,
velocities and angular velocities (A); forces, torques, contact histories and
touch masks (C); the flag words, partial sums and engine record (both) --
redirected to copies, so the run itself is untouched: a tuned run equals an
untuned run of the shape the tuner picked, bit for bit
(tests/test_gpu_ensemble.py).  The shape changes only the order in which the
virial partials are summed.
"""

from __future__ import annotations

import ctypes

import torch

from . import _device, _lib

CANDIDATES = (1, 2, 4, 8, 16, 32)


def _moved(ptr: int, src: torch.Tensor, dst: torch.Tensor) -> int:
    """The address in `dst` of what `ptr` addresses inside `src` (a same-layout copy)."""
    off = int(ptr) - src.data_ptr()
    if off < 0 or off >= src.numel() * src.element_size():
        raise RuntimeError("autotune: a kernel output is not inside the tensor it was taken from")
    return dst.data_ptr() + off


class _Trial:
    """One instance's descriptor with every output of A and C pointing at a copy (its engine
    record at `rec`, a row of the batch's table of record copies)."""

    def __init__(self, eng, rec: torch.Tensor) -> None:
        sim = eng.sim
        self.eng = eng
        d = eng.instance(0, eng.a_blocks, 0, eng.c_blocks)
        self.keep = []

        def redirect(ptr, t):
            c = t.clone()
            self.keep.append(c)
            return _moved(ptr, t, c)

        b = sim.atom.buffers
        if eng.mixed:
            for name, t in (("pos32", eng.pos32), ("pos32lo", eng.pos32lo), ("vel32", eng.vel32),
                            ("lo32", eng.lo32), ("wlz32", eng.wlz32), ("om32", eng.om32),
                            ("f32", eng.f32), ("torque32", eng.t32)):
                setattr(d.a, name, redirect(getattr(d.a, name), t))
        else:
            for name, t in (("xr", b.xr), ("vm", b.vm), ("om", b.om)):
                setattr(d.a, name, redirect(getattr(d.a, name), t))
        d.a.f = redirect(d.a.f, b.f)
        d.a.torque = redirect(d.a.torque, b.torque)
        h = sim.history
        d.nl.touch = redirect(d.nl.touch, h.touch)
        d.nl.shear = redirect(d.nl.shear, h.shear)
        if d.nl.rolling:
            d.nl.rolling = redirect(d.nl.rolling, h.rolling)
        d.scratch = redirect(d.scratch, eng.part)
        rec.copy_(eng._eng)
        d.eng = rec.data_ptr()
        self.d = d


def _time(launch, reps: int) -> float:
    launch()  # warm-up (first flag words of this shape)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        launch()
    e1.record()
    torch.cuda.synchronize()
    return 1e3 * e0.elapsed_time(e1) / reps


def tune_launch_shape(batched, candidates=CANDIDATES, reps: int = 8) -> dict:
    """Times the batched A and C kernels for each candidate groups-per-warp count on the batch's
    current state (after every engine's begin()); returns {"launch_shape": (a, c), "a_us": {...},
    "c_us": {...}} with microseconds per launch."""
    L = _device.lib()
    st = _device.stream()
    mixed = 1 if batched.mixed else 0
    size = ctypes.sizeof(_lib.Instance)
    esize = ctypes.sizeof(_lib.Engine)
    # every instance's engine record copy, one row each, rows 16-byte aligned
    stride = (esize + 15) // 16 * 16
    recs = torch.zeros((len(batched.engines), stride), dtype=torch.uint8, device=batched.dev)
    trials = [_Trial(e, recs[i, :esize]) for i, e in enumerate(batched.engines)]
    nb_word = _lib.Engine.nblocks.offset // 4
    a_us, c_us = {}, {}
    a_b, c_b = ctypes.c_int32(), ctypes.c_int32()
    tables = {}
    for g in candidates:
        a_map, c_map, blob = [], [], bytearray()
        nblocks = []
        for i, t in enumerate(trials):
            # A and C of the same shape in one descriptor table
            _lib.check(L.tmps_fused_shape(t.eng._n, batched.style, mixed, int(g), int(g), ctypes.byref(a_b),
                                          ctypes.byref(c_b)), "tmps_fused_shape")
            nblocks.append(a_b.value + c_b.value)
            t.d.a_first, t.d.a_blocks, t.d.c_first, t.d.c_blocks = len(a_map), a_b.value, len(c_map), c_b.value
            a_map += [i] * a_b.value
            c_map += [i] * c_b.value
            blob += ctypes.string_at(ctypes.addressof(t.d), size)
        tables[int(g)] = (torch.frombuffer(blob, dtype=torch.uint8).to(batched.dev),
                          torch.tensor(a_map, dtype=torch.int32, device=batched.dev),
                          torch.tensor(c_map, dtype=torch.int32, device=batched.dev), nblocks)

    def shape(g):
        d_inst, d_a, d_c, nblocks = tables[g]
        # the partial layout of this shape, in every record copy at once
        recs.view(torch.int32)[:, nb_word] = torch.tensor(nblocks, dtype=torch.int32).to(batched.dev)
        return d_inst, d_a, d_c

    # C first: its trials move no atom, so A's trials (which do, in the copies) cannot trip the
    # skin check C's trials look at
    for g in tables:
        d_inst, _, d_c = shape(g)
        c_us[g] = _time(lambda: _lib.check(L.tmps_batch_c(d_inst.data_ptr(), d_c.data_ptr(), d_c.numel(),
                                                          batched.style, mixed, st), "tmps_batch_c"), reps)
    for g in tables:
        d_inst, d_a, _ = shape(g)
        a_us[g] = _time(lambda: _lib.check(L.tmps_batch_a(d_inst.data_ptr(), d_a.data_ptr(), d_a.numel(), mixed,
                                                          st), "tmps_batch_a"), reps)
    del trials, recs
    best_a = min(a_us, key=lambda k: (a_us[k], k))
    best_c = min(c_us, key=lambda k: (c_us[k], k))
    return {"launch_shape": (best_a, best_c), "a_us": a_us, "c_us": c_us}

"""
Batched runs: many independent systems advanced together.

No reference counterpart -- the reference runs one system per process.  Each
instance is an ordinary ``Simulation`` (its own box, atoms, list, history,
pair coefficients, servo) with its own ``FusedEngine`` state; ``BatchedEngine``
advances all of them with one launch of each of the three step kernels per
step (tmps_batch_a / tmps_batch_c / tmps_batch_servo), captured in chunks as a
CUDA graph.  Every block of a batched grid belongs to one instance and runs
that instance's single-instance arithmetic with the block index it would have
in a single-instance launch of the same launch shape (tmps_fused_shape), so a
batched step is bit-identical to the instance's own fused step of that shape.
The shape -- how many 32-atom groups each warp of the update and contact
kernels takes -- is picked by the autotuner (autotune.py) unless given.

When an instance's skin check asks for a rebuild, that instance alone stops
(its later launches return at once); between chunks the host rebuilds it
exactly as a single run does, finishes its step, updates its descriptor and
lets it catch up while instances that reached the target step idle.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _device, _lib
from .engine import FusedEngine, fusable


class BatchedEngine:
    def __init__(self, sims, precision: str = "mixed", chunk: int = 64, graphs: bool = True,
                 cull: bool = True, launch_shape: tuple[int, int] | str = "auto") -> None:
        if not sims:
            raise ValueError("a batched run needs at least one Simulation")
        styles = {int(s.pair_style.params.style) for s in sims}
        if len(styles) != 1:
            raise ValueError("every instance of a batched run uses the same pair style")
        for s in sims:
            if not fusable(s):
                raise NotImplementedError("batched runs cover fix nve/sphere + optional damping/cundall and "
                                          "deform/pressure")
        self.sims = list(sims)
        self.precision = precision
        self.mixed = precision == "mixed"
        self.style = styles.pop()
        self.chunk = int(chunk)
        self.graphs = bool(graphs)
        # launch shape of every instance (tmps_fused_shape: groups per warp of A and of C); "auto":
        # measured by the autotuner (autotune.py) at the start of the first run
        self._tune = isinstance(launch_shape, str)
        if self._tune and launch_shape != "auto":
            raise ValueError("launch_shape is 'auto' or (a_groups_per_warp, c_groups_per_warp)")
        self.launch_shape = (0, 0) if self._tune else (int(launch_shape[0]), int(launch_shape[1]))
        self.tuning = None
        # the batched C (tmps_batch_c) runs the screened path for every instance
        self.engines = [FusedEngine(s, precision, chunk=chunk, graphs=False, cull=cull,
                                    launch_shape=self.launch_shape, contact_path="screened") for s in self.sims]
        self.dev = _device.device()
        self.status = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self._graph = None
        self.rebuilds = 0
        self.graph_replays = 0

    # ---------------------------------------------------------------- tables

    def _tables(self) -> None:
        ninst = len(self.engines)
        self._a_first, self._a_blocks, self._c_first, self._c_blocks = [], [], [], []
        a_inst, c_inst = [], []
        for i, e in enumerate(self.engines):
            # each instance owns the grids its own single run of the same launch shape uses
            self._a_first.append(len(a_inst))
            self._c_first.append(len(c_inst))
            self._a_blocks.append(e.a_blocks)
            self._c_blocks.append(e.c_blocks)
            a_inst += [i] * e.a_blocks
            c_inst += [i] * e.c_blocks
        i32 = dict(dtype=torch.int32, device=self.dev)
        self.a_inst = torch.tensor(a_inst, **i32)
        self.c_inst = torch.tensor(c_inst, **i32)
        self.d_inst = torch.zeros(ninst * ctypes.sizeof(_lib.Instance), dtype=torch.uint8, device=self.dev)
        for i in range(ninst):
            self._push(i)
        self.state = torch.zeros(2 * ninst, dtype=torch.int64, device=self.dev)

    def _push(self, i: int) -> None:
        """Write instance i's current descriptor (buffers move at every rebuild)."""
        d = self.engines[i].instance(self._a_first[i], self._a_blocks[i], self._c_first[i], self._c_blocks[i])
        size = ctypes.sizeof(_lib.Instance)
        host = torch.frombuffer(bytearray(ctypes.string_at(ctypes.addressof(d), size)), dtype=torch.uint8)
        self.d_inst[i * size:(i + 1) * size].copy_(host)

    # ---------------------------------------------------------------- steps

    def _launch_step(self, L, st) -> None:
        mixed = 1 if self.mixed else 0
        _lib.check(L.tmps_batch_a(self.d_inst.data_ptr(), self.a_inst.data_ptr(), len(self.a_inst), mixed, st),
                   "tmps_batch_a")
        _lib.check(L.tmps_batch_c(self.d_inst.data_ptr(), self.c_inst.data_ptr(), len(self.c_inst), self.style,
                                  mixed, st), "tmps_batch_c")
        _lib.check(L.tmps_batch_servo(self.d_inst.data_ptr(), len(self.engines), self.status.data_ptr(), st),
                   "tmps_batch_servo")

    def _chunk(self, L) -> None:
        if not self.graphs:
            st = _device.stream()
            for _ in range(self.chunk):
                self._launch_step(L, st)
            return
        if self._graph is None:
            def chunk():
                st = _device.stream()
                for _ in range(self.chunk):
                    self._launch_step(L, st)

            self._graph = _device.capture_graph(chunk)
        self._graph.replay()
        self.graph_replays += 1

    def run(self, nsteps: int) -> None:
        """Advance every instance by `nsteps` steps (Simulation.run of each, batched)."""
        L = _device.lib()
        targets = []
        for s, e in zip(self.sims, self.engines):
            s.setup_run(nsteps)
            if s.run_pre or not s.setup_done:
                s.init_simulation()
            targets.append(s.timestep + int(nsteps))
            e.begin(stop_step=targets[-1])
        targets = np.array(targets, dtype=np.int64)
        self.status.zero_()
        if self._tune:
            from .autotune import tune_launch_shape
            self.tuning = tune_launch_shape(self)
            self.launch_shape = self.tuning["launch_shape"]
            for e in self.engines:
                e.set_launch_shape(self.launch_shape)
            self._tune = False
        self._tables()
        try:
            while True:
                _lib.check(L.tmps_batch_state(self.d_inst.data_ptr(), len(self.engines), self.state.data_ptr(),
                                              _device.stream()), "tmps_batch_state")
                st = self.state.cpu().numpy().reshape(-1, 2)
                steps = st[:, 0].copy()
                for i in np.nonzero(st[:, 1])[0]:
                    self.engines[i]._rebuild_step(int(steps[i]) + 1)
                    self.rebuilds += 1
                    steps[i] += 1
                    self._push(int(i))
                self._check_status()
                if (steps >= targets).all():
                    break
                self._chunk(L)
        finally:
            for s, e in zip(self.sims, self.engines):
                e.finish()
                s.check_device_status()
                s.domain.pull()
            self._graph = None

    def _check_status(self) -> None:
        if int(self.status.item()) & _lib.STATUS_BOX_NONPOSITIVE:
            bad = []
            for i, s in enumerate(self.sims):
                s.domain.mark_device_authoritative()
                s.domain.pull()
                if np.any(np.asarray(s.domain.prd) <= 0):
                    bad.append(i)
            raise RuntimeError(f"fix deform/pressure drove a box dimension non-positive in instance(s) {bad}")

"""
The fused step engine behind ``Simulation.run``.

One step of Simulation._sub_step_inner (simulation.py:205-247) with fix
nve/sphere, optionally damping/cundall and deform/pressure, becomes three
kernels (tmps_fused_a, tmps_fused_c, tmps_fused_servo) that decide on the
device whether the step needs a neighbor rebuild.  Steps are queued in
chunks (replayed as CUDA graphs) with one host synchronisation per chunk.
When a step finds it needs a rebuild, every later launch of the chunk does
nothing; the host then rebuilds exactly as the reference does at that step
(save history, wrap, build, restore history), finishes the step, and
carries on.

Two precisions:
  "fp64"  every operation FP64 (the plain FP64 form);
  "mixed" FP32 contact arithmetic and per-atom force accumulation;
          positions (offsets from each atom's cell origin), velocities and
          angular velocities as double-word FP32 (hi + lo, ~48 bits) updated
          with error-free transforms; the contact histories as double words
          too while the run lasts (doubles before a rebuild carries them over
          and at the end); virial partials as double words, their totals --
          what the servo reads -- in FP64.
"""

from __future__ import annotations

import ctypes
import weakref

import numpy as np
import torch

from . import _device, _lib
from .EXTRA_FIX.damping_cundall import FixDampingCundall
from .EXTRA_FIX.deform_pressure import FixDeformPressure


def fusable(sim) -> bool:
    """The configurations the fused step covers."""
    if sim.integrator is None or sim.pair_style is None or sim.neighbor is None or sim.history is None:
        return False
    kinds = [type(f) for f in sim.fixes]
    if any(k not in (FixDampingCundall, FixDeformPressure) for k in kinds):
        return False
    if kinds.count(FixDampingCundall) > 1 or kinds.count(FixDeformPressure) > 1:
        return False
    # damping must act on the pair force before the servo reads the virial: the
    # reference calls post_force hooks (Cundall) and end_of_step hooks (servo) in
    # that order regardless of insertion order, so any order is fine here.
    return True


class FusedEngine:
    # kernels per step: A, C, S
    LAUNCHES_PER_STEP = 3

    def __init__(self, sim, precision: str = "fp64", chunk: int = 64, graphs: bool = True,
                 cull: bool = True, launch_shape: tuple[int, int] | None = None,
                 contact_path: str | None = None) -> None:
        if precision not in ("fp64", "mixed"):
            raise ValueError("precision must be 'fp64' or 'mixed'")
        if contact_path is None:
            contact_path = getattr(sim, "contact_path", "auto")
        if contact_path not in ("auto", "screened", "rows"):
            raise ValueError("contact_path must be 'auto', 'screened' or 'rows'")
        # the Simulation keeps its last engine (Simulation.last_engine); the engine refers back
        # weakly, so a finished run's device memory goes with the Simulation instead of waiting
        # for the cycle collector
        self._sim = weakref.ref(sim)
        self.precision = precision
        self.mixed = precision == "mixed"
        self.chunk = int(chunk)
        self.dev = _device.device()
        self.cundall = next((f for f in sim.fixes if isinstance(f, FixDampingCundall)), None)
        self.deform = next((f for f in sim.fixes if isinstance(f, FixDeformPressure)), None)
        self._eng = _device.struct_buffer(_lib.Engine())
        self.status = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self._dummy_servo = _device.struct_buffer(_lib.Servo())
        self._n = -1
        self.rebuilds = 0
        # A chunk of `chunk` steps is captured once as a CUDA graph and replayed;
        # a rebuild swaps buffers, so the graph is captured again after one.
        self.graphs = bool(graphs)
        # C skips 32-atom groups whose gap bound rules out any contact (exact;
        # off screens every group, with bit-identical results)
        self.cull = bool(cull)
        # C's path (tmps_fused_c): "screened" rules contact-free 32-atom groups out and runs the contacts
        # of the rest 32 at a time; "rows" runs every atom's row, one thread per atom; "auto" picks rows
        # for the mixed form at a build where more than half of the atoms touch or overlap at the build
        # positions (their gap bound is <= 0), screened otherwise (the FP64 form's screened path was
        # measured faster on contact-dense states too).  Both paths sum each atom's contacts in slot
        # order with the same per-contact code; only the order of the virial partial sums differs.
        self.contact_path = contact_path
        self.rows = contact_path == "rows"
        # launch shape (tmps_fused_shape): 32-atom groups per warp of A and of C, 0 = the default grid;
        # it fixes the order of the virial sum, so equal shapes give bit-identical runs
        shape = getattr(sim, "launch_shape", (0, 0)) if launch_shape is None else launch_shape
        self.launch_shape = (int(shape[0]), int(shape[1]))
        self._graph = None
        self._graph_key = None
        # the arguments of the last chunk that ran as plain launches; the next chunk with the same
        # arguments is captured (`capture_first`: capture at the first chunk instead)
        self._seen_key = None
        self.capture_first = False
        self._hist_dw = False
        self.graph_replays = 0
        self.graph_kernel_launches = 0
        # (engine record, status) as the last run() left them, while nothing has been launched since:
        # the next run() starts from it instead of another synchronisation
        self._known = None

    @property
    def sim(self):
        sim = self._sim()
        if sim is None:
            raise RuntimeError("the Simulation of this fused engine no longer exists")
        return sim

    # ------------------------------------------------------------ storage

    def _alloc(self, n: int) -> None:
        if n == self._n:
            return
        # every per-atom array here is written in full by tmps_fused_prepare before any kernel reads
        # it: left unset, in one allocation for the mixed form's eleven
        self.rinv = None if self.mixed else torch.empty((2, n), dtype=torch.float64, device=self.dev)
        style, mixed = int(self.sim.pair_style.params.style), 1 if self.mixed else 0
        self._shape(n)
        self.part = torch.zeros(int(_device.lib().tmps_fused_scratch_bytes(n, style, mixed)), dtype=torch.uint8,
                                device=self.dev)
        if self.mixed:
            # (name, FP32 words per atom, shape); each slice starts on a 256-byte boundary
            parts = [("pos32", 4, (n, 4)), ("pos32lo", 4, (n, 4)), ("lo32", 4, (n, 4)), ("wlz32", 1, (n,)),
                     ("inv32", 2, (n, 2)), ("vel32", 4, (n, 4)), ("om32", 4, (n, 4)), ("f32", 3, (3, n)),
                     ("t32", 3, (3, n)), ("o0", 3, (3, n)), ("cell32", 1, (n,))]
            r64 = lambda w: (w + 63) // 64 * 64
            flat = torch.empty(sum(r64(w * n) for _, w, _ in parts), dtype=torch.float32, device=self.dev)
            off = 0
            for name, w, shape in parts:
                t = flat[off:off + w * n].view(shape)
                setattr(self, name, t.view(torch.int32) if name == "cell32" else t)
                off += r64(w * n)
        self._n = n

    def _shape(self, n: int) -> None:
        """Grids of A and C for n atoms under this engine's launch shape; nblocks = virial partials."""
        a_b, c_b = ctypes.c_int32(), ctypes.c_int32()
        style, mixed = int(self.sim.pair_style.params.style), 1 if self.mixed else 0
        _lib.check(_device.lib().tmps_fused_shape(n, style, mixed, self.launch_shape[0], self.launch_shape[1],
                                                  ctypes.byref(a_b), ctypes.byref(c_b)), "tmps_fused_shape")
        self.a_blocks, self.c_blocks = a_b.value, c_b.value
        self.nblocks = self.a_blocks + self.c_blocks

    def set_launch_shape(self, shape: tuple[int, int]) -> None:
        """Change the launch shape between steps (the scratch holds any shape's partials)."""
        self._known = None
        self.launch_shape = (int(shape[0]), int(shape[1]))
        if self._n < 0:
            return
        self._shape(self._n)
        e = self._engine_state()
        e.nblocks = self.nblocks
        _device.push_struct(self._eng, e)
        self._graph = None

    def atoms(self) -> _lib.Atoms:
        s = self.sim.atom.cstruct()
        s.rinv = None if self.rinv is None else self.rinv.data_ptr()
        if self.mixed:
            s.pos32, s.vel32, s.om32 = self.pos32.data_ptr(), self.vel32.data_ptr(), self.om32.data_ptr()
            s.f32, s.torque32, s.o0_32 = self.f32.data_ptr(), self.t32.data_ptr(), self.o0.data_ptr()
            s.cell32 = self.cell32.data_ptr()
            s.pos32lo = self.pos32lo.data_ptr()
            s.lo32, s.wlz32, s.inv32 = self.lo32.data_ptr(), self.wlz32.data_ptr(), self.inv32.data_ptr()
        return s

    def _servo_ptr(self) -> int:
        return self.deform._dservo.data_ptr() if self.deform is not None else self._dummy_servo.data_ptr()

    # ------------------------------------------------------------ lifecycle

    def begin(self, stop_step: int | None = None) -> None:
        """After Simulation.init_simulation(): hand the state to the fused step.  `stop_step`: fused
        launches do nothing once the step count reaches it (batched runs)."""
        self._known = None
        sim = self.sim
        atom, nl = sim.atom, sim.neighbor
        n = atom.nlocal
        self._alloc(n)
        if sim.pair_style.params.rolling_id:
            sim.history.enable_rolling()
        if self.mixed:
            g = nl.grid_dim
            if np.any(g > 1023):
                raise NotImplementedError("the mixed form packs cell coordinates in 10 bits (<= 1023 bins per axis)")
        e = _lib.Engine()
        e.step = sim.timestep
        e.last_build_step = nl.last_build_step
        e.delay, e.every, e.check = int(nl.delay), max(1, int(nl.every)), 1 if nl.check else 0
        e.cundall = 1 if self.cundall is not None else 0
        e.servo = 1 if self.deform is not None else 0
        e.mixed = 1 if self.mixed else 0
        e.nblocks = self.nblocks
        e.dt = float(sim.dt)
        if self.cundall is not None:
            e.gamma_lin, e.gamma_ang = self.cundall.gamma_lin, self.cundall.gamma_ang
        e.trigger_sq = 0.25 * nl.skin * nl.skin
        e.remap_scale[0] = e.remap_scale[1] = e.remap_scale[2] = 1.0
        e.stop_step = (1 << 62) if stop_step is None else int(stop_step)
        _device.push_struct(self._eng, e)
        if self.deform is not None:
            # the run counters only; the rest of the servo record stays as the device has it
            fx = self.deform
            sv = _lib.Servo()
            sv.nsteps, sv.nsteps_total, sv.step_count, sv.nevery = fx.nsteps, fx.nsteps_total, fx.step_count, fx.nevery
            _device.push_fields(fx._dservo, sv, "nsteps", "nevery")
        self._prepare()
        log = self.deform.pressure_log if self.deform is not None else None
        rc = _device.lib().tmps_fused_pressure_log(self._eng.data_ptr(), None if log is None else log.data_ptr(),
                                                   0 if log is None else len(log), _device.stream())
        _lib.check(rc, "tmps_fused_pressure_log")
        # (the mixed form's first half-kick takes the setup forces, which tmps_fused_prepare copied
        # into f32, t32)
        self.status.zero_()
        # the record as pushed above, in the fields run() reads (step, aborted), and a clear status:
        # the first run() starts without a synchronisation
        self._known = (e, 0)

    def _prepare(self) -> None:
        """Split state and per-step constants for the current list, then the per-group
        contact bounds C uses to skip groups that cannot touch."""
        self._known = None
        sim = self.sim
        nl = sim.neighbor
        L, st = _device.lib(), _device.stream()
        atoms = self.atoms()
        rc = L.tmps_fused_prepare(atoms, sim.domain.dbox, self._eng.data_ptr(), nl.cell_of.data_ptr(), st)
        _lib.check(rc, "tmps_fused_prepare")
        rc = L.tmps_fused_bounds(atoms, sim.history.cstruct(nl), sim.domain.dbox, self._eng.data_ptr(),
                                 sim.pair_style.params, 1 if self.cull else 0, self.part.data_ptr(), st)
        _lib.check(rc, "tmps_fused_bounds")
        # one synchronisation for what the host needs before the steps: the count of touching atoms
        # (the contact path) and the status of a neighbor build that did not wait for the device
        auto_rows = self.contact_path == "auto" and self.mixed
        items = []
        if auto_rows:
            off = _lib.Engine.touching.offset
            items.append((self._eng[off:off + 4], None))
        if nl.status_pending:
            items.append((nl.status, None))
        got = _device.pull_many(items) if items else []
        if nl.status_pending:
            nl.check_status(int(got[-1].view(np.int32)[0]))
        if self.contact_path == "auto" and not self.mixed:
            self.rows = False
        elif auto_rows:
            # the bounds kernel counted the atoms whose gap bound is <= 0 into the engine record
            touching = int(got[0].view(np.int32)[0])
            self.rows = self._n > 0 and touching * 2 > self._n
        self._history_form(True)

    def _history_form(self, dw: bool) -> None:
        """The mixed form keeps the contact histories as FP32 double words while it runs, and
        hands them back as doubles (before a rebuild carries them over, and at the end)."""
        if not self.mixed or self._hist_dw == dw:
            return
        sim = self.sim
        rc = _device.lib().tmps_mixed_history(sim.history.cstruct(sim.neighbor), 1 if dw else 0, _device.stream())
        _lib.check(rc, "tmps_mixed_history")
        self._hist_dw = dw

    def _launch_step(self, L, st, atoms, nl_struct, params) -> None:
        self._known = None
        dbox, eng = self.sim.domain.dbox, self._eng.data_ptr()
        with _device.timed("fused_a"):
            rc = L.tmps_fused_a(atoms, dbox, eng, self.a_blocks, self.part.data_ptr(), st)
        _lib.check(rc, "tmps_fused_a")
        with _device.timed("fused_c"):
            rc = L.tmps_fused_c(atoms, nl_struct, dbox, eng, params, self.c_blocks, self.part.data_ptr(),
                                1 if self.rows else 0, st)
        _lib.check(rc, "tmps_fused_c")
        with _device.timed("fused_s"):
            rc = L.tmps_fused_servo(dbox, self._servo_ptr(), eng, self.part.data_ptr(), self.status.data_ptr(), st)
        _lib.check(rc, "tmps_fused_servo")

    def instance(self, a_first: int, a_blocks: int, c_first: int, c_blocks: int) -> _lib.Instance:
        """This system's descriptor for a batched run (tmps_instance)."""
        sim = self.sim
        d = _lib.Instance()
        d.a = self.atoms()
        d.nl = sim.history.cstruct(sim.neighbor)
        d.p = sim.pair_style.params
        d.box = sim.domain.dbox
        d.eng = self._eng.data_ptr()
        d.servo = self._servo_ptr()
        d.scratch = self.part.data_ptr()
        d.a_first, d.a_blocks, d.c_first, d.c_blocks = a_first, a_blocks, c_first, c_blocks
        return d

    def _engine_state(self) -> _lib.Engine:
        return _device.pull_struct(self._eng, _lib.Engine)

    def _engine_and_status(self) -> tuple[_lib.Engine, int]:
        """The engine record and the status word with one synchronisation (two copies into
        page-locked memory)."""
        nbytes = self._eng.numel()
        if getattr(self, "_pull_host", None) is None or self._pull_host.numel() != nbytes + 4:
            self._pull_host = torch.empty(nbytes + 4, dtype=torch.uint8, pin_memory=True)
        h = self._pull_host
        h[:nbytes].copy_(self._eng, non_blocking=True)
        h[nbytes:].copy_(self.status.view(torch.uint8), non_blocking=True)
        torch.cuda.current_stream().synchronize()
        raw = h.numpy()
        return _lib.Engine.from_buffer_copy(raw[:nbytes].tobytes()), int(raw[nbytes:].view(np.int32)[0])

    def run(self, nsteps: int) -> None:
        """Advance `nsteps` steps."""
        sim = self.sim
        L = _device.lib()
        st = _device.stream()
        start = sim.timestep
        target = start + int(nsteps)
        while True:
            if self._known is not None:
                e, status = self._known
                self._known = None
            else:
                e, status = self._engine_and_status()  # after a chunk: its status too, in the same copy
            self._check_status(status)
            done = int(e.step)
            if e.aborted:
                self._rebuild_step(done + 1)
                continue
            if done >= target:
                self._known = (e, status)
                break
            count = min(self.chunk, target - done)
            if self.graphs and count == self.chunk and _device.TIMED is None:
                self._replay_chunk(L)
            else:
                atoms = self.atoms()
                nl_struct = sim.history.cstruct(sim.neighbor)
                params = sim.pair_style.params
                for _ in range(count):
                    self._launch_step(L, st, atoms, nl_struct, params)
        sim.timestep = target

    def _replay_chunk(self, L) -> None:
        """One chunk of steps as a CUDA graph (captured on first use and after a rebuild; the launch
        arguments are built only for a capture)."""
        self._known = None
        sim = self.sim
        key = (sim.neighbor.build_count, sim.atom.buffers.xr.data_ptr(), sim.history.touch.data_ptr(),
               sim.neighbor.nbr.data_ptr(), self.rows, self.chunk)
        if self._graph is None or self._graph_key != key:
            self._graph = None
            atoms = self.atoms()
            nl_struct = sim.history.cstruct(sim.neighbor)
            params = sim.pair_style.params
            if self._seen_key != key and not self.capture_first:
                # a chunk whose arguments have not been seen before runs as plain launches: the device
                # starts on it at once, where a capture would hold it idle, and a run of one chunk
                # (or one chunk between rebuilds) never pays for a graph it would replay once
                self._seen_key = key
                st = _device.stream()
                for _ in range(self.chunk):
                    self._launch_step(L, st, atoms, nl_struct, params)
                return

            def chunk():
                st = _device.stream()
                for _ in range(self.chunk):
                    self._launch_step(L, st, atoms, nl_struct, params)

            self._graph, self._graph_key = _device.capture_graph(chunk), key
        self._graph.replay()
        self.graph_replays += 1
        self.graph_kernel_launches += self.chunk * self.LAUNCHES_PER_STEP

    def cull_stats(self) -> tuple[int, int]:
        """(32-atom groups, groups the contact bound rules out right now), from the
        device state.  No reference counterpart; for reports and tests."""
        n = self._n
        ng = (n + 31) // 32
        e = self._engine_state()
        if not e.cull or ng == 0:
            return ng, 0
        # scratch layout: flag words (ng + 1, 256-byte aligned), then the gaps
        off = ((ng + 1) * 4 + 255) // 256 * 256
        gap = self.part[off:off + 4 * ng].view(torch.float32).cpu().numpy()
        f32 = np.float32
        md = np.sqrt(np.array([e.maxd2_bits], dtype=np.uint32).view(np.float32)[0])
        thr = (f32(2.0) * md) * f32(1.0001) + f32(e.shift_bound) + f32(e.cull_tol)
        return ng, int(np.count_nonzero(gap > thr))

    def flagged_count(self) -> int:
        """Atoms C flagged (some neighbor within reach of contact) in the last step, from the flag
        words.  No reference counterpart; for reports and tests."""
        ng = (self._n + 31) // 32
        if ng == 0:
            return 0
        w = self.part[:4 * ng].view(torch.int32).cpu().numpy().view(np.uint32)
        return int(np.unpackbits(w.view(np.uint8)).sum())

    def _check_status(self, st: int | None = None) -> None:
        st = int(self.status.item()) if st is None else st
        if st & _lib.STATUS_BOX_NONPOSITIVE and self.deform is not None:
            self.deform.status.fill_(st)
            self.deform.status_clean = False
            self.deform.check_status()

    def _rebuild_step(self, s: int) -> None:
        """Step `s` has had its first half-kick and drift; rebuild, then finish it."""
        self._known = None
        sim = self.sim
        L = _device.lib()
        st = _device.stream()
        atom, nl = sim.atom, sim.neighbor
        self.rebuilds += 1
        sim.timestep = s
        nl.current_step = s
        if self.mixed:
            _lib.check(L.tmps_mixed_unpack(self.atoms(), sim.domain.dbox, st), "tmps_mixed_unpack")
        self._history_form(False)
        sim.domain.mark_device_authoritative()
        sim.domain.pull()
        sim.history.save_state(atom, nl)
        sim.domain.pbc(atom)
        nl.build(atom, defer_check=True)  # its status is read with the engine's next pull
        sim.history.restore_state(atom, nl)
        e = self._engine_state()
        e.aborted = 0
        e.disp_stamp = 0
        e.last_build_step = s
        _device.push_struct(self._eng, e)
        if atom.nlocal != self._n:
            raise RuntimeError("atom count changed during a fused run")
        self._prepare()
        atoms = self.atoms()
        nl_struct = sim.history.cstruct(nl)
        dbox, eng = sim.domain.dbox, self._eng.data_ptr()
        _lib.check(L.tmps_fused_c(atoms, nl_struct, dbox, eng, sim.pair_style.params, self.c_blocks,
                                  self.part.data_ptr(), 1 if self.rows else 0, st), "tmps_fused_c")
        _lib.check(L.tmps_fused_servo(dbox, self._servo_ptr(), eng, self.part.data_ptr(), self.status.data_ptr(),
                                      st), "tmps_fused_servo")

    def finish(self) -> None:
        """Settle pending updates and hand the state back to the per-hook path."""
        self._known = None
        # the captured graph goes now, not whenever the engine is collected (which may be
        # during a later capture)
        self._graph = self._graph_key = None
        sim = self.sim
        L = _device.lib()
        st = _device.stream()
        atoms = self.atoms()
        _lib.check(L.tmps_fused_settle(atoms, sim.domain.dbox, self._eng.data_ptr(), st), "tmps_fused_settle")
        if self.mixed:
            _lib.check(L.tmps_mixed_unpack(atoms, sim.domain.dbox, st), "tmps_mixed_unpack")
        self._history_form(False)
        sim.domain.mark_device_authoritative()
        # the engine record, the status word, the box and the servo record: one synchronisation
        items = [(self._eng, _lib.Engine), (self.status, None), (sim.domain.dbox_tensor, _lib.Box)]
        if self.deform is not None:
            items.append((self.deform._dservo, _lib.Servo))
        got = _device.pull_many(items)
        e, status, box = got[0], int(got[1].view(np.int32)[0]), got[2]
        sim.domain.take_pulled(box)
        sim.timestep = int(e.step)
        sim.neighbor.current_step = int(e.step)
        sim.neighbor.last_build_step = int(e.last_build_step)
        for fx in sim.fixes:
            fx.timestep = sim.timestep
        if self.deform is not None:
            sv = got[3]
            self.deform.nsteps, self.deform.step_count = int(sv.nsteps), int(sv.step_count)
        if sim.integrator is not None:
            sim.integrator.timestep = sim.timestep
        self._check_status(status)

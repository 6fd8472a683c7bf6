"""
The step orchestrator: LAMMPS Verlet order over the GB300 kernels.

Mirrors taichimps ``Simulation`` (src/taichimps/simulation.py:21-332) -- the
same constructor, hooks and step order:

  1. fix nve/sphere initial_integrate
  2. reneighbor if needed (save history -> pbc -> build -> restore history)
  3. clear forces                   } one kernel: the contact kernel writes
  4. pair compute                   } f / torque / virial instead of adding
  5. fix post_force (Cundall damping ...)
  6. fix nve/sphere final_integrate
  7. fix end_of_step (deform/pressure servo ...)

The setup force evaluation at the start of every run uses shearupdate=False
(simulation.py:170-203).  Device-side errors (a box driven non-positive, a
neighbor overflow) are raised at synchronisation points: rebuilds and the
end of a run.
"""

from __future__ import annotations

from typing import Any

from .atom import AtomSystem
from .computes.thermo import Computes
from .contact_history import ContactHistory
from .EXTRA_FIX.base import Fix
from .EXTRA_FIX.nve_sphere import FixNVESphere
from .GRANULAR.base import GranularPair
from .neighbor import NeighborList


class Simulation:
    def __init__(self, domain, atom: AtomSystem | None = None, neighbor: NeighborList | None = None,
                 history: ContactHistory | None = None, pair: GranularPair | None = None,
                 max_atoms: int = 100000, max_neighbors_per_atom: int = 64, skin: float = 0.001,
                 dt: float = 1e-4, thermo_freq: int = 100, float_type: Any = None,
                 precision: str = "fp64", fused: bool = True) -> None:
        self.domain = domain
        # run() executes supported configurations through the fused step
        # (engine.py); `precision` picks its arithmetic ("fp64" or "mixed").
        self.precision = precision
        self.fused = fused
        # launch shape of the fused step (tmps_fused_shape): 32-atom groups
        # per warp of its update and contact kernels, 0 = the default grids
        self.launch_shape = (0, 0)
        # path of the fused step's contact kernel (FusedEngine): "auto" (by the
        # packing at each build), "screened" or "rows"
        self.contact_path = "auto"
        self.last_engine = None
        self.dt = dt
        self.float_type = float_type
        self.timestep = 0
        self.atom = atom if atom is not None else AtomSystem(max_atoms=max_atoms, float_type=float_type)
        self.neighbor = neighbor if neighbor is not None else NeighborList(
            domain=domain, max_atoms=max_atoms, max_neighbors_per_atom=max_neighbors_per_atom, skin=skin,
            float_type=float_type)
        self.history = history if history is not None else ContactHistory(
            max_atoms=max_atoms, max_neighbors=max_neighbors_per_atom, float_type=float_type)
        self.pair_style: GranularPair | None = pair
        self.integrator: FixNVESphere | None = None
        self.fixes: list[Fix] = []
        self.dumps: list = []
        self.restart_every = 0
        self.restart_file = None
        self.restart_writer = None
        self.setup_done = False
        self.run_pre = True
        self.thermo_freq = thermo_freq
        self.computes = Computes(float_type=float_type)

    def add_dump(self, dump, freq: int = 100) -> None:
        raise NotImplementedError("dump output is outside the GB300 contact path")

    def set_restart(self, every: int, path, writer=None) -> None:
        """Periodic restart output, `restart N file` (simulation.py:86-90): run() writes one every `every`
        steps through writer(path with the step for a `*`, step).  With no writer, the file is a LAMMPS
        restart of this system written by taichimps_gb300.restart.write_restart (atoms, box, pair style
        and the contact history)."""
        self.restart_every = int(every)
        self.restart_file = None if path is None else str(path)
        self.restart_writer = writer

    def write_restart_now(self) -> None:
        """Write one periodic restart file for the current step (simulation.py:92-98)."""
        if not self.restart_file:
            return
        path = self.restart_file.replace("*", str(self.timestep))
        if self.restart_writer is not None:
            self.restart_writer(path, self.timestep)
            return
        from .restart import write_restart
        write_restart(path, self.atom, self.domain, timestep=self.timestep, dt=self.dt, history=self.history,
                      pair=self.pair_style, nlist=self.neighbor if self.neighbor.has_built else None)

    def set_pair_style(self, pair: GranularPair) -> None:
        self.pair_style = pair

    def add_fix(self, fix: Fix) -> None:
        if isinstance(fix, FixNVESphere):
            self.integrator = fix
        else:
            self.fixes.append(fix)

    def remove_fix(self, fix: Fix) -> None:
        if fix in self.fixes:
            self.fixes.remove(fix)
        elif self.integrator is fix:
            self.integrator = None

    def check_device_status(self) -> None:
        if self.neighbor is not None:
            self.neighbor.check_status()
        for fix in self.fixes:
            fix.check_status()

    def reneighbor_if_needed(self, force: bool = False) -> bool:
        """simulation.py:122-159: save -> pbc -> pull -> build -> restore."""
        if self.neighbor is None:
            return False
        forced = force
        for fix in self.fixes:
            if fix.force_reneighbor:
                forced = True
                fix.force_reneighbor = False
        if not self.neighbor.decide(self.atom, self.timestep) and not forced:
            return False
        self.check_device_status()
        if self.history is not None:
            self.history.save_state(self.atom, self.neighbor)
        self.domain.pbc(self.atom)
        self.domain.pull()
        # the build's status is read at the next synchronisation (NeighborList.check_status), so the
        # host goes on queueing the steps after it while the device builds
        self.neighbor.build(self.atom, defer_check=True)
        if self.history is not None:
            self.history.restore_state(self.atom, self.neighbor)
        return True

    def setup_run(self, nsteps_total: int) -> None:
        for fix in self.fixes:
            if hasattr(fix, "note_atom_count"):
                fix.note_atom_count(self.atom.nlocal)
            fix.setup(nsteps_total, self.dt)
        if self.integrator is not None:
            self.integrator.setup(nsteps_total, self.dt)

    def init_simulation(self) -> None:
        """Verlet::setup(): rebuild and evaluate forces without advancing history."""
        self.setup_done = True
        self.atom.clear_forces()
        if self.pair_style is not None:
            self.reneighbor_if_needed(force=True)
            self.pair_style.compute(self.atom, self.neighbor, self.history, self.dt, shearupdate=False)
        for fix in self.fixes:
            fix.history_update = False
        for fix in self.fixes:
            fix.post_force(self.atom, self.dt)
        for fix in self.fixes:
            fix.history_update = True

    def _sub_step_inner(self) -> None:
        self.timestep += 1
        for fix in self.fixes:
            fix.timestep = self.timestep
        if self.integrator is not None:
            self.integrator.timestep = self.timestep
            self.integrator.initial_integrate(self.atom, self.dt)
        self.reneighbor_if_needed()
        if self.pair_style is not None and self.neighbor is not None:
            # clear_forces fused into the contact kernel (it writes, not adds)
            self.pair_style._launch(self.atom, self.neighbor, self.history, self.dt, True, accumulate=False)
        else:
            self.atom.clear_forces()
        for fix in self.fixes:
            fix.post_force(self.atom, self.dt)
        if self.integrator is not None:
            self.integrator.final_integrate(self.atom, self.dt)
        for fix in self.fixes:
            fix.end_of_step(self.atom, self.dt)

    def step(self) -> None:
        self._sub_step_inner()

    def run(self, steps: int) -> None:
        from .engine import FusedEngine, fusable

        self.setup_run(steps)
        if self.run_pre or not self.setup_done:
            self.init_simulation()
        if self.precision == "mixed" and not (self.fused and fusable(self)):
            raise NotImplementedError("the mixed form runs through the fused step: fix nve/sphere with "
                                      "optional damping/cundall and deform/pressure")
        # with periodic restart output the run stops at each multiple of restart_every to write one
        # (the next segment continues without a setup pass, as `run N pre no` would)
        remaining = int(steps)
        while True:
            seg = remaining
            if self.restart_every > 0:
                seg = min(seg, self.restart_every - self.timestep % self.restart_every)
            if self.fused and seg > 0 and fusable(self) and self.atom.nlocal > 0:
                eng = FusedEngine(self, self.precision)
                self.last_engine = eng
                eng.begin()
                try:
                    eng.run(seg)
                finally:
                    eng.finish()
            else:
                for _ in range(seg):
                    self._sub_step_inner()
            remaining -= seg
            if self.restart_every > 0 and seg > 0 and self.timestep % self.restart_every == 0:
                self.check_device_status()
                self.write_restart_now()
            if remaining <= 0:
                break
        self.check_device_status()
        self.domain.pull()

    def run_gpu(self, steps: int) -> None:
        """The reference's batched run; with no host I/O on this path it is run()."""
        self.run(steps)

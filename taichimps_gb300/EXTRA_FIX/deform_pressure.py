"""
fix deform/pressure: per-axis strain control and the pressure servo, on the device.

Mirrors taichimps ``FixDeformPressure`` (src/taichimps/EXTRA_FIX/deform_pressure.py:135-1219)
for orthogonal boxes: x/y/z styles none, erate, trate, vel, wiggle, final,
delta, scale, pressure and pressure/mean; ``couple``, ``max/rate``,
``normalize/pressure``, ``remap x|v|none`` and ``nevery``.

Every step's update runs on the device whatever the remap mode (the
reference keeps its default ``remap x`` on the host, reading the pressure
back every step): virial reduction with the kinetic term, the servo
(tmps_servo_step), then the affine remap (tmps_remap_x).  The host never
waits.  A box driven non-positive is recorded in a device status word and
raised at the next synchronisation point (a rebuild or the end of the run)
with the reference's message.

The ``volume`` style (with ``vol/balance/p``) and the ``box`` style
(isotropic volume or mean-pressure control of the whole box), which the
reference keeps on its host path, run on the device too: a one-thread pass
after the per-axis targets (csrc/tmps_servo.cuh).  ``variable`` (host-side
expressions) and tilt factors (triclinic boxes) raise NotImplementedError.
"""

from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Any, Callable

import numpy as np
import torch

from .. import _device, _lib
from .base import Fix

STYLE_CODE = {"none": 0, "erate": 1, "trate": 2, "vel": 3, "wiggle": 4, "final": 5, "delta": 6,
              "scale": 7, "pressure": 8, "pressure/mean": 9, "volume": 10}
BOX_STYLES = ("none", "volume", "pressure")
BOX_CODE = {"none": 0, "volume": 1, "pressure": 2}
VSUB_CODE = {"one_from_one": 0, "one_from_two": 1, "two_from_one": 2}
PRESSURE_STYLES = ("pressure", "pressure/mean")
NEEDS_RUN_LENGTH = ("final", "scale", "delta")
COUPLE_CODE = {"none": 0, "xyz": 1, "xy": 2, "yz": 3, "xz": 4}
REMAP_CODE = {"none": 0, "x": 1, "v": 2}


@dataclass
class AxisSet:
    style: str = "none"
    rate: float = 0.0
    vel: float = 0.0
    scale: float = 1.0
    flo: float = 0.0
    fhi: float = 0.0
    dlo: float = 0.0
    dhi: float = 0.0
    amplitude: float = 0.0
    tperiod: float = 0.0
    ptarget: float = 0.0
    pgain: float = 0.0
    lo_start: float = 0.0
    hi_start: float = 0.0
    coupled: bool = False
    # volume style links (deform_pressure.py:358-380)
    substyle: str = ""
    fixed: int = -1
    dynamic1: int = -1
    dynamic2: int = -1


class FixDeformPressure(Fix):
    def __init__(self, domain, axes: dict | None = None, box: dict | None = None, couple: str = "none",
                 max_rate: float = 0.0, normalize_pressure: bool = False, vol_balance_p: bool = False,
                 remap: str = "x", nevery: int = 1, flip: bool = True,
                 var_eval: Callable[[str], float] | None = None, float_type: Any = None,
                 p_target: float | None = None, p_gain: float | None = None) -> None:
        super().__init__(domain, float_type)
        self.nevery = int(nevery)
        if self.nevery < 1:
            raise ValueError("fix deform/pressure nevery must be >= 1")
        if couple not in COUPLE_CODE:
            raise ValueError(f"couple must be one of {tuple(COUPLE_CODE)}, got {couple!r}")
        if remap not in REMAP_CODE:
            raise ValueError("remap must be 'x', 'v' or 'none'")
        self.couple = couple
        self.remap = remap
        self.flip = bool(flip)
        self.max_rate = float(max_rate)
        self.normalize_pressure = bool(normalize_pressure)
        self.vol_balance_p = bool(vol_balance_p)
        self.var_eval = var_eval
        self.sets = [AxisSet() for _ in range(3)]
        self.set_box = AxisSet()
        if axes is None and box is None:
            # legacy isotropic form (deform_pressure.py:190-199)
            target = 50000.0 if p_target is None else float(p_target)
            gain = 1e-4 if p_gain is None else float(p_gain)
            for s in self.sets:
                s.style, s.ptarget, s.pgain = "pressure", target, gain
            if couple == "none":
                self.couple = "xyz"
        else:
            self._configure(axes or {}, box)
        self._validate()
        self.dev = _device.device()
        self._dservo = _device.struct_buffer(_lib.Servo())
        self._virial = torch.zeros(6, dtype=torch.float64, device=self.dev)
        self._ws = torch.zeros(0, dtype=torch.uint8, device=self.dev)
        self.status = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self.step_count = 0
        self.nsteps = 0
        self.nsteps_total = 0
        self._started = False
        self.on_device = True
        self.device_reason = ""
        self._vol_start = 0.0
        # optional per-step record of the pressure tensor in pinned host memory (record_pressure)
        self.pressure_log: torch.Tensor | None = None

    def _configure(self, axes: dict, box: dict | None = None) -> None:
        for name, spec in axes.items():
            if name in ("yz", "xz", "xy"):
                if spec.get("style", "none") != "none":
                    raise NotImplementedError("tilt-factor control is outside the GB300 path")
                continue
            if name not in ("x", "y", "z"):
                raise ValueError(f"Unknown deform dimension {name!r}")
            style = spec["style"]
            if style == "erate/rescale":
                raise ValueError("fix deform erate/rescale exists for NEMD with fix nvt/sllod, "
                                 "which taichimps does not have")
            if style == "variable":
                raise NotImplementedError("fix deform/pressure style 'variable' (host-side expressions) is "
                                          "outside the GB300 path")
            if style not in STYLE_CODE:
                raise ValueError(f"Unsupported fix deform/pressure style {style!r} for {name}")
            s = self.sets["xyz".index(name)]
            s.style = style
            for key, value in spec.items():
                if key == "style":
                    continue
                if not hasattr(s, key):
                    raise ValueError(f"Unknown parameter {key!r} for dimension {name}")
                setattr(s, key, float(value))
        if box is not None:
            style = box["style"]
            if style not in BOX_STYLES:
                raise ValueError(f"Unsupported fix deform/pressure box style {style!r}; implemented: {BOX_STYLES}")
            self.set_box.style = style
            for key, value in box.items():
                if key != "style":
                    setattr(self.set_box, key, float(value))

    def _validate(self) -> None:
        """deform_pressure.py:284-356, for the x/y/z entries."""
        for i, s in enumerate(self.sets):
            if s.style in PRESSURE_STYLES and s.pgain <= 0.0:
                raise ValueError(f"fix deform/pressure gain for {'xyz'[i]} must be positive")
            if s.style == "wiggle" and s.tperiod <= 0.0:
                raise ValueError(f"fix deform/pressure wiggle for {'xyz'[i]} needs a period")
        has_p = any(s.style in PRESSURE_STYLES for s in self.sets) or self.set_box.style == "pressure"
        if self.normalize_pressure and not has_p:
            raise ValueError("normalize/pressure only applies to pressure-controlled dimensions")
        if self.max_rate < 0.0:
            raise ValueError("max/rate must be positive")
        if self.normalize_pressure and self.max_rate == 0.0 and any(
                s.style in PRESSURE_STYLES and s.ptarget == 0.0 for s in self.sets):
            raise ValueError("cannot normalize the error for a zero target pressure without a max/rate")
        if self.couple != "none":
            idx = [i for i, c in enumerate("xyz") if c in self.couple]
            ref = next((i for i in idx if self.sets[i].style in PRESSURE_STYLES), None)
            if ref is None:
                raise ValueError("couple needs at least one of the coupled dimensions to be pressure controlled")
            for i in idx:
                s = self.sets[i]
                s.coupled = True
                if s.style == "none":
                    s.style, s.ptarget, s.pgain = self.sets[ref].style, self.sets[ref].ptarget, self.sets[ref].pgain
                elif s.style not in PRESSURE_STYLES:
                    raise ValueError("cannot couple non-pressure-controlled dimensions")
                elif s.pgain != self.sets[ref].pgain or s.ptarget != self.sets[ref].ptarget:
                    raise ValueError("coupled dimensions must have identical target and gain")
        # deform_pressure.py:316-330
        volume_dims = [i for i in range(3) if self.sets[i].style == "volume"]
        if volume_dims and any(s.style == "pressure/mean" for s in self.sets):
            raise ValueError("cannot ask fix deform/pressure for constant volume and a mean pressure at the same time")
        if self.set_box.style != "none":
            bad = ("final", "delta", "scale", "pressure/mean", "variable", "volume")
            for i in range(3):
                if self.sets[i].style in bad:
                    raise ValueError("fix deform/pressure box may only be combined with x/y/z styles vel, erate, "
                                     f"trate, wiggle and pressure, not {self.sets[i].style!r}")
            if self.set_box.style == "pressure" and self.set_box.pgain <= 0.0:
                raise ValueError("fix deform/pressure gain for box must be positive")
        if self.vol_balance_p and not volume_dims:
            raise ValueError("vol/balance/p only applies with the volume style")
        self._setup_volume_links()

    def _setup_volume_links(self) -> None:
        """Which dimensions a `volume` axis derives its size from (deform_pressure.py:358-385)."""
        for i in range(3):
            s = self.sets[i]
            if s.style != "volume":
                continue
            o1, o2 = (i + 1) % 3, (i + 2) % 3
            s1, s2 = self.sets[o1].style, self.sets[o2].style
            if s1 in ("none", "volume") and s2 in ("none", "volume"):
                raise ValueError("the volume style needs at least one other deformed dimension")
            if s1 == "none":
                s.substyle, s.fixed, s.dynamic1 = "one_from_one", o1, o2
            elif s2 == "none":
                s.substyle, s.fixed, s.dynamic1 = "one_from_one", o2, o1
            elif s1 == "volume":
                s.substyle, s.fixed, s.dynamic1 = "two_from_one", o1, o2
            elif s2 == "volume":
                s.substyle, s.fixed, s.dynamic1 = "two_from_one", o2, o1
            else:
                s.substyle, s.dynamic1, s.dynamic2 = "one_from_two", o1, o2
            if self.vol_balance_p and s.substyle != "two_from_one":
                raise ValueError("vol/balance/p needs two dimensions holding the volume constant")

    def note_atom_count(self, nlocal: int) -> None:
        self._nlocal_hint = int(nlocal)

    def _strain_h_rate(self, dt: float) -> np.ndarray:
        """deform_pressure.py:447-472, x/y/z part."""
        h = np.zeros(6)
        delt = self.nsteps_total * dt
        for i, s in enumerate(self.sets):
            length = s.hi_start - s.lo_start
            if s.style in ("erate", "trate"):
                h[i] = s.rate * length
            elif s.style == "vel":
                h[i] = s.vel
            elif s.style == "wiggle":
                h[i] = 2.0 * math.pi / s.tperiod * s.amplitude
            elif s.style in NEEDS_RUN_LENGTH and delt > 0.0:
                if s.style == "final":
                    stop = s.fhi - s.flo
                elif s.style == "delta":
                    stop = length + s.dhi - s.dlo
                else:
                    stop = s.scale * length
                h[i] = (stop - length) / delt
        return h

    def servo_struct(self) -> _lib.Servo:
        sv = _lib.Servo()
        for i, s in enumerate(self.sets):
            sv.style[i] = STYLE_CODE[s.style]
            sv.rate[i], sv.vel[i], sv.scale[i] = s.rate, s.vel, s.scale
            sv.flo[i], sv.fhi[i], sv.dlo[i], sv.dhi[i] = s.flo, s.fhi, s.dlo, s.dhi
            sv.amp[i], sv.tper[i] = s.amplitude, s.tperiod
            sv.ptarget[i], sv.pgain[i] = s.ptarget, s.pgain
            sv.lo_start[i], sv.hi_start[i] = s.lo_start, s.hi_start
            sv.cum[i] = 0.0
        sv.couple = COUPLE_CODE[self.couple]
        sv.normalize = 1 if self.normalize_pressure else 0
        sv.remap = REMAP_CODE[self.remap]
        sv.max_rate = self.max_rate
        sv.nsteps, sv.nsteps_total, sv.step_count, sv.nevery = self.nsteps, self.nsteps_total, self.step_count, self.nevery
        for i, s in enumerate(self.sets):
            sv.vsub[i] = VSUB_CODE.get(s.substyle, 0)
            sv.vfixed[i], sv.vdyn1[i], sv.vdyn2[i] = max(s.fixed, 0), max(s.dynamic1, 0), max(s.dynamic2, 0)
        sv.vol_balance_p = 1 if self.vol_balance_p else 0
        sv.box_style = BOX_CODE[self.set_box.style]
        sv.box_ptarget, sv.box_pgain = self.set_box.ptarget, self.set_box.pgain
        sv.vol_start = self._vol_start
        sv.post = 1 if (sv.box_style != 0 or any(s.style == "volume" for s in self.sets)) else 0
        sv.saved = 0
        return sv

    def setup(self, nsteps_total: int = 0, dt: float = 0.0) -> None:
        """Latch the box at the start of a run (deform_pressure.py:392-445)."""
        dom = self.domain
        dom.pull()
        self.nsteps = 0
        self.nsteps_total = int(nsteps_total)
        self._started = True
        self._vol_start = float(dom.volume)
        for i, s in enumerate(self.sets):
            s.lo_start = float(dom.boxlo[i])
            s.hi_start = float(dom.boxhi[i])
            if s.style in NEEDS_RUN_LENGTH and self.nsteps_total <= 0:
                raise ValueError(f"fix deform/pressure style {s.style!r} needs the run length; "
                                 "call setup(nsteps_total) before running")
        dom.set_h_rate(self._strain_h_rate(dt), vremap=(self.remap == "v"))
        _device.push_struct(self._dservo, self.servo_struct())
        self.status.zero_()
        # no kernel has written the status word since it was cleared: check_status need not read it
        self.status_clean = True

    def end_of_step(self, atom, dt: float) -> None:
        if self.domain is None:
            return
        if not self._started:
            self.setup(0)
        self.step_count += 1
        self.nsteps += 1
        if self.step_count % self.nevery != 0:
            return
        L = _device.lib()
        st = _device.stream()
        self.status_clean = False
        wsb = int(L.tmps_virial_workspace_bytes(atom.nlocal))
        if self._ws.numel() < wsb:
            self._ws = torch.zeros(wsb, dtype=torch.uint8, device=self.dev)
        if atom.nlocal:
            with _device.timed("virial"):
                rc = L.tmps_virial_reduce(atom.cstruct(), 1, self._virial.data_ptr(), self._ws.data_ptr(), wsb, st)
            _lib.check(rc, "tmps_virial_reduce")
        else:
            self._virial.zero_()
        elapsed = self.nsteps * dt
        frac = self.nsteps / self.nsteps_total if self.nsteps_total > 0 else 0.0
        with _device.timed("servo"):
            rc = L.tmps_servo_step(self.domain.dbox, self._dservo.data_ptr(), self._virial.data_ptr(),
                                   float(elapsed), float(frac), float(dt), self.status.data_ptr(), st)
        _lib.check(rc, "tmps_servo_step")
        if self.remap == "x":
            with _device.timed("remap_x"):
                rc = L.tmps_remap_x(atom.cstruct(), self.domain.dbox, st)
            _lib.check(rc, "tmps_remap_x")
        self.domain.mark_device_authoritative()

    def check_status(self) -> None:
        if getattr(self, "status_clean", False):
            return
        if int(self.status.item()) & _lib.STATUS_BOX_NONPOSITIVE:
            self.domain.pull()
            raise RuntimeError(
                f"fix deform/pressure drove a box dimension to {self.domain.prd}, which is "
                "not positive; check the gain, max/rate or strain rate")

    def last_pressure(self) -> np.ndarray:
        """The pressure tensor the servo used on its last update (synchronises)."""
        return np.array(_device.pull_struct(self._dservo, _lib.Servo).pressure[:])

    def record_pressure(self, capacity: int) -> None:
        """Have every fused step write its pressure tensor to pinned host memory (a ring of
        `capacity` rows, row = timestep % capacity), with no host synchronisation: the
        per-step read-back of the reference's host servo path (deform_pressure.py:1113-1219)
        without the round trip.  capacity 0 stops recording."""
        self.pressure_log = (torch.zeros((int(capacity), 6), dtype=torch.float64).pin_memory()
                             if capacity > 0 else None)

    def pressure_history(self, steps) -> np.ndarray:
        """Recorded pressure tensors of the given timesteps (rows of 6), after the run returned."""
        if self.pressure_log is None:
            raise RuntimeError("record_pressure() was not called")
        torch.cuda.synchronize()
        log = self.pressure_log.numpy()
        return np.stack([log[int(s) % len(log)] for s in steps])

"""
Differentiable DEM run with a hand-written adjoint.

A gran/hertz/history packing under nve/sphere and fix deform/pressure (x/y/z
styles none, erate or pressure; couple; max/rate; remap x) is run forward in
FP64 on the GPU, and the gradient of its deviatoric-stress curve
q(s) = p_zz - (p_xx + p_yy) / 2, sampled every `sample_every` steps, with
respect to kn, kt, gamman, gammat, xmu and every particle radius comes from
the reverse of each step (taichimps_gb300/csrc/tmps_adjoint.cu):

* the forward keeps a checkpoint of the state every `checkpoint_every`
  steps and nothing else;
* the reverse restores a checkpoint, recomputes that segment recording a
  per-step tape (positions after the drift, velocities, forces, the history
  entering the contact pass and the per-contact masks), and runs the
  segment's steps backwards;
* the masks the forward recorded (contact on, Coulomb slip, |shear| != 0,
  the damping clamp; the servo's max/rate clamp) are replayed, so the
  gradient is that of the piecewise-smooth map the forward computed -- no
  smoothing of the Coulomb cap or the contact switch;
* neighbor rebuilds (the reference's skin rule, neighbor.py:214-245) carry
  the history by pair identity; the reverse carries its adjoint back the
  same way.

`stress_curve(...)` wraps this in a torch.autograd.Function.  The
reference has no differentiable path; the forward follows the reference's
step (Simulation._sub_step_inner, simulation.py:205-247: setup force
evaluation with shearupdate off, then per step nve/sphere initial, contacts,
nve/sphere final, deform/pressure end_of_step) with the contact law of
GRANULAR/hertz_history.py:92-157.
"""

from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _device, _lib

STYLE = {"none": 0, "erate": 1, "pressure": 8}
COUPLE = {"none": 0, "xyz": 1, "xy": 2, "yz": 3, "xz": 4}
_REC = ctypes.sizeof(_lib.AdjRec)
_Q_OFF = _lib.AdjRec.q.offset // 8


def _p(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


class _Pairs:
    """A half pair list (i < j) in (i, j) order, and its incidence by j."""

    def __init__(self, n: int, pi: torch.Tensor, pj: torch.Tensor, ibeg: torch.Tensor):
        self.n, self.npairs = n, int(pi.numel())
        dev = pi.device
        self.pi, self.pj, self.ibeg = pi, pj, ibeg
        if self.npairs:
            key = pj.long() * n + pi.long()
            self.jlist = torch.argsort(key).to(torch.int32)
            jc = torch.bincount(pj.long(), minlength=n)
        else:
            self.jlist = torch.zeros(1, dtype=torch.int32, device=dev)
            jc = torch.zeros(n, dtype=torch.int64, device=dev)
        self.jbeg = torch.zeros(n + 1, dtype=torch.int32, device=dev)
        self.jbeg[1:] = torch.cumsum(jc, 0).to(torch.int32)

    @staticmethod
    def build(x: torch.Tensor, radius: torch.Tensor, rec_ptr: int, skin: float) -> "_Pairs":
        L = _device.lib()
        st = _device.stream()
        n = radius.numel()
        dev = radius.device
        count = torch.zeros(max(n, 1), dtype=torch.int32, device=dev)
        _lib.check(L.tmps_adj_pairs(n, _p(x), _p(radius), rec_ptr, skin, _p(count), None, None, None, st),
                   "tmps_adj_pairs")
        ibeg = torch.zeros(n + 1, dtype=torch.int32, device=dev)
        ibeg[1:] = torch.cumsum(count[:n], 0).to(torch.int32)
        npairs = int(ibeg[-1].item())
        pi = torch.zeros(max(npairs, 1), dtype=torch.int32, device=dev)
        pj = torch.zeros(max(npairs, 1), dtype=torch.int32, device=dev)
        if npairs:
            _lib.check(L.tmps_adj_pairs(n, _p(x), _p(radius), rec_ptr, skin, None, _p(ibeg), _p(pi), _p(pj), st),
                       "tmps_adj_pairs")
        return _Pairs(n, pi[:npairs], pj[:npairs], ibeg)


class _Tape:
    """One step's record (atom arrays [3][n], pair arrays [3][npairs])."""

    def __init__(self, n: int, npairs: int, dev):
        f64 = dict(dtype=torch.float64, device=dev)
        self.xh, self.vh, self.wh = (torch.zeros((3, n), **f64) for _ in range(3))
        self.f, self.t = torch.zeros((3, n), **f64), torch.zeros((3, n), **f64)
        self.resize(npairs, dev)

    def resize(self, npairs: int, dev) -> None:
        self.shear = torch.zeros((3, max(npairs, 1)), dtype=torch.float64, device=dev)
        self.mask = torch.zeros(max(npairs, 1), dtype=torch.uint8, device=dev)

    def cstruct(self) -> _lib.AdjTape:
        return _lib.AdjTape(_p(self.xh), _p(self.vh), _p(self.wh), _p(self.f), _p(self.t), _p(self.shear),
                            _p(self.mask))


class AdjointRun:
    """One differentiable run.

    x: [n, 3] initial positions; radius: [n]; density: scalar; box_lo/box_hi:
    the periodic box; axes: {"x": {"style": "pressure", "ptarget": 1.0,
    "pgain": 1e-3}, "z": {"style": "erate", "rate": -1e-3}, ...}; v / omega:
    initial velocities (zero if None); skin: neighbor skin (rebuild when an
    atom moved more than skin / 2 since the last build)."""

    def __init__(self, x, radius, density: float, box_lo, box_hi, *, dt: float, steps: int, axes: dict,
                 couple: str = "none", max_rate: float = 0.0, normalize: bool = False, sample_every: int = 50,
                 checkpoint_every: int = 100, skin: float = 0.1, v=None, omega=None, limit_damping: bool = False):
        self.dev = _device.device()
        f64 = dict(dtype=torch.float64, device=self.dev)
        x = torch.as_tensor(np.asarray(x, dtype=np.float64) if not torch.is_tensor(x) else x, **f64)
        self.n = int(x.shape[0])
        self.x0 = x.T.contiguous()
        self.v0 = (torch.zeros((3, self.n), **f64) if v is None
                   else torch.as_tensor(np.asarray(v, dtype=np.float64), **f64).T.contiguous())
        self.w0 = (torch.zeros((3, self.n), **f64) if omega is None
                   else torch.as_tensor(np.asarray(omega, dtype=np.float64), **f64).T.contiguous())
        self.radius0 = torch.as_tensor(np.asarray(radius, dtype=np.float64), **f64).contiguous()
        self.density = float(density)
        self.box_lo = [float(a) for a in box_lo]
        self.box_hi = [float(a) for a in box_hi]
        self.dt, self.steps = float(dt), int(steps)
        self.sample_every, self.checkpoint_every = int(sample_every), int(checkpoint_every)
        if self.sample_every < 1 or self.checkpoint_every < 1 or self.steps < 1:
            raise ValueError("steps, sample_every and checkpoint_every must be positive")
        self.skin = float(skin)
        self.limit_damping = 1 if limit_damping else 0
        sv = _lib.AdjServo()
        for d, name in enumerate("xyz"):
            spec = dict(axes.get(name, {"style": "none"}))
            style = spec.pop("style", "none")
            if style not in STYLE:
                raise ValueError(f"axis {name}: style {style!r} is not differentiable here (none, erate, pressure)")
            sv.style[d] = STYLE[style]
            sv.rate[d] = float(spec.pop("rate", 0.0))
            sv.ptarget[d] = float(spec.pop("ptarget", 0.0))
            sv.pgain[d] = float(spec.pop("pgain", 0.0))
            if spec:
                raise ValueError(f"axis {name}: unknown keys {sorted(spec)}")
            if style == "pressure" and sv.pgain[d] <= 0.0:
                raise ValueError(f"fix deform/pressure gain for {name} must be positive")
            sv.lo_start[d], sv.hi_start[d] = self.box_lo[d], self.box_hi[d]
        if couple not in COUPLE:
            raise ValueError(f"couple must be one of {tuple(COUPLE)}")
        sv.couple = COUPLE[couple]
        sv.normalize = 1 if normalize else 0
        sv.max_rate = float(max_rate)
        self.servo = sv
        self.samples = np.arange(self.sample_every, self.steps + 1, self.sample_every)
        self._fwd = None

    # ----------------------------------------------------------- helpers

    def _rec_ptr(self, k: int) -> int:
        return self.rec.data_ptr() + k * _REC

    def _sys(self, st: dict, pairs: _Pairs, shear: torch.Tensor) -> _lib.AdjSys:
        return _lib.AdjSys(self.n, pairs.npairs, _p(st["x"]), _p(st["v"]), _p(st["w"]), _p(st["f"]), _p(st["t"]),
                           _p(self.r), _p(self.m), _p(shear), _p(pairs.pi) if pairs.npairs else None,
                           _p(pairs.pj) if pairs.npairs else None, _p(pairs.ibeg), _p(pairs.jbeg), _p(pairs.jlist))

    def _work(self, npairs: int) -> torch.Tensor:
        nb = int(_device.lib().tmps_adj_workspace_bytes(self.n, npairs))
        if self._workbuf is None or self._workbuf.numel() < nb:
            self._workbuf = torch.zeros(nb, dtype=torch.uint8, device=self.dev)
        return self._workbuf

    def _carry(self, old: _Pairs, new: _Pairs, m: torch.Tensor, src: torch.Tensor, reverse: bool) -> torch.Tensor:
        L = _device.lib()
        if reverse:
            out = torch.zeros((3, max(old.npairs, 1)), dtype=torch.float64, device=self.dev)
            _lib.check(L.tmps_adj_carry(old.npairs, new.npairs, _p(m), _p(out), _p(src), 1, _device.stream()),
                       "tmps_adj_carry")
        else:
            out = torch.zeros((3, max(new.npairs, 1)), dtype=torch.float64, device=self.dev)
            _lib.check(L.tmps_adj_carry(old.npairs, new.npairs, _p(m), _p(src), _p(out), 0, _device.stream()),
                       "tmps_adj_carry")
        return out

    # ----------------------------------------------------------- forward

    def forward(self, kn: float, kt: float, gamman: float, gammat: float, xmu: float,
                radius: torch.Tensor | None = None, track_masks: bool = False) -> torch.Tensor:
        """Runs `steps` steps; returns q at the sample steps (device tensor).  track_masks: also keep
        `mask_digest`, an integer fingerprint of every step's per-pair masks (contact on, Coulomb slip,
        |shear| != 0, damping clamp) and rebuild steps -- two runs with equal digests took the same
        branch of every piecewise law at every step, so the loss is smooth between them."""
        L = _device.lib()
        sc = _device.stream()
        f64 = dict(dtype=torch.float64, device=self.dev)
        self.r = (self.radius0 if radius is None else radius.detach().to(**f64)).contiguous().clone()
        self.m = ((4.0 / 3.0) * math.pi * (self.r ** 3)) * self.density
        self.prm = _lib.AdjParams(float(kn), float(kt), float(gamman), float(gammat), float(xmu), self.dt,
                                  self.limit_damping, 0)
        self._workbuf = None
        self.rec = torch.zeros((self.steps + 1) * _REC, dtype=torch.uint8, device=self.dev)
        r0 = _lib.AdjRec()
        for d in range(3):
            r0.lo[d] = self.box_lo[d]
            r0.prd[d] = self.box_hi[d] - self.box_lo[d]
        self.rec[:_REC].copy_(torch.from_numpy(np.frombuffer(bytes(r0), dtype=np.uint8).copy()))
        st = dict(x=self.x0.clone(), v=self.v0.clone(), w=self.w0.clone(), f=torch.zeros((3, self.n), **f64),
                  t=torch.zeros((3, self.n), **f64))
        pairs = _Pairs.build(st["x"], self.r, self._rec_ptr(0), self.skin)
        self.lists, self.events = [pairs], {}
        li = 0
        shear = torch.zeros((3, max(pairs.npairs, 1)), **f64)
        tape = _Tape(self.n, pairs.npairs, self.dev)
        _lib.check(L.tmps_adj_setup(self._sys(st, pairs, shear), self.prm, self._rec_ptr(0), tape.cstruct(),
                                    _p(self._work(pairs.npairs)), sc), "tmps_adj_setup")
        self.ckpt = {}
        xbuild = st["x"].clone()
        disp = torch.zeros(1, dtype=torch.int64, device=self.dev)
        trig = 0.25 * self.skin * self.skin
        self.rebuilds = 0
        digest = torch.zeros((), dtype=torch.int64, device=self.dev)
        for s in range(1, self.steps + 1):
            if (s - 1) % self.checkpoint_every == 0:
                self.ckpt[s - 1] = ({k: a.clone() for k, a in st.items()}, shear.clone(), li)
            disp.zero_()
            _lib.check(L.tmps_adj_initial(self._sys(st, pairs, shear), self.prm, tape.cstruct(), _p(xbuild), _p(disp),
                                          sc), "tmps_adj_initial")
            if float(disp.view(torch.float64).item()) > trig:
                new = _Pairs.build(tape.xh, self.r, self._rec_ptr(s - 1), self.skin)
                m = torch.zeros(max(pairs.npairs, 1), dtype=torch.int32, device=self.dev)
                _lib.check(L.tmps_adj_pair_map(pairs.npairs, _p(pairs.pi), _p(pairs.pj), _p(new.ibeg), _p(new.pj),
                                               _p(m), sc), "tmps_adj_pair_map")
                shear = self._carry(pairs, new, m, shear, False)
                self.lists.append(new)
                li = len(self.lists) - 1
                self.events[s] = (li, m)
                pairs = new
                tape.resize(pairs.npairs, self.dev)
                xbuild = tape.xh.clone()
                self.rebuilds += 1
            _lib.check(L.tmps_adj_finish(self._sys(st, pairs, shear), self.prm, self.servo, tape.cstruct(),
                                         self.rec.data_ptr(), s, _p(self._work(pairs.npairs)), sc), "tmps_adj_finish")
            if track_masks:
                digest = self._digest_step(digest, tape.mask[:pairs.npairs], s if s in self.events else 0)
        self.final_state = st
        self.mask_digest = int(digest.item()) if track_masks else None
        self._fwd = True
        return self.q_samples()

    @staticmethod
    def _digest_step(digest: torch.Tensor, mask: torch.Tensor, rebuilt: int) -> torch.Tensor:
        """digest * 1000003 + sum_k mask_k (k + 1) + 7 sum_k mask_k (k + 1)^2 + rebuild step (int64,
        wrapping): any change of one pair's mask bits changes it."""
        k = torch.arange(1, mask.numel() + 1, dtype=torch.int64, device=mask.device)
        m = mask.to(torch.int64)
        return digest * 1000003 + (m * k).sum() + 7 * (m * k * k).sum() + rebuilt

    def records(self) -> np.ndarray:
        """The per-step records as a structured view: q, w, box (host copy)."""
        raw = self.rec.cpu().numpy()
        return np.frombuffer(raw.tobytes(), dtype=np.float64).reshape(self.steps + 1, _REC // 8)

    def q_all(self) -> np.ndarray:
        """q of steps 1..steps (host)."""
        return self.records()[1:, _Q_OFF].copy()

    def q_samples(self) -> torch.Tensor:
        recs = self.rec.view(torch.float64).view(self.steps + 1, _REC // 8)
        idx = torch.as_tensor(self.samples, dtype=torch.long, device=self.dev)
        return recs[idx, _Q_OFF].clone()

    # ----------------------------------------------------------- reverse

    def backward(self, qbar) -> dict:
        """dL/d(kn, kt, gamman, gammat, xmu, radius) for dL/dq = qbar at the sample steps."""
        if not self._fwd:
            raise RuntimeError("backward() needs a forward() first")
        L = _device.lib()
        sc = _device.stream()
        f64 = dict(dtype=torch.float64, device=self.dev)
        qb = np.zeros(self.steps + 1)
        qb[self.samples] = np.asarray(qbar, dtype=np.float64).reshape(-1)
        n = self.n
        bar = {k: torch.zeros((3, n), **f64) for k in ("x", "v", "w", "f", "t")}
        bar["radius"], bar["mass"] = torch.zeros(n, **f64), torch.zeros(n, **f64)
        bar["params"], bar["box"] = torch.zeros(8, **f64), torch.zeros(18, **f64)
        li_last = max([0] + [li for s, (li, _) in self.events.items()])
        bar_sh = torch.zeros((3, max(self.lists[li_last].npairs, 1)), **f64)

        def bar_struct(sh):
            return _lib.AdjBar(_p(bar["x"]), _p(bar["v"]), _p(bar["w"]), _p(bar["f"]), _p(bar["t"]), _p(sh),
                               _p(bar["radius"]), _p(bar["mass"]), _p(bar["params"]), _p(bar["box"]))

        disp = torch.zeros(1, dtype=torch.int64, device=self.dev)
        for start in sorted(self.ckpt, reverse=True):
            end = min(start + self.checkpoint_every, self.steps)
            saved, shear, li = self.ckpt[start]
            st = {k: a.clone() for k, a in saved.items()}
            shear = shear.clone()
            pairs = self.lists[li]
            tapes = {}
            for s in range(start + 1, end + 1):
                ev = self.events.get(s)
                npairs = self.lists[ev[0]].npairs if ev else pairs.npairs
                tape = _Tape(n, npairs, self.dev)
                _lib.check(L.tmps_adj_initial(self._sys(st, pairs, shear), self.prm, tape.cstruct(), _p(st["x"]),
                                              _p(disp), sc), "tmps_adj_initial")
                if ev:
                    new = self.lists[ev[0]]
                    shear = self._carry(pairs, new, ev[1], shear, False)
                    pairs = new
                _lib.check(L.tmps_adj_finish(self._sys(st, pairs, shear), self.prm, self.servo, tape.cstruct(),
                                             self.rec.data_ptr(), s, _p(self._work(pairs.npairs)), sc),
                           "tmps_adj_finish")
                tapes[s] = (tape, pairs)
            for s in range(end, start, -1):
                tape, pairs = tapes[s]
                prev = tapes[s - 1][0] if s - 1 > start else None
                fprev = prev.f if prev is not None else saved["f"]
                tprev = prev.t if prev is not None else saved["t"]
                _lib.check(L.tmps_adj_step_back(self._sys(st, pairs, tape.shear), self.prm, self.servo,
                                                tape.cstruct(), self.rec.data_ptr(), s, _p(fprev), _p(tprev),
                                                float(qb[s]), bar_struct(bar_sh), _p(self._work(pairs.npairs)), sc),
                           "tmps_adj_step_back")
                ev = self.events.get(s)
                if ev:
                    old = tapes[s - 1][1] if s - 1 > start else self.lists[self.ckpt[start][2]]
                    bar_sh = self._carry(old, pairs, ev[1], bar_sh, True)
            del tapes
        # the setup force evaluation
        saved, _, li = self.ckpt[0]
        pairs = self.lists[li]
        st = {k: a.clone() for k, a in saved.items()}
        shear = torch.zeros((3, max(pairs.npairs, 1)), **f64)
        tape = _Tape(n, pairs.npairs, self.dev)
        _lib.check(L.tmps_adj_setup(self._sys(st, pairs, shear), self.prm, self._rec_ptr(0), tape.cstruct(),
                                    _p(self._work(pairs.npairs)), sc), "tmps_adj_setup")
        st = {k: a.clone() for k, a in saved.items()}
        _lib.check(L.tmps_adj_setup_back(self._sys(st, pairs, shear), self.prm, self._rec_ptr(0), tape.cstruct(),
                                         bar_struct(bar_sh), _p(self._work(pairs.npairs)), sc), "tmps_adj_setup_back")
        # m = (4/3) pi r^3 rho: dm/dr = 3 m / r
        g_r = bar["radius"] + bar["mass"] * (3.0 * self.m / self.r)
        gp = bar["params"][:5].cpu().numpy()
        return {"kn": float(gp[0]), "kt": float(gp[1]), "gamman": float(gp[2]), "gammat": float(gp[3]),
                "xmu": float(gp[4]), "radius": g_r}


class _StressCurve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, run: AdjointRun, kn, kt, gamman, gammat, xmu, radius):
        q = run.forward(float(kn), float(kt), float(gamman), float(gammat), float(xmu), radius.detach())
        ctx.run = run
        ctx.meta = [(a.dtype, a.device) for a in (kn, kt, gamman, gammat, xmu, radius)]
        return q

    @staticmethod
    def backward(ctx, gq):
        g = ctx.run.backward(gq.detach().cpu().numpy())
        out = [None]
        for key, (dtype, dev) in zip(("kn", "kt", "gamman", "gammat", "xmu"), ctx.meta[:5]):
            out.append(torch.tensor(g[key], dtype=dtype, device=dev))
        dtype, dev = ctx.meta[5]
        out.append(g["radius"].to(dtype=dtype, device=dev))
        return tuple(out)


def stress_curve(run: AdjointRun, kn, kt, gamman, gammat, xmu, radius) -> torch.Tensor:
    """q at the run's sample steps as a differentiable function of the contact
    parameters (0-d tensors) and the radii ([n] tensor)."""
    T = lambda a: a if torch.is_tensor(a) else torch.tensor(float(a), dtype=torch.float64)
    return _StressCurve.apply(run, T(kn), T(kt), T(gamman), T(gammat), T(xmu), radius)

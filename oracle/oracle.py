"""
ORACLE — test infrastructure only.

Python driver around the C restatement in ``tmps_oracle.c``.  It reproduces the
reference's step order and host-side logic, so that the CUDA product path can
be checked against the reference's arithmetic on the same inputs:

* ``OracleSim.step``      follows Simulation._sub_step_inner   (simulation.py:205-247)
* ``OracleSim.setup``     follows Simulation.init_simulation   (simulation.py:170-203)
* ``OracleSim._reneighbor`` follows reneighbor_if_needed       (simulation.py:122-159)
* ``OracleNeighbor.decide`` follows NeighborList.decide        (neighbor.py:371-403)
* ``OracleDeform``        follows FixDeformPressure's servo for the orthogonal
  x/y/z styles (deform_pressure.py:392-489, 583-596, 706-857, 1113-1219)

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU baseline use
this module.  The product package never imports it.

Parity status: pinned by the reference's own known answers and invariants
(tests/test_oracle_pins.py).  The reference itself cannot run here (Taichi
1.7.4 is not installable offline), so no output of the reference is compared
directly.
"""

from __future__ import annotations

import ctypes
import math
import os
import subprocess
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
_BUILD = _HERE / "_build"
_SO = _BUILD / "libtmps_oracle.so"

_i32p = ctypes.POINTER(ctypes.c_int32)
_f64p = ctypes.POINTER(ctypes.c_double)


class OrBox(ctypes.Structure):
    _fields_ = [
        ("lo", ctypes.c_double * 3),
        ("hi", ctypes.c_double * 3),
        ("prd", ctypes.c_double * 3),
        ("h_rate", ctypes.c_double * 6),
        ("per", ctypes.c_int32 * 3),
        ("vremap", ctypes.c_int32),
    ]


class OrPair(ctypes.Structure):
    _fields_ = [
        ("kn", ctypes.c_double), ("kt", ctypes.c_double), ("gamman", ctypes.c_double),
        ("gammat", ctypes.c_double), ("xmu", ctypes.c_double),
        ("limit_damping", ctypes.c_int32),
        ("normal_id", ctypes.c_int32), ("damping_id", ctypes.c_int32),
        ("tangential_id", ctypes.c_int32),
        ("damp", ctypes.c_double), ("xt", ctypes.c_double), ("mu", ctypes.c_double),
        ("rolling_id", ctypes.c_int32),
        ("k_roll", ctypes.c_double), ("gamma_roll", ctypes.c_double), ("mu_roll", ctypes.c_double),
    ]


STYLE_IDS = {"hooke": 0, "hooke/history": 1, "hertz": 2, "hertz/history": 3, "granular": 4}


def build(force: bool = False) -> Path:
    """Compile the C restatement into oracle/_build (gcc, no fast-math, no FMA contraction)."""
    src = _HERE / "tmps_oracle.c"
    if _SO.exists() and not force and _SO.stat().st_mtime >= src.stat().st_mtime:
        return _SO
    _BUILD.mkdir(exist_ok=True)
    tmp = _SO.with_suffix(f".{os.getpid()}.tmp")
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-fopenmp", str(src), "-o", str(tmp), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _SO)
    return _SO


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(str(build()))
        _lib.or_setup_grid.restype = ctypes.c_int
        _lib.or_build_neighbor_list.restype = ctypes.c_int
        _lib.or_build_pair_list.restype = ctypes.c_int
        _lib.or_skin_check.restype = ctypes.c_int
        _lib.or_has_openmp.restype = ctypes.c_int
    return _lib


def set_threads(n: int) -> None:
    lib().or_set_threads(int(n))


def _p(a: np.ndarray, t=_f64p):
    return a.ctypes.data_as(t)


# --------------------------------------------------------------------- domain


@dataclass
class OracleDomain:
    """Orthogonal box, host-side (domain.py:45-89 without the device mirror)."""

    boxlo: np.ndarray
    boxhi: np.ndarray
    periodicity: np.ndarray
    h_rate: np.ndarray = field(default_factory=lambda: np.zeros(6))
    vremap: bool = False

    @classmethod
    def make(cls, boxlo, boxhi, boundary=("p", "p", "p")):
        return cls(np.array(boxlo, dtype=np.float64), np.array(boxhi, dtype=np.float64),
                   np.array([1 if b == "p" else 0 for b in boundary], dtype=np.int32))

    @property
    def prd(self) -> np.ndarray:
        return self.boxhi - self.boxlo

    @property
    def volume(self) -> float:
        p = self.prd
        return float(p[0] * p[1] * p[2])

    def cbox(self) -> OrBox:
        b = OrBox()
        prd = self.prd
        for k in range(3):
            b.lo[k] = float(self.boxlo[k])
            b.hi[k] = float(self.boxhi[k])
            b.prd[k] = float(prd[k])
            b.per[k] = int(self.periodicity[k])
        for k in range(6):
            b.h_rate[k] = float(self.h_rate[k])
        b.vremap = 1 if self.vremap else 0
        return b


# --------------------------------------------------------------------- atoms


class OracleAtoms:
    """Per-atom state in the reference's [n][3] layout (atom.py:36-53)."""

    def __init__(self, x, radius, density, v=None, omega=None, tag=None):
        x = np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(-1, 3))
        n = len(x)
        self.n = n
        self.x = x.copy()
        self.v = np.zeros((n, 3)) if v is None else np.ascontiguousarray(np.asarray(v, dtype=np.float64).reshape(n, 3)).copy()
        self.omega = np.zeros((n, 3)) if omega is None else np.ascontiguousarray(np.asarray(omega, dtype=np.float64).reshape(n, 3)).copy()
        r = np.asarray(radius, dtype=np.float64)
        self.radius = np.full(n, float(r)) if r.ndim == 0 else r.copy()
        d = np.asarray(density, dtype=np.float64)
        dens = np.full(n, float(d)) if d.ndim == 0 else d
        # atom.py:110-111
        self.rmass = ((4.0 / 3.0) * np.pi * (self.radius ** 3)) * dens
        self.tag = (np.arange(1, n + 1, dtype=np.int32) if tag is None
                    else np.asarray(tag, dtype=np.int32).copy())
        self.f = np.zeros((n, 3))
        self.torque = np.zeros((n, 3))
        self.virial = np.zeros((n, 6))

    def clear_forces(self):
        lib().or_clear_forces(self.n, _p(self.f), _p(self.torque), _p(self.virial))


# ------------------------------------------------------------------ neighbors


class OracleNeighbor:
    """NeighborList (neighbor.py:23-435): half list, counting-sort bins."""

    MAX_GRID_CELLS = 200000

    def __init__(self, domain: OracleDomain, skin: float, max_neighbors: int = 64):
        self.domain = domain
        self.skin = float(skin)
        self.max_nb = int(max_neighbors)
        self.delay, self.every, self.check = 0, 1, True
        self.last_build_step = -1
        self.current_step = 0
        self.has_built = False
        self.build_count = 0
        self.grid_dim = np.zeros(3, dtype=np.int32)
        self.csize = np.zeros(3)
        self.npairs = 0
        self.pair_i = np.zeros(0, dtype=np.int32)
        self.pair_j = np.zeros(0, dtype=np.int32)
        self.x0 = None
        self.cell_of = None

    def build(self, atoms: OracleAtoms) -> None:
        n = atoms.n
        if n == 0:
            return
        L = lib()
        box = self.domain.cbox()
        max_r = float(np.max(atoms.radius))
        ncell = L.or_setup_grid(ctypes.byref(box), ctypes.c_double(2.0 * max_r),
                                ctypes.c_double(self.skin), self.MAX_GRID_CELLS,
                                _p(self.grid_dim, _i32p), _p(self.csize))
        self.cell_of = np.zeros(n, dtype=np.int32)
        self.cell_start = np.zeros(ncell + 1, dtype=np.int32)
        self.cell_particles = np.zeros(n, dtype=np.int32)
        L.or_build_grid(ctypes.byref(box), _p(self.grid_dim, _i32p), _p(self.csize), n,
                        _p(atoms.x), _p(self.cell_of, _i32p), _p(self.cell_start, _i32p),
                        _p(self.cell_particles, _i32p))
        self.num_neighbors = np.zeros(n, dtype=np.int32)
        self.neighbors = np.zeros((n, self.max_nb), dtype=np.int32)
        ovf = L.or_build_neighbor_list(ctypes.byref(box), _p(self.grid_dim, _i32p), _p(self.csize), n,
                                       _p(atoms.x), _p(atoms.radius), ctypes.c_double(self.skin),
                                       _p(self.cell_start, _i32p), _p(self.cell_particles, _i32p),
                                       self.max_nb, _p(self.num_neighbors, _i32p),
                                       _p(self.neighbors, _i32p))
        total = int(self.num_neighbors.sum())
        self.pair_start = np.zeros(n + 1, dtype=np.int32)
        self.pair_i = np.zeros(max(total, 1), dtype=np.int32)
        self.pair_j = np.zeros(max(total, 1), dtype=np.int32)
        self.npairs = L.or_build_pair_list(n, self.max_nb, _p(self.num_neighbors, _i32p),
                                           _p(self.neighbors, _i32p), _p(self.pair_start, _i32p),
                                           _p(self.pair_i, _i32p), _p(self.pair_j, _i32p))
        if ovf:
            raise RuntimeError(
                f"Neighbor list overflow: more than {self.max_nb} neighbors for at least one "
                "particle. Increase max_neighbors_per_atom, or reduce the neighbor skin.")
        self.x0 = atoms.x.copy()
        self.has_built = True
        self.build_count += 1
        self.last_build_step = self.current_step

    def decide(self, atoms: OracleAtoms, timestep: int | None = None) -> bool:
        if not self.has_built:
            return True
        self.current_step = timestep if timestep is not None else self.current_step + 1
        since = self.current_step - self.last_build_step
        if since < self.delay:
            return False
        if since % self.every != 0:
            return False
        if not self.check:
            return True
        if atoms.n == 0:
            return False
        return bool(lib().or_skin_check(atoms.n, _p(atoms.x), _p(self.x0),
                                        ctypes.c_double(0.25 * self.skin * self.skin)))

    def contact_count(self, atoms: OracleAtoms) -> np.ndarray:
        """ComputeContactAtom.compute (computes/contact_atom.py:21-63): per-atom contact counts."""
        out = np.zeros(atoms.n, dtype=np.int32)
        if atoms.n:
            lib().or_contact_count(ctypes.byref(self.domain.cbox()), atoms.n, _p(atoms.x), _p(atoms.radius),
                                   self.max_nb, _p(self.num_neighbors, _i32p), _p(self.neighbors, _i32p),
                                   _p(out, _i32p))
        return out

    def pair_set(self, tags: np.ndarray) -> set[tuple[int, int]]:
        """The built half list as a set of (tag_i, tag_j) with tag_i < tag_j."""
        out = set()
        for i in range(len(self.num_neighbors)):
            for k in range(self.num_neighbors[i]):
                a, b = int(tags[i]), int(tags[self.neighbors[i, k]])
                out.add((min(a, b), max(a, b)))
        return out


class OracleHistory:
    """ContactHistory (contact_history.py:25-154), per flat pair."""

    def __init__(self, max_neighbors: int = 64):
        self.max_nb = int(max_neighbors)
        self.partner = np.full(1, -1, dtype=np.int32)
        self.shear = np.zeros((1, 3))
        self.rolling = np.zeros((1, 3))   # rolling displacement per pair (contact_history.py:58-59)
        self.setup_pending = False
        self._saved = None

    def save_state(self, atoms: OracleAtoms, nl: OracleNeighbor) -> None:
        if atoms.n == 0 or self.setup_pending:
            return
        n = atoms.n
        cnt = np.zeros(n, dtype=np.int32)
        stag = np.zeros((n, self.max_nb), dtype=np.int32)
        ssh = np.zeros((n, self.max_nb, 3))
        srl = np.zeros((n, self.max_nb, 3))
        if nl.npairs > 0:
            lib().or_history_save(n, nl.npairs, _p(nl.pair_i, _i32p), _p(self.partner, _i32p),
                                  _p(self.shear), _p(self.rolling), self.max_nb, _p(cnt, _i32p),
                                  _p(stag, _i32p), _p(ssh), _p(srl))
        self._saved = (cnt, stag, ssh, srl)

    def restore_state(self, atoms: OracleAtoms, nl: OracleNeighbor) -> None:
        if atoms.n == 0:
            return
        m = max(nl.npairs, 1)
        self.partner = np.full(m, -1, dtype=np.int32)
        self.shear = np.zeros((m, 3))
        self.rolling = np.zeros((m, 3))
        if self._saved is None:
            cnt = np.zeros(atoms.n, dtype=np.int32)
            stag = np.zeros((atoms.n, self.max_nb), dtype=np.int32)
            ssh = np.zeros((atoms.n, self.max_nb, 3))
            srl = np.zeros((atoms.n, self.max_nb, 3))
        else:
            cnt, stag, ssh, srl = self._saved
        if nl.npairs > 0:
            lib().or_history_restore(nl.npairs, _p(nl.pair_i, _i32p), _p(nl.pair_j, _i32p),
                                     _p(atoms.tag, _i32p), self.max_nb, _p(cnt, _i32p),
                                     _p(stag, _i32p), _p(ssh), _p(srl), _p(self.partner, _i32p),
                                     _p(self.shear), _p(self.rolling))
        self.setup_pending = False

    def touching(self, atoms: OracleAtoms, nl: OracleNeighbor) -> dict[tuple[int, int], np.ndarray]:
        """{(tag_i, tag_j): shear in the i->j convention} over touching pairs."""
        out = {}
        for nc in range(nl.npairs):
            if self.partner[nc] >= 0:
                ti = int(atoms.tag[nl.pair_i[nc]])
                tj = int(self.partner[nc])
                out[(ti, tj)] = self.shear[nc].copy()
        return out


# ------------------------------------------------------------------ pair styles


def _mix_e(e1, e2, p1, p2):
    # granular.py:94-96
    return 1.0 / ((1 - p1 * p1) / e1 + (1 - p2 * p2) / e2)


def _mix_g(e1, e2, p1, p2):
    # granular.py:99-103
    return 1.0 / (2 * (2 - p1) * (1 + p1) / e1 + 2 * (2 - p2) * (1 + p2) / e2)


class OraclePair:
    """Coefficients of one pair style, resolved as the reference constructors do."""

    def __init__(self, style: str, **kw):
        self.style = style
        self.sid = STYLE_IDS[style]
        self.P = OrPair()
        if style != "granular":
            # hooke.py:41-50, hooke_history.py:98-106, hertz_history.py:48-55
            self.P.kn = float(kw["kn"])
            self.P.kt = float(kw["kt"])
            self.P.gamman = float(kw["gamman"])
            damp = int(kw.get("dampflag", 1))
            self.P.gammat = 0.0 if damp == 0 else float(kw["gammat"])
            self.P.xmu = float(kw["xmu"])
            self.P.limit_damping = 1 if kw.get("limit_damping", False) else 0
            self.uses_history = style in ("hooke/history", "hertz/history")
        else:
            self._granular(**kw)

    def _granular(self, normal, normal_coeffs, tangential="none", tangential_coeffs=None,
                  damping="viscoelastic", limit_damping=False, rolling="none", rolling_coeffs=None):
        # granular.py:122-269
        nid = {"hooke": 0, "hertz": 1, "hertz/material": 2}[normal]
        did = {"none": 0, "velocity": 1, "mass_velocity": 2, "viscoelastic": 3, "tsuji": 4,
               "coeff_restitution": 5}[damping]
        tid = {"none": 0, "linear_nohistory": 1, "linear_history": 2, "mindlin": 3}[tangential]
        P = self.P
        P.normal_id, P.damping_id, P.tangential_id = nid, did, tid
        P.limit_damping = 1 if limit_damping else 0
        emod = poiss = 0.0
        if nid == 2:
            emod, cor, poiss = (float(c) for c in normal_coeffs)
            P.kn = (4.0 / 3.0) * _mix_e(emod, emod, poiss, poiss)
        else:
            P.kn, cor = (float(c) for c in normal_coeffs)
        if did in (4, 5):
            logcor = math.log(cor)
            if did == 4:
                d = (1.2728 - 4.2783 * cor + 11.087 * cor ** 2 - 22.348 * cor ** 3
                     + 27.467 * cor ** 4 - 18.022 * cor ** 5 + 4.8218 * cor ** 6)
                P.damp = d * math.sqrt(2.0)
            elif normal == "hooke":
                P.damp = -2 * logcor / math.sqrt(math.pi ** 2 + logcor ** 2)
            else:
                P.damp = (-1.22474487139158894067 * 1.82574185835055380345 * logcor
                          / math.sqrt(math.pi ** 2 + logcor ** 2))
        else:
            P.damp = float(cor)
        tc = list(tangential_coeffs or [])
        if tid == 1:
            P.xt, P.mu = float(tc[0]), float(tc[1])
        elif tid in (2, 3):
            k_raw, xt, mu = tc
            P.xt, P.mu = float(xt), float(mu)
            if k_raw is None:
                P.kt = 8.0 * _mix_g(emod, emod, poiss, poiss)
            else:
                P.kt = float(k_raw)
        # rolling resistance (rolling.py:16-27): coefficients k_roll, gamma_roll, mu_roll
        if rolling not in ("none", "sds", "epsd"):
            raise ValueError(f"unknown rolling model {rolling!r}")
        if rolling != "none":
            P.rolling_id = 1
            P.k_roll, P.gamma_roll, P.mu_roll = (float(c) for c in rolling_coeffs)
        self.uses_history = tid in (2, 3) or rolling != "none"

    def compute(self, atoms: OracleAtoms, nl: OracleNeighbor, hist: OracleHistory, dom: OracleDomain,
                dt: float, shearupdate: bool = True) -> None:
        if atoms.n == 0 or nl.npairs == 0:
            return
        box = dom.cbox()
        lib().or_pair_compute(self.sid, ctypes.byref(self.P), ctypes.byref(box), nl.npairs,
                              _p(nl.pair_i, _i32p), _p(nl.pair_j, _i32p), _p(atoms.x), _p(atoms.v),
                              _p(atoms.omega), _p(atoms.radius), _p(atoms.rmass), _p(atoms.tag, _i32p),
                              _p(hist.partner, _i32p), _p(hist.shear), _p(hist.rolling), ctypes.c_double(dt),
                              1 if shearupdate else 0, _p(atoms.f), _p(atoms.torque), _p(atoms.virial))


# ----------------------------------------------------------------------- fixes


def virial_chunks(n: int) -> int:
    """thermo.py:28-30"""
    return int(min(1024, max(64, 2.0 * math.sqrt(max(n, 1)))))


def virial_tensor(atoms: OracleAtoms, keflag: bool, chunks: int | None = None) -> np.ndarray:
    out = np.zeros(6)
    if atoms.n == 0:
        return out
    c = virial_chunks(atoms.n) if chunks is None else chunks
    lib().or_virial(atoms.n, _p(atoms.virial), _p(atoms.v), _p(atoms.rmass), 1 if keflag else 0, c,
                    _p(out))
    return out


def pressure_tensor(atoms: OracleAtoms, dom: OracleDomain, kinetic: bool = True) -> np.ndarray:
    """Computes.compute_pressure_tensor (thermo.py:141-170)."""
    if atoms.n == 0:
        return np.zeros(6)
    vol = dom.volume
    if vol <= 0.0:
        return np.zeros(6)
    return virial_tensor(atoms, kinetic) / vol


class OracleNVE:
    def initial_integrate(self, atoms, dt):
        lib().or_nve_initial(atoms.n, ctypes.c_double(dt), _p(atoms.x), _p(atoms.v), _p(atoms.omega),
                             _p(atoms.f), _p(atoms.torque), _p(atoms.radius), _p(atoms.rmass))

    def final_integrate(self, atoms, dt):
        lib().or_nve_final(atoms.n, ctypes.c_double(dt), _p(atoms.v), _p(atoms.omega), _p(atoms.f),
                           _p(atoms.torque), _p(atoms.radius), _p(atoms.rmass))


class OracleCundall:
    def __init__(self, gamma_lin=0.3, gamma_ang=0.3):
        self.gl, self.ga = float(gamma_lin), float(gamma_ang)

    def post_force(self, atoms, dt):
        lib().or_cundall(atoms.n, ctypes.c_double(self.gl), ctypes.c_double(self.ga), _p(atoms.f),
                         _p(atoms.torque), _p(atoms.v), _p(atoms.omega))


class _WallC(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int) for k in ("kind", "axis", "side", "history", "hertz", "limit_damping",
                                             "shear_axis", "has_axis_bounds")] + \
               [(k, ctypes.c_double) for k in ("coord", "vwall_n", "vwall_s", "c1", "c2", "radius", "axis_lo",
                                                "axis_hi", "kn", "kt", "gamman", "gammat", "xmu")]


class _OracleWall:
    history_update = True

    def _run(self, atoms, dt, w: _WallC):
        if self.shear is None or len(self.touch) != atoms.n:
            self.shear = np.zeros((atoms.n, 3))
            self.touch = np.zeros(atoms.n, dtype=np.int32)
        lib().or_wall(ctypes.byref(w), atoms.n, ctypes.c_double(dt), 1 if self.history_update else 0,
                      _p(atoms.x), _p(atoms.v), _p(atoms.omega), _p(atoms.radius), _p(atoms.rmass),
                      _p(atoms.f), _p(atoms.torque), _p(self.shear), _p(self.touch, _i32p))


class OracleWallGran(_OracleWall):
    """FixWallGran (EXTRA_FIX/wall_gran.py:39-242): plane wall, history or not, shear / wiggle motion."""

    def __init__(self, wall_axis, wall_side, wall_coord, kn, gamman, kt, gammat, xmu, dampflag=1, history=True,
                 limit_damping=False, shear_axis=-1, shear_vel=0.0, wiggle_amplitude=0.0, wiggle_period=0.0):
        self.w = _WallC(kind=0, axis=int(wall_axis), side=int(wall_side), history=1 if history else 0, hertz=0,
                        limit_damping=1 if limit_damping else 0, shear_axis=int(shear_axis), has_axis_bounds=0,
                        vwall_s=float(shear_vel), kn=float(kn), kt=float(kt), gamman=float(gamman),
                        gammat=0.0 if int(dampflag) == 0 else float(gammat), xmu=float(xmu))
        self.wall_coord = float(wall_coord)
        self.amp, self.period = float(wiggle_amplitude), float(wiggle_period)
        self.elapsed = 0.0
        self.shear = self.touch = None

    def setup(self, nsteps_total, dt, n):
        self.elapsed = 0.0

    def post_force(self, atoms, dt):
        # wall_gran.py:230-239
        coord, vn = self.wall_coord, 0.0
        if self.amp != 0.0:
            omega_w = 2.0 * math.pi / self.period
            arg = omega_w * self.elapsed
            coord += self.amp * (1.0 - math.cos(arg))
            vn = self.amp * omega_w * math.sin(arg)
        self.w.coord, self.w.vwall_n = coord, vn
        self._run(atoms, dt, self.w)
        self.elapsed += dt


class OracleWallGranRegion(_OracleWall):
    """FixWallGranRegion (EXTRA_FIX/wall_gran_region.py:33-290): the side of a cylinder region."""

    def __init__(self, axis=2, c1=0.0, c2=0.0, radius=1.0, side="in", axis_lo=None, axis_hi=None, fstyle="hooke",
                 kn=1e5, gamman=0.0, kt=None, gammat=None, xmu=0.0, dampflag=1, history=None, limit_damping=False):
        if isinstance(axis, str):
            axis = {"x": 0, "y": 1, "z": 2}[axis.lower()]
        if isinstance(side, str):
            sd = -1 if side.lower() in ("in", "inside", "-1") else 1
        else:
            sd = -1 if side < 0 else 1
        fstyle = fstyle.lower()
        gt = float(gammat) if gammat is not None else 0.5 * float(gamman)
        self.w = _WallC(kind=1, axis=int(axis), side=sd,
                        history=1 if (fstyle.endswith("history") if history is None else history) else 0,
                        hertz=1 if "hertz" in fstyle else 0, limit_damping=1 if limit_damping else 0, shear_axis=-1,
                        has_axis_bounds=1 if (axis_lo is not None or axis_hi is not None) else 0,
                        c1=float(c1), c2=float(c2), radius=float(radius),
                        axis_lo=float(axis_lo) if axis_lo is not None else -1e30,
                        axis_hi=float(axis_hi) if axis_hi is not None else 1e30,
                        kn=float(kn), kt=float(kt) if kt is not None else 2.0 / 7.0 * float(kn), gamman=float(gamman),
                        gammat=0.0 if int(dampflag) == 0 else gt, xmu=float(xmu))
        self.shear = self.touch = None

    def post_force(self, atoms, dt):
        self._run(atoms, dt, self.w)


PRESSURE_STYLES = ("pressure", "pressure/mean")


@dataclass
class _Axis:
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
    lo_target: float = 0.0
    hi_target: float = 0.0
    cumulative_shift: float = 0.0
    # volume style and vol/balance/p (deform_pressure.py:358-385, 905-956)
    vol_start: float = 0.0
    substyle: str = ""
    fixed: int = -1
    dynamic1: int = -1
    dynamic2: int = -1
    saved: bool = False
    prior_rate: float = 0.0
    prior_pressure: float = 0.0
    pressure_now: float = 0.0
    cumulative_vshift: list = field(default_factory=lambda: [0.0, 0.0, 0.0])


class OracleDeform:
    """
    FixDeformPressure restricted to orthogonal x/y/z styles none, erate, trate,
    vel, wiggle, final, delta, scale, pressure, pressure/mean and volume, the
    box style (volume or pressure), with couple, max/rate, normalize/pressure,
    vol/balance/p and remap x|v|none.  The arithmetic is that of the host path
    (deform_pressure.py:758-1001, 1113-1219); the device path
    (deform_pressure.py:598-702) computes the same expressions.
    """

    def __init__(self, domain: OracleDomain, axes: dict, couple="none", max_rate=0.0,
                 normalize_pressure=False, remap="x", nevery=1, box=None, vol_balance_p=False):
        self.domain = domain
        self.axes = [_Axis() for _ in range(3)]
        self.set_box = _Axis()
        if box is not None:
            self.set_box.style = box["style"]
            for k, v in box.items():
                if k != "style":
                    setattr(self.set_box, k, float(v))
        self.vol_balance_p = bool(vol_balance_p)
        for name, spec in (axes or {}).items():
            a = self.axes["xyz".index(name)]
            for k, v in spec.items():
                setattr(a, k, v if isinstance(v, str) else float(v)) if k != "style" else setattr(a, "style", v)
        self.couple = couple
        self.max_rate = float(max_rate)
        self.normalize = bool(normalize_pressure)
        self.remap = remap
        self.nevery = int(nevery)
        if couple != "none":
            # deform_pressure.py:332-356
            idx = [i for i, c in enumerate("xyz") if c in couple]
            ref = next(i for i in idx if self.axes[i].style in PRESSURE_STYLES)
            for i in idx:
                s = self.axes[i]
                if s.style == "none":
                    s.style = self.axes[ref].style
                    s.ptarget = self.axes[ref].ptarget
                    s.pgain = self.axes[ref].pgain
        # _setup_volume_links (deform_pressure.py:358-385)
        for i in range(3):
            s = self.axes[i]
            if s.style != "volume":
                continue
            o1, o2 = (i + 1) % 3, (i + 2) % 3
            s1, s2 = self.axes[o1].style, self.axes[o2].style
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
        self.nsteps = 0
        self.step_count = 0
        self.nsteps_total = 0
        self.chunks = 64
        self.history_update = True
        self.force_reneighbor = False

    def setup(self, nsteps_total, dt, natoms):
        # deform_pressure.py:392-445
        dom = self.domain
        self.nsteps = 0
        self.nsteps_total = int(nsteps_total)
        for i in range(3):
            s = self.axes[i]
            s.lo_start = float(dom.boxlo[i])
            s.hi_start = float(dom.boxhi[i])
            s.lo_target, s.hi_target = s.lo_start, s.hi_start
            s.cumulative_shift = 0.0
            s.vol_start = dom.volume
            s.saved = False
        self.set_box.vol_start = dom.volume
        self.set_box.cumulative_vshift = [0.0, 0.0, 0.0]
        dom.h_rate = self._strain_h_rate(dt)
        dom.vremap = self.remap == "v"
        self.chunks = virial_chunks(natoms)

    def _strain_h_rate(self, dt):
        # deform_pressure.py:447-472 (x/y/z part)
        h = np.zeros(6)
        delt = self.nsteps_total * dt
        for i in range(3):
            s = self.axes[i]
            length = s.hi_start - s.lo_start
            if s.style in ("erate", "trate"):
                h[i] = s.rate * length
            elif s.style == "vel":
                h[i] = s.vel
            elif s.style == "wiggle":
                h[i] = 2.0 * math.pi / s.tperiod * s.amplitude
            elif s.style in ("final", "delta", "scale") and delt > 0.0:
                if s.style == "final":
                    stop = s.fhi - s.flo
                elif s.style == "delta":
                    stop = length + s.dhi - s.dlo
                else:
                    stop = s.scale * length
                h[i] = (stop - length) / delt
        return h

    def _adjust_linked_rates(self, e_larger, e_smaller, e3, vi, v, dt):
        # deform_pressure.py:858-870
        m = self.max_rate
        e_lim_pos = (vi - v * (1 + m * dt)) / (v * (1 + m * dt) * dt)
        e_lim_neg = (vi - v * (1 - m * dt)) / (v * (1 - m * dt) * dt)
        if e_larger * e3 >= 0:
            if e_larger > 0.0:
                return e_lim_neg, -m
            return e_lim_pos, m
        if e_larger > 0.0:
            return m, e_lim_pos
        return -m, e_lim_neg

    def _apply_volume(self, prd, dt):
        # deform_pressure.py:872-956
        linked_done, e2_linked = False, 0.0
        for i in range(3):
            s = self.axes[i]
            if s.style != "volume":
                continue
            v0 = s.vol_start
            if s.substyle == "one_from_one":
                d1, fx = self.axes[s.dynamic1], self.axes[s.fixed]
                half = 0.5 * (v0 / (d1.hi_target - d1.lo_target) / (fx.hi_start - fx.lo_start))
            elif s.substyle == "one_from_two":
                d1, d2 = self.axes[s.dynamic1], self.axes[s.dynamic2]
                half = 0.5 * (v0 / (d1.hi_target - d1.lo_target) / (d2.hi_target - d2.lo_target))
            elif not self.vol_balance_p:
                d1, fx = self.axes[s.dynamic1], self.axes[s.fixed]
                half = 0.5 * math.sqrt(v0 * (s.hi_start - s.lo_start) / (d1.hi_target - d1.lo_target)
                                       / (fx.hi_start - fx.lo_start))
            else:
                fx, d1 = self.axes[s.fixed], self.axes[s.dynamic1]
                l1i, l2i, l3i = float(prd[i]), float(prd[s.fixed]), float(prd[s.dynamic1])
                l3 = d1.hi_target - d1.lo_target
                vi = l1i * l2i * l3i
                v = l3 * l1i * l2i
                e3 = (l3 / l3i - 1.0) / dt
                e1i, e2i = s.prior_rate, fx.prior_rate
                p1, p2 = s.pressure_now, fx.pressure_now
                p1i, p2i = s.prior_pressure, fx.prior_pressure
                if e3 == 0.0:
                    half = 0.5 * l1i
                elif e1i == 0.0 or e2i == 0.0 or (p2 == p2i and p1 == p1i):
                    half = 0.5 * math.sqrt(s.vol_start * l1i / l3 / l2i)
                elif linked_done:
                    half = 0.5 * l1i * (1.0 + e2_linked * dt)
                else:
                    denominator = p2 - p2i + e2i * ((p1 - p1i) / e1i)
                    if denominator != 0.0:
                        e1 = (((p2 - p2i) * (vi - v) / (v * dt)) - e2i * (p1 - p2)) / denominator
                    else:
                        e1 = e2i
                    e2 = (vi - v * (1 + e1 * dt)) / (v * (1 + e1 * dt) * dt)
                    if self.max_rate != 0.0 and (abs(e1) > self.max_rate or abs(e2) > self.max_rate):
                        if abs(e1) > abs(e2):
                            e1, e2 = self._adjust_linked_rates(e1, e2, e3, vi, v, dt)
                        else:
                            e2, e1 = self._adjust_linked_rates(e2, e1, e3, vi, v, dt)
                    half = 0.5 * l1i * (1.0 + e1 * dt)
                    linked_done, e2_linked = True, e2
            mid = 0.5 * (s.lo_start + s.hi_start)
            s.lo_target, s.hi_target = mid - half, mid + half

    def _apply_box(self, tensor, dt):
        # deform_pressure.py:958-991
        sb = self.set_box
        if sb.style == "volume":
            v = 1.0
            for i in range(3):
                v *= self.axes[i].hi_target - self.axes[i].lo_target
            scale = (sb.vol_start / v) ** (1.0 / 3.0)
            for i in range(3):
                s = self.axes[i]
                half = 0.5 * (s.hi_target - s.lo_target) * scale
                mid = 0.5 * (s.lo_start + s.hi_start)
                s.lo_target, s.hi_target = mid - half, mid + half
            return
        v_rate = self._limit(sb.pgain * (float(np.mean(tensor[:3])) - sb.ptarget), sb.ptarget)
        for i in range(3):
            s = self.axes[i]
            shift = (s.hi_target - s.lo_target) * dt * v_rate
            sb.cumulative_vshift[i] += shift
            if s.style == "none":
                s.lo_target, s.hi_target = s.lo_start, s.hi_start
            s.lo_target -= 0.5 * sb.cumulative_vshift[i]
            s.hi_target += 0.5 * sb.cumulative_vshift[i]

    def _limit(self, rate, ptarget):
        # deform_pressure.py:737-752
        if self.normalize:
            if ptarget == 0.0:
                if rate != 0.0:
                    rate = math.copysign(self.max_rate, rate)
            else:
                rate /= abs(ptarget)
        if self.max_rate != 0.0 and abs(rate) > self.max_rate:
            rate = math.copysign(self.max_rate, rate)
        return rate

    def end_of_step(self, atoms: OracleAtoms, dt: float, chunks: int | None = None) -> np.ndarray:
        """Returns the pressure tensor it servoed on (zeros when none was needed)."""
        dom = self.domain
        self.step_count += 1
        self.nsteps += 1
        if self.step_count % self.nevery != 0:
            return np.zeros(6)
        axes = self.axes
        needs_p = (any(s.style in PRESSURE_STYLES for s in axes) or self.set_box.style == "pressure"
                   or self.vol_balance_p)
        tensor = np.zeros(6)
        p = np.zeros(3)
        if needs_p:
            vol = dom.volume
            tensor = (virial_tensor(atoms, True, self.chunks if chunks is None else chunks) / vol
                      if atoms.n and vol > 0.0 else np.zeros(6))
            scalar = float(np.mean(tensor[:3]))
            if self.couple == "xyz":
                p[:] = np.mean(tensor[:3])
            elif self.couple in ("xy", "yz", "xz"):
                idx = [i for i, c in enumerate("xyz") if c in self.couple]
                other = [i for i in range(3) if i not in idx]
                p[idx] = np.mean(tensor[idx])
                for i in other:
                    p[i] = tensor[i]
            else:
                for i in range(3):
                    if axes[i].style == "pressure":
                        p[i] = tensor[i]
                    elif axes[i].style == "pressure/mean":
                        p[i] = scalar
            # deform_pressure.py:1144-1151
            for i in range(3):
                s = axes[i]
                s.pressure_now = float(tensor[i])
                if not s.saved:
                    s.saved = True
                    s.prior_rate = 0.0
                    s.prior_pressure = float(tensor[i])
        old_prd = dom.prd.copy()
        old_lo = dom.boxlo.copy()
        elapsed = self.nsteps * dt
        frac = self.nsteps / self.nsteps_total if self.nsteps_total > 0 else 0.0
        for i in range(3):
            # _apply_strain (deform_pressure.py:770-805)
            s = axes[i]
            if s.style == "none":
                s.lo_target, s.hi_target = float(dom.boxlo[i]), float(dom.boxhi[i])
            elif s.style == "trate":
                mid = 0.5 * (s.lo_start + s.hi_start)
                half = 0.5 * (s.hi_start - s.lo_start) * math.exp(s.rate * elapsed)
                s.lo_target, s.hi_target = mid - half, mid + half
            elif s.style == "erate":
                shift = 0.5 * elapsed * s.rate * (s.hi_start - s.lo_start)
                s.lo_target, s.hi_target = s.lo_start - shift, s.hi_start + shift
            elif s.style == "vel":
                shift = 0.5 * elapsed * s.vel
                s.lo_target, s.hi_target = s.lo_start - shift, s.hi_start + shift
            elif s.style == "wiggle":
                shift = 0.5 * s.amplitude * math.sin(2.0 * math.pi * elapsed / s.tperiod)
                s.lo_target, s.hi_target = s.lo_start - shift, s.hi_start + shift
            elif s.style in ("final", "delta", "scale"):
                if s.style == "final":
                    lo_stop, hi_stop = s.flo, s.fhi
                elif s.style == "delta":
                    lo_stop, hi_stop = s.lo_start + s.dlo, s.hi_start + s.dhi
                else:
                    mid = 0.5 * (s.lo_start + s.hi_start)
                    half = 0.5 * s.scale * (s.hi_start - s.lo_start)
                    lo_stop, hi_stop = mid - half, mid + half
                s.lo_target = s.lo_start + frac * (lo_stop - s.lo_start)
                s.hi_target = s.hi_start + frac * (hi_stop - s.hi_start)
        if needs_p:
            # _apply_pressure (deform_pressure.py:833-847)
            for i in range(3):
                s = axes[i]
                if s.style not in PRESSURE_STYLES:
                    continue
                rate = self._limit(s.pgain * (p[i] - s.ptarget), s.ptarget)
                s.cumulative_shift += dt * rate * float(old_prd[i])
                s.lo_target = s.lo_start - 0.5 * s.cumulative_shift
                s.hi_target = s.hi_start + 0.5 * s.cumulative_shift
        self._apply_volume(old_prd, dt)
        if self.set_box.style != "none":
            self._apply_box(tensor, dt)
        new_lo = np.array([axes[i].lo_target for i in range(3)])
        new_hi = np.array([axes[i].hi_target for i in range(3)])
        new_prd = new_hi - new_lo
        if np.any(new_prd <= 0.0):
            raise RuntimeError(
                f"fix deform/pressure drove a box dimension to {new_prd}, which is not positive; "
                "check the gain, max/rate or strain rate")
        if needs_p:
            # deform_pressure.py:1177-1184
            for i in range(3):
                s = axes[i]
                s.prior_pressure = float(tensor[i])
                s.prior_rate = ((s.hi_target - s.lo_target) / old_prd[i] - 1.0) / dt
        h_rate = np.zeros(6)
        h_rate[:3] = (new_prd - old_prd) / dt
        if self.remap == "x" and atoms.n > 0:
            lib().or_remap_x(atoms.n, _p(atoms.x), _p(np.ascontiguousarray(old_lo)),
                             _p(np.ascontiguousarray(old_prd)), _p(np.ascontiguousarray(new_lo)),
                             _p(np.ascontiguousarray(new_prd)))
        dom.boxlo, dom.boxhi = new_lo, new_hi
        dom.h_rate = h_rate
        dom.vremap = self.remap == "v"
        return tensor


# ------------------------------------------------------------------ simulation


class OracleSim:
    """Simulation (simulation.py:22-332) for one pair style + NVE + optional fixes."""

    def __init__(self, domain: OracleDomain, atoms: OracleAtoms, neighbor: OracleNeighbor,
                 history: OracleHistory, pair: OraclePair, dt: float, fixes=()):
        self.domain, self.atoms, self.neighbor, self.history, self.pair = domain, atoms, neighbor, history, pair
        self.dt = float(dt)
        self.timestep = 0
        self.integrator = OracleNVE()
        self.fixes = list(fixes)
        self.setup_done = False
        self.last_pressure = np.zeros(6)

    def _reneighbor(self, force=False) -> bool:
        forced = force
        for fx in self.fixes:
            if getattr(fx, "force_reneighbor", False):
                forced = True
                fx.force_reneighbor = False
        if not self.neighbor.decide(self.atoms, self.timestep) and not forced:
            return False
        self.history.save_state(self.atoms, self.neighbor)
        lib().or_pbc(ctypes.byref(self.domain.cbox()), self.atoms.n, _p(self.atoms.x), _p(self.atoms.v))
        self.neighbor.build(self.atoms)
        self.history.restore_state(self.atoms, self.neighbor)
        return True

    def setup(self, nsteps_total: int = 0) -> None:
        for fx in self.fixes:
            if hasattr(fx, "setup"):
                fx.setup(nsteps_total, self.dt, self.atoms.n)
        self.setup_done = True
        self.atoms.clear_forces()
        self._reneighbor(force=True)
        if self.pair is not None:
            self.pair.compute(self.atoms, self.neighbor, self.history, self.domain, self.dt, shearupdate=False)
        # simulation.py:198-203: the setup force evaluation does not advance fix histories
        for fx in self.fixes:
            fx.history_update = False
        for fx in self.fixes:
            if hasattr(fx, "post_force"):
                fx.post_force(self.atoms, self.dt)
        for fx in self.fixes:
            fx.history_update = True

    def step(self) -> None:
        self.timestep += 1
        self.integrator.initial_integrate(self.atoms, self.dt)
        self._reneighbor()
        self.atoms.clear_forces()
        if self.pair is not None:
            self.pair.compute(self.atoms, self.neighbor, self.history, self.domain, self.dt)
        for fx in self.fixes:
            if hasattr(fx, "post_force"):
                fx.post_force(self.atoms, self.dt)
        self.integrator.final_integrate(self.atoms, self.dt)
        for fx in self.fixes:
            if hasattr(fx, "end_of_step"):
                p = fx.end_of_step(self.atoms, self.dt)
                if p is not None:
                    self.last_pressure = p

    def run(self, nsteps: int) -> None:
        # Simulation.run (simulation.py:320-332): fix setup, then the setup
        # force evaluation at the start of every run (run_pre on by default).
        self.setup(nsteps)
        for _ in range(nsteps):
            self.step()

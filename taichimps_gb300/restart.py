"""
LAMMPS binary restart files for ``atom_style sphere``, with the per-contact
shear history (fix NEIGH_HISTORY) -- the reference's restart API
(src/taichimps/restart.py: RestartData, read_restart :196, parse_neigh_history
:438, write_restart :505) for systems of a million spheres.

The file is a flat little-endian sequence (LAMMPS write_restart.cpp,
read_restart.cpp, lmprestart.h):

    magic "LammpS RestartT\\0", int endian (1), int format revision (3)
    header       (int flag, payload) pairs up to flag -1
    groups       int count, then that many length-prefixed names
    type arrays  (flag, payload) pairs up to -1
    force field  (flag, payload) pairs up to -1; PAIR carries the pair
                 style's own binary settings after its name
    fixes        fixes with global state (id, style, blob), then fixes with
                 per-atom state (id, style, largest record)
    file layout  (flag, payload) pairs up to -1
    atoms        PERPROC chunks: int flag, int count, count doubles
    magic again

An atom record is [length, x, y, z, tag, type, mask, image, vx, vy, vz,
radius, rmass, omegax, omegay, omegaz, fix data...], the integers carried in
a double's bits.  FixNeighHistory's data is [length, npartner, (partner tag,
value[dnum]) per partner]: every contact under both of its atoms, each copy
in that atom's i -> j sense (the two are exact negatives).

Records are packed and unpacked as numpy arrays; only the walk from one
variable-length atom record to the next is a loop.  The contact history is
read straight from the GPU's full neighbor list, which already holds both
copies of every contact, so nothing is expanded on the host.  Beyond the
reference: a rolling-resistance history (pair granular ... rolling) is
written as three more values per contact (dnum 6, the LAMMPS order: tangential
then rolling) and read back by ContactHistory.load_restart.
"""

from __future__ import annotations

import struct
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

MAGIC = b"LammpS RestartT\x00"
ENDIAN = 0x0001
FORMAT_REVISION = 3
# LAMMPS turns the version string into a release date (utils::date2num), so
# it must be a release date; the reference's writer states this one.
VERSION_STRING = "2 Sep 2026"

# The section flags, in the order LAMMPS numbers them (lmprestart.h); the
# order is the format.
_FLAG_ORDER = (
    "VERSION SMALLINT TAGINT BIGINT UNITS NTIMESTEP DIMENSION NPROCS PROCGRID NEWTON_PAIR NEWTON_BOND "
    "XPERIODIC YPERIODIC ZPERIODIC BOUNDARY ATOM_STYLE NATOMS NTYPES NBONDS NBONDTYPES BOND_PER_ATOM "
    "NANGLES NANGLETYPES ANGLE_PER_ATOM NDIHEDRALS NDIHEDRALTYPES DIHEDRAL_PER_ATOM NIMPROPERS "
    "NIMPROPERTYPES IMPROPER_PER_ATOM TRICLINIC BOXLO BOXHI XY XZ YZ SPECIAL_LJ SPECIAL_COUL MASS PAIR "
    "BOND ANGLE DIHEDRAL IMPROPER MULTIPROC MPIIO PROCSPERFILE PERPROC IMAGEINT BOUNDMIN TIMESTEP ATOM_ID "
    "ATOM_MAP_STYLE ATOM_MAP_USER ATOM_SORTFREQ ATOM_SORTBIN COMM_MODE COMM_CUTOFF COMM_VEL NO_PAIR "
    "EXTRA_BOND_PER_ATOM EXTRA_ANGLE_PER_ATOM EXTRA_DIHEDRAL_PER_ATOM EXTRA_IMPROPER_PER_ATOM "
    "EXTRA_SPECIAL_PER_ATOM ATOM_MAXSPECIAL NELLIPSOIDS NLINES NTRIS NBODIES ATIME ATIMESTEP LABELMAP "
    "TRICLINIC_GENERAL ROTATE_G2R ATOM_MAXEXCHANGE"
).split()
FLAG = {name: value for value, name in enumerate(_FLAG_ORDER)}

# payload kind of each flag
_KIND = {}
for _n in ("SMALLINT TAGINT BIGINT IMAGEINT DIMENSION NPROCS NEWTON_PAIR NEWTON_BOND XPERIODIC YPERIODIC "
           "ZPERIODIC NTYPES NBONDTYPES BOND_PER_ATOM NANGLETYPES ANGLE_PER_ATOM NDIHEDRALTYPES "
           "DIHEDRAL_PER_ATOM NIMPROPERTYPES IMPROPER_PER_ATOM TRICLINIC TRICLINIC_GENERAL MULTIPROC MPIIO "
           "PROCSPERFILE ATOM_ID ATOM_MAP_STYLE ATOM_MAP_USER ATOM_SORTFREQ COMM_MODE COMM_VEL NO_PAIR "
           "EXTRA_BOND_PER_ATOM EXTRA_ANGLE_PER_ATOM EXTRA_DIHEDRAL_PER_ATOM EXTRA_IMPROPER_PER_ATOM "
           "EXTRA_SPECIAL_PER_ATOM ATOM_MAXSPECIAL ATOM_MAXEXCHANGE LABELMAP").split():
    _KIND[FLAG[_n]] = "int"
for _n in "NTIMESTEP NATOMS NBONDS NANGLES NDIHEDRALS NIMPROPERS NELLIPSOIDS NLINES NTRIS NBODIES ATIMESTEP".split():
    _KIND[FLAG[_n]] = "bigint"
for _n in "TIMESTEP XY XZ YZ ATIME ATOM_SORTBIN COMM_CUTOFF".split():
    _KIND[FLAG[_n]] = "double"
for _n in "VERSION UNITS ATOM_STYLE".split():
    _KIND[FLAG[_n]] = "string"
for _n in "PROCGRID BOUNDARY".split():
    _KIND[FLAG[_n]] = "ints"
for _n in "BOXLO BOXHI SPECIAL_LJ SPECIAL_COUL BOUNDMIN ROTATE_G2R MASS".split():
    _KIND[FLAG[_n]] = "doubles"
_KIND[FLAG["PAIR"]] = "pair"
_KIND[FLAG["NO_PAIR"]] = "string"

_BOUNDARY = {0: "p", 1: "f", 2: "s", 3: "m"}
_GRAN_SLOTS = ("normal", "damping", "tangential", "rolling", "twisting", "heat")
_LEGACY_STYLES = ("gran/hooke", "gran/hooke/history", "gran/hertz/history")
# FixNeighHistory's id, by pair style (a reader matches per-atom data on id and style)
_HISTORY_FIX_ID = {"granular": "NEIGH_HISTORY_GRANULAR0", "gran/hooke/history": "NEIGH_HISTORY_HH0",
                   "gran/hertz/history": "NEIGH_HISTORY_HH0"}
# image flags (512, 512, 512): no periodic crossing yet
_IMAGE_ZERO = (512 << 20) | (512 << 10) | 512
_BASE_WORDS = 16  # an atom_style sphere record without fix data


def _values_2d(vals, m: int) -> np.ndarray:
    """Per-contact values as an (m, dnum) array (dnum 3 when there are none)."""
    a = np.asarray(vals, dtype=np.float64)
    return a.reshape(m, -1) if m else np.zeros((0, a.shape[-1] if a.ndim == 2 and a.shape[-1] else 3))


def _bits_as_double(v) -> np.ndarray:
    """int64 values carried in doubles' bits (LAMMPS' ubuf)."""
    return np.ascontiguousarray(np.asarray(v, dtype=np.int64)).view(np.float64)


def _double_as_bits(v) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(v, dtype=np.float64)).view(np.int64)


class RaggedRecords:
    """Per-atom variable-length fix data: ``len``, indexing, iteration and truth like a list of
    arrays, held as one flat array and offsets."""

    def __init__(self, flat: np.ndarray, offsets: np.ndarray) -> None:
        self.flat, self.offsets = flat, offsets

    def __len__(self) -> int:
        return len(self.offsets) - 1

    def __bool__(self) -> bool:
        return len(self) > 0

    def __getitem__(self, i: int) -> np.ndarray:
        if i < 0:
            i += len(self)
        return self.flat[self.offsets[i]:self.offsets[i + 1]]

    def __iter__(self):
        for i in range(len(self)):
            yield self[i]


@dataclass
class RestartData:
    """What a restart file holds that this path can use (the reference's RestartData fields)."""

    timestep: int = 0
    dt: float = 0.0
    natoms: int = 0
    ntypes: int = 1
    dimension: int = 3
    units: str = "si"
    atom_style: str = "sphere"
    boxlo: list = field(default_factory=lambda: [0.0, 0.0, 0.0])
    boxhi: list = field(default_factory=lambda: [0.0, 0.0, 0.0])
    tilt: list = field(default_factory=lambda: [0.0, 0.0, 0.0])
    boundary: tuple = ("p", "p", "p")
    pair_style: str = ""
    pair_settings: dict = field(default_factory=dict)
    fix_global: dict = field(default_factory=dict)
    fix_peratom_styles: list = field(default_factory=list)
    tag: np.ndarray = field(default_factory=lambda: np.zeros(0, dtype=np.int32))
    atom_type: np.ndarray = field(default_factory=lambda: np.zeros(0, dtype=np.int32))
    x: np.ndarray = field(default_factory=lambda: np.zeros((0, 3)))
    v: np.ndarray = field(default_factory=lambda: np.zeros((0, 3)))
    omega: np.ndarray = field(default_factory=lambda: np.zeros((0, 3)))
    radius: np.ndarray = field(default_factory=lambda: np.zeros(0))
    rmass: np.ndarray = field(default_factory=lambda: np.zeros(0))
    fix_extra: RaggedRecords = field(default_factory=lambda: RaggedRecords(np.zeros(0), np.zeros(1, np.int64)))

    @property
    def density(self) -> np.ndarray:
        """rmass / (4/3 pi r^3): what AtomSystem.add_particles takes (0 for a zero radius)."""
        vol = (4.0 / 3.0) * np.pi * self.radius ** 3
        return np.divide(self.rmass, vol, out=np.zeros_like(self.rmass), where=vol > 0)

    def neigh_history(self):
        """Every per-atom NEIGH_HISTORY record at once: (atom index, partner tag, values[dnum]) as flat
        arrays in file order, dnum read from the records (0 contacts: dnum 3).  The bulk form of
        parse_neigh_history over fix_extra."""
        return _neigh_history_flat(self.fix_extra)


# ------------------------------------------------------------------ reading


class _Cursor:
    def __init__(self, raw: bytes) -> None:
        self.raw, self.pos = raw, 0

    def take(self, n: int) -> bytes:
        if n < 0 or self.pos + n > len(self.raw):
            raise ValueError("restart file ended mid-record")
        b = self.raw[self.pos:self.pos + n]
        self.pos += n
        return b

    def i32(self) -> int:
        return struct.unpack_from("<i", self.take(4))[0]

    def i64(self) -> int:
        return struct.unpack_from("<q", self.take(8))[0]

    def f64(self) -> float:
        return struct.unpack_from("<d", self.take(8))[0]

    def ints(self) -> list:
        n = self.i32()
        return list(struct.unpack(f"<{n}i", self.take(4 * n)))

    def doubles(self) -> list:
        n = self.i32()
        return list(struct.unpack(f"<{n}d", self.take(8 * n)))

    def string(self) -> str:
        return self.take(self.i32()).rstrip(b"\x00").decode("utf-8")


def read_restart(path) -> RestartData:
    """A single-file LAMMPS restart of atom_style sphere (read_restart.cpp), history records kept
    per atom in fix_extra.  Multi-file restarts (`write_restart file.%`) raise."""
    raw = Path(path).read_bytes()
    c = _Cursor(raw)
    if c.take(len(MAGIC)) != MAGIC:
        raise ValueError(f"{path} is not a LAMMPS restart file")
    if c.i32() != ENDIAN:
        raise ValueError(f"{path} was written on a machine with the opposite byte order")
    rev = c.i32()
    if rev > FORMAT_REVISION:
        raise ValueError(f"{path} uses restart format revision {rev}; this reader understands up to "
                         f"{FORMAT_REVISION}")
    d = RestartData()
    _flags(c, d)                       # header
    ngroup, seen = c.i32(), 0          # groups: deleted groups are zero-length names
    while seen < ngroup:
        if c.take(c.i32()):
            seen += 1
    _flags(c, d)                       # type arrays
    _flags(c, d)                       # force field
    for _ in range(c.i32()):           # fixes with global state
        c.take(c.i32())
        style = c.take(c.i32()).rstrip(b"\x00").decode("utf-8")
        d.fix_global[style] = c.take(c.i32())
    for _ in range(c.i32()):           # fixes with per-atom state
        c.take(c.i32())
        d.fix_peratom_styles.append(c.take(c.i32()).rstrip(b"\x00").decode("utf-8"))
        c.i32()
    _flags(c, d)                       # file layout
    _atoms(c, d)
    return d


def _flags(c: _Cursor, d: RestartData) -> None:
    while True:
        flag = c.i32()
        if flag < 0:
            return
        kind = _KIND.get(flag)
        if kind == "int":
            v = c.i32()
            if flag == FLAG["DIMENSION"]:
                d.dimension = v
            elif flag == FLAG["NTYPES"]:
                d.ntypes = v
            elif flag == FLAG["MULTIPROC"] and v:
                raise ValueError("multi-processor restart files are not supported; write a single-file "
                                 "restart instead")
        elif kind == "bigint":
            v = c.i64()
            if flag == FLAG["NTIMESTEP"]:
                d.timestep = v
            elif flag == FLAG["NATOMS"]:
                d.natoms = v
        elif kind == "double":
            v = c.f64()
            if flag == FLAG["TIMESTEP"]:
                d.dt = v
            elif flag in (FLAG["XY"], FLAG["XZ"], FLAG["YZ"]):
                d.tilt[flag - FLAG["XY"]] = v
        elif kind == "string" and flag != FLAG["NO_PAIR"]:
            v = c.string()
            if flag == FLAG["UNITS"]:
                d.units = v
            elif flag == FLAG["ATOM_STYLE"]:
                d.atom_style = v.split()[0]
                for _ in range(c.i32()):  # the style's arguments: a count, then strings
                    c.string()
        elif kind == "ints":
            v = c.ints()
            if flag == FLAG["BOUNDARY"]:
                d.boundary = tuple(_BOUNDARY.get(v[2 * k], "f") for k in range(3))
        elif kind == "doubles":
            v = c.doubles()
            if flag == FLAG["BOXLO"]:
                d.boxlo = v
            elif flag == FLAG["BOXHI"]:
                d.boxhi = v
        elif flag == FLAG["NO_PAIR"]:
            d.pair_style = c.string()
        elif kind == "pair":
            d.pair_style = c.string()
            _pair_settings(c, d)
        else:
            raise ValueError(f"unknown restart header flag {flag}; the file may have been written by an "
                             "incompatible LAMMPS version")


def _pair_settings(c: _Cursor, d: RestartData) -> None:
    """The pair style's own binary (PairGranular / PairGranHookeHistory::write_restart): it carries no
    flags, so only styles whose layout is known can be read past."""
    style, nt = d.pair_style, d.ntypes
    if style == "granular":
        models = []
        for _ in range(c.i32()):
            m = {}
            for slot in _GRAN_SLOTS:
                name = c.take(c.i32()).decode("utf-8")  # not NUL-terminated here
                m[slot] = (name, [c.f64() for _ in range(c.i32())])
            m["limit_damping"] = c.i32()
            models.append(m)
        for i in range(nt):  # setflag, cutoff and model index per type pair (upper triangle)
            for _ in range(i, nt):
                if c.i32():
                    c.f64()
                    c.i32()
        d.pair_settings = {"models": models}
    elif style in _LEGACY_STYLES:
        keys = ("kn", "kt", "gamman", "gammat", "xmu")
        s = {k: c.f64() for k in keys}
        s["dampflag"] = c.i32()
        s["limit_damping"] = c.i32()
        for i in range(nt):
            for _ in range(i, nt):
                c.i32()
        d.pair_settings = s
    else:
        raise ValueError(f"restart file stores pair_style {style!r}, whose binary layout is unknown here; "
                         "its bytes cannot be skipped safely")


def _atoms(c: _Cursor, d: RestartData) -> None:
    chunks = []
    while c.pos + len(MAGIC) <= len(c.raw) and c.raw[c.pos:c.pos + len(MAGIC)] != MAGIC:
        if c.i32() != FLAG["PERPROC"]:
            raise ValueError("expected a PERPROC chunk of atom records")
        m = c.i32()
        chunks.append(np.frombuffer(c.take(8 * m), dtype="<f8"))
    buf = np.concatenate(chunks) if chunks else np.zeros(0)
    # walk the variable-length records: each one starts with its own length
    starts = []
    m, nd = 0, len(buf)
    while m < nd:
        size = int(buf[m])
        if size < _BASE_WORDS:
            raise ValueError(f"atom record of {size} doubles is too short for atom_style sphere")
        starts.append(m)
        m += size
    s = np.asarray(starts, dtype=np.int64)
    size = buf[s].astype(np.int64) if len(s) else np.zeros(0, np.int64)
    col = lambda k: buf[s + k]
    d.x = np.stack([col(1), col(2), col(3)], axis=1) if len(s) else np.zeros((0, 3))
    d.tag = _double_as_bits(col(4)).astype(np.int32)
    d.atom_type = _double_as_bits(col(5)).astype(np.int32)
    d.v = np.stack([col(8), col(9), col(10)], axis=1) if len(s) else np.zeros((0, 3))
    d.radius = col(11).copy()
    d.rmass = col(12).copy()
    d.omega = np.stack([col(13), col(14), col(15)], axis=1) if len(s) else np.zeros((0, 3))
    # the fix data of each record, flattened
    extra_len = size - _BASE_WORDS
    offsets = np.zeros(len(s) + 1, dtype=np.int64)
    np.cumsum(extra_len, out=offsets[1:])
    if offsets[-1]:
        src = np.repeat(s + _BASE_WORDS - offsets[:-1], extra_len) + np.arange(offsets[-1])
        flat = buf[src].copy()
    else:
        flat = np.zeros(0)
    d.fix_extra = RaggedRecords(flat, offsets)
    if d.natoms and len(s) != d.natoms:
        raise ValueError(f"restart header declares {d.natoms} atoms but {len(s)} were found")


def parse_neigh_history(record: np.ndarray, dnum: int | None = 3) -> tuple[np.ndarray, np.ndarray]:
    """One FixNeighHistory record [length, npartner, (tag, value[dnum]) ...] -> (partner tags,
    values of shape (npartner, dnum)).  dnum None: read it from the record's length."""
    record = np.asarray(record, dtype=np.float64)
    if record.size == 0:
        return np.zeros(0, dtype=np.int32), np.zeros((0, 3 if dnum is None else dnum))
    npartner = int(record[1])
    if dnum is None:
        dnum = (record.size - 2) // npartner - 1 if npartner else 3
    body = record[2:2 + npartner * (1 + dnum)].reshape(npartner, 1 + dnum)
    return _double_as_bits(body[:, 0]).astype(np.int32), body[:, 1:].copy()


def _neigh_history_flat(extra: RaggedRecords):
    """(atom index, partner tag, values) of every contact in every NEIGH_HISTORY record."""
    off = extra.offsets
    has = off[1:] > off[:-1]
    idx = np.nonzero(has)[0]
    if len(idx) == 0:
        return np.zeros(0, np.int64), np.zeros(0, np.int32), np.zeros((0, 3))
    flat = extra.flat
    npart = flat[off[idx] + 1].astype(np.int64)
    length = flat[off[idx]].astype(np.int64)
    with_c = npart > 0
    if not with_c.any():
        return np.zeros(0, np.int64), np.zeros(0, np.int32), np.zeros((0, 3))
    dn = (length[with_c] - 2) // npart[with_c] - 1
    if np.any(dn != dn[0]) or np.any((length[with_c] - 2) % npart[with_c]):
        raise ValueError("NEIGH_HISTORY records of mixed value counts")
    dnum = int(dn[0])
    rows = np.repeat(idx, npart)
    pos = np.repeat(off[idx] + 2, npart) + (np.arange(npart.sum()) - np.repeat(np.cumsum(npart) - npart, npart)) * (1 + dnum)
    tags = _double_as_bits(flat[pos]).astype(np.int32)
    vals = flat[pos[:, None] + 1 + np.arange(dnum)[None, :]]
    return rows, tags, vals


# ------------------------------------------------------------------ writing


class _Out:
    def __init__(self) -> None:
        self.parts = []

    def raw(self, b: bytes) -> None:
        self.parts.append(b)

    def i32(self, *v) -> None:
        self.parts.append(struct.pack(f"<{len(v)}i", *v))

    def flag_int(self, name: str, v: int) -> None:
        self.i32(FLAG[name], int(v))

    def flag_bigint(self, name: str, v: int) -> None:
        self.parts.append(struct.pack("<iq", FLAG[name], int(v)))

    def flag_double(self, name: str, v: float) -> None:
        self.parts.append(struct.pack("<id", FLAG[name], float(v)))

    def flag_string(self, name: str, v: str) -> None:
        b = v.encode("utf-8") + b"\x00"
        self.parts.append(struct.pack("<ii", FLAG[name], len(b)) + b)

    def flag_ints(self, name: str, v) -> None:
        self.parts.append(struct.pack(f"<ii{len(v)}i", FLAG[name], len(v), *v))

    def flag_doubles(self, name: str, v) -> None:
        self.parts.append(struct.pack(f"<ii{len(v)}d", FLAG[name], len(v), *[float(a) for a in v]))

    def counted(self, s: str) -> None:
        b = s.encode("utf-8") + b"\x00"
        self.parts.append(struct.pack("<i", len(b)) + b)

    def end(self) -> None:
        self.i32(-1)

    def bytes(self) -> bytes:
        return b"".join(self.parts)


def pack_atom_records(x, v, omega, radius, rmass, tag, atom_type, contacts=None) -> np.ndarray:
    """The PERPROC payload: one atom_style sphere record per atom, followed (when `contacts` is given)
    by its NEIGH_HISTORY record.  contacts = (rows, partner tags, values[dnum]) as flat arrays, rows in
    0..n-1; each atom's partners are written in the order they appear."""
    n = len(radius)
    base = np.empty((n, _BASE_WORDS), dtype=np.float64)
    base[:, 1:4] = x
    base[:, 4] = _bits_as_double(np.asarray(tag, dtype=np.int64))
    base[:, 5] = _bits_as_double(np.asarray(atom_type, dtype=np.int64))
    base[:, 6] = _bits_as_double(np.ones(n, dtype=np.int64))       # group mask: "all"
    base[:, 7] = _bits_as_double(np.full(n, _IMAGE_ZERO, dtype=np.int64))
    base[:, 8:11] = v
    base[:, 11] = radius
    base[:, 12] = rmass
    base[:, 13:16] = omega
    if contacts is None:
        base[:, 0] = _BASE_WORDS
        return base.reshape(-1)
    rows, ptag, vals = contacts
    rows = np.asarray(rows, dtype=np.int64).reshape(-1)
    vals = _values_2d(vals, len(rows))
    dnum = vals.shape[1]
    order = np.argsort(rows, kind="stable")  # each atom's partners together, in their given order
    rows, ptag, vals = rows[order], np.asarray(ptag, dtype=np.int64)[order], vals[order]
    npart = np.bincount(rows, minlength=n)
    hist_len = 2 + npart * (1 + dnum)
    rec_len = _BASE_WORDS + hist_len
    start = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(rec_len, out=start[1:])
    out = np.empty(start[-1], dtype=np.float64)
    cols = start[:-1, None] + np.arange(_BASE_WORDS)[None, :]
    base[:, 0] = rec_len
    out[cols] = base
    h0 = start[:-1] + _BASE_WORDS
    out[h0] = hist_len
    out[h0 + 1] = npart
    first = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(npart, out=first[1:])
    k = np.arange(len(rows)) - first[rows]           # position of each contact within its atom
    p = h0[rows] + 2 + k * (1 + dnum)
    out[p] = _bits_as_double(ptag)
    out[p[:, None] + 1 + np.arange(dnum)[None, :]] = vals
    return out


def write_restart_arrays(path, *, x, v, omega, radius, rmass, tag, atom_type, boxlo, boxhi, periodicity,
                         timestep: int, dt: float, units: str = "si", pair_style: str | None = None,
                         pair_settings=None, contacts=None, history_style: str = "granular") -> None:
    """write_restart from plain arrays (what write_restart extracts from a running system).
    pair_style/pair_settings: "granular" with {"submodels": {slot: (name, coeffs)}, "limit_damping"} or a
    gran/* style with its kn, kt, gamman, gammat, xmu, dampflag, limit_damping; None writes no force field.
    contacts: (rows, partner tags, values) of the both-sided history, or None for no NEIGH_HISTORY."""
    n = len(radius)
    ntypes = int(np.max(atom_type)) if n else 1
    w = _Out()
    w.raw(MAGIC)
    w.i32(ENDIAN, FORMAT_REVISION)
    w.flag_string("VERSION", VERSION_STRING)
    w.flag_int("SMALLINT", 4)
    w.flag_int("IMAGEINT", 4)
    w.flag_int("TAGINT", 4)
    w.flag_int("BIGINT", 8)
    w.flag_string("UNITS", units)
    w.flag_bigint("NTIMESTEP", timestep)
    w.flag_int("DIMENSION", 3)
    w.flag_int("NPROCS", 1)
    w.flag_ints("PROCGRID", [1, 1, 1])
    # each contact is evaluated once per side, which is LAMMPS' newton off for a granular run
    w.flag_int("NEWTON_PAIR", 0)
    w.flag_int("NEWTON_BOND", 0)
    per = [int(a) for a in periodicity]
    for name, p in zip(("XPERIODIC", "YPERIODIC", "ZPERIODIC"), per):
        w.flag_int(name, p)
    w.flag_ints("BOUNDARY", [0 if per[k] else 1 for k in range(3) for _ in range(2)])
    w.flag_string("ATOM_STYLE", "sphere")
    w.i32(0)  # atom_style sphere takes no arguments
    w.flag_bigint("NATOMS", n)
    w.flag_int("NTYPES", ntypes)
    w.flag_int("TRICLINIC", 0)
    w.flag_doubles("BOXLO", list(boxlo))
    w.flag_doubles("BOXHI", list(boxhi))
    w.flag_double("TIMESTEP", dt)
    w.end()
    w.i32(1)            # groups: "all"
    w.counted("all")
    w.end()             # type arrays: sphere atoms carry their own mass
    if pair_style is not None:
        _write_pair(w, pair_style, pair_settings or {}, ntypes)
    w.end()
    w.i32(0)            # no fix with global state
    if contacts is not None:
        rows = np.asarray(contacts[0], dtype=np.int64).reshape(-1)
        dnum = _values_2d(contacts[2], len(rows)).shape[1]
        most = int(np.bincount(rows, minlength=max(n, 1)).max()) if len(rows) else 0
        w.i32(1)
        w.counted(_HISTORY_FIX_ID.get(history_style, _HISTORY_FIX_ID["granular"]))
        w.counted("NEIGH_HISTORY")
        w.i32(2 + (1 + dnum) * most)
    else:
        w.i32(0)
    w.flag_int("MULTIPROC", 0)
    w.end()
    payload = pack_atom_records(x, v, omega, radius, rmass, tag, atom_type, contacts)
    w.i32(FLAG["PERPROC"], len(payload))
    w.raw(payload.astype("<f8").tobytes())
    w.raw(MAGIC)
    Path(path).write_bytes(w.bytes())


def _write_pair(w: _Out, style: str, s: dict, ntypes: int) -> None:
    """WriteRestart::force_fields for the two pair families this path runs."""
    if style == "granular":
        sub = s["submodels"]
        w.flag_string("PAIR", "granular")
        w.i32(1)  # one model
        for slot in _GRAN_SLOTS:
            name, coeffs = sub.get(slot, ("none", []))
            b = name.encode("utf-8")
            w.raw(struct.pack("<i", len(b)) + b)
            w.raw(struct.pack(f"<i{len(coeffs)}d", len(coeffs), *[float(c) for c in coeffs]))
        w.i32(int(s.get("limit_damping", 0)))
        # every type pair set, no explicit cutoff (-1: derived from the radii), model 0
        for i in range(ntypes):
            for _ in range(i, ntypes):
                w.raw(struct.pack("<idi", 1, -1.0, 0))
    elif style in _LEGACY_STYLES:
        w.flag_string("PAIR", style)
        w.raw(struct.pack("<5d", *(float(s[k]) for k in ("kn", "kt", "gamman", "gammat", "xmu"))))
        w.i32(int(s.get("dampflag", 1)), int(s.get("limit_damping", 0)))
        for i in range(ntypes):
            for _ in range(i, ntypes):
                w.i32(1)
    else:
        raise ValueError(f"storing pair_style {style!r} in a restart file is not implemented")


def _pair_description(pair):
    """(style, settings) of a pair object of this package, or (None, None)."""
    if pair is None:
        return None, None
    from .GRANULAR import GranHertzHistory, GranHooke, GranHookeHistory, PairGranular
    if isinstance(pair, PairGranular):
        sub = dict(pair.submodels)
        for slot in _GRAN_SLOTS:
            sub.setdefault(slot, ("none", []))
        return "granular", {"submodels": sub, "limit_damping": int(pair.limit_damping)}
    for cls, style in ((GranHertzHistory, "gran/hertz/history"), (GranHookeHistory, "gran/hooke/history"),
                       (GranHooke, "gran/hooke")):
        if type(pair) is cls:
            return style, {k: getattr(pair, k) for k in ("kn", "kt", "gamman", "gammat", "xmu", "dampflag",
                                                         "limit_damping")}
    raise ValueError(f"storing pair style {type(pair).__name__} in a restart file is not implemented; omit "
                     "`pair` to write the file without a force field section")


def write_restart(path, atom, domain, timestep: int, dt: float, history=None, units: str = "si", pair=None,
                  pair_style: str = "granular", nlist=None) -> None:
    """Write a single-file LAMMPS restart of the system (the reference's write_restart, same arguments).

    With `history` and `nlist`, every touching contact is stored in FixNeighHistory's both-sided form,
    so LAMMPS, the reference and read_restart get the frictional state back.  With `pair` (any pair
    style of this package whose layout LAMMPS restart files define: pair granular, gran/hooke,
    gran/hooke/history, gran/hertz/history) the force field is stored too.  The atoms are written in
    insertion order."""
    n = atom.nlocal
    host = atom._gather_all() if n else None
    if n:
        xr, vm, om = host["xr"][:n], host["vm"][:n], host["om"][:n]
        x, radius, v, rmass, omega = xr[:, :3], xr[:, 3], vm[:, :3], vm[:, 3], om[:, :3]
        tag = host["tag"][:n]
    else:
        x = v = omega = np.zeros((0, 3))
        radius = rmass = np.zeros(0)
        tag = np.zeros(0, np.int32)
    atype = np.asarray(atom.atom_type[:n], dtype=np.int32)
    contacts = None
    style, settings = _pair_description(pair)
    hist_style = style if style in _HISTORY_FIX_ID else pair_style
    if history is not None and nlist is not None and n:
        contacts = history.both_sided_contacts(nlist)
    elif history is not None and nlist is not None:
        contacts = (np.zeros(0, np.int64), np.zeros(0, np.int32), np.zeros((0, 3)))
    domain.pull()
    if np.any(np.asarray(domain.tilt) != 0.0):
        raise NotImplementedError("restart files of triclinic boxes are not written on this path")
    write_restart_arrays(path, x=x, v=v, omega=omega, radius=radius, rmass=rmass, tag=tag, atom_type=atype,
                         boxlo=[float(a) for a in domain.boxlo], boxhi=[float(a) for a in domain.boxhi],
                         periodicity=[int(a) for a in domain.periodicity], timestep=int(timestep), dt=float(dt),
                         units=units, pair_style=style, pair_settings=settings, contacts=contacts,
                         history_style=hist_style)


def pair_from_restart(data: RestartData, domain):
    """The pair style a restart file stores, as a pair object of this package (the reference's input
    parser, input.py:547-593), or None when the file has no force field."""
    from .GRANULAR import GranHertzHistory, GranHooke, GranHookeHistory, PairGranular
    style = data.pair_style
    if not style:
        return None
    if style == "granular":
        models = data.pair_settings.get("models") or []
        if not models:
            return None
        m = models[0]
        if m.get("twisting", ("none", []))[0] != "none":
            raise ValueError(f"restart file uses pair granular twisting model {m['twisting'][0]!r}, which is "
                             "not implemented")
        normal, ncoeffs = m["normal"]
        tangential, tcoeffs = m["tangential"]
        rolling, rcoeffs = m.get("rolling", ("none", []))
        # LAMMPS stores an unset tangential stiffness (NULL) as -1
        tcoeffs = [None if abs(c + 1.0) < 1e-15 else c for c in tcoeffs]
        return PairGranular(domain=domain, normal=normal, normal_coeffs=list(ncoeffs), tangential=tangential,
                            tangential_coeffs=tcoeffs, damping=m["damping"][0],
                            limit_damping=bool(m.get("limit_damping", 0)), rolling=rolling,
                            rolling_coeffs=list(rcoeffs) or None)
    cls = {"gran/hooke": GranHooke, "gran/hooke/history": GranHookeHistory,
           "gran/hertz/history": GranHertzHistory}.get(style)
    if cls is None:
        raise ValueError(f"restart file uses pair_style {style!r}, which is not implemented")
    s = data.pair_settings
    return cls(domain=domain, kn=s["kn"], kt=s["kt"], gamman=s["gamman"], gammat=s["gammat"], xmu=s["xmu"],
               dampflag=s["dampflag"], limit_damping=bool(s["limit_damping"]))


def system_from_restart(data: RestartData, max_atoms: int | None = None, max_neighbors: int = 64):
    """What the reference's `read_restart` command rebuilds (input.py:501-545): the box, the atoms (in
    file order, with the stored masses), a ContactHistory holding the file's contact history (applied
    at the first neighbor build) and the stored pair style.  Returns dict(domain, atom, history, pair,
    timestep, dt); the caller adds a NeighborList, the fixes and a Simulation whose timestep it sets
    to `timestep`."""
    from .atom import AtomSystem
    from .contact_history import ContactHistory
    from .domain import Domain
    if any(data.tilt):
        raise NotImplementedError("restart files of triclinic boxes are not read on this path")
    n = len(data.radius)
    cap = n if max_atoms is None else int(max_atoms)
    domain = Domain(boxlo=data.boxlo, boxhi=data.boxhi, boundary=data.boundary)
    atom = AtomSystem(max_atoms=cap)
    if n:
        atom.add_particles(x=data.x, radius=data.radius, density=data.density, v=data.v, omega=data.omega,
                           tag=data.tag, atom_type=data.atom_type, rmass=data.rmass)
    history = ContactHistory(max_atoms=cap, max_neighbors=max_neighbors)
    if "NEIGH_HISTORY" in data.fix_peratom_styles and data.fix_extra:
        rows, tags, vals = data.neigh_history()
        history.load_restart_arrays(rows, tags, vals)
    return {"domain": domain, "atom": atom, "history": history, "pair": pair_from_restart(data, domain),
            "timestep": int(data.timestep), "dt": float(data.dt)}

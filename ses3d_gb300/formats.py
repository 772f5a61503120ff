"""Readers and writers for the SES3D file formats.

These are the files the reference solver reads and writes, parsed the way it
parses them:

* ASCII inputs are read by line position with Fortran list-directed reads: each
  read statement consumes one line and takes its first token (so trailing
  ``! comment`` text is ignored). Reals are converted with ``strtof``, as
  gfortran converts REAL(4) input. (``INPUT/setup`` per
  SOURCE/ses3d_input.f90:264-310, ``INPUT/event_<id>`` per :201-249,
  ``INPUT/relax`` per :338-350, ``INPUT/stf`` per :419-428 -- four lines skipped,
  ``INPUT/recfile_<id>`` per :533-538, ``MODELS/MODELS/boxfile`` per :51-98,
  ``ADJOINT/<id>/ad_srcfile`` per :594-598, ``ad_src_<k>`` per
  SOURCE/ses3d_init.f90:479-490, ``saving_vector_<rank>`` per
  SOURCE/ses3d_input.f90:570-574.)
* Binary fields are gfortran sequential-unformatted records: a 4-byte
  little-endian length, the payload, the same length again; payload FP32 in
  Fortran column-major order (model records SOURCE/ses3d_input.f90:479-484,
  snapshots and kernels SOURCE/ses3d_output.f90:304-337, forward fields
  :150-154).
* Seismograms are written in the layout of SOURCE/ses3d_output.f90:404-447
  with gfortran list-directed number formatting (9 significant digits, which
  round-trips FP32).
"""
from __future__ import annotations

import ctypes
import ctypes.util
import math
import os
import struct
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

_libc = ctypes.CDLL(ctypes.util.find_library("c") or "libc.so.6")
_libc.strtof.restype = ctypes.c_float
_libc.strtof.argtypes = [ctypes.c_char_p, ctypes.c_void_p]

PI_F32 = np.float32(3.1415926535898)  # SOURCE/ses3d_modules.f90:25


def strtof(token: str) -> np.float32:
    """Decimal -> FP32 with a single rounding (libgfortran reads REAL(4) with strtof)."""
    t = token.strip().replace("d", "e").replace("D", "e")
    return np.float32(_libc.strtof(t.encode(), None))


def _tokens(line: str) -> List[str]:
    # list-directed separators: blanks, commas; a slash ends the record
    line = line.split("/")[0] if not line.lstrip().startswith((".", "/")) else line
    return line.replace(",", " ").split()


class LineReader:
    """Line-positional reader mimicking successive list-directed READ statements."""

    def __init__(self, path: str):
        with open(path, "r") as f:
            self.lines = f.read().splitlines()
        self.pos = 0
        self.path = path

    def _next(self) -> str:
        if self.pos >= len(self.lines):
            raise EOFError("unexpected end of file in %s" % self.path)
        s = self.lines[self.pos]
        self.pos += 1
        return s

    def skip(self, n: int = 1):
        for _ in range(n):
            self._next()

    def values(self, n: int) -> List[str]:
        """First n tokens; like list-directed input, blank records are skipped."""
        out: List[str] = []
        while len(out) < n:
            s = self._next()
            toks = _tokens(s.split("!")[0]) if "!" in s else _tokens(s)
            out.extend(toks[: n - len(out)])
        return out

    def int(self) -> int:
        return int(self.values(1)[0])

    def real(self) -> np.float32:
        return strtof(self.values(1)[0])

    def token(self) -> str:
        return self.values(1)[0]

    def text(self) -> str:
        """A '(A1000)' formatted read: the whole line."""
        return self._next().rstrip()


# ------------------------------------------------------------------------------------------------
# setup / event / relax / event_list
# ------------------------------------------------------------------------------------------------

@dataclass
class Setup:
    xmin: np.float32 = np.float32(0)   # degrees, as in the file
    xmax: np.float32 = np.float32(0)
    ymin: np.float32 = np.float32(0)
    ymax: np.float32 = np.float32(0)
    zmin: np.float32 = np.float32(0)   # m
    zmax: np.float32 = np.float32(0)
    is_diss: int = 1
    model_type: int = 1
    nx_global: int = 0
    ny_global: int = 0
    nz_global: int = 0
    lpd: int = 4
    px: int = 1
    py: int = 1
    pz: int = 1
    adjoint_flag: int = 0
    samp_ad: int = 10
    ffd: str = "../DATA/OUTPUT/ADJOINT"


def read_setup(path: str) -> Setup:
    r = LineReader(path)
    s = Setup()
    r.skip()
    s.xmin, s.xmax, s.ymin, s.ymax, s.zmin, s.zmax = (r.real() for _ in range(6))
    s.is_diss = r.int(); s.model_type = r.int()
    r.skip()
    s.nx_global, s.ny_global, s.nz_global, s.lpd, s.px, s.py, s.pz = (r.int() for _ in range(7))
    r.skip()
    s.adjoint_flag = r.int(); s.samp_ad = r.int()
    s.ffd = r.text().strip()
    return s


def write_setup(path: str, s: Setup):
    L = [
        "MODEL " + "=" * 60,
        "%-44s! theta_min (colatitude) in degrees" % fmt_plain(s.xmin),
        "%-44s! theta_max (colatitude) in degrees" % fmt_plain(s.xmax),
        "%-44s! phi_min (longitude) in degrees" % fmt_plain(s.ymin),
        "%-44s! phi_max (longitude) in degrees" % fmt_plain(s.ymax),
        "%-44s! z_min (radius) in m" % fmt_plain(s.zmin),
        "%-44s! z_max (radius) in m" % fmt_plain(s.zmax),
        "%-44s! is_diss" % s.is_diss,
        "%-44s! model_type" % s.model_type,
        "COMPUTATIONAL SETUP (PARALLELISATION) " + "=" * 40,
        "%-44s! nx_global, (nx_global+px = global # elements in theta direction)" % s.nx_global,
        "%-44s! ny_global, (ny_global+py = global # elements in phi direction)" % s.ny_global,
        "%-44s! nz_global, (nz_global+pz = global # of elements in r direction)" % s.nz_global,
        "%-44s! lpd, LAGRANGE polynomial degree" % s.lpd,
        "%-44s! px, processors in theta direction" % s.px,
        "%-44s! py, processors in phi direction" % s.py,
        "%-44s! pz, processors in r direction" % s.pz,
        "ADJOINT PARAMETERS " + "=" * 60,
        "%-44s! adjoint_flag (0=normal simulation, 1=adjoint forward, 2=adjoint reverse)" % s.adjoint_flag,
        "%-44s! samp_ad, sampling rate of forward field" % s.samp_ad,
        s.ffd,
    ]
    _write_lines(path, L)


@dataclass
class Event:
    nt: int = 0
    dt: np.float32 = np.float32(0)
    xxs: np.float32 = np.float32(0)  # colatitude, degrees
    yys: np.float32 = np.float32(0)  # longitude, degrees
    zzs: np.float32 = np.float32(0)  # depth, m
    source_type: int = 10
    mom: np.ndarray = field(default_factory=lambda: np.zeros(6, np.float32))  # xx yy zz xy xz yz
    ofd: str = "../DATA/OUTPUT/"
    ssamp: int = 100000
    output_displacement: int = 0


def read_event(path: str) -> Event:
    r = LineReader(path)
    e = Event()
    r.skip()
    e.nt = r.int(); e.dt = r.real()
    r.skip()
    e.xxs, e.yys, e.zzs = r.real(), r.real(), r.real()
    e.source_type = r.int()
    e.mom = np.array([r.real() for _ in range(6)], dtype=np.float32)
    r.skip()
    e.ofd = r.text().strip()
    r.skip()
    e.ssamp = r.int(); e.output_displacement = r.int()
    return e


def write_event(path: str, e: Event):
    names = ["M_theta_theta", "M_phi_phi", "M_r_r", "M_theta_phi", "M_theta_r", "M_phi_r"]
    L = ["SIMULATION PARAMETERS " + "=" * 60,
         "%-24s! nt, number of time steps" % e.nt,
         "%-24s! dt in sec, time increment" % fmt_plain(e.dt),
         "SOURCE " + "=" * 60,
         "%-24s! xxs, theta-coord. center of source in degrees" % fmt_plain(e.xxs),
         "%-24s! yys, phi-coord. center of source in degrees" % fmt_plain(e.yys),
         "%-24s! zzs, source depth in (m)" % fmt_plain(e.zzs),
         "%-24s! srctype, 1:f_x, 2:f_y, 3:f_z, 10:M_ij" % e.source_type]
    for nm, m in zip(names, e.mom):
        L.append("%-24s! %s" % (fmt_plain(m), nm))
    L += ["OUTPUT DIRECTORY " + "=" * 60, e.ofd,
          "OUTPUT FLAGS " + "=" * 60,
          "%-24s! ssamp, snapshot sampling" % e.ssamp,
          "%-24s! output_displacement, output displacement field (1=yes,0=no)" % e.output_displacement]
    _write_lines(path, L)


def read_relax(path: str):
    r = LineReader(path)
    r.skip()
    tau = np.array([r.real() for _ in range(3)], np.float32)
    r.skip()
    D = np.array([r.real() for _ in range(3)], np.float32)
    return tau, D


def write_relax(path: str, tau: Sequence[float], D: Sequence[float]):
    L = ["RELAXATION TIMES [s] =====================", *[fmt_plain(t) for t in tau],
         "WEIGHTS OF RELAXATION MECHANISMS =========", *[fmt_plain(d) for d in D]]
    _write_lines(path, L)


def read_event_list(path: str) -> List[str]:
    r = LineReader(path)
    n = r.int()
    return [r.token() for _ in range(n)]


def write_event_list(path: str, events: Sequence[str]):
    _write_lines(path, ["%-55s! n_events = number of events" % len(events), *events])


# ------------------------------------------------------------------------------------------------
# source time functions, receivers, adjoint sources
# ------------------------------------------------------------------------------------------------

def read_stf(path: str, nt: int) -> np.ndarray:
    """nt samples after four skipped lines (SOURCE/ses3d_input.f90:419-428)."""
    r = LineReader(path)
    r.skip(4)
    return np.array([strtof(t) for t in r.values(nt)], np.float32)


def write_stf(path: str, so: np.ndarray, dt: float, note: str = "filtered Heaviside"):
    """Writes the 4-line header of TOOLS/make_stf.py followed by one sample per line."""
    L = ["source time function, ses3d version 4.1",
         "nt= %d, dt=%s" % (len(so) - 1, fmt_plain(dt)),
         note,
         "-- samples --"]
    L += [fmt_plain(v) for v in so]
    _write_lines(path, L)


@dataclass
class Receivers:
    names: List[str]
    loc: np.ndarray  # (nr, 3): colatitude deg, longitude deg, depth m (FP32)


def read_recfile(path: str) -> Receivers:
    r = LineReader(path)
    n = r.int()
    names, loc = [], np.zeros((n, 3), np.float32)
    for i in range(n):
        names.append(r.token()[:12].ljust(12))
        loc[i] = [strtof(t) for t in r.values(3)]
    return Receivers(names, loc)


def write_recfile(path: str, rec: Receivers):
    L = [str(len(rec.names))]
    for nm, l in zip(rec.names, rec.loc):
        L.append(nm.strip())
        L.append(" ".join(fmt_plain(v) for v in l))
    _write_lines(path, L)


def read_ad_srcfile(path: str) -> np.ndarray:
    r = LineReader(path)
    n = r.int()
    return np.array([[strtof(t) for t in r.values(3)] for _ in range(n)], np.float32).reshape(n, 3)


def write_ad_srcfile(path: str, loc: np.ndarray):
    _write_lines(path, [str(len(loc))] + [" ".join(fmt_plain(v) for v in l) for l in loc] + [""])


def read_ad_src(path: str, nt: int) -> np.ndarray:
    """(3, nt) adjoint source time function (x, y, z), four header lines skipped."""
    r = LineReader(path)
    r.skip(4)
    vals = np.array([strtof(t) for t in r.values(3 * nt)], np.float32).reshape(nt, 3)
    return np.ascontiguousarray(vals.T)


def write_ad_src(path: str, stf3: np.ndarray, loc: Sequence[float]):
    L = ["-- adjoint source ------------------", "-- source coordinates (colat,lon,depth)",
         " ".join(fmt_plain(v) for v in loc), "-- source time function (x, y, z) --"]
    for k in range(stf3.shape[1]):
        L.append(" ".join(fmt_plain(stf3[c, k]) for c in range(3)))
    _write_lines(path, L)


def read_saving_vector(path: str, nt: int) -> np.ndarray:
    r = LineReader(path)
    return np.array([int(t) for t in r.values(nt)], np.int32)


def write_saving_vector(path: str, sv: Sequence[int]):
    _write_lines(path, [" %11d" % int(v) for v in sv])


# ------------------------------------------------------------------------------------------------
# boxfile
# ------------------------------------------------------------------------------------------------

@dataclass
class Box:
    index: int
    multi: tuple
    nx_min: int
    nx_max: int
    ny_min: int
    ny_max: int
    nz_min: int
    nz_max: int
    xmin: np.float32  # radians
    xmax: np.float32
    ymin: np.float32
    ymax: np.float32
    zmin: np.float32  # m
    zmax: np.float32

    @property
    def nx(self):
        return self.nx_max - self.nx_min

    @property
    def ny(self):
        return self.ny_max - self.ny_min

    @property
    def nz(self):
        return self.nz_max - self.nz_min


def read_boxfile(path: str) -> List[Box]:
    r = LineReader(path)
    r.skip(14)
    pp = r.int(); px = r.int(); py = r.int(); pz = r.int()
    r.skip()
    boxes = []
    for _ in range(pp):
        idx = r.int()
        multi = tuple(int(t) for t in r.values(3))
        a = [int(t) for t in r.values(2)]; b = [int(t) for t in r.values(2)]; c = [int(t) for t in r.values(2)]
        x = [strtof(t) for t in r.values(2)]; y = [strtof(t) for t in r.values(2)]; z = [strtof(t) for t in r.values(2)]
        r.skip()
        boxes.append(Box(idx, multi, a[0], a[1], b[0], b[1], c[0], c[1], x[0], x[1], y[0], y[1], z[0], z[1]))
    return boxes


def make_boxes(s: Setup) -> List[Box]:
    """Processor boxes as MODELS/SOURCE/generate_models.f90:200-283 computes them (FP32)."""
    f = np.float32
    pi = f(3.14159265358979)  # MODELS/SOURCE/modules_gm.f90
    x_min = f(s.xmin) * pi / f(180); x_max = f(s.xmax) * pi / f(180)
    y_min = f(s.ymin) * pi / f(180); y_max = f(s.ymax) * pi / f(180)
    z_min, z_max = f(s.zmin), f(s.zmax)
    nx, ny, nz, px, py, pz = s.nx_global, s.ny_global, s.nz_global, s.px, s.py, s.pz
    dz = (z_max - z_min) / f(nz + pz)
    dy = (y_max - y_min) / f(ny + py)
    dx = (x_max - x_min) / f(nx + px)
    bnx, bny, bnz = (nx + 1) // px, (ny + 1) // py, (nz + 1) // pz
    boxes = []
    for k in range(1, pz + 1):
        for j in range(1, py + 1):
            for i in range(1, px + 1):
                mi = (k - 1) * py * px + (j - 1) * px + i
                mn = ((i - 1) * bnx, (j - 1) * bny, (k - 1) * bnz)
                mx = (i * bnx if i != px else nx, j * bny if j != py else ny, k * bnz if k != pz else nz)
                boxes.append(Box(mi, (i, j, k), mn[0], mx[0], mn[1], mx[1], mn[2], mx[2],
                                 x_min + f(mn[0] + i - 1) * dx, x_min + f(mx[0] + i) * dx,
                                 y_min + f(mn[1] + j - 1) * dy, y_min + f(mx[1] + j) * dy,
                                 z_min + f(mn[2] + k - 1) * dz, z_min + f(mx[2] + k) * dz))
    return boxes


def box_offsets(boxes: List[Box]):
    """Global element counts (ex, ey, ez) of a decomposition and each box's global element
    offset (ox, oy, oz). Box (mx, my, mz) starts at element nx_min + mx - 1 in x (and y);
    the boxfile counts z upward (mz = 1 is the bottom box, SOURCE/ses3d_init.f90:600-611)
    while element k counts down from the top (z = zmax - k dz), so oz = ez - nz_max - mz."""
    ex = max(b.nx_max + b.multi[0] for b in boxes)
    ey = max(b.ny_max + b.multi[1] for b in boxes)
    ez = max(b.nz_max + b.multi[2] for b in boxes)
    offs = [(b.nx_min + b.multi[0] - 1, b.ny_min + b.multi[1] - 1, ez - (b.nz_max + b.multi[2])) for b in boxes]
    return (ex, ey, ez), offs


def split_field(field: np.ndarray, boxes: List[Box], pad=None) -> List[np.ndarray]:
    """Per-box pieces of a global element-local field (reference F-order, element index
    fastest). pad = (nx_max, ny_max, nz_max) lays each piece out with the reference build's
    array extents (0:nx_max, ...), zeros outside the box, as its output files are written."""
    (ex, ey, ez), offs = box_offsets(boxes)
    g = np.asarray(field).reshape(125, ez, ey, ex)
    out = []
    for b, (ox, oy, oz) in zip(boxes, offs):
        piece = g[:, oz:oz + b.nz + 1, oy:oy + b.ny + 1, ox:ox + b.nx + 1]
        if pad is not None:
            full = np.zeros((125, pad[2] + 1, pad[1] + 1, pad[0] + 1), g.dtype)
            full[:, :b.nz + 1, :b.ny + 1, :b.nx + 1] = piece
            piece = full
        out.append(np.ascontiguousarray(piece).reshape(-1))
    return out


def stitch_field(pieces: Sequence[np.ndarray], boxes: List[Box], pad=None) -> np.ndarray:
    """Inverse of split_field."""
    (ex, ey, ez), offs = box_offsets(boxes)
    g = np.zeros((125, ez, ey, ex), np.asarray(pieces[0]).dtype)
    for piece, b, (ox, oy, oz) in zip(pieces, boxes, offs):
        dims = (pad[2] + 1, pad[1] + 1, pad[0] + 1) if pad is not None else (b.nz + 1, b.ny + 1, b.nx + 1)
        a = np.asarray(piece).reshape(125, *dims)[:, :b.nz + 1, :b.ny + 1, :b.nx + 1]
        g[:, oz:oz + b.nz + 1, oy:oy + b.ny + 1, ox:ox + b.nx + 1] = a
    return g.reshape(-1)


def write_boxfile(path: str, boxes: List[Box], px: int, py: int, pz: int):
    L = [" - format description -", " total number of processes", " number of processes in x direction",
         " number of processes in y direction", " number of processes in z direction",
         " single index (npz-1)*py*px+(npy-1)*px+npx", " multi index (npx, npy, npz)",
         " index boundaries x (x_min, x_max)", " index boundaries y (y_min, y_max)",
         " index boundaries z (z_min, z_max)", " physical boundaries x", " physical boundaries y",
         " phyiscal boundaries z", " -------------------",
         fmt_int(px * py * pz), fmt_int(px), fmt_int(py), fmt_int(pz), " -------------------"]
    for b in boxes:
        L += [fmt_int(b.index), fmt_int(*b.multi), fmt_int(b.nx_min, b.nx_max), fmt_int(b.ny_min, b.ny_max),
              fmt_int(b.nz_min, b.nz_max), fmt_reals(b.xmin, b.xmax), fmt_reals(b.ymin, b.ymax),
              fmt_reals(b.zmin, b.zmax), " -------------------"]
    _write_lines(path, L)


# ------------------------------------------------------------------------------------------------
# binary records
# ------------------------------------------------------------------------------------------------

def write_records(path: str, arrays: Sequence[np.ndarray], append: bool = False):
    """Fortran sequential-unformatted records of FP32 payload (arrays already flat in F-order)."""
    with open(path, "ab" if append else "wb") as f:
        for a in arrays:
            b = np.ascontiguousarray(a, dtype=np.float32).tobytes()
            n = struct.pack("<i", len(b))
            f.write(n); f.write(b); f.write(n)


def read_records(path: str) -> List[np.ndarray]:
    out = []
    with open(path, "rb") as f:
        data = f.read()
    pos = 0
    while pos < len(data):
        if pos + 4 > len(data):
            raise ValueError("truncated record in %s" % path)
        (n,) = struct.unpack_from("<i", data, pos)
        if n < 0 or n % 4 or pos + 8 + n > len(data):
            raise ValueError("truncated record in %s" % path)
        payload = data[pos + 4: pos + 4 + n]
        (m,) = struct.unpack_from("<i", data, pos + 4 + n)
        if m != n:
            raise ValueError("corrupt record markers in %s" % path)
        out.append(np.frombuffer(payload, dtype=np.float32).copy())
        pos += 8 + n
    return out


def read_record(path: str, count: Optional[int] = None) -> np.ndarray:
    recs = read_records(path)
    if not recs:
        raise ValueError("no record in %s" % path)
    if count is not None and recs[0].size != count:
        raise ValueError("%s holds %d values, expected %d" % (path, recs[0].size, count))
    return recs[0]


MODEL_NAMES = ("rhoinv", "mu", "lambda", "A", "B", "C", "Q")


def read_model(dirpath: str, rank: int, n: int, is_diss: int) -> dict:
    """MODELS/MODELS/<name><rank> records (SOURCE/ses3d_input.f90:472-499)."""
    out = {}
    for nm in MODEL_NAMES:
        if nm == "Q" and not is_diss:
            continue
        out[nm] = read_record(os.path.join(dirpath, "%s%d" % (nm, rank)), n)
    return out


def write_model(dirpath: str, rank: int, model: dict):
    os.makedirs(dirpath, exist_ok=True)
    for nm in MODEL_NAMES:
        if nm in model:
            write_records(os.path.join(dirpath, "%s%d" % (nm, rank)), [model[nm]])


# ------------------------------------------------------------------------------------------------
# seismograms (SOURCE/ses3d_output.f90:398-451) and number formatting
# ------------------------------------------------------------------------------------------------

def fmt_real(x) -> str:
    """gfortran list-directed REAL(4): leading blank, 9 significant digits, G-style field."""
    v = float(np.float32(x))
    if v == 0.0:
        body = "0.00000000"
        return " " + body.rjust(12) + "    "
    a = abs(v)
    s9 = "%.8e" % v
    mant_exp = int(s9.split("e")[1])
    if 0.1 <= float("%.9g" % a) < 1e9:
        decimals = 8 - mant_exp
        body = "%.*f" % (max(decimals, 0), v)
        return " " + body.rjust(12) + "    "
    body = "%.8E" % v
    m, e = body.split("E")
    ei = int(e)
    body = "%sE%s%02d" % (m, "-" if ei < 0 else "+", abs(ei))
    return " " + body.rjust(16)


def fmt_int(*vals) -> str:
    return "".join(" %11d" % v for v in vals)


def fmt_reals(*vals) -> str:
    return "".join(fmt_real(v) for v in vals)


def fmt_plain(x) -> str:
    """Shortest decimal that strtof maps back to the same FP32 value."""
    v = np.float32(x)
    for p in range(1, 10):
        s = "%.*g" % (p, float(v))
        if strtof(s) == v:
            return s
    return "%.9g" % float(v)


def write_seismograms(ofd: str, name12: str, sx, sy, sz, nt: int, dt, recloc, src):
    """Three files <ofd><name>.{x,y,z}; name keeps its 12-character padding like the reference.
    recloc/src: (colat deg, lon deg, depth m) as the reference prints them."""
    heads = ("theta component seismograms", "phi component seismograms", "r component seismograms")
    for comp, data, head in zip("xyz", (sx, sy, sz), heads):
        L = [" " + head, " nt=" + fmt_int(nt), " dt=" + fmt_real(dt),
             " receiver location (colat [deg],lon [deg],depth [m])",
             " x=" + fmt_real(recloc[0]) + " y=" + fmt_real(recloc[1]) + " z=" + fmt_real(recloc[2]),
             " source location (colat [deg],lon [deg],depth [m])",
             " x=" + fmt_real(src[0]) + " y=" + fmt_real(src[1]) + " z=" + fmt_real(src[2])]
        L += [fmt_real(v) for v in np.asarray(data, np.float32)[:nt]]
        _write_lines(os.path.join(ofd, name12.ljust(12)[:12] + "." + comp), L)


def read_seismogram(path: str):
    """(nt, dt, trace) of one component file, as TOOLS/seismograms.py:37-97 reads it."""
    with open(path) as f:
        lines = f.read().splitlines()
    nt = int(lines[1].split("=")[1])
    dt = float(lines[2].split("=")[1])
    tr = np.array([float(l) for l in lines[7:7 + nt]], np.float32)
    return nt, dt, tr


def _write_lines(path: str, lines: Sequence[str]):
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def deg(rad) -> np.float32:
    """radians -> degrees as the reference prints them (x*180/pi in FP32)."""
    return np.float32(np.float32(rad) * np.float32(180)) / PI_F32


def isfinite_all(*arrays) -> bool:
    return all(np.isfinite(a).all() for a in arrays)


__all__ = [n for n in dir() if not n.startswith("_") and n not in ("annotations", "math")]

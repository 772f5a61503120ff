"""Model generation for SES3D trees, restated from the reference's pre-processing:

* MODELS/SOURCE/generate_models.f90: processor boxes (boxfile), GLL coordinates per box
  (`xco_/yco_/zco_<rank>` coordinate files), a 1-D background evaluated at every GLL point
  and the per-rank model records rhoinv, mu, lambda, A, B, C, Q (`MODELS/MODELS/*<rank>`);
* MODELS/SOURCE/add_perturbation.f90: block-model perturbations of vsh, vsv, vp and rho
  (`MODELS_3D/{block_x,block_y,block_z,dvsh,dvsv,dvp,drho}`) added to the velocities of
  every GLL point inside a block cell, then mu, B, lambda and rhoinv recomputed;
* the block format itself (TOOLS/models.py:157-310).

All arithmetic is FP32 in the reference's expression order, so the records equal what the
Fortran programs write.

The background is the setup's model_type (`builtin_model`: homogeneous, isotropic PREM,
homogeneous + QL6 Q, EUMOD, ak135 from ses3d_gb300.earth_models, MODELS/MODELS_1D) or any
callable `profile(z)` of the GLL radii giving (rho [g/cm^3], vp [km/s], vs [km/s], Q),
converted exactly as those routines convert theirs (MODELS_1D/prem_iso.f90:214-228);
`LayeredProfile` builds a piecewise-constant profile from a depth table.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import formats as F

f32 = np.float32
PI_SOLVER = f32(3.1415926535898)   # SOURCE/ses3d_modules.f90:25 (add_perturbation uses the solver's modules)
KNOTS4 = np.array([-1.0, -0.6546536707079772, 0.0, 0.6546536707079772, 1.0], np.float32)


# ------------------------------------------------------------------------------------------------
# GLL coordinates of a processor box (generate_models.f90:333-360; add_perturbation.f90:268-293)
# ------------------------------------------------------------------------------------------------

def box_axes(box: F.Box) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """x[i, n], y[j, n] (radians) and z[k, n] (radius, m) of a box, FP32:
    x = xmin + i dx + 0.5 (1 + knot_n) dx with dx = (xmax - xmin) / (nx + 1), z counted down
    from zmax."""
    ex, ey, ez = box.nx + 1, box.ny + 1, box.nz + 1
    dx = f32(f32(box.xmax) - f32(box.xmin)) / f32(ex)
    dy = f32(f32(box.ymax) - f32(box.ymin)) / f32(ey)
    dz = f32(f32(box.zmax) - f32(box.zmin)) / f32(ez)
    half = (f32(0.5) * (f32(1) + KNOTS4)).astype(np.float32)
    ix = np.arange(ex, dtype=np.float32)[:, None]
    jy = np.arange(ey, dtype=np.float32)[:, None]
    kz = np.arange(ez, dtype=np.float32)[:, None]
    x = ((f32(box.xmin) + ix * dx).astype(np.float32) + half[None, :] * dx).astype(np.float32)
    y = ((f32(box.ymin) + jy * dy).astype(np.float32) + half[None, :] * dy).astype(np.float32)
    z = ((f32(box.zmax) - kz * dz).astype(np.float32) - half[None, :] * dz).astype(np.float32)
    return x, y, z


def write_coordinates(directory: str, rank: int, box: F.Box):
    """DATA/COORDINATES/{xco,yco,zco}_<rank>: one list-directed REAL(4) per line, element
    index outer, GLL index inner (generate_models.f90:333-356)."""
    os.makedirs(directory, exist_ok=True)
    for name, a in zip(("xco_", "yco_", "zco_"), box_axes(box)):
        with open(os.path.join(directory, name + str(rank)), "w") as f:
            f.write("\n".join(F.fmt_real(v) for v in a.reshape(-1)) + "\n")


def _grid(a_i: np.ndarray, a_j: np.ndarray, a_k: np.ndarray, ex, ey, ez):
    """Per-axis node values -> reference-layout (i, j, k, in, jn, kn) arrays (i fastest)."""
    X = np.broadcast_to(a_i.T[None, None, :, None, None, :], (5, 5, 5, ez, ey, ex))  # [kn,jn,in,k,j,i]
    Y = np.broadcast_to(a_j.T[None, :, None, None, :, None], (5, 5, 5, ez, ey, ex))
    Z = np.broadcast_to(a_k.T[:, None, None, :, None, None], (5, 5, 5, ez, ey, ex))
    return X.reshape(-1), Y.reshape(-1), Z.reshape(-1)


# ------------------------------------------------------------------------------------------------
# 1-D backgrounds (generate_models.f90:392-426; MODELS_1D/*)
# ------------------------------------------------------------------------------------------------

Profile = Callable[[np.ndarray], Tuple[np.ndarray, np.ndarray, np.ndarray, np.ndarray]]


def homogeneous(box: F.Box, is_diss: int) -> Dict[str, np.ndarray]:
    """model_type 1 (MODELS_1D/homogeneous.f90): rho = 1, mu = lambda = A = B = C = 0; Q is
    left at zero as the reference leaves it unset."""
    n = 125 * (box.nx + 1) * (box.ny + 1) * (box.nz + 1)
    out = {k: np.zeros(n, np.float32) for k in ("mu", "lambda", "A", "B", "C")}
    out["rhoinv"] = np.full(n, f32(1) / f32(1), np.float32)
    if is_diss:
        out["Q"] = np.zeros(n, np.float32)
    return out


@dataclass
class LayeredProfile:
    """Piecewise-constant 1-D model: layer l spans depths (top[l], top[l+1]] in km (the last
    layer extends downward); rho [g/cm^3], vp, vs [km/s], Q."""
    top_km: Sequence[float]
    rho: Sequence[float]
    vp: Sequence[float]
    vs: Sequence[float]
    Q: Sequence[float] = field(default_factory=list)
    r_earth: float = 6371000.0

    @classmethod
    def read(cls, path: str) -> "LayeredProfile":
        """Text table, one layer per line: top depth [km], rho, vp, vs[, Q]; '#' comments."""
        rows = []
        with open(path) as fh:
            for line in fh:
                line = line.split("#")[0].strip()
                if line:
                    rows.append([float(t) for t in line.split()])
        a = np.array(rows)
        return cls(a[:, 0], a[:, 1], a[:, 2], a[:, 3], a[:, 4] if a.shape[1] > 4 else [])

    def __call__(self, z: np.ndarray):
        depth_km = (f32(self.r_earth) - np.asarray(z, np.float32)).astype(np.float64) / 1000.0
        idx = np.clip(np.searchsorted(np.asarray(self.top_km, np.float64), depth_km, side="left") - 1, 0,
                      len(self.top_km) - 1)
        q = np.asarray(self.Q, np.float32)[idx] if len(self.Q) else np.full(idx.shape, f32(100000.0), np.float32)
        return (np.asarray(self.rho, np.float32)[idx], np.asarray(self.vp, np.float32)[idx],
                np.asarray(self.vs, np.float32)[idx], q)


def profile_model(box: F.Box, profile: Profile, is_diss: int) -> Dict[str, np.ndarray]:
    """A 1-D background on the box's GLL radii, converted like the reference's 1-D models
    (MODELS_1D/prem_iso.f90:214-228): units x1000, rhoinv = 1/rho, mu = cs cs rho,
    lambda = (cp cp - 2 cs cs) rho, A = B = C = 0."""
    x, y, z = box_axes(box)
    rho, cp, cs, q = (np.asarray(v, np.float32) for v in profile(z))
    rho = (f32(1000.0) * rho).astype(np.float32)
    cp = (f32(1000.0) * cp).astype(np.float32)
    cs = (f32(1000.0) * cs).astype(np.float32)
    return records_from_si(box, rho, cp, cs, q, is_diss)


def records_from_si(box: F.Box, rho, cp, cs, q, is_diss: int) -> Dict[str, np.ndarray]:
    """MODELS records from a 1-D model in SI units on the box's (nz+1, 5) radii:
    rhoinv = 1/rho, mu = cs cs rho, lambda = (cp cp - 2 cs cs) rho, Q, A = B = C = 0, each
    constant over (i, j, in, jn) (MODELS_1D/prem_iso.f90:214-228)."""
    ex, ey, ez = box.nx + 1, box.ny + 1, box.nz + 1
    x, y, z = box_axes(box)
    rho, cp, cs = (np.asarray(v, np.float32).reshape(ez, 5) for v in (rho, cp, cs))
    rhoinv1 = (f32(1) / rho).astype(np.float32)
    mu1 = ((cs * cs).astype(np.float32) * rho).astype(np.float32)
    lam1 = (((cp * cp).astype(np.float32) - (f32(2) * cs * cs).astype(np.float32)).astype(np.float32)
            * rho).astype(np.float32)
    out = {}
    for name, a in (("rhoinv", rhoinv1), ("mu", mu1), ("lambda", lam1), ("Q", np.asarray(q, np.float32))):
        if name == "Q" and not is_diss:
            continue
        _, _, Z = _grid(np.zeros_like(x), np.zeros_like(y), a.reshape(ez, 5), ex, ey, ez)
        out[name] = np.ascontiguousarray(Z, np.float32)
    n = 125 * ex * ey * ez
    for name in ("A", "B", "C"):
        out[name] = np.zeros(n, np.float32)
    return out


MODEL_TYPES = {1: "homogeneous", 2: "prem_iso", 3: "homogeneous_plus_Q", 4: "eumod_bg", 7: "ak135"}


def builtin_model(box: F.Box, model_type: int, is_diss: int) -> Dict[str, np.ndarray]:
    """The MODELS records of one box for the setup's model_type (generate_models.f90:389-417):
    1 homogeneous, 2 isotropic PREM, 3 homogeneous + QL6 Q, 4 EUMOD background, 7 ak135
    (ses3d_gb300.earth_models). Q is part of the records only with attenuation, as
    generate_models writes it (generate_models.f90:436-453); type 1 leaves it at zero."""
    from . import earth_models as EM
    if model_type not in MODEL_TYPES:
        raise ValueError("model_type %d is not one of the reference's 1-D models %s" % (model_type, sorted(MODEL_TYPES)))
    if model_type == 1:
        return homogeneous(box, is_diss)
    _, _, z = box_axes(box)
    if model_type == 3:
        out = homogeneous(box, is_diss)
        if is_diss:
            ex, ey, ez = box.nx + 1, box.ny + 1, box.nz + 1
            _, _, Z = _grid(np.zeros((ex, 5), np.float32), np.zeros((ey, 5), np.float32),
                            EM.ql6(z, is_diss).reshape(ez, 5), ex, ey, ez)
            out["Q"] = np.ascontiguousarray(Z, np.float32)
        return out
    fn = {2: EM.prem_iso, 4: EM.eumod_bg, 7: EM.ak135}[model_type]
    rho, vp, vs, q = fn(z, is_diss)
    return records_from_si(box, rho, vp, vs, q, is_diss)


def generate_models(setup: F.Setup, root: str, profile: Optional[Profile] = None,
                    coordinates: bool = True) -> List[F.Box]:
    """generate_models: boxfile, coordinate files and per-rank model records of a SES3D tree
    under root (MODELS/MODELS/, DATA/COORDINATES/). profile None: the setup's model_type
    (builtin_model)."""
    boxes = F.make_boxes(setup)
    mdir = os.path.join(root, "MODELS", "MODELS")
    os.makedirs(mdir, exist_ok=True)
    F.write_boxfile(os.path.join(mdir, "boxfile"), boxes, setup.px, setup.py, setup.pz)
    for r, b in enumerate(boxes):
        m = (builtin_model(b, setup.model_type, setup.is_diss) if profile is None
             else profile_model(b, profile, setup.is_diss))
        F.write_model(mdir, r, m)
        if coordinates:
            write_coordinates(os.path.join(root, "DATA", "COORDINATES"), r, b)
    return boxes


# ------------------------------------------------------------------------------------------------
# block models (TOOLS/models.py:157-310) and add_perturbation (add_perturbation.f90:296-534)
# ------------------------------------------------------------------------------------------------

@dataclass
class SubVolume:
    x: np.ndarray          # colatitude of the cell boundaries [deg] (block_x)
    y: np.ndarray          # longitude [deg] (block_y)
    z: np.ndarray          # radius [km] (block_z)
    v: np.ndarray          # (len(x)-1, len(y)-1, len(z)-1) cell values


def _read_list(path: str) -> List[str]:
    with open(path) as fh:
        return [ln.strip() for ln in fh.read().strip().split("\n")]


def read_block_lines(path: str) -> List[np.ndarray]:
    """block_x / block_y / block_z: number of subvolumes, then per subvolume a count and that
    many coordinates (read as REAL(4))."""
    t = _read_list(path)
    nsub, pos, out = int(t[0]), 1, []
    for _ in range(nsub):
        n = int(t[pos])
        out.append(np.array([F.strtof(v) for v in t[pos + 1:pos + 1 + n]], np.float32))
        pos += 1 + n
    return out


def read_block_values(path: str, shapes: Sequence[Tuple[int, int, int]]) -> List[np.ndarray]:
    """A block model file: number of subvolumes, then per subvolume its cell count and the
    values with x outermost and z innermost."""
    t = _read_list(path)
    pos, out = 1, []
    for shp in shapes:
        n = int(t[pos])
        out.append(np.array([F.strtof(v) for v in t[pos + 1:pos + 1 + n]], np.float32).reshape(shp))
        pos += 1 + n
    return out


def read_block_model(directory: str, name: str) -> List[SubVolume]:
    bx = read_block_lines(os.path.join(directory, "block_x"))
    by = read_block_lines(os.path.join(directory, "block_y"))
    bz = read_block_lines(os.path.join(directory, "block_z"))
    vals = read_block_values(os.path.join(directory, name),
                             [(len(a) - 1, len(b) - 1, len(c) - 1) for a, b, c in zip(bx, by, bz)])
    return [SubVolume(a, b, c, v) for a, b, c, v in zip(bx, by, bz, vals)]


def write_block_lines(path: str, lines: Sequence[np.ndarray]):
    L = [str(len(lines))]
    for a in lines:
        L.append(str(len(a)))
        L += [F.fmt_plain(v) for v in a]
    with open(path, "w") as fh:
        fh.write("\n".join(L) + "\n")


def write_block_model(directory: str, name: str, subvols: Sequence[SubVolume], coords: bool = True):
    """Writes <name> (and block_x/y/z when coords) in the block format."""
    os.makedirs(directory, exist_ok=True)
    if coords:
        write_block_lines(os.path.join(directory, "block_x"), [s.x for s in subvols])
        write_block_lines(os.path.join(directory, "block_y"), [s.y for s in subvols])
        write_block_lines(os.path.join(directory, "block_z"), [s.z for s in subvols])
    L = [str(len(subvols))]
    for s in subvols:
        L.append(str(s.v.size))
        L += [F.fmt_plain(v) for v in np.asarray(s.v, np.float32).reshape(-1)]
    with open(os.path.join(directory, name), "w") as fh:
        fh.write("\n".join(L) + "\n")


def _cell_range(b: np.ndarray, lo: f32, hi: f32) -> Tuple[int, int]:
    """start/end cell (1-based, inclusive) of add_perturbation.f90:423-462: start = last cell
    whose lower boundary lies below the box, end = first cell from the top whose lower
    boundary lies above it."""
    nb = len(b)
    start, end = 1, nb - 1
    for i in range(1, nb):
        if b[i - 1] < lo:
            start = i
    for i in range(nb - 1, 0, -1):
        if b[i - 1] > hi:
            end = i
    return start, end


def _axis_cells(coord: np.ndarray, b: np.ndarray, start: int, end: int, upper_closed: bool) -> np.ndarray:
    """Cell index (0-based) per node coordinate, -1 where the node is in no cell of
    [start, end]: b[i] <= c < b[i+1] (x, y) or b[i] < c <= b[i+1] (z, upper_closed).
    Cells are scanned like the reference loops; a node in several (overlapping) cells takes
    the last, which is what sequential `where` additions within one subvolume would need
    and never happens for increasing boundaries."""
    out = np.full(coord.shape, -1, np.int64)
    for i in range(start, end + 1):
        lo, hi = b[i - 1], b[i]
        m = (coord > lo) & (coord <= hi) if upper_closed else (coord >= lo) & (coord < hi)
        out[m] = i - 1
    return out


def add_perturbation(model: Dict[str, np.ndarray], box: F.Box, directory: str) -> Dict[str, np.ndarray]:
    """add_perturbation for one box: velocities from the model, block perturbations dvsh,
    dvsv, dvp [km/s] and drho [g/cm^3] of `directory` added at the GLL points inside each
    cell (subvolumes in file order), then mu = rho csh^2, B = rho csv^2 - mu,
    lambda = rho cp^2 - 2 mu, rhoinv = 1/rho (add_perturbation.f90:327-534). A, C and Q are
    unchanged."""
    rhoinv, mu, lam, B = (np.asarray(model[k], np.float32) for k in ("rhoinv", "mu", "lambda", "B"))
    csh = np.sqrt((mu * rhoinv).astype(np.float32)).astype(np.float32)
    csv = np.sqrt(((mu + B).astype(np.float32) * rhoinv).astype(np.float32)).astype(np.float32)
    cp = np.sqrt(((lam + (f32(2) * mu).astype(np.float32)).astype(np.float32) * rhoinv).astype(np.float32)).astype(
        np.float32)
    rho = (f32(1) / rhoinv).astype(np.float32)
    x, y, z = box_axes(box)
    ex, ey, ez = box.nx + 1, box.ny + 1, box.nz + 1
    sh = read_block_model(directory, "dvsh")
    sv = read_block_values(os.path.join(directory, "dvsv"), [s.v.shape for s in sh])
    vp = read_block_values(os.path.join(directory, "dvp"), [s.v.shape for s in sh])
    dr = read_block_values(os.path.join(directory, "drho"), [s.v.shape for s in sh])
    for s, dsv, dvp, drh in zip(sh, sv, vp, dr):
        bx = ((s.x * PI_SOLVER).astype(np.float32) / f32(180)).astype(np.float32)
        by = ((s.y * PI_SOLVER).astype(np.float32) / f32(180)).astype(np.float32)
        bz = (s.z * f32(1000)).astype(np.float32)
        sx0, sx1 = _cell_range(bx, f32(box.xmin), f32(box.xmax))
        sy0, sy1 = _cell_range(by, f32(box.ymin), f32(box.ymax))
        sz0, sz1 = _cell_range(bz, f32(box.zmin), f32(box.zmax))
        cx = _axis_cells(x, bx, sx0, sx1, False)     # (ex, 5)
        cy = _axis_cells(y, by, sy0, sy1, False)
        cz = _axis_cells(z, bz, sz0, sz1, True)
        I, J, K = _grid(cx, cy, cz, ex, ey, ez)
        inside = (I >= 0) & (J >= 0) & (K >= 0)
        q = (I[inside], J[inside], K[inside])
        d_sh = (f32(1000) * s.v).astype(np.float32)[q]
        d_sv = (f32(1000) * dsv).astype(np.float32)[q]
        d_vp = (f32(1000) * dvp).astype(np.float32)[q]
        d_rh = (f32(1000) * drh).astype(np.float32)[q]
        csv[inside] = (csv[inside] + d_sv).astype(np.float32)
        csh[inside] = (csh[inside] + d_sh).astype(np.float32)
        cp[inside] = (cp[inside] + d_vp).astype(np.float32)
        rho[inside] = (rho[inside] + d_rh).astype(np.float32)
    out = dict(model)
    mu2 = ((rho * csh).astype(np.float32) * csh).astype(np.float32)
    out["mu"] = mu2
    out["B"] = (((rho * csv).astype(np.float32) * csv).astype(np.float32) - mu2).astype(np.float32)
    out["lambda"] = (((rho * cp).astype(np.float32) * cp).astype(np.float32) - (f32(2) * mu2).astype(np.float32)
                     ).astype(np.float32)
    out["rhoinv"] = (f32(1) / rho).astype(np.float32)
    return out


def add_perturbation_tree(root: str, block_dir: Optional[str] = None) -> List[F.Box]:
    """add_perturbation over every box of a tree (MODELS/MODELS/boxfile and records, block
    model in MODELS/MODELS_3D unless block_dir is given); records are rewritten in place."""
    mdir = os.path.join(root, "MODELS", "MODELS")
    block_dir = block_dir or os.path.join(root, "MODELS", "MODELS_3D")
    boxes = F.read_boxfile(os.path.join(mdir, "boxfile"))
    for r, b in enumerate(boxes):
        n = 125 * (b.nx + 1) * (b.ny + 1) * (b.nz + 1)
        m = {}
        for nm in ("rhoinv", "mu", "lambda", "A", "B", "C"):
            m[nm] = F.read_record(os.path.join(mdir, "%s%d" % (nm, r)), n)
        new = add_perturbation(m, b, block_dir)
        F.write_model(mdir, r, {k: new[k] for k in ("rhoinv", "mu", "lambda", "A", "B", "C")})
    return boxes

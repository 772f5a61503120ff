"""Seeded synthetic SES3D problems in the reference file formats.

The reference ships no model binaries (its MODELS/MODELS directory is produced
by generate_models.exe, which needs Fortran + MPI), so the workloads are
generated here: a spherical section, a 1-D layered model with optional 3-D
perturbations, SLS relaxation parameters fitted for constant Q, a filtered
Heaviside source-time function, a seeded moment tensor and seeded surface
receivers. Everything is written exactly in the formats the solver reads
(formats.py), so the GPU library, the CPU oracle and the reference consume the
same inputs.

Workloads (element counts; lpd = 4):
  c1  22 x 22 x 10, 1-D two-layer model, 10 receivers, dt 0.1 s, nt 1000
  c2  96 x 96 x 40, 1-D + Gaussian-correlated perturbation (100 km), 200 receivers, dt 0.05 s, nt 5000
  c3  64 x 64 x 32 gradient workload, 50 receivers, nt 4000, samp_ad 10
  c4  48 x 48 x 24, 16 events, 20-200 receivers each, dt 0.08 s, nt 3000
  c5  96 x 96 x 40, 16 events (gradient), nt 4000
"""
from __future__ import annotations

import copy
import os
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from . import formats as F

KNOTS4 = np.array([-1.0, -0.6546536707079772, 0.0, 0.6546536707079772, 1.0], np.float32)
R_EARTH = 6371000.0


@dataclass
class EventSpec:
    event: F.Event
    stf: np.ndarray                 # nt+1 samples (the solver reads the first nt)
    receivers: F.Receivers
    name: str = "1"


@dataclass
class Problem:
    setup: F.Setup
    box: F.Box
    tau: np.ndarray
    D: np.ndarray
    model: Dict[str, np.ndarray]     # reference-layout FP32 arrays
    events: List[EventSpec]
    pml: int = 3
    label: str = ""

    @property
    def nx(self):
        return self.box.nx

    @property
    def ny(self):
        return self.box.ny

    @property
    def nz(self):
        return self.box.nz

    @property
    def n_elements(self):
        return (self.nx + 1) * (self.ny + 1) * (self.nz + 1)

    @property
    def n_nodes(self):
        return 125 * self.n_elements


# -----------------------------------------------------------------------------------------------
# building blocks
# -----------------------------------------------------------------------------------------------

def node_axes(box: F.Box):
    """Node coordinates per axis as generate_models.f90:336-358 computes them (FP32):
    x[i, n] (rad), y[j, n] (rad), z[k, n] (radius m)."""
    f = np.float32
    ex, ey, ez = box.nx + 1, box.ny + 1, box.nz + 1
    dx = (box.xmax - box.xmin) / f(ex)
    dy = (box.ymax - box.ymin) / f(ey)
    dz = (box.zmax - box.zmin) / f(ez)
    half = (f(0.5) * (f(1) + KNOTS4)).astype(np.float32)
    x = (box.xmin + np.arange(ex, dtype=np.float32)[:, None] * dx + half[None, :] * dx).astype(np.float32)
    y = (box.ymin + np.arange(ey, dtype=np.float32)[:, None] * dy + half[None, :] * dy).astype(np.float32)
    z = (box.zmax - np.arange(ez, dtype=np.float32)[:, None] * dz - half[None, :] * dz).astype(np.float32)
    return x, y, z


def to_reference_layout(t: np.ndarray, ex: int, ey: int, ez: int) -> np.ndarray:
    """Tensor-grid array (ex*5, ey*5, ez*5) -> flat reference layout (i,j,k,in,jn,kn), i fastest."""
    a = t.reshape(ex, 5, ey, 5, ez, 5).transpose(0, 2, 4, 1, 3, 5)
    return np.ascontiguousarray(a.ravel(order="F"), dtype=np.float32)


def sls_weights(tau_s: np.ndarray, fmin: float, fmax: float) -> np.ndarray:
    """Weights D_p for an approximately constant Q over [fmin, fmax]: least-squares fit of
    sum_p D_p w tau_p / (1 + w^2 tau_p^2) = 1, the loss term of the discrete
    absorption-band formula in TOOLS/Q_discrete.py:89-92."""
    w = 2 * np.pi * np.logspace(np.log10(fmin), np.log10(fmax), 200)
    Amat = np.stack([w * t / (1 + (w * t) ** 2) for t in tau_s], axis=1)
    D, *_ = np.linalg.lstsq(Amat, np.ones_like(w), rcond=None)
    return D.astype(np.float32)


def heaviside_stf(nt: int, dt: float, period: float, highpass: Optional[float] = None) -> np.ndarray:
    """Low-passed Heaviside, causal 5-pole Butterworth (TOOLS/make_stf.py:23-29 with
    scipy.signal standing in for obspy.signal.filter), nt+1 samples."""
    from scipy.signal import butter, sosfilt
    h = np.ones(nt + 1)
    fny = 0.5 / dt
    if highpass:
        h = sosfilt(butter(3, highpass / fny, btype="high", output="sos"), h)
    h = sosfilt(butter(5, (1.0 / period) / fny, output="sos"), h)
    return h.astype(np.float32)


def deviatoric_moment(rng: np.random.Generator, M0: float = 1e18) -> np.ndarray:
    m = rng.standard_normal((3, 3))
    m = 0.5 * (m + m.T)
    m -= np.trace(m) / 3 * np.eye(3)
    m *= M0 / np.sqrt(0.5 * np.sum(m * m))
    # order Mtt, Mpp, Mrr, Mtp, Mtr, Mpr (x = theta, y = phi, z = r)
    return np.array([m[0, 0], m[1, 1], m[2, 2], m[0, 1], m[0, 2], m[1, 2]], np.float32)


def layered_1d(depth_m: np.ndarray):
    """Two-layer model: crust 0-35 km (2.9 g/cc, 6.8, 3.9 km/s, Qmu 300),
    mantle (3.4, 8.1, 4.5, Qmu 150). Returns rho (kg/m^3), vp, vs (m/s), Qmu."""
    crust = depth_m <= 35000.0
    rho = np.where(crust, 2900.0, 3400.0)
    vp = np.where(crust, 6800.0, 8100.0)
    vs = np.where(crust, 3900.0, 4500.0)
    q = np.where(crust, 300.0, 150.0)
    return rho, vp, vs, q


def correlated_field(rng, box: F.Box, corr_len_m: float, spacing_m: float = 20000.0,
                     x=None, y=None, z=None) -> np.ndarray:
    """Seeded Gaussian-correlated random field on the node tensor grid, scaled to max |f| = 1."""
    from scipy.ndimage import gaussian_filter
    xmid = 0.5 * (float(box.xmin) + float(box.xmax))
    Lx = (float(box.xmax) - float(box.xmin)) * R_EARTH
    Ly = (float(box.ymax) - float(box.ymin)) * R_EARTH * np.sin(xmid)
    Lz = float(box.zmax) - float(box.zmin)
    nxc, nyc, nzc = (max(4, int(np.ceil(L / spacing_m)) + 1) for L in (Lx, Ly, Lz))
    g = rng.standard_normal((nxc, nyc, nzc))
    g = gaussian_filter(g, sigma=corr_len_m / spacing_m / np.sqrt(2.0), mode="wrap")
    g /= np.abs(g).max()
    if x is None:
        x, y, z = node_axes(box)
    ux = (x.ravel() - float(box.xmin)) / (float(box.xmax) - float(box.xmin)) * (nxc - 1)
    uy = (y.ravel() - float(box.ymin)) / (float(box.ymax) - float(box.ymin)) * (nyc - 1)
    uz = (z.ravel() - float(box.zmin)) / (float(box.zmax) - float(box.zmin)) * (nzc - 1)

    def interp_matrix(u, n):
        i0 = np.clip(np.floor(u).astype(int), 0, n - 2)
        t = u - i0
        W = np.zeros((u.size, n))
        W[np.arange(u.size), i0] = 1 - t
        W[np.arange(u.size), i0 + 1] = t
        return W

    Wx, Wy, Wz = interp_matrix(ux, nxc), interp_matrix(uy, nyc), interp_matrix(uz, nzc)
    t = np.einsum("ai,ijk->ajk", Wx, g)
    t = np.einsum("bj,ajk->abk", Wy, t)
    t = np.einsum("ck,abk->abc", Wz, t)
    m = np.abs(t).max()
    return (t / m if m > 0 else t).astype(np.float32)


def build_model(box: F.Box, rng=None, dvs=0.0, dvp=0.0, drho_scale=0.3, corr_len=100e3,
                blob=None, checker=None, is_diss=1) -> Dict[str, np.ndarray]:
    """Reference-layout model records. dvs/dvp: amplitudes of the correlated perturbation;
    blob=(dvs, radius_m, depth_m); checker=(dvs, cell_m)."""
    x, y, z = node_axes(box)
    ex, ey, ez = box.nx + 1, box.ny + 1, box.nz + 1
    depth = R_EARTH - z.ravel().astype(np.float64)
    rho1, vp1, vs1, q1 = layered_1d(depth)
    shape = (ex * 5, ey * 5, ez * 5)
    rho = np.broadcast_to(rho1[None, None, :], shape).astype(np.float64)
    vp = np.broadcast_to(vp1[None, None, :], shape).astype(np.float64)
    vs = np.broadcast_to(vs1[None, None, :], shape).astype(np.float64)
    q = np.broadcast_to(q1[None, None, :], shape).astype(np.float64)
    pert = np.zeros(shape)
    if dvs or dvp:
        f = correlated_field(rng, box, corr_len, x=x, y=y, z=z).astype(np.float64)
        vs = vs * (1 + dvs * f)
        vp = vp * (1 + dvp * f)
        rho = rho * (1 + drho_scale * dvs * f)
    if blob is not None:
        amp, rad, dep = blob
        xm = 0.5 * (float(box.xmin) + float(box.xmax)); ym = 0.5 * (float(box.ymin) + float(box.ymax))
        X = x.ravel()[:, None, None].astype(np.float64); Y = y.ravel()[None, :, None].astype(np.float64)
        Zr = z.ravel()[None, None, :].astype(np.float64)
        cx = R_EARTH - dep
        d2 = ((X - xm) * cx) ** 2 + ((Y - ym) * cx * np.sin(xm)) ** 2 + (Zr - cx) ** 2
        pert = amp * np.exp(-d2 / rad ** 2)
        vs = vs * (1 + pert)
    if checker is not None:
        amp, cell = checker
        X = x.ravel()[:, None, None] * R_EARTH; Y = y.ravel()[None, :, None] * R_EARTH
        Zr = z.ravel()[None, None, :]
        s = np.sign(np.sin(np.pi * X / cell) * np.sin(np.pi * Y / cell) * np.sin(np.pi * Zr / cell))
        vs = vs * (1 + amp * s)
    mu = rho * vs * vs
    lam = rho * vp * vp - 2 * mu
    out = {
        "rhoinv": to_reference_layout(1.0 / rho, ex, ey, ez),
        "mu": to_reference_layout(mu, ex, ey, ez),
        "lambda": to_reference_layout(lam, ex, ey, ez),
        "A": np.zeros(ex * ey * ez * 125, np.float32),
        "B": np.zeros(ex * ey * ez * 125, np.float32),
        "C": np.zeros(ex * ey * ez * 125, np.float32),
    }
    if is_diss:
        out["Q"] = to_reference_layout(q, ex, ey, ez)
    return out


def surface_receivers(rng, setup: F.Setup, n: int, margin_frac: float = 0.2, prefix: str = "R") -> F.Receivers:
    """n seeded surface receivers (depth 0) away from the PML bands."""
    lat = rng.uniform(float(setup.xmin) + margin_frac * float(setup.xmax - setup.xmin),
                      float(setup.xmax) - margin_frac * float(setup.xmax - setup.xmin), n)
    lon = rng.uniform(float(setup.ymin) + margin_frac * float(setup.ymax - setup.ymin),
                      float(setup.ymax) - margin_frac * float(setup.ymax - setup.ymin), n)
    loc = np.zeros((n, 3), np.float32)
    for i in range(n):
        loc[i] = [F.strtof("%.4f" % lat[i]), F.strtof("%.4f" % lon[i]), 0.0]
    names = [("%s%04d_.XX.__" % (prefix, i))[:12] for i in range(n)]
    return F.Receivers(names, loc)


def make_setup(n_el, colat=(40.0, 60.0), lon=(0.0, 20.0), r=(5771000.0, 6371000.0), is_diss=1,
               adjoint_flag=0, samp_ad=10) -> F.Setup:
    s = F.Setup()
    s.xmin, s.xmax = F.strtof(F.fmt_plain(colat[0])), F.strtof(F.fmt_plain(colat[1]))
    s.ymin, s.ymax = F.strtof(F.fmt_plain(lon[0])), F.strtof(F.fmt_plain(lon[1]))
    s.zmin, s.zmax = F.strtof(F.fmt_plain(r[0])), F.strtof(F.fmt_plain(r[1]))
    s.is_diss = is_diss
    s.model_type = 1
    s.nx_global, s.ny_global, s.nz_global = n_el[0] - 1, n_el[1] - 1, n_el[2] - 1
    s.lpd = 4
    s.px = s.py = s.pz = 1
    s.adjoint_flag = adjoint_flag
    s.samp_ad = samp_ad
    s.ffd = "../DATA/OUTPUT/ADJOINT"
    return s


def make_event(rng, setup: F.Setup, nt: int, dt: float, depth_m: float, period: float, n_rec: int,
               name: str = "1", source_type: int = 10, jitter_deg: float = 1.0) -> EventSpec:
    e = F.Event()
    e.nt = nt
    e.dt = F.strtof(F.fmt_plain(dt))
    cx = 0.5 * (float(setup.xmin) + float(setup.xmax)) + rng.uniform(-jitter_deg, jitter_deg)
    cy = 0.5 * (float(setup.ymin) + float(setup.ymax)) + rng.uniform(-jitter_deg, jitter_deg)
    e.xxs = F.strtof("%.3f" % cx)
    e.yys = F.strtof("%.3f" % cy)
    e.zzs = F.strtof("%.1f" % depth_m)
    e.source_type = source_type
    e.mom = deviatoric_moment(rng)
    e.mom = np.array([F.strtof(F.fmt_plain(m)) for m in e.mom], np.float32)
    e.ofd = "../DATA/OUTPUT/%s/" % name
    e.ssamp = nt
    e.output_displacement = 0
    stf = heaviside_stf(nt, float(e.dt), period)
    rec = surface_receivers(rng, setup, n_rec)
    return EventSpec(e, stf, rec, name)


def homogeneous_problem(n_el=(10, 9, 6), colat=(48.0, 52.0), lon=(8.0, 12.0), r=(6071000.0, 6371000.0),
                        nt: int = 600, dt: float = 0.1, pml: int = 3, source_type: int = 1,
                        depth_m: float = 150000.0, rho: float = 3000.0, vp: float = 7000.0, vs: float = 4000.0,
                        t0: float = 8.0, sigma: float = 3.0, amplitude: float = 1e15) -> Problem:
    """Known-answer workload: an elastic homogeneous box (rho, vp, vs), a point source at the
    box centre, depth_m below one surface receiver, with a Gaussian source time function
    exp(-((t - t0) / sigma)^2) * amplitude. source_type 1/2/3: single force along
    colatitude / longitude / radius; 10: the moment tensor diag(1, 1, 1) * amplitude."""
    rng = np.random.default_rng(0)
    setup = make_setup(n_el, colat=colat, lon=lon, r=r, is_diss=0)
    box = F.make_boxes(setup)[0]
    m = build_model(box, rng, is_diss=0)
    for k, v in {"rhoinv": 1.0 / rho, "mu": rho * vs ** 2, "lambda": rho * (vp ** 2 - 2.0 * vs ** 2)}.items():
        m[k][:] = np.float32(v)
    ev = make_event(rng, setup, nt, dt, depth_m, 5.0, 1, jitter_deg=0.0)
    ev.event.source_type = source_type
    if source_type == 10:
        ev.event.mom = np.array([amplitude, amplitude, amplitude, 0.0, 0.0, 0.0], np.float32)
        amp = 1.0
    else:
        amp = amplitude
    t = np.arange(nt + 1) * float(ev.event.dt)
    ev.stf = (np.exp(-((t - t0) / sigma) ** 2) * amp).astype(np.float32)
    ev.receivers.loc[:] = [[float(ev.event.xxs), float(ev.event.yys), 0.0]]
    relax_tau = np.array([1.7, 17.0, 170.0], np.float32)
    return Problem(setup, box, relax_tau, np.zeros(3, np.float32), m, [ev], pml=pml, label="homogeneous")


def make_problem(name: str, seed: int = 1234, nt: Optional[int] = None, n_el=None, is_diss: int = 1,
                 adjoint_flag: int = 0, n_events: Optional[int] = None, pml: int = 3,
                 n_rec: Optional[int] = None, model: bool = True) -> Problem:
    """Builds one of the workloads c1..c5, or 'tiny' (small test mesh)."""
    rng = np.random.default_rng(seed)
    specs = {
        #        elements      dt    nt    depth    period  nrec  perturbation
        "tiny": ((6, 5, 4), 0.1, 60, 10000.0, 10.0, 4, None),
        "small": ((10, 9, 6), 0.1, 200, 10000.0, 10.0, 6, None),
        "c1": ((22, 22, 10), 0.1, 1000, 10000.0, 10.0, 10, None),
        "c2": ((96, 96, 40), 0.05, 5000, 15000.0, 8.0, 200, "random"),
        "c3": ((64, 64, 32), 0.08, 4000, 15000.0, 10.0, 50, None),
        "c4": ((48, 48, 24), 0.08, 3000, None, None, None, "random"),
        "c5": ((96, 96, 40), 0.05, 4000, None, None, None, "checker"),
    }
    if name not in specs:
        raise ValueError("unknown workload %r" % name)
    el, dt, nt0, depth, period, nrec, pert = specs[name]
    if n_el is not None:
        el = tuple(n_el)
    nt = nt0 if nt is None else nt
    setup = make_setup(el, is_diss=is_diss, adjoint_flag=adjoint_flag)
    boxes = F.make_boxes(setup)
    box = boxes[0]
    relax_tau = np.array([F.strtof(F.fmt_plain(t)) for t in np.logspace(np.log10(1.7), np.log10(170.0), 3)],
                         np.float32)
    D = sls_weights(relax_tau.astype(np.float64), 1.0 / 100.0, 1.0 / 8.0)
    D = np.array([F.strtof(F.fmt_plain(d)) for d in D], np.float32)
    mdl = {}
    if model:
        if pert == "random":
            mdl = build_model(box, rng, dvs=0.05, dvp=0.03, is_diss=is_diss)
        elif pert == "checker":
            mdl = build_model(box, rng, checker=(0.04, 200e3), is_diss=is_diss)
        else:
            mdl = build_model(box, rng, is_diss=is_diss)
    nev = n_events if n_events is not None else (16 if name in ("c4", "c5") else 1)
    events = []
    for k in range(nev):
        if name in ("c4", "c5"):
            d = rng.uniform(5000.0, 60000.0)
            per = rng.uniform(6.0, 20.0)
            nr = int(rng.integers(20, 201)) if n_rec is None else n_rec
        else:
            d, per, nr = depth, period, (nrec if n_rec is None else n_rec)
        events.append(make_event(rng, setup, nt, dt, d, per, nr, name=str(k + 1)))
    return Problem(setup, box, relax_tau, D, mdl, events, pml=pml, label=name)


def split_setup(setup: F.Setup, n_el, procs) -> F.Setup:
    """The setup of the same mesh decomposed into px x py x pz processor boxes
    (nx_global = elements - px, INPUT/setup:11)."""
    s = copy.deepcopy(setup)
    s.px, s.py, s.pz = procs
    s.nx_global, s.ny_global, s.nz_global = n_el[0] - procs[0], n_el[1] - procs[1], n_el[2] - procs[2]
    return s


def write_problem(p: Problem, root: str, procs=(1, 1, 1)):
    """Writes the reference directory tree under root (INPUT/, MODELS/MODELS/, MAIN/);
    procs = (px, py, pz) > 1 writes it decomposed into processor boxes the way the
    reference's model generator does (per-rank model files, boxfile of all boxes)."""
    inp = os.path.join(root, "INPUT")
    os.makedirs(inp, exist_ok=True)
    os.makedirs(os.path.join(root, "MAIN"), exist_ok=True)
    os.makedirs(os.path.join(root, "MODELS", "MODELS"), exist_ok=True)
    F.write_setup(os.path.join(inp, "setup"), p.setup)
    F.write_relax(os.path.join(inp, "relax"), p.tau, p.D)
    F.write_event_list(os.path.join(inp, "event_list"), [e.name for e in p.events])
    for e in p.events:
        F.write_event(os.path.join(inp, "event_" + e.name), e.event)
        F.write_recfile(os.path.join(inp, "recfile_" + e.name), e.receivers)
    # the reference reads one stf file for every event (SOURCE/ses3d_input.f90:415)
    F.write_stf(os.path.join(inp, "stf"), p.events[0].stf, float(p.events[0].event.dt))
    mdir = os.path.join(root, "MODELS", "MODELS")
    if tuple(procs) == (1, 1, 1):
        F.write_boxfile(os.path.join(mdir, "boxfile"), [p.box], 1, 1, 1)
        F.write_model(mdir, 0, p.model)
        return
    s = split_setup(p.setup, (p.nx + 1, p.ny + 1, p.nz + 1), procs)
    F.write_setup(os.path.join(inp, "setup"), s)
    boxes = F.make_boxes(s)
    F.write_boxfile(os.path.join(mdir, "boxfile"), boxes, *procs)
    pieces = {k: F.split_field(v, boxes) for k, v in p.model.items()}
    for r in range(len(boxes)):
        F.write_model(mdir, r, {k: v[r] for k, v in pieces.items()})

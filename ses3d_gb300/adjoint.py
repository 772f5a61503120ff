"""Differentiable waveform misfit: torch.autograd.Function from the model (rho, vp, vsh,
vsv, Q_mu) to the L2 misfit of band-passed velocity seismograms, whose backward is the
adjoint solve of the reference (adjoint_flag 2 with time-reversed adjoint sources,
SOURCE/ses3d_main.f90:142-176) and its Frechet kernels (SOURCE/ses3d_grad.f90:77-83,
SOURCE/ses3d_grad_Q.f90:115-128).

Model parameters are element-local node values in the reference layout, FP32 tensors on
the GPU. The model records follow the radially anisotropic mapping of
MODELS/SOURCE/add_perturbation.f90:512-520 (mu = rho vsh^2, B = rho vsv^2 - mu,
lambda = rho vp^2 - 2 mu, A = C = 0). The misfit and its time series accumulate in FP64.

Gradient. The kernels K_m of the reference are densities for absolute perturbations of
(rho at fixed velocities, vp, vsh, vsv) and a relative kernel for Q_mu, integrated with
the rectangle rule over the stored iterations (weight samp_ad dt) and divided by the
element Jacobian. The gradient with respect to the value of m at element-local GLL point
(e, n) is Jac W_(e,n) K_m(e, n), W = w_i w_j w_k Jac r^2 sin(theta) the point's
quadrature volume; for Q_mu it is divided by Q. This is the continuous-adjoint gradient of
the reference (not the exact discrete adjoint of the time stepping); the test suite
reports its agreement with central finite differences.

Exact gradient (MisfitSetup.exact = True): the backward pass is the exact discrete adjoint
of the forward time stepping (ses3d_gpu_exact_*): the forward run keeps full-state
checkpoints every K iterations, the seismogram derivative dchi/du(t) = dt F^T F (u - d)(t)
enters at the receivers, the library runs the transposed iterations nt .. 1 and returns
dchi/d(rhoinv, mu, lambda, A, B, C, Q), and the chain rule through the record mapping
(model_gradients_from_records) gives dchi/d(rho, vp, vsh, vsv, Q). It is the derivative of
the computed misfit itself, which central finite differences of the forward run converge
to.

Adjoint source of a velocity misfit: a(t) = dchi/du_vel(t) = dt F^T F (u - d)(t); the
force applied in adjoint iteration it is the time derivative of the time-reversed a
(TOOLS/adjoint_source.py writes the reversed -d/dt of the velocity residual).
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from . import _lib as L
from .solver import Simulation, config_from, select_device


class Bandpass:
    """Zero-phase band-pass with a raised-cosine response, applied by zero-padded FFT.
    Its matrix is symmetric (real even response), so it is its own adjoint."""

    def __init__(self, nt: int, dt: float, fmin: float, fmax: float, taper: float = 0.5):
        self.nt = nt
        self.nfft = 1 << int(math.ceil(math.log2(2 * nt)))
        f = np.fft.rfftfreq(self.nfft, dt)
        H = np.zeros_like(f)
        lo0, lo1 = fmin * (1 - taper), fmin
        hi0, hi1 = fmax, fmax * (1 + taper)
        H[(f >= lo1) & (f <= hi0)] = 1.0
        m = (f > lo0) & (f < lo1)
        H[m] = 0.5 - 0.5 * np.cos(np.pi * (f[m] - lo0) / (lo1 - lo0))
        m = (f > hi0) & (f < hi1)
        H[m] = 0.5 + 0.5 * np.cos(np.pi * (f[m] - hi0) / (hi1 - hi0))
        self.H = H

    def __call__(self, x: np.ndarray) -> np.ndarray:
        X = np.fft.rfft(np.asarray(x, np.float64), n=self.nfft, axis=-1)
        return np.fft.irfft(X * self.H, n=self.nfft, axis=-1)[..., : self.nt]


def model_records(rho, vp, vsh, vsv, Q):
    """SES3D model records from (rho, vp, vsh, vsv, Q) tensors (add_perturbation.f90:512-520)."""
    import torch
    with torch.no_grad():
        mu = rho * vsh * vsh
        rec = {"rhoinv": 1.0 / rho, "mu": mu, "lambda": rho * vp * vp - 2.0 * mu,
               "A": torch.zeros_like(rho), "B": rho * vsv * vsv - mu, "C": torch.zeros_like(rho), "Q": Q}
        return {k: v.float().contiguous() for k, v in rec.items()}


@dataclass
class EventData:
    """One event of an inversion: source, receivers and observed velocity seismograms."""
    xxs: float
    yys: float
    zzs: float
    source_type: int
    mom: np.ndarray
    stf: np.ndarray
    recloc: np.ndarray               # (nr, 3) colat deg, lon deg, depth m
    observed: Optional[np.ndarray] = None   # (3, nr, nt) velocity


@dataclass
class MemoryPlan:
    """Sub-batches of `events_per_batch` events, checkpoint segment length K (0: keep
    every record) and sub-segment length K2 (0: one checkpoint level)."""
    events_per_batch: int
    K: int
    n_events: int
    K2: int = 0

    @property
    def groups(self) -> List[List[int]]:
        g = self.events_per_batch
        return [list(range(a, min(a + g, self.n_events))) for a in range(0, self.n_events, g)]


@dataclass
class MisfitSetup:
    """Mesh, time axis and events of a misfit; built from a synth.Problem by from_problem."""
    cfg_template: object
    events: List[EventData]
    fmin: float = 1.0 / 50.0
    fmax: float = 1.0 / 10.0
    samp_ad: int = 10
    memory_budget: Optional[float] = None  # device bytes a gradient may use; None: free device memory
    grad_q: bool = True
    exact: bool = False          # backward = exact discrete adjoint of the time stepping
    checkpoint_steps: Optional[int] = None  # exact: forward iterations per checkpoint (None: planned)
    lean: bool = True            # reference kernels: forward and adjoint runs step lean (displacement
                                 # gradients outside the PML from the displacement, on stored iterations)
    last: dict = field(default_factory=dict)

    @classmethod
    def from_problem(cls, p, n_events: Optional[int] = None, samp_ad: int = 10, **kw) -> "MisfitSetup":
        nev = len(p.events) if n_events is None else n_events
        ev0 = p.events[0].event
        cfg = config_from(p.box, p.setup, ev0.nt, ev0.dt, p.tau, p.D, pml=p.pml, adjoint_flag=1, n_events=nev,
                          grad_variant=1)
        cfg.samp_ad = samp_ad
        evs = [EventData(float(e.event.xxs), float(e.event.yys), float(e.event.zzs), e.event.source_type,
                         np.asarray(e.event.mom, np.float32), np.asarray(e.stf, np.float32),
                         np.asarray(e.receivers.loc, np.float32)) for e in p.events[:nev]]
        return cls(cfg, evs, samp_ad=samp_ad, **kw)

    # -- simulation plumbing --------------------------------------------------------------------
    def _config(self, adjoint_flag: int, n_events: Optional[int] = None):
        c = L.Config()
        ctypes_copy(c, self.cfg_template)
        c.adjoint_flag = adjoint_flag
        c.samp_ad = self.samp_ad
        c.n_events = len(self.events) if n_events is None else n_events
        c.grad_variant = 1 if self.grad_q else 0
        return c

    def simulate(self, records: dict, adjoint: bool = False, events: Optional[Sequence[int]] = None,
                 K: Optional[int] = None, K2: int = 0) -> Simulation:
        """Forward run of the given events (default: all) on the model records (device
        tensors). adjoint: keep the forward records, or checkpoints every K records (and,
        with K2, second-level checkpoints every K2 records of a segment)."""
        evs = list(range(len(self.events))) if events is None else list(events)
        self.check_records(records)
        select_device(next(iter(records.values())).device.index or 0)  # the handle lives with the model
        sim = Simulation(self._config(1 if adjoint else 0, len(evs)))
        sim.set_model_device([records[k].data_ptr() if k in records else 0 for k in
                              ("rhoinv", "mu", "lambda", "A", "B", "C", "Q")])
        for slot, k in enumerate(evs):
            e = self.events[k]
            sim.set_source(slot, e.xxs, e.yys, e.zzs, e.source_type, e.mom, e.stf)
            sim.set_receivers(slot, e.recloc)
        sim.use_graph(True, 10)   # plain iterations (between stored ones) replay from CUDA graphs
        # lean stepping: outside the PML no displacement gradients are kept; seismograms do not
        # need them and records take them from the displacement
        sim.set_lean(self.lean or not adjoint)
        if adjoint:
            if K is None:
                pl = self.plan()
                K, K2 = pl.K, pl.K2
            if K:
                L.check(sim.lib.ses3d_gpu_set_checkpoint_levels(sim.h, K, K2), sim.h)
            self.last["records_per_segment"] = K
            self.last["records_per_subsegment"] = K2
        sim.run()
        return sim

    def simulate_exact(self, records: dict, events: Sequence[int], K: int, K2: int = 0) -> Simulation:
        """Plain forward run of the given events that keeps full-state checkpoints every K
        iterations for the exact discrete adjoint (ses3d_gpu_exact_adjoint; with K2 a second
        checkpoint level every K2 iterations of a segment)."""
        self.check_records(records)
        select_device(next(iter(records.values())).device.index or 0)
        sim = Simulation(self._config(0, len(events)))
        sim.set_model_device([records[k].data_ptr() if k in records else 0 for k in
                              ("rhoinv", "mu", "lambda", "A", "B", "C", "Q")])
        for slot, k in enumerate(events):
            e = self.events[k]
            sim.set_source(slot, e.xxs, e.yys, e.zzs, e.source_type, e.mom, e.stf)
            sim.set_receivers(slot, e.recloc)
        sim.exact_adjoint(K, K2)
        sim.set_lean(True)        # the run starts at rest: lean iterations are exact for it
        sim.use_graph(True, 10)
        sim.run()
        return sim

    def exact_plan(self) -> MemoryPlan:
        """Events per sub-batch and checkpointing of the exact adjoint. Per event: the state,
        velocity and forces, the adjoint state and its FP64 gradients, and either
        ceil(nt / K) checkpoints and K iteration slots (one level, K ~ sqrt(nt)), or
        ceil(nt / K) + ceil(K / K2) - 1 checkpoints and K2 slots (two levels, one more
        recompute pass). The largest sub-batch that fits wins, with one level before two."""
        c = self.cfg_template
        E = (c.nx + 1) * (c.ny + 1) * (c.nz + 1)
        N, G = 125.0 * E, float((4 * c.nx + 5) * (4 * c.ny + 5) * (4 * c.nz + 5))
        nt = int(c.nt)
        # an iteration slot keeps the 9 displacement gradients, the 6 memory-variable sums
        # (attenuation only; element blocks of 1,876 or 1,128 floats), the velocity and the
        # assembled forces
        ckpt, slot = (36.0 * N + 3.0 * G) * 4, ((1876.0 if c.is_diss else 1128.0) * E + 6.0 * G) * 4
        shared = 64.0 * N + 12.0 * G
        event = (36.0 * N + 3.0 * G + 3.0 * N) * 4 + (39.0 * N + 6.0 * G) * 4 + (6.0 * N + G) * 8 + ckpt
        if self.checkpoint_steps:
            K = min(nt, self.checkpoint_steps)
        else:
            K = max(1, min(nt, int(round(math.sqrt(nt * ckpt / slot)))))
        one = event + math.ceil(nt / K) * ckpt + K * slot
        best = None
        for K1 in range(2, nt + 1):
            k2c = max(1, min(K1 - 1, int(round(math.sqrt(K1 * ckpt / slot)))))
            for K2 in range(max(1, k2c - 1), min(K1 - 1, k2c + 1) + 1):
                mem = math.ceil(nt / K1) * ckpt + (math.ceil(K1 / K2) - 1) * ckpt + K2 * slot
                if best is None or mem < best[0]:
                    best = (mem, K1, K2)
        two = event + best[0] if best else one
        budget = self.budget()
        nev = len(self.events)
        for g in range(nev, 0, -1):
            if shared + g * one <= budget:
                return MemoryPlan(g, K, nev)
            if best and shared + g * two <= budget:
                return MemoryPlan(g, best[1], nev, best[2])
        return MemoryPlan(1, best[1], nev, best[2]) if best else MemoryPlan(1, K, nev)

    @property
    def n_points(self) -> int:
        """GLL points of the mesh (the length of every model record)."""
        c = self.cfg_template
        return 125 * (c.nx + 1) * (c.ny + 1) * (c.nz + 1)

    def check_records(self, records: dict):
        """Model records must be contiguous FP32 CUDA tensors of n_points values: the library
        reads them through raw device pointers."""
        import torch
        for k, t in records.items():
            if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()):
                raise TypeError("model record %s must be a contiguous float32 CUDA tensor" % k)
            if t.numel() != self.n_points:
                raise ValueError("model record %s holds %d values; the mesh has %d GLL points"
                                 % (k, t.numel(), self.n_points))

    # -- memory plan ---------------------------------------------------------------------------
    def budget(self) -> float:
        """Device bytes a gradient may use: memory_budget, or the free device memory less a
        reserve (5 % of the device, at least 8 GB)."""
        if self.memory_budget is not None:
            return float(self.memory_budget)
        import torch
        free, total = torch.cuda.mem_get_info()
        return max(0.0, float(free) - max(8e9, 0.05 * float(total)))

    def plan(self) -> "MemoryPlan":
        """Events per sub-batch and checkpointing so that one sub-batch's device memory fits
        the budget. Per event: element state, velocity and forces, FP64 kernel accumulators,
        and either every record (9 floats per GLL point and stored iteration), or
        ceil(nrec / K) full-state checkpoints, K records and a second wavefield (one level),
        or ceil(nrec / K) + ceil(K / K2) - 1 checkpoints, K2 records and a second wavefield
        (two levels); shared per handle: material, geometry, mass matrix. The storage with
        the fewest recompute passes that fits wins (records kept, then one level, then two),
        with the largest sub-batch it allows; K and K2 minimise memory. With nothing
        fitting, one event per sub-batch with two levels."""
        m = self.memory_model()
        budget = self.budget()
        nev = len(self.events)
        # a recompute pass costs a whole forward sweep, while batching saves a few per cent
        # (the material traffic shared by the events): the fewest passes come first
        for per, K, K2 in ((m["keep"], 0, 0), (m["one_level"], m["K"], 0), (m["two_level"], m["K1"], m["K2"])):
            g = min(nev, int((budget - m["shared"]) // per)) if budget > m["shared"] else 0
            if g >= 1:
                return MemoryPlan(g, K, nev, K2)
        return MemoryPlan(1, m["K1"], nev, m["K2"])

    def memory_model(self) -> dict:
        """Device bytes: per handle ("shared"), per event keeping every record ("keep"), with
        one checkpoint level every K records ("one_level") and with two levels every K1 and
        K2 records ("two_level"), and the K, K1, K2 that minimise those."""
        c = self.cfg_template
        E = (c.nx + 1) * (c.ny + 1) * (c.nz + 1)
        N, G = 125.0 * E, float((4 * c.nx + 5) * (4 * c.ny + 5) * (4 * c.nz + 5))
        nt, smp = int(c.nt), self.samp_ad
        nrec = len([it for it in range(1, nt + 1) if it % smp == 0 or it == 1 or it == nt])
        shared = 64.0 * N + 12.0 * G
        # per event: element state, velocity and displacement, element forces, FP64 kernels
        event = (36.0 * N + 6.0 * G + 3.0 * N) * 4 + 64.0 * N
        rec = 36.0 * N
        wave2 = (36.0 * N + 6.0 * G) * 4       # the recomputing wavefield
        if self.lean:   # lean runs checkpoint 24 fields per element, all 36 in PML elements
            p = int(c.pml)
            ex, ey, ez = c.nx + 1, c.ny + 1, c.nz + 1
            e_pml = E - max(0, ex - 2 * p) * max(0, ey - 2 * p) * max(0, ez - p)
            ckpt = (24.0 * N + 12.0 * 125 * e_pml + 6.0 * G) * 4
        else:
            ckpt = wave2
        K = max(1, int(round(math.sqrt(nrec * ckpt / rec))))
        one = event + wave2 + math.ceil(nrec / K) * ckpt + K * rec
        best = None
        for K1 in range(2, max(3, nrec + 1)):
            k2c = max(1, min(K1 - 1, int(round(math.sqrt(K1 * ckpt / rec)))))
            for K2 in range(max(1, k2c - 2), min(K1 - 1, k2c + 2) + 1):
                mem = wave2 + math.ceil(nrec / K1) * ckpt + (math.ceil(K1 / K2) - 1) * ckpt + K2 * rec
                if best is None or mem < best[0]:
                    best = (mem, K1, K2)
        return {"shared": shared, "keep": event + nrec * rec, "one_level": one, "K": K,
                "two_level": event + best[0], "K1": best[1], "K2": best[2]}

    def filt(self, nt: int, dt: float) -> Bandpass:
        return Bandpass(nt, dt, self.fmin, self.fmax)

    def seismograms(self, sim: Simulation) -> List[np.ndarray]:
        """(3, nr, nt) FP64 per event of the handle (its events in slot order)."""
        out = []
        for k in range(sim.n_events):
            sx, sy, sz = sim.seismograms(k)
            out.append(np.stack([sx, sy, sz]).astype(np.float64))  # (3, nr, nt)
        return out

    def forward_seismograms(self, records: dict) -> List[np.ndarray]:
        """Plain forward seismograms of every event, sub-batched like the gradient."""
        syn = []
        for grp in self.plan().groups:
            sim = self.simulate(records, events=grp)
            syn += self.seismograms(sim)
            sim.close()
        return syn

    def set_observed(self, model_tensors: Sequence):
        """Observed data = synthetics of the given (rho, vp, vsh, vsv, Q) model."""
        for e, s in zip(self.events, self.forward_seismograms(model_records(*model_tensors))):
            e.observed = s

    def misfit_value(self, syn: List[np.ndarray], dt: float) -> float:
        F = self.filt(syn[0].shape[-1], dt)
        chi = 0.0
        for e, s in zip(self.events, syn):
            r = F(s - e.observed)
            chi += 0.5 * float(np.sum(r * r)) * dt
        return chi

    def adjoint_sources(self, syn: List[np.ndarray], dt: float, shift: float = 0.0,
                        events: Optional[Sequence[int]] = None):
        """Per event (all, or the listed ones, matching syn): (nr, 3, nt) forces in
        adjoint-iteration order. The force density is the functional derivative of
        chi = 1/2 int |F(u - d)|^2 dt, i.e. F^T F (u - d)(t) per unit time; `shift` delays
        it by a fraction of a sample (alignment studies)."""
        nt = syn[0].shape[-1]
        F = self.filt(nt, dt)
        out = []
        evs = self.events if events is None else [self.events[k] for k in events]
        for e, s in zip(evs, syn):
            a = F(F(s - e.observed))                        # dchi/du_vel(t), (3, nr, nt)
            if shift:
                fr = np.fft.rfftfreq(F.nfft, dt)
                A_ = np.fft.rfft(a, n=F.nfft, axis=-1) * np.exp(-2j * np.pi * fr * shift * dt)
                a = np.fft.irfft(A_, n=F.nfft, axis=-1)[..., :nt]
            g = a[..., ::-1]                                # time reversed: adjoint iteration order
            f = np.gradient(g, dt, axis=-1)                 # d/dtau of the reversed residual
            out.append(np.ascontiguousarray(np.transpose(f, (1, 0, 2)), np.float32))
        return out


def ctypes_copy(dst, src):
    for name, _ in src._fields_:
        v = getattr(src, name)
        if hasattr(v, "_length_"):
            arr = getattr(dst, name)
            for i in range(v._length_):
                arr[i] = v[i]
        else:
            setattr(dst, name, v)


def kernel_sums_device(sim: Simulation, device, acc: Optional[list] = None) -> list:
    """Event-summed kernels of KERNEL_NAMES as FP64 tensors on `device` (no host copy); with
    `acc` (the sums of earlier event sub-batches) the sums are added to it in place."""
    import torch
    torch.cuda.synchronize(device)
    out = []
    for i, nm in enumerate(KERNEL_NAMES):
        if acc is None:
            t = torch.empty(sim.N, dtype=torch.float64, device=device)
            sim.kernel_sum_device(nm, t.data_ptr())   # returns after the library's stream finished
        else:
            t = acc[i]
            sim.add_kernel_sum_device(nm, t.data_ptr())
        out.append(t)
    return out


def misfit_gradients_device(cfg: L.Config, ksum: list, grad_out: float, Q) -> list:
    """dL/dm for (rho, vp, vsh, vsv, Q) from the event-summed kernels, in Q's dtype on Q's
    device: (K * W) * (-grad_out * Jac) with W the quadrature volume of each GLL point, the
    Q_mu one divided by Q (ses3d's kernel sign convention: dchi = -Jac sum W K dm, checked
    against finite differences). One library kernel per model record."""
    import torch
    if Q.dtype not in (torch.float32, torch.float64):
        raise TypeError("model tensors must be float32 or float64")
    n = 125 * (cfg.nx + 1) * (cfg.ny + 1) * (cfg.nz + 1)
    if not Q.is_cuda or Q.numel() != n or any(k.numel() != n or k.dtype != torch.float64 or not k.is_cuda
                                               or not k.is_contiguous() for k in ksum):
        raise ValueError("kernels and Q must be CUDA tensors of %d values (kernels contiguous float64)" % n)
    lib = L.load()
    select_device(Q.device.index or 0)
    f64 = int(Q.dtype == torch.float64)
    q = Q.detach().contiguous()
    torch.cuda.synchronize(Q.device)
    grads = []
    for i, k in enumerate(ksum):
        g = torch.empty(q.shape, dtype=Q.dtype, device=Q.device)
        L.check(lib.ses3d_gpu_misfit_gradient_device(ctypes.byref(cfg), ctypes.c_void_p(k.data_ptr()),
                                                       -float(grad_out),
                                                       ctypes.c_void_p(q.data_ptr()) if i == 4 else None,
                                                       ctypes.c_void_p(g.data_ptr()), f64))
        grads.append(g)
    return grads


KERNEL_NAMES = ("rho", "cp", "csh", "csv", "Q_mu")
RECORD_NAMES = ("rhoinv", "mu", "lambda", "A", "B", "C", "Q")


def record_gradients_device(sim: Simulation, device, acc: Optional[list] = None) -> list:
    """d misfit / d model record (RECORD_NAMES; Q only with attenuation, else None) after an
    exact backward run, FP64 tensors on `device`, added to `acc` (earlier sub-batches)."""
    import torch
    out = []
    for i, nm in enumerate(RECORD_NAMES):
        if nm == "Q" and not sim.cfg.is_diss:
            out.append(None)
            continue
        t = torch.empty(sim.N, dtype=torch.float64, device=device)
        sim.exact_gradient_device(nm, t.data_ptr())
        out.append(t if acc is None else acc[i] + t)
    return out


def model_gradients_from_records(grec: list, rho, vp, vsh, vsv, Q, grad_out: float) -> list:
    """Chain rule through model_records (mu = rho vsh^2, lambda = rho vp^2 - 2 mu,
    B = rho vsv^2 - mu, rhoinv = 1 / rho; A = C = 0) in FP64: d misfit / d (rho, vp, vsh,
    vsv, Q) from the gradients with respect to the records."""
    import torch
    with torch.enable_grad():
        xs = [t.detach().double().requires_grad_(True) for t in (rho, vp, vsh, vsv, Q)]
        r, p_, sh, sv, q = xs
        mu = r * sh * sh
        outs = [1.0 / r, mu, r * p_ * p_ - 2.0 * mu, r * sv * sv - mu, q]
        gl = [grec[0], grec[1], grec[2], grec[4], grec[6]]
        pairs = [(o, g) for o, g in zip(outs, gl) if g is not None]
        gr = torch.autograd.grad([o for o, _ in pairs], xs, grad_outputs=[g for _, g in pairs], allow_unused=True)
    out = []
    for g, x in zip(gr, (rho, vp, vsh, vsv, Q)):
        g = torch.zeros_like(x, dtype=torch.float64) if g is None else g
        out.append((g * float(grad_out)).to(x.dtype))
    return out


class _Misfit:
    """torch.autograd.Function factory (keeps torch an optional import)."""

    @staticmethod
    def build():
        import torch

        class WaveformMisfit(torch.autograd.Function):
            @staticmethod
            def forward(ctx, setup: MisfitSetup, rho, vp, vsh, vsv, Q):
                recs = model_records(rho, vp, vsh, vsv, Q)
                if setup.exact:
                    return WaveformMisfit.forward_exact(ctx, setup, recs, rho, vp, vsh, vsv, Q)
                plan = setup.plan()
                setup.last["plan"] = plan
                dt = float(setup.cfg_template.dt)
                ctx.setup, ctx.dt, ctx.plan = setup, dt, plan
                ctx.save_for_backward(Q)
                if len(plan.groups) == 1:  # one handle keeps the forward records for backward
                    sim = setup.simulate(recs, adjoint=True, K=plan.K, K2=plan.K2)
                    syn = setup.seismograms(sim)
                    ctx.sim, ctx.syn, ctx.kernels = sim, syn, None
                else:
                    # sub-batches: an event's adjoint sources depend on its own residual only,
                    # so each sub-batch runs forward, adjoint and kernel sum here and is freed;
                    # backward scales the summed kernels
                    syn, ksum = [], None
                    for grp in plan.groups:
                        sim = setup.simulate(recs, adjoint=True, events=grp, K=plan.K, K2=plan.K2)
                        sg = setup.seismograms(sim)
                        srcs = setup.adjoint_sources(sg, dt, setup.last.get("shift", 0.0), events=grp)
                        for slot, k in enumerate(grp):
                            sim.set_adjoint_sources(slot, setup.events[k].recloc, srcs[slot])
                        sim.begin_adjoint()
                        sim.set_lean(setup.lean)
                        sim.run()
                        ksum = kernel_sums_device(sim, rho.device, ksum)   # events in index order
                        sim.close()
                        syn += sg
                    ctx.sim, ctx.syn, ctx.kernels = None, syn, ksum
                chi = setup.misfit_value(syn, dt)
                setup.last["seismograms"] = syn
                return torch.tensor(chi, dtype=torch.float64, device=rho.device)

            @staticmethod
            def forward_exact(ctx, setup, recs, rho, vp, vsh, vsv, Q):
                """Forward runs with exact-adjoint checkpoints; with one sub-batch the handle is
                kept for backward, with several each sub-batch runs its backward here (an
                event's seismogram adjoint depends on its own residual only)."""
                plan = setup.exact_plan()
                setup.last["plan"] = plan
                setup.last["steps_per_checkpoint"] = plan.K
                setup.last["steps_per_subsegment"] = plan.K2
                dt = float(setup.cfg_template.dt)
                ctx.setup, ctx.dt, ctx.plan = setup, dt, plan
                ctx.save_for_backward(rho, vp, vsh, vsv, Q)
                ctx.exact = True
                syn, grec = [], None
                ctx.sim = None
                for grp in plan.groups:
                    sim = setup.simulate_exact(recs, grp, plan.K, plan.K2)
                    sg = setup.seismograms(sim)
                    syn += sg
                    if len(plan.groups) == 1:
                        ctx.sim = sim
                    else:
                        WaveformMisfit.exact_backward(setup, sim, sg, grp, dt)
                        grec = record_gradients_device(sim, rho.device, grec)
                        sim.close()
                ctx.syn, ctx.grec = syn, grec
                chi = setup.misfit_value(syn, dt)
                setup.last["seismograms"] = syn
                return torch.tensor(chi, dtype=torch.float64, device=rho.device)

            @staticmethod
            def exact_backward(setup, sim, syn, events, dt):
                """d chi / d seismogram = dt F^T F (u - d) per sample into the handle, then the
                backward run."""
                F = setup.filt(syn[0].shape[-1], dt)
                for slot, (k, s) in enumerate(zip(events, syn)):
                    g = dt * F(F(s - setup.events[k].observed))        # (3, nr, nt)
                    sim.set_seismogram_adjoint(slot, g[0], g[1], g[2])
                sim.exact_backward()

            @staticmethod
            def backward(ctx, grad_out):
                if getattr(ctx, "exact", False):
                    rho, vp, vsh, vsv, Q = ctx.saved_tensors
                    grec = ctx.grec
                    if ctx.sim is not None:
                        WaveformMisfit.exact_backward(ctx.setup, ctx.sim, ctx.syn, ctx.plan.groups[0], ctx.dt)
                        grec = record_gradients_device(ctx.sim, Q.device)
                        ctx.sim.close()
                        ctx.sim = None
                    ctx.setup.last["record_gradients"] = dict(zip(RECORD_NAMES, grec))
                    grads = model_gradients_from_records(grec, rho, vp, vsh, vsv, Q, float(grad_out))
                    ctx.setup.last["kernels"] = {n: g for n, g in zip(("rho", "vp", "vsh", "vsv", "Q"), grads)}
                    return (None,) + tuple(grads)
                (Q,) = ctx.saved_tensors
                setup, syn, dt = ctx.setup, ctx.syn, ctx.dt
                if ctx.kernels is None:
                    sim = ctx.sim
                    srcs = setup.adjoint_sources(syn, dt, setup.last.get("shift", 0.0))
                    for k, e in enumerate(setup.events):
                        sim.set_adjoint_sources(k, e.recloc, srcs[k])
                    sim.begin_adjoint()
                    sim.set_lean(setup.lean)
                    sim.run()
                    ksum = kernel_sums_device(sim, Q.device)
                    sim.close()
                    ctx.sim = None
                else:
                    ksum = ctx.kernels
                grads = misfit_gradients_device(setup.cfg_template, ksum, float(grad_out), Q)
                setup.last["kernels"] = {n: g for n, g in zip(("rho", "vp", "vsh", "vsv", "Q"), grads)}
                return (None,) + tuple(grads)

        return WaveformMisfit


_fn = None


def waveform_misfit(setup: MisfitSetup, rho, vp, vsh, vsv, Q):
    """chi(rho, vp, vsh, vsv, Q) for all events of `setup`; differentiable (backward = adjoint solve)."""
    global _fn
    if _fn is None:
        _fn = _Misfit.build()
    return _fn.apply(setup, rho, vp, vsh, vsv, Q)


def misfit_only(setup: MisfitSetup, rho, vp, vsh, vsv, Q) -> float:
    """chi without keeping records (finite-difference checks)."""
    syn = setup.forward_seismograms(model_records(rho, vp, vsh, vsv, Q))
    return setup.misfit_value(syn, float(setup.cfg_template.dt))


def problem_tensors(p, device="cuda"):
    """(rho, vp, vsh, vsv, Q) tensors of a synth.Problem's model records."""
    import torch
    m = p.model
    rho = 1.0 / m["rhoinv"].astype(np.float64)
    mu = m["mu"].astype(np.float64)
    vsh = np.sqrt(mu / rho)
    vsv = np.sqrt((m["B"].astype(np.float64) + mu) / rho)
    vp = np.sqrt((m["lambda"].astype(np.float64) + 2 * mu) / rho)
    Q = m.get("Q", np.full_like(rho, 1e5)).astype(np.float64)
    return tuple(torch.tensor(a, dtype=torch.float32, device=device) for a in (rho, vp, vsh, vsv, Q))

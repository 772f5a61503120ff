"""Python host interface of the GB300 SES3D solver.

``Simulation`` mirrors the reference program flow (SOURCE/ses3d_main.f90:77-180):
configuration from the boxfile/setup/event/relax values, ``set_model`` for the
MODELS records, sources and receivers per event, ``step`` for the time loop and
getters for seismograms, snapshots, forward-field records and Frechet kernels.
All compute runs in libses3d_gpu.so; arrays crossing this interface use the
reference layout (Fortran order, element index fastest).
"""
from __future__ import annotations

import ctypes
from typing import Dict, Optional, Sequence

import numpy as np

from . import _lib as L
from . import formats as F

RECORD_NAMES = ("rhoinv", "mu", "lambda", "A", "B", "C", "Q")


def config_from(box: F.Box, setup: F.Setup, nt: int, dt, tau, D, pml: int = 2, adjoint_flag: Optional[int] = None,
                n_events: int = 1, grad_variant: int = 0) -> L.Config:
    """ses3d_config from parsed inputs (SOURCE/ses3d_input.f90:96-357)."""
    c = L.Config()
    c.nx, c.ny, c.nz = box.nx, box.ny, box.nz
    c.lpd = setup.lpd
    c.pml = pml
    c.is_diss = setup.is_diss
    c.adjoint_flag = setup.adjoint_flag if adjoint_flag is None else adjoint_flag
    c.samp_ad = setup.samp_ad
    c.nt = nt
    c.n_events = n_events
    c.grad_variant = grad_variant
    c.dt = float(dt)
    c.xmin, c.xmax, c.ymin, c.ymax = float(box.xmin), float(box.xmax), float(box.ymin), float(box.ymax)
    c.zmin, c.zmax = float(box.zmin), float(box.zmax)
    c.zmax_global = float(setup.zmax)
    for k in range(3):
        c.tau_p[k] = float(tau[k])
        c.D_p[k] = float(D[k])
    return c


def select_device(device: int):
    """Creates later handles of this thread on GPU `device` (one rank per GPU)."""
    L.check(L.load().ses3d_gpu_select_device(int(device)))


class Simulation:
    """One handle of the native library: one mesh, one model, n_events events."""

    def __init__(self, cfg: L.Config):
        self.lib = L.load()
        self.cfg = cfg
        h = ctypes.c_void_p()
        rc = self.lib.ses3d_gpu_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc < 0:
            raise L.Ses3dError(rc, (self.lib.ses3d_gpu_last_error(None) or b"").decode())
        self.h = h
        ex, ey, ez = cfg.nx + 1, cfg.ny + 1, cfg.nz + 1
        self.N = 125 * ex * ey * ez
        self.G = (ex * 4 + 1) * (ey * 4 + 1) * (ez * 4 + 1)
        self.nt = cfg.nt
        self.n_events = cfg.n_events
        self._nr = [0] * cfg.n_events
        self._kept = [np.zeros(0, np.int32)] * cfg.n_events
        self._shape = {"elements_per_cta": 1, "element_shape": 0, "node_block": 256}

    # -- construction helpers -------------------------------------------------------------------
    @classmethod
    def from_problem(cls, p, adjoint_flag: Optional[int] = None, n_events: Optional[int] = None,
                     nt: Optional[int] = None, grad_variant: int = 0, model: bool = True) -> "Simulation":
        """A Simulation for a synth.Problem (all its events unless n_events is given)."""
        nev = len(p.events) if n_events is None else n_events
        ev0 = p.events[0].event
        cfg = config_from(p.box, p.setup, ev0.nt if nt is None else nt, ev0.dt, p.tau, p.D, pml=p.pml,
                          adjoint_flag=adjoint_flag, n_events=nev, grad_variant=grad_variant)
        sim = cls(cfg)
        if model:
            sim.set_model(p.model)
        for k in range(nev):
            e = p.events[k]
            sim.set_source(k, e.event.xxs, e.event.yys, e.event.zzs, e.event.source_type, e.event.mom, e.stf)
            if sim.cfg.adjoint_flag != 2:
                sim.set_receivers(k, e.receivers.loc)
        return sim

    def close(self):
        if getattr(self, "h", None):
            self.lib.ses3d_gpu_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        return L.check(rc, self.h)

    # -- inputs ----------------------------------------------------------------------------------
    def set_model(self, model: Dict[str, np.ndarray]):
        arrs = [np.ascontiguousarray(model[k], np.float32) if k in model else None for k in F.MODEL_NAMES]
        for a in arrs[:6]:
            if a is None or a.size != self.N:
                raise ValueError("model arrays must hold %d values" % self.N)
        self._check(self.lib.ses3d_gpu_set_model(self.h, *[L.fptr(a) for a in arrs]))

    def set_model_device(self, ptrs: Sequence[int]):
        """Model records already in device memory (reference layout), e.g. torch tensors' data_ptr()."""
        self._check(self.lib.ses3d_gpu_set_model_device(self.h, *[ctypes.c_void_p(p) if p else None for p in ptrs]))

    def set_source(self, event: int, xxs_deg, yys_deg, zzs, source_type: int, mom, stf) -> int:
        so = np.ascontiguousarray(np.asarray(stf, np.float32)[: self.nt])
        if so.size < self.nt:
            raise ValueError("the stf needs at least nt samples")
        m = np.ascontiguousarray(np.asarray(mom, np.float32).reshape(6))
        isrc = ctypes.c_int(0)
        self._check(self.lib.ses3d_gpu_set_source(self.h, event, float(xxs_deg), float(yys_deg), float(zzs),
                                                  int(source_type), L.fptr(m), L.fptr(so), ctypes.byref(isrc)))
        return isrc.value

    def set_receivers(self, event: int, recloc: np.ndarray) -> np.ndarray:
        loc = np.ascontiguousarray(np.asarray(recloc, np.float32).reshape(-1, 3))
        nr = ctypes.c_int(0)
        kept = np.zeros(max(1, len(loc)), np.int32)
        self._check(self.lib.ses3d_gpu_set_receivers(self.h, event, len(loc), L.fptr(loc), ctypes.byref(nr),
                                                     L.iptr(kept)))
        self._nr[event] = nr.value
        self._kept[event] = kept[: nr.value].copy()
        return self._kept[event]

    def set_adjoint_sources(self, event: int, loc: np.ndarray, stf: np.ndarray) -> int:
        loc = np.ascontiguousarray(np.asarray(loc, np.float32).reshape(-1, 3))
        s = np.ascontiguousarray(np.asarray(stf, np.float32).reshape(len(loc), 3, -1)[:, :, : self.nt])
        n = ctypes.c_int(0)
        self._check(self.lib.ses3d_gpu_set_adjoint_sources(self.h, event, len(loc), L.fptr(loc), L.fptr(s),
                                                           ctypes.byref(n)))
        return n.value

    # -- time loop -------------------------------------------------------------------------------
    def step(self, n: int = 1):
        self._check(self.lib.ses3d_gpu_step(self.h, int(n)))

    def run(self):
        self.step(self.nt - self.it)

    @property
    def it(self) -> int:
        return self.lib.ses3d_gpu_current_step(self.h)

    def use_graph(self, enable: bool = True, n_per_graph: int = 10):
        self._check(self.lib.ses3d_gpu_use_graph(self.h, int(enable), int(n_per_graph)))

    def set_lean(self, enable: bool = True):
        """Plain forward runs: keep displacement gradients only in PML elements (see ses3d_gpu.h)."""
        self._check(self.lib.ses3d_gpu_set_lean(self.h, int(enable)))

    def set_block_elements(self, n: int):
        self._check(self.lib.ses3d_gpu_set_block_elements(self.h, int(n)))
        self._shape["elements_per_cta"] = int(n) or 1

    def set_kernel_shape(self, element_shape: int = 0, node_block: int = 256):
        """Block shapes of the persistent element kernel and the node kernel (ses3d_gpu.h)."""
        self._check(self.lib.ses3d_gpu_set_kernel_shape(self.h, int(element_shape), int(node_block)))
        self._shape.update(element_shape=int(element_shape), node_block=int(node_block))

    @property
    def shape(self) -> dict:
        return dict(self._shape)

    def autotune(self, steps_each: int = 2, node_blocks=(256, 128, 512)) -> dict:
        """Block-shape autotuner over the kernels' real shapes: the persistent element kernel
        in each of its compiled shapes (resident CTAs per SM, refill point) and the
        register-staged kernel with 2 and 4 elements per CTA, then the node kernel's block
        sizes. Each candidate runs one untimed iteration (first launch of its instance) and
        steps_each iterations timed per launch with CUDA events on the library's stream; the
        fastest is kept. The iterations are part of the run (the time axis advances), so call
        it during warm-up; it stops early when the run has too few iterations left. Returns
        {"element": {candidate: ms}, "node": {block: ms}, "chosen": shape}."""
        n_shapes = int(self.lib.ses3d_gpu_kernel_shape_count())
        cands = [("persistent", 1, s) for s in range(n_shapes)] + [("register", 2, 0), ("register", 4, 0)]
        el = {}
        nodes = {}

        def timed(which):
            if self.nt - self.it < steps_each + 1:
                return None
            self.step(1)
            self.profile(True)
            self.step(steps_each)
            ms, n = self.kernel_time(which)
            self.profile(False)
            return ms / max(n, 1)

        for kind, epb, shp in cands:
            self.set_block_elements(epb)
            self.set_kernel_shape(shp, self._shape["node_block"])
            t = timed("element")
            if t is None:
                break
            el["%s epb=%d shape=%d" % (kind, epb, shp)] = (t, epb, shp)
        if el:
            _, epb, shp = min(el.values(), key=lambda v: v[0])
            self.set_block_elements(epb)
            self._shape.update(elements_per_cta=epb, element_shape=shp)
        for nb in node_blocks:
            self.set_kernel_shape(self._shape["element_shape"], nb)
            t = timed("node")
            if t is None:
                break
            nodes[nb] = t
        if nodes:
            self._shape["node_block"] = min(nodes, key=nodes.get)
        self.set_block_elements(self._shape["elements_per_cta"])
        self.set_kernel_shape(self._shape["element_shape"], self._shape["node_block"])
        return {"element": {k: v[0] for k, v in el.items()}, "node": nodes, "chosen": self.shape}

    def begin_adjoint(self):
        self._check(self.lib.ses3d_gpu_begin_adjoint(self.h))
        self.cfg.adjoint_flag = 2

    # -- outputs ---------------------------------------------------------------------------------
    def n_receivers(self, event: int = 0) -> int:
        return self._nr[event]

    def seismograms(self, event: int = 0):
        """(sx, sy, sz), each (nr, nt) with entry [:, it-1] recorded in iteration it."""
        nr = self._nr[event]
        out = [np.zeros((self.nt, nr), np.float32) for _ in range(3)]
        if nr:
            self._check(self.lib.ses3d_gpu_get_seismograms(self.h, event, *[L.fptr(o) for o in out]))
        return tuple(np.ascontiguousarray(o.T) for o in out)

    def field(self, name: str, event: int = 0) -> np.ndarray:
        fid = L.FIELD_ID[name]
        n = self.G if name.endswith("_global") else (3 * self.N if name.startswith("M") and name != "MM_global" else self.N)
        out = np.zeros(n, np.float32)
        self._check(self.lib.ses3d_gpu_get_field(self.h, event, fid, L.fptr(out)))
        return out

    def set_field(self, name: str, values: np.ndarray, event: int = 0):
        a = np.ascontiguousarray(values, np.float32)
        self._check(self.lib.ses3d_gpu_set_field(self.h, event, L.FIELD_ID[name], L.fptr(a)))

    def kernel(self, name: str, event: int = 0) -> np.ndarray:
        out = np.zeros(self.N, np.float64)
        self._check(self.lib.ses3d_gpu_get_kernel(self.h, event, L.KERNEL_ID[name], L.dptr(out)))
        return out

    def kernel_sum(self, name: str) -> np.ndarray:
        """Sum of one kernel over all events (summed on the device in event order)."""
        out = np.zeros(self.N, np.float64)
        self._check(self.lib.ses3d_gpu_get_kernel_sum(self.h, L.KERNEL_ID[name], L.dptr(out)))
        return out

    def kernel_sum_device(self, name: str, out_ptr: int):
        """Event sum of one kernel written to device memory at out_ptr (N doubles)."""
        self._check(self.lib.ses3d_gpu_get_kernel_sum_device(self.h, L.KERNEL_ID[name], ctypes.c_void_p(out_ptr)))

    def add_kernel_sum_device(self, name: str, acc_ptr: int):
        """Event sum of one kernel added to the N doubles in device memory at acc_ptr."""
        self._check(self.lib.ses3d_gpu_add_kernel_sum_device(self.h, L.KERNEL_ID[name], ctypes.c_void_p(acc_ptr)))

    def record_count(self, event: int = 0) -> int:
        return self._check(self.lib.ses3d_gpu_record_count(self.h, event))

    def record(self, r: int, event: int = 0) -> np.ndarray:
        out = np.zeros(9 * self.N, np.float32)
        self._check(self.lib.ses3d_gpu_get_record(self.h, event, r, L.fptr(out)))
        return out.reshape(9, self.N)

    def put_record(self, r: int, data: np.ndarray, event: int = 0):
        a = np.ascontiguousarray(data, np.float32).reshape(-1)
        self._check(self.lib.ses3d_gpu_put_record(self.h, event, r, L.fptr(a)))

    def saving_vector(self) -> np.ndarray:
        out = np.zeros(self.nt, np.int32)
        self._check(self.lib.ses3d_gpu_get_saving_vector(self.h, L.iptr(out)))
        return out

    def set_saving_vector(self, sv):
        a = np.ascontiguousarray(sv, np.int32)
        self._check(self.lib.ses3d_gpu_set_saving_vector(self.h, L.iptr(a)))

    def setup_int(self, name: str, event: int = 0) -> np.ndarray:
        n = self._check(self.lib.ses3d_gpu_get_setup_int(self.h, event, name.encode(), None))
        out = np.zeros(max(n, 1), np.int32)
        self._check(self.lib.ses3d_gpu_get_setup_int(self.h, event, name.encode(), L.iptr(out)))
        return out[:n]

    def setup_real(self, name: str, event: int = 0) -> np.ndarray:
        n = self._check(self.lib.ses3d_gpu_get_setup_real(self.h, event, name.encode(), None))
        out = np.zeros(max(n, 1), np.float32)
        self._check(self.lib.ses3d_gpu_get_setup_real(self.h, event, name.encode(), L.fptr(out)))
        return out[:n]

    def vmax(self) -> np.ndarray:
        out = np.zeros(self.n_events, np.float32)
        self._check(self.lib.ses3d_gpu_vmax(self.h, L.fptr(out)))
        return out

    def profile(self, enable: bool = True):
        """Per-kernel CUDA-event timing of eager iterations (resets the totals when enabled)."""
        self._check(self.lib.ses3d_gpu_profile(self.h, int(enable)))

    def kernel_time(self, which: str):
        """(total ms, launches) of 'element', 'node', 'receivers' or 'inject' since profile(True)."""
        idx = {"element": 0, "node": 1, "receivers": 2, "inject": 3}[which]
        ms = ctypes.c_double(0)
        n = ctypes.c_int64(0)
        self._check(self.lib.ses3d_gpu_kernel_time(self.h, idx, ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    # -- exact discrete adjoint -------------------------------------------------------------------
    def exact_adjoint(self, steps_per_checkpoint: int, steps_per_subsegment: int = 0):
        """Plain forward run whose time step is reversed by exact_backward (see ses3d_gpu.h);
        call before stepping, lean stepping off."""
        self._check(self.lib.ses3d_gpu_exact_adjoint(self.h, int(steps_per_checkpoint), int(steps_per_subsegment)))

    def set_seismogram_adjoint(self, event: int, gx, gy, gz):
        """d misfit / d seismogram of one event, each (nr, nt) like seismograms()."""
        nr = self._nr[event]
        arrs = [np.ascontiguousarray(np.asarray(g, np.float32).reshape(nr, self.nt).T) for g in (gx, gy, gz)]
        self._check(self.lib.ses3d_gpu_exact_set_seismogram_adjoint(self.h, event, *[L.fptr(a) for a in arrs]))

    def exact_backward(self):
        self._check(self.lib.ses3d_gpu_exact_backward(self.h))

    def exact_gradient(self, name: str) -> np.ndarray:
        """Event-summed d misfit / d model record (rhoinv, mu, lambda, A, B, C, Q), FP64."""
        out = np.zeros(self.N, np.float64)
        self._check(self.lib.ses3d_gpu_exact_gradient(self.h, RECORD_NAMES.index(name), L.dptr(out), 0))
        return out

    def exact_gradient_device(self, name: str, out_ptr: int):
        """The same, written to N doubles of device memory at out_ptr."""
        self._check(self.lib.ses3d_gpu_exact_gradient(self.h, RECORD_NAMES.index(name), ctypes.c_void_p(out_ptr), 1))

    def exact_field(self, name: str, event: int = 0) -> np.ndarray:
        """A field of the exact adjoint's state (after exact_backward: the adjoint of the
        initial state)."""
        n = self.G if name.endswith("_global") else (3 * self.N if name.startswith("M") else self.N)
        out = np.zeros(n, np.float32)
        self._check(self.lib.ses3d_gpu_exact_get_field(self.h, event, L.FIELD_ID[name], L.fptr(out)))
        return out

    def set_exact_field(self, name: str, values: np.ndarray, event: int = 0):
        """Sets a field of the exact adjoint's state (before exact_backward: the adjoint of the
        final state)."""
        a = np.ascontiguousarray(values, np.float32)
        self._check(self.lib.ses3d_gpu_exact_set_field(self.h, event, L.FIELD_ID[name], L.fptr(a)))

    @property
    def launch_count(self) -> int:
        return int(self.lib.ses3d_gpu_launch_count(self.h))

    @property
    def stream(self) -> int:
        return int(self.lib.ses3d_gpu_stream(self.h) or 0)

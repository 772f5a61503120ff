"""Python binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle (ses3d_oracle.cpp) restates the reference Fortran solver statement by
statement in the reference layout; this module builds it, feeds it a synthetic
problem and reads its results. Only tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py use it, as the checker or as the timed CPU
baseline. Parity with the reference is unpinned by the reference's own tests
(the reference ships none and cannot be compiled here); the oracle is pinned by
the known-answer tests in tests/test_oracle.py.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "build", "libses3d_oracle.so")

NREAL = 23
(OR_DT, OR_XMIN, OR_XMAX, OR_YMIN, OR_YMAX, OR_ZMIN, OR_ZMAX, OR_ZMAX_GLOBAL, OR_XXS, OR_YYS, OR_ZZS,
 OR_MXX, OR_MYY, OR_MZZ, OR_MXY, OR_MXZ, OR_MYZ, OR_TAU1, OR_TAU2, OR_TAU3, OR_D1, OR_D2, OR_D3) = range(NREAL)

P_f = ctypes.POINTER(ctypes.c_float)
P_d = ctypes.POINTER(ctypes.c_double)
P_i = ctypes.POINTER(ctypes.c_int)


class OracleInput(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("lpd", ctypes.c_int),
                ("pml", ctypes.c_int), ("is_diss", ctypes.c_int), ("adjoint_flag", ctypes.c_int),
                ("samp_ad", ctypes.c_int), ("nt", ctypes.c_int), ("source_type", ctypes.c_int),
                ("grad_variant", ctypes.c_int), ("nr_global", ctypes.c_int), ("nr_adsrc_global", ctypes.c_int),
                ("rf", P_f), ("rd", P_d), ("so_f", P_f), ("so_d", P_d), ("rec_f", P_f), ("rec_d", P_d),
                ("adloc_f", P_f), ("adloc_d", P_d), ("adstf_f", P_f), ("adstf_d", P_d),
                ("rhoinv", P_f), ("mu", P_f), ("lambda_", P_f), ("A", P_f), ("B", P_f), ("C", P_f), ("Q", P_f),
                ("saving_vector", P_i)]


def build(verbose: bool = False) -> str:
    """Compiles the oracle (g++, -ffp-contract=off, OpenMP) into oracle/build/."""
    src = [os.path.join(HERE, f) for f in ("ses3d_oracle.cpp", "ses3d_oracle.h")]
    if os.path.exists(LIB) and all(os.path.getmtime(s) <= os.path.getmtime(LIB) for s in src):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-shared",
           "-o", LIB, src[0]]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB)
        lib.oracle_create.restype = ctypes.c_void_p
        lib.oracle_create.argtypes = [ctypes.POINTER(OracleInput), ctypes.c_int]
        lib.oracle_destroy.argtypes = [ctypes.c_void_p]
        lib.oracle_run.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.oracle_it.argtypes = [ctypes.c_void_p]
        lib.oracle_size.restype = ctypes.c_long
        lib.oracle_size.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        lib.oracle_get.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p]
        lib.oracle_set.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p]
        lib.oracle_get_int.restype = ctypes.c_long
        lib.oracle_get_int.argtypes = [ctypes.c_void_p, ctypes.c_char_p, P_i]
        lib.oracle_nrecords.argtypes = [ctypes.c_void_p]
        lib.oracle_get_record.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        lib.oracle_set_records.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        lib.oracle_strtof.restype = ctypes.c_float
        lib.oracle_strtof.argtypes = [ctypes.c_char_p]
        _lib = lib
    return _lib


def _shortest(v) -> str:
    """The decimal text the input files hold for an FP32 value (shortest round-trip form)."""
    f = np.float32(v)
    for p in range(1, 10):
        s = "%.*g" % (p, float(f))
        if np.float32(float(s)) == f and load().oracle_strtof(s.encode()) == f:
            return s
    return "%.9g" % float(f)


class Oracle:
    """The reference solver restated on the CPU, run on one event of a synth.Problem."""

    def __init__(self, problem, event: int = 0, fp64: bool = False, adjoint_flag: Optional[int] = None,
                 nt: Optional[int] = None, grad_variant: int = 0, saving_vector=None, ad_loc=None, ad_stf=None):
        lib = load()
        self.lib = lib
        self.fp64 = fp64
        self.dtype = np.float64 if fp64 else np.float32
        p = problem
        ev = p.events[event]
        e = ev.event
        self.nt = e.nt if nt is None else nt
        flag = p.setup.adjoint_flag if adjoint_flag is None else adjoint_flag
        vals = [e.dt, p.box.xmin, p.box.xmax, p.box.ymin, p.box.ymax, p.box.zmin, p.box.zmax, p.setup.zmax,
                e.xxs, e.yys, e.zzs, *e.mom, *p.tau, *p.D]
        txt = [_shortest(v) for v in vals]
        self._keep = []

        def keep(a):
            self._keep.append(a)
            return a

        rf = keep(np.array([lib.oracle_strtof(t.encode()) for t in txt], np.float32))
        rd = keep(np.array([float(t) for t in txt], np.float64))
        so_f = keep(np.ascontiguousarray(ev.stf[: self.nt], np.float32))
        so_d = keep(np.array([float(_shortest(v)) for v in so_f], np.float64))
        rec = ev.receivers.loc
        rec_f = keep(np.ascontiguousarray(rec, np.float32).reshape(-1))
        rec_d = keep(np.array([float(_shortest(v)) for v in rec_f], np.float64))
        inp = OracleInput()
        inp.nx, inp.ny, inp.nz = p.box.nx, p.box.ny, p.box.nz
        inp.lpd, inp.pml, inp.is_diss = 4, p.pml, p.setup.is_diss
        inp.adjoint_flag, inp.samp_ad, inp.nt, inp.source_type = flag, p.setup.samp_ad, self.nt, e.source_type
        inp.grad_variant = grad_variant
        inp.nr_global = len(rec)
        inp.rf, inp.rd = rf.ctypes.data_as(P_f), rd.ctypes.data_as(P_d)
        inp.so_f, inp.so_d = so_f.ctypes.data_as(P_f), so_d.ctypes.data_as(P_d)
        inp.rec_f, inp.rec_d = rec_f.ctypes.data_as(P_f), rec_d.ctypes.data_as(P_d)
        if ad_loc is not None:
            adl = keep(np.ascontiguousarray(ad_loc, np.float32).reshape(-1))
            adld = keep(np.array([float(_shortest(v)) for v in adl], np.float64))
            ads = keep(np.ascontiguousarray(np.asarray(ad_stf, np.float32)[:, :, : self.nt]).reshape(-1))
            adsd = keep(ads.astype(np.float64))
            inp.nr_adsrc_global = len(adl) // 3
            inp.adloc_f, inp.adloc_d = adl.ctypes.data_as(P_f), adld.ctypes.data_as(P_d)
            inp.adstf_f, inp.adstf_d = ads.ctypes.data_as(P_f), adsd.ctypes.data_as(P_d)
        m = {k: keep(np.ascontiguousarray(v, np.float32)) for k, v in p.model.items()}
        for nm, attr in (("rhoinv", "rhoinv"), ("mu", "mu"), ("lambda", "lambda_"), ("A", "A"), ("B", "B"),
                         ("C", "C"), ("Q", "Q")):
            if nm in m:
                setattr(inp, attr, m[nm].ctypes.data_as(P_f))
        if saving_vector is not None:
            sv = keep(np.ascontiguousarray(saving_vector, np.int32))
            inp.saving_vector = sv.ctypes.data_as(P_i)
        self.h = lib.oracle_create(ctypes.byref(inp), int(fp64))
        if not self.h:
            raise RuntimeError("oracle_create failed")
        self._keep = []

    def close(self):
        if getattr(self, "h", None):
            self.lib.oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, n: int):
        self.lib.oracle_run(self.h, int(n))

    @property
    def it(self) -> int:
        return self.lib.oracle_it(self.h)

    def get(self, name: str) -> np.ndarray:
        n = self.lib.oracle_size(self.h, name.encode())
        if n < 0:
            raise KeyError(name)
        out = np.zeros(n, self.dtype)
        self.lib.oracle_get(self.h, name.encode(), out.ctypes.data_as(ctypes.c_void_p))
        return out

    def set(self, name: str, values) -> None:
        """Overwrites a named real array (an initial state), converted to the handle's precision."""
        n = self.lib.oracle_size(self.h, name.encode())
        a = np.ascontiguousarray(np.asarray(values).reshape(-1), self.dtype)
        if n < 0 or a.size != n:
            raise KeyError("%s: %d values for an array of %d" % (name, a.size, n))
        if self.lib.oracle_set(self.h, name.encode(), a.ctypes.data_as(ctypes.c_void_p)) != 0:
            raise KeyError(name)

    def get_int(self, name: str) -> np.ndarray:
        n = self.lib.oracle_get_int(self.h, name.encode(), None)
        if n < 0:
            raise KeyError(name)
        out = np.zeros(n, np.int32)
        self.lib.oracle_get_int(self.h, name.encode(), out.ctypes.data_as(P_i))
        return out

    def seismograms(self):
        """(sx, sy, sz), each (nr, nt): the reference's seismogram_?(1:nr, 1:nt)."""
        nr = int(self.get_int("nr")[0])
        out = []
        for c in "xyz":
            a = self.get("seismogram_" + c).reshape(self.nt + 1, nr + 1)
            out.append(np.ascontiguousarray(a[1:, 1:].T))
        return tuple(out)

    def nrecords(self) -> int:
        return self.lib.oracle_nrecords(self.h)

    def record(self, r: int) -> np.ndarray:
        n = self.lib.oracle_size(self.h, b"vx")
        out = np.zeros(9 * n, self.dtype)
        self.lib.oracle_get_record(self.h, r, out.ctypes.data_as(ctypes.c_void_p))
        return out.reshape(9, n)

    def set_records(self, recs: np.ndarray):
        a = np.ascontiguousarray(recs, self.dtype)
        self.lib.oracle_set_records(self.h, a.shape[0], a.ctypes.data_as(ctypes.c_void_p))

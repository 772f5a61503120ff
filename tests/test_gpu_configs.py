"""Parity against the oracle at the benchmark workload sizes themselves.

The GPU path and the oracle (FP32 and FP64) start from the same seeded random state:
velocity at every global node, the nine PML stresses, the nine displacement gradients and
the memory variables at every GLL point (random_state below). A point source at rest would leave most of a
large mesh at zero for the few tens of steps the oracle can afford there; a random state
makes every node and every element carry a value from the first step on, so the
comparison covers the index arithmetic of the whole mesh: the PML bands, the far ends of
the arrays (32-bit offsets), the node gather's division by GX, the last elements of each
axis. Mirror stresses start equal to their partners (as in a run that starts at rest), so
lean stepping applies.

Tolerances are the ones stated for the path: seismograms rel-L2 <= 1e-5 against the FP32
oracle and <= 1e-4 against FP64; fields <= 1e-4 against FP64; Frechet kernels <= 1e-3
against FP64; set-up integers and the mass matrix bit-exact. Measured errors are printed.
"""
import numpy as np
import pytest
from wavefields import GRADS, MEMVARS, MIRROR, STRESS, VELOCITY, random_state

from ses3d_gb300 import synth

pytestmark = pytest.mark.gpu

SEIS_TOL_FP32 = 1e-5
SEIS_TOL_FP64 = 1e-4
FIELD_TOL_FP64 = 1e-4
KERNEL_TOL_FP64 = 1e-3

def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def load_gpu(sim, st, event=0):
    for k, a in st.items():
        sim.set_field(k, a, event)


def load_oracle(o, st):
    for k, a in st.items():
        o.set(k, a)


def compare_fields(tag, gpu_field, o64, names, o32=None):
    """Fields of one run against the FP64 oracle (asserted) and the FP32 oracle (printed)."""
    worst = 0.0
    for k in names:
        g = gpu_field(k)
        r64 = rel(g, o64.get(k))
        worst = max(worst, r64)
        msg = "%s %s vs FP64 %.2e" % (tag, k, r64)
        if o32 is not None:
            msg += " vs FP32 %.2e" % rel(g, o32.get(k))
        print(msg)
        assert r64 <= FIELD_TOL_FP64, msg
    return worst


@pytest.fixture(scope="module")
def c2():
    return synth.make_problem("c2", nt=20, seed=1234)


@pytest.fixture(scope="module")
def c2_gpu(native, c2):
    """96 x 96 x 40 from the random state: full-state (eager) and lean (CUDA graph) runs."""
    from ses3d_gb300.solver import Simulation
    st = random_state(c2, 77)
    out = {}
    for lean in (False, True):
        with Simulation.from_problem(c2) as sim:
            load_gpu(sim, st)
            sim.set_lean(lean)
            if lean:
                sim.use_graph(True, 10)
            sim.run()
            names = VELOCITY + STRESS + tuple(MIRROR) + MEMVARS + (() if lean else GRADS)
            out[lean] = ({k: sim.field(k) for k in names}, sim.seismograms(0))
    return st, out


def test_c2_setup_bit_exact(native, oracle_mod, c2):
    """96 x 96 x 40: element-node coordinates, receiver and source location, PML profiles,
    taper and the assembled mass matrix bit for bit (the index work of ses3d_init)."""
    from ses3d_gb300.solver import Simulation
    with Simulation.from_problem(c2) as sim:
        o = oracle_mod.Oracle(c2)
        for name in ("x", "y", "z", "Jac", "xxs_loc", "yys_loc", "zzs_loc", "prof_x", "prof_y", "prof_z",
                     "taper"):
            assert np.array_equal(sim.setup_real(name), o.get(name)), name
        nr = int(o.get_int("nr")[0])
        assert nr == sim.n_receivers(0) == 200
        for name in ("rx", "ry", "rz"):
            assert np.array_equal(sim.setup_int(name), o.get_int(name)[1:nr + 1]), name
        assert np.array_equal(sim.setup_real("recloc_std"), o.get("recloc_std")[: 3 * nr])
        for name in ("isx", "isy", "isz", "is_source"):
            assert int(sim.setup_int(name)[0]) == int(o.get_int(name)[0]), name
        assert np.array_equal(sim.field("MM_global"), o.get("MM_global"))
        o.close()


@pytest.mark.parametrize("fp64", [False, True])
def test_c2_random_state_matches_oracle(oracle_mod, c2, c2_gpu, fp64):
    """96 x 96 x 40, 20 steps from the random state: seismograms of all 200 receivers and
    every field, full-state and lean stepping, against the oracle."""
    st, out = c2_gpu
    o = oracle_mod.Oracle(c2, fp64=fp64)
    load_oracle(o, st)
    o.run(20)
    r = o.seismograms()
    tol = SEIS_TOL_FP64 if fp64 else SEIS_TOL_FP32
    for lean in (False, True):
        fields, seis = out[lean]
        tag = "c2 %s %s" % ("lean" if lean else "full", "fp64" if fp64 else "fp32")
        for c in range(3):
            e = rel(seis[c], r[c])
            print("%s seismogram %s %.2e" % (tag, "xyz"[c], e))
            assert np.abs(r[c]).max() > 0
            assert e <= tol, (tag, c, e)
        if fp64:
            compare_fields(tag, fields.__getitem__, o, tuple(fields))
        else:
            for k in fields:
                print("%s %s vs FP32 %.2e" % (tag, k, rel(fields[k], o.get(k))))
    o.close()


def test_c4_batch_events_match_oracle(native, oracle_mod):
    """48 x 48 x 24 with 16 events in one handle (lean, CUDA graph): events 0 and 15 start
    from their own random states (the others at rest) and are checked against single-event
    oracle runs over 20 steps, seismograms and fields."""
    from ses3d_gb300.solver import Simulation
    steps = 20
    p = synth.make_problem("c4", nt=steps, seed=1234)
    states = {k: random_state(p, 100 + k) for k in (0, 15)}
    gpu = {}
    with Simulation.from_problem(p) as sim:
        for k, st in states.items():
            load_gpu(sim, st, k)
        sim.set_lean(True)
        sim.use_graph(True, 10)
        sim.run()
        for k in states:
            gpu[k] = ({f: sim.field(f, k) for f in VELOCITY + STRESS + MEMVARS}, sim.seismograms(k))
    for k, st in states.items():
        for fp64 in (False, True):
            o = oracle_mod.Oracle(p, event=k, fp64=fp64)
            load_oracle(o, st)
            o.run(steps)
            r = o.seismograms()
            fields, seis = gpu[k]
            tag = "c4 event %d %s" % (k, "fp64" if fp64 else "fp32")
            tol = SEIS_TOL_FP64 if fp64 else SEIS_TOL_FP32
            assert seis[0].shape == r[0].shape and seis[0].shape[0] > 0
            for c in range(3):
                e = rel(seis[c], r[c])
                print("%s seismogram %s %.2e" % (tag, "xyz"[c], e))
                assert e <= tol, (tag, c, e)
            if fp64:
                compare_fields(tag, fields.__getitem__, o, tuple(fields))
            o.close()


@pytest.mark.parametrize("lean", [False, True])
def test_c3_adjoint_kernels_match_oracle(native, oracle_mod, lean):
    """64 x 64 x 32: forward run with records (samp_ad 10, 30 steps) and adjoint run with the
    ses3d_grad_Q kernels (30 steps), each from its own random state, with adjoint sources
    at five receivers; records and all kernels against the oracle. Lean runs (displacement
    gradients outside the PML from the displacement) start with zero displacement
    gradients, the condition they need; full-state runs with random ones."""
    from ses3d_gb300.solver import Simulation
    nt, samp = 30, 10
    p = synth.make_problem("c3", nt=nt, seed=1234, adjoint_flag=1)
    p.setup.samp_ad = samp
    fwd = random_state(p, 5)
    adj = random_state(p, 6)
    if lean:
        fwd = {k: a for k, a in fwd.items() if k not in GRADS}
        adj = {k: a for k, a in adj.items() if k not in GRADS}
    loc = p.events[0].receivers.loc[:5].copy()
    loc[:, 2] = np.float32(1000.0)
    stf = np.random.default_rng(7).standard_normal((5, 3, nt)).astype(np.float32) * np.float32(1e9)
    names = ("rho", "cp", "csh", "csv", "Q_mu", "alpha_mu", "Q_kappa")
    with Simulation.from_problem(p, adjoint_flag=1, grad_variant=1) as sim:
        load_gpu(sim, fwd)
        sim.set_lean(lean)
        sim.run()
        g_records = [sim.record(r) for r in range(sim.record_count())]
        g_sv = sim.saving_vector()
        assert sim.set_adjoint_sources(0, loc, stf) == 5
        sim.begin_adjoint()
        load_gpu(sim, adj)
        sim.set_lean(lean)
        sim.run()
        g_kernels = {k: sim.kernel(k) for k in names}
        g_v = sim.field("vz_global")
    for fp64 in (False, True):
        o = oracle_mod.Oracle(p, fp64=fp64, adjoint_flag=1)
        load_oracle(o, fwd)
        o.run(nt)
        recs = np.stack([o.record(r) for r in range(o.nrecords())])
        sv = o.get_int("saving_vector")[1:nt + 1]
        o.close()
        assert np.array_equal(sv, g_sv)
        assert len(recs) == len(g_records) == 4
        tag = "c3%s %s" % (" lean" if lean else "", "fp64" if fp64 else "fp32")
        if fp64:
            for r in range(len(recs)):
                for f in range(9):
                    e = rel(g_records[r][f], recs[r][f])
                    print("%s record %d field %d %.2e" % (tag, r, f, e))
                    assert e <= FIELD_TOL_FP64, (r, f, e)
        oa = oracle_mod.Oracle(p, fp64=fp64, adjoint_flag=2, saving_vector=sv, ad_loc=loc, ad_stf=stf,
                               grad_variant=1)
        oa.set_records(recs)
        del recs
        load_oracle(oa, adj)
        oa.run(nt)
        print("%s adjoint vz_global %.2e" % (tag, rel(g_v, oa.get("vz_global"))))
        for k in names:
            ok = oa.get("grad_" + k)
            e = rel(g_kernels[k], ok)
            print("%s kernel %s %.2e" % (tag, k, e))
            assert np.abs(ok).max() > 0, k
            if fp64:
                assert e <= KERNEL_TOL_FP64, (k, e)
        oa.close()

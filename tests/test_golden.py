"""The committed golden fixture (tests/golden/oracle_tiny.npz, FP64 oracle outputs written by
tests/golden/make_golden.py) replays: the FP64 oracle reproduces it to rounding, and the FP32
oracle stays within the FP32-vs-FP64 tolerance of the forward tests (1e-4)."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden as G  # noqa: E402


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def golden():
    return dict(np.load(os.path.join(HERE, "golden", "oracle_tiny.npz")))


@pytest.mark.parametrize("fp64,tol", [(True, 1e-10), (False, 1e-4)])
def test_forward_replays(oracle_mod, golden, fp64, tol):
    p = G.problem_from(golden, "fwd_")
    o = oracle_mod.Oracle(p, fp64=fp64, adjoint_flag=0)
    o.run(G.NT)
    seis = np.stack(o.seismograms())
    assert seis.shape == golden["fwd_seismograms"].shape
    for c in range(3):
        assert rel(seis[c], golden["fwd_seismograms"][c]) <= tol, c
    assert rel(o.get("vz_global"), golden["fwd_vz_global"]) <= max(tol, 1e-7)


@pytest.mark.parametrize("fp64,tol", [(True, 1e-10), (False, 1e-3)])
def test_adjoint_kernels_replay(oracle_mod, golden, fp64, tol):
    p = G.problem_from(golden, "adj_")
    o = oracle_mod.Oracle(p, fp64=fp64, adjoint_flag=1)
    o.run(G.NT)
    recs = np.stack([o.record(r) for r in range(o.nrecords())])
    sv = o.get_int("saving_vector")[1:G.NT + 1]
    oa = oracle_mod.Oracle(p, fp64=fp64, adjoint_flag=2, saving_vector=sv, ad_loc=golden["adj_adsrc_loc"],
                           ad_stf=golden["adj_adsrc_stf"])
    oa.set_records(recs)
    oa.run(G.NT)
    for k in ("rho", "cp", "csh", "csv"):
        full = oa.get("grad_" + k)
        assert np.abs(golden["adj_grad_" + k]).max() > 0, k
        assert rel(full[::G.STRIDE], golden["adj_grad_" + k]) <= tol, k
        assert abs(np.linalg.norm(full) / golden["adj_norm_" + k] - 1) <= tol, k

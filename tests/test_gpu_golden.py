"""The CUDA path against the committed golden fixture (FP64 oracle outputs,
tests/golden/oracle_tiny.npz): seismograms and velocity within 1e-4, Frechet kernels
within 1e-3 (rel-L2), the tolerances of the forward and adjoint parity tests."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden as G  # noqa: E402

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def golden():
    return dict(np.load(os.path.join(HERE, "golden", "oracle_tiny.npz")))


@pytest.mark.parametrize("lean", [False, True])
def test_forward_matches_golden(native, golden, lean):
    from ses3d_gb300.solver import Simulation
    p = G.problem_from(golden, "fwd_")
    with Simulation.from_problem(p, adjoint_flag=0) as sim:
        sim.set_lean(lean)
        sim.run()
        seis = np.stack(sim.seismograms(0))
        vz = sim.field("vz_global")
    for c in range(3):
        assert rel(seis[c], golden["fwd_seismograms"][c]) <= 1e-4, c
    assert rel(vz, golden["fwd_vz_global"]) <= 1e-4


def test_adjoint_kernels_match_golden(native, golden):
    from ses3d_gb300.solver import Simulation
    p = G.problem_from(golden, "adj_")
    with Simulation.from_problem(p, adjoint_flag=1) as sim:
        sim.run()
        sim.set_adjoint_sources(0, golden["adj_adsrc_loc"], golden["adj_adsrc_stf"])
        sim.begin_adjoint()
        sim.run()
        for k in ("rho", "cp", "csh", "csv"):
            full = sim.kernel(k)
            assert rel(full[::G.STRIDE], golden["adj_grad_" + k]) <= 1e-3, k
            assert abs(np.linalg.norm(full) / golden["adj_norm_" + k] - 1) <= 1e-3, k

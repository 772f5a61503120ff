"""Parity at the full workload sizes through properties that do not depend on size (the
oracle is too slow there): equivalent paths give identical bits. Each run is a few tens of
time steps."""
import numpy as np
import pytest

from ses3d_gb300 import synth

pytestmark = pytest.mark.gpu


def run(p, steps, lean=False, epb=1, graph=0):
    from ses3d_gb300.solver import Simulation
    with Simulation.from_problem(p) as sim:
        sim.set_lean(lean)
        sim.set_block_elements(epb)
        if graph:
            sim.use_graph(True, graph)
        sim.step(steps)
        return ([sim.field(k, e) for e in range(sim.n_events) for k in ("vx_global", "vz_global")],
                [np.concatenate(sim.seismograms(e)) for e in range(sim.n_events)], sim.vmax())


def same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


@pytest.fixture(scope="module")
def c2():
    return synth.make_problem("c2", nt=60, seed=1234)


def test_c2_lean_equals_full_state(native, c2):
    """96 x 96 x 40: lean stepping (graph) and full-state stepping give the same bits."""
    full = run(c2, 40)
    lean = run(c2, 40, lean=True, graph=10)
    assert np.abs(full[1][0]).max() > 0 and np.all(np.isfinite(full[2]))
    assert same(full[0], lean[0]) and same(full[1], lean[1])


def test_c2_persistent_equals_register_staged(native, c2):
    """96 x 96 x 40: the persistent bulk-copy element kernel and the register-staged kernel
    (2 elements per CTA) give the same bits."""
    a = run(c2, 20, epb=1)
    b = run(c2, 20, epb=2)
    assert same(a[0], b[0]) and same(a[1], b[1])


def test_c4_sixteen_batched_events_equal_single_runs(native):
    """48 x 48 x 24 with 16 events (uneven receiver counts): events 0 and 15 of the batch
    equal their single-event runs."""
    p = synth.make_problem("c4", nt=30, seed=1234)
    batch = run(p, 20, lean=True, graph=10)
    for k in (0, 15):
        q = synth.Problem(p.setup, p.box, p.tau, p.D, p.model, [p.events[k]], pml=p.pml)
        one = run(q, 20, lean=True, graph=10)
        assert same(batch[0][2 * k:2 * k + 2], one[0]) and np.array_equal(batch[1][k], one[1][0])


def test_c3_checkpointed_kernels_equal_stored(native):
    """64 x 64 x 32: Frechet kernels from forward records kept in HBM and from full-state
    checkpoints every 4 records with segment recompute are the same bits."""
    from ses3d_gb300 import _lib
    from ses3d_gb300.solver import Simulation
    nt = 60
    p = synth.make_problem("c3", nt=nt, seed=1234, adjoint_flag=1)
    p.setup.samp_ad = 5
    loc = p.events[0].receivers.loc[:3].copy()
    loc[:, 2] = np.float32(1000.0)
    stf = np.random.default_rng(2).standard_normal((3, 3, nt)).astype(np.float32) * np.float32(1e8)
    kernels = []
    for K in (0, 4):
        with Simulation.from_problem(p, adjoint_flag=1) as sim:
            if K:
                _lib.check(sim.lib.ses3d_gpu_set_checkpointing(sim.h, K), sim.h)
            sim.run()
            sim.set_adjoint_sources(0, loc, stf)
            sim.begin_adjoint()
            sim.run()
            kernels.append({k: sim.kernel(k) for k in ("rho", "cp", "csh", "csv")})
    for k in kernels[0]:
        assert np.abs(kernels[0][k]).max() > 0
        assert np.array_equal(kernels[0][k], kernels[1][k]), k

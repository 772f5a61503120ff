"""Run-time block shapes of the element and node kernels (ses3d_gpu_set_kernel_shape) and the
autotuner that searches them: every shape gives the same bits, lean and full state, and
the autotuner keeps one of the timed candidates."""
import numpy as np
import pytest

from ses3d_gb300 import synth

pytestmark = pytest.mark.gpu


def run(p, steps, lean, shape, node_block, graph=10):
    from ses3d_gb300.solver import Simulation
    with Simulation.from_problem(p) as sim:
        sim.set_lean(lean)
        sim.set_kernel_shape(shape, node_block)
        if graph:
            sim.use_graph(True, graph)
        sim.step(steps)
        return [sim.field("vx_global"), sim.field("vz_global"), sim.field("sxz_pml"),
                np.concatenate(sim.seismograms(0))]


@pytest.mark.parametrize("lean", [False, True])
@pytest.mark.parametrize("n_el", [None, (20, 20, 10)])
def test_all_shapes_bit_identical(native, lean, n_el):
    """Every element shape and node block size gives the same bits, on the 10 x 9 x 6 mesh
    (at most one element per CTA of the persistent kernel) and on 20 x 20 x 10 (several, so
    that every shape's copy pipeline runs ahead of its compute)."""
    from ses3d_gb300 import _lib
    p = synth.make_problem("small", nt=30, seed=81, n_el=n_el)
    ref = run(p, 30, lean, 0, 256)
    assert np.abs(ref[0]).max() > 0
    n = int(_lib.load().ses3d_gpu_kernel_shape_count())
    assert n >= 2
    for shape in range(n):
        for nb in (128, 256, 512):
            out = run(p, 30, lean, shape, nb)
            for a, b in zip(ref, out):
                assert np.array_equal(a, b), (shape, nb)


def test_shape_arguments_checked(native):
    from ses3d_gb300.solver import Simulation
    p = synth.make_problem("tiny", nt=4, seed=82)
    with Simulation.from_problem(p) as sim:
        assert sim.lib.ses3d_gpu_set_kernel_shape(sim.h, -1, 256) == -1
        assert sim.lib.ses3d_gpu_set_kernel_shape(sim.h, 0, 300) == -1
        assert sim.lib.ses3d_gpu_set_kernel_shape(sim.h, 99, 256) == -1


def test_autotune_keeps_a_timed_candidate(native):
    from ses3d_gb300.solver import Simulation
    p = synth.make_problem("small", nt=60, seed=83)
    with Simulation.from_problem(p) as sim:
        tuned = sim.autotune(steps_each=2)
        chosen = tuned["chosen"]
        assert tuned["element"] and tuned["node"]
        best = min(tuned["element"], key=tuned["element"].get)
        assert "epb=%d" % chosen["elements_per_cta"] in best
        assert chosen["node_block"] == min(tuned["node"], key=tuned["node"].get)
        assert sim.shape == chosen
        it = sim.it
        sim.run()                                   # the run continues with the chosen shape
        assert sim.it == 60 and it < 60


def adjoint_run(p, epb, nt):
    """Forward with records (adjoint_flag 1), then the adjoint with the kernel correlation,
    with the element kernel chosen by epb (1: persistent bulk-copy kernel, 2: register-staged)."""
    from ses3d_gb300.solver import Simulation
    sim = Simulation.from_problem(p, adjoint_flag=1, grad_variant=1)
    try:
        sim.set_block_elements(epb)
        sim.run()
        records = [sim.record(r) for r in range(sim.record_count())]
        seis = sim.seismograms(0)
        loc = p.events[0].receivers.loc[:2].copy()
        stf = np.zeros((2, 3, nt), np.float32)
        for k in range(2):
            for c in range(3):
                stf[k, c] = seis[c][k][::-1]
        stf *= np.float32(1e10) / np.abs(stf).max()
        sim.set_adjoint_sources(0, loc, stf)
        sim.begin_adjoint()
        sim.run()
        names = ("rho", "cp", "csh", "csv") + (("Q_mu", "alpha_mu", "Q_kappa") if p.setup.is_diss else ())
        kernels = [sim.kernel(k) for k in names]
        return records, kernels
    finally:
        sim.close()


@pytest.mark.parametrize("is_diss", [1, 0])
def test_record_and_correlation_kernels_bit_identical(native, is_diss):
    """Record (forward store) and kernel-correlation iterations give the same records and
    Frechet kernels on the persistent element kernel as on the register-staged one."""
    nt = 40
    p = synth.make_problem("small", nt=nt, seed=84, adjoint_flag=1, is_diss=is_diss)
    p.setup.samp_ad = 4
    rec1, ker1 = adjoint_run(p, 1, nt)
    rec2, ker2 = adjoint_run(p, 2, nt)
    assert len(rec1) == len(rec2) == 1 + nt // 4   # iteration 1 and every samp_ad-th
    assert np.abs(rec1[-1]).max() > 0      # the first record (iteration 1) is still zero
    for a, b in zip(rec1, rec2):
        assert np.array_equal(a, b)
    assert len(ker1) == len(ker2) == (7 if is_diss else 4)
    for k, (a, b) in enumerate(zip(ker1, ker2)):
        assert np.abs(a).max() > 0 and np.array_equal(a, b), k


def random_velocities(sim, nev, rng):
    for ev in range(nev):
        for k in ("vx_global", "vy_global", "vz_global"):
            n = sim.field(k, ev).size
            sim.set_field(k, (1e-3 * rng.standard_normal(n)).astype(np.float32), ev)


def correlation_run(p, epb, nt, lean, seed):
    """Forward with records from random initial velocities, then the adjoint run from random
    velocities with random adjoint sources at two receivers of every event, so that every
    element holds forward and adjoint fields and every correlation item contributes."""
    from ses3d_gb300.solver import Simulation
    rng = np.random.default_rng(seed)
    nev = len(p.events)
    names = ("rho", "cp", "csh", "csv", "Q_mu", "alpha_mu", "Q_kappa")
    sim = Simulation.from_problem(p, adjoint_flag=1, grad_variant=1)
    try:
        sim.set_block_elements(epb)
        sim.set_lean(lean)
        random_velocities(sim, nev, rng)
        sim.run()
        records = [sim.record(r, ev) for ev in range(nev) for r in range(sim.record_count())]
        for ev in range(nev):
            stf = (1e10 * rng.standard_normal((2, 3, nt))).astype(np.float32)
            sim.set_adjoint_sources(ev, p.events[ev].receivers.loc[:2].copy(), stf)
        sim.begin_adjoint()
        random_velocities(sim, nev, rng)
        sim.run()
        return records, [sim.kernel(k, ev) for ev in range(nev) for k in names]
    finally:
        sim.close()


@pytest.mark.parametrize("n_events", [1, 2])
def test_correlation_with_several_items_per_cta(native, n_events):
    """On a 20 x 20 x 10 mesh (4,000 elements per event) each CTA of the persistent element
    kernel steps several items, staging the next item's record, adjoint model and FP64
    kernels while it works on the current one. Records and kernels equal the register-staged
    kernel's bit for bit; lean runs (displacement gradients from the displacement outside the
    PML) follow within FP32 rounding."""
    nt = 40
    p = synth.make_problem("small", nt=nt, seed=89, adjoint_flag=1, n_el=(20, 20, 10), n_events=n_events)
    p.setup.samp_ad = 4
    rec_r, ker_r = correlation_run(p, 2, nt, False, 5)
    rec_p, ker_p = correlation_run(p, 1, nt, False, 5)
    rec_l, ker_l = correlation_run(p, 1, nt, True, 5)
    assert len(rec_r) == n_events * (1 + nt // 4)
    for a, b in zip(rec_r, rec_p):
        assert np.array_equal(a, b)
    for k, (a, b) in enumerate(zip(ker_r, ker_p)):
        assert np.abs(a).max() > 0 and np.array_equal(a, b), k
    rel = lambda a, b: float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))
    for r, (a, b) in enumerate(zip(rec_l, rec_r)):
        if np.abs(b).max() > 0:
            assert rel(a, b) <= 1e-4, (r, rel(a, b))
    for k, (a, b) in enumerate(zip(ker_l, ker_r)):
        assert rel(a, b) <= 1e-3, (k, rel(a, b))


def test_isotropy_follows_the_model_and_drops_the_graph(native):
    """The model's A, B, C decide whether the element kernels read three or six material
    fields: an isotropic model reports 1, a model with non-zero A, B, C set later in the run
    reports 0, and a CUDA graph captured before the change is not replayed with the old
    setting: graph and eager stepping agree bit for bit across the switch."""
    from ses3d_gb300.solver import Simulation
    p = synth.make_problem("small", nt=24, seed=85)
    m = dict(p.model)
    rng = np.random.default_rng(5)
    mu = np.asarray(p.model["mu"], np.float64)
    for k, s in (("A", 0.02), ("B", 0.03), ("C", -0.02)):
        m[k] = (s * mu * rng.uniform(0.5, 1.0, mu.size)).astype(np.float32)
    out = []
    for graph in (True, False):
        with Simulation.from_problem(p) as sim:
            assert sim.setup_int("isotropic")[0] == 1
            if graph:
                sim.use_graph(True, 4)
            sim.step(12)
            sim.set_model(m)
            assert sim.setup_int("isotropic")[0] == 0
            sim.step(12)
            out.append([sim.field("vx_global"), sim.field("sxz_pml"), np.concatenate(sim.seismograms(0))])
    for a, b in zip(*out):
        assert np.abs(a).max() > 0 and np.array_equal(a, b)

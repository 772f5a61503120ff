"""GPU parity of the adjoint path: forward-field records (adjoint_flag 1) and Frechet
kernels (adjoint_flag 2, SOURCE/ses3d_grad.f90 and SOURCE/ses3d_grad_Q.f90) against the
CPU oracle. Kernel tolerance: rel-L2 <= 1e-3 against the FP64 oracle."""
import numpy as np
import pytest

from ses3d_gb300 import synth

pytestmark = pytest.mark.gpu

NT = 60
SAMP = 5


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def adjoint_inputs(p, seis):
    """Two adjoint sources at the first two receivers, driven by the time-reversed forward
    velocity (the shape TOOLS/adjoint_source.py writes for a waveform misfit)."""
    loc = p.events[0].receivers.loc[:2].copy()
    loc[:, 2] = np.float32(1000.0)  # 1 km depth, as in ADJOINT/1/ad_srcfile of the reference
    stf = np.zeros((2, 3, NT), np.float32)
    for k in range(2):
        for c in range(3):
            stf[k, c] = seis[c][k][::-1]
    stf *= np.float32(1e10) / np.abs(stf).max()
    return loc, stf


@pytest.fixture(scope="module")
def problem():
    p = synth.make_problem("small", nt=NT, seed=31, adjoint_flag=1)
    p.setup.samp_ad = SAMP
    return p


@pytest.fixture(scope="module")
def runs(native, oracle_mod, problem):
    from ses3d_gb300.solver import Simulation
    p = problem
    out = {}
    sim = Simulation.from_problem(p, adjoint_flag=1, grad_variant=1)
    sim.run()
    out["gpu_records"] = [sim.record(r) for r in range(sim.record_count())]
    out["gpu_sv"] = sim.saving_vector()
    gseis = sim.seismograms(0)
    loc, stf = adjoint_inputs(p, gseis)
    out["nad"] = sim.set_adjoint_sources(0, loc, stf)
    sim.begin_adjoint()
    sim.run()
    out["gpu_kernels"] = {k: sim.kernel(k) for k in ("rho", "cp", "csh", "csv", "Q_mu", "alpha_mu", "Q_kappa")}
    out["gpu_is"] = sim.setup_int("is")
    sim.close()
    # the same runs stepped lean: records and correlations outside the PML take the
    # displacement gradients from the displacement
    lean = Simulation.from_problem(p, adjoint_flag=1, grad_variant=1)
    lean.set_lean(True)
    lean.run()
    out["lean_records"] = [lean.record(r) for r in range(lean.record_count())]
    out["lean_seis"] = lean.seismograms(0)
    lean.set_adjoint_sources(0, loc, stf)
    lean.begin_adjoint()
    lean.set_lean(True)
    lean.run()
    out["lean_kernels"] = {k: lean.kernel(k) for k in ("rho", "cp", "csh", "csv", "Q_mu", "alpha_mu", "Q_kappa")}
    lean.close()
    out["gpu_seis"] = gseis
    for fp64 in (False, True):
        o = oracle_mod.Oracle(p, fp64=fp64, adjoint_flag=1)
        o.run(NT)
        recs = np.stack([o.record(r) for r in range(o.nrecords())])
        sv = o.get_int("saving_vector")[1:NT + 1]
        oa = oracle_mod.Oracle(p, fp64=fp64, adjoint_flag=2, saving_vector=sv, ad_loc=loc, ad_stf=stf,
                               grad_variant=1)
        oa.set_records(recs)
        oa.run(NT)
        tag = "64" if fp64 else "32"
        out["o_records" + tag] = recs
        out["o_sv" + tag] = sv
        out["o_kernels" + tag] = {k: oa.get("grad_" + k) for k in ("rho", "cp", "csh", "csv", "Q_mu",
                                                                   "alpha_mu", "Q_kappa")}
        out["o_is" + tag] = oa.get_int("is")
        out["o_nad" + tag] = int(oa.get_int("nr_adsrc")[0])
    return out


@pytest.mark.parametrize("lean", [False, True])
@pytest.mark.parametrize("K,K2", [(1, 0), (3, 0), (100, 0), (5, 2), (12, 5), (4, 3)])
def test_checkpointed_records_give_identical_kernels(native, problem, runs, K, K2, lean):
    """Checkpoints every K records + segment recompute (K2 = 0), or two levels (segments of
    K records recomputed into checkpoints every K2 records, sub-segments recomputed from
    those) = keeping every record, bit for bit."""
    from ses3d_gb300 import _lib
    from ses3d_gb300.solver import Simulation
    p = problem
    sim = Simulation.from_problem(p, adjoint_flag=1, grad_variant=1)
    _lib.check(sim.lib.ses3d_gpu_set_checkpoint_levels(sim.h, K, K2), sim.h)
    sim.set_lean(lean)
    sim.run()
    assert sim.record_count() == len(runs["gpu_records"])
    assert np.array_equal(sim.saving_vector(), runs["gpu_sv"])
    gseis = sim.seismograms(0)
    loc, stf = adjoint_inputs(p, gseis)
    sim.set_adjoint_sources(0, loc, stf)
    sim.begin_adjoint()
    sim.set_lean(lean)
    sim.run()
    ref = runs["lean_kernels" if lean else "gpu_kernels"]
    for k in ("rho", "cp", "csh", "csv", "Q_mu"):
        assert np.array_equal(sim.kernel(k), ref[k]), k
    sim.close()


def test_checkpoint_levels_rejects_bad_lengths(native, problem):
    from ses3d_gb300.solver import Simulation
    with Simulation.from_problem(problem, adjoint_flag=1) as sim:
        for K, K2 in ((4, 4), (0, 2), (-1, 0), (3, -2)):
            assert sim.lib.ses3d_gpu_set_checkpoint_levels(sim.h, K, K2) == -1
        assert sim.lib.ses3d_gpu_set_checkpoint_levels(sim.h, 4, 2) == 0


def test_lean_records_and_kernels_follow_full_state(runs):
    """Lean runs with records: the same seismograms bit for bit, records and kernels equal
    to the full-state run's within FP32 rounding (outside the PML the displacement gradients
    are the strain-rate proxies of the displacement, summed in another order)."""
    for a, b in zip(runs["lean_seis"], runs["gpu_seis"]):
        assert np.abs(b).max() > 0 and np.array_equal(a, b)
    for r, (a, b) in enumerate(zip(runs["lean_records"], runs["gpu_records"])):
        for f in range(9):
            if np.abs(b[f]).max() == 0:
                continue
            assert rel(a[f], b[f]) <= 2e-5, (r, f, rel(a[f], b[f]))
    for k, b in runs["gpu_kernels"].items():
        assert rel(runs["lean_kernels"][k], b) <= 1e-4, (k, rel(runs["lean_kernels"][k], b))


def test_lean_choice_is_fixed_once_a_run_with_records_starts(native, problem):
    from ses3d_gb300 import _lib
    from ses3d_gb300.solver import Simulation
    with Simulation.from_problem(problem, adjoint_flag=1) as sim:
        sim.set_lean(True)
        sim.step(3)
        assert sim.lib.ses3d_gpu_set_lean(sim.h, 0) == -4
        assert sim.lib.ses3d_gpu_set_lean(sim.h, 1) == 0
        with pytest.raises(_lib.Ses3dError):
            sim.field("dxux")
        sim.run()
        sim.begin_adjoint()
        assert sim.lib.ses3d_gpu_set_lean(sim.h, 0) == 0   # a new run: free to choose again
    with Simulation.from_problem(problem, adjoint_flag=1) as sim:
        # lean records add the gradients of the displacement since the start: a run whose
        # displacement gradients were set is refused
        sim.set_field("dxux", np.zeros(sim.N, np.float32))
        sim.set_lean(True)
        with pytest.raises(_lib.Ses3dError) as err:
            sim.step(1)
        assert err.value.code == -4 and sim.it == 0
        sim.set_lean(False)
        sim.step(1)
        assert sim.it == 1


def test_saving_vector(runs):
    assert np.array_equal(runs["gpu_sv"], runs["o_sv32"])
    expected = [it if (it % SAMP == 0 or it == 1 or it == NT) else 0 for it in range(1, NT + 1)]
    assert list(runs["gpu_sv"]) == expected


@pytest.mark.parametrize("which", ["gpu_records", "lean_records"])
def test_records(runs, which):
    g, o = runs[which], runs["o_records64"]
    assert len(g) == len(o)
    for r in range(len(g)):
        for f in range(9):
            if np.abs(o[r][f]).max() == 0:
                assert np.abs(g[r][f]).max() == 0
                continue
            assert rel(g[r][f], o[r][f]) <= 1e-4, (r, f, rel(g[r][f], o[r][f]))


def test_adjoint_source_location_bit_exact(runs):
    assert runs["nad"] == runs["o_nad32"] == 2
    assert np.array_equal(runs["gpu_is"], runs["o_is32"][: 3 * runs["nad"]])


@pytest.mark.parametrize("which", ["gpu_kernels", "lean_kernels"])
@pytest.mark.parametrize("name", ["rho", "cp", "csh", "csv"])
def test_kernels(runs, name, which):
    g = runs[which][name]
    o64 = runs["o_kernels64"][name]
    o32 = runs["o_kernels32"][name]
    assert np.abs(o64).max() > 0
    assert rel(g, o64) <= 1e-3, (name, rel(g, o64), rel(o32, o64))


@pytest.mark.parametrize("which", ["gpu_kernels", "lean_kernels"])
@pytest.mark.parametrize("name", ["Q_mu", "alpha_mu", "Q_kappa"])
def test_q_kernels(runs, name, which):
    g = runs[which][name]
    o64 = runs["o_kernels64"][name]
    assert np.abs(o64).max() > 0
    assert rel(g, o64) <= 1e-3, (name, rel(g, o64))


def test_kernel_sum_over_events(native):
    """ses3d_gpu_get_kernel_sum equals the per-event kernels added in event order."""
    from ses3d_gb300.solver import Simulation
    p = synth.make_problem("tiny", nt=NT, seed=37, adjoint_flag=1, n_events=3)
    p.setup.samp_ad = SAMP
    for k, e in enumerate(p.events):
        e.event.zzs = np.float32(5000.0 + 6000.0 * k)
    with Simulation.from_problem(p, adjoint_flag=1, grad_variant=1) as sim:
        sim.run()
        for k in range(3):
            loc, stf = adjoint_inputs(p, sim.seismograms(k))
            sim.set_adjoint_sources(k, loc, stf)
        sim.begin_adjoint()
        sim.run()
        for name in ("rho", "csv", "Q_mu"):
            per = [sim.kernel(name, k) for k in range(3)]
            assert all(np.abs(a).max() > 0 for a in per)
            assert np.array_equal(sim.kernel_sum(name), per[0] + per[1] + per[2]), name


def test_device_kernel_sums_and_misfit_gradient(native):
    """ses3d_gpu_add_kernel_sum_device adds the event sum to device memory exactly;
    ses3d_gpu_misfit_gradient_device equals (K W)(scale Jac) [/ Q] evaluated in FP64 on the
    host from the handle's geometry (W = w_i w_j w_k Jac r^2 sin(theta)), FP32 and FP64."""
    torch = pytest.importorskip("torch")
    from ses3d_gb300 import adjoint as A
    from ses3d_gb300.solver import Simulation
    p = synth.make_problem("tiny", nt=NT, seed=38, adjoint_flag=1, n_events=2)
    p.setup.samp_ad = SAMP
    with Simulation.from_problem(p, adjoint_flag=1, grad_variant=1) as sim:
        sim.run()
        for k in range(2):
            loc, stf = adjoint_inputs(p, sim.seismograms(k))
            sim.set_adjoint_sources(k, loc, stf)
        sim.begin_adjoint()
        sim.run()
        host = {nm: sim.kernel_sum(nm) for nm in A.KERNEL_NAMES}
        acc = [torch.full((sim.N,), 0.25, dtype=torch.float64, device="cuda") for _ in A.KERNEL_NAMES]
        A.kernel_sums_device(sim, "cuda", acc)
        for t, nm in zip(acc, A.KERNEL_NAMES):
            assert np.array_equal(t.cpu().numpy(), 0.25 + host[nm]), nm
        ksum = A.kernel_sums_device(sim, "cuda")
        c = sim.cfg
        ex, ey, ez = c.nx + 1, c.ny + 1, c.nz + 1
        w = sim.setup_real("w").astype(np.float64)
        jac = float(sim.setup_real("Jac")[0])
        x = sim.setup_real("x").astype(np.float64).reshape(5, ex)
        z = sim.setup_real("z").astype(np.float64).reshape(5, ez)
    W = np.empty((5, 5, 5, ez, ey, ex))
    for kn in range(5):
        for jn in range(5):
            for i_ in range(5):
                W[kn, jn, i_] = (((w[i_] * w[jn]) * w[kn]) * jac) * (z[kn] * z[kn])[:, None, None] * \
                    np.sin(x[i_])[None, None, :]
    W = W.reshape(-1)
    Q = p.model["Q"].astype(np.float32)
    for dt in (torch.float32, torch.float64):
        Qt = torch.tensor(Q, dtype=dt, device="cuda")
        grads = A.misfit_gradients_device(sim.cfg, ksum, 2.0, Qt)
        for i, (g, nm) in enumerate(zip(grads, A.KERNEL_NAMES)):
            want = (host[nm] * W) * (-2.0 * jac)
            if i == 4:
                want = want / Q.astype(np.float64)
            got = g.cpu().numpy()
            assert got.dtype == (np.float32 if dt == torch.float32 else np.float64)
            assert np.abs(want).max() > 0
            if dt == torch.float64:
                assert np.allclose(got, want, rtol=1e-14, atol=0), nm
            else:
                assert np.allclose(got, want.astype(np.float32), rtol=1e-6, atol=0), nm


@pytest.mark.parametrize("K", [0, 3])
def test_graph_replay_in_record_and_adjoint_runs(native, problem, runs, K):
    """Flag-1 and flag-2 runs replaying their plain stretches from CUDA graphs store the same
    records and give the same seismograms and kernels as eager runs, with records kept or
    checkpointed."""
    from ses3d_gb300 import _lib
    from ses3d_gb300.solver import Simulation
    p = problem
    with Simulation.from_problem(p, adjoint_flag=1, grad_variant=1) as sim:
        sim.use_graph(True, 10)
        if K:
            _lib.check(sim.lib.ses3d_gpu_set_checkpointing(sim.h, K), sim.h)
        before = sim.launch_count
        sim.run()
        assert sim.launch_count - before > 0
        if not K:
            for r in range(sim.record_count()):
                assert np.array_equal(sim.record(r), runs["gpu_records"][r]), r
        loc, stf = adjoint_inputs(p, sim.seismograms(0))
        sim.set_adjoint_sources(0, loc, stf)
        sim.begin_adjoint()
        sim.run()
        for k in ("rho", "cp", "csh", "csv", "Q_mu"):
            assert np.array_equal(sim.kernel(k), runs["gpu_kernels"][k]), k


@pytest.mark.parametrize("lean", [False, True])
def test_elastic_adjoint_kernels_match_oracle(native, oracle_mod, lean):
    """is_diss = 0 (no memory variables, the elastic element kernels): forward records and
    the four elastic Frechet kernels against the FP64 oracle, in full state and lean."""
    from ses3d_gb300.solver import Simulation
    p = synth.make_problem("small", nt=NT, seed=33, adjoint_flag=1, is_diss=0)
    p.setup.samp_ad = SAMP
    with Simulation.from_problem(p, adjoint_flag=1) as sim:
        sim.set_lean(lean)
        sim.run()
        g_rec = [sim.record(r) for r in range(sim.record_count())]
        loc, stf = adjoint_inputs(p, sim.seismograms(0))
        sim.set_adjoint_sources(0, loc, stf)
        sim.begin_adjoint()
        sim.set_lean(lean)
        sim.run()
        g = {k: sim.kernel(k) for k in ("rho", "cp", "csh", "csv")}
    o = oracle_mod.Oracle(p, fp64=True, adjoint_flag=1)
    o.run(NT)
    recs = np.stack([o.record(r) for r in range(o.nrecords())])
    assert len(g_rec) == len(recs)
    assert rel(np.stack(g_rec), recs) <= 1e-4
    sv = o.get_int("saving_vector")[1:NT + 1]
    oa = oracle_mod.Oracle(p, fp64=True, adjoint_flag=2, saving_vector=sv, ad_loc=loc, ad_stf=stf)
    oa.set_records(recs)
    oa.run(NT)
    for k in g:
        ref = oa.get("grad_" + k)
        assert np.abs(ref).max() > 0, k
        assert rel(g[k], ref) <= 1e-3, (k, rel(g[k], ref))

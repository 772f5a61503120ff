"""Differentiable misfit (torch.autograd.Function): the adjoint gradient against central
finite differences along seeded smooth model directions.

The gradient is the reference's continuous-adjoint kernel gradient (time-reversed adjoint
solve, rectangle-rule kernel integration), not the exact discrete adjoint; measured
agreement with FD on this workload is 2-6 % for rho, vp, vsh, vsv. The research Q_mu kernel
of SOURCE/ses3d_grad_Q.f90 correlates adjoint memory variables with forward strain and
recovers about half of the FD derivative; the test pins its sign and order of magnitude.
"""
import numpy as np
import pytest

from ses3d_gb300 import synth

pytestmark = pytest.mark.gpu

ELASTIC_TOL = 0.10


@pytest.fixture(scope="module")
def fd_case(native):
    import torch
    from ses3d_gb300 import adjoint as A
    p = synth.make_problem("small", nt=1500, n_el=(24, 24, 12), seed=41, adjoint_flag=1)
    setup = A.MisfitSetup.from_problem(p, samp_ad=10, fmin=1 / 80, fmax=1 / 25)
    m0 = A.problem_tensors(p)
    truth = synth.build_model(p.box, blob=(0.05, 150e3, 200e3), is_diss=1)
    setup.set_observed(A.problem_tensors(synth.Problem(p.setup, p.box, p.tau, p.D, truth, p.events, pml=p.pml)))
    rng = np.random.default_rng(5)
    ex, ey, ez = p.nx + 1, p.ny + 1, p.nz + 1
    dirs = [torch.tensor(synth.to_reference_layout(synth.correlated_field(rng, p.box, 150e3).astype(np.float64),
                                                   ex, ey, ez), device="cuda") for _ in range(5)]
    scales = [2e-3, 2e-3, 2e-3, 2e-3, 2e-2]
    deltas = [s * d * m for s, d, m in zip(scales, dirs, m0)]
    ms = [t.clone().requires_grad_(True) for t in m0]
    chi = A.waveform_misfit(setup, *ms)
    chi.backward()
    out = {}
    for k, nm in enumerate(("rho", "vp", "vsh", "vsv", "Q")):
        g = float(torch.sum(ms[k].grad.double() * deltas[k].double()))
        mp = [t.clone() for t in m0]
        mm = [t.clone() for t in m0]
        mp[k] = mp[k] + deltas[k].float()
        mm[k] = mm[k] - deltas[k].float()
        fd = (A.misfit_only(setup, *mp) - A.misfit_only(setup, *mm)) / 2
        out[nm] = (g, fd)
    return float(chi.detach()), out


def test_misfit_positive(fd_case):
    chi, _ = fd_case
    assert chi > 0 and np.isfinite(chi)


@pytest.mark.parametrize("name", ["rho", "vp", "vsh", "vsv"])
def test_elastic_gradient_matches_finite_differences(fd_case, name):
    _, out = fd_case
    g, fd = out[name]
    assert fd != 0
    assert abs(g / fd - 1.0) < ELASTIC_TOL, (name, g, fd, g / fd)


def test_q_kernel_sign_and_magnitude(fd_case):
    _, out = fd_case
    g, fd = out["Q"]
    assert 0.3 < g / fd < 1.5, (g, fd)


def test_checkpointed_gradient_equals_stored(native):
    """An HBM budget that forces checkpoint + recompute gives the same gradient bit for bit."""
    import torch
    from ses3d_gb300 import adjoint as A
    p = synth.make_problem("tiny", nt=120, seed=43, adjoint_flag=1)
    grads = []
    for budget in (1e12, 1.0):
        setup = A.MisfitSetup.from_problem(p, samp_ad=5, fmin=1 / 40, fmax=1 / 8, memory_budget=budget)
        setup.set_observed([t * 1.01 for t in A.problem_tensors(p)])
        ms = [t.clone().requires_grad_(True) for t in A.problem_tensors(p)]
        chi = A.waveform_misfit(setup, *ms)
        chi.backward()
        grads.append([m.grad.cpu().numpy() for m in ms])
        assert (setup.last["records_per_segment"] > 0) == (budget < 10)
    for a, b in zip(*grads):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("per_batch,ckpt", [(1, False), (2, True)])
def test_sub_batched_gradient_equals_one_batch(native, per_batch, ckpt):
    """A budget that admits only per_batch events at a time runs the events in sub-batches
    (forward recomputed in the backward pass) and gives the one-batch gradient."""
    import torch
    from ses3d_gb300 import adjoint as A
    # the plan takes the storage with the fewest recompute passes that fits: for the checkpoint
    # case the records of one event must not fit where two checkpointed events do, which
    # takes ~200 records (1000 steps store 201)
    p = synth.make_problem("tiny", nt=1000 if ckpt else 80, seed=47, adjoint_flag=1, n_events=3)
    for k, e in enumerate(p.events):
        e.event.zzs = np.float32(6000.0 + 7000.0 * k)
    grads, plans = [], []
    for sub in (False, True):
        setup = A.MisfitSetup.from_problem(p, samp_ad=5, fmin=1 / 40, fmax=1 / 8)
        m = setup.memory_model()
        shared, keep = m["shared"], m["keep"]
        per = m["one_level"] if ckpt else keep
        setup.memory_budget = (shared + per * (per_batch + 0.5)) if sub else 1e13
        if sub and ckpt:
            assert shared + keep > setup.memory_budget      # the records of one event do not fit
        setup.set_observed([t * 1.01 for t in A.problem_tensors(p)])
        ms = [t.clone().requires_grad_(True) for t in A.problem_tensors(p)]
        chi = A.waveform_misfit(setup, *ms)
        chi.backward()
        grads.append((float(chi.detach()), [m.grad.cpu().numpy() for m in ms]))
        plans.append(setup.last["plan"])
    assert len(plans[0].groups) == 1 and plans[1].events_per_batch == per_batch
    assert (plans[1].K > 0) == ckpt
    assert grads[0][0] == grads[1][0]
    for a, b in zip(grads[0][1], grads[1][1]):
        if per_batch == 1:
            assert np.array_equal(a, b)              # same FP64 summation order
        else:
            assert np.allclose(a, b, rtol=1e-12, atol=0)


def test_wrong_sized_model_tensors_are_rejected_before_any_device_work(native):
    """The library reads model records and kernels through raw device pointers, so the
    Python side checks their sizes and types first."""
    import torch
    from ses3d_gb300 import adjoint as A
    p = synth.make_problem("tiny", nt=20, seed=43, adjoint_flag=1)
    setup = A.MisfitSetup.from_problem(p, samp_ad=5)
    m = list(A.problem_tensors(p))
    short = [t[:-1].contiguous() for t in m]
    with pytest.raises(ValueError, match="GLL points"):
        A.waveform_misfit(setup, *short)
    with pytest.raises(TypeError, match="CUDA"):
        setup.simulate({"rhoinv": torch.ones(setup.n_points)})
    ksum = [torch.zeros(setup.n_points, dtype=torch.float64, device="cuda") for _ in range(5)]
    with pytest.raises(ValueError, match="CUDA tensors"):
        A.misfit_gradients_device(setup.cfg_template, ksum[:4] + [ksum[4][:-1]], 1.0, m[4])
    g = A.misfit_gradients_device(setup.cfg_template, ksum, 1.0, m[4])
    assert all(t.shape == m[4].shape and torch.all(t == 0) for t in g)

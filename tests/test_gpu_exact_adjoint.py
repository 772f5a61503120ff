"""The exact discrete adjoint (ses3d_gpu_exact_*): the backward run is the transpose of the
forward time step.

* Dot-product tests: for random states x (forward, initial) and y (adjoint, final),
  <Phi^n x, y> = <x, (Phi^T)^n y> for one iteration and for several iterations spread over
  checkpoint segments, with and without attenuation. Sources are off (the iteration is then
  linear in the state).
* Model gradient of one iteration: J(m) = <Phi_m x, y> differentiated with respect to each
  model record (rhoinv, mu, lambda, A, B, C, Q) against central finite differences of the
  forward iteration.
Tolerances are those of FP32 arithmetic on sums over the whole state.
"""
import numpy as np
import pytest
from wavefields import GRADS, MEMVARS, MIRROR, STRESS, VELOCITY, random_state

from ses3d_gb300 import synth

pytestmark = pytest.mark.gpu

FIELDS = VELOCITY + STRESS + tuple(MIRROR) + GRADS
RECORDS = ("rhoinv", "mu", "lambda", "A", "B", "C", "Q")


def dot(a, b, names):
    return sum(float(np.dot(np.asarray(a[k], np.float64), np.asarray(b[k], np.float64))) for k in names)


def silent_problem(nt, is_diss, seed):
    """The 10 x 9 x 6 test mesh (PML 3: PML and interior elements) without sources."""
    p = synth.make_problem("small", nt=nt, seed=seed, is_diss=is_diss)
    p.events[0].stf[:] = 0.0
    return p


def independent_state(p, seed, is_diss):
    """A random state whose mirror stresses differ from their partners (the iteration's
    state has nine independent stress components)."""
    st = random_state(p, seed, is_diss)
    rng = np.random.default_rng(seed + 1000)
    for k in MIRROR:
        st[k] = (st[k] + np.float32(1e5) * rng.standard_normal(st[k].size).astype(np.float32)).astype(np.float32)
    return st


def forward_then_backward(p, x, y, nt, K, is_diss, K2=0):
    from ses3d_gb300.solver import Simulation
    names = FIELDS + (MEMVARS if is_diss else ())
    with Simulation.from_problem(p) as sim:
        sim.exact_adjoint(K, K2)
        for k in names:
            sim.set_field(k, x[k])
        sim.step(nt)
        phix = {k: sim.field(k) for k in names}
        for k in names:
            sim.set_exact_field(k, y[k])
        sim.exact_backward()
        aty = {k: sim.exact_field(k) for k in names}
    return dot(phix, y, names), dot(x, aty, names), names


@pytest.mark.parametrize("is_diss", [1, 0])
def test_dot_product_one_iteration(native, is_diss):
    p = silent_problem(1, is_diss, 61)
    x = independent_state(p, 3, is_diss)
    y = independent_state(p, 4, is_diss)
    lhs, rhs, _ = forward_then_backward(p, x, y, 1, 1, is_diss)
    print("dot one iteration is_diss=%d: %.9e %.9e rel %.2e" % (is_diss, lhs, rhs, abs(lhs - rhs) / abs(lhs)))
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)


@pytest.mark.parametrize("K,K2", [(1, 0), (3, 0), (7, 0), (7, 3), (4, 3), (5, 2)])
def test_dot_product_several_iterations(native, K, K2):
    """Seven iterations with checkpoints every K (segments of K iterations recomputed), and
    with a second level every K2 iterations of a segment."""
    p = silent_problem(7, 1, 62)
    x = independent_state(p, 5, 1)
    y = independent_state(p, 6, 1)
    lhs, rhs, _ = forward_then_backward(p, x, y, 7, K, 1, K2)
    print("dot seven iterations K=%d K2=%d: %.9e %.9e rel %.2e" % (K, K2, lhs, rhs, abs(lhs - rhs) / abs(lhs)))
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)


def test_dot_product_several_items_per_cta(native):
    """The 20 x 20 x 10 mesh (4,000 elements): each CTA of the persistent forward and
    transposed element kernels steps several elements, so the copies of the next item are in
    flight while the current one is computed. Five iterations, checkpoints every 3."""
    p = synth.make_problem("small", nt=5, seed=65, n_el=(20, 20, 10))
    p.events[0].stf[:] = 0.0
    x = independent_state(p, 7, 1)
    y = independent_state(p, 8, 1)
    lhs, rhs, _ = forward_then_backward(p, x, y, 5, 3, 1)
    print("dot 20x20x10: %.9e %.9e rel %.2e" % (lhs, rhs, abs(lhs - rhs) / abs(lhs)))
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)


def one_iteration_misfit(p, x, y, names, model):
    from ses3d_gb300.solver import Simulation
    q = synth.Problem(p.setup, p.box, p.tau, p.D, model, p.events, pml=p.pml)
    with Simulation.from_problem(q) as sim:
        for k in names:
            sim.set_field(k, x[k])
        sim.step(1)
        return dot({k: sim.field(k) for k in names}, y, names)


@pytest.mark.parametrize("case", ["stress_to_velocity", "velocity_to_stress"])
def test_model_gradient_one_iteration(native, case):
    """dJ/dm of J = <Phi_m x, y> (one iteration) for each model record against central
    differences of the forward iteration along a random direction (relative step 1e-2 of
    the record, or of mu for the anisotropic records, which are zero). Two cases keep the
    identity part of the iteration out of J, so that FP32 rounding of the state does not
    swamp the differences: x without velocity and y on the velocity only (the assembled
    stress divergence and the mass matrix), and x without stresses and y on the stresses
    only (the stress rates)."""
    from ses3d_gb300.solver import Simulation
    p = silent_problem(1, 1, 63)
    x = independent_state(p, 7, 1)
    y = independent_state(p, 8, 1)
    names = FIELDS + MEMVARS
    if case == "stress_to_velocity":
        x.update({k: np.zeros_like(x[k]) for k in VELOCITY})
        y.update({k: np.zeros_like(y[k]) for k in names if k not in VELOCITY})
        records = RECORDS
    else:
        x.update({k: np.zeros_like(x[k]) for k in STRESS + tuple(MIRROR)})
        y.update({k: np.zeros_like(y[k]) for k in names if k not in STRESS + tuple(MIRROR)})
        records = RECORDS[1:]          # 1/rho does not reach the stresses within one iteration
    with Simulation.from_problem(p) as sim:
        sim.exact_adjoint(1)
        for k in names:
            sim.set_field(k, x[k])
        sim.step(1)
        for k in names:
            sim.set_exact_field(k, y[k])
        sim.exact_backward()
        grads = {r: sim.exact_gradient(r) for r in records}
    rng = np.random.default_rng(9)
    mu_scale = float(np.mean(np.abs(p.model["mu"])))
    for r in records:
        base = p.model[r].astype(np.float64)
        scale = np.abs(base) if np.any(base != 0) else np.full(base.shape, mu_scale)
        d = rng.uniform(0.5, 1.0, base.size) * scale
        js = []
        for sgn in (1, -1):
            m = dict(p.model)
            if r == "Q":
                # the iteration is linear in 1/Q: perturb 1/Q (10 %), so that the difference
                # has no truncation error, and take the gradient along the same step
                tau = (1.0 / base + sgn * 0.1 * d / base / base).astype(np.float64)
                m[r] = (1.0 / tau).astype(np.float32)
            else:
                m[r] = (base + sgn * 1e-2 * d).astype(np.float32)
            js.append((one_iteration_misfit(p, x, y, names, m), m[r].astype(np.float64)))
        fd = js[0][0] - js[1][0]
        if r == "Q":   # <dJ/dQ, dQ> along 1/Q: dJ/d(1/Q) = -Q^2 dJ/dQ
            an = float(np.dot(-grads[r] * base * base, 1.0 / js[0][1] - 1.0 / js[1][1]))
        else:
            an = float(np.dot(grads[r], js[0][1] - js[1][1]))
        err = abs(fd - an) / max(abs(fd), 1e-300)
        print("one-iteration gradient %s %s: fd %.6e exact %.6e rel %.2e" % (case, r, fd, an, err))
        assert abs(fd) > 0
        assert err <= 1e-3, (case, r, fd, an)


@pytest.fixture(scope="module")
def c3_misfit(native):
    """The 64 x 64 x 32 misfit workload over a shortened time axis (nt = 300, 24 s): receivers
    on a ring 40-90 km from the source so that they record within the run, observed data from
    a model 1 % faster with 1 % more attenuation, misfit band 6-30 s."""
    import torch
    from ses3d_gb300 import adjoint as A
    nt = 300
    p = synth.make_problem("c3", nt=nt, seed=1234, adjoint_flag=1)
    ev = p.events[0]
    rng = np.random.default_rng(71)
    az = rng.uniform(0, 2 * np.pi, 12)
    dist = rng.uniform(40e3, 90e3, 12) / 6371e3 * 180 / np.pi            # degrees of arc
    loc = np.stack([float(ev.event.xxs) + dist * np.cos(az), float(ev.event.yys) + dist * np.sin(az),
                    np.zeros(12)], axis=1).astype(np.float32)
    ev.receivers.loc = loc
    ev.receivers.names = ["R%02d" % k for k in range(12)]
    setup = A.MisfitSetup.from_problem(p, samp_ad=10, fmin=1 / 30, fmax=1 / 6)
    m0 = A.problem_tensors(p)
    truth = [m0[0], m0[1] * 1.01, m0[2] * 1.01, m0[3] * 1.01, m0[4] * 0.99]
    setup.set_observed(truth)
    ex, ey, ez = p.nx + 1, p.ny + 1, p.nz + 1
    dirs = [torch.tensor(synth.to_reference_layout(synth.correlated_field(rng, p.box, 100e3).astype(np.float64),
                                                   ex, ey, ez), device="cuda") for _ in range(5)]
    deltas = [d * m.double() for d, m in zip(dirs, m0)]
    return p, setup, m0, deltas


def misfit_gradient(setup, m0, exact):
    from ses3d_gb300 import adjoint as A
    setup.exact = exact
    ms = [t.clone().requires_grad_(True) for t in m0]
    chi = A.waveform_misfit(setup, *ms)
    chi.backward()
    setup.exact = False
    return float(chi.detach()), [m.grad.double() for m in ms]


def test_exact_misfit_gradient_matches_finite_differences(c3_misfit):
    """The exact discrete-adjoint gradient of the L2 waveform misfit (torch.autograd, FP64
    misfit) against central finite differences of the forward run along a seeded smooth
    random direction for each of rho, vp, vsh, vsv and Q_mu, Richardson-extrapolated from two
    step sizes: <= 1e-3 relative. The continuous-adjoint (ses3d_grad) gradient of the same
    misfit is printed beside it. (Smaller steps, 1e-3, let FP32 rounding of the forward runs
    show at about 1e-3 of the differences.)"""
    import torch
    from ses3d_gb300 import adjoint as A
    p, setup, m0, deltas = c3_misfit
    chi0, g_exact = misfit_gradient(setup, m0, True)
    _, g_cont = misfit_gradient(setup, m0, False)
    assert chi0 > 0
    names = ("rho", "vp", "vsh", "vsv", "Q")
    # relative steps: large enough that FP32 rounding of the forward runs (about 1e-5 of the
    # seismograms) stays far below the differences, with the O(h^2) truncation removed by
    # Richardson extrapolation over h and 2 h
    steps = (1e-2, 1e-2, 1e-2, 1e-2, 5e-2)
    for k, nm in enumerate(names):
        d = deltas[k]
        ge = float(torch.sum(g_exact[k] * d))
        gc = float(torch.sum(g_cont[k] * d))
        fds = []
        for h in (2 * steps[k], steps[k]):
            js = []
            for sgn in (1.0, -1.0):
                ms = [t.clone() for t in m0]
                ms[k] = (m0[k].double() + sgn * h * d).float()
                js.append(A.misfit_only(setup, *ms))
            fds.append((js[0] - js[1]) / (2 * h))
        fd = (4 * fds[1] - fds[0]) / 3
        err = abs(ge - fd) / abs(fd)
        print("misfit gradient %s: fd %.8e (h: %.8e, 2h: %.8e) exact %.8e rel %.2e | ses3d_grad %.8e rel %.2e"
              % (nm, fd, fds[1], fds[0], ge, err, gc, abs(gc - fd) / abs(fd)))
        assert abs(fd) > 0
        assert err <= 1e-3, (nm, fd, ge)


@pytest.mark.parametrize("K,K2,n_el", [(7, 0, None), (7, 3, None), (7, 3, (20, 20, 10))])
def test_lean_forward_gives_the_same_gradient(native, K, K2, n_el):
    """A run from rest stepped lean (elements outside the PML keep neither displacement
    gradients nor mirror stresses) gives the exact gradient and the adjoint of the initial
    state of the full-state run bit for bit, with one and two checkpoint levels (and on a
    20 x 20 x 10 mesh, several elements per CTA of the persistent kernels); the choice
    cannot change once the forward run has started."""
    from ses3d_gb300 import _lib
    from ses3d_gb300.solver import Simulation
    nt = 30
    p = synth.make_problem("small", nt=nt, seed=64, n_el=n_el)
    out = []
    for lean in (False, True):
        with Simulation.from_problem(p) as sim:
            sim.exact_adjoint(K, K2)
            sim.set_lean(lean)
            sim.step(5)
            with pytest.raises(_lib.Ses3dError) as err:
                sim.set_lean(not lean)
            assert err.value.code == -4
            sim.set_lean(lean)                      # the same choice again is accepted
            sim.run()
            seis = sim.seismograms(0)
            assert np.abs(seis[2]).max() > 0
            sim.set_seismogram_adjoint(0, *seis)
            sim.exact_backward()
            out.append(([sim.exact_gradient(r) for r in RECORDS],
                        [sim.exact_field(k) for k in ("vx_global", "vz_global", "sxx_pml", "Mxx", "dxux")]))
    for a, b in zip(out[0][0] + out[0][1], out[1][0] + out[1][1]):
        assert np.abs(a).max() > 0
        assert np.array_equal(a, b)


def test_untouched_adjoint_gradients_skip_outside_the_pml(native):
    """A backward run whose adjoint displacement gradients start at zero leaves them out
    outside the PML (they stay zero there); setting them to zero explicitly takes the path
    that reads and writes them everywhere. Both give the same gradient and adjoint initial
    state bit for bit."""
    from ses3d_gb300.solver import Simulation
    nt = 20
    p = synth.make_problem("small", nt=nt, seed=66)
    out = []
    for explicit in (False, True):
        with Simulation.from_problem(p) as sim:
            sim.exact_adjoint(6)
            sim.run()
            seis = sim.seismograms(0)
            sim.set_seismogram_adjoint(0, *seis)
            if explicit:
                for k in GRADS:
                    sim.set_exact_field(k, np.zeros(sim.N, np.float32))
            sim.exact_backward()
            out.append([sim.exact_gradient(r) for r in RECORDS] +
                       [sim.exact_field(k) for k in ("vx_global", "sxz_pml", "dxux", "dzuy", "Myz")])
    for q, (a, b) in enumerate(zip(*out)):
        if q < len(RECORDS):
            assert np.abs(a).max() > 0
        assert np.array_equal(a, b), q

"""Known-answer tests that pin the CPU oracle (the reference ships no tests or golden
vectors, so these builder-made identities are what the oracle is checked against)."""
import numpy as np
import pytest

from ses3d_gb300 import synth

EXACT_KNOTS = np.array([-1.0, -np.sqrt(3.0 / 7.0), 0.0, np.sqrt(3.0 / 7.0), 1.0])


def lagrange_derivative_matrix(x):
    """D[i, j] = l_i'(x_j) for the Lagrange basis on knots x (float64 closed form)."""
    n = len(x)
    D = np.zeros((n, n))
    for i in range(n):
        for j in range(n):
            if i == j:
                D[i, j] = sum(1.0 / (x[i] - x[k]) for k in range(n) if k != i)
            else:
                num = np.prod([x[j] - x[k] for k in range(n) if k not in (i, j)])
                den = np.prod([x[i] - x[k] for k in range(n) if k != i])
                D[i, j] = num / den
    return D


@pytest.fixture(scope="module")
def tiny():
    return synth.make_problem("tiny", nt=30, seed=7)


@pytest.fixture(scope="module")
def oracles(oracle_mod, tiny):
    o32 = oracle_mod.Oracle(tiny)
    o64 = oracle_mod.Oracle(tiny, fp64=True)
    return o32, o64


def test_knots_and_weights(oracles):
    o32, o64 = oracles
    k64, w64 = o64.get("knots"), o64.get("w")
    assert np.allclose(k64, EXACT_KNOTS, atol=1e-15)
    assert np.array_equal(o32.get("knots"), EXACT_KNOTS.astype(np.float32))
    # truncated decimal weights (ses3d_init.f90:135-139): sum 2 to 13 digits
    assert abs(w64.sum() - 2.0) < 1e-12
    assert abs(float(o32.get("w").astype(np.float64).sum()) - 2.0) < 1e-6


@pytest.mark.parametrize("power", range(8))
def test_gll_quadrature_exact_to_degree_7(oracles, power):
    _, o64 = oracles
    x, w = o64.get("knots"), o64.get("w")
    exact = 0.0 if power % 2 else 2.0 / (power + 1)
    assert abs(np.sum(w * x ** power) - exact) < 1e-11


def test_dl_closed_form_and_row_sums(oracles):
    o32, o64 = oracles
    D = lagrange_derivative_matrix(EXACT_KNOTS)
    dl64 = o64.get("dl").reshape(5, 5, order="F")  # dl(i,j) = l_i'(x_j)
    dl32 = o32.get("dl").reshape(5, 5, order="F").astype(np.float64)
    assert np.allclose(dl64, D, atol=1e-12)
    assert np.allclose(dl32, D, atol=2e-6)
    # derivative of the constant function: sum_i l_i'(x_j) = 0
    assert np.abs(dl64.sum(axis=0)).max() < 1e-12


def test_dl_differentiates_polynomials_exactly(oracles):
    _, o64 = oracles
    x = o64.get("knots")
    dl = o64.get("dl").reshape(5, 5, order="F")
    rng = np.random.default_rng(0)
    c = rng.standard_normal(5)
    p = np.polyval(c, x)
    dp = np.polyval(np.polyder(c), x)
    assert np.allclose(dl.T @ p, dp, atol=1e-11)


def test_jacobian_and_element_widths(oracles, tiny):
    o32, _ = oracles
    b = tiny.box
    dx = (b.xmax - b.xmin) / np.float32(b.nx + 1)
    dy = (b.ymax - b.ymin) / np.float32(b.ny + 1)
    dz = (b.zmax - b.zmin) / np.float32(b.nz + 1)
    assert o32.get("dx")[0] == dx and o32.get("dy")[0] == dy and o32.get("dz")[0] == dz
    assert o32.get("Jac")[0] == dx * dy * dz / np.float32(8)


def test_mass_matrix_negative_and_complete(oracles):
    """MM = -sum w w w Jac r^2 sin(theta) / rhoinv (ses3d_init.f90:267-270): strictly negative."""
    o32, o64 = oracles
    mm = o64.get("MM_global")
    assert np.all(mm < 0)
    # total mass: sum of -MM equals the quadrature of rho r^2 sin(theta) over the box
    rho = 1.0 / o64.get("rhoinv")
    jac, w = o64.get("Jac")[0], o64.get("w")
    W = np.einsum("i,j,k->ijk", w, w, w).reshape(-1, order="F")
    r, st = o64.get("r"), o64.get("sin_theta")
    E = rho.size // 125
    vol = np.sum(np.repeat(W, E) * jac * r * r * st * rho)
    assert abs(-mm.sum() - vol) / vol < 1e-12


def test_fp32_tracks_fp64(oracle_mod):
    p = synth.make_problem("tiny", nt=60, seed=12)
    a, b = oracle_mod.Oracle(p), oracle_mod.Oracle(p, fp64=True)
    a.run(60)
    b.run(60)
    s32, s64 = np.concatenate(a.seismograms()), np.concatenate(b.seismograms())
    assert np.abs(s64).max() > 0
    # three-component rel-L2 (a weak single component alone can sit near 1e-4)
    assert np.linalg.norm(s32 - s64) / np.linalg.norm(s64) < 1e-5


def test_deterministic(oracle_mod):
    p = synth.make_problem("tiny", nt=15, seed=13)
    runs = []
    for _ in range(2):
        o = oracle_mod.Oracle(p)
        o.run(15)
        runs.append(o.get("vz_global"))
    assert np.array_equal(runs[0], runs[1])


def test_first_sample_is_zero(oracles):
    """record_seismograms interpolates the pre-update velocity: seismogram(1) = 0."""
    o32, _ = oracles
    o32.run(3)
    for s in o32.seismograms():
        assert np.all(s[:, 0] == 0)


def test_p_wave_travel_time(oracle_mod):
    """Homogeneous elastic medium, vertical single force 100 km below a surface receiver:
    the vertical displacement peaks one P travel time (distance / vp) after the peak of
    the Gaussian force."""
    p = synth.make_problem("small", nt=300, seed=17, is_diss=0)
    vals = {"rhoinv": 1.0 / 3000.0, "mu": 3000.0 * 4000.0 ** 2, "lambda": 3000.0 * (7000.0 ** 2 - 2 * 4000.0 ** 2)}
    for k, v in vals.items():
        p.model[k][:] = np.float32(v)
    ev = p.events[0]
    ev.event.source_type = 3
    ev.event.zzs = np.float32(100000.0)
    ev.event.xxs, ev.event.yys = np.float32(50.0), np.float32(10.0)
    dt = float(ev.event.dt)
    t = np.arange(len(ev.stf)) * dt
    ev.stf = (np.exp(-((t - 8.0) / 3.0) ** 2) * 1e15).astype(np.float32)
    ev.receivers.loc[:] = [[50.0, 10.0, 0.0]] * len(ev.receivers.loc)
    o = oracle_mod.Oracle(p, fp64=True)
    o.run(300)
    uz = np.cumsum(o.seismograms()[2][0]) * dt
    t_peak = np.argmax(np.abs(uz)) * dt
    expected = 8.0 + 100e3 / 7000.0
    assert abs(t_peak - expected) < 2.0, (t_peak, expected)


@pytest.mark.parametrize("source_type,comp,speed", [(1, 0, 4000.0), (2, 1, 4000.0), (3, 2, 7000.0)])
def test_body_wave_travel_times(oracle_mod, source_type, comp, speed):
    """Homogeneous elastic box (vp 7 km/s, vs 4 km/s) resolved at the source band: a force
    150 km below a surface receiver, Gaussian in time (peak at 8 s, sigma 3 s). A horizontal
    force gives a transverse displacement peaking one S travel time (150 km / vs) after the
    force peak, a vertical force a vertical displacement peaking one P travel time later."""
    p = synth.homogeneous_problem(source_type=source_type)
    o = oracle_mod.Oracle(p, fp64=True)
    o.run(p.events[0].event.nt)
    dt = float(p.events[0].event.dt)
    u = np.cumsum(o.seismograms()[comp][0]) * dt
    t_peak = np.argmax(np.abs(u)) * dt
    expected = 8.0 + 150e3 / speed
    assert abs(t_peak - expected) < 1.5, (t_peak, expected)


ENERGY_BOX = dict(n_el=(6, 6, 4), colat=(44.0, 46.0), lon=(9.0, 11.0), r=(6171000.0, 6371000.0), nt=800, dt=0.05,
                  source_type=10, depth_m=60000.0, t0=3.0, sigma=1.0)


def test_energy_conserved_without_pml_and_absorbed_with_pml(oracle_mod, wave_energy):
    """Elastic homogeneous box, explosion at 60 km depth ending by 6 s. With every boundary
    traction-free (pml 0) the total energy stays constant to the scheme's fluctuation; with
    PML on the sides and bottom it never increases and the PML absorbs most of it by 40 s."""
    series = {}
    for pml in (0, 2):
        p = synth.homogeneous_problem(pml=pml, **ENERGY_BOX)
        o = oracle_mod.Oracle(p, fp64=True)
        e = []
        for _ in range(20):                     # t = 2, 4, ..., 40 s
            o.run(40)
            e.append(wave_energy(o.get, o.get, p))
        series[pml] = np.array(e)
    free, absorbed = series[0][3:], series[2][4:]      # t >= 8 s, t >= 10 s
    assert free.max() - free.min() < 0.03 * free.mean(), free
    assert np.all(absorbed[1:] <= 1.005 * absorbed[:-1]), absorbed
    assert absorbed[-1] < 0.35 * series[2][3], (absorbed[-1], series[2][3])

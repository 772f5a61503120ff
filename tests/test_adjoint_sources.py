"""Adjoint-source generation (TOOLS/adjoint_source.py, TOOLS/seismograms.py restated):
known answers and first-order identities of each measurement, file formats."""
import os

import numpy as np
import pytest

from ses3d_gb300 import adjoint_sources as AS
from ses3d_gb300 import formats as F


def pulse(nt=600, dt=0.1, t0=25.0, period=8.0):
    t = np.arange(nt) * dt
    return np.exp(-((t - t0) / (0.35 * period)) ** 2) * np.cos(2 * np.pi * (t - t0) / period)


def seismo(tr, dt=0.1, integrate=True):
    traces = np.stack([tr, 0.5 * tr, -0.25 * tr])
    return AS.Seismogram.from_traces(traces, dt, receiver=(50.36, 27.88, 0.0), source=(45.0, 10.0, 15000.0),
                                     integrate=False) if not integrate else _displacement(traces, dt)


def _displacement(traces, dt):
    s = AS.Seismogram.from_traces(traces, dt, receiver=(50.36, 27.88, 0.0), source=(45.0, 10.0, 15000.0))
    s.integrate = True  # traces taken as displacement directly
    return s


def test_python2_semantics():
    assert AS.round_half_away(2.5) == 3 and AS.round_half_away(-2.5) == -3 and AS.round_half_away(3.49) == 3
    assert AS.py2_str(0.0) == "0.0" and AS.py2_str(1.0) == "1.0"
    assert AS.py2_str(1.0 / 3.0) == "0.333333333333"
    assert AS.py2_str(50.36000061035156) == "50.3600006104"
    assert AS.py2_str(1e-20) == "1e-20"


def test_seismogram_file_round_trip(tmp_path):
    nt, dt = 120, 0.25
    rng = np.random.default_rng(0)
    tr = rng.standard_normal((3, nt)).astype(np.float32)
    F.write_seismograms(str(tmp_path) + "/", "STAT01      ", tr[0], tr[1], tr[2], nt, np.float32(dt),
                        (np.float32(50.36), np.float32(27.88), np.float32(0.0)),
                        (np.float32(45.0), np.float32(10.0), np.float32(15000.0)))
    s = AS.Seismogram().read(str(tmp_path) + "/", "STAT01      ")
    assert s.nt == nt and s.dt == pytest.approx(dt)
    assert (s.rx, s.ry, s.rz) == pytest.approx((50.36, 27.88, 0.0), rel=1e-6)
    assert (s.sx, s.sy, s.sz) == pytest.approx((45.0, 10.0, 15000.0), rel=1e-6)
    assert np.array_equal(s.trace_x.astype(np.float32), tr[0])
    assert np.array_equal(s.trace_z.astype(np.float32), tr[2])
    assert s.t[-1] == pytest.approx(nt * dt) and len(s.t) == nt  # the reference's stretched axis
    si = AS.Seismogram().read(str(tmp_path) + "/", "STAT01      ", integrate=True)
    assert np.allclose(si.trace_y, np.cumsum(tr[1].astype(np.float64)) * s.dt)


def test_window_taper_shape():
    a = AS.AdjointSource()
    a.fetch_seismogram(seismo(pulse()))
    tp = a._window_taper(10.0, 40.0, 2.0)
    s = a.s
    inside = (s.t > 12.5) & (s.t < 37.5)
    assert np.all(tp[inside] == 1.0)
    assert np.all(tp[s.t < 9.9] == 0.0) and np.all(tp[s.t > 40.1] == 0.0)
    assert np.all((tp >= 0) & (tp <= 1))


def test_l2amp_identity_displacement():
    """sum(adsrc * d_tapered) dt = 2 for the L2 amplitude source on displacement."""
    d = pulse()
    a = AS.AdjointSource()
    a.fetch_seismogram(seismo(d))
    a.make_adsrc_L2amp("x", 10.0, 40.0, 2.0)
    dt_ = a._trace("x") * a._window_taper(10.0, 40.0, 2.0)
    assert np.sum(a.adsrc_x * dt_) * a.s.dt == pytest.approx(2.0, rel=1e-12)
    assert np.all(a.adsrc_y == 0) and np.all(a.adsrc_z == 0)


def test_cc_identity_and_velocity_derivative():
    """cc source = -d'/(sum d'^2 dt); for velocity seismograms it is differentiated once
    more with forward differences and a zero last sample."""
    d = pulse()
    a = AS.AdjointSource()
    a.fetch_seismogram(seismo(d))
    a.make_adsrc_cc("y", 10.0, 40.0, 2.0)
    dtap = a._trace("y") * a._window_taper(10.0, 40.0, 2.0)
    dp = np.append(np.diff(dtap) / a.s.dt, 0.0)
    assert np.sum(a.adsrc_y * dp) * a.s.dt == pytest.approx(-1.0, rel=1e-12)
    v = AS.AdjointSource()
    v.fetch_seismogram(seismo(d, integrate=False))
    v.make_adsrc_cc("y", 10.0, 40.0, 2.0)
    ref = a.adsrc_y
    assert np.allclose(v.adsrc_y[:-1], -np.diff(ref) / a.s.dt, rtol=1e-12, atol=0)
    assert v.adsrc_y[-1] == 0.0


def test_prolate_spheroidal_sequences():
    N, kmax = 101, 4
    W = 3.0 * kmax / (2.0 * N)
    eig, c = AS.ps_sequences(N, W)
    good = eig[np.isfinite(eig)]
    assert good.size > 2 * kmax and np.array_equal(eig[:good.size], good)   # NaNs (if any) last
    assert np.all(np.diff(good) <= 1e-12)
    assert np.all(eig[:kmax + 1] > 0.99) and np.all(good <= 1 + 1e-9)
    # concentration identity: eig_k = (c^T K c)_k / (c^T c)_k with the sinc kernel
    n = np.arange(N)
    K = 2 * W * np.sinc(2 * W * (n[:, None] - n[None, :]))
    for k in range(kmax + 1):
        ck = c[:, k]
        assert (ck @ K @ ck) / (ck @ ck) == pytest.approx(eig[k], rel=1e-8)
    e2, Psi = AS.ps_frequency(N, W, kmax, np.array([0.0]))
    assert np.allclose(Psi[0], c[:, :kmax + 1].sum(axis=0))
    e3, psi = AS.ps_index(N, W, kmax, np.arange(-(N - 1) / 2, (N - 1) / 2 + 1))
    assert np.array_equal(e2, e3) and psi.shape == (N, kmax + 1)


def _mt_phase_amp(a, comp, wl, wr, nu):
    _, u, _, _, nu_n = a._multitaper(comp, wl, wr, nu)
    return np.angle(u), np.log(np.abs(u)), nu_n


@pytest.mark.parametrize("kind", ["mttime", "mtamp"])
def test_multitaper_sources_are_measurement_derivatives(kind):
    """sum(adsrc * delta_d) dt equals the first-order change of the measurement: the phase
    of the multitaper spectral estimate over 2 pi nu_n (mttime), its log amplitude (mtamp)."""
    d = pulse(nt=800, dt=0.1, t0=30.0, period=10.0)
    rng = np.random.default_rng(3)
    dd = 1e-6 * np.convolve(rng.standard_normal(d.size), np.ones(15) / 15, mode="same")
    a = AS.AdjointSource()
    a.fetch_seismogram(seismo(d))
    getattr(a, "make_adsrc_" + kind)("z", 15.0, 45.0, 0.1)
    b = AS.AdjointSource()
    b.fetch_seismogram(seismo(d + dd))
    p0, l0, nu_n = _mt_phase_amp(a, "z", 15.0, 45.0, 0.1)
    p1, l1, _ = _mt_phase_amp(b, "z", 15.0, 45.0, 0.1)
    lin = np.sum(a.adsrc_z * (-0.25 * dd)) * a.s.dt  # component z carries -0.25 d
    want = (p1 - p0) / (2 * np.pi * nu_n) if kind == "mttime" else (l1 - l0)
    assert lin == pytest.approx(want, rel=1e-4)


def test_write_reads_back_time_reversed(tmp_path):
    a = AS.AdjointSource()
    a.fetch_seismogram(seismo(pulse(nt=50)))
    a.make_adsrc_L2amp("x", 0.5, 4.5, 0.5)
    a.adsrc_z = np.linspace(-1, 1, a.s.nt)
    loc = AS.write_adjoint_directory(str(tmp_path), [a, a], depth=1000.0)
    assert loc.shape == (2, 3) and loc[0, 2] == np.float32(1000.0)
    lines = open(os.path.join(str(tmp_path), "ad_src_1")).read().splitlines()
    assert lines[0] == "-- adjoint source ------------------"
    assert lines[2] == "50.36 27.88 0.0"
    stf = F.read_ad_src(os.path.join(str(tmp_path), "ad_src_2"), a.s.nt)
    assert np.allclose(stf[0], a.adsrc_x[::-1], rtol=1e-6, atol=1e-30)
    assert np.allclose(stf[2], a.adsrc_z[::-1], rtol=1e-6)
    assert np.allclose(F.read_ad_srcfile(os.path.join(str(tmp_path), "ad_srcfile")), loc)


def test_bandpass_is_zero_phase_and_band_limited():
    from scipy import signal
    dt, nt = 0.1, 4000
    t = np.arange(nt) * dt
    s = AS.Seismogram.from_traces(np.stack([np.sin(2 * np.pi * 0.05 * t), np.sin(2 * np.pi * 1.5 * t),
                                            np.exp(-((t - 200) / 3.0) ** 2)]), dt)
    s.bandpass(0.02, 0.1)
    mid = slice(1000, 3000)
    assert np.abs(s.trace_y[mid]).max() < 1e-3            # 1.5 Hz removed
    assert 0.5 < np.abs(s.trace_x[mid]).max() < 1.05       # 0.05 Hz passed
    pk = s.trace_z
    c = int(200 / dt)
    assert np.allclose(pk[c - 300:c], pk[c + 300:c:-1], atol=1e-6 * np.abs(pk).max())  # symmetric: zero phase
    sos = signal.butter(2, [0.02 / 5.0, 0.1 / 5.0], btype="band", output="sos")
    x = np.sin(2 * np.pi * 0.05 * t)
    ref = signal.sosfilt(sos, signal.sosfilt(sos, x)[::-1])[::-1]
    assert np.allclose(s.trace_x, ref, rtol=1e-9, atol=1e-12)


def test_cli_writes_adjoint_directory(tmp_path):
    from ses3d_gb300.__main__ import main
    nt, dt = 300, 0.1
    d = pulse(nt=nt, dt=dt, t0=12.0)
    ofd = str(tmp_path / "ofd") + "/"
    os.makedirs(ofd)
    for k, nm in enumerate(("ST1", "ST2")):
        F.write_seismograms(ofd, nm, d, 0.5 * d, (1 + k) * d, nt, np.float32(dt),
                            (np.float32(50.0 + k), np.float32(20.0), np.float32(0.0)),
                            (np.float32(45.0), np.float32(10.0), np.float32(15000.0)))
    out = str(tmp_path / "ADJOINT" / "1")
    assert main(["adjoint-sources", "--seismograms", ofd, "--out", out, "--kind", "cc", "--component", "z",
                 "--window", "5", "20", "--taper", "2", "--depth", "1000"]) == 0
    loc = F.read_ad_srcfile(os.path.join(out, "ad_srcfile"))
    assert loc.shape == (2, 3) and loc[1, 0] == np.float32(51.0) and loc[0, 2] == np.float32(1000.0)
    a = AS.AdjointSource()
    a.fetch_seismogram(AS.Seismogram().read(ofd, "ST2         "))
    a.make_adsrc_cc("z", 5.0, 20.0, 2.0)
    stf = F.read_ad_src(os.path.join(out, "ad_src_2"), nt)
    assert np.abs(stf[2]).max() > 0 and np.all(stf[:2] == 0)
    assert np.allclose(stf[2], a.adsrc_z[::-1], rtol=1e-6, atol=1e-6 * np.abs(a.adsrc_z).max())

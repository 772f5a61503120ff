"""Adjoint-source generation from SES3D seismogram files: the measurement-kernel adjoint
sources of the reference's TOOLS/adjoint_source.py and the seismogram reader of
TOOLS/seismograms.py, restated for Python 3 / numpy (the reference tools are Python 2 and
import matplotlib and obspy, neither of which is needed here).

Measurements (each returns the adjoint source time function in forward time, as the
reference computes it, and `write` stores it time-reversed in the ad_src_<k> format that
ses3d reads):

  make_adsrc_L2amp   L2 amplitude in a cosine-tapered window      (adjoint_source.py:323-398)
  make_adsrc_cc      cross-correlation time shift, same window     (adjoint_source.py:400-472)
  make_adsrc_mttime  multitaper time delay at one frequency        (adjoint_source.py:99-205)
  make_adsrc_mtamp   multitaper relative amplitude, one frequency  (adjoint_source.py:211-317)

The reference's developments assume displacement seismograms; for velocity seismograms
(`integrate=False`) the adjoint source is differentiated once more (-d/dt), with the
reference's index conventions kept as written.

Two Python-2 semantics the reference relies on are kept explicitly: `round` rounds halves
away from zero (Python 3 rounds them to even), and `str(float)` prints 12 significant
digits (used by `write`).

Prolate spheroidal sequences (Slepian 1978) follow TOOLS/prolate_spheroidal.py: the
tridiagonal commuting matrix, normalisation to unit energy on [-W, W], eigenvalues from
the sinc-kernel concentration, descending order.
"""
from __future__ import annotations

import math
import os
from typing import Optional, Tuple

import numpy as np


def round_half_away(x: float) -> float:
    """Python 2 `round`: halves go away from zero."""
    return math.copysign(math.floor(abs(x) + 0.5), x)


def py2_str(x: float) -> str:
    """Python 2 `str(float)`: 12 significant digits, shortest of %g's forms."""
    s = "%.12g" % float(x)
    if "e" not in s and "." not in s and "inf" not in s and "nan" not in s:
        s += ".0"
    return s


# ------------------------------------------------------------------------------------------------
# seismograms (TOOLS/seismograms.py:11-97)
# ------------------------------------------------------------------------------------------------

class Seismogram:
    """Three-component SES3D seismogram read from <directory><station>.{x,y,z}."""

    def __init__(self):
        self.nt, self.dt = 10, 1.0
        self.t = np.linspace(0, 10, 10)
        self.rx = self.ry = self.rz = 0.0
        self.sx = self.sy = self.sz = 0.0
        self.trace_x = np.zeros(10)
        self.trace_y = np.zeros(10)
        self.trace_z = np.zeros(10)
        self.integrate = False

    @staticmethod
    def _coords(line: str) -> Tuple[float, float, float]:
        # "x= <colat> y= <lon> z= <depth>" (TOOLS/seismograms.py:60-70)
        parts = line.strip().split("=")
        return float(parts[1].split("y")[0]), float(parts[2].split("z")[0]), float(parts[3])

    def read(self, directory: str, station: str, integrate: bool = False) -> "Seismogram":
        """Reads the three component files; with integrate=True the velocity traces are
        integrated to displacement by a cumulative sum times dt (TOOLS/seismograms.py:89-92)."""
        self.integrate = integrate
        comps = {}
        for c in "xyz":
            with open(os.path.join(directory, station + "." + c)) as f:
                lines = f.read().splitlines()
            comps[c] = lines
        lx = comps["x"]
        self.nt = int(lx[1].strip().split("=")[1])
        self.dt = float(lx[2].strip().split("=")[1])
        self.rx, self.ry, self.rz = self._coords(lx[4])
        self.sx, self.sy, self.sz = self._coords(lx[6])
        for c in "xyz":
            tr = np.array([float(v) for v in comps[c][7:7 + self.nt]], np.float64)
            if integrate:
                tr = np.cumsum(tr) * self.dt
            setattr(self, "trace_" + c, tr)
        # the reference's time axis: nt points from 0 to nt*dt (spacing nt dt / (nt - 1))
        self.t = np.linspace(0, self.nt * self.dt, self.nt)
        return self

    @classmethod
    def from_traces(cls, traces: np.ndarray, dt: float, receiver=(0.0, 0.0, 0.0), source=(0.0, 0.0, 0.0),
                    integrate: bool = False) -> "Seismogram":
        """A seismogram from in-memory (3, nt) traces (velocity unless integrate=True, in
        which case they are integrated like `read` does)."""
        s = cls()
        tr = np.asarray(traces, np.float64)
        s.nt, s.dt = tr.shape[1], float(dt)
        s.rx, s.ry, s.rz = (float(v) for v in receiver)
        s.sx, s.sy, s.sz = (float(v) for v in source)
        s.integrate = integrate
        for k, c in enumerate("xyz"):
            setattr(s, "trace_" + c, np.cumsum(tr[k]) * s.dt if integrate else tr[k].copy())
        s.t = np.linspace(0, s.nt * s.dt, s.nt)
        return s

    def bandpass(self, fmin: float, fmax: float):
        """Zero-phase band-pass of all traces (TOOLS/seismograms.py:140-154), which calls
        obspy.signal.filter.bandpass(corners=2, zerophase=True). obspy is not installed;
        its published algorithm is restated: a Butterworth band-pass of order `corners`
        designed in zero-pole-gain form on the normalised band [fmin, fmax] / (fs / 2),
        converted to second-order sections and applied forward, then again on the
        reversed output (no padding). As in obspy, an upper corner at or above Nyquist
        turns the filter into a high-pass."""
        from scipy import signal
        fe = 0.5 / self.dt
        low, high = fmin / fe, fmax / fe
        if high - 1.0 > -1e-6:
            z, p, k = signal.iirfilter(2, low, btype="highpass", ftype="butter", output="zpk")
        else:
            z, p, k = signal.iirfilter(2, [low, high], btype="bandpass", ftype="butter", output="zpk")
        sos = signal.zpk2sos(z, p, k)
        for c in "xyz":
            x = getattr(self, "trace_" + c)
            y = signal.sosfilt(sos, x)
            y = signal.sosfilt(sos, y[::-1])[::-1]
            setattr(self, "trace_" + c, y)


# ------------------------------------------------------------------------------------------------
# prolate spheroidal sequences (TOOLS/prolate_spheroidal.py:8-156)
# ------------------------------------------------------------------------------------------------

def ps_matrix(N: int, W: float) -> np.ndarray:
    """Tridiagonal matrix commuting with the time-and-band limiting operator."""
    i = np.arange(N, dtype=np.float64)
    S = np.diag(((0.5 * (N - 1) - i) ** 2) * math.cos(2 * math.pi * W))
    off = 0.5 * (i[1:]) * (N - i[1:])          # S[i, i-1] = i (N - i) / 2
    S[np.arange(1, N), np.arange(N - 1)] = off
    S[np.arange(N - 1), np.arange(1, N)] = off  # S[i, i+1] = (i+1)(N-i-1)/2
    return S


def ps_sequences(N: int, W: float) -> Tuple[np.ndarray, np.ndarray]:
    """Eigenvalues (concentrations, descending) and sequences c[:, k], each normalised so
    that its spectrum has unit energy on [-W, W]."""
    from scipy import linalg
    _, c = linalg.eig(ps_matrix(N, W))
    c = np.real(c)
    n = np.arange(N)
    K = np.sinc(2 * W * (n[:, None] - n[None, :]))          # sinc(2W (n - m))
    Kc = K @ c
    # the sequences far outside the band have concentrations below rounding: their
    # normalisation can be NaN, as in the reference; they sort last and are never used
    with np.errstate(invalid="ignore", divide="ignore"):
        const = np.sqrt(2 * W * np.einsum("nk,nk->k", c, Kc))
        eig = np.sum(np.abs(Kc) ** 2, axis=0)
        c = c / const
        eig = 4 * W * W * eig / const ** 2
    order = np.argsort(-eig, kind="stable")
    return eig[order], c[:, order]


def ps_frequency(N: int, W: float, k_max: int, nu: np.ndarray):
    """Frequency-domain prolate spheroidal wave functions Psi[:, k] at frequencies nu."""
    eig, c = ps_sequences(N, W)
    nu = np.asarray(nu, np.float64)
    n = np.arange(N)
    ph = np.exp(-2j * np.pi * n[None, :] * nu[:, None])      # (len(nu), N)
    Psi = (ph @ c[:, :k_max + 1]) * np.exp(1j * np.pi * (N - 1) * nu)[:, None]
    return eig[:k_max + 1], Psi


def ps_index(N: int, W: float, k_max: int, n: np.ndarray):
    """Index-domain prolate spheroidal sequences psi[:, k] at indices n (centred)."""
    eig, c = ps_sequences(N, W)
    n = np.asarray(n, np.float64)
    m = np.arange(N)
    A = 2 * W * np.sinc(W * (N - 1 - 2 * m[None, :] + 2 * n[:, None]))   # (len(n), N)
    return eig[:k_max + 1], (A @ c[:, :k_max + 1]).astype(complex)


# ------------------------------------------------------------------------------------------------
# adjoint sources (TOOLS/adjoint_source.py:12-472)
# ------------------------------------------------------------------------------------------------

class AdjointSource:
    """Adjoint source of one receiver: fetch a Seismogram, compute one of the make_adsrc_*
    measurements per component, write it in the ses3d ad_src format."""

    def __init__(self):
        self.s = Seismogram()
        self.adsrc_x = np.zeros(10)
        self.adsrc_y = np.zeros(10)
        self.adsrc_z = np.zeros(10)

    def fetch_seismogram(self, seismogram: Seismogram):
        self.s = seismogram
        self.adsrc_x = np.zeros(seismogram.nt)
        self.adsrc_y = np.zeros(seismogram.nt)
        self.adsrc_z = np.zeros(seismogram.nt)

    # -- helpers -------------------------------------------------------------------------------
    def _trace(self, component: str) -> np.ndarray:
        if component not in ("x", "y", "z"):
            raise ValueError("component must be 'x', 'y' or 'z'")
        return np.array(getattr(self.s, "trace_" + component), np.float64)

    def _set(self, component: str, a: np.ndarray):
        setattr(self, "adsrc_" + component, np.asarray(a, np.float64))

    def _window_taper(self, win_left: float, win_right: float, taper_width: float) -> np.ndarray:
        """Boxcar on (win_left, win_right) with cosine flanks (adjoint_source.py:346-360).
        The flanks are sampled on the first samples of the time axis (t <= taper_width) and
        placed at the window edges, as the reference does."""
        s = self.s
        N0 = int(round_half_away(win_left / s.dt))
        N = int(round_half_away(win_right / s.dt) - N0)
        taper = np.zeros(s.nt)
        taper[(s.t > win_left) & (s.t < win_right)] = 1.0
        tw = s.t[s.t <= taper_width]
        h = 0.5 * (1.0 - np.cos(np.pi * tw / taper_width))
        taper[N0:N0 + len(h)] = h
        h = 0.5 * (1.0 + np.cos(np.pi * tw / taper_width))
        taper[N0 + N - len(h):N0 + N] = h
        return taper

    def _velocity(self, a: np.ndarray) -> np.ndarray:
        """-d/dt for velocity seismograms (adjoint_source.py:383-385): forward differences,
        last sample zero."""
        if self.s.integrate:
            return a
        out = a.copy()
        out[:-1] = -np.diff(a) / self.s.dt
        out[-1] = 0.0
        return out

    # -- measurements --------------------------------------------------------------------------
    def make_adsrc_L2amp(self, component: str, win_left: float, win_right: float, taper_width: float):
        """L2 amplitude in a tapered window: 2 d / (sum d^2 dt) (adjoint_source.py:323-398)."""
        d = self._trace(component) * self._window_taper(win_left, win_right, taper_width)
        a = 2.0 * d / (np.sum(d * d) * self.s.dt)
        self._set(component, self._velocity(a))

    def make_adsrc_cc(self, component: str, win_left: float, win_right: float, taper_width: float):
        """Cross-correlation time shift: -d' / (sum d'^2 dt), d' the forward difference of
        the tapered trace (adjoint_source.py:400-472)."""
        d = self._trace(component) * self._window_taper(win_left, win_right, taper_width)
        d[:-1] = np.diff(d) / self.s.dt
        d[-1] = 0.0
        a = -d / (np.sum(d * d) * self.s.dt)
        self._set(component, self._velocity(a))

    def _multitaper(self, component: str, win_left: float, win_right: float, nu: float):
        s = self.s
        d = self._trace(component)
        N0 = int(round_half_away(win_left / s.dt))
        N = int(2 * round_half_away((round_half_away(win_right / s.dt) - N0) / 2.0) + 1)
        nu_n = nu * s.dt                       # normalised frequency
        k_max = 4                              # five tapers
        W = 3.0 * k_max / (2.0 * N)            # bandwidth
        eig, Psi = ps_frequency(N, W, k_max, np.arange(0, 1))
        eig, psi = ps_index(N, W, k_max, np.arange(-(N - 1) / 2, (N - 1) / 2 + 1))
        n = np.arange(N0, N0 + N)
        ph = np.exp(-2 * np.pi * 1j * n * nu_n)
        eta = np.array([np.sum(d[n] * psi[:, k] * ph) for k in range(k_max + 1)])
        u = 0.0 + 0.0j
        for k in range(k_max + 1):
            u = u + eta[k] * Psi[0, k] / eig[k]
        a = np.zeros(s.nt, dtype=complex)
        for k in range(k_max + 1):
            a[n] = a[n] + Psi[0, k] * psi[:, k] * ph / eig[k]
        return a, u, N0, N, nu_n

    def _mt_velocity(self, a: np.ndarray, N0: int, N: int) -> np.ndarray:
        """-d/dt inside the window for velocity seismograms (adjoint_source.py:189-191):
        samples N0 .. N0+N-2 get the forward difference, sample N0+N is zeroed."""
        if self.s.integrate:
            return a
        a = a.copy()
        a[N0:N0 + N - 1] = -np.diff(a[N0:N0 + N]) / self.s.dt
        a[N0 + N] = 0.0
        return a

    def make_adsrc_mttime(self, component: str, win_left: float, win_right: float, nu: float):
        """Multitaper time delay at frequency nu [Hz] (adjoint_source.py:99-205)."""
        a, u, N0, N, nu_n = self._multitaper(component, win_left, win_right, nu)
        a = a / (2 * np.pi * self.s.dt * nu_n * u)
        self._set(component, np.imag(self._mt_velocity(a, N0, N)))

    def make_adsrc_mtamp(self, component: str, win_left: float, win_right: float, nu: float):
        """Multitaper relative amplitude at frequency nu [Hz] (adjoint_source.py:211-317)."""
        a, u, N0, N, _ = self._multitaper(component, win_left, win_right, nu)
        a = a / (self.s.dt * u)
        self._set(component, np.real(self._mt_velocity(a, N0, N)))

    # -- output --------------------------------------------------------------------------------
    def reversed_stf(self) -> np.ndarray:
        """(3, nt) in adjoint-iteration order (time-reversed), as `write` stores it."""
        return np.stack([self.adsrc_x[::-1], self.adsrc_y[::-1], self.adsrc_z[::-1]])

    def write(self, directory: str, filename: str):
        """ad_src file: 4 header lines with the receiver coordinates, then (x, y, z) from the
        last sample to the first (adjoint_source.py:76-92)."""
        lines = ["-- adjoint source ------------------", "-- source coordinates (colat,lon,depth)",
                 "%s %s %s" % (py2_str(self.s.rx), py2_str(self.s.ry), py2_str(self.s.rz)),
                 "-- source time function (x, y, z) --"]
        for k in range(self.s.nt - 1, -1, -1):
            lines.append("%s %s %s" % (py2_str(self.adsrc_x[k]), py2_str(self.adsrc_y[k]), py2_str(self.adsrc_z[k])))
        with open(os.path.join(directory, filename), "w") as f:
            f.write("\n".join(lines) + "\n")


def write_adjoint_directory(directory: str, sources, depth: Optional[float] = None):
    """Writes ad_srcfile and ad_src_1..n for a list of AdjointSource objects (the layout
    ses3d reads from ADJOINT/<event>/, SOURCE/ses3d_input.f90:584-618). The ad_srcfile
    lists each receiver's colatitude, longitude and depth (depth overridden if given)."""
    from . import formats as F
    os.makedirs(directory, exist_ok=True)
    loc = np.array([[a.s.rx, a.s.ry, a.s.rz if depth is None else depth] for a in sources], np.float32)
    F.write_ad_srcfile(os.path.join(directory, "ad_srcfile"), loc)
    for k, a in enumerate(sources):
        a.write(directory, "ad_src_%d" % (k + 1))
    return loc

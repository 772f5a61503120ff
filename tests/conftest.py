import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def native():
    """The built native library (built on first use)."""
    from ses3d_gb300 import build
    build.build()
    from ses3d_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


def _wave_energy(field, setup_real, p):
    """Kinetic plus elastic strain energy of an isotropic wavefield, in FP64: 1/2 sum of
    M |v|^2 over the global nodes (M = -MM, the reference's mass matrix is negative) plus
    1/2 sum of W sigma : C^-1 sigma over the GLL points, W = w_i w_j w_k Jac r^2 sin(theta),
    with sigma the element stress state (sxx_pml ... syz_pml). field / setup_real read
    arrays by the reference's names (Oracle.get, or Simulation.field / setup_real)."""
    import numpy as np
    ex, ey, ez = p.nx + 1, p.ny + 1, p.nz + 1
    f = lambda name: np.asarray(field(name), np.float64)
    w = np.asarray(setup_real("w"), np.float64)
    jac = float(np.asarray(setup_real("Jac"))[0])
    x = np.asarray(setup_real("x"), np.float64).reshape(5, ex)
    z = np.asarray(setup_real("z"), np.float64).reshape(5, ez)
    W = np.empty((5, 5, 5, ez, ey, ex))
    for kn in range(5):
        for jn in range(5):
            for i_ in range(5):
                W[kn, jn, i_] = (w[i_] * w[jn] * w[kn] * jac) * (z[kn] ** 2)[:, None, None] * np.sin(x[i_])[None, None, :]
    W = W.reshape(-1)
    kinetic = 0.5 * np.sum(-f("MM_global") * (f("vx_global") ** 2 + f("vy_global") ** 2 + f("vz_global") ** 2))
    s = {c: f("s%s_pml" % c) for c in ("xx", "yy", "zz", "xy", "xz", "yz")}
    mu = p.model["mu"].astype(np.float64)
    lam = p.model["lambda"].astype(np.float64)
    tr = s["xx"] + s["yy"] + s["zz"]
    ss = s["xx"] ** 2 + s["yy"] ** 2 + s["zz"] ** 2 + 2 * (s["xy"] ** 2 + s["xz"] ** 2 + s["yz"] ** 2)
    strain = 0.5 * np.sum(W * (ss - lam / (3 * lam + 2 * mu) * tr ** 2) / (2 * mu))
    return kinetic + strain


@pytest.fixture(scope="session")
def wave_energy():
    return _wave_energy

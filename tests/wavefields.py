"""Seeded random wavefields for tests that start the GPU path and the oracle from the same
state instead of at rest (not collected by pytest: imported by the test modules)."""
import numpy as np

STRESS = ("sxx_pml", "syy_pml", "szz_pml", "sxy_pml", "sxz_pml", "syz_pml")
MIRROR = {"syx_pml": "sxy_pml", "szx_pml": "sxz_pml", "szy_pml": "syz_pml"}
GRADS = ("dxux", "dyuy", "dzuz", "dxuy", "dyux", "dxuz", "dzux", "dyuz", "dzuy")
MEMVARS = ("Mxx", "Myy", "Mzz", "Mxy", "Mxz", "Myz")
VELOCITY = ("vx_global", "vy_global", "vz_global")


def _smooth_global(rng, ex, ey, ez):
    """Random field on the global nodes that is linear between element corners: independent
    normal values at the (ex+1)(ey+1)(ez+1) corners, interpolated along each axis."""
    f = rng.standard_normal((ez + 1, ey + 1, ex + 1)).astype(np.float32)
    for axis, ne in ((2, ex), (1, ey), (0, ez)):
        t = np.arange(4 * ne + 1) / np.float32(4.0)
        i0 = np.minimum(t.astype(np.int64), ne - 1)
        w = (t - i0).astype(np.float32)
        shape = [1, 1, 1]
        shape[axis] = -1
        w = w.reshape(shape)
        f = np.take(f, i0, axis=axis) * (1 - w) + np.take(f, i0 + 1, axis=axis) * w
    return f.reshape(-1)


def random_state(p, seed, is_diss=1):
    """Seeded random wavefield in the reference layout (field name -> FP32 array). Velocity,
    stresses and displacement gradients are smooth random fields (linear between element
    corners, sampled at the GLL nodes) plus 1 % white noise; memory variables are white
    noise. Every value differs from its neighbours, so a wrong index changes the result far
    beyond the tolerances, while the wavefield stays smooth enough that the rounding of the
    receiver coordinates (FP32 against FP64 set-up) stays below the seismogram tolerance."""
    rng = np.random.default_rng(seed)
    ex, ey, ez = p.nx + 1, p.ny + 1, p.nz + 1
    G = (4 * ex + 1) * (4 * ey + 1) * (4 * ez + 1)
    N = p.n_nodes
    E = ex * ey * ez
    q = np.arange(N, dtype=np.int64)
    e, n = q % E, q // E
    i, j, k = e % ex, (e // ex) % ey, e // (ex * ey)
    gi = (4 * i + n % 5) + (4 * ex + 1) * ((4 * j + (n // 5) % 5) + (4 * ey + 1) * (4 * k + n // 25))
    del q, e, n, i, j, k

    def noisy(a, scale):
        a = a + np.float32(0.01) * rng.standard_normal(a.size, dtype=np.float32)
        a *= np.float32(scale)
        return a

    st = {key: noisy(_smooth_global(rng, ex, ey, ez), 1.0) for key in VELOCITY}
    assert st["vx_global"].size == G
    for key in STRESS:
        st[key] = noisy(_smooth_global(rng, ex, ey, ez)[gi], 1e6)
    st.update({key: st[v] for key, v in MIRROR.items()})
    for key in GRADS:
        st[key] = noisy(_smooth_global(rng, ex, ey, ez)[gi], 1e-4)
    if is_diss:
        for key in MEMVARS:
            a = rng.standard_normal(3 * N, dtype=np.float32)
            a *= np.float32(1e-5)
            st[key] = a
    return st

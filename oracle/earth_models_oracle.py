"""CPU restatement of the reference's built-in 1-D Earth models (TEST INFRASTRUCTURE ONLY).

Statement by statement, in FP32 scalar arithmetic, for one processor box's radii
z(0:nz, 0:lpd):
  MODELS/MODELS_1D/prem_iso.f90:30-232            (model_type 2)
  MODELS/MODELS_1D/homogeneous_plus_Q.f90:10-88   (model_type 3)
  MODELS/MODELS_1D/eumod_bg.f90:30-221            (model_type 4)
  MODELS/MODELS_1D/ak135.f90:94-153               (model_type 7; the table is passed in)
Each returns the 1-D arrays (rho1d, cp1d, cs1d, Q1d) in SI units as the routines hold them
just before they fill the 3-D records, and records() fills those as the routines do. It
is the checker of ses3d_gb300.earth_models / models.builtin_model; only tests/ import it.
Integer powers r**p are taken as a Fortran compiler expands them (repeated squaring).
Parity with the reference is unpinned by the reference's own tests (it ships no generated
model records and cannot be compiled here).
"""
import numpy as np

f32 = np.float32


def _pow(r, p):
    r2 = r * r
    return {2: r2, 3: r2 * r, 4: r2 * r2, 5: (r2 * r2) * r}[p]


def ql6(z, is_diss):
    """homogeneous_plus_Q.f90:38-74 / eumod_bg.f90:140-172 (smooth QL6)."""
    nz, L = z.shape
    Q1d = np.zeros((nz, L), f32)
    r = (f32(6371.0) - z / f32(1000.0)) / f32(271.0)
    for i in range(nz):
        for k in range(L):
            zz, rr = z[i, k], r[i, k]
            if not is_diss:
                Q1d[i, k] = f32(100000.0)
            elif zz <= f32(6371000.0) and zz >= f32(6100000.0):
                Q1d[i, k] = (f32(300.0) - f32(5370.82) * _pow(rr, 2) + f32(14401.62) * _pow(rr, 3)
                             - f32(13365.78) * _pow(rr, 4) + f32(4199.98) * _pow(rr, 5))
            elif zz <= f32(6100000.0) and zz >= f32(5701000.0):
                Q1d[i, k] = f32(165.0)
            elif zz <= f32(5701000.0) and zz >= f32(3480000.0):
                Q1d[i, k] = f32(355.0)
            elif zz <= f32(3480000.0) and zz >= f32(1221000.0):
                Q1d[i, k] = f32(0.0)
            else:
                Q1d[i, k] = f32(104.0)
    return Q1d


def _mantle_core(zz, r, eumod):
    """The layers below 24.4 km of prem_iso.f90:54-124 (eumod False) or eumod_bg.f90:54-133
    (eumod True): (rho, cp, cs) in g/cm^3, km/s; None outside every layer."""
    a, b = f32(0.035), f32(0.065)
    c = f32(0.12)
    if zz <= f32(6346600.0) and zz >= f32(6291000.0):
        rho = f32(2.6910) + f32(0.6924) * r
        cp = f32(4.1875) + f32(3.9382) * r
        cs = f32(2.1519) + f32(2.3481) * r
        return (rho, cp - a, cs - b) if eumod else (rho, cp, cs)
    if not eumod and zz <= f32(6291000.0) and zz >= f32(6151000.0):
        return (f32(2.6910) + f32(0.6924) * r, f32(4.1875) + f32(3.9382) * r, f32(2.1519) + f32(2.3481) * r)
    if not eumod and zz <= f32(6151000.0) and zz >= f32(5971000.0):
        return (f32(7.1089) - f32(3.8045) * r, f32(20.3926) - f32(12.2569) * r, f32(8.9496) - f32(4.4597) * r)
    if eumod and zz <= f32(6291000.0) and zz >= f32(6191000.0):
        return (f32(2.6910) + f32(0.6924) * r, f32(4.1875) + f32(3.9382) * r - a, f32(2.1519) + f32(2.3481) * r - b)
    if eumod and zz <= f32(6191000.0) and zz >= f32(6051000.0):
        return (f32(9.1790) - f32(5.9841) * r, f32(40.5988) - f32(33.5317) * r - a,
                f32(16.8261) - f32(12.7527) * r - b)
    if eumod and zz <= f32(6051000.0) and zz >= f32(5971000.0):
        return (f32(7.1089) - f32(3.8045) * r, f32(20.3926) - f32(12.2569) * r - a, f32(8.9496) - f32(4.4597) * r - b)
    if zz <= f32(5971000.0) and zz >= f32(5771000.0):
        cs = f32(22.3512) - f32(18.5856) * r
        return (f32(11.2494) - f32(8.0298) * r, f32(39.7027) - f32(32.6166) * r - (a if eumod else f32(0)),
                cs - c if eumod else cs)
    if zz <= f32(5771000.0) and zz >= f32(5701000.0):
        cs = f32(9.9839) - f32(4.9324) * r
        return (f32(5.3197) - f32(1.4836) * r, f32(19.0957) - f32(9.8672) * r - (a if eumod else f32(0)),
                cs - c if eumod else cs)
    rho_lm = f32(7.9565) - f32(6.4761) * r + f32(5.5283) * r * r - f32(3.0807) * r * r * r
    if zz <= f32(5701000.0) and zz >= f32(5600000.0):
        cs = f32(22.3459) - f32(17.2473) * r - f32(2.0834) * r * r + f32(0.9783) * r * r * r
        return (rho_lm, f32(29.2766) - f32(23.6026) * r + f32(5.5242) * r * r - f32(2.5514) * r * r * r,
                cs - c if eumod else cs)
    if zz <= f32(5600000.0) and zz >= f32(3630000.0):
        cs = f32(11.1671) - f32(13.7818) * r + f32(17.4575) * r * r - f32(9.2777) * r * r * r
        return (rho_lm, f32(24.9520) - f32(40.4673) * r + f32(51.4832) * r * r - f32(26.6419) * r * r * r,
                cs - c if eumod else cs)
    if zz <= f32(3630000.0) and zz >= f32(3480000.0):
        cs = f32(6.9254) + f32(1.4672) * r - f32(2.0834) * r * r + f32(0.9783) * r * r * r
        return (rho_lm, f32(15.3891) - f32(5.3181) * r + f32(5.5242) * r * r - f32(2.5514) * r * r * r,
                cs - c if eumod else cs)
    if zz <= f32(3480000.0) and zz >= f32(1221500.0):
        return (f32(12.5815) - f32(1.2638) * r - f32(3.6426) * r * r - f32(5.5281) * r * r * r,
                f32(11.0487) - f32(4.0362) * r + f32(4.8023) * r * r - f32(13.5732) * r * r * r, f32(0.0))
    if zz <= f32(1221500.0):
        return (f32(13.0885) - f32(8.8381) * r * r, f32(11.2622) - f32(6.3640) * r * r,
                f32(3.6678) - f32(4.4475) * r * r)
    return None


def _crust(zz):
    if zz <= f32(6371000.0) and zz >= f32(6356000.0):
        return f32(2.60), f32(5.80), f32(3.20)
    if zz <= f32(6356000.0) and zz >= f32(6346600.0):
        return f32(2.90), f32(6.80), f32(3.90)
    return None


def _prem_q(zz):
    for top, bot, q in ((6371000.0, 6356000.0, 600.0), (6356000.0, 6346600.0, 600.0), (6346600.0, 6291000.0, 600.0),
                        (6291000.0, 6151000.0, 80.0), (6151000.0, 5971000.0, 143.0), (5971000.0, 5771000.0, 143.0),
                        (5771000.0, 5701000.0, 143.0), (5701000.0, 5600000.0, 312.0), (5600000.0, 3630000.0, 312.0),
                        (3630000.0, 3480000.0, 312.0), (3480000.0, 1221500.0, 100000.0)):
        if zz <= f32(top) and zz >= f32(bot):
            return f32(q)
    if zz <= f32(1221500.0):
        return f32(84.6)
    return f32(0.0)


def prem_iso(z, is_diss):
    z = np.asarray(z, f32)
    nz, L = z.shape
    rho1d, cp1d, cs1d, Q1d = (np.zeros((nz, L), f32) for _ in range(4))
    r = z / f32(6371e3)
    for i in range(nz):
        for k in range(L):
            v = _crust(z[i, k]) or _mantle_core(z[i, k], r[i, k], False)
            if v is not None:
                rho1d[i, k], cp1d[i, k], cs1d[i, k] = v
            Q1d[i, k] = _prem_q(z[i, k]) if is_diss else f32(100000.0)
    return f32(1000.0) * rho1d, f32(1000.0) * cp1d, f32(1000.0) * cs1d, Q1d


def eumod_bg(z, is_diss):
    z = np.asarray(z, f32)
    nz, L = z.shape
    rho1d, cp1d, cs1d = (np.zeros((nz, L), f32) for _ in range(3))
    r = z / f32(6371e3)
    for i in range(nz):
        for k in range(L):
            v = _crust(z[i, k]) or _mantle_core(z[i, k], r[i, k], True)
            if v is not None:
                rho1d[i, k], cp1d[i, k], cs1d[i, k] = v
    Q1d = ql6(z, is_diss)
    if z[0, 0] == f32(6371000.0):          # eumod_bg.f90:178-185
        rho1d[0, :] = f32(3.00)
        cp1d[0, :] = f32(7.20)
        cs1d[0, :] = f32(4.10)
    return f32(1000.0) * rho1d, f32(1000.0) * cp1d, f32(1000.0) * cs1d, Q1d


def ak135(z, table, is_diss):
    """table: (139, 4) radius [km], rho, vp, vs as the routine tabulates them."""
    z = np.asarray(z, f32)
    nz, L = z.shape
    ak_r = f32(1000) * np.asarray(table[:, 0], f32)
    ak_rho = f32(1000) * np.asarray(table[:, 1], f32)
    ak_cp = f32(1000) * np.asarray(table[:, 2], f32)
    ak_cs = f32(1000) * np.asarray(table[:, 3], f32)
    rho1d, cp1d, cs1d = (np.zeros((nz, L), f32) for _ in range(3))
    for i in range(nz):
        for k in range(L):
            for n in range(138):             # do n=1,138 (0-based here)
                if z[i, k] >= ak_r[n + 1] and z[i, k] <= ak_r[n]:
                    if ak_r[n] - ak_r[n + 1] == 0:
                        cp1d[i, k], cs1d[i, k], rho1d[i, k] = ak_cp[n], ak_cs[n], ak_rho[n]
                    else:
                        ratio = (ak_r[n] - z[i, k]) / (ak_r[n] - ak_r[n + 1])
                        cp1d[i, k] = ak_cp[n] * (f32(1) - ratio) + ak_cp[n + 1] * ratio
                        cs1d[i, k] = ak_cs[n] * (f32(1) - ratio) + ak_cs[n + 1] * ratio
                        rho1d[i, k] = ak_rho[n] * (f32(1) - ratio) + ak_rho[n + 1] * ratio
    return rho1d, cp1d, cs1d, np.full((nz, L), f32(100000.0), f32)


def records(rho1d, cp1d, cs1d, Q1d, ex, ey, is_diss):
    """rhoinv(:,:,i,:,:,k) = 1/rho1d(i,k), mu = cs cs rho, lambda = (cp cp - 2 cs cs) rho,
    Q, A = B = C = 0, in the reference layout (i, j, k, in, jn, kn), i fastest."""
    nz = rho1d.shape[0]
    out = {}
    one = {"rhoinv": f32(1) / rho1d, "mu": cs1d * cs1d * rho1d,
           "lambda": (cp1d * cp1d - f32(2) * cs1d * cs1d) * rho1d}
    if is_diss:
        one["Q"] = Q1d
    for name, a in one.items():
        full = np.zeros((5, 5, 5, nz, ey, ex), f32)   # (kn, jn, in, k, j, i)
        for k in range(nz):
            for kn in range(5):
                full[kn, :, :, k, :, :] = a[k, kn]
        out[name] = full.reshape(-1)
    for name in ("A", "B", "C"):
        out[name] = np.zeros(125 * ex * ey * nz, f32)
    return out

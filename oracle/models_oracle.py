"""CPU restatement of MODELS/SOURCE/add_perturbation.f90:327-534 (TEST INFRASTRUCTURE ONLY).

A literal transcription of the reference's array statements for one processor box, in
FP32 numpy: velocities from the model records, then for every subvolume and every cell
in the start..end ranges a whole-array `where` on the cell's half-open bounds adding the
cell's perturbations, then the moduli recomputed. It is the checker of
ses3d_gb300.models.add_perturbation; only tests/ import it. Parity with the reference is
unpinned by the reference's own tests (the reference ships no dv* perturbation files and
cannot be compiled here).
"""
import numpy as np

f32 = np.float32


def add_perturbation(rhoinv, mu, lam, B, cox, coy, coz, box, subvols):
    """cox/coy/coz: FP32 coordinates of every GLL point (radians, radians, m) in the
    reference layout; box: (xmin, xmax, ymin, ymax, zmin, zmax) FP32; subvols: list of
    (bx_deg, by_deg, bz_km, dvsh, dvsv, dvp, drho) with the value arrays shaped
    (nbx-1, nby-1, nbz-1). Returns (rhoinv, mu, lambda, B)."""
    pi = f32(3.1415926535898)                                    # SOURCE/ses3d_modules.f90:25
    csh = np.sqrt(mu * rhoinv)                                   # add_perturbation.f90:331
    csv = np.sqrt((mu + B) * rhoinv)                             # :332
    cp = np.sqrt((lam + f32(2) * mu) * rhoinv)                   # :333
    rho = f32(1) / rhoinv                                        # :334
    xmin, xmax, ymin, ymax, zmin, zmax = box
    for bx_deg, by_deg, bz_km, d_sh, d_sv, d_a, d_r in subvols:  # :374
        bx = np.array([f32(v) * pi / f32(180) for v in bx_deg], f32)   # :389-392
        by = np.array([f32(v) * pi / f32(180) for v in by_deg], f32)
        bz = np.array([f32(v) * f32(1000) for v in bz_km], f32)
        d_beta_sh = f32(1000) * d_sh                             # :420-423
        d_beta_sv = f32(1000) * d_sv
        d_alpha = f32(1000) * d_a
        d_rho = f32(1000) * d_r
        nbx, nby, nbz = len(bx), len(by), len(bz)
        start_x, start_y, start_z, end_x, end_y, end_z = 1, 1, 1, nbx - 1, nby - 1, nbz - 1
        for i in range(1, nbx):                                  # :433-462
            if bx[i - 1] < xmin:
                start_x = i
        for i in range(nbx - 1, 0, -1):
            if bx[i - 1] > xmax:
                end_x = i
        for i in range(1, nby):
            if by[i - 1] < ymin:
                start_y = i
        for i in range(nby - 1, 0, -1):
            if by[i - 1] > ymax:
                end_y = i
        for i in range(1, nbz):
            if bz[i - 1] < zmin:
                start_z = i
        for i in range(nbz - 1, 0, -1):
            if bz[i - 1] > zmax:
                end_z = i
        for i in range(start_x, end_x + 1):                      # :464-481
            for j in range(start_y, end_y + 1):
                for k in range(start_z, end_z + 1):
                    m = ((cox >= bx[i - 1]) & (cox < bx[i]) & (coy >= by[j - 1]) & (coy < by[j]) &
                         (coz > bz[k - 1]) & (coz <= bz[k]))
                    csv = np.where(m, csv + d_beta_sv[i - 1, j - 1, k - 1], csv)
                    csh = np.where(m, csh + d_beta_sh[i - 1, j - 1, k - 1], csh)
                    cp = np.where(m, cp + d_alpha[i - 1, j - 1, k - 1], cp)
                    rho = np.where(m, rho + d_rho[i - 1, j - 1, k - 1], rho)
    mu2 = rho * csh * csh                                        # :508-510
    B2 = rho * csv * csv - mu2
    lam2 = rho * cp * cp - f32(2) * mu2
    return (f32(1) / rho).astype(f32), mu2.astype(f32), lam2.astype(f32), B2.astype(f32)

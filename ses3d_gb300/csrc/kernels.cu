// kernels.cu -- sm_103a kernels of the SES3D time step.
//
// One iteration of SOURCE/ses3d_evolution.f90 is three launches (four with point forces):
//   k_receivers  record_seismograms on the pre-update velocity (ses3d_output.f90:456-497)
//   k_element    everything element-local (k_element_tma: persistent, bulk-copy staged;
//                k_element: register-staged, record and adjoint iterations): gather,
//                strain rates, spherical terms,
//                displacement gradients, PML strain, stress rates, memory variables,
//                PML stress march, moment source, weak divergence, taper
//                (ses3d_evolution.f90:27-271,334-360,368-371; ses3d_miscellaneous.f90:97-150)
//   k_inject     single-force / adjoint forces into the element forces (ses3d_miscellaneous.f90:11-94)
//   k_node       deterministic assembly, mass matrix, leapfrog, taper (ses3d_evolution.f90:282-328,366)
// The MPI face exchange of the reference (ses3d_miscellaneous.f90:257-368) becomes the
// node-centric gather of k_node: each global node sums its (up to 8) element
// contributions in the reference loop order, without atomics, so runs are bit-reproducible.
#include "kernels.cuh"
#include "assembly.cuh"
#include "pipeline.cuh"

// Minimum resident CTAs per SM requested from ptxas for k_element (register cap).
#ifndef SES3D_ELEM_MINB
#define SES3D_ELEM_MINB 6
#endif
// Threads per k_node CTA and the minimum resident CTAs per SM requested from ptxas.
#ifndef SES3D_NODE_TPB
#define SES3D_NODE_TPB 256
#endif
#ifndef SES3D_NODE_MINB
#define SES3D_NODE_MINB 7
#endif
#ifndef SES3D_NODE_MAGIC
#define SES3D_NODE_MAGIC 1
#endif

namespace ses3d {

// ---------------------------------------------------------------------------------------
// Per-node work of one element after its velocities are in shared memory: strain rates,
// spherical terms, displacement gradients, PML strain, stress rates, memory variables,
// PML stress march, moment source, taper, record/kernel epilogues, weak divergence and the
// element forces. Shared by both element kernels (one barrier inside).
// ---------------------------------------------------------------------------------------
struct ElemCtx {
  bool act, full;
  int n, nn, in, jn, kn, ii, j, k, ev;
  unsigned e;
  size_t N, m0;
  float *S;  // this node's state in global memory: field f at S[f * 125]
  float vx, vy, vz, clam, c2mut, c2mt, cA, cB2, cC;
  const float *lt;  // this element's 1-D table entries in shared memory (LT_*), or null
  // Correlation operands staged in shared memory by cp.async (persistent kernel), or null:
  // [CS_FLOATS][TPE] floats (record, adjoint model), then [NGRAD][TPE] doubles (kernels).
  float *cstage;
  bool cstage_more;       // a later cp.async group (the next item's velocity) is in flight
  long long cstage_next;  // item whose operands to stage once these are consumed, or -1
  // Displacement at this item's nodes staged in shared memory ([3][TPE]; lean record and
  // correlation items outside the PML), or null.
  const float *su;
};

// Correlation operands per point: the NREC record fields, then rho, cp, cs.
constexpr int CS_FLOATS = 12;
constexpr size_t CS_BYTES = CS_FLOATS * 128 * sizeof(float) + 8 * 128 * sizeof(double);

// Per-element copy of the 1-D tables (five entries per axis) and the event's source
// element, prefetched into shared memory by the persistent element kernel.
enum { LT_SIN = 0, LT_COT = 5, LT_ISIN = 10, LT_PX = 15, LT_PY = 20, LT_R = 25, LT_IR = 30, LT_PZ = 35,
       LT_SRC = 40, LT_FLOATS = 48 };

// Element forces: component c of node n of element e at 375 e + 125 c + n of its event.
__device__ __forceinline__ unsigned force_offset(const Consts &c, int i, int j, int k, int in, int jn, int kn) {
  return ((unsigned)i + (unsigned)c.ex * ((unsigned)j + (unsigned)c.ey * (unsigned)k)) * 375u +
         (unsigned)(in + 5 * jn + 25 * kn);
}

// Element-kernel modes: 0 plain, 1 forward record, 2 kernel correlation, in full state; 3,
// 4, 5 the same lean: outside the PML neither displacement gradients nor mirror stresses
// are kept, and record and correlation iterations there take the displacement gradients
// from the displacement field u (both are the time integral of the same linear map of v).
__host__ __device__ constexpr bool lean_mode(int m) { return m >= 3; }
__host__ __device__ constexpr bool record_mode(int m) { return m == 1 || m == 4; }
__host__ __device__ constexpr bool corr_mode(int m) { return m == 2 || m == 5; }

struct NoHook {
  __device__ void operator()() const {}
};

__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}

// Stages one point's correlation operands of `item` (thread nn of its element) into cs, as
// one cp.async group: the forward record, the adjoint-model fields, the FP64 kernels.
template <bool DISS>
__device__ __forceinline__ void stage_corr(const Consts &c, const Ptrs &p, long long item, int nn, float *cs) {
  const int ev = (int)(item % c.nev);
  const size_t N = (size_t)c.N, m0 = (size_t)(item / c.nev) * 125 + nn;
  const float *R = p.rec + (size_t)ev * NREC * N + m0;
#pragma unroll
  for (int f = 0; f < NREC; ++f) cp_async4(cs + f * TPE + nn, R + f * N);
  cp_async4(cs + 9 * TPE + nn, p.gmat + G_RHO * N + m0);
  cp_async4(cs + 10 * TPE + nn, p.gmat + G_CP * N + m0);
  cp_async4(cs + 11 * TPE + nn, p.gmat + G_CS * N + m0);
  double *cd = reinterpret_cast<double *>(cs + CS_FLOATS * TPE) + nn;
  const double *GR = p.grad + (size_t)ev * NGRAD * N + m0;
  const int nk = (DISS && p.grad_q) ? 8 : 4;
  for (int q = 0; q < nk; ++q) cp_async8(cd + q * TPE, GR + q * N);
  asm volatile("cp.async.commit_group;" ::: "memory");
}

// after_barrier() runs on every thread right after the barrier between the stress and
// divergence phases (the persistent kernel issues its next bulk copies there).
template <bool DISS, int MODE, class Hook = NoHook>
__device__ __forceinline__ void element_compute(const Consts &c, const Ptrs &p, const KTab &tab, float (*s_v)[TPE],
                                                float (*s_p)[TPE], const ElemCtx &x, float *sv,
                                                const Hook &after_barrier = Hook()) {
  constexpr int NS = DISS ? NSTATE : 18;
  const bool act = x.act, full = x.full;
  const int n = x.n, nn = x.nn, in = x.in, jn = x.jn, kn = x.kn, ii = x.ii, j = x.j, k = x.k, ev = x.ev;
  const unsigned e = x.e;
  const size_t N = x.N, m0 = x.m0;
  float *S = x.S;
  const float vx = x.vx, vy = x.vy, vz = x.vz;
  const float clam = x.clam, c2mut = x.c2mut, c2mt = x.c2mt, cA = x.cA, cB2 = x.cB2, cC = x.cC;
  (void)j;
  // Record or correlation iteration, lean, outside the PML: the displacement gradients at the
  // end of the iteration are the strain-rate proxies (ses3d_evolution.f90:57-103) of the
  // displacement u + dt v, by the same contraction through shared memory (s_p is free until
  // the stress phase); every thread of the CTA takes part (one item per CTA in these modes).
  float du[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if constexpr (MODE == 4 || MODE == 5) {
    if (!full) {
      const float dtu = c.dt;
      float ux = 0.f, uy = 0.f, uz = 0.f;
      if (act) {
        float u0, u1, u2;
        if (x.su) {
          u0 = x.su[n]; u1 = x.su[TPE + n]; u2 = x.su[2 * TPE + n];
        } else {
          const size_t g =
              (size_t)(ii * 4 + in) + (size_t)c.GX * ((size_t)(j * 4 + jn) + (size_t)c.GY * (size_t)(k * 4 + kn));
          const float *U = p.u + (size_t)ev * 3 * c.G + g;
          u0 = U[0]; u1 = U[c.G]; u2 = U[2 * c.G];
        }
        ux = __fadd_rn(u0, __fmul_rn(dtu, vx));
        uy = __fadd_rn(u1, __fmul_rn(dtu, vy));
        uz = __fadd_rn(u2, __fmul_rn(dtu, vz));
      }
      s_p[0][n] = ux; s_p[1][n] = uy; s_p[2][n] = uz;
      __syncthreads();
      if (act) {
        float dxx = 0.f, dxy = 0.f, dxz = 0.f, dyx = 0.f, dyy = 0.f, dyz = 0.f, dzx = 0.f, dzy = 0.f, dzz = 0.f;
#pragma unroll
        for (int q = 0; q < 5; ++q) {
          const int ix = q + 5 * jn + 25 * kn, iy = in + 5 * q + 25 * kn, iz = in + 5 * jn + 25 * q;
          const float dxq = tab.Dx[in][q], dyq = tab.Dy[jn][q], dzq = tab.Dz[kn][q];
          dxx = fmaf(s_p[0][ix], dxq, dxx); dxy = fmaf(s_p[1][ix], dxq, dxy); dxz = fmaf(s_p[2][ix], dxq, dxz);
          dyx = fmaf(s_p[0][iy], dyq, dyx); dyy = fmaf(s_p[1][iy], dyq, dyy); dyz = fmaf(s_p[2][iy], dyq, dyz);
          dzx = fmaf(s_p[0][iz], dzq, dzx); dzy = fmaf(s_p[1][iz], dzq, dzy); dzz = fmaf(s_p[2][iz], dzq, dzz);
        }
        const float *lt0 = x.lt;
        const float ir0 = lt0 ? lt0[LT_IR + kn] : __ldg(p.inv_r + k * 5 + kn);
        const float irs0 = ir0 * (lt0 ? lt0[LT_ISIN + in] : __ldg(p.inv_sin + ii * 5 + in));
        const float ct0 = lt0 ? lt0[LT_COT + in] : __ldg(p.cot_x + ii * 5 + in);
        du[0] = (uz + dxx) * ir0;                  // dxux
        du[1] = dyy * irs0 + (uz + ux * ct0) * ir0;  // dyuy
        du[2] = -dzz;                              // dzuz
        du[3] = dxy * ir0;                         // dxuy
        du[4] = -uy * ct0 * ir0 + dyx * irs0;      // dyux
        du[5] = (dxz - ux) * ir0;                  // dxuz
        du[6] = -dzx;                              // dzux
        du[7] = -uy * ir0 + dyz * irs0;            // dyuz
        du[8] = -dzy;                              // dzuy
      }
      __syncthreads();  // s_p read before the stress phase writes it
    }
  }
  float r = 1.f, st = 1.f;
  if (act) {
    // strain-rate proxies (ses3d_evolution.f90:57-87)
    float exx = 0.f, exy = 0.f, exz = 0.f, eyx = 0.f, eyy = 0.f, eyz = 0.f, ezx = 0.f, ezy = 0.f, ezz = 0.f;
#pragma unroll
    for (int q = 0; q < 5; ++q) {
      const int ix = q + 5 * jn + 25 * kn, iy = in + 5 * q + 25 * kn, iz = in + 5 * jn + 25 * q;
      const float dxq = tab.Dx[in][q], dyq = tab.Dy[jn][q], dzq = tab.Dz[kn][q];
      exx = fmaf(s_v[0][ix], dxq, exx);
      exy = fmaf(s_v[1][ix], dxq, exy);
      exz = fmaf(s_v[2][ix], dxq, exz);
      eyx = fmaf(s_v[0][iy], dyq, eyx);
      eyy = fmaf(s_v[1][iy], dyq, eyy);
      eyz = fmaf(s_v[2][iy], dyq, eyz);
      ezx = fmaf(s_v[0][iz], dzq, ezx);
      ezy = fmaf(s_v[1][iz], dzq, ezy);
      ezz = fmaf(s_v[2][iz], dzq, ezz);
    }
    // spherical completion (ses3d_evolution.f90:93-103), divisions by r and r sin(theta)
    // taken as products with the tabulated reciprocals
    const float *lt = x.lt;
    r = lt ? lt[LT_R + kn] : __ldg(p.r_z + k * 5 + kn);
    st = lt ? lt[LT_SIN + in] : __ldg(p.sin_x + ii * 5 + in);
    const float ir = lt ? lt[LT_IR + kn] : __ldg(p.inv_r + k * 5 + kn);
    const float irs = ir * (lt ? lt[LT_ISIN + in] : __ldg(p.inv_sin + ii * 5 + in));
    const float ct = lt ? lt[LT_COT + in] : __ldg(p.cot_x + ii * 5 + in);
    ezz = -ezz;
    eyy = eyy * irs + (vz + vx * ct) * ir;
    exx = (vz + exx) * ir;
    ezx = -ezx;
    exz = (exz - vx) * ir;
    ezy = -ezy;
    eyz = -vy * ir + eyz * irs;
    exy = exy * ir;
    eyx = -vy * ct * ir + eyx * irs;
    const float dt = c.dt;
    // Lean iterations in elements outside the PML: every profile there is zero and the taper
    // one, so the displacement gradients enter nothing and the PML strain terms add zeros;
    // both are skipped (the strain rates keep their values).
    const bool pml_free = lean_mode(MODE) && !full;
    float dxux = 0.f, dyuy = 0.f, dzuz = 0.f, dxuy = 0.f, dyux = 0.f, dxuz = 0.f, dzux = 0.f, dyuz = 0.f, dzuy = 0.f;
    float px = 0.f, py = 0.f, pz = 0.f, taper = 1.f;
    if (!pml_free) {
      // displacement gradients (ses3d_evolution.f90:109-117)
      dxux = sv[F_DXUX] + dt * exx; dyuy = sv[F_DYUY] + dt * eyy; dzuz = sv[F_DZUZ] + dt * ezz;
      dxuy = sv[F_DXUY] + dt * exy; dyux = sv[F_DYUX] + dt * eyx;
      dxuz = sv[F_DXUZ] + dt * exz; dzux = sv[F_DZUX] + dt * ezx;
      dyuz = sv[F_DYUZ] + dt * eyz; dzuy = sv[F_DZUY] + dt * ezy;
      if (full) {
        S[F_DXUX * 125] = dxux; S[F_DYUY * 125] = dyuy; S[F_DZUZ * 125] = dzuz;
        S[F_DXUY * 125] = dxuy; S[F_DYUX * 125] = dyux; S[F_DXUZ * 125] = dxuz;
        S[F_DZUX * 125] = dzux; S[F_DYUZ * 125] = dyuz; S[F_DZUY * 125] = dzuy;
      }
      // PML profiles of this node (ses3d_init.f90:678-686), corners normalised
      const float pxr = lt ? lt[LT_PX + in] : __ldg(p.pxr + ii * 5 + in);
      const float pyr = lt ? lt[LT_PY + jn] : __ldg(p.pyr + j * 5 + jn);
      const float pzr = lt ? lt[LT_PZ + kn] : __ldg(p.pzr + k * 5 + kn);
      const float praw = __fadd_rn(__fadd_rn(pxr, pyr), pzr);
      if (praw != 0.f) {
        const float den = __fadd_rn(1.f, __fdiv_rn(praw, 1.2f));
        pz = __fdiv_rn(__fmul_rn(2.f, pzr), den);
        py = __fdiv_rn(__fmul_rn(2.f, pyr), den);
        px = __fdiv_rn(__fmul_rn(2.f, pxr), den);
        const float prof = __fadd_rn(__fadd_rn(px, py), pz);
        taper = expf(-__fmul_rn(__fmul_rn(0.1f, prof), prof));
      }
      // PML strain rates (ses3d_evolution.f90:123-134)
      exx = exx + (pz + py) * dxux;
      eyy = eyy + (px + pz) * dyuy;
      ezz = ezz + (px + py) * dzuz;
      exy = exy + (py + pz) * dxuy;
      eyx = eyx + (px + pz) * dyux;
      exz = exz + (py + pz) * dxuz;
      ezx = ezx + (px + py) * dzux;
      eyz = eyz + (px + pz) * dyuz;
      ezy = ezy + (px + py) * dzuy;
    }
    if constexpr (MODE == 4 || MODE == 5) {
      if (pml_free) {
        dxux = du[0]; dyuy = du[1]; dzuz = du[2]; dxuy = du[3]; dyux = du[4];
        dxuz = du[5]; dzux = du[6]; dyuz = du[7]; dzuy = du[8];
      }
    }
    // symmetrisation (ses3d_evolution.f90:136-138)
    exy = (exy + eyx) * 0.5f;
    exz = (exz + ezx) * 0.5f;
    eyz = (eyz + ezy) * 0.5f;
    // stress rates (ses3d_evolution.f90:146-202)
    const float tr = exx + eyy + ezz;
    float sxx, syy, szz, sxy, sxz, syz;
    float Mv[18];
    if (DISS) {
#pragma unroll
      for (int t = 0; t < 18; ++t) Mv[t] = sv[(F_M + t) % NS];
      const float Mdx = Mv[0] + Mv[1] + Mv[2], Mdy = Mv[3] + Mv[4] + Mv[5], Mdz = Mv[6] + Mv[7] + Mv[8];
      const float Mxy = Mv[9] + Mv[10] + Mv[11], Mxz = Mv[12] + Mv[13] + Mv[14], Myz = Mv[15] + Mv[16] + Mv[17];
      const float Lw = clam * tr - c2mt * (Mdx + Mdy + Mdz) * (1.f / 3.f);
      sxx = Lw + c2mut * exx + c2mt * Mdx + cC * ezz + cA * (eyy + exx);
      syy = Lw + c2mut * eyy + c2mt * Mdy + cC * ezz + cA * (eyy + exx);
      szz = Lw + c2mut * ezz + c2mt * Mdz + cC * (eyy + exx);
      sxy = c2mut * exy + c2mt * Mxy;
      sxz = c2mut * exz + c2mt * Mxz + cB2 * exz;
      syz = c2mut * eyz + c2mt * Myz + cB2 * eyz;
      // memory variables with the PML-modified, symmetrised strain rates (ses3d_evolution.f90:334-360)
      const float ecomp[6] = {exx, eyy, ezz, exy, exz, eyz};
#pragma unroll
      for (int cc = 0; cc < 6; ++cc)
#pragma unroll
        for (int m = 0; m < 3; ++m) {
          float M = Mv[3 * cc + m];
          M = M - M * c.a_k[m] - c.L_k[m] * ecomp[cc];
          Mv[3 * cc + m] = M;
          S[(F_M + 3 * cc + m) * 125] = M;
        }
    } else {
      const float Lw = clam * tr;
      sxx = Lw + c2mut * exx + cC * ezz + cA * (eyy + exx);
      syy = Lw + c2mut * eyy + cC * ezz + cA * (eyy + exx);
      szz = Lw + c2mut * ezz + cC * (eyy + exx);
      sxy = c2mut * exy;
      sxz = c2mut * exz + cB2 * exz;
      syz = c2mut * eyz + cB2 * eyz;
    }
    // march PML stresses (ses3d_evolution.f90:208-219)
    float s_xx = sv[F_SXX], s_yy = sv[F_SYY], s_zz = sv[F_SZZ];
    float s_xy = sv[F_SXY], s_yx = sv[F_SYX], s_xz = sv[F_SXZ];
    float s_zx = sv[F_SZX], s_yz = sv[F_SYZ], s_zy = sv[F_SZY];
    if (pml_free) {  // zero profiles; the mirrors equal their partners (lean stepping)
      s_xx = s_xx + dt * sxx;
      s_yy = s_yy + dt * syy;
      s_zz = s_zz + dt * szz;
      s_xy = s_xy + dt * sxy;
      s_xz = s_xz + dt * sxz;
      s_yz = s_yz + dt * syz;
      s_yx = s_xy; s_zx = s_xz; s_zy = s_yz;
    } else {
      s_xx = s_xx + dt * (sxx - px * s_xx);
      s_yy = s_yy + dt * (syy - py * s_yy);
      s_zz = s_zz + dt * (szz - pz * s_zz);
      s_xy = s_xy + dt * (sxy - px * s_xy);
      s_yx = s_yx + dt * (sxy - py * s_yx);
      s_xz = s_xz + dt * (sxz - px * s_xz);
      s_zx = s_zx + dt * (sxz - pz * s_zx);
      s_yz = s_yz + dt * (syz - py * s_yz);
      s_zy = s_zy + dt * (syz - pz * s_zy);
    }
    // taper (ses3d_evolution.f90:368-371); the divergence below uses the untapered values
    S[F_SXX * 125] = s_xx * taper; S[F_SYY * 125] = s_yy * taper; S[F_SZZ * 125] = s_zz * taper;
    S[F_SXY * 125] = s_xy * taper; S[F_SXZ * 125] = s_xz * taper; S[F_SYZ * 125] = s_yz * taper;
    if (full) { S[F_SYX * 125] = s_yx * taper; S[F_SZX * 125] = s_zx * taper; S[F_SZY * 125] = s_zy * taper; }
    // moment-tensor source field (ses3d_miscellaneous.f90:115-147)
    if (!corr_mode(MODE) && (int)e == (lt ? __float_as_int(lt[LT_SRC]) : __ldg(p.src_elem + ev))) {
      const int it = *p.d_it + 1;
      const float d = p.src_delta[ev * 125 + nn];
      const float so = p.stf[(size_t)ev * c.nt + (it - 1)];
      const float *mom = p.src_mom + ev * 6;
      const float sxxs = -(__fmul_rn(__fmul_rn(mom[0], d), so)), syys = -(__fmul_rn(__fmul_rn(mom[1], d), so));
      const float szzs = -(__fmul_rn(__fmul_rn(mom[2], d), so)), sxys = -(__fmul_rn(__fmul_rn(mom[3], d), so));
      const float sxzs = -(__fmul_rn(__fmul_rn(mom[4], d), so)), syzs = -(__fmul_rn(__fmul_rn(mom[5], d), so));
      s_xx += sxxs; s_yy += syys; s_zz += szzs;
      s_xy += sxys; s_yx += sxys; s_xz += sxzs; s_zx += sxzs; s_yz += syzs; s_zy += syzs;
    }
    // node-local weights of the weak divergence (ses3d_evolution.f90:247-249)
    const float wx = tab.w[in] * st, wy = tab.w[jn], wz = tab.w[kn] * r * r;
    s_p[0][n] = wx * s_xx; s_p[1][n] = wx * s_xy; s_p[2][n] = wx * s_xz;
    s_p[3][n] = wy * s_yx; s_p[4][n] = wy * s_yy; s_p[5][n] = wy * s_yz;
    s_p[6][n] = wz * s_zx; s_p[7][n] = wz * s_zy; s_p[8][n] = wz * s_zz;

    if (record_mode(MODE)) {  // forward record (ses3d_main.f90:148-158)
      float *R = p.rec + (size_t)ev * NREC * N + m0;
      R[R_VX * N] = vx; R[R_VY * N] = vy; R[R_VZ * N] = vz;
      R[R_EXX * N] = dxux; R[R_EYY * N] = dyuy; R[R_EZZ * N] = dzuz;
      R[R_EXY * N] = (dxuy + dyux) * 0.5f; R[R_EXZ * N] = (dxuz + dzux) * 0.5f; R[R_EYZ * N] = (dyuz + dzuy) * 0.5f;
    }
    if (corr_mode(MODE) && p.rec) {  // kernel correlation (ses3d_grad.f90:53-83, ses3d_grad_Q.f90:111-143)
      // operands from the shared-memory stage when the persistent kernel staged them
      const float *cf = x.cstage;
      size_t fs = TPE;
      if (cf) {
        if (x.cstage_more) asm volatile("cp.async.wait_group 1;" ::: "memory");
        else asm volatile("cp.async.wait_group 0;" ::: "memory");
        cf += n;
      } else {
        cf = p.rec + (size_t)ev * NREC * N + m0;
        fs = N;
      }
      const float *R = cf;
      const float vxf = R[R_VX * fs], vyf = R[R_VY * fs], vzf = R[R_VZ * fs];
      const float exxf = R[R_EXX * fs], eyyf = R[R_EYY * fs], ezzf = R[R_EZZ * fs];
      const float exyf = R[R_EXY * fs], exzf = R[R_EXZ * fs], eyzf = R[R_EYZ * fs];
      const float exx_ad = dxux, eyy_ad = dyuy, ezz_ad = dzuz;
      const float exy_ad = 0.5f * (dxuy + dyux), exz_ad = 0.5f * (dxuz + dzux), eyz_ad = 0.5f * (dyuz + dzuy);
      const float tr_ad = exx_ad + eyy_ad + ezz_ad, tr_fw = exxf + eyyf + ezzf;
      const float edde = exx_ad * exxf + eyy_ad * eyyf + ezz_ad * ezzf + 2.f * exy_ad * exyf +
                         2.f * exz_ad * exzf + 2.f * eyz_ad * eyzf;
      float rho, cp, cs;
      if (x.cstage) {
        rho = cf[9 * TPE]; cp = cf[10 * TPE]; cs = cf[11 * TPE];
      } else {
        const float *GM = p.gmat + m0;
        rho = GM[G_RHO * N]; cp = GM[G_CP * N]; cs = GM[G_CS * N];
      }
      const double *G0 = x.cstage ? reinterpret_cast<const double *>(x.cstage + CS_FLOATS * TPE) + n
                                  : p.grad + (size_t)ev * NGRAD * N + m0;
      const size_t gs = x.cstage ? (size_t)TPE : N;
      const double sj = c.s_jac;
      double *GR = p.grad + (size_t)ev * NGRAD * N + m0;
      GR[0 * N] = G0[0 * gs] + sj * (double)((vxf * vx + vyf * vy + vzf * vz) +
                                            ((cp * cp - 2.f * cs * cs) * tr_fw * tr_ad + 2.f * cs * cs * edde));
      GR[1 * N] = G0[1 * gs] + sj * (double)(2.f * rho * cp * tr_fw * tr_ad);
      GR[2 * N] = G0[2 * gs] + sj * (double)(4.f * rho * cs * (edde - tr_ad * tr_fw - 2.f * exzf * exz_ad -
                                                               2.f * eyzf * eyz_ad));
      GR[3 * N] = G0[3 * gs] + sj * (double)(8.f * rho * cs * (exzf * exz_ad + eyzf * eyz_ad));
      if (DISS && p.grad_q) {
        // The three mechanisms' terms are summed in FP32 and the sum accumulated in FP64:
        // one conversion and one FMA per kernel (FP64 issue is scarce on this part).
        const float ef[6] = {exxf, eyyf, ezzf, exyf, exzf, eyzf};
        float gq = 0.f, ga = 0.f, gk = 0.f, gak = 0.f;
#pragma unroll
        for (int m = 0; m < 3; ++m) {
          const float tsum = Mv[m] + Mv[3 + m] + Mv[6 + m];
          float Md = 0.f;
#pragma unroll
          for (int cc = 0; cc < 6; ++cc) Md += Mv[3 * cc + m] * ef[cc];
          Md = Md - tr_fw * tsum / 3.f;
          gq += Md * c.tau_p[m];
          ga += Md * c.q_alpha_w[m];
          const float Mk = tsum * tr_fw;
          gk += Mk * c.tau_p[m];
          gak += Mk * c.q_alpha_w[m];
        }
        GR[4 * N] = G0[4 * gs] + sj * (double)gq;
        GR[5 * N] = G0[5 * gs] + sj * (double)ga;
        GR[6 * N] = G0[6 * gs] + sj * (double)gk;
        GR[7 * N] = G0[7 * gs] + sj * (double)gak;
      }
      // this point's operands are in registers and used: stage the next item's
      if (x.cstage && x.cstage_next >= 0) stage_corr<DISS>(c, p, x.cstage_next, nn, x.cstage);
    }
  }
  __syncthreads();
  after_barrier();

  if (act) {
    // weak-form divergence (ses3d_evolution.f90:235-270)
    float ax0 = 0.f, ax1 = 0.f, ax2 = 0.f, ay0 = 0.f, ay1 = 0.f, ay2 = 0.f, az0 = 0.f, az1 = 0.f, az2 = 0.f;
#pragma unroll
    for (int q = 0; q < 5; ++q) {
      const int ix = q + 5 * jn + 25 * kn, iy = in + 5 * q + 25 * kn, iz = in + 5 * jn + 25 * q;
      const float dxq = tab.dlT[in][q], dyq = tab.dlT[jn][q], dzq = tab.dlT[kn][q];
      ax0 = fmaf(s_p[0][ix], dxq, ax0);
      ax1 = fmaf(s_p[1][ix], dxq, ax1);
      ax2 = fmaf(s_p[2][ix], dxq, ax2);
      ay0 = fmaf(s_p[3][iy], dyq, ay0);
      ay1 = fmaf(s_p[4][iy], dyq, ay1);
      ay2 = fmaf(s_p[5][iy], dyq, ay2);
      az0 = fmaf(s_p[6][iz], dzq, az0);
      az1 = fmaf(s_p[7][iz], dzq, az1);
      az2 = fmaf(s_p[8][iz], dzq, az2);
    }
    const float cx = tab.CX[jn][kn] * r, cy = tab.CY[in][kn] * r, cz = tab.CZ[in][jn] * st;
    float *F = p.f + (size_t)ev * 3 * N + force_offset(c, ii, j, k, in, jn, kn);
    F[0] = cx * ax0 + cy * ay0 + cz * az0;
    F[125] = cx * ax1 + cy * ay1 + cz * az1;
    F[250] = cx * ax2 + cy * ay2 + cz * az2;
  }
}

// ---------------------------------------------------------------------------------------
// k_element: one element per 128 threads (thread = GLL node), EPB consecutive x-elements
// per CTA; grid (ceil(ex/EPB), ey, ez * n_events). MODE 0 plain, 1 store forward record,
// 2 adjoint with kernel correlation, 3 lean plain (displacement gradients in PML elements only). Every independent global load (state, material, v)
// is issued before the first barrier so that a thread has all its bytes in flight at once.
// ---------------------------------------------------------------------------------------
template <bool DISS, int MODE, int EPB>
__global__ void __launch_bounds__(TPE * EPB, (SES3D_ELEM_MINB / EPB > 0 ? SES3D_ELEM_MINB / EPB : 1)) k_element(const Consts c, const Ptrs p) {
  static_assert(MODE <= 3, "lean record and correlation iterations run the persistent kernel");
  __shared__ KTab tab;
  __shared__ float s_v[EPB][3][TPE];
  __shared__ float s_p[EPB][9][TPE];

  for (int t = threadIdx.x; t < KTAB_FLOATS; t += blockDim.x)
    reinterpret_cast<float *>(&tab)[t] = reinterpret_cast<const float *>(p.ktab)[t];

  const int sub = threadIdx.x / TPE;
  const int n = threadIdx.x % TPE;
  const int i = blockIdx.x * EPB + sub;
  const int j = blockIdx.y;
  const int k = (int)blockIdx.z / c.nev;
  const int ev = (int)blockIdx.z - k * c.nev;
  bool act = i < c.ex && n < 125;
  const int nn = act ? n : 0;
  const int ii = act ? i : 0;
  const int in = nn % 5, jn = (nn / 5) % 5, kn = nn / 25;
  const unsigned e = (unsigned)ii + (unsigned)c.ex * ((unsigned)j + (unsigned)c.ey * (unsigned)k);
  const size_t N = (size_t)c.N;
  const size_t m0 = (size_t)e * 125 + nn;  // element-major index of field-major arrays (records, gmat)
  float *S = p.state + ((size_t)ev * c.E + e) * ELEM_STATE + nn;  // field f at S[f * 125]
  const float *MT = p.mat + (size_t)e * ELEM_MAT + nn;             // field f at MT[f * MAT_ROW]

  constexpr int NS = DISS ? NSTATE : 18;  // elastic runs carry no memory variables
  // Outside the PML the displacement gradients enter no output of a plain forward run
  // (ses3d_evolution.f90:123-134 multiplies them by zero profiles); lean runs skip them there.
  const bool full =
      MODE != 3 || i < c.pml || i >= c.ex - c.pml || j < c.pml || j >= c.ey - c.pml || k >= c.ez - c.pml;
  float sv[NS];
  float clam = 0.f, c2mut = 0.f, c2mt = 0.f, cA = 0.f, cB2 = 0.f, cC = 0.f;
  float vx = 0.f, vy = 0.f, vz = 0.f;
#ifndef SES3D_CHECKED
  if (MODE == 3)
#endif
  {  // index self-check (lean stepping, and every mode in SES3D_CHECKED builds): every index
     // derived below must lie inside its buffer; a violation is reported and the access skipped
    const size_t g = (size_t)(ii * 4 + in) + (size_t)c.GX * ((size_t)(j * 4 + jn) + (size_t)c.GY * (size_t)(k * 4 + kn));
    int bad = 0;
    if (act && (ev < 0 || ev >= c.nev)) bad = 1;
    if (act && m0 >= N) bad = 2;
    if (act && g >= (size_t)c.G) bad = 3;
    if (act && (ii * 5 + in >= c.ex * 5 || j * 5 + jn >= c.ey * 5 || k * 5 + kn >= c.ez * 5)) bad = 4;
    if (bad) {
      printf("k_element<%d,%d,%d> bad index kind %d block (%d,%d,%d) thread %d m0 %llu g %llu\n", (int)DISS, MODE, EPB,
             bad, blockIdx.x, blockIdx.y, blockIdx.z, threadIdx.x, (unsigned long long)m0, (unsigned long long)g);
      act = false;
    }
  }
  if (act) {
    // gather v_global -> element-local v (ses3d_evolution.f90:27-51)
    const size_t g = (size_t)(ii * 4 + in) + (size_t)c.GX * ((size_t)(j * 4 + jn) + (size_t)c.GY * (size_t)(k * 4 + kn));
    const float *v = p.v + (size_t)ev * 3 * c.G + g;
    vx = v[0]; vy = v[c.G]; vz = v[2 * c.G];
#pragma unroll
    for (int f = 0; f < F_SYX; ++f) sv[f] = S[f * 125];
    if (full) {
#pragma unroll
      for (int f = F_SYX; f <= F_DZUY; ++f) sv[f] = S[f * 125];
    } else {  // lean stepping outside the PML: mirrors from their partners, no gradients
      sv[F_SYX] = sv[F_SXY]; sv[F_SZX] = sv[F_SXZ]; sv[F_SZY] = sv[F_SYZ];
#pragma unroll
      for (int f = F_DXUX; f <= F_DZUY; ++f) sv[f] = 0.f;
    }
#pragma unroll
    for (int f = F_DZUY + 1; f < NS; ++f) sv[f] = S[f * 125];
    clam = __ldg(MT + M_CLAM * MAT_ROW); c2mut = __ldg(MT + M_C2MUT * MAT_ROW);
    if (DISS) c2mt = __ldg(MT + M_C2MT * MAT_ROW);
    if (!c.iso) { cA = __ldg(MT + M_A * MAT_ROW); cB2 = __ldg(MT + M_B2 * MAT_ROW); cC = __ldg(MT + M_C * MAT_ROW); }
  } else {
#pragma unroll
    for (int f = 0; f < NS; ++f) sv[f] = 0.f;
  }
  s_v[sub][0][n] = vx; s_v[sub][1][n] = vy; s_v[sub][2][n] = vz;
  __syncthreads();
  ElemCtx x{act, full, n, nn, in, jn, kn, ii, j, k, ev, e, N, m0, S, vx, vy, vz, clam, c2mut, c2mt, cA, cB2, cC, nullptr,
            nullptr, false, -1, nullptr};
  element_compute<DISS, MODE>(c, p, tab, s_v[sub], s_p[sub], x, sv);
}


// ---------------------------------------------------------------------------------------
// k_element_tma: persistent element kernel for plain and lean forward iterations. Each
// 128-thread CTA walks (element, event) items with a stride of the grid; one thread copies
// an item's whole state block (18,000 B) and material block (3,072 B) into shared memory
// with cp.async.bulk on an mbarrier, ahead of the compute (the next item's copy is issued
// as soon as the current one has been read into registers), so the loads leave the
// register file and overlap the current item's arithmetic. Results equal k_element's bit
// for bit (same arithmetic, only the source of the loaded values differs).
// Every mbarrier wait is bounded (2 s of %globaltimer): on expiry the block records an
// error in p.err, waits (bounded again) for its copies still in flight and returns; the
// host reports the failed step.
// ---------------------------------------------------------------------------------------
// Shape of k_element_tma (measured on the 96 x 96 x 40 mesh): one state stage refilled as
// soon as it has been read, at most 102 registers (5 CTAs per SM), and the element-local
// velocity gathered one item ahead with cp.async.
#ifndef SES3D_TMA_STAGES
#define SES3D_TMA_STAGES 1
#endif
#ifndef SES3D_TMA_MINB
#define SES3D_TMA_MINB 5
#endif
#ifndef SES3D_TMA_VPREF
#define SES3D_TMA_VPREF 1
#endif
constexpr int TMA_STAGES = SES3D_TMA_STAGES;
constexpr int TMA_VBUF = SES3D_TMA_VPREF ? 2 : 1;  // element-local velocity buffers
struct __align__(16) ElemStage {
  float state[ELEM_STATE];  // 18,000 B
  float mat[ELEM_MAT];      // 3,072 B
};
constexpr size_t TMA_LT_OFF =
    TMA_STAGES * sizeof(ElemStage) + (9 + 3 * TMA_VBUF) * TPE * sizeof(float) + ((sizeof(KTab) + 15) / 16) * 16;
constexpr size_t TMA_BAR_OFF = TMA_LT_OFF + TMA_VBUF * LT_FLOATS * sizeof(float);
constexpr size_t TMA_SMEM = TMA_BAR_OFF + TMA_STAGES * sizeof(unsigned long long);
// Correlation iterations also stage their epilogue operands (CS_BYTES) behind the barriers.
constexpr size_t TMA_CS_OFF = (TMA_SMEM + 15) / 16 * 16;
__host__ __device__ constexpr bool tma_cstage(int mode) { return corr_mode(mode) && TMA_VBUF == 2; }
// Lean record and correlation iterations also stage the displacement at the next item's
// nodes, double-buffered like the velocity, behind that.
__host__ __device__ constexpr bool tma_ustage(int mode) { return (mode == 4 || mode == 5) && TMA_VBUF == 2; }
__host__ __device__ constexpr size_t tma_u_off(int mode) { return tma_cstage(mode) ? TMA_CS_OFF + CS_BYTES : TMA_CS_OFF; }
__host__ __device__ constexpr size_t tma_smem(int mode) {
  return tma_ustage(mode) ? tma_u_off(mode) + 2 * 3 * TPE * sizeof(float)
                          : (tma_cstage(mode) ? TMA_CS_OFF + CS_BYTES : TMA_SMEM);
}

// Copies of one item into a stage. Byte ranges (element block of 18,000 B, fields of 500 B):
// all 36 fields; elastic: fields 0-17 (9,008 B, the last 8 B inside field 18); lean outside
// the PML: fields 0-5 (3,008 B) and, with attenuation, 18-35 (from byte 8,992, 9,008 B),
// skipping the mirror stresses and the displacement gradients. Every range starts and ends 16-B aligned inside the block.
template <bool DISS, int MODE>
__device__ __forceinline__ void issue_item(const Consts &c, const Ptrs &p, long long item, ElemStage *st,
                                           unsigned long long *bar) {
  const int ev = (int)(item % c.nev);
  const unsigned e = (unsigned)(item / c.nev);
  const int i = (int)(e % (unsigned)c.ex), j = (int)((e / (unsigned)c.ex) % (unsigned)c.ey);
  const int k = (int)(e / ((unsigned)c.ex * (unsigned)c.ey));
  const char *src = reinterpret_cast<const char *>(p.state + ((size_t)ev * c.E + e) * ELEM_STATE);
  const char *msrc = reinterpret_cast<const char *>(p.mat + (size_t)e * ELEM_MAT);
  char *dst = reinterpret_cast<char *>(st->state);
  const unsigned MB = (c.iso ? 3 * MAT_ROW : ELEM_MAT) * (unsigned)sizeof(float);
  if (!DISS && lean_mode(MODE) && !in_pml_element(c, i, j, k)) {
    mbar_arrive_expect_tx(bar, 3008u + MB);
    bulk_g2s(dst, src, 3008u, bar);
  } else if (!DISS) {
    mbar_arrive_expect_tx(bar, 9008u + MB);
    bulk_g2s(dst, src, 9008u, bar);
  } else if (lean_mode(MODE) && !in_pml_element(c, i, j, k)) {
    mbar_arrive_expect_tx(bar, 3008u + 9008u + MB);
    bulk_g2s(dst, src, 3008u, bar);
    bulk_g2s(dst + 8992, src + 8992, 9008u, bar);
  } else {
    mbar_arrive_expect_tx(bar, (unsigned)(ELEM_STATE * sizeof(float)) + MB);
    bulk_g2s(dst, src, (unsigned)(ELEM_STATE * sizeof(float)), bar);
  }
  bulk_g2s(st->mat, msrc, MB, bar);
}

// The element-local velocity of one item, gathered from the assembled field straight into
// shared memory with 4-byte cp.async (ses3d_evolution.f90:27-51), and, with TABLES, the
// item's 1-D table entries and source element into lt (threads 0..15), in one commit group. (The table copies pay off in
// lean iterations; with the full state they cost more than the loads they replace.)
template <bool TABLES>
__device__ __forceinline__ void gather_v_async(const Consts &c, const Ptrs &p, long long item, float (*dst)[TPE],
                                               float *lt, int n, int in, int jn, int kn, float *udst = nullptr) {
  const int ev = (int)(item % c.nev);
  const unsigned e = (unsigned)(item / c.nev);
  const int i = (int)(e % (unsigned)c.ex), j = (int)((e / (unsigned)c.ex) % (unsigned)c.ey);
  const int k = (int)(e / ((unsigned)c.ex * (unsigned)c.ey));
  if (n < 125) {
    const size_t g = (size_t)(i * 4 + in) + (size_t)c.GX * ((size_t)(j * 4 + jn) + (size_t)c.GY * (size_t)(k * 4 + kn));
    const float *v = p.v + (size_t)ev * 3 * c.G + g;
#pragma unroll
    for (int q = 0; q < 3; ++q) cp_async4(&dst[q][n], v + (size_t)q * c.G);
    if (udst && !in_pml_element(c, i, j, k)) {  // the displacement, read outside the PML only
      const float *u = p.u + (size_t)ev * 3 * c.G + g;
#pragma unroll
      for (int q = 0; q < 3; ++q) cp_async4(udst + q * TPE + n, u + (size_t)q * c.G);
    }
  }
  if (!TABLES) {
  } else if (n < 5) {
    cp_async4(lt + LT_SIN + n, p.sin_x + i * 5 + n);
    cp_async4(lt + LT_COT + n, p.cot_x + i * 5 + n);
    cp_async4(lt + LT_ISIN + n, p.inv_sin + i * 5 + n);
    cp_async4(lt + LT_PX + n, p.pxr + i * 5 + n);
  } else if (n < 10) {
    cp_async4(lt + LT_PY + (n - 5), p.pyr + j * 5 + (n - 5));
  } else if (n < 15) {
    cp_async4(lt + LT_R + (n - 10), p.r_z + k * 5 + (n - 10));
    cp_async4(lt + LT_IR + (n - 10), p.inv_r + k * 5 + (n - 10));
    cp_async4(lt + LT_PZ + (n - 10), p.pzr + k * 5 + (n - 10));
  } else if (n == 15) {
    cp_async4(lt + LT_SRC, p.src_elem + ev);
  }
  asm volatile("cp.async.commit_group;" ::: "memory");
}

// L2 prefetch of what a correlation item's epilogue reads with plain loads (the forward
// record, the adjoint-model fields and the FP64 kernel accumulators at the item's points),
// issued one item ahead by the threads that will read them.
template <bool DISS>
__device__ __forceinline__ void prefetch_corr(const Consts &c, const Ptrs &p, long long item, int nn) {
  const int ev = (int)(item % c.nev);
  const size_t N = (size_t)c.N, m0 = (size_t)(item / c.nev) * 125 + nn;
  const float *R = p.rec + (size_t)ev * NREC * N + m0;
#pragma unroll
  for (int f = 0; f < NREC; ++f) prefetch_l2(R + f * N);
  prefetch_l2(p.gmat + G_RHO * N + m0);
  prefetch_l2(p.gmat + G_CP * N + m0);
  prefetch_l2(p.gmat + G_CS * N + m0);
  const double *GR = p.grad + (size_t)ev * NGRAD * N + m0;
  const int nk = (DISS && p.grad_q) ? 8 : 4;
  for (int q = 0; q < nk; ++q) prefetch_l2(GR + q * N);
}

// MINB: resident CTAs per SM requested from ptxas (register cap); REFILL: when the next
// item's bulk copy is issued (0: the measured rule below, 1: the other point). PACK: also
// write the fields of each item's starting state that the exact adjoint's transposed step
// reads (displacement gradients, memory-variable sums) to p.slot.
template <bool DISS, int MODE, int MINB = SES3D_TMA_MINB, int REFILL = 0, bool PACK = false>
__global__ void __launch_bounds__(TPE, MINB) k_element_tma(const Consts c, const Ptrs p) {
  extern __shared__ __align__(128) unsigned char smem[];
  ElemStage *stage = reinterpret_cast<ElemStage *>(smem);
  float (*s_vb)[TPE] = reinterpret_cast<float (*)[TPE]>(smem + TMA_STAGES * sizeof(ElemStage));  // [TMA_VBUF][3]
  float (*s_p)[TPE] = s_vb + 3 * TMA_VBUF;
  KTab *tab = reinterpret_cast<KTab *>(s_p + 9);
  float *s_lt = reinterpret_cast<float *>(smem + TMA_LT_OFF);  // [TMA_VBUF][LT_FLOATS]
  unsigned long long *bar = reinterpret_cast<unsigned long long *>(smem + TMA_BAR_OFF);

  const int n = threadIdx.x;
  const long long total = c.E * (long long)c.nev;
  const long long first = blockIdx.x, stride = gridDim.x;
  if (n == 0) {
    for (int s = 0; s < TMA_STAGES; ++s) mbar_init(&bar[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int t = n; t < KTAB_FLOATS; t += TPE)
    reinterpret_cast<float *>(tab)[t] = reinterpret_cast<const float *>(p.ktab)[t];
  __syncthreads();
  if (n == 0)
    for (int s = 0; s < TMA_STAGES; ++s)
      if (first + s * stride < total) issue_item<DISS, MODE>(c, p, first + s * stride, &stage[s], &bar[s]);

  constexpr int NS = DISS ? NSTATE : 18;
  const bool on = n < 125;
  const int nn = on ? n : 0;
  const int in = nn % 5, jn = (nn / 5) % 5, kn = nn / 25;
  constexpr bool TABLES = lean_mode(MODE);
  float *s_ub = nullptr;  // [2][3][TPE] displacement stages
  if constexpr (tma_ustage(MODE)) s_ub = reinterpret_cast<float *>(smem + tma_u_off(MODE));
  if (TMA_VBUF == 2 && first < total) gather_v_async<TABLES>(c, p, first, s_vb, s_lt, n, in, jn, kn, s_ub);
  // correlation operands: staged one item ahead, each thread its own point (cp.async groups
  // in the order velocity(t), operands(t), velocity(t + 1), operands(t + 1), ...)
  float *cstage = nullptr;
  if constexpr (tma_cstage(MODE))
    if (p.rec) cstage = reinterpret_cast<float *>(smem + TMA_CS_OFF);
  if (cstage && on && first < total) stage_corr<DISS>(c, p, first, nn, cstage);
  for (int t = 0;; ++t) {
    const long long item = first + (long long)t * stride;
    if (item >= total) break;
    const int s = t % TMA_STAGES;
    const unsigned parity = (unsigned)(t / TMA_STAGES) & 1u;
    float (*s_v)[TPE] = s_vb + 3 * (t % TMA_VBUF);
    const int ev = (int)(item % c.nev);
    const unsigned e = (unsigned)(item / c.nev);
    const int i = (int)(e % (unsigned)c.ex), j = (int)((e / (unsigned)c.ex) % (unsigned)c.ey);
    const int k = (int)(e / ((unsigned)c.ex * (unsigned)c.ey));
    const bool full = !lean_mode(MODE) || in_pml_element(c, i, j, k);
    float vx = 0.f, vy = 0.f, vz = 0.f;
    if (TMA_VBUF == 2) {  // this item's velocity was gathered one item ahead
      if (cstage) asm volatile("cp.async.wait_group 1;" ::: "memory");  // operands(t) may stay in flight
      else asm volatile("cp.async.wait_group 0;" ::: "memory");
      if (on) { vx = s_v[0][n]; vy = s_v[1][n]; vz = s_v[2][n]; }
    } else if (on) {
      // gather v_global -> element-local v (ses3d_evolution.f90:27-51), issued before the wait
      const size_t g = (size_t)(i * 4 + in) + (size_t)c.GX * ((size_t)(j * 4 + jn) + (size_t)c.GY * (size_t)(k * 4 + kn));
      const float *v = p.v + (size_t)ev * 3 * c.G + g;
      vx = v[0]; vy = v[c.G]; vz = v[2 * c.G];
    }
    const bool ok = mbar_wait_bounded(&bar[s], parity, p.err);
    float sv[NS];
    float clam = 0.f, c2mut = 0.f, c2mt = 0.f, cA = 0.f, cB2 = 0.f, cC = 0.f;
    if (on) {
      const float *ss = stage[s].state + nn;
      const float *sm = stage[s].mat + nn;
#pragma unroll
      for (int f = 0; f < F_SYX; ++f) sv[f] = ss[f * 125];
      if (full) {
#pragma unroll
        for (int f = F_SYX; f <= F_DZUY; ++f) sv[f] = ss[f * 125];
      } else {  // lean stepping outside the PML: mirrors from their partners, no gradients
        sv[F_SYX] = sv[F_SXY]; sv[F_SZX] = sv[F_SXZ]; sv[F_SZY] = sv[F_SYZ];
#pragma unroll
        for (int f = F_DXUX; f <= F_DZUY; ++f) sv[f] = 0.f;
      }
#pragma unroll
      for (int f = F_DZUY + 1; f < NS; ++f) sv[f] = ss[f * 125];
      clam = sm[M_CLAM * MAT_ROW]; c2mut = sm[M_C2MUT * MAT_ROW];
      if (DISS) c2mt = sm[M_C2MT * MAT_ROW];
      if (!c.iso) { cA = sm[M_A * MAT_ROW]; cB2 = sm[M_B2 * MAT_ROW]; cC = sm[M_C * MAT_ROW]; }
      if (PACK) {  // displacement gradients in PML elements only: outside, the transposed step
                   // multiplies them by zero profiles and does not read them
        float *D = p.slot + ((size_t)ev * c.E + e) * slot_stride(DISS) + nn;
        if (in_pml_element(c, i, j, k)) {
#pragma unroll
          for (int f = 0; f < 9; ++f) D[f * 125] = sv[F_DXUX + f];
        }
        if (DISS) {
#pragma unroll
          for (int cc = 0; cc < 6; ++cc) D[(9 + cc) * 125] = sv[F_M + 3 * cc] + sv[F_M + 3 * cc + 1] + sv[F_M + 3 * cc + 2];
        }
      }
    } else {
#pragma unroll
      for (int f = 0; f < NS; ++f) sv[f] = 0.f;
    }
    if (TMA_VBUF == 1) { s_v[0][n] = vx; s_v[1][n] = vy; s_v[2][n] = vz; }
    if (__syncthreads_or(!ok)) {  // a copy never arrived: drain the stages, then leave
      asm volatile("cp.async.wait_all;" ::: "memory");
      if (n == 0) {
        mbar_wait_bounded(&bar[s], parity, p.err);
        if constexpr (TMA_STAGES == 2)
          if (item + stride < total) mbar_wait_bounded(&bar[s ^ 1], (unsigned)((t + 1) / TMA_STAGES) & 1u, p.err);
      }
      return;
    }
    // stage s fully read, s_v complete; the other velocity buffer was last read before the
    // previous item's divergence barrier
    if (TMA_VBUF == 2 && item + stride < total)
      gather_v_async<TABLES>(c, p, item + stride, s_vb + 3 * ((t + 1) % 2), s_lt + LT_FLOATS * ((t + 1) % 2), n, in,
                             jn, kn, s_ub ? s_ub + 3 * TPE * ((t + 1) % 2) : nullptr);
    if constexpr (corr_mode(MODE))
      if (on && p.rec && item + stride < total) prefetch_corr<DISS>(c, p, item + stride, nn);
    const long long refill = item + TMA_STAGES * stride;
    auto issue_refill = [&]() {
      if (n == 0 && refill < total) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        issue_item<DISS, MODE>(c, p, refill, &stage[s], &bar[s]);
      }
    };
    // When to issue the next item's bulk copy (measured on 96 x 96 x 40): lean items are
    // short, so right after this item's state has been read; full-state items after the
    // stress/divergence barrier, which keeps thread 0's copy work off that barrier
    // (2.65 -> 2.42 ms per launch), while lean iterations lose 6 % that way.
    constexpr bool LATE_REFILL = (!lean_mode(MODE)) != (REFILL == 1);
    if (!LATE_REFILL) issue_refill();
    const size_t m0 = (size_t)e * 125 + nn;
    float *S = p.state + ((size_t)ev * c.E + e) * ELEM_STATE + nn;
    const float *lt = (TMA_VBUF == 2 && TABLES) ? s_lt + LT_FLOATS * (t % 2) : nullptr;
    const bool more = item + stride < total;
    ElemCtx x{on,  full, n,  nn, in, jn, kn, i, j, k, ev, e, (size_t)c.N, m0, S, vx, vy, vz, clam, c2mut, c2mt, cA, cB2,
              cC,  lt,   cstage, TMA_VBUF == 2 && more, more ? item + stride : -1,
              s_ub ? s_ub + 3 * TPE * (t % 2) : nullptr};
    if (LATE_REFILL) element_compute<DISS, MODE>(c, p, *tab, s_v, s_p, x, sv, issue_refill);
    else element_compute<DISS, MODE>(c, p, *tab, s_v, s_p, x, sv);
  }
}

// ---------------------------------------------------------------------------------------
// k_node: one thread per (global node, event); grid (ceil(GX*GY/TPB), GZ, n_events).
// Deterministic assembly in the reference order (element i, then j, then k ascending;
// ses3d_evolution.f90:286-310), then a = s / MM, v += dt (a - prof v), v *= taper
// (ses3d_evolution.f90:318-328,366).
// ---------------------------------------------------------------------------------------
// KIND 1: also write the assembled forces (a run whose states the exact adjoint replays);
// KIND 2: also integrate the displacement, u += dt v with the velocity before the update.
// TPB threads per CTA, MINB resident CTAs per SM requested from ptxas.
template <int KIND, int TPB = SES3D_NODE_TPB, int MINB = SES3D_NODE_MINB>
__global__ void __launch_bounds__(TPB, MINB) k_node(const Consts c, const Ptrs p) {
  const int gz = blockIdx.y, ev = blockIdx.z;
  if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0)
    *p.d_it += 1;  // every reader of the counter ran earlier in stream order
  const unsigned GXY = (unsigned)c.GX * (unsigned)c.GY;
  const unsigned t = blockIdx.x * (unsigned)TPB + threadIdx.x;
  if (t >= GXY) return;
#if SES3D_NODE_MAGIC
  const int gy = node_row(c, t);
#else
  const int gy = (int)(t / (unsigned)c.GX);
#endif
  const int gx = (int)t - gy * c.GX;
  const size_t g = (size_t)gz * GXY + t;
  // node-local loads first: they do not depend on the element forces
  float *V = p.v + (size_t)ev * 3 * c.G + g;
  float vx = V[0], vy = V[c.G], vz = V[2 * c.G];
  const float imm = __ldg(p.iMM + g);
  const float pxr = __ldg(p.pxg + gx), pyr = __ldg(p.pyg + gy), pzr = __ldg(p.pzg + gz);
  float sx, sy, sz;
  gather_node(c, p.f + (size_t)ev * 3 * (size_t)c.N, gx, gy, gz, sx, sy, sz);
  if (KIND == 1) {
    float *Fo = p.fg + (size_t)ev * 3 * c.G + g;
    Fo[0] = sx; Fo[c.G] = sy; Fo[2 * c.G] = sz;
  }
  if (KIND == 2) {  // the element kernel forms the same sums for its record iterations
    float *U = p.u + (size_t)ev * 3 * c.G + g;
    U[0] = __fadd_rn(U[0], __fmul_rn(c.dt, vx));
    U[c.G] = __fadd_rn(U[c.G], __fmul_rn(c.dt, vy));
    U[2 * c.G] = __fadd_rn(U[2 * c.G], __fmul_rn(c.dt, vz));
  }
  // a = s / MM with the reciprocal of the mass matrix (ses3d_evolution.f90:318-320)
  const float ax = sx * imm, ay = sy * imm, az = sz * imm;
  float px, py, pz, prof, taper;
  pml_profiles(pxr, pyr, pzr, px, py, pz, prof, taper);
  const float dt = c.dt;
  vx = vx + dt * (ax - prof * vx);
  vy = vy + dt * (ay - prof * vy);
  vz = vz + dt * (az - prof * vz);
  V[0] = taper * vx; V[c.G] = taper * vy; V[2 * c.G] = taper * vz;
}

// ---------------------------------------------------------------------------------------
// k_receivers: one warp per receiver; Lagrange interpolation of the pre-update local
// velocity (ses3d_output.f90:475-493). Fixed lane order + xor tree: deterministic.
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_receivers(const Consts c, const float *__restrict__ v,
                                                   const int *__restrict__ rec_elem, const int *__restrict__ rec_ev,
                                                   const float *__restrict__ rec_w, float *__restrict__ seis, int R,
                                                   const int *__restrict__ d_it) {
  const int r = blockIdx.x * 4 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= R) return;
  const int it = *d_it + 1;
  const long long e = rec_elem[r];
  const int ev = rec_ev[r];
  const int i = (int)(e % c.ex), j = (int)((e / c.ex) % c.ey), k = (int)(e / ((long long)c.ex * c.ey));
  const float *V = v + (long long)ev * 3 * c.G;
  float ax = 0.f, ay = 0.f, az = 0.f;
  for (int n = lane; n < 125; n += 32) {
    const int in = n % 5, jn = (n / 5) % 5, kn = n / 25;
    const long long g = (long long)(i * 4 + in) + (long long)c.GX * ((j * 4 + jn) + (long long)c.GY * (k * 4 + kn));
    const float w = rec_w[(long long)r * 125 + n];
    ax = fmaf(V[g], w, ax); ay = fmaf(V[c.G + g], w, ay); az = fmaf(V[2 * c.G + g], w, az);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ax += __shfl_xor_sync(0xffffffffu, ax, o);
    ay += __shfl_xor_sync(0xffffffffu, ay, o);
    az += __shfl_xor_sync(0xffffffffu, az, o);
  }
  if (lane == 0 && it <= c.nt) {
    seis[((long long)0 * c.nt + (it - 1)) * R + r] = ax;
    seis[((long long)1 * c.nt + (it - 1)) * R + r] = ay;
    seis[((long long)2 * c.nt + (it - 1)) * R + r] = az;
  }
}

// ---------------------------------------------------------------------------------------
// k_inject: point forces into the element forces, one CTA per (event, element) group,
// sources of a group applied in file order (ses3d_miscellaneous.f90:33-90).
// group = {event, element, first source, end source}; stf = [source][3][nt]; mask bit c
// selects the components a source drives (single force: one; adjoint source: all three).
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_inject(const Consts c, float *__restrict__ f, const int4 *__restrict__ groups,
                                                const float *__restrict__ delta, const float *__restrict__ stf,
                                                const int *__restrict__ mask, const int *__restrict__ d_it) {
  const int4 gr = groups[blockIdx.x];
  const int n = threadIdx.x;
  if (n >= 125) return;
  const int it = *d_it + 1;
  const long long N = c.N;
  const int e = gr.y, i = e % c.ex, j = (e / c.ex) % c.ey, k = e / (c.ex * c.ey);
  float *F = f + (long long)gr.x * 3 * N + force_offset(c, i, j, k, n % 5, (n / 5) % 5, n / 25);
  float fx = F[0], fy = F[125], fz = F[250];
  for (int s = gr.z; s < gr.w; ++s) {
    const float d = delta[(long long)s * 125 + n];
    const float *S = stf + (long long)s * 3 * c.nt + (it - 1);
    const int m = mask[s];
    if (m & 1) fx = fx - d * S[0];
    if (m & 2) fy = fy - d * S[c.nt];
    if (m & 4) fz = fz - d * S[2 * c.nt];
  }
  F[0] = fx; F[125] = fy; F[250] = fz;
}

// ---------------------------------------------------------------------------------------
// Layout conversion between the reference layout (element fastest: idx = e + E n) and
// the internal element-major layout (idx = e*125 + n): 32x32 tiled transpose.
// in is rows x cols row-major, out is cols x rows row-major.
// ---------------------------------------------------------------------------------------
__global__ void k_transpose(const float *__restrict__ in, float *__restrict__ out, long long rows, long long cols) {
  __shared__ float tile[32][33];
  const long long c0 = (long long)blockIdx.x * 32, r0 = (long long)blockIdx.y * 32;
  for (int t = threadIdx.y; t < 32; t += blockDim.y) {
    const long long rr = r0 + t, cc = c0 + threadIdx.x;
    if (rr < rows && cc < cols) tile[t][threadIdx.x] = in[rr * cols + cc];
  }
  __syncthreads();
  for (int t = threadIdx.y; t < 32; t += blockDim.y) {
    const long long cc = c0 + t, rr = r0 + threadIdx.x;
    if (rr < rows && cc < cols) out[cc * rows + rr] = tile[threadIdx.x][t];
  }
}

// ACC: out += transposed in (out's old value first), else out = transposed in.
template <bool ACC>
__global__ void k_transpose_d(const double *__restrict__ in, double *__restrict__ out, long long rows, long long cols) {
  __shared__ double tile[32][33];
  const long long c0 = (long long)blockIdx.x * 32, r0 = (long long)blockIdx.y * 32;
  for (int t = threadIdx.y; t < 32; t += blockDim.y) {
    const long long rr = r0 + t, cc = c0 + threadIdx.x;
    if (rr < rows && cc < cols) tile[t][threadIdx.x] = in[rr * cols + cc];
  }
  __syncthreads();
  for (int t = threadIdx.y; t < 32; t += blockDim.y) {
    const long long cc = c0 + t, rr = r0 + threadIdx.x;
    if (rr < rows && cc < cols) {
      if (ACC) out[cc * rows + rr] = out[cc * rows + rr] + tile[threadIdx.x][t];
      else out[cc * rows + rr] = tile[threadIdx.x][t];
    }
  }
}

// ---------------------------------------------------------------------------------------
// Misfit gradient from an event-summed kernel K (reference layout (i,j,k,in,jn,kn), FP64):
// out[q] = (K[q] * W[q]) * s, divided by div[q] when div is given, rounded to T. W is the
// quadrature volume w_in w_jn w_kn Jac r^2 sin(theta) of GLL point q, assembled from three
// FP64 tables: coef[kn][jn][in] = ((w_in w_jn) w_kn) Jac, r2[kn][k] = r^2,
// sinx[in][i] = sin(theta), as W = (coef * r2) * sinx.
// ---------------------------------------------------------------------------------------
template <typename T>
__global__ void k_misfit_gradient(const double *__restrict__ K, const double *__restrict__ coef,
                                  const double *__restrict__ r2, const double *__restrict__ sinx, int ex, int ey,
                                  int ez, double s, const T *__restrict__ div, T *__restrict__ out, long long N) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= N) return;
  long long t = q;
  const int i = (int)(t % ex); t /= ex;
  t /= ey;                                   // j: W does not depend on it
  const int k = (int)(t % ez); t /= ez;
  const int in = (int)(t % 5); t /= 5;
  const int jn = (int)(t % 5);
  const int kn = (int)(t / 5);
  const double W = (coef[(kn * 5 + jn) * 5 + in] * r2[(long long)kn * ez + k]) * sinx[(long long)in * ex + i];
  double g = (K[q] * W) * s;
  if (div) g = g / (double)div[q];
  out[q] = (T)g;
}

// ---------------------------------------------------------------------------------------
// Model derivation (SOURCE/ses3d_input.f90:499, SOURCE/ses3d_init.f90:47-61; rounding as
// the reference, no contraction) fused with the change of layout. In: the model records
// rec[0..6] = rhoinv, mu, lambda, A, B, C, Q in the reference layout (element fastest:
// index e + E n; Q may be null without attenuation). Out: the stress-rate coefficients
// element-blocked, mat[e][NMAT][128] (nodes 125..127 zero), and the adjoint quantities
// gm[f][e * 125 + n]. One 32 x 32 tile (elements e0.., nodes n0..) per 256-thread CTA:
// reads coalesced along e, writes along n through shared memory. grid (ceil(E / 32),
// node tiles) from node tile y0; block (32, 8).
// ---------------------------------------------------------------------------------------
struct ModelRecords {
  const float *r[7];
};

__device__ __forceinline__ void derive_point(const ModelRecords &m, long long q, int is_diss, float sum_D_p,
                                             float out[NMAT + NGMAT]) {
  const float rhoinv = m.r[0][q], mu = m.r[1][q], lam = m.r[2][q];
  const float A = m.r[3][q], B = m.r[4][q], C = m.r[5][q];
  const float kappa = __fadd_rn(lam, __fdiv_rn(__fmul_rn(2.f, mu), 3.f));
  float tau = 0.f, QQ = 0.f, mu_tau = 0.f;
  if (is_diss) {
    QQ = m.r[6][q];
    tau = __fdiv_rn(1.f, QQ);
    mu_tau = __fmul_rn(__fadd_rn(1.f, __fmul_rn(sum_D_p, tau)), mu);
    out[M_CLAM] = __fsub_rn(kappa, __fdiv_rn(__fmul_rn(2.f, mu_tau), 3.f));
    out[M_C2MUT] = __fmul_rn(2.f, mu_tau);
    out[M_C2MT] = __fmul_rn(__fmul_rn(2.f, mu), tau);
  } else {
    out[M_CLAM] = lam;
    out[M_C2MUT] = __fmul_rn(2.f, mu);
    out[M_C2MT] = 0.f;
  }
  out[M_A] = A;
  out[M_B2] = __fmul_rn(2.f, B);
  out[M_C] = C;
  out[NMAT + G_CS] = sqrtf(__fmul_rn(mu, rhoinv));
  out[NMAT + G_CP] = sqrtf(__fmul_rn(__fadd_rn(lam, __fmul_rn(2.f, mu)), rhoinv));
  out[NMAT + G_RHO] = rhoinv > 0.f ? __fdiv_rn(1.f, rhoinv) : 0.f;
  out[NMAT + G_MU] = mu;
  out[NMAT + G_KAPPA] = kappa;
  out[NMAT + G_QQ] = QQ;
}

__global__ void __launch_bounds__(256) k_derive_blocked(const ModelRecords m, float *__restrict__ mat,
                                                        float *__restrict__ gm, long long E, int y0, int is_diss,
                                                        float sum_D_p, int *__restrict__ aniso) {
  __shared__ float tile[NMAT][32][33];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const long long e0 = (long long)blockIdx.x * 32;
  const int n0 = (y0 + (int)blockIdx.y) * 32;
  const long long N = E * 125;
  float v[4][NMAT + NGMAT];
  bool nz = false;  // a non-zero (or NaN) A, B or C
#pragma unroll
  for (int a = 0; a < 4; ++a) {  // node n0 + ty + 8 a of element e0 + tx
    const int n = n0 + ty + 8 * a;
    const long long e = e0 + tx;
    if (n < 125 && e < E) {
      derive_point(m, (long long)n * E + e, is_diss, sum_D_p, v[a]);
      nz = nz || !(v[a][M_A] == 0.f) || !(v[a][M_B2] == 0.f) || !(v[a][M_C] == 0.f);
    } else {
#pragma unroll
      for (int f = 0; f < NMAT + NGMAT; ++f) v[a][f] = 0.f;
    }
  }
  if (__any_sync(0xffffffffu, nz) && tx == 0) atomicOr(aniso, 1);  // a warp is one row ty
#pragma unroll
  for (int half = 0; half < 2; ++half) {  // coefficients, then the adjoint quantities
    if (half) __syncthreads();
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int f = 0; f < NMAT; ++f) tile[f][ty + 8 * a][tx] = v[a][half * NMAT + f];
    __syncthreads();
#pragma unroll
    for (int a = 0; a < 4; ++a) {  // element e0 + ty + 8 a, node n0 + tx
      const long long e = e0 + ty + 8 * a;
      const int n = n0 + tx;
      if (e >= E) continue;
      if (half == 0 && n < MAT_ROW) {
#pragma unroll
        for (int f = 0; f < NMAT; ++f) mat[e * ELEM_MAT + f * MAT_ROW + n] = tile[f][tx][ty + 8 * a];
      } else if (half == 1 && n < 125) {
#pragma unroll
        for (int f = 0; f < NGMAT; ++f) gm[f * N + e * 125 + n] = tile[f][tx][ty + 8 * a];
      }
    }
  }
}

// Element-blocked fields <-> the reference layout, as a 32 x 32 shared-memory transpose:
// blocked[e * stride + off + n] (n < 125) <-> ref[n * E + e].
// grid (ceil(E / 32), 4, nfields); field z uses off + z * field_step and ref + z * 125 E.
__global__ void k_blocked_ref(float *__restrict__ blocked, long long stride, long long off, long long field_step,
                              float *__restrict__ ref, long long E, int to_ref) {
  __shared__ float tile[32][33];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const long long e0 = (long long)blockIdx.x * 32;
  const int n0 = blockIdx.y * 32;
  float *blk = blocked + off + (long long)blockIdx.z * field_step;
  float *rf = ref + (long long)blockIdx.z * 125 * E;
  if (!to_ref) {
    for (int r = ty; r < 32; r += 8) {
      const int n = n0 + r;
      const long long e = e0 + tx;
      tile[r][tx] = (n < 125 && e < E) ? rf[(long long)n * E + e] : 0.f;
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
      const long long e = e0 + r;
      const int n = n0 + tx;
      if (e < E && n < 125) blk[e * stride + n] = tile[tx][r];
    }
  } else {
    for (int r = ty; r < 32; r += 8) {
      const long long e = e0 + r;
      const int n = n0 + tx;
      if (e < E && n < 125) tile[tx][r] = blk[e * stride + n];
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
      const int n = n0 + r;
      const long long e = e0 + tx;
      if (n < 125 && e < E) rf[(long long)n * E + e] = tile[r][tx];
    }
  }
}

// Compact state of a lean run (checkpoints): fields 0-5 and 18-35 of every element, 24 x 125
// floats per element, then fields 6-17 (mirror stresses, displacement gradients) of the PML
// elements in the order of pml_el; lean iterations read no others. to_ck: state -> ck, else
// ck -> state (the fields left out keep what they held).
__global__ void k_compact_state(const Consts c, float *__restrict__ state, float *__restrict__ ck,
                                const int *__restrict__ pml_el, long long npml, int to_ck) {
  const long long partA = (long long)c.nev * c.E * 24 * 125, partB = (long long)c.nev * npml * 12 * 125;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < partA + partB;
       q += (long long)gridDim.x * blockDim.x) {
    long long s;
    if (q < partA) {
      const long long r = q / 125, n = q - r * 125;
      const long long el = r / 24, fi = r - el * 24;
      s = (el * NSTATE + (fi < 6 ? fi : fi + 12)) * 125 + n;
    } else {
      const long long q2 = q - partA, r = q2 / 125, n = q2 - r * 125;
      const long long r2 = r / 12, fi = r - r2 * 12;
      const long long ev = r2 / npml, pe = r2 - ev * npml;
      s = ((ev * c.E + pml_el[pe]) * NSTATE + 6 + fi) * 125 + n;
    }
    if (to_ck) ck[q] = state[s];
    else state[s] = ck[q];
  }
}

// Mirror stresses of the elements outside the PML from their partners (syx = sxy,
// szx = sxz, szy = syz there), after lean iterations that left them out.
__global__ void k_sync_mirrors(const Consts c, float *__restrict__ state) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;  // (event, element, node)
  if (q >= (long long)c.nev * c.E * 125) return;
  const long long el = q / 125;
  const int n = (int)(q - el * 125);
  const unsigned e = (unsigned)(el % c.E);
  const int i = (int)(e % (unsigned)c.ex), j = (int)((e / (unsigned)c.ex) % (unsigned)c.ey);
  const int k = (int)(e / ((unsigned)c.ex * (unsigned)c.ey));
  if (in_pml_element(c, i, j, k)) return;
  float *S = state + el * ELEM_STATE + n;
  S[F_SYX * 125] = S[F_SXY * 125];
  S[F_SZX * 125] = S[F_SXZ * 125];
  S[F_SZY * 125] = S[F_SYZ * 125];
}

// Mass matrix (SOURCE/ses3d_init.f90:254-279): each global node sums its element
// contributions in the reference loop order with IEEE round-to-nearest products, so
// the result is bit-identical to the reference's FP32 MM_global. rhoinv in reference layout.
__global__ void k_mass(const Consts c, const float *__restrict__ rhoinv, const float *__restrict__ z,
                       const float *__restrict__ sinx, const float *__restrict__ w, float Jac, float *__restrict__ MM,
                       float *__restrict__ iMM) {
  const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= c.G) return;
  const int gx = (int)(g % c.GX);
  const int gy = (int)((g / c.GX) % c.GY);
  const int gz = (int)(g / ((long long)c.GX * c.GY));
  const int i0 = gx == 0 ? 0 : (gx - 1) >> 2, i1 = min(gx >> 2, c.ex - 1);
  const int j0 = gy == 0 ? 0 : (gy - 1) >> 2, j1 = min(gy >> 2, c.ey - 1);
  const int k0 = gz == 0 ? 0 : (gz - 1) >> 2, k1 = min(gz >> 2, c.ez - 1);
  float mm = 0.f;
  for (int i = i0; i <= i1; ++i)
    for (int j = j0; j <= j1; ++j)
      for (int k = k0; k <= k1; ++k) {
        const int l = gx - 4 * i, m = gy - 4 * j, n = gz - 4 * k;
        const long long e = (long long)i + (long long)c.ex * (j + (long long)c.ey * k);
        const long long q = e + c.E * (l + 5 * (m + 5 * n));
        const float zz = z[k * 5 + n];
        float t = __fmul_rn(__fmul_rn(w[l], w[m]), w[n]);
        t = __fmul_rn(t, Jac);
        t = __fmul_rn(t, zz);
        t = __fmul_rn(t, zz);
        t = __fmul_rn(t, sinx[i * 5 + l]);
        t = __fdiv_rn(t, rhoinv[q]);
        mm = __fsub_rn(mm, t);
      }
  MM[g] = mm;
  iMM[g] = __frcp_rn(mm);
}

// Max |v| per event (NaN-aware watchdog). out: [nev] as float bits, non-negative.
__global__ void k_vmax(const float *__restrict__ v, long long G3, unsigned int *__restrict__ out) {
  const int ev = blockIdx.y;
  float m = 0.f;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < G3; q += (long long)gridDim.x * blockDim.x) {
    const float a = fabsf(v[(long long)ev * G3 + q]);
    m = (a != a) ? __int_as_float(0x7f800000) : fmaxf(m, a);
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out + ev, __float_as_uint(m));
}

// Normalisation of the Q kernels after the last iteration (ses3d_grad_Q.f90:151-158).
__global__ void k_grad_q_norm(const Consts c, const float *__restrict__ gm, double *__restrict__ grad) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int ev = blockIdx.y;
  if (q >= c.N) return;
  const long long N = c.N;
  double *G = grad + (long long)ev * NGRAD * N + q;
  const double mu = gm[G_MU * N + q], kappa = gm[G_KAPPA * N + q], QQ = gm[G_QQ * N + q];
  const double alpha = 0.3, Q_kappa = 57823.0;
  G[4 * N] = 2.0 * mu * G[4 * N] / QQ;
  G[5 * N] = -2.0 * alpha * mu * G[5 * N] / QQ;
  G[6 * N] = kappa * G[6 * N] / Q_kappa;
  G[5 * N] = -alpha * kappa * G[7 * N] / Q_kappa;  // the reference overwrites grad_alpha_mu here
}

// ---------------------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------------------
template <bool DISS, int MODE, int EPB>
static cudaError_t launch_elem(const Consts &c, const Ptrs &p, cudaStream_t st) {
  dim3 grid((unsigned)((c.ex + EPB - 1) / EPB), (unsigned)c.ey, (unsigned)(c.ez * c.nev));
  k_element<DISS, MODE, EPB><<<grid, TPE * EPB, 0, st>>>(c, p);
  return cudaGetLastError();
}

template <bool DISS, int MODE>
static cudaError_t launch_elem_epb(int epb, const Consts &c, const Ptrs &p, cudaStream_t st) {
  switch (epb) {
    case 2: return launch_elem<DISS, MODE, 2>(c, p, st);
    case 4: return launch_elem<DISS, MODE, 4>(c, p, st);
    default: return launch_elem<DISS, MODE, 1>(c, p, st);
  }
}

// Block shapes of the persistent element kernel selectable at run time (the autotuner's
// search space): {resident CTAs per SM, refill point}.
constexpr int kTmaShapes = 4;
template <int S> struct TmaShape;
template <> struct TmaShape<0> { static constexpr int minb = 5, refill = 0; };  // measured default
template <> struct TmaShape<1> { static constexpr int minb = 4, refill = 0; };
template <> struct TmaShape<2> { static constexpr int minb = 6, refill = 0; };
template <> struct TmaShape<3> { static constexpr int minb = 5, refill = 1; };

// Resident CTAs of one instantiation of k_element_tma on the current device (set by prepare_tma).
template <bool DISS, int MODE, int S, bool PACK = false>
static int &tma_grid_cap() {
  static int cap = 0;
  return cap;
}
template <bool DISS, int MODE, int S, bool PACK = false>
static cudaError_t prepare_tma() {
  auto kern = k_element_tma<DISS, MODE, TmaShape<S>::minb, TmaShape<S>::refill, PACK>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tma_smem(MODE));
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0, per_sm = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TPE, tma_smem(MODE));
  if (e != cudaSuccess) return e;
  tma_grid_cap<DISS, MODE, S, PACK>() = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
  return cudaSuccess;
}
template <int S>
static cudaError_t prepare_tma_shape() {
  cudaError_t e;
  if ((e = prepare_tma<false, 0, S>()) != cudaSuccess) return e;
  if ((e = prepare_tma<false, 3, S>()) != cudaSuccess) return e;
  if ((e = prepare_tma<true, 0, S>()) != cudaSuccess) return e;
  return prepare_tma<true, 3, S>();
}
// Sets the shared-memory limit and grid size of the persistent element kernels; called
// when a handle is created, before any stream capture.
cudaError_t prepare_element_kernels() {
  cudaError_t e;
  if ((e = prepare_tma<false, 1, 0>()) != cudaSuccess) return e;
  if ((e = prepare_tma<false, 2, 0>()) != cudaSuccess) return e;
  if ((e = prepare_tma<true, 1, 0>()) != cudaSuccess) return e;
  if ((e = prepare_tma<true, 2, 0>()) != cudaSuccess) return e;
  if ((e = prepare_tma<false, 4, 1>()) != cudaSuccess) return e;
  if ((e = prepare_tma<false, 5, 1>()) != cudaSuccess) return e;
  if ((e = prepare_tma<true, 4, 1>()) != cudaSuccess) return e;
  if ((e = prepare_tma<true, 5, 1>()) != cudaSuccess) return e;
  if ((e = prepare_tma<false, 0, 0, true>()) != cudaSuccess) return e;
  if ((e = prepare_tma<false, 3, 0, true>()) != cudaSuccess) return e;
  if ((e = prepare_tma<true, 0, 0, true>()) != cudaSuccess) return e;
  if ((e = prepare_tma<true, 3, 0, true>()) != cudaSuccess) return e;
  if ((e = prepare_tma_shape<0>()) != cudaSuccess) return e;
  if ((e = prepare_tma_shape<1>()) != cudaSuccess) return e;
  if ((e = prepare_tma_shape<2>()) != cudaSuccess) return e;
  return prepare_tma_shape<3>();
}

template <bool DISS, int MODE, int S, bool PACK = false>
static cudaError_t launch_tma(const Consts &c, const Ptrs &p, cudaStream_t st) {
  const int grid_cap = tma_grid_cap<DISS, MODE, S, PACK>();
  if (grid_cap <= 0) return cudaErrorInitializationError;
  const long long total = c.E * (long long)c.nev;
  const unsigned blocks = (unsigned)(total < grid_cap ? total : grid_cap);
  k_element_tma<DISS, MODE, TmaShape<S>::minb, TmaShape<S>::refill, PACK><<<blocks, TPE, tma_smem(MODE), st>>>(c, p);
  return cudaGetLastError();
}

template <bool DISS, int MODE>
static cudaError_t launch_tma_shape(int shape, const Consts &c, const Ptrs &p, cudaStream_t st) {
  switch (shape) {
    case 1: return launch_tma<DISS, MODE, 1>(c, p, st);
    case 2: return launch_tma<DISS, MODE, 2>(c, p, st);
    case 3: return launch_tma<DISS, MODE, 3>(c, p, st);
    default: return launch_tma<DISS, MODE, 0>(c, p, st);
  }
}

int element_shape_count() { return kTmaShapes; }

// shape: block shape of the persistent kernel (epb 1); epb 2, 4: register-staged kernel.
// Record (1) and correlation (2) iterations run the persistent kernel in the default shape
// 0 (they are one iteration in samp_ad; the searched shapes serve the plain iterations).
// With p.slot set (plain or lean iterations), the persistent kernel in shape 0 also packs
// each item's starting state into the slot, whatever epb and shape say.
// Lean handles map modes 0, 1, 2 to 3, 4, 5; modes 4 and 5 (they need p.u) run the
// persistent kernel in shape 1 (4 CTAs per SM: their displacement contraction needs the
// registers).
cudaError_t launch_element(int diss, int mode, int epb, int shape, const Consts &c, const Ptrs &p, cudaStream_t st) {
  if (c.lean && mode <= 2) mode += 3;
  if (mode == 4 || mode == 5) {
    if (!p.u) return cudaErrorInvalidValue;
    if (mode == 4) return diss ? launch_tma<true, 4, 1>(c, p, st) : launch_tma<false, 4, 1>(c, p, st);
    return diss ? launch_tma<true, 5, 1>(c, p, st) : launch_tma<false, 5, 1>(c, p, st);
  }
  if (p.slot) {
    if (mode == 0) return diss ? launch_tma<true, 0, 0, true>(c, p, st) : launch_tma<false, 0, 0, true>(c, p, st);
    if (mode == 3) return diss ? launch_tma<true, 3, 0, true>(c, p, st) : launch_tma<false, 3, 0, true>(c, p, st);
    return cudaErrorInvalidValue;
  }
  if (epb <= 1) {  // persistent bulk-copy-pipelined kernel
    if (mode == 1) return diss ? launch_tma<true, 1, 0>(c, p, st) : launch_tma<false, 1, 0>(c, p, st);
    if (mode == 2) return diss ? launch_tma<true, 2, 0>(c, p, st) : launch_tma<false, 2, 0>(c, p, st);
    if (diss) return mode == 3 ? launch_tma_shape<true, 3>(shape, c, p, st) : launch_tma_shape<true, 0>(shape, c, p, st);
    return mode == 3 ? launch_tma_shape<false, 3>(shape, c, p, st) : launch_tma_shape<false, 0>(shape, c, p, st);
  }
  if (diss) {
    if (mode == 1) return launch_elem_epb<true, 1>(epb, c, p, st);
    if (mode == 2) return launch_elem_epb<true, 2>(epb, c, p, st);
    if (mode == 3) return launch_elem_epb<true, 3>(epb, c, p, st);
    return launch_elem_epb<true, 0>(epb, c, p, st);
  }
  if (mode == 1) return launch_elem_epb<false, 1>(epb, c, p, st);
  if (mode == 2) return launch_elem_epb<false, 2>(epb, c, p, st);
  if (mode == 3) return launch_elem_epb<false, 3>(epb, c, p, st);
  return launch_elem_epb<false, 0>(epb, c, p, st);
}

template <int KIND, int TPB, int MINB>
static cudaError_t launch_node_tpb(const Consts &c, const Ptrs &p, cudaStream_t st) {
  dim3 grid((unsigned)(((long long)c.GX * c.GY + TPB - 1) / TPB), (unsigned)c.GZ, (unsigned)c.nev);
  k_node<KIND, TPB, MINB><<<grid, TPB, 0, st>>>(c, p);
  return cudaGetLastError();
}

// node_block: threads per CTA of the node kernel, 128, 256 (default) or 512, each with the
// resident CTAs per SM that fill 1,536-1,792 thread slots.
template <int KIND>
static cudaError_t launch_node_shape(int node_block, const Consts &c, const Ptrs &p, cudaStream_t st) {
  if (node_block == 128) return launch_node_tpb<KIND, 128, 14>(c, p, st);
  if (node_block == 512) return launch_node_tpb<KIND, 512, 3>(c, p, st);
  return launch_node_tpb<KIND, SES3D_NODE_TPB, SES3D_NODE_MINB>(c, p, st);
}

// With p.fg the assembled forces are stored too; with p.u the displacement is integrated.
cudaError_t launch_node(int node_block, const Consts &c, const Ptrs &p, cudaStream_t st) {
  if (p.fg && p.u) return cudaErrorInvalidValue;
  if (p.fg) return launch_node_shape<1>(node_block, c, p, st);
  if (p.u) return launch_node_shape<2>(node_block, c, p, st);
  return launch_node_shape<0>(node_block, c, p, st);
}

cudaError_t launch_receivers(const Consts &c, const float *v, const int *rec_elem, const int *rec_ev,
                             const float *rec_w, float *seis, int R, const int *d_it, cudaStream_t st) {
  if (R <= 0) return cudaSuccess;
  k_receivers<<<(R + 3) / 4, 128, 0, st>>>(c, v, rec_elem, rec_ev, rec_w, seis, R, d_it);
  return cudaGetLastError();
}

cudaError_t launch_inject(const Consts &c, float *f, const int4 *groups, int ngroups, const float *delta,
                          const float *stf, const int *mask, const int *d_it, cudaStream_t st) {
  if (ngroups <= 0) return cudaSuccess;
  k_inject<<<ngroups, 128, 0, st>>>(c, f, groups, delta, stf, mask, d_it);
  return cudaGetLastError();
}

cudaError_t launch_transpose(const float *in, float *out, long long rows, long long cols, cudaStream_t st) {
  dim3 grid((unsigned)((cols + 31) / 32), (unsigned)((rows + 31) / 32));
  k_transpose<<<grid, dim3(32, 8), 0, st>>>(in, out, rows, cols);
  return cudaGetLastError();
}

// Sum over events of one kernel slot, events in index order (deterministic).
__global__ void k_sum_events_d(const double *__restrict__ grad, int slot, int nev, long long N,
                               double *__restrict__ out) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= N) return;
  double s = 0.0;
  for (int ev = 0; ev < nev; ++ev) s += grad[((long long)ev * NGRAD + slot) * N + q];
  out[q] = s;
}

cudaError_t launch_sum_events_d(const double *grad, int slot, int nev, long long N, double *out, cudaStream_t st) {
  k_sum_events_d<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(grad, slot, nev, N, out);
  return cudaGetLastError();
}

cudaError_t launch_transpose_d(const double *in, double *out, long long rows, long long cols, bool accumulate,
                               cudaStream_t st) {
  dim3 grid((unsigned)((cols + 31) / 32), (unsigned)((rows + 31) / 32));
  if (accumulate) k_transpose_d<true><<<grid, dim3(32, 8), 0, st>>>(in, out, rows, cols);
  else k_transpose_d<false><<<grid, dim3(32, 8), 0, st>>>(in, out, rows, cols);
  return cudaGetLastError();
}

cudaError_t launch_misfit_gradient(const double *K, const double *tables, int ex, int ey, int ez, double s,
                                   const void *div, void *out, bool f64, cudaStream_t st) {
  const long long N = (long long)ex * ey * ez * 125;
  const double *coef = tables, *r2 = tables + 125, *sinx = r2 + 5LL * ez;
  const unsigned blocks = (unsigned)((N + 255) / 256);
  if (f64)
    k_misfit_gradient<double><<<blocks, 256, 0, st>>>(K, coef, r2, sinx, ex, ey, ez, s, (const double *)div,
                                                      (double *)out, N);
  else
    k_misfit_gradient<float><<<blocks, 256, 0, st>>>(K, coef, r2, sinx, ex, ey, ez, s, (const float *)div,
                                                     (float *)out, N);
  return cudaGetLastError();
}

// Node tiles y0 .. y1 - 1 (32 nodes each, 4 tiles cover 0..127) of the fused model
// derivation; rec: the 7 model records (reference layout), Q null without attenuation.
cudaError_t launch_derive_blocked(const float *const rec[7], float *mat, float *gm, long long E, int y0, int y1,
                                  int is_diss, float sum_D_p, int *aniso, cudaStream_t st) {
  if (y0 < 0 || y1 > 4 || y0 >= y1) return cudaErrorInvalidValue;
  ModelRecords m;
  for (int k = 0; k < 7; ++k) m.r[k] = rec[k];
  k_derive_blocked<<<dim3((unsigned)((E + 31) / 32), (unsigned)(y1 - y0)), dim3(32, 8), 0, st>>>(
      m, mat, gm, E, y0, is_diss, sum_D_p, aniso);
  return cudaGetLastError();
}

cudaError_t launch_mass(const Consts &c, const float *rhoinv, const float *z, const float *sinx, const float *w,
                        float Jac, float *MM, float *iMM, cudaStream_t st) {
  k_mass<<<(unsigned)((c.G + 255) / 256), 256, 0, st>>>(c, rhoinv, z, sinx, w, Jac, MM, iMM);
  return cudaGetLastError();
}

cudaError_t launch_state_field(float *state_ev, int field, float *ref, long long E, int to_ref, cudaStream_t st) {
  k_blocked_ref<<<dim3((unsigned)((E + 31) / 32), 4, 1), dim3(32, 8), 0, st>>>(
      state_ev, ELEM_STATE, (long long)field * 125, 0, ref, E, to_ref);
  return cudaGetLastError();
}

cudaError_t launch_compact_state(const Consts &c, float *state, float *ck, const int *pml_el, long long npml, int to_ck,
                                 cudaStream_t st) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  k_compact_state<<<(unsigned)((sms > 0 ? sms : 1) * 8), 256, 0, st>>>(c, state, ck, pml_el, npml, to_ck);
  return cudaGetLastError();
}

cudaError_t launch_sync_mirrors(const Consts &c, float *state, cudaStream_t st) {
  const long long n = (long long)c.nev * c.E * 125;
  k_sync_mirrors<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(c, state);
  return cudaGetLastError();
}

// Self-test of the bounded wait: one CTA arms an mbarrier for 16 bytes that no copy ever
// delivers and waits on it with the element kernel's wait; the wait must give up after
// limit_ns and leave its code in *err. No copy is in flight when the CTA exits.
__global__ void k_wait_selftest(int *err, unsigned long long limit_ns) {
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    mbar_arrive_expect_tx(&bar, 16u);
    mbar_wait_bounded(&bar, 0u, err, limit_ns);
  }
}

cudaError_t launch_wait_selftest(int *err, unsigned long long limit_ns, cudaStream_t st) {
  k_wait_selftest<<<1, 32, 0, st>>>(err, limit_ns);
  return cudaGetLastError();
}

cudaError_t launch_vmax(const float *v, long long G3, int nev, unsigned int *out, cudaStream_t st) {
  dim3 grid(304, (unsigned)nev);
  k_vmax<<<grid, 256, 0, st>>>(v, G3, out);
  return cudaGetLastError();
}

cudaError_t launch_grad_q_norm(const Consts &c, const float *gm, double *grad, cudaStream_t st) {
  dim3 grid((unsigned)((c.N + 255) / 256), (unsigned)c.nev);
  k_grad_q_norm<<<grid, 256, 0, st>>>(c, gm, grad);
  return cudaGetLastError();
}

// Local (gathered) form of a global field in the reference layout (ses3d_evolution.f90:27-51).
__global__ void k_gather_ref(const Consts c, const float *__restrict__ v, float *__restrict__ out) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= c.N) return;
  const long long e = q % c.E;
  const int n = (int)(q / c.E);
  const int in = n % 5, jn = (n / 5) % 5, kn = n / 25;
  const int i = (int)(e % c.ex), j = (int)((e / c.ex) % c.ey), k = (int)(e / ((long long)c.ex * c.ey));
  out[q] = v[(long long)(i * 4 + in) + (long long)c.GX * ((j * 4 + jn) + (long long)c.GY * (k * 4 + kn))];
}

cudaError_t launch_gather_ref(const Consts &c, const float *v, float *out, cudaStream_t st) {
  k_gather_ref<<<(unsigned)((c.N + 255) / 256), 256, 0, st>>>(c, v, out);
  return cudaGetLastError();
}

}  // namespace ses3d

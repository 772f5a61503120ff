// adjoint.cu -- exact discrete adjoint of the time step (the transpose of one iteration of
// kernels.cu, SOURCE/ses3d_evolution.f90:7-373 as this library computes it), for misfit
// gradients that are the derivative of the discrete forward run itself.
//
// One forward iteration maps the state x = (v_global, 9 PML stresses, 9 displacement
// gradients, 18 memory variables) linearly to the next (plus model-independent source
// terms); the model enters through the six stress-rate coefficients of every GLL point
// (kappa - 2 mu_tau / 3, 2 mu_tau, 2 mu tau, A, 2 B, C) and the reciprocal mass matrix.
// A backward iteration takes the adjoint of the iteration's output state (lambda_t) and the
// forward state before it (x_{t-1}, and the assembled forces F_t the forward iteration
// computed) and produces lambda_{t-1}, adding lambda_t . d(iteration)/d(coefficients) to
// FP64 accumulators. Three launches per iteration, mirroring the forward ones:
//   k_adj_node1    node level, in reverse: taper and leapfrog of v, adjoint of the
//                  assembled forces (dt / MM taper lambda_v), the 1 / MM gradient
//   k_adj_element  element level, in reverse: weak divergence, stress march, stress rates
//                  and memory variables (coefficient gradients), symmetrisation, PML
//                  strain, displacement gradients, spherical terms, strain contraction;
//                  writes each element's contributions to the adjoint velocity
//   k_adj_node2    assembles those contributions (the transpose of the gather) in the
//                  forward node kernel's deterministic order
// Receiver adjoint sources (d misfit / d seismogram) enter between the last two as point
// forces on the element contributions (k_inject), the transpose of the receiver
// interpolation. No atomics: every gradient slot is written by one thread per event.
#include "kernels.cuh"
#include "assembly.cuh"
#include "pipeline.cuh"

namespace ses3d {

// k_adj_node1: per (global node, event).
__global__ void __launch_bounds__(256) k_adj_node1(const Consts c, const Ptrs p, const AdjPtrs a) {
  const int gz = blockIdx.y, ev = blockIdx.z;
  const unsigned GXY = (unsigned)c.GX * (unsigned)c.GY;
  const unsigned t = blockIdx.x * 256u + threadIdx.x;
  if (t >= GXY) return;
  const int gy = node_row(c, t);
  const int gx = (int)t - gy * c.GX;
  const size_t g = (size_t)gz * GXY + t;
  const size_t o = (size_t)ev * 3 * c.G + g;
  float px, py, pz, prof, taper;
  pml_profiles(__ldg(p.pxg + gx), __ldg(p.pyg + gy), __ldg(p.pzg + gz), px, py, pz, prof, taper);
  const float dt = c.dt;
  const float imm = __ldg(p.iMM + g);
  // v' = taper (v + dt (F / MM - prof v))
  const float mx = taper * a.av[o], my = taper * a.av[o + c.G], mz = taper * a.av[o + 2 * c.G];
  const float damp = 1.f - dt * prof;
  const float sF = dt * imm;
  a.aF[o] = sF * mx; a.aF[o + c.G] = sF * my; a.aF[o + 2 * c.G] = sF * mz;
  a.av[o] = damp * mx; a.av[o + c.G] = damp * my; a.av[o + 2 * c.G] = damp * mz;
  // the iteration's term in FP32, accumulated in FP64 (one conversion and one add: FP64
  // issue is scarce on this part)
  const float dF = mx * a.fg[o] + my * a.fg[o + c.G] + mz * a.fg[o + 2 * c.G];
  double *gi = a.gimm + (size_t)ev * c.G + g;
  *gi += (double)(dt * dF);
}

// k_adj_node2: per (global node, event); thread 0 of the grid steps the adjoint counter back.
__global__ void __launch_bounds__(256) k_adj_node2(const Consts c, const AdjPtrs a) {
  const int gz = blockIdx.y, ev = blockIdx.z;
  if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0) *a.d_ait -= 1;
  const unsigned GXY = (unsigned)c.GX * (unsigned)c.GY;
  const unsigned t = blockIdx.x * 256u + threadIdx.x;
  if (t >= GXY) return;
  const int gy = node_row(c, t);
  const int gx = (int)t - gy * c.GX;
  const size_t o = (size_t)ev * 3 * c.G + (size_t)gz * GXY + t;
  float sx, sy, sz;
  gather_node(c, a.af + (size_t)ev * 3 * (size_t)c.N, gx, gy, gz, sx, sy, sz);
  a.av[o] += sx; a.av[o + c.G] += sy; a.av[o + 2 * c.G] += sz;
}

// k_adj_element: persistent, one item (element, event) at a time per 128-thread CTA
// (thread = GLL node), items first + t * gridDim. Thread 0 copies each item's adjoint-state,
// packed-forward-state, material and FP64 gradient blocks into shared memory with
// cp.async.bulk on an mbarrier; the next item's copies are issued as soon as this one's
// are read into registers. The forward velocity and the adjoint of the assembled forces at
// the item's nodes arrive by 4-byte cp.async, one item ahead. Bounded waits as in the
// forward persistent kernel.
struct __align__(16) AdjStage {
  float astate[ELEM_STATE];               // 18,000 B
  float slot[SLOT_FIELDS_DISS * 125 + 1];  // 7,504 B (the elastic block is 4,512 B)
  float mat[ELEM_MAT];                    // 3,072 B
  double gm[NMAT * 125];                  // 6,000 B
};
static_assert(sizeof(AdjStage) == 34576, "AdjStage layout");
static_assert(slot_stride(true) == SLOT_FIELDS_DISS * 125 + 1, "slot stride");
constexpr int ADJ_MINB = 4;
constexpr size_t ADJ_G_OFF = sizeof(AdjStage) + 9 * TPE * sizeof(float);   // gathers [2][6][TPE]
constexpr size_t ADJ_TAB_OFF = ADJ_G_OFF + 12 * TPE * sizeof(float);
constexpr size_t ADJ_BAR_OFF = ADJ_TAB_OFF + ((sizeof(KTab) + 15) / 16) * 16;
constexpr size_t ADJ_SMEM = ADJ_BAR_OFF + sizeof(unsigned long long);

// Copies of one item into the stage. Byte ranges, 16-B aligned inside their blocks:
// adjoint state (18,000 B): all 36 fields; elastic: fields 0-17 (9,008 B); when the item's
// adjoint displacement gradients are left out: fields 0-8 (4,512 B) and, with attenuation,
// 18-35 (from byte 8,992, 9,008 B). Slot (7,504 B; elastic 4,512 B): all of it in PML
// elements; outside, the memory-variable sums only (from byte 4,496, 3,008 B), nothing
// when elastic. Material: 3 or 6 fields (1,536 or 3,072 B). Gradients: 6,000 B.
template <bool DISS>
__device__ __forceinline__ void adj_issue_item(const Consts &c, const Ptrs &p, const AdjPtrs &a, long long item,
                                               AdjStage *st, unsigned long long *bar) {
  const int ev = (int)(item % c.nev);
  const unsigned e = (unsigned)(item / c.nev);
  const int i = (int)(e % (unsigned)c.ex), j = (int)((e / (unsigned)c.ex) % (unsigned)c.ey);
  const int k = (int)(e / ((unsigned)c.ex * (unsigned)c.ey));
  const bool pml = in_pml_element(c, i, j, k);
  const bool skip_ad = !pml && a.zero_d;
  const size_t b = (size_t)ev * c.E + e;
  const char *as = reinterpret_cast<const char *>(a.astate + b * ELEM_STATE);
  const char *sl = reinterpret_cast<const char *>(a.fstate + b * slot_stride(DISS));
  char *das = reinterpret_cast<char *>(st->astate);
  char *dsl = reinterpret_cast<char *>(st->slot);
  const unsigned ab0 = skip_ad ? 4512u : (DISS ? (unsigned)(ELEM_STATE * sizeof(float)) : 9008u);
  const unsigned ab1 = (skip_ad && DISS) ? 9008u : 0u;
  const unsigned s_off = pml ? 0u : 4496u;
  const unsigned sb = DISS ? (pml ? 7504u : 3008u) : (pml ? 4512u : 0u);
  const unsigned mb = (c.iso ? 3 * MAT_ROW : ELEM_MAT) * (unsigned)sizeof(float);
  const unsigned gb = NMAT * 125 * (unsigned)sizeof(double);
  mbar_arrive_expect_tx(bar, ab0 + ab1 + sb + mb + gb);
  bulk_g2s(das, as, ab0, bar);
  if (ab1) bulk_g2s(das + 8992, as + 8992, ab1, bar);
  if (sb) bulk_g2s(dsl + s_off, sl + s_off, sb, bar);
  bulk_g2s(st->mat, p.mat + (size_t)e * ELEM_MAT, mb, bar);
  bulk_g2s(st->gm, a.gmat + b * (NMAT * 125), gb, bar);
}

// The forward velocity and the adjoint of the assembled forces at one item's nodes into
// dst[0..5] (one commit group).
__device__ __forceinline__ void adj_gather_async(const Consts &c, const AdjPtrs &a, long long item, float (*dst)[TPE],
                                                 int n, int in, int jn, int kn) {
  const int ev = (int)(item % c.nev);
  const unsigned e = (unsigned)(item / c.nev);
  const int i = (int)(e % (unsigned)c.ex), j = (int)((e / (unsigned)c.ex) % (unsigned)c.ey);
  const int k = (int)(e / ((unsigned)c.ex * (unsigned)c.ey));
  if (n < 125) {
    const size_t g = (size_t)(i * 4 + in) + (size_t)c.GX * ((size_t)(j * 4 + jn) + (size_t)c.GY * (size_t)(k * 4 + kn));
    const size_t ov = (size_t)ev * 3 * c.G + g;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      cp_async4(&dst[q][n], a.fv + ov + (size_t)q * c.G);
      cp_async4(&dst[3 + q][n], a.aF + ov + (size_t)q * c.G);
    }
  }
  asm volatile("cp.async.commit_group;" ::: "memory");
}

template <bool DISS>
__global__ void __launch_bounds__(TPE, ADJ_MINB) k_adj_element(const Consts c, const Ptrs p, const AdjPtrs a) {
  extern __shared__ __align__(128) unsigned char smem[];
  AdjStage *stage = reinterpret_cast<AdjStage *>(smem);
  float (*s_a)[TPE] = reinterpret_cast<float (*)[TPE]>(smem + sizeof(AdjStage));
  float (*s_g)[TPE] = reinterpret_cast<float (*)[TPE]>(smem + ADJ_G_OFF);  // [2 buffers][6]
  KTab &tab = *reinterpret_cast<KTab *>(smem + ADJ_TAB_OFF);
  unsigned long long *bar = reinterpret_cast<unsigned long long *>(smem + ADJ_BAR_OFF);
  const int n = threadIdx.x;
  const long long total = c.E * (long long)c.nev;
  const long long first = blockIdx.x, stride = gridDim.x;
  if (n == 0) {
    mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int q = n; q < KTAB_FLOATS; q += TPE)
    reinterpret_cast<float *>(&tab)[q] = reinterpret_cast<const float *>(p.ktab)[q];
  __syncthreads();
  if (n == 0 && first < total) adj_issue_item<DISS>(c, p, a, first, stage, bar);
  const bool act = n < 125;
  const int nn = act ? n : 0;
  const int in = nn % 5, jn = (nn / 5) % 5, kn = nn / 25;
  if (first < total) adj_gather_async(c, a, first, s_g, n, in, jn, kn);
  const float dt = c.dt;
  for (int t = 0;; ++t) {
    const long long item = first + (long long)t * stride;
    if (item >= total) break;
    const int ev = (int)(item % c.nev);
    const unsigned e = (unsigned)(item / c.nev);
    const int i = (int)(e % (unsigned)c.ex), j = (int)((e / (unsigned)c.ex) % (unsigned)c.ey);
    const int k = (int)(e / ((unsigned)c.ex * (unsigned)c.ey));
    float (*s_gt)[TPE] = s_g + 6 * (t & 1);
    float *AS = a.astate + ((size_t)ev * c.E + e) * ELEM_STATE + nn;  // adjoint state: lambda_t in, lambda_{t-1} out

    // Outside the PML the profiles are zero: the forward displacement gradients enter nothing
    // there and are neither packed nor read, and adjoint ones that start at zero stay zero.
    const bool pml = in_pml_element(c, i, j, k);
    const bool skip_ad = !pml && a.zero_d;

    // ---- the item's data into registers: gathered velocity and adjoint forces, adjoint
    // state, packed forward state, material, gradient accumulators; then the 1-D tables
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    const bool ok = mbar_wait_bounded(bar, (unsigned)t & 1u, p.err);
    float vx = 0.f, vy = 0.f, vz = 0.f, lF0 = 0.f, lF1 = 0.f, lF2 = 0.f;
    if (act) {
      vx = s_gt[0][n]; vy = s_gt[1][n]; vz = s_gt[2][n];
      lF0 = s_gt[3][n]; lF1 = s_gt[4][n]; lF2 = s_gt[5][n];
    }
    const float *SA = stage->astate + nn;
    const float *SS = stage->slot + nn;
    const float *SM = stage->mat + nn;
    float as_s[9], as_d[9], as_m[DISS ? 18 : 1];
#pragma unroll
    for (int f = 0; f < 9; ++f) as_s[f] = SA[f * 125];
#pragma unroll
    for (int q = 0; q < 9; ++q) as_d[q] = skip_ad ? 0.f : SA[(F_DXUX + q) * 125];
    if (DISS) {
#pragma unroll
      for (int q = 0; q < 18; ++q) as_m[q] = SA[(F_M + q) * 125];
    }
    float fd[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) fd[q] = pml ? SS[q * 125] : 0.f;
    float Md[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // forward memory-variable sums per component
    if (DISS) {
#pragma unroll
      for (int cc = 0; cc < 6; ++cc) Md[cc] = SS[(9 + cc) * 125];
    }
    const float clam = SM[M_CLAM * MAT_ROW], c2mut = SM[M_C2MUT * MAT_ROW];
    const float c2mt = DISS ? SM[M_C2MT * MAT_ROW] : 0.f;
    const float cA = c.iso ? 0.f : SM[M_A * MAT_ROW], cB2 = c.iso ? 0.f : SM[M_B2 * MAT_ROW];
    const float cC = c.iso ? 0.f : SM[M_C * MAT_ROW];
    double gm0[NMAT];
#pragma unroll
    for (int q = 0; q < NMAT; ++q) gm0[q] = stage->gm[q * 125 + nn];
    if (__syncthreads_or(!ok)) {  // a copy never arrived: drain, then leave
      if (n == 0) mbar_wait_bounded(bar, (unsigned)t & 1u, p.err);
      return;
    }
    // the stage and this item's gathers are read: the next item's copies and gathers
    {
      const long long next = item + stride;
      if (next < total) {
        adj_gather_async(c, a, next, s_g + 6 * ((t + 1) & 1), n, in, jn, kn);
        if (n == 0) {
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          adj_issue_item<DISS>(c, p, a, next, stage, bar);
        }
      }
    }
    const float r = __ldg(p.r_z + k * 5 + kn), st = __ldg(p.sin_x + i * 5 + in);
    const float ir = __ldg(p.inv_r + k * 5 + kn);
    const float irs = ir * __ldg(p.inv_sin + i * 5 + in);
    const float ct = __ldg(p.cot_x + i * 5 + in);
    const float pxr = __ldg(p.pxr + i * 5 + in), pyr = __ldg(p.pyr + j * 5 + jn), pzr = __ldg(p.pzr + k * 5 + kn);

    // ---- forward quantities of the iteration (as k_element computes them)
    s_a[0][n] = vx; s_a[1][n] = vy; s_a[2][n] = vz;
    __syncthreads();
    float exx = 0.f, exy = 0.f, exz = 0.f, eyx = 0.f, eyy = 0.f, eyz = 0.f, ezx = 0.f, ezy = 0.f, ezz = 0.f;
#pragma unroll
    for (int q = 0; q < 5; ++q) {
      const int ix = q + 5 * jn + 25 * kn, iy = in + 5 * q + 25 * kn, iz = in + 5 * jn + 25 * q;
      const float dxq = tab.Dx[in][q], dyq = tab.Dy[jn][q], dzq = tab.Dz[kn][q];
      exx = fmaf(s_a[0][ix], dxq, exx); exy = fmaf(s_a[1][ix], dxq, exy); exz = fmaf(s_a[2][ix], dxq, exz);
      eyx = fmaf(s_a[0][iy], dyq, eyx); eyy = fmaf(s_a[1][iy], dyq, eyy); eyz = fmaf(s_a[2][iy], dyq, eyz);
      ezx = fmaf(s_a[0][iz], dzq, ezx); ezy = fmaf(s_a[1][iz], dzq, ezy); ezz = fmaf(s_a[2][iz], dzq, ezz);
    }
    ezz = -ezz;
    eyy = eyy * irs + (vz + vx * ct) * ir;
    exx = (vz + exx) * ir;
    ezx = -ezx;
    exz = (exz - vx) * ir;
    ezy = -ezy;
    eyz = -vy * ir + eyz * irs;
    exy = exy * ir;
    eyx = -vy * ct * ir + eyx * irs;
    float px, py, pz, prof, taper;
    pml_profiles(pxr, pyr, pzr, px, py, pz, prof, taper);
    const float Pxx = pz + py, Pyy = px + pz, Pzz = px + py, Pxy = py + pz, Pyx = px + pz, Pxz = py + pz,
                Pzx = px + py, Pyz = px + pz, Pzy = px + py;
    float es[6];  // PML-modified, symmetrised strain rates of the iteration
    {
      const float dxux = fd[0] + dt * exx, dyuy = fd[1] + dt * eyy;
      const float dzuz = fd[2] + dt * ezz, dxuy = fd[3] + dt * exy;
      const float dyux = fd[4] + dt * eyx, dxuz = fd[5] + dt * exz;
      const float dzux = fd[6] + dt * ezx, dyuz = fd[7] + dt * eyz;
      const float dzuy = fd[8] + dt * ezy;
      es[0] = exx + Pxx * dxux;
      es[1] = eyy + Pyy * dyuy;
      es[2] = ezz + Pzz * dzuz;
      es[3] = ((exy + Pxy * dxuy) + (eyx + Pyx * dyux)) * 0.5f;
      es[4] = ((exz + Pxz * dxuz) + (ezx + Pzx * dzux)) * 0.5f;
      es[5] = ((eyz + Pyz * dyuz) + (ezy + Pzy * dzuy)) * 0.5f;
    }

    // ---- weak divergence, in reverse: lambda of the weighted stresses
    const float cx = tab.CX[jn][kn] * r, cy = tab.CY[in][kn] * r, cz = tab.CZ[in][jn] * st;
    __syncthreads();  // s_a (forward velocity) fully read
    const bool on = act;
    s_a[0][n] = on ? cx * lF0 : 0.f; s_a[1][n] = on ? cx * lF1 : 0.f; s_a[2][n] = on ? cx * lF2 : 0.f;
    s_a[3][n] = on ? cy * lF0 : 0.f; s_a[4][n] = on ? cy * lF1 : 0.f; s_a[5][n] = on ? cy * lF2 : 0.f;
    s_a[6][n] = on ? cz * lF0 : 0.f; s_a[7][n] = on ? cz * lF1 : 0.f; s_a[8][n] = on ? cz * lF2 : 0.f;
    __syncthreads();
    float lsp[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int q = 0; q < 5; ++q) {
      const int ix = q + 5 * jn + 25 * kn, iy = in + 5 * q + 25 * kn, iz = in + 5 * jn + 25 * q;
      const float dxq = tab.dlT[q][in], dyq = tab.dlT[q][jn], dzq = tab.dlT[q][kn];
      lsp[0] = fmaf(s_a[0][ix], dxq, lsp[0]); lsp[1] = fmaf(s_a[1][ix], dxq, lsp[1]);
      lsp[2] = fmaf(s_a[2][ix], dxq, lsp[2]);
      lsp[3] = fmaf(s_a[3][iy], dyq, lsp[3]); lsp[4] = fmaf(s_a[4][iy], dyq, lsp[4]);
      lsp[5] = fmaf(s_a[5][iy], dyq, lsp[5]);
      lsp[6] = fmaf(s_a[6][iz], dzq, lsp[6]); lsp[7] = fmaf(s_a[7][iz], dzq, lsp[7]);
      lsp[8] = fmaf(s_a[8][iz], dzq, lsp[8]);
    }
    const float wx = tab.w[in] * st, wy = tab.w[jn], wz = tab.w[kn] * r * r;
    // lambda of the marched PML stresses s' (before the taper): divergence + stored (tapered) state.
    // State order: sxx syy szz sxy sxz syz syx szx szy; divergence order: xx xy xz | yx yy yz | zx zy zz.
    const float lxx = wx * lsp[0] + taper * as_s[F_SXX];
    const float lxy = wx * lsp[1] + taper * as_s[F_SXY];
    const float lxz = wx * lsp[2] + taper * as_s[F_SXZ];
    const float lyx = wy * lsp[3] + taper * as_s[F_SYX];
    const float lyy = wy * lsp[4] + taper * as_s[F_SYY];
    const float lyz = wy * lsp[5] + taper * as_s[F_SYZ];
    const float lzx = wz * lsp[6] + taper * as_s[F_SZX];
    const float lzy = wz * lsp[7] + taper * as_s[F_SZY];
    const float lzz = wz * lsp[8] + taper * as_s[F_SZZ];
    // PML stress march s' = s + dt (sigma - p s)
    if (act) {
      AS[F_SXX * 125] = lxx * (1.f - dt * px);
      AS[F_SYY * 125] = lyy * (1.f - dt * py);
      AS[F_SZZ * 125] = lzz * (1.f - dt * pz);
      AS[F_SXY * 125] = lxy * (1.f - dt * px);
      AS[F_SYX * 125] = lyx * (1.f - dt * py);
      AS[F_SXZ * 125] = lxz * (1.f - dt * px);
      AS[F_SZX * 125] = lzx * (1.f - dt * pz);
      AS[F_SYZ * 125] = lyz * (1.f - dt * py);
      AS[F_SZY * 125] = lzy * (1.f - dt * pz);
    }
    const float ls_xx = dt * lxx, ls_yy = dt * lyy, ls_zz = dt * lzz;
    const float ls_xy = dt * (lxy + lyx), ls_xz = dt * (lxz + lzx), ls_yz = dt * (lyz + lzy);

    // ---- stress rates and memory variables, in reverse (ses3d_evolution.f90:146-202,334-360)
    const float sd = ls_xx + ls_yy + ls_zz;
    float les[6];
    les[0] = clam * sd + c2mut * ls_xx + cA * (ls_xx + ls_yy) + cC * ls_zz;
    les[1] = clam * sd + c2mut * ls_yy + cA * (ls_xx + ls_yy) + cC * ls_zz;
    les[2] = clam * sd + c2mut * ls_zz + cC * (ls_xx + ls_yy);
    les[3] = c2mut * ls_xy;
    les[4] = (c2mut + cB2) * ls_xz;
    les[5] = (c2mut + cB2) * ls_yz;
    const float tr = es[0] + es[1] + es[2];
    double gsum[6];
    gsum[M_CLAM] = (double)(tr * sd);
    gsum[M_C2MUT] = (double)(es[0] * ls_xx + es[1] * ls_yy + es[2] * ls_zz + es[3] * ls_xy + es[4] * ls_xz +
                             es[5] * ls_yz);
    gsum[M_A] = (double)((es[1] + es[0]) * (ls_xx + ls_yy));
    gsum[M_B2] = (double)(es[4] * ls_xz + es[5] * ls_yz);
    gsum[M_C] = (double)(es[2] * (ls_xx + ls_yy) + (es[1] + es[0]) * ls_zz);
    gsum[M_C2MT] = 0.0;
    if (DISS) {
      const float third = sd * (1.f / 3.f);
      const float lMd[6] = {c2mt * (ls_xx - third), c2mt * (ls_yy - third), c2mt * (ls_zz - third),
                            c2mt * ls_xy, c2mt * ls_xz, c2mt * ls_yz};
      const float msum3 = (Md[0] + Md[1] + Md[2]) * (1.f / 3.f);
      gsum[M_C2MT] = (double)((Md[0] - msum3) * ls_xx + (Md[1] - msum3) * ls_yy + (Md[2] - msum3) * ls_zz +
                              Md[3] * ls_xy + Md[4] * ls_xz + Md[5] * ls_yz);
      // M' = M - (dt / tau_k) M - (dt D_k / tau_k) e
#pragma unroll
      for (int cc = 0; cc < 6; ++cc)
#pragma unroll
        for (int m = 0; m < 3; ++m) {
          const float lM = as_m[3 * cc + m];
          les[cc] -= c.L_k[m] * lM;
          if (act) AS[(F_M + 3 * cc + m) * 125] = (1.f - c.a_k[m]) * lM + lMd[cc];
        }
    }
    if (act) {
      double *GR = a.gmat + ((size_t)ev * c.E + e) * (NMAT * 125) + nn;
#pragma unroll
      for (int q = 0; q < NMAT; ++q) GR[q * 125] = gm0[q] + gsum[q];
    }

    // ---- symmetrisation, PML strain and displacement gradients, in reverse
    float lE[9];  // order of the state's displacement gradients: xx yy zz xy yx xz zx yz zy
    {
      const float l2[9] = {les[0], les[1], les[2], 0.5f * les[3], 0.5f * les[3], 0.5f * les[4], 0.5f * les[4],
                           0.5f * les[5], 0.5f * les[5]};
      const float P[9] = {Pxx, Pyy, Pzz, Pxy, Pyx, Pxz, Pzx, Pyz, Pzy};
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        const float lD = skip_ad ? 0.f : as_d[q] + P[q] * l2[q];  // d' = d + dt e;  e2 = e + P d'
        if (act && !skip_ad) AS[(F_DXUX + q) * 125] = lD;
        lE[q] = l2[q] + dt * lD;
      }
    }
    // spherical terms, in reverse (ses3d_evolution.f90:93-103): lambda of the raw contractions
    // and the velocity's own terms
    float lvx = 0.f, lvy = 0.f, lvz = 0.f;
    const float l_exx = ir * lE[0];                 lvz += ir * lE[0];
    const float l_eyy = irs * lE[1];                lvz += ir * lE[1]; lvx += ct * ir * lE[1];
    const float l_ezz = -lE[2];
    const float l_exy = ir * lE[3];
    const float l_eyx = irs * lE[4];                lvy -= ct * ir * lE[4];
    const float l_exz = ir * lE[5];                 lvx -= ir * lE[5];
    const float l_ezx = -lE[6];
    const float l_eyz = irs * lE[7];                lvy -= ir * lE[7];
    const float l_ezy = -lE[8];
    __syncthreads();  // s_a (divergence terms) fully read
    s_a[0][n] = on ? l_exx : 0.f; s_a[1][n] = on ? l_exy : 0.f; s_a[2][n] = on ? l_exz : 0.f;
    s_a[3][n] = on ? l_eyx : 0.f; s_a[4][n] = on ? l_eyy : 0.f; s_a[5][n] = on ? l_eyz : 0.f;
    s_a[6][n] = on ? l_ezx : 0.f; s_a[7][n] = on ? l_ezy : 0.f; s_a[8][n] = on ? l_ezz : 0.f;
    __syncthreads();
    // strain contraction, in reverse: e_x?(in) = sum_q v?(q) Dx[in][q]
#pragma unroll
    for (int q = 0; q < 5; ++q) {
      const int ix = q + 5 * jn + 25 * kn, iy = in + 5 * q + 25 * kn, iz = in + 5 * jn + 25 * q;
      const float dxq = tab.Dx[q][in], dyq = tab.Dy[q][jn], dzq = tab.Dz[q][kn];
      lvx = fmaf(s_a[0][ix], dxq, lvx); lvy = fmaf(s_a[1][ix], dxq, lvy); lvz = fmaf(s_a[2][ix], dxq, lvz);
      lvx = fmaf(s_a[3][iy], dyq, lvx); lvy = fmaf(s_a[4][iy], dyq, lvy); lvz = fmaf(s_a[5][iy], dyq, lvz);
      lvx = fmaf(s_a[6][iz], dzq, lvx); lvy = fmaf(s_a[7][iz], dzq, lvy); lvz = fmaf(s_a[8][iz], dzq, lvz);
    }
    if (act) {
      float *AF = a.af + (size_t)ev * 3 * c.N + (size_t)e * 375 + nn;
      AF[0] = lvx; AF[125] = lvy; AF[250] = lvz;
    }
    __syncthreads();  // s_a read by every thread before the next item writes it
  }
}

cudaError_t launch_adjoint_node1(const Consts &c, const Ptrs &p, const AdjPtrs &a, cudaStream_t st) {
  dim3 grid((unsigned)(((long long)c.GX * c.GY + 255) / 256), (unsigned)c.GZ, (unsigned)c.nev);
  k_adj_node1<<<grid, 256, 0, st>>>(c, p, a);
  return cudaGetLastError();
}

cudaError_t launch_adjoint_node2(const Consts &c, const AdjPtrs &a, cudaStream_t st) {
  dim3 grid((unsigned)(((long long)c.GX * c.GY + 255) / 256), (unsigned)c.GZ, (unsigned)c.nev);
  k_adj_node2<<<grid, 256, 0, st>>>(c, a);
  return cudaGetLastError();
}

// Resident CTAs of k_adj_element<DISS> on the current device (set by prepare_adjoint_kernels).
static int g_adj_cap[2] = {0, 0};

template <bool DISS>
static cudaError_t prepare_adj() {
  auto kern = k_adj_element<DISS>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ADJ_SMEM);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0, per_sm = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TPE, ADJ_SMEM)) != cudaSuccess) return e;
  g_adj_cap[DISS ? 1 : 0] = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
  return cudaSuccess;
}

// Sets the shared-memory limit and grid size of the persistent adjoint element kernel;
// called when a handle is created, before any stream capture.
cudaError_t prepare_adjoint_kernels() {
  cudaError_t e = prepare_adj<false>();
  return e == cudaSuccess ? prepare_adj<true>() : e;
}

cudaError_t launch_adjoint_element(int diss, const Consts &c, const Ptrs &p, const AdjPtrs &a, cudaStream_t st) {
  const int cap = g_adj_cap[diss ? 1 : 0];
  if (cap <= 0) return cudaErrorInitializationError;
  const long long total = c.E * (long long)c.nev;
  const unsigned blocks = (unsigned)(total < cap ? total : cap);
  if (diss) k_adj_element<true><<<blocks, TPE, ADJ_SMEM, st>>>(c, p, a);
  else k_adj_element<false><<<blocks, TPE, ADJ_SMEM, st>>>(c, p, a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
// Gradient with respect to the model records (rhoinv, mu, lambda, A, B, C, Q) from the
// coefficient and 1/MM gradients, summed over events, in the reference layout (FP64).
// The coefficients follow SOURCE/ses3d_init.f90:47-61 (k_derive_blocked): with tau = 1/Q and
// sD = sum D_p, kappa - 2 mu_tau / 3 = lambda - (2/3) sD tau mu, 2 mu_tau = 2 (1 + sD tau) mu,
// 2 mu tau; elastic runs: lambda, 2 mu, 0. The mass matrix MM = -sum_q W_q / rhoinv_q
// (SOURCE/ses3d_init.f90:254-279, W_q = w w w Jac r^2 sin(theta)) gives
// d/d rhoinv_q = -(g_1/MM / MM^2) W_q / rhoinv_q^2 at q's global node.
// ---------------------------------------------------------------------------------------
__global__ void k_adj_model_gradient(const Consts c, const Ptrs p, const double *__restrict__ gmat,
                                     const double *__restrict__ gimm, int which, int is_diss, double sD,
                                     const float *__restrict__ z, const float *__restrict__ sinx,
                                     const float *__restrict__ w, double *__restrict__ out) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;  // reference layout: e + E n
  if (q >= c.N) return;
  const long long e = q % c.E;
  const int n = (int)(q / c.E);
  const size_t EN = (size_t)c.E * NMAT * 125;
  double gc[NMAT] = {0, 0, 0, 0, 0, 0};
  for (int ev = 0; ev < c.nev; ++ev)
#pragma unroll
    for (int f = 0; f < NMAT; ++f) gc[f] += gmat[ev * EN + ((size_t)e * NMAT + f) * 125 + n];
  const size_t m = (size_t)e * 125 + n;  // element-major index of the field-major adjoint material
  const double mu = p.gmat[G_MU * c.N + m], QQ = p.gmat[G_QQ * c.N + m];
  double v = 0.0;
  if (which == 1 || which == 2 || which == 6) {
    if (is_diss) {
      const double tau = 1.0 / QQ;
      if (which == 2) v = gc[M_CLAM];
      if (which == 1)
        v = gc[M_CLAM] * (-(2.0 / 3.0) * sD * tau) + gc[M_C2MUT] * 2.0 * (1.0 + sD * tau) + gc[M_C2MT] * 2.0 * tau;
      if (which == 6) {
        const double dtau = gc[M_CLAM] * (-(2.0 / 3.0) * sD * mu) + gc[M_C2MUT] * 2.0 * sD * mu + gc[M_C2MT] * 2.0 * mu;
        v = -dtau / (QQ * QQ);
      }
    } else {
      if (which == 2) v = gc[M_CLAM];
      if (which == 1) v = 2.0 * gc[M_C2MUT];
    }
  } else if (which == 3) {
    v = gc[M_A];
  } else if (which == 4) {
    v = 2.0 * gc[M_B2];
  } else if (which == 5) {
    v = gc[M_C];
  } else if (which == 0) {
    const int i = (int)(e % c.ex), j = (int)((e / c.ex) % c.ey), k = (int)(e / ((long long)c.ex * c.ey));
    const int in = n % 5, jn = (n / 5) % 5, kn = n / 25;
    const size_t g = (size_t)(i * 4 + in) + (size_t)c.GX * ((size_t)(j * 4 + jn) + (size_t)c.GY * (size_t)(k * 4 + kn));
    double gi = 0.0;
    for (int ev = 0; ev < c.nev; ++ev) gi += gimm[(size_t)ev * c.G + g];
    const double MM = p.MM[g];
    const double zz = z[k * 5 + kn];
    const double W = (double)w[in] * (double)w[jn] * (double)w[kn] * (double)c.Jac * zz * zz * (double)sinx[i * 5 + in];
    const double rhoinv = 1.0 / (double)p.gmat[G_RHO * c.N + m];
    v = -(gi / (MM * MM)) * W / (rhoinv * rhoinv);
  }
  out[q] = v;
}

cudaError_t launch_adjoint_model_gradient(const Consts &c, const Ptrs &p, const double *gmat, const double *gimm,
                                          int which, int is_diss, double sD, const float *z, const float *sinx,
                                          const float *w, double *out, cudaStream_t st) {
  k_adj_model_gradient<<<(unsigned)((c.N + 255) / 256), 256, 0, st>>>(c, p, gmat, gimm, which, is_diss, sD, z, sinx,
                                                                      w, out);
  return cudaGetLastError();
}

}  // namespace ses3d

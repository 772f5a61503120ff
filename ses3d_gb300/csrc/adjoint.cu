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

// k_adj_element: one element per 128-thread CTA (thread = GLL node); grid (ex, ey, ez * nev).
// Every global load of the element is issued first, before the first barrier.
template <bool DISS>
__global__ void __launch_bounds__(TPE, 4) k_adj_element(const Consts c, const Ptrs p, const AdjPtrs a) {
  __shared__ KTab tab;
  __shared__ float s_a[9][TPE];
  for (int q = threadIdx.x; q < KTAB_FLOATS; q += TPE)
    reinterpret_cast<float *>(&tab)[q] = reinterpret_cast<const float *>(p.ktab)[q];
  const int n = threadIdx.x;
  const int i = blockIdx.x, j = blockIdx.y;
  const int k = (int)blockIdx.z / c.nev;
  const int ev = (int)blockIdx.z - k * c.nev;
  const bool act = n < 125;
  const int nn = act ? n : 0;
  const int in = nn % 5, jn = (nn / 5) % 5, kn = nn / 25;
  const unsigned e = (unsigned)i + (unsigned)c.ex * ((unsigned)j + (unsigned)c.ey * (unsigned)k);
  const size_t g = (size_t)(i * 4 + in) + (size_t)c.GX * ((size_t)(j * 4 + jn) + (size_t)c.GY * (size_t)(k * 4 + kn));
  const size_t ov = (size_t)ev * 3 * c.G + g;
  const size_t os = ((size_t)ev * c.E + e) * ELEM_STATE + nn;
  constexpr int SF = slot_fields(DISS);
  const float *FS = a.fstate + ((size_t)ev * c.E + e) * (SF * 125) + nn;  // packed forward state before the iteration
  float *AS = a.astate + os;        // adjoint state: lambda_t in, lambda_{t-1} out
  const float dt = c.dt;

  // Outside the PML the profiles are zero: the forward displacement gradients enter nothing
  // there and are neither packed nor read, and adjoint ones that start at zero stay zero.
  const bool pml = in_pml_element(c, i, j, k);
  const bool skip_ad = !pml && a.zero_d;

  // ---- loads: forward velocity and the adjoint of the assembled forces at the element's
  // nodes, the adjoint state, the packed forward state, the material and the 1-D tables
  float vx = 0.f, vy = 0.f, vz = 0.f, lF0 = 0.f, lF1 = 0.f, lF2 = 0.f;
  if (act) {
    vx = a.fv[ov]; vy = a.fv[ov + c.G]; vz = a.fv[ov + 2 * c.G];
    lF0 = a.aF[ov]; lF1 = a.aF[ov + c.G]; lF2 = a.aF[ov + 2 * c.G];
  }
  float as_s[9], as_d[9], as_m[DISS ? 18 : 1];
#pragma unroll
  for (int f = 0; f < 9; ++f) as_s[f] = AS[f * 125];
#pragma unroll
  for (int q = 0; q < 9; ++q) as_d[q] = skip_ad ? 0.f : AS[(F_DXUX + q) * 125];
  if (DISS) {
#pragma unroll
    for (int q = 0; q < 18; ++q) as_m[q] = AS[(F_M + q) * 125];
  }
  float fd[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) fd[q] = pml ? FS[q * 125] : 0.f;
  float Md[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // forward memory-variable sums per component
  if (DISS) {
#pragma unroll
    for (int cc = 0; cc < 6; ++cc) Md[cc] = FS[(9 + cc) * 125];
  }
  const float *MT = p.mat + (size_t)e * ELEM_MAT + nn;
  const float clam = __ldg(MT + M_CLAM * MAT_ROW), c2mut = __ldg(MT + M_C2MUT * MAT_ROW);
  const float c2mt = DISS ? __ldg(MT + M_C2MT * MAT_ROW) : 0.f;
  const float cA = c.iso ? 0.f : __ldg(MT + M_A * MAT_ROW), cB2 = c.iso ? 0.f : __ldg(MT + M_B2 * MAT_ROW);
  const float cC = c.iso ? 0.f : __ldg(MT + M_C * MAT_ROW);
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
    for (int q = 0; q < NMAT; ++q) GR[q * 125] += gsum[q];
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

cudaError_t launch_adjoint_element(int diss, const Consts &c, const Ptrs &p, const AdjPtrs &a, cudaStream_t st) {
  dim3 grid((unsigned)c.ex, (unsigned)c.ey, (unsigned)(c.ez * c.nev));
  if (diss) k_adj_element<true><<<grid, TPE, 0, st>>>(c, p, a);
  else k_adj_element<false><<<grid, TPE, 0, st>>>(c, p, a);
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

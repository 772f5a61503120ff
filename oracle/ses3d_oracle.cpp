// ses3d_oracle.cpp -- CPU oracle: C++ restatement of the reference SES3D solver.
//
// TEST INFRASTRUCTURE ONLY (checker and timed CPU baseline); the product never
// links it. Each function cites the reference file:line it restates. Whole-array
// Fortran statements become flat loops in the same statement order and the same
// left-to-right expression order; build with -ffp-contract=off so that the FP32
// instantiation rounds like gfortran -O3 on x86-64 (no FMA contraction).
// Parity with the reference is unpinned by the reference's own tests (it has none).
#include "ses3d_oracle.h"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

template <class T> struct Lit;
template <> struct Lit<float>  { static float  v(double, float f) { return f; } };
template <> struct Lit<double> { static double v(double d, float) { return d; } };
// A real literal of default kind: parsed straight to float (REAL(4)) or double.
#define LIT(x) Lit<T>::v(x, x##f)

// GLL knots of degree n, as the literals in SOURCE/ses3d_miscellaneous.f90:396-456
// (identical tables in ses3d_init.f90:91-195 and ses3d_output.f90:42-103).
template <class T> void gll_knots(int n, T *k) {
  switch (n) {
    case 0: k[0] = LIT(0.0); break;
    case 1: k[0] = LIT(-1.0); k[1] = LIT(1.0); break;
    case 2: k[0] = LIT(-1.0); k[1] = LIT(0.0); k[2] = LIT(1.0); break;
    case 3: k[0] = LIT(-1.0); k[1] = LIT(-0.4472135954999579); k[2] = LIT(0.4472135954999579); k[3] = LIT(1.0); break;
    case 4: k[0] = LIT(-1.0); k[1] = LIT(-0.6546536707079772); k[2] = LIT(0.0); k[3] = LIT(0.6546536707079772); k[4] = LIT(1.0); break;
    case 5: k[0] = LIT(-1.0); k[1] = LIT(-0.7650553239294647); k[2] = LIT(-0.2852315164806451);
            k[3] = LIT(0.2852315164806451); k[4] = LIT(0.7650553239294647); k[5] = LIT(1.0); break;
    case 6: k[0] = LIT(-1.0); k[1] = LIT(-0.8302238962785670); k[2] = LIT(-0.4688487934707142); k[3] = LIT(0.0);
            k[4] = LIT(0.4688487934707142); k[5] = LIT(0.8302238962785670); k[6] = LIT(1.0); break;
    default: k[0] = LIT(-1.0); k[1] = LIT(-0.8717401485096066); k[2] = LIT(-0.5917001814331423);
            k[3] = LIT(-0.2092992179024789); k[4] = LIT(0.2092992179024789); k[5] = LIT(0.5917001814331423);
            k[6] = LIT(0.8717401485096066); k[7] = LIT(1.0); break;
  }
}

// Integration weights, SOURCE/ses3d_init.f90:91-195 (truncated decimal literals).
template <class T> void gll_weights(int n, T *w) {
  switch (n) {
    case 0: w[0] = LIT(2.0); break;
    case 1: w[0] = LIT(1.0); w[1] = LIT(1.0); break;
    case 2: w[0] = LIT(1.0) / LIT(3.0); w[1] = LIT(4.0) / LIT(3.0); w[2] = LIT(1.0) / LIT(3.0); break;
    case 3: w[0] = LIT(0.1666666666666); w[1] = LIT(0.8333333333333); w[2] = LIT(0.8333333333333); w[3] = LIT(0.1666666666666); break;
    case 4: w[0] = LIT(0.1000000000000); w[1] = LIT(0.5444444444444); w[2] = LIT(0.7111111111111);
            w[3] = LIT(0.5444444444444); w[4] = LIT(0.1000000000000); break;
    case 5: w[0] = LIT(0.0666666666666667); w[1] = LIT(0.3784749562978470); w[2] = LIT(0.5548583770354862);
            w[3] = LIT(0.5548583770354862); w[4] = LIT(0.3784749562978470); w[5] = LIT(0.0666666666666667); break;
    case 6: w[0] = LIT(0.0476190476190476); w[1] = LIT(0.2768260473615659); w[2] = LIT(0.4317453812098627);
            w[3] = LIT(0.4876190476190476); w[4] = LIT(0.4317453812098627); w[5] = LIT(0.2768260473615659);
            w[6] = LIT(0.0476190476190476); break;
    default: w[0] = LIT(0.0357142857142857); w[1] = LIT(0.2107042271435061); w[2] = LIT(0.3411226924835044);
            w[3] = LIT(0.4124587946587038); w[4] = LIT(0.4124587946587038); w[5] = LIT(0.3411226924835044);
            w[6] = LIT(0.2107042271435061); w[7] = LIT(0.0357142857142857); break;
  }
}

// lgll: SOURCE/ses3d_miscellaneous.f90:377-481.
template <class T> T lgll(int n, int i, T x) {
  T knots[8];
  gll_knots<T>(n, knots);
  T r = LIT(1.0);
  if (n > 0) {
    for (int k = 0; k <= n; ++k)
      if (k != i) r = r * (x - knots[k]) / (knots[i] - knots[k]);
  } else {
    r = LIT(1.0);
  }
  return r;
}

// dlgll: SOURCE/ses3d_miscellaneous.f90:492-613.
template <class T> T dlgll(int n, int i, int j) {
  T knots[8];
  gll_knots<T>(n, knots);
  T y;
  if (n == 0) return LIT(0.0);
  if (i == j) {
    y = LIT(0.0);
    for (int k = 0; k <= n; ++k)
      if (k != i) y = y + LIT(1.0) / (knots[i] - knots[k]);
  } else {
    y = LIT(1.0) / (knots[i] - knots[j]);
    for (int k = 0; k <= n; ++k)
      if (k != i && k != j) y = y * (knots[j] - knots[k]) / (knots[i] - knots[k]);
  }
  return y;
}

template <class T> T tsin(T x) { return std::sin(x); }
template <class T> T tcos(T x) { return std::cos(x); }
template <class T> T texp(T x) { return std::exp(x); }
template <class T> T tsqrt(T x) { return std::sqrt(x); }

struct Base {
  virtual ~Base() {}
  virtual int run(int n) = 0;
  virtual int it() const = 0;
  virtual long size(const std::string &name) = 0;
  virtual int get(const std::string &name, void *out) = 0;
  virtual long get_int(const std::string &name, int *out) = 0;
  virtual int nrecords() const = 0;
  virtual int get_record(int r, void *out) = 0;
  virtual int set_records(int nrec, const void *data) = 0;
  virtual int set(const std::string &name, const void *in) = 0;
};

template <class T> struct Sim : Base {
  typedef std::vector<T> V;
  // ---- sizes
  int nx, ny, nz, lpd, L, pml;
  long E, N, GX, GY, GZ, G;
  // ---- flags and scalars (module variables, SOURCE/ses3d_modules.f90:33-233)
  int is_diss, adjoint_flag, samp_ad, nt, source_type, grad_variant;
  int ix_multi = 1, iy_multi = 1, iz_multi = 1, px = 1, py = 1, pz = 1;
  T ispml, dt, xmin, xmax, ymin, ymax, zmin, zmax, zmax_global;
  T xxs, yys, zzs, xxs_loc, yys_loc, zzs_loc;
  T MOM_xx, MOM_yy, MOM_zz, MOM_xy, MOM_xz, MOM_yz;
  T tau_p[3], D_p[3], sum_D_p;
  T knots[8], w[8], dl[8][8];
  T dx, dy, dz, Jac;
  T is_source;
  int isx = 0, isy = 0, isz = 0, isx_n = 0, isy_n = 0, isz_n = 0;
  int it_ = 0;
  V so;
  V x, y, z;  // (0:nx,0:lpd) etc., first index fastest
  // ---- element-local arrays (N each)
  V rhoinv, mu, lambda, kappa, mu_tau, A, B, C, tau, QQ, cp, cs, rho;
  V sin_theta, r, cot_theta;
  V vx, vy, vz;
  V exx, eyy, ezz, exy, exz, eyz, eyx, ezx, ezy;
  V dxux, dyux, dzux, dxuy, dyuy, dzuy, dxuz, dyuz, dzuz;
  V Mxx, Myy, Mzz, Mxy, Mxz, Myz;  // (1:nrdiss, ...) mechanism fastest
  V src_xx, src_yy, src_zz, src_xy, src_yx, src_xz, src_zx, src_yz, src_zy;
  V sx, sy, sz;
  V sxx, syy, szz, sxy, sxz, syz;
  V sxx_pml, syy_pml, szz_pml, sxy_pml, syz_pml, sxz_pml, syx_pml, szy_pml, szx_pml;
  V prof_x, prof_y, prof_z, prof, taper;
  V Lw, M_dummy, Mdx, Mdy, Mdz, r_sin_theta;  // ses3d_evolution.f90:19-20 locals
  // ---- global arrays (G each)
  V MM_global, sx_global, sy_global, sz_global, vx_global, vy_global, vz_global, prof_global, taper_global;
  // ---- receivers
  int nr = 0;
  std::vector<int> rx, ry, rz;
  V recloc_std, recloc;  // (1:3, 1:maxnr)
  V seismogram_x, seismogram_y, seismogram_z;  // (1:nr, 1:nt), receiver fastest
  // ---- adjoint
  int nr_adsrc = 0;
  std::vector<int> saving_vector;
  std::vector<int> is_, isn_;  // (1:3, idx)
  V xxs_ad_loc, yys_ad_loc, zzs_ad_loc, ad_stf_x, ad_stf_y, ad_stf_z;  // stf: (idx, it) idx fastest
  V grad_rho, grad_cp, grad_csh, grad_csv, grad_Q_mu, grad_Q_kappa, grad_alpha_mu, grad_alpha_kappa;
  V vx_fw, vy_fw, vz_fw, exx_fw, eyy_fw, ezz_fw, exy_fw, exz_fw, eyz_fw;
  std::vector<V> records;  // forward-field records: 9 fields of N each
  int record_cursor = 0;

  long id(long e, int in, int jn, int kn) const { return e + E * (in + L * (jn + L * kn)); }
  long gid(long gx, long gy, long gz) const { return gx + GX * (gy + GY * gz); }

  explicit Sim(const oracle_input *in) {
    const bool dbl = sizeof(T) == 8;
    auto R = [&](int k) -> T { return dbl ? (T)in->rd[k] : (T)in->rf[k]; };
    nx = in->nx; ny = in->ny; nz = in->nz; lpd = in->lpd; L = lpd + 1; pml = in->pml;
    E = (long)(nx + 1) * (ny + 1) * (nz + 1);
    N = E * L * L * L;
    GX = (long)(nx + 1) * lpd + 1; GY = (long)(ny + 1) * lpd + 1; GZ = (long)(nz + 1) * lpd + 1;
    G = GX * GY * GZ;
    is_diss = in->is_diss; adjoint_flag = in->adjoint_flag; samp_ad = in->samp_ad; nt = in->nt;
    source_type = in->source_type; grad_variant = in->grad_variant;
    const T pi = LIT(3.1415926535898);  // SOURCE/ses3d_modules.f90:25
    dt = R(OR_DT);
    xmin = R(OR_XMIN); xmax = R(OR_XMAX); ymin = R(OR_YMIN); ymax = R(OR_YMAX);
    zmin = R(OR_ZMIN); zmax = R(OR_ZMAX); zmax_global = R(OR_ZMAX_GLOBAL);
    xxs = R(OR_XXS); yys = R(OR_YYS); zzs = R(OR_ZZS);
    MOM_xx = R(OR_MXX); MOM_yy = R(OR_MYY); MOM_zz = R(OR_MZZ);
    MOM_xy = R(OR_MXY); MOM_xz = R(OR_MXZ); MOM_yz = R(OR_MYZ);
    for (int k = 0; k < 3; ++k) { tau_p[k] = R(OR_TAU1 + k); D_p[k] = R(OR_D1 + k); }
    // ses3d_input.f90:319-320 (degrees -> radians); 353 sum_D_p
    xxs = xxs * pi / (T)180; yys = yys * pi / (T)180;
    sum_D_p = D_p[0]; sum_D_p = sum_D_p + D_p[1]; sum_D_p = sum_D_p + D_p[2];
    // ses3d_input.f90:405-437: is the source in this box? read stf.
    so.assign(nt + 1, (T)0);
    if (adjoint_flag == 0 || adjoint_flag == 1) {
      if (xmin <= xxs && xmax >= xxs && ymin <= yys && ymax >= yys &&
          zmin <= zmax_global - zzs && zmax >= zmax_global - zzs) {
        is_source = LIT(1.0);
        for (int i = 1; i <= nt; ++i) so[i] = dbl ? (T)in->so_d[i - 1] : (T)in->so_f[i - 1];
      } else {
        is_source = LIT(0.0);
      }
    } else {
      is_source = LIT(0.0);
    }
    // ses3d_input.f90:472-499 model records
    auto load = [&](V &a, const float *p) { a.resize(N); for (long q = 0; q < N; ++q) a[q] = (T)p[q]; };
    load(rhoinv, in->rhoinv); load(mu, in->mu); load(lambda, in->lambda);
    load(A, in->A); load(B, in->B); load(C, in->C);
    QQ.assign(N, (T)0); tau.assign(N, (T)0);
    if (is_diss == 1) {
      load(QQ, in->Q);
      for (long q = 0; q < N; ++q) tau[q] = LIT(1.0) / QQ[q];
    }
    // receivers (ses3d_input.f90:533-544)
    int nr_global = in->nr_global;
    V recloc_global(3 * (size_t)nr_global + 3);
    for (int i = 0; i < nr_global; ++i) {
      for (int c = 0; c < 3; ++c)
        recloc_global[3 * i + c] = dbl ? (T)in->rec_d[3 * i + c] : (T)in->rec_f[3 * i + c];
      recloc_global[3 * i + 0] = recloc_global[3 * i + 0] * pi / (T)180;
      recloc_global[3 * i + 1] = recloc_global[3 * i + 1] * pi / (T)180;
    }
    // saving vector (ses3d_input.f90:562-578)
    saving_vector.assign(nt + 2, 0);
    if (adjoint_flag == 2 && in->saving_vector)
      for (int k = 1; k <= nt; ++k) saving_vector[k] = in->saving_vector[k - 1];
    // adjoint source locations (ses3d_input.f90:584-618)
    int nr_adsrc_global = in->nr_adsrc_global;
    V ad_srcloc_global(3 * (size_t)nr_adsrc_global + 3);
    for (int k = 0; k < nr_adsrc_global; ++k) {
      for (int c = 0; c < 3; ++c)
        ad_srcloc_global[3 * k + c] = dbl ? (T)in->adloc_d[3 * k + c] : (T)in->adloc_f[3 * k + c];
      ad_srcloc_global[3 * k + 0] = ad_srcloc_global[3 * k + 0] * pi / (T)180;
      ad_srcloc_global[3 * k + 1] = ad_srcloc_global[3 * k + 1] * pi / (T)180;
    }
    init(pi, nr_global, recloc_global, nr_adsrc_global, ad_srcloc_global, in);
  }

  // ses3d_init: SOURCE/ses3d_init.f90:7-729
  void init(T pi, int nr_global, const V &recloc_global, int nr_adsrc_global, const V &ad_srcloc_global,
            const oracle_input *in) {
    const bool dbl = sizeof(T) == 8;
    ispml = LIT(1.0);                              // :27
    T tol = pi / (T)(180 * 100000);                // :28
    // :47-85
    kappa.resize(N); cs.resize(N); cp.resize(N); rho.assign(N, (T)0); mu_tau.assign(N, (T)0);
    for (long q = 0; q < N; ++q) {
      kappa[q] = lambda[q] + (T)2 * mu[q] / (T)3;
      cs[q] = tsqrt(mu[q] * rhoinv[q]);
      cp[q] = tsqrt((lambda[q] + (T)2 * mu[q]) * rhoinv[q]);
      if (rhoinv[q] > 0) rho[q] = (T)1 / rhoinv[q];
    }
    if (is_diss == 1)
      for (long q = 0; q < N; ++q) mu_tau[q] = ((T)1 + sum_D_p * tau[q]) * mu[q];
    auto zero = [&](V &a, long n) { a.assign(n, (T)0); };
    for (V *a : {&dxux, &dyux, &dzux, &dxuy, &dyuy, &dzuy, &dxuz, &dyuz, &dzuz, &sxx_pml, &syy_pml, &szz_pml,
                 &sxy_pml, &syx_pml, &sxz_pml, &szx_pml, &syz_pml, &szy_pml, &src_xx, &src_yy, &src_zz,
                 &src_xy, &src_yx, &src_xz, &src_zx, &src_yz, &src_zy, &vx, &vy, &vz, &exx, &eyy, &ezz,
                 &exy, &exz, &eyz, &eyx, &ezx, &ezy, &sx, &sy, &sz, &sxx, &syy, &szz, &sxy, &sxz, &syz,
                 &Lw, &M_dummy, &Mdx, &Mdy, &Mdz, &r_sin_theta})
      zero(*a, N);
    for (V *a : {&Mxx, &Myy, &Mzz, &Mxy, &Mxz, &Myz}) zero(*a, 3 * N);
    for (V *a : {&vx_global, &vy_global, &vz_global, &sx_global, &sy_global, &sz_global}) zero(*a, G);
    if (adjoint_flag == 2) {
      for (V *a : {&grad_rho, &grad_cp, &grad_csh, &grad_csv, &grad_Q_mu, &grad_Q_kappa, &grad_alpha_mu,
                   &grad_alpha_kappa, &vx_fw, &vy_fw, &vz_fw, &exx_fw, &eyy_fw, &ezz_fw, &exy_fw, &exz_fw,
                   &eyz_fw})
        zero(*a, N);
    }
    // :91-207 knots, weights, dl(i,j) = derivative of poly i at knot j
    gll_knots<T>(lpd, knots);
    gll_weights<T>(lpd, w);
    for (int i = 0; i <= lpd; ++i)
      for (int j = 0; j <= lpd; ++j) dl[i][j] = dlgll<T>(lpd, i, j);
    // :213-248 geometry
    dx = (xmax - xmin) / (T)(nx + 1);
    dy = (ymax - ymin) / (T)(ny + 1);
    dz = (zmax - zmin) / (T)(nz + 1);
    x.resize((nx + 1) * L); y.resize((ny + 1) * L); z.resize((nz + 1) * L);
    sin_theta.resize(N); cot_theta.resize(N); r.resize(N);
    for (int i = 0; i <= nx; ++i)
      for (int n = 0; n <= lpd; ++n)
        x[i + (nx + 1) * n] = xmin + (T)i * dx + LIT(0.5) * ((T)1 + knots[n]) * dx;
    for (int j = 0; j <= ny; ++j)
      for (int n = 0; n <= lpd; ++n)
        y[j + (ny + 1) * n] = ymin + (T)j * dy + LIT(0.5) * ((T)1 + knots[n]) * dy;
    for (int k = 0; k <= nz; ++k)
      for (int n = 0; n <= lpd; ++n)
        z[k + (nz + 1) * n] = zmax - (T)k * dz - LIT(0.5) * ((T)1 + knots[n]) * dz;
    for (int kn = 0; kn < L; ++kn)
      for (int jn = 0; jn < L; ++jn)
        for (int in_ = 0; in_ < L; ++in_)
          for (int k = 0; k <= nz; ++k)
            for (int j = 0; j <= ny; ++j)
              for (int i = 0; i <= nx; ++i) {
                long e = i + (nx + 1) * (j + (long)(ny + 1) * k);
                long q = id(e, in_, jn, kn);
                T xv = X(i, in_);
                sin_theta[q] = tsin(xv);
                cot_theta[q] = tcos(xv) / tsin(xv);
                r[q] = Z(k, kn);
              }
    Jac = dx * dy * dz / (T)8;
    // :254-279 mass matrix, assembled in loop order i,j,k,l,m,n
    MM_global.assign(G, (T)0);
    for (int i = 0; i <= nx; ++i)
      for (int j = 0; j <= ny; ++j)
        for (int k = 0; k <= nz; ++k)
          for (int l = 0; l <= lpd; ++l)
            for (int m = 0; m <= lpd; ++m)
              for (int n = 0; n <= lpd; ++n) {
                long e = i + (nx + 1) * (j + (long)(ny + 1) * k);
                long q = id(e, l, m, n);
                long g = gid((long)i * lpd + l, (long)j * lpd + m, (long)k * lpd + n);
                T zz = Z(k, n);
                MM_global[g] = MM_global[g] - w[l] * w[m] * w[n] * Jac * zz * zz * sin_theta[q] / rhoinv[q];
              }
    // :285-357 receivers
    rx.assign(nr_global + 1, 0); ry.assign(nr_global + 1, 0); rz.assign(nr_global + 1, 0);
    recloc_std.assign(3 * (nr_global + 1), (T)0); recloc.assign(3 * (nr_global + 1), (T)0);
    nr = 0;
    if (adjoint_flag == 0 || adjoint_flag == 1) {
      for (int n = 0; n < nr_global; ++n) {
        T rc1 = recloc_global[3 * n], rc2 = recloc_global[3 * n + 1], rc3 = recloc_global[3 * n + 2];
        if (rc1 <= xmax && rc1 > xmin && rc2 <= ymax && rc2 > ymin && zmax_global - rc3 <= zmax &&
            zmax_global - rc3 > zmin) {
          nr = nr + 1;
          for (int i = 0; i <= nx; ++i)
            for (int j = 0; j <= ny; ++j)
              for (int k = 0; k <= nz; ++k) {
                if (rc1 <= X(i, lpd) + tol && rc1 >= X(i, 0) - tol && rc2 <= Y(j, lpd) + tol &&
                    rc2 >= Y(j, 0) - tol && zmax_global - rc3 <= Z(k, 0) && zmax_global - rc3 >= Z(k, lpd)) {
                  recloc_std[3 * nr - 3] = (T)2 * ((rc1 - xmin) / dx - (T)i) - (T)1;
                  recloc_std[3 * nr - 2] = (T)2 * ((rc2 - ymin) / dy - (T)j) - (T)1;
                  recloc_std[3 * nr - 1] = -(T)2 * ((zmax_global - rc3 - zmax) / dz + (T)k) - (T)1;
                  recloc[3 * nr - 3] = rc1; recloc[3 * nr - 2] = rc2; recloc[3 * nr - 1] = rc3;
                  rx[nr] = i; ry[nr] = j; rz[nr] = k;
                }
              }
        }
      }
    }
    seismogram_x.assign((size_t)(nr + 1) * (nt + 1), (T)0);
    seismogram_y.assign((size_t)(nr + 1) * (nt + 1), (T)0);
    seismogram_z.assign((size_t)(nr + 1) * (nt + 1), (T)0);
    // :363-439 point source location (nearest knot per axis, strict <)
    if ((adjoint_flag == 0 || adjoint_flag == 1) && is_source == LIT(1.0)) {
      T delta_x = dx, delta_y = dy, delta_z = dz;
      for (int i = 0; i <= nx; ++i)
        for (int n = 0; n <= lpd; ++n)
          if (std::fabs(X(i, n) - xxs) < delta_x) { delta_x = std::fabs(X(i, n) - xxs); isx = i; isx_n = n; }
      for (int j = 0; j <= ny; ++j)
        for (int n = 0; n <= lpd; ++n)
          if (std::fabs(Y(j, n) - yys) < delta_y) { delta_y = std::fabs(Y(j, n) - yys); isy = j; isy_n = n; }
      for (int k = 0; k <= nz; ++k)
        for (int n = 0; n <= lpd; ++n)
          if (std::fabs(zmax_global - Z(k, n) - zzs) < delta_z) {
            delta_z = std::fabs(zmax_global - Z(k, n) - zzs); isz = k; isz_n = n;
          }
      zzs_loc = (Z(isz, lpd) + Z(isz, 0) - (T)2 * (zmax_global - zzs)) / (Z(isz, 0) - Z(isz, lpd));
      yys_loc = ((T)2 * yys - Y(isy, lpd) - Y(isy, 0)) / (Y(isy, lpd) - Y(isy, 0));
      xxs_loc = ((T)2 * xxs - X(isx, lpd) - X(isx, 0)) / (X(isx, lpd) - X(isx, 0));
    } else {
      xxs_loc = yys_loc = zzs_loc = (T)0;
    }
    // :445-572 adjoint sources: box test, stf, nearest knot
    nr_adsrc = 0;
    is_.assign(3 * (nr_adsrc_global + 1), 0); isn_.assign(3 * (nr_adsrc_global + 1), 0);
    xxs_ad_loc.assign(nr_adsrc_global + 1, (T)0); yys_ad_loc = xxs_ad_loc; zzs_ad_loc = xxs_ad_loc;
    std::vector<int> local_to_global;
    V ad_srcloc(3 * (nr_adsrc_global + 1));
    if (adjoint_flag == 2) {
      for (int k = 0; k < nr_adsrc_global; ++k) {
        T a1 = ad_srcloc_global[3 * k], a2 = ad_srcloc_global[3 * k + 1], a3 = ad_srcloc_global[3 * k + 2];
        if (a1 <= xmax && a1 > xmin && a2 <= ymax && a2 > ymin && zmax_global - a3 <= zmax &&
            zmax_global - a3 > zmin) {
          nr_adsrc = nr_adsrc + 1;
          ad_srcloc[3 * nr_adsrc - 3] = a1; ad_srcloc[3 * nr_adsrc - 2] = a2; ad_srcloc[3 * nr_adsrc - 1] = a3;
          local_to_global.push_back(k);
        }
      }
      ad_stf_x.assign((size_t)(nr_adsrc + 1) * (nt + 1), (T)0);
      ad_stf_y = ad_stf_x; ad_stf_z = ad_stf_x;
      for (int idx = 1; idx <= nr_adsrc; ++idx) {
        int kg = local_to_global[idx - 1];
        for (int i = 1; i <= nt; ++i) {
          size_t base = ((size_t)kg * 3) * nt + (i - 1);
          T vxv = dbl ? (T)in->adstf_d[base] : (T)in->adstf_f[base];
          T vyv = dbl ? (T)in->adstf_d[base + nt] : (T)in->adstf_f[base + nt];
          T vzv = dbl ? (T)in->adstf_d[base + 2 * nt] : (T)in->adstf_f[base + 2 * nt];
          ad_stf_x[idx + (size_t)(nr_adsrc + 1) * i] = vxv;
          ad_stf_y[idx + (size_t)(nr_adsrc + 1) * i] = vyv;
          ad_stf_z[idx + (size_t)(nr_adsrc + 1) * i] = vzv;
        }
      }
      for (int idx = 1; idx <= nr_adsrc; ++idx) {
        T p1 = ad_srcloc[3 * idx - 3], p2 = ad_srcloc[3 * idx - 2], p3 = ad_srcloc[3 * idx - 1];
        T delta_x = xmax - xmin;
        for (int i = 0; i <= nx; ++i)
          for (int k = 0; k <= lpd; ++k)
            if (std::fabs(p1 - X(i, k)) < delta_x) {
              is_[3 * idx - 3] = i; isn_[3 * idx - 3] = k; delta_x = std::fabs(p1 - X(i, k));
            }
        int a = is_[3 * idx - 3];
        xxs_ad_loc[idx] = ((T)2 * p1 - X(a, lpd) - X(a, 0)) / (X(a, lpd) - X(a, 0));
        T delta_y = ymax - ymin;
        for (int i = 0; i <= ny; ++i)
          for (int k = 0; k <= lpd; ++k)
            if (std::fabs(p2 - Y(i, k)) < delta_y) {
              is_[3 * idx - 2] = i; isn_[3 * idx - 2] = k; delta_y = std::fabs(p2 - Y(i, k));
            }
        a = is_[3 * idx - 2];
        yys_ad_loc[idx] = ((T)2 * p2 - Y(a, lpd) - Y(a, 0)) / (Y(a, lpd) - Y(a, 0));
        T delta_z = zmax - zmin;
        for (int i = 0; i <= nz; ++i)
          for (int k = 0; k <= lpd; ++k)
            if (std::fabs(zmax_global - p3 - Z(i, k)) < delta_z) {
              is_[3 * idx - 1] = i; isn_[3 * idx - 1] = k; delta_z = std::fabs(zmax_global - p3 - Z(i, k));
            }
        a = is_[3 * idx - 1];
        zzs_ad_loc[idx] = (Z(a, lpd) + Z(a, 0) - (T)2 * (zmax_global - p3)) / (Z(a, 0) - Z(a, lpd));
      }
    }
    // :574-709 PML profiles
    T alpha = LIT(1.2);
    prof_x.assign(N, (T)0); prof_y.assign(N, (T)0); prof_z.assign(N, (T)0);
    // upper z-boundary disabled by `if (1==0)` (:586)
    if (iz_multi == 1) {
      for (int k = nz - pml + 1; k <= nz; ++k)
        for (int n = 0; n <= lpd; ++n) {
          if (k < 0) continue;
          T d = (zmin + (T)pml * dz - Z(k, n)) / ((T)pml * dz);
          T val = alpha * d * d;
          for (int jn = 0; jn < L; ++jn) for (int in_ = 0; in_ < L; ++in_)
            for (int j = 0; j <= ny; ++j) for (int i = 0; i <= nx; ++i)
              prof_z[id(i + (nx + 1) * (j + (long)(ny + 1) * k), in_, jn, n)] = val;
        }
    }
    if (ix_multi == 1) {
      for (int i = 0; i <= pml - 1; ++i)
        for (int n = 0; n <= lpd; ++n) {
          if (i > nx) continue;
          T d = (xmin + (T)pml * dx - X(i, n)) / ((T)pml * dx);
          T val = alpha * d * d;
          for (int kn = 0; kn < L; ++kn) for (int jn = 0; jn < L; ++jn)
            for (int k = 0; k <= nz; ++k) for (int j = 0; j <= ny; ++j)
              prof_x[id(i + (nx + 1) * (j + (long)(ny + 1) * k), n, jn, kn)] = val;
        }
    }
    if (ix_multi == px) {
      for (int i = nx - pml + 1; i <= nx; ++i)
        for (int n = 0; n <= lpd; ++n) {
          if (i < 0) continue;
          T d = (xmax - dx * (T)pml - X(i, n)) / ((T)pml * dx);
          T val = alpha * d * d;
          for (int kn = 0; kn < L; ++kn) for (int jn = 0; jn < L; ++jn)
            for (int k = 0; k <= nz; ++k) for (int j = 0; j <= ny; ++j)
              prof_x[id(i + (nx + 1) * (j + (long)(ny + 1) * k), n, jn, kn)] = val;
        }
    }
    if (iy_multi == 1) {
      for (int i = 0; i <= pml - 1; ++i)
        for (int n = 0; n <= lpd; ++n) {
          if (i > ny) continue;
          T d = (ymin + (T)pml * dy - Y(i, n)) / ((T)pml * dy);
          T val = alpha * d * d;
          for (int kn = 0; kn < L; ++kn) for (int in_ = 0; in_ < L; ++in_)
            for (int k = 0; k <= nz; ++k) for (int ii = 0; ii <= nx; ++ii)
              prof_y[id(ii + (nx + 1) * (i + (long)(ny + 1) * k), in_, n, kn)] = val;
        }
    }
    if (iy_multi == py) {
      for (int i = ny - pml + 1; i <= ny; ++i)
        for (int n = 0; n <= lpd; ++n) {
          if (i < 0) continue;
          T d = (ymax - dy * (T)pml - Y(i, n)) / ((T)pml * dy);
          T val = alpha * d * d;
          for (int kn = 0; kn < L; ++kn) for (int in_ = 0; in_ < L; ++in_)
            for (int k = 0; k <= nz; ++k) for (int ii = 0; ii <= nx; ++ii)
              prof_y[id(ii + (nx + 1) * (i + (long)(ny + 1) * k), in_, n, kn)] = val;
        }
    }
    // :678-686 corner normalisation and taper
    prof.resize(N); taper.resize(N);
    for (long q = 0; q < N; ++q) prof[q] = prof_x[q] + prof_y[q] + prof_z[q];
    for (long q = 0; q < N; ++q) {
      prof_z[q] = (T)2 * prof_z[q] / ((T)1 + prof[q] / alpha);
      prof_y[q] = (T)2 * prof_y[q] / ((T)1 + prof[q] / alpha);
      prof_x[q] = (T)2 * prof_x[q] / ((T)1 + prof[q] / alpha);
    }
    for (long q = 0; q < N; ++q) prof[q] = prof_x[q] + prof_y[q] + prof_z[q];
    for (long q = 0; q < N; ++q) taper[q] = texp(-(LIT(0.1) * prof[q] * prof[q]));
    // :690-709 local -> global, last writer in loop order i,j,k,in,jn,kn wins
    prof_global.assign(G, (T)0); taper_global.assign(G, (T)0);
    for (int i = 0; i <= nx; ++i)
      for (int j = 0; j <= ny; ++j)
        for (int k = 0; k <= nz; ++k)
          for (int in_ = 0; in_ <= lpd; ++in_)
            for (int jn = 0; jn <= lpd; ++jn)
              for (int kn = 0; kn <= lpd; ++kn) {
                long e = i + (nx + 1) * (j + (long)(ny + 1) * k);
                long q = id(e, in_, jn, kn);
                long g = gid((long)i * lpd + in_, (long)j * lpd + jn, (long)k * lpd + kn);
                prof_global[g] = prof[q];
                taper_global[g] = taper[q];
              }
    (void)dbl;
  }

  T X(int i, int n) const { return x[i + (nx + 1) * n]; }
  T Y(int j, int n) const { return y[j + (ny + 1) * n]; }
  T Z(int k, int n) const { return z[k + (nz + 1) * n]; }

  // make_moment_source: SOURCE/ses3d_miscellaneous.f90:97-150
  void make_moment_source(int it) {
    for (V *a : {&src_xx, &src_yy, &src_zz, &src_xy, &src_yx, &src_xz, &src_zx, &src_yz, &src_zy})
      std::fill(a->begin(), a->end(), (T)0);
    if (is_source > 0 && source_type == 10) {
      long e = isx + (nx + 1) * (isy + (long)(ny + 1) * isz);
      for (int in_ = 0; in_ <= lpd; ++in_)
        for (int jn = 0; jn <= lpd; ++jn)
          for (int kn = 0; kn <= lpd; ++kn) {
            T delta = lgll<T>(lpd, in_, xxs_loc) * lgll<T>(lpd, jn, yys_loc) * lgll<T>(lpd, kn, zzs_loc) /
                      (w[in_] * w[jn] * w[kn]);
            delta = delta / (Z(isz, kn) * Z(isz, kn) * tsin(X(isx, in_)) * Jac);
            long q = id(e, in_, jn, kn);
            src_xx[q] = src_xx[q] - MOM_xx * delta * so[it];
            src_yy[q] = src_yy[q] - MOM_yy * delta * so[it];
            src_zz[q] = src_zz[q] - MOM_zz * delta * so[it];
            src_xy[q] = src_xy[q] - MOM_xy * delta * so[it];
            src_yx[q] = src_yx[q] - MOM_xy * delta * so[it];
            src_xz[q] = src_xz[q] - MOM_xz * delta * so[it];
            src_zx[q] = src_zx[q] - MOM_xz * delta * so[it];
            src_yz[q] = src_yz[q] - MOM_yz * delta * so[it];
            src_zy[q] = src_zy[q] - MOM_yz * delta * so[it];
          }
    }
  }

  // add_single_force: SOURCE/ses3d_miscellaneous.f90:11-94
  void add_single_force(int it) {
    if (adjoint_flag == 0 || adjoint_flag == 1) {
      if (is_source > 0 && source_type < 10) {
        long e = isx + (nx + 1) * (isy + (long)(ny + 1) * isz);
        for (int in_ = 0; in_ <= lpd; ++in_)
          for (int jn = 0; jn <= lpd; ++jn)
            for (int kn = 0; kn <= lpd; ++kn) {
              T delta = lgll<T>(lpd, in_, xxs_loc) * lgll<T>(lpd, jn, yys_loc) * lgll<T>(lpd, kn, zzs_loc);
              long q = id(e, in_, jn, kn);
              if (source_type == 1) sx[q] = sx[q] - delta * so[it];
              else if (source_type == 2) sy[q] = sy[q] - delta * so[it];
              else if (source_type == 3) sz[q] = sz[q] - delta * so[it];
            }
      }
    }
    if (adjoint_flag == 2) {
      for (int idx = 1; idx <= nr_adsrc; ++idx) {
        long e = is_[3 * idx - 3] + (nx + 1) * (is_[3 * idx - 2] + (long)(ny + 1) * is_[3 * idx - 1]);
        size_t sidx = idx + (size_t)(nr_adsrc + 1) * it;
        for (int in_ = 0; in_ <= lpd; ++in_)
          for (int jn = 0; jn <= lpd; ++jn)
            for (int kn = 0; kn <= lpd; ++kn) {
              T delta = lgll<T>(lpd, in_, xxs_ad_loc[idx]) * lgll<T>(lpd, jn, yys_ad_loc[idx]) *
                        lgll<T>(lpd, kn, zzs_ad_loc[idx]);
              long q = id(e, in_, jn, kn);
              sx[q] = sx[q] - delta * ad_stf_x[sidx];
              sy[q] = sy[q] - delta * ad_stf_y[sidx];
              sz[q] = sz[q] - delta * ad_stf_z[sidx];
            }
      }
    }
  }

  // ses3d_evolution: SOURCE/ses3d_evolution.f90:7-373
  void evolution(int it) {
    const long NN = N;
    // :27-51 gather global v
    #pragma omp parallel for schedule(static)
    for (long q = 0; q < NN; ++q) {
      long e = q % E, n = q / E;
      int in_ = n % L, jn = (n / L) % L, kn = n / (L * L);
      long i = e % (nx + 1), j = (e / (nx + 1)) % (ny + 1), k = e / ((long)(nx + 1) * (ny + 1));
      long g = gid(i * lpd + in_, j * lpd + jn, k * lpd + kn);
      vx[q] = vx_global[g]; vy[q] = vy_global[g]; vz[q] = vz_global[g];
    }
    // :57
    for (V *a : {&exx, &eyy, &ezz, &exy, &exz, &eyz, &eyx, &ezx, &ezy}) std::fill(a->begin(), a->end(), (T)0);
    // :63-87 derivative proxies
    const long S1 = E, S2 = E * L, S3 = E * L * L;
    for (int i = 0; i <= lpd; ++i)
      for (int q = 0; q <= lpd; ++q) {
        T d3 = (T)2 * dl[q][i] / dz;
        T d2 = (T)2 * dl[q][i] / dy;
        T d1 = (T)2 * dl[q][i] / dx;
        // last GLL index (kn) = i, from kn = q
        #pragma omp parallel for schedule(static)
        for (long t = 0; t < S3; ++t) {
          long o = t + S3 * i, s = t + S3 * q;
          ezz[o] = ezz[o] + vz[s] * d3;
          ezy[o] = ezy[o] + vy[s] * d3;
          ezx[o] = ezx[o] + vx[s] * d3;
        }
        // middle GLL index (jn)
        #pragma omp parallel for schedule(static)
        for (long t = 0; t < S2 * L; ++t) {
          long lo = t % S2, kn = t / S2;
          long o = lo + S2 * i + S3 * kn, s = lo + S2 * q + S3 * kn;
          eyy[o] = eyy[o] + vy[s] * d2;
          eyx[o] = eyx[o] + vx[s] * d2;
          eyz[o] = eyz[o] + vz[s] * d2;
        }
        // first GLL index (in)
        #pragma omp parallel for schedule(static)
        for (long t = 0; t < S1 * L * L; ++t) {
          long e = t % S1, rest = t / S1;  // rest = jn + L*kn
          long o = e + S1 * i + S2 * rest, s = e + S1 * q + S2 * rest;
          exx[o] = exx[o] + vx[s] * d1;
          exy[o] = exy[o] + vy[s] * d1;
          exz[o] = exz[o] + vz[s] * d1;
        }
      }
    // :93-103 complete velocity gradients in spherical coordinates
    #pragma omp parallel for schedule(static)
    for (long q = 0; q < NN; ++q) {
      r_sin_theta[q] = r[q] * sin_theta[q];
      ezz[q] = -ezz[q];
      eyy[q] = eyy[q] / (r_sin_theta[q]) + (vz[q] + vx[q] * cot_theta[q]) / r[q];
      exx[q] = (vz[q] + exx[q]) / r[q];
      ezx[q] = -ezx[q];
      exz[q] = (exz[q] - vx[q]) / r[q];
      ezy[q] = -ezy[q];
      eyz[q] = -vy[q] / r[q] + eyz[q] / (r_sin_theta[q]);
      exy[q] = exy[q] / r[q];
      eyx[q] = -vy[q] * cot_theta[q] / r[q] + eyx[q] / (r_sin_theta[q]);
    }
    // :109-117 integrate to displacement gradients
    #pragma omp parallel for schedule(static)
    for (long q = 0; q < NN; ++q) {
      dzuz[q] = dzuz[q] + dt * ezz[q];
      dyuy[q] = dyuy[q] + dt * eyy[q];
      dxux[q] = dxux[q] + dt * exx[q];
      dzux[q] = dzux[q] + dt * ezx[q];
      dxuz[q] = dxuz[q] + dt * exz[q];
      dzuy[q] = dzuy[q] + dt * ezy[q];
      dyuz[q] = dyuz[q] + dt * eyz[q];
      dxuy[q] = dxuy[q] + dt * exy[q];
      dyux[q] = dyux[q] + dt * eyx[q];
    }
    // :123-138 apml strain rates, symmetrise
    #pragma omp parallel for schedule(static)
    for (long q = 0; q < NN; ++q) {
      exx[q] = exx[q] + (prof_z[q] + prof_y[q]) * dxux[q] * ispml;
      eyy[q] = eyy[q] + (prof_x[q] + prof_z[q]) * dyuy[q] * ispml;
      ezz[q] = ezz[q] + (prof_x[q] + prof_y[q]) * dzuz[q] * ispml;
      exy[q] = exy[q] + (prof_y[q] + prof_z[q]) * dxuy[q] * ispml;
      eyx[q] = eyx[q] + (prof_x[q] + prof_z[q]) * dyux[q] * ispml;
      exz[q] = exz[q] + (prof_y[q] + prof_z[q]) * dxuz[q] * ispml;
      ezx[q] = ezx[q] + (prof_x[q] + prof_y[q]) * dzux[q] * ispml;
      eyz[q] = eyz[q] + (prof_x[q] + prof_z[q]) * dyuz[q] * ispml;
      ezy[q] = ezy[q] + (prof_x[q] + prof_y[q]) * dzuy[q] * ispml;
      exy[q] = (exy[q] + eyx[q]) / LIT(2.0);
      exz[q] = (exz[q] + ezx[q]) / LIT(2.0);
      eyz[q] = (eyz[q] + ezy[q]) / LIT(2.0);
    }
    // :146-202 strong-form stress rates
    if (is_diss == 1) {
      #pragma omp parallel for schedule(static)
      for (long q = 0; q < NN; ++q) {
        Mdx[q] = 0; Mdy[q] = 0; Mdz[q] = 0;
        for (int k = 0; k < 3; ++k) {
          Mdx[q] = Mdx[q] + Mxx[k + 3 * q]; Mdy[q] = Mdy[q] + Myy[k + 3 * q]; Mdz[q] = Mdz[q] + Mzz[k + 3 * q];
        }
        M_dummy[q] = Mdx[q] + Mdy[q] + Mdz[q];
        Lw[q] = (kappa[q] - LIT(2.0) * mu_tau[q] / LIT(3.0)) * (exx[q] + eyy[q] + ezz[q]) -
                LIT(2.0) * mu[q] * tau[q] * M_dummy[q] / LIT(3.0);
        sxx[q] = Lw[q] + LIT(2.0) * mu_tau[q] * exx[q] + LIT(2.0) * mu[q] * tau[q] * Mdx[q] + C[q] * ezz[q] +
                 A[q] * (eyy[q] + exx[q]);
        syy[q] = Lw[q] + LIT(2.0) * mu_tau[q] * eyy[q] + LIT(2.0) * mu[q] * tau[q] * Mdy[q] + C[q] * ezz[q] +
                 A[q] * (eyy[q] + exx[q]);
        szz[q] = Lw[q] + LIT(2.0) * mu_tau[q] * ezz[q] + LIT(2.0) * mu[q] * tau[q] * Mdz[q] + C[q] * (eyy[q] + exx[q]);
      }
    } else {
      #pragma omp parallel for schedule(static)
      for (long q = 0; q < NN; ++q) {
        Lw[q] = lambda[q] * (exx[q] + eyy[q] + ezz[q]);
        sxx[q] = Lw[q] + (T)2 * mu[q] * exx[q] + C[q] * ezz[q] + A[q] * (eyy[q] + exx[q]);
        syy[q] = Lw[q] + (T)2 * mu[q] * eyy[q] + C[q] * ezz[q] + A[q] * (eyy[q] + exx[q]);
        szz[q] = Lw[q] + (T)2 * mu[q] * ezz[q] + C[q] * (eyy[q] + exx[q]);
      }
    }
    if (is_diss == 1) {
      #pragma omp parallel for schedule(static)
      for (long q = 0; q < NN; ++q) {
        Mdx[q] = 0; Mdy[q] = 0; Mdz[q] = 0;
        for (int k = 0; k < 3; ++k) {
          Mdx[q] = Mdx[q] + Mxy[k + 3 * q]; Mdy[q] = Mdy[q] + Mxz[k + 3 * q]; Mdz[q] = Mdz[q] + Myz[k + 3 * q];
        }
        sxy[q] = LIT(2.0) * mu_tau[q] * exy[q] + LIT(2.0) * mu[q] * tau[q] * Mdx[q];
        sxz[q] = LIT(2.0) * mu_tau[q] * exz[q] + LIT(2.0) * mu[q] * tau[q] * Mdy[q] + LIT(2.0) * B[q] * exz[q];
        syz[q] = LIT(2.0) * mu_tau[q] * eyz[q] + LIT(2.0) * mu[q] * tau[q] * Mdz[q] + LIT(2.0) * B[q] * eyz[q];
      }
    } else {
      #pragma omp parallel for schedule(static)
      for (long q = 0; q < NN; ++q) {
        sxy[q] = LIT(2.0) * mu[q] * exy[q];
        sxz[q] = LIT(2.0) * mu[q] * exz[q] + LIT(2.0) * B[q] * exz[q];
        syz[q] = LIT(2.0) * mu[q] * eyz[q] + LIT(2.0) * B[q] * eyz[q];
      }
    }
    // :208-219 march pml stresses
    #pragma omp parallel for schedule(static)
    for (long q = 0; q < NN; ++q) {
      sxx_pml[q] = sxx_pml[q] + dt * (sxx[q] - ispml * prof_x[q] * sxx_pml[q]);
      syy_pml[q] = syy_pml[q] + dt * (syy[q] - ispml * prof_y[q] * syy_pml[q]);
      szz_pml[q] = szz_pml[q] + dt * (szz[q] - ispml * prof_z[q] * szz_pml[q]);
      sxy_pml[q] = sxy_pml[q] + dt * (sxy[q] - ispml * prof_x[q] * sxy_pml[q]);
      syx_pml[q] = syx_pml[q] + dt * (sxy[q] - ispml * prof_y[q] * syx_pml[q]);
      sxz_pml[q] = sxz_pml[q] + dt * (sxz[q] - ispml * prof_x[q] * sxz_pml[q]);
      szx_pml[q] = szx_pml[q] + dt * (sxz[q] - ispml * prof_z[q] * szx_pml[q]);
      syz_pml[q] = syz_pml[q] + dt * (syz[q] - ispml * prof_y[q] * syz_pml[q]);
      szy_pml[q] = szy_pml[q] + dt * (syz[q] - ispml * prof_z[q] * szy_pml[q]);
    }
    // :227-231
    if (adjoint_flag == 0 || adjoint_flag == 1) make_moment_source(it);
    // :235-270 weak-form stress divergence
    std::fill(sx.begin(), sx.end(), (T)0); std::fill(sy.begin(), sy.end(), (T)0); std::fill(sz.begin(), sz.end(), (T)0);
    for (int i = 0; i <= lpd; ++i)
      for (int j = 0; j <= lpd; ++j)
        for (int k = 0; k <= lpd; ++k) {
          T d1 = (LIT(2.0) / dx) * Jac * w[j] * w[k];
          T d2 = (LIT(2.0) / dy) * Jac * w[i] * w[k];
          T d3 = -((LIT(2.0) / dz) * Jac * w[i] * w[j]);
          for (int q = 0; q <= lpd; ++q) {
            long o = E * (i + L * (j + L * k));
            long ox = E * (q + L * (j + L * k)), oy = E * (i + L * (q + L * k)), oz = E * (i + L * (j + L * q));
            #pragma omp parallel for schedule(static)
            for (long e = 0; e < E; ++e) {
              T dmx = w[q] * dl[i][q] * r[ox + e] * sin_theta[ox + e] * d1;
              T dmy = w[q] * dl[j][q] * r[oy + e] * d2;
              T dmz = w[q] * dl[k][q] * r[oz + e] * r[oz + e] * sin_theta[oz + e] * d3;
              sx[o + e] = sx[o + e] + (szx_pml[oz + e] + src_zx[oz + e]) * dmz +
                          (syx_pml[oy + e] + src_yx[oy + e]) * dmy + (sxx_pml[ox + e] + src_xx[ox + e]) * dmx;
              sy[o + e] = sy[o + e] + (szy_pml[oz + e] + src_zy[oz + e]) * dmz +
                          (syy_pml[oy + e] + src_yy[oy + e]) * dmy + (sxy_pml[ox + e] + src_xy[ox + e]) * dmx;
              sz[o + e] = sz[o + e] + (szz_pml[oz + e] + src_zz[oz + e]) * dmz +
                          (syz_pml[oy + e] + src_yz[oy + e]) * dmy + (sxz_pml[ox + e] + src_xz[ox + e]) * dmx;
            }
          }
        }
    // :276
    add_single_force(it);
    // :282-310 assemble in loop order i,in,j,jn,k,kn; parallel over disjoint x-columns of the
    // global grid keeps each node's summation order.
    std::fill(sx_global.begin(), sx_global.end(), (T)0);
    std::fill(sy_global.begin(), sy_global.end(), (T)0);
    std::fill(sz_global.begin(), sz_global.end(), (T)0);
    #pragma omp parallel for schedule(static)
    for (long gyz = 0; gyz < GY * GZ; ++gyz) {
      long gy = gyz % GY, gz = gyz / GY;
      // elements touching this (gy,gz) column, ascending: at most two per axis
      int j0 = gy == 0 ? 0 : (int)((gy - 1) / lpd);
      int k0 = gz == 0 ? 0 : (int)((gz - 1) / lpd);
      for (int i = 0; i <= nx; ++i)
        for (int in_ = 0; in_ <= lpd; ++in_) {
          long gx = (long)i * lpd + in_;
          for (int j = j0; j <= ny && j <= j0 + 1; ++j) {
            long jn = gy - (long)j * lpd;
            if (jn < 0 || jn > lpd) continue;
            for (int k = k0; k <= nz && k <= k0 + 1; ++k) {
              long kn = gz - (long)k * lpd;
              if (kn < 0 || kn > lpd) continue;
              long e = i + (nx + 1) * (j + (long)(ny + 1) * k);
              long q = id(e, in_, (int)jn, (int)kn);
              long g = gid(gx, gy, gz);
              sx_global[g] = sx_global[g] + sx[q];
              sy_global[g] = sy_global[g] + sy[q];
              sz_global[g] = sz_global[g] + sz[q];
            }
          }
        }
    }
    // :312 communicate_global_acceleration: a single processor box exchanges nothing.
    // :318-328
    #pragma omp parallel for schedule(static)
    for (long g = 0; g < G; ++g) {
      sx_global[g] = sx_global[g] / MM_global[g];
      sy_global[g] = sy_global[g] / MM_global[g];
      sz_global[g] = sz_global[g] / MM_global[g];
      vx_global[g] = vx_global[g] + dt * (sx_global[g] - ispml * prof_global[g] * vx_global[g]);
      vy_global[g] = vy_global[g] + dt * (sy_global[g] - ispml * prof_global[g] * vy_global[g]);
      vz_global[g] = vz_global[g] + dt * (sz_global[g] - ispml * prof_global[g] * vz_global[g]);
    }
    // :334-360 memory variables
    if (is_diss == 1) {
      for (int k = 0; k < 3; ++k) {
        T Lk = dt * D_p[k] / tau_p[k];
        #pragma omp parallel for schedule(static)
        for (long q = 0; q < NN; ++q) {
          long m = k + 3 * q;
          Mxx[m] = Mxx[m] - dt * Mxx[m] / tau_p[k] - Lk * exx[q];
          Myy[m] = Myy[m] - dt * Myy[m] / tau_p[k] - Lk * eyy[q];
          Mzz[m] = Mzz[m] - dt * Mzz[m] / tau_p[k] - Lk * ezz[q];
          Mxy[m] = Mxy[m] - dt * Mxy[m] / tau_p[k] - Lk * exy[q];
          Mxz[m] = Mxz[m] - dt * Mxz[m] / tau_p[k] - Lk * exz[q];
          Myz[m] = Myz[m] - dt * Myz[m] / tau_p[k] - Lk * eyz[q];
        }
      }
    }
    // :366-371 taper
    #pragma omp parallel for schedule(static)
    for (long g = 0; g < G; ++g) {
      vx_global[g] = taper_global[g] * vx_global[g];
      vy_global[g] = taper_global[g] * vy_global[g];
      vz_global[g] = taper_global[g] * vz_global[g];
    }
    #pragma omp parallel for schedule(static)
    for (long q = 0; q < NN; ++q) {
      sxx_pml[q] = sxx_pml[q] * taper[q]; syy_pml[q] = syy_pml[q] * taper[q]; szz_pml[q] = szz_pml[q] * taper[q];
      sxy_pml[q] = sxy_pml[q] * taper[q]; syx_pml[q] = syx_pml[q] * taper[q];
      szx_pml[q] = szx_pml[q] * taper[q]; sxz_pml[q] = sxz_pml[q] * taper[q];
      syz_pml[q] = syz_pml[q] * taper[q]; szy_pml[q] = szy_pml[q] * taper[q];
    }
  }

  // record_seismograms: SOURCE/ses3d_output.f90:456-497
  void record_seismograms(int it) {
    for (int idx = 1; idx <= nr; ++idx) {
      long e = rx[idx] + (nx + 1) * (ry[idx] + (long)(ny + 1) * rz[idx]);
      size_t s = idx + (size_t)(nr + 1) * it;
      for (int i = 0; i <= lpd; ++i)
        for (int j = 0; j <= lpd; ++j)
          for (int k = 0; k <= lpd; ++k) {
            T dm = lgll<T>(lpd, i, recloc_std[3 * idx - 3]) * lgll<T>(lpd, j, recloc_std[3 * idx - 2]) *
                   lgll<T>(lpd, k, recloc_std[3 * idx - 1]);
            long q = id(e, i, j, k);
            seismogram_x[s] = seismogram_x[s] + vx[q] * dm;
            seismogram_y[s] = seismogram_y[s] + vy[q] * dm;
            seismogram_z[s] = seismogram_z[s] + vz[q] * dm;
          }
    }
  }

  // ses3d_store calls of SOURCE/ses3d_main.f90:148-158 (deg = lpd: no compression)
  void store() {
    V rec(9 * N);
    for (long q = 0; q < N; ++q) {
      rec[q] = vx[q]; rec[N + q] = vy[q]; rec[2 * N + q] = vz[q];
      rec[3 * N + q] = dxux[q]; rec[4 * N + q] = dyuy[q]; rec[5 * N + q] = dzuz[q];
      rec[6 * N + q] = (dxuy[q] + dyux[q]) / (T)2;
      rec[7 * N + q] = (dxuz[q] + dzux[q]) / (T)2;
      rec[8 * N + q] = (dyuz[q] + dzuy[q]) / (T)2;
    }
    records.push_back(std::move(rec));
  }

  // ses3d_restore, read backwards: SOURCE/ses3d_output.f90:172-267
  void restore() {
    if (record_cursor <= 0) return;
    const V &rec = records[--record_cursor];
    for (long q = 0; q < N; ++q) {
      vx_fw[q] = rec[q]; vy_fw[q] = rec[N + q]; vz_fw[q] = rec[2 * N + q];
      exx_fw[q] = rec[3 * N + q]; eyy_fw[q] = rec[4 * N + q]; ezz_fw[q] = rec[5 * N + q];
      exy_fw[q] = rec[6 * N + q]; exz_fw[q] = rec[7 * N + q]; eyz_fw[q] = rec[8 * N + q];
    }
  }

  // ses3d_grad: SOURCE/ses3d_grad.f90:25-85 and SOURCE/ses3d_grad_Q.f90:44-158
  void grad(int it) {
    if (saving_vector[nt + 1 - it] > 0) {
      restore();
      const T s = (T)samp_ad * dt;
      #pragma omp parallel for schedule(static)
      for (long q = 0; q < N; ++q) {
        T exx_ad = dxux[q], eyy_ad = dyuy[q], ezz_ad = dzuz[q];
        T exy_ad = LIT(0.5) * (dxuy[q] + dyux[q]);
        T exz_ad = LIT(0.5) * (dxuz[q] + dzux[q]);
        T eyz_ad = LIT(0.5) * (dyuz[q] + dzuy[q]);
        T tr_e_ad = exx_ad + eyy_ad + ezz_ad;
        T tr_e_fw = exx_fw[q] + eyy_fw[q] + ezz_fw[q];
        T e_ddot_e = exx_ad * exx_fw[q] + eyy_ad * eyy_fw[q] + ezz_ad * ezz_fw[q] + LIT(2.0) * exy_ad * exy_fw[q] +
                     LIT(2.0) * exz_ad * exz_fw[q] + LIT(2.0) * eyz_ad * eyz_fw[q];
        grad_cp[q] = grad_cp[q] + s * (LIT(2.0) * rho[q] * cp[q] * tr_e_fw * tr_e_ad) / Jac;
        grad_rho[q] = grad_rho[q] + s * (vx_fw[q] * vx[q] + vy_fw[q] * vy[q] + vz_fw[q] * vz[q]) / Jac;
        grad_rho[q] = grad_rho[q] + s * ((cp[q] * cp[q] - LIT(2.0) * cs[q] * cs[q]) * tr_e_fw * tr_e_ad +
                                         LIT(2.0) * cs[q] * cs[q] * e_ddot_e) / Jac;
        grad_csh[q] = grad_csh[q] + s * (LIT(4.0) * rho[q] * cs[q] *
                                         (e_ddot_e - tr_e_ad * tr_e_fw - LIT(2.0) * exz_fw[q] * exz_ad -
                                          LIT(2.0) * eyz_fw[q] * eyz_ad)) / Jac;
        grad_csv[q] = grad_csv[q] + s * (LIT(8.0) * rho[q] * cs[q] * (exz_fw[q] * exz_ad + eyz_fw[q] * eyz_ad)) / Jac;
        if (grad_variant == 1 && is_diss == 1) {
          const T dPdalpha[3] = {LIT(-3.06), LIT(-1.54), LIT(2.56)};
          T Md[3];
          for (int k = 0; k < 3; ++k) {
            long m = k + 3 * q;
            Md[k] = Mxx[m] * exx_fw[q] + Myy[m] * eyy_fw[q] + Mzz[m] * ezz_fw[q] + Mxy[m] * exy_fw[q] +
                    Mxz[m] * exz_fw[q] + Myz[m] * eyz_fw[q] - tr_e_fw * (Mxx[m] + Myy[m] + Mzz[m]) / LIT(3.0);
          }
          for (int k = 0; k < 3; ++k) {
            grad_Q_mu[q] = grad_Q_mu[q] + s * Md[k] * tau_p[k] / Jac;
            grad_alpha_mu[q] = grad_alpha_mu[q] + s * Md[k] * dPdalpha[k] * tau_p[k] / (D_p[k] * Jac);
          }
          for (int k = 0; k < 3; ++k) {
            long m = k + 3 * q;
            Md[k] = (Mxx[m] + Myy[m] + Mzz[m]) * tr_e_fw;
          }
          for (int k = 0; k < 3; ++k) {
            grad_Q_kappa[q] = grad_Q_kappa[q] + s * Md[k] * tau_p[k] / Jac;
            grad_alpha_kappa[q] = grad_alpha_kappa[q] + s * Md[k] * dPdalpha[k] * tau_p[k] / (D_p[k] * Jac);
          }
        }
      }
    }
    if (grad_variant == 1 && it == nt) {
      // ses3d_grad_Q.f90:151-158, including the overwrite of grad_alpha_mu at :156
      const T alpha = LIT(0.3), Q_kappa = LIT(57823.0);
      for (long q = 0; q < N; ++q) {
        grad_Q_mu[q] = LIT(2.0) * mu[q] * grad_Q_mu[q] / QQ[q];
        grad_alpha_mu[q] = -(LIT(2.0) * alpha * mu[q] * grad_alpha_mu[q] / QQ[q]);
        grad_Q_kappa[q] = kappa[q] * grad_Q_kappa[q] / Q_kappa;
        grad_alpha_mu[q] = -(alpha * kappa[q] * grad_alpha_kappa[q] / Q_kappa);
      }
    }
  }

  // body of the time loop, SOURCE/ses3d_main.f90:95-178
  int run(int n) override {
    for (int s = 0; s < n && it_ < nt; ++s) {
      int it = ++it_;
      evolution(it);
      if (adjoint_flag == 0 || adjoint_flag == 1) record_seismograms(it);
      if (adjoint_flag == 1 && (it % samp_ad == 0 || it == 1 || it == nt)) {
        store();
        saving_vector[it] = it;
      }
      if (adjoint_flag == 2) grad(it);
    }
    return 0;
  }
  int it() const override { return it_; }

  V *field(const std::string &nm) {
    static const char *names[] = {"rhoinv", "mu", "lambda", "kappa", "mu_tau", "A", "B", "C", "tau", "QQ", "cp",
                                  "cs", "rho", "sin_theta", "r", "cot_theta", "vx", "vy", "vz", "exx", "eyy",
                                  "ezz", "exy", "exz", "eyz", "dxux", "dyux", "dzux", "dxuy", "dyuy", "dzuy",
                                  "dxuz", "dyuz", "dzuz", "Mxx", "Myy", "Mzz", "Mxy", "Mxz", "Myz", "sxx_pml",
                                  "syy_pml", "szz_pml", "sxy_pml", "syz_pml", "sxz_pml", "syx_pml", "szy_pml",
                                  "szx_pml", "prof_x", "prof_y", "prof_z", "prof", "taper", "MM_global",
                                  "vx_global", "vy_global", "vz_global", "prof_global", "taper_global",
                                  "grad_rho", "grad_cp", "grad_csh", "grad_csv", "grad_Q_mu", "grad_Q_kappa",
                                  "grad_alpha_mu", "grad_alpha_kappa", "x", "y", "z", "recloc_std",
                                  "seismogram_x", "seismogram_y", "seismogram_z", "sx", "sy", "sz",
                                  "xxs_ad_loc", "yys_ad_loc", "zzs_ad_loc", nullptr};
    V *ptrs[] = {&rhoinv, &mu, &lambda, &kappa, &mu_tau, &A, &B, &C, &tau, &QQ, &cp, &cs, &rho, &sin_theta, &r,
                 &cot_theta, &vx, &vy, &vz, &exx, &eyy, &ezz, &exy, &exz, &eyz, &dxux, &dyux, &dzux, &dxuy,
                 &dyuy, &dzuy, &dxuz, &dyuz, &dzuz, &Mxx, &Myy, &Mzz, &Mxy, &Mxz, &Myz, &sxx_pml, &syy_pml,
                 &szz_pml, &sxy_pml, &syz_pml, &sxz_pml, &syx_pml, &szy_pml, &szx_pml, &prof_x, &prof_y,
                 &prof_z, &prof, &taper, &MM_global, &vx_global, &vy_global, &vz_global, &prof_global,
                 &taper_global, &grad_rho, &grad_cp, &grad_csh, &grad_csv, &grad_Q_mu, &grad_Q_kappa,
                 &grad_alpha_mu, &grad_alpha_kappa, &x, &y, &z, &recloc_std, &seismogram_x, &seismogram_y,
                 &seismogram_z, &sx, &sy, &sz, &xxs_ad_loc, &yys_ad_loc, &zzs_ad_loc};
    for (int k = 0; names[k]; ++k)
      if (nm == names[k]) return ptrs[k];
    return nullptr;
  }
  // scalar reals exported as 1-element arrays
  bool scalar(const std::string &nm, T &v) {
    if (nm == "dx") v = dx; else if (nm == "dy") v = dy; else if (nm == "dz") v = dz;
    else if (nm == "Jac") v = Jac; else if (nm == "xxs_loc") v = xxs_loc; else if (nm == "yys_loc") v = yys_loc;
    else if (nm == "zzs_loc") v = zzs_loc;
    else return false;
    return true;
  }
  long size(const std::string &nm) override {
    T v;
    if (scalar(nm, v)) return 1;
    if (nm == "dl") return (long)L * L;
    if (nm == "w" || nm == "knots") return L;
    V *f = field(nm);
    return f ? (long)f->size() : -1;
  }
  int get(const std::string &nm, void *out) override {
    T *o = (T *)out;
    T v;
    if (nm == "dl") { for (int i = 0; i < L; ++i) for (int j = 0; j < L; ++j) o[i + L * j] = dl[i][j]; return 0; }
    if (nm == "w") { for (int i = 0; i < L; ++i) o[i] = w[i]; return 0; }
    if (nm == "knots") { for (int i = 0; i < L; ++i) o[i] = knots[i]; return 0; }
    if (scalar(nm, v)) { o[0] = v; return 0; }
    V *f = field(nm);
    if (!f) return -1;
    std::memcpy(out, f->data(), f->size() * sizeof(T));
    return 0;
  }
  // Overwrites a named state array (initial conditions of parity runs that start from an
  // arbitrary state rather than at rest); values in the handle's precision.
  int set(const std::string &nm, const void *in) override {
    V *f = field(nm);
    if (!f) return -1;
    std::memcpy(f->data(), in, f->size() * sizeof(T));
    return 0;
  }
  long get_int(const std::string &nm, int *out) override {
    auto put = [&](const std::vector<int> &a) { if (out) std::memcpy(out, a.data(), a.size() * sizeof(int)); return (long)a.size(); };
    auto one = [&](int v) { if (out) out[0] = v; return 1L; };
    if (nm == "nr") return one(nr);
    if (nm == "rx") return put(rx);
    if (nm == "ry") return put(ry);
    if (nm == "rz") return put(rz);
    if (nm == "isx") return one(isx);
    if (nm == "isy") return one(isy);
    if (nm == "isz") return one(isz);
    if (nm == "isx_n") return one(isx_n);
    if (nm == "isy_n") return one(isy_n);
    if (nm == "isz_n") return one(isz_n);
    if (nm == "is_source") return one(is_source > 0 ? 1 : 0);
    if (nm == "nr_adsrc") return one(nr_adsrc);
    if (nm == "is") return put(is_);
    if (nm == "isn") return put(isn_);
    if (nm == "saving_vector") return put(saving_vector);
    return -1;
  }
  int nrecords() const override { return (int)records.size(); }
  int get_record(int r, void *out) override {
    if (r < 0 || r >= (int)records.size()) return -1;
    std::memcpy(out, records[r].data(), records[r].size() * sizeof(T));
    return 0;
  }
  int set_records(int nrec, const void *data) override {
    // records in the handle's precision (FP32 as on disk; FP64 for the -fdefault-real-8 stand-in)
    const T *p = (const T *)data;
    records.assign(nrec, V(9 * N));
    for (int r = 0; r < nrec; ++r)
      for (long q = 0; q < 9 * N; ++q) records[r][q] = (T)p[(size_t)r * 9 * N + q];
    record_cursor = nrec;
    return 0;
  }
};

}  // namespace

extern "C" {

void *oracle_create(const oracle_input *in, int fp64) {
  if (!in || in->lpd < 1 || in->lpd > 7) return nullptr;
  if (fp64) return static_cast<Base *>(new Sim<double>(in));
  return static_cast<Base *>(new Sim<float>(in));
}
void oracle_destroy(void *h) { delete static_cast<Base *>(h); }
int oracle_run(void *h, int n) { return static_cast<Base *>(h)->run(n); }
int oracle_it(void *h) { return static_cast<Base *>(h)->it(); }
long oracle_size(void *h, const char *name) { return static_cast<Base *>(h)->size(name); }
int oracle_get(void *h, const char *name, void *out) { return static_cast<Base *>(h)->get(name, out); }
int oracle_set(void *h, const char *name, const void *in) { return static_cast<Base *>(h)->set(name, in); }
long oracle_get_int(void *h, const char *name, int *out) { return static_cast<Base *>(h)->get_int(name, out); }
int oracle_nrecords(void *h) { return static_cast<Base *>(h)->nrecords(); }
int oracle_get_record(void *h, int r, void *out) { return static_cast<Base *>(h)->get_record(r, out); }
int oracle_set_records(void *h, int nrec, const void *data) { return static_cast<Base *>(h)->set_records(nrec, data); }
float oracle_strtof(const char *s) { return std::strtof(s, nullptr); }

}  // extern "C"

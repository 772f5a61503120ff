// setup.cpp -- FP32-exact mesh set-up (see setup.hpp). Compile with -ffp-contract=off.
#include "setup.hpp"

#include <algorithm>
#include <cmath>

namespace ses3d {

namespace {
// GLL knots for lpd = 4 (SOURCE/ses3d_init.f90:127-133; REAL(4) literals).
const float kKnots[NP] = {-1.0f, -0.6546536707079772f, 0.0f, 0.6546536707079772f, 1.0f};
// Integration weights, truncated decimals as in SOURCE/ses3d_init.f90:135-139.
const float kWeights[NP] = {0.1000000000000f, 0.5444444444444f, 0.7111111111111f, 0.5444444444444f,
                            0.1000000000000f};

// dlgll(lpd, i, j): derivative of Lagrange polynomial i at knot j
// (SOURCE/ses3d_miscellaneous.f90:575-605).
float dlgll(int i, int j) {
  const float *k = kKnots;
  float y;
  if (i == j) {
    y = 0.0f;
    for (int m = 0; m <= LPD; ++m)
      if (m != i) y = y + 1.0f / (k[i] - k[m]);
  } else {
    y = 1.0f / (k[i] - k[j]);
    for (int m = 0; m <= LPD; ++m)
      if (m != i && m != j) y = y * (k[j] - k[m]) / (k[i] - k[m]);
  }
  return y;
}
}  // namespace

float lgll(int i, float x) {
  float r = 1.0f;
  for (int m = 0; m <= LPD; ++m)
    if (m != i) r = r * (x - kKnots[m]) / (kKnots[i] - kKnots[m]);
  return r;
}

void pml_normalise(float pxr, float pyr, float pzr, float &px, float &py, float &pz, float &prof, float &taper) {
  const float alpha = 1.2f;
  float p = pxr + pyr + pzr;
  pz = 2.0f * pzr / (1.0f + p / alpha);
  py = 2.0f * pyr / (1.0f + p / alpha);
  px = 2.0f * pxr / (1.0f + p / alpha);
  prof = px + py + pz;
  taper = std::exp(-(0.1f * prof * prof));
}

std::string build_geometry(Geometry &g, int nx, int ny, int nz, int pml, float xmin, float xmax, float ymin,
                           float ymax, float zmin, float zmax, float zmax_global) {
  if (nx < 0 || ny < 0 || nz < 0) return "nx, ny, nz must be >= 0";
  if (pml < 0) return "pml must be >= 0";
  g.nx = nx; g.ny = ny; g.nz = nz;
  g.ex = nx + 1; g.ey = ny + 1; g.ez = nz + 1;
  g.E = (long long)g.ex * g.ey * g.ez;
  g.N = g.E * NPE;
  g.GX = g.ex * LPD + 1; g.GY = g.ey * LPD + 1; g.GZ = g.ez * LPD + 1;
  g.G = (long long)g.GX * g.GY * g.GZ;
  g.pml = pml;
  g.xmin = xmin; g.xmax = xmax; g.ymin = ymin; g.ymax = ymax; g.zmin = zmin; g.zmax = zmax;
  g.zmax_global = zmax_global;
  g.pi = 3.1415926535898f;  // SOURCE/ses3d_modules.f90:25
  for (int n = 0; n < NP; ++n) { g.knots[n] = kKnots[n]; g.w[n] = kWeights[n]; }
  for (int i = 0; i < NP; ++i)
    for (int j = 0; j < NP; ++j) g.dl[i][j] = dlgll(i, j);   // ses3d_init.f90:201-207
  // ses3d_init.f90:213-248
  g.dx = (xmax - xmin) / (float)(nx + 1);
  g.dy = (ymax - ymin) / (float)(ny + 1);
  g.dz = (zmax - zmin) / (float)(nz + 1);
  g.x.resize((size_t)g.ex * NP); g.y.resize((size_t)g.ey * NP); g.z.resize((size_t)g.ez * NP);
  g.sin_x.resize(g.x.size()); g.cot_x.resize(g.x.size());
  for (int i = 0; i <= nx; ++i)
    for (int n = 0; n < NP; ++n) {
      float xv = xmin + (float)i * g.dx + 0.5f * (1.0f + kKnots[n]) * g.dx;
      g.x[(size_t)i * NP + n] = xv;
      g.sin_x[(size_t)i * NP + n] = std::sin(xv);
      g.cot_x[(size_t)i * NP + n] = std::cos(xv) / std::sin(xv);
    }
  for (int j = 0; j <= ny; ++j)
    for (int n = 0; n < NP; ++n) g.y[(size_t)j * NP + n] = ymin + (float)j * g.dy + 0.5f * (1.0f + kKnots[n]) * g.dy;
  for (int k = 0; k <= nz; ++k)
    for (int n = 0; n < NP; ++n) g.z[(size_t)k * NP + n] = zmax - (float)k * g.dz - 0.5f * (1.0f + kKnots[n]) * g.dz;
  g.Jac = g.dx * g.dy * g.dz / 8.0f;

  // PML raw profiles (ses3d_init.f90:578-674). prof_x depends on (i,in) only,
  // prof_y on (j,jn), prof_z on (k,kn). The upper z boundary is disabled in the
  // reference (`if (1==0)`, :586): free surface at the top.
  const float alpha = 1.2f;
  g.pxr.assign(g.x.size(), 0.0f); g.pyr.assign(g.y.size(), 0.0f); g.pzr.assign(g.z.size(), 0.0f);
  for (int k = nz - pml + 1; k <= nz; ++k) {  // lower z-boundary (iz_multi == 1)
    if (k < 0) continue;
    for (int n = 0; n < NP; ++n) {
      float d = (zmin + (float)pml * g.dz - g.Z(k, n)) / ((float)pml * g.dz);
      g.pzr[(size_t)k * NP + n] = alpha * d * d;
    }
  }
  for (int i = 0; i <= pml - 1; ++i) {  // left x-boundary
    if (i > nx) continue;
    for (int n = 0; n < NP; ++n) {
      float d = (xmin + (float)pml * g.dx - g.X(i, n)) / ((float)pml * g.dx);
      g.pxr[(size_t)i * NP + n] = alpha * d * d;
    }
  }
  for (int i = nx - pml + 1; i <= nx; ++i) {  // right x-boundary
    if (i < 0) continue;
    for (int n = 0; n < NP; ++n) {
      float d = (xmax - g.dx * (float)pml - g.X(i, n)) / ((float)pml * g.dx);
      g.pxr[(size_t)i * NP + n] = alpha * d * d;
    }
  }
  for (int j = 0; j <= pml - 1; ++j) {  // left y-boundary
    if (j > ny) continue;
    for (int n = 0; n < NP; ++n) {
      float d = (ymin + (float)pml * g.dy - g.Y(j, n)) / ((float)pml * g.dy);
      g.pyr[(size_t)j * NP + n] = alpha * d * d;
    }
  }
  for (int j = ny - pml + 1; j <= ny; ++j) {  // right y-boundary
    if (j < 0) continue;
    for (int n = 0; n < NP; ++n) {
      float d = (ymax - g.dy * (float)pml - g.Y(j, n)) / ((float)pml * g.dy);
      g.pyr[(size_t)j * NP + n] = alpha * d * d;
    }
  }
  // Local -> global map of prof/taper (ses3d_init.f90:690-709): the element with the
  // largest index along each axis writes last, so each global index takes the
  // profile of element min(g/LPD, n_axis) at local index g - LPD*element.
  auto last = [](std::vector<float> &out, const std::vector<float> &raw, int ne, int GN) {
    out.resize(GN);
    for (int gi = 0; gi < GN; ++gi) {
      int e = std::min(gi / LPD, ne - 1);
      out[gi] = raw[(size_t)e * NP + (gi - e * LPD)];
    }
  };
  last(g.pxg, g.pxr, g.ex, g.GX);
  last(g.pyg, g.pyr, g.ey, g.GY);
  last(g.pzg, g.pzr, g.ez, g.GZ);
  return "";
}

void locate_source(const Geometry &g, float xxs_deg, float yys_deg, float zzs, int source_type, PointSource &s) {
  const float pi = g.pi;
  s = PointSource();
  s.xxs = xxs_deg * pi / 180.0f;  // ses3d_input.f90:319-320
  s.yys = yys_deg * pi / 180.0f;
  s.zzs = zzs;
  // ses3d_input.f90:407-409
  if (g.xmin <= s.xxs && g.xmax >= s.xxs && g.ymin <= s.yys && g.ymax >= s.yys &&
      g.zmin <= g.zmax_global - zzs && g.zmax >= g.zmax_global - zzs)
    s.is_source = 1;
  for (int n = 0; n < NPE; ++n) s.delta[n] = 0.0f;
  if (!s.is_source) return;
  // nearest knot per axis, strict <, starting from one element width (ses3d_init.f90:367-417)
  float delta_x = g.dx, delta_y = g.dy, delta_z = g.dz;
  for (int i = 0; i <= g.nx; ++i)
    for (int n = 0; n < NP; ++n)
      if (std::fabs(g.X(i, n) - s.xxs) < delta_x) { delta_x = std::fabs(g.X(i, n) - s.xxs); s.isx = i; s.isx_n = n; }
  for (int j = 0; j <= g.ny; ++j)
    for (int n = 0; n < NP; ++n)
      if (std::fabs(g.Y(j, n) - s.yys) < delta_y) { delta_y = std::fabs(g.Y(j, n) - s.yys); s.isy = j; s.isy_n = n; }
  for (int k = 0; k <= g.nz; ++k)
    for (int n = 0; n < NP; ++n)
      if (std::fabs(g.zmax_global - g.Z(k, n) - zzs) < delta_z) {
        delta_z = std::fabs(g.zmax_global - g.Z(k, n) - zzs); s.isz = k; s.isz_n = n;
      }
  // local coordinates, possibly outside [-1,1] (ses3d_init.f90:431-433)
  s.zzs_loc = (g.Z(s.isz, LPD) + g.Z(s.isz, 0) - 2.0f * (g.zmax_global - zzs)) / (g.Z(s.isz, 0) - g.Z(s.isz, LPD));
  s.yys_loc = (2.0f * s.yys - g.Y(s.isy, LPD) - g.Y(s.isy, 0)) / (g.Y(s.isy, LPD) - g.Y(s.isy, 0));
  s.xxs_loc = (2.0f * s.xxs - g.X(s.isx, LPD) - g.X(s.isx, 0)) / (g.X(s.isx, LPD) - g.X(s.isx, 0));
  for (int in = 0; in < NP; ++in)
    for (int jn = 0; jn < NP; ++jn)
      for (int kn = 0; kn < NP; ++kn) {
        float d = lgll(in, s.xxs_loc) * lgll(jn, s.yys_loc) * lgll(kn, s.zzs_loc);
        if (source_type == 10) {  // ses3d_miscellaneous.f90:126-127
          d = d / (g.w[in] * g.w[jn] * g.w[kn]);
          d = d / (g.Z(s.isz, kn) * g.Z(s.isz, kn) * std::sin(g.X(s.isx, in)) * g.Jac);
        }
        s.delta[in + NP * jn + NP * NP * kn] = d;
      }
}

std::vector<Receiver> locate_receivers(const Geometry &g, int nr_global, const float *recloc_deg) {
  const float pi = g.pi;
  const float tol = pi / (float)(180 * 100000);  // ses3d_init.f90:28
  std::vector<Receiver> out;
  for (int n = 0; n < nr_global; ++n) {
    float rc1 = recloc_deg[3 * n] * pi / 180.0f;  // ses3d_input.f90:541-542
    float rc2 = recloc_deg[3 * n + 1] * pi / 180.0f;
    float rc3 = recloc_deg[3 * n + 2];
    if (!(rc1 <= g.xmax && rc1 > g.xmin && rc2 <= g.ymax && rc2 > g.ymin && g.zmax_global - rc3 <= g.zmax &&
          g.zmax_global - rc3 > g.zmin))
      continue;
    Receiver r;  // a receiver in the box that matches no element keeps zeros, as the reference's static arrays
    r.global_index = n;
    // The reference tests every element (i outer, j, k inner; ses3d_init.f90:300-325) and
    // keeps the last match. The test is a conjunction of one condition per axis, so the
    // matches form a product set whose last element in that order is the largest matching
    // index on each axis: three scans instead of one over all elements.
    int im = -1, jm = -1, km = -1;
    for (int i = 0; i <= g.nx; ++i)
      if (rc1 <= g.X(i, LPD) + tol && rc1 >= g.X(i, 0) - tol) im = i;
    for (int j = 0; j <= g.ny; ++j)
      if (rc2 <= g.Y(j, LPD) + tol && rc2 >= g.Y(j, 0) - tol) jm = j;
    for (int k = 0; k <= g.nz; ++k)
      if (g.zmax_global - rc3 <= g.Z(k, 0) && g.zmax_global - rc3 >= g.Z(k, LPD)) km = k;
    if (im >= 0 && jm >= 0 && km >= 0) {
      r.std[0] = 2.0f * ((rc1 - g.xmin) / g.dx - (float)im) - 1.0f;
      r.std[1] = 2.0f * ((rc2 - g.ymin) / g.dy - (float)jm) - 1.0f;
      r.std[2] = -2.0f * ((g.zmax_global - rc3 - g.zmax) / g.dz + (float)km) - 1.0f;
      r.loc[0] = rc1; r.loc[1] = rc2; r.loc[2] = rc3;
      r.rx = im; r.ry = jm; r.rz = km;
    }
    for (int i = 0; i < NP; ++i)
      for (int j = 0; j < NP; ++j)
        for (int k = 0; k < NP; ++k)
          r.weight[i + NP * j + NP * NP * k] = lgll(i, r.std[0]) * lgll(j, r.std[1]) * lgll(k, r.std[2]);
    out.push_back(r);
  }
  return out;
}

std::vector<AdjointSource> locate_adjoint_sources(const Geometry &g, int n, const float *loc_deg) {
  const float pi = g.pi;
  std::vector<AdjointSource> out;
  for (int k = 0; k < n; ++k) {
    float a1 = loc_deg[3 * k] * pi / 180.0f;  // ses3d_input.f90:600-601
    float a2 = loc_deg[3 * k + 1] * pi / 180.0f;
    float a3 = loc_deg[3 * k + 2];
    if (!(a1 <= g.xmax && a1 > g.xmin && a2 <= g.ymax && a2 > g.ymin && g.zmax_global - a3 <= g.zmax &&
          g.zmax_global - a3 > g.zmin))
      continue;
    AdjointSource s;
    s.global_index = k;
    // ses3d_init.f90:512-568: nearest knot from a start of the box width
    float delta_x = g.xmax - g.xmin;
    for (int i = 0; i <= g.nx; ++i)
      for (int m = 0; m < NP; ++m)
        if (std::fabs(a1 - g.X(i, m)) < delta_x) { s.is[0] = i; s.isn[0] = m; delta_x = std::fabs(a1 - g.X(i, m)); }
    s.loc_std[0] = (2.0f * a1 - g.X(s.is[0], LPD) - g.X(s.is[0], 0)) / (g.X(s.is[0], LPD) - g.X(s.is[0], 0));
    float delta_y = g.ymax - g.ymin;
    for (int i = 0; i <= g.ny; ++i)
      for (int m = 0; m < NP; ++m)
        if (std::fabs(a2 - g.Y(i, m)) < delta_y) { s.is[1] = i; s.isn[1] = m; delta_y = std::fabs(a2 - g.Y(i, m)); }
    s.loc_std[1] = (2.0f * a2 - g.Y(s.is[1], LPD) - g.Y(s.is[1], 0)) / (g.Y(s.is[1], LPD) - g.Y(s.is[1], 0));
    float delta_z = g.zmax - g.zmin;
    for (int i = 0; i <= g.nz; ++i)
      for (int m = 0; m < NP; ++m)
        if (std::fabs(g.zmax_global - a3 - g.Z(i, m)) < delta_z) {
          s.is[2] = i; s.isn[2] = m; delta_z = std::fabs(g.zmax_global - a3 - g.Z(i, m));
        }
    s.loc_std[2] = (g.Z(s.is[2], LPD) + g.Z(s.is[2], 0) - 2.0f * (g.zmax_global - a3)) /
                   (g.Z(s.is[2], 0) - g.Z(s.is[2], LPD));
    for (int in = 0; in < NP; ++in)
      for (int jn = 0; jn < NP; ++jn)
        for (int kn = 0; kn < NP; ++kn)
          s.delta[in + NP * jn + NP * NP * kn] =
              lgll(in, s.loc_std[0]) * lgll(jn, s.loc_std[1]) * lgll(kn, s.loc_std[2]);
    out.push_back(s);
  }
  return out;
}

}  // namespace ses3d

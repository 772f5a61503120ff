// setup.hpp -- host-side set-up of the SES3D mesh: GLL tables, element-node
// coordinates, PML profiles, source/receiver location.
//
// All arithmetic is FP32 in the reference's expression order; this file is
// compiled with -ffp-contract=off so the results are bit-identical to the
// reference's gfortran build (index and location work must be bit-exact).
// Fields that the reference stores as 6-D arrays but that depend on one axis
// only (x, sin/cot theta, r, raw PML profiles) are kept as 1-D tables.
#pragma once
#include <string>
#include <vector>

namespace ses3d {

constexpr int LPD = 4;     // Lagrange degree implemented by the kernels
constexpr int NP = LPD + 1;
constexpr int NPE = NP * NP * NP;  // GLL nodes per element

struct Geometry {
  int nx = 0, ny = 0, nz = 0;    // reference nx: elements - 1
  int ex = 0, ey = 0, ez = 0;    // elements per axis
  long long E = 0, N = 0;        // elements, local nodes
  int GX = 0, GY = 0, GZ = 0;    // global nodes per axis
  long long G = 0;
  int pml = 2;
  float xmin = 0, xmax = 0, ymin = 0, ymax = 0, zmin = 0, zmax = 0, zmax_global = 0;
  float pi = 0;
  float knots[NP], w[NP], dl[NP][NP];  // dl[i][j]: derivative of poly i at knot j
  float dx = 0, dy = 0, dz = 0, Jac = 0;
  std::vector<float> x, y, z;          // [i*NP + n]
  std::vector<float> sin_x, cot_x;     // [i*NP + n]
  std::vector<float> pxr, pyr, pzr;    // raw PML profile per element node [i*NP + n]
  std::vector<float> pxg, pyg, pzg;    // raw PML profile of the last writer per global index

  float X(int i, int n) const { return x[(size_t)i * NP + n]; }
  float Y(int j, int n) const { return y[(size_t)j * NP + n]; }
  float Z(int k, int n) const { return z[(size_t)k * NP + n]; }
};

// Builds the geometry (SOURCE/ses3d_init.f90:91-248 and 574-709).
// Returns an empty string on success, else an error message.
std::string build_geometry(Geometry &g, int nx, int ny, int nz, int pml, float xmin, float xmax, float ymin,
                           float ymax, float zmin, float zmax, float zmax_global);

// lgll(lpd, i, x): SOURCE/ses3d_miscellaneous.f90:377-481.
float lgll(int i, float x);

// Normalised PML profiles and taper of one node from its raw axis profiles
// (SOURCE/ses3d_init.f90:678-686).
void pml_normalise(float pxr, float pyr, float pzr, float &px, float &py, float &pz, float &prof, float &taper);

struct PointSource {
  int is_source = 0;
  int isx = 0, isy = 0, isz = 0, isx_n = 0, isy_n = 0, isz_n = 0;
  float xxs = 0, yys = 0, zzs = 0;            // radians, radians, m
  float xxs_loc = 0, yys_loc = 0, zzs_loc = 0;
  float delta[NPE];                           // per node, n = in + 5 jn + 25 kn
};

// Source in event-file units; type 10 gives the moment-tensor delta
// (SOURCE/ses3d_miscellaneous.f90:126-127), types 1-3 the single-force delta (:39).
// SOURCE/ses3d_input.f90:319-320,407-409 and SOURCE/ses3d_init.f90:363-439.
void locate_source(const Geometry &g, float xxs_deg, float yys_deg, float zzs, int source_type, PointSource &s);

struct Receiver {
  int global_index = 0;
  int rx = 0, ry = 0, rz = 0;
  float std[3] = {0, 0, 0};   // recloc_std
  float loc[3] = {0, 0, 0};   // recloc (radians, radians, depth)
  float weight[NPE];          // lgll(i)*lgll(j)*lgll(k) per node (ses3d_output.f90:483)
};

// SOURCE/ses3d_input.f90:541-542 and SOURCE/ses3d_init.f90:292-347.
std::vector<Receiver> locate_receivers(const Geometry &g, int nr_global, const float *recloc_deg);

struct AdjointSource {
  int global_index = 0;
  int is[3] = {0, 0, 0}, isn[3] = {0, 0, 0};
  float loc_std[3] = {0, 0, 0};  // xxs_ad_loc, yys_ad_loc, zzs_ad_loc
  float delta[NPE];
};

// SOURCE/ses3d_input.f90:600-601 and SOURCE/ses3d_init.f90:453-572.
std::vector<AdjointSource> locate_adjoint_sources(const Geometry &g, int n, const float *loc_deg);

}  // namespace ses3d

// kernels.cuh -- device data structures shared by the SES3D kernels and the C ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ses3d {

constexpr int TPE = 128;  // threads per element (125 GLL nodes + 3 idle lanes)

// Element-local state, element-blocked: [event][element][36 fields][125 nodes] (node
// n = in + 5 jn + 25 kn), i.e. the 36 fields of one element are 18,000 contiguous bytes.
// Outside the PML all profiles vanish and the three mirror stresses (syx, szx, szy) stay
// equal to their partners (sxy, sxz, syz); they are stored last of the nine so that lean
// stepping can leave them out as one range.
enum StateField {
  F_SXX = 0, F_SYY, F_SZZ, F_SXY, F_SXZ, F_SYZ, F_SYX, F_SZX, F_SZY,        // PML-split stresses
  F_DXUX = 9, F_DYUY, F_DZUZ, F_DXUY, F_DYUX, F_DXUZ, F_DZUX, F_DYUZ, F_DZUY, // displacement gradients
  F_M = 18,  // memory variables: F_M + 3*comp + mech, comp = xx, yy, zz, xy, xz, yz
  NSTATE = 36
};

// Per-node material coefficients, element-blocked with 128-float rows:
// [element][6 fields][128] (nodes 125..127 zero), 3,072 bytes per element.
enum MatField { M_CLAM = 0, M_C2MUT, M_C2MT, M_A, M_B2, M_C, NMAT };
constexpr int ELEM_STATE = NSTATE * 125;  // floats of one element's state
constexpr int MAT_ROW = 128;
constexpr int ELEM_MAT = NMAT * MAT_ROW;  // floats of one element's material block
// Adjoint-only per-node quantities.
enum GMatField { G_RHO = 0, G_CP, G_CS, G_MU, G_KAPPA, G_QQ, NGMAT };
// Forward record fields (the ffd files of the reference).
enum RecField { R_VX = 0, R_VY, R_VZ, R_EXX, R_EYY, R_EZZ, R_EXY, R_EXZ, R_EYZ, NREC };
constexpr int NGRAD = 8;  // rho, cp, csh, csv, Q_mu, alpha_mu, Q_kappa, alpha_kappa

// Small per-mesh coefficient tables, copied into shared memory by each CTA.
struct KTab {
  float Dx[5][5], Dy[5][5], Dz[5][5];  // strain: D[i][q] = 2 dl(q,i) / d   (ses3d_evolution.f90:66-68)
  float dlT[5][5];                     // divergence: dl(i,q)               (ses3d_evolution.f90:247-249)
  float CX[5][5], CY[5][5], CZ[5][5];  // (2/dx)Jac w_j w_k, (2/dy)Jac w_i w_k, -(2/dz)Jac w_i w_j
  float w[5];
};
constexpr int KTAB_FLOATS = sizeof(KTab) / sizeof(float);

struct Consts {
  int ex, ey, ez, nev, nt;
  int GX, GY, GZ;
  long long E, N, G;
  float dt;
  float a_k[3];   // dt / tau_p(k)
  float L_k[3];   // dt * D_p(k) / tau_p(k)
  float s_grad;   // samp_ad * dt
  float Jac;
  float tau_p[3], D_p[3];
  float q_alpha_w[3];  // dP/dalpha_k tau_k / D_k of the alpha kernels (ses3d_grad_Q.f90:126)
  int pml;        // PML width in elements
  int lean;       // plain forward: displacement gradients kept only in PML elements
  int iso;        // the model's A, B and C records are zero: the element kernels read the
                  // first three material fields only (the others multiply zeros)
  // t / GX for 32-bit t as (m + ((t - m) >> 1)) >> shift with m = umulhi(t, gx_magic)
  // (division by an invariant integer, Granlund & Montgomery 1994); GX >= 2
  unsigned gx_magic;
  int gx_shift;
  double s_jac;   // samp_ad dt / Jac in FP64: the weight of one kernel-correlation term
};

// Fields of the forward state the backward iteration reads, packed per element into an
// iteration slot: the 9 displacement gradients, then (with attenuation) the 6 per-component
// sums of the 3 memory variables, Mxx .. Myz.
constexpr int SLOT_FIELDS_DISS = 15, SLOT_FIELDS_ELASTIC = 9;
__host__ __device__ constexpr int slot_fields(bool diss) { return diss ? SLOT_FIELDS_DISS : SLOT_FIELDS_ELASTIC; }
// Floats of one element's slot block: its fields rounded up to a multiple of 4 floats, so
// that every block starts 16-byte aligned (1,876 and 1,128).
__host__ __device__ constexpr int slot_stride(bool diss) { return (slot_fields(diss) * 125 + 3) & ~3; }

struct Ptrs {
  const KTab *ktab;
  const float *sin_x, *cot_x, *r_z;     // [i*5+n], [k*5+n]
  const float *inv_sin, *inv_r;         // reciprocals of sin_x and r_z
  const float *pxr, *pyr, *pzr;         // raw PML per element node
  const float *pxg, *pyg, *pzg;         // raw PML per global index (last writer)
  const float *MM;                      // [G]
  const float *iMM;                     // [G] 1 / MM
  const float *mat;                     // [E][NMAT][128]
  const float *gmat;                    // [NGMAT][E][125] (adjoint)
  float *state;                         // [nev][E][NSTATE][125]
  float *v;                             // [nev][3][G]
  float *f;                             // [nev][E][3][125] element-local forces (scratch)
  float *fg;                            // [nev][3][G] assembled forces of the iteration, or null
  int *d_it;                            // completed iterations
  int *err;                             // device error word (bounded waits that gave up)
  // moment-tensor source per event
  const int *src_elem;                  // [nev], -1: none
  const float *src_delta;               // [nev][125]
  const float *src_mom;                 // [nev][6]
  const float *stf;                     // [nev][nt]
  // forward records / kernels
  float *rec;                           // record of this iteration: [nev][NREC][N]
  double *grad;                         // [nev][NGRAD][N]
  int grad_q;                           // accumulate the Q kernels too
  float *u;                             // [nev][3][G] displacement (time integral of v) of runs that
                                        // store records or correlate kernels lean, or null
  float *slot;                          // [nev][E][slot_stride]: the iteration's starting state,
                                        // packed for the exact adjoint, or null
};

// Exact discrete adjoint of one iteration (adjoint.cu): the forward state the iteration
// started from and the forces it assembled, the adjoint state, scratch and the FP64
// gradient accumulators.
struct AdjPtrs {
  const float *fstate;                  // [nev][E][slot_stride] packed forward state before the iteration
  const float *fv;                      // [nev][3][G] forward velocity before the iteration
  const float *fg;                      // [nev][3][G] assembled forces of the iteration
  float *astate;                        // [nev][E][NSTATE][125] adjoint state (in: after, out: before)
  float *av;                            // [nev][3][G] adjoint velocity (in: after, out: before)
  float *aF;                            // [nev][3][G] adjoint of the assembled forces (scratch)
  float *af;                            // [nev][E][3][125] element contributions to the adjoint velocity
  double *gmat;                         // [nev][E][NMAT][125] d misfit / d stress-rate coefficient
  double *gimm;                         // [nev][G] d misfit / d (1 / MM)
  int *d_ait;                           // iteration counter of the backward run (iteration - 1)
  int zero_d;                           // the adjoint displacement gradients outside the PML are
                                        // zero (a backward run started with them zero keeps them so)
};

}  // namespace ses3d

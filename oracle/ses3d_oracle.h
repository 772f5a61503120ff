/*
 * ses3d_oracle.h -- C interface of the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY. The oracle is a line-by-line C++ restatement of the
 * reference SES3D Fortran solver (SOURCE/ses3d_init.f90, ses3d_evolution.f90,
 * ses3d_miscellaneous.f90, ses3d_output.f90, ses3d_grad.f90, ses3d_grad_Q.f90,
 * ses3d_main.f90). It is used by tests/, by __graft_entry__.smoke() and by the
 * cpu_baseline / reference legs of bench.py as the checker and as the timed CPU
 * baseline. Nothing in the product (ses3d_gb300/) links or calls it.
 *
 * Parity status: the reference ships no tests, golden vectors or fixtures with
 * expected outputs, and it cannot be compiled here (Fortran + MPI); the oracle is
 * pinned against builder-made known answers only (GLL identities, quadrature
 * exactness, analytic travel times) -- "parity unpinned" by the reference itself.
 *
 * Layout: every field uses the reference layout, Fortran column-major
 * (i,j,k,in,jn,kn) with the element index i fastest
 * (SOURCE/ses3d_modules.f90:58-83), so flat index = e + E*n with
 * e = i + (nx+1)*(j + (ny+1)*k) and n = in + L*(jn + L*kn), L = lpd+1.
 * Global (assembled) fields are (0:(nx+1)*lpd, 0:(ny+1)*lpd, 0:(nz+1)*lpd),
 * first index fastest (SOURCE/ses3d_modules.f90:105-108).
 */
#ifndef SES3D_ORACLE_H
#define SES3D_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Indices of the real scalars read from the text inputs. Each is passed twice:
 * parsed with strtof (the FP32 oracle, as gfortran reads REAL(4)) and with
 * strtod (the FP64 oracle, standing in for a -fdefault-real-8 build). */
enum {
  OR_DT = 0,                       /* event: dt (ses3d_input.f90:204)            */
  OR_XMIN, OR_XMAX, OR_YMIN, OR_YMAX, OR_ZMIN, OR_ZMAX,  /* boxfile (ses3d_input.f90:96-98) */
  OR_ZMAX_GLOBAL,                  /* setup z_max (ses3d_input.f90:275)          */
  OR_XXS, OR_YYS, OR_ZZS,          /* event source, degrees/degrees/m depth      */
  OR_MXX, OR_MYY, OR_MZZ, OR_MXY, OR_MXZ, OR_MYZ,        /* ses3d_input.f90:219-229 */
  OR_TAU1, OR_TAU2, OR_TAU3,       /* relax (ses3d_input.f90:339-341)            */
  OR_D1, OR_D2, OR_D3,             /* relax (ses3d_input.f90:348-350)            */
  OR_NREAL
};

typedef struct {
  int nx, ny, nz;          /* reference nx: elements - 1 (ses3d_input.f90:107) */
  int lpd;                 /* Lagrange degree 1..7 */
  int pml;                 /* PML width in elements (compile-time `pml` in the reference) */
  int is_diss, adjoint_flag, samp_ad, nt, source_type;
  int grad_variant;        /* 0: ses3d_grad.f90 (linked by s_make); 1: ses3d_grad_Q.f90 */
  int nr_global;           /* receivers in recfile */
  int nr_adsrc_global;     /* adjoint sources in ad_srcfile */
  const float  *rf;        /* OR_NREAL scalars, strtof */
  const double *rd;        /* OR_NREAL scalars, strtod */
  const float  *so_f;  const double *so_d;      /* nt samples of the stf */
  const float  *rec_f; const double *rec_d;     /* 3*nr_global: colat deg, lon deg, depth m */
  const float  *adloc_f; const double *adloc_d; /* 3*nr_adsrc_global, same units */
  const float  *adstf_f; const double *adstf_d; /* [nr_adsrc_global][3][nt] */
  const float *rhoinv, *mu, *lambda, *A, *B, *C, *Q; /* compact model records, F-order */
  const int *saving_vector;                     /* nt entries, adjoint (flag 2) run */
} oracle_input;

void *oracle_create(const oracle_input *in, int fp64);
void  oracle_destroy(void *h);
/* Runs n iterations of the ses3d_main.f90:95-178 loop body. Returns 0. */
int   oracle_run(void *h, int n);
int   oracle_it(void *h);
/* Size (elements) of a named array, -1 if unknown. */
long  oracle_size(void *h, const char *name);
/* Copies a named real array (float or double, per the handle) into out. */
int   oracle_get(void *h, const char *name, void *out);
/* Overwrites a named real array (same names and sizes as oracle_get; values in the
 * handle's precision): initial states of parity runs. Returns -1 for an unknown name. */
int   oracle_set(void *h, const char *name, const void *in);
/* Named integer scalars / arrays (nr, rx, ry, rz, isx, ... ). */
long  oracle_get_int(void *h, const char *name, int *out);
/* Forward-field records kept by a flag-1 run (9 fields each, ses3d_main.f90:148-158). */
int   oracle_nrecords(void *h);
int   oracle_get_record(void *h, int r, void *out);
/* Records supplied to a flag-2 run; read last to first (ses3d_output.f90:201-226). */
int   oracle_set_records(void *h, int nrec, const void *data);
/* Reals parsed exactly as gfortran's list-directed read of REAL(4). */
float oracle_strtof(const char *s);

#ifdef __cplusplus
}
#endif
#endif

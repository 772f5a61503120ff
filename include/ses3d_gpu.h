/*
 * ses3d_gpu.h -- C ABI of the GB300 SES3D time-stepping library (libses3d_gpu.so).
 *
 * The reference solver has no library interface: its hot path is a set of
 * argument-less Fortran subroutines that mutate `module variables`
 * (SOURCE/ses3d_modules.f90:33-233) and are called in a fixed order by
 * `program ses3d_main` (SOURCE/ses3d_main.f90:77-180). Each entry point below
 * replaces one of those subroutines (or the part of one that touches the hot
 * path) and states which. A Fortran driver binds them with ISO_C_BINDING; the
 * Python package binds them with ctypes.
 *
 * Conventions
 *  - Every entry point returns 0 on success or a negative SES3D_E* code;
 *    ses3d_gpu_last_error() gives a message for the last failure on a handle.
 *  - Host arrays are caller-owned and only read/written during the call.
 *    Arrays use the reference layout: Fortran column-major
 *    (i,j,k,in,jn,kn), element index i fastest, exactly the records of
 *    MODELS/MODELS/<name><rank> and of the ofd/ffd output files.
 *  - The library owns all device memory of a handle. One handle per
 *    (process, device); calls on one handle are not thread-safe.
 *  - Several events that share one mesh and model run together in one handle
 *    (config.n_events > 1): every time step is one launch sequence for all of
 *    them. `event` arguments are 0-based.
 *  - All field arithmetic is FP32 as in the reference; the Frechet-kernel
 *    time integrals accumulate in FP64.
 */
#ifndef SES3D_GPU_H
#define SES3D_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SES3D_OK 0
#define SES3D_E_CONFIG (-1)   /* invalid configuration or argument */
#define SES3D_E_OOM (-2)      /* device allocation failed */
#define SES3D_E_CUDA (-3)     /* CUDA runtime error */
#define SES3D_E_STATE (-4)    /* call out of order (e.g. step before set_model) */
#define SES3D_E_NAN (-5)      /* non-finite wavefield detected by the watchdog */
#define SES3D_E_NOTFOUND (-6) /* reserved: a source or receiver outside the box is not an error; it is
                                 reported through is_source / nr_out, as each reference rank does */
#define SES3D_E_NODEV (-7)    /* no CUDA device */

typedef struct ses3d_gpu ses3d_gpu;

/* Run configuration: the values ses3d_input reads from the boxfile, the setup,
 * event and relax files (SOURCE/ses3d_input.f90:44-357), plus the reference's
 * compile-time `pml` (SOURCE/ses3d_modules.f90:21), here a run-time value. */
typedef struct {
  int32_t nx, ny, nz;     /* elements - 1 in x (colatitude), y (longitude), z (radius) */
  int32_t lpd;            /* Lagrange degree; this library implements lpd = 4 */
  int32_t pml;            /* PML width in elements (reference default 2) */
  int32_t is_diss;        /* 1: anelastic (3 SLS mechanisms), 0: elastic */
  int32_t adjoint_flag;   /* 0 forward, 1 forward + store, 2 adjoint + kernels */
  int32_t samp_ad;        /* forward-field storing rate */
  int32_t nt;             /* time steps */
  int32_t n_events;       /* events sharing this mesh (1 = plain run) */
  int32_t grad_variant;   /* 0: SOURCE/ses3d_grad.f90, 1: SOURCE/ses3d_grad_Q.f90 */
  int32_t reserved;
  float dt;
  float xmin, xmax, ymin, ymax; /* box, radians (boxfile physical boundaries) */
  float zmin, zmax;             /* box radii, m */
  float zmax_global;            /* setup z_max, m (depths are measured from it) */
  float tau_p[3], D_p[3];       /* relax file */
} ses3d_config;

/* Library version string. */
const char *ses3d_gpu_version(void);

/* Makes `device` the current device of this library's CUDA runtime for the calling thread;
 * handles are created on the current device. A process that drives one GPU of several
 * (one rank per GPU) selects its GPU before creating handles. No counterpart in the
 * reference (one MPI rank per core). */
int ses3d_gpu_select_device(int device);

/* Creates a handle: GLL tables, geometry, PML profiles and all device buffers.
 * Replaces the geometry part of ses3d_init (SOURCE/ses3d_init.f90:87-248,574-709). */
int ses3d_gpu_create(const ses3d_config *cfg, ses3d_gpu **out);

/* Frees every resource of the handle. */
int ses3d_gpu_destroy(ses3d_gpu *h);

/* Message for the last failure on h (or for the last failed create if h is NULL). */
const char *ses3d_gpu_last_error(const ses3d_gpu *h);

/* Model records rhoinv, mu, lambda, A, B, C, Q: compact (nx+1,ny+1,nz+1,5,5,5)
 * F-order FP32 arrays. Q may be NULL when is_diss == 0. Derives kappa, mu_tau,
 * cp, cs, rho and the mass matrix.
 * Replaces SOURCE/ses3d_input.f90:472-501 and SOURCE/ses3d_init.f90:47-61,254-279. */
int ses3d_gpu_set_model(ses3d_gpu *h, const float *rhoinv, const float *mu, const float *lambda,
                        const float *A, const float *B, const float *C, const float *Q);

/* Point source of one event, in the event-file units: colatitude and longitude
 * in degrees, depth in m; source_type 1/2/3 single force, 10 moment tensor with
 * mom = {Mxx, Myy, Mzz, Mxy, Mxz, Myz}; so = nt source-time-function samples.
 * Locates the source element and local coordinates as the reference does.
 * *is_source (may be NULL) receives 1 if the source lies in the box.
 * Replaces SOURCE/ses3d_input.f90:319-320,405-437 and SOURCE/ses3d_init.f90:363-439
 * (the per-step injection, SOURCE/ses3d_miscellaneous.f90:11-150, runs on the GPU). */
int ses3d_gpu_set_source(ses3d_gpu *h, int event, float xxs_deg, float yys_deg, float zzs,
                         int source_type, const float mom[6], const float *so, int *is_source);

/* Receivers of one event: recloc = nr_global x (colatitude deg, longitude deg,
 * depth m) as in recfile_<id>. Locates each receiver (last matching element
 * wins). *nr_out receives the number kept (receivers inside the box);
 * kept (may be NULL, nr_global entries) receives for each kept receiver, in
 * order, its 0-based index in recloc.
 * Replaces SOURCE/ses3d_input.f90:533-544 and SOURCE/ses3d_init.f90:285-357. */
int ses3d_gpu_set_receivers(ses3d_gpu *h, int event, int nr_global, const float *recloc,
                            int *nr_out, int *kept);

/* Adjoint sources of one event (adjoint_flag == 2): loc = n x (colat deg, lon
 * deg, depth m) as in ad_srcfile; stf = n x 3 x nt samples (x, y, z) as in
 * ad_src_<k>, applied in file order. *n_out receives the number in the box.
 * Replaces SOURCE/ses3d_input.f90:584-618 and SOURCE/ses3d_init.f90:445-572. */
int ses3d_gpu_set_adjoint_sources(ses3d_gpu *h, int event, int n, const float *loc,
                                  const float *stf, int *n_out);

/* Runs n iterations of the time loop body for all events: ses3d_evolution,
 * record_seismograms (flags 0/1), forward-field store (flag 1) and ses3d_grad
 * (flag 2). Replaces SOURCE/ses3d_main.f90:95-178 with
 * SOURCE/ses3d_evolution.f90:7-373, SOURCE/ses3d_output.f90:456-497,
 * SOURCE/ses3d_main.f90:142-166 and SOURCE/ses3d_grad.f90:25-85. */
int ses3d_gpu_step(ses3d_gpu *h, int n);

/* Completed iterations (the reference `it` after the last step). */
int ses3d_gpu_current_step(const ses3d_gpu *h);

/* Velocity seismograms of one event, each (nr, nt) with the receiver index
 * fastest (seismogram_x(1:nr,1:nt), SOURCE/ses3d_modules.f90:196-198). Entry
 * it-1 holds the value recorded in iteration it (the pre-update velocity). */
int ses3d_gpu_get_seismograms(ses3d_gpu *h, int event, float *sx, float *sy, float *sz);

/* Field identifiers for ses3d_gpu_get_field. */
enum {
  SES3D_FIELD_VX = 0, SES3D_FIELD_VY, SES3D_FIELD_VZ, /* local form of the current global v */
  SES3D_FIELD_VX_GLOBAL, SES3D_FIELD_VY_GLOBAL, SES3D_FIELD_VZ_GLOBAL, /* assembled v */
  SES3D_FIELD_SXX_PML, SES3D_FIELD_SYY_PML, SES3D_FIELD_SZZ_PML, SES3D_FIELD_SXY_PML,
  SES3D_FIELD_SYX_PML, SES3D_FIELD_SXZ_PML, SES3D_FIELD_SZX_PML, SES3D_FIELD_SYZ_PML,
  SES3D_FIELD_SZY_PML,
  SES3D_FIELD_DXUX, SES3D_FIELD_DYUY, SES3D_FIELD_DZUZ, SES3D_FIELD_DXUY, SES3D_FIELD_DYUX,
  SES3D_FIELD_DXUZ, SES3D_FIELD_DZUX, SES3D_FIELD_DYUZ, SES3D_FIELD_DZUY,
  SES3D_FIELD_MXX, SES3D_FIELD_MYY, SES3D_FIELD_MZZ, SES3D_FIELD_MXY, SES3D_FIELD_MXZ,
  SES3D_FIELD_MYZ, /* memory variables: (3, nx+1, ..., 5) mechanism fastest */
  SES3D_FIELD_MM_GLOBAL, /* assembled mass matrix */
  SES3D_FIELD_COUNT
};

/* One field of one event in the reference layout (local fields: N = 125(nx+1)(ny+1)(nz+1)
 * floats; memory variables 3N; global fields ((nx+1)*4+1)((ny+1)*4+1)((nz+1)*4+1)).
 * SES3D_FIELD_VX..VZ are the snapshot fields of ses3d_output (SOURCE/ses3d_output.f90:293-312).
 * SES3D_E_STATE: a displacement gradient after lean iterations (ses3d_gpu_set_lean), or a
 * handle that steps caller-owned wavefields (ses3d_gpu_step_external). */
int ses3d_gpu_get_field(ses3d_gpu *h, int event, int field, float *out);

/* Sets one state field (same layout as get_field) -- restart / test injection. */
int ses3d_gpu_set_field(ses3d_gpu *h, int event, int field, const float *in);

/* Kernel identifiers for ses3d_gpu_get_kernel. */
enum {
  SES3D_KERNEL_RHO = 0, SES3D_KERNEL_CP, SES3D_KERNEL_CSH, SES3D_KERNEL_CSV,
  SES3D_KERNEL_Q_MU, SES3D_KERNEL_ALPHA_MU, SES3D_KERNEL_Q_KAPPA, SES3D_KERNEL_ALPHA_KAPPA,
  SES3D_KERNEL_COUNT
};

/* Frechet kernel of one event (FP64 accumulator) in the reference layout, N doubles:
 * grad_rho, grad_cp, grad_csh, grad_csv (SOURCE/ses3d_output.f90:318-342) and the
 * research Q kernels of SOURCE/ses3d_grad_Q.f90 (normalised after the last step). */
int ses3d_gpu_get_kernel(ses3d_gpu *h, int event, int which, double *out);

/* Sum over all events of one kernel (FP64, events added in index order on the device),
 * N doubles in the reference layout: the multi-event misfit gradient. The reference runs
 * one event per job and sums the grad_* files afterwards; this returns that sum with one
 * transfer. */
int ses3d_gpu_get_kernel_sum(ses3d_gpu *h, int which, double *out);

/* The same sum written to device memory (N doubles on the handle's device, reference
 * layout), for callers that keep the gradient on the GPU (PyTorch). No counterpart in the
 * reference. */
int ses3d_gpu_get_kernel_sum_device(ses3d_gpu *h, int which, double *out);

/* acc[q] = acc[q] + (the event sum of get_kernel_sum_device) on the handle's device: sums
 * of event sub-batches run in separate handles, added in sub-batch order. No counterpart
 * in the reference (its per-event grad_* files are summed afterwards). */
int ses3d_gpu_add_kernel_sum_device(ses3d_gpu *h, int which, double *acc);

/* Misfit gradient with respect to a model record from an event-summed kernel (N doubles,
 * reference layout, device memory): out[q] = (ksum[q] * W[q]) * (scale * Jac), divided by
 * divisor[q] when divisor is not NULL, where W[q] = w_in w_jn w_kn Jac r^2 sin(theta) is the
 * quadrature volume of GLL point q of cfg's box (FP64). With ses3d's kernel convention
 * (grad_* carry 1/Jac, SOURCE/ses3d_grad.f90:77-83) and scale = -dL/dchi this is dL/dm;
 * the Q_mu kernel takes divisor = Q. out and divisor are FP32 (f64 = 0) or FP64 (f64 = 1),
 * N values. Needs no handle (the handles of event sub-batches may be gone); runs on the
 * current device of this library and returns when done. No counterpart in the reference. */
int ses3d_gpu_misfit_gradient_device(const ses3d_config *cfg, const double *ksum, double scale,
                                     const void *divisor, void *out, int f64);

/* Forward-field records kept in device memory by an adjoint_flag == 1 run: one
 * record per stored iteration (it == 1, it % samp_ad == 0, it == nt), 9 fields of
 * N floats each: vx, vy, vz, exx, eyy, ezz, exy, exz, eyz -- the fields and order of
 * the ffd/<name>_<rank> files (SOURCE/ses3d_main.f90:148-158, SOURCE/ses3d_output.f90:138-162). */
int ses3d_gpu_record_count(const ses3d_gpu *h, int event);
int ses3d_gpu_get_record(ses3d_gpu *h, int event, int record, float *out);
int ses3d_gpu_put_record(ses3d_gpu *h, int event, int record, const float *in);

/* Checkpointed forward-field storage for adjoint runs. With records_per_segment = K > 0
 * a flag-1 run keeps one full-state checkpoint (element state and assembled velocity of
 * every event) before every K-th stored iteration instead of the records, and the flag-2
 * run recomputes the records of one segment at a time from its checkpoint on a second
 * wavefield (one extra forward pass in total). K = 0 (default) keeps every record in
 * device memory. Memory with K > 0: ceil(nrec / K) checkpoints, K records of 9 N floats
 * and one extra wavefield, per event. A checkpoint holds the element state (36 N floats,
 * or with lean stepping 24 N + 1500 E_pml: outside the PML the fields lean iterations do
 * not read are left out), the velocity and the displacement (6 G). Call before the flag-1
 * run starts. Replaces the disk store/restore of SOURCE/ses3d_output.f90:5-267. */
int ses3d_gpu_set_checkpointing(ses3d_gpu *h, int records_per_segment);

/* Two checkpoint levels (records_per_subsegment = K2 with 0 < K2 < K): the flag-2 run
 * recomputes a segment of K records once, keeping a full-state checkpoint before every
 * K2-th of its records, and then each sub-segment of K2 records from those as the adjoint
 * run reaches it (two extra forward passes in total). Memory per event: ceil(nrec / K)
 * + ceil(K / K2) - 1 checkpoints, K2 records and one extra wavefield -- for 96 x 96 x 40,
 * nt = 4000, samp_ad = 10 (401 records of 1.66 GB, full-state checkpoints of 7.2 GB)
 * K = 81, K2 = 21 need about 114 GB against 163 GB with one level (lean runs' 5.4-GB
 * checkpoints: one level, K = 36, about 146 GB). K2 = 0 is ses3d_gpu_set_checkpointing(h, K).
 * Extends the disk store/restore of SOURCE/ses3d_output.f90:5-267 (no counterpart). */
int ses3d_gpu_set_checkpoint_levels(ses3d_gpu *h, int records_per_segment, int records_per_subsegment);

/* Device memory the handle holds now, in bytes. */
int64_t ses3d_gpu_memory_bytes(const ses3d_gpu *h);

/* saving_vector of the forward run (nt entries; it where stored, else 0);
 * SOURCE/ses3d_main.f90:162 and SOURCE/ses3d_output.f90:379-392. */
int ses3d_gpu_get_saving_vector(const ses3d_gpu *h, int *out);
int ses3d_gpu_set_saving_vector(ses3d_gpu *h, const int *in);

/* Switches a handle that completed a flag-1 forward run into the flag-2 adjoint
 * run over the same records: zeroes the wavefield, keeps model, records and
 * saving_vector, sets it = 0 (the reference runs this as a second program start). */
int ses3d_gpu_begin_adjoint(ses3d_gpu *h);

/* Setup quantities for bit-exact checks of the index work of ses3d_init.
 * Integers: "nr", "rx", "ry", "rz", "isx", "isy", "isz", "is_source", "nr_adsrc", "is"
 * (3 x nr_adsrc), "isotropic" (1 when the model's A, B and C records are all zero: the
 * element kernels then read three of the six material fields per point); reals: "recloc_std" (3 x nr), "xxs_loc", "yys_loc", "zzs_loc",
 * "x", "y", "z" (element-node coordinates), "dl", "knots", "w", "Jac", "dx", "dy", "dz",
 * "prof_x", "prof_y", "prof_z", "taper" (N, reference layout). Returns the count
 * written (out may be NULL to query the size) or a negative code. */
long ses3d_gpu_get_setup_int(ses3d_gpu *h, int event, const char *name, int *out);
long ses3d_gpu_get_setup_real(ses3d_gpu *h, int event, const char *name, float *out);

/* Non-finite watchdog: the max |v| of each event at the last step (the quantity the
 * reference prints every step, SOURCE/ses3d_main.f90:111-130). */
int ses3d_gpu_vmax(ses3d_gpu *h, float *out);

/* Self-test of the device-side failure path (no counterpart in the reference): launches a
 * kernel whose wait on an mbarrier can never complete (it expects bytes no copy delivers)
 * and that gives up after limit_ms, exactly as the element kernel's bounded waits do.
 * Returns SES3D_E_CUDA with the bounded-wait message; the device error word is cleared
 * and the handle stays usable. */
int ses3d_gpu_selftest_wait(ses3d_gpu *h, int limit_ms);

/* Device-resident interface (zero-copy for PyTorch / CUDA callers). Pointers are
 * device pointers on the handle's device; layouts are the reference layouts.
 * Model upload from device memory: */
int ses3d_gpu_set_model_device(ses3d_gpu *h, const float *rhoinv, const float *mu,
                               const float *lambda, const float *A, const float *B,
                               const float *C, const float *Q);

/* The CUDA stream the handle launches on (cudaStream_t as void*). */
void *ses3d_gpu_stream(ses3d_gpu *h);

/* Timing/diagnostic counters: kernel launches issued by the library since create. */
int64_t ses3d_gpu_launch_count(const ses3d_gpu *h);

/* Captures the launch sequence of `n_per_graph` plain forward iterations into a
 * CUDA graph and replays it for subsequent ses3d_gpu_step calls (adjoint_flag 0
 * only; stored/gradient iterations always run eagerly). enable = 0 disables it. */
int ses3d_gpu_use_graph(ses3d_gpu *h, int enable, int n_per_graph);

/* Per-kernel device time: with profiling enabled, each eager iteration records CUDA
 * events on the handle's stream around its launches; which = 0 k_element, 1 k_node,
 * 2 k_receivers, 3 k_inject. ses3d_gpu_profile(h, 1) also resets the totals. */
int ses3d_gpu_profile(ses3d_gpu *h, int enable);
int ses3d_gpu_kernel_time(const ses3d_gpu *h, int which, double *total_ms, int64_t *launches);

/* Allocation-free forward iterations, for callers that cannot call cudaMalloc at the
 * point where they step the solver: code whose device memory belongs to another
 * allocator (a PyTorch or JAX caching allocator, a pre-sized memory pool) or that runs
 * in a loop where allocating is not allowed. It has no counterpart in the reference
 * (whose arrays are all static Fortran module variables).
 * The caller owns the wavefield and passes it in device memory:
 *   state: n_events x E x 36 x 125 floats (16-byte aligned) -- per event and element
 *          (i + ex (j + ey k)) a block of 36 fields of 125 nodes (in + 5 jn + 25 kn), the
 *          fields in the order sxx, syy, szz, sxy, sxz, syz, syx, szx, szy (PML
 *          stresses), dxux, dyuy, dzuz, dxuy, dyux, dxuz, dzux, dyuz, dzuy, then the
 *          memory variables Mxx, Myy, Mzz, Mxy, Mxz, Myz with the mechanism fastest
 *          (fields 18-35 unused when is_diss = 0);
 *   v:     n_events x 3 x G floats -- assembled velocity, component-major, global node
 *          gx + GX (gy + GY gz), GX = 4 ex + 1, GY = 4 ey + 1.
 * Zeroed buffers start a run at rest. Model, sources, receivers and the step counter
 * stay in the handle (set up earlier with the calls above); seismograms are recorded
 * into the handle. Only plain forward runs (adjoint_flag 0) are accepted.
 * Ordering: the library launches on its own stream (ses3d_gpu_stream). The caller's
 * writes to state and v must be complete before the call (synchronise, or make
 * ses3d_gpu_stream wait on an event recorded after the writes); the call returns after
 * its own work on the buffers has finished.
 * Lean stepping (ses3d_gpu_set_lean) applies: elements outside the PML then keep only the
 * first six stresses and the memory variables up to date; the displacement gradients
 * there are not integrated, and the mirror stresses there are brought up to date at the
 * start of the next call made with lean stepping off.
 * One handle steps either its own wavefield (ses3d_gpu_step) or caller-owned ones (this
 * call), not both: after the first external call, ses3d_gpu_step and the wavefield
 * fields of ses3d_gpu_get_field / set_field return SES3D_E_STATE, and a handle that has
 * already run ses3d_gpu_step rejects this call with SES3D_E_STATE.
 * The element forces between the element and node kernels live in a fixed array in
 * the library's device memory, 8,388,608 floats (32 MiB), which every GPU that loads
 * the library holds until the process exits: n_events x 3 x N must not exceed it
 * (e.g. one event of at most 2,796,202 GLL points); larger runs get SES3D_E_CONFIG.
 * The first call on a handle looks up that array's device address (which may load the
 * library's device code); make it before any stream capture. Calls that overlap on the
 * GPU (two handles or threads stepping at once) share the array and race.
 * The handle's device must be current. No cudaMalloc, cudaFree or other allocating
 * routine is called. */
int ses3d_gpu_step_external(ses3d_gpu *h, float *state, float *v, int n);

/* Exact discrete adjoint (no counterpart in the reference, whose ses3d_grad kernels are a
 * continuous-adjoint approximation: SOURCE/ses3d_grad.f90:77-83). The backward run of a
 * plain forward run is the transpose of its time step: the derivative of a misfit of the
 * seismograms with respect to the model records is the gradient of the discrete forward
 * run itself (what finite differences of the forward run converge to).
 * Call ses3d_gpu_exact_adjoint on a flag-0 handle before stepping: the forward run keeps a
 * full-state checkpoint every steps_per_checkpoint iterations. Lean stepping, chosen before
 * the forward run starts and kept for it, is exact for runs whose starting state has the
 * mirror stresses equal to their partners outside the PML (a run from rest): the
 * transposed step reads the velocities, memory variables, assembled forces and the
 * displacement gradients inside the PML, which lean iterations keep as full-state ones do.
 * After nt iterations, give each event's d misfit / d seismogram with
 * ses3d_gpu_exact_set_seismogram_adjoint (gx, gy, gz: (nr, nt) each, receiver fastest, the
 * layout of ses3d_gpu_get_seismograms; NULL = zero) and call ses3d_gpu_exact_backward: it
 * recomputes one checkpoint segment at a time (one extra forward pass) and runs the adjoint
 * iterations nt .. 1, accumulating the gradient in FP64. ses3d_gpu_exact_gradient returns
 * the event-summed d misfit / d record for which = 0..6: rhoinv, mu, lambda, A, B, C, Q
 * (N doubles, reference layout; device = 1: out is device memory on the handle's device).
 * Memory per event: ceil(nt / K) checkpoints of (36 N + 3 G) floats, K iteration slots of
 * (1876 E + 6 G) floats (1128 E + 6 G without attenuation: the displacement gradients, the
 * memory-variable sums, velocity and assembled forces of the iteration), the adjoint state
 * and 6 N + G doubles of gradient. With steps_per_subsegment = K2 (0 < K2 < K) a second
 * level: each segment of K iterations is recomputed once into checkpoints every K2
 * iterations and each sub-segment of K2 iterations from those (one more forward pass), so
 * K2 slots and ceil(K / K2) - 1 more checkpoints instead of K slots (for 64 x 64 x 32,
 * nt = 4000: one level, K = 91, needs about 226 GB; two levels, K = 364, K2 = 28, about
 * 100 GB).
 * ses3d_gpu_exact_set_field / get_field access the adjoint state (field ids as
 * ses3d_gpu_get_field, without MM_global): set before the backward run it is the adjoint of
 * the final state (zero by default); read after it, the adjoint of the initial state. */
int ses3d_gpu_exact_adjoint(ses3d_gpu *h, int steps_per_checkpoint, int steps_per_subsegment);
int ses3d_gpu_exact_set_seismogram_adjoint(ses3d_gpu *h, int event, const float *gx, const float *gy,
                                           const float *gz);
int ses3d_gpu_exact_backward(ses3d_gpu *h);
int ses3d_gpu_exact_gradient(ses3d_gpu *h, int which, double *out, int device);
int ses3d_gpu_exact_get_field(ses3d_gpu *h, int event, int field, float *out);
int ses3d_gpu_exact_set_field(ses3d_gpu *h, int event, int field, const float *in);

/* Lean stepping (off by default). Outside the PML
 * all profiles vanish, so (SOURCE/ses3d_evolution.f90:123-134,208-219) the displacement
 * gradients dxux..dzuy enter no output and the mirror stresses syx, szx, szy stay equal
 * to sxy, sxz, syz. With lean stepping, elements outside the PML read and write neither:
 * 96 of the 318 bytes the element kernel moves per GLL point there. Seismograms,
 * velocities, stresses and memory variables are unchanged bit for bit: the mirror
 * stresses are brought up to date before any field transfer and when lean stepping is
 * switched off. The displacement gradients outside the PML are not integrated, so once a
 * lean iteration has run, ses3d_gpu_get_field(SES3D_FIELD_DXUX..DZUY) returns
 * SES3D_E_STATE (for the rest of the run, or until that field is set) instead of values
 * the reference would not produce. begin_adjoint switches lean stepping off.
 * Handles with adjoint_flag 1 or 2 keep the displacement u = sum of dt v (3 G floats more per
 * event, in checkpoints too): lean record and kernel-correlation iterations take the
 * displacement gradients outside the PML as the strain-rate proxies of u (equal to their
 * time integral up to FP32 rounding of the summation order), so the forward run with
 * records and the adjoint run step lean as well; recomputes of checkpointed records replay
 * the forward run's choice. Such a run must start with zero displacement gradients (a run
 * from rest, or after begin_adjoint): stepping it lean after ses3d_gpu_set_field set one
 * returns SES3D_E_STATE. On such handles, and with the exact adjoint enabled, the choice
 * cannot change once stepping has started (SES3D_E_STATE); begin_adjoint starts a new run.
 * Every lean run assumes the mirror stresses outside the PML equal their partners, as they
 * do from rest. */
int ses3d_gpu_set_lean(ses3d_gpu *h, int enable);

/* Element-kernel block shape: elements per CTA (1, 2 or 4); 0 selects the default.
 * 1 is the persistent bulk-copy kernel (plain and lean forward iterations), 2 and 4 the
 * register-staged kernel. Simulation.autotune (ses3d_gb300/solver.py) searches it. */
int ses3d_gpu_set_block_elements(ses3d_gpu *h, int elements_per_cta);

/* Block shapes of the persistent element kernel and of the node kernel, selected at run
 * time (each is a separately compiled instance; results are bit-identical across shapes):
 * element_shape 0 .. ses3d_gpu_kernel_shape_count() - 1 =
 *   0: 5 resident CTAs per SM (102 registers), next item's copy issued at the measured point
 *   1: 4 CTAs per SM (128 registers)   2: 6 CTAs per SM (85 registers)
 *   3: 5 CTAs per SM, copy issued at the other point (after the stress phase in lean
 *      iterations, after the state read in full-state ones);
 * node_block: threads per node-kernel CTA, 128, 256 (default) or 512. Defaults 0, 256.
 * Simulation.autotune searches them per mesh and event count. No counterpart in the
 * reference. */
int ses3d_gpu_set_kernel_shape(ses3d_gpu *h, int element_shape, int node_block);
int ses3d_gpu_kernel_shape_count(void);

#ifdef __cplusplus
}
#endif
#endif /* SES3D_GPU_H */

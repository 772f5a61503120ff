// capi.cu -- implementation of the C ABI declared in include/ses3d_gpu.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/ses3d_gpu.h"
#include "kernels.cuh"
#include "setup.hpp"

namespace {
// NVTX range for the phases of a run (step, model set-up, checkpoint recompute, adjoint
// start): visible in Nsight timelines, free when no tool is attached.
struct Range {
  explicit Range(const char *name) { nvtxRangePushA(name); }
  ~Range() { nvtxRangePop(); }
};
}  // namespace

namespace ses3d {
cudaError_t launch_element(int diss, int mode, int epb, int shape, const Consts &c, const Ptrs &p, cudaStream_t st);
cudaError_t launch_node(int node_block, const Consts &c, const Ptrs &p, cudaStream_t st);
int element_shape_count();
cudaError_t launch_receivers(const Consts &c, const float *v, const int *rec_elem, const int *rec_ev,
                             const float *rec_w, float *seis, int R, const int *d_it, cudaStream_t st);
cudaError_t launch_inject(const Consts &c, float *f, const int4 *groups, int ngroups, const float *delta,
                          const float *stf, const int *mask, const int *d_it, cudaStream_t st);
cudaError_t launch_transpose(const float *in, float *out, long long rows, long long cols, cudaStream_t st);
cudaError_t launch_transpose_d(const double *in, double *out, long long rows, long long cols, bool accumulate,
                               cudaStream_t st);
cudaError_t launch_misfit_gradient(const double *K, const double *tables, int ex, int ey, int ez, double s,
                                   const void *div, void *out, bool f64, cudaStream_t st);
cudaError_t launch_derive_blocked(const float *const rec[7], float *mat, float *gm, long long E, int y0, int y1,
                                  int is_diss, float sum_D_p, int *aniso, cudaStream_t st);
cudaError_t launch_mass(const Consts &c, const float *rhoinv, const float *z, const float *sinx, const float *w,
                        float Jac, float *MM, float *iMM, cudaStream_t st);
cudaError_t launch_vmax(const float *v, long long G3, int nev, unsigned int *out, cudaStream_t st);
cudaError_t launch_grad_q_norm(const Consts &c, const float *gm, double *grad, cudaStream_t st);
cudaError_t launch_gather_ref(const Consts &c, const float *v, float *out, cudaStream_t st);
cudaError_t prepare_element_kernels();
cudaError_t prepare_adjoint_kernels();
cudaError_t launch_sync_mirrors(const Consts &c, float *state, cudaStream_t st);
cudaError_t launch_compact_state(const Consts &c, float *state, float *ck, const int *pml_el, long long npml, int to_ck,
                                 cudaStream_t st);
cudaError_t launch_wait_selftest(int *err, unsigned long long limit_ns, cudaStream_t st);
cudaError_t launch_sum_events_d(const double *grad, int slot, int nev, long long N, double *out, cudaStream_t st);
cudaError_t launch_state_field(float *state_ev, int field, float *ref, long long E, int to_ref, cudaStream_t st);
cudaError_t launch_adjoint_node1(const Consts &c, const Ptrs &p, const AdjPtrs &a, cudaStream_t st);
cudaError_t launch_adjoint_node2(const Consts &c, const AdjPtrs &a, cudaStream_t st);
cudaError_t launch_adjoint_element(int diss, const Consts &c, const Ptrs &p, const AdjPtrs &a, cudaStream_t st);
cudaError_t launch_adjoint_model_gradient(const Consts &c, const Ptrs &p, const double *gmat, const double *gimm,
                                          int which, int is_diss, double sD, const float *z, const float *sinx,
                                          const float *w, double *out, cudaStream_t st);
}  // namespace ses3d

using namespace ses3d;

namespace {
thread_local std::string g_create_error;

struct EventHost {
  int source_type = 0;
  PointSource src;
  std::vector<float> so;
  std::vector<Receiver> recs;
  std::vector<AdjointSource> adj;
  std::vector<float> adj_stf;  // [n_local][3][nt]
};

struct ForceSet {
  int4 *groups = nullptr;
  float *delta = nullptr, *stf = nullptr;
  int *mask = nullptr;
  int n = 0;
};

// The wavefield an iteration advances: the handle's own, or the recomputing forward run's.
struct Wave {
  float *state;
  float *v;
  int *d_it;
  bool adjoint;    // adjoint-run iteration: adjoint forces, no moment source
  bool receivers;  // record seismograms
};
}  // namespace

struct ses3d_gpu {
  ses3d_config cfg;
  Geometry geo;
  int device = 0;
  cudaStream_t st = nullptr;
  cudaStream_t st2 = nullptr;  // model set-up kernels beside the host-to-device copies
  std::string err;
  int it = 0;
  int mode_flag = 0;  // current adjoint_flag
  bool model_set = false;
  int epb = 1;
  int shape = 0;        // block shape of the persistent element kernel
  int node_block = 256;  // threads per CTA of the node kernel
  long long launches = 0;
  Consts c;
  // device memory
  KTab *d_ktab = nullptr;
  float *d_tab = nullptr;  // sin_x | cot_x | r_z | pxr | pyr | pzr | pxg | pyg | pzg | z | w
  float *d_MM = nullptr, *d_mat = nullptr, *d_gmat = nullptr;
  float *d_state = nullptr, *d_v = nullptr, *d_f = nullptr;
  bool state_zero = false;  // d_state holds zeros only (since zero_wavefield, before any step or field write)
  bool has_u = false;       // runs with records or kernel correlation (adjoint_flag 1, 2): d_v and d_v2
                            // hold the displacement [nev][3][G] after the velocity
  bool fwd_lean = false;    // the forward run with records stepped lean (its recomputes do too)
  bool du_set = false;      // displacement gradients were set since the wavefield was zeroed
  int *d_pml_el = nullptr;  // PML elements in ascending order (compact checkpoints of lean runs)
  long long n_pml_el = 0;
  int *d_aniso = nullptr;   // set by the model derivation when A, B or C is non-zero
  int *d_it = nullptr;
  int *d_err = nullptr;  // device error word (bounded waits)
  bool mirrors_stale = false;  // lean iterations left the mirror stresses outside the PML behind
  unsigned du_stale = 0;       // bit f: displacement gradient f (dxux..dzuy) not integrated outside the
                               // PML by lean iterations since the wavefield was last zeroed or set
  // allocation-free stepping over caller-owned wavefields (ses3d_gpu_step_external)
  bool external_stepped = false;     // this handle's time axis belongs to an external wavefield
  bool ext_mirrors_stale = false;    // the last external call stepped lean
  float *ext_forces = nullptr;       // device address of the fixed element-force array
  int *d_src_elem = nullptr;
  float *d_src_delta = nullptr, *d_src_mom = nullptr, *d_stf = nullptr;
  int *d_src_none = nullptr;  // all -1: no moment source (adjoint iterations)
  ForceSet fset[2];           // point forces of the forward (0) and the adjoint (1) runs
  int R = 0;
  int *d_rec_elem = nullptr, *d_rec_ev = nullptr;
  float *d_rec_w = nullptr, *d_seis = nullptr;
  std::vector<int> rec_off;  // [nev+1]
  double *d_grad = nullptr;
  unsigned int *d_scratch_u = nullptr;
  std::vector<float *> records;  // each [nev][NREC][N], inside record_blocks
  std::vector<float *> record_blocks;  // owned allocations holding the records
  std::vector<float *> record_slots;   // preallocated record places of a flag-1 run
  int record_cursor = 0;
  std::vector<int> store_steps;   // iterations whose forward fields are stored (1-based)
  int nrec_done = 0;              // records produced by the forward run so far
  // checkpointed storage: a full-state checkpoint before every ckpt_K-th record, records
  // recomputed segment by segment during the adjoint run
  int ckpt_K = 0;
  std::vector<float *> ckpts;     // each [nev][NSTATE N + 3 G]
  std::vector<int> ckpt_it;       // completed iterations at each checkpoint
  std::vector<float *> segbuf;    // the records of the recomputed (sub-)segment
  int seg_loaded = -1;
  // second level (ckpt_K2 > 0): a segment of ckpt_K records is recomputed once into
  // checkpoints before every ckpt_K2-th of its records, and each sub-segment of ckpt_K2
  // records is recomputed from those when the adjoint run reaches it
  int ckpt_K2 = 0;
  std::vector<float *> ckpt2;     // checkpoints of sub-segments 1.. of the loaded segment
  std::vector<int> ckpt2_it;
  int sub_loaded = -1;            // sub-segment of seg_loaded whose records are in segbuf
  // exact discrete adjoint (ses3d_gpu_exact_*): full-state checkpoints of the plain forward
  // run every ex_K iterations; the backward run recomputes one segment at a time into
  // per-iteration slots (state, velocity, assembled forces) and steps the adjoint through it
  int ex_K = 0;
  int ex_K2 = 0;                           // two levels: a segment is recomputed into checkpoints every ex_K2
  std::vector<float *> ex_ckpts;           // at completed iterations 0, ex_K, 2 ex_K, ...
  std::vector<float *> ex_ckpts2;          // second-level checkpoints of the segment being reversed
  std::vector<float *> ex_slots;
  std::vector<float *> ex_blocks;          // owned allocations holding ex_ckpts, ex_ckpts2, ex_slots
  size_t ex_block_floats = 0;
  float *d_astate = nullptr, *d_av = nullptr, *d_aF = nullptr, *d_af = nullptr;
  double *d_egmat = nullptr, *d_egimm = nullptr;
  int *d_ait = nullptr;
  std::vector<std::vector<float>> seis_adj;  // per event: d misfit / d seismogram, [3][nt][nr]
  ForceSet fseis;                            // the receivers' adjoint sources as point forces
  bool ex_done = false;
  bool ex_zero_d = true;  // the adjoint displacement gradients were not set (zero from the start)
  float *d_state2 = nullptr, *d_v2 = nullptr;  // wavefield of the recomputing forward run
  int *d_it2 = nullptr;
  std::vector<int> saving_vector;  // [nt+1]
  std::vector<EventHost> ev;
  // tables offsets
  size_t o_isin = 0, o_ir = 0;
  size_t o_sin = 0, o_cot = 0, o_r = 0, o_pxr = 0, o_pyr = 0, o_pzr = 0, o_pxg = 0, o_pyg = 0, o_pzg = 0, o_z = 0,
         o_w = 0;
  // per-kernel timing
  bool prof_on = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_pending;
  double prof_ms[4] = {0, 0, 0, 0};
  long long prof_n[4] = {0, 0, 0, 0};
  // graph
  bool graph_on = false;
  int graph_n = 0;
  int graph_len = 0;  // iterations in the captured graph
  cudaGraphExec_t graph_exec = nullptr;
  bool graph_dirty = true;
};

namespace {

int fail(ses3d_gpu *h, int code, const std::string &msg) {
  if (h) h->err = msg; else g_create_error = msg;
  return code;
}

int cuda_fail(ses3d_gpu *h, cudaError_t e, const char *where) {
  std::string m = std::string(where) + ": " + cudaGetErrorString(e);
  // a failed allocation also sets the runtime's last error; clear it so that the next
  // launch check (cudaGetLastError) does not report it again
  cudaGetLastError();
  return fail(h, e == cudaErrorMemoryAllocation ? SES3D_E_OOM : SES3D_E_CUDA, m);
}

#define CK(h, call)                                              \
  do {                                                           \
    cudaError_t _e = (call);                                     \
    if (_e != cudaSuccess) return cuda_fail((h), _e, #call);     \
  } while (0)

template <class T> cudaError_t dalloc(T **p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  return cudaMalloc((void **)p, count * sizeof(T));
}

void dfree(void *p) {
  if (p) cudaFree(p);
}

Ptrs make_ptrs(ses3d_gpu *h) {
  Ptrs p;
  std::memset(&p, 0, sizeof(p));
  p.ktab = h->d_ktab;
  p.sin_x = h->d_tab + h->o_sin; p.cot_x = h->d_tab + h->o_cot; p.r_z = h->d_tab + h->o_r;
  p.inv_sin = h->d_tab + h->o_isin; p.inv_r = h->d_tab + h->o_ir;
  p.pxr = h->d_tab + h->o_pxr; p.pyr = h->d_tab + h->o_pyr; p.pzr = h->d_tab + h->o_pzr;
  p.pxg = h->d_tab + h->o_pxg; p.pyg = h->d_tab + h->o_pyg; p.pzg = h->d_tab + h->o_pzg;
  p.MM = h->d_MM; p.iMM = h->d_MM + h->geo.G; p.mat = h->d_mat; p.gmat = h->d_gmat;
  p.state = h->d_state; p.v = h->d_v; p.f = h->d_f; p.d_it = h->d_it;
  p.src_elem = h->d_src_elem; p.src_delta = h->d_src_delta; p.src_mom = h->d_src_mom; p.stf = h->d_stf;
  p.grad = h->d_grad;
  p.grad_q = h->cfg.grad_variant == 1;
  p.err = h->d_err;
  return p;
}

void destroy_graph(ses3d_gpu *h) {
  if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
  h->graph_exec = nullptr;
  h->graph_dirty = true;
}

void free_forces(ForceSet &f) {
  dfree(f.groups); dfree(f.delta); dfree(f.stf); dfree(f.mask);
  f = ForceSet();
}

// Rebuild the point-force groups of all events: single forces of the forward run (set 0) and
// adjoint sources of the adjoint run (set 1). One group per (event, element); a group's
// sources keep file order.
int rebuild_forces(ses3d_gpu *h) {
  const int nt = h->cfg.nt;
  for (int which = 0; which < 2; ++which) {
    std::map<std::pair<int, long long>, std::vector<int>> groups;  // (event, element) -> sources
    std::vector<float> delta, stf;
    std::vector<int> mask;
    int ns = 0;
    for (int e = 0; e < h->cfg.n_events; ++e) {
      const EventHost &E = h->ev[e];
      const Geometry &g = h->geo;
      if (which == 0 && E.src.is_source && E.source_type >= 1 && E.source_type <= 3) {
        long long el = E.src.isx + (long long)g.ex * (E.src.isy + (long long)g.ey * E.src.isz);
        groups[{e, el}].push_back(ns++);
        delta.insert(delta.end(), E.src.delta, E.src.delta + NPE);
        for (int cc = 0; cc < 3; ++cc) {
          if (cc == E.source_type - 1) stf.insert(stf.end(), E.so.begin(), E.so.end());
          else stf.insert(stf.end(), (size_t)nt, 0.f);
        }
        mask.push_back(1 << (E.source_type - 1));
      }
      if (which == 1) {
        for (size_t s = 0; s < E.adj.size(); ++s) {
          const AdjointSource &A = E.adj[s];
          long long el = A.is[0] + (long long)g.ex * (A.is[1] + (long long)g.ey * A.is[2]);
          groups[{e, el}].push_back(ns++);
          delta.insert(delta.end(), A.delta, A.delta + NPE);
          stf.insert(stf.end(), E.adj_stf.begin() + s * 3 * nt, E.adj_stf.begin() + (s + 1) * 3 * nt);
          mask.push_back(7);
        }
      }
    }
    std::vector<int4> gr;
    std::vector<float> d2, s2;
    std::vector<int> m2;
    int k = 0;
    for (auto &kv : groups) {
      int4 g4;
      g4.x = kv.first.first; g4.y = (int)kv.first.second; g4.z = k;
      for (int s : kv.second) {
        d2.insert(d2.end(), delta.begin() + (size_t)s * NPE, delta.begin() + (size_t)(s + 1) * NPE);
        s2.insert(s2.end(), stf.begin() + (size_t)s * 3 * nt, stf.begin() + (size_t)(s + 1) * 3 * nt);
        m2.push_back(mask[s]);
        ++k;
      }
      g4.w = k;
      gr.push_back(g4);
    }
    ForceSet &F = h->fset[which];
    free_forces(F);
    F.n = (int)gr.size();
    if (F.n) {
      CK(h, dalloc(&F.groups, gr.size()));
      CK(h, dalloc(&F.delta, d2.size()));
      CK(h, dalloc(&F.stf, s2.size()));
      CK(h, dalloc(&F.mask, m2.size()));
      CK(h, cudaMemcpy(F.groups, gr.data(), gr.size() * sizeof(int4), cudaMemcpyHostToDevice));
      CK(h, cudaMemcpy(F.delta, d2.data(), d2.size() * sizeof(float), cudaMemcpyHostToDevice));
      CK(h, cudaMemcpy(F.stf, s2.data(), s2.size() * sizeof(float), cudaMemcpyHostToDevice));
      CK(h, cudaMemcpy(F.mask, m2.data(), m2.size() * sizeof(int), cudaMemcpyHostToDevice));
    }
  }
  destroy_graph(h);
  return SES3D_OK;
}

int upload_moment_sources(ses3d_gpu *h) {
  const int nev = h->cfg.n_events, nt = h->cfg.nt;
  std::vector<int> el(nev, -1);
  std::vector<float> delta((size_t)nev * NPE, 0.f), stf((size_t)nev * nt, 0.f);
  for (int e = 0; e < nev; ++e) {
    const EventHost &E = h->ev[e];
    if (E.src.is_source && E.source_type == 10) {
      el[e] = E.src.isx + h->geo.ex * (E.src.isy + h->geo.ey * E.src.isz);
      std::memcpy(&delta[(size_t)e * NPE], E.src.delta, NPE * sizeof(float));
    }
    if (!E.so.empty()) std::memcpy(&stf[(size_t)e * nt], E.so.data(), nt * sizeof(float));
  }
  CK(h, cudaMemcpy(h->d_src_elem, el.data(), nev * sizeof(int), cudaMemcpyHostToDevice));
  CK(h, cudaMemcpy(h->d_src_delta, delta.data(), delta.size() * sizeof(float), cudaMemcpyHostToDevice));
  CK(h, cudaMemcpy(h->d_stf, stf.data(), stf.size() * sizeof(float), cudaMemcpyHostToDevice));
  destroy_graph(h);
  return SES3D_OK;
}

// Transpose of an N-sized field: internal (E x 125) -> reference (125 x E).
int to_ref(ses3d_gpu *h, const float *d_int, float *d_ref) {
  CK(h, launch_transpose(d_int, d_ref, h->geo.E, NPE, h->st));
  return SES3D_OK;
}
int from_ref(ses3d_gpu *h, const float *d_ref, float *d_int) {
  CK(h, launch_transpose(d_ref, d_int, NPE, h->geo.E, h->st));
  return SES3D_OK;
}

int check_event(ses3d_gpu *h, int event) {
  if (!h) return SES3D_E_CONFIG;
  if (event < 0 || event >= h->cfg.n_events) return fail(h, SES3D_E_CONFIG, "event index out of range");
  return SES3D_OK;
}

// Launches the model set-up for node tiles y0 .. y1 - 1 of the derivation (4 tiles cover
// every node) and, with mass, the mass matrix; rec: the 7 model records on the device.
static cudaError_t model_kernels(ses3d_gpu *h, const float *const rec[7], int y0, int y1, bool mass, cudaStream_t st) {
  float sum_D_p = h->cfg.D_p[0];
  sum_D_p = sum_D_p + h->cfg.D_p[1];
  sum_D_p = sum_D_p + h->cfg.D_p[2];
  cudaError_t e = cudaSuccess;
  if (mass) {
    e = launch_mass(h->c, rec[0], h->d_tab + h->o_z, h->d_tab + h->o_sin, h->d_tab + h->o_w, h->geo.Jac, h->d_MM,
                    h->d_MM + h->geo.G, st);
    ++h->launches;
  }
  if (e == cudaSuccess && y1 > y0) {
    e = launch_derive_blocked(rec, h->d_mat, h->d_gmat, h->geo.E, y0, y1, h->cfg.is_diss, sum_D_p, h->d_aniso, st);
    ++h->launches;
  }
  return e;
}

// After the model kernels completed: isotropic models (A, B, C all zero) let the element
// kernels read three of the six material fields. Kernel parameters captured in a CUDA
// graph hold the old setting, so a change drops the graph.
static cudaError_t note_isotropy(ses3d_gpu *h) {
  int aniso = 1;
  cudaError_t e = cudaMemcpy(&aniso, h->d_aniso, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return e;
  const int iso = aniso ? 0 : 1;
  if (iso != h->c.iso) {
    h->c.iso = iso;
    destroy_graph(h);
  }
  return cudaSuccess;
}

// Model set-up from 7 records already on the device (reference layout), on the handle's stream.
int set_model_common(ses3d_gpu *h, const float *const rec[7]) {
  cudaError_t e = cudaMemsetAsync(h->d_aniso, 0, sizeof(int), h->st);
  if (e == cudaSuccess) e = model_kernels(h, rec, 0, 4, true, h->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
  if (e == cudaSuccess) e = note_isotropy(h);
  if (e != cudaSuccess) return cuda_fail(h, e, "set_model");
  h->model_set = true;
  return SES3D_OK;
}

// Floats of the velocity allocation: the velocity of every event, and the displacement after
// it on handles that keep one.
size_t v_floats(const ses3d_gpu *h) {
  return (size_t)h->cfg.n_events * 3 * (size_t)h->geo.G * (h->has_u ? 2 : 1);
}

int zero_wavefield(ses3d_gpu *h) {
  const size_t nev = h->cfg.n_events;
  CK(h, cudaMemsetAsync(h->d_state, 0, nev * NSTATE * h->geo.N * sizeof(float), h->st));
  CK(h, cudaMemsetAsync(h->d_v, 0, v_floats(h) * sizeof(float), h->st));
  CK(h, cudaMemsetAsync(h->d_f, 0, nev * 3 * h->geo.N * sizeof(float), h->st));
  CK(h, cudaMemsetAsync(h->d_it, 0, sizeof(int), h->st));
  if (h->d_seis) CK(h, cudaMemsetAsync(h->d_seis, 0, (size_t)3 * h->cfg.nt * h->R * sizeof(float), h->st));
  h->mirrors_stale = false;
  h->du_stale = 0;
  h->it = 0;
  h->state_zero = true;
  h->du_set = false;
  return SES3D_OK;
}

cudaEvent_t pool_event(ses3d_gpu *h) {
  if (!h->ev_pool.empty()) {
    cudaEvent_t e = h->ev_pool.back();
    h->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// Adds the durations of completed timed launches (the stream has been synchronised).
void collect_times(ses3d_gpu *h) {
  for (auto &pe : h->ev_pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, pe.second.first, pe.second.second) == cudaSuccess) {
      h->prof_ms[pe.first] += ms;
      h->prof_n[pe.first] += 1;
    }
    h->ev_pool.push_back(pe.second.first);
    h->ev_pool.push_back(pe.second.second);
  }
  h->ev_pending.clear();
}

struct Timed {
  ses3d_gpu *h;
  int which;
  cudaEvent_t a = nullptr, b = nullptr;
  Timed(ses3d_gpu *h_, int w, bool on) : h(h_), which(w) {
    if (on) { a = pool_event(h); b = pool_event(h); cudaEventRecord(a, h->st); }
  }
  ~Timed() {
    if (a) { cudaEventRecord(b, h->st); h->ev_pending.push_back({which, {a, b}}); }
  }
};

Wave primary_wave(ses3d_gpu *h) {
  return Wave{h->d_state, h->d_v, h->d_it, h->mode_flag == 2, h->mode_flag <= 1};
}

// one iteration of a wavefield: receivers, element, inject, node (+ record / kernel work)
// fg: also store the assembled forces there; slot: also pack the iteration's starting state
// there for the exact adjoint (plain iterations only).
int launch_iteration(ses3d_gpu *h, const Wave &w, int mode, float *rec, bool timed = false, float *fg = nullptr,
                     float *slot = nullptr) {
  Ptrs p = make_ptrs(h);
  p.fg = fg;
  p.slot = slot;
  h->state_zero = false;
  p.state = w.state;
  p.v = w.v;
  // the displacement is integrated in lean runs, the only ones that read it (the stepping of
  // a run with records is fixed for the run, so u covers every iteration since its start)
  p.u = (h->has_u && h->c.lean) ? w.v + (size_t)h->cfg.n_events * 3 * h->geo.G : nullptr;
  p.d_it = w.d_it;
  p.rec = rec;
  p.src_elem = w.adjoint ? h->d_src_none : h->d_src_elem;
  const ForceSet &F = h->fset[w.adjoint ? 1 : 0];
  if (w.receivers && h->R > 0) {
    Timed t(h, 2, timed);
    CK(h, launch_receivers(h->c, w.v, h->d_rec_elem, h->d_rec_ev, h->d_rec_w, h->d_seis, h->R, w.d_it, h->st));
    ++h->launches;
  }
  {
    Timed t(h, 0, timed);
    CK(h, launch_element(h->cfg.is_diss, mode, h->epb, h->shape, h->c, p, h->st));
    ++h->launches;
  }
  if (F.n) {
    Timed t(h, 3, timed);
    CK(h, launch_inject(h->c, h->d_f, F.groups, F.n, F.delta, F.stf, F.mask, w.d_it, h->st));
    ++h->launches;
  }
  {
    Timed t(h, 1, timed);
    CK(h, launch_node(h->node_block, h->c, p, h->st));
    ++h->launches;
  }
  return SES3D_OK;
}

// Floats of one full-state checkpoint (all events): element state, assembled velocity and,
// where kept, the displacement.
size_t ckpt_floats(const ses3d_gpu *h) {
  return (size_t)h->cfg.n_events * (size_t)NSTATE * h->geo.N + v_floats(h);
}

// Element-state floats of a compact checkpoint (lean runs): 24 fields of every element and
// the other 12 of the PML elements, all events.
size_t compact_state_floats(const ses3d_gpu *h) {
  return (size_t)h->cfg.n_events * 125 * (24 * (size_t)h->geo.E + 12 * (size_t)h->n_pml_el);
}

// Floats of one record checkpoint: compact when the forward run with records steps lean
// (its recomputes read no other fields), else the full state.
size_t rec_ckpt_floats(const ses3d_gpu *h) {
  return h->fwd_lean ? compact_state_floats(h) + v_floats(h) : ckpt_floats(h);
}

// A wavefield (element state, velocity and displacement) into a checkpoint, or back.
int wave_to_ckpt(ses3d_gpu *h, float *state, float *v, float *ck, bool compact, bool to_ck) {
  const size_t ns = compact ? compact_state_floats(h) : (size_t)h->cfg.n_events * NSTATE * h->geo.N;
  if (compact) {
    CK(h, launch_compact_state(h->c, state, ck, h->d_pml_el, h->n_pml_el, to_ck ? 1 : 0, h->st));
    ++h->launches;
  } else if (to_ck) {
    CK(h, cudaMemcpyAsync(ck, state, ns * sizeof(float), cudaMemcpyDeviceToDevice, h->st));
  } else {
    CK(h, cudaMemcpyAsync(state, ck, ns * sizeof(float), cudaMemcpyDeviceToDevice, h->st));
  }
  if (to_ck) CK(h, cudaMemcpyAsync(ck + ns, v, v_floats(h) * sizeof(float), cudaMemcpyDeviceToDevice, h->st));
  else CK(h, cudaMemcpyAsync(v, ck + ns, v_floats(h) * sizeof(float), cudaMemcpyDeviceToDevice, h->st));
  return SES3D_OK;
}

int save_checkpoint(ses3d_gpu *h, int completed_it) {
  Range range_("ses3d checkpoint");
  float *c = nullptr;
  CK(h, dalloc(&c, rec_ckpt_floats(h)));
  h->ckpts.push_back(c);
  h->ckpt_it.push_back(completed_it);
  return wave_to_ckpt(h, h->d_state, h->d_v, c, h->fwd_lean, true);
}

// Grows `views` to `count` buffers of `floats` each (rounded up to 256 bytes), carved from
// one new allocation: a few large allocations instead of one per buffer.
int grow_exact_buffers(ses3d_gpu *h, std::vector<float *> &views, size_t count, size_t floats) {
  if (views.size() >= count) return SES3D_OK;
  const size_t stride = (floats + 63) & ~(size_t)63;
  const size_t add = count - views.size();
  float *block = nullptr;
  CK(h, dalloc(&block, add * stride));
  h->ex_blocks.push_back(block);
  h->ex_block_floats += add * stride;
  for (size_t q = 0; q < add; ++q) views.push_back(block + q * stride);
  return SES3D_OK;
}

// Full-state checkpoint of the primary wavefield for the exact adjoint (completed
// iterations = 0, ex_K, 2 ex_K, ...); kept for the whole run.
int save_exact_checkpoint(ses3d_gpu *h, int completed_it) {
  const int idx = completed_it / h->ex_K;
  const size_t ns = (size_t)h->cfg.n_events * NSTATE * h->geo.N;
  const size_t nv = (size_t)h->cfg.n_events * 3 * h->geo.G;
  const size_t nseg = ((size_t)h->cfg.nt + h->ex_K - 1) / h->ex_K;
  int rc = grow_exact_buffers(h, h->ex_ckpts, std::max(nseg, (size_t)idx + 1), ckpt_floats(h));
  if (rc) return rc;
  CK(h, cudaMemcpyAsync(h->ex_ckpts[idx], h->d_state, ns * sizeof(float), cudaMemcpyDeviceToDevice, h->st));
  CK(h, cudaMemcpyAsync(h->ex_ckpts[idx] + ns, h->d_v, nv * sizeof(float), cudaMemcpyDeviceToDevice, h->st));
  return SES3D_OK;
}

// The second wavefield (the recomputing forward run), allocated on first use.
int ensure_wave2(ses3d_gpu *h) {
  if (h->d_state2) return SES3D_OK;
  CK(h, dalloc(&h->d_state2, (size_t)h->cfg.n_events * NSTATE * h->geo.N));
  CK(h, dalloc(&h->d_v2, v_floats(h)));
  CK(h, dalloc(&h->d_it2, 1));
  return SES3D_OK;
}

// Loads a checkpoint (completed iterations it0; compact: a lean run's) into the second
// wavefield.
int load_wave2(ses3d_gpu *h, const float *ckpt, const int &it0, bool compact = false) {
  int rc = ensure_wave2(h);
  if (rc) return rc;
  rc = wave_to_ckpt(h, h->d_state2, h->d_v2, const_cast<float *>(ckpt), compact, false);
  if (rc) return rc;
  CK(h, cudaMemcpyAsync(h->d_it2, &it0, sizeof(int), cudaMemcpyHostToDevice, h->st));
  return SES3D_OK;
}

// Recomputes of the forward run step as it did (lean or full state) while this is in scope.
struct ForwardStepping {
  ses3d_gpu *h;
  int saved;
  explicit ForwardStepping(ses3d_gpu *hh) : h(hh), saved(hh->c.lean) { h->c.lean = h->fwd_lean ? 1 : 0; }
  ~ForwardStepping() { h->c.lean = saved; }
};

// Runs the second wavefield from completed iteration it0 and stores records rA .. rB - 1
// into segbuf[0 ..] (record iterations in MODE 1, the others plain).
int recompute_records(ses3d_gpu *h, int it0, int rA, int rB) {
  ForwardStepping fs(h);
  const size_t rec_floats = (size_t)h->cfg.n_events * NREC * h->geo.N;
  if (!h->d_state2) return fail(h, SES3D_E_STATE, "the recomputing wavefield is not loaded");
  while ((int)h->segbuf.size() < rB - rA) {
    float *r = nullptr;
    CK(h, dalloc(&r, rec_floats));
    h->segbuf.push_back(r);
  }
  Wave w{h->d_state2, h->d_v2, h->d_it2, false, false};
  int r = rA;
  for (int it = it0 + 1; r < rB; ++it) {
    float *rec = nullptr;
    int mode = 0;
    if (it == h->store_steps[r]) {
      rec = h->segbuf[r - rA];
      mode = 1;
      ++r;
    }
    int rc = launch_iteration(h, w, mode, rec);
    if (rc) return rc;
  }
  return SES3D_OK;
}

// One level: recomputes the records of segment s (records s K .. min((s+1) K, nrec) - 1)
// into segbuf by a forward run from checkpoint s on the second wavefield.
int recompute_segment(ses3d_gpu *h, int s) {
  Range range_("ses3d recompute segment");
  int rc = load_wave2(h, h->ckpts[s], h->ckpt_it[s], h->fwd_lean);
  if (rc) return rc;
  const int r0 = s * h->ckpt_K;
  const int r1 = std::min((int)h->store_steps.size(), r0 + h->ckpt_K);
  rc = recompute_records(h, h->ckpt_it[s], r0, r1);
  if (rc) return rc;
  h->seg_loaded = s;
  return SES3D_OK;
}

// Two levels, first pass: runs segment s forward from its checkpoint and keeps a full-state
// checkpoint before the first record of each of its sub-segments 1, 2, ... (sub-segment 0
// starts at the segment's own checkpoint).
int recompute_level2(ses3d_gpu *h, int s) {
  Range range_("ses3d recompute checkpoints");
  ForwardStepping fs(h);
  const int r0 = s * h->ckpt_K;
  const int r1 = std::min((int)h->store_steps.size(), r0 + h->ckpt_K);
  const int nsub = (r1 - r0 + h->ckpt_K2 - 1) / h->ckpt_K2;
  while ((int)h->ckpt2.size() < nsub - 1) {
    float *c = nullptr;
    CK(h, dalloc(&c, rec_ckpt_floats(h)));
    h->ckpt2.push_back(c);
  }
  h->ckpt2_it.assign(std::max(0, nsub - 1), 0);
  int rc = load_wave2(h, h->ckpts[s], h->ckpt_it[s], h->fwd_lean);
  if (rc) return rc;
  Wave w{h->d_state2, h->d_v2, h->d_it2, false, false};
  int it = h->ckpt_it[s];
  for (int j = 1; j < nsub; ++j) {
    const int target = h->store_steps[r0 + j * h->ckpt_K2] - 1;  // completed iterations at the checkpoint
    for (; it < target; ++it) {
      rc = launch_iteration(h, w, 0, nullptr);
      if (rc) return rc;
    }
    rc = wave_to_ckpt(h, h->d_state2, h->d_v2, h->ckpt2[j - 1], h->fwd_lean, true);
    if (rc) return rc;
    h->ckpt2_it[j - 1] = target;
  }
  h->seg_loaded = s;
  h->sub_loaded = -1;
  return SES3D_OK;
}

// The forward record r for the adjoint run, recomputed as the checkpointing asks.
int checkpointed_record(ses3d_gpu *h, int r, float **out) {
  const int s = r / h->ckpt_K;
  if (s >= (int)h->ckpts.size()) return fail(h, SES3D_E_STATE, "no checkpoint for this record");
  if (h->ckpt_K2 <= 0) {
    if (h->seg_loaded != s) {
      int rc = recompute_segment(h, s);
      if (rc) return rc;
    }
    *out = h->segbuf[r - s * h->ckpt_K];
    return SES3D_OK;
  }
  if (h->seg_loaded != s) {
    int rc = recompute_level2(h, s);
    if (rc) return rc;
  }
  const int r0 = s * h->ckpt_K;
  const int j = (r - r0) / h->ckpt_K2;
  if (h->sub_loaded != j) {
    Range range_("ses3d recompute segment");
    const int rA = r0 + j * h->ckpt_K2;
    const int rB = std::min({(int)h->store_steps.size(), r0 + h->ckpt_K, rA + h->ckpt_K2});
    const float *src = j == 0 ? h->ckpts[s] : h->ckpt2[j - 1];
    const int it0 = j == 0 ? h->ckpt_it[s] : h->ckpt2_it[j - 1];
    int rc = load_wave2(h, src, it0, h->fwd_lean);
    if (!rc) rc = recompute_records(h, it0, rA, rB);
    if (rc) return rc;
    h->sub_loaded = j;
  }
  *out = h->segbuf[r - r0 - j * h->ckpt_K2];
  return SES3D_OK;
}

// Captures `len` plain iterations of the primary wavefield as one CUDA graph.
int build_graph(ses3d_gpu *h, int len) {
  Range range_("ses3d graph capture");
  destroy_graph(h);
  cudaGraph_t graph;
  CK(h, cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
  long long before = h->launches;
  for (int s = 0; s < len; ++s) {
    int rc = launch_iteration(h, primary_wave(h), 0, nullptr);
    if (rc) {
      cudaStreamEndCapture(h->st, &graph);
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
  }
  h->launches = before;  // counted at replay
  CK(h, cudaStreamEndCapture(h->st, &graph));
  cudaError_t e = cudaGraphInstantiate(&h->graph_exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaGraphInstantiate");
  h->graph_dirty = false;
  h->graph_len = len;
  return SES3D_OK;
}

// Iteration `it` of a flag-1 run stores a forward record (ses3d_main.f90:144), of a flag-2
// run correlates one (ses3d_main.f90:168); every other iteration is plain.
bool special_iteration(const ses3d_gpu *h, int it) {
  const int nt = h->cfg.nt;
  if (h->mode_flag == 0) return h->ex_K > 0 && (it - 1) % h->ex_K == 0;  // exact-adjoint checkpoint
  if (h->mode_flag == 1) return it % h->cfg.samp_ad == 0 || it == 1 || it == nt;
  if (h->mode_flag == 2) return h->saving_vector[nt + 1 - it] > 0 && h->record_cursor > 0;
  return false;
}

int launches_per_iteration(ses3d_gpu *h) {
  int n = 2;
  if ((h->mode_flag == 0 || h->mode_flag == 1) && h->R > 0) ++n;
  if (h->fset[h->mode_flag == 2 ? 1 : 0].n) ++n;
  return n;
}

}  // namespace

extern "C" {

const char *ses3d_gpu_version(void) { return "ses3d_gb300 0.1 (sm_103a)"; }

int ses3d_gpu_select_device(int device) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return fail(nullptr, SES3D_E_NODEV, "no CUDA device");
  }
  if (device < 0 || device >= ndev) return fail(nullptr, SES3D_E_CONFIG, "device index out of range");
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaSetDevice");
  return SES3D_OK;
}

const char *ses3d_gpu_last_error(const ses3d_gpu *h) { return h ? h->err.c_str() : g_create_error.c_str(); }

int ses3d_gpu_create(const ses3d_config *cfg, ses3d_gpu **out) {
  if (!cfg || !out) return fail(nullptr, SES3D_E_CONFIG, "null argument");
  *out = nullptr;
  if (cfg->lpd != LPD) return fail(nullptr, SES3D_E_CONFIG, "only lpd = 4 is implemented");
  if (cfg->n_events < 1) return fail(nullptr, SES3D_E_CONFIG, "n_events must be >= 1");
  if (cfg->nt < 1) return fail(nullptr, SES3D_E_CONFIG, "nt must be >= 1");
  if (!(cfg->dt > 0.f)) return fail(nullptr, SES3D_E_CONFIG, "dt must be > 0");
  if (cfg->adjoint_flag < 0 || cfg->adjoint_flag > 2) return fail(nullptr, SES3D_E_CONFIG, "adjoint_flag must be 0, 1 or 2");
  if (cfg->adjoint_flag >= 1 && cfg->samp_ad < 1) return fail(nullptr, SES3D_E_CONFIG, "samp_ad must be >= 1");
  if (cfg->is_diss != 0 && cfg->is_diss != 1) return fail(nullptr, SES3D_E_CONFIG, "is_diss must be 0 or 1");
  if (cfg->is_diss == 1)
    for (int k = 0; k < 3; ++k)
      if (!(cfg->tau_p[k] > 0.f)) return fail(nullptr, SES3D_E_CONFIG, "relaxation times must be > 0");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return fail(nullptr, SES3D_E_NODEV, "no CUDA device");
  ses3d_gpu *h = new ses3d_gpu();
  h->cfg = *cfg;
  h->mode_flag = cfg->adjoint_flag;
  cudaGetDevice(&h->device);
  std::string msg = build_geometry(h->geo, cfg->nx, cfg->ny, cfg->nz, cfg->pml, cfg->xmin, cfg->xmax, cfg->ymin,
                                   cfg->ymax, cfg->zmin, cfg->zmax, cfg->zmax_global);
  if (!msg.empty()) { delete h; return fail(nullptr, SES3D_E_CONFIG, msg); }
  const Geometry &g = h->geo;
  if (g.N * (long long)cfg->n_events > (1LL << 40) || 3 * g.N >= (1LL << 32) || g.E >= (1LL << 31)) {
    delete h;
    return fail(nullptr, SES3D_E_CONFIG, "mesh too large");
  }
  // constants
  Consts &c = h->c;
  std::memset(&c, 0, sizeof(c));
  c.ex = g.ex; c.ey = g.ey; c.ez = g.ez; c.nev = cfg->n_events; c.nt = cfg->nt;
  c.GX = g.GX; c.GY = g.GY; c.GZ = g.GZ; c.E = g.E; c.N = g.N; c.G = g.G;
  c.dt = cfg->dt;
  for (int k = 0; k < 3; ++k) {
    c.tau_p[k] = cfg->tau_p[k]; c.D_p[k] = cfg->D_p[k];
    if (cfg->is_diss) {
      c.a_k[k] = cfg->dt / cfg->tau_p[k];
      c.L_k[k] = cfg->dt * cfg->D_p[k] / cfg->tau_p[k];
    }
    const float dPdalpha[3] = {-3.06f, -1.54f, 2.56f};  // ses3d_grad_Q.f90:30-32
    c.q_alpha_w[k] = cfg->D_p[k] != 0.f ? dPdalpha[k] * cfg->tau_p[k] / cfg->D_p[k] : 0.f;
  }
  c.s_grad = (float)cfg->samp_ad * cfg->dt;
  c.pml = cfg->pml;
  c.lean = 0;
  {  // magic multiplier for t / GX in k_node: l = ceil(log2 GX), m = floor(2^32 (2^l - GX) / GX) + 1
    const unsigned long long d = (unsigned long long)g.GX;
    int l = 0;
    while ((1ull << l) < d) ++l;
    c.gx_magic = (unsigned)((((1ull << 32) * ((1ull << l) - d)) / d + 1) & 0xffffffffull);
    c.gx_shift = l - 1;
  }
  c.Jac = g.Jac;
  c.s_jac = (double)c.s_grad / (double)g.Jac;
  // coefficient tables
  KTab kt;
  for (int i = 0; i < NP; ++i)
    for (int q = 0; q < NP; ++q) {
      kt.Dx[i][q] = 2.0f * g.dl[q][i] / g.dx;
      kt.Dy[i][q] = 2.0f * g.dl[q][i] / g.dy;
      kt.Dz[i][q] = 2.0f * g.dl[q][i] / g.dz;
      kt.dlT[i][q] = g.dl[i][q];
    }
  for (int a = 0; a < NP; ++a)
    for (int b = 0; b < NP; ++b) {
      kt.CX[a][b] = (2.0f / g.dx) * g.Jac * g.w[a] * g.w[b];
      kt.CY[a][b] = (2.0f / g.dy) * g.Jac * g.w[a] * g.w[b];
      kt.CZ[a][b] = -((2.0f / g.dz) * g.Jac * g.w[a] * g.w[b]);
    }
  for (int n = 0; n < NP; ++n) kt.w[n] = g.w[n];
  // table block
  std::vector<float> tab;
  auto put = [&](size_t &off, const std::vector<float> &v) { off = tab.size(); tab.insert(tab.end(), v.begin(), v.end()); };
  put(h->o_sin, g.sin_x); put(h->o_cot, g.cot_x); put(h->o_r, g.z);
  put(h->o_pxr, g.pxr); put(h->o_pyr, g.pyr); put(h->o_pzr, g.pzr);
  put(h->o_pxg, g.pxg); put(h->o_pyg, g.pyg); put(h->o_pzg, g.pzg);
  put(h->o_z, g.z);
  put(h->o_w, std::vector<float>(g.w, g.w + NP));
  std::vector<float> isin(g.sin_x.size()), ir(g.z.size());
  for (size_t q = 0; q < isin.size(); ++q) isin[q] = 1.0f / g.sin_x[q];
  for (size_t q = 0; q < ir.size(); ++q) ir[q] = 1.0f / g.z[q];
  put(h->o_isin, isin);
  put(h->o_ir, ir);
  const size_t nev = cfg->n_events;
  cudaError_t e = cudaSuccess;
  auto chk = [&](cudaError_t x) { if (x != cudaSuccess && e == cudaSuccess) e = x; };
  chk(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
  chk(cudaStreamCreateWithFlags(&h->st2, cudaStreamNonBlocking));
  chk(dalloc(&h->d_ktab, 1));
  chk(dalloc(&h->d_tab, tab.size()));
  chk(dalloc(&h->d_MM, (size_t)2 * g.G));  // MM_global and its reciprocal
  chk(dalloc(&h->d_mat, (size_t)ELEM_MAT * g.E));
  chk(dalloc(&h->d_err, 1));
  chk(dalloc(&h->d_aniso, 1));
  {  // PML elements (pml elements on the x and y sides and at the bottom), ascending
    std::vector<int> pel;
    for (int k = 0; k < g.ez; ++k)
      for (int j = 0; j < g.ey; ++j)
        for (int i = 0; i < g.ex; ++i)
          if (i < cfg->pml || i >= g.ex - cfg->pml || j < cfg->pml || j >= g.ey - cfg->pml || k >= g.ez - cfg->pml)
            pel.push_back(i + g.ex * (j + g.ey * k));
    h->n_pml_el = (long long)pel.size();
    if (!pel.empty()) {
      chk(dalloc(&h->d_pml_el, pel.size()));
      if (e == cudaSuccess) chk(cudaMemcpy(h->d_pml_el, pel.data(), pel.size() * sizeof(int), cudaMemcpyHostToDevice));
    }
  }
  chk(dalloc(&h->d_gmat, (size_t)NGMAT * g.N));
  chk(dalloc(&h->d_state, nev * NSTATE * g.N));
  h->has_u = cfg->adjoint_flag >= 1;
  chk(dalloc(&h->d_v, v_floats(h)));
  chk(dalloc(&h->d_f, nev * 3 * g.N));
  chk(dalloc(&h->d_it, 1));
  chk(dalloc(&h->d_src_elem, nev));
  chk(dalloc(&h->d_src_none, nev));
  chk(dalloc(&h->d_src_delta, nev * NPE));
  chk(dalloc(&h->d_src_mom, nev * 6));
  chk(dalloc(&h->d_stf, nev * cfg->nt));
  chk(dalloc(&h->d_scratch_u, nev));
  if (cfg->adjoint_flag == 2) chk(dalloc(&h->d_grad, nev * NGRAD * g.N));
  if (e != cudaSuccess) {
    std::string m = std::string("allocation: ") + cudaGetErrorString(e);
    cudaGetLastError();  // clear the failed allocation's last error
    ses3d_gpu_destroy(h);
    return fail(nullptr, e == cudaErrorMemoryAllocation ? SES3D_E_OOM : SES3D_E_CUDA, m);
  }
  // zero the wavefield first: the memsets run on the handle's stream while the tables below
  // are uploaded and the kernels prepared
  if (int rc0 = zero_wavefield(h)) {
    std::string m = h->err;
    ses3d_gpu_destroy(h);
    return fail(nullptr, rc0, m);
  }
  chk(cudaMemcpy(h->d_ktab, &kt, sizeof(KTab), cudaMemcpyHostToDevice));
  chk(cudaMemcpy(h->d_tab, tab.data(), tab.size() * sizeof(float), cudaMemcpyHostToDevice));
  std::vector<int> minus1(nev, -1);
  chk(cudaMemcpy(h->d_src_elem, minus1.data(), nev * sizeof(int), cudaMemcpyHostToDevice));
  chk(cudaMemcpy(h->d_src_none, minus1.data(), nev * sizeof(int), cudaMemcpyHostToDevice));
  chk(cudaMemset(h->d_src_delta, 0, nev * NPE * sizeof(float)));
  chk(cudaMemset(h->d_src_mom, 0, nev * 6 * sizeof(float)));
  chk(cudaMemset(h->d_stf, 0, nev * cfg->nt * sizeof(float)));
  chk(cudaMemset(h->d_MM, 0, (size_t)2 * g.G * sizeof(float)));
  chk(cudaMemset(h->d_err, 0, sizeof(int)));
  if (e == cudaSuccess) e = prepare_element_kernels();
  if (e == cudaSuccess) e = prepare_adjoint_kernels();
  if (h->d_grad) chk(cudaMemset(h->d_grad, 0, nev * NGRAD * g.N * sizeof(double)));
  if (e != cudaSuccess) {
    std::string m = std::string("initialisation: ") + cudaGetErrorString(e);
    ses3d_gpu_destroy(h);
    return fail(nullptr, SES3D_E_CUDA, m);
  }
  h->ev.resize(nev);
  h->rec_off.assign(nev + 1, 0);
  h->saving_vector.assign(cfg->nt + 2, 0);
  for (int it = 1; it <= cfg->nt; ++it)  // stored iterations of a flag-1 run (ses3d_main.f90:144)
    if (cfg->samp_ad > 0 && (it % cfg->samp_ad == 0 || it == 1 || it == cfg->nt)) h->store_steps.push_back(it);
  e = cudaStreamSynchronize(h->st);
  if (e != cudaSuccess) {
    std::string m = std::string("initialisation: ") + cudaGetErrorString(e);
    ses3d_gpu_destroy(h);
    return fail(nullptr, SES3D_E_CUDA, m);
  }
  *out = h;
  return SES3D_OK;
}

int ses3d_gpu_destroy(ses3d_gpu *h) {
  if (!h) return SES3D_OK;
  if (h->st) cudaStreamSynchronize(h->st);
  destroy_graph(h);
  for (auto &pe : h->ev_pending) { h->ev_pool.push_back(pe.second.first); h->ev_pool.push_back(pe.second.second); }
  for (cudaEvent_t e : h->ev_pool) cudaEventDestroy(e);
  void *ptrs[] = {h->d_ktab, h->d_tab, h->d_MM, h->d_mat, h->d_gmat, h->d_state, h->d_v, h->d_f, h->d_it,
                  h->d_src_elem, h->d_src_delta, h->d_src_mom, h->d_stf, h->d_src_none, h->d_rec_elem,
                  h->d_rec_ev, h->d_rec_w, h->d_seis, h->d_grad, h->d_scratch_u, h->d_state2, h->d_v2, h->d_it2, h->d_err,
                  h->d_aniso, h->d_pml_el};
  for (void *p : ptrs) dfree(p);
  free_forces(h->fset[0]);
  free_forces(h->fset[1]);
  for (float *r : h->record_blocks) dfree(r);
  for (float *r : h->ckpts) dfree(r);
  for (float *r : h->segbuf) dfree(r);
  for (float *r : h->ckpt2) dfree(r);
  for (float *r : h->ex_blocks) dfree(r);
  free_forces(h->fseis);
  {
    void *ex[] = {h->d_astate, h->d_av, h->d_aF, h->d_af, h->d_egmat, h->d_egimm, h->d_ait};
    for (void *q : ex) dfree(q);
  }
  if (h->st) cudaStreamDestroy(h->st);
  if (h->st2) cudaStreamDestroy(h->st2);
  delete h;
  return SES3D_OK;
}

int ses3d_gpu_set_model(ses3d_gpu *h, const float *rhoinv, const float *mu, const float *lambda, const float *A,
                        const float *B, const float *C, const float *Q) {
  Range range_("ses3d set model");
  if (!h) return SES3D_E_CONFIG;
  if (!rhoinv || !mu || !lambda || !A || !B || !C) return fail(h, SES3D_E_CONFIG, "null model array");
  if (h->cfg.is_diss && !Q) return fail(h, SES3D_E_CONFIG, "Q is required when is_diss = 1");
  const long long N = h->geo.N, E = h->geo.E;
  const int nrec = h->cfg.is_diss ? 7 : 6;
  // Staging for the records: the element state while it holds zeros only (a handle that has
  // not stepped; at least 36 N floats), zeroed again afterwards; else a buffer of its own.
  const bool in_state = h->state_zero;
  float *d_raw = in_state ? h->d_state : nullptr;
  if (!in_state) CK(h, dalloc(&d_raw, (size_t)nrec * N));
  const float *src[7] = {rhoinv, mu, lambda, A, B, C, Q};
  const float *rec[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  for (int k = 0; k < nrec; ++k) rec[k] = d_raw + (size_t)k * N;
  // The copies run on the handle's stream: rhoinv first, then the other records in four node
  // ranges (32 nodes of every element each, E floats per node). The set-up kernels run on
  // the second stream behind them: the mass matrix once rhoinv has arrived, each node
  // range's derivation once its records have, overlapping the copies still in flight.
  cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  cudaError_t e = cudaSuccess;
  for (int q = 0; q < 6 && e == cudaSuccess; ++q) e = cudaEventCreateWithFlags(&ev[q], cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_raw, src[0], N * sizeof(float), cudaMemcpyHostToDevice, h->st);
  if (e == cudaSuccess) e = cudaEventRecord(ev[0], h->st);
  for (int t = 0; t < 4 && e == cudaSuccess; ++t) {
    const long long n0 = 32 * t, n1 = t == 3 ? 125 : 32 * t + 32;
    for (int k = 1; k < nrec && e == cudaSuccess; ++k)
      e = cudaMemcpyAsync(d_raw + (size_t)k * N + n0 * E, src[k] + n0 * E, (size_t)(n1 - n0) * E * sizeof(float),
                          cudaMemcpyHostToDevice, h->st);
    if (e == cudaSuccess) e = cudaEventRecord(ev[1 + t], h->st);
  }
  if (e == cudaSuccess) e = cudaMemsetAsync(h->d_aniso, 0, sizeof(int), h->st2);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(h->st2, ev[0], 0);
  if (e == cudaSuccess) e = model_kernels(h, rec, 0, 0, true, h->st2);
  for (int t = 0; t < 4 && e == cudaSuccess; ++t) {
    e = cudaStreamWaitEvent(h->st2, ev[1 + t], 0);
    if (e == cudaSuccess) e = model_kernels(h, rec, t, t + 1, false, h->st2);
  }
  if (e == cudaSuccess) e = cudaEventRecord(ev[5], h->st2);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(h->st, ev[5], 0);
  if (e == cudaSuccess && in_state) e = cudaMemsetAsync(d_raw, 0, (size_t)nrec * N * sizeof(float), h->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
  if (e == cudaSuccess) e = note_isotropy(h);
  for (cudaEvent_t x : ev)
    if (x) cudaEventDestroy(x);
  if (in_state) {
    if (e != cudaSuccess) {  // the staged records may remain in the state: zero it again
      cudaStreamSynchronize(h->st);
      cudaStreamSynchronize(h->st2);
      cudaMemset(d_raw, 0, (size_t)nrec * N * sizeof(float));
    }
  } else {
    dfree(d_raw);
  }
  if (e != cudaSuccess) return cuda_fail(h, e, "set_model");
  h->model_set = true;
  return SES3D_OK;
}

int ses3d_gpu_set_model_device(ses3d_gpu *h, const float *rhoinv, const float *mu, const float *lambda,
                               const float *A, const float *B, const float *C, const float *Q) {
  if (!h) return SES3D_E_CONFIG;
  if (!rhoinv || !mu || !lambda || !A || !B || !C) return fail(h, SES3D_E_CONFIG, "null model array");
  if (h->cfg.is_diss && !Q) return fail(h, SES3D_E_CONFIG, "Q is required when is_diss = 1");
  const float *rec[7] = {rhoinv, mu, lambda, A, B, C, h->cfg.is_diss ? Q : nullptr};
  return set_model_common(h, rec);
}

int ses3d_gpu_set_source(ses3d_gpu *h, int event, float xxs_deg, float yys_deg, float zzs, int source_type,
                         const float mom[6], const float *so, int *is_source) {
  int rc = check_event(h, event);
  if (rc) return rc;
  if (!so) return fail(h, SES3D_E_CONFIG, "null stf");
  if (source_type == 10 && !mom) return fail(h, SES3D_E_CONFIG, "null moment tensor");
  EventHost &E = h->ev[event];
  E.source_type = source_type;
  locate_source(h->geo, xxs_deg, yys_deg, zzs, source_type, E.src);
  E.so.assign(so, so + h->cfg.nt);
  if (is_source) *is_source = E.src.is_source;
  rc = upload_moment_sources(h);
  if (rc) return rc;
  if (source_type == 10) {
    float m6[6];
    for (int q = 0; q < 6; ++q) m6[q] = mom[q];
    CK(h, cudaMemcpy(h->d_src_mom + (size_t)event * 6, m6, 6 * sizeof(float), cudaMemcpyHostToDevice));
  }
  return rebuild_forces(h);
}

int ses3d_gpu_set_receivers(ses3d_gpu *h, int event, int nr_global, const float *recloc, int *nr_out, int *kept) {
  int rc = check_event(h, event);
  if (rc) return rc;
  if (nr_global < 0 || (nr_global > 0 && !recloc)) return fail(h, SES3D_E_CONFIG, "bad receiver list");
  EventHost &E = h->ev[event];
  E.recs = locate_receivers(h->geo, nr_global, recloc);
  if (nr_out) *nr_out = (int)E.recs.size();
  if (kept)
    for (size_t r = 0; r < E.recs.size(); ++r) kept[r] = E.recs[r].global_index;
  // rebuild the receiver table of all events
  const int nev = h->cfg.n_events;
  std::vector<int> el, evi;
  std::vector<float> w;
  h->rec_off.assign(nev + 1, 0);
  for (int e = 0; e < nev; ++e) {
    h->rec_off[e] = (int)el.size();
    for (const Receiver &r : h->ev[e].recs) {
      el.push_back(r.rx + h->geo.ex * (r.ry + h->geo.ey * r.rz));
      evi.push_back(e);
      w.insert(w.end(), r.weight, r.weight + NPE);
    }
  }
  h->rec_off[nev] = (int)el.size();
  dfree(h->d_rec_elem); dfree(h->d_rec_ev); dfree(h->d_rec_w); dfree(h->d_seis);
  h->d_rec_elem = nullptr; h->d_rec_ev = nullptr; h->d_rec_w = nullptr; h->d_seis = nullptr;
  h->R = (int)el.size();
  if (h->R) {
    CK(h, dalloc(&h->d_rec_elem, el.size()));
    CK(h, dalloc(&h->d_rec_ev, evi.size()));
    CK(h, dalloc(&h->d_rec_w, w.size()));
    CK(h, dalloc(&h->d_seis, (size_t)3 * h->cfg.nt * h->R));
    CK(h, cudaMemcpy(h->d_rec_elem, el.data(), el.size() * sizeof(int), cudaMemcpyHostToDevice));
    CK(h, cudaMemcpy(h->d_rec_ev, evi.data(), evi.size() * sizeof(int), cudaMemcpyHostToDevice));
    CK(h, cudaMemcpy(h->d_rec_w, w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice));
    CK(h, cudaMemset(h->d_seis, 0, (size_t)3 * h->cfg.nt * h->R * sizeof(float)));
  }
  destroy_graph(h);
  return SES3D_OK;
}

int ses3d_gpu_set_adjoint_sources(ses3d_gpu *h, int event, int n, const float *loc, const float *stf, int *n_out) {
  int rc = check_event(h, event);
  if (rc) return rc;
  if (n < 0 || (n > 0 && (!loc || !stf))) return fail(h, SES3D_E_CONFIG, "bad adjoint source list");
  EventHost &E = h->ev[event];
  E.adj = locate_adjoint_sources(h->geo, n, loc);
  const int nt = h->cfg.nt;
  E.adj_stf.clear();
  for (const AdjointSource &a : E.adj)
    E.adj_stf.insert(E.adj_stf.end(), stf + (size_t)a.global_index * 3 * nt, stf + (size_t)(a.global_index + 1) * 3 * nt);
  if (n_out) *n_out = (int)E.adj.size();
  return rebuild_forces(h);
}

// Brings the mirror stresses outside the PML up to date after lean iterations.
static int sync_mirrors(ses3d_gpu *h) {
  if (!h->mirrors_stale) return SES3D_OK;
  CK(h, launch_sync_mirrors(h->c, h->d_state, h->st));
  ++h->launches;
  h->mirrors_stale = false;
  return SES3D_OK;
}

// Reads and clears the device error word after the stream has drained.
static int check_device_error(ses3d_gpu *h) {
  int err = 0;
  CK(h, cudaMemcpy(&err, h->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (err == 0) return SES3D_OK;
  CK(h, cudaMemset(h->d_err, 0, sizeof(int)));
  return fail(h, SES3D_E_CUDA, "bounded wait expired: a bulk copy into shared memory did not complete in time");
}

int ses3d_gpu_step(ses3d_gpu *h, int n) {
  Range range_("ses3d step");
  if (!h) return SES3D_E_CONFIG;
  if (!h->model_set) return fail(h, SES3D_E_STATE, "set_model must be called before step");
  if (n < 0) return fail(h, SES3D_E_CONFIG, "n must be >= 0");
  if (h->external_stepped)
    return fail(h, SES3D_E_STATE, "this handle steps a caller-owned wavefield (ses3d_gpu_step_external)");
  // Lean record and correlation iterations add the displacement gradients of the
  // displacement integrated since the wavefield was zeroed: exact for runs whose
  // displacement gradients start at zero.
  if (h->c.lean && h->mode_flag != 0 && h->du_set)
    return fail(h, SES3D_E_STATE,
                "lean stepping of a run with records or kernel correlation needs it to start with zero displacement "
                "gradients; some were set (set_field)");
  const int nt = h->cfg.nt;
  int done = 0;
  while (done < n && h->it < nt) {
    const int it = h->it + 1;
    const int flag = h->mode_flag;
    // plain iterations replay from a CUDA graph: runs of graph_n in plain forward runs, and
    // in record / adjoint runs the stretches of samp_ad - 1 between stored iterations
    const int L = flag == 0 ? (h->ex_K > 0 ? std::min(h->graph_n, h->ex_K - 1) : h->graph_n)
                            : std::min(h->graph_n, h->cfg.samp_ad - 1);
    if (h->graph_on && L > 0 && n - done >= L && nt - h->it >= L) {
      bool plain = true;
      for (int q = 1; (flag != 0 || h->ex_K > 0) && q <= L && plain; ++q) plain = !special_iteration(h, h->it + q);
      if (plain) {
        if (h->graph_dirty || !h->graph_exec || h->graph_len != L) {
          int rc = build_graph(h, L);
          if (rc) return rc;
        }
        CK(h, cudaGraphLaunch(h->graph_exec, h->st));
        h->launches += (long long)L * launches_per_iteration(h);
        h->it += L;
        done += L;
        continue;
      }
    }
    int mode = 0;
    float *rec = nullptr;
    if (flag == 0 && h->ex_K > 0 && (it - 1) % h->ex_K == 0) {
      int rc = save_exact_checkpoint(h, it - 1);
      if (rc) return rc;
    }
    if (flag == 1 && it == 1) h->fwd_lean = h->c.lean != 0;
    if (flag == 1 && (it % h->cfg.samp_ad == 0 || it == 1 || it == nt)) {
      if (h->ckpt_K > 0) {  // checkpoint before every ckpt_K-th record, no records kept
        if (h->nrec_done % h->ckpt_K == 0) {
          int rc = save_checkpoint(h, it - 1);
          if (rc) return rc;
        }
      } else {
        const size_t rec_floats = (size_t)h->cfg.n_events * NREC * h->geo.N;
        if (h->records.empty()) {  // one allocation for every record of the run
          const size_t n = std::max<size_t>(1, h->store_steps.size());
          float *block = nullptr;
          CK(h, dalloc(&block, n * rec_floats));
          h->record_blocks.push_back(block);
          for (size_t r = 0; r < n; ++r) h->record_slots.push_back(block + r * rec_floats);
        }
        if (h->records.size() < h->record_slots.size()) {
          rec = h->record_slots[h->records.size()];
        } else {
          CK(h, dalloc(&rec, rec_floats));
          h->record_blocks.push_back(rec);
        }
        h->records.push_back(rec);
        mode = 1;
      }
      ++h->nrec_done;
      h->saving_vector[it] = it;
    } else if (flag == 2 && h->saving_vector[nt + 1 - it] > 0 && h->record_cursor > 0) {
      const int r = --h->record_cursor;
      if (h->ckpt_K > 0) {
        int rc = checkpointed_record(h, r, &rec);
        if (rc) return rc;
      } else {
        rec = h->records[r];
      }
      mode = 2;
    }
    int rc = launch_iteration(h, primary_wave(h), mode, rec, h->prof_on);
    if (rc) return rc;
    h->it = it;
    ++done;
    if (flag == 2 && h->cfg.grad_variant == 1 && it == nt && h->cfg.is_diss == 1) {
      CK(h, launch_grad_q_norm(h->c, h->d_gmat, h->d_grad, h->st));
      ++h->launches;
    }
  }
  if (done > 0 && h->c.lean) {
    h->mirrors_stale = true;
    const Geometry &g = h->geo;  // elements outside the PML exist
    if (g.ex > 2 * h->cfg.pml && g.ey > 2 * h->cfg.pml && g.ez > h->cfg.pml) h->du_stale = 0x1ffu;
  }
  CK(h, cudaStreamSynchronize(h->st));
  collect_times(h);
  return check_device_error(h);
}

int ses3d_gpu_current_step(const ses3d_gpu *h) { return h ? h->it : SES3D_E_CONFIG; }

int ses3d_gpu_get_seismograms(ses3d_gpu *h, int event, float *sx, float *sy, float *sz) {
  int rc = check_event(h, event);
  if (rc) return rc;
  const int nr = h->rec_off[event + 1] - h->rec_off[event];
  if (nr == 0) return SES3D_OK;
  float *out[3] = {sx, sy, sz};
  for (int c = 0; c < 3; ++c) {
    if (!out[c]) continue;
    CK(h, cudaMemcpy2DAsync(out[c], nr * sizeof(float), h->d_seis + (size_t)c * h->cfg.nt * h->R + h->rec_off[event],
                            h->R * sizeof(float), nr * sizeof(float), h->cfg.nt, cudaMemcpyDeviceToHost, h->st));
  }
  CK(h, cudaStreamSynchronize(h->st));
  return SES3D_OK;
}

static int state_field_index(int field) {
  static const int map[] = {F_SXX, F_SYY, F_SZZ, F_SXY, F_SYX, F_SXZ, F_SZX, F_SYZ, F_SZY,
                            F_DXUX, F_DYUY, F_DZUZ, F_DXUY, F_DYUX, F_DXUZ, F_DZUX, F_DYUZ, F_DZUY};
  if (field >= SES3D_FIELD_SXX_PML && field <= SES3D_FIELD_DZUY) return map[field - SES3D_FIELD_SXX_PML];
  return -1;
}

// One field of one event, from / into the handle's wavefield or (adjoint) the exact
// adjoint's state.
static int field_io(ses3d_gpu *h, int event, int field, float *hout, const float *hin, bool adjoint = false) {
  int rc = check_event(h, event);
  if (rc) return rc;
  if (field < 0 || field >= SES3D_FIELD_COUNT) return fail(h, SES3D_E_CONFIG, "unknown field");
  if (h->external_stepped && field != SES3D_FIELD_MM_GLOBAL)
    return fail(h, SES3D_E_STATE, "the wavefield of this handle lives in caller-owned buffers (ses3d_gpu_step_external)");
  if (hout && !adjoint && field >= SES3D_FIELD_DXUX && field <= SES3D_FIELD_DZUY &&
      ((h->du_stale >> (field - SES3D_FIELD_DXUX)) & 1u))
    return fail(h, SES3D_E_STATE,
                "lean iterations did not integrate this displacement gradient outside the PML (set_lean)");
  const long long N = h->geo.N, G = h->geo.G;
  if (hin && !adjoint) {
    h->state_zero = false;
    if (field >= SES3D_FIELD_DXUX && field <= SES3D_FIELD_DZUY) h->du_set = true;
  }
  float *vbase = (adjoint ? h->d_av : h->d_v) + (size_t)event * 3 * G;
  float *sbase = (adjoint ? h->d_astate : h->d_state) + (size_t)event * NSTATE * N;
  if (field >= SES3D_FIELD_VX_GLOBAL && field <= SES3D_FIELD_VZ_GLOBAL) {
    float *d = vbase + (size_t)(field - SES3D_FIELD_VX_GLOBAL) * G;
    if (hout) CK(h, cudaMemcpy(hout, d, G * sizeof(float), cudaMemcpyDeviceToHost));
    else CK(h, cudaMemcpy(d, hin, G * sizeof(float), cudaMemcpyHostToDevice));
    return SES3D_OK;
  }
  if (field == SES3D_FIELD_MM_GLOBAL) {
    if (!hout) return fail(h, SES3D_E_CONFIG, "MM_global is read-only");
    CK(h, cudaMemcpy(hout, h->d_MM, G * sizeof(float), cudaMemcpyDeviceToHost));
    return SES3D_OK;
  }
  float *tmp = nullptr, *tmp2 = nullptr;
  CK(h, dalloc(&tmp, (size_t)N));
  CK(h, dalloc(&tmp2, (size_t)N));
  auto done = [&](int r) { dfree(tmp); dfree(tmp2); return r; };
  if (field >= SES3D_FIELD_VX && field <= SES3D_FIELD_VZ) {
    if (!hout) return done(fail(h, SES3D_E_CONFIG, "local v is derived from the global v; set the global field"));
    Consts c1 = h->c;
    cudaError_t e = launch_gather_ref(c1, vbase + (size_t)(field - SES3D_FIELD_VX) * G, tmp, h->st);
    if (e != cudaSuccess) return done(cuda_fail(h, e, "gather"));
    e = cudaMemcpyAsync(hout, tmp, N * sizeof(float), cudaMemcpyDeviceToHost, h->st);
    if (e != cudaSuccess) return done(cuda_fail(h, e, "copy"));
  } else if (state_field_index(field) >= 0) {
    const int f = state_field_index(field);
    if (!adjoint)
      if (int r = sync_mirrors(h)) return done(r);
    cudaError_t e;
    if (hout) {
      e = launch_state_field(sbase, f, tmp, h->geo.E, 1, h->st);
      if (e == cudaSuccess) e = cudaMemcpyAsync(hout, tmp, N * sizeof(float), cudaMemcpyDeviceToHost, h->st);
    } else {
      e = cudaMemcpyAsync(tmp, hin, N * sizeof(float), cudaMemcpyHostToDevice, h->st);
      if (e == cudaSuccess) e = launch_state_field(sbase, f, tmp, h->geo.E, 0, h->st);
      if (e == cudaSuccess && !adjoint && field >= SES3D_FIELD_DXUX && field <= SES3D_FIELD_DZUY)
        h->du_stale &= ~(1u << (field - SES3D_FIELD_DXUX));
    }
    if (e != cudaSuccess) return done(cuda_fail(h, e, "field transfer"));
  } else if (field >= SES3D_FIELD_MXX && field <= SES3D_FIELD_MYZ) {
    const int cc = field - SES3D_FIELD_MXX;
    std::vector<float> buf((size_t)N), inter;
    if (hout) {
      for (int m = 0; m < 3; ++m) {
        cudaError_t e = launch_state_field(sbase, F_M + 3 * cc + m, tmp, h->geo.E, 1, h->st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(buf.data(), tmp, N * sizeof(float), cudaMemcpyDeviceToHost, h->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
        if (e != cudaSuccess) return done(cuda_fail(h, e, "memory variable transfer"));
        for (long long q = 0; q < N; ++q) hout[m + 3 * q] = buf[q];
      }
    } else {
      for (int m = 0; m < 3; ++m) {
        for (long long q = 0; q < N; ++q) buf[q] = hin[m + 3 * q];
        cudaError_t e = cudaMemcpyAsync(tmp, buf.data(), N * sizeof(float), cudaMemcpyHostToDevice, h->st);
        if (e == cudaSuccess) e = launch_state_field(sbase, F_M + 3 * cc + m, tmp, h->geo.E, 0, h->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
        if (e != cudaSuccess) return done(cuda_fail(h, e, "memory variable transfer"));
      }
    }
  }
  cudaError_t e = cudaStreamSynchronize(h->st);
  if (e != cudaSuccess) return done(cuda_fail(h, e, "field sync"));
  return done(SES3D_OK);
}

int ses3d_gpu_get_field(ses3d_gpu *h, int event, int field, float *out) {
  if (!out) return fail(h, SES3D_E_CONFIG, "null output");
  return field_io(h, event, field, out, nullptr);
}

int ses3d_gpu_set_field(ses3d_gpu *h, int event, int field, const float *in) {
  if (!in) return fail(h, SES3D_E_CONFIG, "null input");
  return field_io(h, event, field, nullptr, in);
}

int ses3d_gpu_get_kernel(ses3d_gpu *h, int event, int which, double *out) {
  int rc = check_event(h, event);
  if (rc) return rc;
  if (which < 0 || which >= SES3D_KERNEL_COUNT || !out) return fail(h, SES3D_E_CONFIG, "bad kernel id");
  if (!h->d_grad) return fail(h, SES3D_E_STATE, "kernels exist only in adjoint runs (adjoint_flag = 2)");
  const long long N = h->geo.N;
  static const int slot[] = {0, 1, 2, 3, 4, 5, 6, 7};
  double *tmp = nullptr;
  CK(h, dalloc(&tmp, (size_t)N));
  cudaError_t e = launch_transpose_d(h->d_grad + ((size_t)event * NGRAD + slot[which]) * N, tmp, h->geo.E, NPE, false,
                                     h->st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, tmp, N * sizeof(double), cudaMemcpyDeviceToHost, h->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
  dfree(tmp);
  if (e != cudaSuccess) return cuda_fail(h, e, "get_kernel");
  return SES3D_OK;
}

// Event sum of one kernel into out (reference layout): host memory, or device memory of
// the handle's device when `device` is set (no host copy); `accumulate` (device only) adds
// the sum to out's values.
static int kernel_sum(ses3d_gpu *h, int which, double *out, bool device, bool accumulate = false) {
  if (!h) return SES3D_E_CONFIG;
  if (which < 0 || which >= SES3D_KERNEL_COUNT || !out) return fail(h, SES3D_E_CONFIG, "bad kernel id");
  if (!h->d_grad) return fail(h, SES3D_E_STATE, "kernels exist only in adjoint runs (adjoint_flag = 2)");
  const long long N = h->geo.N;
  double *tmp = nullptr, *sum = nullptr;
  CK(h, dalloc(&sum, (size_t)N));
  cudaError_t e = device ? cudaSuccess : dalloc(&tmp, (size_t)N);
  if (e == cudaSuccess) e = launch_sum_events_d(h->d_grad, which, h->cfg.n_events, N, sum, h->st);
  if (e == cudaSuccess) e = launch_transpose_d(sum, device ? out : tmp, h->geo.E, NPE, device && accumulate, h->st);
  if (e == cudaSuccess && !device) e = cudaMemcpyAsync(out, tmp, N * sizeof(double), cudaMemcpyDeviceToHost, h->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
  dfree(tmp);
  dfree(sum);
  if (e != cudaSuccess) return cuda_fail(h, e, "get_kernel_sum");
  h->launches += 2;
  return SES3D_OK;
}

int ses3d_gpu_get_kernel_sum(ses3d_gpu *h, int which, double *out) { return kernel_sum(h, which, out, false); }

int ses3d_gpu_get_kernel_sum_device(ses3d_gpu *h, int which, double *out) { return kernel_sum(h, which, out, true); }

int ses3d_gpu_add_kernel_sum_device(ses3d_gpu *h, int which, double *acc) {
  return kernel_sum(h, which, acc, true, true);
}

int ses3d_gpu_misfit_gradient_device(const ses3d_config *cfg, const double *ksum, double scale, const void *divisor,
                                     void *out, int f64) {
  Range range_("ses3d misfit gradient");
  if (!cfg || !ksum || !out) return fail(nullptr, SES3D_E_CONFIG, "null argument");
  if (cfg->lpd != LPD) return fail(nullptr, SES3D_E_CONFIG, "this library implements lpd = 4 only");
  Geometry g;
  std::string msg = build_geometry(g, cfg->nx, cfg->ny, cfg->nz, cfg->pml, cfg->xmin, cfg->xmax, cfg->ymin, cfg->ymax,
                                   cfg->zmin, cfg->zmax, cfg->zmax_global);
  if (!msg.empty()) return fail(nullptr, SES3D_E_CONFIG, msg);
  // FP64 tables of the quadrature volume: coef[kn][jn][in] = ((w_in w_jn) w_kn) Jac,
  // r2[kn][k] = r^2, sinx[in][i] = sin(theta) (theta, r the FP32 GLL coordinates)
  std::vector<double> tab((size_t)NPE + (size_t)NP * g.ez + (size_t)NP * g.ex);
  const double jac = (double)g.Jac;
  for (int kn = 0; kn < NP; ++kn)
    for (int jn = 0; jn < NP; ++jn)
      for (int in = 0; in < NP; ++in)
        tab[(kn * NP + jn) * NP + in] = (((double)g.w[in] * (double)g.w[jn]) * (double)g.w[kn]) * jac;
  double *r2 = tab.data() + NPE, *sinx = r2 + (size_t)NP * g.ez;
  for (int kn = 0; kn < NP; ++kn)
    for (int k = 0; k < g.ez; ++k) {
      const double z = (double)g.Z(k, kn);
      r2[(size_t)kn * g.ez + k] = z * z;
    }
  for (int in = 0; in < NP; ++in)
    for (int i = 0; i < g.ex; ++i) sinx[(size_t)in * g.ex + i] = std::sin((double)g.X(i, in));
  double *d_tab = nullptr;
  cudaError_t e = dalloc(&d_tab, tab.size());
  if (e == cudaSuccess) e = cudaMemcpy(d_tab, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = launch_misfit_gradient(ksum, d_tab, g.ex, g.ey, g.ez, scale * jac, divisor, out, f64 != 0, 0);
  if (e == cudaSuccess) e = cudaStreamSynchronize(0);
  dfree(d_tab);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "misfit_gradient");
  return SES3D_OK;
}

int ses3d_gpu_record_count(const ses3d_gpu *h, int event) {
  if (!h || event < 0 || event >= h->cfg.n_events) return SES3D_E_CONFIG;
  return h->ckpt_K > 0 ? h->nrec_done : (int)h->records.size();
}

int ses3d_gpu_get_record(ses3d_gpu *h, int event, int record, float *out) {
  int rc = check_event(h, event);
  if (rc) return rc;
  if (h->ckpt_K > 0) return fail(h, SES3D_E_STATE, "records are recomputed from checkpoints, not kept");
  if (record < 0 || record >= (int)h->records.size() || !out) return fail(h, SES3D_E_CONFIG, "bad record index");
  const long long N = h->geo.N;
  float *tmp = nullptr;
  CK(h, dalloc(&tmp, (size_t)N));
  cudaError_t e = cudaSuccess;
  for (int f = 0; f < NREC && e == cudaSuccess; ++f) {
    e = launch_transpose(h->records[record] + ((size_t)event * NREC + f) * N, tmp, h->geo.E, NPE, h->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out + (size_t)f * N, tmp, N * sizeof(float), cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
  }
  dfree(tmp);
  if (e != cudaSuccess) return cuda_fail(h, e, "get_record");
  return SES3D_OK;
}

int ses3d_gpu_put_record(ses3d_gpu *h, int event, int record, const float *in) {
  int rc = check_event(h, event);
  if (rc) return rc;
  if (record < 0 || record > (int)h->records.size() || !in) return fail(h, SES3D_E_CONFIG, "bad record index");
  const long long N = h->geo.N;
  if (record == (int)h->records.size()) {
    float *r = nullptr;
    CK(h, dalloc(&r, (size_t)h->cfg.n_events * NREC * N));
    h->record_blocks.push_back(r);
    CK(h, cudaMemset(r, 0, (size_t)h->cfg.n_events * NREC * N * sizeof(float)));
    h->records.push_back(r);
    h->record_cursor = (int)h->records.size();
    h->nrec_done = (int)h->records.size();
  }
  float *tmp = nullptr;
  CK(h, dalloc(&tmp, (size_t)N));
  cudaError_t e = cudaSuccess;
  for (int f = 0; f < NREC && e == cudaSuccess; ++f) {
    e = cudaMemcpyAsync(tmp, in + (size_t)f * N, N * sizeof(float), cudaMemcpyHostToDevice, h->st);
    if (e == cudaSuccess) e = launch_transpose(tmp, h->records[record] + ((size_t)event * NREC + f) * N, NPE, h->geo.E, h->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
  }
  dfree(tmp);
  if (e != cudaSuccess) return cuda_fail(h, e, "put_record");
  return SES3D_OK;
}

int ses3d_gpu_get_saving_vector(const ses3d_gpu *h, int *out) {
  if (!h || !out) return SES3D_E_CONFIG;
  for (int k = 1; k <= h->cfg.nt; ++k) out[k - 1] = h->saving_vector[k];
  return SES3D_OK;
}

int ses3d_gpu_set_saving_vector(ses3d_gpu *h, const int *in) {
  if (!h || !in) return SES3D_E_CONFIG;
  for (int k = 1; k <= h->cfg.nt; ++k) h->saving_vector[k] = in[k - 1];
  return SES3D_OK;
}

int ses3d_gpu_begin_adjoint(ses3d_gpu *h) {
  Range range_("ses3d begin adjoint");
  if (!h) return SES3D_E_CONFIG;
  h->mode_flag = 2;
  h->cfg.adjoint_flag = 2;
  h->c.lean = 0;  // the adjoint run chooses its own stepping; the wavefield is zeroed below
  if (!h->d_grad) {
    CK(h, dalloc(&h->d_grad, (size_t)h->cfg.n_events * NGRAD * h->geo.N));
  }
  CK(h, cudaMemsetAsync(h->d_grad, 0, (size_t)h->cfg.n_events * NGRAD * h->geo.N * sizeof(double), h->st));
  h->record_cursor = h->ckpt_K > 0 ? h->nrec_done : (int)h->records.size();
  h->seg_loaded = -1;
  h->sub_loaded = -1;
  destroy_graph(h);
  int rc = zero_wavefield(h);
  if (rc) return rc;
  CK(h, cudaStreamSynchronize(h->st));
  return SES3D_OK;
}

long ses3d_gpu_get_setup_int(ses3d_gpu *h, int event, const char *name, int *out) {
  int rc = check_event(h, event);
  if (rc) return rc;
  const std::string nm = name ? name : "";
  const EventHost &E = h->ev[event];
  auto one = [&](int v) -> long { if (out) out[0] = v; return 1; };
  auto vec = [&](const std::vector<int> &v) -> long { if (out) std::copy(v.begin(), v.end(), out); return (long)v.size(); };
  if (nm == "nr") return one((int)E.recs.size());
  if (nm == "isotropic") return one(h->c.iso);
  if (nm == "rx" || nm == "ry" || nm == "rz") {
    std::vector<int> v;
    for (const Receiver &r : E.recs) v.push_back(nm == "rx" ? r.rx : nm == "ry" ? r.ry : r.rz);
    return vec(v);
  }
  if (nm == "kept") { std::vector<int> v; for (const Receiver &r : E.recs) v.push_back(r.global_index); return vec(v); }
  if (nm == "isx") return one(E.src.isx);
  if (nm == "isy") return one(E.src.isy);
  if (nm == "isz") return one(E.src.isz);
  if (nm == "isx_n") return one(E.src.isx_n);
  if (nm == "isy_n") return one(E.src.isy_n);
  if (nm == "isz_n") return one(E.src.isz_n);
  if (nm == "is_source") return one(E.src.is_source);
  if (nm == "nr_adsrc") return one((int)E.adj.size());
  if (nm == "is" || nm == "isn") {
    std::vector<int> v;
    for (const AdjointSource &a : E.adj)
      for (int c = 0; c < 3; ++c) v.push_back(nm == "is" ? a.is[c] : a.isn[c]);
    return vec(v);
  }
  return fail(h, SES3D_E_CONFIG, "unknown setup integer " + nm);
}

long ses3d_gpu_get_setup_real(ses3d_gpu *h, int event, const char *name, float *out) {
  int rc = check_event(h, event);
  if (rc) return rc;
  const std::string nm = name ? name : "";
  const EventHost &E = h->ev[event];
  const Geometry &g = h->geo;
  auto one = [&](float v) -> long { if (out) out[0] = v; return 1; };
  auto vec = [&](const std::vector<float> &v) -> long { if (out) std::copy(v.begin(), v.end(), out); return (long)v.size(); };
  if (nm == "xxs_loc") return one(E.src.xxs_loc);
  if (nm == "yys_loc") return one(E.src.yys_loc);
  if (nm == "zzs_loc") return one(E.src.zzs_loc);
  if (nm == "dx") return one(g.dx);
  if (nm == "dy") return one(g.dy);
  if (nm == "dz") return one(g.dz);
  if (nm == "Jac") return one(g.Jac);
  if (nm == "knots") return vec(std::vector<float>(g.knots, g.knots + NP));
  if (nm == "w") return vec(std::vector<float>(g.w, g.w + NP));
  if (nm == "dl") {  // F-order (i,j): dl(i,j) at i + 5 j
    std::vector<float> v(NP * NP);
    for (int i = 0; i < NP; ++i) for (int j = 0; j < NP; ++j) v[i + NP * j] = g.dl[i][j];
    return vec(v);
  }
  auto axis = [&](const std::vector<float> &t, int ne) {  // (0:ne-1, 0:lpd) F-order
    std::vector<float> v((size_t)ne * NP);
    for (int i = 0; i < ne; ++i) for (int n = 0; n < NP; ++n) v[i + (size_t)ne * n] = t[(size_t)i * NP + n];
    return v;
  };
  if (nm == "x") return vec(axis(g.x, g.ex));
  if (nm == "y") return vec(axis(g.y, g.ey));
  if (nm == "z") return vec(axis(g.z, g.ez));
  if (nm == "recloc_std") {
    std::vector<float> v;
    for (const Receiver &r : E.recs) v.insert(v.end(), r.std, r.std + 3);
    return vec(v);
  }
  if (nm == "ad_loc_std") {
    std::vector<float> v;
    for (const AdjointSource &a : E.adj) v.insert(v.end(), a.loc_std, a.loc_std + 3);
    return vec(v);
  }
  if (nm == "prof_x" || nm == "prof_y" || nm == "prof_z" || nm == "prof" || nm == "taper") {
    if (!out) return (long)g.N;
    for (int kn = 0; kn < NP; ++kn)
      for (int jn = 0; jn < NP; ++jn)
        for (int in = 0; in < NP; ++in)
          for (int k = 0; k < g.ez; ++k)
            for (int j = 0; j < g.ey; ++j)
              for (int i = 0; i < g.ex; ++i) {
                float px, py, pz, prof, taper;
                pml_normalise(g.pxr[(size_t)i * NP + in], g.pyr[(size_t)j * NP + jn], g.pzr[(size_t)k * NP + kn],
                              px, py, pz, prof, taper);
                long long e = i + (long long)g.ex * (j + (long long)g.ey * k);
                long long q = e + g.E * (in + NP * (jn + NP * kn));
                out[q] = nm == "prof_x" ? px : nm == "prof_y" ? py : nm == "prof_z" ? pz : nm == "prof" ? prof : taper;
              }
    return (long)g.N;
  }
  return fail(h, SES3D_E_CONFIG, "unknown setup real " + nm);
}

int ses3d_gpu_selftest_wait(ses3d_gpu *h, int limit_ms) {
  if (!h) return SES3D_E_CONFIG;
  if (limit_ms < 1 || limit_ms > 10000) return fail(h, SES3D_E_CONFIG, "limit_ms must be in 1..10000");
  CK(h, launch_wait_selftest(h->d_err, (unsigned long long)limit_ms * 1000000ull, h->st));
  CK(h, cudaStreamSynchronize(h->st));
  return check_device_error(h);
}

int ses3d_gpu_vmax(ses3d_gpu *h, float *out) {
  if (!h || !out) return SES3D_E_CONFIG;
  const int nev = h->cfg.n_events;
  CK(h, cudaMemsetAsync(h->d_scratch_u, 0, nev * sizeof(unsigned int), h->st));
  CK(h, launch_vmax(h->d_v, 3 * h->geo.G, nev, h->d_scratch_u, h->st));
  ++h->launches;
  std::vector<unsigned int> u(nev);
  CK(h, cudaMemcpyAsync(u.data(), h->d_scratch_u, nev * sizeof(unsigned int), cudaMemcpyDeviceToHost, h->st));
  CK(h, cudaStreamSynchronize(h->st));
  bool bad = false;
  for (int e = 0; e < nev; ++e) {
    std::memcpy(&out[e], &u[e], sizeof(float));
    if (!(out[e] < 3.0e38f)) bad = true;
  }
  if (bad) return fail(h, SES3D_E_NAN, "non-finite velocity field");
  return SES3D_OK;
}

void *ses3d_gpu_stream(ses3d_gpu *h) { return h ? (void *)h->st : nullptr; }

int64_t ses3d_gpu_launch_count(const ses3d_gpu *h) { return h ? h->launches : 0; }

int ses3d_gpu_use_graph(ses3d_gpu *h, int enable, int n_per_graph) {
  if (!h) return SES3D_E_CONFIG;
  if (enable && n_per_graph < 1) return fail(h, SES3D_E_CONFIG, "n_per_graph must be >= 1");
  destroy_graph(h);
  h->graph_on = enable != 0;
  h->graph_n = enable ? n_per_graph : 0;
  return SES3D_OK;
}

int ses3d_gpu_set_checkpointing(ses3d_gpu *h, int records_per_segment) {
  return ses3d_gpu_set_checkpoint_levels(h, records_per_segment, 0);
}

int ses3d_gpu_set_checkpoint_levels(ses3d_gpu *h, int records_per_segment, int records_per_subsegment) {
  if (!h) return SES3D_E_CONFIG;
  if (records_per_segment < 0 || records_per_subsegment < 0)
    return fail(h, SES3D_E_CONFIG, "records per segment and sub-segment must be >= 0");
  if (records_per_subsegment > 0 && (records_per_segment == 0 || records_per_subsegment >= records_per_segment))
    return fail(h, SES3D_E_CONFIG, "records per sub-segment must lie between 1 and records per segment - 1");
  if (h->it != 0 || h->mode_flag != 1) return fail(h, SES3D_E_STATE, "set checkpointing before a flag-1 run starts");
  h->ckpt_K = records_per_segment;
  h->ckpt_K2 = records_per_subsegment;
  return SES3D_OK;
}

int64_t ses3d_gpu_memory_bytes(const ses3d_gpu *h) {
  if (!h) return 0;
  const size_t N = h->geo.N, G = h->geo.G, nev = h->cfg.n_events;
  // tables, mass matrix, material, adjoint material; per event the element state and forces;
  // velocity (and displacement)
  size_t f = (size_t)KTAB_FLOATS + 2 * G + (size_t)ELEM_MAT * h->geo.E + (size_t)NGMAT * N +
             nev * ((size_t)NSTATE * N + 3 * N) + v_floats(h);
  size_t bytes = f * sizeof(float);
  if (h->d_grad) bytes += nev * NGRAD * N * sizeof(double);
  bytes += std::max(h->records.size(), h->record_slots.size()) * nev * NREC * N * sizeof(float);
  bytes += h->ckpts.size() * rec_ckpt_floats(h) * sizeof(float);
  bytes += h->segbuf.size() * nev * NREC * N * sizeof(float);
  bytes += h->ckpt2.size() * rec_ckpt_floats(h) * sizeof(float);
  bytes += h->ex_block_floats * sizeof(float);
  if (h->d_astate) bytes += nev * (((size_t)NSTATE * N + 6 * G + 3 * N) * sizeof(float) + ((size_t)NMAT * N + G) * sizeof(double));
  if (h->d_state2) bytes += (nev * (size_t)NSTATE * N + v_floats(h)) * sizeof(float);
  bytes += (size_t)3 * h->cfg.nt * h->R * sizeof(float);
  return (int64_t)bytes;
}

int ses3d_gpu_set_lean(ses3d_gpu *h, int enable) {
  if (!h) return SES3D_E_CONFIG;
  // A run with records or kernel correlation takes displacement gradients from its state in
  // PML elements and from the displacement elsewhere: its stepping is chosen before it starts.
  if (h->mode_flag != 0 && h->it != 0 && (enable != 0) != (h->c.lean != 0))
    return fail(h, SES3D_E_STATE, "lean stepping of a run with records or kernel correlation is chosen before the run starts");
  // An exact-adjoint run replays its iterations from checkpoints in the same stepping as its
  // forward run, so the choice is made before that run starts and kept.
  if (h->ex_K > 0 && h->it != 0 && (enable != 0) != (h->c.lean != 0))
    return fail(h, SES3D_E_STATE, "lean stepping of an exact-adjoint run is chosen before its forward run starts");
  if (!enable) {
    int rc = sync_mirrors(h);
    if (rc) return rc;
    CK(h, cudaStreamSynchronize(h->st));
  }
  h->c.lean = enable ? 1 : 0;
  destroy_graph(h);
  return SES3D_OK;
}

int ses3d_gpu_profile(ses3d_gpu *h, int enable) {
  if (!h) return SES3D_E_CONFIG;
  h->prof_on = enable != 0;
  if (enable)
    for (int k = 0; k < 4; ++k) { h->prof_ms[k] = 0; h->prof_n[k] = 0; }
  return SES3D_OK;
}

int ses3d_gpu_kernel_time(const ses3d_gpu *h, int which, double *total_ms, int64_t *launches) {
  if (!h || which < 0 || which > 3) return SES3D_E_CONFIG;
  if (total_ms) *total_ms = h->prof_ms[which];
  if (launches) *launches = h->prof_n[which];
  return SES3D_OK;
}

int ses3d_gpu_set_kernel_shape(ses3d_gpu *h, int element_shape, int node_block) {
  if (!h) return SES3D_E_CONFIG;
  if (element_shape < 0 || element_shape >= element_shape_count())
    return fail(h, SES3D_E_CONFIG, "element_shape must be 0 .. " + std::to_string(element_shape_count() - 1));
  if (node_block != 128 && node_block != 256 && node_block != 512)
    return fail(h, SES3D_E_CONFIG, "node_block must be 128, 256 or 512");
  h->shape = element_shape;
  h->node_block = node_block;
  destroy_graph(h);
  return SES3D_OK;
}

int ses3d_gpu_kernel_shape_count(void) { return element_shape_count(); }

int ses3d_gpu_set_block_elements(ses3d_gpu *h, int elements_per_cta) {
  if (!h) return SES3D_E_CONFIG;
  if (elements_per_cta == 0) elements_per_cta = 1;
  if (elements_per_cta != 1 && elements_per_cta != 2 && elements_per_cta != 4)
    return fail(h, SES3D_E_CONFIG, "elements_per_cta must be 1, 2 or 4");
  h->epb = elements_per_cta;
  destroy_graph(h);
  return SES3D_OK;
}

// ---------------------------------------------------------------------------------------
// Exact discrete adjoint
// ---------------------------------------------------------------------------------------
int ses3d_gpu_exact_adjoint(ses3d_gpu *h, int steps_per_checkpoint, int steps_per_subsegment) {
  if (!h) return SES3D_E_CONFIG;
  if (h->mode_flag != 0)
    return fail(h, SES3D_E_CONFIG, "the exact adjoint differentiates plain forward runs (adjoint_flag 0)");
  if (steps_per_checkpoint < 1) return fail(h, SES3D_E_CONFIG, "steps_per_checkpoint must be >= 1");
  if (steps_per_subsegment < 0 || (steps_per_subsegment > 0 && steps_per_subsegment >= steps_per_checkpoint))
    return fail(h, SES3D_E_CONFIG, "steps_per_subsegment must be 0 or between 1 and steps_per_checkpoint - 1");
  if (h->it != 0 || h->external_stepped)
    return fail(h, SES3D_E_STATE, "enable the exact adjoint before the forward run starts");
  const size_t nev = h->cfg.n_events, N = h->geo.N, G = h->geo.G;
  if (!h->d_astate) {
    CK(h, dalloc(&h->d_astate, nev * NSTATE * N));
    CK(h, dalloc(&h->d_av, nev * 3 * G));
    CK(h, dalloc(&h->d_aF, nev * 3 * G));
    CK(h, dalloc(&h->d_af, nev * 3 * N));
    CK(h, dalloc(&h->d_egmat, nev * NMAT * N));
    CK(h, dalloc(&h->d_egimm, nev * G));
    CK(h, dalloc(&h->d_ait, 1));
  }
  CK(h, cudaMemsetAsync(h->d_astate, 0, nev * NSTATE * N * sizeof(float), h->st));
  CK(h, cudaMemsetAsync(h->d_av, 0, nev * 3 * G * sizeof(float), h->st));
  CK(h, cudaStreamSynchronize(h->st));
  h->ex_K = steps_per_checkpoint;
  h->ex_K2 = steps_per_subsegment;
  h->ex_zero_d = true;
  h->seis_adj.assign(nev, std::vector<float>());
  h->ex_done = false;
  destroy_graph(h);
  return SES3D_OK;
}

int ses3d_gpu_exact_set_seismogram_adjoint(ses3d_gpu *h, int event, const float *gx, const float *gy, const float *gz) {
  int rc = check_event(h, event);
  if (rc) return rc;
  if (h->ex_K <= 0) return fail(h, SES3D_E_STATE, "enable the exact adjoint first (ses3d_gpu_exact_adjoint)");
  const int nr = h->rec_off[event + 1] - h->rec_off[event], nt = h->cfg.nt;
  std::vector<float> &g = h->seis_adj[event];
  g.assign((size_t)3 * nt * nr, 0.f);
  const float *src[3] = {gx, gy, gz};
  for (int c = 0; c < 3; ++c)
    if (src[c]) std::memcpy(g.data() + (size_t)c * nt * nr, src[c], (size_t)nt * nr * sizeof(float));
  return SES3D_OK;
}

// The receivers' adjoint sources as point forces on the element contributions to the
// adjoint velocity: one group per (event, element), receivers in order, weights the
// receivers' Lagrange weights, time functions -d misfit / d seismogram (k_inject subtracts).
static int build_seismogram_forces(ses3d_gpu *h) {
  const int nt = h->cfg.nt;
  std::map<std::pair<int, long long>, std::vector<int>> groups;
  std::vector<const Receiver *> recs;
  std::vector<const float *> series;  // [3][nt][nr] of the receiver's event
  std::vector<int> rloc, nrs;
  for (int e = 0; e < h->cfg.n_events; ++e) {
    const int nr = (int)h->ev[e].recs.size();
    for (int r = 0; r < nr; ++r) {
      const Receiver &R = h->ev[e].recs[r];
      const long long el = R.rx + (long long)h->geo.ex * (R.ry + (long long)h->geo.ey * R.rz);
      groups[{e, el}].push_back((int)recs.size());
      recs.push_back(&R);
      series.push_back(h->seis_adj[e].empty() ? nullptr : h->seis_adj[e].data());
      rloc.push_back(r);
      nrs.push_back(nr);
    }
  }
  std::vector<int4> gr;
  std::vector<float> delta, stf;
  std::vector<int> mask;
  int k = 0;
  for (auto &kv : groups) {
    int4 g4;
    g4.x = kv.first.first; g4.y = (int)kv.first.second; g4.z = k;
    for (int q : kv.second) {
      delta.insert(delta.end(), recs[q]->weight, recs[q]->weight + NPE);
      for (int c = 0; c < 3; ++c)
        for (int t = 0; t < nt; ++t)
          stf.push_back(series[q] ? -series[q][((size_t)c * nt + t) * nrs[q] + rloc[q]] : 0.f);
      mask.push_back(7);
      ++k;
    }
    g4.w = k;
    gr.push_back(g4);
  }
  ForceSet &F = h->fseis;
  free_forces(F);
  F.n = (int)gr.size();
  if (F.n) {
    CK(h, dalloc(&F.groups, gr.size()));
    CK(h, dalloc(&F.delta, delta.size()));
    CK(h, dalloc(&F.stf, stf.size()));
    CK(h, dalloc(&F.mask, mask.size()));
    CK(h, cudaMemcpy(F.groups, gr.data(), gr.size() * sizeof(int4), cudaMemcpyHostToDevice));
    CK(h, cudaMemcpy(F.delta, delta.data(), delta.size() * sizeof(float), cudaMemcpyHostToDevice));
    CK(h, cudaMemcpy(F.stf, stf.data(), stf.size() * sizeof(float), cudaMemcpyHostToDevice));
    CK(h, cudaMemcpy(F.mask, mask.data(), mask.size() * sizeof(int), cudaMemcpyHostToDevice));
  }
  return SES3D_OK;
}

int ses3d_gpu_exact_backward(ses3d_gpu *h) {
  Range range_("ses3d exact backward");
  if (!h) return SES3D_E_CONFIG;
  if (h->ex_K <= 0) return fail(h, SES3D_E_STATE, "enable the exact adjoint before the forward run");
  const int nt = h->cfg.nt, K = h->ex_K;
  if (h->it != nt) return fail(h, SES3D_E_STATE, "the forward run must be complete (nt iterations)");
  if (h->ex_done) return fail(h, SES3D_E_STATE, "the backward run of this forward run is done");
  const int nseg = (nt + K - 1) / K;
  if ((int)h->ex_ckpts.size() < nseg) return fail(h, SES3D_E_STATE, "missing exact-adjoint checkpoints");
  int rc = build_seismogram_forces(h);
  if (rc) return rc;
  const size_t nev = h->cfg.n_events, N = h->geo.N, G = h->geo.G;
  const size_t ns = nev * NSTATE * N, nv = nev * 3 * G;
  const size_t nsl = nev * (size_t)slot_stride(h->cfg.is_diss) * h->geo.E;  // packed forward state of an iteration slot
  CK(h, cudaMemsetAsync(h->d_egmat, 0, nev * NMAT * N * sizeof(double), h->st));
  CK(h, cudaMemsetAsync(h->d_egimm, 0, nev * G * sizeof(double), h->st));
  const int ait0 = nt - 1;
  CK(h, cudaMemcpyAsync(h->d_ait, &ait0, sizeof(int), cudaMemcpyHostToDevice, h->st));
  const int K2 = h->ex_K2 > 0 ? h->ex_K2 : K;  // iterations recomputed into slots at a time
  rc = grow_exact_buffers(h, h->ex_slots, (size_t)std::min(K2, nt), nsl + 2 * nv);
  if (rc) return rc;
  const int nsub_max = (std::min(K, nt) + K2 - 1) / K2;
  rc = grow_exact_buffers(h, h->ex_ckpts2, (size_t)std::max(0, nsub_max - 1), ckpt_floats(h));
  if (rc) return rc;
  Ptrs p = make_ptrs(h);
  AdjPtrs a;
  std::memset(&a, 0, sizeof(a));
  a.astate = h->d_astate; a.av = h->d_av; a.aF = h->d_aF; a.af = h->d_af;
  a.gmat = h->d_egmat; a.gimm = h->d_egimm; a.d_ait = h->d_ait;
  a.zero_d = h->ex_zero_d ? 1 : 0;
  rc = ensure_wave2(h);  // the recomputing wavefield must exist before its pointers are taken
  if (rc) return rc;
  const Wave w{h->d_state2, h->d_v2, h->d_it2, false, false};
  for (int sg = nseg - 1; sg >= 0; --sg) {
    const int t0 = sg * K, t1 = std::min(t0 + K, nt);
    const int nsub = (t1 - t0 + K2 - 1) / K2;
    if (nsub > 1) {  // second level: checkpoints before sub-segments 1 .. nsub - 1 of the segment
      Range r2("ses3d exact recompute checkpoints");
      rc = load_wave2(h, h->ex_ckpts[sg], t0);
      if (rc) return rc;
      int t = t0;
      for (int j = 1; j < nsub; ++j) {
        for (; t < t0 + j * K2; ++t) {
          rc = launch_iteration(h, w, 0, nullptr);
          if (rc) return rc;
        }
        CK(h, cudaMemcpyAsync(h->ex_ckpts2[j - 1], h->d_state2, ns * sizeof(float), cudaMemcpyDeviceToDevice, h->st));
        CK(h, cudaMemcpyAsync(h->ex_ckpts2[j - 1] + ns, h->d_v2, nv * sizeof(float), cudaMemcpyDeviceToDevice,
                              h->st));
      }
    }
    for (int j = nsub - 1; j >= 0; --j) {
      const int a0 = t0 + j * K2, a1 = std::min(a0 + K2, t1);
      {  // forward recompute of the sub-segment, keeping the state before each iteration and its forces
        Range r2("ses3d exact recompute");
        rc = load_wave2(h, j == 0 ? h->ex_ckpts[sg] : h->ex_ckpts2[j - 1], a0);
        if (rc) return rc;
        for (int t = a0 + 1; t <= a1; ++t) {
          float *slot = h->ex_slots[t - a0 - 1];
          CK(h, cudaMemcpyAsync(slot + nsl, h->d_v2, nv * sizeof(float), cudaMemcpyDeviceToDevice, h->st));
          rc = launch_iteration(h, w, 0, nullptr, false, slot + nsl + nv, slot);
          if (rc) return rc;
        }
      }
      for (int t = a1; t > a0; --t) {  // backward iterations a1 .. a0 + 1
        const float *slot = h->ex_slots[t - a0 - 1];
        a.fstate = slot; a.fv = slot + nsl; a.fg = slot + nsl + nv;
        CK(h, launch_adjoint_node1(h->c, p, a, h->st));
        CK(h, launch_adjoint_element(h->cfg.is_diss, h->c, p, a, h->st));
        if (h->fseis.n)
          CK(h, launch_inject(h->c, h->d_af, h->fseis.groups, h->fseis.n, h->fseis.delta, h->fseis.stf,
                              h->fseis.mask, h->d_ait, h->st));
        CK(h, launch_adjoint_node2(h->c, a, h->st));
        h->launches += h->fseis.n ? 4 : 3;
      }
    }
  }
  CK(h, cudaStreamSynchronize(h->st));
  rc = check_device_error(h);
  if (rc) return rc;
  h->ex_done = true;
  return SES3D_OK;
}

int ses3d_gpu_exact_gradient(ses3d_gpu *h, int which, double *out, int device) {
  if (!h) return SES3D_E_CONFIG;
  if (which < 0 || which > 6 || !out) return fail(h, SES3D_E_CONFIG, "which must be 0..6 (rhoinv, mu, lambda, A, B, C, Q)");
  if (!h->ex_done) return fail(h, SES3D_E_STATE, "run ses3d_gpu_exact_backward first");
  if (which == 6 && !h->cfg.is_diss) return fail(h, SES3D_E_CONFIG, "Q is a model record only with attenuation");
  const long long N = h->geo.N;
  double *dst = out, *tmp = nullptr;
  if (!device) {
    CK(h, dalloc(&tmp, (size_t)N));
    dst = tmp;
  }
  float sD = h->cfg.D_p[0];
  sD = sD + h->cfg.D_p[1];
  sD = sD + h->cfg.D_p[2];
  Ptrs p = make_ptrs(h);
  cudaError_t e = launch_adjoint_model_gradient(h->c, p, h->d_egmat, h->d_egimm, which, h->cfg.is_diss, (double)sD,
                                                h->d_tab + h->o_z, h->d_tab + h->o_sin, h->d_tab + h->o_w, dst, h->st);
  if (e == cudaSuccess && !device) e = cudaMemcpyAsync(out, tmp, N * sizeof(double), cudaMemcpyDeviceToHost, h->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
  dfree(tmp);
  if (e != cudaSuccess) return cuda_fail(h, e, "exact_gradient");
  ++h->launches;
  return SES3D_OK;
}

int ses3d_gpu_exact_get_field(ses3d_gpu *h, int event, int field, float *out) {
  if (!h) return SES3D_E_CONFIG;
  if (!out) return fail(h, SES3D_E_CONFIG, "null output");
  if (!h->d_astate) return fail(h, SES3D_E_STATE, "enable the exact adjoint first (ses3d_gpu_exact_adjoint)");
  if (field == SES3D_FIELD_MM_GLOBAL) return fail(h, SES3D_E_CONFIG, "MM_global is not part of the adjoint state");
  return field_io(h, event, field, out, nullptr, true);
}

int ses3d_gpu_exact_set_field(ses3d_gpu *h, int event, int field, const float *in) {
  if (!h) return SES3D_E_CONFIG;
  if (!in) return fail(h, SES3D_E_CONFIG, "null input");
  if (!h->d_astate) return fail(h, SES3D_E_STATE, "enable the exact adjoint first (ses3d_gpu_exact_adjoint)");
  if (field == SES3D_FIELD_MM_GLOBAL) return fail(h, SES3D_E_CONFIG, "MM_global is not part of the adjoint state");
  if (field >= SES3D_FIELD_DXUX && field <= SES3D_FIELD_DZUY) h->ex_zero_d = false;
  return field_io(h, event, field, nullptr, in, true);
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// Allocation-free iterations over a caller-owned wavefield (ses3d_gpu_step_external).
// The element forces, scratch between k_element and k_node, live in this fixed array;
// each handle looks up its device address on its first external call (the handle was
// created on that device, after any earlier reset of it) and hands it to the kernels.
// ---------------------------------------------------------------------------------------
namespace {
constexpr size_t kStaticForceFloats = (size_t)8 << 20;  // 8,388,608 floats = 32 MiB
static __device__ __align__(256) float g_static_forces[kStaticForceFloats];
}  // namespace

extern "C" int ses3d_gpu_step_external(ses3d_gpu *h, float *state, float *v, int n) {
  if (!h) return SES3D_E_CONFIG;
  if (!state || !v) return fail(h, SES3D_E_CONFIG, "null state or velocity buffer");
  if (reinterpret_cast<uintptr_t>(state) % 16 != 0) return fail(h, SES3D_E_CONFIG, "state buffer must be 16-byte aligned");
  if (n < 0) return fail(h, SES3D_E_CONFIG, "n must be >= 0");
  if (!h->model_set) return fail(h, SES3D_E_STATE, "set_model must be called before stepping");
  if (h->mode_flag != 0) return fail(h, SES3D_E_CONFIG, "the external-wavefield step runs plain forward runs only");
  if (!h->external_stepped && h->it > 0)
    return fail(h, SES3D_E_STATE, "this handle already stepped its own wavefield (ses3d_gpu_step)");
  const size_t need = (size_t)h->cfg.n_events * 3 * (size_t)h->geo.N;
  if (need > kStaticForceFloats) {
    char msg[256];
    std::snprintf(msg, sizeof(msg),
                  "run needs %zu element-force floats (n_events x 3 x %lld GLL points); the fixed array holds %zu "
                  "(32 MiB)",
                  need, (long long)h->geo.N, kStaticForceFloats);
    return fail(h, SES3D_E_CONFIG, msg);
  }
  int dev = -1;
  CK(h, cudaGetDevice(&dev));
  if (dev != h->device) return fail(h, SES3D_E_CONFIG, "the handle's device must be current");
  if (!h->ext_forces) {
    void *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_static_forces);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaGetSymbolAddress(g_static_forces)");
    if (!ptr) return fail(h, SES3D_E_CUDA, "cudaGetSymbolAddress(g_static_forces) returned no address");
    h->ext_forces = static_cast<float *>(ptr);
  }
  float *forces = h->ext_forces;
  h->external_stepped = true;
  if (h->ext_mirrors_stale && !h->c.lean) {  // lean calls left the mirrors outside the PML behind
    CK(h, launch_sync_mirrors(h->c, state, h->st));
    ++h->launches;
    h->ext_mirrors_stale = false;
  }
  Ptrs p = make_ptrs(h);
  p.state = state;
  p.v = v;
  p.f = forces;
  int done = 0;
  for (; done < n && h->it < h->cfg.nt; ++done) {
    if (h->R > 0) {
      CK(h, launch_receivers(h->c, v, h->d_rec_elem, h->d_rec_ev, h->d_rec_w, h->d_seis, h->R, h->d_it, h->st));
      ++h->launches;
    }
    CK(h, launch_element(h->cfg.is_diss, 0, h->epb, h->shape, h->c, p, h->st));
    ++h->launches;
    if (h->fset[0].n) {
      const ForceSet &F = h->fset[0];
      CK(h, launch_inject(h->c, forces, F.groups, F.n, F.delta, F.stf, F.mask, h->d_it, h->st));
      ++h->launches;
    }
    CK(h, launch_node(h->node_block, h->c, p, h->st));
    ++h->launches;
    h->it += 1;
  }
  if (done > 0 && h->c.lean) h->ext_mirrors_stale = true;
  CK(h, cudaStreamSynchronize(h->st));
  return check_device_error(h);
}

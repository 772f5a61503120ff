// driver.cpp -- ses3d_gpu_main: the reference program flow (SOURCE/ses3d_main.f90:8-205) on
// libses3d_gpu.so. Run from the MAIN directory of a SES3D tree, like the reference
// (`mpirun -n 1 ./ses3d.exe`, MAIN/job_run_ses3d:7): it reads ../INPUT/{event_list,
// event_<id>,setup,relax,stf,recfile_<id>}, ../MODELS/MODELS/{boxfile,<field>0} and, for
// adjoint runs, ../ADJOINT/<id>/{ad_srcfile,ad_src_<k>} and the forward fields in ffd; it
// writes seismograms, snapshots, forward fields, saving_vector and grad_* kernels in the
// reference layouts (SOURCE/ses3d_output.f90).
//
// A boxfile of several processor boxes (px, py, pz > 1) is run as one mesh on the GPU:
// the per-rank model files are stitched on input, and every per-rank output (snapshots
// v?_<rank>_<it>, forward fields <name>_<rank>, saving_vector_<rank>, grad_*_<rank>) is
// split back out, padded to the reference build's array extents nx_max, ny_max, nz_max
// (--max-elements; default: the largest box). Seismograms are written once per receiver.
//
//   ses3d_gpu_main [--main DIR] [--pml N] [--grad-q] [--max-elements NX NY NZ]
//                  [--stitch-model OUTDIR]
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ses3d_gpu.h"
#include "formats.hpp"

using namespace ses3d;

namespace {

const char *kRecordNames[9] = {"vx", "vy", "vz", "exx", "eyy", "ezz", "exy", "exz", "eyz"};
const char *kKernelNames[4] = {"grad_rho", "grad_cp", "grad_csh", "grad_csv"};

int die(const std::string &msg) {
  std::fprintf(stderr, "ses3d_gpu_main: %s\n", msg.c_str());
  return 1;
}

int api(int rc, ses3d_gpu *h, const char *what) {
  if (rc < 0) std::fprintf(stderr, "ses3d_gpu_main: %s failed (%d): %s\n", what, rc, ses3d_gpu_last_error(h));
  return rc;
}

std::string join(const std::string &main, const std::string &rel) {
  if (!rel.empty() && rel[0] == '/') return rel;
  return main + "/" + rel;
}

std::string trimmed(const std::string &s) {
  size_t b = s.find_first_not_of(' '), e = s.find_last_not_of(' ');
  return b == std::string::npos ? "" : s.substr(b, e - b + 1);
}

struct Args {
  std::string main = ".";
  int pml = 2;  // the reference's compile-time default (SOURCE/ses3d_modules.f90:21)
  int grad_q = 0;
  int max_el[3] = {-1, -1, -1};  // nx_max, ny_max, nz_max of the reference build
  std::string stitch_out;        // write the stitched single-box model there and stop
};

const char *kModelNames[7] = {"rhoinv", "mu", "lambda", "A", "B", "C", "Q"};

// Boxfile -> decomposition with the build's array extents.
bool load_decomposition(const Args &a, Decomposition &dec, std::string &err) {
  int px, py, pz;
  std::vector<BoxEntry> boxes;
  if (!read_boxfile(join(a.main, "../MODELS/MODELS/boxfile"), px, py, pz, boxes, err)) return false;
  if (!make_decomposition(boxes, px, py, pz, dec, err)) return false;
  if (a.max_el[0] >= 0) {
    if (a.max_el[0] < dec.pad_x || a.max_el[1] < dec.pad_y || a.max_el[2] < dec.pad_z) {
      err = "--max-elements smaller than a processor box";
      return false;
    }
    dec.pad_x = a.max_el[0]; dec.pad_y = a.max_el[1]; dec.pad_z = a.max_el[2];
  }
  return true;
}

// The union of the boxes as one box (physical bounds from the boxfile).
BoxEntry union_box(const Decomposition &dec) {
  BoxEntry u = dec.boxes[0];
  for (const BoxEntry &b : dec.boxes) {
    u.xmin = std::min(u.xmin, b.xmin); u.xmax = std::max(u.xmax, b.xmax);
    u.ymin = std::min(u.ymin, b.ymin); u.ymax = std::max(u.ymax, b.ymax);
    u.zmin = std::min(u.zmin, b.zmin); u.zmax = std::max(u.zmax, b.zmax);
  }
  u.index = 1; u.mx = u.my = u.mz = 1;
  u.nx_min = 0; u.nx_max = dec.ex - 1; u.ny_min = 0; u.ny_max = dec.ey - 1; u.nz_min = 0; u.nz_max = dec.ez - 1;
  return u;
}

// MODELS/MODELS/<name><rank> of every box (SOURCE/ses3d_input.f90:472-499), stitched.
bool read_stitched_model(const Args &a, const Decomposition &dec, int k, std::vector<float> &out, std::string &err) {
  out.assign(dec.global_points(), 0.0f);
  for (size_t b = 0; b < dec.boxes.size(); ++b) {
    std::vector<std::vector<float>> recs;
    const std::string nm = std::string(kModelNames[k]) + std::to_string(dec.boxes[b].index - 1);
    if (!read_records(join(a.main, "../MODELS/MODELS/" + nm), recs, err)) return false;
    if (recs.empty() || recs[0].size() != dec.box_points(b, false)) {
      err = "model record " + nm + " does not hold " + std::to_string(dec.box_points(b, false)) + " values";
      return false;
    }
    dec.gather(b, recs[0].data(), false, out.data());
  }
  return true;
}

// One record per box: <prefix><rank><suffix>, padded to the build's extents.
bool write_split(const Decomposition &dec, const std::string &prefix, const std::string &suffix, const float *global,
                 bool append, std::string &err) {
  std::vector<float> local;
  for (size_t b = 0; b < dec.boxes.size(); ++b) {
    local.resize(dec.box_points(b, true));
    dec.scatter(b, global, true, local.data());
    if (!write_record(prefix + std::to_string(dec.boxes[b].index - 1) + suffix, local.data(), local.size(), append, err))
      return false;
  }
  return true;
}

// Stitched single-box copy of a multi-box model (boxfile + <name>0), no GPU needed.
int stitch_model(const Args &a) {
  std::string err;
  Decomposition dec;
  if (!load_decomposition(a, dec, err)) return die(err);
  SetupFile su;
  if (!read_setup(join(a.main, "../INPUT/setup"), su, err)) return die(err);
  make_dirs(a.stitch_out);
  for (int k = 0; k < 7; ++k) {
    if (k == 6 && !su.is_diss) continue;
    std::vector<float> g;
    if (!read_stitched_model(a, dec, k, g, err)) return die(err);
    if (!write_record(a.stitch_out + "/" + kModelNames[k] + "0", g.data(), g.size(), false, err)) return die(err);
  }
  if (!write_single_boxfile(a.stitch_out + "/boxfile", union_box(dec), err)) return die(err);
  std::printf("stitched %zu boxes into %d x %d x %d elements\n", dec.boxes.size(), dec.ex, dec.ey, dec.ez);
  return 0;
}

int run_event(const Args &a, const std::string &id) {
  const auto t_start = std::chrono::steady_clock::now();
  std::string err;
  const std::string in = join(a.main, "../INPUT/");
  // ---- ses3d_input (SOURCE/ses3d_input.f90:44-618)
  Decomposition dec;
  if (!load_decomposition(a, dec, err)) return die(err);
  const BoxEntry b = union_box(dec);
  EventFile ev;
  SetupFile su;
  float tau[3], D[3];
  if (!read_event(in + "event_" + id, ev, err) || !read_setup(in + "setup", su, err) || !read_relax(in + "relax", tau, D, err))
    return die(err);
  ses3d_config cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.nx = b.nx_max - b.nx_min; cfg.ny = b.ny_max - b.ny_min; cfg.nz = b.nz_max - b.nz_min;
  cfg.lpd = su.lpd; cfg.pml = a.pml; cfg.is_diss = su.is_diss; cfg.adjoint_flag = su.adjoint_flag;
  cfg.samp_ad = su.samp_ad; cfg.nt = ev.nt; cfg.n_events = 1; cfg.grad_variant = a.grad_q;
  cfg.dt = ev.dt;
  cfg.xmin = b.xmin; cfg.xmax = b.xmax; cfg.ymin = b.ymin; cfg.ymax = b.ymax; cfg.zmin = b.zmin; cfg.zmax = b.zmax;
  cfg.zmax_global = su.zmax;
  for (int k = 0; k < 3; ++k) { cfg.tau_p[k] = tau[k]; cfg.D_p[k] = D[k]; }
  const std::string ofd = join(a.main, trimmed(ev.ofd) + "/");
  const std::string ffd = join(a.main, trimmed(su.ffd) + "/" + id + "/");
  make_dirs(ofd);
  make_dirs(ffd);
  ses3d_gpu *h = nullptr;
  if (api(ses3d_gpu_create(&cfg, &h), nullptr, "create") < 0) return 1;
  const size_t N = dec.global_points();
  // model records (SOURCE/ses3d_input.f90:472-499), stitched over the processor boxes
  std::vector<std::vector<float>> model(7);
  for (int k = 0; k < 7; ++k) {
    if (k == 6 && !cfg.is_diss) continue;
    if (!read_stitched_model(a, dec, k, model[k], err)) return die(err);
  }
  if (api(ses3d_gpu_set_model(h, model[0].data(), model[1].data(), model[2].data(), model[3].data(), model[4].data(),
                              model[5].data(), cfg.is_diss ? model[6].data() : nullptr), h, "set_model") < 0)
    return 1;
  model.clear();
  Receivers rec;
  std::vector<int> kept;
  int nr = 0;
  const float pi = 3.1415926535898f;
  if (cfg.adjoint_flag <= 1) {
    std::vector<float> so;
    if (!read_stf(in + "stf", cfg.nt, so, err)) return die(err);
    int is_src = 0;
    if (api(ses3d_gpu_set_source(h, 0, ev.xxs, ev.yys, ev.zzs, ev.source_type, ev.mom, so.data(), &is_src), h,
            "set_source") < 0)
      return 1;
    if (!is_src) std::fprintf(stderr, "ses3d_gpu_main: source not located in this processor box\n");
    if (!read_recfile(in + "recfile_" + id, rec, err)) return die(err);
    kept.resize(rec.names.size() + 1);
    if (api(ses3d_gpu_set_receivers(h, 0, (int)rec.names.size(), rec.loc.data(), &nr, kept.data()), h,
            "set_receivers") < 0)
      return 1;
  } else {
    // forward fields, read as the reference reads them back (SOURCE/ses3d_output.f90:172-267)
    std::vector<int> sv;
    if (!read_saving_vector(ffd + "saving_vector_" + std::to_string(dec.boxes[0].index - 1), cfg.nt, sv, err))
      return die(err);
    // per box and field all records of that file; stitched one record at a time
    std::vector<std::vector<std::vector<std::vector<float>>>> fields(dec.boxes.size(),
                                                                     std::vector<std::vector<std::vector<float>>>(9));
    size_t nrec = 0;
    for (size_t bx = 0; bx < dec.boxes.size(); ++bx)
      for (int f = 0; f < 9; ++f) {
        const std::string fn = ffd + kRecordNames[f] + "_" + std::to_string(dec.boxes[bx].index - 1);
        if (!read_records(fn, fields[bx][f], err)) return die(err);
        if (bx == 0 && f == 0) nrec = fields[0][0].size();
        if (fields[bx][f].size() != nrec) return die("inconsistent forward-field records in " + fn);
        for (const std::vector<float> &rr : fields[bx][f])
          if (rr.size() != dec.box_points(bx, true) && rr.size() != dec.box_points(bx, false))
            return die("forward-field record size in " + fn + " fits neither the box nor --max-elements");
      }
    std::vector<float> one(9 * N);
    for (size_t r = 0; r < nrec; ++r) {
      for (size_t bx = 0; bx < dec.boxes.size(); ++bx)
        for (int f = 0; f < 9; ++f) {
          const std::vector<float> &rr = fields[bx][f][r];
          dec.gather(bx, rr.data(), rr.size() == dec.box_points(bx, true), &one[(size_t)f * N]);
        }
      if (api(ses3d_gpu_put_record(h, 0, (int)r, one.data()), h, "put_record") < 0) return 1;
    }
    fields.clear();
    if (api(ses3d_gpu_set_saving_vector(h, sv.data()), h, "set_saving_vector") < 0) return 1;
    std::vector<float> loc;
    const std::string adir = join(a.main, "../ADJOINT/" + id + "/");
    if (!read_ad_srcfile(adir + "ad_srcfile", loc, err)) return die(err);
    const int nad = (int)loc.size() / 3;
    std::vector<float> stf((size_t)nad * 3 * cfg.nt);
    for (int k = 0; k < nad; ++k) {
      std::vector<float> s3;
      if (!read_ad_src(adir + "ad_src_" + std::to_string(k + 1), cfg.nt, s3, err)) return die(err);
      std::memcpy(&stf[(size_t)k * 3 * cfg.nt], s3.data(), s3.size() * sizeof(float));
    }
    int nin = 0;
    if (api(ses3d_gpu_set_adjoint_sources(h, 0, nad, loc.data(), stf.data(), &nin), h, "set_adjoint_sources") < 0)
      return 1;
  }
  // plain iterations replay from CUDA graphs; plain forward runs step lean (their outputs,
  // seismograms and velocity snapshots, do not depend on the displacement gradients)
  if (api(ses3d_gpu_use_graph(h, 1, 10), h, "use_graph") < 0) return 1;
  if (cfg.adjoint_flag == 0 && api(ses3d_gpu_set_lean(h, 1), h, "set_lean") < 0) return 1;
  // ---- time loop (SOURCE/ses3d_main.f90:95-178) with ses3d_output every ssamp iterations
  std::vector<float> sx((size_t)nr * cfg.nt), sy(sx.size()), sz(sx.size()), snap(N);
  const float src_deg[3] = {ev.xxs * pi / 180.0f * 180.0f / pi, ev.yys * pi / 180.0f * 180.0f / pi, ev.zzs};
  auto write_seismograms = [&]() -> bool {
    if (nr == 0 || cfg.adjoint_flag == 2) return true;
    if (api(ses3d_gpu_get_seismograms(h, 0, sx.data(), sy.data(), sz.data()), h, "get_seismograms") < 0) return false;
    std::vector<float> tx(cfg.nt), ty(cfg.nt), tz(cfg.nt);
    for (int r = 0; r < nr; ++r) {
      for (int t = 0; t < cfg.nt; ++t) {
        tx[t] = sx[(size_t)t * nr + r]; ty[t] = sy[(size_t)t * nr + r]; tz[t] = sz[(size_t)t * nr + r];
      }
      const int g = kept[r];
      const float rl[3] = {rec.loc[3 * g] * pi / 180.0f * 180.0f / pi, rec.loc[3 * g + 1] * pi / 180.0f * 180.0f / pi,
                           rec.loc[3 * g + 2]};
      if (!write_seismogram_files(ofd, rec.names[g], tx.data(), ty.data(), tz.data(), cfg.nt, cfg.dt, rl, src_deg, err)) {
        die(err);
        return false;
      }
    }
    return true;
  };
  auto write_snapshot = [&](int it) -> bool {
    if (ev.output_displacement != 1) return true;
    const char *nm[3] = {"vx_", "vy_", "vz_"};
    for (int c = 0; c < 3; ++c) {
      if (api(ses3d_gpu_get_field(h, 0, SES3D_FIELD_VX + c, snap.data()), h, "get_field") < 0) return false;
      if (!write_split(dec, ofd + nm[c], "_" + std::to_string(it), snap.data(), false, err)) { die(err); return false; }
    }
    return true;
  };
  // ses3d_output runs at every iteration with mod(it, ssamp) == 0 and once more after the loop
  // (it = nt); its snapshot is the velocity gathered at the start of that iteration.
  std::vector<int> outputs;
  const int ssamp = ev.ssamp > 0 ? ev.ssamp : cfg.nt + 1;
  for (int o = ssamp; o <= cfg.nt; o += ssamp) outputs.push_back(o);
  if (outputs.empty() || outputs.back() != cfg.nt) outputs.push_back(cfg.nt);
  int it = 0;
  for (int o : outputs) {
    if (o - 1 > it) {
      if (api(ses3d_gpu_step(h, o - 1 - it), h, "step") < 0) return 1;
      it = o - 1;
    }
    if (!write_snapshot(o)) return 1;
    if (api(ses3d_gpu_step(h, 1), h, "step") < 0) return 1;
    it = o;
    float vmax = 0.f;
    if (ses3d_gpu_vmax(h, &vmax) == SES3D_E_NAN) return die("non-finite velocity at iteration " + std::to_string(it));
    if (o != cfg.nt && !write_seismograms()) return 1;
  }
  // ---- final ses3d_output(nt) (SOURCE/ses3d_main.f90:180, SOURCE/ses3d_output.f90:270-453)
  if (!write_seismograms()) return 1;
  if (cfg.adjoint_flag == 2) {
    std::vector<double> kd(N);
    std::vector<float> kf(N);
    for (int k = 0; k < 4; ++k) {
      if (api(ses3d_gpu_get_kernel(h, 0, SES3D_KERNEL_RHO + k, kd.data()), h, "get_kernel") < 0) return 1;
      for (size_t q = 0; q < N; ++q) kf[q] = (float)kd[q];
      if (!write_split(dec, ofd + kKernelNames[k] + "_", "", kf.data(), false, err)) return die(err);
    }
  }
  if (cfg.adjoint_flag == 1) {
    std::vector<int> sv(cfg.nt);
    ses3d_gpu_get_saving_vector(h, sv.data());
    for (const BoxEntry &bx : dec.boxes)  // every rank writes the same vector
      if (!write_saving_vector(ffd + "saving_vector_" + std::to_string(bx.index - 1), sv, err)) return die(err);
    const int nrec = ses3d_gpu_record_count(h, 0);
    std::vector<float> one(9 * N);
    for (int r = 0; r < nrec; ++r) {  // ses3d_store records (SOURCE/ses3d_output.f90:138-162)
      if (api(ses3d_gpu_get_record(h, 0, r, one.data()), h, "get_record") < 0) return 1;
      for (int f = 0; f < 9; ++f)
        if (!write_split(dec, ffd + kRecordNames[f] + "_", "", &one[(size_t)f * N], r > 0, err)) return die(err);
    }
  }
  // one structured line per event (the reference logs a line per step instead)
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  std::printf("{\"event\": \"%s\", \"iterations\": %d, \"receivers\": %d, \"boxes\": %zu, \"gll_points\": %zu, "
              "\"launches\": %lld, \"seconds\": %.6f, \"gll_point_steps_per_s\": %.6e}\n",
              id.c_str(), cfg.nt, nr, dec.boxes.size(), N, (long long)ses3d_gpu_launch_count(h), secs,
              secs > 0 ? (double)N * cfg.nt / secs : 0.0);
  ses3d_gpu_destroy(h);
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  Args a;
  for (int k = 1; k < argc; ++k) {
    std::string s = argv[k];
    auto val = [&](const char *name) -> std::string {
      if (k + 1 >= argc) { std::fprintf(stderr, "missing value for %s\n", name); std::exit(2); }
      return argv[++k];
    };
    if (s == "--main") a.main = val("--main");
    else if (s == "--pml") a.pml = std::atoi(val("--pml").c_str());
    else if (s == "--grad-q") a.grad_q = 1;
    else if (s == "--max-elements") {
      for (int q = 0; q < 3; ++q) a.max_el[q] = std::atoi(val("--max-elements").c_str());
    } else if (s == "--stitch-model") a.stitch_out = val("--stitch-model");
    else if (s == "-h" || s == "--help") {
      std::printf("usage: ses3d_gpu_main [--main DIR] [--pml N] [--grad-q] [--max-elements NX NY NZ] "
                  "[--stitch-model OUTDIR]\n");
      return 0;
    } else {
      std::fprintf(stderr, "unknown argument %s\n", s.c_str());
      return 2;
    }
  }
  if (!a.stitch_out.empty()) return stitch_model(a);
  std::string err;
  std::vector<std::string> ids;
  if (!read_event_list(join(a.main, "../INPUT/event_list"), ids, err)) return die(err);
  for (const std::string &id : ids) {
    int rc = run_event(a, id);
    if (rc) return rc;
  }
  return 0;
}

// formats.hpp -- the SES3D input/output files, read and written as the reference does.
//
// ASCII inputs are line-positional Fortran list-directed reads: every READ consumes one
// line and takes its leading tokens; REAL(4) values are converted with strtof as
// libgfortran does. Binary fields are gfortran sequential-unformatted records (4-byte
// little-endian length, payload, length). Seismograms use gfortran's list-directed REAL(4)
// layout (9 significant digits, exact round trip).
#pragma once
#include <string>
#include <vector>

namespace ses3d {

class LineReader {
 public:
  bool open(const std::string &path);
  void skip(int n = 1);
  std::vector<std::string> values(int n);  // next n tokens, blank lines skipped
  int integer();
  float real();
  std::string token();
  std::string text();  // '(A1000)' read: the whole line, trailing blanks removed
  bool ok() const { return ok_; }
  const std::string &error() const { return err_; }

 private:
  std::vector<std::string> lines_;
  size_t pos_ = 0;
  bool ok_ = true;
  std::string err_, path_;
  std::string next_line();
};

struct SetupFile {
  float xmin = 0, xmax = 0, ymin = 0, ymax = 0, zmin = 0, zmax = 0;  // degrees, m
  int is_diss = 0, model_type = 0, nx_global = 0, ny_global = 0, nz_global = 0, lpd = 4, px = 1, py = 1, pz = 1;
  int adjoint_flag = 0, samp_ad = 1;
  std::string ffd;
};

struct EventFile {
  int nt = 0;
  float dt = 0, xxs = 0, yys = 0, zzs = 0;
  int source_type = 10;
  float mom[6] = {0, 0, 0, 0, 0, 0};
  std::string ofd;
  int ssamp = 1, output_displacement = 0;
};

struct BoxEntry {
  int index = 0, mx = 1, my = 1, mz = 1;
  int nx_min = 0, nx_max = 0, ny_min = 0, ny_max = 0, nz_min = 0, nz_max = 0;
  float xmin = 0, xmax = 0, ymin = 0, ymax = 0, zmin = 0, zmax = 0;
};

// Processor-box decomposition of a boxfile (SOURCE/ses3d_input.f90:44-170, boxes as
// MODELS/SOURCE/generate_models.f90:200-283 writes them): box (mx, my, mz) holds the
// global elements nx_min + mx - 1 .. nx_max + mx - 1 (likewise in y; in z the boxfile
// counts upward while element k counts down from the top), so boxes are element-disjoint
// and tile the mesh. Per-box arrays are the reference's F-order
// (i, j, k, in, jn, kn) with element index fastest; `pad` gives the compile-time array
// extents nx_max, ny_max, nz_max of the reference build (0:nx_max etc.), which its
// snapshot, forward-field and kernel files are written with.
struct Decomposition {
  int ex = 0, ey = 0, ez = 0;                     // global element counts
  std::vector<BoxEntry> boxes;
  std::vector<int> ox, oy, oz;                    // global element offset of each box
  int pad_x = 0, pad_y = 0, pad_z = 0;            // nx_max, ny_max, nz_max (>= every box's nx, ny, nz)
  size_t global_points() const { return (size_t)125 * ex * ey * ez; }
  size_t box_points(size_t b, bool padded) const;
  // local (exact or padded) -> global, and global -> local (padding left zero)
  void gather(size_t b, const float *local, bool padded, float *global) const;
  void scatter(size_t b, const float *global, bool padded, float *local) const;
};
bool make_decomposition(const std::vector<BoxEntry> &boxes, int px, int py, int pz, Decomposition &d,
                        std::string &err);

struct Receivers {
  std::vector<std::string> names;  // 12 characters, blank padded
  std::vector<float> loc;          // 3 per receiver
};

bool read_setup(const std::string &path, SetupFile &s, std::string &err);
bool read_event(const std::string &path, EventFile &e, std::string &err);
bool read_relax(const std::string &path, float tau[3], float D[3], std::string &err);
bool read_event_list(const std::string &path, std::vector<std::string> &ids, std::string &err);
bool read_stf(const std::string &path, int nt, std::vector<float> &so, std::string &err);
bool read_recfile(const std::string &path, Receivers &r, std::string &err);
bool read_boxfile(const std::string &path, int &px, int &py, int &pz, std::vector<BoxEntry> &boxes, std::string &err);
bool read_ad_srcfile(const std::string &path, std::vector<float> &loc, std::string &err);
bool read_ad_src(const std::string &path, int nt, std::vector<float> &stf3, std::string &err);  // [3][nt]
bool read_saving_vector(const std::string &path, int nt, std::vector<int> &sv, std::string &err);

// Fortran sequential-unformatted records of FP32 payload.
bool read_records(const std::string &path, std::vector<std::vector<float>> &recs, std::string &err);
bool write_record(const std::string &path, const float *data, size_t n, bool append, std::string &err);

// gfortran list-directed REAL(4) / default INTEGER fields.
std::string fmt_real(float v);
std::string fmt_int(long v);

bool write_seismogram_files(const std::string &ofd, const std::string &name12, const float *sx, const float *sy,
                            const float *sz, int nt, float dt, const float recloc_deg[3], const float src_deg[3],
                            std::string &err);
bool write_saving_vector(const std::string &path, const std::vector<int> &sv, std::string &err);
bool write_single_boxfile(const std::string &path, const BoxEntry &b, std::string &err);
bool make_dirs(const std::string &path);

}  // namespace ses3d

// formats.cpp -- SES3D file formats (see formats.hpp).
#include "formats.hpp"

#include <sys/stat.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

namespace ses3d {

namespace {
std::vector<std::string> split_tokens(const std::string &line) {
  // list-directed separators: blanks, tabs and commas; a slash ends the record
  std::vector<std::string> out;
  std::string cur;
  for (char c : line) {
    if (c == '/' && cur.empty() && out.empty()) break;
    if (c == ' ' || c == '\t' || c == ',' || c == '\r') {
      if (!cur.empty()) { out.push_back(cur); cur.clear(); }
    } else if (c == '!') {
      break;
    } else {
      cur.push_back(c);
    }
  }
  if (!cur.empty()) out.push_back(cur);
  return out;
}

float to_real(const std::string &tok) {
  std::string t = tok;
  for (char &c : t)
    if (c == 'd' || c == 'D') c = 'e';
  return std::strtof(t.c_str(), nullptr);
}
}  // namespace

bool LineReader::open(const std::string &path) {
  path_ = path;
  std::ifstream f(path);
  if (!f) { ok_ = false; err_ = "cannot open " + path; return false; }
  std::string line;
  while (std::getline(f, line)) lines_.push_back(line);
  return true;
}

std::string LineReader::next_line() {
  if (pos_ >= lines_.size()) {
    if (ok_) err_ = "unexpected end of file in " + path_;
    ok_ = false;
    return "";
  }
  return lines_[pos_++];
}

void LineReader::skip(int n) {
  for (int k = 0; k < n; ++k) next_line();
}

std::vector<std::string> LineReader::values(int n) {
  std::vector<std::string> out;
  while ((int)out.size() < n && ok_) {
    std::vector<std::string> t = split_tokens(next_line());
    for (size_t k = 0; k < t.size() && (int)out.size() < n; ++k) out.push_back(t[k]);
  }
  while ((int)out.size() < n) out.push_back("0");
  return out;
}

int LineReader::integer() { return std::atoi(values(1)[0].c_str()); }
float LineReader::real() { return to_real(values(1)[0]); }
std::string LineReader::token() { return values(1)[0]; }
std::string LineReader::text() {
  std::string s = next_line();
  while (!s.empty() && (s.back() == ' ' || s.back() == '\r' || s.back() == '\t')) s.pop_back();
  size_t b = s.find_first_not_of(' ');
  return b == std::string::npos ? "" : s.substr(b);
}

// SOURCE/ses3d_input.f90:264-310
bool read_setup(const std::string &path, SetupFile &s, std::string &err) {
  LineReader r;
  if (!r.open(path)) { err = r.error(); return false; }
  r.skip();
  s.xmin = r.real(); s.xmax = r.real(); s.ymin = r.real(); s.ymax = r.real(); s.zmin = r.real(); s.zmax = r.real();
  s.is_diss = r.integer(); s.model_type = r.integer();
  r.skip();
  s.nx_global = r.integer(); s.ny_global = r.integer(); s.nz_global = r.integer(); s.lpd = r.integer();
  s.px = r.integer(); s.py = r.integer(); s.pz = r.integer();
  r.skip();
  s.adjoint_flag = r.integer(); s.samp_ad = r.integer();
  s.ffd = r.text();
  if (!r.ok()) { err = r.error(); return false; }
  return true;
}

// SOURCE/ses3d_input.f90:201-249
bool read_event(const std::string &path, EventFile &e, std::string &err) {
  LineReader r;
  if (!r.open(path)) { err = r.error(); return false; }
  r.skip();
  e.nt = r.integer(); e.dt = r.real();
  r.skip();
  e.xxs = r.real(); e.yys = r.real(); e.zzs = r.real();
  e.source_type = r.integer();
  for (int k = 0; k < 6; ++k) e.mom[k] = r.real();
  r.skip();
  e.ofd = r.text();
  r.skip();
  e.ssamp = r.integer(); e.output_displacement = r.integer();
  if (!r.ok()) { err = r.error(); return false; }
  return true;
}

// SOURCE/ses3d_input.f90:338-350
bool read_relax(const std::string &path, float tau[3], float D[3], std::string &err) {
  LineReader r;
  if (!r.open(path)) { err = r.error(); return false; }
  r.skip();
  for (int k = 0; k < 3; ++k) tau[k] = r.real();
  r.skip();
  for (int k = 0; k < 3; ++k) D[k] = r.real();
  if (!r.ok()) { err = r.error(); return false; }
  return true;
}

// SOURCE/ses3d_main.f90:35-43
bool read_event_list(const std::string &path, std::vector<std::string> &ids, std::string &err) {
  LineReader r;
  if (!r.open(path)) { err = r.error(); return false; }
  int n = r.integer();
  ids.clear();
  for (int k = 0; k < n; ++k) ids.push_back(r.token());
  if (!r.ok()) { err = r.error(); return false; }
  return true;
}

// SOURCE/ses3d_input.f90:419-428: four lines skipped, then nt samples
bool read_stf(const std::string &path, int nt, std::vector<float> &so, std::string &err) {
  LineReader r;
  if (!r.open(path)) { err = r.error(); return false; }
  r.skip(4);
  so.resize(nt);
  for (int k = 0; k < nt; ++k) so[k] = r.real();
  if (!r.ok()) { err = r.error(); return false; }
  return true;
}

// SOURCE/ses3d_input.f90:533-538; names are character(len=12)
bool read_recfile(const std::string &path, Receivers &rec, std::string &err) {
  LineReader r;
  if (!r.open(path)) { err = r.error(); return false; }
  int n = r.integer();
  rec.names.clear();
  rec.loc.clear();
  for (int k = 0; k < n; ++k) {
    std::string nm = r.token();
    nm = nm.substr(0, 12);
    nm.resize(12, ' ');
    rec.names.push_back(nm);
    std::vector<std::string> v = r.values(3);
    for (int c = 0; c < 3; ++c) rec.loc.push_back(to_real(v[c]));
  }
  if (!r.ok()) { err = r.error(); return false; }
  return true;
}

// SOURCE/ses3d_input.f90:51-98
bool read_boxfile(const std::string &path, int &px, int &py, int &pz, std::vector<BoxEntry> &boxes,
                  std::string &err) {
  LineReader r;
  if (!r.open(path)) { err = r.error(); return false; }
  r.skip(14);
  int pp = r.integer();
  px = r.integer(); py = r.integer(); pz = r.integer();
  r.skip();
  boxes.clear();
  for (int k = 0; k < pp; ++k) {
    BoxEntry b;
    b.index = r.integer();
    std::vector<std::string> m = r.values(3);
    b.mx = std::atoi(m[0].c_str()); b.my = std::atoi(m[1].c_str()); b.mz = std::atoi(m[2].c_str());
    std::vector<std::string> a = r.values(2);
    b.nx_min = std::atoi(a[0].c_str()); b.nx_max = std::atoi(a[1].c_str());
    a = r.values(2);
    b.ny_min = std::atoi(a[0].c_str()); b.ny_max = std::atoi(a[1].c_str());
    a = r.values(2);
    b.nz_min = std::atoi(a[0].c_str()); b.nz_max = std::atoi(a[1].c_str());
    a = r.values(2);
    b.xmin = to_real(a[0]); b.xmax = to_real(a[1]);
    a = r.values(2);
    b.ymin = to_real(a[0]); b.ymax = to_real(a[1]);
    a = r.values(2);
    b.zmin = to_real(a[0]); b.zmax = to_real(a[1]);
    r.skip();
    boxes.push_back(b);
  }
  if (!r.ok()) { err = r.error(); return false; }
  return true;
}

bool make_decomposition(const std::vector<BoxEntry> &boxes, int px, int py, int pz, Decomposition &d,
                        std::string &err) {
  if (boxes.empty() || (size_t)px * py * pz != boxes.size()) {
    err = "boxfile: " + std::to_string(boxes.size()) + " boxes for px * py * pz = " + std::to_string(px * py * pz);
    return false;
  }
  d = Decomposition();
  d.boxes = boxes;
  for (const BoxEntry &b : boxes) {
    if (b.mx < 1 || b.mx > px || b.my < 1 || b.my > py || b.mz < 1 || b.mz > pz || b.nx_max < b.nx_min ||
        b.ny_max < b.ny_min || b.nz_max < b.nz_min) {
      err = "boxfile: inconsistent box " + std::to_string(b.index);
      return false;
    }
    d.ox.push_back(b.nx_min + b.mx - 1);
    d.oy.push_back(b.ny_min + b.my - 1);
    d.ex = std::max(d.ex, b.nx_max + b.mx);
    d.ey = std::max(d.ey, b.ny_max + b.my);
    d.ez = std::max(d.ez, b.nz_max + b.mz);
    d.pad_x = std::max(d.pad_x, b.nx_max - b.nx_min);
    d.pad_y = std::max(d.pad_y, b.ny_max - b.ny_min);
    d.pad_z = std::max(d.pad_z, b.nz_max - b.nz_min);
  }
  // z: the boxfile counts upward (box mz = 1 at the bottom, SOURCE/ses3d_init.f90:600-611),
  // element k downward from the top of each box (z = zmax - k dz, :238-242)
  for (const BoxEntry &b : boxes) d.oz.push_back(d.ez - (b.nz_max + b.mz));
  // every global element in exactly one box
  std::vector<unsigned char> cover((size_t)d.ex * d.ey * d.ez, 0);
  for (size_t q = 0; q < boxes.size(); ++q) {
    const BoxEntry &b = boxes[q];
    for (int k = 0; k <= b.nz_max - b.nz_min; ++k)
      for (int j = 0; j <= b.ny_max - b.ny_min; ++j)
        for (int i = 0; i <= b.nx_max - b.nx_min; ++i) {
          unsigned char &c = cover[(size_t)(d.ox[q] + i) + (size_t)d.ex * ((d.oy[q] + j) + (size_t)d.ey * (d.oz[q] + k))];
          if (c) { err = "boxfile: boxes overlap"; return false; }
          c = 1;
        }
  }
  for (unsigned char c : cover)
    if (!c) { err = "boxfile: boxes leave elements uncovered"; return false; }
  return true;
}

size_t Decomposition::box_points(size_t b, bool padded) const {
  const BoxEntry &x = boxes[b];
  const size_t lx = padded ? pad_x + 1 : x.nx_max - x.nx_min + 1, ly = padded ? pad_y + 1 : x.ny_max - x.ny_min + 1,
               lz = padded ? pad_z + 1 : x.nz_max - x.nz_min + 1;
  return 125 * lx * ly * lz;
}

namespace {
template <bool TO_GLOBAL>
void move_box(const Decomposition &d, size_t b, const float *src, bool padded, float *dst) {
  const BoxEntry &x = d.boxes[b];
  const int nx = x.nx_max - x.nx_min + 1, ny = x.ny_max - x.ny_min + 1, nz = x.nz_max - x.nz_min + 1;
  const size_t lx = padded ? d.pad_x + 1 : nx, ly = padded ? d.pad_y + 1 : ny, lz = padded ? d.pad_z + 1 : nz;
  for (int n = 0; n < 125; ++n)  // n = in + 5 jn + 25 kn, the slowest F-order index group
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j) {
        const size_t lrow = lx * (j + ly * (k + lz * (size_t)n));
        const size_t grow = (size_t)d.ox[b] + (size_t)d.ex * ((d.oy[b] + j) + (size_t)d.ey * ((d.oz[b] + k) + (size_t)d.ez * n));
        if (TO_GLOBAL) std::memcpy(dst + grow, src + lrow, (size_t)nx * sizeof(float));
        else std::memcpy(dst + lrow, src + grow, (size_t)nx * sizeof(float));
      }
}
}  // namespace

void Decomposition::gather(size_t b, const float *local, bool padded, float *global) const {
  move_box<true>(*this, b, local, padded, global);
}

void Decomposition::scatter(size_t b, const float *global, bool padded, float *local) const {
  std::fill(local, local + box_points(b, padded), 0.0f);
  move_box<false>(*this, b, global, padded, local);
}

// SOURCE/ses3d_input.f90:594-598
bool read_ad_srcfile(const std::string &path, std::vector<float> &loc, std::string &err) {
  LineReader r;
  if (!r.open(path)) { err = r.error(); return false; }
  int n = r.integer();
  loc.clear();
  for (int k = 0; k < n; ++k) {
    std::vector<std::string> v = r.values(3);
    for (int c = 0; c < 3; ++c) loc.push_back(to_real(v[c]));
  }
  if (!r.ok()) { err = r.error(); return false; }
  return true;
}

// SOURCE/ses3d_init.f90:479-490
bool read_ad_src(const std::string &path, int nt, std::vector<float> &stf3, std::string &err) {
  LineReader r;
  if (!r.open(path)) { err = r.error(); return false; }
  r.skip(4);
  stf3.assign((size_t)3 * nt, 0.f);
  for (int i = 0; i < nt; ++i) {
    std::vector<std::string> v = r.values(3);
    for (int c = 0; c < 3; ++c) stf3[(size_t)c * nt + i] = to_real(v[c]);
  }
  if (!r.ok()) { err = r.error(); return false; }
  return true;
}

// SOURCE/ses3d_input.f90:570-574
bool read_saving_vector(const std::string &path, int nt, std::vector<int> &sv, std::string &err) {
  LineReader r;
  if (!r.open(path)) { err = r.error(); return false; }
  sv.resize(nt);
  for (int k = 0; k < nt; ++k) sv[k] = r.integer();
  if (!r.ok()) { err = r.error(); return false; }
  return true;
}

bool read_records(const std::string &path, std::vector<std::vector<float>> &recs, std::string &err) {
  std::ifstream f(path, std::ios::binary);
  if (!f) { err = "cannot open " + path; return false; }
  recs.clear();
  while (true) {
    int32_t n1 = 0, n2 = 0;
    if (!f.read(reinterpret_cast<char *>(&n1), 4)) break;
    if (n1 < 0 || n1 % 4) { err = "corrupt record length in " + path; return false; }
    std::vector<float> v((size_t)n1 / 4);
    if (!f.read(reinterpret_cast<char *>(v.data()), n1) || !f.read(reinterpret_cast<char *>(&n2), 4) || n1 != n2) {
      err = "truncated record in " + path;
      return false;
    }
    recs.push_back(std::move(v));
  }
  return true;
}

bool write_record(const std::string &path, const float *data, size_t n, bool append, std::string &err) {
  std::ofstream f(path, std::ios::binary | (append ? std::ios::app : std::ios::trunc));
  if (!f) { err = "cannot write " + path; return false; }
  if (n * 4 > 0x7fffffffull) { err = "record too large for a 4-byte marker: " + path; return false; }
  int32_t m = (int32_t)(n * 4);
  f.write(reinterpret_cast<const char *>(&m), 4);
  f.write(reinterpret_cast<const char *>(data), (std::streamsize)(n * 4));
  f.write(reinterpret_cast<const char *>(&m), 4);
  return (bool)f;
}

std::string fmt_real(float vf) {
  const double v = vf;
  char body[64];
  auto pad = [](const std::string &s, size_t w) { return s.size() >= w ? s : std::string(w - s.size(), ' ') + s; };
  if (v == 0.0) return " " + pad("0.00000000", 12) + "    ";
  char s9[64];
  std::snprintf(s9, sizeof(s9), "%.9g", std::fabs(v));
  const double a9 = std::strtod(s9, nullptr);
  if (a9 >= 0.1 && a9 < 1e9) {
    char se[64];
    std::snprintf(se, sizeof(se), "%.8e", v);
    const int ex = std::atoi(std::strchr(se, 'e') + 1);
    int decimals = 8 - ex;
    if (decimals < 0) decimals = 0;
    std::snprintf(body, sizeof(body), "%.*f", decimals, v);
    return " " + pad(body, 12) + "    ";
  }
  std::snprintf(body, sizeof(body), "%.8E", v);
  std::string b(body);
  size_t epos = b.find('E');
  int ex = std::atoi(b.c_str() + epos + 1);
  char tail[16];
  std::snprintf(tail, sizeof(tail), "E%c%02d", ex < 0 ? '-' : '+', std::abs(ex));
  return " " + pad(b.substr(0, epos) + tail, 16);
}

std::string fmt_int(long v) {
  char b[32];
  std::snprintf(b, sizeof(b), " %11ld", v);
  return b;
}

// Boxfile of one processor box, in the layout generate_models.f90 writes
// (MODELS/SOURCE/generate_models.f90:285-330): 14 description lines, the process counts,
// then the box entry.
bool write_single_boxfile(const std::string &path, const BoxEntry &b, std::string &err) {
  std::ofstream f(path);
  if (!f) { err = "cannot write " + path; return false; }
  const char *desc[14] = {" - format description -", " total number of processes", " number of processes in x direction",
                          " number of processes in y direction", " number of processes in z direction",
                          " single index (npz-1)*py*px+(npy-1)*px+npx", " multi index (npx, npy, npz)",
                          " index boundaries x (x_min, x_max)", " index boundaries y (y_min, y_max)",
                          " index boundaries z (z_min, z_max)", " physical boundaries x", " physical boundaries y",
                          " phyiscal boundaries z", " -------------------"};
  for (const char *d : desc) f << d << "\n";
  f << fmt_int(1) << "\n" << fmt_int(1) << "\n" << fmt_int(1) << "\n" << fmt_int(1) << "\n";
  f << " -------------------\n";
  f << fmt_int(1) << "\n" << fmt_int(1) << fmt_int(1) << fmt_int(1) << "\n";
  f << fmt_int(b.nx_min) << fmt_int(b.nx_max) << "\n" << fmt_int(b.ny_min) << fmt_int(b.ny_max) << "\n";
  f << fmt_int(b.nz_min) << fmt_int(b.nz_max) << "\n";
  f << fmt_real(b.xmin) << fmt_real(b.xmax) << "\n" << fmt_real(b.ymin) << fmt_real(b.ymax) << "\n";
  f << fmt_real(b.zmin) << fmt_real(b.zmax) << "\n";
  f << " -------------------\n";
  return (bool)f;
}

// SOURCE/ses3d_output.f90:398-451
bool write_seismogram_files(const std::string &ofd, const std::string &name12, const float *sx, const float *sy,
                            const float *sz, int nt, float dt, const float recloc_deg[3], const float src_deg[3],
                            std::string &err) {
  const char *heads[3] = {"theta component seismograms", "phi component seismograms", "r component seismograms"};
  const char *ext[3] = {".x", ".y", ".z"};
  const float *data[3] = {sx, sy, sz};
  std::string nm = name12.substr(0, 12);
  nm.resize(12, ' ');
  for (int c = 0; c < 3; ++c) {
    std::ofstream f(ofd + nm + ext[c]);
    if (!f) { err = "cannot write " + ofd + nm + ext[c]; return false; }
    f << " " << heads[c] << "\n";
    f << " nt=" << fmt_int(nt) << "\n";
    f << " dt=" << fmt_real(dt) << "\n";
    f << " receiver location (colat [deg],lon [deg],depth [m])\n";
    f << " x=" << fmt_real(recloc_deg[0]) << " y=" << fmt_real(recloc_deg[1]) << " z=" << fmt_real(recloc_deg[2]) << "\n";
    f << " source location (colat [deg],lon [deg],depth [m])\n";
    f << " x=" << fmt_real(src_deg[0]) << " y=" << fmt_real(src_deg[1]) << " z=" << fmt_real(src_deg[2]) << "\n";
    for (int k = 0; k < nt; ++k) f << fmt_real(data[c][k]) << "\n";
  }
  return true;
}

// SOURCE/ses3d_output.f90:379-392
bool write_saving_vector(const std::string &path, const std::vector<int> &sv, std::string &err) {
  std::ofstream f(path);
  if (!f) { err = "cannot write " + path; return false; }
  for (int v : sv) f << fmt_int(v) << "\n";
  return true;
}

bool make_dirs(const std::string &path) {
  std::string cur;
  for (size_t k = 0; k < path.size(); ++k) {
    cur.push_back(path[k]);
    if (path[k] == '/' && cur.size() > 1) mkdir(cur.c_str(), 0755);
  }
  if (!cur.empty()) mkdir(cur.c_str(), 0755);
  struct stat st;
  return stat(path.c_str(), &st) == 0;
}

}  // namespace ses3d

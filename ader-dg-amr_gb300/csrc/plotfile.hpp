// AMReX plotfile format, host side: the files the reference writes for every
// conserved variable q, <data_dir>/tstep_<n>_q_<q>_plt, with the Np_s modal
// coefficients of U_w as components (Solver::PlotFile,
// Source/Core/Solver.h:922-968, through amrex::WriteMultiLevelPlotfile), and
// reads back for a restart (Solver::ReadPlotFile, Source/Core/Solver.h:599-652,
// through amrex::PlotFileDataImpl).
//
// Layout of one plotfile directory:
//   Header                 text: "HyperCLaw-V1.1", component names, dimension,
//                          time, finest level, problem extents, refinement
//                          ratios, level domains, level steps, cell sizes,
//                          coordinate system, then per level its box count,
//                          the physical extents of each box and the relative
//                          path of the level's multifab ("Level_<l>/Cell").
//   Level_<l>/Cell_H       multifab header (version 1): component and ghost
//                          counts, the box list, one "FabOnDisk: <file>
//                          <offset>" entry per box, per-box minima and maxima.
//   Level_<l>/Cell_D_00000 the boxes' data, each a one-line FAB header
//                          ("FAB ((8, (64 11 52 0 1 12 0 1023)),(8, (<byte
//                          order>)))<box> <ncomp>") followed by the values,
//                          x fastest, component slowest.
//
// The writer emits IEEE doubles in the host's byte order; the reader accepts
// 4- and 8-byte IEEE data in either byte order and FABs grown by ghost cells.
// Everything here is plain C++ (no CUDA): it also runs without a GPU.
#pragma once

#include <sys/stat.h>

#include <algorithm>
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

#include "amr_grids.hpp"

namespace adg {
namespace plt {

struct LevelMeta {
  std::vector<amr::IBox> boxes;  // valid boxes in the level's index space
  amr::IBox domain;              // the level's index domain
  double dx[3] = {1.0, 1.0, 1.0};
  int step = 0;
  std::string mf_path;  // multifab prefix relative to the plotfile, e.g. "Level_0/Cell"
};

struct Meta {
  int D = 2;
  int ncomp = 0;
  double time = 0.0;
  double prob_lo[3] = {0.0, 0.0, 0.0};
  double prob_hi[3] = {1.0, 1.0, 1.0};
  std::vector<int> ref_ratio;      // [finest level]
  std::vector<std::string> names;  // [ncomp]
  std::vector<LevelMeta> levels;   // [finest level + 1]
  int coord = 0;                   // 0: Cartesian
};

// One level's data: per box, ncomp * cells values, x fastest, component slowest.
using LevelData = std::vector<std::vector<double>>;

inline long long box_cells(const amr::IBox& b, int D) { return b.volume(D); }

inline std::string box_text(const amr::IBox& b, int D) {
  std::ostringstream os;
  auto tuple = [&](const int* v) {
    os << '(';
    for (int d = 0; d < D; ++d) os << (d ? "," : "") << v[d];
    os << ')';
  };
  const int zero[3] = {0, 0, 0};
  os << '(';
  tuple(b.lo);
  os << ' ';
  tuple(b.hi);
  os << ' ';
  tuple(zero);  // cell-centred index type
  os << ')';
  return os.str();
}

inline bool host_little_endian() {
  const uint16_t one = 1;
  unsigned char c;
  std::memcpy(&c, &one, 1);
  return c == 1;
}

inline bool make_dir(const std::string& p, std::string* err) {
  if (mkdir(p.c_str(), 0755) != 0 && errno != EEXIST) {
    *err = "cannot create directory " + p + ": " + std::strerror(errno);
    return false;
  }
  struct stat st;
  if (stat(p.c_str(), &st) != 0 || !S_ISDIR(st.st_mode)) {
    *err = p + " exists and is not a directory";
    return false;
  }
  return true;
}

// Creates every missing directory of path (like mkdir -p).
inline bool make_dirs(const std::string& path, std::string* err) {
  for (size_t pos = 1; pos <= path.size(); ++pos) {
    if (pos < path.size() && path[pos] != '/') continue;
    const std::string part = path.substr(0, pos);
    if (part.empty() || part == "/" || part.back() == '/') continue;
    if (!make_dir(part, err)) return false;
  }
  return true;
}

inline bool write_text(const std::string& path, const std::string& text, std::string* err) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) {
    *err = "cannot open " + path + ": " + std::strerror(errno);
    return false;
  }
  const bool ok = std::fwrite(text.data(), 1, text.size(), f) == text.size();
  if (std::fclose(f) != 0 || !ok) {
    *err = "write failed: " + path;
    return false;
  }
  return true;
}

// Writes one plotfile directory.  data[l][b] holds ncomp * cells(box b of
// level l) values.
inline bool write(const std::string& dir, const Meta& m, const std::vector<LevelData>& data, std::string* err) {
  const int D = m.D, nlev = (int)m.levels.size();
  if (nlev < 1 || (int)data.size() != nlev || (int)m.names.size() != m.ncomp || (int)m.ref_ratio.size() != nlev - 1) {
    *err = "plotfile: inconsistent metadata";
    return false;
  }
  if (!make_dirs(dir, err)) return false;
  std::ostringstream h;
  h.precision(17);
  h << "HyperCLaw-V1.1\n" << m.ncomp << '\n';
  for (const auto& n : m.names) h << n << '\n';
  h << D << '\n' << m.time << '\n' << nlev - 1 << '\n';
  for (int d = 0; d < D; ++d) h << m.prob_lo[d] << ' ';
  h << '\n';
  for (int d = 0; d < D; ++d) h << m.prob_hi[d] << ' ';
  h << '\n';
  for (int r : m.ref_ratio) h << r << ' ';
  h << '\n';
  for (const auto& L : m.levels) h << box_text(L.domain, D) << ' ';
  h << '\n';
  for (const auto& L : m.levels) h << L.step << ' ';
  h << '\n';
  for (const auto& L : m.levels) {
    for (int d = 0; d < D; ++d) h << L.dx[d] << ' ';
    h << '\n';
  }
  h << m.coord << '\n' << 0 << '\n';  // coordinate system, boundary width

  const bool little = host_little_endian();
  const char* order = little ? "8 7 6 5 4 3 2 1" : "1 2 3 4 5 6 7 8";
  for (int l = 0; l < nlev; ++l) {
    const LevelMeta& L = m.levels[l];
    const int nb = (int)L.boxes.size();
    if ((int)data[l].size() != nb) {
      *err = "plotfile: data does not match the box list";
      return false;
    }
    h << l << ' ' << nb << ' ' << m.time << '\n' << L.step << '\n';
    for (const auto& b : L.boxes)
      for (int d = 0; d < D; ++d)
        h << m.prob_lo[d] + L.dx[d] * b.lo[d] << ' ' << m.prob_lo[d] + L.dx[d] * (b.hi[d] + 1) << '\n';
    const std::string level_dir = "Level_" + std::to_string(l);
    h << level_dir << "/Cell\n";
    if (!make_dir(dir + "/" + level_dir, err)) return false;

    // data file: FAB header line + values per box
    const std::string dname = "Cell_D_00000";
    const std::string dpath = dir + "/" + level_dir + "/" + dname;
    FILE* f = std::fopen(dpath.c_str(), "wb");
    if (!f) {
      *err = "cannot open " + dpath + ": " + std::strerror(errno);
      return false;
    }
    std::vector<long long> offs(nb);
    std::vector<std::vector<double>> mn(nb), mx(nb);
    long long pos = 0;
    bool ok = true;
    for (int b = 0; b < nb && ok; ++b) {
      const long long nc = box_cells(L.boxes[b], D);
      if ((long long)data[l][b].size() != nc * m.ncomp) {
        *err = "plotfile: box data has the wrong size";
        std::fclose(f);
        return false;
      }
      std::string fh = std::string("FAB ((8, (64 11 52 0 1 12 0 1023)),(8, (") + order + ")))" +
                       box_text(L.boxes[b], D) + " " + std::to_string(m.ncomp) + "\n";
      offs[b] = pos;
      ok = std::fwrite(fh.data(), 1, fh.size(), f) == fh.size();
      ok = ok && std::fwrite(data[l][b].data(), sizeof(double), data[l][b].size(), f) == data[l][b].size();
      pos += (long long)fh.size() + (long long)data[l][b].size() * 8;
      mn[b].assign(m.ncomp, 0.0);
      mx[b].assign(m.ncomp, 0.0);
      for (int c = 0; c < m.ncomp; ++c) {
        const double* v = data[l][b].data() + (size_t)c * nc;
        double lo = v[0], hi = v[0];
        for (long long i = 1; i < nc; ++i) {
          lo = v[i] < lo ? v[i] : lo;
          hi = v[i] > hi ? v[i] : hi;
        }
        mn[b][c] = lo;
        mx[b][c] = hi;
      }
    }
    if (std::fclose(f) != 0 || !ok) {
      *err = "write failed: " + dpath;
      return false;
    }
    // multifab header
    std::ostringstream c;
    c.precision(17);
    c << 1 << '\n' << 1 << '\n' << m.ncomp << '\n' << 0 << '\n';  // version, files layout, ncomp, ghost cells
    c << '(' << nb << " 0\n";
    for (const auto& b : L.boxes) c << box_text(b, D) << '\n';
    c << ")\n" << nb << '\n';
    for (int b = 0; b < nb; ++b) c << "FabOnDisk: " << dname << ' ' << offs[b] << '\n';
    c << '\n';
    for (const auto* tab : {&mn, &mx}) {
      c << nb << ',' << m.ncomp << '\n';
      for (int b = 0; b < nb; ++b) {
        for (int k = 0; k < m.ncomp; ++k) c << (*tab)[b][k] << ',';
        c << '\n';
      }
      c << '\n';
    }
    if (!write_text(dir + "/" + level_dir + "/Cell_H", c.str(), err)) return false;
  }
  return write_text(dir + "/Header", h.str(), err);
}

// ---------------------------------------------------------------- reading

inline bool read_text(const std::string& path, std::string* out, std::string* err) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) {
    *err = "cannot open " + path + ": " + std::strerror(errno);
    return false;
  }
  out->clear();
  char buf[1 << 16];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) {
    out->append(buf, n);
    if (out->size() > ((size_t)1 << 30)) {
      std::fclose(f);
      *err = path + ": header too large";
      return false;
    }
  }
  std::fclose(f);
  return true;
}

inline std::vector<std::string> split_lines(const std::string& s) {
  std::vector<std::string> v;
  size_t a = 0;
  while (a < s.size()) {
    size_t b = s.find('\n', a);
    if (b == std::string::npos) b = s.size();
    std::string line = s.substr(a, b - a);
    while (!line.empty() && (line.back() == '\r' || line.back() == ' ' || line.back() == '\t')) line.pop_back();
    v.push_back(line);
    a = b + 1;
  }
  return v;
}

// All integers of s in order (a '-' directly before digits is a sign);
// values saturate at 2^50, which every caller's range check rejects.
inline std::vector<long long> ints_in(const std::string& s) {
  std::vector<long long> v;
  size_t i = 0;
  while (i < s.size()) {
    const bool neg = s[i] == '-' && i + 1 < s.size() && s[i + 1] >= '0' && s[i + 1] <= '9';
    if (neg || (s[i] >= '0' && s[i] <= '9')) {
      if (neg) ++i;
      long long x = 0;
      while (i < s.size() && s[i] >= '0' && s[i] <= '9') {
        x = std::min(10 * x + (s[i] - '0'), 1LL << 50);
        ++i;
      }
      v.push_back(neg ? -x : x);
    } else {
      ++i;
    }
  }
  return v;
}

inline bool doubles_in(const std::string& s, int n, double* out) {
  const char* p = s.c_str();
  for (int k = 0; k < n; ++k) {
    char* e = nullptr;
    errno = 0;
    out[k] = std::strtod(p, &e);
    if (e == p || errno == ERANGE) return false;
    p = e;
  }
  return true;
}

inline bool parse_int(const std::string& s, long long lo, long long hi, int* out) {
  const char* p = s.c_str();
  char* e = nullptr;
  errno = 0;
  const long long v = std::strtoll(p, &e, 10);
  if (e == p || errno == ERANGE || v < lo || v > hi) return false;
  while (*e == ' ' || *e == '\t') ++e;
  if (*e) return false;
  *out = (int)v;
  return true;
}

// Boxes "((lo) (hi) (type))" from consecutive integers: 3*D per box.
inline bool boxes_from_ints(const std::vector<long long>& v, size_t at, int D, int n, std::vector<amr::IBox>* out) {
  if (v.size() < at + (size_t)(3 * D * n)) return false;
  for (int b = 0; b < n; ++b) {
    amr::IBox bx;
    const long long* p = &v[at + (size_t)3 * D * b];
    for (int d = 0; d < D; ++d) {
      if (p[d] < -(1LL << 30) || p[d] > (1LL << 30) || p[D + d] < -(1LL << 30) || p[D + d] > (1LL << 30)) return false;
      if (p[2 * D + d] != 0) return false;  // cell-centred data only
      bx.lo[d] = (int)p[d];
      bx.hi[d] = (int)p[D + d];
    }
    if (bx.empty(D)) return false;
    out->push_back(bx);
  }
  return true;
}

struct Cursor {
  const std::string& s;
  size_t i = 0;
  explicit Cursor(const std::string& t) : s(t) {}
  void ws() {
    while (i < s.size() && (s[i] == ' ' || s[i] == '\n' || s[i] == '\r' || s[i] == '\t')) ++i;
  }
  bool ch(char c) {
    ws();
    if (i < s.size() && s[i] == c) {
      ++i;
      return true;
    }
    return false;
  }
  bool integer(long long* v) {
    ws();
    const char* p = s.c_str() + i;
    char* e = nullptr;
    errno = 0;
    *v = std::strtoll(p, &e, 10);
    if (e == p || errno == ERANGE) return false;
    i += (size_t)(e - p);
    return true;
  }
  bool token(std::string* t) {
    ws();
    size_t a = i;
    while (i < s.size() && s[i] != ' ' && s[i] != '\n' && s[i] != '\r' && s[i] != '\t') ++i;
    *t = s.substr(a, i - a);
    return !t->empty();
  }
  // a balanced "( ... )" group
  bool group(std::string* g) {
    ws();
    if (i >= s.size() || s[i] != '(') return false;
    int depth = 0;
    size_t a = i;
    for (; i < s.size(); ++i) {
      if (s[i] == '(') ++depth;
      if (s[i] == ')' && --depth == 0) {
        ++i;
        *g = s.substr(a, i - a);
        return true;
      }
    }
    return false;
  }
};

struct FabRef {
  std::string file;
  long long offset = 0;
};

// Cell_H of one level: box list and data locations.
inline bool read_mf_header(const std::string& path, int D, int ncomp, std::vector<amr::IBox>* boxes,
                           std::vector<FabRef>* fabs, std::string* err) {
  std::string text;
  if (!read_text(path, &text, err)) return false;
  Cursor c(text);
  long long vers, how, nc, nb, hash, nf;
  std::string g;
  auto bad = [&](const char* what) {
    *err = path + ": " + what;
    return false;
  };
  if (!c.integer(&vers) || !c.integer(&how) || !c.integer(&nc)) return bad("malformed header");
  if (vers != 1) return bad("unsupported multifab header version");
  if (nc != ncomp) return bad("component count differs from the plotfile header");
  c.ws();
  if (c.i < text.size() && text[c.i] == '(') {  // ghost counts per direction
    if (!c.group(&g)) return bad("malformed ghost count");
    for (long long x : ints_in(g))
      if (x < 0) return bad("negative ghost count");
  } else {
    long long ng;
    if (!c.integer(&ng) || ng < 0) return bad("malformed ghost count");
  }
  if (!c.ch('(') || !c.integer(&nb) || !c.integer(&hash) || nb < 1 || nb > (1 << 24)) return bad("malformed box list");
  for (long long b = 0; b < nb; ++b) {
    if (!c.group(&g)) return bad("malformed box");
    if (!boxes_from_ints(ints_in(g), 0, D, 1, boxes)) return bad("malformed box");
  }
  if (!c.ch(')') || !c.integer(&nf) || nf != nb) return bad("box list and data list differ");
  for (long long b = 0; b < nf; ++b) {
    std::string tag, file;
    FabRef r;
    if (!c.token(&tag) || tag != "FabOnDisk:" || !c.token(&file) || !c.integer(&r.offset) || r.offset < 0)
      return bad("malformed FabOnDisk entry");
    if (file.find('/') != std::string::npos || file == "..") return bad("data file outside the level directory");
    r.file = file;
    fabs->push_back(r);
  }
  return true;
}

struct FabHeader {
  int bytes = 8;  // 4 or 8
  bool swap = false;
  amr::IBox box;
  int ncomp = 0;
  long long header_len = 0;
};

inline bool read_fab_header(FILE* f, const std::string& where, int D, FabHeader* fh, std::string* err) {
  std::string line;
  int ch;
  while ((ch = std::fgetc(f)) != EOF && ch != '\n') {
    line.push_back((char)ch);
    if (line.size() > 4096) break;
  }
  if (ch != '\n' || line.compare(0, 4, "FAB ") != 0) {
    *err = where + ": missing FAB header";
    return false;
  }
  fh->header_len = (long long)line.size() + 1;
  const std::vector<long long> v = ints_in(line);
  // fmt bytes, 8 format numbers, order bytes, order list, box (3*D), ncomp
  if (v.size() < 10) {
    *err = where + ": malformed FAB header";
    return false;
  }
  const long long fb = v[0];
  static const long long f64[8] = {64, 11, 52, 0, 1, 12, 0, 1023};
  static const long long f32[8] = {32, 8, 23, 0, 1, 9, 0, 127};
  const long long* want = fb == 8 ? f64 : fb == 4 ? f32 : nullptr;
  if (!want || !std::equal(want, want + 8, v.begin() + 1) || v[9] != fb ||
      v.size() != (size_t)(10 + fb + 3 * D + 1)) {
    *err = where + ": unsupported number format (IEEE 4- or 8-byte reals only)";
    return false;
  }
  bool asc = true, desc = true;
  for (long long k = 0; k < fb; ++k) {
    asc = asc && v[10 + k] == k + 1;
    desc = desc && v[10 + k] == fb - k;
  }
  if (!asc && !desc) {
    *err = where + ": unsupported byte order";
    return false;
  }
  const bool file_little = desc;  // least significant byte first
  fh->bytes = (int)fb;
  fh->swap = file_little != host_little_endian();
  std::vector<amr::IBox> bx;
  if (!boxes_from_ints(v, (size_t)(10 + fb), D, 1, &bx)) {
    *err = where + ": malformed FAB box";
    return false;
  }
  fh->box = bx[0];
  fh->ncomp = (int)v.back();
  return true;
}

inline double decode(const unsigned char* p, int bytes, bool swap) {
  unsigned char b[8];
  for (int k = 0; k < bytes; ++k) b[k] = swap ? p[bytes - 1 - k] : p[k];
  if (bytes == 8) {
    double d;
    std::memcpy(&d, b, 8);
    return d;
  }
  float x;
  std::memcpy(&x, b, 4);
  return (double)x;
}

// Reads the valid box vb of one FAB into out (ncomp * cells, x fastest,
// component slowest); with out == nullptr only the header and the file size
// are checked.
inline bool read_fab(const std::string& path, long long offset, int D, int ncomp, const amr::IBox& vb,
                     std::vector<double>* out, std::string* err) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) {
    *err = "cannot open " + path + ": " + std::strerror(errno);
    return false;
  }
  auto fail = [&](const std::string& m) {
    std::fclose(f);
    *err = m;
    return false;
  };
  const std::string where = path + " @" + std::to_string(offset);
  if (std::fseek(f, (long)offset, SEEK_SET) != 0) return fail(where + ": bad offset");
  FabHeader fh;
  if (!read_fab_header(f, where, D, &fh, err)) {
    std::fclose(f);
    return false;
  }
  if (fh.ncomp < ncomp) return fail(where + ": fewer components than the plotfile header");
  for (int d = 0; d < D; ++d)
    if (vb.lo[d] < fh.box.lo[d] || vb.hi[d] > fh.box.hi[d]) return fail(where + ": FAB does not contain its box");
  long long n[3] = {1, 1, 1};
  for (int d = 0; d < D; ++d) n[d] = fh.box.hi[d] - fh.box.lo[d] + 1;
  const long long cells = n[0] * n[1] * n[2];
  const long long bytes = cells * ncomp * fh.bytes;
  const long long start = offset + fh.header_len;
  if (std::fseek(f, 0, SEEK_END) != 0 || std::ftell(f) < start + cells * fh.ncomp * fh.bytes)
    return fail(where + ": data file too short");
  if (!out) {
    std::fclose(f);
    return true;
  }
  std::vector<unsigned char> raw((size_t)bytes);
  if (std::fseek(f, (long)start, SEEK_SET) != 0 || std::fread(raw.data(), 1, raw.size(), f) != raw.size())
    return fail(where + ": read failed");
  std::fclose(f);
  const long long vc = box_cells(vb, D);
  out->assign((size_t)(vc * ncomp), 0.0);
  size_t o = 0;
  for (int c = 0; c < ncomp; ++c)
    for (int k = vb.lo[2]; k <= (D > 2 ? vb.hi[2] : vb.lo[2]); ++k)
      for (int j = vb.lo[1]; j <= (D > 1 ? vb.hi[1] : vb.lo[1]); ++j)
        for (int i = vb.lo[0]; i <= vb.hi[0]; ++i) {
          const long long ii = i - fh.box.lo[0];
          const long long jj = D > 1 ? j - fh.box.lo[1] : 0;
          const long long kk = D > 2 ? k - fh.box.lo[2] : 0;
          const long long at = (long long)c * cells + (kk * n[1] + jj) * n[0] + ii;
          (*out)[o++] = decode(&raw[(size_t)at * fh.bytes], fh.bytes, fh.swap);
        }
  return true;
}

// Reads a plotfile: the whole header, and the data of levels < data_levels
// into data (nullptr: the FAB headers of every level are checked, no values
// read).
inline bool read(const std::string& dir, int data_levels, Meta* m, std::vector<LevelData>* data, std::string* err) {
  std::string text;
  if (!read_text(dir + "/Header", &text, err)) return false;
  const std::vector<std::string> L = split_lines(text);
  size_t i = 0;
  auto bad = [&](const std::string& what) {
    *err = dir + "/Header: " + what + " (line " + std::to_string(i + 1) + ")";
    return false;
  };
  auto line = [&](std::string* s) {
    if (i >= L.size()) return false;
    *s = L[i++];
    return true;
  };
  std::string s;
  if (!line(&s) || s != "HyperCLaw-V1.1") return bad("not a HyperCLaw-V1.1 plotfile");
  if (!line(&s) || !parse_int(s, 1, 1 << 20, &m->ncomp)) return bad("bad component count");
  m->names.clear();
  for (int c = 0; c < m->ncomp; ++c) {
    if (!line(&s)) return bad("missing component name");
    m->names.push_back(s);
  }
  int finest = 0;
  if (!line(&s) || !parse_int(s, 1, 3, &m->D)) return bad("bad dimension");
  const int D = m->D;
  if (!line(&s) || !doubles_in(s, 1, &m->time)) return bad("bad time");
  if (!line(&s) || !parse_int(s, 0, 30, &finest)) return bad("bad finest level");
  if (!line(&s) || !doubles_in(s, D, m->prob_lo)) return bad("bad lower problem corner");
  if (!line(&s) || !doubles_in(s, D, m->prob_hi)) return bad("bad upper problem corner");
  if (!line(&s)) return bad("missing refinement ratios");
  std::vector<long long> v = ints_in(s);
  if ((int)v.size() != finest) return bad("refinement ratio count differs from the finest level");
  m->ref_ratio.assign(v.begin(), v.end());
  for (int r : m->ref_ratio)
    if (r < 1) return bad("bad refinement ratio");
  m->levels.assign(finest + 1, LevelMeta{});
  std::vector<amr::IBox> dom;
  if (!line(&s) || !boxes_from_ints(ints_in(s), 0, D, finest + 1, &dom) ||
      ints_in(s).size() != (size_t)(3 * D * (finest + 1)))
    return bad("bad level domains");
  if (!line(&s) || (v = ints_in(s)).size() != (size_t)(finest + 1)) return bad("bad level steps");
  for (int l = 0; l <= finest; ++l) {
    m->levels[l].domain = dom[l];
    m->levels[l].step = (int)v[l];
  }
  for (int l = 0; l <= finest; ++l)
    if (!line(&s) || !doubles_in(s, D, m->levels[l].dx)) return bad("bad cell size");
  int bw = 0;
  if (!line(&s) || !parse_int(s, 0, 2, &m->coord)) return bad("bad coordinate system");
  if (!line(&s) || !parse_int(s, 0, 1 << 20, &bw)) return bad("bad boundary width");
  std::vector<int> nbox(finest + 1);
  for (int l = 0; l <= finest; ++l) {
    {  // "<level> <boxes> <time>"
      std::istringstream ls(line(&s) ? s : std::string());
      long long lv = -1, nb = 0;
      double tl = 0.0;
      if (!(ls >> lv >> nb >> tl) || lv != l || nb < 1 || nb > (1 << 24)) return bad("bad level line");
      nbox[l] = (int)nb;
    }
    if (!line(&s)) return bad("missing level step");
    for (int b = 0; b < nbox[l] * D; ++b) {
      double ext[2];
      if (!line(&s) || !doubles_in(s, 2, ext)) return bad("bad box extents");
    }
    if (!line(&s) || s.empty() || s.find("..") != std::string::npos || s[0] == '/') return bad("bad multifab path");
    m->levels[l].mf_path = s;
  }
  if (data) data->assign(std::min(data_levels, finest + 1), LevelData{});
  for (int l = 0; l <= finest; ++l) {
    LevelMeta& lm = m->levels[l];
    std::vector<FabRef> fabs;
    const std::string mf = dir + "/" + lm.mf_path;
    if (!read_mf_header(mf + "_H", D, m->ncomp, &lm.boxes, &fabs, err)) return false;
    if ((int)lm.boxes.size() != nbox[l]) {
      *err = mf + "_H: box count differs from the plotfile header";
      return false;
    }
    const std::string base = mf.substr(0, mf.find_last_of('/') + 1);
    const bool load = data && l < data_levels;
    if (load) (*data)[l].resize(lm.boxes.size());
    for (size_t b = 0; b < lm.boxes.size(); ++b)
      if (!read_fab(base + fabs[b].file, fabs[b].offset, D, m->ncomp, lm.boxes[b], load ? &(*data)[l][b] : nullptr,
                    err))
        return false;
  }
  return true;
}

}  // namespace plt
}  // namespace adg

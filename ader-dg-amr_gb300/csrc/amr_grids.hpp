// Block-structured AMR grid generation (host, header-only C++17).
//
// AMReX is not available to this project, so the box layout the reference
// gets from amrex::AmrCore (Source/Core/Mesh.h:126-196; regrid loop
// Source/NumericalMethod/AmrDG/AmrDG.h:935-986) is produced here:
//   * tags per level (cells flagged by the refinement criterion),
//   * buffering by n_error_buf cells, coarsening by blocking_factor / ratio,
//   * proper nesting of level l+2 inside level l+1 (projected tags),
//   * Berger-Rigoutsos clustering (holes, then the steepest sign change of
//     the second difference of the signature, else bisection) until every
//     cluster's efficiency reaches grid_eff,
//   * refinement back to the fine level and chopping to max_grid.
// Both the CUDA path and the CPU oracle use this one implementation, so their
// box layouts are identical by construction.
#pragma once

#include <algorithm>
#include <array>
#include <cstdint>
#include <cstdlib>
#include <vector>

namespace adg {
namespace amr {

struct IBox {
  int lo[3] = {0, 0, 0};
  int hi[3] = {0, 0, 0};
  bool empty(int D) const {
    for (int d = 0; d < D; ++d)
      if (hi[d] < lo[d]) return true;
    return false;
  }
  long long volume(int D) const {
    long long v = 1;
    for (int d = 0; d < D; ++d) v *= (long long)(hi[d] - lo[d] + 1);
    return v;
  }
  bool operator==(const IBox& o) const {
    for (int d = 0; d < 3; ++d)
      if (lo[d] != o.lo[d] || hi[d] != o.hi[d]) return false;
    return true;
  }
  bool contains(int D, const int* c) const {
    for (int d = 0; d < D; ++d)
      if (c[d] < lo[d] || c[d] > hi[d]) return false;
    return true;
  }
};

inline int floordiv(int a, int b) { return (a >= 0) ? a / b : -((-a + b - 1) / b); }

inline IBox coarsen(const IBox& b, int D, int r) {
  IBox c = b;
  for (int d = 0; d < D; ++d) {
    c.lo[d] = floordiv(b.lo[d], r);
    c.hi[d] = floordiv(b.hi[d], r);
  }
  return c;
}

inline IBox refine(const IBox& b, int D, int r) {
  IBox c = b;
  for (int d = 0; d < D; ++d) {
    c.lo[d] = b.lo[d] * r;
    c.hi[d] = (b.hi[d] + 1) * r - 1;
  }
  return c;
}

inline IBox grow(const IBox& b, int D, int g) {
  IBox c = b;
  for (int d = 0; d < D; ++d) {
    c.lo[d] -= g;
    c.hi[d] += g;
  }
  return c;
}

inline bool intersect(const IBox& a, const IBox& b, int D, IBox* out) {
  IBox c = a;
  for (int d = 0; d < D; ++d) {
    c.lo[d] = std::max(a.lo[d], b.lo[d]);
    c.hi[d] = std::min(a.hi[d], b.hi[d]);
    if (c.hi[d] < c.lo[d]) return false;
  }
  if (out) *out = c;
  return true;
}

// Split boxes so no edge exceeds max_grid: every oversized direction is cut
// into the fewest nearly equal pieces, keeping piece sizes multiples of the
// largest power of two dividing both the edge and max_grid.
inline std::vector<IBox> chop_max_size(std::vector<IBox> boxes, int D, int max_grid) {
  std::vector<IBox> out;
  for (size_t i = 0; i < boxes.size(); ++i) {
    IBox b = boxes[i];
    bool split = false;
    for (int d = 0; d < D && !split; ++d) {
      const int len = b.hi[d] - b.lo[d] + 1;
      if (len <= max_grid) continue;
      int ratio = 1, bs = max_grid, nlen = len;
      while (bs % 2 == 0 && nlen % 2 == 0) {
        ratio *= 2;
        bs /= 2;
        nlen /= 2;
      }
      const int numblk = nlen / bs + (nlen % bs ? 1 : 0);
      const int sz = nlen / numblk, extra = nlen % numblk;
      int start = b.lo[d];
      for (int k = 0; k < numblk; ++k) {
        const int ksize = (k < extra ? sz + 1 : sz) * ratio;
        IBox p = b;
        p.lo[d] = start;
        p.hi[d] = start + ksize - 1;
        start += ksize;
        boxes.push_back(p);  // re-examined for the other directions
      }
      split = true;
    }
    if (!split) out.push_back(b);
  }
  return out;
}

// ---------------------------------------------------------------------------
// Berger-Rigoutsos clustering of tagged points.
// ---------------------------------------------------------------------------
enum CutKind { CUT_HOLE = 0, CUT_STEEP = 1, CUT_BISECT = 2, CUT_INVALID = 3 };

inline int find_cut(const std::vector<int>& hist, int lo, int hi, CutKind* kind) {
  const int MINOFF = 2, CUT_THRESH = 2;
  *kind = CUT_INVALID;
  const int len = hi - lo + 1;
  if (len <= 1) return lo;
  const int mid = len / 2;
  int cut = -1;
  for (int i = 0; i < len; ++i) {  // most central hole
    if (hist[i] == 0) {
      *kind = CUT_HOLE;
      if (std::abs(cut - mid) > std::abs(i - mid)) {
        cut = i;
        if (i > mid) break;
      }
    }
  }
  if (*kind == CUT_HOLE) return lo + cut;
  std::vector<int> dh(len, 0);
  for (int i = 1; i < len - 1; ++i) dh[i] = hist[i + 1] - 2 * hist[i] + hist[i - 1];
  int locmax = -1;
  for (int i = MINOFF; i < len - MINOFF; ++i) {
    const int a = dh[i - 1], b = dh[i];
    const int dif = std::abs(a - b);
    if ((long long)a * b < 0 && dif >= locmax) {
      if (dif > locmax) {
        *kind = CUT_STEEP;
        cut = i;
        locmax = dif;
      } else if (std::abs(i - mid) < std::abs(cut - mid)) {
        cut = i;
      }
    }
  }
  if (locmax <= CUT_THRESH) {
    cut = mid;
    *kind = CUT_BISECT;
  }
  return lo + cut;
}

struct Cluster {
  std::vector<std::array<int, 3>> pts;
  IBox box;
  void min_box(int D) {
    for (int d = 0; d < 3; ++d) {
      box.lo[d] = d < D ? pts[0][d] : 0;
      box.hi[d] = d < D ? pts[0][d] : 0;
    }
    for (const auto& p : pts)
      for (int d = 0; d < D; ++d) {
        box.lo[d] = std::min(box.lo[d], p[d]);
        box.hi[d] = std::max(box.hi[d], p[d]);
      }
  }
  double eff(int D) const { return (double)pts.size() / (double)box.volume(D); }
};

inline Cluster chop_cluster(Cluster& c, int D) {
  std::vector<int> hist[3];
  for (int d = 0; d < D; ++d) {
    hist[d].assign(c.box.hi[d] - c.box.lo[d] + 1, 0);
    for (const auto& p : c.pts) hist[d][p[d] - c.box.lo[d]]++;
  }
  CutKind kind[3];
  int cut[3];
  CutKind best = CUT_INVALID;
  for (int d = 0; d < D; ++d) {
    cut[d] = find_cut(hist[d], c.box.lo[d], c.box.hi[d], &kind[d]);
    if (kind[d] < best) best = kind[d];
  }
  int dir = -1, minlen = -1;
  for (int d = 0; d < D; ++d)
    if (kind[d] == best) {
      const int l = std::min(cut[d] - c.box.lo[d], c.box.hi[d] - cut[d]);
      if (l > minlen) {
        dir = d;
        minlen = l;
      }
    }
  Cluster upper;
  std::vector<std::array<int, 3>> lower;
  for (const auto& p : c.pts) (p[dir] < cut[dir] ? lower : upper.pts).push_back(p);
  c.pts.swap(lower);
  c.min_box(D);
  upper.min_box(D);
  return upper;
}

inline std::vector<IBox> cluster(const std::vector<std::array<int, 3>>& tags, int D, double grid_eff) {
  std::vector<Cluster> lst;
  if (tags.empty()) return {};
  Cluster all;
  all.pts = tags;
  all.min_box(D);
  lst.push_back(all);
  for (size_t i = 0; i < lst.size();) {
    if (lst[i].eff(D) < grid_eff && lst[i].pts.size() > 1) {
      Cluster up = chop_cluster(lst[i], D);
      lst.push_back(up);
    } else {
      ++i;
    }
  }
  std::vector<IBox> out;
  for (auto& c : lst) out.push_back(c.box);
  return out;
}

// ---------------------------------------------------------------------------
// New grids for levels lbase+1 .. from tags of levels lbase .. finest.
// ---------------------------------------------------------------------------
struct GridParams {
  int D = 2;
  int n_cell0[3] = {1, 1, 1};
  int periodic[3] = {1, 1, 1};
  int max_level = 0;
  int ref_ratio = 2;
  int blocking_factor = 8;
  int max_grid = 32;
  double grid_eff = 0.7;
  int n_error_buf = 1;
  int n_proper = 1;
};

// Dense cell flags of one level's index space.
struct TagField {
  int n[3] = {1, 1, 1};
  std::vector<uint8_t> f;
  void init(const int* nn) {
    for (int d = 0; d < 3; ++d) n[d] = nn[d];
    f.assign((size_t)n[0] * n[1] * n[2], 0);
  }
  size_t idx(int i, int j, int k) const { return ((size_t)k * n[1] + j) * n[0] + i; }
};

inline void level_dims(const GridParams& P, int l, int* n) {
  for (int d = 0; d < 3; ++d) n[d] = d < P.D ? P.n_cell0[d] << l : 1;
}

// Level 0 boxes: the domain chopped to max_grid.
inline std::vector<IBox> base_grids(const GridParams& P) {
  IBox dom;
  for (int d = 0; d < 3; ++d) {
    dom.lo[d] = 0;
    dom.hi[d] = d < P.D ? P.n_cell0[d] - 1 : 0;
  }
  return chop_max_size({dom}, P.D, P.max_grid);
}

// tags[l]: flags over level l's index space (only cells of level l boxes can
// be set).  grids[l]: current boxes of level l (l <= finest).  Returns the new
// boxes of levels 0 .. new_finest (level 0 unchanged).
inline std::vector<std::vector<IBox>> make_new_grids(const GridParams& P, const std::vector<std::vector<IBox>>& grids,
                                                     const std::vector<TagField>& tags) {
  const int D = P.D;
  const int finest = (int)grids.size() - 1;
  const int max_crse = std::min(finest, P.max_level - 1);
  const int bf = std::max(1, P.blocking_factor / P.ref_ratio);  // coarsening of the tag field
  std::vector<std::vector<IBox>> out(std::max(finest, max_crse + 1) + 1);
  out[0] = grids[0];
  int new_finest = 0;
  for (int levc = max_crse; levc >= 0; --levc) {
    const int levf = levc + 1;
    int nl[3];
    level_dims(P, levc, nl);
    // coarsened tag field (tag space = level levc coarsened by bf)
    int nc[3];
    for (int d = 0; d < 3; ++d) nc[d] = d < D ? (nl[d] + bf - 1) / bf : 1;
    TagField ct;
    ct.init(nc);
    auto set_ct = [&](int i, int j, int k) {
      int c[3] = {i, j, k};
      for (int d = 0; d < D; ++d) {
        c[d] = floordiv(c[d], bf);
        if (P.periodic[d])
          c[d] = ((c[d] % nc[d]) + nc[d]) % nc[d];
        else if (c[d] < 0 || c[d] >= nc[d])
          return;
      }
      ct.f[ct.idx(c[0], c[1], c[2])] = 1;
    };
    // buffered tags of level levc
    const TagField& tf = tags[levc];
    const int b = P.n_error_buf;
    for (int k = 0; k < nl[2]; ++k)
      for (int j = 0; j < nl[1]; ++j)
        for (int i = 0; i < nl[0]; ++i) {
          if (!tf.f[tf.idx(i, j, k)]) continue;
          const int bz = D > 2 ? b : 0, by = D > 1 ? b : 0;
          for (int dk = -bz; dk <= bz; ++dk)
            for (int dj = -by; dj <= by; ++dj)
              for (int di = -b; di <= b; ++di) set_ct(i + di, j + dj, k + dk);
        }
    // proper nesting: the new level levf+1 grids, grown by n_proper cells of
    // level levf, must be covered by the new level levf.
    if (levf < new_finest) {
      for (const IBox& fb : out[levf + 1]) {
        IBox g = grow(coarsen(fb, D, P.ref_ratio), D, P.n_proper);  // level levf space
        IBox c = coarsen(g, D, P.ref_ratio);                          // level levc space
        for (int k = c.lo[2]; k <= c.hi[2]; ++k)
          for (int j = c.lo[1]; j <= c.hi[1]; ++j)
            for (int i = c.lo[0]; i <= c.hi[0]; ++i) set_ct(i, j, k);
      }
    }
    std::vector<std::array<int, 3>> pts;
    for (int k = 0; k < nc[2]; ++k)
      for (int j = 0; j < nc[1]; ++j)
        for (int i = 0; i < nc[0]; ++i)
          if (ct.f[ct.idx(i, j, k)]) pts.push_back({i, j, k});
    if (pts.empty()) continue;
    new_finest = std::max(new_finest, levf);
    std::vector<IBox> cl = cluster(pts, D, P.grid_eff);
    IBox dom;
    for (int d = 0; d < 3; ++d) {
      dom.lo[d] = 0;
      dom.hi[d] = nl[d] - 1;
    }
    std::vector<IBox> nb;
    for (const IBox& c : cl) {
      IBox r = refine(c, D, bf), x;
      if (intersect(r, dom, D, &x)) nb.push_back(refine(x, D, P.ref_ratio));
    }
    out[levf] = chop_max_size(nb, D, P.max_grid);
  }
  out.resize(new_finest + 1);
  return out;
}

}  // namespace amr
}  // namespace adg

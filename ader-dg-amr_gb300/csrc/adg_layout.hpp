// Host layout of the packed element list of an AMR hierarchy: elements
// (valid cells of every level, then the ghost elements the predictor needs at
// coarse-fine boundaries), their faces, and the tables the kernels index
// (faces, coarse-fine flux corrections, average-down, ghost fill).  Replaces
// the box / MultiFab / iMultiFab bookkeeping AMReX does for the reference
// (Source/Core/Mesh.h, Source/NumericalMethod/AmrDG/AmrDG_Level.tpp:240-414).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "adg.h"
#include "amr_grids.hpp"

namespace adg {

struct Hierarchy {
  int D = 2;
  int nlev = 0;
  int n_cell0[3] = {1, 1, 1};
  int periodic[3] = {1, 1, 1};
  std::vector<std::vector<amr::IBox>> grids;

  // elements: valid cells of level 0, 1, ... (x-fastest per level), then ghosts
  std::vector<int> elem_cell;      // [elem][3]
  std::vector<int8_t> elem_level;  // [elem]
  std::vector<size_t> lev_valid_off, lev_valid_cnt;
  size_t n_valid_ = 0, n_elem_ = 0;
  std::vector<std::vector<int>> cellmap;   // per level: cell -> element (valid or ghost), -1
  std::vector<std::vector<int>> cellbox;   // per level: cell -> box index (valid cells), -1

  // faces, grouped by direction
  std::vector<int> face_left, face_right;
  int face_off[4] = {0, 0, 0, 0};
  std::vector<int> elem_face;  // [valid elem][2D]

  // coarse-fine corrections (reflux): one record per coarse cell with entries
  std::vector<int> rf_elem;       // [rec] coarse element
  std::vector<int> rf_off;        // [rec+1] entry range
  std::vector<int> rf_face;       // [ent] coarse face id
  std::vector<int8_t> rf_dside;   // [ent] 2*d + side (side 1: the coarse cell's high face)
  std::vector<int> rf_fine;       // [ent][2^(D-1)] fine face ids, child order
  // average down: per fine level lf (1..nlev-1), records (coarse, 2^D fine)
  std::vector<std::vector<int>> ad_rec;   // [lf] flat: coarse, fine_0 .. fine_{2^D-1}
  // ghost fill: ghost element, coarse parent element, child index
  std::vector<int> gf_elem, gf_parent;
  std::vector<int8_t> gf_child;

  int nlevels() const { return nlev; }
  size_t n_valid() const { return n_valid_; }
  size_t n_elem() const { return n_elem_; }
  size_t level_valid_offset(int l) const { return lev_valid_off[l]; }
  size_t level_valid_count(int l) const { return lev_valid_cnt[l]; }

  void dims(int l, int* n) const {
    for (int d = 0; d < 3; ++d) n[d] = d < D ? n_cell0[d] << l : 1;
  }
  size_t cidx(int l, const int* c) const {
    int n[3];
    dims(l, n);
    return ((size_t)c[2] * n[1] + c[1]) * n[0] + c[0];
  }
  // wrap periodically; false if outside a non-periodic domain
  bool wrap(int l, int* c) const {
    int n[3];
    dims(l, n);
    for (int d = 0; d < D; ++d) {
      if (c[d] >= 0 && c[d] < n[d]) continue;
      if (!periodic[d]) return false;
      c[d] = ((c[d] % n[d]) + n[d]) % n[d];
    }
    return true;
  }
  int elem_at(int l, const int* cin) const {
    int c[3] = {cin[0], cin[1], cin[2]};
    if (!wrap(l, c)) return -1;
    return cellmap[l][cidx(l, c)];
  }
  bool is_valid_elem(int e) const { return e >= 0 && (size_t)e < n_valid_; }
  bool covered(int l, const int* c) const {
    if (l + 1 >= nlev) return false;
    int f[3] = {0, 0, 0};
    for (int d = 0; d < D; ++d) f[d] = 2 * c[d];
    return is_valid_elem(elem_at(l + 1, f));
  }

  bool build_single_level(const adg_config& c, std::string* msg) {
    amr::GridParams gp = params(c);
    std::vector<std::vector<amr::IBox>> g;
    amr::IBox dom;
    for (int d = 0; d < 3; ++d) {
      dom.lo[d] = 0;
      dom.hi[d] = d < gp.D ? gp.n_cell0[d] - 1 : 0;
    }
    g.push_back({dom});
    return build(gp, g, 0, msg);
  }

  static amr::GridParams params(const adg_config& c) {
    amr::GridParams gp;
    gp.D = c.D;
    for (int d = 0; d < 3; ++d) {
      gp.n_cell0[d] = d < c.D ? c.n_cell[d] : 1;
      gp.periodic[d] = d < c.D ? c.periodic[d] : 1;
    }
    gp.max_level = c.max_level;
    gp.blocking_factor = c.blocking_factor > 0 ? c.blocking_factor : 8;
    gp.max_grid = c.max_grid > 0 ? c.max_grid : 32;
    gp.grid_eff = c.grid_eff > 0 ? c.grid_eff : 0.7;
    gp.n_error_buf = c.n_error_buf >= 0 ? c.n_error_buf : 1;
    return gp;
  }

  // Build every table for the given boxes.  reflux_quirk reproduces the
  // reference's per-box reflux mask (AmrDG_Interpolater.tpp:41-56 with the
  // face ownership rule of AmrDG_Level.tpp:316-330): a coarse cell is
  // corrected only if one of its coarse-fine faces is flagged in its own
  // box's face array, where a box never flags its own low face.
  // reflux = false leaves out every coarse-fine flux correction (the
  // reference's runs without AMR_flux_correction).
  bool build(const amr::GridParams& gp, const std::vector<std::vector<amr::IBox>>& g, int reflux_quirk,
             std::string* msg, bool reflux = true) {
    D = gp.D;
    for (int d = 0; d < 3; ++d) {
      n_cell0[d] = gp.n_cell0[d];
      periodic[d] = gp.periodic[d];
    }
    grids = g;
    nlev = (int)g.size();
    cellmap.assign(nlev, {});
    cellbox.assign(nlev, {});
    elem_cell.clear();
    elem_level.clear();
    lev_valid_off.assign(nlev, 0);
    lev_valid_cnt.assign(nlev, 0);
    // ---- valid elements
    for (int l = 0; l < nlev; ++l) {
      int n[3];
      dims(l, n);
      const size_t nc = (size_t)n[0] * n[1] * n[2];
      if (nc > (size_t)1 << 31) {
        if (msg) *msg = "level too large";
        return false;
      }
      cellmap[l].assign(nc, -1);
      cellbox[l].assign(nc, -1);
      for (size_t b = 0; b < g[l].size(); ++b) {
        const amr::IBox& bx = g[l][b];
        for (int k = bx.lo[2]; k <= bx.hi[2]; ++k)
          for (int j = bx.lo[1]; j <= bx.hi[1]; ++j)
            for (int i = bx.lo[0]; i <= bx.hi[0]; ++i) {
              int c[3] = {i, j, k};
              for (int d = 0; d < D; ++d)
                if (c[d] < 0 || c[d] >= n[d]) {
                  if (msg) *msg = "box outside the domain";
                  return false;
                }
              size_t id = cidx(l, c);
              if (cellbox[l][id] >= 0) {
                if (msg) *msg = "overlapping boxes";
                return false;
              }
              cellbox[l][id] = (int)b;
            }
      }
      lev_valid_off[l] = elem_level.size();
      for (int k = 0; k < n[2]; ++k)
        for (int j = 0; j < n[1]; ++j)
          for (int i = 0; i < n[0]; ++i) {
            int c[3] = {i, j, k};
            size_t id = cidx(l, c);
            if (cellbox[l][id] < 0) continue;
            cellmap[l][id] = (int)elem_level.size();
            elem_level.push_back((int8_t)l);
            elem_cell.insert(elem_cell.end(), {i, j, k});
          }
      lev_valid_cnt[l] = elem_level.size() - lev_valid_off[l];
    }
    n_valid_ = elem_level.size();
    if (n_valid_ == 0 || lev_valid_cnt[0] != (size_t)n_cell0[0] * n_cell0[1] * n_cell0[2]) {
      if (msg) *msg = "level 0 must cover the domain";
      return false;
    }
    // ---- ghost elements at coarse-fine boundaries (face neighbours only)
    gf_elem.clear();
    gf_parent.clear();
    gf_child.clear();
    for (int l = 1; l < nlev; ++l) {
      const size_t e0 = lev_valid_off[l], e1 = e0 + lev_valid_cnt[l];
      for (size_t e = e0; e < e1; ++e)
        for (int d = 0; d < D; ++d)
          for (int s = -1; s <= 1; s += 2) {
            int nb[3] = {elem_cell[3 * e], elem_cell[3 * e + 1], elem_cell[3 * e + 2]};
            nb[d] += s;
            if (!wrap(l, nb)) continue;
            size_t id = cidx(l, nb);
            if (cellmap[l][id] >= 0) continue;
            const int ge = (int)elem_level.size();
            cellmap[l][id] = ge;
            elem_level.push_back((int8_t)l);
            elem_cell.insert(elem_cell.end(), {nb[0], nb[1], nb[2]});
            int par[3] = {0, 0, 0}, child = 0;
            for (int a = 0; a < D; ++a) {
              par[a] = nb[a] >> 1;
              child += (nb[a] & 1) << (D - 1 - a);
            }
            const int pe = cellmap[l - 1][cidx(l - 1, par)];
            if (!is_valid_elem(pe)) {
              if (msg) *msg = "level " + std::to_string(l) + " is not properly nested in level " + std::to_string(l - 1);
              return false;
            }
            gf_elem.push_back(ge);
            gf_parent.push_back(pe);
            gf_child.push_back((int8_t)child);
          }
    }
    n_elem_ = elem_level.size();
    // ---- faces
    face_left.clear();
    face_right.clear();
    elem_face.assign(n_valid_ * 2 * D, -1);
    for (int d = 0; d < D; ++d) {
      face_off[d] = (int)face_left.size();
      for (int l = 0; l < nlev; ++l) {
        const size_t e0 = lev_valid_off[l], e1 = e0 + lev_valid_cnt[l];
        for (size_t e = e0; e < e1; ++e) {
          int nb[3] = {elem_cell[3 * e], elem_cell[3 * e + 1], elem_cell[3 * e + 2]};
          nb[d] -= 1;
          int left = elem_at(l, nb);
          int tmp[3] = {nb[0], nb[1], nb[2]};
          if (!wrap(l, tmp)) left = (int)e;  // outflow: zero-gradient mirror
          if (left < 0) {
            if (msg) *msg = "missing neighbour element";
            return false;
          }
          elem_face[e * 2 * D + 2 * d] = (int)face_left.size();
          face_left.push_back(left);
          face_right.push_back((int)e);
        }
        for (size_t e = e0; e < e1; ++e) {
          int nb[3] = {elem_cell[3 * e], elem_cell[3 * e + 1], elem_cell[3 * e + 2]};
          nb[d] += 1;
          int tmp[3] = {nb[0], nb[1], nb[2]};
          const bool inside = wrap(l, tmp);
          const int right = inside ? elem_at(l, nb) : (int)e;
          if (inside && is_valid_elem(right)) {
            elem_face[e * 2 * D + 2 * d + 1] = elem_face[(size_t)right * 2 * D + 2 * d];
          } else {
            if (right < 0) {
              if (msg) *msg = "missing neighbour element";
              return false;
            }
            elem_face[e * 2 * D + 2 * d + 1] = (int)face_left.size();
            face_left.push_back((int)e);
            face_right.push_back(right);
          }
        }
      }
    }
    face_off[D] = (int)face_left.size();
    for (int d = D + 1; d < 4; ++d) face_off[d] = face_off[D];
    // ---- coarse-fine flux corrections
    rf_elem.clear();
    rf_off.assign(1, 0);
    rf_face.clear();
    rf_dside.clear();
    rf_fine.clear();
    const int nfc = 1 << (D - 1);
    for (int l = 0; reflux && l + 1 < nlev; ++l) {
      const size_t e0 = lev_valid_off[l], e1 = e0 + lev_valid_cnt[l];
      for (size_t e = e0; e < e1; ++e) {
        const int* c = &elem_cell[3 * e];
        if (covered(l, c)) continue;
        const int nent0 = (int)rf_face.size();
        bool apply = !reflux_quirk;
        const amr::IBox& box = grids[l][cellbox[l][cidx(l, c)]];
        for (int d = 0; d < D; ++d)
          for (int side = 0; side < 2; ++side) {
            int nb[3] = {c[0], c[1], c[2]};
            nb[d] += side ? 1 : -1;
            if (!wrap(l, nb)) continue;
            if (!is_valid_elem(cellmap[l][cidx(l, nb)]) || !covered(l, nb)) continue;
            rf_face.push_back(elem_face[e * 2 * D + 2 * d + side]);
            rf_dside.push_back((int8_t)(2 * d + side));
            for (int k = 0; k < nfc; ++k) {
              int f[3] = {0, 0, 0}, bit = 0;
              for (int a = 0; a < D; ++a) {
                if (a == d) {
                  f[a] = side ? 2 * nb[a] : 2 * nb[a] + 1;
                } else {
                  f[a] = 2 * c[a] + ((k >> bit) & 1);
                  bit++;
                }
              }
              const int fe = cellmap[l + 1][cidx(l + 1, f)];
              if (!is_valid_elem(fe)) {
                if (msg) *msg = "coarse-fine face without fine cells";
                return false;
              }
              rf_fine.push_back(elem_face[(size_t)fe * 2 * D + 2 * d + (side ? 0 : 1)]);
            }
            if (side == 1 || c[d] > box.lo[d]) apply = true;
          }
        if ((int)rf_face.size() == nent0) continue;
        if (!apply) {  // the reference never applies these corrections
          rf_face.resize(nent0);
          rf_dside.resize(nent0);
          rf_fine.resize((size_t)nent0 * nfc);
          continue;
        }
        rf_elem.push_back((int)e);
        rf_off.push_back((int)rf_face.size());
      }
    }
    // ---- average down
    ad_rec.assign(nlev, {});
    for (int lf = 1; lf < nlev; ++lf) {
      const int l = lf - 1;
      const size_t e0 = lev_valid_off[l], e1 = e0 + lev_valid_cnt[l];
      for (size_t e = e0; e < e1; ++e) {
        const int* c = &elem_cell[3 * e];
        if (!covered(l, c)) continue;
        ad_rec[lf].push_back((int)e);
        for (int k = 0; k < (1 << D); ++k) {
          int f[3] = {0, 0, 0};
          for (int a = 0; a < D; ++a) f[a] = 2 * c[a] + ((k >> (D - 1 - a)) & 1);
          ad_rec[lf].push_back(cellmap[lf][cidx(lf, f)]);
        }
      }
    }
    return true;
  }
};

}  // namespace adg

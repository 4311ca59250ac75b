// Host layout of the packed element list: elements (valid cells of every
// level, then ghost elements), their faces and the face -> element tables the
// kernels index.  Replaces the box/MultiFab bookkeeping AMReX does for the
// reference (Source/Core/Mesh.h, Source/NumericalMethod/AmrDG/AmrDG_Level.tpp).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "adg.h"

namespace adg {

struct Hierarchy {
  int D = 2;
  int nlev = 0;
  int n_cell0[3] = {1, 1, 1};
  int periodic[3] = {1, 1, 1};
  std::vector<int> face_left, face_right;  // per face: element on each side
  int face_off[4] = {0, 0, 0, 0};          // faces of direction d: [face_off[d], face_off[d+1])
  std::vector<int> elem_face;              // [elem][2D]
  std::vector<int> elem_cell;              // [elem][3] cell index within its level
  std::vector<int8_t> elem_level;          // [elem]
  std::vector<size_t> lev_valid_off, lev_valid_cnt;
  size_t n_valid_ = 0, n_elem_ = 0;

  int nlevels() const { return nlev; }
  size_t n_valid() const { return n_valid_; }
  size_t n_elem() const { return n_elem_; }
  size_t level_valid_offset(int l) const { return lev_valid_off[l]; }
  size_t level_valid_count(int l) const { return lev_valid_cnt[l]; }

  // One level covering the domain; elements in x-fastest order.  Periodic
  // directions wrap; outflow boundaries get a face whose outer side is the
  // boundary element itself (zero-gradient mode copy: the ghost's polynomial
  // equals the interior one, so its trace at the shared face is the interior
  // element's trace on the opposite side).
  bool build_single_level(const adg_config& c, std::string* msg) {
    D = c.D;
    nlev = 1;
    long long n = 1;
    for (int d = 0; d < 3; ++d) {
      n_cell0[d] = d < D ? c.n_cell[d] : 1;
      periodic[d] = d < D ? c.periodic[d] : 1;
      n *= n_cell0[d];
    }
    if (n <= 0 || n > (1LL << 31) / 8) {
      if (msg) *msg = "level too large for 32-bit element indices";
      return false;
    }
    n_valid_ = n_elem_ = (size_t)n;
    lev_valid_off.assign(1, 0);
    lev_valid_cnt.assign(1, (size_t)n);
    elem_cell.resize((size_t)n * 3);
    elem_level.assign((size_t)n, 0);
    const int nx = n_cell0[0], ny = n_cell0[1], nz = n_cell0[2];
    auto lin = [&](int i, int j, int k) { return (int)(i + (long long)nx * (j + (long long)ny * k)); };
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          int e = lin(i, j, k);
          elem_cell[3 * e] = i;
          elem_cell[3 * e + 1] = j;
          elem_cell[3 * e + 2] = k;
        }
    elem_face.assign((size_t)n * 2 * D, -1);
    face_left.clear();
    face_right.clear();
    for (int d = 0; d < D; ++d) {
      face_off[d] = (int)face_left.size();
      const int nd = n_cell0[d];
      // low face of every element
      for (int e = 0; e < n; ++e) {
        int ijk[3] = {elem_cell[3 * e], elem_cell[3 * e + 1], elem_cell[3 * e + 2]};
        int nb[3] = {ijk[0], ijk[1], ijk[2]};
        nb[d] -= 1;
        int left;
        if (nb[d] >= 0)
          left = lin(nb[0], nb[1], nb[2]);
        else if (periodic[d]) {
          nb[d] += nd;
          left = lin(nb[0], nb[1], nb[2]);
        } else
          left = e;  // outflow: mirror
        elem_face[(size_t)e * 2 * D + 2 * d + 0] = (int)face_left.size();
        face_left.push_back(left);
        face_right.push_back(e);
      }
      // high faces: shared with the next element's low face, or a boundary face
      for (int e = 0; e < n; ++e) {
        int ijk[3] = {elem_cell[3 * e], elem_cell[3 * e + 1], elem_cell[3 * e + 2]};
        int nb[3] = {ijk[0], ijk[1], ijk[2]};
        nb[d] += 1;
        if (nb[d] < nd || periodic[d]) {
          if (nb[d] >= nd) nb[d] -= nd;
          int right = lin(nb[0], nb[1], nb[2]);
          elem_face[(size_t)e * 2 * D + 2 * d + 1] = elem_face[(size_t)right * 2 * D + 2 * d + 0];
        } else {
          elem_face[(size_t)e * 2 * D + 2 * d + 1] = (int)face_left.size();
          face_left.push_back(e);
          face_right.push_back(e);  // outflow: mirror
        }
      }
    }
    face_off[D] = (int)face_left.size();
    for (int d = D + 1; d < 4; ++d) face_off[d] = face_off[D];
    return true;
  }
};

}  // namespace adg

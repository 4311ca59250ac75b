// CPU oracle (test infrastructure only; never linked into the product).
//
// Stage-by-stage restatement of one ADER-DG time step of the reference,
// on a per-level "domain array" (the level's index space grown by one ghost
// layer; cells flagged valid / ghost / unused).  A cell that is a ghost of
// several boxes holds one value, exactly as the reference's per-box ghost
// copies agree after FillBoundary / FillPatch.
//
//   ADER sequence               Source/NumericalMethod/AmrDG/AmrDG.h:1071-1165
//   set_predictor               Source/NumericalMethod/AmrDG/AmrDG.tpp:495-537
//   get_H_from_H_w              Source/NumericalMethod/AmrDG/AmrDG.tpp:387-435
//   get_H_from_H_w_bd           Source/NumericalMethod/AmrDG/AmrDG.tpp:437-493
//   flux / flux_bd              Source/NumericalMethod/AmrDG/AmrDG.h:1167-1251
//   numflux + LLF               Source/NumericalMethod/AmrDG/AmrDG.tpp:539-650,
//                               Source/NumericalMethod/AmrDG/AmrDG_NumericalFlux.tpp:4-41
//   update_U_w                  Source/NumericalMethod/AmrDG/AmrDG.tpp:652-742
//   update_H_w                  Source/NumericalMethod/AmrDG/AmrDG.tpp:744-827
//   get_U_from_U_w              Source/NumericalMethod/AmrDG/AmrDG.tpp:337-385
//   set_Dt                      Source/NumericalMethod/AmrDG/AmrDG.h:1253-1357
//   set_initial_condition       Source/NumericalMethod/AmrDG/AmrDG.h:782-836
//   LpNorm_DG_AMR / L2 points   Source/NumericalMethod/AmrDG/AmrDG.h:1399-1655,
//                               Source/NumericalMethod/AmrDG/AmrDG_Quadrature.tpp:248-268
#pragma once

#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "oracle_basis.hpp"
#include "oracle_euler.hpp"

namespace oracle {

struct Box {
  int lo[3] = {0, 0, 0};
  int hi[3] = {0, 0, 0};
};

enum CellStatus : int8_t { ST_NONE = 0, ST_VALID = 1, ST_GHOST = 2 };

struct Level {
  int D = 2;
  int n[3] = {1, 1, 1};
  int g[3] = {0, 0, 0};
  int s[3] = {1, 1, 1};
  long ncell = 0;
  double dx[3] = {1, 1, 1};
  std::vector<Box> boxes;
  std::vector<int8_t> status;
  // component-major arrays: index = comp * ncell + cell
  std::vector<double> Uw, Hw, H, F, Hm, Hp, Fm, Fp, DFm, DFp, Fnum;

  long cell(int i, int j, int k) const {
    return ((long)(k + g[2]) * s[1] + (j + g[1])) * s[0] + (i + g[0]);
  }
  void coords(long c, int& i, int& j, int& k) const {
    i = (int)(c % s[0]) - g[0];
    long r = c / s[0];
    j = (int)(r % s[1]) - g[1];
    k = (int)(r / s[1]) - g[2];
  }
  bool in_array(int i, int j, int k) const {
    return i >= -g[0] && i < n[0] + g[0] && j >= -g[1] && j < n[1] + g[1] && k >= -g[2] && k < n[2] + g[2];
  }
};

struct SimConfig {
  int D = 2, P = 1;
  double gamma = 1.4;
  double c_dt = 0.5;
  int n_cell[3] = {32, 32, 1};
  double prob_lo[3] = {0, 0, 0};
  double prob_hi[3] = {10, 10, 1};
  int periodic[3] = {1, 1, 1};
  ICParams icp;
};

class Sim {
 public:
  SimConfig cfg;
  Elem el;
  int D, P, Q, Np_s, Np_st, qst, qbd, qs;
  std::vector<Level> lev;
  double Dt = 0.0;
  double t = 0.0;
  int nstep = 0;

  // Precomputed basis products (bitwise equal to the reference's on-the-fly
  // products, which are evaluated in the same order).
  std::vector<double> phi_st;     // [n][m]   space-time modes at ST points
  std::vector<double> phi_bd;     // [d][side][n][m]  ST modes at face ST points
  std::vector<double> phi_s;      // [n][m]   spatial modes at spatial points

  explicit Sim(const SimConfig& c) : cfg(c), el(c.D, c.P) {
    D = c.D;
    P = c.P;
    Q = D + 2;
    Np_s = el.Np_s;
    Np_st = el.Np_st;
    qst = el.qMp_st;
    qbd = el.qMp_st_bd;
    qs = el.qMp_s;
    build_tables();
  }

  void build_tables() {
    const GL& gl = el.gl;
    phi_st.assign((size_t)Np_st * qst, 0.0);
    for (int n = 0; n < Np_st; ++n)
      for (int m = 0; m < qst; ++m) {
        double phi = 1.0;
        for (int d = 0; d < D + 1; ++d) phi *= gl.val[el.mi_st[n][d]][gl.node_idx(m, d, D + 1)];
        phi_st[(size_t)n * qst + m] = phi;
      }
    phi_bd.assign((size_t)D * 2 * Np_st * qbd, 0.0);
    for (int d = 0; d < D; ++d)
      for (int side = 0; side < 2; ++side)
        for (int n = 0; n < Np_st; ++n)
          for (int m = 0; m < qbd; ++m) {
            double phi = 1.0;
            for (int a = 0; a <= D; ++a) {
              if (a == d)
                phi *= gl.bd_val[el.mi_st[n][a]][side];
              else
                phi *= gl.val[el.mi_st[n][a]][gl.node_idx(m, bd_free_pos(a, d), D)];
            }
            phi_bd[(((size_t)d * 2 + side) * Np_st + n) * qbd + m] = phi;
          }
    phi_s.assign((size_t)Np_s * qs, 0.0);
    for (int n = 0; n < Np_s; ++n)
      for (int m = 0; m < qs; ++m) {
        double phi = 1.0;
        for (int d = 0; d < D; ++d) phi *= gl.val[el.mi_s[n][d]][gl.node_idx(m, d, D)];
        phi_s[(size_t)n * qs + m] = phi;
      }
  }

  // ---------------------------------------------------------------- layout
  void define_level(int l, const std::vector<Box>& boxes) {
    if ((int)lev.size() <= l) lev.resize(l + 1);
    Level& L = lev[l];
    L.D = D;
    int r = 1 << l;
    for (int d = 0; d < 3; ++d) {
      L.n[d] = (d < D) ? cfg.n_cell[d] * r : 1;
      L.g[d] = (d < D) ? 1 : 0;
      L.s[d] = L.n[d] + 2 * L.g[d];
      L.dx[d] = (d < D) ? (cfg.prob_hi[d] - cfg.prob_lo[d]) / L.n[d] : 1.0;
    }
    L.ncell = (long)L.s[0] * L.s[1] * L.s[2];
    L.boxes = boxes;
    L.status.assign(L.ncell, ST_NONE);
    for (const Box& b : boxes) {
      int glo[3], ghi[3];
      for (int d = 0; d < 3; ++d) {
        glo[d] = b.lo[d] - L.g[d];
        ghi[d] = b.hi[d] + L.g[d];
      }
      for (int k = glo[2]; k <= ghi[2]; ++k)
        for (int j = glo[1]; j <= ghi[1]; ++j)
          for (int i = glo[0]; i <= ghi[0]; ++i) {
            long c = L.cell(i, j, k);
            bool valid = i >= b.lo[0] && i <= b.hi[0] && j >= b.lo[1] && j <= b.hi[1] && k >= b.lo[2] && k <= b.hi[2];
            if (valid)
              L.status[c] = ST_VALID;
            else if (L.status[c] == ST_NONE)
              L.status[c] = ST_GHOST;
          }
    }
    size_t nc = L.ncell;
    L.Uw.assign((size_t)Q * Np_s * nc, 0.0);
    L.Hw.assign((size_t)Q * Np_st * nc, 0.0);
    L.H.assign((size_t)Q * qst * nc, 0.0);
    L.F.assign((size_t)D * Q * qst * nc, 0.0);
    L.Hm.assign((size_t)Q * qbd * nc, 0.0);
    L.Hp.assign((size_t)Q * qbd * nc, 0.0);
    L.Fm.assign((size_t)Q * qbd * nc, 0.0);
    L.Fp.assign((size_t)Q * qbd * nc, 0.0);
    L.DFm.assign((size_t)Q * qbd * nc, 0.0);
    L.DFp.assign((size_t)Q * qbd * nc, 0.0);
    L.Fnum.assign((size_t)D * Q * qbd * nc, 0.0);
  }

  // Single level covering the whole domain with boxes of at most max_grid cells.
  void define_single_level(int max_grid) {
    std::vector<Box> boxes;
    int nb[3] = {1, 1, 1};
    for (int d = 0; d < D; ++d) nb[d] = (cfg.n_cell[d] + max_grid - 1) / max_grid;
    for (int bk = 0; bk < nb[2]; ++bk)
      for (int bj = 0; bj < nb[1]; ++bj)
        for (int bi = 0; bi < nb[0]; ++bi) {
          Box b;
          int bb[3] = {bi, bj, bk};
          for (int d = 0; d < 3; ++d) {
            if (d < D) {
              b.lo[d] = bb[d] * max_grid;
              b.hi[d] = std::min(cfg.n_cell[d], (bb[d] + 1) * max_grid) - 1;
            } else {
              b.lo[d] = b.hi[d] = 0;
            }
          }
          boxes.push_back(b);
        }
    lev.clear();
    define_level(0, boxes);
  }

  // --------------------------------------------------------- initial state
  // AmrDG.h:782-836: L2 projection of pde_IC at the spatial GL points, on the
  // grown box (valid and ghost cells).
  void set_initial_condition(int l) {
    Level& L = lev[l];
    const double* dx = L.dx;
#pragma omp parallel for schedule(static)
    for (long c = 0; c < L.ncell; ++c) {
      if (L.status[c] == ST_NONE) continue;
      int ijk[3];
      L.coords(c, ijk[0], ijk[1], ijk[2]);
      // linear index of the covering level-0 cell (periodically wrapped) for
      // the noise hash
      int w[3] = {0, 0, 0}, n0[3] = {1, 1, 1};
      for (int d = 0; d < D; ++d) {
        n0[d] = cfg.n_cell[d];
        w[d] = ijk[d] >> l;
        w[d] = ((w[d] % n0[d]) + n0[d]) % n0[d];
      }
      uint64_t cell_l0 = (uint64_t)w[0] + (uint64_t)n0[0] * ((uint64_t)w[1] + (uint64_t)n0[1] * (uint64_t)w[2]);
      std::vector<double> icv((size_t)Q * qs);
      for (int m = 0; m < qs; ++m) {
        double x[3] = {0, 0, 0};
        for (int d = 0; d < D; ++d) {
          double xc = cfg.prob_lo[d] + (ijk[d] + 0.5) * dx[d];
          x[d] = (dx[d] / 2.0) * el.xi_s[m][d] + xc;
        }
        for (int q = 0; q < Q; ++q) icv[(size_t)q * qs + m] = pde_IC(q, x, D, cfg.gamma, cfg.icp, cell_l0, m);
      }
      for (int q = 0; q < Q; ++q)
        for (int n = 0; n < Np_s; ++n) {
          double sum = 0.0;
          for (int m = 0; m < qs; ++m) sum += icv[(size_t)q * qs + m] * el.quadmat(n, m);
          L.Uw[((size_t)q * Np_s + n) * L.ncell + c] = (sum / (el.refMat_phiphi(n, el.mi_s, n, el.mi_s)));
        }
    }
  }

  // ------------------------------------------------------- ghost handling
  // Periodic wrap of index i in dim d; returns false if outside a
  // non-periodic domain.
  bool wrap(const Level& L, int d, int& i) const {
    if (i >= 0 && i < L.n[d]) return true;
    if (!cfg.periodic[d]) return false;
    i = ((i % L.n[d]) + L.n[d]) % L.n[d];
    return true;
  }

  // FillBoundary (same level, periodic) followed by the physical BC
  // (outflow = zero-gradient mode copy, AMReX foextrap semantics).
  // BoundaryCondition.h:303-324.
  // FillBoundary alone: ghost cells that are valid cells of the same level
  // (other boxes, periodic images) take their current data.
  void fill_internal(int l) {
    Level& L = lev[l];
    const int ncomp = Q * Np_s;
#pragma omp parallel for schedule(static)
    for (long c = 0; c < L.ncell; ++c) {
      if (L.status[c] != ST_GHOST) continue;
      int ijk[3];
      L.coords(c, ijk[0], ijk[1], ijk[2]);
      bool inside = true;
      int w[3] = {ijk[0], ijk[1], ijk[2]};
      for (int d = 0; d < D; ++d) inside = inside && wrap(L, d, w[d]);
      if (!inside) continue;
      long src = L.cell(w[0], w[1], w[2]);
      if (L.status[src] != ST_VALID) continue;
      for (int k = 0; k < ncomp; ++k) L.Uw[(size_t)k * L.ncell + c] = L.Uw[(size_t)k * L.ncell + src];
    }
  }

  void fill_boundary(int l) {
    Level& L = lev[l];
    const int ncomp = Q * Np_s;
    fill_internal(l);
    bool any_nonper = false;
    for (int d = 0; d < D; ++d) any_nonper = any_nonper || !cfg.periodic[d];
    if (!any_nonper) return;
#pragma omp parallel for schedule(static)
    for (long c = 0; c < L.ncell; ++c) {
      if (L.status[c] != ST_GHOST) continue;
      int ijk[3];
      L.coords(c, ijk[0], ijk[1], ijk[2]);
      bool outside = false;
      int w[3] = {ijk[0], ijk[1], ijk[2]};
      for (int d = 0; d < D; ++d) {
        if (cfg.periodic[d]) {
          w[d] = ((w[d] % L.n[d]) + L.n[d]) % L.n[d];
          continue;
        }
        if (w[d] < 0) { w[d] = 0; outside = true; }
        if (w[d] >= L.n[d]) { w[d] = L.n[d] - 1; outside = true; }
      }
      if (!outside) continue;
      long src = L.cell(w[0], w[1], w[2]);
      for (int k = 0; k < ncomp; ++k) L.Uw[(size_t)k * L.ncell + c] = L.Uw[(size_t)k * L.ncell + src];
    }
  }

  // ------------------------------------------------------- ADER stages
  bool active(const Level& L, long c) const { return L.status[c] != ST_NONE; }

  void set_predictor(int l) {  // AmrDG.tpp:495-537
    Level& L = lev[l];
#pragma omp parallel for schedule(static)
    for (long c = 0; c < L.ncell; ++c) {
      if (!active(L, c)) continue;
      for (int q = 0; q < Q; ++q)
        for (int n = 0; n < Np_st; ++n)
          L.Hw[((size_t)q * Np_st + n) * L.ncell + c] = (n < Np_s) ? L.Uw[((size_t)q * Np_s + n) * L.ncell + c] : 0.0;
    }
  }

  void get_H_from_H_w(int l) {  // AmrDG.tpp:387-435
    Level& L = lev[l];
#pragma omp parallel for schedule(static)
    for (long c = 0; c < L.ncell; ++c) {
      if (!active(L, c)) continue;
      for (int q = 0; q < Q; ++q) {
        double* h = &L.H[(size_t)q * qst * L.ncell];
        for (int m = 0; m < qst; ++m) h[(size_t)m * L.ncell + c] = 0.0;
        for (int n = 0; n < Np_st; ++n) {
          double hw = L.Hw[((size_t)q * Np_st + n) * L.ncell + c];
          const double* ph = &phi_st[(size_t)n * qst];
          for (int m = 0; m < qst; ++m) h[(size_t)m * L.ncell + c] += hw * ph[m];
        }
      }
    }
  }

  void flux_vol(int l, int d) {  // AmrDG.h:1167-1205 over all M = qMp_st points
    Level& L = lev[l];
#pragma omp parallel for schedule(static)
    for (long c = 0; c < L.ncell; ++c) {
      if (!active(L, c)) continue;
      for (int m = 0; m < qst; ++m) {
        double u[5];
        for (int q = 0; q < Q; ++q) u[q] = L.H[((size_t)q * qst + m) * L.ncell + c];
        for (int q = 0; q < Q; ++q)
          L.F[(((size_t)d * Q + q) * qst + m) * L.ncell + c] = pde_flux(d, q, u, D, cfg.gamma);
      }
    }
  }

  void update_H_w(int l) {  // AmrDG.tpp:744-827
    Level& L = lev[l];
    std::vector<double> dtdx(D);
    for (int d = 0; d < D; ++d) dtdx[d] = Dt / (double)L.dx[d];
#pragma omp parallel for schedule(static)
    for (long c = 0; c < L.ncell; ++c) {
      if (!active(L, c)) continue;
      std::vector<double> rhs(Np_st);
      for (int q = 0; q < Q; ++q) {
        for (int n = 0; n < Np_st; ++n) {
          double r = 0.0;
          for (int m = 0; m < Np_s; ++m) r += el.Mk_pred(n, m) * L.Uw[((size_t)q * Np_s + m) * L.ncell + c];
          rhs[n] = r;
        }
        for (int d = 0; d < D; ++d)
          for (int n = 0; n < Np_st; ++n) {
            double r = rhs[n];
            for (int m = 0; m < qst; ++m)
              r -= ((dtdx[d] * el.Sk_predVinv[d](n, m)) * L.F[(((size_t)d * Q + q) * qst + m) * L.ncell + c]);
            rhs[n] = r;
          }
        for (int n = 0; n < Np_st; ++n) {
          double hw = 0.0;
          for (int m = 0; m < Np_st; ++m) hw += el.Mk_h_w_inv(n, m) * rhs[m];
          L.Hw[((size_t)q * Np_st + n) * L.ncell + c] = hw;
        }
      }
    }
  }

  void get_H_from_H_w_bd(int l, int d, int side, std::vector<double>& Hb) {  // AmrDG.tpp:437-493
    Level& L = lev[l];
    const double* tab = &phi_bd[((size_t)d * 2 + side) * Np_st * qbd];
#pragma omp parallel for schedule(static)
    for (long c = 0; c < L.ncell; ++c) {
      if (!active(L, c)) continue;
      for (int q = 0; q < Q; ++q) {
        double* h = &Hb[(size_t)q * qbd * L.ncell];
        for (int m = 0; m < qbd; ++m) h[(size_t)m * L.ncell + c] = 0.0;
        for (int n = 0; n < Np_st; ++n) {
          double hw = L.Hw[((size_t)q * Np_st + n) * L.ncell + c];
          for (int m = 0; m < qbd; ++m) h[(size_t)m * L.ncell + c] += hw * tab[(size_t)n * qbd + m];
        }
      }
    }
  }

  void flux_bd(int l, int d, const std::vector<double>& Hb, std::vector<double>& Fb, std::vector<double>& DFb) {
    Level& L = lev[l];  // AmrDG.h:1207-1251
#pragma omp parallel for schedule(static)
    for (long c = 0; c < L.ncell; ++c) {
      if (!active(L, c)) continue;
      for (int m = 0; m < qbd; ++m) {
        double u[5];
        for (int q = 0; q < Q; ++q) u[q] = Hb[((size_t)q * qbd + m) * L.ncell + c];
        for (int q = 0; q < Q; ++q) {
          Fb[((size_t)q * qbd + m) * L.ncell + c] = pde_flux(d, q, u, D, cfg.gamma);
          DFb[((size_t)q * qbd + m) * L.ncell + c] = pde_dflux(d, u, D, cfg.gamma);
        }
      }
    }
  }

  // Faces that belong to some valid box: lo face of cell c along d where c
  // or its lower neighbour along d is valid.
  bool face_active(const Level& L, long c, int d) const {
    int ijk[3];
    L.coords(c, ijk[0], ijk[1], ijk[2]);
    int lo[3] = {ijk[0], ijk[1], ijk[2]};
    lo[d] -= 1;
    if (!L.in_array(lo[0], lo[1], lo[2])) return false;
    long cl = L.cell(lo[0], lo[1], lo[2]);
    return L.status[c] == ST_VALID || L.status[cl] == ST_VALID;
  }

  void numflux(int l, int d) {  // AmrDG.tpp:539-650 + LLF_numflux
    Level& L = lev[l];
    const long shift = (d == 0) ? 1 : (d == 1 ? L.s[0] : (long)L.s[0] * L.s[1]);
#pragma omp parallel for schedule(static)
    for (long c = 0; c < L.ncell; ++c) {
      if (!face_active(L, c, d)) continue;
      long cl = c - shift;
      for (int m = 0; m < qbd; ++m) {
        for (int q = 0; q < Q; ++q) {
          size_t o = ((size_t)q * qbd + m) * L.ncell;
          double uL = L.Hp[o + cl];
          double uR = L.Hm[o + c];
          double fL = L.Fp[o + cl];
          double fR = L.Fm[o + c];
          double DfL = L.DFp[o + cl];
          double DfR = L.DFm[o + c];
          double C = std::max(std::abs(DfL), std::abs(DfR));
          L.Fnum[(((size_t)d * Q + q) * qbd + m) * L.ncell + c] = 0.5 * ((fL + fR) - C * (uR - uL));
        }
      }
    }
  }

  void update_U_w(int l) {  // AmrDG.tpp:652-742
    Level& L = lev[l];
    std::vector<long> shift(D);
    for (int d = 0; d < D; ++d) shift[d] = (d == 0) ? 1 : (d == 1 ? L.s[0] : (long)L.s[0] * L.s[1]);
#pragma omp parallel for schedule(static)
    for (long c = 0; c < L.ncell; ++c) {
      if (L.status[c] != ST_VALID) continue;
      for (int q = 0; q < Q; ++q) {
        for (int n = 0; n < Np_s; ++n) {
          double rhs = 0.0;
          rhs += (el.Mk_corr(n, n) * L.Uw[((size_t)q * Np_s + n) * L.ncell + c]);
          for (int d = 0; d < D; ++d) {
            double S_norm = (Dt / (double)L.dx[d]);
            for (int m = 0; m < qst; ++m)
              rhs += S_norm * (el.Sk_corr[d](n, m) * L.F[(((size_t)d * Q + q) * qst + m) * L.ncell + c]);
            double Mbd_norm = (Dt / (double)L.dx[d]);
            const double* fn = &L.Fnum[(((size_t)d * Q + q) * qbd) * L.ncell];
            for (int m = 0; m < qbd; ++m)
              rhs -= (Mbd_norm * (el.Mkbdp[d](n, m) * fn[(size_t)m * L.ncell + c + shift[d]] -
                                  el.Mkbdm[d](n, m) * fn[(size_t)m * L.ncell + c]));
          }
          rhs /= el.Mk_corr(n, n);
          L.Uw[((size_t)q * Np_s + n) * L.ncell + c] = rhs;
        }
      }
    }
  }

  // One level's share of ADER (AmrDG.h:1095-1157), without flux registers.
  void ader_level(int l) {
    fill_boundary(l);
    set_predictor(l);
    for (int it = 0; it < P; ++it) {
      get_H_from_H_w(l);
      for (int d = 0; d < D; ++d) flux_vol(l, d);
      update_H_w(l);
    }
    get_H_from_H_w(l);
    for (int d = 0; d < D; ++d) {
      flux_vol(l, d);
      get_H_from_H_w_bd(l, d, 0, lev[l].Hm);
      flux_bd(l, d, lev[l].Hm, lev[l].Fm, lev[l].DFm);
      get_H_from_H_w_bd(l, d, 1, lev[l].Hp);
      flux_bd(l, d, lev[l].Hp, lev[l].Fp, lev[l].DFp);
      numflux(l, d);
    }
    update_U_w(l);
  }

  // ------------------------------------------------------------- set_Dt
  // AmrDG.h:1253-1357: CFL speed at spatial quadrature point m = 0.
  double compute_Dt() {
    double dt_min = 1.0;
    std::vector<double> dt_lev;
    for (size_t l = 0; l < lev.size(); ++l) {
      Level& L = lev[l];
      double dx_avg = 0.0;
      for (int d = 0; d < D; ++d) dx_avg += (double)L.dx[d];
      dx_avg /= (double)D;
      double CFL = (1.0 / (2.0 * (double)P + 1.0)) * (1.0 / (double)D);
      double lmin = 1.0;
      bool any = false;
#pragma omp parallel
      {
        double my = 0.0;
        bool myany = false;
#pragma omp for schedule(static)
        for (long c = 0; c < L.ncell; ++c) {
          if (L.status[c] != ST_VALID) continue;
          double u[5];
          for (int q = 0; q < Q; ++q) {
            double s = 0.0;
            for (int nn = 0; nn < Np_s; ++nn) s += L.Uw[((size_t)q * Np_s + nn) * L.ncell + c] * phi_s[(size_t)nn * qs + 0];
            u[q] = s;
          }
          double lambda_max = pde_cfl_lambda(0, u, D, cfg.gamma);
          for (int d = 1; d < D; ++d) lambda_max = std::max(lambda_max, pde_cfl_lambda(d, u, D, cfg.gamma));
          double dt_cfl = CFL * (dx_avg / lambda_max);
          if (!myany || dt_cfl < my) my = dt_cfl;
          myany = true;
        }
#pragma omp critical
        {
          if (myany && (!any || my < lmin)) lmin = my;
          any = any || myany;
        }
      }
      dt_lev.push_back(any ? lmin : 1.0);
    }
    if (!dt_lev.empty()) dt_min = *std::min_element(dt_lev.begin(), dt_lev.end());
    return cfg.c_dt * dt_min;
  }

  // ------------------------------------------------------------ norms
  // AmrDG_Quadrature.tpp:248-268
  static void NewtonRhapson(double& x, int n) {
    int niter = 1000;
    double TOL = 1e-15;
    for (int it = 0; it < niter; ++it) {
      double df = (std::assoc_legendre(n, 1, x)) / (std::sqrt(1.0 - std::pow(x, 2.0)));
      double f = std::legendre(n, x);
      double x_new = x - (f / df);
      double error = std::abs(x_new - x);
      x = x_new;
      if (error <= TOL) break;
    }
  }

  // AmrDG.h:1589-1655 (2(p+1) points per dimension)
  std::vector<double> l2_points_1d() const {
    int N = 2 * (P + 1);
    std::vector<double> pts;
    for (int i = 1; i <= N / 2; ++i) {
      double theta = M_PI * (i - 0.25) / ((double)N + 0.5);
      double xiq;
      if ((1 <= i) && (i <= (int)((1.0 / 3.0) * (double)N))) {
        xiq = (1 - 0.125 * (1.0 / std::pow(N, 2)) + 0.125 * (1.0 / std::pow(N, 3)) -
               (1.0 / 384.0) * (1.0 / std::pow(N, 4)) * (39.0 - 28.0 * (1.0 / std::pow(std::sin(theta), 2)))) *
              std::cos(theta);
      } else {
        xiq = (1.0 - (1.0 / (8.0 * std::pow((double)N, 2))) + (1.0 / (8.0 * std::pow((double)N, 3)))) * std::cos(theta);
      }
      NewtonRhapson(xiq, N);
      pts.push_back(xiq);
      pts.push_back(-xiq);
    }
    return pts;
  }

  // phi_s via the Legendre<P> recurrence (AmrDG_Basis.tpp:19-28)
  double phi_s_at(int idx, const double* x) const {
    double result = 1.0;
    for (int d = 0; d < D; ++d) result *= legendre_rec(el.mi_s[idx][d], x[d]);
    return result;
  }
};

}  // namespace oracle

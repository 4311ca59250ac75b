// CPU oracle (test infrastructure only; never linked into the product).
//
// Time loop of the reference (AmrDG::evolve, Source/NumericalMethod/AmrDG/AmrDG.h:853-1055)
// around the single-level ADER stages of oracle_solver.hpp.
#pragma once

#include <algorithm>
#include <vector>

#include "oracle_solver.hpp"

namespace oracle {

struct AmrConfig {
  int max_level = 0;
  int max_grid = 32;
  int blocking_factor = 8;
  int dtn_regrid = 4;
  int tag_kind = 0;
  double tag_threshold = 0.1;
  double grid_eff = 0.7;
  int n_error_buf = 1;
  int reflux_box_quirk = 1;
};

class AmrSim {
 public:
  Sim sim;
  AmrConfig amr;

  AmrSim(const SimConfig& s, const AmrConfig& a) : sim(s), amr(a) {}

  double init() {
    sim.define_single_level(amr.max_grid);
    sim.set_initial_condition(0);
    sim.t = 0.0;
    sim.nstep = 0;
    sim.Dt = sim.compute_Dt();
    return sim.Dt;
  }

  void ader() {
    for (int l = (int)sim.lev.size() - 1; l >= 0; --l) sim.ader_level(l);
  }

  double step() {
    ader();
    sim.nstep += 1;
    sim.t += sim.Dt;
    sim.Dt = sim.compute_Dt();
    return sim.Dt;
  }

  void predictor_only(int l) {
    sim.fill_boundary(l);
    sim.set_predictor(l);
    for (int it = 0; it < sim.P; ++it) {
      sim.get_H_from_H_w(l);
      for (int d = 0; d < sim.D; ++d) sim.flux_vol(l, d);
      sim.update_H_w(l);
    }
  }

  // Valid cells of level l in canonical order (x fastest over the level's
  // index space), element-major [cell][q][n].
  long get_uw(int l, double* out) const {
    const Level& L = sim.lev[l];
    long w = 0;
    const int nc = sim.Q * sim.Np_s;
    for (int k = 0; k < L.n[2]; ++k)
      for (int j = 0; j < L.n[1]; ++j)
        for (int i = 0; i < L.n[0]; ++i) {
          long c = L.cell(i, j, k);
          if (L.status[c] != ST_VALID) continue;
          for (int x = 0; x < nc; ++x) out[w * nc + x] = L.Uw[(size_t)x * L.ncell + c];
          ++w;
        }
    return w;
  }

  long set_uw(int l, const double* in) {
    Level& L = sim.lev[l];
    long w = 0;
    const int nc = sim.Q * sim.Np_s;
    for (int k = 0; k < L.n[2]; ++k)
      for (int j = 0; j < L.n[1]; ++j)
        for (int i = 0; i < L.n[0]; ++i) {
          long c = L.cell(i, j, k);
          if (L.status[c] != ST_VALID) continue;
          for (int x = 0; x < nc; ++x) L.Uw[(size_t)x * L.ncell + c] = in[w * nc + x];
          ++w;
        }
    return w;
  }

  // Whole grown array (x fastest), element-major. which: 0 U_w, 1 H_w.
  long get_grown(int l, int which, double* out) const {
    const Level& L = sim.lev[l];
    int nc = sim.Q * (which == 0 ? sim.Np_s : sim.Np_st);
    const std::vector<double>& a = (which == 0) ? L.Uw : L.Hw;
    for (long c = 0; c < L.ncell; ++c)
      for (int x = 0; x < nc; ++x) out[c * nc + x] = a[(size_t)x * L.ncell + c];
    return L.ncell;
  }

  long tags_valid(int, int8_t*) const { return 0; }

  // ------------------------------------------------------------------ norms
  // LpNorm_DG_AMR (AmrDG.h:1399-1655). other == nullptr: error against the
  // analytic initial condition; otherwise against the other DG solution.
  double norm(const AmrSim* other, int p, int q) const {
    const int D = sim.D;
    int N1;
    std::vector<double> pts1;
    if (p == 1) {
      N1 = sim.P + 1;
      pts1 = sim.el.gl.nodes;
    } else {
      N1 = 2 * (sim.P + 1);
      pts1 = sim.l2_points_1d();
    }
    int M = 1;
    for (int d = 0; d < D; ++d) M *= N1;
    std::vector<std::array<double, 3>> qp(M);
    for (int m = 0; m < M; ++m) {
      int rem = m;
      int idx[3] = {0, 0, 0};
      for (int d = D - 1; d >= 0; --d) {
        idx[d] = rem % N1;
        rem /= N1;
      }
      for (int d = 0; d < 3; ++d) qp[m][d] = (d < D) ? pts1[idx[d]] : 0.0;
    }
    std::vector<double> wq(M, 1.0);
    for (int m = 0; m < M; ++m) {
      double w = 1.0;
      for (int d = 0; d < D; ++d) w *= 2.0 / std::pow(std::assoc_legendre(N1, 1, qp[m][d]), 2);
      wq[m] = w;
    }
    // basis at the points
    std::vector<double> phi((size_t)sim.Np_s * M);
    for (int n = 0; n < sim.Np_s; ++n)
      for (int m = 0; m < M; ++m) phi[(size_t)n * M + m] = sim.phi_s_at(n, qp[m].data());

    double total = 0.0, V_amr = 0.0;
    for (size_t l = 0; l < sim.lev.size(); ++l) {
      const Level& L = sim.lev[l];
      double vol = 1.0;
      for (int d = 0; d < D; ++d) vol *= L.dx[d];
      double coeff = vol / std::pow(2.0, D);
      double lev_sum = 0.0;
      long nleaf = 0;
#pragma omp parallel for reduction(+ : lev_sum, nleaf) schedule(static)
      for (long c = 0; c < L.ncell; ++c) {
        if (L.status[c] != ST_VALID) continue;
        int ijk[3];
        L.coords(c, ijk[0], ijk[1], ijk[2]);
        if (covered(l, ijk)) continue;
        nleaf++;
        double cell = 0.0;
        for (int m = 0; m < M; ++m) {
          double u_h = 0.0;
          for (int n = 0; n < sim.Np_s; ++n) u_h += L.Uw[((size_t)q * sim.Np_s + n) * L.ncell + c] * phi[(size_t)n * M + m];
          double u;
          if (other == nullptr) {
            double x[3] = {0, 0, 0};
            for (int d = 0; d < D; ++d) {
              double xc = sim.cfg.prob_lo[d] + (ijk[d] + 0.5) * L.dx[d];
              x[d] = (L.dx[d] / 2.0) * qp[m][d] + xc;
            }
            uint64_t cl0 = 0;
            u = pde_IC(q, x, D, sim.cfg.gamma, sim.cfg.icp, cl0, 0);
          } else {
            const Level& O = other->sim.lev[l];
            u = 0.0;
            for (int n = 0; n < sim.Np_s; ++n) u += O.Uw[((size_t)q * sim.Np_s + n) * O.ncell + c] * phi[(size_t)n * M + m];
          }
          double f = std::pow(std::abs(u - u_h), (double)p);
          cell += f * wq[m];
        }
        lev_sum += cell * coeff;
      }
      total += lev_sum;
      V_amr += vol * (double)nleaf;
    }
    return std::pow(total / V_amr, 1.0 / (double)p);
  }

  // True if cell ijk of level l is covered by a valid cell of level l+1.
  bool covered(size_t l, const int* ijk) const {
    if (l + 1 >= sim.lev.size()) return false;
    const Level& F = sim.lev[l + 1];
    int f[3];
    for (int d = 0; d < 3; ++d) f[d] = (d < sim.D) ? 2 * ijk[d] : 0;
    return F.status[F.cell(f[0], f[1], f[2])] == ST_VALID;
  }
};

}  // namespace oracle

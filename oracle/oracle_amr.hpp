// CPU oracle (test infrastructure only; never linked into the product).
//
// Multi-level time loop of the reference around the single-level stages of
// oracle_solver.hpp:
//   evolve loop body             Source/NumericalMethod/AmrDG/AmrDG.h:935-1029
//   ADER + flux registers        Source/NumericalMethod/AmrDG/AmrDG.h:1071-1165
//   C-F flux projections         Source/NumericalMethod/AmrDG/AmrDG.tpp:554-647
//   C-F face masks (ownership)   Source/NumericalMethod/AmrDG/AmrDG_Level.tpp:240-414
//   AMR_flux_correction          Source/NumericalMethod/AmrDG/AmrDG_Level.tpp:416-446
//   L2ProjInterp::reflux         Source/NumericalMethod/AmrDG/AmrDG_Interpolater.tpp:7-72
//   amr_scatter / amr_gather     Source/NumericalMethod/AmrDG/AmrDG_Interpolater.tpp:344-398
//   FillPatch / FillFromCoarse   Source/NumericalMethod/AmrDG/AmrDG_Level.tpp:137-224
//   RemakeLevel / new level      Source/NumericalMethod/AmrDG/AmrDG_Level.tpp:52-132
// Third-party semantics the reference takes from AMReX (absent from the
// reference tree) are restated from AMReX's documented behaviour:
// FluxRegister CrseAdd/FineAdd/Reflux (face-summed fine fluxes, mult, and the
// -/+ orientation signs of Reflux), FillPatchTwoLevels (fine data first,
// coarse interpolation for the rest), and AmrCore regrid (shared with the
// product in ader-dg-amr_gb300/csrc/amr_grids.hpp).
#pragma once

#include <algorithm>
#include <map>
#include <vector>

#include "amr_grids.hpp"
#include "oracle_solver.hpp"

namespace oracle {

struct AmrConfig {
  int max_level = 0;
  int max_grid = 32;
  int blocking_factor = 8;
  int dtn_regrid = 4;
  // time-based regrid cadence (Mesh::dt_regrid, AmrDG.h:936-941; <= 0: off)
  double dt_regrid = 0.0;
  // 0 normalised density gradient, 1 pressure jump (this project's criteria);
  // 2 vortex radius r <= amr_c[l]^2, 3 KH characteristic TVB troubled cell
  // (the reference's pde_tag_cell_refinement, Compressible_Euler.h:606-685)
  int tag_kind = 0;
  double tag_threshold = 0.1;
  double amr_c[8] = {1, 1, 1, 1, 1, 1, 1, 1};
  // kind 2: 1 moves the tagging centre with the free stream (x0 + u_inf t)
  int tag_advect = 0;
  // analytic IC on every level (Solver::setValidationMode, Solver.h:711-734):
  // 0 off (projection), 1 with the ghost FillPatch of every level, 2 with
  // the finer levels' ghost cells left at the analytic projection
  int validation_mode = 0;
  // 1 skips the coarse-fine flux correction (the reference's NO REFLUX runs)
  int no_reflux = 0;
  double grid_eff = 0.7;
  int n_error_buf = 1;
  int reflux_box_quirk = 1;
  // TVB limiter (AmrDG.h:995-997): every t_limit steps (0: off), threshold
  // tvb_c[l] * tvb_M * h^2
  int t_limit = 0;
  double tvb_M = 0.0;
  double tvb_c[8] = {1, 1, 1, 1, 1, 1, 1, 1};
};

namespace A = adg::amr;

class AmrSim {
 public:
  Sim sim;
  AmrConfig amr;
  A::GridParams gp;
  std::vector<std::vector<A::IBox>> grids;
  bool first_step = true;
  double t_last_regrid = 0.0;
  int n_regrids = 0;
  // regrids that changed the layout, plus the first one (the reference's
  // n_regrids, AmrDG.h:968-983)
  int n_layout_changes = 0;
  long n_limited = 0;

  AmrSim(const SimConfig& s, const AmrConfig& a) : sim(s), amr(a) {
    gp.D = s.D;
    for (int d = 0; d < 3; ++d) {
      gp.n_cell0[d] = d < s.D ? s.n_cell[d] : 1;
      gp.periodic[d] = d < s.D ? s.periodic[d] : 1;
    }
    gp.max_level = a.max_level;
    gp.blocking_factor = a.blocking_factor;
    gp.max_grid = a.max_grid;
    gp.grid_eff = a.grid_eff;
    gp.n_error_buf = a.n_error_buf;
  }

  int D() const { return sim.D; }
  int finest() const { return (int)sim.lev.size() - 1; }

  static std::vector<Box> to_boxes(const std::vector<A::IBox>& v) {
    std::vector<Box> b(v.size());
    for (size_t i = 0; i < v.size(); ++i)
      for (int d = 0; d < 3; ++d) {
        b[i].lo[d] = v[i].lo[d];
        b[i].hi[d] = v[i].hi[d];
      }
    return b;
  }

  // ---------------------------------------------------------------- init
  double init() {
    if (amr.max_level == 0) {
      grids = {A::chop_max_size({full_domain(0)}, D(), amr.max_grid)};
      sim.lev.clear();
      sim.define_level(0, to_boxes(grids[0]));
      sim.set_initial_condition(0);
    } else {
      // AmrCore::InitFromScratch (Solver.h:567-571) tags the levels while
      // their state is still zero (set_init_data_component, AmrDG.tpp:306-307).
      // The geometric vortex criterion tags its disc; the data criteria see a
      // zero state (the reference's TVB test reads NaN eigenvectors there and
      // flags every cell), so every level starts as a full-domain grid.
      grids.clear();
      sim.lev.clear();
      if (amr.tag_kind == 2) {
        grids.push_back(A::chop_max_size({full_domain(0)}, D(), amr.max_grid));
        sim.define_level(0, to_boxes(grids[0]));
        // one new level per pass (AmrMesh::MakeNewGrids(time)), then passes
        // over all levels until the boxes stop changing (iterate_on_new_grids)
        for (int pass = 0; pass < amr.max_level + 4; ++pass) {
          std::vector<A::TagField> tags(grids.size());
          for (size_t l = 0; l < grids.size(); ++l) tags[l] = compute_tags((int)l);
          std::vector<std::vector<A::IBox>> ng = A::make_new_grids(gp, grids, tags);
          bool same = ng.size() == grids.size();
          for (size_t l = 0; same && l < ng.size(); ++l) same = same_boxes(ng[l], grids[l]);
          if (same) break;
          grids = ng;
          for (size_t l = 0; l < grids.size(); ++l) sim.define_level((int)l, to_boxes(grids[l]));
          sim.lev.resize(grids.size());
        }
      } else {
        for (int l = 0; l <= amr.max_level; ++l) {
          grids.push_back(A::chop_max_size({full_domain(l)}, D(), amr.max_grid));
          sim.define_level(l, to_boxes(grids[l]));
        }
      }
      // Solver::set_initial_condition (Solver.h:711-734): the analytic IC on
      // level 0, on finer levels too in validation mode, else the projection
      // of the coarser level (AMR_interpolate_initial_condition,
      // AmrDG_Level.tpp:134-137); then AMR_sync_initial_condition
      // (AmrDG_Level.tpp:94-120): average down after an analytic IC, and the
      // ghost cells of every level, coarsest first.
      sim.set_initial_condition(0);
      for (int l = 1; l <= finest(); ++l) {
        if (amr.validation_mode)
          sim.set_initial_condition(l);
        else
          fill_from_coarse(l, nullptr);
      }
      // Validation mode 2 leaves the finer levels' coarse-fine ghost cells
      // with their own analytic projection until the first step's FillPatch,
      // which is how the reference's recorded static-refinement convergence
      // runs were initialised (Source/PostProcessing/convergence.py:22-27);
      // mode 1 is the FillPatch of every level of the current
      // AMR_sync_initial_condition.
      if (amr.validation_mode)
        for (int l = finest(); l > 0; --l) average_down(l);
      for (int l = 0; l <= finest(); ++l)
        if (l == 0 || amr.validation_mode != 2) fill_patch(l);
    }
    sim.t = 0.0;
    sim.nstep = 0;
    t_last_regrid = 0.0;
    first_step = true;
    sim.Dt = sim.compute_Dt();
    return sim.Dt;
  }

  A::IBox full_domain(int l) const {
    A::IBox b;
    for (int d = 0; d < 3; ++d) {
      b.lo[d] = 0;
      b.hi[d] = d < D() ? (sim.cfg.n_cell[d] << l) - 1 : 0;
    }
    return b;
  }

  // ----------------------------------------------------------- cell utils
  // Periodic wrap; false if outside a non-periodic domain.
  bool wrap(const Level& L, int* c) const {
    for (int d = 0; d < D(); ++d) {
      if (c[d] >= 0 && c[d] < L.n[d]) continue;
      if (!sim.cfg.periodic[d]) return false;
      c[d] = ((c[d] % L.n[d]) + L.n[d]) % L.n[d];
    }
    return true;
  }

  bool valid_at(int l, const int* cin) const {
    const Level& L = sim.lev[l];
    int c[3] = {cin[0], cin[1], cin[2]};
    if (!wrap(L, c)) return false;
    return L.status[L.cell(c[0], c[1], c[2])] == ST_VALID;
  }

  bool covered(int l, const int* c) const {
    if (l + 1 > finest()) return false;
    int f[3] = {0, 0, 0};
    for (int d = 0; d < D(); ++d) f[d] = 2 * c[d];
    return valid_at(l + 1, f);
  }

  // amr_scatter (AmrDG_Interpolater.tpp:344-364): fine cell c of level l
  // from its coarse parent on level l-1 (periodically wrapped).
  bool scatter_into(int l, const int* c, double* out /*Q*Np_s element-major*/) const {
    const Level& C = sim.lev[l - 1];
    int cc[3] = {0, 0, 0}, idx = 0;
    int f[3] = {c[0], c[1], c[2]};
    const Level& F = sim.lev[l];
    if (!wrap(F, f)) return false;
    for (int d = 0; d < D(); ++d) {
      cc[d] = f[d] >> 1;
      idx += (f[d] - 2 * cc[d]) * (1 << (D() - 1 - d));
    }
    long src = C.cell(cc[0], cc[1], cc[2]);
    const int Ns = sim.Np_s;
    const Elem& el = sim.el;
    for (int q = 0; q < sim.Q; ++q)
      for (int n = 0; n < Ns; ++n) {
        double s = 0.0;
        for (int m = 0; m < Ns; ++m) {
          double mp = el.Minv(n, n) * el.P_cf[idx](n, m);  // (Minv * P_cf)(n, m)
          s += mp * C.Uw[((size_t)q * Ns + m) * C.ncell + src];
        }
        out[q * Ns + n] = s;
      }
    return true;
  }

  void put(Level& L, long c, const double* v) {
    const int nc = sim.Q * sim.Np_s;
    for (int k = 0; k < nc; ++k) L.Uw[(size_t)k * L.ncell + c] = v[k];
  }

  // InterpFromCoarseLevel with the L2 projection (AMR_FillFromCoarsePatch,
  // AmrDG_Level.tpp:137-166): every active cell of level l from level l-1.
  // old_valid: if given, cells that were valid on the old level l take the
  // old data (FillPatchTwoLevels used by RemakeLevel).
  void fill_from_coarse(int l, const Level* old) {
    Level& L = sim.lev[l];
    const int nc = sim.Q * sim.Np_s;
#pragma omp parallel for schedule(static)
    for (long c = 0; c < L.ncell; ++c) {
      if (L.status[c] == ST_NONE) continue;
      int ijk[3];
      L.coords(c, ijk[0], ijk[1], ijk[2]);
      if (old) {
        int w[3] = {ijk[0], ijk[1], ijk[2]};
        if (wrap(*old, w)) {
          long oc = old->cell(w[0], w[1], w[2]);
          if (old->status[oc] == ST_VALID) {
            for (int k = 0; k < nc; ++k) L.Uw[(size_t)k * L.ncell + c] = old->Uw[(size_t)k * old->ncell + oc];
            continue;
          }
        }
      }
      std::vector<double> v(nc);
      if (scatter_into(l, ijk, v.data()))
        for (int k = 0; k < nc; ++k) L.Uw[(size_t)k * L.ncell + c] = v[k];
      else
        for (int k = 0; k < nc; ++k) L.Uw[(size_t)k * L.ncell + c] = 0.0;
    }
  }

  // AMR_FillPatch (AmrDG_Level.tpp:172-224) on a zeroed copy: valid cells,
  // same-level periodic copies, coarse interpolation elsewhere in the
  // domain; outside a non-periodic domain the cells stay zero (the physical
  // BC is applied by FillBoundaryCells at the next ADER).
  void fill_patch(int l) {
    Level& L = sim.lev[l];
    const int nc = sim.Q * sim.Np_s;
    std::vector<double> out((size_t)nc * L.ncell, 0.0);
#pragma omp parallel for schedule(static)
    for (long c = 0; c < L.ncell; ++c) {
      if (L.status[c] == ST_NONE) continue;
      int ijk[3];
      L.coords(c, ijk[0], ijk[1], ijk[2]);
      int w[3] = {ijk[0], ijk[1], ijk[2]};
      if (!wrap(L, w)) continue;
      long src = L.cell(w[0], w[1], w[2]);
      if (L.status[src] == ST_VALID) {
        for (int k = 0; k < nc; ++k) out[(size_t)k * L.ncell + c] = L.Uw[(size_t)k * L.ncell + src];
      } else if (l > 0) {
        std::vector<double> v(nc);
        if (scatter_into(l, ijk, v.data()))
          for (int k = 0; k < nc; ++k) out[(size_t)k * L.ncell + c] = v[k];
      }
    }
    L.Uw.swap(out);
  }

  // average_down / amr_gather (AmrDG_Interpolater.tpp:283-342, 366-398).
  void average_down(int lf) {
    Level& C = sim.lev[lf - 1];
    const Level& F = sim.lev[lf];
    const int Ns = sim.Np_s, nov = 1 << D();
    const Elem& el = sim.el;
#pragma omp parallel for schedule(static)
    for (long c = 0; c < C.ncell; ++c) {
      if (C.status[c] != ST_VALID) continue;
      int ijk[3];
      C.coords(c, ijk[0], ijk[1], ijk[2]);
      if (!covered(lf - 1, ijk)) continue;
      for (int q = 0; q < sim.Q; ++q) {
        std::vector<double> sum(Ns, 0.0);
        for (int l = 0; l < nov; ++l) {
          int f[3] = {0, 0, 0};
          for (int d = 0; d < D(); ++d) f[d] = 2 * ijk[d] + ((l >> (D() - 1 - d)) & 1);
          long fc = F.cell(f[0], f[1], f[2]);
          for (int n = 0; n < Ns; ++n) {
            double s = 0.0;
            for (int m = 0; m < Ns; ++m) s += el.P_fc[l](n, m) * F.Uw[((size_t)q * Ns + m) * F.ncell + fc];
            sum[n] += s;
          }
        }
        for (int n = 0; n < Ns; ++n)
          C.Uw[((size_t)q * Ns + n) * C.ncell + c] = (1.0 / nov) * (el.Minv(n, n) * sum[n]);
      }
    }
  }

  // ------------------------------------------------------------ C-F masks
  // cf_mask of level l (AmrDG_Level.tpp:290-298): 1 on valid cells covered by
  // level l+1 (periodic images included), copied from the adjacent valid
  // cell outside a non-periodic domain, 0 elsewhere.
  int cf_mask(int l, const int* cin) const {
    const Level& L = sim.lev[l];
    int c[3] = {cin[0], cin[1], cin[2]};
    for (int d = 0; d < D(); ++d)
      if (!sim.cfg.periodic[d]) c[d] = std::min(std::max(c[d], 0), L.n[d] - 1);
    if (!wrap(L, c)) return 0;
    if (L.status[L.cell(c[0], c[1], c[2])] != ST_VALID) return 0;
    return covered(l, c) ? 1 : 0;
  }

  // cf_face_b_coarse of box b of level l at the low face of cell f along d
  // (AmrDG_Level.tpp:300-331), with the reference's ownership rule: the low
  // face of the box is never flagged in the box's own face array.
  int b_coarse(int l, const Box& b, int d, const int* f) const {
    if (f[d] == b.lo[d]) return 0;
    int left[3] = {f[0], f[1], f[2]};
    left[d] -= 1;
    int ml = cf_mask(l, left), mr = cf_mask(l, f);
    if (ml == mr) return 0;
    return (ml == 0) ? 1 : -1;
  }

  int vmask(int l, const int* cin) const {
    const Level& L = sim.lev[l];
    int c[3] = {cin[0], cin[1], cin[2]};
    for (int d = 0; d < D(); ++d)
      if (!sim.cfg.periodic[d] && (c[d] < 0 || c[d] >= L.n[d])) return 1;
    return valid_at(l, c) ? 1 : 0;
  }

  // cf_face_b_fine and cf_face_child_idx (AmrDG_Level.tpp:342-396).
  int b_fine(int l, int d, const int* f, int* child) const {
    int left[3] = {f[0], f[1], f[2]};
    left[d] -= 1;
    int vl = vmask(l, left), vr = vmask(l, f);
    if (vl == vr) return 0;
    int ci = 0, bit = 0;
    for (int dir = 0; dir < D(); ++dir) {
      if (dir == d) continue;
      if (f[dir] % 2 != 0) ci |= (1 << bit);
      bit++;
    }
    *child = ci;
    return (vl == 0) ? 1 : -1;
  }

  double face_jacobian(int l, int d) const {
    const Level& L = sim.lev[l];
    double dvol = 1.0;
    for (int a = 0; a < D(); ++a)
      if (a != d) dvol *= L.dx[a];
    return (sim.Dt / 2.0) * (dvol / std::pow(2.0, D() - 1));
  }

  // J * mat * fnum at face (lo face of cell f) of level l, into out[q*Ns+n].
  void face_project(int l, int d, const int* f, const Mat& mat, bool mat_first, double* out) const {
    const Level& L = sim.lev[l];
    const long c = L.cell(f[0], f[1], f[2]);
    const double J = face_jacobian(l, d);
    const int Ns = sim.Np_s, qbd = sim.qbd;
    for (int q = 0; q < sim.Q; ++q) {
      const double* fn = &L.Fnum[(((size_t)d * sim.Q + q) * qbd) * L.ncell];
      for (int n = 0; n < Ns; ++n) {
        double s = 0.0;
        for (int m = 0; m < qbd; ++m) {
          double fv = fn[(size_t)m * L.ncell + c];
          s += mat_first ? mat(n, m) * fv : fv * mat(n, m);
        }
        out[q * Ns + n] = s * J;
      }
    }
  }

  // ------------------------------------------------------ flux registers
  // Register of fine level lf: per fine box, per orientation (d, side),
  // values on the coarse faces of the coarsened box boundary.
  struct Reg {
    int box, d, side;
    A::IBox cb;                  // coarsened fine box
    std::vector<double> v;       // [tangential face][q*Ns+n]
  };

  static long tang_index(const A::IBox& cb, int D, int d, const int* f) {
    long idx = 0, mul = 1;
    for (int a = 0; a < D; ++a) {
      if (a == d) continue;
      idx += (f[a] - cb.lo[a]) * mul;
      mul *= (cb.hi[a] - cb.lo[a] + 1);
    }
    return idx;
  }

  std::vector<Reg> make_regs(int lf) const {
    std::vector<Reg> regs;
    const int nc = sim.Q * sim.Np_s;
    // orientation order of the reference's Reflux loop: low faces of every
    // direction, then high faces
    for (int side = 0; side < 2; ++side)
      for (int d = 0; d < D(); ++d)
        for (size_t b = 0; b < grids[lf].size(); ++b) {
          Reg r;
          r.box = (int)b;
          r.d = d;
          r.side = side;
          r.cb = A::coarsen(grids[lf][b], D(), 2);
          long nt = 1;
          for (int a = 0; a < D(); ++a)
            if (a != d) nt *= (r.cb.hi[a] - r.cb.lo[a] + 1);
          r.v.assign((size_t)nt * nc, 0.0);
          regs.push_back(r);
        }
    return regs;
  }

  // FineAdd (+1): fine C-F face fluxes summed over the coarse face.
  void fine_add(int lf, int d, std::vector<Reg>& regs) const {
    const int Ns = sim.Np_s, nc = sim.Q * Ns;
    const Elem& el = sim.el;
    for (Reg& r : regs) {
      if (r.d != d) continue;
      const Box b = to_boxes({grids[lf][r.box]})[0];
      const int fface = r.side == 0 ? b.lo[d] : b.hi[d] + 1;
      // loop over fine faces on this side
      int lo[3] = {b.lo[0], b.lo[1], b.lo[2]}, hi[3] = {b.hi[0], b.hi[1], b.hi[2]};
      lo[d] = hi[d] = fface;
      for (int k = lo[2]; k <= hi[2]; ++k)
        for (int j = lo[1]; j <= hi[1]; ++j)
          for (int i = lo[0]; i <= hi[0]; ++i) {
            int f[3] = {i, j, k}, child = 0;
            int bf = b_fine(lf, d, f, &child);
            if (bf == 0) continue;
            const Mat& P = (bf == 1) ? el.P_flux_high[d][child] : el.P_flux_low[d][child];
            std::vector<double> v(nc);
            face_project(lf, d, f, P, true, v.data());
            int cf[3] = {0, 0, 0};
            for (int a = 0; a < D(); ++a) cf[a] = (a == d) ? fface / 2 : (f[a] >> 1);
            long t = tang_index(r.cb, D(), d, cf);
            for (int x = 0; x < nc; ++x) r.v[(size_t)t * nc + x] += 1.0 * v[x];
          }
    }
  }

  // CrseAdd (-1): coarse C-F face fluxes of every coarse box whose face array
  // holds the face (periodic images included).
  void crse_add(int lc, int d, std::vector<Reg>& regs) const {
    const Level& C = sim.lev[lc];
    const int nc = sim.Q * sim.Np_s;
    const Elem& el = sim.el;
    const std::vector<Box> cboxes = to_boxes(grids[lc]);
    for (Reg& r : regs) {
      if (r.d != d) continue;
      const int cface = r.side == 0 ? r.cb.lo[d] : r.cb.hi[d] + 1;
      int lo[3] = {r.cb.lo[0], r.cb.lo[1], r.cb.lo[2]}, hi[3] = {r.cb.hi[0], r.cb.hi[1], r.cb.hi[2]};
      lo[d] = hi[d] = cface;
      for (int k = lo[2]; k <= hi[2]; ++k)
        for (int j = lo[1]; j <= hi[1]; ++j)
          for (int i = lo[0]; i <= hi[0]; ++i) {
            int f[3] = {i, j, k};
            long t = tang_index(r.cb, D(), d, f);
            // the face and its periodic images
            std::vector<std::array<int, 3>> imgs = {{f[0], f[1], f[2]}};
            if (sim.cfg.periodic[d]) {
              if (f[d] == 0) imgs.push_back({d == 0 ? C.n[0] : f[0], d == 1 ? C.n[1] : f[1], d == 2 ? C.n[2] : f[2]});
              if (f[d] == C.n[d]) imgs.push_back({d == 0 ? 0 : f[0], d == 1 ? 0 : f[1], d == 2 ? 0 : f[2]});
            }
            for (const auto& im : imgs)
              for (const Box& cb : cboxes) {
                bool in = true;
                for (int a = 0; a < D(); ++a) {
                  int lo_a = cb.lo[a], hi_a = cb.hi[a] + (a == d ? 1 : 0);
                  if (im[a] < lo_a || im[a] > hi_a) in = false;
                }
                if (!in) continue;
                int bc = b_coarse(lc, cb, d, im.data());
                if (bc == 0) continue;
                const Mat& M = (bc == 1) ? el.Mkbdp[d] : el.Mkbdm[d];
                std::vector<double> v(nc);
                face_project(lc, d, im.data(), M, false, v.data());
                for (int x = 0; x < nc; ++x) r.v[(size_t)t * nc + x] += -1.0 * v[x];
              }
          }
    }
  }

  // AMR_flux_correction: FluxRegister::Reflux into a zeroed correction
  // array, then L2ProjInterp::reflux applies it to coarse cells flagged at
  // a C-F face in their own box's face arrays.
  void reflux(int lf, const std::vector<Reg>& regs) {
    const int lc = lf - 1;
    Level& C = sim.lev[lc];
    const int Ns = sim.Np_s, nc = sim.Q * Ns;
    std::map<long, std::vector<double>> corr;
    for (const Reg& r : regs) {
      const int d = r.d;
      const int cface = r.side == 0 ? r.cb.lo[d] : r.cb.hi[d] + 1;
      int lo[3] = {r.cb.lo[0], r.cb.lo[1], r.cb.lo[2]}, hi[3] = {r.cb.hi[0], r.cb.hi[1], r.cb.hi[2]};
      lo[d] = hi[d] = cface;
      for (int k = lo[2]; k <= hi[2]; ++k)
        for (int j = lo[1]; j <= hi[1]; ++j)
          for (int i = lo[0]; i <= hi[0]; ++i) {
            int f[3] = {i, j, k};
            long t = tang_index(r.cb, D(), d, f);
            int cell[3] = {i, j, k};
            if (r.side == 0) cell[d] -= 1;
            if (!wrap(C, cell)) continue;
            long c = C.cell(cell[0], cell[1], cell[2]);
            if (C.status[c] != ST_VALID) continue;
            auto& v = corr[c];
            if (v.empty()) v.assign(nc, 0.0);
            const double sgn = r.side == 0 ? -1.0 : 1.0;
            for (int x = 0; x < nc; ++x) v[x] += sgn * r.v[(size_t)t * nc + x] / 1.0;
          }
    }
    double vol = 1.0;
    for (int a = 0; a < D(); ++a) vol *= C.dx[a];
    const double inv_jac = std::pow(2.0, D()) / vol;
    const std::vector<Box> cboxes = to_boxes(grids[lc]);
    for (auto& kv : corr) {
      const long c = kv.first;
      int ijk[3];
      C.coords(c, ijk[0], ijk[1], ijk[2]);
      bool at_interface = false;
      if (amr.reflux_box_quirk) {
        for (const Box& b : cboxes) {
          bool in = true;
          for (int a = 0; a < D(); ++a)
            if (ijk[a] < b.lo[a] || ijk[a] > b.hi[a]) in = false;
          if (!in) continue;
          for (int d = 0; d < D() && !at_interface; ++d) {
            int lof[3] = {ijk[0], ijk[1], ijk[2]}, hif[3] = {ijk[0], ijk[1], ijk[2]};
            hif[d] += 1;
            if (b_coarse(lc, b, d, lof) != 0 || b_coarse(lc, b, d, hif) != 0) at_interface = true;
          }
          break;
        }
      } else {
        at_interface = true;
      }
      if (!at_interface) continue;
      for (int q = 0; q < sim.Q; ++q)
        for (int n = 0; n < Ns; ++n) {
          double delta = inv_jac * (sim.el.Minv(n, n) * kv.second[q * Ns + n]);
          C.Uw[((size_t)q * Ns + n) * C.ncell + c] += delta;
        }
    }
  }

  // ----------------------------------------------------------------- ADER
  void ader() {
    const int F = finest();
    std::vector<std::vector<Reg>> regs(F + 1);
    for (int l = 1; l <= F; ++l) regs[l] = make_regs(l);
    for (int l = F; l >= 0; --l) {
      Sim& s = sim;
      s.fill_boundary(l);
      s.set_predictor(l);
      for (int it = 0; it < s.P; ++it) {
        s.get_H_from_H_w(l);
        for (int d = 0; d < D(); ++d) s.flux_vol(l, d);
        s.update_H_w(l);
      }
      s.get_H_from_H_w(l);
      for (int d = 0; d < D(); ++d) {
        s.flux_vol(l, d);
        s.get_H_from_H_w_bd(l, d, 0, s.lev[l].Hm);
        s.flux_bd(l, d, s.lev[l].Hm, s.lev[l].Fm, s.lev[l].DFm);
        s.get_H_from_H_w_bd(l, d, 1, s.lev[l].Hp);
        s.flux_bd(l, d, s.lev[l].Hp, s.lev[l].Fp, s.lev[l].DFp);
        s.numflux(l, d);
        if (F > 0) {
          if (l < F) crse_add(l, d, regs[l + 1]);
          if (l > 0) fine_add(l, d, regs[l]);
        }
      }
      s.update_U_w(l);
    }
    if (!amr.no_reflux)
      for (int l = F; l > 0; --l) reflux(l, regs[l]);
  }

  // ---------------------------------------------------------------- tags
  double tag_indicator(const Level& L, long c, const int* ijk) const {
    const int Ns = sim.Np_s, Dd = D();
    auto mean = [&](long cc, int q) { return L.Uw[((size_t)q * Ns + 0) * L.ncell + cc]; };
    auto pres = [&](long cc) {
      double ke = 0.0;
      for (int d = 0; d < Dd; ++d) ke = ke + (mean(cc, d + 1) * mean(cc, d + 1)) / mean(cc, 0);
      return (sim.cfg.gamma - 1.0) * (mean(cc, Dd + 1) - 0.5 * ke);
    };
    double ind = 0.0;
    for (int d = 0; d < Dd; ++d) {
      int a[3] = {ijk[0], ijk[1], ijk[2]}, b[3] = {ijk[0], ijk[1], ijk[2]};
      a[d] += 1;
      b[d] -= 1;
      long ca = L.cell(a[0], a[1], a[2]), cb = L.cell(b[0], b[1], b[2]);
      double v;
      if (amr.tag_kind == 0)
        v = std::abs(mean(ca, 0) - mean(cb, 0)) / (2.0 * mean(c, 0));
      else
        v = std::abs(pres(ca) - pres(cb)) / (2.0 * pres(c));
      ind = std::max(ind, v);
    }
    return ind;
  }

  // The reference's isentropic-vortex criterion (Compressible_Euler.h:615-644):
  // the cell centre within amr_c^2 of the vortex centre, distances wrapped
  // once by half the domain.  tag_advect moves the centre with the free
  // stream (the commented "+ u_infty * time" of that code).
  bool tag_vortex(const Level& L, const int* ijk, double amr_c_lev) const {
    const double x0 = sim.cfg.icp.xc, y0 = sim.cfg.icp.yc;
    const double Lx = sim.cfg.prob_hi[0] - sim.cfg.prob_lo[0];
    const double Ly = sim.cfg.prob_hi[1] - sim.cfg.prob_lo[1];
    const double x = sim.cfg.prob_lo[0] + (ijk[0] + 0.5) * L.dx[0];
    const double y = sim.cfg.prob_lo[1] + (ijk[1] + 0.5) * L.dx[1];
    double xc = x0, yc = y0;
    if (amr.tag_advect) {
      xc = x0 + sim.cfg.icp.u_inf * sim.t;
      yc = y0 + sim.cfg.icp.v_inf * sim.t;
    }
    double dxv = x - xc, dyv = y - yc;
    if (dxv > Lx / 2.0) dxv -= Lx;
    if (dxv < -Lx / 2.0) dxv += Lx;
    if (dyv > Ly / 2.0) dyv -= Ly;
    if (dyv < -Ly / 2.0) dyv += Ly;
    const double r = std::sqrt(dxv * dxv + dyv * dyv);
    return r <= std::pow(amr_c_lev, 2);
  }

  // The reference's Kelvin-Helmholtz criterion (Compressible_Euler.h:645-682):
  // per direction, the left eigenvectors at the cell mean project the linear
  // mode and the halved differences to the neighbours' means; a cell is
  // tagged as soon as one characteristic slope fails minmodB's TVB test
  // |slope| <= AMR_TVB_C[l] * amr_c[l] * h^2 (AmrDG_Limiter.tpp:40-61): the
  // differences only feed minmod's value, never the flag.
  bool tag_kh_tvb(int l, const Level& L, long c) const {
    const int Dd = D(), Q = sim.Q, Ns = sim.Np_s;
    double h = L.dx[0];
    for (int d = 1; d < Dd; ++d) h = std::min(h, L.dx[d]);
    const double thr = amr.tvb_c[l] * amr.amr_c[l] * std::pow(h, 2.0);
    auto U = [&](int q, int n, long cc) { return L.Uw[((size_t)q * Ns + n) * L.ncell + cc]; };
    double ub[5];
    for (int q = 0; q < Q; ++q) ub[q] = U(q, 0, c);
    for (int d = 0; d < Dd; ++d) {
      const int s = lin_mode(d);
      double R[5][5], Lm[5][5];
      eigenvectors(d, ub, Dd, sim.cfg.gamma, R, Lm);
      for (int q = 0; q < Q; ++q) {
        double Du = 0.0;
        for (int k = 0; k < Q; ++k) Du += Lm[q][k] * U(k, s, c);
        if (!(std::abs(Du) <= thr)) return true;
      }
    }
    return false;
  }

  // Spatial mode of degree one in direction d alone (get_lin_mode_idx).
  int lin_mode(int d) const {
    for (int n = 0; n < sim.Np_s; ++n) {
      bool ok = sim.el.mi_s[n][d] == 1;
      for (int a = 0; a < D(); ++a)
        if (a != d && sim.el.mi_s[n][a] != 0) ok = false;
      if (ok) return n;
    }
    return 0;
  }

  // AMR_tag_cell_refinement (AmrDG_TagCellRef.tpp:4-52): FillBoundary, then
  // the criterion on every valid cell.
  A::TagField compute_tags(int l) {
    sim.fill_boundary(l);
    const Level& L = sim.lev[l];
    A::TagField t;
    t.init(L.n);
    for (long c = 0; c < L.ncell; ++c) {
      if (L.status[c] != ST_VALID) continue;
      int ijk[3];
      L.coords(c, ijk[0], ijk[1], ijk[2]);
      bool tag;
      if (amr.tag_kind == 2)
        tag = tag_vortex(L, ijk, amr.amr_c[l]);
      else if (amr.tag_kind == 3)
        tag = tag_kh_tvb(l, L, c);
      else
        tag = tag_indicator(L, c, ijk) > amr.tag_threshold;
      if (tag) t.f[t.idx(ijk[0], ijk[1], ijk[2])] = 1;
    }
    return t;
  }

  long tags_valid(int l, int8_t* out) {
    A::TagField t = compute_tags(l);
    const Level& L = sim.lev[l];
    long w = 0;
    for (int k = 0; k < L.n[2]; ++k)
      for (int j = 0; j < L.n[1]; ++j)
        for (int i = 0; i < L.n[0]; ++i) {
          if (L.status[L.cell(i, j, k)] != ST_VALID) continue;
          out[w++] = (int8_t)t.f[t.idx(i, j, k)];
        }
    return w;
  }

  // --------------------------------------------------------------- regrid
  void regrid() {
    const int F = finest();
    const int max_crse = std::min(F, amr.max_level - 1);
    std::vector<A::TagField> tags(F + 1);
    for (int l = 0; l <= max_crse; ++l) tags[l] = compute_tags(l);
    for (int l = max_crse + 1; l <= F; ++l) tags[l].init(sim.lev[l].n);
    std::vector<std::vector<A::IBox>> ng = A::make_new_grids(gp, grids, tags);
    const int new_finest = (int)ng.size() - 1;
    bool coarse_changed = false, coarse_changed_any = false;
    for (int l = 1; l <= new_finest; ++l) {
      bool changed = l > F || !same_boxes(ng[l], grids[l]);
      if (l <= F) {
        if (changed || coarse_changed) {
          Level old = sim.lev[l];
          sim.define_level(l, to_boxes(ng[l]));
          grids[l] = ng[l];
          fill_from_coarse(l, &old);
        }
      } else {
        grids.resize(l + 1);
        grids[l] = ng[l];
        sim.define_level(l, to_boxes(ng[l]));
        fill_from_coarse(l, nullptr);
      }
      coarse_changed = changed;
      coarse_changed_any = coarse_changed_any || changed;
    }
    const bool changed_any = new_finest != F || coarse_changed_any;
    sim.lev.resize(new_finest + 1);
    grids.resize(new_finest + 1);
    n_regrids++;
    if (changed_any || first_step) n_layout_changes++;
  }

  static bool same_boxes(const std::vector<A::IBox>& a, const std::vector<A::IBox>& b) {
    if (a.size() != b.size()) return false;
    for (size_t i = 0; i < a.size(); ++i)
      for (int d = 0; d < 3; ++d)
        if (a[i].lo[d] != b[i].lo[d] || a[i].hi[d] != b[i].hi[d]) return false;
    return true;
  }

  // ----------------------------------------------------------------- step
  double step() {
    if (amr.max_level > 0) {
      // AmrDG.h:936-986: at the first step, every dtn_regrid steps, or once
      // dt_regrid of time has passed since the last regrid
      bool due = first_step || (amr.dtn_regrid > 0 && sim.nstep % amr.dtn_regrid == 0) ||
                 (amr.dt_regrid > 0 && sim.t - t_last_regrid >= amr.dt_regrid - 1e-12);
      if (due) {
        regrid();
        t_last_regrid = sim.t;
      }
      first_step = false;
    }
    ader();
    // limiter on the finest level only (AmrDG.h:990-997)
    if (amr.t_limit > 0 && sim.nstep % amr.t_limit == 0) n_limited += limit_tvb(finest());
    for (int l = finest(); l > 0; --l) average_down(l);
    if (amr.max_level > 0)
      for (int l = 0; l <= finest(); ++l) fill_patch(l);
    sim.nstep += 1;
    sim.t += sim.Dt;
    sim.Dt = sim.compute_Dt();
    return sim.Dt;
  }

  // TVB limiter of one level (Limiter_w + Limiter_linear_tvb,
  // AmrDG.h:1657-1855): after FillBoundary, per valid cell and direction the
  // left eigenvectors at the cell means project the linear mode and the
  // halved differences to the neighbours' means; minmodB limits each
  // characteristic slope; if any changed, all modes above the mean are
  // dropped and the linear modes take the right-eigenvector images.  The
  // cell means are never written, so the cells are independent.
  int limit_tvb(int l) {
    sim.fill_internal(l);
    Level& L = sim.lev[l];
    const int Dd = D(), Q = sim.Q, Ns = sim.Np_s;
    double h = L.dx[0];
    for (int d = 1; d < Dd; ++d) h = std::min(h, L.dx[d]);
    const double thr = amr.tvb_c[l] * amr.tvb_M * std::pow(h, 2.0);
    int lin[3] = {0, 0, 0};
    for (int d = 0; d < Dd; ++d)
      for (int n = 0; n < Ns; ++n) {
        bool ok = sim.el.mi_s[n][d] == 1;
        for (int a = 0; a < Dd; ++a)
          if (a != d && sim.el.mi_s[n][a] != 0) ok = false;
        if (ok) {
          lin[d] = n;
          break;
        }
      }
    auto U = [&](int q, int n, long c) -> double& { return L.Uw[((size_t)q * Ns + n) * L.ncell + c]; };
    int count = 0;
#pragma omp parallel for schedule(static) reduction(+ : count)
    for (long c = 0; c < L.ncell; ++c) {
      if (L.status[c] != ST_VALID) continue;
      int ijk[3];
      L.coords(c, ijk[0], ijk[1], ijk[2]);
      double ub[5], res[3][5];
      for (int q = 0; q < Q; ++q) ub[q] = U(q, 0, c);
      bool troubled = false;
      for (int d = 0; d < Dd; ++d) {
        int a[3] = {ijk[0], ijk[1], ijk[2]}, b[3] = {ijk[0], ijk[1], ijk[2]};
        a[d] -= 1;
        b[d] += 1;
        const long cm = L.cell(a[0], a[1], a[2]), cp = L.cell(b[0], b[1], b[2]);
        double R[5][5], Lm[5][5], v[5];
        eigenvectors(d, ub, Dd, sim.cfg.gamma, R, Lm);
        for (int q = 0; q < Q; ++q) {
          double Dm = 0.0, Dp = 0.0, Du = 0.0;
          for (int k = 0; k < Q; ++k) {
            Dm += 0.5 * Lm[q][k] * (ub[k] - U(k, 0, cm));
            Dp += 0.5 * Lm[q][k] * (U(k, 0, cp) - ub[k]);
            Du += Lm[q][k] * U(k, lin[d], c);
          }
          v[q] = minmodB(Du, Dm, Dp, thr);
          troubled = troubled || (v[q] != Du);
        }
        for (int q = 0; q < Q; ++q) {
          double sum = 0.0;
          for (int k = 0; k < Q; ++k) sum += R[q][k] * v[k];
          res[d][q] = sum;
        }
      }
      if (!troubled) continue;
      for (int q = 0; q < Q; ++q) {
        for (int n = 1; n < Ns; ++n) U(q, n, c) = 0.0;
        for (int d = 0; d < Dd; ++d) U(q, lin[d], c) = res[d][q];
      }
      ++count;
    }
    return count;
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

  long get_grown(int l, int which, double* out) const {
    const Level& L = sim.lev[l];
    int nc = sim.Q * (which == 0 ? sim.Np_s : sim.Np_st);
    const std::vector<double>& a = (which == 0) ? L.Uw : L.Hw;
    for (long c = 0; c < L.ncell; ++c)
      for (int x = 0; x < nc; ++x) out[c * nc + x] = a[(size_t)x * L.ncell + c];
    return L.ncell;
  }

  // ------------------------------------------------------------------ norms
  // LpNorm_DG_AMR (AmrDG.h:1399-1655) over leaf cells.  other == nullptr:
  // error against the analytic initial condition; otherwise against the
  // other solution (same layout).
  double norm(const AmrSim* other, int p, int q) const {
    const int Dd = D();
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
    for (int d = 0; d < Dd; ++d) M *= N1;
    std::vector<std::array<double, 3>> qp(M);
    for (int m = 0; m < M; ++m) {
      int rem = m, idx[3] = {0, 0, 0};
      for (int d = Dd - 1; d >= 0; --d) {
        idx[d] = rem % N1;
        rem /= N1;
      }
      for (int d = 0; d < 3; ++d) qp[m][d] = (d < Dd) ? pts1[idx[d]] : 0.0;
    }
    std::vector<double> wq(M, 1.0);
    for (int m = 0; m < M; ++m) {
      double w = 1.0;
      for (int d = 0; d < Dd; ++d) w *= 2.0 / std::pow(std::assoc_legendre(N1, 1, qp[m][d]), 2);
      wq[m] = w;
    }
    std::vector<double> phi((size_t)sim.Np_s * M);
    for (int n = 0; n < sim.Np_s; ++n)
      for (int m = 0; m < M; ++m) phi[(size_t)n * M + m] = sim.phi_s_at(n, qp[m].data());
    double total = 0.0, V_amr = 0.0;
    for (int l = 0; l <= finest(); ++l) {
      const Level& L = sim.lev[l];
      double vol = 1.0;
      for (int d = 0; d < Dd; ++d) vol *= L.dx[d];
      double coeff = vol / std::pow(2.0, Dd);
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
            for (int d = 0; d < Dd; ++d) {
              double xc = sim.cfg.prob_lo[d] + (ijk[d] + 0.5) * L.dx[d];
              x[d] = (L.dx[d] / 2.0) * qp[m][d] + xc;
            }
            u = pde_IC(q, x, Dd, sim.cfg.gamma, sim.cfg.icp, 0, 0);
          } else {
            const Level& O = other->sim.lev[l];
            u = 0.0;
            for (int n = 0; n < sim.Np_s; ++n) u += O.Uw[((size_t)q * sim.Np_s + n) * O.ncell + c] * phi[(size_t)n * M + m];
          }
          cell += std::pow(std::abs(u - u_h), (double)p) * wq[m];
        }
        lev_sum += cell * coeff;
      }
      total += lev_sum;
      V_amr += vol * (double)nleaf;
    }
    return std::pow(total / V_amr, 1.0 / (double)p);
  }
};

}  // namespace oracle

// CPU oracle (test infrastructure only; never linked into the product).
// C entry points used by the tests and by bench.py's CPU-baseline leg.
#include <cstdint>
#include <cstring>
#include <string>

#include "oracle_amr.hpp"

using namespace oracle;

extern "C" {

struct oracle_cfg {
  int D, P;
  double gamma, c_dt;
  int n_cell[3];
  double prob_lo[3], prob_hi[3];
  int periodic[3];
  int ic;
  double u_inf, v_inf, beta, xc, yc;
  uint64_t seed;
  double noise_amp;
  int max_grid;
  // AMR (max_level = 0: single level)
  int max_level;
  int blocking_factor;
  int dtn_regrid;
  int tag_kind;       // 0 density gradient, 1 pressure jump, 2 vortex radius, 3 KH TVB
  double tag_threshold;
  double grid_eff;
  int n_error_buf;
  int reflux_box_quirk;  // 1: reproduce the reference's per-box reflux mask
  int t_limit;           // TVB limiter every t_limit steps (0: off)
  double tvb_M;
  double tvb_c[8];       // per-level TVB coefficient
  double dt_regrid;      // regrid once this much time has passed (<= 0: off)
  double amr_c[8];       // per-level coefficient of tag kinds 2 and 3
  int tag_advect;        // kind 2: centre moves with the free stream
  int validation_mode;   // analytic IC on every level (1, 2: see AmrConfig)
  int no_reflux;         // 1: no coarse-fine flux correction
};

void* oracle_create(const oracle_cfg* c) {
  SimConfig s;
  s.D = c->D;
  s.P = c->P;
  s.gamma = c->gamma;
  s.c_dt = c->c_dt;
  for (int d = 0; d < 3; ++d) {
    s.n_cell[d] = c->n_cell[d];
    s.prob_lo[d] = c->prob_lo[d];
    s.prob_hi[d] = c->prob_hi[d];
    s.periodic[d] = c->periodic[d];
  }
  s.icp.ic = c->ic;
  s.icp.u_inf = c->u_inf;
  s.icp.v_inf = c->v_inf;
  s.icp.beta = c->beta;
  s.icp.xc = c->xc;
  s.icp.yc = c->yc;
  s.icp.seed = c->seed;
  s.icp.noise_amp = c->noise_amp;
  AmrConfig a;
  a.max_level = c->max_level;
  a.max_grid = c->max_grid > 0 ? c->max_grid : 32;
  a.blocking_factor = c->blocking_factor > 0 ? c->blocking_factor : 8;
  a.dtn_regrid = c->dtn_regrid;
  a.tag_kind = c->tag_kind;
  a.tag_threshold = c->tag_threshold;
  a.grid_eff = c->grid_eff > 0 ? c->grid_eff : 0.7;
  a.n_error_buf = c->n_error_buf >= 0 ? c->n_error_buf : 1;
  a.reflux_box_quirk = c->reflux_box_quirk;
  a.t_limit = c->t_limit;
  a.tvb_M = c->tvb_M;
  for (int l = 0; l < 8; ++l) a.tvb_c[l] = c->tvb_c[l];
  a.dt_regrid = c->dt_regrid;
  for (int l = 0; l < 8; ++l) a.amr_c[l] = c->amr_c[l];
  a.tag_advect = c->tag_advect;
  a.validation_mode = c->validation_mode;
  a.no_reflux = c->no_reflux;
  try {
    return new AmrSim(s, a);
  } catch (...) {
    return nullptr;
  }
}

void oracle_destroy(void* h) { delete (AmrSim*)h; }

long oracle_limited_count(void* h) { return ((AmrSim*)h)->n_limited; }

// Regrids that changed the layout, plus the first one (AmrDG.h:968-983).
int oracle_layout_changes(void* h) { return ((AmrSim*)h)->n_layout_changes; }

int oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

// Initial condition (+ initial AMR hierarchy) and the first Dt.
double oracle_init(void* h) { return ((AmrSim*)h)->init(); }

double oracle_get_dt(void* h) { return ((AmrSim*)h)->sim.Dt; }
void oracle_set_dt(void* h, double dt) { ((AmrSim*)h)->sim.Dt = dt; }
double oracle_get_time(void* h) { return ((AmrSim*)h)->sim.t; }

// One full time step of the reference's evolve loop body
// (regrid?, ADER, average down, FillPatch, t += Dt, set_Dt). Returns new Dt.
double oracle_step(void* h) { return ((AmrSim*)h)->step(); }

// The TVB limiter of the finest level on the current state; returns the
// cells it modified.
long oracle_limit(void* h) {
  AmrSim* s = (AmrSim*)h;
  return s->limit_tvb(s->finest());
}

// The ghost cells of every level from the valid data (the end-of-step
// FillPatch, AmrDG.h:1004-1013).
void oracle_fill_patch(void* h) {
  AmrSim* s = (AmrSim*)h;
  for (int l = 0; l <= s->finest(); ++l) s->fill_patch(l);
}

// Only the ADER part of a step with the current Dt (no Dt update).
void oracle_ader(void* h) { ((AmrSim*)h)->ader(); }

int oracle_num_levels(void* h) { return (int)((AmrSim*)h)->sim.lev.size(); }

// Boxes of a level: out[6*b + {lo0,lo1,lo2,hi0,hi1,hi2}]. Returns count.
int oracle_get_boxes(void* h, int l, int* out, int cap) {
  AmrSim* s = (AmrSim*)h;
  if (l < 0 || l >= (int)s->sim.lev.size()) return -1;
  const auto& bx = s->sim.lev[l].boxes;
  int n = (int)bx.size();
  for (int b = 0; b < n && b < cap; ++b)
    for (int d = 0; d < 3; ++d) {
      out[6 * b + d] = bx[b].lo[d];
      out[6 * b + 3 + d] = bx[b].hi[d];
    }
  return n;
}

// Valid cells of level l in box order then x-fastest order within each box,
// element-major [cell][q][n].  Returns number of cells written.
long oracle_get_uw(void* h, int l, double* out) { return ((AmrSim*)h)->get_uw(l, out); }
long oracle_set_uw(void* h, int l, const double* in) { return ((AmrSim*)h)->set_uw(l, in); }

// Whole grown level array, element-major [cell][q][n] with x fastest over
// the grown index space (for stage-level comparisons).
long oracle_get_uw_grown(void* h, int l, double* out) { return ((AmrSim*)h)->get_grown(l, 0, out); }
long oracle_get_hw_grown(void* h, int l, double* out) { return ((AmrSim*)h)->get_grown(l, 1, out); }

// Run only the predictor of level l (fill_boundary + set_predictor + P sweeps).
void oracle_predictor(void* h, int l) { ((AmrSim*)h)->predictor_only(l); }

// Lp error norm of component q over leaf cells (AmrDG.h:1399-1655):
// against the analytic IC (other == NULL) or another solution.
double oracle_norm(void* h, void* other, int p, int q) { return ((AmrSim*)h)->norm((AmrSim*)other, p, q); }

// Lp norm of component q of (other - this) over the leaf cells, the other
// solution given per level as valid cells in canonical order on this
// solution's layout (the reference's norm machinery applied to two DG
// solutions).
double oracle_norm_diff(void* h, const double* const* other_levels, int p, int q) {
  AmrSim* s = (AmrSim*)h;
  AmrSim tmp(*s);
  for (int l = 0; l < (int)tmp.sim.lev.size(); ++l) tmp.set_uw(l, other_levels[l]);
  return s->norm(&tmp, p, q);
}

// Tags of level l from the current state (1 per valid cell, box order).
long oracle_tags(void* h, int l, int8_t* out) { return ((AmrSim*)h)->tags_valid(l, out); }

// Element matrix export for structural tests.
int oracle_matrix(int D, int P, const char* name, int idx, double* out, int cap, int* rows, int* cols) {
  Elem e(D, P);
  const Mat* m = nullptr;
  std::string s(name);
  if (s == "V") m = &e.V;
  else if (s == "Vinv") m = &e.Vinv;
  else if (s == "Mk_h_w") m = &e.Mk_h_w;
  else if (s == "Mk_h_w_inv") m = &e.Mk_h_w_inv;
  else if (s == "Mk_pred") m = &e.Mk_pred;
  else if (s == "Mk_corr") m = &e.Mk_corr;
  else if (s == "quadmat") m = &e.quadmat;
  else if (s == "Minv") m = &e.Minv;
  else if (s == "Sk_pred") m = &e.Sk_pred[idx];
  else if (s == "Sk_predVinv") m = &e.Sk_predVinv[idx];
  else if (s == "Sk_corr") m = &e.Sk_corr[idx];
  else if (s == "Mkbdm") m = &e.Mkbdm[idx];
  else if (s == "Mkbdp") m = &e.Mkbdp[idx];
  else if (s == "P_cf") m = &e.P_cf[idx];
  else if (s == "P_fc") m = &e.P_fc[idx];
  else if (s == "P_flux_low") m = &e.P_flux_low[idx / 8][idx % 8];
  else if (s == "P_flux_high") m = &e.P_flux_high[idx / 8][idx % 8];
  if (!m) return -1;
  *rows = m->r;
  *cols = m->c;
  if ((int)m->a.size() > cap) return -2;
  std::memcpy(out, m->a.data(), m->a.size() * sizeof(double));
  return 0;
}

int oracle_gl_nodes(int P, double* nodes, double* weights) {
  GL g(P);
  for (int i = 0; i <= P; ++i) {
    nodes[i] = g.nodes[i];
    weights[i] = g.weights[i];
  }
  return P + 1;
}

}  // extern "C"

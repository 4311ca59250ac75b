// Compiled test of the zero-copy patch boundary through include/AmrDG_GB300.h
// built against the AMReX stand-in: a three-level Kelvin-Helmholtz hierarchy
// held in per-(level, q) FArrayBox-style device arrays (one ghost cell, boxes
// split differently from the library's own), stepped through the adapter,
// must equal bit for bit a context that steps its own packed state.
// Test infrastructure only; prints "ok ..." and exits 0 on success.
#include "amrex_standin.h"
// the adapter as a maintainer adds it to the reference
#include "AmrDG_GB300.h"

#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <array>

static int fails = 0;
#define EXPECT(c, msg)                                         \
  do {                                                         \
    if (!(c)) {                                                \
      std::fprintf(stderr, "FAIL %s:%d %s\n", __FILE__, __LINE__, msg); \
      ++fails;                                                 \
    }                                                          \
  } while (0)

static void ok(adg_ctx* c, int rc, const char* what) { adg_gb300::check(c, rc, what); }

static adg_config kh_config() {
  adg_config c{};
  c.D = 2;
  c.P = 3;
  c.gamma = 1.4;
  c.c_dt = 0.5;
  for (int d = 0; d < 3; ++d) {
    c.n_cell[d] = d < 2 ? 16 : 1;
    c.prob_lo[d] = 0.0;
    c.prob_hi[d] = 1.0;
    c.periodic[d] = 1;
  }
  c.ic = ADG_IC_KH_NOISE;
  c.seed = 12345;
  c.noise_amp = 1e-3;
  c.max_grid = 16;
  c.max_level = 2;
  c.blocking_factor = 8;
  c.dtn_regrid = 4;
  c.tag_kind = ADG_TAG_DENSITY_GRADIENT;
  c.tag_threshold = 0.1;
  c.grid_eff = 0.7;
  c.n_error_buf = 1;
  c.reflux_box_quirk = 0;  // corrections independent of how the boxes are cut
  return c;
}

struct Hier {
  std::vector<amrex::BoxArray> ba;
  std::vector<std::vector<amrex::MultiFab*>> mf;  // [level][q]
  amrex::MultiFab& operator()(int l, int q) { return *mf[l][q]; }
  ~Hier() {
    for (auto& v : mf)
      for (auto* m : v) delete m;
  }
};

// The layout of ctx with every box cut in two along x where it is wide
// enough, and MultiFabs over it filled with NaN bytes.
static void make_hierarchy(adg_ctx* ctx, int Q, int Np_s, Hier& H) {
  int nlev = 0;
  ok(ctx, adg_num_levels(ctx, &nlev), "levels");
  for (int l = 0; l < nlev; ++l) {
    std::vector<int> b(6 * 4096);
    int nb = 0;
    ok(ctx, adg_get_boxes(ctx, l, b.data(), 4096, &nb), "boxes");
    amrex::BoxArray ba;
    for (int i = 0; i < nb; ++i) {
      amrex::Box bx;
      for (int d = 0; d < 3; ++d) {
        bx.lo[d] = b[6 * i + d];
        bx.hi[d] = b[6 * i + 3 + d];
      }
      if (bx.length(0) >= 4) {
        amrex::Box a = bx, c = bx;
        a.hi[0] = bx.lo[0] + bx.length(0) / 2 - 1;
        c.lo[0] = a.hi[0] + 1;
        ba.boxes.push_back(a);
        ba.boxes.push_back(c);
      } else {
        ba.boxes.push_back(bx);
      }
    }
    H.ba.push_back(ba);
    H.mf.emplace_back();
    for (int q = 0; q < Q; ++q) {
      auto* m = new amrex::MultiFab();
      m->define(ba, Np_s, 1);
      for (int f = 0; f < m->nfabs(); ++f)
        cudaMemset(m->fab(f).d, 0xFF, (size_t)m->fab(f).bx.numPts() * Np_s * sizeof(double));
      H.mf.back().push_back(m);
    }
  }
}

// Host copy of the valid cells of the hierarchy in the packed order of ctx's
// level l; ghost cells checked to still hold the NaN pattern.
static std::vector<double> gather_host(adg_ctx* ctx, Hier& H, int l, int Q, int Np_s, bool* ghosts_untouched) {
  int64_t n = 0;
  ok(ctx, adg_level_cells(ctx, l, &n), "cells");
  std::vector<int> ijk(3 * n);
  ok(ctx, adg_level_cell_coords(ctx, l, ijk.data()), "coords");
  std::vector<std::vector<std::vector<double>>> host(Q);  // [q][fab]
  for (int q = 0; q < Q; ++q)
    for (int f = 0; f < H(l, q).nfabs(); ++f) {
      auto& fab = H(l, q).fab(f);
      std::vector<double> v((size_t)fab.bx.numPts() * Np_s);
      cudaMemcpy(v.data(), fab.d, v.size() * sizeof(double), cudaMemcpyDeviceToHost);
      host[q].push_back(std::move(v));
    }
  std::vector<double> out((size_t)n * Q * Np_s);
  std::vector<std::vector<char>> seen(H(l, 0).nfabs());
  for (int f = 0; f < H(l, 0).nfabs(); ++f) seen[f].assign(H(l, 0).fab(f).bx.numPts(), 0);
  for (int64_t e = 0; e < n; ++e) {
    const int i = ijk[3 * e], j = ijk[3 * e + 1];
    int f = -1;
    for (int b = 0; b < H.ba[l].size(); ++b) {
      const amrex::Box& v = H.ba[l].boxes[b];
      if (i >= v.lo[0] && i <= v.hi[0] && j >= v.lo[1] && j <= v.hi[1]) f = b;
    }
    if (f < 0) continue;
    const amrex::Box& g = H(l, 0).fab(f).bx;
    const long long pts = g.numPts(), off = (i - g.lo[0]) + (long long)(j - g.lo[1]) * g.length(0);
    seen[f][off] = 1;
    for (int q = 0; q < Q; ++q)
      for (int m = 0; m < Np_s; ++m) out[((size_t)e * Q + q) * Np_s + m] = host[q][f][off + m * pts];
  }
  bool untouched = true;
  for (int q = 0; q < Q; ++q)
    for (int f = 0; f < H(l, q).nfabs(); ++f) {
      const long long pts = H(l, q).fab(f).bx.numPts();
      for (long long o = 0; o < pts; ++o)
        if (!seen[f][o])
          for (int m = 0; m < Np_s; ++m) untouched = untouched && std::isnan(host[q][f][o + m * pts]);
    }
  *ghosts_untouched = untouched;
  return out;
}

static std::vector<double> state(adg_ctx* ctx, int l, int Q, int Np_s) {
  int64_t n = 0;
  ok(ctx, adg_level_cells(ctx, l, &n), "cells");
  std::vector<double> v((size_t)n * Q * Np_s);
  ok(ctx, adg_get_state(ctx, l, v.data(), ADG_MEM_HOST), "get_state");
  return v;
}

int main() {
  try {
    const adg_config cfg = kh_config();
    const int Q = 4, Np_s = 10;
    // the library-owned run: its own layout and packed state
    adg_ctx* A = nullptr;
    ok(nullptr, adg_ctx_create(&cfg, &A), "create");
    ok(A, adg_init(A), "init");
    ok(A, adg_step(A), "step");  // the first step regrids from the full-domain start
    int nlev = 0;
    ok(A, adg_num_levels(A, &nlev), "levels");
    EXPECT(nlev == 3, "three levels after the first regrid");

    // the caller's hierarchy (AMReX side), boxes cut differently
    Hier H;
    make_hierarchy(A, Q, Np_s, H);
    std::vector<adg_patch> pa = adg_gb300::patches_of(H, nlev, Q);
    ok(A, adg_set_patches(A, pa.data(), (int)pa.size()), "set_patches on A");
    ok(A, adg_write_patches(A), "write_patches");
    ok(A, adg_synchronize(A), "sync");
    long long ncells = 0;
    for (int l = 0; l < nlev; ++l) {
      bool untouched = false;
      std::vector<double> got = gather_host(A, H, l, Q, Np_s, &untouched);
      std::vector<double> ref = state(A, l, Q, Np_s);
      EXPECT(got.size() == ref.size() && std::memcmp(got.data(), ref.data(), ref.size() * 8) == 0,
             "written patches hold the packed state");
      EXPECT(untouched, "ghost cells are the caller's");
      ncells += (long long)ref.size() / (Q * Np_s);
    }

    // the adapter's context, bound to the caller's arrays
    adg_gb300::Context B;
    B.create(cfg);
    B.bind(H.ba, H);
    double dt = 0.0;
    ok(A, adg_get_dt(A, &dt), "dt");
    ok(B.ctx, adg_set_dt(B.ctx, dt), "set dt");

    // three evolve-loop bodies (A regrids again only at its fourth step)
    const int steps = 3;
    double ms = 0.0;
    for (int s = 0; s < steps; ++s) {
      auto t0 = std::chrono::steady_clock::now();
      const double dtb = B.step();
      ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      ok(A, adg_step(A), "step A");
      double dta = 0.0;
      ok(A, adg_get_dt(A, &dta), "dt A");
      EXPECT(dta == dtb, "same Dt");
    }
    // one ADER stage through the adapter
    ok(A, adg_get_dt(A, &dt), "dt");
    B.ADER(dt);
    ok(A, adg_ader(A), "ader A");
    for (int l = 0; l < nlev; ++l) {
      bool untouched = false;
      std::vector<double> got = gather_host(B.ctx, H, l, Q, Np_s, &untouched);
      std::vector<double> ref = state(A, l, Q, Np_s);
      EXPECT(got.size() == ref.size() && std::memcmp(got.data(), ref.data(), ref.size() * 8) == 0,
             "adapter run equals the packed run bit for bit");
      EXPECT(untouched, "ghost cells are the caller's");
    }

    // errors: an incomplete tiling, and patches of an old layout
    std::vector<adg_patch> part(pa.begin(), pa.end() - 1);
    EXPECT(adg_set_patches(B.ctx, part.data(), (int)part.size()) == ADG_ERR_LAYOUT, "uncovered cells rejected");
    std::vector<int> nb = {1};
    std::vector<int> box = {0, 0, 0, 15, 15, 0};
    ok(B.ctx, adg_set_layout(B.ctx, 1, nb.data(), box.data()), "single level layout");
    EXPECT(adg_read_patches(B.ctx) == ADG_ERR_LAYOUT, "patches of an old layout rejected");

    adg_ctx_destroy(A);
    if (fails) return 1;
    std::printf("ok %lld cells in %d patches (the library's boxes cut in two), %d steps + 1 ADER bit for bit, "
                "%.3f ms per adapter step\n",
                ncells, (int)pa.size(), steps, ms / steps);
    return 0;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "FAIL exception: %s\n", e.what());
    return 1;
  }
}

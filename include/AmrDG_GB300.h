// AmrDG_GB300.h -- C++ adapter between the reference's AMReX data and the
// GB300 ADER-DG library (adg.h).
//
// The reference advances its hierarchy with AmrDG<P>::ADER
// (Source/NumericalMethod/AmrDG/AmrDG.h:1071-1165) on one MultiFab per
// (level, q), U_w(l, q), whose FArrayBoxes hold the Np_s modes as components
// with nghost ghost cells (AmrDG.tpp:300-333).  This header binds those
// MultiFabs to a library context without a host copy: the context mirrors
// the BoxArrays (adg_set_layout), the FArrayBoxes are registered as patches
// (adg_set_patches), and every step gathers the valid cells on the device,
// runs the library's step and scatters them back (adg_read_patches,
// adg_write_patches).  The MultiFab data must be device memory (an AMReX
// GPU build); ghost cells stay the caller's (its FillPatch).
//
// It uses only these AMReX names, so a stand-in with the same interface
// builds it too: amrex::MFIter (constructed from a MultiFab; isValid,
// operator++, validbox), MultiFab::nGrow, MultiFab::operator[](MFIter) ->
// FArrayBox with box() (the grown box) and dataPtr(), Box::smallEnd,
// Box::bigEnd, Box::length, BoxArray::size, BoxArray::operator[](int) -> Box,
// amrex::Abort, and the macro AMREX_SPACEDIM.
#ifndef AMRDG_GB300_H
#define AMRDG_GB300_H

#include <string>
#include <vector>

#include "adg.h"

namespace adg_gb300 {

inline void check(adg_ctx* c, int rc, const char* what) {
  if (rc != ADG_OK)
    amrex::Abort(std::string("adg: ") + what + ": " + (c ? adg_last_error(c) : "status " + std::to_string(rc)));
}

// The patches of the hierarchy: every FArrayBox of U_w(l, 0 .. Q-1) for
// l < nlev (the Q MultiFabs of a level share BoxArray and ghost width).
template <class UW>
std::vector<adg_patch> patches_of(UW& U_w, int nlev, int Q) {
  std::vector<adg_patch> out;
  for (int l = 0; l < nlev; ++l) {
    auto& mf0 = U_w(l, 0);
    for (amrex::MFIter mfi(mf0); mfi.isValid(); ++mfi) {
      adg_patch p{};
      p.level = l;
      const auto vb = mfi.validbox();
      const auto gb = mf0[mfi].box();
      long long len[3] = {1, 1, 1};
      for (int d = 0; d < 3; ++d) {
        p.lo[d] = d < AMREX_SPACEDIM ? vb.smallEnd(d) : 0;
        p.hi[d] = d < AMREX_SPACEDIM ? vb.bigEnd(d) : 0;
        if (d < AMREX_SPACEDIM) len[d] = gb.length(d);
      }
      p.nghost = mf0.nGrow();
      p.jstride = len[0];
      p.kstride = len[0] * len[1];
      p.nstride = len[0] * len[1] * len[2];
      for (int q = 0; q < Q && q < 5; ++q) p.U_w[q] = U_w(l, q)[mfi].dataPtr();
      out.push_back(p);
    }
  }
  return out;
}

// One library context per solver.
struct Context {
  adg_ctx* ctx = nullptr;
  int Q = 0;

  Context() = default;
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
  ~Context() {
    if (ctx) adg_ctx_destroy(ctx);
  }

  // From AmrDG<P>::init (AmrDG.tpp:82-246): the element operators for (D, P)
  // and the level-0 geometry.  The context follows the caller's regrids
  // (dtn_regrid = 0).
  void create(adg_config c) {
    c.dtn_regrid = 0;
    c.dt_regrid = 0.0;
    if (c.ic < 0) c.ic = ADG_IC_CONST;  // the state comes from the MultiFabs
    check(nullptr, adg_ctx_create(&c, &ctx), "adg_ctx_create");
    check(ctx, adg_init(ctx), "adg_init");
    Q = c.D + 2;
  }

  // After Mesh::regrid (Mesh.h:156-196) or a restart: the BoxArray of every
  // level, then the arrays of the (re)allocated MultiFabs.
  template <class BA, class UW>
  void bind(const std::vector<BA>& ba, UW& U_w) {
    std::vector<int> nbox, boxes;
    for (const auto& b : ba) {
      nbox.push_back((int)b.size());
      for (int i = 0; i < (int)b.size(); ++i) {
        const auto bx = b[i];
        for (int d = 0; d < 3; ++d) boxes.push_back(d < AMREX_SPACEDIM ? bx.smallEnd(d) : 0);
        for (int d = 0; d < 3; ++d) boxes.push_back(d < AMREX_SPACEDIM ? bx.bigEnd(d) : 0);
      }
    }
    check(ctx, adg_set_layout(ctx, (int)ba.size(), nbox.data(), boxes.data()), "adg_set_layout");
    std::vector<adg_patch> p = patches_of(U_w, (int)ba.size(), Q);
    check(ctx, adg_set_patches(ctx, p.data(), (int)p.size()), "adg_set_patches");
  }

  // AmrDG<P>::ADER (AmrDG.h:1071-1165) with the solver's Dt: predictor,
  // numerical flux, corrector and reflux of every level, on the device
  // arrays in place.
  void ADER(double Dt) {
    check(ctx, adg_read_patches(ctx), "adg_read_patches");
    check(ctx, adg_set_dt(ctx, Dt), "adg_set_dt");
    check(ctx, adg_ader(ctx), "adg_ader");
    check(ctx, adg_write_patches(ctx), "adg_write_patches");
    check(ctx, adg_synchronize(ctx), "adg_synchronize");
  }

  // The whole evolve-loop body (ADER, average down, ghost fill, t += Dt, new
  // Dt; AmrDG.h:935-1029) on the library's side, the arrays updated in place.
  double step() {
    check(ctx, adg_read_patches(ctx), "adg_read_patches");
    check(ctx, adg_step(ctx), "adg_step");
    check(ctx, adg_write_patches(ctx), "adg_write_patches");
    double dt = 0.0;
    check(ctx, adg_get_dt(ctx, &dt), "adg_get_dt");
    return dt;
  }
};

}  // namespace adg_gb300

#endif  // AMRDG_GB300_H

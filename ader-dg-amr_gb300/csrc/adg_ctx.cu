// Host side of the GB300 ADER-DG element path: context, device buffers,
// element/face tables of the layout, step sequencing (with CUDA-graph replay)
// and the C ABI declared in include/adg.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include "adg.h"
#include "adg_kernelset.hpp"
#include "adg_layout.hpp"
#include "adg_mlp.cuh"
#include "adg_patches.cuh"
#include "plotfile.hpp"
#include <random>
#include <cstdlib>
#include <filesystem>
#include <fstream>
#include <sstream>

namespace adg {

// Device buffer that grows on demand and is freed with the context.
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  // Grows only; a re-growth takes 25% slack so that layouts of slowly
  // changing size (AMR regrids) do not reallocate every time.
  cudaError_t ensure(size_t count) {
    if (count <= n && p) return cudaSuccess;
    const size_t cap = p ? count + count / 4 : count;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(cap, 1) * sizeof(T));
    if (e == cudaSuccess) n = cap;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

// A layout table: a view into the packed table buffer of a context.
template <class T>
struct TableView {
  T* p = nullptr;
  void release() { p = nullptr; }
};

// Pack W (row-major in x out) of one layer as the B operand: row n = output,
// K-major with K = Kp (zero padded), Np rows (zero padded), rounded to TF32.
__global__ void k_seed_pack_tc(const float* W, int in, int out, int Kp, int Np, float* dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Kp * Np) return;
  const int n = i / Kp, k = i % Kp;
  dst[tc::kmajor_off(n, k, Kp)] = (n < out && k < in) ? tc::to_tf32(W[(size_t)k * out + n]) : 0.0f;
}

// FP64 throughput probe: independent DFMA chains.
__global__ void k_fp64_probe(double* out, int iters) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  double a0 = tid * 1e-9, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
  const double b = 0.999, c = 0.001;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
      a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
    }
  }
  out[tid] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

}  // namespace adg

using namespace adg;

struct adg_seed {
  int D = 2, P = 1, Q = 4, n_in = 0, n_out = 0, h = 128;
  const KernelSet* ks = nullptr;
  cudaStream_t stream = nullptr;
  size_t off[8] = {}, sz[8] = {};
  size_t nparam = 0;
  DevBuf<float> params, grads, am, av;
  DevBuf<float> x_mean, x_istd, y_mean, y_std;
  bool normalised = false;
  DevBuf<float> X, T;  // data set
  long long nsamp = 0;
  DevBuf<float> Z1, A1, Z2, A2, Z3, A3, Y, dY, dA, dZ, Xb, Tb;
  DevBuf<float> red;  // partial sums of the split reductions (added in a fixed order)
  long long work_rows = 0;
  DevBuf<int> idx;
  DevBuf<double> loss;
  std::mt19937_64 rng;
  long long adam_t = 0;
  std::string err;
  // weights packed for the tensor-core inference kernel (hidden width 128)
  DevBuf<float> wpack;
  long long w_off[4] = {};
  bool packed = false;
  ~adg_seed() {
    DevBuf<float>* bufs[] = {&params, &grads, &am, &av, &x_mean, &x_istd, &y_mean, &y_std, &X, &T,
                             &Z1, &A1, &Z2, &A2, &Z3, &A3, &Y, &dY, &dA, &dZ, &Xb, &Tb, &wpack, &red};
    for (auto* b : bufs) b->release();
    idx.release();
    loss.release();
    if (stream) cudaStreamDestroy(stream);
  }
};

struct adg_ctx {
  adg_config cfg{};
  const KernelSet* ks = nullptr;
  int E = 0;  // elements per predictor block
  int sweeps = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;
  long long launches = 0;

  Hierarchy hier;       // host layout (levels, boxes, element and face tables)
  amr::GridParams gp;
  bool initialised = false;
  bool tables_dirty = true;
  long long nstep = 0;  // completed steps (regrid schedule)
  long long dof_updates = 0;  // sum over steps of valid elements * Q * Np_s
  long long leaf_dof_updates = 0;  // the same over leaf (uncovered) elements
  size_t n_leaf = 0;               // leaf elements of the current layout
  bool ghosts_stale = false;       // a coarse level's state was set since the last ghost fill
  double regrid_ms = 0.0;     // host wall time spent in regrids
  bool first_step = true;
  int n_regrids = 0;
  double t_last_regrid = 0.0;  // time of the last regrid (dt_regrid cadence)
  // caller's per-box arrays (adg_set_patches), valid for the layout they were
  // registered on
  DevBuf<int> patch_pid;
  DevBuf<long long> patch_off, patch_nstride;
  DevBuf<double*> patch_qptr;
  std::vector<std::vector<amr::IBox>> patch_grids;
  bool patches_set = false;

  // device state
  DevBuf<double> Uw, Rvol, Tr, Fnum, Hw_dbg;
  TableView<int> face_left, face_right, elem_face, elem_cell;
  TableView<int8_t> elem_level;
  DevBuf<double> scal;  // scalar block: [0] Dt, [1] t, Dt/dx per level (kScalDtDx)
  DevBuf<unsigned int> dt_done;  // blocks of the Dt reduction that have finished
  DevBuf<unsigned long long> rate_bits;  // Dt reduction: max of lambda / dx as IEEE bits
  DevBuf<unsigned int> status;
  // AMR tables
  TableView<int> rf_elem, rf_off, rf_face, rf_fine, ad_all, gf_elem, gf_parent, rf_rec_of_elem;
  // the work of a step on an AMR layout (empty: every element, face, valid element)
  TableView<int> pred_list, face_list, corr_list;
  size_t n_pred = 0, n_face_list = 0, n_corr = 0;
  TableView<int8_t> rf_dside, gf_child;
  // all layout tables packed in one device buffer, uploaded by one copy from
  // a pinned staging buffer (tab_ev: that copy has completed)
  DevBuf<uint8_t> tab_dev;
  uint8_t* tab_host = nullptr;
  size_t tab_host_cap = 0;
  cudaEvent_t tab_ev = nullptr;
  std::vector<size_t> ad_off;  // offset (ints) of level lf's records in ad_all
  DevBuf<uint8_t> tags;
  DevBuf<uint8_t> l2_flush;  // written between timed steps to evict the L2
  DevBuf<double> ubar_old;   // [elem][q] cell means at the start of the step (TVB limiter)
  DevBuf<unsigned long long> limited;  // elements the limiter modified
  DevBuf<double> Uw_alt;   // regrid target state (swapped with Uw)
  DevBuf<double> xfer_in, xfer_out;  // host batches of adg_interp_scatter / adg_interp_gather
  DevBuf<int8_t> xfer_child;
  TableView<int> remap_i;     // regrid remap entries: dst | parent | src_old
  TableView<int8_t> remap_c;  // regrid remap child indices
  double rg_phase_ms[6] = {0, 0, 0, 0, 0, 0};  // regrid host time by phase
  // regrid tags in pinned host memory (tag_ev: their copy has landed)
  uint8_t* tags_host = nullptr;
  size_t tags_host_cap = 0;
  cudaEvent_t tag_ev = nullptr;
  // device state of a step that overlaps the host's clustering, restored
  // when the clustering changes the boxes: every element's state, the
  // scalar block, the limiter and fallback counters and the status word
  DevBuf<double> snap_Uw, snap_scal;
  DevBuf<unsigned long long> snap_cnt;
  DevBuf<unsigned int> snap_status;
  int n_rollbacks = 0;
  // learned seed
  adg_seed* seed = nullptr;
  int Es = 0;  // elements per block of the seeded predictor (0: 8 for the FP32 sweeps at D = 2, else E)
  int seed_mode = 0, seed_sweeps = 1;
  double seed_tol = 1e-3;
  DevBuf<float> sx, sy0, sy1, syo;     // features, ping-pong activations, outputs
  DevBuf<double> hseed;
  DevBuf<float> hseed_f;  // FP32 seeds for FP32 sweeps (tensor-core path)
  DevBuf<int> fb_list, fb_count;
  DevBuf<unsigned long long> fb_total;
  long long seed_predicted = 0;
  int seed_path = 1;  // 1: tensor-core inference when the seed supports it, 0: SIMT kernels

  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  int graph_kernels = 0;
  bool graph_stale = false;
  // side stream of the step: the ghost fill runs there beside the average
  // down and the Dt reduction (disjoint elements)
  cudaStream_t side = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  // step readback (adg_set_readback): page-locked host buffers that receive
  // a level's valid state at the end of every step, copied on their own
  // stream once the step's last writer of the level has run
  double* rb_host[kMaxLevels] = {};
  int64_t rb_cap[kMaxLevels] = {};  // capacity in cells
  double* rb_all = nullptr;         // every level packed in level order (ADG_ALL_LEVELS)
  int64_t rb_all_cap = 0;
  cudaStream_t rb = nullptr;
  cudaEvent_t rb_ev[kMaxLevels] = {};
  cudaEvent_t rb_join = nullptr;
  bool rb_pending = false;

  ~adg_ctx() {
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    if (graph) cudaGraphDestroy(graph);
    Uw.release(); Rvol.release(); Tr.release(); Fnum.release(); Hw_dbg.release();
    face_left.release(); face_right.release(); elem_face.release(); elem_cell.release();
    elem_level.release(); scal.release(); dt_done.release(); rate_bits.release(); status.release();
    rf_elem.release(); rf_off.release(); rf_face.release(); rf_fine.release(); ad_all.release();
    pred_list.release(); face_list.release(); corr_list.release();
    gf_elem.release(); gf_parent.release(); rf_dside.release(); gf_child.release(); tags.release();
    sx.release(); sy0.release(); sy1.release(); syo.release(); hseed.release(); hseed_f.release(); fb_list.release(); fb_count.release();
    fb_total.release(); Uw_alt.release(); remap_i.release(); remap_c.release(); l2_flush.release();
    ubar_old.release(); limited.release();
    patch_pid.release(); patch_off.release(); patch_nstride.release(); patch_qptr.release();
    xfer_in.release(); xfer_out.release(); xfer_child.release();
    if (tab_ev) cudaEventSynchronize(tab_ev), cudaEventDestroy(tab_ev);
    if (tag_ev) cudaEventSynchronize(tag_ev), cudaEventDestroy(tag_ev);
    if (tags_host) cudaFreeHost(tags_host);
    snap_Uw.release(); snap_scal.release(); snap_cnt.release(); snap_status.release();
    tab_dev.release();
    if (tab_host) cudaFreeHost(tab_host);
    if (fork_ev) cudaEventDestroy(fork_ev);
    if (join_ev) cudaEventDestroy(join_ev);
    if (side) cudaStreamDestroy(side);
    if (rb) cudaStreamSynchronize(rb), cudaStreamDestroy(rb);
    for (cudaEvent_t& e : rb_ev)
      if (e) cudaEventDestroy(e);
    if (rb_join) cudaEventDestroy(rb_join);
    if (own_stream && stream) cudaStreamDestroy(stream);
  }
};

namespace {

int fail(adg_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_fail(adg_ctx* c, cudaError_t e, const char* where) {
  return fail(c, ADG_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define ADG_CUDA(call, where)                  \
  do {                                         \
    cudaError_t _e = (call);                   \
    if (_e != cudaSuccess) return cuda_fail(ctx, _e, where); \
  } while (0)

// Per-level coefficient of the reference's tagging criteria (1.0 when unset,
// the reference's default, Source/main.cpp:125).
double amr_coeff(const adg_config& c, int l) {
  const double v = c.amr_c[l < 8 ? l : 7];
  return v > 0.0 ? v : 1.0;
}

LevelGeom level_geom(const adg_ctx* ctx) {
  LevelGeom g{};
  for (int l = 0; l < kMaxLevels; ++l)
    for (int d = 0; d < 3; ++d) {
      int n = ctx->cfg.n_cell[d] << l;
      g.dx[l][d] = (d < ctx->cfg.D) ? (ctx->cfg.prob_hi[d] - ctx->cfg.prob_lo[d]) / n : 1.0;
    }
  return g;
}

// Upload element and face tables of the current layout and size the work
// buffers.
// Remap entries of a regrid, uploaded with the tables.
struct RemapTable {
  std::vector<int> dst, par, src;
  std::vector<int8_t> ch;
};

int upload_tables(adg_ctx* ctx, const RemapTable* rm = nullptr) {
  const Hierarchy& H = ctx->hier;
  const KernelSet* ks = ctx->ks;
  const int D = ctx->cfg.D, Q = ks->Q;
  const size_t ne = H.n_elem();
  const size_t nf = H.face_left.size();
  ADG_CUDA(ctx->Rvol.ensure(ne * Q * ks->Np_s), "alloc Rvol");
  ADG_CUDA(ctx->Tr.ensure(ne * 2 * D * (size_t)ks->TR_TILE), "alloc traces");
  ADG_CUDA(ctx->Fnum.ensure(nf * Q * (size_t)ks->NM), "alloc Fnum");
  if (ctx->cfg.limiter_t > 0) ADG_CUDA(ctx->ubar_old.ensure(ne * Q), "alloc limiter means");
  if (ctx->seed) {
    const adg_seed* sd = ctx->seed;
    ADG_CUDA(ctx->sx.ensure(ne * sd->n_in), "alloc seed features");
    ADG_CUDA(ctx->sy0.ensure(ne * sd->h), "alloc seed activations");
    ADG_CUDA(ctx->sy1.ensure(ne * sd->h), "alloc seed activations");
    ADG_CUDA(ctx->syo.ensure(ne * sd->n_out), "alloc seed outputs");
    ADG_CUDA(ctx->hseed.ensure(ne * (size_t)ks->Q * ks->Np_st), "alloc seed H_w");
    ADG_CUDA(ctx->hseed_f.ensure(ne * (size_t)ks->Q * ks->Np_st), "alloc seed H_w");
    ADG_CUDA(ctx->fb_list.ensure(ne), "alloc fallback list");
  }
  std::vector<int> ad;
  ctx->ad_off.assign(H.nlevels() + 1, 0);
  for (int lf = 0; lf < H.nlevels(); ++lf) {
    ctx->ad_off[lf] = ad.size();
    ad.insert(ad.end(), H.ad_rec[lf].begin(), H.ad_rec[lf].end());
  }
  ctx->ad_off[H.nlevels()] = ad.size();
  {
    const size_t nov1 = ((size_t)1 << D) + 1;  // one record per covered coarse element
    ctx->n_leaf = H.n_valid() - ad.size() / nov1;
  }
  // pack every table (256-byte aligned) into the pinned staging buffer
  struct Item {
    const void* src;
    size_t bytes, off;
    std::function<void(uint8_t*)> bind;
  };
  std::vector<Item> items;
  size_t total = 0;
  auto add = [&](auto& view, const auto& vec) {
    using T = std::remove_reference_t<decltype(*view.p)>;
    const size_t bytes = vec.size() * sizeof(vec[0]);
    items.push_back({vec.data(), bytes, total, [&view](uint8_t* at) { view.p = reinterpret_cast<T*>(at); }});
    total += (bytes + 255) & ~size_t(255);
  };
  add(ctx->face_left, H.face_left);
  add(ctx->face_right, H.face_right);
  add(ctx->elem_face, H.elem_face);
  add(ctx->elem_cell, H.elem_cell);
  add(ctx->elem_level, H.elem_level);
  add(ctx->rf_elem, H.rf_elem);
  add(ctx->rf_off, H.rf_off);
  add(ctx->rf_face, H.rf_face);
  add(ctx->rf_dside, H.rf_dside);
  add(ctx->rf_fine, H.rf_fine);
  std::vector<int> roe(H.n_valid(), -1);
  for (size_t r = 0; r < H.rf_elem.size(); ++r) roe[H.rf_elem[r]] = (int)r;
  add(ctx->rf_rec_of_elem, roe);
  add(ctx->ad_all, ad);
  // A covered element's state is replaced by the average down, so the step
  // needs its predictor only for the faces it shares with an uncovered
  // element, and its corrector not at all: the faces of the step are those
  // with an uncovered valid side (and those the coarse-fine corrections
  // read), its predictor elements the sides of those faces and every
  // uncovered element, its corrector elements the uncovered ones (record
  // elements are updated by the record threads).  The state after the step
  // is the one of computing everything.
  std::vector<int> pred_l, face_l, corr_l;
  {
    const size_t nv = H.n_valid(), ne = H.n_elem(), nf = H.face_left.size();
    const size_t nov1 = ((size_t)1 << D) + 1;
    std::vector<uint8_t> covered(ne, 0);
    for (size_t r = 0; r + nov1 <= ad.size(); r += nov1) covered[ad[r]] = 1;
    if (ad.size() >= nov1) {
      std::vector<uint8_t> fneed(nf, 0), eneed(ne, 0);
      auto uncovered = [&](int e) { return (size_t)e < nv && !covered[e]; };
      for (size_t f = 0; f < nf; ++f)
        if (uncovered(H.face_left[f]) || uncovered(H.face_right[f])) fneed[f] = 1;
      for (int f : H.rf_face) fneed[f] = 1;
      for (int f : H.rf_fine) fneed[f] = 1;
      for (size_t f = 0; f < nf; ++f)
        if (fneed[f]) {
          face_l.push_back((int)f);
          eneed[H.face_left[f]] = eneed[H.face_right[f]] = 1;
        }
      for (size_t e = 0; e < nv; ++e)
        if (!covered[e]) {
          eneed[e] = 1;
          if (roe[e] < 0) corr_l.push_back((int)e);
        }
      for (size_t e = 0; e < ne; ++e)
        if (eneed[e]) pred_l.push_back((int)e);
    }
  }
  ctx->n_pred = pred_l.size();
  ctx->n_face_list = face_l.size();
  ctx->n_corr = corr_l.size();
  add(ctx->pred_list, pred_l);
  add(ctx->face_list, face_l);
  add(ctx->corr_list, corr_l);
  // ghost fills grouped by child index: the warps of the fill kernel then
  // mostly run a single coarse-to-fine operator
  std::vector<size_t> gperm(H.gf_elem.size());
  for (size_t i = 0; i < gperm.size(); ++i) gperm[i] = i;
  std::stable_sort(gperm.begin(), gperm.end(), [&](size_t x, size_t y) { return H.gf_child[x] < H.gf_child[y]; });
  std::vector<int> gfe(gperm.size()), gfp(gperm.size());
  std::vector<int8_t> gfc(gperm.size());
  for (size_t i = 0; i < gperm.size(); ++i) {
    gfe[i] = H.gf_elem[gperm[i]];
    gfp[i] = H.gf_parent[gperm[i]];
    gfc[i] = H.gf_child[gperm[i]];
  }
  add(ctx->gf_elem, gfe);
  add(ctx->gf_parent, gfp);
  add(ctx->gf_child, gfc);
  std::vector<int> remap_packed;
  if (rm) {
    const size_t nr = rm->dst.size();
    remap_packed.resize(3 * nr);
    std::copy(rm->dst.begin(), rm->dst.end(), remap_packed.begin());
    std::copy(rm->par.begin(), rm->par.end(), remap_packed.begin() + nr);
    std::copy(rm->src.begin(), rm->src.end(), remap_packed.begin() + 2 * nr);
    add(ctx->remap_i, remap_packed);
    add(ctx->remap_c, rm->ch);
  }
  if (!ctx->tab_ev) ADG_CUDA(cudaEventCreateWithFlags(&ctx->tab_ev, cudaEventDisableTiming), "table event");
  ADG_CUDA(cudaEventSynchronize(ctx->tab_ev), "table staging reuse");  // the previous upload has been read
  if (total > ctx->tab_host_cap) {
    if (ctx->tab_host) cudaFreeHost(ctx->tab_host);
    ctx->tab_host = nullptr;
    ctx->tab_host_cap = 0;
    const size_t cap = total + total / 4;
    ADG_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&ctx->tab_host), cap, cudaHostAllocDefault), "alloc table staging");
    ctx->tab_host_cap = cap;
  }
  ADG_CUDA(ctx->tab_dev.ensure(std::max<size_t>(total, 256)), "alloc tables");
  for (const Item& it : items) {
    if (it.bytes) std::memcpy(ctx->tab_host + it.off, it.src, it.bytes);
    it.bind(ctx->tab_dev.p + it.off);
  }
  ADG_CUDA(cudaMemcpyAsync(ctx->tab_dev.p, ctx->tab_host, total, cudaMemcpyHostToDevice, ctx->stream), "h2d tables");
  ADG_CUDA(cudaEventRecord(ctx->tab_ev, ctx->stream), "table event");
  ctx->tables_dirty = false;
  ctx->graph_stale = true;  // re-captured before the next replay
  return ADG_OK;
}

}  // namespace
int launch_seeded_predictor(adg_ctx* ctx, const PredictorArgs& base, cudaEvent_t* ev);
namespace {

int flush_ghosts(adg_ctx* ctx);

// ADER of every level with the current device Dt (AmrDG.h:1071-1165).
// in_step: the average down follows (a step), so the work lists of the
// layout apply; alone (adg_ader) every valid element is updated.
int launch_ader(adg_ctx* ctx, double* hw_out, cudaEvent_t* ev = nullptr, bool in_step = false) {
  int rc0 = flush_ghosts(ctx);
  if (rc0) return rc0;
  const Hierarchy& H = ctx->hier;
  const KernelSet* ks = ctx->ks;
  const int D = ctx->cfg.D;
  PredictorArgs pa{};
  pa.Uw = ctx->Uw.p;
  pa.n_elem = (int)H.n_elem();
  pa.elem_level = H.nlevels() > 1 ? ctx->elem_level.p : nullptr;
  pa.geom = level_geom(ctx);
  pa.gamma = ctx->cfg.gamma;
  pa.dt = ctx->scal.p;
  pa.sweeps = ctx->sweeps;
  pa.Rvol = ctx->Rvol.p;
  pa.Tr = ctx->Tr.p;
  pa.Hw_out = hw_out;
  pa.ubar_old = ctx->cfg.limiter_t > 0 ? ctx->ubar_old.p : nullptr;
  const bool lists = in_step && ctx->n_pred > 0 && !hw_out;
  if (lists) {
    pa.elem_list = ctx->pred_list.p;
    pa.n_elem = (int)ctx->n_pred;
  }
  if (ev) cudaEventRecord(ev[0], ctx->stream);
  cudaError_t e = cudaSuccess;
  if (ctx->seed_mode && ctx->seed) {
    int rc = launch_seeded_predictor(ctx, pa, ev);
    if (rc) return rc;
  } else {
    e = ks->predictor(pa, ctx->E, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "predictor launch");
    ctx->launches++;
  }
  if (ev) cudaEventRecord(ev[1], ctx->stream);

  FaceArgs fa{};
  fa.Tr = ctx->Tr.p;
  fa.face_left = ctx->face_left.p;
  fa.face_right = ctx->face_right.p;
  for (int d = 0; d <= 3; ++d) fa.face_off[d] = (d <= D) ? H.face_off[d] : H.face_off[D];
  fa.Fnum = ctx->Fnum.p;
  if (lists) {
    fa.face_list = ctx->face_list.p;
    fa.n_list = (long long)ctx->n_face_list;
  }
  const bool split_tiles = ctx->seed_mode == 2 && ctx->seed;  // predictor modes 2 and 3
  e = ks->numflux(fa, lists ? (long long)ctx->n_face_list : (long long)H.face_left.size(), ctx->stream, split_tiles);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "numflux launch");
  ctx->launches++;
  if (ev) cudaEventRecord(ev[2], ctx->stream);

  CorrectorArgs ca{};
  ca.Uw = ctx->Uw.p;
  ca.Rvol = ctx->Rvol.p;
  ca.Fnum = ctx->Fnum.p;
  ca.elem_face = ctx->elem_face.p;
  ca.n_valid = (int)H.n_valid();
  if (lists) {
    ca.elem_list = ctx->corr_list.p;
    ca.n_list = (int)ctx->n_corr;
  }
  ca.elem_level = pa.elem_level;
  ca.geom = pa.geom;
  ca.dt = ctx->scal.p;
  if (!H.rf_elem.empty()) {  // coarse-fine flux correction (AmrDG.h:1159-1162), fused
    ca.nrec = (int)H.rf_elem.size();
    ca.rec_elem = ctx->rf_elem.p;
    ca.rec_of_elem = ctx->rf_rec_of_elem.p;
    ca.rec_off = ctx->rf_off.p;
    ca.ent_face = ctx->rf_face.p;
    ca.ent_dside = ctx->rf_dside.p;
    ca.ent_fine = ctx->rf_fine.p;
  }
  e = ks->corrector(ca, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "corrector launch");
  ctx->launches++;
  if (ev) cudaEventRecord(ev[3], ctx->stream);
  return ADG_OK;
}

// Fine -> coarse average down (finest first) and the coarse -> fine ghost
// fill (AmrDG.h:999-1015).
// Coarse -> fine projection into the ghost elements at coarse-fine faces
// (FillPatchTwoLevels); every ghost's parent is a valid coarse element.
int launch_ghost_fill(adg_ctx* ctx) {
  const Hierarchy& H = ctx->hier;
  if (!H.gf_elem.empty()) {
    ScatterArgs sa{};
    sa.Uw = ctx->Uw.p;
    sa.dst = ctx->gf_elem.p;
    sa.parent = ctx->gf_parent.p;
    sa.child = ctx->gf_child.p;
    sa.n = (int)H.gf_elem.size();
    cudaError_t e = ctx->ks->scatter(sa, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "ghost fill launch");
    ctx->launches++;
  }
  return ADG_OK;
}

// The coarse-fine ghosts after adg_set_state: filled once, before the next
// kernel that reads them (predictor, limiter, tags), however many levels were
// set in between.
int flush_ghosts(adg_ctx* ctx) {
  if (!ctx->ghosts_stale) return ADG_OK;
  ctx->ghosts_stale = false;
  return ctx->hier.nlevels() > 1 ? launch_ghost_fill(ctx) : ADG_OK;
}

// Readback of level lev (adg_set_readback) once the step's last writer of
// the level is queued on the context's stream: the copy waits for that point
// only and runs on the readback stream beside the rest of the step.  A
// registration whose buffer no longer holds the level is dropped, so that it
// never writes past a buffer or into one the caller has released.
int readback_level(adg_ctx* ctx, int lev) {
  if (lev < 0 || lev >= kMaxLevels) return ADG_OK;
  const Hierarchy& H = ctx->hier;
  if (ctx->rb_host[lev] && (lev >= H.nlevels() || (int64_t)H.level_valid_count(lev) > ctx->rb_cap[lev])) {
    ctx->rb_host[lev] = nullptr;
    ctx->rb_cap[lev] = 0;
  }
  if (ctx->rb_all && (int64_t)H.n_valid() > ctx->rb_all_cap) {
    ctx->rb_all = nullptr;
    ctx->rb_all_cap = 0;
  }
  if (lev >= H.nlevels() || (!ctx->rb_host[lev] && !ctx->rb_all)) return ADG_OK;
  const size_t per = (size_t)ctx->ks->Q * ctx->ks->Np_s;
  const size_t off = H.level_valid_offset(lev) * per, bytes = H.level_valid_count(lev) * per * sizeof(double);
  ADG_CUDA(cudaEventRecord(ctx->rb_ev[lev], ctx->stream), "readback fork");
  ADG_CUDA(cudaStreamWaitEvent(ctx->rb, ctx->rb_ev[lev], 0), "readback fork");
  if (ctx->rb_host[lev])
    ADG_CUDA(cudaMemcpyAsync(ctx->rb_host[lev], ctx->Uw.p + off, bytes, cudaMemcpyDeviceToHost, ctx->rb),
             "readback copy");
  if (ctx->rb_all)  // the packed buffer holds the levels at the same offsets as the state
    ADG_CUDA(cudaMemcpyAsync(ctx->rb_all + off, ctx->Uw.p + off, bytes, cudaMemcpyDeviceToHost, ctx->rb),
             "readback copy");
  ctx->rb_pending = true;
  return ADG_OK;
}

// The step's readback copies joined back into the context's stream: later
// work on the stream (the next step, a regrid, adg_set_state) waits for them.
int readback_join(adg_ctx* ctx) {
  if (!ctx->rb_pending) return ADG_OK;
  ctx->rb_pending = false;
  ADG_CUDA(cudaEventRecord(ctx->rb_join, ctx->rb), "readback join");
  ADG_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->rb_join, 0), "readback join");
  return ADG_OK;
}

// Registrations of levels the layout no longer has, or that outgrew their
// buffer, are dropped (they never reactivate into a buffer the caller may
// have released); true if any remains.
bool readback_prune(adg_ctx* ctx) {
  if (ctx->rb_all && (int64_t)ctx->hier.n_valid() > ctx->rb_all_cap) {
    ctx->rb_all = nullptr;
    ctx->rb_all_cap = 0;
  }
  bool any = ctx->rb_all != nullptr;
  for (int l = 0; l < kMaxLevels; ++l) {
    if (!ctx->rb_host[l]) continue;
    if (l >= ctx->hier.nlevels() || (int64_t)ctx->hier.level_valid_count(l) > ctx->rb_cap[l]) {
      ctx->rb_host[l] = nullptr;
      ctx->rb_cap[l] = 0;
    } else {
      any = true;
    }
  }
  return any;
}

// readback: each coarser level is read back once its average down is queued
// (the finest one before the call).
int launch_average_down(adg_ctx* ctx, bool readback = false) {
  const Hierarchy& H = ctx->hier;
  if (H.nlevels() <= 1) return ADG_OK;
  const int NOV1 = (1 << ctx->cfg.D) + 1;
  for (int lf = H.nlevels() - 1; lf >= 1; --lf) {
    const int nrec = (int)(H.ad_rec[lf].size() / NOV1);
    if (nrec) {
      cudaError_t e = ctx->ks->average_down(ctx->Uw.p, ctx->ad_all.p + ctx->ad_off[lf], nrec, ctx->stream);
      if (e != cudaSuccess) return cuda_fail(ctx, e, "average down launch");
      ctx->launches++;
    }
    if (readback) {
      int rc = readback_level(ctx, lf - 1);
      if (rc) return rc;
    }
  }
  return ADG_OK;
}

int launch_amr_sync(adg_ctx* ctx, bool readback = false) {
  int rc = launch_average_down(ctx, readback);
  if (rc) return rc;
  return ctx->hier.nlevels() > 1 ? launch_ghost_fill(ctx) : ADG_OK;
}

// Arguments of the Dt reduction; advance_time adds the old Dt to t first.
DtArgs dt_args(adg_ctx* ctx, int advance_time) {
  const Hierarchy& H = ctx->hier;
  DtArgs da{};
  da.Uw = ctx->Uw.p;
  da.n_valid = (int)H.n_valid();
  da.elem_level = H.nlevels() > 1 ? ctx->elem_level.p : nullptr;
  LevelGeom g = level_geom(ctx);
  for (int l = 0; l < kMaxLevels; ++l) {
    double s = 0.0;
    for (int d = 0; d < ctx->cfg.D; ++d) s += g.dx[l][d];
    da.inv_dx_avg[l] = 1.0 / (s / (double)ctx->cfg.D);
    for (int d = 0; d < 3; ++d) da.inv_geom.dx[l][d] = 1.0 / g.dx[l][d];
  }
  da.gamma = ctx->cfg.gamma;
  da.rate_bits = ctx->rate_bits.p;
  da.status = ctx->status.p;
  da.scal = ctx->scal.p;
  da.done = ctx->dt_done.p;
  da.c_dt = ctx->cfg.c_dt;
  da.advance_time = advance_time;
  da.D = ctx->cfg.D;
  return da;
}

// Dt from the current state; advance_time adds the old Dt to t first.
int launch_dt(adg_ctx* ctx, int advance_time) {
  cudaError_t e = ctx->ks->dt_reduce(dt_args(ctx, advance_time), ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "dt launch");
  ctx->launches += 1;
  return ADG_OK;
}


// TVB limiter of the finest level (AmrDG.h:990-997, 1657-1855).
int launch_limiter(adg_ctx* ctx) {
  int rc0 = flush_ghosts(ctx);
  if (rc0) return rc0;
  const Hierarchy& H = ctx->hier;
  const int F = H.nlevels() - 1;
  const LevelGeom g = level_geom(ctx);
  double h = g.dx[F][0];
  for (int d = 1; d < ctx->cfg.D; ++d) h = std::min(h, g.dx[F][d]);
  LimiterArgs la{};
  la.Uw = ctx->Uw.p;
  la.ubar_old = ctx->ubar_old.p;
  la.elem_face = ctx->elem_face.p;
  la.face_left = ctx->face_left.p;
  la.face_right = ctx->face_right.p;
  la.e0 = (int)H.level_valid_offset(F);
  la.n = (int)H.level_valid_count(F);
  for (int d = 0; d < 3; ++d) la.periodic[d] = ctx->cfg.periodic[d];
  la.gamma = ctx->cfg.gamma;
  la.thr = ctx->cfg.tvb_c[F] * ctx->cfg.tvb_M * std::pow(h, 2.0);
  la.count = ctx->limited.p;
  cudaError_t e = ctx->ks->limit_tvb(la, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "limiter launch");
  ctx->launches++;
  return ADG_OK;
}

int launch_step(adg_ctx* ctx, cudaEvent_t* ev = nullptr) {
  int rc = launch_ader(ctx, nullptr, ev, true);
  if (rc) return rc;
  if (ctx->cfg.limiter_t > 0 && ctx->nstep % ctx->cfg.limiter_t == 0) {
    rc = launch_limiter(ctx);
    if (rc) return rc;
  }
  // the finest level is final here (the average down writes coarser ones)
  const bool rb = !ev && ctx->rb && readback_prune(ctx);
  if (rb) {
    rc = readback_level(ctx, ctx->hier.nlevels() - 1);
    if (rc) return rc;
  }
  const bool fork = !ev && ctx->side && ctx->hier.nlevels() > 1 && !ctx->hier.gf_elem.empty();
  if (!fork) {
    rc = launch_amr_sync(ctx, rb);
    if (rc) return rc;
    if (ev) cudaEventRecord(ev[4], ctx->stream);
    rc = launch_dt(ctx, 1);
    if (ev) cudaEventRecord(ev[5], ctx->stream);
    if (rc == ADG_OK && rb) rc = readback_join(ctx);
    return rc;
  }
  // ghost fill on the side stream: it reads valid coarse parents (never
  // covered, so not touched by the average down) and writes only ghosts,
  // which neither the average down nor the Dt reduction reads
  ADG_CUDA(cudaEventRecord(ctx->fork_ev, ctx->stream), "fork");
  ADG_CUDA(cudaStreamWaitEvent(ctx->side, ctx->fork_ev, 0), "fork");
  cudaStream_t main = ctx->stream;
  ctx->stream = ctx->side;
  rc = launch_ghost_fill(ctx);
  ctx->stream = main;
  if (rc) return rc;
  ADG_CUDA(cudaEventRecord(ctx->join_ev, ctx->side), "join");
  rc = launch_average_down(ctx, rb);
  if (rc == ADG_OK) rc = launch_dt(ctx, 1);
  if (rc == ADG_OK && rb) rc = readback_join(ctx);
  ADG_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->join_ev, 0), "join");
  return rc;
}

// Regrid (AmrDG.h:935-986): refinement indicator on the device, tags to the
// host, new boxes (amr_grids.hpp), new layout, and the level-by-level remap
// of the state (RemakeLevel / MakeNewLevelFromCoarse, AmrDG_Level.tpp:52-132).
double ms_between(std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

int apply_layout(adg_ctx* ctx, const std::vector<std::vector<amr::IBox>>& ng,
                 std::chrono::steady_clock::time_point t2);

// Arguments of the refinement indicator for elements e0 .. e0+n-1.
TagArgs tag_args(const adg_ctx* ctx, int e0, int n) {
  const adg_config& c = ctx->cfg;
  TagArgs ta{};
  ta.Uw = ctx->Uw.p;
  ta.elem_face = ctx->elem_face.p;
  ta.face_left = ctx->face_left.p;
  ta.face_right = ctx->face_right.p;
  ta.e0 = e0;
  ta.n = n;
  ta.kind = c.tag_kind;
  ta.threshold = c.tag_threshold;
  ta.gamma = c.gamma;
  ta.tags = ctx->tags.p;
  ta.elem_cell = ctx->elem_cell.p;
  ta.elem_level = ctx->elem_level.p;
  ta.scal = ctx->scal.p;
  ta.geom = level_geom(ctx);
  for (int d = 0; d < 2; ++d) {
    ta.prob_lo[d] = c.prob_lo[d];
    ta.extent[d] = c.prob_hi[d] - c.prob_lo[d];
  }
  ta.xc = c.xc;
  ta.yc = c.yc;
  ta.u_inf = c.u_inf;
  ta.v_inf = c.v_inf;
  ta.advect = c.tag_advect;
  for (int l = 0; l < kMaxLevels; ++l) {
    const double ac = amr_coeff(c, l);
    ta.r_max[l] = ac * ac;
    double h = ta.geom.dx[l][0];
    for (int d = 1; d < c.D; ++d) h = std::min(h, ta.geom.dx[l][d]);
    ta.tvb_thr[l] = c.tvb_c[l < 8 ? l : 7] * ac * std::pow(h, 2.0);
  }
  return ta;
}

// Regrid, device half: the refinement indicator of every level that may be
// refined, its tags copied into pinned host memory (tag_ev marks the copy).
int regrid_tags(adg_ctx* ctx, size_t* nt_out) {
  Hierarchy& H = ctx->hier;
  const KernelSet* ks = ctx->ks;
  const int F = H.nlevels() - 1;
  const int max_crse = std::min(F, ctx->cfg.max_level - 1);
  const size_t nt = H.level_valid_offset(max_crse) + H.level_valid_count(max_crse);
  ADG_CUDA(ctx->tags.ensure(nt), "alloc tags");
  {  // the valid elements of levels 0 .. max_crse are contiguous: one launch
    TagArgs ta = tag_args(ctx, 0, (int)nt);
    cudaError_t e = ks->tag(ta, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "tag launch");
    ctx->launches++;
  }
  if (!ctx->tag_ev) ADG_CUDA(cudaEventCreateWithFlags(&ctx->tag_ev, cudaEventDisableTiming), "tag event");
  ADG_CUDA(cudaEventSynchronize(ctx->tag_ev), "tag buffer reuse");  // the previous copy has been read
  if (nt > ctx->tags_host_cap) {
    if (ctx->tags_host) cudaFreeHost(ctx->tags_host);
    ctx->tags_host = nullptr;
    ctx->tags_host_cap = 0;
    ADG_CUDA(cudaMallocHost(&ctx->tags_host, nt + nt / 4), "pinned tags");
    ctx->tags_host_cap = nt + nt / 4;
  }
  ADG_CUDA(cudaMemcpyAsync(ctx->tags_host, ctx->tags.p, nt, cudaMemcpyDeviceToHost, ctx->stream), "tags d2h");
  ADG_CUDA(cudaEventRecord(ctx->tag_ev, ctx->stream), "tag event");
  *nt_out = nt;
  return ADG_OK;
}

// Regrid, host half: wait for the tags only, then the new boxes
// (amr_grids.hpp) from the current ones.
int regrid_boxes(adg_ctx* ctx, size_t nt, std::vector<std::vector<amr::IBox>>* ng) {
  Hierarchy& H = ctx->hier;
  auto t0 = std::chrono::steady_clock::now();
  ADG_CUDA(cudaEventSynchronize(ctx->tag_ev), "tags wait");
  auto t1 = std::chrono::steady_clock::now();
  ctx->rg_phase_ms[0] += ms_between(t0, t1);
  const int F = H.nlevels() - 1;
  const int max_crse = std::min(F, ctx->cfg.max_level - 1);
  const uint8_t* ht = ctx->tags_host;
  std::vector<amr::TagField> tf(F + 1);
  for (int l = 0; l <= F; ++l) {
    int n[3];
    H.dims(l, n);
    tf[l].init(n);
    if (l > max_crse) continue;
    for (size_t e = H.level_valid_offset(l); e < H.level_valid_offset(l) + H.level_valid_count(l) && e < nt; ++e)
      if (ht[e]) tf[l].f[tf[l].idx(H.elem_cell[3 * e], H.elem_cell[3 * e + 1], H.elem_cell[3 * e + 2])] = 1;
  }
  *ng = amr::make_new_grids(ctx->gp, H.grids, tf);
  ctx->rg_phase_ms[1] += ms_between(t1, std::chrono::steady_clock::now());
  ctx->n_regrids++;
  return ADG_OK;
}

// Regrid (AmrDG.h:935-986), synchronous: tags, boxes, and a new layout with
// the state remapped when the boxes changed.
int regrid(adg_ctx* ctx) {
  size_t nt = 0;
  int rc = regrid_tags(ctx, &nt);
  if (rc) return rc;
  std::vector<std::vector<amr::IBox>> ng;
  rc = regrid_boxes(ctx, nt, &ng);
  if (rc) return rc;
  if (ng == ctx->hier.grids) return ADG_OK;  // same boxes in the same order: layout and valid data unchanged
  return apply_layout(ctx, ng, std::chrono::steady_clock::now());
}

// What a step changes beyond its scratch, copied on the stream before a step
// that runs while the host clusters, and back if the boxes change.
int snapshot_step_state(adg_ctx* ctx) {
  const size_t nu = ctx->hier.n_elem() * ctx->ks->Q * ctx->ks->Np_s;
  ADG_CUDA(ctx->snap_Uw.ensure(nu), "alloc snapshot");
  ADG_CUDA(ctx->snap_scal.ensure(kScalCount), "alloc snapshot");
  ADG_CUDA(ctx->snap_cnt.ensure(2), "alloc snapshot");
  ADG_CUDA(ctx->snap_status.ensure(1), "alloc snapshot");
  cudaStream_t s = ctx->stream;
  ADG_CUDA(cudaMemcpyAsync(ctx->snap_Uw.p, ctx->Uw.p, nu * sizeof(double), cudaMemcpyDeviceToDevice, s), "snapshot");
  ADG_CUDA(cudaMemcpyAsync(ctx->snap_scal.p, ctx->scal.p, kScalCount * sizeof(double), cudaMemcpyDeviceToDevice, s),
           "snapshot");
  ADG_CUDA(cudaMemcpyAsync(ctx->snap_cnt.p, ctx->limited.p, sizeof(unsigned long long), cudaMemcpyDeviceToDevice, s),
           "snapshot");
  if (ctx->fb_total.p)
    ADG_CUDA(cudaMemcpyAsync(ctx->snap_cnt.p + 1, ctx->fb_total.p, sizeof(unsigned long long),
                             cudaMemcpyDeviceToDevice, s), "snapshot");
  ADG_CUDA(cudaMemcpyAsync(ctx->snap_status.p, ctx->status.p, sizeof(unsigned int), cudaMemcpyDeviceToDevice, s),
           "snapshot");
  return ADG_OK;
}

int restore_step_state(adg_ctx* ctx) {
  const size_t nu = ctx->hier.n_elem() * ctx->ks->Q * ctx->ks->Np_s;
  cudaStream_t s = ctx->stream;
  ADG_CUDA(cudaMemcpyAsync(ctx->Uw.p, ctx->snap_Uw.p, nu * sizeof(double), cudaMemcpyDeviceToDevice, s), "restore");
  ADG_CUDA(cudaMemcpyAsync(ctx->scal.p, ctx->snap_scal.p, kScalCount * sizeof(double), cudaMemcpyDeviceToDevice, s),
           "restore");
  ADG_CUDA(cudaMemcpyAsync(ctx->limited.p, ctx->snap_cnt.p, sizeof(unsigned long long), cudaMemcpyDeviceToDevice, s),
           "restore");
  if (ctx->fb_total.p)
    ADG_CUDA(cudaMemcpyAsync(ctx->fb_total.p, ctx->snap_cnt.p + 1, sizeof(unsigned long long),
                             cudaMemcpyDeviceToDevice, s), "restore");
  ADG_CUDA(cudaMemcpyAsync(ctx->status.p, ctx->snap_status.p, sizeof(unsigned int), cudaMemcpyDeviceToDevice, s),
           "restore");
  return ADG_OK;
}

// Switch to the layout of the given boxes per level and remap the state:
// level 0 is kept, level l takes the old level's data where the cell was
// valid there and the projection of the new level l-1 elsewhere (FillPatch
// semantics of RemakeLevel / MakeNewLevelFromCoarse, AmrDG_Level.tpp:52-132).
int apply_layout(adg_ctx* ctx, const std::vector<std::vector<amr::IBox>>& ng,
                 std::chrono::steady_clock::time_point t2) {
  Hierarchy& H = ctx->hier;
  const KernelSet* ks = ctx->ks;
  Hierarchy NH;
  std::string msg;
  if (!NH.build(ctx->gp, ng, ctx->cfg.reflux_box_quirk, &msg, !ctx->cfg.no_reflux))
    return fail(ctx, ADG_ERR_LAYOUT, "layout: " + msg);
  // remap: level 0 is unchanged; level l from the old level l where a cell
  // was valid there, else from the new level l-1 (levels in order on the stream).
  const int Q = ks->Q, Ns = ks->Np_s;
  ADG_CUDA(ctx->Uw_alt.ensure(NH.n_elem() * Q * Ns), "alloc regrid state");
  double* nU = ctx->Uw_alt.p;
  ADG_CUDA(cudaMemcpyAsync(nU, ctx->Uw.p, H.level_valid_count(0) * Q * Ns * sizeof(double), cudaMemcpyDeviceToDevice,
                           ctx->stream), "regrid copy level 0");
  RemapTable rm;
  std::vector<size_t> lo(NH.nlevels() + 1, 0);
  for (int l = 1; l < NH.nlevels(); ++l) {
    lo[l] = rm.dst.size();
    for (size_t e = 0; e < NH.n_elem(); ++e) {
      if (NH.elem_level[e] != l) continue;
      const int* c = &NH.elem_cell[3 * e];
      int pc[3] = {0, 0, 0}, child = 0;
      for (int a = 0; a < NH.D; ++a) {
        pc[a] = c[a] >> 1;
        child += (c[a] & 1) << (NH.D - 1 - a);
      }
      int old = -1;
      if (l < H.nlevels()) {
        int oe = H.elem_at(l, c);
        if (H.is_valid_elem(oe)) old = oe;
      }
      rm.dst.push_back((int)e);
      rm.par.push_back(NH.cellmap[l - 1][NH.cidx(l - 1, pc)]);
      rm.src.push_back(old);
      rm.ch.push_back((int8_t)child);
    }
  }
  lo[NH.nlevels()] = rm.dst.size();
  const size_t nr = rm.dst.size();
  auto t3 = std::chrono::steady_clock::now();
  ctx->rg_phase_ms[2] += ms_between(t2, t3);
  ctx->hier = std::move(NH);
  int rc = upload_tables(ctx, &rm);
  if (rc) return rc;
  auto t4 = std::chrono::steady_clock::now();
  ctx->rg_phase_ms[3] += ms_between(t3, t4);
  for (int l = 1; l < ctx->hier.nlevels(); ++l) {
    const size_t o = lo[l], n = lo[l + 1] - lo[l];
    if (!n) continue;
    ScatterArgs sa{};
    sa.Uw = nU;
    sa.Uw_old = ctx->Uw.p;
    sa.dst = ctx->remap_i.p + o;
    sa.parent = ctx->remap_i.p + nr + o;
    sa.src_old = ctx->remap_i.p + 2 * nr + o;
    sa.child = ctx->remap_c.p + o;
    sa.n = (int)n;
    cudaError_t e = ks->scatter(sa, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "regrid remap launch");
    ctx->launches++;
  }
  std::swap(ctx->Uw, ctx->Uw_alt);
  ctx->rg_phase_ms[4] += ms_between(t4, std::chrono::steady_clock::now());
  return ADG_OK;
}

// AmrDG.h:936-941: at the first step, every dtn_regrid steps, or once
// dt_regrid of time has passed since the last regrid (the time is read from
// the device only while dt_regrid is on).
bool regrid_due(adg_ctx* ctx) {
  if (ctx->cfg.max_level <= 0) return false;
  if (ctx->first_step || (ctx->cfg.dtn_regrid > 0 && ctx->nstep % ctx->cfg.dtn_regrid == 0)) return true;
  if (ctx->cfg.dt_regrid > 0.0) {
    double t = 0.0;
    if (cudaMemcpyAsync(&t, ctx->scal.p + 1, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
      return false;  // the step's own launches report the error
    return t - ctx->t_last_regrid >= ctx->cfg.dt_regrid - 1e-12;
  }
  return false;
}

// Time of the step about to run, recorded as the last regrid's (dt_regrid).
void note_regrid_time(adg_ctx* ctx) {
  if (ctx->cfg.dt_regrid <= 0.0) return;
  double t = 0.0;
  if (cudaMemcpyAsync(&t, ctx->scal.p + 1, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream) == cudaSuccess &&
      cudaStreamSynchronize(ctx->stream) == cudaSuccess)
    ctx->t_last_regrid = t;
}

// One evolve-loop body: regrid when due (host), then the step kernels.
int host_step(adg_ctx* ctx, bool use_graph, cudaEvent_t* ev = nullptr);

int check_ready(adg_ctx* ctx) {
  if (!ctx) return ADG_ERR_ARG;
  if (!ctx->initialised) return fail(ctx, ADG_ERR_STATE, "adg_init has not been called");
  if (ctx->tables_dirty) return upload_tables(ctx);
  return ADG_OK;
}

// Capture the step; an existing executable graph of the same topology is
// updated in place (cheaper than instantiating after every regrid).
int capture_graph(adg_ctx* ctx) {
  long long before = ctx->launches;
  ADG_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
  int rc = launch_step(ctx);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(ctx, e, "end capture");
  bool updated = false;
  if (ctx->graph_exec) {
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(ctx->graph_exec, g, &info) == cudaSuccess) {
      updated = true;
    } else {
      cudaGetLastError();  // clear the update error
      cudaGraphExecDestroy(ctx->graph_exec);
      ctx->graph_exec = nullptr;
    }
  }
  if (ctx->graph) cudaGraphDestroy(ctx->graph);
  ctx->graph = g;
  if (!updated) ADG_CUDA(cudaGraphInstantiate(&ctx->graph_exec, g, 0), "graph instantiate");
  ctx->graph_kernels = (int)(ctx->launches - before);
  ctx->launches = before;
  ctx->graph_stale = false;
  return ADG_OK;
}

// The step's kernels on the current layout: the captured graph (updated or
// re-captured after a layout change) or direct launches.
int launch_one_step(adg_ctx* ctx, bool use_graph, cudaEvent_t* ev) {
  int rc0 = flush_ghosts(ctx);  // outside the graph
  if (rc0) return rc0;
  if (use_graph && !ev) {
    if (!ctx->graph_exec || ctx->graph_stale) {
      auto t0 = std::chrono::steady_clock::now();
      int rc = capture_graph(ctx);
      if (rc) return rc;
      ctx->rg_phase_ms[5] += ms_between(t0, std::chrono::steady_clock::now());
    }
    ADG_CUDA(cudaGraphLaunch(ctx->graph_exec, ctx->stream), "graph launch");
    ctx->launches += ctx->graph_kernels;
    return ADG_OK;
  }
  return launch_step(ctx, ev);
}

void count_step(adg_ctx* ctx) {
  ctx->dof_updates += (long long)ctx->hier.n_valid() * ctx->ks->Q * ctx->ks->Np_s;
  if (ctx->seed_mode && ctx->seed) ctx->seed_predicted += (long long)ctx->hier.n_elem();
  ctx->leaf_dof_updates += (long long)ctx->n_leaf * ctx->ks->Q * ctx->ks->Np_s;
}

// One evolve-loop body.  A due regrid normally overlaps the step: the tags
// go to the host, the step runs on the current boxes while the host
// clusters, and only if the clustering changes the boxes is the step's state
// restored, the new layout applied and the step run again; either way the
// result is the one of regridding first.  The first step and the per-stage
// timing path regrid synchronously.
int host_step(adg_ctx* ctx, bool use_graph, cudaEvent_t* ev) {
  if (ctx->cfg.limiter_t > 1) use_graph = false;  // the step's kernels then differ from step to step
  int rc = flush_ghosts(ctx);  // the regrid's tags read them
  if (rc) return rc;
  const bool due = regrid_due(ctx);
  if (due) note_regrid_time(ctx);
  if (due && !ctx->first_step && !ev) {
    auto t0 = std::chrono::steady_clock::now();
    size_t nt = 0;
    rc = regrid_tags(ctx, &nt);
    if (rc == ADG_OK) rc = snapshot_step_state(ctx);
    if (rc == ADG_OK) rc = launch_one_step(ctx, use_graph, nullptr);
    std::vector<std::vector<amr::IBox>> ng;
    if (rc == ADG_OK) rc = regrid_boxes(ctx, nt, &ng);
    if (rc == ADG_OK && ng != ctx->hier.grids) {
      ctx->n_rollbacks++;
      rc = restore_step_state(ctx);
      if (rc == ADG_OK) rc = apply_layout(ctx, ng, std::chrono::steady_clock::now());
      if (rc == ADG_OK) rc = launch_one_step(ctx, use_graph, nullptr);
    }
    if (rc) return rc;
    ctx->regrid_ms += ms_between(t0, std::chrono::steady_clock::now());
    count_step(ctx);
    ctx->nstep++;
    return ADG_OK;
  }
  if (due) {
    auto t0 = std::chrono::steady_clock::now();
    rc = regrid(ctx);
    if (rc) return rc;
    ctx->regrid_ms += ms_between(t0, std::chrono::steady_clock::now());
  }
  count_step(ctx);
  ctx->first_step = false;
  rc = launch_one_step(ctx, use_graph, ev);
  if (rc) return rc;
  ctx->nstep++;
  return ADG_OK;
}

}  // namespace

namespace {
// ---- quadrature for the Lp norms (host) -----------------------------------
// Legendre P_n and its derivative by the three-term recurrence.
void legendre_pd(int n, double x, double* p, double* dp) {
  double p0 = 1.0, p1 = x, d0 = 0.0, d1 = 1.0;
  if (n == 0) {
    *p = 1.0;
    *dp = 0.0;
    return;
  }
  for (int k = 2; k <= n; ++k) {
    const double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
    const double d2 = d0 + (2.0 * k - 1.0) * p1;
    p0 = p1;
    p1 = p2;
    d0 = d1;
    d1 = d2;
  }
  *p = p1;
  *dp = d1;
}

// n-point Gauss-Legendre nodes (Newton from cos(pi (i - 1/4) / (n + 1/2)),
// in the order x_1, -x_1, x_2, ...) and weights 2 / ((1 - x^2) P_n'(x)^2).
void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
  x.clear();
  for (int i = 1; i <= n / 2; ++i) {
    double xi = std::cos(3.14159265358979323846 * (i - 0.25) / (n + 0.5));
    for (int it = 0; it < 100; ++it) {
      double p, dp;
      legendre_pd(n, xi, &p, &dp);
      const double dx = p / dp;
      xi -= dx;
      if (std::fabs(dx) < 1e-16) break;
    }
    x.push_back(xi);
    x.push_back(-xi);
  }
  if (n % 2) x.push_back(0.0);
  w.resize(x.size());
  for (size_t k = 0; k < x.size(); ++k) {
    double p, dp;
    legendre_pd(n, x[k], &p, &dp);
    w[k] = 2.0 / ((1.0 - x[k] * x[k]) * dp * dp);
  }
}

// Spatial modes in the reference's order: total degree <= P, first index
// slowest (MultiIndex, AmrDG.h:62-122).
void multi_index(int D, int left, int depth, std::array<int, 3>& cur, std::vector<std::array<int, 3>>& out) {
  if (depth == D) {
    out.push_back(cur);
    return;
  }
  for (int v = 0; v <= left; ++v) {
    cur[depth] = v;
    multi_index(D, left - v, depth + 1, cur, out);
  }
  cur[depth] = 0;
}

}  // namespace

extern "C" {

int adg_ctx_create(const adg_config* cfg, adg_ctx** out) {
  if (!cfg || !out) return ADG_ERR_ARG;
  *out = nullptr;
  const KernelSet* ks = kernel_set(cfg->D, cfg->P);
  if (!ks) return ADG_ERR_ARG;
  for (int d = 0; d < cfg->D; ++d)
    if (cfg->n_cell[d] <= 0 || !(cfg->prob_hi[d] > cfg->prob_lo[d])) return ADG_ERR_ARG;
  if (cfg->max_level < 0 || cfg->max_level >= kMaxLevels) return ADG_ERR_ARG;
  if (cfg->limiter_t < 0 || !(cfg->tvb_M >= 0.0)) return ADG_ERR_ARG;
  if (!(cfg->gamma > 1.0) || !(cfg->c_dt > 0.0)) return ADG_ERR_ARG;
  adg_ctx* ctx = new adg_ctx();
  ctx->cfg = *cfg;
  ctx->ks = ks;
  ctx->sweeps = cfg->picard_sweeps > 0 ? cfg->picard_sweeps : cfg->P;
  if (ctx->sweeps < 1) ctx->sweeps = 1;
  std::vector<int> ch = ks->elems_per_block_choices();
  const int E0 = cfg->D == 2 ? 16 : 8;  // default where it is built, else the one choice of the configuration
  ctx->E = (cfg->elems_per_block > 0 && std::find(ch.begin(), ch.end(), cfg->elems_per_block) != ch.end())
               ? cfg->elems_per_block
               : (std::find(ch.begin(), ch.end(), E0) != ch.end() ? E0 : ch.front());
  cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete ctx;
    return ADG_ERR_CUDA;
  }
  ctx->own_stream = true;
  if (cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->fork_ev, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->join_ev, cudaEventDisableTiming) != cudaSuccess) {
    delete ctx;
    return ADG_ERR_CUDA;
  }
  if (ctx->scal.ensure(kScalCount) != cudaSuccess || ctx->dt_done.ensure(1) != cudaSuccess ||
      ctx->limited.ensure(1) != cudaSuccess ||
      ctx->rate_bits.ensure(1) != cudaSuccess || ctx->status.ensure(1) != cudaSuccess) {
    delete ctx;
    return ADG_ERR_CUDA;
  }
  double z[kScalCount] = {};
  unsigned int zero = 0;
  if (cudaMemcpy(ctx->scal.p, z, sizeof(z), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(ctx->dt_done.p, 0, sizeof(unsigned int)) != cudaSuccess ||
      cudaMemset(ctx->limited.p, 0, sizeof(unsigned long long)) != cudaSuccess ||
      cudaMemset(ctx->rate_bits.p, 0, sizeof(unsigned long long)) != cudaSuccess ||
      cudaMemcpy(ctx->status.p, &zero, sizeof(zero), cudaMemcpyHostToDevice) != cudaSuccess) {
    delete ctx;
    return ADG_ERR_CUDA;
  }
  *out = ctx;
  return ADG_OK;
}

int adg_ctx_destroy(adg_ctx* ctx) {
  if (!ctx) return ADG_ERR_ARG;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  delete ctx;
  return ADG_OK;
}

const char* adg_last_error(const adg_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int adg_set_stream(adg_ctx* ctx, void* stream) {
  if (!ctx) return ADG_ERR_ARG;
  if (ctx->own_stream && ctx->stream) {
    cudaStreamSynchronize(ctx->stream);
    cudaStreamDestroy(ctx->stream);
  }
  ctx->stream = (cudaStream_t)stream;
  ctx->own_stream = false;
  if (ctx->graph_exec) {
    cudaGraphExecDestroy(ctx->graph_exec);
    ctx->graph_exec = nullptr;
  }
  return ADG_OK;
}

static void apply_tuned_choices(adg_ctx* ctx);

int adg_init(adg_ctx* ctx) {
  if (!ctx) return ADG_ERR_ARG;
  for (int l = 0; l < kMaxLevels; ++l) ctx->rb_host[l] = nullptr, ctx->rb_cap[l] = 0;  // a new layout
  ctx->rb_all = nullptr;
  ctx->rb_all_cap = 0;
  const adg_config& c = ctx->cfg;
  const KernelSet* ks = ctx->ks;
  std::string msg;
  ctx->gp = Hierarchy::params(c);
  if (c.validation_mode < 0 || c.validation_mode > 2) return fail(ctx, ADG_ERR_ARG, "validation_mode must be 0, 1 or 2");
  if (c.tag_kind < 0 || c.tag_kind > 3) return fail(ctx, ADG_ERR_ARG, "unknown tag_kind");
  // Single level: one box over the domain.  AMR: AmrCore::InitFromScratch
  // (Source/Core/Solver.h:567-571) tags the levels while their state is still
  // zero.  The geometric vortex criterion tags its disc, so the hierarchy is
  // clustered from it level by level; the data criteria see a zero state
  // (the reference's TVB test reads NaN eigenvectors there and flags every
  // cell), so every finer level starts as a full-domain grid and the first
  // step regrids from the refinement indicator.
  const bool geometric = c.max_level > 0 && c.tag_kind == ADG_TAG_VORTEX;
  std::vector<std::vector<amr::IBox>> g;
  if (c.max_level <= 0) {
    if (!ctx->hier.build_single_level(c, &msg)) return fail(ctx, ADG_ERR_LAYOUT, msg);
  } else {
    const int top = geometric ? 0 : c.max_level;
    for (int l = 0; l <= top; ++l) {
      amr::IBox dom;
      for (int d = 0; d < 3; ++d) {
        dom.lo[d] = 0;
        dom.hi[d] = d < c.D ? (c.n_cell[d] << l) - 1 : 0;
      }
      g.push_back(amr::chop_max_size({dom}, c.D, ctx->gp.max_grid));
    }
    if (!ctx->hier.build(ctx->gp, g, c.reflux_box_quirk, &msg, !c.no_reflux))
      return fail(ctx, ADG_ERR_LAYOUT, msg);
  }
  ADG_CUDA(ctx->Uw.ensure(ctx->hier.n_elem() * ks->Q * ks->Np_s), "alloc Uw");
  {
    const double t0 = 0.0;
    ADG_CUDA(cudaMemcpyAsync(ctx->scal.p + 1, &t0, sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "reset t");
  }
  int rc = upload_tables(ctx);
  if (rc) return rc;
  if (geometric) {
    // one new level per pass (AmrMesh::MakeNewGrids(time)), then passes over
    // all levels until the boxes stop changing (its iterate_on_new_grids)
    ADG_CUDA(cudaMemsetAsync(ctx->Uw.p, 0, ctx->hier.n_elem() * ks->Q * ks->Np_s * sizeof(double), ctx->stream),
             "zero state");
    for (int pass = 0; pass < c.max_level + 4; ++pass) {
      size_t nt = 0;
      rc = regrid_tags(ctx, &nt);
      if (rc) return rc;
      std::vector<std::vector<amr::IBox>> ng;
      rc = regrid_boxes(ctx, nt, &ng);
      if (rc) return rc;
      if (ng == ctx->hier.grids) break;
      rc = apply_layout(ctx, ng, std::chrono::steady_clock::now());
      if (rc) return rc;
    }
    ctx->n_regrids = 0;
    for (double& v : ctx->rg_phase_ms) v = 0.0;
  }
  const Hierarchy& H = ctx->hier;
  // the analytic IC on level 0, on every level in validation mode (with the
  // coarse-fine ghosts too in mode 2) (AmrDG.h:782-836, Solver.h:711-734)
  ICArgs ia{};
  ia.Uw = ctx->Uw.p;
  ia.elem_cell = ctx->elem_cell.p;
  ia.elem_level = c.validation_mode ? ctx->elem_level.p : nullptr;  // level 0 elements come first
  ia.n_elem = (int)(c.validation_mode == 2 ? H.n_elem()
                    : c.validation_mode == 1 ? H.n_valid()
                                             : H.level_valid_count(0));
  ia.geom = level_geom(ctx);
  for (int d = 0; d < 3; ++d) {
    ia.prob_lo[d] = c.prob_lo[d];
    ia.n_cell0[d] = c.n_cell[d];
  }
  ia.gamma = c.gamma;
  ia.icp.ic = c.ic;
  ia.icp.u_inf = c.u_inf;
  ia.icp.v_inf = c.v_inf;
  ia.icp.beta = c.beta;
  ia.icp.xc = c.xc;
  ia.icp.yc = c.yc;
  ia.icp.seed = c.seed;
  ia.icp.noise_amp = c.noise_amp;
  cudaError_t e = ks->init_ic(ia, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "init_ic launch");
  ctx->launches++;
  // finer levels otherwise: projection from the coarser level
  // (AMR_interpolate_initial_condition)
  DevBuf<int> d_dst, d_par;
  DevBuf<int8_t> d_ch;
  for (int l = 1; !c.validation_mode && l < H.nlevels(); ++l) {
    std::vector<int> dst, par;
    std::vector<int8_t> ch;
    for (size_t x = H.level_valid_offset(l); x < H.level_valid_offset(l) + H.level_valid_count(l); ++x) {
      const int* cc = &H.elem_cell[3 * x];
      int pc[3] = {0, 0, 0}, child = 0;
      for (int a = 0; a < H.D; ++a) {
        pc[a] = cc[a] >> 1;
        child += (cc[a] & 1) << (H.D - 1 - a);
      }
      dst.push_back((int)x);
      par.push_back(H.cellmap[l - 1][H.cidx(l - 1, pc)]);
      ch.push_back((int8_t)child);
    }
    ADG_CUDA(d_dst.ensure(dst.size()), "alloc");
    ADG_CUDA(d_par.ensure(dst.size()), "alloc");
    ADG_CUDA(d_ch.ensure(dst.size()), "alloc");
    ADG_CUDA(cudaMemcpyAsync(d_dst.p, dst.data(), dst.size() * 4, cudaMemcpyHostToDevice, ctx->stream), "h2d");
    ADG_CUDA(cudaMemcpyAsync(d_par.p, par.data(), dst.size() * 4, cudaMemcpyHostToDevice, ctx->stream), "h2d");
    ADG_CUDA(cudaMemcpyAsync(d_ch.p, ch.data(), dst.size(), cudaMemcpyHostToDevice, ctx->stream), "h2d");
    ScatterArgs sa{};
    sa.Uw = ctx->Uw.p;
    sa.dst = d_dst.p;
    sa.parent = d_par.p;
    sa.child = d_ch.p;
    sa.n = (int)dst.size();
    e = ks->scatter(sa, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "initial projection launch");
    ctx->launches++;
    ADG_CUDA(cudaStreamSynchronize(ctx->stream), "init projection sync");
  }
  d_dst.release(); d_par.release(); d_ch.release();
  ctx->initialised = true;
  ctx->nstep = 0;
  ctx->first_step = true;
  ctx->t_last_regrid = 0.0;
  ctx->ghosts_stale = false;
  // AMR_sync_initial_condition (AmrDG_Level.tpp:94-118): average down, then
  // the ghost cells of every level (validation mode 2: the finer levels'
  // coarse-fine ghosts keep their analytic projection until the first step)
  rc = c.validation_mode == 2 ? launch_average_down(ctx) : launch_amr_sync(ctx);
  if (rc) return rc;
  rc = launch_dt(ctx, 0);
  if (rc) return rc;
  ADG_CUDA(cudaStreamSynchronize(ctx->stream), "init sync");
  apply_tuned_choices(ctx);
  return ADG_OK;
}

int adg_num_levels(const adg_ctx* ctx, int* nlev) {
  if (!ctx || !nlev) return ADG_ERR_ARG;
  *nlev = ctx->hier.nlevels();
  return ADG_OK;
}

int adg_level_cells(const adg_ctx* ctx, int lev, int64_t* ncells) {
  if (!ctx || !ncells || lev < 0 || lev >= ctx->hier.nlevels()) return ADG_ERR_ARG;
  *ncells = (int64_t)ctx->hier.level_valid_count(lev);
  return ADG_OK;
}

int adg_get_state(adg_ctx* ctx, int lev, double* dst, int mem) {
  int rc = check_ready(ctx);
  if (rc) return rc;
  const bool all = lev == ADG_ALL_LEVELS;
  if (!dst || (!all && (lev < 0 || lev >= ctx->hier.nlevels())) || mem < 0 || mem > 2)
    return fail(ctx, ADG_ERR_ARG, "bad level, pointer or memory kind");
  const size_t per = (size_t)ctx->ks->Q * ctx->ks->Np_s;
  const size_t off = all ? 0 : ctx->hier.level_valid_offset(lev) * per;  // the levels are stored in order
  const size_t cnt = (all ? ctx->hier.n_valid() : ctx->hier.level_valid_count(lev)) * per;
  ADG_CUDA(cudaMemcpyAsync(dst, ctx->Uw.p + off, cnt * sizeof(double),
                           mem == ADG_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, ctx->stream),
           "get_state copy");
  if (mem != ADG_MEM_HOST_ASYNC) ADG_CUDA(cudaStreamSynchronize(ctx->stream), "get_state sync");
  return ADG_OK;
}

int adg_set_state(adg_ctx* ctx, int lev, const double* src, int mem) {
  int rc = check_ready(ctx);
  if (rc) return rc;
  const bool all = lev == ADG_ALL_LEVELS;
  if (!src || (!all && (lev < 0 || lev >= ctx->hier.nlevels())) || mem < 0 || mem > 2)
    return fail(ctx, ADG_ERR_ARG, "bad level, pointer or memory kind");
  const size_t per = (size_t)ctx->ks->Q * ctx->ks->Np_s;
  const size_t off = all ? 0 : ctx->hier.level_valid_offset(lev) * per;
  const size_t cnt = (all ? ctx->hier.n_valid() : ctx->hier.level_valid_count(lev)) * per;
  ADG_CUDA(cudaMemcpyAsync(ctx->Uw.p + off, src, cnt * sizeof(double),
                           mem == ADG_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, ctx->stream),
           "set_state copy");
  if (all ? ctx->hier.nlevels() > 1 : lev + 1 < ctx->hier.nlevels())
    ctx->ghosts_stale = true;  // the finer level's ghosts project from this level
  if (mem != ADG_MEM_HOST_ASYNC) ADG_CUDA(cudaStreamSynchronize(ctx->stream), "set_state sync");
  return ADG_OK;
}

int adg_set_readback(adg_ctx* ctx, int lev, double* host, int64_t capacity_cells) {
  int rc = check_ready(ctx);
  if (rc) return rc;
  const bool all = lev == ADG_ALL_LEVELS;
  if (!all && (lev < 0 || lev >= ctx->hier.nlevels() || lev >= kMaxLevels)) return fail(ctx, ADG_ERR_ARG, "bad level");
  if (!host) {
    if (all) {
      ctx->rb_all = nullptr;
      ctx->rb_all_cap = 0;
    } else {
      ctx->rb_host[lev] = nullptr;
      ctx->rb_cap[lev] = 0;
    }
    ctx->graph_stale = true;
    return ADG_OK;
  }
  if (capacity_cells < (int64_t)(all ? ctx->hier.n_valid() : ctx->hier.level_valid_count(lev)))
    return fail(ctx, ADG_ERR_ARG, "readback buffer smaller than the level's valid cells");
  cudaPointerAttributes pa{};
  if (cudaPointerGetAttributes(&pa, host) != cudaSuccess || pa.type != cudaMemoryTypeHost) {
    cudaGetLastError();
    return fail(ctx, ADG_ERR_ARG, "readback buffer must be page-locked host memory");
  }
  if (!ctx->rb) {
    ADG_CUDA(cudaStreamCreateWithFlags(&ctx->rb, cudaStreamNonBlocking), "readback stream");
    for (cudaEvent_t& e : ctx->rb_ev) ADG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "readback event");
    ADG_CUDA(cudaEventCreateWithFlags(&ctx->rb_join, cudaEventDisableTiming), "readback event");
  }
  if (all) {
    ctx->rb_all = host;
    ctx->rb_all_cap = capacity_cells;
  } else {
    ctx->rb_host[lev] = host;
    ctx->rb_cap[lev] = capacity_cells;
  }
  ctx->graph_stale = true;  // the step's graph now carries the copy
  return ADG_OK;
}

int adg_readback_active(adg_ctx* ctx, int lev, int* active) {
  if (!ctx || !active || (lev < 0 && lev != ADG_ALL_LEVELS)) return ADG_ERR_ARG;
  readback_prune(ctx);
  *active = lev == ADG_ALL_LEVELS ? ctx->rb_all != nullptr : (lev < kMaxLevels && ctx->rb_host[lev] != nullptr);
  return ADG_OK;
}

int adg_synchronize(adg_ctx* ctx) {
  if (!ctx) return ADG_ERR_ARG;
  ADG_CUDA(cudaStreamSynchronize(ctx->stream), "synchronize");
  return ADG_OK;
}

int adg_get_dt(adg_ctx* ctx, double* dt) {
  if (!ctx || !dt) return ADG_ERR_ARG;
  ADG_CUDA(cudaMemcpyAsync(dt, ctx->scal.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "get_dt");
  ADG_CUDA(cudaStreamSynchronize(ctx->stream), "get_dt sync");
  return ADG_OK;
}

int adg_set_dt(adg_ctx* ctx, double dt) {
  if (!ctx || !(dt > 0.0)) return ADG_ERR_ARG;
  const LevelGeom g = level_geom(ctx);
  double blk[3 * kMaxLevels];
  for (int l = 0; l < kMaxLevels; ++l)
    for (int d = 0; d < 3; ++d) blk[3 * l + d] = d < ctx->cfg.D ? dt / g.dx[l][d] : 0.0;
  ADG_CUDA(cudaMemcpyAsync(ctx->scal.p, &dt, sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "set_dt");
  ADG_CUDA(cudaMemcpyAsync(ctx->scal.p + kScalDtDx, blk, sizeof(blk), cudaMemcpyHostToDevice, ctx->stream), "set_dt");
  ADG_CUDA(cudaStreamSynchronize(ctx->stream), "set_dt sync");
  return ADG_OK;
}

int adg_compute_dt(adg_ctx* ctx, double* dt) {
  int rc = check_ready(ctx);
  if (rc) return rc;
  rc = launch_dt(ctx, 0);
  if (rc) return rc;
  if (dt) return adg_get_dt(ctx, dt);
  return ADG_OK;
}

int adg_get_time(adg_ctx* ctx, double* t) {
  if (!ctx || !t) return ADG_ERR_ARG;
  ADG_CUDA(cudaMemcpyAsync(t, ctx->scal.p + 1, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "get_time");
  ADG_CUDA(cudaStreamSynchronize(ctx->stream), "get_time sync");
  return ADG_OK;
}

int adg_ader(adg_ctx* ctx) {
  int rc = check_ready(ctx);
  if (rc) return rc;
  rc = launch_ader(ctx, nullptr);
  if (rc) return rc;
  if (ctx->seed_mode && ctx->seed) ctx->seed_predicted += (long long)ctx->hier.n_elem();
  ADG_CUDA(cudaStreamSynchronize(ctx->stream), "ader sync");
  return ADG_OK;
}

int adg_step(adg_ctx* ctx) {
  int rc = check_ready(ctx);
  if (rc) return rc;
  rc = host_step(ctx, false);
  if (rc) return rc;
  ADG_CUDA(cudaStreamSynchronize(ctx->stream), "step sync");
  return ADG_OK;
}

int adg_advance(adg_ctx* ctx, int nsteps, int use_graph) {
  int rc = check_ready(ctx);
  if (rc) return rc;
  if (nsteps < 0) return fail(ctx, ADG_ERR_ARG, "negative step count");
  for (int s = 0; s < nsteps; ++s) {
    rc = host_step(ctx, use_graph != 0);
    if (rc) return rc;
  }
  return ADG_OK;
}

int adg_lp_norm(adg_ctx* ctx, int p, int q, double* out) {
  int rc = check_ready(ctx);
  if (rc) return rc;
  const Hierarchy& H = ctx->hier;
  const KernelSet* ks = ctx->ks;
  const int D = ctx->cfg.D, P = ctx->cfg.P;
  if (!out || (p != 1 && p != 2) || q < 0 || q >= ks->Q) return fail(ctx, ADG_ERR_ARG, "bad norm arguments");
  // points: the method's N = P + 1 GL nodes for p = 1, 2N for p = 2 (AmrDG.h:1399-1578)
  std::vector<double> x1, w1;
  gauss_legendre(p == 1 ? P + 1 : 2 * (P + 1), x1, w1);
  const int N1 = (int)x1.size();
  int M = 1;
  for (int d = 0; d < D; ++d) M *= N1;
  std::vector<std::array<int, 3>> mi;
  std::array<int, 3> cur{0, 0, 0};
  multi_index(D, P, 0, cur, mi);
  std::vector<double> tab((size_t)mi.size() * M + M + 3 * (size_t)M);
  double* phi = tab.data();
  double* wq = phi + mi.size() * M;
  double* qp = wq + M;
  for (int m = 0; m < M; ++m) {
    int rem = m, id[3] = {0, 0, 0};
    for (int d = D - 1; d >= 0; --d) {
      id[d] = rem % N1;
      rem /= N1;
    }
    wq[m] = 1.0;
    for (int d = 0; d < 3; ++d) {
      qp[3 * m + d] = d < D ? x1[id[d]] : 0.0;
      if (d < D) wq[m] *= w1[id[d]];
    }
    for (size_t n = 0; n < mi.size(); ++n) {
      double v = 1.0;
      for (int d = 0; d < D; ++d) {
        double pv, dp;
        legendre_pd(mi[n][d], x1[id[d]], &pv, &dp);
        v *= pv;
      }
      phi[n * M + m] = v;
    }
  }
  // covered flags (average-down records' coarse elements) and the leaf volume
  const size_t nv = H.n_valid();
  std::vector<int8_t> cov(nv, 0);
  const size_t nov1 = ((size_t)1 << D) + 1;
  for (int lf = 1; lf < H.nlevels(); ++lf)
    for (size_t r = 0; r + nov1 <= H.ad_rec[lf].size(); r += nov1) cov[H.ad_rec[lf][r]] = 1;
  const LevelGeom g = level_geom(ctx);
  double V_amr = 0.0;
  for (int l = 0; l < H.nlevels(); ++l) {
    double vol = 1.0;
    for (int d = 0; d < D; ++d) vol *= g.dx[l][d];
    size_t nleaf = 0;
    for (size_t e = H.level_valid_offset(l); e < H.level_valid_offset(l) + H.level_valid_count(l); ++e)
      nleaf += cov[e] ? 0 : 1;
    V_amr += vol * (double)nleaf;
  }
  DevBuf<double> dtab, dcell;
  DevBuf<int8_t> dcov;
  ADG_CUDA(dtab.ensure(tab.size()), "alloc norm tables");
  ADG_CUDA(dcell.ensure(nv), "alloc norm cells");
  ADG_CUDA(dcov.ensure(nv), "alloc norm cells");
  ADG_CUDA(cudaMemcpyAsync(dtab.p, tab.data(), tab.size() * 8, cudaMemcpyHostToDevice, ctx->stream), "h2d");
  ADG_CUDA(cudaMemcpyAsync(dcov.p, cov.data(), nv, cudaMemcpyHostToDevice, ctx->stream), "h2d");
  LpArgs a{};
  a.Uw = ctx->Uw.p;
  a.elem_cell = ctx->elem_cell.p;
  a.elem_level = H.nlevels() > 1 ? ctx->elem_level.p : nullptr;
  a.covered = dcov.p;
  a.n_valid = (int)nv;
  a.q = q;
  a.p = p;
  a.M = M;
  a.phi = dtab.p;
  a.wq = dtab.p + mi.size() * M;
  a.qp = a.wq + M;
  a.geom = g;
  for (int d = 0; d < 3; ++d) a.prob_lo[d] = ctx->cfg.prob_lo[d];
  a.gamma = ctx->cfg.gamma;
  const adg_config& c = ctx->cfg;
  a.icp.ic = c.ic;
  a.icp.u_inf = c.u_inf;
  a.icp.v_inf = c.v_inf;
  a.icp.beta = c.beta;
  a.icp.xc = c.xc;
  a.icp.yc = c.yc;
  a.icp.seed = c.seed;
  a.icp.noise_amp = c.noise_amp;
  a.cell_out = dcell.p;
  cudaError_t e = ks->lp_norm(a, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "norm launch");
  ctx->launches++;
  std::vector<double> cells(nv);
  ADG_CUDA(cudaMemcpyAsync(cells.data(), dcell.p, nv * 8, cudaMemcpyDeviceToHost, ctx->stream), "d2h");
  ADG_CUDA(cudaStreamSynchronize(ctx->stream), "norm sync");
  double total = 0.0;
  for (size_t k = 0; k < nv; ++k) total += cells[k];
  *out = std::pow(total / V_amr, 1.0 / (double)p);
  return ADG_OK;
}

int adg_limited_count(adg_ctx* ctx, int64_t* n) {
  if (!ctx || !n) return ADG_ERR_ARG;
  unsigned long long v = 0;
  ADG_CUDA(cudaMemcpyAsync(&v, ctx->limited.p, sizeof(v), cudaMemcpyDeviceToHost, ctx->stream), "limited count");
  ADG_CUDA(cudaStreamSynchronize(ctx->stream), "limited count");
  *n = (int64_t)v;
  return ADG_OK;
}

int adg_leaf_dof_updates(const adg_ctx* ctx, int64_t* total) {
  if (!ctx || !total) return ADG_ERR_ARG;
  *total = ctx->leaf_dof_updates;
  return ADG_OK;
}

int adg_regrid_profile(const adg_ctx* ctx, double* ms, int n) {
  if (!ctx || !ms || n < 0) return ADG_ERR_ARG;
  for (int i = 0; i < n && i < 6; ++i) ms[i] = ctx->rg_phase_ms[i];
  return ADG_OK;
}

int adg_dof_updates(const adg_ctx* ctx, int64_t* total, double* regrid_ms) {
  if (!ctx || !total) return ADG_ERR_ARG;
  *total = ctx->dof_updates;
  if (regrid_ms) *regrid_ms = ctx->regrid_ms;
  return ADG_OK;
}

int adg_regrid_count(const adg_ctx* ctx, int* n) {
  if (!ctx || !n) return ADG_ERR_ARG;
  *n = ctx->n_regrids;
  return ADG_OK;
}

int adg_get_boxes(const adg_ctx* ctx, int lev, int* out, int cap, int* nbox) {
  if (!ctx || !nbox || lev < 0 || lev >= ctx->hier.nlevels()) return ADG_ERR_ARG;
  const auto& g = ctx->hier.grids[lev];
  *nbox = (int)g.size();
  for (int b = 0; b < (int)g.size() && b < cap; ++b)
    for (int d = 0; d < 3; ++d) {
      out[6 * b + d] = g[b].lo[d];
      out[6 * b + 3 + d] = g[b].hi[d];
    }
  return ADG_OK;
}

int adg_set_layout(adg_ctx* ctx, int nlev, const int* nbox, const int* boxes) {
  int rc = check_ready(ctx);
  if (rc) return rc;
  if (nlev < 1 || nlev > ctx->cfg.max_level + 1 || !nbox || !boxes)
    return fail(ctx, ADG_ERR_ARG, "bad layout arguments");
  std::vector<std::vector<amr::IBox>> ng(nlev);
  size_t o = 0;
  for (int l = 0; l < nlev; ++l) {
    if (nbox[l] < 0) return fail(ctx, ADG_ERR_ARG, "bad layout arguments");
    for (int b = 0; b < nbox[l]; ++b, o += 6) {
      amr::IBox bx;
      for (int d = 0; d < 3; ++d) {
        bx.lo[d] = d < ctx->cfg.D ? boxes[o + d] : 0;
        bx.hi[d] = d < ctx->cfg.D ? boxes[o + 3 + d] : 0;
      }
      ng[l].push_back(bx);
    }
  }
  if (ng != ctx->hier.grids) {
    rc = apply_layout(ctx, ng, std::chrono::steady_clock::now());
    if (rc) return rc;
  }
  ctx->first_step = false;  // the caller owns the layout from now on
  ADG_CUDA(cudaStreamSynchronize(ctx->stream), "layout");
  return ADG_OK;
}

int adg_level_cell_coords(const adg_ctx* ctx, int lev, int* ijk) {
  if (!ctx || !ijk || lev < 0 || lev >= ctx->hier.nlevels()) return ADG_ERR_ARG;
  const Hierarchy& H = ctx->hier;
  const size_t e0 = H.level_valid_offset(lev), n = H.level_valid_count(lev);
  std::copy(H.elem_cell.begin() + 3 * e0, H.elem_cell.begin() + 3 * (e0 + n), ijk);
  return ADG_OK;
}

int adg_tags(adg_ctx* ctx, int lev, uint8_t* out) {
  int rc = check_ready(ctx);
  if (rc) return rc;
  const Hierarchy& H = ctx->hier;
  if (!out || lev < 0 || lev >= H.nlevels()) return fail(ctx, ADG_ERR_ARG, "bad level");
  rc = flush_ghosts(ctx);
  if (rc) return rc;
  ADG_CUDA(ctx->tags.ensure(H.n_valid()), "alloc tags");
  TagArgs ta = tag_args(ctx, (int)H.level_valid_offset(lev), (int)H.level_valid_count(lev));
  cudaError_t e = ctx->ks->tag(ta, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "tag launch");
  ctx->launches++;
  ADG_CUDA(cudaMemcpyAsync(out, ctx->tags.p, ta.n, cudaMemcpyDeviceToHost, ctx->stream), "tags d2h");
  ADG_CUDA(cudaStreamSynchronize(ctx->stream), "tags sync");
  return ADG_OK;
}

// L2ProjInterp::amr_scatter on a caller batch (AmrDG_Interpolater.tpp:344-364).
int adg_interp_scatter(adg_ctx* ctx, const double* coarse, const int8_t* child, int64_t n, double* fine, int mem) {
  if (!ctx) return ADG_ERR_ARG;
  if (n < 0 || (n > 0 && (!coarse || !child || !fine)) || (mem != ADG_MEM_HOST && mem != ADG_MEM_DEVICE))
    return fail(ctx, ADG_ERR_ARG, "bad interpolation arguments");
  if (n == 0) return ADG_OK;
  const KernelSet* ks = ctx->ks;
  const size_t cnt = (size_t)n * ks->Q * ks->Np_s;
  cudaError_t e;
  if (mem == ADG_MEM_HOST) {
    for (int64_t i = 0; i < n; ++i)
      if (child[i] < 0 || child[i] >= (1 << ctx->cfg.D)) return fail(ctx, ADG_ERR_ARG, "child index out of range");
    ADG_CUDA(ctx->xfer_in.ensure(cnt), "alloc");
    ADG_CUDA(ctx->xfer_out.ensure(cnt), "alloc");
    ADG_CUDA(ctx->xfer_child.ensure((size_t)n), "alloc");
    ADG_CUDA(cudaMemcpyAsync(ctx->xfer_in.p, coarse, cnt * 8, cudaMemcpyHostToDevice, ctx->stream), "h2d");
    ADG_CUDA(cudaMemcpyAsync(ctx->xfer_child.p, child, (size_t)n, cudaMemcpyHostToDevice, ctx->stream), "h2d");
    e = ks->interp_scatter(ctx->xfer_in.p, ctx->xfer_child.p, n, ctx->xfer_out.p, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "scatter launch");
    ADG_CUDA(cudaMemcpyAsync(fine, ctx->xfer_out.p, cnt * 8, cudaMemcpyDeviceToHost, ctx->stream), "d2h");
  } else {
    e = ks->interp_scatter(coarse, child, n, fine, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "scatter launch");
  }
  ctx->launches++;
  ADG_CUDA(cudaStreamSynchronize(ctx->stream), "scatter sync");
  return ADG_OK;
}

// L2ProjInterp::amr_gather on a caller batch (AmrDG_Interpolater.tpp:366-398).
int adg_interp_gather(adg_ctx* ctx, const double* fine, int64_t n, double* coarse, int mem) {
  if (!ctx) return ADG_ERR_ARG;
  if (n < 0 || (n > 0 && (!coarse || !fine)) || (mem != ADG_MEM_HOST && mem != ADG_MEM_DEVICE))
    return fail(ctx, ADG_ERR_ARG, "bad interpolation arguments");
  if (n == 0) return ADG_OK;
  const KernelSet* ks = ctx->ks;
  const size_t cnt = (size_t)n * ks->Q * ks->Np_s, cnt_f = cnt << ctx->cfg.D;
  cudaError_t e;
  if (mem == ADG_MEM_HOST) {
    ADG_CUDA(ctx->xfer_in.ensure(cnt_f), "alloc");
    ADG_CUDA(ctx->xfer_out.ensure(cnt), "alloc");
    ADG_CUDA(cudaMemcpyAsync(ctx->xfer_in.p, fine, cnt_f * 8, cudaMemcpyHostToDevice, ctx->stream), "h2d");
    e = ks->interp_gather(ctx->xfer_in.p, n, ctx->xfer_out.p, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "gather launch");
    ADG_CUDA(cudaMemcpyAsync(coarse, ctx->xfer_out.p, cnt * 8, cudaMemcpyDeviceToHost, ctx->stream), "d2h");
  } else {
    e = ks->interp_gather(fine, n, coarse, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "gather launch");
  }
  ctx->launches++;
  ADG_CUDA(cudaStreamSynchronize(ctx->stream), "gather sync");
  return ADG_OK;
}

int adg_average_down(adg_ctx* ctx) {
  int rc = check_ready(ctx);
  if (rc) return rc;
  rc = launch_average_down(ctx);
  if (rc) return rc;
  ADG_CUDA(cudaStreamSynchronize(ctx->stream), "average down sync");
  return ADG_OK;
}

int adg_set_patches(adg_ctx* ctx, const adg_patch* patches, int n) {
  int rc = check_ready(ctx);
  if (rc) return rc;
  const Hierarchy& H = ctx->hier;
  const int D = ctx->cfg.D, Q = ctx->ks->Q;
  if (n < 0 || (n > 0 && !patches)) return fail(ctx, ADG_ERR_ARG, "bad patch list");
  const size_t nv = H.n_valid();
  std::vector<int> pid(nv, -1);
  std::vector<long long> off(nv, 0), nstr((size_t)n, 0);
  std::vector<double*> qptr((size_t)n * Q, nullptr);
  for (int p = 0; p < n; ++p) {
    const adg_patch& pt = patches[p];
    if (pt.level < 0 || pt.level >= H.nlevels() || pt.nghost < 0)
      return fail(ctx, ADG_ERR_ARG, "patch " + std::to_string(p) + ": bad level or ghost width");
    int dims[3];
    H.dims(pt.level, dims);
    long long ext[3] = {1, 1, 1};
    for (int d = 0; d < 3; ++d) {
      const int lo = d < D ? pt.lo[d] : 0, hi = d < D ? pt.hi[d] : 0;
      if (lo > hi || lo < 0 || hi >= dims[d])
        return fail(ctx, ADG_ERR_ARG, "patch " + std::to_string(p) + ": box outside the level");
      if (d < D) ext[d] = hi - lo + 1 + 2LL * pt.nghost;
    }
    if (pt.jstride < ext[0] || (D > 2 && pt.kstride < pt.jstride * ext[1]) ||
        pt.nstride < (D > 2 ? pt.kstride * ext[2] : pt.jstride * ext[1]))
      return fail(ctx, ADG_ERR_ARG, "patch " + std::to_string(p) + ": strides smaller than the grown box");
    for (int q = 0; q < Q; ++q) {
      if (!pt.U_w[q]) return fail(ctx, ADG_ERR_ARG, "patch " + std::to_string(p) + ": null array");
      qptr[(size_t)p * Q + q] = pt.U_w[q];
    }
    nstr[p] = pt.nstride;
    const int lo2 = D > 2 ? pt.lo[2] : 0, hi2 = D > 2 ? pt.hi[2] : 0;
    for (int k = lo2; k <= hi2; ++k)
      for (int j = pt.lo[1]; j <= pt.hi[1]; ++j)
        for (int i = pt.lo[0]; i <= pt.hi[0]; ++i) {
          const int c[3] = {i, j, k};
          const int e = H.elem_at(pt.level, c);
          if (e < 0 || (size_t)e >= nv)
            return fail(ctx, ADG_ERR_LAYOUT, "patch " + std::to_string(p) + " covers a cell outside the layout");
          if (pid[e] >= 0) return fail(ctx, ADG_ERR_LAYOUT, "patches overlap");
          pid[e] = p;
          off[e] = (long long)(i - pt.lo[0] + pt.nghost) + (long long)(j - pt.lo[1] + pt.nghost) * pt.jstride +
                   (D > 2 ? (long long)(k - lo2 + pt.nghost) * pt.kstride : 0LL);
        }
  }
  for (size_t e = 0; e < nv; ++e)
    if (pid[e] < 0) return fail(ctx, ADG_ERR_LAYOUT, "patches leave a valid cell of the layout uncovered");
  ADG_CUDA(ctx->patch_pid.ensure(nv), "alloc patch table");
  ADG_CUDA(ctx->patch_off.ensure(nv), "alloc patch table");
  ADG_CUDA(ctx->patch_nstride.ensure(std::max(n, 1)), "alloc patch table");
  ADG_CUDA(ctx->patch_qptr.ensure((size_t)std::max(n, 1) * Q), "alloc patch table");
  ADG_CUDA(cudaMemcpyAsync(ctx->patch_pid.p, pid.data(), nv * sizeof(int), cudaMemcpyHostToDevice, ctx->stream), "h2d");
  ADG_CUDA(cudaMemcpyAsync(ctx->patch_off.p, off.data(), nv * sizeof(long long), cudaMemcpyHostToDevice, ctx->stream),
           "h2d");
  if (n > 0) {
    ADG_CUDA(cudaMemcpyAsync(ctx->patch_nstride.p, nstr.data(), n * sizeof(long long), cudaMemcpyHostToDevice,
                             ctx->stream), "h2d");
    ADG_CUDA(cudaMemcpyAsync(ctx->patch_qptr.p, qptr.data(), qptr.size() * sizeof(double*), cudaMemcpyHostToDevice,
                             ctx->stream), "h2d");
  }
  ADG_CUDA(cudaStreamSynchronize(ctx->stream), "patch table upload");
  ctx->patch_grids = H.grids;
  ctx->patches_set = true;
  return ADG_OK;
}

static int patch_copy(adg_ctx* ctx, int dir) {
  int rc = check_ready(ctx);
  if (rc) return rc;
  if (!ctx->patches_set || ctx->patch_grids != ctx->hier.grids)
    return fail(ctx, ADG_ERR_LAYOUT, "no patches registered for the current layout (adg_set_patches)");
  PatchTab t{};
  t.pid = ctx->patch_pid.p;
  t.off = ctx->patch_off.p;
  t.qptr = ctx->patch_qptr.p;
  t.nstride = ctx->patch_nstride.p;
  t.n = (int)ctx->hier.n_valid();
  t.Q = ctx->ks->Q;
  t.NS = ctx->ks->Np_s;
  cudaError_t e = launch_patch_copy(dir, t, ctx->Uw.p, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "patch copy launch");
  ctx->launches++;
  if (dir == 0 && ctx->hier.nlevels() > 1) ctx->ghosts_stale = true;
  return ADG_OK;
}

int adg_read_patches(adg_ctx* ctx) { return patch_copy(ctx, 0); }
int adg_write_patches(adg_ctx* ctx) { return patch_copy(ctx, 1); }

int adg_limit(adg_ctx* ctx, int64_t* n_limited) {
  int rc = check_ready(ctx);
  if (rc) return rc;
  if (ctx->cfg.limiter_t <= 0 || !ctx->ubar_old.p)
    return fail(ctx, ADG_ERR_STATE, "adg_limit needs a context created with the TVB limiter (limiter_t > 0)");
  unsigned long long before = 0, after = 0;
  ADG_CUDA(cudaMemcpyAsync(&before, ctx->limited.p, sizeof(before), cudaMemcpyDeviceToHost, ctx->stream), "count");
  rc = launch_limiter(ctx);
  if (rc) return rc;
  ADG_CUDA(cudaMemcpyAsync(&after, ctx->limited.p, sizeof(after), cudaMemcpyDeviceToHost, ctx->stream), "count");
  ADG_CUDA(cudaStreamSynchronize(ctx->stream), "limiter sync");
  if (n_limited) *n_limited = (int64_t)(after - before);
  return ADG_OK;
}

int adg_fill_ghosts(adg_ctx* ctx) {
  int rc = check_ready(ctx);
  if (rc) return rc;
  ctx->ghosts_stale = false;
  if (ctx->hier.nlevels() > 1) {
    rc = launch_ghost_fill(ctx);
    if (rc) return rc;
  }
  ADG_CUDA(cudaStreamSynchronize(ctx->stream), "ghost fill sync");
  return ADG_OK;
}

int adg_get_step(const adg_ctx* ctx, int64_t* n) {
  if (!ctx || !n) return ADG_ERR_ARG;
  *n = (int64_t)ctx->nstep;
  return ADG_OK;
}

// Solver::PlotFile (Source/Core/Solver.h:922-968): per q one plotfile whose
// components are the Np_s modes of U_w(l, q) on the valid boxes of each level.
int adg_write_plotfile(adg_ctx* ctx, const char* data_dir, int tstep, int level, const char* const* var_names) {
  int rc = check_ready(ctx);
  if (rc) return rc;
  const Hierarchy& H = ctx->hier;
  const int D = ctx->cfg.D, Q = ctx->ks->Q, Ns = ctx->ks->Np_s;
  if (!data_dir || tstep < 0 || level >= H.nlevels()) return fail(ctx, ADG_ERR_ARG, "bad plotfile arguments");
  if (var_names)
    for (int q = 0; q < Q; ++q)
      if (!var_names[q] || !var_names[q][0] || std::strpbrk(var_names[q], " \t\r\n"))
        return fail(ctx, ADG_ERR_ARG, "variable names must be non-empty words");
  const int l0 = level < 0 ? 0 : level, l1 = level < 0 ? H.nlevels() - 1 : level;
  std::vector<double> hs(H.n_valid() * Q * Ns);
  double t = 0.0;
  ADG_CUDA(cudaMemcpyAsync(hs.data(), ctx->Uw.p, hs.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream),
           "plotfile state d2h");
  ADG_CUDA(cudaMemcpyAsync(&t, ctx->scal.p + 1, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "plotfile time");
  ADG_CUDA(cudaStreamSynchronize(ctx->stream), "plotfile sync");
  // Compressible_Euler::VarNames (Compressible_Euler.h:15-24); that list is
  // ordered for 2D, so 3D names momentum_z before energy_density.
  static const char* const names2[] = {"mass_density", "momentum_x", "momentum_y", "energy_density"};
  static const char* const names3[] = {"mass_density", "momentum_x", "momentum_y", "momentum_z", "energy_density"};
  const LevelGeom g = level_geom(ctx);
  for (int q = 0; q < Q; ++q) {
    plt::Meta m;
    m.D = D;
    m.ncomp = Ns;
    m.time = t;
    for (int d = 0; d < D; ++d) {
      m.prob_lo[d] = ctx->cfg.prob_lo[d];
      m.prob_hi[d] = ctx->cfg.prob_hi[d];
    }
    const std::string base = var_names ? var_names[q] : (D == 3 ? names3[q] : names2[q]);
    for (int k = 0; k < Ns; ++k) m.names.push_back(base + "_" + std::to_string(k));
    std::vector<plt::LevelData> data;
    for (int l = l0; l <= l1; ++l) {
      plt::LevelMeta L;
      L.boxes = H.grids[l];
      for (int d = 0; d < 3; ++d) L.domain.hi[d] = d < D ? (ctx->cfg.n_cell[d] << l) - 1 : 0;
      for (int d = 0; d < D; ++d) L.dx[d] = g.dx[l][d];
      L.step = tstep;
      m.levels.push_back(L);
      if (l < l1) m.ref_ratio.push_back(2);
      plt::LevelData ld(L.boxes.size());
      for (size_t b = 0; b < L.boxes.size(); ++b) {
        const amr::IBox& bx = L.boxes[b];
        const size_t nc = (size_t)bx.volume(D);
        std::vector<double>& v = ld[b];
        v.resize(nc * Ns);
        size_t o = 0;
        for (int k = bx.lo[2]; k <= bx.hi[2]; ++k)
          for (int j = bx.lo[1]; j <= bx.hi[1]; ++j)
            for (int i = bx.lo[0]; i <= bx.hi[0]; ++i, ++o) {
              const int c[3] = {i, j, k};
              const size_t e = (size_t)H.cellmap[l][H.cidx(l, c)];
              const double* u = &hs[(e * Q + q) * Ns];
              for (int k2 = 0; k2 < Ns; ++k2) v[k2 * nc + o] = u[k2];
            }
      }
      data.push_back(std::move(ld));
    }
    std::string err;
    const std::string dir =
        std::string(data_dir) + "/tstep_" + std::to_string(tstep) + "_q_" + std::to_string(q) + "_plt";
    if (!plt::write(dir, m, data, &err)) return fail(ctx, ADG_ERR_IO, err);
  }
  return ADG_OK;
}

// Solver::ReadPlotFile (Source/Core/Solver.h:599-652) and the FillPatch of
// every restored level that follows it (Solver.h:572-593).
int adg_read_plotfile(adg_ctx* ctx, const char* data_dir, int tstep, double* time) {
  int rc = check_ready(ctx);
  if (rc) return rc;
  if (!data_dir || tstep < 0) return fail(ctx, ADG_ERR_ARG, "bad plotfile arguments");
  const int D = ctx->cfg.D, Q = ctx->ks->Q, Ns = ctx->ks->Np_s;
  std::vector<plt::Meta> meta(Q);
  std::vector<std::vector<plt::LevelData>> data(Q);
  std::string err;
  for (int q = 0; q < Q; ++q) {
    const std::string dir =
        std::string(data_dir) + "/tstep_" + std::to_string(tstep) + "_q_" + std::to_string(q) + "_plt";
    if (!plt::read(dir, ctx->cfg.max_level + 1, &meta[q], &data[q], &err)) return fail(ctx, ADG_ERR_IO, err);
    if (meta[q].D != D) return fail(ctx, ADG_ERR_IO, dir + ": dimension differs from the configuration");
    if (meta[q].ncomp != Ns) return fail(ctx, ADG_ERR_IO, dir + ": component count is not Np_s");
  }
  const plt::Meta& m0 = meta[0];
  const int nlev = std::min((int)m0.levels.size(), ctx->cfg.max_level + 1);  // ReadPlotFile caps at max_level
  std::vector<std::vector<amr::IBox>> ng(nlev);
  for (int l = 0; l < nlev; ++l) {
    const amr::IBox& dom = m0.levels[l].domain;
    for (int d = 0; d < D; ++d)
      if (dom.lo[d] != 0 || dom.hi[d] != (ctx->cfg.n_cell[d] << l) - 1)
        return fail(ctx, ADG_ERR_IO, "plotfile level " + std::to_string(l) + " domain differs from the configuration");
    if (l > 0 && m0.ref_ratio[l - 1] != 2) return fail(ctx, ADG_ERR_IO, "plotfile refinement ratio is not 2");
    ng[l] = m0.levels[l].boxes;
    for (int q = 1; q < Q; ++q)
      if ((int)meta[q].levels.size() <= l || !(meta[q].levels[l].boxes == ng[l]))
        return fail(ctx, ADG_ERR_IO, "plotfiles of the variables have different boxes");
  }
  for (int q = 1; q < Q; ++q)
    if (meta[q].time != m0.time) return fail(ctx, ADG_ERR_IO, "plotfiles of the variables have different times");
  if (ng != ctx->hier.grids) {
    rc = apply_layout(ctx, ng, std::chrono::steady_clock::now());  // checks nesting before any change
    if (rc) return rc;
  }
  const Hierarchy& H = ctx->hier;
  std::vector<double> hs(H.n_valid() * Q * Ns);
  for (int q = 0; q < Q; ++q)
    for (int l = 0; l < nlev; ++l)
      for (size_t b = 0; b < ng[l].size(); ++b) {
        const amr::IBox& bx = ng[l][b];
        const size_t nc = (size_t)bx.volume(D);
        const std::vector<double>& v = data[q][l][b];
        size_t o = 0;
        for (int k = bx.lo[2]; k <= bx.hi[2]; ++k)
          for (int j = bx.lo[1]; j <= bx.hi[1]; ++j)
            for (int i = bx.lo[0]; i <= bx.hi[0]; ++i, ++o) {
              const int c[3] = {i, j, k};
              const size_t e = (size_t)H.cellmap[l][H.cidx(l, c)];
              double* u = &hs[(e * Q + q) * Ns];
              for (int k2 = 0; k2 < Ns; ++k2) u[k2] = v[k2 * nc + o];
            }
      }
  const double t = m0.time;
  ADG_CUDA(cudaMemcpyAsync(ctx->Uw.p, hs.data(), hs.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream),
           "plotfile state h2d");
  ADG_CUDA(cudaMemcpyAsync(ctx->scal.p + 1, &t, sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "plotfile time");
  if (H.nlevels() > 1) {
    rc = launch_ghost_fill(ctx);
    if (rc) return rc;
  }
  rc = launch_dt(ctx, 0);
  if (rc) return rc;
  ADG_CUDA(cudaStreamSynchronize(ctx->stream), "plotfile restart sync");
  ctx->nstep = m0.levels[0].step;
  ctx->first_step = true;  // the evolve loop regrids before its first step after a restart
  if (time) *time = t;
  return ADG_OK;
}

int adg_plotfile_info(const char* plotfile_dir, int* dim, int* ncomp, int* finest_level, double* time, int* step,
                      char* err, int err_cap) {
  if (!plotfile_dir) return ADG_ERR_ARG;
  plt::Meta m;
  std::string e;
  if (!plt::read(plotfile_dir, 0, &m, nullptr, &e)) {
    if (err && err_cap > 0) {
      const size_t n = std::min(e.size(), (size_t)err_cap - 1);
      std::memcpy(err, e.data(), n);
      err[n] = '\0';
    }
    return ADG_ERR_IO;
  }
  if (dim) *dim = m.D;
  if (ncomp) *ncomp = m.ncomp;
  if (finest_level) *finest_level = (int)m.levels.size() - 1;
  if (time) *time = m.time;
  if (step) *step = m.levels[0].step;
  if (err && err_cap > 0) err[0] = '\0';
  return ADG_OK;
}

int adg_set_device(int device) {
  return cudaSetDevice(device) == cudaSuccess ? ADG_OK : ADG_ERR_CUDA;
}

int adg_advance_timed(adg_ctx* ctx, int nsteps, int use_graph, double* ms) {
  int rc = check_ready(ctx);
  if (rc) return rc;
  if (!ms) return ADG_ERR_ARG;
  if (use_graph && (!ctx->graph_exec || ctx->graph_stale) && !regrid_due(ctx)) {  // capture outside the timed region
    rc = capture_graph(ctx);
    if (rc) return rc;
  }
  cudaEvent_t e0, e1;
  ADG_CUDA(cudaEventCreate(&e0), "event");
  ADG_CUDA(cudaEventCreate(&e1), "event");
  cudaEventRecord(e0, ctx->stream);
  rc = adg_advance(ctx, nsteps, use_graph);
  cudaEventRecord(e1, ctx->stream);
  cudaError_t e = cudaEventSynchronize(e1);
  float f = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&f, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(ctx, e, "timed advance");
  *ms = f;
  return ADG_OK;
}

int adg_advance_timed_flushed(adg_ctx* ctx, int nsteps, int use_graph, int64_t flush_bytes, double* ms) {
  int rc = check_ready(ctx);
  if (rc) return rc;
  if (!ms || nsteps < 0 || flush_bytes < 0) return ADG_ERR_ARG;
  if (use_graph && (!ctx->graph_exec || ctx->graph_stale) && !regrid_due(ctx)) {
    rc = capture_graph(ctx);
    if (rc) return rc;
  }
  if (flush_bytes > 0) ADG_CUDA(ctx->l2_flush.ensure((size_t)flush_bytes), "alloc L2 flush buffer");
  std::vector<cudaEvent_t> ev(2 * (size_t)nsteps);
  for (auto& x : ev) ADG_CUDA(cudaEventCreate(&x), "event");
  for (int k = 0; k < nsteps && rc == ADG_OK; ++k) {
    if (flush_bytes > 0) {
      cudaError_t e = cudaMemsetAsync(ctx->l2_flush.p, k & 0xff, (size_t)flush_bytes, ctx->stream);
      if (e != cudaSuccess) rc = cuda_fail(ctx, e, "L2 flush");
    }
    cudaEventRecord(ev[2 * k], ctx->stream);
    if (rc == ADG_OK) rc = host_step(ctx, use_graph != 0);
    cudaEventRecord(ev[2 * k + 1], ctx->stream);
  }
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  double total = 0.0;
  for (int k = 0; k < nsteps && e == cudaSuccess && rc == ADG_OK; ++k) {
    float f = 0.f;
    e = cudaEventElapsedTime(&f, ev[2 * k], ev[2 * k + 1]);
    total += f;
  }
  for (auto& x : ev) cudaEventDestroy(x);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(ctx, e, "timed advance");
  *ms = total;
  return ADG_OK;
}

// ---- autotuner: elements per block of the predictor stages ---------------
// Per GPU model, (D, P), level-0 grid, finest level and stage, the fastest
// elements-per-block choice measured by adg_autotune, kept in a text file
// (ADG_TUNE_CACHE, else $HOME/.cache/adg_gb300/tune.txt), one "key E" line each.
namespace {

std::string tune_cache_path() {
  const char* p = std::getenv("ADG_TUNE_CACHE");
  if (p && *p) return p;
  const char* h = std::getenv("HOME");
  return std::string(h && *h ? h : "/tmp") + "/.cache/adg_gb300/tune.txt";
}

std::string tune_key(const adg_ctx* ctx, const char* stage) {
  int dev = 0;
  cudaDeviceProp prop{};
  std::string gpu = "gpu";
  if (cudaGetDevice(&dev) == cudaSuccess && cudaGetDeviceProperties(&prop, dev) == cudaSuccess) {
    gpu = prop.name;
    for (char& ch : gpu)
      if (ch == ' ' || ch == '\t') ch = '_';
    gpu += "/" + std::to_string(prop.multiProcessorCount) + "sm";
  }
  const adg_config& c = ctx->cfg;
  std::ostringstream k;
  k << gpu << "/D" << c.D << "P" << c.P << "/n" << c.n_cell[0] << "x" << (c.D > 1 ? c.n_cell[1] : 1) << "x"
    << (c.D > 2 ? c.n_cell[2] : 1) << "/L" << c.max_level << "/" << stage;
  return k.str();
}

bool tune_lookup(const std::string& key, int* E) {
  std::ifstream f(tune_cache_path());
  std::string k;
  int e = 0;
  bool found = false;
  while (f >> k >> e)
    if (k == key) {
      *E = e;
      found = true;
    }
  return found;
}

void tune_store(const std::string& key, int E) {
  const std::string path = tune_cache_path();
  std::vector<std::pair<std::string, int>> rows;
  {
    std::ifstream f(path);
    std::string k;
    int e = 0;
    while (f >> k >> e)
      if (k != key) rows.emplace_back(k, e);
  }
  rows.emplace_back(key, E);
  std::error_code ec;
  std::filesystem::create_directories(std::filesystem::path(path).parent_path(), ec);
  std::ofstream f(path, std::ios::trunc);
  for (const auto& r : rows) f << r.first << " " << r.second << "\n";
}

bool choice_built(const KernelSet* ks, int E) {
  const std::vector<int> ch = ks->elems_per_block_choices();
  return std::find(ch.begin(), ch.end(), E) != ch.end();
}

}  // namespace

// Cached choices for a context created with elems_per_block = 0.
static void apply_tuned_choices(adg_ctx* ctx) {
  if (ctx->cfg.elems_per_block > 0) return;
  int E = 0;
  if (tune_lookup(tune_key(ctx, "plain"), &E) && choice_built(ctx->ks, E)) ctx->E = E;
  if (ctx->seed_mode && tune_lookup(tune_key(ctx, ctx->seed_mode == 2 ? "seeded_fp32" : "seeded_fp64"), &E) &&
      choice_built(ctx->ks, E))
    ctx->Es = E;
}

int adg_autotune(adg_ctx* ctx, int nsteps, int* E_out, double* ms, int cap) {
  int rc = check_ready(ctx);
  if (rc) return rc;
  if (nsteps < 1) return fail(ctx, ADG_ERR_ARG, "nsteps must be positive");
  rc = flush_ghosts(ctx);
  if (rc) return rc;
  const std::vector<int> ch = ctx->ks->elems_per_block_choices();
  const bool seeded = ctx->seed_mode && ctx->seed;
  // host counters a step moves; the device state is snapshotted
  const long long nstep = ctx->nstep, dof = ctx->dof_updates, leaf = ctx->leaf_dof_updates,
                  pred = ctx->seed_predicted, launches = ctx->launches;
  const int E0 = ctx->E, Es0 = ctx->Es;
  rc = snapshot_step_state(ctx);
  if (rc) return rc;
  const int NEV = 8;
  std::vector<cudaEvent_t> ev((size_t)NEV * nsteps);
  for (auto& x : ev) ADG_CUDA(cudaEventCreate(&x), "event");
  std::vector<double> t(ch.size(), 0.0);
  for (size_t i = 0; i < ch.size() && rc == ADG_OK; ++i) {
    if (seeded)
      ctx->Es = ch[i];
    else
      ctx->E = ch[i];
    for (int s = 0; s < nsteps && rc == ADG_OK; ++s) rc = launch_step(ctx, &ev[(size_t)s * NEV]);
    if (rc == ADG_OK) {
      cudaError_t e = cudaStreamSynchronize(ctx->stream);
      if (e != cudaSuccess) rc = cuda_fail(ctx, e, "autotune");
    }
    for (int s = 0; s < nsteps && rc == ADG_OK; ++s) {
      float f = 0.f;
      // the predictor stage (plain) or the seeded predictor alone
      cudaEventElapsedTime(&f, ev[(size_t)s * NEV + (seeded ? 6 : 0)], ev[(size_t)s * NEV + (seeded ? 7 : 1)]);
      t[i] += f / nsteps;
    }
    if (rc == ADG_OK) rc = restore_step_state(ctx);
  }
  for (auto& x : ev) cudaEventDestroy(x);
  ctx->nstep = nstep;
  ctx->dof_updates = dof;
  ctx->leaf_dof_updates = leaf;
  ctx->seed_predicted = pred;
  ctx->launches = launches;
  ctx->E = E0;
  ctx->Es = Es0;
  if (rc) return rc;
  ADG_CUDA(cudaStreamSynchronize(ctx->stream), "autotune restore");
  size_t best = 0;
  for (size_t i = 1; i < ch.size(); ++i)
    if (t[i] < t[best]) best = i;
  if (seeded)
    ctx->Es = ch[best];
  else
    ctx->E = ch[best];
  tune_store(tune_key(ctx, seeded ? (ctx->seed_mode == 2 ? "seeded_fp32" : "seeded_fp64") : "plain"), ch[best]);
  ctx->graph_stale = true;  // the captured step used the old choice
  if (E_out) *E_out = ch[best];
  for (int i = 0; i < cap && ms; ++i) ms[i] = i < (int)ch.size() ? t[i] : 0.0;
  return ADG_OK;
}

int adg_block_choices(const adg_ctx* ctx, int* choices, int cap, int* n, int* E_plain, int* E_seeded) {
  if (!ctx) return ADG_ERR_ARG;
  const std::vector<int> ch = ctx->ks->elems_per_block_choices();
  for (int i = 0; i < cap && choices && i < (int)ch.size(); ++i) choices[i] = ch[i];
  if (n) *n = (int)ch.size();
  if (E_plain) *E_plain = ctx->E;
  if (E_seeded) *E_seeded = ctx->Es > 0 ? ctx->Es : (ctx->seed_mode == 2 && ctx->cfg.D == 2 ? 8 : ctx->E);
  return ADG_OK;
}

int adg_time_kernels(adg_ctx* ctx, int nsteps, double* ms, int nkinds) {
  int rc = check_ready(ctx);
  if (rc) return rc;
  if (!ms || nkinds < 1 || nsteps < 1) return ADG_ERR_ARG;
  const int NEV = 8, NK = 8;
  const bool seeded = ctx->seed_mode && ctx->seed;
  std::vector<cudaEvent_t> ev((size_t)NEV * nsteps);
  for (auto& x : ev) ADG_CUDA(cudaEventCreate(&x), "event");
  for (int s = 0; s < nsteps && rc == ADG_OK; ++s) rc = host_step(ctx, false, &ev[(size_t)s * NEV]);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  double acc[NK] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (rc == ADG_OK && e == cudaSuccess) {
    // kinds: predictor stage, numflux, corrector, Dt, AMR sync, seed
    // inference, seeded predictor, fallback pass
    const int from[NK] = {0, 1, 2, 4, 3, 0, 6, 7}, to[NK] = {1, 2, 3, 5, 4, 6, 7, 1};
    for (int s = 0; s < nsteps; ++s)
      for (int k = 0; k < NK; ++k) {
        if (k >= 5 && !seeded) continue;
        float f = 0.f;
        cudaEventElapsedTime(&f, ev[(size_t)s * NEV + from[k]], ev[(size_t)s * NEV + to[k]]);
        acc[k] += f;
      }
  }
  for (auto& x : ev) cudaEventDestroy(x);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(ctx, e, "time kernels");
  for (int k = 0; k < nkinds; ++k) ms[k] = (k < NK) ? acc[k] / nsteps : 0.0;
  return ADG_OK;
}

int adg_host_alloc(size_t bytes, void** ptr) {
  if (!ptr) return ADG_ERR_ARG;
  return cudaHostAlloc(ptr, bytes, cudaHostAllocDefault) == cudaSuccess ? ADG_OK : ADG_ERR_CUDA;
}

int adg_host_free(void* ptr) { return cudaFreeHost(ptr) == cudaSuccess ? ADG_OK : ADG_ERR_CUDA; }

int adg_predictor(adg_ctx* ctx, int lev, double* dst_dev) {
  int rc = check_ready(ctx);
  if (rc) return rc;
  if (!dst_dev || lev < 0 || lev >= ctx->hier.nlevels()) return fail(ctx, ADG_ERR_ARG, "bad level or pointer");
  const size_t ne = ctx->hier.n_elem();
  const size_t per = (size_t)ctx->ks->Q * ctx->ks->Np_st;
  ADG_CUDA(ctx->Hw_dbg.ensure(ne * per), "alloc Hw");
  // Run the ADER stages on a scratch copy of the state so the state is unchanged.
  DevBuf<double> save;
  ADG_CUDA(save.ensure(ctx->Uw.n), "alloc save");
  ADG_CUDA(cudaMemcpyAsync(save.p, ctx->Uw.p, ctx->Uw.n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream), "save");
  rc = launch_ader(ctx, ctx->Hw_dbg.p);
  if (rc) {
    save.release();
    return rc;
  }
  ADG_CUDA(cudaMemcpyAsync(ctx->Uw.p, save.p, ctx->Uw.n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream), "restore");
  const size_t off = ctx->hier.level_valid_offset(lev) * per;
  const size_t cnt = ctx->hier.level_valid_count(lev) * per;
  ADG_CUDA(cudaMemcpyAsync(dst_dev, ctx->Hw_dbg.p + off, cnt * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream), "hw copy");
  ADG_CUDA(cudaStreamSynchronize(ctx->stream), "predictor sync");
  save.release();
  return ADG_OK;
}

int adg_status(adg_ctx* ctx, uint32_t* st) {
  if (!ctx || !st) return ADG_ERR_ARG;
  unsigned int v = 0, zero = 0;
  ADG_CUDA(cudaMemcpyAsync(&v, ctx->status.p, sizeof(v), cudaMemcpyDeviceToHost, ctx->stream), "status");
  ADG_CUDA(cudaMemcpyAsync(ctx->status.p, &zero, sizeof(zero), cudaMemcpyHostToDevice, ctx->stream), "status clear");
  ADG_CUDA(cudaStreamSynchronize(ctx->stream), "status sync");
  *st = v;
  return ADG_OK;
}

int adg_launch_count(const adg_ctx* ctx, int64_t* n) {
  if (!ctx || !n) return ADG_ERR_ARG;
  *n = ctx->launches;
  return ADG_OK;
}

int adg_fp64_peak_probe(double* gflops) {
  if (!gflops) return ADG_ERR_ARG;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return ADG_ERR_CUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return ADG_ERR_CUDA;
  const int blocks = sms * 8, threads = 256, iters = 1000;
  double* out = nullptr;
  if (cudaMalloc(&out, (size_t)blocks * threads * sizeof(double)) != cudaSuccess) return ADG_ERR_CUDA;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fp64_probe<<<blocks, threads>>>(out, 16);
  float best = 1e30f;
  for (int r = 0; r < 3; ++r) {
    cudaEventRecord(e0);
    k_fp64_probe<<<blocks, threads>>>(out, iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    best = std::min(best, ms);
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return ADG_ERR_CUDA;
  const double flops = 2.0 * 32.0 * iters * (double)blocks * threads;
  *gflops = flops / (best * 1e-3) / 1e9;
  return ADG_OK;
}

int adg_flops_per_element(int D, int P, double* algorithmic, double* issued) {
  const KernelSet* ks = kernel_set(D, P);
  if (!ks) return ADG_ERR_ARG;
  const double Q = ks->Q, Nps = ks->Np_s, Npst = ks->Np_st, qst = ks->NQ_ST, qbd = ks->NQ_BD;
  // Dense matvec count of the method (stage-wise reference formulation,
  // Mk_pred U hoisted out of the sweep loop).
  const double Fp = 2 * Q * Npst * Nps + P * 2 * Q * (qst * Npst + D * Npst * qst + Npst * Npst);
  const double Fc = 2 * Q * qst * Npst + 2 * D * 2 * Q * qbd * Npst + 2 * Q * (D * Nps * qst + 2 * D * Nps * qbd) + 2 * Q * Nps;
  if (algorithmic) *algorithmic = Fp + Fc;
  if (issued) *issued = Q * (double)ks->linear_fp64_per_column;
  return ADG_OK;
}

}  // extern "C"

// ===========================================================================
// Learned predictor seed: network, training, inference inside the step.
// ===========================================================================
namespace {

// Few output tiles and a long K split K into slices whose partial sums go to
// red (slice z at z M N) and are then added in slice order: the same result
// on every run, unlike atomic accumulation.
void sgemm(int TA, int TB, int M, int N, int K, const float* A, const float* B, float* C, const float* bias,
           float* aux, int epi, cudaStream_t st, DevBuf<float>* red = nullptr) {
  dim3 grid((N + 63) / 64, (M + 63) / 64, 1);
  const int tiles = grid.x * grid.y;
  const size_t mn = (size_t)M * N;
  if (red && epi == mlp::EPI_STORE && tiles < 64 && K >= 512)
    grid.z = (unsigned)std::min<size_t>(std::min(64, std::max(1, K / 256)), red->n / std::max<size_t>(mn, 1));
  float* out = grid.z > 1 ? red->p : C;
  if (!TA && !TB) mlp::k_sgemm<0, 0><<<grid, 256, 0, st>>>(M, N, K, A, B, out, bias, aux, epi);
  else if (TA && !TB) mlp::k_sgemm<1, 0><<<grid, 256, 0, st>>>(M, N, K, A, B, out, bias, aux, epi);
  else if (!TA && TB) mlp::k_sgemm<0, 1><<<grid, 256, 0, st>>>(M, N, K, A, B, out, bias, aux, epi);
  else mlp::k_sgemm<1, 1><<<grid, 256, 0, st>>>(M, N, K, A, B, out, bias, aux, epi);
  if (grid.z > 1) mlp::k_sum_slices<<<(unsigned)((mn + 255) / 256), 256, 0, st>>>((long long)mn, (int)grid.z, red->p, C);
}

float* P(adg_seed* s, int k) { return s->params.p + s->off[k]; }
float* G(adg_seed* s, int k) { return s->grads.p + s->off[k]; }

cudaError_t seed_work(adg_seed* s, long long rows) {
  if (rows <= s->work_rows) return cudaSuccess;
  const size_t h = s->h;
  DevBuf<float>* hb[] = {&s->Z1, &s->A1, &s->Z2, &s->A2, &s->Z3, &s->A3, &s->dA, &s->dZ};
  for (auto* b : hb) {
    cudaError_t e = b->ensure((size_t)rows * h);
    if (e != cudaSuccess) return e;
  }
  cudaError_t e = s->Y.ensure((size_t)rows * s->n_out);
  if (e == cudaSuccess) {  // split-K slices of the weight gradients and the column-sum blocks
    const size_t mn = std::max({(size_t)s->n_in * h, h * h, h * (size_t)s->n_out});
    e = s->red.ensure(std::max(64 * mn, (size_t)128 * std::max(h, (size_t)s->n_out)));
  }
  if (e == cudaSuccess) e = s->dY.ensure((size_t)rows * s->n_out);
  if (e == cudaSuccess) e = s->Xb.ensure((size_t)rows * s->n_in);
  if (e == cudaSuccess) e = s->Tb.ensure((size_t)rows * s->n_out);
  if (e == cudaSuccess) s->work_rows = rows;
  return e;
}

// Forward with stored pre-activations (training).
void seed_forward_train(adg_seed* s, const float* X, int B, cudaStream_t st) {
  using namespace mlp;
  sgemm(0, 0, B, s->h, s->n_in, X, P(s, 0), s->A1.p, P(s, 1), s->Z1.p, EPI_BIAS_GELU, st);
  sgemm(0, 0, B, s->h, s->h, s->A1.p, P(s, 2), s->A2.p, P(s, 3), s->Z2.p, EPI_BIAS_GELU, st);
  sgemm(0, 0, B, s->h, s->h, s->A2.p, P(s, 4), s->A3.p, P(s, 5), s->Z3.p, EPI_BIAS_GELU, st);
  sgemm(0, 0, B, s->n_out, s->h, s->A3.p, P(s, 6), s->Y.p, P(s, 7), nullptr, EPI_BIAS, st);
}

// Backward from dY (in s->dY) into s->grads.
// Column sums of X[M x N] by row blocks into red, then the blocks added in
// order into out.
void colsum(int M, int N, const float* X, float* out, DevBuf<float>& red, cudaStream_t st) {
  dim3 grid((N + 127) / 128, std::max(1, std::min(128, M / 64)));
  grid.y = (unsigned)std::max<size_t>(1, std::min<size_t>(grid.y, red.n / std::max(N, 1)));
  mlp::k_colsum<<<grid, 128, 0, st>>>(M, N, X, red.p);
  mlp::k_sum_slices<<<(unsigned)((N + 255) / 256), 256, 0, st>>>((long long)N, (int)grid.y, red.p, out);
}

void seed_backward(adg_seed* s, const float* X, int B, cudaStream_t st) {
  using namespace mlp;
  const int h = s->h;
  sgemm(1, 0, h, s->n_out, B, s->A3.p, s->dY.p, G(s, 6), nullptr, nullptr, EPI_STORE, st, &s->red);
  colsum(B, s->n_out, s->dY.p, G(s, 7), s->red, st);
  sgemm(0, 1, B, h, s->n_out, s->dY.p, P(s, 6), s->dZ.p, nullptr, s->Z3.p, EPI_GELU_BWD, st);  // dZ3
  sgemm(1, 0, h, h, B, s->A2.p, s->dZ.p, G(s, 4), nullptr, nullptr, EPI_STORE, st, &s->red);
  colsum(B, h, s->dZ.p, G(s, 5), s->red, st);
  sgemm(0, 1, B, h, h, s->dZ.p, P(s, 4), s->dA.p, nullptr, s->Z2.p, EPI_GELU_BWD, st);  // dZ2
  sgemm(1, 0, h, h, B, s->A1.p, s->dA.p, G(s, 2), nullptr, nullptr, EPI_STORE, st, &s->red);
  colsum(B, h, s->dA.p, G(s, 3), s->red, st);
  sgemm(0, 1, B, h, h, s->dA.p, P(s, 2), s->dZ.p, nullptr, s->Z1.p, EPI_GELU_BWD, st);  // dZ1
  sgemm(1, 0, s->n_in, h, B, X, s->dZ.p, G(s, 0), nullptr, nullptr, EPI_STORE, st, &s->red);
  colsum(B, h, s->dZ.p, G(s, 1), s->red, st);
}

// Inference with ping-pong activations a0, a1 (rows x h each).
void seed_forward_infer(adg_seed* s, const float* X, int B, float* a0, float* a1, float* Y, cudaStream_t st) {
  using namespace mlp;
  sgemm(0, 0, B, s->h, s->n_in, X, P(s, 0), a0, P(s, 1), nullptr, EPI_BIAS_GELU, st);
  sgemm(0, 0, B, s->h, s->h, a0, P(s, 2), a1, P(s, 3), nullptr, EPI_BIAS_GELU, st);
  sgemm(0, 0, B, s->h, s->h, a1, P(s, 4), a0, P(s, 5), nullptr, EPI_BIAS_GELU, st);
  sgemm(0, 0, B, s->n_out, s->h, a0, P(s, 6), Y, P(s, 7), nullptr, EPI_BIAS, st);
}

cudaError_t grow_rows(DevBuf<float>& b, size_t keep, size_t need) {
  if (need <= b.n) return cudaSuccess;
  DevBuf<float> nb;
  cudaError_t e = nb.ensure(std::max(need, b.n * 2));
  if (e != cudaSuccess) return e;
  if (keep) e = cudaMemcpy(nb.p, b.p, keep * sizeof(float), cudaMemcpyDeviceToDevice);
  b.release();
  b = nb;
  nb.p = nullptr;
  nb.n = 0;
  return e;
}

}  // namespace

// Seeded predictor: network inference, seeded sweeps with residual test,
// fallback of rejected elements to the full Picard predictor.
// Pack the weights for k_seed_infer_tc (hidden width 128 only): each layer
// as a K-major B operand, at 4 KB aligned offsets.
int seed_pack_tc(adg_seed* s) {
  s->packed = false;
  if (s->h != kSeedTcHidden || !seed_tc_fits(s->Q, (s->n_in - 1) / s->Q, s->n_out / s->Q)) return ADG_OK;
  const int K1 = seed_tc_k1(s->n_in), N4 = seed_tc_n4(s->n_out), H = s->h;
  const int Kp[4] = {K1, H, H, H}, Np[4] = {H, H, H, N4};
  const int fin[4] = {s->n_in, H, H, H}, fout[4] = {H, H, H, s->n_out};
  long long o = 0;
  for (int L = 0; L < 4; ++L) {
    s->w_off[L] = o;
    o += ((long long)Kp[L] * Np[L] + 1023) / 1024 * 1024;
  }
  if (s->wpack.ensure((size_t)o) != cudaSuccess) return ADG_ERR_CUDA;
  for (int L = 0; L < 4; ++L) {
    const int n = Kp[L] * Np[L];
    k_seed_pack_tc<<<(n + 255) / 256, 256, 0, s->stream>>>(s->params.p + s->off[2 * L], fin[L], fout[L], Kp[L], Np[L],
                                                            s->wpack.p + s->w_off[L]);
  }
  if (cudaStreamSynchronize(s->stream) != cudaSuccess) return ADG_ERR_CUDA;
  s->packed = true;
  return ADG_OK;
}

// H_w seeds of every element of the current layout into dst: the fused
// tensor-core kernel (path 1, when the seed is packed for it) or features +
// four SGEMMs + assembly (path 0).
int seed_infer(adg_ctx* ctx, double* dst, int path, float* dst_f = nullptr) {
  adg_seed* sd = ctx->seed;
  const Hierarchy& H = ctx->hier;
  const KernelSet* ks = ctx->ks;
  const int n = (int)H.n_elem();
  cudaStream_t st = ctx->stream;
  const int8_t* lev = H.nlevels() > 1 ? ctx->elem_level.p : nullptr;
  const LevelGeom geom = level_geom(ctx);
  if (path == 1 && sd->packed) {
    SeedTCArgs ta{};
    ta.Uw = ctx->Uw.p;
    ta.n = n;
    ta.elem_level = lev;
    ta.geom = geom;
    ta.dt = ctx->scal.p;
    ta.wpack = sd->wpack.p;
    for (int L = 0; L < 4; ++L) {
      ta.w_off[L] = sd->w_off[L];
      ta.bias[L] = sd->params.p + sd->off[2 * L + 1];
      if (L < 3 && (reinterpret_cast<uintptr_t>(ta.bias[L]) & 15u))  // read as float4 by the epilogues
        return fail(ctx, ADG_ERR_ARG, "seed biases not 16-byte aligned");
    }
    ta.x_mean = sd->x_mean.p;
    ta.x_istd = sd->x_istd.p;
    ta.y_mean = sd->y_mean.p;
    ta.y_std = sd->y_std.p;
    ta.Hseed = dst;
    ta.Hseed_f = dst_f;
    ta.status = ctx->status.p;
    cudaError_t e = ks->seed_infer_tc(ta, st);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "seed inference (tensor cores)");
    ctx->launches += 1;
    return ADG_OK;
  }
  SeedFeatArgs fa{};
  fa.Uw = ctx->Uw.p;
  fa.e0 = 0;
  fa.n = n;
  fa.elem_level = lev;
  fa.geom = geom;
  fa.dt = ctx->scal.p;
  fa.x_mean = sd->x_mean.p;
  fa.x_istd = sd->x_istd.p;
  fa.X = ctx->sx.p;
  cudaError_t e = ks->seed_features(fa, st);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "seed features");
  seed_forward_infer(sd, ctx->sx.p, n, ctx->sy0.p, ctx->sy1.p, ctx->syo.p, st);
  e = ks->seed_assemble(ctx->Uw.p, ctx->syo.p, sd->y_mean.p, sd->y_std.p, n, lev, geom, ctx->scal.p, dst, st);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "seed assemble");
  ctx->launches += 1 + 4 + 1;  // features, 4 GEMMs, assemble
  return ADG_OK;
}

int launch_seeded_predictor(adg_ctx* ctx, const PredictorArgs& base, cudaEvent_t* ev) {
  const int n = (int)ctx->hier.n_elem();
  const KernelSet* ks = ctx->ks;
  cudaStream_t st = ctx->stream;
  // FP32 sweeps from the tensor-core path take an FP32 seed
  const bool f32 = ctx->seed_mode == 2 && ctx->seed_path == 1 && ctx->seed->packed;
  int rc = seed_infer(ctx, ctx->hseed.p, ctx->seed_path, f32 ? ctx->hseed_f.p : nullptr);
  if (rc) return rc;
  if (ev) cudaEventRecord(ev[6], st);  // end of the seed inference (stage timing)
  cudaError_t e;
  ADG_CUDA(cudaMemsetAsync(ctx->fb_count.p, 0, sizeof(int), st), "fallback reset");
  PredictorArgs pa = base;
  pa.Hseed = ctx->hseed.p;
  pa.Hseed_f = f32 ? ctx->hseed_f.p : nullptr;
  pa.seed_tol = ctx->seed_tol;
  pa.fb_list = ctx->fb_list.p;
  pa.fb_count = ctx->fb_count.p;
  pa.sweeps = ctx->seed_sweeps;
  // the FP32 predictor at D = 2 runs one-warp blocks (8 elements): 16 of them
  // per SM, so the element groups spread evenly over the SMs (at D = 3 the
  // 40-thread blocks of 8 elements idle 3/8 of their lanes: the tuned E stays)
  const int Es = ctx->Es > 0 ? ctx->Es : (ctx->seed_mode == 2 && ctx->cfg.D == 2 ? 8 : ctx->E);
  e = ks->predictor(pa, Es, st, ctx->seed_mode);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "seeded predictor");
  if (ev) cudaEventRecord(ev[7], st);  // end of the seeded predictor, start of the fallback pass
  // full FP64 Picard for the rejected elements; in a mode-2 step with the
  // seeded elements' final stage (mode 3), so that every trace tile is a split tile
  PredictorArgs fb = base;
  fb.elem_list = ctx->fb_list.p;
  fb.list_count = ctx->fb_count.p;
  fb.count_total = ctx->fb_total.p;
  e = ks->predictor(fb, ctx->E, st, ctx->seed_mode == 2 ? 3 : 0);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "fallback predictor");
  ctx->launches += 2;
  return ADG_OK;
}

extern "C" {

int adg_seed_create(int D, int P, int hidden, uint64_t rng_seed, adg_seed** out) {
  if (!out) return ADG_ERR_ARG;
  *out = nullptr;
  const KernelSet* ks = kernel_set(D, P);
  if (!ks || hidden <= 0 || hidden > 4096) return ADG_ERR_ARG;
  adg_seed* s = new adg_seed();
  s->D = D;
  s->P = P;
  s->Q = ks->Q;
  s->ks = ks;
  s->h = hidden;
  s->n_in = ks->Q * ks->Np_s + 1;
  s->n_out = ks->Q * ks->Np_st;
  const size_t h = hidden;
  const size_t sizes[8] = {(size_t)s->n_in * h, h, h * h, h, h * h, h, h * s->n_out, (size_t)s->n_out};
  size_t o = 0;
  for (int k = 0; k < 8; ++k) {
    s->off[k] = o;
    s->sz[k] = sizes[k];
    o += sizes[k];
  }
  s->nparam = o;
  s->rng.seed(rng_seed);
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess ||
      s->params.ensure(o) != cudaSuccess || s->grads.ensure(o) != cudaSuccess || s->am.ensure(o) != cudaSuccess ||
      s->av.ensure(o) != cudaSuccess || s->x_mean.ensure(s->n_in) != cudaSuccess ||
      s->x_istd.ensure(s->n_in) != cudaSuccess || s->y_mean.ensure(s->n_out) != cudaSuccess ||
      s->y_std.ensure(s->n_out) != cudaSuccess || s->loss.ensure(1) != cudaSuccess) {
    delete s;
    return ADG_ERR_CUDA;
  }
  // Glorot-uniform weights, zero biases, identity standardisation
  std::vector<float> hp(o, 0.0f);
  const int fin[4] = {s->n_in, hidden, hidden, hidden}, fout[4] = {hidden, hidden, hidden, s->n_out};
  for (int L = 0; L < 4; ++L) {
    const double a = std::sqrt(6.0 / (fin[L] + fout[L]));
    std::uniform_real_distribution<double> U(-a, a);
    for (size_t i = 0; i < sizes[2 * L]; ++i) hp[s->off[2 * L] + i] = (float)U(s->rng);
  }
  std::vector<float> zin(s->n_in, 0.f), oin(s->n_in, 1.f), zout(s->n_out, 0.f), oout(s->n_out, 1.f);
  cudaMemcpy(s->params.p, hp.data(), o * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemset(s->am.p, 0, o * sizeof(float));
  cudaMemset(s->av.p, 0, o * sizeof(float));
  cudaMemcpy(s->x_mean.p, zin.data(), zin.size() * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(s->x_istd.p, oin.data(), oin.size() * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(s->y_mean.p, zout.data(), zout.size() * 4, cudaMemcpyHostToDevice);
  if (cudaMemcpy(s->y_std.p, oout.data(), oout.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      seed_pack_tc(s) != ADG_OK) {
    delete s;
    return ADG_ERR_CUDA;
  }
  *out = s;
  return ADG_OK;
}

int adg_seed_destroy(adg_seed* s) {
  if (!s) return ADG_ERR_ARG;
  cudaDeviceSynchronize();
  delete s;
  return ADG_OK;
}

int adg_seed_num_samples(const adg_seed* s, int64_t* n) {
  if (!s || !n) return ADG_ERR_ARG;
  *n = s->nsamp;
  return ADG_OK;
}

int adg_seed_collect(adg_ctx* ctx, adg_seed* s, int target_sweeps) {
  int rc = check_ready(ctx);
  if (rc) return rc;
  if (!s || s->D != ctx->cfg.D || s->P != ctx->cfg.P || target_sweeps < 1) return fail(ctx, ADG_ERR_ARG, "bad seed");
  if (s->normalised) return fail(ctx, ADG_ERR_STATE, "data set already standardised by training");
  const Hierarchy& H = ctx->hier;
  const KernelSet* ks = ctx->ks;
  const size_t nv = H.n_valid();
  ADG_CUDA(ctx->Hw_dbg.ensure(H.n_elem() * (size_t)ks->Q * ks->Np_st), "alloc Hw");
  DevBuf<double> save;
  ADG_CUDA(save.ensure(ctx->Uw.n), "alloc save");
  ADG_CUDA(cudaMemcpyAsync(save.p, ctx->Uw.p, ctx->Uw.n * 8, cudaMemcpyDeviceToDevice, ctx->stream), "save");
  const int sw = ctx->sweeps, mode = ctx->seed_mode;
  ctx->sweeps = target_sweeps;
  ctx->seed_mode = 0;
  rc = launch_ader(ctx, ctx->Hw_dbg.p);
  ctx->sweeps = sw;
  ctx->seed_mode = mode;
  if (rc) {
    save.release();
    return rc;
  }
  ADG_CUDA(cudaMemcpyAsync(ctx->Uw.p, save.p, ctx->Uw.n * 8, cudaMemcpyDeviceToDevice, ctx->stream), "restore");
  ADG_CUDA(cudaStreamSynchronize(ctx->stream), "collect sync");
  save.release();
  ADG_CUDA(grow_rows(s->X, (size_t)s->nsamp * s->n_in, (s->nsamp + nv) * (size_t)s->n_in), "grow X");
  ADG_CUDA(grow_rows(s->T, (size_t)s->nsamp * s->n_out, (s->nsamp + nv) * (size_t)s->n_out), "grow T");
  SeedFeatArgs fa{};
  fa.Uw = ctx->Uw.p;
  fa.Hw = ctx->Hw_dbg.p;
  fa.e0 = 0;
  fa.n = (int)nv;
  fa.elem_level = H.nlevels() > 1 ? ctx->elem_level.p : nullptr;
  fa.geom = level_geom(ctx);
  fa.dt = ctx->scal.p;
  fa.X = s->X.p + (size_t)s->nsamp * s->n_in;
  fa.T = s->T.p + (size_t)s->nsamp * s->n_out;
  cudaError_t e = ks->seed_features(fa, ctx->stream);
  if (e == cudaSuccess) e = ks->seed_targets(fa, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "collect kernels");
  ctx->launches += 2;
  ADG_CUDA(cudaStreamSynchronize(ctx->stream), "collect sync");
  s->nsamp += (long long)nv;
  return ADG_OK;
}

static int seed_normalise(adg_seed* s) {
  const long long M = s->nsamp;
  auto moments = [&](DevBuf<float>& X, int F, std::vector<double>& mean, std::vector<double>& sd) -> cudaError_t {
    constexpr int NB = 64;  // blocks per column; their partial sums are added in order here
    DevBuf<double> acc;
    cudaError_t e = acc.ensure(2 * (size_t)F * NB);
    if (e != cudaSuccess) return e;
    dim3 grid(NB, F);
    mlp::k_col_moments<<<grid, 256, 0, s->stream>>>(M, F, X.p, acc.p);
    std::vector<double> h(2 * (size_t)F * NB);
    e = cudaMemcpyAsync(h.data(), acc.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    acc.release();
    mean.resize(F);
    sd.resize(F);
    for (int f = 0; f < F; ++f) {
      double sum = 0.0, sumsq = 0.0;
      for (int b = 0; b < NB; ++b) {
        sum += h[((size_t)f * NB + b) * 2];
        sumsq += h[((size_t)f * NB + b) * 2 + 1];
      }
      mean[f] = sum / M;
      const double var = std::max(0.0, sumsq / M - mean[f] * mean[f]);
      sd[f] = std::sqrt(var);
    }
    return e;
  };
  std::vector<double> xm, xs, ym, ys;
  if (moments(s->X, s->n_in, xm, xs) != cudaSuccess || moments(s->T, s->n_out, ym, ys) != cudaSuccess) return ADG_ERR_CUDA;
  std::vector<float> fxm(s->n_in), fxi(s->n_in), fym(s->n_out), fys(s->n_out), fyi(s->n_out);
  // Feature scale: the spread in the data, floored at 10 % of the feature's
  // mean magnitude so a nearly constant feature (Dt/dx within one run, a
  // mode that is almost zero) does not turn small changes into large inputs.
  double xmax = 0.0;
  for (int f = 0; f < s->n_in; ++f) xmax = std::max(xmax, std::abs(xm[f]) + xs[f]);
  for (int f = 0; f < s->n_in; ++f) {
    fxm[f] = (float)xm[f];
    const double sc = std::max({xs[f], 0.1 * std::abs(xm[f]), 1e-6 * xmax, 1e-30});
    fxi[f] = (float)(1.0 / sc);
  }
  for (int f = 0; f < s->n_out; ++f) {
    fym[f] = (float)ym[f];
    const double sd = ys[f] > 1e-30 ? ys[f] : 1.0;
    fys[f] = (float)sd;
    fyi[f] = (float)(1.0 / sd);
  }
  DevBuf<float> yi;
  if (yi.ensure(s->n_out) != cudaSuccess) return ADG_ERR_CUDA;
  cudaMemcpy(s->x_mean.p, fxm.data(), s->n_in * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(s->x_istd.p, fxi.data(), s->n_in * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(s->y_mean.p, fym.data(), s->n_out * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(s->y_std.p, fys.data(), s->n_out * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(yi.p, fyi.data(), s->n_out * 4, cudaMemcpyHostToDevice);
  mlp::k_standardise<<<(unsigned)((M * s->n_in + 255) / 256), 256, 0, s->stream>>>(M, s->n_in, s->X.p, s->x_mean.p,
                                                                                     s->x_istd.p);
  mlp::k_standardise<<<(unsigned)((M * s->n_out + 255) / 256), 256, 0, s->stream>>>(M, s->n_out, s->T.p, s->y_mean.p,
                                                                                      yi.p);
  cudaError_t e = cudaStreamSynchronize(s->stream);
  yi.release();
  if (e != cudaSuccess) return ADG_ERR_CUDA;
  s->normalised = true;
  return ADG_OK;
}

int adg_seed_train(adg_seed* s, int epochs, int batch, double lr, double* last_loss) {
  if (!s || epochs < 0 || batch <= 0 || !(lr > 0)) return ADG_ERR_ARG;
  if (s->nsamp <= 0) return ADG_ERR_STATE;
  if (!s->normalised) {
    int rc = seed_normalise(s);
    if (rc) return rc;
  }
  if (seed_work(s, batch) != cudaSuccess || s->idx.ensure(s->nsamp) != cudaSuccess) return ADG_ERR_CUDA;
  std::vector<int> perm(s->nsamp);
  for (long long i = 0; i < s->nsamp; ++i) perm[i] = (int)i;
  double epoch_loss = 0.0;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int ep = 0; ep < epochs; ++ep) {
    std::shuffle(perm.begin(), perm.end(), s->rng);
    cudaMemcpyAsync(s->idx.p, perm.data(), perm.size() * 4, cudaMemcpyHostToDevice, s->stream);
    cudaMemsetAsync(s->loss.p, 0, sizeof(double), s->stream);
    for (long long b0 = 0; b0 < s->nsamp; b0 += batch) {
      const int B = (int)std::min<long long>(batch, s->nsamp - b0);
      mlp::k_gather_rows<<<(unsigned)(((long long)B * s->n_in + 255) / 256), 256, 0, s->stream>>>(
          B, s->n_in, s->idx.p + b0, s->X.p, s->Xb.p);
      mlp::k_gather_rows<<<(unsigned)(((long long)B * s->n_out + 255) / 256), 256, 0, s->stream>>>(
          B, s->n_out, s->idx.p + b0, s->T.p, s->Tb.p);
      seed_forward_train(s, s->Xb.p, B, s->stream);
      mlp::k_mse_grad<<<(unsigned)(((long long)B * s->n_out + 255) / 256), 256, 0, s->stream>>>(
          B, s->n_out, s->Y.p, s->Tb.p, s->dY.p, s->loss.p);
      seed_backward(s, s->Xb.p, B, s->stream);
      s->adam_t++;
      const float bc1 = 1.f - (float)std::pow(b1, (double)s->adam_t), bc2 = 1.f - (float)std::pow(b2, (double)s->adam_t);
      mlp::k_adam<<<(unsigned)((s->nparam + 255) / 256), 256, 0, s->stream>>>((int)s->nparam, s->params.p, s->grads.p,
                                                                              s->am.p, s->av.p, (float)lr, b1, b2, eps,
                                                                              bc1, bc2);
    }
    double l = 0.0;
    cudaMemcpyAsync(&l, s->loss.p, sizeof(double), cudaMemcpyDeviceToHost, s->stream);
    if (cudaStreamSynchronize(s->stream) != cudaSuccess) return ADG_ERR_CUDA;
    epoch_loss = l / ((double)s->nsamp * s->n_out);
  }
  if (last_loss) *last_loss = epoch_loss;
  return seed_pack_tc(s);
}

int adg_seed_forward(adg_seed* s, const float* X, int n, float* Y) {
  if (!s || !X || !Y || n <= 0) return ADG_ERR_ARG;
  DevBuf<float> dx, a0, a1, dy;
  if (dx.ensure((size_t)n * s->n_in) != cudaSuccess || a0.ensure((size_t)n * s->h) != cudaSuccess ||
      a1.ensure((size_t)n * s->h) != cudaSuccess || dy.ensure((size_t)n * s->n_out) != cudaSuccess)
    return ADG_ERR_CUDA;
  cudaMemcpyAsync(dx.p, X, (size_t)n * s->n_in * 4, cudaMemcpyHostToDevice, s->stream);
  seed_forward_infer(s, dx.p, n, a0.p, a1.p, dy.p, s->stream);
  cudaMemcpyAsync(Y, dy.p, (size_t)n * s->n_out * 4, cudaMemcpyDeviceToHost, s->stream);
  cudaError_t e = cudaStreamSynchronize(s->stream);
  dx.release(); a0.release(); a1.release(); dy.release();
  return e == cudaSuccess ? ADG_OK : ADG_ERR_CUDA;
}

int adg_seed_gradients(adg_seed* s, const float* X, const float* T, int n, float* grads, double* loss) {
  if (!s || !X || !T || !grads || n <= 0) return ADG_ERR_ARG;
  if (seed_work(s, n) != cudaSuccess) return ADG_ERR_CUDA;
  cudaMemcpyAsync(s->Xb.p, X, (size_t)n * s->n_in * 4, cudaMemcpyHostToDevice, s->stream);
  cudaMemcpyAsync(s->Tb.p, T, (size_t)n * s->n_out * 4, cudaMemcpyHostToDevice, s->stream);
  cudaMemsetAsync(s->loss.p, 0, sizeof(double), s->stream);
  seed_forward_train(s, s->Xb.p, n, s->stream);
  mlp::k_mse_grad<<<(unsigned)(((long long)n * s->n_out + 255) / 256), 256, 0, s->stream>>>(n, s->n_out, s->Y.p,
                                                                                          s->Tb.p, s->dY.p, s->loss.p);
  seed_backward(s, s->Xb.p, n, s->stream);
  double l = 0.0;
  cudaMemcpyAsync(&l, s->loss.p, sizeof(double), cudaMemcpyDeviceToHost, s->stream);
  cudaMemcpyAsync(grads, s->grads.p, s->nparam * 4, cudaMemcpyDeviceToHost, s->stream);
  if (cudaStreamSynchronize(s->stream) != cudaSuccess) return ADG_ERR_CUDA;
  if (loss) *loss = l / ((double)n * s->n_out);
  return ADG_OK;
}

int adg_seed_num_params(const adg_seed* s, int64_t* n_weights, int64_t* n_total) {
  if (!s) return ADG_ERR_ARG;
  if (n_weights) *n_weights = (int64_t)s->nparam;
  if (n_total) *n_total = (int64_t)(s->nparam + 2 * s->n_in + 2 * s->n_out);
  return ADG_OK;
}

int adg_seed_get_params(adg_seed* s, float* out) {
  if (!s || !out) return ADG_ERR_ARG;
  size_t o = 0;
  cudaMemcpy(out, s->params.p, s->nparam * 4, cudaMemcpyDeviceToHost);
  o += s->nparam;
  cudaMemcpy(out + o, s->x_mean.p, s->n_in * 4, cudaMemcpyDeviceToHost);
  o += s->n_in;
  cudaMemcpy(out + o, s->x_istd.p, s->n_in * 4, cudaMemcpyDeviceToHost);
  o += s->n_in;
  cudaMemcpy(out + o, s->y_mean.p, s->n_out * 4, cudaMemcpyDeviceToHost);
  o += s->n_out;
  return cudaMemcpy(out + o, s->y_std.p, s->n_out * 4, cudaMemcpyDeviceToHost) == cudaSuccess ? ADG_OK : ADG_ERR_CUDA;
}

int adg_seed_set_params(adg_seed* s, const float* in) {
  if (!s || !in) return ADG_ERR_ARG;
  size_t o = 0;
  cudaMemcpy(s->params.p, in, s->nparam * 4, cudaMemcpyHostToDevice);
  o += s->nparam;
  cudaMemcpy(s->x_mean.p, in + o, s->n_in * 4, cudaMemcpyHostToDevice);
  o += s->n_in;
  cudaMemcpy(s->x_istd.p, in + o, s->n_in * 4, cudaMemcpyHostToDevice);
  o += s->n_in;
  cudaMemcpy(s->y_mean.p, in + o, s->n_out * 4, cudaMemcpyHostToDevice);
  o += s->n_out;
  s->normalised = true;
  if (cudaMemcpy(s->y_std.p, in + o, s->n_out * 4, cudaMemcpyHostToDevice) != cudaSuccess) return ADG_ERR_CUDA;
  return seed_pack_tc(s);
}

int adg_seed_attach(adg_ctx* ctx, adg_seed* s, int mode, int sweeps, double tol) {
  if (!ctx) return ADG_ERR_ARG;
  if (mode == 0 || !s) {
    ctx->seed = nullptr;
    ctx->seed_mode = 0;
  } else {
    if (s->D != ctx->cfg.D || s->P != ctx->cfg.P || mode < 1 || mode > 2 || sweeps < 0 || !(tol > 0))
      return fail(ctx, ADG_ERR_ARG, "bad seed attach arguments");
    if (!ctx->ks->seed_modes())
      return fail(ctx, ADG_ERR_ARG, "the learned seed is built for D = 2 with P <= 3 and D = 3 with P <= 2");
    ctx->seed = s;
    ctx->seed_mode = mode;
    ctx->seed_sweeps = sweeps;
    ctx->seed_tol = tol;
    ADG_CUDA(ctx->fb_count.ensure(1), "alloc");
    ADG_CUDA(ctx->fb_total.ensure(1), "alloc");
    ADG_CUDA(cudaMemset(ctx->fb_total.p, 0, sizeof(unsigned long long)), "reset");
    ctx->seed_predicted = 0;
    apply_tuned_choices(ctx);
  }
  ctx->tables_dirty = true;  // resizes the inference buffers, drops the graph
  return ADG_OK;
}

int adg_seed_set_path(adg_ctx* ctx, int path) {
  if (!ctx || path < 0 || path > 1) return ADG_ERR_ARG;
  ctx->seed_path = path;
  ctx->graph_stale = true;
  return ADG_OK;
}

int adg_seed_infer(adg_ctx* ctx, double* dst_dev, int path) {
  int rc = check_ready(ctx);
  if (rc) return rc;
  if (!dst_dev || path < 0 || path > 1) return fail(ctx, ADG_ERR_ARG, "bad seed inference arguments");
  if (!ctx->seed) return fail(ctx, ADG_ERR_STATE, "no seed attached");
  rc = seed_infer(ctx, dst_dev, path);
  if (rc) return rc;
  ADG_CUDA(cudaStreamSynchronize(ctx->stream), "seed inference");
  return ADG_OK;
}

int adg_seed_stats(adg_ctx* ctx, int64_t* fallbacks, int64_t* predicted) {
  if (!ctx) return ADG_ERR_ARG;
  unsigned long long t = 0;
  if (ctx->fb_total.p) {
    ADG_CUDA(cudaMemcpyAsync(&t, ctx->fb_total.p, sizeof(t), cudaMemcpyDeviceToHost, ctx->stream), "stats");
    ADG_CUDA(cudaStreamSynchronize(ctx->stream), "stats sync");
  }
  if (fallbacks) *fallbacks = (int64_t)t;
  if (predicted) *predicted = (int64_t)ctx->seed_predicted;
  return ADG_OK;
}

}  // extern "C"

// One (D, P) instantiation of the kernel set.  The build compiles this file
// once per configuration with -DADG_D, -DADG_HDR (generated operator header),
// -DADG_NS (its namespace) and -DADG_FACTORY (factory function name).
#include <atomic>
#include "adg_kernelset.hpp"
#include ADG_HDR

namespace adg {
namespace {

using O = ADG_NS::Ops;

// Dynamic shared memory of k_predictor per phase (ld = E Q + 1 slots per point):
//   FP64 sweeps             D NQ_ST ld doubles   (MODE 0 first sweep: D NQ_INIT)
//   FP32 sweeps (MODE 2)    D NQ_S ld floats     (one time slice at a time)
//   final volume slices     (1 + D) NQ_S ld doubles
//   face traces             2 NQ_BD ld doubles   (one direction at a time)
//   MODE 2, 3 final stage   split_epilogue_doubles (volume and face phases)
//   seed residual           2 E Q doubles
template <int E, int MODE>
constexpr size_t smem_bytes() {
  constexpr size_t ld = E * O::Q + 1;
  constexpr bool split = MODE == 2 || MODE == 3;
  constexpr size_t sweeps = MODE == 2 ? O::D * O::NQ_S * ld * sizeof(float) : O::D * O::NQ_ST * ld * sizeof(double);
  constexpr size_t fin = split ? split_epilogue_doubles<O>(ld) * sizeof(double)
                               : (1 + O::D) * O::NQ_S * ld * sizeof(double);
  constexpr size_t faces = split ? 0 : 2 * O::NQ_BD * ld * sizeof(double);
  constexpr size_t red = 2 * E * O::Q * sizeof(double);
  constexpr size_t m1 = sweeps > fin ? sweeps : fin;
  constexpr size_t m2 = faces > red ? faces : red;
  return m1 > m2 ? m1 : m2;
}

// The dynamic shared-memory limit of a kernel is an attribute of the current
// device's context: it is set once per device (bit d of mask; devices past 63
// set it on every launch), so a process that moves between GPUs sets it on
// each of them.
template <class F>
cudaError_t ensure_smem_attr(std::atomic<unsigned long long>& mask, F* func, size_t bytes) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = (dev >= 0 && dev < 64) ? (1ull << dev) : 0ull;
  if (bit && (mask.load(std::memory_order_acquire) & bit)) return cudaSuccess;
  e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess && bit) mask.fetch_or(bit, std::memory_order_acq_rel);
  return e;
}

template <int E, int MODE>
cudaError_t launch_predictor_mode(const PredictorArgs& a, cudaStream_t s) {
  constexpr size_t smem = smem_bytes<E, MODE>();
  if (a.elem_list && a.list_count) {  // fallback pass (modes 0 and 3): two blocks per SM stride over the list
    if constexpr (MODE == 0 || MODE == 3) {
      static std::atomic<unsigned long long> attr{0};
      cudaError_t e = ensure_smem_attr(attr, k_predictor_list<O, E, MODE>, smem);
      if (e != cudaSuccess) return e;
      int dev = 0, sms = 0;
      if (cudaGetDevice(&dev) != cudaSuccess ||
          cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
        sms = 152;
      int grid = (a.n_elem + E - 1) / E;
      if (grid > 2 * sms) grid = 2 * sms;
      if (grid <= 0) return cudaSuccess;
      k_predictor_list<O, E, MODE><<<grid, E * O::Q, smem, s>>>(a);
      return cudaGetLastError();
    } else {
      return cudaErrorInvalidValue;
    }
  }
  if constexpr (MODE == 3) {
    return cudaErrorInvalidValue;  // mode 3 runs on element lists only
  } else {
    static std::atomic<unsigned long long> attr{0};
    cudaError_t e = ensure_smem_attr(attr, k_predictor<O, E, MODE>, smem);
    if (e != cudaSuccess) return e;
    const int grid = (a.n_elem + E - 1) / E;
    if (grid <= 0) return cudaSuccess;
    k_predictor<O, E, MODE><<<grid, E * O::Q, smem, s>>>(a);
    return cudaGetLastError();
  }
}

// The learned-seed path (predictor modes 1-3, the fused TF32 inference) is
// built for the elements whose network layers fit the fused kernel
// (seed_tc_fits: D = 2 with P <= 3, D = 3 with P <= 2).  Higher degrees run
// the plain FP64 path only, with one elements-per-block choice, which keeps
// their (large, generated) translation units quick to compile.
constexpr bool kSeedModes = seed_tc_fits(O::Q, O::NP_S, O::NP_ST);

template <int E>
cudaError_t launch_predictor(const PredictorArgs& a, cudaStream_t s, int mode) {
  if constexpr (kSeedModes) {
    if (mode == 1) return launch_predictor_mode<E, 1>(a, s);
    if (mode == 2) return launch_predictor_mode<E, 2>(a, s);
    if (mode == 3) return launch_predictor_mode<E, 3>(a, s);
  } else {
    if (mode != 0) return cudaErrorNotSupported;
  }
  return launch_predictor_mode<E, 0>(a, s);
}

// Elements per block of the plain-only configurations: the largest of 16, 8,
// 4 whose FP64 sweep buffers fit the 227 KB of shared memory of a block.
constexpr int lite_elems() {
  return smem_bytes<16, 0>() <= 227 * 1024 ? 16 : smem_bytes<8, 0>() <= 227 * 1024 ? 8 : 4;
}

struct Impl final : KernelSet {
  Impl() {
    D = O::D;
    P = O::P;
    Q = O::Q;
    Np_s = O::NP_S;
    Np_st = O::NP_ST;
    NQ_ST = O::NQ_ST;
    NQ_BD = O::NQ_BD;
    NQ_S = O::NQ_S;
    NM = O::NM;
    TR_TILE = tr_tile<O>();
    linear_fp64_per_column = O::LINEAR_FP64_PER_COLUMN;
  }
  bool seed_modes() const override { return kSeedModes; }
#if ADG_LITE
  std::vector<int> elems_per_block_choices() const override { return {lite_elems()}; }
  size_t predictor_smem(int) const override { return smem_bytes<lite_elems(), 0>(); }
  cudaError_t predictor(const PredictorArgs& a, int, cudaStream_t s, int mode) const override {
    return launch_predictor<lite_elems()>(a, s, mode);
  }
#elif ADG_D == 2
  std::vector<int> elems_per_block_choices() const override { return {8, 16, 32}; }
  size_t predictor_smem(int E) const override {
    return E == 8 ? smem_bytes<8, 0>() : E == 16 ? smem_bytes<16, 0>() : smem_bytes<32, 0>();
  }
  cudaError_t predictor(const PredictorArgs& a, int E, cudaStream_t s, int mode) const override {
    if (E == 8) return launch_predictor<8>(a, s, mode);
    if (E == 16) return launch_predictor<16>(a, s, mode);
    return launch_predictor<32>(a, s, mode);
  }
#else
  std::vector<int> elems_per_block_choices() const override { return {4, 8, 16}; }
  size_t predictor_smem(int E) const override {
    return E == 4 ? smem_bytes<4, 0>() : E == 8 ? smem_bytes<8, 0>() : smem_bytes<16, 0>();
  }
  cudaError_t predictor(const PredictorArgs& a, int E, cudaStream_t s, int mode) const override {
    if (E == 4) return launch_predictor<4>(a, s, mode);
    if (E == 8) return launch_predictor<8>(a, s, mode);
    return launch_predictor<16>(a, s, mode);
  }
#endif
  cudaError_t numflux(const FaceArgs& a, long long nface, cudaStream_t s, bool split) const override {
    if (nface <= 0) return cudaSuccess;
    constexpr int FB = numflux_faces_per_block<O>();
    const unsigned grid = (unsigned)((nface + FB - 1) / FB);
    if (split)
      k_numflux_split<O><<<grid, FB * O::NQ_BD, 0, s>>>(a);
    else
      k_numflux<O><<<grid, FB * O::NQ_BD, 0, s>>>(a);
    return cudaGetLastError();
  }
  cudaError_t corrector(const CorrectorArgs& a, cudaStream_t s) const override {
    const long long n = ((long long)(a.elem_list ? a.n_list : a.n_valid) + (a.rec_of_elem ? a.nrec : 0)) * O::Q;
    // one-warp blocks: at its ~130 registers an SM holds 15 of them, so the
    // columns of ~16k elements run in one wave instead of 1.2
    const int bs = 32;
    k_corrector<O><<<(unsigned)((n + bs - 1) / bs), bs, 0, s>>>(a);
    return cudaGetLastError();
  }
  cudaError_t dt_reduce(const DtArgs& a, cudaStream_t s) const override {
    k_dt_reduce<O><<<(a.n_valid + kDtElems - 1) / kDtElems, 128, 0, s>>>(a);
    return cudaGetLastError();
  }
  cudaError_t average_down(double* Uw, const int* rec, int nrec, cudaStream_t s) const override {
    if (nrec <= 0) return cudaSuccess;
    constexpr int RB = ad_records_per_block<O>();
    k_average_down<O><<<(unsigned)((nrec + RB - 1) / RB), dim3(RB * O::Q, 1 << O::D), 0, s>>>(Uw, rec, nrec);
    return cudaGetLastError();
  }
  cudaError_t scatter(const ScatterArgs& a, cudaStream_t s) const override {
    const long long n = (long long)a.n * O::Q;
    if (n == 0) return cudaSuccess;
    k_scatter<O><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(a);
    return cudaGetLastError();
  }
  cudaError_t interp_scatter(const double* coarse, const int8_t* child, long long n, double* fine,
                             cudaStream_t s) const override {
    if (n <= 0) return cudaSuccess;
    const long long t = n * O::Q;
    k_interp_scatter<O><<<(unsigned)((t + 127) / 128), 128, 0, s>>>(coarse, child, n, fine);
    return cudaGetLastError();
  }
  cudaError_t interp_gather(const double* fine, long long n, double* coarse, cudaStream_t s) const override {
    if (n <= 0) return cudaSuccess;
    const long long t = n * O::Q;
    k_interp_gather<O><<<(unsigned)((t + 127) / 128), 128, 0, s>>>(fine, n, coarse);
    return cudaGetLastError();
  }
  cudaError_t tag(const TagArgs& a, cudaStream_t s) const override {
    if (a.n == 0) return cudaSuccess;
    k_tag<O><<<(a.n + 127) / 128, 128, 0, s>>>(a);
    return cudaGetLastError();
  }
  cudaError_t seed_features(const SeedFeatArgs& a, cudaStream_t s) const override {
    const long long n = (long long)a.n * (O::Q * O::NP_S + 1);
    if (n == 0) return cudaSuccess;
    k_seed_features<O><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a);
    return cudaGetLastError();
  }
  cudaError_t seed_targets(const SeedFeatArgs& a, cudaStream_t s) const override {
    const long long n = (long long)a.n * O::Q;
    if (n == 0) return cudaSuccess;
    k_seed_targets<O><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(a);
    return cudaGetLastError();
  }
  cudaError_t seed_assemble(const double* Uw, const float* Y, const float* y_mean, const float* y_std, int n,
                            const int8_t* elem_level, const LevelGeom& geom, const double* dt, double* Hseed,
                            cudaStream_t s) const override {
    const long long t = (long long)n * O::Q;
    if (t == 0) return cudaSuccess;
    k_seed_assemble<O><<<(unsigned)((t + 127) / 128), 128, 0, s>>>(Uw, Y, y_mean, y_std, n, elem_level, geom, dt,
                                                                    Hseed);
    return cudaGetLastError();
  }
  cudaError_t seed_infer_tc(const SeedTCArgs& a, cudaStream_t s) const override {
    if constexpr (!seed_tc_fits(O::Q, O::NP_S, O::NP_ST)) {
      return cudaErrorNotSupported;  // layers too wide for the fused kernel: the SIMT path serves
    } else {
      if (a.n <= 0) return cudaSuccess;
      static std::atomic<unsigned long long> attr{0};
      cudaError_t e = ensure_smem_attr(attr, k_seed_infer_tc<O>, kSeedTcSmem);
      if (e != cudaSuccess) return e;
      k_seed_infer_tc<O><<<(a.n + kSeedTcRows - 1) / kSeedTcRows, kSeedTcThreads, kSeedTcSmem, s>>>(a);
      return cudaGetLastError();
    }
  }
  cudaError_t limit_tvb(const LimiterArgs& a, cudaStream_t s) const override {
    if (a.n <= 0) return cudaSuccess;
    k_limit_tvb<O><<<(a.n + 127) / 128, 128, 0, s>>>(a);
    return cudaGetLastError();
  }
  cudaError_t lp_norm(const LpArgs& a, cudaStream_t s) const override {
    if (a.n_valid <= 0) return cudaSuccess;
    k_lp_norm<O><<<(a.n_valid + 127) / 128, 128, 0, s>>>(a);
    return cudaGetLastError();
  }
  cudaError_t init_ic(const ICArgs& a, cudaStream_t s) const override {
    const int bs = 64;
    k_init_ic<O><<<(a.n_elem + bs - 1) / bs, bs, 0, s>>>(a);
    return cudaGetLastError();
  }
};

}  // namespace

const KernelSet* ADG_FACTORY() {
  static Impl impl;
  return &impl;
}

}  // namespace adg

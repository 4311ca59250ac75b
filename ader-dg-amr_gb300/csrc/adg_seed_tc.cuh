// Fused learned-seed inference on the 5th-generation tensor cores (sm_103a):
// one CTA takes a tile of 128 elements through
//   features (U / rho_mean, Dt/dx, standardised)            -> tensor memory
//   4 layers  X W + b (GELU on the hidden ones), TF32 MMA   -> TMEM accumulators
//   H_seed = W U + rho_mean (Dt/dx) (Y y_std + y_mean)      -> HBM (FP32 or FP64)
// The same computation as k_seed_features + 4 SGEMMs + k_seed_assemble, with
// the activations kept on chip.
//
// Activations are rounded to TF32 (nearest) and kept in tensor memory, where
// the MMA reads its A operand (row i in lane i).  The weights (B operand) use
// the tcgen05 canonical K-major layout without swizzling: 8-row x 16-byte
// core matrices, contiguous along K (LBO = 128 B) and then along rows
// (SBO = K * 32 B); they are packed into that layout once per parameter
// version (k_seed_pack_tc) and streamed per layer with cp.async.bulk into two
// 64 KB buffers, the next layer's copy overlapping the current epilogue.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "adg_async.cuh"
#include "adg_gelu.cuh"
#include "adg_kernels.cuh"

namespace adg {
namespace tc {

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// TMEM allocation by one whole warp; the address lands in *slot.
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// Shared-memory matrix descriptor: start address, leading (K) and stride
// (8-row group) byte offsets, descriptor version 1, no swizzling.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::tf32: F32 accumulator, TF32 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24.
constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// Arrives on the mbarrier once every MMA issued so far by this thread is done.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// 32 lanes x 32 consecutive 32-bit columns (thread i: lane base+i), waited on.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// FP32 -> TF32 rounded to nearest (ties away from zero), kept in an FP32
// container with the low 13 mantissa bits clear: operands stored this way are
// used exactly by the TF32 MMA, which otherwise drops those bits.
__device__ __forceinline__ float to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// GELU in its logistic form 0.5 z (1 + tanh y) = z / (1 + 2^t) with
// t = -2 log2(e) y = z (c1 + c3 z^2), y = k (z + a z^3): one exponential
// (ex2.approx) and one fast reciprocal.  t is capped at 126, where the
// quotient is below 2^-126 |z|, so the reciprocal stays in its accurate
// range; for t -> -inf the quotient is z.  Its error (~1e-7 relative) is far
// below the TF32 rounding of the activations that follows.
constexpr float kGeluC1 = -2.0f * 1.4426950408889634f * mlp::kGeluK;
constexpr float kGeluC3 = kGeluC1 * mlp::kGeluA;
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float gelu_fast(float z) {
  const float t = fminf(z * fmaf(kGeluC3, z * z, kGeluC1), 126.0f);
  return __fdividef(z, 1.0f + ex2_approx(t));
}

// Float offset of (row, k) in the canonical K-major layout of a matrix with K
// columns (K a multiple of 4): core matrix (row/8, k/4) of 8 x 4 floats.
__host__ __device__ __forceinline__ int kmajor_off(int row, int k, int K) {
  return (row >> 3) * (K * 8) + (k >> 2) * 32 + (row & 7) * 4 + (k & 3);
}

// TMEM stores: 32 lanes x N consecutive 32-bit columns (thread i: lane base+i).
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const float* v) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32};" ::"r"(taddr),
      "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7]), "f"(v[8]), "f"(v[9]),
      "f"(v[10]), "f"(v[11]), "f"(v[12]), "f"(v[13]), "f"(v[14]), "f"(v[15]), "f"(v[16]), "f"(v[17]), "f"(v[18]),
      "f"(v[19]), "f"(v[20]), "f"(v[21]), "f"(v[22]), "f"(v[23]), "f"(v[24]), "f"(v[25]), "f"(v[26]), "f"(v[27]),
      "f"(v[28]), "f"(v[29]), "f"(v[30]), "f"(v[31])
      : "memory");
}
__device__ __forceinline__ void tmem_st4(uint32_t taddr, const float* v) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1, %2, %3, %4};" ::"r"(taddr), "f"(v[0]), "f"(v[1]),
               "f"(v[2]), "f"(v[3])
               : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// N consecutive columns (N a multiple of 4) in loads of four, one wait for
// all of them; the empty asm ties every register to a point after the wait.
template <int N>
__device__ __forceinline__ void tmem_ld_cols(uint32_t taddr, float* v) {
  static_assert(N % 4 == 0, "columns in fours");
  uint32_t r[N];
#pragma unroll
  for (int j = 0; j < N; j += 4)
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];\n"
                 : "=r"(r[j]), "=r"(r[j + 1]), "=r"(r[j + 2]), "=r"(r[j + 3])
                 : "r"(taddr + (uint32_t)j)
                 : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < N; ++j) {
    asm volatile("" : "+r"(r[j]));
    v[j] = __uint_as_float(r[j]);
  }
}

// D[tmem] (+)= A[tmem] B[smem]: the A operand read from tensor memory (row i
// in lane i, K element k in column k).
__device__ __forceinline__ void mma_tf32_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}\n" ::"r"(
          d_tmem),
      "r"(a_tmem), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// double -> float rounded to nearest even, on the integer pipes (the FP64
// pipe of this GPU converts at the DFMA rate, a few lanes per clock).  IEEE
// 754 binary64 -> binary32: a result in the normal range keeps the top 23
// fraction bits, rounds on the 29 dropped ones (adding 2^28 - 1 plus the
// kept lowest bit carries exactly when the dropped bits exceed half, or equal
// it with the kept bit odd) and rebiases the exponent by 1023 - 127 (the
// 8-bit field wraps modulo 2^32 into place).  Subnormal results, overflow and
// NaN take the out-of-line path.
static __device__ __noinline__ uint32_t f64_to_f32_rare(unsigned long long b) {
  const uint32_t e = (uint32_t)(b >> 52) & 0x7ffu;
  if (e >= 1151u) return (e == 2047u && (b & 0xfffffffffffffull) != 0ull) ? 0x7fffffffu : 0x7f800000u;
  if (e < 873u) return 0u;  // below half the smallest subnormal
  const unsigned long long m = (b & 0xfffffffffffffull) | (1ull << 52);
  const uint32_t s = 926u - e;  // 30 .. 53 dropped bits
  const unsigned long long rem = m & ((1ull << s) - 1ull), half = 1ull << (s - 1u);
  uint32_t r = (uint32_t)(m >> s);
  r += (rem > half || (rem == half && (r & 1u))) ? 1u : 0u;
  return r;
}
__device__ __forceinline__ float f64_to_f32_rn(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned long long m = b & 0x7fffffffffffffffull;
  const uint32_t hi = (uint32_t)(b >> 32);
  const uint32_t e = (hi >> 20) & 0x7ffu;
  uint32_t r;
  if (e - 897u < 254u) {  // biased exponents 897 .. 1150: a normal float
    const unsigned long long mr = m + 0x0fffffffull + ((m >> 29) & 1ull);
    r = (uint32_t)(mr >> 29) + 0x40000000u;
  } else if (m == 0ull) {
    r = 0u;
  } else {
    r = f64_to_f32_rare(b);
  }
  return __uint_as_float(r | (hi & 0x80000000u));
}

}  // namespace tc

// Layer sizes of the fused kernel: hidden width fixed at 128, input padded
// to a multiple of 8 (the TF32 MMA's K), output to a multiple of 16 (N of an
// M = 128 MMA).
constexpr int kSeedTcHidden = 128;
constexpr int kSeedTcThreads = 512;  // four threads per row and layer column quarter
constexpr int kSeedTcRows = 128;
constexpr size_t kSeedTcBuf = 65536;                      // one operand buffer
constexpr int kSeedTcUfLd = 53;                           // odd row stride of the FP32 states: lanes = rows
constexpr size_t kSeedTcUf = (size_t)128 * kSeedTcUfLd * 4;
constexpr size_t kSeedTcAux = 6912;                       // barriers, per-row and per-column scalars
constexpr uint32_t kSeedTcTmemCols = 256;                 // accumulator [0, 128), A operand [128, 256)
// staging buffer, two weight buffers, FP32 states, scalars, alignment slack
constexpr size_t kSeedTcSmem = 3 * kSeedTcBuf + kSeedTcUf + kSeedTcAux + 1024;
static_assert(kSeedTcSmem <= 232448, "above the per-block shared memory of sm_103a");

__host__ __device__ constexpr int seed_tc_k1(int n_in) { return (n_in + 7) / 8 * 8; }
__host__ __device__ constexpr int seed_tc_n4(int n_out) { return (n_out + 15) / 16 * 16; }

struct SeedTCArgs {
  const double* Uw;
  int n;                      // elements 0 .. n-1
  const int8_t* elem_level;   // nullptr: all level 0
  LevelGeom geom;
  const double* dt;
  const float* wpack;         // packed W1 | W2 | W3 | W4 (float offsets w_off)
  long long w_off[4];
  const float* bias[4];
  const float* x_mean;
  const float* x_istd;
  const float* y_mean;
  const float* y_std;
  double* Hseed;              // [elem][q][Np_st] (FP64 seed), or
  float* Hseed_f;             // the same in FP32 for FP32 sweeps (used when non-null)
  unsigned int* status;       // kStatusSeedWait on a wait that gave up
};

constexpr uint32_t kStatusSeedWait = 8u;

// The fused kernel's buffers hold layers of at most 128 inputs and outputs,
// a state row of kSeedTcUfLd values and a staged output tile of 128 rows of
// N4 + 4 floats: (D, P) with Q Np_s + 1 <= 128 inputs and Q Np_st <= 112
// outputs (D = 2, P <= 3; D = 3, P <= 2).  Larger elements infer the seed
// with the SIMT kernels.
__host__ __device__ constexpr bool seed_tc_fits(int Q, int np_s, int np_st) {
  return seed_tc_k1(Q * np_s + 1) <= 128 && seed_tc_n4(Q * np_st) <= 128 && Q * np_s <= kSeedTcUfLd &&
         (size_t)kSeedTcRows * (seed_tc_n4(Q * np_st) + 4) * 4 <= kSeedTcBuf;
}

// One CTA of 512 threads per 128 elements (one CTA per SM by its shared
// memory).  Thread 0 issues the copies and the MMAs; every thread takes part
// in the conversions and the epilogues, the four warps of a TMEM lane quarter
// splitting the columns.
//   setup      copies of the state tile and W1 start first; the per-column
//              constants (standardisation, biases) and the rows' Dt/dx are
//              staged while they fly
//   features   states -> FP32 (integer pipes, flat and conflict-free), then
//              x = (U / rho_mean, Dt/dx) standardised, rounded to TF32 and
//              stored into the A columns of TMEM
//   layers     MMA (A from TMEM, B = packed weights from shared memory) ->
//              accumulator; hidden epilogue bias + GELU -> TF32 -> A columns;
//              the next layer's weights stream into the free buffer
//   output     Y y_std + (b y_std + y_mean) scaled by rho_mean Dt/dx plus the
//              copied spatial modes, staged row-major and written as one
//              coalesced block
template <class O>
__global__ void __launch_bounds__(kSeedTcThreads, 1) k_seed_infer_tc(SeedTCArgs a) {
  constexpr int Q = O::Q, NP_S = O::NP_S, NP_ST = O::NP_ST;
  constexpr int NS = Q * NP_S, NIN = NS + 1, NOUT = Q * NP_ST;
  constexpr int K1 = seed_tc_k1(NIN), N4 = seed_tc_n4(NOUT), H = kSeedTcHidden;
  static_assert(seed_tc_fits(Q, NP_S, NP_ST), "layer sizes exceed the fused kernel's buffers");
  // layer L: K = K1 (L = 0) or H; N = N4 (L = 3) or H; packed weight bytes N K 4
  auto kdim = [](int L) { return L == 0 ? K1 : H; };
  auto wbytes = [](int L) { return (uint32_t)((L == 3 ? N4 : H) * (L == 0 ? K1 : H) * 4); };
  constexpr int YLD = N4 + 4;     // staged output row stride: float4 rows, conflict-free quarter-warps
  constexpr int CPQ = N4 / 4;     // output columns per lane quarter thread
  constexpr uint32_t kACol = 128; // first TMEM column of the A operand

  extern __shared__ uint8_t smraw[];
  uint8_t* base = (uint8_t*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  float* act = (float*)base;                            // staged output tile
  float* wbuf[2] = {(float*)(base + kSeedTcBuf), (float*)(base + 2 * kSeedTcBuf)};
  float* uf = (float*)(base + 3 * kSeedTcBuf);          // [row][kSeedTcUfLd]: U_w in FP32
  uint64_t* bars = (uint64_t*)(base + 3 * kSeedTcBuf + kSeedTcUf);  // [0], [1]: weights, [2]: MMA, [3]: states
  uint32_t* tslot = (uint32_t*)(bars + 4);              // TMEM address
  volatile int* issued_flag = (volatile int*)(tslot + 1); // thread 0 issued this layer's MMAs
  double* rowscale = (double*)(bars + 8);               // [128] Dt/dx, then rho_mean Dt/dx
  float* rowscale_f = (float*)(rowscale + kSeedTcRows); // [128] the same in FP32
  float* cdt_s = rowscale_f + kSeedTcRows;              // [128] Dt/dx in FP32
  int* wu_src = (int*)(cdt_s + kSeedTcRows);            // [32] spatial source of a space-time slot
  float* ocst = (float*)(wu_src + 32);                  // [N4][2] y_std, b y_std + y_mean
  int* owu = (int*)(ocst + 2 * 128);                    // [N4] state column copied into an output, or -1
  float* xcs = (float*)(owu + 128);                     // [2][K1] x_mean, x_istd
  float* bcs = xcs + 2 * 128;                           // [3][H] hidden biases
  static_assert(NP_ST <= 32, "space-time slots exceed the copy table");
  static_assert(64 + 8 * 128 + 3 * 4 * 128 + 4 * 32 + 4 * 2 * 128 + 4 * 128 + 4 * 2 * 128 + 4 * 3 * H <= kSeedTcAux,
                "scalars exceed their shared memory");

  const int t = threadIdx.x, warp = t >> 5;
  const int row0 = blockIdx.x * kSeedTcRows;
  const int rows = min(kSeedTcRows, a.n - row0);
  // the tile's states (rows x Q*Np_s doubles, contiguous) go to weight buffer
  // 1 first; W2 follows there once they are converted
  const uint32_t ubytes = (uint32_t)rows * NS * 8u;
  uint32_t issued[2] = {0, 0}, waited[2] = {0, 0};  // weight copies per buffer (thread 0)
  uint32_t mma_issued = 0, mma_waited = 0;          // MMA batches (thread 0)

  if (t == 0) {
    tc::mbar_init(&bars[0], 1);
    tc::mbar_init(&bars[1], 1);
    tc::mbar_init(&bars[2], 1);
    tc::mbar_init(&bars[3], 1);
    tc::fence_mbar_init();
    tc::mbar_expect_tx(&bars[3], ubytes);
    tc::bulk_g2s(wbuf[1], a.Uw + (size_t)row0 * NS, ubytes, &bars[3]);
    tc::mbar_expect_tx(&bars[0], wbytes(0));
    tc::bulk_g2s(wbuf[0], a.wpack + a.w_off[0], wbytes(0), &bars[0]);
    issued[0]++;
  }
  if (warp == 0) tc::tmem_alloc(tslot, kSeedTcTmemCols);
  if (t < NP_ST) {  // W U is a copy of spatial modes into space-time slots
    int idx[NP_S], w[NP_ST];
#pragma unroll
    for (int i = 0; i < NP_S; ++i) idx[i] = i + 1;
    O::template wu<int>(RegInT<int>{idx}, RegOutT<int>{w});
    int s = -1;
#pragma unroll
    for (int k = 0; k < NP_ST; ++k)
      if (k == t) s = w[k] - 1;
    wu_src[t] = s;
  }
  for (int f = t; f < N4; f += kSeedTcThreads) {
    float ys = 0.0f, c = 0.0f;
    if (f < NOUT) {
      ys = __ldg(a.y_std + f);
      c = fmaf(__ldg(a.bias[3] + f), ys, __ldg(a.y_mean + f));
    }
    ocst[2 * f] = ys;
    ocst[2 * f + 1] = c;
  }
  for (int f = t; f < K1; f += kSeedTcThreads) {
    xcs[f] = f < NIN ? __ldg(a.x_mean + f) : 0.0f;
    xcs[K1 + f] = f < NIN ? __ldg(a.x_istd + f) : 0.0f;
  }
  if (t < 3 * H) {
    const float* bp = t < H ? a.bias[0] : (t < 2 * H ? a.bias[1] : a.bias[2]);
    bcs[t] = __ldg(bp + (t & (H - 1)));
  }
  if (t < kSeedTcRows) {
    const int e = min(row0 + t, a.n - 1);
    const int lev = a.elem_level ? a.elem_level[e] : 0;
    const double cdt = a.dt[kScalDtDx + 3 * lev];
    rowscale[t] = cdt;
    cdt_s[t] = tc::f64_to_f32_rn(cdt);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  for (int f = t; f < N4; f += kSeedTcThreads) {
    int off = -1;
    if (f < NOUT) {
      const int q = f / NP_ST, k = f - q * NP_ST;
      off = wu_src[k] >= 0 ? q * NP_S + wu_src[k] : -1;
    }
    owu[f] = off;
  }
  const bool u_ok = tc::mbar_wait(&bars[3], 0);
  if (!u_ok && t == 0) atomicOr(a.status, kStatusSeedWait);

  const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
  {
    // states -> FP32, flat over the tile (conflict-free 8-byte reads)
    const double* uflat = reinterpret_cast<const double*>(wbuf[1]);
    if (u_ok) {
      constexpr int DR = kSeedTcThreads / NS, DF = kSeedTcThreads % NS;
      int r = t / NS, f = t - (t / NS) * NS;
      for (int i = t; i < rows * NS; i += kSeedTcThreads) {
        uf[r * kSeedTcUfLd + f] = tc::f64_to_f32_rn(uflat[i]);
        r += DR;
        f += DF;
        if (f >= NS) {
          f -= NS;
          ++r;
        }
      }
    }
    if (t < kSeedTcRows) {
      const int r = t;
      if (r < rows && u_ok) {
        const double sc = uflat[(size_t)r * NS] * rowscale[r];
        rowscale[r] = sc;
        rowscale_f[r] = tc::f64_to_f32_rn(sc);
      } else {
        rowscale[r] = 0.0;
        rowscale_f[r] = 0.0f;
        cdt_s[r] = 0.0f;
      }
    }
    __syncthreads();
    // features of row r (lane = row: four threads per row, groups of four
    // columns dealt round robin), into the A columns of TMEM
    constexpr int TPR = kSeedTcThreads / kSeedTcRows;
    const int r = t & (kSeedTcRows - 1), part = t >> 7;
    const bool live = r < rows && u_ok;
    const float rinv = live ? __frcp_rn(uf[r * kSeedTcUfLd]) : 1.0f;
    const float cdt = cdt_s[r];
#pragma unroll
    for (int g = part; g < K1 / 4; g += TPR) {
      const int k0 = 4 * g;
      float v[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int f = k0 + i;
        float x = 0.0f;
        if (live && f < NIN) {
          x = f < NS ? uf[r * kSeedTcUfLd + f] * rinv : cdt;
          x = (x - xcs[f]) * xcs[K1 + f];
        }
        v[i] = tc::to_tf32(x);
      }
      tc::tmem_st4(tmem + lane_base + kACol + (uint32_t)k0, v);
    }
  }
  tc::tmem_wait_st();
  tc::fence_before_sync();
  const bool all_u = __syncthreads_and(u_ok) != 0;
  if (t == 0 && all_u) {  // the states are converted: stream W2 into buffer 1
    tc::mbar_expect_tx(&bars[1], wbytes(1));
    tc::bulk_g2s(wbuf[1], a.wpack + a.w_off[1], wbytes(1), &bars[1]);
    issued[1]++;
  }

  bool ok = all_u;
  const int r = (warp & 3) * 32 + (t & 31);  // this thread's row (TMEM lane) in the epilogues
  const int cq = warp >> 2;                   // and its quarter of the columns
#pragma unroll 1
  for (int L = 0; L < 4 && ok; ++L) {
    const int wb = L & 1;
    if (t == 0) {
      bool w_ok = tc::mbar_wait(&bars[wb], waited[wb] & 1);
      if (w_ok) waited[wb]++;
      tc::fence_after_sync();
      if (w_ok) {
        constexpr uint32_t id0 = tc::idesc_tf32(128, H), id3 = tc::idesc_tf32(128, N4);
        const uint32_t idesc = (L == 3) ? id3 : id0;
        // B descriptor of K step s: 256 bytes (16 in the start field) further
        const uint64_t bd = tc::sdesc(tc::smem_u32(wbuf[wb]), 128u, (uint32_t)kdim(L) * 32u);
        if (L == 0) {
#pragma unroll
          for (int s = 0; s < K1 / 8; ++s) tc::mma_tf32_ts(tmem, tmem + kACol + 8u * s, bd + 16u * s, id0, s > 0);
        } else {
#pragma unroll
          for (int s = 0; s < H / 8; ++s) tc::mma_tf32_ts(tmem, tmem + kACol + 8u * s, bd + 16u * s, idesc, s > 0);
        }
        tc::mma_commit(&bars[2]);
        mma_issued++;
      } else {
        atomicOr(a.status, kStatusSeedWait);
      }
      *issued_flag = w_ok ? 1 : 0;
    }
    __syncthreads();
    if (!*issued_flag) {
      ok = false;
      break;
    }
    if (!tc::mbar_wait(&bars[2], L & 1)) {
      if (t == 0) atomicOr(a.status, kStatusSeedWait);
      ok = false;
    }
    tc::fence_after_sync();
    // every thread must agree before touching TMEM the MMA may still use
    if (__syncthreads_and(ok) == 0) {
      ok = false;
      break;
    }
    mma_waited = mma_issued;
    if (t == 0 && L < 2) {  // the buffer of this layer is free: stream layer L + 2
      tc::mbar_expect_tx(&bars[wb], wbytes(L + 2));
      tc::bulk_g2s(wbuf[wb], a.wpack + a.w_off[L + 2], wbytes(L + 2), &bars[wb]);
      issued[wb]++;
    }
    if (L < 3) {
      // hidden epilogue: bias + GELU, rounded to TF32, into the A columns
      const int col0 = cq * 32;
      float v[32];
      tc::tmem_ld32(tmem + lane_base + (uint32_t)col0, v);
      const float* bl = bcs + L * H + col0;
#pragma unroll
      for (int i = 0; i < 32; ++i) v[i] = tc::to_tf32(tc::gelu_fast(v[i] + bl[i]));
      tc::tmem_st32(tmem + lane_base + kACol + (uint32_t)col0, v);
      tc::tmem_wait_st();
      tc::fence_before_sync();
      __syncthreads();
    } else {
      // output layer: row r's seeds (FP32 path) or network outputs Y (FP64
      // path) for this quarter's columns, staged row-major in the free buffer
      const float rs = rowscale_f[r];
      float vv[CPQ];
      tc::tmem_ld_cols<CPQ>(tmem + lane_base + (uint32_t)(cq * CPQ), vv);
#pragma unroll
      for (int j = 0; j < CPQ; j += 4) {
        const int col0 = cq * CPQ + j;
        float o[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int f = col0 + i;
          const float y = fmaf(vv[j + i], ocst[2 * f], ocst[2 * f + 1]);
          if (a.Hseed_f) {
            const int off = owu[f];
            o[i] = fmaf(rs, y, off >= 0 ? uf[r * kSeedTcUfLd + off] : 0.0f);
          } else {
            o[i] = y;
          }
        }
        *reinterpret_cast<float4*>(act + r * YLD + col0) = make_float4(o[0], o[1], o[2], o[3]);
      }
      __syncthreads();
      // the tile's contiguous [rows][NOUT] block, coalesced
      if (a.Hseed_f) {
        if constexpr (NOUT % 4 == 0) {
          float4* dst = reinterpret_cast<float4*>(a.Hseed_f + (size_t)row0 * NOUT);
          for (int i = t; i < rows * (NOUT / 4); i += kSeedTcThreads) {
            const int rr = i / (NOUT / 4), f = 4 * (i - rr * (NOUT / 4));
            dst[i] = *reinterpret_cast<const float4*>(act + rr * YLD + f);
          }
        } else {
          for (int i = t; i < rows * NOUT; i += kSeedTcThreads) {
            const int rr = i / NOUT, f = i - rr * NOUT;
            a.Hseed_f[(size_t)row0 * NOUT + i] = act[rr * YLD + f];
          }
        }
      } else {
        for (int i = t; i < rows * NOUT; i += kSeedTcThreads) {
          const int rr = i / NOUT, f = i - rr * NOUT;
          const int q = f / NP_ST, k = f - q * NP_ST;
          const int src = wu_src[k];
          const double wu = src >= 0 ? a.Uw[((size_t)(row0 + rr) * Q + q) * NP_S + src] : 0.0;
          a.Hseed[(size_t)row0 * NOUT + i] = wu + rowscale[rr] * (double)act[rr * YLD + f];
        }
      }
    }
  }

  // ---- teardown: no copy may still target this CTA's shared memory and no
  // MMA may still use its TMEM
  if (t == 0) {
    while (mma_waited < mma_issued) {
      if (!tc::mbar_wait(&bars[2], mma_waited & 1)) break;
      mma_waited++;
    }
    for (int wb = 0; wb < 2; ++wb)
      while (waited[wb] < issued[wb]) {
        if (!tc::mbar_wait(&bars[wb], waited[wb] & 1)) {
          atomicOr(a.status, kStatusSeedWait);
          break;
        }
        waited[wb]++;
      }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, kSeedTcTmemCols);
  }
}

}  // namespace adg

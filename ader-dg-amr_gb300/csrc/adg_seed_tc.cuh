// Fused learned-seed inference on the 5th-generation tensor cores (sm_103a):
// one CTA takes a tile of 128 elements through
//   features (U / rho_mean, Dt/dx, standardised)            -> shared memory
//   4 layers  X W + b (GELU on the hidden ones), TF32 MMA   -> TMEM accumulators
//   H_seed = W U + rho_mean (Dt/dx) (Y y_std + y_mean)      -> HBM (FP64)
// The same computation as k_seed_features + 4 SGEMMs + k_seed_assemble, with
// the activations kept on chip.
//
// Operands are rounded to TF32 (nearest) as they are written to shared memory.
// Operands use the tcgen05 canonical K-major layout without swizzling: 8-row x
// 16-byte core matrices, contiguous along K (LBO = 128 B) and then along rows
// (SBO = K * 32 B).  Weights are packed into that layout once per parameter
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

// GELU in its logistic form 0.5 z (1 + tanh y) = z / (1 + exp(-2y)) on the
// fast exponential and reciprocal; |y| clamped to 15, where tanh is 1 in
// FP32.  Its error (~1e-7) is far below the TF32 rounding of the
// activations that follows.
__device__ __forceinline__ float gelu_fast(float z) {
  float y = mlp::kGeluK * fmaf(mlp::kGeluA * z, z * z, z);
  y = fminf(fmaxf(y, -15.0f), 15.0f);
  return __fdividef(z, 1.0f + __expf(-2.0f * y));
}

// Float offset of (row, k) in the canonical K-major layout of a matrix with K
// columns (K a multiple of 4): core matrix (row/8, k/4) of 8 x 4 floats.
__host__ __device__ __forceinline__ int kmajor_off(int row, int k, int K) {
  return (row >> 3) * (K * 8) + (k >> 2) * 32 + (row & 7) * 4 + (k & 3);
}

}  // namespace tc

// Layer sizes of the fused kernel: hidden width fixed at 128, input padded
// to a multiple of 8 (the TF32 MMA's K), output to a multiple of 16 (N of an
// M = 128 MMA).
constexpr int kSeedTcHidden = 128;
constexpr int kSeedTcThreads = 512;  // four threads per row and layer column quarter
constexpr int kSeedTcRows = 128;
constexpr size_t kSeedTcBuf = 65536;                     // one operand buffer
constexpr int kSeedTcUfLd = 52;                           // row stride of the FP32 copy of the states
constexpr size_t kSeedTcUf = (size_t)128 * kSeedTcUfLd * 4;
// act, wA, wB, FP32 states, barriers/scalars, alignment slack
constexpr size_t kSeedTcSmem = 3 * kSeedTcBuf + kSeedTcUf + 2048 + 1024;

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

// The fused kernel's buffers hold layers of at most 128 inputs and outputs
// and a state row of kSeedTcUfLd values: (D, P) with Q Np_s + 1 <= 128
// inputs and Q Np_st <= 128 outputs (D = 2, P <= 3; D = 3, P <= 2).  Larger
// elements infer the seed with the SIMT kernels.
__host__ __device__ constexpr bool seed_tc_fits(int Q, int np_s, int np_st) {
  return seed_tc_k1(Q * np_s + 1) <= 128 && seed_tc_n4(Q * np_st) <= 128 && Q * np_s <= kSeedTcUfLd;
}

template <class O>
__global__ void __launch_bounds__(kSeedTcThreads, 1) k_seed_infer_tc(SeedTCArgs a) {
  constexpr int Q = O::Q, NP_S = O::NP_S, NP_ST = O::NP_ST;
  constexpr int NIN = Q * NP_S + 1, NOUT = Q * NP_ST;
  constexpr int K1 = seed_tc_k1(NIN), N4 = seed_tc_n4(NOUT), H = kSeedTcHidden;
  static_assert(K1 <= 128 && N4 <= 128, "layer sizes exceed the operand buffers");
  // layer L: K = K1 (L = 0) or H; N = N4 (L = 3) or H; packed weight bytes N K 4
  auto kdim = [](int L) { return L == 0 ? K1 : H; };
  auto wbytes = [](int L) { return (uint32_t)((L == 3 ? N4 : H) * (L == 0 ? K1 : H) * 4); };
  constexpr int YLD = N4 + 1;  // padded row stride of the staged outputs

  extern __shared__ uint8_t smraw[];
  uint8_t* base = (uint8_t*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  float* act = (float*)base;
  float* wbuf[2] = {(float*)(base + kSeedTcBuf), (float*)(base + 2 * kSeedTcBuf)};
  float* uf = (float*)(base + 3 * kSeedTcBuf);          // [row][kSeedTcUfLd]: U_w in FP32
  uint64_t* bars = (uint64_t*)(base + 3 * kSeedTcBuf + kSeedTcUf);  // [0], [1]: weights, [2]: MMA, [3]: states
  uint32_t* tslot = (uint32_t*)(bars + 4);              // TMEM address
  volatile int* issued_flag = (volatile int*)(tslot + 1); // thread 0 issued this layer's MMAs
  double* rowscale = (double*)(bars + 8);                // 128 doubles after the barriers
  float* rowscale_f = (float*)(rowscale + kSeedTcRows);  // the same in FP32
  int* wu_src = (int*)(rowscale_f + kSeedTcRows);        // NP_ST entries
  static_assert(Q * NP_S <= kSeedTcUfLd, "state row exceeds the FP32 copy");

  const int t = threadIdx.x, warp = t >> 5;
  const int row0 = blockIdx.x * kSeedTcRows;

  if (t == 0) {
    tc::mbar_init(&bars[0], 1);
    tc::mbar_init(&bars[1], 1);
    tc::mbar_init(&bars[2], 1);
    tc::mbar_init(&bars[3], 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) tc::tmem_alloc(tslot, 128);
  if (t < NP_ST) {  // W U is a copy of spatial modes into space-time slots
    double idx[NP_S], w[NP_ST];
#pragma unroll
    for (int i = 0; i < NP_S; ++i) idx[i] = (double)(i + 1);
    O::wu(RegIn{idx}, RegOut{w});
    wu_src[t] = (int)w[t] - 1;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;

  uint32_t issued[2] = {0, 0}, waited[2] = {0, 0};  // weight copies per buffer (thread 0)
  uint32_t mma_issued = 0, mma_waited = 0;          // MMA batches (thread 0)
  const int rows = min(kSeedTcRows, a.n - row0);
  // the tile's states (rows x Q*Np_s doubles, contiguous) go to weight buffer
  // 1 first; W2 follows there once the features are built
  const uint32_t ubytes = (uint32_t)rows * Q * NP_S * 8u;
  if (t == 0) {
    tc::mbar_expect_tx(&bars[0], wbytes(0));
    tc::bulk_g2s(wbuf[0], a.wpack + a.w_off[0], wbytes(0), &bars[0]);
    issued[0]++;
    tc::mbar_expect_tx(&bars[3], ubytes);
    tc::bulk_g2s(wbuf[1], a.Uw + (size_t)row0 * Q * NP_S, ubytes, &bars[3]);
  }
  const bool u_ok = tc::mbar_wait(&bars[3], 0);
  if (!u_ok && t == 0) atomicOr(a.status, kStatusSeedWait);

  // ---- features of row r (four threads per row, groups of four columns
  // dealt round robin)
  {
    constexpr int TPR = kSeedTcThreads / kSeedTcRows;
    const int r = t & (kSeedTcRows - 1), part = t >> 7;
    const int e = row0 + r;
    const bool live = r < rows && u_ok;
    float rinv = 1.0f;
    double cdt = 0.0;
    const double* u = reinterpret_cast<const double*>(wbuf[1]) + (size_t)(live ? r : 0) * Q * NP_S;
    if (live) {
      const double rho = u[0];
      rinv = (float)(1.0 / rho);
      const int lev = a.elem_level ? a.elem_level[e] : 0;
      cdt = a.dt[kScalDtDx + 3 * lev];
      if (part == 0) {
        rowscale[r] = rho * cdt;
        rowscale_f[r] = (float)(rho * cdt);
      }
    } else if (part == 0) {
      rowscale[r] = 0.0;
      rowscale_f[r] = 0.0f;
    }
#pragma unroll
    for (int g = part; g < K1 / 4; g += TPR) {
      const int k0 = 4 * g;
      float v[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int f = k0 + i;
        float x = 0.0f;
        if (live && f < NIN) {
          if (f < Q * NP_S) {
            const float uf32 = (float)u[f];
            uf[r * kSeedTcUfLd + f] = uf32;
            x = uf32 * rinv;
          } else {
            x = (float)cdt;
          }
          x = (x - a.x_mean[f]) * a.x_istd[f];
        }
        v[i] = tc::to_tf32(x);
      }
      *reinterpret_cast<float4*>(act + tc::kmajor_off(r, k0, K1)) = make_float4(v[0], v[1], v[2], v[3]);
    }
  }
  tc::fence_proxy_async();  // generic reads of buffer 1 and writes of act before the async proxy
  tc::fence_before_sync();
  const bool all_u = __syncthreads_and(u_ok) != 0;
  if (t == 0 && all_u) {  // the states are read: stream W2 into buffer 1
    tc::mbar_expect_tx(&bars[1], wbytes(1));
    tc::bulk_g2s(wbuf[1], a.wpack + a.w_off[1], wbytes(1), &bars[1]);
    issued[1]++;
  }

  bool ok = all_u;
  const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
  const int r = (warp & 3) * 32 + (t & 31);  // this thread's row in the epilogues
  const int cq = warp >> 2;                   // and its quarter of the columns
#pragma unroll 1
  for (int L = 0; L < 4 && ok; ++L) {
    const int wb = L & 1;
    if (t == 0) {
      bool w_ok = tc::mbar_wait(&bars[wb], waited[wb] & 1);
      if (w_ok) waited[wb]++;
      tc::fence_after_sync();
      if (w_ok) {
        const uint32_t a0 = tc::smem_u32(act), b0 = tc::smem_u32(wbuf[wb]);
        constexpr uint32_t id0 = tc::idesc_tf32(128, H), id3 = tc::idesc_tf32(128, N4);
        const uint32_t idesc = (L == 3) ? id3 : id0;
        const uint32_t sbo = (uint32_t)kdim(L) * 32u;
        for (int s = 0; s < kdim(L) / 8; ++s)
          tc::mma_tf32(tmem, tc::sdesc(a0 + 256u * s, 128u, sbo), tc::sdesc(b0 + 256u * s, 128u, sbo), idesc,
                       s > 0 ? 1u : 0u);
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
    // every thread must agree before touching shared memory the MMA may still read
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
      // hidden epilogue: bias + GELU, back to shared memory as the next A operand
      const float* b = a.bias[L];
      {
        const int col0 = cq * 32;
        float v[32];
        tc::tmem_ld32(tmem + lane_base + (uint32_t)col0, v);
#pragma unroll
        for (int i = 0; i < 32; i += 4) {
          // biases 16-byte aligned (their offsets in the packed parameters are
          // multiples of 4 floats at hidden width 128; checked by the launcher)
          const float4 bb = __ldg(reinterpret_cast<const float4*>(b + col0 + i));
          float4 o;
          o.x = tc::to_tf32(tc::gelu_fast(v[i + 0] + bb.x));
          o.y = tc::to_tf32(tc::gelu_fast(v[i + 1] + bb.y));
          o.z = tc::to_tf32(tc::gelu_fast(v[i + 2] + bb.z));
          o.w = tc::to_tf32(tc::gelu_fast(v[i + 3] + bb.w));
          *reinterpret_cast<float4*>(act + tc::kmajor_off(r, col0 + i, H)) = o;
        }
      }
      tc::fence_proxy_async();
      tc::fence_before_sync();
      __syncthreads();
    } else {
      // output layer: stage Y + b (rows x N4, padded stride) in the free act buffer
      const float* b = a.bias[3];
#pragma unroll 1
      for (int g = cq; g < N4 / 8; g += 4) {  // groups of 8 columns dealt round robin
        const int col0 = 8 * g;
        float v[8];
        tc::tmem_ld8(tmem + lane_base + (uint32_t)col0, v);
#pragma unroll
        for (int i = 0; i < 8; ++i)
          if (col0 + i < NOUT) act[r * YLD + col0 + i] = v[i] + __ldg(b + col0 + i);
      }
      tc::fence_before_sync();
      __syncthreads();
      // H_seed, coalesced over the tile's contiguous [rows][NOUT] block
      for (int i = t; i < rows * NOUT; i += kSeedTcThreads) {
        const int rr = i / NOUT, f = i - rr * NOUT;
        const int q = f / NP_ST, k = f - q * NP_ST;
        const int src = wu_src[k];
        const float y = act[rr * YLD + f] * __ldg(a.y_std + f) + __ldg(a.y_mean + f);
        if (a.Hseed_f) {
          const float wu = src >= 0 ? uf[rr * kSeedTcUfLd + q * NP_S + src] : 0.0f;
          a.Hseed_f[(size_t)row0 * NOUT + i] = fmaf(rowscale_f[rr], y, wu);
        } else {
          const double wu = src >= 0 ? a.Uw[((size_t)(row0 + rr) * Q + q) * NP_S + src] : 0.0;
          a.Hseed[(size_t)row0 * NOUT + i] = wu + rowscale[rr] * (double)y;
        }
      }
    }
  }

  // ---- teardown: no copy may still target this CTA's shared memory and no
  // MMA may still write its TMEM
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
    tc::tmem_dealloc(tmem, 128);
  }
}

}  // namespace adg

// FP32 kernels of the learned predictor seed: a multilayer perceptron
// (input -> 3 hidden layers with GELU -> output) trained on the GPU.
// Row-major matrices; a batch of B samples is a B x features matrix.
#pragma once

#include <cuda_runtime.h>

#include "adg_gelu.cuh"

namespace adg {
namespace mlp {

enum Epilogue : int {
  EPI_STORE = 0,      // C = acc
  EPI_BIAS = 1,       // C = acc + bias
  EPI_BIAS_GELU = 2,  // Z = acc + bias (stored to aux), C = gelu(Z)
  EPI_GELU_BWD = 3,   // C = acc * gelu'(aux)   (aux = pre-activation Z)
};

// C[M x N] = op(A) op(B) with op(A) = A[M x K] (TA = 0) or A^T with A[K x M]
// (TA = 1), op(B) = B[K x N] (TB = 0) or B^T with B[N x K] (TB = 1).
// 64 x 64 tile per block, 256 threads, 4 x 4 outputs per thread.
template <int TA, int TB>
__global__ void __launch_bounds__(256) k_sgemm(int M, int N, int K, const float* __restrict__ A,
                                               const float* __restrict__ B, float* __restrict__ C,
                                               const float* __restrict__ bias, float* __restrict__ aux, int epi) {
  constexpr int BM = 64, BN = 64, BK = 16;
  __shared__ float As[BK][BM + 4];
  __shared__ float Bs[BK][BN + 4];
  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  // split-K: block z covers K range [kz0, kz1) and, when gridDim.z > 1,
  // stores its partial sums in slice z of C (z M N floats; k_sum_slices adds
  // them in order, so the result does not depend on block timing)
  const int kchunk = (((K + gridDim.z - 1) / gridDim.z) + BK - 1) / BK * BK;
  const int kz0 = blockIdx.z * kchunk, kz1 = min(K, kz0 + kchunk);
  float acc[4][4] = {};
  for (int k0 = kz0; k0 < kz1; k0 += BK) {
    for (int i = tid; i < BM * BK; i += 256) {
      const int m = i % BM, k = i / BM;
      const int gm = m0 + m, gk = k0 + k;
      float v = 0.f;
      if (gm < M && gk < kz1) v = TA ? A[(size_t)gk * M + gm] : A[(size_t)gm * K + gk];
      As[k][m] = v;
    }
    for (int i = tid; i < BN * BK; i += 256) {
      const int n = i % BN, k = i / BN;
      const int gn = n0 + n, gk = k0 + k;
      float v = 0.f;
      if (gn < N && gk < kz1) v = TB ? B[(size_t)gn * K + gk] : B[(size_t)gk * N + gn];
      Bs[k][n] = v;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < BK; ++k) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[k][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[k][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + ty * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gn = n0 + tx * 4 + j;
      if (gn >= N) continue;
      const size_t o = (size_t)gm * N + gn;
      float v = acc[i][j];
      if (gridDim.z > 1) {  // split-K partial sum (EPI_STORE only)
        C[(size_t)blockIdx.z * M * N + o] = v;
        continue;
      }
      if (epi == EPI_BIAS) {
        v += bias[gn];
      } else if (epi == EPI_BIAS_GELU) {
        v += bias[gn];
        if (aux) aux[o] = v;
        v = gelu(v);
      } else if (epi == EPI_GELU_BWD) {
        v *= gelu_grad(aux[o]);
      }
      C[o] = v;
    }
  }
}

// part[y][n] = sum over row block y of X[m][n]; grid.x covers columns,
// grid.y splits the rows (k_sum_slices adds the blocks in order).
__global__ void k_colsum(int M, int N, const float* X, float* part) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const int rows = (M + gridDim.y - 1) / gridDim.y;
  const int m0 = blockIdx.y * rows, m1 = min(M, m0 + rows);
  float s = 0.f;
  for (int m = m0; m < m1; ++m) s += X[(size_t)m * N + n];
  part[(size_t)blockIdx.y * N + n] = s;
}

// dst[i] = sum over s of src[s n + i], added in s order: split partial sums
// reduced the same way on every run.
__global__ void k_sum_slices(long long n, int ns, const float* __restrict__ src, float* __restrict__ dst) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float v = 0.f;
  for (int s = 0; s < ns; ++s) v += src[(size_t)s * n + i];
  dst[i] = v;
}

// dY = (2 / (M N)) (Y - T); loss partial sums into loss_acc (double).
__global__ void k_mse_grad(int M, int N, const float* Y, const float* T, float* dY, double* loss_acc) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  float e = 0.f;
  if (i < (long long)M * N) {
    const float d = Y[i] - T[i];
    dY[i] = 2.0f * d / ((float)M * (float)N);
    e = d * d;
  }
  for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
  if ((threadIdx.x & 31) == 0 && loss_acc) atomicAdd(loss_acc, (double)e);
}

// Adam (Kingma & Ba 2015) on a flat parameter vector.
__global__ void k_adam(int n, float* p, const float* g, float* m, float* v, float lr, float b1, float b2, float eps,
                       float bc1, float bc2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

// Rows idx[b] of X (stride F) into Xb; rows of T likewise.
__global__ void k_gather_rows(int B, int F, const int* idx, const float* X, float* Xb) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)B * F) return;
  const int b = (int)(i / F), f = (int)(i % F);
  Xb[i] = X[(size_t)idx[b] * F + f];
}

// (X - mean) * istd per column, in place.
__global__ void k_standardise(long long M, int F, float* X, const float* mean, const float* istd) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M * F) return;
  const int f = (int)(i % F);
  X[i] = (X[i] - mean[f]) * istd[f];
}

// Column sums and sums of squares (double) over M rows, per block:
// part[(f gridDim.x + block) 2 + {0, 1}], added in order by the host.
__global__ void __launch_bounds__(256) k_col_moments(long long M, int F, const float* X, double* part) {
  const int f = blockIdx.y;
  double s = 0.0, s2 = 0.0;
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < M; m += (long long)gridDim.x * blockDim.x) {
    const double v = X[m * F + f];
    s += v;
    s2 += v * v;
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  __shared__ double ws[8][2];
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    ws[w][0] = s;
    ws[w][1] = s2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
      a += ws[k][0];
      b += ws[k][1];
    }
    double* p = part + ((size_t)f * gridDim.x + blockIdx.x) * 2;
    p[0] = a;
    p[1] = b;
  }
}

}  // namespace mlp
}  // namespace adg

// Zero-copy boundary to a caller's per-box arrays: the state of every valid
// element gathered from (or scattered to) the caller's device arrays laid out
// as AMReX FArrayBoxes, one array per (box, conserved variable) with the Np_s
// modes as components (the reference's U_w(lev, q) MultiFabs,
// Source/NumericalMethod/AmrDG/AmrDG.tpp:300-333).  Device to device, one
// launch per direction, coalesced on both sides through shared memory.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace adg {

// Per valid element: the patch holding it and the element's offset in that
// patch's arrays (i + j jstride + k kstride from the grown box's corner);
// per patch: the Q array pointers and the component stride.
struct PatchTab {
  const int* pid;
  const long long* off;
  double* const* qptr;      // [patch][q]
  const long long* nstride;  // [patch]
  int n;                     // valid elements
  int Q, NS;                 // conserved variables, modes
};

// Elements per block of the copy kernels (block of 256 threads).
constexpr int kPatchElems = 32;

// dir 0: patches -> packed state; dir 1: packed state -> patches.  Shared
// memory holds the block's kPatchElems elements as [element][q * NS + n] with
// an odd row stride: the patch side is read or written with consecutive
// threads on consecutive elements (one (q, n) plane at a time, contiguous
// along x within a box row), the packed side with consecutive threads on
// consecutive doubles.
template <int DIR>
__global__ void k_patch_copy(PatchTab t, double* Uw) {
  extern __shared__ double sm[];
  const int QN = t.Q * t.NS, ld = QN + 1;
  const int e0 = blockIdx.x * kPatchElems;
  const int ne = min(kPatchElems, t.n - e0);
  if (ne <= 0) return;
  if (DIR == 0) {
    for (int idx = threadIdx.x; idx < kPatchElems * QN; idx += blockDim.x) {
      const int el = idx % kPatchElems, c = idx / kPatchElems;
      if (el >= ne) continue;
      const int e = e0 + el, p = t.pid[e], q = c / t.NS, m = c % t.NS;
      sm[el * ld + c] = t.qptr[(size_t)p * t.Q + q][t.off[e] + (long long)m * t.nstride[p]];
    }
    __syncthreads();
    double* dst = Uw + (size_t)e0 * QN;
    for (int idx = threadIdx.x; idx < ne * QN; idx += blockDim.x) dst[idx] = sm[(idx / QN) * ld + idx % QN];
  } else {
    const double* src = Uw + (size_t)e0 * QN;
    for (int idx = threadIdx.x; idx < ne * QN; idx += blockDim.x) sm[(idx / QN) * ld + idx % QN] = src[idx];
    __syncthreads();
    for (int idx = threadIdx.x; idx < kPatchElems * QN; idx += blockDim.x) {
      const int el = idx % kPatchElems, c = idx / kPatchElems;
      if (el >= ne) continue;
      const int e = e0 + el, p = t.pid[e], q = c / t.NS, m = c % t.NS;
      t.qptr[(size_t)p * t.Q + q][t.off[e] + (long long)m * t.nstride[p]] = sm[el * ld + c];
    }
  }
}

inline cudaError_t launch_patch_copy(int dir, const PatchTab& t, double* Uw, cudaStream_t s) {
  if (t.n <= 0) return cudaSuccess;
  const unsigned grid = (unsigned)((t.n + kPatchElems - 1) / kPatchElems);
  const size_t smem = (size_t)kPatchElems * (t.Q * t.NS + 1) * sizeof(double);
  if (dir == 0)
    k_patch_copy<0><<<grid, 256, smem, s>>>(t, Uw);
  else
    k_patch_copy<1><<<grid, 256, smem, s>>>(t, Uw);
  return cudaGetLastError();
}

}  // namespace adg

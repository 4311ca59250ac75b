// One ADER-DG step on a uniform periodic grid that allocates no memory.
//
// Some callers cannot allocate GPU memory at the time they want a step
// done: code running inside another framework's memory pool or arena, a
// pre-sized real-time or embedded loop that must not touch the allocator
// after start-up, or a host that has already handed all device memory to
// its own allocator.  adg_ader_step_noalloc serves them: the caller passes
// the state (input and output, in place) and the step size; every
// intermediate array (volume residuals, face traces, face fluxes, face
// tables) lives in one fixed file-scope device array of
// ADG_NOALLOC_SCRATCH_BYTES bytes, which every GPU that loads the library
// holds until the process exits.
#include <cuda_runtime.h>

#include <atomic>

#include "adg.h"
#include "adg_kernelset.hpp"

namespace adg {
namespace {

constexpr size_t kScratchBytes = (size_t)ADG_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

// The scratch array.  In host code this name is only a host-side stand-in
// for the device symbol; the device address comes from
// cudaGetSymbolAddress once per device (scratch_address below).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device address of the array per device.  Host threads may call at the same
// time: every thread that finds an entry empty looks the address up itself
// and stores the same value, so the entries are atomics.
static std::atomic<void*> g_scratch_addr[kMaxDevices];

// Per-device set-up: the device address of the scratch array on the current
// device.  Returns nullptr if the runtime cannot provide it.
void* scratch_address(int dev) {
  if (dev < 0 || dev >= kMaxDevices) return nullptr;
  void* p = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (!p) {
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess) return nullptr;
    g_scratch_addr[dev].store(p, std::memory_order_release);
  }
  return p;
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// Step size and the periodic face tables, written into the scratch on every
// call (the scratch keeps the previous call's contents, which are never read).
__global__ void k_noalloc_setup(int D, int nx, int ny, int nz, double dt, LevelGeom g, double* dt_slot,
                                int* face_left, int* face_right, int* elem_face) {
  const long long n = (long long)nx * ny * nz;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t == 0) {  // the scalar block the element kernels read: Dt, t, Dt/dx of level 0
    dt_slot[0] = dt;
    dt_slot[1] = 0.0;
    for (int d = 0; d < 3; ++d) dt_slot[kScalDtDx + d] = d < D ? dt / g.dx[0][d] : 0.0;
  }
  if (t >= n) return;
  const int e = (int)t;
  const int i = e % nx, j = (e / nx) % ny, k = e / (nx * ny);
  const int dims[3] = {nx, ny, nz};
  for (int d = 0; d < D; ++d) {
    int lo[3] = {i, j, k}, hi[3] = {i, j, k};
    lo[d] = (lo[d] - 1 + dims[d]) % dims[d];
    hi[d] = (hi[d] + 1) % dims[d];
    const int left = lo[0] + nx * (lo[1] + ny * lo[2]);
    const int right = hi[0] + nx * (hi[1] + ny * hi[2]);
    // face of direction d with index d*n + e is the low face of element e
    face_left[(long long)d * n + e] = left;
    face_right[(long long)d * n + e] = e;
    elem_face[(long long)e * 2 * D + 2 * d + 0] = (int)((long long)d * n + e);
    elem_face[(long long)e * 2 * D + 2 * d + 1] = (int)((long long)d * n + right);
  }
}

}  // namespace
}  // namespace adg

using namespace adg;

extern "C" int adg_ader_step_noalloc(int D, int P, const int n_cell[3], const double prob_lo[3],
                                     const double prob_hi[3], double gamma, double dt, double* U_w,
                                     void* stream) {
  const KernelSet* ks = kernel_set(D, P);
  if (!ks || !n_cell || !prob_lo || !prob_hi || !U_w || !(gamma > 1.0) || !(dt > 0.0)) return ADG_ERR_ARG;
  // An error left pending by earlier work is the caller's: report it without
  // consuming it or launching anything.
  if (cudaPeekAtLastError() != cudaSuccess) return ADG_ERR_CUDA;
  long long n = 1;
  for (int d = 0; d < 3; ++d) {
    const int nd = d < D ? n_cell[d] : 1;
    if (nd <= 0) return ADG_ERR_ARG;
    if (d < D && !(prob_hi[d] > prob_lo[d])) return ADG_ERR_ARG;
    n *= nd;
  }
  if (n > (1LL << 30)) return ADG_ERR_NOALLOC_CAPACITY;
  const int Q = ks->Q;
  const size_t nface = (size_t)D * (size_t)n;
  size_t off = 0;
  const size_t o_dt = off;
  off = align256(off + kScalCount * sizeof(double));
  const size_t o_fl = off;
  off = align256(off + nface * sizeof(int));
  const size_t o_fr = off;
  off = align256(off + nface * sizeof(int));
  const size_t o_ef = off;
  off = align256(off + (size_t)n * 2 * D * sizeof(int));
  const size_t o_rv = off;
  off = align256(off + (size_t)n * Q * ks->Np_s * sizeof(double));
  const size_t o_tr = off;
  off = align256(off + (size_t)n * 2 * D * ks->TR_TILE * sizeof(double));
  const size_t o_fn = off;
  off = align256(off + nface * Q * ks->NM * sizeof(double));
  if (off > kScratchBytes) return ADG_ERR_NOALLOC_CAPACITY;

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return ADG_ERR_CUDA;
  unsigned char* base = (unsigned char*)scratch_address(dev);
  if (!base) return ADG_ERR_CUDA;
  cudaStream_t s = (cudaStream_t)stream;
  double* dt_slot = (double*)(base + o_dt);
  int* face_left = (int*)(base + o_fl);
  int* face_right = (int*)(base + o_fr);
  int* elem_face = (int*)(base + o_ef);

  LevelGeom g{};
  for (int l = 0; l < kMaxLevels; ++l)
    for (int d = 0; d < 3; ++d)
      g.dx[l][d] = d < D ? (prob_hi[d] - prob_lo[d]) / (double)(n_cell[d] << l) : 1.0;

  const int nx = n_cell[0], ny = D > 1 ? n_cell[1] : 1, nz = D > 2 ? n_cell[2] : 1;
  k_noalloc_setup<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(D, nx, ny, nz, dt, g, dt_slot, face_left, face_right,
                                                               elem_face);
  if (cudaGetLastError() != cudaSuccess) return ADG_ERR_CUDA;

  PredictorArgs pa{};
  pa.Uw = U_w;
  pa.n_elem = (int)n;
  pa.elem_level = nullptr;
  pa.geom = g;
  pa.gamma = gamma;
  pa.dt = dt_slot;
  pa.sweeps = P;
  pa.Rvol = (double*)(base + o_rv);
  pa.Tr = (double*)(base + o_tr);
  pa.Hw_out = nullptr;
  int E = D == 2 ? 16 : 8;
  {
    const std::vector<int> ch = ks->elems_per_block_choices();
    bool built = false;
    for (int c : ch) built = built || c == E;
    if (!built) E = ch.front();  // the higher degrees build one choice
  }
  if (ks->predictor(pa, E, s) != cudaSuccess) return ADG_ERR_CUDA;

  FaceArgs fa{};
  fa.Tr = pa.Tr;
  fa.face_left = face_left;
  fa.face_right = face_right;
  for (int d = 0; d < 4; ++d) fa.face_off[d] = (int)((long long)(d < D ? d : D) * n);
  fa.Fnum = (double*)(base + o_fn);
  if (ks->numflux(fa, (long long)nface, s) != cudaSuccess) return ADG_ERR_CUDA;

  CorrectorArgs ca{};
  ca.Uw = U_w;
  ca.Rvol = pa.Rvol;
  ca.Fnum = fa.Fnum;
  ca.elem_face = elem_face;
  ca.n_valid = (int)n;
  ca.elem_level = nullptr;
  ca.geom = g;
  ca.dt = dt_slot;
  if (ks->corrector(ca, s) != cudaSuccess) return ADG_ERR_CUDA;
  return ADG_OK;
}

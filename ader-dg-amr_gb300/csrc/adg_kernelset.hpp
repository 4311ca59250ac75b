// Per-(D, P) kernel set: the host-side view of one instantiation of the
// sm_103a kernels (adg_inst.cu compiled once per configuration).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "adg_kernels.cuh"
#include "adg_seed_tc.cuh"

namespace adg {

struct KernelSet {
  int D, P, Q, Np_s, Np_st, NQ_ST, NQ_BD, NQ_S;
  int NM;       // tangential flux moments per face and variable (Fnum entries)
  int TR_TILE;  // doubles per (element, face) trace tile (Tr entries)
  int linear_fp64_per_column;
  virtual ~KernelSet() = default;
  virtual std::vector<int> elems_per_block_choices() const = 0;
  // the learned-seed predictor modes (1-3) are built for this (D, P)
  virtual bool seed_modes() const = 0;
  virtual size_t predictor_smem(int E) const = 0;
  // mode 0: FP64 Picard; 1 / 2: seeded, FP64 / FP32 sweeps; 3: FP64 Picard with
  // mode 2's final stage (element lists only: the fallback of a mode-2 step).
  // An element list counted on the device (a.list_count, modes 0 and 3: the
  // fallback) is strided over by a short grid; one counted on the host
  // (a.list_count == nullptr, a.n_elem entries) runs one group per block.
  virtual cudaError_t predictor(const PredictorArgs& a, int E, cudaStream_t s, int mode = 0) const = 0;
  // split: the trace tiles are split tiles (predictor modes 2 and 3);
  // nface: the faces computed (a.n_list with a face list)
  virtual cudaError_t numflux(const FaceArgs& a, long long nface, cudaStream_t s, bool split = false) const = 0;
  virtual cudaError_t corrector(const CorrectorArgs& a, cudaStream_t s) const = 0;
  virtual cudaError_t dt_reduce(const DtArgs& a, cudaStream_t s) const = 0;
  virtual cudaError_t init_ic(const ICArgs& a, cudaStream_t s) const = 0;
  virtual cudaError_t average_down(double* Uw, const int* rec, int nrec, cudaStream_t s) const = 0;
  virtual cudaError_t scatter(const ScatterArgs& a, cudaStream_t s) const = 0;
  virtual cudaError_t interp_scatter(const double* coarse, const int8_t* child, long long n, double* fine,
                                     cudaStream_t s) const = 0;
  virtual cudaError_t interp_gather(const double* fine, long long n, double* coarse, cudaStream_t s) const = 0;
  virtual cudaError_t tag(const TagArgs& a, cudaStream_t s) const = 0;
  virtual cudaError_t seed_features(const SeedFeatArgs& a, cudaStream_t s) const = 0;
  virtual cudaError_t seed_targets(const SeedFeatArgs& a, cudaStream_t s) const = 0;
  virtual cudaError_t seed_assemble(const double* Uw, const float* Y, const float* y_mean, const float* y_std, int n,
                                    const int8_t* elem_level, const LevelGeom& geom, const double* dt, double* Hseed,
                                    cudaStream_t s) const = 0;
  virtual cudaError_t seed_infer_tc(const SeedTCArgs& a, cudaStream_t s) const = 0;
  virtual cudaError_t limit_tvb(const LimiterArgs& a, cudaStream_t s) const = 0;
  virtual cudaError_t lp_norm(const LpArgs& a, cudaStream_t s) const = 0;
};

const KernelSet* kernels_D2P1();
const KernelSet* kernels_D2P2();
const KernelSet* kernels_D2P3();
const KernelSet* kernels_D3P1();
const KernelSet* kernels_D3P2();
const KernelSet* kernels_D2P4();
const KernelSet* kernels_D2P5();
const KernelSet* kernels_D2P6();
const KernelSet* kernels_D3P3();

inline const KernelSet* kernel_set(int D, int P) {
  if (D == 2 && P == 1) return kernels_D2P1();
  if (D == 2 && P == 2) return kernels_D2P2();
  if (D == 2 && P == 3) return kernels_D2P3();
  if (D == 2 && P == 4) return kernels_D2P4();
  if (D == 2 && P == 5) return kernels_D2P5();
  if (D == 2 && P == 6) return kernels_D2P6();
  if (D == 3 && P == 1) return kernels_D3P1();
  if (D == 3 && P == 2) return kernels_D3P2();
  if (D == 3 && P == 3) return kernels_D3P3();
  return nullptr;
}

}  // namespace adg

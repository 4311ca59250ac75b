// sm_103a kernels of the ADER-DG element path.
//
// Data layout (HBM, FP64):
//   Uw    [elem][q][n]                 n < Np_s   (spatial modes)
//   Rvol  [elem][q][n]                 M U + sum_d (Dt/dx_d) Sk_corr[d] F_d
//   Tr    [elem][face 2d+s][tile]      tile = field * NQ_BD + t * NS_BD + x (time node t,
//                                      spatial face point x < NS_BD = NQ_BD / N), field: u_q (Q),
//                                      f_q (Q), |un|+c (1); tiles padded to an even count of doubles.
//                                      Seeded FP32 path (split tiles, same size): u_q and f_q at
//                                      the NS_BD spatial points in FP64, then the FP32 changes
//                                      of u_q and f_q over time and |un|+c at the NQ_BD points
//   Fnum  [face][q][j]                 tangential moments (j < NM) of the local
//                                      Lax-Friedrichs flux over the face
// Element-level work is organised in "columns": one thread owns one
// (element, variable) pair and runs the generated straight-line FP64
// operators on it; point-wise physics runs one thread per (element, point).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "adg_device.cuh"

namespace adg {

constexpr int kMaxLevels = 8;

struct LevelGeom {
  double dx[kMaxLevels][3];
};

// Device scalar block of a context: [0] Dt, [1] t, then Dt/dx_d of level l at
// kScalDtDx + 3 l + d, refreshed whenever Dt changes so that the element
// kernels read the ratios instead of dividing per thread.
constexpr int kScalDtDx = 2;
constexpr int kScalCount = kScalDtDx + 3 * kMaxLevels;

// Doubles per (element, face) trace tile in Tr: the 2Q+1 fields at the NQ_BD
// face points, padded to an even count so that every tile starts on a
// 16-byte boundary.
template <class O>
constexpr int tr_tile() {
  return ((2 * O::Q + 1) * O::NQ_BD + 1) & ~1;
}

// Split trace tile of the seeded FP32 path, in the same TT doubles:
//   doubles [0, Q NSB)         u_q at the face's spatial points x        [q][x]
//   doubles [Q NSB, 2 Q NSB)   the normal flux f_q(u) there              [q][x]
//   floats from split_tr_float_off: the changes of u_q and f_q at the
//   space-time face points p = t NSB + x ([q][p] each), then |un|+c [p].
template <class O>
constexpr int split_tr_float_off() {
  return 2 * 2 * O::Q * (O::NQ_BD / O::N);
}
template <class O>
constexpr bool split_tr_fits() {
  return split_tr_float_off<O>() + (2 * O::Q + 1) * O::NQ_BD <= 2 * tr_tile<O>();
}

struct PredictorArgs {
  const double* Uw;
  int n_elem;                 // elements that need a predictor (valid + ghost)
  const int8_t* elem_level;   // nullptr: all level 0
  LevelGeom geom;
  double gamma;
  const double* dt;           // device scalar block (Dt, t, Dt/dx)
  int sweeps;
  double* Rvol;
  double* Tr;
  double* Hw_out;             // optional: final H_w per element [elem][q][Np_st]
  // learned seed (modes 1, 2): initial H_w per element, residual tolerance,
  // fallback list of elements whose seed residual exceeds it
  const double* Hseed;
  const float* Hseed_f;       // FP32 seed (MODE 2; used instead of Hseed when non-null)
  double seed_tol;
  int* fb_list;
  int* fb_count;
  // optional element list (fallback pass): element = elem_list[i], i < *list_count;
  // count_total (optional) accumulates *list_count once per launch
  const int* elem_list;
  const int* list_count;
  unsigned long long* count_total;
  double* ubar_old;           // optional [elem][q]: cell means at the start of the step (TVB limiter)
};

// Point-wise flux stage: H at NQ points of E elements (shared, [point][col])
// -> F_d for every direction d, written over H (d = 0) and into the next
// NQ x ld slabs (d >= 1).
template <class O, int E, int NQ, class T = double>
__device__ __forceinline__ void flux_stage(T* sm, int ld, T gm1) {
  constexpr int Q = O::Q, D = O::D;
  // two points per iteration: their independent FP64 chains hide each
  // other's latency (occupancy is bounded by shared memory, not registers)
#pragma unroll 2
  for (int it = threadIdx.x; it < E * NQ; it += blockDim.x) {
    const int m = it % NQ;
    const int e = it / NQ;
    T* base = sm + m * ld + e * Q;
    T u[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) u[q] = base[q];
    T F[D * Q];
    euler_flux_all<D, T>(u, gm1, F);
#pragma unroll
    for (int d = 0; d < D; ++d)
#pragma unroll
      for (int q = 0; q < Q; ++q) base[d * NQ * ld + q] = F[d * Q + q];
  }
}

// One Picard sweep (AmrDG.tpp:744-827, folded): H = V H_w at the space-time
// points, F_d = f_d(H), H_w' = W U - sum_d c_d A_d F_d.  T: arithmetic of
// the sweep (double on the plain path; float allowed on the seeded path).
template <class O, int E, class T>
__device__ __forceinline__ void picard_sweep(const double* hw, const double* wu, const double* c, T* sm, int col,
                                             double gm1, double* out) {
  constexpr int D = O::D, NP_ST = O::NP_ST, NQ = O::NQ_ST;
  constexpr int LD = E * O::Q + 1;
  O::template vol_eval<T>(RegIn{hw}, ColOutT<T>{sm + col, LD});
  __syncthreads();
  flux_stage<O, E, NQ, T>(sm, LD, (T)gm1);
  __syncthreads();
#pragma unroll
  for (int n = 0; n < NP_ST; ++n) out[n] = wu[n];
  T y[NP_ST];
  O::template proj<0, T>(ColInT<T>{sm + col, LD}, RegOutT<T>{y});
#pragma unroll
  for (int n = 0; n < NP_ST; ++n) out[n] = fma(-c[0], (double)y[n], out[n]);
  O::template proj<1, T>(ColInT<T>{sm + NQ * LD + col, LD}, RegOutT<T>{y});
#pragma unroll
  for (int n = 0; n < NP_ST; ++n) out[n] = fma(-c[1], (double)y[n], out[n]);
  if constexpr (D == 3) {
    O::template proj<2, T>(ColInT<T>{sm + 2 * NQ * LD + col, LD}, RegOutT<T>{y});
#pragma unroll
    for (int n = 0; n < NP_ST; ++n) out[n] = fma(-c[2], (double)y[n], out[n]);
  }
  __syncthreads();
}

// Time slice K of an FP32 Picard sweep: H at the spatial points of time node
// K (vol_eval_slice), its fluxes (F_0 over H, F_d in slab d), and their
// projections accumulated into the space-time modes with the sliced form of
// proj<d>: A_d F = C_d sum_k T_k V_s^T F(., t_k), acc[d] = sum_k T_k V_s^T F_d.
// A column reads and writes only its own entries of the slabs, so the slice
// needs two barriers (columns -> points -> columns).
template <class O, int E, int K>
__device__ __forceinline__ void sweep_slice_f32(const float* hw, float* sm, int col, float gm1,
                                                float (&acc)[O::D][O::NP_ST]) {
  constexpr int D = O::D, Q = O::Q, NS = O::NQ_S, NP_S = O::NP_S, NP_ST = O::NP_ST, LD = E * Q + 1;
  O::template vol_eval_slice<K, float>(RegInT<float>{hw}, ColOutT<float>{sm + col, LD});
  __syncthreads();
  flux_stage<O, E, NS, float>(sm, LD, gm1);
  __syncthreads();
#pragma unroll
  for (int d = 0; d < D; ++d) {
    float v[NP_S];
    O::template vt_sp<float>(ColInT<float>{sm + d * NS * LD + col, LD}, RegOutT<float>{v});
#pragma unroll
    for (int n = 0; n < NP_ST; ++n) {
      const float tv = O::time_val_f(O::st_time(n), K);
      acc[d][n] = K == 0 ? tv * v[O::st_space(n)] : fmaf(tv, v[O::st_space(n)], acc[d][n]);
    }
  }
  if constexpr (K + 1 < O::N) sweep_slice_f32<O, E, K + 1>(hw, sm, col, gm1, acc);
}

// One Picard sweep entirely in FP32 (the seeded path's sweeps), one time
// slice at a time (D NS ld floats of shared memory): H = V hw, F_d = f_d(H),
// and only the change dlt = -sum_d c_d A_d F_d is returned, so that the
// caller forms H_w' = W U + dlt in the precision it needs.
template <class O, int E>
__device__ __forceinline__ void picard_sweep_f32(const float* hw, const float* c, float* sm, int col, float gm1,
                                                 float* dlt) {
  constexpr int D = O::D, NP_ST = O::NP_ST;
  float acc[D][NP_ST];
  sweep_slice_f32<O, E, 0>(hw, sm, col, gm1, acc);
  float y[NP_ST];
  O::template cproj<0, float>(RegInT<float>{acc[0]}, RegOutT<float>{y});
#pragma unroll
  for (int n = 0; n < NP_ST; ++n) dlt[n] = -c[0] * y[n];
  O::template cproj<1, float>(RegInT<float>{acc[1]}, RegOutT<float>{y});
#pragma unroll
  for (int n = 0; n < NP_ST; ++n) dlt[n] = fmaf(-c[1], y[n], dlt[n]);
  if constexpr (D == 3) {
    O::template cproj<2, float>(RegInT<float>{acc[2]}, RegOutT<float>{y});
#pragma unroll
    for (int n = 0; n < NP_ST; ++n) dlt[n] = fmaf(-c[2], y[n], dlt[n]);
  }
  __syncthreads();
}

// Point-wise fluxes of time slice K (H at the NS spatial points of time node
// K in sh, shared [point][col]) accumulated into the time integrals
// Fbar_d = sum_k w_k F_d(., t_k) (fbar, shared [d][point][col]); K = 0
// initialises.  The sum runs in the order of vol_term's time stage.
template <class O, int E, int K>
__device__ __forceinline__ void flux_slice_accumulate(const double* sh, double* fbar, int ld, double gm1) {
  constexpr int Q = O::Q, D = O::D, NS = O::NQ_S;
  const double w = O::weight(K);
#pragma unroll 2
  for (int it = threadIdx.x; it < E * NS; it += blockDim.x) {
    const int m = it % NS;
    const int e = it / NS;
    const double* base = sh + m * ld + e * Q;
    double u[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) u[q] = base[q];
    double F[D * Q];
    euler_flux_all<D, double>(u, gm1, F);
    double* fb = fbar + m * ld + e * Q;
#pragma unroll
    for (int d = 0; d < D; ++d)
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        double& dst = fb[d * NS * ld + q];
        dst = K == 0 ? w * F[d * Q + q] : fma(w, F[d * Q + q], dst);
      }
  }
}

// Volume fluxes of the final H_w, one time slice after the other: shared
// memory holds (1 + D) NS ld doubles instead of the D NQ_ST ld of all
// space-time points at once.  With FACE_FROM_SLICES each column also
// extrapolates its face values of the slice (face_slice) and writes them to
// its element's trace tiles (variable q at time node K).
template <class O, int E, int K>
__device__ __forceinline__ void final_volume_flux(const double* hw, double* sh, double* fbar, int col, int ld,
                                                  double gm1, double* tr_elem, int q) {
  constexpr int D = O::D, NB = O::NQ_BD, NSB = NB / O::N, TT = tr_tile<O>();
  O::template vol_eval_slice<K>(RegIn{hw}, ColOut{sh + col, ld});
  if constexpr (O::FACE_FROM_SLICES) {
    if (tr_elem) {
      double fv[NSB];
#define ADG_FS(DD, SS)                                                           \
  {                                                                              \
    O::template face_slice<DD, SS>(ColIn{sh + col, ld}, RegOut{fv});             \
    double* t = tr_elem + (2 * DD + SS) * TT + q * NB + K * NSB;                 \
    _Pragma("unroll") for (int x = 0; x < NSB; ++x) t[x] = fv[x];               \
  }
      ADG_FS(0, 0)
      ADG_FS(0, 1)
      ADG_FS(1, 0)
      ADG_FS(1, 1)
      if constexpr (D == 3) {
        ADG_FS(2, 0)
        ADG_FS(2, 1)
      }
#undef ADG_FS
    }
  }
  __syncthreads();
  flux_slice_accumulate<O, E, K>(sh, fbar, ld, gm1);
  __syncthreads();
  if constexpr (K + 1 < O::N) final_volume_flux<O, E, K + 1>(hw, sh, fbar, col, ld, gm1, tr_elem, q);
}

// Face traces of direction DIR: H at the points of its two faces
// (AmrDG.tpp:437-493; from the modes, or already in Tr with
// FACE_FROM_SLICES), then the normal flux and wave speed there
// (AmrDG.h:1207-1251), written to Tr in tile order.
template <class O, int E, int DIR>
__device__ __forceinline__ void face_traces(const double* hw, double* sm, int col, int ld, const PredictorArgs& a,
                                            int e0, int limit) {
  constexpr int D = O::D, Q = O::Q, N = O::N, NB = O::NQ_BD, NSB = NB / N, NF = 2 * D, TT = tr_tile<O>();
  if constexpr (!O::FACE_FROM_SLICES) {
    O::template face_eval<DIR, 0>(RegIn{hw}, ColOut{sm + col, ld});
    O::template face_eval<DIR, 1>(RegIn{hw}, ColOut{sm + NB * ld + col, ld});
    __syncthreads();
  }
#pragma unroll 2
  for (int it = threadIdx.x; it < E * 2 * NB; it += blockDim.x) {
    const int p = it % NB;  // tile position t NSB + x
    const int side = (it / NB) & 1;
    const int ee = it / (2 * NB);
    if (e0 + ee >= limit) continue;
    const int elem = a.elem_list ? a.elem_list[e0 + ee] : e0 + ee;
    double* t = a.Tr + ((size_t)elem * NF + 2 * DIR + side) * TT + p;
    double uu[Q], F[Q];
    if constexpr (O::FACE_FROM_SLICES) {
#pragma unroll
      for (int k = 0; k < Q; ++k) uu[k] = t[k * NB];
    } else {
      // face_eval's point m = x N + t (time fastest)
      const double* h = sm + (side * NB + (p % NSB) * N + p / NSB) * ld + ee * Q;
#pragma unroll
      for (int k = 0; k < Q; ++k) uu[k] = h[k];
    }
    const double df = euler_flux_normal<D>(DIR, uu, a.gamma, F);
#pragma unroll
    for (int k = 0; k < Q; ++k) {
      if constexpr (!O::FACE_FROM_SLICES) t[k * NB] = uu[k];
      t[(Q + k) * NB] = F[k];
    }
    t[2 * Q * NB] = df;
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Final stage of the seeded FP32 path.  W U is U constant in time, so the
// final H_w = W U + dlt is H(x, t) = U(x) + delta(x, t) with delta the
// expansion of dlt, the FP32 sweeps' change.  FP64 work is kept to the
// time-independent part: U and F(U) at the NS spatial points (whose volume
// term is taken once, times the sum of the time weights) and at the NSB
// spatial points of every face.  The time-dependent part is the FP32 change
// of the flux F(U + delta) - F(U) (euler_dflux_*), whose rounding is
// relative to the change; it is added to the FP64 part in modal space for
// the volume term (Rvol), and kept apart in the split trace tiles (U and
// f_n(U) in FP64, the changes of u and f_n and the wave speed in FP32) that
// k_numflux_split reads.
// ---------------------------------------------------------------------------

// Shared memory of split_epilogue (doubles): region A = D NS ld doubles (U,
// then F(U) at the spatial points; later the FP32 delta slice and flux
// change sums; later the face buffers), then NS ld floats of U in FP32.
template <class O>
constexpr size_t split_epilogue_doubles(size_t ld) {
  constexpr size_t NS = O::NQ_S, NB = O::NQ_BD, NSB = NB / O::N;
  const size_t vol = O::D * NS * ld + (NS * ld + 1) / 2;
  const size_t faces = (2 * NSB + (2 * NSB + 2 * NB + 1) / 2) * ld;
  return vol > faces ? vol : faces;
}

// Time slice K: delta at the spatial points of time node K (column), then the
// flux changes at those points accumulated with the time weights (points).
template <class O, int E, int K>
__device__ __forceinline__ void delta_slices(const float* dlt, const float* us32, float* ds32, float* fb32, int col,
                                             float gm1f) {
  constexpr int D = O::D, Q = O::Q, NS = O::NQ_S, LD = E * Q + 1;
  O::template vol_eval_slice<K, float>(RegInT<float>{dlt}, ColOutT<float>{ds32 + col, LD});
  __syncthreads();
  const float w = O::weight_f(K);
#pragma unroll 2
  for (int it = threadIdx.x; it < E * NS; it += blockDim.x) {
    const int m = it % NS;
    const int ee = it / NS;
    float uu[Q], du[Q], dF[D * Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) {
      uu[k] = us32[m * LD + ee * Q + k];
      du[k] = ds32[m * LD + ee * Q + k];
    }
    euler_dflux_all<D>(uu, du, gm1f, dF);
    float* f = fb32 + m * LD + ee * Q;
#pragma unroll
    for (int d = 0; d < D; ++d)
#pragma unroll
      for (int k = 0; k < Q; ++k) {
        float& dst = f[d * NS * LD + k];
        dst = K == 0 ? w * dF[d * Q + k] : fmaf(w, dF[d * Q + k], dst);
      }
  }
  __syncthreads();
  if constexpr (K + 1 < O::N) delta_slices<O, E, K + 1>(dlt, us32, ds32, fb32, col, gm1f);
}

// Column part of one face side: U at the face's spatial points (FP64) and
// delta at its space-time points (FP32), to shared memory and to the split
// trace tile (u_q and its change).
template <class O, int E, int DIR, int S>
__device__ __forceinline__ void split_face_column(const double* u, const float* dlt, double* uface64, float* uf32,
                                                  float* dface32, int col, int q, double* tr_elem) {
  constexpr int N = O::N, NB = O::NQ_BD, NSB = NB / N, LD = E * O::Q + 1, TT = tr_tile<O>();
  double uf[NSB];
  float df[NB];
  O::template face_eval_sp<DIR, S>(RegIn{u}, RegOut{uf});
  O::template face_eval<DIR, S, float>(RegInT<float>{dlt}, RegOutT<float>{df});  // point x N + t
  double* t = tr_elem ? tr_elem + (2 * DIR + S) * TT : nullptr;
#pragma unroll
  for (int x = 0; x < NSB; ++x) {
    uface64[(S * NSB + x) * LD + col] = uf[x];
    uf32[(S * NSB + x) * LD + col] = (float)uf[x];
    if (t) t[q * NSB + x] = uf[x];
  }
  float* tf = t ? reinterpret_cast<float*>(t) + split_tr_float_off<O>() + q * NB : nullptr;
#pragma unroll
  for (int tt = 0; tt < N; ++tt)
#pragma unroll
    for (int x = 0; x < NSB; ++x) {
      const int p = tt * NSB + x;  // tile position
      const float d = df[x * N + tt];
      dface32[(S * NB + p) * LD + col] = d;
      if (tf) tf[p] = d;
    }
}

// The two faces of direction DIR as split trace tiles: u and its change
// (columns), then f_n(u) at the faces' spatial points (FP64) and, per
// space-time face point, the change of f_n and the wave speed (FP32).
template <class O, int E, int DIR>
__device__ __forceinline__ void split_faces(const double* u, const float* dlt, double* sm, int col, int q,
                                            double* tr_elem, const PredictorArgs& a, int e0, int limit) {
  constexpr int D = O::D, Q = O::Q, N = O::N, NB = O::NQ_BD, NSB = NB / N, NF = 2 * D, TT = tr_tile<O>();
  constexpr int LD = E * Q + 1, FO = split_tr_float_off<O>();
  static_assert(split_tr_fits<O>(), "split trace tile larger than the FP64 tile");
  double* uface64 = sm;                                         // [side][x][col]
  float* uf32 = reinterpret_cast<float*>(sm + 2 * NSB * LD);    // [side][x][col]
  float* dface32 = uf32 + 2 * NSB * LD;                         // [side][t NSB + x][col]
  split_face_column<O, E, DIR, 0>(u, dlt, uface64, uf32, dface32, col, q, tr_elem);
  split_face_column<O, E, DIR, 1>(u, dlt, uface64, uf32, dface32, col, q, tr_elem);
  __syncthreads();
  for (int it = threadIdx.x; it < E * 2 * NSB; it += blockDim.x) {
    const int x = it % NSB;
    const int s = (it / NSB) & 1;
    const int ee = it / (2 * NSB);
    if (e0 + ee >= limit) continue;
    const int elem = a.elem_list ? a.elem_list[e0 + ee] : e0 + ee;
    const double* b = uface64 + (s * NSB + x) * LD + ee * Q;
    double uu[Q], F[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) uu[k] = b[k];
    (void)euler_flux_normal<D>(DIR, uu, a.gamma, F);
    double* t = a.Tr + ((size_t)elem * NF + 2 * DIR + s) * TT + Q * NSB + x;
#pragma unroll
    for (int k = 0; k < Q; ++k) t[k * NSB] = F[k];
  }
  const float gm1f = (float)(a.gamma - 1.0), gf = (float)a.gamma;
#pragma unroll 2
  for (int it = threadIdx.x; it < E * 2 * NB; it += blockDim.x) {
    const int p = it % NB;
    const int s = (it / NB) & 1;
    const int ee = it / (2 * NB);
    if (e0 + ee >= limit) continue;
    const int elem = a.elem_list ? a.elem_list[e0 + ee] : e0 + ee;
    const int x = p % NSB;
    float uu[Q], du[Q], dF[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) {
      uu[k] = uf32[(s * NSB + x) * LD + ee * Q + k];
      du[k] = dface32[(s * NB + p) * LD + ee * Q + k];
    }
    const float ws = euler_dflux_normal<D>(DIR, uu, du, gm1f, gf, dF);
    float* t = reinterpret_cast<float*>(a.Tr + ((size_t)elem * NF + 2 * DIR + s) * TT) + FO + p;
#pragma unroll
    for (int k = 0; k < Q; ++k) t[(Q + k) * NB] = dF[k];
    t[2 * Q * NB] = ws;
  }
  __syncthreads();
}

template <class O, int E>
__device__ __forceinline__ void split_epilogue(const double* u, const float* uf, const float* dlt, const double* c,
                                               double gm1, double* sm, int col, int q, bool live, int e, int e0,
                                               int limit, const PredictorArgs& a) {
  constexpr int D = O::D, Q = O::Q, NP_S = O::NP_S, NS = O::NQ_S, NF = 2 * D;
  constexpr int LD = E * Q + 1;
  double* us64 = sm;  // U, then F_0(U) in place
  double* fU64 = sm;  // F_d(U) in slab d
  float* us32 = reinterpret_cast<float*>(sm + D * NS * LD);

  // U at the spatial points (FP64, and in FP32 from the FP32 modes uf for
  // the flux changes)
  O::sp_eval(RegIn{u}, ColOut{us64 + col, LD});
  O::template sp_eval<float>(RegInT<float>{uf}, ColOutT<float>{us32 + col, LD});
  __syncthreads();
  // F(U) at the spatial points (FP64)
  flux_stage<O, E, NS, double>(us64, LD, gm1);
  __syncthreads();
  // volume term of the time-constant part (AmrDG.tpp:696-709 with F = F(U)):
  // M U + sum_d c_d (sum_k w_k) Sk_d F_d(U)
  double R[NP_S], v[NP_S];
#pragma unroll
  for (int n = 0; n < NP_S; ++n) R[n] = O::mdiag(n) * u[n];
  O::template vol_term_sp<0>(ColIn{fU64 + col, LD}, RegOut{v});
#pragma unroll
  for (int n = 0; n < NP_S; ++n) R[n] = fma(c[0] * O::WEIGHT_SUM, v[n], R[n]);
  O::template vol_term_sp<1>(ColIn{fU64 + NS * LD + col, LD}, RegOut{v});
#pragma unroll
  for (int n = 0; n < NP_S; ++n) R[n] = fma(c[1] * O::WEIGHT_SUM, v[n], R[n]);
  if constexpr (D == 3) {
    O::template vol_term_sp<2>(ColIn{fU64 + 2 * NS * LD + col, LD}, RegOut{v});
#pragma unroll
    for (int n = 0; n < NP_S; ++n) R[n] = fma(c[2] * O::WEIGHT_SUM, v[n], R[n]);
  }
  __syncthreads();
  // time-dependent part: the time integrals of the flux changes (FP32)
  float* ds32 = reinterpret_cast<float*>(sm);
  float* fb32 = ds32 + NS * LD;
  delta_slices<O, E, 0>(dlt, us32, ds32, fb32, col, (float)gm1);
  {  // summed over the directions in FP32, one conversion per mode
    float w[NP_S], ws[NP_S];
    O::template vol_term_sp<0, float>(ColInT<float>{fb32 + col, LD}, RegOutT<float>{w});
#pragma unroll
    for (int n = 0; n < NP_S; ++n) ws[n] = (float)c[0] * w[n];
    O::template vol_term_sp<1, float>(ColInT<float>{fb32 + NS * LD + col, LD}, RegOutT<float>{w});
#pragma unroll
    for (int n = 0; n < NP_S; ++n) ws[n] = fmaf((float)c[1], w[n], ws[n]);
    if constexpr (D == 3) {
      O::template vol_term_sp<2, float>(ColInT<float>{fb32 + 2 * NS * LD + col, LD}, RegOutT<float>{w});
#pragma unroll
      for (int n = 0; n < NP_S; ++n) ws[n] = fmaf((float)c[2], w[n], ws[n]);
    }
#pragma unroll
    for (int n = 0; n < NP_S; ++n) R[n] += (double)ws[n];
  }
  if (live) {
    double* dst = a.Rvol + ((size_t)e * Q + q) * NP_S;
#pragma unroll
    for (int n = 0; n < NP_S; ++n) dst[n] = R[n];
  }
  __syncthreads();
  // face traces, one direction at a time
  double* tr_elem = live ? a.Tr + (size_t)e * NF * tr_tile<O>() : nullptr;
  split_faces<O, E, 0>(u, dlt, sm, col, q, tr_elem, a, e0, limit);
  split_faces<O, E, 1>(u, dlt, sm, col, q, tr_elem, a, e0, limit);
  if constexpr (D == 3) split_faces<O, E, 2>(u, dlt, sm, col, q, tr_elem, a, e0, limit);
}

// Final stage of the FP64 paths: the corrector volume term and the face
// traces of the final H_w.
template <class O, int E>
__device__ __forceinline__ void fp64_epilogue(const double* hw, const double* u, const double* c, double gm1,
                                              double* sm, int col, int q, bool live, int e, int e0, int limit,
                                              const PredictorArgs& a) {
  constexpr int D = O::D, Q = O::Q, NP_S = O::NP_S, NS = O::NQ_S;
  constexpr int LD = E * Q + 1;
  // ---- corrector volume term (AmrDG.tpp:696-709): M U + sum_d c_d Sk_corr[d] F_d,
  // one time slice of points at a time (the slice's H, then its fluxes
  // accumulated into the time integral of F_d at the spatial points)
  {
    double* fbar = sm + NS * LD;
    final_volume_flux<O, E, 0>(hw, sm, fbar, col, LD, gm1,
                               live ? a.Tr + (size_t)e * 2 * D * tr_tile<O>() : nullptr, q);
    double R[NP_S], v[NP_S];
#pragma unroll
    for (int n = 0; n < NP_S; ++n) R[n] = O::mdiag(n) * u[n];
    O::template vol_term_sp<0>(ColIn{fbar + col, LD}, RegOut{v});
#pragma unroll
    for (int n = 0; n < NP_S; ++n) R[n] = fma(c[0], v[n], R[n]);
    O::template vol_term_sp<1>(ColIn{fbar + NS * LD + col, LD}, RegOut{v});
#pragma unroll
    for (int n = 0; n < NP_S; ++n) R[n] = fma(c[1], v[n], R[n]);
    if constexpr (D == 3) {
      O::template vol_term_sp<2>(ColIn{fbar + 2 * NS * LD + col, LD}, RegOut{v});
#pragma unroll
      for (int n = 0; n < NP_S; ++n) R[n] = fma(c[2], v[n], R[n]);
    }
    if (live) {
      double* dst = a.Rvol + ((size_t)e * Q + q) * NP_S;
#pragma unroll
      for (int n = 0; n < NP_S; ++n) dst[n] = R[n];
    }
  }
  __syncthreads();

  // ---- face traces of H (AmrDG.tpp:437-493) and face physics (AmrDG.h:1207-1251),
  // the two faces of one direction at a time
  face_traces<O, E, 0>(hw, sm, col, LD, a, e0, limit);
  face_traces<O, E, 1>(hw, sm, col, LD, a, e0, limit);
  if constexpr (D == 3) face_traces<O, E, 2>(hw, sm, col, LD, a, e0, limit);
}

// MODE 0: plain FP64 Picard (the reference's initial guess, P sweeps);
// MODE 1 / 2: seeded, `sweeps` sweeps from the learned seed in FP64 / FP32,
// the first one judging the seed by its residual;
// MODE 3: the FP64 Picard of MODE 0 with the final stage and split trace
// tiles of MODE 2 (the fallback elements of a MODE 2 step).
// Resident blocks per SM that MODE 2 asks for: 16 warps (at most 128
// registers a thread); its sliced sweeps leave the shared memory for them.
template <int E, int Q, int MODE>
constexpr int predictor_min_blocks() {
  constexpr int warps = (E * Q + 31) / 32;
  return MODE == 2 && 16 / warps > 0 ? 16 / warps : 1;
}

// One group of E elements (positions chunk E .. chunk E + E - 1 of the
// element range or list, limit = its length).
template <class O, int E, int MODE>
__device__ __forceinline__ void predictor_chunk(const PredictorArgs& a, double* sm, int chunk, int limit) {
  constexpr int D = O::D, Q = O::Q, NP_S = O::NP_S, NP_ST = O::NP_ST;
  constexpr int NQ = O::NQ_ST, NI = O::NQ_INIT;
  constexpr int NCOL = E * Q;
  constexpr int LD = NCOL + 1;  // odd stride: conflict-free point-major access

  const int col = threadIdx.x;
  const int el = col / Q;
  const int q = col % Q;
  const int e0 = chunk * E;
  int e_raw = e0 + el;
  const bool live = e_raw < limit;
  if (a.elem_list) e_raw = a.elem_list[live ? e_raw : limit - 1];
  const int e = live || a.elem_list ? e_raw : limit - 1;
  const int lev = a.elem_level ? a.elem_level[e] : 0;
  double c[D];
#pragma unroll
  for (int d = 0; d < D; ++d) c[d] = a.dt[kScalDtDx + 3 * lev + d];
  const double gm1 = a.gamma - 1.0;

  double u[NP_S];
  const double* src = a.Uw + ((size_t)e * Q + q) * NP_S;
#pragma unroll
  for (int n = 0; n < NP_S; ++n) u[n] = src[n];
  if (a.ubar_old && live) a.ubar_old[(size_t)e * Q + q] = u[0];

  double wu[NP_ST];
  O::wu(RegIn{u}, RegOut{wu});
  double hw[NP_ST];
  float dlt[NP_ST];  // MODES 2, 3: H_w - W U in FP32
  float uf[NP_S];    // MODES 2, 3: U_w in FP32

  if constexpr (MODE == 0 || MODE == 3) {
    // ---- sweep 1: the reference's initial guess H_w = [U_w, 0, ...]
    // (AmrDG.tpp:520-533) does not depend on x_0; evaluate on the (x_1.., t) grid.
    O::vol_eval_init(RegIn{u}, ColOut{sm + col, LD});
    __syncthreads();
    flux_stage<O, E, NI>(sm, LD, gm1);
    __syncthreads();
  #pragma unroll
    for (int n = 0; n < NP_ST; ++n) hw[n] = wu[n];
    {  // (A_0 F = 0 here: the initial guess, and so its flux, does not depend on x_0)
      double y[NP_ST];
      if constexpr (!O::proj_init_zero(0)) {
        O::template proj_init<0>(ColIn{sm + col, LD}, RegOut{y});
  #pragma unroll
        for (int n = 0; n < NP_ST; ++n) hw[n] = fma(-c[0], y[n], hw[n]);
      }
      if constexpr (!O::proj_init_zero(1)) {
        O::template proj_init<1>(ColIn{sm + NI * LD + col, LD}, RegOut{y});
  #pragma unroll
        for (int n = 0; n < NP_ST; ++n) hw[n] = fma(-c[1], y[n], hw[n]);
      }
      if constexpr (D == 3 && !O::proj_init_zero(2)) {
        O::template proj_init<2>(ColIn{sm + 2 * NI * LD + col, LD}, RegOut{y});
  #pragma unroll
        for (int n = 0; n < NP_ST; ++n) hw[n] = fma(-c[2], y[n], hw[n]);
      }
    }
    __syncthreads();

    // ---- remaining Picard sweeps (AmrDG.h:1103-1119)
    for (int s = 1; s < a.sweeps; ++s) {
      O::vol_eval(RegIn{hw}, ColOut{sm + col, LD});
      __syncthreads();
      flux_stage<O, E, NQ>(sm, LD, gm1);
      __syncthreads();
  #pragma unroll
      for (int n = 0; n < NP_ST; ++n) hw[n] = wu[n];
      double y[NP_ST];
      O::template proj<0>(ColIn{sm + col, LD}, RegOut{y});
  #pragma unroll
      for (int n = 0; n < NP_ST; ++n) hw[n] = fma(-c[0], y[n], hw[n]);
      O::template proj<1>(ColIn{sm + NQ * LD + col, LD}, RegOut{y});
  #pragma unroll
      for (int n = 0; n < NP_ST; ++n) hw[n] = fma(-c[1], y[n], hw[n]);
      if constexpr (D == 3) {
        O::template proj<2>(ColIn{sm + 2 * NQ * LD + col, LD}, RegOut{y});
  #pragma unroll
        for (int n = 0; n < NP_ST; ++n) hw[n] = fma(-c[2], y[n], hw[n]);
      }
      __syncthreads();
    }
  } else {
    // ---- learned seed: H_w from the network, then `sweeps` sweeps; the
    // first sweep's change judges the seed (residual relative to the
    // element's largest cell mean), failures go to the fallback list.
    const size_t hoff = ((size_t)e * Q + q) * NP_ST;
    double res = 0.0;
    if constexpr (MODE == 1) {
      const double* hs = a.Hseed + hoff;
#pragma unroll
      for (int n = 0; n < NP_ST; ++n) hw[n] = hs[n];
      for (int s = 0; s < a.sweeps; ++s) {
        double nw[NP_ST];
        picard_sweep<O, E, double>(hw, wu, c, sm, col, gm1, nw);
        if (s == 0)
#pragma unroll
          for (int n = 0; n < NP_ST; ++n) res = fmax(res, fabs(nw[n] - hw[n]));
#pragma unroll
        for (int n = 0; n < NP_ST; ++n) hw[n] = nw[n];
      }
    } else {
      // FP32 sweeps on a float copy; the final H_w = W U + dlt
      float hf[NP_ST], wf[NP_ST], cf[D];
      if (a.Hseed_f) {
#pragma unroll
        for (int n = 0; n < NP_ST; ++n) hf[n] = a.Hseed_f[hoff + n];
      } else {
#pragma unroll
        for (int n = 0; n < NP_ST; ++n) hf[n] = (float)a.Hseed[hoff + n];
      }
#pragma unroll
      for (int n = 0; n < NP_S; ++n) uf[n] = (float)u[n];
      O::template wu<float>(RegInT<float>{uf}, RegOutT<float>{wf});
#pragma unroll
      for (int d = 0; d < D; ++d) cf[d] = (float)c[d];
      float resf = 0.0f;
      for (int s = 0; s < a.sweeps; ++s) {
        picard_sweep_f32<O, E>(hf, cf, reinterpret_cast<float*>(sm), col, (float)gm1, dlt);
#pragma unroll
        for (int n = 0; n < NP_ST; ++n) {
          const float nf = wf[n] + dlt[n];
          if (s == 0) resf = fmaxf(resf, fabsf(nf - hf[n]));
          hf[n] = nf;
        }
      }
      res = (double)resf;
      if (a.sweeps == 0)  // the seed itself (a diagnostic setting): its change from W U in FP32
#pragma unroll
        for (int n = 0; n < NP_ST; ++n) dlt[n] = hf[n] - wf[n];
    }
    // per-element reduction over its Q columns through shared memory
    double* red = sm;
    red[col] = res;
    red[NCOL + col] = fabs(u[0]);
    __syncthreads();
    if (q == 0 && live) {
      double r = 0.0, scale = 0.0;
      for (int k = 0; k < Q; ++k) {
        r = fmax(r, red[el * Q + k]);
        scale = fmax(scale, red[NCOL + el * Q + k]);
      }
      if (!(r <= a.seed_tol * scale)) {  // NaN fails too
        const int slot = atomicAdd(a.fb_count, 1);
        a.fb_list[slot] = e;
      }
    }
    __syncthreads();
  }

  if (a.Hw_out && live) {
    double* dst = a.Hw_out + ((size_t)e * Q + q) * NP_ST;
#pragma unroll
    for (int n = 0; n < NP_ST; ++n) dst[n] = MODE == 2 ? wu[n] + (double)dlt[n] : hw[n];
  }
  if constexpr (MODE == 2 || MODE == 3) {
    if constexpr (MODE == 3) {
#pragma unroll
      for (int n = 0; n < NP_ST; ++n) dlt[n] = (float)(hw[n] - wu[n]);
#pragma unroll
      for (int n = 0; n < NP_S; ++n) uf[n] = (float)u[n];
    }
    split_epilogue<O, E>(u, uf, dlt, c, gm1, sm, col, q, live, e, e0, limit, a);
  } else {
    fp64_epilogue<O, E>(hw, u, c, gm1, sm, col, q, live, e, e0, limit, a);
  }
}

// The kernels: one element group per block over the element range
// (k_predictor), or a short grid striding over the groups of an element
// list whose length is known only on the device (k_predictor_list, the
// fallback pass).  Every phase of a group ends with a barrier, so the next
// group may reuse the shared memory.
template <class O, int E, int MODE = 0>
__global__ void __launch_bounds__(E * O::Q, (predictor_min_blocks<E, O::Q, MODE>()))
    k_predictor(PredictorArgs a) {
  extern __shared__ double sm[];
  predictor_chunk<O, E, MODE>(a, sm, blockIdx.x, a.n_elem);
}

template <class O, int E, int MODE>
__global__ void __launch_bounds__(E * O::Q) k_predictor_list(PredictorArgs a) {
  extern __shared__ double sm[];
  const int limit = *a.list_count;
  if (a.count_total && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(a.count_total, (unsigned long long)limit);
#pragma unroll 1
  for (int chunk = blockIdx.x; chunk * E < limit; chunk += gridDim.x) predictor_chunk<O, E, MODE>(a, sm, chunk, limit);
}

// N consecutive doubles to registers (and back): 16-byte accesses when every
// run of the array starts on a 16-byte boundary (even run length).
template <int N>
__device__ __forceinline__ void load_run(const double* __restrict__ p, double* v) {
  if constexpr (N % 2 == 0) {
    const double2* p2 = reinterpret_cast<const double2*>(p);
#pragma unroll
    for (int i = 0; i < N / 2; ++i) {
      const double2 x = __ldg(p2 + i);
      v[2 * i] = x.x;
      v[2 * i + 1] = x.y;
    }
  } else {
#pragma unroll
    for (int i = 0; i < N; ++i) v[i] = __ldg(p + i);
  }
}
template <int N>
__device__ __forceinline__ void store_run(double* p, const double* v) {
  if constexpr (N % 2 == 0) {
    double2* p2 = reinterpret_cast<double2*>(p);
#pragma unroll
    for (int i = 0; i < N / 2; ++i) p2[i] = make_double2(v[2 * i], v[2 * i + 1]);
  } else {
#pragma unroll
    for (int i = 0; i < N; ++i) p[i] = v[i];
  }
}

// Local Lax-Friedrichs flux at every face point (AmrDG_NumericalFlux.tpp:4-41).
// Face f separates left element face_left[f] (its high face in d) and right
// element face_right[f] (its low face).
struct FaceArgs {
  const double* Tr;
  const int* face_left;
  const int* face_right;
  int face_off[4];  // faces of direction d: [face_off[d], face_off[d+1])
  double* Fnum;
  // optional: only the faces face_list[0 .. n_list) (those whose flux an
  // update reads); nullptr: every face
  const int* face_list;
  long long n_list;
};

// Faces per block of k_numflux: one thread per (face, point), about 256.
template <class O>
constexpr int numflux_faces_per_block() {
  return 256 / O::NQ_BD > 0 ? 256 / O::NQ_BD : 1;
}

// Numerical flux of FB faces per block, as the tangential moments of the LLF
// flux (AmrDG_NumericalFlux.tpp:4-41) over each face, the only part of the
// flux the corrector's boundary operators and the coarse-fine corrections
// read (Mkbd, P_flux_fc).
//   Phase 1, thread (face, point): fL + fR - C (uR - uL), twice the flux.
//   Phase 2, thread (face, variable, spatial point x): the time integral at x
//   with the weights w_t / 2.
//   Phase 3, thread (face, variable): the tangential moments (face_mom_sp).
template <class O>
__global__ void k_numflux(FaceArgs a) {
  constexpr int D = O::D, Q = O::Q, N = O::N, NB = O::NQ_BD, NSB = NB / N, NF = 2 * D, NM = O::NM;
  constexpr int TT = tr_tile<O>(), FB = numflux_faces_per_block<O>(), NT = FB * NB;
  constexpr int LDH = NB + 1, LDG = NSB + 1;  // padded column strides
  __shared__ double h[FB * Q * LDH];
  __shared__ double g[FB * Q * LDG];
  const int64_t npos = a.face_list ? a.n_list : a.face_off[D];
  const int64_t fbase = (int64_t)blockIdx.x * FB;
  const int nfb = (int)(npos - fbase < FB ? npos - fbase : FB);
  {
    const int lf = threadIdx.x / NB, m = threadIdx.x % NB;  // m = t NSB + x
    if (lf < nfb) {
      const int64_t f = a.face_list ? a.face_list[fbase + lf] : fbase + lf;
      int d = 0;
#pragma unroll
      for (int k = 1; k < D; ++k)
        if (f >= a.face_off[k]) d = k;
      const int L = a.face_left[f], R = a.face_right[f];
      const double* tl = a.Tr + ((size_t)L * NF + 2 * d + 1) * TT + m;
      const double* tr = a.Tr + ((size_t)R * NF + 2 * d + 0) * TT + m;
      const double C = fmax(fabs(tl[2 * Q * NB]), fabs(tr[2 * Q * NB]));
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        const double uL = tl[q * NB], uR = tr[q * NB];
        const double fL = tl[(Q + q) * NB], fR = tr[(Q + q) * NB];
        h[(lf * Q + q) * LDH + m] = fma(-C, uR - uL, fL + fR);  // twice the LLF flux
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nfb * Q * NSB; i += NT) {
    const int x = i % NSB, c = i / NSB;  // c = face * Q + q
    const double* hc = h + c * LDH + x;
    double sum = (0.5 * O::weight(0)) * hc[0];
#pragma unroll
    for (int t = 1; t < N; ++t) sum = fma(0.5 * O::weight(t), hc[t * NSB], sum);
    g[c * LDG + x] = sum;
  }
  __syncthreads();
  for (int c = threadIdx.x; c < nfb * Q; c += NT) {
    double mom[NM];
    O::face_mom_sp(ColIn{g + c * LDG, 1}, RegOut{mom});
    const int64_t f = a.face_list ? a.face_list[fbase + c / Q] : fbase + c / Q;
    store_run<NM>(a.Fnum + ((size_t)f * Q + c % Q) * NM, mom);
  }
}

// k_numflux on split trace tiles (the seeded FP32 path).  With u = U + du and
// f = F + df on each side (U, F time-independent, FP64), twice the LLF flux
// integrated over time with the weights w_t / 2 is
//   (sum_t w_t / 2) (F_L + F_R) + A - S (U_R - U_L),
//   A = sum_t (w_t / 2) (df_L + df_R - C_t (du_R - du_L)),  S = sum_t (w_t / 2) C_t,
// so the time-dependent part (A, S) runs in FP32 and FP64 is spent once per
// spatial face point.
//   Phase 0, thread (face): the face's two tile addresses into shared memory.
//   Phase 1, thread (face, point): C_t and the FP32 terms of A; the same
//     thread loads the FP64 values of its phase-2 items beside them.
//   Phase 2, thread (face, variable, x): A, S and the FP64 sum.
//   Phase 3, thread (face, variable): the tangential moments (face_mom_sp).
template <class O>
__global__ void k_numflux_split(FaceArgs a) {
  constexpr int D = O::D, Q = O::Q, N = O::N, NB = O::NQ_BD, NSB = NB / N, NF = 2 * D, NM = O::NM;
  constexpr int TT = tr_tile<O>(), FB = numflux_faces_per_block<O>(), NT = FB * NB, FO = split_tr_float_off<O>();
  constexpr int LDH = NB + 1, LDG = NSB + 1, IT = (FB * Q * NSB + NT - 1) / NT;
  __shared__ float h[FB * Q * LDH];
  __shared__ float cs[FB * LDH];
  __shared__ double g[FB * Q * LDG];
  __shared__ const double* tile[FB][2];  // the left element's high-side and the right one's low-side tile
  __shared__ int64_t fid[FB];
  const int64_t npos = a.face_list ? a.n_list : a.face_off[D];
  const int64_t fbase = (int64_t)blockIdx.x * FB;
  const int nfb = (int)(npos - fbase < FB ? npos - fbase : FB);
  // the block's face indices once, so that every tile load below is issued
  // in one round
  if ((int)threadIdx.x < nfb) {
    const int lf = threadIdx.x;
    const int64_t f = a.face_list ? a.face_list[fbase + lf] : fbase + lf;
    int d = 0;
#pragma unroll
    for (int k = 1; k < D; ++k)
      if (f >= a.face_off[k]) d = k;
    fid[lf] = f;
    tile[lf][0] = a.Tr + ((size_t)a.face_left[f] * NF + 2 * d + 1) * TT;
    tile[lf][1] = a.Tr + ((size_t)a.face_right[f] * NF + 2 * d + 0) * TT;
  }
  __syncthreads();
  // the FP64 U and F_n(U) values of this thread's (face, variable, point)
  // items, loaded together with the FP32 changes of phase 1
  double fsum[IT], jump[IT];
#pragma unroll
  for (int k = 0; k < IT; ++k) {
    const int i = threadIdx.x + k * NT;
    fsum[k] = jump[k] = 0.0;
    if (i < nfb * Q * NSB) {
      const int x = i % NSB, c = i / NSB, lf = c / Q, q = c % Q;
      const double* tl = tile[lf][0] + q * NSB + x;
      const double* tr = tile[lf][1] + q * NSB + x;
      fsum[k] = tl[Q * NSB] + tr[Q * NSB];
      jump[k] = tr[0] - tl[0];
    }
  }
  {
    const int lf = threadIdx.x / NB, m = threadIdx.x % NB;  // m = t NSB + x
    if (lf < nfb) {
      const float* tl = reinterpret_cast<const float*>(tile[lf][0]) + FO + m;
      const float* tr = reinterpret_cast<const float*>(tile[lf][1]) + FO + m;
      const float C = fmaxf(fabsf(tl[2 * Q * NB]), fabsf(tr[2 * Q * NB]));
      cs[lf * LDH + m] = C;
#pragma unroll
      for (int q = 0; q < Q; ++q)
        h[(lf * Q + q) * LDH + m] = fmaf(-C, tr[q * NB] - tl[q * NB], tl[(Q + q) * NB] + tr[(Q + q) * NB]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < IT; ++k) {
    const int i = threadIdx.x + k * NT;
    if (i < nfb * Q * NSB) {
      const int x = i % NSB, c = i / NSB;  // c = face * Q + q
      const float* hc = h + c * LDH + x;
      const float* cc = cs + (c / Q) * LDH + x;
      float A = (0.5f * O::weight_f(0)) * hc[0], S = (0.5f * O::weight_f(0)) * cc[0];
#pragma unroll
      for (int t = 1; t < N; ++t) {
        A = fmaf(0.5f * O::weight_f(t), hc[t * NSB], A);
        S = fmaf(0.5f * O::weight_f(t), cc[t * NSB], S);
      }
      g[c * LDG + x] = fma(-(double)S, jump[k], fma(0.5 * O::WEIGHT_SUM, fsum[k], (double)A));
    }
  }
  __syncthreads();
  for (int c = threadIdx.x; c < nfb * Q; c += NT) {
    double mom[NM];
    O::face_mom_sp(ColIn{g + c * LDG, 1}, RegOut{mom});
    store_run<NM>(a.Fnum + ((size_t)fid[c / Q] * Q + c % Q) * NM, mom);
  }
}

// Runtime child / face index dispatch to the compile-time generated
// coarse-fine operators.
template <class O, class In, class Out>
__device__ __forceinline__ void pcf_rt(int l, const In& in, Out out) {
  switch (l) {
    case 0: O::template pcf<0>(in, out); break;
    case 1: O::template pcf<1>(in, out); break;
    case 2: O::template pcf<2>(in, out); break;
    case 3: O::template pcf<3>(in, out); break;
    default:
      if constexpr (O::D == 3) {
        switch (l) {
          case 4: O::template pcf<4>(in, out); break;
          case 5: O::template pcf<5>(in, out); break;
          case 6: O::template pcf<6>(in, out); break;
          default: O::template pcf<7>(in, out); break;
        }
      }
  }
}

template <class O, int DD, int S, class In, class Out>
__device__ __forceinline__ void pflux_mom_k(int k, const In& in, Out out) {
  if constexpr (O::D == 2) {
    if (k == 0) O::template pflux_mom<DD, S, 0>(in, out);
    else O::template pflux_mom<DD, S, 1>(in, out);
  } else {
    switch (k) {
      case 0: O::template pflux_mom<DD, S, 0>(in, out); break;
      case 1: O::template pflux_mom<DD, S, 1>(in, out); break;
      case 2: O::template pflux_mom<DD, S, 2>(in, out); break;
      default: O::template pflux_mom<DD, S, 3>(in, out); break;
    }
  }
}

// Corrector update of the valid elements (AmrDG.tpp:711-738):
// U_w = (Rvol - sum_d (Dt/dx_d) (Mkbdp[d] Fnum_hi - Mkbdm[d] Fnum_lo)) / M.
struct CorrectorArgs {
  double* Uw;
  const double* Rvol;
  const double* Fnum;
  const int* elem_face;  // [elem][2D]: face index of (d, side)
  int n_valid;
  // optional: the elements the non-record threads update (elem_list[0 ..
  // n_list), the valid elements whose state no average down replaces and
  // that have no reflux record); nullptr: every valid element
  const int* elem_list;
  int n_list;
  const int8_t* elem_level;
  LevelGeom geom;
  const double* dt;
  // coarse-fine flux corrections applied after the update (nullptr: none):
  // record of element e = rec_of_elem[e] (-1: none), element of record r =
  // rec_elem[r], its face entries rec_off[r] .. rec_off[r+1].  Elements with a
  // record are updated by the first nrec * Q threads, so the warps that run
  // the correction run nothing else and, having the longest chains, start first.
  int nrec;
  const int* rec_elem;
  const int* rec_of_elem;
  const int* rec_off;
  const int* ent_face;
  const int8_t* ent_dside;
  const int* ent_fine;
};

// Coarse-fine flux correction of one coarse element (FluxRegister CrseAdd /
// FineAdd / Reflux + L2ProjInterp::reflux, AmrDG.h:1138-1161,
// AmrDG_Interpolater.tpp:7-72):
//   corr = sum_faces sgn * (J_c Mkbd Fnum_c - sum_k J_f P_flux[k] Fnum_f[k]),
//   U_c += (2^D / vol_c) Minv corr,  sgn = +1 on the coarse cell's high face.
template <class O>
__device__ __forceinline__ void reflux_add(const CorrectorArgs& a, int r, int lc, int q, double* u) {
  constexpr int D = O::D, Q = O::Q, NP_S = O::NP_S, NM = O::NM, NFC = 1 << (D - 1);
  const double dt = a.dt[0];
  double corr[NP_S];
#pragma unroll
  for (int n = 0; n < NP_S; ++n) corr[n] = 0.0;
  for (int x = a.rec_off[r]; x < a.rec_off[r + 1]; ++x) {
    const int ds = a.ent_dside[x];
    const int d = ds >> 1, side = ds & 1;
    double area_c = 1.0, area_f = 1.0;
    for (int k = 0; k < D; ++k)
      if (k != d) {
        area_c *= a.geom.dx[lc][k];
        area_f *= a.geom.dx[lc + 1][k];
      }
    const double Jc = (dt / 2.0) * (area_c / (double)NFC);
    const double Jf = (dt / 2.0) * (area_f / (double)NFC);
    double fc[NP_S], ff[NP_S], tmp[NP_S], mc[NM];
    load_run<NM>(a.Fnum + ((size_t)a.ent_face[x] * Q + q) * NM, mc);
#define ADG_FC(DD, SS) O::template bd_mom<DD, SS>(RegIn{mc}, RegOut{fc})
    if (d == 0) { if (side) ADG_FC(0, 1); else ADG_FC(0, 0); }
    else if (d == 1) { if (side) ADG_FC(1, 1); else ADG_FC(1, 0); }
    else if constexpr (D == 3) { if (side) ADG_FC(2, 1); else ADG_FC(2, 0); }
#undef ADG_FC
#pragma unroll
    for (int n = 0; n < NP_S; ++n) ff[n] = 0.0;
    for (int k = 0; k < NFC; ++k) {
      double mf[NM];
      load_run<NM>(a.Fnum + ((size_t)a.ent_fine[(size_t)x * NFC + k] * Q + q) * NM, mf);
#define ADG_FF(DD, SS) pflux_mom_k<O, DD, SS>(k, RegIn{mf}, RegOut{tmp})
      if (d == 0) { if (side) ADG_FF(0, 1); else ADG_FF(0, 0); }
      else if (d == 1) { if (side) ADG_FF(1, 1); else ADG_FF(1, 0); }
      else if constexpr (D == 3) { if (side) ADG_FF(2, 1); else ADG_FF(2, 0); }
#undef ADG_FF
#pragma unroll
      for (int n = 0; n < NP_S; ++n) ff[n] += tmp[n];
    }
    const double sgn = side ? 1.0 : -1.0;
#pragma unroll
    for (int n = 0; n < NP_S; ++n) corr[n] += sgn * (Jc * fc[n] - Jf * ff[n]);
  }
  double vol = 1.0;
  for (int k = 0; k < D; ++k) vol *= a.geom.dx[lc][k];
  const double inv_jac = (double)(1 << D) / vol;
#pragma unroll
  for (int n = 0; n < NP_S; ++n) u[n] += inv_jac * (O::minv(n) * corr[n]);
}

template <class O>
__global__ void k_corrector(CorrectorArgs a) {
  constexpr int D = O::D, Q = O::Q, NP_S = O::NP_S, NM = O::NM, NF = 2 * D;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  // record threads first: their chains are the longest, so they start first
  const int64_t nrq = a.rec_of_elem ? (int64_t)a.nrec * Q : 0;
  int e, q, r = -1;
  if (t < nrq) {
    r = (int)(t / Q);
    q = (int)(t % Q);
    e = a.rec_elem[r];
  } else {
    const int64_t t2 = t - nrq;
    if (t2 >= (int64_t)(a.elem_list ? a.n_list : a.n_valid) * Q) return;
    e = a.elem_list ? a.elem_list[t2 / Q] : (int)(t2 / Q);
    q = (int)(t2 % Q);
    // updated by a record thread (a list holds no such element)
    if (nrq && !a.elem_list && a.rec_of_elem[e] >= 0) return;
  }
  const int lev = a.elem_level ? a.elem_level[e] : 0;
  double R[NP_S];
  load_run<NP_S>(a.Rvol + ((size_t)e * Q + q) * NP_S, R);
  // every load first (Rvol, then the moments of the 2D faces), then the update
  double mf[NF][NM];
  const int* ef = a.elem_face + (size_t)e * NF;
#pragma unroll
  for (int k = 0; k < NF; ++k) load_run<NM>(a.Fnum + ((size_t)ef[k] * Q + q) * NM, mf[k]);
  double bp[NP_S], bm[NP_S];
#define ADG_BD(DD)                                                                      \
  {                                                                                     \
    const double cd = a.dt[kScalDtDx + 3 * lev + DD];                                  \
    O::template bd_mom<DD, 1>(RegIn{mf[2 * DD + 1]}, RegOut{bp});                       \
    O::template bd_mom<DD, 0>(RegIn{mf[2 * DD + 0]}, RegOut{bm});                       \
    _Pragma("unroll") for (int n = 0; n < NP_S; ++n) R[n] = fma(-cd, bp[n] - bm[n], R[n]); \
  }
  ADG_BD(0)
  ADG_BD(1)
  if constexpr (D == 3) ADG_BD(2)
#undef ADG_BD
#pragma unroll
  for (int n = 0; n < NP_S; ++n) R[n] = R[n] * O::minv(n);
  if (r >= 0) reflux_add<O>(a, r, lev, q, R);
  store_run<NP_S>(a.Uw + ((size_t)e * Q + q) * NP_S, R);
}

// ---------------------------------------------------------------------------
// TVB limiter (Limiter_w / Limiter_linear_tvb, AmrDG.h:1657-1855; minmod /
// minmodB, AmrDG_Limiter.tpp:40-85; eigenvectors, Compressible_Euler.cpp:
// 138-276).  IEEE operations in the reference's order without contraction,
// so the troubled-cell decisions are the ones the CPU oracle makes.
// ---------------------------------------------------------------------------
#define ADG_M(a, b) __dmul_rn((a), (b))
#define ADG_A(a, b) __dadd_rn((a), (b))
#define ADG_S(a, b) __dsub_rn((a), (b))
#define ADG_V(a, b) __ddiv_rn((a), (b))

template <int D>
__device__ __forceinline__ void euler_eigenvectors(int d, const double* u, double gamma, double R[D + 2][D + 2],
                                                   double L[D + 2][D + 2]) {
  // Soundspeed / Pressure (Compressible_Euler.h:562-604)
  double prs = 0.0;
#pragma unroll
  for (int k = 0; k < D; ++k) prs = ADG_A(prs, ADG_V(ADG_M(u[k + 1], u[k + 1]), u[0]));
  prs = ADG_M(prs, -0.5);
  prs = ADG_A(prs, u[D + 1]);
  prs = ADG_M(prs, ADG_S(gamma, 1.0));
  prs = (prs < kPdeLimit) ? kPdeLimit : prs;
  const double rho = (u[0] < kPdeLimit) ? kPdeLimit : u[0];
  const double c = __dsqrt_rn(ADG_M(gamma, ADG_V(prs, rho)));
  const double g = ADG_S(gamma, 1.0);
  const double u1 = ADG_V(u[1], u[0]), u2 = ADG_V(u[2], u[0]);
  const double u3 = (D == 3) ? ADG_V(u[D == 3 ? 3 : 2], u[0]) : 0.0;
  double ek = ADG_A(ADG_M(u1, u1), ADG_M(u2, u2));
  if (D == 3) ek = ADG_A(ek, ADG_M(u3, u3));
  ek = ADG_M(0.5, ek);
  const double c2 = ADG_M(c, c);
  const double h = ADG_A(ADG_V(c2, g), ek);
  const double beta = ADG_V(1.0, ADG_M(2.0, c2));
  const double phi = ADG_M(g, ek);
  const double mb = -beta, b2 = ADG_M(2.0, beta), mb2 = ADG_M(-2.0, beta);
  const double bg = ADG_M(beta, g), mbg = ADG_M(mb, g), b2g = ADG_M(b2, g), mb2g = ADG_M(mb2, g);
  const double row1[5] = {ADG_S(1.0, ADG_M(b2, phi)), ADG_M(b2g, u1), ADG_M(b2g, u2), ADG_M(b2g, u3), mb2g};
  const double uv[3] = {u1, u2, u3};
  const double ud = uv[d];
  // rows 0 and 2: the acoustic waves of direction d; in row 2 the reference
  // writes the first other component as -beta*(gamma*u) and a second one
  // (3D) as -beta*gamma*u, which round differently
  const int kp = (d == 0) ? 1 : 0;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const double uk = uv[k];
    L[0][k + 1] = (k == d) ? ADG_M(mb, ADG_A(ADG_M(g, uk), c)) : ADG_M(mbg, uk);
    L[2][k + 1] = (k == d) ? ADG_M(mb, ADG_S(ADG_M(g, uk), c)) : (k == kp ? ADG_M(mb, ADG_M(g, uk)) : ADG_M(mbg, uk));
  }
  L[0][0] = ADG_M(beta, ADG_A(phi, ADG_M(c, ud)));
  L[2][0] = ADG_M(beta, ADG_S(phi, ADG_M(c, ud)));
  L[0][D + 1] = bg;
  L[2][D + 1] = bg;
#pragma unroll
  for (int k = 0; k < D + 1; ++k) L[1][k] = row1[k];
  L[1][D + 1] = mb2g;
  // rows 3 (and 4): the shear waves, and R, as listed per direction
#pragma unroll
  for (int i = 0; i < D + 2; ++i)
#pragma unroll
    for (int j = 0; j < D + 2; ++j) R[i][j] = 0.0;
  R[0][0] = 1.0; R[0][1] = 1.0; R[0][2] = 1.0;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const double uk = uv[k];
    R[k + 1][0] = (k == d) ? ADG_S(uk, c) : uk;
    R[k + 1][1] = uk;
    R[k + 1][2] = (k == d) ? ADG_A(uk, c) : uk;
  }
  R[D + 1][0] = ADG_S(h, ADG_M(c, ud));
  R[D + 1][1] = ek;
  R[D + 1][2] = ADG_A(h, ADG_M(c, ud));
  if (D == 2) {
    const double s0[2][4] = {{u2, 0.0, -1.0, 0.0}, {-u1, 1.0, 0.0, 0.0}};
#pragma unroll
    for (int j = 0; j < 4; ++j) L[3][j] = s0[d][j];
    if (d == 0) { R[2][3] = -1.0; R[3][3] = -u2; }
    else        { R[1][3] = 1.0;  R[3][3] = u1; }
  } else {
    double l3[5] = {0, 0, 0, 0, 0}, l4[5] = {0, 0, 0, 0, 0};
    if (d == 0) {
      l3[0] = u2; l3[2] = -1.0; l4[0] = -u3; l4[3] = 1.0;
      R[2][3] = -1.0; R[3][4] = 1.0; R[4][3] = -u2; R[4][4] = u3;
    } else if (d == 1) {
      l3[0] = -u1; l3[1] = 1.0; l4[0] = u3; l4[3] = -1.0;
      R[1][3] = 1.0; R[3][4] = -1.0; R[4][3] = u1; R[4][4] = -u3;
    } else {
      l3[0] = u1; l3[1] = -1.0; l4[0] = -u2; l4[2] = 1.0;
      R[1][3] = -1.0; R[2][4] = 1.0; R[4][3] = -u1; R[4][4] = u2;
    }
#pragma unroll
    for (int j = 0; j < D + 2; ++j) {
      L[3][j] = l3[j];
      L[D == 3 ? 4 : 3][j] = l4[j];
    }
  }
}

__device__ __forceinline__ double minmod3(double a1, double a2, double a3) {
  const bool same = (signbit(a1) == signbit(a2)) && (signbit(a2) == signbit(a3));
  if (!same) return 0.0;
  const double m = fmin(fabs(a1), fmin(fabs(a2), fabs(a3)));
  return signbit(a1) ? -m : m;
}

struct LimiterArgs {
  double* Uw;
  const double* ubar_old;  // [elem][q] cell means at the start of the step
  const int* elem_face;
  const int* face_left;
  const int* face_right;
  int e0, n;               // the finest level's valid elements
  int periodic[3];
  double gamma;
  double thr;              // AMR_TVB_C[l] * M * h^2
  unsigned long long* count;
};

template <class O>
__global__ void k_limit_tvb(LimiterArgs a) {
  constexpr int D = O::D, Q = O::Q, NP_S = O::NP_S;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int e = a.e0 + i;
  double ub[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) ub[q] = a.Uw[((size_t)e * Q + q) * NP_S];
  double res[D][Q];
  bool troubled = false;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const int s = O::lin_mode(d);
    const int lo = a.face_left[a.elem_face[(size_t)e * 2 * D + 2 * d]];
    const int hi = a.face_right[a.elem_face[(size_t)e * 2 * D + 2 * d + 1]];
    // a physical-boundary neighbour is the element itself: the reference's
    // ghost there holds the copy made at the start of the step
    const bool bnd = !a.periodic[d];
    double um[Q], up[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      um[q] = (bnd && lo == e) ? a.ubar_old[(size_t)e * Q + q] : a.Uw[((size_t)lo * Q + q) * NP_S];
      up[q] = (bnd && hi == e) ? a.ubar_old[(size_t)e * Q + q] : a.Uw[((size_t)hi * Q + q) * NP_S];
    }
    double R[Q][Q], L[Q][Q], v[Q];
    euler_eigenvectors<D>(d, ub, a.gamma, R, L);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      double Dm = 0.0, Dp = 0.0, Du = 0.0;
#pragma unroll
      for (int k = 0; k < Q; ++k) {
        const double hl = ADG_M(0.5, L[q][k]);
        Dm = ADG_A(Dm, ADG_M(hl, ADG_S(ub[k], um[k])));
        Dp = ADG_A(Dp, ADG_M(hl, ADG_S(up[k], ub[k])));
        Du = ADG_A(Du, ADG_M(L[q][k], a.Uw[((size_t)e * Q + k) * NP_S + s]));
      }
      v[q] = (fabs(Du) <= a.thr) ? Du : minmod3(Du, Dm, Dp);
      troubled = troubled || (v[q] != Du);
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      double sum = 0.0;
#pragma unroll
      for (int k = 0; k < Q; ++k) sum = ADG_A(sum, ADG_M(R[q][k], v[k]));
      res[d][q] = sum;
    }
  }
  if (!troubled) return;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    double* uq = a.Uw + ((size_t)e * Q + q) * NP_S;
#pragma unroll
    for (int n = 1; n < NP_S; ++n) uq[n] = 0.0;
#pragma unroll
    for (int d = 0; d < D; ++d) uq[O::lin_mode(d)] = res[d][q];
  }
  if (a.count) atomicAdd(a.count, 1ull);
}
#undef ADG_M
#undef ADG_A
#undef ADG_S
#undef ADG_V

// Time step (AmrDG.h:1253-1357): dt_cell = CFL * dx_avg / lambda(U at spatial
// quadrature point 0), Dt = c_dt min over cells.  Reduced as the maximum of
// the rate lambda / dx_avg (a product with the host's reciprocal instead of
// a division per cell; Dt = c_dt * CFL / max): block maximum, then a global
// atomic maximum on the IEEE bit pattern (non-negative doubles order like
// their bits).
struct DtArgs {
  const double* Uw;
  int n_valid;
  const int8_t* elem_level;
  double inv_dx_avg[kMaxLevels];
  double gamma;
  unsigned long long* rate_bits;  // 0 between reductions
  unsigned int* status;
  // finalisation by the last block: Dt, t += old Dt when advance_time,
  // Dt/dx of every level (products with inv_geom); rate_bits and done reset
  double* scal;
  unsigned int* done;
  double c_dt;
  int advance_time;
  int D;
  LevelGeom inv_geom;  // 1 / dx per level and direction
};

// Elements per block of k_dt_reduce (block of 128 threads).
constexpr int kDtElems = 32;

template <class O>
__global__ void k_dt_reduce(DtArgs a) {
  constexpr int D = O::D, Q = O::Q, NP_S = O::NP_S, EL = Q * NP_S, EB = kDtElems;
  static_assert(EL % 2 == 0, "element blocks must be whole 16-byte units");
  // the block's states (contiguous) staged with coalesced 16-byte loads
  __shared__ __align__(16) double st[EB * EL];
  __shared__ double upt[EB][Q + 1];
  const int e0 = blockIdx.x * EB;
  const int ne = a.n_valid - e0 < EB ? a.n_valid - e0 : EB;
  // the level of this thread's element, loaded beside the states
  const int lev = a.elem_level && (int)threadIdx.x < ne ? a.elem_level[e0 + threadIdx.x] : 0;
  for (int i = threadIdx.x; i < ne * (EL / 2); i += blockDim.x)
    reinterpret_cast<double2*>(st)[i] = __ldg(reinterpret_cast<const double2*>(a.Uw + (size_t)e0 * EL) + i);
  __syncthreads();
  for (int i = threadIdx.x; i < ne * Q; i += blockDim.x) {
    double v;
    O::u_pt0(RegIn{st + (i / Q) * EL + (i % Q) * NP_S}, RegOut{&v});
    upt[i / Q][i % Q] = v;
  }
  __syncthreads();
  double rate = 0.0;
  unsigned int st_bits = 0;
  if ((int)threadIdx.x < ne) {
    double u[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) u[q] = upt[threadIdx.x][q];
    rate = euler_cfl_lambda<D>(u, a.gamma) * a.inv_dx_avg[lev];
    if (!(u[0] > 0.0)) st_bits |= kStatusNonPositiveDensity;
    if (!(rate == rate)) {
      st_bits |= kStatusNaN;
      rate = 0.0;
    }
  }
  // warp then block maximum
  for (int o = 16; o > 0; o >>= 1) rate = fmax(rate, __shfl_xor_sync(0xffffffffu, rate, o));
  __shared__ double wmax[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) wmax[wid] = rate;
  __syncthreads();
  if (wid == 0) {
    double v = (lane < (int)(blockDim.x + 31) / 32) ? wmax[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (lane == 0) atomicMax(a.rate_bits, (unsigned long long)__double_as_longlong(v));
  }
  if (st_bits) atomicOr(a.status, st_bits);
  // the last block to finish publishes Dt (threadFenceReduction pattern)
  __shared__ bool last;
  __shared__ double dt_s;
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(a.done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last) {  // block-uniform
    if (threadIdx.x == 0) {
      __threadfence();
      const unsigned long long bits = atomicAdd(a.rate_bits, 0ull);
      const double dt = a.c_dt * (O::CFL / __longlong_as_double((long long)bits));
      if (a.advance_time) a.scal[1] += a.scal[0];
      a.scal[0] = dt;
      dt_s = dt;
      *a.rate_bits = 0ull;
      *a.done = 0u;
    }
    __syncthreads();
    const int i = threadIdx.x;
    if (i < 3 * kMaxLevels) a.scal[kScalDtDx + i] = i % 3 < a.D ? dt_s * a.inv_geom.dx[i / 3][i % 3] : 0.0;
  }
}

// Lp norm of the difference to the analytic initial condition over the leaf
// cells (LpNorm_DG_AMR, AmrDG.h:1399-1578): per valid, uncovered element the
// sum over the tensor quadrature points of |u_ex - u_h|^p w_m, times
// vol / 2^D; covered elements give 0.  The host adds the cells in order.
struct LpArgs {
  const double* Uw;
  const int* elem_cell;
  const int8_t* elem_level;   // nullptr: all level 0
  const int8_t* covered;      // [valid elem] 1: covered by a finer level
  int n_valid, q, p, M;       // M quadrature points
  const double* phi;          // [Np_s][M] basis values
  const double* wq;           // [M] weights
  const double* qp;           // [M][3] reference coordinates
  LevelGeom geom;
  double prob_lo[3];
  double gamma;
  ICParams icp;
  double* cell_out;           // [valid elem]
};

template <class O>
__global__ void k_lp_norm(LpArgs a) {
  constexpr int D = O::D, Q = O::Q, NP_S = O::NP_S;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.n_valid) return;
  if (a.covered && a.covered[e]) {
    a.cell_out[e] = 0.0;
    return;
  }
  const int lev = a.elem_level ? a.elem_level[e] : 0;
  double uw[NP_S];
#pragma unroll
  for (int n = 0; n < NP_S; ++n) uw[n] = a.Uw[((size_t)e * Q + a.q) * NP_S + n];
  double vol = 1.0;
  for (int d = 0; d < D; ++d) vol *= a.geom.dx[lev][d];
  double cell = 0.0;
  for (int m = 0; m < a.M; ++m) {
    double uh = 0.0;
#pragma unroll
    for (int n = 0; n < NP_S; ++n) uh += uw[n] * a.phi[(size_t)n * a.M + m];
    double x[3] = {0.0, 0.0, 0.0};
    for (int d = 0; d < D; ++d) {
      const double dx = a.geom.dx[lev][d];
      const double xc = a.prob_lo[d] + (a.elem_cell[3 * e + d] + 0.5) * dx;
      x[d] = (dx / 2.0) * a.qp[3 * m + d] + xc;
    }
    double v[5];
    pde_ic(x, D, a.gamma, a.icp, 0, 0, v);
    const double err = fabs(v[a.q] - uh);
    cell += (a.p == 1 ? err : err * err) * a.wq[m];
  }
  a.cell_out[e] = cell * (vol / (double)(1 << D));
}

// L2 projection of the initial condition at the spatial GL points
// (AmrDG.h:782-836); one thread per element.
struct ICArgs {
  double* Uw;
  const int* elem_cell;  // [elem][3] cell index within its level
  const int8_t* elem_level;
  int n_elem;
  LevelGeom geom;
  double prob_lo[3];
  int n_cell0[3];  // level-0 cells (noise hash index)
  double gamma;
  ICParams icp;
};

template <class O>
__global__ void k_init_ic(ICArgs a) {
  constexpr int D = O::D, Q = O::Q, NP_S = O::NP_S, NS = O::NQ_S, N = O::N;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.n_elem) return;
  const int lev = a.elem_level ? a.elem_level[e] : 0;
  int ijk[3] = {a.elem_cell[3 * e], a.elem_cell[3 * e + 1], a.elem_cell[3 * e + 2]};
  // level-0 linear index of the covering level-0 cell, periodically wrapped
  uint64_t lin = 0, mul = 1;
  for (int d = 0; d < D; ++d) {
    int w = ijk[d] >> lev;
    w = ((w % a.n_cell0[d]) + a.n_cell0[d]) % a.n_cell0[d];
    lin += (uint64_t)w * mul;
    mul *= (uint64_t)a.n_cell0[d];
  }
  double vals[Q][NS];
  for (int m = 0; m < NS; ++m) {
    double x[3] = {0, 0, 0};
    int rem = m;
    int idx[3] = {0, 0, 0};
    for (int d = D - 1; d >= 0; --d) {
      idx[d] = rem % N;
      rem /= N;
    }
    for (int d = 0; d < D; ++d) {
      const double dx = a.geom.dx[lev][d];
      const double xc = a.prob_lo[d] + (ijk[d] + 0.5) * dx;
      x[d] = (dx / 2.0) * O::node(idx[d]) + xc;
    }
    double v[5];
    pde_ic(x, D, a.gamma, a.icp, lin, m, v);
    for (int q = 0; q < Q; ++q) vals[q][m] = v[q];
  }
  for (int q = 0; q < Q; ++q) {
    double s[NP_S];
    O::ic_proj(RegIn{vals[q]}, RegOut{s});
    double* dst = a.Uw + ((size_t)e * Q + q) * NP_S;
    for (int n = 0; n < NP_S; ++n) dst[n] = s[n] * O::minv(n);
  }
}


// ===========================================================================
// AMR transfer kernels (L2ProjInterp, Source/NumericalMethod/AmrDG/AmrDG_Interpolater.tpp)
// One thread per (element, variable) column; runtime child / face indices are
// dispatched to the compile-time generated operators.
// ===========================================================================
// average_down / amr_gather (AmrDG_Interpolater.tpp:283-342, 366-398):
// u_c = 2^-D Minv sum_l P_fc[l] u_f[l].  rec: coarse, fine_0 .. fine_{2^D-1}.
// Block (32, 2^D): warp l projects child l of 32 (record, variable) pairs, so
// every warp runs one operator; warp 0 sums the children in order.
// Records per block of k_average_down.
template <class O>
constexpr int ad_records_per_block() {
  return O::D == 2 ? 8 : 4;
}

// Block (RB Q, 2^D): records r0 .. r0+RB-1; the children's states are staged
// in shared memory with coalesced 16-byte loads (each element's Q Np_s
// doubles are contiguous), thread (r, q, child) projects one child, row 0
// sums and scales, and the coarse states leave through shared memory again.
template <class O>
__global__ void k_average_down(double* Uw, const int* rec, int nrec) {
  constexpr int D = O::D, Q = O::Q, NP_S = O::NP_S, NOV = 1 << D, RB = ad_records_per_block<O>();
  constexpr int EL = Q * NP_S, EL2 = EL / 2, NT = RB * Q * NOV;
  static_assert(EL % 2 == 0, "element blocks must be whole 16-byte units");
  __shared__ __align__(16) double fine[NOV * RB * EL];
  __shared__ double part[NOV][NP_S][RB * Q + 1];
  const int tid = threadIdx.x + threadIdx.y * blockDim.x;
  const int r0 = blockIdx.x * RB;
  const int nr = nrec - r0 < RB ? nrec - r0 : RB;
  for (int i = tid; i < NOV * nr * EL2; i += NT) {
    const int L = i / (nr * EL2), rem = i % (nr * EL2);
    const int r = rem / EL2, off = rem % EL2;
    const int e = rec[(size_t)(r0 + r) * (NOV + 1) + 1 + L];
    reinterpret_cast<double2*>(fine)[(L * RB + r) * EL2 + off] =
        __ldg(reinterpret_cast<const double2*>(Uw + (size_t)e * EL) + off);
  }
  __syncthreads();
  const int x = threadIdx.x, L = threadIdx.y;
  const int r = x / Q, q = x % Q;
  if (r < nr) {
    const double* uf = fine + (L * RB + r) * EL + q * NP_S;
    double tmp[NP_S];
    switch (L) {
      case 0: O::template pfc<0>(RegIn{uf}, RegOut{tmp}); break;
      case 1: O::template pfc<1>(RegIn{uf}, RegOut{tmp}); break;
      case 2: O::template pfc<2>(RegIn{uf}, RegOut{tmp}); break;
      case 3: O::template pfc<3>(RegIn{uf}, RegOut{tmp}); break;
      default:
        if constexpr (D == 3) {
          switch (L) {
            case 4: O::template pfc<4>(RegIn{uf}, RegOut{tmp}); break;
            case 5: O::template pfc<5>(RegIn{uf}, RegOut{tmp}); break;
            case 6: O::template pfc<6>(RegIn{uf}, RegOut{tmp}); break;
            default: O::template pfc<7>(RegIn{uf}, RegOut{tmp}); break;
          }
        }
    }
#pragma unroll
    for (int n = 0; n < NP_S; ++n) part[L][n][x] = tmp[n];
  }
  __syncthreads();
  double* out = fine;  // the children are consumed: [RB][EL] coarse states
  // mode n of every (record, variable) summed by row n mod 2^D: the FP64 work
  // of the sums spread over all warps (and so over the SM's four schedulers)
  if (r < nr) {
#pragma unroll
    for (int n0 = 0; n0 < NP_S; n0 += NOV) {
      const int n = n0 + L;
      if (n < NP_S) {
        double sum = 0.0;
#pragma unroll
        for (int l = 0; l < NOV; ++l) sum = __dadd_rn(sum, part[l][n][x]);  // as k_interp_gather
        out[r * EL + q * NP_S + n] = (1.0 / NOV) * (O::minv(n) * sum);
      }
    }
  }
  __syncthreads();
  for (int i = tid; i < nr * EL2; i += NT) {
    const int rr = i / EL2, off = i % EL2;
    reinterpret_cast<double2*>(Uw + (size_t)rec[(size_t)(r0 + rr) * (NOV + 1)] * EL)[off] =
        reinterpret_cast<const double2*>(out)[rr * EL2 + off];
  }
}

// L2ProjInterp on caller batches (AmrDG_Interpolater.tpp:344-398): thread
// per (cell, variable).  Scatter: fine[i] = Minv P_cf[child[i]] coarse[i];
// gather: coarse[i] = 2^-D Minv sum_l P_fc[l] fine[i][l], children summed in
// order as k_average_down does.  Layouts [n][Q][Np_s] and [n][2^D][Q][Np_s].
template <class O>
__global__ void k_interp_scatter(const double* coarse, const int8_t* child, long long n, double* fine) {
  constexpr int Q = O::Q, NP_S = O::NP_S;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * Q) return;
  const long long i = t / Q;  // cell; variable t % Q
  double out[NP_S];
  const int l = child[i];
#pragma unroll
  for (int k = 0; k < NP_S; ++k) out[k] = __longlong_as_double(0x7ff8000000000000LL);  // NaN: child out of range
  if (l >= 0 && l < (1 << O::D)) pcf_rt<O>(l, RegIn{coarse + (size_t)t * NP_S}, RegOut{out});
#pragma unroll
  for (int k = 0; k < NP_S; ++k) fine[(size_t)t * NP_S + k] = out[k];
}

template <class O>
__global__ void k_interp_gather(const double* fine, long long n, double* coarse) {
  constexpr int D = O::D, Q = O::Q, NP_S = O::NP_S, NOV = 1 << D;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * Q) return;
  const long long i = t / Q;
  const int q = (int)(t % Q);
  double part[NOV][NP_S];
#pragma unroll
  for (int l = 0; l < NOV; ++l) {
    const double* uf = fine + (((size_t)i * NOV + l) * Q + q) * NP_S;
    switch (l) {
      case 0: O::template pfc<0>(RegIn{uf}, RegOut{part[l]}); break;
      case 1: O::template pfc<1>(RegIn{uf}, RegOut{part[l]}); break;
      case 2: O::template pfc<2>(RegIn{uf}, RegOut{part[l]}); break;
      case 3: O::template pfc<3>(RegIn{uf}, RegOut{part[l]}); break;
      default:
        if constexpr (D == 3) {
          switch (l) {
            case 4: O::template pfc<4>(RegIn{uf}, RegOut{part[l]}); break;
            case 5: O::template pfc<5>(RegIn{uf}, RegOut{part[l]}); break;
            case 6: O::template pfc<6>(RegIn{uf}, RegOut{part[l]}); break;
            default: O::template pfc<7>(RegIn{uf}, RegOut{part[l]}); break;
          }
        }
    }
  }
#pragma unroll
  for (int k = 0; k < NP_S; ++k) {
    double sum = 0.0;
#pragma unroll
    for (int l = 0; l < NOV; ++l) sum = __dadd_rn(sum, part[l][k]);  // never fused with a child's last product
    coarse[(size_t)t * NP_S + k] = (1.0 / NOV) * (O::minv(k) * sum);
  }
}

// Coarse -> fine projection (amr_scatter, AmrDG_Interpolater.tpp:344-364)
// into ghost elements (FillPatchTwoLevels) or, with src_old, the regrid
// remap of a level (valid data of the old layout where it existed).
struct ScatterArgs {
  double* Uw;            // destination array (and coarse source)
  const double* Uw_old;  // optional: old layout's state
  const int* dst;        // [n] destination element
  const int* parent;     // [n] coarse parent element in Uw
  const int8_t* child;   // [n] child index
  const int* src_old;    // optional [n]: element in Uw_old, -1 = project
  int n;
};

template <class O>
__global__ void k_scatter(ScatterArgs a) {
  constexpr int Q = O::Q, NP_S = O::NP_S;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)a.n * Q) return;
  const int i = (int)(t / Q), q = (int)(t % Q);
  double* dst = a.Uw + ((size_t)a.dst[i] * Q + q) * NP_S;
  if (a.src_old && a.src_old[i] >= 0) {
    const double* s = a.Uw_old + ((size_t)a.src_old[i] * Q + q) * NP_S;
#pragma unroll
    for (int n = 0; n < NP_S; ++n) dst[n] = s[n];
    return;
  }
  double v[NP_S];
  pcf_rt<O>(a.child[i], RegIn{a.Uw + ((size_t)a.parent[i] * Q + q) * NP_S}, RegOut{v});
#pragma unroll
  for (int n = 0; n < NP_S; ++n) dst[n] = v[n];
}

// Refinement indicator on cell means (mode 0), tag when above threshold:
// kind 0 normalised density gradient max_d |rho(i+e_d)-rho(i-e_d)|/(2 rho(i)),
// kind 1 the same on pressure.  IEEE operations in a fixed order (no FMA
// contraction) so the indicator is the one the CPU oracle evaluates.
struct TagArgs {
  const double* Uw;
  const int* elem_face;
  const int* face_left;
  const int* face_right;
  int e0, n;
  int kind;               // ADG_TAG_* of include/adg.h
  double threshold, gamma;
  uint8_t* tags;
  // the reference's criteria (kinds 2 and 3)
  const int* elem_cell;
  const int8_t* elem_level;
  const double* scal;     // device scalar block: [1] = t
  LevelGeom geom;
  double prob_lo[2], extent[2];
  double xc, yc, u_inf, v_inf;
  int advect;
  double r_max[kMaxLevels];    // amr_c[l]^2
  double tvb_thr[kMaxLevels];  // AMR_TVB_C[l] * amr_c[l] * h_l^2
};

template <class O>
__device__ __forceinline__ double cell_pressure(const double* Uw, int e, double gamma) {
  constexpr int D = O::D, Q = O::Q, NP_S = O::NP_S;
  const double rho = Uw[((size_t)e * Q + 0) * NP_S];
  double ke = 0.0;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const double m = Uw[((size_t)e * Q + d + 1) * NP_S];
    ke = __dadd_rn(ke, __ddiv_rn(__dmul_rn(m, m), rho));
  }
  const double E = Uw[((size_t)e * Q + D + 1) * NP_S];
  return __dmul_rn(gamma - 1.0, __dsub_rn(E, __dmul_rn(0.5, ke)));
}

// The reference's isentropic-vortex criterion (Compressible_Euler.h:615-644),
// IEEE operations in its order so that the host oracle tags the same cells.
__device__ __forceinline__ bool tag_vortex(const TagArgs& a, int e) {
  const int lev = a.elem_level[e];
  const double x = __dadd_rn(a.prob_lo[0], __dmul_rn((double)a.elem_cell[3 * e] + 0.5, a.geom.dx[lev][0]));
  const double y = __dadd_rn(a.prob_lo[1], __dmul_rn((double)a.elem_cell[3 * e + 1] + 0.5, a.geom.dx[lev][1]));
  double xc = a.xc, yc = a.yc;
  if (a.advect) {
    const double t = a.scal[1];
    xc = __dadd_rn(xc, __dmul_rn(a.u_inf, t));
    yc = __dadd_rn(yc, __dmul_rn(a.v_inf, t));
  }
  double dx = __dsub_rn(x, xc), dy = __dsub_rn(y, yc);
  const double hx = a.extent[0] / 2.0, hy = a.extent[1] / 2.0;
  if (dx > hx) dx = __dsub_rn(dx, a.extent[0]);
  if (dx < -hx) dx = __dadd_rn(dx, a.extent[0]);
  if (dy > hy) dy = __dsub_rn(dy, a.extent[1]);
  if (dy < -hy) dy = __dadd_rn(dy, a.extent[1]);
  const double r = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
  return r <= a.r_max[lev];
}

// The reference's Kelvin-Helmholtz criterion (Compressible_Euler.h:645-682):
// the cell is tagged as soon as one characteristic linear slope L_EV(u_mean)
// u_lin fails minmodB's TVB test (AmrDG_Limiter.tpp:40-61); the neighbour
// differences minmod would take do not change the flag, so they are not
// formed.  NaN slopes tag the cell, as in the reference.
template <class O>
__device__ __forceinline__ bool tag_kh_tvb(const TagArgs& a, int e) {
  constexpr int D = O::D, Q = O::Q, NP_S = O::NP_S;
  const double thr = a.tvb_thr[a.elem_level[e]];
  double ub[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) ub[q] = a.Uw[((size_t)e * Q + q) * NP_S];
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const int s = O::lin_mode(d);
    double R[Q][Q], L[Q][Q];
    euler_eigenvectors<D>(d, ub, a.gamma, R, L);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      double du = 0.0;
#pragma unroll
      for (int k = 0; k < Q; ++k) du = __dadd_rn(du, __dmul_rn(L[q][k], a.Uw[((size_t)e * Q + k) * NP_S + s]));
      if (!(fabs(du) <= thr)) return true;
    }
  }
  return false;
}

template <class O>
__global__ void k_tag(TagArgs a) {
  constexpr int D = O::D, Q = O::Q, NP_S = O::NP_S;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int e = a.e0 + i;
  if (a.kind == 2 || a.kind == 3) {
    a.tags[i] = (a.kind == 2 ? tag_vortex(a, e) : tag_kh_tvb<O>(a, e)) ? 1 : 0;
    return;
  }
  double ind = 0.0;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const int hi = a.face_right[a.elem_face[(size_t)e * 2 * D + 2 * d + 1]];
    const int lo = a.face_left[a.elem_face[(size_t)e * 2 * D + 2 * d]];
    double v;
    if (a.kind == 0) {
      const double rp = a.Uw[((size_t)hi * Q) * NP_S], rm = a.Uw[((size_t)lo * Q) * NP_S];
      const double rc = a.Uw[((size_t)e * Q) * NP_S];
      v = __ddiv_rn(fabs(__dsub_rn(rp, rm)), __dmul_rn(2.0, rc));
    } else {
      const double pp = cell_pressure<O>(a.Uw, hi, a.gamma), pm = cell_pressure<O>(a.Uw, lo, a.gamma);
      const double pc = cell_pressure<O>(a.Uw, e, a.gamma);
      v = __ddiv_rn(fabs(__dsub_rn(pp, pm)), __dmul_rn(2.0, pc));
    }
    ind = fmax(ind, v);
  }
  a.tags[i] = ind > a.threshold ? 1 : 0;
}

// ===========================================================================
// Learned predictor seed: features, training targets, seed assembly.
// Features of element e: U_w (Q * Np_s modal coefficients) and Dt/dx_0 of
// its level, standardised; targets: H_w - W U_w (the part of the predictor
// the time evolution adds), standardised.
// ===========================================================================
struct SeedFeatArgs {
  const double* Uw;
  const double* Hw;      // targets only
  int e0, n;             // elements e0 .. e0+n-1
  const int8_t* elem_level;
  LevelGeom geom;
  const double* dt;
  const float* x_mean;   // optional standardisation
  const float* x_istd;
  float* X;              // n x (Q*Np_s + 1)
  float* T;              // n x (Q*Np_st)
};

template <class O>
__global__ void k_seed_features(SeedFeatArgs a) {
  constexpr int Q = O::Q, NP_S = O::NP_S, NIN = Q * NP_S + 1;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)a.n * NIN) return;
  const int i = (int)(t / NIN), f = (int)(t % NIN);
  const int e = a.e0 + i;
  double v;
  if (f < Q * NP_S) {
    // the Euler flux is homogeneous of degree one in U: scale by the cell
    // mean density so the network sees density-free states
    v = a.Uw[(size_t)e * Q * NP_S + f] * (1.0 / a.Uw[(size_t)e * Q * NP_S]);
  } else {
    const int lev = a.elem_level ? a.elem_level[e] : 0;
    v = a.dt[kScalDtDx + 3 * lev];
  }
  float x = (float)v;
  if (a.x_mean) x = (x - a.x_mean[f]) * a.x_istd[f];
  a.X[t] = x;
}

template <class O>
__global__ void k_seed_targets(SeedFeatArgs a) {
  constexpr int Q = O::Q, NP_S = O::NP_S, NP_ST = O::NP_ST;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)a.n * Q) return;
  const int i = (int)(t / Q), q = (int)(t % Q);
  const int e = a.e0 + i;
  double wu[NP_ST];
  O::wu(RegIn{a.Uw + ((size_t)e * Q + q) * NP_S}, RegOut{wu});
  const double* h = a.Hw + ((size_t)e * Q + q) * NP_ST;
  float* out = a.T + (size_t)i * Q * NP_ST + q * NP_ST;
  // the predictor's change over the step, per unit density and Dt/dx
  const int lev = a.elem_level ? a.elem_level[e] : 0;
  const double scale = a.Uw[(size_t)e * Q * NP_S] * a.dt[kScalDtDx + 3 * lev];
#pragma unroll
  for (int n = 0; n < NP_ST; ++n) out[n] = (float)((h[n] - wu[n]) / scale);
}

// H_seed = W U + rho_mean * (Dt/dx) * (Y * y_std + y_mean)
template <class O>
__global__ void k_seed_assemble(const double* Uw, const float* Y, const float* y_mean, const float* y_std, int n,
                                const int8_t* elem_level, LevelGeom geom, const double* dt, double* Hseed) {
  constexpr int Q = O::Q, NP_S = O::NP_S, NP_ST = O::NP_ST;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n * Q) return;
  const int e = (int)(t / Q), q = (int)(t % Q);
  double wu[NP_ST];
  O::wu(RegIn{Uw + ((size_t)e * Q + q) * NP_S}, RegOut{wu});
  const int lev = elem_level ? elem_level[e] : 0;
  const double scale = Uw[(size_t)e * Q * NP_S] * dt[kScalDtDx + 3 * lev];
  const float* y = Y + (size_t)e * Q * NP_ST + q * NP_ST;
  double* h = Hseed + ((size_t)e * Q + q) * NP_ST;
#pragma unroll
  for (int k = 0; k < NP_ST; ++k) {
    const int f = q * NP_ST + k;
    h[k] = wu[k] + scale * (double)(y[k] * y_std[f] + y_mean[f]);
  }
}

}  // namespace adg

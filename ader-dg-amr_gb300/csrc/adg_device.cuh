// Device helpers of the ADER-DG element path: operand accessors for the
// generated operators and the compressible-Euler point physics.
#pragma once

#include <cfloat>
#include <cstdint>

namespace adg {

// Operand accessors: the generated operators are written against these, so
// the same code reads registers (stride 1, compile-time indices) or a shared
// memory column (runtime stride).
template <class T>
struct RegInT {
  const T* p;
  __device__ __forceinline__ T operator()(int i) const { return p[i]; }
};
template <class T>
struct RegOutT {
  T* p;
  __device__ __forceinline__ T& operator()(int i) const { return p[i]; }
};
template <class T>
struct ColInT {
  const T* p;
  int s;
  __device__ __forceinline__ T operator()(int i) const { return p[i * s]; }
};
template <class T>
struct ColOutT {
  T* p;
  int s;
  __device__ __forceinline__ T& operator()(int i) const { return p[i * s]; }
};
using RegIn = RegInT<double>;
using RegOut = RegOutT<double>;
using ColIn = ColInT<double>;
using ColOut = ColOutT<double>;

// Pressure floor of the reference model: 10 * machine epsilon
// (Source/Model/CompressibleEuler/Compressible_Euler.cpp:50-55).
constexpr double kPdeLimit = 10.0 * DBL_EPSILON;

// Status bits reported through adg_status().
constexpr uint32_t kStatusNaN = 1u;
constexpr uint32_t kStatusNonPositiveDensity = 2u;
constexpr uint32_t kStatusPressureFloor = 4u;

// Floor that keeps NaN (std::max(_prs, limit) semantics, Compressible_Euler.h:586).
__device__ __forceinline__ double floor_limit(double p) { return (p < kPdeLimit) ? kPdeLimit : p; }

// Physical flux of the compressible Euler equations in every direction at one
// point (Compressible_Euler.h:370-487; pressure Compressible_Euler.h:562-589).
// u: Q = D+2 conserved variables; F[d*Q + q].
template <int D, class T = double>
__device__ __forceinline__ void euler_flux_all(const T* u, T gm1, T* F) {
  constexpr int Q = D + 2;
  const T r = T(1) / u[0];
  T v[D];
#pragma unroll
  for (int d = 0; d < D; ++d) v[d] = u[d + 1] * r;
  T ke = u[1] * v[0];
#pragma unroll
  for (int d = 1; d < D; ++d) ke = fma(u[d + 1], v[d], ke);
  T p = gm1 * fma(T(-0.5), ke, u[D + 1]);
  p = (p < T(kPdeLimit)) ? T(kPdeLimit) : p;
  const T ep = u[D + 1] + p;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    F[d * Q + 0] = u[d + 1];
#pragma unroll
    for (int k = 0; k < D; ++k) {
      if (k < d)
        F[d * Q + k + 1] = F[k * Q + d + 1];  // m_d v_k = m_k v_d (symmetric)
      else if (k == d)
        F[d * Q + k + 1] = fma(u[d + 1], v[k], p);
      else
        F[d * Q + k + 1] = u[d + 1] * v[k];
    }
    F[d * Q + D + 1] = ep * v[d];
  }
}

// Normal flux in direction d and the LLF wave-speed bound
// max(|un-c|, |un|, |un+c|) = |un| + c (Compressible_Euler.h:489-518, 591-604).
template <int D>
__device__ __forceinline__ double euler_flux_normal(int d, const double* u, double gamma, double* F) {
  const double r = 1.0 / u[0];
  double v[D];
#pragma unroll
  for (int k = 0; k < D; ++k) v[k] = u[k + 1] * r;
  double ke = u[1] * v[0];
#pragma unroll
  for (int k = 1; k < D; ++k) ke = fma(u[k + 1], v[k], ke);
  const double p = floor_limit((gamma - 1.0) * fma(-0.5, ke, u[D + 1]));
  // 1 / max(rho, floor) from the reciprocal already at hand
  const double rinv_c = (u[0] < kPdeLimit) ? 1.0 / kPdeLimit : r;
  double vd = v[0], md = u[1];
#pragma unroll
  for (int k = 1; k < D; ++k)
    if (k == d) {
      vd = v[k];
      md = u[k + 1];
    }
  F[0] = md;
#pragma unroll
  for (int k = 0; k < D; ++k) F[k + 1] = (k == d) ? fma(md, v[k], p) : md * v[k];
  F[D + 1] = (u[D + 1] + p) * vd;
  const double c = sqrt(gamma * (p * rinv_c));
  return fabs(vd) + c;
}

// Change of the physical flux F(u + du) - F(u) between a state u and a nearby
// state u + du, in FP32, written with the algebraic differences of its terms
// (v' - v = (dm - v drho) / rho', m'.v' - m.v = m.dv + dm.v', ...) so that no
// two rounded fluxes are subtracted: the rounding error is relative to the
// change, not to the flux.  The pressure floor of euler_flux_all applies to
// both states (the change of the floored pressure).
struct DeltaState {
  float v1[3], dv[3];  // velocity of u + du, its change
  float p, dp;         // floored pressure of u, change of the floored pressure
};

template <int D>
__device__ __forceinline__ DeltaState euler_delta_state(const float* u, const float* du, float gm1) {
  DeltaState s;
  const float r = __frcp_rn(u[0]);
  const float r1 = __frcp_rn(u[0] + du[0]);
  float ke = 0.0f, dke = 0.0f;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const float v = u[d + 1] * r;
    s.dv[d] = fmaf(-v, du[0], du[d + 1]) * r1;
    s.v1[d] = v + s.dv[d];
    ke = fmaf(u[d + 1], v, ke);
    dke = fmaf(du[d + 1], s.v1[d], fmaf(u[d + 1], s.dv[d], dke));
  }
  const float L = (float)kPdeLimit;
  const float p = gm1 * fmaf(-0.5f, ke, u[D + 1]);
  const float dp = gm1 * fmaf(-0.5f, dke, du[D + 1]);
  const float p1 = p + dp;
  if (p < L || p1 < L) {
    const float pf = p < L ? L : p;
    const float pf1 = p1 < L ? L : p1;
    s.p = pf;
    s.dp = pf1 - pf;
  } else {
    s.p = p;
    s.dp = dp;
  }
  return s;
}

// Change of the flux in every direction; dF[d*Q + q].
template <int D>
__device__ __forceinline__ void euler_dflux_all(const float* u, const float* du, float gm1, float* dF) {
  constexpr int Q = D + 2;
  const DeltaState s = euler_delta_state<D>(u, du, gm1);
  const float ep = u[D + 1] + s.p, dep = du[D + 1] + s.dp;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    dF[d * Q] = du[d + 1];
#pragma unroll
    for (int k = 0; k < D; ++k) {
      const float t = fmaf(du[k + 1], s.v1[d], u[k + 1] * s.dv[d]);
      dF[d * Q + k + 1] = k == d ? t + s.dp : t;
    }
    dF[d * Q + D + 1] = fmaf(dep, s.v1[d], ep * s.dv[d]);
  }
}

// Change of the normal flux in direction d, and the LLF wave-speed bound of
// the state u + du (as euler_flux_normal, in FP32).
template <int D>
__device__ __forceinline__ float euler_dflux_normal(int d, const float* u, const float* du, float gm1, float gamma,
                                                    float* dF) {
  const DeltaState s = euler_delta_state<D>(u, du, gm1);
  float v1d = s.v1[0], dvd = s.dv[0];
#pragma unroll
  for (int k = 1; k < D; ++k)
    if (k == d) {
      v1d = s.v1[k];
      dvd = s.dv[k];
    }
  float dmd = du[1];
#pragma unroll
  for (int k = 1; k < D; ++k)
    if (k == d) dmd = du[k + 1];
  dF[0] = dmd;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const float t = fmaf(du[k + 1], v1d, u[k + 1] * dvd);
    dF[k + 1] = k == d ? t + s.dp : t;
  }
  dF[D + 1] = fmaf(du[D + 1] + s.dp, v1d, (u[D + 1] + s.p) * dvd);
  const float rho1 = u[0] + du[0];
  const float L = (float)kPdeLimit;
  const float rinv_c = rho1 < L ? 1.0f / L : __frcp_rn(rho1);
  const float c = sqrtf(gamma * ((s.p + s.dp) * rinv_c));
  return fabsf(v1d) + c;
}

// CFL speed max_d(|u_d/rho| + c) at one point (Compressible_Euler.cpp:57-70).
template <int D>
__device__ __forceinline__ double euler_cfl_lambda(const double* u, double gamma) {
  const double r = 1.0 / u[0];
  double ke = 0.0;
#pragma unroll
  for (int d = 0; d < D; ++d) ke += (u[d + 1] * u[d + 1]) * r;
  const double p = floor_limit((gamma - 1.0) * (u[D + 1] - 0.5 * ke));
  const double rinv_c = (u[0] < kPdeLimit) ? 1.0 / kPdeLimit : r;
  const double c = sqrt(gamma * (p * rinv_c));
  double lam = fabs(u[1] * r) + c;
#pragma unroll
  for (int d = 1; d < D; ++d) lam = fmax(lam, fabs(u[d + 1] * r) + c);
  return lam;
}

// ---------------------------------------------------------------------------
// Initial conditions (Compressible_Euler.h:120-368) and the seeded noise hash.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ULL;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
  return x ^ (x >> 31);
}

__host__ __device__ __forceinline__ double hash_noise(uint64_t seed, uint64_t cell, uint64_t m) {
  uint64_t h = splitmix64(seed ^ splitmix64(cell * 0x100000001B3ULL + m));
  double u = (double)(h >> 11) * 0x1p-53;
  return 2.0 * u - 1.0;
}

struct ICParams {
  int ic;
  double u_inf, v_inf, beta, xc, yc;
  uint64_t seed;
  double noise_amp;
};

__device__ __forceinline__ void pde_ic(const double* x, int D, double gamma, const ICParams& p, uint64_t cell_l0,
                                       int m, double* out) {
  const double PI = 3.14159265358979323846;
  if (p.ic == 0) {  // isentropic vortex
    double dx = x[0] - p.xc, dy = x[1] - p.yc;
    double r = sqrt(dx * dx + dy * dy);
    double beta = p.beta;
    double rho = pow(1.0 - (((gamma - 1.0) * (beta * beta)) / (8.0 * gamma * (PI * PI))) * exp(1.0 - r * r),
                     (1.0 / (gamma - 1.0)));
    double prs = pow(rho, gamma);
    double du1 = -dy * (beta / (PI * 2.0)) * exp((1.0 - r * r) / 2.0);
    double du2 = dx * (beta / (PI * 2.0)) * exp((1.0 - r * r) / 2.0);
    double u1 = p.u_inf + du1, u2 = p.v_inf + du2;
    double e = (prs / (rho * (gamma - 1.0))) + 0.5 * (u1 * u1 + u2 * u2);
    out[0] = rho;
    out[1] = rho * u1;
    out[2] = rho * u2;
    out[3] = rho * e;
    return;
  }
  if (p.ic == 1 || p.ic == 2) {  // Kelvin-Helmholtz
    double y = x[1];
    bool in = (y > 0.25) && (y < 0.75);
    double rho = in ? 2.0 : 1.0;
    double prs = 2.5;
    double u1 = in ? 0.5 : -0.5;
    double u2;
    if (p.ic == 1) {
      u2 = 0.01 * sin(4.0 * PI * x[0]) + p.noise_amp * hash_noise(p.seed, cell_l0, (uint64_t)m);
    } else {
      double w0 = 0.2, sigma = 0.05 / sqrt(2.0);
      u2 = w0 * sin(4.0 * PI * x[0]) *
           (exp(-((y - 0.25) * (y - 0.25)) / (2.0 * sigma * sigma)) + exp(-((y - 0.75) * (y - 0.75)) / (2.0 * sigma * sigma)));
    }
    double rho_e = (prs / (gamma - 1.0)) + 0.5 * rho * (u1 * u1 + u2 * u2);
    out[0] = rho;
    out[1] = rho * u1;
    out[2] = rho * u2;
    out[3] = rho_e;
    if (D == 3) {  // KH is 2D; keep a consistent 3D state if asked for
      out[3] = 0.0;
      out[4] = rho_e;
    }
    return;
  }
  if (p.ic == 3) {  // spherical blast
    double a = x[0] - 0.5, b = x[1] - 0.5, c = (D == 3) ? x[2] - 0.5 : 0.0;
    double r = sqrt(a * a + b * b + c * c);
    double prs = (r < 0.1) ? 10.0 : 0.1;
    out[0] = 1.0;
    for (int d = 0; d < D; ++d) out[d + 1] = 0.0;
    out[D + 1] = prs / (gamma - 1.0);
    return;
  }
  // uniform free stream
  double v[3] = {p.u_inf, p.v_inf, 0.0};
  double ke = 0.0;
  out[0] = 1.0;
  for (int d = 0; d < D; ++d) {
    out[d + 1] = v[d];
    ke += v[d] * v[d];
  }
  out[D + 1] = 1.0 / (gamma - 1.0) + 0.5 * ke;
}

}  // namespace adg

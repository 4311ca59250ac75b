// CPU oracle (test infrastructure only; never linked into the product).
//
// Compressible Euler physics restated from the reference:
//   Pressure        Source/Model/CompressibleEuler/Compressible_Euler.h:562-589
//   Soundspeed      Source/Model/CompressibleEuler/Compressible_Euler.h:591-604
//   pde_flux        Source/Model/CompressibleEuler/Compressible_Euler.h:370-487
//   pde_dflux       Source/Model/CompressibleEuler/Compressible_Euler.h:489-518
//   pde_cfl_lambda  Source/Model/CompressibleEuler/Compressible_Euler.cpp:57-70
//   PDE_NUMERIC_LIMIT = 10*eps   Compressible_Euler.cpp:50-55
//   pde_EV_Rmatrix / Lmatrix     Compressible_Euler.cpp:138-276
//   pde_IC (vortex, KH)          Compressible_Euler.h:120-368
// The KH variant with sin(4 pi x) + seeded noise and the 3D blast IC are the
// synthetic workloads of this project; the reference has no 3D IC
// (Compressible_Euler.h:358-367).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <limits>

namespace oracle {

constexpr double kPdeNumericLimit = 10 * std::numeric_limits<double>::epsilon();

// u[0]=rho, u[1..D]=momentum, u[D+1]=total energy density
inline double pressure(const double* u, int D, double gamma) {
  double _prs = 0.0;
  for (int d = 0; d < D; ++d) _prs += ((u[d + 1] * u[d + 1]) / u[0]);
  _prs *= (-0.5);
  _prs += u[D + 1];
  _prs *= (gamma - 1.0);
  return std::max(_prs, kPdeNumericLimit);
}

inline double soundspeed(const double* u, int D, double gamma) {
  double prs = pressure(u, D, gamma);
  double rho = std::max(u[0], kPdeNumericLimit);
  return std::sqrt(gamma * (prs / rho));
}

// Physical flux component q in direction d (Compressible_Euler.h:370-487).
inline double pde_flux(int d, int q, const double* u, int D, double gamma) {
  double prs = pressure(u, D, gamma);
  double f = 0.0;
  if (D == 2) {
    if (d == 0) {
      if (q == 0) f = u[1];
      else if (q == 1) f = ((u[1] * u[1]) / u[0]) + prs;
      else if (q == 2) f = u[1] * u[2] / u[0];
      else if (q == 3) f = (u[3] + prs) * (u[1] / u[0]);
    } else {
      if (q == 0) f = u[2];
      else if (q == 1) f = u[2] * u[1] / u[0];
      else if (q == 2) f = ((u[2] * u[2]) / u[0]) + prs;
      else if (q == 3) f = (u[3] + prs) * (u[2] / u[0]);
    }
  } else {
    if (d == 0) {
      if (q == 0) f = u[1];
      else if (q == 1) f = ((u[1] * u[1]) / u[0]) + prs;
      else if (q == 2) f = u[1] * u[2] / u[0];
      else if (q == 3) f = u[1] * u[3] / u[0];
      else if (q == 4) f = (u[4] + prs) * (u[1] / u[0]);
    } else if (d == 1) {
      if (q == 0) f = u[2];
      else if (q == 1) f = u[2] * u[1] / u[0];
      else if (q == 2) f = ((u[2] * u[2]) / u[0]) + prs;
      else if (q == 3) f = u[2] * u[3] / u[0];
      else if (q == 4) f = (u[4] + prs) * (u[2] / u[0]);
    } else {
      if (q == 0) f = u[3];
      else if (q == 1) f = u[3] * u[1] / u[0];
      else if (q == 2) f = u[3] * u[2] / u[0];
      else if (q == 3) f = ((u[3] * u[3]) / u[0]) + prs;
      else if (q == 4) f = (u[4] + prs) * (u[3] / u[0]);
    }
  }
  return f;
}

// Max characteristic speed in direction d (Compressible_Euler.h:489-518).
inline double pde_dflux(int d, const double* u, int D, double gamma) {
  double c = soundspeed(u, D, gamma);
  double un = 0.0;
  for (int dd = 0; dd < D; ++dd) un += ((u[dd + 1] / u[0]) * (dd == d ? 1.0 : 0.0));
  return std::max({std::abs(un - c), std::abs(un), std::abs(un + c)});
}

// Compressible_Euler.cpp:57-70
inline double pde_cfl_lambda(int d, const double* u, int D, double gamma) {
  double c = soundspeed(u, D, gamma);
  return std::abs(u[d + 1] / u[0]) + c;
}

// ---------------------------------------------------------------------------
// Seeded noise: a counter-based hash of (seed, level-0 cell index, quadrature
// point index), so it is identical on every device and layout.
// ---------------------------------------------------------------------------
inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ULL;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
  return x ^ (x >> 31);
}

inline double hash_noise(uint64_t seed, uint64_t cell, uint64_t m) {
  uint64_t h = splitmix64(seed ^ splitmix64(cell * 0x100000001B3ULL + m));
  double u = (double)(h >> 11) * 0x1p-53;  // [0, 1)
  return 2.0 * u - 1.0;                    // [-1, 1)
}

enum ICCase : int {
  IC_VORTEX = 0,      // isentropic vortex, free stream (u_inf, v_inf)
  IC_KH_NOISE = 1,    // KH: sin(4 pi x) + seeded uniform noise (level 0 only)
  IC_KH_REF = 2,      // reference KH with Gaussian-localised v (Compressible_Euler.h:237-258)
  IC_BLAST3D = 3,     // spherical blast in [0,1]^3
  IC_CONST = 4,       // uniform free stream (for free-stream preservation tests)
};

struct ICParams {
  int ic = IC_VORTEX;
  double u_inf = 1.0, v_inf = 0.0;  // vortex free stream
  double beta = 5.0, xc = 5.0, yc = 5.0;
  uint64_t seed = 12345;
  double noise_amp = 1e-3;
};

// Point value of the IC at physical point x (Compressible_Euler.h:120-368).
// cell_l0 is the level-0 linear cell index used only by the noise hash.
inline double pde_IC(int q, const double* x, int D, double gamma, const ICParams& p,
                     uint64_t cell_l0, int m) {
  const double PI = M_PI;
  if (p.ic == IC_VORTEX) {
    double r = std::sqrt(((x[0] - p.xc) * (x[0] - p.xc) + (x[1] - p.yc) * (x[1] - p.yc)));
    double beta = p.beta;
    double rho = std::pow(1.0 - (((gamma - 1.0) * std::pow(beta, 2.0)) / (8.0 * gamma * std::pow(PI, 2))) *
                                    std::exp(1.0 - std::pow(r, 2.0)),
                          (1.0 / (gamma - 1.0)));
    double prs = std::pow(rho, gamma);
    double du1 = -(x[1] - p.yc) * (beta / (PI * 2.0)) * std::exp((1.0 - std::pow(r, 2.0)) / 2.0);
    double du2 = (x[0] - p.xc) * (beta / (PI * 2.0)) * std::exp((1.0 - std::pow(r, 2.0)) / 2.0);
    double u1 = p.u_inf + du1;
    double u2 = p.v_inf + du2;
    double e = (prs / (rho * (gamma - 1.0))) + 0.5 * (std::pow(u1, 2.0) + std::pow(u2, 2.0));
    if (q == 0) return rho;
    if (q == 1) return rho * u1;
    if (q == 2) return rho * u2;
    return rho * e;
  }
  if (p.ic == IC_KH_NOISE || p.ic == IC_KH_REF) {
    double y = x[1];
    double rho = ((y > 0.25) && (y < 0.75)) ? 2.0 : 1.0;
    double prs = 2.5;
    double u1 = ((y > 0.25) && (y < 0.75)) ? 0.5 : -0.5;
    double u2;
    if (p.ic == IC_KH_NOISE) {
      u2 = 0.01 * std::sin(4.0 * PI * x[0]) + p.noise_amp * hash_noise(p.seed, cell_l0, (uint64_t)m);
    } else {
      double w0 = 0.2;
      double sigma = 0.05 / std::sqrt(2.0);
      u2 = w0 * std::sin(4.0 * PI * x[0]) *
           (std::exp(-(std::pow(y - 0.25, 2.0)) / (2.0 * std::pow(sigma, 2.0))) +
            std::exp(-(std::pow(y - 0.75, 2.0)) / (2.0 * std::pow(sigma, 2))));
    }
    double rho_e = (prs / (gamma - 1.0)) + 0.5 * rho * (std::pow(u1, 2.0) + std::pow(u2, 2.0));
    if (q == 0) return rho;
    if (q == 1) return rho * u1;
    if (q == 2) return rho * u2;
    return rho_e;
  }
  if (p.ic == IC_BLAST3D) {
    double dx0 = x[0] - 0.5, dx1 = x[1] - 0.5, dx2 = (D == 3 ? x[2] - 0.5 : 0.0);
    double r = std::sqrt(dx0 * dx0 + dx1 * dx1 + dx2 * dx2);
    double prs = (r < 0.1) ? 10.0 : 0.1;
    if (q == 0) return 1.0;
    if (q == D + 1) return prs / (gamma - 1.0);
    return 0.0;
  }
  // IC_CONST
  {
    double rho = 1.0, prs = 1.0;
    double v[3] = {p.u_inf, p.v_inf, 0.0};
    if (q == 0) return rho;
    if (q == D + 1) {
      double ke = 0.0;
      for (int d = 0; d < D; ++d) ke += v[d] * v[d];
      return prs / (gamma - 1.0) + 0.5 * rho * ke;
    }
    return rho * v[q - 1];
  }
}

// Right / left eigenvectors of the flux Jacobian in direction d at state u
// (the cell means), R[q][q'] and L[q][q'] as the reference lists them
// (Compressible_Euler.cpp:138-276), same expressions in the same order.
inline void eigenvectors(int d, const double* u, int D, double gamma, double R[5][5], double L[5][5]) {
  const double c = soundspeed(u, D, gamma);
  const double g = gamma - 1.0;
  if (D == 2) {
    const double u1 = u[1] / u[0], u2 = u[2] / u[0];
    const double ek = 0.5 * (std::pow(u1, 2) + std::pow(u2, 2));
    const double h = (std::pow(c, 2) / (gamma - 1.0)) + ek;
    const double beta = 1.0 / (2.0 * std::pow(c, 2));
    const double phi = g * ek;
    if (d == 0) {
      const double r[4][4] = {{1.0, 1.0, 1.0, 0.0}, {u1 - c, u1, u1 + c, 0.0}, {u2, u2, u2, -1.0},
                              {h - c * u1, ek, h + c * u1, -u2}};
      const double l[4][4] = {{beta * (phi + c * u1), -beta * (g * u1 + c), -beta * g * u2, beta * g},
                              {1.0 - 2.0 * beta * phi, 2.0 * beta * g * u1, 2.0 * beta * g * u2, -2.0 * beta * g},
                              {beta * (phi - c * u1), -beta * (g * u1 - c), -beta * (g * u2), beta * g},
                              {u2, 0.0, -1.0, 0.0}};
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) R[i][j] = r[i][j], L[i][j] = l[i][j];
    } else {
      const double r[4][4] = {{1.0, 1.0, 1.0, 0.0}, {u1, u1, u1, 1.0}, {u2 - c, u2, u2 + c, 0.0},
                              {h - c * u2, ek, h + c * u2, u1}};
      const double l[4][4] = {{beta * (phi + c * u2), -beta * g * u1, -beta * (g * u2 + c), beta * g},
                              {1.0 - 2.0 * beta * phi, 2.0 * beta * g * u1, 2.0 * beta * g * u2, -2.0 * beta * g},
                              {beta * (phi - c * u2), -beta * (g * u1), -beta * (g * u2 - c), beta * g},
                              {-u1, 1.0, 0.0, 0.0}};
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) R[i][j] = r[i][j], L[i][j] = l[i][j];
    }
    return;
  }
  const double u1 = u[1] / u[0], u2 = u[2] / u[0], u3 = u[3] / u[0];
  const double ek = 0.5 * (std::pow(u1, 2) + std::pow(u2, 2) + std::pow(u3, 2));
  const double h = (std::pow(c, 2) / (gamma - 1.0)) + ek;
  const double beta = 1.0 / (2.0 * std::pow(c, 2));
  const double phi = g * ek;
  double r[5][5], l[5][5];
  if (d == 0) {
    const double rr[5][5] = {{1.0, 1.0, 1.0, 0.0, 0.0}, {u1 - c, u1, u1 + c, 0.0, 0.0}, {u2, u2, u2, -1.0, 0.0},
                             {u3, u3, u3, 0.0, 1.0}, {h - c * u1, ek, h + c * u1, -u2, u3}};
    const double ll[5][5] = {
        {beta * (phi + c * u1), -beta * (g * u1 + c), -beta * g * u2, -beta * g * u3, beta * g},
        {1.0 - 2.0 * beta * phi, 2.0 * beta * g * u1, 2.0 * beta * g * u2, 2.0 * beta * g * u3, -2.0 * beta * g},
        {beta * (phi - c * u1), -beta * (g * u1 - c), -beta * (g * u2), -beta * g * u3, beta * g},
        {u2, 0.0, -1.0, 0.0, 0.0},
        {-u3, 0.0, 0.0, 1.0, 0.0}};
    std::copy(&rr[0][0], &rr[0][0] + 25, &r[0][0]);
    std::copy(&ll[0][0], &ll[0][0] + 25, &l[0][0]);
  } else if (d == 1) {
    const double rr[5][5] = {{1.0, 1.0, 1.0, 0.0, 0.0}, {u1, u1, u1, 1.0, 0.0}, {u2 - c, u2, u2 + c, 0.0, 0.0},
                             {u3, u3, u3, 0.0, -1.0}, {h - c * u2, ek, h + c * u2, u1, -u3}};
    const double ll[5][5] = {
        {beta * (phi + c * u2), -beta * g * u1, -beta * (g * u2 + c), -beta * g * u3, beta * g},
        {1.0 - 2.0 * beta * phi, 2.0 * beta * g * u1, 2.0 * beta * g * u2, 2.0 * beta * g * u3, -2.0 * beta * g},
        {beta * (phi - c * u2), -beta * (g * u1), -beta * (g * u2 - c), -beta * g * u3, beta * g},
        {-u1, 1.0, 0.0, 0.0, 0.0},
        {u3, 0.0, 0.0, -1.0, 0.0}};
    std::copy(&rr[0][0], &rr[0][0] + 25, &r[0][0]);
    std::copy(&ll[0][0], &ll[0][0] + 25, &l[0][0]);
  } else {
    const double rr[5][5] = {{1.0, 1.0, 1.0, 0.0, 0.0}, {u1, u1, u1, -1.0, 0.0}, {u2, u2, u2, 0.0, 1.0},
                             {u3 - c, u3, u3 + c, 0.0, 0.0}, {h - c * u3, ek, h + c * u3, -u1, u2}};
    const double ll[5][5] = {
        {beta * (phi + c * u3), -beta * g * u1, -beta * g * u2, -beta * (g * u3 + c), beta * g},
        {1.0 - 2.0 * beta * phi, 2.0 * beta * g * u1, 2.0 * beta * g * u2, 2.0 * beta * g * u3, -2.0 * beta * g},
        {beta * (phi - c * u3), -beta * (g * u1), -beta * g * u2, -beta * (g * u3 - c), beta * g},
        {u1, -1.0, 0.0, 0.0, 0.0},
        {-u2, 0.0, 1.0, 0.0, 0.0}};
    std::copy(&rr[0][0], &rr[0][0] + 25, &r[0][0]);
    std::copy(&ll[0][0], &ll[0][0] + 25, &l[0][0]);
  }
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 5; ++j) R[i][j] = r[i][j], L[i][j] = l[i][j];
}

// minmod / minmodB (Source/NumericalMethod/AmrDG/AmrDG_Limiter.tpp:40-85).
inline double minmod(double a1, double a2, double a3) {
  const bool same = (std::signbit(a1) == std::signbit(a2)) && (std::signbit(a2) == std::signbit(a3));
  const int sign = std::signbit(a1) ? -1 : +1;
  if (same) return sign * std::min({std::abs(a1), std::abs(a2), std::abs(a3)});
  return 0;
}

inline double minmodB(double a1, double a2, double a3, double thr /* AMR_TVB_C[l] * M * h^2 */) {
  if (std::abs(a1) <= thr) return a1;
  return minmod(a1, a2, a3);
}

}  // namespace oracle

// CPU oracle (test infrastructure only; never linked into the product).
//
// Basis, Gauss-Legendre quadrature and element matrices of the modal
// ADER-DG method, restated from the reference in plain C++17.  Every
// routine follows the reference's own arithmetic order so that the oracle
// reproduces the reference's numbers as closely as a restatement can:
//
//   MultiIndex<P,D>            Source/NumericalMethod/AmrDG/AmrDG.h:62-122
//   GL nodes / weights / tables Source/NumericalMethod/AmrDG/AmrDG.h:145-353
//   quadrature point sets      Source/NumericalMethod/AmrDG/AmrDG_Quadrature.tpp:6-246
//   Legendre recurrences       Source/NumericalMethod/AmrDG/AmrDG_Basis.tpp:4-15
//   V, Vinv (pseudo-inverse)   Source/NumericalMethod/AmrDG/AmrDG_ElementMatrix.tpp:7-26
//   predictor/corrector mats   Source/NumericalMethod/AmrDG/AmrDG_ElementMatrix.tpp:28-198
//   refMat_* integrals         Source/NumericalMethod/AmrDG/AmrDG_ElementMatrix.tpp:200-305
//   AMR projection matrices    Source/NumericalMethod/AmrDG/AmrDG_Interpolater.tpp:85-231
//
// Third-party pieces the reference delegates to Eigen 3.4.0 (absent from the
// reference tree): JacobiSVD pseudo-inverse and PartialPivLU inverse.  They are
// restated here as the exact Moore-Penrose pseudo-inverse (normal equations
// solved in long double) and Gauss-Jordan inversion with partial pivoting in
// long double, each rounded once to double.  Both agree with Eigen's results
// to O(1e-16) relative; bitwise agreement with Eigen is not claimed.
#pragma once

#include <array>
#include <cmath>
#include <vector>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>

namespace oracle {

// ---------------------------------------------------------------------------
// Multi-index of the total-degree Legendre basis (ii slowest, last index
// fastest).  For the space-time basis the last index is time.
// AmrDG.h:62-122
// ---------------------------------------------------------------------------
inline std::vector<std::array<int, 4>> multi_index(int P, int Dtot) {
  std::vector<std::array<int, 4>> r;
  if (Dtot == 1) {
    for (int ii = 0; ii <= P; ++ii) r.push_back({ii, 0, 0, 0});
  } else if (Dtot == 2) {
    for (int ii = 0; ii <= P; ++ii)
      for (int jj = 0; jj <= P - ii; ++jj) r.push_back({ii, jj, 0, 0});
  } else if (Dtot == 3) {
    for (int ii = 0; ii <= P; ++ii)
      for (int jj = 0; jj <= P - ii; ++jj)
        for (int kk = 0; kk <= P - ii - jj; ++kk) r.push_back({ii, jj, kk, 0});
  } else if (Dtot == 4) {
    for (int ii = 0; ii <= P; ++ii)
      for (int jj = 0; jj <= P - ii; ++jj)
        for (int kk = 0; kk <= P - ii - jj; ++kk)
          for (int tt = 0; tt <= P - ii - jj - kk; ++tt) r.push_back({ii, jj, kk, tt});
  }
  return r;
}

// ---------------------------------------------------------------------------
// Constexpr-style GL helpers of QuadratureGaussLegendre<P> (AmrDG.h:151-318).
// ---------------------------------------------------------------------------
inline double cx_cos(double x) {  // AmrDG.h:157-165 (30-term Taylor series)
  double result = 1.0;
  double term = 1.0;
  for (int n = 1; n <= 30; ++n) {
    term *= -x * x / ((2 * n - 1) * (2 * n));
    result += term;
  }
  return result;
}

inline double cx_legendre(int n, double x) {  // AmrDG.h:168-177 (Bonnet)
  if (n == 0) return 1.0;
  if (n == 1) return x;
  double p0 = 1.0, p1 = x;
  for (int k = 2; k <= n; ++k) {
    double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
    p0 = p1;
    p1 = p2;
  }
  return p1;
}

inline double cx_dlegendre(int n, double x) {  // AmrDG.h:180-191
  if (n == 0) return 0.0;
  double p0 = 1.0, p1 = x;
  double dp1 = 1.0;
  for (int k = 2; k <= n; ++k) {
    double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
    double dp2 = k * p1 + x * dp1;
    p0 = p1;
    p1 = p2;
    dp1 = dp2;
  }
  return dp1;
}

struct GL {
  int P = 0, N = 0;
  std::vector<double> nodes, weights;
  // val[k][q] = P_k(nodes[q]); dval likewise; bd_val[k][side]; shifted tables.
  std::vector<std::vector<double>> val, dval, bd_val, shifted_lo, shifted_hi;

  explicit GL(int P_) : P(P_), N(P_ + 1) {
    const double cx_pi = 3.14159265358979323846;
    nodes.assign(N, 0.0);
    int idx = 0;
    for (int i = 1; i <= N / 2; ++i) {  // AmrDG.h:211-237
      double theta = cx_pi * (i - 0.25) / (N + 0.5);
      double x = cx_cos(theta);
      for (int iter = 0; iter < 30; ++iter) {
        double pval = cx_legendre(N, x);
        double dpval = cx_dlegendre(N, x);
        double dx = pval / dpval;
        x -= dx;
        if ((dx >= 0.0 ? dx : -dx) < 1e-16) break;
      }
      nodes[idx++] = x;
      nodes[idx++] = -x;
    }
    if (N % 2 != 0) nodes[idx] = 0.0;
    weights.assign(N, 0.0);
    for (int q = 0; q < N; ++q) {  // AmrDG.h:240-249
      double x = nodes[q];
      double dp = cx_dlegendre(N, x);
      weights[q] = 2.0 / ((1.0 - x * x) * dp * dp);
    }
    val.assign(P + 1, std::vector<double>(N));
    dval.assign(P + 1, std::vector<double>(N));
    shifted_lo.assign(P + 1, std::vector<double>(N));
    shifted_hi.assign(P + 1, std::vector<double>(N));
    bd_val.assign(P + 1, std::vector<double>(2));
    for (int k = 0; k <= P; ++k) {
      for (int q = 0; q < N; ++q) {
        val[k][q] = cx_legendre(k, nodes[q]);
        dval[k][q] = cx_dlegendre(k, nodes[q]);
        shifted_lo[k][q] = cx_legendre(k, 0.5 * nodes[q] - 0.5);
        shifted_hi[k][q] = cx_legendre(k, 0.5 * nodes[q] + 0.5);
      }
      bd_val[k][0] = cx_legendre(k, -1.0);
      bd_val[k][1] = cx_legendre(k, 1.0);
    }
  }

  // AmrDG.h:337-341: flat index m -> 1D node index of dim d (d=0 slowest).
  int node_idx(int m, int d, int Dtot) const {
    int divisor = 1;
    for (int i = 0; i < Dtot - 1 - d; ++i) divisor *= N;
    return (m / divisor) % N;
  }
};

// AmrDG.h:345-348
inline int bd_free_pos(int a, int d_fixed) {
  if (a == d_fixed) return -1;
  return (a < d_fixed) ? a : a - 1;
}

// Legendre<P> value recurrence (AmrDG_Basis.tpp:4-15), used by phi_t.
inline double legendre_rec(int n, double x) {
  std::vector<double> v(std::max(n + 1, 2));
  v[0] = 1.0;
  v[1] = x;
  for (int k = 2; k <= n; ++k) v[k] = ((2 * k - 1) * x * v[k - 1] - (k - 1) * v[k - 2]) / k;
  return v[n];
}

// Dense row-major matrix.
struct Mat {
  int r = 0, c = 0;
  std::vector<double> a;
  Mat() = default;
  Mat(int r_, int c_) : r(r_), c(c_), a((size_t)r_ * c_, 0.0) {}
  double& operator()(int i, int j) { return a[(size_t)i * c + j]; }
  double operator()(int i, int j) const { return a[(size_t)i * c + j]; }
};

inline Mat matmul(const Mat& A, const Mat& B) {
  Mat C(A.r, B.c);
  for (int i = 0; i < A.r; ++i)
    for (int j = 0; j < B.c; ++j) {
      double s = 0.0;
      for (int k = 0; k < A.c; ++k) s += A(i, k) * B(k, j);
      C(i, j) = s;
    }
  return C;
}

// Inverse with partial pivoting, long double, rounded once (stands in for
// Eigen's PartialPivLU inverse used at AmrDG_ElementMatrix.tpp:58).
inline Mat inverse_ld(const Mat& A) {
  int n = A.r;
  std::vector<long double> m((size_t)n * 2 * n, 0.0L);
  for (int i = 0; i < n; ++i) {
    for (int j = 0; j < n; ++j) m[(size_t)i * 2 * n + j] = A(i, j);
    m[(size_t)i * 2 * n + n + i] = 1.0L;
  }
  for (int col = 0; col < n; ++col) {
    int piv = col;
    long double best = fabsl(m[(size_t)col * 2 * n + col]);
    for (int r = col + 1; r < n; ++r) {
      long double v = fabsl(m[(size_t)r * 2 * n + col]);
      if (v > best) { best = v; piv = r; }
    }
    if (best == 0.0L) throw std::runtime_error("singular matrix");
    if (piv != col)
      for (int j = 0; j < 2 * n; ++j) std::swap(m[(size_t)col * 2 * n + j], m[(size_t)piv * 2 * n + j]);
    long double d = m[(size_t)col * 2 * n + col];
    for (int j = 0; j < 2 * n; ++j) m[(size_t)col * 2 * n + j] /= d;
    for (int r = 0; r < n; ++r) {
      if (r == col) continue;
      long double f = m[(size_t)r * 2 * n + col];
      if (f == 0.0L) continue;
      for (int j = 0; j < 2 * n; ++j) m[(size_t)r * 2 * n + j] -= f * m[(size_t)col * 2 * n + j];
    }
  }
  Mat R(n, n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) R(i, j) = (double)m[(size_t)i * 2 * n + n + j];
  return R;
}

// Moore-Penrose pseudo-inverse of a full-column-rank matrix: (A^T A)^-1 A^T in
// long double, rounded once (stands in for the JacobiSVD pseudo-inverse of
// AmrDG_ElementMatrix.tpp:21-25).
inline Mat pinv_ld(const Mat& A) {
  int m = A.r, n = A.c;
  std::vector<long double> G((size_t)n * n, 0.0L);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      long double s = 0.0L;
      for (int k = 0; k < m; ++k) s += (long double)A(k, i) * (long double)A(k, j);
      G[(size_t)i * n + j] = s;
    }
  // invert G (long double Gauss-Jordan)
  std::vector<long double> aug((size_t)n * 2 * n, 0.0L);
  for (int i = 0; i < n; ++i) {
    for (int j = 0; j < n; ++j) aug[(size_t)i * 2 * n + j] = G[(size_t)i * n + j];
    aug[(size_t)i * 2 * n + n + i] = 1.0L;
  }
  for (int col = 0; col < n; ++col) {
    int piv = col;
    long double best = fabsl(aug[(size_t)col * 2 * n + col]);
    for (int r = col + 1; r < n; ++r) {
      long double v = fabsl(aug[(size_t)r * 2 * n + col]);
      if (v > best) { best = v; piv = r; }
    }
    if (piv != col)
      for (int j = 0; j < 2 * n; ++j) std::swap(aug[(size_t)col * 2 * n + j], aug[(size_t)piv * 2 * n + j]);
    long double d = aug[(size_t)col * 2 * n + col];
    for (int j = 0; j < 2 * n; ++j) aug[(size_t)col * 2 * n + j] /= d;
    for (int r = 0; r < n; ++r) {
      if (r == col) continue;
      long double f = aug[(size_t)r * 2 * n + col];
      if (f == 0.0L) continue;
      for (int j = 0; j < 2 * n; ++j) aug[(size_t)r * 2 * n + j] -= f * aug[(size_t)col * 2 * n + j];
    }
  }
  Mat R(n, m);
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < m; ++k) {
      long double s = 0.0L;
      for (int j = 0; j < n; ++j) s += aug[(size_t)i * 2 * n + n + j] * (long double)A(k, j);
      R(i, k) = (double)s;
    }
  return R;
}

// ---------------------------------------------------------------------------
// All element matrices of AmrDG<P> for a given (D, P).
// ---------------------------------------------------------------------------
struct Elem {
  int D, P, N;
  int Np_s, Np_st, qMp_s, qMp_st, qMp_st_bd, qMp_s_bd;
  GL gl;
  std::vector<std::array<int, 4>> mi_s, mi_st;
  std::vector<std::vector<double>> xi_s, xi_t;  // quadrature points (spatial, temporal)
  Mat V, Vinv, Mk_h_w, Mk_h_w_inv, Mk_pred, Mk_corr, quadmat;
  std::vector<Mat> Sk_pred, Sk_predVinv, Sk_corr, Mkbdm, Mkbdp;
  std::vector<std::vector<double>> quad_weights_st_bd;  // [d][m]
  // L2ProjInterp
  Mat Mref, Minv;
  std::vector<Mat> P_cf, P_fc;                          // [2^D]
  std::vector<std::vector<Mat>> P_flux_low, P_flux_high;  // [d][2^(D-1)]

  Elem(int D_, int P_) : D(D_), P(P_), N(P_ + 1), gl(P_) {
    mi_s = multi_index(P, D);
    mi_st = multi_index(P, D + 1);
    Np_s = (int)mi_s.size();
    Np_st = (int)mi_st.size();
    qMp_s = ipow(N, D);
    qMp_st = ipow(N, D + 1);
    qMp_st_bd = ipow(N, D);
    qMp_s_bd = ipow(N, D - 1);
    set_quadpoints();
    set_vandermat();
    set_ref_element_matrix();
    interp_proj_mat();
    flux_proj_mat();
  }

  static int ipow(int b, int e) {
    int r = 1;
    for (int i = 0; i < e; ++i) r *= b;
    return r;
  }

  // AmrDG_Quadrature.tpp:22-246 (spatial and temporal point sets only; the
  // space-time sets are addressed through node_idx).
  void set_quadpoints() {
    xi_s.assign(qMp_s, std::vector<double>(D));
    for (int m = 0; m < qMp_s; ++m)
      for (int d = 0; d < D; ++d) xi_s[m][d] = gl.nodes[gl.node_idx(m, d, D)];
    xi_t.assign(N, std::vector<double>(1));
    for (int i = 0; i < N; ++i) xi_t[i][0] = gl.nodes[i];
  }

  // AmrDG_ElementMatrix.tpp:7-26
  void set_vandermat() {
    V = Mat(qMp_st, Np_st);
    for (int i = 0; i < qMp_st; ++i)
      for (int j = 0; j < Np_st; ++j) {
        double phi = 1.0;
        for (int d = 0; d < D + 1; ++d) phi *= gl.val[mi_st[j][d]][gl.node_idx(i, d, D + 1)];
        V(i, j) = phi;
      }
    Vinv = pinv_ld(V);
  }

  // AmrDG_ElementMatrix.tpp:200-213 (only the D spatial indices enter)
  double refMat_phiphi(int j, const std::vector<std::array<int, 4>>& mj, int i,
                       const std::vector<std::array<int, 4>>& mi) const {
    double m = 1.0;
    for (int d = 0; d < D; ++d)
      m *= (double)(mi[i][d] == mj[j][d] ? 1 : 0) * (2.0 / (2.0 * (double)mj[j][d] + 1.0));
    return m;
  }

  // AmrDG_ElementMatrix.tpp:215-254 (libstdc++ special functions, as the reference)
  double refMat_phiDphi(int j, int i, int dim) const {
    double sum = 0.0;
    for (int q = 0; q < qMp_s; ++q) {
      double w = 1.0;
      double phi = 1.0;
      for (int d = 0; d < D; ++d) phi *= std::legendre(mi_st[j][d], xi_s[q][d]);
      double dphi = 1.0;
      for (int a = 0; a < D; ++a) {
        if (a != dim)
          dphi *= std::legendre(mi_st[i][a], xi_s[q][a]);
        else
          dphi *= (std::assoc_legendre(mi_st[i][dim], 1, xi_s[q][dim])) /
                  (std::sqrt(1.0 - std::pow(xi_s[q][dim], 2.0)));
      }
      for (int d = 0; d < D; ++d) w *= 2.0 / std::pow(std::assoc_legendre(N, 1, xi_s[q][d]), 2.0);
      sum += (phi * dphi * w);
    }
    return sum;
  }

  // AmrDG_ElementMatrix.tpp:257-271
  double refMat_tphitphi(int j, int i) const {
    int ti = mi_st[i][D], tj = mi_st[j][D];
    return (double)(ti == tj ? 1 : 0) * (2.0 / (2.0 * (double)tj + 1.0));
  }

  // AmrDG_ElementMatrix.tpp:274-305
  double refMat_tphiDtphi(int j, int i) const {
    double tphiDtphi = 0.0;
    for (int q = 0; q < N; ++q) {
      double w = 1.0;
      w *= 2.0 / (double)std::pow((double)std::assoc_legendre(N, 1, xi_t[q][0]), 2.0);
      double phi_val = std::legendre(mi_st[i][D], xi_t[q][0]);
      int n_t = mi_st[j][D];
      double x_t = xi_t[q][0];
      double dphi_val = 0.0;
      if (n_t >= 1) {
        double p_prev = 1.0, p_curr = x_t;
        dphi_val = 1.0;
        for (int nn = 2; nn <= n_t; ++nn) {
          double p_next = ((2 * nn - 1) * x_t * p_curr - (nn - 1) * p_prev) / nn;
          dphi_val = nn * p_curr + x_t * dphi_val;
          p_prev = p_curr;
          p_curr = p_next;
        }
      }
      tphiDtphi += (phi_val * dphi_val * w);
    }
    return tphiDtphi;
  }

  double phi_t(int idx, double tau) const { return legendre_rec(mi_st[idx][D], tau); }

  // AmrDG_ElementMatrix.tpp:28-198
  void set_ref_element_matrix() {
    Mk_h_w = Mat(Np_st, Np_st);
    Mk_pred = Mat(Np_st, Np_s);
    Sk_pred.assign(D, Mat(Np_st, Np_st));
    for (int j = 0; j < Np_st; ++j) {
      for (int i = 0; i < Np_st; ++i) {
        Mk_h_w(j, i) = refMat_phiphi(j, mi_st, i, mi_st) *
                       ((phi_t(j, 1.0) * phi_t(i, 1.0)) - refMat_tphiDtphi(j, i));
        for (int d = 0; d < D; ++d) Sk_pred[d](j, i) = refMat_tphitphi(j, i) * refMat_phiDphi(j, i, d);
      }
      for (int i = 0; i < Np_s; ++i) Mk_pred(j, i) = phi_t(j, -1.0) * refMat_phiphi(j, mi_st, i, mi_s);
    }
    Sk_predVinv.clear();
    for (int d = 0; d < D; ++d) Sk_predVinv.push_back(matmul(Sk_pred[d], Vinv));
    Mk_h_w_inv = inverse_ld(Mk_h_w);

    Mk_corr = Mat(Np_s, Np_s);
    for (int j = 0; j < Np_s; ++j)
      for (int i = 0; i < Np_s; ++i) Mk_corr(j, i) = refMat_phiphi(j, mi_s, i, mi_s);

    Sk_corr.assign(D, Mat(Np_s, qMp_st));
    Mkbdm.assign(D, Mat(Np_s, qMp_st_bd));
    Mkbdp.assign(D, Mat(Np_s, qMp_st_bd));
    quad_weights_st_bd.assign(D, std::vector<double>(qMp_st_bd));
    for (int d = 0; d < D; ++d) {
      for (int i = 0; i < qMp_st; ++i) {
        double w = 1.0;
        for (int d_ = 0; d_ < D + 1; ++d_) w *= gl.weights[gl.node_idx(i, d_, D + 1)];
        for (int j = 0; j < Np_s; ++j) {
          double dphi = 1.0;
          for (int a = 0; a < D; ++a) {
            int q_a = gl.node_idx(i, a, D + 1);
            if (a != d)
              dphi *= gl.val[mi_s[j][a]][q_a];
            else
              dphi *= gl.dval[mi_s[j][a]][q_a];
          }
          Sk_corr[d](j, i) = dphi * w;
        }
      }
      for (int i = 0; i < qMp_st_bd; ++i) {
        double wm = 1.0, wp = 1.0;
        for (int pos = 0; pos < D; ++pos) {
          int q_idx = gl.node_idx(i, pos, D);
          wm *= gl.weights[q_idx];
          wp *= gl.weights[q_idx];
        }
        quad_weights_st_bd[d][i] = wm;
        for (int j = 0; j < Np_s; ++j) {
          double phi_m = 1.0, phi_p = 1.0;
          for (int a = 0; a < D; ++a) {
            if (a == d) {
              phi_m *= gl.bd_val[mi_s[j][a]][0];
              phi_p *= gl.bd_val[mi_s[j][a]][1];
            } else {
              int q_a = gl.node_idx(i, bd_free_pos(a, d), D);
              phi_m *= gl.val[mi_s[j][a]][q_a];
              phi_p *= gl.val[mi_s[j][a]][q_a];
            }
          }
          Mkbdm[d](j, i) = phi_m * wm;
          Mkbdp[d](j, i) = phi_p * wp;
        }
      }
    }

    quadmat = Mat(Np_s, qMp_s);
    for (int i = 0; i < qMp_s; ++i) {
      double w = 1.0;
      for (int d = 0; d < D; ++d) w *= gl.weights[gl.node_idx(i, d, D)];
      for (int j = 0; j < Np_s; ++j) {
        double phi = 1.0;
        for (int d = 0; d < D; ++d) phi *= gl.val[mi_s[j][d]][gl.node_idx(i, d, D)];
        quadmat(j, i) = phi * w;
      }
    }
  }

  // AmrDG_Interpolater.tpp:157-231
  void interp_proj_mat() {
    const int nov = 1 << D;
    Mref = Mat(Np_s, Np_s);
    for (int j = 0; j < Np_s; ++j)
      for (int n = 0; n < Np_s; ++n) Mref(j, n) = refMat_phiphi(j, mi_s, n, mi_s);
    // The SVD pseudo-inverse of the diagonal mass matrix is exactly the
    // reciprocal diagonal (a diagonal input needs no Jacobi rotations).
    Minv = Mat(Np_s, Np_s);
    for (int j = 0; j < Np_s; ++j) Minv(j, j) = 1.0 / Mref(j, j);
    P_cf.assign(nov, Mat(Np_s, Np_s));
    P_fc.assign(nov, Mat(Np_s, Np_s));
    for (int l = 0; l < nov; ++l) {
      double shift[3];
      for (int d = 0; d < D; ++d) shift[d] = ((l >> (D - 1 - d)) & 1) ? 0.5 : -0.5;
      for (int j = 0; j < Np_s; ++j)
        for (int m = 0; m < Np_s; ++m) {
          double sum_cf = 0.0, sum_fc = 0.0;
          for (int q = 0; q < qMp_s; ++q) {
            double phi_m = 1.0, phi_j = 1.0;
            for (int d = 0; d < D; ++d) {
              int q_d = gl.node_idx(q, d, D);
              const auto& tbl = (shift[d] < 0.0) ? gl.shifted_lo : gl.shifted_hi;
              phi_m *= tbl[mi_s[m][d]][q_d];
              phi_j *= tbl[mi_s[j][d]][q_d];
            }
            sum_cf += quadmat(j, q) * phi_m;
            sum_fc += quadmat(m, q) * phi_j;
          }
          P_cf[l](j, m) = sum_cf;
          P_fc[l](j, m) = sum_fc;
        }
    }
  }

  // AmrDG_Interpolater.tpp:85-155
  void flux_proj_mat() {
    const int nfc = 1 << (D - 1);
    P_flux_low.assign(D, std::vector<Mat>(nfc, Mat(Np_s, qMp_st_bd)));
    P_flux_high.assign(D, std::vector<Mat>(nfc, Mat(Np_s, qMp_st_bd)));
    for (int d = 0; d < D; ++d)
      for (int k = 0; k < nfc; ++k) {
        double t_shifts[3] = {0, 0, 0};
        int bit_counter = 0;
        for (int dir = 0; dir < D; ++dir) {
          if (dir == d) continue;
          int is_upper = (k >> bit_counter) & 1;
          t_shifts[dir] = is_upper ? 0.5 : -0.5;
          bit_counter++;
        }
        for (int r = 0; r < Np_s; ++r)
          for (int m = 0; m < qMp_st_bd; ++m) {
            double phi_low = 1.0, phi_high = 1.0;
            for (int dim = 0; dim < D; ++dim) {
              if (dim == d) {
                phi_low *= gl.bd_val[mi_s[r][dim]][0];
                phi_high *= gl.bd_val[mi_s[r][dim]][1];
              } else {
                int q_a = gl.node_idx(m, bd_free_pos(dim, d), D);
                const auto& tbl = (t_shifts[dim] < 0.0) ? gl.shifted_lo : gl.shifted_hi;
                phi_low *= tbl[mi_s[r][dim]][q_a];
                phi_high *= tbl[mi_s[r][dim]][q_a];
              }
            }
            double w = quad_weights_st_bd[d][m];
            P_flux_low[d][k](r, m) = phi_low * w;
            P_flux_high[d][k](r, m) = phi_high * w;
          }
      }
  }
};

}  // namespace oracle

// The fourth-order (p = 4) SBP-SAT operator per point.  Coefficients restate
// the p == 4 branches of diagonal_sbp_D2 / diagonal_sbp_D1
// (diagonal_sbp.jl:198-210, 62-67): norm weights 1/bhinv on the first and
// last four points, interior D2 stencil d, 4 x 6 boundary closure bd
// (mirrored with the same values at the far end) and boundary derivative BS;
// the penalty parameters are those of Assembling_matrix
// (level_2_multigrid_new.jl:145-150): h tau_D = -13, tau_N = -1, beta = 1.
//
// With everything scaled by the H~ of the assembly, the operator is a
// Kronecker sum (as for p = 2):
//   (-A u)(i, j) = w_j (X u(:, j))_i + w_i (Y u(i, :))_j
//   X = diag(w) h^2 D2 + h tau_N (E_1 + E_n) BS          (Neumann, along i)
//   Y = diag(w) h^2 D2 + h tau_D (E_1 + E_n)
//       + beta h (BS' E_1 + BS' E_n)                     (Dirichlet, along j)
// X and Y equal d in the interior rows; their first four rows are the
// tables below (the last four mirror them: X[n-1-r][n-1-c] = X[r][c]).
#pragma once

namespace sbp {
namespace p4 {

// Host tables (the reference's values).
constexpr double kBhinv[4] = {48.0 / 17.0, 48.0 / 59.0, 48.0 / 43.0, 48.0 / 49.0};
constexpr double kBd[4][6] = {{2.0, -5.0, 4.0, -1.0, 0.0, 0.0},
                              {1.0, -2.0, 1.0, 0.0, 0.0, 0.0},
                              {-4.0 / 43.0, 59.0 / 43.0, -110.0 / 43.0, 59.0 / 43.0, -4.0 / 43.0, 0.0},
                              {-1.0 / 49.0, 0.0, 59.0 / 49.0, -118.0 / 49.0, 64.0 / 49.0, -4.0 / 49.0}};
constexpr double kBs[4] = {11.0 / 6.0, -3.0, 3.0 / 2.0, -1.0 / 3.0};
constexpr double kTauDh = -13.0, kTauN = -1.0, kBeta = 1.0;

// Interior D2 stencil d (usable in device code).
constexpr double kD0 = -1.0 / 12.0, kD1 = 4.0 / 3.0, kD2 = -5.0 / 2.0;

// norm weight of point k from either end (k = 0 .. 3), device and host
__host__ __device__ constexpr double w_end(int k) {
  return k == 0 ? 17.0 / 48.0 : (k == 1 ? 59.0 / 48.0 : (k == 2 ? 43.0 / 48.0 : 49.0 / 48.0));
}

// first-four-row coefficients of X and Y (host: filled into constant memory)
inline double x_coef(int r, int c) {
  return w_end(r) * kBd[r][c] + (r == 0 && c < 4 ? kTauN * kBs[c] : 0.0);
}
inline double y_coef(int r, int c) {
  return w_end(r) * kBd[r][c] + (r == 0 && c == 0 ? kTauDh : 0.0) + (c == 0 ? kBeta * kBs[r] : 0.0);
}

// smallest grid the closures fit (n - 1 >= max(bn, 2 bm) = 8)
constexpr int kMinN = 9;

}  // namespace p4
}  // namespace sbp

// Higher-order (p = 4, p = 6) SBP-SAT operators per point.
//
// Coefficients restate the p == 4 and p == 6 branches of diagonal_sbp_D2 /
// diagonal_sbp_D1 (diagonal_sbp.jl:198-222, 62-79):
// - norm weights 1/bhinv on the first and last bm points;
// - the interior D2 stencil d;
// - the bm x bn boundary closure bd, mirrored with the same values at the
//   far end;
// - the boundary derivative BS.
// The penalty parameters are those of Assembling_matrix
// (level_2_multigrid_new.jl:145-150): h tau_D = -13, tau_N = -1, beta = 1,
// the same for every order.
//
// Scaled by the H~ of the assembly, the operator is a Kronecker sum, as for
// p = 2 (w = the norm weights over h):
//   (-A u)(i, j) = w_j (X u(:, j))_i + w_i (Y u(i, :))_j
//   X = diag(w) h^2 D2 + h tau_N (E_1 + E_n) BS          (Neumann, along i)
//   Y = diag(w) h^2 D2 + h tau_D (E_1 + E_n)
//       + beta h (BS' E_1 + BS' E_n)                     (Dirichlet, along j)
// X and Y equal d in the interior rows.  Their first bm rows are
// x_coef / y_coef below; the last bm rows mirror them:
// X[n-1-r][n-1-c] = X[r][c].
#pragma once

#include <cuda_runtime.h>

namespace sbp {
namespace ho {

constexpr double kTauDh = -13.0, kTauN = -1.0, kBeta = 1.0;

template <int P>
struct Order;

template <>
struct Order<4> {
  static constexpr int kBm = 4;      // closure rows
  static constexpr int kBn = 6;      // closure columns
  static constexpr int kHalf = 2;    // interior stencil half-width
  static constexpr int kNbs = 4;     // length of BS
  static constexpr int kMinN = 8;    // n >= max(bn, 2 bm), diagonal_sbp.jl:417-420
  // interior D2 stencil at offset +-k (device and host)
  __host__ __device__ static constexpr double d(int k) {
    return k == 0 ? -5.0 / 2.0 : (k == 1 ? 4.0 / 3.0 : -1.0 / 12.0);
  }
  // norm weight of point k (0 .. bm-1) from either end
  __host__ __device__ static constexpr double w_end(int k) {
    return k == 0 ? 17.0 / 48.0 : (k == 1 ? 59.0 / 48.0 : (k == 2 ? 43.0 / 48.0 : 49.0 / 48.0));
  }
  static constexpr double kBd[4][6] = {
      {2.0, -5.0, 4.0, -1.0, 0.0, 0.0},
      {1.0, -2.0, 1.0, 0.0, 0.0, 0.0},
      {-4.0 / 43.0, 59.0 / 43.0, -110.0 / 43.0, 59.0 / 43.0, -4.0 / 43.0, 0.0},
      {-1.0 / 49.0, 0.0, 59.0 / 49.0, -118.0 / 49.0, 64.0 / 49.0, -4.0 / 49.0}};
  static constexpr double kBs[4] = {11.0 / 6.0, -3.0, 3.0 / 2.0, -1.0 / 3.0};
};

template <>
struct Order<6> {
  static constexpr int kBm = 6;
  static constexpr int kBn = 9;
  static constexpr int kHalf = 3;
  static constexpr int kNbs = 5;
  static constexpr int kMinN = 12;
  __host__ __device__ static constexpr double d(int k) {
    return k == 0 ? -49.0 / 18.0 : (k == 1 ? 3.0 / 2.0 : (k == 2 ? -3.0 / 20.0 : 1.0 / 90.0));
  }
  __host__ __device__ static constexpr double w_end(int k) {
    return k == 0   ? 13649.0 / 43200.0
           : k == 1 ? 12013.0 / 8640.0
           : k == 2 ? 2711.0 / 4320.0
           : k == 3 ? 5359.0 / 4320.0
           : k == 4 ? 7877.0 / 8640.0
                    : 43801.0 / 43200.0;
  }
  static constexpr double kBd[6][9] = {
      {114170.0 / 40947.0, -438107.0 / 54596.0, 336409.0 / 40947.0, -276997.0 / 81894.0,
       3747.0 / 13649.0, 21035.0 / 163788.0, 0.0, 0.0, 0.0},
      {6173.0 / 5860.0, -2066.0 / 879.0, 3283.0 / 1758.0, -303.0 / 293.0, 2111.0 / 3516.0,
       -601.0 / 4395.0, 0.0, 0.0, 0.0},
      {-52391.0 / 81330.0, 134603.0 / 32532.0, -21982.0 / 2711.0, 112915.0 / 16266.0,
       -46969.0 / 16266.0, 30409.0 / 54220.0, 0.0, 0.0, 0.0},
      {68603.0 / 321540.0, -12423.0 / 10718.0, 112915.0 / 32154.0, -75934.0 / 16077.0,
       53369.0 / 21436.0, -54899.0 / 160770.0, 48.0 / 5359.0, 0.0, 0.0},
      {-7053.0 / 39385.0, 86551.0 / 94524.0, -46969.0 / 23631.0, 53369.0 / 15754.0,
       -87904.0 / 23631.0, 820271.0 / 472620.0, -1296.0 / 7877.0, 96.0 / 7877.0, 0.0},
      {21035.0 / 525612.0, -24641.0 / 131403.0, 30409.0 / 87602.0, -54899.0 / 131403.0,
       820271.0 / 525612.0, -117600.0 / 43801.0, 64800.0 / 43801.0, -6480.0 / 43801.0,
       480.0 / 43801.0}};
  static constexpr double kBs[5] = {25.0 / 12.0, -4.0, 3.0, -4.0 / 3.0, 1.0 / 4.0};
};

// Closure rows r = 0 .. bm-1 of X and Y (host: filled into constant memory).
template <int P>
inline double x_coef(int r, int c) {
  using O = Order<P>;
  return O::w_end(r) * O::kBd[r][c] + (r == 0 && c < O::kNbs ? kTauN * O::kBs[c] : 0.0);
}
template <int P>
inline double y_coef(int r, int c) {
  using O = Order<P>;
  return O::w_end(r) * O::kBd[r][c] + (r == 0 && c == 0 ? kTauDh : 0.0) +
         (c == 0 && r < O::kNbs ? kBeta * O::kBs[r] : 0.0);
}

// Norm weight (over h) of index k on an n-point line.
template <int P>
__host__ __device__ inline double weight(int k, int n) {
  using O = Order<P>;
  return k < O::kBm ? O::w_end(k) : (k > n - 1 - O::kBm ? O::w_end(n - 1 - k) : 1.0);
}

// Dense 1D operators X (Neumann) and Y (Dirichlet) on n points, row-major.
template <int P>
inline void one_d(int n, double* X, double* Y) {
  using O = Order<P>;
  for (int k = 0; k < n * n; ++k) X[k] = Y[k] = 0.0;
  for (int r = 0; r < n; ++r) {
    if (r >= O::kBm && r <= n - 1 - O::kBm) {
      for (int o = -O::kHalf; o <= O::kHalf; ++o) {
        X[r * n + r + o] = O::d(o < 0 ? -o : o);
        Y[r * n + r + o] = O::d(o < 0 ? -o : o);
      }
    } else {
      const bool lo = r < O::kBm;
      const int rr = lo ? r : n - 1 - r;
      for (int c = 0; c < O::kBn; ++c) {
        const int cc = lo ? c : n - 1 - c;
        X[r * n + cc] = x_coef<P>(rr, c);
        Y[r * n + cc] = y_coef<P>(rr, c);
      }
    }
  }
}

}  // namespace ho
}  // namespace sbp

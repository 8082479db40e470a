// Second-order SBP-SAT operator for div(c grad u) with nodal coefficients c.
//
// The 1D operator is variable_diagonal_sbp_D2(2, N, B)
// (diagonal_sbp.jl:470-495, 709-740):
// - M is symmetric with face values (c_k + c_k+1)/2;
// - S0 = -c_0 BS/h and SN = c_n-1 BS/h, with BS = (3/2, -2, 1/2);
// - D = HI (-M + SN - S0).
// Every grid line carries the operator built from its own coefficients, with
// the SATs of Assembling_matrix (level_2_multigrid_new.jl:145-150):
// - Neumann along the fast index i (tau_N = -1 cancels the boundary flux);
// - Dirichlet along the slow index j with penalty tau_D * c at the boundary
//   point, plus beta (SN - S0)'.
// With c = 1 this is the constant-coefficient operator.
//
// Scaled by H~, -A is a symmetric stencil: five points plus a coupling two
// columns apart next to each Dirichlet side.  Stored per point:
//   E(i, j)  coupling (i, j) <-> (i+1, j)  = w_j (c(i,j) + c(i+1,j)) / 2
//   N(i, j)  coupling (i, j) <-> (i, j+1)  = w_i ((c(i,j) + c(i,j+1)) / 2
//                                            - 2 c(i,0)    [j = 0]
//                                            - 2 c(i,n-1)  [j = n-2])
//   D(i, j)  minus the diagonal of -A      = sum of the face couplings
//                                            + 10 w_i c(i,j) [j = 0, n-1]
//   Flo(i)   coupling (i, 0) <-> (i, 2)    = w_i c(i,0) / 2
//   Fhi(i)   coupling (i, n-1) <-> (i, n-3) = w_i c(i,n-1) / 2
// (w = 1/2 on the first and last index, 1 elsewhere), so that
//   (-A u)(i, j) = E(i-1,j) u(i-1,j) + E(i,j) u(i+1,j)
//                + N(i,j-1) u(i,j-1) + N(i,j) u(i,j+1) - D(i,j) u(i,j)
//                + the F couplings on columns 0, 2, n-3, n-1.
#pragma once

#include <cuda_runtime.h>

namespace sbp {
namespace vc {

constexpr double kTauDh = -13.0;   // h tau_D
constexpr double kBs0 = 1.5, kBs1 = -2.0, kBs2 = 0.5;

// Separately rounded product and sum (no FMA contraction), so that host and
// device code give the same bits.
__host__ __device__ inline double mul_rn(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  volatile double t = a * b;
  return t;
#endif
}
__host__ __device__ inline double add_rn(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(a, b);
#else
  volatile double t = a + b;
  return t;
#endif
}

__host__ __device__ inline int clamp_index(int k, int n) { return k < 0 ? 0 : (k >= n ? n - 1 : k); }

// Coarse nodal coefficient (I, J) of the nc x nc grid below the fine field cf
// ((2nc - 1)^2 values, i fast): the harmonic mean of cf over the
// full-weighting stencil of (2I, 2J),
//   1 / sum_ab w_a w_b / cf(2I + a, 2J + b),  a, b in {-1, 0, 1},
// w = (1/4, 1/2, 1/4), fine indices clamped to the grid.  The sums run along
// j first, then along i, left to right.  Injection (cf(2I, 2J)) under-samples
// layers thinner than the coarse spacing; the harmonic mean keeps their
// conductance.
__host__ __device__ inline double coarse_coefficient(const double* cf, int nc, int I, int J) {
  const int nf = 2 * nc - 1;
  const double w[3] = {0.25, 0.5, 0.25};
  double both = 0.0;
  for (int a = 0; a < 3; ++a) {
    const int i = clamp_index(2 * I + a - 1, nf);
    double col = 0.0;
    for (int b = 0; b < 3; ++b) {
      const int j = clamp_index(2 * J + b - 1, nf);
      const double t = mul_rn(w[b], 1.0 / cf[(size_t)j * nf + i]);
      col = b == 0 ? t : add_rn(col, t);
    }
    const double t = mul_rn(w[a], col);
    both = a == 0 ? t : add_rn(both, t);
  }
  return 1.0 / both;
}

__host__ __device__ inline double weight(int k, int n) {
  return (k == 0 || k == n - 1) ? 0.5 : 1.0;
}

// Coefficients of point (i, j) from the nodal field c (column-major, ld n):
// e = E(i, j), nn = N(i, j), d = D(i, j).  Flo / Fhi come from f_lo / f_hi.
template <typename C>
__host__ __device__ inline void coefficients(const C& c, int i, int j, int n, double& e,
                                             double& nn, double& d) {
  const double wi = weight(i, n), wj = weight(j, n);
  const double cij = c(i, j);
  const double fxm = i > 0 ? 0.5 * (c(i - 1, j) + cij) : 0.0;
  const double fxp = i < n - 1 ? 0.5 * (cij + c(i + 1, j)) : 0.0;
  const double fym = j > 0 ? 0.5 * (c(i, j - 1) + cij) : 0.0;
  const double fyp = j < n - 1 ? 0.5 * (cij + c(i, j + 1)) : 0.0;
  e = wj * fxp;
  double ny = fyp;
  if (j == 0) ny += kBs1 * c(i, 0);
  if (j == n - 2) ny += kBs1 * c(i, n - 1);
  nn = j < n - 1 ? wi * ny : 0.0;
  // -(diagonal of -A): the faces, and at a Dirichlet side the closure
  // -(BS_0 + h tau_D + beta BS_0) c = 10 c
  d = wj * (fxm + fxp) + wi * (fym + fyp);
  if (j == 0 || j == n - 1) d += wi * -(kBs0 + kTauDh + kBs0) * cij;
}

__host__ __device__ inline double f_lo(double c_i0, int i, int n) {
  return weight(i, n) * kBs2 * c_i0;
}
__host__ __device__ inline double f_hi(double c_in, int i, int n) {
  return weight(i, n) * kBs2 * c_in;
}

}  // namespace vc
}  // namespace sbp

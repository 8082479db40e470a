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

// ---------------------------------------------------------------------------
// Galerkin coarse operators A_c = P' A P (P: bilinear prolongation, nc ->
// 2nc - 1 per direction).  For the variable-coefficient operator A_c is a
// symmetric 9-point stencil at every coarse point, and P' A_c P stays one.
// A 9-point level stores per point D (the diagonal of A) and the couplings
// of -A to (i+1, j), (i, j+1), (i+1, j+1) and (i-1, j+1): E, N, NE, NW.
// ---------------------------------------------------------------------------
struct Stencil9 {
  double d, e, n, ne, nw;
};

// A(p, p + (di, dj)) of the fine operator at p = (i, j) on n x n points, for
// the offsets of `galerkin_row` (|di| <= 1, |dj| <= 2).
// FineVc: the variable-coefficient operator from nodal c (c(i, j) accessor).
template <typename C>
struct FineVc {
  const C& c;
  int n;
  __host__ __device__ double operator()(int i, int j, int di, int dj) const {
    double e, nn, d;
    if (di == 0 && dj == 0) {
      coefficients(c, i, j, n, e, nn, d);
      return d;
    }
    if (dj == 0) {   // E(min(i, i + di), j)
      coefficients(c, di > 0 ? i : i - 1, j, n, e, nn, d);
      return -e;
    }
    if (di != 0) return 0.0;
    if (dj == 1 || dj == -1) {   // N(i, min(j, j + dj))
      coefficients(c, i, dj > 0 ? j : j - 1, n, e, nn, d);
      return -nn;
    }
    // the couplings two columns apart next to the Dirichlet sides
    const int a = dj > 0 ? j : j - 2;   // the pair (a, a + 2)
    double v = 0.0;
    if (a == 0) v -= f_lo(c(i, 0), i, n);
    if (a + 2 == n - 1) v -= f_hi(c(i, n - 1), i, n);
    return v;
  }
};

// A 9-point level (arrays of n x n points, i fast) as the same accessor.
struct FineNine {
  const double *d, *e, *n_, *ne, *nw;
  int n;
  __host__ __device__ double operator()(int i, int j, int di, int dj) const {
    if (di < -1 || di > 1 || dj < -1 || dj > 1) return 0.0;
    const auto at = [&](const double* a, int ii, int jj) { return a[(size_t)jj * n + ii]; };
    if (di == 0 && dj == 0) return at(d, i, j);
    if (dj == 0) return -at(e, di > 0 ? i : i - 1, j);
    if (di == 0) return -at(n_, i, dj > 0 ? j : j - 1);
    if (di == dj) return -at(ne, di > 0 ? i : i - 1, di > 0 ? j : j - 1);
    return -at(nw, di < 0 ? i : i + 1, dj > 0 ? j : j - 1);   // (-1, 1) or (1, -1)
  }
};

// Row (I, J) of P' A P on the nc x nc coarse grid: out[1 + dJ][1 + dI] =
// A_c((I, J), (I + dI, J + dJ)).  Each fine point p of P(:, (I, J)) (the
// 3 x 3 block around (2I, 2J), weights 1, 1/2, 1/4) meets each fine
// neighbour q it couples to (offsets up to 1 in i, 2 in j), and q passes
// A(p, q) P(p, K) on to its coarse parents (one, two or four points, weights
// 1, 1/2, 1/4), all within one coarse point of (I, J).  Fixed loop order:
// deterministic.
template <typename Fine>
__host__ __device__ inline void galerkin_row(const Fine& A, int nc, int I, int J,
                                             double out[3][3]) {
  const int nf = 2 * nc - 1;
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) out[a][b] = 0.0;
  for (int pb = -1; pb <= 1; ++pb) {
    const int pj = 2 * J + pb;
    if (pj < 0 || pj >= nf) continue;
    const double wpj = pb == 0 ? 1.0 : 0.5;
    for (int pa = -1; pa <= 1; ++pa) {
      const int pi = 2 * I + pa;
      if (pi < 0 || pi >= nf) continue;
      const double wp = wpj * (pa == 0 ? 1.0 : 0.5);
      for (int dj = -2; dj <= 2; ++dj) {
        const int qj = pj + dj;
        if (qj < 0 || qj >= nf) continue;
        for (int di = -1; di <= 1; ++di) {
          const int qi = pi + di;
          if (qi < 0 || qi >= nf) continue;
          const double apq = A(pi, pj, di, dj);
          if (apq == 0.0) continue;
          const double v = wp * apq;
          // coarse parents of q
          const int i0 = qi >> 1, j0 = qj >> 1;
          const bool oi = qi & 1, oj = qj & 1;
          for (int sj = 0; sj <= (oj ? 1 : 0); ++sj)
            for (int si = 0; si <= (oi ? 1 : 0); ++si) {
              const double w = (oi ? 0.5 : 1.0) * (oj ? 0.5 : 1.0);
              const int dI = i0 + si - I, dJ = j0 + sj - J;
              // always within one point (the two-apart couplings join even
              // columns); the bound only guards the array
              if (dI < -1 || dI > 1 || dJ < -1 || dJ > 1) continue;
              out[1 + dJ][1 + dI] += w * v;
            }
        }
      }
    }
  }
}

// The stored form of a Galerkin row.
__host__ __device__ inline Stencil9 stencil9_of(const double r[3][3]) {
  return Stencil9{r[1][1], -r[1][2], -r[2][1], -r[2][2], -r[2][0]};
}

}  // namespace vc
}  // namespace sbp

// Shared definitions for the SBP-SAT Poisson kernels (sm_103a).
//
// Grid functions are column-major n x n arrays: point (i, j) lives at
// p[j * ld + i], i the fast index.  This is the layout of the reference's
// CuArray{Float64,2} arguments (split_matrix_free.jl:444), where i runs along
// x and j along y; the reference's W/E (Dirichlet) sides are j = 0 / n-1 and
// its S/N (Neumann) sides are i = 0 / n-1.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sbp {

// ---------------------------------------------------------------------------
// Operator constants.  The reference hard-codes tau_W = tau_E = -13/h,
// tau_S = tau_N = -1 and beta = 1 (level_2_multigrid_new.jl:145-150,
// split_matrix_free.jl:453-455).  After the H-tilde scaling every SAT term is
// h-free, which is what makes the operator a fixed-coefficient stencil.
// ---------------------------------------------------------------------------
constexpr double kTauDh = -13.0;              // h * tau_D
constexpr double kTauN = -1.0;
constexpr double kBeta = 1.0;
// Dirichlet SAT weights on the three columns next to a Dirichlet side:
// tau_D*h*u + beta*BS^T u with BS = [3/2, -2, 1/2]  (SBP_W!, :391-408).
constexpr double kCD0 = kTauDh + 1.5 * kBeta;  // -11.5 on the boundary column
constexpr double kCD1 = -2.0 * kBeta;          // spread into the next column
constexpr double kCD2 = 0.5 * kBeta;           // and the one after
// i-direction terms of a Neumann row, wi*Li + tau_N*BS: the one-sided D2
// (c - 2u1 + u2)/2 plus tau_N*(1.5c - 2u1 + 0.5u2) (SBP_N!, :324-355).
constexpr double kN0 = 0.5 + 1.5 * kTauN;     // on u(i)    = -1
constexpr double kN1 = -1.0 - 2.0 * kTauN;    // on u(i+-1) = +1
constexpr double kN2 = 0.5 + 0.5 * kTauN;     // on u(i+-2) =  0
static_assert(kN2 == 0.0,
              "with tau_N = -1 a Neumann row needs no second neighbour; the "
              "tile halo of one point relies on it");

// Restriction kinds (mirrors sbp_restriction in sbpmg.h).
enum Restriction : int { kRestrictNormal = 0, kRestrictSbp = 1, kRestrictGalerkin = 2 };
enum Smoother : int { kSmoothJacobi = 0, kSmoothRichardson = 1 };

// ---------------------------------------------------------------------------
// The operator.  negA returns (-A u)(i, j) = (H~ (D2 + SAT) u)(i, j), i.e. the
// value the reference's matrix_free_A_full_GPU writes.  It is the assembled
// -H~ (D2 + SAT_W + SAT_E + SAT_S + SAT_N) of Assembling_matrix
// (level_2_multigrid_new.jl:125-188) written per point:
//   -A u = wj * (wi Li u + Neu_i u) + wi * (wj Lj u + Dir_j u)
// with w = 1/2 on the boundary rows/columns, L the 1D D2 (one-sided on the
// boundary), Neu the Neumann SAT and Dir the Dirichlet SAT.
// `u(di, dj)` returns the field at (i + di, j + dj).  Offsets used:
// (0,0), (+-1,0), (0,+-1) everywhere; (0,+-2) only on columns 0, 2, n-3, n-1.
// ---------------------------------------------------------------------------
template <typename R, typename U>
__host__ __device__ __forceinline__ R negA(const U& u, int i, int j, int n) {
  const R c = u(0, 0);
  if (i > 0 && i < n - 1 && j > 2 && j < n - 3) {
    return (u(-1, 0) + u(1, 0)) + (u(0, -1) + u(0, 1)) - R(4) * c;
  }
  R xi;
  if (i == 0) {
    xi = R(kN0) * c + R(kN1) * u(1, 0);
  } else if (i == n - 1) {
    xi = R(kN0) * c + R(kN1) * u(-1, 0);
  } else {
    xi = u(-1, 0) - R(2) * c + u(1, 0);
  }
  R yj;
  if (j == 0) {
    yj = R(0.5) * (c - R(2) * u(0, 1) + u(0, 2));
  } else if (j == n - 1) {
    yj = R(0.5) * (c - R(2) * u(0, -1) + u(0, -2));
  } else {
    yj = u(0, -1) - R(2) * c + u(0, 1);
  }
  if (j <= 2) yj += R(j == 0 ? kCD0 : (j == 1 ? kCD1 : kCD2)) * u(0, -j);
  if (j >= n - 3) {
    const int d = n - 1 - j;
    yj += R(d == 0 ? kCD0 : (d == 1 ? kCD1 : kCD2)) * u(0, d);
  }
  const R wi = (i == 0 || i == n - 1) ? R(0.5) : R(1);
  const R wj = (j == 0 || j == n - 1) ? R(0.5) : R(1);
  return wj * xi + wi * yj;
}

// diag(A)(i, j): minus the coefficient of u(i, j) in negA.  Interior 4,
// Neumann edge 2, Dirichlet edge 12, corner 6.
__host__ __device__ __forceinline__ double diagA(int i, int j, int n) {
  const bool bi = (i == 0 || i == n - 1);
  const bool bj = (j == 0 || j == n - 1);
  const double wi = bi ? 0.5 : 1.0;
  const double wj = bj ? 0.5 : 1.0;
  const double xi0 = bi ? kN0 : -2.0;
  double yj0 = bj ? 0.5 : -2.0;
  if (bj) yj0 += kCD0;
  return -(wj * xi0 + wi * yj0);
}

// 1 / diag(A)(i, j) without a division: the diagonal only takes the four
// values above (n >= 3).
template <typename R>
__host__ __device__ __forceinline__ R inv_diagA(int i, int j, int n) {
  const bool bi = (i == 0 || i == n - 1);
  const bool bj = (j == 0 || j == n - 1);
  if (!bi && !bj) return R(0.25);
  if (bi && bj) return R(1.0 / 6.0);
  if (bj) return R(1.0 / 12.0);
  return R(0.5);
}

// 1D restriction weights: coefficient of fine index 2c + a (a in -1..1) in
// coarse index c.  normal = restriction_matrix_normal (boundary 1/2, 1/4),
// sbp = restriction_matrix (boundary 1/2, 1/2), galerkin = P^T = 2*normal
// (level_2_multigrid_new.jl:205-233).
// Computed in the kernel's own precision R: every weight is a power of two.
template <typename R = double>
__host__ __device__ __forceinline__ R restrict_w1(int kind, int c, int nc, int a) {
  if ((c == 0 && a < 0) || (c == nc - 1 && a > 0)) return R(0);
  const bool edge = (c == 0 || c == nc - 1);
  const bool gal = (kind == kRestrictGalerkin);
  if (a == 0) return gal ? R(1) : R(0.5);
  if (kind == kRestrictSbp && edge) return R(0.5);
  return gal ? R(0.5) : R(0.25);
}

// sign * (A u)(i, j) with the sign folded into the stencil's final FMA (no
// separate multiply: on GB300 every FP64 instruction counts).
template <typename R, typename U>
__host__ __device__ __forceinline__ R signedA(const U& u, int i, int j, int n, int sign) {
  if (i > 0 && i < n - 1 && j > 2 && j < n - 3) {
    const R c = u(0, 0);
    const R sum = (u(-1, 0) + u(1, 0)) + (u(0, -1) + u(0, 1));
    return sign > 0 ? fma(R(4), c, -sum) : fma(R(-4), c, sum);
  }
  const R v = negA<R>(u, i, j, n);
  return sign > 0 ? -v : v;
}

// ---------------------------------------------------------------------------
// Device-resident solver state: scalars of the Krylov recurrences live on
// the GPU so an iteration needs no host round trip.
// ---------------------------------------------------------------------------
struct SolveState {
  double rz;        // r.z of the current iterate (r.r for plain CG)
  double rz_new;
  double pAp;
  double alpha;
  double beta;
  double rr;        // ||r||^2 of the latest iterate
  double rr0;       // ||r0||^2
  double thresh2;   // stop when rr < thresh2
  int iter;         // completed iterations
  int done;         // 1 = converged, 2 = breakdown/non-finite, 3 = max iter
  int maxiter;
  int pad;
  // r.z of a post-smoothing pass split between the boundary tiles and the
  // interior wave (running concurrently): each side leaves its share and
  // counts in; the second to arrive finishes (ring + wave, in that order)
  double rz_part;
  double rz_wave;
  unsigned join;
  int pad2;
};

constexpr int kDoneConverged = 1;
constexpr int kDoneBreakdown = 2;
constexpr int kDoneMaxIter = 3;

// Scratch for deterministic grid reductions: one partial per CTA plus a
// completion ticket that the last CTA resets to zero.
struct ReduceBuf {
  double* partials;
  unsigned* ticket;
};

// Simple strided view of a grid function.
template <typename T>
struct Grid {
  T* p;
  int ld;
  __host__ __device__ __forceinline__ T& at(int i, int j) const {
    return p[(size_t)j * (size_t)ld + (size_t)i];
  }
};

}  // namespace sbp

// Coarse direct solve by fast diagonalisation (host set-up, cached).
//
// The operator is a Kronecker sum: (-A u)(i, j) = w_j (X u(:, j))_i +
// w_i (Y u(i, :))_j with X the 1D Neumann operator along i, Y the 1D
// Dirichlet operator along j and w the boundary weights (1/2 on the first and
// last index, 1 elsewhere).  With Kx = -X, Ky = -Y and W = diag(w):
//   A = W (x) Kx + Ky (x) W      (column-major vec, i fastest).
// The generalised eigenproblems Kx Vx = W Vx Lx, Ky Vy = W Vy Ly with
// Vx^T W Vx = Vy^T W Vy = I diagonalise A:
//   A^{-1} B = Vx [ (Vx^T B Vy) ./ (lx_i + ly_j) ] Vy^T     (B an nc x nc grid).
#pragma once

#include <memory>
#include <vector>

namespace sbp {

struct CoarseFactors {
  int nc = 0;
  // All nc x nc, column-major (element (r, c) at r + c * nc).
  std::vector<double> Vx, VxT, Vy, VyT;
  std::vector<double> dinv;  // 1 / (lx_i + ly_j) at i + j * nc
};

// Largest coarse grid of the fast-diagonalisation solve (p = 2; 257 for
// p = 4, 6).  Grids above 257 take the GPU eigen-solver at set-up, so they
// need a current CUDA device.
constexpr int kCoarseMaxN = 1025;

// Factors of the coarse operator of SBP order p (2, 4 or 6) on an nc x nc
// grid (3 <= nc <= kCoarseMaxN for p = 2; ho_min_points(p) <= nc <= 257
// otherwise).  For
// p = 2 the Kronecker structure is checked against the kernels' own stencil
// coefficients.  Throws std::runtime_error on failure.
std::shared_ptr<const CoarseFactors> coarse_factors(int nc, int p = 2);

// Smallest grid of the order-p operator (p = 4, 6; 0 otherwise).
int ho_min_points(int p);

// x = A^{-1} b on the host with the factors (column-major nc x nc grids).
void coarse_solve_host(const CoarseFactors& f, const double* b, double* x);

// Row-major (= column-major, it is symmetric) nc^2 x nc^2 inverse of the
// order-p operator A, column by column from the factors.
std::shared_ptr<const std::vector<double>> coarse_inverse(int nc, int p = 2);

}  // namespace sbp

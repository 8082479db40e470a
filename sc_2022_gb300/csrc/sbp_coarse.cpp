// Host-side set-up of the coarse direct solve: assemble the re-discretised
// coarse operator A_c (the reference builds it with Assembling_matrix(level-1)
// and factors it with lu(), matrix_free_mg_cg.jl:455,460), factor it with a
// banded Cholesky (A_c is SPD with half-bandwidth 2*nc in the flat ordering
// because the Dirichlet SAT couples columns j and j+2), and form the dense
// inverse so the per-V-cycle solve is one bandwidth-bound GEMV on the GPU
// instead of a latency-bound triangular solve.  The inverse of each coarse
// size is computed once per process and cached.
#include <algorithm>
#include <cmath>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <thread>
#include <vector>

#include "sbp_common.cuh"
#include "sbp_coarse.h"

namespace sbp {

namespace {

// Indicator accessor: evaluating negA with it yields the coefficient of the
// neighbour at offset (di, dj).
struct Indicator {
  int di, dj;
  double operator()(int a, int b) const { return (a == di && b == dj) ? 1.0 : 0.0; }
};

struct Band {
  int N, w;                 // order, half-bandwidth
  std::vector<double> a;    // a[k*(w+1) + d] = M(k, k-d), d = 0..w
  double& at(int k, int d) { return a[(size_t)k * (w + 1) + d]; }
  double get(int r, int c) const {  // r >= c
    const int d = r - c;
    return (d > w) ? 0.0 : a[(size_t)r * (w + 1) + d];
  }
};

Band assemble_band(int nc) {
  Band B;
  B.N = nc * nc;
  B.w = 2 * nc;
  B.a.assign((size_t)B.N * (B.w + 1), 0.0);
  static const int offs[7][2] = {{0, 0}, {-1, 0}, {1, 0}, {0, -1}, {0, 1}, {0, -2}, {0, 2}};
  for (int j = 0; j < nc; ++j) {
    for (int i = 0; i < nc; ++i) {
      const int row = j * nc + i;
      for (const auto& o : offs) {
        const int ii = i + o[0], jj = j + o[1];
        if (ii < 0 || ii >= nc || jj < 0 || jj >= nc) continue;
        const double c = -negA<double>(Indicator{o[0], o[1]}, i, j, nc);
        if (c == 0.0) continue;
        const int col = jj * nc + ii;
        if (col <= row) B.at(row, row - col) += c;  // lower triangle (A is symmetric)
      }
    }
  }
  return B;
}

// In-place banded Cholesky A = L L^T (lower band).
void band_cholesky(Band& B) {
  const int N = B.N, w = B.w;
  for (int k = 0; k < N; ++k) {
    const int j0 = std::max(0, k - w);
    for (int j = j0; j <= k; ++j) {
      double s = B.get(k, j);
      const int m0 = std::max(j0, j - w);
      for (int m = m0; m < j; ++m) s -= B.get(k, m) * B.get(j, m);
      if (j == k) {
        if (!(s > 0.0)) throw std::runtime_error("coarse operator is not positive definite");
        B.at(k, 0) = std::sqrt(s);
      } else {
        B.at(k, k - j) = s / B.get(j, j);
      }
    }
  }
}

std::shared_ptr<const std::vector<double>> build_inverse(int nc) {
  Band L = assemble_band(nc);
  band_cholesky(L);
  const int N = L.N, w = L.w;
  auto X = std::make_shared<std::vector<double>>((size_t)N * N, 0.0);
  unsigned nt = std::max(1u, std::thread::hardware_concurrency());
  nt = std::min(nt, 64u);
  auto worker = [&](unsigned t) {
    std::vector<double> y(N), x(N);
    for (int c = (int)t; c < N; c += (int)nt) {
      // Forward: L y = e_c (y is zero above c).
      for (int k = c; k < N; ++k) {
        double s = (k == c) ? 1.0 : 0.0;
        const int m0 = std::max(c, k - w);
        for (int m = m0; m < k; ++m) s -= L.get(k, m) * y[m];
        y[k] = s / L.get(k, k);
      }
      // Backward: L^T x = y, only rows >= c are needed (symmetry).
      for (int k = N - 1; k >= c; --k) {
        double s = y[k];
        const int m1 = std::min(N - 1, k + w);
        for (int m = k + 1; m <= m1; ++m) s -= L.get(m, k) * x[m];
        x[k] = s / L.get(k, k);
      }
      for (int k = c; k < N; ++k) {
        (*X)[(size_t)k * N + c] = x[k];
        (*X)[(size_t)c * N + k] = x[k];
      }
    }
  };
  std::vector<std::thread> th;
  for (unsigned t = 1; t < nt; ++t) th.emplace_back(worker, t);
  worker(0);
  for (auto& t : th) t.join();
  return X;
}

}  // namespace

std::shared_ptr<const std::vector<double>> coarse_inverse(int nc) {
  static std::mutex mu;
  static std::map<int, std::shared_ptr<const std::vector<double>>> cache;
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find(nc);
  if (it != cache.end()) return it->second;
  auto X = build_inverse(nc);
  cache[nc] = X;
  return X;
}

}  // namespace sbp

// Host-side set-up of the coarse direct solve.  The reference assembles the
// re-discretised coarse operator (Assembling_matrix(level-1)) and factors it
// with lu() (matrix_free_mg_cg.jl:455,460).  Here the same operator is
// inverted by fast diagonalisation: it is the Kronecker sum of two symmetric
// 1D operators, so two dense nc x nc eigenbases replace the LU factors and the
// GPU solve is four small matrix products instead of a sparse triangular
// solve.  The 1D operators are checked, coefficient by coefficient, against
// the stencil negA that every kernel applies.
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "sbp_coarse.h"
#include "sbp_common.cuh"
#include "sbp_high_order.cuh"

namespace sbp {

namespace {

// Indicator accessor: evaluating negA with it yields the coefficient of the
// neighbour at offset (di, dj).
struct Indicator {
  int di, dj;
  double operator()(int a, int b) const { return (a == di && b == dj) ? 1.0 : 0.0; }
};

double weight(int k, int n) { return (k == 0 || k == n - 1) ? 0.5 : 1.0; }

// 1D operators of negA (dense n x n, row-major): X along i (Neumann SAT),
// Y along j (Dirichlet SAT).
void one_d_operators(int n, std::vector<double>& X, std::vector<double>& Y) {
  X.assign((size_t)n * n, 0.0);
  Y.assign((size_t)n * n, 0.0);
  auto x = [&](int r, int c) -> double& { return X[(size_t)r * n + c]; };
  auto y = [&](int r, int c) -> double& { return Y[(size_t)r * n + c]; };
  for (int r = 0; r < n; ++r) {
    if (r == 0 || r == n - 1) {
      const int in = (r == 0) ? 1 : n - 2;
      x(r, r) += kN0;
      x(r, in) += kN1;
    } else {
      x(r, r - 1) += 1.0;
      x(r, r) += -2.0;
      x(r, r + 1) += 1.0;
    }
    if (r == 0 || r == n - 1) {
      const int s = (r == 0) ? 1 : -1;
      y(r, r) += 0.5;
      y(r, r + s) += -1.0;
      y(r, r + 2 * s) += 0.5;
    } else {
      y(r, r - 1) += 1.0;
      y(r, r) += -2.0;
      y(r, r + 1) += 1.0;
    }
    if (r <= 2) y(r, 0) += (r == 0 ? kCD0 : (r == 1 ? kCD1 : kCD2));
    if (r >= n - 3) {
      const int d = n - 1 - r;
      y(r, n - 1) += (d == 0 ? kCD0 : (d == 1 ? kCD1 : kCD2));
    }
  }
}

// negA(i, j) must equal w_j X(i, :) u(:, j) + w_i Y(j, :) u(i, :) for every
// point and every neighbour offset the stencil can reach.
void check_kronecker(int n, const std::vector<double>& X, const std::vector<double>& Y) {
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i)
      for (int dj = -2; dj <= 2; ++dj)
        for (int di = -2; di <= 2; ++di) {
          const int ii = i + di, jj = j + dj;
          if (ii < 0 || ii >= n || jj < 0 || jj >= n) continue;
          const double got = negA<double>(Indicator{di, dj}, i, j, n);
          double want = 0.0;
          if (dj == 0) want += weight(j, n) * X[(size_t)i * n + ii];
          if (di == 0) want += weight(i, n) * Y[(size_t)j * n + jj];
          if (std::fabs(got - want) > 1e-14 * (1.0 + std::fabs(want)))
            throw std::runtime_error("coarse operator is not a Kronecker sum at (" +
                                     std::to_string(i) + "," + std::to_string(j) + ")");
        }
}

// Cyclic Jacobi eigenvalue algorithm (Golub & Van Loan, Matrix Computations,
// 4th ed., Alg. 8.5.3) on a dense symmetric n x n matrix S (row-major,
// destroyed).  On return lam[k] are the eigenvalues and Q (row-major) holds
// the orthonormal eigenvectors in its columns.
void jacobi_eigen(int n, std::vector<double>& S, std::vector<double>& Q, std::vector<double>& lam) {
  Q.assign((size_t)n * n, 0.0);
  for (int k = 0; k < n; ++k) Q[(size_t)k * n + k] = 1.0;
  auto s = [&](int r, int c) -> double& { return S[(size_t)r * n + c]; };
  double total = 0.0;
  for (double v : S) total += v * v;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) off += s(p, q) * s(p, q);
    if (off <= 1e-32 * total) break;
    for (int p = 0; p < n - 1; ++p) {
      for (int q = p + 1; q < n; ++q) {
        const double apq = s(p, q);
        if (apq == 0.0) continue;
        const double theta = (s(q, q) - s(p, p)) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0);
        const double sn = t * c;
        for (int k = 0; k < n; ++k) {  // columns p, q
          const double akp = s(k, p), akq = s(k, q);
          s(k, p) = c * akp - sn * akq;
          s(k, q) = sn * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {  // rows p, q
          const double apk = s(p, k), aqk = s(q, k);
          s(p, k) = c * apk - sn * aqk;
          s(q, k) = sn * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          double& vkp = Q[(size_t)k * n + p];
          double& vkq = Q[(size_t)k * n + q];
          const double a = vkp, b = vkq;
          vkp = c * a - sn * b;
          vkq = sn * a + c * b;
        }
      }
    }
  }
  lam.resize(n);
  for (int k = 0; k < n; ++k) lam[k] = s(k, k);
}

// Eigenpairs of a dense symmetric n x n matrix S (row-major = column-major)
// on the current GPU with cuSOLVER's divide-and-conquer solver (set-up of the
// large coarse grids, where the O(n^3)-per-sweep Jacobi method takes seconds
// to minutes).  Q row-major with the eigenvectors in its columns.
void gpu_eigen(int n, const std::vector<double>& S, std::vector<double>& Q,
               std::vector<double>& lam) {
  cusolverDnHandle_t h = nullptr;
  double *dA = nullptr, *dW = nullptr, *dwork = nullptr;
  int* dinfo = nullptr;
  std::string err;
  auto cuda_ok = [&](cudaError_t e, const char* what) {
    if (e != cudaSuccess && err.empty()) err = std::string(what) + ": " + cudaGetErrorString(e);
    return err.empty();
  };
  auto solver_ok = [&](cusolverStatus_t st, const char* what) {
    if (st != CUSOLVER_STATUS_SUCCESS && err.empty())
      err = std::string(what) + " failed (status " + std::to_string((int)st) + ")";
    return err.empty();
  };
  const size_t bytes = (size_t)n * n * sizeof(double);
  int lwork = 0, info = -1;
  if (solver_ok(cusolverDnCreate(&h), "cusolverDnCreate") &&
      cuda_ok(cudaMalloc((void**)&dA, bytes), "cudaMalloc") &&
      cuda_ok(cudaMalloc((void**)&dW, (size_t)n * sizeof(double)), "cudaMalloc") &&
      cuda_ok(cudaMalloc((void**)&dinfo, sizeof(int)), "cudaMalloc") &&
      cuda_ok(cudaMemcpy(dA, S.data(), bytes, cudaMemcpyHostToDevice), "cudaMemcpy") &&
      solver_ok(cusolverDnDsyevd_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n,
                                            dA, n, dW, &lwork),
                "cusolverDnDsyevd_bufferSize") &&
      cuda_ok(cudaMalloc((void**)&dwork, (size_t)std::max(lwork, 1) * sizeof(double)),
              "cudaMalloc") &&
      solver_ok(cusolverDnDsyevd(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, dA, n, dW,
                                 dwork, lwork, dinfo),
                "cusolverDnDsyevd") &&
      cuda_ok(cudaMemcpy(&info, dinfo, sizeof(int), cudaMemcpyDeviceToHost), "cudaMemcpy")) {
    std::vector<double> A((size_t)n * n);
    lam.resize(n);
    if (cuda_ok(cudaMemcpy(A.data(), dA, bytes, cudaMemcpyDeviceToHost), "cudaMemcpy") &&
        cuda_ok(cudaMemcpy(lam.data(), dW, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost),
                "cudaMemcpy")) {
      Q.resize((size_t)n * n);
      for (int r = 0; r < n; ++r)   // column-major eigenvectors -> row-major Q
        for (int c = 0; c < n; ++c) Q[(size_t)r * n + c] = A[(size_t)c * n + r];
    }
  }
  if (dwork) cudaFree(dwork);
  if (dinfo) cudaFree(dinfo);
  if (dW) cudaFree(dW);
  if (dA) cudaFree(dA);
  if (h) cusolverDnDestroy(h);
  if (!err.empty()) throw std::runtime_error("coarse eigen-decomposition: " + err);
  if (info != 0) throw std::runtime_error("coarse eigen-decomposition did not converge");
}

// Grids up to this size take the host Jacobi eigen-solver (also used by the
// host-only entry points); larger ones the GPU solver.
constexpr int kJacobiMaxN = 257;

// Generalised eigenvectors of K v = l W v (K = -M, M row-major, W = diag(w)):
// V column-major with V^T W V = I.
void pencil_eigen(int n, const std::vector<double>& M, const std::vector<double>& w,
                  std::vector<double>& V, std::vector<double>& lam) {
  std::vector<double> S((size_t)n * n);
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c)
      S[(size_t)r * n + c] = -M[(size_t)r * n + c] / std::sqrt(w[r] * w[c]);
  // symmetrise exactly (the 1D operators are symmetric; guard the rounding)
  for (int r = 0; r < n; ++r)
    for (int c = r + 1; c < n; ++c) {
      const double a = S[(size_t)r * n + c], b = S[(size_t)c * n + r];
      if (std::fabs(a - b) > 1e-13 * (1.0 + std::fabs(a)))
        throw std::runtime_error("1D operator is not symmetric");
      S[(size_t)r * n + c] = S[(size_t)c * n + r] = 0.5 * (a + b);
    }
  std::vector<double> Q;
  if (n <= kJacobiMaxN)
    jacobi_eigen(n, S, Q, lam);
  else
    gpu_eigen(n, S, Q, lam);
  V.resize((size_t)n * n);
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) V[(size_t)c * n + r] = Q[(size_t)r * n + c] / std::sqrt(w[r]);
}

// 1D operators and norm weights of order p (p = 4, 6: the closure tables of
// sbp_high_order.cuh).
template <int P>
void one_d_high(int n, std::vector<double>& X, std::vector<double>& Y, std::vector<double>& w) {
  X.assign((size_t)n * n, 0.0);
  Y.assign((size_t)n * n, 0.0);
  ho::one_d<P>(n, X.data(), Y.data());
  w.resize(n);
  for (int k = 0; k < n; ++k) w[k] = ho::weight<P>(k, n);
}

// (-A u) from the Kronecker form: w_j (X u(:, j))_i + w_i (Y u(i, :))_j.
void kron_apply(int n, const std::vector<double>& X, const std::vector<double>& Y,
                const std::vector<double>& w, const double* u, double* out) {
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      double xi = 0.0, yj = 0.0;
      for (int k = 0; k < n; ++k) {
        xi += X[(size_t)i * n + k] * u[(size_t)j * n + k];
        yj += Y[(size_t)j * n + k] * u[(size_t)k * n + i];
      }
      out[(size_t)j * n + i] = w[j] * xi + w[i] * yj;
    }
}

std::shared_ptr<const CoarseFactors> build_factors(int nc, int p) {
  std::vector<double> X, Y, w;
  if (p == 2) {
    one_d_operators(nc, X, Y);
    check_kronecker(nc, X, Y);
    w.resize(nc);
    for (int k = 0; k < nc; ++k) w[k] = weight(k, nc);
  } else if (p == 4) {
    one_d_high<4>(nc, X, Y, w);
  } else if (p == 6) {
    one_d_high<6>(nc, X, Y, w);
  } else {
    throw std::runtime_error("SBP order must be 2, 4 or 6");
  }
  auto f = std::make_shared<CoarseFactors>();
  f->nc = nc;
  std::vector<double> lx, ly;
  pencil_eigen(nc, X, w, f->Vx, lx);
  pencil_eigen(nc, Y, w, f->Vy, ly);
  const size_t N = (size_t)nc * nc;
  f->VxT.resize(N);
  f->VyT.resize(N);
  f->dinv.resize(N);
  for (int r = 0; r < nc; ++r)
    for (int c = 0; c < nc; ++c) {
      f->VxT[(size_t)c * nc + r] = f->Vx[(size_t)r * nc + c];
      f->VyT[(size_t)c * nc + r] = f->Vy[(size_t)r * nc + c];
    }
  for (int j = 0; j < nc; ++j)
    for (int i = 0; i < nc; ++i) {
      const double d = lx[i] + ly[j];
      if (!(d > 0.0)) throw std::runtime_error("coarse operator is not positive definite");
      f->dinv[(size_t)j * nc + i] = 1.0 / d;
    }
  if (nc > kJacobiMaxN) {
    // large grids: the eigen-residuals K v = l W v of every pair and the
    // W-orthonormality of a sample of pairs (O(n^2) each; the full check
    // below is O(n^3))
    auto pencil_check = [&](const std::vector<double>& M, const std::vector<double>& V,
                            const std::vector<double>& lam) {
      double worst = 0.0;
      for (int k = 0; k < nc; ++k) {
        const double* v = V.data() + (size_t)k * nc;
        for (int r = 0; r < nc; ++r) {
          double kv = 0.0;
          for (int c = std::max(0, r - 3); c < std::min(nc, r + 4); ++c)
            kv -= M[(size_t)r * nc + c] * v[c];
          worst = std::max(worst, std::fabs(kv - lam[k] * w[r] * v[r]) /
                                      (1.0 + std::fabs(lam[k])));
        }
      }
      for (int t = 0; t < 64; ++t) {
        const int a = (int)((37u * (unsigned)t + 11u) % (unsigned)nc);
        const int c = (int)((101u * (unsigned)t + 5u) % (unsigned)nc);
        double dot = 0.0;
        for (int r = 0; r < nc; ++r)
          dot += V[(size_t)a * nc + r] * w[r] * V[(size_t)c * nc + r];
        worst = std::max(worst, std::fabs(dot - (a == c ? 1.0 : 0.0)));
      }
      return worst;
    };
    if (p != 2) throw std::runtime_error("coarse size out of range for SBP order p");
    const double ex = pencil_check(X, f->Vx, lx), ey = pencil_check(Y, f->Vy, ly);
    if (!(ex <= 1e-9) || !(ey <= 1e-9))
      throw std::runtime_error("coarse fast-diagonalisation self-check failed");
    return f;
  }
  // Self-check: A (A^{-1} b) == b on a fixed vector.
  std::vector<double> b(N), x(N);
  for (size_t k = 0; k < N; ++k) b[k] = std::sin(0.37 * (double)k + 0.11) + 0.25;
  coarse_solve_host(*f, b.data(), x.data());
  double err = 0.0, nb = 0.0;
  std::vector<double> kx;
  if (p != 2) {   // the order-p stencil's own Kronecker form (p = 2: the kernels' negA)
    kx.resize(N);
    kron_apply(nc, X, Y, w, x.data(), kx.data());
  }
  for (int j = 0; j < nc; ++j)
    for (int i = 0; i < nc; ++i) {
      struct G {
        const double* x; int i, j, n;
        double operator()(int di, int dj) const { return x[(size_t)(j + dj) * n + (i + di)]; }
      } g{x.data(), i, j, nc};
      const double ax = p == 2 ? -negA<double>(g, i, j, nc) : -kx[(size_t)j * nc + i];
      err = std::max(err, std::fabs(ax - b[(size_t)j * nc + i]));
      nb = std::max(nb, std::fabs(b[(size_t)j * nc + i]));
    }
  if (!(err <= 1e-9 * nb)) throw std::runtime_error("coarse fast-diagonalisation self-check failed");
  return f;
}

}  // namespace

void coarse_solve_host(const CoarseFactors& f, const double* b, double* x) {
  const int n = f.nc;
  const size_t N = (size_t)n * n;
  std::vector<double> t(N), y(N);
  // t = B Vy ; y = Vx^T t ./ D ; t = y Vy^T ; x = Vx t
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      double a = 0.0;
      for (int k = 0; k < n; ++k) a += b[(size_t)k * n + i] * f.Vy[(size_t)j * n + k];
      t[(size_t)j * n + i] = a;
    }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      double a = 0.0;
      for (int k = 0; k < n; ++k) a += f.VxT[(size_t)k * n + i] * t[(size_t)j * n + k];
      y[(size_t)j * n + i] = a * f.dinv[(size_t)j * n + i];
    }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      double a = 0.0;
      for (int k = 0; k < n; ++k) a += y[(size_t)k * n + i] * f.VyT[(size_t)j * n + k];
      t[(size_t)j * n + i] = a;
    }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      double a = 0.0;
      for (int k = 0; k < n; ++k) a += f.Vx[(size_t)k * n + i] * t[(size_t)j * n + k];
      x[(size_t)j * n + i] = a;
    }
}

std::shared_ptr<const CoarseFactors> coarse_factors(int nc, int p) {
  const int lo = p == 2 ? 3 : ho_min_points(p);
  if (lo == 0 || nc < lo || nc > kCoarseMaxN || (p != 2 && nc > kJacobiMaxN))
    throw std::runtime_error("coarse size out of range");
  static std::mutex mu;
  static std::map<std::pair<int, int>, std::shared_ptr<const CoarseFactors>> cache;
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find({nc, p});
  if (it != cache.end()) return it->second;
  auto f = build_factors(nc, p);
  cache[{nc, p}] = f;
  return f;
}

int ho_min_points(int p) {
  return p == 4 ? ho::Order<4>::kMinN : (p == 6 ? ho::Order<6>::kMinN : 0);
}

std::shared_ptr<const std::vector<double>> coarse_inverse(int nc, int p) {
  auto f = coarse_factors(nc, p);
  const int N = nc * nc;
  auto X = std::make_shared<std::vector<double>>((size_t)N * N, 0.0);
  unsigned nt = std::max(1u, std::thread::hardware_concurrency());
  nt = std::min(nt, 64u);
  auto worker = [&](unsigned t) {
    std::vector<double> e(N, 0.0), x(N);
    for (int c = (int)t; c < N; c += (int)nt) {
      e[c] = 1.0;
      coarse_solve_host(*f, e.data(), x.data());
      e[c] = 0.0;
      for (int k = 0; k < N; ++k) (*X)[(size_t)k * N + c] = x[k];
    }
  };
  std::vector<std::thread> th;
  for (unsigned t = 1; t < nt; ++t) th.emplace_back(worker, t);
  worker(0);
  for (auto& t : th) t.join();
  // exact symmetry (A^{-1} is symmetric; the columns differ by rounding)
  for (int r = 0; r < N; ++r)
    for (int c = r + 1; c < N; ++c) {
      const double v = 0.5 * ((*X)[(size_t)r * N + c] + (*X)[(size_t)c * N + r]);
      (*X)[(size_t)r * N + c] = (*X)[(size_t)c * N + r] = v;
    }
  return X;
}

}  // namespace sbp

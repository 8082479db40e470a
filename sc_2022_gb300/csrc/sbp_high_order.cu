// Higher-order (p = 4, 6) SBP-SAT kernels, FP64, on contiguous n x n grids.
//
// One kernel template covers the operator's three uses:
// - the apply (out = sign * A u, optionally u . out into the Krylov state);
// - the residual (out = b - A u, optionally ||out||^2);
// - a weighted-Jacobi sweep (out = u + omega D^-1 (b - A u)).
// The reference builds these operators only as assembled CPU matrices
// (Operators_2d / Assembling_matrix with p = 4, 6,
// level_2_multigrid_new.jl:48-188) and smooths with weighted Jacobi in its
// CPU multigrid preconditioner (precond_matrix, initial_guess_cg.jl:458-510).
//
// Access pattern: each thread owns a row i and marches along j over a run of
// columns, keeping the 2R+1 columns of its own row that the j-direction
// stencil needs in registers.  The i-neighbours come from the cache: a warp
// covers 32 consecutive rows of a column, so those loads are coalesced.
// Boundary rows and columns (the first and last bm) apply the bm x bn closure
// tables from constant memory.
#include <algorithm>
#include <mutex>

#include "sbp_high_order.cuh"
#include "sbp_kernels.cuh"
#include "sbp_launch.h"

namespace sbp {

namespace {

__constant__ double c_ho4[2][4 * 6];   // [X | Y][r * bn + c]
__constant__ double c_ho6[2][6 * 9];
__constant__ float c_ho4f[2][4 * 6];   // the same, rounded to FP32
__constant__ float c_ho6f[2][6 * 9];

template <int P, typename T>
__device__ __forceinline__ const T* tab(int which);
template <>
__device__ __forceinline__ const double* tab<4, double>(int which) {
  return c_ho4[which];
}
template <>
__device__ __forceinline__ const double* tab<6, double>(int which) {
  return c_ho6[which];
}
template <>
__device__ __forceinline__ const float* tab<4, float>(int which) {
  return c_ho4f[which];
}
template <>
__device__ __forceinline__ const float* tab<6, float>(int which) {
  return c_ho6f[which];
}

__device__ __forceinline__ double fmaT(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fmaT(float a, float b, float c) { return fmaf(a, b, c); }

template <int P, int MODE, bool DOT, typename T>
__global__ void __launch_bounds__(kThreads) k_ho(const HoArgsT<T> a) {
  using O = ho::Order<P>;
  constexpr int R = O::kHalf, W = 2 * R + 1, BM = O::kBm, BN = O::kBn;
  // interior A diagonal is -2 d(0); its reciprocal needs no division
  constexpr T kInvDiagIn = T(-0.5 / O::d(0));
  constexpr T kD0 = T(O::d(0)), kD1 = T(O::d(1)), kD2 = T(O::d(2)), kD3 = T(O::d(3 % (R + 1)));
  auto dk = [](int k) { return k == 1 ? kD1 : (k == 2 ? kD2 : kD3); };
  pdl_begin();
  if (a.st && a.st->done) return;
  const int n = a.n;
  const int cols = a.cols;
  const int nrb = (n + kThreads - 1) / kThreads;
  const int items = nrb * ((n + cols - 1) / cols);
  const T* __restrict__ u = a.u;
  const T* __restrict__ b = a.b;
  T* __restrict__ out = a.out;
  const T* tx = tab<P, T>(0);
  const T* ty = tab<P, T>(1);
  const T omega = T(a.omega);
  const T winv_in = omega * kInvDiagIn;   // the interior Jacobi factor
  DotAcc<T> acc;
  for (int w = blockIdx.x; w < items; w += gridDim.x) {
    const int i = (w % nrb) * kThreads + threadIdx.x;
    if (i >= n) continue;
    const int j0 = (w / nrb) * cols;
    const int j1 = min(n, j0 + cols);
    const T wi = T(ho::weight<P>(i, n));
    const bool xin = i >= BM && i <= n - 1 - BM;
    const bool xlo = i < BM;
    const int xr = xlo ? i : n - 1 - i;   // closure row when !xin
    const T dxx = xin ? kD0 : tx[xr * BN + xr];
    if (MODE == kHoJacobi && a.zero_in) {
      // first sweep from v = 0: out = omega D^-1 b
      for (int j = j0; j < j1; ++j) {
        const bool yin = j >= BM && j <= n - 1 - BM;
        const int yr = j < BM ? j : n - 1 - j;
        const T dyy = yin ? kD0 : ty[yr * BN + yr];
        const T winv =
            a.richardson ? omega
            : (xin && yin) ? winv_in
                           : omega * (T(-1) / (T(ho::weight<P>(j, n)) * dxx + wi * dyy));
        out[(size_t)j * n + i] = winv * __ldg(b + (size_t)j * n + i);
      }
      continue;
    }
    const T* row = u + i;
    auto at = [&](int ii, int jj) { return __ldg(u + (size_t)jj * n + ii); };
    auto col = [&](int jj) { return (jj >= 0 && jj < n) ? __ldg(row + (size_t)jj * n) : T(0); };
    T c[W];
#pragma unroll
    for (int k = 0; k < W - 1; ++k) c[k] = col(j0 - R + k);
    // chunks of kHoChunk columns: the chunk's window columns and right-hand
    // sides are loaded together, so a warp keeps several DRAM lines in flight
    // (p = 6: the wider window and closures leave no registers for it;
    // measured slower)
    constexpr int kHoChunk = P == 4 ? 4 : 1;
    for (int jc = j0; jc < j1; jc += kHoChunk) {
      T cn[kHoChunk], bn[kHoChunk];
  #pragma unroll
      for (int q = 0; q < kHoChunk; ++q) {
        cn[q] = col(jc + q + R);
        bn[q] = (MODE != kHoApply && jc + q < j1) ? __ldg(b + (size_t)(jc + q) * n + i) : T(0);
      }
  #pragma unroll
      for (int q = 0; q < kHoChunk; ++q) {
        const int j = jc + q;
        if (j >= j1) break;
        c[W - 1] = cn[q];
        const bool yin = j >= BM && j <= n - 1 - BM;
        const bool ylo = j < BM;
        const int yr = ylo ? j : n - 1 - j;
        const T wj = T(ho::weight<P>(j, n));
        T na;   // (-A u)(i, j)
        // (p = 6 in FP32 keeps the two directions apart: measured faster)
        if (xin && yin && (sizeof(T) == 8 || P == 4)) {
          // interior: both weights are 1 and the directions share d_k, so
          // -A u = 2 d_0 u + sum_k d_k (u(i-k) + u(i+k) + u(j-k) + u(j+k))
          na = (T(2) * kD0) * c[R];
  #pragma unroll
          for (int k = 1; k <= R; ++k)
            na = fmaT(dk(k), (at(i - k, j) + at(i + k, j)) + (c[R - k] + c[R + k]), na);
        } else {
          T xi;
          if (xin) {
            xi = kD0 * c[R];
  #pragma unroll
            for (int k = 1; k <= R; ++k) xi = fmaT(dk(k), at(i - k, j) + at(i + k, j), xi);
          } else {
            xi = T(0);
  #pragma unroll
            for (int q = 0; q < BN; ++q)
              xi = fmaT(tx[xr * BN + q], at(xlo ? q : n - 1 - q, j), xi);
          }
          T yj;
          if (yin) {
            yj = kD0 * c[R];
  #pragma unroll
            for (int k = 1; k <= R; ++k) yj = fmaT(dk(k), c[R - k] + c[R + k], yj);
          } else {
            yj = T(0);
  #pragma unroll
            for (int q = 0; q < BN; ++q)
              yj = fmaT(ty[yr * BN + q], col(ylo ? q : n - 1 - q), yj);
          }
          na = fmaT(wj, xi, wi * yj);
        }
        T v;
        if (MODE == kHoApply) {
          v = a.sign > 0 ? -na : na;
        } else if (MODE == kHoResid) {
          v = bn[q] + (a.sign > 0 ? na : -na);
        } else {
          T winv = omega;   // omega D^-1 (Jacobi) or omega (Richardson)
          if (!a.richardson) {
            const T dyy = yin ? kD0 : ty[yr * BN + yr];
            winv = (xin && yin) ? winv_in : omega * (T(-1) / (wj * dxx + wi * dyy));
          }
          v = fmaT(winv, bn[q] + na, c[R]);
        }
        out[(size_t)j * n + i] = v;
        if (DOT) acc.add_prod(MODE == kHoApply ? c[R] : v, v);
  #pragma unroll
        for (int k = 0; k < W - 1; ++k) c[k] = c[k + 1];
      }
    }
  }
  if (DOT)
    grid_reduce(acc.value(), a.rb, [&](double tot) {
      if (a.dot_out) *a.dot_out = tot;
      SolveState* st = a.st;
      if (!st) return;
      if (MODE == kHoApply) {   // CG: p.Ap -> alpha
        st->pAp = tot;
        if (!isfinite(tot) || tot == 0.0)
          st->done = kDoneBreakdown;
        else
          st->alpha = st->rz / tot;
      } else if (MODE == kHoResid && a.init) {   // Krylov set-up from ||r0||^2
        st->rr0 = st->rr = tot;
        st->rz = tot;
        st->thresh2 = a.abstol > 0.0 ? a.abstol * a.abstol : a.reltol * a.reltol * tot;
        st->iter = 0;
        if (a.norms) a.norms[0] = sqrt(tot);
        if (!isfinite(tot))
          st->done = kDoneBreakdown;
        else if (tot < st->thresh2 || tot == 0.0)
          st->done = kDoneConverged;
        else if (st->maxiter <= 0)
          st->done = kDoneMaxIter;
      }
    });
}

// r.z into the Krylov state: beta = rz_new / rz (0 on the first direction).
template <typename Tz>
__global__ void __launch_bounds__(kThreads)
    k_ho_rz(const double* __restrict__ r, const Tz* __restrict__ z, long long N,
            SolveState* st, ReduceBuf rb, int first) {
  pdl_begin();
  if (st->done) return;
  double acc = 0.0;
  for (long long k = (long long)blockIdx.x * kThreads + threadIdx.x; k < N;
       k += (long long)gridDim.x * kThreads)
    acc = fma(__ldg(r + k), convert<double>(__ldg(z + k)), acc);
  grid_reduce(acc, rb, [&](double tot) {
    st->beta = first ? 0.0 : tot / st->rz;
    st->rz = tot;
    if (!isfinite(tot) || tot <= 0.0) st->done = kDoneBreakdown;
  });
}

// p = z + beta p (p = z on the first direction).
template <typename Tz>
__global__ void __launch_bounds__(kThreads)
    k_ho_dir(const Tz* __restrict__ z, double* __restrict__ p, long long N,
             const SolveState* st, int first) {
  pdl_begin();
  if (st->done) return;
  const double beta = st->beta;
  for (long long k = (long long)blockIdx.x * kThreads + threadIdx.x; k < N;
       k += (long long)gridDim.x * kThreads) {
    const double zk = convert<double>(__ldg(z + k));
    p[k] = first ? zk : fma(beta, p[k], zk);
  }
}

// Mixed-precision CG direction for the order-p operator (z = the FP32
// V-cycle output, p and Ap FP64, both updated in place):
//   p  = z + beta p          Ap = A z + beta Ap          p.Ap -> alpha
// A p by linearity, so the FP64 apply (12 to 16 FP64 instructions per
// point) becomes A z on the FP32 pipe plus three FP64 instructions.  At
// interior points A z is summed in float-float: each coefficient d_k is an
// unevaluated float pair, the products are exact on the high part, and the
// sums use two_sum.  The result is within about 2^-45 of the largest term.
// Closure rows and columns (2 bm of n each way) use FP64 on the exact FP32
// values.  p.Ap comes from the FP32 roundings with compensated accumulation
// (alpha needs ~1e-7; the FP64 recurrences keep their accuracy).
template <int P>
__global__ void __launch_bounds__(kThreads)
    k_ho_dir_mixed(const float* __restrict__ z, double* __restrict__ p, double* __restrict__ ap,
                   int n, int cols, SolveState* st, ReduceBuf rb) {
  using O = ho::Order<P>;
  constexpr int R = O::kHalf, W = 2 * R + 1, BM = O::kBm, BN = O::kBn;
  pdl_begin();
  if (st->done) return;
  const bool first = st->iter == 0;
  const double beta = st->beta;
  const int nrb = (n + kThreads - 1) / kThreads;
  const int items = nrb * ((n + cols - 1) / cols);
  const double* tx = tab<P, double>(0);
  const double* ty = tab<P, double>(1);
  // d_k as float pairs (folded at compile time); the centre weight is 2 d_0
  auto dhi = [](int k) { return k == 0 ? (float)(2.0 * O::d(0)) : (float)O::d(k); };
  auto dlo = [](int k) {
    const double d = k == 0 ? 2.0 * O::d(0) : O::d(k);
    return (float)(d - (double)(float)d);
  };
  DotAcc<float> acc;
  for (int w = blockIdx.x; w < items; w += gridDim.x) {
    const int i = (w % nrb) * kThreads + threadIdx.x;
    if (i >= n) continue;
    const int j0 = (w / nrb) * cols;
    const int j1 = min(n, j0 + cols);
    const double wi = ho::weight<P>(i, n);
    const bool xin = i >= BM && i <= n - 1 - BM;
    const bool xlo = i < BM;
    const int xr = xlo ? i : n - 1 - i;
    const float* row = z + i;
    auto at = [&](int ii, int jj) { return __ldg(z + (size_t)jj * n + ii); };
    auto col = [&](int jj) { return (jj >= 0 && jj < n) ? __ldg(row + (size_t)jj * n) : 0.0f; };
    float c[W];
#pragma unroll
    for (int k = 0; k < W - 1; ++k) c[k] = col(j0 - R + k);
    for (int j = j0; j < j1; ++j) {
      c[W - 1] = col(j + R);
      const bool yin = j >= BM && j <= n - 1 - BM;
      double azd;   // (A z)(i, j)
      if (xin && yin) {
        // sum_k d_k (z(i-k) + z(i+k) + z(j-k) + z(j+k)) + 2 d_0 z, float-float
        float hi, lo;
        {
          const float z0 = c[R];
          hi = dhi(0) * z0;
          lo = fmaf(dhi(0), z0, -hi);
          lo = fmaf(dlo(0), z0, lo);
        }
#pragma unroll
        for (int k = 1; k <= R; ++k) {
          float a, ea, b, eb, sk, es;
          two_sum(at(i - k, j), at(i + k, j), a, ea);
          two_sum(c[R - k], c[R + k], b, eb);
          two_sum(a, b, sk, es);
          const float sl = es + (ea + eb);
          const float pr = dhi(k) * sk;
          float e = fmaf(dhi(k), sk, -pr);
          e = fmaf(dhi(k), sl, e);
          e = fmaf(dlo(k), sk, e);
          float t, te;
          two_sum(hi, pr, t, te);
          hi = t;
          lo += te + e;
        }
        azd = -(f32_to_f64(hi) + f32_to_f64(lo));   // A z = -(-A z)
      } else {
        // closure rows / columns: the FP64 formula on the exact FP32 values
        double xi;
        if (xin) {
          xi = O::d(0) * f32_to_f64(c[R]);
#pragma unroll
          for (int k = 1; k <= R; ++k)
            xi = fma(O::d(k), f32_to_f64(at(i - k, j)) + f32_to_f64(at(i + k, j)), xi);
        } else {
          xi = 0.0;
#pragma unroll
          for (int q = 0; q < BN; ++q)
            xi = fma(tx[xr * BN + q], f32_to_f64(at(xlo ? q : n - 1 - q, j)), xi);
        }
        const bool ylo = j < BM;
        const int yr = ylo ? j : n - 1 - j;
        double yj;
        if (yin) {
          yj = O::d(0) * f32_to_f64(c[R]);
#pragma unroll
          for (int k = 1; k <= R; ++k)
            yj = fma(O::d(k), f32_to_f64(c[R - k]) + f32_to_f64(c[R + k]), yj);
        } else {
          yj = 0.0;
#pragma unroll
          for (int q = 0; q < BN; ++q)
            yj = fma(ty[yr * BN + q], f32_to_f64(col(ylo ? q : n - 1 - q)), yj);
        }
        azd = -fma(ho::weight<P>(j, n), xi, wi * yj);
      }
      const size_t k = (size_t)j * n + i;
      const double zd = f32_to_f64(c[R]);
      const double pv = first ? zd : fma(beta, p[k], zd);
      const double av = first ? azd : fma(beta, ap[k], azd);
      p[k] = pv;
      ap[k] = av;
      acc.add_prod(f64_to_f32(pv), f64_to_f32(av));
#pragma unroll
      for (int q = 0; q < W - 1; ++q) c[q] = c[q + 1];
    }
  }
  grid_reduce(acc.value(), rb, [&](double tot) {
    st->pAp = tot;
    if (!isfinite(tot) || tot == 0.0)
      st->done = kDoneBreakdown;
    else
      st->alpha = st->rz / tot;
  });
}

int flat_ctas(long long N) {
  const long long want = (N + (long long)kThreads * 4 - 1) / ((long long)kThreads * 4);
  return (int)std::max(1LL, std::min<long long>(want, kMaxPersistCtas));
}

template <int P>
void fill_tables(double* x, double* y) {
  using O = ho::Order<P>;
  for (int r = 0; r < O::kBm; ++r)
    for (int c = 0; c < O::kBn; ++c) {
      x[r * O::kBn + c] = ho::x_coef<P>(r, c);
      y[r * O::kBn + c] = ho::y_coef<P>(r, c);
    }
}

template <int P, int MODE, typename T>
cudaError_t launch_mode(const HoArgsT<T>& a, dim3 grid, cudaStream_t s) {
  if (a.rb.partials)
    return launch_pdl(k_ho<P, MODE, true, T>, grid, dim3(kThreads), 0, s, a);
  return launch_pdl(k_ho<P, MODE, false, T>, grid, dim3(kThreads), 0, s, a);
}

template <int P, typename T>
cudaError_t launch_order(int mode, const HoArgsT<T>& a, dim3 grid, cudaStream_t s) {
  switch (mode) {
    case kHoApply: return launch_mode<P, kHoApply>(a, grid, s);
    case kHoResid: return launch_mode<P, kHoResid>(a, grid, s);
    case kHoJacobi: return launch_mode<P, kHoJacobi>(a, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

int ho_min_n(int p) {
  return p == 4 ? ho::Order<4>::kMinN : (p == 6 ? ho::Order<6>::kMinN : 0);
}

cudaError_t prepare_ho_tables() {
  static std::once_flag once;
  static cudaError_t err = cudaSuccess;
  std::call_once(once, [] {
    double t4[2][4 * 6], t6[2][6 * 9];
    float f4[2][4 * 6], f6[2][6 * 9];
    fill_tables<4>(t4[0], t4[1]);
    fill_tables<6>(t6[0], t6[1]);
    for (int w = 0; w < 2; ++w) {
      for (int k = 0; k < 4 * 6; ++k) f4[w][k] = (float)t4[w][k];
      for (int k = 0; k < 6 * 9; ++k) f6[w][k] = (float)t6[w][k];
    }
    err = cudaMemcpyToSymbol(c_ho4, t4, sizeof(t4));
    if (err == cudaSuccess) err = cudaMemcpyToSymbol(c_ho6, t6, sizeof(t6));
    if (err == cudaSuccess) err = cudaMemcpyToSymbol(c_ho4f, f4, sizeof(f4));
    if (err == cudaSuccess) err = cudaMemcpyToSymbol(c_ho6f, f6, sizeof(f6));
  });
  return err;
}

int ho_cols(int n) {
  // columns per work item: enough items to fill the GPU on small grids,
  // long column runs (fewer window refills) on large ones
  const long long nrb = (n + kThreads - 1) / kThreads;
  const long long c = (long long)n * nrb / (2LL * 152);
  return (int)std::max(1LL, std::min(32LL, c));
}

template <typename T>
cudaError_t launch_ho(int p, int mode, HoArgsT<T> a, cudaStream_t s) {
  if (ho_min_n(p) == 0 || a.n < ho_min_n(p) || !a.out) return cudaErrorInvalidValue;
  if (a.cols <= 0) a.cols = ho_cols(a.n);
  const long long nrb = (a.n + kThreads - 1) / kThreads;
  const long long items = nrb * ((a.n + a.cols - 1) / a.cols);
  const dim3 grid((unsigned)std::min<long long>(items, kMaxPersistCtas));
  return p == 4 ? launch_order<4>(mode, a, grid, s) : launch_order<6>(mode, a, grid, s);
}

template <typename Tz>
cudaError_t launch_ho_rz(const double* r, const Tz* z, long long N, SolveState* st,
                         ReduceBuf rb, int first, cudaStream_t s) {
  return launch_pdl(k_ho_rz<Tz>, dim3(flat_ctas(N)), dim3(kThreads), 0, s, r, z, N, st, rb,
                    first);
}

template <typename Tz>
cudaError_t launch_ho_dir(const Tz* z, double* p, long long N, const SolveState* st,
                          int first, cudaStream_t s) {
  return launch_pdl(k_ho_dir<Tz>, dim3(flat_ctas(N)), dim3(kThreads), 0, s, z, p, N, st, first);
}

cudaError_t launch_ho_dir_mixed(int p, const float* z, double* pd, double* ap, int n,
                                SolveState* st, ReduceBuf rb, cudaStream_t s) {
  if (ho_min_n(p) == 0 || n < ho_min_n(p) || !rb.partials) return cudaErrorInvalidValue;
  const int cols = ho_cols(n);
  const long long nrb = (n + kThreads - 1) / kThreads;
  const long long items = nrb * ((n + cols - 1) / cols);
  const dim3 grid((unsigned)std::min<long long>(items, kMaxPersistCtas));
  if (p == 4)
    return launch_pdl(k_ho_dir_mixed<4>, grid, dim3(kThreads), 0, s, z, pd, ap, n, cols, st, rb);
  return launch_pdl(k_ho_dir_mixed<6>, grid, dim3(kThreads), 0, s, z, pd, ap, n, cols, st, rb);
}

template cudaError_t launch_ho<double>(int, int, HoArgsT<double>, cudaStream_t);
template cudaError_t launch_ho<float>(int, int, HoArgsT<float>, cudaStream_t);
template cudaError_t launch_ho_rz<double>(const double*, const double*, long long, SolveState*,
                                          ReduceBuf, int, cudaStream_t);
template cudaError_t launch_ho_rz<float>(const double*, const float*, long long, SolveState*,
                                         ReduceBuf, int, cudaStream_t);
template cudaError_t launch_ho_dir<double>(const double*, double*, long long, const SolveState*,
                                           int, cudaStream_t);
template cudaError_t launch_ho_dir<float>(const float*, double*, long long, const SolveState*,
                                          int, cudaStream_t);

}  // namespace sbp

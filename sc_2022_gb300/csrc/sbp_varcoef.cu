// Variable-coefficient (div(c grad u)) second-order SBP-SAT kernels.
//
// - k_vc_apply_c: -A u straight from the nodal coefficients.  It is the
//   standalone apply and reads u, c and writes out: 24 bytes per point in
//   FP64.
// - k_vc_stencil: the per-point stencil arrays E, N, D (and omega / D for
//   the Jacobi sweeps) and the boundary couplings Flo / Fhi of sbp_varcoef.cuh,
//   computed once per level from c.
// - k_vc<MODE>: the solver's apply / residual / Jacobi sweep on those
//   arrays, in FP64 or FP32.  Five multiply-adds per point instead of the
//   face averages.
// - k_vc_coarsen: the coarse coefficients, a full-weighting harmonic mean.
// - k_dense_gemv: the coarse direct solve, x = A^-1 b with a dense inverse.
// The access pattern is that of the other stencil kernels: a row per thread,
// a march along j with the row's own values in registers, and i-neighbours
// from the cache (a warp covers 32 consecutive rows of a column).
#include <algorithm>

#include "sbp_kernels.cuh"
#include "sbp_launch.h"
#include "sbp_varcoef.cuh"

namespace sbp {

namespace {

__device__ __forceinline__ double fmaT(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fmaT(float a, float b, float c) { return fmaf(a, b, c); }

int vc_cols(int n) {
  const long long nrb = (n + kThreads - 1) / kThreads;
  const long long c = (long long)n * nrb / (2LL * 152);
  return (int)std::max(1LL, std::min(32LL, c));
}

dim3 vc_grid(int n, int cols) {
  const long long nrb = (n + kThreads - 1) / kThreads;
  const long long items = nrb * ((n + cols - 1) / cols);
  return dim3((unsigned)std::min<long long>(items, kMaxPersistCtas));
}

// out = sign * A u from nodal c (FP64); dot: u . out.
template <bool DOT>
__global__ void __launch_bounds__(kThreads)
    k_vc_apply_c(const double* __restrict__ u, const double* __restrict__ c,
                 double* __restrict__ out, int n, int sign, int cols, ReduceBuf rb,
                 double* dot_out) {
  pdl_begin();
  const int nrb = (n + kThreads - 1) / kThreads;
  const int items = nrb * ((n + cols - 1) / cols);
  double acc = 0.0;
  for (int w = blockIdx.x; w < items; w += gridDim.x) {
    const int i = (w % nrb) * kThreads + threadIdx.x;
    if (i >= n) continue;
    const int j0 = (w / nrb) * cols;
    const int j1 = min(n, j0 + cols);
    const double wi = vc::weight(i, n);
    auto U = [&](int ii, int jj) { return __ldg(u + (size_t)jj * n + ii); };
    auto Cf = [&](int ii, int jj) { return __ldg(c + (size_t)jj * n + ii); };
    // register window along j: u and c at j-1, j, j+1; the face sum
    // c(j) + c(j+1) is carried to the next column as c(j-1) + c(j).  Face
    // sums enter unhalved and the 1/2 is applied once per direction.
    double um = j0 > 0 ? U(i, j0 - 1) : 0.0, u0 = U(i, j0);
    double c0 = Cf(i, j0);
    double sm = j0 > 0 ? Cf(i, j0 - 1) + c0 : 0.0;   // c(j-1) + c(j)
    for (int j = j0; j < j1; ++j) {
      const double up = j + 1 < n ? U(i, j + 1) : 0.0;
      const double cp = j + 1 < n ? Cf(i, j + 1) : 0.0;
      const double sp = c0 + cp;                       // c(j) + c(j+1)
      double x = 0.0;
      if (i > 0) x = (Cf(i - 1, j) + c0) * (U(i - 1, j) - u0);
      if (i < n - 1) x = fma(c0 + Cf(i + 1, j), U(i + 1, j) - u0, x);
      double y = 0.0;
      if (j > 0) y = sm * (um - u0);
      if (j < n - 1) y = fma(sp, up - u0, y);
      y *= 0.5;
      if (j <= 2 || j >= n - 3) {   // Dirichlet closure, scaled by the boundary c
        if (j == 0)
          y += c0 * (vc::kBs0 * u0 + vc::kBs1 * up + vc::kBs2 * U(i, 2) +
                     (vc::kTauDh + vc::kBs0) * u0);
        if (j == n - 1)
          y += c0 * (vc::kBs0 * u0 + vc::kBs1 * um + vc::kBs2 * U(i, n - 3) +
                     (vc::kTauDh + vc::kBs0) * u0);
        if (j == 1) y += vc::kBs1 * Cf(i, 0) * U(i, 0);
        if (j == 2) y += vc::kBs2 * Cf(i, 0) * U(i, 0);
        if (j == n - 2) y += vc::kBs1 * Cf(i, n - 1) * U(i, n - 1);
        if (j == n - 3) y += vc::kBs2 * Cf(i, n - 1) * U(i, n - 1);
      }
      const double na = fma(0.5 * vc::weight(j, n), x, wi * y);   // (-A u)(i, j)
      const double v = sign > 0 ? -na : na;
      out[(size_t)j * n + i] = v;
      if (DOT) acc = fma(u0, v, acc);
      um = u0;
      u0 = up;
      c0 = cp;
      sm = sp;
    }
  }
  if (DOT) grid_reduce(acc, rb, [&](double tot) { *dot_out = tot; });
}

// Stencil arrays of one level from its nodal coefficients.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_vc_stencil(const double* __restrict__ c, T* __restrict__ E, T* __restrict__ N,
                 T* __restrict__ D, T* __restrict__ flo, T* __restrict__ fhi,
                 T* __restrict__ Dinv, double wscale, int n) {
  const long long total = (long long)n * n;
  struct Acc {
    const double* c;
    int n;
    __device__ double operator()(int i, int j) const { return __ldg(c + (size_t)j * n + i); }
  } acc{c, n};
  for (long long k = (long long)blockIdx.x * kThreads + threadIdx.x; k < total;
       k += (long long)gridDim.x * kThreads) {
    const int i = (int)(k % n), j = (int)(k / n);
    double e, nn, d;
    vc::coefficients(acc, i, j, n, e, nn, d);
    E[k] = (T)e;
    N[k] = (T)nn;
    D[k] = (T)d;
    Dinv[k] = (T)(wscale / d);
    if (j == 0) flo[i] = (T)vc::f_lo(acc(i, 0), i, n);
    if (j == n - 1) fhi[i] = (T)vc::f_hi(acc(i, n - 1), i, n);
  }
}

// cc(I, J) = vc::coarse_coefficient(cf, nc, I, J); the host entry point
// sbp_vc_coarsen_host gives the same bits.
__global__ void __launch_bounds__(kThreads)
    k_vc_coarsen(const double* __restrict__ cf, double* __restrict__ cc, int nc) {
  const long long total = (long long)nc * nc;
  for (long long k = (long long)blockIdx.x * kThreads + threadIdx.x; k < total;
       k += (long long)gridDim.x * kThreads) {
    const int I = (int)(k % nc), J = (int)(k / nc);
    cc[k] = vc::coarse_coefficient(cf, nc, I, J);
  }
}

template <int MODE, bool DOT, typename T>
__global__ void __launch_bounds__(kThreads) k_vc(const VcArgsT<T> a) {
  pdl_begin();
  if (a.st && a.st->done) return;
  const int n = a.n, cols = a.cols;
  const int nrb = (n + kThreads - 1) / kThreads;
  const int items = nrb * ((n + cols - 1) / cols);
  const T* __restrict__ u = a.u;
  const T* __restrict__ b = a.b;
  const T* __restrict__ E = a.E;
  const T* __restrict__ Nc = a.N;
  const T* __restrict__ D = a.D;
  const T* __restrict__ Dinv = a.Dinv;
  // a Jacobi sweep reads omega / D instead of D: (1 - omega) u + omega D^-1 (b + neighbours)
  const bool jac = MODE == kHoJacobi && !a.richardson;
  T* __restrict__ out = a.out;
  const T omega = T(a.omega);
  DotAcc<T> acc;
  for (int w = blockIdx.x; w < items; w += gridDim.x) {
    const int i = (w % nrb) * kThreads + threadIdx.x;
    if (i >= n) continue;
    const int j0 = (w / nrb) * cols;
    const int j1 = min(n, j0 + cols);
    if (MODE == kHoJacobi && a.zero_in) {   // first sweep from v = 0
      for (int j = j0; j < j1; ++j) {
        const size_t k = (size_t)j * n + i;
        out[k] = a.richardson ? omega * __ldg(b + k) : __ldg(b + k) * __ldg(Dinv + k);
      }
      continue;
    }
    const T flo = __ldg(a.flo + i), fhi = __ldg(a.fhi + i);
    auto U = [&](int ii, int jj) { return __ldg(u + (size_t)jj * n + ii); };
    T um = j0 > 0 ? U(i, j0 - 1) : T(0), u0 = U(i, j0);
    T nm = j0 > 0 ? __ldg(Nc + (size_t)(j0 - 1) * n + i) : T(0);
    // chunks of kVcChunk columns: the chunk's own-row loads are issued
    // together, so a warp keeps several DRAM lines in flight
    constexpr int kVcChunk = 4;
    for (int jc = j0; jc < j1; jc += kVcChunk) {
      T upc[kVcChunk], nc[kVcChunk], dc[kVcChunk], ec[kVcChunk], bc[kVcChunk];
  #pragma unroll
      for (int q = 0; q < kVcChunk; ++q) {
        const int j = jc + q;
        const bool in = j < j1;
        const size_t k = (size_t)j * n + i;
        upc[q] = (in && j + 1 < n) ? U(i, j + 1) : T(0);
        nc[q] = in ? __ldg(Nc + k) : T(0);
        dc[q] = in ? __ldg((jac ? Dinv : D) + k) : T(0);
        ec[q] = (in && i < n - 1) ? __ldg(E + k) : T(0);
        bc[q] = (in && MODE != kHoApply) ? __ldg(b + k) : T(0);
      }
  #pragma unroll
      for (int q = 0; q < kVcChunk; ++q) {
        const int j = jc + q;
        if (j >= j1) break;
        const size_t k = (size_t)j * n + i;
        const T up = upc[q];
        const T n0 = nc[q];
        const T d = dc[q];
        // neighbours; the diagonal term joins below (d holds omega / D on a Jacobi sweep)
        T na = jac ? T(0) : -d * u0;
        na = fmaT(nm, um, na);
        na = fmaT(n0, up, na);
        if (i > 0) na = fmaT(__ldg(E + k - 1), U(i - 1, j), na);
        if (i < n - 1) na = fmaT(ec[q], U(i + 1, j), na);
        if (j <= 2 || j >= n - 3) {
          if (j == 0) na = fmaT(flo, U(i, 2), na);
          if (j == 2) na = fmaT(flo, U(i, 0), na);
          if (j == n - 1) na = fmaT(fhi, U(i, n - 3), na);
          if (j == n - 3) na = fmaT(fhi, U(i, n - 1), na);
        }
        T v;
        if (MODE == kHoApply) {
          v = a.sign > 0 ? -na : na;
        } else if (MODE == kHoResid) {
          v = bc[q] + (a.sign > 0 ? na : -na);
        } else if (jac) {
          v = fmaT(d, bc[q] + na, (T(1) - omega) * u0);   // d = omega / D
        } else {
          v = fmaT(omega, bc[q] + na, u0);
        }
        out[k] = v;
        if (DOT) acc.add_prod(MODE == kHoApply ? u0 : v, v);
        um = u0;
        u0 = up;
        nm = n0;
      }
    }
  }
  if (DOT)
    grid_reduce(acc.value(), a.rb, [&](double tot) {
      if (a.dot_out) *a.dot_out = tot;
      SolveState* st = a.st;
      if (!st) return;
      if (MODE == kHoApply) {
        st->pAp = tot;
        if (!isfinite(tot) || tot == 0.0)
          st->done = kDoneBreakdown;
        else
          st->alpha = st->rz / tot;
      } else if (MODE == kHoResid && a.init) {
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

// Split FP64 stencil coefficients into float pairs (hi = nearest float, lo =
// the nearest float of the remainder): the coefficients of the mixed CG
// direction, to about 2^-48.
__global__ void __launch_bounds__(kThreads)
    k_split_pairs(const double* __restrict__ in, float2* __restrict__ out, long long count) {
  for (long long k = (long long)blockIdx.x * kThreads + threadIdx.x; k < count;
       k += (long long)gridDim.x * kThreads) {
    const double d = in[k];
    const float hi = __double2float_rn(d);
    out[k] = make_float2(hi, __double2float_rn(d - (double)hi));
  }
}

// acc += c * z for a coefficient pair c and an FP32 value z, in float-float.
__device__ __forceinline__ void ff_fma(float2 c, float z, float& hi, float& lo) {
  const float p = c.x * z;
  const float e = fmaf(c.y, z, fmaf(c.x, z, -p));
  float s, t;
  two_sum(hi, p, s, t);
  hi = s;
  lo += t + e;
}

// Mixed-precision CG direction of the variable-coefficient operator, in
// place (z the FP32 V-cycle output, p and Ap FP64):
//   p = z + beta p,  Ap = A z + beta Ap,  p.Ap -> alpha
// A z = D z - (the couplings of z) from the stencil as float pairs, summed in
// float-float on the FP32 pipe; three FP64 instructions per point.
__global__ void __launch_bounds__(kThreads)
    k_vc_dir_mixed(const float* __restrict__ z, const float2* __restrict__ E,
                   const float2* __restrict__ Nc, const float2* __restrict__ D,
                   const float2* __restrict__ flo_p, const float2* __restrict__ fhi_p,
                   double* __restrict__ p, double* __restrict__ ap, int n, int cols,
                   SolveState* st, ReduceBuf rb) {
  pdl_begin();
  if (st->done) return;
  const bool first = st->iter == 0;
  const double beta = st->beta;
  const int nrb = (n + kThreads - 1) / kThreads;
  const int items = nrb * ((n + cols - 1) / cols);
  DotAcc<float> acc;
  for (int w = blockIdx.x; w < items; w += gridDim.x) {
    const int i = (w % nrb) * kThreads + threadIdx.x;
    if (i >= n) continue;
    const int j0 = (w / nrb) * cols;
    const int j1 = min(n, j0 + cols);
    const float2 flo = __ldg(flo_p + i), fhi = __ldg(fhi_p + i);
    auto Z = [&](int ii, int jj) { return __ldg(z + (size_t)jj * n + ii); };
    float um = j0 > 0 ? Z(i, j0 - 1) : 0.0f, u0 = Z(i, j0);
    float2 nm = j0 > 0 ? __ldg(Nc + (size_t)(j0 - 1) * n + i) : make_float2(0.0f, 0.0f);
    for (int j = j0; j < j1; ++j) {
      const size_t k = (size_t)j * n + i;
      const float up = j + 1 < n ? Z(i, j + 1) : 0.0f;
      const float2 n0 = __ldg(Nc + k);
      // -A z = couplings - D z; accumulate A z = D z - couplings
      float hi = 0.0f, lo = 0.0f;
      ff_fma(__ldg(D + k), u0, hi, lo);
      ff_fma(make_float2(-nm.x, -nm.y), um, hi, lo);
      ff_fma(make_float2(-n0.x, -n0.y), up, hi, lo);
      if (i > 0) {
        const float2 e = __ldg(E + k - 1);
        ff_fma(make_float2(-e.x, -e.y), Z(i - 1, j), hi, lo);
      }
      if (i < n - 1) {
        const float2 e = __ldg(E + k);
        ff_fma(make_float2(-e.x, -e.y), Z(i + 1, j), hi, lo);
      }
      if (j <= 2 || j >= n - 3) {
        const float2 fl = make_float2(-flo.x, -flo.y), fh = make_float2(-fhi.x, -fhi.y);
        if (j == 0) ff_fma(fl, Z(i, 2), hi, lo);
        if (j == 2) ff_fma(fl, Z(i, 0), hi, lo);
        if (j == n - 1) ff_fma(fh, Z(i, n - 3), hi, lo);
        if (j == n - 3) ff_fma(fh, Z(i, n - 1), hi, lo);
      }
      const double azd = f32_to_f64(hi) + f32_to_f64(lo);
      const double zd = f32_to_f64(u0);
      const double pv = first ? zd : fma(beta, p[k], zd);
      const double av = first ? azd : fma(beta, ap[k], azd);
      p[k] = pv;
      ap[k] = av;
      acc.add_prod(f64_to_f32(pv), f64_to_f32(av));
      um = u0;
      u0 = up;
      nm = n0;
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

// x = Ainv b on the coarse grid: one warp per row, FP64 accumulation.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_dense_gemv(const double* __restrict__ Ainv, const T* __restrict__ b, T* __restrict__ x,
                 int N, const SolveState* st) {
  pdl_begin();
  if (st && st->done) return;
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * kWarps;
  for (int r = blockIdx.x * kWarps + (threadIdx.x >> 5); r < N; r += warps) {
    const double* row = Ainv + (size_t)r * N;
    double s = 0.0;
    for (int k = lane; k < N; k += 32) s = fma(__ldg(row + k), (double)__ldg(b + k), s);
    s = warp_sum(s);
    if (lane == 0) x[r] = (T)s;
  }
}

template <int MODE, typename T>
cudaError_t launch_vc_mode(const VcArgsT<T>& a, dim3 grid, cudaStream_t s) {
  if (a.rb.partials) return launch_pdl(k_vc<MODE, true, T>, grid, dim3(kThreads), 0, s, a);
  return launch_pdl(k_vc<MODE, false, T>, grid, dim3(kThreads), 0, s, a);
}

}  // namespace

cudaError_t launch_vc_apply_c(const double* u, const double* c, double* out, int n, int sign,
                              ReduceBuf rb, double* dot_out, cudaStream_t s) {
  if (n < 3) return cudaErrorInvalidValue;
  const int cols = vc_cols(n);
  const dim3 g = vc_grid(n, cols);
  if (dot_out)
    return launch_pdl(k_vc_apply_c<true>, g, dim3(kThreads), 0, s, u, c, out, n, sign, cols, rb,
                      dot_out);
  return launch_pdl(k_vc_apply_c<false>, g, dim3(kThreads), 0, s, u, c, out, n, sign, cols, rb,
                    dot_out);
}

template <typename T>
cudaError_t launch_vc_stencil(const double* c, T* E, T* N, T* D, T* flo, T* fhi, T* Dinv,
                              double wscale, int n, cudaStream_t s) {
  const long long total = (long long)n * n;
  const int g = (int)std::max(1LL, std::min<long long>((total + kThreads - 1) / kThreads, 4096));
  k_vc_stencil<T><<<g, kThreads, 0, s>>>(c, E, N, D, flo, fhi, Dinv, wscale, n);
  return cudaGetLastError();
}

cudaError_t launch_vc_coarsen(const double* cf, double* cc, int nc, cudaStream_t s) {
  if (nc < 2) return cudaErrorInvalidValue;
  const long long total = (long long)nc * nc;
  const int g = (int)std::max(1LL, std::min<long long>((total + kThreads - 1) / kThreads, 4096));
  k_vc_coarsen<<<g, kThreads, 0, s>>>(cf, cc, nc);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_vc(int mode, VcArgsT<T> a, cudaStream_t s) {
  if (a.n < 3 || !a.out) return cudaErrorInvalidValue;
  if (a.cols <= 0) a.cols = vc_cols(a.n);
  const dim3 g = vc_grid(a.n, a.cols);
  switch (mode) {
    case kHoApply: return launch_vc_mode<kHoApply>(a, g, s);
    case kHoResid: return launch_vc_mode<kHoResid>(a, g, s);
    case kHoJacobi: return launch_vc_mode<kHoJacobi>(a, g, s);
    default: return cudaErrorInvalidValue;
  }
}

template <typename T>
cudaError_t launch_dense_gemv(const double* Ainv, const T* b, T* x, int N, const SolveState* st,
                              cudaStream_t s) {
  const int g = std::max(1, std::min((N + kWarps - 1) / kWarps, 1024));
  return launch_pdl(k_dense_gemv<T>, dim3(g), dim3(kThreads), 0, s, Ainv, b, x, N, st);
}

cudaError_t launch_split_pairs(const double* in, float2* out, long long count, cudaStream_t s) {
  const int g = (int)std::max(1LL, std::min<long long>((count + kThreads - 1) / kThreads, 4096));
  k_split_pairs<<<g, kThreads, 0, s>>>(in, out, count);
  return cudaGetLastError();
}

cudaError_t launch_vc_dir_mixed(const float* z, const float2* const* st, double* pd, double* ap,
                                int n, SolveState* state, ReduceBuf rb, cudaStream_t s) {
  if (n < 3 || !rb.partials) return cudaErrorInvalidValue;
  const int cols = vc_cols(n);
  return launch_pdl(k_vc_dir_mixed, vc_grid(n, cols), dim3(kThreads), 0, s, z, st[0], st[1],
                    st[2], st[3], st[4], pd, ap, n, cols, state, rb);
}

template cudaError_t launch_vc_stencil<double>(const double*, double*, double*, double*, double*,
                                               double*, double*, double, int, cudaStream_t);
template cudaError_t launch_vc_stencil<float>(const double*, float*, float*, float*, float*,
                                              float*, float*, double, int, cudaStream_t);
template cudaError_t launch_vc<double>(int, VcArgsT<double>, cudaStream_t);
template cudaError_t launch_vc<float>(int, VcArgsT<float>, cudaStream_t);
template cudaError_t launch_dense_gemv<double>(const double*, const double*, double*, int,
                                               const SolveState*, cudaStream_t);
template cudaError_t launch_dense_gemv<float>(const double*, const float*, float*, int,
                                              const SolveState*, cudaStream_t);

}  // namespace sbp

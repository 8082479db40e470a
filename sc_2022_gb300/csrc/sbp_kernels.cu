// SBP-SAT Poisson kernels for sm_103a: operator apply, fused CG updates,
// multigrid smoothing / transfer / coarse solve, right-hand-side assembly.
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include "sbp_kernels.cuh"
#include "sbp_launch.h"

namespace sbp {

// Output tile of the stencil kernels: 64 points along the contiguous index
// i (two 256-byte FP64 rows per warp pass) by 32 along j.  The staged tile
// with halo is at most 67 x 37 = 19.8 KB in FP64.
constexpr int TI = 64;
constexpr int TJ = 32;
using TileT = Tile<TI, TJ>;
constexpr int kSmemPts = TileT::SI * TileT::SJ;
constexpr int kIntPts = (TI + 1) * (TJ + 1);     // interior-staged operand
// Coarse region under a fine tile (prolongation operand).
constexpr int EP = TI / 2 + 4;
constexpr int EJ = TJ / 2 + 6;

// Coarse tile of the fused residual + restriction kernel.
constexpr int RTI = 32;
constexpr int RTJ = 16;
constexpr int RVI = 2 * (RTI + 1) + 3;  // staged fine v region (max)
constexpr int RVJ = 2 * (RTJ + 1) + 3;
constexpr int RRI = RVI - 2;            // fine residual region (max)
constexpr int RRJ = RVJ - 2;

// Coarse dense solve: rows of Ainv per warp.
constexpr int kGemvRowsPerWarp = 2;

// Flat (pointwise) kernels: CTAs per launch cap (152 SMs x 8).
constexpr int kFlatCtas = 1216;

static inline dim3 tile_grid(int n) { return dim3(ntiles(n, TI), ntiles(n, TJ)); }

static inline int flat_grid(long long N, int per) {
  const long long want = (N + (long long)kThreads * per - 1) / ((long long)kThreads * per);
  return (int)std::max(1LL, std::min<long long>(want, kFlatCtas));
}

int max_reduce_ctas(int n) {
  const dim3 g = tile_grid(n);
  return std::max((int)(g.x * g.y), kFlatCtas);
}

// Visit the points of a tile without shared memory (pointwise 2D kernels).
template <typename Fn>
__device__ __forceinline__ void for_points(const TileT& t, Fn&& fn) {
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const int mi = t.i_hi - t.i_lo;
  const int mj = t.j_hi - t.j_lo;
  for (int c = w; c < mj; c += kWarps)
    for (int r = lane; r < mi; r += 32) fn(t.i_lo + r, t.j_lo + c);
}

// ---------------------------------------------------------------------------
// Operator apply: out = sign * (-A) u, optional fused dot u.out.
// ---------------------------------------------------------------------------
template <typename T, bool DOT>
__global__ void __launch_bounds__(kThreads) k_apply(Grid<const T> u, Grid<T> out, int n, int sign,
                                                    ReduceBuf rb, double* dot_out) {
  __shared__ T s[kSmemPts];
  TileT t;
  t.init(blockIdx.x, blockIdx.y, n);
  stage_tile_async(s, t, u, n);
  cp_async_wait_all();
  __syncthreads();
  double acc = 0.0;
  for_tile_points(s, t, [&](int i, int j, const SAcc<T>& a, int) {
    const T v = signedA<T>(a, i, j, n, sign);
    out.at(i, j) = v;
    if (DOT) acc += (double)a(0, 0) * (double)v;
  });
  if (DOT) grid_reduce(acc, rb, [&](double tot) { *dot_out = tot; });
}

template <typename T>
cudaError_t launch_apply(Grid<const T> u, Grid<T> out, int n, int sign, ReduceBuf rb,
                         double* dot_out, cudaStream_t s) {
  if (dot_out)
    k_apply<T, true><<<tile_grid(n), kThreads, 0, s>>>(u, out, n, sign, rb, dot_out);
  else
    k_apply<T, false><<<tile_grid(n), kThreads, 0, s>>>(u, out, n, sign, rb, nullptr);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Initial residual r = b - opsign*A*x with ||r||^2 and Krylov-state setup.
// ---------------------------------------------------------------------------
struct ResFin {
  SolveState* st;
  double* norms;
  double abstol;
  double reltol;
  int plain;
  double* out2;
};

template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_residual(Grid<const T> x, Grid<const T> b, Grid<T> r, Grid<float> rlo, int n, int opsign,
               ResFin rf, ReduceBuf rb) {
  __shared__ T s[kSmemPts];
  __shared__ T sb[kIntPts];
  TileT t;
  t.init(blockIdx.x, blockIdx.y, n);
  stage_tile_async(s, t, x, n);
  stage_interior_async(sb, t, b, n);
  cp_async_wait_all();
  __syncthreads();
  double acc = 0.0;
  for_tile_points(s, t, [&](int i, int j, const SAcc<T>& a, int k) {
    const T rv = sb[k] + signedA<T>(a, i, j, n, -opsign);
    r.at(i, j) = rv;
    if (rlo.p) rlo.at(i, j) = (float)rv;
    acc += (double)rv * (double)rv;
  });
  grid_reduce(acc, rb, [&](double tot) {
    if (rf.out2) *rf.out2 = tot;
    SolveState* st = rf.st;
    if (st) {
      st->rr0 = tot;
      st->rr = tot;
      st->thresh2 = rf.abstol > 0.0 ? rf.abstol * rf.abstol : rf.reltol * rf.reltol * tot;
      st->iter = 0;
      st->beta = 0.0;
      st->alpha = 0.0;
      if (rf.plain) st->rz = tot;
      if (rf.norms) rf.norms[0] = sqrt(tot);
      if (!isfinite(tot))
        st->done = kDoneBreakdown;
      else if (tot < st->thresh2 || tot == 0.0)
        st->done = kDoneConverged;
      else
        st->done = 0;
    }
  });
}

template <typename T>
cudaError_t launch_residual(Grid<const T> x, Grid<const T> b, Grid<T> r, Grid<float> rlo, int n,
                            int opsign, SolveState* st, double* norms, double abstol,
                            double reltol, int plain, double* out2, ReduceBuf rb,
                            cudaStream_t s) {
  ResFin rf{st, norms, abstol, reltol, plain, out2};
  k_residual<T><<<tile_grid(n), kThreads, 0, s>>>(x, b, r, rlo, n, opsign, rf, rb);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// CG direction + operator + p.Ap  (one HBM pass: reads z, p_old; writes p, Ap)
// ---------------------------------------------------------------------------
template <typename T, typename Tz>
__global__ void __launch_bounds__(kThreads)
    k_cg_dir(Grid<const Tz> z, Grid<const T> pold, Grid<T> pnew, Grid<T> Ap, int n, int opsign,
             SolveState* st, ReduceBuf rb) {
  if (st->done) return;
  __shared__ T s[kSmemPts];
  __shared__ Tz sz[kSmemPts];
  TileT t;
  t.init(blockIdx.x, blockIdx.y, n);
  const bool first = (st->iter == 0);
  const T beta = T(st->beta);
  stage_tile_async(sz, t, z, n);
  if (!first) stage_tile_async(s, t, pold, n);
  cp_async_wait_all();
  __syncthreads();
  {
    constexpr int SI = TileT::SI;
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    const int ei = t.i_hi - t.i_lo + 2;
    const int ej = t.j_hi - t.j_lo + t.hl + t.hr;
    for (int c = w; c < ej; c += kWarps)
      for (int r = lane; r < ei; r += 32) {
        const int q = c * SI + r;
        s[q] = first ? T(sz[q]) : T(sz[q]) + beta * s[q];
      }
  }
  __syncthreads();
  double acc = 0.0;
  for_tile_points(s, t, [&](int i, int j, const SAcc<T>& a, int) {
    const T pv = a(0, 0);
    const T ap = signedA<T>(a, i, j, n, opsign);
    pnew.at(i, j) = pv;
    Ap.at(i, j) = ap;
    acc += (double)pv * (double)ap;
  });
  grid_reduce(acc, rb, [&](double tot) {
    st->pAp = tot;
    if (!isfinite(tot) || tot == 0.0)
      st->done = kDoneBreakdown;
    else
      st->alpha = st->rz / tot;
  });
}

template <typename T, typename Tz>
cudaError_t launch_cg_dir(Grid<const Tz> z, Grid<const T> pold, Grid<T> pnew, Grid<T> Ap, int n,
                          int opsign, SolveState* st, ReduceBuf rb, cudaStream_t s) {
  k_cg_dir<T, Tz><<<tile_grid(n), kThreads, 0, s>>>(z, pold, pnew, Ap, n, opsign, st, rb);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// CG update (pointwise, flat, 16-byte vectors): x += alpha p; r -= alpha Ap;
// ||r||^2; convergence test.  All solver arrays are contiguous n*n.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cg_update_pt(double& x, double& r, double p, double ap,
                                             double alpha, double& acc) {
  x += alpha * p;
  r -= alpha * ap;
  acc += r * r;
}

template <bool VEC>
__global__ void __launch_bounds__(kThreads)
    k_cg_update(double* __restrict__ x, double* __restrict__ r, const double* __restrict__ p,
                const double* __restrict__ Ap, float* __restrict__ rlo, long long N, int plain,
                SolveState* st, double* norms, ReduceBuf rb) {
  if (st->done) return;
  const double alpha = st->alpha;
  double acc = 0.0;
  const long long tid = (long long)blockIdx.x * kThreads + threadIdx.x;
  const long long stride = (long long)gridDim.x * kThreads;
  long long done_to = 0;
  if (VEC) {
    const long long nv = N / 2;
    double2* x2 = reinterpret_cast<double2*>(x);
    double2* r2 = reinterpret_cast<double2*>(r);
    const double2* p2 = reinterpret_cast<const double2*>(p);
    const double2* a2 = reinterpret_cast<const double2*>(Ap);
#pragma unroll 2
    for (long long k = tid; k < nv; k += stride) {
      const double2 pv = __ldg(p2 + k);
      const double2 av = __ldg(a2 + k);
      double2 xv = x2[k];
      double2 rv = r2[k];
      cg_update_pt(xv.x, rv.x, pv.x, av.x, alpha, acc);
      cg_update_pt(xv.y, rv.y, pv.y, av.y, alpha, acc);
      x2[k] = xv;
      r2[k] = rv;
      if (rlo) reinterpret_cast<float2*>(rlo)[k] = make_float2((float)rv.x, (float)rv.y);
    }
    done_to = 2 * nv;
  }
  for (long long k = done_to + tid; k < N; k += stride) {
    double xv = x[k], rv = r[k];
    cg_update_pt(xv, rv, p[k], Ap[k], alpha, acc);
    x[k] = xv;
    r[k] = rv;
    if (rlo) rlo[k] = (float)rv;
  }
  grid_reduce(acc, rb, [&](double tot) {
    const int it = st->iter + 1;
    st->iter = it;
    st->rr = tot;
    if (norms) norms[it] = sqrt(tot);
    if (plain) {
      st->beta = tot / st->rz;
      st->rz = tot;
    }
    if (!isfinite(tot))
      st->done = kDoneBreakdown;
    else if (tot < st->thresh2)
      st->done = kDoneConverged;
    else if (it >= st->maxiter)
      st->done = kDoneMaxIter;
  });
}

static inline bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

template <typename T>
cudaError_t launch_cg_update(Grid<T> x, Grid<T> r, Grid<const T> p, Grid<const T> Ap,
                             Grid<float> rlo, int n, int plain, SolveState* st, double* norms,
                             ReduceBuf rb, cudaStream_t s) {
  static_assert(sizeof(T) == 8, "the Krylov vectors are FP64");
  if (x.ld != n || r.ld != n || p.ld != n || Ap.ld != n) return cudaErrorInvalidValue;
  const long long N = (long long)n * n;
  const bool vec = aligned16(x.p) && aligned16(r.p) && aligned16(p.p) && aligned16(Ap.p) &&
                   (!rlo.p || ((uintptr_t)rlo.p & 7u) == 0);
  const int g = flat_grid(N, vec ? 4 : 2);
  if (vec)
    k_cg_update<true><<<g, kThreads, 0, s>>>(x.p, r.p, p.p, Ap.p, rlo.p, N, plain, st, norms, rb);
  else
    k_cg_update<false><<<g, kThreads, 0, s>>>(x.p, r.p, p.p, Ap.p, rlo.p, N, plain, st, norms, rb);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Smoothing pass (Jacobi / Richardson) with the field variants.
// ---------------------------------------------------------------------------
template <typename T, int FIELD, int EPI, bool DOT>
__global__ void __launch_bounds__(kThreads)
    k_smooth(Grid<const T> vin, Grid<const T> e, Grid<const T> b, Grid<T> vout, int n,
             int smoother, T omega, SolveState* st, ReduceBuf rb) {
  if (st && st->done) return;
  __shared__ T s[kSmemPts];
  __shared__ T sb[kIntPts];
  __shared__ T se[FIELD == kFieldProlong ? EP * EJ : 1];
  TileT t;
  t.init(blockIdx.x, blockIdx.y, n);
  const bool jac = (smoother == kSmoothJacobi);
  const bool need_b = (EPI == kEpiSweep) || DOT;
  int I0 = 0, J0 = 0;
  if (FIELD == kFieldZero) {
    stage_tile_async(s, t, b, n);
    if (need_b) stage_interior_async(sb, t, b, n);
  } else {
    stage_tile_async(s, t, vin, n);
    if (need_b) stage_interior_async(sb, t, b, n);
  }
  if (FIELD == kFieldProlong) {
    const int nc = (n + 1) / 2;
    I0 = (t.i_lo - 1) >> 1;
    J0 = (t.j_lo - t.hl) >> 1;
    const int ei = (t.i_hi >> 1) - I0 + 2;
    const int ej = ((t.j_hi + t.hr - 1) >> 1) - J0 + 2;
    stage_async<EP>(se, e, I0, J0, ei, ej, nc);
  }
  cp_async_wait_all();
  __syncthreads();
  if (FIELD == kFieldProlong) {
    transform_staged(s, t, n, [&](int i, int j, T& v) { v += prolong_smem<EP>(se, I0, J0, i, j); });
    __syncthreads();
  } else if (FIELD == kFieldZero) {
    // first sweep from zero, once per staged point: v1 = omega D^-1 b
    transform_staged(s, t, n, [&](int i, int j, T& v) {
      v *= jac ? omega * inv_diagA<T>(i, j, n) : omega;
    });
    __syncthreads();
  }
  double acc = 0.0;
  for_tile_points(s, t, [&](int i, int j, const SAcc<T>& a, int k) {
    const T f = a(0, 0);
    const T bb = need_b ? sb[k] : T(0);
    T vn = f;
    if (EPI == kEpiSweep) {
      const T m = jac ? omega * inv_diagA<T>(i, j, n) : omega;
      vn = fma(m, bb + negA<T>(a, i, j, n), f);
    }
    vout.at(i, j) = vn;
    if (DOT) acc += (double)bb * (double)vn;
  });
  if (DOT) {
    grid_reduce(acc, rb, [&](double tot) {
      if (!isfinite(tot)) {
        st->done = kDoneBreakdown;
      } else {
        st->rz_new = tot;
        if (st->iter > 0) st->beta = tot / st->rz;
        st->rz = tot;
      }
    });
  }
}

template <typename T, int FIELD, int EPI>
static cudaError_t launch_smooth_fe(Grid<const T> vin, Grid<const T> e, Grid<const T> b,
                                    Grid<T> vout, int n, int smoother, double omega, int dot,
                                    SolveState* st, ReduceBuf rb, cudaStream_t s) {
  if (dot)
    k_smooth<T, FIELD, EPI, true><<<tile_grid(n), kThreads, 0, s>>>(vin, e, b, vout, n, smoother,
                                                                    T(omega), st, rb);
  else
    k_smooth<T, FIELD, EPI, false><<<tile_grid(n), kThreads, 0, s>>>(vin, e, b, vout, n, smoother,
                                                                     T(omega), st, rb);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_smooth(int field, int epi, Grid<const T> vin, Grid<const T> e, Grid<const T> b,
                          Grid<T> vout, int n, int smoother, double omega, int dot,
                          SolveState* st, ReduceBuf rb, cudaStream_t s) {
  if (dot && !st) return cudaErrorInvalidValue;
#define SBP_SMOOTH_CASE(F, E)                                                                  \
  if (field == F && epi == E)                                                                  \
    return launch_smooth_fe<T, F, E>(vin, e, b, vout, n, smoother, omega, dot, st, rb, s);
  SBP_SMOOTH_CASE(kFieldPlain, kEpiSweep)
  SBP_SMOOTH_CASE(kFieldPlain, kEpiStore)
  SBP_SMOOTH_CASE(kFieldZero, kEpiSweep)
  SBP_SMOOTH_CASE(kFieldZero, kEpiStore)
  SBP_SMOOTH_CASE(kFieldProlong, kEpiSweep)
  SBP_SMOOTH_CASE(kFieldProlong, kEpiStore)
#undef SBP_SMOOTH_CASE
  return cudaErrorInvalidValue;
}

// ---------------------------------------------------------------------------
// Fused residual + restriction: f = R (b - A v).  Tiles live on the coarse
// grid; the CTA stages b (as the residual buffer) and v for the fine region
// under its coarse tile, forms r in shared memory, then applies the 3x3
// restriction weights.  One HBM pass over v and b, a quarter-size write.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_resrestrict(Grid<const T> v, Grid<const T> b, Grid<T> f, int nf, int kind,
                  const SolveState* st) {
  if (st && st->done) return;
  __shared__ T sv[RVI * RVJ];
  __shared__ T sr[RRI * RRJ];
  const int nc = (nf + 1) / 2;
  Tile<RTI, RTJ> t;
  t.init(blockIdx.x, blockIdx.y, nc);
  const int m = t.i_hi - t.i_lo;
  const int mp = t.j_hi - t.j_lo;
  const int ri0 = 2 * t.i_lo - 1;
  const int rj0 = 2 * t.j_lo - 1;
  const int rei = 2 * m + 1;
  const int rej = 2 * mp + 1;
  stage_async<RRI>(sr, b, ri0, rj0, rei, rej, nf);
  if (v.p) stage_async<RVI>(sv, v, ri0 - 1, rj0 - 1, rei + 2, rej + 2, nf);
  cp_async_wait_all();
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  if (v.p) {
    for (int c = w; c < rej; c += kWarps) {
      const int j = rj0 + c;
      if (j < 0 || j >= nf) continue;
      for (int r = lane; r < rei; r += 32) {
        const int i = ri0 + r;
        if (i < 0 || i >= nf) continue;
        SAcc<T> a{sv + (c + 1) * RVI + (r + 1), RVI};
        sr[c * RRI + r] += negA<T>(a, i, j, nf);
      }
    }
    __syncthreads();
  }
  for (int c = w; c < mp; c += kWarps) {
    const int J = t.j_lo + c;
    for (int r = lane; r < m; r += 32) {
      const int I = t.i_lo + r;
      T acc = T(0);
#pragma unroll
      for (int bj = -1; bj <= 1; ++bj) {
        const T wj = restrict_w1<T>(kind, J, nc, bj);
#pragma unroll
        for (int ai = -1; ai <= 1; ++ai) {
          const T wi = restrict_w1<T>(kind, I, nc, ai);
          acc += wi * wj * sr[(2 * c + 1 + bj) * RRI + (2 * r + 1 + ai)];
        }
      }
      f.at(I, J) = acc;
    }
  }
}

template <typename T>
cudaError_t launch_resrestrict(Grid<const T> v, Grid<const T> b, Grid<T> f, int nf, int kind,
                               const SolveState* st, cudaStream_t s) {
  const int nc = (nf + 1) / 2;
  const dim3 g(ntiles(nc, RTI), ntiles(nc, RTJ));
  k_resrestrict<T><<<g, kThreads, 0, s>>>(v, b, f, nf, kind, st);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Standalone prolongation out (+)= P e.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_prolong(Grid<const T> e, Grid<T> out, int nc, int accumulate, const SolveState* st) {
  if (st && st->done) return;
  const int nf = 2 * nc - 1;
  TileT t;
  t.init(blockIdx.x, blockIdx.y, nf);
  for_points(t, [&](int i, int j) {
    const T v = prolong_at(e, i, j);
    out.at(i, j) = accumulate ? out.at(i, j) + v : v;
  });
}

template <typename T>
cudaError_t launch_prolong(Grid<const T> e, Grid<T> out, int nc, int accumulate,
                           const SolveState* st, cudaStream_t s) {
  k_prolong<T><<<tile_grid(2 * nc - 1), kThreads, 0, s>>>(e, out, nc, accumulate, st);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Coarse direct solve as a dense FP64 GEMV with the precomputed inverse.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_coarse_gemv(const double* __restrict__ Ainv, Grid<const T> f, Grid<T> e, int nc,
                  const SolveState* st) {
  if (st && st->done) return;
  extern __shared__ double sf[];
  const int N = nc * nc;
  for (int k = threadIdx.x; k < N; k += kThreads) {
    const int j = k / nc;
    const int i = k - j * nc;
    sf[k] = (double)f.at(i, j);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < kGemvRowsPerWarp; ++q) {
    const int row = (blockIdx.x * kWarps + w) * kGemvRowsPerWarp + q;
    if (row >= N) break;
    const double* a = Ainv + (size_t)row * (size_t)N;
    double acc = 0.0;
#pragma unroll 8
    for (int c = lane; c < N; c += 32) acc += __ldg(a + c) * sf[c];
    acc = warp_sum(acc);
    if (lane == 0) {
      const int j = row / nc;
      const int i = row - j * nc;
      e.at(i, j) = (T)acc;
    }
  }
}

template <typename T>
cudaError_t launch_coarse_gemv(const double* Ainv, Grid<const T> f, Grid<T> e, int nc,
                               const SolveState* st, cudaStream_t s) {
  const int N = nc * nc;
  const int rows_per_cta = kWarps * kGemvRowsPerWarp;
  const int grid = (N + rows_per_cta - 1) / rows_per_cta;
  const size_t smem = (size_t)N * sizeof(double);
  if (smem > 48 * 1024) {
    cudaError_t err = cudaFuncSetAttribute(k_coarse_gemv<T>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
  }
  k_coarse_gemv<T><<<grid, kThreads, smem, s>>>(Ainv, f, e, nc, st);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Copy / convert and dot (pointwise, flat over contiguous n*n arrays).
// ---------------------------------------------------------------------------
template <typename Tin, typename Tout>
__global__ void __launch_bounds__(kThreads)
    k_copy(const Tin* __restrict__ in, Tout* __restrict__ out, long long N) {
  const long long stride = (long long)gridDim.x * kThreads;
  for (long long k = (long long)blockIdx.x * kThreads + threadIdx.x; k < N; k += stride)
    out[k] = (Tout)__ldg(in + k);
}

template <typename Tin, typename Tout>
cudaError_t launch_copy(Grid<const Tin> in, Grid<Tout> out, int n, cudaStream_t s) {
  if (in.ld != n || out.ld != n) return cudaErrorInvalidValue;
  const long long N = (long long)n * n;
  k_copy<Tin, Tout><<<flat_grid(N, 4), kThreads, 0, s>>>(in.p, out.p, N);
  return cudaGetLastError();
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_dot(const T* __restrict__ a, const T* __restrict__ b, long long N, double* out,
          ReduceBuf rb) {
  double acc = 0.0;
  const long long stride = (long long)gridDim.x * kThreads;
  for (long long k = (long long)blockIdx.x * kThreads + threadIdx.x; k < N; k += stride)
    acc += (double)__ldg(a + k) * (double)__ldg(b + k);
  grid_reduce(acc, rb, [&](double tot) { *out = tot; });
}

template <typename T>
cudaError_t launch_dot(Grid<const T> a, Grid<const T> b, int n, double* out, ReduceBuf rb,
                       cudaStream_t s) {
  if (a.ld != n || b.ld != n) return cudaErrorInvalidValue;
  const long long N = (long long)n * n;
  k_dot<T><<<flat_grid(N, 4), kThreads, 0, s>>>(a.p, b.p, N, out, rb);
  return cudaGetLastError();
}

__global__ void k_state_init(SolveState* st, int maxiter) {
  SolveState z = {};
  z.maxiter = maxiter;
  *st = z;
}

cudaError_t launch_state_init(SolveState* st, int maxiter, cudaStream_t s) {
  k_state_init<<<1, 1, 0, s>>>(st, maxiter);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Right-hand side b(f, g) and its transpose.
//   b(i,j) = -[ h^2 wi wj fsign f(i,j)
//               + wi (sum_{j<=2} cD[j] gW[i] + sum_{j>=n-3} cD[n-1-j] gE[i])
//               + h wj tauN (delta_{i,0} gS[j] + delta_{i,n-1} gN[j]) ]
// i.e. -H~ (f + SAT_W_r gW + SAT_E_r gE + SAT_S_r gS + SAT_N_r gN).
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ double cD(int d) {
  return d == 0 ? kCD0 : (d == 1 ? kCD1 : kCD2);
}

__global__ void __launch_bounds__(kThreads)
    k_rhs(Grid<const double> f, const double* gW, const double* gE, const double* gS,
          const double* gN, Grid<double> b, int n, double fsign) {
  TileT t;
  t.init(blockIdx.x, blockIdx.y, n);
  const double h = 1.0 / (n - 1);
  for_points(t, [&](int i, int j) {
    const double wi = (i == 0 || i == n - 1) ? 0.5 : 1.0;
    const double wj = (j == 0 || j == n - 1) ? 0.5 : 1.0;
    double acc = h * h * wi * wj * fsign * f.at(i, j);
    double dir = 0.0;
    if (j <= 2) dir += cD(j) * gW[i];
    if (j >= n - 3) dir += cD(n - 1 - j) * gE[i];
    acc += wi * dir;
    double neu = 0.0;
    if (i == 0) neu += gS[j];
    if (i == n - 1) neu += gN[j];
    acc += h * wj * kTauN * neu;
    b.at(i, j) = -acc;
  });
}

cudaError_t launch_rhs(Grid<const double> f, const double* gW, const double* gE,
                       const double* gS, const double* gN, Grid<double> b, int n, double fsign,
                       cudaStream_t s) {
  k_rhs<<<tile_grid(n), kThreads, 0, s>>>(f, gW, gE, gS, gN, b, n, fsign);
  return cudaGetLastError();
}

__global__ void __launch_bounds__(kThreads)
    k_rhs_adjoint_f(Grid<const double> lam, Grid<double> df, int n, double fsign) {
  TileT t;
  t.init(blockIdx.x, blockIdx.y, n);
  const double h = 1.0 / (n - 1);
  for_points(t, [&](int i, int j) {
    const double wi = (i == 0 || i == n - 1) ? 0.5 : 1.0;
    const double wj = (j == 0 || j == n - 1) ? 0.5 : 1.0;
    df.at(i, j) = -h * h * wi * wj * fsign * lam.at(i, j);
  });
}

__global__ void k_rhs_adjoint_g(Grid<const double> lam, double* dgW, double* dgE, double* dgS,
                                double* dgN, int n) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const double h = 1.0 / (n - 1);
  const double wk = (k == 0 || k == n - 1) ? 0.5 : 1.0;
  double w = 0.0, e = 0.0;
  for (int j = 0; j <= 2 && j < n; ++j) w += cD(j) * lam.at(k, j);
  for (int j = (n - 3 > 0 ? n - 3 : 0); j < n; ++j) e += cD(n - 1 - j) * lam.at(k, j);
  if (dgW) dgW[k] = -wk * w;
  if (dgE) dgE[k] = -wk * e;
  if (dgS) dgS[k] = -h * wk * kTauN * lam.at(0, k);
  if (dgN) dgN[k] = -h * wk * kTauN * lam.at(n - 1, k);
}

cudaError_t launch_rhs_adjoint(Grid<const double> lam, Grid<double> df, double* dgW, double* dgE,
                               double* dgS, double* dgN, int n, double fsign, cudaStream_t s) {
  if (df.p) k_rhs_adjoint_f<<<tile_grid(n), kThreads, 0, s>>>(lam, df, n, fsign);
  k_rhs_adjoint_g<<<(n + 255) / 256, 256, 0, s>>>(lam, dgW, dgE, dgS, dgN, n);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Explicit instantiations.
// ---------------------------------------------------------------------------
#define SBP_INST_T(T)                                                                           \
  template cudaError_t launch_apply<T>(Grid<const T>, Grid<T>, int, int, ReduceBuf, double*,    \
                                       cudaStream_t);                                           \
  template cudaError_t launch_residual<T>(Grid<const T>, Grid<const T>, Grid<T>, Grid<float>,   \
                                          int, int, SolveState*, double*, double, double, int,  \
                                          double*, ReduceBuf, cudaStream_t);                    \
  template cudaError_t launch_smooth<T>(int, int, Grid<const T>, Grid<const T>, Grid<const T>,  \
                                        Grid<T>, int, int, double, int, SolveState*, ReduceBuf, \
                                        cudaStream_t);                                          \
  template cudaError_t launch_resrestrict<T>(Grid<const T>, Grid<const T>, Grid<T>, int, int,   \
                                             const SolveState*, cudaStream_t);                  \
  template cudaError_t launch_prolong<T>(Grid<const T>, Grid<T>, int, int, const SolveState*,   \
                                         cudaStream_t);                                         \
  template cudaError_t launch_coarse_gemv<T>(const double*, Grid<const T>, Grid<T>, int,        \
                                             const SolveState*, cudaStream_t);                  \
  template cudaError_t launch_dot<T>(Grid<const T>, Grid<const T>, int, double*, ReduceBuf,     \
                                     cudaStream_t);

SBP_INST_T(double)
SBP_INST_T(float)
#undef SBP_INST_T

template cudaError_t launch_cg_dir<double, double>(Grid<const double>, Grid<const double>,
                                                   Grid<double>, Grid<double>, int, int,
                                                   SolveState*, ReduceBuf, cudaStream_t);
template cudaError_t launch_cg_dir<double, float>(Grid<const float>, Grid<const double>,
                                                  Grid<double>, Grid<double>, int, int,
                                                  SolveState*, ReduceBuf, cudaStream_t);
template cudaError_t launch_cg_update<double>(Grid<double>, Grid<double>, Grid<const double>,
                                              Grid<const double>, Grid<float>, int, int,
                                              SolveState*, double*, ReduceBuf, cudaStream_t);
template cudaError_t launch_copy<double, double>(Grid<const double>, Grid<double>, int,
                                                 cudaStream_t);
template cudaError_t launch_copy<double, float>(Grid<const double>, Grid<float>, int,
                                                cudaStream_t);
template cudaError_t launch_copy<float, double>(Grid<const float>, Grid<double>, int,
                                                cudaStream_t);
template cudaError_t launch_copy<float, float>(Grid<const float>, Grid<float>, int,
                                               cudaStream_t);

}  // namespace sbp

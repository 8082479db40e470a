// Kernel templates for the SBP-SAT Poisson path.  Included by sbp_kernels.cu
// only; the launch wrappers declared in sbp_launch.h are the interface.
//
// Design (GB300, HBM-bound stencil, no tensor cores):
//  * Every stencil kernel works on 2D tiles of the column-major grid.  A CTA
//    stages its tile of the stencil input plus a one-point halo into shared
//    memory with fully unrolled coalesced loads (all loads of a thread are in
//    flight together), then evaluates the operator from shared memory and
//    writes coalesced outputs.  Tile t covers [t*T + (t>0), (t+1)*T + 1), so
//    a grid of n = 2^k + 1 points splits into whole tiles with the extra
//    point folded into the first tile.
//  * The stencil input is a "field" computed while staging (p = z + beta*p,
//    v + P e, omega*D^-1*b, ...), so vector updates ride along with the
//    operator pass instead of costing their own HBM sweep.
//  * Reductions (dot products) are per-CTA partial sums in fixed order plus a
//    last-CTA-done final pass in fixed order: deterministic, one launch.
//  * Krylov scalars live in a device SolveState; kernels read alpha/beta
//    from it and early-exit once `done` is set, so a captured iteration
//    needs no host round trip.
#pragma once

#include "sbp_common.cuh"

namespace sbp {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;

__host__ __device__ __forceinline__ int ntiles(int n, int t) {
  return n <= 1 ? 1 : (n - 1 + t - 1) / t;
}

// Tile t of a dimension covers [t*T + (t > 0), (t+1)*T + 1) clipped to n.
// The staged region adds one halo point in i and, in j, one column on each
// side, or two on a side where the tile holds a column whose Dirichlet terms
// reach two columns away (j = 2 and n-1 look back, j = 0 and n-3 ahead).
template <int TI, int TJ>
struct Tile {
  static constexpr int SI = TI + 3;
  static constexpr int SJ = TJ + 5;
  int i_lo, i_hi, j_lo, j_hi, hl, hr;
  __device__ __forceinline__ void init(int ti, int tj, int n) {
    i_lo = ti == 0 ? 0 : ti * TI + 1;
    i_hi = min(n, (ti + 1) * TI + 1);
    j_lo = tj == 0 ? 0 : tj * TJ + 1;
    j_hi = min(n, (tj + 1) * TJ + 1);
    const bool back2 = (j_lo <= 2 && 2 < j_hi) || (j_hi == n);
    const bool ahead2 = (j_lo == 0) || (j_lo <= n - 3 && n - 3 < j_hi);
    hl = back2 ? 2 : 1;
    hr = ahead2 ? 2 : 1;
  }
};

// Shared-memory accessor centred on one point.
template <typename T>
struct SAcc {
  const T* s;
  int si;
  __device__ __forceinline__ T operator()(int di, int dj) const { return s[dj * si + di]; }
};

// Stage field values f(i, j) of the region [i0, i0+ei) x [j0, j0+ej) into s
// (row pitch MAXI).  Loads are fully unrolled into registers first so every
// thread has all of its loads in flight before the first shared store.
// Points outside the n x n domain are set to zero.
template <int MAXI, int MAXJ, typename T, typename F>
__device__ __forceinline__ void stage_region(T* s, int i0, int j0, int ei, int ej, int n,
                                             const F& f) {
  constexpr int NR = (MAXI + 31) / 32;
  constexpr int NC = (MAXJ + kWarps - 1) / kWarps;
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  T buf[NC][NR];
#pragma unroll
  for (int a = 0; a < NC; ++a) {
#pragma unroll
    for (int b = 0; b < NR; ++b) {
      const int c = w + a * kWarps;
      const int r = lane + b * 32;
      const int i = i0 + r;
      const int j = j0 + c;
      const bool ok = (c < ej) && (r < ei) && (i >= 0) && (i < n) && (j >= 0) && (j < n);
      buf[a][b] = ok ? f(i, j) : T(0);
    }
  }
#pragma unroll
  for (int a = 0; a < NC; ++a) {
#pragma unroll
    for (int b = 0; b < NR; ++b) {
      const int c = w + a * kWarps;
      const int r = lane + b * 32;
      if (c < ej && r < ei) s[c * MAXI + r] = buf[a][b];
    }
  }
}

// Stage a tile plus its halo.
template <int TI, int TJ, typename T, typename F>
__device__ __forceinline__ void stage_tile(T* s, const Tile<TI, TJ>& t, int n, const F& f) {
  stage_region<Tile<TI, TJ>::SI, Tile<TI, TJ>::SJ>(s, t.i_lo - 1, t.j_lo - t.hl,
                                                   t.i_hi - t.i_lo + 2,
                                                   t.j_hi - t.j_lo + t.hl + t.hr, n, f);
}

// Visit every output point of the tile: fn(i, j, SAcc centred on (i, j)).
template <int TI, int TJ, typename T, typename Fn>
__device__ __forceinline__ void for_tile_points(const T* s, const Tile<TI, TJ>& t, Fn&& fn) {
  constexpr int SI = Tile<TI, TJ>::SI;
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const int mi = t.i_hi - t.i_lo;
  const int mj = t.j_hi - t.j_lo;
  for (int c = w; c < mj; c += kWarps) {
    for (int r = lane; r < mi; r += 32) {
      SAcc<T> acc{s + (c + t.hl) * SI + (r + 1), SI};
      fn(t.i_lo + r, t.j_lo + c, acc);
    }
  }
}

// ---------------------------------------------------------------------------
// Deterministic block + grid reduction.  `fin(total)` runs on one thread of
// the last CTA to finish, after all partials are visible.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double red[kWarps];
  __shared__ double tot;
  v = warp_sum(v);
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kWarps; ++k) s += red[k];
    tot = s;
  }
  __syncthreads();
  return tot;
}

template <typename Fin>
__device__ __forceinline__ void grid_reduce(double v, const ReduceBuf& red, Fin&& fin) {
  __shared__ bool is_last;
  const double bs = block_sum(v);
  const unsigned nb = gridDim.x * gridDim.y;
  if (threadIdx.x == 0) {
    red.partials[blockIdx.y * gridDim.x + blockIdx.x] = bs;
    __threadfence();
    const unsigned t = atomicAdd(red.ticket, 1u);
    is_last = (t == nb - 1);
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  double s = 0.0;
  for (unsigned k = threadIdx.x; k < nb; k += blockDim.x) s += __ldcg(red.partials + k);
  const double total = block_sum(s);
  if (threadIdx.x == 0) {
    fin(total);
    *red.ticket = 0u;
  }
}

__device__ __forceinline__ bool finite_d(double x) { return isfinite(x); }

// ---------------------------------------------------------------------------
// Fields (stencil inputs computed while staging).
// ---------------------------------------------------------------------------
template <typename T>
struct FieldPlain {
  Grid<const T> u;
  __device__ __forceinline__ T operator()(int i, int j) const { return __ldg(&u.at(i, j)); }
};

// CG search direction: p = z + beta * p_old (beta from the device state;
// first iteration p = z).
template <typename T, typename Tz>
struct FieldDir {
  Grid<const Tz> z;
  Grid<const T> pold;
  T beta;
  bool first;
  __device__ __forceinline__ T operator()(int i, int j) const {
    const T zz = T(__ldg(&z.at(i, j)));
    return first ? zz : zz + beta * __ldg(&pold.at(i, j));
  }
};

// First smoothing sweep from v = 0: v1 = omega * D^-1 * b (Jacobi) or
// omega * b (Richardson).
template <typename T>
struct FieldZeroSweep {
  Grid<const T> b;
  int n;
  T omega;
  int smoother;
  __device__ __forceinline__ T operator()(int i, int j) const {
    const T bb = __ldg(&b.at(i, j));
    if (smoother == kSmoothJacobi) return omega * bb * inv_diagA<T>(i, j, n);
    return omega * bb;
  }
};

// Bilinear prolongation of the coarse correction e (nc x nc) to fine point
// (i, j) (prolongation_2D_kernel, matrix_free_mg_cg.jl:41-67).
template <typename T>
__device__ __forceinline__ T prolong_at(const Grid<const T>& e, int i, int j) {
  const int i0 = i >> 1, j0 = j >> 1;
  const bool oi = i & 1, oj = j & 1;
  T v = __ldg(&e.at(i0, j0));
  if (oi) v += __ldg(&e.at(i0 + 1, j0));
  if (oj) {
    v += __ldg(&e.at(i0, j0 + 1));
    if (oi) v += __ldg(&e.at(i0 + 1, j0 + 1));
  }
  const T scale = (oi && oj) ? T(0.25) : ((oi || oj) ? T(0.5) : T(1));
  return v * scale;
}

// v + P e: the coarse-grid correction folded into the following sweep.
template <typename T>
struct FieldProlong {
  Grid<const T> v;
  Grid<const T> e;
  __device__ __forceinline__ T operator()(int i, int j) const {
    return __ldg(&v.at(i, j)) + prolong_at(e, i, j);
  }
};

}  // namespace sbp

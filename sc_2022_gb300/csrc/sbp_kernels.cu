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
// with halo is at most 67 x 37 points.
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

// Flat (pointwise) kernels: CTAs per launch cap.
constexpr int kFlatCtas = 1216;
// Upper bound on the CTAs of a persistent launch (SMs x resident CTAs).
constexpr int kMaxPersistCtas = 4096;

__host__ __device__ constexpr int align16(int b) { return (b + 15) & ~15; }

static inline dim3 tile_grid(int n) { return dim3(ntiles(n, TI), ntiles(n, TJ)); }

static inline int flat_grid(long long N, int per) {
  const long long want = (N + (long long)kThreads * per - 1) / ((long long)kThreads * per);
  return (int)std::max(1LL, std::min<long long>(want, kFlatCtas));
}

int max_reduce_ctas(int n) {
  const dim3 g = tile_grid(n);
  return std::max((int)(g.x * g.y), kMaxPersistCtas);
}

static int sm_count() {
  static int cache[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
  if (cache[dev] == 0) {
    int c = 0;
    cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev);
    cache[dev] = c > 0 ? c : 152;
  }
  return cache[dev];
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

template <int A, int B>
__device__ __forceinline__ Tile<A, B> tile_at(int id, int ntx, int n) {
  Tile<A, B> t;
  t.init(id % ntx, id / ntx, n);
  return t;
}

// ---------------------------------------------------------------------------
// Persistent, double-buffered tile pipeline.  A CTA walks tiles blockIdx.x,
// blockIdx.x + gridDim.x, ...; while it computes tile k from one shared
// buffer, cp.async is already fetching tile k+1 into the other, so HBM
// latency overlaps compute instead of stalling every tile.  The grid is one
// wave (SMs x resident CTAs), so neighbouring CTAs work on neighbouring tiles
// and halo re-reads hit L2.
//
// A Job provides: kStage (bytes of one buffer), kReduce, Acc (accumulator),
// prepare() (reads device state; true = skip the launch), tiles(),
// stage(buf, tile), compute(buf, tile, acc) and finish(total).
// ---------------------------------------------------------------------------
template <class Job>
__global__ void __launch_bounds__(kThreads) k_persist(const Job job_in) {
  extern __shared__ __align__(16) unsigned char smem[];
  Job job = job_in;
  if (job.prepare()) return;
  const int total = job.tiles();
  unsigned char* const buf0 = smem;
  unsigned char* const buf1 = smem + Job::kStage;
  typename Job::Acc acc;
  int tile = blockIdx.x;
  if (tile < total) job.stage(buf0, tile);
  cp_async_commit();
  for (int k = 0; tile < total; ++k, tile += gridDim.x) {
    const int next = tile + gridDim.x;
    if (next < total) job.stage((k & 1) ? buf0 : buf1, next);
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    job.compute((k & 1) ? buf1 : buf0, tile, acc);
    __syncthreads();
  }
  cp_async_wait<0>();
  if (Job::kReduce) grid_reduce(acc.value(), job.rb, [&](double tot) { job.finish(tot); });
}

template <class Job>
static int persist_ctas_per_sm() {
  static const int v = [] {
    const int smem = 2 * Job::kStage;
    if (smem > 48 * 1024)
      cudaFuncSetAttribute(k_persist<Job>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_persist<Job>, kThreads, smem) !=
            cudaSuccess ||
        b < 1)
      b = 1;
    return b;
  }();
  return v;
}

template <class Job>
static cudaError_t launch_persist(const Job& job, int total, cudaStream_t s) {
  const int cap = std::min(kMaxPersistCtas, sm_count() * persist_ctas_per_sm<Job>());
  const int grid = std::max(1, std::min(total, cap));
  k_persist<Job><<<grid, kThreads, 2 * Job::kStage, s>>>(job);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Operator apply: out = sign * A u, optional fused dot u.out.
// ---------------------------------------------------------------------------
template <typename T, bool DOT>
struct ApplyJob {
  static constexpr int kStage = align16(sizeof(T) * kSmemPts);
  static constexpr bool kReduce = DOT;
  using Acc = DotAcc<T>;
  Grid<const T> u;
  Grid<T> out;
  int n, ntx, ntot, sign;
  ReduceBuf rb;
  double* dot_out;
  __device__ bool prepare() { return false; }
  __device__ int tiles() const { return ntot; }
  __device__ void stage(unsigned char* buf, int id) const {
    stage_tile_async(reinterpret_cast<T*>(buf), tile_at<TI, TJ>(id, ntx, n), u, n);
  }
  __device__ void compute(unsigned char* buf, int id, Acc& acc) const {
    const TileT t = tile_at<TI, TJ>(id, ntx, n);
    for_tile_points(reinterpret_cast<T*>(buf), t, [&](int i, int j, const SAcc<T>& a, int) {
      const T v = signedA<T>(a, i, j, n, sign);
      out.at(i, j) = v;
      if (DOT) acc.add_prod(a(0, 0), v);
    });
  }
  __device__ void finish(double tot) const { *dot_out = tot; }
};

template <typename T>
cudaError_t launch_apply(Grid<const T> u, Grid<T> out, int n, int sign, ReduceBuf rb,
                         double* dot_out, cudaStream_t s) {
  const dim3 g = tile_grid(n);
  const int total = (int)(g.x * g.y);
  if (dot_out)
    return launch_persist(ApplyJob<T, true>{u, out, n, (int)g.x, total, sign, rb, dot_out}, total,
                          s);
  return launch_persist(ApplyJob<T, false>{u, out, n, (int)g.x, total, sign, rb, nullptr}, total,
                        s);
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
struct ResidualJob {
  static constexpr int kStage = align16(sizeof(T) * (kSmemPts + kIntPts));
  static constexpr bool kReduce = true;
  using Acc = DotAcc<double>;
  Grid<const T> x, b;
  Grid<T> r;
  Grid<float> rlo;
  int n, ntx, ntot, opsign;
  ResFin rf;
  ReduceBuf rb;
  __device__ bool prepare() { return false; }
  __device__ int tiles() const { return ntot; }
  __device__ void stage(unsigned char* buf, int id) const {
    const TileT t = tile_at<TI, TJ>(id, ntx, n);
    T* s = reinterpret_cast<T*>(buf);
    stage_tile_async(s, t, x, n);
    stage_interior_async(s + kSmemPts, t, b, n);
  }
  __device__ void compute(unsigned char* buf, int id, Acc& acc) const {
    const TileT t = tile_at<TI, TJ>(id, ntx, n);
    const T* s = reinterpret_cast<const T*>(buf);
    const T* sb = s + kSmemPts;
    for_tile_points(s, t, [&](int i, int j, const SAcc<T>& a, int k) {
      const T rv = sb[k] + signedA<T>(a, i, j, n, -opsign);
      r.at(i, j) = rv;
      if (rlo.p) rlo.at(i, j) = convert<float>(rv);
      acc.add_prod((double)rv, (double)rv);
    });
  }
  __device__ void finish(double tot) const {
    if (rf.out2) *rf.out2 = tot;
    SolveState* st = rf.st;
    if (!st) return;
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
};

template <typename T>
cudaError_t launch_residual(Grid<const T> x, Grid<const T> b, Grid<T> r, Grid<float> rlo, int n,
                            int opsign, SolveState* st, double* norms, double abstol,
                            double reltol, int plain, double* out2, ReduceBuf rb,
                            cudaStream_t s) {
  const dim3 g = tile_grid(n);
  const int total = (int)(g.x * g.y);
  ResFin rf{st, norms, abstol, reltol, plain, out2};
  return launch_persist(ResidualJob<T>{x, b, r, rlo, n, (int)g.x, total, opsign, rf, rb}, total,
                        s);
}

// ---------------------------------------------------------------------------
// CG direction + operator + p.Ap  (one HBM pass: reads z, p_old; writes p, Ap)
// ---------------------------------------------------------------------------
template <typename T, typename Tz>
struct CgDirJob {
  static constexpr int kOffZ = align16(sizeof(T) * kSmemPts);
  static constexpr int kStage = kOffZ + align16(sizeof(Tz) * kSmemPts);
  static constexpr bool kReduce = true;
  using Acc = DotAcc<double>;
  Grid<const Tz> z;
  Grid<const T> pold;
  Grid<T> pnew, Ap;
  int n, ntx, ntot, opsign;
  SolveState* st;
  ReduceBuf rb;
  bool first;
  T beta;
  __device__ bool prepare() {
    if (st->done) return true;
    first = (st->iter == 0);
    beta = T(st->beta);
    return false;
  }
  __device__ int tiles() const { return ntot; }
  __device__ void stage(unsigned char* buf, int id) const {
    const TileT t = tile_at<TI, TJ>(id, ntx, n);
    T* s = reinterpret_cast<T*>(buf);
    Tz* sz = reinterpret_cast<Tz*>(buf + kOffZ);
    stage_tile_async(sz, t, z, n);
    if (!first) stage_tile_async(s, t, pold, n);
  }
  __device__ void compute(unsigned char* buf, int id, Acc& acc) const {
    const TileT t = tile_at<TI, TJ>(id, ntx, n);
    T* s = reinterpret_cast<T*>(buf);
    const Tz* sz = reinterpret_cast<const Tz*>(buf + kOffZ);
    {
      constexpr int SI = TileT::SI;
      const int lane = threadIdx.x & 31;
      const int w = threadIdx.x >> 5;
      const int ei = t.i_hi - t.i_lo + 2;
      const int ej = t.j_hi - t.j_lo + t.hl + t.hr;
      for (int c = w; c < ej; c += kWarps)
        for (int r = lane; r < ei; r += 32) {
          const int q = c * SI + r;
          const T zz = convert<T>(sz[q]);
          s[q] = first ? zz : fma(beta, s[q], zz);
        }
    }
    __syncthreads();
    for_tile_points(s, t, [&](int i, int j, const SAcc<T>& a, int) {
      const T pv = a(0, 0);
      const T ap = signedA<T>(a, i, j, n, opsign);
      pnew.at(i, j) = pv;
      Ap.at(i, j) = ap;
      acc.add_prod(pv, ap);
    });
  }
  __device__ void finish(double tot) const {
    st->pAp = tot;
    if (!isfinite(tot) || tot == 0.0)
      st->done = kDoneBreakdown;
    else
      st->alpha = st->rz / tot;
  }
};

template <typename T, typename Tz>
cudaError_t launch_cg_dir(Grid<const Tz> z, Grid<const T> pold, Grid<T> pnew, Grid<T> Ap, int n,
                          int opsign, SolveState* st, ReduceBuf rb, cudaStream_t s) {
  const dim3 g = tile_grid(n);
  const int total = (int)(g.x * g.y);
  return launch_persist(
      CgDirJob<T, Tz>{z, pold, pnew, Ap, n, (int)g.x, total, opsign, st, rb, false, T(0)}, total,
      s);
}

// ---------------------------------------------------------------------------
// CG update (pointwise, flat, 16-byte vectors): x += alpha p; r -= alpha Ap;
// ||r||^2; convergence test.  All solver arrays are contiguous n*n.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cg_update_pt(double& x, double& r, double p, double ap,
                                             double alpha, double& acc) {
  x = fma(alpha, p, x);
  r = fma(-alpha, ap, r);
  acc = fma(r, r, acc);
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
      if (rlo) reinterpret_cast<float2*>(rlo)[k] = make_float2(f64_to_f32(rv.x), f64_to_f32(rv.y));
    }
    done_to = 2 * nv;
  }
  for (long long k = done_to + tid; k < N; k += stride) {
    double xv = x[k], rv = r[k];
    cg_update_pt(xv, rv, p[k], Ap[k], alpha, acc);
    x[k] = xv;
    r[k] = rv;
    if (rlo) rlo[k] = f64_to_f32(rv);
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
struct SmoothJob {
  static constexpr bool kNeedB = (EPI == kEpiSweep) || DOT;
  static constexpr int kOffB = align16(sizeof(T) * kSmemPts);
  static constexpr int kOffE = kOffB + (kNeedB ? align16(sizeof(T) * kIntPts) : 0);
  static constexpr int kStage = kOffE + (FIELD == kFieldProlong ? align16(sizeof(T) * EP * EJ) : 0);
  static constexpr bool kReduce = DOT;
  using Acc = DotAcc<T>;
  Grid<const T> vin, e, b;
  Grid<T> vout;
  int n, ntx, ntot, smoother;
  T omega;
  SolveState* st;
  ReduceBuf rb;
  __device__ bool prepare() { return st && st->done; }
  __device__ int tiles() const { return ntot; }
  __device__ void stage(unsigned char* buf, int id) const {
    const TileT t = tile_at<TI, TJ>(id, ntx, n);
    T* s = reinterpret_cast<T*>(buf);
    stage_tile_async(s, t, FIELD == kFieldZero ? b : vin, n);
    if (kNeedB) stage_interior_async(reinterpret_cast<T*>(buf + kOffB), t, b, n);
    if (FIELD == kFieldProlong) {
      const int nc = (n + 1) / 2;
      const int I0 = (t.i_lo - 1) >> 1;
      const int J0 = (t.j_lo - t.hl) >> 1;
      const int ei = (t.i_hi >> 1) - I0 + 2;
      const int ej = ((t.j_hi + t.hr - 1) >> 1) - J0 + 2;
      stage_async<EP>(reinterpret_cast<T*>(buf + kOffE), e, I0, J0, ei, ej, nc);
    }
  }
  __device__ void compute(unsigned char* buf, int id, Acc& acc) const {
    const TileT t = tile_at<TI, TJ>(id, ntx, n);
    T* s = reinterpret_cast<T*>(buf);
    const T* sb = reinterpret_cast<const T*>(buf + kOffB);
    const bool jac = (smoother == kSmoothJacobi);
    if (FIELD == kFieldProlong) {
      const T* se = reinterpret_cast<const T*>(buf + kOffE);
      const int I0 = (t.i_lo - 1) >> 1;
      const int J0 = (t.j_lo - t.hl) >> 1;
      transform_staged(s, t, n,
                       [&](int i, int j, T& v) { v += prolong_smem<EP>(se, I0, J0, i, j); });
      __syncthreads();
    } else if (FIELD == kFieldZero) {
      // first sweep from zero, once per staged point: v1 = omega D^-1 b
      transform_staged(s, t, n, [&](int i, int j, T& v) {
        v *= jac ? omega * inv_diagA<T>(i, j, n) : omega;
      });
      __syncthreads();
    }
    for_tile_points(s, t, [&](int i, int j, const SAcc<T>& a, int k) {
      const T f = a(0, 0);
      const T bb = kNeedB ? sb[k] : T(0);
      T vn = f;
      if (EPI == kEpiSweep) {
        const T m = jac ? omega * inv_diagA<T>(i, j, n) : omega;
        vn = fma(m, bb + negA<T>(a, i, j, n), f);
      }
      vout.at(i, j) = vn;
      if (DOT) acc.add_prod(bb, vn);
    });
  }
  __device__ void finish(double tot) const {
    if (!isfinite(tot)) {
      st->done = kDoneBreakdown;
    } else {
      st->rz_new = tot;
      if (st->iter > 0) st->beta = tot / st->rz;
      st->rz = tot;
    }
  }
};

template <typename T, int FIELD, int EPI>
static cudaError_t launch_smooth_fe(Grid<const T> vin, Grid<const T> e, Grid<const T> b,
                                    Grid<T> vout, int n, int smoother, double omega, int dot,
                                    SolveState* st, ReduceBuf rb, cudaStream_t s) {
  const dim3 g = tile_grid(n);
  const int total = (int)(g.x * g.y);
  if (dot)
    return launch_persist(SmoothJob<T, FIELD, EPI, true>{vin, e, b, vout, n, (int)g.x, total,
                                                         smoother, T(omega), st, rb},
                          total, s);
  return launch_persist(SmoothJob<T, FIELD, EPI, false>{vin, e, b, vout, n, (int)g.x, total,
                                                        smoother, T(omega), st, rb},
                        total, s);
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
struct ResRestrictJob {
  static constexpr int kOffV = align16(sizeof(T) * RRI * RRJ);
  static constexpr int kStage = kOffV + align16(sizeof(T) * RVI * RVJ);
  static constexpr bool kReduce = false;
  using Acc = DotAcc<double>;
  Grid<const T> v, b;
  Grid<T> f;
  int nf, nc, ntx, ntot, kind;
  const SolveState* st;
  ReduceBuf rb;
  __device__ bool prepare() { return st && st->done; }
  __device__ int tiles() const { return ntot; }
  __device__ void stage(unsigned char* buf, int id) const {
    const Tile<RTI, RTJ> t = tile_at<RTI, RTJ>(id, ntx, nc);
    const int m = t.i_hi - t.i_lo, mp = t.j_hi - t.j_lo;
    const int ri0 = 2 * t.i_lo - 1, rj0 = 2 * t.j_lo - 1;
    stage_async<RRI>(reinterpret_cast<T*>(buf), b, ri0, rj0, 2 * m + 1, 2 * mp + 1, nf);
    if (v.p)
      stage_async<RVI>(reinterpret_cast<T*>(buf + kOffV), v, ri0 - 1, rj0 - 1, 2 * m + 3,
                       2 * mp + 3, nf);
  }
  __device__ void compute(unsigned char* buf, int id, Acc&) const {
    const Tile<RTI, RTJ> t = tile_at<RTI, RTJ>(id, ntx, nc);
    T* sr = reinterpret_cast<T*>(buf);
    const T* sv = reinterpret_cast<const T*>(buf + kOffV);
    const int m = t.i_hi - t.i_lo, mp = t.j_hi - t.j_lo;
    const int ri0 = 2 * t.i_lo - 1, rj0 = 2 * t.j_lo - 1;
    const int rei = 2 * m + 1, rej = 2 * mp + 1;
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
            acc = fma(wi * wj, sr[(2 * c + 1 + bj) * RRI + (2 * r + 1 + ai)], acc);
          }
        }
        f.at(I, J) = acc;
      }
    }
  }
  __device__ void finish(double) const {}
};

template <typename T>
cudaError_t launch_resrestrict(Grid<const T> v, Grid<const T> b, Grid<T> f, int nf, int kind,
                               const SolveState* st, cudaStream_t s) {
  const int nc = (nf + 1) / 2;
  const int ntx = ntiles(nc, RTI), nty = ntiles(nc, RTJ);
  const int total = ntx * nty;
  return launch_persist(ResRestrictJob<T>{v, b, f, nf, nc, ntx, total, kind, st, ReduceBuf{}},
                        total, s);
}

// Resolve the launch configuration of every persistent kernel up front
// (shared-memory attribute and occupancy), outside any stream capture.
template <typename T>
static void prepare_precision() {
  persist_ctas_per_sm<ApplyJob<T, false>>();
  persist_ctas_per_sm<ApplyJob<T, true>>();
  persist_ctas_per_sm<ResidualJob<T>>();
  persist_ctas_per_sm<ResRestrictJob<T>>();
  persist_ctas_per_sm<SmoothJob<T, kFieldPlain, kEpiSweep, false>>();
  persist_ctas_per_sm<SmoothJob<T, kFieldPlain, kEpiSweep, true>>();
  persist_ctas_per_sm<SmoothJob<T, kFieldPlain, kEpiStore, false>>();
  persist_ctas_per_sm<SmoothJob<T, kFieldPlain, kEpiStore, true>>();
  persist_ctas_per_sm<SmoothJob<T, kFieldZero, kEpiSweep, false>>();
  persist_ctas_per_sm<SmoothJob<T, kFieldZero, kEpiSweep, true>>();
  persist_ctas_per_sm<SmoothJob<T, kFieldZero, kEpiStore, false>>();
  persist_ctas_per_sm<SmoothJob<T, kFieldZero, kEpiStore, true>>();
  persist_ctas_per_sm<SmoothJob<T, kFieldProlong, kEpiSweep, false>>();
  persist_ctas_per_sm<SmoothJob<T, kFieldProlong, kEpiSweep, true>>();
  persist_ctas_per_sm<SmoothJob<T, kFieldProlong, kEpiStore, false>>();
  persist_ctas_per_sm<SmoothJob<T, kFieldProlong, kEpiStore, true>>();
}

cudaError_t prepare_kernels() {
  sm_count();
  prepare_precision<double>();
  prepare_precision<float>();
  persist_ctas_per_sm<CgDirJob<double, double>>();
  persist_ctas_per_sm<CgDirJob<double, float>>();
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
    sf[k] = convert<double>(f.at(i, j));
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
      e.at(i, j) = convert<T>(acc);
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

// SBP-SAT Poisson kernels for sm_103a: operator apply, fused CG updates,
// multigrid smoothing / transfer / coarse solve, right-hand-side assembly.
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <type_traits>
#include <cstring>
#include <climits>
#include <mutex>
#include <utility>

#include "sbp_coarse.h"
#include "sbp_kernels.cuh"
#include "sbp_launch.h"
#include "sbp_tma.h"

namespace sbp {

// ---------------------------------------------------------------------------
// Tiling.  Output tiles are 64 (i) x 32 (j) points; tile t of a dimension
// covers [t*T + (t > 0), (t+1)*T + 1), so n = 2^k + 1 splits into whole tiles
// (the extra point goes to the first tile).  Every tile stages fixed boxes:
//   stencil box 72 x 37 at (64 ti - 4, j_lo - 2)   operand + halo (>= 2 in j)
//   inner box   68 x 33 at (64 ti,     j_lo)       pointwise operands
//   coarse box  40 x 20 at (32 ti - 4, (j_lo-2)>>1) prolongation source
// The x origins are multiples of four elements (16 bytes for FP32), as TMA
// requires; out-of-range elements read as zero.  The same boxes are staged
// element-wise with cp.async when an operand is not TMA-addressable (the
// caller's own arrays: n is odd, so their columns are not 16-byte aligned).
// ---------------------------------------------------------------------------
constexpr int TI = 64;
constexpr int TJ = 32;
using TileT = Tile<TI, TJ>;
constexpr int BI = kBoxI, BJ = kBoxJ;   // stencil box
constexpr int QI = kInI, QJ = kInJ;     // inner box
constexpr int CI = kCoI, CJ = kCoJ;     // coarse box
static_assert(BI >= TI + 8 && BJ >= TJ + 5 && QI >= TI + 4 && QJ >= TJ + 1, "box sizes");

// Coarse tile of the fused residual + restriction kernel: its fine region
// fits the same 72 x 37 stencil box at (64 ti - 4, 32 tj - 2).
constexpr int RTI = 32;
constexpr int RTJ = 16;

// Coarse dense solve: rows of Ainv per warp.
// Flat (pointwise) kernels: CTAs per launch cap.
constexpr int kFlatCtas = 1216;
// Upper bound on the CTAs of a persistent launch (SMs x resident CTAs).

__host__ __device__ constexpr int align128(int b) { return (b + 127) & ~127; }

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
// Operand staging: a TMA map when the operand allows it, else element-wise
// cp.async of the same box.
// ---------------------------------------------------------------------------
template <typename T>
struct DevOperand {
  const T* p;
  int ld;
  CUtensorMap box;
  CUtensorMap inner;
  CUtensorMap coarse;
};

template <typename T>
static DevOperand<T> dev_operand(const Operand& o) {
  DevOperand<T> d;
  d.p = static_cast<const T*>(o.p);
  d.ld = o.ld;
  d.box = o.box;
  d.inner = o.inner;
  d.coarse = o.coarse;
  return d;
}

// Stage a BW x BH box at (x0, y0) of an n x n operand into s (pitch BW).
// TMA: thread 0 issues it (the caller has armed `bar` with the byte count).
// cp.async: every thread copies its share; out-of-range elements are zeroed.
template <bool TMA, int BW, int BH, typename T>
__device__ __forceinline__ void stage_box(T* s, const DevOperand<T>& op, const CUtensorMap* map,
                                          int x0, int y0, int n, unsigned long long* bar) {
  if (TMA) {
    if (threadIdx.x == 0) tma_load_2d(s, map, x0, y0, bar);
  } else {
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    if (x0 >= 0 && y0 >= 0 && x0 + BW <= n && y0 + BH <= n) {
      // the box lies inside the array: no bounds checks, pointer increments
      for (int c = w; c < BH; c += kWarps) {
        const T* src = op.p + (size_t)(y0 + c) * (size_t)op.ld + (x0 + lane);
        T* dst = s + c * BW + lane;
#pragma unroll
        for (int r = 0; r < BW; r += 32)
          if (r + lane < BW) cp_async_elem(dst + r, src + r);
      }
      return;
    }
    for (int c = w; c < BH; c += kWarps) {
      const int j = y0 + c;
      const bool jok = (j >= 0 && j < n);
      for (int r = lane; r < BW; r += 32) {
        const int i = x0 + r;
        if (jok && i >= 0 && i < n)
          cp_async_elem(&s[c * BW + r], op.p + (size_t)j * op.ld + i);
        else
          s[c * BW + r] = T(0);
      }
    }
  }
}

template <typename T, int BW, int BH>
__host__ __device__ constexpr unsigned box_bytes() {
  return (unsigned)(sizeof(T) * BW * BH);
}

// Fine-tile box origins.
struct TileBoxes {
  int x0, y0;    // stencil box
  int xi, yi;    // inner box
  int xc, yc;    // coarse box
  __device__ __forceinline__ TileBoxes(int ti, int j_lo) {
    x0 = 64 * ti - 4;
    y0 = j_lo - 2;
    xi = 64 * ti;
    yi = j_lo;
    xc = 32 * ti - 4;
    yc = (j_lo - 2) >> 1;
  }
};

template <int A, int B>
__device__ __forceinline__ bool tile_interior(const Tile<A, B>& t, int n) {
  return t.i_lo > 0 && t.i_hi < n && t.j_lo > 2 && t.j_hi < n - 3;
}

// Generic visitor (any tile): fn(i, j, SAcc centred on (i, j), inner index).
template <typename T, typename Fn>
__device__ __forceinline__ void visit_generic(const T* s, const TileT& t, const TileBoxes& bx,
                                              Fn&& fn) {
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const int mi = t.i_hi - t.i_lo;
  const int mj = t.j_hi - t.j_lo;
  for (int c = w; c < mj; c += kWarps) {
    const int j = t.j_lo + c;
    for (int r = lane; r < mi; r += 32) {
      const int i = t.i_lo + r;
      SAcc<T> a{s + (j - bx.y0) * BI + (i - bx.x0), BI};
      fn(i, j, a, (j - bx.yi) * QI + (i - bx.xi));
    }
  }
}

// Interior tile (64 x 32, every point a plain 5-point stencil): thread
// (r = tid & 63, g = tid >> 6) marches down columns 8g..8g+7 of row r,
// keeping the j-1 / j / j+1 values in registers.  fn(i, j, um, u0, up, uw,
// ue, inner index).
template <typename T, typename Fn>
__device__ __forceinline__ void visit_interior(const T* s, const TileT& t, Fn&& fn) {
  const int r = threadIdx.x & 63;
  const int g = threadIdx.x >> 6;
  // stencil box: i - x0 = r + 5, j - y0 = c + 2; inner box: i - xi = r + 1, j - yi = c
  const T* col = s + (8 * g + 2) * BI + r + 5;
  T um = col[-BI];
  T u0 = col[0];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const T up = col[(q + 1) * BI];
    const T uw = col[q * BI - 1];
    const T ue = col[q * BI + 1];
    fn(t.i_lo + r, t.j_lo + 8 * g + q, um, u0, up, uw, ue, (8 * g + q) * QI + r + 1);
    um = u0;
    u0 = up;
  }
}

// Apply fn(i, j, value&) to the staged box points a tile's stencil reads:
// rows [i_lo-1, i_hi], columns [j_lo-hl, j_hi+hr-1], inside the domain.
template <typename T, typename Fn>
__device__ __forceinline__ void transform_box(T* s, const TileT& t, const TileBoxes& bx, int n,
                                              Fn&& fn) {
  const int i0 = max(t.i_lo - 1, 0), i1 = min(t.i_hi, n - 1);
  const int j0 = max(t.j_lo - t.hl, 0), j1 = min(t.j_hi + t.hr - 1, n - 1);
  const int ei = i1 - i0 + 1;
  const int ej = j1 - j0 + 1;
  const int cnt = ei * ej;
  for (int k = threadIdx.x; k < cnt; k += kThreads) {
    const int c = k / ei;
    const int r = k - c * ei;
    const int i = i0 + r, j = j0 + c;
    fn(i, j, s[(j - bx.y0) * BI + (i - bx.x0)]);
  }
}

// ---------------------------------------------------------------------------
// Persistent, double-buffered tile pipeline.  A CTA walks tiles blockIdx.x,
// blockIdx.x + gridDim.x, ...; while it computes tile k from one buffer, the
// copies of tile k+1 (TMA boxes completing on an mbarrier, or cp.async) are
// already in flight into the other, so HBM latency overlaps compute.  The
// grid is one wave (SMs x resident CTAs), so neighbouring CTAs work on
// neighbouring tiles and halo re-reads hit L2.
//
// A Job provides: kStage (bytes of one buffer), kReduce, Acc, Ctx (per-launch
// values read from device state), prepare(ctx) (true = skip the launch),
// tiles(), tx_bytes(tile) (TMA bytes of one stage), issue(buf, bar, tile, ctx)
// (called by all threads), compute(buf, tile, acc, ctx) and finish(total).
// ---------------------------------------------------------------------------
template <class Job>
__global__ void __launch_bounds__(kThreads) k_persist(const __grid_constant__ Job job) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) unsigned long long bar[2];
  pdl_begin();
  typename Job::Ctx ctx;
  if (job.prepare(ctx)) return;
  const int total = job.tiles();
  // TMA destinations must sit on 128-byte shared-memory boundaries; the
  // launch reserves 128 extra bytes for this alignment.
  unsigned char* const smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  unsigned char* const buf0 = smem;
  unsigned char* const buf1 = smem + Job::kStage;
  unsigned char* const scratch = smem + 2 * Job::kStage;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  typename Job::Acc acc;
  int tile = blockIdx.x;
  if (tile < total) {
    const unsigned tx = job.tx_bytes(tile);
    if (threadIdx.x == 0) mbar_arrive_expect_tx(&bar[0], tx);
    // failure test only: the declared copy is never issued (TMA stages)
    const bool drop = tx != 0u && blockIdx.x == 0 && g_sbp_drop_copy != 0u;
    if (!drop) job.issue(buf0, &bar[0], tile, ctx);
  }
  cp_async_commit();
  bool ok = true;
  for (int k = 0; tile < total; ++k, tile += gridDim.x) {
    const int next = tile + gridDim.x;
    const int nb = (k + 1) & 1;
    if (next < total) {
      if (threadIdx.x == 0) {
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&bar[nb], job.tx_bytes(next));
      }
      job.issue(nb ? buf1 : buf0, &bar[nb], next, ctx);
    }
    cp_async_commit();
    cp_async_wait<1>();
    // TMA stages: one thread observes the transaction barrier, the block
    // barrier then orders the staged data for every thread (and gives every
    // thread the same result)
    bool arrived = true;
    if (threadIdx.x == 0) arrived = mbar_wait_bounded(&bar[k & 1], (k >> 1) & 1);
    ok = __syncthreads_and(arrived);
    if (!ok) {
      // the copy of `next` into the other buffer may still be in flight:
      // wait for it (bounded) so that no copy lands after the CTA has left
      if (threadIdx.x == 0 && next < total) mbar_wait_bounded(&bar[nb], ((k + 1) >> 1) & 1);
      __syncthreads();
      break;
    }
    job.compute((k & 1) ? buf1 : buf0, tile, acc, ctx, scratch);
    // this buffer is refilled by TMA (async proxy) after the barrier
    fence_proxy_async_smem();
    __syncthreads();
  }
  cp_async_wait<0>();
  // A CTA whose copy never arrived still takes part in the reduction, with a
  // NaN partial: the ticket count stays whole (the last CTA resets it for the
  // next launch) and the result is non-finite, which the solver reports as a
  // breakdown; the fault flag is set as well.
  if (Job::kReduce)
    grid_reduce(ok ? acc.value() : __longlong_as_double(0x7ff8000000000000LL), job.rb,
                [&](double tot) { job.finish(tot); });
}

// ---------------------------------------------------------------------------
// Batched persistent kernel: `count` problems, each with its own Job (tensor
// maps included) in device memory, `tpp` tiles each; work item id covers
// problem id / tpp, tile id % tpp.  A CTA visits problems in increasing order,
// keeps one accumulator per visited problem (block-summed into shared
// memory when the problem changes), writes all `count` per-problem partials
// at the end ([cta][problem], coalesced), and the last CTA finishes each
// problem on its own thread (partials summed in CTA order: deterministic).
// Problems whose prepare() says skip (done) stage nothing and compute
// nothing.
// ---------------------------------------------------------------------------
template <class Job>
constexpr size_t batch_smem_bytes() {
  return (size_t)(2 * Job::kStage + Job::kScratch + 128) +
         (Job::kReduce ? (size_t)kMaxBatchSlots * sizeof(double) : 0);
}

template <class Job>
__global__ void __launch_bounds__(kThreads)
    k_persist_batch(const unsigned char* __restrict__ blobs, int stride, int count, int tpp,
                    double* partials, unsigned* ticket) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) unsigned long long bar[2];
  __shared__ bool is_last;
  pdl_begin();
  const int total = count * tpp;
  unsigned char* const smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  unsigned char* const buf0 = smem;
  unsigned char* const buf1 = smem + Job::kStage;
  unsigned char* const scratch = smem + 2 * Job::kStage;
  double* const slot_part = reinterpret_cast<double*>(scratch + Job::kScratch);
  auto job_at = [&](int slot) -> const Job& {
    return *reinterpret_cast<const Job*>(blobs + (size_t)slot * (size_t)stride);
  };
  if (Job::kReduce)
    for (int k = threadIdx.x; k < count; k += kThreads) slot_part[k] = 0.0;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  // stage tile `id` into buf on barrier b (problems that are done: an empty
  // transaction, so the barrier phase still completes)
  auto stage = [&](int id, unsigned char* buf, unsigned long long* b, bool fence) {
    const int slot = id / tpp;
    const Job& J = job_at(slot);
    typename Job::Ctx c;
    const bool act = !J.prepare(c);
    if (threadIdx.x == 0) {
      if (fence) fence_proxy_async_smem();
      mbar_arrive_expect_tx(b, act ? J.tx_bytes(id - slot * tpp) : 0u);
    }
    if (act) J.issue(buf, b, id - slot * tpp, c);
  };
  typename Job::Acc acc;
  int cur = -1;   // problem of acc
  auto flush = [&]() {
    const double v = block_sum(acc.value());
    if (threadIdx.x == 0) slot_part[cur] = v;
  };
  int tile = blockIdx.x;
  if (tile < total) stage(tile, buf0, &bar[0], false);
  cp_async_commit();
  bool ok = true;
  for (int k = 0; tile < total; ++k, tile += gridDim.x) {
    const int next = tile + gridDim.x;
    const int nb = (k + 1) & 1;
    if (next < total) stage(next, nb ? buf1 : buf0, &bar[nb], true);
    cp_async_commit();
    cp_async_wait<1>();
    bool arrived = true;
    if (threadIdx.x == 0) arrived = mbar_wait_bounded(&bar[k & 1], (k >> 1) & 1);
    ok = __syncthreads_and(arrived);
    if (!ok) {
      // drain the copy of `next` (bounded) before the CTA leaves
      if (threadIdx.x == 0 && next < total) mbar_wait_bounded(&bar[nb], ((k + 1) >> 1) & 1);
      __syncthreads();
      break;
    }
    const int slot = tile / tpp;
    if (Job::kReduce && slot != cur) {
      if (cur >= 0) flush();
      cur = slot;
      acc = typename Job::Acc{};
    }
    const Job& J = job_at(slot);
    typename Job::Ctx c;
    if (!J.prepare(c)) J.compute((k & 1) ? buf1 : buf0, tile - slot * tpp, acc, c, scratch);
    fence_proxy_async_smem();
    __syncthreads();
  }
  cp_async_wait<0>();
  if (!Job::kReduce) return;
  if (cur >= 0) flush();
  __syncthreads();
  // a copy never arrived: every problem gets a NaN partial from this CTA (the
  // ticket count stays whole; the results are non-finite, the fault flag set)
  if (!ok)
    for (int k = threadIdx.x; k < count; k += kThreads)
      slot_part[k] = __longlong_as_double(0x7ff8000000000000LL);
  __syncthreads();
  for (int k = threadIdx.x; k < count; k += kThreads)
    partials[(size_t)blockIdx.x * count + k] = slot_part[k];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) is_last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  for (int k = threadIdx.x; k < count; k += kThreads) {
    double tot = 0.0;
    for (unsigned c = 0; c < gridDim.x; ++c) tot += __ldcg(partials + (size_t)c * count + k);
    const Job& J = job_at(k);
    typename Job::Ctx c;
    if (!J.prepare(c)) J.finish(tot);
  }
  __syncthreads();
  if (threadIdx.x == 0) *ticket = 0u;
}

template <class Job>
static int batch_ctas_per_sm() {
  static const int v = [] {
    const int smem = (int)batch_smem_bytes<Job>();
    if (smem > 48 * 1024)
      cudaFuncSetAttribute(k_persist_batch<Job>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           smem);
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_persist_batch<Job>, kThreads, smem) !=
            cudaSuccess ||
        b < 1)
      b = 1;
    return b;
  }();
  return v;
}

// BatchLaunchFn of a persistent job: aux[0] = tiles per problem.
template <class Job>
cudaError_t launch_persist_batch(const unsigned char* blobs, int stride, int count, const int* aux,
                                 const BatchScratch& scr, cudaStream_t s) {
  int cap = std::min(kMaxPersistCtas, sm_count() * batch_ctas_per_sm<Job>());
  if (scr.cta_budget > 0) cap = std::min(cap, scr.cta_budget);
  if (count == 0) return cudaGetLastError();
  if (count > kMaxBatchSlots || stride % alignof(Job) != 0) return cudaErrorInvalidValue;
  const long long total = (long long)count * aux[0];
  if (total > INT_MAX) return cudaErrorInvalidValue;
  const int grid = (int)std::max(1LL, std::min<long long>(total, cap));
  if (Job::kReduce && (long long)grid * count > scr.cap) return cudaErrorInvalidValue;
  return launch_pdl(k_persist_batch<Job>, dim3(grid), dim3(kThreads), batch_smem_bytes<Job>(), s,
                    blobs, stride, count, aux[0], scr.partials, scr.ticket);
}

int batch_sm_count() { return sm_count(); }

Recorder*& recorder_slot() {
  static thread_local Recorder* r = nullptr;
  return r;
}

LaunchTimer*& timer_slot() {
  static thread_local LaunchTimer* t = nullptr;
  return t;
}

void timer_mark(LaunchTimer* t, const void* fn, cudaStream_t s, bool after) {
  if (!after) {
    LaunchTimer::Rec r;
    r.fn = fn;
    if (cudaEventCreate(&r.e0) != cudaSuccess || cudaEventCreate(&r.e1) != cudaSuccess) {
      t->failed = true;
      return;
    }
    cudaEventRecord(r.e0, s);
    t->recs.push_back(r);
  } else if (!t->recs.empty() && t->recs.back().fn == fn) {
    cudaEventRecord(t->recs.back().e1, s);
  }
}

template <class Args>
static cudaError_t record_launch(BatchLaunchFn fn, const Args& a, int aux0, int aux1 = 0,
                                 int aux2 = 0, int aux3 = 0) {
  static_assert(std::is_trivially_copyable<Args>::value, "launch arguments are copied as bytes");
  LaunchRecord r;
  r.fn = fn;
  r.aux[0] = aux0;
  r.aux[1] = aux1;
  r.aux[2] = aux2;
  r.aux[3] = aux3;
  r.align = (int)std::max<size_t>(16, alignof(Args));
  r.blob.resize(sizeof(Args));
  std::memcpy(r.blob.data(), &a, sizeof(Args));
  recorder_slot()->recs.push_back(std::move(r));
  return cudaSuccess;
}

template <class Job>
static int persist_ctas_per_sm() {
  static const int v = [] {
    const int smem = 2 * Job::kStage + Job::kScratch + 128;
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
  if (recorder_slot()) return record_launch(&launch_persist_batch<Job>, job, total);
  const int cap = std::min(kMaxPersistCtas, sm_count() * persist_ctas_per_sm<Job>());
  const int grid = std::max(1, std::min(total, cap));
  return launch_pdl(k_persist<Job>, dim3(grid), dim3(kThreads),
                    (size_t)(2 * Job::kStage + Job::kScratch + 128), s, job);
}

struct NoCtx {};

// ---------------------------------------------------------------------------
// Operator apply: out = sign * A u, optional fused dot u.out.
// ---------------------------------------------------------------------------
// Thread groups (64 threads each, 4 per CTA) of the FP64 apply that use FP64
// instructions for the interior stencil; the rest use the integer pipe.
constexpr int kFp64Groups = 2;
// The same split for FP64 kernels that also spend FP64 instructions outside
// the stencil (sweeps, residuals, CG direction): one group on the FP64 pipe.
constexpr int kFp64GroupsFused = 1;

// S = (uw + ue) + (um + up) - 4 u0, i.e. (-A u) at an interior point.  FP64
// with `exact`: the integer-pipe sum of exact_stencil5 (FP64 instructions
// when it declines); otherwise one FP add chain + FMA in T.
template <typename T>
__device__ __forceinline__ T neg_stencil(T um, T u0, T up, T uw, T ue, bool exact) {
  if constexpr (sizeof(T) == 8) {
    double sx;
    if (exact && exact_stencil5((double)u0, (double)uw, (double)ue, (double)um, (double)up, sx))
      return (T)sx;
  }
  return fma(T(-4), u0, (uw + ue) + (um + up));
}
// This thread's group uses the integer path (FP64 kernels only).
template <typename T, int FP64_GROUPS>
__device__ __forceinline__ bool exact_group() {
  return sizeof(T) == 8 && (int)(threadIdx.x >> 6) >= FP64_GROUPS;
}

template <typename T, bool DOT, bool TMA>
struct ApplyJob {
  static constexpr int kStage = align128(box_bytes<T, BI, BJ>());
  static constexpr int kScratch = 0;
  static constexpr bool kReduce = DOT;
  using Acc = DotAcc<T>;
  using Ctx = NoCtx;
  DevOperand<T> u;
  Grid<T> out;
  int n, ntx, ntot, sign;
  ReduceBuf rb;
  double* dot_out;
  __device__ bool prepare(Ctx&) const { return false; }
  __device__ int tiles() const { return ntot; }
  __device__ unsigned tx_bytes(int) const { return TMA ? box_bytes<T, BI, BJ>() : 0u; }
  __device__ void issue(unsigned char* buf, unsigned long long* bar, int id, const Ctx&) const {
    const TileBoxes bx(id % ntx, tile_at<TI, TJ>(id, ntx, n).j_lo);
    stage_box<TMA, BI, BJ>(reinterpret_cast<T*>(buf), u, &u.box, bx.x0, bx.y0, n, bar);
  }
  __device__ void compute(unsigned char* buf, int id, Acc& acc, const Ctx&, unsigned char*) const {
    const TileT t = tile_at<TI, TJ>(id, ntx, n);
    const TileBoxes bx(id % ntx, t.j_lo);
    const T* s = reinterpret_cast<const T*>(buf);
    if (tile_interior(t, n)) {
      // FP64: thread groups g >= kFp64Groups form the sum on the integer pipe
      // (exact_stencil5), the others with FP64 instructions, so both pipes
      // are busy; FP32: the FP32 pipe.
      const bool exact = sizeof(T) == 8 && (threadIdx.x >> 6) >= kFp64Groups;
      visit_interior(s, t, [&](int i, int j, T um, T u0, T up, T uw, T ue, int) {
        T v;
        double sx;
        if (exact && exact_stencil5((double)u0, (double)uw, (double)ue, (double)um, (double)up,
                                    sx)) {
          v = (T)(sign > 0 ? -sx : sx);
        } else {
          const T sum = (uw + ue) + (um + up);
          v = sign > 0 ? fma(T(4), u0, -sum) : fma(T(-4), u0, sum);
        }
        out.at(i, j) = v;
        if (DOT) acc.add_prod(u0, v);
      });
    } else {
      visit_generic(s, t, bx, [&](int i, int j, const SAcc<T>& a, int) {
        const T v = signedA<T>(a, i, j, n, sign);
        out.at(i, j) = v;
        if (DOT) acc.add_prod(a(0, 0), v);
      });
    }
  }
  __device__ void finish(double tot) const { *dot_out = tot; }
};

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

template <typename T, bool TMAX, bool TMAB>
struct ResidualJob {
  static constexpr int kOffB = align128(box_bytes<T, BI, BJ>());
  static constexpr int kStage = kOffB + align128(box_bytes<T, QI, QJ>());
  static constexpr int kScratch = 0;
  static constexpr bool kReduce = true;
  using Acc = DotAcc<double>;
  using Ctx = NoCtx;
  DevOperand<T> x, b;
  Grid<T> r;
  Grid<float> rlo;
  int n, ntx, ntot, opsign;
  ResFin rf;
  ReduceBuf rb;
  // when set, x is also written here (the solver's padded iterate): the
  // copy of the caller's x rides on the residual pass
  Grid<T> xcopy;
  __device__ bool prepare(Ctx&) const { return false; }
  __device__ int tiles() const { return ntot; }
  __device__ unsigned tx_bytes(int) const {
    return (TMAX ? box_bytes<T, BI, BJ>() : 0u) + (TMAB ? box_bytes<T, QI, QJ>() : 0u);
  }
  __device__ void issue(unsigned char* buf, unsigned long long* bar, int id, const Ctx&) const {
    const TileBoxes bx(id % ntx, tile_at<TI, TJ>(id, ntx, n).j_lo);
    stage_box<TMAX, BI, BJ>(reinterpret_cast<T*>(buf), x, &x.box, bx.x0, bx.y0, n, bar);
    stage_box<TMAB, QI, QJ>(reinterpret_cast<T*>(buf + kOffB), b, &b.inner, bx.xi, bx.yi, n, bar);
  }
  __device__ void compute(unsigned char* buf, int id, Acc& acc, const Ctx&, unsigned char*) const {
    const TileT t = tile_at<TI, TJ>(id, ntx, n);
    const TileBoxes bx(id % ntx, t.j_lo);
    const T* s = reinterpret_cast<const T*>(buf);
    const T* sb = reinterpret_cast<const T*>(buf + kOffB);
    auto emit = [&](int i, int j, T rv, T xv) {
      if (xcopy.p) xcopy.at(i, j) = xv;
      r.at(i, j) = rv;
      if (rlo.p) rlo.at(i, j) = convert<float>(rv);
      acc.add_prod((double)rv, (double)rv);
    };
    if constexpr (sizeof(T) == 8) {
      // The iterate is zero on the whole stencil box (a zero initial guess):
      // r = b exactly, without FP64 stencil arithmetic.
      const unsigned long long* w = reinterpret_cast<const unsigned long long*>(s);
      int nz = 0;
      for (int k = threadIdx.x; k < BI * BJ; k += kThreads) nz |= (w[k] << 1) != 0ull;
      if (!__syncthreads_or(nz)) {
        visit_generic(s, t, bx,
                      [&](int i, int j, const SAcc<T>& a, int k) { emit(i, j, sb[k], a(0, 0)); });
        return;
      }
    }
    if (tile_interior(t, n)) {
      const bool exact = exact_group<T, kFp64GroupsFused>();
      visit_interior(s, t, [&](int i, int j, T um, T u0, T up, T uw, T ue, int k) {
        // r = b - opsign*A x, A x = 4 u0 - sum = -S
        const T S = neg_stencil<T>(um, u0, up, uw, ue, exact);
        emit(i, j, opsign > 0 ? sb[k] + S : sb[k] - S, u0);
      });
    } else {
      visit_generic(s, t, bx, [&](int i, int j, const SAcc<T>& a, int k) {
        emit(i, j, sb[k] + signedA<T>(a, i, j, n, -opsign), a(0, 0));
      });
    }
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

// ---------------------------------------------------------------------------
// CG direction + operator + p.Ap  (one HBM pass: reads z, p_old; writes p, Ap)
// ---------------------------------------------------------------------------
struct DirCtx {
  bool first;
  double beta;
};

template <typename T, typename Tz, bool TMA>
struct CgDirJob {
  static constexpr int kOffZ = align128(box_bytes<T, BI, BJ>());
  static constexpr int kStage = kOffZ + align128(box_bytes<Tz, BI, BJ>());
  static constexpr int kScratch = 0;
  static constexpr bool kReduce = true;
  using Acc = DotAcc<double>;
  using Ctx = DirCtx;
  DevOperand<Tz> z;
  DevOperand<T> pold;
  Grid<T> pnew, Ap;
  int n, ntx, ntot, opsign;
  SolveState* st;
  ReduceBuf rb;
  __device__ bool prepare(Ctx& c) const {
    if (st->done) return true;
    c.first = (st->iter == 0);
    c.beta = st->beta;
    return false;
  }
  __device__ int tiles() const { return ntot; }
  __device__ unsigned tx_bytes(int) const {
    // on the first iteration p_old is not read; prepare() is per CTA, so the
    // byte count is recomputed from the state here
    return TMA ? box_bytes<Tz, BI, BJ>() + (st->iter == 0 ? 0u : box_bytes<T, BI, BJ>()) : 0u;
  }
  __device__ void issue(unsigned char* buf, unsigned long long* bar, int id, const Ctx& c) const {
    const TileBoxes bx(id % ntx, tile_at<TI, TJ>(id, ntx, n).j_lo);
    stage_box<TMA, BI, BJ>(reinterpret_cast<Tz*>(buf + kOffZ), z, &z.box, bx.x0, bx.y0, n, bar);
    if (!c.first)
      stage_box<TMA, BI, BJ>(reinterpret_cast<T*>(buf), pold, &pold.box, bx.x0, bx.y0, n, bar);
  }
  __device__ void compute(unsigned char* buf, int id, Acc& acc, const Ctx& c, unsigned char*) const {
    const TileT t = tile_at<TI, TJ>(id, ntx, n);
    const TileBoxes bx(id % ntx, t.j_lo);
    T* s = reinterpret_cast<T*>(buf);
    const Tz* sz = reinterpret_cast<const Tz*>(buf + kOffZ);
    const T beta = T(c.beta);
    const bool first = c.first;
    // p = z + beta p_old on every staged point the stencil reads
    transform_box(s, t, bx, n, [&](int i, int j, T& v) {
      const T zz = convert<T>(sz[&v - s]);
      v = first ? zz : fma(beta, v, zz);
    });
    __syncthreads();
    auto emit = [&](int i, int j, T pv, T ap) {
      pnew.at(i, j) = pv;
      Ap.at(i, j) = ap;
      acc.add_prod(pv, ap);
    };
    if (tile_interior(t, n)) {
      const bool exact = exact_group<T, kFp64GroupsFused>();
      visit_interior(s, t, [&](int i, int j, T um, T u0, T up, T uw, T ue, int) {
        const T S = neg_stencil<T>(um, u0, up, uw, ue, exact);   // -A p
        emit(i, j, u0, opsign > 0 ? -S : S);
      });
    } else {
      visit_generic(s, t, bx, [&](int i, int j, const SAcc<T>& a, int) {
        emit(i, j, a(0, 0), signedA<T>(a, i, j, n, opsign));
      });
    }
  }
  __device__ void finish(double tot) const {
    st->pAp = tot;
    if (!isfinite(tot) || tot == 0.0)
      st->done = kDoneBreakdown;
    else
      st->alpha = st->rz / tot;
  }
};


// ---------------------------------------------------------------------------
// Mixed-precision CG direction with an FP32 direction vector:
//   p~ = fl32(z + beta p~_old)      (z and p~_old FP32, staged with halos)
//   Ap = A p~                       (exact: float-float stencil of FP32 values)
//   p~.Ap -> alpha
// x += alpha p~ and r -= alpha Ap then use the same p~, so the recurrence
// residual stays the residual of x in FP64; rounding the direction to FP32
// only perturbs its conjugacy (by ~6e-8, below the FP32 V-cycle's own
// perturbation of z).  20 bytes per point instead of 36, and no FP64
// instruction per point besides the conversion of A p~ to FP64.
// ---------------------------------------------------------------------------
// A p~ at one point from the float pair hi + lo of -A p~ (negA; the plain
// 5-point stencil in the interior): FP64 for the Krylov vectors (rounded
// once, without FP64 arithmetic), and in apf its FP32 rounding for p~.Ap.
__device__ __forceinline__ double dir_ap(float hi, float lo, float& apf) {
  apf = -(hi + lo);
  return ff_neg_f64(hi, lo);
}

// The end of the direction pass's p.Ap reduction: pAp and alpha.
__device__ __forceinline__ void finish_pap(SolveState* st, double tot) {
  st->pAp = tot;
  if (!isfinite(tot) || tot == 0.0)
    st->done = kDoneBreakdown;
  else
    st->alpha = st->rz / tot;
}

template <bool TMA>
struct CgDirF32Job {
  static constexpr int kOffZ = align128(box_bytes<float, BI, BJ>());
  static constexpr int kStage = kOffZ + align128(box_bytes<float, BI, BJ>());
  static constexpr int kScratch = 0;
  static constexpr bool kReduce = true;
  // p~.Ap from the FP32 rounding of Ap, accumulated with the compensated
  // float pair (alpha and beta only need ~1e-7)
  using Acc = DotAcc<float>;
  using Ctx = DirCtx;
  DevOperand<float> z, pold;
  Grid<float> pnew;
  Grid<double> Ap;
  int n, ntx, ntot;
  SolveState* st;
  ReduceBuf rb;
  __device__ bool prepare(Ctx& c) const {
    if (st->done) return true;
    c.first = (st->iter == 0);
    c.beta = st->beta;
    return false;
  }
  __device__ int tiles() const { return ntot; }
  __device__ unsigned tx_bytes(int) const {
    // on the first iteration p~_old is not read
    return TMA ? box_bytes<float, BI, BJ>() + (st->iter == 0 ? 0u : box_bytes<float, BI, BJ>())
               : 0u;
  }
  __device__ void issue(unsigned char* buf, unsigned long long* bar, int id, const Ctx& c) const {
    const TileBoxes bx(id % ntx, tile_at<TI, TJ>(id, ntx, n).j_lo);
    stage_box<TMA, BI, BJ>(reinterpret_cast<float*>(buf + kOffZ), z, &z.box, bx.x0, bx.y0, n, bar);
    if (!c.first)
      stage_box<TMA, BI, BJ>(reinterpret_cast<float*>(buf), pold, &pold.box, bx.x0, bx.y0, n,
                             bar);
  }
  __device__ void compute(unsigned char* buf, int id, Acc& acc, const Ctx& c, unsigned char*) const {
    const TileT t = tile_at<TI, TJ>(id, ntx, n);
    const TileBoxes bx(id % ntx, t.j_lo);
    float* s = reinterpret_cast<float*>(buf);
    const float* sz = reinterpret_cast<const float*>(buf + kOffZ);
    const float beta = (float)c.beta;
    const bool first = c.first;
    // p~ on every staged point the stencil reads (each tile computes the
    // same value for a shared halo point: same inputs, same instruction)
    transform_box(s, t, bx, n, [&](int, int, float& v) {
      const float zz = sz[&v - s];
      v = first ? zz : fmaf(beta, v, zz);
    });
    __syncthreads();
    auto emit = [&](int i, int j, float pv, float hi, float lo) {
      float apf;
      pnew.at(i, j) = pv;
      Ap.at(i, j) = dir_ap(hi, lo, apf);
      acc.add_prod(pv, apf);
    };
    if (tile_interior(t, n)) {
      visit_interior(s, t, [&](int i, int j, float um, float u0, float up, float uw, float ue,
                               int) {
        float hi, lo;
        stencil_ff(uw, ue, um, up, u0, hi, lo);
        emit(i, j, u0, hi, lo);
      });
    } else {
      visit_generic(s, t, bx, [&](int i, int j, const SAcc<float>& a, int) {
        struct D {
          const SAcc<float>* a;
          __device__ FF operator()(int di, int dj) const { return FF((*a)(di, dj), 0.0f); }
        } d{&a};
        const FF na = negA<FF>(d, i, j, n);
        emit(i, j, a(0, 0), na.hi, na.lo);
      });
    }
  }
  __device__ void finish(double tot) const { finish_pap(st, tot); }
};

// The staged direction pass over every tile (small grids, batched solves).
static cudaError_t launch_cg_dir_f32_staged(const Operand& z, const Operand& pold,
                                            Grid<float> pnew, Grid<double> Ap, int n,
                                            SolveState* st, ReduceBuf rb, cudaStream_t s) {
  const dim3 g = tile_grid(n);
  const int ntx = (int)g.x;
  const int total = (int)(g.x * g.y);
  const DevOperand<float> dz = dev_operand<float>(z), dp = dev_operand<float>(pold);
  if (z.tma && pold.tma)
    return launch_persist(CgDirF32Job<true>{dz, dp, pnew, Ap, n, ntx, total, st, rb}, total, s);
  return launch_persist(CgDirF32Job<false>{dz, dp, pnew, Ap, n, ntx, total, st, rb}, total, s);
}

// ---------------------------------------------------------------------------
// CG update (pointwise, flat, 16-byte vectors): x += alpha p; r -= alpha Ap;
// ||r||^2; convergence test.  The arrays share one layout; padding entries
// are zero and stay zero.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cg_update_pt(double& x, double& r, double p, double ap,
                                             double alpha, double& acc) {
  x = fma(alpha, p, x);
  r = fma(-alpha, ap, r);
  acc = fma(r, r, acc);
}

struct CgUpdateArgs {
  double* x;
  double* r;
  const double* p;
  const float* pf;   // FP32 direction (mixed MGCG); p unused when set
  const double* Ap;
  float* rlo;
  long long N;
  int plain;
  SolveState* st;
  double* norms;
  ReduceBuf rb;
};

// The update over CTAs cta = 0 .. ncta-1 of one problem.
template <bool VEC>
__device__ __forceinline__ void cg_update_run(const CgUpdateArgs& a, unsigned cta, unsigned ncta) {
  SolveState* st = a.st;
  if (st->done) return;
  const double alpha = st->alpha;
  double acc = 0.0;
  const long long N = a.N;
  const long long tid = (long long)cta * kThreads + threadIdx.x;
  const long long stride = (long long)ncta * kThreads;
  long long done_to = 0;
  double* __restrict__ x = a.x;
  double* __restrict__ r = a.r;
  const double* __restrict__ p = a.p;
  const float* __restrict__ pf = a.pf;
  const double* __restrict__ Ap = a.Ap;
  float* __restrict__ rlo = a.rlo;
  if (VEC) {
    const long long nv = N / 2;
    double2* x2 = reinterpret_cast<double2*>(x);
    double2* r2 = reinterpret_cast<double2*>(r);
    const double2* p2 = reinterpret_cast<const double2*>(p);
    const double2* a2 = reinterpret_cast<const double2*>(Ap);
#pragma unroll 2
    for (long long k = tid; k < nv; k += stride) {
      double2 pv;
      if (pf) {
        const float2 q = __ldg(reinterpret_cast<const float2*>(pf) + k);
        pv = make_double2(f32_to_f64(q.x), f32_to_f64(q.y));
      } else {
        pv = __ldg(p2 + k);
      }
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
    cg_update_pt(xv, rv, pf ? f32_to_f64(pf[k]) : p[k], Ap[k], alpha, acc);
    x[k] = xv;
    r[k] = rv;
    if (rlo) rlo[k] = f64_to_f32(rv);
  }
  double* norms = a.norms;
  const int plain = a.plain;
  grid_reduce_n(acc, a.rb, [&](double tot) {
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
  }, cta, ncta);
}

template <bool VEC>
__global__ void __launch_bounds__(kThreads) k_cg_update(const CgUpdateArgs a) {
  pdl_begin();
  cg_update_run<VEC>(a, blockIdx.x, gridDim.x);
}

// one problem per blockIdx.y
template <bool VEC>
__global__ void __launch_bounds__(kThreads)
    k_cg_update_batch(const unsigned char* __restrict__ blobs, int stride) {
  pdl_begin();
  const CgUpdateArgs a =
      *reinterpret_cast<const CgUpdateArgs*>(blobs + (size_t)blockIdx.y * (size_t)stride);
  cg_update_run<VEC>(a, blockIdx.x, gridDim.x);
}

// BatchLaunchFn: aux[0] = CTAs per problem.
template <bool VEC>
cudaError_t launch_cg_update_batch(const unsigned char* blobs, int stride, int count,
                                   const int* aux, const BatchScratch&, cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  if (count > 65535) return cudaErrorInvalidValue;
  return launch_pdl(k_cg_update_batch<VEC>, dim3(aux[0], count), dim3(kThreads), 0, s, blobs,
                    stride);
}

static inline bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

// CTAs of one resident wave of k_cg_update: the grid-stride loop gives every
// CTA the same share, so a grid beyond one wave leaves a partial second wave
// running alone at the end (1216 CTAs at 6 resident per SM: 1.33 waves).
template <bool VEC>
static int cg_update_wave() {
  static const int v = [] {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_cg_update<VEC>, kThreads, 0) !=
            cudaSuccess ||
        b < 1)
      b = 1;
    return b * sm_count();
  }();
  return v;
}

// ---------------------------------------------------------------------------
// Smoothing pass (Jacobi / Richardson) with the field variants.
// ---------------------------------------------------------------------------
struct SmoothCtx {};

template <typename T, int FIELD, int EPI, bool DOT, bool TMA>
struct SmoothJob {
  static constexpr bool kNeedB = (EPI == kEpiSweep) || DOT;
  static constexpr int kOffB = align128(box_bytes<T, BI, BJ>());
  static constexpr int kOffE = kOffB + (kNeedB ? align128(box_bytes<T, QI, QJ>()) : 0);
  static constexpr int kStage =
      kOffE + (FIELD == kFieldProlong ? align128(box_bytes<T, CI, CJ>()) : 0);
  static constexpr int kScratch = 0;
  static constexpr bool kReduce = DOT;
  using Acc = DotAcc<T>;
  using Ctx = NoCtx;
  DevOperand<T> vin, e, b;
  Grid<T> vout;
  int n, ntx, ntot, smoother;
  T omega;
  SolveState* st;
  ReduceBuf rb;
  __device__ bool prepare(Ctx&) const { return st && st->done; }
  __device__ int tiles() const { return ntot; }
  __device__ unsigned tx_bytes(int) const {
    if (!TMA) return 0u;
    return box_bytes<T, BI, BJ>() + (kNeedB ? box_bytes<T, QI, QJ>() : 0u) +
           (FIELD == kFieldProlong ? box_bytes<T, CI, CJ>() : 0u);
  }
  __device__ void issue(unsigned char* buf, unsigned long long* bar, int id, const Ctx&) const {
    const TileBoxes bx(id % ntx, tile_at<TI, TJ>(id, ntx, n).j_lo);
    const DevOperand<T>& src = (FIELD == kFieldZero) ? b : vin;
    stage_box<TMA, BI, BJ>(reinterpret_cast<T*>(buf), src, &src.box, bx.x0, bx.y0, n, bar);
    if (kNeedB)
      stage_box<TMA, QI, QJ>(reinterpret_cast<T*>(buf + kOffB), b, &b.inner, bx.xi, bx.yi, n,
                             bar);
    if (FIELD == kFieldProlong)
      stage_box<TMA, CI, CJ>(reinterpret_cast<T*>(buf + kOffE), e, &e.coarse, bx.xc, bx.yc,
                             (n + 1) / 2, bar);
  }
  __device__ void compute(unsigned char* buf, int id, Acc& acc, const Ctx&, unsigned char*) const {
    const TileT t = tile_at<TI, TJ>(id, ntx, n);
    const TileBoxes bx(id % ntx, t.j_lo);
    T* s = reinterpret_cast<T*>(buf);
    const T* sb = reinterpret_cast<const T*>(buf + kOffB);
    const bool jac = (smoother == kSmoothJacobi);
    const bool interior = tile_interior(t, n);
    if (FIELD == kFieldProlong) {
      const T* se = reinterpret_cast<const T*>(buf + kOffE);
      transform_box(s, t, bx, n, [&](int i, int j, T& v) {
        const int a = (i >> 1) - bx.xc, b2 = (j >> 1) - bx.yc;
        const T* q = se + b2 * CI + a;
        const bool oi = i & 1, oj = j & 1;
        T pe = q[0];
        if (oi) pe += q[1];
        if (oj) {
          pe += q[CI];
          if (oi) pe += q[CI + 1];
        }
        v += pe * ((oi && oj) ? T(0.25) : ((oi || oj) ? T(0.5) : T(1)));
      });
      __syncthreads();
    } else if (FIELD == kFieldZero && !interior) {
      // first sweep from zero, once per staged point: v1 = omega D^-1 b
      transform_box(s, t, bx, n, [&](int i, int j, T& v) {
        v *= jac ? omega * inv_diagA<T>(i, j, n) : omega;
      });
      __syncthreads();
    }
    auto emit = [&](int i, int j, T bb, T vn) {
      vout.at(i, j) = vn;
      if (DOT) acc.add_prod(bb, vn);
    };
    if (interior) {
      const T m = jac ? omega * T(0.25) : omega;   // interior diag(A) = 4
      const bool exact = exact_group<T, kFp64GroupsFused>();
      visit_interior(s, t, [&](int i, int j, T um, T u0, T up, T uw, T ue, int k) {
        if (FIELD == kFieldZero) {
          // staged raw b: F = m b, the stencil of F is m times the stencil of b
          const T f = m * u0;
          T vn = f;
          if (EPI == kEpiSweep) vn = fma(m, fma(m, neg_stencil<T>(um, u0, up, uw, ue, exact), u0), f);
          emit(i, j, u0, vn);
        } else {
          const T bb = kNeedB ? sb[k] : T(0);
          T vn = u0;
          if (EPI == kEpiSweep) vn = fma(m, bb + neg_stencil<T>(um, u0, up, uw, ue, exact), u0);
          emit(i, j, bb, vn);
        }
      });
    } else {
      visit_generic(s, t, bx, [&](int i, int j, const SAcc<T>& a, int k) {
        const T f = a(0, 0);
        const T bb = kNeedB ? sb[k] : T(0);
        T vn = f;
        if (EPI == kEpiSweep) {
          const T m = jac ? omega * inv_diagA<T>(i, j, n) : omega;
          vn = fma(m, bb + negA<T>(a, i, j, n), f);
        }
        emit(i, j, bb, vn);
      });
    }
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

// ---------------------------------------------------------------------------
// Fused residual + restriction: f = R (b - A v).  Tiles live on the coarse
// grid (32 x 16 coarse points); the CTA stages b and v over the fine region
// under its coarse tile (the same 72 x 37 box as the fine tiles), forms r in
// place of b in shared memory, then applies the 3x3 restriction weights.
// One HBM pass over v and b, a quarter-size write.
// ---------------------------------------------------------------------------
template <typename T, bool TMA>
struct ResRestrictJob {
  static constexpr int kOffV = align128(box_bytes<T, BI, BJ>());
  static constexpr int kStage = kOffV + align128(box_bytes<T, BI, BJ>());
  static constexpr int kScratch = 0;
  static constexpr bool kReduce = false;
  using Acc = DotAcc<double>;
  using Ctx = NoCtx;
  DevOperand<T> v, b;
  Grid<T> f;
  int nf, nc, ntx, ntot, kind, has_v;
  const SolveState* st;
  ReduceBuf rb;
  __device__ bool prepare(Ctx&) const { return st && st->done; }
  __device__ int tiles() const { return ntot; }
  __device__ unsigned tx_bytes(int) const {
    return TMA ? box_bytes<T, BI, BJ>() * (has_v ? 2u : 1u) : 0u;
  }
  __device__ void issue(unsigned char* buf, unsigned long long* bar, int id, const Ctx&) const {
    const int ti = id % ntx, tj = id / ntx;
    const int x0 = 64 * ti - 4, y0 = 32 * tj - 2;
    stage_box<TMA, BI, BJ>(reinterpret_cast<T*>(buf), b, &b.box, x0, y0, nf, bar);
    if (has_v)
      stage_box<TMA, BI, BJ>(reinterpret_cast<T*>(buf + kOffV), v, &v.box, x0, y0, nf, bar);
  }
  __device__ void compute(unsigned char* buf, int id, Acc&, const Ctx&, unsigned char*) const {
    const int ti = id % ntx, tj = id / ntx;
    const Tile<RTI, RTJ> t = tile_at<RTI, RTJ>(id, ntx, nc);
    const int x0 = 64 * ti - 4, y0 = 32 * tj - 2;
    T* sr = reinterpret_cast<T*>(buf);
    const T* sv = reinterpret_cast<const T*>(buf + kOffV);
    const int m = t.i_hi - t.i_lo, mp = t.j_hi - t.j_lo;
    const int ri0 = max(2 * t.i_lo - 1, 0), ri1 = min(2 * t.i_hi - 1, nf - 1);
    const int rj0 = max(2 * t.j_lo - 1, 0), rj1 = min(2 * t.j_hi - 1, nf - 1);
    if (has_v) {
      const int ei = ri1 - ri0 + 1, ej = rj1 - rj0 + 1;
      const int cnt = ei * ej;
      const bool interior = ri0 > 0 && ri1 < nf - 1 && rj0 > 2 && rj1 < nf - 3;
      const bool exact = exact_group<T, kFp64GroupsFused>();
      for (int k = threadIdx.x; k < cnt; k += kThreads) {
        const int c = k / ei;
        const int r = k - c * ei;
        const int i = ri0 + r, j = rj0 + c;
        const int q = (j - y0) * BI + (i - x0);
        T na;
        if (interior) {
          const T* a = sv + q;
          na = neg_stencil<T>(a[-BI], a[0], a[BI], a[-1], a[1], exact);
        } else {
          na = negA<T>(SAcc<T>{sv + q, BI}, i, j, nf);
        }
        sr[q] += na;
      }
      __syncthreads();
    }
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    for (int c = w; c < mp; c += kWarps) {
      const int J = t.j_lo + c;
      for (int r = lane; r < m; r += 32) {
        const int I = t.i_lo + r;
        const T* q = sr + (2 * J - y0) * BI + (2 * I - x0);
        T acc = T(0);
        if (I > 0 && I < nc - 1 && J > 0 && J < nc - 1) {
          // interior coarse point: weights (1/2, 1, 1/2) x (1/2, 1, 1/2)
          // (galerkin), times 1/4 for the full-weighting kinds
          T cs[3];
#pragma unroll
          for (int bj = -1; bj <= 1; ++bj) {
            const T* col = q + bj * BI;
            cs[bj + 1] = fma(T(0.5), col[-1] + col[1], col[0]);
          }
          acc = fma(T(0.5), cs[0] + cs[2], cs[1]);
          if (kind != kRestrictGalerkin) acc *= T(0.25);
        } else {
#pragma unroll
          for (int bj = -1; bj <= 1; ++bj) {
            const T wj = restrict_w1<T>(kind, J, nc, bj);
#pragma unroll
            for (int ai = -1; ai <= 1; ++ai)
              acc = fma(restrict_w1<T>(kind, I, nc, ai) * wj, q[bj * BI + ai], acc);
          }
        }
        f.at(I, J) = acc;
      }
    }
  }
  __device__ void finish(double) const {}
};

// ---------------------------------------------------------------------------
// Temporal blocking of the V-cycle.  One kernel runs all pre-smoothing sweeps
// from v = 0 plus the residual and its restriction; another runs the
// prolongation and all post-smoothing sweeps.  A CTA stages its operands with
// a halo as wide as the number of sweeps, recomputes the halo in shared
// memory and writes only its own points: per fine point the level's HBM
// traffic drops from ~66 to ~22 bytes (FP32) and six launches become two.
// ---------------------------------------------------------------------------
constexpr int kMaxFusedSweeps = 3;

// Column march over a region [i0,i1] x [j0,j1] (global coordinates) of
// shared-memory boxes with origin (X0, Y0) and pitch P: thread t takes row
// i0 + t % w and a contiguous run of columns of group t / w, keeping the
// j-1 / j / j+1 values in registers (three shared loads per point).
// fn(i, j, k, um, u0, up, uw, ue) gets the box index k of (i, j) and the
// five stencil values of `in`.  Threads beyond the last full group idle.
template <typename T, int P, typename Fn>
__device__ __forceinline__ void march_region(const T* in, int X0, int Y0, int i0, int i1, int j0,
                                             int j1, Fn&& fn) {
  static_assert(P <= kThreads, "a box row must fit in one thread block");
  const int w = i1 - i0 + 1, h = j1 - j0 + 1;
  if (w <= 0 || h <= 0) return;
  const int G = kThreads / w;
  const int g = threadIdx.x / w;
  if (g >= G) return;
  const int r = threadIdx.x - g * w;
  const int per = (h + G - 1) / G;
  const int cb = j0 + g * per;
  const int ce = min(j1 + 1, cb + per);
  if (cb >= ce) return;
  const int i = i0 + r;
  int k = (cb - Y0) * P + (i - X0);
  T um = in[k - P], u0 = in[k];
  for (int j = cb; j < ce; ++j, k += P) {
    const T up = in[k + P];
    fn(i, j, k, um, u0, up, in[k - 1], in[k + 1]);
    um = u0;
    u0 = up;
  }
}

// The same march over a region of compile-time shape W x H whose (0, 0)
// point sits at shared-memory index `base`, for the interior tiles of the
// fused kernels: the column loop is unrolled, so every shared-memory access
// is a base register plus an immediate offset, and runs in chunks of four
// columns whose loads are all issued before the chunk's first store (the
// shared-memory latency overlaps within a chunk).  For each point
//   v = val(um, u0, up, uw, ue, a);  out[k] = v (if OUT);  epi(r, c, u0, v, a)
// with r, c the region row and column and a = aux[k] (0 without AUX).
template <typename T, int P, int W, int H, bool AUX, bool OUT, typename Val, typename Epi>
__device__ __forceinline__ void sweep_fixed(const T* in, const T* aux, T* out, int base, Val&& val,
                                            Epi&& epi) {
  constexpr int G = kThreads / W;
  static_assert(G >= 1 && W <= P, "a region row must fit in one thread block and one box row");
  constexpr int C = (H + G - 1) / G;
  const int g = threadIdx.x / W;
  if (g >= G) return;
  const int r = threadIdx.x - g * W;
  const int c0 = g * C;
  const int k0 = base + c0 * P + r;
  const int cnt = min(C, H - c0);
  const T* p = in + k0;
  T um = p[-P], u0 = p[0];
#pragma unroll
  for (int q0 = 0; q0 < C; q0 += 4) {
    T up[4], uw[4], ue[4], a[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int q = q0 + u;
      if (q < C && q < cnt) {
        up[u] = p[(q + 1) * P];
        uw[u] = p[q * P - 1];
        ue[u] = p[q * P + 1];
        a[u] = AUX ? aux[k0 + q * P] : T(0);
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int q = q0 + u;
      if (q < C && q < cnt) {
        const T v = val(um, u0, up[u], uw[u], ue[u], a[u]);
        if (OUT) out[k0 + q * P] = v;
        epi(r, c0 + q, u0, v, a[u]);
        um = u0;
        u0 = up[u];
      }
    }
  }
}

// out = in + m (b + (-A in)) on the region [i0,i1] x [j0,j1].
template <typename T, int P>
__device__ __forceinline__ void box_sweep(T* out, const T* in, const T* bsm, int X0, int Y0, int i0,
                                          int i1, int j0, int j1, int n, bool jac, T omega) {
  const bool interior = i0 > 0 && i1 < n - 1 && j0 > 2 && j1 < n - 3;
  if (interior) {
    const T m = jac ? omega * T(0.25) : omega;
    march_region<T, P>(in, X0, Y0, i0, i1, j0, j1,
                       [&](int, int, int k, T um, T u0, T up, T uw, T ue) {
                         const T na = ((uw + ue) + (um + up)) - T(4) * u0;
                         out[k] = fma(m, bsm[k] + na, u0);
                       });
    return;
  }
  const int w = i1 - i0 + 1, h = j1 - j0 + 1;
  if (w <= 0 || h <= 0) return;
  const int cnt = w * h;
  const float inv_w = 1.0f / (float)w;
  for (int q = threadIdx.x; q < cnt; q += kThreads) {
    const int c = (int)(((float)q + 0.5f) * inv_w);
    const int r = q - c * w;
    const int i = i0 + r, j = j0 + c;
    const int k = (j - Y0) * P + (i - X0);
    const T* a = in + k;
    const T na = negA<T>(SAcc<T>{a, P}, i, j, n);
    const T m = jac ? omega * inv_diagA<T>(i, j, n) : omega;
    out[k] = fma(m, bsm[k] + na, a[0]);
  }
}

// Visit the global-coordinate region [i0,i1]x[j0,j1]: fn(i, j).
template <typename Fn>
__device__ __forceinline__ void region_for(int i0, int i1, int j0, int j1, Fn&& fn) {
  const int w = i1 - i0 + 1, h = j1 - j0 + 1;
  if (w <= 0 || h <= 0) return;
  const int cnt = w * h;
  const float inv_w = 1.0f / (float)w;
  for (int q = threadIdx.x; q < cnt; q += kThreads) {
    const int c = (int)(((float)q + 0.5f) * inv_w);
    fn(i0 + (q - c * w), j0 + c);
  }
}

// Pre-smoothing (S sweeps from zero) + residual + restriction.  Tiles are
// RI x RJ coarse points; the fine box (BI x BJ at (2 RI ti - 4, 2 RJ tj - 4))
// holds b around the residual region with a halo of S <= 3.  The residual
// region of a tile spans box indices 5 .. 2R + 5 in each direction, so a box
// needs 2R + 9 points; BI is rounded up for 16-byte TMA rows.
// - PreLarge: 32 x 16 tiles (76 x 41 boxes), with the unrolled interior path.
// - PreSmall: 16 x 8 tiles (44 x 25 boxes), for levels with fewer large
//   tiles than SMs: a quarter of the serial work per CTA on four times the
//   CTAs.  Every tile takes the generic path.
template <int RI_, int RJ_, int BI_, int BJ_, bool LEAN_>
struct PreGeom {
  static constexpr int RI = RI_, RJ = RJ_, BI = BI_, BJ = BJ_;
  static constexpr bool kLean = LEAN_;
  static_assert(BI >= 2 * RI + 9 && BJ >= 2 * RJ + 9 && BI % 4 == 0, "pre-smoothing box");
};
using PreLarge = PreGeom<RTI, RTJ, 76, 41, true>;
using PreSmall = PreGeom<16, 8, 44, 25, false>;
constexpr int PBI = PreLarge::BI;

template <typename T, bool TMA, class Geo = PreLarge>
struct PreFusedJob {
  static constexpr int kBox = align128(box_bytes<T, Geo::BI, Geo::BJ>());
  static constexpr int kStage = kBox;
  static constexpr int kScratch = 2 * kBox;
  static constexpr bool kReduce = false;
  using Acc = DotAcc<double>;
  using Ctx = NoCtx;
  DevOperand<T> b;
  CUtensorMap bmap;    // BI x BJ box of b
  Grid<T> vout, f;
  int nf, nc, ntx, ntot, sweeps, smoother, kind;
  T omega;
  const SolveState* st;
  ReduceBuf rb;
  // ring = w > 0: only the boundary ring of tiles w deep (the first and
  // last w tile rows and columns; nty = tile rows) is visited,
  // k -> ring_id(k); the interior tiles are done by the register wave kernel
  // (k_pre_wave)
  int ring, nty;
  __device__ int ring_id(int k) const {
    const int w = ring;
    if (!w) return k;
    if (k < w * ntx) return k;
    if (k < 2 * w * ntx) return (k - w * ntx) + (nty - w) * ntx;
    const int k2 = k - 2 * w * ntx;
    const int r = k2 % (2 * w);
    return (r < w ? r : ntx - 2 * w + r) + (w + k2 / (2 * w)) * ntx;
  }
  __device__ bool prepare(Ctx&) const { return st && st->done; }
  __device__ int tiles() const { return ntot; }
  __device__ unsigned tx_bytes(int) const { return TMA ? box_bytes<T, Geo::BI, Geo::BJ>() : 0u; }
  __device__ void issue(unsigned char* buf, unsigned long long* bar, int k, const Ctx&) const {
    const int id = ring_id(k);
    const int ti = id % ntx, tj = id / ntx;
    stage_box<TMA, Geo::BI, Geo::BJ>(reinterpret_cast<T*>(buf), b, &bmap, 2 * Geo::RI * ti - 4,
                                 2 * Geo::RJ * tj - 4, nf, bar);
  }
  // Interior tile (full 32 x 16 coarse tile; every swept fine point has the
  // plain 5-point stencil and the constant smoother weight m).  Box offsets:
  // the residual region Rr (65 x 33 fine points) starts at box (5, 5); the
  // sweep k output lives on Rr grown by S - k + 1.  v1 = m b is never
  // formed: v2 = v1 + m (b - A v1) = (2m - 4m^2) b + m^2 (sum of the four
  // neighbours of b).
  __device__ bool lean_ok(const Tile<RTI, RTJ>& t) const {
    const int S = sweeps;
    const int ri0 = 2 * t.i_lo - 1, ri1 = 2 * t.i_hi - 1;
    const int rj0 = 2 * t.j_lo - 1, rj1 = 2 * t.j_hi - 1;
    return t.i_lo > 0 && t.j_lo > 0 && t.i_hi - t.i_lo == RTI && t.j_hi - t.j_lo == RTJ &&
           ri0 - S >= 1 && ri1 + S <= nf - 2 && rj0 - S >= 1 && rj1 + S <= nf - 2 &&
           rj0 - (S - 1) >= 3 && rj1 + (S - 1) <= nf - 4;
  }

  template <int S>
  __device__ void compute_lean(const Tile<RTI, RTJ>& t, int X0, int Y0, const T* B, T* V0,
                               T* V1) const {
    constexpr int R0 = 5;                      // box index of Rr's first row / column
    const T m = (smoother == kSmoothJacobi) ? omega * T(0.25) : omega;
    const T k1 = T(2) * m - T(4) * m * m, m2 = m * m;
    const T* vs;                               // v_S on Rr + 1
    auto none = [](int, int, T, T, T) {};
    if constexpr (S >= 2) {
      constexpr int h = S - 1;                 // v2 on Rr + (S - 1), straight from b
      sweep_fixed<T, PBI, 65 + 2 * h, 33 + 2 * h, false, true>(
          B, nullptr, V0, (R0 - h) * PBI + (R0 - h),
          [&](T um, T u0, T up, T uw, T ue, T) { return fma(m2, (uw + ue) + (um + up), k1 * u0); },
          none);
      __syncthreads();
      vs = V0;
      if constexpr (S == 3) {                  // v3 on Rr + 1
        sweep_fixed<T, PBI, 67, 35, true, true>(
            V0, B, V1, (R0 - 1) * PBI + (R0 - 1),
            [&](T um, T u0, T up, T uw, T ue, T bb) {
              return fma(m, bb + (((uw + ue) + (um + up)) - T(4) * u0), u0);
            },
            none);
        __syncthreads();
        vs = V1;
      }
    } else {
      vs = B;                                  // S = 1: v1 = m b, formed on the fly
    }
    // residual on Rr into the free buffer; own points of v_S (Rr minus its
    // first row and column) to global
    T* const R = (S == 3) ? V0 : V1;
    const int gi0 = X0 + R0, gj0 = Y0 + R0;
    sweep_fixed<T, PBI, 65, 33, true, true>(
        vs, B, R, R0 * PBI + R0,
        [&](T um, T u0, T up, T uw, T ue, T bb) {
          const T nb = (uw + ue) + (um + up);
          if constexpr (S == 1) return fma(m, nb - T(4) * u0, bb);
          else return bb + (nb - T(4) * u0);
        },
        [&](int r, int c, T u0, T, T) {
          if (r > 0 && c > 0) vout.at(gi0 + r, gj0 + c) = (S == 1) ? m * u0 : u0;
        });
    __syncthreads();
    // restriction, constant interior weights: thread = (coarse row, pair of
    // coarse columns); fine centres at box (6 + 2 a, 6 + 2 b)
    const T sc = (kind == kRestrictGalerkin) ? T(1) : T(0.25);
    const int a = threadIdx.x & 31, bp = threadIdx.x >> 5;
    const T* q = R + (5 + 4 * bp) * PBI + (6 + 2 * a);
    T cs[5];
#pragma unroll
    for (int u = 0; u < 5; ++u) {
      const T* col = q + u * PBI;
      cs[u] = fma(T(0.5), col[-1] + col[1], col[0]);
    }
    const int I = t.i_lo + a, J = t.j_lo + 2 * bp;
    f.at(I, J) = sc * fma(T(0.5), cs[0] + cs[2], cs[1]);
    f.at(I, J + 1) = sc * fma(T(0.5), cs[2] + cs[4], cs[3]);
  }

  __device__ void compute(unsigned char* buf, int k, Acc&, const Ctx&, unsigned char* scr) const {
    constexpr int BW = Geo::BI;   // box row length
    const int id = ring_id(k);
    const int ti = id % ntx, tj = id / ntx;
    const Tile<Geo::RI, Geo::RJ> t = tile_at<Geo::RI, Geo::RJ>(id, ntx, nc);
    const int X0 = 2 * Geo::RI * ti - 4, Y0 = 2 * Geo::RJ * tj - 4;
    const T* B = reinterpret_cast<const T*>(buf);
    T* const V0 = reinterpret_cast<T*>(scr);
    T* const V1 = reinterpret_cast<T*>(scr + kBox);
    if constexpr (Geo::kLean) {
      if (lean_ok(t)) {
        if (sweeps == 3) compute_lean<3>(t, X0, Y0, B, V0, V1);
        else if (sweeps == 2) compute_lean<2>(t, X0, Y0, B, V0, V1);
        else compute_lean<1>(t, X0, Y0, B, V0, V1);
        return;
      }
    }
    const bool jac = (smoother == kSmoothJacobi);
    // residual region and its expansions, clipped to the domain
    const int ri0 = 2 * t.i_lo - 1, ri1 = 2 * t.i_hi - 1;
    const int rj0 = 2 * t.j_lo - 1, rj1 = 2 * t.j_hi - 1;
    auto lo = [](int v, int h) { return max(v - h, 0); };
    auto hi = [&](int v, int h) { return min(v + h, nf - 1); };
    // v1 = m b on the residual region + S
    {
      const int h = sweeps;
      region_for(lo(ri0, h), hi(ri1, h), lo(rj0, h), hi(rj1, h), [&](int i, int j) {
        const int k = (j - Y0) * BW + (i - X0);
        V0[k] = (jac ? omega * inv_diagA<T>(i, j, nf) : omega) * B[k];
      });
    }
    __syncthreads();
    bool cur1 = false;   // v_k lives in V1 (else V0)
    for (int sw = 2; sw <= sweeps; ++sw) {
      const int h = sweeps - sw + 1;
      box_sweep<T, BW>(cur1 ? V0 : V1, cur1 ? V1 : V0, B, X0, Y0, lo(ri0, h), hi(ri1, h),
                        lo(rj0, h), hi(rj1, h), nf, jac, omega);
      __syncthreads();
      cur1 = !cur1;
    }
    // own fine points of v_S to global, residual into the other buffer
    T* const R = cur1 ? V0 : V1;
    const T* const VS = cur1 ? V1 : V0;
    region_for(max(2 * t.i_lo, 0), min(2 * t.i_hi - 1, nf - 1), max(2 * t.j_lo, 0),
               min(2 * t.j_hi - 1, nf - 1), [&](int i, int j) {
                 vout.at(i, j) = VS[(j - Y0) * BW + (i - X0)];
               });
    {
      const int i0 = max(ri0, 0), i1 = min(ri1, nf - 1), j0 = max(rj0, 0), j1 = min(rj1, nf - 1);
      const bool interior = i0 > 0 && i1 < nf - 1 && j0 > 2 && j1 < nf - 3;
      if (interior) {
        march_region<T, BW>(VS, X0, Y0, i0, i1, j0, j1,
                             [&](int, int, int k, T um, T u0, T up, T uw, T ue) {
                               R[k] = B[k] + (((uw + ue) + (um + up)) - T(4) * u0);
                             });
      } else {
        region_for(i0, i1, j0, j1, [&](int i, int j) {
          const int k = (j - Y0) * BW + (i - X0);
          R[k] = B[k] + negA<T>(SAcc<T>{VS + k, BW}, i, j, nf);
        });
      }
    }
    __syncthreads();
    // restriction of r on the coarse tile (out-of-domain r entries carry
    // weight zero; they were never written, so read them as zero)
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    const int m = t.i_hi - t.i_lo, mp = t.j_hi - t.j_lo;
    for (int c = w; c < mp; c += kWarps) {
      const int J = t.j_lo + c;
      for (int rr = lane; rr < m; rr += 32) {
        const int I = t.i_lo + rr;
        T acc = T(0);
#pragma unroll
        for (int bj = -1; bj <= 1; ++bj) {
          const T wj = restrict_w1<T>(kind, J, nc, bj);
          if (wj == T(0)) continue;
#pragma unroll
          for (int ai = -1; ai <= 1; ++ai) {
            const T wi = restrict_w1<T>(kind, I, nc, ai);
            if (wi == T(0)) continue;
            acc = fma(wi * wj, R[(2 * J + bj - Y0) * BW + (2 * I + ai - X0)], acc);
          }
        }
        f.at(I, J) = acc;
      }
    }
  }
  __device__ void finish(double) const {}
};

// The end of the preconditioner's r.z reduction: beta and rz.
__device__ __forceinline__ void finish_rz(SolveState* st, double tot) {
  if (!isfinite(tot)) {
    st->done = kDoneBreakdown;
  } else {
    st->rz_new = tot;
    if (st->iter > 0) st->beta = tot / st->rz;
    st->rz = tot;
  }
}

// One side of an r.z split between two concurrent kernels (the boundary
// tiles and the interior wave of a post-smoothing pass): called once by each
// side after its own reduction; the second side to arrive finishes with
// ring + wave (fixed order) and re-arms the counter.
__device__ __forceinline__ void rz_join(SolveState* st, double* mine, double tot) {
  *mine = tot;
  __threadfence();
  if (atomicAdd(&st->join, 1u) == 1u) {
    __threadfence();
    finish_rz(st, __ldcg(&st->rz_part) + __ldcg(&st->rz_wave));
    st->join = 0u;
  }
}

// Prolongation + post-smoothing (S sweeps).  Fine tiles TI x TJ; boxes of
// v_in and b: BI x BJ at (TI ti - 4, j_lo - 4); coarse e: CI x CJ at
// (TI/2 ti - 4, (j_lo - 4) >> 1).  With S <= 3 the swept region reaches box
// index TI + 6 in i and TJ + 7 in j, and the coarse values it interpolates
// reach TI/2 + 6 and TJ/2 + 4.
// - PostLarge: 64 x 32 tiles, with the unrolled interior path.
// - PostSmall: 32 x 16 tiles, for levels with fewer large tiles than SMs;
//   every tile takes the generic path.
template <int TI_, int TJ_, int BI_, int BJ_, int CI_, int CJ_, bool LEAN_>
struct PostGeom {
  static constexpr int TI = TI_, TJ = TJ_, BI = BI_, BJ = BJ_, CI = CI_, CJ = CJ_;
  static constexpr bool kLean = LEAN_;
  static_assert(BI >= TI + 7 && BJ >= TJ + 8 && CI >= TI / 2 + 7 && CJ >= TJ / 2 + 5 &&
                    BI % 4 == 0 && CI % 4 == 0,
                "post-smoothing boxes");
};
using PostLarge = PostGeom<TI, TJ, 72, 41, 40, 22, true>;
using PostSmall = PostGeom<32, 16, 40, 25, 24, 14, false>;
constexpr int QBI = PostLarge::BI, QCI = PostLarge::CI;

template <typename T, bool DOT, bool TMA, class Geo = PostLarge>
struct PostFusedJob {
  static constexpr int kBox = align128(box_bytes<T, Geo::BI, Geo::BJ>());
  static constexpr int kOffB = kBox;
  static constexpr int kOffE = 2 * kBox;
  static constexpr int kStage = kOffE + align128(box_bytes<T, Geo::CI, Geo::CJ>());
  static constexpr int kScratch = kBox;
  static constexpr bool kReduce = DOT;
  using Acc = DotAcc<T>;
  using Ctx = NoCtx;
  DevOperand<T> vin, e, b;
  CUtensorMap vmap, bmap, emap;   // BI x BJ boxes of v_in and b, CI x CJ of e
  Grid<T> vout;
  int n, ntx, ntot, sweeps, smoother;
  T omega;
  SolveState* st;
  ReduceBuf rb;
  // ring = w > 0: only the boundary ring of tiles w deep is visited (the
  // interior is done by k_post_wave); partial: the dot's total goes to
  // st->rz_part for k_post_wave to finish
  int ring, nty, partial;
  __device__ int ring_id(int k) const {
    const int w = ring;
    if (!w) return k;
    if (k < w * ntx) return k;
    if (k < 2 * w * ntx) return (k - w * ntx) + (nty - w) * ntx;
    const int k2 = k - 2 * w * ntx;
    const int r = k2 % (2 * w);
    return (r < w ? r : ntx - 2 * w + r) + (w + k2 / (2 * w)) * ntx;
  }
  __device__ bool prepare(Ctx&) const { return st && st->done; }
  __device__ int tiles() const { return ntot; }
  __device__ unsigned tx_bytes(int) const {
    return TMA ? 2u * box_bytes<T, Geo::BI, Geo::BJ>() + box_bytes<T, Geo::CI, Geo::CJ>() : 0u;
  }
  __device__ void issue(unsigned char* buf, unsigned long long* bar, int k, const Ctx&) const {
    const int id = ring_id(k);
    const int ti = id % ntx;
    const int jl = tile_at<Geo::TI, Geo::TJ>(id, ntx, n).j_lo;
    const int x0 = Geo::TI * ti - 4;
    stage_box<TMA, Geo::BI, Geo::BJ>(reinterpret_cast<T*>(buf), vin, &vmap, x0, jl - 4, n, bar);
    stage_box<TMA, Geo::BI, Geo::BJ>(reinterpret_cast<T*>(buf + kOffB), b, &bmap, x0, jl - 4, n,
                                 bar);
    stage_box<TMA, Geo::CI, Geo::CJ>(reinterpret_cast<T*>(buf + kOffE), e, &emap,
                                 (Geo::TI / 2) * ti - 4, (jl - 4) >> 1, (n + 1) / 2, bar);
  }
  // Interior tile (full 64 x 32 fine tile, every swept point with the plain
  // stencil and constant weight m).  Box offsets: the tile Rt starts at box
  // (5, 4) of v and b; fine (i, j) of the F0 region has coarse box
  // coordinates ((bi >> 1) + 2, (bj + 1) >> 1), i odd <=> bi odd and
  // j odd <=> bj even.
  __device__ bool lean_ok(const TileT& t) const {
    const int S = sweeps;
    return S >= 1 && t.i_lo > 0 && t.j_lo > 0 && t.i_hi - t.i_lo == TI &&
           t.j_hi - t.j_lo == TJ && t.i_lo - S >= 1 && t.i_hi - 1 + S <= n - 2 &&
           t.j_lo - S >= 1 && t.j_hi - 1 + S <= n - 2 && t.j_lo - (S - 1) >= 3 &&
           t.j_hi - 1 + (S - 1) <= n - 4;
  }

  template <int S>
  __device__ void compute_lean(const TileT& t, T* V0, T* V1, const T* B, const T* E,
                               Acc& acc) const {
    constexpr int RI = 5, RJ = 4;              // box index of Rt's first row / column
    constexpr int W = TI + 2 * S, H = TJ + 2 * S;
    const T m = (smoother == kSmoothJacobi) ? omega * T(0.25) : omega;
    // F0 = v_in + P e on Rt + S.  Thread = (fine row, run of C columns, C
    // even); the row-interpolated coarse values rv(J) are carried along.
    {
      constexpr int G = kThreads / W;
      constexpr int C = (((H + G - 1) / G) + 1) & ~1;
      const int g = threadIdx.x / W;
      if (g < G) {
        const int r = threadIdx.x - g * W;
        const int bi = RI - S + r;
        const int c0 = g * C;
        const T w1 = (bi & 1) ? T(0.5) : T(0);
        const T w0 = (bi & 1) ? T(0.5) : T(1);
        const int bj0 = RJ - S + c0;                       // c0 even: parity of RJ - S
        const T* erow = E + ((bi >> 1) + 2);
        auto rv = [&](int cj) { return fma(w1, erow[cj * QCI + 1], w0 * erow[cj * QCI]); };
        T* v = V0 + bj0 * QBI + bi;
        // invariant before column bj: ra = rv(bj >> 1), rb = rv((bj >> 1) + 1)
        int cj = bj0 >> 1;
        T ra = rv(cj), rb = rv(cj + 1);
#pragma unroll
        for (int q = 0; q < C; ++q) {
          if (c0 + q < H) {
            // bj = bj0 + q; bj even -> j odd: average of rv(cj), rv(cj + 1)
            if (((RJ - S + q) & 1) == 0) {
              v[q * QBI] += T(0.5) * (ra + rb);
            } else {
              // bj odd -> j even: rv((bj + 1) >> 1) = rv(cj + 1); advance
              v[q * QBI] += rb;
              ra = rb;
              ++cj;
              rb = rv(cj + 1);
            }
          }
        }
      }
    }
    __syncthreads();
    T* cur = V0;
    T* nxt = V1;
    auto sweep = [&](T um, T u0, T up, T uw, T ue, T bb) {
      return fma(m, bb + (((uw + ue) + (um + up)) - T(4) * u0), u0);
    };
    auto none = [](int, int, T, T, T) {};
    if constexpr (S >= 2) {
      constexpr int h = S - 1;                 // sweep 1 on Rt + (S - 1)
      sweep_fixed<T, QBI, TI + 2 * h, TJ + 2 * h, true, true>(
          cur, B, nxt, (RJ - h) * QBI + (RI - h), sweep, none);
      __syncthreads();
      T* tmp = cur; cur = nxt; nxt = tmp;
    }
    if constexpr (S == 3) {                    // sweep 2 on Rt + 1
      sweep_fixed<T, QBI, TI + 2, TJ + 2, true, true>(cur, B, nxt, (RJ - 1) * QBI + (RI - 1),
                                                      sweep, none);
      __syncthreads();
      T* tmp = cur; cur = nxt; nxt = tmp;
    }
    // last sweep on Rt, to global
    const int gi0 = t.i_lo, gj0 = t.j_lo;
    sweep_fixed<T, QBI, TI, TJ, true, false>(cur, B, nullptr, RJ * QBI + RI, sweep,
                                             [&](int r, int c, T, T vn, T bb) {
                                               vout.at(gi0 + r, gj0 + c) = vn;
                                               if (DOT) acc.add_prod(bb, vn);
                                             });
  }

  __device__ void compute(unsigned char* buf, int k, Acc& acc, const Ctx&,
                          unsigned char* scr) const {
    constexpr int BW = Geo::BI, CW = Geo::CI;   // box row lengths
    const int id = ring_id(k);
    const Tile<Geo::TI, Geo::TJ> t = tile_at<Geo::TI, Geo::TJ>(id, ntx, n);
    const int ti = id % ntx;
    const int X0 = Geo::TI * ti - 4, Y0 = t.j_lo - 4;
    const int XC = (Geo::TI / 2) * ti - 4, YC = (t.j_lo - 4) >> 1;
    T* const V0 = reinterpret_cast<T*>(buf);
    T* const V1 = reinterpret_cast<T*>(scr);
    const T* B = reinterpret_cast<const T*>(buf + kOffB);
    const T* E = reinterpret_cast<const T*>(buf + kOffE);
    if constexpr (Geo::kLean) {
      if (lean_ok(t)) {
        if (sweeps == 3) compute_lean<3>(t, V0, V1, B, E, acc);
        else if (sweeps == 2) compute_lean<2>(t, V0, V1, B, E, acc);
        else compute_lean<1>(t, V0, V1, B, E, acc);
        return;
      }
    }
    const bool jac = (smoother == kSmoothJacobi);
    auto lo = [](int v, int h) { return max(v - h, 0); };
    auto hi = [&](int v, int h) { return min(v + h, n - 1); };
    const int ti0 = t.i_lo, ti1 = t.i_hi - 1, tj0 = t.j_lo, tj1 = t.j_hi - 1;
    // F0 = v_in + P e on the tile + S
    region_for(lo(ti0, sweeps), hi(ti1, sweeps), lo(tj0, sweeps), hi(tj1, sweeps),
               [&](int i, int j) {
                 const T* q = E + ((j >> 1) - YC) * CW + ((i >> 1) - XC);
                 const bool oi = i & 1, oj = j & 1;
                 T pe = q[0];
                 if (oi) pe += q[1];
                 if (oj) {
                   pe += q[CW];
                   if (oi) pe += q[CW + 1];
                 }
                 V0[(j - Y0) * BW + (i - X0)] +=
                     pe * ((oi && oj) ? T(0.25) : ((oi || oj) ? T(0.5) : T(1)));
               });
    __syncthreads();
    bool cur1 = false;
    for (int sw = 1; sw < sweeps; ++sw) {
      const int h = sweeps - sw;
      box_sweep<T, BW>(cur1 ? V0 : V1, cur1 ? V1 : V0, B, X0, Y0, lo(ti0, h), hi(ti1, h),
                        lo(tj0, h), hi(tj1, h), n, jac, omega);
      __syncthreads();
      cur1 = !cur1;
    }
    // last pass on the tile itself: to global (sweep, or F0 when S = 0)
    const T* in = cur1 ? V1 : V0;
    const bool interior = tile_interior(t, n);
    if (interior && sweeps > 0) {
      const T m = jac ? omega * T(0.25) : omega;
      march_region<T, BW>(in, X0, Y0, ti0, ti1, tj0, tj1,
                           [&](int i, int j, int k, T um, T u0, T up, T uw, T ue) {
                             const T bb = B[k];
                             const T vn = fma(m, bb + (((uw + ue) + (um + up)) - T(4) * u0), u0);
                             vout.at(i, j) = vn;
                             if (DOT) acc.add_prod(bb, vn);
                           });
    } else {
      region_for(ti0, ti1, tj0, tj1, [&](int i, int j) {
        const int k = (j - Y0) * BW + (i - X0);
        const T* a = in + k;
        const T bb = B[k];
        T vn = a[0];
        if (sweeps > 0) {
          const T na = negA<T>(SAcc<T>{a, BW}, i, j, n);
          const T m = jac ? omega * inv_diagA<T>(i, j, n) : omega;
          vn = fma(m, bb + na, a[0]);
        }
        vout.at(i, j) = vn;
        if (DOT) acc.add_prod(bb, vn);
      });
    }
  }
  __device__ void finish(double tot) const {
    if (partial)
      rz_join(st, &st->rz_part, tot);
    else
      finish_rz(st, tot);
  }
};

// ---------------------------------------------------------------------------
// Launchers.
// ---------------------------------------------------------------------------
static inline Operand raw_operand(const void* p, int n, int ld) {
  Operand o;
  o.p = p;
  o.n = n;
  o.ld = ld;
  o.tma = false;
  return o;
}


// Operator apply on any layout (the caller's arrays, ld = n) without
// shared-memory staging: a CTA takes a block of 256 rows and a run of
// kApplyCols columns, each thread one row, marching down the columns with
// the j-1 / j / j+1 values in registers; the i-1 / i+1 neighbours are the
// neighbouring threads' values and come from L1.  DRAM traffic is one read
// and one write per point (plus the run's two halo columns).  FP64: odd warps
// form interior sums on the integer pipe (exact_stencil5), even warps with
// FP64 instructions.
constexpr int kApplyCols = 32;
// columns whose loads are issued together (FP64 keeps fewer in registers)
template <typename T>
__host__ __device__ constexpr int apply_chunk() { return sizeof(T) == 8 ? 4 : 8; }
static_assert(kApplyCols % 8 == 0 && kApplyCols % 4 == 0, "column runs are whole chunks");

template <typename T, bool DOT>
__global__ void __launch_bounds__(kThreads)
    k_apply_direct(Grid<const T> u, Grid<T> out, int n, int sign, ReduceBuf rb, double* dot_out) {
  pdl_begin();
  constexpr int kApplyChunk = apply_chunk<T>();
  const int nrb = (n + kThreads - 1) / kThreads;
  const int items = nrb * ((n + kApplyCols - 1) / kApplyCols);
  const bool exact = sizeof(T) == 8 && ((threadIdx.x >> 5) & 1);
  const size_t ld = (size_t)u.ld;
  DotAcc<T> acc;
  for (int w = blockIdx.x; w < items; w += gridDim.x) {
    const int i = (w % nrb) * kThreads + threadIdx.x;
    if (i >= n) continue;
    const int j0 = (w / nrb) * kApplyCols;
    const int j1 = min(n, j0 + kApplyCols);
    const T* col = u.p + (size_t)j0 * ld + i;
    const bool irow = (i > 0 && i < n - 1);
    T um = j0 > 0 ? __ldg(col - ld) : T(0);
    T u0 = __ldg(col);
    // chunks of kApplyChunk columns: all their loads are issued first, so a
    // warp keeps several DRAM lines in flight
    for (int jc = j0; jc < j1; jc += kApplyChunk, col += kApplyChunk * ld) {
      T cu[kApplyChunk + 2], cw[kApplyChunk], ce[kApplyChunk];
      cu[0] = um;
      cu[1] = u0;
#pragma unroll
      for (int q = 0; q < kApplyChunk; ++q) {
        const int j = jc + q;
        cu[q + 2] = (j + 1 < n) ? __ldg(col + (size_t)(q + 1) * ld) : T(0);
        if (j < j1 && irow) {
          cw[q] = __ldg(col + (size_t)q * ld - 1);
          ce[q] = __ldg(col + (size_t)q * ld + 1);
        } else {
          cw[q] = ce[q] = T(0);
        }
      }
#pragma unroll
      for (int q = 0; q < kApplyChunk; ++q) {
        const int j = jc + q;
        if (j >= j1) break;
        const T cm = cu[q], c0 = cu[q + 1], cp = cu[q + 2];
        T v;
        if (irow && j > 2 && j < n - 3) {
          double sx;
          if (exact && exact_stencil5((double)c0, (double)cw[q], (double)ce[q], (double)cm,
                                      (double)cp, sx)) {
            v = (T)(sign > 0 ? -sx : sx);
          } else {
            const T sum = (cw[q] + ce[q]) + (cm + cp);
            v = sign > 0 ? fma(T(4), c0, -sum) : fma(T(-4), c0, sum);
          }
        } else {
          // SAT rows and columns: negA reads only in-domain neighbours
          struct G {
            const T* p;
            size_t ld;
            __device__ T operator()(int di, int dj) const {
              return __ldg(p + (ptrdiff_t)dj * (ptrdiff_t)ld + di);
            }
          } g{col + (size_t)q * ld, ld};
          const T na = negA<T>(g, i, j, n);
          v = sign > 0 ? -na : na;
        }
        out.at(i, j) = v;
        if (DOT) acc.add_prod(c0, v);
      }
      um = cu[kApplyChunk];
      u0 = cu[kApplyChunk + 1];
    }
  }
  if (DOT) grid_reduce(acc.value(), rb, [&](double tot) { *dot_out = tot; });
}

// Strip width (columns of a strip, from `cands`) that minimises the march
// steps of the busiest warp: rounds of strips per warp x steps per strip
// (fill + width x per_col).
static int best_strip_cols(int rows_strips, int cols_total, int warps, const int* cands, int nc,
                           int fill, int per_col) {
  long long best = -1;
  int pick = cands[0];
  for (int k = 0; k < nc; ++k) {
    const int w = cands[k];
    const long long items = (long long)rows_strips * ((cols_total + w - 1) / w);
    const long long rounds = (items + warps - 1) / warps;
    const long long cost = rounds * (fill + (long long)per_col * w);
    if (best < 0 || cost < best) {
      best = cost;
      pick = w;
    }
  }
  return pick;
}

// ---------------------------------------------------------------------------
// FP32 operator apply on any layout as a register wave.  The plain 5-point
// interior (rows 1 .. n-2, columns 3 .. n-4) is split into strips of 62 rows
// x `cols` columns; a warp loads 64 rows, lane l holding rows rb0 + 2l and
// rb0 + 2l + 1, and marches along j.  Columns arrive through a register
// queue kApplyAhead columns deep: while column c is used, the load of column
// c + kApplyAhead is issued into the register it frees (the march is
// unrolled by the queue depth, so every queue index is static).  A column
// 8-byte aligned at rb0 (and wholly in the grid) takes one 8-byte load per
// lane, otherwise two 4-byte loads; with an odd leading dimension the two
// alternate from column to column.  The output of column c - 1 is formed
// from the columns c - 2, c - 1, c in registers and the rows above and below
// by one shuffle each way (rows rb0 and rb0 + 63 are halo).  CTAs past the
// wave's take the SAT boundary (rows 0 and n-1, columns 0-2 and n-3..n-1)
// point by point with negA.  Arithmetic per point as in k_apply_direct.
// A queue in registers, instead of a cp.async ring in shared memory, issues
// no shared-memory traffic and no copy-group bookkeeping: 31.3 -> 23.6 us at
// N = 4097.
// ---------------------------------------------------------------------------
constexpr int kApplyRows = 62;
constexpr int kApplyAhead = 8;                   // columns in flight per warp
constexpr int kApplyBoundaryCtas = 32;

struct ApplyWaveArgs {
  const float* u;
  float* out;
  long long ld;
  int n, nsi, nsj, cols, wave_ctas;
};

// 64 registers (the queue is 16 of them): 4 CTAs, 32 warps per SM.
template <bool POS>
__global__ void __launch_bounds__(kThreads, 4) k_apply_wave(const ApplyWaveArgs a) {
  pdl_begin();
  const int n = a.n;
  const long long ld = a.ld;
  const float* __restrict__ u = a.u;
  float* __restrict__ out = a.out;
  if ((int)blockIdx.x >= a.wave_ctas) {
    // SAT boundary: rows 0 and n-1 (all columns), then columns 0, 1, 2,
    // n-3, n-2, n-1 of rows 1 .. n-2
    const long long nb = 2LL * n + 6LL * (n - 2);
    for (long long k = (long long)(blockIdx.x - a.wave_ctas) * kThreads + threadIdx.x; k < nb;
         k += (long long)(gridDim.x - a.wave_ctas) * kThreads) {
      int i, j;
      if (k < 2LL * n) {
        i = (k < n) ? 0 : n - 1;
        j = (int)(k < n ? k : k - n);
      } else {
        const long long k2 = k - 2LL * n;
        const int c = (int)(k2 / (n - 2));
        i = 1 + (int)(k2 % (n - 2));
        j = c < 3 ? c : n - 6 + c;
      }
      struct G {
        const float* p;
        long long ld;
        __device__ float operator()(int di, int dj) const { return __ldg(p + dj * ld + di); }
      } g{u + (long long)j * ld + i, ld};
      const float na = negA<float>(g, i, j, n);
      out[(long long)j * ld + i] = POS ? -na : na;
    }
    return;
  }
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * kThreads + threadIdx.x) >> 5;
  const int nw = (a.wave_ctas * kThreads) >> 5;
  const int items = a.nsi * a.nsj;
  const unsigned FULL = 0xffffffffu;
  const int ldodd = (int)(ld & 1);
  for (int it = gw; it < items; it += nw) {
    const int si = it % a.nsi, sj = it / a.nsi;
    const int rb0 = kApplyRows * si;                       // rows rb0 + 1 .. rb0 + 62 owned
    const int r_hi = min(rb0 + 1 + kApplyRows, n - 1);
    const int c0 = 3 + a.cols * sj;
    const int c1 = min(c0 + a.cols, n - 3);                // output columns [c0, c1)
    const int rown = rb0 + 2 * lane;
    const int dx = min(rown, n - 1) - rown;                // 0, or back to row n-1 past the
    const int dy = min(rown + 1, n - 1) - rown;            // last row (last strip only)
    const bool own_x = lane > 0 && rown < r_hi;
    const bool own_y = lane < 31 && rown + 1 < r_hi;
    const bool in_grid = rb0 + 63 <= n - 1;
    // bit 2 of the address of row rb0 of the next column to load (0: 8-byte
    // aligned), and of the next output column
    int par = (int)(((uintptr_t)(u + rb0 + (long long)(c0 - 1) * ld) >> 2) & 1u);
    int opar = (int)(((uintptr_t)(out + rb0 + (long long)c0 * ld) >> 2) & 1u);
    const float* pf = u + rown + (long long)(c0 - 1) * ld;  // this lane's rows, next column
    auto load = [&]() -> float2 {
      float2 v;
      if (in_grid && par == 0)
        v = __ldg(reinterpret_cast<const float2*>(pf));
      else
        v = make_float2(__ldg(pf + dx), __ldg(pf + dy));
      pf += ld;
      par ^= ldodd;
      return v;
    };
    float2 q2 = load();                                    // column c0 - 1
    float2 q1 = load();                                    // column c0
    const int S = c1 - c0;   // step s: column c0 + 1 + s arrives, column c0 + s is output
    float2 qb[kApplyAhead];
#pragma unroll
    for (int k = 0; k < kApplyAhead; ++k) qb[k] = (k < S) ? load() : make_float2(0.f, 0.f);
    float* o = out + rown + (long long)c0 * ld;
    auto step = [&](const float2 q0) {
      const float up = __shfl_up_sync(FULL, q1.y, 1);     // row rown - 1
      const float dn = __shfl_down_sync(FULL, q1.x, 1);   // row rown + 2
      const float sx = (up + q1.y) + (q2.x + q0.x);
      const float sy = (q1.x + dn) + (q2.y + q0.y);
      const float vx = POS ? fmaf(4.f, q1.x, -sx) : fmaf(-4.f, q1.x, sx);
      const float vy = POS ? fmaf(4.f, q1.y, -sy) : fmaf(-4.f, q1.y, sy);
      if (opar == 0 && own_x && own_y) {
        *reinterpret_cast<float2*>(o) = make_float2(vx, vy);
      } else {
        if (own_x) o[0] = vx;
        if (own_y) o[1] = vy;
      }
      o += ld;
      opar ^= ldodd;
      q2 = q1;
      q1 = q0;
    };
    int s = 0;
    // whole chunks whose refills all stay inside the strip: no guards
    for (; s + 2 * kApplyAhead <= S; s += kApplyAhead) {
#pragma unroll
      for (int k = 0; k < kApplyAhead; ++k) {
        const float2 q0 = qb[k];
        qb[k] = load();
        step(q0);
      }
    }
    for (; s < S; s += kApplyAhead) {
#pragma unroll
      for (int k = 0; k < kApplyAhead; ++k) {
        if (s + k < S) {
          const float2 q0 = qb[k];
          if (s + k + kApplyAhead < S) qb[k] = load();
          step(q0);
        }
      }
    }
  }
}

static int apply_wave_per_sm() {
  static const int v = [] {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_apply_wave<true>, kThreads, 0) !=
            cudaSuccess ||
        b < 1)
      b = 1;
    return b;
  }();
  return v;
}

static cudaError_t launch_apply_wave(const float* u, float* out, long long ld, int n, int sign,
                                     cudaStream_t s) {
  ApplyWaveArgs a;
  a.u = u;
  a.out = out;
  a.ld = ld;
  a.n = n;
  a.nsi = (n - 2 + kApplyRows - 1) / kApplyRows;
  const int slots = sm_count() * apply_wave_per_sm();
  static const int cands[] = {16, 24, 32, 40, 48, 64, 96, 128};
  a.cols = best_strip_cols(a.nsi, n - 6, slots * kWarps, cands, 8, 4, 1);
  a.nsj = (n - 6 + a.cols - 1) / a.cols;
  const int items = a.nsi * a.nsj;
  a.wave_ctas = std::max(1, std::min((items + kWarps - 1) / kWarps, slots));
  if (sign > 0)
    return launch_pdl(k_apply_wave<true>, dim3(a.wave_ctas + kApplyBoundaryCtas), dim3(kThreads),
                      0, s, a);
  return launch_pdl(k_apply_wave<false>, dim3(a.wave_ctas + kApplyBoundaryCtas), dim3(kThreads),
                    0, s, a);
}

template <typename T>
cudaError_t launch_apply(Grid<const T> u, Grid<T> out, int n, int sign, ReduceBuf rb,
                         double* dot_out, cudaStream_t s) {
  if (std::is_same<T, float>::value && !dot_out && n >= 65 && u.ld == out.ld)
    return launch_apply_wave(reinterpret_cast<const float*>(u.p), reinterpret_cast<float*>(out.p),
                             u.ld, n, sign, s);
  const long long items = (long long)((n + kThreads - 1) / kThreads) *
                          ((n + kApplyCols - 1) / kApplyCols);
  const int grid = (int)std::min<long long>(items, kMaxPersistCtas);
  if (dot_out)
    return launch_pdl(k_apply_direct<T, true>, dim3(grid), dim3(kThreads), 0, s, u, out, n, sign,
                      rb, dot_out);
  return launch_pdl(k_apply_direct<T, false>, dim3(grid), dim3(kThreads), 0, s, u, out, n, sign,
                    rb, dot_out);
}

template <typename T>
cudaError_t launch_residual_op(const Operand& x, const Operand& b, Grid<T> r, Grid<float> rlo,
                               int n, int opsign, SolveState* st, double* norms, double abstol,
                               double reltol, int plain, double* out2, ReduceBuf rb,
                               cudaStream_t s, Grid<T> xcopy) {
  const dim3 g = tile_grid(n);
  const int total = (int)(g.x * g.y);
  ResFin rf{st, norms, abstol, reltol, plain, out2};
  const DevOperand<T> dx = dev_operand<T>(x), db = dev_operand<T>(b);
#define SBP_RES(MX, MB)                                                                          \
  return launch_persist(                                                                         \
      ResidualJob<T, MX, MB>{dx, db, r, rlo, n, (int)g.x, total, opsign, rf, rb, xcopy}, total, s)
  if (x.tma && b.tma) SBP_RES(true, true);
  if (x.tma) SBP_RES(true, false);
  if (b.tma) SBP_RES(false, true);
  SBP_RES(false, false);
#undef SBP_RES
}

template <typename T>
cudaError_t launch_residual(Grid<const T> x, Grid<const T> b, Grid<T> r, Grid<float> rlo, int n,
                            int opsign, SolveState* st, double* norms, double abstol,
                            double reltol, int plain, double* out2, ReduceBuf rb,
                            cudaStream_t s) {
  return launch_residual_op<T>(raw_operand(x.p, n, x.ld), raw_operand(b.p, n, b.ld), r, rlo, n,
                               opsign, st, norms, abstol, reltol, plain, out2, rb, s);
}

template <typename T, typename Tz>
cudaError_t launch_cg_dir_op(const Operand& z, const Operand& pold, Grid<T> pnew, Grid<T> Ap,
                             int n, int opsign, SolveState* st, ReduceBuf rb, cudaStream_t s) {
  const dim3 g = tile_grid(n);
  const int total = (int)(g.x * g.y);
  const DevOperand<Tz> dz = dev_operand<Tz>(z);
  const DevOperand<T> dp = dev_operand<T>(pold);
  if (z.tma && pold.tma)
    return launch_persist(
        CgDirJob<T, Tz, true>{dz, dp, pnew, Ap, n, (int)g.x, total, opsign, st, rb}, total, s);
  return launch_persist(
      CgDirJob<T, Tz, false>{dz, dp, pnew, Ap, n, (int)g.x, total, opsign, st, rb}, total, s);
}

template <typename T, typename Tz>
cudaError_t launch_cg_dir(Grid<const Tz> z, Grid<const T> pold, Grid<T> pnew, Grid<T> Ap, int n,
                          int opsign, SolveState* st, ReduceBuf rb, cudaStream_t s) {
  return launch_cg_dir_op<T, Tz>(raw_operand(z.p, n, z.ld), raw_operand(pold.p, n, pold.ld), pnew,
                                 Ap, n, opsign, st, rb, s);
}

template <typename T>
cudaError_t launch_cg_update(Grid<T> x, Grid<T> r, Grid<const T> p, Grid<const T> Ap,
                             Grid<float> rlo, int n, int plain, SolveState* st, double* norms,
                             ReduceBuf rb, cudaStream_t s, const float* pf) {
  static_assert(sizeof(T) == 8, "the Krylov vectors are FP64");
  const int ld = x.ld;
  if (r.ld != ld || (!pf && p.ld != ld) || Ap.ld != ld || (rlo.p && rlo.ld != ld) || ld < n)
    return cudaErrorInvalidValue;
  const long long N = (long long)ld * n;
  const bool vec = aligned16(x.p) && aligned16(r.p) && (pf ? ((uintptr_t)pf & 7u) == 0
                                                           : aligned16(p.p)) &&
                   aligned16(Ap.p) && (!rlo.p || ((uintptr_t)rlo.p & 7u) == 0) &&
                   (ld % 2 == 0 || N % 2 == 0);
  const int g =
      std::min(flat_grid(N, vec ? 4 : 2), vec ? cg_update_wave<true>() : cg_update_wave<false>());
  const CgUpdateArgs a{x.p, r.p, pf ? nullptr : p.p, pf, Ap.p, rlo.p, N, plain, st, norms, rb};
  if (recorder_slot())
    return vec ? record_launch(&launch_cg_update_batch<true>, a, g)
               : record_launch(&launch_cg_update_batch<false>, a, g);
  if (vec) return launch_pdl(k_cg_update<true>, dim3(g), dim3(kThreads), 0, s, a);
  return launch_pdl(k_cg_update<false>, dim3(g), dim3(kThreads), 0, s, a);
}

template <typename T, int FIELD, int EPI, bool TMA>
static cudaError_t launch_smooth_fem(const DevOperand<T>& vin, const DevOperand<T>& e,
                                     const DevOperand<T>& b, Grid<T> vout, int n, int smoother,
                                     double omega, int dot, SolveState* st, ReduceBuf rb,
                                     cudaStream_t s) {
  const dim3 g = tile_grid(n);
  const int total = (int)(g.x * g.y);
  if (dot)
    return launch_persist(SmoothJob<T, FIELD, EPI, true, TMA>{vin, e, b, vout, n, (int)g.x, total,
                                                              smoother, T(omega), st, rb},
                          total, s);
  return launch_persist(SmoothJob<T, FIELD, EPI, false, TMA>{vin, e, b, vout, n, (int)g.x, total,
                                                             smoother, T(omega), st, rb},
                        total, s);
}

template <typename T>
cudaError_t launch_smooth_op(int field, int epi, const Operand& vin, const Operand& e,
                             const Operand& b, Grid<T> vout, int n, int smoother, double omega,
                             int dot, SolveState* st, ReduceBuf rb, cudaStream_t s) {
  if (dot && !st) return cudaErrorInvalidValue;
  const DevOperand<T> dv = dev_operand<T>(vin), de = dev_operand<T>(e), db = dev_operand<T>(b);
  // TMA only when every operand the variant stages is TMA-addressable
  const bool need_b = (epi == kEpiSweep) || dot;
  bool tma = (field == kFieldZero ? b.tma : vin.tma);
  if (need_b) tma = tma && b.tma;
  if (field == kFieldProlong) tma = tma && e.tma;
#define SBP_SMOOTH_CASE(F, E)                                                                    \
  if (field == F && epi == E) {                                                                  \
    if (tma)                                                                                     \
      return launch_smooth_fem<T, F, E, true>(dv, de, db, vout, n, smoother, omega, dot, st, rb, \
                                              s);                                                \
    return launch_smooth_fem<T, F, E, false>(dv, de, db, vout, n, smoother, omega, dot, st, rb,  \
                                             s);                                                 \
  }
  SBP_SMOOTH_CASE(kFieldPlain, kEpiSweep)
  SBP_SMOOTH_CASE(kFieldPlain, kEpiStore)
  SBP_SMOOTH_CASE(kFieldZero, kEpiSweep)
  SBP_SMOOTH_CASE(kFieldZero, kEpiStore)
  SBP_SMOOTH_CASE(kFieldProlong, kEpiSweep)
  SBP_SMOOTH_CASE(kFieldProlong, kEpiStore)
#undef SBP_SMOOTH_CASE
  return cudaErrorInvalidValue;
}

template <typename T>
cudaError_t launch_smooth(int field, int epi, Grid<const T> vin, Grid<const T> e, Grid<const T> b,
                          Grid<T> vout, int n, int smoother, double omega, int dot,
                          SolveState* st, ReduceBuf rb, cudaStream_t s) {
  const int nc = (n + 1) / 2;
  return launch_smooth_op<T>(field, epi, raw_operand(vin.p, n, vin.ld),
                             raw_operand(e.p, nc, e.ld), raw_operand(b.p, n, b.ld), vout, n,
                             smoother, omega, dot, st, rb, s);
}

template <typename T>
cudaError_t launch_resrestrict_op(const Operand* v, const Operand& b, Grid<T> f, int nf, int kind,
                                  const SolveState* st, cudaStream_t s) {
  const int nc = (nf + 1) / 2;
  const int ntx = ntiles(nc, RTI), nty = ntiles(nc, RTJ);
  const int total = ntx * nty;
  const Operand vv = v ? *v : Operand();
  const DevOperand<T> dv = dev_operand<T>(vv), db = dev_operand<T>(b);
  const int has_v = v ? 1 : 0;
  if (b.tma && (!v || v->tma))
    return launch_persist(
        ResRestrictJob<T, true>{dv, db, f, nf, nc, ntx, total, kind, has_v, st, ReduceBuf{}},
        total, s);
  return launch_persist(
      ResRestrictJob<T, false>{dv, db, f, nf, nc, ntx, total, kind, has_v, st, ReduceBuf{}},
      total, s);
}

template <typename T>
cudaError_t launch_resrestrict(Grid<const T> v, Grid<const T> b, Grid<T> f, int nf, int kind,
                               const SolveState* st, cudaStream_t s) {
  const Operand vo = raw_operand(v.p, nf, v.ld);
  return launch_resrestrict_op<T>(v.p ? &vo : nullptr, raw_operand(b.p, nf, b.ld), f, nf, kind, st,
                                  s);
}

// Levels with fewer than four large tiles per SM take the small tiles.
// Below one tile per SM a launch is bound by the serial work of one tile per
// CTA, not by HBM.  Between one and four, whole tiles balance badly over the
// resident CTAs: 512 large tiles of the N = 1025 level on 456 CTAs leave 56
// CTAs a second tile.  Mixed V-cycle at N = 4097: 454 us with large tiles
// everywhere, 432 us with small tiles below 152 large ones, 430 us below 608.
static bool small_fused_tiles(int ncoarse) {
  return ntiles(ncoarse, RTI) * ntiles(ncoarse, RTJ) < 4 * sm_count();
}

template <typename T, class G>
static cudaError_t launch_pre_fused_geom(const Operand& b, Grid<T> vout, Grid<T> f, int nf,
                                         int sweeps, int smoother, double omega, int kind,
                                         const SolveState* st, cudaStream_t s, int ring = 0) {
  const int nc = (nf + 1) / 2;
  const int ntx = ntiles(nc, G::RI), nty = ntiles(nc, G::RJ);
  const int total = ring ? ntx * nty - (ntx - 2 * ring) * (nty - 2 * ring) : ntx * nty;
  const DevOperand<T> db = dev_operand<T>(b);
  CUtensorMap bm{};
  const bool tma = b.tma && make_box_map(bm, b, sizeof(T) == 8, G::BI, G::BJ);
  if (tma)
    return launch_persist(PreFusedJob<T, true, G>{db, bm, vout, f, nf, nc, ntx, total, sweeps,
                                                  smoother, kind, T(omega), st, ReduceBuf{},
                                                  ring, nty},
                          total, s);
  return launch_persist(PreFusedJob<T, false, G>{db, bm, vout, f, nf, nc, ntx, total, sweeps,
                                                 smoother, kind, T(omega), st, ReduceBuf{},
                                                 ring, nty},
                        total, s);
}

// ---------------------------------------------------------------------------
// Register wave pre-smoothing for the interior of a fine level (FP32, three
// Jacobi/Richardson sweeps from zero, residual, restriction), the job of
// PreFusedJob's interior tiles without shared memory or block barriers.
//
// A warp owns a strip of 28 coarse rows x `cols` coarse columns of the
// interior rectangle [Ia, Ib) x [Ja, Jb) (the union of the PreSmall tiles
// that are neither in the first nor in the last tile row or column: every
// point there and in its halo has the plain 5-point stencil and the
// constant smoother weight); the last row strip is moved up to end at Ib.  Lane l holds fine rows 2 I0 - 4 + 2l and the
// row after it (64 rows: 56 owned plus a 4-row halo on each side), and the
// warp marches along j with every stage one column behind the previous:
//   step c: b at column c (loaded D columns ahead as one float2 per lane),
//           v2 at c - 1 (from b, v1 = m b folded in),
//           v3 at c - 2, residual r at c - 3,
//           f(I, J) once r reaches column 2J + 1.
// The i-neighbours of a lane's two rows are its own other row and one row of
// the lane above or below (one shuffle per point per stage); the
// j-neighbours are the stage's previous and next columns, kept in registers.
// v3 on owned points and f are stored straight from registers.  The sums are
// formed in the same order as PreFusedJob's interior path.
// ---------------------------------------------------------------------------
constexpr int kWaveRows = 28;     // coarse rows of a strip
constexpr int kWaveAhead = 16;    // columns of b in flight per warp
constexpr int kWaveSlots = kWaveAhead + 1;   // per-warp ring of b columns

struct PreWaveArgs {
  const float* b;
  int ldb;
  float* vout;
  int ldv;
  float* f;
  int ldf;
  int nf, Ia, Ib, Ja, Jb, nsi, nsj, cols;   // cols: coarse columns of a strip
  float m, k1, m2, sc;
  const SolveState* st;
};

__device__ __forceinline__ void cp_async8(void* sdst, const void* gsrc) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(smem_u32(sdst)), "l"(gsrc)
               : "memory");
}

// b columns come through a per-lane ring in shared memory filled by cp.async
// kWaveAhead columns ahead (one commit group per column; a lane reads only
// its own slots, so the wait needs no warp or block barrier).  The slot a
// copy refills was read one step earlier.
__global__ void __launch_bounds__(kThreads) k_pre_wave(const PreWaveArgs a) {
  __shared__ __align__(16) float2 ring[kWarps][kWaveSlots][32];
  pdl_begin();
  if (a.st && a.st->done) return;
  const int lane = threadIdx.x & 31;
  const int wl = threadIdx.x >> 5;
  const int gw = (blockIdx.x * kThreads + threadIdx.x) >> 5;
  const int nw = (gridDim.x * kThreads) >> 5;
  const int items = a.nsi * a.nsj;
  const unsigned FULL = 0xffffffffu;
  for (int it = gw; it < items; it += nw) {
    const int si = it % a.nsi, sj = it / a.nsi;
    // the strip owns coarse rows [In, I1); the last one is moved up to end
    // at Ib so that its loads stay 28 fine rows inside the grid
    const int In = a.Ia + kWaveRows * si;
    const int I0 = min(In, a.Ib - kWaveRows);
    const int I1 = min(In + kWaveRows, a.Ib);
    const int J0 = a.Ja + a.cols * sj;
    const int J1 = min(J0 + a.cols, a.Jb);
    const int ra = 2 * I0 - 4 + 2 * lane;               // this lane's first fine row
    const int I = I0 + lane - 2;                          // coarse row centred on ra
    const bool own_rows = lane >= 2 && I >= In && I < I1;
    const bool own_f = own_rows;
    const int c_first = 2 * J0 - 4, c_last = 2 * J1 + 2;  // leading columns marched
    const float* bp = a.b + (size_t)ra;
    float2* const mine = &ring[wl][0][lane];
    // prologue: columns c_first .. c_first + kWaveAhead - 1 (empty groups
    // past the strip keep the group count per column)
#pragma unroll
    for (int k = 0; k < kWaveAhead; ++k) {
      const int c = c_first + k;
      if (c <= c_last) cp_async8(mine + k * 32, bp + (size_t)c * a.ldb);
      cp_async_commit();
    }
    int slot = 0, fill = kWaveAhead;                      // ring slots of columns c, c + ahead
    float2 b1 = make_float2(0.f, 0.f), b2 = b1, b3 = b1;  // b at c-1, c-2, c-3
    float2 v2a = b1, v2b = b1;                            // v2 at c-2, c-3
    float2 v3a = b1, v3b = b1;                            // v3 at c-3, c-4
    float t1 = 0.f, t2 = 0.f;                             // row-combined r at c-4, c-5
    for (int c = c_first; c <= c_last; ++c) {
      cp_async_wait<kWaveAhead - 1>();                    // column c has landed
      const float2 b0 = mine[slot * 32];
      {
        const int cn = c + kWaveAhead;
        if (cn <= c_last) cp_async8(mine + fill * 32, bp + (size_t)cn * a.ldb);
        cp_async_commit();
      }
      slot = slot + 1 == kWaveSlots ? 0 : slot + 1;
      fill = fill + 1 == kWaveSlots ? 0 : fill + 1;
      // v2 at column c - 1 from b at c - 2, c - 1, c
      float2 v2;
      {
        const float up = __shfl_up_sync(FULL, b1.y, 1);    // row ra - 1
        const float dn = __shfl_down_sync(FULL, b1.x, 1);  // row ra + 2
        v2.x = fmaf(a.m2, (up + b1.y) + (b2.x + b0.x), a.k1 * b1.x);
        v2.y = fmaf(a.m2, (b1.x + dn) + (b2.y + b0.y), a.k1 * b1.y);
      }
      // v3 at column c - 2 from v2 at c - 3, c - 2, c - 1
      float2 v3;
      {
        const float up = __shfl_up_sync(FULL, v2a.y, 1);
        const float dn = __shfl_down_sync(FULL, v2a.x, 1);
        v3.x = fmaf(a.m, b2.x + (((up + v2a.y) + (v2b.x + v2.x)) - 4.f * v2a.x), v2a.x);
        v3.y = fmaf(a.m, b2.y + (((v2a.x + dn) + (v2b.y + v2.y)) - 4.f * v2a.y), v2a.y);
      }
      // v3 at column c - 2 is final: store the owned points
      if (own_rows && c - 2 >= 2 * J0 && c - 2 <= 2 * J1 - 1)
        *reinterpret_cast<float2*>(a.vout + (size_t)(c - 2) * a.ldv + ra) = v3;
      // residual at column c - 3 from v3 at c - 4, c - 3, c - 2
      float2 r;
      {
        const float up = __shfl_up_sync(FULL, v3a.y, 1);
        const float dn = __shfl_down_sync(FULL, v3a.x, 1);
        const float nbx = (up + v3a.y) + (v3b.x + v3.x);
        const float nby = (v3a.x + dn) + (v3b.y + v3.y);
        r.x = b3.x + (nbx - 4.f * v3a.x);
        r.y = b3.y + (nby - 4.f * v3a.y);
      }
      // restriction: row-combine at column c - 3 for the coarse row centred
      // on ra (rows ra - 1, ra, ra + 1), then f when c - 3 = 2J + 1
      const float rup = __shfl_up_sync(FULL, r.y, 1);
      const float t0 = fmaf(0.5f, rup + r.y, r.x);
      const int cr = c - 3;
      if (((cr - 1) & 1) == 0 && cr >= 2 * J0 + 1 && cr <= 2 * J1 - 1) {
        const int J = (cr - 1) >> 1;
        if (own_f) a.f[(size_t)J * a.ldf + I] = a.sc * fmaf(0.5f, t2 + t0, t1);
      }
      // shift the windows
      t2 = t1;
      t1 = t0;
      v3b = v3a;
      v3a = v3;
      v2b = v2a;
      v2a = v2;
      b3 = b2;
      b2 = b1;
      b1 = b0;
    }
    cp_async_wait<0>();   // no copy outlives the strip
  }
}

// Whether the interior rectangle of the PreSmall tiling (all but its first
// and last tile rows and columns) is non-empty and which coarse range it
// covers; the boundary ring around it is one small tile deep.
static bool pre_wave_rect(int nc, int& Ia, int& Ib, int& Ja, int& Jb) {
  constexpr int RI = PreSmall::RI, RJ = PreSmall::RJ;
  const int ntx = ntiles(nc, RI), nty = ntiles(nc, RJ);
  if (ntx < 3 || nty < 3) return false;
  if ((nc - 1) % RI != 0 || (nc - 1) % RJ != 0) return false;   // full tiles only
  Ia = RI + 1;
  Ib = RI * (ntx - 1) + 1;
  Ja = RJ + 1;
  Jb = RJ * (nty - 1) + 1;
  return Ib - Ia >= kWaveRows && Ja < Jb;
}

static cudaError_t launch_pre_wave(const Operand& b, Grid<float> vout, Grid<float> f, int nf,
                                   int Ia, int Ib, int Ja, int Jb, int smoother, double omega,
                                   int kind, const SolveState* st, cudaStream_t s) {
  PreWaveArgs a;
  a.b = static_cast<const float*>(b.p);
  a.ldb = b.ld;
  a.vout = vout.p;
  a.ldv = vout.ld;
  a.f = f.p;
  a.ldf = f.ld;
  a.nf = nf;
  a.Ia = Ia;
  a.Ib = Ib;
  a.Ja = Ja;
  a.Jb = Jb;
  a.nsi = (Ib - Ia + kWaveRows - 1) / kWaveRows;
  const float m = (smoother == kSmoothJacobi) ? (float)omega * 0.25f : (float)omega;
  a.m = m;
  a.k1 = 2.f * m - 4.f * m * m;
  a.m2 = m * m;
  a.sc = (kind == kRestrictGalerkin) ? 1.f : 0.25f;
  a.st = st;
  static const int per_sm = [] {
    int v = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_pre_wave, kThreads, 0) != cudaSuccess ||
        v < 1)
      v = 1;
    return v;
  }();
  static const int cands[] = {4, 8, 12, 16, 24, 32};   // coarse columns
  a.cols = best_strip_cols(a.nsi, Jb - Ja, sm_count() * per_sm * kWarps, cands, 6, 7, 2);
  a.nsj = (Jb - Ja + a.cols - 1) / a.cols;
  const int items = a.nsi * a.nsj;
  const int grid = std::max(1, std::min((items + kWarps - 1) / kWarps, sm_count() * per_sm));
  return launch_pdl(k_pre_wave, dim3(grid), dim3(kThreads), 0, s, a);
}

// Fine levels from this size up smooth their interior as a register wave
// (FP32, three sweeps).  At N = 1025 the staged small tiles took about four
// times the wave's time: one tile's serial passes per CTA.
constexpr int kWaveMinFine = 1025;

int pre_fused_launches(int nf, int sweeps, bool f32) {
  int Ia, Ib, Ja, Jb;
  if (f32 && sweeps == 3 && nf >= kWaveMinFine && pre_wave_rect((nf + 1) / 2, Ia, Ib, Ja, Jb))
    return 2;
  return 1;
}

template <typename T>
cudaError_t launch_pre_fused(const Operand& b, Grid<T> vout, Grid<T> f, int nf, int sweeps,
                             int smoother, double omega, int kind, const SolveState* st,
                             cudaStream_t s, cudaStream_t aux, cudaEvent_t fork,
                             cudaEvent_t join) {
  if (sweeps < 1 || sweeps > kMaxFusedSweeps) return cudaErrorInvalidValue;
  int Ia, Ib, Ja, Jb;
  if (std::is_same<T, float>::value && sweeps == 3 && nf >= kWaveMinFine && !recorder_slot() &&
      (b.ld % 2) == 0 && (vout.ld % 2) == 0 && ((uintptr_t)b.p & 7u) == 0 &&
      ((uintptr_t)vout.p & 7u) == 0 && pre_wave_rect((nf + 1) / 2, Ia, Ib, Ja, Jb)) {
    // boundary tiles by the staged job (on a forked branch when one is
    // given: it is latency-bound and overlaps the wave), the interior by the
    // register wave
    const bool forked = aux && fork && join;
    cudaError_t e = cudaSuccess;
    if (forked) {
      e = cudaEventRecord(fork, s);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(aux, fork, 0);
    }
    // the ring: one small tile deep
    if (e == cudaSuccess)
      e = launch_pre_fused_geom<T, PreSmall>(b, vout, f, nf, sweeps, smoother, omega, kind, st,
                                             forked ? aux : s, 1);
    if (forked && e == cudaSuccess) e = cudaEventRecord(join, aux);
    if (e != cudaSuccess) return e;
    e = launch_pre_wave(b, Grid<float>{reinterpret_cast<float*>(vout.p), vout.ld},
                        Grid<float>{reinterpret_cast<float*>(f.p), f.ld}, nf, Ia, Ib, Ja, Jb,
                        smoother, omega, kind, st, s);
    if (forked && e == cudaSuccess) e = cudaStreamWaitEvent(s, join, 0);
    return e;
  }
  if (small_fused_tiles((nf + 1) / 2))
    return launch_pre_fused_geom<T, PreSmall>(b, vout, f, nf, sweeps, smoother, omega, kind, st,
                                              s);
  return launch_pre_fused_geom<T, PreLarge>(b, vout, f, nf, sweeps, smoother, omega, kind, st,
                                            s);
}

template <typename T, class G>
static cudaError_t launch_post_fused_geom(const Operand& vin, const Operand& e, const Operand& b,
                                          Grid<T> vout, int n, int sweeps, int smoother,
                                          double omega, int dot, SolveState* st, ReduceBuf rb,
                                          cudaStream_t s, int ring = 0, int partial = 0) {
  const int ntx = ntiles(n, G::TI), nty = ntiles(n, G::TJ);
  const int total = ring ? ntx * nty - (ntx - 2 * ring) * (nty - 2 * ring) : ntx * nty;
  const bool f64 = sizeof(T) == 8;
  CUtensorMap vm{}, bm{}, em{};
  const bool tma = vin.tma && b.tma && e.tma && make_box_map(vm, vin, f64, G::BI, G::BJ) &&
                   make_box_map(bm, b, f64, G::BI, G::BJ) && make_box_map(em, e, f64, G::CI, G::CJ);
  const DevOperand<T> dv = dev_operand<T>(vin), de = dev_operand<T>(e), db = dev_operand<T>(b);
#define SBP_POST(D, M)                                                                           \
  return launch_persist(PostFusedJob<T, D, M, G>{dv, de, db, vm, bm, em, vout, n, ntx, total,   \
                                                 sweeps, smoother, T(omega), st, rb, ring, nty,  \
                                                 partial},                                      \
                        total, s)
  if (dot) {
    if (tma) SBP_POST(true, true);
    SBP_POST(true, false);
  }
  if (tma) SBP_POST(false, true);
  SBP_POST(false, false);
#undef SBP_POST
}

// ---------------------------------------------------------------------------
// Register wave post-smoothing for the interior of a fine level (FP32,
// prolongation of the coarse correction + three sweeps, optional b.v dot),
// the job of PostFusedJob's interior tiles without shared-memory sweeps or
// block barriers.  A warp owns a strip of up to 56 fine rows x `cols` fine
// columns of the interior rectangle [Ra, Rb) x [Ca, Cb) (the union of the
// PostSmall tiles outside the first and last tile rows and columns); the
// last row strip loads from higher up so that it ends inside the grid.  Lane l
// holds fine rows rb0 + 2l (even: coarse row rb0/2 + l) and rb0 + 2l + 1;
// the warp marches along j:
//   step c: F0 = v_in + P e at column c, sweep 1 at c - 1, sweep 2 at
//           c - 2, sweep 3 at c - 3 (final: stored, and b.v accumulated).
// The odd row of a lane interpolates its coarse row and the next lane's; an
// odd column averages the coarse columns on either side.  v_in and b come
// through per-lane cp.async rings kPostAhead columns ahead; e (coarse) is
// loaded two coarse columns ahead.  Arithmetic order as in the interior
// path of PostFusedJob.
// ---------------------------------------------------------------------------
constexpr int kPostRows = 56;
constexpr int kRingPartialsOffset = 2080;
static_assert(kRingPartialsOffset + 2080 <= kMaxPersistCtas + 64, "split partials buffer");
constexpr int kPostAhead = 10;
constexpr int kPostSlots = kPostAhead + 1;

struct PostWaveArgs {
  const float* vin;
  int ldv;
  const float* b;
  int ldb;
  const float* e;
  int lde;
  float* vout;
  int ldo;
  int n, Ra, Rb, Ca, Cb, nsi, nsj, cols;   // cols: fine columns of a strip
  float m;
  SolveState* st;
  ReduceBuf rb;
};

template <bool DOT>
__global__ void __launch_bounds__(kThreads, 4) k_post_wave(const PostWaveArgs a) {
  __shared__ __align__(16) float2 vring[kWarps][kPostSlots][32];
  __shared__ __align__(16) float2 bring[kWarps][kPostSlots][32];
  pdl_begin();
  if (a.st && a.st->done) return;   // uniform: the state was final before this launch
  const int lane = threadIdx.x & 31;
  const int wl = threadIdx.x >> 5;
  const int gw = (blockIdx.x * kThreads + threadIdx.x) >> 5;
  const int nw = (gridDim.x * kThreads) >> 5;
  const int items = a.nsi * a.nsj;
  const unsigned FULL = 0xffffffffu;
  const float m = a.m;
  DotAcc<float> acc;
  for (int it = gw; it < items; it += nw) {
    const int si = it % a.nsi, sj = it / a.nsi;
    // the strip owns rows [r_lo, r_hi); the last one loads from the even row
    // at or above Rb - 60, so that its loads stay inside the grid
    const int rbn = (a.Ra & ~1) - 4 + kPostRows * si;
    const int rb0 = min(rbn, (a.Rb - 4 - kPostRows + 1) & ~1);   // even
    const int r_lo = max(rbn + 4, a.Ra), r_hi = min(rbn + 4 + kPostRows, a.Rb);
    const int c0 = a.Ca + a.cols * sj;
    const int c1 = min(c0 + a.cols, a.Cb);
    const int ra = rb0 + 2 * lane;
    const bool own_x = ra >= r_lo && ra < r_hi;
    const bool own_y = ra + 1 >= r_lo && ra + 1 < r_hi;
    const int er = (rb0 >> 1) + lane;                       // this lane's coarse row
    const int c_first = c0 - 3, c_last = c1 + 2;
    const float* vp = a.vin + (size_t)ra;
    const float* bp = a.b + (size_t)ra;
    const float* ep = a.e + (size_t)er;
    float2* const vmine = &vring[wl][0][lane];
    float2* const bmine = &bring[wl][0][lane];
#pragma unroll
    for (int k = 0; k < kPostAhead; ++k) {
      const int c = c_first + k;
      if (c <= c_last) {
        cp_async8(vmine + k * 32, vp + (size_t)c * a.ldv);
        cp_async8(bmine + k * 32, bp + (size_t)c * a.ldb);
      }
      cp_async_commit();
    }
    int slot = 0, fill = kPostAhead;
    // row-interpolated coarse values of columns J = c >> 1 and J + 1
    auto rv = [&](float ev) {
      const float en = __shfl_down_sync(FULL, ev, 1);    // coarse row er + 1
      return make_float2(ev, fmaf(0.5f, en, 0.5f * ev));
    };
    int J = c_first >> 1;
    float2 rvc = rv(__ldg(ep + (size_t)J * a.lde));
    float2 rvn = rv(__ldg(ep + (size_t)(J + 1) * a.lde));
    float epre = __ldg(ep + (size_t)(J + 2) * a.lde);
    float2 f1 = make_float2(0.f, 0.f), f2 = f1;             // F0 at c-1, c-2
    float2 w1a = f1, w1b = f1;                              // sweep 1 at c-2, c-3
    float2 w2a = f1, w2b = f1;                              // sweep 2 at c-3, c-4
    float2 b1 = f1, b2 = f1, b3 = f1;                       // b at c-1, c-2, c-3
    for (int c = c_first; c <= c_last; ++c) {
      cp_async_wait<kPostAhead - 1>();                      // column c has landed
      const float2 vi = vmine[slot * 32];
      const float2 b0 = bmine[slot * 32];
      {
        const int cn = c + kPostAhead;
        if (cn <= c_last) {
          cp_async8(vmine + fill * 32, vp + (size_t)cn * a.ldv);
          cp_async8(bmine + fill * 32, bp + (size_t)cn * a.ldb);
        }
        cp_async_commit();
      }
      slot = slot + 1 == kPostSlots ? 0 : slot + 1;
      fill = fill + 1 == kPostSlots ? 0 : fill + 1;
      if (!(c & 1) && c != c_first) {                       // next coarse column
        ++J;
        rvc = rvn;
        rvn = rv(epre);
        epre = __ldg(ep + (size_t)(J + 2) * a.lde);
      }
      float2 f0;
      if (c & 1) {
        f0.x = vi.x + 0.5f * (rvc.x + rvn.x);
        f0.y = vi.y + 0.5f * (rvc.y + rvn.y);
      } else {
        f0.x = vi.x + rvc.x;
        f0.y = vi.y + rvc.y;
      }
      // sweep 1 at column c - 1
      float2 w1;
      {
        const float up = __shfl_up_sync(FULL, f1.y, 1);
        const float dn = __shfl_down_sync(FULL, f1.x, 1);
        w1.x = fmaf(m, b1.x + (((up + f1.y) + (f2.x + f0.x)) - 4.f * f1.x), f1.x);
        w1.y = fmaf(m, b1.y + (((f1.x + dn) + (f2.y + f0.y)) - 4.f * f1.y), f1.y);
      }
      // sweep 2 at column c - 2
      float2 w2;
      {
        const float up = __shfl_up_sync(FULL, w1a.y, 1);
        const float dn = __shfl_down_sync(FULL, w1a.x, 1);
        w2.x = fmaf(m, b2.x + (((up + w1a.y) + (w1b.x + w1.x)) - 4.f * w1a.x), w1a.x);
        w2.y = fmaf(m, b2.y + (((w1a.x + dn) + (w1b.y + w1.y)) - 4.f * w1a.y), w1a.y);
      }
      // sweep 3 at column c - 3: final
      {
        const float up = __shfl_up_sync(FULL, w2a.y, 1);
        const float dn = __shfl_down_sync(FULL, w2a.x, 1);
        float2 w3;
        w3.x = fmaf(m, b3.x + (((up + w2a.y) + (w2b.x + w2.x)) - 4.f * w2a.x), w2a.x);
        w3.y = fmaf(m, b3.y + (((w2a.x + dn) + (w2b.y + w2.y)) - 4.f * w2a.y), w2a.y);
        const int cw = c - 3;
        if (cw >= c0 && cw < c1) {
          float* o = a.vout + (size_t)cw * a.ldo + ra;
          if (own_x && own_y) {
            *reinterpret_cast<float2*>(o) = w3;
          } else {
            if (own_x) o[0] = w3.x;
            if (own_y) o[1] = w3.y;
          }
          if (DOT) {
            if (own_x) acc.add_prod(b3.x, w3.x);
            if (own_y) acc.add_prod(b3.y, w3.y);
          }
        }
      }
      w2b = w2a;
      w2a = w2;
      w1b = w1a;
      w1a = w1;
      f2 = f1;
      f1 = f0;
      b3 = b2;
      b2 = b1;
      b1 = b0;
    }
    cp_async_wait<0>();   // no copy outlives the strip
  }
  // the boundary tiles' share comes from the staged pass running beside
  if (DOT) grid_reduce(acc.value(), a.rb, [&](double tot) { rz_join(a.st, &a.st->rz_wave, tot); });
}

// The interior rectangle of a T1 x T2 tiling of the fine grid (all but its
// first and last tile rows and columns).
template <int T1, int T2>
static bool interior_rect(int n, int& Ra, int& Rb, int& Ca, int& Cb) {
  const int ntx = ntiles(n, T1), nty = ntiles(n, T2);
  if (ntx < 3 || nty < 3) return false;
  if ((n - 1) % T1 != 0 || (n - 1) % T2 != 0) return false;   // full tiles only
  Ra = T1 + 1;
  Rb = T1 * (ntx - 1) + 1;
  Ca = T2 + 1;
  Cb = T2 * (nty - 1) + 1;
  return Ra < Rb && Ca < Cb;
}
// the post-smoothing wave: inside the PostSmall tiling (ring one small tile
// deep)
static bool post_wave_rect(int n, int& Ra, int& Rb, int& Ca, int& Cb) {
  return interior_rect<PostSmall::TI, PostSmall::TJ>(n, Ra, Rb, Ca, Cb) &&
         Rb - Ra >= 4 + kPostRows;
}


int post_fused_launches(int n, int sweeps, bool f32) {
  int Ra, Rb, Ca, Cb;
  if (f32 && sweeps == 3 && n >= kWaveMinFine && post_wave_rect(n, Ra, Rb, Ca, Cb)) return 2;
  return 1;
}

template <typename T>
cudaError_t launch_post_fused(const Operand& vin, const Operand& e, const Operand& b, Grid<T> vout,
                              int n, int sweeps, int smoother, double omega, int dot,
                              SolveState* st, ReduceBuf rb, cudaStream_t s, cudaStream_t aux,
                              cudaEvent_t fork, cudaEvent_t join) {
  if (sweeps < 0 || sweeps > kMaxFusedSweeps || (dot && !st)) return cudaErrorInvalidValue;
  int Ra, Rb, Ca, Cb;
  if (std::is_same<T, float>::value && sweeps == 3 && n >= kWaveMinFine && !recorder_slot() &&
      vin.ld % 2 == 0 &&
      b.ld % 2 == 0 && vout.ld % 2 == 0 && ((uintptr_t)vin.p & 7u) == 0 &&
      ((uintptr_t)b.p & 7u) == 0 && ((uintptr_t)vout.p & 7u) == 0 &&
      post_wave_rect(n, Ra, Rb, Ca, Cb)) {
    // the boundary ring (one quarter-size tile deep) by the staged job on a
    // forked branch; with the dot, the two reductions meet in rz_join
    const bool forked = aux && fork && join;
    cudaError_t e2 = cudaSuccess;
    if (forked) {
      e2 = cudaEventRecord(fork, s);
      if (e2 == cudaSuccess) e2 = cudaStreamWaitEvent(aux, fork, 0);
    }
    // the two reductions run at the same time: the ring takes the upper half
    // of the partials buffer (a solver's holds max_reduce_ctas(n) + 64 >=
    // 4160 slots; neither grid exceeds SMs x 8 = 1216 CTAs) and its own ticket
    const ReduceBuf rb_ring{rb.partials ? rb.partials + kRingPartialsOffset : nullptr,
                            rb.ticket ? rb.ticket + 8 : nullptr};
    if (e2 == cudaSuccess)
      e2 = launch_post_fused_geom<T, PostSmall>(vin, e, b, vout, n, sweeps, smoother, omega, dot,
                                                st, rb_ring, forked ? aux : s, 1, dot ? 1 : 0);
    if (forked && e2 == cudaSuccess) e2 = cudaEventRecord(join, aux);
    if (e2 != cudaSuccess) return e2;
    PostWaveArgs a;
    a.vin = static_cast<const float*>(vin.p);
    a.ldv = vin.ld;
    a.b = static_cast<const float*>(b.p);
    a.ldb = b.ld;
    a.e = static_cast<const float*>(e.p);
    a.lde = e.ld;
    a.vout = reinterpret_cast<float*>(vout.p);
    a.ldo = vout.ld;
    a.n = n;
    a.Ra = Ra;
    a.Rb = Rb;
    a.Ca = Ca;
    a.Cb = Cb;
    a.nsi = (Rb - (Ra & ~1) + kPostRows - 1) / kPostRows;   // strips own from Ra & ~1 on
    a.m = (smoother == kSmoothJacobi) ? (float)omega * 0.25f : (float)omega;
    a.st = st;
    a.rb = rb;
    static const int per_sm[2] = {
        [] {
          int v = 0;
          if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_post_wave<false>, kThreads, 0) !=
                  cudaSuccess ||
              v < 1)
            v = 1;
          return v;
        }(),
        [] {
          int v = 0;
          if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_post_wave<true>, kThreads, 0) !=
                  cudaSuccess ||
              v < 1)
            v = 1;
          return v;
        }()};
    static const int cands[] = {8, 16, 24, 32, 48, 64};   // fine columns
    a.cols = best_strip_cols(a.nsi, Cb - Ca, sm_count() * per_sm[dot ? 1 : 0] * kWarps, cands, 6,
                             6, 1);
    a.nsj = (Cb - Ca + a.cols - 1) / a.cols;
    const int items = a.nsi * a.nsj;
    const int grid =
        std::max(1, std::min((items + kWarps - 1) / kWarps, sm_count() * per_sm[dot ? 1 : 0]));
    e2 = dot ? launch_pdl(k_post_wave<true>, dim3(grid), dim3(kThreads), 0, s, a)
             : launch_pdl(k_post_wave<false>, dim3(grid), dim3(kThreads), 0, s, a);
    if (forked && e2 == cudaSuccess) e2 = cudaStreamWaitEvent(s, join, 0);
    return e2;
  }
  if (small_fused_tiles((n + 1) / 2))
    return launch_post_fused_geom<T, PostSmall>(vin, e, b, vout, n, sweeps, smoother, omega, dot,
                                                st, rb, s);
  return launch_post_fused_geom<T, PostLarge>(vin, e, b, vout, n, sweeps, smoother, omega, dot,
                                              st, rb, s);
}

// ---------------------------------------------------------------------------
// Register wave of the FP32 CG direction (mixed MGCG) over the whole fine
// grid, in one launch.  The plain 5-point points (rows 1 .. n-2, columns
// 3 .. n-4) are split into strips of 62 rows x `cols` columns.  A warp loads
// 64 rows, lane l holding rows rb0 + 2l and rb0 + 2l + 1 (the 62 owned and
// one halo row on either side), and marches along j:
//   step c: p~ = fl32(z + beta p~_old) at column c (stored where owned);
//           A p~ at column c - 1 in float-float from the p~ of columns
//           c - 2, c - 1, c and of the lanes above and below (one shuffle
//           each way), stored in FP64, and p~ . fl32(A p~) accumulated.
// z and p~_old come through per-lane cp.async rings kDirAhead columns ahead;
// a lane reads only its own slots, so no barrier is needed.  The last strip
// starts at the even row at or above n - 64, so on an odd grid its last
// loaded row is row n, a padding row of the solver's arrays (ld > n).
// CTAs past the wave's take the SAT rows and columns (rows 0 and n-1,
// columns 0-2 and n-3 .. n-1) point by point: p~ there and at the
// neighbours negA reads (recomputed from z and p~_old, which no one writes
// in this pass), negA in float-float.  All CTAs then meet in one reduction.
// The arithmetic per point is that of CgDirF32Job.
// ---------------------------------------------------------------------------
constexpr int kDirRows = 62;
constexpr int kDirAhead = 8;
constexpr int kDirSlots = kDirAhead + 1;
constexpr int kDirWaveMinN = 1025;
constexpr int kDirBoundaryCtas = 32;

struct DirWaveArgs {
  const float* z;
  int ldz;
  const float* pold;
  int ldp;
  float* pnew;
  int ldn;
  double* Ap;
  int lda;
  int n, nsi, nsj, cols, wave_ctas;
  SolveState* st;
  ReduceBuf rb;
};

__global__ void __launch_bounds__(kThreads, 5) k_dir_wave(const DirWaveArgs a) {
  __shared__ __align__(16) float2 zring[kWarps][kDirSlots][32];
  __shared__ __align__(16) float2 pring[kWarps][kDirSlots][32];
  pdl_begin();
  SolveState* st = a.st;
  if (st->done) return;   // uniform: the state was final before this launch
  const bool first = (st->iter == 0);   // p~_old is not read
  const float2 beta = make_float2((float)st->beta, (float)st->beta);
  const int n = a.n;
  double partial;
  if ((int)blockIdx.x >= a.wave_ctas) {
    // SAT rows and columns, one point per thread and step
    DotAcc<float> acc;
    const long long nb = 2LL * n + 6LL * (n - 2);
    for (long long k = (long long)(blockIdx.x - a.wave_ctas) * kThreads + threadIdx.x; k < nb;
         k += (long long)(gridDim.x - a.wave_ctas) * kThreads) {
      int i, j;
      if (k < 2LL * n) {
        i = (k < n) ? 0 : n - 1;
        j = (int)(k < n ? k : k - n);
      } else {
        const long long k2 = k - 2LL * n;
        const int c = (int)(k2 / (n - 2));
        i = 1 + (int)(k2 % (n - 2));
        j = c < 3 ? c : n - 6 + c;
      }
      struct G {
        const float* z;
        const float* p;
        int ldz, ldp, i, j;
        float b;
        bool first;
        __device__ float pt(int di, int dj) const {
          const float zz = __ldg(z + (size_t)(j + dj) * ldz + (i + di));
          return first ? zz : fmaf(b, __ldg(p + (size_t)(j + dj) * ldp + (i + di)), zz);
        }
        __device__ FF operator()(int di, int dj) const { return FF(pt(di, dj), 0.0f); }
      } g{a.z, a.pold, a.ldz, a.ldp, i, j, beta.x, first};
      const float pv = g.pt(0, 0);
      const FF na = negA<FF>(g, i, j, n);
      float apf;
      const double ap = dir_ap(na.hi, na.lo, apf);
      a.pnew[(size_t)j * a.ldn + i] = pv;
      a.Ap[(size_t)j * a.lda + i] = ap;
      acc.add_prod(pv, apf);
    }
    partial = acc.value();
  } else {
    const int lane = threadIdx.x & 31;
    const int wl = threadIdx.x >> 5;
    const int gw = (blockIdx.x * kThreads + threadIdx.x) >> 5;
    const int nw = (a.wave_ctas * kThreads) >> 5;
    const int items = a.nsi * a.nsj;
    const unsigned FULL = 0xffffffffu;
    float2* const zmine = &zring[wl][0][lane];
    float2* const pmine = &pring[wl][0][lane];
    DotAcc2 acc;   // p~ . fl32(-A p~), negated at the end
    const int rb_last = (n - 64 + 1) & ~1;                  // even, >= n - 64
    for (int it = gw; it < items; it += nw) {
      const int si = it % a.nsi, sj = it / a.nsi;
      const int rbn = kDirRows * si;
      const int rb0 = min(rbn, rb_last);
      const int r_lo = rbn + 1, r_hi = min(rbn + 1 + kDirRows, n - 1);   // owned rows
      const int c0 = 3 + a.cols * sj;
      const int c1 = min(c0 + a.cols, n - 3);
      const int ra = rb0 + 2 * lane;
      const bool own_x = lane > 0 && ra >= r_lo && ra < r_hi;
      const bool own_y = lane < 31 && ra + 1 >= r_lo && ra + 1 < r_hi;
      const int c_first = c0 - 1, c_last = c1;
      const float* zp = a.z + (size_t)ra;
      const float* pp = a.pold + (size_t)ra;
#pragma unroll
      for (int k = 0; k < kDirAhead; ++k) {
        const int c = c_first + k;
        if (c <= c_last) {
          cp_async8(zmine + k * 32, zp + (size_t)c * a.ldz);
          if (!first) cp_async8(pmine + k * 32, pp + (size_t)c * a.ldp);
        }
        cp_async_commit();
      }
      int slot = 0, fill = kDirAhead;
      float2 q1 = make_float2(0.f, 0.f), q2 = q1;             // p~ at c - 1, c - 2
      for (int c = c_first; c <= c_last; ++c) {
        cp_async_wait<kDirAhead - 1>();                       // column c has landed
        const float2 zv = zmine[slot * 32];
        const float2 q0 = first ? zv : fma2(beta, pmine[slot * 32], zv);
        {
          const int cn = c + kDirAhead;
          if (cn <= c_last) {
            cp_async8(zmine + fill * 32, zp + (size_t)cn * a.ldz);
            if (!first) cp_async8(pmine + fill * 32, pp + (size_t)cn * a.ldp);
          }
          cp_async_commit();
        }
        slot = slot + 1 == kDirSlots ? 0 : slot + 1;
        fill = fill + 1 == kDirSlots ? 0 : fill + 1;
        if (c >= c0 && c < c1) {
          float* o = a.pnew + (size_t)c * a.ldn + ra;
          if (own_x && own_y) {
            *reinterpret_cast<float2*>(o) = q0;
          } else {
            if (own_x) o[0] = q0.x;
            if (own_y) o[1] = q0.y;
          }
        }
        const float above = __shfl_up_sync(FULL, q1.y, 1);    // row ra - 1, column c - 1
        const float below = __shfl_down_sync(FULL, q1.x, 1);  // row ra + 2, column c - 1
        if (c > c0) {                                         // column c - 1 is in [c0, c1)
          // both rows at once: the stencil_ff and dir_ap of the staged path,
          // lane by lane
          float2 hi, lo, sum;
          stencil_ff2(make_float2(above, q1.x), make_float2(q1.y, below), q2, q0, q1, hi, lo);
          double ax, ay;
          ff_neg_f64_2(hi, lo, ax, ay, sum);                  // fl32(A p~) = -sum
          double* o = a.Ap + (size_t)(c - 1) * a.lda + ra;
          if (own_x && own_y) {
            *reinterpret_cast<double2*>(o) = make_double2(ax, ay);
          } else {
            if (own_x) o[0] = ax;
            if (own_y) o[1] = ay;
          }
          // rows not owned (halo, and the padding row n) add exact zeros
          acc.add_prod(make_float2(own_x ? q1.x : 0.f, own_y ? q1.y : 0.f),
                       make_float2(own_x ? sum.x : 0.f, own_y ? sum.y : 0.f));
        }
        q2 = q1;
        q1 = q0;
      }
      cp_async_wait<0>();   // no copy outlives the strip
    }
    partial = -acc.value();
  }
  grid_reduce(partial, a.rb, [&](double tot) { finish_pap(st, tot); });
}

static int dir_wave_per_sm() {
  static const int v = [] {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_dir_wave, kThreads, 0) !=
            cudaSuccess ||
        b < 1)
      b = 1;
    return b;
  }();
  return v;
}

// The wave needs odd n >= kDirWaveMinN (its last strip reads the padding
// row n), arrays with ld > n, and 8-byte aligned columns.
cudaError_t launch_cg_dir_f32(const Operand& z, const Operand& pold, Grid<float> pnew,
                              Grid<double> Ap, int n, SolveState* st, ReduceBuf rb,
                              cudaStream_t s) {
  const bool wave = n >= kDirWaveMinN && (n & 1) && !recorder_slot() && z.ld > n &&
                    pold.ld > n && z.ld % 2 == 0 && pold.ld % 2 == 0 && pnew.ld % 2 == 0 &&
                    Ap.ld % 2 == 0 && ((uintptr_t)z.p & 7u) == 0 &&
                    ((uintptr_t)pold.p & 7u) == 0 && ((uintptr_t)pnew.p & 7u) == 0 &&
                    aligned16(Ap.p);
  if (!wave) return launch_cg_dir_f32_staged(z, pold, pnew, Ap, n, st, rb, s);
  DirWaveArgs a;
  a.z = static_cast<const float*>(z.p);
  a.ldz = z.ld;
  a.pold = static_cast<const float*>(pold.p);
  a.ldp = pold.ld;
  a.pnew = pnew.p;
  a.ldn = pnew.ld;
  a.Ap = Ap.p;
  a.lda = Ap.ld;
  a.n = n;
  a.nsi = (n - 2 + kDirRows - 1) / kDirRows;
  a.st = st;
  a.rb = rb;
  const int warps = sm_count() * dir_wave_per_sm() * kWarps;
  static const int cands[] = {16, 24, 32, 40, 48, 64, 96};
  a.cols = best_strip_cols(a.nsi, n - 6, warps, cands, 7, 8, 1);
  a.nsj = (n - 6 + a.cols - 1) / a.cols;
  const int items = a.nsi * a.nsj;
  a.wave_ctas = std::max(1, std::min((items + kWarps - 1) / kWarps, sm_count() * dir_wave_per_sm()));
  return launch_pdl(k_dir_wave, dim3(a.wave_ctas + kDirBoundaryCtas), dim3(kThreads), 0, s, a);
}

// Resolve the launch configuration of every persistent kernel up front
// (shared-memory attribute and occupancy), outside any stream capture.
template <typename T, int F, int E, bool M>
static void prep_smooth() {
  persist_ctas_per_sm<SmoothJob<T, F, E, false, M>>();
  persist_ctas_per_sm<SmoothJob<T, F, E, true, M>>();
}
template <typename T, bool M>
static void prepare_precision() {
  persist_ctas_per_sm<ApplyJob<T, false, M>>();
  persist_ctas_per_sm<ApplyJob<T, true, M>>();
  persist_ctas_per_sm<ResRestrictJob<T, M>>();
  prep_smooth<T, kFieldPlain, kEpiSweep, M>();
  prep_smooth<T, kFieldPlain, kEpiStore, M>();
  prep_smooth<T, kFieldZero, kEpiSweep, M>();
  prep_smooth<T, kFieldZero, kEpiStore, M>();
  prep_smooth<T, kFieldProlong, kEpiSweep, M>();
  prep_smooth<T, kFieldProlong, kEpiStore, M>();
}

cudaError_t prepare_coarse_kernels();

cudaError_t prepare_kernels() {
  sm_count();
  if (cudaError_t e = prepare_coarse_kernels(); e != cudaSuccess) return e;
  prepare_precision<double, false>();
  prepare_precision<double, true>();
  prepare_precision<float, false>();
  prepare_precision<float, true>();
  persist_ctas_per_sm<ResidualJob<double, false, false>>();
  persist_ctas_per_sm<ResidualJob<double, true, false>>();
  persist_ctas_per_sm<ResidualJob<double, true, true>>();
  persist_ctas_per_sm<ResidualJob<double, false, true>>();
  persist_ctas_per_sm<CgDirJob<double, double, false>>();
  persist_ctas_per_sm<CgDirJob<double, double, true>>();
  persist_ctas_per_sm<CgDirJob<double, float, false>>();
  persist_ctas_per_sm<CgDirJob<double, float, true>>();
  persist_ctas_per_sm<CgDirF32Job<false>>();
  persist_ctas_per_sm<PreFusedJob<float, true>>();
  persist_ctas_per_sm<PreFusedJob<float, false>>();
  persist_ctas_per_sm<PreFusedJob<double, true>>();
  persist_ctas_per_sm<PreFusedJob<double, false>>();
  persist_ctas_per_sm<PostFusedJob<float, false, true>>();
  persist_ctas_per_sm<PostFusedJob<float, true, true>>();
  persist_ctas_per_sm<PostFusedJob<float, false, false>>();
  persist_ctas_per_sm<PostFusedJob<float, true, false>>();
  persist_ctas_per_sm<PostFusedJob<double, false, true>>();
  persist_ctas_per_sm<PostFusedJob<double, true, true>>();
  persist_ctas_per_sm<PostFusedJob<double, false, false>>();
  persist_ctas_per_sm<PostFusedJob<double, true, false>>();
  persist_ctas_per_sm<PreFusedJob<float, true, PreSmall>>();
  persist_ctas_per_sm<PreFusedJob<float, false, PreSmall>>();
  persist_ctas_per_sm<PreFusedJob<double, true, PreSmall>>();
  persist_ctas_per_sm<PreFusedJob<double, false, PreSmall>>();
  persist_ctas_per_sm<PostFusedJob<float, false, true, PostSmall>>();
  persist_ctas_per_sm<PostFusedJob<float, true, true, PostSmall>>();
  persist_ctas_per_sm<PostFusedJob<float, false, false, PostSmall>>();
  persist_ctas_per_sm<PostFusedJob<float, true, false, PostSmall>>();
  persist_ctas_per_sm<PostFusedJob<double, false, true, PostSmall>>();
  persist_ctas_per_sm<PostFusedJob<double, true, true, PostSmall>>();
  persist_ctas_per_sm<PostFusedJob<double, false, false, PostSmall>>();
  persist_ctas_per_sm<PostFusedJob<double, true, false, PostSmall>>();
  persist_ctas_per_sm<CgDirF32Job<true>>();
  cg_update_wave<true>();
  cg_update_wave<false>();
  dir_wave_per_sm();
  return cudaGetLastError();
}

unsigned int read_device_fault() {
  unsigned int v = 0;
  cudaMemcpyFromSymbol(&v, g_sbp_fault, sizeof(v));
  return v;
}

// Elements 2t, 2t+1 per step: the packed form of the direction wave for
// even t, the scalar form of the staged direction tiles for odd t.
__global__ void k_pair_to_f64(const float* __restrict__ hi, const float* __restrict__ lo,
                              double* __restrict__ out, long long n) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; 2 * t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const long long k = 2 * t;
    if (k + 1 < n && (t & 1) == 0) {
      double rx, ry;
      float2 s;
      ff_neg_f64_2(make_float2(hi[k], hi[k + 1]), make_float2(lo[k], lo[k + 1]), rx, ry, s);
      out[k] = rx;
      out[k + 1] = ry;
    } else {
      out[k] = ff_neg_f64(hi[k], lo[k]);
      if (k + 1 < n) out[k + 1] = ff_neg_f64(hi[k + 1], lo[k + 1]);
    }
  }
}

cudaError_t launch_pair_to_f64(const float* hi, const float* lo, double* out, long long n,
                               cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  k_pair_to_f64<<<flat_grid(n, 4), kThreads, 0, s>>>(hi, lo, out, n);
  return cudaGetLastError();
}

cudaError_t set_copy_drop(int drop, unsigned polls) {
  const unsigned d = drop ? 1u : 0u;
  const unsigned p = polls ? polls : kWaitPollsDefault;
  cudaError_t e = cudaMemcpyToSymbol(g_sbp_drop_copy, &d, sizeof(d));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_sbp_wait_polls, &p, sizeof(p));
  return e;
}

unsigned int take_device_fault() {
  const unsigned int v = read_device_fault();
  if (v != 0u) {
    const unsigned int zero = 0u;
    cudaMemcpyToSymbol(g_sbp_fault, &zero, sizeof(zero));
  }
  return v;
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
// Coarse direct solve by fast diagonalisation, in FP64:
//   E = Vx [ (Vx^T B Vy) ./ D ] Vy^T
// as two launches of one kernel, each computing out(:, j) = M (in c_j)
// [.* dinv(:, j)] with one CTA per grid column j: pass 1 has in = B,
// c_j = Vy(:, j), M = Vx^T and scales by dinv; pass 2 has in = Y,
// c_j = Vy^T(:, j), M = Vx.  Every matrix is nc x nc column-major, so the
// threads of a row slice read consecutive addresses.  Sums run in a fixed
// order (four interleaved slices, then a fixed combine): deterministic.
// ---------------------------------------------------------------------------
constexpr int kFdSlices = kThreads / 64;
// Coarse sizes up to this stage the input grid and M in shared memory (one
// parallel load instead of a chain of dependent L2 reads per thread).
constexpr int kFdStageMaxN = 65;

__host__ __device__ constexpr size_t fd_smem_bytes(int nc, bool stage) {
  return ((size_t)(2 + kFdSlices) * nc + (stage ? 2 * (size_t)nc * nc : 0)) * sizeof(double);
}

struct FdArgs {
  const void* in;
  int in_ld;
  const double* C;
  const double* M;
  const double* dinv;
  void* out;
  int out_ld;
  int nc;
  const SolveState* st;
};

// Column j of one pass (one CTA).
template <typename Tin, typename Tout, bool STAGE>
__device__ __forceinline__ void fd_run(const FdArgs& a, int j) {
  if (a.st && a.st->done) return;
  const Grid<const Tin> in{static_cast<const Tin*>(a.in), a.in_ld};
  const Grid<Tout> out{static_cast<Tout*>(a.out), a.out_ld};
  const double* __restrict__ C = a.C;
  const double* __restrict__ M = a.M;
  const double* __restrict__ dinv = a.dinv;
  const int nc = a.nc;
  extern __shared__ double fd_sm[];
  double* c = fd_sm;                  // nc
  double* sv = c + nc;                // nc
  double* part = sv + nc;             // kFdSlices * nc
  double* is = part + kFdSlices * nc; // STAGE: the input grid, nc * nc (as Tin)
  double* ms = is + nc * nc;          // STAGE: M, nc * nc
  Tin* isr = reinterpret_cast<Tin*>(is);
  const int q = threadIdx.x >> 6, r = threadIdx.x & 63;
  for (int k = threadIdx.x; k < nc; k += kThreads) c[k] = C[(size_t)j * nc + k];
  if (STAGE) {
    // every element's copy in flight at once (cp.async), converted at use
    for (int k = threadIdx.x; k < nc * nc; k += kThreads) {
      const int jj = k / nc;
      cp_async_elem(isr + k, in.p + (size_t)jj * in.ld + (k - jj * nc));
      cp_async_elem(ms + k, M + k);
    }
    cp_async_wait_all();
  }
  __syncthreads();
  for (int i = r; i < nc; i += 64) {
    double a = 0.0;
#pragma unroll 4
    for (int k = q; k < nc; k += kFdSlices)
      a = fma(convert<double>(STAGE ? isr[k * nc + i] : in.at(i, k)), c[k], a);
    part[q * nc + i] = a;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nc; i += kThreads)
    sv[i] = (part[i] + part[nc + i]) + (part[2 * nc + i] + part[3 * nc + i]);
  __syncthreads();
  for (int i = r; i < nc; i += 64) {
    double a = 0.0;
#pragma unroll 4
    for (int k = q; k < nc; k += kFdSlices)
      a = fma(STAGE ? ms[k * nc + i] : __ldg(M + (size_t)k * nc + i), sv[k], a);
    part[q * nc + i] = a;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nc; i += kThreads) {
    double t = (part[i] + part[nc + i]) + (part[2 * nc + i] + part[3 * nc + i]);
    if (dinv) t *= __ldg(dinv + (size_t)j * nc + i);
    out.at(i, j) = convert<Tout>(t);
  }
}
template <typename Tin, typename Tout, bool STAGE>
__global__ void __launch_bounds__(kThreads) k_coarse_fd(const FdArgs a) {
  pdl_begin();
  fd_run<Tin, Tout, STAGE>(a, blockIdx.x);
}

template <typename Tin, typename Tout, bool STAGE>
__global__ void __launch_bounds__(kThreads)
    k_coarse_fd_batch(const unsigned char* __restrict__ blobs, int stride) {
  pdl_begin();
  const FdArgs a = *reinterpret_cast<const FdArgs*>(blobs + (size_t)blockIdx.y * (size_t)stride);
  fd_run<Tin, Tout, STAGE>(a, blockIdx.x);
}

// BatchLaunchFn: aux[0] = nc.
template <typename Tin, typename Tout, bool STAGE>
cudaError_t launch_fd_batch(const unsigned char* blobs, int stride, int count, const int* aux,
                            const BatchScratch&, cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  return launch_pdl(k_coarse_fd_batch<Tin, Tout, STAGE>, dim3(aux[0], count), dim3(kThreads),
                    fd_smem_bytes(aux[0], STAGE), s, blobs, stride);
}
static_assert(kFdSlices == 4, "the combine step sums four slices");

template <typename Tin, typename Tout>
cudaError_t launch_fd_pass(Grid<const Tin> in, const double* C, const double* M,
                           const double* dinv, Grid<Tout> out, int nc, const SolveState* st,
                           cudaStream_t s) {
  const FdArgs a{in.p, in.ld, C, M, dinv, out.p, out.ld, nc, st};
  const bool stage = nc <= kFdStageMaxN;
  if (recorder_slot())
    return stage ? record_launch(&launch_fd_batch<Tin, Tout, true>, a, nc)
                 : record_launch(&launch_fd_batch<Tin, Tout, false>, a, nc);
  if (stage)
    return launch_pdl(k_coarse_fd<Tin, Tout, true>, dim3(nc), dim3(kThreads),
                      fd_smem_bytes(nc, true), s, a);
  return launch_pdl(k_coarse_fd<Tin, Tout, false>, dim3(nc), dim3(kThreads),
                    fd_smem_bytes(nc, false), s, a);
}

template <typename Tin, typename Tout>
cudaError_t allow_fd_smem() {
  cudaError_t e = cudaFuncSetAttribute(k_coarse_fd<Tin, Tout, true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)fd_smem_bytes(kFdStageMaxN, true));
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_coarse_fd_batch<Tin, Tout, true>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)fd_smem_bytes(kFdStageMaxN, true));
  if (e != cudaSuccess) return e;
  // the unstaged pass of the largest coarse grids (1025: 49 KB)
  e = cudaFuncSetAttribute(k_coarse_fd<Tin, Tout, false>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)fd_smem_bytes(kCoarseMaxN, false));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_coarse_fd_batch<Tin, Tout, false>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)fd_smem_bytes(kCoarseMaxN, false));
}

// The staged coarse kernels need more than the default 48 KB of dynamic
// shared memory; set once, outside any stream capture.
cudaError_t prepare_coarse_kernels() {
  cudaError_t e = allow_fd_smem<float, double>();
  if (e == cudaSuccess) e = allow_fd_smem<double, float>();
  if (e == cudaSuccess) e = allow_fd_smem<double, double>();
  return e;
}

template <typename T>
cudaError_t launch_coarse_solve(const CoarseDev& f, Grid<const T> b, Grid<T> e,
                                const SolveState* st, cudaStream_t s) {
  const int nc = f.nc;
  cudaError_t err =
      launch_fd_pass<T, double>(b, f.Vy, f.VxT, f.dinv, Grid<double>{f.y, nc}, nc, st, s);
  if (err != cudaSuccess) return err;
  return launch_fd_pass<double, T>(Grid<const double>{f.y, nc}, f.VyT, f.Vx, nullptr, e, nc, st,
                                   s);
}

// ---------------------------------------------------------------------------
// Copy / convert and dot (pointwise, flat over contiguous n*n arrays).
// ---------------------------------------------------------------------------
template <typename Tin, typename Tout>
__global__ void __launch_bounds__(kThreads)
    k_copy(Grid<const Tin> in, Grid<Tout> out, int n) {
  // grid-stride over columns, threads over rows
  for (int j = blockIdx.x; j < n; j += gridDim.x)
    for (int i = threadIdx.x; i < n; i += kThreads) out.at(i, j) = convert<Tout>(__ldg(&in.at(i, j)));
}

template <typename Tin, typename Tout>
cudaError_t launch_copy(Grid<const Tin> in, Grid<Tout> out, int n, cudaStream_t s) {
  k_copy<Tin, Tout><<<std::min(n, 4096), kThreads, 0, s>>>(in, out, n);
  return cudaGetLastError();
}


// ---------------------------------------------------------------------------
// CSR SpMV y = A x (the assembled-operator comparator).  A CTA takes 256
// consecutive rows; their nonzeros are one contiguous segment, staged into
// shared memory with coalesced loads (at most kSpmvSeg entries, else each
// thread reads its row from global memory), then each thread sums its row,
// gathering x (the stencil's neighbours: L1/L2 hits).
// ---------------------------------------------------------------------------
constexpr int kSpmvSeg = 256 * 9;

__global__ void __launch_bounds__(kThreads)
    k_csr_spmv(long long nrows, const long long* __restrict__ row_ptr,
               const int* __restrict__ col, const double* __restrict__ val,
               const double* __restrict__ x, double* __restrict__ y) {
  __shared__ int scol[kSpmvSeg];
  __shared__ double sval[kSpmvSeg];
  for (long long r0 = (long long)blockIdx.x * kThreads; r0 < nrows;
       r0 += (long long)gridDim.x * kThreads) {
    const long long r1 = min(nrows, r0 + kThreads);
    const long long s0 = __ldg(row_ptr + r0), s1 = __ldg(row_ptr + r1);
    const int seg = (int)(s1 - s0);
    const bool staged = seg <= kSpmvSeg;
    if (staged)
      for (int k = threadIdx.x; k < seg; k += kThreads) {
        scol[k] = __ldg(col + s0 + k);
        sval[k] = __ldg(val + s0 + k);
      }
    __syncthreads();
    const long long r = r0 + threadIdx.x;
    if (r < r1) {
      const long long a = __ldg(row_ptr + r), b = __ldg(row_ptr + r + 1);
      double acc = 0.0;
      if (staged) {
        for (long long k = a - s0; k < b - s0; ++k) acc = fma(sval[k], __ldg(x + scol[k]), acc);
      } else {
        for (long long k = a; k < b; ++k) acc = fma(__ldg(val + k), __ldg(x + __ldg(col + k)), acc);
      }
      y[r] = acc;
    }
    __syncthreads();
  }
}

cudaError_t launch_csr_spmv(long long nrows, const long long* row_ptr, const int* col,
                            const double* val, const double* x, double* y, cudaStream_t s) {
  const long long blocks = (nrows + kThreads - 1) / kThreads;
  const int grid = (int)std::min<long long>(blocks, (long long)sm_count() * 8);
  k_csr_spmv<<<std::max(grid, 1), kThreads, 0, s>>>(nrows, row_ptr, col, val, x, y);
  return cudaGetLastError();
}

// g = H~ (u - ut) and *loss = 1/2 (u - ut)' H~ (u - ut), H~ = h^2 diag(w_i w_j)
// (w = 1/2 on the first and last index): the H-norm misfit of the adjoint
// configuration and its gradient.  Columns over CTAs, rows over threads;
// deterministic reduction.
__global__ void __launch_bounds__(kThreads)
    k_h_misfit(Grid<const double> u, Grid<const double> ut, Grid<double> g, int n, double h2,
               double* loss, ReduceBuf rb) {
  double acc = 0.0;
  for (int j = blockIdx.x; j < n; j += gridDim.x) {
    const double cj = (j == 0 || j == n - 1) ? 0.5 * h2 : h2;
    for (int i = threadIdx.x; i < n; i += kThreads) {
      const double d = __ldg(&u.at(i, j)) - __ldg(&ut.at(i, j));
      const double hd = ((i == 0 || i == n - 1) ? 0.5 * cj : cj) * d;
      if (g.p) g.at(i, j) = hd;
      acc = fma(hd, d, acc);
    }
  }
  grid_reduce(acc, rb, [&](double tot) {
    if (loss) *loss = 0.5 * tot;
  });
}

cudaError_t launch_h_misfit(Grid<const double> u, Grid<const double> ut, Grid<double> g, int n,
                            double* loss, ReduceBuf rb, cudaStream_t s) {
  const double h = 1.0 / (double)(n - 1);
  k_h_misfit<<<std::min(n, kFlatCtas), kThreads, 0, s>>>(u, ut, g, n, h * h, loss, rb);
  return cudaGetLastError();
}

__global__ void k_state_init(SolveState* st, int maxiter) {
  pdl_begin();
  SolveState z = {};
  z.maxiter = maxiter;
  *st = z;
}

struct StateInitArgs {
  SolveState* st;
  int maxiter;
};

__global__ void k_state_init_batch(const unsigned char* __restrict__ blobs, int stride) {
  pdl_begin();
  const StateInitArgs a =
      *reinterpret_cast<const StateInitArgs*>(blobs + (size_t)blockIdx.x * (size_t)stride);
  SolveState z = {};
  z.maxiter = a.maxiter;
  *a.st = z;
}

cudaError_t launch_state_init_batch(const unsigned char* blobs, int stride, int count, const int*,
                                    const BatchScratch&, cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  return launch_pdl(k_state_init_batch, dim3(count), dim3(1), 0, s, blobs, stride);
}

cudaError_t launch_state_init(SolveState* st, int maxiter, cudaStream_t s) {
  if (recorder_slot()) return record_launch(&launch_state_init_batch, StateInitArgs{st, maxiter}, 0);
  return launch_pdl(k_state_init, dim3(1), dim3(1), 0, s, st, maxiter);
}

// Grid copies between leading dimensions (the caller's layout <-> the
// padded one): plain copies when launched alone, one kernel per batch.
struct Copy2DArgs {
  double* dst;
  int dld;
  const double* src;
  int sld;
  int n;
};

__global__ void __launch_bounds__(kThreads)
    k_copy_grid_batch(const unsigned char* __restrict__ blobs, int stride) {
  pdl_begin();
  const Copy2DArgs a =
      *reinterpret_cast<const Copy2DArgs*>(blobs + (size_t)blockIdx.y * (size_t)stride);
  for (int j = blockIdx.x; j < a.n; j += gridDim.x)
    for (int i = threadIdx.x; i < a.n; i += kThreads)
      a.dst[(size_t)j * a.dld + i] = __ldg(a.src + (size_t)j * a.sld + i);
}

cudaError_t launch_copy_grid_batch(const unsigned char* blobs, int stride, int count,
                                   const int* aux, const BatchScratch&, cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  return launch_pdl(k_copy_grid_batch, dim3(std::min(aux[0], 1024), count), dim3(kThreads), 0, s,
                    blobs, stride);
}

__global__ void __launch_bounds__(kThreads) k_copy_grid(const Copy2DArgs a) {
  pdl_begin();
  for (int j = blockIdx.x; j < a.n; j += gridDim.x)
    for (int i = threadIdx.x; i < a.n; i += kThreads)
      a.dst[(size_t)j * a.dld + i] = __ldg(a.src + (size_t)j * a.sld + i);
}

// Grid copy between leading dimensions by the SMs: at N = 4097 a pitched
// device-to-device cudaMemcpy2DAsync (copy engine) took 138 us, this kernel
// 56 us.
cudaError_t copy_grid(double* dst, int dld, const double* src, int sld, int n, cudaStream_t s) {
  if (recorder_slot())
    return record_launch(&launch_copy_grid_batch, Copy2DArgs{dst, dld, src, sld, n}, n);
  if (n <= 0) return cudaSuccess;
  return launch_pdl(k_copy_grid, dim3(std::min(n, 4096)), dim3(kThreads), 0, s,
                    Copy2DArgs{dst, dld, src, sld, n});
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
  template cudaError_t launch_coarse_solve<T>(const CoarseDev&, Grid<const T>, Grid<T>,         \
                                              const SolveState*, cudaStream_t);

SBP_INST_T(double)
SBP_INST_T(float)
#undef SBP_INST_T

#define SBP_INST_OP(T)                                                                         \
  template cudaError_t launch_pre_fused<T>(const Operand&, Grid<T>, Grid<T>, int, int, int,      \
                                           double, int, const SolveState*, cudaStream_t,         \
                                           cudaStream_t, cudaEvent_t, cudaEvent_t);              \
  template cudaError_t launch_post_fused<T>(const Operand&, const Operand&, const Operand&,      \
                                            Grid<T>, int, int, int, double, int, SolveState*,    \
                                            ReduceBuf, cudaStream_t, cudaStream_t, cudaEvent_t,  \
                                            cudaEvent_t);                                        \
  template cudaError_t launch_smooth_op<T>(int, int, const Operand&, const Operand&,             \
                                           const Operand&, Grid<T>, int, int, double, int,       \
                                           SolveState*, ReduceBuf, cudaStream_t);                \
  template cudaError_t launch_resrestrict_op<T>(const Operand*, const Operand&, Grid<T>, int, int, \
                                                const SolveState*, cudaStream_t);
SBP_INST_OP(double)
SBP_INST_OP(float)
#undef SBP_INST_OP
template cudaError_t launch_residual_op<double>(const Operand&, const Operand&, Grid<double>,
                                                Grid<float>, int, int, SolveState*, double*, double,
                                                double, int, double*, ReduceBuf, cudaStream_t,
                                                Grid<double>);
template cudaError_t launch_cg_dir_op<double, double>(const Operand&, const Operand&, Grid<double>,
                                                      Grid<double>, int, int, SolveState*,
                                                      ReduceBuf, cudaStream_t);
template cudaError_t launch_cg_dir_op<double, float>(const Operand&, const Operand&, Grid<double>,
                                                     Grid<double>, int, int, SolveState*,
                                                     ReduceBuf, cudaStream_t);
template cudaError_t launch_cg_dir<double, double>(Grid<const double>, Grid<const double>,
                                                   Grid<double>, Grid<double>, int, int,
                                                   SolveState*, ReduceBuf, cudaStream_t);
template cudaError_t launch_cg_dir<double, float>(Grid<const float>, Grid<const double>,
                                                  Grid<double>, Grid<double>, int, int,
                                                  SolveState*, ReduceBuf, cudaStream_t);
template cudaError_t launch_cg_update<double>(Grid<double>, Grid<double>, Grid<const double>,
                                              Grid<const double>, Grid<float>, int, int,
                                              SolveState*, double*, ReduceBuf, cudaStream_t,
                                              const float*);
template cudaError_t launch_copy<double, double>(Grid<const double>, Grid<double>, int,
                                                 cudaStream_t);
template cudaError_t launch_copy<double, float>(Grid<const double>, Grid<float>, int,
                                                cudaStream_t);
template cudaError_t launch_copy<float, double>(Grid<const float>, Grid<double>, int,
                                                cudaStream_t);
template cudaError_t launch_copy<float, float>(Grid<const float>, Grid<float>, int,
                                               cudaStream_t);

// ---------------------------------------------------------------------------
// Allocation-free operator apply + dot (sbp_apply_dot_f64_noalloc).
//
// The regular sbp_apply_dot_f64 takes its per-CTA partial sums from
// stream-ordered scratch (cudaMallocAsync).  This variant keeps that scratch
// in the file-scope array below instead, so a call never reaches the CUDA
// allocator.  The array is loaded with the library and stays resident on
// every GPU that uses it until the process exits.
// ---------------------------------------------------------------------------
namespace {

// Partial-sum slots: one per CTA of the launch.  A persistent launch uses
// SMs x resident CTAs (760 for this kernel on a 152-SM GB300), so 1024 slots
// cover it; a launch needing more is rejected.
constexpr int kNoAllocSlots = 1024;
constexpr size_t kNoAllocTicketOffset = kNoAllocSlots * sizeof(double);
constexpr size_t kNoAllocBytes = kNoAllocTicketOffset + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Device address of g_noalloc_scratch, resolved once per device.  Host code
// must not pass the symbol itself to a kernel: on the host it names a
// stand-in, not device memory.
std::mutex g_noalloc_mu;
void* g_noalloc_addr[64] = {nullptr};

cudaError_t noalloc_scratch(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_noalloc_addr[dev] = p;
  }
  *out = g_noalloc_addr[dev];
  return cudaSuccess;
}

}  // namespace

// Returns 0, or -1 (arguments), -2 (CUDA error, kept in *err), -6 (scratch
// too small).
int apply_dot_f64_noalloc(const double* u, double* out, int n, int sign, double* dot,
                          cudaStream_t s, cudaError_t* err) {
  *err = cudaSuccess;
  if (!u || !out || !dot || n < 3 || (sign != 1 && sign != -1)) return -1;
  void* scratch = nullptr;
  if ((*err = noalloc_scratch(&scratch)) != cudaSuccess) return -2;
  using Job = ApplyJob<double, true, false>;
  const dim3 g = tile_grid(n);
  const int total = (int)(g.x * g.y);
  const int cap = std::min(kMaxPersistCtas, sm_count() * persist_ctas_per_sm<Job>());
  const int grid = std::max(1, std::min(total, cap));
  if (grid > kNoAllocSlots) return -6;
  unsigned char* base = static_cast<unsigned char*>(scratch);
  ReduceBuf rb{reinterpret_cast<double*>(base),
               reinterpret_cast<unsigned*>(base + kNoAllocTicketOffset)};
  // the ticket must start at zero; the partial slots are overwritten by
  // every launch before they are read
  if ((*err = cudaMemsetAsync(rb.ticket, 0, sizeof(unsigned), s)) != cudaSuccess) return -2;
  const Operand uo = raw_operand(u, n, n);
  const Job job{dev_operand<double>(uo), Grid<double>{out, n}, n, (int)g.x, total, sign, rb, dot};
  k_persist<Job><<<grid, kThreads, 2 * Job::kStage + Job::kScratch + 128, s>>>(job);
  *err = cudaGetLastError();
  return *err == cudaSuccess ? 0 : -2;
}

// ---------------------------------------------------------------------------
// FP64 FMA issue rate of this GPU (roofline denominator of the FP64-bound
// kernels): eight independent FMA chains per thread, one full wave of CTAs.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_fp64_fma_rate(double* sink, int iters, double m) {
  double a[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) a[c] = 1.0 + 1e-3 * (double)(threadIdx.x + 37 * c);
  const double add = 1e-9;
  for (int k = 0; k < iters; ++k) {
#pragma unroll
    for (int c = 0; c < 8; ++c) a[c] = fma(a[c], m, add);
  }
  double t = 0.0;
#pragma unroll
  for (int c = 0; c < 8; ++c) t += a[c];
  if (t == -1.0) sink[blockIdx.x] = t;  // never true: keeps the chains live
}

cudaError_t measure_fp64_fma_rate(double* gfma_per_s, cudaStream_t s) {
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fp64_fma_rate, kThreads, 0);
  if (e != cudaSuccess) return e;
  const int grid = sm_count() * std::max(1, per_sm);
  const int iters = 2048;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if ((e = cudaEventCreate(&e0)) != cudaSuccess) return e;
  if ((e = cudaEventCreate(&e1)) != cudaSuccess) {
    cudaEventDestroy(e0);
    return e;
  }
  float best = 0.f;
  for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {
    cudaEventRecord(e0, s);
    k_fp64_fma_rate<<<grid, kThreads, 0, s>>>(nullptr, iters, 0.9999999);
    cudaEventRecord(e1, s);
    e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess && rep > 0 && (best == 0.f || ms < best)) best = ms;
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return e;
  const double fmas = (double)grid * kThreads * 8.0 * iters;
  *gfma_per_s = fmas / (best * 1e-3) / 1e9;
  return cudaSuccess;
}

}  // namespace sbp

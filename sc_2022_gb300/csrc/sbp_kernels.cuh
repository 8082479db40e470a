// Kernel templates for the SBP-SAT Poisson path.  Included by the kernel
// translation units (sbp_kernels.cu, sbp_high_order.cu); the launch wrappers
// declared in sbp_launch.h are the interface.
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

#include <cuda.h>

#include <utility>

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

// ---------------------------------------------------------------------------
// Asynchronous staging.  cp.async copies global -> shared without passing
// through registers, so every element a CTA stages is in flight at once
// (the staged tile of one CTA is ~20 KB; with several CTAs per SM this keeps
// well over the ~40 KB per SM that HBM latency x bandwidth requires).  It
// needs only element alignment, so it works on the caller's column-major
// arrays whatever their leading dimension (n = 2^k + 1 is odd, so columns
// are not 16-byte aligned and TMA tensor copies could not address them).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cp_async_elem(double* sdst, const double* gsrc) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_elem(float* sdst, const float* gsrc) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gsrc) : "memory");
}
// Wait for this thread's copies; a __syncthreads() must follow before other
// threads read the staged data.
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;\n" ::: "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
// Wait until at most N of this thread's committed groups are still pending.
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// ---------------------------------------------------------------------------
// TMA (cp.async.bulk.tensor) and mbarrier helpers.  One thread issues a 2D
// tensor copy of a whole staged box; the copy reports its bytes to an
// mbarrier that the CTA waits on.  Out-of-range box elements are zero-filled
// by the hardware, which replaces every bounds check of the staging.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
// Order this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy (TMA) writes to the same buffer.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];\n" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned phase) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0u;
}

// Set (never cleared by the kernels) when a bounded wait gives up; read by
// the host through read_device_fault().  Internal linkage: each translation
// unit that includes this header has its own copy; the kernels with bounded
// waits all live in sbp_kernels.cu, whose copy read_device_fault() reads.
static __device__ unsigned int g_sbp_fault = 0u;

// try_wait polls of a bounded wait before it gives up, and the failure
// test's switch (sbp_test_drop_copy): while set, CTA 0 of every persistent
// launch declares its first tile's bytes but issues no copy, so that wait
// runs out.  Set only through sbp_test_drop_copy (this translation unit's
// copies, like g_sbp_fault).
constexpr unsigned kWaitPollsDefault = 1u << 22;
static __device__ unsigned int g_sbp_wait_polls = kWaitPollsDefault;
static __device__ unsigned int g_sbp_drop_copy = 0u;

// Bounded wait on an mbarrier phase.  try_wait suspends for a bounded,
// hardware-defined time per call, so the default limit is seconds: far beyond
// any legitimate TMA latency, short enough that a lost copy cannot hang the
// GPU.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned phase) {
  const unsigned polls = *const_cast<volatile unsigned*>(&g_sbp_wait_polls);
  for (unsigned it = 0; it < polls; ++it)
    if (mbar_try_wait(bar, phase)) return true;
  atomicOr(&g_sbp_fault, 1u);
  return false;
}

// ---------------------------------------------------------------------------
// Programmatic dependent launch.  Kernels of the solver are launched with the
// programmatic-serialization attribute: the next kernel in the stream (or
// graph) may be scheduled as soon as every CTA of this one has started, and
// waits in pdl_begin() until this one has finished and its writes are
// visible.  The launch latency of the dependent kernel thus overlaps this
// kernel's execution.  pdl_begin() must precede every global-memory access.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void pdl_begin() {
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
}

// Per-launch timing for diagnostics (sbp_solver_profile): while a LaunchTimer
// is installed on the calling host thread, launch_pdl brackets every launch
// with a pair of CUDA events on the launching stream.
struct LaunchTimer;
LaunchTimer*& timer_slot();
void timer_mark(LaunchTimer* t, const void* fn, cudaStream_t s, bool after);

// Launch with programmatic dependent launch enabled (see pdl_begin()).
template <typename... KArgs, typename... Args>
static cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                              cudaStream_t s, Args&&... args) {
  if (LaunchTimer* t = timer_slot()) {
    timer_mark(t, reinterpret_cast<const void*>(kernel), s, false);
    timer_slot() = nullptr;
    const cudaError_t e = launch_pdl(kernel, grid, block, smem, s, std::forward<Args>(args)...);
    timer_slot() = t;
    timer_mark(t, reinterpret_cast<const void*>(kernel), s, true);
    return e;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// ---------------------------------------------------------------------------
// float <-> double with integer instructions only.  On GB300 the FP64 pipe
// issues about two lanes per clock per SM, and the hardware conversions run
// there too; the solver's conversions (r -> FP32 for the V-cycle, z -> FP64
// for the Krylov direction) are pure bit moves on the integer pipe instead.
// Float denormals map to signed zero and double values below the float
// normal range flush to signed zero (both far below any residual the solver
// produces); Inf/NaN map to Inf/NaN (double -> float: to Inf).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double f32_to_f64(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned sign = u & 0x80000000u;
  const unsigned e = (u >> 23) & 0xFFu;
  const unsigned m = u & 0x7FFFFFu;
  unsigned hi = sign;
  if (e == 0xFFu)
    hi |= 0x7FF00000u | (m >> 3);
  else if (e != 0u)
    hi |= ((e + 896u) << 20) | (m >> 3);
  const unsigned lo = (e == 0u) ? 0u : (m << 29);
  return __hiloint2double((int)hi, (int)lo);
}
__device__ __forceinline__ float f64_to_f32(double d) {
  const unsigned hi = (unsigned)__double2hiint(d);
  const unsigned lo = (unsigned)__double2loint(d);
  const unsigned sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7FFu) - 896;           // float biased exponent
  const unsigned m = ((hi & 0xFFFFFu) << 3) | (lo >> 29);  // top 23 mantissa bits
  const unsigned rnd = (lo >> 28) & 1u;                    // round half away
  unsigned f;
  if (e <= 0)
    f = sign;
  else if (e >= 255)
    f = sign | 0x7F800000u;
  else
    f = sign | (((unsigned)e << 23) + m + rnd);            // a carry rounds up the exponent
  return __uint_as_float(f);
}
template <typename To, typename From>
__device__ __forceinline__ To convert(From v) { return (To)v; }
template <>
__device__ __forceinline__ double convert<double, float>(float v) { return f32_to_f64(v); }
template <>
__device__ __forceinline__ float convert<float, double>(double v) { return f64_to_f32(v); }

// ---------------------------------------------------------------------------
// The 5-point sum S = (w + e + m + p) - 4c of FP64 values on the integer pipe.
// Every operand's 53-bit significand is aligned to the largest exponent in a
// signed 64-bit integer with 7 guard bits (|sum| < 5 * 2^60), the five terms
// are added exactly, and the sum is rounded once to nearest-even.  Bits
// shifted out during alignment are dropped (each term rounds toward -inf:
// error below 5 units of 2^-7 ulp of the largest term; the FP64 evaluation
// order errs by up to ~2 ulp of it).
// GB300 issues about 2 FP64 lanes per clock per SM but 64x more integer
// lanes, so this keeps FP64 stencils off the FP64 pipe.  Returns false (and
// leaves s unset) for Inf/NaN operands or a result outside the normal range;
// the caller then uses FP64 arithmetic.
// ---------------------------------------------------------------------------
struct ExactTerm {
  long long v;   // signed significand, aligned later
  int e;         // effective biased exponent (>= 1)
};
__device__ __forceinline__ bool exact_term(double x, int escale, ExactTerm& t) {
  const unsigned hi = (unsigned)__double2hiint(x);
  const unsigned lo = (unsigned)__double2loint(x);
  const int ex = (int)((hi >> 20) & 0x7FFu);
  const unsigned long long m =
      ((unsigned long long)((hi & 0xFFFFFu) | (ex ? 0x100000u : 0u)) << 32) | lo;
  t.v = (hi >> 31) ? -(long long)(m << 7) : (long long)(m << 7);
  t.e = (ex ? ex : 1) + escale;
  return ex != 0x7FF;
}
__device__ __forceinline__ long long exact_align(const ExactTerm& t, int E) {
  const int d = E - t.e;
  return d >= 63 ? 0LL : (t.v >> d);   // arithmetic shift: rounds toward -inf
}
__device__ __forceinline__ bool exact_stencil5(double c, double w, double e, double m, double p,
                                               double& s) {
  ExactTerm tc, tw, te, tm, tp;
  bool ok = exact_term(c, 2, tc);   // 4 c: exponent + 2, exact
  ok &= exact_term(w, 0, tw);
  ok &= exact_term(e, 0, te);
  ok &= exact_term(m, 0, tm);
  ok &= exact_term(p, 0, tp);
  const int E = max(max(max(tw.e, te.e), max(tm.e, tp.e)), tc.e);
  const long long S = (exact_align(tw, E) + exact_align(te, E)) +
                      (exact_align(tm, E) + exact_align(tp, E)) - exact_align(tc, E);
  // value = S * 2^(E - 1082); round |S| to 53 bits
  const unsigned long long a = S < 0 ? (unsigned long long)(-S) : (unsigned long long)S;
  if (a == 0ULL) {
    s = 0.0;
    return ok;
  }
  const int msb = 63 - __clzll((long long)a);
  int k = msb - 52;
  unsigned long long mm;
  if (k > 0) {
    mm = a >> k;
    const unsigned long long rem = a & ((1ULL << k) - 1ULL);
    const unsigned long long half = 1ULL << (k - 1);
    if (rem > half || (rem == half && (mm & 1ULL))) ++mm;
    if (mm >> 53) {
      mm >>= 1;
      ++k;
    }
  } else {
    mm = a << (-k);
  }
  const int be = k + E - 7;
  if (be <= 0 || be >= 0x7FF) return false;
  const unsigned hi = (S < 0 ? 0x80000000u : 0u) | ((unsigned)be << 20) |
                      ((unsigned)(mm >> 32) & 0xFFFFFu);
  s = __hiloint2double((int)hi, (int)(unsigned)mm);
  return ok;
}

// ---------------------------------------------------------------------------
// Error-free FP32 arithmetic.  two_sum gives s + e == a + b exactly (Knuth).
// stencil_ff returns the 5-point stencil (uw + ue) + (um + up) - 4 u0 of FP32
// values as an unevaluated float pair hi + lo whose error is below 2^-45 of
// the largest term: FP64-grade accuracy from the FP32 pipe, which GB300
// issues 64x faster than FP64.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ void stencil_ff(float uw, float ue, float um, float up, float u0,
                                           float& hi, float& lo) {
  float a, ea, b, eb, c, ec, d, ed;
  two_sum(uw, ue, a, ea);
  two_sum(um, up, b, eb);
  two_sum(a, b, c, ec);
  two_sum(c, -4.0f * u0, d, ed);
  hi = d;
  lo = (ea + eb) + (ec + ed);
}

// -(hi + lo) of two floats rounded to nearest-even in FP64, with an FP64
// instruction only in rare cases.  two_sum gives s + e == hi + lo with |e| at
// most half an FP32 ulp of s, so the sum stays in the binade of s (unless s
// is a power of two and e points down) and is s plus k FP64 ulps of s, k =
// rn(e * 2^(179 - E)) with E the biased exponent of s (|k| < 2^29): an exact
// power-of-two scaling and one float -> int conversion, whose ties-to-even
// is the parity of the FP64 result.  Adding k to the bit pattern of (double)s
// gives the FP64 sum.  |s| < 2^-75, zero, non-finite s and the binade
// crossing take the FP64 add, which returns the same bits.
__device__ __forceinline__ double ff_neg_f64(float hi, float lo) {
  float s, e;
  two_sum(hi, lo, s, e);
  const unsigned u = __float_as_uint(s);
  const unsigned E = (u >> 23) & 0xFFu;
  const unsigned neg = u & 0x80000000u;
  if (E >= 52u && E != 255u &&
      ((u & 0x7FFFFFu) != 0u || ((neg ^ __float_as_uint(e)) & 0x80000000u) == 0u || e == 0.0f)) {
    const unsigned long long ds = ((unsigned long long)neg << 32) |
                                  ((unsigned long long)(E + 896u) << 52) |
                                  ((unsigned long long)(u & 0x7FFFFFu) << 29);
    const int k = __float2int_rn(e * __uint_as_float((306u - E) << 23));   // e / ulp64(s)
    const long long step = neg ? -(long long)k : (long long)k;
    return __longlong_as_double(
        (long long)((ds + (unsigned long long)step) ^ 0x8000000000000000ull));
  }
  return -((double)hi + (double)lo);
}

// ---------------------------------------------------------------------------
// FF: an unevaluated float pair hi + lo with the arithmetic negA needs, for
// evaluating the SAT stencil of FP32 values on the FP32 pipe.  Sums use
// two_sum and products the FMA split, so results carry about 48 bits.  The
// constructor from double takes the stencil's constants, all exact in FP32.
// ---------------------------------------------------------------------------
struct FF {
  float hi, lo;
  __device__ FF() {}
  __device__ FF(float h, float l) : hi(h), lo(l) {}
  __device__ explicit FF(double c) : hi((float)c), lo(0.0f) {}
};
__device__ __forceinline__ FF ff_norm(float s, float e) {
  const float h = s + e;
  return FF(h, e - (h - s));
}
__device__ __forceinline__ FF operator+(FF a, FF b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  return ff_norm(s, e + (a.lo + b.lo));
}
__device__ __forceinline__ FF operator-(FF a, FF b) { return a + FF(-b.hi, -b.lo); }
__device__ __forceinline__ FF operator*(FF a, FF b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return ff_norm(p, e);
}
__device__ __forceinline__ FF& operator+=(FF& a, FF b) {
  a = a + b;
  return a;
}

// ---------------------------------------------------------------------------
// Dot-product accumulators.  FP64 data: an FP64 FMA per term.  FP32 data:
// each product is split exactly into p + e (FMA) and summed with a
// compensated (TwoSum) float-float accumulator, converted to FP64 once per
// thread -- FP64-quality accumulation without FP64 instructions per term.
// ---------------------------------------------------------------------------
template <typename T>
struct DotAcc;
template <>
struct DotAcc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add_prod(double a, double b) { s = fma(a, b, s); }
  __device__ __forceinline__ double value() const { return s; }
};
template <>
struct DotAcc<float> {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add_prod(float a, float b) {
    const float p = a * b;
    const float e = fmaf(a, b, -p);
    const float s = hi + p;
    const float bb = s - hi;
    const float err = (hi - (s - bb)) + (p - bb);
    hi = s;
    lo += err + e;
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// ---------------------------------------------------------------------------
// Packed FP32 pairs: Blackwell issues one instruction for both lanes of a
// float2 (f32x2 add/mul/fma), each lane rounded exactly as the scalar
// operation.  The register waves hold two grid rows per thread, so their
// per-row arithmetic pairs up; issue, not the FP32 rate, bounds them.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// a - b: b * -1 is exact, so the FMA rounds once, as the subtraction does
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
  return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
}
__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2& s, float2& e) {
  s = add2(a, b);
  const float2 bb = sub2(s, a);
  e = add2(sub2(a, sub2(s, bb)), sub2(b, bb));
}
// stencil_ff on two rows at once: w/e the i-1/i+1 neighbours, m/p the
// j-1/j+1 neighbours, c the centre; the same operations per lane.
__device__ __forceinline__ void stencil_ff2(float2 w, float2 e, float2 m, float2 p, float2 c,
                                            float2& hi, float2& lo) {
  float2 a, ea, b, eb, cc, ec, d, ed;
  two_sum2(w, e, a, ea);
  two_sum2(m, p, b, eb);
  two_sum2(a, b, cc, ec);
  two_sum2(cc, mul2(make_float2(-4.f, -4.f), c), d, ed);
  hi = d;
  lo = add2(add2(ea, eb), add2(ec, ed));
}
// ff_neg_f64 for two pairs (the two-sum and the scaling packed); s returns
// fl32(hi + lo) per lane
__device__ __forceinline__ void ff_neg_f64_2(float2 hi, float2 lo, double& rx, double& ry,
                                             float2& s) {
  float2 e;
  two_sum2(hi, lo, s, e);
  const unsigned ux = __float_as_uint(s.x), uy = __float_as_uint(s.y);
  const unsigned Ex = (ux >> 23) & 0xFFu, Ey = (uy >> 23) & 0xFFu;
  // 2^(179 - E) as a float; E outside [52, 254] takes the FP64 add below
  const float2 sc = make_float2(__uint_as_float((306u - min(max(Ex, 52u), 254u)) << 23),
                                __uint_as_float((306u - min(max(Ey, 52u), 254u)) << 23));
  const float2 kf = mul2(e, sc);
  auto one = [](float hv, float lv, float sv, float ev, unsigned u, unsigned E, float k) {
    const unsigned neg = u & 0x80000000u;
    if (E >= 52u && E != 255u &&
        ((u & 0x7FFFFFu) != 0u || ((neg ^ __float_as_uint(ev)) & 0x80000000u) == 0u ||
         ev == 0.0f)) {
      const unsigned long long ds = ((unsigned long long)neg << 32) |
                                    ((unsigned long long)(E + 896u) << 52) |
                                    ((unsigned long long)(u & 0x7FFFFFu) << 29);
      const int kk = __float2int_rn(k);
      const long long step = neg ? -(long long)kk : (long long)kk;
      return __longlong_as_double(
          (long long)((ds + (unsigned long long)step) ^ 0x8000000000000000ull));
    }
    return -((double)hv + (double)lv);
  };
  rx = one(hi.x, lo.x, s.x, e.x, ux, Ex, kf.x);
  ry = one(hi.y, lo.y, s.y, e.y, uy, Ey, kf.y);
}

// Compensated dot accumulation of two rows at once (one float pair per
// row, added together at the end).
struct DotAcc2 {
  float2 hi = make_float2(0.f, 0.f), lo = make_float2(0.f, 0.f);
  __device__ __forceinline__ void add_prod(float2 a, float2 b) {
    const float2 p = mul2(a, b);
    const float2 e = fma2(a, b, make_float2(-p.x, -p.y));
    float2 s, err;
    two_sum2(hi, p, s, err);
    hi = s;
    lo = add2(lo, add2(err, e));
  }
  __device__ __forceinline__ double value() const {
    return ((double)hi.x + (double)lo.x) + ((double)hi.y + (double)lo.y);
  }
};

// Stage the raw values of g over [i0, i0+ei) x [j0, j0+ej) into s with row
// pitch P; points outside the n x n domain are zero-filled.
template <int P, typename T>
__device__ __forceinline__ void stage_async(T* s, Grid<const T> g, int i0, int j0, int ei, int ej,
                                            int n) {
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  for (int c = w; c < ej; c += kWarps) {
    const int j = j0 + c;
    const bool jok = (j >= 0 && j < n);
    for (int r = lane; r < ei; r += 32) {
      const int i = i0 + r;
      if (jok && i >= 0 && i < n)
        cp_async_elem(&s[c * P + r], &g.at(i, j));
      else
        s[c * P + r] = T(0);
    }
  }
}

// Stage a tile plus its halo (pitch Tile::SI).
template <int TI, int TJ, typename T>
__device__ __forceinline__ void stage_tile_async(T* s, const Tile<TI, TJ>& t, Grid<const T> g,
                                                 int n) {
  stage_async<Tile<TI, TJ>::SI>(s, g, t.i_lo - 1, t.j_lo - t.hl, t.i_hi - t.i_lo + 2,
                                t.j_hi - t.j_lo + t.hl + t.hr, n);
}

// Stage only the tile's own points (pitch TI + 1), for pointwise operands.
template <int TI, int TJ, typename T>
__device__ __forceinline__ void stage_interior_async(T* s, const Tile<TI, TJ>& t,
                                                     Grid<const T> g, int n) {
  stage_async<TI + 1>(s, g, t.i_lo, t.j_lo, t.i_hi - t.i_lo, t.j_hi - t.j_lo, n);
}

// Apply fn(i, j, value&) to every staged point of a tile (halo included).
template <int TI, int TJ, typename T, typename Fn>
__device__ __forceinline__ void transform_staged(T* s, const Tile<TI, TJ>& t, int n, Fn&& fn) {
  constexpr int SI = Tile<TI, TJ>::SI;
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const int ei = t.i_hi - t.i_lo + 2;
  const int ej = t.j_hi - t.j_lo + t.hl + t.hr;
  for (int c = w; c < ej; c += kWarps) {
    const int j = t.j_lo - t.hl + c;
    if (j < 0 || j >= n) continue;
    for (int r = lane; r < ei; r += 32) {
      const int i = t.i_lo - 1 + r;
      if (i >= 0 && i < n) fn(i, j, s[c * SI + r]);
    }
  }
}

// Visit every output point of the tile: fn(i, j, SAcc centred on (i, j),
// k) with k the point's index in an interior-staged array (pitch TI + 1).
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
      fn(t.i_lo + r, t.j_lo + c, acc, c * (TI + 1) + r);
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

// The reduction over the CTAs cta = 0 .. nb-1 that share `red` (a batched
// launch reduces each problem over blockIdx.x alone).
template <typename Fin>
__device__ __forceinline__ void grid_reduce_n(double v, const ReduceBuf& red, Fin&& fin,
                                              unsigned cta, unsigned nb) {
  __shared__ bool is_last;
  const double bs = block_sum(v);
  if (threadIdx.x == 0) {
    red.partials[cta] = bs;
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

template <typename Fin>
__device__ __forceinline__ void grid_reduce(double v, const ReduceBuf& red, Fin&& fin) {
  grid_reduce_n(v, red, fin, blockIdx.y * gridDim.x + blockIdx.x, gridDim.x * gridDim.y);
}

__device__ __forceinline__ bool finite_d(double x) { return isfinite(x); }

// ---------------------------------------------------------------------------
// Multigrid transfer helpers.
// ---------------------------------------------------------------------------
// Bilinear prolongation of the coarse correction e (nc x nc) to fine point
// (i, j) from global memory (prolongation_2D_kernel, matrix_free_mg_cg.jl:41-67).
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

// The same from a staged coarse region with origin (I0, J0) and pitch EP.
template <int EP, typename T>
__device__ __forceinline__ T prolong_smem(const T* se, int I0, int J0, int i, int j) {
  const T* q = se + ((j >> 1) - J0) * EP + ((i >> 1) - I0);
  const bool oi = i & 1, oj = j & 1;
  T v = q[0];
  if (oi) v += q[1];
  if (oj) {
    v += q[EP];
    if (oi) v += q[EP + 1];
  }
  const T scale = (oi && oj) ? T(0.25) : ((oi || oj) ? T(0.5) : T(1));
  return v * scale;
}

}  // namespace sbp

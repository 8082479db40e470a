// C ABI of libsbpmg: solver handles (multigrid hierarchy, workspace, CUDA
// graphs of one Krylov iteration) and the single-grid entry points.
#include <cuda_runtime.h>
#include <cxxabi.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/sbpmg.h"
#include "sbp_coarse.h"
#include "sbp_host.h"
#include "sbp_launch.h"

using namespace sbp;

namespace {
thread_local std::string g_last_error;
}  // namespace

namespace sbp {

void set_last_error(const std::string& msg) { g_last_error = msg; }

int fail_cuda(cudaError_t e, const char* what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  return SBP_ERR_CUDA;
}

int check_device_fault(const char* what) {
  if (take_device_fault() == 0u) return SBP_OK;
  g_last_error = std::string(what) +
                 ": a kernel's bounded wait on an asynchronous copy gave up; results are void";
  return SBP_ERR_TIMEOUT;
}

int finish_result(const SolveState& fs, sbp_result* res) {
  int status;
  if (fs.done == kDoneConverged)
    status = SBP_OK;
  else if (fs.done == kDoneBreakdown)
    status = SBP_ERR_BREAKDOWN;
  else
    status = SBP_ERR_MAXITER;
  if (res) {
    res->iters = fs.iter;
    res->status = status;
    res->initial_norm = std::sqrt(fs.rr0);
    res->final_norm = std::sqrt(fs.rr);
    res->threshold = std::sqrt(fs.thresh2);
  }
  return status;
}

}  // namespace sbp

namespace {

bool valid_mg_n(int n) {
  if (n < 3) return false;
  const int m = n - 1;
  return (m & (m - 1)) == 0;
}

template <typename T>
Grid<T> grid(void* p, int ld) {
  return Grid<T>{static_cast<T*>(p), ld};
}
template <typename T>
Grid<const T> cgrid(const void* p, int ld) {
  return Grid<const T>{static_cast<const T*>(p), ld};
}

struct Level {
  int n = 0;
  int ld = 0;               // padded leading dimension (16-byte aligned columns)
  void* b = nullptr;        // right-hand side (level 0: the solver's r or r_lo)
  void* v[2] = {nullptr, nullptr};
  Operand ob, ov[2];        // TMA operands of b and v
  int out = 0;              // buffer holding the V-cycle result
  bool own_b = false;
  cudaEvent_t fork = nullptr, join = nullptr;   // boundary branch of the pre-smoothing
  cudaEvent_t pfork = nullptr, pjoin = nullptr; // and of the post-smoothing
};

}  // namespace

struct sbp_solver {
  int n = 0;
  int device = 0;
  bool mg = false;
  sbp_options opts{};
  size_t esize = 8;                 // element size of the V-cycle levels
  std::vector<Level> levels;
  CoarseDev coarse{};               // fast-diagonalisation factors of the last level
  // Krylov vectors (FP64, padded leading dimension ld; padding stays zero)
  int ld = 0;
  double* x = nullptr;              // the iterate (the caller's x is copied in and out)
  double* r = nullptr;
  double* p[2] = {nullptr, nullptr};
  double* Ap = nullptr;
  float* r_lo = nullptr;            // FP32 copy of r (mixed precision)
  Operand ox, orr, op[2], oap, orlo;
  float* p32[2] = {nullptr, nullptr};   // FP32 direction of mixed MGCG (ping-pong)
  Operand op32[2];
  SolveState* st = nullptr;
  SolveState* st_host = nullptr;    // pinned, 2 slots
  double* norms = nullptr;
  int norms_cap = 0;
  ReduceBuf rb{nullptr, nullptr};
  long long dev_bytes = 0;
  std::vector<void*> allocs;
  cudaStream_t cap = nullptr;       // private stream for graph capture
  cudaStream_t aux = nullptr;       // forked branch (boundary tiles of the wave levels)
  cudaEvent_t ev[2] = {nullptr, nullptr};
  // cached iteration graphs: [kind][parity]; kind 0 = MGCG, 1 = CG
  cudaGraphExec_t iter_exec[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  bool iter_valid[2] = {false, false};
  int iter_key_sign[2] = {0, 0};
  int iter_key_maxiter[2] = {0, 0};
  // kernel launches: per captured iteration graph, and of the last solve
  long long launches_per_iter[2] = {0, 0};
  long long last_launches = 0;
  long long counting = 0;          // launches enqueued since the counter reset
};

namespace {

int dalloc(sbp_solver* s, void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    g_last_error = std::string("cudaMalloc: ") + cudaGetErrorString(e);
    return SBP_ERR_NOMEM;
  }
  s->allocs.push_back(*p);
  s->dev_bytes += (long long)bytes;
  return SBP_OK;
}

void destroy_graphs(sbp_solver* s) {
  for (auto& k : s->iter_exec)
    for (auto& g : k)
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
  s->iter_valid[0] = s->iter_valid[1] = false;
}

// ---------------------------------------------------------------------------
// V-cycle schedule.  Level l < last:
//   pre:  F = first sweep from zero, fused with the second sweep when
//         nu_pre >= 2; remaining sweeps ping-pong between v[0] and v[1];
//   f_{l+1} = R (b - A v)            (fused residual + restriction)
//   recurse
//   post: first pass reads v + P e (prolongation folded into the sweep);
//         remaining sweeps ping-pong.  On level 0 the last pass also reduces
//         b.z into the Krylov state when `dot` is set.
// Last level: v = A^{-1} b by fast diagonalisation (FP64, two launches).
// ---------------------------------------------------------------------------
// Temporal blocking (one fused pre-smoothing and one fused post-smoothing
// kernel per level) for FP32 levels: their sweeps are memory-bound, so
// recomputing halos in shared memory is cheap.  FP64 levels are bound by the
// FP64 pipe and keep the one-sweep-per-pass schedule, which does no redundant
// halo arithmetic.
// Levels up to this size use the fused passes (all FP32 levels at present).
constexpr int kFuseMaxN = 1 << 30;

template <typename T>
bool use_fused(const sbp_solver* s, int n) {
  const sbp_options& o = s->opts;
  return sizeof(T) == 4 && n <= kFuseMaxN && o.nu_pre >= 1 && o.nu_pre <= 3 && o.nu_post >= 0 &&
         o.nu_post <= 3;
}

template <typename T>
cudaError_t enqueue_vcycle(sbp_solver* s, size_t l, bool dot, SolveState* st, cudaStream_t q) {
  Level& L = s->levels[l];
  const sbp_options& o = s->opts;
  const int n = L.n;
  const double om = o.omega;
  const int sm = o.smoother;
  const Operand none;
  cudaError_t e;
  if (l + 1 == s->levels.size()) {
    L.out = 0;
    e = launch_coarse_solve<T>(s->coarse, cgrid<T>(L.b, L.ld), grid<T>(L.v[0], L.ld), st, q);
    if (e != cudaSuccess) return e;
    if (dot && l == 0) {
      // single-level hierarchy: still reduce b.z for the Krylov state
      e = launch_smooth_op<T>(kFieldPlain, kEpiStore, L.ov[0], none, L.ob, grid<T>(L.v[1], L.ld),
                              n, sm, om, 1, st, s->rb, q);
      L.out = 1;
    }
    return e;
  }
  if (use_fused<T>(s, n)) {
    Level& C = s->levels[l + 1];
    e = launch_pre_fused<T>(L.ob, grid<T>(L.v[0], L.ld), grid<T>(C.b, C.ld), n, o.nu_pre, sm, om,
                            o.restriction, st, q, s->aux, L.fork, L.join);
    if (e != cudaSuccess) return e;
    e = enqueue_vcycle<T>(s, l + 1, false, st, q);
    if (e != cudaSuccess) return e;
    e = launch_post_fused<T>(L.ov[0], C.ov[C.out], L.ob, grid<T>(L.v[1], L.ld), n, o.nu_post, sm,
                             om, dot ? 1 : 0, st, s->rb, q, s->aux, L.pfork, L.pjoin);
    L.out = 1;
    return e;
  }
  int k;
  e = launch_smooth_op<T>(kFieldZero, o.nu_pre >= 2 ? kEpiSweep : kEpiStore, none, none, L.ob,
                          grid<T>(L.v[0], L.ld), n, sm, om, 0, st, s->rb, q);
  k = o.nu_pre >= 2 ? 2 : 1;
  if (e != cudaSuccess) return e;
  int cur = 0;
  for (; k < o.nu_pre; ++k) {
    e = launch_smooth_op<T>(kFieldPlain, kEpiSweep, L.ov[cur], none, L.ob,
                            grid<T>(L.v[1 - cur], L.ld), n, sm, om, 0, st, s->rb, q);
    if (e != cudaSuccess) return e;
    cur = 1 - cur;
  }
  Level& C = s->levels[l + 1];
  e = launch_resrestrict_op<T>(&L.ov[cur], L.ob, grid<T>(C.b, C.ld), n, o.restriction, st, q);
  if (e != cudaSuccess) return e;
  e = enqueue_vcycle<T>(s, l + 1, false, st, q);
  if (e != cudaSuccess) return e;
  const Operand& ec = C.ov[C.out];
  const int npost = std::max(1, o.nu_post);
  for (int pass = 0; pass < npost; ++pass) {
    const bool last = (pass == npost - 1);
    const int field = (pass == 0) ? kFieldProlong : kFieldPlain;
    const int epi = (o.nu_post == 0) ? kEpiStore : kEpiSweep;
    e = launch_smooth_op<T>(field, epi, L.ov[cur], ec, L.ob, grid<T>(L.v[1 - cur], L.ld), n, sm,
                            om, (dot && last) ? 1 : 0, st, s->rb, q);
    if (e != cudaSuccess) return e;
    cur = 1 - cur;
  }
  L.out = cur;
  return cudaSuccess;
}

// Kernel launches of one V-cycle (mirrors enqueue_vcycle).
long long vcycle_launches(const sbp_solver* s, bool dot) {
  const sbp_options& o = s->opts;
  long long c = 0;
  const size_t nl = s->levels.size();
  const bool mixed = (s->opts.precision == SBP_PREC_MIXED);
  for (size_t l = 0; l + 1 < nl; ++l) {
    const int n = s->levels[l].n;
    if (mixed ? use_fused<float>(s, n) : use_fused<double>(s, n)) {
      // fused pre-smoothing (one or two kernels), fused post-smoothing
      c += pre_fused_launches(n, o.nu_pre, mixed) + post_fused_launches(n, o.nu_post, mixed);
      continue;
    }
    c += (o.nu_pre >= 2) ? 1 + (o.nu_pre - 2) : 1;
    c += 1;                               // residual + restriction
    c += std::max(1, o.nu_post);          // prolongation + post sweeps
  }
  c += 2;                                 // coarse solve (two passes)
  if (dot && nl == 1) c += 1;
  return c;
}

// Kernel launches of one Krylov iteration (mirrors enqueue_iteration).
long long iteration_launches(const sbp_solver* s, int kind) {
  return 2 + (kind == 0 ? vcycle_launches(s, true) : 0);
}

cudaError_t enqueue_vcycle_any(sbp_solver* s, bool dot, SolveState* st, cudaStream_t q) {
  if (s->opts.precision == SBP_PREC_MIXED) return enqueue_vcycle<float>(s, 0, dot, st, q);
  return enqueue_vcycle<double>(s, 0, dot, st, q);
}

// V-cycle output on level 0 (valid after a schedule has been enqueued once:
// the schedule is static).
const void* vcycle_out(sbp_solver* s) {
  Level& L = s->levels[0];
  return L.v[L.out];
}
const Operand& vcycle_out_op(sbp_solver* s) {
  Level& L = s->levels[0];
  return L.ov[L.out];
}

// One Krylov iteration: direction + operator + alpha, update + convergence,
// then (MGCG) the V-cycle with the r.z / beta reduction.
cudaError_t enqueue_iteration(sbp_solver* s, int kind, int parity, int sign, cudaStream_t q) {
  const int n = s->n, ld = s->ld;
  double* pnew = s->p[1 - parity];
  cudaError_t e;
  const bool mixed = (kind == 0 && s->opts.precision == SBP_PREC_MIXED);
  if (kind == 0) {
    if (mixed)
      // FP32 direction p~ and Ap = A p~ (exact) in one pass
      e = launch_cg_dir_f32(vcycle_out_op(s), s->op32[parity], grid<float>(s->p32[1 - parity], ld),
                            grid<double>(s->Ap, ld), n, s->st, s->rb, q);
    else
      e = launch_cg_dir_op<double, double>(vcycle_out_op(s), s->op[parity], grid<double>(pnew, ld),
                                           grid<double>(s->Ap, ld), n, +1, s->st, s->rb, q);
  } else {
    e = launch_cg_dir_op<double, double>(s->orr, s->op[parity], grid<double>(pnew, ld),
                                         grid<double>(s->Ap, ld), n, sign, s->st, s->rb, q);
  }
  if (e != cudaSuccess) return e;
  e = launch_cg_update<double>(grid<double>(s->x, ld), grid<double>(s->r, ld),
                               cgrid<double>(pnew, ld), cgrid<double>(s->Ap, ld),
                               Grid<float>{mixed ? s->r_lo : nullptr, ld}, n, kind == 1 ? 1 : 0,
                               s->st, s->norms, s->rb, q, mixed ? s->p32[1 - parity] : nullptr);
  if (e != cudaSuccess) return e;
  if (kind == 0) e = enqueue_vcycle_any(s, true, s->st, q);
  return e;
}

int ensure_norms(sbp_solver* s, int maxiter) {
  if (maxiter + 1 <= s->norms_cap) return SBP_OK;
  // grow (old buffer stays in allocs until destroy; norms are small)
  void* p = nullptr;
  const int cap = std::max(maxiter + 1, 2 * s->norms_cap);
  int rc = dalloc(s, &p, (size_t)cap * sizeof(double));
  if (rc) return rc;
  s->norms = static_cast<double*>(p);
  s->norms_cap = cap;
  destroy_graphs(s);  // graphs captured the old pointer
  return SBP_OK;
}

int capture_iteration(sbp_solver* s, int kind, int sign) {
  for (int par = 0; par < 2; ++par) {
    cudaGraph_t g = nullptr;
    SBP_CUDA(cudaStreamBeginCapture(s->cap, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = enqueue_iteration(s, kind, par, sign, s->cap);
    cudaError_t e2 = cudaStreamEndCapture(s->cap, &g);
    if (e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return fail_cuda(e, "enqueue_iteration (capture)");
    }
    if (e2 != cudaSuccess) return fail_cuda(e2, "cudaStreamEndCapture");
    if (s->iter_exec[kind][par]) cudaGraphExecDestroy(s->iter_exec[kind][par]);
    s->iter_exec[kind][par] = nullptr;
    e = cudaGraphInstantiate(&s->iter_exec[kind][par], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail_cuda(e, "cudaGraphInstantiate");
  }
  s->iter_valid[kind] = true;
  s->iter_key_sign[kind] = sign;
  s->launches_per_iter[kind] = iteration_launches(s, kind);
  return SBP_OK;
}

// Argument checks and per-solve buffers of a Krylov solve.
int krylov_prepare(sbp_solver* s, int kind, const double* b, double* x, double abstol,
                   double reltol, int maxiter) {
  if (!s || !b || !x) return SBP_ERR_ARGS;
  if (maxiter < 0) return SBP_ERR_ARGS;
  if (kind == 0 && !s->mg) return SBP_ERR_UNSUPPORTED;
  if (abstol <= 0.0 && reltol <= 0.0) return SBP_ERR_ARGS;
  SBP_CUDA(cudaSetDevice(s->device));
  return ensure_norms(s, maxiter);
}

// Set-up of a solve: the caller's x into the padded iterate, state,
// r0 = b - sign*A*x0, and (MGCG) z0 = M r0 with r.z.
cudaError_t enqueue_setup(sbp_solver* s, int kind, const double* b, double* x, int sign,
                          double abstol, double reltol, int maxiter, cudaStream_t q) {
  const int n = s->n, ld = s->ld;
  const bool mixed = (kind == 0 && s->opts.precision == SBP_PREC_MIXED);
  cudaError_t e = launch_state_init(s->st, maxiter, q);
  // b and the caller's x are read in place; the residual pass also writes x
  // into the padded iterate
  Operand ob, ox;
  ob.p = b;
  ob.n = n;
  ob.ld = n;
  ob.tma = false;
  ox.p = x;
  ox.n = n;
  ox.ld = n;
  ox.tma = false;
  if (e == cudaSuccess)
    e = launch_residual_op<double>(ox, ob, grid<double>(s->r, ld),
                                   Grid<float>{mixed ? s->r_lo : nullptr, ld}, n, sign, s->st,
                                   s->norms, abstol, reltol, kind == 1 ? 1 : 0, nullptr, s->rb, q,
                                   grid<double>(s->x, ld));
  if (e == cudaSuccess && kind == 0) e = enqueue_vcycle_any(s, true, s->st, q);
  return e;
}

// Status and result fields from a final solver state.
// Shared driver of sbp_mgcg_solve (kind 0) and sbp_cg_solve (kind 1).
int run_krylov(sbp_solver* s, int kind, const double* b, double* x, int sign, double abstol,
               double reltol, int maxiter, sbp_result* res, double* norms_out, int norms_cap,
               cudaStream_t q) {
  int rc = krylov_prepare(s, kind, b, x, abstol, reltol, maxiter);
  if (rc) return rc;
  const int n = s->n, ld = s->ld;
  SBP_CUDA(enqueue_setup(s, kind, b, x, sign, abstol, reltol, maxiter, q));
  if (!s->iter_valid[kind] || s->iter_key_sign[kind] != sign || !s->iter_exec[kind][0]) {
    rc = capture_iteration(s, kind, sign);
    if (rc) return rc;
  }
  // Iterate: keep one iteration queued ahead of the one being checked.
  long long launches = 2 + (kind == 0 ? vcycle_launches(s, true) : 0);   // set-up + V-cycle
  int k = 0;
  bool finished = false;
  if (maxiter == 0) finished = true;
  while (!finished) {
    SBP_CUDA(cudaGraphLaunch(s->iter_exec[kind][k & 1], q));
    launches += s->launches_per_iter[kind];
    SBP_CUDA(cudaMemcpyAsync(&s->st_host[k & 1], s->st, sizeof(SolveState),
                             cudaMemcpyDeviceToHost, q));
    SBP_CUDA(cudaEventRecord(s->ev[k & 1], q));
    if (k >= 1) {
      SBP_CUDA(cudaEventSynchronize(s->ev[(k - 1) & 1]));
      if (s->st_host[(k - 1) & 1].done) finished = true;
    }
    ++k;
    if (k > maxiter + 2) finished = true;  // safety net; kernels stop at maxiter
  }
  SBP_CUDA(copy_grid(x, n, s->x, ld, n, q));
  SBP_CUDA(cudaMemcpyAsync(&s->st_host[0], s->st, sizeof(SolveState), cudaMemcpyDeviceToHost, q));
  SBP_CUDA(cudaStreamSynchronize(q));
  if (const int fr = check_device_fault("solve")) return fr;
  const SolveState fs = s->st_host[0];
  s->last_launches = launches;
  if (norms_out && norms_cap > 0) {
    const int cnt = std::min(norms_cap, fs.iter + 1);
    SBP_CUDA(cudaMemcpy(norms_out, s->norms, (size_t)cnt * sizeof(double),
                        cudaMemcpyDeviceToHost));
  }
  return finish_result(fs, res);
}

// Stream-ordered scratch for the single-grid reducing entry points.
struct TempReduce {
  ReduceBuf rb{nullptr, nullptr};
  double* out = nullptr;
  void* base = nullptr;
  cudaStream_t q = nullptr;
  int alloc(int n, cudaStream_t stream) {
    q = stream;
    const size_t parts = (size_t)max_reduce_ctas(n);
    const size_t bytes = parts * sizeof(double) + 2 * sizeof(double);
    SBP_CUDA(cudaMallocAsync(&base, bytes, q));
    rb.partials = static_cast<double*>(base);
    out = rb.partials + parts;
    rb.ticket = reinterpret_cast<unsigned*>(out + 1);
    SBP_CUDA(cudaMemsetAsync(rb.ticket, 0, sizeof(unsigned), q));
    return SBP_OK;
  }
  ~TempReduce() {
    if (base) cudaFreeAsync(base, q);
  }
};

int smooth_sweeps(double* v, double* tmp, const double* b, int n, int iters, double omega,
                  int smoother, cudaStream_t q) {
  if (!v || !tmp || !b || n < 3 || iters < 0) return SBP_ERR_ARGS;
  double* bufs[2] = {v, tmp};
  int cur = 0;
  ReduceBuf none{nullptr, nullptr};
  for (int k = 0; k < iters; ++k) {
    SBP_CUDA(launch_smooth<double>(kFieldPlain, kEpiSweep, cgrid<double>(bufs[cur], n),
                                   Grid<const double>{nullptr, 0}, cgrid<double>(b, n),
                                   grid<double>(bufs[1 - cur], n), n, smoother, omega, 0,
                                   nullptr, none, q));
    cur = 1 - cur;
  }
  // leave the result in both buffers, as the reference's in-place loop does
  SBP_CUDA(cudaMemcpyAsync(bufs[1 - cur], bufs[cur], (size_t)n * n * sizeof(double),
                           cudaMemcpyDeviceToDevice, q));
  return SBP_OK;
}

}  // namespace

extern "C" {

int sbp_version(void) { return 100; }

const char* sbp_last_error(void) { return g_last_error.c_str(); }

int sbp_coarse_inverse_host(int nc, double* out, long long cap) {
  if (!out || !valid_mg_n(nc) || nc > 129) return SBP_ERR_ARGS;
  const long long N = (long long)nc * nc;
  if (cap < N * N) return SBP_ERR_ARGS;
  try {
    auto X = coarse_inverse(nc);
    std::memcpy(out, X->data(), (size_t)(N * N) * sizeof(double));
  } catch (const std::exception& ex) {
    g_last_error = ex.what();
    return SBP_ERR_CUDA;
  }
  return SBP_OK;
}

int sbp_coarse_inverse_order_host(int nc, int p, double* out, long long cap) {
  if (!out || nc > 129 || (p != 2 && p != 4 && p != 6)) return SBP_ERR_ARGS;
  if (nc < (p == 2 ? 3 : ho_min_points(p))) return SBP_ERR_ARGS;
  const long long N = (long long)nc * nc;
  if (cap < N * N) return SBP_ERR_ARGS;
  try {
    auto X = coarse_inverse(nc, p);
    std::memcpy(out, X->data(), (size_t)(N * N) * sizeof(double));
  } catch (const std::exception& ex) {
    g_last_error = ex.what();
    return SBP_ERR_ARGS;
  }
  return SBP_OK;
}

const char* sbp_status_string(int status) {
  switch (status) {
    case SBP_OK: return "ok";
    case SBP_ERR_ARGS: return "invalid argument";
    case SBP_ERR_CUDA: return g_last_error.empty() ? "CUDA error" : g_last_error.c_str();
    case SBP_ERR_NOMEM: return "out of memory";
    case SBP_ERR_MAXITER: return "maximum iterations reached";
    case SBP_ERR_BREAKDOWN: return "breakdown (p'Ap == 0 or non-finite residual)";
    case SBP_ERR_UNSUPPORTED: return "unsupported option combination";
    case SBP_ERR_TIMEOUT:
      return "a kernel's bounded wait on an asynchronous copy gave up (results void)";
    default: return "unknown status";
  }
}

void sbp_options_default(sbp_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->smoother = SBP_SMOOTH_JACOBI;
  o->omega = 2.0 / 3.0;
  o->nu_pre = 3;
  o->nu_post = 3;
  o->restriction = SBP_RESTRICT_GALERKIN;
  o->coarse_n = 65;
  o->precision = SBP_PREC_FP64;
}

void sbp_options_reference_two_level(sbp_options* o, int n) {
  if (!o) return;
  sbp_options_default(o);
  o->smoother = SBP_SMOOTH_RICHARDSON;
  o->omega = 0.15;
  o->nu_pre = 3;
  o->nu_post = 3;
  o->restriction = SBP_RESTRICT_NORMAL;
  o->coarse_n = (n + 1) / 2;
}

int sbp_apply_f64(const double* u, double* out, int n, int sign, void* stream) {
  if (!u || !out || n < 3 || (sign != 1 && sign != -1)) return SBP_ERR_ARGS;
  ReduceBuf none{nullptr, nullptr};
  SBP_CUDA(launch_apply<double>(cgrid<double>(u, n), grid<double>(out, n), n, sign, none, nullptr,
                                (cudaStream_t)stream));
  return SBP_OK;
}

int sbp_apply_f32(const float* u, float* out, int n, int sign, void* stream) {
  if (!u || !out || n < 3 || (sign != 1 && sign != -1)) return SBP_ERR_ARGS;
  ReduceBuf none{nullptr, nullptr};
  SBP_CUDA(launch_apply<float>(cgrid<float>(u, n), grid<float>(out, n), n, sign, none, nullptr,
                               (cudaStream_t)stream));
  return SBP_OK;
}

int sbp_apply_dot_f64(const double* u, double* out, int n, int sign, double* dot, void* stream) {
  if (!u || !out || !dot || n < 3 || (sign != 1 && sign != -1)) return SBP_ERR_ARGS;
  cudaStream_t q = (cudaStream_t)stream;
  TempReduce t;
  int rc = t.alloc(n, q);
  if (rc) return rc;
  SBP_CUDA(launch_apply<double>(cgrid<double>(u, n), grid<double>(out, n), n, sign, t.rb, dot, q));
  return SBP_OK;
}

int sbp_apply_dot_f64_noalloc(const double* u, double* out, int n, int sign, double* dot,
                              void* stream) {
  cudaError_t err = cudaSuccess;
  const int rc = apply_dot_f64_noalloc(u, out, n, sign, dot, (cudaStream_t)stream, &err);
  if (rc == SBP_ERR_CUDA) g_last_error = cudaGetErrorString(err);
  if (rc == SBP_ERR_UNSUPPORTED)
    g_last_error = "sbp_apply_dot_f64_noalloc: the launch needs more than the 1024 partial-sum "
                   "slots of the static scratch";
  return rc;
}

int sbp_residual_norm_f64(const double* x, const double* b, int n, int sign, double* norm_host,
                          void* stream) {
  if (!x || !b || !norm_host || n < 3 || (sign != 1 && sign != -1)) return SBP_ERR_ARGS;
  cudaStream_t q = (cudaStream_t)stream;
  TempReduce t;
  int rc = t.alloc(n, q);
  if (rc) return rc;
  double* r = nullptr;
  SBP_CUDA(cudaMallocAsync((void**)&r, (size_t)n * n * sizeof(double), q));
  cudaError_t e = launch_residual<double>(cgrid<double>(x, n), cgrid<double>(b, n),
                                          grid<double>(r, n), Grid<float>{nullptr, n}, n, sign,
                                          nullptr, nullptr, 0.0, 0.0, 0, t.out, t.rb, q);
  double v = 0.0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&v, t.out, sizeof(double), cudaMemcpyDeviceToHost, q);
  cudaFreeAsync(r, q);
  if (e == cudaSuccess) e = cudaStreamSynchronize(q);
  if (e != cudaSuccess) return fail_cuda(e, "sbp_residual_norm_f64");
  if (const int fr = check_device_fault("sbp_residual_norm_f64")) return fr;
  *norm_host = std::sqrt(v);
  return SBP_OK;
}

int sbp_restrict_f64(const double* fine, double* coarse, int n_fine, int kind, void* stream) {
  if (!fine || !coarse || n_fine < 3 || (n_fine % 2) == 0 || kind < 0 || kind > 2)
    return SBP_ERR_ARGS;
  const int nc = (n_fine + 1) / 2;
  SBP_CUDA(launch_resrestrict<double>(Grid<const double>{nullptr, 0}, cgrid<double>(fine, n_fine),
                                      grid<double>(coarse, nc), n_fine, kind, nullptr,
                                      (cudaStream_t)stream));
  return SBP_OK;
}

int sbp_prolong_f64(const double* coarse, double* fine, int n_coarse, int accumulate,
                    void* stream) {
  if (!coarse || !fine || n_coarse < 2) return SBP_ERR_ARGS;
  SBP_CUDA(launch_prolong<double>(cgrid<double>(coarse, n_coarse),
                                  grid<double>(fine, 2 * n_coarse - 1), n_coarse, accumulate,
                                  nullptr, (cudaStream_t)stream));
  return SBP_OK;
}

int sbp_richardson_f64(double* v, double* tmp, const double* b, int n, int iters, double omega,
                       void* stream) {
  return smooth_sweeps(v, tmp, b, n, iters, omega, SBP_SMOOTH_RICHARDSON, (cudaStream_t)stream);
}

int sbp_jacobi_f64(double* v, double* tmp, const double* b, int n, int iters, double omega,
                   void* stream) {
  return smooth_sweeps(v, tmp, b, n, iters, omega, SBP_SMOOTH_JACOBI, (cudaStream_t)stream);
}

int sbp_rhs_f64(const double* f, const double* gW, const double* gE, const double* gS,
                const double* gN, double* b, int n, double fsign, void* stream) {
  if (!f || !gW || !gE || !gS || !gN || !b || n < 3) return SBP_ERR_ARGS;
  SBP_CUDA(launch_rhs(cgrid<double>(f, n), gW, gE, gS, gN, grid<double>(b, n), n, fsign,
                      (cudaStream_t)stream));
  return SBP_OK;
}

int sbp_rhs_adjoint_f64(const double* lam, double* df, double* dgW, double* dgE, double* dgS,
                        double* dgN, int n, double fsign, void* stream) {
  if (!lam || n < 3) return SBP_ERR_ARGS;
  SBP_CUDA(launch_rhs_adjoint(cgrid<double>(lam, n), grid<double>(df, n), dgW, dgE, dgS, dgN, n,
                              fsign, (cudaStream_t)stream));
  return SBP_OK;
}

int sbp_csr_spmv_f64(long long nrows, const long long* row_ptr, const int* col,
                     const double* val, const double* x, double* y, void* stream) {
  if (nrows < 1 || !row_ptr || !col || !val || !x || !y) return SBP_ERR_ARGS;
  SBP_CUDA(launch_csr_spmv(nrows, row_ptr, col, val, x, y, (cudaStream_t)stream));
  return SBP_OK;
}

int sbp_h_misfit_f64(const double* u, const double* ut, double* g, int n, double* loss,
                     void* stream) {
  if (!u || !ut || n < 3 || (!g && !loss)) return SBP_ERR_ARGS;
  cudaStream_t q = (cudaStream_t)stream;
  TempReduce t;
  int rc = t.alloc(n, q);
  if (rc) return rc;
  SBP_CUDA(launch_h_misfit(cgrid<double>(u, n), cgrid<double>(ut, n), grid<double>(g, n), n,
                           loss, t.rb, q));
  return SBP_OK;
}

int sbp_solver_create(sbp_solver** out, int n, const sbp_options* opts) {
  if (!out) return SBP_ERR_ARGS;
  *out = nullptr;
  if (n < 3) return SBP_ERR_ARGS;
  sbp_solver* s = new (std::nothrow) sbp_solver();
  if (!s) return SBP_ERR_NOMEM;
  std::unique_ptr<sbp_solver, int (*)(sbp_solver*)> guard(s, sbp_solver_destroy);
  s->n = n;
  SBP_CUDA(cudaGetDevice(&s->device));
  SBP_CUDA(prepare_kernels());
  if (opts) {
    s->mg = true;
    s->opts = *opts;
    sbp_options& o = s->opts;
    if (o.omega <= 0.0) o.omega = (o.smoother == SBP_SMOOTH_JACOBI) ? 2.0 / 3.0 : 0.15;
    if (!valid_mg_n(n) || !valid_mg_n(o.coarse_n) || o.coarse_n > n) return SBP_ERR_ARGS;
    if (o.coarse_n > kCoarseMaxN) return SBP_ERR_UNSUPPORTED;  // limit of the coarse factors
    if (o.nu_pre < 1 || o.nu_post < 0 || o.nu_pre > 64 || o.nu_post > 64) return SBP_ERR_UNSUPPORTED;
    if (o.smoother != SBP_SMOOTH_JACOBI && o.smoother != SBP_SMOOTH_RICHARDSON) return SBP_ERR_ARGS;
    if (o.restriction < 0 || o.restriction > 2) return SBP_ERR_ARGS;
    if (o.precision != SBP_PREC_FP64 && o.precision != SBP_PREC_MIXED) return SBP_ERR_ARGS;
    s->esize = (o.precision == SBP_PREC_MIXED) ? sizeof(float) : sizeof(double);
  }
  s->ld = padded_ld(n);
  const size_t nn = (size_t)s->ld * n;
  int rc;
  void* p;
  rc = dalloc(s, &p, nn * 8); if (rc) return rc; s->x = (double*)p;
  rc = dalloc(s, &p, nn * 8); if (rc) return rc; s->r = (double*)p;
  rc = dalloc(s, &p, nn * 8); if (rc) return rc; s->p[0] = (double*)p;
  rc = dalloc(s, &p, nn * 8); if (rc) return rc; s->p[1] = (double*)p;
  rc = dalloc(s, &p, nn * 8); if (rc) return rc; s->Ap = (double*)p;
  for (double* a : {s->x, s->r, s->p[0], s->p[1], s->Ap}) SBP_CUDA(cudaMemset(a, 0, nn * 8));
  make_operand(s->ox, s->x, n, s->ld, true);
  make_operand(s->orr, s->r, n, s->ld, true);
  make_operand(s->op[0], s->p[0], n, s->ld, true);
  make_operand(s->op[1], s->p[1], n, s->ld, true);
  make_operand(s->oap, s->Ap, n, s->ld, true);
  rc = dalloc(s, &p, sizeof(SolveState)); if (rc) return rc; s->st = (SolveState*)p;
  const size_t parts = (size_t)max_reduce_ctas(n) + 64;
  rc = dalloc(s, &p, parts * sizeof(double)); if (rc) return rc; s->rb.partials = (double*)p;
  rc = dalloc(s, &p, 64); if (rc) return rc; s->rb.ticket = (unsigned*)p;
  SBP_CUDA(cudaMemset(s->rb.ticket, 0, 64));
  SBP_CUDA(cudaMallocHost((void**)&s->st_host, 2 * sizeof(SolveState)));
  SBP_CUDA(cudaStreamCreateWithFlags(&s->cap, cudaStreamNonBlocking));
  SBP_CUDA(cudaEventCreateWithFlags(&s->ev[0], cudaEventDisableTiming));
  SBP_CUDA(cudaEventCreateWithFlags(&s->ev[1], cudaEventDisableTiming));
  rc = ensure_norms(s, 1024);
  if (rc) return rc;
  if (s->mg) {
    const bool mixed = s->opts.precision == SBP_PREC_MIXED;
    const bool f64 = !mixed;
    if (mixed) {
      rc = dalloc(s, &p, nn * sizeof(float)); if (rc) return rc; s->r_lo = (float*)p;
      SBP_CUDA(cudaMemset(s->r_lo, 0, nn * sizeof(float)));
      make_operand(s->orlo, s->r_lo, n, s->ld, false);
      for (int k = 0; k < 2; ++k) {
        rc = dalloc(s, &p, nn * sizeof(float)); if (rc) return rc; s->p32[k] = (float*)p;
        SBP_CUDA(cudaMemset(s->p32[k], 0, nn * sizeof(float)));
        make_operand(s->op32[k], s->p32[k], n, s->ld, false);
      }
    }
    int m = n;
    while (true) {
      Level L;
      L.n = m;
      L.ld = padded_ld(m);
      const size_t bytes = (size_t)L.ld * m * s->esize;
      if (s->levels.empty()) {
        L.b = mixed ? (void*)s->r_lo : (void*)s->r;
      } else {
        rc = dalloc(s, &L.b, bytes); if (rc) return rc;
        SBP_CUDA(cudaMemset(L.b, 0, bytes));
        L.own_b = true;
      }
      rc = dalloc(s, &L.v[0], bytes); if (rc) return rc;
      rc = dalloc(s, &L.v[1], bytes); if (rc) return rc;
      SBP_CUDA(cudaMemset(L.v[0], 0, bytes));
      SBP_CUDA(cudaMemset(L.v[1], 0, bytes));
      make_operand(L.ob, L.b, m, L.ld, f64);
      make_operand(L.ov[0], L.v[0], m, L.ld, f64);
      make_operand(L.ov[1], L.v[1], m, L.ld, f64);
      s->levels.push_back(L);
      if (mixed && pre_fused_launches(m, s->opts.nu_pre, true) == 2) {
        Level& B = s->levels.back();
        SBP_CUDA(cudaEventCreateWithFlags(&B.fork, cudaEventDisableTiming));
        SBP_CUDA(cudaEventCreateWithFlags(&B.join, cudaEventDisableTiming));
        if (!s->aux) SBP_CUDA(cudaStreamCreateWithFlags(&s->aux, cudaStreamNonBlocking));
      }
      if (mixed && post_fused_launches(m, s->opts.nu_post, true) == 2) {
        Level& B = s->levels.back();
        SBP_CUDA(cudaEventCreateWithFlags(&B.pfork, cudaEventDisableTiming));
        SBP_CUDA(cudaEventCreateWithFlags(&B.pjoin, cudaEventDisableTiming));
        if (!s->aux) SBP_CUDA(cudaStreamCreateWithFlags(&s->aux, cudaStreamNonBlocking));
      }
      if (m == s->opts.coarse_n) break;
      m = (m + 1) / 2;
    }
    const int nc = s->opts.coarse_n;
    std::shared_ptr<const CoarseFactors> F;
    try {
      F = coarse_factors(nc);
    } catch (const std::exception& ex) {
      g_last_error = ex.what();
      return SBP_ERR_CUDA;
    }
    const size_t mb = (size_t)nc * nc * sizeof(double);
    const std::vector<double>* src[5] = {&F->Vx, &F->VxT, &F->Vy, &F->VyT, &F->dinv};
    double* dst[6];
    for (int k = 0; k < 6; ++k) {
      rc = dalloc(s, &p, mb); if (rc) return rc;
      dst[k] = (double*)p;
      if (k < 5) SBP_CUDA(cudaMemcpy(dst[k], src[k]->data(), mb, cudaMemcpyHostToDevice));
    }
    s->coarse = CoarseDev{dst[0], dst[1], dst[2], dst[3], dst[4], dst[5], nc};
  }
  SBP_CUDA(cudaDeviceSynchronize());
  guard.release();
  *out = s;
  return SBP_OK;
}

int sbp_solver_destroy(sbp_solver* s) {
  if (!s) return SBP_OK;
  cudaSetDevice(s->device);
  destroy_graphs(s);
  for (void* p : s->allocs) cudaFree(p);
  if (s->st_host) cudaFreeHost(s->st_host);
  if (s->cap) cudaStreamDestroy(s->cap);
  if (s->aux) cudaStreamDestroy(s->aux);
  for (auto& e : s->ev)
    if (e) cudaEventDestroy(e);
  for (Level& L : s->levels) {
    for (cudaEvent_t ev : {L.fork, L.join, L.pfork, L.pjoin})
      if (ev) cudaEventDestroy(ev);
  }
  delete s;
  return SBP_OK;
}

int sbp_solver_levels(const sbp_solver* s) {
  if (!s) return SBP_ERR_ARGS;
  return s->mg ? (int)s->levels.size() : 1;
}

long long sbp_solver_device_bytes(const sbp_solver* s) { return s ? s->dev_bytes : 0; }

long long sbp_solver_last_launches(const sbp_solver* s) { return s ? s->last_launches : 0; }

int sbp_mgcg_solve(sbp_solver* s, const double* b, double* x, double abstol, double reltol,
                   int maxiter, sbp_result* res, double* norms, int norms_cap, void* stream) {
  return run_krylov(s, 0, b, x, +1, abstol, reltol, maxiter, res, norms, norms_cap,
                    (cudaStream_t)stream);
}

int sbp_cg_solve(sbp_solver* s, const double* b, double* x, int sign, double abstol,
                 double reltol, int maxiter, sbp_result* res, double* norms, int norms_cap,
                 void* stream) {
  if (sign != 1 && sign != -1) return SBP_ERR_ARGS;
  return run_krylov(s, 1, b, x, sign, abstol, reltol, maxiter, res, norms, norms_cap,
                    (cudaStream_t)stream);
}

int sbp_mgcg_adjoint_f64(sbp_solver* s, const double* gu, double* lam, double* df, double* dgW,
                         double* dgE, double* dgS, double* dgN, double fsign, double abstol,
                         double reltol, int maxiter, sbp_result* res, void* stream) {
  if (!s || !gu || !lam) return SBP_ERR_ARGS;
  cudaStream_t q = (cudaStream_t)stream;
  SBP_CUDA(cudaSetDevice(s->device));
  const int n = s->n;
  // A is symmetric: the adjoint solve is the forward MGCG on gu, from zero
  SBP_CUDA(cudaMemsetAsync(lam, 0, (size_t)n * n * sizeof(double), q));
  const int rc = run_krylov(s, 0, gu, lam, +1, abstol, reltol, maxiter, res, nullptr, 0, q);
  if (rc != SBP_OK && rc != SBP_ERR_MAXITER) return rc;
  if (df || dgW || dgE || dgS || dgN)
    SBP_CUDA(launch_rhs_adjoint(cgrid<double>(lam, n), grid<double>(df, n), dgW, dgE, dgS, dgN,
                                n, fsign, q));
  return rc;
}

int sbp_test_drop_copy(int drop, unsigned wait_polls) {
  SBP_CUDA(cudaDeviceSynchronize());
  SBP_CUDA(set_copy_drop(drop, wait_polls));
  return SBP_OK;
}

int sbp_test_pair_to_f64(const float* hi, const float* lo, double* out, long long n,
                         void* stream) {
  if (n < 0 || (n > 0 && (!hi || !lo || !out))) return SBP_ERR_ARGS;
  SBP_CUDA(launch_pair_to_f64(hi, lo, out, n, (cudaStream_t)stream));
  return SBP_OK;
}

int sbp_fp64_fma_rate(double* gfma_per_s, void* stream) {
  if (!gfma_per_s) return SBP_ERR_ARGS;
  SBP_CUDA(measure_fp64_fma_rate(gfma_per_s, (cudaStream_t)stream));
  return SBP_OK;
}

int sbp_solver_profile(sbp_solver* s, int kind, const double* b, double* x, int sign,
                       double reltol, int maxiter, sbp_result* res, sbp_kernel_time* out,
                       int cap, int* count, void* stream) {
  if ((kind != 0 && kind != 1) || (kind == 1 && sign != 1 && sign != -1) || !count ||
      (cap > 0 && !out) || reltol <= 0.0)
    return SBP_ERR_ARGS;
  if (kind == 0) sign = +1;
  int rc = krylov_prepare(s, kind, b, x, 0.0, reltol, maxiter);
  if (rc) return rc;
  cudaStream_t q = (cudaStream_t)stream;
  const int n = s->n, ld = s->ld;
  LaunchTimer timer;
  timer_slot() = &timer;
  cudaError_t e = enqueue_setup(s, kind, b, x, sign, 0.0, reltol, maxiter, q);
  for (int k = 0; e == cudaSuccess && k < maxiter; ++k) {
    e = enqueue_iteration(s, kind, k & 1, sign, q);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(&s->st_host[0], s->st, sizeof(SolveState), cudaMemcpyDeviceToHost, q);
    if (e == cudaSuccess) e = cudaStreamSynchronize(q);
    if (e == cudaSuccess && s->st_host[0].done) break;
  }
  timer_slot() = nullptr;
  if (e == cudaSuccess) e = copy_grid(x, n, s->x, ld, n, q);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&s->st_host[0], s->st, sizeof(SolveState), cudaMemcpyDeviceToHost, q);
  if (e == cudaSuccess) e = cudaStreamSynchronize(q);
  // aggregate by kernel (first-launch order), then sort by total time
  struct Agg {
    const void* fn;
    int launches;
    double ms;
  };
  std::vector<Agg> agg;
  for (const LaunchTimer::Rec& r : timer.recs) {
    float ms = 0.f;
    if (e == cudaSuccess && r.e1) e = cudaEventElapsedTime(&ms, r.e0, r.e1);
    size_t k = 0;
    while (k < agg.size() && agg[k].fn != r.fn) ++k;
    if (k == agg.size()) agg.push_back({r.fn, 0, 0.0});
    agg[k].launches += 1;
    agg[k].ms += ms;
  }
  for (const LaunchTimer::Rec& r : timer.recs) {
    if (r.e0) cudaEventDestroy(r.e0);
    if (r.e1) cudaEventDestroy(r.e1);
  }
  if (e != cudaSuccess) return fail_cuda(e, "sbp_solver_profile");
  if (timer.failed) return fail_cuda(cudaErrorMemoryAllocation, "sbp_solver_profile (events)");
  if (const int fr = check_device_fault("sbp_solver_profile")) return fr;
  std::stable_sort(agg.begin(), agg.end(), [](const Agg& a, const Agg& b) { return a.ms > b.ms; });
  *count = (int)agg.size();
  for (int k = 0; k < cap && k < (int)agg.size(); ++k) {
    const char* mangled = nullptr;
    std::string name = "?";
    if (cudaFuncGetName(&mangled, agg[k].fn) == cudaSuccess && mangled) {
      int st = 0;
      char* dm = abi::__cxa_demangle(mangled, nullptr, nullptr, &st);
      name = (st == 0 && dm) ? dm : mangled;
      std::free(dm);
    }
    std::snprintf(out[k].name, sizeof(out[k].name), "%s", name.c_str());
    out[k].launches = agg[k].launches;
    out[k].total_ms = agg[k].ms;
  }
  return finish_result(s->st_host[0], res);
}

int sbp_vcycle_apply(sbp_solver* s, const double* b, double* v, void* stream) {
  if (!s || !b || !v) return SBP_ERR_ARGS;
  if (!s->mg) return SBP_ERR_UNSUPPORTED;
  cudaStream_t q = (cudaStream_t)stream;
  SBP_CUDA(cudaSetDevice(s->device));
  const int n = s->n, ld = s->ld;
  if (s->opts.precision == SBP_PREC_MIXED) {
    SBP_CUDA((launch_copy<double, float>(cgrid<double>(b, n), grid<float>(s->r_lo, ld), n, q)));
    SBP_CUDA(enqueue_vcycle<float>(s, 0, false, nullptr, q));
    SBP_CUDA((launch_copy<float, double>(cgrid<float>(vcycle_out(s), ld), grid<double>(v, n), n, q)));
  } else {
    SBP_CUDA(copy_grid(s->r, ld, b, n, n, q));
    SBP_CUDA(enqueue_vcycle<double>(s, 0, false, nullptr, q));
    SBP_CUDA(copy_grid(v, n, static_cast<const double*>(vcycle_out(s)), ld, n, q));
  }
  return SBP_OK;
}

}  // extern "C"

// ===========================================================================
// Batched MGCG.  Every problem keeps its own solver (buffers, hierarchy,
// Krylov state); the launches of one problem's set-up, iteration and finish
// are recorded instead of launched, and the records at one position of all
// problems of one grid size are launched as one batched kernel (one CTA pool
// over all their tiles, per-problem reductions and early exit).  Grid sizes
// are independent branches on their own streams, forked from and joined into
// the caller's stream; one iteration of the whole batch is one CUDA graph per
// p parity, and the host reads all problems' states once per iteration.
// ===========================================================================
namespace {

struct BatchGroup {
  BatchLaunchFn fn = nullptr;
  int aux[4] = {0, 0, 0, 0};
  int stride = 0;
  size_t offset = 0;  // of the argument blobs in the arena
};

struct BatchArena {
  unsigned char* dev = nullptr;
  size_t cap = 0;
  std::vector<BatchGroup> groups;
};

struct BatchClass {
  int n = 0;
  std::vector<int> members;  // problem indices, increasing
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  BatchScratch scr;
  BatchArena iter[2], setup, finish;
};

}  // namespace

struct sbp_batch {
  int device = 0;
  int count = 0;
  sbp_options opts{};
  std::vector<sbp_solver*> solvers;
  std::vector<BatchClass> classes;  // decreasing n
  SolveState* states = nullptr;       // device, one per problem
  SolveState* states_host = nullptr;  // pinned, 2 x count
  std::vector<void*> allocs;
  cudaGraphExec_t iter_exec[2] = {nullptr, nullptr};
  bool iter_valid = false;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  cudaStream_t cap = nullptr;
  long long launches_per_iter = 0;
  long long last_launches = 0;
  std::vector<double*> captured_norms;  // norm buffers the iteration graphs write
};

namespace {

void batch_free_arena(BatchArena& a) {
  if (a.dev) cudaFree(a.dev);
  a.dev = nullptr;
  a.cap = 0;
  a.groups.clear();
}

// Record `enqueue(solver)` for every member of class c and merge the records
// position by position into the arena (one host-to-device copy).
template <class F>
int batch_record(sbp_batch* B, BatchClass& c, BatchArena& arena, F&& enqueue, cudaStream_t q) {
  const size_t cnt = c.members.size();
  std::vector<std::vector<LaunchRecord>> recs(cnt);
  for (size_t m = 0; m < cnt; ++m) {
    Recorder rec;
    recorder_slot() = &rec;
    const cudaError_t e = enqueue(B->solvers[c.members[m]]);
    recorder_slot() = nullptr;
    if (e != cudaSuccess) return fail_cuda(e, "batched schedule");
    recs[m] = std::move(rec.recs);
  }
  const size_t len = recs[0].size();
  std::vector<BatchGroup> groups(len);
  size_t bytes = 0;
  for (size_t k = 0; k < len; ++k) {
    const LaunchRecord& r0 = recs[0][k];
    BatchGroup& g = groups[k];
    g.fn = r0.fn;
    std::memcpy(g.aux, r0.aux, sizeof(g.aux));
    const size_t al = (size_t)std::max(r0.align, 64);
    g.stride = (int)((r0.blob.size() + al - 1) / al * al);
    bytes = (bytes + 255) & ~(size_t)255;
    g.offset = bytes;
    bytes += (size_t)g.stride * cnt;
  }
  std::vector<unsigned char> host(std::max<size_t>(bytes, 1), 0);
  for (size_t m = 0; m < cnt; ++m) {
    if (recs[m].size() != len) {
      g_last_error = "batched schedule: problems of one size recorded different launches";
      return SBP_ERR_CUDA;
    }
    for (size_t k = 0; k < len; ++k) {
      const LaunchRecord& r = recs[m][k];
      const BatchGroup& g = groups[k];
      if (r.fn != g.fn || std::memcmp(r.aux, g.aux, sizeof(g.aux)) != 0 ||
          r.blob.size() != recs[0][k].blob.size()) {
        g_last_error = "batched schedule: launch shapes differ within a grid size";
        return SBP_ERR_CUDA;
      }
      std::memcpy(host.data() + g.offset + (size_t)g.stride * m, r.blob.data(), r.blob.size());
    }
  }
  if (bytes > arena.cap) {
    if (arena.dev) SBP_CUDA(cudaFree(arena.dev));
    arena.dev = nullptr;
    arena.cap = 0;
    SBP_CUDA(cudaMalloc((void**)&arena.dev, bytes));
    arena.cap = bytes;
  }
  if (bytes) SBP_CUDA(cudaMemcpyAsync(arena.dev, host.data(), bytes, cudaMemcpyHostToDevice, q));
  arena.groups = std::move(groups);
  return SBP_OK;
}

cudaError_t batch_launch(BatchClass& c, const BatchArena& a, cudaStream_t s) {
  const int cnt = (int)c.members.size();
  for (const BatchGroup& g : a.groups) {
    const cudaError_t e = g.fn(a.dev + g.offset, g.stride, cnt, g.aux, c.scr, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Run `pick(class)`'s arena on every class stream, forked from and joined
// into q.
template <class Pick>
cudaError_t batch_run(sbp_batch* B, cudaStream_t q, Pick&& pick) {
  for (BatchClass& c : B->classes) {
    cudaError_t e = cudaEventRecord(c.fork, q);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c.stream, c.fork, 0);
    if (e == cudaSuccess) e = batch_launch(c, pick(c), c.stream);
    if (e == cudaSuccess) e = cudaEventRecord(c.join, c.stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(q, c.join, 0);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Resolve every batched launch's configuration outside stream capture.
cudaError_t batch_prepare(BatchClass& c, const BatchArena& a) {
  for (const BatchGroup& g : a.groups) {
    const cudaError_t e = g.fn(nullptr, g.stride, 0, g.aux, c.scr, nullptr);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

void batch_destroy_graphs(sbp_batch* B) {
  for (auto& g : B->iter_exec)
    if (g) cudaGraphExecDestroy(g);
  B->iter_exec[0] = B->iter_exec[1] = nullptr;
  B->iter_valid = false;
}

int batch_capture(sbp_batch* B, cudaStream_t q) {
  long long per_iter = 0;
  for (BatchClass& c : B->classes) {
    for (int par = 0; par < 2; ++par) {
      const int rc = batch_record(
          B, c, c.iter[par],
          [&](sbp_solver* s) { return enqueue_iteration(s, 0, par, +1, nullptr); }, q);
      if (rc) return rc;
      SBP_CUDA(batch_prepare(c, c.iter[par]));
    }
    per_iter += (long long)c.iter[0].groups.size();
  }
  SBP_CUDA(cudaStreamSynchronize(q));  // arenas uploaded before the graphs read them
  batch_destroy_graphs(B);
  for (int par = 0; par < 2; ++par) {
    cudaGraph_t g = nullptr;
    SBP_CUDA(cudaStreamBeginCapture(B->cap, cudaStreamCaptureModeThreadLocal));
    const cudaError_t e = batch_run(B, B->cap, [&](BatchClass& c) -> const BatchArena& {
      return c.iter[par];
    });
    const cudaError_t e2 = cudaStreamEndCapture(B->cap, &g);
    if (e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return fail_cuda(e, "batched iteration (capture)");
    }
    if (e2 != cudaSuccess) return fail_cuda(e2, "cudaStreamEndCapture");
    const cudaError_t e3 = cudaGraphInstantiate(&B->iter_exec[par], g, 0);
    cudaGraphDestroy(g);
    if (e3 != cudaSuccess) return fail_cuda(e3, "cudaGraphInstantiate");
  }
  B->launches_per_iter = per_iter;
  B->captured_norms.clear();
  for (const sbp_solver* s : B->solvers) B->captured_norms.push_back(s->norms);
  B->iter_valid = true;
  return SBP_OK;
}

// The iteration graphs stay valid while no solver's norm buffer was regrown.
bool batch_graphs_current(const sbp_batch* B) {
  if (!B->iter_valid || B->captured_norms.size() != B->solvers.size()) return false;
  for (size_t k = 0; k < B->solvers.size(); ++k)
    if (B->solvers[k]->norms != B->captured_norms[k]) return false;
  return true;
}

int batch_destroy(sbp_batch* B) {
  if (!B) return SBP_OK;
  cudaSetDevice(B->device);
  batch_destroy_graphs(B);
  for (BatchClass& c : B->classes) {
    for (BatchArena* a : {&c.iter[0], &c.iter[1], &c.setup, &c.finish}) batch_free_arena(*a);
    if (c.stream) cudaStreamDestroy(c.stream);
    if (c.fork) cudaEventDestroy(c.fork);
    if (c.join) cudaEventDestroy(c.join);
  }
  for (sbp_solver* s : B->solvers) sbp_solver_destroy(s);
  for (void* p : B->allocs) cudaFree(p);
  if (B->states_host) cudaFreeHost(B->states_host);
  for (auto& e : B->ev)
    if (e) cudaEventDestroy(e);
  if (B->cap) cudaStreamDestroy(B->cap);
  delete B;
  return SBP_OK;
}

}  // namespace

extern "C" {

int sbp_batch_create(sbp_batch** out, const int* ns, int count, const sbp_options* opts) {
  if (!out || !ns || !opts || count < 1) return SBP_ERR_ARGS;
  *out = nullptr;
  for (int k = 0; k < count; ++k)
    if (!valid_mg_n(ns[k]) || ns[k] < opts->coarse_n) return SBP_ERR_ARGS;
  sbp_batch* B = new (std::nothrow) sbp_batch();
  if (!B) return SBP_ERR_NOMEM;
  std::unique_ptr<sbp_batch, int (*)(sbp_batch*)> guard(B, batch_destroy);
  SBP_CUDA(cudaGetDevice(&B->device));
  B->count = count;
  B->opts = *opts;
  void* p = nullptr;
  SBP_CUDA(cudaMalloc(&p, (size_t)count * sizeof(SolveState)));
  B->allocs.push_back(p);
  B->states = static_cast<SolveState*>(p);
  SBP_CUDA(cudaMallocHost((void**)&B->states_host, 2 * (size_t)count * sizeof(SolveState)));
  B->solvers.assign(count, nullptr);
  for (int k = 0; k < count; ++k) {
    const int rc = sbp_solver_create(&B->solvers[k], ns[k], opts);
    if (rc) return rc;
    sbp_solver* s = B->solvers[k];
    s->st = B->states + k;  // the batch reads every state in one copy
    // resolve the V-cycle schedule (which buffer holds its output) before any
    // iteration is recorded: record one V-cycle and discard it
    Recorder scratch;
    recorder_slot() = &scratch;
    const cudaError_t e = enqueue_vcycle_any(s, true, s->st, nullptr);
    recorder_slot() = nullptr;
    if (e != cudaSuccess) return fail_cuda(e, "batched schedule");
  }
  std::vector<int> sizes(ns, ns + count);
  std::sort(sizes.begin(), sizes.end(), std::greater<int>());
  sizes.erase(std::unique(sizes.begin(), sizes.end()), sizes.end());
  B->classes.resize(sizes.size());
  for (size_t c = 0; c < sizes.size(); ++c) {
    BatchClass& C = B->classes[c];
    C.n = sizes[c];
    for (int k = 0; k < count; ++k)
      if (ns[k] == C.n) C.members.push_back(k);
    if ((int)C.members.size() > kMaxBatchSlots) return SBP_ERR_UNSUPPORTED;
    SBP_CUDA(cudaStreamCreateWithFlags(&C.stream, cudaStreamNonBlocking));
    SBP_CUDA(cudaEventCreateWithFlags(&C.fork, cudaEventDisableTiming));
    SBP_CUDA(cudaEventCreateWithFlags(&C.join, cudaEventDisableTiming));
    const long long parts = (long long)kMaxPersistCtas * (long long)C.members.size();
    SBP_CUDA(cudaMalloc(&p, (size_t)parts * sizeof(double) + 256));
    B->allocs.push_back(p);
    C.scr.partials = static_cast<double*>(p);
    C.scr.ticket = reinterpret_cast<unsigned*>(static_cast<unsigned char*>(p) +
                                               (size_t)parts * sizeof(double));
    C.scr.cap = parts;
    SBP_CUDA(cudaMemset(C.scr.ticket, 0, sizeof(unsigned)));
  }
  SBP_CUDA(cudaStreamCreateWithFlags(&B->cap, cudaStreamNonBlocking));
  for (auto& e : B->ev) SBP_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  SBP_CUDA(cudaDeviceSynchronize());
  guard.release();
  *out = B;
  return SBP_OK;
}

int sbp_batch_destroy(sbp_batch* B) { return batch_destroy(B); }

int sbp_batch_size(const sbp_batch* B) { return B ? B->count : SBP_ERR_ARGS; }

long long sbp_batch_device_bytes(const sbp_batch* B) {
  if (!B) return SBP_ERR_ARGS;
  long long t = (long long)B->count * (long long)sizeof(SolveState);
  for (const sbp_solver* s : B->solvers) t += sbp_solver_device_bytes(s);
  for (const BatchClass& c : B->classes) t += c.scr.cap * (long long)sizeof(double);
  return t;
}

long long sbp_batch_last_launches(const sbp_batch* B) { return B ? B->last_launches : 0; }

int sbp_batch_autotune(sbp_batch* B, const double* const* b, double* const* x, int* budgets,
                       void* stream) {
  if (!B || !b || !x) return SBP_ERR_ARGS;
  cudaStream_t q = (cudaStream_t)stream;
  SBP_CUDA(cudaSetDevice(B->device));
  const int kIters = 3;
  for (int k = 0; k < B->count; ++k) {
    const int rc = krylov_prepare(B->solvers[k], 0, b[k], x[k], 0.0, 1e-30, kIters + 4);
    if (rc) return rc;
  }
  if (!batch_graphs_current(B)) {
    const int rc = batch_capture(B, q);
    if (rc) return rc;
  }
  const int sms = batch_sm_count();
  const int cands[4] = {0, 2 * sms, sms, sms / 2};
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  SBP_CUDA(cudaEventCreate(&t0));
  SBP_CUDA(cudaEventCreate(&t1));
  int rc = SBP_OK;
  for (size_t ci = 0; ci < B->classes.size() && rc == SBP_OK; ++ci) {
    BatchClass& c = B->classes[ci];
    rc = batch_record(
        B, c, c.setup,
        [&](sbp_solver* s) {
          const int k = (int)(s->st - B->states);
          return enqueue_setup(s, 0, b[k], x[k], +1, 0.0, 1e-30, kIters + 4, nullptr);
        },
        q);
    if (rc) break;
    if (cudaError_t e = batch_prepare(c, c.setup); e != cudaSuccess) {
      rc = fail_cuda(e, "autotune");
      break;
    }
    float best = 0.f;
    int best_budget = 0;
    for (int cand : cands) {
      c.scr.cta_budget = cand;
      cudaError_t e = cudaEventRecord(c.fork, q);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(c.stream, c.fork, 0);
      if (e == cudaSuccess) e = batch_launch(c, c.setup, c.stream);
      if (e == cudaSuccess) e = cudaEventRecord(t0, c.stream);
      for (int it = 0; it < kIters && e == cudaSuccess; ++it)
        e = batch_launch(c, c.iter[it & 1], c.stream);
      if (e == cudaSuccess) e = cudaEventRecord(t1, c.stream);
      if (e == cudaSuccess) e = cudaEventSynchronize(t1);
      float ms = 0.f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, t0, t1);
      if (e != cudaSuccess) {
        rc = fail_cuda(e, "autotune");
        break;
      }
      if (best_budget == 0 && cand == 0) best = ms;
      if (ms < best) {
        best = ms;
        best_budget = cand;
      }
    }
    c.scr.cta_budget = best_budget;
    if (budgets) budgets[ci] = best_budget;
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  if (rc) return rc;
  SBP_CUDA(cudaStreamSynchronize(q));
  if (const int fr = check_device_fault("sbp_batch_autotune")) return fr;
  B->iter_valid = false;  // recapture with the chosen launch shapes
  return batch_capture(B, q);
}

int sbp_batch_classes(const sbp_batch* B, int* ns, int cap) {
  if (!B) return SBP_ERR_ARGS;
  const int cnt = (int)B->classes.size();
  for (int c = 0; c < cnt && ns && c < cap; ++c) ns[c] = B->classes[c].n;
  return cnt;
}

int sbp_batch_mgcg_solve(sbp_batch* B, const double* const* b, double* const* x, double abstol,
                         double reltol, int maxiter, sbp_result* results, void* stream) {
  if (!B || !b || !x) return SBP_ERR_ARGS;
  cudaStream_t q = (cudaStream_t)stream;
  SBP_CUDA(cudaSetDevice(B->device));
  for (int k = 0; k < B->count; ++k) {
    const int rc = krylov_prepare(B->solvers[k], 0, b[k], x[k], abstol, reltol, maxiter);
    if (rc) return rc;
  }
  if (!batch_graphs_current(B)) {
    const int rc = batch_capture(B, q);
    if (rc) return rc;
  }
  // set-up and finish schedules carry this solve's pointers and tolerances
  for (BatchClass& c : B->classes) {
    int rc = batch_record(
        B, c, c.setup,
        [&](sbp_solver* s) {
          const int k = (int)(s->st - B->states);
          return enqueue_setup(s, 0, b[k], x[k], +1, abstol, reltol, maxiter, nullptr);
        },
        q);
    if (rc) return rc;
    rc = batch_record(
        B, c, c.finish,
        [&](sbp_solver* s) {
          const int k = (int)(s->st - B->states);
          return copy_grid(x[k], s->n, s->x, s->ld, s->n, nullptr);
        },
        q);
    if (rc) return rc;
    SBP_CUDA(batch_prepare(c, c.setup));
    SBP_CUDA(batch_prepare(c, c.finish));
  }
  long long launches = 0;
  for (BatchClass& c : B->classes) launches += (long long)c.setup.groups.size();
  SBP_CUDA(batch_run(B, q, [](BatchClass& c) -> const BatchArena& { return c.setup; }));
  const size_t sb = (size_t)B->count * sizeof(SolveState);
  int k = 0;
  bool finished = (maxiter == 0);
  while (!finished) {
    SBP_CUDA(cudaGraphLaunch(B->iter_exec[k & 1], q));
    launches += B->launches_per_iter;
    SBP_CUDA(cudaMemcpyAsync(B->states_host + (size_t)(k & 1) * B->count, B->states, sb,
                             cudaMemcpyDeviceToHost, q));
    SBP_CUDA(cudaEventRecord(B->ev[k & 1], q));
    if (k >= 1) {
      SBP_CUDA(cudaEventSynchronize(B->ev[(k - 1) & 1]));
      const SolveState* h = B->states_host + (size_t)((k - 1) & 1) * B->count;
      bool all = true;
      for (int m = 0; m < B->count && all; ++m) all = h[m].done != 0;
      if (all) finished = true;
    }
    ++k;
    if (k > maxiter + 2) finished = true;  // safety net; kernels stop at maxiter
  }
  SBP_CUDA(batch_run(B, q, [](BatchClass& c) -> const BatchArena& { return c.finish; }));
  for (BatchClass& c : B->classes) launches += (long long)c.finish.groups.size();
  SBP_CUDA(cudaMemcpyAsync(B->states_host, B->states, sb, cudaMemcpyDeviceToHost, q));
  SBP_CUDA(cudaStreamSynchronize(q));
  if (const int fr = check_device_fault("sbp_batch_mgcg_solve")) return fr;
  B->last_launches = launches;
  int status = SBP_OK;
  for (int m = 0; m < B->count; ++m) {
    const int st = finish_result(B->states_host[m], results ? results + m : nullptr);
    if (st != SBP_OK && status == SBP_OK) status = st;
  }
  return status;
}

}  // extern "C"

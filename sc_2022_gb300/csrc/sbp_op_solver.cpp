// Solver handles for the operators beyond the second-order constant-
// coefficient one: the higher-order (p = 4, 6) SBP-SAT operators and the
// variable-coefficient second-order operator.  Both get matrix-free CG and
// multigrid-preconditioned CG, in FP64 or mixed precision (FP32 V-cycle
// inside FP64 PCG).
//
// The reference solves these operators on the CPU only:
// - Assembling_matrix(level; p = SBPp) with the multigrid preconditioner
//   precond_matrix(A, b; SBPp) (initial_guess_cg.jl:458-510);
// - get_operators(p, h) over variable_diagonal_sbp_D2
//   (legacy_functions.jl:100-174).
// Its preconditioner is weighted Jacobi (omega = 2/3, m = 3 sweeps) with
// standard transfers and the re-discretised coarse operator.  Here the same
// V-cycle runs on the GPU over any number of levels:
// - each level re-discretises the operator; the coarse coefficients are the
//   full-weighting harmonic mean of the fine ones (injection under-samples
//   thin layers and costs iterations);
// - the smoother is Jacobi or Richardson;
// - the transfers are the second-order path's restriction and prolongation
//   kernels;
// - the coarse level is solved exactly: fast diagonalisation of the order-p
//   Kronecker sum, or a dense inverse for variable coefficients.
// One (P)CG iteration is captured once as a CUDA graph. Its kernels read
// alpha and beta from a device SolveState and exit at once after
// convergence; the host checks the state one iteration behind.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <new>
#include <stdexcept>
#include <thread>
#include <vector>

#include "../../include/sbpmg.h"
#include "sbp_coarse.h"
#include "sbp_host.h"
#include "sbp_launch.h"
#include "sbp_varcoef.cuh"

using namespace sbp;

namespace {

enum OpKind { kOpHighOrder = 0, kOpVariable = 1 };

// Largest coarse grid of the variable-coefficient hierarchy (dense inverse
// of (nc^2)^2 doubles, built on the host at creation).
constexpr int kVcMaxCoarse = 33;

struct OpSolver {
  // Level buffers hold doubles, or floats for the mixed-precision V-cycle.
  struct Lvl {
    int n = 0;
    void* b = nullptr;   // level 0: the solver's r (FP64) or r_lo (mixed)
    void* v[2] = {nullptr, nullptr};
    void* t = nullptr;   // residual scratch
    // variable coefficients: nodal c (FP64) and the stencil arrays in the
    // V-cycle's precision
    double* c = nullptr;
    void* st[6] = {};   // E, N, D, flo, fhi, 1/D
  };
  int kind = kOpHighOrder;
  int n = 0, p = 0, device = 0;
  bool mg = false;
  bool mixed = false;
  sbp_options opts{};
  std::vector<Lvl> lv;
  CoarseDev coarse{};          // order p: fast-diagonalisation factors
  double* ainv = nullptr;      // variable: dense coarse inverse
  int ainv_n = 0;              // its order (nc^2)
  double* st64[6] = {};        // level-0 FP64 stencil arrays
  float2* pairs[5] = {};       // mixed: level-0 E, N, D, flo, fhi as float pairs
  double* c0 = nullptr;        // variable: the caller's coefficients (device copy)
  float* r_lo = nullptr;       // mixed: FP32 copy of r, written by the update
  double *x = nullptr, *r = nullptr, *pd = nullptr, *ap = nullptr;
  double* norms = nullptr;
  int norms_cap = 0;
  SolveState* st = nullptr;
  SolveState* st_host = nullptr;   // pinned, two slots
  ReduceBuf rb[3]{};
  cudaStream_t cap = nullptr;
  cudaGraphExec_t exec[2] = {nullptr, nullptr};   // 0: MGCG, 1: CG
  int exec_sign[2] = {0, 0};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  std::vector<void*> allocs;
  long long dev_bytes = 0;
};

}  // namespace

struct sbp_ho_solver : OpSolver {};
struct sbp_vc_solver : OpSolver {};

namespace {

bool pow2_plus1(int n) {
  const int m = n - 1;
  return n >= 3 && (m & (m - 1)) == 0;
}

template <typename T>
int dalloc(OpSolver* s, T** out, size_t count) {
  void* p = nullptr;
  const size_t bytes = std::max<size_t>(count * sizeof(T), 256);
  const cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) {
    set_last_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return SBP_ERR_NOMEM;
  }
  s->allocs.push_back(p);
  s->dev_bytes += (long long)bytes;
  *out = static_cast<T*>(p);
  return SBP_OK;
}

template <typename T = double>
HoArgsT<T> op_args(int n) {
  HoArgsT<T> a{};
  a.n = n;
  a.sign = 1;
  return a;
}

template <typename T>
T* as(void* p) {
  return static_cast<T*>(p);
}

// One operator launch on grid level l (stencil: the level's arrays in T;
// level 0 in FP64 for the Krylov apply and residual).
template <typename T>
cudaError_t op_launch(OpSolver* s, size_t l, int mode, const HoArgsT<T>& a, cudaStream_t q) {
  if (s->kind == kOpHighOrder) return launch_ho<T>(s->p, mode, a, q);
  VcArgsT<T> v;
  static_cast<HoArgsT<T>&>(v) = a;
  const bool fp64_level0 = sizeof(T) == sizeof(double) && l == 0;
  for (int k = 0; k < 6; ++k) {
    const void* arr = fp64_level0 ? (const void*)s->st64[k] : s->lv[l].st[k];
    const T* pa = static_cast<const T*>(arr);
    if (k == 0) v.E = pa;
    if (k == 1) v.N = pa;
    if (k == 2) v.D = pa;
    if (k == 3) v.flo = pa;
    if (k == 4) v.fhi = pa;
    if (k == 5) v.Dinv = pa;
  }
  return launch_vc<T>(mode, v, q);
}

// Smoothing sweeps on level l from v[cur]; returns the buffer index holding
// the result.  zero: start from v = 0.
template <typename T>
int smooth(OpSolver* s, size_t l, int cur, int sweeps, bool zero, cudaStream_t q,
           cudaError_t& err) {
  const auto& L = s->lv[l];
  const bool rich = s->opts.smoother == SBP_SMOOTH_RICHARDSON;
  const double omega = s->opts.omega > 0.0 ? s->opts.omega : (rich ? 0.15 : 2.0 / 3.0);
  for (int k = 0; k < sweeps && err == cudaSuccess; ++k) {
    HoArgsT<T> a = op_args<T>(L.n);
    a.u = as<T>(L.v[cur]);
    a.b = as<T>(L.b);
    a.out = as<T>(L.v[1 - cur]);
    a.omega = omega;
    a.richardson = rich ? 1 : 0;
    a.zero_in = (zero && k == 0) ? 1 : 0;
    a.st = s->st;
    err = op_launch<T>(s, l, kHoJacobi, a, q);
    cur = 1 - cur;
  }
  return cur;
}

template <typename T>
cudaError_t coarse_solve(OpSolver* s, const OpSolver::Lvl& L, cudaStream_t q) {
  if (s->kind == kOpHighOrder)
    return launch_coarse_solve<T>(s->coarse, Grid<const T>{as<T>(L.b), L.n},
                                  Grid<T>{as<T>(L.v[0]), L.n}, s->st, q);
  return launch_dense_gemv<T>(s->ainv, as<T>(L.b), as<T>(L.v[0]), s->ainv_n, s->st, q);
}

// One V-cycle from v = 0 on level l for the right-hand side lv[l].b; returns
// the buffer holding the result.  T: the V-cycle's arithmetic (the coarse
// solve accumulates in FP64 either way).
template <typename T>
T* vcycle(OpSolver* s, size_t l, cudaStream_t q, cudaError_t& err) {
  auto& L = s->lv[l];
  const int n = L.n;
  if (l + 1 == s->lv.size()) {
    err = coarse_solve<T>(s, L, q);
    return as<T>(L.v[0]);
  }
  int cur = 0;
  if (s->opts.nu_pre > 0) {
    cur = smooth<T>(s, l, 1, s->opts.nu_pre, true, q, err);
  } else {
    err = cudaMemsetAsync(L.v[0], 0, (size_t)n * n * sizeof(T), q);
  }
  if (err != cudaSuccess) return nullptr;
  HoArgsT<T> a = op_args<T>(n);
  a.u = as<T>(L.v[cur]);
  a.b = as<T>(L.b);
  a.out = as<T>(L.t);
  a.st = s->st;
  err = op_launch<T>(s, l, kHoResid, a, q);
  if (err != cudaSuccess) return nullptr;
  auto& C = s->lv[l + 1];
  err = launch_resrestrict<T>(Grid<const T>{nullptr, 0}, Grid<const T>{as<T>(L.t), n},
                              Grid<T>{as<T>(C.b), C.n}, n, s->opts.restriction, s->st, q);
  if (err != cudaSuccess) return nullptr;
  T* e = vcycle<T>(s, l + 1, q, err);
  if (err != cudaSuccess) return nullptr;
  err = launch_prolong<T>(Grid<const T>{e, C.n}, Grid<T>{as<T>(L.v[cur]), n}, C.n, 1, s->st, q);
  if (err != cudaSuccess) return nullptr;
  cur = smooth<T>(s, l, cur, s->opts.nu_post, false, q, err);
  return as<T>(L.v[cur]);
}

// z = V(r), then beta = r.z / r.z_old and p = z + beta p (first: p = z).
template <typename T>
cudaError_t precondition(OpSolver* s, int first, cudaStream_t q) {
  cudaError_t err = cudaSuccess;
  const long long N = (long long)s->n * s->n;
  T* z = vcycle<T>(s, 0, q, err);
  if (err != cudaSuccess) return err;
  err = launch_ho_rz<T>(s->r, z, N, s->st, s->rb[2], first, q);
  if (err != cudaSuccess) return err;
  return launch_ho_dir<T>(z, s->pd, N, s->st, first, q);
}

// Mixed-precision MGCG forms Ap with the direction: z = V(r), beta, then
// p = z + beta p and Ap = A z + beta Ap with p.Ap -> alpha in one kernel
// (A z on the FP32 pipe), so an iteration has no FP64 apply.
bool fused_direction(const OpSolver* s) { return s->mixed; }

cudaError_t precondition_fused(OpSolver* s, int first, cudaStream_t q) {
  cudaError_t err = cudaSuccess;
  const long long N = (long long)s->n * s->n;
  float* z = vcycle<float>(s, 0, q, err);
  if (err != cudaSuccess) return err;
  err = launch_ho_rz<float>(s->r, z, N, s->st, s->rb[2], first, q);
  if (err != cudaSuccess) return err;
  if (s->kind == kOpHighOrder)
    return launch_ho_dir_mixed(s->p, z, s->pd, s->ap, s->n, s->st, s->rb[0], q);
  return launch_vc_dir_mixed(z, s->pairs, s->pd, s->ap, s->n, s->st, s->rb[0], q);
}

// The iteration body: Ap and alpha, x/r update and ||r||^2, then the new
// direction (MGCG: z = V(r), beta = r.z / r.z_old; CG: beta from ||r||^2).
cudaError_t enqueue_iteration(OpSolver* s, int kind, int sign, cudaStream_t q) {
  const int n = s->n;
  const long long N = (long long)n * n;
  if (kind == 0 && fused_direction(s)) {   // update, V-cycle, beta, direction + Ap + alpha
    cudaError_t err = launch_cg_update<double>(
        Grid<double>{s->x, n}, Grid<double>{s->r, n}, Grid<const double>{s->pd, n},
        Grid<const double>{s->ap, n}, Grid<float>{s->r_lo, n}, n, 0, s->st, s->norms, s->rb[1],
        q);
    if (err != cudaSuccess) return err;
    return precondition_fused(s, 0, q);
  }
  HoArgs a = op_args(n);
  a.u = s->pd;
  a.out = s->ap;
  a.sign = sign;
  a.rb = s->rb[0];
  a.st = s->st;
  cudaError_t err = op_launch<double>(s, 0, kHoApply, a, q);
  if (err != cudaSuccess) return err;
  // the update also refreshes the FP32 copy of r for a mixed V-cycle
  const bool lo = kind == 0 && s->mixed;
  err = launch_cg_update<double>(Grid<double>{s->x, n}, Grid<double>{s->r, n},
                                 Grid<const double>{s->pd, n}, Grid<const double>{s->ap, n},
                                 Grid<float>{lo ? s->r_lo : nullptr, n}, n, kind == 1 ? 1 : 0,
                                 s->st, s->norms, s->rb[1], q);
  if (err != cudaSuccess) return err;
  if (kind == 1) return launch_ho_dir<double>(s->r, s->pd, N, s->st, 0, q);
  return s->mixed ? precondition<float>(s, 0, q) : precondition<double>(s, 0, q);
}

void destroy_graphs(OpSolver* s) {
  for (auto& g : s->exec)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

int capture(OpSolver* s, int kind, int sign) {
  if (s->exec[kind]) {
    cudaGraphExecDestroy(s->exec[kind]);
    s->exec[kind] = nullptr;
  }
  SBP_CUDA(cudaStreamBeginCapture(s->cap, cudaStreamCaptureModeThreadLocal));
  const cudaError_t e = enqueue_iteration(s, kind, sign, s->cap);
  cudaGraph_t g = nullptr;
  const cudaError_t e2 = cudaStreamEndCapture(s->cap, &g);
  if (e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return fail_cuda(e, "capturing the iteration");
  }
  SBP_CUDA(e2);
  const cudaError_t e3 = cudaGraphInstantiate(&s->exec[kind], g, 0);
  cudaGraphDestroy(g);
  SBP_CUDA(e3);
  s->exec_sign[kind] = sign;
  return SBP_OK;
}

// The residual-norm history holds maxiter + 1 entries.  A larger request
// replaces the array; the iteration graphs that point at the old one are
// dropped (every solve has finished before the next one starts).
int ensure_norms(OpSolver* s, int maxiter) {
  if (maxiter + 1 <= s->norms_cap) return SBP_OK;
  double* p = nullptr;
  const int cap = std::max(maxiter + 1, 1024);
  const int rc = dalloc(s, &p, (size_t)cap);
  if (rc) return rc;
  if (s->norms) {
    destroy_graphs(s);
    for (auto it = s->allocs.begin(); it != s->allocs.end(); ++it)
      if (*it == s->norms) {
        cudaFree(*it);
        s->allocs.erase(it);
        s->dev_bytes -= (long long)std::max<size_t>((size_t)s->norms_cap * sizeof(double), 256);
        break;
      }
  }
  s->norms = p;
  s->norms_cap = cap;
  return SBP_OK;
}

int solve(OpSolver* s, int kind, const double* b, double* x, int sign, double abstol,
          double reltol, int maxiter, sbp_result* res, double* norms_out, int norms_cap,
          cudaStream_t q) {
  if (!s || !b || !x || maxiter < 0 || (sign != 1 && sign != -1)) return SBP_ERR_ARGS;
  if (abstol <= 0.0 && reltol <= 0.0) return SBP_ERR_ARGS;
  if (kind == 0 && (!s->mg || sign != 1)) return SBP_ERR_UNSUPPORTED;
  SBP_CUDA(cudaSetDevice(s->device));
  int rc = ensure_norms(s, maxiter);
  if (rc) return rc;
  const int n = s->n;
  const long long N = (long long)n * n;
  // set-up: x, r = b - sign A x, the state, the first direction
  SBP_CUDA(cudaMemcpyAsync(s->x, x, (size_t)N * sizeof(double), cudaMemcpyDeviceToDevice, q));
  SBP_CUDA(launch_state_init(s->st, maxiter, q));
  HoArgs a = op_args(n);
  a.u = s->x;
  a.b = b;
  a.out = s->r;
  a.sign = sign;
  a.rb = s->rb[1];
  a.st = s->st;
  a.init = 1;
  a.abstol = abstol;
  a.reltol = reltol;
  a.norms = s->norms;
  SBP_CUDA(op_launch<double>(s, 0, kHoResid, a, q));
  if (kind == 1) {
    SBP_CUDA(launch_ho_dir<double>(s->r, s->pd, N, s->st, 1, q));
  } else if (s->mixed) {
    SBP_CUDA(launch_copy<double, float>(Grid<const double>{s->r, n}, Grid<float>{s->r_lo, n}, n,
                                        q));
    if (fused_direction(s))
      SBP_CUDA(precondition_fused(s, 1, q));
    else
      SBP_CUDA(precondition<float>(s, 1, q));
  } else {
    SBP_CUDA(precondition<double>(s, 1, q));
  }
  if (!s->exec[kind] || s->exec_sign[kind] != sign) {
    rc = capture(s, kind, sign);
    if (rc) return rc;
  }
  int k = 0;
  bool finished = maxiter == 0;
  while (!finished) {
    SBP_CUDA(cudaGraphLaunch(s->exec[kind], q));
    SBP_CUDA(cudaMemcpyAsync(&s->st_host[k & 1], s->st, sizeof(SolveState),
                             cudaMemcpyDeviceToHost, q));
    SBP_CUDA(cudaEventRecord(s->ev[k & 1], q));
    if (k >= 1) {
      SBP_CUDA(cudaEventSynchronize(s->ev[(k - 1) & 1]));
      if (s->st_host[(k - 1) & 1].done) finished = true;
    }
    ++k;
    if (k > maxiter + 2) finished = true;   // the kernels stop at maxiter
  }
  SBP_CUDA(cudaMemcpyAsync(x, s->x, (size_t)N * sizeof(double), cudaMemcpyDeviceToDevice, q));
  SBP_CUDA(cudaMemcpyAsync(&s->st_host[0], s->st, sizeof(SolveState), cudaMemcpyDeviceToHost, q));
  SBP_CUDA(cudaStreamSynchronize(q));
  if (const int fr = check_device_fault("solve")) return fr;
  const SolveState fs = s->st_host[0];
  if (norms_out && norms_cap > 0) {
    const int cnt = std::min(norms_cap, fs.iter + 1);
    SBP_CUDA(cudaMemcpy(norms_out, s->norms, (size_t)cnt * sizeof(double),
                        cudaMemcpyDeviceToHost));
  }
  return finish_result(fs, res);
}

int vcycle_apply(OpSolver* s, const double* b, double* v, cudaStream_t q) {
  if (!s || !b || !v) return SBP_ERR_ARGS;
  if (!s->mg) return SBP_ERR_UNSUPPORTED;
  SBP_CUDA(cudaSetDevice(s->device));
  const int n = s->n;
  const size_t bytes = (size_t)n * n * sizeof(double);
  // the V-cycle kernels exit early on a finished state: run it on a fresh one
  SBP_CUDA(launch_state_init(s->st, 1, q));
  SBP_CUDA(cudaMemcpyAsync(s->r, b, bytes, cudaMemcpyDeviceToDevice, q));
  cudaError_t err = cudaSuccess;
  if (s->mixed) {
    SBP_CUDA(launch_copy<double, float>(Grid<const double>{s->r, n}, Grid<float>{s->r_lo, n}, n,
                                        q));
    float* z = vcycle<float>(s, 0, q, err);
    SBP_CUDA(err);
    SBP_CUDA(launch_copy<float, double>(Grid<const float>{z, n}, Grid<double>{v, n}, n, q));
  } else {
    double* z = vcycle<double>(s, 0, q, err);
    SBP_CUDA(err);
    SBP_CUDA(cudaMemcpyAsync(v, z, bytes, cudaMemcpyDeviceToDevice, q));
  }
  SBP_CUDA(cudaStreamSynchronize(q));
  return check_device_fault("vcycle");
}

// ---- creation ----------------------------------------------------------

// Buffers shared by both operator kinds; the hierarchy's grid sizes in ns.
int create_common(OpSolver* s, int n, const sbp_options& o, int coarse_cap, int min_n,
                  std::vector<int>& ns) {
  SBP_CUDA(prepare_kernels());
  SBP_CUDA(cudaGetDevice(&s->device));
  s->n = n;
  s->opts = o;
  s->mixed = o.precision == SBP_PREC_MIXED;
  const size_t N = (size_t)n * n;
  int rc = 0;
  for (double** v : {&s->x, &s->r, &s->pd, &s->ap}) {
    rc = dalloc(s, v, N);
    if (rc) return rc;
    SBP_CUDA(cudaMemset(*v, 0, N * sizeof(double)));
  }
  const size_t parts = (size_t)max_reduce_ctas(n);
  for (auto& rb : s->rb) {
    double* base = nullptr;
    rc = dalloc(s, &base, parts + 32);
    if (rc) return rc;
    rb.partials = base;
    rb.ticket = reinterpret_cast<unsigned*>(base + parts);
    SBP_CUDA(cudaMemset(rb.ticket, 0, sizeof(unsigned)));
  }
  double* stp = nullptr;
  rc = dalloc(s, &stp, 64);
  if (rc) return rc;
  s->st = reinterpret_cast<SolveState*>(stp);
  SBP_CUDA(cudaMallocHost((void**)&s->st_host, 2 * sizeof(SolveState)));
  SBP_CUDA(cudaStreamCreateWithFlags(&s->cap, cudaStreamNonBlocking));
  for (auto& e : s->ev) SBP_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  rc = ensure_norms(s, 1023);
  if (rc) return rc;
  // multigrid hierarchy: n, (n+1)/2, ... down to the coarse size, or n alone
  // (the direct solve) when n <= the coarse size.  Other grids get CG only.
  const int cn = std::min(o.coarse_n, coarse_cap);
  const bool direct = n <= cn;
  s->mg = direct || (pow2_plus1(n) && pow2_plus1(cn) && cn >= min_n);
  ns.clear();
  if (!s->mg) return SBP_OK;
  if (s->mixed) {
    rc = dalloc(s, &s->r_lo, N);
    if (rc) return rc;
  }
  const size_t esize = s->mixed ? sizeof(float) : sizeof(double);
  int m = n;
  while (true) {
    ns.push_back(m);
    OpSolver::Lvl L;
    L.n = m;
    const size_t M = (size_t)m * m * esize / sizeof(float);   // in floats
    float* buf = nullptr;
    if (s->lv.empty()) {
      L.b = s->mixed ? (void*)s->r_lo : (void*)s->r;
    } else {
      rc = dalloc(s, &buf, M);
      if (rc) return rc;
      L.b = buf;
    }
    for (void** dst : {&L.v[0], &L.v[1], &L.t}) {
      rc = dalloc(s, &buf, M);
      if (rc) return rc;
      *dst = buf;
    }
    s->lv.push_back(L);
    if (direct || m == cn) break;
    m = (m + 1) / 2;
  }
  return SBP_OK;
}

// Dense inverse of the variable-coefficient operator on an nc x nc grid
// (row-major (nc^2)^2) by Cholesky on the host.
int dense_inverse(int nc, const std::vector<double>& c, std::vector<double>& inv) {
  const int N = nc * nc;
  std::vector<double> A((size_t)N * N, 0.0);
  struct Acc {
    const double* c;
    int n;
    double operator()(int i, int j) const { return c[(size_t)j * n + i]; }
  } acc{c.data(), nc};
  auto at = [&](int r, int q) -> double& { return A[(size_t)r * N + q]; };
  for (int j = 0; j < nc; ++j)
    for (int i = 0; i < nc; ++i) {
      double e, nn, d;
      vc::coefficients(acc, i, j, nc, e, nn, d);
      const int k = j * nc + i;
      at(k, k) += d;   // A = -(-A)
      if (i < nc - 1) {
        at(k, k + 1) -= e;
        at(k + 1, k) -= e;
      }
      if (j < nc - 1) {
        at(k, k + nc) -= nn;
        at(k + nc, k) -= nn;
      }
      if (j == 0 && nc > 2) {
        const double f = vc::f_lo(acc(i, 0), i, nc);
        at(k, k + 2 * nc) -= f;
        at(k + 2 * nc, k) -= f;
      }
      if (j == nc - 1 && nc > 2) {
        const double f = vc::f_hi(acc(i, nc - 1), i, nc);
        at(k, k - 2 * nc) -= f;
        at(k - 2 * nc, k) -= f;
      }
    }
  // Cholesky A = L L^T in place (lower triangle)
  for (int q = 0; q < N; ++q) {
    double d = at(q, q);
    for (int k = 0; k < q; ++k) d -= at(q, k) * at(q, k);
    if (!(d > 0.0)) {
      set_last_error("coarse variable-coefficient operator is not positive definite");
      return SBP_ERR_ARGS;
    }
    const double lqq = std::sqrt(d);
    at(q, q) = lqq;
    for (int r = q + 1; r < N; ++r) {
      double v = at(r, q);
      const double* ar = &A[(size_t)r * N];
      const double* aq = &A[(size_t)q * N];
      for (int k = 0; k < q; ++k) v -= ar[k] * aq[k];
      at(r, q) = v / lqq;
    }
  }
  // columns of A^-1: forward and back substitution, in parallel
  inv.assign((size_t)N * N, 0.0);
  unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  auto worker = [&](unsigned t) {
    std::vector<double> y(N);
    for (int col = (int)t; col < N; col += (int)nt) {
      for (int r = 0; r < N; ++r) {   // L y = e_col
        double v = r == col ? 1.0 : 0.0;
        const double* ar = &A[(size_t)r * N];
        for (int k = col; k < r; ++k) v -= ar[k] * y[k];
        y[r] = r < col ? 0.0 : v / ar[r];
      }
      for (int r = N - 1; r >= 0; --r) {   // L^T x = y
        double v = y[r];
        for (int k = r + 1; k < N; ++k) v -= A[(size_t)k * N + r] * y[k];
        y[r] = v / A[(size_t)r * N + r];
      }
      for (int r = 0; r < N; ++r) inv[(size_t)r * N + col] = y[r];
    }
  };
  std::vector<std::thread> th;
  for (unsigned t = 1; t < nt; ++t) th.emplace_back(worker, t);
  worker(0);
  for (auto& t : th) t.join();
  for (int r = 0; r < N; ++r)   // exact symmetry
    for (int q = r + 1; q < N; ++q) {
      const double v = 0.5 * (inv[(size_t)r * N + q] + inv[(size_t)q * N + r]);
      inv[(size_t)r * N + q] = inv[(size_t)q * N + r] = v;
    }
  return SBP_OK;
}

// The variable-coefficient hierarchy: nodal c per level, stencil arrays, and
// the dense coarse inverse.
int build_variable(OpSolver* s, const double* c) {
  const int n = s->n;
  // the Jacobi weight, folded into the stored inverse diagonal
  const double jw = s->opts.omega > 0.0 ? s->opts.omega : 2.0 / 3.0;
  int rc = dalloc(s, &s->c0, (size_t)n * n);
  if (rc) return rc;
  SBP_CUDA(cudaMemcpy(s->c0, c, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToDevice));
  // level-0 FP64 stencil (the Krylov apply)
  for (int k = 0; k < 6; ++k) {
    rc = dalloc(s, &s->st64[k], (k < 3 || k == 5) ? (size_t)n * n : (size_t)n);
    if (rc) return rc;
  }
  SBP_CUDA(launch_vc_stencil<double>(s->c0, s->st64[0], s->st64[1], s->st64[2], s->st64[3],
                                     s->st64[4], s->st64[5], jw, n, nullptr));
  if (!s->mg) return SBP_OK;
  if (s->mixed) {   // the fused CG direction's coefficients
    for (int k = 0; k < 5; ++k) {
      const size_t cnt = k < 3 ? (size_t)n * n : (size_t)n;
      rc = dalloc(s, &s->pairs[k], cnt);
      if (rc) return rc;
      SBP_CUDA(launch_split_pairs(s->st64[k], s->pairs[k], (long long)cnt, nullptr));
    }
  }
  for (size_t l = 0; l < s->lv.size(); ++l) {
    auto& L = s->lv[l];
    const int m = L.n;
    if (l == 0) {
      L.c = s->c0;
    } else {
      rc = dalloc(s, &L.c, (size_t)m * m);
      if (rc) return rc;
      SBP_CUDA(launch_vc_coarsen(s->lv[l - 1].c, L.c, m, nullptr));
    }
    if (!s->mixed && l == 0) {
      for (int k = 0; k < 6; ++k) L.st[k] = s->st64[k];
      continue;
    }
    for (int k = 0; k < 6; ++k) {
      const size_t cnt = (k < 3 || k == 5) ? (size_t)m * m : (size_t)m;
      if (s->mixed) {
        float* p = nullptr;
        rc = dalloc(s, &p, cnt);
        if (rc) return rc;
        L.st[k] = p;
      } else {
        double* p = nullptr;
        rc = dalloc(s, &p, cnt);
        if (rc) return rc;
        L.st[k] = p;
      }
    }
    cudaError_t e;
    if (s->mixed)
      e = launch_vc_stencil<float>(L.c, as<float>(L.st[0]), as<float>(L.st[1]),
                                   as<float>(L.st[2]), as<float>(L.st[3]), as<float>(L.st[4]),
                                   as<float>(L.st[5]), jw, m, nullptr);
    else
      e = launch_vc_stencil<double>(L.c, as<double>(L.st[0]), as<double>(L.st[1]),
                                    as<double>(L.st[2]), as<double>(L.st[3]),
                                    as<double>(L.st[4]), as<double>(L.st[5]), jw, m, nullptr);
    SBP_CUDA(e);
  }
  // dense inverse of the coarsest operator
  const auto& C = s->lv.back();
  const int nc = C.n;
  std::vector<double> ch((size_t)nc * nc), inv;
  SBP_CUDA(cudaMemcpy(ch.data(), C.c, ch.size() * sizeof(double), cudaMemcpyDeviceToHost));
  rc = dense_inverse(nc, ch, inv);
  if (rc) return rc;
  s->ainv_n = nc * nc;
  rc = dalloc(s, &s->ainv, inv.size());
  if (rc) return rc;
  SBP_CUDA(cudaMemcpy(s->ainv, inv.data(), inv.size() * sizeof(double), cudaMemcpyHostToDevice));
  return SBP_OK;
}

int build_high_order(OpSolver* s) {
  if (!s->mg) return SBP_OK;
  const int nc = s->lv.back().n;
  std::shared_ptr<const CoarseFactors> F;
  try {
    F = coarse_factors(nc, s->p);
  } catch (const std::exception& ex) {
    set_last_error(ex.what());
    return SBP_ERR_ARGS;
  }
  const size_t mc = (size_t)nc * nc;
  const std::vector<double>* src[5] = {&F->Vx, &F->VxT, &F->Vy, &F->VyT, &F->dinv};
  double* dst[6];
  for (int k = 0; k < 6; ++k) {
    const int rc = dalloc(s, &dst[k], mc);
    if (rc) return rc;
    if (k < 5)
      SBP_CUDA(cudaMemcpy(dst[k], src[k]->data(), mc * sizeof(double), cudaMemcpyHostToDevice));
  }
  s->coarse = CoarseDev{dst[0], dst[1], dst[2], dst[3], dst[4], dst[5], nc};
  return SBP_OK;
}

int check_options(const sbp_options* opts, sbp_options& o) {
  sbp_options_default(&o);
  if (opts) o = *opts;
  if (o.precision != SBP_PREC_FP64 && o.precision != SBP_PREC_MIXED) return SBP_ERR_ARGS;
  if (o.nu_pre < 0 || o.nu_post < 0 || o.restriction < 0 || o.restriction > 2 ||
      (o.smoother != SBP_SMOOTH_JACOBI && o.smoother != SBP_SMOOTH_RICHARDSON))
    return SBP_ERR_ARGS;
  return SBP_OK;
}

void destroy(OpSolver* s) {
  cudaSetDevice(s->device);
  destroy_graphs(s);
  for (void* p : s->allocs) cudaFree(p);
  if (s->st_host) cudaFreeHost(s->st_host);
  if (s->cap) cudaStreamDestroy(s->cap);
  for (auto& e : s->ev)
    if (e) cudaEventDestroy(e);
}

}  // namespace

extern "C" {

// ---- higher order -----------------------------------------------------

int sbp_apply_ho_f64(const double* u, double* out, int n, int p, int sign, void* stream) {
  if (!u || !out || (sign != 1 && sign != -1) || ho_min_n(p) == 0 || n < ho_min_n(p))
    return SBP_ERR_ARGS;
  SBP_CUDA(prepare_ho_tables());
  HoArgs a = op_args(n);
  a.u = u;
  a.out = out;
  a.sign = sign;
  SBP_CUDA(launch_ho(p, kHoApply, a, (cudaStream_t)stream));
  return SBP_OK;
}

int sbp_ho_solver_create(sbp_ho_solver** out, int n, int p, const sbp_options* opts) {
  if (!out) return SBP_ERR_ARGS;
  *out = nullptr;
  if (ho_min_n(p) == 0 || n < ho_min_n(p)) return SBP_ERR_ARGS;
  sbp_options o;
  int rc = check_options(opts, o);
  if (rc) return rc;
  SBP_CUDA(prepare_ho_tables());
  std::unique_ptr<sbp_ho_solver> s(new (std::nothrow) sbp_ho_solver());
  if (!s) return SBP_ERR_NOMEM;
  s->kind = kOpHighOrder;
  s->p = p;
  std::vector<int> ns;
  rc = create_common(s.get(), n, o, 257, ho_min_n(p), ns);
  if (rc == SBP_OK) rc = build_high_order(s.get());
  if (rc == SBP_OK) {
    const cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) rc = fail_cuda(e, "sbp_ho_solver_create");
  }
  if (rc) {
    destroy(s.get());
    return rc;
  }
  *out = s.release();
  return SBP_OK;
}

int sbp_ho_solver_destroy(sbp_ho_solver* s) {
  if (!s) return SBP_OK;
  destroy(s);
  delete s;
  return SBP_OK;
}

int sbp_ho_solver_levels(const sbp_ho_solver* s) {
  if (!s) return SBP_ERR_ARGS;
  return s->mg ? (int)s->lv.size() : 0;
}

long long sbp_ho_solver_device_bytes(const sbp_ho_solver* s) { return s ? s->dev_bytes : 0; }

int sbp_ho_mgcg_solve(sbp_ho_solver* s, const double* b, double* x, double abstol, double reltol,
                      int maxiter, sbp_result* res, double* norms, int norms_cap, void* stream) {
  return solve(s, 0, b, x, 1, abstol, reltol, maxiter, res, norms, norms_cap,
               (cudaStream_t)stream);
}

int sbp_ho_cg_solve(sbp_ho_solver* s, const double* b, double* x, int sign, double abstol,
                    double reltol, int maxiter, sbp_result* res, double* norms, int norms_cap,
                    void* stream) {
  return solve(s, 1, b, x, sign, abstol, reltol, maxiter, res, norms, norms_cap,
               (cudaStream_t)stream);
}

int sbp_ho_vcycle_apply(sbp_ho_solver* s, const double* b, double* v, void* stream) {
  return vcycle_apply(s, b, v, (cudaStream_t)stream);
}

// ---- variable coefficients -------------------------------------------

int sbp_apply_vc_f64(const double* u, const double* c, double* out, int n, int sign,
                     void* stream) {
  if (!u || !c || !out || n < 3 || (sign != 1 && sign != -1)) return SBP_ERR_ARGS;
  SBP_CUDA(launch_vc_apply_c(u, c, out, n, sign, ReduceBuf{nullptr, nullptr}, nullptr,
                             (cudaStream_t)stream));
  return SBP_OK;
}

int sbp_vc_solver_create(sbp_vc_solver** out, int n, const double* c, const sbp_options* opts) {
  if (!out) return SBP_ERR_ARGS;
  *out = nullptr;
  if (!c || n < 3) return SBP_ERR_ARGS;
  sbp_options o;
  int rc = check_options(opts, o);
  if (rc) return rc;
  std::unique_ptr<sbp_vc_solver> s(new (std::nothrow) sbp_vc_solver());
  if (!s) return SBP_ERR_NOMEM;
  s->kind = kOpVariable;
  s->p = 2;
  std::vector<int> ns;
  rc = create_common(s.get(), n, o, kVcMaxCoarse, 3, ns);
  if (rc == SBP_OK) rc = build_variable(s.get(), c);
  if (rc == SBP_OK) {
    const cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) rc = fail_cuda(e, "sbp_vc_solver_create");
  }
  if (rc) {
    destroy(s.get());
    return rc;
  }
  *out = s.release();
  return SBP_OK;
}

int sbp_vc_solver_destroy(sbp_vc_solver* s) {
  if (!s) return SBP_OK;
  destroy(s);
  delete s;
  return SBP_OK;
}

int sbp_vc_solver_levels(const sbp_vc_solver* s) {
  if (!s) return SBP_ERR_ARGS;
  return s->mg ? (int)s->lv.size() : 0;
}

long long sbp_vc_solver_device_bytes(const sbp_vc_solver* s) { return s ? s->dev_bytes : 0; }

int sbp_vc_mgcg_solve(sbp_vc_solver* s, const double* b, double* x, double abstol, double reltol,
                      int maxiter, sbp_result* res, double* norms, int norms_cap, void* stream) {
  return solve(s, 0, b, x, 1, abstol, reltol, maxiter, res, norms, norms_cap,
               (cudaStream_t)stream);
}

int sbp_vc_cg_solve(sbp_vc_solver* s, const double* b, double* x, int sign, double abstol,
                    double reltol, int maxiter, sbp_result* res, double* norms, int norms_cap,
                    void* stream) {
  return solve(s, 1, b, x, sign, abstol, reltol, maxiter, res, norms, norms_cap,
               (cudaStream_t)stream);
}

int sbp_vc_vcycle_apply(sbp_vc_solver* s, const double* b, double* v, void* stream) {
  return vcycle_apply(s, b, v, (cudaStream_t)stream);
}

int sbp_vc_coarse_inverse_host(int nc, const double* c, double* out, long long cap) {
  if (nc < 3 || nc > kVcMaxCoarse || !c || !out) return SBP_ERR_ARGS;
  const long long N = (long long)nc * nc;
  if (cap < N * N) return SBP_ERR_ARGS;
  std::vector<double> ch(c, c + N), inv;
  const int rc = dense_inverse(nc, ch, inv);
  if (rc) return rc;
  std::copy(inv.begin(), inv.end(), out);
  return SBP_OK;
}

int sbp_vc_coarsen_host(int nc, const double* cf, double* cc) {
  if (nc < 1 || nc > (1 << 15) || !cf || !cc) return SBP_ERR_ARGS;
  for (int J = 0; J < nc; ++J)
    for (int I = 0; I < nc; ++I) cc[(size_t)J * nc + I] = vc::coarse_coefficient(cf, nc, I, J);
  return SBP_OK;
}

namespace {
void store9(const vc::Stencil9& s, size_t k, double* D, double* E, double* N, double* NE,
            double* NW) {
  D[k] = s.d;
  E[k] = s.e;
  N[k] = s.n;
  NE[k] = s.ne;
  NW[k] = s.nw;
}
}  // namespace

int sbp_vc_galerkin_coarse_host(int n, const double* c, double* D, double* E, double* N,
                                double* NE, double* NW) {
  if (n < 3 || n % 2 == 0 || n > (1 << 15) || !c || !D || !E || !N || !NE || !NW)
    return SBP_ERR_ARGS;
  struct Acc {
    const double* c;
    int n;
    double operator()(int i, int j) const { return c[(size_t)j * n + i]; }
  } acc{c, n};
  const vc::FineVc<Acc> A{acc, n};
  const int nc = (n + 1) / 2;
  double r[3][3];
  for (int J = 0; J < nc; ++J)
    for (int I = 0; I < nc; ++I) {
      vc::galerkin_row(A, nc, I, J, r);
      store9(vc::stencil9_of(r), (size_t)J * nc + I, D, E, N, NE, NW);
    }
  return SBP_OK;
}

int sbp_galerkin9_coarse_host(int n, const double* D, const double* E, const double* N,
                              const double* NE, const double* NW, double* Dc, double* Ec,
                              double* Nc, double* NEc, double* NWc) {
  if (n < 3 || n % 2 == 0 || n > (1 << 15) || !D || !E || !N || !NE || !NW || !Dc || !Ec ||
      !Nc || !NEc || !NWc)
    return SBP_ERR_ARGS;
  const vc::FineNine A{D, E, N, NE, NW, n};
  const int nc = (n + 1) / 2;
  double r[3][3];
  for (int J = 0; J < nc; ++J)
    for (int I = 0; I < nc; ++I) {
      vc::galerkin_row(A, nc, I, J, r);
      store9(vc::stencil9_of(r), (size_t)J * nc + I, Dc, Ec, Nc, NEc, NWc);
    }
  return SBP_OK;
}

int sbp_vc_assemble_host(int n, const double* c, long long* row_ptr, int* col, double* val,
                         long long cap, long long* nnz) {
  if (n < 3 || !c || !row_ptr || !nnz) return SBP_ERR_ARGS;
  struct Acc {
    const double* c;
    int n;
    double operator()(int i, int j) const { return c[(size_t)j * n + i]; }
  } acc{c, n};
  long long k = 0;
  row_ptr[0] = 0;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      // row (i, j) of A: the couplings of -A negated, in column order
      double e, nn, d;
      vc::coefficients(acc, i, j, n, e, nn, d);
      struct Entry {
        long long col;
        double v;
      } ent[10];
      int m = 0;
      auto coupling_n = [&](int jj) {   // N(i, jj)
        double e2, n2, d2;
        vc::coefficients(acc, i, jj, n, e2, n2, d2);
        return n2;
      };
      auto coupling_e = [&](int ii) {   // E(ii, j)
        double e2, n2, d2;
        vc::coefficients(acc, ii, j, n, e2, n2, d2);
        return e2;
      };
      const long long row = (long long)j * n + i;
      if (j == 2) ent[m++] = {row - 2LL * n, -vc::f_lo(acc(i, 0), i, n)};
      if (j == n - 1) ent[m++] = {row - 2LL * n, -vc::f_hi(acc(i, n - 1), i, n)};
      if (j > 0) ent[m++] = {row - n, -coupling_n(j - 1)};
      if (i > 0) ent[m++] = {row - 1, -coupling_e(i - 1)};
      ent[m++] = {row, d};
      if (i < n - 1) ent[m++] = {row + 1, -e};
      if (j < n - 1) ent[m++] = {row + n, -nn};
      if (j == 0 && n > 2) ent[m++] = {row + 2LL * n, -vc::f_lo(acc(i, 0), i, n)};
      if (j == n - 3 && n > 2) ent[m++] = {row + 2LL * n, -vc::f_hi(acc(i, n - 1), i, n)};
      // merge duplicates (n = 3: both end couplings land on the same pair)
      std::sort(ent, ent + m, [](const Entry& a, const Entry& b) { return a.col < b.col; });
      for (int q = 0; q < m; ++q) {
        if (q > 0 && ent[q].col == ent[q - 1].col) {
          if (k - 1 < cap && val) val[k - 1] += ent[q].v;
          continue;
        }
        if (k < cap && col && val) {
          col[k] = (int)ent[q].col;
          val[k] = ent[q].v;
        }
        ++k;
      }
      row_ptr[row + 1] = k;
    }
  *nnz = k;
  return k <= cap ? SBP_OK : SBP_ERR_ARGS;
}

}  // extern "C"

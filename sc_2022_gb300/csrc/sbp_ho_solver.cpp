// Higher-order (p = 4, 6) solver handles: matrix-free CG and multigrid-
// preconditioned CG on the order-p SBP-SAT operator, FP64.
//
// The reference solves these operators on the CPU: Assembling_matrix(level;
// p = SBPp) and the multigrid preconditioner precond_matrix(A, b; SBPp)
// (initial_guess_cg.jl:458-510).  That preconditioner uses weighted Jacobi
// (omega = 2/3, m = 3 sweeps), standard restriction and prolongation, and the
// re-discretised order-p coarse operator get_operators(SBPp, 2h).  Here the
// same V-cycle runs on the GPU over any number of levels:
// - each level re-discretises the order-p operator;
// - the smoother is Jacobi or Richardson;
// - the transfers are the second-order path's restriction and prolongation
//   kernels;
// - the coarse level is solved exactly by fast diagonalisation of the
//   order-p Kronecker sum.
// One (P)CG iteration is captured once as a CUDA graph. Its kernels read
// alpha and beta from a device SolveState and exit at once after
// convergence; the host checks the state one iteration behind.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <new>
#include <stdexcept>
#include <vector>

#include "../../include/sbpmg.h"
#include "sbp_coarse.h"
#include "sbp_host.h"
#include "sbp_launch.h"

using namespace sbp;

struct sbp_ho_solver {
  // Level buffers hold doubles, or floats for the mixed-precision V-cycle.
  struct Lvl {
    int n = 0;
    void* b = nullptr;   // level 0: the solver's r (FP64) or r_lo (mixed)
    void* v[2] = {nullptr, nullptr};
    void* t = nullptr;   // residual scratch
  };
  int n = 0, p = 0, device = 0;
  bool mg = false;
  bool mixed = false;
  float* r_lo = nullptr;   // mixed: FP32 copy of r, written by the update
  sbp_options opts{};
  std::vector<Lvl> lv;
  CoarseDev coarse{};
  double *x = nullptr, *r = nullptr, *pd = nullptr, *ap = nullptr;
  double* norms = nullptr;
  int norms_cap = 0;
  SolveState* st = nullptr;
  SolveState* st_host = nullptr;   // pinned, two slots
  ReduceBuf rb[3]{};
  cudaStream_t cap = nullptr;
  cudaGraphExec_t exec[2] = {nullptr, nullptr};   // kind 0: MGCG, 1: CG
  int exec_sign[2] = {0, 0};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  std::vector<void*> allocs;
  long long dev_bytes = 0;
};

namespace {

bool pow2_plus1(int n) {
  const int m = n - 1;
  return n >= 3 && (m & (m - 1)) == 0;
}

template <typename T>
int dalloc(sbp_ho_solver* s, T** out, size_t count) {
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
HoArgsT<T> ho_args(int n) {
  HoArgsT<T> a{};
  a.n = n;
  a.sign = 1;
  return a;
}

template <typename T>
T* as(void* p) {
  return static_cast<T*>(p);
}

// Smoothing sweeps on level L from v[cur]; returns the buffer index holding
// the result.  zero: start from v = 0.
template <typename T>
int smooth(sbp_ho_solver* s, const sbp_ho_solver::Lvl& L, int cur, int sweeps, bool zero,
           cudaStream_t q, cudaError_t& err) {
  const bool rich = s->opts.smoother == SBP_SMOOTH_RICHARDSON;
  const double omega = s->opts.omega > 0.0 ? s->opts.omega : (rich ? 0.15 : 2.0 / 3.0);
  for (int k = 0; k < sweeps && err == cudaSuccess; ++k) {
    HoArgsT<T> a = ho_args<T>(L.n);
    a.u = as<T>(L.v[cur]);
    a.b = as<T>(L.b);
    a.out = as<T>(L.v[1 - cur]);
    a.omega = omega;
    a.richardson = rich ? 1 : 0;
    a.zero_in = (zero && k == 0) ? 1 : 0;
    a.st = s->st;
    err = launch_ho(s->p, kHoJacobi, a, q);
    cur = 1 - cur;
  }
  return cur;
}

// One V-cycle from v = 0 on level l for the right-hand side lv[l].b; returns
// the buffer holding the result.  T: the V-cycle's arithmetic (the coarse
// solve computes in FP64 either way).
template <typename T>
T* vcycle(sbp_ho_solver* s, size_t l, cudaStream_t q, cudaError_t& err) {
  auto& L = s->lv[l];
  const int n = L.n;
  if (l + 1 == s->lv.size()) {
    err = launch_coarse_solve<T>(s->coarse, Grid<const T>{as<T>(L.b), n},
                                 Grid<T>{as<T>(L.v[0]), n}, s->st, q);
    return as<T>(L.v[0]);
  }
  int cur = 0;
  if (s->opts.nu_pre > 0) {
    cur = smooth<T>(s, L, 1, s->opts.nu_pre, true, q, err);
  } else {
    err = cudaMemsetAsync(L.v[0], 0, (size_t)n * n * sizeof(T), q);
  }
  if (err != cudaSuccess) return nullptr;
  HoArgsT<T> a = ho_args<T>(n);
  a.u = as<T>(L.v[cur]);
  a.b = as<T>(L.b);
  a.out = as<T>(L.t);
  a.st = s->st;
  err = launch_ho(s->p, kHoResid, a, q);
  if (err != cudaSuccess) return nullptr;
  auto& C = s->lv[l + 1];
  err = launch_resrestrict<T>(Grid<const T>{nullptr, 0}, Grid<const T>{as<T>(L.t), n},
                              Grid<T>{as<T>(C.b), C.n}, n, s->opts.restriction, s->st, q);
  if (err != cudaSuccess) return nullptr;
  T* e = vcycle<T>(s, l + 1, q, err);
  if (err != cudaSuccess) return nullptr;
  err = launch_prolong<T>(Grid<const T>{e, C.n}, Grid<T>{as<T>(L.v[cur]), n}, C.n, 1, s->st, q);
  if (err != cudaSuccess) return nullptr;
  cur = smooth<T>(s, L, cur, s->opts.nu_post, false, q, err);
  return as<T>(L.v[cur]);
}

// z = V(r), then beta = r.z / r.z_old and p = z + beta p (first: p = z).
template <typename T>
cudaError_t precondition(sbp_ho_solver* s, int first, cudaStream_t q) {
  cudaError_t err = cudaSuccess;
  const long long N = (long long)s->n * s->n;
  T* z = vcycle<T>(s, 0, q, err);
  if (err != cudaSuccess) return err;
  err = launch_ho_rz<T>(s->r, z, N, s->st, s->rb[2], first, q);
  if (err != cudaSuccess) return err;
  return launch_ho_dir<T>(z, s->pd, N, s->st, first, q);
}

// The iteration body: Ap and alpha, x/r update and ||r||^2, then the new
// direction (MGCG: z = V(r), beta = r.z / r.z_old; CG: beta from ||r||^2).
cudaError_t enqueue_iteration(sbp_ho_solver* s, int kind, int sign, cudaStream_t q) {
  const int n = s->n;
  const long long N = (long long)n * n;
  HoArgs a = ho_args(n);
  a.u = s->pd;
  a.out = s->ap;
  a.sign = sign;
  a.rb = s->rb[0];
  a.st = s->st;
  cudaError_t err = launch_ho(s->p, kHoApply, a, q);
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

void destroy_graphs(sbp_ho_solver* s) {
  for (auto& g : s->exec)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

int capture(sbp_ho_solver* s, int kind, int sign) {
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

int ensure_norms(sbp_ho_solver* s, int maxiter) {
  if (maxiter + 1 <= s->norms_cap) return SBP_OK;
  double* p = nullptr;
  const int cap = std::max(maxiter + 1, 1024);
  const int rc = dalloc(s, &p, (size_t)cap);
  if (rc) return rc;
  s->norms = p;   // the old array stays owned by allocs until destroy
  s->norms_cap = cap;
  destroy_graphs(s);
  return SBP_OK;
}

int solve(sbp_ho_solver* s, int kind, const double* b, double* x, int sign, double abstol,
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
  HoArgs a = ho_args(n);
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
  SBP_CUDA(launch_ho(s->p, kHoResid, a, q));
  if (kind == 1) {
    SBP_CUDA(launch_ho_dir<double>(s->r, s->pd, N, s->st, 1, q));
  } else if (s->mixed) {
    SBP_CUDA(launch_copy<double, float>(Grid<const double>{s->r, n}, Grid<float>{s->r_lo, n}, n,
                                        q));
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
  const SolveState fs = s->st_host[0];
  if (norms_out && norms_cap > 0) {
    const int cnt = std::min(norms_cap, fs.iter + 1);
    SBP_CUDA(cudaMemcpy(norms_out, s->norms, (size_t)cnt * sizeof(double),
                        cudaMemcpyDeviceToHost));
  }
  return finish_result(fs, res);
}

}  // namespace

extern "C" {

int sbp_apply_ho_f64(const double* u, double* out, int n, int p, int sign, void* stream) {
  if (!u || !out || (sign != 1 && sign != -1) || ho_min_n(p) == 0 || n < ho_min_n(p))
    return SBP_ERR_ARGS;
  SBP_CUDA(prepare_ho_tables());
  HoArgs a = ho_args(n);
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
  sbp_options_default(&o);
  if (opts) o = *opts;
  if (o.precision != SBP_PREC_FP64 && o.precision != SBP_PREC_MIXED) return SBP_ERR_ARGS;
  if (o.nu_pre < 0 || o.nu_post < 0 || o.restriction < 0 || o.restriction > 2 ||
      (o.smoother != SBP_SMOOTH_JACOBI && o.smoother != SBP_SMOOTH_RICHARDSON))
    return SBP_ERR_ARGS;
  SBP_CUDA(prepare_ho_tables());
  SBP_CUDA(prepare_kernels());
  std::unique_ptr<sbp_ho_solver> s(new (std::nothrow) sbp_ho_solver());
  if (!s) return SBP_ERR_NOMEM;
  struct Guard {
    std::unique_ptr<sbp_ho_solver>& s;
    ~Guard() {
      if (s) sbp_ho_solver_destroy(s.release());
    }
  } guard{s};
  SBP_CUDA(cudaGetDevice(&s->device));
  s->n = n;
  s->p = p;
  s->opts = o;
  s->mixed = o.precision == SBP_PREC_MIXED;
  const size_t esize = s->mixed ? sizeof(float) : sizeof(double);
  const size_t N = (size_t)n * n;
  int rc = 0;
  for (double** v : {&s->x, &s->r, &s->pd, &s->ap}) {
    rc = dalloc(s.get(), v, N);
    if (rc) return rc;
    SBP_CUDA(cudaMemset(*v, 0, N * sizeof(double)));
  }
  const size_t parts = (size_t)max_reduce_ctas(n);
  for (auto& rb : s->rb) {
    double* base = nullptr;
    rc = dalloc(s.get(), &base, parts + 32);
    if (rc) return rc;
    rb.partials = base;
    rb.ticket = reinterpret_cast<unsigned*>(base + parts);
    SBP_CUDA(cudaMemset(rb.ticket, 0, sizeof(unsigned)));
  }
  double* stp = nullptr;
  rc = dalloc(s.get(), &stp, 64);
  if (rc) return rc;
  s->st = reinterpret_cast<SolveState*>(stp);
  SBP_CUDA(cudaMallocHost((void**)&s->st_host, 2 * sizeof(SolveState)));
  SBP_CUDA(cudaStreamCreateWithFlags(&s->cap, cudaStreamNonBlocking));
  for (auto& e : s->ev) SBP_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  rc = ensure_norms(s.get(), 1023);
  if (rc) return rc;
  // multigrid hierarchy: n, (n+1)/2, ... down to coarse_n, or n alone (the
  // direct solve) when n <= min(coarse_n, 257).  Other grids get CG only.
  const int cn = o.coarse_n;
  const bool direct = n <= std::min(cn, 257);
  s->mg = direct || (pow2_plus1(n) && pow2_plus1(cn) && cn >= ho_min_n(p) && cn <= 257);
  if (s->mg) {
    if (s->mixed) {
      rc = dalloc(s.get(), &s->r_lo, N);
      if (rc) return rc;
    }
    int m = n;
    while (true) {
      sbp_ho_solver::Lvl L;
      L.n = m;
      const size_t M = (size_t)m * m * esize / sizeof(float);   // in floats
      float* buf = nullptr;
      if (s->lv.empty()) {
        L.b = s->mixed ? (void*)s->r_lo : (void*)s->r;
      } else {
        rc = dalloc(s.get(), &buf, M);
        if (rc) return rc;
        L.b = buf;
      }
      for (void** dst : {&L.v[0], &L.v[1], &L.t}) {
        rc = dalloc(s.get(), &buf, M);
        if (rc) return rc;
        *dst = buf;
      }
      s->lv.push_back(L);
      if (direct || m == cn) break;
      m = (m + 1) / 2;
    }
    const int nc = s->lv.back().n;
    std::shared_ptr<const CoarseFactors> F;
    try {
      F = coarse_factors(nc, p);
    } catch (const std::exception& ex) {
      set_last_error(ex.what());
      return SBP_ERR_ARGS;
    }
    const size_t mc = (size_t)nc * nc;
    const std::vector<double>* src[5] = {&F->Vx, &F->VxT, &F->Vy, &F->VyT, &F->dinv};
    double* dst[6];
    for (int k = 0; k < 6; ++k) {
      rc = dalloc(s.get(), &dst[k], mc);
      if (rc) return rc;
      if (k < 5)
        SBP_CUDA(cudaMemcpy(dst[k], src[k]->data(), mc * sizeof(double), cudaMemcpyHostToDevice));
    }
    s->coarse = CoarseDev{dst[0], dst[1], dst[2], dst[3], dst[4], dst[5], nc};
  }
  SBP_CUDA(cudaDeviceSynchronize());
  *out = s.release();
  return SBP_OK;
}

int sbp_ho_solver_destroy(sbp_ho_solver* s) {
  if (!s) return SBP_OK;
  cudaSetDevice(s->device);
  destroy_graphs(s);
  for (void* p : s->allocs) cudaFree(p);
  if (s->st_host) cudaFreeHost(s->st_host);
  if (s->cap) cudaStreamDestroy(s->cap);
  for (auto& e : s->ev)
    if (e) cudaEventDestroy(e);
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
  if (!s || !b || !v) return SBP_ERR_ARGS;
  if (!s->mg) return SBP_ERR_UNSUPPORTED;
  cudaStream_t q = (cudaStream_t)stream;
  SBP_CUDA(cudaSetDevice(s->device));
  const size_t bytes = (size_t)s->n * s->n * sizeof(double);
  // the V-cycle kernels exit early on a finished state: run it on a fresh one
  SBP_CUDA(launch_state_init(s->st, 1, q));
  SBP_CUDA(cudaMemcpyAsync(s->r, b, bytes, cudaMemcpyDeviceToDevice, q));
  cudaError_t err = cudaSuccess;
  const int n = s->n;
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
  return SBP_OK;
}

}  // extern "C"

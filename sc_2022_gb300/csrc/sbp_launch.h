// Host-side launch wrappers for the SBP-SAT kernels (defined in
// sbp_kernels.cu).  All launches are asynchronous on `s`; none allocates.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "sbp_common.cuh"
#include "sbp_tma.h"

namespace sbp {

// Operand-based launchers (TMA staging when the operands allow it).  The
// Grid-based launchers below use element-wise cp.async staging and accept any
// leading dimension.
template <typename T>
// With xcopy set, x is also written into xcopy (one pass instead of a copy
// followed by the residual).
cudaError_t launch_residual_op(const Operand& x, const Operand& b, Grid<T> r, Grid<float> rlo,
                               int n, int opsign, SolveState* st, double* norms, double abstol,
                               double reltol, int plain, double* out2, ReduceBuf rb,
                               cudaStream_t s, Grid<T> xcopy = Grid<T>{nullptr, 0});
template <typename T, typename Tz>
cudaError_t launch_cg_dir_op(const Operand& z, const Operand& pold, Grid<T> pnew, Grid<T> Ap,
                             int n, int opsign, SolveState* st, ReduceBuf rb, cudaStream_t s);
// Mixed-precision CG direction kept in FP32: p~ = fl32(z + beta p~_old),
// Ap = A p~ exactly (float-float stencil), p~.Ap -> alpha.  On odd grids
// from N = 1025 with padded arrays (ld > n) one register-wave launch covers
// the interior and, in extra CTAs, the SAT rows and columns; elsewhere z and
// p~_old are staged tile by tile (TMA when both allow it).
cudaError_t launch_cg_dir_f32(const Operand& z, const Operand& pold, Grid<float> pnew,
                              Grid<double> Ap, int n, SolveState* st, ReduceBuf rb,
                              cudaStream_t s);
template <typename T>
cudaError_t launch_smooth_op(int field, int epi, const Operand& vin, const Operand& e,
                             const Operand& b, Grid<T> vout, int n, int smoother, double omega,
                             int dot, SolveState* st, ReduceBuf rb, cudaStream_t s);
// Fused V-cycle passes (temporal blocking, sweeps <= 3): pre-smoothing from
// zero + residual + restriction into f, and prolongation + post-smoothing.
template <typename T>
// With aux, fork and join given, a level whose interior runs the register
// wave does its boundary tiles on `aux` concurrently (fork recorded on s,
// join waited on by s).
cudaError_t launch_pre_fused(const Operand& b, Grid<T> vout, Grid<T> f, int nf, int sweeps,
                             int smoother, double omega, int kind, const SolveState* st,
                             cudaStream_t s, cudaStream_t aux = nullptr,
                             cudaEvent_t fork = nullptr, cudaEvent_t join = nullptr);
// FP32 levels from N = 1025 with three sweeps: the boundary ring (one small
// tile deep) by the staged job (forked onto `aux` when aux/fork/join are
// given), the interior by the register wave kernel; with the dot, the two
// shares of r.z meet in a fixed order.
template <typename T>
cudaError_t launch_post_fused(const Operand& vin, const Operand& e, const Operand& b, Grid<T> vout,
                              int n, int sweeps, int smoother, double omega, int dot,
                              SolveState* st, ReduceBuf rb, cudaStream_t s,
                              cudaStream_t aux = nullptr, cudaEvent_t fork = nullptr,
                              cudaEvent_t join = nullptr);
template <typename T>
cudaError_t launch_resrestrict_op(const Operand* v, const Operand& b, Grid<T> f, int nf, int kind,
                                  const SolveState* st, cudaStream_t s);

// Allocation-free apply + dot with the reduction scratch in a static device
// array (see sbp_apply_dot_f64_noalloc in sbpmg.h).  Returns 0 or a negative
// sbp_status value; on a CUDA error (-2) *err holds the error that caused it.
int apply_dot_f64_noalloc(const double* u, double* out, int n, int sign, double* dot,
                          cudaStream_t s, cudaError_t* err);

// FP64 FMA lane-operations per second of the current GPU (in units of 1e9),
// timed with CUDA events on s (blocking).
cudaError_t measure_fp64_fma_rate(double* gfma_per_s, cudaStream_t s);

// Kernel launches of one launch_pre_fused call on a solver level (the
// interior of the FP32 levels from N = 1025 takes a second, register-wave
// kernel).
int pre_fused_launches(int nf, int sweeps, bool f32);
// The same for launch_post_fused.
int post_fused_launches(int n, int sweeps, bool f32);

// Non-zero once a kernel's bounded wait on an asynchronous copy gave up.
unsigned int read_device_fault();
// The same, clearing the flag (the current device's copy).
unsigned int take_device_fault();
// Failure test switch: drop = 1 makes CTA 0 of every persistent launch skip
// its first TMA copy (its wait then runs out after `polls` try_wait polls);
// drop = 0, polls = 0 restores normal operation.
cudaError_t set_copy_drop(int drop, unsigned polls);
// out[k] = -(hi[k] + lo[k]) in FP64 by the direction pass's conversion
// (test hook).
cudaError_t launch_pair_to_f64(const float* hi, const float* lo, double* out, long long n,
                               cudaStream_t s);

// Upper bound on the CTAs any reducing launch uses for an n x n grid; the
// partials buffer of a ReduceBuf must hold this many doubles.
int max_reduce_ctas(int n);

// out = sign * (-A) u.  If dot_out != nullptr also writes sum(u .* out)
// to *dot_out (device), using `rb` as scratch.
template <typename T>
cudaError_t launch_apply(Grid<const T> u, Grid<T> out, int n, int sign, ReduceBuf rb,
                         double* dot_out, cudaStream_t s);

// r = b - opsign*A*x (and rlo = float(r) if rlo.p); sum(r.*r) goes to
// *out2 (if non-null) and, if st != nullptr, initialises the Krylov state:
// rr0, rr, thresh2 (abstol^2 if abstol > 0 else reltol^2*rr0), norms[0],
// iter = 0, done, and rz = rr0 when `plain`.
template <typename T>
cudaError_t launch_residual(Grid<const T> x, Grid<const T> b, Grid<T> r, Grid<float> rlo, int n,
                            int opsign, SolveState* st, double* norms, double abstol,
                            double reltol, int plain, double* out2, ReduceBuf rb,
                            cudaStream_t s);

// p_new = z + beta*p_old (p_new = z on the first iteration), Ap = opsign*A*p_new,
// pAp = p_new.Ap, alpha = rz / pAp.
template <typename T, typename Tz>
cudaError_t launch_cg_dir(Grid<const Tz> z, Grid<const T> pold, Grid<T> pnew, Grid<T> Ap, int n,
                          int opsign, SolveState* st, ReduceBuf rb, cudaStream_t s);

// x += alpha p, r -= alpha Ap, rlo = float(r) (if rlo.p), rr = r.r,
// iter += 1, norms[iter] = sqrt(rr), convergence / max-iteration test.
// `plain`: unpreconditioned CG, also beta = rr/rz and rz = rr.
// pf (optional): an FP32 direction used in place of p (p is then ignored).
template <typename T>
cudaError_t launch_cg_update(Grid<T> x, Grid<T> r, Grid<const T> p, Grid<const T> Ap,
                             Grid<float> rlo, int n, int plain, SolveState* st, double* norms,
                             ReduceBuf rb, cudaStream_t s, const float* pf = nullptr);

// One smoothing pass on level n.  The stencil input ("field") is
//   kFieldPlain:   vin
//   kFieldZero:    the first sweep from v = 0 (omega D^-1 b or omega b)
//   kFieldProlong: vin + P e  (e on the (n+1)/2 grid)
// and the output is vout = F + omega M (b - A F) (sweep) or vout = F (store),
// M = D^-1 (Jacobi) or I (Richardson).  With dot != 0 the pass also reduces
// b.vout into the Krylov state: beta = b.vout / rz (after the first
// iteration), rz = b.vout.
enum FieldKind : int { kFieldPlain = 0, kFieldZero = 1, kFieldProlong = 2 };
enum EpiKind : int { kEpiSweep = 0, kEpiStore = 1 };
template <typename T>
cudaError_t launch_smooth(int field, int epi, Grid<const T> vin, Grid<const T> e, Grid<const T> b,
                          Grid<T> vout, int n, int smoother, double omega, int dot,
                          SolveState* st, ReduceBuf rb, cudaStream_t s);

// f = R (b - A v) on the (nf+1)/2 grid (v == nullptr: f = R b).
template <typename T>
cudaError_t launch_resrestrict(Grid<const T> v, Grid<const T> b, Grid<T> f, int nf, int kind,
                               const SolveState* st, cudaStream_t s);

// out = P e  (accumulate: out += P e), e on nc x nc, out on (2nc-1)^2.
template <typename T>
cudaError_t launch_prolong(Grid<const T> e, Grid<T> out, int nc, int accumulate,
                           const SolveState* st, cudaStream_t s);

// Device copy of the coarse fast-diagonalisation factors (all nc x nc,
// column-major, FP64) plus an nc x nc FP64 scratch grid y.
struct CoarseDev {
  const double* Vx;
  const double* VxT;
  const double* Vy;
  const double* VyT;
  const double* dinv;
  double* y;
  int nc;
};

// e = A^{-1} f on the coarse grid (FP64 arithmetic regardless of T); two
// launches.
template <typename T>
cudaError_t launch_coarse_solve(const CoarseDev& f, Grid<const T> b, Grid<T> e,
                                const SolveState* st, cudaStream_t s);

// out = convert(in) on an n x n grid (any leading dimensions).
template <typename Tin, typename Tout>
cudaError_t launch_copy(Grid<const Tin> in, Grid<Tout> out, int n, cudaStream_t s);

// Resolve the launch configuration of every persistent kernel on the current
// device; call once outside stream capture (solver creation does).
cudaError_t prepare_kernels();

// Krylov state reset (iter = done = 0, maxiter) before a solve.
cudaError_t launch_state_init(SolveState* st, int maxiter, cudaStream_t s);

// b = -H~ (fsign*f + SAT_W gW + SAT_E gE + SAT_S gS + SAT_N gN), the right-hand
// side of Assembling_matrix (level_2_multigrid_new.jl:169-185) with f in
// the Delta u = f convention times fsign.
cudaError_t launch_rhs(Grid<const double> f, const double* gW, const double* gE,
                       const double* gS, const double* gN, Grid<double> b, int n, double fsign,
                       cudaStream_t s);

// Transpose of launch_rhs's linear map applied to lambda: gradients of
// lambda.b with respect to f and the four boundary vectors.
cudaError_t launch_rhs_adjoint(Grid<const double> lam, Grid<double> df, double* dgW, double* dgE,
                               double* dgS, double* dgN, int n, double fsign, cudaStream_t s);

// ---------------------------------------------------------------------------
// Launch recording for batched solves.  While a Recorder is installed on the
// calling host thread, the solver's launchers (persistent jobs, the CG
// update, the coarse-solve passes, the state initialisation and grid copies)
// append a LaunchRecord instead of launching.  Records of several problems
// that agree in `fn` and `aux` are launched together as one batched kernel:
// fn(blobs, stride, count, aux, scratch, stream) with `count` argument blobs
// (one per problem, `stride` bytes apart) in device memory.  count == 0 only
// resolves the launch configuration (occupancy, shared-memory attribute);
// do that once outside stream capture.
// ---------------------------------------------------------------------------
struct BatchScratch {
  double* partials = nullptr;   // per-CTA, per-problem partial sums
  unsigned* ticket = nullptr;   // zero between launches
  long long cap = 0;            // doubles in partials
  int cta_budget = 0;           // most CTAs of a batched persistent launch (0: one full wave)
};
using BatchLaunchFn = cudaError_t (*)(const unsigned char* blobs, int stride, int count,
                                      const int* aux, const BatchScratch& scr, cudaStream_t s);
struct LaunchRecord {
  BatchLaunchFn fn = nullptr;
  int aux[4] = {0, 0, 0, 0};     // launch shape; equal within a batched group
  int align = 16;                // alignment of the argument blob in device memory
  std::vector<unsigned char> blob;
};
struct Recorder {
  std::vector<LaunchRecord> recs;
};
// The calling thread's recorder (nullptr: launch normally).
Recorder*& recorder_slot();

// Per-launch CUDA-event timing (sbp_solver_profile): installed through
// timer_slot() (sbp_kernels.cuh), filled by launch_pdl.
struct LaunchTimer {
  struct Rec {
    const void* fn = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
  };
  std::vector<Rec> recs;
  bool failed = false;
};
LaunchTimer*& timer_slot();
// Most problems one batched launch can carry (per-CTA partials live in
// shared memory).
constexpr int kMaxBatchSlots = 512;
// Largest grid of a persistent kernel (one wave: SMs x resident CTAs).
constexpr int kMaxPersistCtas = 4096;

// Streaming multiprocessors of the current device.
int batch_sm_count();

// dst (ld dld) = src (ld sld) on an n x n FP64 grid; recordable.
cudaError_t copy_grid(double* dst, int dld, const double* src, int sld, int n, cudaStream_t s);


// ---- higher-order (p = 4, 6) operators, FP64, contiguous n x n grids ----
enum { kHoApply = 0, kHoResid = 1, kHoJacobi = 2 };
template <typename T>
struct HoArgsT {
  const T* u;          // operator input (unused by a Jacobi sweep with zero_in)
  const T* b;          // right-hand side (residual, Jacobi)
  T* out;
  int n;
  int sign;            // apply: out = sign * A u; residual: out = b - sign * A u
  double omega;        // smoother weight
  int richardson;      // smoother: out = u + omega (b - A u) instead of Jacobi
  int zero_in;         // smoother from u = 0: out = omega D^-1 b
  int cols;            // columns per work item (0: chosen by the launcher)
  ReduceBuf rb;        // non-null partials: reduce (apply: u . out, residual: ||out||^2)
  double* dot_out;     // the reduction, if non-null
  SolveState* st;      // kernels exit at once when st->done; apply: p.Ap -> alpha
  int init;            // residual with st: set up the Krylov state from ||r0||^2
  double abstol, reltol;
  double* norms;       // init: norms[0] = ||r0||
};
using HoArgs = HoArgsT<double>;
// The variable-coefficient kernels take the same arguments plus the level's
// stencil arrays (sbp_varcoef.cuh).
template <typename T>
struct VcArgsT : HoArgsT<T> {
  const T* E;
  const T* N;
  const T* D;
  const T* flo;
  const T* fhi;
  const T* Dinv;   // omega / D (Jacobi sweeps)
};
// Smallest grid of order p (0 if p is not 4 or 6).
int ho_min_n(int p);
// Upload the closure tables once (outside stream capture).
cudaError_t prepare_ho_tables();
// T = double (FP64 arithmetic) or float (FP32 arithmetic, the mixed V-cycle).
template <typename T>
cudaError_t launch_ho(int p, int mode, HoArgsT<T> a, cudaStream_t s);
// r.z -> beta (0 when first) and rz in the state; p = z + beta p (p = z
// when first).  Tz = double or float (the mixed V-cycle's z).
template <typename Tz>
cudaError_t launch_ho_rz(const double* r, const Tz* z, long long N, SolveState* st,
                         ReduceBuf rb, int first, cudaStream_t s);
template <typename Tz>
cudaError_t launch_ho_dir(const Tz* z, double* p, long long N, const SolveState* st,
                          int first, cudaStream_t s);
// Mixed-precision order-p CG direction, in place: p = z + beta p,
// Ap = A z + beta Ap (A z on the FP32 pipe), p.Ap -> alpha; the first
// direction (state iteration 0) takes p = z, Ap = A z.
cudaError_t launch_ho_dir_mixed(int p, const float* z, double* pd, double* ap, int n,
                                SolveState* st, ReduceBuf rb, cudaStream_t s);

// ---- variable-coefficient operator (sbp_varcoef.cuh), contiguous grids ----
// out = sign * A u straight from the nodal coefficients c (FP64; dot_out: u . out).
cudaError_t launch_vc_apply_c(const double* u, const double* c, double* out, int n, int sign,
                              ReduceBuf rb, double* dot_out, cudaStream_t s);
// The level's stencil arrays from its nodal coefficients; Dinv = wscale / D
// (the Jacobi weight over the diagonal).
template <typename T>
cudaError_t launch_vc_stencil(const double* c, T* E, T* N, T* D, T* flo, T* fhi, T* Dinv,
                              double wscale, int n, cudaStream_t s);
// Coarse nodal coefficients (nc x nc) of the fine field cf ((2nc-1)^2): the
// harmonic mean of cf over the full-weighting stencil of (2I, 2J).
cudaError_t launch_vc_coarsen(const double* cf, double* cc, int nc, cudaStream_t s);
// Apply / residual / smoother on the stencil arrays (modes as launch_ho).
template <typename T>
cudaError_t launch_vc(int mode, VcArgsT<T> a, cudaStream_t s);
// FP64 values as float pairs (hi = nearest float, lo = the remainder's).
cudaError_t launch_split_pairs(const double* in, float2* out, long long count, cudaStream_t s);
// Mixed-precision CG direction of the variable-coefficient operator, in
// place: p = z + beta p, Ap = A z + beta Ap (A z in float-float from the
// level-0 stencil as float pairs st = {E, N, D, flo, fhi}), p.Ap -> alpha;
// the first direction (state iteration 0) takes p = z, Ap = A z.
cudaError_t launch_vc_dir_mixed(const float* z, const float2* const* st, double* pd, double* ap,
                                int n, SolveState* state, ReduceBuf rb, cudaStream_t s);
// x = Ainv b with a dense FP64 N x N inverse (row-major).
template <typename T>
cudaError_t launch_dense_gemv(const double* Ainv, const T* b, T* x, int N, const SolveState* st,
                              cudaStream_t s);

// y = A x for a CSR matrix with nrows rows (64-bit row pointers).
cudaError_t launch_csr_spmv(long long nrows, const long long* row_ptr, const int* col,
                            const double* val, const double* x, double* y, cudaStream_t s);

// g = H~ (u - ut) (g.p may be null) and *loss = 1/2 (u - ut)' H~ (u - ut)
// (loss may be null); H~ = h^2 diag(w_i w_j).
cudaError_t launch_h_misfit(Grid<const double> u, Grid<const double> ut, Grid<double> g, int n,
                            double* loss, ReduceBuf rb, cudaStream_t s);

}  // namespace sbp

/*
 * sbpmg.h - C ABI of libsbpmg, a GB300 (sm_103a) matrix-free SBP-SAT 2D
 * Poisson solver: operator apply, matrix-free CG, and geometric-multigrid
 * preconditioned CG (MGCG), in FP64 and in mixed precision.
 *
 * It replaces the GPU entry points of AlexandreChern/SC_2022 (Julia +
 * CUDA.jl).  Each declaration names the reference function it stands in for
 * (path:line inside that repository).
 *
 * Conventions
 *  - Grid functions are column-major n x n double (or float) arrays in
 *    device memory: point (i, j) at p[j*n + i], i the fast index (x), exactly
 *    the CuArray{Float64,2} layout of the reference.  n = 2^k + 1 for the
 *    multigrid entry points; any n >= 3 for the single-grid ones.
 *  - A is the SPD operator of the reference's Assembling_matrix
 *    (preconditioned_CG/level_2_multigrid_new.jl:125-188):
 *    A = -H~ (D2 + SAT_W + SAT_E + SAT_S + SAT_N), 2nd-order SBP, Dirichlet
 *    SAT on the j = 0 / n-1 sides (tau = -13/h, beta = 1), Neumann SAT on the
 *    i = 0 / n-1 sides (tau = -1).
 *  - Callers own inputs and outputs.  Solver handles own all temporaries.
 *  - `stream` is a cudaStream_t (NULL = legacy default stream).  Calls are
 *    stream ordered; the solve entry points return after the solve finished.
 *  - Every function returns 0 (SBP_OK) or a negative sbp_status; no
 *    exceptions cross the ABI.  A handle may be used by one host thread at a
 *    time.
 *  - Kernels that wait on asynchronous copies wait a bounded time.  If a
 *    wait gives up, the kernel ends (its results are non-finite) and sets a
 *    device flag; the next call that waits for the GPU (the solve entry
 *    points, sbp_residual_norm_f64) reads and clears it and returns
 *    SBP_ERR_TIMEOUT.
 */
#ifndef SBPMG_H_
#define SBPMG_H_

#ifdef __cplusplus
extern "C" {
#endif

typedef enum sbp_status {
  SBP_OK = 0,
  SBP_ERR_ARGS = -1,        /* invalid argument (size, null pointer, option) */
  SBP_ERR_CUDA = -2,        /* a CUDA runtime call failed */
  SBP_ERR_NOMEM = -3,       /* device or host allocation failed */
  SBP_ERR_MAXITER = -4,     /* solver stopped at maxiter without converging */
  SBP_ERR_BREAKDOWN = -5,   /* p'Ap == 0 or a non-finite residual */
  SBP_ERR_UNSUPPORTED = -6, /* option combination not supported */
  SBP_ERR_TIMEOUT = -7      /* a kernel's bounded wait on an asynchronous copy gave up: the
                               call's results are void; the library stays usable */
} sbp_status;

typedef enum sbp_smoother { SBP_SMOOTH_JACOBI = 0, SBP_SMOOTH_RICHARDSON = 1 } sbp_smoother;

/* Residual restriction on the multigrid hierarchy.
 * NORMAL:   full weighting with zero padding, restriction_matrix_normal
 *           (level_2_multigrid_new.jl:220-233); what the reference's GPU
 *           restriction kernel computes (matrix_free_mg_cg.jl:98-131).
 * SBP:      kron of the SBP-preserving restriction_matrix (:205-218).
 * GALERKIN: P^T, the SBP-compatible restriction H2h^-1 P^T Hh re-expressed
 *           for the H~-scaled residuals of this operator (= 4 x NORMAL). */
typedef enum sbp_restriction {
  SBP_RESTRICT_NORMAL = 0,
  SBP_RESTRICT_SBP = 1,
  SBP_RESTRICT_GALERKIN = 2
} sbp_restriction;

typedef enum sbp_precision {
  SBP_PREC_FP64 = 0,  /* everything in FP64 */
  SBP_PREC_MIXED = 1  /* FP32 V-cycle (apply, smoother, transfers) inside
                         FP64 PCG; FP64 residual, update, dots, coarse solve */
} sbp_precision;

typedef struct sbp_options {
  int smoother;     /* sbp_smoother */
  double omega;     /* smoother weight (0 = default: 2/3 Jacobi, 0.15 Richardson) */
  int nu_pre;       /* pre-smoothing sweeps */
  int nu_post;      /* post-smoothing sweeps */
  int restriction;  /* sbp_restriction */
  int coarse_n;     /* grid size of the direct coarse solve (<= 1025) */
  int precision;    /* sbp_precision */
  int reserved[5];
} sbp_options;

typedef struct sbp_result {
  int iters;           /* completed (P)CG iterations */
  int status;          /* 0 converged, or SBP_ERR_MAXITER / SBP_ERR_BREAKDOWN */
  double initial_norm; /* ||b - A x0||_2 */
  double final_norm;   /* ||r||_2 of the last iterate (recurrence residual) */
  double threshold;    /* the absolute stopping threshold used */
} sbp_result;

typedef struct sbp_solver sbp_solver;

/* Library version (major*10000 + minor*100 + patch). */
int sbp_version(void);
const char* sbp_status_string(int status);

/* Default options: the V-cycle preconditioner of the N=4097 benchmark
 * configuration: Jacobi omega = 2/3, 3 + 3 sweeps, GALERKIN restriction,
 * coarse direct solve at 65 x 65, FP64. */
void sbp_options_default(sbp_options* opts);

/* The reference's own two-level GPU preconditioner
 * (matrix_free_Two_level_multigrid, matrix_free_mg_cg.jl:143-176):
 * Richardson omega = 0.15, nu = 3 + 3, NORMAL restriction, exact coarse
 * solve at (n+1)/2.  Requires (n+1)/2 <= 1025 (n <= 2049); coarse grids
 * above 257 compute their eigenbases on the GPU at handle creation. */
void sbp_options_reference_two_level(sbp_options* opts, int n);

/* ---- single-grid operators (no handle) ------------------------------- */

/* out = sign * A * u, sign = -1 reproduces the reference's
 * matrix_free_A_full_GPU(idata, odata), which writes -A*idata
 * (split_matrix_free.jl:444-486). */
int sbp_apply_f64(const double* u, double* out, int n, int sign, void* stream);
int sbp_apply_f32(const float* u, float* out, int n, int sign, void* stream);

/* out = sign*A*u and *dot = sum(u .* out) (device pointer) in one pass: the
 * fused operator + p'Ap of the CG loop (split_matrix_free.jl:665-666,
 * matrix_free_mg_cg.jl:303-304).  Uses stream-ordered scratch
 * (cudaMallocAsync) for the per-CTA partial sums. */
int sbp_apply_dot_f64(const double* u, double* out, int n, int sign, double* dot,
                      void* stream);

/* Same result as sbp_apply_dot_f64, but the call allocates nothing.  It is
 * for callers that cannot let a library allocate device memory on their
 * behalf: hosts whose device memory is owned by their own allocator or pool
 * (a language runtime's managed heap, a fixed memory budget) and
 * latency-critical loops that must not enter the CUDA allocator.  No
 * counterpart in the reference.
 *
 * The per-CTA partial sums of the dot product live in a static device
 * array of the library: 1024 slots of 8 bytes plus a counter, about 8 KB,
 * resident on every GPU that has used it until the process exits.  A launch
 * needing more than 1024 CTAs is rejected with SBP_ERR_UNSUPPORTED (a
 * 152-SM GB300 uses 760).  The first call on a device resolves the array's
 * device address (cudaGetSymbolAddress) and caches it; make that first call
 * before any stream capture.  Every call uses the same array: calls that
 * may run concurrently on the GPU (different streams without ordering) race
 * on it, so order them.  The counter is cleared at the start of each call;
 * the partial slots are fully rewritten by every launch. */
int sbp_apply_dot_f64_noalloc(const double* u, double* out, int n, int sign, double* dot,
                              void* stream);

/* *norm_host = ||b - sign*A*x||_2 (blocking).  The reference's residual
 * check norm(-Av - b) (matrix_free_mg_cg.jl:175). */
int sbp_residual_norm_f64(const double* x, const double* b, int n, int sign, double* norm_host,
                          void* stream);

/* coarse = R fine, fine n_fine x n_fine, coarse (n_fine+1)/2 squared, R one
 * of sbp_restriction.  SBP_RESTRICT_NORMAL reproduces
 * matrix_free_restriction_2d_GPU (matrix_free_mg_cg.jl:120-131). */
int sbp_restrict_f64(const double* fine, double* coarse, int n_fine, int kind, void* stream);

/* fine = P coarse (accumulate != 0: fine += P coarse), bilinear, coarse
 * n_coarse^2 -> fine (2 n_coarse - 1)^2.  matrix_free_prolongation_2d_GPU
 * (matrix_free_mg_cg.jl:69-77). */
int sbp_prolong_f64(const double* coarse, double* fine, int n_coarse, int accumulate,
                    void* stream);

/* `iters` Richardson sweeps v <- v + omega (b - A v) on the caller's v,
 * using `tmp` (n x n) as the second buffer; on return v and tmp both hold
 * the result.  matrix_free_richardson(idata, odata, b; maxiter, omega)
 * (matrix_free_mg_cg.jl:134-140), which mutates both arrays. */
int sbp_richardson_f64(double* v, double* tmp, const double* b, int n, int iters, double omega,
                       void* stream);

/* Weighted Jacobi v <- v + omega D^-1 (b - A v), `iters` sweeps, same
 * buffer contract (jacobi_brittany!, level_2_multigrid_new.jl:335-344). */
int sbp_jacobi_f64(double* v, double* tmp, const double* b, int n, int iters, double omega,
                   void* stream);

/* b = -H~ (fsign*f + SAT_W_r gW + SAT_E_r gE + SAT_S_r gS + SAT_N_r gN): the
 * right-hand side of Assembling_matrix (level_2_multigrid_new.jl:169-185).
 * f is n x n in the D2 convention (Delta u = f) times fsign (fsign = -1 for
 * -Delta u = f); gW/gE are the Dirichlet data along j = 0 / n-1 (indexed by
 * i), gS/gN the outward normal derivatives along i = 0 / n-1 (indexed by j). */
int sbp_rhs_f64(const double* f, const double* gW, const double* gE, const double* gS,
                const double* gN, double* b, int n, double fsign, void* stream);

/* Transpose of sbp_rhs_f64's map: given lam (n x n), writes df (n x n) and
 * dgW, dgE, dgS, dgN (length n) with lam.b = df.f + sum dg_side.g_side.
 * Any output may be NULL.  No reference counterpart: the adjoint path is
 * new. */
int sbp_rhs_adjoint_f64(const double* lam, double* df, double* dgW, double* dgE, double* dgS,
                        double* dgN, int n, double fsign, void* stream);

/* The H-norm misfit of the adjoint configuration: g = H~ (u - ut) and
 * *loss = 1/2 (u - ut)' H~ (u - ut) with H~ = h^2 diag(w_i w_j), w = 1/2 on
 * the first and last index (the H~ of Assembling_matrix,
 * level_2_multigrid_new.jl:119).  g (n x n) and loss (one double in device
 * memory) may each be NULL, not both.  Stream-ordered.  No reference
 * counterpart: the adjoint path is new. */
int sbp_h_misfit_f64(const double* u, const double* ut, double* g, int n, double* loss,
                     void* stream);

/* ---- higher-order operators (p = 4, 6) ------------------------------- */

/* The order-p diagonal-norm SBP-SAT operator of Operators_2d(...; p) /
 * Assembling_matrix(level; p) (level_2_multigrid_new.jl:48-188 with the
 * p == 4 and p == 6 branches of diagonal_sbp.jl:62-79, 198-222):
 * - interior D2 stencils (-1/12, 4/3, -5/2, 4/3, -1/12) for p = 4 and
 *   (1/90, -3/20, 3/2, -49/18, ...) for p = 6;
 * - 4 x 6 and 6 x 9 boundary closures;
 * - the same SAT penalties as p = 2.
 * The reference assembles these on the CPU only; its GPU kernels are
 * second order.  Arrays are contiguous FP64 n x n device grids (ld = n),
 * n >= 8 (p = 4) or 12 (p = 6). */
int sbp_apply_ho_f64(const double* u, double* out, int n, int p, int sign, void* stream);

/* Order-p solver handle.  opts (NULL = sbp_options_default) must be FP64;
 * the V-cycle re-discretises the order-p operator on every level.  It
 * smooths with the chosen Jacobi or Richardson sweeps, uses the chosen
 * restriction and bilinear prolongation, and solves the coarse level
 * exactly by fast diagonalisation.  This is precond_matrix(A, b; SBPp)
 * (initial_guess_cg.jl:458-510) over any number of levels.
 * Multigrid needs n = 2^k + 1 coarsening to coarse_n (2^m + 1, at least
 * the minimum n of p, at most 257), or n <= min(coarse_n, 257): a single
 * direct level.  Any n >= the minimum gets plain CG. */
typedef struct sbp_ho_solver sbp_ho_solver;
int sbp_ho_solver_create(sbp_ho_solver** out, int n, int p, const sbp_options* opts);
int sbp_ho_solver_destroy(sbp_ho_solver* s);
/* Multigrid levels (0 when the handle supports CG only). */
int sbp_ho_solver_levels(const sbp_ho_solver* s);
long long sbp_ho_solver_device_bytes(const sbp_ho_solver* s);
/* MGCG on A_p x = b; stopping rule, norms and results as sbp_mgcg_solve. */
int sbp_ho_mgcg_solve(sbp_ho_solver* s, const double* b, double* x, double abstol, double reltol,
                      int maxiter, sbp_result* res, double* norms, int norms_cap, void* stream);
/* Plain CG on (sign * A_p) x = b (CG_CPU, level_2_multigrid_new.jl:258-291,
 * on the order-p matrix), as sbp_cg_solve. */
int sbp_ho_cg_solve(sbp_ho_solver* s, const double* b, double* x, int sign, double abstol,
                    double reltol, int maxiter, sbp_result* res, double* norms, int norms_cap,
                    void* stream);
/* v = one V-cycle from zero for the right-hand side b. */
int sbp_ho_vcycle_apply(sbp_ho_solver* s, const double* b, double* v, void* stream);

/* ---- variable coefficients (p = 2) ------------------------------------ */

/* The second-order SBP-SAT operator for div(c grad u) = f with nodal
 * coefficients c > 0.  Every grid line carries variable_diagonal_sbp_D2(2, N,
 * B) (diagonal_sbp.jl:470-495, 709-740) of its own coefficients; the 2D
 * assembly is get_operators' (legacy_functions.jl:100-174) with the SATs of
 * Assembling_matrix (level_2_multigrid_new.jl:145-150).  The boundary flux
 * and the Dirichlet penalty tau_D are scaled by c at the boundary point.
 * c = 1 gives the constant-coefficient operator.  Arrays are contiguous FP64
 * n x n device grids (ld = n), n >= 3.  Computed straight from c: u, c and
 * out are the only traffic. */
int sbp_apply_vc_f64(const double* u, const double* c, double* out, int n, int sign,
                     void* stream);

/* Variable-coefficient solver handle for the coefficient field c (copied
 * at creation).  opts (NULL = sbp_options_default) as for sbp_ho_solver_create.
 * - V-cycle levels re-discretise the operator.  Coarse coefficients are
 *   the harmonic mean of the fine ones over the full-weighting stencil,
 *   1 / sum_ab w_a w_b / c(2I+a, 2J+b), w = (1/4, 1/2, 1/4), clamped at
 *   the edges.
 * - The coarse level is solved exactly with a dense inverse; coarse_n is
 *   capped at 33.
 * - Any n >= 3 gets plain CG; multigrid needs n = 2^k + 1 or n <= 33. */
typedef struct sbp_vc_solver sbp_vc_solver;
int sbp_vc_solver_create(sbp_vc_solver** out, int n, const double* c, const sbp_options* opts);
int sbp_vc_solver_destroy(sbp_vc_solver* s);
int sbp_vc_solver_levels(const sbp_vc_solver* s);
long long sbp_vc_solver_device_bytes(const sbp_vc_solver* s);
int sbp_vc_mgcg_solve(sbp_vc_solver* s, const double* b, double* x, double abstol, double reltol,
                      int maxiter, sbp_result* res, double* norms, int norms_cap, void* stream);
int sbp_vc_cg_solve(sbp_vc_solver* s, const double* b, double* x, int sign, double abstol,
                    double reltol, int maxiter, sbp_result* res, double* norms, int norms_cap,
                    void* stream);
int sbp_vc_vcycle_apply(sbp_vc_solver* s, const double* b, double* v, void* stream);
/* The variable-coefficient A as CSR on the host (rows in column order),
 * from the same per-point stencil the GPU solver uses; c is a host array.
 * Needs no GPU.  Returns SBP_ERR_ARGS with *nnz set when cap is too small. */
int sbp_vc_assemble_host(int n, const double* c, long long* row_ptr, int* col, double* val,
                         long long cap, long long* nnz);
/* The coarse coefficients the variable-coefficient multigrid derives from a
 * fine field: cc (nc x nc) from cf ((2nc - 1) x (2nc - 1)), host arrays,
 * i fast, with the arithmetic of the solver's device kernel (the same bits).
 * The reference samples its coefficient function on each grid
 * (diagonal_sbp.jl:462-465); a nodal field is averaged instead, as the
 * solver handle describes.  Needs no GPU. */
int sbp_vc_coarsen_host(int nc, const double* cf, double* cc);

/* Galerkin coarse operators A_c = P' A P of the variable-coefficient
 * operator (P: the bilinear prolongation of sbp_prolong_f64), the set-up
 * arithmetic of a Galerkin multigrid hierarchy.  A_c is a symmetric 9-point
 * stencil at every point, stored as five host arrays of nc x nc (i fast):
 * D = A_c(p, p) and the couplings of -A_c to (i+1, j), (i, j+1), (i+1, j+1)
 * and (i-1, j+1): E, N, NE, NW (zero where the neighbour is outside).
 * sbp_vc_galerkin_coarse_host takes the fine operator from the nodal field c
 * on n x n points (n odd); sbp_galerkin9_coarse_host takes a 9-point level
 * in the same five-array form.  nc = (n + 1) / 2.  Needs no GPU.
 * The reference re-discretises each level instead (get_operators,
 * legacy_functions.jl:100-174); for a layered field the Galerkin operators
 * keep the MGCG iteration count independent of N. */
int sbp_vc_galerkin_coarse_host(int n, const double* c, double* D, double* E, double* N,
                                double* NE, double* NW);
int sbp_galerkin9_coarse_host(int n, const double* D, const double* E, const double* N,
                              const double* NE, const double* NW, double* Dc, double* Ec,
                              double* Nc, double* NEc, double* NWc);

/* The dense inverse the variable-coefficient solver uses on its coarse grid
 * (nc <= 33; c a host array of nc * nc coefficients), row-major, by the same
 * host Cholesky.  Needs no GPU. */
int sbp_vc_coarse_inverse_host(int nc, const double* c, double* out, long long cap);

/* ---- assembled-operator comparator ------------------------------------ */

/* The reference compares its matrix-free apply with SpMV on the assembled
 * matrix (Poisson_CG.jl:217, 244-271; kernel_comparisons/SPMV_test.jl).
 * sbp_csr_assemble_host writes A (SPD, = -H~(D2 + SAT) of Assembling_matrix)
 * on n x n points as CSR into host arrays: row_ptr (n^2 + 1 entries), col
 * and val (cap entries, increasing columns per row; rows and columns are
 * j * n + i).  With NULL arrays it only reports *nnz.  Needs no GPU. */
int sbp_csr_assemble_host(int n, long long* row_ptr, int* col, double* val, long long cap,
                          long long* nnz);
/* y = A x for a CSR matrix in device memory (row pointers as 64-bit ints). */
int sbp_csr_spmv_f64(long long nrows, const long long* row_ptr, const int* col,
                     const double* val, const double* x, double* y, void* stream);

/* ---- solver handle ---------------------------------------------------- */

/* Create a solver for n x n grids on the current device.  opts == NULL
 * creates a plain-CG solver (no multigrid hierarchy); otherwise the MG
 * hierarchy, its buffers and the coarse direct solver are built (the
 * reference's lu(A_2h), matrix_free_mg_cg.jl:460): the coarse operator is a
 * Kronecker sum of two 1D operators, so it is inverted exactly by fast
 * diagonalisation with two dense nc x nc FP64 eigenbases. */
int sbp_solver_create(sbp_solver** out, int n, const sbp_options* opts);
int sbp_solver_destroy(sbp_solver* s);
/* Number of levels of the hierarchy (1 for a plain-CG solver). */
int sbp_solver_levels(const sbp_solver* s);
/* Bytes of device memory held by the handle. */
long long sbp_solver_device_bytes(const sbp_solver* s);
/* Kernel launches of the last solve on this handle (set-up, every
 * iteration graph launched, including the one queued past convergence). */
long long sbp_solver_last_launches(const sbp_solver* s);

/* Preconditioned CG: solve A x = b from the caller's initial x (overwritten
 * with the solution).  Stops when ||r||_2 < abstol (abstol > 0) or
 * ||r||_2 < reltol * ||b - A x0|| (abstol <= 0), or after maxiter
 * iterations.  norms (host, capacity norms_cap, may be NULL) receives
 * ||r_k||_2 for k = 0..iters.  matrix_free_MGCG(b, x; A_2h, maxiter, abstol,
 * nu) (matrix_free_mg_cg.jl:281-324), which returns (iters, norms, x).
 * Returns SBP_OK, SBP_ERR_MAXITER or SBP_ERR_BREAKDOWN (res filled in all
 * three cases). */
int sbp_mgcg_solve(sbp_solver* s, const double* b, double* x, double abstol, double reltol,
                   int maxiter, sbp_result* res, double* norms, int norms_cap, void* stream);

/* Matrix-free CG on (sign*A) x = b.  sign = -1 is the reference's
 * CG_full_GPU / CG_Matrix_Free_GPU_v2 (split_matrix_free.jl:647-714), which
 * iterate with matrix_free_A_full_GPU and so solve (-A) x = b; sign = +1 is
 * CG_CPU on the assembled A (level_2_multigrid_new.jl:258-291).  Works on
 * any handle. */
int sbp_cg_solve(sbp_solver* s, const double* b, double* x, int sign, double abstol,
                 double reltol, int maxiter, sbp_result* res, double* norms, int norms_cap,
                 void* stream);

/* One V-cycle from v = 0: v = M b.  matrix_free_Two_level_multigrid(b, A_2h;
 * nu) (matrix_free_mg_cg.jl:143-176) for the two-level options. */
int sbp_vcycle_apply(sbp_solver* s, const double* b, double* v, void* stream);

/* Test hook for the failure path of the bounded waits (no counterpart in
 * the reference).  drop != 0: from the next launch on, CTA 0 of every
 * persistent stencil launch declares its first staged tile to its mbarrier
 * but issues no copy, and every bounded wait gives up after wait_polls
 * try_wait polls (0 = the default of about a second).  The affected calls
 * end with non-finite results and the solve entry points return
 * SBP_ERR_TIMEOUT; no memory access goes astray and no wait is unbounded.
 * drop = 0, wait_polls = 0 restores normal operation.  Synchronises the
 * device first.  Not for production use. */
int sbp_test_drop_copy(int drop, unsigned wait_polls);

/* Test hook for the direction pass's FP64 conversion (no counterpart in the
 * reference): out[k] = -(hi[k] + lo[k]) for float pairs, formed as the mixed
 * MGCG direction forms A p~ in FP64, without FP64 arithmetic (an FP32 two-sum and
 * an integer step on the FP64 bit pattern; the packed two-row form of the
 * interior wave on alternate pairs, the scalar form of the boundary tiles
 * on the others).  Must equal -((double)hi + (double)lo) bit for bit.
 * Device arrays of length n. */
int sbp_test_pair_to_f64(const float* hi, const float* lo, double* out, long long n,
                         void* stream);

/* Measured FP64 FMA rate of the current GPU in 1e9 lane-operations per
 * second (blocking): eight independent FMA chains per thread over one full
 * wave of CTAs, best of three CUDA-event timings.  The denominator of the
 * FP64-pipe roofline of the FP64 kernels.  Diagnostics; no reference
 * counterpart. */
int sbp_fp64_fma_rate(double* gfma_per_s, void* stream);

/* Per-kernel time of one solve (diagnostics). */
typedef struct sbp_kernel_time {
  char name[160];  /* demangled kernel name, truncated */
  int launches;    /* launches during the solve */
  double total_ms; /* sum of the launches' CUDA-event durations */
} sbp_kernel_time;

/* One solve as sbp_mgcg_solve (kind 0, sign ignored) or sbp_cg_solve
 * (kind 1) from the caller's x, stopping at reltol, but launched directly
 * instead of through CUDA graphs, with a pair of CUDA events on `stream`
 * around every kernel launch.  Per-kernel launch counts and summed
 * durations, aggregated by kernel and sorted by time, go to out (cap
 * entries); *count receives the number of distinct kernels.  The events
 * serialise the launches, so the sum exceeds a graph solve's time by the
 * launch gaps; each duration is the kernel's own.  The reference measures
 * this path with nsys and @elapsed around whole calls
 * (matrix_free_mg_cg.jl:577-597); it has no per-kernel timer of its own. */
int sbp_solver_profile(sbp_solver* s, int kind, const double* b, double* x, int sign,
                       double reltol, int maxiter, sbp_result* res, sbp_kernel_time* out,
                       int cap, int* count, void* stream);

/* Adjoint MGCG: lam = A^-T gu = A^-1 gu (A is SPD) with the handle's MGCG
 * from lam = 0 (tolerances as sbp_mgcg_solve), then the transpose of
 * sbp_rhs_f64's map applied to lam.  For u = A^-1 sbp_rhs_f64(f, g, fsign)
 * and a loss L(u) with dL/du = gu this gives dL/df (df, n x n) and dL/dg_side
 * (dgW, dgE, dgS, dgN, length n); each of those may be NULL.  lam (n x n) is
 * required.  Returns the solve's status (SBP_ERR_MAXITER still fills the
 * gradients).  No reference counterpart: the reference has no adjoint. */
int sbp_mgcg_adjoint_f64(sbp_solver* s, const double* gu, double* lam, double* df, double* dgW,
                         double* dgE, double* dgS, double* dgN, double fsign, double abstol,
                         double reltol, int maxiter, sbp_result* res, void* stream);

/* ---- batched solves --------------------------------------------------- */

/* A batch of independent MGCG problems of any grid sizes ns[0..count-1]
 * (each 2^m+1 and >= opts->coarse_n; opts as sbp_solver_create, required).
 * Every problem gets its own buffers, hierarchy and Krylov state; a solve
 * runs all problems together: the problems of one grid size share every
 * kernel launch (one pool of CTAs over all their tiles, per-problem
 * reductions, finished problems skip their tiles), the grid sizes run as
 * parallel branches, and one iteration of the whole batch is one CUDA graph.
 * At most 512 problems per grid size.  No reference counterpart: the
 * reference solves one problem per call (matrix_free_MGCG,
 * matrix_free_mg_cg.jl:281-324). */
typedef struct sbp_batch sbp_batch;
int sbp_batch_create(sbp_batch** out, const int* ns, int count, const sbp_options* opts);
int sbp_batch_destroy(sbp_batch* b);
int sbp_batch_size(const sbp_batch* b);
long long sbp_batch_device_bytes(const sbp_batch* b);
/* Kernel launches of the last batched solve (batched launches, not per
 * problem). */
long long sbp_batch_last_launches(const sbp_batch* b);
/* Number of grid sizes (classes) of the batch; their sizes, largest first,
 * into ns (cap entries, may be NULL). */
int sbp_batch_classes(const sbp_batch* b, int* ns, int cap);
/* Launch-shape autotuner: for every grid size, time three batch iterations
 * after a fresh set-up on the given problems (xs are overwritten) with each
 * candidate CTA budget of the batched persistent kernels (one full wave,
 * 2 x SMs, 1 x SMs, SMs / 2) and keep the fastest; the iteration graphs are
 * recaptured with the choice.  budgets (one per class, may be NULL) receives
 * the chosen budget, 0 meaning one full wave. */
int sbp_batch_autotune(sbp_batch* b, const double* const* bs, double* const* xs, int* budgets,
                       void* stream);
/* MGCG on A_k x_k = b_k for every problem k from the caller's x_k (device
 * pointers in the caller's layout, ld = n_k; host arrays of count pointers),
 * with the stopping rule of sbp_mgcg_solve applied per problem.  results
 * (count entries, may be NULL) receives each problem's outcome.  Returns
 * SBP_OK when every problem converged, else the first other status. */
int sbp_batch_mgcg_solve(sbp_batch* b, const double* const* bs, double* const* xs, double abstol,
                         double reltol, int maxiter, sbp_result* results, void* stream);

/* ---- host-only helpers ------------------------------------------------ */

/* Dense inverse of the coarse operator A on an nc x nc grid (row-major,
 * nc^2 x nc^2, nc <= 129), computed on the host column by column from the
 * same fast-diagonalisation factors the solver uploads to replace the
 * reference's per-V-cycle host LU solve (matrix_free_mg_cg.jl:166).  `cap`
 * is the capacity of `out` in doubles.  Needs no GPU. */
int sbp_coarse_inverse_host(int nc, double* out, long long cap);
/* The same for the operator of SBP order p (2, 4 or 6) on any nc x nc grid
 * (nc <= 129, at least 3 for p = 2, 8 for p = 4 and 12 for p = 6), from the
 * fast-diagonalisation factors that the order-p solver's coarse level uses.
 * Needs no GPU. */
int sbp_coarse_inverse_order_host(int nc, int p, double* out, long long cap);

/* Message of the last SBP_ERR_CUDA / SBP_ERR_NOMEM on this host thread. */
const char* sbp_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* SBPMG_H_ */

/*
 * sbp_cpu.c - CPU restatement of the reference's sparse solver path.
 *
 * TEST INFRASTRUCTURE ONLY: the CPU baseline timed beside the GPU library
 * (bench.py's cpu_baseline and --impl reference legs) and a second oracle
 * checked against sbp_oracle.py.  The product library never links it.
 *
 * Restates, with CSR sparse matrices and OpenMP row-parallel SpMV:
 *  - Assembling_matrix (preconditioned_CG/level_2_multigrid_new.jl:125-188)
 *    via the 1D p=2 SBP pieces of diagonal_sbp.jl:56-61, 189-197, 414-452:
 *    A = -H~ (D2x + D2y + SAT_W + SAT_E + SAT_S + SAT_N), one row per point;
 *  - restriction_2d / prolongation_2d as kron CSR matrices (:190-246);
 *  - modified_richardson! / jacobi_brittany! (:335-350);
 *  - Two_level_multigrid (:358-382), recursive here for a V-cycle;
 *  - the coarse solve A_2h \ f (matrix_free_mg_cg.jl:166) as a banded
 *    Cholesky factor + triangular solves (exact up to rounding, like LU);
 *  - mg_preconditioned_CG (:480-524) and CG_CPU (:258-291).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  int rows, cols, nnz;
  int* rp;
  int* ci;
  double* v;
} csr;

typedef struct {
  int smoother;      /* 0 Jacobi, 1 Richardson */
  double omega;
  int nu_pre, nu_post;
  int restriction;   /* 0 normal, 1 sbp, 2 galerkin */
  int coarse_n;
} cpu_opts;

typedef struct {
  int nlev;
  int n[32];
  csr A[32];
  double* dinv[32];
  csr R[32];          /* level l -> l+1 */
  csr P[32];          /* level l+1 -> l */
  double* b[32];
  double* v[32];
  double* t[32];
  /* coarse banded Cholesky */
  int cN, cw;
  double* L;          /* L[k*(cw+1)+d] = L(k, k-d) */
  cpu_opts o;
  /* CG vectors */
  double *r, *z, *p, *Ap;
} cpu_mg;

static void csr_free(csr* m) {
  free(m->rp);
  free(m->ci);
  free(m->v);
  memset(m, 0, sizeof(*m));
}

/* ---- row builder ------------------------------------------------------ */
typedef struct {
  int cnt;
  int col[16];
  double val[16];
} rowbuf;

static void row_add(rowbuf* rb, int col, double v) {
  for (int k = 0; k < rb->cnt; ++k)
    if (rb->col[k] == col) {
      rb->val[k] += v;
      return;
    }
  rb->col[rb->cnt] = col;
  rb->val[rb->cnt] = v;
  rb->cnt++;
}

static int cmp_int(const void* a, const void* b) { return *(const int*)a - *(const int*)b; }

/* 1D D2 row r (times h^2) as (cols, coefs): interior [1 -2 1], boundary rows
 * the same coefficients one-sided (diagonal_sbp.jl:191-197, bd = d). */
static int d2_row(int r, int n, int* c, double* w) {
  if (r == 0) { c[0] = 0; c[1] = 1; c[2] = 2; }
  else if (r == n - 1) { c[0] = n - 1; c[1] = n - 2; c[2] = n - 3; }
  else { c[0] = r - 1; c[1] = r; c[2] = r + 1; }
  if (r == 0 || r == n - 1) { w[0] = 1; w[1] = -2; w[2] = 1; }
  else { w[0] = 1; w[1] = -2; w[2] = 1; }
  return 3;
}

/* BS row (times h) at boundary index: BS = SN - S0, row 0: [3/2, -2, 1/2] on
 * cols 0..2; row n-1: [3/2, -2, 1/2] on cols n-1..n-3. */
static const double BS[3] = {1.5, -2.0, 0.5};

static csr build_A(int n) {
  const double h = 1.0 / (n - 1);
  const double tauD = -13.0 / h, tauN = -1.0, beta = 1.0;
  const int N = n * n;
  csr A;
  A.rows = A.cols = N;
  A.rp = (int*)malloc(sizeof(int) * (N + 1));
  A.ci = (int*)malloc(sizeof(int) * (size_t)N * 9);
  A.v = (double*)malloc(sizeof(double) * (size_t)N * 9);
  int nnz = 0;
  for (int j = 0; j < n; ++j) {
    for (int i = 0; i < n; ++i) {
      rowbuf rb;
      rb.cnt = 0;
      const double wi = (i == 0 || i == n - 1) ? 0.5 : 1.0;
      const double wj = (j == 0 || j == n - 1) ? 0.5 : 1.0;
      const double Ht = h * h * wi * wj;   /* H~ = kron(H1x, H1y) */
      int c[3];
      double w[3];
      /* D2x (slow index j) and D2y (fast index i): 1/h^2 scaled */
      d2_row(j, n, c, w);
      for (int k = 0; k < 3; ++k) row_add(&rb, c[k] * n + i, Ht * w[k] / (h * h));
      d2_row(i, n, c, w);
      for (int k = 0; k < 3; ++k) row_add(&rb, j * n + c[k], Ht * w[k] / (h * h));
      /* SAT_W = tau HI_x E_W + beta HI_x BS_x' E_W:
       * (HI_x)(j) = 1/(h wj); E_W selects j' = 0; BS_x'[j,0] = BS row 0 at col j */
      const double hix = 1.0 / (h * wj);
      if (j == 0) row_add(&rb, 0 * n + i, Ht * hix * tauD);
      if (j <= 2) row_add(&rb, 0 * n + i, Ht * hix * beta * BS[j] / h);
      if (j == n - 1) row_add(&rb, (n - 1) * n + i, Ht * hix * tauD);
      if (j >= n - 3) row_add(&rb, (n - 1) * n + i, Ht * hix * beta * BS[n - 1 - j] / h);
      /* SAT_S = tau HI_y E_S BS_y: row i = 0 gets tau/(h wi) * BS row 0 */
      const double hiy = 1.0 / (h * wi);
      if (i == 0)
        for (int k = 0; k < 3; ++k) row_add(&rb, j * n + k, Ht * hiy * tauN * BS[k] / h);
      if (i == n - 1)
        for (int k = 0; k < 3; ++k) row_add(&rb, j * n + (n - 1 - k), Ht * hiy * tauN * BS[k] / h);
      /* A = -H~ (...), drop exact zeros, sort columns */
      A.rp[j * n + i] = nnz;
      int order[16];
      for (int k = 0; k < rb.cnt; ++k) order[k] = rb.col[k];
      qsort(order, rb.cnt, sizeof(int), cmp_int);
      for (int q = 0; q < rb.cnt; ++q)
        for (int k = 0; k < rb.cnt; ++k)
          if (rb.col[k] == order[q] && rb.val[k] != 0.0) {
            A.ci[nnz] = rb.col[k];
            A.v[nnz] = -rb.val[k];
            nnz++;
          }
    }
  }
  A.rp[N] = nnz;
  A.nnz = nnz;
  return A;
}

/* 1D restriction weight of fine index 2c+a in coarse c (restriction_matrix /
 * restriction_matrix_normal, level_2_multigrid_new.jl:205-233). */
static double r1(int kind, int c, int nc, int a) {
  if ((c == 0 && a < 0) || (c == nc - 1 && a > 0)) return 0.0;
  const int edge = (c == 0 || c == nc - 1);
  double w = (a == 0) ? 0.5 : 0.25;
  if (kind == 1 && edge && a != 0) w = 0.5;
  if (kind == 2) w *= 2.0;
  return w;
}

static csr build_R(int nf, int kind) {
  const int nc = (nf + 1) / 2;
  csr R;
  R.rows = nc * nc;
  R.cols = nf * nf;
  R.rp = (int*)malloc(sizeof(int) * (R.rows + 1));
  R.ci = (int*)malloc(sizeof(int) * (size_t)R.rows * 9);
  R.v = (double*)malloc(sizeof(double) * (size_t)R.rows * 9);
  int nnz = 0;
  for (int J = 0; J < nc; ++J)
    for (int I = 0; I < nc; ++I) {
      R.rp[J * nc + I] = nnz;
      for (int b = -1; b <= 1; ++b)
        for (int a = -1; a <= 1; ++a) {
          const double w = r1(kind, I, nc, a) * r1(kind, J, nc, b);
          if (w == 0.0) continue;
          R.ci[nnz] = (2 * J + b) * nf + (2 * I + a);
          R.v[nnz] = w;
          nnz++;
        }
    }
  R.rp[R.rows] = nnz;
  R.nnz = nnz;
  return R;
}

/* prolongation_matrix (:190-203) kron'd */
static csr build_P(int nc) {
  const int nf = 2 * nc - 1;
  csr P;
  P.rows = nf * nf;
  P.cols = nc * nc;
  P.rp = (int*)malloc(sizeof(int) * (P.rows + 1));
  P.ci = (int*)malloc(sizeof(int) * (size_t)P.rows * 4);
  P.v = (double*)malloc(sizeof(double) * (size_t)P.rows * 4);
  int nnz = 0;
  for (int j = 0; j < nf; ++j)
    for (int i = 0; i < nf; ++i) {
      P.rp[j * nf + i] = nnz;
      int ci[2], cj[2];
      double wi[2], wj[2];
      int ki = 0, kj = 0;
      if (i % 2 == 0) { ci[0] = i / 2; wi[0] = 1.0; ki = 1; }
      else { ci[0] = i / 2; ci[1] = i / 2 + 1; wi[0] = wi[1] = 0.5; ki = 2; }
      if (j % 2 == 0) { cj[0] = j / 2; wj[0] = 1.0; kj = 1; }
      else { cj[0] = j / 2; cj[1] = j / 2 + 1; wj[0] = wj[1] = 0.5; kj = 2; }
      for (int b = 0; b < kj; ++b)
        for (int a = 0; a < ki; ++a) {
          P.ci[nnz] = cj[b] * nc + ci[a];
          P.v[nnz] = wi[a] * wj[b];
          nnz++;
        }
    }
  P.rp[P.rows] = nnz;
  P.nnz = nnz;
  return P;
}

static void spmv(const csr* M, const double* x, double* y) {
#pragma omp parallel for schedule(static)
  for (int r = 0; r < M->rows; ++r) {
    double s = 0.0;
    for (int k = M->rp[r]; k < M->rp[r + 1]; ++k) s += M->v[k] * x[M->ci[k]];
    y[r] = s;
  }
}

static double dot(const double* a, const double* b, int N) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (int k = 0; k < N; ++k) s += a[k] * b[k];
  return s;
}

/* ---- coarse banded Cholesky ------------------------------------------- */
static double band_get(const double* L, int w, int r, int c) {
  const int d = r - c;
  return (d > w || d < 0) ? 0.0 : L[(size_t)r * (w + 1) + d];
}

static int band_factor(cpu_mg* m, const csr* A) {
  const int N = A->rows;
  int w = 0;
  for (int r = 0; r < N; ++r)
    for (int k = A->rp[r]; k < A->rp[r + 1]; ++k)
      if (r - A->ci[k] > w) w = r - A->ci[k];
  m->cN = N;
  m->cw = w;
  m->L = (double*)calloc((size_t)N * (w + 1), sizeof(double));
  for (int r = 0; r < N; ++r)
    for (int k = A->rp[r]; k < A->rp[r + 1]; ++k)
      if (A->ci[k] <= r) m->L[(size_t)r * (w + 1) + (r - A->ci[k])] = A->v[k];
  double* L = m->L;
  for (int k = 0; k < N; ++k) {
    const int j0 = k - w > 0 ? k - w : 0;
    for (int j = j0; j <= k; ++j) {
      double s = band_get(L, w, k, j);
      const int m0 = (j - w > j0) ? j - w : j0;
      for (int q = m0; q < j; ++q) s -= band_get(L, w, k, q) * band_get(L, w, j, q);
      if (j == k) {
        if (!(s > 0.0)) return -1;
        L[(size_t)k * (w + 1)] = sqrt(s);
      } else {
        L[(size_t)k * (w + 1) + (k - j)] = s / band_get(L, w, j, j);
      }
    }
  }
  return 0;
}

static void band_solve(const cpu_mg* m, const double* f, double* x) {
  const int N = m->cN, w = m->cw;
  const double* L = m->L;
  for (int k = 0; k < N; ++k) {
    double s = f[k];
    const int m0 = k - w > 0 ? k - w : 0;
    for (int q = m0; q < k; ++q) s -= L[(size_t)k * (w + 1) + (k - q)] * x[q];
    x[k] = s / L[(size_t)k * (w + 1)];
  }
  for (int k = N - 1; k >= 0; --k) {
    double s = x[k];
    const int m1 = k + w < N - 1 ? k + w : N - 1;
    for (int q = k + 1; q <= m1; ++q) s -= L[(size_t)q * (w + 1) + (q - k)] * x[q];
    x[k] = s / L[(size_t)k * (w + 1)];
  }
}

/* ---- public API ---------------------------------------------------------- */
void cpu_set_threads(int t) {
#ifdef _OPENMP
  if (t > 0) omp_set_num_threads(t);
#else
  (void)t;
#endif
}

int cpu_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void cpu_mg_destroy(cpu_mg* m) {
  if (!m) return;
  for (int l = 0; l < m->nlev; ++l) {
    csr_free(&m->A[l]);
    free(m->dinv[l]);
    if (l + 1 < m->nlev) {
      csr_free(&m->R[l]);
      csr_free(&m->P[l]);
    }
    if (l > 0) free(m->b[l]);
    free(m->v[l]);
    free(m->t[l]);
  }
  free(m->L);
  free(m->r);
  free(m->z);
  free(m->p);
  free(m->Ap);
  free(m);
}

/* opts == NULL: single level (plain CG only). */
cpu_mg* cpu_mg_create(int n, const cpu_opts* o) {
  cpu_mg* m = (cpu_mg*)calloc(1, sizeof(cpu_mg));
  if (o) m->o = *o;
  int nn = n;
  while (1) {
    const int l = m->nlev++;
    m->n[l] = nn;
    m->A[l] = build_A(nn);
    const int N = nn * nn;
    m->dinv[l] = (double*)malloc(sizeof(double) * N);
    for (int r = 0; r < N; ++r)
      for (int k = m->A[l].rp[r]; k < m->A[l].rp[r + 1]; ++k)
        if (m->A[l].ci[k] == r) m->dinv[l][r] = 1.0 / m->A[l].v[k];
    m->v[l] = (double*)malloc(sizeof(double) * N);
    m->t[l] = (double*)malloc(sizeof(double) * N);
    if (l > 0) m->b[l] = (double*)malloc(sizeof(double) * N);
    if (!o || nn <= o->coarse_n || nn <= 3) break;
    m->R[l] = build_R(nn, o->restriction);
    m->P[l] = build_P((nn + 1) / 2);
    nn = (nn + 1) / 2;
  }
  if (o && band_factor(m, &m->A[m->nlev - 1]) != 0) {
    cpu_mg_destroy(m);
    return NULL;
  }
  const size_t N0 = (size_t)n * n;
  m->r = (double*)malloc(sizeof(double) * N0);
  m->z = (double*)malloc(sizeof(double) * N0);
  m->p = (double*)malloc(sizeof(double) * N0);
  m->Ap = (double*)malloc(sizeof(double) * N0);
  return m;
}

static void smooth(cpu_mg* m, int l, double* v, const double* b, int iters) {
  const int N = m->n[l] * m->n[l];
  double* t = m->t[l];
  const double w = m->o.omega;
  for (int it = 0; it < iters; ++it) {
    spmv(&m->A[l], v, t);
    if (m->o.smoother == 0) {
#pragma omp parallel for schedule(static)
      for (int k = 0; k < N; ++k) v[k] += w * (b[k] - t[k]) * m->dinv[l][k];
    } else {
#pragma omp parallel for schedule(static)
      for (int k = 0; k < N; ++k) v[k] += w * (b[k] - t[k]);
    }
  }
}

/* v = M b (one V-cycle from zero) on level l. */
static void vcycle(cpu_mg* m, int l, const double* b, double* v) {
  const int N = m->n[l] * m->n[l];
  if (l == m->nlev - 1) {
    band_solve(m, b, v);
    return;
  }
  memset(v, 0, sizeof(double) * N);
  smooth(m, l, v, b, m->o.nu_pre);
  double* t = m->t[l];
  spmv(&m->A[l], v, t);
#pragma omp parallel for schedule(static)
  for (int k = 0; k < N; ++k) t[k] = b[k] - t[k];
  spmv(&m->R[l], t, m->b[l + 1]);
  vcycle(m, l + 1, m->b[l + 1], m->v[l + 1]);
  spmv(&m->P[l], m->v[l + 1], t);
#pragma omp parallel for schedule(static)
  for (int k = 0; k < N; ++k) v[k] += t[k];
  smooth(m, l, v, b, m->o.nu_post);
}

void cpu_vcycle(cpu_mg* m, const double* b, double* v) { vcycle(m, 0, b, v); }

void cpu_apply(cpu_mg* m, const double* u, double* out) { spmv(&m->A[0], u, out); }

int cpu_nnz(cpu_mg* m, int l) { return m->A[l].nnz; }

void cpu_export_A(cpu_mg* m, int l, int* rp, int* ci, double* v) {
  memcpy(rp, m->A[l].rp, sizeof(int) * (m->A[l].rows + 1));
  memcpy(ci, m->A[l].ci, sizeof(int) * m->A[l].nnz);
  memcpy(v, m->A[l].v, sizeof(double) * m->A[l].nnz);
}

/* mg_preconditioned_CG: returns iterations; norms[0..iters] */
int cpu_mgcg(cpu_mg* m, const double* b, double* x, double abstol, int maxiter, double* norms) {
  const int N = m->n[0] * m->n[0];
  double *r = m->r, *z = m->z, *p = m->p, *Ap = m->Ap;
  spmv(&m->A[0], x, Ap);
  for (int k = 0; k < N; ++k) r[k] = b[k] - Ap[k];
  vcycle(m, 0, r, z);
  memcpy(p, z, sizeof(double) * N);
  double rz = dot(r, z, N);
  norms[0] = sqrt(dot(r, r, N));
  int it = 0;
  for (int step = 0; step < maxiter; ++step) {
    ++it;
    spmv(&m->A[0], p, Ap);
    const double alpha = rz / dot(p, Ap, N);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < N; ++k) {
      x[k] += alpha * p[k];
      r[k] -= alpha * Ap[k];
    }
    const double rs = dot(r, r, N);
    norms[it] = sqrt(rs);
    if (sqrt(rs) < abstol) break;
    vcycle(m, 0, r, z);
    const double rzn = dot(r, z, N);
    const double beta = rzn / rz;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < N; ++k) p[k] = z[k] + beta * p[k];
    rz = rzn;
  }
  return it;
}

/* CG_CPU */
int cpu_cg(cpu_mg* m, const double* b, double* x, double abstol, int maxiter, double* norms) {
  const int N = m->n[0] * m->n[0];
  double *r = m->r, *p = m->p, *Ap = m->Ap;
  spmv(&m->A[0], x, Ap);
  for (int k = 0; k < N; ++k) r[k] = b[k] - Ap[k];
  memcpy(p, r, sizeof(double) * N);
  double rs = dot(r, r, N);
  norms[0] = sqrt(rs);
  int it = 0;
  for (int step = 0; step < maxiter; ++step) {
    ++it;
    spmv(&m->A[0], p, Ap);
    const double alpha = rs / dot(p, Ap, N);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < N; ++k) {
      x[k] += alpha * p[k];
      r[k] -= alpha * Ap[k];
    }
    const double rsn = dot(r, r, N);
    norms[it] = sqrt(rsn);
    if (sqrt(rsn) < abstol) break;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < N; ++k) p[k] = r[k] + (rsn / rs) * p[k];
    rs = rsn;
  }
  return it;
}

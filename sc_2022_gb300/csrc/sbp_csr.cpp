// The assembled operator A as a CSR matrix, for the sparse comparator (the
// reference's matrix-free vs assembled-SpMV comparison, Poisson_CG.jl:217,
// 244-271 and kernel_comparisons/SPMV_test.jl: A = Assembling_matrix(...) on
// the GPU as CuSparseMatrixCSR).  Rows and columns are flattened j * n + i;
// the coefficients come from negA, the formula every kernel applies, so the
// matrix equals Assembling_matrix's A (level_2_multigrid_new.jl:125-188).

#include "sbp_common.cuh"
#include "sbpmg.h"

namespace {

struct Indicator {
  int di, dj;
  double operator()(int a, int b) const { return (a == di && b == dj) ? 1.0 : 0.0; }
};

// Nonzeros of row (i, j) in increasing column order; returns the count (<= 7).
// negA reaches (0,0), (+-1,0), (0,+-1) and (0,+-2) only; listed in (dj, di)
// order, which is the order of the flattened column index jj * n + ii.
int row_entries(int n, int i, int j, long long* cols, double* vals) {
  static const int offs[7][2] = {{0, -2}, {0, -1}, {-1, 0}, {0, 0}, {1, 0}, {0, 1}, {0, 2}};
  int cnt = 0;
  for (const auto& o : offs) {
    const int ii = i + o[0], jj = j + o[1];
    if (ii < 0 || ii >= n || jj < 0 || jj >= n) continue;
    const double c = -sbp::negA<double>(Indicator{o[0], o[1]}, i, j, n);
    if (c != 0.0) {
      cols[cnt] = (long long)jj * n + ii;
      vals[cnt] = c;
      ++cnt;
    }
  }
  return cnt;
}

}  // namespace

extern "C" int sbp_csr_assemble_host(int n, long long* row_ptr, int* col, double* val,
                                     long long cap, long long* nnz) {
  if (n < 3 || !nnz) return SBP_ERR_ARGS;
  if ((long long)n * n > 2147483647LL) return SBP_ERR_UNSUPPORTED;
  long long k = 0;
  long long cols[7];
  double vals[7];
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      const long long r = (long long)j * n + i;
      if (row_ptr) row_ptr[r] = k;
      const int c = row_entries(n, i, j, cols, vals);
      if (col && val) {
        if (k + c > cap) return SBP_ERR_ARGS;
        for (int q = 0; q < c; ++q) {
          col[k + q] = (int)cols[q];
          val[k + q] = vals[q];
        }
      }
      k += c;
    }
  if (row_ptr) row_ptr[(long long)n * n] = k;
  *nnz = k;
  return SBP_OK;
}

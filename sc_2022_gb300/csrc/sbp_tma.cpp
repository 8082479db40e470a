// TMA tensor-map encoding through the driver entry point (no -lcuda link).
#include "sbp_tma.h"

#include <cudaTypedefs.h>

#include <cstdint>
#include <cstring>

namespace sbp {

namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }();
  return fn;
}

bool encode(CUtensorMap* m, const void* p, int n, int ld, bool f64, int bi, int bj) {
  auto fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)n, (cuuint64_t)n};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * (f64 ? 8u : 4u)};
  const cuuint32_t box[2] = {(cuuint32_t)bi, (cuuint32_t)bj};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = fn(m, f64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                        2, const_cast<void*>(p), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

}  // namespace

bool make_box_map(CUtensorMap& m, const Operand& op, bool f64, int bi, int bj) {
  if (!op.tma) return false;
  return encode(&m, op.p, op.n, op.ld, f64, bi, bj);
}

bool make_operand(Operand& op, const void* p, int n, int ld, bool f64) {
  op.p = p;
  op.n = n;
  op.ld = ld;
  op.tma = false;
  std::memset(&op.box, 0, sizeof(CUtensorMap));
  std::memset(&op.inner, 0, sizeof(CUtensorMap));
  std::memset(&op.coarse, 0, sizeof(CUtensorMap));
  const size_t es = f64 ? 8 : 4;
  if (((uintptr_t)p & 15u) != 0 || ((size_t)ld * es) % 16 != 0) return false;
  if (!encode(&op.box, p, n, ld, f64, kBoxI, kBoxJ)) return false;
  if (!encode(&op.inner, p, n, ld, f64, kInI, kInJ)) return false;
  if (!encode(&op.coarse, p, n, ld, f64, kCoI, kCoJ)) return false;
  op.tma = true;
  return true;
}

}  // namespace sbp

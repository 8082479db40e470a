// Host-side construction of TMA tensor maps for the solver's grid arrays.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

namespace sbp {

// Staged boxes (see sbp_kernels.cu): the 64 x 32 output tile with its halo,
// the tile interior of pointwise operands, and the coarse region under a
// tile (prolongation source).
constexpr int kBoxI = 72, kBoxJ = 37;
constexpr int kInI = 68, kInJ = 33;
constexpr int kCoI = 40, kCoJ = 20;

// A grid array as a kernel operand: raw pointer + leading dimension, and,
// when the layout allows it (16-byte aligned base and column pitch), TMA
// maps for the three boxes.
struct Operand {
  const void* p = nullptr;
  int n = 0;
  int ld = 0;
  bool tma = false;
  CUtensorMap box{};
  CUtensorMap inner{};
  CUtensorMap coarse{};
};

// Fill the tensor maps of `op` for an n x n array of `f64 ? double : float`
// with leading dimension ld.  Returns false (and leaves op.tma = false) when
// the layout is not TMA-addressable or the driver entry point is missing.
bool make_operand(Operand& op, const void* p, int n, int ld, bool f64);

// A tensor map of `op`'s array with an arbitrary box (bi x bj elements).
bool make_box_map(CUtensorMap& m, const Operand& op, bool f64, int bi, int bj);

// Leading dimension the solver uses for its own n x n arrays: a multiple of
// four elements, so every column starts on a 16-byte boundary.
inline int padded_ld(int n) { return (n + 3) & ~3; }

}  // namespace sbp

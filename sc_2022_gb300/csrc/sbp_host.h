// Host-side helpers shared by the C-ABI translation units.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "../../include/sbpmg.h"
#include "sbp_common.cuh"

namespace sbp {

// The message sbp_last_error() returns on this thread.
void set_last_error(const std::string& msg);
// Record "what: <CUDA error string>" and return SBP_ERR_CUDA.
int fail_cuda(cudaError_t e, const char* what);
// After a stream synchronisation: SBP_ERR_TIMEOUT (message recorded) if a
// kernel's bounded wait gave up since the last check (the flag is cleared),
// else SBP_OK.
int check_device_fault(const char* what);
// sbp_result and status code from a finished Krylov state.
int finish_result(const SolveState& fs, sbp_result* res);

}  // namespace sbp

#define SBP_CUDA(...)                                                 \
  do {                                                                \
    cudaError_t _e = (__VA_ARGS__);                                   \
    if (_e != cudaSuccess) return ::sbp::fail_cuda(_e, #__VA_ARGS__); \
  } while (0)

// Shared helpers for the grada CUDA sources: error type, launch checks and
// small numeric utilities.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <nvtx3/nvToolsExt.h>

#include <stdexcept>
#include <string>

namespace grada {

// Error carried from the internals to the C ABI, where it becomes a status.
struct Error : public std::runtime_error {
  int status;
  Error(int s, const std::string &m) : std::runtime_error(m), status(s) {}
};

#define GRADA_CUDA_CHECK(expr)                                                              \
  do {                                                                                      \
    cudaError_t e_ = (expr);                                                                \
    if (e_ != cudaSuccess) {                                                                \
      int st_ = (e_ == cudaErrorMemoryAllocation) ? -3 : -2;                                \
      throw ::grada::Error(st_, std::string(#expr) + ": " + cudaGetErrorString(e_));        \
    }                                                                                       \
  } while (0)

#define GRADA_LAUNCH_CHECK() GRADA_CUDA_CHECK(cudaGetLastError())

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }
inline int64_t round_up(int64_t a, int64_t b) { return ceil_div(a, b) * b; }

// NVTX range around a host-side operation (visible in Nsight timelines; a
// no-op without a tool attached).
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

// Store helpers used by the G writers.
__device__ __forceinline__ void store_entry(double *p, double v) { *p = v; }
__device__ __forceinline__ void store_entry(float *p, double v) { *p = (float)v; }

}  // namespace grada

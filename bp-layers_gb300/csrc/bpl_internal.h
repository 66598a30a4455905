// Host-side helpers shared by the C-ABI translation units.
#pragma once

#include <cuda_runtime.h>

#include <nvtx3/nvToolsExt.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/bpl_gb300.h"

namespace bpl {

// Records a message for bpl_last_error() and returns `status`.
int set_error(int status, const char* fmt, ...);

inline int cuda_status(cudaError_t e, const char* where) {
  if (e == cudaSuccess) return BPL_OK;
  return set_error(BPL_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
}

#define BPL_REQUIRE(cond, ...)                                  \
  do {                                                          \
    if (!(cond)) return ::bpl::set_error(BPL_ERR_INVALID_ARG, __VA_ARGS__); \
  } while (0)

#define BPL_CUDA_TRY(expr, where)                               \
  do {                                                          \
    cudaError_t _e = (expr);                                    \
    if (_e != cudaSuccess) return ::bpl::cuda_status(_e, where); \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// NVTX range over the host-side scope of an entry point or of one sweep
// phase's launch: named ranges in Nsight Systems / Compute timelines, a few
// nanoseconds and no dependency when no tool is attached (NVTX v3 is
// header-only).
struct TraceRange {
  explicit TraceRange(const char* name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};
#define BPL_TRACE(name) ::bpl::TraceRange bpl_trace_scope_(name)

// Number of SMs of the current device (cached per device).
int sm_count();
// Opt-in shared memory per block of the current device.
int max_smem_optin();
// Shared memory per SM and the runtime's reservation per resident block.
int smem_per_sm();
int smem_reserved_per_block();

}  // namespace bpl

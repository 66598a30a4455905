// C-ABI housekeeping: version, status text, per-thread error messages, the
// device error word, device properties.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <string>

#include "bpl_device.cuh"
#include "bpl_internal.h"

namespace bpl {

namespace {
thread_local std::string t_last_error;
}

int set_error(int status, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  t_last_error = buf;
  return status;
}

namespace {
struct DevProps {
  int sms = 0;
  int smem_optin = 0;
  int smem_sm = 0;
  int smem_reserved = 0;
};
std::mutex g_props_mu;
DevProps g_props[64];
bool g_props_ok[64] = {};

const DevProps& props() {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  std::lock_guard<std::mutex> lk(g_props_mu);
  if (!g_props_ok[dev]) {
    cudaDeviceGetAttribute(&g_props[dev].sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&g_props[dev].smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&g_props[dev].smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&g_props[dev].smem_reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    g_props_ok[dev] = true;
  }
  return g_props[dev];
}
}  // namespace

int sm_count() { return props().sms > 0 ? props().sms : 152; }
int max_smem_optin() { return props().smem_optin > 0 ? props().smem_optin : 48 * 1024; }
int smem_per_sm() { return props().smem_sm > 0 ? props().smem_sm : 228 * 1024; }
int smem_reserved_per_block() { return props().smem_reserved > 0 ? props().smem_reserved : 1024; }

}  // namespace bpl

extern "C" {

int bpl_version(void) { return 100; }

const char* bpl_status_string(int status) {
  switch (status) {
    case BPL_OK: return "ok";
    case BPL_ERR_INVALID_ARG: return "invalid argument";
    case BPL_ERR_UNSUPPORTED: return "unsupported configuration";
    case BPL_ERR_CUDA: return "CUDA error";
    case BPL_ERR_DEVICE_TIMEOUT: return "device wait timed out";
    default: return "unknown status";
  }
}

const char* bpl_last_error(void) { return bpl::t_last_error.c_str(); }

int bpl_read_device_error(int* code) {
  if (!code) return bpl::set_error(BPL_ERR_INVALID_ARG, "read_device_error: null pointer");
  int v = 0;
  BPL_CUDA_TRY(cudaDeviceSynchronize(), "read_device_error: synchronize");
  BPL_CUDA_TRY(cudaMemcpyFromSymbol(&v, bpl::g_bpl_error, sizeof(int)), "read_device_error: copy");
  const int zero = 0;
  BPL_CUDA_TRY(cudaMemcpyToSymbol(bpl::g_bpl_error, &zero, sizeof(int)), "read_device_error: clear");
  *code = v;
  return BPL_OK;
}

int bpl_set_wait_limit(unsigned polls) {
  const unsigned v = polls;
  BPL_CUDA_TRY(cudaMemcpyToSymbol(bpl::g_bpl_wait_limit, &v, sizeof(unsigned)), "set_wait_limit");
  return BPL_OK;
}

}  // extern "C"

// LBP reference adjoint without any device allocation by the library or the
// caller: the scratch that bpl_lbp_backward takes as a caller-provided
// workspace lives here in a fixed, file-scope device array.
//
// Who needs this: hosts that cannot call cudaMalloc when they run the
// backward -- an embedding application whose device memory is owned and
// pooled by another runtime, code paths with a fixed device-memory budget
// decided at start-up, or latency-critical loops where an allocation (which
// may synchronise the device) is not acceptable.  They still pass their own
// inputs and outputs; only the scratch moves into the library.
//
// Costs and limits:
//   * every GPU on which the library's module is loaded holds
//     kNoAllocScratchBytes of device memory for this array until the process
//     exits.  With CUDA's lazy module loading (the default) the module, and
//     with it the array, is loaded on a device by the library's first use
//     there, which may be this entry point's first call: that call may then
//     allocate the array and synchronise.  Hosts that need every call to be
//     allocation-free make one warm-up call per device at start-up;
//   * problems whose scratch (B*2*H*W*L floats) exceeds that size are
//     rejected with BPL_ERR_INVALID_ARG;
//   * all calls share the one array per device, so calls whose work overlaps
//     on the GPU (different streams, or different host threads without
//     ordering) race on it and corrupt each other's results: serialise them.
//     Nothing in the array has to start at zero: each call writes every
//     element it reads (the vertical sweeps write the chain gradients,
//     including the zero rows at the image border, before the horizontal
//     sweeps read them), so contents left by a previous call are harmless;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress with that device current) and caches it per
//     device ordinal: only the device's primary context (the runtime API's
//     context, which torch uses) is supported.  Make that first call before
//     any stream capture.
#include <cuda_runtime.h>

#include <mutex>

#include "bpl_internal.h"

namespace bpl {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;  // 16 MiB per device

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (looked up once
// per device; the host-side name of the array is not a device address).
int scratch_address(void** out) {
  int dev = 0;
  BPL_CUDA_TRY(cudaGetDevice(&dev), "lbp_backward_noalloc: cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices)
    return set_error(BPL_ERR_UNSUPPORTED, "lbp_backward_noalloc: device %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    BPL_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch), "lbp_backward_noalloc: cudaGetSymbolAddress");
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return BPL_OK;
}

}  // namespace
}  // namespace bpl

extern "C" int bpl_lbp_backward_noalloc(int variant, const float* jump, const float* edge, const float* in_grad,
                                        const float* messages, const void* argmin, int argmin_kind,
                                        const float* scale, float* grad_cost, float* grad_jump,
                                        float* grad_edge, int B, int H, int W, int L, int Lv, int jump_batch,
                                        int edge_batch, void* stream) {
  BPL_TRACE("bpl_lbp_backward_noalloc");
  BPL_REQUIRE(B >= 1 && H >= 1 && W >= 1 && L >= 1, "lbp_backward_noalloc: bad shape B=%d H=%d W=%d L=%d", B, H,
              W, L);
  const size_t need = bpl_lbp_backward_workspace_size(B, H, W, L);
  BPL_REQUIRE(need <= bpl::kNoAllocScratchBytes,
              "lbp_backward_noalloc: scratch of %zu bytes (B*2*H*W*L floats) exceeds the fixed %zu-byte device "
              "array; use bpl_lbp_backward with a caller workspace",
              need, bpl::kNoAllocScratchBytes);
  void* scratch = nullptr;
  const int st = bpl::scratch_address(&scratch);
  if (st != BPL_OK) return st;
  return bpl_lbp_backward(variant, jump, edge, in_grad, messages, argmin, argmin_kind, scale, grad_cost,
                          grad_jump, grad_edge, scratch, bpl::kNoAllocScratchBytes, B, H, W, L, Lv, jump_batch,
                          edge_batch, stream);
}

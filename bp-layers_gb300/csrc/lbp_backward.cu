// C-ABI entry of the LBP reference adjoint (argument checks, output
// zero-fill, dispatch).
#include <algorithm>

#include "lbp_backward.cuh"

using namespace bpl;

extern "C" size_t bpl_lbp_backward_workspace_size(int B, int H, int W, int L) {
  if (B < 1 || H < 1 || W < 1 || L < 1) return 0;
  return static_cast<size_t>(B) * 2 * H * W * L * sizeof(float);
}

namespace {

// storage: 0 = float messages (reference layout), 1 = half messages with the
// label axis padded to Lp = L rounded up to 8
// Completes the exact message gradient (the pass's input messages) from
// what the horizontal adjoint sweeps left in gmsg: slot UP holds the h
// gradients of the horizontal senders (they read the input vertical
// messages at every pixel), slots LEFT at x=0 / RIGHT at x=W-1 the chain
// inputs' gradients.  Adds, where a slot is never written by the pass (its
// input passes through and is read by the sweeps there): the upstream
// gradient, and the vertical sweeps' h gradients (saved accumulators) --
// UP at y=0 (the DOWN sweep's chain input), DOWN at y=H-1, and both for the
// horizontal slots at the image's left and right columns.
__global__ void assemble_message_grad_kernel(const float* in_grad, const float* saved, float* gmsg, int B, int H,
                                             int W, int L, int Ls) {
  const int64_t HW = static_cast<int64_t>(H) * W;
  const int64_t HWL = HW * Ls;
  const int64_t total = static_cast<int64_t>(B) * HW * Ls;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int t = static_cast<int>(i % Ls);
    const int64_t pix = i / Ls;
    const int n = static_cast<int>(pix / HW);
    const int64_t pin = pix % HW;
    const int y = static_cast<int>(pin / W), x = static_cast<int>(pin % W);
    float* gm = gmsg + static_cast<int64_t>(n) * 4 * HWL + pin * Ls + t;
    const float* gi = in_grad + static_cast<int64_t>(n) * 4 * HWL + pin * Ls + t;
    if (t >= L) {
      gm[LEFT * HWL] = gm[RIGHT * HWL] = gm[UP * HWL] = gm[DOWN * HWL] = 0.0f;
      continue;
    }
    const float sU = saved[(static_cast<int64_t>(n) * 2 + 0) * HWL + pin * Ls + t];
    const float sD = saved[(static_cast<int64_t>(n) * 2 + 1) * HWL + pin * Ls + t];
    const float gh = gm[UP * HWL];
    gm[UP * HWL] = gh + ((y == 0) ? gi[UP * HWL] + sU : 0.0f);
    gm[DOWN * HWL] = gh + ((y == H - 1) ? gi[DOWN * HWL] + sD : 0.0f);
    gm[LEFT * HWL] = (x == 0) ? gm[LEFT * HWL] + gi[LEFT * HWL] + sU + sD : 0.0f;
    gm[RIGHT * HWL] = (x == W - 1) ? gm[RIGHT * HWL] + gi[RIGHT * HWL] + sU + sD : 0.0f;
  }
}

int lbp_backward_impl(int storage, int variant, const float* jump, const float* edge, const void* in_grad,
                      const void* messages, const void* argmin, int argmin_kind, const float* scale,
                      float* grad_cost, float* grad_jump, float* grad_edge, void* workspace, size_t workspace_bytes,
                      int B, int H, int W, int L, int Lv, int jump_batch, int edge_batch, void* stream,
                      float* grad_messages = nullptr, int reps = 1, int64_t g_bstride = -1,
                      int64_t g_sstride = -1, float cost_sign = 0.0f, int gc_ls = -1, int layer_taps = 0) {
  BPL_REQUIRE(variant >= 0 && variant <= 3, "lbp_backward: unknown variant %d", variant);
  // the pixel variant with the layer's two pairwise planes: same kernels, a
  // gradient of the planes' layout
  const int planes2 = (variant == BPL_LBP_SEM_PIXEL_LAYER) ? 1 : 0;
  if (planes2) variant = BPL_LBP_SEM_PIXEL;
  BPL_REQUIRE(B >= 1 && H >= 1 && W >= 1, "lbp_backward: bad shape B=%d H=%d W=%d", B, H, W);
  BPL_REQUIRE(H <= 65535 && W <= 65535, "lbp_backward: H and W must be <= 65535");
  BPL_REQUIRE(L >= 1 && L <= 1024, "lbp_backward: L=%d outside [1, 1024]", L);
  // the scale is part of the reference's signature (FP32 storage); FP16
  // storage recomputes the normalisation from the rows and takes NULL
  BPL_REQUIRE(edge && in_grad && messages && argmin && (scale || storage == 1) && grad_cost && grad_jump,
              "lbp_backward: null pointer");
  BPL_REQUIRE(variant == BPL_LBP_SEM_PIXEL || (jump && grad_edge), "lbp_backward: null jump/grad_edge");
  BPL_REQUIRE(argmin_kind >= BPL_ARGMIN_F32 && argmin_kind <= BPL_ARGMIN_U16, "lbp_backward: bad argmin kind");
  BPL_REQUIRE(edge_batch == 1 || edge_batch == B, "lbp_backward: edge batch %d must be 1 or B", edge_batch);
  const int Ls = (storage == 0) ? L : ((L + 7) & ~7);
  // cost_sign 0: grad_cost is an output (zeroed here, label stride Ls);
  // +-1: contributions are added, times cost_sign, onto what grad_cost holds
  // (label stride gc_ls, L or Ls)
  const bool accumulate = cost_sign != 0.0f;
  if (gc_ls < 0) gc_ls = Ls;
  BPL_REQUIRE(!accumulate || cost_sign == 1.0f || cost_sign == -1.0f, "lbp_backward: cost sign must be +-1");
  BPL_REQUIRE(gc_ls == Ls || gc_ls == L, "lbp_backward: cost-gradient label stride %d must be L or Ls", gc_ls);
  BPL_REQUIRE(reps >= 1 && (reps == 1 || grad_messages == nullptr), "lbp_backward: bad pass count %d", reps);
  BPL_REQUIRE(workspace && workspace_bytes >= reps * bpl_lbp_backward_workspace_size(B, H, W, Ls),
              "lbp_backward: workspace of %zu bytes needed", reps * bpl_lbp_backward_workspace_size(B, H, W, Ls));
  BPL_REQUIRE(!layer_taps || (variant == BPL_LBP_STEREO && Lv == 6),
              "lbp_backward: the layer's packed taps are stereo taps with Lv = 6");
  if (variant == BPL_LBP_STEREO) {
    BPL_REQUIRE(Lv >= 2 && Lv <= 16, "lbp_backward: Lv=%d outside [2, 16]", Lv);
    BPL_REQUIRE(jump_batch == 1 || jump_batch == B, "lbp_backward: jump batch %d must be 1 or B", jump_batch);
  }

  cudaStream_t s = as_stream(stream);
  const int64_t HW = static_cast<int64_t>(H) * W;
  size_t gj_elems;
  if (variant == BPL_LBP_STEREO) gj_elems = static_cast<size_t>(jump_batch) * 4 * Lv * HW;
  else if (variant == BPL_LBP_SEM_GLOBAL) gj_elems = static_cast<size_t>(B) * 4 * L * L;
  else gj_elems = static_cast<size_t>(planes2 ? 2 : 4) * HW * L * L;
  if (!accumulate)
    BPL_CUDA_TRY(cudaMemsetAsync(grad_cost, 0, sizeof(float) * B * HW * Ls, s), "lbp_backward: memset");
  BPL_CUDA_TRY(cudaMemsetAsync(grad_jump, 0, sizeof(float) * gj_elems, s), "lbp_backward: memset");
  if (grad_edge)
    BPL_CUDA_TRY(cudaMemsetAsync(grad_edge, 0, sizeof(float) * edge_batch * 4 * HW, s), "lbp_backward: memset");
  if (grad_messages)
    BPL_CUDA_TRY(cudaMemsetAsync(grad_messages, 0, sizeof(float) * B * 4 * HW * Ls, s), "lbp_backward: memset");

  BwdArgs a{};
  a.jump = jump;
  a.edge = edge;
  a.in_grad = in_grad;
  a.msgs = messages;
  a.argmin = argmin;
  a.scale = scale;
  a.grad_cost = grad_cost;
  a.grad_jump = grad_jump;
  a.grad_edge = grad_edge;
  a.saved = static_cast<float*>(workspace);
  a.gmsg = grad_messages;
  a.reps = reps;
  a.g_bstride = (g_bstride < 0) ? 4 * HW * Ls : g_bstride;
  a.g_sstride = (g_sstride < 0) ? HW * Ls : g_sstride;
  a.B = B;
  a.H = H;
  a.W = W;
  a.L = L;
  a.Ls = Ls;
  a.Lv = (variant == BPL_LBP_STEREO) ? Lv : 0;
  a.jb = jump_batch;
  a.eb = edge_batch;
  a.argmin_kind = argmin_kind;
  a.gc_ls = gc_ls;
  a.gc_sign = accumulate ? cost_sign : 1.0f;
  a.planes2 = planes2;
  a.layer_taps = layer_taps ? 1 : 0;
  const int am_size = (argmin_kind == BPL_ARGMIN_U8) ? 1 : (argmin_kind == BPL_ARGMIN_U16 ? 2 : 4);
  if (storage == 0) {
    a.lrow = bwd::a4(L);
    a.vec4 = (L % 4 == 0) ? 1 : 0;
  } else {
    a.lrow = Ls;
    a.vec4 = 1;
  }
  a.am_bulk = (a.vec4 && (Ls * am_size) % 16 == 0) ? 1 : 0;
  a.ns = 0;  // rows are prefetched into registers: no shared-memory ring
  if (storage == 1)
    return (variant == BPL_LBP_STEREO)       ? lbp_backward_stereo_f16(a, s)
           : (variant == BPL_LBP_SEM_GLOBAL) ? lbp_backward_sem_global_f16(a, s)
                                             : lbp_backward_sem_pixel_f16(a, s);
  int st;
  switch (variant) {
    case BPL_LBP_STEREO: st = lbp_backward_stereo(a, s); break;
    case BPL_LBP_SEM_GLOBAL: st = lbp_backward_sem_global(a, s); break;
    default: st = lbp_backward_sem_pixel(a, s); break;
  }
  if (st != BPL_OK || grad_messages == nullptr) return st;
  const int64_t total = static_cast<int64_t>(B) * HW * Ls;
  const int blocks = static_cast<int>(std::min<int64_t>((total + 255) / 256, 8 * 152 * 8));
  assemble_message_grad_kernel<<<blocks, 256, 0, s>>>(static_cast<const float*>(in_grad), a.saved, grad_messages, B,
                                                     H, W, L, Ls);
  BPL_CUDA_TRY(cudaGetLastError(), "lbp_backward: message-gradient launch");
  return BPL_OK;
}

}  // namespace

extern "C" int bpl_lbp_backward(int variant, const float* jump, const float* edge, const float* in_grad,
                                const float* messages, const void* argmin, int argmin_kind,
                                const float* scale, float* grad_cost, float* grad_jump, float* grad_edge,
                                void* workspace, size_t workspace_bytes, int B, int H, int W, int L,
                                int Lv, int jump_batch, int edge_batch, void* stream) {
  BPL_TRACE("bpl_lbp_backward");
  return lbp_backward_impl(0, variant, jump, edge, in_grad, messages, argmin, argmin_kind, scale, grad_cost,
                           grad_jump, grad_edge, workspace, workspace_bytes, B, H, W, L, Lv, jump_batch, edge_batch,
                           stream);
}

extern "C" int bpl_lbp_backward_exact(int variant, const float* jump, const float* edge, const float* in_grad,
                                      const float* messages, const void* argmin, int argmin_kind,
                                      const float* scale, float* grad_cost, float* grad_jump, float* grad_edge,
                                      float* grad_messages, void* workspace, size_t workspace_bytes, int B, int H,
                                      int W, int L, int Lv, int jump_batch, int edge_batch, void* stream) {
  BPL_TRACE("bpl_lbp_backward_exact");
  BPL_REQUIRE(grad_messages, "lbp_backward_exact: null grad_messages");
  return lbp_backward_impl(0, variant, jump, edge, in_grad, messages, argmin, argmin_kind, scale, grad_cost,
                           grad_jump, grad_edge, workspace, workspace_bytes, B, H, W, L, Lv, jump_batch, edge_batch,
                           stream, grad_messages);
}

extern "C" int bpl_lbp_backward_passes(int variant, const float* jump, const float* edge, const float* in_grad,
                                       int64_t in_grad_batch_stride, int64_t in_grad_slot_stride,
                                       const float* messages, const void* argmin, int argmin_kind,
                                       const float* scale, float* grad_cost, float* grad_jump, float* grad_edge,
                                       void* workspace, size_t workspace_bytes, int B, int H, int W, int L, int Lv,
                                       int jump_batch, int edge_batch, int passes, void* stream) {
  BPL_TRACE("bpl_lbp_backward_passes");
  BPL_REQUIRE(in_grad_batch_stride >= 0 && in_grad_slot_stride >= 0, "lbp_backward_passes: negative stride");
  return lbp_backward_impl(0, variant, jump, edge, in_grad, messages, argmin, argmin_kind, scale, grad_cost,
                           grad_jump, grad_edge, workspace, workspace_bytes, B, H, W, L, Lv, jump_batch, edge_batch,
                           stream, nullptr, passes, in_grad_batch_stride, in_grad_slot_stride);
}

extern "C" int bpl_lbp_backward_passes_f16(int variant, const float* jump, const float* edge, const void* in_grad,
                                           int64_t in_grad_batch_stride, int64_t in_grad_slot_stride,
                                           const void* messages, const void* argmin, int argmin_kind,
                                           const float* scale, float* grad_cost, float* grad_jump,
                                           float* grad_edge, void* workspace, size_t workspace_bytes, int B, int H,
                                           int W, int L, int Lv, int jump_batch, int edge_batch, int passes,
                                           void* stream) {
  BPL_TRACE("bpl_lbp_backward_passes_f16");
  BPL_REQUIRE(in_grad_batch_stride >= 0 && in_grad_slot_stride >= 0, "lbp_backward_passes: negative stride");
  return lbp_backward_impl(1, variant, jump, edge, in_grad, messages, argmin, argmin_kind, scale, grad_cost,
                           grad_jump, grad_edge, workspace, workspace_bytes, B, H, W, L, Lv, jump_batch, edge_batch,
                           stream, nullptr, passes, in_grad_batch_stride, in_grad_slot_stride);
}

extern "C" int bpl_lbp_backward_passes_into(int storage, int variant, const float* jump, const float* edge,
                                            const void* in_grad, int64_t in_grad_batch_stride,
                                            int64_t in_grad_slot_stride, const void* messages, const void* argmin,
                                            int argmin_kind, const float* scale, float* grad_cost, int grad_cost_ls,
                                            float cost_sign, float* grad_jump, float* grad_edge, void* workspace,
                                            size_t workspace_bytes, int B, int H, int W, int L, int Lv,
                                            int jump_batch, int edge_batch, int passes, int layer_taps,
                                            void* stream) {
  BPL_TRACE("bpl_lbp_backward_passes_into");
  BPL_REQUIRE(storage == 0 || storage == 1, "lbp_backward_passes_into: storage must be 0 or 1");
  BPL_REQUIRE(cost_sign == 1.0f || cost_sign == -1.0f, "lbp_backward_passes_into: cost sign must be +-1");
  BPL_REQUIRE(in_grad_batch_stride >= 0 && in_grad_slot_stride >= 0, "lbp_backward_passes: negative stride");
  BPL_REQUIRE(in_grad != grad_cost, "lbp_backward_passes_into: in_grad must not alias grad_cost");
  return lbp_backward_impl(storage, variant, jump, edge, in_grad, messages, argmin, argmin_kind, scale, grad_cost,
                           grad_jump, grad_edge, workspace, workspace_bytes, B, H, W, L, Lv, jump_batch, edge_batch,
                           stream, nullptr, passes, in_grad_batch_stride, in_grad_slot_stride, cost_sign,
                           grad_cost_ls, layer_taps);
}

extern "C" int bpl_lbp_backward_f16(int variant, const float* jump, const float* edge, const void* in_grad,
                                    const void* messages, const void* argmin, int argmin_kind, const float* scale,
                                    float* grad_cost, float* grad_jump, float* grad_edge, void* workspace,
                                    size_t workspace_bytes, int B, int H, int W, int L, int Lv, int jump_batch,
                                    int edge_batch, void* stream) {
  BPL_TRACE("bpl_lbp_backward_f16");
  return lbp_backward_impl(1, variant, jump, edge, in_grad, messages, argmin, argmin_kind, scale, grad_cost,
                           grad_jump, grad_edge, workspace, workspace_bytes, B, H, W, L, Lv, jump_batch, edge_batch,
                           stream);
}

// C-ABI entry of the min-sum LBP forward (argument checks and dispatch).
#include "lbp_forward.cuh"

namespace bpl {
__device__ int g_bpl_error = 0;
__device__ unsigned g_bpl_wait_limit = kWaitLimit;
__device__ __align__(16) float g_zero_pairwise[96 * 96];
}  // namespace bpl


using namespace bpl;

namespace {

// storage: 0 = float (reference layout), 1 = half (label stride rounded to 8)
int lbp_forward_impl(int storage, int variant, const void* cost, const void* jump, const float* edge,
                     void* messages, void* argmin, int argmin_kind, float* scale, int B, int H, int W, int L,
                     int Lv, int jump_batch, int edge_batch, int delta, void* stream) {
  BPL_REQUIRE(variant >= 0 && variant <= 3, "lbp_forward: unknown variant %d", variant);
  // the pixel variant with the layer's two pairwise planes: same kernels,
  // the shift and transpose applied when a matrix is staged
  const int planes2 = (variant == BPL_LBP_SEM_PIXEL_LAYER) ? 1 : 0;
  if (planes2) variant = BPL_LBP_SEM_PIXEL;
  BPL_REQUIRE(B >= 1 && H >= 1 && W >= 1, "lbp_forward: bad shape B=%d H=%d W=%d", B, H, W);
  BPL_REQUIRE(H <= 65535 && W <= 65535, "lbp_forward: H and W must be <= 65535");
  BPL_REQUIRE(L >= 1 && L <= 1024, "lbp_forward: L=%d outside [1, 1024]", L);
  // scale: required for FP32 storage (the reference's output), optional for
  // FP16 storage (its adjoint recomputes the normalisation from the rows)
  BPL_REQUIRE(cost && jump && edge && messages && (scale || storage == 1), "lbp_forward: null pointer");
  BPL_REQUIRE(delta >= 0 && delta <= 65535, "lbp_forward: delta=%d is not a uint16", delta);
  BPL_REQUIRE(edge_batch == 1 || edge_batch == B, "lbp_forward: edge batch %d must be 1 or B", edge_batch);
  BPL_REQUIRE(argmin_kind >= BPL_ARGMIN_NONE && argmin_kind <= BPL_ARGMIN_U16, "lbp_forward: bad argmin kind");
  BPL_REQUIRE(argmin_kind == BPL_ARGMIN_NONE || argmin, "lbp_forward: argmin pointer is null");
  BPL_REQUIRE(argmin_kind != BPL_ARGMIN_U8 || L <= 256, "lbp_forward: uint8 argmin needs L <= 256");
  if (variant == BPL_LBP_STEREO) {
    BPL_REQUIRE(Lv >= 2 && Lv <= 16, "lbp_forward: Lv=%d outside [2, 16]", Lv);
    BPL_REQUIRE(jump_batch == 1 || jump_batch == B, "lbp_forward: jump batch %d must be 1 or B", jump_batch);
  }

  FwdArgs a{};
  a.cost = cost;
  a.jump = jump;
  a.edge = edge;
  a.msgs = messages;
  a.argmin = argmin;
  a.scale = scale;
  a.B = B;
  a.H = H;
  a.W = W;
  a.L = L;
  a.Lv = (variant == BPL_LBP_STEREO) ? Lv : 0;
  a.jb = jump_batch;
  a.eb = edge_batch;
  a.delta = delta;
  a.argmin_kind = argmin_kind;
  a.planes2 = planes2;
  a.lrow = align4(L);
  if (storage == 0) {
    a.Ls = L;
    a.Lm = L;
    a.lmat = 0;
    a.vec4 = (L % 4 == 0) ? 1 : 0;
    if (variant == BPL_LBP_SEM_PIXEL && L <= kPixelRingMaxL) {
      a.lmat = align4(L * L);
      a.vec4 = a.vec4 && ((L * L) % 4 == 0);
    }
  } else {
    a.Ls = (L + 7) & ~7;
    a.Lm = a.Ls;
    a.lmat = (variant == BPL_LBP_SEM_PIXEL && L <= kPixelRingMaxL) ? L * a.Lm : 0;
    a.vec4 = 1;
  }
  // shared-memory ring (pixel variant up to kPixelRingMaxL labels): 4 steps
  // in flight, one step per mbarrier group; the other variants, and wider
  // pixel rows, prefetch rows into registers (wider pixel rows read their
  // matrices from global memory)
  a.ns = (variant == BPL_LBP_SEM_PIXEL && L <= kPixelRingMaxL) ? (a.vec4 ? 4 : kRingCpAsync) : 0;
  a.sps = 1;
  cudaStream_t s = as_stream(stream);
  if (storage == 1) {
    if (variant == BPL_LBP_STEREO) return lbp_forward_stereo_f16(a, s);
    return (variant == BPL_LBP_SEM_GLOBAL) ? lbp_forward_sem_global_f16(a, s) : lbp_forward_sem_pixel_f16(a, s);
  }
  switch (variant) {
    case BPL_LBP_STEREO: return lbp_forward_stereo(a, s);
    case BPL_LBP_SEM_GLOBAL: return lbp_forward_sem_global(a, s);
    default: return lbp_forward_sem_pixel(a, s);
  }
}

}  // namespace

extern "C" int bpl_lbp_forward(int variant, const float* cost, const float* jump, const float* edge,
                               float* messages, void* argmin, int argmin_kind, float* scale, int B,
                               int H, int W, int L, int Lv, int jump_batch, int edge_batch, int delta,
                               void* stream) {
  BPL_TRACE("bpl_lbp_forward");
  return lbp_forward_impl(0, variant, cost, jump, edge, messages, argmin, argmin_kind, scale, B, H, W, L, Lv,
                          jump_batch, edge_batch, delta, stream);
}

extern "C" int bpl_lbp_forward_f16(int variant, const void* cost, const void* jump, const float* edge,
                                   void* messages, void* argmin, int argmin_kind, float* scale, int B, int H,
                                   int W, int L, int Lv, int jump_batch, int edge_batch, int delta,
                                   void* stream) {
  BPL_TRACE("bpl_lbp_forward_f16");
  return lbp_forward_impl(1, variant, cost, jump, edge, messages, argmin, argmin_kind, scale, B, H, W, L, Lv,
                          jump_batch, edge_batch, delta, stream);
}

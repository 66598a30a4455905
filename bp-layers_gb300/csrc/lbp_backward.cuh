// Reference adjoint of the min-sum LBP pass for sm_103a (kernel template;
// instantiated per pairwise variant in lbp_backward_*.cu).
//
// Reference semantics: ops/lbp_stereo/src/lbp_min_sum_kernel.cu:215-417
// (kernel) and :513-621 (host loops: per batch item, reversed sweeps DOWN,
// UP, LEFT, RIGHT, one launch plus an at::zeros scratch allocation per
// column/row).  What the reference computes at a backward step (sender p,
// receiver q, message slot db at q, forward direction fd = db^1), per
// receiver label c:
//   add_hor = J^T in_grad[q] + J^T acc_HOR         (LSE Jacobian, :328-369)
//   add_up  = saved_UP[q] + acc_UP,  add_down = saved_DOWN[q] + acc_DOWN
//             (horizontal sweeps only, no Jacobian, :380-386)
//   s* = argmin[q][c]
//   grad_cost[p][s*] += add_hor + add_up + add_down
//   grad_jump[fd][tap(c - s*)][p] += w * (...), grad_edge[fd][p] += f(c,s*) * (...)
//   acc_X_new[s*] += add_X;  saved_db[p] = acc_HOR_new (:404-416)
// and grad_messages = in_grad (:534-536).
//
// GB300 design: one warp walks one scanline of one backward sweep, the
// accumulator stays in registers, the scatter "by argmin" goes through a
// per-warp shared-memory row with shared atomics, and the two sweeps of each
// orientation run concurrently (DOWN+UP, then LEFT+RIGHT): 2 launches per
// backward instead of 2(W-1)+2(H-1).  The J^T product is taken in O(L) as
// g_c - p_c * sum(g) instead of the reference's O(L^2) loop.
//
// One accumulator instead of HOR/UP/DOWN.  acc_UP/acc_DOWN are scatters of
// the saved vertical accumulators, which are themselves scatters of J^T
// outputs; J^T = I - p 1^T produces vectors that sum to zero and a scatter
// keeps the sum, so J^T leaves acc_UP + saved_UP unchanged.  Applying J^T
// to (in_grad + saved_UP + saved_DOWN + acc) in a single accumulator
// therefore gives the reference's sums, up to float rounding, with a third
// of the scatter atomics and row traffic.
#pragma once
#include <cuda_runtime.h>

#include <cuda_fp16.h>

#include <algorithm>

#include "bpl_device.cuh"
#include "bpl_internal.h"

namespace bpl {

// Messages and their upstream gradient are stored as T (float, or __half
// with the label axis padded to Ls = L rounded up to 8); everything else is
// float.  Ls is the label stride of messages, in_grad, argmin, grad_cost and
// the workspace.
struct BwdArgs {
  const float* jump;
  const float* edge;
  const void* in_grad;
  const void* msgs;
  const void* argmin;
  const float* scale;
  float* grad_cost;
  float* grad_jump;
  float* grad_edge;
  float* saved;  // workspace (B,2,H,W,L): slot 0 = UP chain, slot 1 = DOWN chain
  // exact adjoint only (else null): (B,4,H,W,Ls) float message gradient.
  // The horizontal sweeps add each sender's h gradient to slot UP (the
  // vertical input messages they read) and write it at their first sender
  // to their own slot (the chain input); bpl_lbp_assemble_message_grad
  // completes it.
  float* gmsg;
  int B, H, W, L, Lv, jb, eb;
  // passes sharing messages and in_grad (the reference adjoint of an
  // in-place iteration loop): argmin, scale and the workspace are stacked
  // (reps, B, ...); the chains of all passes run in one launch and their
  // gradients accumulate into the same outputs
  int reps;
  // in_grad strides (elements) between batch items and between message
  // slots: 4*H*W*Ls and H*W*Ls for a (B,4,H,W,Ls) tensor; a slot stride of
  // 0 reads one (B,H,W,Ls) gradient for every slot (the beliefs' gradient
  // broadcast over the four messages)
  int64_t g_bstride, g_sstride;
  int Ls;
  int argmin_kind;
  // grad_cost: label stride (Ls, or L for a gradient accumulated onto the
  // layer's (B,H,W,L) cost gradient) and the sign its contributions are
  // added with (+1; -1 when the buffer holds the gradient of -cost)
  int gc_ls;
  float gc_sign;
  // jump holds the stereo layer's packed taps [offset, L2, L1, 0, L1, L2]
  // (Lv = 6): taps 1 and 5 carry the same value and the layer's fold adds
  // their gradients, tap 3 is 0 and its gradient is dropped.  The adjoint
  // then bins three ways (|d| >= 2, d = -1, d = +1) and writes the L2
  // gradient to tap 1 only, nothing to taps 3 and 5.
  int layer_taps;
  int phase;  // 0: DOWN+UP over columns, 1: LEFT+RIGHT over rows
  int nchains;
  int ns;
  int lrow;
  int vec4;     // float rows are 16-byte sized: bulk copies
  int am_bulk;  // the argmin row is 16-byte sized too: staged with the floats
  // pixel variant: grad_jump is the layer's (2,H,W,L,L) LR / UD planes; the
  // gradient of direction RL goes to the LR matrix of the pixel to the left,
  // transposed, DU to the UD matrix above, transposed, and the zero matrix
  // of a first RL / DU sender receives none (message_passing_op_pw_pixel.py:
  // 47-51)
  int planes2;
};

constexpr int kBwdRingCpAsync = 4;

namespace bwd {

__host__ __device__ inline int a4(int v) { return (v + 3) & ~3; }

// rows per stage: messages and in_grad (T), saved UP and saved DOWN (float)
// and the argmin row (up to 4 bytes per label), each lrow labels long
__host__ __device__ inline int stage_floats(int lrow, int tsize) { return 2 * lrow * tsize / 4 + 3 * lrow; }

__host__ __device__ inline int tile_floats(int Lv) { return a4(2 * (Lv + 2) * 33); }

__host__ __device__ inline int warp_smem_floats(int K, int ns, int lrow, int Lv, int L, int variant, int tsize) {
  const int ring = ns * stage_floats(lrow, tsize);
  const int bars = 2 * a4(ns);
  const int rows = 3 * 32 * K;                      // scatter rows of acc HOR/UP/DOWN
  const int jacc = (variant == BPL_LBP_SEM_GLOBAL) ? a4(L * L) : 0;
  return a4(ring) + bars + rows + jacc + tile_floats(Lv);
}

struct Smem {
  float* ring;
  uint64_t* bars;
  float* rows;  // [3][32K]
  float* jacc;  // [L*L] (semantic global)
  float* tile;  // [2][Lv+2][33]: taps, edge weight, scale
};

template <int K>
__device__ __forceinline__ Smem carve(float* base, const BwdArgs& a, int variant, int tsize) {
  Smem s;
  s.ring = base;
  float* p = base + a4(a.ns * stage_floats(a.lrow, tsize));
  s.bars = reinterpret_cast<uint64_t*>(p);
  p += 2 * a4(a.ns);
  s.rows = p;
  p += 3 * 32 * K;
  s.jacc = p;
  if (variant == BPL_LBP_SEM_GLOBAL) p += a4(a.L * a.L);
  s.tile = p;
  return s;
}

}  // namespace bwd

// LV: number of stereo jump taps when known at compile time (6 or 8), 16 for
// any Lv <= 16 given at run time, 0 for the semantic variants.  CROSS: the
// horizontal phase (LEFT+RIGHT, with the vertical chains' saved gradients).
template <typename T>
__device__ __forceinline__ float bldf(T v);
template <>
__device__ __forceinline__ float bldf<float>(float v) { return v; }
template <>
__device__ __forceinline__ float bldf<__half>(__half v) { return __half2float(v); }

// The vertical phase (one scanline per column) runs 2-warp blocks, 9 of
// them resident per SM (18 warps).  The horizontal phase runs 4-warp blocks,
// 4 resident per SM (registers capped near 128): with the passes of an
// iteration loop batched its scanlines number 2 * passes * rows (2256 at
// 3 x 376 rows), which 16 warps per SM hold in one wave; uncapped (161
// registers, 12 warps per SM) the last quarter ran as a second wave of
// full-length chains.
template <bool CROSS, int K>
constexpr int bwd_warps_per_block() { return (CROSS || K > 8) ? 4 : 2; }
template <bool CROSS, int K>
constexpr int bwd_min_blocks() { return K > 8 ? 1 : (CROSS ? 4 : 9); }

template <int K, int VARIANT, int LV, bool CROSS, typename T, bool LT = false>
__global__ void __launch_bounds__(32 * bwd_warps_per_block<CROSS, K>(), bwd_min_blocks<CROSS, K>())
    lbp_backward_kernel(BwdArgs a) {
  static_assert(!LT || (VARIANT == BPL_LBP_STEREO && LV == 6), "layer taps: stereo, 6 taps");
  using namespace bwd;
  extern __shared__ __align__(16) float smem[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int chain_id = blockIdx.x * (blockDim.x >> 5) + wib;
  if (chain_id >= a.nchains) return;

  const int per_warp = warp_smem_floats(K, a.ns, a.lrow, a.Lv, a.L, VARIANT, sizeof(T));
  Smem sm = carve<K>(smem + static_cast<int64_t>(wib) * per_warp, a, VARIANT, sizeof(T));

  const int L = a.L;
  const int Ls = a.Ls;
  const int64_t HW = static_cast<int64_t>(a.H) * a.W;
  const int64_t HWL = HW * Ls;
  // chain: sender of step k is pin0 + k*dpin (pixel index within the image),
  // its receiver is dq further
  int n, v, db, pin0, dpin, dq, nsteps;  // v: pass-major item of argmin/scale/workspace, n: batch item
  {
    const int r = chain_id >> 1;
    if (!CROSS) {
      db = (chain_id & 1) ? UP : DOWN;
      v = r / a.W;
      const int x = r % a.W;
      nsteps = a.H - 1;
      pin0 = (db == DOWN) ? a.W + x : (a.H - 2) * a.W + x;  // DOWN: y = 1.., UP: y = H-2..
      dpin = (db == DOWN) ? a.W : -a.W;
      dq = -dpin;
    } else {
      db = (chain_id & 1) ? RIGHT : LEFT;
      v = r / a.H;
      const int y = r % a.H;
      nsteps = a.W - 1;
      pin0 = (db == LEFT) ? y * a.W + a.W - 2 : y * a.W + 1;  // LEFT: x = W-2.., RIGHT: x = 1..
      dpin = (db == LEFT) ? -1 : 1;
      dq = -dpin;
    }
    n = v % a.B;
  }
  const int fd = db ^ 1;
  const bool stereo = (VARIANT == BPL_LBP_STEREO);
  // label validity: only the last slot can hold labels >= L when K = ceil(L/32) (the
  // stereo and global dispatch is exact up to K = 8; the pixel variant's
  // K = 8 and 32 serve several label counts and test every slot)
  auto lvalid = [&](int kk) -> bool {
    return (VARIANT != BPL_LBP_SEM_PIXEL && K <= 8 && kk < K - 1) || (lane + 32 * kk < L);
  };
  const int nj = (a.jb == 1) ? 0 : n;
  const int ne = (a.eb == 1) ? 0 : n;
  const uint32_t am_size = (a.argmin_kind == BPL_ARGMIN_U8) ? 1u : (a.argmin_kind == BPL_ARGMIN_U16 ? 2u : 4u);
  const T* msgs_db = static_cast<const T*>(a.msgs) + (static_cast<int64_t>(n) * 4 + db) * HWL;
  const T* grad_db = static_cast<const T*>(a.in_grad) + n * a.g_bstride + db * a.g_sstride;
  const uint8_t* am_db = static_cast<const uint8_t*>(a.argmin) + (static_cast<int64_t>(v) * 4 + db) * HWL * am_size;
  const float* saved_up = a.saved + (static_cast<int64_t>(v) * 2 + 0) * HWL;
  const float* saved_dn = a.saved + (static_cast<int64_t>(v) * 2 + 1) * HWL;
  float* saved_out = a.saved + (static_cast<int64_t>(v) * 2 + (db == UP ? 0 : 1)) * HWL;
  float* gcost_n = a.grad_cost + static_cast<int64_t>(n) * HW * a.gc_ls;
  const float* edge_fd = a.edge + (static_cast<int64_t>(ne) * 4 + fd) * HW;
  const float* jump_fd = stereo ? a.jump + (static_cast<int64_t>(nj) * 4 + fd) * a.Lv * HW : nullptr;
  float* gjump_fd = stereo ? a.grad_jump + (static_cast<int64_t>(nj) * 4 + fd) * a.Lv * HW : nullptr;
  float* gedge_fd = (VARIANT != BPL_LBP_SEM_PIXEL) ? a.grad_edge + (static_cast<int64_t>(ne) * 4 + fd) * HW : nullptr;

  // saved rows never written by a sender are read as zero by the horizontal
  // sweeps: the DOWN chain's row 0 and the UP chain's row H-1
  if (!CROSS) {
    const int x = (chain_id >> 1) % a.W;
    float* dst = saved_out + (static_cast<int64_t>((db == DOWN) ? 0 : a.H - 1) * a.W + x) * Ls;
    for (int t = lane; t < L; t += 32) dst[t] = 0.0f;
  }
  if (nsteps <= 0) return;

  // zero scatter rows / accumulators
  for (int t = lane; t < 3 * 32 * K; t += 32) sm.rows[t] = 0.0f;
  if (VARIANT == BPL_LBP_SEM_GLOBAL)
    for (int t = lane; t < L * L; t += 32) sm.jacc[t] = 0.0f;

  // The next step's rows (messages and in_grad as T, the argmin, the saved
  // vertical gradients) are prefetched into registers one step ahead:
  // coalesced loads of data no sweep of this phase writes.  They stay raw
  // until used, so the loads do not stall the step that issues them.
  T pm_[K], pg_[K];
  uint32_t pa_[K];
  float pu_[K], pd_[K];
  auto prefetch = [&](int k) {
    const int64_t qo = static_cast<int64_t>(pin0 + k * dpin + dq) * Ls;
    if (a.argmin_kind == BPL_ARGMIN_U8) {
      const uint8_t* ab = am_db + qo;
#pragma unroll
      for (int kk = 0; kk < K; ++kk) pa_[kk] = __ldg(ab + (lvalid(kk) ? lane + 32 * kk : 0));
    } else if (a.argmin_kind == BPL_ARGMIN_U16) {
      const uint16_t* ab = reinterpret_cast<const uint16_t*>(am_db) + qo;
#pragma unroll
      for (int kk = 0; kk < K; ++kk) pa_[kk] = __ldg(ab + (lvalid(kk) ? lane + 32 * kk : 0));
    } else {
      const float* ab = reinterpret_cast<const float*>(am_db) + qo;
#pragma unroll
      for (int kk = 0; kk < K; ++kk)
        pa_[kk] = __float_as_uint(__ldg(ab + (lvalid(kk) ? lane + 32 * kk : 0)));
    }
#pragma unroll
    for (int kk = 0; kk < K; ++kk) {
      const int t = lane + 32 * kk;
      const int64_t o = qo + (lvalid(kk) ? t : 0);  // labels >= L read label 0 (ignored)
      pm_[kk] = __ldg(msgs_db + o);
      pg_[kk] = __ldg(grad_db + o);
      if (CROSS) {
        pu_[kk] = __ldg(saved_up + o);
        pd_[kk] = __ldg(saved_dn + o);
      }
    }
  };

  // per-step tile: stereo taps (Lv rows), edge weight (row Lv); row Lv+1 is
  // unused (the normalisation's Jacobian needs no scale: see below)
  const int trow = a.Lv + 2;
  // Loaded 32 steps ahead and written to the tile when its block starts; the
  // registers are not read before then, so the loads never stall a step.
  // Constant register indices (a run-time index would put rg on the stack);
  // NR of them, the tap count when it is a compile-time constant.
  constexpr int NR = (LV == 6 || LV == 8) ? LV : 16;
  float ev = 0.0f;
  auto load_tile_regs = [&](int b, float (&rg)[NR]) {
    const int k = min(32 * b + lane, nsteps - 1);  // lanes past the end reload the last step
    const int p = pin0 + k * dpin;
    ev = __ldg(edge_fd + p);
    if (stereo) {
#pragma unroll
      for (int j = 0; j < NR; ++j)
        if (NR == LV || j < a.Lv) rg[j] = __ldg(jump_fd + static_cast<int64_t>(j) * HW + p);
    }
  };
  auto store_tile = [&](float* tile, const float (&rg)[NR]) {
    if (stereo) {
#pragma unroll
      for (int j = 0; j < NR; ++j)
        if (NR == LV || j < a.Lv) tile[j * 33 + lane] = rg[j];
    }
    tile[a.Lv * 33 + lane] = ev;
  };

  prefetch(0);
  float rg[NR];
#pragma unroll
  for (int j = 0; j < NR; ++j) rg[j] = 0.0f;
  load_tile_regs(0, rg);
  store_tile(sm.tile, rg);
  if (nsteps > 32) load_tile_regs(1, rg);
  __syncwarp();

  float accH[K];
#pragma unroll
  for (int k = 0; k < K; ++k) accH[k] = 0.0f;
  float* rowH = sm.rows;
  const bool am_f32 = a.argmin_kind == BPL_ARGMIN_F32;

  int p = pin0;
  for (int k = 0; k < nsteps; ++k, p += dpin) {
    const int j = k & 31;
    const int b = k >> 5;
    const float* tile = sm.tile + (b & 1) * (trow * 33);

    const float w = tile[a.Lv * 33 + j];
    float g[K], pr[K];
    int am[K];
    float sg = 0.0f, sa = 0.0f, se = 0.0f;
#pragma unroll
    for (int kk = 0; kk < K; ++kk) {
      const bool valid = lvalid(kk);
      am[kk] = valid ? (am_f32 ? static_cast<int>(__uint_as_float(pa_[kk])) : static_cast<int>(pa_[kk])) : 0;
      // horizontal sweeps: the vertical chains' saved gradients join in_grad
      // in the one accumulator (see the kernel's comment on the vertical
      // accumulators)
      g[kk] = valid ? (CROSS ? (bldf<T>(pg_[kk]) + pu_[kk]) + pd_[kk] : bldf<T>(pg_[kk])) : 0.0f;
      // exp(m_raw) / S of the reference (:328-341), with m_raw rebuilt from
      // the saved message plus log S, is exp(m) of the saved normalised
      // message m: the messages' softmax over labels, whatever pass S came
      // from.  Float rows are normalised (p = exp(m)); half rows hold
      // m_raw - min h of the last pass, a constant away, so p = exp(row) /
      // sum(exp(row)) with the sum taken here (se)
      pr[kk] = valid ? __expf(bldf<T>(pm_[kk])) : 0.0f;
      se += pr[kk];
      sg += g[kk];
      sa += accH[kk];
    }
    if (k + 1 < nsteps) prefetch(k + 1);

    if (sizeof(T) == 4) {
      // both sums in one reduce-scatter: lanes < 16 end with sum(g), the
      // others with sum(accH)
      float v = (lane & 16) ? sa : sg;
      const float o = __shfl_xor_sync(FULL, (lane & 16) ? sg : sa, 16);
      v += o;
#pragma unroll
      for (int o2 = 8; o2 > 0; o2 >>= 1) v += __shfl_xor_sync(FULL, v, o2);
      sg = __shfl_sync(FULL, v, 0);
      sa = __shfl_sync(FULL, v, 16);
    } else {
      // three sums in one reduce-scatter: lanes 0-7 end with sum(g), 8-15
      // with sum(accH), 16-23 with sum(exp(row)); p = exp(row) / se, so the
      // two sums are scaled instead of every p
      const bool h16 = lane & 16, h8 = lane & 8;
      const float w0 = (h16 ? se : sg) + __shfl_xor_sync(FULL, h16 ? sg : se, 16);
      const float w1 = (h16 ? 0.0f : sa) + __shfl_xor_sync(FULL, h16 ? sa : 0.0f, 16);
      float v = (h8 ? w1 : w0) + __shfl_xor_sync(FULL, h8 ? w0 : w1, 8);
#pragma unroll
      for (int o2 = 4; o2 > 0; o2 >>= 1) v += __shfl_xor_sync(FULL, v, o2);
      const float inv_s = 1.0f / __shfl_sync(FULL, v, 16);
      sg = __shfl_sync(FULL, v, 0) * inv_s;
      sa = __shfl_sync(FULL, v, 8) * inv_s;
    }
    float addH[K], addU[K], addD[K];
#pragma unroll
    for (int kk = 0; kk < K; ++kk) {
      addH[kk] = (g[kk] - pr[kk] * sg) + (accH[kk] - pr[kk] * sa);
      addU[kk] = 0.0f;
      addD[kk] = 0.0f;
    }

    // Scatter by argmin.  Most labels share one argmin (the label of the
    // global minimum of h, for every label farther than the truncation window
    // from it): that group is summed with warp shuffles, the few others go
    // through shared-memory atomics with little contention.
    // the slot of label L-1: K-1 where K = ceil(L/32) (the stereo and global
    // dispatch), else from L
    const int kL = (VARIANT != BPL_LBP_SEM_PIXEL && K <= 8) ? K - 1 : ((L - 1) >> 5);
    int amL = 0;
#pragma unroll
    for (int kk = 0; kk < K; ++kk)
      if (kk == kL) amL = am[kk];
    const int g0 = __shfl_sync(FULL, am[0], 0);
    const int gL = __shfl_sync(FULL, amL, (L - 1) & 31);
    // the dominant group: the first and last labels' shared argmin (labels
    // far from the window winners take the global minimum's label), else the
    // larger of their two groups
    int gd = g0;
    if (g0 != gL) {
      int c0 = 0, cL = 0;
#pragma unroll
      for (int kk = 0; kk < K; ++kk) {
        const bool v = lvalid(kk);
        c0 += (v && am[kk] == g0) ? 1 : 0;
        cL += (v && am[kk] == gL) ? 1 : 0;
      }
      c0 = __reduce_add_sync(FULL, c0);
      cL = __reduce_add_sync(FULL, cL);
      gd = (c0 >= cL) ? g0 : gL;
    }
    float dsum[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) dsum[q] = 0.0f;
    bool any_nd = false;
#pragma unroll
    for (int kk = 0; kk < K; ++kk) {
      const bool v = lvalid(kk);
      const bool dom = v && am[kk] == gd;
      dsum[0] += dom ? addH[kk] : 0.0f;
      any_nd = any_nd || (v && !dom);
    }
    if (__any_sync(FULL, any_nd)) {
#pragma unroll
      for (int kk = 0; kk < K; ++kk)
        if (lvalid(kk) && am[kk] != gd) atomicAdd(&rowH[am[kk]], addH[kk]);
    }

    // pairwise and edge gradients: per-tap sums of the total contribution,
    // tap index clamp(Lv/2 + t - s*), reduced together with the dominant
    // group's sums (tap bins in values 3..7 for Lv <= 6, else a second pass)
    float ge = 0.0f;
    if (LT) {
      // the layer's taps: bins |d| >= 2 (taps 1 and 5), d = -1 (tap 2),
      // d = +1 (tap 4), d = t - s*; reduced with the dominant sum (values
      // 0..3 at lanes 0, 8, 16, 24)
      float v4[4] = {dsum[0], 0.0f, 0.0f, 0.0f};
#pragma unroll
      for (int kk = 0; kk < K; ++kk) {
        const int d = lane + 32 * kk - am[kk];
        const float tot = lvalid(kk) ? addH[kk] : 0.0f;
        v4[1] += (static_cast<unsigned>(d + 1) > 2u) ? tot : 0.0f;
        v4[2] += (d == -1) ? tot : 0.0f;
        v4[3] += (d == 1) ? tot : 0.0f;
      }
      const float r = warp_reduce_scatter4(v4, lane);
      const int q = (lane >> 3) & 3;
      if ((lane & 7) == 0 && q >= 1) {
        const int bb = (q == 1) ? 1 : (q == 2 ? 2 : 4);
        ge = tile[bb * 33 + j] * r;
        if (r != 0.0f) atomicAdd(gjump_fd + static_cast<int64_t>(bb) * HW + p, w * r);
      }
      if (lane == 0) rowH[gd] += r;  // no other lane touches label gd
      ge = warp_sum(ge);
      if (lane == 0 && ge != 0.0f) atomicAdd(gedge_fd + p, ge);
    } else if (stereo) {
      constexpr int NB = (LV > 0) ? LV : 16;
      const int lv = (LV == 6 || LV == 8) ? LV : a.Lv;
      float bins[NB];
#pragma unroll
      for (int bb = 0; bb < NB; ++bb) bins[bb] = 0.0f;
#pragma unroll
      for (int kk = 0; kk < K; ++kk) {
        const int t = lane + 32 * kk;
        const float tot = lvalid(kk) ? (addH[kk] + addU[kk]) + addD[kk] : 0.0f;
        const int ti = max(1, min(lv - 1, lv / 2 + (t - am[kk])));
#pragma unroll
        for (int bb = 1; bb < NB; ++bb)
          if (LV == 6 || LV == 8 || bb < lv) bins[bb] += (ti == bb) ? tot : 0.0f;
      }
      if (LV == 6) {
        // values 0..2: dominant sums, 3..7: taps 1..5
#pragma unroll
        for (int bb = 1; bb < 6; ++bb) dsum[2 + bb] = bins[bb];
        const float r = warp_reduce_scatter8(dsum, lane);
        const int q = (lane >> 2) & 7;
        if ((lane & 3) == 0 && q >= 3) {
          const int bb = q - 2;
          ge = tile[bb * 33 + j] * r;
          if (r != 0.0f) atomicAdd(gjump_fd + static_cast<int64_t>(bb) * HW + p, w * r);
        }
        if (lane == 0) rowH[gd] += r;  // no other lane touches label gd
      } else {
        const float r = warp_reduce_scatter8(dsum, lane);
        if (lane == 0) rowH[gd] += r;
        // taps 1..NB-1 in passes of 8
#pragma unroll
        for (int b0 = 0; b0 < NB; b0 += 8) {
          float tv[8];
#pragma unroll
          for (int q = 0; q < 8; ++q) tv[q] = (b0 + q >= 1 && b0 + q < NB) ? bins[(b0 + q < NB) ? b0 + q : 0] : 0.0f;
          const float rb = warp_reduce_scatter8(tv, lane);
          const int bb = b0 + ((lane >> 2) & 7);
          if ((lane & 3) == 0 && bb >= 1 && bb < lv) {
            ge += tile[bb * 33 + j] * rb;
            if (rb != 0.0f) atomicAdd(gjump_fd + static_cast<int64_t>(bb) * HW + p, w * rb);
          }
        }
      }
      ge = warp_sum(ge);
      if (lane == 0 && ge != 0.0f) atomicAdd(gedge_fd + p, ge);
    } else {
      const float r = warp_reduce_scatter8(dsum, lane);
      if (lane == 0) rowH[gd] += r;
#pragma unroll
      for (int kk = 0; kk < K; ++kk) {
        const int t = lane + 32 * kk;
        if (t < L) {
          const float tot = (addH[kk] + addU[kk]) + addD[kk];
          const int s = am[kk];
          if (VARIANT == BPL_LBP_SEM_GLOBAL) {
            sm.jacc[s * L + t] += w * tot;  // distinct t per lane: no conflict
            ge += __ldg(a.jump + (static_cast<int64_t>(fd) * L + s) * L + t) * tot;
          } else if (!a.planes2) {
            // (4,H,W,L,L) has no batch axis: batch items accumulate
            atomicAdd(a.grad_jump + ((static_cast<int64_t>(fd) * HW + p) * L + s) * L + t, w * tot);
          } else if (!(fd & 1)) {
            atomicAdd(a.grad_jump + ((static_cast<int64_t>(fd >> 1) * HW + p) * L + s) * L + t, w * tot);
          } else if (fd == RIGHT ? (p % a.W != 0) : (p >= a.W)) {
            const int pp = p - (fd == RIGHT ? 1 : a.W);
            atomicAdd(a.grad_jump + ((static_cast<int64_t>(fd >> 1) * HW + pp) * L + t) * L + s, w * tot);
          }
        }
      }
      if (VARIANT == BPL_LBP_SEM_GLOBAL) {
        ge = warp_sum(ge);
        if (lane == 0) atomicAdd(gedge_fd + p, ge);
      }
    }
    __syncwarp();

    // read back the chain accumulators (and clear the rows for the next
    // step); grad_cost[p][s] receives the row.  The rows are 32K
    // long, so labels >= L read zeros.
    float* gc = gcost_n + static_cast<int64_t>(p) * a.gc_ls;
#pragma unroll
    for (int kk = 0; kk < K; ++kk) {
      const int t = lane + 32 * kk;
      accH[kk] = rowH[t];
      rowH[t] = 0.0f;
      const float v = accH[kk];
      if (lvalid(kk) && v != 0.0f) atomicAdd(gc + t, a.gc_sign * v);
      if (!CROSS && lvalid(kk)) saved_out[static_cast<int64_t>(p) * Ls + t] = accH[kk];
      if (CROSS && a.gmsg != nullptr && lvalid(kk)) {
        float* gm = a.gmsg + static_cast<int64_t>(n) * 4 * HWL;
        if (v != 0.0f) atomicAdd(gm + UP * HWL + static_cast<int64_t>(p) * Ls + t, v);
        if (k == nsteps - 1) gm[db * HWL + static_cast<int64_t>(p) * Ls + t] = v;
      }
    }

    if (j == 31 || k == nsteps - 1) {
      __syncwarp();
      if (32 * (b + 1) < nsteps) {
        store_tile(sm.tile + ((b + 1) & 1) * (trow * 33), rg);
        if (32 * (b + 2) < nsteps) load_tile_regs(b + 2, rg);
      }
    }
    __syncwarp();
  }

  if (VARIANT == BPL_LBP_SEM_GLOBAL) {
    // global pairwise gradient: summed over batch items into item 0, as the
    // reference does (ops/lbp_semantic_pw/src/lbp_min_sum_kernel.cu:395-397)
    __syncwarp();
    for (int t = lane; t < L * L; t += 32) {
      const float v = sm.jacc[t];
      if (v != 0.0f) atomicAdd(a.grad_jump + static_cast<int64_t>(fd) * L * L + t, v);
    }
  }
}

template <int K, int V, int LV, typename T>
int launch_bwd_k(const BwdArgs& a0, cudaStream_t stream) {
  BwdArgs a = a0;
  const int per_warp = bwd::warp_smem_floats(K, a.ns, a.lrow, a.Lv, a.L, V, sizeof(T)) * 4;
  for (int phase = 0; phase < 2; ++phase) {
    BPL_TRACE(phase == 0 ? "lbp_backward: vertical sweeps" : "lbp_backward: horizontal sweeps");
    auto kern = (phase == 0) ? lbp_backward_kernel<K, V, LV, false, T> : lbp_backward_kernel<K, V, LV, true, T>;
    if constexpr (V == BPL_LBP_STEREO && LV == 6 && K <= 8) {
      if (a.layer_taps)
        kern = (phase == 0) ? lbp_backward_kernel<K, V, LV, false, T, true> : lbp_backward_kernel<K, V, LV, true, T, true>;
    }
    const int wmax = (phase == 0) ? bwd_warps_per_block<false, K>() : bwd_warps_per_block<true, K>();
    const int wpb = std::max(1, std::min(wmax, (200 * 1024) / per_warp));
    const size_t smem = static_cast<size_t>(per_warp) * wpb;
    if (smem > 48 * 1024) {
      if (static_cast<int>(smem) > max_smem_optin())
        return set_error(BPL_ERR_UNSUPPORTED, "lbp_backward: shared memory %zu exceeds device limit", smem);
      BPL_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)),
                   "cudaFuncSetAttribute");
    }
    a.phase = phase;
    a.nchains = 2 * a.B * a.reps * (phase == 0 ? a.W : a.H);
    const int blocks = (a.nchains + wpb - 1) / wpb;
    kern<<<blocks, 32 * wpb, smem, stream>>>(a);
    BPL_CUDA_TRY(cudaGetLastError(), "lbp_backward launch");
  }
  return BPL_OK;
}

template <int V, int LV, typename T = float>
int dispatch_bwd(const BwdArgs& a, cudaStream_t s) {
  const int k = (a.L + 31) / 32;
  if constexpr (V == BPL_LBP_SEM_PIXEL) {
    if (k == 1) return launch_bwd_k<1, V, LV, T>(a, s);
    if (k == 2) return launch_bwd_k<2, V, LV, T>(a, s);
    if (k == 3) return launch_bwd_k<3, V, LV, T>(a, s);
    if (k <= 8) return launch_bwd_k<8, V, LV, T>(a, s);
    return launch_bwd_k<32, V, LV, T>(a, s);
  }
  switch (k) {
    case 1: return launch_bwd_k<1, V, LV, T>(a, s);
    case 2: return launch_bwd_k<2, V, LV, T>(a, s);
    case 3: return launch_bwd_k<3, V, LV, T>(a, s);
    case 4: return launch_bwd_k<4, V, LV, T>(a, s);
    case 5: return launch_bwd_k<5, V, LV, T>(a, s);
    case 6: return launch_bwd_k<6, V, LV, T>(a, s);
    case 7: return launch_bwd_k<7, V, LV, T>(a, s);
    case 8: return launch_bwd_k<8, V, LV, T>(a, s);
    default:
      if (k <= 12) return launch_bwd_k<12, V, LV, T>(a, s);
      if (k <= 16) return launch_bwd_k<16, V, LV, T>(a, s);
      if (k <= 24) return launch_bwd_k<24, V, LV, T>(a, s);
      return launch_bwd_k<32, V, LV, T>(a, s);
  }
}

int lbp_backward_stereo_lv6(const BwdArgs& a, cudaStream_t s);
int lbp_backward_stereo_lv8(const BwdArgs& a, cudaStream_t s);
int lbp_backward_stereo(const BwdArgs& a, cudaStream_t s);
int lbp_backward_stereo_f16(const BwdArgs& a, cudaStream_t s);
int lbp_backward_sem_pixel_f16(const BwdArgs& a, cudaStream_t s);
int lbp_backward_sem_global_f16(const BwdArgs& a, cudaStream_t s);
int lbp_backward_sem_global(const BwdArgs& a, cudaStream_t s);
int lbp_backward_sem_pixel(const BwdArgs& a, cudaStream_t s);

}  // namespace bpl

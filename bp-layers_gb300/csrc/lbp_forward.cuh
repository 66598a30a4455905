// Min-sum LBP forward for sm_103a: persistent warp-per-scanline sweeps.
// (kernel template; instantiated per pairwise variant in lbp_forward_*.cu)
//
// Reference semantics: ops/lbp_stereo/src/lbp_min_sum_kernel.cu:9-213 (one
// column/row step per launch, 2(W-1)+2(H-1) launches per pass, :461-491) and
// the two semantic variants (ops/lbp_semantic_pw*/src/lbp_min_sum_kernel.cu).
//
// GB300 design:
//   * One warp owns one whole scanline of one sweep and walks it; the message
//     it just produced stays in registers as the next pixel's incoming
//     message, so the dependency chain never touches memory.
//   * The RIGHT and LEFT sweeps never read each other's output (a sweep
//     leaves out the slot of its own direction, lbp_min_sum_kernel.cu:69-72),
//     and likewise DOWN and UP, so one launch runs RIGHT+LEFT for all rows
//     and a second runs DOWN+UP for all columns: 2 launches per pass instead
//     of 2(W-1)+2(H-1).
//   * The per-pixel inputs that do not depend on the chain (cost and the two
//     cross-direction messages) are prefetched into registers one step ahead
//     (coalesced loads of slots the running phase does not write).  The
//     pixel-pairwise variant, whose step also needs an L x L matrix, streams
//     them instead through a per-warp shared-memory ring NS pixels ahead with
//     TMA 1-D bulk copies (cp.async.bulk + mbarrier, bounded waits), or
//     4-byte cp.async when a row is not 16-byte sized.
//   * Labels are spread over lanes (label = lane + 32k).  min/argmin and the
//     exp-sum reproduce the reference's reduction tree (bpl_device.cuh); the
//     exp/log of the normalisation are correctly rounded float evaluations
//     equal to the reference's double-precision ones (bpl_crmath.cuh).
#pragma once
#include <cuda_runtime.h>

#include <cuda_fp16.h>

#include <algorithm>

#include "bpl_crmath.cuh"
#include "bpl_device.cuh"
#include "bpl_internal.h"

namespace bpl {

// ring depth when rows are fetched with 4-byte cp.async (compile-time for
// cp.async.wait_group)
constexpr int kRingCpAsync = 4;

// largest label count of the pixel-pairwise variant whose per-pixel L x L
// matrices are staged through the shared-memory ring (K <= 3 slots)
constexpr int kPixelRingMaxL = 96;

// largest truncation half-width served by the unrolled zero-offset window
constexpr int kFastDelta = 4;
// +inf padding on each side of the per-warp h row
constexpr int kHsPad = 4;
// A phase whose scanlines number fewer than this many per SM splits each
// scanline's labels over several warps (0: never; the split pays only when
// the per-label work dominates the per-step reductions).
constexpr int kSplitChainsPerSm = 0;
// scanlines per SM above which a phase runs the high-occupancy instantiation
constexpr int kHiOccChainsPerSm = 8;

// Storage type T of cost, messages (and the pixel-pairwise matrices): float
// (reference layout, bit-exact) or __half (FP16 storage, FP32 arithmetic).
// Rows of L labels are stored with a label stride Ls >= L (Ls = L for float;
// L rounded up to 8 for __half, so every row is 16-byte sized).
struct FwdArgs {
  const void* cost;
  const void* jump;
  const float* edge;
  void* msgs;
  void* argmin;
  float* scale;
  int B, H, W, L, Lv, jb, eb, delta;
  int Ls;     // label stride of cost / messages / argmin rows
  int Lm;     // row stride of the pixel-pairwise matrices (pixel variant)
  int argmin_kind;
  int phase;  // 0: RIGHT+LEFT over rows, 1: DOWN+UP over columns
  int nchains;
  int ns;     // ring depth (steps)
  int sps;    // steps per ring group (one mbarrier per group)
  int lrow;   // unused
  int lmat;   // elements of the per-pixel pairwise matrix in a stage (pixel variant), else 0
  int vec4;   // rows are 16-byte sized: use bulk copies
  // pixel variant: the pairwise input is the layer's (2,H,W,L,Lm) LR / UD
  // planes; direction RL reads the LR matrix of the pixel to its left,
  // transposed, DU the UD matrix of the pixel above, transposed
  // (message_passing_op_pw_pixel.py:27-38)
  int planes2;
};

// exp/log of the message normalisation with the reference's results
// ((float)exp((double)m) and (float)log(max((double)sum, 1e-45)),
// lbp_min_sum_kernel.cu:167, :180-181): correctly rounded float-float
// evaluation, double precision only when the rounding is undecided.
__device__ __forceinline__ float norm_exp(float m, const float* ehi, const float* elo) {
  float y;
  if (!crm::exp_fast(m, y, ehi, elo)) y = static_cast<float>(exp(static_cast<double>(m)));
  return y;
}
// exp of the normalisation: the exact evaluation above (float storage) or
// the hardware approximation (half storage, not bit-exact by design)
template <bool EXACT>
__device__ __forceinline__ bool exp_try(float x, float& y, const float* ehi, const float* elo) {
  if (EXACT) return crm::exp_fast(x, y, ehi, elo);
  y = __expf(x);
  return true;
}
__device__ __forceinline__ float norm_log(float sum) {
  float y;
  if (!crm::log_fast(sum, y)) y = static_cast<float>(log(fmax(static_cast<double>(sum), 1e-45)));
  return y;
}

// Shared memory of a block: CPB chains of NW warps each.
//   per chain: hs   32K floats + kHsPad of +inf on both sides (h of the pixel)
//              erow 32K floats (exp values, NW > 1 only)
//              red  16 words   (per-warp partial minima / tie counts / labels)
//   per warp:  ring ns stages x 3 rows x lroww floats (cost and the two
//              cross-direction messages of the warp's own labels [+ the
//              pixel's L x L pairwise matrix, pixel variant]), ns mbarriers,
//              taps tile 2 x (Lv+3) x 33 floats.
__host__ __device__ inline int align4(int v) { return (v + 3) & ~3; }

// elements of T per ring stage
__host__ __device__ inline int stage_elems(int lrow, int lmat) { return 3 * lrow + lmat; }

// rows of a warp's tap tile: Lv taps, the edge weight, the window class of
// the sender (two rows)
__host__ __device__ inline int tap_tile_rows(int Lv) { return Lv + 3; }

__host__ __device__ inline int chain_smem_floats(int K) { return align4(32 * K + 2 * kHsPad) + 32 * K + 16; }

__host__ __device__ inline int ring_floats(int ns, int lroww, int lmat, int tsize) {
  return align4((ns * stage_elems(lroww, lmat) * tsize + 3) / 4);
}

__host__ __device__ inline int warp_smem_floats(int ns, int lroww, int lmat, int Lv, int tsize) {
  return ring_floats(ns, lroww, lmat, tsize) + 2 * align4(ns) + align4(2 * tap_tile_rows(Lv) * 33);
}

template <typename T>
__device__ __forceinline__ float ldf(T v);
template <>
__device__ __forceinline__ float ldf<float>(float v) { return v; }
template <>
__device__ __forceinline__ float ldf<__half>(__half v) { return __half2float(v); }
template <typename T>
__device__ __forceinline__ T stf(float v);
template <>
__device__ __forceinline__ float stf<float>(float v) { return v; }
template <>
__device__ __forceinline__ __half stf<__half>(float v) { return __float2half_rn(v); }

struct WarpSmem {
  float* ring;
  uint64_t* bars;
  float* taps;
};

struct ChainSmem {
  float* hs;
  float* erow;
  float* red;
};

// One scanline of one sweep.  Pixels are addressed by their index within the
// image (pin = y*W + x); the sender of step i is pin0 + i*dpin and its
// receiver is one dpin further.
template <typename T>
struct Chain {
  int n, dir;
  int pin0, dpin;
  const T* cost;       // batch item n
  const T* slot_a;     // cross-direction message slots read at the sender
  const T* slot_b;
  T* slot_out;         // slot written at the receiver (= the incoming chain slot)
  int64_t out_off;     // element offset of slot_out within the messages tensor
  const T* pjump;      // per-pixel pairwise matrices of this direction (pixel variant)
  int pshift;          // pixel offset of a sender's matrix (-1 or -W for the layer's planes)
  int ps, pt;          // strides of sender / receiver label in a staged matrix
  int t0, cnt;         // first label of this warp; labels it copies per row
};

// a zero L x L pairwise matrix (L <= 96, float or half), read by the first
// sender of the RL / DU directions with the layer's pairwise planes
extern __device__ __align__(16) float g_zero_pairwise[96 * 96];

// Issues ring slot `st` for step i: the warp's labels [t0, t0+cnt) of the
// sender's cost and cross-direction messages (+ the pixel's pairwise matrix,
// pixel variant).  Bulk copies complete on `bar`; the caller arms it.
template <int VARIANT, typename T>
__device__ __forceinline__ void issue_slot(const FwdArgs& a, const Chain<T>& c, const WarpSmem& sm, int lroww,
                                           int i, int st, uint64_t* bar, int lane) {
  T* dst = reinterpret_cast<T*>(sm.ring) + st * stage_elems(lroww, a.lmat);
  const int64_t pin = c.pin0 + i * c.dpin;
  const int64_t po = pin * a.Ls + c.t0;
  const T* src0 = c.cost + po;
  const T* src1 = c.slot_a + po;
  const T* src2 = c.slot_b + po;
  // the first sender of a shifted direction reads the zero matrix (the
  // layer's shifted tensor is zero there)
  const T* src3 = (VARIANT == BPL_LBP_SEM_PIXEL)
                      ? ((c.pshift != 0 && i == 0) ? reinterpret_cast<const T*>(g_zero_pairwise)
                                                   : c.pjump + (pin + c.pshift) * a.L * a.Lm)
                      : nullptr;
  if (a.vec4) {
    if (lane == 0) {
      const uint32_t rb = static_cast<uint32_t>(c.cnt) * static_cast<uint32_t>(sizeof(T));
      if (rb > 0) {
        bulk_g2s(dst, src0, rb, bar);
        bulk_g2s(dst + lroww, src1, rb, bar);
        bulk_g2s(dst + 2 * lroww, src2, rb, bar);
      }
      if (VARIANT == BPL_LBP_SEM_PIXEL)
        bulk_g2s(dst + 3 * lroww, src3, static_cast<uint32_t>(a.L * a.Lm) * static_cast<uint32_t>(sizeof(T)), bar);
    }
  } else if constexpr (sizeof(T) == 4) {
    // rows not 16-byte sized (float storage only; half rows are padded)
    for (int t = lane; t < c.cnt; t += 32) {
      cp_async4(dst + t, src0 + t);
      cp_async4(dst + lroww + t, src1 + t);
      cp_async4(dst + 2 * lroww + t, src2 + t);
    }
    if (VARIANT == BPL_LBP_SEM_PIXEL)
      for (int t = lane; t < a.L * a.Lm; t += 32) cp_async4(dst + 3 * lroww + t, src3 + t);
  }
}

// Issues ring group g (slots [g*sps, (g+1)*sps)) for steps [i0, i0 + sps)
// below nsteps: one mbarrier armed with the bytes of all of them.  With
// cp.async rows (sps = 1) the caller commits one group per step.
template <int VARIANT, typename T>
__device__ __forceinline__ bool issue_group(const FwdArgs& a, const Chain<T>& c, const WarpSmem& sm, int lroww,
                                            int i0, int g, int nsteps, int lane) {
  const int n = min(a.sps, nsteps - i0);
  if (n <= 0) return false;  // nothing to stage: the group stays unarmed
  uint64_t* bar = &sm.bars[g];
  if (a.vec4 && lane == 0) {
    const uint32_t rb = static_cast<uint32_t>(c.cnt) * static_cast<uint32_t>(sizeof(T));
    const uint32_t mb =
        (VARIANT == BPL_LBP_SEM_PIXEL) ? static_cast<uint32_t>(a.L * a.Lm) * static_cast<uint32_t>(sizeof(T)) : 0u;
    // the slots were last read through the generic proxy
    fence_proxy_async();
    mbar_arrive_expect_tx(bar, static_cast<uint32_t>(n) * (3u * rb + mb));
  }
  for (int k = 0; k < n; ++k) issue_slot<VARIANT, T>(a, c, sm, lroww, i0 + k, g * a.sps + k, bar, lane);
  return true;
}

// Stereo taps + edge weight for the 32 pixels of block b: lane j loads the
// sender of step 32b + j.  Held in registers until written to the tile.
struct TapRegs {
  float t[16];
  float w;
};

template <typename T>
__device__ __forceinline__ void load_taps(const FwdArgs& a, const Chain<T>& c, int b, int lane, int nsteps,
                                          TapRegs& r, bool stereo) {
  const int i = 32 * b + lane;
  if (i >= nsteps) return;
  const int64_t HW = static_cast<int64_t>(a.H) * a.W;
  const int pin = c.pin0 + i * c.dpin;
  const int ne = (a.eb == 1) ? 0 : c.n;
  r.w = __ldg(a.edge + (static_cast<int64_t>(ne) * 4 + c.dir) * HW + pin);
  if (stereo) {
    const int nj = (a.jb == 1) ? 0 : c.n;
    const float* base = static_cast<const float*>(a.jump) + ((static_cast<int64_t>(nj) * 4 + c.dir) * a.Lv) * HW + pin;
#pragma unroll
    for (int k = 0; k < 16; ++k)
      if (k < a.Lv) r.t[k] = __ldg(base + static_cast<int64_t>(k) * HW);
  }
}

// Window classes of a sender's zero-offset truncation window (stereo, delta
// <= kFastDelta).  A window term fmaf(f, w, h(s)) whose tap has f*w >= L2*w
// is >= the global candidate fmaf(L2, w, min h) (h(s) >= min h, rounding is
// monotone): it can tie the candidate but never beat it ("tie-only"
// offset).  When the offsets that can beat it are exactly |jd| <= R, the
// message needs only those 2R+1 terms plus an exact check of the tie-only
// offsets against the few senders that can reach the candidate there.
//   code 0: no fast form (offset, delta or tap pattern)
//   code 1..4: R = code - 2 (R = -1: no offset beats the candidate)
//   bit 8: the window holds tie-only offsets; the tile row Lv+1 then holds
//          the tie-only tap of smallest product with w
//   bit 9: every tie-only tap is bitwise L2
constexpr int kWinGeneric = 0;
constexpr int kWinHasTieOnly = 0x100;
constexpr int kWinTieIsL2 = 0x200;  // every tie-only tap equals L2 bitwise

__device__ __forceinline__ void store_taps(const FwdArgs& a, float* tile, int lane, const TapRegs& r,
                                           bool stereo) {
  // tile layout: [Lv+3][33]; rows 0..Lv-1 taps, row Lv the edge weight,
  // row Lv+1 the smallest-product tie-only tap, row Lv+2 the window code
  tile[a.Lv * 33 + lane] = r.w;
  if (stereo) {
#pragma unroll
    for (int k = 0; k < 16; ++k)
      if (k < a.Lv) tile[k * 33 + lane] = r.t[k];
    // each lane classifies its own column (no other lane's values are read)
    const float w = r.w;
    const float L2 = tile[(a.Lv - 1) * 33 + lane];
    int code = kWinGeneric;
    float fnr = 0.0f;
    if (tile[lane] == 0.0f && a.delta <= kFastDelta) {
      int R = -1;
      bool ok = true, seen_tie = false, have_tie = false, tie_l2 = true;
      for (int q = 0; q <= a.delta; ++q) {
        const float fp = tile[max(1, min(a.Lv - 1, a.Lv / 2 - q)) * 33 + lane];  // jd = +q
        const float fm = tile[max(1, min(a.Lv - 1, a.Lv / 2 + q)) * 33 + lane];  // jd = -q
        const bool tp = (w > 0.0f) ? (fp >= L2) : ((w < 0.0f) ? (fp <= L2) : true);
        const bool tm = (w > 0.0f) ? (fm >= L2) : ((w < 0.0f) ? (fm <= L2) : true);
        if (!tp && !tm) {
          if (seen_tie) ok = false;
          R = q;
        } else if (tp && tm) {
          seen_tie = true;
          tie_l2 = tie_l2 && __float_as_int(fp) == __float_as_int(L2) && __float_as_int(fm) == __float_as_int(L2);
          // tie-only tap of smallest product f*w
          const float f = (w >= 0.0f) ? fminf(fp, fm) : fmaxf(fp, fm);
          fnr = !have_tie ? f : ((w >= 0.0f) ? fminf(fnr, f) : fmaxf(fnr, f));
          have_tie = true;
        } else {
          ok = false;
        }
      }
      if (ok && R <= 2) code = (R + 2) | (have_tie ? kWinHasTieOnly : 0) | ((have_tie && tie_l2) ? kWinTieIsL2 : 0);
    }
    tile[(a.Lv + 1) * 33 + lane] = fnr;
    tile[(a.Lv + 2) * 33 + lane] = __int_as_float(code);
  }
}

// Barrier over the NW warps of one chain (named barrier `id`), returning the
// AND of `v` over them.
template <int NW>
__device__ __forceinline__ bool chain_sync_and(int id, bool v) {
  if (NW == 1) return __all_sync(FULL, v);
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 q, %1, 0;\n barrier.red.and.pred p, %2, %3, q;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(r)
      : "r"(static_cast<uint32_t>(v)), "r"(id), "r"(NW * 32)
      : "memory");
  return r != 0;
}

template <int NW>
__device__ __forceinline__ void chain_sync(int id) {
  if (NW == 1) {
    __syncwarp();
    return;
  }
  asm volatile("barrier.sync.aligned %0, %1;" ::"r"(id), "r"(NW * 32) : "memory");
}

// K labels per lane over the chain (label = lane + 32k), KW = K/NW of them
// owned by each of the chain's NW warps (slots [w*KW, (w+1)*KW)).
// OCC: blocks per SM the register allocation must allow.  1: 4-warp blocks
// with every register the compiler wants (the latency-bound phase with few
// scanlines); kHiOcc: 1-warp blocks, kHiOcc of them per SM (the phase whose
// scanlines outnumber what a wave of 4-warp blocks holds).
constexpr int kHiOcc = 17;
template <int OCC>
constexpr int fwd_block_warps() { return (OCC > 1) ? 1 : 4; }

template <int K, int VARIANT, int NW, typename T, int OCC>
__global__ void __launch_bounds__(32 * fwd_block_warps<OCC>(), OCC) lbp_forward_kernel(FwdArgs a) {
  constexpr bool kExact = sizeof(T) == 4;  // float storage: the reference's exact arithmetic
  static_assert(K % NW == 0, "labels must split evenly over the chain's warps");
  static_assert(NW == 1 || VARIANT != BPL_LBP_SEM_PIXEL, "pixel variant runs one warp per chain");
  constexpr int KW = K / NW;
  extern __shared__ __align__(16) float smem[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int cpb = (blockDim.x >> 5) / NW;  // chains per block
  const int cic = wib / NW;                // chain within block
  const int wic = wib % NW;                // warp within chain
  const int chain_id = blockIdx.x * cpb + cic;
  if (chain_id >= a.nchains) return;  // the chain's warps leave together; no block-wide barriers below
  const int bar_id = 1 + cic;

  const int L = a.L;
  const int lroww = 32 * KW;
  ChainSmem cs;
  {
    float* p = smem + cic * chain_smem_floats(K);
    cs.hs = p + kHsPad;
    cs.erow = p + align4(32 * K + 2 * kHsPad);
    cs.red = cs.erow + 32 * K;
  }
  WarpSmem sm;
  {
    float* p = smem + cpb * chain_smem_floats(K) + wib * warp_smem_floats(a.ns, lroww, a.lmat, a.Lv, sizeof(T));
    sm.ring = p;
    p += ring_floats(a.ns, lroww, a.lmat, sizeof(T));
    sm.bars = reinterpret_cast<uint64_t*>(p);
    p += 2 * align4(a.ns);
    sm.taps = p;
  }
  // exp table for lane-varying lookups: every warp writes the same values
  __shared__ float s_ehi[64], s_elo[64];
  s_ehi[lane] = crm::kTab.exp_hi[lane];
  s_ehi[lane + 32] = crm::kTab.exp_hi[lane + 32];
  s_elo[lane] = crm::kTab.exp_lo[lane];
  s_elo[lane + 32] = crm::kTab.exp_lo[lane + 32];
  if (wic == 0 && lane < kHsPad) {
    cs.hs[-1 - lane] = __int_as_float(0x7f800000);
    cs.hs[32 * K + lane] = __int_as_float(0x7f800000);
  }
  __syncwarp();

  const int64_t HW = static_cast<int64_t>(a.H) * a.W;
  const int64_t HWL = HW * a.Ls;  // elements per message slot / cost image
  const int Ls = a.Ls;
  Chain<T> c;
  int len;
  {
    const int r = chain_id >> 1;
    if (a.phase == 0) {
      c.dir = (chain_id & 1) ? LEFT : RIGHT;
      c.n = r / a.H;
      const int y = r % a.H;
      len = a.W;
      c.pin0 = y * a.W + ((c.dir == RIGHT) ? 0 : a.W - 1);
      c.dpin = (c.dir == RIGHT) ? 1 : -1;
    } else {
      c.dir = (chain_id & 1) ? UP : DOWN;
      c.n = r / a.W;
      const int x = r % a.W;
      len = a.H;
      c.pin0 = ((c.dir == DOWN) ? 0 : a.H - 1) * a.W + x;
      c.dpin = (c.dir == DOWN) ? a.W : -a.W;
    }
  }
  const int nsteps = len - 1;
  if (nsteps <= 0) return;
  const int od = c.dir ^ 1;
  const int sa = (a.phase == 0) ? UP : RIGHT;
  const int sb = (a.phase == 0) ? DOWN : LEFT;
  c.cost = static_cast<const T*>(a.cost) + static_cast<int64_t>(c.n) * HWL;
  c.slot_a = static_cast<const T*>(a.msgs) + (static_cast<int64_t>(c.n) * 4 + sa) * HWL;
  c.slot_b = static_cast<const T*>(a.msgs) + (static_cast<int64_t>(c.n) * 4 + sb) * HWL;
  c.out_off = (static_cast<int64_t>(c.n) * 4 + od) * HWL;
  c.slot_out = static_cast<T*>(a.msgs) + c.out_off;
  c.pjump = (VARIANT == BPL_LBP_SEM_PIXEL)
                ? static_cast<const T*>(a.jump) + static_cast<int64_t>(a.planes2 ? (c.dir >> 1) : c.dir) * HW * L * a.Lm
                : nullptr;
  {
    const bool tr = (VARIANT == BPL_LBP_SEM_PIXEL) && a.planes2 && (c.dir & 1);
    c.pshift = tr ? ((c.dir == LEFT || c.dir == RIGHT) ? -1 : -a.W) : 0;
    c.ps = tr ? 1 : a.Lm;
    c.pt = tr ? a.Lm : 1;
  }
  c.t0 = 32 * KW * wic;
  // label validity: with K = ceil(L/32) (the stereo K <= 8 instantiations
  // are dispatched exactly) only the last slot of a one-warp scanline can
  // hold labels >= L; the test folds away for the other slots.  The semantic
  // variants share instantiations between label counts (K = 8 serves 129..256)
  // and test every slot.
  auto lvalid = [&](int kk) -> bool {
    return (VARIANT == BPL_LBP_STEREO && K <= 8 && NW == 1 && kk < KW - 1) || (c.t0 + lane + 32 * kk < L);
  };
  // labels copied per row: the warp's labels below Ls (padding included, so
  // half rows stay 16-byte sized)
  c.cnt = max(0, min(lroww, Ls - c.t0));
  float* scale_out = a.scale ? a.scale + (static_cast<int64_t>(c.n) * 4 + od) * HW : nullptr;  // NULL: FP16, not asked for
  const float* gjump =
      (VARIANT == BPL_LBP_SEM_GLOBAL) ? static_cast<const float*>(a.jump) + static_cast<int64_t>(c.dir) * L * L : nullptr;
  const bool stereo = (VARIANT == BPL_LBP_STEREO);
  // Global pairwise with one label per lane (L <= 32): the lane's column of
  // the direction's matrix, P[s][t] for its label t, held in registers for
  // the whole scanline, so the full minimisation is L register FMAs against
  // broadcast reads of h instead of L global (L1) loads per step.
  constexpr bool kPcolRegs = (VARIANT == BPL_LBP_SEM_GLOBAL) && K == 1 && NW == 1;
  float pcol[kPcolRegs ? 32 : 1];
  if constexpr (kPcolRegs) {
#pragma unroll
    for (int s = 0; s < 32; ++s) pcol[s] = (s < L && lane < L) ? __ldg(gjump + s * L + lane) : 0.0f;
  }

  // Pixel variant: a shared-memory ring of the steps' rows and L x L
  // matrices (groups of sps steps, one mbarrier each).  Other variants: the
  // next step's own rows are prefetched into registers (coalesced loads of
  // data no sweep of this phase writes), one step ahead.
  // (pixel variant above 96 labels: a sender's L x L matrix no longer fits
  // a ring stage, so its entries are read from global memory as used)
  constexpr bool kRing = (VARIANT == BPL_LBP_SEM_PIXEL) && K <= 3;
  constexpr bool kPixGlobal = (VARIANT == BPL_LBP_SEM_PIXEL) && !kRing;
  const int G = kRing ? a.sps : 1;
  T ncst[KW], nva[KW], nvb[KW];  // raw: converted when used, so the loads do not stall here
  auto prefetch = [&](int i) {
    const int64_t po = static_cast<int64_t>(c.pin0 + i * c.dpin) * Ls;
#pragma unroll
    for (int kk = 0; kk < KW; ++kk) {
      const int t = c.t0 + lane + 32 * kk;
      const int64_t o = po + (lvalid(kk) ? t : 0);  // labels >= L read label 0 (ignored)
      ncst[kk] = __ldg(c.cost + o);
      nva[kk] = __ldg(c.slot_a + o);
      nvb[kk] = __ldg(c.slot_b + o);
    }
  };
  if (!kRing) prefetch(0);
  if (kRing && a.vec4 && lane == 0) {
    for (int g = 0; g < a.ns / G; ++g) mbar_init(&sm.bars[g], 1);
    fence_mbar_init();
  }
  __syncwarp();
  // ring groups with copies in flight (bit g), for the drain of a failed wait
  uint32_t armed = 0u;
  if (kRing) {
    for (int i0 = 0; i0 < a.ns; i0 += G) {
      if (issue_group<VARIANT, T>(a, c, sm, lroww, i0, i0 / G, nsteps, lane)) armed |= 1u << (i0 / G);
      if (!a.vec4) cp_async_commit();
    }
  }

  // incoming chain message at the first sender: the slot the sweep writes
  float chain[KW];
  {
    const T* src = c.slot_out + static_cast<int64_t>(c.pin0) * Ls;
#pragma unroll
    for (int kk = 0; kk < KW; ++kk) {
      const int t = c.t0 + lane + 32 * kk;
      chain[kk] = lvalid(kk) ? ldf<T>(src[t]) : 0.0f;
    }
  }

  TapRegs tr;
  load_taps(a, c, 0, lane, nsteps, tr, stereo);
  store_taps(a, sm.taps, lane, tr, stereo);
  if (nsteps > 32) load_taps(a, c, 1, lane, nsteps, tr, stereo);
  __syncwarp();

  const int delta = a.delta;
  const int tile_stride = tap_tile_rows(a.Lv) * 33;
  const int sf = stage_elems(lroww, a.lmat);
  const float kInf = __int_as_float(0x7f800000);
  bool failed = false;
  int st = 0;
  uint32_t par = 0;
  int pin = c.pin0;
  for (int i = 0; i < nsteps; ++i, pin += c.dpin) {
    const int j = i & 31;
    const int b = i >> 5;
    const float* tile = sm.taps + (b & 1) * tile_stride;
    const T* stg = reinterpret_cast<const T*>(sm.ring) + st * sf;
    // the sender's pairwise entry f(t, s): staged (ring) or read from global
    // memory (wide pixel rows; the first sender of a shifted direction reads
    // the layer's zero matrix)
    const T* pmat = nullptr;
    if constexpr (kPixGlobal)
      pmat = (c.pshift != 0 && i == 0) ? nullptr : c.pjump + static_cast<int64_t>(pin + c.pshift) * L * a.Lm;
    auto pairf = [&](int s_, int t_) -> float {
      if constexpr (kRing) return ldf<T>(stg[3 * lroww + s_ * c.ps + t_ * c.pt]);
      else if constexpr (kPixGlobal) return pmat ? ldf<T>(pmat[s_ * c.ps + t_ * c.pt]) : 0.0f;
      else return 0.0f;
    };

    // wait for the ring group of step i (own labels) at its first step
    const int grp = st / G;
    bool ok = true;
    if (kRing && st == grp * G) {
      if (a.vec4) {
        ok = mbar_wait_bounded(&sm.bars[grp], (par >> grp) & 1u);
        // a group whose wait ran out keeps its pending phase in `par` (and
        // its bit in `armed`) for the drain below
        if (ok) {
          par ^= 1u << grp;
          armed &= ~(1u << grp);
        }
      } else {
        // groups 0..i have landed (one group per step, a.ns in flight)
        if (a.ns == 4) cp_async_wait<3>();
        else if (a.ns == 3) cp_async_wait<2>();
        else cp_async_wait<1>();
      }
      __syncwarp();
    }

    // h = cost + incoming messages except the chain direction's own slot,
    // added in the reference order RIGHT, LEFT, UP, DOWN.
    float h[KW];
#pragma unroll
    for (int kk = 0; kk < KW; ++kk) {
      // branch-free: the ring rows are lroww long; labels >= L read padding
      // and get +inf (never a minimum)
      const int tl = lane + 32 * kk;  // label within the warp's range
      const float cst = ldf<T>(kRing ? stg[tl] : ncst[kk]);
      const float va = ldf<T>(kRing ? stg[lroww + tl] : nva[kk]);
      const float vb = ldf<T>(kRing ? stg[2 * lroww + tl] : nvb[kk]);
      const float hv = (a.phase == 0) ? __fadd_rn(__fadd_rn(__fadd_rn(cst, chain[kk]), va), vb)
                                      : __fadd_rn(__fadd_rn(__fadd_rn(cst, va), vb), chain[kk]);
      h[kk] = lvalid(kk) ? hv : kInf;
      cs.hs[c.t0 + tl] = h[kk];
    }
    // partial minimum over the warp's labels (one redux), with its tie count
    // and, when the minimum is unique, its label
    float pm = h[0];
#pragma unroll
    for (int kk = 1; kk < KW; ++kk) pm = fminf(pm, h[kk]);
    pm = warp_min_redux(pm);
    int lcnt = 0, llab = 0;
#pragma unroll
    for (int kk = 0; kk < KW; ++kk) {
      const bool eq = h[kk] == pm;
      lcnt += eq ? 1 : 0;
      llab = eq ? c.t0 + lane + 32 * kk : llab;
    }
    const int pcnt = __reduce_add_sync(FULL, lcnt);
    const int plab = __reduce_max_sync(FULL, llab);
    if (NW > 1 && lane == 0) {
      cs.red[wic] = pm;
      reinterpret_cast<int*>(cs.red)[4 + wic] = pcnt;
      reinterpret_cast<int*>(cs.red)[8 + wic] = plab;
    }
    __syncwarp();
    if (!kRing && i + 1 < nsteps) prefetch(i + 1);
    // h of the whole pixel and the partial minima are visible to the chain
    if (NW == 1) {
      if (!__all_sync(FULL, ok)) {
        failed = true;
        break;
      }
    } else if (!chain_sync_and<NW>(bar_id, ok)) {
      failed = true;
      break;
    }

    const float w = tile[a.Lv * 33 + j];
    float msg[KW];
    int am[KW];
    float e[KW];
    // Half storage keeps every message relative to the minimum of h (the
    // labels near the row's minimum, the ones the beliefs depend on, get
    // half's finest steps; a log-normalised row sits near -log L, where a
    // half step is 2^-8).  The row's scale is then the sum of exp of the
    // stored row, and the log-normalised message is stored - log(scale).
    float ref = 0.0f;
    if (!kExact) {
      ref = pm;
      if (NW > 1) {
        ref = cs.red[0];
#pragma unroll
        for (int w2 = 1; w2 < NW; ++w2) ref = fminf(ref, cs.red[w2]);
      }
    }
    auto earg = [ref](float x) { return kExact ? x : __fsub_rn(x, ref); };

    if (kPcolRegs && delta >= L) {
      // full minimisation with the register column (see kPcolRegs); same
      // order and tie rule as below.  The 32 senders run as four
      // independent chains over the contiguous ranges [8c, 8c+8), combined
      // in sender order: the minimum's value (a left fold of fminf over the
      // senders in order, whatever fminf returns for equal operands) and
      // the last sender that attains it are those of the single chain.
      // Senders s >= L have h = +inf and a zero column entry: their terms
      // are +inf (NaN for an infinite w) and neither lower a minimum nor
      // equal it, so they need no test.
      float mc[4] = {1e15f, kInf, kInf, kInf};
      int ac[4] = {0, 0, 0, 0};
#pragma unroll
      for (int q = 0; q < 8; ++q) {
#pragma unroll
        for (int ch = 0; ch < 4; ++ch) {
          const int s = 8 * ch + q;
          const float nm = __fmaf_rn(pcol[s], w, cs.hs[s]);
          mc[ch] = fminf(mc[ch], nm);
          if (mc[ch] == nm) ac[ch] = s;
        }
      }
      float m = mc[0];
      int arg = ac[0];
#pragma unroll
      for (int ch = 1; ch < 4; ++ch) {
        m = fminf(m, mc[ch]);
        // chain ch holds a sender at the minimum (it started at +inf, the
        // minimum is at most 1e15): its last such sender is the latest
        arg = (mc[ch] == m) ? ac[ch] : arg;
      }
      msg[0] = (lane < L) ? m : 1e15f;
      am[0] = (lane < L) ? arg : 0;
      bool eok0 = exp_try<kExact>(earg(msg[0]), e[0], s_ehi, s_elo);
      if (lane >= L) {
        e[0] = 0.0f;
        eok0 = true;
      }
      if (!__all_sync(FULL, eok0) && !eok0) e[0] = static_cast<float>(exp(static_cast<double>(msg[0])));
    } else if (delta >= L) {
      // full minimisation (lbp_min_sum_kernel.cu:88-111): last minimiser wins
#pragma unroll
      for (int kk = 0; kk < KW; ++kk) {
        const int t = c.t0 + lane + 32 * kk;
        float m = 1e15f;
        int arg = 0;
        if (t < L) {
          for (int s = 0; s < L; ++s) {
            float f;
            if (stereo) {
              const int ti = max(1, min(a.Lv - 1, a.Lv / 2 + (t - s)));
              f = tile[ti * 33 + j];
            } else if (VARIANT == BPL_LBP_SEM_GLOBAL) {
              f = __ldg(gjump + s * L + t);
            } else {
              f = pairf(s, t);
            }
            const float nm = __fmaf_rn(f, w, cs.hs[s]);
            m = fminf(m, nm);
            if (m == nm) arg = s;
          }
        }
        msg[kk] = m;
        am[kk] = arg;
      }
      bool all_ok = true;
      bool eok[KW];
#pragma unroll
      for (int kk = 0; kk < KW; ++kk) {
        eok[kk] = exp_try<kExact>(earg(msg[kk]), e[kk], s_ehi, s_elo);
        if (c.t0 + lane + 32 * kk >= L) {
          e[kk] = 0.0f;
          eok[kk] = true;
        }
        all_ok = all_ok && eok[kk];
      }
      if (!__all_sync(FULL, all_ok)) {
#pragma unroll
        for (int kk = 0; kk < KW; ++kk)
          if (!eok[kk]) e[kk] = static_cast<float>(exp(static_cast<double>(msg[kk])));
      }
    } else {
      // Truncated branch (lbp_min_sum_kernel.cu:112-164).  The reference
      // starts from the global candidate fmaf(L2, w, min h) and scans the
      // window in increasing label order with `<=`; that equals taking the
      // window's own minimum (last label on ties) when it is <= the global
      // candidate.  A sender s can only reach the candidate if
      // fmaf(f*, w, h(s)) <= fmaf(L2, w, min h), f* the tap of smallest
      // product (rounding is monotone), so with a zero offset only the slots
      // whose windows hold such a sender are scanned; every other label takes
      // the candidate, its argmin and its exp.
      float L2, off = 0.0f;
      if (stereo) {
        L2 = tile[(a.Lv - 1) * 33 + j];
        off = tile[0 * 33 + j];
      } else if (VARIANT == BPL_LBP_SEM_GLOBAL) {
        L2 = __ldg(gjump + (L - 1));
      } else {
        L2 = pairf(0, L - 1);
      }
      // The global candidate needs only the minimum value of h, which any
      // reduction order gives exactly.
      float min_h = pm;
      int argmin_h = plab, tot = pcnt;
      if (NW > 1) {
        min_h = cs.red[0];
#pragma unroll
        for (int w2 = 1; w2 < NW; ++w2) min_h = fminf(min_h, cs.red[w2]);
        tot = 0;
#pragma unroll
        for (int w2 = 0; w2 < NW; ++w2)
          if (cs.red[w2] == min_h) {
            tot += reinterpret_cast<const int*>(cs.red)[4 + w2];
            argmin_h = reinterpret_cast<const int*>(cs.red)[8 + w2];
          }
      }
      // exact ties of the minimum: the reference tree picks the label (and,
      // between -0 and +0, the value)
      if (tot > 1) {
        float tv[K];
        int tl[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
          tv[k] = cs.hs[lane + 32 * k];
          tl[k] = lane + 32 * k;
        }
        float mv;
        tree_argmin<K>(tv, tl, L, lane, mv, argmin_h);
        min_h = cs.hs[argmin_h];
      }
      const float msg_g = __fmaf_rn(L2, w, min_h);

      // Fast form (one warp per scanline, stereo zero-offset windows whose
      // beating offsets are |jd| <= R): the 2R+1 terms for every label, and
      // the tie-only offsets checked against the one sender s1 that can reach
      // the candidate there (fmaf(f_tie, w, h(s1)) <= candidate for the
      // smallest-product tie-only tap); with several such senders, or no
      // fast form, every window term is scanned.
      int R = -2;
      int s1 = -1;
      int wcode = kWinGeneric;
      // The tie-only count's two reductions are issued here and first read
      // after the window terms below, which run in their shadow: the count
      // only sends the step to the full scan (several senders) or names the
      // one sender s1 for the fix.
      int nn = 0, smax = -1;
      if (NW == 1 && stereo) {
        wcode = __float_as_int(tile[(a.Lv + 2) * 33 + j]);
        if ((wcode & 0xff) != kWinGeneric) {
          R = (wcode & 0xff) - 2;
          if (wcode & kWinHasTieOnly) {
            const float fnr = tile[(a.Lv + 1) * 33 + j];
            int lc = 0, ll = -1;
#pragma unroll
            for (int kk = 0; kk < KW; ++kk) {
              const bool nr = __fmaf_rn(fnr, w, h[kk]) <= msg_g;  // +inf (no label) never is
              lc += nr ? 1 : 0;
              ll = nr ? c.t0 + lane + 32 * kk : ll;
            }
            nn = __reduce_add_sync(FULL, lc);
            smax = __reduce_max_sync(FULL, ll);
          }
        }
      }
      bool own[KW];
      float mw[KW];
      int aw[KW];
      const int c0 = a.Lv / 2;
      if (R >= -1) {
        // the 2R+1 beating terms of every label, straight-line per path
        // (uniform branches outside the label loops keep the slots
        // independent); hs holds +inf outside [0, L)
        if (R == 1) {
          const float fm1 = tile[min(a.Lv - 1, c0 + 1) * 33 + j];  // sender t-1
          const float f00 = tile[c0 * 33 + j];                     // sender t
          const float fp1 = tile[max(1, c0 - 1) * 33 + j];         // sender t+1
#pragma unroll
          for (int kk = 0; kk < KW; ++kk) {
            const int t = c.t0 + lane + 32 * kk;
            // increasing sender order, `<=`: the last minimiser wins
            float m = __fmaf_rn(fm1, w, cs.hs[t - 1]);
            int arg = t - 1;
            const float n0 = __fmaf_rn(f00, w, h[kk]);
            const float n1 = __fmaf_rn(fp1, w, cs.hs[t + 1]);
            const bool k0 = n0 <= m;
            m = k0 ? n0 : m;
            arg = k0 ? t : arg;
            const bool k1 = n1 <= m;
            mw[kk] = k1 ? n1 : m;
            aw[kk] = k1 ? t + 1 : arg;
          }
        } else if (R >= 0) {
          float fR[5];  // taps of senders t-2 .. t+2
#pragma unroll
          for (int q = 0; q < 5; ++q) fR[q] = tile[max(1, min(a.Lv - 1, c0 - (q - 2))) * 33 + j];
#pragma unroll
          for (int kk = 0; kk < KW; ++kk) {
            const int t = c.t0 + lane + 32 * kk;
            float m = kInf;
            int arg = 0;
#pragma unroll
            for (int q = 0; q < 5; ++q) {
              const int jd = q - 2;
              const float nm = __fmaf_rn(fR[q], w, cs.hs[t + jd]);
              const bool take = (jd >= -R) && (jd <= R) && (nm <= m);
              m = take ? nm : m;
              arg = take ? t + jd : arg;
            }
            mw[kk] = m;
            aw[kk] = arg;
          }
        } else {
#pragma unroll
          for (int kk = 0; kk < KW; ++kk) {
            mw[kk] = kInf;
            aw[kk] = 0;
          }
        }
      }
      if (nn > 1) R = -2;
      else if (nn == 1) s1 = smax;
      if (R >= -1) {
#pragma unroll
        for (int kk = 0; kk < KW; ++kk) {
          const bool valid = lvalid(kk);
          const bool win = valid && mw[kk] <= msg_g;
          msg[kk] = win ? mw[kk] : msg_g;
          am[kk] = win ? aw[kk] : argmin_h;
          own[kk] = win && mw[kk] < msg_g;
        }
        bool fix = s1 >= 0;
        if (fix && (wcode & kWinTieIsL2) && s1 == argmin_h) {
          // s1 is the minimum of h and the tie-only taps are L2: every
          // tie-only term of s1 equals the candidate, which only changes the
          // argmin of a label whose beating terms reach exactly the candidate
          bool eq = false;
#pragma unroll
          for (int kk = 0; kk < KW; ++kk) eq = eq || (mw[kk] == msg_g);
          fix = __any_sync(FULL, eq);
        }
        if (fix) {
          // a tie with the candidate at a tie-only offset of s1: the last
          // sender at the candidate value takes the argmin
          const float hs1 = cs.hs[s1];
#pragma unroll
          for (int kk = 0; kk < KW; ++kk) {
            const int t = c.t0 + lane + 32 * kk;
            const int jd = s1 - t;
            const int ajd = jd < 0 ? -jd : jd;
            const float f = tile[max(1, min(a.Lv - 1, c0 - jd)) * 33 + j];
            const bool tie = lvalid(kk) && ajd > R && ajd <= delta && __fmaf_rn(f, w, hs1) == msg_g && !(mw[kk] < msg_g);
            am[kk] = tie ? ((mw[kk] == msg_g) ? max(aw[kk], s1) : s1) : am[kk];
          }
        }
      } else {
        const bool fast = stereo && delta <= kFastDelta && off == 0.0f;
        // taps of the zero-offset window: the tap of sender s = t + jd is
        // clamp(Lv/2 - jd, 1, Lv-1), the same for every label
        float fj[2 * kFastDelta + 1];
        if (fast) {
#pragma unroll
          for (int q = 0; q <= 2 * kFastDelta; ++q) {
            const int ti = max(1, min(a.Lv - 1, a.Lv / 2 - (q - kFastDelta)));
            fj[q] = tile[ti * 33 + j];
          }
        }
#pragma unroll
        for (int kk = 0; kk < KW; ++kk) {
          const int t = c.t0 + lane + 32 * kk;
          const bool valid = t < L;
          float m = kInf;
          int arg = 0;
          if (fast && delta == 3) {
            // hs holds +inf outside [0, L), which never wins against the
            // finite global candidate, in place of the clipping
#pragma unroll
            for (int q = kFastDelta - 3; q <= kFastDelta + 3; ++q) {
              const float nm = __fmaf_rn(fj[q], w, cs.hs[t + q - kFastDelta]);
              const bool take = nm <= m;
              m = take ? nm : m;
              arg = take ? t + q - kFastDelta : arg;
            }
          } else if (fast) {
#pragma unroll
            for (int q = 0; q <= 2 * kFastDelta; ++q) {
              const int jd = q - kFastDelta;
              const float nm = __fmaf_rn(fj[q], w, cs.hs[t + jd]);
              const bool take = (jd >= -delta) && (jd <= delta) && (nm <= m);  // branch-free
              m = take ? nm : m;
              arg = take ? t + jd : arg;
            }
          } else if (valid) {
            int start, stop;
            if (stereo) {
              start = sat_u16(roundf(__fsub_rn(__fadd_rn(static_cast<float>(t - (delta - 1)), off), 1.0f)));
              stop = min(sat_u16(roundf(__fadd_rn(__fadd_rn(static_cast<float>(t + delta), off), 1.0f))), L);
            } else {
              start = max(t - delta + 1, 0);
              stop = min(t + delta - 1, L - 1) + 1;
            }
            for (int s = start; s < stop; ++s) {
              float f;
              if (stereo) {
                const int ti = max(1, min(a.Lv - 1, a.Lv / 2 + (t - s)));
                f = tile[ti * 33 + j];
              } else if (VARIANT == BPL_LBP_SEM_GLOBAL) {
                f = __ldg(gjump + s * L + t);
              } else {
                f = pairf(s, t);
              }
              const float nm = __fmaf_rn(f, w, cs.hs[s]);
              if (nm <= m) {
                m = nm;
                arg = s;
              }
            }
          }
          const bool win = valid && m <= msg_g;
          msg[kk] = win ? m : msg_g;
          am[kk] = win ? arg : argmin_h;
          own[kk] = win && m < msg_g;
        }
      }

      // Exps: the labels below the candidate need their own, every other
      // label shares the candidate's.  When one slot holds all the own labels
      // (the usual case) that slot's lanes evaluate them and its other lanes
      // the candidate, in one lane-parallel pass; otherwise the own values
      // are packed into the warp's lanes (in label order) with the
      // candidate after them.
      float e_g;
      bool all_ok = true;
      unsigned bsel = 0u;
      int nslot = 0;
      float xs = msg_g;
#pragma unroll
      for (int kk = 0; kk < KW; ++kk) {
        const unsigned b = __ballot_sync(FULL, own[kk]);
        nslot += (b != 0u) ? 1 : 0;
        bsel = (b != 0u) ? b : bsel;
        xs = own[kk] ? msg[kk] : xs;
      }
      if (nslot <= 1 && bsel != FULL) {
        float y;
        const bool okx = exp_try<kExact>(earg(xs), y, s_ehi, s_elo);
        all_ok = __all_sync(FULL, okx);
        e_g = __shfl_sync(FULL, y, __ffs(~bsel) - 1);
#pragma unroll
        for (int kk = 0; kk < KW; ++kk) {
          const bool valid = lvalid(kk);
          e[kk] = own[kk] ? y : (valid ? e_g : 0.0f);
        }
      } else {
        float* eb = cs.erow + c.t0;  // the warp's part of erow (free until the sum)
        const unsigned lt = (1u << lane) - 1u;
        int n_own = 0;
        int pos[KW];
#pragma unroll
        for (int kk = 0; kk < KW; ++kk) {
          const unsigned b = __ballot_sync(FULL, own[kk]);
          pos[kk] = n_own + __popc(b & lt);
          if (own[kk] && pos[kk] < 32) eb[pos[kk]] = msg[kk];
          n_own += __popc(b);
        }
        __syncwarp();
        if (n_own < 32) {
          const float x = (lane < n_own) ? eb[lane] : msg_g;
          float y;
          const bool okx = exp_try<kExact>(earg(x), y, s_ehi, s_elo);
          all_ok = __all_sync(FULL, lane > n_own || okx);
          __syncwarp();
          if (lane < n_own) eb[lane] = y;
          e_g = __shfl_sync(FULL, y, n_own);
          __syncwarp();
#pragma unroll
          for (int kk = 0; kk < KW; ++kk) {
            const bool valid = lvalid(kk);
            const float eo = eb[own[kk] ? pos[kk] : 0];
            e[kk] = own[kk] ? eo : (valid ? e_g : 0.0f);
          }
        } else {
          // more than a warp's worth: one pass per slot that has own labels
          all_ok = exp_try<kExact>(earg(msg_g), e_g, s_ehi, s_elo);
#pragma unroll
          for (int kk = 0; kk < KW; ++kk) {
            const bool valid = lvalid(kk);
            e[kk] = valid ? e_g : 0.0f;
            if (__any_sync(FULL, own[kk])) {
              float ex;
              const bool okx = exp_try<kExact>(earg(msg[kk]), ex, s_ehi, s_elo);
              e[kk] = own[kk] ? ex : e[kk];
              all_ok = all_ok && (okx || !own[kk]);
            }
          }
          all_ok = __all_sync(FULL, all_ok);
        }
        __syncwarp();  // erow is read again only after this step's sum
      }
      if (!all_ok) {
        // rounding undecided in float-float (rare): the reference expression
        e_g = static_cast<float>(exp(static_cast<double>(msg_g)));
#pragma unroll
        for (int kk = 0; kk < KW; ++kk) {
          const bool valid = lvalid(kk);
          e[kk] = own[kk] ? static_cast<float>(exp(static_cast<double>(msg[kk]))) : (valid ? e_g : 0.0f);
        }
      }
    }

    if constexpr (kRing) {
      __syncwarp();
      if (st == grp * G + G - 1 && issue_group<VARIANT, T>(a, c, sm, lroww, i + 1 - G + a.ns, grp, nsteps, lane))
        armed |= 1u << grp;
      if (!a.vec4) cp_async_commit();
    }

    // normalisation (lbp_min_sum_kernel.cu:166-181): sum tree over all labels
    float sum;
    if (NW == 1) {
      float ev[K];
#pragma unroll
      for (int k = 0; k < K; ++k) ev[k] = e[k % KW];
      sum = tree_sum<K>(ev, L, lane);
    } else {
#pragma unroll
      for (int kk = 0; kk < KW; ++kk) cs.erow[c.t0 + lane + 32 * kk] = e[kk];
      chain_sync<NW>(bar_id);
      float ev[K];
#pragma unroll
      for (int k = 0; k < K; ++k) ev[k] = cs.erow[lane + 32 * k];
      sum = tree_sum<K>(ev, L, lane);
    }
    // subtracted from every label: log of the sum (the reference's
    // normalisation) for float storage, the minimum of h for half storage
    const float lse = kExact ? norm_log(sum) : ref;

    // write the message at the receiver
    const int pq = pin + c.dpin;
    const int64_t qo = static_cast<int64_t>(pq) * Ls;
    T* dstm = c.slot_out + qo;
#pragma unroll
    for (int kk = 0; kk < KW; ++kk) {
      const int t = c.t0 + lane + 32 * kk;
      const T o = stf<T>(__fsub_rn(msg[kk], lse));
      chain[kk] = ldf<T>(o);  // the stored value, so the chain matches memory
      if (lvalid(kk)) dstm[t] = o;
    }
    {
      const int64_t ao = c.out_off + qo;
      if (a.argmin_kind == BPL_ARGMIN_U8) {
        uint8_t* d = static_cast<uint8_t*>(a.argmin) + ao;
#pragma unroll
        for (int kk = 0; kk < KW; ++kk)
          if (lvalid(kk)) d[c.t0 + lane + 32 * kk] = static_cast<uint8_t>(am[kk]);
      } else if (a.argmin_kind == BPL_ARGMIN_U16) {
        uint16_t* d = static_cast<uint16_t*>(a.argmin) + ao;
#pragma unroll
        for (int kk = 0; kk < KW; ++kk)
          if (lvalid(kk)) d[c.t0 + lane + 32 * kk] = static_cast<uint16_t>(am[kk]);
      } else if (a.argmin_kind == BPL_ARGMIN_F32) {
        float* d = static_cast<float*>(a.argmin) + ao;
#pragma unroll
        for (int kk = 0; kk < KW; ++kk)
          if (lvalid(kk)) d[c.t0 + lane + 32 * kk] = static_cast<float>(am[kk]);
      }
    }
    // (float)max((double)sum, 1e-45): the smallest positive float when sum is 0
    if (wic == 0 && lane == 0 && scale_out) scale_out[pq] = (sum > 0.0f) ? sum : __int_as_float(1);

    // next tap block
    if (j == 31 || i == nsteps - 1) {
      __syncwarp();
      if (32 * (b + 1) < nsteps) {
        store_taps(a, sm.taps + ((b + 1) & 1) * tile_stride, lane, tr, stereo);
        if (32 * (b + 2) < nsteps) load_taps(a, c, b + 2, lane, nsteps, tr, stereo);
      }
      __syncwarp();
    }
    if (kRing && ++st == a.ns) st = 0;
  }

  if (kRing && failed && a.vec4 && lane == 0) {
    // drain bulk copies still in flight before the warp's shared memory goes
    // away: each armed group's pending phase is the one `par` expects next
    // (one phase per group at most is outstanding, so the parity is
    // unambiguous)
    for (int g = 0; g < a.ns / G; ++g)
      if ((armed >> g) & 1u) (void)mbar_wait_bounded(&sm.bars[g], (par >> g) & 1u, kDrainLimit);
  }
  if (kRing && !a.vec4) cp_async_wait<0>();
}

// Host-side launch of one phase for one (K, variant, NW) instantiation.
template <int K, int V, int NW, typename T>
int launch_phase(const FwdArgs& a0, cudaStream_t stream) {
  FwdArgs a = a0;
  const int lroww = 32 * (K / NW);
  if (V == BPL_LBP_SEM_PIXEL && NW == 1 && a.ns > 0 && a.nchains > kHiOccChainsPerSm * sm_count()) {
    // one-warp blocks: the deepest ring (4..2 steps) whose shared memory lets
    // every scanline of the phase be resident at once; a second, partial
    // wave of full-length scanlines costs more than a shallower prefetch
    for (int ns = a.ns; ns >= 2; --ns) {
      const size_t pc = 4 * (static_cast<size_t>(chain_smem_floats(K)) +
                             static_cast<size_t>(warp_smem_floats(ns, lroww, a.lmat, a.Lv, sizeof(T))));
      const int per_sm = std::min(32, static_cast<int>(smem_per_sm() / (pc + smem_reserved_per_block())));
      a.ns = ns;
      if (static_cast<int64_t>(per_sm) * sm_count() >= a.nchains) break;
    }
  }
  const size_t per_chain = 4 * (static_cast<size_t>(chain_smem_floats(K)) +
                                static_cast<size_t>(NW) * warp_smem_floats(a.ns, lroww, a.lmat, a.Lv, sizeof(T)));
  // a phase with more scanlines than about 8 warps per SM runs 1-warp
  // blocks, kHiOcc resident per SM (registers capped near 120); fewer
  // scanlines run latency-bound in 4-warp blocks and keep every register
  // they use
  auto kern = lbp_forward_kernel<K, V, NW, T, 1>;
  int wmax = 4;
  if constexpr (K <= 8) {
    if (NW == 1 && a.nchains > kHiOccChainsPerSm * sm_count()) {
      kern = lbp_forward_kernel<K, V, NW, T, kHiOcc>;
      wmax = fwd_block_warps<kHiOcc>();
    }
  }
  // chains per block: up to wmax warps while the block fits in 200 KB
  const int cpb = std::max(1, std::min(wmax / NW, static_cast<int>((200 * 1024) / per_chain)));
  const size_t smem = per_chain * cpb;
  if (smem > 48 * 1024) {
    if (static_cast<int>(smem) > max_smem_optin())
      return set_error(BPL_ERR_UNSUPPORTED, "lbp_forward: shared memory %zu exceeds device limit", smem);
    BPL_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)),
                 "cudaFuncSetAttribute");
  }
  const int blocks = (a.nchains + cpb - 1) / cpb;
  kern<<<blocks, 32 * NW * cpb, smem, stream>>>(a);
  BPL_CUDA_TRY(cudaGetLastError(), "lbp_forward launch");
  return BPL_OK;
}

// Scanlines of a phase that a one-warp-per-scanline launch keeps busy: below
// about six per SM the sweep is latency-bound and the labels of each scanline
// are split over several warps.
inline bool split_chains(int nchains) { return nchains < kSplitChainsPerSm * sm_count(); }

// K: register slots per lane (K * 32 >= L).  KS, NS: the instantiation and
// warp count used when a phase's scanlines are split.
template <int K, int V, int KS, int NS, typename T>
int launch_k(const FwdArgs& a0, cudaStream_t stream) {
  FwdArgs a = a0;
  for (int phase = 0; phase < 2; ++phase) {
    BPL_TRACE(phase == 0 ? "lbp_forward: horizontal sweeps" : "lbp_forward: vertical sweeps");
    a.phase = phase;
    a.nchains = 2 * a.B * (phase == 0 ? a.H : a.W);
    int st;
    if (NS > 1 && split_chains(a.nchains)) st = launch_phase<KS, V, NS, T>(a, stream);
    else st = launch_phase<K, V, 1, T>(a, stream);
    if (st != BPL_OK) return st;
  }
  return BPL_OK;
}

template <int V, typename T = float>
int dispatch_k(const FwdArgs& a, cudaStream_t s) {
  const int k = (a.L + 31) / 32;
  if constexpr (V != BPL_LBP_STEREO) {
    // semantic variants: one warp per scanline
    if constexpr (V == BPL_LBP_SEM_PIXEL) {
      // per-pixel L x L matrices: staged through the ring up to L = 96,
      // read from global memory above
      if (k == 1) return launch_k<1, V, 1, 1, T>(a, s);
      if (k == 2) return launch_k<2, V, 2, 1, T>(a, s);
      if (k == 3) return launch_k<3, V, 3, 1, T>(a, s);
      if (k <= 8) return launch_k<8, V, 8, 1, T>(a, s);
      return launch_k<32, V, 32, 1, T>(a, s);
    }
    switch (k) {
      case 1: return launch_k<1, V, 1, 1, T>(a, s);
      case 2: return launch_k<2, V, 2, 1, T>(a, s);
      case 3: return launch_k<3, V, 3, 1, T>(a, s);
      case 4: return launch_k<4, V, 4, 1, T>(a, s);
      default:
        if (k <= 8) return launch_k<8, V, 8, 1, T>(a, s);
        if (k <= 16) return launch_k<16, V, 16, 1, T>(a, s);
        return launch_k<32, V, 32, 1, T>(a, s);
    }
  } else {
    // (the split-scanline instantiations KS/NS are enabled together with
    // kSplitChainsPerSm; with it at 0 every phase runs one warp per scanline)
    switch (k) {
      case 1: return launch_k<1, V, 1, 1, T>(a, s);
      case 2: return launch_k<2, V, 2, 1, T>(a, s);
      case 3: return launch_k<3, V, 3, 1, T>(a, s);
      case 4: return launch_k<4, V, 4, 1, T>(a, s);
      case 5: return launch_k<5, V, 5, 1, T>(a, s);
      case 6: return launch_k<6, V, 6, 1, T>(a, s);
      case 7: return launch_k<7, V, 7, 1, T>(a, s);
      case 8: return launch_k<8, V, 8, 1, T>(a, s);
      default:
        if (k <= 12) return launch_k<12, V, 12, 1, T>(a, s);
        if (k <= 16) return launch_k<16, V, 16, 1, T>(a, s);
        if (k <= 24) return launch_k<24, V, 24, 1, T>(a, s);
        return launch_k<32, V, 32, 1, T>(a, s);
    }
  }
}

int lbp_forward_stereo(const FwdArgs& a, cudaStream_t s);
int lbp_forward_sem_global(const FwdArgs& a, cudaStream_t s);
int lbp_forward_sem_pixel(const FwdArgs& a, cudaStream_t s);
int lbp_forward_stereo_f16(const FwdArgs& a, cudaStream_t s);
int lbp_forward_sem_pixel_f16(const FwdArgs& a, cudaStream_t s);
int lbp_forward_sem_global_f16(const FwdArgs& a, cudaStream_t s);

}  // namespace bpl

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
//     cross-direction messages) are streamed into a per-warp shared-memory
//     ring NS pixels ahead with TMA 1-D bulk copies (cp.async.bulk +
//     mbarrier), or 4-byte cp.async when a row is not 16-byte sized.
//   * Labels are spread over lanes (label = lane + 32k); min/argmin and the
//     exp-sum follow the reference's reduction tree exactly (bpl_device.cuh).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>

#include "bpl_crmath.cuh"
#include "bpl_device.cuh"
#include "bpl_internal.h"

namespace bpl {

// ring depth when rows are fetched with 4-byte cp.async (compile-time for
// cp.async.wait_group)
constexpr int kRingCpAsync = 4;

struct FwdArgs {
  const float* cost;
  const float* jump;
  const float* edge;
  float* msgs;
  void* argmin;
  float* scale;
  int B, H, W, L, Lv, jb, eb, delta;
  int argmin_kind;
  int phase;  // 0: RIGHT+LEFT over rows, 1: DOWN+UP over columns
  int nchains;
  int ns;     // ring depth
  int lrow;   // floats per ring row (L rounded up to 4)
  int lmat;   // floats of the per-pixel pairwise matrix in a stage (pixel variant), else 0
  int vec4;   // rows are 16-byte sized: use bulk copies
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
__device__ __forceinline__ float norm_log(float sum) {
  float y;
  if (!crm::log_fast(sum, y)) y = static_cast<float>(log(fmax(static_cast<double>(sum), 1e-45)));
  return y;
}

// Per-warp shared memory carve-up (all offsets in floats, 16-byte aligned).
struct WarpSmem {
  float* ring;      // ns * (3*lrow + lmat)
  uint64_t* bars;   // ns
  float* hs;        // 32*K : h of the current pixel
  float* taps;      // 2 * (Lv+1) * 33 : stereo taps + edge weight for 32 pixels
};

__host__ __device__ inline int align4(int v) { return (v + 3) & ~3; }

__host__ __device__ inline int stage_floats(int lrow, int lmat) { return 3 * lrow + lmat; }

__host__ __device__ inline int warp_smem_floats(int K, int ns, int lrow, int lmat, int Lv) {
  const int ring = ns * stage_floats(lrow, lmat);
  const int bars = 2 * align4(ns);  // ns uint64 -> 2 floats each, padded
  const int hs = 32 * K;
  const int taps = align4(2 * (Lv + 1) * 33);
  return align4(ring) + bars + align4(hs) + taps;
}

template <int K>
__device__ __forceinline__ WarpSmem carve(float* base, const FwdArgs& a) {
  WarpSmem s;
  s.ring = base;
  float* p = base + align4(a.ns * stage_floats(a.lrow, a.lmat));
  s.bars = reinterpret_cast<uint64_t*>(p);
  p += 2 * align4(a.ns);
  s.hs = p;
  p += align4(32 * K);
  s.taps = p;
  return s;
}

// Chain geometry helpers --------------------------------------------------
struct Chain {
  int n, dir, fixed;  // fixed = y (horizontal) or x (vertical)
  int len;            // pixels along the chain
  int64_t HW;
};

__device__ __forceinline__ int chain_coord(const Chain& c, int i) {
  // coordinate along the chain of the sender at step i
  return (c.dir == RIGHT || c.dir == DOWN) ? i : (c.len - 1 - i);
}

__device__ __forceinline__ int64_t pix_index(const FwdArgs& a, const Chain& c, int i) {
  const int v = chain_coord(c, i);
  const int y = (a.phase == 0) ? c.fixed : v;
  const int x = (a.phase == 0) ? v : c.fixed;
  return (static_cast<int64_t>(c.n) * a.H + y) * a.W + x;
}

// messages offset (floats) of slot `slot` at pixel linear index p of batch n
__device__ __forceinline__ int64_t msg_off(const FwdArgs& a, int n, int slot, int64_t p) {
  const int64_t HW = static_cast<int64_t>(a.H) * a.W;
  const int64_t pin = p - static_cast<int64_t>(n) * HW;  // pixel index within image
  return ((static_cast<int64_t>(n) * 4 + slot) * HW + pin) * a.L;
}

// Issues the ring stage for step i (cost + the two cross-direction messages
// [+ the per-pixel pairwise matrix]).
template <int VARIANT>
__device__ __forceinline__ void issue_stage(const FwdArgs& a, const Chain& c, const WarpSmem& sm,
                                            int i, int lane) {
  const int st = i % a.ns;
  float* dst = sm.ring + static_cast<int64_t>(st) * stage_floats(a.lrow, a.lmat);
  const int64_t p = pix_index(a, c, i);
  const int sa = (a.phase == 0) ? UP : RIGHT;
  const int sb = (a.phase == 0) ? DOWN : LEFT;
  const float* src0 = a.cost + p * a.L;
  const float* src1 = a.msgs + msg_off(a, c.n, sa, p);
  const float* src2 = a.msgs + msg_off(a, c.n, sb, p);
  const float* src3 = nullptr;
  int bytes3 = 0;
  if (VARIANT == BPL_LBP_SEM_PIXEL) {
    const int v = chain_coord(c, i);
    const int y = (a.phase == 0) ? c.fixed : v;
    const int x = (a.phase == 0) ? v : c.fixed;
    src3 = a.jump + (((static_cast<int64_t>(c.dir) * a.H + y) * a.W + x) * a.L) * a.L;
    bytes3 = a.L * a.L * 4;
  }
  if (a.vec4) {
    if (lane == 0) {
      const uint32_t rb = static_cast<uint32_t>(a.L) * 4u;
      fence_proxy_async();
      mbar_arrive_expect_tx(&sm.bars[st], 3u * rb + static_cast<uint32_t>(bytes3));
      bulk_g2s(dst, src0, rb, &sm.bars[st]);
      bulk_g2s(dst + a.lrow, src1, rb, &sm.bars[st]);
      bulk_g2s(dst + 2 * a.lrow, src2, rb, &sm.bars[st]);
      if (VARIANT == BPL_LBP_SEM_PIXEL) bulk_g2s(dst + 3 * a.lrow, src3, static_cast<uint32_t>(bytes3), &sm.bars[st]);
    }
  } else {
    for (int t = lane; t < a.L; t += 32) {
      cp_async4(dst + t, src0 + t);
      cp_async4(dst + a.lrow + t, src1 + t);
      cp_async4(dst + 2 * a.lrow + t, src2 + t);
    }
    if (VARIANT == BPL_LBP_SEM_PIXEL)
      for (int t = lane; t < a.L * a.L; t += 32) cp_async4(dst + 3 * a.lrow + t, src3 + t);
  }
}

// Stereo taps + edge weight for the 32 pixels of block b: lane j loads pixel
// (32b + j).  Held in registers until written to the tile.
struct TapRegs {
  float t[16];
  float w;
};

__device__ __forceinline__ void load_taps(const FwdArgs& a, const Chain& c, int b, int lane, int nsteps,
                                          TapRegs& r, bool stereo) {
  const int i = 32 * b + lane;
  if (i >= nsteps) return;
  const int v = chain_coord(c, i);
  const int y = (a.phase == 0) ? c.fixed : v;
  const int x = (a.phase == 0) ? v : c.fixed;
  const int64_t HW = static_cast<int64_t>(a.H) * a.W;
  const int ne = (a.eb == 1) ? 0 : c.n;
  r.w = __ldg(a.edge + (static_cast<int64_t>(ne) * 4 + c.dir) * HW + static_cast<int64_t>(y) * a.W + x);
  if (stereo) {
    const int nj = (a.jb == 1) ? 0 : c.n;
    const float* base = a.jump + ((static_cast<int64_t>(nj) * 4 + c.dir) * a.Lv) * HW + static_cast<int64_t>(y) * a.W + x;
#pragma unroll
    for (int k = 0; k < 16; ++k)
      if (k < a.Lv) r.t[k] = __ldg(base + static_cast<int64_t>(k) * HW);
  }
}

__device__ __forceinline__ void store_taps(const FwdArgs& a, float* tile, int lane, const TapRegs& r,
                                           bool stereo) {
  // tile layout: [Lv+1][33]; row Lv holds the edge weight
  tile[a.Lv * 33 + lane] = r.w;
  if (stereo) {
#pragma unroll
    for (int k = 0; k < 16; ++k)
      if (k < a.Lv) tile[k * 33 + lane] = r.t[k];
  }
}

template <int K, int VARIANT>
__global__ void __launch_bounds__(128) lbp_forward_kernel(FwdArgs a) {
  extern __shared__ __align__(16) float smem[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int chain_id = blockIdx.x * (blockDim.x >> 5) + wib;
  if (chain_id >= a.nchains) return;  // whole warp leaves; no block barriers below

  const int per_warp = warp_smem_floats(K, a.ns, a.lrow, a.lmat, a.Lv);
  WarpSmem sm = carve<K>(smem + static_cast<int64_t>(wib) * per_warp, a);
  // exp table for lane-varying lookups: every warp writes the same values
  __shared__ float s_ehi[64], s_elo[64];
  s_ehi[lane] = crm::kTab.exp_hi[lane];
  s_ehi[lane + 32] = crm::kTab.exp_hi[lane + 32];
  s_elo[lane] = crm::kTab.exp_lo[lane];
  s_elo[lane + 32] = crm::kTab.exp_lo[lane + 32];
  __syncwarp();

  Chain c;
  const int r = chain_id >> 1;
  if (a.phase == 0) {
    c.dir = (chain_id & 1) ? LEFT : RIGHT;
    c.n = r / a.H;
    c.fixed = r % a.H;
    c.len = a.W;
  } else {
    c.dir = (chain_id & 1) ? UP : DOWN;
    c.n = r / a.W;
    c.fixed = r % a.W;
    c.len = a.H;
  }
  const int nsteps = c.len - 1;
  if (nsteps <= 0) return;
  const int od = c.dir ^ 1;
  const int L = a.L;
  const bool stereo = (VARIANT == BPL_LBP_STEREO);

  // ring start-up
  if (a.vec4 && lane == 0) {
    for (int s = 0; s < a.ns; ++s) mbar_init(&sm.bars[s], 1);
    fence_mbar_init();
  }
  __syncwarp();
  for (int i = 0; i < a.ns; ++i) {
    if (i < nsteps) issue_stage<VARIANT>(a, c, sm, i, lane);
    if (!a.vec4) cp_async_commit();
  }

  // incoming chain message at the first sender (slot = chain direction's
  // opposite side, i.e. the slot the sweep itself writes)
  float chain[K];
  {
    const int64_t p0 = pix_index(a, c, 0);
    const float* src = a.msgs + msg_off(a, c.n, od, p0);
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int t = lane + 32 * k;
      chain[k] = (t < L) ? src[t] : 0.0f;
    }
  }

  TapRegs tr;
  load_taps(a, c, 0, lane, nsteps, tr, stereo);
  store_taps(a, sm.taps, lane, tr, stereo);
  if (nsteps > 32) load_taps(a, c, 1, lane, nsteps, tr, stereo);
  __syncwarp();

  bool failed = false;
  for (int i = 0; i < nsteps; ++i) {
    const int st = i % a.ns;
    const int j = i & 31;
    const int b = i >> 5;
    const float* tile = sm.taps + (b & 1) * ((a.Lv + 1) * 33);
    const float* stg = sm.ring + static_cast<int64_t>(st) * stage_floats(a.lrow, a.lmat);

    // wait for stage i
    if (a.vec4) {
      const bool ok = mbar_wait_bounded(&sm.bars[st], static_cast<uint32_t>((i / a.ns) & 1));
      if (!__all_sync(FULL, ok)) { failed = true; break; }
    } else {
      cp_async_wait<kRingCpAsync - 1>();  // groups 0..i have landed
      __syncwarp();
    }

    // h = cost + incoming messages except the chain direction's own slot,
    // added in the reference order RIGHT, LEFT, UP, DOWN.
    float h[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int t = lane + 32 * k;
      if (t < L) {
        const float cst = stg[t];
        const float va = stg[a.lrow + t];
        const float vb = stg[2 * a.lrow + t];
        h[k] = (a.phase == 0) ? __fadd_rn(__fadd_rn(__fadd_rn(cst, chain[k]), va), vb)
                              : __fadd_rn(__fadd_rn(__fadd_rn(cst, va), vb), chain[k]);
      } else {
        h[k] = 0.0f;
      }
    }
    float pw_reg[K];  // per-pixel pairwise row read later (pixel variant)
    (void)pw_reg;
#pragma unroll
    for (int k = 0; k < K; ++k) sm.hs[lane + 32 * k] = h[k];

    // pixel variant: keep the stage until the window loop has read it
    __syncwarp();
    if (VARIANT != BPL_LBP_SEM_PIXEL) {
      // stage st is free: refill it with step i + ns
      if (i + a.ns < nsteps) issue_stage<VARIANT>(a, c, sm, i + a.ns, lane);
      if (!a.vec4) cp_async_commit();
    }

    // per-pixel parameters
    const float w = tile[a.Lv * 33 + j];
    const int delta = a.delta;
    float msg[K];
    int am[K];

    if (delta >= L) {
      // full minimisation (lbp_min_sum_kernel.cu:88-111): last minimiser wins
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const int t = lane + 32 * k;
        float m = 1e15f;
        int arg = 0;
        if (t < L) {
          for (int s = 0; s < L; ++s) {
            float f;
            if (stereo) {
              int ti = a.Lv / 2 + (t - s);
              ti = max(1, min(a.Lv - 1, ti));
              f = tile[ti * 33 + j];
            } else if (VARIANT == BPL_LBP_SEM_GLOBAL) {
              f = __ldg(a.jump + (static_cast<int64_t>(c.dir) * L + s) * L + t);
            } else {
              f = stg[3 * a.lrow + s * L + t];
            }
            const float nm = __fmaf_rn(f, w, sm.hs[s]);
            m = fminf(m, nm);
            if (m == nm) arg = s;
          }
        }
        msg[k] = m;
        am[k] = arg;
      }
    } else {
      // truncated branch (lbp_min_sum_kernel.cu:112-164)
      float tv[K];
      int tl[K];
#pragma unroll
      for (int k = 0; k < K; ++k) {
        tv[k] = h[k];
        tl[k] = lane + 32 * k;
      }
      float min_h;
      int argmin_h;
      tree_argmin<K>(tv, tl, L, lane, min_h, argmin_h);
      float L2, off = 0.0f;
      if (stereo) {
        L2 = tile[(a.Lv - 1) * 33 + j];
        off = tile[0 * 33 + j];
      } else if (VARIANT == BPL_LBP_SEM_GLOBAL) {
        L2 = __ldg(a.jump + (static_cast<int64_t>(c.dir) * L + 0) * L + (L - 1));
      } else {
        L2 = stg[3 * a.lrow + (L - 1)];
      }
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const int t = lane + 32 * k;
        float m = __fmaf_rn(L2, w, min_h);
        int arg = argmin_h;
        if (t < L) {
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
              int ti = a.Lv / 2 + (t - s);
              ti = max(1, min(a.Lv - 1, ti));
              f = tile[ti * 33 + j];
            } else if (VARIANT == BPL_LBP_SEM_GLOBAL) {
              f = __ldg(a.jump + (static_cast<int64_t>(c.dir) * L + s) * L + t);
            } else {
              f = stg[3 * a.lrow + s * L + t];
            }
            const float nm = __fmaf_rn(f, w, sm.hs[s]);
            if (nm <= m) {
              m = nm;
              arg = s;
            }
          }
        }
        msg[k] = m;
        am[k] = arg;
      }
    }

    if (VARIANT == BPL_LBP_SEM_PIXEL) {
      __syncwarp();
      if (i + a.ns < nsteps) issue_stage<VARIANT>(a, c, sm, i + a.ns, lane);
      if (!a.vec4) cp_async_commit();
    }

    // normalisation (lbp_min_sum_kernel.cu:166-181)
    float e[K];
#pragma unroll
    for (int k = 0; k < K; ++k) e[k] = (lane + 32 * k < L) ? norm_exp(msg[k], s_ehi, s_elo) : 0.0f;
    const float sum = tree_sum<K>(e, L, lane);
    const double sum_exp = fmax(static_cast<double>(sum), 1e-45);
    const float lse = norm_log(sum);

    // write the message at the receiver
    const int64_t pq = pix_index(a, c, i) + ((a.phase == 0) ? ((c.dir == RIGHT) ? 1 : -1)
                                                            : ((c.dir == DOWN) ? a.W : -a.W));
    const int64_t qo = msg_off(a, c.n, od, pq);
    float* dstm = a.msgs + qo;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int t = lane + 32 * k;
      const float o = __fsub_rn(msg[k], lse);
      chain[k] = o;
      if (t < L) {
        dstm[t] = o;
        if (a.argmin_kind == BPL_ARGMIN_F32) static_cast<float*>(a.argmin)[qo + t] = static_cast<float>(am[k]);
        else if (a.argmin_kind == BPL_ARGMIN_U8) static_cast<uint8_t*>(a.argmin)[qo + t] = static_cast<uint8_t>(am[k]);
        else if (a.argmin_kind == BPL_ARGMIN_U16) static_cast<uint16_t*>(a.argmin)[qo + t] = static_cast<uint16_t>(am[k]);
      }
    }
    if (lane == 0) a.scale[qo / L] = static_cast<float>(sum_exp);

    // next tap block
    if (j == 31 || i == nsteps - 1) {
      __syncwarp();
      if (32 * (b + 1) < nsteps) {
        store_taps(a, sm.taps + ((b + 1) & 1) * ((a.Lv + 1) * 33), lane, tr, stereo);
        if (32 * (b + 2) < nsteps) load_taps(a, c, b + 2, lane, nsteps, tr, stereo);
      }
      __syncwarp();
    }
  }

  if (failed && a.vec4 && lane == 0) {
    // drain bulk copies still in flight before the warp's shared memory goes
    // away: every stage issued so far completes one more phase
    for (int s = 0; s < a.ns; ++s)
      if (!mbar_try_wait(&sm.bars[s], 0) && !mbar_try_wait(&sm.bars[s], 1))
        (void)mbar_wait_bounded(&sm.bars[s], 0, 1u << 16);
  }
  if (!a.vec4) cp_async_wait<0>();
}
// Host-side launch of both phases for one (K, variant) instantiation.
template <int K, int V>
int launch_k(const FwdArgs& a0, cudaStream_t stream) {
  FwdArgs a = a0;
  const int per_warp = warp_smem_floats(K, a.ns, a.lrow, a.lmat, a.Lv) * 4;
  // up to 4 warps (scanlines) per block while the block fits in 200 KB
  const int kWarpsPerBlock = std::max(1, std::min(4, (200 * 1024) / per_warp));
  const size_t smem = static_cast<size_t>(per_warp) * kWarpsPerBlock;
  auto kern = lbp_forward_kernel<K, V>;
  if (smem > 48 * 1024) {
    if (static_cast<int>(smem) > max_smem_optin())
      return set_error(BPL_ERR_UNSUPPORTED, "lbp_forward: shared memory %zu exceeds device limit", smem);
    BPL_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)),
                 "cudaFuncSetAttribute");
  }
  for (int phase = 0; phase < 2; ++phase) {
    a.phase = phase;
    a.nchains = 2 * a.B * (phase == 0 ? a.H : a.W);
    const int blocks = (a.nchains + kWarpsPerBlock - 1) / kWarpsPerBlock;
    kern<<<blocks, 32 * kWarpsPerBlock, smem, stream>>>(a);
    BPL_CUDA_TRY(cudaGetLastError(), "lbp_forward launch");
  }
  return BPL_OK;
}

template <int V>
int dispatch_k(const FwdArgs& a, cudaStream_t s) {
  const int k = (a.L + 31) / 32;
  if constexpr (V == BPL_LBP_SEM_PIXEL) {
    // per-pixel L x L matrices: L <= 96 (checked at the entry point)
    if (k == 1) return launch_k<1, V>(a, s);
    if (k == 2) return launch_k<2, V>(a, s);
    return launch_k<3, V>(a, s);
  }
  switch (k) {
    case 1: return launch_k<1, V>(a, s);
    case 2: return launch_k<2, V>(a, s);
    case 3: return launch_k<3, V>(a, s);
    case 4: return launch_k<4, V>(a, s);
    case 5: return launch_k<5, V>(a, s);
    case 6: return launch_k<6, V>(a, s);
    case 7: return launch_k<7, V>(a, s);
    case 8: return launch_k<8, V>(a, s);
    default:
      if (k <= 12) return launch_k<12, V>(a, s);
      if (k <= 16) return launch_k<16, V>(a, s);
      if (k <= 24) return launch_k<24, V>(a, s);
      return launch_k<32, V>(a, s);
  }
}


int lbp_forward_stereo(const FwdArgs& a, cudaStream_t s);
int lbp_forward_sem_global(const FwdArgs& a, cudaStream_t s);
int lbp_forward_sem_pixel(const FwdArgs& a, cudaStream_t s);

}  // namespace bpl

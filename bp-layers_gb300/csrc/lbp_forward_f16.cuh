// Min-sum LBP forward with FP16 storage, stereo pairwise: the lean step.
//
// Same sweeps, scanline ownership and label layout as lbp_forward_kernel
// (one warp walks one scanline of one sweep, label = lane + 32k, the chain
// message stays in registers), but the step is built for FP16 storage, which
// has no bitwise target:
//   * every stored row is the min-sum message minus the minimum of h over
//     the sender's labels (min-normalisation): no exp, no sum, no log on the
//     scanline's dependency chain.  The row is a constant per (pixel,
//     direction) away from the reference's log-normalised message, which
//     changes neither the next minimisation's argmin nor the beliefs' softmin;
//     the adjoint recomputes the normalisation from the row it reads;
//   * ties are broken by whichever minimiser the warp's reduction finds (the
//     label of an exact tie carries the same value; the reference's tree order
//     matters only for bitwise equality);
//   * window terms that cannot beat the global candidate (their tap times w
//     is at least the candidate's, the "tie-only" offsets of the FP32 kernel)
//     are not evaluated at all;
//   * the per-message scale (the sum of exp of the stored row) is computed
//     only when the caller asks for it (SCALE), off the chain.
// All arithmetic is FP32 (cost and messages are converted when loaded); the
// rounding of each stored message to half is the only FP16 operation.
//
// Reference semantics followed (sweep order, h, window, candidate):
// ops/lbp_stereo/src/lbp_min_sum_kernel.cu:55-164.
#pragma once

#include <type_traits>
#include <utility>

#include "lbp_forward.cuh"

namespace bpl {

// compile-time loop: f(integral_constant<int, 0>), ..., f(integral_constant<int, N-1>)
template <typename F, int... I>
__device__ __forceinline__ void static_for_impl(F& f, std::integer_sequence<int, I...>) {
  (f(std::integral_constant<int, I>{}), ...);
}
template <int N, typename F>
__device__ __forceinline__ void static_for(F&& f) {
  static_for_impl(f, std::make_integer_sequence<int, N>{});
}

template <int OCC>
constexpr int f16_block_warps() { return (OCC > 1) ? 1 : 4; }

// PF: prefetch depth (steps whose rows are in flight).  The lean step is
// short, so one step ahead does not cover a DRAM load (ncu: long-scoreboard
// stalls led the one-ahead version); the 4-warp, latency-bound launch keeps
// three steps in flight, the high-occupancy launch one (its other warps hide
// the latency, and it has no registers to spare).
template <int K, int OCC, bool SCALE, int PF>
__global__ void __launch_bounds__(32 * f16_block_warps<OCC>(), OCC) lbp_forward_f16_kernel(FwdArgs a) {
  extern __shared__ __align__(16) float smem[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int chain_id = blockIdx.x * (blockDim.x >> 5) + wib;
  if (chain_id >= a.nchains) return;

  // per warp: h row (32K + 2 pads) and the two-block tap tile
  const int tile_stride = tap_tile_rows(a.Lv) * 33;
  float* base = smem + static_cast<int64_t>(wib) * (align4(32 * K + 2 * kHsPad) + 2 * tile_stride);
  float* hs = base + kHsPad;
  float* taps = base + align4(32 * K + 2 * kHsPad);
  if (lane < kHsPad) {
    hs[-1 - lane] = __int_as_float(0x7f800000);
    hs[32 * K + lane] = __int_as_float(0x7f800000);
  }

  const int L = a.L;
  const int Ls = a.Ls;
  const int64_t HW = static_cast<int64_t>(a.H) * a.W;
  const int64_t HWL = HW * Ls;
  Chain<__half> c;
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
  const __half* cost = static_cast<const __half*>(a.cost) + static_cast<int64_t>(c.n) * HWL;
  const __half* slot_a = static_cast<const __half*>(a.msgs) + (static_cast<int64_t>(c.n) * 4 + sa) * HWL;
  const __half* slot_b = static_cast<const __half*>(a.msgs) + (static_cast<int64_t>(c.n) * 4 + sb) * HWL;
  c.out_off = (static_cast<int64_t>(c.n) * 4 + od) * HWL;
  __half* slot_out = static_cast<__half*>(a.msgs) + c.out_off;
  c.t0 = 0;
  float* scale_out = SCALE ? a.scale + (static_cast<int64_t>(c.n) * 4 + od) * HW : nullptr;
  // only the last slot can hold labels >= L (K = ceil(L/32))
  auto lvalid = [&](int kk) -> bool { return kk < K - 1 || lane + 32 * kk < L; };

  // the next step's cost and cross-direction messages, one step ahead
  __half pcst[PF][K], pva[PF][K], pvb[PF][K];
  auto prefetch = [&](auto SL, int i) {
    constexpr int sl = decltype(SL)::value;
    const int64_t po = static_cast<int64_t>(c.pin0 + i * c.dpin) * Ls;
#pragma unroll
    for (int kk = 0; kk < K; ++kk) {
      const int64_t o = po + (lvalid(kk) ? lane + 32 * kk : 0);
      pcst[sl][kk] = __ldg(cost + o);
      pva[sl][kk] = __ldg(slot_a + o);
      pvb[sl][kk] = __ldg(slot_b + o);
    }
  };
  static_for<PF>([&](auto SL) {
    constexpr int s = decltype(SL)::value;
    if (s < nsteps) prefetch(SL, s);
  });

  float chain[K];
  {
    const __half* src = slot_out + static_cast<int64_t>(c.pin0) * Ls;
#pragma unroll
    for (int kk = 0; kk < K; ++kk) chain[kk] = lvalid(kk) ? __half2float(src[lane + 32 * kk]) : 0.0f;
  }

  TapRegs tr;
  load_taps(a, c, 0, lane, nsteps, tr, true);
  store_taps(a, taps, lane, tr, true);
  if (nsteps > 32) load_taps(a, c, 1, lane, nsteps, tr, true);
  __syncwarp();

  const int delta = a.delta;
  const bool store_am = a.argmin_kind != BPL_ARGMIN_NONE;
  const float kInf = __int_as_float(0x7f800000);
  const int c0 = a.Lv / 2;
  auto step = [&](auto SL, const int i) {
    constexpr int sl = decltype(SL)::value;
    const int pin = c.pin0 + i * c.dpin;
    const int j = i & 31;
    const int b = i >> 5;
    const float* tile = taps + (b & 1) * tile_stride;

    // h = cost + incoming messages except the chain direction's own slot,
    // in the reference's order (RIGHT, LEFT, UP, DOWN)
    float h[K];
    float pm = kInf;
#pragma unroll
    for (int kk = 0; kk < K; ++kk) {
      const float cst = __half2float(pcst[sl][kk]);
      const float va = __half2float(pva[sl][kk]);
      const float vb = __half2float(pvb[sl][kk]);
      const float hv = (a.phase == 0) ? ((cst + chain[kk]) + va) + vb : ((cst + va) + vb) + chain[kk];
      h[kk] = lvalid(kk) ? hv : kInf;
      hs[lane + 32 * kk] = h[kk];
      pm = fminf(pm, h[kk]);
    }
    pm = warp_min_redux(pm);
    int argmin_h = 0;
    if (store_am) {
      int ll = -1;
#pragma unroll
      for (int kk = 0; kk < K; ++kk) ll = (h[kk] == pm) ? lane + 32 * kk : ll;
      argmin_h = __reduce_max_sync(FULL, ll);
    }
    __syncwarp();  // h of the whole pixel is visible in hs
    if (i + PF < nsteps) prefetch(SL, i + PF);

    const float w = tile[a.Lv * 33 + j];
    float msg[K];
    int am[K];
    if (delta >= L) {
      // full minimisation (lbp_min_sum_kernel.cu:88-111)
#pragma unroll
      for (int kk = 0; kk < K; ++kk) {
        const int t = lane + 32 * kk;
        float m = kInf;
        int arg = 0;
        if (t < L) {
          for (int s = 0; s < L; ++s) {
            const float f = tile[max(1, min(a.Lv - 1, c0 + (t - s))) * 33 + j];
            const float nm = __fmaf_rn(f, w, hs[s]);
            if (nm <= m) {
              m = nm;
              arg = s;
            }
          }
        }
        msg[kk] = m;
        am[kk] = arg;
      }
    } else {
      // truncated branch (lbp_min_sum_kernel.cu:112-164): the global
      // candidate L2*w + min h, and the window terms that can beat it
      const float L2 = tile[(a.Lv - 1) * 33 + j];
      const float msg_g = __fmaf_rn(L2, w, pm);
      const int wcode = __float_as_int(tile[(a.Lv + 2) * 33 + j]);
      const int R = ((wcode & 0xff) != kWinGeneric) ? (wcode & 0xff) - 2 : -2;
      float mw[K];
      int aw[K];
      if (R == 1) {
        const float fm1 = tile[min(a.Lv - 1, c0 + 1) * 33 + j];  // sender t-1
        const float f00 = tile[c0 * 33 + j];                     // sender t
        const float fp1 = tile[max(1, c0 - 1) * 33 + j];         // sender t+1
#pragma unroll
        for (int kk = 0; kk < K; ++kk) {
          const int t = lane + 32 * kk;
          const float n0 = __fmaf_rn(f00, w, h[kk]);
          const float nl = __fmaf_rn(fm1, w, hs[t - 1]);
          const float nr = __fmaf_rn(fp1, w, hs[t + 1]);
          float m = n0;
          int arg = t;
          m = (nl < m) ? nl : m;
          arg = (nl < n0) ? t - 1 : arg;
          const bool kr = nr < m;
          mw[kk] = kr ? nr : m;
          aw[kk] = kr ? t + 1 : arg;
        }
      } else if (R >= -1) {
        // R in {-1, 0, 2}: taps of senders t-2 .. t+2 (terms beyond R skipped)
        float fR[5];
#pragma unroll
        for (int q = 0; q < 5; ++q) fR[q] = tile[max(1, min(a.Lv - 1, c0 - (q - 2))) * 33 + j];
#pragma unroll
        for (int kk = 0; kk < K; ++kk) {
          const int t = lane + 32 * kk;
          float m = kInf;
          int arg = 0;
#pragma unroll
          for (int q = 0; q < 5; ++q) {
            const int jd = q - 2;
            const float nm = __fmaf_rn(fR[q], w, hs[t + jd]);
            const bool take = (jd >= -R) && (jd <= R) && (nm < m);
            m = take ? nm : m;
            arg = take ? t + jd : arg;
          }
          mw[kk] = m;
          aw[kk] = arg;
        }
      } else {
        // generic window (offsets, wider beating ranges): the reference's
        // rounded start / stop around t + offset
        const float off = tile[0 * 33 + j];
#pragma unroll
        for (int kk = 0; kk < K; ++kk) {
          const int t = lane + 32 * kk;
          float m = kInf;
          int arg = 0;
          if (t < L) {
            const int start = sat_u16(roundf(__fsub_rn(__fadd_rn(static_cast<float>(t - (delta - 1)), off), 1.0f)));
            const int stop = min(sat_u16(roundf(__fadd_rn(__fadd_rn(static_cast<float>(t + delta), off), 1.0f))), L);
            for (int s = start; s < stop; ++s) {
              const float f = tile[max(1, min(a.Lv - 1, c0 + (t - s))) * 33 + j];
              const float nm = __fmaf_rn(f, w, hs[s]);
              if (nm < m) {
                m = nm;
                arg = s;
              }
            }
          }
          mw[kk] = m;
          aw[kk] = arg;
        }
      }
#pragma unroll
      for (int kk = 0; kk < K; ++kk) {
        const bool win = mw[kk] < msg_g;
        msg[kk] = win ? mw[kk] : msg_g;
        am[kk] = win ? aw[kk] : argmin_h;
      }
    }

    // store the row relative to the minimum of h; the chain carries the
    // stored (half-rounded) value, so it matches memory
    const int pq = pin + c.dpin;
    const int64_t qo = static_cast<int64_t>(pq) * Ls;
    __half* dstm = slot_out + qo;
    float esum = 0.0f;
#pragma unroll
    for (int kk = 0; kk < K; ++kk) {
      const __half o = __float2half_rn(msg[kk] - pm);
      chain[kk] = __half2float(o);
      if (lvalid(kk)) {
        dstm[lane + 32 * kk] = o;
        if (SCALE) esum += __expf(chain[kk]);
      }
    }
    if (store_am) {
      const int64_t ao = c.out_off + qo;
      if (a.argmin_kind == BPL_ARGMIN_U8) {
        uint8_t* d = static_cast<uint8_t*>(a.argmin) + ao;
#pragma unroll
        for (int kk = 0; kk < K; ++kk)
          if (lvalid(kk)) d[lane + 32 * kk] = static_cast<uint8_t>(am[kk]);
      } else if (a.argmin_kind == BPL_ARGMIN_U16) {
        uint16_t* d = static_cast<uint16_t*>(a.argmin) + ao;
#pragma unroll
        for (int kk = 0; kk < K; ++kk)
          if (lvalid(kk)) d[lane + 32 * kk] = static_cast<uint16_t>(am[kk]);
      } else {
        float* d = static_cast<float*>(a.argmin) + ao;
#pragma unroll
        for (int kk = 0; kk < K; ++kk)
          if (lvalid(kk)) d[lane + 32 * kk] = static_cast<float>(am[kk]);
      }
    }
    if (SCALE) {
      esum = warp_sum(esum);
      if (lane == 0) scale_out[pq] = esum;
    }

    // next tap block
    if (j == 31 || i == nsteps - 1) {
      __syncwarp();
      if (32 * (b + 1) < nsteps) {
        store_taps(a, taps + ((b + 1) & 1) * tile_stride, lane, tr, true);
        if (32 * (b + 2) < nsteps) load_taps(a, c, b + 2, lane, nsteps, tr, true);
      }
    }
    __syncwarp();  // hs is rewritten by the next step
  };
  for (int i0 = 0; i0 < nsteps; i0 += PF) {
    static_for<PF>([&](auto SL) {
      constexpr int s = decltype(SL)::value;
      const int i = i0 + s;
      if (i < nsteps) step(SL, i);
    });
  }
}

// Launch of one phase: 4-warp blocks for a phase with few scanlines (the
// latency-bound horizontal sweeps at small batch), 1-warp blocks at high
// occupancy otherwise.
constexpr int kF16HiOcc = 17;

template <int K, bool SCALE>
int launch_f16_phase(const FwdArgs& a, cudaStream_t stream) {
  auto kern = lbp_forward_f16_kernel<K, 1, SCALE, 3>;
  int wpb = 4;
  if (a.nchains > kHiOccChainsPerSm * sm_count()) {
    kern = lbp_forward_f16_kernel<K, kF16HiOcc, SCALE, 1>;
    wpb = 1;
  }
  const size_t per_warp = 4 * static_cast<size_t>(align4(32 * K + 2 * kHsPad) + 2 * tap_tile_rows(a.Lv) * 33);
  const size_t smem = per_warp * wpb;
  if (smem > 48 * 1024)
    BPL_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)),
                 "cudaFuncSetAttribute");
  const int blocks = (a.nchains + wpb - 1) / wpb;
  kern<<<blocks, 32 * wpb, smem, stream>>>(a);
  BPL_CUDA_TRY(cudaGetLastError(), "lbp_forward_f16 launch");
  return BPL_OK;
}

template <int K>
int launch_f16_k(const FwdArgs& a0, cudaStream_t stream) {
  FwdArgs a = a0;
  for (int phase = 0; phase < 2; ++phase) {
    BPL_TRACE(phase == 0 ? "lbp_forward_f16: horizontal sweeps" : "lbp_forward_f16: vertical sweeps");
    a.phase = phase;
    a.nchains = 2 * a.B * (phase == 0 ? a.H : a.W);
    const int st = a.scale ? launch_f16_phase<K, true>(a, stream) : launch_f16_phase<K, false>(a, stream);
    if (st != BPL_OK) return st;
  }
  return BPL_OK;
}

inline int dispatch_f16(const FwdArgs& a, cudaStream_t s) {
  switch ((a.L + 31) / 32) {
    case 1: return launch_f16_k<1>(a, s);
    case 2: return launch_f16_k<2>(a, s);
    case 3: return launch_f16_k<3>(a, s);
    case 4: return launch_f16_k<4>(a, s);
    case 5: return launch_f16_k<5>(a, s);
    case 6: return launch_f16_k<6>(a, s);
    case 7: return launch_f16_k<7>(a, s);
    case 8: return launch_f16_k<8>(a, s);
    default: return set_error(BPL_ERR_UNSUPPORTED, "lbp_forward_f16: the lean kernel serves L <= 256");
  }
}

}  // namespace bpl

// Flow max-projected SAD for sm_103a.
//
// Reference: ops/flow_mp_sad/src/flow_mp_sad_kernel.cu
//   forward  :10-124  per pixel, a K x K window (K = sws+1, displacement
//            u, v in [-sws/2, sws/2] plus offsets) of channel-ordered SADs,
//            40 where the match is outside the image; then
//            cv_u[u] = min_v, u_star[u] = argmin_v + blockIdx_v*sws and
//            cv_v[v] = min_u, v_star[v] = argmin_u + blockIdx_u*sws,
//            strict `<` from 9999999 (first index wins ties); one block of
//            K threads per pixel (:231-245), K*K floats of shared memory
//   backward :126-200 routes in_grad_u / in_grad_v through the stored
//            argmins to df0 (local sum) and df1 (atomics), one thread per
//            (channel, pixel)
//
// GB300 design.
//
// Forward (FP32-issue bound: K*K*C abs-diff-adds per pixel).  A block owns
// 32 pixels of one row and every displacement u; it walks the window rows v
// in order.  For each row the f1 row segment the 32 windows touch is staged
// in shared memory, double-buffered, by one bulk copy per channel row behind
// an mbarrier (16-byte aligned rows) or by 4-byte cp.async, and each thread
// accumulates a 4 x 4 register tile of (pixel, u) SADs: per channel one
// 16-byte load of f0, two of f1 and 16 sub+abs-add pairs, channels summed in
// order (bit-identical SADs).  cv_u is a running minimum over the rows in
// registers (v ascending, strict <); cv_v is the minimum over u of the row:
// per thread over its 4 displacements, then over the warp by shuffles and
// over the warps through a shared table, each step on (value, index) as one
// 64-bit key that reproduces the first-index strict-< scan.  The window
// never sits in shared memory, so any K up to 256 fits.
//
// Backward.  The four (B,H,W,K) volumes are read once (the reference reads
// them once per channel).  One warp per pixel, lane = channel: for every
// window entry the warp reads the entry's argmin and gradient once, gathers
// the C channels of the matched f1 pixel from a channel-last copy of f1 (one
// coalesced 128-byte load) and adds into a channel-last df1 with one
// coalesced atomic per entry; df0 is the lane's running sum in the
// reference's entry order (bit-identical).  Two small transposes bring f1
// into and df1 out of channel-last layout.
#include <cuda_runtime.h>

#include <algorithm>

#include "bpl_device.cuh"
#include "bpl_internal.h"

namespace bpl {
namespace {

constexpr int kFTX = 32;      // pixels of a row per block
constexpr int kFCC = 32;      // channels per staged chunk
constexpr int kFMaxK = 256;   // window sizes served (8 * UCp threads <= 512)

struct FlowArgs {
  const float* f0;
  const float* f1;
  float* cv_u;
  float* cv_v;
  float* u_star;
  float* v_star;
  int B, C, H, W, sws, K, hs;
  int off_u, off_v, blk_u, blk_v;
  int UCp;   // groups of 4 displacements, rounded up to a multiple of 4 (one warp = 4 groups)
  int span;  // staged f1 row length in floats (4*UCp + 32)
};

// shared memory: f0 tile [C][32], two f1 stages [CC][span], cv_v keys of
// two rows [2][warps][32] (u64), two mbarriers
inline size_t flow_fwd_smem_bytes(int C, int span, int warps) {
  return sizeof(float) * (static_cast<size_t>(C) * kFTX + 2u * kFCC * span) + 2u * warps * kFTX * 8u + 2u * 8u;
}

// __byte_perm selectors that replace byte j of the first operand by byte 0
// of the second
__host__ __device__ constexpr unsigned byte_pick(int j) {
  return j == 0 ? 0x3214u : j == 1 ? 0x3240u : j == 2 ? 0x3410u : 0x4210u;
}

// (value, index) as one 64-bit key whose unsigned minimum is the smallest
// value and, among equal values, the smallest index: the result of the
// reference's ascending strict-< scan from (9999999, 0) when that start key
// takes part.  Window values are sums of |x| from +0 (or 40), so their bit
// patterns are non-negative floats, which order like unsigned integers, with
// NaN (positive after any float add) above +inf: a NaN never wins, as it
// never compares < in the scan.
__device__ __forceinline__ unsigned long long flow_key(float v, int idx) {
  return (static_cast<unsigned long long>(__float_as_uint(v)) << 32) | static_cast<unsigned>(idx);
}

// grid (ceil(W/32), H, B); block 8*UCp threads.  Thread (xc, uc): pixels
// x0 + 4xc .. +3, displacements 4uc .. +3; a warp holds xc = 0..7 for four
// consecutive uc, so its f0 loads are 8 distinct 16-byte chunks and its f1
// loads 11.  BULK: the staged rows start on a 16-byte boundary (W and
// off_u - hs multiples of 4) and come in by one bulk copy per channel row;
// otherwise by 4-byte cp.async.
template <bool BULK, int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB) flow_forward_kernel(FlowArgs a) {
  extern __shared__ __align__(16) float sm[];
  float* f0s = sm;                                              // [C][32]
  float* stg = f0s + a.C * kFTX;                                // [2][CC][span]
  const int tid = threadIdx.x, nt = blockDim.x, nw = nt >> 5;
  unsigned long long* keys = reinterpret_cast<unsigned long long*>(stg + 2 * kFCC * a.span);  // [2][nw][32]
  uint64_t* bars = reinterpret_cast<uint64_t*>(keys + 2 * nw * kFTX);                         // [2]
  const int lane = tid & 31;
  const int xc = lane & 7;
  const int uc = 4 * (tid >> 5) + (lane >> 3);
  const int n = blockIdx.z, y = blockIdx.y, x0 = blockIdx.x * kFTX;
  const int64_t HW = static_cast<int64_t>(a.H) * a.W;
  const float* f0 = a.f0 + static_cast<int64_t>(n) * a.C * HW + static_cast<int64_t>(y) * a.W;
  const float* f1 = a.f1 + static_cast<int64_t>(n) * a.C * HW;
  const unsigned long long key0 = flow_key(9999999.0f, 0);

  for (int i = tid; i < a.C * kFTX; i += nt) {
    const int c = i / kFTX, xx = i % kFTX;
    f0s[i] = (x0 + xx < a.W) ? __ldg(f0 + c * HW + x0 + xx) : 0.0f;
  }
  if (BULK && tid == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_mbar_init();
  }
  // window rows with a match inside the image: v = vi - hs <= hs and
  // 0 <= y + off_v + v < H
  const int vlo = max(0, a.hs - y - a.off_v);
  const int vhi = min(2 * a.hs, a.H - 1 - y - a.off_v + a.hs);
  const int nch = (a.C + kFCC - 1) / kFCC;
  const int nstage = (vhi >= vlo) ? (vhi - vlo + 1) * nch : 0;
  const int xs = x0 + a.off_u - a.hs;  // image column of staged index 0
  // the staged columns inside the image (BULK: whole 16-byte chunks)
  const int b_lo = max(0, -xs), b_hi = min(a.span, a.W - xs);

  auto issue = [&](int s) {
    const int vi = vlo + s / nch, ch = s % nch;
    const int64_t ym = y + a.off_v + vi - a.hs;
    const int c0 = ch * kFCC, cn = min(kFCC, a.C - c0);
    float* dst = stg + (s & 1) * kFCC * a.span;
    const float* src = f1 + c0 * HW + ym * a.W + xs;
    if (BULK) {
      if (tid == 0) {
        fence_proxy_async();
        const uint32_t rb = (b_hi > b_lo) ? static_cast<uint32_t>(b_hi - b_lo) * 4u : 0u;
        mbar_arrive_expect_tx(&bars[s & 1], rb * static_cast<uint32_t>(cn));
        if (rb)
          for (int c = 0; c < cn; ++c) bulk_g2s(dst + c * a.span + b_lo, src + c * HW + b_lo, rb, &bars[s & 1]);
      }
    } else {
      for (int c = 0; c < cn; ++c)
        for (int b = b_lo + tid; b < b_hi; b += nt) cp_async4(dst + c * a.span + b, src + c * HW + b);
      cp_async_commit();
    }
  };

  // running minimum over v of every (pixel i, displacement j) and its row,
  // one byte per displacement (K <= 256)
  float mn[4][4];
  unsigned amn[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    amn[i] = 0u;
#pragma unroll
    for (int j = 0; j < 4; ++j) mn[i][j] = 9999999.0f;
  }
  // matched column of (pixel i, displacement j): xs + 4(xc + uc) + i + j;
  // bit k of colok: column xs + 4(xc + uc) + k is inside the image
  unsigned colok = 0u;
#pragma unroll
  for (int k = 0; k < 7; ++k) {
    const int xm = xs + 4 * (xc + uc) + k;
    colok |= (xm >= 0 && xm < a.W) ? (1u << k) : 0u;
  }
  __syncthreads();  // f0s, keys, barriers
  if (nstage > 0) issue(0);
  bool failed = false;
  int s = 0;
  int s_stop = -1;  // the last stage waited for when a wait ran out
  for (int vi = 0; vi < a.K; ++vi) {
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = 0.0f;
    const bool row_ok = vi >= vlo && vi <= vhi;  // block-uniform
    if (row_ok) {
      for (int ch = 0; ch < nch; ++ch, ++s) {
        if (s + 1 < nstage) issue(s + 1);
        if (BULK) {
          if (!mbar_wait_bounded(&bars[s & 1], (s >> 1) & 1)) failed = true;
        } else {
          if (s + 1 < nstage) cp_async_wait<1>();
          else cp_async_wait<0>();
          __syncthreads();
        }
        const float* F1 = stg + (s & 1) * kFCC * a.span + 4 * (xc + uc);
        const float* F0 = f0s + ch * kFCC * kFTX + 4 * xc;
        const int cn = min(kFCC, a.C - ch * kFCC);
        if (cn == kFCC) {
#pragma unroll 8
          for (int c = 0; c < kFCC; ++c) {
            const float4 p = *reinterpret_cast<const float4*>(F0 + c * kFTX);
            const float4 q0 = *reinterpret_cast<const float4*>(F1 + c * a.span);
            const float4 q1 = *reinterpret_cast<const float4*>(F1 + c * a.span + 4);
            const float pa[4] = {p.x, p.y, p.z, p.w};
            const float qa[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
              for (int j = 0; j < 4; ++j) acc[i][j] += fabsf(pa[i] - qa[i + j]);
          }
        } else {
          for (int c = 0; c < cn; ++c) {
            const float4 p = *reinterpret_cast<const float4*>(F0 + c * kFTX);
            const float4 q0 = *reinterpret_cast<const float4*>(F1 + c * a.span);
            const float4 q1 = *reinterpret_cast<const float4*>(F1 + c * a.span + 4);
            const float pa[4] = {p.x, p.y, p.z, p.w};
            const float qa[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
              for (int j = 0; j < 4; ++j) acc[i][j] += fabsf(pa[i] - qa[i + j]);
          }
        }
        // buffer s & 1 is restaged by issue(s + 2), which the row's closing
        // barrier orders after this read for the row's last chunk; a wait
        // that ran out in any thread stops the block before it issues more
        if (ch + 1 < nch && __syncthreads_or(failed)) {
          failed = true;
          s_stop = s;
          break;
        }
      }
    }
    // window values (40 where the match is outside the image), the running
    // minimum over v, and this thread's minimum over its u of the row
    // keys of this row: written here, read after the barrier, rewritten two
    // rows later (after the next row's barrier)
    unsigned long long* kr = keys + (vi & 1) * nw * kFTX;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      float m = 9999999.0f;
      int am = 0;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float val = (row_ok && ((colok >> (i + j)) & 1u)) ? acc[i][j] : 40.0f;
        if (val < mn[i][j]) {
          mn[i][j] = val;
          amn[i] = __byte_perm(amn[i], static_cast<unsigned>(vi), byte_pick(j));
        }
        if (4 * uc + j < a.K && val < m) {
          m = val;
          am = 4 * uc + j;
        }
      }
      // the warp's four displacement groups of this pixel
      unsigned long long kmin = flow_key(m, am);
      kmin = min(kmin, __shfl_xor_sync(FULL, kmin, 8));
      kmin = min(kmin, __shfl_xor_sync(FULL, kmin, 16));
      if ((lane >> 3) == 0) kr[(tid >> 5) * kFTX + 4 * xc + i] = kmin;
    }
    // a timed-out wait stops the whole block
    if (__syncthreads_or(failed)) {
      if (s_stop < 0) s_stop = s - 1;  // the row's last chunk (s was advanced past it)
      failed = true;
      break;
    }
    if (tid < kFTX) {
      unsigned long long kv = key0;
      for (int w2 = 0; w2 < nw; ++w2) kv = min(kv, kr[w2 * kFTX + tid]);
      if (x0 + tid < a.W) {
        const int64_t o = ((static_cast<int64_t>(n) * a.H + y) * a.W + x0 + tid) * a.K + vi;
        a.cv_v[o] = __uint_as_float(static_cast<unsigned>(kv >> 32));
        a.v_star[o] = static_cast<float>(static_cast<int>(kv & 0xffffffffu) + a.blk_u * a.sws);
      }
    }
  }
  if (failed) {
    // the stage whose wait ran out and the one issued after it may still be
    // landing: each is the only phase of its barrier not yet observed, so
    // its parity identifies it.  Thread 0 (the issuer) waits for both
    // before the block, and its shared memory, goes away.
    if (BULK && tid == 0 && s_stop >= 0) {
      (void)mbar_wait_bounded(&bars[s_stop & 1], (s_stop >> 1) & 1, kDrainLimit);
      if (s_stop + 1 < nstage) (void)mbar_wait_bounded(&bars[(s_stop + 1) & 1], ((s_stop + 1) >> 1) & 1, kDrainLimit);
    }
    if (!BULK) cp_async_wait<0>();
    return;
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int x = x0 + 4 * xc + i;
    if (x >= a.W) continue;
    const int64_t o = ((static_cast<int64_t>(n) * a.H + y) * a.W + x) * a.K;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int ui = 4 * uc + j;
      if (ui < a.K) {
        a.cv_u[o + ui] = mn[i][j];
        a.u_star[o + ui] = static_cast<float>(static_cast<int>((amn[i] >> (8 * j)) & 0xffu) + a.blk_v * a.sws);
      }
    }
  }
}

// (B, C, P) <-> (B, P, C) transposes through a 32 x 33 tile.
// grid (ceil(P/32), ceil(C/32), B); block (32, 8)
template <bool TO_LAST>
__global__ void __launch_bounds__(256) channel_transpose_kernel(const float* __restrict__ in,
                                                                float* __restrict__ out, int C, int64_t P) {
  __shared__ float t[32][33];
  const int n = blockIdx.z;
  const int64_t p0 = static_cast<int64_t>(blockIdx.x) * 32;
  const int c0 = blockIdx.y * 32;
  const int tx = threadIdx.x;
  const int64_t base = static_cast<int64_t>(n) * C * P;
  for (int k = threadIdx.y; k < 32; k += 8) {
    if (TO_LAST) {  // read (c0 + k, p0 + tx)
      if (c0 + k < C && p0 + tx < P) t[k][tx] = in[base + (c0 + k) * P + p0 + tx];
    } else {  // read (p0 + k, c0 + tx)
      if (c0 + tx < C && p0 + k < P) t[k][tx] = in[base + (p0 + k) * C + c0 + tx];
    }
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += 8) {
    if (TO_LAST) {  // write (p0 + k, c0 + tx)
      if (c0 + tx < C && p0 + k < P) out[base + (p0 + k) * C + c0 + tx] = t[tx][k];
    } else {  // write (c0 + k, p0 + tx)
      if (c0 + k < C && p0 + tx < P) out[base + (c0 + k) * P + p0 + tx] = t[tx][k];
    }
  }
}

struct FlowBwdArgs {
  const float* f0;
  const float* f1t;  // (B, H*W, C)
  const float* gu;
  const float* gv;
  const float* us;
  const float* vs;
  float* df0;
  float* df1t;  // (B, H*W, C), zero-filled
  int B, C, H, W, sws, K, hs;
};

constexpr int kBwdPx = 8;      // pixels (warps) per block
constexpr int kBwdUnroll = 8;  // window entries gathered together

// grid (ceil(W/8), H, B); block 256: warp w = pixel x0 + w, lane = channel;
// registers capped for 4 resident blocks per SM (the gathers are
// latency-bound: more warps in flight).
// Offsets inside one batch item are 32-bit (H*W*C < 2^31, checked by the
// host).
__global__ void __launch_bounds__(256, 4) flow_backward_kernel(FlowBwdArgs a) {
  __shared__ float d0s[32][kBwdPx + 1];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int n = blockIdx.z, y = blockIdx.y, x0 = blockIdx.x * kBwdPx;
  const int x = x0 + w;
  const bool px = x < a.W;
  const int64_t HW = static_cast<int64_t>(a.H) * a.W;
  const int64_t o = ((static_cast<int64_t>(n) * a.H + y) * a.W + x) * a.K;
  const float* f1t = a.f1t + static_cast<int64_t>(n) * HW * a.C;
  float* d1t = a.df1t + static_cast<int64_t>(n) * HW * a.C;
  // entries u (or v) in [-hs, hs]: the last of K = sws + 1 entries is not
  // visited when sws is odd (:153, :176)
  const int nent = 2 * a.hs + 1;
  for (int cg = 0; cg < a.C; cg += 32) {
    const int c = cg + lane;
    const bool cok = c < a.C;
    const float a0 = (px && cok) ? __ldg(a.f0 + (static_cast<int64_t>(n) * a.C + c) * HW +
                                         static_cast<int64_t>(y) * a.W + x)
                                 : 0.0f;
    float g0 = 0.0f;
    if (px) {
      // u pass (entries of cv_u, v from u_star), then v pass: the
      // reference's order of the df0 sum
      for (int pass = 0; pass < 2; ++pass) {
        const float* star = pass ? a.vs : a.us;
        const float* gin = pass ? a.gv : a.gu;
        for (int e0 = 0; e0 < nent; e0 += 32) {
          // lane e: the matched pixel of entry e0 + e as a channel-row
          // offset (-1 outside the image) and the entry's gradient
          int tq = -1;
          float tg = 0.0f;
          {
            const int e = e0 + lane;
            if (e < nent) {
              // the stored index is converted to short as in the reference (:156, :179)
              const int si = static_cast<int>(static_cast<short>(__ldg(star + o + e))) - a.hs;
              const int i = e - a.hs;
              const int u = pass ? si : i;
              const int v = pass ? i : si;
              if (x + u >= 0 && x + u < a.W && y + v >= 0 && y + v < a.H) tq = ((y + v) * a.W + x + u) * a.C;
              tg = __ldg(gin + o + e);
            }
          }
          const int ne = min(32, nent - e0);
          // groups of kBwdUnroll entries: the f1 gathers of a group are in
          // flight together, the updates then follow in entry order
          for (int k0 = 0; k0 < ne; k0 += kBwdUnroll) {
            float fv[kBwdUnroll], gg[kBwdUnroll];
            int qv[kBwdUnroll];
#pragma unroll
            for (int t = 0; t < kBwdUnroll; ++t) {
              const int k = (k0 + t) & 31;  // k0 + t >= ne is masked below
              qv[t] = __shfl_sync(FULL, tq, k);
              gg[t] = __shfl_sync(FULL, tg, k);
              fv[t] = (cok && qv[t] >= 0 && k0 + t < ne) ? __ldg(f1t + qv[t] + c) : 0.0f;
            }
#pragma unroll
            for (int t = 0; t < kBwdUnroll; ++t) {
              const float diff = a0 - fv[t];
              if (cok && qv[t] >= 0 && k0 + t < ne && fabsf(diff) > 1e-15f) {
                // diff / |diff| is exactly +-1 for finite diff and NaN for an
                // infinite one, so the reference's update (diff/|diff|) * g is
                const float sgn = (fabsf(diff) == __int_as_float(0x7f800000))
                                      ? __int_as_float(0x7fffffff)
                                      : (diff > 0.0f ? 1.0f : -1.0f);
                const float upd = sgn * gg[t];
                g0 += upd;
                atomicAdd(d1t + qv[t] + c, -upd);
              }
            }
          }
        }
      }
    }
    // df0 through shared memory: 8 consecutive pixels per channel row
    d0s[lane][w] = g0;
    __syncthreads();
    {
      const int cc = threadIdx.x / kBwdPx, ww = threadIdx.x % kBwdPx;
      const int ch = cg + cc;
      if (ch < a.C && x0 + ww < a.W)
        a.df0[(static_cast<int64_t>(n) * a.C + ch) * HW + static_cast<int64_t>(y) * a.W + x0 + ww] = d0s[cc][ww];
    }
    __syncthreads();
  }
}

int flow_ups(int K) {
  const int uc = (K + 3) / 4;
  return (uc + 3) / 4 * 4;
}

}  // namespace
}  // namespace bpl

using namespace bpl;

extern "C" int bpl_flow_forward(const float* f0, const float* f1, float* cv_u, float* cv_v, float* u_star,
                                float* v_star, int B, int C, int H, int W, int sws, int offset_u, int offset_v,
                                int block_u, int block_v, void* stream) {
  BPL_TRACE("bpl_flow_forward");
  BPL_REQUIRE(f0 && f1 && cv_u && cv_v && u_star && v_star, "flow_forward: null pointer");
  BPL_REQUIRE(B >= 1 && C >= 1 && H >= 1 && W >= 1, "flow_forward: bad shape");
  BPL_REQUIRE(B <= 65535 && H <= 65535, "flow_forward: B and H must be <= 65535");
  BPL_REQUIRE(sws >= 0 && sws + 1 <= kFMaxK, "flow_forward: window size %d outside [1, %d]", sws + 1, kFMaxK);
  const int K = sws + 1;
  const int UCp = flow_ups(K);
  const int span = 4 * UCp + kFTX;
  FlowArgs a{f0, f1, cv_u, cv_v, u_star, v_star, B, C, H, W, sws, K, sws / 2,
             offset_u, offset_v, block_u, block_v, UCp, span};
  const size_t smem = flow_fwd_smem_bytes(C, span, 8 * UCp / 32);
  BPL_REQUIRE(smem <= static_cast<size_t>(max_smem_optin()),
              "flow_forward: %d channels need %zu bytes of shared memory", C, smem);
  // bulk row copies need 16-byte aligned rows and staged starts
  const bool bulk = (W % 4 == 0) && ((((offset_u - sws / 2) % 4) + 4) % 4 == 0) &&
                    (reinterpret_cast<uintptr_t>(f1) % 16 == 0);
  auto launch = [&](auto kern) -> int {
    if (smem > 48 * 1024)
      BPL_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)),
                   "cudaFuncSetAttribute");
    dim3 grid((W + kFTX - 1) / kFTX, H, B);
    kern<<<grid, 8 * UCp, smem, as_stream(stream)>>>(a);
    BPL_CUDA_TRY(cudaGetLastError(), "flow_forward launch");
    return BPL_OK;
  };
  // up to 160 threads (K <= 80): four blocks per SM, registers capped for it
  if (8 * UCp <= 160)
    return bulk ? launch(flow_forward_kernel<true, 160, 4>) : launch(flow_forward_kernel<false, 160, 4>);
  return bulk ? launch(flow_forward_kernel<true, 512, 1>) : launch(flow_forward_kernel<false, 512, 1>);
}

extern "C" size_t bpl_flow_backward_workspace_size(int B, int C, int H, int W) {
  if (B < 1 || C < 1 || H < 1 || W < 1) return 0;
  return 2 * sizeof(float) * static_cast<size_t>(B) * C * H * W;
}

extern "C" int bpl_flow_backward_ws(const float* f0, const float* f1, const float* in_grad_u,
                                    const float* in_grad_v, const float* u_star, const float* v_star, float* df0,
                                    float* df1, void* workspace, size_t workspace_bytes, int B, int C, int H, int W,
                                    int sws, void* stream) {
  BPL_TRACE("bpl_flow_backward_ws");
  BPL_REQUIRE(f0 && f1 && in_grad_u && in_grad_v && u_star && v_star && df0 && df1 && workspace,
              "flow_backward: null pointer");
  BPL_REQUIRE(B >= 1 && C >= 1 && H >= 1 && W >= 1 && sws >= 0, "flow_backward: bad shape");
  BPL_REQUIRE(B <= 65535 && H <= 65535 && C <= 65535 * 32, "flow_backward: B, H or C too large");
  BPL_REQUIRE(static_cast<int64_t>(H) * W * C < (int64_t{1} << 31), "flow_backward: H*W*C must be < 2^31");
  const size_t need = bpl_flow_backward_workspace_size(B, C, H, W);
  BPL_REQUIRE(workspace_bytes >= need, "flow_backward: workspace of %zu bytes, %zu needed", workspace_bytes, need);
  BPL_REQUIRE(reinterpret_cast<uintptr_t>(workspace) % 16 == 0, "flow_backward: workspace not 16-byte aligned");
  cudaStream_t st = as_stream(stream);
  const int64_t P = static_cast<int64_t>(H) * W;
  const size_t nel = static_cast<size_t>(B) * C * P;
  float* f1t = static_cast<float*>(workspace);
  float* d1t = f1t + nel;
  BPL_CUDA_TRY(cudaMemsetAsync(d1t, 0, sizeof(float) * nel, st), "flow_backward: memset");
  const dim3 tgrid(static_cast<unsigned>((P + 31) / 32), (C + 31) / 32, B);
  channel_transpose_kernel<true><<<tgrid, dim3(32, 8), 0, st>>>(f1, f1t, C, P);
  BPL_CUDA_TRY(cudaGetLastError(), "flow_backward transpose launch");
  FlowBwdArgs a{f0, f1t, in_grad_u, in_grad_v, u_star, v_star, df0, d1t, B, C, H, W, sws, sws + 1, sws / 2};
  dim3 grid((W + kBwdPx - 1) / kBwdPx, H, B);
  flow_backward_kernel<<<grid, 32 * kBwdPx, 0, st>>>(a);
  BPL_CUDA_TRY(cudaGetLastError(), "flow_backward launch");
  channel_transpose_kernel<false><<<tgrid, dim3(32, 8), 0, st>>>(d1t, df1, C, P);
  BPL_CUDA_TRY(cudaGetLastError(), "flow_backward transpose launch");
  return BPL_OK;
}

extern "C" int bpl_flow_backward(const float* f0, const float* f1, const float* in_grad_u, const float* in_grad_v,
                                 const float* u_star, const float* v_star, float* df0, float* df1, int B, int C,
                                 int H, int W, int sws, void* stream) {
  BPL_TRACE("bpl_flow_backward");
  BPL_REQUIRE(B >= 1 && C >= 1 && H >= 1 && W >= 1 && sws >= 0, "flow_backward: bad shape");
  cudaStream_t st = as_stream(stream);
  const size_t ws = bpl_flow_backward_workspace_size(B, C, H, W);
  void* p = nullptr;
  BPL_CUDA_TRY(cudaMallocAsync(&p, ws, st), "flow_backward: workspace allocation");
  const int rc = bpl_flow_backward_ws(f0, f1, in_grad_u, in_grad_v, u_star, v_star, df0, df1, p, ws, B, C, H, W,
                                      sws, stream);
  const cudaError_t fe = cudaFreeAsync(p, st);
  if (rc != BPL_OK) return rc;
  BPL_CUDA_TRY(fe, "flow_backward: workspace release");
  return BPL_OK;
}

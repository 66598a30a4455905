// Epilogue kernels on either side of the BP passes: the cost volume from a
// SAD volume, the per-pixel disparity from the messages, and the inference
// modes on a belief volume.  Each replaces a chain of full-volume torch
// passes with one memory-bound pass (one warp per pixel, labels spread over
// the lanes, label = lane + 32k, coalesced 128-byte row segments).
//
// Reference semantics:
//   cost = -softmax(-SAD / T)      matching.py:22-25, message_passing_op_cuda.py:162
//   disparity = argmin_t ((((M0 + M1) + M2) + M3) + cost)[t], first index:
//       the argmax of the beliefs softmin(...) (message_passing_op_cuda.py:
//       170-173, inference_op.py:23-27) except where the softmin's rounding
//       ties two labels
//   wta / sub-exp on beliefs         inference_op.py:22-27, :53-97
#include <cuda_fp16.h>
#include <algorithm>
#include <cuda_runtime.h>

#include "bpl_device.cuh"
#include "bpl_internal.h"

namespace bpl {
namespace {

constexpr int kEpiWarps = 8;  // warps (pixels) per block

template <typename T>
__device__ __forceinline__ float ld_as_float(const T* p);
template <>
__device__ __forceinline__ float ld_as_float<float>(const float* p) { return __ldg(p); }
template <>
__device__ __forceinline__ float ld_as_float<__half>(const __half* p) { return __half2float(__ldg(p)); }

// (value, label) minimum with the smallest label among equal values: one
// 64-bit key per lane, reduced by shuffles (redux has no 64-bit form)
__device__ __forceinline__ unsigned long long min_key(float v, int t) {
  return (static_cast<unsigned long long>(f2ord(v)) << 32) | static_cast<unsigned>(t);
}
__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long k) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_xor_sync(FULL, k, o);
    k = x < k ? x : k;
  }
  return k;
}

// cost (B,H,W,Ls) = -softmax_t(-sad[t] / T), labels >= D of a padded row set
// to zero.  exp(x - max) by expf, the sum in any order.
template <typename TO>
__global__ void __launch_bounds__(32 * kEpiWarps) cost_from_sad_kernel(const float* __restrict__ sad, TO* __restrict__ cost,
                                                                       int64_t npix, int D, int Ls, float inv_t) {
  const int lane = threadIdx.x & 31;
  const int64_t pix = static_cast<int64_t>(blockIdx.x) * kEpiWarps + (threadIdx.x >> 5);
  if (pix >= npix) return;
  const float* row = sad + pix * D;
  TO* out = cost + pix * Ls;
  float mn = __int_as_float(0x7f800000);
  for (int t = lane; t < D; t += 32) mn = fminf(mn, __ldg(row + t));
  mn = warp_min_redux(mn);
  float s = 0.0f;
  for (int t = lane; t < D; t += 32) s += expf((mn - __ldg(row + t)) * inv_t);
  s = warp_sum(s);
  const float inv_s = 1.0f / s;
  for (int t = lane; t < Ls; t += 32) {
    const float v = (t < D) ? -(expf((mn - __ldg(row + t)) * inv_t) * inv_s) : 0.0f;
    if constexpr (sizeof(TO) == 2) out[t] = __float2half_rn(v);
    else out[t] = v;
  }
}

// disparity (B,H,W) = argmin_t ((((M0+M1)+M2)+M3)+cost)[t], first index
template <typename TM, typename TC, typename TO>
__global__ void __launch_bounds__(32 * kEpiWarps) messages_argmin_kernel(const TM* __restrict__ msgs, const TC* __restrict__ cost,
                                                                         TO* __restrict__ out, int64_t HW, int64_t npix,
                                                                         int L, int Ls, int Lc) {
  const int lane = threadIdx.x & 31;
  const int64_t pix = static_cast<int64_t>(blockIdx.x) * kEpiWarps + (threadIdx.x >> 5);
  if (pix >= npix) return;
  const int64_t n = pix / HW, p = pix % HW;
  const TM* m0 = msgs + (n * 4 * HW + p) * Ls;
  const int64_t slot = HW * Ls;
  const TC* c = cost + pix * Lc;
  unsigned long long best = ~0ull;
  for (int t = lane; t < L; t += 32) {
    const float z = (((ld_as_float(m0 + t) + ld_as_float(m0 + slot + t)) + ld_as_float(m0 + 2 * slot + t)) +
                     ld_as_float(m0 + 3 * slot + t)) +
                    ld_as_float(c + t);
    const unsigned long long k = min_key(z, t);
    best = k < best ? k : best;
  }
  best = warp_min_u64(best);
  if (lane == 0) out[pix] = static_cast<TO>(best & 0xffffffffu);
}

// wta: argmax_t beliefs[t] (first index, as torch.argmax); sub-exp: the
// expectation of the label over the argmax's +-support window, clamped to
// [0, L-1] (repeated labels at the border count repeatedly), renormalised
template <bool SUBEXP>
__global__ void __launch_bounds__(32 * kEpiWarps) beliefs_infer_kernel(const float* __restrict__ beliefs,
                                                                       void* __restrict__ out, int64_t npix, int L,
                                                                       int support) {
  const int lane = threadIdx.x & 31;
  const int64_t pix = static_cast<int64_t>(blockIdx.x) * kEpiWarps + (threadIdx.x >> 5);
  if (pix >= npix) return;
  const float* b = beliefs + pix * L;
  // argmax with the first index: minimum of (-value) keys
  unsigned long long best = ~0ull;
  for (int t = lane; t < L; t += 32) {
    const unsigned long long k = min_key(-__ldg(b + t), t);
    best = k < best ? k : best;
  }
  best = warp_min_u64(best);
  const int d = static_cast<int>(best & 0xffffffffu);
  if (!SUBEXP) {
    if (lane == 0) static_cast<int64_t*>(out)[pix] = d;
    return;
  }
  // window entries on lanes 0 .. 2*support
  const int ws = 2 * support + 1;
  float v = 0.0f, lab = 0.0f;
  if (lane < ws) {
    const int t = min(max(d + lane - support, 0), L - 1);
    v = __ldg(b + t);
    lab = static_cast<float>(t);
  }
  const float s = warp_sum(v);
  const float e = warp_sum((v / s) * lab);
  if (lane == 0) static_cast<float*>(out)[pix] = e;
}

inline unsigned blocks_for(int64_t npix) { return static_cast<unsigned>((npix + kEpiWarps - 1) / kEpiWarps); }

// Stereo jump taps from affinities (message_passing_op_cuda.py:35-60): for
// K affinities [.., L3] per direction and Kp = K + 3 taps,
//   tap 0 = offset, taps 1 and Kp-1 = the last affinity (L3), tap Kp/2 = 0,
//   tap i in [2, Kp/2): affinity 2(i-2) on directions 0, 2 (LR, UD) and
//   2(i-2)+1 on directions 1, 3 (RL, DU); tap Kp-i: the other one of the pair.
// Returns the affinity index of tap i of direction d, -1 for the offset,
// -2 for the zero centre tap.
__device__ __forceinline__ int tap_source(int i, int d, int K) {
  const int Kp = K + 3, c = Kp / 2;
  if (i == 0) return -1;
  if (i == c) return -2;
  if (i == 1 || i == Kp - 1) return K - 1;
  const bool mirror = i > c;
  const int m = mirror ? Kp - i - 2 : i - 2;
  const bool first = mirror == ((d & 1) != 0);  // LR/UD: i takes the pair's first, Kp-i its second
  return 2 * m + (first ? 0 : 1);
}

// one thread per (n, d, pixel): taps[n,d,:,p] from aff[n,d,:,p] and offset[n,d,p]
__global__ void pack_taps_kernel(const float* __restrict__ aff, const float* __restrict__ off, float* __restrict__ taps,
                                 int N, int K, int64_t HW) {
  const int64_t total = static_cast<int64_t>(N) * 4 * HW;
  const int Kp = K + 3;
  for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < total;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t nd = e / HW, p = e % HW;
    const int d = static_cast<int>(nd & 3);
    const float* a = aff + nd * K * HW + p;
    float* t = taps + nd * Kp * HW + p;
    for (int i = 0; i < Kp; ++i) {
      const int src = tap_source(i, d, K);
      t[i * HW] = (src == -1) ? __ldg(off + e) : (src == -2 ? 0.0f : __ldg(a + src * HW));
    }
  }
}

// the fold of the tap gradient (message_passing_op_cuda.py:75-93): each
// affinity sums the gradients of the taps it fills (L3: taps 1 and Kp-1,
// added in that order), the offset takes tap 0, the centre tap is dropped
__global__ void unpack_tap_grad_kernel(const float* __restrict__ gtaps, float* __restrict__ gaff,
                                       float* __restrict__ goff, int N, int K, int64_t HW) {
  const int64_t total = static_cast<int64_t>(N) * 4 * HW;
  const int Kp = K + 3;
  for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < total;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t nd = e / HW, p = e % HW;
    const int d = static_cast<int>(nd & 3);
    const float* g = gtaps + nd * Kp * HW + p;
    float* a = gaff + nd * K * HW + p;
    for (int k = 0; k < K - 1; ++k) a[k * HW] = 0.0f;
    a[(K - 1) * HW] = (0.0f + __ldg(g + HW)) + __ldg(g + (Kp - 1) * HW);
    for (int i = 2; i < Kp - 1; ++i) {
      const int src = tap_source(i, d, K);
      if (src >= 0 && src != K - 1) a[src * HW] = __ldg(g + i * HW);
    }
    goff[e] = __ldg(g);
  }
}

// dst (rows, Ls) half = sign * src (rows, L) float, padding labels zeroed:
// the FP16-storage cost volume straight from the layer's probability volume
// (cost = -prob), one pass.  One thread per label pair (Ls is even).
__global__ void half_padded_kernel(const float* __restrict__ src, float sign, __half2* __restrict__ dst, int64_t rows,
                                   int L, int Ls) {
  const int hp = Ls / 2;
  const int64_t total = rows * hp;
  for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < total;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t r = e / hp;
    const int t = 2 * static_cast<int>(e % hp);
    const float* s = src + r * L;
    const float a = (t < L) ? sign * __ldg(s + t) : 0.0f;
    const float b = (t + 1 < L) ? sign * __ldg(s + t + 1) : 0.0f;
    dst[e] = __floats2half2_rn(a, b);
  }
}

}  // namespace
}  // namespace bpl

using namespace bpl;

extern "C" int bpl_half_padded(const float* src, float sign, void* dst, int64_t rows, int L, int Ls, void* stream) {
  BPL_TRACE("bpl_half_padded");
  BPL_REQUIRE(src && dst, "half_padded: null pointer");
  BPL_REQUIRE(rows >= 1 && L >= 1 && Ls == ((L + 7) & ~7), "half_padded: bad shape (rows %lld, L %d, Ls %d)",
              static_cast<long long>(rows), L, Ls);
  BPL_REQUIRE(sign == 1.0f || sign == -1.0f, "half_padded: sign must be +-1");
  BPL_REQUIRE(reinterpret_cast<uintptr_t>(dst) % 4 == 0, "half_padded: dst must be 4-byte aligned");
  const int64_t total = rows * (Ls / 2);
  const unsigned blocks = static_cast<unsigned>(std::min<int64_t>((total + 255) / 256, 152 * 16));
  half_padded_kernel<<<blocks, 256, 0, as_stream(stream)>>>(src, sign, static_cast<__half2*>(dst), rows, L, Ls);
  BPL_CUDA_TRY(cudaGetLastError(), "half_padded launch");
  return BPL_OK;
}

extern "C" int bpl_cost_from_sad(const float* sad, void* cost, int cost_half, int B, int H, int W, int D, int Ls,
                                 float temperature, void* stream) {
  BPL_TRACE("bpl_cost_from_sad");
  BPL_REQUIRE(sad && cost, "cost_from_sad: null pointer");
  BPL_REQUIRE(B >= 1 && H >= 1 && W >= 1 && D >= 1 && Ls >= D, "cost_from_sad: bad shape");
  BPL_REQUIRE(temperature > 0.0f, "cost_from_sad: temperature must be positive");
  const int64_t npix = static_cast<int64_t>(B) * H * W;
  if (cost_half)
    cost_from_sad_kernel<__half><<<blocks_for(npix), 32 * kEpiWarps, 0, as_stream(stream)>>>(
        sad, static_cast<__half*>(cost), npix, D, Ls, 1.0f / temperature);
  else
    cost_from_sad_kernel<float><<<blocks_for(npix), 32 * kEpiWarps, 0, as_stream(stream)>>>(
        sad, static_cast<float*>(cost), npix, D, Ls, 1.0f / temperature);
  BPL_CUDA_TRY(cudaGetLastError(), "cost_from_sad launch");
  return BPL_OK;
}

extern "C" int bpl_messages_argmin(const void* messages, int messages_half, const void* cost, int cost_half,
                                   void* disparity, int disparity_int64, int B, int H, int W, int L, int Ls, int Lc,
                                   void* stream) {
  BPL_TRACE("bpl_messages_argmin");
  BPL_REQUIRE(messages && cost && disparity, "messages_argmin: null pointer");
  BPL_REQUIRE(B >= 1 && H >= 1 && W >= 1 && L >= 1 && Ls >= L && Lc >= L, "messages_argmin: bad shape");
  const int64_t HW = static_cast<int64_t>(H) * W, npix = B * HW;
  const dim3 g(blocks_for(npix)), blk(32 * kEpiWarps);
  cudaStream_t s = as_stream(stream);
  auto go = [&](auto tm, auto tc) {
    using TM = decltype(tm);
    using TC = decltype(tc);
    if (disparity_int64)
      messages_argmin_kernel<TM, TC, int64_t><<<g, blk, 0, s>>>(static_cast<const TM*>(messages),
                                                                 static_cast<const TC*>(cost),
                                                                 static_cast<int64_t*>(disparity), HW, npix, L, Ls, Lc);
    else
      messages_argmin_kernel<TM, TC, int32_t><<<g, blk, 0, s>>>(static_cast<const TM*>(messages),
                                                                 static_cast<const TC*>(cost),
                                                                 static_cast<int32_t*>(disparity), HW, npix, L, Ls, Lc);
  };
  if (messages_half) {
    if (cost_half) go(__half(), __half());
    else go(__half(), 0.0f);
  } else {
    if (cost_half) go(0.0f, __half());
    else go(0.0f, 0.0f);
  }
  BPL_CUDA_TRY(cudaGetLastError(), "messages_argmin launch");
  return BPL_OK;
}

extern "C" int bpl_beliefs_infer(const float* beliefs, int mode, int support, void* out, int B, int H, int W, int L,
                                 void* stream) {
  BPL_TRACE("bpl_beliefs_infer");
  BPL_REQUIRE(beliefs && out, "beliefs_infer: null pointer");
  BPL_REQUIRE(B >= 1 && H >= 1 && W >= 1 && L >= 1, "beliefs_infer: bad shape");
  BPL_REQUIRE(mode == 0 || mode == 1, "beliefs_infer: mode must be 0 (wta) or 1 (sub-exp)");
  BPL_REQUIRE(mode == 0 || (support >= 0 && 2 * support + 1 <= 32), "beliefs_infer: support must be 0..15");
  const int64_t npix = static_cast<int64_t>(B) * H * W;
  if (mode == 0)
    beliefs_infer_kernel<false><<<blocks_for(npix), 32 * kEpiWarps, 0, as_stream(stream)>>>(beliefs, out, npix, L, support);
  else
    beliefs_infer_kernel<true><<<blocks_for(npix), 32 * kEpiWarps, 0, as_stream(stream)>>>(beliefs, out, npix, L, support);
  BPL_CUDA_TRY(cudaGetLastError(), "beliefs_infer launch");
  return BPL_OK;
}

extern "C" int bpl_pack_taps(const float* affinities, const float* offset, float* taps, int N, int K, int H, int W,
                             void* stream) {
  BPL_TRACE("bpl_pack_taps");
  BPL_REQUIRE(affinities && offset && taps, "pack_taps: null pointer");
  BPL_REQUIRE(N >= 1 && H >= 1 && W >= 1, "pack_taps: bad shape");
  BPL_REQUIRE(K >= 3 && K % 2 == 1 && K + 3 <= 16, "pack_taps: K=%d affinities (odd, 3..13) expected", K);
  const int64_t HW = static_cast<int64_t>(H) * W, total = static_cast<int64_t>(N) * 4 * HW;
  const unsigned blocks = static_cast<unsigned>(std::min<int64_t>((total + 255) / 256, 152 * 16));
  pack_taps_kernel<<<blocks, 256, 0, as_stream(stream)>>>(affinities, offset, taps, N, K, HW);
  BPL_CUDA_TRY(cudaGetLastError(), "pack_taps launch");
  return BPL_OK;
}

extern "C" int bpl_unpack_tap_grad(const float* grad_taps, float* grad_affinities, float* grad_offset, int N, int K,
                                   int H, int W, void* stream) {
  BPL_TRACE("bpl_unpack_tap_grad");
  BPL_REQUIRE(grad_taps && grad_affinities && grad_offset, "unpack_tap_grad: null pointer");
  BPL_REQUIRE(N >= 1 && H >= 1 && W >= 1, "unpack_tap_grad: bad shape");
  BPL_REQUIRE(K >= 3 && K % 2 == 1 && K + 3 <= 16, "unpack_tap_grad: K=%d affinities (odd, 3..13) expected", K);
  const int64_t HW = static_cast<int64_t>(H) * W, total = static_cast<int64_t>(N) * 4 * HW;
  const unsigned blocks = static_cast<unsigned>(std::min<int64_t>((total + 255) / 256, 152 * 16));
  unpack_tap_grad_kernel<<<blocks, 256, 0, as_stream(stream)>>>(grad_taps, grad_affinities, grad_offset, N, K, HW);
  BPL_CUDA_TRY(cudaGetLastError(), "unpack_tap_grad launch");
  return BPL_OK;
}

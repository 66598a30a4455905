// Fused belief epilogue of the BP layer:
//   beliefs = softmin(((((M0 + M1) + M2) + M3) + cost) / T)   over labels
// (the reference computes messages.sum(dim=1) + cost and then
// TemperatureSoftmin as separate torch passes:
// ops/lbp_stereo/message_passing_op_cuda.py:170-173, corenet.py:106-113),
// and its backward: the gradient of z = sum + cost (which is also every
// message slot's gradient) and of the temperature.
//
// One warp per pixel, labels lane + 32k, grid-stride over pixels.  HBM-bound
// streaming: the forward reads the 4 message slots and the cost once and
// writes the beliefs; the backward recomputes z from the same inputs, reads
// the beliefs and their gradient and writes the gradient of z.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "bpl_device.cuh"
#include "bpl_internal.h"

namespace bpl {
namespace {

template <typename T>
__device__ __forceinline__ float tof(T v);
template <>
__device__ __forceinline__ float tof<float>(float v) { return v; }
template <>
__device__ __forceinline__ float tof<__half>(__half v) { return __half2float(v); }

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(FULL, v, o));
  return v;
}

// z / T for the labels of one pixel (K per lane); invalid labels -> +inf.
// The cost is float (label stride L) or the FP16-storage half volume (label
// stride Ls), taken times csign (+1; -1 reads the probability volume the
// layer's cost is the negation of, exactly: negation is exact).
template <int K, typename T, typename TC>
__device__ __forceinline__ void load_z(const T* msgs, const TC* cost, float csign, int64_t pix, int64_t HWLs, int Ls,
                                       int L, int n, int64_t HW, float Tm, int lane, float (&zt)[K]) {
  const int64_t p = pix % HW;
  const T* m = msgs + (static_cast<int64_t>(n) * 4) * HWLs + p * Ls;
  const TC* c = cost + pix * (sizeof(TC) == 4 ? L : Ls);
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const int t = lane + 32 * k;
    if (t < L) {
      const float s = __fadd_rn(__fadd_rn(__fadd_rn(tof<T>(m[t]), tof<T>(m[HWLs + t])), tof<T>(m[2 * HWLs + t])),
                                tof<T>(m[3 * HWLs + t]));
      zt[k] = __fdiv_rn(__fadd_rn(s, csign * tof<TC>(c[t])), Tm);
    } else {
      zt[k] = __int_as_float(0x7f800000);
    }
  }
}

// lnorm (B,H,W), may be null: per pixel c = min(z/T) - log(sum), with which
// the backward recovers z/T = c - log(beliefs) without re-reading messages
// and cost.
template <int K, typename T, typename TC>
__global__ void __launch_bounds__(256) beliefs_fwd_kernel(const T* msgs, const TC* cost, float csign, const float* Tp,
                                                          float* out, float* lnorm, int B, int H, int W, int L,
                                                          int Ls) {
  const int lane = threadIdx.x & 31;
  const int64_t HW = static_cast<int64_t>(H) * W;
  const int64_t npix = B * HW;
  const int64_t HWLs = HW * Ls;
  const int64_t warps = static_cast<int64_t>(gridDim.x) * (blockDim.x >> 5);
  const float Tm = __ldg(Tp);
  for (int64_t pix = blockIdx.x * static_cast<int64_t>(blockDim.x >> 5) + (threadIdx.x >> 5); pix < npix;
       pix += warps) {
    const int n = static_cast<int>(pix / HW);
    float zt[K];
    load_z<K, T, TC>(msgs, cost, csign, pix, HWLs, Ls, L, n, HW, Tm, lane, zt);
    // softmin(x) = softmax(-x): shift by the minimum of x
    float mn = zt[0];
#pragma unroll
    for (int k = 1; k < K; ++k) mn = fminf(mn, zt[k]);
    mn = -warp_max(-mn);
    float e[K], s = 0.0f;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      e[k] = (lane + 32 * k < L) ? expf(mn - zt[k]) : 0.0f;
      s += e[k];
    }
    s = warp_sum(s);
    const float inv = 1.0f / s;
    if (lnorm != nullptr && lane == 0) lnorm[pix] = mn - logf(s);
    float* o = out + pix * L;
#pragma unroll
    for (int k = 0; k < K; ++k)
      if (lane + 32 * k < L) o[lane + 32 * k] = e[k] * inv;
  }
}

// Gradient outputs: gz (B,H,W,L) float receives gz_sign * dL/dz; `copy`, by
// copy_kind, a second copy of +dL/dz: kCopyHalf (B,H,W,Ls) half with the
// padding zeroed, kCopySlots (B,4,H,W,L) float in every message slot,
// kCopyFloat (B,H,W,L) float.  The temperature's gradient needs z / T:
// from lnorm (the forward's c) as c - log(beliefs) when given (a label whose
// belief is 0 has du = 0 and adds nothing; labels of tiny beliefs, where the
// log is coarse, add du * z / T with du of their size), else recomputed from
// messages and cost.
enum { kCopyNone = 0, kCopyHalf = 1, kCopySlots = 2, kCopyFloat = 3 };

template <int K, typename T, typename TC>
__global__ void __launch_bounds__(256) beliefs_bwd_kernel(const T* msgs, const TC* cost, float csign, const float* Tp,
                                                          const float* y, const float* gy, float* gz, float gz_sign,
                                                          void* copy, int copy_kind, float* gT, const float* lnorm,
                                                          int B, int H, int W, int L, int Ls) {
  const int lane = threadIdx.x & 31;
  const int64_t HW = static_cast<int64_t>(H) * W;
  const int64_t npix = B * HW;
  const int64_t HWLs = HW * Ls;
  const int64_t warps = static_cast<int64_t>(gridDim.x) * (blockDim.x >> 5);
  const float Tm = __ldg(Tp);
  float tacc = 0.0f;
  for (int64_t pix = blockIdx.x * static_cast<int64_t>(blockDim.x >> 5) + (threadIdx.x >> 5); pix < npix;
       pix += warps) {
    const int n = static_cast<int>(pix / HW);
    float zt[K];
    if (gT != nullptr && lnorm == nullptr) load_z<K, T, TC>(msgs, cost, csign, pix, HWLs, Ls, L, n, HW, Tm, lane, zt);
    const float* yp = y + pix * L;
    const float* gp = gy + pix * L;
    float yv[K], gv[K], d = 0.0f;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int t = lane + 32 * k;
      yv[k] = (t < L) ? yp[t] : 0.0f;
      gv[k] = (t < L) ? gp[t] : 0.0f;
      d += yv[k] * gv[k];
    }
    d = warp_sum(d);
    if (gT != nullptr && lnorm != nullptr) {
      const float c = __ldg(lnorm + pix);
#pragma unroll
      for (int k = 0; k < K; ++k) zt[k] = (yv[k] > 0.0f) ? c - logf(yv[k]) : 0.0f;
    }
    float* o = gz + pix * L;
    const int64_t p = pix % HW;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int t = lane + 32 * k;
      // u = -z/T: du = y (g - sum(y g)); dz = -du / T; dT += du * z / T^2
      const float du = yv[k] * (gv[k] - d);
      const float g = -du / Tm;
      if (t < L) {
        o[t] = gz_sign * g;
        if (gT != nullptr) tacc += du * (zt[k] / Tm);
        if (copy_kind == kCopySlots) {
          float* c = static_cast<float*>(copy) + static_cast<int64_t>(n) * 4 * HW * L + p * L + t;
#pragma unroll
          for (int sl = 0; sl < 4; ++sl) c[sl * HW * L] = g;
        } else if (copy_kind == kCopyFloat) {
          static_cast<float*>(copy)[pix * L + t] = g;
        }
      }
      if (copy_kind == kCopyHalf && t < Ls)
        static_cast<__half*>(copy)[pix * Ls + t] = __float2half_rn(t < L ? g : 0.0f);
    }
  }
  if (gT != nullptr) {
    tacc = warp_sum(tacc);
    if (lane == 0 && tacc != 0.0f) atomicAdd(gT, tacc);
  }
}

int grid_for(int64_t npix) {
  const int64_t blocks = (npix + 7) / 8;  // 8 warps per block
  return static_cast<int>(std::min<int64_t>(blocks, static_cast<int64_t>(sm_count()) * 16));
}

template <typename T, typename TC>
int fwd_impl(const T* msgs, const TC* cost, const float* Tm, float* out, int B, int H, int W, int L, int Ls,
             cudaStream_t s, float csign = 1.0f, float* lnorm = nullptr) {
  const int g = grid_for(static_cast<int64_t>(B) * H * W);
  const int k = (L + 31) / 32;
#define BPL_BFWD(KK) \
  beliefs_fwd_kernel<KK, T, TC><<<g, 256, 0, s>>>(msgs, cost, csign, Tm, out, lnorm, B, H, W, L, Ls)
  if (k <= 1) BPL_BFWD(1);
  else if (k <= 2) BPL_BFWD(2);
  else if (k <= 4) BPL_BFWD(4);
  else if (k <= 6) BPL_BFWD(6);
  else if (k <= 8) BPL_BFWD(8);
  else if (k <= 16) BPL_BFWD(16);
  else BPL_BFWD(32);
#undef BPL_BFWD
  BPL_CUDA_TRY(cudaGetLastError(), "beliefs_forward launch");
  return BPL_OK;
}

template <typename T, typename TC>
int bwd_impl(const T* msgs, const TC* cost, const float* Tm, const float* y, const float* gy, float* gz, float* gT,
             int B, int H, int W, int L, int Ls, cudaStream_t s, float gz_sign = 1.0f, void* copy = nullptr,
             int copy_kind = kCopyNone, float csign = 1.0f, const float* lnorm = nullptr) {
  if (gT) BPL_CUDA_TRY(cudaMemsetAsync(gT, 0, sizeof(float), s), "beliefs_backward: memset");
  const int g = grid_for(static_cast<int64_t>(B) * H * W);
  const int k = (L + 31) / 32;
#define BPL_BBWD(KK)                                                                                  \
  beliefs_bwd_kernel<KK, T, TC><<<g, 256, 0, s>>>(msgs, cost, csign, Tm, y, gy, gz, gz_sign, copy, copy_kind, gT, \
                                                  lnorm, B, H, W, L, Ls)
  if (k <= 1) BPL_BBWD(1);
  else if (k <= 2) BPL_BBWD(2);
  else if (k <= 4) BPL_BBWD(4);
  else if (k <= 6) BPL_BBWD(6);
  else if (k <= 8) BPL_BBWD(8);
  else if (k <= 16) BPL_BBWD(16);
  else BPL_BBWD(32);
#undef BPL_BBWD
  BPL_CUDA_TRY(cudaGetLastError(), "beliefs_backward launch");
  return BPL_OK;
}

// dst (B, 4, n) = src (B, n) repeated over the four message slots, in units
// of E (16-byte vectors where the rows allow).  grid (x, B)
template <typename E>
__global__ void __launch_bounds__(256) slots_broadcast_kernel(const E* __restrict__ src, E* __restrict__ dst,
                                                              int64_t n) {
  const int64_t b = blockIdx.y;
  const E* s = src + b * n;
  E* d = dst + b * 4 * n;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const E v = __ldg(s + i);
    d[i] = v;
    d[n + i] = v;
    d[2 * n + i] = v;
    d[3 * n + i] = v;
  }
}

}  // namespace
}  // namespace bpl

using namespace bpl;

extern "C" int bpl_broadcast_slots(const void* src, void* dst, int B, int64_t row_elems, int elem_bytes,
                                   void* stream) {
  BPL_TRACE("bpl_broadcast_slots");
  BPL_REQUIRE(src && dst, "broadcast_slots: null pointer");
  BPL_REQUIRE(B >= 1 && B <= 65535 && row_elems >= 1, "broadcast_slots: bad shape");
  BPL_REQUIRE(elem_bytes == 2 || elem_bytes == 4, "broadcast_slots: element size %d not 2 or 4", elem_bytes);
  const int64_t bytes = row_elems * elem_bytes;
  const bool vec = bytes % 16 == 0 && reinterpret_cast<uintptr_t>(src) % 16 == 0 &&
                   reinterpret_cast<uintptr_t>(dst) % 16 == 0;
  const int64_t n = vec ? bytes / 16 : row_elems;
  const unsigned gx = static_cast<unsigned>(std::min<int64_t>((n + 255) / 256, 8 * static_cast<int64_t>(sm_count())));
  const dim3 grid(std::max(1u, gx), B);
  cudaStream_t st = as_stream(stream);
  if (vec)
    slots_broadcast_kernel<uint4><<<grid, 256, 0, st>>>(static_cast<const uint4*>(src), static_cast<uint4*>(dst), n);
  else if (elem_bytes == 4)
    slots_broadcast_kernel<unsigned><<<grid, 256, 0, st>>>(static_cast<const unsigned*>(src),
                                                           static_cast<unsigned*>(dst), n);
  else
    slots_broadcast_kernel<unsigned short><<<grid, 256, 0, st>>>(static_cast<const unsigned short*>(src),
                                                                 static_cast<unsigned short*>(dst), n);
  BPL_CUDA_TRY(cudaGetLastError(), "broadcast_slots launch");
  return BPL_OK;
}

extern "C" int bpl_beliefs_forward(const void* messages, int messages_half, const float* cost,
                                   const float* temperature, float* beliefs, int B, int H, int W, int L, int Ls,
                                   void* stream) {
  BPL_TRACE("bpl_beliefs_forward");
  BPL_REQUIRE(messages && cost && beliefs && temperature, "beliefs_forward: null pointer");
  BPL_REQUIRE(B >= 1 && H >= 1 && W >= 1 && L >= 1 && L <= 1024 && Ls >= L, "beliefs_forward: bad shape");
  if (messages_half)
    return fwd_impl(static_cast<const __half*>(messages), cost, temperature, beliefs, B, H, W, L, Ls,
                    as_stream(stream));
  return fwd_impl(static_cast<const float*>(messages), cost, temperature, beliefs, B, H, W, L, Ls,
                  as_stream(stream));
}

extern "C" int bpl_beliefs_forward_ex(const void* messages, int messages_half, const void* cost, int cost_half,
                                      float cost_sign, const float* temperature, float* beliefs, float* log_norm,
                                      int B, int H, int W, int L, int Ls, void* stream) {
  BPL_TRACE("bpl_beliefs_forward_ex");
  BPL_REQUIRE(messages && cost && beliefs && temperature, "beliefs_forward: null pointer");
  BPL_REQUIRE(B >= 1 && H >= 1 && W >= 1 && L >= 1 && L <= 1024 && Ls >= L, "beliefs_forward: bad shape");
  BPL_REQUIRE(!cost_half || Ls == ((L + 7) & ~7), "beliefs_forward: a half cost has the padded label stride");
  BPL_REQUIRE(cost_sign == 1.0f || cost_sign == -1.0f, "beliefs_forward: cost sign must be +-1");
  cudaStream_t st = as_stream(stream);
  const float cs = cost_sign;
  float* ln = log_norm;
  if (messages_half) {
    const __half* m = static_cast<const __half*>(messages);
    return cost_half ? fwd_impl(m, static_cast<const __half*>(cost), temperature, beliefs, B, H, W, L, Ls, st, cs, ln)
                     : fwd_impl(m, static_cast<const float*>(cost), temperature, beliefs, B, H, W, L, Ls, st, cs, ln);
  }
  const float* m = static_cast<const float*>(messages);
  return cost_half ? fwd_impl(m, static_cast<const __half*>(cost), temperature, beliefs, B, H, W, L, Ls, st, cs, ln)
                   : fwd_impl(m, static_cast<const float*>(cost), temperature, beliefs, B, H, W, L, Ls, st, cs, ln);
}

extern "C" int bpl_beliefs_backward_ex(const void* messages, int messages_half, const void* cost, int cost_half,
                                       float cost_sign, const float* temperature, const float* beliefs, const float* grad_beliefs,
                                       float* grad_z, float grad_z_sign, void* grad_copy, int copy_kind,
                                       float* grad_temperature, const float* log_norm, int B, int H, int W, int L,
                                       int Ls, void* stream) {
  BPL_TRACE("bpl_beliefs_backward_ex");
  BPL_REQUIRE(beliefs && grad_beliefs && grad_z && temperature, "beliefs_backward: null pointer");
  BPL_REQUIRE(grad_temperature == nullptr || log_norm || (messages && cost), "beliefs_backward: null messages/cost");
  BPL_REQUIRE(B >= 1 && H >= 1 && W >= 1 && L >= 1 && L <= 1024 && Ls >= L, "beliefs_backward: bad shape");
  BPL_REQUIRE(!cost_half || Ls == ((L + 7) & ~7), "beliefs_backward: a half cost has the padded label stride");
  BPL_REQUIRE(grad_z_sign == 1.0f || grad_z_sign == -1.0f, "beliefs_backward: sign must be +-1");
  BPL_REQUIRE(cost_sign == 1.0f || cost_sign == -1.0f, "beliefs_backward: cost sign must be +-1");
  BPL_REQUIRE(copy_kind >= kCopyNone && copy_kind <= kCopyFloat, "beliefs_backward: bad copy kind %d", copy_kind);
  BPL_REQUIRE(copy_kind == kCopyNone || grad_copy, "beliefs_backward: null gradient copy");
  BPL_REQUIRE(copy_kind != kCopyHalf || Ls == ((L + 7) & ~7), "beliefs_backward: the half copy has stride Lp");
  cudaStream_t st = as_stream(stream);
#define BPL_BBWD_EX(MT, CT)                                                                                      \
  bwd_impl(static_cast<const MT*>(messages), static_cast<const CT*>(cost), temperature, beliefs, grad_beliefs, \
           grad_z, grad_temperature, B, H, W, L, Ls, st, grad_z_sign, grad_copy, copy_kind, cost_sign, log_norm)
  if (messages_half) return cost_half ? BPL_BBWD_EX(__half, __half) : BPL_BBWD_EX(__half, float);
  return cost_half ? BPL_BBWD_EX(float, __half) : BPL_BBWD_EX(float, float);
#undef BPL_BBWD_EX
}

extern "C" int bpl_beliefs_backward(const void* messages, int messages_half, const float* cost,
                                    const float* temperature, const float* beliefs, const float* grad_beliefs,
                                    float* grad_z, float* grad_temperature, int B, int H, int W, int L, int Ls,
                                    void* stream) {
  BPL_TRACE("bpl_beliefs_backward");
  BPL_REQUIRE(beliefs && grad_beliefs && grad_z && temperature, "beliefs_backward: null pointer");
  BPL_REQUIRE(grad_temperature == nullptr || (messages && cost), "beliefs_backward: null messages/cost");
  BPL_REQUIRE(B >= 1 && H >= 1 && W >= 1 && L >= 1 && L <= 1024 && Ls >= L, "beliefs_backward: bad shape");
  if (messages_half)
    return bwd_impl(static_cast<const __half*>(messages), cost, temperature, beliefs, grad_beliefs, grad_z,
                    grad_temperature, B, H, W, L, Ls, as_stream(stream));
  return bwd_impl(static_cast<const float*>(messages), cost, temperature, beliefs, grad_beliefs, grad_z,
                  grad_temperature, B, H, W, L, Ls, as_stream(stream));
}

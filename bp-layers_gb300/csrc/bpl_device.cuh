// Device-side building blocks shared by the BP-Layers kernels (sm_103a).
//
// Label layout used by every LBP kernel: one warp owns one scanline and the
// L labels of a pixel are spread over the lanes as  label = lane + 32*k,
// k = 0..K-1 (K = ceil(L/32), held in registers).  With this mapping the
// reference's shared-memory stride-halving reductions over labels
// (ops/lbp_stereo/src/lbp_min_sum_kernel.cu:121-139 and :170-177: position i
// combines with i+s for s = P/2 .. 1, P = next power of two of L, only while
// i < s and i+s < L) become register steps for s >= 32 and warp shuffles for
// s < 32, in exactly the same order, so min/argmin ties and the float sum
// come out bit-identical.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace bpl {

constexpr unsigned FULL = 0xffffffffu;

enum Dir { LEFT = 0, RIGHT = 1, UP = 2, DOWN = 3 };

__host__ __device__ constexpr int np2(int k) {
  int p = 1;
  while (p < k) p <<= 1;
  return p;
}

// Error word written by kernels whose bounded waits ran out.  Read with
// bpl_read_device_error().  Declared for relocatable units only (the ones
// device-linked with its definition): a unit compiled as a whole program
// that used it would get a private copy the library never reads, so there
// it does not compile.
#ifdef __CUDACC_RDC__
extern __device__ int g_bpl_error;
// Poll limit of the bounded waits (default kWaitLimit; bpl_set_wait_limit
// lowers it so that a test can make a wait run out).
extern __device__ unsigned g_bpl_wait_limit;
#endif
constexpr unsigned kWaitLimit = 1u << 24;
// Poll limit of the drain that waits for a failed kernel's copies in flight
// (independent of g_bpl_wait_limit: those copies always land).
constexpr unsigned kDrainLimit = 1u << 20;

enum DeviceError { DEV_ERR_NONE = 0, DEV_ERR_WAIT_TIMEOUT = 1 };

#ifdef __CUDACC_RDC__
__device__ __forceinline__ void raise_device_error(int code) { atomicCAS(&g_bpl_error, 0, code); }
#endif

// ---------------------------------------------------------------------------
// Warp reductions with the reference's tree order.

// Min / argmin tree.  v[k], lab[k] hold label lane+32k.  L = number of valid
// labels.  Ties go to the element at the higher tree position (`<=`,
// lbp_min_sum_kernel.cu:128).  Result is returned warp-uniform.
template <int K>
__device__ __forceinline__ void tree_argmin(float (&v)[K], int (&lab)[K], int L, int lane,
                                            float& out_v, int& out_l) {
  // register levels: s = 32*m, m = np2(K)/2 .. 1
#pragma unroll
  for (int m = np2(K) / 2; m >= 1; m >>= 1) {
#pragma unroll
    for (int k = 0; k < m; ++k) {
      if (k + m < K) {
        const int t = lane + 32 * k;
        if (t + 32 * m < L && v[k + m] <= v[k]) {
          v[k] = v[k + m];
          lab[k] = lab[k + m];
        }
      }
    }
  }
  // shuffle levels on slot 0
  float v0 = v[0];
  int l0 = lab[0];
  int s = (K > 1) ? 16 : (np2(L) / 2);
  for (; s > 0; s >>= 1) {
    const float ov = __shfl_down_sync(FULL, v0, s);
    const int ol = __shfl_down_sync(FULL, l0, s);
    if (lane < s && lane + s < L && ov <= v0) {
      v0 = ov;
      l0 = ol;
    }
  }
  out_v = __shfl_sync(FULL, v0, 0);
  out_l = __shfl_sync(FULL, l0, 0);
}

// Sum tree (lbp_min_sum_kernel.cu:170-177) of non-negative values.  Returns
// the warp-uniform sum.  Branch-free: a position that does not take part at a
// level adds +0.0, which leaves a non-negative float unchanged.
template <int K>
__device__ __forceinline__ float tree_sum(float (&v)[K], int L, int lane) {
#pragma unroll
  for (int m = np2(K) / 2; m >= 1; m >>= 1) {
#pragma unroll
    for (int k = 0; k < m; ++k) {
      if (k + m < K) {
        const int t = lane + 32 * k;
        v[k] = __fadd_rn(v[k], (t + 32 * m < L) ? v[k + m] : 0.0f);
      }
    }
  }
  float v0 = v[0];
  if (K > 1) {
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
      const float o = __shfl_down_sync(FULL, v0, s);
      v0 = __fadd_rn(v0, (lane < s) ? o : 0.0f);
    }
  } else {
    for (int s = np2(L) / 2; s > 0; s >>= 1) {
      const float o = __shfl_down_sync(FULL, v0, s);
      v0 = __fadd_rn(v0, (lane < s && lane + s < L) ? o : 0.0f);
    }
  }
  return __shfl_sync(FULL, v0, 0);
}

// Order-preserving map of floats onto unsigned integers (-0 below +0, NaN
// above +inf), so that a warp minimum is one redux.sync instruction.
__device__ __forceinline__ unsigned f2ord(float f) {
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}
__device__ __forceinline__ float warp_min_redux(float v) { return ord2f(__reduce_min_sync(0xffffffffu, f2ord(v))); }

// Reduce-scatter of 8 per-lane values over the warp in 9 shuffles (instead
// of 8 full warp sums): returns in every lane the warp total of value
// (lane >> 2) & 7, i.e. lanes 4b..4b+3 hold the total of value b.  Any
// summation order (for the adjoint kernels, which have no bitwise target).
__device__ __forceinline__ float warp_reduce_scatter8(const float (&v)[8], int lane) {
  const bool h16 = lane & 16, h8 = lane & 8, h4 = lane & 4;
  float w4[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float keep = h16 ? v[i + 4] : v[i];
    const float send = h16 ? v[i] : v[i + 4];
    w4[i] = keep + __shfl_xor_sync(FULL, send, 16);
  }
  float w2[2];
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const float keep = h8 ? w4[i + 2] : w4[i];
    const float send = h8 ? w4[i] : w4[i + 2];
    w2[i] = keep + __shfl_xor_sync(FULL, send, 8);
  }
  float w1 = (h4 ? w2[1] : w2[0]) + __shfl_xor_sync(FULL, h4 ? w2[0] : w2[1], 4);
  w1 += __shfl_xor_sync(FULL, w1, 2);
  w1 += __shfl_xor_sync(FULL, w1, 1);
  return w1;
}

// The same for four values: value q summed over the warp ends in lanes
// 8q .. 8q+7.
__device__ __forceinline__ float warp_reduce_scatter4(const float (&v)[4], int lane) {
  const bool h16 = lane & 16, h8 = lane & 8;
  float w2[2];
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const float keep = h16 ? v[i + 2] : v[i];
    const float send = h16 ? v[i] : v[i + 2];
    w2[i] = keep + __shfl_xor_sync(FULL, send, 16);
  }
  float w1 = (h8 ? w2[1] : w2[0]) + __shfl_xor_sync(FULL, h8 ? w2[0] : w2[1], 8);
  w1 += __shfl_xor_sync(FULL, w1, 4);
  w1 += __shfl_xor_sync(FULL, w1, 2);
  w1 += __shfl_xor_sync(FULL, w1, 1);
  return w1;
}

// Plain warp sum (any order) for the adjoint kernels, which have no bitwise
// parity target (the reference uses float atomics).
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}

// ---------------------------------------------------------------------------
// mbarrier + bulk (TMA 1-D) copies.

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// Bulk global->shared copy completing on `bar`.  dst, src 16-byte aligned,
// bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

#ifdef __CUDACC_RDC__
// Bounded wait: gives up after `limit` polls (each poll may suspend for a
// hardware-defined interval), raising DEV_ERR_WAIT_TIMEOUT.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t limit) {
  for (uint32_t i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  raise_device_error(DEV_ERR_WAIT_TIMEOUT);
  return false;
}
// ... with the library's poll limit (g_bpl_wait_limit)
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  return mbar_wait_bounded(bar, parity, *static_cast<volatile unsigned*>(&g_bpl_wait_limit));
}
#endif

// 4-byte cp.async (any alignment) with group commit/wait, for rows whose
// length is not a multiple of 16 bytes.
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// float -> unsigned short as the reference's static_cast compiles (PTX
// float-to-integer conversions clamp to the destination range, NaN -> 0).
__device__ __forceinline__ int sat_u16(float v) {
  unsigned short r;
  asm("cvt.rzi.u16.f32 %0, %1;" : "=h"(r) : "f"(v));
  return static_cast<int>(r);
}

}  // namespace bpl

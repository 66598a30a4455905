// Flow max-projected SAD for sm_103a.
//
// Reference: ops/flow_mp_sad/src/flow_mp_sad_kernel.cu
//   forward  :10-124  per pixel, a K x K window (K = sws+1, displacement
//            u, v in [-sws/2, sws/2] plus offsets) of channel-ordered SADs,
//            40 where the match is outside the image; then
//            cv_u[u] = min_v, u_star[u] = argmin_v + blockIdx_v*sws and
//            cv_v[v] = min_u, v_star[v] = argmin_u + blockIdx_u*sws,
//            strict `<` from 9999999 (first index wins ties); one block of
//            K threads per pixel (:231-245)
//   backward :126-200 routes in_grad_u / in_grad_v through the stored
//            argmins to df0 (local sum) and df1 (atomics)
//
// GB300 design.  Forward: a block owns P pixels of one row (P chosen so the
// P windows fit in shared memory) and K threads per pixel, one per u.  Each
// thread computes its window column over v with the pixel's f0 channels in
// registers (channels summed in order: bit-identical SADs), keeps the running
// column minimum (cv_u, v ascending, strict <), and stores the column in the
// block's window buffer; after one barrier the thread for v scans the row
// (cv_v, u ascending, strict <).  f1 is read through L1: neighbouring pixels
// of the block read overlapping windows.  Backward: as the reference, one
// thread per (channel, pixel).
#include <cuda_runtime.h>

#include <algorithm>

#include "bpl_device.cuh"
#include "bpl_internal.h"

namespace bpl {
namespace {

constexpr int kMaxC = 64;  // channels held in registers

struct FlowArgs {
  const float* f0;
  const float* f1;
  float* cv_u;
  float* cv_v;
  float* u_star;
  float* v_star;
  int B, C, H, W, sws, K, hs;
  int off_u, off_v, blk_u, blk_v;
  int P;  // pixels per block
};

// grid (ceil(W/P), H, B); block (K, P)
template <int CR>
__global__ void __launch_bounds__(1024) flow_forward_kernel(FlowArgs a) {
  extern __shared__ __align__(16) float win[];  // [P][K][K]: win[p][v][u]
  const int ui = threadIdx.x;
  const int p = threadIdx.y;
  const int n = blockIdx.z, y = blockIdx.y;
  const int x = blockIdx.x * a.P + p;
  const int K = a.K;
  float* wp = win + static_cast<int64_t>(p) * K * K;
  const bool px_ok = x < a.W;
  const int64_t HW = static_cast<int64_t>(a.H) * a.W;
  const float* f0 = a.f0 + static_cast<int64_t>(n) * a.C * HW;
  const float* f1 = a.f1 + static_cast<int64_t>(n) * a.C * HW;

  float fv[CR > 0 ? CR : 1];
  if (px_ok) {
#pragma unroll
    for (int c = 0; c < CR; ++c)
      if (c < a.C) fv[c] = __ldg(f0 + c * HW + static_cast<int64_t>(y) * a.W + x);
  }
  const int u = ui - a.hs;
  const int xm = x + a.off_u + u;
  const bool col_ok = px_ok && xm >= 0 && xm < a.W;
  float mn = 9999999.0f;
  int amn = 0;
  for (int vi = 0; vi < K; ++vi) {
    const int v = vi - a.hs;
    const int ym = y + a.off_v + v;
    float sad = 40.0f;
    // v runs over [-hs, hs] only: the last row stays 40 when sws is odd
    if (col_ok && v <= a.hs && ym >= 0 && ym < a.H) {
      const float* q = f1 + static_cast<int64_t>(ym) * a.W + xm;
      float s = 0.0f;
      if (CR > 0) {
#pragma unroll
        for (int c = 0; c < CR; ++c)
          if (c < a.C) s = __fadd_rn(s, fabsf(__fsub_rn(fv[c], __ldg(q + c * HW))));
      } else {
        const float* r0 = f0 + static_cast<int64_t>(y) * a.W + x;
        for (int c = 0; c < a.C; ++c) s = __fadd_rn(s, fabsf(__fsub_rn(__ldg(r0 + c * HW), __ldg(q + c * HW))));
      }
      sad = s;
    }
    wp[vi * K + ui] = sad;
    if (sad < mn) {
      mn = sad;
      amn = vi;
    }
  }
  __syncthreads();
  if (!px_ok) return;
  const int64_t o = ((static_cast<int64_t>(n) * a.H + y) * a.W + x) * K;
  a.cv_u[o + ui] = mn;
  a.u_star[o + ui] = static_cast<float>(amn + a.blk_v * a.sws);
  // row ui of the window: min over u (thread index reused as v)
  float mr = 9999999.0f;
  int amr = 0;
  const float* row = wp + ui * K;
  for (int uu = 0; uu < K; ++uu) {
    const float s = row[uu];
    if (s < mr) {
      mr = s;
      amr = uu;
    }
  }
  a.cv_v[o + ui] = mr;
  a.v_star[o + ui] = static_cast<float>(amr + a.blk_u * a.sws);
}

struct FlowBwdArgs {
  const float* f0;
  const float* f1;
  const float* gu;
  const float* gv;
  const float* us;
  const float* vs;
  float* df0;
  float* df1;
  int B, C, H, W, sws, K, hs;
};

// grid (ceil(W/32), H, B*C); block 32
__global__ void __launch_bounds__(128) flow_backward_kernel(FlowBwdArgs a) {
  const int n = blockIdx.z / a.C, c = blockIdx.z % a.C;
  const int y = blockIdx.y;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= a.W) return;
  const int64_t HW = static_cast<int64_t>(a.H) * a.W;
  const float* r1 = a.f1 + (static_cast<int64_t>(n) * a.C + c) * HW;
  float* d1 = a.df1 + (static_cast<int64_t>(n) * a.C + c) * HW;
  const float a0 = a.f0[(static_cast<int64_t>(n) * a.C + c) * HW + static_cast<int64_t>(y) * a.W + x];
  const int64_t o = ((static_cast<int64_t>(n) * a.H + y) * a.W + x) * a.K;
  float g0 = 0.0f;
  for (int pass = 0; pass < 2; ++pass) {
    for (int i = -a.hs; i <= a.hs; ++i) {
      const int idx = i + a.hs;
      int u, v;
      // the stored index is converted to short as in the reference (:156, :179)
      if (pass == 0) {
        u = i;
        v = static_cast<int>(static_cast<short>(__ldg(a.us + o + idx))) - a.hs;
      } else {
        v = i;
        u = static_cast<int>(static_cast<short>(__ldg(a.vs + o + idx))) - a.hs;
      }
      if (x + u >= 0 && x + u < a.W && y + v >= 0 && y + v < a.H) {
        const int64_t q = static_cast<int64_t>(y + v) * a.W + x + u;
        const float diff = __fsub_rn(a0, __ldg(r1 + q));
        if (fabsf(diff) > 1e-15f) {
          const float gg = __ldg((pass == 0 ? a.gu : a.gv) + o + idx);
          const float upd = __fmul_rn(__fdiv_rn(diff, fabsf(diff)), gg);
          g0 = __fadd_rn(g0, upd);
          atomicAdd(d1 + q, -upd);
        }
      }
    }
  }
  a.df0[(static_cast<int64_t>(n) * a.C + c) * HW + static_cast<int64_t>(y) * a.W + x] = g0;
}

}  // namespace
}  // namespace bpl

using namespace bpl;

extern "C" int bpl_flow_forward(const float* f0, const float* f1, float* cv_u, float* cv_v, float* u_star,
                                float* v_star, int B, int C, int H, int W, int sws, int offset_u, int offset_v,
                                int block_u, int block_v, void* stream) {
  BPL_REQUIRE(f0 && f1 && cv_u && cv_v && u_star && v_star, "flow_forward: null pointer");
  BPL_REQUIRE(B >= 1 && C >= 1 && H >= 1 && W >= 1, "flow_forward: bad shape");
  BPL_REQUIRE(sws >= 0 && sws + 1 <= 1024, "flow_forward: window size %d outside [1, 1024]", sws + 1);
  FlowArgs a{f0, f1, cv_u, cv_v, u_star, v_star, B, C, H, W, sws, sws + 1, sws / 2,
             offset_u, offset_v, block_u, block_v, 1};
  const int K = a.K;
  const size_t per_px = sizeof(float) * static_cast<size_t>(K) * K;
  const size_t budget = std::min<size_t>(static_cast<size_t>(max_smem_optin()), 200 * 1024);
  BPL_REQUIRE(per_px <= budget, "flow_forward: window %d x %d does not fit in shared memory", K, K);
  a.P = static_cast<int>(std::max<size_t>(1, std::min<size_t>({budget / per_px, static_cast<size_t>(1024 / K),
                                                                 static_cast<size_t>(32)})));
  const size_t smem = per_px * a.P;
  dim3 grid((W + a.P - 1) / a.P, H, B);
  dim3 block(K, a.P);
  auto launch = [&](auto kern) -> int {
    if (smem > 48 * 1024)
      BPL_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)),
                   "cudaFuncSetAttribute");
    kern<<<grid, block, smem, as_stream(stream)>>>(a);
    BPL_CUDA_TRY(cudaGetLastError(), "flow_forward launch");
    return BPL_OK;
  };
  if (C <= 16) return launch(flow_forward_kernel<16>);
  if (C <= 32) return launch(flow_forward_kernel<32>);
  if (C <= kMaxC) return launch(flow_forward_kernel<kMaxC>);
  return launch(flow_forward_kernel<0>);
}

extern "C" int bpl_flow_backward(const float* f0, const float* f1, const float* in_grad_u, const float* in_grad_v,
                                 const float* u_star, const float* v_star, float* df0, float* df1, int B, int C,
                                 int H, int W, int sws, void* stream) {
  BPL_REQUIRE(f0 && f1 && in_grad_u && in_grad_v && u_star && v_star && df0 && df1, "flow_backward: null pointer");
  BPL_REQUIRE(B >= 1 && C >= 1 && H >= 1 && W >= 1 && sws >= 0, "flow_backward: bad shape");
  FlowBwdArgs a{f0, f1, in_grad_u, in_grad_v, u_star, v_star, df0, df1, B, C, H, W, sws, sws + 1, sws / 2};
  BPL_CUDA_TRY(cudaMemsetAsync(df1, 0, sizeof(float) * B * C * H * W, as_stream(stream)), "flow_backward: memset");
  dim3 grid((W + 31) / 32, H, B * C);
  flow_backward_kernel<<<grid, 32, 0, as_stream(stream)>>>(a);
  BPL_CUDA_TRY(cudaGetLastError(), "flow_backward launch");
  return BPL_OK;
}

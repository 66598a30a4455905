// Coarse-to-fine glue between the BP levels of the stereo network.
//
// Reference: stereo.py:104-113.  The next (finer) level's probability volume
// pv (N, 2h, 2w, 2d) receives the coarse beliefs (N, h, w, d) upsampled by 2
// along rows, columns and labels (F.interpolate(..., scale_factor=2.0,
// mode='trilinear'), align_corners False) and halved: pv += up(beliefs) / 2.
// PyTorch runs this as three full-volume passes (interpolate into a
// temporary, divide, add); here one pass reads pv once, writes it once and
// reads the coarse volume through the cache.
//
// Interpolation as PyTorch defines it (UpSampleTrilinear3d with scale 1/2):
// the source coordinate of output index o is max(0, 0.5 * (o + 0.5) - 0.5),
// i0 its integer part, i1 = i0 + 1 unless i0 is the last input index,
// lambda1 = src - i0, lambda0 = 1 - lambda1; the value nests rows outside,
// columns, labels inside.  For scale 2 every coordinate and weight is a
// multiple of 1/4, so the weights are exact; the products and sums are
// rounded in that nesting order.
#include <cuda_runtime.h>

#include <algorithm>

#include "bpl_device.cuh"
#include "bpl_internal.h"

namespace bpl {
namespace {

struct Lin {
  int i0, i1;
  float l0, l1;
};

__device__ __forceinline__ Lin lin2(int o, int in) {
  float src = __fsub_rn(__fmul_rn(0.5f, __fadd_rn(static_cast<float>(o), 0.5f)), 0.5f);
  src = src < 0.0f ? 0.0f : src;
  Lin r;
  r.i0 = static_cast<int>(src);
  r.i1 = r.i0 + ((r.i0 < in - 1) ? 1 : 0);
  r.l1 = __fsub_rn(src, static_cast<float>(r.i0));
  r.l0 = __fsub_rn(1.0f, r.l1);
  return r;
}

// one warp per fine pixel (row, column), lanes over its labels; grid-stride
// over pixels
__global__ void __launch_bounds__(256) upsample_add_kernel(const float* __restrict__ coarse, float* __restrict__ pv,
                                                           int N, int h, int w, int d, float weight) {
  const int H = 2 * h, W = 2 * w, D = 2 * d;
  const int lane = threadIdx.x & 31;
  const int64_t npx = static_cast<int64_t>(N) * H * W;
  for (int64_t p = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; p < npx;
       p += (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5) {
    const int x = static_cast<int>(p % W);
    const int64_t r = p / W;
    const int y = static_cast<int>(r % H);
    const int n = static_cast<int>(r / H);
    const Lin ty = lin2(y, h), tx = lin2(x, w);
    const float* c = coarse + static_cast<int64_t>(n) * h * w * d;
    const float* c00 = c + (static_cast<int64_t>(ty.i0) * w + tx.i0) * d;
    const float* c01 = c + (static_cast<int64_t>(ty.i0) * w + tx.i1) * d;
    const float* c10 = c + (static_cast<int64_t>(ty.i1) * w + tx.i0) * d;
    const float* c11 = c + (static_cast<int64_t>(ty.i1) * w + tx.i1) * d;
    float* out = pv + p * D;
    for (int z = lane; z < D; z += 32) {
      const Lin tz = lin2(z, d);
      auto row = [&](const float* q) {
        return __fadd_rn(__fmul_rn(tz.l0, __ldg(q + tz.i0)), __fmul_rn(tz.l1, __ldg(q + tz.i1)));
      };
      const float p0 = __fadd_rn(__fmul_rn(tx.l0, row(c00)), __fmul_rn(tx.l1, row(c01)));
      const float p1 = __fadd_rn(__fmul_rn(tx.l0, row(c10)), __fmul_rn(tx.l1, row(c11)));
      const float val = __fadd_rn(__fmul_rn(ty.l0, p0), __fmul_rn(ty.l1, p1));
      out[z] = __fadd_rn(out[z], __fmul_rn(val, weight));
    }
  }
}

}  // namespace
}  // namespace bpl

using namespace bpl;

extern "C" int bpl_upsample_add_beliefs(const float* beliefs, float* pv, int N, int h, int w, int d, float weight,
                                        void* stream) {
  BPL_TRACE("bpl_upsample_add_beliefs");
  BPL_REQUIRE(beliefs && pv, "upsample_add_beliefs: null pointer");
  BPL_REQUIRE(N >= 1 && h >= 1 && w >= 1 && d >= 1, "upsample_add_beliefs: bad shape");
  const int64_t npx = static_cast<int64_t>(N) * 4 * h * w;  // fine pixels, one warp each
  const int64_t blocks = std::min<int64_t>((npx + 7) / 8, 16 * static_cast<int64_t>(sm_count()));
  upsample_add_kernel<<<static_cast<unsigned>(std::max<int64_t>(blocks, 1)), 256, 0, as_stream(stream)>>>(
      beliefs, pv, N, h, w, d, weight);
  BPL_CUDA_TRY(cudaGetLastError(), "upsample_add_beliefs launch");
  return BPL_OK;
}

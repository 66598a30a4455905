// Stereo SAD cost volume for sm_103a.
//
// Reference: ops/sad/src/stereo_sad_kernel.cu
//   forward  :16-62   out[n,y,x,di] = sum_c |f0[n,c,y,x] - f1[n,c,y,x-d]|,
//             d = (int)(di*step + min_disp), channels summed in order, 40
//             where x-d is outside the image (:125), one thread per output
//   backward :64-108  df0 = sum_d sign(f0-f1) g, df1 = -sum_d sign(.) g(x+d),
//             gather form, d in increasing order, |diff| <= 1e-15 skipped
//
// GB300 design.  Forward: a block owns one row segment of TX pixels and all
// D disparities.  The f0 segment (C x TX) and the f1 segment it can match
// (C x (TX + dmax - dmin)) are staged in shared memory once; each thread
// accumulates a 4-pixel x 8-disparity register tile over the channels in
// order (two FP32 instructions per term, no FMA: bit-identical to the
// reference), then writes its 8 disparities of each pixel as two 16-byte
// stores.  FP32-issue bound (about 29 flop/byte at 376x1240x64x192); the
// channel chunks are double-buffered (cp.async of chunk i+1 while chunk i is
// summed), and blocks of up to 384 threads run with registers capped so that
// 2-3 are resident per SM: one block's chunk barrier then leaves the others
// issuing (a 512-thread block, D > 192, stays alone on its SM).
// Backward: lanes are channels and each thread owns 4 pixels; both sums walk
// the disparities in the reference order (additions of +-g in the same
// sequence: bit-identical).  Per chunk of 32 disparities the block stages
// (cp.async, double-buffered) its channels' f1 segment x - d, f0 segment
// x + d and the two gradient tables g[x, d] and g[x + d, d], which the warp
// reads as broadcasts; the thread slides a register window over its feature
// rows, so a term is a subtraction, a sign-bit operation, the |diff| test
// and a predicated add (ALU-pipe bound).
#include <cuda_runtime.h>

#include <algorithm>

#include "bpl_device.cuh"
#include "bpl_internal.h"

namespace bpl {
namespace {

constexpr int kTX = 64;          // pixels per block (forward)
constexpr int kPX = 4;           // pixels per thread
constexpr int kPD = 8;           // disparities per thread
constexpr int kCChunk = 16;      // channels staged per pass

struct SadArgs {
  const float* f0;
  const float* f1;
  float* out;
  int B, C, H, W, D;
  int min_disp;
  float step;
  int unit_step;  // step == 1: d = di + min_disp
  int dlo, dhi;   // smallest / largest disparity
};

__device__ __forceinline__ int disparity(const SadArgs& a, int di) {
  if (a.unit_step) return di + a.min_disp;
  // (d_idx * step) + min_disp in float, truncated (stereo_sad_kernel.cu:35)
  return static_cast<int>(__fadd_rn(__fmul_rn(static_cast<float>(di), a.step), static_cast<float>(a.min_disp)));
}

// Shared-memory layout and lane mapping: lanes take consecutive pixel groups
// (16 per disparity group) so a quarter-warp's reads of its f1 windows are
// consecutive 16-byte chunks; each f1 row is staged with a leading pad that
// makes every thread's 11-value window start 16-byte aligned (three 128-bit
// loads, conflict-free).  With lanes on consecutive disparity groups the
// windows were 8 floats apart: an 8-way bank conflict.
constexpr int kPXG = kTX / kPX;  // pixel groups per block

// leading pad of an f1 row: (window start + pad) % 4 == 0 for every thread
__host__ __device__ inline int sad_pad(int dhi, int dlo) { return ((7 - (dhi - dlo)) % 4 + 4) % 4; }

// grid (ceil(W/kTX), H, B); block kPXG x (D/kPD rounded up) threads.
// MAXT/MINB: blocks of up to 384 threads run with registers capped (80, no
// spills) so that 2-3 blocks stay resident per SM and one block's chunk
// barrier does not idle the SM; 512-thread blocks (D > 192) keep theirs.
template <int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB) sad_forward_kernel(SadArgs a) {
  extern __shared__ __align__(16) float sm[];
  const int n = blockIdx.z, y = blockIdx.y, x0 = blockIdx.x * kTX;
  const int span = kTX + (a.dhi - a.dlo);      // f1 columns a block can match
  const int pad = a.unit_step ? sad_pad(a.dhi, a.dlo) : 0;
  const int spanp = (pad + span + 3) & ~3;
  const int bufsz = kCChunk * (kTX + spanp);   // one chunk: s0 [kCChunk][kTX], s1 [kCChunk][spanp]
  const int xb = x0 - a.dhi - pad;             // f1 column of s1[.][0]
  const int ndg = (a.D + kPD - 1) / kPD;
  const int tid = threadIdx.x;
  const int nthreads = blockDim.x;
  const int xg = tid % kPXG;                   // pixel group
  const int dg = tid / kPXG;                   // disparity group
  const bool active = dg < ndg;
  const int64_t HW = static_cast<int64_t>(a.H) * a.W;
  const float* f0 = a.f0 + static_cast<int64_t>(n) * a.C * HW + static_cast<int64_t>(y) * a.W;
  const float* f1 = a.f1 + static_cast<int64_t>(n) * a.C * HW + static_cast<int64_t>(y) * a.W;

  int dv[kPD];
#pragma unroll
  for (int q = 0; q < kPD; ++q) dv[q] = disparity(a, min(dg * kPD + q, a.D - 1));
  float acc[kPX][kPD];
#pragma unroll
  for (int p = 0; p < kPX; ++p)
#pragma unroll
    for (int q = 0; q < kPD; ++q) acc[p][q] = 0.0f;

  // stage chunk `ci` into buffer ci & 1 (cp.async; zeros outside the image)
  auto stage = [&](int ci) {
    const int c0 = ci * kCChunk;
    const int cn = min(kCChunk, a.C - c0);
    float* s0 = sm + (ci & 1) * bufsz;
    float* s1 = s0 + kCChunk * kTX;
    for (int e = tid; e < cn * kTX; e += nthreads) {
      const int cc = e / kTX, xx = e % kTX, x = x0 + xx;
      if (x < a.W) cp_async4(s0 + cc * kTX + xx, f0 + (c0 + cc) * HW + x);
      else s0[cc * kTX + xx] = 0.0f;
    }
    for (int e = tid; e < cn * spanp; e += nthreads) {
      const int cc = e / spanp, xx = e % spanp, x = xb + xx;
      if (x >= 0 && x < a.W && xx >= pad && xx < pad + span) cp_async4(s1 + cc * spanp + xx, f1 + (c0 + cc) * HW + x);
      else s1[cc * spanp + xx] = 0.0f;
    }
    cp_async_commit();
  };
  const int nchunk = (a.C + kCChunk - 1) / kCChunk;
  stage(0);
  for (int ci = 0; ci < nchunk; ++ci) {
    const int c0 = ci * kCChunk;
    const int cn = min(kCChunk, a.C - c0);
    if (ci + 1 < nchunk) {
      stage(ci + 1);
      cp_async_wait<1>();  // chunk ci has landed (ci + 1 may be in flight)
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const float* s0 = sm + (ci & 1) * bufsz;
    const float* s1 = s0 + kCChunk * kTX;
    if (active) {
      for (int cc = 0; cc < cn; ++cc) {
        float v0[kPX];
        {
          const float4 q0 = *reinterpret_cast<const float4*>(s0 + cc * kTX + xg * kPX);
          v0[0] = q0.x; v0[1] = q0.y; v0[2] = q0.z; v0[3] = q0.w;
        }
        const float* r1 = s1 + cc * spanp;
        // f1 column x - d sits at s1 index xl + pad + dhi - d (xl: pixel in block)
        if (a.unit_step) {
          // d = d0 + q: the 4 x 8 tile reads 11 consecutive f1 values, from a
          // 16-byte aligned start (indices below 0 of the last, partial
          // disparity group land in the f0 tile and feed only outputs that
          // are not stored)
          const int base = xg * kPX + pad + a.dhi - dv[0];
          float v1[kPX + kPD + 1];
          const float4* q1 = reinterpret_cast<const float4*>(r1 + base - (kPD - 1));
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            const float4 t = q1[k];
            v1[4 * k] = t.x; v1[4 * k + 1] = t.y; v1[4 * k + 2] = t.z; v1[4 * k + 3] = t.w;
          }
#pragma unroll
          for (int p = 0; p < kPX; ++p)
#pragma unroll
            for (int q = 0; q < kPD; ++q)
              acc[p][q] = __fadd_rn(acc[p][q], fabsf(__fsub_rn(v0[p], v1[p - q + kPD - 1])));
        } else {
#pragma unroll
          for (int p = 0; p < kPX; ++p) {
            const int xl = xg * kPX + p;
#pragma unroll
            for (int q = 0; q < kPD; ++q) {
              const float v1 = r1[xl + pad + a.dhi - dv[q]];
              acc[p][q] = __fadd_rn(acc[p][q], fabsf(__fsub_rn(v0[p], v1)));
            }
          }
        }
      }
    }
    __syncthreads();  // buffer ci & 1 is restaged by the next iteration's stage(ci + 2)
  }
  if (!active) return;
  float* out = a.out + ((static_cast<int64_t>(n) * a.H + y) * a.W) * a.D;
#pragma unroll
  for (int p = 0; p < kPX; ++p) {
    const int x = x0 + xg * kPX + p;
    if (x >= a.W) continue;
    float r[kPD];
#pragma unroll
    for (int q = 0; q < kPD; ++q) {
      const int xm = x - dv[q];
      r[q] = (xm >= 0 && xm < a.W) ? acc[p][q] : 40.0f;
    }
    float* o = out + static_cast<int64_t>(x) * a.D + dg * kPD;
    if ((a.D % 4 == 0) && dg * kPD + kPD <= a.D) {
      reinterpret_cast<float4*>(o)[0] = make_float4(r[0], r[1], r[2], r[3]);
      reinterpret_cast<float4*>(o)[1] = make_float4(r[4], r[5], r[6], r[7]);
    } else {
#pragma unroll
      for (int q = 0; q < kPD; ++q)
        if (dg * kPD + q < a.D) o[q] = r[q];
    }
  }
}

struct SadBwdArgs {
  const float* f0;
  const float* f1;
  const float* g;
  float* df0;
  float* df1;
  int B, C, H, W, D, min_disp, max_disp;
  int channel_limit;
};

constexpr int kBX = 32;            // pixels per block (backward)
constexpr int kBPX = 4;            // pixels per thread
constexpr int kBCH = 32;           // channels per block: lane = channel
constexpr int kBDC = 32;           // disparities per staged chunk
constexpr int kBFS = kBX + kBDC - 1;  // staged feature row (odd: lanes' rows fall in distinct banks)

// One term of the reference's sums: acc += (diff/|diff|) * g when |diff| >
// 1e-15 (df0), acc -= ... (df1).  diff/|diff| is exactly +-1, so the update
// is g with the sign of diff (flipped for df1): one sign-bit operation; a
// NaN diff never passes the test, as in the reference.
template <bool NEG>
__device__ __forceinline__ void sad_term(float& acc, float diff, float g) {
  const unsigned sb = (NEG ? ~__float_as_uint(diff) : __float_as_uint(diff)) & 0x80000000u;
  const float t = __uint_as_float(__float_as_uint(g) ^ sb);
  if (fabsf(diff) > 1e-15f) acc = __fadd_rn(acc, t);
}

// grid (ceil(W/32), H, B*ceil(C/32)); block 256 = 8 warps.  Warp w owns
// pixels x0 + 4w .. +3, lane the channel; both sums run over d ascending
// (the reference's order), chunk by chunk of 32 disparities staged in
// shared memory: the f1 row segment x - d and the f0 row segment x + d of
// the block's channels (NaN outside the image, which the |diff| test drops
// like the reference's bounds checks), g[y, x, d] and the diagonal
// g[y, x + d, d] (zero past max_disp: a zero update leaves the sum as it
// is, which is never -0).  Each thread slides a 4-value window over the
// staged rows, so a disparity costs it one new value per row and one
// broadcast 16-byte load per gradient table.
__global__ void __launch_bounds__(256, 3) sad_backward_kernel(SadBwdArgs a) {
  // two buffers: chunk ci + 1 lands (cp.async) while chunk ci is summed
  __shared__ float f1s[2][kBCH * kBFS];   // f1[c, x0 - d0 - 31 + k]
  __shared__ float f0s[2][kBCH * kBFS];   // f0[c, x0 + d0 + k]
  __shared__ __align__(16) float gA[2][kBDC * kBX];  // g[y, x0 + x, d0 + dd]
  __shared__ __align__(16) float gD[2][kBDC * kBX];  // g[y, x0 + x + d0 + dd, d0 + dd]
  const int ncb = (a.C + kBCH - 1) / kBCH;
  const int n = blockIdx.z / ncb;
  const int c0 = (blockIdx.z % ncb) * kBCH;
  const int y = blockIdx.y;
  const int x0 = blockIdx.x * kBX;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int c = c0 + lane;
  const int64_t HW = static_cast<int64_t>(a.H) * a.W;
  const float* grow = a.g + ((static_cast<int64_t>(n) * a.H + y) * a.W) * a.D;
  const float* f0b = a.f0 + (static_cast<int64_t>(n) * a.C + c0) * HW + static_cast<int64_t>(y) * a.W;
  const float* f1b = a.f1 + (static_cast<int64_t>(n) * a.C + c0) * HW + static_cast<int64_t>(y) * a.W;
  const float qnan = __int_as_float(0x7fffffff);
  // the thread's own pixels: f0[c, x] (df0) and f1[c, x] (df1)
  float a0[kBPX], b0[kBPX], acc0[kBPX], acc1[kBPX];
#pragma unroll
  for (int i = 0; i < kBPX; ++i) {
    const int x = x0 + 4 * w + i;
    const bool ok = c < a.C && x < a.W;
    a0[i] = ok ? __ldg(f0b + lane * HW + x) : 0.0f;
    b0[i] = ok ? __ldg(f1b + lane * HW + x) : 0.0f;
    acc0[i] = 0.0f;
    acc1[i] = 0.0f;
  }
  // stage chunk ci into buffer ci & 1: cp.async for what lies inside the
  // image and the disparity range, plain stores of the fill values
  const int nchunk = (a.max_disp - a.min_disp) / kBDC + 1;
  auto stage = [&](int ci) {
    const int b = ci & 1;
    const int d0 = a.min_disp + ci * kBDC;
    const int i0 = d0 - a.min_disp;
    const int nd = min(kBDC, a.max_disp - d0 + 1);
    for (int e = tid; e < kBCH * kBFS; e += 256) {
      const int cc = e / kBFS, k = e - cc * kBFS;
      const bool cok = c0 + cc < a.C;
      const int xa = x0 - d0 - (kBDC - 1) + k, xb = x0 + d0 + k;
      if (cok && xa >= 0 && xa < a.W) cp_async4(&f1s[b][e], f1b + cc * HW + xa);
      else f1s[b][e] = qnan;
      if (cok && xb >= 0 && xb < a.W) cp_async4(&f0s[b][e], f0b + cc * HW + xb);
      else f0s[b][e] = qnan;
    }
    for (int e = tid; e < kBDC * kBX; e += 256) {
      const int dd = e / kBX, x = e - dd * kBX;
      const int xa = x0 + x, xd = x0 + x + d0 + dd;
      if (dd < nd && xa < a.W) cp_async4(&gA[b][e], grow + static_cast<int64_t>(xa) * a.D + i0 + dd);
      else gA[b][e] = 0.0f;
      if (dd < nd && xd >= 0 && xd < a.W) cp_async4(&gD[b][e], grow + static_cast<int64_t>(xd) * a.D + i0 + dd);
      else gD[b][e] = 0.0f;
    }
    cp_async_commit();
  };
  stage(0);
  for (int ci = 0; ci < nchunk; ++ci) {
    const int b = ci & 1;
    if (ci + 1 < nchunk) {
      stage(ci + 1);  // buffer (ci + 1) & 1 was last read by chunk ci - 1, before its closing barrier
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const float* F1 = f1s[b] + lane * kBFS + 4 * w + (kBDC - 1);  // F1[i - dd] = f1[c, x0 + 4w + i - (d0 + dd)]
    const float* F0 = f0s[b] + lane * kBFS + 4 * w;               // F0[i + dd] = f0[c, x0 + 4w + i + (d0 + dd)]
    float v1[kBPX], v0[kBPX];
#pragma unroll
    for (int i = 0; i < kBPX; ++i) {
      v1[i] = F1[i];
      v0[i] = F0[i];
    }
#pragma unroll
    for (int dd = 0; dd < kBDC; ++dd) {
      if (dd > 0) {
#pragma unroll
        for (int i = kBPX - 1; i > 0; --i) v1[i] = v1[i - 1];
        v1[0] = F1[-dd];
#pragma unroll
        for (int i = 0; i < kBPX - 1; ++i) v0[i] = v0[i + 1];
        v0[kBPX - 1] = F0[kBPX - 1 + dd];
      }
      const float4 ga = *reinterpret_cast<const float4*>(gA[b] + dd * kBX + 4 * w);
      const float4 gd = *reinterpret_cast<const float4*>(gD[b] + dd * kBX + 4 * w);
      const float gav[4] = {ga.x, ga.y, ga.z, ga.w};
      const float gdv[4] = {gd.x, gd.y, gd.z, gd.w};
#pragma unroll
      for (int i = 0; i < kBPX; ++i) {
        sad_term<false>(acc0[i], __fsub_rn(a0[i], v1[i]), gav[i]);
        sad_term<true>(acc1[i], __fsub_rn(v0[i], b0[i]), gdv[i]);
      }
    }
    __syncthreads();  // buffer b is restaged by chunk ci + 2
  }
  if (c >= a.C || c >= a.channel_limit) return;
#pragma unroll
  for (int i = 0; i < kBPX; ++i) {
    const int x = x0 + 4 * w + i;
    if (x >= a.W) continue;
    const int64_t o = (static_cast<int64_t>(n) * a.C + c) * HW + static_cast<int64_t>(y) * a.W + x;
    a.df0[o] = acc0[i];
    a.df1[o] = acc1[i];
  }
}

}  // namespace
}  // namespace bpl

using namespace bpl;

extern "C" int bpl_sad_volume_depth(int min_disp, int max_disp, float step) {
  if (!(step > 0.0f)) return -1;
  return static_cast<int>(static_cast<float>(max_disp - min_disp + 1) / step);
}

extern "C" int bpl_sad_forward(const float* f0, const float* f1, float* out, int B, int C, int H, int W,
                               int min_disp, int max_disp, float step, void* stream) {
  BPL_TRACE("bpl_sad_forward");
  BPL_REQUIRE(f0 && f1 && out, "sad_forward: null pointer");
  BPL_REQUIRE(B >= 1 && C >= 1 && H >= 1 && W >= 1, "sad_forward: bad shape");
  BPL_REQUIRE(step > 0.0f, "sad_forward: step must be > 0");
  const int D = bpl_sad_volume_depth(min_disp, max_disp, step);
  BPL_REQUIRE(D >= 1, "sad_forward: empty disparity range");
  SadArgs a{f0, f1, out, B, C, H, W, D, min_disp, step, step == 1.0f ? 1 : 0, 0, 0};
  int lo = 1 << 30, hi = -(1 << 30);
  for (int di = 0; di < D; ++di) {
    const int d = a.unit_step ? di + min_disp
                              : static_cast<int>(static_cast<float>(di) * step + static_cast<float>(min_disp));
    lo = std::min(lo, d);
    hi = std::max(hi, d);
  }
  // for fractional steps the host's float rounding may differ from the
  // device's by one: widen the staged span by one on each side
  a.dlo = a.unit_step ? lo : lo - 1;
  a.dhi = a.unit_step ? hi : hi + 1;
  BPL_REQUIRE(a.dhi - a.dlo <= 4096, "sad_forward: disparity span %d too large", a.dhi - a.dlo);
  const int ndg = (D + kPD - 1) / kPD;
  const int threads = ndg * kPXG;
  BPL_REQUIRE(threads <= 1024, "sad_forward: D=%d too large (at most %d disparities)", D, 1024 / (kTX / kPX) * kPD);
  const int span = kTX + (a.dhi - a.dlo);
  const int pad = a.unit_step ? sad_pad(a.dhi, a.dlo) : 0;
  const size_t smem = 2 * sizeof(float) * kCChunk * (kTX + ((pad + span + 3) & ~3));  // two chunk buffers
  BPL_REQUIRE(static_cast<int>(smem) <= max_smem_optin(), "sad_forward: disparity span too large");
  auto launch = [&](auto kern) -> int {
    if (smem > 48 * 1024)
      BPL_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)),
                   "cudaFuncSetAttribute");
    dim3 grid((W + kTX - 1) / kTX, H, B);
    kern<<<grid, threads, smem, as_stream(stream)>>>(a);
    BPL_CUDA_TRY(cudaGetLastError(), "sad_forward launch");
    return BPL_OK;
  };
  if (threads <= 256) return launch(sad_forward_kernel<256, 3>);
  if (threads <= 384) return launch(sad_forward_kernel<384, 2>);
  return launch(sad_forward_kernel<512, 1>);
}

extern "C" int bpl_sad_backward(const float* f0, const float* f1, const float* in_grad, float* df0, float* df1,
                                int B, int C, int H, int W, int min_disp, int max_disp, int reference_channel_limit,
                                void* stream) {
  BPL_TRACE("bpl_sad_backward");
  BPL_REQUIRE(f0 && f1 && in_grad && df0 && df1, "sad_backward: null pointer");
  BPL_REQUIRE(B >= 1 && C >= 1 && H >= 1 && W >= 1 && max_disp >= min_disp, "sad_backward: bad shape");
  const int D = max_disp - min_disp + 1;
  SadBwdArgs a{f0, f1, in_grad, df0, df1, B, C, H, W, D, min_disp, max_disp, C};
  // the reference launch covers only 4*ceil(D/4) channels (stereo_sad_kernel.cu:152-157)
  if (reference_channel_limit) a.channel_limit = std::min(C, 4 * ((D + 3) / 4));
  BPL_CUDA_TRY(cudaMemsetAsync(df0, 0, sizeof(float) * B * C * H * W, as_stream(stream)), "sad_backward: memset");
  BPL_CUDA_TRY(cudaMemsetAsync(df1, 0, sizeof(float) * B * C * H * W, as_stream(stream)), "sad_backward: memset");
  BPL_REQUIRE(static_cast<int64_t>(B) * ((C + kBCH - 1) / kBCH) <= 65535 && H <= 65535, "sad_backward: grid too large");
  dim3 grid((W + kBX - 1) / kBX, H, B * ((C + kBCH - 1) / kBCH));
  sad_backward_kernel<<<grid, 256, 0, as_stream(stream)>>>(a);
  BPL_CUDA_TRY(cudaGetLastError(), "sad_backward launch");
  return BPL_OK;
}

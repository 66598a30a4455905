// Correctly rounded exp and log for the message normalisation, in FP32
// arithmetic.
//
// The reference normalises every message with exp and log evaluated in double
// precision and rounded to float (ops/lbp_stereo/src/lbp_min_sum_kernel.cu:167,
// :180-181).  GB300's FP64 rate is a small fraction of its FP32 rate, so
// evaluating one double exp per message label makes the kernel FP64-bound.
// Here exp(x) and log(s) are evaluated in float-float arithmetic (about 2^-44
// relative error) with table-driven argument reduction after
//   P. T. P. Tang, "Table-driven implementation of the exponential function
//   in IEEE floating-point arithmetic", ACM TOMS 15(2), 1989, and
//   P. T. P. Tang, "Table-driven implementation of the logarithm function in
//   IEEE floating-point arithmetic", ACM TOMS 16(4), 1990,
// then rounded to float.  When the float-float value lies so close to a
// rounding boundary that the rounding cannot be decided from it (about one
// evaluation in 10^4-10^5), the reference's own double-precision expression is
// evaluated instead (Ziv's strategy).  Either way the float result equals the
// reference's (float)exp((double)x) / (float)log((double)s).
//
// Tables (2^(j/64) and log(1+j/64) as float-float pairs) are computed at
// compile time from power series in double precision.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define BPL_HD __device__ __forceinline__
#else
#define BPL_HD inline
#include <cmath>
#include <cstring>
#endif

namespace bpl {
namespace crm {

// ---------------------------------------------------------------------------
// compile-time tables
constexpr double kLn2 = 0.69314718055994530941723212145818;

constexpr double cx_exp(double y) {
  // exp(y) for 0 <= y < 0.7 by its Taylor series (terms decrease fast)
  double term = 1.0, sum = 1.0;
  for (int k = 1; k < 30; ++k) {
    term = term * y / k;
    sum += term;
  }
  return sum;
}

constexpr double cx_log(double x) {
  // log(x) for x in [1, 2] as 2*atanh((x-1)/(x+1))
  const double z = (x - 1.0) / (x + 1.0);
  const double z2 = z * z;
  double p = z, sum = 0.0;
  for (int k = 0; k < 40; ++k) {
    sum += p / (2 * k + 1);
    p *= z2;
  }
  return 2.0 * sum;
}

struct Tables {
  float exp_hi[64], exp_lo[64];  // 2^(j/64)
  float log_hi[65], log_lo[65];  // log(1 + j/64)
  float inv[65];                 // RN(1 / (1 + j/64))
};

constexpr Tables make_tables() {
  Tables t{};
  for (int j = 0; j < 64; ++j) {
    const double v = cx_exp(kLn2 * j / 64.0);
    t.exp_hi[j] = static_cast<float>(v);
    t.exp_lo[j] = static_cast<float>(v - static_cast<double>(t.exp_hi[j]));
  }
  for (int j = 0; j <= 64; ++j) {
    const double F = 1.0 + j / 64.0;
    const double v = cx_log(F);
    t.log_hi[j] = static_cast<float>(v);
    t.log_lo[j] = static_cast<float>(v - static_cast<double>(t.log_hi[j]));
    t.inv[j] = static_cast<float>(1.0 / F);
  }
  return t;
}

#if defined(__CUDACC__)
// Used for the (warp-uniform) log lookups and as the source of the per-block
// shared-memory copy of the exp table (lane-varying lookups).
__constant__ constexpr Tables kTab = make_tables();
#else
constexpr Tables kTab = make_tables();
#endif

// ln2/64 and ln2 split so that the leading parts times small integers are
// exact: ln2/64 = C_hi + C_mid + C_lo (C_hi = 1420 * 2^-17),
// ln2 = L_hi + L_mid + L_lo (L_hi and L_mid with 16 significant bits).
// Values from a 60-digit evaluation of ln 2.
constexpr float kC_hi = 0.010833740234375f;
constexpr float kC_mid = -3.3155381515825866e-06f;
constexpr float kC_lo = 2.572804640231345e-14f;
constexpr float kL_hi = 0.693145751953125f;
constexpr float kL_mid = 1.4286197256296873e-06f;
constexpr float kL_lo = -1.2905320041778356e-11f;

// ---------------------------------------------------------------------------
// exact float transforms (explicit rounding: no contraction)
#if defined(__CUDACC__)
BPL_HD float add_(float a, float b) { return __fadd_rn(a, b); }
BPL_HD float sub_(float a, float b) { return __fsub_rn(a, b); }
BPL_HD float mul_(float a, float b) { return __fmul_rn(a, b); }
BPL_HD float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
BPL_HD int f2i(float f) { return __float_as_int(f); }
BPL_HD float i2f(int i) { return __int_as_float(i); }
#else
inline float add_(float a, float b) { volatile float r = a + b; return r; }
inline float sub_(float a, float b) { volatile float r = a - b; return r; }
inline float mul_(float a, float b) { volatile float r = a * b; return r; }
inline float fma_(float a, float b, float c) { return std::fmaf(a, b, c); }
inline int f2i(float f) { int i; std::memcpy(&i, &f, 4); return i; }
inline float i2f(int i) { float f; std::memcpy(&f, &i, 4); return f; }
#endif

BPL_HD void two_sum(float a, float b, float& s, float& e) {
  s = add_(a, b);
  const float bb = sub_(s, a);
  e = add_(sub_(a, sub_(s, bb)), sub_(b, bb));
}

BPL_HD void fast_two_sum(float a, float b, float& s, float& e) {  // |a| >= |b|
  s = add_(a, b);
  e = sub_(b, sub_(s, a));
}

// half the distance to the next float below/above the normal float z, on the
// side of the residual d (smaller below an exact power of two)
BPL_HD float half_ulp_side(float z, float d) {
  const int b = f2i(z) & 0x7fffffff;
  const int ex = b & 0x7f800000;
  float h = i2f(ex - (24 << 23));  // 2^(e-24) = ulp/2
  if ((b & 0x007fffff) == 0 && ((d < 0.0f) == (z > 0.0f))) h = mul_(h, 0.5f);
  return h;
}

// exp(x) rounded to float; returns false (ambiguous or out of the fast range)
// when the caller must evaluate the reference expression instead.
BPL_HD bool exp_fast(float x, float& out, const float* exp_hi = kTab.exp_hi, const float* exp_lo = kTab.exp_lo) {
  if (!(x > -87.0f && x < 88.0f)) return false;
  // N = rint(x * 64/ln2) by the 1.5 * 2^23 shift: |x * 64/ln2| < 2^13, so the
  // sum lies in [2^23, 2^24), where the float spacing is 1 and the addition
  // rounds to the nearest integer (ties to even, as rint); n is read from
  // the sum's bits (no float-to-int conversion on the chain)
  const float tN = add_(mul_(x, 92.332482616893656f), 12582912.0f);  // 64/ln2, 1.5 * 2^23
  const float N = sub_(tN, 12582912.0f);                              // exact
  const int n = f2i(tN) - 0x4b400000;
  const int j = n & 63;
  const int m = n >> 6;
  // r = x - N * ln2/64 as a float-float (rh, rl)
  const float r1 = fma_(-N, kC_hi, x);                   // exact
  const float p2 = mul_(N, kC_mid);
  const float p2e = fma_(N, kC_mid, -p2);
  float s, se;
  two_sum(r1, -p2, s, se);
  float rl = sub_(sub_(se, p2e), mul_(N, kC_lo));
  float rh;
  two_sum(s, rl, rh, rl);
  // expm1(r) = a + tail
  const float sq = mul_(rh, rh);
  const float sqe = fma_(rh, rh, -sq);
  float a, ae;
  fast_two_sum(rh, mul_(0.5f, sq), a, ae);
  const float poly = mul_(mul_(rh, sq), fma_(rh, fma_(rh, 0.0083333333333333333f, 0.041666666666666667f),
                                             0.16666666666666667f));
  const float tail = add_(add_(add_(ae, rl), add_(mul_(0.5f, sqe), mul_(rh, rl))), poly);
  // 2^(j/64) * (1 + a + tail)
  const float Th = exp_hi[j], Tl = exp_lo[j];
  const float P = mul_(Th, a);
  const float Pe = fma_(Th, a, -P);
  float y, ye;
  fast_two_sum(Th, P, y, ye);
  const float corr = add_(add_(add_(ye, Pe), mul_(Th, tail)), fma_(Tl, a, Tl));
  const float z = add_(y, corr);
  const float d = add_(sub_(y, z), corr);
  const float err = mul_(z, 9.094947017729282e-13f);  // 2^-40 relative
  const float ad = d < 0.0f ? -d : d;
  if (ad > sub_(half_ulp_side(z, d), err)) return false;
  out = mul_(z, i2f((m + 127) << 23));
  return true;
}

// log(s) rounded to float for a positive float s; false when the caller must
// evaluate the reference expression instead.
BPL_HD bool log_fast(float s, float& out) {
  const int bits = f2i(s);
  if (!(s > 0.0f) || (bits & 0x7f800000) == 0 || (bits & 0x7f800000) == 0x7f800000) return false;
  const int e = ((bits >> 23) & 0xff) - 127;
  const float mnt = i2f((bits & 0x007fffff) | 0x3f800000);
  // j = (int)(64 (mnt - 1) + 0.5) and F = 1 + j/64, both exact, from the
  // mantissa bits m: 64 (mnt - 1) = m 2^-17, so j = (m + 2^16) >> 17 and F
  // has mantissa field j << 17 (j = 64 gives 2.0)
  const int j = ((bits & 0x007fffff) + (1 << 16)) >> 17;
  const float F = i2f(0x3f800000 + (j << 17));
  const float f = sub_(mnt, F);  // exact
  const float inv = kTab.inv[j];
  const float uh = mul_(f, inv);
  const float ul = mul_(fma_(-uh, F, f), inv);
  const float sq = mul_(uh, uh);
  const float sqe = fma_(uh, uh, -sq);
  float a, ae;
  fast_two_sum(uh, mul_(-0.5f, sq), a, ae);
  const float poly = mul_(mul_(uh, sq), fma_(uh, fma_(uh, 0.2f, -0.25f), 0.33333333333333333f));
  const float tail = add_(add_(add_(ae, ul), sub_(mul_(-0.5f, sqe), mul_(uh, ul))), poly);
  const float ef = static_cast<float>(e);
  const float E1 = mul_(ef, kL_hi);   // exact
  const float E2 = mul_(ef, kL_mid);  // exact
  float s1, s1e, s2, s2e;
  two_sum(E1, kTab.log_hi[j], s1, s1e);
  two_sum(s1, a, s2, s2e);
  float s3, s3e;
  two_sum(s2, E2, s3, s3e);
  const float lo = add_(add_(add_(s2e, s1e), s3e), add_(add_(mul_(ef, kL_lo), kTab.log_lo[j]), tail));
  float z, d;
  two_sum(s3, lo, z, d);
  const float az = z < 0.0f ? -z : z;
  const float err = add_(7.105427357601002e-15f, mul_(az, 5.684341886080802e-14f));  // 2^-47 + 2^-44|z|
  const float ad = d < 0.0f ? -d : d;
  if (z == 0.0f || ad > sub_(half_ulp_side(z, d), err)) return false;
  out = z;
  return true;
}

}  // namespace crm
}  // namespace bpl

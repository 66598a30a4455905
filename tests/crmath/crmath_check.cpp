// Host check of the correctly rounded exp/log used by the LBP kernels
// (bp-layers_gb300/csrc/bpl_crmath.cuh): whenever the fast path returns a
// value it must equal the reference expression (float)exp((double)x) /
// (float)log((double)s).  Usage: crmath_check N_RANDOM SEED
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "../../bp-layers_gb300/csrc/bpl_crmath.cuh"

int main(int argc, char** argv) {
  const long n = argc > 1 ? atol(argv[1]) : 1000000;
  std::mt19937_64 rng(argc > 2 ? atol(argv[2]) : 1);
  long bad_e = 0, slow_e = 0, bad_l = 0, slow_l = 0, tot_e = 0, tot_l = 0;
  std::uniform_real_distribution<double> ue(-87.5, 88.5), un(-40.0, 2.0);
  std::uniform_int_distribution<uint32_t> bits(0x00800000u, 0x7f7fffffu);
  auto chk_e = [&](float x) {
    float y;
    ++tot_e;
    if (!bpl::crm::exp_fast(x, y)) { ++slow_e; return; }
    const float r = static_cast<float>(std::exp(static_cast<double>(x)));
    if (y != r) { if (bad_e < 10) printf("exp mismatch x=%.9g fast=%.9g ref=%.9g\n", x, y, r); ++bad_e; }
  };
  auto chk_l = [&](float s) {
    float y;
    ++tot_l;
    if (!bpl::crm::log_fast(s, y)) { ++slow_l; return; }
    const float r = static_cast<float>(std::log(static_cast<double>(s)));
    if (y != r) { if (bad_l < 10) printf("log mismatch s=%.9g fast=%.9g ref=%.9g\n", s, y, r); ++bad_l; }
  };
  for (long i = 0; i < n; ++i) {
    chk_e(static_cast<float>(ue(rng)));
    chk_e(static_cast<float>(un(rng)));
    uint32_t b = bits(rng);
    float s;
    std::memcpy(&s, &b, 4);
    chk_l(s);
  }
  // every float in [-32, -8] with a stride, and around 0 / powers of two
  for (float x = -32.0f; x < -8.0f; x = std::nextafter(x, 0.0f) + 1e-6f) chk_e(x);
  for (int k = -126; k < 127; ++k) {
    float p = std::ldexp(1.0f, k);
    chk_l(p); chk_l(std::nextafter(p, 0.0f)); chk_l(std::nextafter(p, 1e30f));
  }
  for (float x : {0.0f, -0.0f, 1e-8f, -1e-8f, 1e-30f, 88.0f, -87.0f, 0.5f, -0.5f}) chk_e(x);
  printf("exp: %ld checked, %ld slow path, %ld mismatches\n", tot_e, slow_e, bad_e);
  printf("log: %ld checked, %ld slow path, %ld mismatches\n", tot_l, slow_l, bad_l);
  return (bad_e || bad_l) ? 1 : 0;
}

// Compares the restated acosf kinds of tmc_gb300/csrc/libm_acosf.h (what the GPU triangle split
// uses) with the platform C library's acosf, which the reference's minAngle calls through std::acos,
// bit for bit over the floats of [-1, 1].
//
//   acos_check [stride] [threads]
// checks every stride-th float magnitude (stride 1: all 2,130,706,434 values, both signs) against
// both fdlibm kinds and prints "ok <kind> <count>" for the kind that matches all of them, or the
// mismatch counts of both kinds.
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include <atomic>
#include <cmath>
#include <thread>
#include <vector>

#include "../../tmc_gb300/csrc/libm_acosf.h"

int main(int argc, char** argv) {
  using tmc::libm::float_to_bits;
  const uint32_t stride = argc > 1 ? (uint32_t)strtoul(argv[1], nullptr, 10) : 1u;
  const int threads = argc > 2 ? atoi(argv[2]) : 1;
  const uint32_t top = 0x3f800000u;  // 1.0f
  std::atomic<uint64_t> checked{0}, bad_sep{0}, bad_fused{0};
  auto work = [&](int t) {
    uint64_t n = 0, bs = 0, bf = 0;
    for (uint64_t u = (uint64_t)t * stride; u <= top; u += (uint64_t)stride * threads) {
      for (uint32_t sign = 0; sign < 2; sign++) {
        const float x = tmc::libm::bits_to_float((uint32_t)u | (sign << 31));
        const uint32_t want = float_to_bits(std::acos(x));
        n++;
        bs += float_to_bits(tmc::libm::acosf_fdlibm<false>(x)) != want;
        bf += float_to_bits(tmc::libm::acosf_fdlibm<true>(x)) != want;
      }
    }
    checked += n;
    bad_sep += bs;
    bad_fused += bf;
  };
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; t++) pool.emplace_back(work, t);
  for (auto& th : pool) th.join();
  const unsigned long long n = checked.load();
  if (bad_sep.load() == 0) {
    printf("ok separate %llu\n", n);
  } else if (bad_fused.load() == 0) {
    printf("ok fused %llu\n", n);
  } else {
    printf("no kind matches: separate %llu, fused %llu mismatches of %llu\n", (unsigned long long)bad_sep.load(),
           (unsigned long long)bad_fused.load(), n);
    return 1;
  }
  return 0;
}

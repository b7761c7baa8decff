// Compares tmc::libm::acosf (tmc_gb300/csrc/libm_acosf.h, the restatement the GPU triangle split
// uses) with the platform C library's acosf, bit for bit, over the floats of [-1, 1].
//
//   acos_check [stride] [threads]
// checks every stride-th float magnitude (stride 1: all 2,130,706,434 values, both signs) on the
// given number of threads, and prints "ok <count>" or the first mismatches.
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include <atomic>
#include <thread>
#include <vector>

#include "../../tmc_gb300/csrc/libm_acosf.h"

int main(int argc, char** argv) {
  const uint32_t stride = argc > 1 ? (uint32_t)strtoul(argv[1], nullptr, 10) : 1u;
  const int threads = argc > 2 ? atoi(argv[2]) : 1;
  const uint32_t top = 0x3f800000u;  // 1.0f
  std::atomic<uint64_t> checked{0}, bad{0};
  auto work = [&](int t) {
    uint64_t n = 0, b = 0;
    for (uint64_t u = (uint64_t)t * stride; u <= top; u += (uint64_t)stride * threads) {
      for (uint32_t sign = 0; sign < 2; sign++) {
        const float x = tmc::libm::bits_to_float((uint32_t)u | (sign << 31));
        const float want = ::acosf(x), got = tmc::libm::acosf(x);
        n++;
        if (tmc::libm::float_to_bits(want) != tmc::libm::float_to_bits(got)) {
          if (b < 3) printf("x=%a libc=%a restated=%a\n", x, want, got);
          b++;
        }
      }
    }
    checked += n;
    bad += b;
  };
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; t++) pool.emplace_back(work, t);
  for (auto& th : pool) th.join();
  if (bad.load()) {
    printf("mismatches %llu of %llu\n", (unsigned long long)bad.load(), (unsigned long long)checked.load());
    return 1;
  }
  printf("ok %llu\n", (unsigned long long)checked.load());
  return 0;
}

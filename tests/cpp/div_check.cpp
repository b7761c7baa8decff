// Host check of Div32 (tmc_gb300/csrc/common.cuh), the invariant-divisor division that splits cell
// indices in every cell kernel: q = n / d exactly, for every divisor 1..70000 (grid axes are at most
// 65535 points) with the dividends around each multiple boundary and spread over the whole 32-bit
// range, and for random divisors up to 2^32 - 1.  Prints "ok" or the first mismatch.
#include <cstdio>
#include <cstdint>
#include <random>

#include "../../tmc_gb300/csrc/common.cuh"

static bool check(uint32_t d, uint32_t n) {
  tmc::Div32 q;
  q.init(d);
  const uint32_t got = q.div(n), want = n / d;
  if (got != want) {
    std::printf("mismatch: %u / %u = %u, Div32 gives %u\n", n, d, want, got);
    return false;
  }
  return true;
}

int main() {
  std::mt19937_64 rng(12345);
  for (uint32_t d = 1; d <= 70000; d++) {
    tmc::Div32 q;
    q.init(d);
    const uint32_t edges[] = {0u, 1u, d - 1, d, d + 1, 2 * d - 1, 2 * d, 0xffffffffu, 0xfffffffeu, 0x80000000u,
                              0x7fffffffu, (0xffffffffu / d) * d, (0xffffffffu / d) * d - 1};
    for (uint32_t n : edges)
      if (q.div(n) != n / d) return check(d, n) ? 0 : 1;
    for (int r = 0; r < 200; r++) {
      const uint32_t n = (uint32_t)rng();
      if (q.div(n) != n / d) return check(d, n) ? 0 : 1;
      const uint32_t b = (uint32_t)(rng() % (0xffffffffu / d)) * d;  // a multiple and its neighbours
      if (q.div(b) != b / d || q.div(b - 1) != (b - 1) / d || q.div(b + d - 1) != (b + d - 1) / d)
        return (check(d, b) && check(d, b - 1) && check(d, b + d - 1)) ? 0 : 1;
    }
  }
  for (int r = 0; r < 200000; r++) {
    const uint32_t d = (uint32_t)(rng() | 1u) >> (rng() % 32);
    const uint32_t n = (uint32_t)rng();
    if (d == 0) continue;
    if (!check(d, n) || !check(d, d) || !check(d, d - 1) || !check(d, 0xffffffffu)) return 1;
  }
  for (uint32_t s = 0; s < 32; s++) {  // powers of two and their neighbours
    const uint32_t p = 1u << s;
    for (uint32_t d : {p - 1, p, p + 1})
      if (d && (!check(d, 0xffffffffu) || !check(d, p) || !check(d, 12345678u))) return 1;
  }
  std::printf("ok\n");
  return 0;
}

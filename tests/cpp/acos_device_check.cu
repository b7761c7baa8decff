// The acosf restatement the GPU triangle split uses, evaluated on the GPU for every float of [-1, 1]
// and compared with this host's C library acosf (what the reference's std::acos calls here), bit
// for bit.  The kind is the one the library selects at run time (host_acosf_kind); the two fdlibm
// kinds must match exactly.  Prints "ok <kind> <count>" or the first mismatches.
//
// Built like the library's device code: nvcc -gencode arch=compute_103a,code=sm_103a -O3
// -fmad=false -Xcompiler -ffp-contract=off.
#include <stdint.h>
#include <stdio.h>

#include <atomic>
#include <cmath>
#include <thread>
#include <vector>

#include "../../tmc_gb300/csrc/libm_acosf.h"

// out[2 i] = acos(+x), out[2 i + 1] = acos(-x) for the float magnitude bits first + i, i < n
__global__ void eval_kernel(uint32_t first, uint32_t n, int kind, float* out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t u = first + i;
  out[2 * (size_t)i] = tmc::libm::acosf_kind(tmc::libm::bits_to_float(u), kind);
  out[2 * (size_t)i + 1] = tmc::libm::acosf_kind(tmc::libm::bits_to_float(u | 0x80000000u), kind);
}

int main() {
  const int kind = tmc::libm::host_acosf_kind();
  const uint32_t top = 0x3f800000u, chunk = 1u << 25;
  float* d = nullptr;
  if (cudaMalloc(&d, 2 * (size_t)chunk * sizeof(float)) != cudaSuccess) return 2;
  std::vector<float> h(2 * (size_t)chunk);
  const int threads = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  std::atomic<uint64_t> bad{0};
  uint64_t checked = 0;
  for (uint64_t first = 0; first <= top; first += chunk) {
    const uint32_t n = (uint32_t)std::min<uint64_t>(chunk, top + 1 - first);
    eval_kernel<<<(n + 255) / 256, 256>>>((uint32_t)first, n, kind, d);
    if (cudaMemcpy(h.data(), d, 2 * (size_t)n * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) return 2;
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; t++)
      pool.emplace_back([&, t] {
        uint64_t b = 0;
        for (uint32_t i = t; i < n; i += threads)
          for (int sign = 0; sign < 2; sign++) {
            const float x = tmc::libm::bits_to_float(((uint32_t)first + i) | (sign ? 0x80000000u : 0u));
            const float want = std::acos(x), got = h[2 * (size_t)i + sign];
            if (tmc::libm::float_to_bits(want) != tmc::libm::float_to_bits(got)) {
              if (b < 2) printf("x=%a host=%a device=%a\n", x, want, got);
              b++;
            }
          }
        bad += b;
      });
    for (auto& th : pool) th.join();
    checked += 2 * (uint64_t)n;
  }
  cudaFree(d);
  const char* names[] = {"separate", "fused", "correct"};
  if (bad.load()) {
    printf("kind %s: %llu mismatches of %llu\n", names[kind], (unsigned long long)bad.load(),
           (unsigned long long)checked);
    return 1;
  }
  printf("ok %s %llu\n", names[kind], (unsigned long long)checked);
  return 0;
}

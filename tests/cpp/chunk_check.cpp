// Host check of slot_chunk (tmc_gb300/csrc/common.cuh), which hands the listed-cell walks of the TMC
// emission and DMC quad kernels their chunks of 32 slots: for every tile count checked, chunks
// 0 .. tiles * 64 - 1 must cover each (tile, part) exactly once, with first = tile * 2048 + part * 32,
// and take the windows of kChunkWindow tiles in order.  Prints "ok" or the first violation.
#include <cstdio>
#include <cstdint>
#include <vector>

#include "../../tmc_gb300/csrc/common.cuh"
#include "../../tmc_gb300/csrc/scan.cuh"

static bool check(int64_t tiles) {
  const int64_t parts = tmc::kScanTile / 32, chunks = tiles * parts;
  std::vector<uint8_t> seen((size_t)chunks, 0);
  for (int64_t q = 0; q < chunks; q++) {
    int64_t tile = -1;
    uint32_t first = 0;
    tmc::slot_chunk(q, tiles, tile, first);
    const int64_t part = ((int64_t)first - tile * tmc::kScanTile) / 32;
    const bool ok = tile >= 0 && tile < tiles && part >= 0 && part < parts &&
                    (int64_t)first == tile * tmc::kScanTile + part * 32 &&
                    tile / tmc::kChunkWindow == q / (tmc::kChunkWindow * parts) && !seen[(size_t)(tile * parts + part)];
    if (!ok) {
      std::printf("tiles %lld: chunk %lld -> tile %lld, first %u\n", (long long)tiles, (long long)q, (long long)tile,
                  first);
      return false;
    }
    seen[(size_t)(tile * parts + part)] = 1;
  }
  return true;
}

int main() {
  for (int64_t t = 1; t <= 1100; t++)
    if (!check(t)) return 1;
  const int64_t big[] = {tmc::kChunkWindow * 3, tmc::kChunkWindow * 3 + 1, 65536, 65539, 524288};
  for (int64_t t : big)
    if (!check(t)) return 1;
  std::printf("ok\n");
  return 0;
}

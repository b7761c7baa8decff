// Access to a context's device, stream, error message and launch counter for C entry points that
// live outside runtime.cu.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/tmc_gb300.h"

namespace tmc {
int ctx_device(const tmc_ctx* ctx);
cudaStream_t ctx_stream(const tmc_ctx* ctx);
// stores msg as the context's last error and returns s
tmc_status ctx_fail(tmc_ctx* ctx, tmc_status s, const char* msg);
void ctx_count_launches(tmc_ctx* ctx, int64_t n);
}  // namespace tmc

// Internal interface: topologically correct Marching Cubes kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

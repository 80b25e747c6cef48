/* ref_launch_pre.h -- CUDA vector types ahead of the reference sources
 * (TEST INFRASTRUCTURE ONLY). */
#pragma once
#include <cuda_runtime.h>

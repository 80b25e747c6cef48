/*
 * shim.h -- forced include that lets the reference's CUDA kernel sources compile
 * as host C++ (TEST INFRASTRUCTURE: builds oracle/_ref, never part of the
 * product).  With __DEVICE_EMULATION__ defined the reference's FETCH macro reads
 * arrays directly (DamBreak.Core/fluid_kernel.cuh:4-12), so the kernels become
 * plain functions; the launcher runs every (block, thread) pair in order.
 */
#pragma once
#include <cuda_runtime.h>
#include <cmath>
#include <cstdio>
#include <cstdint>

struct cmref_dim3 { unsigned x, y, z; };
extern thread_local cmref_dim3 threadIdx, blockIdx, blockDim;

/* __umul24/__mul24: product of the low 24 bits of each operand */
static inline unsigned __umul24(unsigned a, unsigned b) { return (a & 0xffffffu) * (b & 0xffffffu); }
static inline int __mul24(int a, int b)
{
    return (int)(((unsigned)a & 0xffffffu) * ((unsigned)b & 0xffffffu));
}
/* Threads of a block run in index order, so the only barrier in the reference
 * (the shared hash halo of reorderDataAndFindCellStartD) sees every value it
 * reads already written by the thread before it. */
#define __syncthreads() do { } while (0)

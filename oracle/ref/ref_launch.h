/*
 * ref_launch.h -- headless CPU launcher for the reference's own CUDA kernels
 * (TEST INFRASTRUCTURE: builds oracle/_ref, never part of the product).
 *
 * The reference's host classes need GL/GLUT/GLEW and cutil, which do not exist
 * here, so each ref_*.cpp replays the stage sequence of the reference update()
 * itself, calling the reference kernels through cmref_launch().  The sort stage
 * (thrust::sort_by_key in the reference) is std::stable_sort on the (hash, index)
 * pairs: both are stable ascending key sorts, so the results are identical.
 */
#pragma once
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "../../include/cmag_sph.h"

thread_local cmref_dim3 threadIdx, blockIdx, blockDim;

/* run kernel body f for n threads in blocks of `block`, block by block and thread
 * by thread (computeGridSize: numThreads = min(block, n), fluidSystem.cu:25-28) */
template <class F>
static void cmref_launch(unsigned n, unsigned block, F f)
{
    if (n == 0) return;
    unsigned threads = std::min(block, n);
    unsigned blocks = (n + threads - 1) / threads;
    blockDim = {threads, 1, 1};
    for (unsigned b = 0; b < blocks; ++b) {
        blockIdx = {b, 0, 0};
        for (unsigned t = 0; t < threads; ++t) {
            threadIdx = {t, 0, 0};
            f();
        }
    }
}

static void cmref_sort(unsigned *hash, unsigned *idx, unsigned n)
{
    std::vector<unsigned> order(n);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(),
                     [&](unsigned a, unsigned b) { return hash[a] < hash[b]; });
    std::vector<unsigned> h(n), v(n);
    for (unsigned i = 0; i < n; ++i) { h[i] = hash[order[i]]; v[i] = idx[order[i]]; }
    std::memcpy(hash, h.data(), sizeof(unsigned) * n);
    std::memcpy(idx, v.data(), sizeof(unsigned) * n);
}

static uint3 cmref_u3(const uint32_t *a) { return make_uint3(a[0], a[1], a[2]); }
static float3 cmref_f3(const float *a) { return make_float3(a[0], a[1], a[2]); }

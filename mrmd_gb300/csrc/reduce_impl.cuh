// Deterministic sums of K doubles over a grid.
//
// Every block reduces its threads' values by a fixed shuffle tree and stores
// one partial; the last block to finish (an atomic ticket, no waiting) sums
// the partials, each thread a fixed strided subset in block order followed by
// the same tree.  With a fixed grid and block size the result is the same
// bits on every run, independent of block scheduling.
#pragma once

#include <cstdint>

namespace mrmd_impl
{
// Sum of v over the block; the result is valid in thread 0.  blockDim.x must
// be a multiple of 32 and at most 1024.
template <int K>
__device__ __forceinline__ void block_sum(double (&v)[K])
{
    __shared__ double sh[32][K];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k)
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
    __syncthreads();  // sh may still be read by a previous call
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < K; ++k) sh[warp][k] = v[k];
    __syncthreads();
    if (warp == 0)
    {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int k = 0; k < K; ++k)
        {
            v[k] = lane < nw ? sh[lane][k] : 0.0;
            for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
        }
    }
}

// Grid-wide sum of v written to out[0..K) by the last block.  partial holds
// gridDim.x * K doubles; *ticket is 0 on entry and is reset to 0 by the last
// block, so the pair can be reused by the next launch (also inside a graph).
template <int K>
__device__ __forceinline__ void grid_sum(double (&v)[K], double* partial, unsigned* ticket, double* out)
{
    __shared__ bool isLast;
    block_sum<K>(v);
    if (threadIdx.x == 0)
    {
#pragma unroll
        for (int k = 0; k < K; ++k) partial[(size_t)blockIdx.x * K + k] = v[k];
        __threadfence();
        isLast = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!isLast) return;
    __threadfence();
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = 0.0;
    for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x)
#pragma unroll
        for (int k = 0; k < K; ++k) v[k] += __ldcg(partial + (size_t)b * K + k);
    block_sum<K>(v);
    if (threadIdx.x == 0)
    {
#pragma unroll
        for (int k = 0; k < K; ++k) out[k] = v[k];
        *ticket = 0u;
    }
}
}  // namespace mrmd_impl

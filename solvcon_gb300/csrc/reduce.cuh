#pragma once

/*
 * Warp-shuffle reductions for the per-block partial sums of the conservation
 * totals and the CFL range (min/max of cflo): each warp folds its 32 values
 * with __shfl_down_sync, lane 0 of every warp leaves the warp's result in
 * shared memory, and the first warp folds those.  Lane 0 of warp 0 ends with
 * the block's result.
 */

#include <cuda_runtime.h>

namespace scg
{
namespace red
{

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        v += __shfl_down_sync(0xffffffffu, v, o);
    }
    return v;
}

__device__ __forceinline__ double warp_min(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        v = fmin(v, __shfl_down_sync(0xffffffffu, v, o));
    }
    return v;
}

__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    }
    return v;
}

enum Op
{
    SUM,
    MIN,
    MAX,
};

template <Op OP>
__device__ __forceinline__ double warp_fold(double v)
{
    if constexpr (OP == SUM)
    {
        return warp_sum(v);
    }
    else if constexpr (OP == MIN)
    {
        return warp_min(v);
    }
    else
    {
        return warp_max(v);
    }
}

template <Op OP>
__device__ __forceinline__ double identity()
{
    if constexpr (OP == SUM)
    {
        return 0.0;
    }
    else if constexpr (OP == MIN)
    {
        return 1.79769313486231570815e+308;
    }
    else
    {
        return -1.79769313486231570815e+308;
    }
}

// Block-wide reduction of v (every thread of the block calls it, blockDim.x a
// multiple of 32 and at most 1024); sh is NWARP doubles of shared memory the
// caller owns, free again when the function returns.  The result is valid in
// thread 0.
template <Op OP, int NWARP>
__device__ __forceinline__ double block_fold(double v, double * sh)
{
    int const lane = static_cast<int>(threadIdx.x) & 31;
    int const warp = static_cast<int>(threadIdx.x) >> 5;
    v = warp_fold<OP>(v);
    if (lane == 0)
    {
        sh[warp] = v;
    }
    __syncthreads();
    double r = identity<OP>();
    if (warp == 0)
    {
        r = warp_fold<OP>(lane < NWARP ? sh[lane] : identity<OP>());
    }
    __syncthreads();
    return r;
}

} // namespace red
} // namespace scg

// common.cuh -- shared host/device helpers of the osiris_gb300 library.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/osiris_gb300.h"

namespace osg {

// last error text of the calling thread (osg_last_error)
void set_error(const char *fmt, ...);

#define OSG_CUDA(call)                                                                        \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) {                                                              \
            ::osg::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
            return OSG_ERR_CUDA;                                                              \
        }                                                                                     \
    } while (0)

#define OSG_CHECK(cond, code, ...)                                                            \
    do {                                                                                      \
        if (!(cond)) {                                                                        \
            ::osg::set_error(__VA_ARGS__);                                                    \
            return (code);                                                                    \
        }                                                                                     \
    } while (0)

// Periodic grid with guard cells, reference t_vdf layout: 3 components fastest, then x, y, z;
// size[d] = nx[d] + gcl[d] + gcu[d]; Fortran cell index i (1-based) sits at position
// i - 1 + gcl along its axis.
struct GridDesc {
    int dim;
    int nx[3];
    int gcl[3];
    int gcu[3];
    int size[3];

    __host__ __device__ long npoints() const { return (long)size[0] * size[1] * size[2]; }
    __host__ __device__ long stride(int d) const
    {
        return d == 0 ? 3L : (d == 1 ? 3L * size[0] : 3L * size[0] * size[1]);
    }
};

inline GridDesc make_grid(int dim, const int *nx, const int *gcl, const int *gcu)
{
    GridDesc g;
    g.dim = dim;
    for (int d = 0; d < 3; d++) {
        g.nx[d] = d < dim ? nx[d] : 1;
        g.gcl[d] = d < dim ? gcl[d] : 0;
        g.gcu[d] = d < dim ? gcu[d] : 0;
        g.size[d] = g.nx[d] + g.gcl[d] + g.gcu[d];
    }
    return g;
}

// guard cells the interpolation order needs (source/particles/os-particles.f03:321-360)
inline void guard_cells(int order, int *gl, int *gu)
{
    *gl = order;
    *gu = order + 1;
}

inline unsigned blocks_for(long n, int threads)
{
    long b = (n + threads - 1) / threads;
    return (unsigned)(b < 1 ? 1 : b);
}

// grid-stride loop helper
#define OSG_GRID_LOOP(i, n)                                                                   \
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < (n);                       \
         i += (long)blockDim.x * gridDim.x)

// block-wide double sum; every thread passes its value, thread 0 gets the total
__device__ __forceinline__ double block_sum(double v)
{
    __shared__ double warp_part[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) warp_part[wid] = v;
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    v = (threadIdx.x < nw) ? warp_part[threadIdx.x] : 0.0;
    if (wid == 0) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    }
    __syncthreads();
    return v;
}

// the same in FP32 (for FP32 energy terms; FP64 arithmetic is slow on this GPU)
__device__ __forceinline__ float block_sum_f(float v)
{
    __shared__ float warp_part_f[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) warp_part_f[wid] = v;
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    v = (threadIdx.x < nw) ? warp_part_f[threadIdx.x] : 0.f;
    if (wid == 0) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    }
    __syncthreads();
    return v;
}

} // namespace osg

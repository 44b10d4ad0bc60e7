// Shared device/host definitions of libjetgpu.
//
// Layout in HBM (all i-fastest, index = i + nx*(j + ny*k), matching Jet's
// Array3, include/jet/detail/array_accessor3-inl.h:197-200):
//   * per multigrid level l (resolution n_l = n >> l): float fluid SDF (cells),
//     float u/v/w face weights, float4 matrix rows {center,right,up,front}
//     (16 B/cell, one aligned vector load per cell), FP32 V-cycle vectors x, b
//     and a residual scratch r;
//   * finest level only: the exact FP64 matrix (4 doubles/cell, the
//     reference's FdmMatrix3 bit for bit), FP64 rhs b, FP64 solution x and FP64
//     residual, plus the FP32 (or FP64) Krylov vectors;
//   * a small block of FP64 scalars (dot products, alpha/beta) and the
//     per-block partial sums of the deterministic reductions.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace jg {

constexpr int kThreads = 256;
// Fixed reduction grid: partial sums are reduced in block order, so every
// reduction is deterministic for a given resolution.
constexpr int kMaxRedBlocks = 1024;
constexpr int kRedSlots = 8;

// Device scalars (indices into Ctx::scal).
enum Scalar : int {
    S_RZ = 0,      // r.z of the current iteration
    S_RZ_OLD = 1,  // r.z of the previous iteration
    S_DQ = 2,      // d.q
    S_RR = 3,      // r.r after the update
    S_B64 = 4,     // ||b||^2 (FP64 rhs)
    S_R64 = 5,     // ||b - A x||^2 (FP64 true residual)
    S_MEAN = 6,    // sum used for mean removal
    S_AUX = 7,
    S_COUNT = 16
};

struct Dims {
    int x, y, z;
    __host__ __device__ long count() const { return (long)x * y * z; }
};

__host__ __device__ __forceinline__ long lin(int i, int j, int k, int nx,
                                             int ny) {
    return (long)i + (long)nx * ((long)j + (long)ny * k);
}

// (i, j, k) of linear index c with 32-bit arithmetic (grids have < 2^31
// cells; 64-bit division costs several times more instructions).
__device__ __forceinline__ void cell_ijk(long c, Dims n, int& i, int& j,
                                         int& k) {
    const unsigned cc = (unsigned)c, nx = (unsigned)n.x, ny = (unsigned)n.y;
    const unsigned q = cc / nx;
    i = (int)(cc - q * nx);
    const unsigned r = q / ny;
    j = (int)(q - r * ny);
    k = (int)r;
}

// A scalar field: a constant or a grid sampled with Jet's trilinear rule.
struct FieldDesc {
    int kind;
    double value;
    const double* data;
    int res[3];
    double origin[3];
    double spacing[3];
};

// Grid geometry of a face-centred grid.
struct GridDesc {
    int res[3];
    double spacing[3];
    double origin[3];
};

// Deterministic FP64 block reduction: block sum in a fixed tree order.
template <int NT>
__device__ __forceinline__ double block_sum(double v, double* smem) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) smem[warp] = v;
    __syncthreads();
    double r = 0.0;
    if (warp == 0) {
        r = (lane < NT / 32) ? smem[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1)
            r += __shfl_down_sync(0xffffffffu, r, o);
    }
    __syncthreads();
    return r;  // valid in thread 0
}

// Publishes this block's partial for `slot`; the last block to arrive sums
// all partials in block order and stores the total in scal[target]. No block
// waits on another: the counter only elects who finishes.
template <int NT>
__device__ __forceinline__ void reduce_publish(double partial, int slot,
                                               int target, double* partials,
                                               unsigned* counters,
                                               double* scal, double* smem) {
    __shared__ bool is_last;
    if (threadIdx.x == 0) {
        partials[slot * kMaxRedBlocks + blockIdx.x] = partial;
        __threadfence();
        unsigned done = atomicAdd(&counters[slot], 1u);
        is_last = (done == gridDim.x - 1);
    }
    __syncthreads();
    if (is_last) {
        __threadfence();
        double v = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += NT)
            v += __ldcg(&partials[slot * kMaxRedBlocks + b]);
        v = block_sum<NT>(v, smem);
        if (threadIdx.x == 0) {
            scal[target] = v;
            counters[slot] = 0u;
        }
    }
}

}  // namespace jg

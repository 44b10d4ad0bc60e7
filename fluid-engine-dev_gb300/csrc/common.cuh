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
constexpr int kMaxRedBlocks = 2048;
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
    S_WAIT = 15,   // set to 1 by a kernel whose bounded stage wait ran out
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

// Double-float accumulator: the unevaluated sum hi + lo carries about 48
// significant bits using FP32 instructions only. GB300's FP64 pipe issues a
// small fraction of the FP32 rate, so a per-element (double)a * (double)b
// makes a streaming dot product FP64-issue-bound; here each product is
// split exactly (a*b = p + fma(a, b, -p)) and added with Knuth's TwoSum,
// which keeps the accumulation as accurate as an FP64 one for the lengths
// used (< 2^31 terms). The __f*_rn intrinsics are never contracted into
// FMAs, which TwoSum's error terms rely on. Per thread the pair is turned
// into one double at the end; the cross-thread reduction runs in FP64.
struct DF {
    float hi = 0.0f, lo = 0.0f;
};
__device__ __forceinline__ void df_add(DF& acc, float p, float pe) {
    const float s = __fadd_rn(acc.hi, p);
    const float bb = __fsub_rn(s, acc.hi);
    const float e = __fadd_rn(__fsub_rn(acc.hi, __fsub_rn(s, bb)),
                              __fsub_rn(p, bb));
    const float t = __fadd_rn(e, __fadd_rn(pe, acc.lo));
    acc.hi = __fadd_rn(s, t);
    acc.lo = __fsub_rn(t, __fsub_rn(acc.hi, s));
}
__device__ __forceinline__ void df_add_prod(DF& acc, float a, float b) {
    const float p = __fmul_rn(a, b);
    df_add(acc, p, __fmaf_rn(a, b, -p));
}
__device__ __forceinline__ double df_value(const DF& a) {
    return (double)a.hi + (double)a.lo;
}

// Double-float arithmetic on pairs (hi, lo) with |lo| <= ulp(hi)/2.
__device__ __forceinline__ DF df_renorm(float s, float t) {
    DF r;
    r.hi = __fadd_rn(s, t);
    r.lo = __fsub_rn(t, __fsub_rn(r.hi, s));
    return r;
}
__device__ __forceinline__ DF df_sum(DF a, DF b) {
    const float s = __fadd_rn(a.hi, b.hi);
    const float bb = __fsub_rn(s, a.hi);
    const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)),
                              __fsub_rn(b.hi, bb));
    return df_renorm(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}
// a - (bh + bl) * (xh + xl), dropping the bl * xl term (below 2^-48 |a|).
__device__ __forceinline__ DF df_sub_prod(DF a, float bh, float bl, float xh,
                                          float xl) {
    const float p = __fmul_rn(bh, xh);
    float e = __fmaf_rn(bh, xh, -p);
    e = __fmaf_rn(bh, xl, __fmaf_rn(bl, xh, e));
    DF q;
    q.hi = -p;
    q.lo = -e;
    return df_sum(a, q);
}
__device__ __forceinline__ DF df_add_f(DF a, float e) {
    DF q;
    q.hi = e;
    q.lo = 0.0f;
    return df_sum(a, q);
}

// Opaque moves between a double and its two 32-bit words. Bit tests written
// as plain integer code on __double_as_longlong are recognised by the
// compiler and turned back into FP64 compares and conversions, which GB300
// issues at a small fraction of the integer rate; moving through PTX keeps
// them on the integer pipe.
__device__ __forceinline__ void dwords(double x, unsigned& lo, unsigned& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "d"(x));
}
__device__ __forceinline__ double djoin(unsigned lo, unsigned hi) {
    double r;
    asm("mov.b64 %0, {%1, %2};" : "=d"(r) : "r"(lo), "r"(hi));
    return r;
}
__device__ __forceinline__ unsigned fbits(float f) {
    unsigned u;
    asm("mov.b32 %0, %1;" : "=r"(u) : "f"(f));
    return u;
}
__device__ __forceinline__ float fjoin(unsigned u) {
    float f;
    asm("mov.b32 %0, %1;" : "=f"(f) : "r"(u));
    return f;
}

// FP64 <-> FP32 conversions on the integer pipe. split_f64 gives hi = the
// FP32 value nearest to a (ties to even — the same result as (float)a) and
// lo = a - hi rounded to FP32, so hi + lo carries about 48 bits of a. Values
// whose FP32 image is subnormal or infinite take the hardware conversion
// (rare; such magnitudes do not occur in the systems solved).
__device__ __forceinline__ void split_f64(double a, float& hi, float& lo) {
    unsigned wl, wh;
    dwords(a, wl, wh);
    const unsigned sign = wh & 0x80000000u;
    const unsigned long long mag =
        ((unsigned long long)(wh & 0x7fffffffu) << 32) | wl;
    if (mag == 0ULL) {  // signed zero
        hi = fjoin(sign);
        lo = 0.0f;
        return;
    }
    // Round the 52-bit mantissa to 23 bits, nearest-even; a carry moves into
    // the exponent field.
    const unsigned long long r =
        (mag + 0x0fffffffULL + ((mag >> 29) & 1ULL)) & ~0x1fffffffULL;
    const int e = (int)(r >> 52);  // biased FP64 exponent of hi
    if (e < 897 || e > 1150) {
        hi = (float)a;
        lo = (float)(a - (double)hi);
        return;
    }
    hi = fjoin(sign | ((unsigned)(e - 896) << 23) |
               (unsigned)((r >> 29) & 0x7fffffULL));
    // a - hi in units of a's last mantissa bit, |d| <= 2^28.
    const int d = (int)((long long)mag - (long long)r);
    const int es = (int)(mag >> 52) - 948;  // biased FP32 exponent of that unit
    const float l = es > 0 ? (float)d * fjoin((unsigned)es << 23) : 0.0f;
    lo = sign ? -l : l;
}
// Exact FP32 -> FP64 widening by bit manipulation (subnormal, inf and NaN
// take the hardware conversion).
__device__ __forceinline__ double widen_f32(float f) {
    const unsigned b = fbits(f);
    const unsigned ef = (b >> 23) & 0xffu;
    if (ef == 0u || ef == 255u) {
        if ((b & 0x7fffffffu) == 0u) return djoin(0u, b);  // signed zero
        return (double)f;
    }
    return djoin(b << 29, (b & 0x80000000u) | ((ef + 896u) << 20) |
                              ((b & 0x7fffffu) >> 3));
}

// Product accumulation in the precision class of the vectors: double-float
// for FP32 vectors (FP32 pipe), plain FP64 for FP64 vectors.
struct AccF {
    DF a;
    __device__ __forceinline__ void add(float x, float y) { df_add_prod(a, x, y); }
    __device__ __forceinline__ double value() const { return df_value(a); }
};
struct AccD {
    double a = 0.0;
    __device__ __forceinline__ void add(double x, double y) { a += x * y; }
    __device__ __forceinline__ double value() const { return a; }
};
template <typename V> struct AccOf;
template <> struct AccOf<float> { using type = AccF; };
template <> struct AccOf<double> { using type = AccD; };

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

// Weights, system build and pressure-gradient kernels (K1-K4, K12).
//
// These kernels replay the reference's double-precision arithmetic exactly so
// that cell classification, face weights, the FP64 matrix and the projected
// velocity are bit-identical to GridFractionalSinglePhasePressureSolver3
// (src/jet/grid_fractional_single_phase_pressure_solver3.cpp). This
// translation unit is compiled with -fmad=false: no multiply-add contraction,
// every product and sum rounds on its own, in the reference's order.
//
// All kernels are HBM-bound elementwise/stencil passes: one thread per output
// element, consecutive threads on consecutive i (coalesced), neighbour loads
// served by L1/L2.

#include "ctx.h"

#include <algorithm>

#include <cfloat>
#include <cmath>
#include <cstring>
#include <map>
#include <utility>
#include <vector>

namespace jg {
namespace {

// ---------------------------------------------------------------------------
// Exact sampling: LinearArraySampler3<double,double>::operator()
// (include/jet/detail/array_samplers3-inl.h:115-149), getBarycentric
// (include/jet/detail/math_utils-inl.h:147-172), lerp/bilerp/trilerp (:177-211).

__device__ __forceinline__ void barycentric(double x, int iHigh, int* i,
                                            double* f) {
    double s = floor(x);
    // Clamp before the integer conversion; the reference converts first, but
    // both select the same branch for every in-range and out-of-range x.
    if (iHigh == 0) {
        *i = 0;
        *f = 0.0;
    } else if (s < 0.0) {
        *i = 0;
        *f = 0.0;
    } else if (s > (double)(iHigh - 1)) {
        *i = iHigh - 1;
        *f = 1.0;
    } else {
        *i = (int)s;
        *f = x - s;
    }
}

__device__ __forceinline__ double lerpd(double a, double b, double f) {
    return (1.0 - f) * a + f * b;
}

// GB300 issues FP64 at a small fraction of its FP32/integer rate, so the
// exact replays below take integer-pipe shortcuts wherever they provably give
// the bit pattern the double arithmetic gives.

// phi < 0 for a double: sign bit set, not a zero, not a NaN (the word
// moves of common.cuh keep these tests on the integer pipe).
__device__ __forceinline__ bool neg_d(double x) {
    unsigned lo, hi;
    dwords(x, lo, hi);
    const unsigned m = hi & 0x7fffffffu;
    return (hi >> 31) != 0u && (m | lo) != 0u &&
           (m < 0x7ff00000u || (m == 0x7ff00000u && lo == 0u));
}
__device__ __forceinline__ unsigned expo_d(double x) {
    unsigned lo, hi;
    dwords(x, lo, hi);
    return (hi >> 20) & 0x7ffu;
}
// x * 0.5 exactly by an exponent decrement when x and x/2 are normal (the
// FP64 fallback out of line, so that it is not predicated into every call).
__device__ __noinline__ double half_slow(double x) { return x * 0.5; }
__device__ __forceinline__ double half_d(double x) {
    unsigned lo, hi;
    dwords(x, lo, hi);
    const unsigned e = (hi >> 20) & 0x7ffu;
    if (e > 1u && e < 0x7ffu) return djoin(lo, hi - 0x100000u);
    return half_slow(x);
}
__device__ __noinline__ double scale_slow(double x, double s) { return x * s; }
// x * 2^k exactly by an exponent add when x and the result are normal;
// zeros pass through; anything else multiplies by the FP64 scale.
__device__ __forceinline__ double scale_pow2(double x, int k, double scale) {
    unsigned lo, hi;
    dwords(x, lo, hi);
    const int e = (int)((hi >> 20) & 0x7ffu);
    if (((hi & 0x7fffffffu) | lo) == 0u) return x;
    if (e > 0 && e < 0x7ff && e + k > 0 && e + k < 0x7ff)
        return djoin(lo, hi + ((unsigned)k << 20));
    return scale_slow(x, scale);
}
// -x exactly by a sign flip, except that -(+0) stays +0 as 0.0 - 0.0 does.
__device__ __forceinline__ double zero_minus(double x) {
    unsigned lo, hi;
    dwords(x, lo, hi);
    if (((hi & 0x7fffffffu) | lo) == 0u) return djoin(0u, 0u);
    return djoin(lo, hi ^ 0x80000000u);
}
// lerp(a, b, f) = (1 - f) * a + f * b (include/jet/detail/math_utils-inl.h)
// with the fraction classes that dominate buildWeights' samples:
//  * f = 0.5: both products are exact halvings, so the result is the one
//    rounding of (a + b) / 2, i.e. half(a + b) — exact whenever a and b are
//    zero or have exponent fields in [2, 0x7fd] (no overflow of a + b, no
//    underflow of a / 2);
//  * f = 0: the result is a + (0 * b), which is a itself when a is non-zero
//    and b finite;
//  * f = 1: (0 * a) + b, which is b when b is non-zero and a finite.
// Everything else takes the reference's expression.
constexpr long long kHalfBits = 0x3FE0000000000000LL;
constexpr long long kOneBits = 0x3FF0000000000000LL;
__device__ __forceinline__ bool half_ok(double x) {
    unsigned lo, hi;
    dwords(x, lo, hi);
    const unsigned e = (hi >> 20) & 0x7ffu;
    return (e >= 2u && e <= 0x7fdu) || ((hi & 0x7fffffffu) | lo) == 0u;
}
__device__ __forceinline__ bool nonzero_d(double x) {
    unsigned lo, hi;
    dwords(x, lo, hi);
    return ((hi & 0x7fffffffu) | lo) != 0u;
}
// The reference's lerp, out of line: the exact shortcuts below cover the
// common fractions, and a call keeps the compiler from predicating this
// FP64 expression into every sample.
__device__ __noinline__ double lerp_slow(double a, double b, double f) {
    return lerpd(a, b, f);
}
__device__ __forceinline__ double lerp_c(double a, double b, double f,
                                         long long fb) {
    if (fb == kHalfBits) {
        if (half_ok(a) && half_ok(b)) return half_d(a + b);
    } else if (fb == 0LL) {
        if (nonzero_d(a) && expo_d(b) != 0x7ffu) return a;
    } else if (fb == kOneBits) {
        if (nonzero_d(b) && expo_d(a) != 0x7ffu) return b;
    }
    return lerp_slow(a, b, f);
}

__device__ double sample_field(const FieldDesc& F, double x, double y,
                               double z) {
    if (F.kind == 0) return F.value;
    const double nx = (x - F.origin[0]) / F.spacing[0];
    const double ny = (y - F.origin[1]) / F.spacing[1];
    const double nz = (z - F.origin[2]) / F.spacing[2];
    int i, j, k;
    double fx, fy, fz;
    barycentric(nx, F.res[0] - 1, &i, &fx);
    barycentric(ny, F.res[1] - 1, &j, &fy);
    barycentric(nz, F.res[2] - 1, &k, &fz);
    const int ip1 = min(i + 1, F.res[0] - 1);
    const int jp1 = min(j + 1, F.res[1] - 1);
    const int kp1 = min(k + 1, F.res[2] - 1);
    const int rx = F.res[0], ry = F.res[1];
    const double* d = F.data;
    const double f000 = d[lin(i, j, k, rx, ry)], f100 = d[lin(ip1, j, k, rx, ry)];
    const double f010 = d[lin(i, jp1, k, rx, ry)], f110 = d[lin(ip1, jp1, k, rx, ry)];
    const double f001 = d[lin(i, j, kp1, rx, ry)], f101 = d[lin(ip1, j, kp1, rx, ry)];
    const double f011 = d[lin(i, jp1, kp1, rx, ry)], f111 = d[lin(ip1, jp1, kp1, rx, ry)];
    const double b0 = lerpd(lerpd(f000, f100, fx), lerpd(f010, f110, fx), fy);
    const double b1 = lerpd(lerpd(f001, f101, fx), lerpd(f011, f111, fx), fy);
    return lerpd(b0, b1, fz);
}

// ---------------------------------------------------------------------------
// Level-set helpers (include/jet/detail/level_set_utils-inl.h:23-147).

__device__ __forceinline__ bool inside(double p) { return p < 0.0; }

__device__ __forceinline__ double frac_sdf(double p0, double p1) {
    if (inside(p0) && inside(p1)) return 1.0;
    if (inside(p0) && !inside(p1)) return p0 / (p0 - p1);
    if (!inside(p0) && inside(p1)) return p1 / (p1 - p0);
    return 0.0;
}

// (l0, l1, l2, l3) rotated left by k (0..3) with constant register moves.
__device__ __forceinline__ void rot4(double& l0, double& l1, double& l2,
                                     double& l3, int k) {
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        if (r < k) {
            const double t = l0;
            l0 = l1;
            l1 = l2;
            l2 = l3;
            l3 = t;
        }
    }
}

// Marching-squares area of the inside region of a face (fractionInside).
// The corners are visited counter-clockwise from bottom-left; each case
// rotates them (the reference's cycleArray) until its anchor corner comes
// first: the rotation count is the first r at which the rotated view stops
// satisfying the reference's loop condition (4 rotations = none).
__device__ __noinline__ double frac_inside(double bl, double br, double tl,
                                           double tr) {
    const double v[4] = {bl, br, tr, tl};
    const bool in[4] = {bl < 0, br < 0, tr < 0, tl < 0};
    const bool ge[4] = {bl >= 0, br >= 0, tr >= 0, tl >= 0};  // NaN: neither
    const int n = in[0] + in[1] + in[2] + in[3];
    const double half = 0.5;  // 0.5f widened, exact
    const double quarter = 0.25;
    if (n == 4) return 1.0;
    if (n == 0) return 0.0;
    int k = 0;
#pragma unroll
    for (int r = 3; r >= 0; --r) {
        bool go;  // the reference's loop condition on the view rotated by r
        if (n == 3) go = in[r];
        else if (n == 2) go = ge[r] || !(in[(r + 1) & 3] || in[(r + 2) & 3]);
        else go = ge[r];
        if (!go) k = r;
    }
    double l0 = v[0], l1 = v[1], l2 = v[2], l3 = v[3];
    rot4(l0, l1, l2, l3, k);
    if (n == 3) {
        const double s0 = 1.0 - frac_sdf(l0, l3);
        const double s1 = 1.0 - frac_sdf(l0, l1);
        return 1.0 - half * s0 * s1;
    }
    if (n == 2) {
        if (l1 < 0) {
            const double sl = frac_sdf(l0, l3);
            const double sr = frac_sdf(l1, l2);
            return half * (sl + sr);
        }
        const double mid = quarter * (l0 + l1 + l2 + l3);
        if (mid < 0) {
            double area = 0.0;
            const double s1 = 1.0 - frac_sdf(l0, l3);
            const double s3 = 1.0 - frac_sdf(l2, l3);
            area += half * s1 * s3;
            const double s2 = 1.0 - frac_sdf(l2, l1);
            const double s0 = 1.0 - frac_sdf(l0, l1);
            area += half * s0 * s2;
            return 1.0 - area;
        }
        double area = 0.0;
        const double s0 = frac_sdf(l0, l1);
        const double s1 = frac_sdf(l0, l3);
        area += half * s0 * s1;
        const double s2 = frac_sdf(l2, l1);
        const double s3 = frac_sdf(l2, l3);
        area += half * s2 * s3;
        return area;
    }
    const double s0 = frac_sdf(l0, l3);
    const double s1 = frac_sdf(l0, l1);
    return half * s0 * s1;
}

__device__ __forceinline__ float face_weight(double p0, double p1, double p2,
                                             double p3) {
    // All four corners on one side: fractionInside is exactly 1 (weight 0)
    // or 0 (weight 1); decided with integer sign tests.
    const int nin = neg_d(p0) + neg_d(p1) + neg_d(p2) + neg_d(p3);
    if (nin == 4) return 0.0f;
    if (nin == 0) return 1.0f;
    const double frac = frac_inside(p0, p1, p2, p3);
    double w = 1.0 - frac;
    w = (w < 0.0) ? 0.0 : ((w > 1.0) ? 1.0 : w);
    if (w < 0.01 && w > 0.0) w = 0.01;  // kMinWeight (:25, :566-570)
    return (float)w;
}

// K1: _fluidSdf[0](i,j,k) = float(fluidSdf.sample(cellCenter)) (:548-551).
__global__ void k_sample_fluid(float* __restrict__ phi, Dims n, GridDesc g,
                               FieldDesc F) {
    const long N = n.count();
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_ijk(c, n, i, j, k);
        // Grid3::cellCenterPosition (src/jet/grid3.cpp:32-38).
        const double px = g.origin[0] + g.spacing[0] * ((double)i + 0.5);
        const double py = g.origin[1] + g.spacing[1] * ((double)j + 0.5);
        const double pz = g.origin[2] + g.spacing[2] * ((double)k + 0.5);
        phi[c] = (float)sample_field(F, px, py, pz);
    }
}

// A constant field (ConstantScalarField3, kind 0) gives every sample its
// value: every face has four equal corner samples and every cell the same
// fluid SDF, so both arrays are fills (k_face_weights and k_sample_fluid
// would compute the same values, with the position arithmetic for nothing).
__global__ void k_fill_face_weight(float* __restrict__ w, long n,
                                   double value) {
    const float wv = face_weight(value, value, value, value);
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n;
         c += (long)gridDim.x * blockDim.x)
        w[c] = wv;
}
__global__ void k_fill_fluid(float* __restrict__ phi, long n, double value) {
    const float v = (float)value;
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n;
         c += (long)gridDim.x * blockDim.x)
        phi[c] = v;
}

// K2: face weights from four boundary-SDF corner samples (:553-617).
// axis 0/1/2 = u/v/w faces.
__global__ void k_face_weights(float* __restrict__ wgt, int axis, Dims fn,
                               GridDesc g, FieldDesc B) {
    const long N = fn.count();
    const double hx = g.spacing[0], hy = g.spacing[1], hz = g.spacing[2];
    // Face data origins (src/jet/face_centered_grid3.cpp:440-442).
    const double ox = g.origin[0] + 0.5 * (axis == 0 ? 0.0 : hx);
    const double oy = g.origin[1] + 0.5 * (axis == 1 ? 0.0 : hy);
    const double oz = g.origin[2] + 0.5 * (axis == 2 ? 0.0 : hz);
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_ijk(c, fn, i, j, k);
        const double px = ox + hx * (double)i;
        const double py = oy + hy * (double)j;
        const double pz = oz + hz * (double)k;
        double p0, p1, p2, p3;
        if (axis == 0) {
            p0 = sample_field(B, px + 0.0, py + -0.5 * hy, pz + -0.5 * hz);
            p1 = sample_field(B, px + 0.0, py + 0.5 * hy, pz + -0.5 * hz);
            p2 = sample_field(B, px + 0.0, py + -0.5 * hy, pz + 0.5 * hz);
            p3 = sample_field(B, px + 0.0, py + 0.5 * hy, pz + 0.5 * hz);
        } else if (axis == 1) {
            p0 = sample_field(B, px + -0.5 * hx, py + 0.0, pz + -0.5 * hz);
            p1 = sample_field(B, px + -0.5 * hx, py + 0.0, pz + 0.5 * hz);
            p2 = sample_field(B, px + 0.5 * hx, py + 0.0, pz + -0.5 * hz);
            p3 = sample_field(B, px + 0.5 * hx, py + 0.0, pz + 0.5 * hz);
        } else {
            p0 = sample_field(B, px + -0.5 * hx, py + -0.5 * hy, pz + 0.0);
            p1 = sample_field(B, px + -0.5 * hx, py + 0.5 * hy, pz + 0.0);
            p2 = sample_field(B, px + 0.5 * hx, py + -0.5 * hy, pz + 0.0);
            p3 = sample_field(B, px + 0.5 * hx, py + 0.5 * hy, pz + 0.0);
        }
        wgt[c] = face_weight(p0, p1, p2, p3);
    }
}

// K3: the anonymous float `restrict` (:29-115): 1-3-3-1/8 on axes where the
// fine size is twice the coarse size, injection {0,1,0} otherwise (the
// face-normal axis of a face array), boundary taps clamped with the coarse
// size. Float sums in the reference's z, y, x order.
__global__ void k_restrict_f32(const float* __restrict__ fine, Dims fs,
                               float* __restrict__ coarse, Dims cs) {
    const long N = cs.count();
    const int ksx = (fs.x != 2 * cs.x) ? 3 : 4;
    const int ksy = (fs.y != 2 * cs.y) ? 3 : 4;
    const int ksz = (fs.z != 2 * cs.z) ? 3 : 4;
    const float cen[4] = {0.125f, 0.375f, 0.375f, 0.125f};
    const float stg[4] = {0.f, 1.f, 0.f, 0.f};
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_ijk(c, cs, i, j, k);
        int iI[4], jI[4], kI[4];
        auto taps = [](int ks, int q, int nq, int* o) {
            o[0] = (q > 0) ? 2 * q - 1 : 2 * q;
            o[1] = 2 * q;
            if (ks == 3) {
                o[2] = (q + 1 < nq) ? 2 * q + 1 : 2 * q;
                o[3] = 0;
            } else {
                o[2] = 2 * q + 1;
                o[3] = (q + 1 < nq) ? 2 * q + 2 : 2 * q + 1;
            }
        };
        taps(ksx, i, cs.x, iI);
        taps(ksy, j, cs.y, jI);
        taps(ksz, k, cs.z, kI);
        const float* kx = (ksx == 3) ? stg : cen;
        const float* ky = (ksy == 3) ? stg : cen;
        const float* kz = (ksz == 3) ? stg : cen;
        float sum = 0.0f;
        for (int z = 0; z < ksz; ++z)
            for (int y = 0; y < ksy; ++y)
                for (int x = 0; x < ksx; ++x) {
                    const float w = kx[x] * ky[y] * kz[z];
                    sum += w * fine[lin(iI[x], jI[y], kI[z], fs.x, fs.y)];
                }
        coarse[c] = sum;
    }
}

// k_restrict_f32 for two coarse cells (2p, 2p+1) of a row per thread, on
// arrays whose x axis is fully restricted (fine x = 2 coarse x, coarse x
// even: the fluid SDF and the v/w face weights). The 6 fine x taps of the
// pair (4p-1 .. 4p+4, clamped) are one aligned 16-byte load and two scalar
// loads per fine row; each output keeps k_restrict_f32's weights and its
// z, y, x order of products and sums, so the results are the same bits.
__global__ void k_restrict_f32x2(const float* __restrict__ fine, Dims fs,
                                 float* __restrict__ coarse, Dims cs) {
    const Dims q{cs.x / 2, cs.y, cs.z};
    const long G = q.count();
    const int ksy = (fs.y != 2 * cs.y) ? 3 : 4;
    const int ksz = (fs.z != 2 * cs.z) ? 3 : 4;
    const float cen[4] = {0.125f, 0.375f, 0.375f, 0.125f};
    const float stg[4] = {0.f, 1.f, 0.f, 0.f};
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < G;
         t += (long)gridDim.x * blockDim.x) {
        int p, j, k;
        cell_ijk(t, q, p, j, k);
        int jI[4], kI[4];
        auto taps = [](int ks, int c, int nc, int* o) {
            o[0] = (c > 0) ? 2 * c - 1 : 2 * c;
            o[1] = 2 * c;
            if (ks == 3) {
                o[2] = (c + 1 < nc) ? 2 * c + 1 : 2 * c;
                o[3] = 0;
            } else {
                o[2] = 2 * c + 1;
                o[3] = (c + 1 < nc) ? 2 * c + 2 : 2 * c + 1;
            }
        };
        taps(ksy, j, cs.y, jI);
        taps(ksz, k, cs.z, kI);
        const float* ky = (ksy == 3) ? stg : cen;
        const float* kz = (ksz == 3) ? stg : cen;
        const int xm = p > 0 ? 4 * p - 1 : 4 * p;           // tap 0 of 2p
        const int x4 = 2 * p + 2 < cs.x ? 4 * p + 4 : 4 * p + 3;  // tap 3 of 2p+1
        float sum0 = 0.0f, sum1 = 0.0f;
        for (int z = 0; z < ksz; ++z)
            for (int y = 0; y < ksy; ++y) {
                const float* row = fine + lin(0, jI[y], kI[z], fs.x, fs.y);
                const float4 f = *reinterpret_cast<const float4*>(row + 4 * p);
                const float v0[4] = {row[xm], f.x, f.y, f.z};
                const float v1[4] = {f.y, f.z, f.w, row[x4]};
                const float wyz = ky[y] * kz[z];
#pragma unroll
                for (int x = 0; x < 4; ++x) {
                    sum0 += cen[x] * wyz * v0[x];
                    sum1 += cen[x] * wyz * v1[x];
                }
            }
        const long o = lin(2 * p, j, k, cs.x, cs.y);
        coarse[o] = sum0;
        coarse[o + 1] = sum1;
    }
}

// Air-side term of buildSingleSystem: term / max(theta, 0.01) with theta =
// fractionInsideSdf(phi_c, phi_n). Out of line, so warps without a
// free-surface face never issue its FP64 divisions.
__device__ __noinline__ double air_term(double term, double cphi, double np) {
    return term / fmax(frac_sdf(cphi, np), 0.01);
}

// Spacing factors of one level: 1/h and 1/h^2 per axis and, when they are
// powers of two (h = 2^-m, the usual unit-cube grids), their exponents, so
// that products with them become exact exponent adds (scale_pow2).
struct SpacingInv {
    double ih[3], ih2[3];
    int k[3], k2[3];
    int pow2;
};

// Appends v to list (length *cnt) when `want`, one atomic per warp.
__device__ __forceinline__ void append_if(bool want, int v,
                                          int* __restrict__ list,
                                          unsigned* __restrict__ cnt) {
    const unsigned act = __activemask();
    const unsigned mask = __ballot_sync(act, want);
    if (mask == 0u) return;
    const int lane = threadIdx.x & 31, leader = __ffs(mask) - 1;
    unsigned base = 0u;
    if (lane == leader) base = atomicAdd(cnt, (unsigned)__popc(mask));
    base = __shfl_sync(act, base, leader);
    if (want) list[base + __popc(mask & ((1u << lane) - 1u))] = v;
}

// K4: buildSingleSystem (:117-267), one cell. Writes the FP32 rows of every
// level; on the finest level also the exact FP64 rows and rhs. u/v/w are the
// input velocity (finest level only; coarse right-hand sides are dead,
// overwritten by restriction in the V-cycle, include/jet/detail/mg-inl.h:
// 28-30). Every FP64 sum and product is the reference's, in its order; what
// changes is how the exact ones are issued: classification on the FP32 SDF,
// exact widening and power-of-two scaling on the integer pipe, divisions out
// of line.
__device__ __forceinline__ void build_cell(long c, Dims n, const SpacingInv& S,
                                           const float* __restrict__ phi,
                                           const float* __restrict__ uw,
                                           const float* __restrict__ vw,
                                           const float* __restrict__ ww,
                                           const double* __restrict__ u,
                                           const double* __restrict__ v,
                                           const double* __restrict__ w,
                                           const double* __restrict__ su,
                                           const double* __restrict__ sv,
                                           const double* __restrict__ sw,
                                           double* __restrict__ A64,
                                           double* __restrict__ b64,
                                           float* __restrict__ A32,
                                           float4* __restrict__ Alo,
                                           float2* __restrict__ bdf,
                                           unsigned char* __restrict__ rflag) {
    const long N = n.count();
    const int ux = n.x + 1;  // u-face row length
    const bool pw = S.pow2 != 0;
    int i, j, k;
    cell_ijk(c, n, i, j, k);
    double center = 0.0, right = 0.0, up = 0.0, front = 0.0, bb = 0.0;
    const float cphf = phi[c];
    bool fluid = false;
    if (cphf < 0.0f) {  // the same test as on the exact widening
        fluid = true;
        const double cphi = widen_f32(cphf);
        const long uR = lin(i + 1, j, k, ux, n.y), uL = lin(i, j, k, ux, n.y);
        const long vU = lin(i, j + 1, k, n.x, n.y + 1),
                   vD = lin(i, j, k, n.x, n.y + 1);
        const long wF = lin(i, j, k + 1, n.x, n.y), wB = lin(i, j, k, n.x, n.y);
        const long sy = n.x, sz = (long)n.x * n.y;
        // One face: the centre term (or the air-side term), the
        // off-diagonal of a fluid neighbour on the upper side, and the
        // rhs term (weighted inside, unweighted on the domain boundary).
        auto face = [&](bool has, const float* wts, long f, long nbc, int a,
                        const double* vel, bool plus, double* off) {
            if (has) {
                const double wd = widen_f32(wts[f]);
                const double term = pw ? scale_pow2(wd, S.k2[a], S.ih2[a])
                                       : wd * S.ih2[a];
                const float npf = phi[nbc];
                if (npf < 0.0f) {
                    center += term;
                    if (off) *off = zero_minus(term);  // 0.0 - term
                } else {
                    center += air_term(term, cphi, widen_f32(npf));
                }
                if (vel) {
                    const double p = wd * vel[f];
                    const double t = pw ? scale_pow2(p, S.k[a], S.ih[a])
                                        : p * S.ih[a];
                    bb = plus ? bb + t : bb - t;
                }
            } else if (vel) {
                const double t = pw ? scale_pow2(vel[f], S.k[a], S.ih[a])
                                    : vel[f] * S.ih[a];
                bb = plus ? bb + t : bb - t;
            }
        };
        face(i + 1 < n.x, uw, uR, c + 1, 0, u, true, &right);
        face(i > 0, uw, uL, c - 1, 0, u, false, nullptr);
        face(j + 1 < n.y, vw, vU, c + sy, 1, v, true, &up);
        face(j > 0, vw, vD, c - sy, 1, v, false, nullptr);
        face(k + 1 < n.z, ww, wF, c + sz, 2, w, true, &front);
        face(k > 0, ww, wB, c - sz, 2, w, false, nullptr);
        if (u && !su && !sv && !sw) {
            // Static collider: every term of the moving-boundary sum is
            // (1 - w) * 0 * invH = +0, so the sum is +0 and adding it
            // only turns -0 into +0 — exactly what this does.
            unsigned lo, hi;
            dwords(bb, lo, hi);
            if (hi == 0x80000000u && lo == 0u) bb = djoin(0u, 0u);
        } else if (u) {
            // Moving-boundary contribution (:241-255), evaluated as the
            // reference's single left-to-right expression.
            const double ihx = S.ih[0], ihy = S.ih[1], ihz = S.ih[2];
            const double sR = su ? su[uR] : 0.0, sL = su ? su[uL] : 0.0;
            const double sU = sv ? sv[vU] : 0.0, sD = sv ? sv[vD] : 0.0;
            const double sF = sw ? sw[wF] : 0.0, sB = sw ? sw[wB] : 0.0;
            const double contrib = (1.0 - (double)uw[uR]) * sR * ihx -
                                   (1.0 - (double)uw[uL]) * sL * ihx +
                                   (1.0 - (double)vw[vU]) * sU * ihy -
                                   (1.0 - (double)vw[vD]) * sD * ihy +
                                   (1.0 - (double)ww[wF]) * sF * ihz -
                                   (1.0 - (double)ww[wB]) * sB * ihz;
            bb += contrib;
        }
        // center < kEpsilonD (:259-262); center is a sum of non-negative
        // terms, so its bit pattern orders like its value.
        unsigned clo, chi;
        dwords(center, clo, chi);
        const unsigned long long cbits =
            ((unsigned long long)chi << 32) | clo;
        if (cbits < 0x3CB0000000000000ULL) {  // DBL_EPSILON
            center = 1.0;
            bb = 0.0;
            if (rflag) rflag[c] = 0;
        } else if (rflag) {
            rflag[c] = 1;  // the rhs pass fills b
        }
    } else {
        center = 1.0;
        if (rflag) rflag[c] = 0;
    }
    if (A64) {  // one 32-byte row as two 16-byte stores
        double2* row = reinterpret_cast<double2*>(A64 + 4 * c);
        row[0] = make_double2(center, right);
        row[1] = make_double2(up, front);
    }
    if (b64) b64[c] = bb;
    // FP32 rows (= the FP32 rounding of the exact rows) and, on the
    // finest level, the low parts that make hi + lo carry ~48 bits of
    // each coefficient and of b for the double-float true residual.
    float4 hi4, lo4;
    float bh, bl;
    if (fluid) {
        split_f64(center, hi4.x, lo4.x);
        split_f64(right, hi4.y, lo4.y);
        split_f64(up, hi4.z, lo4.z);
        split_f64(front, hi4.w, lo4.w);
        split_f64(bb, bh, bl);
    } else {
        hi4 = make_float4(1.0f, 0.0f, 0.0f, 0.0f);
        lo4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        bh = bl = 0.0f;
    }
    A32[c] = hi4.x;  // structure of arrays: center, right, up, front
    A32[N + c] = hi4.y;
    A32[2 * N + c] = hi4.z;
    A32[3 * N + c] = hi4.w;
    if (Alo) Alo[c] = lo4;
    if (bdf) bdf[c] = make_float2(bh, bl);
}

// K4's kernel. Latency-bound at the 94 registers it would take freely (two
// blocks per SM): capped at 40 for six blocks, with a few spilled values,
// it runs 1.9x faster (1.21 -> 0.77 ms per 256^3 solve at four blocks,
// 0.64 ms at six; eight blocks spill too much, 0.79 ms). (Compacting the
// fluid cells next to air into full warps for their FP64 divisions, as the
// face weights do, made it slower: the sums and the rhs of every fluid cell
// are FP64 too, so little of its FP64 work is divergent.)
template <bool kMarkRhs>
__global__ void __launch_bounds__(kThreads, 6)
    k_build_system(Dims n, SpacingInv S,
                   const float* __restrict__ phi,
                   const float* __restrict__ uw,
                   const float* __restrict__ vw,
                   const float* __restrict__ ww,
                   const double* __restrict__ u,
                   const double* __restrict__ v,
                   const double* __restrict__ w,
                   const double* __restrict__ su,
                   const double* __restrict__ sv,
                   const double* __restrict__ sw,
                   double* __restrict__ A64,
                   double* __restrict__ b64,
                   float* __restrict__ A32,
                   float4* __restrict__ Alo,
                   float2* __restrict__ bdf,
                   unsigned char* __restrict__ rflag) {
    const long N = n.count();
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x)
        build_cell(c, n, S, phi, uw, vw, ww, u, v, w, su, sv, sw, A64, b64,
                   A32, Alo, bdf, kMarkRhs ? rflag : nullptr);
}

// The level-0 rhs alone, for a host-pointer solve whose rows were built
// (k_build_system without velocities, marking in rflag the fluid cells
// whose centre was kept) while the velocities were still uploading: the
// same faces, order and expressions as build_cell's rhs, so b is the same.
__global__ void __launch_bounds__(kThreads)
    k_build_rhs(Dims n, SpacingInv S, const unsigned char* __restrict__ rflag,
                const float* __restrict__ uw, const float* __restrict__ vw,
                const float* __restrict__ ww, const double* __restrict__ u,
                const double* __restrict__ v, const double* __restrict__ w,
                const double* __restrict__ su, const double* __restrict__ sv,
                const double* __restrict__ sw, double* __restrict__ b64,
                float2* __restrict__ bdf) {
    const long N = n.count();
    const int ux = n.x + 1;
    const bool pw = S.pow2 != 0;
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x) {
        double bb = 0.0;
        const bool fl = rflag[c] != 0;
        if (fl) {
            int i, j, k;
            cell_ijk(c, n, i, j, k);
            const long uR = lin(i + 1, j, k, ux, n.y), uL = lin(i, j, k, ux, n.y);
            const long vU = lin(i, j + 1, k, n.x, n.y + 1),
                       vD = lin(i, j, k, n.x, n.y + 1);
            const long wF = lin(i, j, k + 1, n.x, n.y), wB = lin(i, j, k, n.x, n.y);
            auto face = [&](bool has, const float* wts, long f, int a,
                            const double* vel, bool plus) {
                if (has) {
                    const double wd = widen_f32(wts[f]);
                    const double p = wd * vel[f];
                    const double t = pw ? scale_pow2(p, S.k[a], S.ih[a])
                                        : p * S.ih[a];
                    bb = plus ? bb + t : bb - t;
                } else {
                    const double t = pw ? scale_pow2(vel[f], S.k[a], S.ih[a])
                                        : vel[f] * S.ih[a];
                    bb = plus ? bb + t : bb - t;
                }
            };
            face(i + 1 < n.x, uw, uR, 0, u, true);
            face(i > 0, uw, uL, 0, u, false);
            face(j + 1 < n.y, vw, vU, 1, v, true);
            face(j > 0, vw, vD, 1, v, false);
            face(k + 1 < n.z, ww, wF, 2, w, true);
            face(k > 0, ww, wB, 2, w, false);
            if (!su && !sv && !sw) {
                unsigned lo, hi;
                dwords(bb, lo, hi);
                if (hi == 0x80000000u && lo == 0u) bb = djoin(0u, 0u);
            } else {
                const double ihx = S.ih[0], ihy = S.ih[1], ihz = S.ih[2];
                const double sR = su ? su[uR] : 0.0, sL = su ? su[uL] : 0.0;
                const double sU = sv ? sv[vU] : 0.0, sD = sv ? sv[vD] : 0.0;
                const double sF = sw ? sw[wF] : 0.0, sB = sw ? sw[wB] : 0.0;
                const double contrib = (1.0 - (double)uw[uR]) * sR * ihx -
                                       (1.0 - (double)uw[uL]) * sL * ihx +
                                       (1.0 - (double)vw[vU]) * sU * ihy -
                                       (1.0 - (double)vw[vD]) * sD * ihy +
                                       (1.0 - (double)ww[wF]) * sF * ihz -
                                       (1.0 - (double)ww[wB]) * sB * ihz;
                bb += contrib;
            }
        }
        b64[c] = bb;
        float bh = 0.0f, bl = 0.0f;
        if (fl) split_f64(bb, bh, bl);
        bdf[c] = make_float2(bh, bl);
    }
}

// Double-float image of a caller-built finest-level system (the FP32 rows
// are written by the caller's conversion; this adds the low parts and b).
__global__ void k_split_system(const double* __restrict__ A64,
                               const double* __restrict__ b64,
                               float4* __restrict__ Alo,
                               float2* __restrict__ bdf, long N) {
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x) {
        float4 hi4, lo4;
        split_f64(A64[4 * c + 0], hi4.x, lo4.x);
        split_f64(A64[4 * c + 1], hi4.y, lo4.y);
        split_f64(A64[4 * c + 2], hi4.z, lo4.z);
        split_f64(A64[4 * c + 3], hi4.w, lo4.w);
        Alo[c] = lo4;
        float bh, bl;
        split_f64(b64[c], bh, bl);
        bdf[c] = make_float2(bh, bl);
    }
}

// Gradient coefficient invH / max(theta, 0.01) of a face with an air side
// (out of line: only free-surface faces issue the FP64 divisions).
__device__ __noinline__ double grad_coef(double ih, float cphf, float npf) {
    return ih / fmax(frac_sdf(widen_f32(cphf), widen_f32(npf)), 0.01);
}

// K12: applyPressureGradient (:715-765). The output starts as a copy of the
// input (grid_fluid_solver3.cpp:245-250); faces with a positive weight and a
// fluid side get u + invH / max(theta, 0.01) * (x_n - x_c). The thread of
// cell c owns the faces i+1/j+1/k+1 of c, and the cells on the lower domain
// boundary also own faces 0, so every output face is written once; with
// `copy` false (output aliasing the input) untouched faces are skipped.
// Between two fluid cells theta = 1 and invH / 1 = invH exactly.
__global__ void k_apply_gradient(Dims n, SpacingInv S,
                                 const float* __restrict__ phi,
                                 const float* __restrict__ uw,
                                 const float* __restrict__ vw,
                                 const float* __restrict__ ww,
                                 const double* __restrict__ x,
                                 const double* u, const double* v,
                                 const double* w, double* ou, double* ov,
                                 double* ow, int copy, int kz0, int kz1) {
    const int ux = n.x + 1;
    const long sz = (long)n.x * n.y;
    const long N = kz1 * sz;
    const bool pw = S.pow2 != 0;
    for (long c = kz0 * sz + blockIdx.x * (long)blockDim.x + threadIdx.x;
         c < N; c += (long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_ijk(c, n, i, j, k);
        const float cphf = phi[c];
        const bool cin = cphf < 0.0f;
        auto face = [&](bool inner, const float* wts, long f, long nbc, int a,
                        const double* in, double* out) {
            if (inner) {
                const float npf = phi[nbc];
                if (wts[f] > 0.0f && (cin || npf < 0.0f)) {
                    const double dx = x[nbc] - x[c];
                    double g;
                    if (cin && npf < 0.0f)
                        g = pw ? scale_pow2(dx, S.k[a], S.ih[a]) : S.ih[a] * dx;
                    else
                        g = grad_coef(S.ih[a], cphf, npf) * dx;
                    out[f] = in[f] + g;
                    return;
                }
            }
            if (copy) out[f] = in[f];
        };
        face(i + 1 < n.x, uw, lin(i + 1, j, k, ux, n.y), c + 1, 0, u, ou);
        face(j + 1 < n.y, vw, lin(i, j + 1, k, n.x, n.y + 1), c + n.x, 1, v, ov);
        face(k + 1 < n.z, ww, lin(i, j, k + 1, n.x, n.y), c + sz, 2, w, ow);
        if (copy) {
            if (i == 0) ou[lin(0, j, k, ux, n.y)] = u[lin(0, j, k, ux, n.y)];
            if (j == 0) ov[lin(i, 0, k, n.x, n.y + 1)] = v[lin(i, 0, k, n.x, n.y + 1)];
            if (k == 0) ow[lin(i, j, 0, n.x, n.y)] = w[lin(i, j, 0, n.x, n.y)];
        }
    }
}

// k_apply_gradient over 4-cell groups (n.x a multiple of 4): the same
// per-face rule and arithmetic for each cell, with the cell values, the
// v and w faces and their weights moved as 16-byte accesses. Every owned
// face is written (its input value when untouched), which with an aliased
// output rewrites the value already there. Four blocks per SM (64
// registers, a few spilled) run it 6% faster than the three that 78
// registers allow.
__global__ void __launch_bounds__(kThreads, 4)
    k_apply_gradient4(Dims n, SpacingInv S, const float* __restrict__ phi,
                      const float* __restrict__ uw,
                      const float* __restrict__ vw,
                      const float* __restrict__ ww,
                      const double* __restrict__ x, const double* u,
                      const double* v, const double* w, double* ou,
                      double* ov, double* ow, int kz0, int kz1) {
    const Dims g{n.x / 4, n.y, n.z};
    const long gz = (long)g.x * g.y;
    const long G = kz1 * gz;
    const int ux = n.x + 1;
    const long sy = n.x, sz = (long)n.x * n.y;
    const bool pw = S.pow2 != 0;
    for (long t = kz0 * gz + blockIdx.x * (long)blockDim.x + threadIdx.x;
         t < G; t += (long)gridDim.x * blockDim.x) {
        int m, j, k;
        cell_ijk(t, g, m, j, k);
        const int i = 4 * m;
        const long c = lin(i, j, k, n.x, n.y);
        const float4 p4 = *reinterpret_cast<const float4*>(phi + c);
        const float P[5] = {p4.x, p4.y, p4.z, p4.w,
                            i + 4 < n.x ? phi[c + 4] : 1.0f};
        const double2 x01 = *reinterpret_cast<const double2*>(x + c);
        const double2 x23 = *reinterpret_cast<const double2*>(x + c + 2);
        const double X[5] = {x01.x, x01.y, x23.x, x23.y,
                             i + 4 < n.x ? x[c + 4] : 0.0};
        // The gradient of one face: in + coefficient * (x_n - x_c).
        auto grad = [&](double in, float wt, float cphf, float npf, double xc,
                        double xn, int a) {
            const bool cin = cphf < 0.0f;
            if (wt > 0.0f && (cin || npf < 0.0f)) {
                const double dx = xn - xc;
                double gr;
                if (cin && npf < 0.0f)
                    gr = pw ? scale_pow2(dx, S.k[a], S.ih[a]) : S.ih[a] * dx;
                else
                    gr = grad_coef(S.ih[a], cphf, npf) * dx;
                return in + gr;
            }
            return in;
        };
        // u faces i+1 .. i+4 (the last one inner only when i + 4 < n.x).
        const long fu = lin(i + 1, j, k, ux, n.y);
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            const double in = u[fu + l];
            ou[fu + l] = (i + l + 1 < n.x)
                             ? grad(in, uw[fu + l], P[l], P[l + 1], X[l],
                                    X[l + 1], 0)
                             : in;
        }
        if (i == 0) ou[lin(0, j, k, ux, n.y)] = u[lin(0, j, k, ux, n.y)];
        // v faces (i..i+3, j+1) and w faces (i..i+3, k+1).
        auto faces4 = [&](bool inner, const float* wts, const double* in,
                          double* out, long f, long nb, int a) {
            const double2 i01 = *reinterpret_cast<const double2*>(in + f);
            const double2 i23 = *reinterpret_cast<const double2*>(in + f + 2);
            double o[4] = {i01.x, i01.y, i23.x, i23.y};
            if (inner) {
                const float4 w4 = *reinterpret_cast<const float4*>(wts + f);
                const float4 q4 = *reinterpret_cast<const float4*>(phi + nb);
                const double2 n01 = *reinterpret_cast<const double2*>(x + nb);
                const double2 n23 = *reinterpret_cast<const double2*>(x + nb + 2);
                const float W[4] = {w4.x, w4.y, w4.z, w4.w};
                const float Q[4] = {q4.x, q4.y, q4.z, q4.w};
                const double XN[4] = {n01.x, n01.y, n23.x, n23.y};
#pragma unroll
                for (int l = 0; l < 4; ++l)
                    o[l] = grad(o[l], W[l], P[l], Q[l], X[l], XN[l], a);
            }
            *reinterpret_cast<double2*>(out + f) = make_double2(o[0], o[1]);
            *reinterpret_cast<double2*>(out + f + 2) = make_double2(o[2], o[3]);
        };
        faces4(j + 1 < n.y, vw, v, ov, lin(i, j + 1, k, n.x, n.y + 1), c + sy,
               1);
        faces4(k + 1 < n.z, ww, w, ow, lin(i, j, k + 1, n.x, n.y), c + sz, 2);
        if (j == 0) {
            const long f = lin(i, 0, k, n.x, n.y + 1);
            *reinterpret_cast<double2*>(ov + f) =
                *reinterpret_cast<const double2*>(v + f);
            *reinterpret_cast<double2*>(ov + f + 2) =
                *reinterpret_cast<const double2*>(v + f + 2);
        }
        if (k == 0) {
            const long f = lin(i, j, 0, n.x, n.y);
            *reinterpret_cast<double2*>(ow + f) =
                *reinterpret_cast<const double2*>(w + f);
            *reinterpret_cast<double2*>(ow + f + 2) =
                *reinterpret_cast<const double2*>(w + f + 2);
        }
    }
}

// ---------------------------------------------------------------------------
// Separable sampling tables.
//
// Every sample position of buildWeights is a per-axis expression: the
// x coordinate of a u-face corner depends on i alone, and so on. The
// barycentric (index, fraction) pair of each coordinate is therefore computed
// once per axis and expression, with the reference's arithmetic, instead of
// twelve times per cell. Corner points shared by several faces resolve to the
// same (index, fraction) triple; the host dedupes the triples into "slots",
// every slot triple is sampled once into a node grid, and the face kernels
// look their four corners up. Because a trilinear sample depends only on its
// (index, fraction) triple and the data, the result is bit-identical to
// sampling each corner directly.
//
// Table kinds per axis a (n = grid resolution along a):
//   N: face-normal coordinate   (o_a + 0.5*0.0) + h_a*i + 0.0,     i in [0,n]
//   M: tangential, lower corner (o_a + 0.5*h_a) + h_a*i + (-0.5*h_a), i < n
//   P: tangential, upper corner (o_a + 0.5*h_a) + h_a*i + 0.5*h_a,    i < n
//   C: cell centre              o_a + h_a*(i + 0.5),                  i < n

__device__ __forceinline__ double trilerp_at(const double* __restrict__ d,
                                             const int* res, int i, double fx,
                                             int j, double fy, int k,
                                             double fz) {
    const int ip1 = min(i + 1, res[0] - 1);
    const int jp1 = min(j + 1, res[1] - 1);
    const int kp1 = min(k + 1, res[2] - 1);
    const int rx = res[0], ry = res[1];
    const double f000 = d[lin(i, j, k, rx, ry)], f100 = d[lin(ip1, j, k, rx, ry)];
    const double f010 = d[lin(i, jp1, k, rx, ry)], f110 = d[lin(ip1, jp1, k, rx, ry)];
    const double f001 = d[lin(i, j, kp1, rx, ry)], f101 = d[lin(ip1, j, kp1, rx, ry)];
    const double f011 = d[lin(i, jp1, kp1, rx, ry)], f111 = d[lin(ip1, jp1, kp1, rx, ry)];
    auto cls = [](double f) {
        unsigned lo, hi;
        dwords(f, lo, hi);
        return (long long)(((unsigned long long)hi << 32) | lo);
    };
    const long long bx = cls(fx), by = cls(fy), bz = cls(fz);
    const double b0 = lerp_c(lerp_c(f000, f100, fx, bx),
                             lerp_c(f010, f110, fx, bx), fy, by);
    const double b1 = lerp_c(lerp_c(f001, f101, fx, bx),
                             lerp_c(f011, f111, fx, bx), fy, by);
    return lerp_c(b0, b1, fz, bz);
}

struct TabLayout {
    int off[3][4];  // [axis][N,M,P,C] entry offsets
    int total;
};

__global__ void k_axis_tables(GridDesc g, FieldDesc B, FieldDesc F,
                              TabLayout L, int* __restrict__ idx,
                              double* __restrict__ frac) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < L.total;
         e += gridDim.x * blockDim.x) {
        int a = 0, kind = 0;
        for (int aa = 0; aa < 3; ++aa)
            for (int kk = 0; kk < 4; ++kk)
                if (e >= L.off[aa][kk]) {
                    a = aa;
                    kind = kk;
                }
        const int i = e - L.off[a][kind];
        const double o = g.origin[a], h = g.spacing[a];
        double coord;
        if (kind == 0) coord = (o + 0.5 * 0.0) + h * (double)i + 0.0;
        else if (kind == 1) coord = (o + 0.5 * h) + h * (double)i + -0.5 * h;
        else if (kind == 2) coord = (o + 0.5 * h) + h * (double)i + 0.5 * h;
        else coord = o + h * ((double)i + 0.5);
        const FieldDesc& S = (kind == 3) ? F : B;
        if (S.kind != 1) {
            idx[e] = 0;
            frac[e] = 0.0;
            continue;
        }
        const double nrm = (coord - S.origin[a]) / S.spacing[a];
        int ii;
        double ff;
        barycentric(nrm, S.res[a] - 1, &ii, &ff);
        idx[e] = ii;
        frac[e] = ff;
    }
}

// One trilinear sample per slot triple (sx fastest).
__global__ void k_node_grid(FieldDesc B, const int* __restrict__ sidx,
                            const double* __restrict__ sfrac, int3 soff,
                            int3 S, double* __restrict__ node) {
    const long N = (long)S.x * S.y * S.z;
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x) {
        int a, b, z;
        cell_ijk(c, Dims{S.x, S.y, S.z}, a, b, z);
        node[c] = trilerp_at(B.data, B.res, sidx[soff.x + a], sfrac[soff.x + a],
                             sidx[soff.y + b], sfrac[soff.y + b],
                             sidx[soff.z + z], sfrac[soff.z + z]);
    }
}

// The four corner samples of face c of axis `axis` from the node grid.
// slot[] maps a table entry to its slot.
template <int axis>
__device__ __forceinline__ void face_corners(long c, Dims fn,
                                             const int* __restrict__ slot,
                                             const TabLayout& L, int3 S,
                                             const double* __restrict__ node,
                                             double p[4]) {
    int i, j, k;
    cell_ijk(c, fn, i, j, k);
    // Lower/upper slot along each axis: N for the normal axis (same for
    // both), M/P for the tangential axes.
    const int q[3] = {i, j, k};
    int lo[3], hi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (a == axis) {
            lo[a] = hi[a] = slot[L.off[a][0] + q[a]];
        } else {
            lo[a] = slot[L.off[a][1] + q[a]];
            hi[a] = slot[L.off[a][2] + q[a]];
        }
    }
    auto at = [&](int x, int y, int z) {
        return node[x + (long)S.x * (y + (long)S.y * z)];
    };
    if (axis == 0) {  // (0,-y,-z) (0,+y,-z) (0,-y,+z) (0,+y,+z)
        p[0] = at(lo[0], lo[1], lo[2]);
        p[1] = at(lo[0], hi[1], lo[2]);
        p[2] = at(lo[0], lo[1], hi[2]);
        p[3] = at(lo[0], hi[1], hi[2]);
    } else if (axis == 1) {  // (-x,0,-z) (-x,0,+z) (+x,0,-z) (+x,0,+z)
        p[0] = at(lo[0], lo[1], lo[2]);
        p[1] = at(lo[0], lo[1], hi[2]);
        p[2] = at(hi[0], lo[1], lo[2]);
        p[3] = at(hi[0], lo[1], hi[2]);
    } else {  // (-x,-y,0) (-x,+y,0) (+x,-y,0) (+x,+y,0)
        p[0] = at(lo[0], lo[1], lo[2]);
        p[1] = at(lo[0], hi[1], lo[2]);
        p[2] = at(hi[0], lo[1], lo[2]);
        p[3] = at(hi[0], hi[1], lo[2]);
    }
}


// Face weights from the node grid, first pass: a face whose four corners
// lie on one side gets weight 0 or 1 from integer sign tests (face_weight's
// own shortcut); every other face (the thin shell around the collider
// surface) is appended to a list for k_face_weights_listed. GB300 issues
// FP64 at a small fraction of its FP32 rate and a warp runs the
// marching-squares divisions for all its lanes, so gathering the few such
// faces into full warps keeps the FP64 pipe from serving idle lanes.
template <int axis>
__global__ void k_face_weights_nodes(float* __restrict__ wgt,
                                     Dims fn, const int* __restrict__ slot,
                                     TabLayout L, int3 S,
                                     const double* __restrict__ node,
                                     int* __restrict__ list,
                                     unsigned* __restrict__ cnt) {
    const long N = fn.count();
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x) {
        double p[4];
        face_corners<axis>(c, fn, slot, L, S, node, p);
        const int nin = neg_d(p[0]) + neg_d(p[1]) + neg_d(p[2]) + neg_d(p[3]);
        const bool hard = nin != 0 && nin != 4;
        if (!hard) wgt[c] = nin == 4 ? 0.0f : 1.0f;
        append_if(hard, (int)c, list, cnt);
    }
}

// Second pass: the listed faces, with the full face_weight.
template <int axis>
__global__ void k_face_weights_listed(float* __restrict__ wgt,
                                      Dims fn, const int* __restrict__ slot,
                                      TabLayout L, int3 S,
                                      const double* __restrict__ node,
                                      const int* __restrict__ list,
                                      const unsigned* __restrict__ cnt) {
    const unsigned m = *cnt;
    for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < m;
         q += gridDim.x * blockDim.x) {
        const long c = list[q];
        double p[4];
        face_corners<axis>(c, fn, slot, L, S, node, p);
        wgt[c] = face_weight(p[0], p[1], p[2], p[3]);
    }
}

// Fluid SDF at cell centres from the C tables.
// 1 in *irregular when some value is zero or not finite.
__global__ void k_values_regular(const double* __restrict__ d, long n,
                                 int* __restrict__ irregular) {
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n;
         c += (long)gridDim.x * blockDim.x) {
        unsigned lo, hi;
        dwords(d[c], lo, hi);
        if (((hi << 1) | lo) == 0u || ((hi >> 20) & 0x7ffu) == 0x7ffu)
            *irregular = 1;
    }
}

// The fluid SDF's samples at the cell centres. With `irregular` non-null the
// SDF lies on the cells (each centre's entry is its own index with fraction
// 0, or for the last centre the one before with fraction 1); when the flag
// is 0 (no zero, no non-finite value) every lerp of a sample returns the
// operand of that cell, so the sample is the cell's own value.
__global__ void k_sample_fluid_tab(float* __restrict__ phi, Dims n,
                                   FieldDesc F, const int* __restrict__ idx,
                                   const double* __restrict__ frac,
                                   TabLayout L,
                                   const int* __restrict__ irregular) {
    const long N = n.count();
    const int ox = L.off[0][3], oy = L.off[1][3], oz = L.off[2][3];
    const bool own = irregular && !*irregular;
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x) {
        if (own) {
            float hi, lo;
            split_f64(F.data[c], hi, lo);
            phi[c] = hi;
            continue;
        }
        int i, j, k;
        cell_ijk(c, n, i, j, k);
        float hi, lo;
        split_f64(trilerp_at(F.data, F.res, idx[ox + i], frac[ox + i],
                             idx[oy + j], frac[oy + j], idx[oz + k],
                             frac[oz + k]),
                  hi, lo);
        phi[c] = hi;  // == (float) of the sample
    }
}

bool same_geom(const FieldDesc& a, const FieldDesc& b) {
    if (a.kind != b.kind) return false;
    for (int d = 0; d < 3; ++d)
        if (a.res[d] != b.res[d] || a.origin[d] != b.origin[d] ||
            a.spacing[d] != b.spacing[d])
            return false;
    return true;
}

bool same_grid(const GridDesc& a, const GridDesc& b) {
    for (int d = 0; d < 3; ++d)
        if (a.res[d] != b.res[d] || a.origin[d] != b.origin[d] ||
            a.spacing[d] != b.spacing[d])
            return false;
    return true;
}

// Builds (or reuses) the axis tables, slots and node-grid geometry for the
// given grid and field geometries.
jetgpu_status ensure_tables(Ctx* c, const GridDesc& g, const FieldDesc& B,
                            const FieldDesc& F) {
    SampleTables& T = c->tabs;
    if (T.valid && same_grid(T.g, g) && same_geom(T.B, B) && same_geom(T.F, F))
        return JETGPU_OK;
    T.valid = false;
    TabLayout L;
    int off = 0;
    for (int a = 0; a < 3; ++a) {
        const int n = g.res[a];
        L.off[a][0] = off; off += n + 1;
        L.off[a][1] = off; off += n;
        L.off[a][2] = off; off += n;
        L.off[a][3] = off; off += n;
    }
    L.total = off;
    if ((size_t)off > T.cap) {
        if (T.idx) cudaFree(T.idx);
        if (T.frac) cudaFree(T.frac);
        if (T.slot) cudaFree(T.slot);
        if (T.sidx) cudaFree(T.sidx);
        if (T.sfrac) cudaFree(T.sfrac);
        T.idx = nullptr; T.frac = nullptr; T.slot = nullptr;
        T.sidx = nullptr; T.sfrac = nullptr; T.cap = 0;
        JG_CUDA(c, cudaMalloc((void**)&T.idx, off * sizeof(int)));
        JG_CUDA(c, cudaMalloc((void**)&T.frac, off * sizeof(double)));
        JG_CUDA(c, cudaMalloc((void**)&T.slot, off * sizeof(int)));
        JG_CUDA(c, cudaMalloc((void**)&T.sidx, off * sizeof(int)));
        JG_CUDA(c, cudaMalloc((void**)&T.sfrac, off * sizeof(double)));
        T.cap = off;
    }
    k_axis_tables<<<blocks_for(off), kThreads, 0, c->stream>>>(g, B, F, L,
                                                               T.idx, T.frac);
    JG_CUDA(c, cudaGetLastError());
    std::vector<int> hidx(off);
    std::vector<double> hfrac(off);
    JG_CUDA(c, cudaMemcpyAsync(hidx.data(), T.idx, off * sizeof(int),
                               cudaMemcpyDeviceToHost, c->stream));
    JG_CUDA(c, cudaMemcpyAsync(hfrac.data(), T.frac, off * sizeof(double),
                               cudaMemcpyDeviceToHost, c->stream));
    JG_CUDA(c, cudaStreamSynchronize(c->stream));
    // Dedupe N/M/P entries of each axis by exact (index, fraction).
    std::vector<int> hslot(off, 0), sidx(off, 0);
    std::vector<double> sfrac(off, 0.0);
    int soff[3], nslot[3], used = 0;
    for (int a = 0; a < 3; ++a) {
        std::map<std::pair<int, uint64_t>, int> seen;
        soff[a] = used;
        for (int e = L.off[a][0]; e < L.off[a][3]; ++e) {
            uint64_t bits;
            std::memcpy(&bits, &hfrac[e], 8);
            auto key = std::make_pair(hidx[e], bits);
            auto it = seen.find(key);
            int s;
            if (it == seen.end()) {
                s = (int)seen.size();
                seen.emplace(key, s);
                sidx[used + s] = hidx[e];
                sfrac[used + s] = hfrac[e];
            } else {
                s = it->second;
            }
            hslot[e] = s;
        }
        nslot[a] = (int)seen.size();
        used += nslot[a];
    }
    JG_CUDA(c, cudaMemcpyAsync(T.slot, hslot.data(), off * sizeof(int),
                               cudaMemcpyHostToDevice, c->stream));
    JG_CUDA(c, cudaMemcpyAsync(T.sidx, sidx.data(), used * sizeof(int),
                               cudaMemcpyHostToDevice, c->stream));
    JG_CUDA(c, cudaMemcpyAsync(T.sfrac, sfrac.data(), used * sizeof(double),
                               cudaMemcpyHostToDevice, c->stream));
    const size_t nodes = (size_t)nslot[0] * nslot[1] * nslot[2];
    const size_t cells = (size_t)(g.res[0] + 1) * (g.res[1] + 1) * (g.res[2] + 1);
    T.use_nodes = nodes <= 4 * cells;
    // getBarycentric puts the last centre at (n - 2, 1): the same value.
    T.fluid_on_cells = F.kind == 1;
    for (int a = 0; a < 3 && T.fluid_on_cells; ++a) {
        const int n = g.res[a];
        T.fluid_on_cells = F.res[a] == n;
        for (int i = 0; i < n && T.fluid_on_cells; ++i) {
            const int e = L.off[a][3] + i;
            T.fluid_on_cells = (hidx[e] == i && hfrac[e] == 0.0 &&
                                !std::signbit(hfrac[e])) ||
                               (i == n - 1 && n >= 2 && hidx[e] == n - 2 &&
                                hfrac[e] == 1.0);
        }
    }
    if (!T.irregular)
        JG_CUDA(c, cudaMalloc((void**)&T.irregular, sizeof(int)));
    if (T.use_nodes && nodes > T.node_cap) {
        if (T.node) cudaFree(T.node);
        T.node = nullptr;
        T.node_cap = 0;
        JG_CUDA(c, cudaMalloc((void**)&T.node, nodes * sizeof(double)));
        T.node_cap = nodes;
    }
    JG_CUDA(c, cudaStreamSynchronize(c->stream));
    for (int a = 0; a < 3; ++a) {
        for (int k = 0; k < 4; ++k) T.off[a][k] = L.off[a][k];
        T.soff[a] = soff[a];
        T.nslot[a] = nslot[a];
    }
    T.total = L.total;
    T.g = g;
    T.B = B;
    T.F = F;
    T.valid = true;
    return JETGPU_OK;
}

TabLayout layout_of(const SampleTables& T) {
    TabLayout L;
    for (int a = 0; a < 3; ++a)
        for (int k = 0; k < 4; ++k) L.off[a][k] = T.off[a][k];
    L.total = T.total;
    return L;
}

}  // namespace

// Grid of a fill: enough blocks to cover the SMs eight times over.
static int grid_cap(const Ctx* c, long n) {
    return blocks_for(n, kThreads, c->num_sms * 8);
}

// The compaction list of the two-pass face-weight kernels: room for n
// entries and a counter.
static jetgpu_status grow_list(Ctx* c, size_t n) {
    if (!c->build_cnt)
        JG_CUDA(c, cudaMalloc((void**)&c->build_cnt, sizeof(unsigned)));
    if (c->build_cap >= n) return JETGPU_OK;
    if (c->build_list) cudaFree(c->build_list);
    c->build_list = nullptr;
    c->build_cap = 0;
    JG_CUDA(c, cudaMalloc((void**)&c->build_list, n * sizeof(int)));
    c->build_cap = n;
    return JETGPU_OK;
}

jetgpu_status build_weights(Ctx* c, const GridDesc& g, const FieldDesc& bsdf,
                            const FieldDesc& fsdf, bool pyramid,
                            cudaEvent_t fluid_ready) {
    Level& L0 = c->levels[0];
    const Dims n = L0.n;
    const Dims fu{n.x + 1, n.y, n.z}, fv{n.x, n.y + 1, n.z},
        fw{n.x, n.y, n.z + 1};
    if (bsdf.kind == 1 || fsdf.kind == 1) {
        jetgpu_status s = ensure_tables(c, g, bsdf, fsdf);
        if (s != JETGPU_OK) return s;
    }
    const SampleTables& T = c->tabs;
    const TabLayout TL = layout_of(T);
    {
        Prof pr(c, K_WEIGHTS, (8.0 + 3.0 * 4.0) * (double)n.count());
        if (bsdf.kind == 1 && T.use_nodes) {
            const int3 S = make_int3(T.nslot[0], T.nslot[1], T.nslot[2]);
            const int3 so = make_int3(T.soff[0], T.soff[1], T.soff[2]);
            const long nodes = (long)S.x * S.y * S.z;
            k_node_grid<<<blocks_for(nodes), kThreads, 0, c->stream>>>(
                bsdf, T.sidx, T.sfrac, so, S, T.node);
            float* wts[3] = {L0.uw, L0.vw, L0.ww};
            const Dims fd[3] = {fu, fv, fw};
            jetgpu_status gs = grow_list(c, (size_t)std::max(
                                                std::max(fu.count(), fv.count()),
                                                fw.count()));
            if (gs != JETGPU_OK) return gs;
            auto axis_pass = [&](auto first, auto listed, int a) {
                JG_CUDA(c, cudaMemsetAsync(c->build_cnt, 0, sizeof(unsigned),
                                           c->stream));
                first<<<blocks_for(fd[a].count()), kThreads, 0, c->stream>>>(
                    wts[a], fd[a], T.slot, TL, S, T.node, c->build_list,
                    c->build_cnt);
                listed<<<c->num_sms * 8, kThreads, 0, c->stream>>>(
                    wts[a], fd[a], T.slot, TL, S, T.node, c->build_list,
                    c->build_cnt);
                return JETGPU_OK;
            };
            if ((gs = axis_pass(k_face_weights_nodes<0>,
                                k_face_weights_listed<0>, 0)) != JETGPU_OK ||
                (gs = axis_pass(k_face_weights_nodes<1>,
                                k_face_weights_listed<1>, 1)) != JETGPU_OK ||
                (gs = axis_pass(k_face_weights_nodes<2>,
                                k_face_weights_listed<2>, 2)) != JETGPU_OK)
                return gs;
        } else if (bsdf.kind == 0) {
            k_fill_face_weight<<<grid_cap(c, fu.count()), kThreads, 0,
                                 c->stream>>>(L0.uw, fu.count(), bsdf.value);
            k_fill_face_weight<<<grid_cap(c, fv.count()), kThreads, 0,
                                 c->stream>>>(L0.vw, fv.count(), bsdf.value);
            k_fill_face_weight<<<grid_cap(c, fw.count()), kThreads, 0,
                                 c->stream>>>(L0.ww, fw.count(), bsdf.value);
        } else {
            k_face_weights<<<blocks_for(fu.count()), kThreads, 0, c->stream>>>(
                L0.uw, 0, fu, g, bsdf);
            k_face_weights<<<blocks_for(fv.count()), kThreads, 0, c->stream>>>(
                L0.vw, 1, fv, g, bsdf);
            k_face_weights<<<blocks_for(fw.count()), kThreads, 0, c->stream>>>(
                L0.ww, 2, fw, g, bsdf);
        }
    }
    // The fluid SDF's samples after the face weights, which need only the
    // collider SDF (a host-pointer solve uploads that one first).
    if (fluid_ready) JG_CUDA(c, cudaStreamWaitEvent(c->stream, fluid_ready, 0));
    {
        Prof pr(c, K_WEIGHTS, (8.0 + 4.0) * (double)n.count());
        if (fsdf.kind == 1) {
            int* irregular = nullptr;
            if (T.fluid_on_cells) {
                irregular = T.irregular;
                JG_CUDA(c, cudaMemsetAsync(irregular, 0, sizeof(int),
                                           c->stream));
                k_values_regular<<<grid_cap(c, n.count()), kThreads, 0,
                                   c->stream>>>(fsdf.data, n.count(),
                                                irregular);
            }
            k_sample_fluid_tab<<<blocks_for(n.count()), kThreads, 0,
                                 c->stream>>>(L0.phi, n, fsdf, T.idx, T.frac,
                                              TL, irregular);
        }
        else if (fsdf.kind == 0)
            k_fill_fluid<<<grid_cap(c, n.count()), kThreads, 0, c->stream>>>(
                L0.phi, n.count(), fsdf.value);
        else
            k_sample_fluid<<<blocks_for(n.count()), kThreads, 0, c->stream>>>(
                L0.phi, n, g, fsdf);
    }
    JG_CUDA(c, cudaGetLastError());
    return pyramid ? build_pyramid(c) : JETGPU_OK;
}

jetgpu_status build_pyramid(Ctx* c) {
    const unsigned nl = c->built_levels;
    Prof pyr(c, K_PYRAMID, 0.0);
    for (unsigned l = 1; l < nl; ++l) {
        const Level& F = c->levels[l - 1];
        Level& C = c->levels[l];
        const Dims f = F.n, s = C.n;
        // Arrays whose x axis is fully restricted take the paired kernel
        // when the coarse rows have even length.
        auto full_x = [&](const float* fine, Dims fd, float* coarse, Dims cd) {
            if (cd.x % 2 == 0)
                k_restrict_f32x2<<<blocks_for(cd.count() / 2), kThreads, 0,
                                   c->stream>>>(fine, fd, coarse, cd);
            else
                k_restrict_f32<<<blocks_for(cd.count()), kThreads, 0,
                                 c->stream>>>(fine, fd, coarse, cd);
        };
        full_x(F.phi, f, C.phi, s);
        k_restrict_f32<<<blocks_for((long)(s.x + 1) * s.y * s.z), kThreads, 0,
                         c->stream>>>(F.uw, Dims{f.x + 1, f.y, f.z}, C.uw,
                                      Dims{s.x + 1, s.y, s.z});
        full_x(F.vw, Dims{f.x, f.y + 1, f.z}, C.vw, Dims{s.x, s.y + 1, s.z});
        full_x(F.ww, Dims{f.x, f.y, f.z + 1}, C.ww, Dims{s.x, s.y, s.z + 1});
    }
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

// 1/h and 1/h^2 as the kernel's double arithmetic forms them, with their
// power-of-two exponents when every factor is an exact power of two.
SpacingInv spacing_inv(double hx, double hy, double hz) {
    SpacingInv S;
    const double h[3] = {hx, hy, hz};
    S.pow2 = 1;
    for (int a = 0; a < 3; ++a) {
        S.ih[a] = 1.0 / h[a];
        S.ih2[a] = S.ih[a] * S.ih[a];
        int e1 = 0, e2 = 0;
        const double m1 = std::frexp(S.ih[a], &e1);
        const double m2 = std::frexp(S.ih2[a], &e2);
        S.k[a] = e1 - 1;
        S.k2[a] = e2 - 1;
        if (m1 != 0.5 || m2 != 0.5) S.pow2 = 0;
    }
    return S;
}

jetgpu_status build_system(Ctx* c, const GridDesc& g, const double* u,
                           const double* v, const double* w,
                           const double* su, const double* sv,
                           const double* sw, unsigned lo, unsigned hi) {
    double hx = g.spacing[0], hy = g.spacing[1], hz = g.spacing[2];
    for (unsigned l = 0; l < c->built_levels && l < hi; ++l) {
        Level& L = c->levels[l];
        if (l > 0) {
            hx *= 2.0;
            hy *= 2.0;
            hz *= 2.0;
        }
        L.h[0] = hx;
        L.h[1] = hy;
        L.h[2] = hz;
        if (l < lo) continue;
        const bool top = (l == 0);
        Prof pr(c, K_SYSTEM, (top ? 16.0 + 32.0 + 8.0 + 24.0 : 16.0 + 16.0) *
                                (double)L.n.count());
        k_build_system<false><<<blocks_for(L.n.count()), kThreads, 0,
                                c->stream>>>(
            L.n, spacing_inv(hx, hy, hz), L.phi, L.uw, L.vw, L.ww,
            top ? u : nullptr,
            top ? v : nullptr, top ? w : nullptr, top ? su : nullptr,
            top ? sv : nullptr, top ? sw : nullptr, top ? c->A64 : nullptr,
            top ? c->b64 : nullptr, L.A, top ? c->Alo : nullptr,
            top ? c->bdf : nullptr, nullptr);
    }
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

jetgpu_status build_system0_rows(Ctx* c, const GridDesc& g) {
    Level& L = c->levels[0];
    const long N = L.n.count();
    if (c->rflag_cap < (size_t)N) {
        JG_CUDA(c, cudaStreamSynchronize(c->stream));
        if (c->rflag) cudaFree(c->rflag);
        c->rflag = nullptr;
        c->rflag_cap = 0;
        JG_CUDA(c, cudaMalloc((void**)&c->rflag, (size_t)N));
        c->rflag_cap = (size_t)N;
    }
    L.h[0] = g.spacing[0];
    L.h[1] = g.spacing[1];
    L.h[2] = g.spacing[2];
    Prof pr(c, K_SYSTEM, (16.0 + 32.0 + 1.0) * (double)N);
    k_build_system<true><<<blocks_for(N), kThreads, 0, c->stream>>>(
        L.n, spacing_inv(g.spacing[0], g.spacing[1], g.spacing[2]), L.phi,
        L.uw, L.vw, L.ww, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
        c->A64, nullptr, L.A, c->Alo, nullptr, c->rflag);
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

jetgpu_status build_system0_rhs(Ctx* c, const GridDesc& g, const double* u,
                                const double* v, const double* w,
                                const double* su, const double* sv,
                                const double* sw) {
    const Level& L = c->levels[0];
    const long N = L.n.count();
    Prof pr(c, K_SYSTEM, (1.0 + 12.0 + 24.0 + 8.0 + 8.0) * (double)N);
    k_build_rhs<<<blocks_for(N), kThreads, 0, c->stream>>>(
        L.n, spacing_inv(g.spacing[0], g.spacing[1], g.spacing[2]), c->rflag,
        L.uw, L.vw, L.ww, u, v, w, su, sv, sw, c->b64, c->bdf);
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

jetgpu_status split_system(Ctx* c) {
    const long N = c->levels[0].n.count();
    k_split_system<<<blocks_for(N), kThreads, 0, c->stream>>>(
        c->A64, c->b64, c->Alo, c->bdf, N);
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

static bool aligned16(const void* p) {
    return (reinterpret_cast<unsigned long long>(p) & 15ull) == 0ull;
}

jetgpu_status apply_gradient(Ctx* c, const GridDesc& g, const double* u,
                             const double* v, const double* w, double* ou,
                             double* ov, double* ow, int kz0, int kz1) {
    const Level& L = c->levels[0];
    const Dims n = L.n;
    const bool alias = (ou == u) && (ov == v) && (ow == w);
    if (!alias && ((ou == u) || (ov == v) || (ow == w)))
        return fail(c, JETGPU_BAD_INPUT,
                    "output faces must all alias the input or none");
    if (kz1 < 0) kz1 = n.z;
    if (kz0 < 0 || kz0 > kz1 || kz1 > n.z)
        return fail(c, JETGPU_BAD_INPUT, "gradient planes out of range");
    if (kz0 == kz1) return JETGPU_OK;
    const long cells = (long)(kz1 - kz0) * n.x * n.y;
    Prof pr(c, K_GRADIENT, (4.0 + 12.0 + 8.0 + 48.0) * (double)cells);
    if (n.x % 4 == 0 && aligned16(u) && aligned16(v) && aligned16(w) &&
        aligned16(ou) && aligned16(ov) && aligned16(ow))
        k_apply_gradient4<<<blocks_for(cells / 4), kThreads, 0, c->stream>>>(
            n, spacing_inv(g.spacing[0], g.spacing[1], g.spacing[2]), L.phi,
            L.uw, L.vw, L.ww, c->x64, u, v, w, ou, ov, ow, kz0, kz1);
    else
        k_apply_gradient<<<blocks_for(cells), kThreads, 0, c->stream>>>(
            n, spacing_inv(g.spacing[0], g.spacing[1], g.spacing[2]), L.phi,
            L.uw, L.vw, L.ww, c->x64, u, v, w, ou, ov, ow, alias ? 0 : 1,
            kz0, kz1);
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

}  // namespace jg

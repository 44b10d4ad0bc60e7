// Trilinear sampling of Jet's grids in double precision, shared by the
// units that replay the reference's arithmetic bit for bit (built with
// -fmad=false, so no multiply-add is contracted).
//
// bary / sample_face restate getBarycentric
// (include/jet/detail/math_utils-inl.h:147-172) and
// LinearArraySampler3::operator() (include/jet/detail/array_samplers3-inl.h:
// 115-149); FaceSet holds the data origins of a FaceCenteredGrid3's three
// face arrays (src/jet/face_centered_grid3.cpp:428-445).
#pragma once

#include <cmath>

#include "common.cuh"

namespace jg {
namespace smp {

// The bit pattern of a double and back. On the device the words move
// through PTX, which keeps the integer tests on them from being turned back
// into FP64 compares and conversions (GB300 issues FP64 at a small fraction
// of its integer rate).
__host__ __device__ __forceinline__ unsigned long long dbits(double x) {
#ifdef __CUDA_ARCH__
    unsigned lo, hi;
    asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "d"(x));
    return ((unsigned long long)hi << 32) | lo;
#else
    unsigned long long b;
    __builtin_memcpy(&b, &x, 8);
    return b;
#endif
}

__host__ __device__ __forceinline__ double bitsd(unsigned long long b) {
#ifdef __CUDA_ARCH__
    double x;
    asm("mov.b64 %0, {%1, %2};"
        : "=d"(x)
        : "r"((unsigned)b), "r"((unsigned)(b >> 32)));
    return x;
#else
    double x;
    __builtin_memcpy(&x, &b, 8);
    return x;
#endif
}

// The FP64 fallbacks of the shortcuts below, out of line: a call keeps the
// compiler from predicating these FP64 instructions into every evaluation,
// where they would occupy the FP64 pipe even when the shortcut is taken.
static __host__ __device__ __noinline__ double mul_slow(double x, double y) {
    return x * y;
}

// x * 2^k (scale = 2^k) exactly: an exponent add on the integer pipe when
// x and the result are normal; zeros pass through; anything else takes the
// FP64 multiply, which rounds the same way.
__host__ __device__ __forceinline__ double scale_exact(double x, int k,
                                                       double scale) {
    const unsigned long long b = dbits(x);
    if ((b << 1) == 0ull) return x;
    const int e = (int)((b >> 52) & 0x7ffu);
    if (e > 0 && e < 0x7ff && e + k > 0 && e + k < 0x7ff)
        return bitsd(b + ((unsigned long long)(long long)k << 52));
    return mul_slow(x, scale);
}

// x / d for a divisor known to be positive: a zero x is the quotient itself
// (IEEE: +-0 / d = +-0 for d > 0), which keeps zero numerators off the
// FP64 divide's special-operand path (several times the cost of a normal
// divide on GB300).
__host__ __device__ __forceinline__ double div_pos(double x, double d) {
    return x == 0.0 ? x : x / d;
}

// x / h for a grid spacing h. IEEE division and multiplication both return
// the correctly rounded exact result, and when h is a power of two x / h and
// x * (1 / h) are the same real number (x * 2^k), so scaling the exponent
// gives the reference's quotient bit for bit without an FP64 divide.
struct Spacing {
    double h, inv;
    int pow2;
    int k;  // inv = 2^k when pow2
    __device__ __forceinline__ double div(double x) const {
        return pow2 ? scale_exact(x, k, inv) : x / h;
    }
};
inline Spacing make_spacing(double h) {
    int e = 0;
    const bool p2 = std::frexp(h, &e) == 0.5;  // h = 2^(e-1)
    return Spacing{h, 1.0 / h, p2 ? 1 : 0, p2 ? 1 - e : 0};
}

template <typename T>
__device__ __forceinline__ void bary(T x, int iHigh, int* i, T* f) {
    T s = floor(x);
    if (iHigh == 0) {
        *i = 0;
        *f = (T)0;
    } else if (s < (T)0) {
        *i = 0;
        *f = (T)0;
    } else if (s > (T)(iHigh - 1)) {
        *i = iHigh - 1;
        *f = (T)1;
    } else {
        *i = (int)s;
        *f = x - s;
    }
}

// The same (i, f) as bary<double>, computed on the integer pipe from the bit
// pattern (GB300 issues FP64 at a small fraction of its integer rate):
//   x < 0 or -0     -> (0, +0)             (floor(x) < 0; -0 gives f = +0)
//   x >= iHigh      -> (iHigh - 1, 1)      (floor(x) > iHigh - 1)
//   0 <= x < iHigh  -> (trunc(x), x - trunc(x))
// x - floor(x) is exact in IEEE arithmetic (its bits are the fraction bits
// of x), so assembling it from those bits gives the FP64 subtraction's
// result bit for bit. A NaN gives (0, NaN) as the FP64 form does (floor,
// both tests false, int conversion of NaN = 0, NaN - NaN).
__host__ __device__ __forceinline__ void bary_bits(double x, int iHigh,
                                                    int* i, double* f) {
    const unsigned long long X = dbits(x);
    const unsigned ex = (unsigned)(X >> 52) & 0x7ffu;
    if (iHigh == 0) {
        *i = 0;
        *f = 0.0;
        return;
    }
    if (X >> 63) {  // negative, -0 or a negative NaN
        *i = 0;
        *f = (ex == 0x7ffu && (X << 12)) ? x : 0.0;
        return;
    }
    if (ex == 0x7ffu && (X << 12)) {  // positive NaN
        *i = 0;
        *f = x;
        return;
    }
    if (X >= dbits((double)iHigh)) {
        *i = iHigh - 1;
        *f = 1.0;
        return;
    }
    const int e = (int)ex - 1023;  // x < iHigh <= 2^31, so e <= 30
    if (e < 0) {                   // 0 <= x < 1
        *i = 0;
        *f = x;
        return;
    }
    const unsigned long long M = (X & 0xfffffffffffffull) | (1ull << 52);
    const int sh = 52 - e;         // fraction bits of x
    *i = (int)(M >> sh);
    const unsigned long long F = M & ((1ull << sh) - 1ull);
    if (F == 0ull) {
        *f = 0.0;
        return;
    }
#ifdef __CUDA_ARCH__
    const int p = 63 - __clzll((long long)F);  // top set bit of F
#else
    const int p = 63 - __builtin_clzll(F);
#endif
    // f = F * 2^-sh, top bit at p: exponent p - sh, mantissa F << (52 - p).
    const unsigned long long be = (unsigned long long)(p - sh + 1023);
    *f = bitsd((be << 52) | ((F << (52 - p)) & 0xfffffffffffffull));
}

template <>
__device__ __forceinline__ void bary<double>(double x, int iHigh, int* i,
                                             double* f) {
    bary_bits(x, iHigh, i, f);
}

// F * 2^-sh for 0 < F <= 2^sh, sh <= 52 (exactly representable: at most 53
// significant bits), assembled on the integer pipe.
__host__ __device__ __forceinline__ double fixed_to_double(
    unsigned long long F, int sh) {
#ifdef __CUDA_ARCH__
    const int p = 63 - __clzll((long long)F);
#else
    const int p = 63 - __builtin_clzll(F);
#endif
    const unsigned long long be = (unsigned long long)(p - sh + 1023);
    return bitsd((be << 52) | ((F << (52 - p)) & 0xfffffffffffffull));
}

static __host__ __device__ __noinline__ double one_minus_slow(double f) {
    return 1 - f;
}

// bary_bits plus g = 1 - f, the reference's (1 - fx), bit for bit. For
// 1 <= x < iHigh the fraction is a multiple of x's last place 2^(e-52), so
// 1 - f = (2^sh - F) * 2^-sh is exactly representable and is assembled from
// that integer; the clamped ends give the constants 1 - 0 = 1 and
// 1 - 1 = +0; f = x < 1 (which 1 - f may round) and NaN take the FP64
// subtraction.
__host__ __device__ __forceinline__ void bary_bits2(double x, int iHigh,
                                                     int* i, double* f,
                                                     double* g) {
    const unsigned long long X = dbits(x);
    const int e = (int)((X >> 52) & 0x7ffu) - 1023;
    if (iHigh != 0 && !(X >> 63) && e >= 0 && X < dbits((double)iHigh)) {
        const unsigned long long M = (X & 0xfffffffffffffull) | (1ull << 52);
        const int sh = 52 - e;  // x < iHigh <= 2^31: 22 <= sh <= 52
        *i = (int)(M >> sh);
        const unsigned long long F = M & ((1ull << sh) - 1ull);
        *f = F ? fixed_to_double(F, sh) : 0.0;
        *g = fixed_to_double((1ull << sh) - F, sh);
        return;
    }
    bary_bits(x, iHigh, i, f);
    const unsigned long long fb = dbits(*f);
    if (fb == 0ull)
        *g = 1.0;
    else if (fb == dbits(1.0))
        *g = 0.0;
    else
        *g = one_minus_slow(*f);
}

// The reference's lerp (include/jet/detail/math_utils-inl.h),
// (1 - f) * a + f * b, evaluated as the same IEEE operations.
__host__ __device__ __forceinline__ double lerp_ref(double a, double b,
                                                    double f) {
    return (1.0 - f) * a + f * b;
}

// The same value with the fractions that grid-aligned samples produce taken
// on the integer pipe:
//  * f = 0.5: both products are exact halvings, so the result is the one
//    rounding of (a + b) / 2 = half(RN(a + b)) — exact whenever a and b are
//    zero or have exponent fields in [2, 0x7fd] (no overflow of a + b; a
//    sum small enough for its half to be subnormal is exact, and so is that
//    half);
//  * f = 0: the result is 1 * a + 0 * b, which is a itself when a is
//    non-zero and b finite;
//  * f = 1: 0 * a + 1 * b, which is b when b is non-zero and a finite.
// Anything else takes the reference's expression. fb is the bit pattern of
// f (computed once per axis by the caller).
__host__ __device__ __forceinline__ unsigned expo_bits(unsigned long long x) {
    return (unsigned)(x >> 52) & 0x7ffu;
}
__host__ __device__ __forceinline__ bool half_safe(unsigned long long x) {
    const unsigned e = expo_bits(x);
    return (e >= 2u && e <= 0x7fdu) || (x << 1) == 0ull;
}
__host__ __device__ __forceinline__ double half_exact(double x) {
    const unsigned long long b = dbits(x);
    const unsigned e = expo_bits(b);
    if (e > 1u && e < 0x7ffu) return bitsd(b - (1ull << 52));
    return mul_slow(x, 0.5);
}
static __host__ __device__ __noinline__ double lerp_slow(double a, double b,
                                                         double f) {
    return lerp_ref(a, b, f);
}
constexpr unsigned long long kHalfD = 0x3FE0000000000000ull;
constexpr unsigned long long kOneD = 0x3FF0000000000000ull;
__host__ __device__ __forceinline__ double lerp_fast(double a, double b,
                                                     double f,
                                                     unsigned long long fb) {
    if (fb == kHalfD) {
        const unsigned long long A = dbits(a), B = dbits(b);
        if (half_safe(A) && half_safe(B)) return half_exact(a + b);
    } else if (fb == 0ull) {
        if ((dbits(a) << 1) != 0ull && expo_bits(dbits(b)) != 0x7ffu) return a;
    } else if (fb == kOneD) {
        if ((dbits(b) << 1) != 0ull && expo_bits(dbits(a)) != 0x7ffu) return b;
    }
    return lerp_slow(a, b, f);
}

template <typename T>
__device__ __forceinline__ T lerp_t(T a, T b, T f) {
    return ((T)1 - f) * a + f * b;
}

// trilerp (include/jet/detail/math_utils-inl.h:177-211): x first, then y,
// then z.
template <typename T>
__device__ __forceinline__ T trilerp(T f000, T f100, T f010, T f110, T f001,
                                     T f101, T f011, T f111, T fx, T fy,
                                     T fz) {
    const T b0 = lerp_t(lerp_t(f000, f100, fx), lerp_t(f010, f110, fx), fy);
    const T b1 = lerp_t(lerp_t(f001, f101, fx), lerp_t(f011, f111, fx), fy);
    return lerp_t(b0, b1, fz);
}
// A fraction for which lerp_fast has an integer-pipe shortcut.
__host__ __device__ __forceinline__ bool aligned_frac(unsigned long long fb) {
    return fb == 0ull || fb == kHalfD || fb == kOneD;
}
static __device__ __noinline__ double trilerp_slow(
    double f000, double f100, double f010, double f110, double f001,
    double f101, double f011, double f111, double fx, double fy, double fz) {
    const double b0 = lerp_ref(lerp_ref(f000, f100, fx),
                               lerp_ref(f010, f110, fx), fy);
    const double b1 = lerp_ref(lerp_ref(f001, f101, fx),
                               lerp_ref(f011, f111, fx), fy);
    return lerp_ref(b0, b1, fz);
}

// trilerp for samples taken at grid-aligned points of the sampled grid
// (faces, nodes, cell centres): when all three fractions are 0, 1/2 or 1 the
// lerps take the integer-pipe shortcuts; any other sample runs the
// reference's lerps unchanged, with one test per sample.
__device__ __forceinline__ double trilerp_grid(
    double f000, double f100, double f010, double f110, double f001,
    double f101, double f011, double f111, double fx, double fy, double fz) {
    const unsigned long long bx = dbits(fx), by = dbits(fy), bz = dbits(fz);
    if (aligned_frac(bx) && aligned_frac(by) && aligned_frac(bz)) {
        const double b0 = lerp_fast(lerp_fast(f000, f100, fx, bx),
                                    lerp_fast(f010, f110, fx, bx), fy, by);
        const double b1 = lerp_fast(lerp_fast(f001, f101, fx, bx),
                                    lerp_fast(f011, f111, fx, bx), fy, by);
        return lerp_fast(b0, b1, fz, bz);
    }
    return trilerp_slow(f000, f100, f010, f110, f001, f101, f011, f111, fx,
                        fy, fz);
}

// Trilinear sample of a face array with the reference's operator() rule
// (normalised coordinate = (x - origin) / spacing).
template <typename V, typename T>
__device__ T sample_face(const V* __restrict__ d, Dims s, T nx, T ny, T nz) {
    int i, j, k;
    T fx, fy, fz;
    bary<T>(nx, s.x - 1, &i, &fx);
    bary<T>(ny, s.y - 1, &j, &fy);
    bary<T>(nz, s.z - 1, &k, &fz);
    const int ip1 = min(i + 1, s.x - 1), jp1 = min(j + 1, s.y - 1),
              kp1 = min(k + 1, s.z - 1);
    const T f000 = d[lin(i, j, k, s.x, s.y)], f100 = d[lin(ip1, j, k, s.x, s.y)];
    const T f010 = d[lin(i, jp1, k, s.x, s.y)], f110 = d[lin(ip1, jp1, k, s.x, s.y)];
    const T f001 = d[lin(i, j, kp1, s.x, s.y)], f101 = d[lin(ip1, j, kp1, s.x, s.y)];
    const T f011 = d[lin(i, jp1, kp1, s.x, s.y)], f111 = d[lin(ip1, jp1, kp1, s.x, s.y)];
    return trilerp<T>(f000, f100, f010, f110, f001, f101, f011, f111, fx, fy,
                      fz);
}

// sample_face<double, double> with the complements 1 - f of the fractions
// taken from the coordinate's bits (bary_bits2) instead of the FP64
// subtraction: the same bits, three FP64 operations fewer per sample.
__device__ __forceinline__ double lerp_g(double a, double b, double f,
                                         double g) {
    return g * a + f * b;
}
__device__ __forceinline__ double sample_face_d(const double* __restrict__ d,
                                                Dims s, double nx, double ny,
                                                double nz) {
    int i, j, k;
    double fx, fy, fz, gx, gy, gz;
    bary_bits2(nx, s.x - 1, &i, &fx, &gx);
    bary_bits2(ny, s.y - 1, &j, &fy, &gy);
    bary_bits2(nz, s.z - 1, &k, &fz, &gz);
    const int ip1 = min(i + 1, s.x - 1), jp1 = min(j + 1, s.y - 1),
              kp1 = min(k + 1, s.z - 1);
    const double f000 = d[lin(i, j, k, s.x, s.y)], f100 = d[lin(ip1, j, k, s.x, s.y)];
    const double f010 = d[lin(i, jp1, k, s.x, s.y)], f110 = d[lin(ip1, jp1, k, s.x, s.y)];
    const double f001 = d[lin(i, j, kp1, s.x, s.y)], f101 = d[lin(ip1, j, kp1, s.x, s.y)];
    const double f011 = d[lin(i, jp1, kp1, s.x, s.y)], f111 = d[lin(ip1, jp1, kp1, s.x, s.y)];
    const double b0 = lerp_g(lerp_g(f000, f100, fx, gx),
                             lerp_g(f010, f110, fx, gx), fy, gy);
    const double b1 = lerp_g(lerp_g(f001, f101, fx, gx),
                             lerp_g(f011, f111, fx, gx), fy, gy);
    return lerp_g(b0, b1, fz, gz);
}

// sample_face for points that usually sit on the sampled grid's lattice
// (collider SDF at faces and cell centres, SDFs at nodes): same result, with
// trilerp_grid's shortcuts. Particle positions use sample_face.
__device__ __forceinline__ double sample_face_grid(const double* __restrict__ d,
                                                   Dims s, double nx,
                                                   double ny, double nz) {
    int i, j, k;
    double fx, fy, fz;
    bary<double>(nx, s.x - 1, &i, &fx);
    bary<double>(ny, s.y - 1, &j, &fy);
    bary<double>(nz, s.z - 1, &k, &fz);
    const int ip1 = min(i + 1, s.x - 1), jp1 = min(j + 1, s.y - 1),
              kp1 = min(k + 1, s.z - 1);
    return trilerp_grid(
        d[lin(i, j, k, s.x, s.y)], d[lin(ip1, j, k, s.x, s.y)],
        d[lin(i, jp1, k, s.x, s.y)], d[lin(ip1, jp1, k, s.x, s.y)],
        d[lin(i, j, kp1, s.x, s.y)], d[lin(ip1, j, kp1, s.x, s.y)],
        d[lin(i, jp1, kp1, s.x, s.y)], d[lin(ip1, jp1, kp1, s.x, s.y)], fx,
        fy, fz);
}

struct FaceSet {
    Dims s[3];
    double o[3][3];
};

inline FaceSet face_set(const GridDesc& g) {
    FaceSet f;
    const int nx = g.res[0], ny = g.res[1], nz = g.res[2];
    f.s[0] = Dims{nx + 1, ny, nz};
    f.s[1] = Dims{nx, ny + 1, nz};
    f.s[2] = Dims{nx, ny, nz + 1};
    for (int a = 0; a < 3; ++a)
        for (int d = 0; d < 3; ++d)
            f.o[a][d] = g.origin[d] + 0.5 * (a == d ? 0.0 : g.spacing[d]);
    return f;
}

}  // namespace smp
}  // namespace jg

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

// x / h for a grid spacing h. IEEE division and multiplication both return
// the correctly rounded exact result, and when h is a power of two x / h and
// x * (1 / h) are the same real number (x * 2^-k), so the multiply gives the
// reference's quotient bit for bit at a fraction of an FP64 divide's cost.
struct Spacing {
    double h, inv;
    int pow2;
    __device__ __forceinline__ double div(double x) const {
        return pow2 ? x * inv : x / h;
    }
};
inline Spacing make_spacing(double h) {
    int e = 0;
    return Spacing{h, 1.0 / h, std::frexp(h, &e) == 0.5 ? 1 : 0};
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

template <typename T>
__device__ __forceinline__ T lerp_t(T a, T b, T f) {
    return ((T)1 - f) * a + f * b;
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
    const T b0 = lerp_t(lerp_t(f000, f100, fx), lerp_t(f010, f110, fx), fy);
    const T b1 = lerp_t(lerp_t(f001, f101, fx), lerp_t(f011, f111, fx), fy);
    return lerp_t(b0, b1, fz);
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

// Boundary conditions on the face-centred velocity (the first widening of
// the pressure path: these run right after every projection and around the
// particle transfers of a FLIP/PIC step).
//
// constrain_velocity replaces
// GridFractionalBoundaryConditionSolver3::constrainVelocity
// (src/jet/grid_fractional_boundary_condition_solver3.cpp:26-233):
//   K19a  faces whose collider fraction 1 - fractionInsideSdf(phi(x - h/2),
//         phi(x + h/2)) is 0 take the collider velocity and are marked
//         invalid (:51-100);
//   K19b  extrapolateToRegion from the valid faces, `depth` Jacobi passes
//         (include/jet/detail/array_utils-inl.h:172-244; a pass writes only
//         cells invalid at its start and reads only cells valid at its start,
//         so it is order-independent and runs in place);
//   K19c  faces inside the collider get the velocity sampled there projected
//         onto the collider's tangent plane with friction
//         (projectAndApplyFriction, src/jet/physics_helpers.h:34-45), the
//         normal from the collider SDF's gradient (ScalarGrid3::gradient,
//         src/jet/scalar_grid3.cpp:89-102, over gradient3,
//         src/jet/fdm_utils.cpp:49-67), into a temporary (:110-175);
//   K19d  copy back and zero the normal velocity on closed domain faces
//         (:177-232).
// The unit is built with -fmad=false and evaluates every expression in the
// reference's order, so results are bit-identical to the reference.
// Bound: HBM (K19a reads 16 B of SDF samples per face from L2-resident
// neighbourhoods; K19b reads 7 values + validity per invalid face per pass).

#include "ctx.h"
#include "sampling.cuh"

namespace jg {
namespace {

using namespace smp;

struct ColliderDesc {
    int present;
    double lin[3], ang[3], centre[3];
    double friction;
};

// RigidBodyCollider3::velocityAt (src/jet/rigid_body_collider3.cpp:25-28)
// with Vector3::cross (include/jet/detail/vector3-inl.h:125-127).
__device__ __forceinline__ void collider_vel(const ColliderDesc& c,
                                             const double p[3], double o[3]) {
    if (!c.present) {
        o[0] = o[1] = o[2] = 0.0;
        return;
    }
    const double r0 = p[0] - c.centre[0], r1 = p[1] - c.centre[1],
                 r2 = p[2] - c.centre[2];
    o[0] = c.lin[0] + (c.ang[1] * r2 - r1 * c.ang[2]);
    o[1] = c.lin[1] + (c.ang[2] * r0 - r2 * c.ang[0]);
    o[2] = c.lin[2] + (c.ang[0] * r1 - r0 * c.ang[1]);
}

struct S3 {
    Spacing s[3];
};

// CellCenteredScalarGrid3::sample (LinearArraySampler3::operator()); `fsp`
// holds the field's spacings.
__device__ double sample_sdf(const FieldDesc& F, const S3& fsp, double x,
                             double y, double z) {
    if (F.kind == 0) return F.value;
    const Dims s{F.res[0], F.res[1], F.res[2]};
    return sample_face_grid(F.data, s, fsp.s[0].div(x - F.origin[0]),
                                       fsp.s[1].div(y - F.origin[1]),
                                       fsp.s[2].div(z - F.origin[2]));
}

// std::max's rule (the first argument unless it is less than the second).
__device__ __forceinline__ double dmax(double a, double b) {
    return a < b ? b : a;
}

__device__ __forceinline__ double frac_inside_sdf(double p0, double p1) {
    const bool i0 = p0 < 0.0, i1 = p1 < 0.0;
    if (i0 && i1) return 1.0;
    if (i0 && !i1) return p0 / (p0 - p1);
    if (!i0 && i1) return p1 / (p1 - p0);
    return 0.0;
}

__device__ __forceinline__ void face_pos(const FaceSet& fs, int a,
                                         const double h[3], int i, int j,
                                         int k, double p[3]) {
    p[0] = fs.o[a][0] + h[0] * (double)i;
    p[1] = fs.o[a][1] + h[1] * (double)j;
    p[2] = fs.o[a][2] + h[2] * (double)k;
}

struct H3 {
    double v[3];
};

// Face classes: bit 0 = the collider fraction 1 - fractionInsideSdf(phi at
// the two ends of the face) is > 0 (a valid fluid face, :55-62); bit 1 = the
// face position is inside the collider (:113). They depend only on the
// collider SDF, so one pass serves every constrainVelocity call made while
// the collider stands still (all calls of a sub-step).
enum : unsigned char { kFaceValid = 1, kFaceInside = 2 };

// The three face arrays of one launch (blockIdx.y = axis): each axis's
// offset in the concatenated per-face buffers (classes, lists, validity,
// temporaries), its velocity array, and its slice of the normal cache.
struct Axes3 {
    long off[3];
    double* vel[3];
    long noff[3], ncap[3];
};

// Appends face c to a list when `take`; one atomic per warp.
__device__ __forceinline__ void push(int* __restrict__ lst,
                                     unsigned* __restrict__ cnt, long c,
                                     bool take) {
    const unsigned active = __activemask();
    const unsigned m = __ballot_sync(active, take);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(cnt, (unsigned)__popc(m));
    base = __shfl_sync(active, base, leader);
    if (take) lst[base + __popc(m & ((1u << lane) - 1u))] = (int)c;
}

// K19a: classification, and the lists of the faces later passes touch:
// those without a valid fraction (collider velocity, then extrapolated) and
// those inside the collider (projected). List order is arbitrary; every
// pass over a list is order-independent.
//
// With `irregular` non-null the collider SDF lies on the velocity grid's
// cell centres, the grid origin is +0 and the spacings are powers of two
// (checked on the host); the flag is 0 when every SDF value is finite and
// non-zero (checked by k_sdf_regular). Then a face's
// two end points are exactly the centres of the cells on either side and
// its centre exactly halfway (the coordinate arithmetic is exact), so the
// samples are the two cell values a and b (each lerp with fraction 0 gives
// its first operand) and half(a + b) (the fraction-1/2 rule, when a and b
// are in its safe exponent range); an interior face then reads two values.
// Boundary faces and out-of-range values take the samples.
__global__ void k_sdf_regular(const double* __restrict__ d, long n,
                              int* __restrict__ irregular) {
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n;
         c += (long)gridDim.x * blockDim.x) {
        const unsigned long long b = dbits(d[c]);
        if ((b << 1) == 0ull || ((b >> 52) & 0x7ffu) == 0x7ffu) *irregular = 1;
    }
}

__global__ void k_bc_classify(FaceSet fs, H3 h, FieldDesc sdf, S3 fsp,
                              Axes3 ax, long nf,
                              unsigned char* __restrict__ cls_all,
                              int* __restrict__ list_all,
                              unsigned* __restrict__ cnt_all,
                              const int* __restrict__ irregular) {
    const int a = blockIdx.y;
    const Dims s = fs.s[a];
    unsigned char* cls = cls_all + ax.off[a];
    int* inv_list = list_all + ax.off[a];
    unsigned* inv_cnt = cnt_all + a;
    int* in_list = list_all + nf + ax.off[a];
    unsigned* in_cnt = cnt_all + 3 + a;
    const long n = s.count();
    const bool reg = irregular && !*irregular;
    const Dims cd{sdf.res[0], sdf.res[1], sdf.res[2]};
    const long step = a == 0 ? 1 : (a == 1 ? (long)cd.x : (long)cd.x * cd.y);
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n;
         c += (long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_ijk(c, s, i, j, k);
        const int ia = a == 0 ? i : (a == 1 ? j : k);  // index along the axis
        if (reg && ia > 0 && ia < (a == 0 ? cd.x : (a == 1 ? cd.y : cd.z))) {
            // The cells on either side of the face.
            const long cb = lin(i, j, k, cd.x, cd.y);  // the upper cell
            const double va = sdf.data[cb - step], vb = sdf.data[cb];
            if (half_safe(dbits(va)) && half_safe(dbits(vb))) {
                double frac = frac_inside_sdf(va, vb);
                frac = 1.0 - (frac < 0.0 ? 0.0 : (frac > 1.0 ? 1.0 : frac));
                unsigned char f = frac > 0.0 ? kFaceValid : 0;
                if (va + vb < 0.0) f |= kFaceInside;
                cls[c] = f;
                push(inv_list, inv_cnt, c, !(f & kFaceValid));
                push(in_list, in_cnt, c, (f & kFaceInside) != 0);
                continue;
            }
        }
        double p[3], q0[3], q1[3];
        face_pos(fs, a, h.v, i, j, k, p);
        for (int d = 0; d < 3; ++d) {
            const double off = d == a ? 0.5 * h.v[d] : 0.0;
            q0[d] = p[d] - off;
            q1[d] = p[d] + off;
        }
        double frac =
            frac_inside_sdf(sample_sdf(sdf, fsp, q0[0], q0[1], q0[2]),
                            sample_sdf(sdf, fsp, q1[0], q1[1], q1[2]));
        frac = 1.0 - (frac < 0.0 ? 0.0 : (frac > 1.0 ? 1.0 : frac));
        unsigned char f = frac > 0.0 ? kFaceValid : 0;
        if (sample_sdf(sdf, fsp, p[0], p[1], p[2]) < 0.0) f |= kFaceInside;
        cls[c] = f;
        push(inv_list, inv_cnt, c, !(f & kFaceValid));
        push(in_list, in_cnt, c, (f & kFaceInside) != 0);
    }
}

// K19a': the faces without a valid fraction take the collider velocity
// (:63-67) and start the extrapolation invalid.
__global__ void k_bc_mark(FaceSet fs, H3 h, ColliderDesc col, Axes3 ax,
                          const int* __restrict__ list_all,
                          const unsigned* __restrict__ cnt_all,
                          unsigned char* __restrict__ st0_all) {
    const int a = blockIdx.y;
    const Dims s = fs.s[a];
    const int* lst = list_all + ax.off[a];
    const unsigned* cnt = cnt_all + a;
    double* vel = ax.vel[a];
    unsigned char* st0 = st0_all + ax.off[a];
    const long m = *cnt;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < m;
         t += (long)gridDim.x * blockDim.x) {
        const long c = lst[t];
        int i, j, k;
        cell_ijk(c, s, i, j, k);
        double p[3], cv[3];
        face_pos(fs, a, h.v, i, j, k, p);
        collider_vel(col, p, cv);
        vel[c] = cv[a];
        st0[c] = 0;
    }
}

// sum / count for a neighbour count in 1..6, the FP64 division's bits:
// counts 1, 2 and 4 are exact (a copy, or an exponent decrement on the
// integer pipe); 3, 5 and 6 divide.
static __device__ __noinline__ double div_slow(double x, double d) {
    return x / d;
}
__device__ __forceinline__ double div_count(double sum, unsigned count) {
    if (count == 1u) return sum;
    if (count == 2u) return scale_exact(sum, -1, 0.5);
    if (count == 4u) return scale_exact(sum, -2, 0.25);
    return sum == 0.0 ? sum : div_slow(sum, (double)count);
}

// K19b': one extrapolation pass over the listed (initially invalid) faces.
// A face outside the list is valid by its class; a listed face is valid
// when its state byte says so.
__global__ void k_extrapolate_list(FaceSet fs, Axes3 ax,
                                   const int* __restrict__ list_all,
                                   const unsigned* __restrict__ cnt_all,
                                   const unsigned char* __restrict__ cls_all,
                                   const unsigned char* __restrict__ st0_all,
                                   unsigned char* __restrict__ st1_all) {
    const int a = blockIdx.y;
    const Dims s = fs.s[a];
    const int* lst = list_all + ax.off[a];
    const long m = cnt_all[a];
    double* data = ax.vel[a];
    const unsigned char* cls = cls_all + ax.off[a];
    const unsigned char* st0 = st0_all + ax.off[a];
    unsigned char* st1 = st1_all + ax.off[a];
    const long sy = s.x, sz = (long)s.x * s.y;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < m;
         t += (long)gridDim.x * blockDim.x) {
        const long c = lst[t];
        if (st0[c]) {
            st1[c] = 1;
            continue;
        }
        int i, j, k;
        cell_ijk(c, s, i, j, k);
        auto ok = [&](long q) { return (cls[q] & kFaceValid) || st0[q]; };
        double sum = 0.0;
        unsigned count = 0;
        if (i + 1 < s.x && ok(c + 1)) { sum += data[c + 1]; ++count; }
        if (i > 0 && ok(c - 1)) { sum += data[c - 1]; ++count; }
        if (j + 1 < s.y && ok(c + sy)) { sum += data[c + sy]; ++count; }
        if (j > 0 && ok(c - sy)) { sum += data[c - sy]; ++count; }
        if (k + 1 < s.z && ok(c + sz)) { sum += data[c + sz]; ++count; }
        if (k > 0 && ok(c - sz)) { sum += data[c - sz]; ++count; }
        if (count > 0) {
            data[c] = div_count(sum, count);
            st1[c] = 1;
        } else {
            st1[c] = 0;
        }
    }
}

// K19b: extrapolateToRegion over its front. A pass of the reference
// changes only the invalid entries with a valid neighbour, so each pass here
// visits just those: an initial full pass stamps validity and lists the
// first front, a pass updates its listed entries (the reference's
// neighbour order and average), and the entries it made valid queue their
// still-open neighbours for the next pass. Stamps: 0 valid at the start,
// t + 1 made valid by pass t, kXpQueued listed for the coming pass, kXpOpen
// neither; an entry is valid for pass t when its stamp is <= t.
constexpr int kXpOpen = 0x7fffffff, kXpQueued = 0x7ffffffe;

// Up to three arrays extrapolated together (blockIdx.y = array): extents,
// data, validity, and offsets into the shared stamp and list buffers.
struct Xp3 {
    Dims s[3];
    double* data[3];
    const unsigned char* valid[3];
    long off[3];
};

__global__ void k_xp_init(Xp3 X, int* __restrict__ stamp_all,
                          int* __restrict__ lst_all,
                          unsigned* __restrict__ cnt_all) {
    const int r = blockIdx.y;
    const Dims s = X.s[r];
    const unsigned char* valid = X.valid[r];
    int* stamp = stamp_all + X.off[r];
    int* lst = lst_all + X.off[r];
    unsigned* cnt = cnt_all + r;
    const long n = s.count();
    const long sy = s.x, sz = (long)s.x * s.y;
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n;
         c += (long)gridDim.x * blockDim.x) {
        bool q = false;
        if (valid[c]) {
            stamp[c] = 0;
        } else {
            int i, j, k;
            cell_ijk(c, s, i, j, k);
            q = (i + 1 < s.x && valid[c + 1]) || (i > 0 && valid[c - 1]) ||
                (j + 1 < s.y && valid[c + sy]) || (j > 0 && valid[c - sy]) ||
                (k + 1 < s.z && valid[c + sz]) || (k > 0 && valid[c - sz]);
            stamp[c] = q ? kXpQueued : kXpOpen;
        }
        push(lst, cnt, c, q);
    }
}

// Pass t over its listed entries, in place on the data: a listed entry reads
// only neighbours valid before the pass (stamp <= t), which no thread of the
// pass writes.
__global__ void k_xp_pass(Xp3 X, int* __restrict__ stamp_all,
                          const int* __restrict__ lst_all,
                          const unsigned* __restrict__ cnt_all, int t) {
    const int r = blockIdx.y;
    const Dims s = X.s[r];
    double* data = X.data[r];
    int* stamp = stamp_all + X.off[r];
    const int* lst = lst_all + X.off[r];
    const long m = cnt_all[r];
    const long sy = s.x, sz = (long)s.x * s.y;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < m;
         e += (long)gridDim.x * blockDim.x) {
        const long c = lst[e];
        int i, j, k;
        cell_ijk(c, s, i, j, k);
        auto ok = [&](long q) { return stamp[q] <= t; };
        double sum = 0.0;
        unsigned count = 0;
        if (i + 1 < s.x && ok(c + 1)) { sum += data[c + 1]; ++count; }
        if (i > 0 && ok(c - 1)) { sum += data[c - 1]; ++count; }
        if (j + 1 < s.y && ok(c + sy)) { sum += data[c + sy]; ++count; }
        if (j > 0 && ok(c - sy)) { sum += data[c - sy]; ++count; }
        if (k + 1 < s.z && ok(c + sz)) { sum += data[c + sz]; ++count; }
        if (k > 0 && ok(c - sz)) { sum += data[c - sz]; ++count; }
        if (count > 0) data[c] = div_count(sum, count);
        stamp[c] = t + 1;
    }
}

// The next front: the open neighbours of the entries pass t made valid,
// each listed once (the stamp's compare-and-swap claims it).
__global__ void k_xp_next(Xp3 X, int* __restrict__ stamp_all,
                          const int* __restrict__ lst_all,
                          const unsigned* __restrict__ cnt_all,
                          int* __restrict__ nlst_all,
                          unsigned* __restrict__ ncnt_all) {
    const int r = blockIdx.y;
    const Dims s = X.s[r];
    int* stamp = stamp_all + X.off[r];
    const int* lst = lst_all + X.off[r];
    const long m = cnt_all[r];
    int* nlst = nlst_all + X.off[r];
    unsigned* ncnt = ncnt_all + r;
    const long sy = s.x, sz = (long)s.x * s.y;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < m;
         e += (long)gridDim.x * blockDim.x) {
        const long c = lst[e];
        int i, j, k;
        cell_ijk(c, s, i, j, k);
        const bool in[6] = {i + 1 < s.x, i > 0, j + 1 < s.y,
                            j > 0,       k + 1 < s.z, k > 0};
        const long d[6] = {1, -1, sy, -sy, sz, -sz};
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const long nb = c + d[q];
            const bool take = in[q] && stamp[nb] == kXpOpen &&
                              atomicCAS(&stamp[nb], kXpOpen, kXpQueued) ==
                                  kXpOpen;
            push(nlst, ncnt, nb, take);
        }
    }
}

// ScalarGrid3::gradient at p: trilinear weights of the cell-centred sampler
// (coordinates scaled by the inverse spacing, as getCoordinatesAndWeights
// does) over the clamped central differences of gradient3.
__device__ void sdf_gradient(const FieldDesc& F, const S3& fsp,
                             const double inv[3], const double p[3],
                             double g[3]) {
    g[0] = g[1] = g[2] = 0.0;
    if (F.kind == 0) return;
    const Dims s{F.res[0], F.res[1], F.res[2]};
    int i, j, k;
    double fx, fy, fz;
    bary<double>((p[0] - F.origin[0]) * inv[0], s.x - 1, &i, &fx);
    bary<double>((p[1] - F.origin[1]) * inv[1], s.y - 1, &j, &fy);
    bary<double>((p[2] - F.origin[2]) * inv[2], s.z - 1, &k, &fz);
    const int ip1 = min(i + 1, s.x - 1), jp1 = min(j + 1, s.y - 1),
              kp1 = min(k + 1, s.z - 1);
    const int ci[8] = {i, ip1, i, ip1, i, ip1, i, ip1};
    const int cj[8] = {j, j, jp1, jp1, j, j, jp1, jp1};
    const int ck[8] = {k, k, k, k, kp1, kp1, kp1, kp1};
    const double w[8] = {(1 - fx) * (1 - fy) * (1 - fz), fx * (1 - fy) * (1 - fz),
                         (1 - fx) * fy * (1 - fz),       fx * fy * (1 - fz),
                         (1 - fx) * (1 - fy) * fz,       fx * (1 - fy) * fz,
                         (1 - fx) * fy * fz,             fx * fy * fz};
    const double* d = F.data;
#pragma unroll
    for (int n = 0; n < 8; ++n) {
        const int x = ci[n], y = cj[n], z = ck[n];
        const double l = d[lin(x > 0 ? x - 1 : x, y, z, s.x, s.y)];
        const double r = d[lin(x + 1 < s.x ? x + 1 : x, y, z, s.x, s.y)];
        const double dn = d[lin(x, y > 0 ? y - 1 : y, z, s.x, s.y)];
        const double up = d[lin(x, y + 1 < s.y ? y + 1 : y, z, s.x, s.y)];
        const double bk = d[lin(x, y, z > 0 ? z - 1 : z, s.x, s.y)];
        const double fr = d[lin(x, y, z + 1 < s.z ? z + 1 : z, s.x, s.y)];
        const double gx = fsp.s[0].div(0.5 * (r - l));
        const double gy = fsp.s[1].div(0.5 * (up - dn));
        const double gz = fsp.s[2].div(0.5 * (fr - bk));
        g[0] = g[0] + w[n] * gx;
        g[1] = g[1] + w[n] * gy;
        g[2] = g[2] + w[n] * gz;
    }
}

// The collider's unit normal at face c of axis a (the SDF gradient over its
// length, :159-163): .w = 1 with the normal, .w = 0 where the gradient
// vanishes.
__device__ double4_32a bc_normal(const FaceSet& fs, int a, const H3& h,
                                 const S3& ssp, const H3& inv,
                                 const FieldDesc& sdf, long c) {
    int i, j, k;
    cell_ijk(c, fs.s[a], i, j, k);
    double p[3], g[3];
    face_pos(fs, a, h.v, i, j, k, p);
    sdf_gradient(sdf, ssp, inv.v, p, g);
    if (g[0] * g[0] + g[1] * g[1] + g[2] * g[2] > 0.0) {
        const double len = sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
        return make_double4_32a(div_pos(g[0], len), div_pos(g[1], len),
                                div_pos(g[2], len), 1.0);
    }
    return make_double4_32a(0.0, 0.0, 0.0, 0.0);
}

// The normals of the first `cap` listed inside faces, once per
// classification (the collider stands still over the passes that use them).
__global__ void k_bc_normals(FaceSet fs, H3 h, S3 ssp, H3 inv, FieldDesc sdf,
                             Axes3 ax, long nf, const int* __restrict__ list_all,
                             const unsigned* __restrict__ cnt_all,
                             double4_32a* __restrict__ nrm_all) {
    const int a = blockIdx.y;
    const int* lst = list_all + nf + ax.off[a];
    double4_32a* nrm = nrm_all + ax.noff[a];
    const long m = min((long)cnt_all[3 + a], ax.ncap[a]);
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < m;
         t += (long)gridDim.x * blockDim.x)
        nrm[t] = bc_normal(fs, a, h, ssp, inv, sdf, lst[t]);
}

// K19c: the listed faces inside the collider (the others keep their
// value); tmp[t] receives the projection of list entry t. Entries below
// `cap` take their normal from the classification's cache.
__global__ void k_bc_project(FaceSet fs, H3 h, S3 gsp, S3 ssp, H3 inv,
                             FieldDesc sdf, ColliderDesc col, Axes3 ax, long nf,
                             const int* __restrict__ list_all,
                             const unsigned* __restrict__ cnt_all,
                             const double4_32a* __restrict__ nrm_all,
                             double* __restrict__ tmp_all) {
    const int a = blockIdx.y;
    const Dims s = fs.s[a];
    const int* lst = list_all + nf + ax.off[a];
    const long m = cnt_all[3 + a];
    const double4_32a* nrm = nrm_all + ax.noff[a];
    const long cap = ax.ncap[a];
    double* tmp = tmp_all + ax.off[a];
    const double* vel[3] = {ax.vel[0], ax.vel[1], ax.vel[2]};
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < m;
         t += (long)gridDim.x * blockDim.x) {
        const long c = lst[t];
        int i, j, k;
        cell_ijk(c, s, i, j, k);
        double p[3];
        face_pos(fs, a, h.v, i, j, k, p);
        double cv[3], fv[3];
        collider_vel(col, p, cv);
        for (int b = 0; b < 3; ++b)  // FaceCenteredGrid3::sample
            fv[b] = sample_face_grid(
                vel[b], fs.s[b], gsp.s[0].div(p[0] - fs.o[b][0]),
                gsp.s[1].div(p[1] - fs.o[b][1]),
                gsp.s[2].div(p[2] - fs.o[b][2]));
        const double4_32a nq =
            t < cap ? nrm[t] : bc_normal(fs, a, h, ssp, inv, sdf, c);
        if (nq.w != 0.0) {
            const double nn[3] = {nq.x, nq.y, nq.z};
            const double vr[3] = {fv[0] - cv[0], fv[1] - cv[1], fv[2] - cv[2]};
            const double dn = vr[0] * nn[0] + vr[1] * nn[1] + vr[2] * nn[2];
            double vt[3] = {vr[0] - nn[0] * dn, vr[1] - nn[1] * dn,
                            vr[2] - nn[2] * dn};
            const double l2 = vt[0] * vt[0] + vt[1] * vt[1] + vt[2] * vt[2];
            if (l2 > 0.0) {
                const double veln = dmax(-dn, 0.0);
                const double sc = dmax(
                    1.0 - div_pos(col.friction * veln, sqrt(l2)), 0.0);
                vt[0] = vt[0] * sc;
                vt[1] = vt[1] * sc;
                vt[2] = vt[2] * sc;
            }
            tmp[t] = vt[a] + cv[a];
        } else {
            tmp[t] = cv[a];
        }
    }
}

// K19d: the projected faces from the temporary (:177-187) ...
__global__ void k_bc_store(Axes3 ax, long nf, const int* __restrict__ list_all,
                           const unsigned* __restrict__ cnt_all,
                           const double* __restrict__ tmp_all) {
    const int a = blockIdx.y;
    const int* lst = list_all + nf + ax.off[a];
    const long m = cnt_all[3 + a];
    const double* tmp = tmp_all + ax.off[a];
    double* vel = ax.vel[a];
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < m;
         t += (long)gridDim.x * blockDim.x)
        vel[lst[t]] = tmp[t];
}

// ... then zero on the closed domain walls (:189-232): the two planes of
// axis a = blockIdx.y, plane 0 when its low wall is closed, the last when
// its high wall is.
__global__ void k_bc_walls(FaceSet fs, Axes3 ax, int closed) {
    const int a = blockIdx.y;
    const Dims s = fs.s[a];
    const int lo = closed & (1 << (2 * a)), hi = closed & (1 << (2 * a + 1));
    if (!lo && !hi) return;
    double* vel = ax.vel[a];
    const int d1 = a == 0 ? s.y : s.x;            // the plane's two extents
    const int d2 = a == 2 ? s.y : s.z;
    const int ext = a == 0 ? s.x : (a == 1 ? s.y : s.z);
    const long P = (long)d1 * d2;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < 2 * P;
         t += (long)gridDim.x * blockDim.x) {
        const int side = (int)(t / P);
        if ((side == 0 && !lo) || (side == 1 && !hi)) continue;
        const long q = t - side * P;
        const int p1 = (int)(q % d1), p2 = (int)(q / d1);
        const int at = side == 0 ? 0 : ext - 1;
        int i, j, k;
        if (a == 0) { i = at; j = p1; k = p2; }
        else if (a == 1) { i = p1; j = at; k = p2; }
        else { i = p1; j = p2; k = at; }
        vel[lin(i, j, k, s.x, s.y)] = 0.0;
    }
}

// Scratch for the passes: two validity planes and one temporary of `n`
// elements (bytes + doubles), grown on demand.
jetgpu_status bc_scratch(Ctx* c, size_t n) {
    if (c->bc_cap >= n) return JETGPU_OK;
    JG_CUDA(c, cudaStreamSynchronize(c->stream));
    if (c->bc_tmp) cudaFree(c->bc_tmp);
    if (c->bc_valid) cudaFree(c->bc_valid);
    c->bc_tmp = nullptr;
    c->bc_valid = nullptr;
    c->bc_cap = 0;
    JG_CUDA(c, cudaMalloc((void**)&c->bc_tmp, n * sizeof(double)));
    JG_CUDA(c, cudaMalloc((void**)&c->bc_valid, 2 * n));
    c->bc_cap = n;
    return JETGPU_OK;
}

}  // namespace

// Entries of the inside-face normal cache for an axis of n faces.
static long bc_normal_cap(long n) { return (n + 7) / 8; }

// Offsets of the three axes in the concatenated face buffers and in the
// normal cache; the total face count.
static size_t bc_axes(const FaceSet& fs, double* u, double* v, double* w,
                      Axes3* ax) {
    size_t o = 0, no = 0;
    for (int a = 0; a < 3; ++a) {
        const long n = fs.s[a].count();
        ax->off[a] = (long)o;
        ax->noff[a] = (long)no;
        ax->ncap[a] = bc_normal_cap(n);
        o += (size_t)n;
        no += (size_t)bc_normal_cap(n);
    }
    ax->vel[0] = u;
    ax->vel[1] = v;
    ax->vel[2] = w;
    return o;
}

// Grid of a launch over up to `n` entries per axis, one y row per axis.
static dim3 bc_grid(const Ctx* c, long n) {
    return dim3((unsigned)blocks_for(n, kThreads, c->num_sms * 4), 3);
}

jetgpu_status bc_classify(Ctx* c, const GridDesc& g, const FieldDesc& sdf) {
    const FaceSet fs = face_set(g);
    Axes3 ax;
    const size_t nf = bc_axes(fs, nullptr, nullptr, nullptr, &ax);
    if (c->bc_cls_cap < nf) {
        JG_CUDA(c, cudaStreamSynchronize(c->stream));
        if (c->bc_cls) cudaFree(c->bc_cls);
        if (c->bc_list) cudaFree(c->bc_list);
        c->bc_cls = nullptr;
        c->bc_list = nullptr;
        c->bc_cls_cap = 0;
        JG_CUDA(c, cudaMalloc((void**)&c->bc_cls, nf));
        JG_CUDA(c, cudaMalloc((void**)&c->bc_list, 2 * nf * sizeof(int)));
        c->bc_cls_cap = nf;
    }
    if (!c->bc_cnt) JG_CUDA(c, cudaMalloc((void**)&c->bc_cnt, 6 * sizeof(unsigned)));
    JG_CUDA(c, cudaMemsetAsync(c->bc_cnt, 0, 6 * sizeof(unsigned), c->stream));
    // Normal cache: up to an eighth of each axis's faces (a collider larger
    // than that computes the rest in every pass).
    const size_t ncap = (size_t)(ax.noff[2] + ax.ncap[2]);
    if (c->bc_nrm_cap < ncap) {
        JG_CUDA(c, cudaStreamSynchronize(c->stream));
        if (c->bc_nrm) cudaFree(c->bc_nrm);
        c->bc_nrm = nullptr;
        c->bc_nrm_cap = 0;
        JG_CUDA(c, cudaMalloc((void**)&c->bc_nrm, ncap * sizeof(double4_32a)));
        c->bc_nrm_cap = ncap;
    }
    H3 h{{g.spacing[0], g.spacing[1], g.spacing[2]}};
    S3 fsp{{make_spacing(sdf.kind == 1 ? sdf.spacing[0] : 1.0),
            make_spacing(sdf.kind == 1 ? sdf.spacing[1] : 1.0),
            make_spacing(sdf.kind == 1 ? sdf.spacing[2] : 1.0)}};
    H3 inv{{0, 0, 0}};
    if (sdf.kind == 1)
        for (int d = 0; d < 3; ++d) inv.v[d] = 1.0 / sdf.spacing[d];
    long nmax = 0;
    for (int a = 0; a < 3; ++a) nmax = std::max(nmax, fs.s[a].count());
    Prof pr(c, K_BOUNDARY, 1.0 * (double)nf);
    // The aligned case of k_bc_classify: the SDF on the grid's cell centres
    // (same resolution and spacing, origin + h/2), grid origin +0 and
    // power-of-two spacings; the values are checked on the device.
    bool aligned = sdf.kind == 1;
    for (int d = 0; d < 3 && aligned; ++d)
        aligned = sdf.res[d] == g.res[d] && sdf.spacing[d] == g.spacing[d] &&
                  dbits(g.origin[d]) == 0ull && fsp.s[d].pow2 &&
                  sdf.origin[d] == 0.5 * g.spacing[d];
    int* irregular = nullptr;
    if (aligned) {
        if (!c->bc_flag) JG_CUDA(c, cudaMalloc((void**)&c->bc_flag, sizeof(int)));
        irregular = c->bc_flag;
        JG_CUDA(c, cudaMemsetAsync(irregular, 0, sizeof(int), c->stream));
        const long ncell = (long)g.res[0] * g.res[1] * g.res[2];
        k_sdf_regular<<<blocks_for(ncell, kThreads, c->num_sms * 8), kThreads,
                        0, c->stream>>>(sdf.data, ncell, irregular);
    }
    // Lists: invalid faces of axis a at bc_list + off[a], inside faces at
    // bc_list + nf + off[a]; counts bc_cnt[a], bc_cnt[3 + a].
    k_bc_classify<<<bc_grid(c, nmax), kThreads, 0, c->stream>>>(
        fs, h, sdf, fsp, ax, (long)nf, c->bc_cls, c->bc_list, c->bc_cnt,
        irregular);
    k_bc_normals<<<bc_grid(c, nmax / 8), kThreads, 0, c->stream>>>(
        fs, h, fsp, inv, sdf, ax, (long)nf, c->bc_list, c->bc_cnt, c->bc_nrm);
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

jetgpu_status bc_apply(Ctx* c, const GridDesc& g, double* u, double* v,
                       double* w, const FieldDesc& sdf,
                       const jetgpu_collider* col, int closed, unsigned depth) {
    const FaceSet fs = face_set(g);
    Axes3 ax;
    const size_t nf = bc_axes(fs, u, v, w, &ax);
    if (jetgpu_status s = bc_scratch(c, nf)) return s;
    ColliderDesc cd{};
    if (col) {
        cd.present = 1;
        for (int d = 0; d < 3; ++d) {
            cd.lin[d] = col->linear_velocity[d];
            cd.ang[d] = col->angular_velocity[d];
            cd.centre[d] = col->centre[d];
        }
        cd.friction = col->friction;
    }
    H3 h{{g.spacing[0], g.spacing[1], g.spacing[2]}};
    S3 gsp{{make_spacing(g.spacing[0]), make_spacing(g.spacing[1]),
            make_spacing(g.spacing[2])}};
    H3 inv{{0, 0, 0}};
    if (sdf.kind == 1)
        for (int d = 0; d < 3; ++d) inv.v[d] = 1.0 / sdf.spacing[d];
    S3 ssp{{make_spacing(sdf.kind == 1 ? sdf.spacing[0] : 1.0),
            make_spacing(sdf.kind == 1 ? sdf.spacing[1] : 1.0),
            make_spacing(sdf.kind == 1 ? sdf.spacing[2] : 1.0)}};
    // The list passes are sized for the worst case and read their counts on
    // the device, so nothing here waits for the classification. One launch
    // per step covers the three axes (blockIdx.y).
    long nmax = 0;
    for (int a = 0; a < 3; ++a) nmax = std::max(nmax, fs.s[a].count());
    const dim3 grid = bc_grid(c, nmax);
    Prof pr(c, K_BOUNDARY, 0.0);
    unsigned char* st0 = c->bc_valid;
    unsigned char* st1 = c->bc_valid + nf;
    k_bc_mark<<<grid, kThreads, 0, c->stream>>>(fs, h, cd, ax, c->bc_list,
                                                c->bc_cnt, st0);
    for (unsigned it = 0; it < depth; ++it) {
        k_extrapolate_list<<<grid, kThreads, 0, c->stream>>>(
            fs, ax, c->bc_list, c->bc_cnt, c->bc_cls, st0, st1);
        std::swap(st0, st1);
    }
    k_bc_project<<<grid, kThreads, 0, c->stream>>>(
        fs, h, gsp, ssp, inv, sdf, cd, ax, (long)nf, c->bc_list, c->bc_cnt,
        c->bc_nrm, c->bc_tmp);
    k_bc_store<<<grid, kThreads, 0, c->stream>>>(ax, (long)nf, c->bc_list,
                                                 c->bc_cnt, c->bc_tmp);
    if (closed) {
        long P = 0;  // the largest wall plane
        for (int a = 0; a < 3; ++a) {
            const Dims s = fs.s[a];
            P = std::max(P, a == 0 ? (long)s.y * s.z
                                   : (a == 1 ? (long)s.x * s.z : (long)s.x * s.y));
        }
        k_bc_walls<<<bc_grid(c, 2 * P), kThreads, 0, c->stream>>>(fs, ax,
                                                                  closed);
    }
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

namespace {

// GridBlockedBoundaryConditionSolver3's no-flux pass
// (src/jet/grid_blocked_boundary_condition_solver3.cpp:29-66): a cell is a
// collider cell when the collider SDF sample at the cell is negative
// (onColliderUpdated, :79-90); each face between a collider cell and a
// non-collider neighbour takes the collider velocity's normal component at
// the face position. The collider side of such a face is unique, so the
// cell's thread is the face's only writer.
__global__ void k_bc_blocked(FaceSet fs, H3 h, Dims n, FieldDesc sdf,
                             ColliderDesc col, double* __restrict__ u,
                             double* __restrict__ v, double* __restrict__ w) {
    const long N = n.count();
    const long sy = n.x, sz = (long)n.x * n.y;
    auto solid = [&](long c) {
        return (sdf.kind == 1 ? sdf.data[c] : sdf.value) < 0.0;
    };
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x) {
        if (!solid(c)) continue;
        int i, j, k;
        cell_ijk(c, n, i, j, k);
        double p[3], cv[3];
        auto set = [&](int a, int fi, int fj, int fk, double* vel) {
            face_pos(fs, a, h.v, fi, fj, fk, p);
            collider_vel(col, p, cv);
            vel[lin(fi, fj, fk, fs.s[a].x, fs.s[a].y)] = cv[a];
        };
        if (i > 0 && !solid(c - 1)) set(0, i, j, k, u);
        if (i < n.x - 1 && !solid(c + 1)) set(0, i + 1, j, k, u);
        if (j > 0 && !solid(c - sy)) set(1, i, j, k, v);
        if (j < n.y - 1 && !solid(c + sy)) set(1, i, j + 1, k, v);
        if (k > 0 && !solid(c - sz)) set(2, i, j, k, w);
        if (k < n.z - 1 && !solid(c + sz)) set(2, i, j, k + 1, w);
    }
}

}  // namespace

jetgpu_status constrain_velocity_blocked(Ctx* c, const GridDesc& g, double* u,
                                         double* v, double* w,
                                         const FieldDesc& sdf,
                                         const jetgpu_collider* col,
                                         int closed, unsigned depth) {
    if (sdf.kind == 1 && (sdf.res[0] != g.res[0] || sdf.res[1] != g.res[1] ||
                          sdf.res[2] != g.res[2]))
        return fail(c, JETGPU_BAD_INPUT,
                    "the blocked constraint needs the collider SDF on the "
                    "velocity grid's cells");
    if (jetgpu_status s = constrain_velocity(c, g, u, v, w, sdf, col, closed,
                                             depth))
        return s;
    ColliderDesc cd{};
    if (col) {
        cd.present = 1;
        for (int d = 0; d < 3; ++d) {
            cd.lin[d] = col->linear_velocity[d];
            cd.ang[d] = col->angular_velocity[d];
            cd.centre[d] = col->centre[d];
        }
        cd.friction = col->friction;
    }
    const Dims n{g.res[0], g.res[1], g.res[2]};
    Prof pr(c, K_BOUNDARY, 8.0 * (double)n.count());
    k_bc_blocked<<<blocks_for(n.count()), kThreads, 0, c->stream>>>(
        face_set(g), H3{{g.spacing[0], g.spacing[1], g.spacing[2]}}, n, sdf,
        cd, u, v, w);
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

jetgpu_status constrain_velocity(Ctx* c, const GridDesc& g, double* u,
                                 double* v, double* w, const FieldDesc& sdf,
                                 const jetgpu_collider* col, int closed,
                                 unsigned depth) {
    if (jetgpu_status s = bc_classify(c, g, sdf)) return s;
    return bc_apply(c, g, u, v, w, sdf, col, closed, depth);
}

jetgpu_status extrapolate_regions(Ctx* c, int na, const Dims* s,
                                  double* const* data,
                                  const unsigned char* const* valid,
                                  unsigned iters) {
    if (iters == 0 || na <= 0) return JETGPU_OK;
    Xp3 X{};
    long tot = 0, nmax = 0;
    for (int r = 0; r < na; ++r) {
        X.s[r] = s[r];
        X.data[r] = data[r];
        X.valid[r] = valid[r];
        X.off[r] = tot;
        tot += s[r].count();
        nmax = std::max(nmax, s[r].count());
    }
    // Stamps and two front lists (tot ints each), two front lengths per
    // array. The callers' validity stays untouched.
    if (c->xp_cap < (size_t)tot) {
        JG_CUDA(c, cudaStreamSynchronize(c->stream));
        if (c->xp_int) cudaFree(c->xp_int);
        c->xp_int = nullptr;
        c->xp_cap = 0;
        JG_CUDA(c, cudaMalloc((void**)&c->xp_int, 3 * (size_t)tot * sizeof(int)));
        c->xp_cap = (size_t)tot;
    }
    if (!c->xp_cnt) JG_CUDA(c, cudaMalloc((void**)&c->xp_cnt, 6 * sizeof(unsigned)));
    int* stamp = c->xp_int;
    int* lst[2] = {stamp + tot, stamp + 2 * tot};
    unsigned* cnt[2] = {c->xp_cnt, c->xp_cnt + 3};
    const dim3 full((unsigned)blocks_for(nmax, kThreads, c->num_sms * 8),
                    (unsigned)na);
    const dim3 grid((unsigned)(c->num_sms * 4), (unsigned)na);
    Prof pr(c, K_BOUNDARY, 5.0 * (double)tot);
    JG_CUDA(c, cudaMemsetAsync(c->xp_cnt, 0, 6 * sizeof(unsigned), c->stream));
    k_xp_init<<<full, kThreads, 0, c->stream>>>(X, stamp, lst[0], cnt[0]);
    for (unsigned t = 0; t < iters; ++t) {
        const int cur = t & 1, nxt = cur ^ 1;
        k_xp_pass<<<grid, kThreads, 0, c->stream>>>(X, stamp, lst[cur],
                                                    cnt[cur], (int)t);
        if (t + 1 < iters) {
            JG_CUDA(c, cudaMemsetAsync(cnt[nxt], 0, 3 * sizeof(unsigned),
                                       c->stream));
            k_xp_next<<<grid, kThreads, 0, c->stream>>>(
                X, stamp, lst[cur], cnt[cur], lst[nxt], cnt[nxt]);
        }
    }
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

jetgpu_status extrapolate_region(Ctx* c, Dims s, double* data,
                                 const unsigned char* valid, unsigned iters) {
    return extrapolate_regions(c, 1, &s, &data, &valid, iters);
}

}  // namespace jg

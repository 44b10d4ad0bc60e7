// FLIP/PIC particle<->grid transfers (K13, K14).
//
// P2G replaces PicSolver3::transferFromParticlesToGrids
// (src/jet/pic_solver3.cpp:118-193), a serial scatter in the reference, and
// FlipSolver3's float snapshot (src/jet/flip_solver3.cpp:27-48). G2P replaces
// FlipSolver3::transferFromGridsToParticles (flip_solver3.cpp:50-99) and
// PicSolver3::transferFromGridsToParticles (pic_solver3.cpp:195-204).
//
// Stencil coordinates and trilinear weights replay
// LinearArraySampler3::getCoordinatesAndWeights
// (include/jet/detail/array_samplers3-inl.h:151-193) in double precision
// without multiply-add contraction (this unit is built with -fmad=false), so
// every particle's eight indices and weights are the reference's. The
// ordered P2G (the default) adds each face's contributions in the
// reference's particle order, so its grids are the reference's bit for bit;
// the atomic scatter accumulates with FP64 atomics, so its sums match the
// reference's serial order to rounding, not bit for bit.

#include "ctx.h"
#include "sampling.cuh"

#include <climits>
#include <mutex>

namespace jg {
namespace {

using namespace smp;

// K13a: scatter vel*w and w with FP64 atomics; markers set to 1.
struct P2gLattice {
    Dims s;                 // the component's face lattice
    double ox, oy, oz;      // its origin
    smp::Spacing sx, sy, sz;  // the grid spacing per axis
};
struct P2gLattice3 {
    P2gLattice l[3];        // u, v, w
};

P2gLattice p2g_lattice(const FaceSet& fs, int a, const double spacing[3]) {
    return P2gLattice{fs.s[a], fs.o[a][0], fs.o[a][1], fs.o[a][2],
                      smp::make_spacing(spacing[0]),
                      smp::make_spacing(spacing[1]),
                      smp::make_spacing(spacing[2])};
}
P2gLattice3 p2g_lattices(const FaceSet& fs, const double spacing[3]) {
    return P2gLattice3{{p2g_lattice(fs, 0, spacing), p2g_lattice(fs, 1, spacing),
                        p2g_lattice(fs, 2, spacing)}};
}

// x * (1 / h), the reference's normalised coordinate: an exponent add when
// 1 / h is a power of two.
__device__ __forceinline__ double p2g_scale(double x, const smp::Spacing& sp) {
    return sp.pow2 ? smp::scale_exact(x, sp.k, sp.inv) : x * sp.inv;
}

// Base corner, fractions f and complements g = 1 - f of particle p on the
// lattice (LinearArraySampler3::getCoordinatesAndWeights, bit for bit).
__device__ __forceinline__ void p2g_base(const double* __restrict__ pos,
                                         long p, const P2gLattice& L, int& i,
                                         int& j, int& k, double3& f,
                                         double3& g) {
    const double nx = p2g_scale(pos[3 * p] - L.ox, L.sx);
    const double ny = p2g_scale(pos[3 * p + 1] - L.oy, L.sy);
    const double nz = p2g_scale(pos[3 * p + 2] - L.oz, L.sz);
    smp::bary_bits2(nx, L.s.x - 1, &i, &f.x, &g.x);
    smp::bary_bits2(ny, L.s.y - 1, &j, &f.y, &g.y);
    smp::bary_bits2(nz, L.s.z - 1, &k, &f.z, &g.z);
}

__global__ void k_p2g_scatter(long np, const double* __restrict__ pos,
                              const double* __restrict__ vel, P2gLattice3 L,
                              double* u, double* v, double* w, double* wu,
                              double* wv, double* ww, unsigned char* mu,
                              unsigned char* mv, unsigned char* mw) {
    double* grid[3] = {u, v, w};
    double* wsum[3] = {wu, wv, ww};
    unsigned char* mark[3] = {mu, mv, mw};
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < np;
         p += (long)gridDim.x * blockDim.x) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const Dims s = L.l[a].s;
            int i, j, k;
            double3 f, g;
            p2g_base(pos, p, L.l[a], i, j, k, f, g);
            const int ip1 = min(i + 1, s.x - 1), jp1 = min(j + 1, s.y - 1),
                      kp1 = min(k + 1, s.z - 1);
            const long idx[8] = {lin(i, j, k, s.x, s.y),     lin(ip1, j, k, s.x, s.y),
                                 lin(i, jp1, k, s.x, s.y),   lin(ip1, jp1, k, s.x, s.y),
                                 lin(i, j, kp1, s.x, s.y),   lin(ip1, j, kp1, s.x, s.y),
                                 lin(i, jp1, kp1, s.x, s.y), lin(ip1, jp1, kp1, s.x, s.y)};
            // The reference's weights, (1 - fx) * (1 - fy) * (1 - fz) and so
            // on, with the (x, y) products formed once.
            const double xy[4] = {g.x * g.y, f.x * g.y, g.x * f.y, f.x * f.y};
            const double va = vel[3 * p + a];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const double wt = xy[q & 3] * ((q & 4) ? f.z : g.z);
                atomicAdd(&grid[a][idx[q]], va * wt);
                atomicAdd(&wsum[a][idx[q]], wt);
                if (mark[a]) mark[a][idx[q]] = 1;
            }
        }
    }
}

// K13b: divide by the weight sum where positive; float snapshot.
__global__ void k_p2g_normalize(double* __restrict__ g,
                                const double* __restrict__ wsum,
                                float* __restrict__ snap, long n) {
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n;
         c += (long)gridDim.x * blockDim.x) {
        double v = g[c];
        const double ws = wsum[c];
        if (ws > 0.0) v = div_pos(v, ws);
        g[c] = v;
        if (snap) snap[c] = (float)v;
    }
}

// Ordered P2G (ordered_p2g): the reference adds the particles' contributions
// to each face in particle order (a serial loop, pic_solver3.cpp:118-193);
// summing each face's contributions in the same order gives the same bits.
// Per component: every particle is binned by the base corner (i, j, k) of
// its trilinear stencil on that component's face lattice; each bin lists its
// particles in increasing index, beside a record of each one's weight
// factors and velocity component; each face then merges the (at most eight)
// bins whose stencils reach it, in particle order, adding each particle's
// corners that land on it in corner order — the reference's products, in
// the reference's order. GB300 issues FP64 at a small fraction of its
// integer rate, so the FP64 work is cut to what the sums need: the lattice
// coordinate is scaled exactly on the integer pipe when the spacing is a
// power of two, the fractions and their complements (1 - f) come from the
// coordinate's bits, the four (x, y) weight products are formed once per
// particle, and a face's step is the z product, the velocity product and
// the two additions.

// Step 1: the bin (base corner) of every particle; bins counted.
__global__ void k_p2g_bin(long np, const double* __restrict__ pos,
                          P2gLattice L, int* __restrict__ key,
                          int* __restrict__ count) {
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < np;
         p += (long)gridDim.x * blockDim.x) {
        int i, j, k;
        double3 f, g;
        p2g_base(pos, p, L, i, j, k, f, g);
        const int b = (int)lin(i, j, k, L.s.x, L.s.y);
        key[p] = b;
        atomicAdd(&count[b], 1);
    }
}

// Step 2: particle indices into their bins (any order within a bin).
__global__ void k_p2g_fill(long np, const int* __restrict__ key,
                          const int* __restrict__ off, int* __restrict__ cursor,
                          int* __restrict__ list) {
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < np;
         p += (long)gridDim.x * blockDim.x) {
        const int b = key[p];
        list[off[b] + atomicAdd(&cursor[b], 1)] = (int)p;
    }
}

// Step 3: every particle at its place in its bin's sorted list (its rank =
// the number of the bin's particles with a smaller index), with its record:
// the weight products (1-fx)(1-fy), fx(1-fy), (1-fx)fy, fx fy, then
// (1 - fz, fz, velocity component, and as a 64-bit integer the next
// particle of the bin shifted left by 3, all ones after the last).
__global__ void k_p2g_place(long np, const double* __restrict__ pos,
                           const double* __restrict__ vel, P2gLattice L,
                           int a, const int* __restrict__ key,
                           const int* __restrict__ off,
                           const int* __restrict__ list,
                           int* __restrict__ slist,
                           double4_32a* __restrict__ rec) {
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < np;
         p += (long)gridDim.x * blockDim.x) {
        const int b = key[p];
        const int lo = off[b], hi = off[b + 1];
        int rank = 0;
        unsigned succ = 0xffffffffu;
        for (int q = lo; q < hi; ++q) {
            const int v = list[q];
            rank += v < (int)p ? 1 : 0;
            if (v > (int)p) succ = min(succ, (unsigned)v);
        }
        int i, j, k;
        double3 f, g;
        p2g_base(pos, p, L, i, j, k, f, g);
        const long s = lo + rank;
        slist[s] = (int)p;
        const unsigned long long nk = succ == 0xffffffffu
                                          ? ~0ull
                                          : (unsigned long long)succ << 3;
        rec[2 * s] = make_double4_32a(g.x * g.y, f.x * g.y, g.x * f.y, f.x * f.y);
        rec[2 * s + 1] = make_double4_32a(g.z, f.z, vel[3 * p + a],
                                      __longlong_as_double((long long)nk));
    }
}

// One corner's contribution (corner q of the reference's order): weight
// xy[q & 3] * z[q >> 2], product velocity * weight, both added.
__device__ __forceinline__ void p2g_corner(int q, const double4_32a& xy,
                                           const double4_32a& zv, double& acc,
                                           double& ws) {
    const double XY = (q & 3) == 0 ? xy.x
                    : (q & 3) == 1 ? xy.y
                    : (q & 3) == 2 ? xy.z : xy.w;
    const double wt = XY * ((q & 4) ? zv.y : zv.x);
    acc += zv.z * wt;
    ws += wt;
}

// Step 4: every face of the component, its contributions in particle order.
// List l of a face holds the bin at the face minus corner offset l (bit 0:
// x, bit 1: y, bit 2: z), whose particles reach the face through corner l;
// on a lattice axis of one line (degenerate mask dm) the upper corner is
// clamped onto the lower one, so such a bin also reaches the face through
// the corners that differ from l only in those bits, in corner order. Each
// list's head is the key (particle index << 3 | l) in a register, so the
// next contribution is the minimum of eight keys; the taken list advances
// through selects, its next key read from the record just loaded, so a
// warp's lanes never split over the lists. A block takes chunks of kGatherChunk consecutive faces from a
// global counter, writes the chunk's empty faces at once, sorts the others
// by contribution count in shared memory (a counting sort) and gives each
// warp 32 faces of (nearly) equal count at a time, so the lanes run the same
// number of steps. K is a 32-bit key when particle indices fit in 28 bits,
// else 64-bit.
constexpr int kGatherThreads = 256;
constexpr int kGatherBuckets = 128;  // counts >= 127 share the last bucket

template <typename K>
__device__ __forceinline__ K p2g_min8(const K (&h)[8]) {
    const K a = min(h[0], h[1]), b = min(h[2], h[3]);
    const K c = min(h[4], h[5]), d = min(h[6], h[7]);
    return min(min(a, b), min(c, d));
}

// The bin of list l of face (fi, fj, fk), or -1 outside the lattice.
__device__ __forceinline__ long p2g_list_bin(const Dims& s, int fi, int fj,
                                             int fk, int l) {
    const int x = fi - (l & 1), y = fj - ((l >> 1) & 1), z = fk - (l >> 2);
    return x >= 0 && y >= 0 && z >= 0 ? lin(x, y, z, s.x, s.y) : -1;
}

template <typename K, int kGatherChunk>
__global__ void __launch_bounds__(kGatherThreads)
k_p2g_gather(Dims s, int dm, const int* __restrict__ count,
             const int* __restrict__ off, const int* __restrict__ slist,
             const double4_32a* __restrict__ rec, double* __restrict__ grid,
             double* __restrict__ wsum, unsigned char* __restrict__ mark,
             unsigned long long* __restrict__ counter) {
    constexpr int kPer = kGatherChunk / kGatherThreads;
    constexpr int kWarps = kGatherThreads / 32;
    __shared__ unsigned short s_face[kGatherChunk];
    __shared__ int s_hist[kGatherBuckets];
    __shared__ long long s_c0;
    __shared__ int s_total;
    const K kNone = ~(K)0;
    const long nf = s.count();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    while (true) {
        if (tid == 0) s_c0 = (long long)atomicAdd(counter, kGatherChunk);
        for (int t = tid; t < kGatherBuckets; t += kGatherThreads)
            s_hist[t] = 0;
        __syncthreads();
        const long c0 = (long)s_c0;
        if (c0 >= nf) break;
        // Contribution counts; empty faces written now.
        int bucket[kPer];
#pragma unroll
        for (int r = 0; r < kPer; ++r) {
            const long f = c0 + tid + r * kGatherThreads;
            bucket[r] = 0;
            if (f < nf) {
                int fi, fj, fk;
                cell_ijk(f, s, fi, fj, fk);
                int n = 0;
#pragma unroll
                for (int l = 0; l < 8; ++l) {
                    const long b = p2g_list_bin(s, fi, fj, fk, l);
                    n += b >= 0 ? count[b] : 0;
                }
                if (n == 0) {
                    grid[f] = 0.0;
                    wsum[f] = 0.0;
                    if (mark) mark[f] = 0;
                } else {
                    bucket[r] = min(n, kGatherBuckets - 1);
                    atomicAdd(&s_hist[bucket[r]], 1);
                }
            }
        }
        __syncthreads();
        // Exclusive scan of the histogram (one warp), then the faces in
        // order of count.
        if (warp == 0) {
            constexpr int kPerLane = kGatherBuckets / 32;
            int v[kPerLane], sum = 0;
#pragma unroll
            for (int t = 0; t < kPerLane; ++t) {
                v[t] = s_hist[lane * kPerLane + t];
                sum += v[t];
            }
            int incl = sum;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int o = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= d) incl += o;
            }
            int run = incl - sum;
#pragma unroll
            for (int t = 0; t < kPerLane; ++t) {
                s_hist[lane * kPerLane + t] = run;
                run += v[t];
            }
            if (lane == 31) s_total = incl;
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < kPer; ++r)
            if (bucket[r] > 0)
                s_face[atomicAdd(&s_hist[bucket[r]], 1)] =
                    (unsigned short)(tid + r * kGatherThreads);
        __syncthreads();
        const int total = s_total;
        for (int g0 = warp * 32; g0 < total; g0 += kWarps * 32) {
            const int i = g0 + lane;
            const long f = i < total ? c0 + s_face[i] : -1;
            int cur[8];
            K head[8];
            int fi = 0, fj = 0, fk = 0;
            if (f >= 0) cell_ijk(f, s, fi, fj, fk);
#pragma unroll
            for (int l = 0; l < 8; ++l) {
                const long b = f >= 0 ? p2g_list_bin(s, fi, fj, fk, l) : -1;
                cur[l] = b >= 0 ? off[b] : 0;
                const int e = b >= 0 ? off[b + 1] : 0;
                head[l] = cur[l] < e ? ((K)slist[cur[l]] << 3) | (K)l : kNone;
            }
            K key = p2g_min8(head);
            bool busy = key != kNone;
            double acc = 0.0, ws = 0.0;
            while (__ballot_sync(0xffffffffu, busy)) {
                if (busy) {
                    const int best = (int)(key & 7);
                    // cur[best] through a three-level select tree.
                    const bool b0 = best & 1, b1 = best & 2, b2 = best & 4;
                    const int s01 = b0 ? cur[1] : cur[0];
                    const int s23 = b0 ? cur[3] : cur[2];
                    const int s45 = b0 ? cur[5] : cur[4];
                    const int s67 = b0 ? cur[7] : cur[6];
                    const int s03 = b1 ? s23 : s01, s47 = b1 ? s67 : s45;
                    const int slot = b2 ? s47 : s03;
                    const double4_32a xy = rec[2 * (long)slot];
                    const double4_32a zv = rec[2 * (long)slot + 1];
                    const K nh = (K)(unsigned long long)__double_as_longlong(
                                     zv.w) |
                                 (K)best;
#pragma unroll
                    for (int l = 0; l < 8; ++l) {
                        cur[l] = best == l ? slot + 1 : cur[l];
                        head[l] = best == l ? nh : head[l];
                    }
                    if (dm == 0) {
                        p2g_corner(best, xy, zv, acc, ws);
                    } else {
                        for (int q = 0; q < 8; ++q)
                            if (((q ^ best) & ~dm & 7) == 0)
                                p2g_corner(q, xy, zv, acc, ws);
                    }
                    key = p2g_min8(head);
                    busy = key != kNone;
                }
            }
            if (f >= 0) {
                grid[f] = acc;
                wsum[f] = ws;
                if (mark) mark[f] = 1;
            }
        }
        __syncthreads();
    }
}

// K14a: snap = float(new) - snap (flip_solver3.cpp:57-70).
__global__ void k_flip_delta(const double* __restrict__ g,
                             float* __restrict__ snap, long n) {
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n;
         c += (long)gridDim.x * blockDim.x)
        snap[c] = (float)g[c] - snap[c];
}

// K14b: v_p += float trilinear(delta) at the float position; optional PIC
// blend toward the double sample of the new grid.
__global__ void k_g2p_flip(long np, const double* __restrict__ pos,
                           double* __restrict__ vel, FaceSet fs, float hfx,
                           float hfy, float hfz, const float* __restrict__ du,
                           const float* __restrict__ dv,
                           const float* __restrict__ dw,
                           const double* __restrict__ u,
                           const double* __restrict__ v,
                           const double* __restrict__ w, Spacing hx,
                           Spacing hy, Spacing hz, double blend) {
    const float* dl[3] = {du, dv, dw};
    const double* g[3] = {u, v, w};
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < np;
         p += (long)gridDim.x * blockDim.x) {
        const double px = pos[3 * p], py = pos[3 * p + 1], pz = pos[3 * p + 2];
        const float xf = (float)px, yf = (float)py, zf = (float)pz;
        double out[3];
        for (int a = 0; a < 3; ++a) {
            const float nx = (xf - (float)fs.o[a][0]) / hfx;
            const float ny = (yf - (float)fs.o[a][1]) / hfy;
            const float nz = (zf - (float)fs.o[a][2]) / hfz;
            const double d = (double)sample_face<float, float>(dl[a], fs.s[a],
                                                               nx, ny, nz);
            out[a] = vel[3 * p + a] + d;
        }
        if (blend > 0.0) {
            double pic[3];
            for (int a = 0; a < 3; ++a)
                pic[a] = sample_face_d(
                    g[a], fs.s[a], hx.div(px - fs.o[a][0]),
                    hy.div(py - fs.o[a][1]), hz.div(pz - fs.o[a][2]));
            for (int a = 0; a < 3; ++a)
                out[a] = (1 - blend) * out[a] + blend * pic[a];
        }
        vel[3 * p] = out[0];
        vel[3 * p + 1] = out[1];
        vel[3 * p + 2] = out[2];
    }
}

// K14c: v_p = sample(new grid) (PIC).
__global__ void k_g2p_pic(long np, const double* __restrict__ pos,
                          double* __restrict__ vel, FaceSet fs,
                          const double* __restrict__ u,
                          const double* __restrict__ v,
                          const double* __restrict__ w, Spacing hx,
                          Spacing hy, Spacing hz) {
    const double* g[3] = {u, v, w};
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < np;
         p += (long)gridDim.x * blockDim.x) {
        const double px = pos[3 * p], py = pos[3 * p + 1], pz = pos[3 * p + 2];
        for (int a = 0; a < 3; ++a)
            vel[3 * p + a] = sample_face_d(
                g[a], fs.s[a], hx.div(px - fs.o[a][0]),
                hy.div(py - fs.o[a][1]), hz.div(pz - fs.o[a][2]));
    }
}

// APIC (ApicSolver3, src/jet/apic_solver3.cpp). Positions are clamped per
// face grid: the two other coordinates half a cell inside the grid's box
// (:55-62), with jet::clamp's rule.
struct ApicBox {
    double lo[3], hi[3];  // box +- half a cell
};
__device__ __forceinline__ double clamp_d(double v, double lo, double hi) {
    return v < lo ? lo : (v > hi ? hi : v);
}

// K22a: the APIC scatter (:51-124): weights as P2G's, each sample carrying
// vel_a + c_a . (x_face - x_clamped). FP64 atomics reorder the reference's
// serial sums (rounding only).
__global__ void k_apic_p2g_scatter(long np, const double* __restrict__ pos,
                                   const double* __restrict__ vel,
                                   const double* __restrict__ aff, FaceSet fs,
                                   double hx, double hy, double hz, double ihx,
                                   double ihy, double ihz, ApicBox box,
                                   double* u, double* v, double* w,
                                   double* wu, double* wv, double* ww,
                                   unsigned char* mu, unsigned char* mv,
                                   unsigned char* mw) {
    double* grid[3] = {u, v, w};
    double* wsum[3] = {wu, wv, ww};
    unsigned char* mark[3] = {mu, mv, mw};
    const double hs[3] = {hx, hy, hz};
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < np;
         p += (long)gridDim.x * blockDim.x) {
        for (int a = 0; a < 3; ++a) {
            double q[3];
            for (int d = 0; d < 3; ++d)
                q[d] = d == a ? pos[3 * p + d]
                              : clamp_d(pos[3 * p + d], box.lo[d], box.hi[d]);
            const Dims s = fs.s[a];
            int i, j, k;
            double fx, fy, fz;
            bary<double>((q[0] - fs.o[a][0]) * ihx, s.x - 1, &i, &fx);
            bary<double>((q[1] - fs.o[a][1]) * ihy, s.y - 1, &j, &fy);
            bary<double>((q[2] - fs.o[a][2]) * ihz, s.z - 1, &k, &fz);
            const int ip1 = min(i + 1, s.x - 1), jp1 = min(j + 1, s.y - 1),
                      kp1 = min(k + 1, s.z - 1);
            const int ci[8] = {i, ip1, i, ip1, i, ip1, i, ip1};
            const int cj[8] = {j, j, jp1, jp1, j, j, jp1, jp1};
            const int ck[8] = {k, k, k, k, kp1, kp1, kp1, kp1};
            const double wt[8] = {(1 - fx) * (1 - fy) * (1 - fz), fx * (1 - fy) * (1 - fz),
                                  (1 - fx) * fy * (1 - fz),       fx * fy * (1 - fz),
                                  (1 - fx) * (1 - fy) * fz,       fx * (1 - fy) * fz,
                                  (1 - fx) * fy * fz,             fx * fy * fz};
            const double* C = aff + 9 * p + 3 * a;
            const double va = vel[3 * p + a];
            for (int n = 0; n < 8; ++n) {
                const double g0 = fs.o[a][0] + hs[0] * (double)ci[n];
                const double g1 = fs.o[a][1] + hs[1] * (double)cj[n];
                const double g2 = fs.o[a][2] + hs[2] * (double)ck[n];
                const double term = C[0] * (g0 - q[0]) + C[1] * (g1 - q[1]) +
                                    C[2] * (g2 - q[2]);
                const long idx = lin(ci[n], cj[n], ck[n], s.x, s.y);
                atomicAdd(&grid[a][idx], wt[n] * (va + term));
                atomicAdd(&wsum[a][idx], wt[n]);
                if (mark[a]) mark[a][idx] = 1;
            }
        }
    }
}

// K22b: the APIC gather (:148-228): the PIC velocity, then c_a = sum of the
// gradient weights of getCoordinatesAndGradientWeights
// (include/jet/detail/array_samplers3-inl.h:196-261) times the grid values.
__global__ void k_apic_g2p(long np, const double* __restrict__ pos,
                           double* __restrict__ vel, double* __restrict__ aff,
                           FaceSet fs, Spacing sx, Spacing sy, Spacing sz,
                           double ix, double iy, double iz, ApicBox box,
                           const double* __restrict__ u,
                           const double* __restrict__ v,
                           const double* __restrict__ w) {
    const double* g[3] = {u, v, w};
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < np;
         p += (long)gridDim.x * blockDim.x) {
        const double px = pos[3 * p], py = pos[3 * p + 1], pz = pos[3 * p + 2];
        for (int a = 0; a < 3; ++a)
            vel[3 * p + a] = sample_face_d(
                g[a], fs.s[a], sx.div(px - fs.o[a][0]), sy.div(py - fs.o[a][1]),
                sz.div(pz - fs.o[a][2]));
        for (int a = 0; a < 3; ++a) {
            double q[3];
            for (int d = 0; d < 3; ++d)
                q[d] = d == a ? pos[3 * p + d]
                              : clamp_d(pos[3 * p + d], box.lo[d], box.hi[d]);
            const Dims s = fs.s[a];
            int i, j, k;
            double fx, fy, fz;
            bary<double>(sx.div(q[0] - fs.o[a][0]), s.x - 1, &i, &fx);
            bary<double>(sy.div(q[1] - fs.o[a][1]), s.y - 1, &j, &fy);
            bary<double>(sz.div(q[2] - fs.o[a][2]), s.z - 1, &k, &fz);
            const int ip1 = min(i + 1, s.x - 1), jp1 = min(j + 1, s.y - 1),
                      kp1 = min(k + 1, s.z - 1);
            const long idx[8] = {lin(i, j, k, s.x, s.y),     lin(ip1, j, k, s.x, s.y),
                                 lin(i, jp1, k, s.x, s.y),   lin(ip1, jp1, k, s.x, s.y),
                                 lin(i, j, kp1, s.x, s.y),   lin(ip1, j, kp1, s.x, s.y),
                                 lin(i, jp1, kp1, s.x, s.y), lin(ip1, jp1, kp1, s.x, s.y)};
            const double gw[8][3] = {
                {-ix * (1 - fy) * (1 - fz), -iy * (1 - fx) * (1 - fz), -iz * (1 - fx) * (1 - fy)},
                {ix * (1 - fy) * (1 - fz), fx * (-iy) * (1 - fz), fx * (1 - fy) * (-iz)},
                {(-ix) * fy * (1 - fz), (1 - fx) * iy * (1 - fz), (1 - fx) * fy * (-iz)},
                {ix * fy * (1 - fz), fx * iy * (1 - fz), fx * fy * (-iz)},
                {(-ix) * (1 - fy) * fz, (1 - fx) * (-iy) * fz, (1 - fx) * (1 - fy) * iz},
                {ix * (1 - fy) * fz, fx * (-iy) * fz, fx * (1 - fy) * iz},
                {(-ix) * fy * fz, (1 - fx) * iy * fz, (1 - fx) * fy * iz},
                {ix * fy * fz, fx * iy * fz, fx * fy * iz}};
            double C0 = 0.0, C1 = 0.0, C2 = 0.0;
#pragma unroll
            for (int n = 0; n < 8; ++n) {
                const double val = g[a][idx[n]];
                C0 = C0 + gw[n][0] * val;
                C1 = C1 + gw[n][1] * val;
                C2 = C2 + gw[n][2] * val;
            }
            aff[9 * p + 3 * a] = C0;
            aff[9 * p + 3 * a + 1] = C1;
            aff[9 * p + 3 * a + 2] = C2;
        }
    }
}

// K20: PicSolver3::moveParticles (src/jet/pic_solver3.cpp:206-282) and,
// with a sphere collider, Collider3::resolveCollision
// (src/jet/collider3.cpp:19-73, radius 0, restitution 0) through the
// transformed Sphere3 queries (src/jet/sphere3.cpp:25-39,
// src/jet/surface3.cpp:23-79, include/jet/detail/transform3-inl.h:45-79).
// One thread per particle; every expression in the reference's order.
struct SphereDesc {
    int present;
    double center[3], radius;
    int flipped;
    double orient[9], inv[9];
    double t[3];  // translation = collider centre
    double lin[3], ang[3], friction;
};

__device__ __forceinline__ void mat3(const double* m, const double v[3],
                                     double o[3]) {
    o[0] = m[0] * v[0] + m[1] * v[1] + m[2] * v[2];
    o[1] = m[3] * v[0] + m[4] * v[1] + m[5] * v[2];
    o[2] = m[6] * v[0] + m[7] * v[1] + m[8] * v[2];
}

__device__ __forceinline__ double dmax(double a, double b) {
    return a < b ? b : a;
}

__device__ void resolve_sphere(const SphereDesc& S, double p[3],
                               double vv[3]) {
    const double dp[3] = {p[0] - S.t[0], p[1] - S.t[1], p[2] - S.t[2]};
    double pl[3];
    mat3(S.inv, dp, pl);
    const double* c = S.center;
    double nl[3];
    const double eps = 2.220446049250313e-16;  // numeric_limits::epsilon()
    if (fabs(c[0] - pl[0]) < eps && fabs(c[1] - pl[1]) < eps &&
        fabs(c[2] - pl[2]) < eps) {
        nl[0] = 1.0;
        nl[1] = 0.0;
        nl[2] = 0.0;
    } else {
        const double d0 = pl[0] - c[0], d1 = pl[1] - c[1], d2 = pl[2] - c[2];
        const double l = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
        nl[0] = d0 / l;
        nl[1] = d1 / l;
        nl[2] = d2 / l;
    }
    const double r = S.radius;
    const double cpl[3] = {r * nl[0] + c[0], r * nl[1] + c[1],
                           r * nl[2] + c[2]};
    const double e0 = c[0] - pl[0], e1 = c[1] - pl[1], e2 = c[2] - pl[2];
    const double dist = fabs(sqrt(e0 * e0 + e1 * e1 + e2 * e2) - r);
    const double o0 = pl[0] - cpl[0], o1 = pl[1] - cpl[1], o2 = pl[2] - cpl[2];
    const bool in_local = o0 * nl[0] + o1 * nl[1] + o2 * nl[2] < 0.0;
    const bool is_in = (S.flipped != 0) == !in_local;
    if (!(is_in || dist < 0.0)) return;
    double cpw[3], nw[3];
    mat3(S.orient, cpl, cpw);
    for (int d = 0; d < 3; ++d) cpw[d] = cpw[d] + S.t[d];
    mat3(S.orient, nl, nw);
    const double fl = S.flipped ? -1.0 : 1.0;
    for (int d = 0; d < 3; ++d) nw[d] *= fl;
    const double* a = S.ang;
    const double r0 = p[0] - S.t[0], r1 = p[1] - S.t[1], r2 = p[2] - S.t[2];
    const double cv[3] = {S.lin[0] + (a[1] * r2 - r1 * a[2]),
                          S.lin[1] + (a[2] * r0 - r2 * a[0]),
                          S.lin[2] + (a[0] * r1 - r0 * a[1])};
    double tp[3];
    for (int d = 0; d < 3; ++d) tp[d] = cpw[d] + 0.0 * nw[d];
    const double rv[3] = {vv[0] - cv[0], vv[1] - cv[1], vv[2] - cv[2]};
    const double ndv = nw[0] * rv[0] + nw[1] * rv[1] + nw[2] * rv[2];
    double rn[3] = {ndv * nw[0], ndv * nw[1], ndv * nw[2]};
    double rt[3] = {rv[0] - rn[0], rv[1] - rn[1], rv[2] - rn[2]};
    if (ndv < 0.0) {
        const double rest = 0.0;
        const double dn[3] = {(-rest - 1.0) * rn[0], (-rest - 1.0) * rn[1],
                              (-rest - 1.0) * rn[2]};
        for (int d = 0; d < 3; ++d) rn[d] *= -rest;
        const double lt2 = rt[0] * rt[0] + rt[1] * rt[1] + rt[2] * rt[2];
        if (lt2 > 0.0) {
            const double ldn = sqrt(dn[0] * dn[0] + dn[1] * dn[1] + dn[2] * dn[2]);
            const double fs = dmax(1.0 - S.friction * ldn / sqrt(lt2), 0.0);
            for (int d = 0; d < 3; ++d) rt[d] *= fs;
        }
        for (int d = 0; d < 3; ++d) vv[d] = rn[d] + rt[d] + cv[d];
    }
    for (int d = 0; d < 3; ++d) p[d] = tp[d];
}

template <bool kZeroOrigin>
__global__ void k_move_particles(long np, double* __restrict__ pos,
                                 double* __restrict__ vel, FaceSet fs,
                                 const double* __restrict__ u,
                                 const double* __restrict__ v,
                                 const double* __restrict__ w, Spacing hx,
                                 Spacing hy, Spacing hz, double sdt,
                                 unsigned nsub, int closed, double lo0,
                                 double lo1, double lo2, double hi0,
                                 double hi1, double hi2, SphereDesc S) {
    const double* grid[3] = {u, v, w};
    const double lo[3] = {lo0, lo1, lo2}, hi[3] = {hi0, hi1, hi2};
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < np;
         q += (long)gridDim.x * blockDim.x) {
        double p0[3] = {pos[3 * q], pos[3 * q + 1], pos[3 * q + 2]};
        double p1[3] = {p0[0], p0[1], p0[2]};
        double vv[3] = {vel[3 * q], vel[3 * q + 1], vel[3 * q + 2]};
        // The three face grids share their data origins axis by axis (the
        // grid origin on a face's normal axis, origin + h/2 on the others),
        // so each point needs six subtractions, not nine; with the grid
        // origin at +0 the normal-axis ones are x - (+0) = x exactly.
        const Spacing sp[3] = {hx, hy, hz};
        auto sample3 = [&](const double q[3], double out[3]) {
            double nn[3], nt[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                nn[d] = sp[d].div(kZeroOrigin ? q[d] : q[d] - fs.o[d][d]);
                nt[d] = sp[d].div(q[d] - fs.o[(d + 1) % 3][d]);
            }
#pragma unroll
            for (int a = 0; a < 3; ++a)
                out[a] = sample_face_d(
                    grid[a], fs.s[a], a == 0 ? nn[0] : nt[0],
                    a == 1 ? nn[1] : nt[1], a == 2 ? nn[2] : nt[2]);
        };
        for (unsigned t = 0; t < nsub; ++t) {
            double v0[3], mid[3], vm[3];
            sample3(p0, v0);
            const double hs = 0.5 * sdt;
            for (int d = 0; d < 3; ++d) mid[d] = p0[d] + hs * v0[d];
            sample3(mid, vm);
            for (int d = 0; d < 3; ++d) p1[d] = p0[d] + sdt * vm[d];
            for (int d = 0; d < 3; ++d) p0[d] = p1[d];
        }
        for (int d = 0; d < 3; ++d) {
            if ((closed & (1 << (2 * d))) && p1[d] <= lo[d]) {
                p1[d] = lo[d];
                vv[d] = 0.0;
            }
            if ((closed & (1 << (2 * d + 1))) && p1[d] >= hi[d]) {
                p1[d] = hi[d];
                vv[d] = 0.0;
            }
        }
        if (S.present) resolve_sphere(S, p1, vv);
        for (int d = 0; d < 3; ++d) {
            pos[3 * q + d] = p1[d];
            vel[3 * q + d] = vv[d];
        }
    }
}

}  // namespace

jetgpu_status move_particles(Ctx* c, const GridDesc& g, long np, double* pos,
                             double* vel, const double* u, const double* v,
                             const double* w, double dt, double max_cfl,
                             int closed, const jetgpu_collider* col,
                             const jetgpu_sphere* sph) {
    const FaceSet fs = face_set(g);
    double lo[3], hi[3];  // Grid3::boundingBox (src/jet/grid3.cpp:77)
    for (int d = 0; d < 3; ++d) {
        const double e = g.origin[d] + g.spacing[d] * (double)g.res[d];
        lo[d] = std::min(g.origin[d], e);
        hi[d] = std::max(g.origin[d], e);
    }
    const unsigned nsub = (unsigned)std::max(max_cfl, 1.0);
    SphereDesc S{};
    if (col && sph) {
        S.present = 1;
        for (int d = 0; d < 3; ++d) {
            S.center[d] = sph->center[d];
            S.t[d] = col->centre[d];
            S.lin[d] = col->linear_velocity[d];
            S.ang[d] = col->angular_velocity[d];
        }
        S.radius = sph->radius;
        S.flipped = sph->normal_flipped;
        for (int i = 0; i < 9; ++i) {
            S.orient[i] = sph->orientation[i];
            S.inv[i] = sph->inverse_orientation[i];
        }
        S.friction = col->friction;
    }
    if (np > 0) {
        Prof pr(c, K_MOVE, 96.0 * np);
        bool zero_origin = true;  // all three components are +0.0
        for (int d = 0; d < 3; ++d)
            zero_origin = zero_origin && dbits(g.origin[d]) == 0ull;
        auto kern = zero_origin ? k_move_particles<true>
                                : k_move_particles<false>;
        kern<<<blocks_for(np, kThreads, c->num_sms * 16), kThreads, 0,
               c->stream>>>(
            np, pos, vel, fs, u, v, w, make_spacing(g.spacing[0]),
            make_spacing(g.spacing[1]), make_spacing(g.spacing[2]), dt / nsub,
            nsub, closed, lo[0], lo[1], lo[2], hi[0],
            hi[1], hi[2], S);
    }
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

// The ordered P2G of all three components (k_p2g_bin .. k_p2g_gather): every
// face's value, weight sum and marker written.
static jetgpu_status p2g_ordered(Ctx* c, const GridDesc& g, long np,
                                 const double* pos, const double* vel,
                                 const FaceSet& fs, const long n[3],
                                 double* const grid[3], double* wsum,
                                 unsigned char* const mark[3]) {
    const long nb = std::max(std::max(n[0], n[1]), n[2]);  // bins (faces)
    const long tiles = scan_tiles(nb);
    // Ints: key, list, sorted list (np each), count, off (nb + 1), cursor,
    // scan totals (tiles), the grand total, and the gather's face counter
    // (two ints, 8-byte aligned).
    const size_t ni = (size_t)(3 * np + 3 * nb + 1 + tiles + 1 + 3);
    if (c->p2g_int_cap < ni) {
        if (c->p2g_int) cudaFree(c->p2g_int);
        c->p2g_int = nullptr;
        c->p2g_int_cap = 0;
        JG_CUDA(c, cudaMalloc((void**)&c->p2g_int, ni * sizeof(int)));
        c->p2g_int_cap = ni;
    }
    const size_t nd = (size_t)(8 * np);  // records: two double4_32a a particle
    if (c->p2g_dbl_cap < nd) {
        if (c->p2g_dbl) cudaFree(c->p2g_dbl);
        c->p2g_dbl = nullptr;
        c->p2g_dbl_cap = 0;
        JG_CUDA(c, cudaMalloc((void**)&c->p2g_dbl, nd * sizeof(double)));
        c->p2g_dbl_cap = nd;
    }
    int* key = c->p2g_int;
    int* list = key + np;
    int* slist = list + np;
    int* count = slist + np;
    int* off = count + nb;
    int* cursor = off + nb + 1;
    int* tile_sum = cursor + nb;
    int* grand = tile_sum + tiles;
    const size_t ci = ((size_t)(grand + 1 - c->p2g_int) + 1) & ~(size_t)1;
    unsigned long long* counter =
        reinterpret_cast<unsigned long long*>(c->p2g_int + ci);
    double4_32a* rec = reinterpret_cast<double4_32a*>(c->p2g_dbl);
    const int cap = c->num_sms * 16;
    // 32-bit keys (particle index << 3 | list) while indices fit 28 bits;
    // 1024-face chunks unless a component has fewer than two per block.
    const bool k32 = np < (1l << 28);
    auto gk = [&](bool small) {
        return k32 ? (small ? (const void*)k_p2g_gather<unsigned, 256>
                            : (const void*)k_p2g_gather<unsigned, 1024>)
                   : (small ? (const void*)k_p2g_gather<unsigned long long, 256>
                            : (const void*)k_p2g_gather<unsigned long long, 1024>);
    };
    int gather_grid = 0;
    JG_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                   &gather_grid, gk(false), kGatherThreads, 0));
    gather_grid = std::max(1, gather_grid) * c->num_sms;
    long woff = 0;
    for (int a = 0; a < 3; ++a) {
        // Algorithmic bytes: a third of the particles' positions and
        // velocities, and the face's value, weight sum and marker.
        Prof pr(c, K_P2G, 16.0 * np + 17.0 * n[a]);
        const Dims s = fs.s[a];
        const P2gLattice L = p2g_lattice(fs, a, g.spacing);
        const int dm = (s.x == 1 ? 1 : 0) | (s.y == 1 ? 2 : 0) |
                       (s.z == 1 ? 4 : 0);
        JG_CUDA(c, cudaMemsetAsync(count, 0, n[a] * sizeof(int), c->stream));
        JG_CUDA(c, cudaMemsetAsync(cursor, 0, n[a] * sizeof(int), c->stream));
        JG_CUDA(c, cudaMemsetAsync(counter, 0, sizeof(unsigned long long),
                                   c->stream));
        k_p2g_bin<<<blocks_for(np, kThreads, cap), kThreads, 0, c->stream>>>(
            np, pos, L, key, count);
        jetgpu_status st = scan_counts(c, count, off, n[a], tile_sum, grand);
        if (st != JETGPU_OK) return st;
        k_p2g_fill<<<blocks_for(np, kThreads, cap), kThreads, 0, c->stream>>>(
            np, key, off, cursor, list);
        k_p2g_place<<<blocks_for(np, kThreads, cap), kThreads, 0,
                      c->stream>>>(np, pos, vel, L, a, key, off, list, slist,
                                   rec);
        const bool small = n[a] < 2048l * gather_grid;
        Dims sa = s;
        int dma = dm;
        const int* count_a = count;
        const int* off_a = off;
        const int* slist_a = slist;
        const double4_32a* rec_a = rec;
        double* grid_a = grid[a];
        double* wsum_a = wsum + woff;
        unsigned char* mark_a = mark[a];
        void* args[] = {&sa,      &dma,    &count_a, &off_a,  &slist_a,
                        &rec_a,   &grid_a, &wsum_a,  &mark_a, &counter};
        JG_CUDA(c, cudaLaunchKernel(gk(small), dim3(gather_grid),
                                    dim3(kGatherThreads), args, 0, c->stream));
        woff += n[a];
    }
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

jetgpu_status p2g(Ctx* c, const GridDesc& g, long np, const double* pos,
                  const double* vel, double* u, double* v, double* w,
                  unsigned char* mu, unsigned char* mv, unsigned char* mw,
                  float* su, float* sv, float* sw) {
    const FaceSet fs = face_set(g);
    const long n[3] = {fs.s[0].count(), fs.s[1].count(), fs.s[2].count()};
    const size_t need = (size_t)(n[0] + n[1] + n[2]) * sizeof(double);
    if (need > c->pscratch_bytes) {
        if (c->pscratch) cudaFree(c->pscratch);
        c->pscratch = nullptr;
        c->pscratch_bytes = 0;
        JG_CUDA(c, cudaMalloc((void**)&c->pscratch, need));
        c->pscratch_bytes = need;
    }
    double* wsum = reinterpret_cast<double*>(c->pscratch);
    double* grid[3] = {u, v, w};
    unsigned char* mark[3] = {mu, mv, mw};
    float* snap[3] = {su, sv, sw};
    // The ordered gather writes every face (value, weight sum, marker) and
    // keeps its particle and bin numbers in ints.
    const bool ordered = np > 0 && c->cfg.ordered_p2g && np < INT_MAX &&
                         std::max(std::max(n[0], n[1]), n[2]) < INT_MAX;
    if (!ordered) {
        JG_CUDA(c, cudaMemsetAsync(wsum, 0, need, c->stream));
        for (int a = 0; a < 3; ++a) {
            JG_CUDA(c, cudaMemsetAsync(grid[a], 0, n[a] * sizeof(double),
                                       c->stream));
            if (mark[a])
                JG_CUDA(c, cudaMemsetAsync(mark[a], 0, n[a], c->stream));
        }
    }
    if (ordered) {
        jetgpu_status os = p2g_ordered(c, g, np, pos, vel, fs, n, grid, wsum,
                                       mark);
        if (os != JETGPU_OK) return os;
    } else if (np > 0) {
        Prof pr(c, K_P2G, 48.0 * np + 2.0 * 3 * 8.0 * (n[0] + n[1] + n[2]));
        k_p2g_scatter<<<blocks_for(np, kThreads, c->num_sms * 16), kThreads, 0,
                        c->stream>>>(np, pos, vel, p2g_lattices(fs, g.spacing),
                                     u, v, w, wsum, wsum + n[0],
                                     wsum + n[0] + n[1], mu, mv, mw);
    }
    long off = 0;
    for (int a = 0; a < 3; ++a) {
        Prof pr(c, K_P2G, 28.0 * n[a]);
        k_p2g_normalize<<<blocks_for(n[a]), kThreads, 0, c->stream>>>(
            grid[a], wsum + off, snap[a], n[a]);
        off += n[a];
    }
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

jetgpu_status g2p_flip(Ctx* c, const GridDesc& g, long np, const double* pos,
                       double* vel, const double* u, const double* v,
                       const double* w, float* su, float* sv, float* sw,
                       double blend) {
    const FaceSet fs = face_set(g);
    const double* grid[3] = {u, v, w};
    float* snap[3] = {su, sv, sw};
    for (int a = 0; a < 3; ++a)
        k_flip_delta<<<blocks_for(fs.s[a].count()), kThreads, 0, c->stream>>>(
            grid[a], snap[a], fs.s[a].count());
    if (np > 0) {
        Prof pr(c, K_G2P, 48.0 * np);
        k_g2p_flip<<<blocks_for(np), kThreads, 0, c->stream>>>(
            np, pos, vel, fs, (float)g.spacing[0], (float)g.spacing[1],
            (float)g.spacing[2], su, sv, sw, u, v, w,
            make_spacing(g.spacing[0]), make_spacing(g.spacing[1]),
            make_spacing(g.spacing[2]), blend);
    }
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

static ApicBox apic_box(const GridDesc& g) {
    ApicBox b;
    for (int d = 0; d < 3; ++d) {
        const double e = g.origin[d] + g.spacing[d] * (double)g.res[d];
        const double hh = g.spacing[d] / 2.0;
        b.lo[d] = std::min(g.origin[d], e) + hh;
        b.hi[d] = std::max(g.origin[d], e) - hh;
    }
    return b;
}

jetgpu_status apic_p2g(Ctx* c, const GridDesc& g, long np, const double* pos,
                       const double* vel, const double* aff, double* u,
                       double* v, double* w, unsigned char* mu,
                       unsigned char* mv, unsigned char* mw) {
    const FaceSet fs = face_set(g);
    const long n[3] = {fs.s[0].count(), fs.s[1].count(), fs.s[2].count()};
    const size_t need = (size_t)(n[0] + n[1] + n[2]) * sizeof(double);
    if (need > c->pscratch_bytes) {
        if (c->pscratch) cudaFree(c->pscratch);
        c->pscratch = nullptr;
        c->pscratch_bytes = 0;
        JG_CUDA(c, cudaMalloc((void**)&c->pscratch, need));
        c->pscratch_bytes = need;
    }
    double* wsum = reinterpret_cast<double*>(c->pscratch);
    double* grid[3] = {u, v, w};
    unsigned char* mark[3] = {mu, mv, mw};
    JG_CUDA(c, cudaMemsetAsync(wsum, 0, need, c->stream));
    for (int a = 0; a < 3; ++a) {
        JG_CUDA(c, cudaMemsetAsync(grid[a], 0, n[a] * sizeof(double), c->stream));
        if (mark[a]) JG_CUDA(c, cudaMemsetAsync(mark[a], 0, n[a], c->stream));
    }
    if (np > 0) {
        Prof pr(c, K_P2G, 120.0 * np + 2.0 * 3 * 8.0 * (n[0] + n[1] + n[2]));
        k_apic_p2g_scatter<<<blocks_for(np, kThreads, c->num_sms * 16),
                             kThreads, 0, c->stream>>>(
            np, pos, vel, aff, fs, g.spacing[0], g.spacing[1], g.spacing[2],
            1.0 / g.spacing[0], 1.0 / g.spacing[1], 1.0 / g.spacing[2],
            apic_box(g), u, v, w, wsum, wsum + n[0], wsum + n[0] + n[1], mu,
            mv, mw);
    }
    long off = 0;
    for (int a = 0; a < 3; ++a) {
        k_p2g_normalize<<<blocks_for(n[a]), kThreads, 0, c->stream>>>(
            grid[a], wsum + off, nullptr, n[a]);
        off += n[a];
    }
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

jetgpu_status apic_g2p(Ctx* c, const GridDesc& g, long np, const double* pos,
                       double* vel, double* aff, const double* u,
                       const double* v, const double* w) {
    const FaceSet fs = face_set(g);
    if (np > 0) {
        Prof pr(c, K_G2P, 120.0 * np);
        k_apic_g2p<<<blocks_for(np, kThreads, c->num_sms * 16), kThreads, 0,
                     c->stream>>>(
            np, pos, vel, aff, fs, make_spacing(g.spacing[0]),
            make_spacing(g.spacing[1]), make_spacing(g.spacing[2]),
            1.0 / g.spacing[0], 1.0 / g.spacing[1], 1.0 / g.spacing[2],
            apic_box(g), u, v, w);
    }
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

jetgpu_status g2p_pic(Ctx* c, const GridDesc& g, long np, const double* pos,
                      double* vel, const double* u, const double* v,
                      const double* w) {
    const FaceSet fs = face_set(g);
    if (np > 0)
        k_g2p_pic<<<blocks_for(np), kThreads, 0, c->stream>>>(
            np, pos, vel, fs, u, v, w, make_spacing(g.spacing[0]),
            make_spacing(g.spacing[1]), make_spacing(g.spacing[2]));
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

}  // namespace jg

// ---------------------------------------------------------------------------
// Allocation-free P2G (jetgpu_p2g_device_noalloc). Its only scratch, the
// per-face weight sums, is this fixed array. In host code the name is only a
// host-side stand-in, so the device address is looked up once per device
// with cudaGetSymbolAddress and handed to the kernels.

namespace {

constexpr size_t kNoAllocFaces = JETGPU_P2G_NOALLOC_MAX_FACES;
__device__ __align__(256) double g_p2g_noalloc_wsum[kNoAllocFaces];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
double* g_noalloc_ptr[kMaxDevices] = {};
int g_noalloc_sms[kMaxDevices] = {};

}  // namespace

extern "C" jetgpu_status jetgpu_p2g_device_noalloc(
    void* stream, const jetgpu_grid* grid, long np, const double* pos,
    const double* vel, double* u, double* v, double* w, unsigned char* mu,
    unsigned char* mv, unsigned char* mw, float* su, float* sv, float* sw) {
    using namespace jg;
    if (!grid || !u || !v || !w) return JETGPU_BAD_INPUT;
    if (np < 0 || (np > 0 && (!pos || !vel))) return JETGPU_BAD_INPUT;
    // The same grid checks as the context entry points: positive finite
    // spacing, finite origin, and fewer than 2^31 cells, so that the face
    // counts below cannot wrap before the capacity test.
    for (int a = 0; a < 3; ++a)
        if (grid->res[a] < 1 || !(grid->spacing[a] > 0.0) ||
            !std::isfinite(grid->spacing[a]) || !std::isfinite(grid->origin[a]))
            return JETGPU_BAD_INPUT;
    if ((double)grid->res[0] * grid->res[1] * grid->res[2] > 2147483647.0)
        return JETGPU_BAD_INPUT;
    GridDesc g;
    for (int a = 0; a < 3; ++a) {
        g.res[a] = grid->res[a];
        g.spacing[a] = grid->spacing[a];
        g.origin[a] = grid->origin[a];
    }
    const FaceSet fs = face_set(g);
    const size_t n[3] = {(size_t)fs.s[0].count(), (size_t)fs.s[1].count(),
                         (size_t)fs.s[2].count()};
    const size_t faces = n[0] + n[1] + n[2];
    if (faces > kNoAllocFaces) return JETGPU_CAPACITY_EXCEEDED;

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return JETGPU_CUDA_ERROR;
    double* wsum = nullptr;
    int sms = 0;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_ptr[dev]) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_p2g_noalloc_wsum) != cudaSuccess ||
                !p)
                return JETGPU_CUDA_ERROR;
            int count = 0;
            if (cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount,
                                       dev) != cudaSuccess)
                return JETGPU_CUDA_ERROR;
            g_noalloc_sms[dev] = count;
            g_noalloc_ptr[dev] = static_cast<double*>(p);
        }
        wsum = g_noalloc_ptr[dev];
        sms = g_noalloc_sms[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    double* grids[3] = {u, v, w};
    unsigned char* mark[3] = {mu, mv, mw};
    float* snap[3] = {su, sv, sw};
    // The array keeps the previous call's sums: clear the part used here.
    if (cudaMemsetAsync(wsum, 0, faces * sizeof(double), st) != cudaSuccess)
        return JETGPU_CUDA_ERROR;
    for (int a = 0; a < 3; ++a) {
        if (cudaMemsetAsync(grids[a], 0, n[a] * sizeof(double), st) !=
            cudaSuccess)
            return JETGPU_CUDA_ERROR;
        if (mark[a] && cudaMemsetAsync(mark[a], 0, n[a], st) != cudaSuccess)
            return JETGPU_CUDA_ERROR;
    }
    if (np > 0)
        k_p2g_scatter<<<blocks_for(np, kThreads, sms * 16), kThreads, 0, st>>>(
            np, pos, vel, p2g_lattices(fs, g.spacing), u, v, w, wsum,
            wsum + n[0], wsum + n[0] + n[1], mu, mv, mw);
    size_t off = 0;
    for (int a = 0; a < 3; ++a) {
        k_p2g_normalize<<<blocks_for((long)n[a]), kThreads, 0, st>>>(
            grids[a], wsum + off, snap[a], (long)n[a]);
        off += n[a];
    }
    return cudaGetLastError() == cudaSuccess ? JETGPU_OK : JETGPU_CUDA_ERROR;
}

// Particle signed-distance field (K21): PicSolver3::buildSignedDistanceField
// (src/jet/pic_solver3.cpp:296-317) followed by
// GridFluidSolver3::extrapolateIntoCollider
// (src/jet/grid_fluid_solver3.cpp:423-438).
//
// The reference searches a hash grid for the particles whose squared distance
// (x - p).(x - p) from a cell centre p is at most band^2 (band = 2r,
// r = 1.2 max(h) / sqrt(2)) and keeps min(band, their distances); the value
// stored is that minimum minus r. The minimum does not depend on how the
// particles are found or visited, so here particles are counting-sorted into
// the cells of the SDF grid (K21a-c), and each cell centre scans the bins of
// a window that covers its band (K21d). Exactness: sqrt is correctly rounded
// and monotone, so min over sqrt(d^2) = sqrt(min d^2); d^2 is formed in FP64
// in the reference's order (this unit is built with -fmad=false) and filtered
// with the reference's `<= band^2`. An FP32 copy of the coordinates gives
// the minimum squared distance to within a proven error bound (`slack`,
// computed on the host from the grid's extent); the exact FP64 distance is
// then formed only for the particles whose FP32 distance is within that
// bound of the nearest found (one or two per cell), and a bin whose lower
// bound on the distance exceeds the nearest found is not read (inside the
// fluid only the cell's own bin is). Bound: FP32 issue and L1 traffic over
// the bins, then HBM for the sort.

#include "ctx.h"
#include "sampling.cuh"

#include <cmath>

namespace jg {
namespace {

using namespace smp;

struct SdfGeom {
    Dims n;
    double o[3];     // grid origin
    double d0[3];    // data origin = origin + h/2 (cell centres)
    double h[3];
    double band, band2, radius;
    int win[3];      // bin window half-width per axis
    float slack;     // FP32 error bound on a squared distance near the band
    Spacing sx, sy, sz;  // the spacing, for exact divisions by it
};

// floor((p - o) / h) clamped to [0, n - 1] (NaN: 0): the quotient exactly
// (an exponent add for a power-of-two h) and the floor on the integer pipe.
__device__ __forceinline__ int bin_axis(double p, double o, const Spacing& sp,
                                        int n) {
    int i;
    double f;
    bary_bits(sp.div(p - o), n, &i, &f);
    return i;
}

// K21a: bin index of every particle; counts per bin.
__global__ void k_sdf_count(long np, const double* __restrict__ pos,
                            SdfGeom G, int* __restrict__ key,
                            int* __restrict__ count) {
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < np;
         q += (long)gridDim.x * blockDim.x) {
        const int bx = bin_axis(pos[3 * q], G.o[0], G.sx, G.n.x);
        const int by = bin_axis(pos[3 * q + 1], G.o[1], G.sy, G.n.y);
        const int bz = bin_axis(pos[3 * q + 2], G.o[2], G.sz, G.n.z);
        const int b = bx + G.n.x * (by + G.n.y * bz);
        key[q] = b;
        atomicAdd(&count[b], 1);
    }
}

// K21b: exclusive scan of `count` (n entries) into `off` (n + 1 entries), in
// three passes: per-block scans with block totals, a one-block scan of the
// totals, and the add-back.
constexpr int kScanT = 1024, kScanPer = 4, kScanTile = kScanT * kScanPer;

__device__ int block_excl_scan(int v, int* sh, int* total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) sh[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int s = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, s, d);
            if (lane >= d) s += y;
        }
        sh[lane] = s;
    }
    __syncthreads();
    const int before = wid > 0 ? sh[wid - 1] : 0;
    *total = sh[(blockDim.x >> 5) - 1];
    __syncthreads();
    return before + x - v;
}

__global__ void __launch_bounds__(kScanT)
    k_scan_tiles(const int* __restrict__ in, int* __restrict__ out, long n,
                 int* __restrict__ tile_sum) {
    __shared__ int sh[32];
    const long base = (long)blockIdx.x * kScanTile + threadIdx.x * kScanPer;
    int v[kScanPer], s = 0;
#pragma unroll
    for (int e = 0; e < kScanPer; ++e) {
        v[e] = base + e < n ? in[base + e] : 0;
        s += v[e];
    }
    int total;
    int run = block_excl_scan(s, sh, &total);
#pragma unroll
    for (int e = 0; e < kScanPer; ++e) {
        if (base + e < n) out[base + e] = run;
        run += v[e];
    }
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
}

// One block: exclusive scan of the tile totals in place (any count), the
// grand total in *grand.
__global__ void __launch_bounds__(kScanT)
    k_scan_totals(int* __restrict__ tile_sum, long tiles,
                  int* __restrict__ grand) {
    __shared__ int sh[32];
    int carry = 0;
    for (long b0 = 0; b0 < tiles; b0 += kScanT) {
        const long i = b0 + threadIdx.x;
        const int v = i < tiles ? tile_sum[i] : 0;
        int total;
        const int ex = block_excl_scan(v, sh, &total);
        if (i < tiles) tile_sum[i] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) *grand = carry;
}

__global__ void k_scan_add(int* __restrict__ out, long n,
                           const int* __restrict__ tile_sum,
                           const int* __restrict__ grand) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i <= n;
         i += (long)gridDim.x * blockDim.x)
        out[i] = i < n ? out[i] + tile_sum[i / kScanTile] : *grand;
}

// K21c: scatter particles into their bins: exact coordinates and an FP32
// copy relative to the grid origin.
__global__ void k_sdf_scatter(long np, const double* __restrict__ pos,
                              SdfGeom G, const int* __restrict__ key,
                              const int* __restrict__ off,
                              int* __restrict__ cursor,
                              double* __restrict__ sp,
                              float4* __restrict__ sf) {
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < np;
         q += (long)gridDim.x * blockDim.x) {
        const int b = key[q];
        const int slot = off[b] + atomicAdd(&cursor[b], 1);
        const double x = pos[3 * q], y = pos[3 * q + 1], z = pos[3 * q + 2];
        sp[3 * (long)slot] = x;
        sp[3 * (long)slot + 1] = y;
        sp[3 * (long)slot + 2] = z;
        sf[slot] = make_float4((float)(x - G.o[0]), (float)(y - G.o[1]),
                               (float)(z - G.o[2]), 0.f);
    }
}

// K21d: SDF at every cell centre from the particles of its window. The
// cell's own bin is searched first; then each row of bins of the window
// only over the bins that can still hold a nearer particle: a particle in a
// bin m bins away along an axis is at least (m - 1/2) h from the centre
// along it (bins are cells and the centre sits mid-cell; a particle outside
// the grid is clamped into a boundary bin and is only farther), so a bin
// whose squared lower bound exceeds the nearest found is skipped. Inside the
// fluid the own bin usually holds a particle nearer than h/2 and nothing
// else is read. An FP32 squared distance (error <= slack) screens the
// particles; the exact FP64 distance is formed for those that can beat the
// nearest found.
__global__ void k_sdf_cells(SdfGeom G, const int* __restrict__ off,
                            const double* __restrict__ sp,
                            const float4* __restrict__ sf,
                            double* __restrict__ out) {
    const long N = G.n.count();
    const float slack2 = 2.0f * G.slack;
    const float band2f = (float)G.band2;
    const float hf[3] = {(float)G.h[0], (float)G.h[1], (float)G.h[2]};
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_ijk(c, G.n, i, j, k);
        const double pt[3] = {G.d0[0] + G.h[0] * (double)i,
                              G.d0[1] + G.h[1] * (double)j,
                              G.d0[2] + G.h[2] * (double)k};
        const float cx = (float)(pt[0] - G.o[0]), cy = (float)(pt[1] - G.o[1]),
                    cz = (float)(pt[2] - G.o[2]);
        double best = INFINITY;  // exact squared distance of the nearest
        float thr = band2f + slack2;  // FP32 screen: nearer candidates pass
        float bound = INFINITY;       // >= best: bins beyond it are skipped
        auto scan = [&](int e0, int e1) {
            for (int e = e0; e < e1; ++e) {
                const float4 p = sf[e];
                const float dx = p.x - cx, dy = p.y - cy, dz = p.z - cz;
                if (dx * dx + dy * dy + dz * dz > thr) continue;
                const double* x = sp + 3 * (long)e;
                const double d0 = x[0] - pt[0], d1 = x[1] - pt[1],
                             d2 = x[2] - pt[2];
                const double dd = d0 * d0 + d1 * d1 + d2 * d2;
                if (dd <= G.band2 && dd < best) {
                    best = dd;
                    const float bf = (float)dd * 1.0001f;
                    bound = bf;
                    thr = fminf(thr, bf + slack2);
                }
            }
        };
        // Squared lower bound, from below, of the distance along axis d to
        // a bin m bins away.
        auto lb = [&](int d, int m) {
            const float t = ((float)m - 0.5f) * hf[d];
            return m > 0 ? t * t * 0.9999f : 0.f;
        };
        const long rowlen = G.n.x, plane = (long)G.n.x * G.n.y;
        scan(off[c], off[c + 1]);
        // The rows of the window: the 3 x 3 around the cell's own first.
        const int z0 = max(k - G.win[2], 0), z1 = min(k + G.win[2], G.n.z - 1);
        const int y0 = max(j - G.win[1], 0), y1 = min(j + G.win[1], G.n.y - 1);
        const int x0 = max(i - G.win[0], 0), x1 = min(i + G.win[0], G.n.x - 1);
        for (int phase = 0; phase < 2; ++phase)
            for (int bz = z0; bz <= z1; ++bz) {
                const int mz = abs(bz - k);
                const float lz = lb(2, mz);
                if (lz > bound) continue;
                for (int by = y0; by <= y1; ++by) {
                    const int my = abs(by - j);
                    if ((phase == 0) != (my <= 1 && mz <= 1)) continue;
                    const float lyz = lz + lb(1, my);
                    if (lyz > bound) continue;
                    // Widest x offset still within the bound.
                    int m = 0;
                    while (m < G.win[0] && lyz + lb(0, m + 1) <= bound) ++m;
                    const int lo = max(x0, i - m), hi = min(x1, i + m);
                    const long row = rowlen * by + plane * bz;
                    if (my == 0 && mz == 0) {  // own bin already searched
                        if (lo < i) scan(off[row + lo], off[row + i]);
                        if (i < hi) scan(off[row + i + 1], off[row + hi + 1]);
                    } else {
                        scan(off[row + lo], off[row + hi + 1]);
                    }
                }
            }
        double minDist = G.band;
        if (best <= G.band2) {
            const double dist = sqrt(best);
            minDist = dist < minDist ? dist : minDist;
        }
        out[c] = minDist - G.radius;
    }
}

// Validity for extrapolateIntoCollider: cells whose centre is not inside the
// collider SDF.
struct Spacing3 {
    Spacing s[3];
};

__global__ void k_sdf_valid(SdfGeom G, FieldDesc col, Spacing3 cs,
                            unsigned char* __restrict__ valid) {
    const long N = G.n.count();
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_ijk(c, G.n, i, j, k);
        double phi = col.value;
        if (col.kind == 1) {
            const double x = G.d0[0] + G.h[0] * (double)i;
            const double y = G.d0[1] + G.h[1] * (double)j;
            const double z = G.d0[2] + G.h[2] * (double)k;
            const Dims s{col.res[0], col.res[1], col.res[2]};
            phi = sample_face_grid(col.data, s, cs.s[0].div(x - col.origin[0]),
                                   cs.s[1].div(y - col.origin[1]),
                                   cs.s[2].div(z - col.origin[2]));
        }
        valid[c] = phi < 0.0 ? 0 : 1;
    }
}

template <typename T>
jetgpu_status grow(Ctx* c, T** p, size_t* cap, size_t n) {
    if (*cap >= n) return JETGPU_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    JG_CUDA(c, cudaMalloc((void**)p, n * sizeof(T)));
    *cap = n;
    return JETGPU_OK;
}

}  // namespace

long scan_tiles(long n) { return (n + kScanTile - 1) / kScanTile; }

jetgpu_status scan_counts(Ctx* c, const int* count, int* off, long n,
                          int* tile_sum, int* grand) {
    cudaStream_t st = c->stream;
    const int cap = c->num_sms * 16;
    const long tiles = scan_tiles(n);
    k_scan_tiles<<<(int)tiles, kScanT, 0, st>>>(count, off, n, tile_sum);
    k_scan_totals<<<1, kScanT, 0, st>>>(tile_sum, tiles, grand);
    k_scan_add<<<blocks_for(n + 1, kThreads, cap), kThreads, 0, st>>>(
        off, n, tile_sum, grand);
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

jetgpu_status build_particle_sdf(Ctx* c, const GridDesc& g, long np,
                                 const double* pos, const FieldDesc& col,
                                 double max_cfl, double* out) {
    SdfGeom G;
    G.n = Dims{g.res[0], g.res[1], g.res[2]};
    double extent = 0.0;
    for (int d = 0; d < 3; ++d) {
        G.o[d] = g.origin[d];
        G.h[d] = g.spacing[d];
        G.d0[d] = g.origin[d] + 0.5 * g.spacing[d];
        extent = std::max(extent, g.spacing[d] * g.res[d]);
    }
    const double maxH = std::max(std::max(G.h[0], G.h[1]), G.h[2]);
    G.radius = 1.2 * maxH / std::sqrt(2.0);
    G.band = 2.0 * G.radius;
    G.band2 = G.band * G.band;
    for (int d = 0; d < 3; ++d)
        G.win[d] = (int)std::ceil(G.band / G.h[d]);
    G.sx = make_spacing(G.h[0]);
    G.sy = make_spacing(G.h[1]);
    G.sz = make_spacing(G.h[2]);
    // FP32 error of a squared distance d^2 <= band^2 + slack between a
    // particle and a centre whose offsets from the origin are at most
    // L = extent + band: each rounded offset is off by <= u L (u = 2^-24), a
    // difference by <= u (2L + band); the squares and sums add <= 4 u d^2.
    const double u = std::ldexp(1.0, -24);
    const double L = extent + G.band;
    const double e = u * (2.0 * L + G.band) + u * L;
    G.slack = (float)(4.0 * (6.0 * G.band * e + 3.0 * e * e + 4.0 * u * G.band2) +
                      1e-30);
    const long N = G.n.count();
    // Scratch: counts/offsets (N + 1), cursors (N), keys (np), sorted exact
    // (3 np) and FP32 (np) coordinates, scan totals, validity (N).
    const long tiles = (N + kScanTile - 1) / kScanTile;
    if (jetgpu_status s = grow(c, &c->sdf_int, &c->sdf_int_cap,
                               (size_t)(3 * N + 2 + tiles + np)))
        return s;
    // The FP32 copy starts on a 16-byte boundary (an even double index).
    const long fstart = (3 * np + 1) & ~1L;
    if (jetgpu_status s = grow(c, &c->sdf_dbl, &c->sdf_dbl_cap,
                               (size_t)(fstart + 2 * np + 2)))
        return s;
    if (jetgpu_status s = grow(c, &c->sdf_valid, &c->sdf_valid_cap, (size_t)N))
        return s;
    int* count = c->sdf_int;
    int* off = count + N;         // N + 1
    int* cursor = off + N + 1;    // N
    int* tile_sum = cursor + N;   // tiles
    int* grand = tile_sum + tiles;
    int* key = grand + 1;         // np
    double* sp = c->sdf_dbl;
    float4* sf = reinterpret_cast<float4*>(sp + fstart);
    cudaStream_t st = c->stream;
    const int cap = c->num_sms * 16;
    {
        Prof pr(c, K_SDF, 24.0 * np + 8.0 * N);
        JG_CUDA(c, cudaMemsetAsync(count, 0, sizeof(int) * N, st));
        JG_CUDA(c, cudaMemsetAsync(cursor, 0, sizeof(int) * N, st));
        if (np > 0)
            k_sdf_count<<<blocks_for(np, kThreads, cap), kThreads, 0, st>>>(
                np, pos, G, key, count);
        k_scan_tiles<<<(int)tiles, kScanT, 0, st>>>(count, off, N, tile_sum);
        k_scan_totals<<<1, kScanT, 0, st>>>(tile_sum, tiles, grand);
        k_scan_add<<<blocks_for(N + 1, kThreads, cap), kThreads, 0, st>>>(
            off, N, tile_sum, grand);
        if (np > 0)
            k_sdf_scatter<<<blocks_for(np, kThreads, cap), kThreads, 0, st>>>(
                np, pos, G, key, off, cursor, sp, sf);
    }
    {
        Prof pr(c, K_SDF, 8.0 * N + 40.0 * np);
        k_sdf_cells<<<blocks_for(N, kThreads, cap), kThreads, 0, st>>>(
            G, off, sp, sf, out);
    }
    const Spacing3 cs{{make_spacing(col.spacing[0]), make_spacing(col.spacing[1]),
                       make_spacing(col.spacing[2])}};
    k_sdf_valid<<<blocks_for(N, kThreads, cap), kThreads, 0, st>>>(
        G, col, cs, c->sdf_valid);
    JG_CUDA(c, cudaGetLastError());
    return extrapolate_region(c, G.n, out, c->sdf_valid,
                              (unsigned)std::ceil(max_cfl));
}

}  // namespace jg

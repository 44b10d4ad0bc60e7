// K8 (fused, TMA): one full red-black SOR sweep of a multigrid level in a
// single pass over memory, with the planes staged into shared memory by the
// Tensor Memory Accelerator.
//
// Replaces one call of FdmGaussSeidelSolver3::relaxRedBlack
// (src/jet/fdm_gauss_seidel_solver3.cpp:150-221): the first colour F, then
// the second colour S, each cell x = (1-w) x + w (b - sum_nb a x_nb) / a_c
// with the 7-point neighbour sum of FdmBlas3::mvm
// (src/jet/fdm_linear_system3.cpp:79-96).
//
// A block owns a tile of TX x TY cells in (i, j) and marches through a run
// of k planes. One elected thread issues the TMA copies
// (cp.async.bulk.tensor): per plane, x with a two-cell ring into the x ring,
// and the four row components (center, right, up, front; one 4-D box) plus b
// with a one-cell ring into the row ring. Boxes that leave the grid are
// zero-filled by the TMA unit, which reproduces the reference's guarded
// neighbour terms (x = 0, a = 0 outside). Every copy completes on an
// mbarrier; x runs D planes ahead of its first use and the rows and b, which
// are first read one plane later, are issued one plane later, so the rings
// hold only the planes a step reads plus those in flight.
//
// Each thread owns a group of 4 consecutive cells of one row; at every plane
// a group holds two cells of each colour. Step t of the march
//   (1) updates the F cells of plane t+1 on the tile plus one ring group /
//       ring row (the S update of the tile needs them) from old values, and
//       publishes them in a two-plane shared buffer;
//   (2) updates the S cells of plane t on the tile from the new F values of
//       planes t-1, t, t+1 (its own registers for t+-1, the shared buffer for
//       the in-plane neighbours) and writes the whole group of plane t as one
//       16-byte store.
// x is read from the staged copy of `xin` and written to `xout` (ping-pong),
// so blocks never observe each other's updates: the result is exactly the
// sequential red-then-black sweep, deterministic, with no inter-block
// synchronisation and one block barrier per plane.
//
// Requirements: nx a multiple of 8 (TMA strides are 16-byte multiples for
// BF16 rows), all arrays 16-byte aligned.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>

#include "tc.cuh"

namespace jg {
namespace tsw {

constexpr int TX = 64;          // tile width in cells
constexpr int TY = 8;           // tile rows
constexpr int G = TX / 4 + 2;   // groups per staged row: tile + one each side
constexpr int FR = TY + 2;      // rows with F updates: tile + one each side
constexpr int NF = G * FR;      // threads with work
constexpr int BLOCK = (NF + 31) / 32 * 32;
constexpr int XW = TX + 8;      // x / b / F-buffer row: cells i0-4 .. i0+TX+3
constexpr int XH = TY + 4;      // x rows j0-2 .. j0+TY+1
constexpr int BH = TY + 2;      // b rows j0-1 .. j0+TY
constexpr int RH = TY + 3;      // row-coefficient rows j0-2 .. j0+TY
constexpr int GAP = 128;        // guard before each region (reads at -1)

__host__ __device__ constexpr int up128(int b) { return (b + 127) / 128 * 128; }

// Row-component element: FP32, or BF16 kept as its 16 bits. The rows box
// starts H cells left of the tile so its first coordinate is 16-byte aligned.
template <typename E> struct Elem;
template <> struct Elem<float> {
    static constexpr int H = 4;
    static constexpr CUtensorMapDataType dtype = CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    __device__ static float4 ld4(const float* p) {
        return *reinterpret_cast<const float4*>(p);
    }
    __device__ static float ld1(const float* p) { return *p; }
};
template <> struct Elem<unsigned short> {
    static constexpr int H = 8;
    static constexpr CUtensorMapDataType dtype = CU_TENSOR_MAP_DATA_TYPE_UINT16;
    __device__ static float4 ld4(const unsigned short* p) {
        const uint2 a = *reinterpret_cast<const uint2*>(p);
        return make_float4(__uint_as_float(a.x << 16),
                           __uint_as_float(a.x & 0xffff0000u),
                           __uint_as_float(a.y << 16),
                           __uint_as_float(a.y & 0xffff0000u));
    }
    __device__ static float ld1(const unsigned short* p) {
        return __uint_as_float((unsigned)*p << 16);
    }
};

// Shared-memory layout (byte offsets from a 128-byte aligned base). Ring
// depths: a step t reads x of planes t+1 (neighbours) and t+2 (own cells)
// and stages x of t+2+D; it reads the rows and b of plane t+1 and stages
// those of t+1+D. Everything a step needs from planes t and t-1 is held in
// registers (see the kernel), so each ring holds the planes read plus those
// in flight.
template <typename E, int D>
struct Layout {
    static constexpr int XR = D + 2, AR = D + 1;
    static constexpr int RW = TX + 2 * Elem<E>::H;
    static constexpr int X_BYTES = XH * XW * 4;
    static constexpr int R_BYTES = 4 * RH * RW * (int)sizeof(E);
    static constexpr int B_BYTES = BH * XW * 4;
    static constexpr int X_STEP = GAP + up128(X_BYTES);
    static constexpr int R_STEP = GAP + up128(R_BYTES);
    static constexpr int B_STEP = GAP + up128(B_BYTES);
    static constexpr int X_OFF = GAP;  // ring entries, each after a guard
    static constexpr int R_OFF = X_OFF + XR * X_STEP;
    static constexpr int B_OFF = R_OFF + AR * R_STEP;
    static constexpr int YF_OFF = B_OFF + AR * B_STEP;
    static constexpr int YF_BYTES = 2 * FR * XW * 4;
    static constexpr int BAR_OFF = YF_OFF + up128(YF_BYTES) + GAP;
    static constexpr int TOTAL = BAR_OFF + 8 * (XR + AR) + 128;
};

__device__ __forceinline__ void expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile(
        "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(
            tc::smem_u32(bar)),
        "r"(bytes)
        : "memory");
}
__device__ __forceinline__ void tma3(void* dst, const CUtensorMap* m, int c0,
                                     int c1, int c2, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::"
        "bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(tc::smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(m)), "r"(c0), "r"(c1), "r"(c2),
        "r"(tc::smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void tma4(void* dst, const CUtensorMap* m, int c0,
                                     int c1, int c2, int c3, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::"
        "bytes [%0], [%1, {%2, %3, %4, %5}], [%6];\n" ::"r"(tc::smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(m)), "r"(c0), "r"(c1), "r"(c2), "r"(c3),
        "r"(tc::smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ float4 lds4(const float* p) {
    return *reinterpret_cast<const float4*>(p);
}
// e ? b : a.
__device__ __forceinline__ float sel(int e, float a, float b) {
    return e ? b : a;
}

// One ring of staged planes: the slot and mbarrier phase of the next plane
// to arrive, advanced one plane at a time (no division in the loop).
struct Ring {
    int slot = 0;
    unsigned phase = 0;
    template <int N>
    __device__ __forceinline__ void advance() {
        if (++slot == N) {
            slot = 0;
            phase ^= 1u;
        }
    }
};

// Rows and rhs a cell pair (offsets s and s+2 of a group) needs for its
// second-colour update, picked out of the group's staged values when the
// plane's first colour is updated one step earlier: centre, left, right,
// down, up, front and back coefficients and b.
struct PairRows {
    float c[2], l[2], r[2], d[2], u[2], f[2], k[2], b[2];
};

// ZERO: the sweep starts from x = 0 (no x is staged). tm_x covers xin
// (nx, ny, nz) FP32, box (XW, XH); tm_r the rows (nx, ny, nz, 4) of E, box
// (RW, RH, 1, 4); tm_b covers b, box (XW, BH). `err` (a device scalar) is set
// to 1 when a copy did not arrive within the wait limit; the kernel then
// stops waiting, finishes its loop on whatever the rings hold, and before it
// exits waits (bounded) for the copies it issued.
//
// Per thread, step t of the march over planes updates the F cells of plane
// t+1 (offsets e and e+2 of its group) and the S cells of plane t (the same
// offsets: the colour pattern flips with the plane). Values a thread uses at
// two consecutive steps stay in registers: x of plane t+1 at its own group
// (loaded as the front neighbour one step earlier), x of plane t at the
// pair, the front coefficients of plane t, and the second-colour rows of
// plane t (PairRows, picked while the same plane's first colour was
// updated). Shared memory is read only for in-plane neighbours and for the
// newly arrived planes. Neighbour products are summed in the order left,
// right, down, up, back, front.
template <bool ZERO, typename E, int D, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB)
    k_rb_sweep_tma(const __grid_constant__ CUtensorMap tm_x,
                   const __grid_constant__ CUtensorMap tm_r,
                   const __grid_constant__ CUtensorMap tm_b,
                   float* __restrict__ xout, Dims n, int first, float omega,
                   int tiles_x, int tiles, int seg_len, long items,
                   double* err) {
    using Lt = Layout<E, D>;
    using El = Elem<E>;
    constexpr int XR = Lt::XR, AR = Lt::AR;
    constexpr int RW = Lt::RW;
    constexpr int RC = RH * RW;
    constexpr int H = El::H;
    extern __shared__ unsigned char smem_raw[];
    unsigned char* base = reinterpret_cast<unsigned char*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    uint64_t* barx = reinterpret_cast<uint64_t*>(base + Lt::BAR_OFF);
    uint64_t* barr = barx + XR;
    float* yfb = reinterpret_cast<float*>(base + Lt::YF_OFF);

    // Thread -> (row, group), row-major: a warp reads contiguous shared
    // memory (the staged row pitch is exactly G groups).
    const int tid = threadIdx.x;
    const bool worker = tid < NF;
    const int ry = worker ? tid / G : 0;  // row j0 - 1 + ry
    const int gq = worker ? tid - ry * G : 0;
    const bool tile_thr =
        worker && ry >= 1 && ry <= TY && gq >= 1 && gq <= G - 2;
    const int xo = (ry + 1) * XW + 4 * gq;            // x: row j in the box
    const int bo = ry * XW + 4 * gq;                  // b and F buffer
    const int ro = (ry + 1) * RW + 4 * gq + (H - 4);  // rows: row j
    const float w1 = 1.0f - omega;

    if (tid == 0) {
        for (int s = 0; s < XR + AR; ++s) tc::mbar_init(&barx[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();

    const int sz = n.x * n.y;  // levels hold < 2^31 cells
    // Issue side (thread 0) and wait side (every thread) of each ring, and
    // the number of copies thread 0 has issued into each.
    Ring ix, ir, wx, wr;
    unsigned nix = 0, nir = 0;
    bool bad = false;
    // Work items are column segments of seg_len planes, numbered segment
    // by segment (item = segment * tiles + tile): a block takes items
    // blockIdx.x, + gridDim.x, ...; the resident blocks then hold
    // neighbouring tiles of the same segment and march through it together.
    for (long it = blockIdx.x; it < items; it += gridDim.x) {
        const int tile = (int)(it % tiles);
        const int k0 = (int)(it / tiles) * seg_len;
        const int k1 = min(n.z, k0 + seg_len);
        const int i0 = (tile % tiles_x) * TX;
        const int j0 = (tile / tiles_x) * TY;
        const int gi = i0 - 4 + 4 * gq;  // first cell of the group
        const int gj = j0 - 1 + ry;
        const bool gv = worker && gi >= 0 && gi < n.x && gj >= 0 && gj < n.y;
        // Steps t0 .. k1-1; x of planes t0 .. k1+1 and rows + b of planes
        // t0 .. k1 are staged, each once.
        const int t0 = k0 - 2;
        auto issue_x = [&](int p) {
            uint64_t* bar = &barx[ix.slot];
            expect_tx(bar, Lt::X_BYTES);
            tma3(base + Lt::X_OFF + ix.slot * Lt::X_STEP, &tm_x, i0 - 4,
                 j0 - 2, p, bar);
            ix.advance<XR>();
            ++nix;
        };
        auto issue_r = [&](int p) {
            uint64_t* bar = &barr[ir.slot];
            expect_tx(bar, Lt::R_BYTES + Lt::B_BYTES);
            tma4(base + Lt::R_OFF + ir.slot * Lt::R_STEP, &tm_r, i0 - H,
                 j0 - 2, p, 0, bar);
            tma3(base + Lt::B_OFF + ir.slot * Lt::B_STEP, &tm_b, i0 - 4,
                 j0 - 1, p, bar);
            ir.advance<AR>();
            ++nir;
        };
        // Waits for the next staged plane of a ring and returns its slot;
        // after one timeout, waits no more.
        auto wait_x = [&]() {
            const int s = wx.slot;
            if (!bad && !tc::mbar_wait(&barx[s], wx.phase)) bad = true;
            wx.advance<XR>();
            return s;
        };
        auto wait_r = [&]() {
            const int s = wr.slot;
            if (!bad && !tc::mbar_wait(&barr[s], wr.phase)) bad = true;
            wr.advance<AR>();
            return s;
        };
        auto xs = [&](int slot) {
            return reinterpret_cast<const float*>(base + Lt::X_OFF +
                                                  slot * Lt::X_STEP) + xo;
        };
        auto rs = [&](int slot) {
            return reinterpret_cast<const E*>(base + Lt::R_OFF +
                                              slot * Lt::R_STEP) + ro;
        };
        auto bs = [&](int slot) {
            return reinterpret_cast<const float*>(base + Lt::B_OFF +
                                                  slot * Lt::B_STEP) + bo;
        };

        __syncthreads();  // the previous run's reads of every ring are done
        if (tid == 0) {
            if (!ZERO)
                for (int p = t0; p <= min(k1 + 1, t0 + 1 + D); ++p) issue_x(p);
            for (int p = t0; p <= min(k1, t0 + D); ++p) issue_r(p);
        }
        // Prologue: x of planes t0 and t0+1 at the own group and the front
        // coefficients of plane t0 into registers.
        float4 xc = make_float4(0.f, 0.f, 0.f, 0.f);  // x(t+1), own group
        float4 xp = xc;                                // x(t), own group
        int sx1 = 0;                                   // slot of x(t+1)
        if (!ZERO) {
            const int s0 = wait_x();
            sx1 = wait_x();
            xp = lds4(xs(s0));
            xc = lds4(xs(sx1));
        }
        float4 ffp = El::ld4(rs(wait_r()) + 3 * RC);  // front coeff. of t
        // Pair of the first step (offsets of plane t0+1's first colour).
        const int e0 = (first + gj + t0 + 1) & 1;
        float xbA = sel(e0, xp.x, xp.y), xbB = sel(e0, xp.z, xp.w);
        PairRows sp{};  // second-colour rows of plane t (set one step ahead)
        float2 fm = make_float2(0.f, 0.f);  // own F results of plane t-1
        float2 f0 = make_float2(0.f, 0.f);  // own F results of plane t
        for (int t = t0; t < k1; ++t) {
            __syncthreads();  // step t-1 is done: its ring slots are free
            if (tid == 0) {
                if (!ZERO && t + 2 + D <= k1 + 1) issue_x(t + 2 + D);
                if (t + 1 + D <= k1) issue_r(t + 1 + D);
            }
            const int sx2 = ZERO ? 0 : wait_x();
            const int sr1 = wait_r();

            // (1) F cells of plane t+1 (offsets e and e+2 of the group).
            const int p1 = t + 1;
            const int e = (first + gj + p1) & 1;
            const E* R1 = rs(sr1);
            const float4 cc = El::ld4(R1);
            const float4 rr = El::ld4(R1 + RC);
            const float rl = El::ld1(R1 + RC - 1);
            const float4 uu = El::ld4(R1 + 2 * RC);
            const float4 ud = El::ld4(R1 + 2 * RC - RW);
            const float4 ff = El::ld4(R1 + 3 * RC);
            const float4 bb = lds4(bs(sr1));
            float4 xf = make_float4(0.f, 0.f, 0.f, 0.f);  // x(t+2), own group
            float2 f1 = make_float2(0.f, 0.f);
            if (!ZERO) xf = lds4(xs(sx2));
            if (gv && p1 >= 0 && p1 < n.z) {
                const float cA = sel(e, cc.x, cc.y), cB = sel(e, cc.z, cc.w);
                const float bA = sel(e, bb.x, bb.y), bB = sel(e, bb.z, bb.w);
                if (ZERO) {
                    f1 = make_float2(omega * __fdividef(bA, cA),
                                     omega * __fdividef(bB, cB));
                } else {
                    const float* X1 = xs(sx1);
                    const float xl = X1[-1], xr = X1[4];
                    const float4 xd = lds4(X1 - XW), xu = lds4(X1 + XW);
                    const float accA = sel(e, rl, rr.x) * sel(e, xl, xc.x) +
                                       sel(e, rr.x, rr.y) * sel(e, xc.y, xc.z) +
                                       sel(e, ud.x, ud.y) * sel(e, xd.x, xd.y) +
                                       sel(e, uu.x, uu.y) * sel(e, xu.x, xu.y) +
                                       sel(e, ffp.x, ffp.y) * xbA +
                                       sel(e, ff.x, ff.y) * sel(e, xf.x, xf.y);
                    const float accB = sel(e, rr.y, rr.z) * sel(e, xc.y, xc.z) +
                                       sel(e, rr.z, rr.w) * sel(e, xc.w, xr) +
                                       sel(e, ud.z, ud.w) * sel(e, xd.z, xd.w) +
                                       sel(e, uu.z, uu.w) * sel(e, xu.z, xu.w) +
                                       sel(e, ffp.z, ffp.w) * xbB +
                                       sel(e, ff.z, ff.w) * sel(e, xf.z, xf.w);
                    f1 = make_float2(
                        w1 * sel(e, xc.x, xc.y) + omega * __fdividef(bA - accA, cA),
                        w1 * sel(e, xc.z, xc.w) + omega * __fdividef(bB - accB, cB));
                }
            }
            if (worker) {
                float4 o;
                o.x = e ? 0.f : f1.x;
                o.y = e ? f1.x : 0.f;
                o.z = e ? 0.f : f1.y;
                o.w = e ? f1.y : 0.f;
                *reinterpret_cast<float4*>(yfb + (p1 & 1) * FR * XW + bo) = o;
            }

            // (2) S cells of plane t: the same offsets e, e+2.
            if (tile_thr && gv && t >= k0) {
                const float* Y = yfb + (t & 1) * FR * XW + bo;
                const float4 yc = lds4(Y);
                const float yl = Y[-1], yr = Y[4];
                const float4 yd = lds4(Y - XW), yu = lds4(Y + XW);
                const float accA = sp.l[0] * sel(e, yl, yc.x) +
                                   sp.r[0] * sel(e, yc.y, yc.z) +
                                   sp.d[0] * sel(e, yd.x, yd.y) +
                                   sp.u[0] * sel(e, yu.x, yu.y) +
                                   sp.k[0] * fm.x + sp.f[0] * f1.x;
                const float accB = sp.l[1] * sel(e, yc.y, yc.z) +
                                   sp.r[1] * sel(e, yc.w, yr) +
                                   sp.d[1] * sel(e, yd.z, yd.w) +
                                   sp.u[1] * sel(e, yu.z, yu.w) +
                                   sp.k[1] * fm.y + sp.f[1] * f1.y;
                const float xA = ZERO ? 0.f : xbA, xB = ZERO ? 0.f : xbB;
                const float2 sv = make_float2(
                    w1 * xA + omega * __fdividef(sp.b[0] - accA, sp.c[0]),
                    w1 * xB + omega * __fdividef(sp.b[1] - accB, sp.c[1]));
                float4 o;  // F of plane t sits at offsets 1-e and 3-e
                o.x = e ? f0.x : sv.x;
                o.y = e ? sv.x : f0.x;
                o.z = e ? f0.y : sv.y;
                o.w = e ? sv.y : f0.y;
                *reinterpret_cast<float4*>(xout + ((size_t)sz * t + gi +
                                                   (size_t)n.x * gj)) = o;
            }

            // Carry plane t+1 to the next step: its second-colour cells are
            // the offsets s = 1-e.
            const int s = 1 - e;
            sp.c[0] = sel(s, cc.x, cc.y);
            sp.c[1] = sel(s, cc.z, cc.w);
            sp.l[0] = sel(s, rl, rr.x);
            sp.r[0] = sel(s, rr.x, rr.y);
            sp.l[1] = sel(s, rr.y, rr.z);
            sp.r[1] = sel(s, rr.z, rr.w);
            sp.d[0] = sel(s, ud.x, ud.y);
            sp.d[1] = sel(s, ud.z, ud.w);
            sp.u[0] = sel(s, uu.x, uu.y);
            sp.u[1] = sel(s, uu.z, uu.w);
            sp.f[0] = sel(s, ff.x, ff.y);
            sp.f[1] = sel(s, ff.z, ff.w);
            sp.k[0] = sel(s, ffp.x, ffp.y);
            sp.k[1] = sel(s, ffp.z, ffp.w);
            sp.b[0] = sel(s, bb.x, bb.y);
            sp.b[1] = sel(s, bb.z, bb.w);
            xbA = sel(s, xc.x, xc.y);
            xbB = sel(s, xc.z, xc.w);
            xc = xf;
            ffp = ff;
            sx1 = sx2;
            fm = f0;
            f0 = f1;
        }
    }
    if (bad) {
        err[0] = 1.0;
        // Let every copy this block issued land before the block exits: the
        // last XR (AR) copies of a ring are the only ones that can still be
        // in flight; wait (bounded) for the latest phase of each.
        if (tid == 0) {
            for (unsigned q = nix > (unsigned)XR ? nix - XR : 0u; q < nix; ++q)
                tc::mbar_wait(&barx[q % XR], (q / XR) & 1u);
            for (unsigned q = nir > (unsigned)AR ? nir - AR : 0u; q < nir; ++q)
                tc::mbar_wait(&barr[q % AR], (q / AR) & 1u);
        }
    }
}

}  // namespace tsw
}  // namespace jg

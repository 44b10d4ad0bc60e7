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
// depths: a step t reads x of planes t..t+2 and stages x of t+2+D; rows of
// t-1..t+1 and b of t..t+1, staging both of t+1+D.
template <typename E, int D>
struct Layout {
    static constexpr int XR = D + 3, AR = D + 3, BR = D + 2;
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
    static constexpr int YF_OFF = B_OFF + BR * B_STEP;
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
__device__ __forceinline__ float sel(int e, float a, float b) {
    return e ? b : a;
}

// F update of the two cells at offsets e and e+2 of the group (e = 0 or 1,
// per thread) of plane t+1. X0, X1, X2: x of planes t, t+1, t+2 at the
// group; R1 / R0: rows of planes t+1 / t at the group; B1: b of plane t+1.
// Neighbour products are summed in the order left, right, down, up, back,
// front.
template <bool ZERO, typename E>
__device__ __forceinline__ float2 f_cells(int e, const float* X0,
                                          const float* X1, const float* X2,
                                          const E* R1, const E* R0,
                                          const float* B1, float omega) {
    using El = Elem<E>;
    constexpr int RW = TX + 2 * El::H;
    constexpr int RC = RH * RW;
    const float4 cc = El::ld4(R1);
    const float4 bb = lds4(B1);
    const float cA = sel(e, cc.x, cc.y), cB = sel(e, cc.z, cc.w);
    const float bA = sel(e, bb.x, bb.y), bB = sel(e, bb.z, bb.w);
    if (ZERO)
        return make_float2(omega * __fdividef(bA, cA),
                           omega * __fdividef(bB, cB));
    const float4 xc = lds4(X1);
    const float xl = X1[-1], xr = X1[4];
    const float4 xd = lds4(X1 - XW), xu = lds4(X1 + XW);
    const float4 xb = lds4(X0), xf = lds4(X2);
    const float4 rr = El::ld4(R1 + RC);
    const float rl = El::ld1(R1 + RC - 1);
    const float4 uu = El::ld4(R1 + 2 * RC);
    const float4 ud = El::ld4(R1 + 2 * RC - RW);
    const float4 ff = El::ld4(R1 + 3 * RC);
    const float4 fb = El::ld4(R0 + 3 * RC);
    const float accA = sel(e, rl, rr.x) * sel(e, xl, xc.x) +
                       sel(e, rr.x, rr.y) * sel(e, xc.y, xc.z) +
                       sel(e, ud.x, ud.y) * sel(e, xd.x, xd.y) +
                       sel(e, uu.x, uu.y) * sel(e, xu.x, xu.y) +
                       sel(e, fb.x, fb.y) * sel(e, xb.x, xb.y) +
                       sel(e, ff.x, ff.y) * sel(e, xf.x, xf.y);
    const float accB = sel(e, rr.y, rr.z) * sel(e, xc.y, xc.z) +
                       sel(e, rr.z, rr.w) * sel(e, xc.w, xr) +
                       sel(e, ud.z, ud.w) * sel(e, xd.z, xd.w) +
                       sel(e, uu.z, uu.w) * sel(e, xu.z, xu.w) +
                       sel(e, fb.z, fb.w) * sel(e, xb.z, xb.w) +
                       sel(e, ff.z, ff.w) * sel(e, xf.z, xf.w);
    return make_float2(
        (1.0f - omega) * sel(e, xc.x, xc.y) + omega * __fdividef(bA - accA, cA),
        (1.0f - omega) * sel(e, xc.z, xc.w) + omega * __fdividef(bB - accB, cB));
}

// S update of the two cells at offsets e and e+2 of plane t. Y: new F values
// of plane t at the group (shared buffer); fm / fp: own F values of planes
// t-1 / t+1 at the same cells; R0 / Rm: rows of planes t / t-1; B0: b of
// plane t; X0: old x of plane t.
template <bool ZERO, typename E>
__device__ __forceinline__ float2 s_cells(int e, const float* Y, float2 fm,
                                          float2 fp, const E* R0, const E* Rm,
                                          const float* B0, const float* X0,
                                          float omega) {
    using El = Elem<E>;
    constexpr int RW = TX + 2 * El::H;
    constexpr int RC = RH * RW;
    const float4 yc = lds4(Y);
    const float yl = Y[-1], yr = Y[4];
    const float4 yd = lds4(Y - XW), yu = lds4(Y + XW);
    const float4 cc = El::ld4(R0);
    const float4 rr = El::ld4(R0 + RC);
    const float rl = El::ld1(R0 + RC - 1);
    const float4 uu = El::ld4(R0 + 2 * RC);
    const float4 ud = El::ld4(R0 + 2 * RC - RW);
    const float4 ff = El::ld4(R0 + 3 * RC);
    const float4 fb = El::ld4(Rm + 3 * RC);
    const float4 bb = lds4(B0);
    float xA = 0.f, xB = 0.f;
    if (!ZERO) {
        const float4 xc = lds4(X0);
        xA = sel(e, xc.x, xc.y);
        xB = sel(e, xc.z, xc.w);
    }
    const float accA = sel(e, rl, rr.x) * sel(e, yl, yc.x) +
                       sel(e, rr.x, rr.y) * sel(e, yc.y, yc.z) +
                       sel(e, ud.x, ud.y) * sel(e, yd.x, yd.y) +
                       sel(e, uu.x, uu.y) * sel(e, yu.x, yu.y) +
                       sel(e, fb.x, fb.y) * fm.x + sel(e, ff.x, ff.y) * fp.x;
    const float accB = sel(e, rr.y, rr.z) * sel(e, yc.y, yc.z) +
                       sel(e, rr.z, rr.w) * sel(e, yc.w, yr) +
                       sel(e, ud.z, ud.w) * sel(e, yd.z, yd.w) +
                       sel(e, uu.z, uu.w) * sel(e, yu.z, yu.w) +
                       sel(e, fb.z, fb.w) * fm.y + sel(e, ff.z, ff.w) * fp.y;
    return make_float2((1.0f - omega) * xA +
                           omega * __fdividef(sel(e, bb.x, bb.y) - accA,
                                              sel(e, cc.x, cc.y)),
                       (1.0f - omega) * xB +
                           omega * __fdividef(sel(e, bb.z, bb.w) - accB,
                                              sel(e, cc.z, cc.w)));
}

// ZERO: the sweep starts from x = 0 (no x is staged). tm_x covers xin
// (nx, ny, nz) FP32, box (XW, XH); tm_r the rows (nx, ny, nz, 4) of E, box
// (RW, RH, 1, 4); tm_b covers b, box (XW, BH). `err` (a device scalar) is set
// to 1 when a copy did not arrive within the wait limit; the kernel then
// stops waiting, finishes its loop on whatever the rings hold, and before it
// exits waits (bounded) for the copies it issued.
template <bool ZERO, typename E, int D>
__global__ void __launch_bounds__(BLOCK, 1)
    k_rb_sweep_tma(const __grid_constant__ CUtensorMap tm_x,
                   const __grid_constant__ CUtensorMap tm_r,
                   const __grid_constant__ CUtensorMap tm_b,
                   float* __restrict__ xout, Dims n, int first, float omega,
                   int tiles_x, long total, long per_block, double* err) {
    using Lt = Layout<E, D>;
    using El = Elem<E>;
    constexpr int XR = Lt::XR, AR = Lt::AR, BR = Lt::BR;
    constexpr int RW = Lt::RW;
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

    if (tid == 0) {
        for (int s = 0; s < XR + AR; ++s) tc::mbar_init(&barx[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();

    const int sz = n.x * n.y;  // levels hold < 2^31 cells
    unsigned seq = 0;          // copies of each kind this block has issued
    bool bad = false;
    long w = (long)blockIdx.x * per_block;
    const long wend = min(total, w + per_block);
    while (w < wend) {
        const int tile = (int)(w / n.z);
        const int k0 = (int)(w - (long)tile * n.z);
        const int k1 = (int)min((long)n.z, k0 + (wend - w));
        w += k1 - k0;
        const int i0 = (tile % tiles_x) * TX;
        const int j0 = (tile / tiles_x) * TY;
        const int gi = i0 - 4 + 4 * gq;  // first cell of the group
        const int gj = j0 - 1 + ry;
        const bool gv = worker && gi >= 0 && gi < n.x && gj >= 0 && gj < n.y;
        // Steps t0 .. k1-1; x of planes t0 .. k1+1 and rows + b of planes
        // t0-1 .. k1 are staged, the same count of each.
        const int t0 = k0 - 2;
        auto qx = [&](int p) { return seq + (unsigned)(p - t0); };
        auto qr = [&](int p) { return seq + (unsigned)(p - t0 + 1); };
        auto xs = [&](int p) {
            return reinterpret_cast<const float*>(
                       base + Lt::X_OFF + (qx(p) % XR) * Lt::X_STEP) + xo;
        };
        auto rs = [&](int p) {
            return reinterpret_cast<const E*>(
                       base + Lt::R_OFF + (qr(p) % AR) * Lt::R_STEP) + ro;
        };
        auto bs = [&](int p) {
            return reinterpret_cast<const float*>(
                       base + Lt::B_OFF + (qr(p) % BR) * Lt::B_STEP) + bo;
        };
        auto issue_x = [&](int p) {
            const unsigned q = qx(p);
            uint64_t* bar = &barx[q % XR];
            expect_tx(bar, Lt::X_BYTES);
            tma3(base + Lt::X_OFF + (q % XR) * Lt::X_STEP, &tm_x, i0 - 4,
                 j0 - 2, p, bar);
        };
        auto issue_r = [&](int p) {
            const unsigned q = qr(p);
            uint64_t* bar = &barr[q % AR];
            expect_tx(bar, Lt::R_BYTES + Lt::B_BYTES);
            tma4(base + Lt::R_OFF + (q % AR) * Lt::R_STEP, &tm_r, i0 - H,
                 j0 - 2, p, 0, bar);
            tma3(base + Lt::B_OFF + (q % BR) * Lt::B_STEP, &tm_b, i0 - 4,
                 j0 - 1, p, bar);
        };
        auto wait_x = [&](int p) {  // after one timeout, wait no more
            const unsigned q = qx(p);
            if (!ZERO && !bad && !tc::mbar_wait(&barx[q % XR], (q / XR) & 1u))
                bad = true;
        };
        auto wait_r = [&](int p) {
            const unsigned q = qr(p);
            if (!bad && !tc::mbar_wait(&barr[q % AR], (q / AR) & 1u))
                bad = true;
        };

        __syncthreads();  // the previous run's reads of every ring are done
        if (tid == 0) {
            for (int p = t0; p <= min(k1 + 1, t0 + 1 + D); ++p)
                if (!ZERO) issue_x(p);
            for (int p = t0 - 1; p <= min(k1, t0 + D); ++p) issue_r(p);
        }
        wait_x(t0);
        wait_x(t0 + 1);
        wait_r(t0 - 1);
        wait_r(t0);

        float2 fm = make_float2(0.f, 0.f);  // own F results of plane t-1
        float2 f0 = make_float2(0.f, 0.f);  // own F results of plane t
        for (int t = t0; t < k1; ++t) {
            __syncthreads();  // step t-1 is done: its ring slots are free
            if (tid == 0) {
                if (!ZERO && t + 2 + D <= k1 + 1) issue_x(t + 2 + D);
                if (t + 1 + D <= k1) issue_r(t + 1 + D);
            }
            wait_x(t + 2);
            wait_r(t + 1);

            // (1) F cells of plane t+1 (offsets e and e+2 of the group).
            const int p1 = t + 1;
            const int e = (first + gj + p1) & 1;
            float2 f1 = make_float2(0.f, 0.f);
            if (gv && p1 >= 0 && p1 < n.z) {
                const float* X0 = ZERO ? nullptr : xs(t);
                const float* X1 = ZERO ? nullptr : xs(t + 1);
                const float* X2 = ZERO ? nullptr : xs(t + 2);
                f1 = f_cells<ZERO, E>(e, X0, X1, X2, rs(t + 1), rs(t),
                                      bs(t + 1), omega);
            }
            if (worker) {
                float4 o;
                o.x = e ? 0.f : f1.x;
                o.y = e ? f1.x : 0.f;
                o.z = e ? 0.f : f1.y;
                o.w = e ? f1.y : 0.f;
                *reinterpret_cast<float4*>(yfb + (p1 & 1) * FR * XW + bo) = o;
            }

            // (2) S cells of plane t (the offsets of F in planes t+-1).
            if (tile_thr && gv && t >= k0) {
                const float* Y = yfb + (t & 1) * FR * XW + bo;
                const float* X0 = ZERO ? nullptr : xs(t);
                const float2 sv = s_cells<ZERO, E>(e, Y, fm, f1, rs(t),
                                                   rs(t - 1), bs(t), X0, omega);
                float4 o;  // F of plane t sits at offsets 1-e and 3-e
                o.x = e ? f0.x : sv.x;
                o.y = e ? sv.x : f0.x;
                o.z = e ? f0.y : sv.y;
                o.w = e ? sv.y : f0.y;
                *reinterpret_cast<float4*>(xout + ((size_t)sz * t + gi +
                                                   (size_t)n.x * gj)) = o;
            }
            fm = f0;
            f0 = f1;
        }
        seq += (unsigned)(k1 - t0 + 2);
    }
    if (bad) {
        err[0] = 1.0;
        // Let every copy this block issued land before the block exits.
        if (tid == 0) {
            for (unsigned q = seq > (unsigned)XR ? seq - XR : 0u; q < seq; ++q)
                if (!ZERO) tc::mbar_wait(&barx[q % XR], (q / XR) & 1u);
            for (unsigned q = seq > (unsigned)AR ? seq - AR : 0u; q < seq; ++q)
                tc::mbar_wait(&barr[q % AR], (q / AR) & 1u);
        }
    }
}

}  // namespace tsw
}  // namespace jg

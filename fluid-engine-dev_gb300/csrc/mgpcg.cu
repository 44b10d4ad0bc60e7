// Multigrid-preconditioned CG on GB300 (K5-K11).
//
// Replaces FdmMgpcgSolver3::solve (src/jet/fdm_mgpcg_solver3.cpp:54-80), the
// generic pcg (include/jet/detail/cg-inl.h:15-94) and mgVCycle
// (include/jet/detail/mg-inl.h:16-68) with red-black SOR smoothing
// (src/jet/fdm_gauss_seidel_solver3.cpp:150-221) and the FdmMgUtils3
// transfer operators (src/jet/fdm_mg_linear_system3.cpp:43-179).
//
// Design (GB300-first):
//   * Krylov vectors FP32 (or FP64), matrix rows as one aligned float4 per
//     cell, V-cycle in FP32; every global reduction is FP64-accurate and
//     deterministic (fixed grid, per-block partials summed in FP64 in block
//     order by the last block to finish; no block ever waits on another).
//     Over FP32 vectors each thread accumulates its products exactly split
//     into a double-float pair on the FP32 pipe (common.cuh, DF): GB300
//     issues FP64 at a small fraction of the FP32 rate, and a per-element
//     FP64 multiply-add made these streaming kernels FP64-issue-bound.
//   * alpha and beta never leave the device: the last block of each reduction
//     computes them, the next kernel reads them. The host reads one scalar per
//     iteration (the residual norm) for the stopping test.
//   * FP32 modes reach the FP64 tolerance by iterative refinement: the FP64
//     residual b - A x is evaluated with the exact FP64 matrix the reference
//     builds, the FP32 PCG solves for a correction, and x accumulates in FP64.
//   * The V-cycle is symmetric (post-smoothing sweeps the colours in reverse
//     order, restriction is 1/8 of the prolongation's transpose — true of the
//     reference's operators including their clamped boundaries) and starts
//     from zero, so it is a fixed SPD preconditioner for CG.

#include "ctx.h"
#include "sweep_tma.cuh"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

namespace jg {
namespace {

enum Fin : int { FIN_NONE = 0, FIN_BETA = 1, FIN_ALPHA = 2 };
enum : int { S_ALPHA = 8, S_BETA = 9, S_FIRST = 10 };
// Device-side PCG loop: target residual norm, iteration cap, iterations run.
enum : int { S_LOOP_TARGET = 11, S_LOOP_MAX = 12, S_LOOP_IT = 13 };

// Finishes a reduction: stores the total and derives alpha/beta.
__device__ __forceinline__ void finish(double* scal, int target, double v,
                                       int fin) {
    scal[target] = v;
    if (fin == FIN_BETA) {
        const double old = scal[S_RZ_OLD];
        scal[S_BETA] = (scal[S_FIRST] != 0.0 || old == 0.0) ? 0.0 : v / old;
        scal[S_RZ_OLD] = v;
        scal[S_FIRST] = 0.0;
    } else if (fin == FIN_ALPHA) {
        scal[S_ALPHA] = scal[S_RZ] / v;
    }
}

template <int NT>
__device__ __forceinline__ void reduce_finish(double partial, int slot,
                                              int target, int fin,
                                              double* partials,
                                              unsigned* counters,
                                              double* scal, double* smem) {
    __shared__ bool is_last;
    double bs = block_sum<NT>(partial, smem);
    if (threadIdx.x == 0) {
        partials[slot * kMaxRedBlocks + blockIdx.x] = bs;
        __threadfence();
        const unsigned done = atomicAdd(&counters[slot], 1u);
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
            finish(scal, target, v, fin);
            counters[slot] = 0u;
        }
    }
}

// ---------------------------------------------------------------------------
// Matrix access: FP32 rows (float4) or the exact FP64 rows (4 doubles).

// Rows of one level as a structure of arrays (center, right, up, front
// planes of N values).
struct RowsF {
    const float* A;
    long N;
    __device__ __forceinline__ float4 row(long c) const {
        return make_float4(__ldg(A + c), __ldg(A + N + c), __ldg(A + 2 * N + c),
                           __ldg(A + 3 * N + c));
    }
    // Component p of cells c..c+3 (c and N multiples of 4).
    __device__ __forceinline__ float4 quad(int p, long c) const {
        return __ldg(reinterpret_cast<const float4*>(A + p * N + c));
    }
    __device__ __forceinline__ float one(int p, long c) const {
        return __ldg(A + p * N + c);
    }
};
// BF16 rows (mixed mode), same layout.
__device__ __forceinline__ float bf_dec(unsigned short u) {
    return __uint_as_float((unsigned)u << 16);
}
struct RowsB {
    const unsigned short* A;
    long N;
    __device__ __forceinline__ float4 row(long c) const {
        return make_float4(bf_dec(__ldg(A + c)), bf_dec(__ldg(A + N + c)),
                           bf_dec(__ldg(A + 2 * N + c)),
                           bf_dec(__ldg(A + 3 * N + c)));
    }
    __device__ __forceinline__ float4 quad(int p, long c) const {
        const uint2 w = __ldg(reinterpret_cast<const uint2*>(A + p * N + c));
        return make_float4(__uint_as_float(w.x << 16),
                           __uint_as_float(w.x & 0xffff0000u),
                           __uint_as_float(w.y << 16),
                           __uint_as_float(w.y & 0xffff0000u));
    }
    __device__ __forceinline__ float one(int p, long c) const {
        return bf_dec(__ldg(A + p * N + c));
    }
};
struct RowsD {
    const double* A;
    __device__ __forceinline__ double4_16a row(long c) const {
        const double2 a = reinterpret_cast<const double2*>(A)[2 * c];
        const double2 b = reinterpret_cast<const double2*>(A)[2 * c + 1];
        return make_double4_16a(a.x, a.y, b.x, b.y);
    }
};

// 7-point symmetric apply at cell c (FdmBlas3::mvm, fdm_linear_system3.cpp:79-96).
template <typename T, typename Rows, typename V>
__device__ __forceinline__ T apply7(const Rows& M, const V* __restrict__ v,
                                    long c, int i, int j, int k, Dims n) {
    const long sy = n.x, sz = (long)n.x * n.y;
    const auto r = M.row(c);
    T s = (T)r.x * (T)v[c];
    if (i > 0) s += (T)M.row(c - 1).y * (T)v[c - 1];
    if (i + 1 < n.x) s += (T)r.y * (T)v[c + 1];
    if (j > 0) s += (T)M.row(c - sy).z * (T)v[c - sy];
    if (j + 1 < n.y) s += (T)r.z * (T)v[c + sy];
    if (k > 0) s += (T)M.row(c - sz).w * (T)v[c - sz];
    if (k + 1 < n.z) s += (T)r.w * (T)v[c + sz];
    return s;
}

__device__ __forceinline__ float4 ld4(const float* p) {
    return *reinterpret_cast<const float4*>(p);
}

// apply7 for the four cells c..c+3 of a row (c and n.x multiples of 4) from
// 16-byte loads: each cell's terms in apply7's order.
template <typename R>
__device__ __forceinline__ void apply7x4(const R& M,
                                         const float* __restrict__ v, long c,
                                         int i, int j, int k, Dims n,
                                         float out[4]) {
    const long sy = n.x, sz = (long)n.x * n.y;
    const float4 cx = M.quad(0, c), cy = M.quad(1, c), cz = M.quad(2, c),
                 cw = M.quad(3, c);
    const float4 vc = ld4(v + c);
    const bool hl = i > 0, hr = i + 4 < n.x, hd = j > 0, hu = j + 1 < n.y,
               hb = k > 0, hf = k + 1 < n.z;
    const float vl = hl ? v[c - 1] : 0.0f, yl = hl ? M.one(1, c - 1) : 0.0f;
    const float vr = hr ? v[c + 4] : 0.0f;
    const float4 z4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const float4 vd = hd ? ld4(v + c - sy) : z4, zd = hd ? M.quad(2, c - sy) : z4;
    const float4 vu = hu ? ld4(v + c + sy) : z4;
    const float4 vb = hb ? ld4(v + c - sz) : z4, wb = hb ? M.quad(3, c - sz) : z4;
    const float4 vf = hf ? ld4(v + c + sz) : z4;
    const float V[6] = {vl, vc.x, vc.y, vc.z, vc.w, vr};
    const float CX[4] = {cx.x, cx.y, cx.z, cx.w}, CY[4] = {cy.x, cy.y, cy.z, cy.w};
    const float YL[4] = {yl, cy.x, cy.y, cy.z};
    const float CZ[4] = {cz.x, cz.y, cz.z, cz.w}, ZD[4] = {zd.x, zd.y, zd.z, zd.w};
    const float CW[4] = {cw.x, cw.y, cw.z, cw.w}, WB[4] = {wb.x, wb.y, wb.z, wb.w};
    const float VD[4] = {vd.x, vd.y, vd.z, vd.w}, VU[4] = {vu.x, vu.y, vu.z, vu.w};
    const float VB[4] = {vb.x, vb.y, vb.z, vb.w}, VF[4] = {vf.x, vf.y, vf.z, vf.w};
#pragma unroll
    for (int l = 0; l < 4; ++l) {
        float s = CX[l] * V[l + 1];
        if (l > 0 || hl) s += YL[l] * V[l];
        if (l < 3 || hr) s += CY[l] * V[l + 2];
        if (hd) s += ZD[l] * VD[l];
        if (hu) s += CZ[l] * VU[l];
        if (hb) s += WB[l] * VB[l];
        if (hf) s += CW[l] * VF[l];
        out[l] = s;
    }
}

// k_residual32 over 4-cell groups (n.x a multiple of 4).
template <typename R>
__global__ void __launch_bounds__(kThreads)
    k_residual32x4(R M, const float* __restrict__ x,
                   const float* __restrict__ b, float* __restrict__ r, Dims n) {
    const Dims q{n.x / 4, n.y, n.z};
    const long G = q.count();
    for (long t = blockIdx.x * (long)kThreads + threadIdx.x; t < G;
         t += (long)gridDim.x * kThreads) {
        int m, j, k;
        cell_ijk(t, q, m, j, k);
        const long c = lin(4 * m, j, k, n.x, n.y);
        float ax[4];
        apply7x4(M, x, c, 4 * m, j, k, n, ax);
        const float4 bb = ld4(b + c);
        *reinterpret_cast<float4*>(r + c) =
            make_float4(bb.x - ax[0], bb.y - ax[1], bb.z - ax[2], bb.w - ax[3]);
    }
}

// k_spmv_dot<float> over 4-cell groups (n.x a multiple of 4).
template <typename R>
__global__ void __launch_bounds__(kThreads)
    k_spmv_dot4(R M, const float* __restrict__ d, float* __restrict__ q,
                Dims n, double* partials, unsigned* counters, double* scal) {
    __shared__ double smem[32];
    const Dims g{n.x / 4, n.y, n.z};
    const long G = g.count();
    AccF acc;
    for (long t = blockIdx.x * (long)kThreads + threadIdx.x; t < G;
         t += (long)gridDim.x * kThreads) {
        int m, j, k;
        cell_ijk(t, g, m, j, k);
        const long c = lin(4 * m, j, k, n.x, n.y);
        float ad[4];
        apply7x4(M, d, c, 4 * m, j, k, n, ad);
        *reinterpret_cast<float4*>(q + c) = make_float4(ad[0], ad[1], ad[2], ad[3]);
        const float4 dd = ld4(d + c);
        acc.add(dd.x, ad[0]);
        acc.add(dd.y, ad[1]);
        acc.add(dd.z, ad[2]);
        acc.add(dd.w, ad[3]);
    }
    reduce_finish<kThreads>(acc.value(), 0, S_DQ, FIN_ALPHA, partials,
                            counters, scal, smem);
}

// K5: q = A d and d.q (FP64).
template <typename V, typename Rows>
__global__ void __launch_bounds__(kThreads)
    k_spmv_dot(Rows M, const V* __restrict__ d, V* __restrict__ q, Dims n,
               double* partials, unsigned* counters, double* scal) {
    __shared__ double smem[32];
    const long N = n.count();
    typename AccOf<V>::type acc;
    for (long c = blockIdx.x * (long)kThreads + threadIdx.x; c < N;
         c += (long)gridDim.x * kThreads) {
        int i, j, k;
        cell_ijk(c, n, i, j, k);
        const V qv = apply7<V>(M, d, c, i, j, k, n);
        q[c] = qv;
        acc.add(d[c], qv);
    }
    reduce_finish<kThreads>(acc.value(), 0, S_DQ, FIN_ALPHA, partials,
                            counters, scal, smem);
}

// K7a: x += alpha d; r -= alpha q; r.r (FP64). Optionally writes an FP32
// copy of r for the V-cycle (FP64 mode).
template <typename V>
__global__ void __launch_bounds__(kThreads)
    k_update_xr(V* __restrict__ x, V* __restrict__ r, const V* __restrict__ d,
                const V* __restrict__ q, float* __restrict__ r32, long N,
                double* partials, unsigned* counters, double* scal) {
    __shared__ double smem[32];
    const V alpha = (V)scal[S_ALPHA];
    typename AccOf<V>::type acc;
    for (long c = blockIdx.x * (long)kThreads + threadIdx.x; c < N;
         c += (long)gridDim.x * kThreads) {
        x[c] += alpha * d[c];
        const V rv = r[c] - alpha * q[c];
        r[c] = rv;
        if (r32) r32[c] = (float)rv;
        acc.add(rv, rv);
    }
    reduce_finish<kThreads>(acc.value(), 1, S_RR, FIN_NONE, partials,
                            counters, scal, smem);
}

// k_update_xr<float> and k_dot_rz<float, float> over 4-element groups
// (N a multiple of 4): 16-byte accesses, the same reductions.
__global__ void __launch_bounds__(kThreads)
    k_update_xr4(float* __restrict__ x, float* __restrict__ r,
                 const float* __restrict__ d, const float* __restrict__ q,
                 long N, double* partials, unsigned* counters, double* scal) {
    __shared__ double smem[32];
    const float alpha = (float)scal[S_ALPHA];
    AccF acc;
    const long G = N / 4;
    for (long t = blockIdx.x * (long)kThreads + threadIdx.x; t < G;
         t += (long)gridDim.x * kThreads) {
        float4 xv = reinterpret_cast<float4*>(x)[t];
        float4 rv = reinterpret_cast<float4*>(r)[t];
        const float4 dv = reinterpret_cast<const float4*>(d)[t];
        const float4 qv = reinterpret_cast<const float4*>(q)[t];
        xv.x += alpha * dv.x;
        xv.y += alpha * dv.y;
        xv.z += alpha * dv.z;
        xv.w += alpha * dv.w;
        rv.x = rv.x - alpha * qv.x;
        rv.y = rv.y - alpha * qv.y;
        rv.z = rv.z - alpha * qv.z;
        rv.w = rv.w - alpha * qv.w;
        reinterpret_cast<float4*>(x)[t] = xv;
        reinterpret_cast<float4*>(r)[t] = rv;
        acc.add(rv.x, rv.x);
        acc.add(rv.y, rv.y);
        acc.add(rv.z, rv.z);
        acc.add(rv.w, rv.w);
    }
    reduce_finish<kThreads>(acc.value(), 1, S_RR, FIN_NONE, partials,
                            counters, scal, smem);
}

__global__ void __launch_bounds__(kThreads)
    k_dot_rz4(const float* __restrict__ r, const float* __restrict__ z,
              long N, double* partials, unsigned* counters, double* scal) {
    __shared__ double smem[32];
    AccF acc;
    const long G = N / 4;
    for (long t = blockIdx.x * (long)kThreads + threadIdx.x; t < G;
         t += (long)gridDim.x * kThreads) {
        const float4 rv = reinterpret_cast<const float4*>(r)[t];
        const float4 zv = reinterpret_cast<const float4*>(z)[t];
        acc.add(rv.x, zv.x);
        acc.add(rv.y, zv.y);
        acc.add(rv.z, zv.z);
        acc.add(rv.w, zv.w);
    }
    reduce_finish<kThreads>(acc.value(), 2, S_RZ, FIN_BETA, partials,
                            counters, scal, smem);
}

__global__ void __launch_bounds__(kThreads)
    k_update_d4(float* __restrict__ d, const float* __restrict__ z, long N,
                const double* scal) {
    const float beta = (float)scal[S_BETA];
    const long G = N / 4;
    for (long t = blockIdx.x * (long)kThreads + threadIdx.x; t < G;
         t += (long)gridDim.x * kThreads) {
        const float4 zv = reinterpret_cast<const float4*>(z)[t];
        if (beta == 0.0f) {
            reinterpret_cast<float4*>(d)[t] = zv;
        } else {
            const float4 dv = reinterpret_cast<const float4*>(d)[t];
            reinterpret_cast<float4*>(d)[t] =
                make_float4(zv.x + beta * dv.x, zv.y + beta * dv.y,
                            zv.z + beta * dv.z, zv.w + beta * dv.w);
        }
    }
}

// K7b: r.z (FP64), finishing beta.
template <typename V, typename Z>
__global__ void __launch_bounds__(kThreads)
    k_dot_rz(const V* __restrict__ r, const Z* __restrict__ z, long N,
             double* partials, unsigned* counters, double* scal) {
    __shared__ double smem[32];
    typename AccOf<V>::type acc;
    for (long c = blockIdx.x * (long)kThreads + threadIdx.x; c < N;
         c += (long)gridDim.x * kThreads)
        acc.add(r[c], (V)z[c]);
    reduce_finish<kThreads>(acc.value(), 2, S_RZ, FIN_BETA, partials,
                            counters, scal, smem);
}

// K7c: d = z + beta d.
template <typename V, typename Z>
__global__ void __launch_bounds__(kThreads)
    k_update_d(V* __restrict__ d, const Z* __restrict__ z, long N,
               const double* scal) {
    const V beta = (V)scal[S_BETA];
    for (long c = blockIdx.x * (long)kThreads + threadIdx.x; c < N;
         c += (long)gridDim.x * kThreads)
        d[c] = (beta == (V)0) ? (V)z[c] : (V)z[c] + beta * d[c];
}

// K6 (FP64): r64 = b64 - A64 x64 with the exact reference rows
// (FdmBlas3::residual, fdm_linear_system3.cpp:98-116); ||r64||^2; optional
// FP32 copy of r64 and zeroing of the FP32 correction.
__global__ void __launch_bounds__(kThreads)
    k_residual64(const double* __restrict__ A64, const double* __restrict__ x,
                 const double* __restrict__ b, double* __restrict__ r,
                 float* __restrict__ r32, float* __restrict__ zero32, Dims n,
                 double* partials, unsigned* counters, double* scal,
                 int target) {
    __shared__ double smem[32];
    const long N = n.count();
    RowsD M{A64};
    double acc = 0.0;
    for (long c = blockIdx.x * (long)kThreads + threadIdx.x; c < N;
         c += (long)gridDim.x * kThreads) {
        int i, j, k;
        cell_ijk(c, n, i, j, k);
        const double rv = b[c] - apply7<double>(M, x, c, i, j, k, n);
        if (r) r[c] = rv;
        if (r32) r32[c] = (float)rv;
        if (zero32) zero32[c] = 0.0f;
        acc += rv * rv;
    }
    reduce_finish<kThreads>(acc, 3, target, FIN_NONE, partials, counters,
                            scal, smem);
}

// Double-float true residual (FP32 modes): r = b - A x with the exact rows,
// rhs and iterate held as hi + lo FP32 pairs (about 48 significant bits),
// evaluated with exact product splitting and TwoSum on the FP32 pipe. Writes
// the FP32 image of r (the next correction's right-hand side), zeroes the
// FP32 correction and reduces ||r||^2 into scal[target].
__global__ void __launch_bounds__(kThreads)
    k_residual_df(RowsF Ahi, const float4* __restrict__ Alo,
                  const float2* __restrict__ x, const float2* __restrict__ b,
                  float* __restrict__ r32, float* __restrict__ zero32, Dims n,
                  double* partials, unsigned* counters, double* scal,
                  int target) {
    __shared__ double smem[32];
    const long N = n.count();
    const long sy = n.x, sz = (long)n.x * n.y;
    AccF acc;
    for (long c = blockIdx.x * (long)kThreads + threadIdx.x; c < N;
         c += (long)gridDim.x * kThreads) {
        int i, j, k;
        cell_ijk(c, n, i, j, k);
        const float4 h = Ahi.row(c), l = Alo[c];
        const float2 xc = x[c], bc = b[c];
        DF r;
        r.hi = bc.x;
        r.lo = bc.y;
        r = df_sub_prod(r, h.x, l.x, xc.x, xc.y);
        if (i > 0) {
            const float2 xn = x[c - 1];
            r = df_sub_prod(r, Ahi.row(c - 1).y, Alo[c - 1].y, xn.x, xn.y);
        }
        if (i + 1 < n.x) {
            const float2 xn = x[c + 1];
            r = df_sub_prod(r, h.y, l.y, xn.x, xn.y);
        }
        if (j > 0) {
            const float2 xn = x[c - sy];
            r = df_sub_prod(r, Ahi.row(c - sy).z, Alo[c - sy].z, xn.x, xn.y);
        }
        if (j + 1 < n.y) {
            const float2 xn = x[c + sy];
            r = df_sub_prod(r, h.z, l.z, xn.x, xn.y);
        }
        if (k > 0) {
            const float2 xn = x[c - sz];
            r = df_sub_prod(r, Ahi.row(c - sz).w, Alo[c - sz].w, xn.x, xn.y);
        }
        if (k + 1 < n.z) {
            const float2 xn = x[c + sz];
            r = df_sub_prod(r, h.w, l.w, xn.x, xn.y);
        }
        const float rv = __fadd_rn(r.hi, r.lo);
        r32[c] = rv;
        zero32[c] = 0.0f;
        acc.add(rv, rv);
    }
    reduce_finish<kThreads>(acc.value(), 3, target, FIN_NONE, partials,
                            counters, scal, smem);
}

// k_residual_df over 4-cell groups (n.x a multiple of 4): each cell's terms
// in k_residual_df's order, from 16-byte loads of the row components and of
// the double-float iterate and rhs; the low parts of the neighbours' rows are
// read as single components. Capped at 64 registers (four blocks per SM
// instead of three), a few values spilled: slightly faster.
__global__ void __launch_bounds__(kThreads, 4)
    k_residual_df4(RowsF Ahi, const float4* __restrict__ Alo,
                   const float2* __restrict__ x, const float2* __restrict__ b,
                   float* __restrict__ r32, float* __restrict__ zero32, Dims n,
                   double* partials, unsigned* counters, double* scal,
                   int target) {
    __shared__ double smem[32];
    const Dims g{n.x / 4, n.y, n.z};
    const long G = g.count();
    const long sy = n.x, sz = (long)n.x * n.y;
    const float* lo = reinterpret_cast<const float*>(Alo);
    AccF acc;
    for (long t = blockIdx.x * (long)kThreads + threadIdx.x; t < G;
         t += (long)gridDim.x * kThreads) {
        int m, j, k;
        cell_ijk(t, g, m, j, k);
        const int i = 4 * m;
        const long c = lin(i, j, k, n.x, n.y);
        const float4 hx = Ahi.quad(0, c), hy = Ahi.quad(1, c),
                     hz = Ahi.quad(2, c), hw = Ahi.quad(3, c);
        const float HX[4] = {hx.x, hx.y, hx.z, hx.w};
        const float HY[4] = {hy.x, hy.y, hy.z, hy.w};
        const float HZ[4] = {hz.x, hz.y, hz.z, hz.w};
        const float HW[4] = {hw.x, hw.y, hw.z, hw.w};
        const bool hl = i > 0, hr = i + 4 < n.x, hd = j > 0, hu = j + 1 < n.y,
                   hb = k > 0, hf = k + 1 < n.z;
        float4 zd = make_float4(0.f, 0.f, 0.f, 0.f), wb = zd;
        if (hd) zd = Ahi.quad(2, c - sy);
        if (hb) wb = Ahi.quad(3, c - sz);
        const float ZD[4] = {zd.x, zd.y, zd.z, zd.w};
        const float WB[4] = {wb.x, wb.y, wb.z, wb.w};
        const float yl = hl ? Ahi.one(1, c - 1) : 0.0f;
        const float yll = hl ? lo[4 * (c - 1) + 1] : 0.0f;
        float rv[4];
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            const long cc = c + l;
            const float4 L = Alo[cc];
            const float2 xc = x[cc], bc = b[cc];
            DF r;
            r.hi = bc.x;
            r.lo = bc.y;
            r = df_sub_prod(r, HX[l], L.x, xc.x, xc.y);
            if (l > 0 || hl) {
                const float2 xn = x[cc - 1];
                const float nh = l > 0 ? HY[l - 1] : yl;
                const float nl = l > 0 ? lo[4 * (cc - 1) + 1] : yll;
                r = df_sub_prod(r, nh, nl, xn.x, xn.y);
            }
            if (l < 3 || hr) {
                const float2 xn = x[cc + 1];
                r = df_sub_prod(r, HY[l], L.y, xn.x, xn.y);
            }
            if (hd) {
                const float2 xn = x[cc - sy];
                r = df_sub_prod(r, ZD[l], lo[4 * (cc - sy) + 2], xn.x, xn.y);
            }
            if (hu) {
                const float2 xn = x[cc + sy];
                r = df_sub_prod(r, HZ[l], L.z, xn.x, xn.y);
            }
            if (hb) {
                const float2 xn = x[cc - sz];
                r = df_sub_prod(r, WB[l], lo[4 * (cc - sz) + 3], xn.x, xn.y);
            }
            if (hf) {
                const float2 xn = x[cc + sz];
                r = df_sub_prod(r, HW[l], L.w, xn.x, xn.y);
            }
            rv[l] = __fadd_rn(r.hi, r.lo);
        }
        *reinterpret_cast<float4*>(r32 + c) = make_float4(rv[0], rv[1], rv[2], rv[3]);
        *reinterpret_cast<float4*>(zero32 + c) = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int l = 0; l < 4; ++l) acc.add(rv[l], rv[l]);
    }
    reduce_finish<kThreads>(acc.value(), 3, target, FIN_NONE, partials,
                            counters, scal, smem);
}

// Start of the FP32-mode solve from x = 0: r = b (its FP32 image is b's hi
// part, the FP32 rounding of b), correction and iterate zeroed, ||b||^2 from
// the double-float b into scal[S_B64].
__global__ void __launch_bounds__(kThreads)
    k_start_df(const float2* __restrict__ b, float* __restrict__ r32,
               float* __restrict__ zero32, float2* __restrict__ x, long N,
               double* partials, unsigned* counters, double* scal) {
    __shared__ double smem[32];
    AccF acc;
    for (long c = blockIdx.x * (long)kThreads + threadIdx.x; c < N;
         c += (long)gridDim.x * kThreads) {
        const float2 bc = b[c];
        r32[c] = bc.x;
        zero32[c] = 0.0f;
        x[c] = make_float2(0.0f, 0.0f);
        acc.add(bc.x, bc.x);
        acc.add(2.0f * bc.x, bc.y);
    }
    reduce_finish<kThreads>(acc.value(), 4, S_R64, FIN_NONE, partials,
                            counters, scal, smem);
}

// x += e on the double-float iterate.
__global__ void k_accumulate_df(float2* __restrict__ x,
                                const float* __restrict__ e, long N) {
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x) {
        const float2 v = x[c];
        DF a;
        a.hi = v.x;
        a.lo = v.y;
        a = df_add_f(a, e[c]);
        x[c] = make_float2(a.hi, a.lo);
    }
}

// x64 = hi + lo (exact widening on the integer pipe, one FP64 add).
__global__ void k_df_to_f64(const float2* __restrict__ x,
                            double* __restrict__ x64, long N) {
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x) {
        const float2 v = x[c];
        x64[c] = widen_f32(v.x) + widen_f32(v.y);
    }
}


// ||v||^2 (FP64).
__global__ void __launch_bounds__(kThreads)
    k_norm2(const double* __restrict__ v, long N, double* partials,
            unsigned* counters, double* scal, int target) {
    __shared__ double smem[32];
    double acc = 0.0;
    for (long c = blockIdx.x * (long)kThreads + threadIdx.x; c < N;
         c += (long)gridDim.x * kThreads)
        acc += v[c] * v[c];
    reduce_finish<kThreads>(acc, 4, target, FIN_NONE, partials, counters,
                            scal, smem);
}

__global__ void k_init_scalars(double* scal) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        scal[S_RZ] = 0.0;
        scal[S_RZ_OLD] = 0.0;
        scal[S_DQ] = 0.0;
        scal[S_RR] = 0.0;
        scal[S_ALPHA] = 0.0;
        scal[S_BETA] = 0.0;
        scal[S_FIRST] = 1.0;
    }
}

// k_init_scalars plus the device-side loop's target, cap and counter.
__global__ void k_loop_start(double* scal, double target, double max_it) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        scal[S_RZ] = 0.0;
        scal[S_RZ_OLD] = 0.0;
        scal[S_DQ] = 0.0;
        scal[S_RR] = 0.0;
        scal[S_ALPHA] = 0.0;
        scal[S_BETA] = 0.0;
        scal[S_FIRST] = 1.0;
        scal[S_LOOP_TARGET] = target;
        scal[S_LOOP_MAX] = max_it;
        scal[S_LOOP_IT] = 0.0;
    }
}

// End of a device-side PCG iteration: counts it and sets the while node's
// condition — continue while the residual norm is above the target, finite,
// below the iteration cap and no sweep reported a stalled copy. Every
// launch sets the condition, and the cap bounds the loop.
__global__ void k_loop_check(cudaGraphConditionalHandle h, double* scal) {
    const double it = scal[S_LOOP_IT] + 1.0;
    scal[S_LOOP_IT] = it;
    const double rr = scal[S_RR];
    const bool go = it < scal[S_LOOP_MAX] && isfinite(rr) &&
                    !(sqrt(rr) <= scal[S_LOOP_TARGET]) && scal[S_WAIT] == 0.0;
    cudaGraphSetConditional(h, go ? 1u : 0u);
}

template <typename V>
__global__ void k_zero(V* __restrict__ p, long N) {
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x)
        p[c] = (V)0;
}

// ---------------------------------------------------------------------------
// V-cycle kernels (FP32).

// K8: one red-black SOR half-sweep (relaxRedBlack, :150-221). One thread per
// pair of cells along i; `color` 0 updates (i+j+k) even cells. With ZERO the
// whole vector is taken as zero on entry: the updated colour gets
// omega*b/center and the other colour is written 0 (no read of x).
template <bool ZERO, typename R>
__global__ void __launch_bounds__(kThreads)
    k_rb_half(R A, const float* __restrict__ b,
              float* __restrict__ x, Dims n, int color, float omega) {
    const int hx = (n.x + 1) >> 1;
    const long N = (long)hx * n.y * n.z;
    const long sy = n.x, sz = (long)n.x * n.y;
    for (long t = blockIdx.x * (long)kThreads + threadIdx.x; t < N;
         t += (long)gridDim.x * kThreads) {
        const int p = (int)(t % hx);
        const long row = t / hx;
        const int j = (int)(row % n.y);
        const int k = (int)(row / n.y);
        const int off = (j + k + color) & 1;
        const int i = 2 * p + off;
        const long base = lin(2 * p, j, k, n.x, n.y);
        if (ZERO) {
            if (i < n.x) {
                const long c = base + off;
                const float4 r = A.row(c);
                x[c] = omega * b[c] / r.x;
            }
            const int io = 2 * p + (off ^ 1);
            if (io < n.x) x[base + (off ^ 1)] = 0.0f;
        } else {
            if (i >= n.x) continue;
            const long c = base + off;
            const float4 r = A.row(c);
            float s = 0.0f;
            if (i > 0) s += A.row(c - 1).y * x[c - 1];
            if (i + 1 < n.x) s += r.y * x[c + 1];
            if (j > 0) s += A.row(c - sy).z * x[c - sy];
            if (j + 1 < n.y) s += r.z * x[c + sy];
            if (k > 0) s += A.row(c - sz).w * x[c - sz];
            if (k + 1 < n.z) s += r.w * x[c + sz];
            x[c] = (1.0f - omega) * x[c] + omega * (b[c] - s) / r.x;
        }
    }
}

// K9a: r = b - A x (FP32).
template <typename R>
__global__ void __launch_bounds__(kThreads)
    k_residual32(R M, const float* __restrict__ x,
                 const float* __restrict__ b, float* __restrict__ r, Dims n) {
    const long N = n.count();
    for (long c = blockIdx.x * (long)kThreads + threadIdx.x; c < N;
         c += (long)gridDim.x * kThreads) {
        int i, j, k;
        cell_ijk(c, n, i, j, k);
        r[c] = b[c] - apply7<float>(M, x, c, i, j, k, n);
    }
}

// K9b: FdmMgUtils3::restrict (fdm_mg_linear_system3.cpp:43-98): 4x4x4
// (1,3,3,1)/8 tensor filter with taps clamped at the edges. Coarse cells
// whose fluid SDF is not negative receive 0: their rows are identity rows
// (no unknown), so the coarse correction there must stay 0, the Dirichlet
// value of the air. The reference passes the residual into those rows and
// prolongates the resulting non-zero values back into the fluid next to the
// free surface, which costs it multigrid's mesh-independent convergence.
__global__ void __launch_bounds__(kThreads)
    k_restrict(const float* __restrict__ fine, float* __restrict__ coarse,
               const float* __restrict__ coarse_phi, Dims c) {
    const long N = c.count();
    const int fx = 2 * c.x, fy = 2 * c.y;
    const float kern[4] = {0.125f, 0.375f, 0.375f, 0.125f};
    for (long t = blockIdx.x * (long)kThreads + threadIdx.x; t < N;
         t += (long)gridDim.x * kThreads) {
        int i, j, k;
        cell_ijk(t, c, i, j, k);
        int iI[4] = {i > 0 ? 2 * i - 1 : 2 * i, 2 * i, 2 * i + 1,
                     i + 1 < c.x ? 2 * i + 2 : 2 * i + 1};
        int jI[4] = {j > 0 ? 2 * j - 1 : 2 * j, 2 * j, 2 * j + 1,
                     j + 1 < c.y ? 2 * j + 2 : 2 * j + 1};
        int kI[4] = {k > 0 ? 2 * k - 1 : 2 * k, 2 * k, 2 * k + 1,
                     k + 1 < c.z ? 2 * k + 2 : 2 * k + 1};
        float sum = 0.0f;
#pragma unroll
        for (int z = 0; z < 4; ++z) {
            float sy = 0.0f;
#pragma unroll
            for (int y = 0; y < 4; ++y) {
                const float* rowp = fine + lin(0, jI[y], kI[z], fx, fy);
                const float sx = kern[0] * rowp[iI[0]] + kern[1] * rowp[iI[1]] +
                                 kern[2] * rowp[iI[2]] + kern[3] * rowp[iI[3]];
                sy += kern[y] * sx;
            }
            sum += kern[z] * sy;
        }
        coarse[t] = (coarse_phi[t] < 0.0f) ? sum : 0.0f;
    }
}

// k_restrict for coarse rows of even length: a thread owns coarse cells
// 2p and 2p+1 of a row, whose fine x taps 4p-1 .. 4p+4 (clamped as in
// k_restrict) are one aligned 16-byte load and two scalar loads per fine
// row instead of eight scalar loads. Same taps, weights and x-then-y-then-z
// order as k_restrict.
__global__ void __launch_bounds__(kThreads)
    k_restrict2(const float* __restrict__ fine, float* __restrict__ coarse,
                const float* __restrict__ coarse_phi, Dims c) {
    const Dims q{c.x / 2, c.y, c.z};
    const long G = q.count();
    const int fx = 2 * c.x, fy = 2 * c.y;
    const float kern[4] = {0.125f, 0.375f, 0.375f, 0.125f};
    for (long t = blockIdx.x * (long)kThreads + threadIdx.x; t < G;
         t += (long)gridDim.x * kThreads) {
        int p, j, k;
        cell_ijk(t, q, p, j, k);
        const int jI[4] = {j > 0 ? 2 * j - 1 : 2 * j, 2 * j, 2 * j + 1,
                           j + 1 < c.y ? 2 * j + 2 : 2 * j + 1};
        const int kI[4] = {k > 0 ? 2 * k - 1 : 2 * k, 2 * k, 2 * k + 1,
                           k + 1 < c.z ? 2 * k + 2 : 2 * k + 1};
        const int xm = p > 0 ? 4 * p - 1 : 4 * p;
        const int x4 = 2 * p + 2 < c.x ? 4 * p + 4 : 4 * p + 3;
        float sum0 = 0.0f, sum1 = 0.0f;
#pragma unroll
        for (int z = 0; z < 4; ++z) {
            float sy0 = 0.0f, sy1 = 0.0f;
#pragma unroll
            for (int y = 0; y < 4; ++y) {
                const float* rowp = fine + lin(0, jI[y], kI[z], fx, fy);
                const float4 f = *reinterpret_cast<const float4*>(rowp + 4 * p);
                const float fm = rowp[xm], f4 = rowp[x4];
                const float sx0 = kern[0] * fm + kern[1] * f.x +
                                  kern[2] * f.y + kern[3] * f.z;
                const float sx1 = kern[0] * f.y + kern[1] * f.z +
                                  kern[2] * f.w + kern[3] * f4;
                sy0 += kern[y] * sx0;
                sy1 += kern[y] * sx1;
            }
            sum0 += kern[z] * sy0;
            sum1 += kern[z] * sy1;
        }
        const long o = lin(2 * p, j, k, c.x, c.y);
        coarse[o] = (coarse_phi[o] < 0.0f) ? sum0 : 0.0f;
        coarse[o + 1] = (coarse_phi[o + 1] < 0.0f) ? sum1 : 0.0f;
    }
}

// K10: FdmMgUtils3::correct (fdm_mg_linear_system3.cpp:100-179): fine +=
// trilinear (1/4, 3/4) prolongation of coarse, clamped at the edges.
__global__ void __launch_bounds__(kThreads)
    k_correct(const float* __restrict__ coarse, float* __restrict__ fine,
              Dims c) {
    const Dims n{2 * c.x, 2 * c.y, 2 * c.z};
    const long N = n.count();
    for (long t = blockIdx.x * (long)kThreads + threadIdx.x; t < N;
         t += (long)gridDim.x * kThreads) {
        int i, j, k;
        cell_ijk(t, n, i, j, k);
        const int ci = i >> 1, cj = j >> 1, ck = k >> 1;
        int i0, i1, j0, j1, k0, k1;
        float wi0, wi1, wj0, wj1, wk0, wk1;
        if ((i & 1) == 0) { i0 = i > 1 ? ci - 1 : ci; i1 = ci; wi0 = 0.25f; wi1 = 0.75f; }
        else { i0 = ci; i1 = i + 1 < n.x ? ci + 1 : ci; wi0 = 0.75f; wi1 = 0.25f; }
        if ((j & 1) == 0) { j0 = j > 1 ? cj - 1 : cj; j1 = cj; wj0 = 0.25f; wj1 = 0.75f; }
        else { j0 = cj; j1 = j + 1 < n.y ? cj + 1 : cj; wj0 = 0.75f; wj1 = 0.25f; }
        if ((k & 1) == 0) { k0 = k > 1 ? ck - 1 : ck; k1 = ck; wk0 = 0.25f; wk1 = 0.75f; }
        else { k0 = ck; k1 = k + 1 < n.z ? ck + 1 : ck; wk0 = 0.75f; wk1 = 0.25f; }
        const float c000 = coarse[lin(i0, j0, k0, c.x, c.y)];
        const float c100 = coarse[lin(i1, j0, k0, c.x, c.y)];
        const float c010 = coarse[lin(i0, j1, k0, c.x, c.y)];
        const float c110 = coarse[lin(i1, j1, k0, c.x, c.y)];
        const float c001 = coarse[lin(i0, j0, k1, c.x, c.y)];
        const float c101 = coarse[lin(i1, j0, k1, c.x, c.y)];
        const float c011 = coarse[lin(i0, j1, k1, c.x, c.y)];
        const float c111 = coarse[lin(i1, j1, k1, c.x, c.y)];
        const float a0 = wj0 * (wi0 * c000 + wi1 * c100) + wj1 * (wi0 * c010 + wi1 * c110);
        const float a1 = wj0 * (wi0 * c001 + wi1 * c101) + wj1 * (wi0 * c011 + wi1 * c111);
        fine[t] += wk0 * a0 + wk1 * a1;
    }
}

// k_correct for fine rows whose length is a multiple of 4, marching through
// a run of coarse planes: a thread owns 4 consecutive fine cells of a row
// (fine i = 4m..4m+3, coarse 2m and 2m+1) and keeps the
// x-interpolated coarse values of the three coarse planes that the fine
// planes 2kc and 2kc+1 read (kc-1, kc, kc+1, clamped), so consecutive fine
// planes share them instead of gathering them again. Same stencil, weights
// and x-then-y-then-z order as k_correct. Five blocks per SM (48
// registers) run it 5% faster than four.
__global__ void __launch_bounds__(kThreads, 5)
    k_correct4z(const float* __restrict__ coarse, float* __restrict__ fine,
                Dims c, int run) {
    const Dims n{2 * c.x, 2 * c.y, 2 * c.z};
    const Dims q{n.x / 4, n.y, 1};  // 4-cell groups of a fine plane
    const long P = (long)q.x * q.y;
    const int runs = (c.z + run - 1) / run;
    const long G = P * runs;
    for (long t = blockIdx.x * (long)kThreads + threadIdx.x; t < G;
         t += (long)gridDim.x * kThreads) {
        const long pr = t % P;
        const int rz = (int)(t / P);
        const int m = (int)(pr % q.x), j = (int)(pr / q.x);
        const int kc0 = rz * run, kc1 = min(kc0 + run, c.z);
        const int cj = j >> 1;
        int j0, j1;
        float wj0, wj1;
        if ((j & 1) == 0) { j0 = j > 1 ? cj - 1 : cj; j1 = cj; wj0 = 0.25f; wj1 = 0.75f; }
        else { j0 = cj; j1 = j + 1 < n.y ? cj + 1 : cj; wj0 = 0.75f; wj1 = 0.25f; }
        const int x0 = 2 * m, xm = m > 0 ? x0 - 1 : x0,
                  x2 = 4 * m + 4 < n.x ? x0 + 2 : x0 + 1;
        // x-interpolated values of coarse plane kc at rows j0 and j1.
        auto rows = [&](int kc, float r0[4], float r1[4]) {
            const int rj[2] = {j0, j1};
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const float* row = coarse + lin(0, rj[e], kc, c.x, c.y);
                const float cm = row[xm], ca = row[x0], cb = row[x0 + 1],
                            cc = row[x2];
                float* r = e == 0 ? r0 : r1;
                r[0] = 0.25f * cm + 0.75f * ca;
                r[1] = 0.75f * ca + 0.25f * cb;
                r[2] = 0.25f * ca + 0.75f * cb;
                r[3] = 0.75f * cb + 0.25f * cc;
            }
        };
        float pm0[4], pm1[4], pc0[4], pc1[4], pp0[4], pp1[4];  // kc-1, kc, kc+1
        rows(kc0, pc0, pc1);
        if (kc0 > 0) {
            rows(kc0 - 1, pm0, pm1);
        } else {
#pragma unroll
            for (int l = 0; l < 4; ++l) { pm0[l] = pc0[l]; pm1[l] = pc1[l]; }
        }
        for (int kc = kc0; kc < kc1; ++kc) {
            if (kc + 1 < c.z) {
                rows(kc + 1, pp0, pp1);
            } else {
#pragma unroll
                for (int l = 0; l < 4; ++l) { pp0[l] = pc0[l]; pp1[l] = pc1[l]; }
            }
            // Fine plane 2kc: coarse kc-1 (1/4) and kc (3/4); 2kc+1: kc (3/4)
            // and kc+1 (1/4).
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int k = 2 * kc + h;
                const float* A0 = h == 0 ? pm0 : pc0;
                const float* A1 = h == 0 ? pm1 : pc1;
                const float* B0 = h == 0 ? pc0 : pp0;
                const float* B1 = h == 0 ? pc1 : pp1;
                const float wk0 = h == 0 ? 0.25f : 0.75f;
                const float wk1 = h == 0 ? 0.75f : 0.25f;
                float4* f4 = reinterpret_cast<float4*>(fine + lin(4 * m, j, k, n.x, n.y));
                float4 v = *f4;
                float o[4];
#pragma unroll
                for (int l = 0; l < 4; ++l) {
                    const float a0 = wj0 * A0[l] + wj1 * A1[l];
                    const float a1 = wj0 * B0[l] + wj1 * B1[l];
                    o[l] = wk0 * a0 + wk1 * a1;
                }
                v.x += o[0];
                v.y += o[1];
                v.z += o[2];
                v.w += o[3];
                *f4 = v;
            }
#pragma unroll
            for (int l = 0; l < 4; ++l) {
                pm0[l] = pc0[l]; pm1[l] = pc1[l];
                pc0[l] = pp0[l]; pc1[l] = pp1[l];
            }
        }
    }
}

// K11: coarsest level in one CTA: x and b in shared memory, `sweeps`
// forward red-black sweeps followed by `sweeps` sweeps in reverse colour
// order (symmetric), starting from x = 0.
constexpr int kCoarsestMaxCells = 4096;
template <typename R>
__global__ void __launch_bounds__(1024)
    k_coarsest(R A, const float* __restrict__ b,
               float* __restrict__ x, Dims n, int sweeps, float omega) {
    __shared__ float sx[kCoarsestMaxCells];
    __shared__ float sb[kCoarsestMaxCells];
    const int N = (int)n.count();
    const int sy = n.x, sz = n.x * n.y;
    for (int c = threadIdx.x; c < N; c += blockDim.x) {
        sx[c] = 0.0f;
        sb[c] = b[c];
    }
    __syncthreads();
    for (int pass = 0; pass < 2 * sweeps; ++pass) {
        for (int h = 0; h < 2; ++h) {
            const int color = (pass < sweeps) ? h : 1 - h;
            for (int c = threadIdx.x; c < N; c += blockDim.x) {
                const int i = c % n.x, j = (c / n.x) % n.y, k = c / sz;
                if (((i + j + k) & 1) != color) continue;
                const float4 r = A.row(c);
                float s = 0.0f;
                if (i > 0) s += A.row(c - 1).y * sx[c - 1];
                if (i + 1 < n.x) s += r.y * sx[c + 1];
                if (j > 0) s += A.row(c - sy).z * sx[c - sy];
                if (j + 1 < n.y) s += r.z * sx[c + sy];
                if (k > 0) s += A.row(c - sz).w * sx[c - sz];
                if (k + 1 < n.z) s += r.w * sx[c + sz];
                sx[c] = (1.0f - omega) * sx[c] + omega * (sb[c] - s) / r.x;
            }
            __syncthreads();
        }
    }
    for (int c = threadIdx.x; c < N; c += blockDim.x) x[c] = sx[c];
}

// ---------------------------------------------------------------------------
// The V-cycle below a level of at most kTailMaxCells cells in one CTA: every
// level of the tail (x, b, r, the fluid SDF and the rows widened to FP32)
// sits in shared memory, and the steps of the multi-kernel path — zero-start
// and continued red-black half-sweeps, residual, masked restriction,
// coarsest sweeps, correction — run as phases separated by block barriers,
// in the order and with the arithmetic of k_rb_half (division as in the
// fused sweep), k_residual32, k_restrict, k_coarsest and k_correct. On the
// small levels those kernels are a few microseconds of launch and drain
// each; here the whole tail is one launch.

constexpr int kTailMaxCells = 4096;
constexpr int kTailMaxLevels = 8;
constexpr int kTailThreads = 1024;

struct TailLevel {
    Dims n;
    const float* A;              // FP32 rows (structure of arrays) or null
    const unsigned short* Ah;    // BF16 rows (mixed mode) or null
    const float* phi;            // fluid SDF (masks the restriction)
};
struct TailArgs {
    TailLevel lv[kTailMaxLevels];
    int count;                   // levels in the tail
    const float* b;              // right-hand side of the first tail level
    float* x;                    // its V-cycle result
    int pre, post, coarsest;     // sweeps
    float omega;
};

// Shared-memory words of a tail level of N cells: x, b, r, phi, 4 rows and
// the packed (i, j, k) of every cell (10 bits each; tail levels are at most
// 4096 cells, so each extent is below 1024).
__host__ __device__ inline long tail_floats(long N) { return 9 * N; }

__device__ __forceinline__ void unpack_ijk(unsigned q, int& i, int& j, int& k) {
    i = (int)(q & 1023u);
    j = (int)((q >> 10) & 1023u);
    k = (int)(q >> 20);
}

// One colour of a red-black SOR sweep over a level held in shared memory
// (k_rb_half's arithmetic, with the fast division of the fused sweep): every
// cell of `color` is updated from its neighbours; with `zero` the sweep
// starts from x = 0, so the colour gets omega b / center and the other
// colour is written 0. One SM does the whole tail, so instructions per cell
// bound it.
__device__ __forceinline__ void tail_half(const float* A, const float* b,
                                          float* x, const unsigned* ijk,
                                          Dims n, int color, bool zero,
                                          float omega) {
    const int N = (int)n.count();
    const int sy = n.x, sz = n.x * n.y;
    for (int c = threadIdx.x; c < N; c += blockDim.x) {
        int i, j, k;
        unpack_ijk(ijk[c], i, j, k);
        const bool mine = ((i + j + k) & 1) == color;
        if (zero) {
            x[c] = mine ? omega * __fdividef(b[c], A[c]) : 0.0f;
            continue;
        }
        if (!mine) continue;
        float s = 0.0f;
        if (i > 0) s += A[N + c - 1] * x[c - 1];
        if (i + 1 < n.x) s += A[N + c] * x[c + 1];
        if (j > 0) s += A[2 * N + c - sy] * x[c - sy];
        if (j + 1 < n.y) s += A[2 * N + c] * x[c + sy];
        if (k > 0) s += A[3 * N + c - sz] * x[c - sz];
        if (k + 1 < n.z) s += A[3 * N + c] * x[c + sz];
        x[c] = (1.0f - omega) * x[c] + omega * __fdividef(b[c] - s, A[c]);
    }
}

// The shared-memory arrays of tail level l.
struct TailViews {
    float *x, *b, *r, *phi, *A;
    unsigned* ijk;
};
__device__ __forceinline__ TailViews tail_views(float* base, const TailArgs& a,
                                                int l) {
    float* q = base;
    for (int m = 0; m < l; ++m) q += tail_floats(a.lv[m].n.count());
    const long N = a.lv[l].n.count();
    return TailViews{q, q + N, q + 2 * N, q + 3 * N, q + 4 * N,
                     reinterpret_cast<unsigned*>(q + 8 * N)};
}

__global__ void __launch_bounds__(kTailThreads) k_vcycle_tail(TailArgs a) {
    extern __shared__ float tsm[];
    // Load: rows (BF16 widened), fluid SDF, cell indices, the first level's
    // b; four independent 16-byte (or 8-byte) loads per thread and step.
    for (int l = 0; l < a.count; ++l) {
        const TailLevel& L = a.lv[l];
        const TailViews v = tail_views(tsm, a, l);
        const int N = (int)L.n.count();
        if (N % 4 == 0) {
            const int N4 = N;  // 4 N floats of rows = N float4
            if (L.Ah) {
                const uint2* src = reinterpret_cast<const uint2*>(L.Ah);
                for (int e = threadIdx.x; e < N4; e += blockDim.x) {
                    const uint2 w = __ldg(src + e);
                    reinterpret_cast<float4*>(v.A)[e] = make_float4(
                        __uint_as_float(w.x << 16),
                        __uint_as_float(w.x & 0xffff0000u),
                        __uint_as_float(w.y << 16),
                        __uint_as_float(w.y & 0xffff0000u));
                }
            } else {
                const float4* src = reinterpret_cast<const float4*>(L.A);
                for (int e = threadIdx.x; e < N4; e += blockDim.x)
                    reinterpret_cast<float4*>(v.A)[e] = __ldg(src + e);
            }
            const float4* ph = reinterpret_cast<const float4*>(L.phi);
            for (int e = threadIdx.x; e < N / 4; e += blockDim.x)
                reinterpret_cast<float4*>(v.phi)[e] = __ldg(ph + e);
        } else {
            for (int e = threadIdx.x; e < 4 * N; e += blockDim.x)
                v.A[e] = L.Ah ? __uint_as_float((unsigned)L.Ah[e] << 16) : L.A[e];
            for (int e = threadIdx.x; e < N; e += blockDim.x) v.phi[e] = L.phi[e];
        }
        for (int c = threadIdx.x; c < N; c += blockDim.x) {
            const int i = c % L.n.x, j = (c / L.n.x) % L.n.y,
                      k = c / (L.n.x * L.n.y);
            v.ijk[c] = (unsigned)i | ((unsigned)j << 10) | ((unsigned)k << 20);
        }
    }
    {
        const TailViews v0 = tail_views(tsm, a, 0);
        for (int e = threadIdx.x; e < (int)a.lv[0].n.count(); e += blockDim.x)
            v0.b[e] = __ldg(a.b + e);
    }
    __syncthreads();
    const float w = a.omega;
    const int last = a.count - 1;
    // Down: pre-smoothing from zero, residual, masked restriction.
    for (int l = 0; l < last; ++l) {
        const TailViews v = tail_views(tsm, a, l);
        const Dims n = a.lv[l].n;
        const int N = (int)n.count();
        for (int s = 0; s < a.pre; ++s) {
            tail_half(v.A, v.b, v.x, v.ijk, n, 0, s == 0, w);
            __syncthreads();
            tail_half(v.A, v.b, v.x, v.ijk, n, 1, false, w);
            __syncthreads();
        }
        if (a.pre == 0) {
            for (int e = threadIdx.x; e < N; e += blockDim.x) v.x[e] = 0.0f;
            __syncthreads();
        }
        const int sy = n.x, sz = n.x * n.y;
        for (int c = threadIdx.x; c < N; c += blockDim.x) {
            int i, j, k;
            unpack_ijk(v.ijk[c], i, j, k);
            const float* x = v.x;
            const float* A = v.A;
            float sacc = A[c] * x[c];
            if (i > 0) sacc += A[N + c - 1] * x[c - 1];
            if (i + 1 < n.x) sacc += A[N + c] * x[c + 1];
            if (j > 0) sacc += A[2 * N + c - sy] * x[c - sy];
            if (j + 1 < n.y) sacc += A[2 * N + c] * x[c + sy];
            if (k > 0) sacc += A[3 * N + c - sz] * x[c - sz];
            if (k + 1 < n.z) sacc += A[3 * N + c] * x[c + sz];
            v.r[c] = v.b[c] - sacc;
        }
        __syncthreads();
        const TailViews cv = tail_views(tsm, a, l + 1);
        const Dims cn = a.lv[l + 1].n;
        const float kern[4] = {0.125f, 0.375f, 0.375f, 0.125f};
        for (int t = threadIdx.x; t < (int)cn.count(); t += blockDim.x) {
            int i, j, k;
            unpack_ijk(cv.ijk[t], i, j, k);
            const int iI[4] = {i > 0 ? 2 * i - 1 : 2 * i, 2 * i, 2 * i + 1,
                               i + 1 < cn.x ? 2 * i + 2 : 2 * i + 1};
            const int jI[4] = {j > 0 ? 2 * j - 1 : 2 * j, 2 * j, 2 * j + 1,
                               j + 1 < cn.y ? 2 * j + 2 : 2 * j + 1};
            const int kI[4] = {k > 0 ? 2 * k - 1 : 2 * k, 2 * k, 2 * k + 1,
                               k + 1 < cn.z ? 2 * k + 2 : 2 * k + 1};
            float sum = 0.0f;
#pragma unroll
            for (int z = 0; z < 4; ++z) {
                float syy = 0.0f;
#pragma unroll
                for (int y = 0; y < 4; ++y) {
                    const float* rowp = v.r + n.x * (jI[y] + n.y * kI[z]);
                    const float sx = kern[0] * rowp[iI[0]] + kern[1] * rowp[iI[1]] +
                                     kern[2] * rowp[iI[2]] + kern[3] * rowp[iI[3]];
                    syy += kern[y] * sx;
                }
                sum += kern[z] * syy;
            }
            cv.b[t] = (cv.phi[t] < 0.0f) ? sum : 0.0f;
        }
        __syncthreads();
    }
    // Coarsest level: forward sweeps from zero, then reverse.
    {
        const TailViews v = tail_views(tsm, a, last);
        const Dims n = a.lv[last].n;
        for (int e = threadIdx.x; e < (int)n.count(); e += blockDim.x)
            v.x[e] = 0.0f;
        __syncthreads();
        for (int pass = 0; pass < 2 * a.coarsest; ++pass)
            for (int h = 0; h < 2; ++h) {
                const int color = (pass < a.coarsest) ? h : 1 - h;
                tail_half(v.A, v.b, v.x, v.ijk, n, color, false, w);
                __syncthreads();
            }
    }
    // Up: correction, post-smoothing (colours reversed).
    for (int l = last - 1; l >= 0; --l) {
        const TailViews v = tail_views(tsm, a, l);
        const Dims n = a.lv[l].n, cn = a.lv[l + 1].n;
        const float* coarse = tail_views(tsm, a, l + 1).x;
        for (int t = threadIdx.x; t < (int)n.count(); t += blockDim.x) {
            int i, j, k;
            unpack_ijk(v.ijk[t], i, j, k);
            const int ci = i >> 1, cj = j >> 1, ck = k >> 1;
            int i0, i1, j0, j1, k0, k1;
            float wi0, wi1, wj0, wj1, wk0, wk1;
            if ((i & 1) == 0) { i0 = i > 1 ? ci - 1 : ci; i1 = ci; wi0 = 0.25f; wi1 = 0.75f; }
            else { i0 = ci; i1 = i + 1 < n.x ? ci + 1 : ci; wi0 = 0.75f; wi1 = 0.25f; }
            if ((j & 1) == 0) { j0 = j > 1 ? cj - 1 : cj; j1 = cj; wj0 = 0.25f; wj1 = 0.75f; }
            else { j0 = cj; j1 = j + 1 < n.y ? cj + 1 : cj; wj0 = 0.75f; wj1 = 0.25f; }
            if ((k & 1) == 0) { k0 = k > 1 ? ck - 1 : ck; k1 = ck; wk0 = 0.25f; wk1 = 0.75f; }
            else { k0 = ck; k1 = k + 1 < n.z ? ck + 1 : ck; wk0 = 0.75f; wk1 = 0.25f; }
            auto C = [&](int a0, int b0, int c0) {
                return coarse[a0 + cn.x * (b0 + cn.y * c0)];
            };
            const float a0 = wj0 * (wi0 * C(i0, j0, k0) + wi1 * C(i1, j0, k0)) +
                             wj1 * (wi0 * C(i0, j1, k0) + wi1 * C(i1, j1, k0));
            const float a1 = wj0 * (wi0 * C(i0, j0, k1) + wi1 * C(i1, j0, k1)) +
                             wj1 * (wi0 * C(i0, j1, k1) + wi1 * C(i1, j1, k1));
            v.x[t] += wk0 * a0 + wk1 * a1;
        }
        __syncthreads();
        for (int s = 0; s < a.post; ++s) {
            tail_half(v.A, v.b, v.x, v.ijk, n, 1, false, w);
            __syncthreads();
            tail_half(v.A, v.b, v.x, v.ijk, n, 0, false, w);
            __syncthreads();
        }
    }
    {
        const TailViews v0 = tail_views(tsm, a, 0);
        for (int e = threadIdx.x; e < (int)a.lv[0].n.count(); e += blockDim.x)
            a.x[e] = v0.x[e];
    }
}

// ---------------------------------------------------------------------------

// Grid of a reduction (or streaming) kernel over n elements: every block
// resident at once (SM count x the kernel's occupancy), so the grid-stride
// work is one wave with no tail; fixed per kernel and device, which keeps the
// block-ordered reductions deterministic.
template <typename K>
int rgrid(Ctx* c, K kernel, long n) {
    const void* key = reinterpret_cast<const void*>(kernel);
    auto it = c->occupancy.find(key);
    int occ = 0;
    if (it == c->occupancy.end()) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel,
                                                          kThreads, 0) !=
                cudaSuccess ||
            occ < 1)
            occ = 1;
        c->occupancy[key] = occ;
    } else {
        occ = it->second;
    }
    long g = (long)c->num_sms * occ;
    if (g > kMaxRedBlocks) g = kMaxRedBlocks;
    return blocks_for(n, kThreads, (int)g);
}

// BF16 rows for the mixed-precision V-cycle: the diagonal rounded up and the
// off-diagonals rounded toward zero, so a row that is diagonally dominant in
// FP32 stays so in BF16 (the V-cycle remains a convergent SPD
// preconditioner); x, b and all arithmetic stay FP32.
__device__ __forceinline__ unsigned bf_trunc(float v) {
    return __float_as_uint(v) >> 16;
}
__device__ __forceinline__ unsigned bf_up(float v) {
    const unsigned u = __float_as_uint(v);
    const unsigned t = u >> 16;
    return (v > 0.0f && (u & 0xffffu) != 0u) ? t + 1u : t;
}
__global__ void k_rows_to_bf16(const float* __restrict__ A,
                               unsigned short* __restrict__ Ah, long N) {
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x) {
        Ah[c] = (unsigned short)bf_up(A[c]);
        Ah[N + c] = (unsigned short)bf_trunc(A[N + c]);
        Ah[2 * N + c] = (unsigned short)bf_trunc(A[2 * N + c]);
        Ah[3 * N + c] = (unsigned short)bf_trunc(A[3 * N + c]);
    }
}

bool mixed(const Ctx* c) {
    return c->cfg.precision == JETGPU_PRECISION_MIXED_BF16;
}
// Calls f with the V-cycle rows of level L: BF16 in mixed mode, else FP32.
template <typename F>
void with_rows(const Ctx* c, const Level& L, F&& f) {
    if (mixed(c)) f(RowsB{L.Ah, L.n.count()});
    else f(RowsF{L.A, L.n.count()});
}
// Bytes per cell of a stored V-cycle row.
double row_bytes(const Ctx* c) { return mixed(c) ? 8.0 : 16.0; }

int grid_for(const Ctx* c, long work) {
    int cap = c->num_sms * 8;
    return blocks_for(work, kThreads, cap);
}

void rb_half(Ctx* c, const Level& L, const float* b, float* x, int color,
             bool zero, int cls) {
    const long pairs = (long)((L.n.x + 1) / 2) * L.n.y * L.n.z;
    const float w = (float)c->cfg.sor;
    Prof pr(c, cls, (6.0 + 0.5 * row_bytes(c)) * L.n.count());
    with_rows(c, L, [&](auto M) {
        if (zero)
            k_rb_half<true><<<grid_for(c, pairs), kThreads, 0, c->stream>>>(
                M, b, x, L.n, color, w);
        else
            k_rb_half<false><<<grid_for(c, pairs), kThreads, 0, c->stream>>>(
                M, b, x, L.n, color, w);
    });
}

// Launch shape of the fused sweep. Blocks that hold neighbouring tiles
// should stage the same plane at the same time: the ring rows and the
// partial lines at a tile's i-edges are then read from L2, where the
// neighbour just brought them. Each tile column is cut into segments of
// seg_len planes (at least 4: a segment pays 2 extra steps to fill the
// pipeline), numbered segment by segment. When every tile fits in one wave,
// each block takes one segment and all march in lock-step; otherwise a grid
// of the resident blocks walks the items in that order, so the resident
// blocks always work on neighbouring tiles of about the same segment.
struct ColLaunch {
    int grid, tiles_x, tiles, seg_len;
    long items;
};
ColLaunch col_launch(const Ctx* c, const Level& L, int tcx, int ty,
                     int blocks_per_sm) {
    ColLaunch r;
    r.tiles_x = (L.n.x + tcx - 1) / tcx;
    r.tiles = r.tiles_x * ((L.n.y + ty - 1) / ty);
    const long resident = std::max<long>(1, (long)c->num_sms * blocks_per_sm);
    if (r.tiles <= resident) {
        const long m = std::max<long>(
            1, std::min<long>(resident / r.tiles, (L.n.z + 3) / 4));
        r.seg_len = (int)((L.n.z + m - 1) / m);
    } else {
        // About four items per resident block.
        const long want = 4 * resident;
        r.seg_len = (int)std::max<long>(
            4, std::min<long>(L.n.z, (long)r.tiles * L.n.z / want));
    }
    r.items = (long)r.tiles * ((L.n.z + r.seg_len - 1) / r.seg_len);
    r.grid = (int)(r.tiles <= resident ? r.items
                                       : std::min<long>(r.items, resident));
    return r;
}

// ---- TMA sweep (sweep_tma.cuh): tensor maps and launch --------------------

// Row element, prefetch distance (planes) and resident blocks per SM the
// register budget is set for, of the TMA sweep: with two planes in flight a
// block holds 68 KB of shared memory with FP32 rows and 51 KB with BF16
// rows; both run three blocks per SM (BF16 rows at four blocks spill a few
// registers and were 1% slower; one plane in flight, or two blocks per SM
// for FP32 rows, were slower too).
template <typename R> struct TmaCfg;
template <> struct TmaCfg<RowsF> {
    using E = float;
    static constexpr int D = 2;
    static constexpr int MINB = 3;
};
template <> struct TmaCfg<RowsB> {
    using E = unsigned short;
    static constexpr int D = 2;
    static constexpr int MINB = 3;
};

bool tma_ok(const Ctx* c, const Level& L) {
    return c->tma_blocks_per_sm[mixed(c) ? 1 : 0] > 0 && L.n.x % 8 == 0 &&
           L.n.x >= 64;
}

// Tiled map over `rank` dims (innermost first) of a dense array at p.
bool encode_map(CUtensorMap* m, CUtensorMapDataType dt, int esize, int rank,
                const void* p, const long* dims, const unsigned* box) {
    cuuint64_t gd[4], gs[3];
    cuuint32_t bx[4], es[4] = {1, 1, 1, 1};
    long stride = esize;
    for (int d = 0; d < rank; ++d) {
        gd[d] = (cuuint64_t)dims[d];
        bx[d] = box[d];
        if (d > 0) gs[d - 1] = (cuuint64_t)stride;
        stride *= dims[d];
    }
    return tma_encoder()(m, dt, (cuuint32_t)rank, const_cast<void*>(p), gd, gs,
                         bx, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                         CU_TENSOR_MAP_SWIZZLE_NONE,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Tensor maps of one smoothing call: b, the rows, and the two ping-pong x
// buffers (the sweeps alternate between them).
struct TmaMaps {
    CUtensorMap b, r, x[2];
};

template <typename R>
bool tma_maps(TmaMaps* m, const R& M, const float* b, const float* x0,
              const float* x1, Dims n) {
    using E = typename TmaCfg<R>::E;
    using Lt = tsw::Layout<E, TmaCfg<R>::D>;
    const long d3[3] = {n.x, n.y, n.z};
    const long d4[4] = {n.x, n.y, n.z, 4};
    const unsigned bx[3] = {tsw::XW, tsw::XH, 1};
    const unsigned bb[3] = {tsw::XW, tsw::BH, 1};
    const unsigned br[4] = {Lt::RW, tsw::RH, 1, 4};
    return encode_map(&m->b, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, 3, b, d3,
                      bb) &&
           encode_map(&m->r, tsw::Elem<E>::dtype, (int)sizeof(E), 4, M.A, d4,
                      br) &&
           encode_map(&m->x[0], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, 3, x0, d3,
                      bx) &&
           encode_map(&m->x[1], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, 3, x1, d3,
                      bx);
}

// One TMA-staged fused sweep from x[src] (or from zero) into xout.
template <typename R>
void launch_tma(Ctx* c, const ColLaunch& cl, const TmaMaps& m, int src,
                bool zero, float* xout, Dims n, int first) {
    using E = typename TmaCfg<R>::E;
    constexpr int D = TmaCfg<R>::D;
    constexpr int smem = tsw::Layout<E, D>::TOTAL;
    double* err = c->scal + S_WAIT;
    if (zero)
        tsw::k_rb_sweep_tma<true, E, D, TmaCfg<R>::MINB>
            <<<cl.grid, tsw::BLOCK, smem, c->stream>>>(
                m.b, m.r, m.b, xout, n, first, (float)c->cfg.sor, cl.tiles_x,
                cl.tiles, cl.seg_len, cl.items, err);
    else
        tsw::k_rb_sweep_tma<false, E, D, TmaCfg<R>::MINB>
            <<<cl.grid, tsw::BLOCK, smem, c->stream>>>(
                m.x[src], m.r, m.b, xout, n, first, (float)c->cfg.sor,
                cl.tiles_x, cl.tiles, cl.seg_len, cl.items, err);
}

// Shared-memory limit and resident blocks per SM of both TMA sweep variants
// with rows R (0 when they cannot run).
template <typename R>
jetgpu_status tma_prepare(Ctx* c, int* blocks) {
    using E = typename TmaCfg<R>::E;
    constexpr int D = TmaCfg<R>::D;
    const int smem = tsw::Layout<E, D>::TOTAL;
    int occ[2] = {0, 0};
    JG_CUDA(c, cudaFuncSetAttribute(tsw::k_rb_sweep_tma<true, E, D, TmaCfg<R>::MINB>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    smem));
    JG_CUDA(c, cudaFuncSetAttribute(tsw::k_rb_sweep_tma<false, E, D, TmaCfg<R>::MINB>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    smem));
    JG_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                   &occ[0], tsw::k_rb_sweep_tma<true, E, D, TmaCfg<R>::MINB>, tsw::BLOCK, smem));
    JG_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                   &occ[1], tsw::k_rb_sweep_tma<false, E, D, TmaCfg<R>::MINB>, tsw::BLOCK, smem));
    *blocks = tma_encoder() ? std::min(occ[0], occ[1]) : 0;
    return JETGPU_OK;
}


// `sweeps` red-black sweeps (colour order reversed when `reverse`) starting
// from x = 0 when `zero`, else from *x. Levels the fused kernel serves
// ping-pong between x and alt; the return value holds the result.
float* smooth(Ctx* c, const Level& L, const float* b, float* x, float* alt,
              unsigned sweeps, bool reverse, bool zero, int l) {
    const int first = reverse ? 1 : 0;
    if (sweeps == 0) {
        if (zero)
            k_zero<float><<<grid_for(c, L.n.count()), kThreads, 0,
                            c->stream>>>(x, L.n.count());
        return x;
    }
    if (alt != nullptr && tma_ok(c, L)) {
        const ColLaunch cl = col_launch(c, L, tsw::TX, tsw::TY,
                                        c->tma_blocks_per_sm[mixed(c) ? 1 : 0]);
        bool done = false;
        float* out = x;
        with_rows(c, L, [&](auto M) {
            using R = decltype(M);
            TmaMaps maps;
            if (!tma_maps(&maps, M, b, x, alt, L.n)) return;  // half sweeps
            float* buf[2] = {x, alt};
            int cur = 0;
            for (unsigned s = 0; s < sweeps; ++s) {
                const bool z0 = zero && s == 0;
                Prof pr(c, l == 0 ? K_SWEEP_L0 : K_SWEEP_COARSE,
                        ((z0 ? 8.0 : 12.0) + row_bytes(c)) * L.n.count());
                launch_tma<R>(c, cl, maps, cur, z0, buf[1 - cur], L.n, first);
                cur = 1 - cur;
            }
            out = buf[cur];
            done = true;
        });
        if (done) return out;
    }
    const int cls = l == 0 ? K_HALF_L0 : K_HALF_COARSE;
    for (unsigned s = 0; s < sweeps; ++s) {
        rb_half(c, L, b, x, first, zero && s == 0, cls);
        rb_half(c, L, b, x, 1 - first, false, cls);
    }
    return x;
}

// First level of the one-CTA tail (k_vcycle_tail): the first level below
// the finest whose cells, with every coarser level's, fit the tail's shared
// memory; nl (no tail) when none does.
unsigned tail_start(const Ctx* c) {
    const unsigned nl = c->built_levels;
    if (nl < 3) return nl;
    for (unsigned l = 1; l + 1 < nl; ++l) {
        if (c->levels[l].n.count() > kTailMaxCells) continue;
        if (nl - l > (unsigned)kTailMaxLevels) return nl;
        long floats = 0;
        for (unsigned m = l; m < nl; ++m)
            floats += tail_floats(c->levels[m].n.count());
        return floats * 4 <= 200 * 1024 ? l : nl;
    }
    return nl;
}

float* vcycle_tail(Ctx* c, unsigned l, const float* b, float* x) {
    const unsigned nl = c->built_levels;
    const jetgpu_config& cfg = c->cfg;
    TailArgs a{};
    a.count = (int)(nl - l);
    long floats = 0;
    for (unsigned m = l; m < nl; ++m) {
        const Level& L = c->levels[m];
        a.lv[m - l] = TailLevel{L.n, mixed(c) ? nullptr : L.A,
                                mixed(c) ? L.Ah : nullptr, L.phi};
        floats += tail_floats(L.n.count());
    }
    a.b = b;
    a.x = x;
    a.pre = (int)cfg.restrict_iter;
    a.post = (int)cfg.correct_iter;
    a.coarsest = (int)cfg.coarsest_iter;
    a.omega = (float)cfg.sor;
    long cells = 0;
    for (unsigned m = l; m < nl; ++m) cells += c->levels[m].n.count();
    Prof pr(c, K_COARSEST, (12.0 + row_bytes(c)) * (double)cells);
    k_vcycle_tail<<<1, kTailThreads, floats * sizeof(float), c->stream>>>(a);
    return x;
}

// Symmetric V-cycle on level l from a zero initial guess; returns the
// buffer (x or alt) that holds the result.
float* vcycle_level(Ctx* c, unsigned l, const float* b, float* x, float* alt) {
    const Level& L = c->levels[l];
    const unsigned nl = c->built_levels;
    const jetgpu_config& cfg = c->cfg;
    if (l > 0 && l == tail_start(c)) return vcycle_tail(c, l, b, x);
    if (l + 1 == nl) {
        if (L.n.count() <= kCoarsestMaxCells) {
            int nt = (int)std::min<long>(1024, ((L.n.count() + 31) / 32) * 32);
            Prof pr(c, K_COARSEST, (12.0 + row_bytes(c)) * L.n.count());
            with_rows(c, L, [&](auto M) {
                k_coarsest<<<1, nt, 0, c->stream>>>(M, b, x, L.n,
                                                    (int)cfg.coarsest_iter,
                                                    (float)cfg.sor);
            });
            return x;
        }
        float* cur = smooth(c, L, b, x, alt, cfg.coarsest_iter, false, true, l);
        return smooth(c, L, b, cur, cur == x ? alt : x, cfg.coarsest_iter,
                      true, false, l);
    }
    const Level& C = c->levels[l + 1];
    float* cur = smooth(c, L, b, x, alt, cfg.restrict_iter, false, true, l);
    float* other = (cur == x) ? alt : x;
    {
        Prof pr(c, K_RESIDUAL, (12.0 + row_bytes(c)) * L.n.count());
        with_rows(c, L, [&](auto M) {
            if (L.n.x % 4 == 0)
                k_residual32x4<<<grid_for(c, L.n.count() / 4), kThreads, 0,
                                 c->stream>>>(M, cur, b, L.r, L.n);
            else
                k_residual32<<<grid_for(c, L.n.count()), kThreads, 0,
                               c->stream>>>(M, cur, b, L.r, L.n);
        });
    }
    {
        Prof pr(c, K_RESTRICT, 4.0 * L.n.count() + 8.0 * C.n.count());
        if (C.n.x % 2 == 0)
            k_restrict2<<<grid_for(c, C.n.count() / 2), kThreads, 0,
                          c->stream>>>(L.r, C.b, C.phi, C.n);
        else
            k_restrict<<<grid_for(c, C.n.count()), kThreads, 0, c->stream>>>(
                L.r, C.b, C.phi, C.n);
    }
    const float* xc = vcycle_level(c, l + 1, C.b, C.x, C.x2);
    {
        Prof pr(c, K_CORRECT, 8.0 * L.n.count() + 4.0 * C.n.count());
        if (L.n.x % 4 == 0) {
            // Runs of coarse planes as long as the grid still fills the
            // GPU (2048 threads per SM), at most 4.
            const long groups = L.n.count() / 4 / L.n.z;
            const long full = (long)c->num_sms * 2048;
            int run = (int)std::min<long>(
                4, std::max<long>(1, groups * C.n.z / full));
            const long items = groups * ((C.n.z + run - 1) / run);
            k_correct4z<<<blocks_for(items), kThreads, 0, c->stream>>>(
                xc, cur, C.n, run);
        } else
            k_correct<<<grid_for(c, L.n.count()), kThreads, 0, c->stream>>>(
                xc, cur, C.n);
    }
    return smooth(c, L, b, cur, other,
                  l == 0 ? cfg.final_iter : cfg.correct_iter, true, false, l);
}

jetgpu_status read_scalars(Ctx* c) {
    JG_CUDA(c, cudaMemcpyAsync(c->h_scal, c->scal, S_COUNT * sizeof(double),
                               cudaMemcpyDeviceToHost, c->stream));
    JG_CUDA(c, cudaStreamSynchronize(c->stream));
    if (c->h_scal[S_WAIT] != 0.0) {
        JG_CUDA(c, cudaMemsetAsync(c->scal + S_WAIT, 0, sizeof(double),
                                   c->stream));
        c->err = "a shared-memory stage of the red-black sweep did not arrive "
                 "within its wait limit";
        return JETGPU_CUDA_ERROR;
    }
    return JETGPU_OK;
}

}  // namespace

PFN_cuTensorMapEncodeTiled_v12000 tma_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p,
                                             12000, cudaEnableDefault,
                                             &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

unsigned level_count(Dims n, unsigned max_levels) {
    unsigned i = 1;
    Dims r = n;
    for (; i < max_levels; ++i) {
        if (r.x % 2 == 0 && r.y % 2 == 0 && r.z % 2 == 0) {
            r.x >>= 1;
            r.y >>= 1;
            r.z >>= 1;
        } else {
            break;
        }
    }
    return i < 1 ? 1 : i;
}

jetgpu_status vcycle(Ctx* c, const float* r, float* z, float* alt,
                     float** result) {
    *result = vcycle_level(c, 0, r, z, alt);
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

jetgpu_status prepare_levels(Ctx* c, unsigned lo, unsigned hi) {
    if (!mixed(c)) return JETGPU_OK;
    for (unsigned l = lo; l < c->built_levels && l < hi; ++l) {
        const Level& L = c->levels[l];
        const long N = L.n.count();
        Prof pr(c, K_SYSTEM, 24.0 * N);
        k_rows_to_bf16<<<grid_for(c, N), kThreads, 0, c->stream>>>(L.A, L.Ah,
                                                                   N);
    }
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

jetgpu_status init_kernels(Ctx* c) {
    jetgpu_status st;
    JG_CUDA(c, cudaFuncSetAttribute(k_vcycle_tail,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    200 * 1024));
    if ((st = tma_prepare<RowsF>(c, &c->tma_blocks_per_sm[0])) != JETGPU_OK)
        return st;
    if ((st = tma_prepare<RowsB>(c, &c->tma_blocks_per_sm[1])) != JETGPU_OK)
        return st;
    return JETGPU_OK;
}

// The V-cycle as one CUDA graph. A V-cycle is about 50 launches, most of
// them on the small coarse levels, where launch latency rather than memory
// bounds the time; replaying a captured graph removes the per-launch host
// work and shortens the gaps between the kernels. The graph is captured on
// first use and again whenever the vectors, the level count or the smoother
// settings differ from the captured ones (the buffers' reallocation destroys
// it). Launches bracketed by the live profile, and any failure to capture,
// take the direct path.
jetgpu_status vcycle_graph(Ctx* c, const float* r, float* z, float* alt,
                           float** result) {
    if (c->prof_on || c->vc_disabled) return vcycle(c, r, z, alt, result);
    const jetgpu_config& f = c->cfg;
    const bool same =
        c->vc_exec && c->vc_key[0] == r && c->vc_key[1] == z &&
        c->vc_key[2] == alt && c->vc_levels == c->built_levels &&
        c->vc_iters[0] == f.restrict_iter && c->vc_iters[1] == f.correct_iter &&
        c->vc_iters[2] == f.coarsest_iter && c->vc_iters[3] == f.final_iter &&
        c->vc_sor == f.sor && c->vc_precision == f.precision;
    if (!same) {
        if (c->vc_exec) {
            cudaGraphExecDestroy(c->vc_exec);
            c->vc_exec = nullptr;
        }
        auto give_up = [&]() {
            c->vc_disabled = true;
            cudaGetLastError();
            return vcycle(c, r, z, alt, result);
        };
        if (cudaStreamBeginCapture(c->stream,
                                   cudaStreamCaptureModeThreadLocal) !=
            cudaSuccess)
            return give_up();
        float* res = vcycle_level(c, 0, r, z, alt);
        cudaGraph_t graph = nullptr;
        const cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
        if (e != cudaSuccess || graph == nullptr) {
            if (graph) cudaGraphDestroy(graph);
            return give_up();
        }
        const cudaError_t ei = cudaGraphInstantiate(&c->vc_exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess) {
            c->vc_exec = nullptr;
            return give_up();
        }
        c->vc_key[0] = r;
        c->vc_key[1] = z;
        c->vc_key[2] = alt;
        c->vc_levels = c->built_levels;
        c->vc_iters[0] = f.restrict_iter;
        c->vc_iters[1] = f.correct_iter;
        c->vc_iters[2] = f.coarsest_iter;
        c->vc_iters[3] = f.final_iter;
        c->vc_sor = f.sor;
        c->vc_precision = f.precision;
        c->vc_result = res;
    }
    JG_CUDA(c, cudaGraphLaunch(c->vc_exec, c->stream));
    *result = c->vc_result;
    return JETGPU_OK;
}

// q = A d and d.q on the FP32 Krylov vectors (kd -> kq).
void spmv_f32(Ctx* c, const RowsF& M, Dims n) {
    const long N = n.count();
    if (n.x % 4 == 0)
        k_spmv_dot4<RowsF><<<rgrid(c, k_spmv_dot4<RowsF>, N / 4), kThreads, 0,
                             c->stream>>>(M, c->kd, c->kq, n, c->partials,
                                          c->counters, c->scal);
    else
        k_spmv_dot<float, RowsF><<<rgrid(c, k_spmv_dot<float, RowsF>, N),
                                   kThreads, 0, c->stream>>>(
            M, c->kd, c->kq, n, c->partials, c->counters, c->scal);
}

// One FP32 PCG iteration after z = M r: r.z (beta), d = z + beta d,
// q = A d (alpha), x += alpha d, r -= alpha q (r.r).
static void pcg_f32_updates(Ctx* c, const RowsF& M, Dims n, const float* z) {
    const long N = n.count();
    k_dot_rz4<<<rgrid(c, k_dot_rz4, N / 4), kThreads, 0, c->stream>>>(
        c->kr, z, N, c->partials, c->counters, c->scal);
    k_update_d4<<<rgrid(c, k_update_d4, N / 4), kThreads, 0, c->stream>>>(
        c->kd, z, N, c->scal);
    spmv_f32(c, M, n);
    k_update_xr4<<<rgrid(c, k_update_xr4, N / 4), kThreads, 0, c->stream>>>(
        c->kx, c->kr, c->kd, c->kq, N, c->partials, c->counters, c->scal);
}

// The multigrid FP32 PCG loop as one graph: a while node whose body is one
// iteration (the V-cycle's launches captured directly, the Krylov updates)
// followed by k_loop_check, which ends the loop on the device. The host
// launches it once per refinement pass and reads the scalars once. It is
// captured for the vectors and settings of the V-cycle graph (vc_exec),
// is rebuilt with it, and any failure to build it turns the path off (the
// host loop below is then used). Rows with nx % 4 != 0 use the host loop.
static jetgpu_status pcg_loop_graph(Ctx* c, double target, unsigned max_it,
                                    unsigned* it_out, double* rr_out,
                                    bool* used) {
    *used = false;
    const Level& L0 = c->levels[0];
    const Dims n = L0.n;
    if (c->prof_on || c->loop_disabled || c->vc_disabled || n.x % 4 != 0 ||
        max_it == 0)
        return JETGPU_OK;
    const jetgpu_config& f = c->cfg;
    const bool same =
        c->vc_exec && c->loop_exec && c->vc_key[0] == c->kr &&
        c->vc_key[1] == c->kz && c->vc_key[2] == L0.x2 &&
        c->vc_levels == c->built_levels && c->vc_iters[0] == f.restrict_iter &&
        c->vc_iters[1] == f.correct_iter && c->vc_iters[2] == f.coarsest_iter &&
        c->vc_iters[3] == f.final_iter && c->vc_sor == f.sor &&
        c->vc_precision == f.precision;
    if (!same) {
        // (Re)capture the V-cycle graph first: it owns the key.
        float* z = nullptr;
        if (c->loop_exec) {
            cudaGraphExecDestroy(c->loop_exec);
            c->loop_exec = nullptr;
        }
        if (c->vc_exec) {
            cudaGraphExecDestroy(c->vc_exec);
            c->vc_exec = nullptr;
        }
        // Capture the V-cycle graph now (vcycle_graph records the key) with
        // nothing enqueued: capture only records launches.
        cudaGraph_t g = nullptr, body = nullptr;
        auto give_up = [&]() {
            if (g) cudaGraphDestroy(g);
            c->loop_disabled = true;
            cudaGetLastError();
            return JETGPU_OK;
        };
        if (cudaGraphCreate(&g, 0) != cudaSuccess) return give_up();
        cudaGraphConditionalHandle h;
        if (cudaGraphConditionalHandleCreate(&h, g, 1,
                                             cudaGraphCondAssignDefault) !=
            cudaSuccess)
            return give_up();
        cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
        std::memset(reinterpret_cast<unsigned char*>(&np), 0, sizeof(np));
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = h;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        cudaGraphNode_t node;
        if (cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np) != cudaSuccess)
            return give_up();
        body = np.conditional.phGraph_out[0];
        if (cudaStreamBeginCaptureToGraph(c->stream, body, nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal) !=
            cudaSuccess)
            return give_up();
        z = vcycle_level(c, 0, c->kr, c->kz, L0.x2);
        pcg_f32_updates(c, RowsF{L0.A, n.count()}, n, z);
        k_loop_check<<<1, 1, 0, c->stream>>>(h, c->scal);
        cudaGraph_t captured = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(c->stream, &captured);
        if (ec != cudaSuccess) return give_up();
        if (cudaGraphInstantiate(&c->loop_exec, g, 0) != cudaSuccess) {
            c->loop_exec = nullptr;
            return give_up();
        }
        cudaGraphDestroy(g);
        // The V-cycle graph of the same key (used by the other solver paths).
        float* vz = nullptr;
        if (jetgpu_status vs = vcycle_graph(c, c->kr, c->kz, L0.x2, &vz)) {
            (void)vz;
            return vs;
        }
        // vcycle_graph launched one V-cycle: harmless (z is rewritten by the
        // loop's first iteration), but keep the stream ordered.
    }
    k_loop_start<<<1, 1, 0, c->stream>>>(c->scal, target, (double)max_it);
    JG_CUDA(c, cudaGraphLaunch(c->loop_exec, c->stream));
    jetgpu_status s = read_scalars(c);
    if (s != JETGPU_OK) return s;
    const double rr = c->h_scal[S_RR];
    if (!std::isfinite(rr))
        return fail(c, JETGPU_NUMERICAL_ERROR, "non-finite residual in FP32 PCG");
    *it_out = (unsigned)c->h_scal[S_LOOP_IT];
    *rr_out = rr;
    *used = true;
    return JETGPU_OK;
}

// PCG on the FP32 rows for a correction e with A e = r (r = kr on entry).
// Stops when ||r_k|| <= target or after max_it iterations.
static jetgpu_status pcg_f32(Ctx* c, double target, unsigned max_it,
                             unsigned* it_out, double* rr_out) {
    const Level& L0 = c->levels[0];
    const Dims n = L0.n;
    const long N = n.count();
    RowsF M{L0.A, N};
    if (c->cfg.preconditioner == JETGPU_PRECOND_MULTIGRID) {
        bool used = false;
        jetgpu_status ls = pcg_loop_graph(c, target, max_it, it_out, rr_out,
                                          &used);
        if (ls != JETGPU_OK || used) return ls;
    }
    k_init_scalars<<<1, 32, 0, c->stream>>>(c->scal);
    unsigned it = 0;
    double rr = 0;
    while (it < max_it) {
        float* z = nullptr;
        if (c->cfg.preconditioner == JETGPU_PRECOND_NONE) {
            z = c->kr;  // plain CG: z = r
        } else if (jetgpu_status vs = vcycle_graph(c, c->kr, c->kz, L0.x2, &z)) {
            return vs;
        }
        {
            Prof pr(c, K_DOT_RZ, 8.0 * N);
            if (N % 4 == 0)
                k_dot_rz4<<<rgrid(c, k_dot_rz4, N / 4), kThreads, 0,
                            c->stream>>>(c->kr, z, N, c->partials,
                                         c->counters, c->scal);
            else
                k_dot_rz<float, float><<<rgrid(c, k_dot_rz<float, float>, N),
                                         kThreads, 0, c->stream>>>(
                    c->kr, z, N, c->partials, c->counters, c->scal);
        }
        {
            Prof pr(c, K_UPDATE_D, 12.0 * N);
            if (N % 4 == 0)
                k_update_d4<<<rgrid(c, k_update_d4, N / 4), kThreads, 0,
                              c->stream>>>(c->kd, z, N, c->scal);
            else
                k_update_d<float, float><<<rgrid(c, k_update_d<float, float>, N),
                                           kThreads, 0, c->stream>>>(
                    c->kd, z, N, c->scal);
        }
        {
            Prof pr(c, K_SPMV, 24.0 * N);
            spmv_f32(c, M, n);
        }
        {
            Prof pr(c, K_UPDATE_XR, 24.0 * N);
            if (N % 4 == 0)
                k_update_xr4<<<rgrid(c, k_update_xr4, N / 4), kThreads, 0,
                               c->stream>>>(c->kx, c->kr, c->kd, c->kq, N,
                                            c->partials, c->counters,
                                            c->scal);
            else
                k_update_xr<float><<<rgrid(c, k_update_xr<float>, N),
                                     kThreads, 0, c->stream>>>(
                    c->kx, c->kr, c->kd, c->kq, nullptr, N, c->partials,
                    c->counters, c->scal);
        }
        ++it;
        jetgpu_status s = read_scalars(c);
        if (s != JETGPU_OK) return s;
        rr = c->h_scal[S_RR];
        if (!std::isfinite(rr))
            return fail(c, JETGPU_NUMERICAL_ERROR,
                        "non-finite residual in FP32 PCG");
        if (std::sqrt(rr) <= target) break;
    }
    *it_out = it;
    *rr_out = rr;
    return JETGPU_OK;
}

// PCG in FP64 on the exact rows; x64 is the iterate, r64 the residual.
static jetgpu_status pcg_f64(Ctx* c, double target, unsigned max_it,
                             unsigned* it_out, double* rr_out) {
    const Level& L0 = c->levels[0];
    const Dims n = L0.n;
    const long N = n.count();
    RowsD M{c->A64};
    k_init_scalars<<<1, 32, 0, c->stream>>>(c->scal);
    unsigned it = 0;
    double rr = 0;
    float* r32 = L0.b;  // FP32 copy of r feeds the V-cycle
    // r32 already holds float(r64) (written by the residual kernel).
    while (it < max_it) {
        float* z = nullptr;
        if (jetgpu_status vs = vcycle(c, r32, L0.x, L0.x2, &z)) return vs;
        {
            Prof pr(c, K_DOT_RZ, 12.0 * N);
            k_dot_rz<double, float><<<rgrid(c, k_dot_rz<double, float>, N), kThreads, 0,
            c->stream>>>(
                c->r64, z, N, c->partials, c->counters, c->scal);
        }
        {
            Prof pr(c, K_UPDATE_D, 20.0 * N);
            k_update_d<double, float><<<rgrid(c, k_update_d<double, float>, N), kThreads, 0,
            c->stream>>>(
                c->dd, z, N, c->scal);
        }
        {
            Prof pr(c, K_SPMV, 48.0 * N);
            k_spmv_dot<double, RowsD><<<rgrid(c, k_spmv_dot<double, RowsD>, N), kThreads, 0,
            c->stream>>>(
                M, c->dd, c->dq, n, c->partials, c->counters, c->scal);
        }
        {
            Prof pr(c, K_UPDATE_XR, 52.0 * N);
            k_update_xr<double><<<rgrid(c, k_update_xr<double>, N), kThreads, 0,
            c->stream>>>(
                c->x64, c->r64, c->dd, c->dq, r32, N, c->partials,
                c->counters, c->scal);
        }
        ++it;
        jetgpu_status s = read_scalars(c);
        if (s != JETGPU_OK) return s;
        rr = c->h_scal[S_RR];
        if (!std::isfinite(rr))
            return fail(c, JETGPU_NUMERICAL_ERROR,
                        "non-finite residual in FP64 PCG");
        if (std::sqrt(rr) <= target) break;
    }
    *it_out = it;
    *rr_out = rr;
    return JETGPU_OK;
}

// ---------------------------------------------------------------------------
// Flexible PCG with the learned preconditioner (K18).

namespace {

// r.z_new -> scal[S_RZ], r.z_old -> scal[S_AUX] (FP64), one pass.
__global__ void __launch_bounds__(kThreads)
    k_dot_pr(const float* __restrict__ r, const float* __restrict__ z,
             const float* __restrict__ zold, long N, double* partials,
             unsigned* counters, double* scal) {
    __shared__ double smem[32];
    AccF a, b;
    for (long c = blockIdx.x * (long)kThreads + threadIdx.x; c < N;
         c += (long)gridDim.x * kThreads) {
        const float rv = r[c];
        a.add(rv, z[c]);
        b.add(rv, zold[c]);
    }
    reduce_finish<kThreads>(a.value(), 5, S_RZ, FIN_NONE, partials, counters,
                            scal, smem);
    __syncthreads();
    reduce_finish<kThreads>(b.value(), 6, S_AUX, FIN_NONE, partials, counters,
                            scal, smem);
}

// Polak-Ribiere beta = r_k.(z_k - z_{k-1}) / (r_{k-1}.z_{k-1}); rolls r.z.
__global__ void k_pr_beta(double* scal, int first) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const double rz = scal[S_RZ], old = scal[S_RZ_OLD];
        scal[S_BETA] = (first || old == 0.0) ? 0.0 : (rz - scal[S_AUX]) / old;
        scal[S_RZ_OLD] = rz;
    }
}

__global__ void __launch_bounds__(kThreads)
    k_norm2f(const float* __restrict__ v, long N, double* partials,
             unsigned* counters, double* scal, int target) {
    __shared__ double smem[32];
    AccF acc;
    for (long c = blockIdx.x * (long)kThreads + threadIdx.x; c < N;
         c += (long)gridDim.x * kThreads)
        acc.add(v[c], v[c]);
    reduce_finish<kThreads>(acc.value(), 7, target, FIN_NONE, partials,
                            counters, scal, smem);
}

}  // namespace

jetgpu_status norm2f(Ctx* c, const float* r, long n, int target) {
    k_norm2f<<<rgrid(c, k_norm2f, n), kThreads, 0, c->stream>>>(
        r, n, c->partials, c->counters, c->scal, target);
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

namespace {

// fine += mask * (trilinear prolongation of coarse), k_correct's stencil and
// order, zero outside the fluid (phi >= 0).
__global__ void __launch_bounds__(kThreads)
    k_correct_masked(const float* __restrict__ coarse,
                     float* __restrict__ fine, const float* __restrict__ phi,
                     Dims c) {
    const Dims n{2 * c.x, 2 * c.y, 2 * c.z};
    const long N = n.count();
    for (long t = blockIdx.x * (long)kThreads + threadIdx.x; t < N;
         t += (long)gridDim.x * kThreads) {
        if (!(phi[t] < 0.0f)) continue;
        int i, j, k;
        cell_ijk(t, n, i, j, k);
        const int ci = i >> 1, cj = j >> 1, ck = k >> 1;
        int i0, i1, j0, j1, k0, k1;
        float wi0, wi1, wj0, wj1, wk0, wk1;
        if ((i & 1) == 0) { i0 = i > 1 ? ci - 1 : ci; i1 = ci; wi0 = 0.25f; wi1 = 0.75f; }
        else { i0 = ci; i1 = i + 1 < n.x ? ci + 1 : ci; wi0 = 0.75f; wi1 = 0.25f; }
        if ((j & 1) == 0) { j0 = j > 1 ? cj - 1 : cj; j1 = cj; wj0 = 0.25f; wj1 = 0.75f; }
        else { j0 = cj; j1 = j + 1 < n.y ? cj + 1 : cj; wj0 = 0.75f; wj1 = 0.25f; }
        if ((k & 1) == 0) { k0 = k > 1 ? ck - 1 : ck; k1 = ck; wk0 = 0.25f; wk1 = 0.75f; }
        else { k0 = ck; k1 = k + 1 < n.z ? ck + 1 : ck; wk0 = 0.75f; wk1 = 0.25f; }
        const float c000 = coarse[lin(i0, j0, k0, c.x, c.y)];
        const float c100 = coarse[lin(i1, j0, k0, c.x, c.y)];
        const float c010 = coarse[lin(i0, j1, k0, c.x, c.y)];
        const float c110 = coarse[lin(i1, j1, k0, c.x, c.y)];
        const float c001 = coarse[lin(i0, j0, k1, c.x, c.y)];
        const float c101 = coarse[lin(i1, j0, k1, c.x, c.y)];
        const float c011 = coarse[lin(i0, j1, k1, c.x, c.y)];
        const float c111 = coarse[lin(i1, j1, k1, c.x, c.y)];
        const float a0 = wj0 * (wi0 * c000 + wi1 * c100) + wj1 * (wi0 * c010 + wi1 * c110);
        const float a1 = wj0 * (wi0 * c001 + wi1 * c101) + wj1 * (wi0 * c011 + wi1 * c111);
        fine[t] += wk0 * a0 + wk1 * a1;
    }
}

// z += e (the network's output on the finest level is already masked).
__global__ void k_add_f32(float* __restrict__ z, const float* __restrict__ e,
                          long N) {
    for (long t = blockIdx.x * (long)kThreads + threadIdx.x; t < N;
         t += (long)gridDim.x * kThreads)
        z[t] += e[t];
}

}  // namespace

// The learned preconditioner (K18): one V-cycle, then the network's
// correction of the error the V-cycle leaves, computed on a coarse level
// from the residual it leaves:
//   z0 = V r,  rho = r - A z0,  z = z0 + mask P^k net(R^k rho)
// with the V-cycle's masked restriction R and trilinear prolongation P, and
// k = net_level(). The network is trained to minimise the A-norm of the
// error left after the correction, so z is at least as good a step as the
// V-cycle's wherever the training holds, and the V-cycle alone bounds how
// bad it can be. Uses the levels' V-cycle buffers as scratch.
jetgpu_status learned_precond(Ctx* c, const float* r, float* z) {
    const Level& L0 = c->levels[0];
    const long N = L0.n.count();
    const unsigned k = net_level(c);
    float* res = nullptr;
    jetgpu_status s = vcycle_graph(c, r, z, L0.x2, &res);
    if (s != JETGPU_OK) return s;
    if (res != z)
        JG_CUDA(c, cudaMemcpyAsync(z, res, N * sizeof(float),
                                   cudaMemcpyDeviceToDevice, c->stream));
    {
        Prof pr(c, K_RESIDUAL, 28.0 * N);
        const RowsF M{L0.A, N};
        if (L0.n.x % 4 == 0)
            k_residual32x4<<<grid_for(c, N / 4), kThreads, 0, c->stream>>>(
                M, z, r, L0.r, L0.n);
        else
            k_residual32<<<grid_for(c, N), kThreads, 0, c->stream>>>(
                M, z, r, L0.r, L0.n);
    }
    const float* rho = L0.r;
    for (unsigned l = 1; l <= k; ++l) {
        const Level& F = c->levels[l - 1];
        const Level& C = c->levels[l];
        Prof pr(c, K_RESTRICT, 4.0 * F.n.count() + 8.0 * C.n.count());
        if (C.n.x % 2 == 0)
            k_restrict2<<<grid_for(c, C.n.count() / 2), kThreads, 0,
                          c->stream>>>(rho, C.b, C.phi, C.n);
        else
            k_restrict<<<grid_for(c, C.n.count()), kThreads, 0, c->stream>>>(
                rho, C.b, C.phi, C.n);
        rho = C.b;
    }
    const Level& K = c->levels[k];
    if ((s = norm2f(c, rho, K.n.count(), S_MEAN)) != JETGPU_OK) return s;
    if ((s = net_apply(c, k, rho, c->scal + S_MEAN, K.x)) != JETGPU_OK)
        return s;
    Prof pr(c, K_CORRECT, 12.0 * N);
    if (k == 0) {
        k_add_f32<<<grid_for(c, N), kThreads, 0, c->stream>>>(z, K.x, N);
    } else {
        for (unsigned l = k - 1; l >= 1; --l) {
            const Level& F = c->levels[l];
            JG_CUDA(c, cudaMemsetAsync(F.x, 0, F.n.count() * sizeof(float),
                                       c->stream));
            k_correct<<<grid_for(c, F.n.count()), kThreads, 0, c->stream>>>(
                c->levels[l + 1].x, F.x, c->levels[l + 1].n);
        }
        k_correct_masked<<<grid_for(c, N), kThreads, 0, c->stream>>>(
            c->levels[1].x, z, L0.phi, c->levels[1].n);
    }
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

// FPCG on the FP32 rows for a correction e with A e = r (r = kr on entry,
// its squared norm in scal[S_R64]). Stops at ||r|| <= target, after max_it
// iterations, or when progress stalls (*stalled = true; x so far is kept).
static jetgpu_status fpcg_f32(Ctx* c, double target, unsigned max_it,
                              unsigned* it_out, double* rr_out,
                              bool* stalled) {
    const Level& L0 = c->levels[0];
    const Dims n = L0.n;
    const long N = n.count();
    RowsF M{L0.A, N};
    *stalled = false;
    k_init_scalars<<<1, 32, 0, c->stream>>>(c->scal);
    k_zero<float><<<grid_for(c, N), kThreads, 0, c->stream>>>(c->kz2, N);
    float* z = c->kz;
    float* zold = c->kz2;
    std::vector<double> hist;
    unsigned it = 0;
    double rr = 0;
    while (it < max_it) {
        if (jetgpu_status s = learned_precond(c, c->kr, z)) return s;
        {
            Prof pr(c, K_DOT_RZ, 12.0 * N);
            k_dot_pr<<<rgrid(c, k_dot_pr, N), kThreads, 0,
            c->stream>>>(c->kr, z, zold, N,
                                                    c->partials, c->counters,
                                                    c->scal);
        }
        k_pr_beta<<<1, 32, 0, c->stream>>>(c->scal, it == 0 ? 1 : 0);
        {
            Prof pr(c, K_UPDATE_D, 12.0 * N);
            k_update_d<float, float><<<rgrid(c, k_update_d<float, float>, N), kThreads, 0,
            c->stream>>>(c->kd, z,
                                                                    N, c->scal);
        }
        {
            Prof pr(c, K_SPMV, 24.0 * N);
            spmv_f32(c, M, n);
        }
        {
            Prof pr(c, K_UPDATE_XR, 24.0 * N);
            k_update_xr<float><<<rgrid(c, k_update_xr<float>, N), kThreads, 0,
            c->stream>>>(
                c->kx, c->kr, c->kd, c->kq, nullptr, N, c->partials,
                c->counters, c->scal);
        }
        std::swap(z, zold);
        ++it;
        jetgpu_status s = read_scalars(c);
        if (s != JETGPU_OK) return s;
        rr = c->h_scal[S_RR];
        const double rz = c->h_scal[S_RZ];
        if (!std::isfinite(rr) || !std::isfinite(rz) || rz <= 0.0) {
            // A non-positive r.z means the network is not acting as a
            // positive preconditioner here: stop and let multigrid finish.
            *stalled = true;
            break;
        }
        hist.push_back(std::sqrt(rr));
        if (std::sqrt(rr) <= target) break;
        const size_t k = hist.size();
        if (k >= 6 && hist[k - 1] > 0.8 * hist[k - 4]) {
            *stalled = true;
            break;
        }
    }
    if (*stalled && !std::isfinite(rr)) {
        // Discard a non-finite correction.
        k_zero<float><<<grid_for(c, N), kThreads, 0, c->stream>>>(c->kx, N);
    }
    *it_out = it;
    *rr_out = rr;
    return JETGPU_OK;
}

jetgpu_status harvest_pairs(Ctx* c, unsigned max_pairs, float* r_out,
                            float* z_out, unsigned* count) {
    const Level& L0 = c->levels[0];
    const Dims n = L0.n;
    const long N = n.count();
    RowsF M{L0.A, N};
    // r = b (x = 0), FP32 image.
    k_zero<double><<<grid_for(c, N), kThreads, 0, c->stream>>>(c->x64, N);
    k_residual64<<<rgrid(c, k_residual64, N), kThreads, 0,
            c->stream>>>(
        c->A64, c->x64, c->b64, c->r64, c->kr, c->kx, n, c->partials,
        c->counters, c->scal, S_R64);
    k_init_scalars<<<1, 32, 0, c->stream>>>(c->scal);
    unsigned k = 0;
    for (; k < max_pairs; ++k) {
        float* z = nullptr;
        if (jetgpu_status vs = vcycle(c, c->kr, c->kz, L0.x2, &z)) return vs;
        JG_CUDA(c, cudaMemcpyAsync(r_out + (size_t)k * N, c->kr, N * sizeof(float),
                                   cudaMemcpyDeviceToDevice, c->stream));
        JG_CUDA(c, cudaMemcpyAsync(z_out + (size_t)k * N, z, N * sizeof(float),
                                   cudaMemcpyDeviceToDevice, c->stream));
        k_dot_rz<float, float><<<rgrid(c, k_dot_rz<float, float>, N), kThreads, 0,
            c->stream>>>(
            c->kr, z, N, c->partials, c->counters, c->scal);
        k_update_d<float, float><<<rgrid(c, k_update_d<float, float>, N), kThreads, 0,
            c->stream>>>(c->kd, z, N,
                                                                c->scal);
        spmv_f32(c, M, n);
        k_update_xr<float><<<rgrid(c, k_update_xr<float>, N), kThreads, 0,
            c->stream>>>(
            c->kx, c->kr, c->kd, c->kq, nullptr, N, c->partials, c->counters,
            c->scal);
    }
    JG_CUDA(c, cudaStreamSynchronize(c->stream));
    *count = k;
    return JETGPU_OK;
}

jetgpu_status mgpcg_solve(Ctx* c, jetgpu_solve_stats* st) {
    const Level& L0 = c->levels[0];
    const Dims n = L0.n;
    const long N = n.count();
    const jetgpu_config& cfg = c->cfg;
    const bool fp64 = (cfg.precision == JETGPU_PRECISION_FP64);

    // FP64 mode: x64 = 0 and ||b|| in FP64. FP32 modes: the double-float
    // start (r = b, x = 0, ||b||) in one pass.
    if (fp64) {
        k_norm2<<<rgrid(c, k_norm2, N), kThreads, 0,
            c->stream>>>(c->b64, N, c->partials,
                                               c->counters, c->scal, S_B64);
        k_zero<double><<<grid_for(c, N), kThreads, 0, c->stream>>>(c->x64, N);
    } else {
        Prof pr(c, K_RESIDUAL64, 24.0 * N);
        k_start_df<<<rgrid(c, k_start_df, N), kThreads, 0,
            c->stream>>>(c->bdf, c->kr, c->kx, c->xdf,
                                                  N, c->partials, c->counters,
                                                  c->scal);
    }
    jetgpu_status s = read_scalars(c);
    if (s != JETGPU_OK) return s;
    const double bnorm = std::sqrt(c->h_scal[fp64 ? S_B64 : S_R64]);
    if (!std::isfinite(bnorm))
        return fail(c, JETGPU_NUMERICAL_ERROR, "non-finite right-hand side");
    st->b_norm = bnorm;
    st->iterations = 0;
    st->refinements = 0;
    st->residual = 0.0;
    st->relative_residual = 0.0;
    // The FP64 solution of the FP32 modes (from the double-float iterate).
    auto finish_x = [&]() -> jetgpu_status {
        if (!fp64) {
            Prof pr(c, K_ACCUMULATE, 16.0 * N);
            k_df_to_f64<<<grid_for(c, N), kThreads, 0, c->stream>>>(c->xdf,
                                                                    c->x64, N);
            JG_CUDA(c, cudaGetLastError());
        }
        return JETGPU_OK;
    };
    if (bnorm == 0.0) {
        if (fp64) return JETGPU_OK;
        return finish_x();
    }

    const bool learned = cfg.preconditioner == JETGPU_PRECOND_LEARNED;
    if (learned && (fp64 || !net_supported(c)))
        return fail(c, JETGPU_BAD_INPUT,
                    "learned preconditioner needs a loaded network, FP32 "
                    "Krylov vectors and a resolution divisible by 8");
    bool fell_back = false;
    const double goal = cfg.tolerance * bnorm;
    double rnorm = bnorm;
    unsigned total = 0;
    const unsigned max_pass = cfg.max_refinements > 0 ? cfg.max_refinements : 1;
    // True residual b - A x (FP64 rows): FP64 in FP64 mode, double-float in
    // the FP32 modes; its FP32 image feeds the next correction solve.
    auto true_residual = [&](float* r32, float* zero32) -> jetgpu_status {
        if (fp64) {
            Prof pr(c, K_RESIDUAL64, 60.0 * N);
            k_residual64<<<rgrid(c, k_residual64, N), kThreads, 0,
            c->stream>>>(
                c->A64, c->x64, c->b64, c->r64, r32, zero32, n, c->partials,
                c->counters, c->scal, S_R64);
        } else {
            Prof pr(c, K_RESIDUAL64, 56.0 * N);
            if (n.x % 4 == 0)
                k_residual_df4<<<rgrid(c, k_residual_df4, N / 4), kThreads, 0,
                                 c->stream>>>(
                    RowsF{L0.A, N}, c->Alo, c->xdf, c->bdf, r32, zero32, n,
                    c->partials, c->counters, c->scal, S_R64);
            else
                k_residual_df<<<rgrid(c, k_residual_df, N), kThreads, 0,
                                c->stream>>>(
                    RowsF{L0.A, N}, c->Alo, c->xdf, c->bdf, r32, zero32, n,
                    c->partials, c->counters, c->scal, S_R64);
        }
        JG_CUDA(c, cudaGetLastError());
        jetgpu_status rs = read_scalars(c);
        if (rs != JETGPU_OK) return rs;
        rnorm = std::sqrt(c->h_scal[S_R64]);
        st->residual = rnorm;
        st->relative_residual = rnorm / bnorm;
        if (!std::isfinite(rnorm))
            return fail(c, JETGPU_NUMERICAL_ERROR, "non-finite residual");
        return JETGPU_OK;
    };
    for (unsigned pass = 0; pass < max_pass && total < cfg.max_cg_iter;
         ++pass) {
        if (fp64 || pass > 0) {
            s = true_residual(fp64 ? L0.b : c->kr, fp64 ? nullptr : c->kx);
            if (s != JETGPU_OK) return s;
        } else {
            st->residual = rnorm;
            st->relative_residual = 1.0;
        }
        if (rnorm <= goal) break;
        st->refinements = pass + 1;
        unsigned it = 0;
        double rr = 0;
        if (fp64) {
            s = pcg_f64(c, goal * 0.9, cfg.max_cg_iter - total, &it, &rr);
        } else {
            // Inner FP32 solve to a relative reduction the FP32 operator can
            // deliver; the refinement loop does the rest. Once the goal is
            // within reach, the inner target sits just below it: the FP32
            // recurrence residual of a correction solve tracks the true
            // residual closely (the correction is small, so the FP32 rows'
            // rounding hardly shows), and a larger safety margin costs a
            // whole extra iteration (each one cuts the residual about 10x).
            double eta = 0.9 * goal / rnorm;
            if (eta < 1e-4) eta = 1e-4;
            if (learned && !fell_back) {
                bool stalled = false;
                s = fpcg_f32(c, eta * rnorm, cfg.max_cg_iter - total, &it, &rr,
                             &stalled);
                if (stalled) {
                    fell_back = true;
                    st->fallback_used = 1;
                }
            } else {
                s = pcg_f32(c, eta * rnorm, cfg.max_cg_iter - total, &it, &rr);
            }
            if (s == JETGPU_OK) {
                Prof pr(c, K_ACCUMULATE, 20.0 * N);
                k_accumulate_df<<<grid_for(c, N), kThreads, 0, c->stream>>>(
                    c->xdf, c->kx, N);
            }
        }
        if (s != JETGPU_OK) return s;
        total += it;
        st->iterations = total;
    }
    if (st->relative_residual > cfg.tolerance) {
        // Final check after the last pass.
        s = true_residual(fp64 ? nullptr : c->kr, fp64 ? nullptr : c->kx);
        if (s != JETGPU_OK) return s;
        if (rnorm > goal) {
            jetgpu_status fs = finish_x();
            if (fs != JETGPU_OK) return fs;
            return fail(c, JETGPU_NOT_CONVERGED,
                        "tolerance not reached within the iteration cap");
        }
    }
    s = finish_x();
    if (s != JETGPU_OK) return s;
    return fell_back ? JETGPU_STALLED_FALLBACK_USED : JETGPU_OK;
}

}  // namespace jg

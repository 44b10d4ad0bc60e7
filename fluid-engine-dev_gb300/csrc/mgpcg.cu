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
//     cell, V-cycle in FP32; every global reduction is FP64, deterministic
//     (fixed grid, per-block partials summed in block order by the last block
//     to finish; no block ever waits on another).
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

#include <chrono>
#include <cmath>
#include <cstring>

namespace jg {
namespace {

enum Fin : int { FIN_NONE = 0, FIN_BETA = 1, FIN_ALPHA = 2 };
enum : int { S_ALPHA = 8, S_BETA = 9, S_FIRST = 10 };

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

struct RowsF {
    const float4* A;
    __device__ __forceinline__ float4 row(long c) const { return A[c]; }
};
struct RowsD {
    const double* A;
    __device__ __forceinline__ double4 row(long c) const {
        const double2 a = reinterpret_cast<const double2*>(A)[2 * c];
        const double2 b = reinterpret_cast<const double2*>(A)[2 * c + 1];
        return make_double4(a.x, a.y, b.x, b.y);
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

// K5: q = A d and d.q (FP64).
template <typename V, typename Rows>
__global__ void __launch_bounds__(kThreads)
    k_spmv_dot(Rows M, const V* __restrict__ d, V* __restrict__ q, Dims n,
               double* partials, unsigned* counters, double* scal) {
    __shared__ double smem[32];
    const long N = n.count();
    double acc = 0.0;
    for (long c = blockIdx.x * (long)kThreads + threadIdx.x; c < N;
         c += (long)gridDim.x * kThreads) {
        int i, j, k;
        cell_ijk(c, n, i, j, k);
        const V qv = apply7<V>(M, d, c, i, j, k, n);
        q[c] = qv;
        acc += (double)d[c] * (double)qv;
    }
    reduce_finish<kThreads>(acc, 0, S_DQ, FIN_ALPHA, partials, counters, scal,
                            smem);
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
    double acc = 0.0;
    for (long c = blockIdx.x * (long)kThreads + threadIdx.x; c < N;
         c += (long)gridDim.x * kThreads) {
        x[c] += alpha * d[c];
        const V rv = r[c] - alpha * q[c];
        r[c] = rv;
        if (r32) r32[c] = (float)rv;
        acc += (double)rv * (double)rv;
    }
    reduce_finish<kThreads>(acc, 1, S_RR, FIN_NONE, partials, counters, scal,
                            smem);
}

// K7b: r.z (FP64), finishing beta.
template <typename V, typename Z>
__global__ void __launch_bounds__(kThreads)
    k_dot_rz(const V* __restrict__ r, const Z* __restrict__ z, long N,
             double* partials, unsigned* counters, double* scal) {
    __shared__ double smem[32];
    double acc = 0.0;
    for (long c = blockIdx.x * (long)kThreads + threadIdx.x; c < N;
         c += (long)gridDim.x * kThreads)
        acc += (double)r[c] * (double)z[c];
    reduce_finish<kThreads>(acc, 2, S_RZ, FIN_BETA, partials, counters, scal,
                            smem);
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

// x64 += e (FP32 correction).
__global__ void k_accumulate(double* __restrict__ x, const float* __restrict__ e,
                             long N) {
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x)
        x[c] += (double)e[c];
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
template <bool ZERO>
__global__ void __launch_bounds__(kThreads)
    k_rb_half(const float4* __restrict__ A, const float* __restrict__ b,
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
                const float4 r = A[c];
                x[c] = omega * b[c] / r.x;
            }
            const int io = 2 * p + (off ^ 1);
            if (io < n.x) x[base + (off ^ 1)] = 0.0f;
        } else {
            if (i >= n.x) continue;
            const long c = base + off;
            const float4 r = A[c];
            float s = 0.0f;
            if (i > 0) s += A[c - 1].y * x[c - 1];
            if (i + 1 < n.x) s += r.y * x[c + 1];
            if (j > 0) s += A[c - sy].z * x[c - sy];
            if (j + 1 < n.y) s += r.z * x[c + sy];
            if (k > 0) s += A[c - sz].w * x[c - sz];
            if (k + 1 < n.z) s += r.w * x[c + sz];
            x[c] = (1.0f - omega) * x[c] + omega * (b[c] - s) / r.x;
        }
    }
}

// K8 (fused): one full red-black SOR sweep in a single pass over memory.
//
// A block owns a 64 x 8 (i, j) tile and marches through a slab of k planes
// (2.5-D blocking). x is read from `xin` and the swept x written to `xout`
// (ping-pong), so blocks never see each other's updates: each block redoes
// the first-colour update on a one-cell ring around its tile, from old
// values, exactly as the sequential sweep would produce them. Per plane the
// block stages x with a two-cell ring, the matrix rows and b with cp.async
// 16-byte copies (zero-filled outside the domain), then
//   (1) updates the first colour of plane t+1 on tile + ring (in shared
//       memory; the 7-point neighbours of a cell all have the other colour),
//   (2) updates the second colour of plane t on the tile, reading first-
//       colour values of planes t-1, t, t+1 that (1) produced, and writes
//       both colours of plane t to global memory as one float2 per thread.
// HBM traffic per sweep: x, b and A read once, x written once — 28 B/cell —
// plus ring re-reads that mostly hit L2. Requires nx % 4 == 0.
namespace fused {
constexpr int TX = 64, TY = 8;          // tile (cells)
constexpr int SX = TX + 8, SY = TY + 4; // staged plane: i0-4 .. i0+67, j0-2 .. j0+9
constexpr int PLANE = SX * SY;          // 864 cells
// Ring depths (planes): in use at step t are x t-1..t+2, A t-1..t+1 and
// b t..t+1; PD more slots each hold the prefetches for steps t+1..t+PD, so
// every block keeps PD planes of loads in flight while it computes.
constexpr int PD = 2;
constexpr int XS = 4 + PD, AS = 3 + PD, BS = 2 + PD;
constexpr size_t SMEM = (size_t)PLANE * (XS * 4 + AS * 16 + BS * 4);

__device__ __forceinline__ int ring(int p, int m) { return ((p % m) + m) % m; }

__device__ __forceinline__ void cp16(void* smem, const void* gmem, bool valid) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    const int src = valid ? 16 : 0;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s),
                 "l"(gmem), "r"(src));
}
__device__ __forceinline__ void cp_commit() {
    asm volatile("cp.async.commit_group;\n" ::);
}
// Waits until at most `pending` committed groups are still in flight.
template <int pending>
__device__ __forceinline__ void cp_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(pending));
}
}  // namespace fused

__global__ void __launch_bounds__(256)
    k_rb_sweep_fused(const float4* __restrict__ A, const float* __restrict__ b,
                     const float* __restrict__ xin, float* __restrict__ xout,
                     Dims n, int first, float omega, int kz) {
    using namespace fused;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* sx = reinterpret_cast<float*>(smem_raw);               // XS planes
    float4* sA = reinterpret_cast<float4*>(sx + XS * PLANE);      // AS planes
    float* sb = reinterpret_cast<float*>(sA + AS * PLANE);        // BS planes
    const int tid = threadIdx.x;
    const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
    const int k0 = blockIdx.z * kz;
    const int k1 = min(n.z, k0 + kz);
    const long sy = n.x, sz = (long)n.x * n.y;
    const int second = first ^ 1;

    // Per-thread copy descriptors. The in-plane offsets of a thread's 16-byte
    // chunks are the same for every plane, so their index arithmetic is done
    // once here; a plane load only adds the plane base.
    // x and b: PLANE/4 = 216 chunks of 4 floats, one per thread below 216.
    int vgo = 0, vso = 0;
    bool vok = false;
    if (tid < PLANE / 4) {
        const int r = tid / (SX / 4), c4 = tid - r * (SX / 4);
        const int gi = i0 - 4 + 4 * c4, gj = j0 - 2 + r;
        vok = gi >= 0 && gi < n.x && gj >= 0 && gj < n.y;
        vgo = vok ? gi + n.x * gj : 0;
        vso = r * SX + 4 * c4;
    }
    // A: PLANE rows of 16 bytes, up to AM per thread.
    constexpr int AM = (PLANE + 255) / 256;
    int ago[AM];
    bool aok[AM];
#pragma unroll
    for (int m = 0; m < AM; ++m) {
        const int f = tid + 256 * m;
        const int r = f / SX, c = f - r * SX;
        const int gi = i0 - 4 + c, gj = j0 - 2 + r;
        aok[m] = f < PLANE && gi >= 0 && gi < n.x && gj >= 0 && gj < n.y;
        ago[m] = aok[m] ? gi + n.x * gj : 0;
    }

    // Stage plane p of x / A / b (zero-filled outside the domain, so the
    // update below needs no bounds tests: an outside neighbour has x = 0 and
    // a zero matrix row, exactly the reference's guarded terms,
    // FdmBlas3::mvm, fdm_linear_system3.cpp:79-96).
    auto load_x = [&](int p) {
        float* dst = sx + ring(p, XS) * PLANE;
        if (xin == nullptr || p < 0 || p >= n.z) {
            for (int q = tid; q < PLANE; q += 256) dst[q] = 0.0f;
            return;
        }
        if (tid < PLANE / 4) {
            const float* base = xin + sz * p;
            cp16(dst + vso, vok ? base + vgo : xin, vok);
        }
    };
    auto load_A = [&](int p) {
        float4* dst = sA + ring(p, AS) * PLANE;
        const bool pin = p >= 0 && p < n.z;
        const float4* base = A + (pin ? sz * p : 0);
#pragma unroll
        for (int m = 0; m < AM; ++m) {
            const int f = tid + 256 * m;
            if (f < PLANE) cp16(dst + f, base + ago[m], pin && aok[m]);
        }
    };
    auto load_b = [&](int p) {
        float* dst = sb + ring(p, BS) * PLANE;
        const bool pin = p >= 0 && p < n.z;
        if (tid < PLANE / 4) {
            const float* base = b + (pin ? sz * p : 0);
            cp16(dst + vso, base + vgo, pin && vok);
        }
    };
    // SOR update at staged index s: xc/Ac/bc this plane, xdn/Adn the plane
    // below, xup the plane above.
    auto relax = [&](const float* xc, const float* xdn, const float* xup,
                     const float4* Ac, const float4* Adn, const float* bc,
                     int s) -> float {
        const float4 row = Ac[s];
        const float acc = Ac[s - 1].y * xc[s - 1] + row.y * xc[s + 1] +
                          Ac[s - SX].z * xc[s - SX] + row.z * xc[s + SX] +
                          Adn[s].w * xdn[s] + row.w * xup[s];
        return (1.0f - omega) * xc[s] + omega * __fdividef(bc[s] - acc, row.x);
    };

    // Step t needs x planes t..t+2, A planes t..t+1 and b plane t+1 staged.
    // Group g holds the loads of step t0+g; groups for steps t+1..t+PD are
    // in flight while step t computes (empty groups keep the count uniform).
    const int t0 = k0 - 2;
    load_x(t0);
    load_x(t0 + 1);
    load_A(t0);
    for (int q = 0; q < PD; ++q) {
        if (t0 + q < k1) {
            load_x(t0 + q + 2);
            load_A(t0 + q + 1);
            load_b(t0 + q + 1);
        }
        fused::cp_commit();
    }
    for (int t = t0; t < k1; ++t) {
        if (t + PD < k1) {
            load_x(t + PD + 2);
            load_A(t + PD + 1);
            load_b(t + PD + 1);
        }
        fused::cp_commit();
        fused::cp_wait<PD>();
        __syncthreads();
        // Slot pointers of the planes this step touches.
        float* xm1 = sx + ring(t - 1, XS) * PLANE;
        float* x0 = sx + ring(t, XS) * PLANE;
        float* x1 = sx + ring(t + 1, XS) * PLANE;
        const float* x2 = sx + ring(t + 2, XS) * PLANE;
        const float4* am1 = sA + ring(t - 1, AS) * PLANE;
        const float4* a0 = sA + ring(t, AS) * PLANE;
        const float4* a1 = sA + ring(t + 1, AS) * PLANE;
        const float* b0 = sb + ring(t, BS) * PLANE;
        const float* b1 = sb + ring(t + 1, BS) * PLANE;
        // (1) first colour of plane t+1 on tile + 1-cell ring.
        const int p1 = t + 1;
        if (p1 >= k0 - 1 && p1 <= k1 && p1 >= 0 && p1 < n.z) {
            const int par = (first - p1 + 1) & 1;
            for (int q = tid; q < 33 * (TY + 2); q += 256) {
                const int row = q / 33;
                const int jj = row - 1;
                const int ii = -1 + 2 * (q - 33 * row) + ((par - jj) & 1);
                const int gi = i0 + ii, gj = j0 + jj;
                if (gi < 0 || gi >= n.x || gj < 0 || gj >= n.y) continue;
                const int s = (jj + 2) * SX + (ii + 4);
                x1[s] = relax(x1, x0, x2, a1, a0, b1, s);
            }
        }
        __syncthreads();
        // (2) second colour of plane t on the tile; write plane t.
        if (t >= k0) {
            const int tx = tid & 31, ty = tid >> 5;
            const int ii = 2 * tx, jj = ty;
            const int gi = i0 + ii, gj = j0 + jj;
            if (gi < n.x && gj < n.y) {
                const int odd = ((ii + jj + t) & 1) != second;  // S cell at ii+odd
                const float* xp = x0;
                const int s = (jj + 2) * SX + (ii + 4);
                float2 out;
                const float vs = relax(x0, xm1, x1, a0, am1, b0, s + odd);
                if (odd) {
                    out.x = xp[s];
                    out.y = vs;
                } else {
                    out.x = vs;
                    out.y = xp[s + 1];
                }
                *reinterpret_cast<float2*>(xout + gi + sy * gj + sz * t) = out;
            }
        }
        __syncthreads();
    }
}

// K9a: r = b - A x (FP32).
__global__ void __launch_bounds__(kThreads)
    k_residual32(const float4* __restrict__ A, const float* __restrict__ x,
                 const float* __restrict__ b, float* __restrict__ r, Dims n) {
    const long N = n.count();
    RowsF M{A};
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

// K11: coarsest level in one CTA: x and b in shared memory, `sweeps`
// forward red-black sweeps followed by `sweeps` sweeps in reverse colour
// order (symmetric), starting from x = 0.
constexpr int kCoarsestMaxCells = 4096;
__global__ void __launch_bounds__(1024)
    k_coarsest(const float4* __restrict__ A, const float* __restrict__ b,
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
                const float4 r = A[c];
                float s = 0.0f;
                if (i > 0) s += A[c - 1].y * sx[c - 1];
                if (i + 1 < n.x) s += r.y * sx[c + 1];
                if (j > 0) s += A[c - sy].z * sx[c - sy];
                if (j + 1 < n.y) s += r.z * sx[c + sy];
                if (k > 0) s += A[c - sz].w * sx[c - sz];
                if (k + 1 < n.z) s += r.w * sx[c + sz];
                sx[c] = (1.0f - omega) * sx[c] + omega * (sb[c] - s) / r.x;
            }
            __syncthreads();
        }
    }
    for (int c = threadIdx.x; c < N; c += blockDim.x) x[c] = sx[c];
}

// ---------------------------------------------------------------------------

int grid_for(const Ctx* c, long work) {
    int cap = c->num_sms * 8;
    return blocks_for(work, kThreads, cap);
}

void rb_half(Ctx* c, const Level& L, const float* b, float* x, int color,
             bool zero, int cls) {
    const long pairs = (long)((L.n.x + 1) / 2) * L.n.y * L.n.z;
    const float w = (float)c->cfg.sor;
    Prof pr(c, cls, 14.0 * L.n.count());
    if (zero)
        k_rb_half<true><<<grid_for(c, pairs), kThreads, 0, c->stream>>>(
            L.A, b, x, L.n, color, w);
    else
        k_rb_half<false><<<grid_for(c, pairs), kThreads, 0, c->stream>>>(
            L.A, b, x, L.n, color, w);
}

bool fused_ok(const Level& L) {
    return L.n.x % 4 == 0 && L.n.x >= 64 && L.n.y >= 8 && L.n.z >= 2;
}

// Slab depth of the fused sweep: about two waves of resident blocks.
int fused_kz(const Ctx* c, const Level& L) {
    const long tiles = (long)((L.n.x + fused::TX - 1) / fused::TX) *
                       ((L.n.y + fused::TY - 1) / fused::TY);
    const long resident = (long)c->num_sms * 2;
    long kz = (long)L.n.z * tiles / (2 * resident);
    if (kz < 8) kz = 8;
    if (kz > 64) kz = 64;
    if (kz > L.n.z) kz = L.n.z;
    return (int)kz;
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
    if (alt != nullptr && fused_ok(L)) {
        const int kz = fused_kz(c, L);
        dim3 grid((L.n.x + fused::TX - 1) / fused::TX,
                  (L.n.y + fused::TY - 1) / fused::TY, (L.n.z + kz - 1) / kz);
        float* cur = x;
        float* oth = alt;
        for (unsigned s = 0; s < sweeps; ++s) {
            const bool z0 = zero && s == 0;
            Prof pr(c, l == 0 ? K_SWEEP_L0 : K_SWEEP_COARSE,
                    (z0 ? 24.0 : 28.0) * L.n.count());
            k_rb_sweep_fused<<<grid, 256, fused::SMEM, c->stream>>>(
                L.A, b, z0 ? nullptr : cur, oth, L.n, first, (float)c->cfg.sor,
                kz);
            std::swap(cur, oth);
        }
        return cur;
    }
    const int cls = l == 0 ? K_HALF_L0 : K_HALF_COARSE;
    for (unsigned s = 0; s < sweeps; ++s) {
        rb_half(c, L, b, x, first, zero && s == 0, cls);
        rb_half(c, L, b, x, 1 - first, false, cls);
    }
    return x;
}

// Symmetric V-cycle on level l from a zero initial guess; returns the
// buffer (x or alt) that holds the result.
float* vcycle_level(Ctx* c, unsigned l, const float* b, float* x, float* alt) {
    const Level& L = c->levels[l];
    const unsigned nl = c->built_levels;
    const jetgpu_config& cfg = c->cfg;
    if (l + 1 == nl) {
        if (L.n.count() <= kCoarsestMaxCells) {
            int nt = (int)std::min<long>(1024, ((L.n.count() + 31) / 32) * 32);
            Prof pr(c, K_COARSEST, 28.0 * L.n.count());
            k_coarsest<<<1, nt, 0, c->stream>>>(L.A, b, x, L.n,
                                                (int)cfg.coarsest_iter,
                                                (float)cfg.sor);
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
        Prof pr(c, K_RESIDUAL, 28.0 * L.n.count());
        k_residual32<<<grid_for(c, L.n.count()), kThreads, 0, c->stream>>>(
            L.A, cur, b, L.r, L.n);
    }
    {
        Prof pr(c, K_RESTRICT, 4.0 * L.n.count() + 8.0 * C.n.count());
        k_restrict<<<grid_for(c, C.n.count()), kThreads, 0, c->stream>>>(
            L.r, C.b, C.phi, C.n);
    }
    const float* xc = vcycle_level(c, l + 1, C.b, C.x, C.x2);
    {
        Prof pr(c, K_CORRECT, 8.0 * L.n.count() + 4.0 * C.n.count());
        k_correct<<<grid_for(c, L.n.count()), kThreads, 0, c->stream>>>(
            xc, cur, C.n);
    }
    return smooth(c, L, b, cur, other,
                  l == 0 ? cfg.final_iter : cfg.correct_iter, true, false, l);
}

double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(
               steady_clock::now().time_since_epoch())
        .count();
}

jetgpu_status read_scalars(Ctx* c) {
    JG_CUDA(c, cudaMemcpyAsync(c->h_scal, c->scal, S_COUNT * sizeof(double),
                               cudaMemcpyDeviceToHost, c->stream));
    JG_CUDA(c, cudaStreamSynchronize(c->stream));
    return JETGPU_OK;
}

}  // namespace

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

jetgpu_status prepare_levels(Ctx* c) {
    (void)c;
    return JETGPU_OK;
}

jetgpu_status init_kernels(Ctx* c) {
    JG_CUDA(c, cudaFuncSetAttribute(k_rb_sweep_fused,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)fused::SMEM));
    return JETGPU_OK;
}

// PCG on the FP32 rows for a correction e with A e = r (r = kr on entry).
// Stops when ||r_k|| <= target or after max_it iterations.
static jetgpu_status pcg_f32(Ctx* c, double target, unsigned max_it,
                             unsigned* it_out, double* rr_out) {
    const Level& L0 = c->levels[0];
    const Dims n = L0.n;
    const long N = n.count();
    const int G = red_blocks(c, N);
    RowsF M{L0.A};
    k_init_scalars<<<1, 32, 0, c->stream>>>(c->scal);
    unsigned it = 0;
    double rr = 0;
    while (it < max_it) {
        float* z = nullptr;
        if (c->cfg.preconditioner == JETGPU_PRECOND_NONE) {
            z = c->kr;  // plain CG: z = r
        } else if (jetgpu_status vs = vcycle(c, c->kr, c->kz, L0.x2, &z)) {
            return vs;
        }
        {
            Prof pr(c, K_DOT_RZ, 8.0 * N);
            k_dot_rz<float, float><<<G, kThreads, 0, c->stream>>>(
                c->kr, z, N, c->partials, c->counters, c->scal);
        }
        {
            Prof pr(c, K_UPDATE_D, 12.0 * N);
            k_update_d<float, float><<<G, kThreads, 0, c->stream>>>(c->kd, z,
                                                                    N, c->scal);
        }
        {
            Prof pr(c, K_SPMV, 24.0 * N);
            k_spmv_dot<float, RowsF><<<G, kThreads, 0, c->stream>>>(
                M, c->kd, c->kq, n, c->partials, c->counters, c->scal);
        }
        {
            Prof pr(c, K_UPDATE_XR, 24.0 * N);
            k_update_xr<float><<<G, kThreads, 0, c->stream>>>(
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
    const int G = red_blocks(c, N);
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
            k_dot_rz<double, float><<<G, kThreads, 0, c->stream>>>(
                c->r64, z, N, c->partials, c->counters, c->scal);
        }
        {
            Prof pr(c, K_UPDATE_D, 20.0 * N);
            k_update_d<double, float><<<G, kThreads, 0, c->stream>>>(
                c->dd, z, N, c->scal);
        }
        {
            Prof pr(c, K_SPMV, 48.0 * N);
            k_spmv_dot<double, RowsD><<<G, kThreads, 0, c->stream>>>(
                M, c->dd, c->dq, n, c->partials, c->counters, c->scal);
        }
        {
            Prof pr(c, K_UPDATE_XR, 52.0 * N);
            k_update_xr<double><<<G, kThreads, 0, c->stream>>>(
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
    double a = 0.0, b = 0.0;
    for (long c = blockIdx.x * (long)kThreads + threadIdx.x; c < N;
         c += (long)gridDim.x * kThreads) {
        const double rv = r[c];
        a += rv * (double)z[c];
        b += rv * (double)zold[c];
    }
    reduce_finish<kThreads>(a, 5, S_RZ, FIN_NONE, partials, counters, scal,
                            smem);
    __syncthreads();
    reduce_finish<kThreads>(b, 6, S_AUX, FIN_NONE, partials, counters, scal,
                            smem);
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
    double acc = 0.0;
    for (long c = blockIdx.x * (long)kThreads + threadIdx.x; c < N;
         c += (long)gridDim.x * kThreads)
        acc += (double)v[c] * (double)v[c];
    reduce_finish<kThreads>(acc, 7, target, FIN_NONE, partials, counters,
                            scal, smem);
}

}  // namespace

jetgpu_status norm2f(Ctx* c, const float* r, long n, int target) {
    k_norm2f<<<red_blocks(c, n), kThreads, 0, c->stream>>>(
        r, n, c->partials, c->counters, c->scal, target);
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
    const int G = red_blocks(c, N);
    RowsF M{L0.A};
    *stalled = false;
    k_init_scalars<<<1, 32, 0, c->stream>>>(c->scal);
    k_zero<float><<<grid_for(c, N), kThreads, 0, c->stream>>>(c->kz2, N);
    float* z = c->kz;
    float* zold = c->kz2;
    std::vector<double> hist;
    unsigned it = 0;
    double rr = 0;
    while (it < max_it) {
        const double* rrp = c->scal + (it == 0 ? S_R64 : S_RR);
        if (jetgpu_status s = net_apply(c, c->kr, rrp, z)) return s;
        {
            Prof pr(c, K_DOT_RZ, 12.0 * N);
            k_dot_pr<<<G, kThreads, 0, c->stream>>>(c->kr, z, zold, N,
                                                    c->partials, c->counters,
                                                    c->scal);
        }
        k_pr_beta<<<1, 32, 0, c->stream>>>(c->scal, it == 0 ? 1 : 0);
        {
            Prof pr(c, K_UPDATE_D, 12.0 * N);
            k_update_d<float, float><<<G, kThreads, 0, c->stream>>>(c->kd, z,
                                                                    N, c->scal);
        }
        {
            Prof pr(c, K_SPMV, 24.0 * N);
            k_spmv_dot<float, RowsF><<<G, kThreads, 0, c->stream>>>(
                M, c->kd, c->kq, n, c->partials, c->counters, c->scal);
        }
        {
            Prof pr(c, K_UPDATE_XR, 24.0 * N);
            k_update_xr<float><<<G, kThreads, 0, c->stream>>>(
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
    const int G = red_blocks(c, N);
    RowsF M{L0.A};
    // r = b (x = 0), FP32 image.
    k_zero<double><<<grid_for(c, N), kThreads, 0, c->stream>>>(c->x64, N);
    k_residual64<<<G, kThreads, 0, c->stream>>>(
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
        k_dot_rz<float, float><<<G, kThreads, 0, c->stream>>>(
            c->kr, z, N, c->partials, c->counters, c->scal);
        k_update_d<float, float><<<G, kThreads, 0, c->stream>>>(c->kd, z, N,
                                                                c->scal);
        k_spmv_dot<float, RowsF><<<G, kThreads, 0, c->stream>>>(
            M, c->kd, c->kq, n, c->partials, c->counters, c->scal);
        k_update_xr<float><<<G, kThreads, 0, c->stream>>>(
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
    const int G = red_blocks(c, N);
    const jetgpu_config& cfg = c->cfg;
    const bool fp64 = (cfg.precision == JETGPU_PRECISION_FP64);

    // ||b||, x64 = 0.
    k_norm2<<<G, kThreads, 0, c->stream>>>(c->b64, N, c->partials,
                                           c->counters, c->scal, S_B64);
    k_zero<double><<<grid_for(c, N), kThreads, 0, c->stream>>>(c->x64, N);
    jetgpu_status s = read_scalars(c);
    if (s != JETGPU_OK) return s;
    const double bnorm = std::sqrt(c->h_scal[S_B64]);
    if (!std::isfinite(bnorm))
        return fail(c, JETGPU_NUMERICAL_ERROR, "non-finite right-hand side");
    st->b_norm = bnorm;
    st->iterations = 0;
    st->refinements = 0;
    st->residual = 0.0;
    st->relative_residual = 0.0;
    if (bnorm == 0.0) return JETGPU_OK;

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
    for (unsigned pass = 0; pass < max_pass && total < cfg.max_cg_iter;
         ++pass) {
        // True FP64 residual r64 = b - A x64 (and its FP32 image).
        float* r32 = fp64 ? L0.b : c->kr;
        {
            Prof pr(c, K_RESIDUAL64, 60.0 * N);
            k_residual64<<<G, kThreads, 0, c->stream>>>(
                c->A64, c->x64, c->b64, c->r64, r32, fp64 ? nullptr : c->kx,
                n, c->partials, c->counters, c->scal, S_R64);
        }
        s = read_scalars(c);
        if (s != JETGPU_OK) return s;
        rnorm = std::sqrt(c->h_scal[S_R64]);
        st->residual = rnorm;
        st->relative_residual = rnorm / bnorm;
        if (!std::isfinite(rnorm))
            return fail(c, JETGPU_NUMERICAL_ERROR, "non-finite residual");
        if (rnorm <= goal) break;
        st->refinements = pass + 1;
        unsigned it = 0;
        double rr = 0;
        if (fp64) {
            s = pcg_f64(c, goal * 0.5, cfg.max_cg_iter - total, &it, &rr);
        } else {
            // Inner FP32 solve to a relative reduction the FP32 operator can
            // deliver; the FP64 pass loop does the rest.
            double eta = 0.5 * goal / rnorm;
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
                k_accumulate<<<grid_for(c, N), kThreads, 0, c->stream>>>(
                    c->x64, c->kx, N);
            }
        }
        if (s != JETGPU_OK) return s;
        total += it;
        st->iterations = total;
    }
    if (st->relative_residual > cfg.tolerance) {
        // Final check after the last pass.
        k_residual64<<<G, kThreads, 0, c->stream>>>(
            c->A64, c->x64, c->b64, c->r64, nullptr, nullptr, n, c->partials,
            c->counters, c->scal, S_R64);
        s = read_scalars(c);
        if (s != JETGPU_OK) return s;
        rnorm = std::sqrt(c->h_scal[S_R64]);
        st->residual = rnorm;
        st->relative_residual = rnorm / bnorm;
        if (rnorm > goal)
            return fail(c, JETGPU_NOT_CONVERGED,
                        "tolerance not reached within the iteration cap");
    }
    return fell_back ? JETGPU_STALLED_FALLBACK_USED : JETGPU_OK;
}

}  // namespace jg

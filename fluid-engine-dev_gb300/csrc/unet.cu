// Learned preconditioner: 3-D U-Net building blocks on the tcgen05 tensor
// cores (K15-K17), plus the C ABI that the training code and the flexible
// PCG use.
//
// Activations are BF16, channels-last: act[v * C + c] with v the cell index
// (i fastest). Convolutions are 3x3x3, stride 1, zero padding 1, computed as
// implicit GEMMs: D[v, co] = sum_{tap, ci} in[v + off(tap), ci] * W[tap, co, ci]
// with M = 128 output cells per CTA, N = C_out, K = 27 * C_in, BF16 operands
// staged K-major in shared memory and FP32 accumulators in tensor memory.
// One elected thread issues tcgen05.mma; completion is tracked with
// tcgen05.commit on an mbarrier; the epilogue reads TMEM with tcgen05.ld.
// These layers have no counterpart in the reference.

#include "ctx.h"
#include "tc.cuh"

#include <cuda_bf16.h>

namespace jg {
namespace {

constexpr int kTile = 128;  // output cells per CTA (MMA M)

__device__ __forceinline__ void cp16z(void* smem, const void* gmem, bool valid) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s),
                 "l"(gmem), "r"(valid ? 16 : 0));
}
__device__ __forceinline__ void cp_commit() {
    asm volatile("cp.async.commit_group;\n" ::);
}
template <int N>
__device__ __forceinline__ void cp_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

struct ConvArgs {
    const __nv_bfloat16* in;  // [V][ci]
    const __nv_bfloat16* w;   // [27][co][ci]
    const float* bias;        // [co] or null
    __nv_bfloat16* out;       // [V][co] or null
    float* out32;             // [V][co] or null (FP32 copy of the result)
    Dims n;
    int ci, co;
    int relu;
    unsigned* err;            // set to nonzero if a wait gave up
};

// Dynamic shared memory of a conv CTA. At least 56 KB, so that at most 4
// CTAs share an SM and their TMEM allocations (<= 128 columns each) always
// fit in the SM's 512 columns: tcgen05.alloc never has to wait.
__host__ __device__ inline size_t conv_smem_bytes(int ci, int co) {
    const size_t need = 2 * (size_t)kTile * ci * 2 + 2 * (size_t)co * ci * 2 + 64;
    const size_t floor_bytes = 56 * 1024;
    return need > floor_bytes ? need : floor_bytes;
}

// K15: 3x3x3 convolution, BF16 in, FP32 accumulate, optional bias + ReLU.
__global__ void __launch_bounds__(128) k_conv3d_tc(ConvArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int ci = a.ci, co = a.co;
    const uint32_t abytes = (uint32_t)kTile * ci * 2, bbytes = (uint32_t)co * ci * 2;
    unsigned char* Abuf[2] = {smem, smem + abytes};
    unsigned char* Bbuf[2] = {smem + 2 * abytes, smem + 2 * abytes + bbytes};
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + 2 * abytes + 2 * bbytes);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 2);
    const int tid = threadIdx.x, warp = tid >> 5;
    const long V = a.n.count();
    const long v = (long)blockIdx.x * kTile + tid;
    const uint32_t ncols = co <= 32 ? 32u : (co <= 64 ? 64u : 128u);
    const uint32_t sbo = (uint32_t)(ci / 8) * 128u;

    if (warp == 0) tc::tmem_alloc(tslot, ncols);
    if (tid == 0) {
        tc::mbar_init(&mbar[0], 1);
        tc::mbar_init(&mbar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;

    int vi = 0, vj = 0, vk = 0;
    const bool vok = v < V;
    if (vok) cell_ijk(v, a.n, vi, vj, vk);

    // Stage tap t into buffer `buf`: this thread's A row (output cell v),
    // and a share of the tap's weights.
    auto stage = [&](int t, int buf) {
        const int dz = t / 9 - 1, dy = (t / 3) % 3 - 1, dx = t % 3 - 1;
        const int ii = vi + dx, jj = vj + dy, kk = vk + dz;
        const bool ok = vok && ii >= 0 && ii < a.n.x && jj >= 0 && jj < a.n.y &&
                        kk >= 0 && kk < a.n.z;
        const __nv_bfloat16* src =
            ok ? a.in + lin(ii, jj, kk, a.n.x, a.n.y) * ci : a.in;
        unsigned char* row = Abuf[buf] + (tid >> 3) * sbo + (tid & 7) * 16;
        for (int kg = 0; kg < ci / 8; ++kg) cp16z(row + kg * 128, src + 8 * kg, ok);
        const __nv_bfloat16* wt = a.w + (long)t * co * ci;
        const int chunks = co * (ci / 8);
        for (int q = tid; q < chunks; q += 128) {
            const int r = q / (ci / 8), kg = q - r * (ci / 8);
            cp16z(Bbuf[buf] + (r >> 3) * sbo + kg * 128 + (r & 7) * 16,
                  wt + r * ci + 8 * kg, true);
        }
    };

    const uint32_t idesc = tc::idesc_bf16_f32(kTile, co);
    uint32_t phase[2] = {0u, 0u};
    bool ok = true;
    stage(0, 0);
    cp_commit();
    for (int t = 0; t < 27; ++t) {
        const int buf = t & 1;
        if (t + 1 < 27) {
            if (t >= 1) {
                // The MMAs of tap t-1 read the other buffer: wait for them
                // before overwriting it.
                ok &= tc::mbar_wait(&mbar[buf ^ 1], phase[buf ^ 1]);
                phase[buf ^ 1] ^= 1u;
            }
            stage(t + 1, buf ^ 1);
            cp_commit();
            cp_wait<1>();
        } else {
            cp_wait<0>();
        }
        tc::fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            const uint32_t ab = tc::smem_u32(Abuf[buf]), bb = tc::smem_u32(Bbuf[buf]);
            for (int kk = 0; kk < ci / 16; ++kk) {
                const uint64_t ad = tc::smem_desc(ab + kk * 256, 128, sbo);
                const uint64_t bd = tc::smem_desc(bb + kk * 256, 128, sbo);
                tc::mma_bf16(tmem, ad, bd, idesc, (t > 0 || kk > 0) ? 1u : 0u);
            }
            tc::mma_commit(&mbar[buf]);
        }
    }
    // tcgen05.commit tracks every earlier MMA of the issuing thread, so the
    // last commit (tap 26, buffer 0) covers the whole accumulation.
    ok &= tc::mbar_wait(&mbar[0], phase[0]);
    if (!ok && a.err) atomicOr(a.err, 1u);
    tc::fence_after_sync();

    const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
    for (int c0 = 0; c0 < co; c0 += 16) {
        float val[16];
        tc::tmem_ld16(trow + (uint32_t)c0, val);
        if (vok) {
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                float x = val[q] + (a.bias ? a.bias[c0 + q] : 0.0f);
                if (a.relu) x = fmaxf(x, 0.0f);
                val[q] = x;
            }
            if (a.out) {
                __align__(16) __nv_bfloat16 h[16];
#pragma unroll
                for (int q = 0; q < 16; ++q) h[q] = __float2bfloat16_rn(val[q]);
                uint4* dst = reinterpret_cast<uint4*>(a.out + v * co + c0);
                dst[0] = reinterpret_cast<const uint4*>(h)[0];
                dst[1] = reinterpret_cast<const uint4*>(h)[1];
            }
            if (a.out32) {
                float4* dst = reinterpret_cast<float4*>(a.out32 + v * co + c0);
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    dst[q] = make_float4(val[4 * q], val[4 * q + 1],
                                         val[4 * q + 2], val[4 * q + 3]);
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

}  // namespace

jetgpu_status conv3d(cudaStream_t st, const __nv_bfloat16* in, int ci,
                     const __nv_bfloat16* w, const float* bias, int co,
                     Dims n, int relu, __nv_bfloat16* out, float* out32,
                     unsigned* err) {
    ConvArgs a{in, w, bias, out, out32, n, ci, co, relu, err};
    const size_t smem = conv_smem_bytes(ci, co);
    static bool attr_set = false;
    if (!attr_set) {
        if (cudaFuncSetAttribute(k_conv3d_tc,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)conv_smem_bytes(128, 128)) != cudaSuccess)
            return JETGPU_CUDA_ERROR;
        attr_set = true;
    }
    const long blocks = (n.count() + kTile - 1) / kTile;
    k_conv3d_tc<<<(unsigned)blocks, 128, smem, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? JETGPU_OK : JETGPU_CUDA_ERROR;
}

}  // namespace jg

extern "C" jetgpu_status jetgpu_conv3d(void* stream, const void* in, int ci,
                                       const void* w, const float* bias,
                                       int co, const int res[3], int relu,
                                       void* out, float* out32,
                                       unsigned* err) {
    using namespace jg;
    if (!in || !w || !res || (!out && !out32)) return JETGPU_BAD_INPUT;
    if (ci < 16 || ci > 128 || ci % 16 || co < 16 || co > 128 || co % 16)
        return JETGPU_BAD_INPUT;
    for (int a = 0; a < 3; ++a)
        if (res[a] < 1) return JETGPU_BAD_INPUT;
    return conv3d(static_cast<cudaStream_t>(stream),
                  static_cast<const __nv_bfloat16*>(in), ci,
                  static_cast<const __nv_bfloat16*>(w), bias, co,
                  Dims{res[0], res[1], res[2]}, relu,
                  static_cast<__nv_bfloat16*>(out), out32, err);
}

// ---------------------------------------------------------------------------
// K16 (training): weight gradient dW[t][co][ci] += sum_v dy[v][co] *
// in[v + off(t)][ci] as a tensor-core GEMM with K = cells. Per 128-cell
// K-tile the threads transpose dy (A: 128 rows = co padded with zeros, K =
// cells) and the tap-shifted input (B: ci rows, K = cells) into K-major
// operand tiles; one thread issues the MMAs of a group of taps, whose
// accumulators sit side by side in TMEM (tg * ci <= 512 columns).
// Persistent CTAs accumulate over their tiles and add the result into the
// FP32 gradient with atomics at the end (the caller zeroes it).

namespace jg {
namespace {

constexpr uint32_t kWgSbo = 16u * 128u;  // 128 K-columns = 16 core matrices

struct WgradArgs {
    const __nv_bfloat16* in;  // [V][ci]
    const __nv_bfloat16* dy;  // [V][co]
    float* dw;                // [27][co][ci]
    Dims n;
    int ci, co, t0, tg;
    unsigned* err;
};

__host__ __device__ inline int wgrad_taps(int ci) {
    int tg = 512 / ci;
    return tg > 27 ? 27 : tg;
}

__host__ __device__ inline size_t wgrad_smem_bytes(int ci) {
    // A (128 rows) + tg B tiles (ci rows each), 128 K-columns of BF16, plus
    // barrier space; at least 120 KB so one CTA holds an SM's TMEM.
    const size_t need = (size_t)128 * 256 + (size_t)wgrad_taps(ci) * ci * 256 + 64;
    const size_t floor_bytes = 120 * 1024;
    return need > floor_bytes ? need : floor_bytes;
}

// Writes the 8 channels of one cell (16 bytes) into column `col` of rows
// r0..r0+7 of a K-major operand tile.
__device__ __forceinline__ void scatter8(unsigned char* tile, int r0, int col,
                                         uint4 chunk) {
    const __nv_bfloat16* h = reinterpret_cast<const __nv_bfloat16*>(&chunk);
    unsigned char* base = tile + (r0 >> 3) * kWgSbo + (col >> 3) * 128 + (col & 7) * 2;
#pragma unroll
    for (int q = 0; q < 8; ++q)
        *reinterpret_cast<__nv_bfloat16*>(base + q * 16) = h[q];
}

__global__ void __launch_bounds__(128) k_conv3d_wgrad_tc(WgradArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int ci = a.ci, co = a.co, tg = a.tg;
    unsigned char* A = smem;
    unsigned char* B = smem + 128 * 256;
    const uint32_t bstride = (uint32_t)ci * 256u;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(B + (size_t)tg * bstride);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 1);
    const int tid = threadIdx.x, warp = tid >> 5;
    const long V = a.n.count();
    const long tiles = (V + 127) / 128;
    uint32_t need = (uint32_t)(tg * ci), ncols = 32;
    while (ncols < need) ncols <<= 1;

    if (warp == 0) tc::tmem_alloc(tslot, ncols);
    if (tid == 0) {
        tc::mbar_init(&mbar[0], 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    // Rows co..127 of A stay zero.
    for (int q = tid; q < 128 * 256 / 16; q += 128)
        reinterpret_cast<uint4*>(A)[q] = make_uint4(0, 0, 0, 0);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;
    const uint32_t idesc = tc::idesc_bf16_f32(128, ci);
    uint32_t phase = 0;
    bool ok = true;
    long done = 0;
    for (long tile = blockIdx.x; tile < tiles; tile += gridDim.x, ++done) {
        const long v = tile * 128 + tid;
        const bool vok = v < V;
        int vi = 0, vj = 0, vk = 0;
        if (vok) cell_ijk(v, a.n, vi, vj, vk);
        for (int c8 = 0; c8 < co; c8 += 8) {
            uint4 chunk = make_uint4(0, 0, 0, 0);
            if (vok) chunk = *reinterpret_cast<const uint4*>(a.dy + v * co + c8);
            scatter8(A, c8, tid, chunk);
        }
        for (int g = 0; g < tg; ++g) {
            const int t = a.t0 + g;
            const int dz = t / 9 - 1, dyy = (t / 3) % 3 - 1, dx = t % 3 - 1;
            const int ii = vi + dx, jj = vj + dyy, kk = vk + dz;
            const bool ok2 = vok && ii >= 0 && ii < a.n.x && jj >= 0 &&
                             jj < a.n.y && kk >= 0 && kk < a.n.z;
            const __nv_bfloat16* src =
                ok2 ? a.in + lin(ii, jj, kk, a.n.x, a.n.y) * ci : nullptr;
            for (int c8 = 0; c8 < ci; c8 += 8) {
                uint4 chunk = make_uint4(0, 0, 0, 0);
                if (ok2) chunk = *reinterpret_cast<const uint4*>(src + c8);
                scatter8(B + g * bstride, c8, tid, chunk);
            }
        }
        tc::fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            const uint32_t ab = tc::smem_u32(A), bb = tc::smem_u32(B);
            for (int g = 0; g < tg; ++g)
                for (int k16 = 0; k16 < 8; ++k16) {
                    const uint64_t ad = tc::smem_desc(ab + k16 * 256, 128, kWgSbo);
                    const uint64_t bd =
                        tc::smem_desc(bb + g * bstride + k16 * 256, 128, kWgSbo);
                    tc::mma_bf16(tmem + (uint32_t)(g * ci), ad, bd, idesc,
                                 (done > 0 || k16 > 0) ? 1u : 0u);
                }
            tc::mma_commit(&mbar[0]);
        }
        // The next tile overwrites the operand tiles: wait for the MMAs.
        ok &= tc::mbar_wait(&mbar[0], phase);
        phase ^= 1u;
        tc::fence_after_sync();
    }
    if (!ok && a.err) atomicOr(a.err, 1u);
    if (done > 0 && warp * 32 < co) {
        const int row = warp * 32 + (tid & 31);
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
        for (int g = 0; g < tg; ++g)
            for (int c0 = 0; c0 < ci; c0 += 16) {
                float val[16];
                tc::tmem_ld16(trow + (uint32_t)(g * ci + c0), val);
                if (row < co) {
                    float* dst = a.dw + ((long)(a.t0 + g) * co + row) * ci + c0;
#pragma unroll
                    for (int q = 0; q < 16; ++q) atomicAdd(dst + q, val[q]);
                }
            }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

}  // namespace

jetgpu_status conv3d_wgrad(cudaStream_t st, const __nv_bfloat16* in, int ci,
                           const __nv_bfloat16* dy, int co, Dims n, float* dw,
                           unsigned* err, int sms) {
    static bool attr_set = false;
    if (!attr_set) {
        if (cudaFuncSetAttribute(k_conv3d_wgrad_tc,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 200 * 1024) != cudaSuccess)
            return JETGPU_CUDA_ERROR;
        attr_set = true;
    }
    const long tiles = (n.count() + 127) / 128;
    const int grid = (int)(tiles < sms ? tiles : sms);
    const int tg = wgrad_taps(ci);
    for (int t0 = 0; t0 < 27; t0 += tg) {
        WgradArgs a{in, dy, dw, n, ci, co, t0, t0 + tg <= 27 ? tg : 27 - t0, err};
        k_conv3d_wgrad_tc<<<grid, 128, wgrad_smem_bytes(ci), st>>>(a);
    }
    return cudaGetLastError() == cudaSuccess ? JETGPU_OK : JETGPU_CUDA_ERROR;
}

}  // namespace jg

extern "C" jetgpu_status jetgpu_conv3d_wgrad(void* stream, const void* in,
                                             int ci, const void* dy, int co,
                                             const int res[3], float* dw,
                                             unsigned* err) {
    using namespace jg;
    if (!in || !dy || !dw || !res) return JETGPU_BAD_INPUT;
    if (ci < 16 || ci > 128 || ci % 16 || co < 16 || co > 128 || co % 16)
        return JETGPU_BAD_INPUT;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
            cudaSuccess)
        return JETGPU_CUDA_ERROR;
    return conv3d_wgrad(static_cast<cudaStream_t>(stream),
                        static_cast<const __nv_bfloat16*>(in), ci,
                        static_cast<const __nv_bfloat16*>(dy), co,
                        Dims{res[0], res[1], res[2]}, dw, err, sms);
}

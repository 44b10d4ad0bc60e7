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

// ---------------------------------------------------------------------------
// K15 on rows of 128 cells (nx a multiple of 128): the input brick of a tile
// staged once, all 27 taps read from it.
//
// A persistent CTA takes output tiles of 128 consecutive cells along i (one
// (j, k) row segment, the MMA's M). Per tile and per chunk of 16 input
// channels, one thread stages the brick the tile's 27 taps read — cells
// i0-1 .. i0+128 of rows j-1 .. j+1 of planes k-1 .. k+1 — with two TMA
// copies (channels 0-7 and 8-15 of the chunk; cells outside the grid arrive
// as zeros, which is the convolution's zero padding). In shared memory each
// copy is a run of 16-byte cells, so the A operand of tap (dx, dy, dz) is
// the same run started at that tap's cell offset: 128 consecutive rows 16
// bytes apart (8-row core matrices 128 bytes apart), the two channel halves
// one copy apart. The CTA's weights, all taps and channels, are loaded once
// into shared memory as K-major B tiles. Bricks are double-buffered: the
// copy of the next chunk (or of the next tile's first chunk) runs under the
// MMAs of the current one. Accumulators in TMEM (128 lanes x C_out FP32
// columns); the epilogue adds the bias, applies the ReLU and stores BF16 or
// FP32 rows of the channels-last output.

constexpr int kBrickX = 130;                  // cells i0-1 .. i0+128
constexpr int kBrickCells = kBrickX * 3 * 3;  // rows j-1..j+1, planes k-1..k+1
constexpr uint32_t kHalfBytes = 18816;        // 16 B x 1170 cells, 128-aligned
static_assert(kHalfBytes >= 16u * kBrickCells && kHalfBytes % 128u == 0u,
              "brick half");

__host__ __device__ inline size_t brick_weight_bytes(int ci, int co) {
    return (size_t)27 * co * ci * 2;
}
__host__ __device__ inline size_t brick_smem_bytes(int ci, int co) {
    // weights | 2 stages x 2 channel halves | barriers, TMEM slot; plus
    // alignment slack for the 128-byte aligned base
    return brick_weight_bytes(ci, co) + 4 * (size_t)kHalfBytes + 64 + 128;
}

struct BrickArgs {
    const __nv_bfloat16* w;  // [27][co][ci]
    const float* bias;       // [co] or null
    __nv_bfloat16* out;      // [V][co] or null
    float* out32;            // [V][co] or null
    Dims n;
    int ci, co, relu;
    unsigned* err;
};

__global__ void __launch_bounds__(128)
    k_conv3d_brick(const __grid_constant__ CUtensorMap tm_in, BrickArgs a) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char* base = reinterpret_cast<unsigned char*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    const int ci = a.ci, co = a.co, nk = ci / 16;
    unsigned char* W = base;
    unsigned char* brick = base + brick_weight_bytes(ci, co);
    uint64_t* full = reinterpret_cast<uint64_t*>(brick + 4 * kHalfBytes);
    uint64_t* empty = full + 2;
    uint64_t* accf = full + 4;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(full + 5);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int tx = a.n.x / 128;
    const long ntiles = (long)tx * a.n.y * a.n.z;
    uint32_t ncols = 32;
    while (ncols < (uint32_t)co) ncols <<= 1;

    if (warp == 0) tc::tmem_alloc(tslot, ncols);
    if (tid == 0) {
        for (int q = 0; q < 5; ++q) tc::mbar_init(&full[q], 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    // Weights, K-major B tiles per (chunk, tap): [kc][t][half][co][8 ch].
    {
        const int groups = ci / 8;
        const long pieces = 27L * co * groups;
        for (long q = tid; q < pieces; q += 128) {
            const int g = (int)(q % groups);
            const long tn = q / groups;
            const int nn = (int)(tn % co), t = (int)(tn / co);
            const uint4 v = __ldg(reinterpret_cast<const uint4*>(
                a.w + ((long)t * co + nn) * ci + 8 * g));
            const long off = ((((long)(g >> 1) * 27 + t) * 2 + (g & 1)) * co + nn) * 16;
            *reinterpret_cast<uint4*>(W + off) = v;
        }
    }
    tc::fence_proxy_async();  // generic-proxy writes seen by the MMAs
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;
    const uint32_t idesc = tc::idesc_bf16_f32(128, co);
    const uint32_t wbase = tc::smem_u32(W), bbase = tc::smem_u32(brick);
    const uint32_t wstep = (uint32_t)co * 32u;  // one (chunk, tap) B tile
    bool ok = true;

    // Chunk q of this CTA's sequence: tile blockIdx.x + (q / nk) * gridDim.x,
    // input channels 16 (q % nk) ...
    const long my_tiles = ntiles > blockIdx.x
        ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const long nq = my_tiles * nk;
    auto issue = [&](long q) {
        const long tile = blockIdx.x + (q / nk) * (long)gridDim.x;
        const int kc = (int)(q % nk);
        const int i0 = (int)(tile % tx) * 128;
        const long r = tile / tx;
        const int j = (int)(r % a.n.y), k = (int)(r / a.n.y);
        const int st = (int)(q & 1);
        uint64_t* bar = &full[st];
        asm volatile(
            "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(
                tc::smem_u32(bar)),
            "r"(2u * 16u * kBrickCells)
            : "memory");
        for (int h = 0; h < 2; ++h) {
            unsigned char* dst = brick + (st * 2 + h) * kHalfBytes;
            asm volatile(
                "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::"
                "complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];\n" ::"r"(
                    tc::smem_u32(dst)),
                "l"(reinterpret_cast<uint64_t>(&tm_in)), "r"(16 * kc + 8 * h),
                "r"(i0 - 1), "r"(j - 1), "r"(k - 1), "r"(tc::smem_u32(bar))
                : "memory");
        }
    };
    // Thread 0 stages bricks one chunk ahead of the MMAs; thread 32 issues
    // the MMAs as each brick lands. A stage is reloaded once the MMAs of the
    // chunk that last used it have completed (`empty`).
    if (tid == 0 && nq > 0) issue(0);
    long q0 = 0;  // first chunk of the current tile
    for (long lt = 0; lt < my_tiles; ++lt, q0 += nk) {
        const long tile = blockIdx.x + lt * (long)gridDim.x;
        if (tid == 0) {
            for (int kc = 0; kc < nk; ++kc) {
                const long q = q0 + kc;
                if (q + 1 < nq) {
                    if (q >= 1)
                        ok &= tc::mbar_wait(&empty[(q + 1) & 1],
                                            (uint32_t)(((q - 1) >> 1) & 1));
                    issue(q + 1);
                }
            }
        } else if (tid == 32) {
            tc::fence_after_sync();
            for (int kc = 0; kc < nk; ++kc) {
                const long q = q0 + kc;
                ok &= tc::mbar_wait(&full[q & 1], (uint32_t)((q >> 1) & 1));
                const uint32_t half0 = bbase + (uint32_t)(q & 1) * 2u * kHalfBytes;
                for (int t = 0; t < 27; ++t) {
                    const uint32_t cell =
                        (uint32_t)((((t / 9) * 3 + (t / 3) % 3) * kBrickX) + t % 3);
                    const uint64_t ad = tc::smem_desc(half0 + cell * 16u,
                                                      kHalfBytes, 128);
                    const uint64_t bd = tc::smem_desc(
                        wbase + (uint32_t)(kc * 27 + t) * wstep, (uint32_t)co * 16u,
                        128);
                    tc::mma_bf16(tmem, ad, bd, idesc,
                                 (kc > 0 || t > 0) ? 1u : 0u);
                }
                tc::mma_commit(&empty[q & 1]);
            }
            tc::mma_commit(accf);
        }
        __syncwarp();
        ok &= tc::mbar_wait(accf, (uint32_t)(lt & 1));
        __syncwarp();  // tcgen05.ld below is warp-collective
        tc::fence_after_sync();
        // Epilogue: warp w holds cells i0 + 32 w + lane.
        const int i0 = (int)(tile % tx) * 128;
        const long r = tile / tx;
        const int j = (int)(r % a.n.y), k = (int)(r / a.n.y);
        const long v = lin(i0 + 32 * warp + (tid & 31), j, k, a.n.x, a.n.y);
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
        for (int c0 = 0; c0 < co; c0 += 16) {
            float val[16];
            tc::tmem_ld16(trow + (uint32_t)c0, val);
#pragma unroll
            for (int qq = 0; qq < 16; ++qq) {
                float x = val[qq] + (a.bias ? a.bias[c0 + qq] : 0.0f);
                if (a.relu) x = fmaxf(x, 0.0f);
                val[qq] = x;
            }
            if (a.out) {
                __align__(16) __nv_bfloat16 hb[16];
#pragma unroll
                for (int qq = 0; qq < 16; ++qq) hb[qq] = __float2bfloat16_rn(val[qq]);
                uint4* dst = reinterpret_cast<uint4*>(a.out + v * co + c0);
                dst[0] = reinterpret_cast<const uint4*>(hb)[0];
                dst[1] = reinterpret_cast<const uint4*>(hb)[1];
            }
            if (a.out32) {
                float4* dst = reinterpret_cast<float4*>(a.out32 + v * co + c0);
#pragma unroll
                for (int qq = 0; qq < 4; ++qq)
                    dst[qq] = make_float4(val[4 * qq], val[4 * qq + 1],
                                          val[4 * qq + 2], val[4 * qq + 3]);
            }
        }
        // The next tile's MMAs overwrite the accumulators.
        tc::fence_before_sync();
        __syncthreads();
    }
    if (!ok && a.err) atomicOr(a.err, 1u);
    if (__syncthreads_or(!ok) && tid == 32 && nq > 0) {
        // A wait gave up: let the last copies and MMAs land (bounded)
        // before the CTA releases its shared memory and TMEM.
        for (long q = nq >= 2 ? nq - 2 : 0; q < nq; ++q)
            tc::mbar_wait(&full[q & 1], (uint32_t)((q >> 1) & 1));
        tc::mbar_wait(accf, (uint32_t)((my_tiles - 1) & 1));
    }
    tc::fence_after_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

// Tensor map of a channels-last BF16 activation [nz][ny][nx][ci] with the
// brick box (8 channels x 130 x 3 x 3).
bool brick_map(CUtensorMap* m, const __nv_bfloat16* in, int ci, Dims n) {
    auto enc = tma_encoder();
    if (!enc) return false;
    cuuint64_t gd[4] = {(cuuint64_t)ci, (cuuint64_t)n.x, (cuuint64_t)n.y,
                        (cuuint64_t)n.z};
    cuuint64_t gs[3] = {(cuuint64_t)ci * 2, (cuuint64_t)n.x * ci * 2,
                        (cuuint64_t)n.y * n.x * ci * 2};
    cuuint32_t bx[4] = {8, (cuuint32_t)kBrickX, 3, 3}, es[4] = {1, 1, 1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4,
               const_cast<__nv_bfloat16*>(in), gd, gs, bx, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

constexpr size_t kMaxConvSmem = 227 * 1024;

}  // namespace

jetgpu_status conv3d(cudaStream_t st, const __nv_bfloat16* in, int ci,
                     const __nv_bfloat16* w, const float* bias, int co,
                     Dims n, int relu, __nv_bfloat16* out, float* out32,
                     unsigned* err) {
    // Rows of 128 cells and a CTA's weights within shared memory: the
    // brick kernel; otherwise the per-tap gather kernel below.
    const size_t bsmem = brick_smem_bytes(ci, co);
    CUtensorMap tm;
    if (n.x % 128 == 0 && bsmem <= kMaxConvSmem &&
        (reinterpret_cast<uintptr_t>(in) & 15u) == 0 && brick_map(&tm, in, ci, n)) {
        // The largest shared-memory carveout, so that two CTAs of the
        // smaller layers fit on an SM (with the default carveout the
        // occupancy query, and so the grid, allowed one).
        static DeviceOnce battr;
        if (!battr.run([] {
                cudaError_t e = cudaFuncSetAttribute(
                    k_conv3d_brick, cudaFuncAttributeMaxDynamicSharedMemorySize,
                    (int)kMaxConvSmem);
                if (e != cudaSuccess) return e;
                return cudaFuncSetAttribute(
                    k_conv3d_brick,
                    cudaFuncAttributePreferredSharedMemoryCarveout,
                    (int)cudaSharedmemCarveoutMaxShared);
            }))
            return JETGPU_CUDA_ERROR;
        int dev = 0, sms = 0, occ = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_conv3d_brick,
                                                          128, bsmem) !=
                cudaSuccess)
            return JETGPU_CUDA_ERROR;
        if (occ < 1) occ = 1;
        if (occ > 2) occ = 2;  // TMEM: <= 2 x 256 columns per SM
        const long tiles = (long)(n.x / 128) * n.y * n.z;
        long grid = (long)sms * occ;
        if (grid > tiles) grid = tiles;
        BrickArgs ba{w, bias, out, out32, n, ci, co, relu, err};
        k_conv3d_brick<<<(unsigned)grid, 128, bsmem, st>>>(tm, ba);
        return cudaGetLastError() == cudaSuccess ? JETGPU_OK : JETGPU_CUDA_ERROR;
    }
    ConvArgs a{in, w, bias, out, out32, n, ci, co, relu, err};
    const size_t smem = conv_smem_bytes(ci, co);
    static DeviceOnce attr;
    if (!attr.run([] {
            cudaError_t e = cudaFuncSetAttribute(
                k_conv3d_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                (int)conv_smem_bytes(128, 128));
            if (e != cudaSuccess) return e;
            return cudaFuncSetAttribute(
                k_conv3d_tc, cudaFuncAttributePreferredSharedMemoryCarveout,
                (int)cudaSharedmemCarveoutMaxShared);
        }))
        return JETGPU_CUDA_ERROR;
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
    static DeviceOnce attr;
    if (!attr.run([] {
            return cudaFuncSetAttribute(
                k_conv3d_wgrad_tc,
                cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        }))
        return JETGPU_CUDA_ERROR;
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

// ---------------------------------------------------------------------------
// K17: the preconditioner network. A 3-D U-Net with 4 levels (16, 32, 48,
// 64 channels), two 3x3x3 convolutions per level and side, 2x2x2 average
// pooling, nearest-neighbour upsampling and skip concatenation
// [upsampled | skip]. It runs on one coarse multigrid level (net_level:
// the finest level at most 64 cells wide) and maps the residual a V-cycle
// leaves, restricted to that level, to a correction of the V-cycle's error
// there (learned_precond in mgpcg.cu). Input: 16 channels of per-cell
// features of the residual and of that level's system (net_features below).
// Output: channel 0 of the last convolution, scaled back to the residual's
// units.

namespace jg {

const NetLayer kNetLayers[kNetLayerCount] = {
    {16, 16, 1, 0},  {16, 16, 1, 0},   // encoder, level 0
    {16, 32, 1, 1},  {32, 32, 1, 1},   // level 1
    {32, 48, 1, 2},  {48, 48, 1, 2},   // level 2
    {48, 64, 1, 3},  {64, 64, 1, 3},   // level 3
    {112, 48, 1, 2}, {48, 48, 1, 2},   // decoder, level 2 ([up(64) | 48])
    {80, 32, 1, 1},  {32, 32, 1, 1},   // level 1 ([up(48) | 32])
    {48, 16, 1, 0},  {16, 16, 0, 0}};  // level 0 ([up(32) | 16]), output

size_t net_param_count() {
    size_t n = 0;
    for (int l = 0; l < kNetLayerCount; ++l)
        n += (size_t)27 * kNetLayers[l].ci * kNetLayers[l].co + kNetLayers[l].co;
    return n;
}

namespace {

// Input features of cell c (16 channels, BF16): residual / rms(residual),
// the six face weights of the cell, fluid indicator, diagonal * h^2 / 6.
__global__ void k_net_features(const float* __restrict__ r,
                               const double* __restrict__ rr, long N,
                               const float* __restrict__ uw,
                               const float* __restrict__ vw,
                               const float* __restrict__ ww,
                               const float* __restrict__ phi,
                               const float* __restrict__ A, float h2, Dims n,
                               __nv_bfloat16* __restrict__ feat) {
    const double ms = rr[0] / (double)N;
    const float inv = ms > 0.0 ? (float)(1.0 / sqrt(ms)) : 0.0f;
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_ijk(c, n, i, j, k);
        float f[16];
        f[0] = r[c] * inv;
        f[1] = uw[lin(i, j, k, n.x + 1, n.y)];
        f[2] = uw[lin(i + 1, j, k, n.x + 1, n.y)];
        f[3] = vw[lin(i, j, k, n.x, n.y + 1)];
        f[4] = vw[lin(i, j + 1, k, n.x, n.y + 1)];
        f[5] = ww[lin(i, j, k, n.x, n.y)];
        f[6] = ww[lin(i, j, k + 1, n.x, n.y)];
        f[7] = phi[c] < 0.0f ? 1.0f : 0.0f;
        f[8] = A[c] * h2 * (1.0f / 6.0f);  // center plane
#pragma unroll
        for (int q = 9; q < 16; ++q) f[q] = 0.0f;
        __align__(16) __nv_bfloat16 h[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) h[q] = __float2bfloat16_rn(f[q]);
        uint4* dst = reinterpret_cast<uint4*>(feat + c * 16);
        dst[0] = reinterpret_cast<const uint4*>(h)[0];
        dst[1] = reinterpret_cast<const uint4*>(h)[1];
    }
}

// 2x2x2 average pooling, channels-last BF16 (FP32 sum, one rounding).
__global__ void k_pool2(const __nv_bfloat16* __restrict__ in, Dims fine,
                        int C, __nv_bfloat16* __restrict__ out) {
    const Dims cs{fine.x / 2, fine.y / 2, fine.z / 2};
    const long total = cs.count() * C;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total;
         e += (long)gridDim.x * blockDim.x) {
        const long c = e / C;
        const int ch = (int)(e - c * C);
        int i, j, k;
        cell_ijk(c, cs, i, j, k);
        float s = 0.0f;
        for (int dz = 0; dz < 2; ++dz)
            for (int dy = 0; dy < 2; ++dy)
                for (int dx = 0; dx < 2; ++dx)
                    s += __bfloat162float(
                        in[lin(2 * i + dx, 2 * j + dy, 2 * k + dz, fine.x, fine.y) * C + ch]);
        out[e] = __float2bfloat16_rn(0.125f * s);
    }
}

// out[v] = [ coarse[v / 2] (C1 channels) | skip[v] (C2 channels) ].
__global__ void k_up_concat(const __nv_bfloat16* __restrict__ coarse, int C1,
                            const __nv_bfloat16* __restrict__ skip, int C2,
                            Dims fine, __nv_bfloat16* __restrict__ out) {
    const int C = C1 + C2;
    const Dims cs{fine.x / 2, fine.y / 2, fine.z / 2};
    const long total = fine.count() * C;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total;
         e += (long)gridDim.x * blockDim.x) {
        const long c = e / C;
        const int ch = (int)(e - c * C);
        int i, j, k;
        cell_ijk(c, fine, i, j, k);
        out[e] = ch < C1 ? coarse[lin(i >> 1, j >> 1, k >> 1, cs.x, cs.y) * C1 + ch]
                         : skip[c * C2 + (ch - C1)];
    }
}

// Output gain of the network: it predicts kNetGain * e / rms(r) for a
// residual r and error e = A^-1 r. For the smooth error modes, e is about
// r / (3 pi^2) whatever the grid spacing (the rows carry 1/h^2 on the unit
// cube), so the target is O(1)-scaled and independent of the resolution.
constexpr float kNetGain = 32.0f;

// z[c] = out32[c][0] * rms(residual) / kNetGain on fluid cells, 0 elsewhere.
__global__ void k_net_output(const float* __restrict__ out32,
                             const double* __restrict__ rr, long N,
                             const float* __restrict__ phi,
                             float* __restrict__ z) {
    const double ms = rr[0] / (double)N;
    const float scale = (float)sqrt(ms > 0.0 ? ms : 0.0) / kNetGain;
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x)
        z[c] = phi[c] < 0.0f ? out32[c * 16] * scale : 0.0f;
}

template <typename T>
cudaError_t nalloc(T** p, size_t count) {
    return cudaMalloc((void**)p, count * sizeof(T));
}

}  // namespace

struct Net {
    Dims n0{0, 0, 0};
    __nv_bfloat16* w[kNetLayerCount] = {};
    float* b[kNetLayerCount] = {};
    // Activations per level.
    __nv_bfloat16 *feat = nullptr, *t0 = nullptr, *e0 = nullptr, *u0 = nullptr,
                  *d0 = nullptr;
    __nv_bfloat16 *p1 = nullptr, *t1 = nullptr, *e1 = nullptr, *u1 = nullptr,
                  *d1 = nullptr;
    __nv_bfloat16 *p2 = nullptr, *t2 = nullptr, *e2 = nullptr, *u2 = nullptr,
                  *d2 = nullptr;
    __nv_bfloat16 *p3 = nullptr, *t3 = nullptr, *e3 = nullptr;
    float* out32 = nullptr;
    unsigned* err = nullptr;
    bool loaded = false;
};

void net_free_acts(Net* net) {
    __nv_bfloat16** acts[] = {&net->feat, &net->t0, &net->e0, &net->u0, &net->d0,
                              &net->p1,   &net->t1, &net->e1, &net->u1, &net->d1,
                              &net->p2,   &net->t2, &net->e2, &net->u2, &net->d2,
                              &net->p3,   &net->t3, &net->e3};
    for (auto p : acts) {
        if (*p) cudaFree(*p);
        *p = nullptr;
    }
    if (net->out32) cudaFree(net->out32);
    net->out32 = nullptr;
    net->n0 = Dims{0, 0, 0};
}

void net_destroy(void* p) {
    Net* net = static_cast<Net*>(p);
    if (!net) return;
    net_free_acts(net);
    for (int l = 0; l < kNetLayerCount; ++l) {
        if (net->w[l]) cudaFree(net->w[l]);
        if (net->b[l]) cudaFree(net->b[l]);
    }
    if (net->err) cudaFree(net->err);
    delete net;
}

namespace {

__global__ void k_f32_to_bf16(const float* __restrict__ in,
                              __nv_bfloat16* __restrict__ out, long n) {
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n;
         e += (long)gridDim.x * blockDim.x)
        out[e] = __float2bfloat16_rn(in[e]);
}

}  // namespace

// Uploads FP32 parameters in the canonical order: per layer w[27][co][ci]
// then b[co].
jetgpu_status net_load(Ctx* c, const float* params, size_t count) {
    if (count != net_param_count())
        return fail(c, JETGPU_BAD_INPUT, "parameter count does not match the network");
    Net* net = static_cast<Net*>(c->unet);
    if (!net) {
        net = new Net();
        c->unet = net;
        JG_CUDA(c, nalloc(&net->err, 1));
        for (int l = 0; l < kNetLayerCount; ++l) {
            const NetLayer& L = kNetLayers[l];
            JG_CUDA(c, nalloc(&net->w[l], (size_t)27 * L.ci * L.co));
            JG_CUDA(c, nalloc(&net->b[l], (size_t)L.co));
        }
    }
    float* tmp = nullptr;
    JG_CUDA(c, nalloc(&tmp, count));
    JG_CUDA(c, cudaMemcpyAsync(tmp, params, count * sizeof(float),
                               cudaMemcpyHostToDevice, c->stream));
    size_t off = 0;
    for (int l = 0; l < kNetLayerCount; ++l) {
        const NetLayer& L = kNetLayers[l];
        const long nw = 27L * L.ci * L.co;
        k_f32_to_bf16<<<blocks_for(nw), kThreads, 0, c->stream>>>(tmp + off,
                                                                  net->w[l], nw);
        off += nw;
        JG_CUDA(c, cudaMemcpyAsync(net->b[l], tmp + off, L.co * sizeof(float),
                                   cudaMemcpyDeviceToDevice, c->stream));
        off += L.co;
    }
    JG_CUDA(c, cudaStreamSynchronize(c->stream));
    cudaFree(tmp);
    JG_CUDA(c, cudaMemsetAsync(net->err, 0, sizeof(unsigned), c->stream));
    net->loaded = true;
    return JETGPU_OK;
}

static jetgpu_status net_ensure_acts(Ctx* c, Net* net, Dims n) {
    if (net->n0.x == n.x && net->n0.y == n.y && net->n0.z == n.z) return JETGPU_OK;
    net_free_acts(net);
    const size_t V0 = n.count(), V1 = V0 / 8, V2 = V1 / 8, V3 = V2 / 8;
    JG_CUDA(c, nalloc(&net->feat, V0 * 16));
    JG_CUDA(c, nalloc(&net->t0, V0 * 16));
    JG_CUDA(c, nalloc(&net->e0, V0 * 16));
    JG_CUDA(c, nalloc(&net->u0, V0 * 48));
    JG_CUDA(c, nalloc(&net->d0, V0 * 16));
    JG_CUDA(c, nalloc(&net->p1, V1 * 16));
    JG_CUDA(c, nalloc(&net->t1, V1 * 32));
    JG_CUDA(c, nalloc(&net->e1, V1 * 32));
    JG_CUDA(c, nalloc(&net->u1, V1 * 80));
    JG_CUDA(c, nalloc(&net->d1, V1 * 32));
    JG_CUDA(c, nalloc(&net->p2, V2 * 32));
    JG_CUDA(c, nalloc(&net->t2, V2 * 48));
    JG_CUDA(c, nalloc(&net->e2, V2 * 48));
    JG_CUDA(c, nalloc(&net->u2, V2 * 112));
    JG_CUDA(c, nalloc(&net->d2, V2 * 48));
    JG_CUDA(c, nalloc(&net->p3, V3 * 48));
    JG_CUDA(c, nalloc(&net->t3, V3 * 64));
    JG_CUDA(c, nalloc(&net->e3, V3 * 64));
    JG_CUDA(c, nalloc(&net->out32, V0 * 16));
    net->n0 = n;
    return JETGPU_OK;
}

unsigned net_level(const Ctx* c) {
    const unsigned nl = c->built_levels;
    for (unsigned l = 0; l < nl; ++l) {
        const Dims n = c->levels[l].n;
        if (n.x <= 64 && n.y <= 64 && n.z <= 64) return l;
    }
    return nl > 0 ? nl - 1 : 0;
}

bool net_supported(const Ctx* c) {
    const Net* net = static_cast<const Net*>(c->unet);
    if (!net || !net->loaded || c->built_levels == 0) return false;
    const Dims n = c->levels[net_level(c)].n;
    return n.x % 8 == 0 && n.y % 8 == 0 && n.z % 8 == 0 && n.x >= 8 &&
           n.y >= 8 && n.z >= 8;
}

// Builds the 16 input channels of residual r on level `level` of the
// current system. rr: device pointer to sum(r^2).
jetgpu_status net_features(Ctx* c, unsigned level, const float* r,
                           const double* rr, void* feat) {
    const Level& L = c->levels[level];
    const float h2 = (float)(L.h[0] * L.h[0]);
    k_net_features<<<blocks_for(L.n.count()), kThreads, 0, c->stream>>>(
        r, rr, L.n.count(), L.uw, L.vw, L.ww, L.phi, L.A, h2, L.n,
        static_cast<__nv_bfloat16*>(feat));
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

// z = net(r) on level `level` of the current system; rr = device sum(r^2).
jetgpu_status net_apply(Ctx* c, unsigned level, const float* r,
                        const double* rr, float* z) {
    Net* net = static_cast<Net*>(c->unet);
    const Level& L0 = c->levels[level];
    const Dims n0 = L0.n, n1{n0.x / 2, n0.y / 2, n0.z / 2},
               n2{n1.x / 2, n1.y / 2, n1.z / 2}, n3{n2.x / 2, n2.y / 2, n2.z / 2};
    jetgpu_status s = net_ensure_acts(c, net, n0);
    if (s != JETGPU_OK) return s;
    Prof pr(c, K_UNET, 0.0);
    cudaStream_t st = c->stream;
    s = net_features(c, level, r, rr, net->feat);
    if (s != JETGPU_OK) return s;
    auto conv = [&](int l, const __nv_bfloat16* in, Dims n, __nv_bfloat16* out,
                    float* out32) {
        const NetLayer& Ly = kNetLayers[l];
        return conv3d(st, in, Ly.ci, net->w[l], net->b[l], Ly.co, n, Ly.relu,
                      out, out32, net->err);
    };
    auto pool = [&](const __nv_bfloat16* in, Dims fine, int C, __nv_bfloat16* out) {
        k_pool2<<<blocks_for(fine.count() / 8 * C), kThreads, 0, st>>>(in, fine, C, out);
    };
    auto upcat = [&](const __nv_bfloat16* coarse, int C1, const __nv_bfloat16* skip,
                     int C2, Dims fine, __nv_bfloat16* out) {
        k_up_concat<<<blocks_for(fine.count() * (C1 + C2)), kThreads, 0, st>>>(
            coarse, C1, skip, C2, fine, out);
    };
    jetgpu_status e = JETGPU_OK;
    auto chk = [&](jetgpu_status x) { if (x != JETGPU_OK) e = x; };
    chk(conv(0, net->feat, n0, net->t0, nullptr));
    chk(conv(1, net->t0, n0, net->e0, nullptr));
    pool(net->e0, n0, 16, net->p1);
    chk(conv(2, net->p1, n1, net->t1, nullptr));
    chk(conv(3, net->t1, n1, net->e1, nullptr));
    pool(net->e1, n1, 32, net->p2);
    chk(conv(4, net->p2, n2, net->t2, nullptr));
    chk(conv(5, net->t2, n2, net->e2, nullptr));
    pool(net->e2, n2, 48, net->p3);
    chk(conv(6, net->p3, n3, net->t3, nullptr));
    chk(conv(7, net->t3, n3, net->e3, nullptr));
    upcat(net->e3, 64, net->e2, 48, n2, net->u2);
    chk(conv(8, net->u2, n2, net->t2, nullptr));
    chk(conv(9, net->t2, n2, net->d2, nullptr));
    upcat(net->d2, 48, net->e1, 32, n1, net->u1);
    chk(conv(10, net->u1, n1, net->t1, nullptr));
    chk(conv(11, net->t1, n1, net->d1, nullptr));
    upcat(net->d1, 32, net->e0, 16, n0, net->u0);
    chk(conv(12, net->u0, n0, net->d0, nullptr));
    chk(conv(13, net->d0, n0, nullptr, net->out32));
    if (e != JETGPU_OK) return fail(c, e, "convolution launch failed");
    k_net_output<<<blocks_for(n0.count()), kThreads, 0, st>>>(
        net->out32, rr, n0.count(), L0.phi, z);
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

}  // namespace jg

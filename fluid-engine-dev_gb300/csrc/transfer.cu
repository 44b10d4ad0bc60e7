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
// scatter accumulates with FP64 atomics, so sums match the reference's
// serial order to rounding, not bit for bit.

#include "ctx.h"
#include "sampling.cuh"

#include <mutex>

namespace jg {
namespace {

using namespace smp;

// K13a: scatter vel*w and w with FP64 atomics; markers set to 1.
__global__ void k_p2g_scatter(long np, const double* __restrict__ pos,
                              const double* __restrict__ vel, FaceSet fs,
                              double ihx, double ihy, double ihz, double* u,
                              double* v, double* w, double* wu, double* wv,
                              double* ww, unsigned char* mu, unsigned char* mv,
                              unsigned char* mw) {
    double* grid[3] = {u, v, w};
    double* wsum[3] = {wu, wv, ww};
    unsigned char* mark[3] = {mu, mv, mw};
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < np;
         p += (long)gridDim.x * blockDim.x) {
        const double px = pos[3 * p], py = pos[3 * p + 1], pz = pos[3 * p + 2];
        for (int a = 0; a < 3; ++a) {
            const Dims s = fs.s[a];
            const double nx = (px - fs.o[a][0]) * ihx;
            const double ny = (py - fs.o[a][1]) * ihy;
            const double nz = (pz - fs.o[a][2]) * ihz;
            int i, j, k;
            double fx, fy, fz;
            bary<double>(nx, s.x - 1, &i, &fx);
            bary<double>(ny, s.y - 1, &j, &fy);
            bary<double>(nz, s.z - 1, &k, &fz);
            const int ip1 = min(i + 1, s.x - 1), jp1 = min(j + 1, s.y - 1),
                      kp1 = min(k + 1, s.z - 1);
            const long idx[8] = {lin(i, j, k, s.x, s.y),     lin(ip1, j, k, s.x, s.y),
                                 lin(i, jp1, k, s.x, s.y),   lin(ip1, jp1, k, s.x, s.y),
                                 lin(i, j, kp1, s.x, s.y),   lin(ip1, j, kp1, s.x, s.y),
                                 lin(i, jp1, kp1, s.x, s.y), lin(ip1, jp1, kp1, s.x, s.y)};
            const double wt[8] = {(1 - fx) * (1 - fy) * (1 - fz), fx * (1 - fy) * (1 - fz),
                                  (1 - fx) * fy * (1 - fz),       fx * fy * (1 - fz),
                                  (1 - fx) * (1 - fy) * fz,       fx * (1 - fy) * fz,
                                  (1 - fx) * fy * fz,             fx * fy * fz};
            const double va = vel[3 * p + a];
            for (int q = 0; q < 8; ++q) {
                atomicAdd(&grid[a][idx[q]], va * wt[q]);
                atomicAdd(&wsum[a][idx[q]], wt[q]);
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
        if (ws > 0.0) v /= ws;
        g[c] = v;
        if (snap) snap[c] = (float)v;
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
                           const double* __restrict__ w, double hx, double hy,
                           double hz, double blend) {
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
                pic[a] = sample_face<double, double>(
                    g[a], fs.s[a], (px - fs.o[a][0]) / hx,
                    (py - fs.o[a][1]) / hy, (pz - fs.o[a][2]) / hz);
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
                          const double* __restrict__ w, double hx, double hy,
                          double hz) {
    const double* g[3] = {u, v, w};
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < np;
         p += (long)gridDim.x * blockDim.x) {
        const double px = pos[3 * p], py = pos[3 * p + 1], pz = pos[3 * p + 2];
        for (int a = 0; a < 3; ++a)
            vel[3 * p + a] = sample_face<double, double>(
                g[a], fs.s[a], (px - fs.o[a][0]) / hx, (py - fs.o[a][1]) / hy,
                (pz - fs.o[a][2]) / hz);
    }
}

}  // namespace

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
    JG_CUDA(c, cudaMemsetAsync(wsum, 0, need, c->stream));
    for (int a = 0; a < 3; ++a) {
        JG_CUDA(c, cudaMemsetAsync(grid[a], 0, n[a] * sizeof(double), c->stream));
        if (mark[a]) JG_CUDA(c, cudaMemsetAsync(mark[a], 0, n[a], c->stream));
    }
    if (np > 0)
        k_p2g_scatter<<<blocks_for(np, kThreads, c->num_sms * 16), kThreads, 0,
                        c->stream>>>(np, pos, vel, fs, 1.0 / g.spacing[0],
                                     1.0 / g.spacing[1], 1.0 / g.spacing[2],
                                     u, v, w, wsum, wsum + n[0],
                                     wsum + n[0] + n[1], mu, mv, mw);
    long off = 0;
    for (int a = 0; a < 3; ++a) {
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
    if (np > 0)
        k_g2p_flip<<<blocks_for(np), kThreads, 0, c->stream>>>(
            np, pos, vel, fs, (float)g.spacing[0], (float)g.spacing[1],
            (float)g.spacing[2], su, sv, sw, u, v, w, g.spacing[0],
            g.spacing[1], g.spacing[2], blend);
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

jetgpu_status g2p_pic(Ctx* c, const GridDesc& g, long np, const double* pos,
                      double* vel, const double* u, const double* v,
                      const double* w) {
    const FaceSet fs = face_set(g);
    if (np > 0)
        k_g2p_pic<<<blocks_for(np), kThreads, 0, c->stream>>>(
            np, pos, vel, fs, u, v, w, g.spacing[0], g.spacing[1],
            g.spacing[2]);
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
    for (int a = 0; a < 3; ++a)
        if (grid->res[a] < 1 || !(grid->spacing[a] > 0.0))
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
            np, pos, vel, fs, 1.0 / g.spacing[0], 1.0 / g.spacing[1],
            1.0 / g.spacing[2], u, v, w, wsum, wsum + n[0], wsum + n[0] + n[1],
            mu, mv, mw);
    size_t off = 0;
    for (int a = 0; a < 3; ++a) {
        k_p2g_normalize<<<blocks_for((long)n[a]), kThreads, 0, st>>>(
            grids[a], wsum + off, snap[a], (long)n[a]);
        off += n[a];
    }
    return cudaGetLastError() == cudaSuccess ? JETGPU_OK : JETGPU_CUDA_ERROR;
}

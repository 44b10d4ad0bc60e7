// GridSinglePhasePressureSolver3 — the blocked ("Lego brick") pressure
// solver — on the GPU, built into the same multigrid hierarchy as the
// fractional solver so that one MGPCG core serves both.
//
//   buildMarkers           (src/jet/grid_single_phase_pressure_solver3.cpp:245-322)
//   buildSingleSystem      (:26-76, the FdmMatrix3 form)
//   buildSystem            (:341-376)
//   applyPressureGradient  (:378-405)
//
// Markers: a cell is boundary if the collider SDF at its centre is negative,
// else fluid if the fluid SDF there is negative, else air. Coarse levels
// take the majority marker (argmax3 of fluid/air/boundary counts) of the
// 4x4x4 block of finer cells around each coarse cell, taps clamped at the
// edges. Rows: the 7-point Laplacian with h^-2 terms for every non-boundary
// neighbour, off-diagonals to fluid neighbours only, identity rows for
// non-fluid cells, b = the velocity divergence at fluid cell centres.
//
// This unit is compiled with -fmad=false: the cell-centre positions, the
// SDF samples, the divergence and the gradient replay the reference's double
// arithmetic bit for bit.
#include "ctx.h"
#include "sampling.cuh"

namespace jg {
namespace {

using namespace smp;

constexpr unsigned char kMFluid = 0, kMAir = 1, kMBoundary = 2;

struct FieldS {
    FieldDesc f;
    Spacing s[3];
};

FieldS field_s(const FieldDesc& f) {
    FieldS r;
    r.f = f;
    for (int a = 0; a < 3; ++a)
        r.s[a] = make_spacing(f.kind == 1 ? f.spacing[a] : 1.0);
    return r;
}

// ScalarField3::sample: a constant, or LinearArraySampler3 on the grid data.
__device__ __forceinline__ double sample(const FieldS& F, double x, double y,
                                         double z) {
    if (F.f.kind == 0) return F.f.value;
    const Dims s{F.f.res[0], F.f.res[1], F.f.res[2]};
    return sample_face_grid(F.f.data, s,
                                       F.s[0].div(x - F.f.origin[0]),
                                       F.s[1].div(y - F.f.origin[1]),
                                       F.s[2].div(z - F.f.origin[2]));
}

// Level-0 markers (:257-267) at Grid3::cellCenterPosition
// (src/jet/grid3.cpp:32-38): o + h * (i + 0.5).
__global__ void k_blocked_markers(Dims n, GridDesc g, FieldS B, FieldS F,
                                  unsigned char* __restrict__ mk,
                                  float* __restrict__ phi) {
    const long N = n.count();
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_ijk(c, n, i, j, k);
        const double x = g.origin[0] + g.spacing[0] * ((double)i + 0.5);
        const double y = g.origin[1] + g.spacing[1] * ((double)j + 0.5);
        const double z = g.origin[2] + g.spacing[2] * ((double)k + 0.5);
        unsigned char m;
        if (sample(B, x, y, z) < 0.0)
            m = kMBoundary;
        else if (sample(F, x, y, z) < 0.0)
            m = kMFluid;
        else
            m = kMAir;
        mk[c] = m;
        phi[c] = m == kMFluid ? -1.0f : 1.0f;
    }
}

// Coarse markers (:270-317): argmax3 (include/jet/detail/math_utils-inl.h:
// 106-113) of the fluid, air and boundary counts over the clamped 4x4x4
// block of finer cells.
__global__ void k_blocked_coarsen(Dims f, Dims c,
                                  const unsigned char* __restrict__ fine,
                                  unsigned char* __restrict__ coarse,
                                  float* __restrict__ phi) {
    const long N = c.count();
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < N;
         t += (long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_ijk(t, c, i, j, k);
        const int iI[4] = {i > 0 ? 2 * i - 1 : 2 * i, 2 * i, 2 * i + 1,
                           i + 1 < c.x ? 2 * i + 2 : 2 * i + 1};
        const int jI[4] = {j > 0 ? 2 * j - 1 : 2 * j, 2 * j, 2 * j + 1,
                           j + 1 < c.y ? 2 * j + 2 : 2 * j + 1};
        const int kI[4] = {k > 0 ? 2 * k - 1 : 2 * k, 2 * k, 2 * k + 1,
                           k + 1 < c.z ? 2 * k + 2 : 2 * k + 1};
        int cnt[3] = {0, 0, 0};
#pragma unroll
        for (int z = 0; z < 4; ++z)
#pragma unroll
            for (int y = 0; y < 4; ++y) {
                const unsigned char* row = fine + lin(0, jI[y], kI[z], f.x, f.y);
#pragma unroll
                for (int x = 0; x < 4; ++x) {
                    const unsigned char v = row[iI[x]];
                    ++cnt[v == kMBoundary ? 2 : (v == kMFluid ? 0 : 1)];
                }
            }
        const unsigned char m =
            cnt[0] > cnt[1] ? (cnt[0] > cnt[2] ? 0 : 2)
                            : (cnt[1] > cnt[2] ? 1 : 2);
        coarse[t] = m;
        phi[t] = m == kMFluid ? -1.0f : 1.0f;
    }
}

// buildSingleSystem (:26-76) on one level. isq = (1/h)^2 per axis as the
// reference computes it (invH * invH, invH = 1.0 / h); hs divides the face
// differences for the divergence (src/jet/face_centered_grid3.cpp:137-152).
// u/v/w are null on coarse levels, whose right-hand sides the multigrid
// overwrites by restriction (include/jet/detail/mg-inl.h:28-30). Outputs as
// k_build_system: FP32 rows (structure of arrays) on every level; on the
// finest level the exact FP64 rows and b and their double-float low parts.
__global__ void k_blocked_system(Dims n, double isx, double isy, double isz,
                                 Spacing hx, Spacing hy, Spacing hz,
                                 const unsigned char* __restrict__ mk,
                                 const double* __restrict__ u,
                                 const double* __restrict__ v,
                                 const double* __restrict__ w,
                                 double* __restrict__ A64,
                                 double* __restrict__ b64,
                                 float* __restrict__ A32,
                                 float4* __restrict__ Alo,
                                 float2* __restrict__ bdf) {
    const long N = n.count();
    const long sy = n.x, sz = (long)n.x * n.y;
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_ijk(c, n, i, j, k);
        double center = 0.0, right = 0.0, up = 0.0, front = 0.0, bb = 0.0;
        const bool fluid = mk[c] == kMFluid;
        if (fluid) {
            if (u) {
                const double du = u[lin(i + 1, j, k, n.x + 1, n.y)] -
                                  u[lin(i, j, k, n.x + 1, n.y)];
                const double dv = v[lin(i, j + 1, k, n.x, n.y + 1)] -
                                  v[lin(i, j, k, n.x, n.y + 1)];
                const double dw = w[lin(i, j, k + 1, n.x, n.y)] -
                                  w[lin(i, j, k, n.x, n.y)];
                bb = hx.div(du) + hy.div(dv) + hz.div(dw);
            }
            if (i + 1 < n.x && mk[c + 1] != kMBoundary) {
                center += isx;
                if (mk[c + 1] == kMFluid) right = -isx;
            }
            if (i > 0 && mk[c - 1] != kMBoundary) center += isx;
            if (j + 1 < n.y && mk[c + sy] != kMBoundary) {
                center += isy;
                if (mk[c + sy] == kMFluid) up = -isy;
            }
            if (j > 0 && mk[c - sy] != kMBoundary) center += isy;
            if (k + 1 < n.z && mk[c + sz] != kMBoundary) {
                center += isz;
                if (mk[c + sz] == kMFluid) front = -isz;
            }
            if (k > 0 && mk[c - sz] != kMBoundary) center += isz;
        } else {
            center = 1.0;
        }
        if (A64) {
            A64[4 * c + 0] = center;
            A64[4 * c + 1] = right;
            A64[4 * c + 2] = up;
            A64[4 * c + 3] = front;
        }
        if (b64) b64[c] = bb;
        float4 hi4, lo4;
        float bh, bl;
        split_f64(center, hi4.x, lo4.x);
        split_f64(right, hi4.y, lo4.y);
        split_f64(up, hi4.z, lo4.z);
        split_f64(front, hi4.w, lo4.w);
        split_f64(bb, bh, bl);
        A32[c] = hi4.x;
        A32[N + c] = hi4.y;
        A32[2 * N + c] = hi4.z;
        A32[3 * N + c] = hi4.w;
        if (Alo) Alo[c] = lo4;
        if (bdf) bdf[c] = make_float2(bh, bl);
    }
}

// applyPressureGradient (:378-405): for a fluid cell, each of its +x/+y/+z
// faces whose neighbour is not a boundary cell gets u + invH * (x_n - x_c).
// The thread of cell c owns the faces i+1/j+1/k+1 of c, and the cells on
// the lower domain boundary also own faces 0, so every output face is
// written once; with `copy` false (output aliasing the input) untouched
// faces are skipped.
__global__ void k_blocked_gradient(Dims n, double ihx, double ihy, double ihz,
                                   const unsigned char* __restrict__ mk,
                                   const double* __restrict__ x,
                                   const double* u, const double* v,
                                   const double* w, double* ou, double* ov,
                                   double* ow, int copy) {
    const long N = n.count();
    const int ux = n.x + 1;
    const long sy = n.x, sz = (long)n.x * n.y;
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_ijk(c, n, i, j, k);
        const bool fluid = mk[c] == kMFluid;
        auto face = [&](bool inner, long f, long nbc, double ih,
                        const double* in, double* out) {
            if (inner && fluid && mk[nbc] != kMBoundary) {
                out[f] = in[f] + ih * (x[nbc] - x[c]);
                return;
            }
            if (copy) out[f] = in[f];
        };
        face(i + 1 < n.x, lin(i + 1, j, k, ux, n.y), c + 1, ihx, u, ou);
        face(j + 1 < n.y, lin(i, j + 1, k, n.x, n.y + 1), c + sy, ihy, v, ov);
        face(k + 1 < n.z, lin(i, j, k + 1, n.x, n.y), c + sz, ihz, w, ow);
        if (copy) {
            if (i == 0) ou[lin(0, j, k, ux, n.y)] = u[lin(0, j, k, ux, n.y)];
            if (j == 0) ov[lin(i, 0, k, n.x, n.y + 1)] = v[lin(i, 0, k, n.x, n.y + 1)];
            if (k == 0) ow[lin(i, j, 0, n.x, n.y)] = w[lin(i, j, 0, n.x, n.y)];
        }
    }
}

}  // namespace

static jetgpu_status blocked_scratch(Ctx* c, size_t* offs) {
    if (c->built_levels > 32)
        return fail(c, JETGPU_BAD_INPUT, "more than 32 multigrid levels");
    size_t total = 0;
    for (unsigned l = 0; l < c->built_levels; ++l) {
        offs[l] = total;
        total += (size_t)c->levels[l].n.count();
    }
    if (total > c->blk_cap) {
        if (c->blk_marks) cudaFree(c->blk_marks);
        c->blk_marks = nullptr;
        c->blk_cap = 0;
        JG_CUDA(c, cudaMalloc((void**)&c->blk_marks, total));
        c->blk_cap = total;
    }
    return JETGPU_OK;
}

jetgpu_status blocked_markers(Ctx* c, const GridDesc& g, const FieldDesc& bsdf,
                              const FieldDesc& fsdf) {
    size_t off[32];
    jetgpu_status s = blocked_scratch(c, off);
    if (s != JETGPU_OK) return s;
    const FieldS B = field_s(bsdf), F = field_s(fsdf);
    for (unsigned l = 0; l < c->built_levels; ++l) {
        Level& L = c->levels[l];
        const long N = L.n.count();
        Prof pr(c, K_WEIGHTS, (l == 0 ? 5.0 + 16.0 : 8.0 + 5.0) * (double)N);
        if (l == 0) {
            k_blocked_markers<<<blocks_for(N), kThreads, 0, c->stream>>>(
                L.n, g, B, F, c->blk_marks, L.phi);
        } else {
            k_blocked_coarsen<<<blocks_for(N), kThreads, 0, c->stream>>>(
                c->levels[l - 1].n, L.n, c->blk_marks + off[l - 1],
                c->blk_marks + off[l], L.phi);
        }
    }
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

jetgpu_status blocked_system(Ctx* c, const GridDesc& g, const double* u,
                             const double* v, const double* w) {
    size_t off[32];
    jetgpu_status s = blocked_scratch(c, off);
    if (s != JETGPU_OK) return s;
    double h[3] = {g.spacing[0], g.spacing[1], g.spacing[2]};
    for (unsigned l = 0; l < c->built_levels; ++l) {
        Level& L = c->levels[l];
        if (l > 0)
            for (double& x : h) x *= 2.0;
        for (int a = 0; a < 3; ++a) L.h[a] = h[a];
        const double ih[3] = {1.0 / h[0], 1.0 / h[1], 1.0 / h[2]};
        const bool top = (l == 0);
        const long N = L.n.count();
        Prof pr(c, K_SYSTEM, (top ? 1.0 + 24.0 + 32.0 + 8.0 + 16.0 + 24.0
                                  : 1.0 + 16.0) * (double)N);
        k_blocked_system<<<blocks_for(N), kThreads, 0, c->stream>>>(
            L.n, ih[0] * ih[0], ih[1] * ih[1], ih[2] * ih[2],
            make_spacing(h[0]), make_spacing(h[1]), make_spacing(h[2]),
            c->blk_marks + off[l], top ? u : nullptr, top ? v : nullptr,
            top ? w : nullptr, top ? c->A64 : nullptr, top ? c->b64 : nullptr,
            L.A, top ? c->Alo : nullptr, top ? c->bdf : nullptr);
    }
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

jetgpu_status blocked_gradient(Ctx* c, const GridDesc& g, const double* u,
                               const double* v, const double* w, double* ou,
                               double* ov, double* ow) {
    const Dims n = c->levels[0].n;
    const bool alias = (ou == u) && (ov == v) && (ow == w);
    if (!alias && ((ou == u) || (ov == v) || (ow == w)))
        return fail(c, JETGPU_BAD_INPUT,
                    "output faces must all alias the input or none");
    Prof pr(c, K_GRADIENT, (1.0 + 8.0 + 48.0) * (double)n.count());
    k_blocked_gradient<<<blocks_for(n.count()), kThreads, 0, c->stream>>>(
        n, 1.0 / g.spacing[0], 1.0 / g.spacing[1], 1.0 / g.spacing[2],
        c->blk_marks, c->x64, u, v, w, ou, ov, ow, alias ? 0 : 1);
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

}  // namespace jg

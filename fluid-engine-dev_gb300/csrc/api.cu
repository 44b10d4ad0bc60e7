// C ABI of libjetgpu (include/jetgpu.h): context lifetime, buffer
// management, input validation and the pressure-projection pipeline.

#include "ctx.h"

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>

struct jetgpu_ctx : public jg::Ctx {};

namespace jg {

jetgpu_status fail(Ctx* c, jetgpu_status s, const std::string& msg) {
    if (c) c->err = msg;
    return s;
}

namespace {

// A solve whose result is applied: converged, capped, or finished by the
// multigrid fallback after the learned preconditioner stalled.
bool usable(jetgpu_status s) {
    return s == JETGPU_OK || s == JETGPU_NOT_CONVERGED ||
           s == JETGPU_STALLED_FALLBACK_USED;
}

template <typename T>
cudaError_t alloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) return cudaSuccess;
    return cudaMalloc((void**)p, count * sizeof(T));
}

template <typename T>
void release(T** p) {
    if (*p) cudaFree((void*)*p);
    *p = nullptr;
}

// Frees the multigrid hierarchy. The captured V-cycle graph (vc_exec) bakes
// in the level buffers' addresses and the TMA tensor maps made from them, so
// it is destroyed here, and every path that reallocates level buffers must
// come through this function. A capture that failed on the old buffers is
// allowed again on the new ones.
void free_buffers(Ctx* c) {
    if (c->vc_exec) {
        cudaGraphExecDestroy(c->vc_exec);
        c->vc_exec = nullptr;
    }
    if (c->loop_exec) {
        cudaGraphExecDestroy(c->loop_exec);
        c->loop_exec = nullptr;
    }
    c->vc_disabled = false;
    c->loop_disabled = false;
    for (Level& L : c->levels) {
        release(&L.phi);
        release(&L.uw);
        release(&L.vw);
        release(&L.ww);
        release(&L.A);
        release(&L.Ah);
        release(&L.x);
        release(&L.x2);
        release(&L.b);
        release(&L.r);
    }
    c->levels.clear();
    release(&c->A64);
    release(&c->b64);
    release(&c->x64);
    release(&c->r64);
    release(&c->Alo);
    release(&c->bdf);
    release(&c->xdf);
    release(&c->kx);
    release(&c->kr);
    release(&c->kd);
    release(&c->kq);
    release(&c->kz);
    release(&c->kz2);
    release(&c->dx);
    release(&c->dr);
    release(&c->dd);
    release(&c->dq);
    release(&c->dz);
    c->n0 = Dims{0, 0, 0};
    c->built_levels = 0;
}

double ms_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(
               std::chrono::steady_clock::now() - t0)
        .count();
}

jetgpu_status check_config(Ctx* c, const jetgpu_config* cfg) {
    if (!cfg) return fail(c, JETGPU_BAD_INPUT, "null config");
    if (cfg->max_levels < 1) return fail(c, JETGPU_BAD_INPUT, "max_levels < 1");
    if (!(cfg->tolerance >= 0.0))
        return fail(c, JETGPU_BAD_INPUT, "tolerance must be >= 0");
    if (!(cfg->sor > 0.0 && cfg->sor < 2.0))
        return fail(c, JETGPU_BAD_INPUT, "sor must be in (0, 2)");
    if (!cfg->red_black)
        return fail(c, JETGPU_BAD_INPUT,
                    "only red-black smoothing is provided on the GPU");
    if (cfg->precision < 0 || cfg->precision > 2)
        return fail(c, JETGPU_BAD_INPUT, "unknown precision");
    if (cfg->preconditioner < 0 || cfg->preconditioner > 2)
        return fail(c, JETGPU_BAD_INPUT, "unknown preconditioner");
    return JETGPU_OK;
}

jetgpu_status check_grid(Ctx* c, const jetgpu_grid* g) {
    if (!g) return fail(c, JETGPU_BAD_INPUT, "null grid");
    for (int a = 0; a < 3; ++a) {
        if (g->res[a] < 1) return fail(c, JETGPU_BAD_INPUT, "resolution < 1");
        if (!(g->spacing[a] > 0.0) || !std::isfinite(g->spacing[a]))
            return fail(c, JETGPU_BAD_INPUT, "grid spacing must be > 0");
        if (!std::isfinite(g->origin[a]))
            return fail(c, JETGPU_BAD_INPUT, "non-finite origin");
    }
    const double cells = (double)g->res[0] * g->res[1] * g->res[2];
    if (cells > 2147483647.0)
        return fail(c, JETGPU_BAD_INPUT, "grid too large");
    return JETGPU_OK;
}

jetgpu_status check_field(Ctx* c, const jetgpu_scalar_field* f,
                          const char* name) {
    if (!f) return fail(c, JETGPU_BAD_INPUT, std::string("null ") + name);
    if (f->kind == 0) return JETGPU_OK;
    if (f->kind != 1)
        return fail(c, JETGPU_BAD_INPUT, std::string(name) + ": unknown kind");
    if (!f->data) return fail(c, JETGPU_BAD_INPUT, std::string(name) + ": null data");
    for (int a = 0; a < 3; ++a) {
        if (f->res[a] < 1)
            return fail(c, JETGPU_BAD_INPUT, std::string(name) + ": resolution < 1");
        if (!(f->spacing[a] > 0.0))
            return fail(c, JETGPU_BAD_INPUT, std::string(name) + ": spacing <= 0");
    }
    return JETGPU_OK;
}

FieldDesc to_desc(const jetgpu_scalar_field* f, const double* data) {
    FieldDesc d;
    d.kind = f->kind;
    d.value = f->value;
    d.data = data;
    for (int a = 0; a < 3; ++a) {
        d.res[a] = f->res[a];
        d.origin[a] = f->origin[a];
        d.spacing[a] = f->spacing[a];
    }
    return d;
}

GridDesc to_desc(const jetgpu_grid* g) {
    GridDesc d;
    for (int a = 0; a < 3; ++a) {
        d.res[a] = g->res[a];
        d.spacing[a] = g->spacing[a];
        d.origin[a] = g->origin[a];
    }
    return d;
}

long field_count(const jetgpu_scalar_field* f) {
    return f->kind == 1 ? (long)f->res[0] * f->res[1] * f->res[2] : 0;
}

__global__ void k_rows_to_f32(const double* __restrict__ A, float* __restrict__ out,
                              long N) {
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x)
        for (int k = 0; k < 4; ++k) out[k * N + c] = (float)A[4 * c + k];
}

__global__ void k_fill_f32(float* __restrict__ p, float v, long N) {
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x)
        p[c] = v;
}

__global__ void k_rows_f32_to_f64(const float* __restrict__ A,
                                  double* __restrict__ out, long N) {
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x) {
        out[4 * c] = A[c];
        out[4 * c + 1] = A[N + c];
        out[4 * c + 2] = A[2 * N + c];
        out[4 * c + 3] = A[3 * N + c];
    }
}

// The bounding box of the fluid cells (phi < 0): box = (i0, j0, k0, i1, j1,
// k1), empty when i1 < i0. A block reduces its cells, then one atomic per
// bound and block.
__global__ void k_box_init(int* box) {
    box[0] = box[1] = box[2] = 0x7fffffff;
    box[3] = box[4] = box[5] = -1;
}
__global__ void k_fluid_box(const double* __restrict__ phi, Dims n,
                            int* __restrict__ box) {
    __shared__ int sb[6];
    if (threadIdx.x < 6) sb[threadIdx.x] = threadIdx.x < 3 ? 0x7fffffff : -1;
    __syncthreads();
    int lo[3] = {0x7fffffff, 0x7fffffff, 0x7fffffff}, hi[3] = {-1, -1, -1};
    const long N = n.count();
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x) {
        if (phi[c] < 0.0) {
            int i, j, k;
            cell_ijk(c, n, i, j, k);
            lo[0] = min(lo[0], i); lo[1] = min(lo[1], j); lo[2] = min(lo[2], k);
            hi[0] = max(hi[0], i); hi[1] = max(hi[1], j); hi[2] = max(hi[2], k);
        }
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[d] = min(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
            hi[d] = max(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
        }
    }
    if ((threadIdx.x & 31) == 0)
        for (int d = 0; d < 3; ++d) {
            atomicMin(&sb[d], lo[d]);
            atomicMax(&sb[3 + d], hi[d]);
        }
    __syncthreads();
    if (threadIdx.x < 3) atomicMin(&box[threadIdx.x], sb[threadIdx.x]);
    else if (threadIdx.x < 6) atomicMax(&box[threadIdx.x], sb[threadIdx.x]);
}

jetgpu_status grow_stage(Ctx* c, size_t bytes) {
    if (bytes <= c->stage_bytes) return JETGPU_OK;
    release(&c->stage);
    c->stage_bytes = 0;
    JG_CUDA(c, cudaMalloc((void**)&c->stage, bytes));
    c->stage_bytes = bytes;
    return JETGPU_OK;
}

}  // namespace

// (Re)allocates the hierarchy for resolution n. Reallocation goes through
// free_buffers, which also drops the captured V-cycle graph built on the old
// buffers.
jetgpu_status ensure_buffers(Ctx* c, Dims n, unsigned max_levels) {
    const unsigned nl = level_count(n, max_levels);
    if (c->n0.x == n.x && c->n0.y == n.y && c->n0.z == n.z &&
        c->built_levels == nl)
        return JETGPU_OK;
    JG_CUDA(c, cudaStreamSynchronize(c->stream));
    JG_CUDA(c, cudaStreamSynchronize(c->side_stream));
    free_buffers(c);
    c->levels.resize(nl);
    Dims s = n;
    for (unsigned l = 0; l < nl; ++l) {
        Level& L = c->levels[l];
        L.n = s;
        const long N = s.count();
        JG_CUDA(c, alloc(&L.phi, N));
        JG_CUDA(c, alloc(&L.uw, (size_t)(s.x + 1) * s.y * s.z));
        JG_CUDA(c, alloc(&L.vw, (size_t)s.x * (s.y + 1) * s.z));
        JG_CUDA(c, alloc(&L.ww, (size_t)s.x * s.y * (s.z + 1)));
        JG_CUDA(c, alloc(&L.A, 4 * (size_t)N));
        JG_CUDA(c, alloc(&L.Ah, 4 * (size_t)N));
        JG_CUDA(c, alloc(&L.x, N));
        JG_CUDA(c, alloc(&L.x2, N));
        JG_CUDA(c, alloc(&L.b, N));
        JG_CUDA(c, alloc(&L.r, N));
        s = Dims{s.x / 2, s.y / 2, s.z / 2};
    }
    const long N = n.count();
    JG_CUDA(c, alloc(&c->A64, 4 * (size_t)N));
    JG_CUDA(c, alloc(&c->b64, N));
    JG_CUDA(c, alloc(&c->x64, N));
    JG_CUDA(c, alloc(&c->r64, N));
    JG_CUDA(c, alloc(&c->Alo, N));
    JG_CUDA(c, alloc(&c->bdf, N));
    JG_CUDA(c, alloc(&c->xdf, N));
    JG_CUDA(c, alloc(&c->kx, N));
    JG_CUDA(c, alloc(&c->kr, N));
    JG_CUDA(c, alloc(&c->kd, N));
    JG_CUDA(c, alloc(&c->kq, N));
    JG_CUDA(c, alloc(&c->kz, N));
    JG_CUDA(c, alloc(&c->kz2, N));
    JG_CUDA(c, alloc(&c->dd, N));
    JG_CUDA(c, alloc(&c->dq, N));
    c->n0 = n;
    c->built_levels = nl;
    return JETGPU_OK;
}

// Runs the launches issued inside its scope on `st` instead of the
// compute stream.
struct OnStream {
    Ctx* c;
    cudaStream_t saved;
    OnStream(Ctx* ctx, cudaStream_t st) : c(ctx), saved(ctx->stream) {
        c->stream = st;
    }
    ~OnStream() { c->stream = saved; }
};

// Everything after the finest level's weights: the coarse levels (weight
// pyramid, rows, BF16 copies) need only those weights, the finest level's
// FP64 rows also the velocities. The coarse levels are built on the
// high-priority side stream while the finest rows are built on the compute
// stream: that kernel is FP64-bound, and the pyramid's memory-bound
// restrictions take the SM slots its blocks free. With host inputs, the
// coarse levels are built while the velocities still upload. The live
// profile times launches on the compute stream, so with it on everything
// stays on that stream.
static jetgpu_status build_levels(Ctx* c, const GridDesc& g, const double* u,
                                  const double* v, const double* w,
                                  const double* su, const double* sv,
                                  const double* sw, const SolveIo* io) {
    const bool fork = !c->prof_on && c->built_levels > 1;
    jetgpu_status s = JETGPU_OK;
    if (fork) {
        JG_CUDA(c, cudaEventRecord(c->side_ev[0], c->stream));
        JG_CUDA(c, cudaStreamWaitEvent(c->side_stream, c->side_ev[0], 0));
    }
    {
        OnStream on(c, fork ? c->side_stream : c->stream);
        if ((s = build_pyramid(c)) != JETGPU_OK) return s;
        if ((s = build_system(c, g, nullptr, nullptr, nullptr, nullptr,
                              nullptr, nullptr, 1)) != JETGPU_OK)
            return s;
        if ((s = prepare_levels(c, 1)) != JETGPU_OK) return s;
        if (fork) JG_CUDA(c, cudaEventRecord(c->side_ev[1], c->stream));
    }
    if (io) {
        // Host inputs: the finest rows while the velocities upload, the rhs
        // once they are in.
        if ((s = build_system0_rows(c, g)) != JETGPU_OK) return s;
        if ((s = prepare_levels(c, 0, 1)) != JETGPU_OK) return s;
        if (io->before_vel && (s = io->before_vel()) != JETGPU_OK) return s;
        JG_CUDA(c, cudaStreamWaitEvent(c->stream, io->vel_in, 0));
        if ((s = build_system0_rhs(c, g, u, v, w, su, sv, sw)) != JETGPU_OK)
            return s;
    } else {
        if ((s = build_system(c, g, u, v, w, su, sv, sw, 0, 1)) != JETGPU_OK)
            return s;
        if ((s = prepare_levels(c, 0, 1)) != JETGPU_OK) return s;
    }
    if (fork) JG_CUDA(c, cudaStreamWaitEvent(c->stream, c->side_ev[1], 0));
    return JETGPU_OK;
}

// The device-resident pipeline shared by the host and device entry points.
jetgpu_status solve_pressure_dev(
    Ctx* c, const jetgpu_grid* grid, const double* u, const double* v,
    const double* w, const jetgpu_scalar_field* bsdf, const double* bdata,
    const jetgpu_scalar_field* fsdf, const double* fdata, const double* su,
    const double* sv, const double* sw, double* ou, double* ov, double* ow,
    double* op, jetgpu_solve_stats* st, const SolveIo* io, bool blocked) {
    auto t0 = std::chrono::steady_clock::now();
    const Dims n{grid->res[0], grid->res[1], grid->res[2]};
    jetgpu_status s = ensure_buffers(c, n, c->cfg.max_levels);
    if (s != JETGPU_OK) return s;
    const GridDesc g = to_desc(grid);
    // Set-up and solve times come from events on the stream, so the host
    // never waits between the set-up kernels and the solve.
    JG_CUDA(c, cudaEventRecord(c->ev[0], c->stream));
    if (io)
        JG_CUDA(c, cudaStreamWaitEvent(c->stream,
                                       blocked ? io->sdf_in : io->bsdf_in, 0));
    s = blocked ? blocked_markers(c, g, to_desc(bsdf, bdata), to_desc(fsdf, fdata))
                : build_weights(c, g, to_desc(bsdf, bdata), to_desc(fsdf, fdata),
                                false, io ? io->sdf_in : nullptr);
    if (s != JETGPU_OK) return s;
    if (!blocked) {
        s = build_levels(c, g, u, v, w, su, sv, sw, io);
        if (s != JETGPU_OK) return s;
    } else {
        if (io && io->before_vel && (s = io->before_vel()) != JETGPU_OK)
            return s;
        if (io) JG_CUDA(c, cudaStreamWaitEvent(c->stream, io->vel_in, 0));
        s = blocked_system(c, g, u, v, w);
        if (s != JETGPU_OK) return s;
        s = prepare_levels(c);
        if (s != JETGPU_OK) return s;
    }
    JG_CUDA(c, cudaEventRecord(c->ev[1], c->stream));
    jetgpu_status solve_status = mgpcg_solve(c, st);
    if (!usable(solve_status))
        return solve_status;
    JG_CUDA(c, cudaEventRecord(c->ev[2], c->stream));
    if (io && io->host_p)
        JG_CUDA(c, cudaEventRecord(io->x_final, c->stream));
    // The reference applies the gradient whatever the solver returned
    // (grid_fractional_single_phase_pressure_solver3.cpp:466-483,
    // grid_single_phase_pressure_solver3.cpp:194-210).
    const int slabs = (io && io->grad_slabs && !blocked) ? *io->grad_slabs : 0;
    if (blocked) {
        s = blocked_gradient(c, g, u, v, w, ou, ov, ow);
    } else if (slabs > 0) {
        for (int k = 0; k < slabs; ++k) {
            s = apply_gradient(c, g, u, v, w, ou, ov, ow, io->grad_cuts[k],
                               io->grad_cuts[k + 1]);
            if (s != JETGPU_OK) return s;
            JG_CUDA(c, cudaEventRecord(c->grad_ev[k], c->stream));
        }
    } else {
        s = apply_gradient(c, g, u, v, w, ou, ov, ow);
    }
    if (s != JETGPU_OK) return s;
    // Issued after the gradient launch, so that a pageable destination
    // (whose copy blocks the host) still overlaps the gradient kernel.
    if (io && io->host_p) {
        JG_CUDA(c, cudaStreamWaitEvent(io->copy, io->x_final, 0));
        JG_CUDA(c, cudaMemcpyAsync(io->host_p, c->x64,
                                   n.count() * sizeof(double),
                                   cudaMemcpyDeviceToHost, io->copy));
    }
    if (op)
        JG_CUDA(c, cudaMemcpyAsync(op, c->x64, n.count() * sizeof(double),
                                   cudaMemcpyDeviceToDevice, c->stream));
    if (io && io->after_grad && (s = io->after_grad()) != JETGPU_OK) return s;
    JG_CUDA(c, cudaStreamSynchronize(c->stream));
    float setup = 0.0f, solve = 0.0f;
    JG_CUDA(c, cudaEventElapsedTime(&setup, c->ev[0], c->ev[1]));
    JG_CUDA(c, cudaEventElapsedTime(&solve, c->ev[1], c->ev[2]));
    st->levels = c->built_levels;
    st->setup_ms = setup;
    st->solve_ms = solve;
    st->total_ms = ms_since(t0);
    return solve_status;
}

}  // namespace jg

using namespace jg;

extern "C" {

const char* jetgpu_version(void) { return "jetgpu 0.1 (sm_103a)"; }

void jetgpu_config_default(jetgpu_config* cfg) {
    if (!cfg) return;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->device = 0;
    cfg->max_cg_iter = 100;
    cfg->max_levels = 6;
    cfg->restrict_iter = 2;
    cfg->correct_iter = 2;
    cfg->coarsest_iter = 5;
    cfg->final_iter = 2;
    cfg->tolerance = 1e-6;
    cfg->sor = 1.2;
    cfg->red_black = 1;
    cfg->precision = JETGPU_PRECISION_FP32;
    cfg->preconditioner = JETGPU_PRECOND_MULTIGRID;
    cfg->max_refinements = 6;
    cfg->ordered_p2g = 1;
}

jetgpu_status jetgpu_create(const jetgpu_config* cfg, jetgpu_ctx** out) {
    if (!out) return JETGPU_BAD_INPUT;
    *out = nullptr;
    jetgpu_ctx* c = new (std::nothrow) jetgpu_ctx();
    if (!c) return JETGPU_OUT_OF_MEMORY;
    jetgpu_config def;
    jetgpu_config_default(&def);
    const jetgpu_config* use = cfg ? cfg : &def;
    jetgpu_status s = check_config(c, use);
    if (s != JETGPU_OK) {
        delete c;
        return s;
    }
    c->cfg = *use;
    c->device = use->device;
    auto init = [&]() -> jetgpu_status {
        JG_CUDA(c, cudaSetDevice(c->device));
        JG_CUDA(c, cudaDeviceGetAttribute(&c->num_sms,
                                          cudaDevAttrMultiProcessorCount,
                                          c->device));
        JG_CUDA(c, cudaStreamCreateWithFlags(&c->stream,
                                             cudaStreamNonBlocking));
        JG_CUDA(c, cudaStreamCreateWithFlags(&c->copy_stream,
                                             cudaStreamNonBlocking));
        int least = 0, greatest = 0;
        JG_CUDA(c, cudaDeviceGetStreamPriorityRange(&least, &greatest));
        JG_CUDA(c, cudaStreamCreateWithPriority(&c->side_stream,
                                                cudaStreamNonBlocking,
                                                greatest));
        for (auto& e : c->io_ev)
            JG_CUDA(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        for (auto& e : c->grad_ev)
            JG_CUDA(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        for (auto& e : c->side_ev)
            JG_CUDA(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        JG_CUDA(c, cudaMalloc((void**)&c->scal, S_COUNT * sizeof(double)));
        JG_CUDA(c, cudaMemset(c->scal, 0, S_COUNT * sizeof(double)));
        JG_CUDA(c, cudaMalloc((void**)&c->partials,
                              (size_t)kRedSlots * kMaxRedBlocks * sizeof(double)));
        JG_CUDA(c, cudaMalloc((void**)&c->counters, kRedSlots * sizeof(unsigned)));
        JG_CUDA(c, cudaMemset(c->counters, 0, kRedSlots * sizeof(unsigned)));
        JG_CUDA(c, cudaMallocHost((void**)&c->h_scal, S_COUNT * sizeof(double)));
        JG_CUDA(c, cudaMalloc((void**)&c->box_dev, 6 * sizeof(int)));
        JG_CUDA(c, cudaMallocHost((void**)&c->box_host, 6 * sizeof(int)));
        JG_CUDA(c, cudaEventCreateWithFlags(&c->box_ev, cudaEventDisableTiming));
        for (auto& e : c->ev) JG_CUDA(c, cudaEventCreate(&e));
        jetgpu_status k = init_kernels(c);
        if (k != JETGPU_OK) return k;
        return JETGPU_OK;
    };
    s = init();
    if (s != JETGPU_OK) {
        jetgpu_destroy(c);
        return s;
    }
    *out = c;
    return JETGPU_OK;
}

void jetgpu_destroy(jetgpu_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
    if (c->side_stream) cudaStreamSynchronize(c->side_stream);
    free_buffers(c);
    release(&c->scal);
    release(&c->partials);
    release(&c->counters);
    release(&c->stage);
    release(&c->pscratch);
    release(&c->p2g_int);
    release(&c->p2g_dbl);
    release(&c->bc_tmp);
    release(&c->bc_valid);
    release(&c->bc_cls);
    release(&c->bc_list);
    release(&c->bc_cnt);
    release(&c->bc_nrm);
    release(&c->bc_flag);
    release(&c->rflag);
    release(&c->xp_int);
    release(&c->xp_cnt);
    release(&c->sdf_int);
    release(&c->sdf_dbl);
    release(&c->sdf_valid);
    release(&c->blk_marks);
    release(&c->build_list);
    release(&c->build_cnt);
    release(&c->flip_marks);
    release(&c->flip_snap);
    release(&c->flip_solid);
    release(&c->flip_cfl);
    net_destroy(c->unet);
    c->unet = nullptr;
    if (c->h_scal) cudaFreeHost(c->h_scal);
    if (c->host_stage) cudaFreeHost(c->host_stage);
    for (auto& e : c->ev)
        if (e) cudaEventDestroy(e);
    for (auto& e : c->prof_ev) cudaEventDestroy(e);
    {
        SampleTables& T = c->tabs;
        release(&T.idx);
        release(&T.frac);
        release(&T.slot);
        release(&T.sidx);
        release(&T.sfrac);
        release(&T.irregular);
        release(&T.node);
    }
    for (auto& e : c->io_ev)
        if (e) cudaEventDestroy(e);
    for (auto& e : c->grad_ev)
        if (e) cudaEventDestroy(e);
    if (c->box_ev) cudaEventDestroy(c->box_ev);
    release(&c->box_dev);
    if (c->box_host) cudaFreeHost(c->box_host);
    for (auto& e : c->side_ev)
        if (e) cudaEventDestroy(e);
    if (c->side_stream) cudaStreamDestroy(c->side_stream);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

const char* jetgpu_last_error(const jetgpu_ctx* c) {
    return c ? c->err.c_str() : "null context";
}

jetgpu_status jetgpu_set_config(jetgpu_ctx* c, const jetgpu_config* cfg) {
    if (!c) return JETGPU_BAD_INPUT;
    jetgpu_status s = check_config(c, cfg);
    if (s != JETGPU_OK) return s;
    if (cfg->device != c->device)
        return fail(c, JETGPU_BAD_INPUT, "device cannot change on a context");
    c->cfg = *cfg;
    return JETGPU_OK;
}

static jetgpu_status solve_device(
    jetgpu_ctx* c, const jetgpu_grid* grid, const double* u, const double* v,
    const double* w, const jetgpu_scalar_field* boundary_sdf,
    const jetgpu_scalar_field* fluid_sdf, const double* solid_u,
    const double* solid_v, const double* solid_w, double* out_u,
    double* out_v, double* out_w, double* out_pressure,
    jetgpu_solve_stats* stats, bool blocked,
    const jetgpu_collider* collider = nullptr) {
    if (!c) return JETGPU_BAD_INPUT;
    jetgpu_status s = check_grid(c, grid);
    if (s != JETGPU_OK) return s;
    if (!u || !v || !w || !out_u || !out_v || !out_w)
        return fail(c, JETGPU_BAD_INPUT, "null velocity pointer");
    if ((s = check_field(c, boundary_sdf, "boundary_sdf")) != JETGPU_OK) return s;
    if ((s = check_field(c, fluid_sdf, "fluid_sdf")) != JETGPU_OK) return s;
    JG_CUDA(c, cudaSetDevice(c->device));
    jetgpu_solve_stats local;
    std::memset(&local, 0, sizeof(local));
    s = solve_pressure_dev(c, grid, u, v, w, boundary_sdf, boundary_sdf->data,
                           fluid_sdf, fluid_sdf->data, solid_u, solid_v,
                           solid_w, out_u, out_v, out_w, out_pressure, &local,
                           nullptr, blocked);
    if (stats) *stats = local;
    return s;
}

jetgpu_status jetgpu_solve_pressure_device(
    jetgpu_ctx* c, const jetgpu_grid* grid, const double* u, const double* v,
    const double* w, const jetgpu_scalar_field* boundary_sdf,
    const jetgpu_scalar_field* fluid_sdf, const double* solid_u,
    const double* solid_v, const double* solid_w, double* out_u,
    double* out_v, double* out_w, double* out_pressure,
    jetgpu_solve_stats* stats) {
    return solve_device(c, grid, u, v, w, boundary_sdf, fluid_sdf, solid_u,
                        solid_v, solid_w, out_u, out_v, out_w, out_pressure,
                        stats, false);
}

jetgpu_status jetgpu_solve_pressure_blocked_device(
    jetgpu_ctx* c, const jetgpu_grid* grid, const double* u, const double* v,
    const double* w, const jetgpu_scalar_field* boundary_sdf,
    const jetgpu_scalar_field* fluid_sdf, double* out_u, double* out_v,
    double* out_w, double* out_pressure, jetgpu_solve_stats* stats) {
    return solve_device(c, grid, u, v, w, boundary_sdf, fluid_sdf, nullptr,
                        nullptr, nullptr, out_u, out_v, out_w, out_pressure,
                        stats, true);
}

// The host-pointer solve of either pressure solver (see solve_pressure_dev).
static jetgpu_status solve_host(
    jetgpu_ctx* c, const jetgpu_grid* grid, const double* u, const double* v,
    const double* w, const jetgpu_scalar_field* boundary_sdf,
    const jetgpu_scalar_field* fluid_sdf, const double* solid_u,
    const double* solid_v, const double* solid_w, double* out_u,
    double* out_v, double* out_w, double* out_pressure,
    jetgpu_solve_stats* stats, bool blocked,
    const jetgpu_collider* collider = nullptr) {
    if (!c) return JETGPU_BAD_INPUT;
    auto t0 = std::chrono::steady_clock::now();
    jetgpu_status s = check_grid(c, grid);
    if (s != JETGPU_OK) return s;
    if (!u || !v || !w || !out_u || !out_v || !out_w)
        return fail(c, JETGPU_BAD_INPUT, "null velocity pointer");
    if ((s = check_field(c, boundary_sdf, "boundary_sdf")) != JETGPU_OK) return s;
    if ((s = check_field(c, fluid_sdf, "fluid_sdf")) != JETGPU_OK) return s;
    JG_CUDA(c, cudaSetDevice(c->device));
    const long nx = grid->res[0], ny = grid->res[1], nz = grid->res[2];
    const size_t nu = (size_t)(nx + 1) * ny * nz, nv = (size_t)nx * (ny + 1) * nz,
                 nw = (size_t)nx * ny * (nz + 1);
    const size_t nb = field_count(boundary_sdf), nf = field_count(fluid_sdf);
    // A moving rigid collider's face velocities are evaluated on the device
    // into the solid part of the staging area (no host arrays).
    const bool col_faces = collider_moves(collider);
    if (col_faces) solid_u = solid_v = solid_w = nullptr;
    const size_t ns = col_faces ? nu + nv + nw
                                : (solid_u ? nu : 0) + (solid_v ? nv : 0) +
                                      (solid_w ? nw : 0);
    // Device staging: inputs u,v,w | solid | sdf data | outputs u,v,w (the
    // pressure is downloaded from the solver's own buffer).
    const size_t total = 2 * (nu + nv + nw) + ns + nb + nf;
    s = grow_stage(c, total * sizeof(double));
    if (s != JETGPU_OK) return s;
    double* base = reinterpret_cast<double*>(c->stage);
    double* du = base;
    double* dv = du + nu;
    double* dw = dv + nv;
    double* p = dw + nw;
    double* dsu = (solid_u || col_faces) ? p : nullptr;
    p += dsu ? nu : 0;
    double* dsv = (solid_v || col_faces) ? p : nullptr;
    p += dsv ? nv : 0;
    double* dsw = (solid_w || col_faces) ? p : nullptr;
    p += dsw ? nw : 0;
    double* db = nb ? p : nullptr;
    p += nb;
    double* df = nf ? p : nullptr;
    p += nf;
    double* ou = p;
    double* ov = ou + nu;
    double* ow = ov + nv;
    // Uploads run in order on the copy stream: the collider SDF first (the
    // face weights need only it and start as soon as it is in), the fluid
    // SDF under them, then the velocities. The copy stream first waits for
    // anything still queued on the compute stream.
    cudaStream_t st = c->stream, cs = c->copy_stream;
    struct Join {  // no exit leaves a copy in flight
        cudaStream_t s;
        ~Join() { cudaStreamSynchronize(s); }
    } join{cs};
    SolveIo io;
    io.sdf_in = c->io_ev[1];
    io.vel_in = c->io_ev[2];
    io.x_final = c->io_ev[3];
    io.bsdf_in = c->io_ev[4];
    io.copy = cs;
    io.host_p = out_pressure;
    JG_CUDA(c, cudaEventRecord(c->io_ev[0], st));
    JG_CUDA(c, cudaStreamWaitEvent(cs, c->io_ev[0], 0));
    if (db) JG_CUDA(c, cudaMemcpyAsync(db, boundary_sdf->data, nb * 8, cudaMemcpyHostToDevice, cs));
    JG_CUDA(c, cudaEventRecord(io.bsdf_in, cs));
    if (df) JG_CUDA(c, cudaMemcpyAsync(df, fluid_sdf->data, nf * 8, cudaMemcpyHostToDevice, cs));
    JG_CUDA(c, cudaEventRecord(io.sdf_in, cs));
    unsigned long long h2d = (unsigned long long)(nb + nf) * 8, d2h = 0;
    // The face boxes of u, v, w moved in each direction (origin and extent
    // in faces): the whole arrays, or with fluid_box_io the bounding box of
    // the fluid cells widened by the faces that close it.
    struct FBox {
        long x0, y0, z0, wx, wy, wz;
    } fb[3] = {{0, 0, 0, nx + 1, ny, nz},
               {0, 0, 0, nx, ny + 1, nz},
               {0, 0, 0, nx, ny, nz + 1}};
    // The part of face box a in face planes [zlo, zhi); the bytes moved
    // are added to `moved`. Host-to-device copies whose rows leave less
    // than 256 bytes between them (a box nearly as wide as the array) run
    // at a fraction of the link's rate on GB300 (25-80 GB/s against 200
    // GB/s, for row pitches that are not multiples of 2 KB), so such boxes
    // go up as whole rows: the extra faces hold the caller's own values.
    // Whole rows go as one run per plane range, or as one row of y-ranges
    // per plane.
    auto copy_box = [&](double* dst, const double* src, int a,
                        cudaMemcpyKind kind, cudaStream_t on,
                        unsigned long long& moved, long zlo = 0,
                        long zhi = LONG_MAX) -> jetgpu_status {
        const FBox& b = fb[a];
        if (b.wx <= 0 || b.wy <= 0 || b.wz <= 0) return JETGPU_OK;
        const long z0 = std::max(b.z0, zlo), z1 = std::min(b.z0 + b.wz, zhi);
        if (z1 <= z0) return JETGPU_OK;
        const long rx = nx + (a == 0), ry = ny + (a == 1);
        long x0 = b.x0, wx = b.wx;
        if (kind == cudaMemcpyHostToDevice && wx < rx && (rx - wx) * 8 < 256) {
            x0 = 0;
            wx = rx;
        }
        if (wx == rx && b.wy == ry) {  // whole planes: one contiguous run
            const size_t off = (size_t)(z0 * rx * ry);
            const size_t bytes = (size_t)(rx * ry * (z1 - z0)) * 8;
            JG_CUDA(c, cudaMemcpyAsync(dst + off, src + off, bytes, kind, on));
            moved += bytes;
            return JETGPU_OK;
        }
        if (wx == rx) {  // whole rows: the y-range of each plane is one run
            const size_t off = (size_t)((z0 * ry + b.y0) * rx);
            const size_t pitch = (size_t)(rx * ry) * 8, width = (size_t)(b.wy * rx) * 8;
            JG_CUDA(c, cudaMemcpy2DAsync(dst + off, pitch, src + off, pitch,
                                         width, (size_t)(z1 - z0), kind, on));
            moved += width * (size_t)(z1 - z0);
            return JETGPU_OK;
        }
        cudaMemcpy3DParms p3 = {};
        p3.srcPtr = make_cudaPitchedPtr(const_cast<double*>(src), rx * 8, rx, ry);
        p3.dstPtr = make_cudaPitchedPtr(dst, rx * 8, rx, ry);
        p3.srcPos = make_cudaPos(x0 * 8, b.y0, z0);
        p3.dstPos = p3.srcPos;
        p3.extent = make_cudaExtent(wx * 8, b.wy, z1 - z0);
        p3.kind = kind;
        JG_CUDA(c, cudaMemcpy3DAsync(&p3, on));
        moved += (unsigned long long)(wx * b.wy * (z1 - z0)) * 8;
        return JETGPU_OK;
    };
    auto upload_velocities = [&]() -> jetgpu_status {
        const double* hv[3] = {u, v, w};
        double* dv3[3] = {du, dv, dw};
        const double* hs[3] = {solid_u, solid_v, solid_w};
        double* ds3[3] = {dsu, dsv, dsw};
        for (int a = 0; a < 3; ++a) {
            jetgpu_status e =
                copy_box(dv3[a], hv[a], a, cudaMemcpyHostToDevice, cs, h2d);
            if (e != JETGPU_OK) return e;
            if (hs[a]) {
                e = copy_box(ds3[a], hs[a], a, cudaMemcpyHostToDevice, cs, h2d);
                if (e != JETGPU_OK) return e;
            }
        }
        JG_CUDA(c, cudaEventRecord(io.vel_in, cs));
        return JETGPU_OK;
    };
    // The gradient runs in slabs of cell planes spread over the box's, and
    // each slab's faces go down under the next slab. Cell plane k writes
    // the u and v faces of plane k and the w faces of plane k + 1 (plane
    // 0 also w plane 0).
    int cuts[Ctx::kGradSlabs + 1];
    int nslab = 0;
    io.grad_cuts = cuts;
    io.grad_slabs = &nslab;
    auto set_cuts = [&](long z0, long z1) {  // the box's cell planes
        if (blocked || z1 <= z0) return;
        nslab = Ctx::kGradSlabs;
        cuts[0] = 0;
        cuts[nslab] = (int)nz;
        for (int k = 1; k < nslab; ++k)
            cuts[k] = (int)(z0 + (z1 - z0) * k / nslab);
    };
    const bool box_io = c->cfg.fluid_box_io != 0 && !blocked;
    if (box_io) {
        // The box is found on the device as soon as the fluid SDF is in;
        // the host reads it back once the set-up that needs no velocity is
        // queued, and only then issues the velocity uploads.
        if (df) {
            const Dims dn{(int)nx, (int)ny, (int)nz};
            k_box_init<<<1, 1, 0, cs>>>(c->box_dev);
            k_fluid_box<<<blocks_for(dn.count(), kThreads, c->num_sms * 4),
                          kThreads, 0, cs>>>(df, dn, c->box_dev);
            JG_CUDA(c, cudaMemcpyAsync(c->box_host, c->box_dev, 6 * sizeof(int),
                                       cudaMemcpyDeviceToHost, cs));
            JG_CUDA(c, cudaEventRecord(c->box_ev, cs));
        }
        io.before_vel = [&]() -> jetgpu_status {
            int bx[6];
            if (df) {
                JG_CUDA(c, cudaEventSynchronize(c->box_ev));
                for (int d = 0; d < 6; ++d) bx[d] = c->box_host[d];
            } else if (fluid_sdf->value < 0.0) {  // all fluid
                bx[0] = bx[1] = bx[2] = 0;
                bx[3] = (int)nx - 1;
                bx[4] = (int)ny - 1;
                bx[5] = (int)nz - 1;
            } else {  // no fluid
                bx[0] = bx[1] = bx[2] = 0;
                bx[3] = bx[4] = bx[5] = -1;
            }
            const bool empty = bx[3] < bx[0];
            for (int a = 0; a < 3; ++a) {
                fb[a].x0 = bx[0];
                fb[a].y0 = bx[1];
                fb[a].z0 = bx[2];
                fb[a].wx = empty ? 0 : bx[3] - bx[0] + 1 + (a == 0);
                fb[a].wy = empty ? 0 : bx[4] - bx[1] + 1 + (a == 1);
                fb[a].wz = empty ? 0 : bx[5] - bx[2] + 1 + (a == 2);
            }
            if (!empty) set_cuts(bx[2], bx[5] + 1);
            return upload_velocities();
        };
    } else {
        set_cuts(0, nz);
        if ((s = upload_velocities()) != JETGPU_OK) return s;
    }
    if (col_faces) {
        GridDesc gd;
        for (int a = 0; a < 3; ++a) {
            gd.res[a] = grid->res[a];
            gd.spacing[a] = grid->spacing[a];
            gd.origin[a] = grid->origin[a];
        }
        if ((s = solid_face_velocities(c, gd, *collider, dsu)) != JETGPU_OK)
            return s;
    }
    // The projected velocity goes down as soon as the gradient is queued:
    // slab by slab on the copy stream, or after the whole gradient.
    io.after_grad = [&]() -> jetgpu_status {
        double* ho[3] = {out_u, out_v, out_w};
        const double* dout[3] = {ou, ov, ow};
        if (nslab > 0) {
            for (int k = 0; k < nslab; ++k) {
                JG_CUDA(c, cudaStreamWaitEvent(cs, c->grad_ev[k], 0));
                for (int a = 0; a < 3; ++a) {
                    const long lo = a < 2 ? cuts[k] : (k ? cuts[k] + 1 : 0);
                    const long hi = cuts[k + 1] + (a == 2);
                    if ((s = copy_box(ho[a], dout[a], a, cudaMemcpyDeviceToHost,
                                      cs, d2h, lo, hi)) != JETGPU_OK)
                        return s;
                }
            }
        } else {
            for (int a = 0; a < 3; ++a)
                if ((s = copy_box(ho[a], dout[a], a, cudaMemcpyDeviceToHost,
                                  st, d2h)) != JETGPU_OK)
                    return s;
        }
        return JETGPU_OK;
    };
    jetgpu_solve_stats local;
    std::memset(&local, 0, sizeof(local));
    jetgpu_status solve_status = solve_pressure_dev(
        c, grid, du, dv, dw, boundary_sdf, db, fluid_sdf, df, dsu, dsv, dsw,
        ou, ov, ow, nullptr, &local, &io, blocked);
    if (!usable(solve_status)) {
        if (stats) *stats = local;
        return solve_status;
    }
    if (out_pressure) d2h += (unsigned long long)nx * ny * nz * 8;
    JG_CUDA(c, cudaStreamSynchronize(st));
    JG_CUDA(c, cudaStreamSynchronize(cs));
    local.total_ms = ms_since(t0);
    local.h2d_bytes = h2d;
    local.d2h_bytes = d2h;
    if (stats) *stats = local;
    return solve_status;
}

jetgpu_status jetgpu_solve_pressure(
    jetgpu_ctx* c, const jetgpu_grid* grid, const double* u, const double* v,
    const double* w, const jetgpu_scalar_field* boundary_sdf,
    const jetgpu_scalar_field* fluid_sdf, const double* solid_u,
    const double* solid_v, const double* solid_w, double* out_u,
    double* out_v, double* out_w, double* out_pressure,
    jetgpu_solve_stats* stats) {
    return solve_host(c, grid, u, v, w, boundary_sdf, fluid_sdf, solid_u,
                      solid_v, solid_w, out_u, out_v, out_w, out_pressure,
                      stats, false);
}

jetgpu_status jetgpu_solve_pressure_collider(
    jetgpu_ctx* c, const jetgpu_grid* grid, const double* u, const double* v,
    const double* w, const jetgpu_scalar_field* boundary_sdf,
    const jetgpu_scalar_field* fluid_sdf, const jetgpu_collider* collider,
    double* out_u, double* out_v, double* out_w, double* out_pressure,
    jetgpu_solve_stats* stats) {
    return solve_host(c, grid, u, v, w, boundary_sdf, fluid_sdf, nullptr,
                      nullptr, nullptr, out_u, out_v, out_w, out_pressure,
                      stats, false, collider);
}

jetgpu_status jetgpu_solve_pressure_blocked(
    jetgpu_ctx* c, const jetgpu_grid* grid, const double* u, const double* v,
    const double* w, const jetgpu_scalar_field* boundary_sdf,
    const jetgpu_scalar_field* fluid_sdf, double* out_u, double* out_v,
    double* out_w, double* out_pressure, jetgpu_solve_stats* stats) {
    return solve_host(c, grid, u, v, w, boundary_sdf, fluid_sdf, nullptr,
                      nullptr, nullptr, out_u, out_v, out_w, out_pressure,
                      stats, true);
}

jetgpu_status jetgpu_mgpcg_solve_system(jetgpu_ctx* c, const int res0[3],
                                        int levels, const double* A,
                                        const double* b, double* x,
                                        jetgpu_solve_stats* stats) {
    if (!c) return JETGPU_BAD_INPUT;
    if (!res0 || !A || !b || !x || levels < 1)
        return fail(c, JETGPU_BAD_INPUT, "null argument or levels < 1");
    for (int a = 0; a < 3; ++a)
        if (res0[a] < 1 || (res0[a] >> (levels - 1)) < 1 ||
            ((res0[a] >> (levels - 1)) << (levels - 1)) != res0[a])
            return fail(c, JETGPU_BAD_INPUT,
                        "level resolutions must halve exactly");
    JG_CUDA(c, cudaSetDevice(c->device));
    auto t0 = std::chrono::steady_clock::now();
    const Dims n{res0[0], res0[1], res0[2]};
    jetgpu_status s = ensure_buffers(c, n, (unsigned)levels);
    if (s != JETGPU_OK) return s;
    if ((int)c->built_levels != levels)
        return fail(c, JETGPU_BAD_INPUT, "level count does not match sizes");
    long total = 0;
    for (int l = 0; l < levels; ++l) total += c->levels[l].n.count();
    s = grow_stage(c, (size_t)total * 4 * sizeof(double));
    if (s != JETGPU_OK) return s;
    double* dA = reinterpret_cast<double*>(c->stage);
    cudaStream_t st = c->stream;
    JG_CUDA(c, cudaMemcpyAsync(dA, A, (size_t)total * 32, cudaMemcpyHostToDevice, st));
    const long N0 = n.count();
    JG_CUDA(c, cudaMemcpyAsync(c->A64, dA, (size_t)N0 * 32, cudaMemcpyDeviceToDevice, st));
    JG_CUDA(c, cudaMemcpyAsync(c->b64, b, (size_t)N0 * 8, cudaMemcpyHostToDevice, st));
    long off = 0;
    for (int l = 0; l < levels; ++l) {
        const long N = c->levels[l].n.count();
        k_rows_to_f32<<<blocks_for(N), kThreads, 0, st>>>(dA + 4 * off,
                                                         c->levels[l].A, N);
        // A caller-built system has no fluid SDF: every cell is an unknown.
        k_fill_f32<<<blocks_for(N), kThreads, 0, st>>>(c->levels[l].phi,
                                                      -1.0f, N);
        off += N;
    }
    JG_CUDA(c, cudaGetLastError());
    s = split_system(c);
    if (s != JETGPU_OK) return s;
    s = prepare_levels(c);
    if (s != JETGPU_OK) return s;
    jetgpu_solve_stats local;
    std::memset(&local, 0, sizeof(local));
    JG_CUDA(c, cudaStreamSynchronize(st));
    local.setup_ms = ms_since(t0);
    auto t1 = std::chrono::steady_clock::now();
    jetgpu_status solve_status = mgpcg_solve(c, &local);
    local.solve_ms = ms_since(t1);
    if (usable(solve_status)) {
        JG_CUDA(c, cudaMemcpyAsync(x, c->x64, (size_t)N0 * 8, cudaMemcpyDeviceToHost, st));
        JG_CUDA(c, cudaStreamSynchronize(st));
    }
    local.levels = c->built_levels;
    local.total_ms = ms_since(t0);
    if (stats) *stats = local;
    return solve_status;
}

jetgpu_status jetgpu_get_level(jetgpu_ctx* c, int level, int what, void* dst,
                               size_t capacity, size_t* count) {
    if (!c || !dst) return JETGPU_BAD_INPUT;
    if (level < 0 || level >= (int)c->built_levels)
        return fail(c, JETGPU_BAD_INPUT, "level out of range");
    JG_CUDA(c, cudaSetDevice(c->device));
    const Level& L = c->levels[level];
    const Dims s = L.n;
    const void* src = nullptr;
    size_t elems = 0, esize = 0;
    double* tmp = nullptr;
    switch (what) {
        case 0: src = L.phi; elems = s.count(); esize = 4; break;
        case 1: src = L.uw; elems = (size_t)(s.x + 1) * s.y * s.z; esize = 4; break;
        case 2: src = L.vw; elems = (size_t)s.x * (s.y + 1) * s.z; esize = 4; break;
        case 3: src = L.ww; elems = (size_t)s.x * s.y * (s.z + 1); esize = 4; break;
        case 4:
            elems = s.count();
            esize = 32;
            if (level == 0) {
                src = c->A64;
            } else {
                jetgpu_status g = grow_stage(c, elems * 32);
                if (g != JETGPU_OK) return g;
                tmp = reinterpret_cast<double*>(c->stage);
                k_rows_f32_to_f64<<<blocks_for(elems), kThreads, 0, c->stream>>>(
                    L.A, tmp, (long)elems);
                src = tmp;
            }
            break;
        case 5:
            if (level != 0)
                return fail(c, JETGPU_BAD_INPUT, "b is kept on level 0 only");
            src = c->b64; elems = s.count(); esize = 8; break;
        case 6:
            if (level != 0)
                return fail(c, JETGPU_BAD_INPUT,
                            "the pressure is kept on level 0 only");
            src = c->x64; elems = s.count(); esize = 8; break;
        default:
            return fail(c, JETGPU_BAD_INPUT, "unknown field selector");
    }
    if (count) *count = elems;
    if (capacity < elems * esize)
        return fail(c, JETGPU_BAD_INPUT, "destination too small");
    JG_CUDA(c, cudaMemcpyAsync(dst, src, elems * esize, cudaMemcpyDeviceToHost,
                               c->stream));
    JG_CUDA(c, cudaStreamSynchronize(c->stream));
    return JETGPU_OK;
}

}  // extern "C"

// ---- particle transfers ----------------------------------------------------

namespace {

jetgpu_status check_transfer(jetgpu_ctx* c, const jetgpu_grid* grid,
                             long np, const void* pos, const void* vel) {
    if (!c) return JETGPU_BAD_INPUT;
    jetgpu_status s = check_grid(c, grid);
    if (s != JETGPU_OK) return s;
    if (np < 0) return fail(c, JETGPU_BAD_INPUT, "negative particle count");
    if (np > 0 && (!pos || !vel))
        return fail(c, JETGPU_BAD_INPUT, "null particle arrays");
    return JETGPU_OK;
}

void face_counts(const jetgpu_grid* g, size_t n[3]) {
    const size_t nx = g->res[0], ny = g->res[1], nz = g->res[2];
    n[0] = (nx + 1) * ny * nz;
    n[1] = nx * (ny + 1) * nz;
    n[2] = nx * ny * (nz + 1);
}

}  // namespace

extern "C" {

jetgpu_status jetgpu_p2g_device(jetgpu_ctx* c, const jetgpu_grid* grid,
                                long np, const double* pos, const double* vel,
                                double* u, double* v, double* w,
                                unsigned char* mu, unsigned char* mv,
                                unsigned char* mw, float* su, float* sv,
                                float* sw) {
    jetgpu_status s = check_transfer(c, grid, np, pos, vel);
    if (s != JETGPU_OK) return s;
    if (!u || !v || !w) return fail(c, JETGPU_BAD_INPUT, "null grid arrays");
    JG_CUDA(c, cudaSetDevice(c->device));
    s = p2g(c, to_desc(grid), np, pos, vel, u, v, w, mu, mv, mw, su, sv, sw);
    if (s != JETGPU_OK) return s;
    JG_CUDA(c, cudaStreamSynchronize(c->stream));
    return JETGPU_OK;
}

jetgpu_status jetgpu_g2p_flip_device(jetgpu_ctx* c, const jetgpu_grid* grid,
                                     long np, const double* pos, double* vel,
                                     const double* u, const double* v,
                                     const double* w, float* su, float* sv,
                                     float* sw, double blend) {
    jetgpu_status s = check_transfer(c, grid, np, pos, vel);
    if (s != JETGPU_OK) return s;
    if (!u || !v || !w || !su || !sv || !sw)
        return fail(c, JETGPU_BAD_INPUT, "null grid arrays");
    if (!(blend >= 0.0 && blend <= 1.0))
        return fail(c, JETGPU_BAD_INPUT, "pic blending factor outside [0,1]");
    JG_CUDA(c, cudaSetDevice(c->device));
    s = g2p_flip(c, to_desc(grid), np, pos, vel, u, v, w, su, sv, sw, blend);
    if (s != JETGPU_OK) return s;
    JG_CUDA(c, cudaStreamSynchronize(c->stream));
    return JETGPU_OK;
}

jetgpu_status jetgpu_g2p_pic_device(jetgpu_ctx* c, const jetgpu_grid* grid,
                                    long np, const double* pos, double* vel,
                                    const double* u, const double* v,
                                    const double* w) {
    jetgpu_status s = check_transfer(c, grid, np, pos, vel);
    if (s != JETGPU_OK) return s;
    if (!u || !v || !w) return fail(c, JETGPU_BAD_INPUT, "null grid arrays");
    JG_CUDA(c, cudaSetDevice(c->device));
    s = g2p_pic(c, to_desc(grid), np, pos, vel, u, v, w);
    if (s != JETGPU_OK) return s;
    JG_CUDA(c, cudaStreamSynchronize(c->stream));
    return JETGPU_OK;
}

jetgpu_status jetgpu_p2g(jetgpu_ctx* c, const jetgpu_grid* grid, long np,
                         const double* pos, const double* vel, double* u,
                         double* v, double* w, unsigned char* mu,
                         unsigned char* mv, unsigned char* mw, float* su,
                         float* sv, float* sw) {
    jetgpu_status s = check_transfer(c, grid, np, pos, vel);
    if (s != JETGPU_OK) return s;
    if (!u || !v || !w) return fail(c, JETGPU_BAD_INPUT, "null grid arrays");
    JG_CUDA(c, cudaSetDevice(c->device));
    size_t n[3];
    face_counts(grid, n);
    const size_t nf = n[0] + n[1] + n[2];
    const size_t bytes = (size_t)np * 48 + nf * (8 + 1 + 4);
    s = grow_stage(c, bytes + 64);
    if (s != JETGPU_OK) return s;
    unsigned char* p = c->stage;
    double* dpos = reinterpret_cast<double*>(p); p += (size_t)np * 24;
    double* dvel = reinterpret_cast<double*>(p); p += (size_t)np * 24;
    double* dg = reinterpret_cast<double*>(p); p += nf * 8;
    float* ds = reinterpret_cast<float*>(p); p += nf * 4;
    unsigned char* dm = p;
    cudaStream_t st = c->stream;
    if (np) {
        JG_CUDA(c, cudaMemcpyAsync(dpos, pos, np * 24, cudaMemcpyHostToDevice, st));
        JG_CUDA(c, cudaMemcpyAsync(dvel, vel, np * 24, cudaMemcpyHostToDevice, st));
    }
    const bool want_m = mu || mv || mw, want_s = su || sv || sw;
    s = p2g(c, to_desc(grid), np, dpos, dvel, dg, dg + n[0], dg + n[0] + n[1],
            want_m ? dm : nullptr, want_m ? dm + n[0] : nullptr,
            want_m ? dm + n[0] + n[1] : nullptr, want_s ? ds : nullptr,
            want_s ? ds + n[0] : nullptr, want_s ? ds + n[0] + n[1] : nullptr);
    if (s != JETGPU_OK) return s;
    double* outs[3] = {u, v, w};
    unsigned char* marks[3] = {mu, mv, mw};
    float* snaps[3] = {su, sv, sw};
    size_t off = 0;
    for (int a = 0; a < 3; ++a) {
        JG_CUDA(c, cudaMemcpyAsync(outs[a], dg + off, n[a] * 8, cudaMemcpyDeviceToHost, st));
        if (marks[a]) JG_CUDA(c, cudaMemcpyAsync(marks[a], dm + off, n[a], cudaMemcpyDeviceToHost, st));
        if (snaps[a]) JG_CUDA(c, cudaMemcpyAsync(snaps[a], ds + off, n[a] * 4, cudaMemcpyDeviceToHost, st));
        off += n[a];
    }
    JG_CUDA(c, cudaStreamSynchronize(st));
    return JETGPU_OK;
}

jetgpu_status jetgpu_g2p_flip(jetgpu_ctx* c, const jetgpu_grid* grid, long np,
                              const double* pos, double* vel, const double* u,
                              const double* v, const double* w, float* su,
                              float* sv, float* sw, double blend) {
    jetgpu_status s = check_transfer(c, grid, np, pos, vel);
    if (s != JETGPU_OK) return s;
    if (!u || !v || !w || !su || !sv || !sw)
        return fail(c, JETGPU_BAD_INPUT, "null grid arrays");
    if (!(blend >= 0.0 && blend <= 1.0))
        return fail(c, JETGPU_BAD_INPUT, "pic blending factor outside [0,1]");
    JG_CUDA(c, cudaSetDevice(c->device));
    size_t n[3];
    face_counts(grid, n);
    const size_t nf = n[0] + n[1] + n[2];
    s = grow_stage(c, (size_t)np * 48 + nf * 12 + 64);
    if (s != JETGPU_OK) return s;
    unsigned char* p = c->stage;
    double* dpos = reinterpret_cast<double*>(p); p += (size_t)np * 24;
    double* dvel = reinterpret_cast<double*>(p); p += (size_t)np * 24;
    double* dg = reinterpret_cast<double*>(p); p += nf * 8;
    float* ds = reinterpret_cast<float*>(p);
    cudaStream_t st = c->stream;
    const double* ins[3] = {u, v, w};
    float* snaps[3] = {su, sv, sw};
    if (np) {
        JG_CUDA(c, cudaMemcpyAsync(dpos, pos, np * 24, cudaMemcpyHostToDevice, st));
        JG_CUDA(c, cudaMemcpyAsync(dvel, vel, np * 24, cudaMemcpyHostToDevice, st));
    }
    size_t off = 0;
    for (int a = 0; a < 3; ++a) {
        JG_CUDA(c, cudaMemcpyAsync(dg + off, ins[a], n[a] * 8, cudaMemcpyHostToDevice, st));
        JG_CUDA(c, cudaMemcpyAsync(ds + off, snaps[a], n[a] * 4, cudaMemcpyHostToDevice, st));
        off += n[a];
    }
    s = g2p_flip(c, to_desc(grid), np, dpos, dvel, dg, dg + n[0],
                 dg + n[0] + n[1], ds, ds + n[0], ds + n[0] + n[1], blend);
    if (s != JETGPU_OK) return s;
    if (np) JG_CUDA(c, cudaMemcpyAsync(vel, dvel, np * 24, cudaMemcpyDeviceToHost, st));
    off = 0;
    for (int a = 0; a < 3; ++a) {
        JG_CUDA(c, cudaMemcpyAsync(snaps[a], ds + off, n[a] * 4, cudaMemcpyDeviceToHost, st));
        off += n[a];
    }
    JG_CUDA(c, cudaStreamSynchronize(st));
    return JETGPU_OK;
}

jetgpu_status jetgpu_g2p_pic(jetgpu_ctx* c, const jetgpu_grid* grid, long np,
                             const double* pos, double* vel, const double* u,
                             const double* v, const double* w) {
    jetgpu_status s = check_transfer(c, grid, np, pos, vel);
    if (s != JETGPU_OK) return s;
    if (!u || !v || !w) return fail(c, JETGPU_BAD_INPUT, "null grid arrays");
    JG_CUDA(c, cudaSetDevice(c->device));
    size_t n[3];
    face_counts(grid, n);
    const size_t nf = n[0] + n[1] + n[2];
    s = grow_stage(c, (size_t)np * 48 + nf * 8 + 64);
    if (s != JETGPU_OK) return s;
    unsigned char* p = c->stage;
    double* dpos = reinterpret_cast<double*>(p); p += (size_t)np * 24;
    double* dvel = reinterpret_cast<double*>(p); p += (size_t)np * 24;
    double* dg = reinterpret_cast<double*>(p);
    cudaStream_t st = c->stream;
    const double* ins[3] = {u, v, w};
    if (np) {
        JG_CUDA(c, cudaMemcpyAsync(dpos, pos, np * 24, cudaMemcpyHostToDevice, st));
        JG_CUDA(c, cudaMemcpyAsync(dvel, vel, np * 24, cudaMemcpyHostToDevice, st));
    }
    size_t off = 0;
    for (int a = 0; a < 3; ++a) {
        JG_CUDA(c, cudaMemcpyAsync(dg + off, ins[a], n[a] * 8, cudaMemcpyHostToDevice, st));
        off += n[a];
    }
    s = g2p_pic(c, to_desc(grid), np, dpos, dvel, dg, dg + n[0], dg + n[0] + n[1]);
    if (s != JETGPU_OK) return s;
    if (np) JG_CUDA(c, cudaMemcpyAsync(vel, dvel, np * 24, cudaMemcpyDeviceToHost, st));
    JG_CUDA(c, cudaStreamSynchronize(st));
    return JETGPU_OK;
}

// The fractional or blocked constraint on device arrays.
static jetgpu_status constrain_any(Ctx* c, const GridDesc& g, double* u,
                                   double* v, double* w, const FieldDesc& f,
                                   const jetgpu_collider* col, int closed,
                                   unsigned depth, bool blocked) {
    return blocked
               ? constrain_velocity_blocked(c, g, u, v, w, f, col, closed, depth)
               : constrain_velocity(c, g, u, v, w, f, col, closed, depth);
}

static jetgpu_status constrain_device(
    jetgpu_ctx* c, const jetgpu_grid* grid, double* u, double* v, double* w,
    const jetgpu_scalar_field* sdf, const jetgpu_collider* col, int closed,
    unsigned int depth, bool blocked) {
    if (!c) return JETGPU_BAD_INPUT;
    jetgpu_status s;
    if ((s = check_grid(c, grid)) != JETGPU_OK) return s;
    if ((s = check_field(c, sdf, "collider_sdf")) != JETGPU_OK) return s;
    if (!u || !v || !w) return fail(c, JETGPU_BAD_INPUT, "null velocity arrays");
    JG_CUDA(c, cudaSetDevice(c->device));
    return constrain_any(c, to_desc(grid), u, v, w, to_desc(sdf, sdf->data),
                         col, closed, depth, blocked);
}

jetgpu_status jetgpu_constrain_velocity_device(
    jetgpu_ctx* c, const jetgpu_grid* grid, double* u, double* v, double* w,
    const jetgpu_scalar_field* sdf, const jetgpu_collider* col, int closed,
    unsigned int depth) {
    return constrain_device(c, grid, u, v, w, sdf, col, closed, depth, false);
}

jetgpu_status jetgpu_constrain_velocity_blocked_device(
    jetgpu_ctx* c, const jetgpu_grid* grid, double* u, double* v, double* w,
    const jetgpu_scalar_field* sdf, const jetgpu_collider* col, int closed,
    unsigned int depth) {
    return constrain_device(c, grid, u, v, w, sdf, col, closed, depth, true);
}

static jetgpu_status constrain_host(
    jetgpu_ctx* c, const jetgpu_grid* grid, double* u, double* v, double* w,
    const jetgpu_scalar_field* sdf, const jetgpu_collider* col, int closed,
    unsigned int depth, bool blocked) {
    if (!c) return JETGPU_BAD_INPUT;
    jetgpu_status s;
    if ((s = check_grid(c, grid)) != JETGPU_OK) return s;
    if ((s = check_field(c, sdf, "collider_sdf")) != JETGPU_OK) return s;
    if (!u || !v || !w) return fail(c, JETGPU_BAD_INPUT, "null velocity arrays");
    JG_CUDA(c, cudaSetDevice(c->device));
    size_t n[3];
    face_counts(grid, n);
    const size_t nf = n[0] + n[1] + n[2];
    const size_t ns = (size_t)field_count(sdf);
    s = grow_stage(c, (nf + ns) * 8 + 64);
    if (s != JETGPU_OK) return s;
    double* dg = reinterpret_cast<double*>(c->stage);
    double* ds = dg + nf;
    cudaStream_t st = c->stream;
    double* io[3] = {u, v, w};
    size_t off = 0;
    for (int a = 0; a < 3; ++a) {
        JG_CUDA(c, cudaMemcpyAsync(dg + off, io[a], n[a] * 8,
                                   cudaMemcpyHostToDevice, st));
        off += n[a];
    }
    if (ns)
        JG_CUDA(c, cudaMemcpyAsync(ds, sdf->data, ns * 8,
                                   cudaMemcpyHostToDevice, st));
    s = constrain_any(c, to_desc(grid), dg, dg + n[0], dg + n[0] + n[1],
                      to_desc(sdf, ns ? ds : nullptr), col, closed, depth,
                      blocked);
    if (s != JETGPU_OK) return s;
    off = 0;
    for (int a = 0; a < 3; ++a) {
        JG_CUDA(c, cudaMemcpyAsync(io[a], dg + off, n[a] * 8,
                                   cudaMemcpyDeviceToHost, st));
        off += n[a];
    }
    JG_CUDA(c, cudaStreamSynchronize(st));
    return JETGPU_OK;
}

jetgpu_status jetgpu_constrain_velocity(
    jetgpu_ctx* c, const jetgpu_grid* grid, double* u, double* v, double* w,
    const jetgpu_scalar_field* sdf, const jetgpu_collider* col, int closed,
    unsigned int depth) {
    return constrain_host(c, grid, u, v, w, sdf, col, closed, depth, false);
}

jetgpu_status jetgpu_constrain_velocity_blocked(
    jetgpu_ctx* c, const jetgpu_grid* grid, double* u, double* v, double* w,
    const jetgpu_scalar_field* sdf, const jetgpu_collider* col, int closed,
    unsigned int depth) {
    return constrain_host(c, grid, u, v, w, sdf, col, closed, depth, true);
}

jetgpu_status jetgpu_apic_p2g_device(jetgpu_ctx* c, const jetgpu_grid* grid,
                                     long np, const double* pos,
                                     const double* vel, const double* affine,
                                     double* u, double* v, double* w,
                                     unsigned char* mu, unsigned char* mv,
                                     unsigned char* mw) {
    jetgpu_status s = check_transfer(c, grid, np, pos, vel);
    if (s != JETGPU_OK) return s;
    if (!u || !v || !w || (np > 0 && !affine))
        return fail(c, JETGPU_BAD_INPUT, "null grid or affine arrays");
    JG_CUDA(c, cudaSetDevice(c->device));
    return apic_p2g(c, to_desc(grid), np, pos, vel, affine, u, v, w, mu, mv,
                    mw);
}

jetgpu_status jetgpu_apic_g2p_device(jetgpu_ctx* c, const jetgpu_grid* grid,
                                     long np, const double* pos, double* vel,
                                     double* affine, const double* u,
                                     const double* v, const double* w) {
    jetgpu_status s = check_transfer(c, grid, np, pos, vel);
    if (s != JETGPU_OK) return s;
    if (!u || !v || !w || (np > 0 && !affine))
        return fail(c, JETGPU_BAD_INPUT, "null grid or affine arrays");
    JG_CUDA(c, cudaSetDevice(c->device));
    return apic_g2p(c, to_desc(grid), np, pos, vel, affine, u, v, w);
}

jetgpu_status jetgpu_move_particles_device(
    jetgpu_ctx* c, const jetgpu_grid* grid, long np, double* pos, double* vel,
    const double* u, const double* v, const double* w, double dt,
    double max_cfl, int closed, const jetgpu_collider* col,
    const jetgpu_sphere* sph) {
    jetgpu_status s = check_transfer(c, grid, np, pos, vel);
    if (s != JETGPU_OK) return s;
    if (!u || !v || !w) return fail(c, JETGPU_BAD_INPUT, "null grid arrays");
    if (!std::isfinite(dt) || !std::isfinite(max_cfl))
        return fail(c, JETGPU_BAD_INPUT, "non-finite time step or CFL");
    if (sph && !(sph->radius >= 0.0))
        return fail(c, JETGPU_BAD_INPUT, "sphere radius must be >= 0");
    JG_CUDA(c, cudaSetDevice(c->device));
    return move_particles(c, to_desc(grid), np, pos, vel, u, v, w, dt, max_cfl,
                          closed, col, sph);
}

jetgpu_status jetgpu_move_particles(
    jetgpu_ctx* c, const jetgpu_grid* grid, long np, double* pos, double* vel,
    const double* u, const double* v, const double* w, double dt,
    double max_cfl, int closed, const jetgpu_collider* col,
    const jetgpu_sphere* sph) {
    jetgpu_status s = check_transfer(c, grid, np, pos, vel);
    if (s != JETGPU_OK) return s;
    if (!u || !v || !w) return fail(c, JETGPU_BAD_INPUT, "null grid arrays");
    if (!std::isfinite(dt) || !std::isfinite(max_cfl))
        return fail(c, JETGPU_BAD_INPUT, "non-finite time step or CFL");
    if (sph && !(sph->radius >= 0.0))
        return fail(c, JETGPU_BAD_INPUT, "sphere radius must be >= 0");
    JG_CUDA(c, cudaSetDevice(c->device));
    size_t n[3];
    face_counts(grid, n);
    const size_t nf = n[0] + n[1] + n[2];
    s = grow_stage(c, (size_t)np * 48 + nf * 8 + 64);
    if (s != JETGPU_OK) return s;
    unsigned char* p = c->stage;
    double* dpos = reinterpret_cast<double*>(p); p += (size_t)np * 24;
    double* dvel = reinterpret_cast<double*>(p); p += (size_t)np * 24;
    double* dg = reinterpret_cast<double*>(p);
    cudaStream_t st = c->stream;
    const double* ins[3] = {u, v, w};
    if (np) {
        JG_CUDA(c, cudaMemcpyAsync(dpos, pos, np * 24, cudaMemcpyHostToDevice, st));
        JG_CUDA(c, cudaMemcpyAsync(dvel, vel, np * 24, cudaMemcpyHostToDevice, st));
    }
    size_t off = 0;
    for (int a = 0; a < 3; ++a) {
        JG_CUDA(c, cudaMemcpyAsync(dg + off, ins[a], n[a] * 8, cudaMemcpyHostToDevice, st));
        off += n[a];
    }
    s = move_particles(c, to_desc(grid), np, dpos, dvel, dg, dg + n[0],
                       dg + n[0] + n[1], dt, max_cfl, closed, col, sph);
    if (s != JETGPU_OK) return s;
    if (np) {
        JG_CUDA(c, cudaMemcpyAsync(pos, dpos, np * 24, cudaMemcpyDeviceToHost, st));
        JG_CUDA(c, cudaMemcpyAsync(vel, dvel, np * 24, cudaMemcpyDeviceToHost, st));
    }
    JG_CUDA(c, cudaStreamSynchronize(st));
    return JETGPU_OK;
}

jetgpu_status jetgpu_build_particle_sdf_device(
    jetgpu_ctx* c, const jetgpu_grid* grid, long np, const double* pos,
    const jetgpu_scalar_field* collider_sdf, double max_cfl, double* sdf) {
    if (!c) return JETGPU_BAD_INPUT;
    jetgpu_status s;
    if ((s = check_grid(c, grid)) != JETGPU_OK) return s;
    if ((s = check_field(c, collider_sdf, "collider_sdf")) != JETGPU_OK) return s;
    if (np < 0 || (np > 0 && !pos) || !sdf)
        return fail(c, JETGPU_BAD_INPUT, "bad particle or output arguments");
    if (np > 2147483647L)
        return fail(c, JETGPU_BAD_INPUT, "more than 2^31 - 1 particles");
    if (!std::isfinite(max_cfl) || max_cfl < 0.0)
        return fail(c, JETGPU_BAD_INPUT, "max_cfl must be finite and >= 0");
    JG_CUDA(c, cudaSetDevice(c->device));
    return build_particle_sdf(c, to_desc(grid), np, pos,
                              to_desc(collider_sdf, collider_sdf->data),
                              max_cfl, sdf);
}

jetgpu_status jetgpu_build_particle_sdf(jetgpu_ctx* c, const jetgpu_grid* grid,
                                        long np, const double* pos,
                                        const jetgpu_scalar_field* collider_sdf,
                                        double max_cfl, double* sdf) {
    if (!c) return JETGPU_BAD_INPUT;
    jetgpu_status s;
    if ((s = check_grid(c, grid)) != JETGPU_OK) return s;
    if ((s = check_field(c, collider_sdf, "collider_sdf")) != JETGPU_OK) return s;
    if (np < 0 || (np > 0 && !pos) || !sdf)
        return fail(c, JETGPU_BAD_INPUT, "bad particle or output arguments");
    if (np > 2147483647L)
        return fail(c, JETGPU_BAD_INPUT, "more than 2^31 - 1 particles");
    if (!std::isfinite(max_cfl) || max_cfl < 0.0)
        return fail(c, JETGPU_BAD_INPUT, "max_cfl must be finite and >= 0");
    JG_CUDA(c, cudaSetDevice(c->device));
    const size_t cells = (size_t)grid->res[0] * grid->res[1] * grid->res[2];
    const size_t ns = (size_t)field_count(collider_sdf);
    s = grow_stage(c, (size_t)np * 24 + (cells + ns) * 8 + 64);
    if (s != JETGPU_OK) return s;
    unsigned char* p = c->stage;
    double* dpos = reinterpret_cast<double*>(p); p += (size_t)np * 24;
    double* dout = reinterpret_cast<double*>(p); p += cells * 8;
    double* dcol = reinterpret_cast<double*>(p);
    cudaStream_t st = c->stream;
    if (np)
        JG_CUDA(c, cudaMemcpyAsync(dpos, pos, np * 24, cudaMemcpyHostToDevice, st));
    if (ns)
        JG_CUDA(c, cudaMemcpyAsync(dcol, collider_sdf->data, ns * 8,
                                   cudaMemcpyHostToDevice, st));
    s = build_particle_sdf(c, to_desc(grid), np, dpos,
                           to_desc(collider_sdf, ns ? dcol : nullptr), max_cfl,
                           dout);
    if (s != JETGPU_OK) return s;
    JG_CUDA(c, cudaMemcpyAsync(sdf, dout, cells * 8, cudaMemcpyDeviceToHost, st));
    JG_CUDA(c, cudaStreamSynchronize(st));
    return JETGPU_OK;
}

void jetgpu_flip_params_default(jetgpu_flip_params* p) {
    if (!p) return;
    p->gravity[0] = 0.0;
    p->gravity[1] = -9.8;
    p->gravity[2] = 0.0;
    p->max_cfl = 5.0;
    p->closed_domain_flags = JETGPU_DIRECTION_ALL;
    p->flip = 1;
    p->pic_blending = 0.0;
}

jetgpu_status jetgpu_fluid_cfl_device(jetgpu_ctx* c, const jetgpu_grid* grid,
                                      const double* u, const double* v,
                                      const double* w, double dt,
                                      const double gravity[3], double* cfl) {
    if (!c) return JETGPU_BAD_INPUT;
    jetgpu_status s;
    if ((s = check_grid(c, grid)) != JETGPU_OK) return s;
    if (!u || !v || !w || !gravity || !cfl)
        return fail(c, JETGPU_BAD_INPUT, "null argument");
    JG_CUDA(c, cudaSetDevice(c->device));
    return fluid_cfl(c, to_desc(grid), u, v, w, dt, gravity, cfl);
}

jetgpu_status jetgpu_flip_substep_device(
    jetgpu_ctx* c, const jetgpu_grid* grid, long np, double* pos, double* vel,
    double* affine, double* u, double* v, double* w, double* fluid_sdf,
    const jetgpu_scalar_field* collider_sdf, const jetgpu_collider* collider,
    const jetgpu_sphere* sphere, const jetgpu_flip_params* prm, double dt,
    jetgpu_solve_stats* stats) {
    jetgpu_status s = check_transfer(c, grid, np, pos, vel);
    if (s != JETGPU_OK) return s;
    if ((s = check_field(c, collider_sdf, "collider_sdf")) != JETGPU_OK) return s;
    if (!u || !v || !w || !fluid_sdf || !prm)
        return fail(c, JETGPU_BAD_INPUT, "null argument");
    if (prm->flip < 0 || prm->flip > 2)
        return fail(c, JETGPU_BAD_INPUT, "flip must be 0 (PIC), 1 or 2 (APIC)");
    if (prm->flip == 2 && np > 0 && !affine)
        return fail(c, JETGPU_BAD_INPUT, "APIC needs the affine array");
    if (np > 2147483647L)
        return fail(c, JETGPU_BAD_INPUT, "more than 2^31 - 1 particles");
    if (!std::isfinite(dt) || !(dt >= 0.0) || !std::isfinite(prm->max_cfl) ||
        prm->max_cfl < 0.0)
        return fail(c, JETGPU_BAD_INPUT, "bad time step or maxCfl");
    if (sphere && !(sphere->radius >= 0.0))
        return fail(c, JETGPU_BAD_INPUT, "sphere radius must be >= 0");
    JG_CUDA(c, cudaSetDevice(c->device));
    jetgpu_solve_stats local;
    std::memset(&local, 0, sizeof(local));
    s = flip_substep(c, to_desc(grid), np, pos, vel, affine, u, v, w,
                     fluid_sdf,
                     to_desc(collider_sdf, collider_sdf->data), collider,
                     sphere, *prm, dt, &local);
    if (stats) *stats = local;
    return s;
}

jetgpu_status jetgpu_extrapolate_to_region_device(jetgpu_ctx* c,
                                                  const int res[3],
                                                  double* data,
                                                  const unsigned char* valid,
                                                  unsigned int iterations) {
    if (!c) return JETGPU_BAD_INPUT;
    if (!res || !data || !valid)
        return fail(c, JETGPU_BAD_INPUT, "null argument");
    for (int a = 0; a < 3; ++a)
        if (res[a] < 1) return fail(c, JETGPU_BAD_INPUT, "resolution < 1");
    if ((double)res[0] * res[1] * res[2] > 2147483647.0)
        return fail(c, JETGPU_BAD_INPUT, "grid too large");
    JG_CUDA(c, cudaSetDevice(c->device));
    return extrapolate_region(c, Dims{res[0], res[1], res[2]}, data, valid,
                              iterations);
}

}  // extern "C"

// ---- live per-kernel profile -------------------------------------------------

namespace jg {

const char* kernel_class_name(int cls) {
    static const char* names[K_CLASS_COUNT] = {
        "rb_sweep_fused_l0", "rb_sweep_fused_coarse", "rb_half_l0",
        "rb_half_coarse", "coarsest", "residual32", "restrict",
        "correct", "spmv_dot", "update_xr", "dot_rz", "update_d",
        "residual64", "accumulate", "weights", "pyramid", "system",
        "gradient", "p2g", "g2p",
        "unet", "boundary", "particle_sdf", "move_particles"};
    return (cls >= 0 && cls < K_CLASS_COUNT) ? names[cls] : "?";
}

int prof_begin(Ctx* c) {
    if (!c->prof_on) return -1;
    if (c->prof_used + 2 > c->prof_ev.size()) {
        for (int i = 0; i < 256; ++i) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return -1;
            c->prof_ev.push_back(e);
        }
    }
    const int e0 = (int)c->prof_used++;
    cudaEventRecord(c->prof_ev[e0], c->stream);
    return e0;
}

void prof_end(Ctx* c, int cls, int e0, double bytes) {
    if (e0 < 0 || !c->prof_on) return;
    const int e1 = (int)c->prof_used++;
    cudaEventRecord(c->prof_ev[e1], c->stream);
    c->prof_recs.push_back(ProfRec{cls, e0, e1, bytes});
}

}  // namespace jg

extern "C" {

jetgpu_status jetgpu_get_stream(jetgpu_ctx* c, void** stream) {
    if (!c || !stream) return JETGPU_BAD_INPUT;
    *stream = (void*)c->stream;
    return JETGPU_OK;
}

jetgpu_status jetgpu_profile(jetgpu_ctx* c, int enable) {
    if (!c) return JETGPU_BAD_INPUT;
    JG_CUDA(c, cudaStreamSynchronize(c->stream));
    c->prof_on = enable != 0;
    c->prof_used = 0;
    c->prof_recs.clear();
    return JETGPU_OK;
}

jetgpu_status jetgpu_profile_read(jetgpu_ctx* c, jetgpu_kernel_stat* out,
                                  int capacity, int* count) {
    if (!c || !count) return JETGPU_BAD_INPUT;
    JG_CUDA(c, cudaStreamSynchronize(c->stream));
    jetgpu_kernel_stat acc[K_CLASS_COUNT];
    std::memset(acc, 0, sizeof(acc));
    for (const ProfRec& r : c->prof_recs) {
        float ms = 0.f;
        JG_CUDA(c, cudaEventElapsedTime(&ms, c->prof_ev[r.e0], c->prof_ev[r.e1]));
        jetgpu_kernel_stat& a = acc[r.cls];
        a.launches += 1;
        a.total_ms += ms;
        a.bytes += r.bytes;
    }
    int n = 0;
    for (int k = 0; k < K_CLASS_COUNT; ++k) {
        if (acc[k].launches == 0) continue;
        if (out && n < capacity) {
            out[n] = acc[k];
            std::snprintf(out[n].name, sizeof(out[n].name), "%s",
                          kernel_class_name(k));
        }
        ++n;
    }
    *count = n;
    return JETGPU_OK;
}

}  // extern "C"

// ---- learned preconditioner ------------------------------------------------

extern "C" {

size_t jetgpu_net_param_count(void) { return net_param_count(); }

jetgpu_status jetgpu_load_unet(jetgpu_ctx* c, const float* params,
                               size_t count) {
    if (!c || !params) return JETGPU_BAD_INPUT;
    JG_CUDA(c, cudaSetDevice(c->device));
    return net_load(c, params, count);
}

jetgpu_status jetgpu_harvest(jetgpu_ctx* c, unsigned int max_pairs,
                             float* r_out, float* z_out, unsigned int* count) {
    if (!c || !r_out || !z_out || !count) return JETGPU_BAD_INPUT;
    if (c->built_levels == 0)
        return fail(c, JETGPU_BAD_INPUT, "no system: run a pressure solve first");
    JG_CUDA(c, cudaSetDevice(c->device));
    return harvest_pairs(c, max_pairs, r_out, z_out, count);
}

unsigned jetgpu_net_level(const jetgpu_ctx* c) {
    return (c && c->built_levels > 0) ? net_level(c) : 0u;
}

jetgpu_status jetgpu_net_features(jetgpu_ctx* c, unsigned level,
                                  const float* r, void* feat) {
    if (!c || !r || !feat) return JETGPU_BAD_INPUT;
    if (c->built_levels == 0)
        return fail(c, JETGPU_BAD_INPUT, "no system: run a pressure solve first");
    if (level >= c->built_levels)
        return fail(c, JETGPU_BAD_INPUT, "level beyond the built hierarchy");
    JG_CUDA(c, cudaSetDevice(c->device));
    jetgpu_status s = norm2f(c, r, c->levels[level].n.count(), S_MEAN);
    if (s != JETGPU_OK) return s;
    s = net_features(c, level, r, c->scal + S_MEAN, feat);
    if (s != JETGPU_OK) return s;
    JG_CUDA(c, cudaStreamSynchronize(c->stream));
    return JETGPU_OK;
}

jetgpu_status jetgpu_vcycle_apply(jetgpu_ctx* c, const float* r, float* z) {
    if (!c || !r || !z) return JETGPU_BAD_INPUT;
    if (c->built_levels == 0)
        return fail(c, JETGPU_BAD_INPUT, "no system: run a pressure solve first");
    JG_CUDA(c, cudaSetDevice(c->device));
    const Level& L0 = c->levels[0];
    const long N = L0.n.count();
    // The V-cycle writes into its own buffers (the finest level's x and its
    // ping-pong partner); r is copied in first so that it may alias z.
    JG_CUDA(c, cudaMemcpyAsync(L0.b, r, N * sizeof(float),
                               cudaMemcpyDeviceToDevice, c->stream));
    float* res = nullptr;
    jetgpu_status s = vcycle(c, L0.b, L0.x, L0.x2, &res);
    if (s != JETGPU_OK) return s;
    JG_CUDA(c, cudaMemcpyAsync(z, res, N * sizeof(float),
                               cudaMemcpyDeviceToDevice, c->stream));
    JG_CUDA(c, cudaStreamSynchronize(c->stream));
    return JETGPU_OK;
}

jetgpu_status jetgpu_net_apply(jetgpu_ctx* c, unsigned level, const float* r,
                               float* e) {
    if (!c || !r || !e) return JETGPU_BAD_INPUT;
    if (c->built_levels == 0 || !c->unet)
        return fail(c, JETGPU_BAD_INPUT,
                    "needs a solved system and a loaded network");
    if (level >= c->built_levels)
        return fail(c, JETGPU_BAD_INPUT, "level beyond the built hierarchy");
    const Dims n = c->levels[level].n;
    if (n.x % 8 || n.y % 8 || n.z % 8)
        return fail(c, JETGPU_BAD_INPUT,
                    "the network needs a level whose extents are multiples "
                    "of 8");
    JG_CUDA(c, cudaSetDevice(c->device));
    jetgpu_status s = norm2f(c, r, n.count(), S_MEAN);
    if (s != JETGPU_OK) return s;
    s = net_apply(c, level, r, c->scal + S_MEAN, e);
    if (s != JETGPU_OK) return s;
    JG_CUDA(c, cudaStreamSynchronize(c->stream));
    return JETGPU_OK;
}

jetgpu_status jetgpu_learned_apply(jetgpu_ctx* c, const float* r, float* z) {
    if (!c || !r || !z || r == z) return JETGPU_BAD_INPUT;
    if (c->built_levels == 0 || !net_supported(c))
        return fail(c, JETGPU_BAD_INPUT,
                    "needs a solved system whose network level has extents "
                    "divisible by 8, and a loaded network");
    JG_CUDA(c, cudaSetDevice(c->device));
    jetgpu_status s = learned_precond(c, r, z);
    if (s != JETGPU_OK) return s;
    JG_CUDA(c, cudaStreamSynchronize(c->stream));
    return JETGPU_OK;
}

}  // extern "C"

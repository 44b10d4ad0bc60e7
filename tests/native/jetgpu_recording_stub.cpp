// A stand-in for libjetgpu that records how the C++ drop-ins call the C ABI
// (test infrastructure: no GPU work). It defines the entry points the
// adapters in fluid-engine-dev_gb300/jet_plugin/ reference, with the
// declarations of include/jetgpu.h. A pressure solve copies the input
// velocity to the output and writes zero pressure; a boundary-condition call
// leaves the velocity as it is. The recorded arguments are read back through
// jetgpu_stub_record().
#include <cstring>

#include "jetgpu.h"

extern "C" {

struct jetgpu_stub_record_t {
    int solve_calls;           // jetgpu_solve_pressure
    int solve_collider_calls;  // jetgpu_solve_pressure_collider
    int blocked_calls;         // jetgpu_solve_pressure_blocked
    int constrain_calls;       // jetgpu_constrain_velocity[_blocked]
    // Arguments of the last pressure solve of either kind.
    const double* solid[3];
    const double* boundary_data;
    const double* fluid_data;
    int boundary_kind, fluid_kind;
    int had_collider;
    jetgpu_collider collider;
};

static jetgpu_stub_record_t g_rec;
static int g_ctx_token;

const jetgpu_stub_record_t* jetgpu_stub_record(void) { return &g_rec; }
void jetgpu_stub_reset(void) { std::memset(&g_rec, 0, sizeof(g_rec)); }

void jetgpu_config_default(jetgpu_config* cfg) {
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->max_cg_iter = 100;
    cfg->max_levels = 6;
    cfg->tolerance = 1e-6;
    cfg->sor = 1.2;
    cfg->red_black = 1;
}

jetgpu_status jetgpu_create(const jetgpu_config*, struct jetgpu_ctx** out) {
    *out = reinterpret_cast<struct jetgpu_ctx*>(&g_ctx_token);
    return JETGPU_OK;
}

void jetgpu_destroy(struct jetgpu_ctx*) {}

const char* jetgpu_last_error(const struct jetgpu_ctx*) { return ""; }

const char* jetgpu_version(void) { return "recording stub"; }

static void copy_faces(const jetgpu_grid* g, const double* u, const double* v,
                       const double* w, double* ou, double* ov, double* ow,
                       double* p) {
    const size_t nx = g->res[0], ny = g->res[1], nz = g->res[2];
    std::memmove(ou, u, (nx + 1) * ny * nz * sizeof(double));
    std::memmove(ov, v, nx * (ny + 1) * nz * sizeof(double));
    std::memmove(ow, w, nx * ny * (nz + 1) * sizeof(double));
    if (p) std::memset(p, 0, nx * ny * nz * sizeof(double));
}

static void record_fields(const jetgpu_scalar_field* b,
                          const jetgpu_scalar_field* f) {
    g_rec.boundary_kind = b->kind;
    g_rec.boundary_data = b->data;
    g_rec.fluid_kind = f->kind;
    g_rec.fluid_data = f->data;
}

jetgpu_status jetgpu_solve_pressure(
    struct jetgpu_ctx*, const jetgpu_grid* grid, const double* u,
    const double* v, const double* w, const jetgpu_scalar_field* boundary_sdf,
    const jetgpu_scalar_field* fluid_sdf, const double* solid_u,
    const double* solid_v, const double* solid_w, double* out_u,
    double* out_v, double* out_w, double* out_pressure,
    jetgpu_solve_stats* stats) {
    ++g_rec.solve_calls;
    g_rec.solid[0] = solid_u;
    g_rec.solid[1] = solid_v;
    g_rec.solid[2] = solid_w;
    g_rec.had_collider = 0;
    record_fields(boundary_sdf, fluid_sdf);
    copy_faces(grid, u, v, w, out_u, out_v, out_w, out_pressure);
    if (stats) std::memset(stats, 0, sizeof(*stats));
    return JETGPU_OK;
}

jetgpu_status jetgpu_solve_pressure_collider(
    struct jetgpu_ctx*, const jetgpu_grid* grid, const double* u,
    const double* v, const double* w, const jetgpu_scalar_field* boundary_sdf,
    const jetgpu_scalar_field* fluid_sdf, const jetgpu_collider* collider,
    double* out_u, double* out_v, double* out_w, double* out_pressure,
    jetgpu_solve_stats* stats) {
    ++g_rec.solve_collider_calls;
    g_rec.solid[0] = g_rec.solid[1] = g_rec.solid[2] = nullptr;
    g_rec.had_collider = collider != nullptr;
    if (collider) g_rec.collider = *collider;
    record_fields(boundary_sdf, fluid_sdf);
    copy_faces(grid, u, v, w, out_u, out_v, out_w, out_pressure);
    if (stats) std::memset(stats, 0, sizeof(*stats));
    return JETGPU_OK;
}

jetgpu_status jetgpu_get_level(struct jetgpu_ctx*, int, int, void* dst,
                               size_t capacity, size_t* count) {
    if (dst && capacity) std::memset(dst, 0, capacity);
    if (count) *count = 0;
    return JETGPU_OK;
}

jetgpu_status jetgpu_solve_pressure_blocked(
    struct jetgpu_ctx*, const jetgpu_grid* grid, const double* u,
    const double* v, const double* w, const jetgpu_scalar_field* boundary_sdf,
    const jetgpu_scalar_field* fluid_sdf, double* out_u, double* out_v,
    double* out_w, double* out_pressure, jetgpu_solve_stats* stats) {
    ++g_rec.blocked_calls;
    record_fields(boundary_sdf, fluid_sdf);
    copy_faces(grid, u, v, w, out_u, out_v, out_w, out_pressure);
    if (stats) std::memset(stats, 0, sizeof(*stats));
    return JETGPU_OK;
}

jetgpu_status jetgpu_constrain_velocity(struct jetgpu_ctx*,
                                        const jetgpu_grid*, double*, double*,
                                        double*, const jetgpu_scalar_field*,
                                        const jetgpu_collider*, int,
                                        unsigned int) {
    ++g_rec.constrain_calls;
    return JETGPU_OK;
}

jetgpu_status jetgpu_constrain_velocity_blocked(
    struct jetgpu_ctx*, const jetgpu_grid*, double*, double*, double*,
    const jetgpu_scalar_field*, const jetgpu_collider*, int, unsigned int) {
    ++g_rec.constrain_calls;
    return JETGPU_OK;
}

}  // extern "C"

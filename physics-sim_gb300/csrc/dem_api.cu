// dem_api.cu -- the C ABI of include/dem.h over a single-scene World.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <new>
#include <string>
#include <vector>

#include "dem.h"
#include "dem_debug.h"
#include "dem_world_host.h"

struct dem_ctx {
    demgb::World world;
    std::string msg;
};

namespace {
thread_local std::string g_create_error;

int set_err(dem_ctx *ctx, int code, const std::string &m) {
    if (ctx) ctx->msg = m;
    else g_create_error = m;
    return code;
}
int world_rc(dem_ctx *ctx, int rc) {
    if (rc != DEM_OK) ctx->msg = ctx->world.err;
    return rc;
}
}  // namespace

extern "C" {

int dem_abi_version(void) { return DEM_ABI_VERSION; }

void dem_ext_defaults(dem_ext *ext) {
    if (!ext) return;
    std::memset(ext, 0, sizeof *ext);
    ext->bond_lambda = 0.5f;
    ext->diagnostics = 1;
}

const char *dem_last_error(const dem_ctx *ctx) {
    if (!ctx) return g_create_error.c_str();
    return ctx->msg.c_str();
}

int dem_grid_capacity(const dem_params *p, const float *radii, int32_t n_radii, int32_t particles,
                      dem_grid_info *out) {
    if (!p || !out || n_radii < 0 || (n_radii > 0 && !radii)) return DEM_E_INVALID;
    // State::load: min/max over the whole radii vector (state.rs:684-698)
    float mn = std::numeric_limits<float>::max(), mx = std::numeric_limits<float>::lowest();
    for (int i = 0; i < n_radii; ++i) {
        mn = radii[i] < mn ? radii[i] : mn;
        mx = radii[i] > mx ? radii[i] : mx;
    }
    if (n_radii == 0) mn = mx = 0.0f;
    // grid_capacity (wgpu_prog.rs:698-717), float arithmetic, Rust `as i32` saturating
    auto as_i32 = [](float x) -> int32_t {
        if (x != x) return 0;
        if (x >= 2147483648.0f) return 2147483647;
        if (x <= -2147483648.0f) return (int32_t)(-2147483647 - 1);
        return (int32_t)x;
    };
    bool variable_rad = mn != mx;
    float width = p->hor_bound * 2.0f;
    float height = p->vert_bound * 2.0f;
    float max_rad = mx * 2.0f;
    float min_rad = variable_rad ? mn : mx;
    int32_t w = as_i32(std::ceil(width / max_rad));
    int32_t h = as_i32(std::ceil(height / max_rad));
    float q = max_rad / min_rad + 1.0f;
    int32_t cap = as_i32(std::ceil(q * q));
    if (cap > particles) cap = particles;
    out->cell_size = max_rad;
    out->cell_cap = cap + 2;
    out->w = w;
    out->h = h;
    if (!(max_rad > 0.0f) || w <= 0 || h <= 0) return DEM_E_INVALID;
    return DEM_OK;
}

int dem_create(const dem_scene *scene, const dem_params *params, const dem_ext *ext, int device,
               dem_ctx **out) {
    if (!out) return set_err(nullptr, DEM_E_INVALID, "out is NULL");
    *out = nullptr;
    if (!scene || !params) return set_err(nullptr, DEM_E_INVALID, "scene/params is NULL");
    dem_ext e;
    if (ext) e = *ext;
    else dem_ext_defaults(&e);
    dem_ctx *ctx = new (std::nothrow) dem_ctx();
    if (!ctx) return set_err(nullptr, DEM_E_OOM, "host allocation failed");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        delete ctx;
        return set_err(nullptr, DEM_E_CUDA, "no CUDA device available");
    }
    if (device >= 0) {
        if (device >= ndev || cudaSetDevice(device) != cudaSuccess) {
            delete ctx;
            return set_err(nullptr, DEM_E_INVALID, "bad device index");
        }
    }
    cudaGetDevice(&ctx->world.device);
    if (cudaStreamCreateWithFlags(&ctx->world.stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete ctx;
        return set_err(nullptr, DEM_E_CUDA, "stream creation failed");
    }
    std::vector<const dem_scene *> scenes{scene};
    std::vector<dem_params> ps{*params};
    std::vector<dem_ext> es{e};
    int rc = ctx->world.build(scenes, ps, es);
    if (rc != DEM_OK) {
        std::string m = ctx->world.err;
        cudaStreamDestroy(ctx->world.stream);
        ctx->world.stream = nullptr;
        delete ctx;
        return set_err(nullptr, rc, m);
    }
    *out = ctx;
    return DEM_OK;
}

void dem_destroy(dem_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->world.device);
    if (ctx->world.stream) cudaStreamSynchronize(ctx->world.stream);
    cudaStream_t st = ctx->world.stream;
    delete ctx;  // frees device memory
    if (st) cudaStreamDestroy(st);
}

#define CTX_GUARD(ctx)                                        \
    do {                                                      \
        if (!(ctx)) return DEM_E_INVALID;                     \
        cudaSetDevice((ctx)->world.device);                   \
    } while (0)

int dem_upload(dem_ctx *ctx, const dem_scene *scene) {
    CTX_GUARD(ctx);
    return world_rc(ctx, ctx->world.upload_scene(0, scene));
}

int dem_set_params(dem_ctx *ctx, const dem_params *params) {
    CTX_GUARD(ctx);
    if (!params) return set_err(ctx, DEM_E_INVALID, "params is NULL");
    return world_rc(ctx, ctx->world.set_params(0, *params));
}

int dem_set_materials(dem_ctx *ctx, const float *materials, int32_t n_materials) {
    CTX_GUARD(ctx);
    return world_rc(ctx, ctx->world.set_materials(0, materials, n_materials));
}

int dem_set_control(dem_ctx *ctx, const int32_t coll_cont[4]) {
    CTX_GUARD(ctx);
    if (!coll_cont) return set_err(ctx, DEM_E_INVALID, "coll_cont is NULL");
    return world_rc(ctx, ctx->world.set_control(0, coll_cont));
}

int dem_get_control(dem_ctx *ctx, int32_t coll_cont[4]) {
    CTX_GUARD(ctx);
    if (!coll_cont) return set_err(ctx, DEM_E_INVALID, "coll_cont is NULL");
    ctx->world.control(0, coll_cont);
    return DEM_OK;
}

int dem_step(dem_ctx *ctx, int32_t n_steps) {
    CTX_GUARD(ctx);
    return world_rc(ctx, ctx->world.step(n_steps));
}

int dem_synchronize(dem_ctx *ctx) {
    CTX_GUARD(ctx);
    return world_rc(ctx, ctx->world.sync());
}

int dem_download(dem_ctx *ctx, dem_scene *out) {
    CTX_GUARD(ctx);
    return world_rc(ctx, ctx->world.download_scene(0, out));
}

int dem_set_properties(dem_ctx *ctx, int32_t *selections, const int32_t props[DEM_PROPS_WORDS]) {
    CTX_GUARD(ctx);
    return world_rc(ctx, ctx->world.set_properties(0, selections, props));
}

int dem_event(dem_ctx *ctx, int32_t kind, int32_t *selections, int32_t throw_particles, float del_x, float del_y,
              int32_t ticks) {
    CTX_GUARD(ctx);
    return world_rc(ctx, ctx->world.fixity_event(0, kind, selections, throw_particles, del_x, del_y, ticks));
}

int dem_get_datum(dem_ctx *ctx, const int32_t *selections, double out[10]) {
    CTX_GUARD(ctx);
    const int rc = ctx->world.get_datum(0, selections, out);
    return rc < 0 ? world_rc(ctx, rc) : rc;
}

int dem_record(dem_ctx *ctx, int32_t n_steps, const int32_t *selections, double *rows) {
    CTX_GUARD(ctx);
    const int rc = ctx->world.record(0, selections, n_steps, rows);
    return rc < 0 ? world_rc(ctx, rc) : rc;
}

int dem_break_events(dem_ctx *ctx, dem_break_event *buf, int32_t cap, int32_t *n) {
    CTX_GUARD(ctx);
    if (cap < 0 || (cap > 0 && !buf)) return set_err(ctx, DEM_E_INVALID, "bad event buffer");
    std::vector<dem_break_event> ev;
    int rc = ctx->world.drain_events(ev);
    if (rc) return world_rc(ctx, rc);
    int32_t k = (int32_t)std::min<size_t>(ev.size(), (size_t)cap);
    if (k) std::memcpy(buf, ev.data(), sizeof(dem_break_event) * k);
    if (n) *n = k;
    if ((size_t)k < ev.size()) return set_err(ctx, DEM_E_CAPACITY, "event buffer smaller than pending events");
    return DEM_OK;
}

int dem_get_stats(dem_ctx *ctx, dem_stats *out) {
    CTX_GUARD(ctx);
    if (!out) return set_err(ctx, DEM_E_INVALID, "out is NULL");
    return world_rc(ctx, ctx->world.stats(out));
}

void *dem_stream(dem_ctx *ctx) { return ctx ? (void *)ctx->world.stream : nullptr; }

// Standalone broad phase over the context's current positions: keys per
// particle (search cell, scene-local), the stable cell order (particle
// indices) and the cell start table.  Declared in dem_debug.h.
int dem_debug_broad_phase(dem_ctx *ctx, int32_t *keys, int32_t *order, int32_t *cell_start,
                          int32_t *n_cells) {
    CTX_GUARD(ctx);
    return world_rc(ctx, ctx->world.broad_phase_snapshot(0, keys, order, cell_start, n_cells));
}

int dem_debug_search_grid(dem_ctx *ctx, float *x0, float *y0, float *inv, int32_t *gw, int32_t *gh) {
    CTX_GUARD(ctx);
    const demgb::ScenePar &P = ctx->world.sh[0].par;
    if (x0) *x0 = P.g_x0;
    if (y0) *y0 = P.g_y0;
    if (inv) *inv = P.g_inv;
    if (gw) *gw = P.g_w;
    if (gh) *gh = P.g_h;
    return DEM_OK;
}

int dem_debug_kernel_timing(dem_ctx *ctx, int32_t enable) {
    CTX_GUARD(ctx);
    ctx->world.set_timing(enable != 0);
    return DEM_OK;
}

int dem_debug_kernel_time(dem_ctx *ctx, const char *kernel, double *total_ms, int64_t *launches) {
    CTX_GUARD(ctx);
    if (!kernel) return set_err(ctx, DEM_E_INVALID, "kernel is NULL");
    static const char *names[6] = {"interact", "lom", "broad_phase", "reorder", "end_step", "candidate_lists"};
    for (int k = 0; k < 6; ++k) {
        if (std::strcmp(kernel, names[k]) == 0) {
            long long n = 0;
            int rc = ctx->world.kernel_time(k, total_ms, &n);
            if (launches) *launches = n;
            return world_rc(ctx, rc);
        }
    }
    return set_err(ctx, DEM_E_INVALID, "unknown kernel name");
}

}  // extern "C"

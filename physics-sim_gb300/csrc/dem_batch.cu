// dem_batch.cu -- C ABI of a batch of independent scenes stepped together
// (include/dem.h, "Batches").  All scenes of a batch live in one device
// world; each step launches the same two kernels over every particle of
// every scene, so many small scenes fill the GPU the way one large scene
// would.  Per-scene arithmetic is exactly the single-scene arithmetic.
#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "dem.h"
#include "dem_debug.h"
#include "dem_world_host.h"

struct dem_batch {
    demgb::World world;
    std::string msg;
};

namespace {
thread_local std::string g_batch_create_error;

int bset(dem_batch *b, int code, const std::string &m) {
    if (b) b->msg = m;
    else g_batch_create_error = m;
    return code;
}
int brc(dem_batch *b, int rc) {
    if (rc != DEM_OK) b->msg = b->world.err;
    return rc;
}
}  // namespace

#define BATCH_GUARD(b)                        \
    do {                                      \
        if (!(b)) return DEM_E_INVALID;       \
        cudaSetDevice((b)->world.device);     \
    } while (0)

extern "C" {

const char *dem_batch_last_error(const dem_batch *b) {
    return b ? b->msg.c_str() : g_batch_create_error.c_str();
}

int dem_batch_create(const dem_scene *const *scenes, const dem_params *params, const dem_ext *exts,
                     int32_t n_scenes, int device, dem_batch **out) {
    if (!out) return bset(nullptr, DEM_E_INVALID, "out is NULL");
    *out = nullptr;
    if (!scenes || !params || n_scenes <= 0) return bset(nullptr, DEM_E_INVALID, "no scenes");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return bset(nullptr, DEM_E_CUDA, "no CUDA device available");
    if (device >= 0 && (device >= ndev || cudaSetDevice(device) != cudaSuccess))
        return bset(nullptr, DEM_E_INVALID, "bad device index");
    dem_batch *b = new (std::nothrow) dem_batch();
    if (!b) return bset(nullptr, DEM_E_OOM, "host allocation failed");
    cudaGetDevice(&b->world.device);
    if (cudaStreamCreateWithFlags(&b->world.stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete b;
        return bset(nullptr, DEM_E_CUDA, "stream creation failed");
    }
    std::vector<const dem_scene *> sc(scenes, scenes + n_scenes);
    std::vector<dem_params> ps(params, params + n_scenes);
    std::vector<dem_ext> es(n_scenes);
    for (int s = 0; s < n_scenes; ++s) {
        if (exts) es[s] = exts[s];
        else dem_ext_defaults(&es[s]);
    }
    int rc = b->world.build(sc, ps, es);
    if (rc != DEM_OK) {
        std::string m = b->world.err;
        cudaStream_t st = b->world.stream;
        delete b;
        cudaStreamDestroy(st);
        return bset(nullptr, rc, m);
    }
    *out = b;
    return DEM_OK;
}

void dem_batch_destroy(dem_batch *b) {
    if (!b) return;
    cudaSetDevice(b->world.device);
    cudaStream_t st = b->world.stream;
    if (st) cudaStreamSynchronize(st);
    delete b;
    if (st) cudaStreamDestroy(st);
}

int dem_batch_scene_count(const dem_batch *b) { return b ? (int)b->world.sh.size() : 0; }

int dem_batch_step(dem_batch *b, int32_t n_steps) {
    BATCH_GUARD(b);
    return brc(b, b->world.step(n_steps));
}

int dem_batch_synchronize(dem_batch *b) {
    BATCH_GUARD(b);
    return brc(b, b->world.sync());
}

int dem_batch_download(dem_batch *b, int32_t scene, dem_scene *out) {
    BATCH_GUARD(b);
    return brc(b, b->world.download_scene(scene, out));
}

int dem_batch_upload(dem_batch *b, int32_t scene, const dem_scene *in) {
    BATCH_GUARD(b);
    return brc(b, b->world.upload_scene(scene, in));
}

int dem_batch_upload_many(dem_batch *b, int32_t n, const int32_t *idx, const dem_scene *const *in) {
    BATCH_GUARD(b);
    return brc(b, b->world.upload_many(idx, in, n));
}

int dem_batch_download_many(dem_batch *b, int32_t n, const int32_t *idx, dem_scene *const *out) {
    BATCH_GUARD(b);
    return brc(b, b->world.download_many(idx, out, n));
}

int dem_batch_set_params(dem_batch *b, int32_t scene, const dem_params *p) {
    BATCH_GUARD(b);
    if (!p) return bset(b, DEM_E_INVALID, "params is NULL");
    return brc(b, b->world.set_params(scene, *p));
}

int dem_batch_set_properties(dem_batch *b, int32_t scene, int32_t *selections,
                             const int32_t props[DEM_PROPS_WORDS]) {
    BATCH_GUARD(b);
    return brc(b, b->world.set_properties(scene, selections, props));
}

int dem_batch_event(dem_batch *b, int32_t scene, int32_t kind, int32_t *selections, int32_t throw_particles,
                    float del_x, float del_y, int32_t ticks) {
    BATCH_GUARD(b);
    return brc(b, b->world.fixity_event(scene, kind, selections, throw_particles, del_x, del_y, ticks));
}

int dem_batch_get_datum(dem_batch *b, int32_t scene, const int32_t *selections, double out[10]) {
    BATCH_GUARD(b);
    const int rc = b->world.get_datum(scene, selections, out);
    return rc < 0 ? brc(b, rc) : rc;
}

int dem_batch_record(dem_batch *b, int32_t scene, int32_t n_steps, const int32_t *selections, double *rows) {
    BATCH_GUARD(b);
    const int rc = b->world.record(scene, selections, n_steps, rows);
    return rc < 0 ? brc(b, rc) : rc;
}

int dem_batch_break_events(dem_batch *b, dem_break_event *buf, int32_t cap, int32_t *n) {
    BATCH_GUARD(b);
    if (cap < 0 || (cap > 0 && !buf)) return bset(b, DEM_E_INVALID, "bad event buffer");
    std::vector<dem_break_event> ev;
    int rc = b->world.drain_events(ev);
    if (rc) return brc(b, rc);
    int32_t k = (int32_t)std::min<size_t>(ev.size(), (size_t)cap);
    if (k) std::memcpy(buf, ev.data(), sizeof(dem_break_event) * k);
    if (n) *n = k;
    if ((size_t)k < ev.size()) return bset(b, DEM_E_CAPACITY, "event buffer smaller than pending events");
    return DEM_OK;
}

int dem_batch_get_stats(dem_batch *b, dem_stats *out) {
    BATCH_GUARD(b);
    if (!out) return bset(b, DEM_E_INVALID, "out is NULL");
    return brc(b, b->world.stats(out));
}

void *dem_batch_stream(dem_batch *b) { return b ? (void *)b->world.stream : nullptr; }

int dem_batch_kernel_timing(dem_batch *b, int32_t enable) {
    BATCH_GUARD(b);
    b->world.set_timing(enable != 0);
    return DEM_OK;
}

int dem_batch_kernel_time(dem_batch *b, const char *kernel, double *total_ms, int64_t *launches) {
    BATCH_GUARD(b);
    if (!kernel) return bset(b, DEM_E_INVALID, "kernel is NULL");
    static const char *names[6] = {"interact", "lom", "broad_phase", "reorder", "end_step", "candidate_lists"};
    for (int k = 0; k < 6; ++k) {
        if (std::strcmp(kernel, names[k]) == 0) {
            long long n = 0;
            int rc = b->world.kernel_time(k, total_ms, &n);
            if (launches) *launches = n;
            return brc(b, rc);
        }
    }
    return bset(b, DEM_E_INVALID, "unknown kernel name");
}

}  // extern "C"

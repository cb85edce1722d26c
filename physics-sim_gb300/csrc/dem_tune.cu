// dem_tune.cu -- autotuner of the knobs that change speed but not results.
//
// A batch's arithmetic does not depend on the search-cell size, the
// candidate-list skin (which sets how often the particles are re-sorted by
// cell), the block size of the particle kernels, the number of steps per
// captured CUDA graph, whether the Simulation pass runs as one kernel or
// two, or whether it carries the next step's LOM pass; their best values
// depend on the scenes and the GPU.
// dem_batch_autotune times short runs of a sample of the batch's scenes with
// candidate values, one knob at a time (coordinate descent from the library
// defaults), and returns the fastest combination as dem_ext fields.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <string>
#include <vector>

#include "dem.h"
#include "dem_world_host.h"

namespace {

thread_local std::string g_tune_error;

int tfail(int code, const std::string &m) {
    g_tune_error = m;
    return code;
}

struct Knobs {
    float cell_factor = 1.0f;
    float skin = 0.2f;
    int block = 256;
    int graph_steps = 35;
    int split = 0;
    int unfused = 0;
};

// ms per step of the sample with the given knobs: warm run (graph capture,
// first rebuild), then `steps` timed steps with events on the world's stream
int trial(const std::vector<const dem_scene *> &sc, const std::vector<dem_params> &ps,
          const std::vector<dem_ext> &base, const Knobs &k, int steps, double *ms_per_step) {
    std::vector<dem_ext> es = base;
    for (auto &e : es) {
        e.search_cell_factor = k.cell_factor;
        e.list_skin = k.skin;
        e.block_size = k.block;
        e.reorder_interval = k.graph_steps;
        e.split_narrow = k.split;
        e.unfused_lom = k.unfused;
        e.plain_launches = 0;
    }
    cudaStream_t st = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
        return tfail(DEM_E_CUDA, "stream creation failed");
    int rc = DEM_OK;
    float ms = 0.0f;
    {
        demgb::World w;
        w.stream = st;
        cudaGetDevice(&w.device);
        rc = w.build(sc, ps, es);
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if (rc == DEM_OK) rc = w.step(steps);
        if (rc == DEM_OK && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess))
            rc = tfail(DEM_E_CUDA, "event creation failed");
        if (rc == DEM_OK) {
            cudaEventRecord(e0, st);
            rc = w.step(steps);
            cudaEventRecord(e1, st);
        }
        if (rc == DEM_OK) rc = w.sync();
        if (rc == DEM_OK && cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
            rc = tfail(DEM_E_CUDA, "event timing failed");
        if (rc != DEM_OK && g_tune_error.empty()) g_tune_error = w.err;
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    }
    cudaStreamDestroy(st);
    if (rc != DEM_OK) return rc;
    *ms_per_step = (double)ms / steps;
    return DEM_OK;
}

}  // namespace

extern "C" {

const char *dem_tune_last_error(void) { return g_tune_error.c_str(); }

int dem_batch_autotune(const dem_scene *const *scenes, const dem_params *params, const dem_ext *exts,
                       int32_t n_scenes, int32_t device, int64_t sample_particles, int32_t trial_steps,
                       dem_tune_result *out) {
    g_tune_error.clear();
    if (!out || !scenes || !params || n_scenes <= 0) return tfail(DEM_E_INVALID, "no scenes or out is NULL");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return tfail(DEM_E_CUDA, "no CUDA device available");
    if (device >= 0 && (device >= ndev || cudaSetDevice(device) != cudaSuccess))
        return tfail(DEM_E_INVALID, "bad device index");
    if (sample_particles <= 0) sample_particles = 2000000;
    if (trial_steps <= 0) trial_steps = 140;
    const auto t_start = std::chrono::steady_clock::now();
    // sample: scenes spread over the size range (every k-th by size) until the
    // particle budget is met, so the sample has the batch's mix of sizes
    std::vector<int> order(n_scenes);
    long long total = 0;
    for (int s = 0; s < n_scenes; ++s) {
        if (!scenes[s]) return tfail(DEM_E_INVALID, "scene pointer is NULL");
        order[s] = s;
        total += scenes[s]->n_particles;
    }
    std::sort(order.begin(), order.end(),
              [&](int a, int b) { return scenes[a]->n_particles < scenes[b]->n_particles; });
    const double frac = total > 0 ? std::min(1.0, (double)sample_particles / (double)total) : 1.0;
    const int stride = std::max(1, (int)(1.0 / std::max(frac, 1e-9)));
    std::vector<const dem_scene *> sc;
    std::vector<dem_params> ps;
    std::vector<dem_ext> es;
    long long taken = 0;
    for (int k = 0; k < n_scenes; k += stride) {
        const int s = order[k];
        sc.push_back(scenes[s]);
        ps.push_back(params[s]);
        dem_ext e;
        if (exts) e = exts[s];
        else dem_ext_defaults(&e);
        es.push_back(e);
        taken += scenes[s]->n_particles;
    }
    // candidate values; cell factors span 1.5 to 3 r_max at the default skin
    const float cells[] = {0.68f, 0.85f, 1.0f, 1.36f};
    const float skins[] = {0.1f, 0.2f, 0.3f, 0.45f};
    const int blocks[] = {128, 256, 512};
    const int graphs[] = {21, 35, 70};
    Knobs best;
    double best_ms = 0.0;
    int trials = 0;
    int rc = trial(sc, ps, es, best, trial_steps, &best_ms);
    if (rc) return rc;
    ++trials;
    const double default_ms = best_ms;
    auto try_knobs = [&](const Knobs &k) -> int {
        double ms = 0.0;
        int r = trial(sc, ps, es, k, trial_steps, &ms);
        if (r) return r;
        ++trials;
        if (ms < best_ms) {
            best_ms = ms;
            best = k;
        }
        return DEM_OK;
    };
    for (float v : skins) {
        if (v == best.skin) continue;
        Knobs k = best;
        k.skin = v;
        if ((rc = try_knobs(k))) return rc;
    }
    for (float v : cells) {
        if (v == best.cell_factor) continue;
        Knobs k = best;
        k.cell_factor = v;
        if ((rc = try_knobs(k))) return rc;
    }
    for (int v : blocks) {
        if (v == best.block) continue;
        Knobs k = best;
        k.block = v;
        if ((rc = try_knobs(k))) return rc;
    }
    for (int v : graphs) {
        if (v == best.graph_steps) continue;
        Knobs k = best;
        k.graph_steps = v;
        if ((rc = try_knobs(k))) return rc;
    }
    {
        Knobs k = best;
        k.split = 1 - best.split;
        if ((rc = try_knobs(k))) return rc;
    }
    {
        Knobs k = best;
        k.unfused = 1 - best.unfused;
        if ((rc = try_knobs(k))) return rc;
    }
    std::memset(out, 0, sizeof *out);
    out->search_cell_factor = best.cell_factor;
    out->list_skin = best.skin;
    out->block_size = best.block;
    out->reorder_interval = best.graph_steps;
    out->split_narrow = best.split;
    out->unfused_lom = best.unfused;
    out->ms_per_step = best_ms;
    out->default_ms_per_step = default_ms;
    out->trials = trials;
    out->sample_scenes = (int32_t)sc.size();
    out->sample_particles = taken;
    out->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    return DEM_OK;
}

}  // extern "C"

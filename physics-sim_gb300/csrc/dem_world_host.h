// dem_world_host.h -- host-side owner of a DevWorld: allocation, scene
// layout (grid geometry, offsets), conversion between the reference's host
// layouts and the internal device layout, and step orchestration.
#pragma once
#include <climits>
#include <cuda_runtime.h>

#include <map>
#include <functional>
#include <string>
#include <vector>

#include "dem.h"
#include "dem_world.cuh"

namespace demgb {

// 2 zeta of the normal dashpot for restitution e (dem_ext.restitution)
float dashpot_factor(float e);

// World limits: the kernels index particles, cells and bonds with 32-bit
// ints, the slot rows as j * N + i (j < K), and a grid-stride loop's index
// must not pass 2^31 on its last stride.
constexpr long long MAX_WORLD_PARTICLES = (long long)INT_MAX / K;  // 153,391,689

struct SceneHost {
    // reference-layout copies of what the step never writes (kept for download;
    // fixity, forces, material pointers and data[7i+3] stay on the device)
    std::vector<float> materials;      // [6m]
    std::vector<int32_t> bond_angle;   // [B] raw bits
    std::vector<float> bond_sn, bond_ss;
    dem_params params;
    dem_grid_info grid;
    int n = 0, n_bonds = 0, n_mat = 0;
    float r_max = 0.0f;                // largest radius the search cells are sized for
    float r_big = 3.0e38f;             // radius above which a particle is large (none: above any radius)
    int n_big = 0;                     // large particles
    int big_cap = 0, big_base = 0;     // big-partner records owned by the scene
    int use_f64 = 0;
    float lambda = 0.5f;
    float damp2 = 0.0f;            // dashpot: 2 zeta (0: off)
    float cell_factor = 1.0f;
    float skin = 0.0f;
    // control words (coll_cont) at step0
    long long step0 = 0;
    int32_t cc0_0 = 0, cc1_0 = 0, cc2_0 = 0;
    bool active = true;
    // layout in the world
    int particle_base = 0, cell_base = 0, n_cells = 0, bond_base = 0, mat_base = 0, pair_base = 0;
    ScenePar par;
};

// First-fit allocator of index ranges [0, capacity) with merging on release.
class RangeAlloc {
  public:
    void reset(long long capacity);
    long long alloc(long long n);  // offset, or -1 when no free range is long enough
    void release(long long off, long long n);
    long long used() const { return used_; }
    long long capacity() const { return cap_; }

  private:
    std::map<long long, long long> free_;  // offset -> length
    long long used_ = 0, cap_ = 0;
};

class World {
  public:
    World() = default;
    ~World();
    World(const World &) = delete;
    World &operator=(const World &) = delete;

    // Lay out the given scenes (host staging), allocate and upload.  Returns DEM_* code.
    int build(const std::vector<const dem_scene *> &scenes, const std::vector<dem_params> &params,
              const std::vector<dem_ext> &exts);
    // Replace one scene's state in place (same particle/bond/material counts).
    int upload_scene(int s, const dem_scene *scene);
    int download_scene(int s, dem_scene *out);
    int upload_many(const int32_t *idx, const dem_scene *const *scenes, int count);
    int download_many(const int32_t *idx, dem_scene *const *outs, int count);
    int set_params(int s, const dem_params &p);
    int set_materials(int s, const float *m, int n);
    int set_properties(int s, int32_t *selections, const int32_t *props);
    int fixity_event(int s, int kind, int32_t *selections, int throw_vel, float del_x, float del_y, int ticks);
    int get_datum(int s, const int32_t *selections, double out[10]);
    int record(int s, const int32_t *selections, int n_steps, double *rows);
    int step(int n_steps);
    int sync();
    int drain_events(std::vector<dem_break_event> &out);
    int stats(dem_stats *out);
    int push_active(int s, bool on, long long steps);
    int broad_phase_snapshot(int s, int32_t *keys, int32_t *order, int32_t *cell_start, int32_t *n_cells);
    void control(int s, int32_t cc[4]) const;
    int set_control(int s, const int32_t cc[4]);

    // capacity mode (served scenes): arenas allocated once, scenes admitted
    // into free ranges and retired from them
    int build_capacity(long long particles, long long cells, long long bonds, int scenes, int materials,
                       const dem_ext &ext);
    // admit a scene that will run `horizon` steps; returns its slot or a negative DEM_E_* code
    int admit(const dem_scene *scene, const dem_params &params, const dem_ext &ext, long long horizon);
    int retire(int slot);
    int free_slot = -1;                 // scene index of unused particles (never active)
    RangeAlloc a_part, a_cell, a_bond, a_mat, a_pair, a_big;
    std::vector<int> free_slots;
    long long bytes_per_particle() const;

    std::string err;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;   // captures the rebuild body of a conditional node
    int device = 0;
    int block = 256;
    int graph_steps = 35;          // steps per captured CUDA graph
    float skin_factor = 0.2f;      // candidate-list skin / r_max
    int reorder_every = 0;         // rebuilds per reorder into cell order (0: by world, see alloc)
    bool diagnostics = true;
    long long host_step = 0;
    std::vector<SceneHost> sh;
    DevWorld d{};
    bool use_graphs = true;
    bool split_narrow = false;     // Simulation pass as two kernels (dem_ext::split_narrow)
    bool fuse_lom = true;          // next step's LOM pass inside the Simulation kernel (dem_ext::unfused_lom)
    bool has_bigs = false;         // some scene has large particles: k_big_narrow runs each step
    long long launches = 0;
    // kernel timing (debug): event pairs per kernel kind, summed on demand
    bool timing = false;
    struct Timer {
        std::vector<cudaEvent_t> ev;  // start/stop pairs
        double ms = 0.0;
        long long n = 0;
    };
    static constexpr int N_TIMERS = 6;
    Timer timers[N_TIMERS];
    void rec_event(int kind, cudaStream_t st);
    int kernel_time(int kind, double *ms, long long *n);
    void set_timing(bool on);

  private:
    int fail(int code, const std::string &msg);
    int alloc(int N, int C, int B, int S, int M, int MP, int TB, uint32_t ev_cap);
    int push_bigs(int s, int scene_or_free);
    void update_has_bigs();
    int push_materials(int s);
    void release();
    int compute_layout(SceneHost &h, const dem_scene *scene);
    void fill_par(SceneHost &h);
    int push_par(int s);
    int push_det();
    int layout_threads = 1;  // host threads compute_layout may use on a large scene
    int kernel_form = -1;     // Simulation kernels' form (launch_interact): -1 carries everything
    void update_kernel_form();
    uint8_t *live_d = nullptr;  // served worlds: the live map of 128-particle chunks (DevWorld::live)
    int update_live();
    int stage_many(const int32_t *idx, const dem_scene *const *scs, int count, const SceneHost *probes,
                   const std::function<int()> &layouts);
    int force_rebuild(bool reorder = true);
    void enqueue_plain_step(bool first, bool last, bool next_last);
    void enqueue_rebuild(cudaStream_t st, const int32_t *gate, bool every_step);
    int capture_graph(int R, cudaGraphExec_t *out, int *kernels);
    void drop_graph();
    bool dense_cells() const;
    DevWorld spare{};
    std::vector<void *> owned;
    // device copy of one scene in the reference layouts (uploads, downloads)
    RefArrays ref{};
    void *ref_block = nullptr;
    long long ref_cap = 0;
    int ensure_ref(long long n);
    void *pin = nullptr;               // page-locked staging of the bulk transfers
    size_t pin_bytes = 0;
    int ensure_pin(size_t bytes);
    // the item table of a staging transfer, one check word per item (plus
    // their OR), and the table of its direct copies
    StageItem *d_items = nullptr;
    int32_t *d_item_err = nullptr;
    int items_cap = 0;
    HostCopy *d_copies = nullptr;
    int copies_cap = 0;
    int ensure_tables(int items, int copies);
    bool host_direct = false;  // the device reads and writes the callers' arrays (dem_ext::host_copies)
    std::vector<cudaEvent_t> xfer_ev;  // one per chunk of a pipelined download
    int ensure_events(int count);
    int stage_error(int32_t e);
    int layout_fits(int s, const SceneHost &probe);
    void apply_layout(int s, const SceneHost &probe);
    int unstage_error(int32_t e);
    // captured graphs, one per buffer parity at their start (a graph of R
    // steps swaps the pr/dp/rr buffers R - 1 times)
    cudaGraphExec_t graph[2] = {nullptr, nullptr};   // graph_steps steps
    cudaGraphExec_t graph1[2] = {nullptr, nullptr};  // one step, for remainders
    int graph_R[2] = {0, 0};
    int graph_kernels[2] = {0, 0};
    int graph1_kernels[2] = {0, 0};
    // Where the Simulation kernels read the scene parameters (launch_interact,
    // PS_*): a world of one scene passes them with each launch, a world whose
    // scenes share their settings passes those.  step() sets both before any
    // launch; graphs keep the values they were captured with, so step()
    // captures anew when these change.
    int par_ps = PS_SCENE;
    ScenePar par_pv{};
    void update_param_source();
    int graph_ps = -1;
    ScenePar graph_par{};
    int parity = 0;                    // which pr/dp/rr buffers are current
    void flip();
    int rebuild_kernels = 0;
};

}  // namespace demgb

/*
 * dem.h -- C ABI of libdemgb.so, the GB300-native per-step DEM pipeline.
 *
 * Drop-in for the compute side of gusjengis/Physics-Sim's WGPUComputeProg
 * (src/wgpu_prog.rs): the scene travels in the reference's host layouts
 * (src/state.rs:69-93), the settings in the 29-word uniform of
 * Settings::collision_settings (src/settings.rs:2086-2119), and one call of
 * dem_step(ctx, n) advances n steps of LOM + Simulation exactly like
 * WGPUComputeProg::compute with gen_per_frame = n (src/wgpu_prog.rs:1420-1473).
 *
 * Conventions: plain pointers and sizes; the caller owns host memory, the
 * library owns device memory; every call returns 0 or a negative DEM_E_* code
 * and never aborts; dem_last_error() describes the last failure.  A context is
 * used by one host thread at a time.
 */
#ifndef DEM_H
#define DEM_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DEM_ABI_VERSION 1
#define DEM_MAX_CONTACTS 14   /* settings.setup.max_contacts = max_bonds + 8 (settings.rs:263, 310) */
#define DEM_DATA_SIZE 7       /* DATA_SIZE (state.rs:67) */
#define DEM_PROPS_WORDS 28    /* Settings::properties (settings.rs:2158-2189) */

enum {
    DEM_OK = 0,
    DEM_E_INVALID = -1,      /* bad argument or inconsistent scene */
    DEM_E_OOM = -2,          /* device or host allocation failed */
    DEM_E_CUDA = -3,         /* CUDA runtime error */
    DEM_E_TIMEOUT = -4,      /* a bounded device wait gave up */
    DEM_E_STATE = -5,        /* device reported an inconsistent state */
    DEM_E_UNSUPPORTED = -6,  /* feature not available */
    DEM_E_CAPACITY = -7      /* a bounded buffer overflowed (see dem_last_error) */
};

/* The Settings uniform, 29 words in the order of collision_settings()
 * (settings.rs:2086-2119) and of `struct Settings` in 2D_LOM.wgsl:26-56 /
 * 2D_Simulation.wgsl:34-64.  Binary-identical to that Vec<f32>. */
typedef struct dem_params {
    int32_t walls;
    float hor_bound;
    float vert_bound;
    int32_t round_bounds;
    float bound_radius;
    float wall_friction;
    int32_t gravity;
    int32_t planet_mode;
    int32_t bonds;
    int32_t collisions;
    float friction_coefficient;
    float gravity_acc;
    float bond_normal_stiffness;
    int32_t bonds_tear;
    float bond_normal_strength;
    float contact_damping;
    float bond_damping;
    float drag;
    float bond_shear_strength;
    float dT;
    float bond_shear_stiffness;
    float gravity_x;
    float gravity_y;
    int32_t mouse_gravity;
    float moment_contribution_factor;
    int32_t collision_interval;
    int32_t local_damping;
    float local_damping_alpha;
    int32_t particles;
} dem_params;

/* GridInfo as uploaded to grid_info_buffer (wgpu_prog.rs:653-675); computed by
 * grid_capacity (wgpu_prog.rs:698-717) or dem_grid_capacity() below. */
typedef struct dem_grid_info {
    float cell_size;
    int32_t cell_cap;
    int32_t w;
    int32_t h;
} dem_grid_info;

/* Extensions.  Zero-initialise, then set bond_lambda = 0.5f and
 * diagnostics = 1 for exact reference behaviour (dem_ext_defaults). */
typedef struct dem_ext {
    int32_t use_f64;                  /* F64 distance branch (2D_Simulation.wgsl:264-284; shader_gen.rs:84) */
    float bond_lambda;                /* parallel-bond radius factor; reference 0.5 (2D_Simulation.wgsl:290) */
    const float *bond_normal_strength;/* optional per-bond strengths [n_bonds]; NULL = global setting */
    const float *bond_shear_strength;
    int32_t diagnostics;              /* 1: maintain data[7n] every step as the reference does */
    int32_t reorder_interval;         /* steps per captured CUDA graph; 0 = library default (35) */
    int32_t block_size;               /* threads per block for particle kernels; 0 = default */
    float search_cell_factor;         /* search-grid cell / (2 r_max + skin), in [0.5, inf); 0 = default
                                         1.0.  Below 1 the cell searches span 5 x 5 cells instead of
                                         3 x 3; results do not depend on it */
    int32_t event_capacity;           /* break-event ring size; 0 = default */
    float list_skin;                  /* candidate-list skin / r_max; 0 = default 0.2.  Lists are rebuilt
                                         when a particle moves beyond half the skin; results do not
                                         depend on it */
    int32_t plain_launches;           /* 1: no CUDA graphs (for profilers that cannot see kernels inside
                                         graphs with conditional nodes, and for hosts that capture the
                                         calls into graphs of their own); results do not depend on it */
    int32_t split_narrow;             /* 1: narrow phase and forces as two kernels (fewer registers
                                         each; faster in dense scenes); results do not depend on it */
    int32_t unfused_lom;              /* 1: every step runs its own LOM kernel instead of the next
                                         step's LOM pass running inside the Simulation kernel (the
                                         default, fewer bytes per step); results do not depend on it */
    int32_t host_copies;              /* 0: transfers read and write the caller's arrays directly from the
                                         device where it reaches pageable host memory through the host's
                                         page tables (Grace), else through a page-locked block; 1: always
                                         through the page-locked block */
    int32_t reorder_every;            /* rebuilds per reorder of the particle arrays into cell order; 0 =
                                         default: 3 in a single-scene context, 8 in batches and servers.
                                         Every rebuild sorts by cell and rebuilds the candidate
                                         lists; the reorder only restores memory locality, which particles
                                         lose slowly (they move a skin between rebuilds, a cell takes
                                         many); results do not depend on it */
    float restitution;                /* particle-particle normal dashpot (an extension: the reference's
                                         contacts are springs only; its one restitution is the walls' 0.5,
                                         2D_LOM.wgsl:110-126).  0 = off, the reference's arithmetic; e in
                                         (0, 1]: linear_model's normal force gains -c v_n with damping
                                         ratio zeta = -ln e / sqrt(pi^2 + ln^2 e), c = 2 zeta sqrt(k_n
                                         m_eff), v_n the normal approach speed of the step's displacements,
                                         and the sum is kept >= 0 (no pull between touching disks) */
} dem_ext;

/* One scene in the reference's host layouts (state.rs:69-93).  Arrays hold
 * n_particles entries (times the per-particle width). */
typedef struct dem_scene {
    int32_t n_particles;       /* p_count */
    int32_t n_bonds;           /* bond records (bonds holds 3*n_bonds words) */
    int32_t n_materials;       /* material records (materials holds 6*n_materials floats) */
    float *pos;                /* [2n] */
    float *radii;              /* [n] */
    float *vel;                /* [2n] */
    float *acc;                /* [2n]  binding 1 of group 1, "accelerations" */
    float *rot;                /* [n] */
    float *rot_vel;            /* [n] */
    float *rot_acc;            /* [n] */
    float *forces;             /* [6n]  {x, y, rot, delX, delY, delRot} */
    int32_t *fixity;           /* [6n]  {x_vel, y_vel, rot_vel, x_vel_2, y_vel_2, rot_vel_2} */
    float *del_pos;            /* [2n] */
    float *del_rot;            /* [n] */
    int32_t *bonds;            /* [3*n_bonds] {index, angle bits, length bits} */
    int32_t *contacts;         /* [6*14*n] {a, b, tangent_force, bond_tangent_force, theta_b, bonded} bits */
    int32_t *material_pointers;/* [n] */
    float *materials;          /* [6*n_materials] {red, green, blue, density, normal_stiffness, shear_stiffness} */
    float *data;               /* [7n] or NULL */
    int32_t coll_cont[4];      /* {detect flag, interval counter, tick, positions-set flag} */
    dem_grid_info grid;
} dem_scene;

/* One bond break, in evaluation order of the step that produced it. */
typedef struct dem_break_event {
    int32_t scene;   /* scene index within a batch (0 for a single-scene context) */
    int32_t step;    /* step counter value of the step that broke the bond */
    int32_t bond;    /* bond record index within the scene */
    int32_t code;    /* -10 + sign(normal displacement) (2D_Simulation.wgsl:323, 403, 426) */
    int32_t a;       /* particle evaluating the break */
    int32_t b;       /* its partner */
} dem_break_event;

typedef struct dem_stats {
    int64_t steps;              /* steps executed */
    int64_t capped;             /* narrow phases that reached 14 contacts */
    int64_t events;             /* bond breaks recorded */
    int64_t events_dropped;     /* breaks beyond the event ring */
    int64_t reorders;           /* rebuilds (cell sort, reorder by cell, candidate lists) */
    int32_t device_error;       /* sticky device error bits, 0 = none: 1 breaks of one step beyond the
                                   pending-break capacity; 2 a touching pair whose first shared bucket
                                   ranks beyond 15 in the scan order, or an AABB 31 or more buckets
                                   wide (the bucket grid is much finer than the particles); 4 a large
                                   particle touching more than 2048 particles at once */
    int32_t reserved;
    int64_t kernel_launches;    /* kernels this library launched on the context's stream */
    int64_t list_overflows;     /* particles whose candidates exceeded the list (searched the cells) */
} dem_stats;

typedef struct dem_ctx dem_ctx;

int dem_abi_version(void);
void dem_ext_defaults(dem_ext *ext);
/* Last error message of ctx, or of the calling thread's last failed create when ctx is NULL. */
const char *dem_last_error(const dem_ctx *ctx);

/* grid_capacity (wgpu_prog.rs:698-717) over the given radii (State::load
 * takes min/max over the whole radii vector, state.rs:684-698). */
int dem_grid_capacity(const dem_params *p, const float *radii, int32_t n_radii, int32_t particles,
                      dem_grid_info *out);

/* WGPUComputeProg::new + restore: copy a scene to the device.  device < 0
 * keeps the current CUDA device.  A context, batch or server holds at most
 * 153,391,689 particles (14 slot rows of 32-bit indices), 2^30 search cells
 * and 2^30 bonds (DEM_E_INVALID beyond; a server sizes its arenas within). */
int dem_create(const dem_scene *scene, const dem_params *params, const dem_ext *ext, int device,
               dem_ctx **out);
void dem_destroy(dem_ctx *ctx);

/* WGPUComputeProg::restore (wgpu_prog.rs:1235-1262): replace the whole state.
 * The control words coll_cont persist across restore, as the device buffer does
 * in the reference; scene->coll_cont is ignored here (see dem_set_control). */
int dem_upload(dem_ctx *ctx, const dem_scene *scene);
/* Uniform::updateUniform of the settings (client.rs:1128-1135). */
int dem_set_params(dem_ctx *ctx, const dem_params *params);
/* Material buffer update (6 floats per material). */
int dem_set_materials(dem_ctx *ctx, const float *materials, int32_t n_materials);
int dem_set_control(dem_ctx *ctx, const int32_t coll_cont[4]);
int dem_get_control(dem_ctx *ctx, int32_t coll_cont[4]);

/* WGPUComputeProg::compute: enqueue n_steps of LOM + Simulation on the
 * context's stream and return without waiting, like queue.submit. */
int dem_step(dem_ctx *ctx, int32_t n_steps);
int dem_synchronize(dem_ctx *ctx);

/* State::update_state (state.rs:264-289): synchronous copy of the whole state
 * into caller-owned arrays of `out` (NULL arrays are skipped). */
int dem_download(dem_ctx *ctx, dem_scene *out);

/* Set_Properties event (Set_Properties.wgsl:68-90): props are the 28 words of
 * Settings::properties; selections [n] is read, and written back with 2 where
 * a fixity was set (Set_Properties.wgsl:87-89). */
int dem_set_properties(dem_ctx *ctx, int32_t *selections, const int32_t props[DEM_PROPS_WORDS]);

/* Drain up to cap break events (oldest first); *n receives the count copied. */
int dem_break_events(dem_ctx *ctx, dem_break_event *buf, int32_t cap, int32_t *n);
int dem_get_stats(dem_ctx *ctx, dem_stats *out);

/* The CUDA stream the context enqueues on (a cudaStream_t), for callers that
 * order their own work against the steps. */
void *dem_stream(dem_ctx *ctx);

/* Fix, Drop and Release events (src/shaders/event_handling/Fix.wgsl,
 * Drop.wgsl, Release.wgsl) applied to the particles marked in selections[n]
 * (the reference's State::selections; Fix and Drop rewrite the marks as the
 * shaders do).  Release with throw_particles != 0 also sets the velocity to
 * (del_x, del_y) / (dT * ticks), the shader's click_info[0] == 1 branch. */
#define DEM_EVENT_FIX 1
#define DEM_EVENT_DROP 2
#define DEM_EVENT_RELEASE 3
int dem_event(dem_ctx *ctx, int32_t kind, int32_t *selections, int32_t throw_particles, float del_x, float del_y,
              int32_t ticks);

/* State::get_datum (src/state.rs:708-737) on the device state: out[10] =
 * means over the selected particles of pos.x, pos.y, data[4], data[5], rot,
 * data[6], data[1], data[2], data[3], except out[6] = sum of |data[0]|, in the
 * reference's order (double accumulation in index order).  Only the selected
 * particles' fields are read back.  Returns the number selected (0: the
 * reference's None, out untouched) or a negative DEM_E_* code. */
int dem_get_datum(dem_ctx *ctx, const int32_t *selections, double out[10]);

/* Advance with Record on (client.rs:931-974, gather_data): n_steps steps,
 * each followed by dem_get_datum of the selected particles, without a state
 * readback per step: the data are gathered on the device and read back in
 * one copy.  rows[10 * n_steps] receives one datum row per step (the columns
 * of dem_get_datum; the reference's CSV adds the timestamp dT * generation
 * and its FPS, settings.rs:2014-2052).  Returns the number of selected
 * particles (0: the steps run and rows is untouched, the reference's None)
 * or a negative DEM_E_* code.  The reference's Advance runs one more step
 * after the recorded ones; call dem_step(ctx, 1) for it. */
int dem_record(dem_ctx *ctx, int32_t n_steps, const int32_t *selections, double *rows);

/* ---- Batches: many independent scenes stepped together ------------------
 * No counterpart in the reference (one scene per program there).  A batch
 * holds n_scenes scenes resident on one GPU; dem_batch_step advances every
 * scene by n_steps with the same launches, each scene with its own settings,
 * materials, bonds and extensions (exts may be NULL for defaults; world-wide
 * options such as block_size are taken from exts[0]).  Per-scene results are
 * exactly those of a single-scene context on the same scene. */
typedef struct dem_batch dem_batch;
int dem_batch_create(const dem_scene *const *scenes, const dem_params *params, const dem_ext *exts,
                     int32_t n_scenes, int device, dem_batch **out);
void dem_batch_destroy(dem_batch *b);
const char *dem_batch_last_error(const dem_batch *b);
int dem_batch_scene_count(const dem_batch *b);
int dem_batch_step(dem_batch *b, int32_t n_steps);
int dem_batch_synchronize(dem_batch *b);
int dem_batch_download(dem_batch *b, int32_t scene, dem_scene *out);
int dem_batch_upload(dem_batch *b, int32_t scene, const dem_scene *in);
/* The same for n scenes at once (scene indices idx[n]): a few large
 * transfers, one conversion launch and one check for all of them, with host
 * threads copying the callers' arrays through a page-locked block that the
 * batch keeps (its size: 468 bytes a particle of the largest transfer, plus
 * the world's bond, material and per-particle reference words).
 * upload_many writes nothing unless every scene passes its checks, and a
 * scene may appear in idx only once; download_many writes no caller's array
 * unless every scene's conversion passed. */
int dem_batch_upload_many(dem_batch *b, int32_t n, const int32_t *idx, const dem_scene *const *in);
int dem_batch_download_many(dem_batch *b, int32_t n, const int32_t *idx, dem_scene *const *out);
int dem_batch_set_params(dem_batch *b, int32_t scene, const dem_params *params);
int dem_batch_set_properties(dem_batch *b, int32_t scene, int32_t *selections,
                             const int32_t props[DEM_PROPS_WORDS]);
int dem_batch_break_events(dem_batch *b, dem_break_event *buf, int32_t cap, int32_t *n);
int dem_batch_event(dem_batch *b, int32_t scene, int32_t kind, int32_t *selections, int32_t throw_particles,
                    float del_x, float del_y, int32_t ticks);
int dem_batch_get_datum(dem_batch *b, int32_t scene, const int32_t *selections, double out[10]);
/* dem_record for one scene of a batch; every scene of the batch steps. */
int dem_batch_record(dem_batch *b, int32_t scene, int32_t n_steps, const int32_t *selections, double *rows);
int dem_batch_get_stats(dem_batch *b, dem_stats *out);
void *dem_batch_stream(dem_batch *b);

/* ---- Autotuning: knobs that change speed, never results ----------------
 * No counterpart in the reference.  dem_batch_autotune builds trial batches
 * from a sample of the given scenes (about sample_particles particles, spread
 * over the size range; <= 0: 2,000,000), times trial_steps steps of each
 * (<= 0: 140) after an equal warm-up, and picks, one knob at a time from the
 * library defaults, the search-cell factor (0.68, 0.85, 1, 1.36 x (2 r_max +
 * skin), i.e. about 1.5 to 3 r_max), the candidate-list skin (0.1, 0.2, 0.3,
 * 0.45 r_max: how often particles are re-sorted by cell), the particle-kernel
 * block size (128, 256, 512), the steps per captured graph (21, 35, 70),
 * whether the Simulation pass runs as one kernel or two (split_narrow) and
 * whether it carries the next step's LOM pass (unfused_lom).
 * Copy the result's six fields into each scene's dem_ext. */
typedef struct dem_tune_result {
    float search_cell_factor;
    float list_skin;
    int32_t block_size;
    int32_t reorder_interval;         /* steps per captured graph */
    double ms_per_step;               /* sample, chosen values */
    double default_ms_per_step;       /* sample, library defaults */
    int32_t trials;
    int32_t sample_scenes;
    int64_t sample_particles;
    double seconds;                   /* wall time of the tuning */
    int32_t split_narrow;
    int32_t unfused_lom;
    int32_t reserved[6];
} dem_tune_result;
int dem_batch_autotune(const dem_scene *const *scenes, const dem_params *params, const dem_ext *exts,
                       int32_t n_scenes, int32_t device, int64_t sample_particles, int32_t trial_steps,
                       dem_tune_result *out);
const char *dem_tune_last_error(void);

/* ---- Bond generation: State::regen_bonds (src/state.rs:291-367) on the GPU
 * Bonds every pair closer than 1.05 (r_i + r_j), at most max_bonds per
 * particle on its own side (pairs taken in the reference's order), numbered
 * in the reference's creation order, each taking the first free contact slot
 * of both particles.  pos[2n] and radii[n] are host arrays; writes
 * bonds[3 * nb] {status 1, angle bits, length bits} (nb <= bonds_cap, else
 * DEM_E_CAPACITY with *n_bonds = nb so the caller can size the array) and
 * contacts[84 n] exactly as regen_bonds does.  max_bonds in [1, 14]; n at
 * most 2^26 (DEM_E_CAPACITY beyond). */
int dem_generate_bonds(const float *pos, const float *radii, int32_t n, int32_t max_bonds, int32_t device,
                       int32_t *bonds, int64_t bonds_cap, int64_t *n_bonds, int32_t *contacts);
const char *dem_bondgen_last_error(void);

/* ---- Serving: continuous batching of scene requests --------------------
 * No counterpart in the reference.  A server owns device arenas sized once
 * from memory_budget_bytes (and at most ~1.25 x max_active_particles
 * particles when that is > 0; 0 leaves the budget alone to size them),
 * cells_per_particle cells and bonds_per_particle bonds per particle.
 * Requests (scene + settings + extensions + horizon in steps) are copied at
 * submit (or borrowed, dem_server_submit_borrowed) and queue on the host.  dem_server_advance(sv, n): (1) the
 * scenes that reached their horizon are copied back to host memory and their
 * device ranges freed; (2) queued requests are admitted first come first
 * served while their particles, cells and bonds fit in free ranges and the
 * running particles stay within max_active_particles; (3) every admitted
 * scene advances n steps in the same launches.  A scene stops exactly at its
 * horizon even inside n, so each result equals the scene run alone for that
 * many steps.  dem_server_poll lists completed ids; dem_server_fetch copies a
 * result and its submit/admit/done times (seconds, monotonic clock). */
typedef struct dem_server dem_server;
typedef struct dem_server_config {
    int64_t memory_budget_bytes;   /* device memory the arenas may use (default 150 GiB) */
    int64_t max_active_particles;  /* admission limit on running particles (default 16 Mi) */
    int32_t max_scenes;            /* concurrent scene slots (default 4096) */
    float cells_per_particle;      /* search cells reserved per particle (default 4) */
    float bonds_per_particle;      /* bond records reserved per particle (default 1) */
    int32_t reserved;
    dem_ext ext;                   /* world-wide options (graph steps, skin, block size) */
} dem_server_config;
typedef struct dem_server_stats {
    int64_t queued, running, completed;
    int64_t active_particles;      /* particles of running scenes */
    int64_t particle_steps;        /* particle-steps executed so far */
    int64_t capacity_particles, used_particles, device_bytes;
    int64_t steps;                 /* steps of the shared world so far */
    /* advances at which the queue's head waited: for running particles to
     * drop below max_active_particles, or for free device ranges (the arenas
     * the memory budget paid for) */
    int64_t waits_active, waits_memory;
} dem_server_stats;
void dem_server_config_defaults(dem_server_config *cfg);
int dem_server_create(const dem_server_config *cfg, int device, dem_server **out);
void dem_server_destroy(dem_server *sv);
const char *dem_server_last_error(const dem_server *sv);
int dem_server_submit(dem_server *sv, const dem_scene *scene, const dem_params *params, const dem_ext *ext,
                      int64_t horizon_steps, int64_t *request_id);
/* dem_server_submit without the copy: the request refers to the caller's
 * scene arrays (and bond strengths are still copied), which must stay valid
 * and unchanged until dem_server_poll reports the request, it is cancelled,
 * or the server is destroyed.  For callers that keep their scenes resident
 * -- a pool of prepared scenes, inputs mapped from files -- and may queue
 * many requests: a queued request then holds no host copy of its scene. */
int dem_server_submit_borrowed(dem_server *sv, const dem_scene *scene, const dem_params *params,
                               const dem_ext *ext, int64_t horizon_steps, int64_t *request_id);
int dem_server_advance(dem_server *sv, int32_t n_steps);
int dem_server_poll(dem_server *sv, int64_t *done_ids, int32_t cap, int32_t *n);
int dem_server_fetch(dem_server *sv, int64_t id, dem_scene *out, double times[3]);
int dem_server_events(dem_server *sv, int64_t id, dem_break_event *buf, int32_t cap, int32_t *n);
int dem_server_release(dem_server *sv, int64_t id);
/* Withdraws a request in any state: a queued one leaves the queue, a running
 * one stops and its device ranges are freed, a finished one is released.
 * Its id is unknown afterwards.  A request with more particles than the
 * particle arena is refused at submit (DEM_E_CAPACITY); one that cannot be
 * admitted even into empty arenas (cells, bonds, materials, large-particle
 * records) is failed: poll lists it and fetch returns the admission error. */
int dem_server_cancel(dem_server *sv, int64_t id);
int dem_server_get_stats(dem_server *sv, dem_server_stats *out);
void *dem_server_stream(dem_server *sv);

/* Broad phase that allocates nothing.  No counterpart in the reference: it is
 * for callers that cannot call cudaMalloc (a framework whose pool owns the
 * device heap, an allocator that forbids it, a real-time loop that must not
 * block on it) and so pass only buffers they own.  Inputs: d_pos_radius, n
 * device float4 {x, y, radius, unused} (16-byte aligned); the search grid
 * (cell of a position = floor((x - x0) * inv_cell), floor((y - y0) * inv_cell)
 * clamped to gw x gh; key = cy * gw + cx; zero-radius particles get key
 * gw * gh).  Outputs (device): d_keys [n], d_order [n] (particle indices in
 * stable cell order: by key, then by index, built by a counting sort whose
 * cost does not depend on how many particles share a cell), d_cell_start
 * [gw * gh + 2].  d_keys also serves as the sort's second buffer and holds
 * the keys only once the work has run.  Unlike the context's broad phase
 * (dem_debug_broad_phase), which puts a scene's large particles in the last
 * cell ahead of its zero-radius ones, every particle with a radius is keyed
 * here by its position, and the last cell holds the zero-radius particles
 * only.  Work is enqueued on `stream` (a cudaStream_t, NULL = default stream)
 * and not waited for.  n is at most 2^30 (DEM_E_CAPACITY beyond).
 * Scratch is a fixed device array inside the library, held by every GPU that
 * loads it until exit: at most DEM_NOALLOC_MAX_CELLS cells (gw * gh + 1),
 * larger grids are rejected with DEM_E_CAPACITY.  All calls share that array
 * and it keeps the last call's contents (each call clears what must start at
 * zero), so calls that overlap on the GPU -- on different streams, or from
 * different threads on one device -- race and must be serialised by the
 * caller.  The first call on a device looks up the array's device address;
 * make it before any stream capture.  Errors: dem_noalloc_last_error(). */
#define DEM_NOALLOC_MAX_CELLS 262144
int dem_broad_phase_noalloc(const float *d_pos_radius, int32_t n, float x0, float y0, float inv_cell,
                            int32_t gw, int32_t gh, int32_t *d_keys, int32_t *d_order,
                            int32_t *d_cell_start, void *stream);
const char *dem_noalloc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif

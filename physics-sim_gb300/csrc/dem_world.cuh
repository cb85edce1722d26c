// dem_world.cuh -- device-resident state of one or more DEM scenes ("world").
//
// A world holds S independent scenes back to back in HBM.  Every particle
// array is in *internal* order: the order of the last reorder by search cell,
// which keeps neighbours close in memory.  orig[i] maps an internal index to
// the scene-local index the reference uses (src/state.rs:69-93).
//
// Per-particle hot state is packed in float4 records so each load is one
// 16-byte transaction:
//   pr  {pos.x, pos.y, radius, range}   range: the AABB's reference-bucket
//       range as a 32-bit code (written by the LOM pass; see range_code)
//   vw  {vel.x, vel.y, rot_vel, rot}
//   ac  {acc.x, acc.y, rot_acc, -}          ("accelerations" / rot_acc bindings)
//   dp  {del_pos.x, del_pos.y, del_rot, -}
//   fx  {forces.x, forces.y, forces.rot, -} (external forces, read when M_FEXT)
//   d4  {v_half.x, v_half.y, w_half, -}     data[4..6] written by the LOM pass
//   dF  {sum Fn, sum Ft, sum M, -}          data[0..2] written by the Simulation pass
// Contact slots are SoA [14][N] (slot j of particle i at j*N+i).  The slot
// word smask[i] holds the occupancy of the 14 slots in bits 0-13, so empty
// slots are never read, and in bits 16-29 whether each slot's `bonded` field
// is >= 0 (kept for empty slots too, whose stale field a new contact
// inherits), so unbonded slots never read `bonded`.  Bit 14 (NL_LIVE) is set
// while the particle's candidate list holds a candidate or a flag, so
// particles with an empty list skip reading it.  Bit 31 (DF_ZERO) records
// that dF is all +0, so particles without contacts skip rewriting it.
#pragma once
#include <cuda_runtime.h>
#include <cstring>
#include <stdint.h>

#include "dem.h"

namespace demgb {

constexpr int K = DEM_MAX_CONTACTS;
constexpr int BSHIFT = 16;  // first bonded-field bit of the slot word
constexpr uint32_t DF_ZERO = 1u << 31;  // slot-word bit: dF holds +0, +0, +0
constexpr uint32_t NL_LIVE = 1u << 14;  // slot-word bit: the candidate list is not empty

// meta word: fixity predicates, external-force flag, material, scene
enum : uint32_t {
    M_KICK_X = 1u << 0,  // fixity.x_vel == 0  (2D_LOM.wgsl:88, 2D_Simulation.wgsl:471)
    M_KICK_Y = 1u << 1,
    M_KICK_R = 1u << 2,
    M_FIX_X = 1u << 3,   // fixity.x_vel == 1  (walls skip the DOF, 2D_LOM.wgsl:108, 119)
    M_FIX_Y = 1u << 4,
    M_FIX_R = 1u << 5,
    M_FEXT = 1u << 6,    // external force record is not all zero
    M_BIG = 1u << 7,     // large particle: kept out of the search cells (see ScenePar::big_cell)
};
__host__ __device__ inline uint32_t meta_mat(uint32_t m) { return (m >> 8) & 0xFFu; }
__host__ __device__ inline uint32_t meta_scene(uint32_t m) { return m >> 16; }
constexpr int MAX_SCENES = 65536;
constexpr int MAX_MATERIALS = 256;

struct Mat {
    float density, kn, ks, pad;
};

struct ScenePar {
    dem_params p;          // the 29-word uniform
    float xW, yH;          // hor_bound / 2, vert_bound / 2 (2D_LOM.wgsl:105-106)
    // reference bucket grid: defines which pairs are candidates and in which order
    float ref_cs, ref_base_x, ref_base_y;
    int32_t ref_w, ref_h;
    // search grid (centre-binned, complete for every pair the reference grid can find)
    float g_x0, g_y0, g_inv, g_cs;
    int32_t g_w, g_h;
    int32_t cell_base;     // first search cell of the scene in the global cell arrays
    int32_t dead_cell;     // global cell of zero-radius particles (never searched)
    int32_t stencil;       // search reach in cells
    int32_t particle_base; // first internal index of the scene (scenes are contiguous)
    int32_t n_particles;
    int32_t bond_base;     // first bond record of the scene
    int32_t mat_base;      // first material of the scene
    int32_t n_mat;
    int32_t use_f64;
    float lambda;
    int32_t has_strength;
    int32_t active;        // host bookkeeping; the kernels read DevWorld::act
    int64_t step0;         // world step at which the scene's interval counter was cc1_0
    int32_t cc1_0;
    int32_t pair_base;     // first entry of the scene's material-pair table
    float kb2, ksb2;       // 1/(1/k + 1/k) of the bond stiffnesses (2D_Simulation.wgsl:378-379)
    float skin;            // candidate-list skin: lists hold pairs within ra + rb + skin
    float disp_limit2;     // (skin/2)^2 shrunk by a rounding margin: a move beyond it forces a rebuild
    // Large particles (radius above 4x the scene's median, few of them) would
    // inflate the search cells for everyone.  They are binned into their own
    // cell, big_cell, which the cell searches never visit: after a rebuild they
    // sit at internal indices [big_begin, big_begin + count) of the scene (in
    // scene-local index order), each small particle's list records whether
    // any of them was within reach, and k_big_narrow gives each its accepted
    // partners with one thread block.
    int32_t big_cell;      // global cell of the scene's large particles
    int32_t big_base;      // first big-partner record of the scene
    int32_t n_big;         // large particles of the scene at the last layout
    float r_grid;          // largest radius the search cells are sized for
    float damp2;           // normal dashpot: 2 zeta (0: off; dem_ext.restitution)
};

// Candidate list of particle i: 32 bytes, 16 int16 {count, b_1 - i, ..., b_15 - i}
// (two int4 at nl[2i], nl[2i+1]), so one warp reads its lists in two coalesced
// 16-byte loads per lane and every candidate is known before the first gather.
constexpr int NL = 15;               // candidate-list capacity per particle
constexpr int32_t NL_OVERFLOW = 255; // count marking a particle that searches the cell table instead
constexpr int32_t NL_BIG = 254;      // count marking a large particle (partners from k_big_narrow)
constexpr int32_t NL_NEAR_BIG = 0x100; // count flag: a large particle was within reach at the rebuild
constexpr int BIG_ACC_MAX = 2048;    // partners a large particle may touch at once

struct Event {
    int32_t scene, step, bond, code, a, b;
};
static_assert(sizeof(Event) == sizeof(dem_break_event), "event record layout");

struct Pending {
    int32_t bond, code;
};

struct DevWorld {
    int32_t N, C, B, S, M, MP;
    float4 *pr, *vw, *ac, *dp, *fx, *d4, *dF;
    float4 *pr_n, *dp_n;        // the other position / displacement buffers (written by fused steps)
    uint32_t *meta;
    int32_t *orig;
    int32_t *o2i;               // [N] particle_base + scene-local index -> internal index (kept by the reorder)
    // what a step never writes, in the reference layout and scene-local order
    // (index particle_base + scene-local index): downloads copy it out whole
    int32_t *fix_ref;           // [6N] fixity {x, y, rot, x2, y2, rot2}
    float *force_ref;           // [6N] external forces
    int32_t *matp_ref;          // [N] material pointers
    float *data3;               // [N] data[7i+3]
    uint32_t *smask;            // bits 0-13: occupied slots; 14: NL_LIVE; 16-29: slot's bonded field >= 0;
                                // 31: DF_ZERO
    int32_t *s_b, *s_bonded;
    float *s_tf, *s_btf, *s_thb;
    int32_t *b_status;
    float *b_length;
    float2 *b_str;
    Mat *mats;
    float2 *pair;               // per scene and material pair: {1/(1/kn_a + 1/kn_b), 1/(1/ks_a + 1/ks_b)}
    ScenePar *par;
    int32_t *cc3;              // per scene "positions set externally" flag
    // broad phase
    uint32_t *keys;
    int32_t *cell_count, *cell_start, *sorted, *inv, *src, *scan_tmp;
    int32_t *wperm;             // rebuild: cell-order position -> position after grouping by contact count
    int32_t *sort_counts;       // [SORT_GRID_MAX][256] digit counts / offsets of the cell sort's passes
    // bond breaks of the current step (applied after the Simulation pass)
    Pending *pend;
    uint32_t *pend_count;
    uint32_t pend_cap;
    // event log
    Event *ev;
    unsigned long long *ev_count;
    uint32_t ev_cap;
    unsigned long long *stats;  // [0] capped, [1] events, [2] dropped, [3] pending overflow, [4] rebuilds, [5] list overflows
    long long *step;            // device step counter
    int32_t *err;
    // candidate lists (built at rebuilds)
    int4 *nl;                   // [N][2] candidate lists (see NL)
    float2 *pbuild;             // [N] position at the last rebuild
    uint32_t *kbuild;           // [N] search cell at the last rebuild
    int32_t *rebuild;           // 1 = the next rebuild body runs
    int32_t *reorder;           // 1 = that rebuild also reorders the particle arrays into cell order
    int32_t reorder_every;      // rebuilds per reorder
    uint32_t *tickets;          // [2] last-warp counters of k_lom and k_interact
    int32_t ticket;             // 1: those kernels' last warps end the step; 0: separate one-warp kernels
    int32_t split;              // 1: the Simulation pass as k_narrow + k_forces instead of k_interact
    int32_t *big_acc;           // [slots][16]: accepted partners of a large particle, [15] = count
    int32_t *big_scene;         // [slots] scene of each big-partner record, -1 unused
    int32_t n_big_slots;
    int32_t *det;               // [S] narrow phase runs in the current step
    const uint8_t *live;        // [ceil(N/128)] 0: every particle of the 128-particle chunk is free
                                // (served worlds: the step kernels skip it); null: all chunks live
    int32_t *act;               // [S] 1 = the scene steps; 0 = frozen (finished or free slot)
    long long *remaining;       // [S] steps left before the scene freezes (served scenes)
};

// ---- stateless detection schedule -----------------------------------------
// The LOM pass's thread 0 does cc1 += 1; if cc1 >= interval {cc0 = 1; cc1 = 0}
// else {cc0 = 0} (2D_LOM.wgsl:155-163).  From cc1_0 at step0 the detect steps
// are j1, j1+P, j1+2P, ... with P = max(interval, 1), j1 = max(0, interval-1-cc1_0).
__host__ __device__ inline bool detect_at(int32_t interval, int32_t cc1_0, long long j) {
    long long P = interval > 1 ? interval : 1;
    long long j1 = (long long)interval - 1 - cc1_0;
    if (j1 < 0) j1 = 0;
    return j >= j1 && ((j - j1) % P) == 0;
}
// counter value after j steps
__host__ __device__ inline int32_t cc1_after(int32_t interval, int32_t cc1_0, long long j) {
    if (j <= 0) return cc1_0;
    long long P = interval > 1 ? interval : 1;
    long long j1 = (long long)interval - 1 - cc1_0;
    if (j1 < 0) j1 = 0;
    if (j <= j1) return (int32_t)(cc1_0 + j);
    long long since = (j - 1 - j1) % P;  // steps after the last detect
    return (int32_t)since;
}

// Worlds up to this many particles end LOM and Simulation passes by last-warp
// election (no extra launches); larger ones use two one-warp kernels instead,
// because the fenced per-warp ticket costs ~0.4 ns x warps on each kernel.
constexpr int TICKET_MAX_N = 131072;

// host launchers (dem_kernels.cu)
// LOM of one step; with in_graph the rebuild conditional is set on the device.
// Both launchers return the number of kernels they launched.
int launch_lom(const DevWorld &w, int block, cudaStream_t st, bool in_graph,
                cudaGraphConditionalHandle cond);
void launch_keys(const DevWorld &w, int block, cudaStream_t st, const int32_t *gate);
// returns the number of kernels launched
int launch_broad_phase(const DevWorld &w, int block, cudaStream_t st, const int32_t *gate);
void launch_reorder(const DevWorld &w, const DevWorld &spare, int block, cudaStream_t st,
                    const int32_t *gate);
int launch_list_build(const DevWorld &w, int block, cudaStream_t st, const int32_t *gate, bool every_step,
                      bool staged);
// the Simulation pass of one step; with `fuse` also the next step's LOM pass
// (into the other pr/dp/rr buffers), whose rebuild condition is set on `cond`
// when in a graph.  A fused step is never a call's last step; lom_final: the
// next one is (its LOM pass keeps data[4..6]).
// form selects the Simulation kernels compiled for what the scenes need:
// 0 or 3 (every scene uses that bond model, none the F64 distances), -2 (any
// bond model, no F64 distances), -1 (anything)
// ps, pv: where the Simulation kernels read the scene parameters.  PS_SCENE
// (pv unused): w.par[scene].  PS_ONE: *pv, equal to w.par[0], the world's
// only scene.  PS_SHARED: the settings every scene of the world shares
// (shared_settings) from *pv, the rest from w.par[scene].
constexpr int PS_SCENE = 0, PS_SHARED = 1, PS_ONE = 2;
int launch_interact(const DevWorld &w, int block, cudaStream_t st, bool bigs, bool fuse, bool lom_final,
                    bool in_graph, cudaGraphConditionalHandle cond, int form, const ScenePar *pv, int ps);

// The fields of a scene's parameters that the Simulation kernels read from
// the launch under PS_SHARED (the settings and model constants), the others
// zero; with bonds false also the bond model's fields, which a scene without
// bond records never reads (it has no bonded slot, so it steps alike under
// any bond settings).  Scenes share their settings when their records agree
// here, the bond fields compared among the scenes that have bonds.
inline ScenePar shared_settings(const ScenePar &P, bool bonds) {
    ScenePar k;
    std::memset(&k, 0, sizeof k);
    k.p.collisions = P.p.collisions;
    k.p.gravity = P.p.gravity;
    k.p.planet_mode = P.p.planet_mode;
    k.p.mouse_gravity = P.p.mouse_gravity;
    k.p.gravity_x = P.p.gravity_x;
    k.p.gravity_y = P.p.gravity_y;
    k.p.gravity_acc = P.p.gravity_acc;
    k.p.dT = P.p.dT;
    k.p.friction_coefficient = P.p.friction_coefficient;
    k.p.round_bounds = P.p.round_bounds;
    k.p.bound_radius = P.p.bound_radius;
    k.n_mat = P.n_mat;
    k.damp2 = P.damp2;
    k.use_f64 = P.use_f64;
    if (bonds) {
        k.p.bonds = P.p.bonds;
        k.p.bond_normal_strength = P.p.bond_normal_strength;
        k.p.bond_shear_strength = P.p.bond_shear_strength;
        k.p.bond_normal_stiffness = P.p.bond_normal_stiffness;
        k.p.bond_shear_stiffness = P.p.bond_shear_stiffness;
        k.p.bonds_tear = P.p.bonds_tear;
        k.p.moment_contribution_factor = P.p.moment_contribution_factor;
        k.p.contact_damping = P.p.contact_damping;
        k.has_strength = P.has_strength;
        k.lambda = P.lambda;
        k.kb2 = P.kb2;
        k.ksb2 = P.ksb2;
    }
    return k;
}
void launch_set_properties(const DevWorld &w, int scene, const int32_t *d_sel, int32_t *d_sel_out,
                           const int32_t *d_props, int block, cudaStream_t st);
int scan_tmp_size(int n);
// out[0..n) = exclusive prefix sums of in[0..n), out[n] = total; tmp holds scan_tmp_size(n) ints
void launch_exclusive_scan(const int32_t *in, int32_t *out, int n, int32_t *tmp, cudaStream_t st);
// A scene in the reference's host layouts (state.rs:69-93), resident on the
// device: uploads copy the caller's arrays here in a few large transfers and
// a kernel builds the internal layout; downloads do the reverse.
struct RefArrays {
    float *pos, *radii, *vel, *acc, *rot, *rot_vel, *rot_acc, *forces, *del_pos, *del_rot, *data;
    int32_t *fixity, *contacts, *material_pointers;
};
// One scene of a staging transfer: particles [off, off + n) of the staging
// block are particles [base, base + n) of the world, which hold scene `scene`.
// A transfer's items are sorted by off and do not overlap; n > 0.  Staged
// positions between items (padding) belong to no item and are skipped.
struct StageItem {
    long long off;
    int base, n, scene, n_mat, n_bonds, has_data;
    float r_big;
    int pad;
};
// validation of the staged arrays (items in device memory, `total` staged
// particles); failures OR bits into err[k] of item k: 1 material pointer,
// 2 bonded index >= n_bonds, 4 partner out of range, 8 record's a differs
// from its owner
void launch_stage_check(const RefArrays &r, const StageItem *items, int count, long long total, int32_t *err,
                        cudaStream_t st);
// reference layout -> internal layout of every item's scene
void launch_stage_in(const DevWorld &w, const RefArrays &r, const StageItem *items, int count, long long total,
                     cudaStream_t st);
// internal layout -> reference layout; err[k] bits: 16 internal map corrupt,
// 32 contact partner outside the scene; err[count] = OR of all
void launch_stage_out(const DevWorld &w, const RefArrays &r, const StageItem *items, int count, long long total,
                      int32_t *err, cudaStream_t st);

// One contiguous copy of a transfer, between the caller's host memory and
// the device (through the device's access to pageable host memory) or
// within the device; bytes a multiple of 4, both ends 4-byte aligned.  It
// runs as pieces of COPY_PIECE bytes; piece0 = pieces of the copies before.
constexpr long long COPY_PIECE = 65536;
struct HostCopy {
    const char *src;
    char *dst;
    long long bytes;
    long long piece0;
};
// every piece of copies c[0..n) (`pieces` in all); nothing if guard != NULL
// and *guard != 0
void launch_copies(const HostCopy *c, int n, long long pieces, const int32_t *guard, cudaStream_t st);

// Fix / Drop / Release events (src/shaders/event_handling/{Fix,Drop,Release}.wgsl)
// on `count` particles of the scene whose first particle is `base`, given
// by scene-local index (kind: DEM_EVENT_FIX, _DROP, _RELEASE); Fix also
// zeroes the velocity and rotational velocity, Release with set_vel sets the
// velocity.
void launch_fixity_event(const DevWorld &w, int base, const int32_t *d_idx, int count, int kind, float vx,
                         float vy, int set_vel, cudaStream_t st);
// gather of the datum fields (state.rs:708-737) of `count` particles, 10 floats each
void launch_gather_datum(const DevWorld &w, int base, const int32_t *d_idx, int count, float *d_out,
                         cudaStream_t st);
// mark particles [first, first + count) as unused: scene `free_scene`, radius 0
void launch_mark_free(const DevWorld &w, int first, int count, int free_scene, cudaStream_t st);

}  // namespace demgb

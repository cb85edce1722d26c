/*
 * dem_oracle.h -- CPU oracle for the per-step DEM pipeline (TEST INFRASTRUCTURE).
 *
 * This is the checker, not the product.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline / reference arm load it.  The product path
 * (libdemgb.so, include/dem.h) never links or calls it.
 *
 * It restates, deterministically and in the reference's operation order, the
 * two WGSL compute passes that make one simulation step of gusjengis/Physics-Sim:
 *   LOM pass         src/shaders/physics/2D_LOM.wgsl:80-201
 *   Simulation pass  src/shaders/physics/2D_Simulation.wgsl:108-478
 * dispatched in that order by WGPUComputeProg::compute (src/wgpu_prog.rs:1420-1473),
 * plus the Set_Properties event (src/shaders/event_handling/Set_Properties.wgsl:68-90).
 *
 * Reference races are resolved deterministically (each choice is a possible
 * execution of the reference):
 *   - coll_cont[0] is updated once per step before any particle reads it
 *     (2D_LOM.wgsl:155-166);
 *   - the bucket grid is filled in particle-index order and is never truncated
 *     (2D_LOM.wgsl:180-199); cells that exceed the reference's cell_cap are
 *     counted in stats[ORC_STAT_CELL_OVERFLOW];
 *   - a bond break written during the Simulation pass becomes visible to the
 *     partner from the next step (2D_Simulation.wgsl:236-239 vs 324).
 *
 * Layouts are the reference's host arrays (src/state.rs:69-93): contacts are
 * 24-byte records {a:i32, b:i32, tangent_force:f32, bond_tangent_force:f32,
 * theta_b:f32, bonded:i32}, 14 per particle; bonds are 12-byte records
 * {index:i32, angle:f32, length:f32}.
 */
#ifndef DEM_ORACLE_H
#define DEM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_CONTACTS 14
#define ORC_DATA_SIZE 7

/* The 29-word Settings uniform, field order of settings.rs:2086-2119. */
typedef struct orc_settings {
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
} orc_settings;

/* Extensions; zeroed struct + bond_lambda=0.5 gives reference behaviour. */
typedef struct orc_ext {
    int32_t use_f64;        /* F64 distance branch (2D_Simulation.wgsl:264-284, shader_gen.rs:84) */
    float bond_lambda;      /* parallel-bond radius factor, reference 0.5 (2D_Simulation.wgsl:290) */
    const float *bond_sn;   /* optional per-bond normal strength [n_bonds], NULL = global */
    const float *bond_ss;   /* optional per-bond shear strength [n_bonds], NULL = global */
    float restitution;      /* particle-particle normal dashpot, an extension (0 = off, the
                               reference's springs only); same definition as dem_ext.restitution */
} orc_ext;

typedef struct orc_state {
    int32_t n;              /* particles */
    int32_t n_bonds;        /* bond records */
    int32_t n_materials;    /* material records (6 floats each) */
    float *pos;             /* [2n] */
    float *radii;           /* [n] */
    float *vel;             /* [2n] */
    float *acc;             /* [2n]  binding "accelerations" */
    float *rot;             /* [n] */
    float *rot_vel;         /* [n] */
    float *rot_acc;         /* [n] */
    float *forces;          /* [6n]  {x, y, rot, 3 unused} */
    int32_t *fixity;        /* [6n]  {x, y, rot, x2, y2, rot2} */
    float *del_pos;         /* [2n] */
    float *del_rot;         /* [n] */
    int32_t *bonds;         /* [3*n_bonds] raw bits {index, angle, length} */
    int32_t *contacts;      /* [6*14*n] raw bits */
    int32_t *material_pointers; /* [n] */
    float *materials;       /* [6*n_materials] {r, g, b, density, kn, ks} */
    float *data;            /* [7n] diagnostics */
    int32_t coll_cont[4];   /* detect flag, interval counter, tick, positions-set flag */
    float cell_size;        /* GridInfo (wgpu_prog.rs:698-717) */
    int32_t cell_cap;
    int32_t grid_w;
    int32_t grid_h;
} orc_state;

typedef struct orc_break {
    int32_t step;      /* step index within the call, offset by step_base */
    int32_t bond;      /* bond record index */
    int32_t code;      /* -10 + sign(normal displacement) */
    int32_t a;         /* particle that evaluated the break */
    int32_t b;         /* its partner */
} orc_break;

enum {
    ORC_STAT_CAPPED = 0,        /* particles whose narrow phase reached 14 contacts */
    ORC_STAT_CELL_OVERFLOW = 1, /* cell fills beyond the reference's cell_cap-2 entries */
    ORC_STAT_BREAKS = 2,        /* break evaluations that fired */
    ORC_STAT_EVENTS_DROPPED = 3,/* events beyond ev_cap */
    ORC_NSTATS = 4
};

/* Advance nsteps in reference mode (FP32, F64 distance when ext->use_f64).
 * threads <= 0 uses the OpenMP default.  Returns 0, or -1 on bad arguments. */
int orc_step_f32(orc_state *s, const orc_settings *p, const orc_ext *e, int nsteps,
                 int step_base, orc_break *ev, int ev_cap, int *ev_n, int64_t *stats,
                 int threads);

/* FP64 twin of the same steps: the state is read as float, evolved entirely in
 * double, and written to the double arrays of *out (same field layout as
 * orc_state, each float array widened to double; contacts/bonds as in s). */
typedef struct orc_state_d {
    double *pos, *vel, *acc, *rot, *rot_vel, *rot_acc, *del_pos, *del_rot, *data;
    double *slot_tf, *slot_btf, *slot_thb;  /* [14n] */
} orc_state_d;
int orc_step_f64(const orc_state *s, const orc_settings *p, const orc_ext *e, int nsteps,
                 orc_state_d *out, int threads);

/* Set_Properties event (Set_Properties.wgsl:68-90). input: 28 words, field
 * order of Settings::properties (settings.rs:2158-2189). selections [n] is
 * updated in place (2 where a fixity was set). */
void orc_set_properties(orc_state *s, int32_t *selections, const int32_t input[28]);

/* grid_capacity (wgpu_prog.rs:698-717) for given bounds and radii extremes. */
void orc_grid_capacity(float hor_bound, float vert_bound, float max_radius, float min_radius,
                       int variable_rad, int particles, float *cell_size, int32_t *cell_cap,
                       int32_t *w, int32_t *h);

/* regen_bonds (state.rs:291-367).  bonds_out needs 3*max_bonds*n ints,
 * contacts_out 6*14*n ints (fully overwritten).  Returns the bond count. */
int orc_regen_bonds(int n, const float *pos, const float *radii, int max_bonds,
                    int32_t *bonds_out, int32_t *contacts_out);

#ifdef __cplusplus
}
#endif
#endif

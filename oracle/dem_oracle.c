/*
 * dem_oracle.c -- CPU oracle for the per-step DEM pipeline (TEST INFRASTRUCTURE).
 *
 * The checker, never the product: see dem_oracle.h for what it restates and
 * how the reference's races are resolved.  Compiled by oracle/build_oracle.py
 * with -O2 -fopenmp -ffp-contract=off -fno-strict-aliasing so that float
 * expressions round exactly as written.
 */
#include "dem_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_PI 3.141592653589793238

/* WGSL i32(f32): truncate toward zero; saturate out of range; NaN -> 0 */
static inline int32_t orc_i32(float x) {
    if (x != x) return 0;
    if (x >= 2147483648.0f) return 2147483647;
    if (x <= -2147483648.0f) return (int32_t)(-2147483647 - 1);
    return (int32_t)x;
}
static inline float orc_len_f32(float x, float y) { return sqrtf(x * x + y * y); }
static inline double orc_len_f64(double x, double y) { return sqrt(x * x + y * y); }

/* 2 zeta of the normal dashpot for restitution e (0: off, and e >= 1 is no
 * damping): zeta = -ln e / sqrt(pi^2 + ln^2 e) in double; the reference-mode
 * step rounds it to float once, the twin keeps the double */
static inline double orc_dashpot_2zeta(float e) {
    if (!(e > 0.0f) || e >= 1.0f) return 0.0;
    const double l = log((double)e);
    return 2.0 * (-l / sqrt(ORC_PI * ORC_PI + l * l));
}

/* ---- reference-mode instantiation (float) ---- */
#define REAL float
#define REAL_IS_FLOAT 1
#define FN(x) x##_f32
#define SLOT slot_f32
#define BOND bond_f32
#define STATE state_f32
#define GRID grid_f32
#define V3 v3_f32
#define EVBUF evbuf_f32
#include "dem_oracle_step.inc"
#undef LEN2
#undef SQRT_R
#undef REAL
#undef REAL_IS_FLOAT
#undef FN
#undef SLOT
#undef BOND
#undef STATE
#undef GRID
#undef V3
#undef EVBUF

/* ---- FP64 twin ---- */
#define REAL double
#define REAL_IS_FLOAT 0
#define FN(x) x##_f64
#define SLOT slot_f64
#define BOND bond_f64
#define STATE state_f64
#define GRID grid_f64
#define V3 v3_f64
#define EVBUF evbuf_f64
#include "dem_oracle_step.inc"
#undef LEN2
#undef SQRT_R
#undef REAL
#undef REAL_IS_FLOAT
#undef FN
#undef SLOT
#undef BOND
#undef STATE
#undef GRID
#undef V3
#undef EVBUF

_Static_assert(sizeof(slot_f32) == 24, "contact record is 24 bytes (2D_Simulation.wgsl:19-26)");
_Static_assert(sizeof(bond_f32) == 12, "bond record is 12 bytes (2D_Simulation.wgsl:28-32)");

static int orc_validate(const orc_state *s) {
    if (!s || s->n < 0 || s->n_bonds < 0 || s->n_materials <= 0) return -1;
    if (s->grid_w <= 0 || s->grid_h <= 0 || !(s->cell_size > 0.0f)) return -1;
    for (int i = 0; i < s->n; ++i) {
        int32_t m = s->material_pointers[i];
        if (m < 0 || m >= s->n_materials) return -1;
    }
    const int64_t ns = (int64_t)s->n * ORC_MAX_CONTACTS;
    for (int64_t k = 0; k < ns; ++k) {
        int32_t bonded = s->contacts[6 * k + 5];
        int32_t a = s->contacts[6 * k], b = s->contacts[6 * k + 1];
        if (bonded >= s->n_bonds) return -1;
        if (b != -1 && (b < 0 || b >= s->n || a < 0 || a >= s->n)) return -1;
    }
    return 0;
}

static state_f32 orc_view_f32(orc_state *s) {
    state_f32 t;
    t.n = s->n; t.n_bonds = s->n_bonds; t.n_materials = s->n_materials;
    t.pos = s->pos; t.radii = s->radii; t.vel = s->vel; t.acc = s->acc; t.rot = s->rot;
    t.rot_vel = s->rot_vel; t.rot_acc = s->rot_acc; t.forces = s->forces; t.fixity = s->fixity;
    t.del_pos = s->del_pos; t.del_rot = s->del_rot;
    t.bonds = (bond_f32 *)(void *)s->bonds;
    t.contacts = (slot_f32 *)(void *)s->contacts;
    t.material_pointers = s->material_pointers; t.materials = s->materials; t.data = s->data;
    t.coll_cont = s->coll_cont;
    t.cell_size = s->cell_size; t.cell_cap = s->cell_cap; t.grid_w = s->grid_w; t.grid_h = s->grid_h;
    return t;
}

int orc_step_f32(orc_state *s, const orc_settings *p, const orc_ext *e, int nsteps, int step_base,
                 orc_break *ev, int ev_cap, int *ev_n, int64_t *stats, int threads) {
    if (!p || !e || nsteps < 0 || orc_validate(s)) return -1;
    state_f32 t = orc_view_f32(s);
    evbuf_f32 all;
    memset(&all, 0, sizeof all);
    int rc = run_steps_f32(&t, p, e, nsteps, step_base, &all, stats, threads);
    int k = all.n < ev_cap ? all.n : ev_cap;
    if (ev && k > 0) memcpy(ev, all.buf, sizeof(orc_break) * (size_t)k);
    if (ev_n) *ev_n = all.n;
    if (stats && all.n > ev_cap) stats[ORC_STAT_EVENTS_DROPPED] += all.n - ev_cap;
    free(all.buf);
    return rc;
}

int orc_step_f64(const orc_state *s, const orc_settings *p, const orc_ext *e, int nsteps,
                 orc_state_d *out, int threads) {
    if (!p || !e || !out || nsteps < 0 || orc_validate(s)) return -1;
    const int n = s->n, nb = s->n_bonds, nm = s->n_materials;
    const int64_t ns = (int64_t)n * ORC_MAX_CONTACTS;
    state_f64 t;
    t.n = n; t.n_bonds = nb; t.n_materials = nm;
    double *buf = (double *)malloc(sizeof(double) * ((size_t)n * 20 + 6 * (size_t)nm));
    int32_t cc[4];
    memcpy(cc, s->coll_cont, sizeof cc);
    t.coll_cont = cc;
    t.bonds = (bond_f64 *)malloc(sizeof(bond_f64) * (size_t)(nb > 0 ? nb : 1));
    t.contacts = (slot_f64 *)malloc(sizeof(slot_f64) * (size_t)(ns > 0 ? ns : 1));
    if (!buf || !t.bonds || !t.contacts) { free(buf); free(t.bonds); free(t.contacts); return -1; }
    double *q = buf;
#define TAKE(dst, src, cnt) do { dst = q; for (int64_t _i = 0; _i < (int64_t)(cnt); ++_i) q[_i] = (double)(src)[_i]; q += (cnt); } while (0)
    TAKE(t.pos, s->pos, 2 * n);
    TAKE(t.radii, s->radii, n);
    TAKE(t.vel, s->vel, 2 * n);
    TAKE(t.acc, s->acc, 2 * n);
    TAKE(t.rot, s->rot, n);
    TAKE(t.rot_vel, s->rot_vel, n);
    TAKE(t.rot_acc, s->rot_acc, n);
    TAKE(t.del_pos, s->del_pos, 2 * n);
    TAKE(t.del_rot, s->del_rot, n);
    TAKE(t.data, s->data, 7 * n);
#undef TAKE
    /* forces: only the first three of each record are read */
    double *forces = (double *)malloc(sizeof(double) * 6 * (size_t)(n > 0 ? n : 1));
    for (int64_t i = 0; i < 6 * (int64_t)n; ++i) forces[i] = (double)s->forces[i];
    t.forces = forces;
    t.materials = q;
    for (int i = 0; i < 6 * nm; ++i) q[i] = (double)s->materials[i];
    t.fixity = s->fixity;
    t.material_pointers = s->material_pointers;
    for (int i = 0; i < nb; ++i) {
        float ang, len;
        memcpy(&ang, &s->bonds[3 * i + 1], 4);
        memcpy(&len, &s->bonds[3 * i + 2], 4);
        t.bonds[i].index = s->bonds[3 * i];
        t.bonds[i].angle = ang;
        t.bonds[i].length = len;
    }
    for (int64_t k = 0; k < ns; ++k) {
        float tf, btf, thb;
        memcpy(&tf, &s->contacts[6 * k + 2], 4);
        memcpy(&btf, &s->contacts[6 * k + 3], 4);
        memcpy(&thb, &s->contacts[6 * k + 4], 4);
        t.contacts[k].a = s->contacts[6 * k];
        t.contacts[k].b = s->contacts[6 * k + 1];
        t.contacts[k].tf = tf;
        t.contacts[k].btf = btf;
        t.contacts[k].thb = thb;
        t.contacts[k].bonded = s->contacts[6 * k + 5];
    }
    t.cell_size = s->cell_size; t.cell_cap = s->cell_cap; t.grid_w = s->grid_w; t.grid_h = s->grid_h;
    int rc = run_steps_f64(&t, p, e, nsteps, 0, NULL, NULL, threads);
#define GIVE(dst, src, cnt) do { if (dst) memcpy(dst, src, sizeof(double) * (size_t)(cnt)); } while (0)
    GIVE(out->pos, t.pos, 2 * n);
    GIVE(out->vel, t.vel, 2 * n);
    GIVE(out->acc, t.acc, 2 * n);
    GIVE(out->rot, t.rot, n);
    GIVE(out->rot_vel, t.rot_vel, n);
    GIVE(out->rot_acc, t.rot_acc, n);
    GIVE(out->del_pos, t.del_pos, 2 * n);
    GIVE(out->del_rot, t.del_rot, n);
    GIVE(out->data, t.data, 7 * n);
#undef GIVE
    for (int64_t k = 0; k < ns; ++k) {
        if (out->slot_tf) out->slot_tf[k] = t.contacts[k].tf;
        if (out->slot_btf) out->slot_btf[k] = t.contacts[k].btf;
        if (out->slot_thb) out->slot_thb[k] = t.contacts[k].thb;
    }
    free(forces); free(buf); free(t.bonds); free(t.contacts);
    return rc;
}

void orc_set_properties(orc_state *s, int32_t *selections, const int32_t in[28]) {
    float f[28];
    memcpy(f, in, sizeof f);
    for (int id = 0; id < s->n; ++id) {
        if (selections[id] == 0) continue;
        if (in[0] == 1) { s->del_pos[2 * id] = f[14] - s->pos[2 * id]; s->pos[2 * id] = f[14]; s->coll_cont[3] = 1; }
        if (in[1] == 1) { s->del_pos[2 * id + 1] = f[15] - s->pos[2 * id + 1]; s->pos[2 * id + 1] = f[15]; s->coll_cont[3] = 1; }
        if (in[2] == 1) { s->del_rot[id] = f[16] - s->rot[id]; s->rot[id] = f[16]; }
        if (in[3] == 1) s->vel[2 * id] = f[17];
        if (in[4] == 1) s->vel[2 * id + 1] = f[18];
        if (in[5] == 1) s->rot_vel[id] = f[19];
        if (in[9] == 1) s->radii[id] = f[23];
        if (in[6] == 1) s->forces[6 * id] = f[20];
        if (in[7] == 1) s->forces[6 * id + 1] = f[21];
        if (in[8] == 1) s->forces[6 * id + 2] = f[22];
        if (in[10] == 1) { s->fixity[6 * id] = in[24]; s->fixity[6 * id + 3] = in[24]; }
        if (in[11] == 1) { s->fixity[6 * id + 1] = in[25]; s->fixity[6 * id + 4] = in[25]; }
        if (in[12] == 1) { s->fixity[6 * id + 2] = in[26]; s->fixity[6 * id + 5] = in[26]; }
        if (in[13] == 1) s->material_pointers[id] = in[27];
        if (in[10] == 1 || in[11] == 1 || in[12] == 1) selections[id] = 2;
    }
}

static int32_t rust_as_i32(float x) { return orc_i32(x); }

void orc_grid_capacity(float hor_bound, float vert_bound, float max_radius, float min_radius,
                       int variable_rad, int particles, float *cell_size, int32_t *cell_cap,
                       int32_t *w, int32_t *h) {
    float width = hor_bound * 2.0f;
    float height = vert_bound * 2.0f;
    float max_rad = max_radius * 2.0f;
    float min_rad = variable_rad ? min_radius : max_radius;
    int32_t ww = rust_as_i32(ceilf(width / max_rad));
    int32_t hh = rust_as_i32(ceilf(height / max_rad));
    float q = max_rad / min_rad + 1.0f;
    int32_t cap = rust_as_i32(ceilf(q * q));
    if (cap > particles) cap = particles;
    *cell_size = max_rad;
    *cell_cap = cap + 2;
    *w = ww;
    *h = hh;
}

int orc_regen_bonds(int n, const float *pos, const float *radii, int max_bonds, int32_t *bonds_out,
                    int32_t *contacts_out) {
    const int64_t ns = (int64_t)n * ORC_MAX_CONTACTS;
    for (int64_t k = 0; k < 6 * ns; ++k) contacts_out[k] = -1;
    int bond_index = 0;
    for (int i = 0; i < n; ++i) {
        int col_num = 0;
        for (int j = i; j < n; ++j) {
            if (i == j) continue;
            float dx = pos[2 * j] - pos[2 * i], dy = pos[2 * j + 1] - pos[2 * i + 1];
            float distance = sqrtf(dx * dx + dy * dy);
            float sum = radii[i] + radii[j];
            if (distance < sum * 1.05f) {
                if (col_num < max_bonds) {
                    float mag = powf(dx * dx + dy * dy, 0.5f);
                    float nx = dx / mag, ny = dy / mag;
                    float angle = atan2f(nx, ny);
                    bonds_out[3 * bond_index] = 1;
                    memcpy(&bonds_out[3 * bond_index + 1], &angle, 4);
                    memcpy(&bonds_out[3 * bond_index + 2], &mag, 4);
                    for (int k = ORC_MAX_CONTACTS * i; k < ORC_MAX_CONTACTS * (i + 1); ++k) {
                        if (contacts_out[6 * k] == -1) {
                            contacts_out[6 * k] = i; contacts_out[6 * k + 1] = j;
                            contacts_out[6 * k + 2] = 0; contacts_out[6 * k + 3] = 0;
                            contacts_out[6 * k + 4] = 0; contacts_out[6 * k + 5] = bond_index;
                            break;
                        }
                    }
                    for (int k = ORC_MAX_CONTACTS * j; k < ORC_MAX_CONTACTS * (j + 1); ++k) {
                        if (contacts_out[6 * k] == -1) {
                            contacts_out[6 * k] = j; contacts_out[6 * k + 1] = i;
                            contacts_out[6 * k + 2] = 0; contacts_out[6 * k + 3] = 0;
                            contacts_out[6 * k + 4] = 0; contacts_out[6 * k + 5] = bond_index;
                            break;
                        }
                    }
                    col_num++;
                    bond_index++;
                } else if (col_num == max_bonds) {
                    break;
                }
            }
        }
    }
    return bond_index;
}

/*
 * dem_debug.h -- introspection entry points of libdemgb.so used by the parity
 * tests.  They have no counterpart in the reference's compute dispatch: they
 * expose the broad phase's intermediate tables so that cell keys and the
 * sorted order can be checked bit for bit.
 */
#ifndef DEM_DEBUG_H
#define DEM_DEBUG_H
#include <stdint.h>

#include "dem.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Run the broad phase on the current positions (no integration) and return,
 * per scene-local particle, its search-cell key; the particle indices in
 * stable cell order; the cell start table (n_cells + 1 entries).  Any pointer
 * may be NULL; *n_cells receives the scene's cell count: the gw * gh search
 * cells plus one last cell, key gw * gh, holding the particles no cell search
 * visits (zero radius, and the scene's large particles, which come first). */
int dem_debug_broad_phase(dem_ctx *ctx, int32_t *keys, int32_t *order, int32_t *cell_start,
                          int32_t *n_cells);

/* Geometry of the search grid: cell (cx, cy) of a position is
 * floor((x - x0) * inv), floor((y - y0) * inv) clamped to [0, gw-1] x [0, gh-1];
 * key = cy * gw + cx. */
int dem_debug_search_grid(dem_ctx *ctx, float *x0, float *y0, float *inv, int32_t *gw, int32_t *gh);

/* Kernel timing: while enabled, dem_step launches without CUDA graphs and
 * brackets every launch of the named kernels with CUDA events on the
 * context's stream.  dem_debug_kernel_time returns the summed device time
 * (milliseconds) and launch count of one kernel kind since timing was
 * enabled: "interact", "lom", "end_step", and the rebuild's three phases
 * "broad_phase" (keys, cell table, sort, grouping), "reorder" and
 * "candidate_lists" (each launched, gated, at every step). */
int dem_debug_kernel_timing(dem_ctx *ctx, int32_t enable);
int dem_debug_kernel_time(dem_ctx *ctx, const char *kernel, double *total_ms, int64_t *launches);
/* The same kernel timing for a batch. */
int dem_batch_kernel_timing(dem_batch *b, int32_t enable);
int dem_batch_kernel_time(dem_batch *b, const char *kernel, double *total_ms, int64_t *launches);

#ifdef __cplusplus
}
#endif
#endif

// dem_kernels.cu -- sm_103a kernels of one DEM step.
//
// Step = integrate (LOM) -> broad phase (keys, counting sort, cell tables,
// in-cell ordering, periodic reorder) -> interact (narrow phase, contact
// slots, forces, half kick) -> end of step (apply bond breaks).
//
// Arithmetic follows the reference's WGSL expression by expression
// (src/shaders/physics/2D_LOM.wgsl, 2D_Simulation.wgsl).  This file is
// compiled with -fmad=false: no multiply-add is contracted, '/' and sqrtf are
// IEEE round-to-nearest, so every float result is the one the expression
// denotes, identical to a CPU evaluating the same expression.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <tuple>
#include <vector>

#include "dem_sort.cuh"
#include "dem_world.cuh"

namespace demgb {

// Particle kernels launch with the world's block size, any multiple of 32 up
// to 1024 (the autotuner tries 128, 256 and 512).
constexpr int PK_MAX_THREADS = 1024;

// ---------------------------------------------------------------- helpers

__device__ __forceinline__ float len2f(float x, float y) { return sqrtf(x * x + y * y); }

// cell range of the particle's AABB in the reference grid (2D_LOM.wgsl:167-178);
// i32() is truncation toward zero, saturating (cvt.rzi).
__device__ __forceinline__ void ref_range(const ScenePar &P, float px, float py, float r, int &x0,
                                          int &x1, int &y0, int &y1) {
    float left = px - r, right = px + r, bottom = py - r, top = py + r;
    int a = __float2int_rz((left - P.ref_base_x) / P.ref_cs);
    int b = __float2int_rz((right - P.ref_base_x) / P.ref_cs);
    int c = __float2int_rz((P.ref_base_y - top) / P.ref_cs);
    int d = __float2int_rz((P.ref_base_y - bottom) / P.ref_cs);
    x0 = a > 0 ? a : 0;
    x1 = b < P.ref_w - 1 ? b : P.ref_w - 1;
    y0 = c > 0 ? c : 0;
    y1 = d < P.ref_h - 1 ? d : P.ref_h - 1;
}

// The range as one 32-bit code, kept in the w word of the particle's
// position record: the first column and row modulo 2048 (11 bits each), then
// the width and the height in buckets (5 bits each: 0 for an empty side, as
// for a particle off the grid; 31 for 31 or more).  Ranges are compared only
// for pairs that touch, and those ranges overlap or abut: the AABBs overlap,
// the roundings of their edges and the truncation to buckets are monotone,
// and intervals that meet pairwise and each meet the grid meet within it.
// Their first columns (rows) then differ by at most a range's width, so the
// 11-bit differences are the true ones, for any grid size.
__device__ __forceinline__ float range_code(int x0, int x1, int y0, int y1) {
    long long wd = (long long)x1 - x0 + 1, ht = (long long)y1 - y0 + 1;
    wd = wd < 0 ? 0 : (wd > 31 ? 31 : wd);
    ht = ht < 0 ? 0 : (ht > 31 ? 31 : ht);
    return __uint_as_float(((uint32_t)x0 & 2047u) | (((uint32_t)y0 & 2047u) << 11) | ((uint32_t)wd << 22) |
                           ((uint32_t)ht << 27));
}

// Whether the ranges ca (particle a) and cb share a bucket; if so, rank =
// the first shared bucket's position in a's scan order (rows top to bottom,
// columns left to right within a's range), the order in which the reference
// meets b while scanning a's buckets (2D_Simulation.wgsl:143-170).  A rank
// beyond 15 (an AABB wider than 4 buckets: the bucket grid is finer than
// 2 r) or a side of 31 buckets or more sets device error 2.
__device__ __forceinline__ bool shared_bucket(const DevWorld &w, uint32_t ca, uint32_t cb, unsigned &rank) {
    const int wa = (int)((ca >> 22) & 31u), ha = (int)(ca >> 27);
    const int wb = (int)((cb >> 22) & 31u), hb = (int)(cb >> 27);
    if (wa == 0 || ha == 0 || wb == 0 || hb == 0) return false;
    const int dx = (int)((cb - ca) << 21) >> 21;                  // bx0 - ax0
    const int dy = (int)(((cb >> 11) - (ca >> 11)) << 21) >> 21;  // by0 - ay0
    if (dx > wa - 1 || dx + wb - 1 < 0 || dy > ha - 1 || dy + hb - 1 < 0) return false;
    rank = (unsigned)((dy > 0 ? dy : 0) * wa + (dx > 0 ? dx : 0));
    if (rank > 15u || wa == 31 || ha == 31 || wb == 31 || hb == 31) {
        atomicOr(w.err, 2);
        rank = rank < 15u ? rank : 15u;
    }
    return true;
}

// the w word of particle b's position record: its range code
__device__ __forceinline__ uint32_t range_of(const DevWorld &w, int b) {
    return __float_as_uint(__ldg(reinterpret_cast<const float *>(w.pr + b) + 3));
}

// search-grid cell of a position (floor, clamped to the grid)
__device__ __forceinline__ void search_xy(const ScenePar &P, float x, float y, int &cx, int &cy) {
    int a = __float2int_rd((x - P.g_x0) * P.g_inv);
    int b = __float2int_rd((y - P.g_y0) * P.g_inv);
    cx = a < 0 ? 0 : (a > P.g_w - 1 ? P.g_w - 1 : a);
    cy = b < 0 ? 0 : (b > P.g_h - 1 ? P.g_h - 1 : b);
}

// The scene's large particles at the last rebuild: the members of its large
// particles' cell, sorted[first + k] for k < cnt (in scene-local index
// order).  The cell list names internal indices whether or not that rebuild
// reordered the particle arrays.
__device__ __forceinline__ void big_cell(const DevWorld &w, const ScenePar &P, int &first, int &cnt) {
    first = w.cell_start[P.big_cell];
    cnt = w.cell_start[P.big_cell + 1] - first;
}

struct F3 {
    float x, y, z;
};

// distance2 (2D_Simulation.wgsl:273-284): |pa-pb| - length, F64 branch optional
__device__ __forceinline__ float distance2(int use_f64, float4 pa, float4 pb, float length) {
    if (use_f64) {
        double dx = (double)pa.x - (double)pb.x, dy = (double)pa.y - (double)pb.y;
        return (float)(sqrt(dx * dx + dy * dy) - (double)length);
    }
    float dx = pa.x - pb.x, dy = pa.y - pb.y;
    return len2f(dx, dy) - length;
}
// distance (2D_Simulation.wgsl:264-271): the F64 branch sums the radii in double
__device__ __forceinline__ float distance1(int use_f64, float4 pa, float4 pb) {
    if (use_f64) {
        double dx = (double)pa.x - (double)pb.x, dy = (double)pa.y - (double)pb.y;
        return (float)(sqrt(dx * dx + dy * dy) - ((double)pa.z + (double)pb.z));
    }
    float dx = pa.x - pb.x, dy = pa.y - pb.y;
    return len2f(dx, dy) - (pa.z + pb.z);
}

struct Acc3 {
    float d0, d1, d2;
};

// linear_model (2D_Simulation.wgsl:338-373)
// kns = {1/(1/kn_a + 1/kn_b), 1/(1/ks_a + 1/ks_b)} of the two materials
// (2D_Simulation.wgsl:345-346), evaluated once per material pair on the host
// with the same float operations
// L = len2f(pa - pb), which the caller computes once per slot (every float
// distance of the slot is this same value)
// GEN: the generic form -- the scene may use the F64 distance and the
// normal dashpot (read from its parameters); false compiles the reference's
// FP32 arithmetic only.
// meff: m_a m_b / (m_a + m_b), read only by the dashpot.
// The dashpot (an extension, off unless the scene asks for it): after the
// normal direction is known, Fn -= c v_n with c = 2 zeta sqrt(kn meff) and
// v_n = ((da - db) . n) / dT, the step's normal approach speed (negative
// while closing), then Fn = max(Fn, 0).
template <bool GEN>
__device__ __forceinline__ F3 linear_model(const ScenePar &P, float2 kns, float4 pa,
                                           float4 da, float4 pb, float4 db, float length, float L, float &tf,
                                           Acc3 &acc, float meff) {
    F3 out = {0.0f, 0.0f, 0.0f};
    float d2 = (GEN && P.use_f64) ? distance2(1, pa, pb, length) : L - length;
    float nd = d2 < 0.0f ? d2 : 0.0f;
    if (nd == 0.0f) return out;
    float kn = kns.x;
    float ks = kns.y;
    float Fn = (-nd) * kn;
    float vx = pa.x - pb.x, vy = pa.y - pb.y;
    float nx = vx / L, ny = vy / L;
    if (GEN && P.damp2 > 0.0f) {
        const float c = P.damp2 * sqrtf(kn * meff);
        const float vn = ((da.x - db.x) * nx + (da.y - db.y) * ny) / P.p.dT;
        Fn = Fn - c * vn;
        Fn = Fn > 0.0f ? Fn : 0.0f;
    }
    float tx = -ny, ty = nx;
    float dra = da.z * pa.z;
    float drb = db.z * pb.z;
    float rx = db.x - da.x, ry = db.y - da.y;
    float rr = drb + dra;
    float rt = (rx * tx + ry * ty) + rr;
    float fl = (Fn < 0.0f ? -Fn : Fn) * P.p.friction_coefficient;
    float t = tf + rt * ks;
    t = t > -fl ? t : -fl;
    t = t < fl ? t : fl;
    tf = t;
    float M = (-pa.z) * tf;
    out.x = nx * Fn + tx * tf;
    out.y = ny * Fn + ty * tf;
    out.z = M;
    acc.d0 = acc.d0 + Fn;
    acc.d1 = acc.d1 + tf;
    acc.d2 = acc.d2 + M;
    return out;
}

__device__ __forceinline__ int sign_i32(float x) { return x > 0.0f ? 1 : (x < 0.0f ? -1 : 0); }

__device__ __forceinline__ void record_break(const DevWorld &w, const ScenePar &P, int scene,
                                             long long step, int bond_global, int code, int a_int,
                                             int b_int) {
    uint32_t p = atomicAdd(w.pend_count, 1u);
    if (p < w.pend_cap) {
        w.pend[p].bond = bond_global;
        w.pend[p].code = code;
    } else {
        atomicAdd(&w.stats[3], 1ull);
    }
    unsigned long long e = atomicAdd(w.ev_count, 1ull);
    if (e < w.ev_cap) {
        Event ev;
        ev.scene = scene;
        ev.step = (int32_t)step;
        ev.bond = bond_global - P.bond_base;
        ev.code = code;
        ev.a = w.orig[a_int];
        ev.b = w.orig[b_int];
        w.ev[e] = ev;
    } else {
        atomicAdd(&w.stats[2], 1ull);
    }
    atomicAdd(&w.stats[1], 1ull);
}

// ------------------------------------------------------------ LOM kernel
// Last-block election: after the block's writes are fenced, one thread takes
// a ticket; the block holding the final ticket sees every other block's writes.
// Last-warp election: after a warp's writes are fenced, lane 0 takes a
// ticket; the warp holding the final ticket sees every other warp's writes.
// Warps never wait for each other (no block barrier).
__device__ __forceinline__ bool last_warp(uint32_t *ticket) {
    __syncwarp();
    uint32_t t = 0;
    if ((threadIdx.x & 31) == 0) {
        __threadfence();
        t = atomicAdd(ticket, 1u);
    }
    t = __shfl_sync(0xffffffffu, t, 0);
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    const bool last = (t == warps - 1);
    if (last) __threadfence();
    return last;
}

// 2D_LOM.wgsl:80-152 per particle, plus the candidate-list validity check:
// a particle that moved more than half the skin since the last rebuild asks
// for a rebuild before this step's Simulation pass.
// 2D_LOM.wgsl:85-152 of one particle from its records (p, v, a, flags m,
// rebuild position b); `ext`: positions were set externally, so the
// displacement is the stored dext.  Position and bucket range go to pr_out,
// the displacement to dp_out, the velocities and rotation to vw, and
// data[4..6] to d4 when keep_d4 (a later LOM pass of the same call would
// overwrite it).
// U: the scene's settings (P.p) and model constants, P its geometry; the
// two are the same record unless the world's scenes share the former.
__device__ __forceinline__ void lom_core(const DevWorld &w, const ScenePar &P, const ScenePar &U, int i,
                                         uint32_t m, float4 p, float4 v, float4 a, float2 b, bool ext, float4 dext,
                                         bool keep_d4, float4 *pr_out, float4 *dp_out) {
    const float dT = U.p.dT;
    float ivx = v.x, ivy = v.y, iw = v.z;
    if (m & M_KICK_X) ivx = ivx + (a.x * dT) * 0.5f;               // :88
    if (m & M_KICK_Y) ivy = ivy + (a.y * dT) * 0.5f;               // :89
    if (m & M_KICK_R) iw = iw + (a.z * dT) * 0.5f;                 // :90
    if (keep_d4) w.d4[i] = make_float4(ivx, ivy, iw, 0.0f);        // :92-94
    float4 d;
    if (!ext) {                                                    // :96-99
        d = make_float4(ivx * dT, ivy * dT, iw * dT, 0.0f);
    } else {
        d = dext;
    }
    float r = p.z;
    float npx = p.x + d.x, npy = p.y + d.y;                        // :103
    if (U.p.round_bounds == 0) {                                   // :104-129
        float yH = P.yH, xW = P.xW;
        if (!(m & M_FIX_Y)) {
            if (npy - r < -yH) {
                ivy = (-ivy) * 0.5f;
                p.y = p.y + ((-yH) - (npy - r));
            } else if (npy + r > yH) {
                ivy = (-ivy) * 0.5f;
                p.y = p.y - ((npy + r) - yH);
            }
        }
        if (!(m & M_FIX_X)) {
            if (npx - r < -xW) {
                ivx = (-ivx) * 0.5f;
                p.x = p.x + ((-xW) - (npx - r));
            } else if (npx + r > xW) {
                ivx = (-ivx) * 0.5f;
                p.x = p.x - ((npx + r) - xW);
            }
        }
    } else if (len2f(npx, npy) + r > U.p.bound_radius) {          // :130-145
        float L = len2f(npx, npy);
        float nx = npx / L, ny = npy / L;
        float dd = d.x * nx + d.y * ny;
        float dcx = dd * nx, dcy = dd * ny;
        float vv = ivx * nx + ivy * ny;
        float cvx = vv * nx, cvy = vv * ny;
        float Rb = U.p.bound_radius;
        if (!(m & M_FIX_X)) {
            p.x = (nx * (Rb - r)) - dcx;
            ivx = (-cvx) * 0.5f;
        }
        if (!(m & M_FIX_Y)) {
            p.y = (ny * (Rb - r)) - dcy;
            ivy = (-cvy) * 0.5f;
        }
    }
    p.x = p.x + d.x;                                               // :148
    p.y = p.y + d.y;
    const float rot = v.w + d.z;                                   // :149
    {
        int x0, x1, y0, y1;                                        // 2D_LOM.wgsl:167-178
        ref_range(P, p.x, p.y, p.z, x0, x1, y0, y1);
        p.w = range_code(x0, x1, y0, y1);
    }
    pr_out[i] = p;
    w.vw[i] = make_float4(ivx, ivy, iw, rot);                      // :151-152
    if (!ext) dp_out[i] = d;
    const float ex = p.x - b.x, ey = p.y - b.y;
    if (!(ex * ex + ey * ey <= P.disp_limit2)) atomicOr(w.rebuild, 1);
}

__device__ __forceinline__ void lom_particle(const DevWorld &w, int i) {
    // all of the particle's records requested at once (valid for any i < N)
    const uint32_t m = w.meta[i];
    const float4 p = w.pr[i];
    const float4 v = w.vw[i];
    const float4 a = w.ac[i];
    const float2 b = w.pbuild[i];
    const int s = (int)meta_scene(m);
    if (!w.act[s]) return;
    const ScenePar &P = w.par[s];
    if (p.z == 0.0f) return;                                       // :83
    const bool ext = w.cc3[s] != 0;
    lom_core(w, P, P, i, m, p, v, a, b, ext, ext ? w.dp[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f), true, w.pr, w.dp);
}

// With w.ticket the kernel's last warp sets the rebuild conditional; without
// it (large worlds, where thousands of fenced ticket atomics cost more than a
// launch) k_decide does it.
// a 128-particle chunk holding at least one particle of a scene (served
// worlds keep the map; elsewhere every chunk is live).  Warps never straddle
// chunks, so the test is warp-uniform.
__device__ __forceinline__ bool chunk_live(const DevWorld &w, int i) {
    return w.live == nullptr || __ldg(&w.live[i >> 7]) != 0;
}

__global__ void __launch_bounds__(PK_MAX_THREADS) k_lom(DevWorld w, int in_graph, cudaGraphConditionalHandle cond) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < w.N && chunk_live(w, i)) lom_particle(w, i);
    if (w.ticket && last_warp(&w.tickets[0])) {
        if ((threadIdx.x & 31) == 0) {
            int need = *(volatile int32_t *)w.rebuild;
            if (in_graph) cudaGraphSetConditional(cond, need != 0 ? 1u : 0u);
            w.tickets[0] = 0u;
        }
    }
}

__global__ void k_decide(DevWorld w, cudaGraphConditionalHandle cond) {
    if (threadIdx.x == 0) cudaGraphSetConditional(cond, *(volatile int32_t *)w.rebuild != 0 ? 1u : 0u);
}

int launch_lom(const DevWorld &w, int block, cudaStream_t st, bool in_graph,
               cudaGraphConditionalHandle cond) {
    int k = 0;
    if (w.N > 0) {
        k_lom<<<(w.N + block - 1) / block, block, 0, st>>>(w, in_graph ? 1 : 0, cond);
        k++;
    }
    if (in_graph && (!w.ticket || w.N == 0)) {
        k_decide<<<1, 32, 0, st>>>(w, cond);
        k++;
    }
    return k;
}

// ------------------------------------------------------------ broad phase
// Every kernel of the rebuild takes a gate: when the gate word is 0 the
// kernel returns at once (plain launches); inside a graph the whole rebuild
// sits under a conditional node and the gate is always 1.
__device__ __forceinline__ bool gated_off(const int32_t *gate) {
    return gate != nullptr && *(volatile const int32_t *)gate == 0;
}
// The reorder kernels (grouping, inverse, gather, copy back) run only in the
// rebuilds that also reorder: every reorder_every-th, and the first after a
// change of layout.  In the others the cell list keeps naming the particles
// at their current internal indices.
__device__ __forceinline__ bool reorder_off(const DevWorld &w, const int32_t *gate) {
    return gated_off(gate) || *(volatile const int32_t *)w.reorder == 0;
}

// Grids of the rebuild kernels are capped at the blocks the SMs hold at
// once (the kernel's occupancy at that block size, times the SMs) and the
// kernels loop over their elements (windows, tiles): with plain launches
// every step launches them and most return at once, and retiring ~35,000
// empty blocks a launch would cost more than the step's real work.  When a
// rebuild runs, one full wave does the same work (a cap above the occupancy
// would leave a partial second wave of long-running blocks).  The candidate
// lists are the exception: inside a graph they are built on a full grid
// (launch_list_build).
static int resident_blocks(const void *fn, int block) {
    static std::mutex mu;
    static std::vector<std::tuple<const void *, int, int, int>> cache;  // kernel, block, device, blocks
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1 << 30;
    std::lock_guard<std::mutex> lock(mu);
    for (const auto &c : cache)
        if (std::get<0>(c) == fn && std::get<1>(c) == block && std::get<2>(c) == dev) return std::get<3>(c);
    int sms = 0, per = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, block, 0) != cudaSuccess || sms <= 0 ||
        per <= 0) {
        cudaGetLastError();
        return 1 << 30;  // uncapped: one block per chunk of elements
    }
    cache.emplace_back(fn, block, dev, sms * per);
    return sms * per;
}

// SMs of the current device (cached per device)
static int device_sms() {
    static std::mutex mu;
    static std::vector<std::pair<int, int>> cache;  // device, SMs
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    std::lock_guard<std::mutex> lock(mu);
    for (const auto &c : cache)
        if (c.first == dev) return c.second;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
        cudaGetLastError();
        return 1;
    }
    cache.emplace_back(dev, sms);
    return sms;
}

template <typename Kernel>
static int capped_grid(Kernel *kernel, long long items, int per_block, int block) {
    const long long need = (items + per_block - 1) / per_block;
    const int cap = resident_blocks(reinterpret_cast<const void *>(kernel), block);
    return (int)(need < cap ? need : cap);
}

#define FOR_EACH_ITEM(i, n) \
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += gridDim.x * blockDim.x)

// search-cell key of every particle (zero-radius ones go to their scene's
// dead cell) and the per-cell histogram
__device__ __forceinline__ void keys_one(const DevWorld &w, int i) {
    if (!chunk_live(w, i)) return;
    uint32_t m = w.meta[i];
    if (!w.act[meta_scene(m)]) return;  // frozen scenes keep their order and take no cells
    const ScenePar &P = w.par[meta_scene(m)];
    float4 p = w.pr[i];
    uint32_t key;
    if (p.z == 0.0f) {
        key = (uint32_t)P.dead_cell;
    } else if (m & M_BIG) {
        key = (uint32_t)P.big_cell;
    } else {
        int cx, cy;
        search_xy(P, p.x, p.y, cx, cy);
        key = (uint32_t)(P.cell_base + cy * P.g_w + cx);
    }
    w.keys[i] = key;
    atomicAdd(&w.cell_count[key], 1);
}

__global__ void __launch_bounds__(PK_MAX_THREADS) k_keys(DevWorld w, const int32_t *gate) {
    if (gated_off(gate)) return;
    FOR_EACH_ITEM(i, w.N) keys_one(w, i);
}

void launch_keys(const DevWorld &w, int block, cudaStream_t st, const int32_t *gate) {
    if (w.N == 0) return;
    k_keys<<<capped_grid(k_keys, w.N, block, block), block, 0, st>>>(w, gate);
}

// Exclusive scan of the per-cell counts with warp-shuffle scans: each block
// scans SCAN_TILE counts, a single block scans the tile sums, a third pass
// adds the tile offsets.
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_PER_THREAD = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_PER_THREAD;

__device__ __forceinline__ int warp_incl_scan(int v) {
    int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// block-wide exclusive scan of one value per thread; returns the block total in *total
__device__ __forceinline__ int block_excl_scan(int v, int *total) {
    __shared__ int wsum[SCAN_THREADS / 32];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int inc = warp_incl_scan(v);
    if (lane == 31) wsum[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int x = lane < SCAN_THREADS / 32 ? wsum[lane] : 0;
        int y = warp_incl_scan(x);
        if (lane < SCAN_THREADS / 32) wsum[lane] = y - x;
        if (lane == SCAN_THREADS / 32 - 1) *total = y;
    }
    __syncthreads();
    int r = inc - v + wsum[wid];
    __syncthreads();
    return r;
}

// clear: when set, every count read is set back to 0 (the world's cell
// counts start the next rebuild's histogram from zero)
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tiles(int32_t *__restrict__ in,
                                                             int32_t *__restrict__ out, int n,
                                                             int32_t *__restrict__ tile_sums,
                                                             const int32_t *gate, int clear) {
    if (gated_off(gate)) return;
    __shared__ int total;
    const int ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {  // uniform for the block
        int base = tile * SCAN_TILE + threadIdx.x * SCAN_PER_THREAD;
        int v[SCAN_PER_THREAD];
        int sum = 0;
#pragma unroll
        for (int k = 0; k < SCAN_PER_THREAD; ++k) {
            int idx = base + k;
            v[k] = idx < n ? in[idx] : 0;
            sum += v[k];
        }
        if (clear) {
#pragma unroll
            for (int k = 0; k < SCAN_PER_THREAD; ++k)
                if (base + k < n) in[base + k] = 0;
        }
        int off = block_excl_scan(sum, &total);
#pragma unroll
        for (int k = 0; k < SCAN_PER_THREAD; ++k) {
            int idx = base + k;
            if (idx < n) out[idx] = off;
            off += v[k];
        }
        if (threadIdx.x == 0) tile_sums[tile] = total;
        __syncthreads();  // `total` is rewritten by the next tile's scan
    }
}

// single block: exclusive scan of the tile sums in place; writes the grand total to out[n]
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_sums(int32_t *tile_sums, int ntiles,
                                                            int32_t *out, int n, const int32_t *gate) {
    if (gated_off(gate)) return;
    __shared__ int total;
    int carry = 0;
    for (int base = 0; base < ntiles; base += SCAN_THREADS) {
        int idx = base + threadIdx.x;
        int v = idx < ntiles ? tile_sums[idx] : 0;
        int off = block_excl_scan(v, &total);
        if (idx < ntiles) tile_sums[idx] = carry + off;
        carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) out[n] = carry;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_add(int32_t *out, int n,
                                                           const int32_t *tile_sums,
                                                           const int32_t *gate) {
    if (gated_off(gate)) return;
    const int ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        int add = tile_sums[tile];
        int base = tile * SCAN_TILE + threadIdx.x * SCAN_PER_THREAD;
#pragma unroll
        for (int k = 0; k < SCAN_PER_THREAD; ++k) {
            int idx = base + k;
            if (idx < n) out[idx] += add;
        }
    }
}

int scan_tmp_size(int n) { return (n + SCAN_TILE - 1) / SCAN_TILE + 1; }

// Stable counting sort of the particles by search-cell key (dem_sort.cuh).
// The sequence is the scenes' particles in scene-local index order -- position
// t = particle_base + scene-local index, the particle being o2i[t] -- so the
// members of every cell come out in scene-local index order, the order in
// which the reference's insertion loop (2D_LOM.wgsl:165-200) would fill its
// buckets if its threads ran in index order.  Positions of frozen scenes and
// of free chunks take no part, as in the histogram (keys_one).
struct SortWorldFirst {
    const uint8_t *live;
    const uint32_t *meta;
    const int32_t *act;
    const int32_t *o2i;
    const uint32_t *keys;
    int n;
    __device__ __forceinline__ int length() const { return n; }
    __device__ __forceinline__ bool get(int t, uint32_t &k, int32_t &v) const {
        if (live != nullptr && __ldg(&live[t >> 7]) == 0) return false;
        if (!act[meta_scene(meta[t])]) return false;  // the scene owning position t
        const int i = o2i[t];
        k = keys[i];
        v = i;
        return true;
    }
};

// Grouping by contact count: within each window of WIN consecutive
// cell-order positions, the particles of a scene's search cells are put in
// order of (any occupied slot bonded, number of occupied slots), ties by
// position, so that the warps of the Simulation kernels hold particles with
// similar contact (and candidate) counts and the same kind of slots, and
// diverge less (c2: 3.7 % per step from the bonded flag); particles stay in
// their window, so neighbours stay close in memory.  Positions of other
// scenes, and of the
// large and zero-radius particles' cells, do not move.  No result depends on
// the order: every order-dependent choice keys on original indices.
// wperm[r] = the position the particle at cell-order position r takes.
// Windows of 128 suit batches of many scenes, which rebuild more often;
// a single large scene gains from windows of 1024.
template <int WIN>
__device__ __forceinline__ void window_order_one(const DevWorld &w, int r0, int total, uint32_t *key,
                                                 uint32_t *seg_id, int *wsum) {
    constexpr int LB = WIN == 1024 ? 10 : 7;  // log2(WIN)
    const int lane = threadIdx.x;
    const int r = r0 + lane;
    const bool valid = r < total;
    uint32_t sid = 0xFFFFFFFFu, cnt = 0u;
    if (valid) {
        const int old = w.sorted[r];
        const uint32_t s = meta_scene(w.meta[old]);
        const ScenePar &P = w.par[s];
        const bool search = r < w.cell_start[P.big_cell];
        sid = (s << 1) | (search ? 0u : 1u);
        // 5 bits: whether an occupied slot is bonded (bond and contact
        // arithmetic differ, so bonded and unbonded lanes would run both),
        // then the number of occupied slots
        const uint32_t sm = w.smask[old];
        const uint32_t occ = sm & ((1u << K) - 1u);
        const uint32_t bonded = (sm >> BSHIFT) & occ;
        cnt = search ? ((bonded != 0u ? 16u : 0u) | (uint32_t)__popc(occ)) : 0u;
    }
    seg_id[lane] = sid;
    __syncthreads();
    // segment number within the window: segments start where the scene or
    // the region (search cells / large and dead cells) changes
    const bool start = lane == 0 || seg_id[lane] != seg_id[lane - 1];
    const unsigned bal = __ballot_sync(0xffffffffu, start);
    if ((lane & 31) == 0) wsum[lane >> 5] = __popc(bal);
    __syncthreads();
    uint32_t seg = (uint32_t)__popc(bal & ((2u << (lane & 31)) - 1u));
    for (int q = 0; q < (lane >> 5); ++q) seg += (uint32_t)wsum[q];
    // unique keys: segment, bonded flag and slot count (search cells only),
    // position (segment < 2^11, so 11 + 5 + 10 bits)
    key[lane] = valid ? (seg << (LB + 5)) | (cnt << LB) | (uint32_t)lane : 0xFFFFFFFFu;
    __syncthreads();
    for (int size = 2; size <= WIN; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            const int partner = lane ^ stride;
            if (partner > lane) {
                const uint32_t a = key[lane], b = key[partner];
                if ((a > b) == ((lane & size) == 0)) {
                    key[lane] = b;
                    key[partner] = a;
                }
            }
            __syncthreads();
        }
    const uint32_t ks = key[lane];
    if (ks != 0xFFFFFFFFu) w.wperm[r0 + (int)(ks & (WIN - 1))] = r0 + lane;
}

template <int WIN>
__global__ void __launch_bounds__(WIN) k_window_order(DevWorld w, const int32_t *gate) {
    if (reorder_off(w, gate)) return;
    __shared__ uint32_t key[WIN];
    __shared__ uint32_t seg_id[WIN];
    __shared__ int wsum[WIN / 32];
    const int total = w.cell_start[w.C];
    // one window per pass, the loop uniform for the block
    for (int r0 = blockIdx.x * WIN; r0 < total; r0 += gridDim.x * WIN) {
        window_order_one<WIN>(w, r0, total, key, seg_id, wsum);
        __syncthreads();  // the next window reuses the shared arrays
    }
}

void launch_exclusive_scan(const int32_t *in, int32_t *out, int n, int32_t *tmp, cudaStream_t st) {
    const int ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (ntiles > 0) k_scan_tiles<<<capped_grid(k_scan_tiles, ntiles, 1, SCAN_THREADS), SCAN_THREADS, 0, st>>>(
        const_cast<int32_t *>(in), out, n, tmp, nullptr, 0);
    k_scan_sums<<<1, SCAN_THREADS, 0, st>>>(tmp, ntiles, out, n, nullptr);
    if (ntiles > 0) k_scan_add<<<capped_grid(k_scan_add, ntiles, 1, SCAN_THREADS), SCAN_THREADS, 0, st>>>(
        out, n, tmp, nullptr);
}

// Cell start table (scan of the histogram, which it clears for the next
// rebuild), then the cell-ordered particle list by the stable counting sort:
// passes of 8 bits over the keys [0, C), ping-ponging through inv/wperm
// (keys) and src/sorted (particles), which the reorder rewrites afterwards;
// the last pass writes the particles to `sorted`.  Returns the kernels launched.
int launch_broad_phase(const DevWorld &w, int block, cudaStream_t st, const int32_t *gate) {
    (void)block;
    if (w.N == 0) return 0;
    int ntiles = (w.C + SCAN_TILE - 1) / SCAN_TILE;
    k_scan_tiles<<<capped_grid(k_scan_tiles, ntiles, 1, SCAN_THREADS), SCAN_THREADS, 0, st>>>(
        w.cell_count, w.cell_start, w.C, w.scan_tmp, gate, 1);
    k_scan_sums<<<1, SCAN_THREADS, 0, st>>>(w.scan_tmp, ntiles, w.cell_start, w.C, gate);
    k_scan_add<<<capped_grid(k_scan_add, ntiles, 1, SCAN_THREADS), SCAN_THREADS, 0, st>>>(w.cell_start, w.C,
                                                                                          w.scan_tmp, gate);
    int k = 3;
    const int passes = sort_passes(w.C);
    const int g = sort_grid(w.N, 2 * device_sms());
    uint32_t *keyA = reinterpret_cast<uint32_t *>(w.inv), *keyB = reinterpret_cast<uint32_t *>(w.wperm);
    SortWorldFirst first{w.live, w.meta, w.act, w.o2i, w.keys, w.N};
    SortArrays prev{nullptr, nullptr, 0, w.cell_start + w.C};
    for (int p = 0; p < passes; ++p) {
        const bool last = p == passes - 1;
        const bool setA = ((passes - 1 - p) & 1) != 0;  // odd distance from the last pass: inv/src
        uint32_t *ok = last ? nullptr : (setA ? keyA : keyB);
        int32_t *ov = last ? w.sorted : (setA ? w.src : w.sorted);
        if (p == 0) launch_sort_pass(first, 0, g, w.sort_counts, ok, ov, st, gate);
        else launch_sort_pass(prev, 8 * p, g, w.sort_counts, ok, ov, st, gate);
        prev.key = ok;
        prev.val = ov;
        k += 3;
    }
    if (w.S == 1)
        k_window_order<1024><<<capped_grid(k_window_order<1024>, w.N, 1024, 1024), 1024, 0, st>>>(w, gate);
    else
        k_window_order<128><<<capped_grid(k_window_order<128>, w.N, 128, 128), 128, 0, st>>>(w, gate);
    return k + 1;
}

// --------------------------------------------------------------- reorder
// Permute every per-particle array into cell order, grouped by contact count
// within windows (new i <- old src[i]), and remap partner indices; the cell
// list then names the new indices.  The particle at cell-order position k
// (sorted[k]) moves to its scene's range at the offset of its grouped
// position: new = particle_base + (wperm[k] - first position of the scene's
// cells).  Particles of frozen scenes stay where they are.
__device__ __forceinline__ void inverse_one(const DevWorld &w, int t) {
    if (t < w.cell_start[w.C]) {
        const int old = w.sorted[t];
        const ScenePar &P = w.par[meta_scene(w.meta[old])];
        const int nw = P.particle_base + (w.wperm[t] - w.cell_start[P.cell_base]);
        w.inv[old] = nw;
        w.src[nw] = old;
        w.sorted[t] = nw;  // the cell list names the new indices
    }
    if (chunk_live(w, t) && !w.act[meta_scene(w.meta[t])]) {  // free chunks are not gathered
        w.inv[t] = t;
        w.src[t] = t;
    }
}

__global__ void __launch_bounds__(PK_MAX_THREADS) k_inverse(DevWorld w, const int32_t *gate) {
    if (reorder_off(w, gate)) return;
    FOR_EACH_ITEM(t, w.N) inverse_one(w, t);
}

__device__ __forceinline__ void gather_one(const DevWorld &w, const DevWorld &o, int i) {
    if (!chunk_live(w, i)) return;  // a free chunk stays as it is
    int src = w.src[i];
    o.pr[i] = w.pr[src];
    o.vw[i] = w.vw[src];
    o.ac[i] = w.ac[src];
    o.dp[i] = w.dp[src];
    o.fx[i] = w.fx[src];
    o.d4[i] = w.d4[src];
    o.dF[i] = w.dF[src];
    o.meta[i] = w.meta[src];
    o.orig[i] = w.orig[src];
    o.smask[i] = w.smask[src];
    const int N = w.N;
#pragma unroll 2
    for (int j = 0; j < K; ++j) {
        int b = w.s_b[j * N + src];
        o.s_b[j * N + i] = (b >= 0 && b < N) ? w.inv[b] : b;
        o.s_bonded[j * N + i] = w.s_bonded[j * N + src];
        o.s_tf[j * N + i] = w.s_tf[j * N + src];
        o.s_btf[j * N + i] = w.s_btf[j * N + src];
        o.s_thb[j * N + i] = w.s_thb[j * N + src];
    }
    const int ss = (int)meta_scene(w.meta[src]);
    if (w.act[ss]) {
        const ScenePar &P = w.par[ss];
        w.o2i[P.particle_base + w.orig[src]] = i;
    }
}

__global__ void __launch_bounds__(PK_MAX_THREADS) k_gather(DevWorld w, DevWorld o, const int32_t *gate) {
    if (reorder_off(w, gate)) return;
    FOR_EACH_ITEM(i, w.N) gather_one(w, o, i);
}

// copy the permuted arrays back, so the live arrays keep their addresses
// (a rebuild may or may not run in a given step; addresses captured in a
// CUDA graph must not depend on it)
__device__ __forceinline__ void copy_back_one(const DevWorld &w, const DevWorld &o, int i) {
    if (!chunk_live(w, i)) return;
    w.pr[i] = o.pr[i];
    w.vw[i] = o.vw[i];
    w.ac[i] = o.ac[i];
    w.dp[i] = o.dp[i];
    w.fx[i] = o.fx[i];
    w.d4[i] = o.d4[i];
    w.dF[i] = o.dF[i];
    w.meta[i] = o.meta[i];
    w.orig[i] = o.orig[i];
    w.smask[i] = o.smask[i];
    const int N = w.N;
#pragma unroll 2
    for (int j = 0; j < K; ++j) {
        w.s_b[j * N + i] = o.s_b[j * N + i];
        w.s_bonded[j * N + i] = o.s_bonded[j * N + i];
        w.s_tf[j * N + i] = o.s_tf[j * N + i];
        w.s_btf[j * N + i] = o.s_btf[j * N + i];
        w.s_thb[j * N + i] = o.s_thb[j * N + i];
    }
}

__global__ void __launch_bounds__(PK_MAX_THREADS) k_copy_back(DevWorld w, DevWorld o, const int32_t *gate) {
    if (reorder_off(w, gate)) return;
    FOR_EACH_ITEM(i, w.N) copy_back_one(w, o, i);
}

void launch_reorder(const DevWorld &w, const DevWorld &spare, int block, cudaStream_t st,
                    const int32_t *gate) {
    if (w.N == 0) return;
    k_inverse<<<capped_grid(k_inverse, w.N, block, block), block, 0, st>>>(w, gate);
    k_gather<<<capped_grid(k_gather, w.N, block, block), block, 0, st>>>(w, spare, gate);
    k_copy_back<<<capped_grid(k_copy_back, w.N, block, block), block, 0, st>>>(w, spare, gate);
}

// ------------------------------------------------------- candidate lists
// After the reorder, each particle collects the particles of the 3x3 (or 5x5,
// with stencil 2) search cells around it whose centres lie within ra + rb + skin: a superset of
// every pair the reference can accept while no particle moves more than
// skin/2.  More than NL candidates, or one farther than an int16 offset can
// reach: the particle searches the cell table (built in the same rebuild) at
// every step instead.
// the list's first word h0 (count and flags) and the slot word's NL_LIVE bit
__device__ __forceinline__ void list_head(const DevWorld &w, int i, int16_t *h, int h0) {
    h[0] = (int16_t)h0;
    const uint32_t sm = w.smask[i];
    const uint32_t nsm = h0 != 0 ? (sm | NL_LIVE) : (sm & ~NL_LIVE);
    if (nsm != sm) w.smask[i] = nsm;
}

// Candidate lists one particle a thread in internal order, the cell table's
// cells read from global memory: the form for sparse worlds (about one
// particle a search cell or fewer, where a block's particles span too many
// cells for staging to pay).
__device__ __forceinline__ void list_build_one(const DevWorld &w, int i) {
    if (!chunk_live(w, i)) return;
    const uint32_t m = w.meta[i];
    const ScenePar &P = w.par[meta_scene(m)];
    const float4 pa = w.pr[i];
    w.pbuild[i] = make_float2(pa.x, pa.y);
    int16_t *h = reinterpret_cast<int16_t *>(w.nl + 2 * (size_t)i);
    if (!w.act[meta_scene(m)] || pa.z == 0.0f) {
        list_head(w, i, h, 0);
        w.kbuild[i] = (uint32_t)P.dead_cell;
        return;
    }
    if (m & M_BIG) {
        list_head(w, i, h, NL_BIG);
        w.kbuild[i] = (uint32_t)P.big_cell;
        return;
    }
    int gx, gy;
    search_xy(P, pa.x, pa.y, gx, gy);
    w.kbuild[i] = (uint32_t)(P.cell_base + gy * P.g_w + gx);
    const int cy0 = max(gy - P.stencil, 0), cy1 = min(gy + P.stencil, P.g_h - 1);
    const int cx0 = max(gx - P.stencil, 0), cx1 = min(gx + P.stencil, P.g_w - 1);
    int cnt = 0;
    bool over = false;
    for (int cy = cy0; cy <= cy1; ++cy) {
        const int row = P.cell_base + cy * P.g_w;
        const int beg = w.cell_start[row + cx0], end = w.cell_start[row + cx1 + 1];
        for (int k = beg; k < end; ++k) {
            const int b = w.sorted[k];
            if (b == i) continue;
            const float4 pb = w.pr[b];
            if (pb.z == 0.0f) continue;
            const float dx = pb.x - pa.x, dy = pb.y - pa.y;
            const float t = (pa.z + pb.z + P.skin) * 1.00001f;
            if (dx * dx + dy * dy > t * t) continue;
            const int off = b - i;
            if (cnt < NL && off >= -32768 && off <= 32767) h[1 + cnt] = (int16_t)off;
            else over = true;
            ++cnt;
        }
    }
    int flags = 0;
    if (P.n_big > 0) {
        int bf, bn;
        big_cell(w, P, bf, bn);
        for (int k = 0; k < bn; ++k) {
            const float4 pb = w.pr[w.sorted[bf + k]];
            const float dx = pb.x - pa.x, dy = pb.y - pa.y;
            const float t = (pa.z + pb.z + P.skin) * 1.00001f;
            if (pb.z != 0.0f && dx * dx + dy * dy <= t * t) {
                flags = NL_NEAR_BIG;
                break;
            }
        }
    }
    list_head(w, i, h, (over ? NL_OVERFLOW : cnt) | flags);
    if (over) atomicAdd(&w.stats[5], 1ull);
}

__global__ void __launch_bounds__(PK_MAX_THREADS) k_list_build(DevWorld w, const int32_t *gate) {
    if (gated_off(gate)) return;
    FOR_EACH_ITEM(i, w.N) list_build_one(w, i);
}

// The candidate-list head of a particle that is not in a search cell
// (frozen scene, zero radius, large particle) and its rebuild records;
// false for the others, whose lists k_list_tiles builds.
__device__ __forceinline__ bool list_head_only(const DevWorld &w, int i) {
    if (!chunk_live(w, i)) return true;
    const uint32_t m = w.meta[i];
    const ScenePar &P = w.par[meta_scene(m)];
    const float4 pa = w.pr[i];
    int16_t *h = reinterpret_cast<int16_t *>(w.nl + 2 * (size_t)i);
    if (!w.act[meta_scene(m)] || pa.z == 0.0f) {
        w.pbuild[i] = make_float2(pa.x, pa.y);
        list_head(w, i, h, 0);
        w.kbuild[i] = (uint32_t)P.dead_cell;
        return true;
    }
    if (m & M_BIG) {
        w.pbuild[i] = make_float2(pa.x, pa.y);
        list_head(w, i, h, NL_BIG);
        w.kbuild[i] = (uint32_t)P.big_cell;
        return true;
    }
    return false;
}

__global__ void __launch_bounds__(PK_MAX_THREADS) k_list_heads(DevWorld w, const int32_t *gate) {
    if (gated_off(gate)) return;
    FOR_EACH_ITEM(i, w.N) list_head_only(w, i);
}

// Candidate lists of the particles in search cells, a block per LT_THREADS
// consecutive entries of the cell list (cell order: each scene's grid row by
// row), one particle per thread.  When the block's particles lie in at most
// LT cells [c0, c1) of one scene, the block first stages in shared memory
// the cell starts and the particles (index and position record) of the cell
// ranges [c0 + d g_w - st, c1 + d g_w + st), d in [-st, st]: every
// neighbour cell of those cells, whether or not the run wraps a grid row.
// Each particle then scans its (2 st + 1)^2 cells there, rows top to bottom
// and cells and members in cell order -- the order and the test of a scan
// of the cell table, so the lists are the same.  Rows the staging does not
// hold (a sparse run of cells, more than LT_CAP particles, another scene's
// particle) are read from the cell table.
constexpr int LT = 256;              // cells a block's particles may span for staging
constexpr int LT_ST = 2;             // largest stencil the staging holds
constexpr int LT_ROWS = 2 * LT_ST + 1;
constexpr int LT_CELLS = LT + 2 * LT_ST + 1;  // cell starts per staged row (one more than its cells)
constexpr int LT_CAP = 512;          // staged particles per block
constexpr int LT_THREADS = 128;

struct ListScan {
    int cnt = 0;
    bool over = false;
};

__device__ __forceinline__ void list_consider(const ScenePar &P, int i, float4 pa, int b, float4 pb, int16_t *h,
                                              ListScan &ls) {
    if (b == i) return;
    if (pb.z == 0.0f) return;
    const float dx = pb.x - pa.x, dy = pb.y - pa.y;
    const float t = (pa.z + pb.z + P.skin) * 1.00001f;
    if (dx * dx + dy * dy > t * t) return;
    const int off = b - i;
    if (ls.cnt < NL && off >= -32768 && off <= 32767) h[1 + ls.cnt] = (int16_t)off;
    else ls.over = true;
    ++ls.cnt;
}

// the search cell of a particle in a search cell (as keys_one files it), or -1
__device__ __forceinline__ int regular_cell(const DevWorld &w, int b, int &scene) {
    const uint32_t m = w.meta[b];
    scene = (int)meta_scene(m);
    const ScenePar &P = w.par[scene];
    const float4 p = w.pr[b];
    if (p.z == 0.0f || (m & M_BIG)) return -1;
    int cx, cy;
    search_xy(P, p.x, p.y, cx, cy);
    return P.cell_base + cy * P.g_w + cx;
}

__global__ void __launch_bounds__(LT_THREADS) k_list_tiles(DevWorld w, const int32_t *gate) {
    if (gated_off(gate)) return;
    __shared__ float4 s_pr[LT_CAP];
    __shared__ int32_t s_idx[LT_CAP];
    __shared__ int32_t s_cs[LT_ROWS * LT_CELLS];
    __shared__ int32_t s_lo[LT_ROWS], s_hi[LT_ROWS], s_off[LT_ROWS];
    __shared__ int s_scene, s_ca[2], s_sa[2];
    const int total = w.cell_start[w.C];  // particles in cells
    const int runs = (total + LT_THREADS - 1) / LT_THREADS;
    for (int run = blockIdx.x; run < runs; run += gridDim.x) {
        const int first = run * LT_THREADS, last = min(first + LT_THREADS, total) - 1;
        __syncthreads();  // the previous run's staging is no longer read
        // the cells of the run's first and last particles (two threads), then
        // each staged row's range (one thread a row), then their offsets
        if (threadIdx.x < 2) s_ca[threadIdx.x] = regular_cell(w, w.sorted[threadIdx.x ? last : first], s_sa[threadIdx.x]);
        __syncthreads();
        const int ca = s_ca[0], cb = s_ca[1], sa = s_sa[0];
        const bool stage = ca >= 0 && cb >= 0 && sa == s_sa[1] && cb - ca < LT && w.par[sa].stencil <= LT_ST;
        if (stage && threadIdx.x < LT_ROWS) {
            const int r = threadIdx.x;
            const ScenePar &P = w.par[sa];
            const int st = P.stencil, gw = P.g_w;
            const int glo = P.cell_base, ghi = P.cell_base + P.g_w * P.g_h;  // the scene's search cells
            const int d = r - LT_ST;
            const int lo = max(ca + d * gw - st, glo), hi = min(cb + 1 + d * gw + st, ghi);
            s_lo[r] = lo;
            s_hi[r] = hi;
            s_off[r] = (d < -st || d > st || lo >= hi) ? -1 : w.cell_start[hi] - w.cell_start[lo];  // count
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int off = 0;
            if (stage)
                for (int r = 0; r < LT_ROWS; ++r) {
                    const int n = s_off[r];
                    if (n < 0 || off + n > LT_CAP) {
                        s_off[r] = -1;  // not staged: read from the cell table
                        continue;
                    }
                    s_off[r] = off;
                    off += n;
                }
            s_scene = stage ? sa : -1;
        }
        __syncthreads();
        const int st_scene = s_scene;
        if (st_scene >= 0) {
            for (int r = 0; r < LT_ROWS; ++r) {
                if (s_off[r] < 0) continue;
                const int lo = s_lo[r], hi = s_hi[r];
                for (int k = threadIdx.x; k <= hi - lo; k += LT_THREADS)
                    s_cs[r * LT_CELLS + k] = w.cell_start[lo + k];
            }
            __syncthreads();
            for (int r = 0; r < LT_ROWS; ++r) {
                if (s_off[r] < 0) continue;
                const int base = s_cs[r * LT_CELLS], n = s_cs[r * LT_CELLS + (s_hi[r] - s_lo[r])] - base;
                for (int k = threadIdx.x; k < n; k += LT_THREADS) {
                    const int b = w.sorted[base + k];
                    s_idx[s_off[r] + k] = b;
                    s_pr[s_off[r] + k] = w.pr[b];
                }
            }
            __syncthreads();
        }
        const int q = first + (int)threadIdx.x;
        if (q > last) continue;
        const int i = w.sorted[q];
        if (!chunk_live(w, i)) continue;
        const uint32_t m = w.meta[i];
        const int s = (int)meta_scene(m);
        const ScenePar &P = w.par[s];
        const float4 pa = w.pr[i];
        if (!w.act[s] || pa.z == 0.0f || (m & M_BIG)) continue;  // k_list_heads
        w.pbuild[i] = make_float2(pa.x, pa.y);
        int16_t *h = reinterpret_cast<int16_t *>(w.nl + 2 * (size_t)i);
        int gx, gy;
        search_xy(P, pa.x, pa.y, gx, gy);
        w.kbuild[i] = (uint32_t)(P.cell_base + gy * P.g_w + gx);
        const int cy0 = max(gy - P.stencil, 0), cy1 = min(gy + P.stencil, P.g_h - 1);
        const int cx0 = max(gx - P.stencil, 0), cx1 = min(gx + P.stencil, P.g_w - 1);
        ListScan ls;
        for (int cy = cy0; cy <= cy1; ++cy) {
            const int row = P.cell_base + cy * P.g_w;
            const int a = row + cx0, z = row + cx1 + 1;  // cells [a, z)
            int hit = -1;
            if (s == st_scene)
                for (int r = 0; r < LT_ROWS; ++r)
                    if (s_off[r] >= 0 && s_lo[r] <= a && z <= s_hi[r]) {
                        hit = r;
                        break;
                    }
            if (hit >= 0) {
                const int *cs = s_cs + hit * LT_CELLS;
                const int at = s_off[hit] - cs[0];
                const int beg = cs[a - s_lo[hit]] + at, fin = cs[z - s_lo[hit]] + at;
                for (int k = beg; k < fin; ++k) list_consider(P, i, pa, s_idx[k], s_pr[k], h, ls);
            } else {
                const int beg = w.cell_start[a], fin = w.cell_start[z];
                for (int k = beg; k < fin; ++k) {
                    const int b = w.sorted[k];
                    list_consider(P, i, pa, b, w.pr[b], h, ls);
                }
            }
        }
        int flags = 0;
        if (P.n_big > 0) {
            int bf, bn;
            big_cell(w, P, bf, bn);
            for (int k = 0; k < bn; ++k) {
                const float4 pb = w.pr[w.sorted[bf + k]];
                const float dx = pb.x - pa.x, dy = pb.y - pa.y;
                const float t = (pa.z + pb.z + P.skin) * 1.00001f;
                if (pb.z != 0.0f && dx * dx + dy * dy <= t * t) {
                    flags = NL_NEAR_BIG;
                    break;
                }
            }
        }
        list_head(w, i, h, (ls.over ? NL_OVERFLOW : ls.cnt) | flags);
        if (ls.over) atomicAdd(&w.stats[5], 1ull);
    }
}

__global__ void k_rebuild_done(DevWorld w, const int32_t *gate) {
    if (gated_off(gate)) return;
    *w.rebuild = 0;
    const unsigned long long n = w.stats[4] + 1ull;
    w.stats[4] = n;
    // the next rebuild reorders when it is the first of a new group of reorder_every
    *w.reorder = (w.reorder_every <= 1 || n % (unsigned long long)w.reorder_every == 0ull) ? 1 : 0;
}

// every_step: launched at every step (plain launches), mostly to return at
// once, so on the capped grid; a rebuild that runs only when due (under a
// conditional graph node) takes one block per chunk instead, since particles
// differ widely in candidate work and the hardware then balances the blocks
// (a single 4 M-particle scene rebuilds 0.5 % faster per step that way)
// staged: the dense form (k_list_heads + k_list_tiles), else k_list_build;
// both build the same lists
int launch_list_build(const DevWorld &w, int block, cudaStream_t st, const int32_t *gate, bool every_step,
                      bool staged) {
    if (w.N == 0) return 0;
    if (staged) {
        k_list_heads<<<capped_grid(k_list_heads, w.N, block, block), block, 0, st>>>(w, gate);
        const long long runs = ((long long)w.N + LT_THREADS - 1) / LT_THREADS;  // particles in cells <= N
        const int g = every_step ? capped_grid(k_list_tiles, runs, 1, LT_THREADS) : (int)runs;
        k_list_tiles<<<g, LT_THREADS, 0, st>>>(w, gate);
    } else {
        const int g = every_step ? capped_grid(k_list_build, w.N, block, block) : (w.N + block - 1) / block;
        k_list_build<<<g, block, 0, st>>>(w, gate);
    }
    k_rebuild_done<<<1, 1, 0, st>>>(w, gate);
    return staged ? 3 : 2;
}

// -------------------------------------------------------------- interact
// 2D_Simulation.wgsl:108-262 per particle.
//
// Narrow phase: the reference accepts partner b when b's AABB shares a bucket
// with the particle's AABB (both inserted into every bucket their AABB covers,
// 2D_LOM.wgsl:180-199) and |p_b - p_a| < r_b + r_a; it stops at 14 and keeps
// them in bucket-scan order (rows top to bottom, columns left to right,
// bucket members in insertion order).  Here candidates come from the
// particle's candidate list (or the 3x3 cells of the last rebuild), the same
// acceptance test is evaluated exactly, and accepted partners are ordered by
// (first shared bucket in scan order, particle index) -- the bucket-scan
// order with insertion in index order -- keeping the first 14.
constexpr int IB = 128;  // threads per k_interact block

// The accepted partners of one thread, kept sorted by (first shared bucket,
// particle index) in shared memory (slot-major, so a warp's accesses fall in
// distinct banks): key = rank << 28 | scene-local index.
__shared__ uint32_t nr_ck[K * IB];  // [K][IB] sort keys of the accepted partners
__shared__ int nr_ci[K * IB];       // [K][IB] their internal indices

struct Narrow {
    int cnt;
};

__device__ __forceinline__ void top14_insert(uint32_t key, int idx, Narrow &nr) {
    const int t = threadIdx.x;
    if (nr.cnt == K && key >= nr_ck[(K - 1) * IB + t]) return;
    int pos = nr.cnt < K ? nr.cnt : K - 1;
    while (pos > 0 && nr_ck[(pos - 1) * IB + t] > key) {
        nr_ck[pos * IB + t] = nr_ck[(pos - 1) * IB + t];
        nr_ci[pos * IB + t] = nr_ci[(pos - 1) * IB + t];
        --pos;
    }
    nr_ck[pos * IB + t] = key;
    nr_ci[pos * IB + t] = idx;
    if (nr.cnt < K) ++nr.cnt;
}

// |p_b - p_a| < r_b + r_a (2D_Simulation.wgsl:159).  The square root is only
// taken near the boundary: while t*t is a normal float, s2 > t*t*1.000001
// cannot pass and s2 < t*t*0.999999 must (each side leaves more than 8e-7
// relative margin for the roundings of t*t, of the factor and of sqrtf), so
// both shortcuts give the result of the full test.
__device__ __forceinline__ bool touching(float4 pa, float4 pb) {
    const float dx = pb.x - pa.x, dy = pb.y - pa.y;
    const float s2 = dx * dx + dy * dy;
    const float t = pb.z + pa.z;
    const float t2 = t * t;
    if (t2 >= 1e-30f) {
        if (s2 > t2 * 1.000001f) return false;
        if (s2 < t2 * 0.999999f) return true;
    }
    return sqrtf(s2) < t;
}

// b (range code cb) passed the distance test: keep it when its AABB shares a
// reference bucket with the particle's (range code ca), keyed by the first
// shared bucket
__device__ __forceinline__ void accept_partner(const DevWorld &w, int b, uint32_t ca, uint32_t cb, Narrow &nr) {
    unsigned rank;
    if (!shared_bucket(w, ca, cb, rank)) return;
    const uint32_t key = (rank << 28) | (uint32_t)__ldg(&w.orig[b]);
    top14_insert(key, b, nr);
}

__device__ __forceinline__ void narrow_test(const DevWorld &w, int i, int b, float4 pa, Narrow &nr) {
    if (b == i) return;
    const float4 pb = __ldg(&w.pr[b]);
    if (!touching(pa, pb)) return;
    accept_partner(w, b, __float_as_uint(pa.w), __float_as_uint(pb.w), nr);
}

// entry k (0..15) of a candidate list held in two int4
__device__ __forceinline__ int nl_entry(int4 a, int4 b, int k) {
    const int q = k >> 1;
    const int v = q == 0 ? a.x : q == 1 ? a.y : q == 2 ? a.z : q == 3 ? a.w
                : q == 4 ? b.x : q == 5 ? b.y : q == 6 ? b.z : b.w;
    return (k & 1) ? (v >> 16) : (int)(int16_t)(v & 0xFFFF);
}

// L1 prefetch of one line (sm_90+ PTX): the later load of the same address
// finds it on chip instead of waiting a DRAM round trip then.
__device__ __forceinline__ void prefetch_l1(const void *p) {
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

// The Simulation pass of one particle.  PART selects what runs: 0 all of it
// (k_interact), 1 the narrow phase and slot bookkeeping (k_narrow), 2 the
// force loop and store_forces (k_forces) -- the split form trades a second
// read of the particle's records for two kernels with fewer registers,
// which pays in dense scenes.
// With FUSE the particle's LOM pass of the next step follows at once
// (2D_LOM.wgsl:85-152 with this step's accelerations and velocities, as the
// next step's LOM would read them): its position, displacement and bucket
// range go to the other buffers (pr_n, dp_n), because neighbours still
// read this step's values.  Particles that do not step on (zero radius, or a
// served scene at its horizon) copy theirs across.
// Accelerations and data[0..2] (this pass) and data[4..6] (the LOM pass) are
// seen only by the caller after a call returns, and every step overwrites
// them; a fused step whose scene steps on within the call therefore leaves
// them to the scene's last step of the call (lom_final: the next step is the
// call's last).  Results are unchanged; the intermediate writes are saved.
// FORM: what the world's scenes need, fixed at compile time so that the
// rest (and the registers it holds) drops out: 0 or 3, every scene uses that
// bond model and none the F64 distances; -2, any bond model, no F64
// distances; -1, anything.  Only -1 carries the double-precision paths.
// PS: where the scene parameters come from.  PS_SCENE: w.par[scene].
// PS_ONE: the world holds a single scene, whose parameters come with the
// launch (Pv, in the kernel's parameter space): the instructions then read
// them where they are used, with no load and no register held for them (on
// the 4 M-particle impact scene the force kernel's spills disappear and the
// Simulation kernels take 7.7 % less time).  PS_SHARED: the scenes differ
// only in geometry and record bases; their common settings and model
// constants (the fields read through U) come with the launch, the rest from
// w.par[scene].  Every field read through U is one that shared_settings
// (dem_world.cuh) copies (tests/test_param_source.py checks this source).
template <int PART, bool FUSE, int FORM, int PS>
__device__ __forceinline__ void interact_particle(const DevWorld &w, int i, Narrow &nr, bool lom_final,
                                                  const ScenePar &Pv) {
    // The particle's own records: the ones needed first are loaded now, the
    // rest (read only after the scene, detection and slot checks resolve)
    // are prefetched now, so the DRAM round trips overlap instead of
    // following one another.
    const uint32_t m = w.meta[i];
    const float4 pa = w.pr[i];
    uint32_t mask = w.smask[i];
    if (PART != 1) {
        prefetch_l1(&w.vw[i]);
        if (FUSE) prefetch_l1(&w.pbuild[i]);
    }
    // the candidate list only when it is not empty, del_pos only for a
    // particle with contacts (its force loop reads it)
    if (PART != 2 && (mask & NL_LIVE)) prefetch_l1(&w.nl[2 * (size_t)i]);
    if (PART != 1 && (mask & ((1u << K) - 1u))) prefetch_l1(&w.dp[i]);
    const int N = w.N;
    for (uint32_t left = mask & ((1u << K) - 1u); left; left &= left - 1) {
        const int j = __ffs(left) - 1;
        prefetch_l1(&w.s_b[j * N + i]);
        if (PART != 1) prefetch_l1(&w.s_tf[j * N + i]);
        if ((mask >> (BSHIFT + j)) & 1u) prefetch_l1(&w.s_bonded[j * N + i]);
    }
    const int s = (int)meta_scene(m);
    if (!w.act[s]) return;
    const ScenePar &P = PS == PS_ONE ? Pv : w.par[s];
    const ScenePar &U = PS == PS_SCENE ? P : Pv;
    if (pa.z == 0.0f) {                                            // :113-118
        if (PART != 1) w.dF[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (FUSE) {
            w.pr_n[i] = pa;
            w.dp_n[i] = w.dp[i];
        }
        return;
    }
    const uint32_t before = mask;
    const int bonds_model = FORM == 0 ? 0 : FORM == 3 ? 3 : U.p.bonds;
    constexpr bool MAY_F64 = FORM == -1;

    // Loads that only some particles need (the bucket range, the second half
    // of the candidate list, del_pos) wait until the particle needs them.
    const bool detect = PART != 2 && U.p.collisions == 1 && w.det[s] != 0;
    if (detect) {                                                  // :126-228
        nr.cnt = 0;
        const uint32_t ca = __float_as_uint(pa.w);  // the particle's bucket range
        bool direct = false;       // accepted partners that own a slot only mark it found
        int n_acc = 0;             // partners accepted in direct mode
        uint32_t found_slots = 0u;
        const int4 la = (mask & NL_LIVE) ? __ldg(&w.nl[2 * (size_t)i]) : make_int4(0, 0, 0, 0);
        const int h0 = la.x & 0xFFFF;
        const int lc = h0 & 0xFF;
        if (lc == NL_BIG) {
            // a large particle: k_big_narrow left its partners, in order, in
            // the record of the particle's rank in its cell (list word 1)
            const int32_t *acc_g = w.big_acc + 16 * (size_t)(P.big_base + la.y);
            const int n = acc_g[15];
            for (int q = 0; q < n; ++q) nr_ci[q * IB + threadIdx.x] = acc_g[q];
            nr.cnt = n;
        } else if (lc != NL_OVERFLOW) {
            const int4 lb = lc > 7 ? __ldg(&w.nl[2 * (size_t)i + 1]) : make_int4(0, 0, 0, 0);
            // distance tests first, all gathers independent; then the bucket
            // test and ordering of the partners that touch.  The unrolled
            // tests stop at the longest list among the warp's lanes here
            // (a warp-uniform exit: sparse warps skip the empty tail).
            uint32_t pass = 0u;
            const int lmax = __reduce_max_sync(__activemask(), lc);
#pragma unroll
            for (int k = 1; k <= NL; ++k) {
                if (k > lmax) break;
                if (k <= lc && touching(pa, __ldg(&w.pr[i + nl_entry(la, lb, k)]))) pass |= 1u << k;
            }
            // With at most 14 partners touching and no large particle near,
            // the accepted list is never cut at 14, so a partner that already
            // owns a slot needs no key: it only marks the slot found.  The
            // others are keyed and ordered for creation as usual.
            direct = !(h0 & NL_NEAR_BIG) && __popc(pass) <= K;
            if (direct) {
                for (; pass; pass &= pass - 1) {
                    const int b = i + nl_entry(la, lb, __ffs(pass) - 1);
                    unsigned rank;
                    if (!shared_bucket(w, ca, range_of(w, b), rank)) continue;
                    ++n_acc;
                    uint32_t hit = 0u;
                    for (uint32_t left = mask & ((1u << K) - 1u); left; left &= left - 1) {
                        const int j = __ffs(left) - 1;
                        if (w.s_b[j * N + i] == b) hit |= 1u << j;
                    }
                    if (hit) {
                        found_slots |= hit;
                        continue;
                    }
                    top14_insert((rank << 28) | (uint32_t)__ldg(&w.orig[b]), b, nr);
                }
            } else {
                for (; pass; pass &= pass - 1) {
                    const int b = i + nl_entry(la, lb, __ffs(pass) - 1);
                    accept_partner(w, b, ca, range_of(w, b), nr);
                }
            }
            if (h0 & NL_NEAR_BIG) {
                int bf, bn;
                big_cell(w, P, bf, bn);
                for (int k = 0; k < bn; ++k) narrow_test(w, i, w.sorted[bf + k], pa, nr);
            }
        } else {
            if (P.n_big > 0) {
                int bf, bn;
                big_cell(w, P, bf, bn);
                for (int k = 0; k < bn; ++k) narrow_test(w, i, w.sorted[bf + k], pa, nr);
            }
            const int local = (int)w.kbuild[i] - P.cell_base;
            const int gx = local % P.g_w, gy = local / P.g_w;
            const int cy0 = max(gy - P.stencil, 0), cy1 = min(gy + P.stencil, P.g_h - 1);
            const int cx0 = max(gx - P.stencil, 0), cx1 = min(gx + P.stencil, P.g_w - 1);
            for (int cy = cy0; cy <= cy1; ++cy) {
                const int row = P.cell_base + cy * P.g_w;
                const int beg = w.cell_start[row + cx0], end = w.cell_start[row + cx1 + 1];
                for (int k = beg; k < end; ++k) narrow_test(w, i, w.sorted[k], pa, nr);
            }
        }
        const int cnt = nr.cnt;
        const int t = threadIdx.x;
        if ((direct ? n_acc : cnt) == K) atomicAdd(&w.stats[0], 1ull);
        // delete contacts that were not found (:185-204); `matched` marks the
        // accepted partners that already own a slot
        uint32_t matched = 0u;
        for (uint32_t left = mask & ((1u << K) - 1u); left; left &= left - 1) {
            const int j = __ffs(left) - 1;
            bool found = (found_slots >> j) & 1u;
            if (!direct) {
                const int sb = w.s_b[j * N + i];
                for (int q = 0; q < cnt; ++q) {
                    const bool hit = nr_ci[q * IB + t] == sb;
                    found |= hit;
                    matched |= hit ? (1u << q) : 0u;
                }
            }
            if (found) continue;
            const bool bonded_nn = (mask >> (BSHIFT + j)) & 1u;   // bonded >= 0
            if (!bonded_nn || bonds_model == 0) {
                mask &= ~(1u << j);
            } else if (bonds_model <= 1 && w.s_bonded[j * N + i] > 0) {
                w.s_tf[j * N + i] = 0.0f;
            }
        }
        // create new contacts in the last empty slot (:207-227); a deleted
        // slot never holds an accepted partner, so `matched` is the
        // reference's "existing" test
        for (int q = 0; q < cnt; ++q) {
            if ((matched >> q) & 1u) continue;
            const uint32_t empty = (~mask) & ((1u << K) - 1u);
            if (empty == 0u) continue;
            const int j = 31 - __clz(empty);
            mask |= 1u << j;
            w.s_b[j * N + i] = nr_ci[q * IB + t];
            w.s_tf[j * N + i] = 0.0f;
        }
    }

    if (PART == 1) {
        if (mask != before) w.smask[i] = mask;
        return;
    }

    // force loop (:230-255), slots in ascending order
    // Per slot, every load is issued before any result is used: the slot
    // fields, then what they index (partner records, bond records), so a
    // slot costs two dependent memory round trips instead of five.
    const float4 da = (mask & ((1u << K) - 1u)) ? w.dp[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float nfx = 0.0f, nfy = 0.0f, nm = 0.0f;
    Acc3 acc = {0.0f, 0.0f, 0.0f};
    for (uint32_t left = mask & ((1u << K) - 1u); left; left &= left - 1) {
        const int j = __ffs(left) - 1;
        const bool bnn = (mask >> (BSHIFT + j)) & 1u;              // bonded >= 0
        const int b = w.s_b[j * N + i];
        const float tf0 = w.s_tf[j * N + i];
        int bonded = -1;                                           // any negative value acts alike
        float btf0 = 0.0f, thb0 = 0.0f;
        if (bnn) {
            bonded = w.s_bonded[j * N + i];
            if (bonds_model == 3) {
                btf0 = w.s_btf[j * N + i];
                thb0 = w.s_thb[j * N + i];
            }
        }
        const float4 pb = __ldg(&w.pr[b]);
        const float4 db = __ldg(&w.dp[b]);
        const uint32_t mb = U.n_mat == 1 ? 0u : __ldg(&w.meta[b]);
        int st = 0;
        float blen = 0.0f;
        float2 str = make_float2(U.p.bond_normal_strength, U.p.bond_shear_strength);
        if (bnn) {
            const int bg = P.bond_base + bonded;
            st = w.b_status[bg];
            blen = w.b_length[bg];
            if (U.has_strength) str = w.b_str[bg];
        }
        if (st < 0) {                                              // :236-239
            w.s_bonded[j * N + i] = st;
            bonded = st;
            mask &= ~(1u << (BSHIFT + j));
        }
        const float2 kns = __ldg(&w.pair[P.pair_base + (int)meta_mat(m) * U.n_mat + (int)meta_mat(mb)]);
        float meff = 0.0f;  // effective mass of the pair, for the dashpot (generic form only)
        if (MAY_F64 && U.damp2 > 0.0f) {
            const float ma = ((w.mats[P.mat_base + meta_mat(m)].density * 3.14159274101257324219f) * pa.z) * pa.z;
            const float mbb = ((w.mats[P.mat_base + meta_mat(mb)].density * 3.14159274101257324219f) * pb.z) * pb.z;
            meff = (ma * mbb) / (ma + mbb);
        }
        F3 f = {0.0f, 0.0f, 0.0f};
        // L = |pa - pb| in float, taken once per slot where the branch needs
        // it: every float distance of the slot is this value (b - a differs
        // from a - b only in sign, so the squares agree)
        if (bonded < 0 || bonds_model == 0) {
            float tf = tf0;
            f = linear_model<MAY_F64>(U, kns, pa, da, pb, db, pa.z + pb.z, len2f(pa.x - pb.x, pa.y - pb.y), tf, acc,
                                     meff);
            w.s_tf[j * N + i] = tf;
        } else {
            const int bg = P.bond_base + bonded;
            const float sn = str.x, ss = str.y;
            if (bonds_model == 3) {                                // :286-336
                const float kn = U.p.bond_normal_stiffness, ks = U.p.bond_shear_stiffness;
                const float Rr = U.lambda * (pa.z < pb.z ? pa.z : pb.z);
                const float A = (2.0f * Rr) * 1.0f;
                const float I = ((2.0f / 3.0f * Rr) * Rr) * Rr;
                const float L = len2f(pa.x - pb.x, pa.y - pb.y);
                const float nd = (MAY_F64 && U.use_f64) ? distance2(1, pa, pb, blen) : L - blen;
                float Fn = ((-kn) * nd) * A;
                const float vx = pa.x - pb.x, vy = pa.y - pb.y;
                const float nx = vx / L, ny = vy / L;
                const float tx = -ny, ty = nx;
                const float dra = da.z * pa.z, drb = db.z * pb.z;
                const float rx = db.x - da.x, ry = db.y - da.y;
                const float rr = drb + dra;
                const float rt = (rx * tx + ry * ty) + rr;
                float btf = btf0;
                float thb = thb0;
                btf = btf + (rt * ks) * A;
                const float dtb = da.z - db.z;
                thb = thb + dtb;
                float M = (((-kn) * I) * thb) - btf * pa.z;
                float Fx = nx * Fn + tx * btf;
                float Fy = ny * Fn + ty * btf;
                float bend = ((-kn) * I) * thb;
                bend = bend < 0.0f ? -bend : bend;
                const float abtf = btf < 0.0f ? -btf : btf;
                if (U.p.bonds_tear == 1 &&
                    ((Fn / A) - (U.p.moment_contribution_factor * (bend * Rr)) / I < -sn ||
                     abtf / A > ss)) {
                    const int code = -10 + sign_i32(nd);
                    record_break(w, P, s, *w.step, bg, code, i, b);
                    w.s_bonded[j * N + i] = code;
                    mask &= ~(1u << (BSHIFT + j));
                    Fn = 0.0f;
                    btf = 0.0f;
                    Fx = 0.0f;
                    Fy = 0.0f;
                    M = 0.0f;
                }
                w.s_btf[j * N + i] = btf;
                w.s_thb[j * N + i] = thb;
                acc.d0 = acc.d0 + (-Fn);
                acc.d1 = acc.d1 + btf;
                acc.d2 = acc.d2 + M;
                float tf = tf0;
                const F3 lm = linear_model<MAY_F64>(U, kns, pa, da, pb, db, blen, L, tf, acc, meff);
                w.s_tf[j * N + i] = tf;
                f.x = Fx + lm.x;
                f.y = Fy + lm.y;
                f.z = M + lm.z;
            } else if (bonds_model == 1) {                         // :419-432
                const float L = len2f(pa.x - pb.x, pa.y - pb.y);
                const float disp = (MAY_F64 && U.use_f64) ? distance1(1, pa, pb) : L - (pa.z + pb.z);
                float fx = 0.0f, fy = 0.0f;
                const float sf = U.p.bond_normal_stiffness * disp;
                const float vx = pb.x - pa.x, vy = pb.y - pa.y;
                fx = fx + sf * (vx / L);
                fy = fy + sf * (vy / L);
                if (U.p.bonds_tear == 1 && sf >= sn) {
                    const int code = -10 + sign_i32(disp);
                    record_break(w, P, s, *w.step, bg, code, i, b);
                    w.s_bonded[j * N + i] = code;
                    mask &= ~(1u << (BSHIFT + j));
                    fx = 0.0f;
                    fy = 0.0f;
                }
                float tf = tf0;
                const F3 lm = linear_model<MAY_F64>(U, kns, pa, da, pb, db, blen, L, tf, acc, meff);
                w.s_tf[j * N + i] = tf;
                f.x = lm.x + fx;
                f.y = lm.y + fy;
                f.z = lm.z + 0.0f;
            } else if (bonds_model == 2) {                         // :375-417
                const float L = len2f(pa.x - pb.x, pa.y - pb.y);
                const float nd = (MAY_F64 && U.use_f64) ? distance1(1, pa, pb) : L - (pa.z + pb.z);
                const float kn = U.kb2;
                const float ks = U.ksb2;
                float Fn = (-nd) * kn;
                const float vx = pa.x - pb.x, vy = pa.y - pb.y;
                const float nx = vx / L, ny = vy / L;
                const float tx = -ny, ty = nx;
                const float dra = da.z * pa.z, drb = db.z * pb.z;
                const float rx = db.x - da.x, ry = db.y - da.y;
                const float rr = drb + dra;
                const float rt = (rx * tx + ry * ty) + rr;
                float tf = tf0;
                tf = tf + rt * ks;
                const float cd = U.p.contact_damping;
                float Fx = cd * (nx * Fn + tx * tf);
                float Fy = cd * (ny * Fn + ty * tf);
                float M = (-pa.z) * tf;
                const float atf = tf < 0.0f ? -tf : tf;
                if (U.p.bonds_tear == 1 && (Fn < -sn || atf > ss)) {
                    const int code = -10 + sign_i32(nd);
                    record_break(w, P, s, *w.step, bg, code, i, b);
                    w.s_bonded[j * N + i] = code;
                    mask &= ~(1u << (BSHIFT + j));
                    Fn = 0.0f;
                    w.s_btf[j * N + i] = 0.0f;
                    Fx = 0.0f;
                    Fy = 0.0f;
                    M = 0.0f;
                }
                w.s_tf[j * N + i] = tf;
                acc.d0 = -Fn;
                acc.d1 = tf;
                acc.d2 = M;
                f.x = Fx;
                f.y = Fy;
                f.z = M;
            }
        }
        nfx = nfx + f.x;
        nfy = nfy + f.y;
        nm = nm + f.z;
    }

    // store_forces (:434-478)
    const Mat MA = w.mats[P.mat_base + meta_mat(m)];
    const float r = pa.z;
    const float mass = ((MA.density * 3.14159274101257324219f) * r) * r;
    const float rot_inertia = ((0.5f * mass) * r) * r;
    float4 fe = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (m & M_FEXT) fe = w.fx[i];
    float fxs = nfx + fe.x;
    float fys = nfy + fe.y;
    float moment = nm + fe.z;
    if (U.p.gravity == 1 && U.p.planet_mode == 1) {
        float cx = 0.0f, cy = 0.0f;
        if (U.p.mouse_gravity == 1) {
            cx = U.p.gravity_x;
            cy = U.p.gravity_y;
        }
        const float dx = cx - pa.x, dy = cy - pa.y;
        if (dx != 0.0f || dy != 0.0f) {
            const float L = len2f(dx, dy);
            fxs = fxs + (((dx / L) * 9.81f) * U.p.gravity_acc) * mass;
            fys = fys + (((dy / L) * 9.81f) * U.p.gravity_acc) * mass;
        }
    } else if (U.p.gravity == 1) {
        const float ga = 9.81f * U.p.gravity_acc;
        fxs = fxs + 0.0f;
        fys = fys + (-ga) * mass;
    }
    const float ax = fxs / mass, ay = fys / mass;
    const float al = moment / rot_inertia;
    const long long rem = FUSE ? w.remaining[s] : 0;
    const bool steps_on = FUSE && rem > 1;  // this scene's next step is in this call
    if (!steps_on) w.ac[i] = make_float4(ax, ay, al, 0.0f);
    float4 v = w.vw[i];
    const float dT = U.p.dT;
    if (m & M_KICK_X) v.x = v.x + (0.5f * ax) * dT;
    if (m & M_KICK_Y) v.y = v.y + (0.5f * ay) * dT;
    if (m & M_KICK_R) v.z = v.z + (0.5f * al) * dT;
    if (!FUSE) {
        w.vw[i] = v;
    } else if (steps_on) {
        lom_core(w, P, U, i, m, pa, v, make_float4(ax, ay, al, 0.0f), w.pbuild[i], false,
                 make_float4(0.0f, 0.0f, 0.0f, 0.0f), lom_final || rem == 2, w.pr_n, w.dp_n);
    } else {
        w.vw[i] = v;
        w.pr_n[i] = pa;
        w.dp_n[i] = w.dp[i];
    }
    // data[0..2]; a particle without contacts writes +0 every step, which the
    // slot word's DF_ZERO bit (set while the stored value is all +0) lets it skip
    if (!steps_on) {
        const bool zero = (__float_as_uint(acc.d0) | __float_as_uint(acc.d1) | __float_as_uint(acc.d2)) == 0u;
        if (!(zero && (mask & DF_ZERO))) w.dF[i] = make_float4(acc.d0, acc.d1, acc.d2, 0.0f);
        mask = zero ? (mask | DF_ZERO) : (mask & ~DF_ZERO);
    }
    if (mask != before) w.smask[i] = mask;
}

// End of step, run by the last warp of k_interact or by k_end_step's block: breaks of this step
// become visible (status = min code), the positions-set flags clear
// (2D_Simulation.wgsl:258-261), the step counter advances, and each scene's
// narrow-phase flag for the next step is set.
template <int NT>
__device__ void end_of_step(const DevWorld &w, int tid) {
    uint32_t n = *(volatile uint32_t *)w.pend_count;
    if (n > w.pend_cap) n = w.pend_cap;
    const long long next = *(volatile long long *)w.step + 1;
    for (uint32_t k = tid; k < n; k += NT) {
        Pending p = w.pend[k];
        atomicMin(&w.b_status[p.bond], p.code);
    }
    for (int s = tid; s < w.S; s += NT) {
        w.cc3[s] = 0;
        const ScenePar &P = w.par[s];
        w.det[s] = detect_at(P.p.collision_interval, P.cc1_0, next - P.step0) ? 1 : 0;
        if (w.act[s]) {
            const long long left = w.remaining[s] - 1;
            w.remaining[s] = left;
            if (left <= 0) w.act[s] = 0;  // a served scene stops at its horizon
        }
    }
    if (NT == 32) __syncwarp();
    else __syncthreads();
    if (tid == 0) {
        *w.pend_count = 0u;
        *w.step = next;
        w.tickets[1] = 0u;
    }
}

// the last warp of a Simulation kernel (small worlds): end of step, and for
// a fused kernel in a graph the next step's rebuild condition
__device__ __forceinline__ void interact_tail(const DevWorld &w, bool fused, int in_graph,
                                              cudaGraphConditionalHandle cond) {
    if (!(w.ticket && last_warp(&w.tickets[1]))) return;
    end_of_step<32>(w, threadIdx.x & 31);
    if (fused && in_graph && (threadIdx.x & 31) == 0)
        cudaGraphSetConditional(cond, *(volatile int32_t *)w.rebuild != 0 ? 1u : 0u);
}

// Minimum blocks per SM: measured on GB300 (c3 mix, c2 scene).  Occupancy
// outweighs the few spilled words down to 40 registers for k_interact (12
// blocks: 7 % faster than 8) and 56 for k_forces (9 blocks).
// pv: the parameters of the world's only scene (PS_ONE), or the settings its
// scenes share (PS_SHARED); unused with PS_SCENE
template <bool FUSE, int FORM, int PS>
__global__ void __launch_bounds__(IB, 12) k_interact(DevWorld w, int in_graph, cudaGraphConditionalHandle cond,
                                                    int lom_final, const __grid_constant__ ScenePar pv) {
    Narrow nr;
    nr.cnt = 0;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < w.N && chunk_live(w, i)) interact_particle<0, FUSE, FORM, PS>(w, i, nr, lom_final != 0, pv);
    interact_tail(w, FUSE, in_graph, cond);
}

template <int FORM, int PS>
__global__ void __launch_bounds__(IB, 12) k_narrow(DevWorld w, const __grid_constant__ ScenePar pv) {
    Narrow nr;
    nr.cnt = 0;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < w.N && chunk_live(w, i)) interact_particle<1, false, FORM, PS>(w, i, nr, false, pv);
}

template <bool FUSE, int FORM, int PS>
__global__ void __launch_bounds__(IB, 9) k_forces(DevWorld w, int in_graph, cudaGraphConditionalHandle cond,
                                                  int lom_final, const __grid_constant__ ScenePar pv) {
    Narrow nr;
    nr.cnt = 0;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < w.N && chunk_live(w, i)) interact_particle<2, FUSE, FORM, PS>(w, i, nr, lom_final != 0, pv);
    interact_tail(w, FUSE, in_graph, cond);
}

constexpr int END_THREADS = 256;
__global__ void __launch_bounds__(END_THREADS) k_end_step(DevWorld w) { end_of_step<END_THREADS>(w, threadIdx.x); }

// Narrow phase of one large particle per block (2D_Simulation.wgsl:126-170
// with the particle's whole neighbourhood): every particle of the search
// cells within r + r_grid + skin of its position at the last rebuild, and
// every other large particle of the scene, goes through the same acceptance
// test as in k_interact; the 14 smallest keys are kept, in key order, for
// the particle's thread in k_interact.
constexpr int BIG_THREADS = 256;

__global__ void __launch_bounds__(BIG_THREADS) k_big_narrow(DevWorld w) {
    __shared__ uint32_t skey[BIG_ACC_MAX];
    __shared__ int32_t sidx[BIG_ACC_MAX];
    __shared__ int scount;
    __shared__ uint32_t wkey[BIG_THREADS / 32];
    __shared__ int32_t wpos[BIG_THREADS / 32];
    const int g = blockIdx.x;
    const int s = w.big_scene[g];
    if (s < 0 || !w.act[s]) return;
    const ScenePar &P = w.par[s];
    if (!(P.p.collisions == 1 && w.det[s] != 0)) return;
    int bf, bn;
    big_cell(w, P, bf, bn);
    const int k = g - P.big_base;
    if (k >= bn) return;  // this record's particle left the big cell (radius 0)
    const int i = w.sorted[bf + k];
    const float4 pa = w.pr[i];
    int32_t *out = w.big_acc + 16 * (size_t)g;
    // the particle's rank in its cell, for its thread in the Simulation
    // kernel (word 1 of its candidate list, unused by large particles)
    if (threadIdx.x == 0) reinterpret_cast<int32_t *>(w.nl + 2 * (size_t)i)[1] = k;
    if (pa.z == 0.0f) {
        if (threadIdx.x == 0) out[15] = 0;
        return;
    }
    const uint32_t ca = __float_as_uint(pa.w);
    const float2 p0 = w.pbuild[i];
    const float reach = pa.z + P.r_grid + P.skin;
    int cx0, cy0, cx1, cy1;
    search_xy(P, p0.x - reach, p0.y - reach, cx0, cy0);
    search_xy(P, p0.x + reach, p0.y + reach, cx1, cy1);
    if (threadIdx.x == 0) scount = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    auto consider = [&](int b) {
        if (b == i) return;
        const float4 pb = __ldg(&w.pr[b]);
        if (!touching(pa, pb)) return;
        unsigned rank;
        if (!shared_bucket(w, ca, __float_as_uint(pb.w), rank)) return;
        const int q = atomicAdd(&scount, 1);
        if (q < BIG_ACC_MAX) {
            skey[q] = (rank << 28) | (uint32_t)__ldg(&w.orig[b]);
            sidx[q] = b;
        }
    };
    for (int cy = cy0 + warp; cy <= cy1; cy += BIG_THREADS / 32) {
        const int row = P.cell_base + cy * P.g_w;
        const int beg = w.cell_start[row + cx0], end = w.cell_start[row + cx1 + 1];
        for (int q = beg + lane; q < end; q += 32) consider(w.sorted[q]);
    }
    for (int q = threadIdx.x; q < bn; q += BIG_THREADS) consider(w.sorted[bf + q]);
    __syncthreads();
    int n = scount;
    if (n > BIG_ACC_MAX) {
        if (threadIdx.x == 0) atomicOr(w.err, 4);
        n = BIG_ACC_MAX;
    }
    const int keep = n < K ? n : K;
    // keys are distinct: round r takes the smallest key above round r-1's
    uint32_t prev = 0u;
    for (int r = 0; r < keep; ++r) {
        uint32_t best = 0xFFFFFFFFu;
        int pos = -1;
        for (int q = threadIdx.x; q < n; q += BIG_THREADS) {
            const uint32_t kq = skey[q];
            if ((r == 0 || kq > prev) && (pos < 0 || kq < best)) {
                best = kq;
                pos = q;
            }
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            const uint32_t ok = __shfl_down_sync(0xffffffffu, best, o);
            const int op = __shfl_down_sync(0xffffffffu, pos, o);
            if (op >= 0 && (pos < 0 || ok < best)) {
                best = ok;
                pos = op;
            }
        }
        if (lane == 0) {
            wkey[warp] = best;
            wpos[warp] = pos;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t bk = 0xFFFFFFFFu;
            int bp = -1;
            for (int v = 0; v < BIG_THREADS / 32; ++v)
                if (wpos[v] >= 0 && (bp < 0 || wkey[v] < bk)) {
                    bk = wkey[v];
                    bp = wpos[v];
                }
            out[r] = sidx[bp];
            wkey[0] = bk;
        }
        __syncthreads();
        prev = wkey[0];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[15] = keep;
}

template <int FORM, int PS>
static int launch_sim_as(const DevWorld &w, int g, cudaStream_t st, bool fuse, int ig, int lf,
                         cudaGraphConditionalHandle cond, const ScenePar &pv) {
    if (w.split) {
        k_narrow<FORM, PS><<<g, IB, 0, st>>>(w, pv);
        if (fuse) k_forces<true, FORM, PS><<<g, IB, 0, st>>>(w, ig, cond, lf, pv);
        else k_forces<false, FORM, PS><<<g, IB, 0, st>>>(w, ig, cond, lf, pv);
        return 2;
    }
    if (fuse) k_interact<true, FORM, PS><<<g, IB, 0, st>>>(w, ig, cond, lf, pv);
    else k_interact<false, FORM, PS><<<g, IB, 0, st>>>(w, ig, cond, lf, pv);
    return 1;
}

template <int FORM>
static int launch_sim(const DevWorld &w, int g, cudaStream_t st, bool fuse, int ig, int lf,
                      cudaGraphConditionalHandle cond, const ScenePar *pv, int ps) {
    if (ps == PS_ONE) return launch_sim_as<FORM, PS_ONE>(w, g, st, fuse, ig, lf, cond, *pv);
    if (ps == PS_SHARED) return launch_sim_as<FORM, PS_SHARED>(w, g, st, fuse, ig, lf, cond, *pv);
    const ScenePar unused{};
    return launch_sim_as<FORM, PS_SCENE>(w, g, st, fuse, ig, lf, cond, unused);
}

int launch_interact(const DevWorld &w, int block, cudaStream_t st, bool bigs, bool fuse, bool lom_final,
                    bool in_graph, cudaGraphConditionalHandle cond, int form, const ScenePar *pv, int ps) {
    (void)block;
    int k = 0;
    if (bigs && w.n_big_slots > 0) {
        k_big_narrow<<<w.n_big_slots, BIG_THREADS, 0, st>>>(w);
        k++;
    }
    const int g = w.N > 0 ? (w.N + IB - 1) / IB : 1;
    const int ig = in_graph ? 1 : 0, lf = lom_final ? 1 : 0;
    switch (form) {
        case 3: k += launch_sim<3>(w, g, st, fuse, ig, lf, cond, pv, ps); break;
        case 0: k += launch_sim<0>(w, g, st, fuse, ig, lf, cond, pv, ps); break;
        case -2: k += launch_sim<-2>(w, g, st, fuse, ig, lf, cond, pv, ps); break;
        default: k += launch_sim<-1>(w, g, st, fuse, ig, lf, cond, pv, ps); break;
    }
    if (!w.ticket) {
        k_end_step<<<1, END_THREADS, 0, st>>>(w);
        k++;
        if (fuse && in_graph) {
            k_decide<<<1, 32, 0, st>>>(w, cond);
            k++;
        }
    }
    return k;
}

// ------------------------------------------------------- free ranges
__global__ void k_mark_free(DevWorld w, int first, int count, int free_scene) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    int i = first + k;
    w.meta[i] = (uint32_t)free_scene << 16;
    w.pr[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    w.pr_n[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    w.smask[i] = 0u;
    w.nl[2 * (size_t)i] = make_int4(0, 0, 0, 0);
    w.orig[i] = k;
}

void launch_mark_free(const DevWorld &w, int first, int count, int free_scene, cudaStream_t st) {
    if (count <= 0) return;
    k_mark_free<<<(count + 255) / 256, 256, 0, st>>>(w, first, count, free_scene);
}

// ------------------------------------------------------- layout conversion
// Every item of a transfer in one launch.  The contact records (84 words a
// particle, 72% of the bytes) are moved whole through shared memory: a tile
// of ST_P particles is read or written as contiguous 16-byte words on the
// reference side and as 32-particle rows on the slot side, so both sides
// are coalesced.
constexpr int ST_P = 64, ST_THREADS = 128, ST_REC = 6 * K, ST_REC4 = ST_REC / 4;
static_assert(ST_REC % 4 == 0, "contact record is a whole number of 16-byte words");

// item holding staged particle t, walking forward from item k (items are
// packed and sorted by off)
__device__ __forceinline__ int item_from(const StageItem *it, int count, int k, long long t) {
    while (k + 1 < count && it[k + 1].off <= t) ++k;
    return k;
}

__device__ __forceinline__ int item_search(const StageItem *it, int count, long long t) {
    int lo = 0, hi = count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (it[mid].off <= t) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// one thread per (particle, slot); a block's first item found by search,
// the rest by walking
__global__ void k_stage_check(RefArrays r, const StageItem *__restrict__ it, int count, long long total,
                              int32_t *err) {
    __shared__ int s_k0;
    const long long u0 = (long long)blockIdx.x * blockDim.x;
    if (threadIdx.x == 0) s_k0 = item_search(it, count, u0 / K);
    __syncthreads();
    const long long u = u0 + threadIdx.x;
    if (u >= total * K) return;
    const long long t = u / K;
    const int k = item_from(it, count, s_k0, t);
    const int n = it[k].n;
    const long long i = t - it[k].off;
    if (i < 0 || i >= n) return;  // padding between items
    const int32_t *c = r.contacts + u * 6;
    int e = 0;
    if (c[5] >= it[k].n_bonds) e |= 2;
    if (c[1] != -1) {
        if (c[1] < 0 || c[1] >= n) e |= 4;
        if (c[0] != i) e |= 8;
    }
    if (u % K == 0) {
        const int mp = r.material_pointers[t];
        if (mp < 0 || mp >= it[k].n_mat) e |= 1;
    }
    if (e) atomicOr(err + k, e);
}

void launch_stage_check(const RefArrays &r, const StageItem *items, int count, long long total, int32_t *err,
                        cudaStream_t st) {
    if (total <= 0 || count <= 0) return;
    const long long t = total * K;
    k_stage_check<<<(unsigned)((t + 255) / 256), 256, 0, st>>>(r, items, count, total, err);
}

// tile of ST_P staged particles: their items and world indices
__device__ __forceinline__ void tile_items(const StageItem *it, int count, long long t0, int np, int *s_item,
                                           int *s_g) {
    __shared__ int s_k0;
    if (threadIdx.x == 0) s_k0 = item_search(it, count, t0);
    __syncthreads();
    if (threadIdx.x < np) {
        const long long t = t0 + threadIdx.x;
        const int k = item_from(it, count, s_k0, t);
        const long long i = t - it[k].off;
        s_item[threadIdx.x] = k;
        s_g[threadIdx.x] = (i >= 0 && i < it[k].n) ? it[k].base + (int)i : -1;  // -1: padding
    }
}

__global__ void __launch_bounds__(ST_THREADS) k_stage_in(DevWorld w, RefArrays r, const StageItem *__restrict__ it,
                                                          int count, long long total) {
    __shared__ __align__(16) int32_t cont[ST_P * ST_REC];
    __shared__ int s_item[ST_P], s_g[ST_P];
    const long long t0 = (long long)blockIdx.x * ST_P;
    const int np = (int)min((long long)ST_P, total - t0);
    const int4 *src = reinterpret_cast<const int4 *>(r.contacts + t0 * ST_REC);
    int4 *c4 = reinterpret_cast<int4 *>(cont);
    for (int v = threadIdx.x; v < np * ST_REC4; v += ST_THREADS) c4[v] = src[v];
    tile_items(it, count, t0, np, s_item, s_g);
    __syncthreads();
    // slot rows (slot j, particle p), p fastest
    for (int q = threadIdx.x; q < K * ST_P; q += ST_THREADS) {
        const int j = q / ST_P, p = q % ST_P;
        if (p >= np || s_g[p] < 0) continue;
        const int32_t *c = cont + p * ST_REC + 6 * j;
        const size_t at = (size_t)j * w.N + s_g[p];
        const int b = c[1];
        w.s_b[at] = b != -1 ? it[s_item[p]].base + b : -1;
        w.s_tf[at] = __int_as_float(c[2]);
        w.s_btf[at] = __int_as_float(c[3]);
        w.s_thb[at] = __int_as_float(c[4]);
        w.s_bonded[at] = c[5];
    }
    if (threadIdx.x >= np || s_g[threadIdx.x] < 0) return;
    const int p = threadIdx.x;
    const StageItem I = it[s_item[p]];
    const long long t = t0 + p;
    const int g = s_g[p], i = (int)(t - I.off);
    const float radius = r.radii[t];
    // the bucket range (w) is written by the LOM pass before any Simulation pass reads it
    const float4 pr = make_float4(r.pos[2 * t], r.pos[2 * t + 1], radius, 0.0f);
    const float4 dp = make_float4(r.del_pos[2 * t], r.del_pos[2 * t + 1], r.del_rot[t], 0.0f);
    w.pr[g] = pr;
    w.pr_n[g] = pr;   // both buffers: a scene that never steps must read the same from either
    w.dp[g] = dp;
    w.dp_n[g] = dp;
    w.vw[g] = make_float4(r.vel[2 * t], r.vel[2 * t + 1], r.rot_vel[t], r.rot[t]);
    w.ac[g] = make_float4(r.acc[2 * t], r.acc[2 * t + 1], r.rot_acc[t], 0.0f);
    const float *f = r.forces + 6 * t;
    w.fx[g] = make_float4(f[0], f[1], f[2], 0.0f);
    float4 d4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), dF = d4;
    if (I.has_data) {
        const float *dd = r.data + 7 * t;
        d4 = make_float4(dd[4], dd[5], dd[6], 0.0f);
        dF = make_float4(dd[0], dd[1], dd[2], 0.0f);
    }
    w.d4[g] = d4;
    w.dF[g] = dF;
    const int32_t *fix = r.fixity + 6 * t;
    uint32_t m = 0;
    m |= fix[0] == 0 ? M_KICK_X : 0u;
    m |= fix[1] == 0 ? M_KICK_Y : 0u;
    m |= fix[2] == 0 ? M_KICK_R : 0u;
    m |= fix[0] == 1 ? M_FIX_X : 0u;
    m |= fix[1] == 1 ? M_FIX_Y : 0u;
    m |= fix[2] == 1 ? M_FIX_R : 0u;
    if (f[0] != 0.0f || f[1] != 0.0f || f[2] != 0.0f) m |= M_FEXT;
    const int mp = r.material_pointers[t];   // range checked before the launch
    m |= ((uint32_t)mp & 0xFFu) << 8;
    for (int k = 0; k < 6; ++k) {
        w.fix_ref[6 * (size_t)g + k] = fix[k];
        w.force_ref[6 * (size_t)g + k] = f[k];
    }
    w.matp_ref[g] = mp;
    w.data3[g] = I.has_data ? r.data[7 * t + 3] : 0.0f;
    m |= (uint32_t)I.scene << 16;
    if (radius > I.r_big) m |= M_BIG;
    w.meta[g] = m;
    w.orig[g] = i;
    w.o2i[g] = g;
    uint32_t mk = 0;
    const int32_t *c = cont + p * ST_REC;
    for (int j = 0; j < K; ++j) {
        if (c[6 * j + 5] >= 0) mk |= 1u << (BSHIFT + j);
        if (c[6 * j + 1] != -1) mk |= 1u << j;
    }
    if ((__float_as_uint(dF.x) | __float_as_uint(dF.y) | __float_as_uint(dF.z)) == 0u) mk |= DF_ZERO;
    w.smask[g] = mk;
}

void launch_stage_in(const DevWorld &w, const RefArrays &r, const StageItem *items, int count, long long total,
                     cudaStream_t st) {
    if (total <= 0 || count <= 0) return;
    k_stage_in<<<(unsigned)((total + ST_P - 1) / ST_P), ST_THREADS, 0, st>>>(w, r, items, count, total);
}

// The world's particles of every item, in world order, to the reference
// layout in original order (orig[g]); the per-particle reference mirrors
// (fixity, forces, material pointers, data[3]) are indexed by original index
// and read by the host directly.
__global__ void __launch_bounds__(ST_THREADS) k_stage_out(DevWorld w, RefArrays r, const StageItem *__restrict__ it,
                                                           int count, long long total, int32_t *err) {
    __shared__ __align__(16) int32_t cont[ST_P * ST_REC];
    __shared__ int s_item[ST_P], s_g[ST_P], s_o[ST_P];
    __shared__ uint32_t s_mask[ST_P];
    const long long t0 = (long long)blockIdx.x * ST_P;
    const int np = (int)min((long long)ST_P, total - t0);
    tile_items(it, count, t0, np, s_item, s_g);
    if (threadIdx.x < np) {
        const int k = s_item[threadIdx.x], g = s_g[threadIdx.x];
        const int o = g < 0 ? -1 : w.orig[g];
        if (g < 0) {
            s_o[threadIdx.x] = -1;  // padding
        } else if (o < 0 || o >= it[k].n) {
            atomicOr(err + k, 16);
            atomicOr(err + count, 16);
            s_o[threadIdx.x] = -1;
        } else {
            s_o[threadIdx.x] = o;
        }
        s_mask[threadIdx.x] = g < 0 ? 0u : w.smask[g];
    }
    __syncthreads();
    for (int q = threadIdx.x; q < K * ST_P; q += ST_THREADS) {
        const int j = q / ST_P, p = q % ST_P;
        if (p >= np || s_o[p] < 0) continue;
        const int g = s_g[p];
        const size_t at = (size_t)j * w.N + g;
        int32_t *c = cont + p * ST_REC + 6 * j;
        if ((s_mask[p] >> j) & 1u) {
            const int pb = w.s_b[at];
            const int base = it[s_item[p]].base, n = it[s_item[p]].n;
            if (pb < base || pb >= base + n) {
                atomicOr(err + s_item[p], 32);
                atomicOr(err + count, 32);
                c[0] = -1;
                c[1] = -1;
            } else {
                c[0] = s_o[p];
                c[1] = w.orig[pb];
            }
        } else {
            c[0] = -1;
            c[1] = -1;
        }
        c[2] = __float_as_int(w.s_tf[at]);
        c[3] = __float_as_int(w.s_btf[at]);
        c[4] = __float_as_int(w.s_thb[at]);
        c[5] = w.s_bonded[at];
    }
    __syncthreads();
    // whole records to their original positions
    const int4 *c4 = reinterpret_cast<const int4 *>(cont);
    for (int v = threadIdx.x; v < np * ST_REC4; v += ST_THREADS) {
        const int p = v / ST_REC4, q = v % ST_REC4;
        if (s_o[p] < 0) continue;
        const long long dst = it[s_item[p]].off + s_o[p];
        reinterpret_cast<int4 *>(r.contacts + dst * ST_REC)[q] = c4[v];
    }
    if (threadIdx.x >= np || s_o[threadIdx.x] < 0) return;
    const int p = threadIdx.x, g = s_g[p];
    const StageItem I = it[s_item[p]];
    const long long o = I.off + s_o[p];
    const float4 pp = w.pr[g], v = w.vw[g], a = w.ac[g], d = w.dp[g], d4 = w.d4[g], dF = w.dF[g];
    r.pos[2 * o] = pp.x;
    r.pos[2 * o + 1] = pp.y;
    r.radii[o] = pp.z;
    r.rot[o] = v.w;
    r.vel[2 * o] = v.x;
    r.vel[2 * o + 1] = v.y;
    r.rot_vel[o] = v.z;
    r.acc[2 * o] = a.x;
    r.acc[2 * o + 1] = a.y;
    r.rot_acc[o] = a.z;
    r.del_pos[2 * o] = d.x;
    r.del_pos[2 * o + 1] = d.y;
    r.del_rot[o] = d.z;
    float *dd = r.data + 7 * o;
    dd[0] = dF.x;
    dd[1] = dF.y;
    dd[2] = dF.z;
    dd[3] = w.data3[I.base + s_o[p]];
    dd[4] = d4.x;
    dd[5] = d4.y;
    dd[6] = d4.z;
}

void launch_stage_out(const DevWorld &w, const RefArrays &r, const StageItem *items, int count, long long total,
                      int32_t *err, cudaStream_t st) {
    if (total <= 0 || count <= 0) return;
    k_stage_out<<<(unsigned)((total + ST_P - 1) / ST_P), ST_THREADS, 0, st>>>(w, r, items, count, total, err);
}

// one block per piece; 16-byte words where both ends allow, else 4-byte
// words, both coalesced
constexpr int COPY_THREADS = 256;
__global__ void __launch_bounds__(COPY_THREADS) k_copies(const HostCopy *__restrict__ c, int n,
                                                          const int32_t *guard) {
    if (guard && *guard) return;
    __shared__ int s_k;
    const long long b = blockIdx.x;
    if (threadIdx.x == 0) {
        int lo = 0, hi = n - 1;  // last copy with piece0 <= b
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (c[mid].piece0 <= b) lo = mid;
            else hi = mid - 1;
        }
        s_k = lo;
    }
    __syncthreads();
    const HostCopy C = c[s_k];
    const long long at = (b - C.piece0) * COPY_PIECE;
    const long long len = min(COPY_PIECE, C.bytes - at);
    if (len <= 0) return;
    const char *src = C.src + at;
    char *dst = C.dst + at;
    if (((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15) == 0) {
        const int n16 = (int)(len >> 4);
        const int4 *s4 = reinterpret_cast<const int4 *>(src);
        int4 *d4 = reinterpret_cast<int4 *>(dst);
#pragma unroll 4
        for (int i = threadIdx.x; i < n16; i += COPY_THREADS) d4[i] = s4[i];
        for (long long i = ((long long)n16 << 4) + 4 * threadIdx.x; i < len; i += 4 * COPY_THREADS)
            *reinterpret_cast<int32_t *>(dst + i) = *reinterpret_cast<const int32_t *>(src + i);
    } else {
        const int n4 = (int)(len >> 2);
        const int32_t *s1 = reinterpret_cast<const int32_t *>(src);
        int32_t *d1 = reinterpret_cast<int32_t *>(dst);
#pragma unroll 4
        for (int i = threadIdx.x; i < n4; i += COPY_THREADS) d1[i] = s1[i];
    }
}

void launch_copies(const HostCopy *c, int n, long long pieces, const int32_t *guard, cudaStream_t st) {
    if (n <= 0 || pieces <= 0) return;
    k_copies<<<(unsigned)pieces, COPY_THREADS, 0, st>>>(c, n, guard);
}

// ------------------------------------------------------- Fix / Drop / Release
__global__ void k_fixity_event(DevWorld w, int base, const int32_t *__restrict__ idx, int count, int kind,
                               float vx, float vy, int set_vel) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const int g = base + idx[t];
    const int i = w.o2i[g];
    int32_t *f = w.fix_ref + 6 * (size_t)g;
    if (kind == DEM_EVENT_FIX) {                                   // Fix.wgsl:44-54
        for (int k = 0; k < 6; ++k) f[k] = 1;
    } else if (kind == DEM_EVENT_DROP) {                           // Drop.wgsl:34-41
        for (int k = 0; k < 6; ++k) f[k] = 0;
    } else {                                                       // Release.wgsl:78-85
        f[0] = f[3];
        f[1] = f[4];
        f[2] = f[5];
    }
    uint32_t m = w.meta[i] & ~(M_KICK_X | M_KICK_Y | M_KICK_R | M_FIX_X | M_FIX_Y | M_FIX_R);
    m |= (f[0] == 0 ? M_KICK_X : 0u) | (f[1] == 0 ? M_KICK_Y : 0u) | (f[2] == 0 ? M_KICK_R : 0u);
    m |= (f[0] == 1 ? M_FIX_X : 0u) | (f[1] == 1 ? M_FIX_Y : 0u) | (f[2] == 1 ? M_FIX_R : 0u);
    w.meta[i] = m;
    float4 v = w.vw[i];
    if (kind == DEM_EVENT_FIX) {                                   // Fix.wgsl:50-52
        v.x = 0.0f;
        v.y = 0.0f;
        v.z = 0.0f;
    }
    if (set_vel) {                                                 // Release.wgsl:86-89
        v.x = vx;
        v.y = vy;
    }
    w.vw[i] = v;
}

void launch_fixity_event(const DevWorld &w, int base, const int32_t *d_idx, int count, int kind, float vx,
                         float vy, int set_vel, cudaStream_t st) {
    if (count <= 0) return;
    k_fixity_event<<<(count + 255) / 256, 256, 0, st>>>(w, base, d_idx, count, kind, vx, vy, set_vel);
}

// per particle: pos.x, pos.y, data[4], data[5], rot, data[6], data[0], data[1], data[2], data[3]
__global__ void k_gather_datum(DevWorld w, int base, const int32_t *__restrict__ idx, int count,
                               float *__restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const int i = w.o2i[base + idx[t]];
    const float4 p = w.pr[i], d4 = w.d4[i], dF = w.dF[i];
    const float rot = w.vw[i].w;
    float *o = out + 10 * (size_t)t;
    o[0] = p.x;
    o[1] = p.y;
    o[2] = d4.x;
    o[3] = d4.y;
    o[4] = rot;
    o[5] = d4.z;
    o[6] = dF.x;
    o[7] = dF.y;
    o[8] = dF.z;
    o[9] = w.data3[base + idx[t]];
}

void launch_gather_datum(const DevWorld &w, int base, const int32_t *d_idx, int count, float *d_out,
                         cudaStream_t st) {
    if (count <= 0) return;
    k_gather_datum<<<(count + 255) / 256, 256, 0, st>>>(w, base, d_idx, count, d_out);
}

// ------------------------------------------------------- Set_Properties
// Set_Properties.wgsl:68-90; selections are indexed by scene-local particle.
__global__ void __launch_bounds__(PK_MAX_THREADS) k_set_properties(DevWorld w, int scene,
                                                        const int32_t *__restrict__ sel,
                                                        int32_t *__restrict__ sel_out,
                                                        const int32_t *__restrict__ in) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.N) return;
    uint32_t m = w.meta[i];
    if ((int)meta_scene(m) != scene) return;
    int o = w.orig[i];
    if (sel[o] == 0) return;
    const float *f = reinterpret_cast<const float *>(in);
    float4 p = w.pr[i], v = w.vw[i], d = w.dp[i], fe = w.fx[i];
    bool setpos = false;
    if (in[0] == 1) { d.x = f[14] - p.x; p.x = f[14]; setpos = true; }
    if (in[1] == 1) { d.y = f[15] - p.y; p.y = f[15]; setpos = true; }
    if (in[2] == 1) { d.z = f[16] - v.w; v.w = f[16]; }
    if (in[3] == 1) v.x = f[17];
    if (in[4] == 1) v.y = f[18];
    if (in[5] == 1) v.z = f[19];
    if (in[9] == 1) p.z = f[23];
    if (in[6] == 1) fe.x = f[20];
    if (in[7] == 1) fe.y = f[21];
    if (in[8] == 1) fe.z = f[22];
    if (in[10] == 1) {
        m &= ~(M_KICK_X | M_FIX_X);
        m |= (in[24] == 0 ? M_KICK_X : 0u) | (in[24] == 1 ? M_FIX_X : 0u);
    }
    if (in[11] == 1) {
        m &= ~(M_KICK_Y | M_FIX_Y);
        m |= (in[25] == 0 ? M_KICK_Y : 0u) | (in[25] == 1 ? M_FIX_Y : 0u);
    }
    if (in[12] == 1) {
        m &= ~(M_KICK_R | M_FIX_R);
        m |= (in[26] == 0 ? M_KICK_R : 0u) | (in[26] == 1 ? M_FIX_R : 0u);
    }
    if (in[13] == 1) m = (m & ~(0xFFu << 8)) | ((uint32_t)(in[27] & 0xFF) << 8);
    if (fe.x != 0.0f || fe.y != 0.0f || fe.z != 0.0f) m |= M_FEXT;
    else m &= ~M_FEXT;
    w.pr[i] = p;
    w.vw[i] = v;
    w.dp[i] = d;
    w.fx[i] = fe;
    w.meta[i] = m;
    const size_t g = (size_t)w.par[scene].particle_base + o;
    if (in[6] == 1) w.force_ref[6 * g] = f[20];
    if (in[7] == 1) w.force_ref[6 * g + 1] = f[21];
    if (in[8] == 1) w.force_ref[6 * g + 2] = f[22];
    for (int k = 0; k < 3; ++k)
        if (in[10 + k] == 1) {
            w.fix_ref[6 * g + k] = in[24 + k];
            w.fix_ref[6 * g + k + 3] = in[24 + k];
        }
    if (in[13] == 1) w.matp_ref[g] = in[27];
    if (setpos) w.cc3[scene] = 1;
    if (in[10] == 1 || in[11] == 1 || in[12] == 1) sel_out[o] = 2;
}

void launch_set_properties(const DevWorld &w, int scene, const int32_t *d_sel, int32_t *d_sel_out,
                           const int32_t *d_props, int block, cudaStream_t st) {
    if (w.N == 0) return;
    k_set_properties<<<(w.N + block - 1) / block, block, 0, st>>>(w, scene, d_sel, d_sel_out, d_props);
}

}  // namespace demgb

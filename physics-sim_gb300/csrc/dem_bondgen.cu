// dem_bondgen.cu -- bond generation on the GPU, the O(n) replacement of the
// reference's O(n^2) State::regen_bonds (src/state.rs:291-367).
//
// regen_bonds walks i = 0..n and, for each i, j = i+1..n in order; a pair
// closer than 1.05 (r_i + r_j) becomes a bond while i has made fewer than
// max_bonds of its own, bonds are numbered in creation order, and each new
// bond takes the first free contact slot of i and of j.  Slots are never
// freed, so a particle's slots hold its bonds in creation order, i.e. in
// bond-index order, and its bonds with partners i' < p (made while i' was
// processed) all precede its own.  The same result is built here without the
// sequential walk:
//   1. a uniform grid of cells at least 2.1 r_max wide (every bonding pair
//      lies in neighbouring cells), the particles binned by cell;
//   2. per i, the first max_bonds partners j > i in index order that pass
//      the reference's test, from the 3x3 cells (the selection keeps the
//      smallest qualifying indices whatever order a cell lists its members
//      in, so the bins need no order);
//   3. bond numbers = exclusive scan of the per-i counts (creation order);
//   4. per particle, its bonds where it is the j side in ascending number --
//      a stable counting sort of the bond numbers by j (dem_sort.cuh) --
//      then its own; the first 14 fill its contact slots.
// The bond record's length and angle are evaluated on the host, one pass
// over the bonds, with the host's powf and atan2f as the reference does
// (state.rs:309-313): the reference takes the length as powf(d2, 0.5), which
// differs from the correctly rounded square root in the last bit for some
// inputs, so it is not recomputed on the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "dem.h"
#include "dem_sort.cuh"
#include "dem_world.cuh"

namespace {

thread_local std::string g_bondgen_error;
using demgb::K;
constexpr int MAXB = K;  // max_bonds may not exceed the 14 contact slots

int bfail(int code, const std::string &m) {
    g_bondgen_error = m;
    return code;
}

struct Grid {
    float x0, y0, inv;
    int gw, gh;
};

__device__ __forceinline__ int cell_of(const Grid &g, float x, float y) {
    int a = __float2int_rd((x - g.x0) * g.inv);
    int b = __float2int_rd((y - g.y0) * g.inv);
    a = a < 0 ? 0 : (a > g.gw - 1 ? g.gw - 1 : a);
    b = b < 0 ? 0 : (b > g.gh - 1 ? g.gh - 1 : b);
    return b * g.gw + a;
}

__global__ void k_bg_keys(const float2 *__restrict__ pos, int n, Grid g, int32_t *__restrict__ keys,
                          int32_t *counts) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = cell_of(g, pos[i].x, pos[i].y);
    keys[i] = c;
    atomicAdd(&counts[c], 1);
}

__global__ void k_bg_scatter(const int32_t *__restrict__ keys, int n, const int32_t *__restrict__ start,
                             int32_t *counts, int32_t *__restrict__ order) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = keys[i];
    order[start[c] + atomicSub(&counts[c], 1) - 1] = i;
}

// the first max_bonds partners j > i (ascending j) that pass state.rs:301-304
__global__ void k_bg_select(const float2 *__restrict__ pos, const float *__restrict__ radii, int n, Grid g,
                            const int32_t *__restrict__ start, const int32_t *__restrict__ order,
                            int max_bonds, int32_t *__restrict__ sel, int32_t *__restrict__ count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float2 pi = pos[i];
    const float ri = radii[i];
    int best[MAXB];
    int nb = 0;
    const int c = cell_of(g, pi.x, pi.y);
    const int cx = c % g.gw, cy = c / g.gw;
    for (int yy = max(cy - 1, 0); yy <= min(cy + 1, g.gh - 1); ++yy) {
        const int row = yy * g.gw;
        const int beg = start[row + max(cx - 1, 0)], end = start[row + min(cx + 1, g.gw - 1) + 1];
        for (int k = beg; k < end; ++k) {
            const int j = order[k];
            if (j <= i) continue;
            if (nb == max_bonds && j >= best[nb - 1]) continue;
            const float2 pj = pos[j];
            const float dx = pj.x - pi.x, dy = pj.y - pi.y;
            const float distance = sqrtf(dx * dx + dy * dy);
            const float sum = ri + radii[j];
            if (!(distance < sum * 1.05f)) continue;
            int q = nb < max_bonds ? nb : max_bonds - 1;
            while (q > 0 && best[q - 1] > j) {
                best[q] = best[q - 1];
                --q;
            }
            best[q] = j;
            if (nb < max_bonds) ++nb;
        }
    }
    for (int q = 0; q < nb; ++q) sel[(size_t)i * max_bonds + q] = best[q];
    count[i] = nb;
}

// bond records (status) and the j side's incoming count
__global__ void k_bg_write(int n, int max_bonds, const int32_t *__restrict__ sel,
                           const int32_t *__restrict__ count, const int32_t *__restrict__ base,
                           int32_t *__restrict__ bonds, int32_t *__restrict__ bond_i, int32_t *__restrict__ bond_j,
                           int32_t *in_count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int q = 0; q < count[i]; ++q) {
        const int b = base[i] + q;
        const int j = sel[(size_t)i * max_bonds + q];
        bonds[3 * (size_t)b] = 1;
        bonds[3 * (size_t)b + 1] = 0;  // angle and length: filled on the host
        bonds[3 * (size_t)b + 2] = 0;
        bond_i[b] = i;
        bond_j[b] = j;
        atomicAdd(&in_count[j], 1);
    }
}

// the sort's input: bond numbers in order, keyed by their j side
struct BgBonds {
    const int32_t *bond_j;
    int n;
    __device__ __forceinline__ int length() const { return n; }
    __device__ __forceinline__ bool get(int t, uint32_t &k, int32_t &v) const {
        k = (uint32_t)bond_j[t];
        v = t;
        return true;
    }
};

// contact slots: bonds where p is the j side (ascending number), then p's own
__global__ void k_bg_slots(int n, int max_bonds, const int32_t *__restrict__ count, const int32_t *__restrict__ base,
                           const int32_t *__restrict__ sel, const int32_t *__restrict__ in_start,
                           const int32_t *__restrict__ in_list, const int32_t *__restrict__ bond_i,
                           int32_t *__restrict__ contacts) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int beg = in_start[p], end = in_start[p + 1];
    int32_t *c = contacts + (size_t)p * K * 6;
    int s = 0;
    for (int a = beg; a < end && s < K; ++a, ++s) {
        const int b = in_list[a];
        c[6 * s] = p;
        c[6 * s + 1] = bond_i[b];
        c[6 * s + 2] = 0;
        c[6 * s + 3] = 0;
        c[6 * s + 4] = 0;
        c[6 * s + 5] = b;
    }
    for (int q = 0; q < count[p] && s < K; ++q, ++s) {
        c[6 * s] = p;
        c[6 * s + 1] = sel[(size_t)p * max_bonds + q];
        c[6 * s + 2] = 0;
        c[6 * s + 3] = 0;
        c[6 * s + 4] = 0;
        c[6 * s + 5] = base[p] + q;
    }
    for (; s < K; ++s)
        for (int f = 0; f < 6; ++f) c[6 * s + f] = -1;
}

struct DevBuf {
    std::vector<void *> ptrs;
    ~DevBuf() {
        for (void *p : ptrs) cudaFree(p);
    }
    template <class T>
    T *get(size_t count) {
        void *p = nullptr;
        if (cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess) return nullptr;
        ptrs.push_back(p);
        return static_cast<T *>(p);
    }
};

}  // namespace

extern "C" {

const char *dem_bondgen_last_error(void) { return g_bondgen_error.c_str(); }

int dem_generate_bonds(const float *pos, const float *radii, int32_t n, int32_t max_bonds, int32_t device,
                       int32_t *bonds, int64_t bonds_cap, int64_t *n_bonds, int32_t *contacts) {
    g_bondgen_error.clear();
    if (n < 0 || !n_bonds) return bfail(DEM_E_INVALID, "n < 0 or n_bonds is NULL");
    // at most 14 bonds a particle: bond numbers (and the incoming-bond sort's
    // sequence) stay below 2^30
    if (n > (1 << 26)) return bfail(DEM_E_CAPACITY, "n is above 2^26 particles");
    if (max_bonds < 1 || max_bonds > MAXB) return bfail(DEM_E_INVALID, "max_bonds must be in [1, 14]");
    if (n > 0 && (!pos || !radii || !contacts)) return bfail(DEM_E_INVALID, "a required array is NULL");
    *n_bonds = 0;
    if (n == 0) return DEM_OK;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return bfail(DEM_E_CUDA, "no CUDA device available");
    if (device >= 0 && (device >= ndev || cudaSetDevice(device) != cudaSuccess))
        return bfail(DEM_E_INVALID, "bad device index");
    // grid over the particles: cells at least 2.1 r_max wide (a bonding pair
    // is closer than 1.05 (r_i + r_j) <= 2.1 r_max), at most ~4n cells
    float rmax = 0.0f, xmin = 0, xmax = 0, ymin = 0, ymax = 0;
    for (int i = 0; i < n; ++i) {
        const float x = pos[2 * i], y = pos[2 * i + 1], r = radii[i];
        if (!std::isfinite(x) || !std::isfinite(y) || !(r >= 0.0f) || !std::isfinite(r))
            return bfail(DEM_E_INVALID, "positions and radii must be finite, radii >= 0");
        rmax = std::max(rmax, r);
        if (i == 0) { xmin = xmax = x; ymin = ymax = y; }
        xmin = std::min(xmin, x); xmax = std::max(xmax, x);
        ymin = std::min(ymin, y); ymax = std::max(ymax, y);
    }
    double cs = std::max(2.1 * (double)rmax * (1.0 + 1e-4), 1e-30);
    const double span_x = (double)xmax - xmin, span_y = (double)ymax - ymin;
    const double cap = std::max(4.0 * n, 1024.0);
    while ((span_x / cs + 1.0) * (span_y / cs + 1.0) > cap) cs *= 1.25;
    Grid g;
    g.x0 = xmin;
    g.y0 = ymin;
    g.inv = (float)(1.0 / cs);
    g.gw = (int)(span_x / cs) + 2;
    g.gh = (int)(span_y / cs) + 2;
    const int cells = g.gw * g.gh;
    cudaStream_t st = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
        return bfail(DEM_E_CUDA, "stream creation failed");
    int rc = DEM_OK;
    {
        DevBuf db;
        float2 *d_pos = db.get<float2>(n);
        float *d_r = db.get<float>(n);
        int32_t *d_keys = db.get<int32_t>(n), *d_cnt = db.get<int32_t>(cells), *d_start = db.get<int32_t>(cells + 1);
        int32_t *d_order = db.get<int32_t>(n), *d_tmp = db.get<int32_t>(demgb::scan_tmp_size(std::max(cells, n + 1)));
        int32_t *d_sel = db.get<int32_t>((size_t)n * max_bonds), *d_count = db.get<int32_t>(n);
        int32_t *d_base = db.get<int32_t>(n + 1);
        if (!d_pos || !d_r || !d_keys || !d_cnt || !d_start || !d_order || !d_tmp || !d_sel || !d_count || !d_base) {
            rc = bfail(DEM_E_OOM, "device allocation failed");
        }
        const int T = 256, G = (n + T - 1) / T;
        if (rc == DEM_OK) {
            cudaMemcpyAsync(d_pos, pos, sizeof(float2) * n, cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(d_r, radii, sizeof(float) * n, cudaMemcpyHostToDevice, st);
            cudaMemsetAsync(d_cnt, 0, sizeof(int32_t) * cells, st);
            k_bg_keys<<<G, T, 0, st>>>(d_pos, n, g, d_keys, d_cnt);
            demgb::launch_exclusive_scan(d_cnt, d_start, cells, d_tmp, st);
            k_bg_scatter<<<G, T, 0, st>>>(d_keys, n, d_start, d_cnt, d_order);
            k_bg_select<<<G, T, 0, st>>>(d_pos, d_r, n, g, d_start, d_order, max_bonds, d_sel, d_count);
            demgb::launch_exclusive_scan(d_count, d_base, n, d_tmp, st);
        }
        int32_t total = 0;
        if (rc == DEM_OK) {
            cudaMemcpyAsync(&total, d_base + n, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
            if (cudaStreamSynchronize(st) != cudaSuccess) rc = bfail(DEM_E_CUDA, cudaGetErrorString(cudaGetLastError()));
        }
        if (rc == DEM_OK) {
            *n_bonds = total;
            if (total > bonds_cap || (total > 0 && !bonds))
                rc = bfail(DEM_E_CAPACITY, "bonds_cap is smaller than the bond count written to *n_bonds");
        }
        if (rc == DEM_OK) {
            int32_t *d_bonds = db.get<int32_t>(3 * (size_t)total), *d_bi = db.get<int32_t>(total);
            int32_t *d_bj = db.get<int32_t>(total), *d_in = db.get<int32_t>(n), *d_in_start = db.get<int32_t>(n + 1);
            int32_t *d_list = db.get<int32_t>(total), *d_v2 = db.get<int32_t>(total);
            uint32_t *d_k1 = db.get<uint32_t>(total), *d_k2 = db.get<uint32_t>(total);
            int32_t *d_sc = db.get<int32_t>((size_t)demgb::SORT_GRID_MAX * demgb::SORT_BINS);
            int32_t *d_contacts = db.get<int32_t>((size_t)n * K * 6);
            if (!d_bonds || !d_bi || !d_bj || !d_in || !d_in_start || !d_list || !d_v2 || !d_k1 || !d_k2 ||
                !d_sc || !d_contacts) {
                rc = bfail(DEM_E_OOM, "device allocation failed");
            } else {
                cudaMemsetAsync(d_in, 0, sizeof(int32_t) * n, st);
                k_bg_write<<<G, T, 0, st>>>(n, max_bonds, d_sel, d_count, d_base, d_bonds, d_bi, d_bj, d_in);
                demgb::launch_exclusive_scan(d_in, d_in_start, n, d_tmp, st);
                if (total > 0) {
                    // incoming bonds of every particle in ascending bond number:
                    // passes ping-pong (d_k1, d_v2) / (d_k2, d_list) and end in d_list
                    int dev = 0, sms = 0;
                    cudaGetDevice(&dev);
                    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
                        sms = 1;
                    const int grid = demgb::sort_grid(total, 2 * sms);
                    const int passes = demgb::sort_passes(n);
                    demgb::SortArrays prev{nullptr, nullptr, (int)total, nullptr};
                    for (int p = 0; p < passes; ++p) {
                        const bool last = p == passes - 1;
                        const bool odd = ((passes - 1 - p) & 1) != 0;
                        uint32_t *ok = last ? nullptr : (odd ? d_k1 : d_k2);
                        int32_t *ov = odd ? d_v2 : d_list;
                        if (p == 0) demgb::launch_sort_pass(BgBonds{d_bj, (int)total}, 0, grid, d_sc, ok, ov, st, nullptr);
                        else demgb::launch_sort_pass(prev, 8 * p, grid, d_sc, ok, ov, st, nullptr);
                        prev.key = ok;
                        prev.val = ov;
                    }
                }
                k_bg_slots<<<G, T, 0, st>>>(n, max_bonds, d_count, d_base, d_sel, d_in_start, d_list, d_bi,
                                            d_contacts);
                std::vector<int32_t> bi(total), bj(total);
                if (total > 0) {
                    cudaMemcpyAsync(bonds, d_bonds, sizeof(int32_t) * 3 * (size_t)total, cudaMemcpyDeviceToHost, st);
                    cudaMemcpyAsync(bi.data(), d_bi, sizeof(int32_t) * total, cudaMemcpyDeviceToHost, st);
                    cudaMemcpyAsync(bj.data(), d_bj, sizeof(int32_t) * total, cudaMemcpyDeviceToHost, st);
                }
                cudaMemcpyAsync(contacts, d_contacts, sizeof(int32_t) * (size_t)n * K * 6, cudaMemcpyDeviceToHost, st);
                if (cudaStreamSynchronize(st) != cudaSuccess) {
                    rc = bfail(DEM_E_CUDA, cudaGetErrorString(cudaGetLastError()));
                } else {
                    // length = (dx*dx + dy*dy)^0.5, angle = atan2(dx / |d|, dy / |d|)
                    // (state.rs:309-313)
                    for (int32_t b = 0; b < total; ++b) {
                        const int i = bi[b], j = bj[b];
                        const float dx = pos[2 * j] - pos[2 * i], dy = pos[2 * j + 1] - pos[2 * i + 1];
                        const float mag = std::pow(dx * dx + dy * dy, 0.5f);
                        const float ang = std::atan2(dx / mag, dy / mag);
                        std::memcpy(&bonds[3 * (size_t)b + 1], &ang, 4);
                        std::memcpy(&bonds[3 * (size_t)b + 2], &mag, 4);
                    }
                }
            }
        }
        cudaStreamSynchronize(st);
    }
    cudaStreamDestroy(st);
    return rc;
}

}  // extern "C"

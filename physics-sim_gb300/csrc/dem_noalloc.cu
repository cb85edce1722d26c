// dem_noalloc.cu -- the broad phase for callers that cannot allocate device memory.
//
// dem_broad_phase_noalloc() computes, for n particles given as device float4
// {x, y, radius, -}, their search-cell keys, the particle indices in stable
// cell order and the cell start table -- the three outputs of the context's
// broad phase (dem_debug_broad_phase), with one difference: the context keeps
// a scene's large particles out of the search cells (they head its last
// cell), while here every particle with a radius is keyed by its position and
// the last cell holds the zero-radius particles only -- without calling
// cudaMalloc, cudaFree or any allocating routine.  Its only scratch (one
// counter per cell and one sum per scan tile, then the sort's per-block digit
// counts in the same words) lives in the file-scope device array below, of
// fixed size, which every GPU that loads the library keeps until the process
// exits.  The order comes from the stable counting sort of dem_sort.cuh, with
// the caller's d_keys buffer as its second buffer (the keys are written last).
//
// Who needs this: code that runs where allocation is not allowed or not
// possible -- inside a caller's memory pool that owns the whole device heap,
// under a custom allocator that forbids cudaMalloc, or in a real-time loop
// where an allocation could block -- and therefore hands the library only
// buffers it already owns.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>

#include "dem.h"
#include "dem_sort.cuh"

namespace {

constexpr int NA_THREADS = 256;
constexpr int NA_PER_THREAD = 8;
constexpr int NA_TILE = NA_THREADS * NA_PER_THREAD;
constexpr int NA_TILES_MAX = (DEM_NOALLOC_MAX_CELLS + NA_TILE - 1) / NA_TILE;
static_assert((long long)demgb::SORT_GRID_MAX * demgb::SORT_BINS <= DEM_NOALLOC_MAX_CELLS,
              "the sort passes' digit counts fit in the cell counters");

// counters [0, DEM_NOALLOC_MAX_CELLS) (cell histogram, then the sort's digit
// counts), then tile sums [.., + NA_TILES_MAX + 1)
static __device__ __align__(256) int32_t g_noalloc_scratch[DEM_NOALLOC_MAX_CELLS + NA_TILES_MAX + 1];

constexpr int MAX_DEVICES = 64;
int32_t *g_scratch_ptr[MAX_DEVICES] = {nullptr};
std::mutex g_scratch_mu;
thread_local std::string g_noalloc_error;

int na_fail(int code, const char *msg) {
    g_noalloc_error = msg;
    return code;
}

// Device address of the scratch array on the current device.  The array's
// name in host code is only a host-side handle, so the address is looked up
// once per device with that device current.
int scratch_for_current_device(int32_t **out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES)
        return na_fail(DEM_E_CUDA, "no current CUDA device");
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return na_fail(DEM_E_CUDA, "cudaGetSymbolAddress failed for the scratch array");
        g_scratch_ptr[dev] = static_cast<int32_t *>(p);
    }
    *out = g_scratch_ptr[dev];
    return DEM_OK;
}

__global__ void k_na_zero(int32_t *counts, int c) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < c; i += gridDim.x * blockDim.x) counts[i] = 0;
}

// search-cell key of a particle record
struct NaGrid {
    float x0, y0, inv;
    int gw, gh;
    __device__ __forceinline__ uint32_t key(float4 p) const {
        if (p.z == 0.0f) return (uint32_t)(gw * gh);
        int a = __float2int_rd((p.x - x0) * inv);
        int b = __float2int_rd((p.y - y0) * inv);
        a = a < 0 ? 0 : (a > gw - 1 ? gw - 1 : a);
        b = b < 0 ? 0 : (b > gh - 1 ? gh - 1 : b);
        return (uint32_t)(b * gw + a);
    }
};

constexpr int NA_GRID_CAP = 4096;  // blocks of the per-particle kernels (grid-stride loops)

inline int na_grid(long long n) {
    long long g = (n + 255) / 256;
    return (int)(g < 1 ? 1 : (g > NA_GRID_CAP ? NA_GRID_CAP : g));
}

__global__ void k_na_count(const float4 *__restrict__ pr, int n, NaGrid g, int32_t *counts) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        atomicAdd(&counts[g.key(pr[i])], 1);
}

__global__ void k_na_write_keys(const float4 *__restrict__ pr, int n, NaGrid g, int32_t *__restrict__ keys) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        keys[i] = (int32_t)g.key(pr[i]);
}

// the sort's inputs: the particles in index order (first pass), then the
// previous pass's particle list, keys recomputed from the positions
struct NaFirst {
    const float4 *pr;
    int n;
    NaGrid g;
    __device__ __forceinline__ int length() const { return n; }
    __device__ __forceinline__ bool get(int t, uint32_t &k, int32_t &v) const {
        k = g.key(pr[t]);
        v = t;
        return true;
    }
};
struct NaNext {
    const float4 *pr;
    const int32_t *val;
    int n;
    NaGrid g;
    __device__ __forceinline__ int length() const { return n; }
    __device__ __forceinline__ bool get(int t, uint32_t &k, int32_t &v) const {
        v = val[t];
        k = g.key(pr[v]);
        return true;
    }
};

__device__ __forceinline__ int na_warp_incl(int v) {
    int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

__device__ __forceinline__ int na_block_excl(int v, int *total) {
    __shared__ int wsum[NA_THREADS / 32];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int inc = na_warp_incl(v);
    if (lane == 31) wsum[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int x = lane < NA_THREADS / 32 ? wsum[lane] : 0;
        int y = na_warp_incl(x);
        if (lane < NA_THREADS / 32) wsum[lane] = y - x;
        if (lane == NA_THREADS / 32 - 1) *total = y;
    }
    __syncthreads();
    int r = inc - v + wsum[wid];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(NA_THREADS) k_na_scan_tiles(const int32_t *in, int32_t *out, int n,
                                                              int32_t *tile_sums) {
    __shared__ int total;
    int base = blockIdx.x * NA_TILE + threadIdx.x * NA_PER_THREAD;
    int v[NA_PER_THREAD];
    int sum = 0;
#pragma unroll
    for (int k = 0; k < NA_PER_THREAD; ++k) {
        v[k] = base + k < n ? in[base + k] : 0;
        sum += v[k];
    }
    int off = na_block_excl(sum, &total);
#pragma unroll
    for (int k = 0; k < NA_PER_THREAD; ++k) {
        if (base + k < n) out[base + k] = off;
        off += v[k];
    }
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(NA_THREADS) k_na_scan_sums(int32_t *tile_sums, int ntiles, int32_t *out,
                                                             int n) {
    __shared__ int total;
    int carry = 0;
    for (int base = 0; base < ntiles; base += NA_THREADS) {
        int idx = base + threadIdx.x;
        int v = idx < ntiles ? tile_sums[idx] : 0;
        int off = na_block_excl(v, &total);
        if (idx < ntiles) tile_sums[idx] = carry + off;
        carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) out[n] = carry;
}

__global__ void __launch_bounds__(NA_THREADS) k_na_scan_add(int32_t *out, int n, const int32_t *tile_sums) {
    int add = tile_sums[blockIdx.x];
    int base = blockIdx.x * NA_TILE + threadIdx.x * NA_PER_THREAD;
#pragma unroll
    for (int k = 0; k < NA_PER_THREAD; ++k)
        if (base + k < n) out[base + k] += add;
}

}  // namespace

extern "C" {

const char *dem_noalloc_last_error(void) { return g_noalloc_error.c_str(); }

int dem_broad_phase_noalloc(const float *d_pos_radius, int32_t n, float x0, float y0, float inv_cell,
                            int32_t gw, int32_t gh, int32_t *d_keys, int32_t *d_order,
                            int32_t *d_cell_start, void *stream) {
    if (n < 0 || gw <= 0 || gh <= 0) return na_fail(DEM_E_INVALID, "n must be >= 0 and the grid non-empty");
    if (n > (1 << 30)) return na_fail(DEM_E_CAPACITY, "n is above 2^30 particles");
    if ((long long)gw * gh + 1 > DEM_NOALLOC_MAX_CELLS)
        return na_fail(DEM_E_CAPACITY, "grid has more cells than DEM_NOALLOC_MAX_CELLS (262144, incl. the "
                                       "cell of zero-radius particles)");
    if (!(inv_cell > 0.0f)) return na_fail(DEM_E_INVALID, "inv_cell must be > 0");
    if (!d_cell_start || (n > 0 && (!d_pos_radius || !d_keys || !d_order)))
        return na_fail(DEM_E_INVALID, "a buffer pointer is NULL");
    if (reinterpret_cast<uintptr_t>(d_pos_radius) & 15u)
        return na_fail(DEM_E_INVALID, "d_pos_radius must be 16-byte aligned (float4 records)");
    int32_t *scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int c = gw * gh + 1;
    int32_t *counts = scratch;  // the cell histogram, then the sort passes' digit counts
    int32_t *tile_sums = scratch + DEM_NOALLOC_MAX_CELLS;
    const int ntiles = (c + NA_TILE - 1) / NA_TILE;
    const float4 *pr = reinterpret_cast<const float4 *>(d_pos_radius);
    const NaGrid g{x0, y0, inv_cell, gw, gh};
    k_na_zero<<<(c + 255) / 256, 256, 0, st>>>(counts, c);
    if (n > 0) k_na_count<<<na_grid(n), 256, 0, st>>>(pr, n, g, counts);
    k_na_scan_tiles<<<ntiles, NA_THREADS, 0, st>>>(counts, d_cell_start, c, tile_sums);
    k_na_scan_sums<<<1, NA_THREADS, 0, st>>>(tile_sums, ntiles, d_cell_start, c);
    k_na_scan_add<<<ntiles, NA_THREADS, 0, st>>>(d_cell_start, c, tile_sums);
    if (n > 0) {
        // passes ping-pong between d_keys and d_order and end in d_order
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 1;
        const int grid = demgb::sort_grid(n, 2 * sms);
        const int passes = demgb::sort_passes(c);
        const int32_t *prev = nullptr;
        for (int p = 0; p < passes; ++p) {
            int32_t *out = ((passes - 1 - p) & 1) ? d_keys : d_order;
            if (p == 0) demgb::launch_sort_pass(NaFirst{pr, n, g}, 0, grid, counts, nullptr, out, st, nullptr);
            else demgb::launch_sort_pass(NaNext{pr, prev, n, g}, 8 * p, grid, counts, nullptr, out, st, nullptr);
            prev = out;
        }
        k_na_write_keys<<<na_grid(n), 256, 0, st>>>(pr, n, g, d_keys);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return na_fail(DEM_E_CUDA, cudaGetErrorString(e));
    return DEM_OK;
}

}  // extern "C"

// dem_sort.cuh -- stable counting sort of particle (or bond) indices by an
// integer key, as least-significant-digit passes of 8 bits.
//
// Each pass is a counting sort by one digit that keeps the input order among
// equal digits, so after the passes that cover the key's bits the sequence is
// ordered by key and, within a key, by its position in the input sequence.
// The cost is O(n) per pass whatever the key distribution: a key shared by
// every element (all particles in one cell, every zero-radius particle in a
// scene's dead cell) costs what distinct keys cost.
//
// A pass is three kernels:
//   count    each block counts the digits of its contiguous range of the
//            sequence (warp-aggregated shared-memory counters);
//   offsets  one block turns the per-block counts into global offsets:
//            offset[b][d] = sum of all counts of digits < d + counts of digit d
//            in blocks < b (an exclusive scan over digit-major order);
//   scatter  each block walks its range again in chunks of SORT_CHUNK; within a
//            chunk each warp owns SORT_IPT rounds of 32 consecutive elements and
//            ranks them by a warp multi-split (a ballot per digit bit gives
//            the lanes with the same digit; popc of the lower ones, added to
//            the warp's running digit count), the warps' digit counts are scanned
//            in warp order, and every element is written to
//            offset[digit] + (its rank among the chunk's equal digits).
// Ranks therefore follow the sequence order inside warps, across warps and
// across chunks and blocks: the pass is stable, and no atomics decide any
// position.
//
// The sequence is read through an input object with
//   int length() const            (device side; may read a device word)
//   bool get(int t, uint32_t &key, int32_t &val) const
// returning false for positions that take no part (they are skipped, and the
// counts used to build the cell tables must skip the same positions).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace demgb {

constexpr int SORT_THREADS = 512;
constexpr int SORT_WARPS = SORT_THREADS / 32;
constexpr int SORT_IPT = 8;                          // rounds of 32 elements per warp and chunk
constexpr int SORT_CHUNK = SORT_THREADS * SORT_IPT;  // 4096 elements
constexpr int SORT_BINS = 256;
constexpr int SORT_GRID_MAX = 1024;                  // blocks per pass: offsets hold SORT_GRID_MAX * 256 ints
constexpr int SORT_OFFSET_THREADS = 1024;

// passes of 8 bits that cover keys in [0, key_bound)
inline int sort_passes(long long key_bound) {
    int bits = 0;
    while (bits < 32 && (1LL << bits) < key_bound) ++bits;
    const int p = (bits + 7) / 8;
    return p > 0 ? p : 1;
}

// blocks of every pass over a sequence of at most max_len elements
inline int sort_grid(long long max_len, int cap) {
    long long g = (max_len + SORT_CHUNK - 1) / SORT_CHUNK;
    if (g > cap) g = cap;
    if (g > SORT_GRID_MAX) g = SORT_GRID_MAX;
    return g > 0 ? (int)g : 1;
}

// The lanes of the warp holding the same digit as this lane (d in [0, 256);
// d = 256 marks a lane without an element, whose result is not used): one
// ballot per digit bit, each lane keeping the lanes that agree with it.
__device__ __forceinline__ unsigned digit_peers(int d) {
    unsigned m = __ballot_sync(0xffffffffu, d < SORT_BINS);
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        const bool bit = (d >> b) & 1;
        const unsigned x = __ballot_sync(0xffffffffu, bit);
        m &= bit ? x : ~x;
    }
    return m;
}

__device__ __forceinline__ bool sort_gated_off(const int32_t *gate) {
    return gate != nullptr && *(volatile const int32_t *)gate == 0;
}

// the block's contiguous range of a sequence of len elements over gridDim.x
// blocks (warp-aligned; the same in the count and scatter kernels)
__device__ __forceinline__ void sort_block_range(int len, int &beg, int &end) {
    const long long per = (((long long)len + gridDim.x - 1) / gridDim.x + 31) & ~31LL;
    const long long b = (long long)blockIdx.x * per;
    const long long e = b + per < (long long)len ? b + per : (long long)len;
    beg = (int)(b < (long long)len ? b : (long long)len);
    end = (int)e;
}

// Keys and values of a pass's input held in arrays (the passes after the first).
struct SortArrays {
    const uint32_t *key;
    const int32_t *val;
    int n;                // length, unless n_dev is set
    const int32_t *n_dev; // device word holding the length
    __device__ __forceinline__ int length() const { return n_dev ? *n_dev : n; }
    __device__ __forceinline__ bool get(int t, uint32_t &k, int32_t &v) const {
        k = key[t];
        v = val[t];
        return true;
    }
};

template <class In>
__global__ void __launch_bounds__(SORT_THREADS) k_sort_count(In in, int shift, int32_t *__restrict__ counts,
                                                             const int32_t *gate) {
    if (sort_gated_off(gate)) return;
    __shared__ int h[SORT_BINS];
    for (int d = threadIdx.x; d < SORT_BINS; d += SORT_THREADS) h[d] = 0;
    __syncthreads();
    int beg, end;
    sort_block_range(in.length(), beg, end);
    const int lane = threadIdx.x & 31;
    // chunks of SORT_CHUNK: every element of the thread is requested before
    // any is counted, so the loads overlap instead of following one another;
    // whole warps step together (the ballots need every lane)
    for (int cb = beg; cb < end; cb += SORT_CHUNK) {
        int dig[SORT_IPT];
#pragma unroll
        for (int k = 0; k < SORT_IPT; ++k) {
            const int t = cb + k * SORT_THREADS + (int)threadIdx.x;
            uint32_t kk = 0;
            int32_t vv = 0;
            const bool ok = t < end && in.get(t, kk, vv);
            dig[k] = ok ? (int)((kk >> shift) & 255u) : SORT_BINS;
        }
#pragma unroll
        for (int k = 0; k < SORT_IPT; ++k) {
            const unsigned peers = digit_peers(dig[k]);
            if (dig[k] < SORT_BINS && lane == __ffs(peers) - 1) atomicAdd(&h[dig[k]], __popc(peers));
        }
    }
    __syncthreads();
    for (int d = threadIdx.x; d < SORT_BINS; d += SORT_THREADS) counts[blockIdx.x * SORT_BINS + d] = h[d];
}

// counts[b][d] (g blocks) -> offsets, in place
static __global__ void __launch_bounds__(SORT_OFFSET_THREADS) k_sort_offsets(int32_t *__restrict__ counts, int g,
                                                                      const int32_t *gate) {
    if (sort_gated_off(gate)) return;
    constexpr int Q = SORT_OFFSET_THREADS / SORT_BINS;  // groups of blocks
    __shared__ int part[Q][SORT_BINS];
    __shared__ int wsum[SORT_BINS / 32];
    __shared__ int dbase[SORT_BINS];
    const int d = threadIdx.x % SORT_BINS, q = threadIdx.x / SORT_BINS;
    const int per = (g + Q - 1) / Q;
    const int b0 = q * per, b1 = b0 + per < g ? b0 + per : g;
    int s = 0;
#pragma unroll 16
    for (int b = b0; b < b1; ++b) s += counts[b * SORT_BINS + d];
    part[q][d] = s;
    __syncthreads();
    // exclusive scan of the digit totals by the first 256 threads (8 whole warps)
    int tot = 0, inc = 0;
    if (q == 0) {
#pragma unroll
        for (int x = 0; x < Q; ++x) tot += part[x][d];
        const int lane = d & 31;
        inc = tot;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (lane == 31) wsum[d >> 5] = inc;
    }
    __syncthreads();
    if (q == 0) {
        int add = 0;
        for (int x = 0; x < (d >> 5); ++x) add += wsum[x];
        dbase[d] = inc - tot + add;
    }
    __syncthreads();
    int run = dbase[d];
    for (int x = 0; x < q; ++x) run += part[x][d];
    // groups of 16 counts loaded together, then rewritten as offsets
    for (int b = b0; b < b1; b += 16) {
        int c[16];
#pragma unroll
        for (int u = 0; u < 16; ++u) c[u] = b + u < b1 ? counts[(b + u) * SORT_BINS + d] : 0;
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            if (b + u < b1) counts[(b + u) * SORT_BINS + d] = run;
            run += c[u];
        }
    }
}

// out_key may be null (last pass: only the values are needed).
// Each chunk is first put in digit order in shared memory (stable), then
// written out by consecutive threads, so that the elements of one digit go
// to consecutive addresses in whole runs instead of one scattered word per
// lane.
template <class In>
__global__ void __launch_bounds__(SORT_THREADS) k_sort_scatter(In in, int shift, const int32_t *__restrict__ offsets,
                                                               uint32_t *__restrict__ out_key,
                                                               int32_t *__restrict__ out_val, const int32_t *gate) {
    if (sort_gated_off(gate)) return;
    // per warp and digit: count, then the warp's offset in the digit (at most
    // SORT_CHUNK, so 16 bits; the static shared memory stays under 48 KB)
    __shared__ uint16_t wh[SORT_WARPS * SORT_BINS];
    __shared__ int run[SORT_BINS];              // next global position of each digit
    __shared__ int cbase[SORT_BINS + 1];        // chunk: first staged position of each digit; [256] = total
    __shared__ int wsum[SORT_BINS / 32];
    __shared__ uint32_t skey[SORT_CHUNK];
    __shared__ int32_t sval[SORT_CHUNK];
    int beg, end;
    sort_block_range(in.length(), beg, end);
    if (beg >= end) return;  // uniform for the block
    for (int d = threadIdx.x; d < SORT_BINS; d += SORT_THREADS) run[d] = offsets[blockIdx.x * SORT_BINS + d];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned below = (1u << lane) - 1u;
    uint16_t *my = wh + warp * SORT_BINS;
    for (int cb = beg; cb < end; cb += SORT_CHUNK) {
        for (int d = lane; d < SORT_BINS; d += 32) my[d] = 0;
        __syncwarp();
        uint32_t key[SORT_IPT];
        int32_t val[SORT_IPT];
        int dig[SORT_IPT], off[SORT_IPT];
        const int w0 = cb + warp * (32 * SORT_IPT);
        // every element of the thread requested before any is ranked
#pragma unroll
        for (int k = 0; k < SORT_IPT; ++k) {
            const int t = w0 + k * 32 + lane;  // < end + SORT_CHUNK <= INT_MAX (lengths are at most 2^30)
            uint32_t kk = 0;
            int32_t vv = 0;
            const bool ok = t < end && in.get(t, kk, vv);
            key[k] = kk;
            val[k] = vv;
            dig[k] = ok ? (int)((kk >> shift) & 255u) : SORT_BINS;
        }
        // rank among the warp's elements of the same digit, in sequence order
#pragma unroll
        for (int k = 0; k < SORT_IPT; ++k) {
            const int d = dig[k];
            const unsigned peers = digit_peers(d);
            int o = 0;
            if (d < SORT_BINS) o = my[d] + __popc(peers & below);
            __syncwarp();
            if (d < SORT_BINS && lane == __ffs(peers) - 1) my[d] = (uint16_t)(my[d] + __popc(peers));
            __syncwarp();
            off[k] = o;
        }
        __syncthreads();
        // per digit: the warps' counts become offsets in warp (= sequence)
        // order; the digit totals are scanned into the chunk's staging order
        int tot = 0;
        if (threadIdx.x < SORT_BINS) {
            const int d = threadIdx.x;
            int s2 = 0;
#pragma unroll
            for (int x = 0; x < SORT_WARPS; ++x) {
                const int c = wh[x * SORT_BINS + d];
                wh[x * SORT_BINS + d] = (uint16_t)s2;
                s2 += c;
            }
            tot = s2;
            int inc = tot;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += y;
            }
            if (lane == 31) wsum[d >> 5] = inc;
            cbase[d] = inc - tot;
        }
        __syncthreads();
        if (threadIdx.x < SORT_BINS) {
            const int d = threadIdx.x;
            int add = 0;
            for (int x = 0; x < (d >> 5); ++x) add += wsum[x];
            cbase[d] += add;
            if (d == SORT_BINS - 1) cbase[SORT_BINS] = cbase[d] + tot;
        }
        __syncthreads();
        // stage in digit order
#pragma unroll
        for (int k = 0; k < SORT_IPT; ++k) {
            if (dig[k] < SORT_BINS) {
                const int q = cbase[dig[k]] + my[dig[k]] + off[k];
                skey[q] = key[k];
                sval[q] = val[k];
            }
        }
        __syncthreads();
        // write out: consecutive staged elements of a digit to consecutive places
        const int staged = cbase[SORT_BINS];
        for (int q = threadIdx.x; q < staged; q += SORT_THREADS) {
            const uint32_t kk = skey[q];
            const int d = (int)((kk >> shift) & 255u);
            const int p = run[d] + (q - cbase[d]);
            if (out_key) out_key[p] = kk;
            out_val[p] = sval[q];
        }
        __syncthreads();
        // the next chunk of each digit goes after this one's
        if (threadIdx.x < SORT_BINS) run[threadIdx.x] += cbase[threadIdx.x + 1] - cbase[threadIdx.x];
        __syncthreads();
    }
}

// One counting pass: counts, offsets, scatter (3 launches).
template <class In>
inline void launch_sort_pass(const In &in, int shift, int g, int32_t *counts, uint32_t *out_key, int32_t *out_val,
                             cudaStream_t st, const int32_t *gate) {
    k_sort_count<In><<<g, SORT_THREADS, 0, st>>>(in, shift, counts, gate);
    k_sort_offsets<<<1, SORT_OFFSET_THREADS, 0, st>>>(counts, g, gate);
    k_sort_scatter<In><<<g, SORT_THREADS, 0, st>>>(in, shift, counts, out_key, out_val, gate);
}

}  // namespace demgb

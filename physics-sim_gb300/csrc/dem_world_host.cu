// dem_world_host.cu -- host owner of the device world (see dem_world_host.h).
#include <sched.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <climits>
#include <limits>
#include <memory>
#include <thread>

#include "dem_sort.cuh"
#include "dem_world_host.h"

namespace demgb {

#define CK(call)                                                                      \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess) return fail(DEM_E_CUDA, std::string(#call) + ": " +     \
                                               cudaGetErrorString(e_));               \
    } while (0)

static inline int32_t f2bits(float f) {
    int32_t i;
    std::memcpy(&i, &f, 4);
    return i;
}
static inline float bits2f(int32_t i) {
    float f;
    std::memcpy(&f, &i, 4);
    return f;
}

void RangeAlloc::reset(long long capacity) {
    free_.clear();
    cap_ = capacity;
    used_ = 0;
    if (capacity > 0) free_[0] = capacity;
}

long long RangeAlloc::alloc(long long n) {
    if (n <= 0) return 0;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
        if (it->second >= n) {
            long long off = it->first, len = it->second;
            free_.erase(it);
            if (len > n) free_[off + n] = len - n;
            used_ += n;
            return off;
        }
    }
    return -1;
}

void RangeAlloc::release(long long off, long long n) {
    if (n <= 0) return;
    used_ -= n;
    auto it = free_.emplace(off, n).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
        it->second += nx->second;
        free_.erase(nx);
    }
    if (it != free_.begin()) {
        auto pv = std::prev(it);
        if (pv->first + pv->second == it->first) {
            pv->second += it->second;
            free_.erase(it);
        }
    }
}

World::~World() {
    set_timing(true);
    set_timing(false);
    release();
    if (ref_block) cudaFree(ref_block);
    if (pin) cudaFreeHost(pin);
    if (d_items) cudaFree(d_items);
    if (d_copies) cudaFree(d_copies);
    for (auto e : xfer_ev) cudaEventDestroy(e);
    if (side) cudaStreamDestroy(side);
}

// staging area for one scene of n particles in the reference layouts:
// 117 words per particle (contacts 84, forces 6, fixity 6, data 7, the rest 14)
int World::ensure_ref(long long n) {
    if (n <= ref_cap && ref_block) return DEM_OK;
    if (ref_block) cudaFree(ref_block);
    ref_block = nullptr;
    ref_cap = 0;
    const long long cap = (std::max(n, 1024LL) + 63) & ~63LL;  // every field 256-byte aligned
    const size_t words = (size_t)cap * 117 + 64;
    if (cudaMalloc(&ref_block, words * 4) != cudaSuccess) {
        ref_block = nullptr;
        return fail(DEM_E_OOM, "staging allocation failed");
    }
    float *f = static_cast<float *>(ref_block);
    auto take = [&](size_t per) {
        float *p = f;
        f += per * (size_t)cap;
        return p;
    };
    ref.pos = take(2);
    ref.radii = take(1);
    ref.vel = take(2);
    ref.acc = take(2);
    ref.rot = take(1);
    ref.rot_vel = take(1);
    ref.rot_acc = take(1);
    ref.forces = take(6);
    ref.del_pos = take(2);
    ref.del_rot = take(1);
    ref.data = take(7);
    ref.fixity = reinterpret_cast<int32_t *>(take(6));
    ref.contacts = reinterpret_cast<int32_t *>(take(84));
    ref.material_pointers = reinterpret_cast<int32_t *>(take(1));
    ref_cap = cap;
    return DEM_OK;
}

// The staging block's fields in order: words per particle and the scene
// array each one mirrors (the device block and the pinned host block share
// this layout, field f at base * cap words).
namespace {
struct RefField {
    int per;
    size_t base;  // words per particle before this field
};
constexpr int N_REF_FIELDS = 14, F_CONTACTS = 12, REF_WORDS = 117;
constexpr RefField REF_FIELDS[N_REF_FIELDS] = {
    {2, 0}, {1, 2}, {2, 3}, {2, 5}, {1, 7}, {1, 8}, {1, 9}, {6, 10}, {2, 16}, {1, 18}, {7, 19}, {6, 26}, {84, 32}, {1, 116}};
// the fields k_stage_out writes (fixity, forces and material pointers are
// read from the world's reference mirrors instead)
constexpr bool OUT_FIELD[N_REF_FIELDS] = {true, true, true, true, true, true, true,
                                          false, true, true, true, false, true, false};
const void *scene_field(const dem_scene *sc, int f) {
    switch (f) {
        case 0: return sc->pos;
        case 1: return sc->radii;
        case 2: return sc->vel;
        case 3: return sc->acc;
        case 4: return sc->rot;
        case 5: return sc->rot_vel;
        case 6: return sc->rot_acc;
        case 7: return sc->forces;
        case 8: return sc->del_pos;
        case 9: return sc->del_rot;
        case 10: return sc->data;
        case 11: return sc->fixity;
        case 12: return sc->contacts;
        default: return sc->material_pointers;
    }
}

// the device reads and writes pageable host memory through the host's page
// tables (hardware-coherent hosts such as Grace)
bool device_reads_pageable() {
    int dev = 0, a = 0, b = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    if (cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) return false;
    if (cudaDeviceGetAttribute(&b, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess)
        return false;
    return a == 1 && b == 1;
}

// cores this process may run on
int host_threads() {
    static const int n = [] {
        int c = (int)std::thread::hardware_concurrency();
        cpu_set_t set;
        CPU_ZERO(&set);
        if (sched_getaffinity(0, sizeof set, &set) == 0) c = CPU_COUNT(&set);
        return std::max(1, c);
    }();
    return n;
}

// run fn(k) for k in [0, count) on up to host_threads() threads
template <class F>
void par_for(int count, F fn) {
    const int T = std::max(1, std::min(count, host_threads()));
    if (T == 1) {
        for (int k = 0; k < count; ++k) fn(k);
        return;
    }
    std::vector<std::thread> pool;
    for (int t = 0; t < T; ++t)
        pool.emplace_back([&, t]() {
            for (int k = t; k < count; k += T) fn(k);
        });
    for (auto &th : pool) th.join();
}

// Host copying beside the transfers.  Chunk c holds units [cum[c], cum[c+1]);
// threads take units in order.  A unit of chunk c starts once the chunk is
// released (downloads release a chunk when its copy has landed; uploads
// start with every chunk released) and wait_chunk(c) returns once all of
// chunk c's units have run (uploads then issue its copy).
class HostPipe {
  public:
    HostPipe(const std::vector<long long> &sizes, bool gated)
        : n_chunks((int)sizes.size()),
          cum(sizes.size() + 1, 0),
          ready(new std::atomic<int>[sizes.size() + 1]),
          left(new std::atomic<long long>[sizes.size() + 1]) {
        for (int c = 0; c < n_chunks; ++c) {
            cum[c + 1] = cum[c] + sizes[c];
            ready[c].store(gated ? 0 : 1);
            left[c].store(sizes[c]);
        }
    }
    ~HostPipe() {
        cancel();
        join();
    }
    template <class F>
    void start(F unit) {
        const int T = (int)std::max(1LL, std::min<long long>(cum[n_chunks], host_threads()));
        for (int t = 0; t < T; ++t)
            pool.emplace_back([this, unit]() {
                for (;;) {
                    const long long u = next.fetch_add(1);
                    if (u >= cum[n_chunks]) return;
                    const int c = (int)(std::upper_bound(cum.begin(), cum.end(), u) - cum.begin()) - 1;
                    while (!ready[c].load(std::memory_order_acquire)) {
                        if (stop.load()) return;
                        std::this_thread::yield();
                    }
                    if (stop.load()) return;
                    unit(c, u - cum[c]);
                    left[c].fetch_sub(1, std::memory_order_acq_rel);
                }
            });
    }
    void wait_chunk(int c) {
        while (left[c].load(std::memory_order_acquire) > 0) std::this_thread::yield();
    }
    void release(int c) { ready[c].store(1, std::memory_order_release); }
    void cancel() { stop.store(1); }
    void join() {
        for (auto &th : pool) th.join();
        pool.clear();
    }

  private:
    int n_chunks;
    std::vector<long long> cum;
    std::unique_ptr<std::atomic<int>[]> ready;
    std::unique_ptr<std::atomic<long long>[]> left;
    std::atomic<long long> next{0};
    std::atomic<int> stop{0};
    std::vector<std::thread> pool;
};

// byte offsets of the regions of one pinned transfer block (16-byte aligned)
struct PinMap {
    size_t bytes = 0;
    size_t take(size_t n) {
        const size_t at = bytes;
        bytes += (n + 15) & ~(size_t)15;
        return at;
    }
};

// [start, start + len) ranges of one array, sorted and merged where they touch
std::vector<std::pair<long long, long long>> merge_runs(std::vector<std::pair<long long, long long>> r) {
    std::sort(r.begin(), r.end());
    std::vector<std::pair<long long, long long>> out;
    for (const auto &x : r) {
        if (x.second <= 0) continue;
        if (!out.empty() && out.back().first + out.back().second == x.first) out.back().second += x.second;
        else out.push_back(x);
    }
    return out;
}

// table items [0, count) in up to `groups` consecutive ranges of about equal
// particle counts
std::vector<std::pair<int, int>> split_items(const std::vector<StageItem> &tab, int groups) {
    std::vector<std::pair<int, int>> g;
    long long total = 0;
    for (const auto &it : tab) total += it.n;
    int i0 = 0;
    long long acc = 0;
    for (int i = 0; i < (int)tab.size(); ++i) {
        acc += tab[i].n;
        if (acc * groups >= total * ((long long)g.size() + 1) || i + 1 == (int)tab.size()) {
            g.emplace_back(i0, i + 1);
            i0 = i + 1;
        }
    }
    return g;
}

// material records and the material-pair stiffness table of one scene:
// 1/(1/k_a + 1/k_b) for normal and shear stiffness (2D_Simulation.wgsl:345-346),
// in float arithmetic, division correctly rounded
void material_tables(const float *materials, int M, Mat *mats, float2 *pair) {
    for (int k = 0; k < M; ++k) {
        const float *mm = materials + 6 * k;
        mats[k] = Mat{mm[3], mm[4], mm[5], 0.0f};
    }
    for (int a = 0; a < M; ++a)
        for (int b = 0; b < M; ++b) {
            volatile float kna = mats[a].kn, knb = mats[b].kn, ksa = mats[a].ks, ksb = mats[b].ks;
            volatile float ia = 1.0f / kna, ib = 1.0f / knb;
            volatile float sum = ia + ib;
            volatile float kn = 1.0f / sum;
            volatile float ja = 1.0f / ksa, jb = 1.0f / ksb;
            volatile float sum2 = ja + jb;
            volatile float ks = 1.0f / sum2;
            pair[(size_t)a * M + b] = make_float2(kn, ks);
        }
}

// appends one copy of `bytes` to a direct transfer's table; returns the
// pieces so far
long long add_copy(HostCopy *tab, int &n, const void *src, void *dst, long long bytes, long long pieces) {
    if (bytes <= 0 || !src || !dst) return pieces;
    tab[n++] = HostCopy{static_cast<const char *>(src), static_cast<char *>(dst), bytes, pieces};
    return pieces + (bytes + COPY_PIECE - 1) / COPY_PIECE;
}

// a transfer's items: the scenes with particles in call order, each starting
// on a multiple of 4 particles (every field of every item 16-byte aligned)
long long pack_items(const std::vector<SceneHost> &sh, const int32_t *idx, int count, std::vector<StageItem> &tab,
                     std::vector<int> &tab_k) {
    long long total = 0;
    for (int k = 0; k < count; ++k) {
        const SceneHost &h = sh[idx[k]];
        if (h.n <= 0) continue;
        const long long off = (total + 3) & ~3LL;
        tab.push_back(StageItem{off, h.particle_base, h.n, idx[k], h.n_mat, h.n_bonds, 0, h.r_big, 0});
        tab_k.push_back(k);
        total = off + h.n;
    }
    return total;
}

// a scene's bond records [status, angle, length bits] split into the
// device arrays' words (strengths from the scene's per-bond values, else 0)
void split_bonds(const SceneHost &h, const int32_t *bonds, int32_t *st, float *len, float2 *str, int32_t *ang) {
    for (int k = 0; k < h.n_bonds; ++k) {
        st[k] = bonds[3 * k];
        ang[k] = bonds[3 * k + 1];
        len[k] = bits2f(bonds[3 * k + 2]);
        str[k] = make_float2(h.bond_sn.empty() ? 0.0f : h.bond_sn[k], h.bond_ss.empty() ? 0.0f : h.bond_ss[k]);
    }
}
}  // namespace

// page-locked host staging of the bulk transfers (grows, kept)
int World::ensure_pin(size_t bytes) {
    if (bytes <= pin_bytes && pin) return DEM_OK;
    if (pin) cudaFreeHost(pin);
    pin = nullptr;
    pin_bytes = 0;
    if (cudaHostAlloc(&pin, bytes, cudaHostAllocDefault) != cudaSuccess) {
        pin = nullptr;
        return fail(DEM_E_OOM, "pinned staging allocation failed");
    }
    pin_bytes = bytes;
    return DEM_OK;
}

// device tables of a transfer: its items with one check word each (plus
// their OR), and its direct copies (grow, kept)
int World::ensure_tables(int items, int copies) {
    if (items > items_cap || !d_items) {
        if (d_items) cudaFree(d_items);
        d_items = nullptr;
        d_item_err = nullptr;
        items_cap = 0;
        const int cap = std::max(items, 64);
        void *p = nullptr;
        if (cudaMalloc(&p, (size_t)cap * (sizeof(StageItem) + 4)) != cudaSuccess)
            return fail(DEM_E_OOM, "staging table allocation failed");
        d_items = static_cast<StageItem *>(p);
        d_item_err = reinterpret_cast<int32_t *>(d_items + cap);
        items_cap = cap;
    }
    if (copies > copies_cap || !d_copies) {
        if (d_copies) cudaFree(d_copies);
        d_copies = nullptr;
        copies_cap = 0;
        const int cap = std::max(copies, 1024);
        if (cudaMalloc(&d_copies, (size_t)cap * sizeof(HostCopy)) != cudaSuccess) {
            d_copies = nullptr;
            return fail(DEM_E_OOM, "copy table allocation failed");
        }
        copies_cap = cap;
    }
    return DEM_OK;
}

// one event per pipelined transfer chunk (created once, kept)
int World::ensure_events(int count) {
    while ((int)xfer_ev.size() < count) {
        cudaEvent_t e = nullptr;
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
            return fail(DEM_E_CUDA, "event creation failed");
        xfer_ev.push_back(e);
    }
    return DEM_OK;
}

int World::fail(int code, const std::string &msg) {
    err = msg;
    return code;
}

void World::release() {
    drop_graph();
    for (void *p : owned) cudaFree(p);
    owned.clear();
    d = DevWorld{};
    spare = DevWorld{};
    live_d = nullptr;
}

// served worlds: the 128-particle chunks that hold a particle of a scene in
// use (the step kernels skip the others)
int World::update_live() {
    if (!live_d) return DEM_OK;
    const size_t chunks = ((size_t)d.N + 127) / 128;
    std::vector<uint8_t> live(chunks, 0);
    for (size_t s = 0; s < sh.size(); ++s) {
        const SceneHost &h = sh[s];
        if ((int)s == free_slot || h.n <= 0) continue;
        for (size_t c = (size_t)h.particle_base / 128; c <= ((size_t)h.particle_base + h.n - 1) / 128; ++c)
            live[c] = 1;
    }
    CK(cudaMemcpyAsync(live_d, live.data(), chunks, cudaMemcpyHostToDevice, stream));
    CK(cudaStreamSynchronize(stream));
    return DEM_OK;
}

template <class T>
static T *dalloc(std::vector<void *> &owned, size_t count, bool &ok) {
    if (!ok) return nullptr;
    void *p = nullptr;
    if (count == 0) count = 1;
    if (cudaMalloc(&p, count * sizeof(T)) != cudaSuccess) {
        ok = false;
        return nullptr;
    }
    owned.push_back(p);
    return static_cast<T *>(p);
}

int World::alloc(int N, int C, int B, int S, int M, int MP, int TB, uint32_t ev_cap) {
    release();
    bool ok = true;
    DevWorld &w = d;
    w.N = N; w.C = C; w.B = B; w.S = S; w.M = M; w.MP = MP;
    w.ticket = N <= TICKET_MAX_N ? 1 : 0;
    w.split = split_narrow ? 1 : 0;
    auto particle_arrays = [&](DevWorld &x) {
        x.pr = dalloc<float4>(owned, N, ok);
        x.vw = dalloc<float4>(owned, N, ok);
        x.ac = dalloc<float4>(owned, N, ok);
        x.dp = dalloc<float4>(owned, N, ok);
        x.fx = dalloc<float4>(owned, N, ok);
        x.d4 = dalloc<float4>(owned, N, ok);
        x.dF = dalloc<float4>(owned, N, ok);
        x.meta = dalloc<uint32_t>(owned, N, ok);
        x.orig = dalloc<int32_t>(owned, N, ok);
        x.o2i = dalloc<int32_t>(owned, N, ok);
        x.smask = dalloc<uint32_t>(owned, N, ok);
        x.s_b = dalloc<int32_t>(owned, (size_t)K * N, ok);
        x.s_bonded = dalloc<int32_t>(owned, (size_t)K * N, ok);
        x.s_tf = dalloc<float>(owned, (size_t)K * N, ok);
        x.s_btf = dalloc<float>(owned, (size_t)K * N, ok);
        x.s_thb = dalloc<float>(owned, (size_t)K * N, ok);
    };
    particle_arrays(w);
    w.pr_n = dalloc<float4>(owned, N, ok);
    w.dp_n = dalloc<float4>(owned, N, ok);
    parity = 0;
    w.b_status = dalloc<int32_t>(owned, B, ok);
    w.b_length = dalloc<float>(owned, B, ok);
    w.b_str = dalloc<float2>(owned, B, ok);
    w.mats = dalloc<Mat>(owned, M, ok);
    w.pair = dalloc<float2>(owned, MP, ok);
    w.par = dalloc<ScenePar>(owned, S, ok);
    w.cc3 = dalloc<int32_t>(owned, S, ok);
    w.keys = dalloc<uint32_t>(owned, N, ok);
    w.cell_count = dalloc<int32_t>(owned, C, ok);
    w.cell_start = dalloc<int32_t>(owned, (size_t)C + 1, ok);
    w.sorted = dalloc<int32_t>(owned, N, ok);
    w.inv = dalloc<int32_t>(owned, N, ok);
    w.src = dalloc<int32_t>(owned, N, ok);
    w.wperm = dalloc<int32_t>(owned, N, ok);
    w.sort_counts = dalloc<int32_t>(owned, (size_t)SORT_GRID_MAX * SORT_BINS, ok);
    w.scan_tmp = dalloc<int32_t>(owned, scan_tmp_size(C), ok);
    w.pend_cap = (uint32_t)std::max<long long>(2LL * B + 64, 64);
    w.pend = dalloc<Pending>(owned, w.pend_cap, ok);
    w.pend_count = dalloc<uint32_t>(owned, 1, ok);
    w.ev_cap = ev_cap;
    w.ev = dalloc<Event>(owned, ev_cap, ok);
    w.ev_count = dalloc<unsigned long long>(owned, 1, ok);
    w.stats = dalloc<unsigned long long>(owned, 6, ok);
    w.step = dalloc<long long>(owned, 1, ok);
    w.err = dalloc<int32_t>(owned, 1, ok);
    w.nl = dalloc<int4>(owned, 2 * (size_t)N, ok);
    w.pbuild = dalloc<float2>(owned, N, ok);
    w.kbuild = dalloc<uint32_t>(owned, N, ok);
    w.rebuild = dalloc<int32_t>(owned, 1, ok);
    w.reorder = dalloc<int32_t>(owned, 1, ok);
    // default: every 3rd rebuild in a single-scene world (a dense scene's
    // warps gain from fresh grouping by contact count), every 8th in a
    // batch or server (many sparse scenes: the reorder's bytes dominate)
    w.reorder_every = reorder_every > 0 ? reorder_every : (S == 1 ? 3 : 8);
    w.tickets = dalloc<uint32_t>(owned, 2, ok);
    w.fix_ref = dalloc<int32_t>(owned, 6 * (size_t)N, ok);
    w.force_ref = dalloc<float>(owned, 6 * (size_t)N, ok);
    w.matp_ref = dalloc<int32_t>(owned, N, ok);
    w.data3 = dalloc<float>(owned, N, ok);
    w.n_big_slots = TB;
    w.big_acc = dalloc<int32_t>(owned, 16 * (size_t)std::max(TB, 1), ok);
    w.big_scene = dalloc<int32_t>(owned, std::max(TB, 1), ok);
    w.det = dalloc<int32_t>(owned, S, ok);
    w.act = dalloc<int32_t>(owned, S, ok);
    w.remaining = dalloc<long long>(owned, S, ok);
    spare = w;
    particle_arrays(spare);
    if (!ok) {
        release();
        return fail(DEM_E_OOM, "device allocation failed");
    }
    CK(cudaMemsetAsync(w.cell_count, 0, sizeof(int32_t) * (size_t)C, stream));
    CK(cudaMemsetAsync(w.pend_count, 0, sizeof(uint32_t), stream));
    CK(cudaMemsetAsync(w.ev_count, 0, sizeof(unsigned long long), stream));
    CK(cudaMemsetAsync(w.stats, 0, 6 * sizeof(unsigned long long), stream));
    CK(cudaMemsetAsync(w.tickets, 0, 2 * sizeof(uint32_t), stream));
    CK(cudaMemsetAsync(w.nl, 0, sizeof(int4) * 2 * (size_t)(N > 0 ? N : 1), stream));
    CK(cudaMemsetAsync(w.err, 0, sizeof(int32_t), stream));
    {
        static const int32_t one = 1;  // the first rebuild reorders
        CK(cudaMemcpyAsync(w.reorder, &one, 4, cudaMemcpyHostToDevice, stream));
    }
    CK(cudaMemsetAsync(w.big_scene, 0xFF, sizeof(int32_t) * (size_t)std::max(TB, 1), stream));
    CK(cudaMemsetAsync(w.big_acc, 0, sizeof(int32_t) * 16 * (size_t)std::max(TB, 1), stream));
    CK(cudaMemsetAsync(w.cc3, 0, sizeof(int32_t) * (size_t)S, stream));
    CK(cudaMemsetAsync(w.act, 0, sizeof(int32_t) * (size_t)S, stream));
    CK(cudaMemcpyAsync(w.step, &host_step, sizeof(long long), cudaMemcpyHostToDevice, stream));
    CK(cudaStreamSynchronize(stream));
    return DEM_OK;
}

// ---- scene validation and grid geometry -----------------------------------
int World::compute_layout(SceneHost &h, const dem_scene *sc) {
    if (!sc) return fail(DEM_E_INVALID, "scene is NULL");
    const int n = sc->n_particles;
    if (n < 0) return fail(DEM_E_INVALID, "n_particles < 0");
    if (sc->n_bonds < 0) return fail(DEM_E_INVALID, "n_bonds < 0");
    if (sc->n_materials <= 0 || sc->n_materials > MAX_MATERIALS)
        return fail(DEM_E_INVALID, "n_materials must be in [1, 256]");
    if (n > 0 && (!sc->pos || !sc->radii || !sc->vel || !sc->acc || !sc->rot || !sc->rot_vel ||
                  !sc->rot_acc || !sc->forces || !sc->fixity || !sc->del_pos || !sc->del_rot ||
                  !sc->contacts || !sc->material_pointers))
        return fail(DEM_E_INVALID, "a required scene array is NULL");
    if (!sc->materials) return fail(DEM_E_INVALID, "materials is NULL");
    if (sc->n_bonds > 0 && !sc->bonds) return fail(DEM_E_INVALID, "bonds is NULL");
    h.n = n;
    h.n_bonds = sc->n_bonds;
    h.n_mat = sc->n_materials;
    // One pass over the particles: the first invalid one, the largest
    // radius, the bounding box of the finite positions of nonzero radii, and
    // the large-particle threshold: 4x the median of the nonzero radii when
    // few particles (at most max(64, n/256)) lie above it; the search cells
    // are then sized by the largest of the others.  Large scenes split the
    // pass over host threads (results identical: the lowest invalid index
    // decides the message, the reductions do not depend on order, and the
    // median is selected exactly).
    const int T = n >= (1 << 18) ? std::max(1, std::min(layout_threads, n >> 16)) : 1;
    struct Part {
        int bad = INT_MAX, bad_kind = 0;
        float rmax = 0.0f, xmin = 0, xmax = 0, ymin = 0, ymax = 0;
        bool any = false;
        std::vector<uint32_t> hist;  // nonzero radii by their 16 high bits
    };
    std::vector<Part> parts(T);
    auto scan = [&](int t) {
        Part &q = parts[t];
        const int i0 = (int)((long long)n * t / T), i1 = (int)((long long)n * (t + 1) / T);
        if (T > 1) q.hist.assign(1 << 16, 0u);
        for (int i = i0; i < i1; ++i) {
            const float r = sc->radii[i];
            if (!(r >= 0.0f) || !std::isfinite(r)) {
                q.bad = i;
                q.bad_kind = 1;
                return;
            }
            q.rmax = std::max(q.rmax, r);
            const int32_t mp = sc->material_pointers[i];
            if (mp < 0 || mp >= sc->n_materials) {
                q.bad = i;
                q.bad_kind = 2;
                return;
            }
            const float x = sc->pos[2 * i], y = sc->pos[2 * i + 1];
            if (std::isfinite(x) && std::isfinite(y) && r > 0.0f) {
                if (!q.any) {
                    q.xmin = q.xmax = x;
                    q.ymin = q.ymax = y;
                    q.any = true;
                }
                q.xmin = std::min(q.xmin, x);
                q.xmax = std::max(q.xmax, x);
                q.ymin = std::min(q.ymin, y);
                q.ymax = std::max(q.ymax, y);
            }
            if (T > 1 && r > 0.0f) {
                uint32_t bits;
                std::memcpy(&bits, &r, 4);
                q.hist[bits >> 16]++;
            }
        }
    };
    if (T == 1) {
        scan(0);
    } else {
        std::vector<std::thread> pool;
        for (int t = 0; t < T; ++t) pool.emplace_back(scan, t);
        for (auto &th : pool) th.join();
    }
    float rmax = 0.0f;
    float xmin = 0, xmax = 0, ymin = 0, ymax = 0;
    bool any = false;
    {
        int bad = INT_MAX, kind = 0;
        for (const Part &q : parts)
            if (q.bad < bad) {
                bad = q.bad;
                kind = q.bad_kind;
            }
        if (kind == 1) return fail(DEM_E_INVALID, "radius must be finite and >= 0");
        if (kind == 2) return fail(DEM_E_INVALID, "material pointer out of range");
        for (const Part &q : parts) {
            rmax = std::max(rmax, q.rmax);
            if (!q.any) continue;
            if (!any) {
                xmin = q.xmin; xmax = q.xmax; ymin = q.ymin; ymax = q.ymax;
                any = true;
            }
            xmin = std::min(xmin, q.xmin); xmax = std::max(xmax, q.xmax);
            ymin = std::min(ymin, q.ymin); ymax = std::max(ymax, q.ymax);
        }
    }
    // contact records are checked on the device as they are staged (stage_many)
    h.r_big = std::numeric_limits<float>::infinity();
    h.n_big = 0;
    {
        // the median of the nonzero radii: the element of rank m/2 in
        // ascending order (what nth_element at rs.size()/2 returns)
        float med = 0.0f;
        long long m = 0;
        if (T == 1) {
            std::vector<float> rs;
            rs.reserve(n);
            for (int i = 0; i < n; ++i)
                if (sc->radii[i] > 0.0f) rs.push_back(sc->radii[i]);
            m = (long long)rs.size();
            if (m > 0) {
                std::nth_element(rs.begin(), rs.begin() + m / 2, rs.end());
                med = rs[m / 2];
            }
        } else {
            // positive floats order as their bit patterns: find the 16-bit
            // bucket holding rank m/2, then select inside that bucket
            std::vector<uint64_t> hist(1 << 16, 0);
            for (const Part &q : parts)
                for (int b = 0; b < (1 << 16); ++b) hist[b] += q.hist[b];
            for (int b = 0; b < (1 << 16); ++b) m += (long long)hist[b];
            if (m > 0) {
                long long k = m / 2, below = 0;
                int bucket = 0;
                while (below + (long long)hist[bucket] <= k) below += (long long)hist[bucket++];
                std::vector<std::vector<float>> ins(T);
                std::vector<std::thread> pool;
                for (int t = 0; t < T; ++t)
                    pool.emplace_back([&, t]() {
                        const int i0 = (int)((long long)n * t / T), i1 = (int)((long long)n * (t + 1) / T);
                        for (int i = i0; i < i1; ++i) {
                            const float r = sc->radii[i];
                            uint32_t bits;
                            std::memcpy(&bits, &r, 4);
                            if (r > 0.0f && (int)(bits >> 16) == bucket) ins[t].push_back(r);
                        }
                    });
                for (auto &th : pool) th.join();
                std::vector<float> in;
                in.reserve(hist[bucket]);
                for (const auto &v : ins) in.insert(in.end(), v.begin(), v.end());
                std::nth_element(in.begin(), in.begin() + (k - below), in.end());
                med = in[k - below];
            }
        }
        if (m > 0) {
            const float thr = 4.0f * med;
            std::vector<long long> cnts(T, 0);
            std::vector<float> smalls(T, 0.0f);
            auto count = [&](int t) {
                const int i0 = (int)((long long)n * t / T), i1 = (int)((long long)n * (t + 1) / T);
                long long c = 0;
                float rs = 0.0f;
                for (int i = i0; i < i1; ++i) {
                    const float r = sc->radii[i];
                    if (!(r > 0.0f)) continue;
                    if (r > thr) ++c;
                    else rs = std::max(rs, r);
                }
                cnts[t] = c;
                smalls[t] = rs;
            };
            if (T == 1) {
                count(0);
            } else {
                std::vector<std::thread> pool;
                for (int t = 0; t < T; ++t) pool.emplace_back(count, t);
                for (auto &th : pool) th.join();
            }
            long long cnt = 0;
            float rsmall = 0.0f;
            for (int t = 0; t < T; ++t) {
                cnt += cnts[t];
                rsmall = std::max(rsmall, smalls[t]);
            }
            if (cnt > 0 && cnt <= std::max(64, n / 256)) {
                h.r_big = thr;
                h.n_big = (int)cnt;
                rmax = rsmall;
            }
        }
    }
    h.r_max = rmax;
    // reference bucket grid
    dem_grid_info g = sc->grid;
    if (!(g.cell_size > 0.0f) || g.w <= 0 || g.h <= 0) {
        if (dem_grid_capacity(&h.params, sc->radii, n, n, &g) != 0)
            return fail(DEM_E_INVALID, "cannot derive the bucket grid");
    }
    h.grid = g;
    // search grid: centre-binned cells of side >= 2 r_max (1 + pad), covering the
    // walls (or the particles, whichever is smaller in cells)
    const dem_params &p = h.params;
    h.skin = skin_factor * rmax;
    // cell side = factor x (2 r_max + skin); below 1 the searches span 5 x 5
    // cells (stencil 2), so the factor may go down to 0.5
    const float factor = std::max(h.cell_factor, 0.5f);
    const int stencil = factor < 1.0f ? 2 : 1;
    float reach = std::max(2.0f * rmax + h.skin, 1e-30f) * factor;
    double ex0, ex1, ey0, ey1;
    if (p.round_bounds == 0) {
        ex0 = -0.5 * p.hor_bound; ex1 = 0.5 * p.hor_bound;
        ey0 = -0.5 * p.vert_bound; ey1 = 0.5 * p.vert_bound;
    } else {
        ex0 = ey0 = -(double)p.bound_radius;
        ex1 = ey1 = (double)p.bound_radius;
    }
    if (any) {
        ex0 = std::min(ex0, (double)xmin); ex1 = std::max(ex1, (double)xmax);
        ey0 = std::min(ey0, (double)ymin); ey1 = std::max(ey1, (double)ymax);
    }
    double cap_cells = std::max(4.0 * n, 65536.0);
    double span_x = (ex1 - ex0) + 2.0 * reach, span_y = (ey1 - ey0) + 2.0 * reach;
    // no particle with a nonzero radius (an empty scene): nothing to search
    if (!any || !(span_x > 0) || !(span_y > 0) || !std::isfinite(span_x) || !std::isfinite(span_y)) {
        span_x = span_y = 2.0 * reach;
        ex0 = ey0 = -reach; ex1 = ey1 = reach;
    }
    if ((span_x / reach) * (span_y / reach) > cap_cells && any) {
        ex0 = xmin; ex1 = xmax; ey0 = ymin; ey1 = ymax;
        span_x = (ex1 - ex0) + 2.0 * reach;
        span_y = (ey1 - ey0) + 2.0 * reach;
    }
    double qmax = std::max(span_x, span_y) / reach + 2.0;
    double pad = 3e-5 + 8.0 * std::ldexp(1.0, -24) * qmax;
    float gcs = (float)(reach * (1.0 + pad));
    int gw = (int)std::ceil(span_x / gcs) + 1;
    int gh = (int)std::ceil(span_y / gcs) + 1;
    gw = std::max(gw, 1);
    gh = std::max(gh, 1);
    if ((double)gw * gh > 2.0e9) return fail(DEM_E_INVALID, "search grid too large");
    h.n_cells = gw * gh + 2;  // search cells, the large particles' cell, the dead cell
    ScenePar &P = h.par;
    std::memset(&P, 0, sizeof P);
    P.g_cs = gcs;
    P.g_inv = 1.0f / gcs;
    P.g_x0 = (float)(ex0 - reach);
    P.g_y0 = (float)(ey0 - reach);
    P.g_w = gw;
    P.g_h = gh;
    P.stencil = stencil;
    return DEM_OK;
}

void World::fill_par(SceneHost &h) {
    ScenePar &P = h.par;
    P.p = h.params;
    P.p.particles = h.n;
    P.xW = h.params.hor_bound / 2.0f;
    P.yH = h.params.vert_bound / 2.0f;
    P.ref_cs = h.grid.cell_size;
    P.ref_w = h.grid.w;
    P.ref_h = h.grid.h;
    P.ref_base_x = ((-h.grid.cell_size) * (float)h.grid.w) * 0.5f;
    P.ref_base_y = (h.grid.cell_size * (float)h.grid.h) * 0.5f;
    P.cell_base = h.cell_base;
    P.dead_cell = h.cell_base + h.n_cells - 1;
    P.big_cell = h.cell_base + P.g_w * P.g_h;
    P.big_base = h.big_base;
    P.n_big = h.n_big;
    P.r_grid = h.r_max;
    P.particle_base = h.particle_base;
    P.n_particles = h.n;
    P.bond_base = h.bond_base;
    P.mat_base = h.mat_base;
    P.n_mat = h.n_mat;
    P.use_f64 = h.use_f64;
    P.lambda = h.lambda;
    P.damp2 = h.damp2;
    P.has_strength = h.bond_sn.empty() ? 0 : 1;
    P.active = h.active ? 1 : 0;
    P.step0 = h.step0;
    P.cc1_0 = h.cc1_0;
    P.pair_base = h.pair_base;
    {
        const float kb = h.params.bond_normal_stiffness, ksb = h.params.bond_shear_stiffness;
        P.kb2 = 1.0f / (1.0f / kb + 1.0f / kb);
        P.ksb2 = 1.0f / (1.0f / ksb + 1.0f / ksb);
    }
    P.skin = h.skin;
    const float half = 0.5f * h.skin * (1.0f - 1e-5f);
    P.disp_limit2 = half * half;
}

// narrow-phase flags of the coming step, one per scene
int World::push_det() {
    std::vector<int32_t> det(sh.size());
    for (size_t s = 0; s < sh.size(); ++s)
        det[s] = detect_at(sh[s].params.collision_interval, sh[s].cc1_0, host_step - sh[s].step0) ? 1 : 0;
    CK(cudaMemcpyAsync(d.det, det.data(), det.size() * 4, cudaMemcpyHostToDevice, stream));
    CK(cudaStreamSynchronize(stream));
    return DEM_OK;
}

// the next step rebuilds the cell table, the particle order and the candidate lists
// (reorder: and reorders the particle arrays into cell order -- after
// uploads, which leave a scene's particles in scene-local order; an admitted
// or retired scene, moved walls or positions set from outside only need new
// cell lists, and the regular reorder interval restores the order later)
int World::force_rebuild(bool reorder) {
    static const int32_t one = 1;
    CK(cudaMemcpyAsync(d.rebuild, &one, 4, cudaMemcpyHostToDevice, stream));
    if (reorder) CK(cudaMemcpyAsync(d.reorder, &one, 4, cudaMemcpyHostToDevice, stream));
    CK(cudaStreamSynchronize(stream));
    return DEM_OK;
}

// big-partner records [big_base, big_base + big_cap) of scene s belong to
// `scene_or_free` (-1: unused)
int World::push_bigs(int s, int scene_or_free) {
    const SceneHost &h = sh[s];
    if (h.big_cap <= 0) return DEM_OK;
    std::vector<int32_t> v(h.big_cap, scene_or_free);
    CK(cudaMemcpyAsync(d.big_scene + h.big_base, v.data(), 4 * (size_t)h.big_cap, cudaMemcpyHostToDevice, stream));
    CK(cudaStreamSynchronize(stream));
    update_has_bigs();
    return DEM_OK;
}

// k_big_narrow is part of the step only while some scene has large
// particles; the captured graphs follow when that changes
void World::update_has_bigs() {
    bool any = false;
    for (const auto &h : sh) any |= h.big_cap > 0;
    if (any != has_bigs) {
        has_bigs = any;
        drop_graph();
    }
}

int World::push_par(int s) {
    fill_par(sh[s]);
    CK(cudaMemcpyAsync(d.par + s, &sh[s].par, sizeof(ScenePar), cudaMemcpyHostToDevice, stream));
    return DEM_OK;
}

// a scene steps (act = 1) for `steps` more steps, or freezes (act = 0)
int World::push_active(int s, bool on, long long steps) {
    int32_t a = on ? 1 : 0;
    long long r = steps;
    CK(cudaMemcpyAsync(d.act + s, &a, 4, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d.remaining + s, &r, 8, cudaMemcpyHostToDevice, stream));
    CK(cudaStreamSynchronize(stream));
    sh[s].active = on;
    return DEM_OK;
}

// ---- staging: reference layout -> internal layout --------------------------
int World::stage_error(int32_t e) {
    if (e & 1) return fail(DEM_E_INVALID, "material pointer out of range");
    if (e & 2) return fail(DEM_E_INVALID, "contact bonded index beyond n_bonds");
    if (e & 4) return fail(DEM_E_INVALID, "contact partner out of range");
    if (e & 8) return fail(DEM_E_INVALID, "contact record's a differs from its owner");
    return DEM_OK;
}

// Staging of `count` scenes (idx[k] from scs[k]).  Every scene's arrays go
// into the staging block -- read by the device straight from the caller's
// memory (host_direct), else copied by host threads into the page-locked
// block as it is sent one field at a time -- and one launch checks them
// all.  `layouts` runs on the host meanwhile (before, on the page-locked
// route) and fills probes[k] with re-uploads' new layouts; a failure there
// or in a check ends the transfer before any scene changed.  Then the
// layouts are adopted, one launch converts every scene, and the bonds,
// materials and scene parameters follow in merged transfers.
int World::stage_many(const int32_t *idx, const dem_scene *const *scs, int count, const SceneHost *probes,
                      const std::function<int()> &layouts) {
    std::vector<StageItem> tab;
    std::vector<int> tab_k;
    const long long total = pack_items(sh, idx, count, tab, tab_k);
    const int nt = (int)tab.size();
    for (int i = 0; i < nt; ++i) tab[i].has_data = scs[tab_k[i]]->data ? 1 : 0;
    int rc = ensure_ref(std::max(total, 1LL));
    if (rc) return rc;
    rc = ensure_tables(nt + 1, N_REF_FIELDS * nt + 1);
    if (rc) return rc;
    PinMap pm;
    const size_t o_fields = host_direct ? 0 : pm.take((size_t)ref_cap * REF_WORDS * 4);
    const size_t o_copies = pm.take(sizeof(HostCopy) * ((size_t)N_REF_FIELDS * nt + 1));
    const size_t o_items = pm.take(sizeof(StageItem) * (size_t)(nt + 1));
    const size_t o_err = pm.take(4 * (size_t)(nt + 1));
    const size_t o_bst = pm.take(4 * (size_t)d.B), o_blen = pm.take(4 * (size_t)d.B);
    const size_t o_bstr = pm.take(8 * (size_t)d.B), o_bang = pm.take(4 * (size_t)d.B);
    const size_t o_mats = pm.take(sizeof(Mat) * (size_t)d.M), o_pair = pm.take(8 * (size_t)d.MP);
    const size_t o_par = pm.take(sizeof(ScenePar) * sh.size());
    rc = ensure_pin(pm.bytes);
    if (rc) return rc;
    char *pb = static_cast<char *>(pin);
    float *hp = reinterpret_cast<float *>(pb + o_fields);
    int32_t *h_err = reinterpret_cast<int32_t *>(pb + o_err);
    int32_t *h_bst = reinterpret_cast<int32_t *>(pb + o_bst);
    float *h_blen = reinterpret_cast<float *>(pb + o_blen);
    float2 *h_bstr = reinterpret_cast<float2 *>(pb + o_bstr);
    int32_t *h_bang = reinterpret_cast<int32_t *>(pb + o_bang);
    Mat *h_mats = reinterpret_cast<Mat *>(pb + o_mats);
    float2 *h_pair = reinterpret_cast<float2 *>(pb + o_pair);
    ScenePar *h_par = reinterpret_cast<ScenePar *>(pb + o_par);
    float *dp0 = static_cast<float *>(ref_block);
    cudaError_t ce = cudaSuccess;
    if (host_direct) {
        HostCopy *hc = reinterpret_cast<HostCopy *>(pb + o_copies);
        int nc = 0;
        long long pieces = 0;
        for (int i = 0; i < nt; ++i)
            for (int f = 0; f < N_REF_FIELDS; ++f) {
                const RefField &F = REF_FIELDS[f];
                pieces = add_copy(hc, nc, scene_field(scs[tab_k[i]], f), dp0 + F.base * ref_cap + F.per * tab[i].off,
                                  4LL * F.per * tab[i].n, pieces);
            }
        if (nc > 0) {
            ce = cudaMemcpyAsync(d_copies, hc, sizeof(HostCopy) * nc, cudaMemcpyHostToDevice, stream);
            if (ce == cudaSuccess) {
                launch_copies(d_copies, nc, pieces, nullptr, stream);
                ce = cudaGetLastError();
            }
        }
        rc = layouts ? layouts() : DEM_OK;
        if (rc != DEM_OK || ce != cudaSuccess) {
            cudaStreamSynchronize(stream);  // the tables in the page-locked block are in use until then
            return ce != cudaSuccess ? fail(DEM_E_CUDA, cudaGetErrorString(ce)) : rc;
        }
    } else {
        rc = layouts ? layouts() : DEM_OK;
        if (rc) return rc;
        struct Chunk {
            int f, i0, i1;
        };
        std::vector<Chunk> chunks;
        std::vector<long long> sizes;
        for (int f = 0; f < N_REF_FIELDS && nt > 0; ++f)
            for (const auto &g : split_items(tab, f == F_CONTACTS ? 8 : 1)) {
                chunks.push_back(Chunk{f, g.first, g.second});
                sizes.push_back(g.second - g.first);
            }
        HostPipe pipe(sizes, false);
        pipe.start([&](int c, long long u) {
            const Chunk &ch = chunks[c];
            const int i = ch.i0 + (int)u;
            const void *src = scene_field(scs[tab_k[i]], ch.f);
            if (!src) return;
            const RefField &F = REF_FIELDS[ch.f];
            std::memcpy(hp + F.base * ref_cap + F.per * tab[i].off, src, sizeof(float) * F.per * (size_t)tab[i].n);
        });
        for (int c = 0; c < (int)chunks.size(); ++c) {
            pipe.wait_chunk(c);
            const Chunk &ch = chunks[c];
            if (ce != cudaSuccess) continue;
            const RefField &F = REF_FIELDS[ch.f];
            const long long o0 = tab[ch.i0].off, o1 = tab[ch.i1 - 1].off + tab[ch.i1 - 1].n;
            ce = cudaMemcpyAsync(dp0 + F.base * ref_cap + F.per * o0, hp + F.base * ref_cap + F.per * o0,
                                 sizeof(float) * F.per * (size_t)(o1 - o0), cudaMemcpyHostToDevice, stream);
        }
        pipe.join();
    }
    // bonds and material tables of every scene into the page-locked block
    par_for(count, [&](int k) {
        const SceneHost &h = sh[idx[k]];
        if (h.n_bonds > 0)
            split_bonds(h, scs[k]->bonds, h_bst + h.bond_base, h_blen + h.bond_base, h_bstr + h.bond_base,
                        h_bang + h.bond_base);
        material_tables(scs[k]->materials, h.n_mat, h_mats + h.mat_base, h_pair + h.pair_base);
    });
    // the items with their (new) large-particle thresholds; one check launch
    for (int i = 0; i < nt; ++i) tab[i].r_big = probes ? probes[tab_k[i]].r_big : sh[tab[i].scene].r_big;
    std::memcpy(pb + o_items, tab.data(), sizeof(StageItem) * nt);
    if (ce == cudaSuccess && nt > 0) {
        ce = cudaMemcpyAsync(d_items, pb + o_items, sizeof(StageItem) * nt, cudaMemcpyHostToDevice, stream);
        if (ce == cudaSuccess) ce = cudaMemsetAsync(d_item_err, 0, 4 * (size_t)(nt + 1), stream);
        if (ce == cudaSuccess) {
            launch_stage_check(ref, d_items, nt, total, d_item_err, stream);
            ce = cudaGetLastError();
        }
        if (ce == cudaSuccess)
            ce = cudaMemcpyAsync(h_err, d_item_err, 4 * (size_t)nt, cudaMemcpyDeviceToHost, stream);
    }
    {
        // waited for even after a failed call: until then the copies may be
        // reading the callers' arrays
        const cudaError_t se = cudaStreamSynchronize(stream);
        if (ce == cudaSuccess) ce = se;
    }
    if (ce != cudaSuccess) return fail(DEM_E_CUDA, cudaGetErrorString(ce));
    for (int i = 0; i < nt; ++i)
        if (h_err[i]) {
            rc = stage_error(h_err[i]);
            err += " (scene " + std::to_string(tab[i].scene) + ")";
            return rc;
        }
    // every scene passed: adopt, convert, and send bonds, materials, parameters
    std::vector<std::pair<long long, long long>> rb, rm, rp, rs;
    for (int k = 0; k < count; ++k) {
        const int s = idx[k];
        SceneHost &h = sh[s];
        if (probes) apply_layout(s, probes[k]);
        h.materials.assign(scs[k]->materials, scs[k]->materials + 6 * (size_t)h.n_mat);
        h.bond_angle.assign(h_bang + h.bond_base, h_bang + h.bond_base + h.n_bonds);
        fill_par(h);
        h_par[s] = h.par;
        rb.emplace_back(h.bond_base, h.n_bonds);
        rm.emplace_back(h.mat_base, h.n_mat);
        rp.emplace_back(h.pair_base, (long long)h.n_mat * h.n_mat);
        rs.emplace_back(s, 1);
    }
    launch_stage_in(d, ref, d_items, nt, total, stream);
    CK(cudaGetLastError());
    auto send = [&](void *dst, const void *src, size_t elem, const std::vector<std::pair<long long, long long>> &r) {
        for (const auto &x : merge_runs(r)) {
            cudaError_t e2 = cudaMemcpyAsync(static_cast<char *>(dst) + elem * x.first,
                                             static_cast<const char *>(src) + elem * x.first, elem * x.second,
                                             cudaMemcpyHostToDevice, stream);
            if (e2 != cudaSuccess) return e2;
        }
        return cudaSuccess;
    };
    CK(send(d.b_status, h_bst, 4, rb));
    CK(send(d.b_length, h_blen, 4, rb));
    CK(send(d.b_str, h_bstr, 8, rb));
    CK(send(d.mats, h_mats, sizeof(Mat), rm));
    CK(send(d.pair, h_pair, 8, rp));
    CK(send(d.par, h_par, sizeof(ScenePar), rs));
    CK(cudaStreamSynchronize(stream));  // the page-locked block is reused by the next transfer
    return DEM_OK;
}

int World::push_materials(int s) {
    SceneHost &h = sh[s];
    const int M = h.n_mat;
    std::vector<Mat> mats(M);
    std::vector<float2> pair((size_t)M * M);
    material_tables(h.materials.data(), M, mats.data(), pair.data());
    CK(cudaMemcpyAsync(d.mats + h.mat_base, mats.data(), M * sizeof(Mat), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d.pair + h.pair_base, pair.data(), pair.size() * sizeof(float2),
                       cudaMemcpyHostToDevice, stream));
    CK(cudaStreamSynchronize(stream));
    return DEM_OK;
}

int World::build(const std::vector<const dem_scene *> &scenes, const std::vector<dem_params> &params,
                 const std::vector<dem_ext> &exts) {
    const int S = (int)scenes.size();
    if (S <= 0 || S > MAX_SCENES) return fail(DEM_E_INVALID, "scene count out of range");
    if ((int)params.size() != S || (int)exts.size() != S) return fail(DEM_E_INVALID, "one params/ext per scene");
    const dem_ext &ext = exts[0];  // world-wide options come from the first scene's ext
    if (ext.block_size) {
        if (ext.block_size < 32 || ext.block_size > 1024 || (ext.block_size & 31))
            return fail(DEM_E_INVALID, "block_size must be a multiple of 32 in [32, 1024]");
        block = ext.block_size;
    }
    if (ext.reorder_interval < 0) return fail(DEM_E_INVALID, "reorder_interval < 0");
    if (ext.reorder_interval > 0) graph_steps = ext.reorder_interval;
    if (ext.list_skin < 0.0f) return fail(DEM_E_INVALID, "list_skin < 0");
    if (ext.list_skin > 0.0f) skin_factor = ext.list_skin;
    if (ext.reorder_every < 0) return fail(DEM_E_INVALID, "reorder_every < 0");
    if (ext.reorder_every > 0) reorder_every = ext.reorder_every;
    use_graphs = ext.plain_launches == 0;
    split_narrow = ext.split_narrow != 0;
    fuse_lom = ext.unfused_lom == 0;
    host_direct = ext.host_copies == 0 && device_reads_pageable();
    layout_threads = host_threads();
    diagnostics = ext.diagnostics != 0;
    sh.assign(S, SceneHost{});
    long long N = 0, C = 0, B = 0, M = 0, MP = 0, TB = 0;
    for (int s = 0; s < S; ++s) {
        SceneHost &h = sh[s];
        const dem_ext &e = exts[s];
        if (!(e.bond_lambda > 0.0f)) return fail(DEM_E_INVALID, "bond_lambda must be > 0");
        h.params = params[s];
        h.use_f64 = e.use_f64 ? 1 : 0;
        h.lambda = e.bond_lambda;
        if (!(e.restitution >= 0.0f && e.restitution <= 1.0f)) return fail(DEM_E_INVALID, "restitution not in [0, 1]");
        h.damp2 = dashpot_factor(e.restitution);
        h.cell_factor = ext.search_cell_factor > 0.0f ? ext.search_cell_factor : 1.0f;
        int rc = compute_layout(h, scenes[s]);
        if (rc) return rc;
        if (e.bond_normal_strength && h.n_bonds > 0)
            h.bond_sn.assign(e.bond_normal_strength, e.bond_normal_strength + h.n_bonds);
        if (e.bond_shear_strength && h.n_bonds > 0)
            h.bond_ss.assign(e.bond_shear_strength, e.bond_shear_strength + h.n_bonds);
        if (h.bond_sn.empty() != h.bond_ss.empty()) {
            if (h.bond_sn.empty()) h.bond_sn.assign(h.n_bonds, params[s].bond_normal_strength);
            if (h.bond_ss.empty()) h.bond_ss.assign(h.n_bonds, params[s].bond_shear_strength);
        }
        h.particle_base = (int)N;
        h.cell_base = (int)C;
        h.bond_base = (int)B;
        h.mat_base = (int)M;
        h.pair_base = (int)MP;
        h.big_base = (int)TB;
        h.big_cap = h.n_big;
        h.step0 = host_step;
        h.cc0_0 = scenes[s]->coll_cont[0];
        h.cc1_0 = scenes[s]->coll_cont[1];
        h.cc2_0 = scenes[s]->coll_cont[2];
        N += h.n;
        C += h.n_cells;
        B += h.n_bonds;
        M += h.n_mat;
        MP += (long long)h.n_mat * h.n_mat;
        TB += h.n_big;
    }
    if (N > MAX_WORLD_PARTICLES || C > (1LL << 30) || B > (1LL << 30))
        return fail(DEM_E_INVALID, "world too large (particles, search cells or bonds beyond the limits in dem.h)");
    uint32_t ev_cap = ext.event_capacity > 0 ? (uint32_t)ext.event_capacity : 1u << 16;
    int rc = alloc((int)N, (int)C, (int)B, S, (int)M, (int)MP, (int)TB, ev_cap);
    if (rc) return rc;
    update_has_bigs();
    {
        std::vector<int32_t> all(S);
        for (int s = 0; s < S; ++s) all[s] = s;
        rc = stage_many(all.data(), scenes.data(), S, nullptr, nullptr);
        if (rc) return rc;
    }
    for (int s = 0; s < S; ++s) {
        rc = push_bigs(s, s);
        if (rc) return rc;
        rc = push_par(s);
        if (rc) return rc;
        rc = push_active(s, true, LLONG_MAX);
        if (rc) return rc;
        int32_t c3 = scenes[s]->coll_cont[3];
        CK(cudaMemcpyAsync(d.cc3 + s, &c3, 4, cudaMemcpyHostToDevice, stream));
    }
    CK(cudaStreamSynchronize(stream));
    rc = push_det();
    if (rc) return rc;
    update_kernel_form();
    return force_rebuild();
}

// the Simulation kernels compiled for what the scenes need (launch_interact):
// the double-precision paths only while some scene uses the F64 distances
// (they cost the FP32 scenes registers), and one bond model built in when
// every scene with bonds uses it (served worlds, whose scenes come and go,
// do not specialise on the model); a change recaptures the graphs.  A scene
// without bond records steps alike under every model: uploads refuse a
// contact whose bonded field names no bond record (>= n_bonds), so none of
// its slots is bonded, and the models differ only for bonded slots.
// 2 zeta of the normal dashpot for restitution e (0: off; e = 1 gives 0,
// no damping): zeta = -ln e / sqrt(pi^2 + ln^2 e), in double, rounded once
float dashpot_factor(float e) {
    if (!(e > 0.0f) || e >= 1.0f) return 0.0f;
    const double l = std::log((double)e);
    return (float)(2.0 * (-l / std::sqrt(M_PI * M_PI + l * l)));
}

void World::update_kernel_form() {
    unsigned models = 0u;
    bool f64 = false;
    for (size_t s = 0; s < sh.size(); ++s) {
        if ((int)s == free_slot) continue;
        const SceneHost &h = sh[s];
        if (h.n_bonds > 0)
            models |= (h.params.bonds >= 0 && h.params.bonds <= 3) ? 1u << h.params.bonds : 0xFu;
        f64 |= h.use_f64 != 0 || h.damp2 > 0.0f;  // the generic kernels carry the F64 paths and the dashpot
    }
    int form = f64 ? -1 : -2;
    if (!f64 && free_slot < 0) form = (models == 1u || models == 0u) ? 0 : models == 8u ? 3 : -2;
    if (form != kernel_form) {
        kernel_form = form;
        drop_graph();
    }
}

long long World::bytes_per_particle() const {
    // live + spare particle records, slots, broad phase and candidate lists
    const long long rec = 7 * 16 + 3 * 4 + (long long)K * 5 * 4;
    return 2 * rec + 4 * 4 + 4 + 32 + 8 + 4;
}

int World::build_capacity(long long particles, long long cells, long long bonds, int scenes, int materials,
                          const dem_ext &ext) {
    if (particles <= 0 || cells <= 0 || scenes <= 0 || materials <= 0)
        return fail(DEM_E_INVALID, "capacities must be positive");
    if (scenes >= MAX_SCENES) return fail(DEM_E_INVALID, "too many scene slots");
    if (particles > MAX_WORLD_PARTICLES || cells > (1LL << 30) || bonds > (1LL << 30))
        return fail(DEM_E_INVALID, "capacity too large (particles, search cells or bonds beyond the limits in dem.h)");
    if (ext.block_size) {
        if (ext.block_size < 32 || ext.block_size > 1024 || (ext.block_size & 31))
            return fail(DEM_E_INVALID, "block_size must be a multiple of 32 in [32, 1024]");
        block = ext.block_size;
    }
    if (ext.reorder_interval > 0) graph_steps = ext.reorder_interval;
    if (ext.list_skin > 0.0f) skin_factor = ext.list_skin;
    if (ext.reorder_every < 0) return fail(DEM_E_INVALID, "reorder_every < 0");
    if (ext.reorder_every > 0) reorder_every = ext.reorder_every;
    use_graphs = ext.plain_launches == 0;
    split_narrow = ext.split_narrow != 0;
    fuse_lom = ext.unfused_lom == 0;
    host_direct = ext.host_copies == 0 && device_reads_pageable();
    layout_threads = host_threads();
    diagnostics = ext.diagnostics != 0;
    const int S = scenes + 1;  // the last slot owns the unused particles
    free_slot = scenes;
    sh.assign(S, SceneHost{});
    for (auto &h : sh) {
        h.active = false;
        h.params.collision_interval = 1;
    }
    const long long pairs = (long long)materials * 16;
    uint32_t ev_cap = ext.event_capacity > 0 ? (uint32_t)ext.event_capacity : 1u << 18;
    const long long bigs = std::max(64LL, particles / 1024);
    int rc = alloc((int)particles, (int)cells, (int)std::max(bonds, 1LL), S, materials, (int)pairs, (int)bigs,
                   ev_cap);
    if (rc) return rc;
    launch_mark_free(d, 0, (int)particles, free_slot, stream);
    {
        // the live map: every chunk free until a scene is admitted
        bool ok = true;
        const size_t chunks = ((size_t)particles + 127) / 128;
        live_d = dalloc<uint8_t>(owned, chunks, ok);
        if (!ok) return fail(DEM_E_OOM, "live map allocation failed");
        CK(cudaMemsetAsync(live_d, 0, chunks, stream));
        d.live = live_d;
    }
    a_big.reset(bigs);
    a_part.reset(particles);
    a_cell.reset(cells);
    a_bond.reset(std::max(bonds, 1LL));
    a_mat.reset(materials);
    a_pair.reset(pairs);
    free_slots.clear();
    for (int s = scenes - 1; s >= 0; --s) free_slots.push_back(s);
    for (int s = 0; s < S; ++s) {
        SceneHost &h = sh[s];
        h.cell_base = 0;
        h.n_cells = 1;
        h.par.g_w = h.par.g_h = 1;
        h.par.g_inv = 1.0f;
        h.grid.cell_size = 1.0f;
        h.grid.w = h.grid.h = 1;
        rc = push_par(s);
        if (rc) return rc;
        rc = push_active(s, false, 0);
        if (rc) return rc;
    }
    CK(cudaStreamSynchronize(stream));
    rc = push_det();
    if (rc) return rc;
    return force_rebuild();
}

int World::admit(const dem_scene *sc, const dem_params &params, const dem_ext &e, long long horizon) {
    if (free_slots.empty()) return fail(DEM_E_CAPACITY, "no free scene slot");
    if (horizon <= 0) return fail(DEM_E_INVALID, "horizon must be > 0");
    if (!(e.bond_lambda > 0.0f)) return fail(DEM_E_INVALID, "bond_lambda must be > 0");
    SceneHost h;
    h.params = params;
    h.use_f64 = e.use_f64 ? 1 : 0;
    h.lambda = e.bond_lambda;
    if (!(e.restitution >= 0.0f && e.restitution <= 1.0f)) return fail(DEM_E_INVALID, "restitution not in [0, 1]");
    h.damp2 = dashpot_factor(e.restitution);
    h.cell_factor = 1.0f;
    int rc = compute_layout(h, sc);
    if (rc) return rc;
    if (h.n_mat > 16) return fail(DEM_E_CAPACITY, "served scenes carry at most 16 materials");
    long long pp = a_part.alloc(h.n);
    long long pc = pp >= 0 ? a_cell.alloc(h.n_cells) : -1;
    long long pb = pc >= 0 ? a_bond.alloc(h.n_bonds) : -1;
    long long pm = pb >= 0 ? a_mat.alloc(h.n_mat) : -1;
    long long pq = pm >= 0 ? a_pair.alloc((long long)h.n_mat * h.n_mat) : -1;
    long long pg = pq >= 0 ? (h.n_big > 0 ? a_big.alloc(h.n_big) : 0) : -1;
    if (pg < 0) {
        if (pq >= 0) a_pair.release(pq, (long long)h.n_mat * h.n_mat);
        if (pm >= 0) a_mat.release(pm, h.n_mat);
        if (pb >= 0) a_bond.release(pb, h.n_bonds);
        if (pc >= 0) a_cell.release(pc, h.n_cells);
        if (pp >= 0) a_part.release(pp, h.n);
        return fail(DEM_E_CAPACITY, "no free range large enough");
    }
    const int s = free_slots.back();
    free_slots.pop_back();
    h.particle_base = (int)pp;
    h.cell_base = (int)pc;
    h.bond_base = (int)pb;
    h.mat_base = (int)pm;
    h.pair_base = (int)pq;
    h.big_base = (int)pg;
    h.big_cap = h.n_big;
    if (e.bond_normal_strength && h.n_bonds > 0)
        h.bond_sn.assign(e.bond_normal_strength, e.bond_normal_strength + h.n_bonds);
    if (e.bond_shear_strength && h.n_bonds > 0)
        h.bond_ss.assign(e.bond_shear_strength, e.bond_shear_strength + h.n_bonds);
    if (h.bond_sn.empty() != h.bond_ss.empty()) {
        if (h.bond_sn.empty()) h.bond_sn.assign(h.n_bonds, params.bond_normal_strength);
        if (h.bond_ss.empty()) h.bond_ss.assign(h.n_bonds, params.bond_shear_strength);
    }
    h.step0 = host_step;
    h.cc0_0 = sc->coll_cont[0];
    h.cc1_0 = sc->coll_cont[1];
    h.cc2_0 = sc->coll_cont[2];
    h.active = true;
    sh[s] = h;
    {
        const int32_t one = s;
        rc = stage_many(&one, &sc, 1, nullptr, nullptr);
    }
    if (rc == DEM_OK) rc = push_bigs(s, s);
    if (rc == DEM_OK) rc = push_par(s);
    if (rc == DEM_OK) {
        int32_t c3 = sc->coll_cont[3];
        cudaError_t ce = cudaMemcpyAsync(d.cc3 + s, &c3, 4, cudaMemcpyHostToDevice, stream);
        if (ce != cudaSuccess) rc = fail(DEM_E_CUDA, cudaGetErrorString(ce));
    }
    if (rc == DEM_OK) rc = push_active(s, true, horizon);
    if (rc == DEM_OK) rc = push_det();
    if (rc == DEM_OK) rc = update_live();
    if (rc == DEM_OK) update_kernel_form();
    if (rc == DEM_OK) rc = force_rebuild(false);
    if (rc != DEM_OK) {
        retire(s);
        return rc;
    }
    return s;
}

int World::retire(int s) {
    if (s < 0 || s >= (int)sh.size() || s == free_slot) return fail(DEM_E_INVALID, "bad scene slot");
    SceneHost &h = sh[s];
    int rc = push_active(s, false, 0);
    if (rc) return rc;
    launch_mark_free(d, h.particle_base, h.n, free_slot, stream);
    CK(cudaStreamSynchronize(stream));
    a_part.release(h.particle_base, h.n);
    a_cell.release(h.cell_base, h.n_cells);
    a_bond.release(h.bond_base, h.n_bonds);
    a_mat.release(h.mat_base, h.n_mat);
    a_pair.release(h.pair_base, (long long)h.n_mat * h.n_mat);
    if (h.big_cap > 0) {
        rc = push_bigs(s, -1);
        if (rc) return rc;
        a_big.release(h.big_base, h.big_cap);
    }
    h = SceneHost{};
    h.params.collision_interval = 1;
    h.n_cells = 1;
    free_slots.push_back(s);
    rc = update_live();
    if (rc) return rc;
    update_kernel_form();
    return force_rebuild(false);
}

// A re-uploaded scene keeps its cell budget and large-particle records and
// adopts the new geometry inside them: layout_fits checks, apply_layout adopts.
int World::layout_fits(int s, const SceneHost &probe) {
    const SceneHost &h = sh[s];
    if (probe.n_cells > h.n_cells)
        return fail(DEM_E_UNSUPPORTED, "uploaded scene needs a larger search grid; create a new context");
    if (probe.n_big > h.big_cap)
        return fail(DEM_E_UNSUPPORTED, "uploaded scene has more large particles; create a new context");
    return DEM_OK;
}

void World::apply_layout(int s, const SceneHost &probe) {
    SceneHost &h = sh[s];
    h.r_max = probe.r_max;
    h.r_big = probe.r_big;
    h.n_big = probe.n_big;
    h.grid = probe.grid;
    h.par.g_cs = probe.par.g_cs;
    h.par.g_inv = probe.par.g_inv;
    h.par.g_x0 = probe.par.g_x0;
    h.par.g_y0 = probe.par.g_y0;
    h.par.g_w = probe.par.g_w;
    h.par.g_h = probe.par.g_h;
}

// Many scenes at once (dem_batch_upload_many): the new layouts are derived
// on host threads while the arrays travel; nothing of any scene changes
// unless every scene passes.
int World::upload_many(const int32_t *idx, const dem_scene *const *scs, int count) {
    if (count <= 0) return DEM_OK;
    if (!idx || !scs) return fail(DEM_E_INVALID, "scene index/pointer arrays are NULL");
    std::vector<SceneHost> probes(count);
    std::vector<char> seen(sh.size(), 0);
    for (int k = 0; k < count; ++k) {
        const int s = idx[k];
        if (s < 0 || s >= (int)sh.size()) return fail(DEM_E_INVALID, "scene index out of range");
        if (seen[s]++) return fail(DEM_E_INVALID, "scene " + std::to_string(s) + " listed twice");
        const SceneHost &h = sh[s];
        const dem_scene *sc = scs[k];
        if (!sc || sc->n_particles != h.n || sc->n_bonds != h.n_bonds || sc->n_materials != h.n_mat)
            return fail(DEM_E_INVALID, "upload must keep particle, bond and material counts (scene " +
                                           std::to_string(s) + ")");
        probes[k] = h;
    }
    auto layouts = [&]() -> int {
        // compute_layout touches only its probe; derive them in parallel
        std::vector<int> rcs(count, DEM_OK);
        std::vector<std::string> errs(count);
        const int T = std::max(1, std::min(count, host_threads()));
        std::vector<std::thread> pool;
        std::vector<World> scratch(T);
        for (int t = 0; t < T; ++t)
            pool.emplace_back([&, t]() {
                scratch[t].skin_factor = skin_factor;
                scratch[t].layout_threads = std::max(1, host_threads() / count);
                for (int k = t; k < count; k += T) {
                    rcs[k] = scratch[t].compute_layout(probes[k], scs[k]);
                    if (rcs[k]) errs[k] = scratch[t].err;
                }
            });
        for (auto &th : pool) th.join();
        for (int k = 0; k < count; ++k)
            if (rcs[k]) return fail(rcs[k], errs[k] + " (scene " + std::to_string(idx[k]) + ")");
        for (int k = 0; k < count; ++k) {
            const int rc = layout_fits(idx[k], probes[k]);
            if (rc) {
                err += " (scene " + std::to_string(idx[k]) + ")";
                return rc;
            }
        }
        return DEM_OK;
    };
    int rc = stage_many(idx, scs, count, probes.data(), layouts);
    if (rc) return rc;
    return force_rebuild();
}

int World::upload_scene(int s, const dem_scene *sc) {
    if (s < 0 || s >= (int)sh.size()) return fail(DEM_E_INVALID, "scene index out of range");
    const int32_t one = s;
    return upload_many(&one, &sc, 1);
}

int World::set_params(int s, const dem_params &p) {
    if (s < 0 || s >= (int)sh.size()) return fail(DEM_E_INVALID, "scene index out of range");
    SceneHost &h = sh[s];
    dem_params old = h.params;
    // the interval counter restarts its schedule from the current step
    int32_t cc[4];
    control(s, cc);
    h.params = p;
    bool geometry = old.hor_bound != p.hor_bound || old.vert_bound != p.vert_bound ||
                    old.round_bounds != p.round_bounds || old.bound_radius != p.bound_radius;
    h.step0 = host_step;
    h.cc0_0 = cc[0];
    h.cc1_0 = cc[1];
    h.cc2_0 = cc[2];
    int rc = push_par(s);
    if (rc) return rc;
    rc = push_det();
    if (rc) return rc;
    update_kernel_form();
    // walls moved: the search grid keeps its allocation (it clamps particles
    // to its extent) and the cell lists are rebuilt before the next step
    return geometry ? force_rebuild(false) : DEM_OK;
}

int World::set_materials(int s, const float *m, int n) {
    if (s < 0 || s >= (int)sh.size()) return fail(DEM_E_INVALID, "scene index out of range");
    SceneHost &h = sh[s];
    if (!m || n != h.n_mat) return fail(DEM_E_INVALID, "material count must stay the same");
    h.materials.assign(m, m + 6 * (size_t)n);
    return push_materials(s);
}

void World::control(int s, int32_t cc[4]) const {
    const SceneHost &h = sh[s];
    long long j = host_step - h.step0;
    int32_t iv = h.params.collision_interval;
    if (j <= 0) {
        cc[0] = h.cc0_0;
        cc[1] = h.cc1_0;
        cc[2] = h.cc2_0;
    } else {
        cc[0] = detect_at(iv, h.cc1_0, j - 1) ? 1 : 0;
        cc[1] = cc1_after(iv, h.cc1_0, j);
        cc[2] = (int32_t)(h.cc2_0 + j);
    }
    cc[3] = 0;
}

int World::set_control(int s, const int32_t cc[4]) {
    if (s < 0 || s >= (int)sh.size()) return fail(DEM_E_INVALID, "scene index out of range");
    SceneHost &h = sh[s];
    h.step0 = host_step;
    h.cc0_0 = cc[0];
    h.cc1_0 = cc[1];
    h.cc2_0 = cc[2];
    int32_t c3 = cc[3];
    CK(cudaMemcpyAsync(d.cc3 + s, &c3, 4, cudaMemcpyHostToDevice, stream));
    int rc = push_par(s);
    if (rc) return rc;
    return push_det();
}

namespace {
enum { T_INTERACT = 0, T_LOM = 1, T_BROAD = 2, T_REORDER = 3, T_END = 4, T_LIST = 5 };
}

void World::set_timing(bool on) {
    if (on && !timing) {
        for (auto &t : timers) {
            for (auto e : t.ev) cudaEventDestroy(e);
            t.ev.clear();
            t.ms = 0.0;
            t.n = 0;
        }
    }
    timing = on;
}

int World::kernel_time(int kind, double *ms, long long *n) {
    if (kind < 0 || kind >= N_TIMERS) return fail(DEM_E_INVALID, "unknown kernel");
    CK(cudaStreamSynchronize(stream));
    Timer &t = timers[kind];
    for (size_t k = 0; k + 1 < t.ev.size(); k += 2) {
        float x = 0.0f;
        CK(cudaEventElapsedTime(&x, t.ev[k], t.ev[k + 1]));
        t.ms += x;
        t.n += 1;
        cudaEventDestroy(t.ev[k]);
        cudaEventDestroy(t.ev[k + 1]);
    }
    t.ev.clear();
    if (ms) *ms = t.ms;
    if (n) *n = t.n;
    return DEM_OK;
}

// The rebuild body: cell keys, counting sort by cell, in-cell order, reorder
// of the particle arrays into cell order, candidate lists.  `gate` is the
// device word that says whether a rebuild is due (kernels return at once when
// it is 0); inside a conditional graph node it is always 1.
// every_step: the kernels are launched at every step and do nothing unless a
// rebuild is due (plain launches); otherwise they run only when it is due
// With kernel timing on (plain launches), the three phases are bracketed by
// events: "broad_phase" (keys, cell table, sort, grouping), "reorder",
// "candidate_lists".
void World::enqueue_rebuild(cudaStream_t st, const int32_t *gate, bool every_step) {
    rec_event(T_BROAD, st);
    launch_keys(d, block, st, gate);
    const int bp = launch_broad_phase(d, block, st, gate);
    rec_event(T_BROAD, st);
    rec_event(T_REORDER, st);
    launch_reorder(d, spare, block, st, gate);
    rec_event(T_REORDER, st);
    rec_event(T_LIST, st);
    const int lk = launch_list_build(d, block, st, gate, every_step, dense_cells());
    rec_event(T_LIST, st);
    rebuild_kernels = 1 + bp + 3 + lk;
}

// whether the active scenes hold 1.5 particles or more a search cell on
// average: then a block's particles span few cells and the candidate lists
// are built from neighbour cells staged in shared memory (k_list_tiles);
// sparser worlds read the cell table directly (measured: the 4 M-particle
// impact bed, 5.3 particles a cell, 0.59 -> 0.38 ms per list build staged;
// the 512-scene mix, 0.74 a cell, 0.21 -> 0.44 ms)
bool World::dense_cells() const {
    long long cells = 0, n = 0;
    for (const auto &h : sh) {
        if (!h.active) continue;
        cells += (long long)h.par.g_w * h.par.g_h;
        n += h.n;
    }
    return cells > 0 && 2 * n >= 3 * cells;
}

void World::rec_event(int kind, cudaStream_t st) {
    if (!timing) return;
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return;
    cudaEventRecord(e, st);
    timers[kind].ev.push_back(e);
}

// One step with plain launches; the rebuild kernels run every step and
// return at once unless a particle moved beyond its skin.  Within a call the
// first step runs its own LOM pass; every step but the last runs the next
// step's LOM pass inside its Simulation kernel.
void World::enqueue_plain_step(bool first, bool last, bool next_last) {
    auto rec = [&](int kind, bool) { rec_event(kind, stream); };
    int k = 0;
    if (first || !fuse_lom) {
        rec(T_LOM, true);
        k += launch_lom(d, block, stream, false, cudaGraphConditionalHandle{});
        rec(T_LOM, false);
    }
    enqueue_rebuild(stream, d.rebuild, true);
    rec(T_INTERACT, true);
    const bool fuse = fuse_lom && !last;
    k += launch_interact(d, block, stream, has_bigs, fuse, next_last, false, cudaGraphConditionalHandle{}, kernel_form,
                         &par_pv, par_ps);
    rec(T_INTERACT, false);
    if (fuse) flip();
    launches += k + rebuild_kernels;
    host_step++;
}

void World::drop_graph() {
    for (int p = 0; p < 2; ++p) {
        if (graph[p]) cudaGraphExecDestroy(graph[p]);
        if (graph1[p]) cudaGraphExecDestroy(graph1[p]);
        graph[p] = graph1[p] = nullptr;
        graph_R[p] = 0;
    }
}

// the current and the other pr/dp buffers trade places (a fused step
// wrote the next step's values into the other ones)
void World::flip() {
    std::swap(d.pr, d.pr_n);
    std::swap(d.dp, d.dp_n);
    parity ^= 1;
}

#define CKG(call)                                                                         \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            cudaGraph_t junk_ = nullptr;                                                  \
            cudaStreamEndCapture(stream, &junk_);                                         \
            if (junk_) cudaGraphDestroy(junk_);                                           \
            return fail(DEM_E_CUDA, std::string("graph capture: ") + #call + ": " +        \
                                        cudaGetErrorString(e_));                          \
        }                                                                                 \
    } while (0)

// Capture R steps as one graph: per step the LOM kernel, a conditional node
// whose body is the rebuild (its condition is set on the device by the LOM
// kernel's last warp or by k_decide), and the Simulation kernel (followed by
// k_end_step in large worlds).
// Capture R steps as one graph: the first step's LOM kernel, then per step a
// conditional node whose body is the rebuild (its condition set on the device
// by the LOM pass before it) and the Simulation kernel, fused with the next
// step's LOM pass for all but the last step (with fuse_lom; otherwise every
// step has its own LOM kernel).  The buffer swaps of the fused
// steps are applied to the captured launches and undone afterwards: they take
// effect when the graph runs.
int World::capture_graph(int R, cudaGraphExec_t *out, int *kernels_out) {
    if (!side) CK(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
    const int parity0 = parity;
    auto restore = [&]() {
        while (parity != parity0) flip();
    };
    CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    int kernels = 0;
    // a launch that fails during capture invalidates it: check the capture
    // before every use of its graph and the launch status after every group
    auto active = [&](cudaStreamCaptureStatus cs, cudaGraph_t g) {
        return cs == cudaStreamCaptureStatusActive && g != nullptr;
    };
#define CKR(call)                  \
    do {                           \
        cudaError_t e2_ = (call);  \
        if (e2_ != cudaSuccess) {  \
            restore();             \
            CKG(e2_);              \
        }                          \
    } while (0)
    cudaGraphConditionalHandle h{};
    for (int k = 0; k < R; ++k) {
        cudaStreamCaptureStatus cs;
        cudaGraph_t g = nullptr;
        if (k == 0 || !fuse_lom) {
            CKR(cudaStreamGetCaptureInfo(stream, &cs, nullptr, &g, nullptr, nullptr, nullptr));
            if (!active(cs, g)) CKR(cudaErrorStreamCaptureInvalidated);
            CKR(cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault));
            kernels += launch_lom(d, block, stream, true, h);
            CKR(cudaGetLastError());
        }
        const cudaGraphNode_t *deps = nullptr;
        size_t ndeps = 0;
        CKR(cudaStreamGetCaptureInfo(stream, &cs, nullptr, &g, &deps, nullptr, &ndeps));
        if (!active(cs, g)) CKR(cudaErrorStreamCaptureInvalidated);
        cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = h;
        np.conditional.type = cudaGraphCondTypeIf;
        np.conditional.size = 1;
        cudaGraphNode_t node;
        CKR(cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &np));
        cudaGraph_t body = np.conditional.phGraph_out[0];
        CKR(cudaStreamBeginCaptureToGraph(side, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        enqueue_rebuild(side, d.rebuild, false);
        const cudaError_t le = cudaGetLastError();
        cudaGraph_t body_out = nullptr;
        const cudaError_t ee = cudaStreamEndCapture(side, &body_out);
        CKR(le);
        CKR(ee);
        CKR(cudaStreamUpdateCaptureDependencies(stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
        if (fuse_lom && k + 1 < R) {
            cudaGraphConditionalHandle hn{};
            CKR(cudaGraphConditionalHandleCreate(&hn, g, 0, cudaGraphCondAssignDefault));
            kernels += launch_interact(d, block, stream, has_bigs, true, k + 2 == R, true, hn, kernel_form, &par_pv, par_ps);
            CKR(cudaGetLastError());
            flip();
            h = hn;
        } else {
            kernels += launch_interact(d, block, stream, has_bigs, false, false, true, cudaGraphConditionalHandle{},
                                       kernel_form, &par_pv, par_ps);
            CKR(cudaGetLastError());
        }
    }
#undef CKR
    restore();
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(stream, &g);
    if (e != cudaSuccess) return fail(DEM_E_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    cudaGraphExec_t ex = nullptr;
    e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(DEM_E_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    *out = ex;
    *kernels_out = kernels;
    return DEM_OK;
}

// the scene parameters' source for the Simulation launches of a step() call:
// the host records equal the device's whenever a call steps
void World::update_param_source() {
    if (sh.size() == 1) {
        par_ps = PS_ONE;
        std::memcpy(&par_pv, &sh[0].par, sizeof(ScenePar));  // padding too: graph_par is compared bytewise
        // what the Simulation kernels never read from it: the interval
        // counter's origin (end_of_step reads w.par) changes with every upload,
        // and would make each step call after one capture its graphs anew
        par_pv.step0 = 0;
        par_pv.cc1_0 = 0;
        par_pv.active = 0;
        return;
    }
    par_ps = PS_SCENE;
    std::memset(&par_pv, 0, sizeof par_pv);
    // scenes the host has frozen (a server's free slots) read no parameters:
    // the kernels stop at their act word first
    int first = -1, bonded = -1;  // an active scene; one with bond records, whose bond settings are shared
    ScenePar k_first, k_bonded;
    for (size_t s = 0; s < sh.size(); ++s) {
        if (!sh[s].active) continue;
        if (first < 0) {
            first = (int)s;
            k_first = shared_settings(sh[s].par, false);
        } else {
            const ScenePar k = shared_settings(sh[s].par, false);
            if (std::memcmp(&k, &k_first, sizeof k) != 0) return;
        }
        if (sh[s].n_bonds <= 0) continue;
        if (bonded < 0) {
            bonded = (int)s;
            k_bonded = shared_settings(sh[s].par, true);
            continue;
        }
        const ScenePar k = shared_settings(sh[s].par, true);
        if (std::memcmp(&k, &k_bonded, sizeof k) != 0) return;
    }
    if (first < 0) return;
    const ScenePar kp = shared_settings(sh[bonded < 0 ? first : bonded].par, true);
    par_ps = PS_SHARED;
    std::memcpy(&par_pv, &kp, sizeof(ScenePar));
}

int World::step(int n_steps) {
    if (n_steps < 0) return fail(DEM_E_INVALID, "n_steps < 0");
    update_param_source();
    int k = 0;
    if (use_graphs && !timing && n_steps > 0) {
        if (par_ps != graph_ps || std::memcmp(&par_pv, &graph_par, sizeof(ScenePar)) != 0) {
            drop_graph();
            graph_ps = par_ps;
            std::memcpy(&graph_par, &par_pv, sizeof(ScenePar));
        }
        while (n_steps - k >= graph_steps) {
            const int p = parity;
            if (!graph[p] || graph_R[p] != graph_steps) {
                if (graph[p]) cudaGraphExecDestroy(graph[p]);
                graph[p] = nullptr;
                int rc = capture_graph(graph_steps, &graph[p], &graph_kernels[p]);
                if (rc) return rc;
                graph_R[p] = graph_steps;
            }
            CK(cudaGraphLaunch(graph[p], stream));
            if (fuse_lom)
                for (int f = 0; f + 1 < graph_steps; ++f) flip();
            launches += graph_kernels[p];
            host_step += graph_steps;
            k += graph_steps;
        }
        for (; k < n_steps; ++k) {
            const int p = parity;
            if (!graph1[p]) {
                int rc = capture_graph(1, &graph1[p], &graph1_kernels[p]);
                if (rc) return rc;
            }
            CK(cudaGraphLaunch(graph1[p], stream));
            launches += graph1_kernels[p];
            host_step += 1;
        }
    }
    const int k0 = k;
    for (; k < n_steps; ++k) enqueue_plain_step(k == k0, k + 1 == n_steps, k + 2 == n_steps);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(DEM_E_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    return DEM_OK;
}

int World::sync() {
    CK(cudaStreamSynchronize(stream));
    int32_t e = 0;
    CK(cudaMemcpy(&e, d.err, 4, cudaMemcpyDeviceToHost));
    if (e) return fail(DEM_E_STATE, "device error flags set: " + std::to_string(e));
    return DEM_OK;
}

int World::unstage_error(int32_t e) {
    if (e & 16) return fail(DEM_E_STATE, "internal particle map is corrupt");
    if (e & 32) return fail(DEM_E_STATE, "contact partner outside its scene");
    return DEM_OK;
}

// One scene: converted into the staging block, then copied straight into
// the caller's arrays.
int World::download_scene(int s, dem_scene *out) {
    if (s < 0 || s >= (int)sh.size()) return fail(DEM_E_INVALID, "scene index out of range");
    if (!out) return fail(DEM_E_INVALID, "out is NULL");
    const int32_t one = s;
    return download_many(&one, &out, 1);
}

// Many scenes at once (dem_batch_download_many).  One launch converts every
// scene into the staging block.  With host_direct one copy launch writes
// the block and the per-particle reference mirrors straight into the
// callers' arrays, skipped on the device if any conversion failed; else the
// block comes back one field at a time into the page-locked block and host
// threads copy each field out as soon as it has landed.  The callers'
// arrays are written only if every scene's conversion passed.
int World::download_many(const int32_t *idx, dem_scene *const *outs, int count) {
    if (count <= 0) return DEM_OK;
    if (!idx || !outs) return fail(DEM_E_INVALID, "scene index/pointer arrays are NULL");
    for (int k = 0; k < count; ++k) {
        const int s = idx[k];
        if (s < 0 || s >= (int)sh.size()) return fail(DEM_E_INVALID, "scene index out of range");
        if (!outs[k]) return fail(DEM_E_INVALID, "out is NULL");
        if (outs[k]->n_particles != sh[s].n)
            return fail(DEM_E_INVALID, "out->n_particles must match the scene (scene " + std::to_string(s) + ")");
    }
    std::vector<StageItem> tab;
    std::vector<int> tab_k;
    const long long total = pack_items(sh, idx, count, tab, tab_k);
    const int nt = (int)tab.size();
    int rc = ensure_ref(std::max(total, 1LL));
    if (rc) return rc;
    rc = ensure_tables(nt + 1, N_REF_FIELDS * nt + 1);
    if (rc) return rc;
    const size_t N = (size_t)d.N;
    PinMap pm;
    const size_t o_fields = host_direct ? 0 : pm.take((size_t)ref_cap * REF_WORDS * 4);
    const size_t o_copies = pm.take(sizeof(HostCopy) * ((size_t)N_REF_FIELDS * nt + 1));
    const size_t o_items = pm.take(sizeof(StageItem) * (size_t)(nt + 1));
    const size_t o_err = pm.take(4 * (size_t)(nt + 1));
    const size_t o_fix = host_direct ? 0 : pm.take(24 * N);
    const size_t o_force = host_direct ? 0 : pm.take(24 * N);
    const size_t o_matp = host_direct ? 0 : pm.take(4 * N);
    const size_t o_bst = pm.take(4 * (size_t)d.B), o_blen = pm.take(4 * (size_t)d.B);
    rc = ensure_pin(pm.bytes);
    if (rc) return rc;
    char *pb = static_cast<char *>(pin);
    float *hp = reinterpret_cast<float *>(pb + o_fields);
    std::memcpy(pb + o_items, tab.data(), sizeof(StageItem) * nt);
    const int32_t *h_err = reinterpret_cast<const int32_t *>(pb + o_err);
    const int32_t *h_fix = reinterpret_cast<const int32_t *>(pb + o_fix);
    const float *h_force = reinterpret_cast<const float *>(pb + o_force);
    const int32_t *h_matp = reinterpret_cast<const int32_t *>(pb + o_matp);
    const int32_t *h_bst = reinterpret_cast<const int32_t *>(pb + o_bst);
    const float *h_blen = reinterpret_cast<const float *>(pb + o_blen);
    float *dp0 = static_cast<float *>(ref_block);

    // the conversion and its check words
    if (nt > 0) {
        CK(cudaMemcpyAsync(d_items, pb + o_items, sizeof(StageItem) * nt, cudaMemcpyHostToDevice, stream));
        CK(cudaMemsetAsync(d_item_err, 0, 4 * (size_t)(nt + 1), stream));
        launch_stage_out(d, ref, d_items, nt, total, d_item_err, stream);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(pb + o_err, d_item_err, 4 * (size_t)(nt + 1), cudaMemcpyDeviceToHost, stream));
    }
    std::vector<std::pair<long long, long long>> rn, rb;
    for (int k = 0; k < count; ++k) {
        const SceneHost &h = sh[idx[k]];
        rn.emplace_back(h.particle_base, h.n);
        rb.emplace_back(h.bond_base, h.n_bonds);
    }
    rn = merge_runs(rn);
    rb = merge_runs(rb);
    auto fetch_bonds = [&]() -> cudaError_t {
        for (const auto &x : rb) {
            cudaError_t e2 = cudaMemcpyAsync(pb + o_bst + 4 * x.first, d.b_status + x.first, 4 * x.second,
                                             cudaMemcpyDeviceToHost, stream);
            if (e2 == cudaSuccess)
                e2 = cudaMemcpyAsync(pb + o_blen + 4 * x.first, d.b_length + x.first, 4 * x.second,
                                     cudaMemcpyDeviceToHost, stream);
            if (e2 != cudaSuccess) return e2;
        }
        return cudaSuccess;
    };
    // what the host fills of scene k (mirrors: also fixity, forces, material pointers)
    auto host_part = [&](int k, bool mirrors) {
        const int s = idx[k];
        const SceneHost &h = sh[s];
        dem_scene *out = outs[k];
        const size_t n = (size_t)h.n, base = (size_t)h.particle_base;
        if (mirrors) {
            if (out->fixity && n) std::memcpy(out->fixity, h_fix + 6 * base, 24 * n);
            if (out->forces && n) std::memcpy(out->forces, h_force + 6 * base, 24 * n);
            if (out->material_pointers && n) std::memcpy(out->material_pointers, h_matp + base, 4 * n);
        }
        if (out->materials && out->n_materials == h.n_mat)
            std::memcpy(out->materials, h.materials.data(), h.materials.size() * 4);
        if (out->bonds && out->n_bonds == h.n_bonds)
            for (int q = 0; q < h.n_bonds; ++q) {
                out->bonds[3 * q] = h_bst[h.bond_base + q];
                out->bonds[3 * q + 1] = h.bond_angle[q];
                out->bonds[3 * q + 2] = f2bits(h_blen[h.bond_base + q]);
            }
        control(s, out->coll_cont);
        out->grid = h.grid;
    };
    auto first_error = [&]() -> int {
        for (int i = 0; i < nt; ++i)
            if (h_err[i]) {
                const int r2 = unstage_error(h_err[i]);
                err += " (scene " + std::to_string(tab[i].scene) + ")";
                return r2;
            }
        return DEM_OK;
    };

    if (host_direct) {
        HostCopy *hc = reinterpret_cast<HostCopy *>(pb + o_copies);
        int nc = 0;
        long long pieces = 0;
        for (int i = 0; i < nt; ++i) {
            dem_scene *out = outs[tab_k[i]];
            for (int f = 0; f < N_REF_FIELDS; ++f) {
                if (!OUT_FIELD[f]) continue;
                const RefField &F = REF_FIELDS[f];
                pieces = add_copy(hc, nc, dp0 + F.base * ref_cap + F.per * tab[i].off,
                                  const_cast<void *>(scene_field(out, f)), 4LL * F.per * tab[i].n, pieces);
            }
            const size_t base = (size_t)tab[i].base;
            pieces = add_copy(hc, nc, d.fix_ref + 6 * base, out->fixity, 24LL * tab[i].n, pieces);
            pieces = add_copy(hc, nc, d.force_ref + 6 * base, out->forces, 24LL * tab[i].n, pieces);
            pieces = add_copy(hc, nc, d.matp_ref + base, out->material_pointers, 4LL * tab[i].n, pieces);
        }
        if (nc > 0) {
            CK(cudaMemcpyAsync(d_copies, hc, sizeof(HostCopy) * nc, cudaMemcpyHostToDevice, stream));
            launch_copies(d_copies, nc, pieces, d_item_err + nt, stream);
            CK(cudaGetLastError());
        }
        cudaError_t ce = fetch_bonds();
        const cudaError_t se = cudaStreamSynchronize(stream);  // the copies write the callers' arrays until then
        if (ce == cudaSuccess) ce = se;
        if (ce != cudaSuccess) return fail(DEM_E_CUDA, cudaGetErrorString(ce));
        rc = first_error();
        if (rc) return rc;
        par_for(count, [&](int k) { host_part(k, false); });
        return DEM_OK;
    }

    struct Chunk {
        int f, i0, i1;
    };
    std::vector<Chunk> chunks;
    std::vector<long long> sizes;
    for (int f = 0; f < N_REF_FIELDS && nt > 0; ++f) {
        if (!OUT_FIELD[f]) continue;
        for (const auto &g : split_items(tab, f == F_CONTACTS ? 8 : 1)) {
            chunks.push_back(Chunk{f, g.first, g.second});
            sizes.push_back(g.second - g.first);
        }
    }
    chunks.push_back(Chunk{-1, 0, count});
    sizes.push_back(count);
    rc = ensure_events((int)chunks.size());
    if (rc) return rc;
    for (int c = 0; c < (int)chunks.size(); ++c) {
        const Chunk &ch = chunks[c];
        if (ch.f >= 0) {
            const RefField &F = REF_FIELDS[ch.f];
            const long long o0 = tab[ch.i0].off, o1 = tab[ch.i1 - 1].off + tab[ch.i1 - 1].n;
            CK(cudaMemcpyAsync(hp + F.base * ref_cap + F.per * o0, dp0 + F.base * ref_cap + F.per * o0,
                               sizeof(float) * F.per * (size_t)(o1 - o0), cudaMemcpyDeviceToHost, stream));
        } else {
            for (const auto &x : rn) {
                CK(cudaMemcpyAsync(pb + o_fix + 24 * x.first, d.fix_ref + 6 * x.first, 24 * x.second,
                                   cudaMemcpyDeviceToHost, stream));
                CK(cudaMemcpyAsync(pb + o_force + 24 * x.first, d.force_ref + 6 * x.first, 24 * x.second,
                                   cudaMemcpyDeviceToHost, stream));
                CK(cudaMemcpyAsync(pb + o_matp + 4 * x.first, d.matp_ref + x.first, 4 * x.second,
                                   cudaMemcpyDeviceToHost, stream));
            }
            CK(fetch_bonds());
        }
        CK(cudaEventRecord(xfer_ev[c], stream));
    }
    HostPipe pipe(sizes, true);
    pipe.start([&](int c, long long u) {
        const Chunk &ch = chunks[c];
        if (ch.f < 0) {
            host_part((int)u, true);
            return;
        }
        const int i = ch.i0 + (int)u;
        void *dst = const_cast<void *>(scene_field(outs[tab_k[i]], ch.f));
        if (!dst) return;
        const RefField &F = REF_FIELDS[ch.f];
        std::memcpy(dst, hp + F.base * ref_cap + F.per * tab[i].off, sizeof(float) * F.per * (size_t)tab[i].n);
    });
    for (int c = 0; c < (int)chunks.size(); ++c) {
        const cudaError_t ce = cudaEventSynchronize(xfer_ev[c]);
        if (ce != cudaSuccess) {
            pipe.cancel();
            pipe.join();
            return fail(DEM_E_CUDA, cudaGetErrorString(ce));
        }
        if (c == 0 && (rc = first_error()) != DEM_OK) {
            pipe.cancel();
            pipe.join();
            return rc;
        }
        pipe.release(c);
    }
    pipe.join();
    return DEM_OK;
}

int World::set_properties(int s, int32_t *selections, const int32_t *props) {
    if (s < 0 || s >= (int)sh.size()) return fail(DEM_E_INVALID, "scene index out of range");
    if (!selections || !props) return fail(DEM_E_INVALID, "selections/props is NULL");
    SceneHost &h = sh[s];
    const int n = h.n;
    if (props[13] == 1 && (props[27] < 0 || props[27] >= h.n_mat))
        return fail(DEM_E_INVALID, "material index out of range");
    float f[28];
    std::memcpy(f, props, sizeof f);
    bool any = false;
    for (int i = 0; i < n; ++i) any |= selections[i] != 0;
    if (props[9] == 1 && any && !(f[23] >= 0.0f && std::isfinite(f[23])))
        return fail(DEM_E_INVALID, "radius must be finite and >= 0");
    if (props[9] == 1 && any && f[23] > h.r_max &&
        (2.0f * f[23] + h.skin) * (1.0f + 1e-3f) > h.par.g_cs * h.par.stencil)
        return fail(DEM_E_UNSUPPORTED, "radius beyond the search grid's reach; create a new context");
    int32_t *dsel = nullptr, *dout = nullptr, *dprops = nullptr;
    CK(cudaMalloc(&dsel, sizeof(int32_t) * (n > 0 ? n : 1)));
    CK(cudaMalloc(&dout, sizeof(int32_t) * (n > 0 ? n : 1)));
    CK(cudaMalloc(&dprops, sizeof(int32_t) * 28));
    cudaMemcpyAsync(dsel, selections, sizeof(int32_t) * n, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(dout, selections, sizeof(int32_t) * n, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(dprops, props, sizeof(int32_t) * 28, cudaMemcpyHostToDevice, stream);
    launch_set_properties(d, s, dsel, dout, dprops, block, stream);
    cudaError_t e = cudaMemcpyAsync(selections, dout, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, stream);
    cudaError_t e2 = cudaStreamSynchronize(stream);
    cudaFree(dsel);
    cudaFree(dout);
    cudaFree(dprops);
    if (e != cudaSuccess || e2 != cudaSuccess) return fail(DEM_E_CUDA, "set_properties failed");
    for (int i = 0; i < n; ++i)
        if (selections[i] != 0 && props[9] == 1) h.r_max = std::max(h.r_max, f[23]);
    if (any && (props[0] == 1 || props[1] == 1 || props[9] == 1)) return force_rebuild(false);
    return DEM_OK;
}

// Fix.wgsl:44-54 (selections == 1 -> 2, fixity all 1, velocity and
// rotational velocity 0), Drop.wgsl:34-41 (selections == 2 -> 1, fixity all
// 0), Release.wgsl:77-92 (selections != 0: fixity = its second triple; with
// throw_vel, velocity = (del_x, del_y) / (dT * ticks)).  The secondary codes
// live in the host copy of fixity, so the new primary codes are formed here
// and the device updates the particles' flags (and velocities).
int World::fixity_event(int s, int kind, int32_t *selections, int throw_vel, float del_x, float del_y,
                        int ticks) {
    if (s < 0 || s >= (int)sh.size()) return fail(DEM_E_INVALID, "scene index out of range");
    if (!selections) return fail(DEM_E_INVALID, "selections is NULL");
    if (kind < DEM_EVENT_FIX || kind > DEM_EVENT_RELEASE) return fail(DEM_E_INVALID, "unknown event kind");
    SceneHost &h = sh[s];
    std::vector<int32_t> idx;
    for (int i = 0; i < h.n; ++i) {
        if (kind == DEM_EVENT_FIX && selections[i] == 1) {
            selections[i] = 2;
        } else if (kind == DEM_EVENT_DROP && selections[i] == 2) {
            selections[i] = 1;
        } else if (!(kind == DEM_EVENT_RELEASE && selections[i] != 0)) {
            continue;
        }
        idx.push_back(i);
    }
    float vx = 0.0f, vy = 0.0f;
    const int set_vel = kind == DEM_EVENT_RELEASE && throw_vel ? 1 : 0;
    if (set_vel) {
        const float q = h.params.dT * (float)ticks;
        vx = del_x / q;
        vy = del_y / q;
    }
    const int k = (int)idx.size();
    if (k == 0) return DEM_OK;
    int32_t *dbuf = nullptr;
    CK(cudaMalloc(&dbuf, sizeof(int32_t) * (size_t)k));
    cudaMemcpyAsync(dbuf, idx.data(), sizeof(int32_t) * k, cudaMemcpyHostToDevice, stream);
    launch_fixity_event(d, h.particle_base, dbuf, k, kind, vx, vy, set_vel, stream);
    const cudaError_t e = cudaStreamSynchronize(stream);
    cudaFree(dbuf);
    if (e != cudaSuccess) return fail(DEM_E_CUDA, std::string("fixity event: ") + cudaGetErrorString(e));
    return DEM_OK;
}

// State::get_datum (state.rs:708-737): means over the selected particles of
// pos, data[4], data[5], rot, data[6], data[1..3] and the sum of |data[0]|,
// accumulated in double in index order as the reference does; only the
// selected particles' fields cross from the device.  Returns the count.
int World::get_datum(int s, const int32_t *selections, double out[10]) {
    if (s < 0 || s >= (int)sh.size()) return fail(DEM_E_INVALID, "scene index out of range");
    if (!selections || !out) return fail(DEM_E_INVALID, "selections/out is NULL");
    const SceneHost &h = sh[s];
    std::vector<int32_t> idx;
    for (int i = 0; i < h.n; ++i)
        if (selections[i] != 0) idx.push_back(i);
    const int k = (int)idx.size();
    if (k == 0) return 0;
    std::vector<float> f(10 * (size_t)k);
    void *dbuf = nullptr;
    CK(cudaMalloc(&dbuf, sizeof(int32_t) * (size_t)k + sizeof(float) * 10 * (size_t)k));
    int32_t *d_idx = static_cast<int32_t *>(dbuf);
    float *d_out = reinterpret_cast<float *>(d_idx + k);
    cudaMemcpyAsync(d_idx, idx.data(), sizeof(int32_t) * k, cudaMemcpyHostToDevice, stream);
    launch_gather_datum(d, h.particle_base, d_idx, k, d_out, stream);
    cudaMemcpyAsync(f.data(), d_out, sizeof(float) * 10 * (size_t)k, cudaMemcpyDeviceToHost, stream);
    const cudaError_t e = cudaStreamSynchronize(stream);
    cudaFree(dbuf);
    if (e != cudaSuccess) return fail(DEM_E_CUDA, std::string("datum: ") + cudaGetErrorString(e));
    double sums[10] = {0.0};
    for (int t = 0; t < k; ++t) {
        const float *g = &f[10 * (size_t)t];
        sums[0] += (double)g[0];
        sums[1] += (double)g[1];
        sums[2] += (double)g[2];
        sums[3] += (double)g[3];
        sums[4] += (double)g[4];
        sums[5] += (double)g[5];
        sums[6] += std::fabs((double)g[6]);
        sums[7] += (double)g[7];
        sums[8] += (double)g[8];
        sums[9] += (double)g[9];
    }
    for (int q = 0; q < 10; ++q) out[q] = q == 6 ? sums[q] : sums[q] / (double)k;
    return k;
}

// Advance with Record on (client.rs:931-974, gather_data): n steps, one at a
// time, each followed by the datum of the selected particles (get_datum,
// state.rs:708-737).  Per step one graph launch and one gather launch into a
// device buffer of rows; the rows come back in one copy per chunk of steps
// (at most 2^24 floats), summed on the host in double in index order.
// Returns the number of selected particles; rows[10 * n_steps] is written
// when it is > 0 (none selected: the steps run and nothing is recorded, as
// the reference clears its data then).
int World::record(int s, const int32_t *selections, int n_steps, double *rows) {
    if (s < 0 || s >= (int)sh.size()) return fail(DEM_E_INVALID, "scene index out of range");
    if (!selections || (n_steps > 0 && !rows)) return fail(DEM_E_INVALID, "selections/rows is NULL");
    if (n_steps < 0) return fail(DEM_E_INVALID, "n_steps < 0");
    const SceneHost &h = sh[s];
    std::vector<int32_t> idx;
    for (int i = 0; i < h.n; ++i)
        if (selections[i] != 0) idx.push_back(i);
    const int k = (int)idx.size();
    if (k == 0) {
        for (int j = 0; j < n_steps; ++j) {
            const int rc = step(1);
            if (rc) return rc;
        }
        return 0;
    }
    const long long per = 10LL * k;  // floats per recorded step
    const int chunk = (int)std::max<long long>(1, std::min<long long>(n_steps, (1LL << 24) / per));
    void *dbuf = nullptr;
    CK(cudaMalloc(&dbuf, sizeof(int32_t) * (size_t)k + sizeof(float) * (size_t)(per * chunk)));
    int32_t *d_idx = static_cast<int32_t *>(dbuf);
    float *d_rows = reinterpret_cast<float *>(d_idx + k);
    std::vector<float> f((size_t)(per * chunk));
    int rc = DEM_OK;
    cudaError_t e = cudaMemcpyAsync(d_idx, idx.data(), sizeof(int32_t) * k, cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) rc = fail(DEM_E_CUDA, std::string("record: ") + cudaGetErrorString(e));
    for (int s0 = 0; rc == DEM_OK && s0 < n_steps; s0 += chunk) {
        const int m = std::min(chunk, n_steps - s0);
        for (int j = 0; j < m && rc == DEM_OK; ++j) {
            rc = step(1);
            if (rc == DEM_OK) launch_gather_datum(d, h.particle_base, d_idx, k, d_rows + per * j, stream);
        }
        if (rc) break;
        e = cudaMemcpyAsync(f.data(), d_rows, sizeof(float) * (size_t)(per * m), cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) {
            rc = fail(DEM_E_CUDA, std::string("record: ") + cudaGetErrorString(e));
            break;
        }
        for (int j = 0; j < m; ++j) {
            double sums[10] = {0.0};
            for (int t = 0; t < k; ++t) {
                const float *g = &f[(size_t)(per * j + 10LL * t)];
                for (int q = 0; q < 10; ++q) sums[q] += q == 6 ? std::fabs((double)g[q]) : (double)g[q];
            }
            double *out = rows + 10LL * (s0 + j);
            for (int q = 0; q < 10; ++q) out[q] = q == 6 ? sums[q] : sums[q] / (double)k;
        }
    }
    cudaStreamSynchronize(stream);
    cudaFree(dbuf);
    return rc ? rc : k;
}

int World::drain_events(std::vector<dem_break_event> &out) {
    CK(cudaStreamSynchronize(stream));
    unsigned long long cnt = 0;
    CK(cudaMemcpy(&cnt, d.ev_count, sizeof cnt, cudaMemcpyDeviceToHost));
    size_t k = (size_t)std::min<unsigned long long>(cnt, d.ev_cap);
    out.resize(k);
    if (k) CK(cudaMemcpy(out.data(), d.ev, k * sizeof(Event), cudaMemcpyDeviceToHost));
    CK(cudaMemset(d.ev_count, 0, sizeof(unsigned long long)));
    std::sort(out.begin(), out.end(), [](const dem_break_event &x, const dem_break_event &y) {
        if (x.step != y.step) return x.step < y.step;
        if (x.scene != y.scene) return x.scene < y.scene;
        if (x.bond != y.bond) return x.bond < y.bond;
        if (x.a != y.a) return x.a < y.a;
        return x.b < y.b;
    });
    return DEM_OK;
}

int World::broad_phase_snapshot(int s, int32_t *keys, int32_t *order, int32_t *cell_start,
                                int32_t *n_cells) {
    if (s < 0 || s >= (int)sh.size()) return fail(DEM_E_INVALID, "scene index out of range");
    const SceneHost &h = sh[s];
    // reported layout: the search cells, then one cell for the large and the
    // zero-radius particles (internally two cells, large first)
    const int grid_cells = h.par.g_w * h.par.g_h;
    if (n_cells) *n_cells = grid_cells + 1;
    launch_keys(d, block, stream, nullptr);
    launch_broad_phase(d, block, stream, nullptr);
    const int n = h.n, base = h.particle_base;
    std::vector<uint32_t> k(n);
    std::vector<int32_t> srt(n), orig(n), cs((size_t)h.n_cells + 1);
    CK(cudaMemcpyAsync(cs.data(), d.cell_start + h.cell_base, cs.size() * 4, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    const int first = cs[0];
    if (n > 0) {
        CK(cudaMemcpyAsync(k.data(), d.keys + base, n * 4, cudaMemcpyDeviceToHost, stream));
        CK(cudaMemcpyAsync(srt.data(), d.sorted + first, n * 4, cudaMemcpyDeviceToHost, stream));
        CK(cudaMemcpyAsync(orig.data(), d.orig + base, n * 4, cudaMemcpyDeviceToHost, stream));
    }
    CK(cudaStreamSynchronize(stream));
    for (int i = 0; i < n; ++i) {
        if (keys) keys[orig[i]] = std::min((int32_t)k[i] - h.cell_base, grid_cells);
        int src = srt[i] - base;
        if (src < 0 || src >= n) return fail(DEM_E_STATE, "sorted order leaves its scene");
        if (order) order[i] = orig[src];
    }
    if (cell_start) {
        for (int c = 0; c <= grid_cells; ++c) cell_start[c] = cs[c] - first;
        cell_start[grid_cells + 1] = cs[h.n_cells] - first;
    }
    // the cell table now describes the current positions, not the last rebuild
    return force_rebuild(false);
}

int World::stats(dem_stats *out) {
    CK(cudaStreamSynchronize(stream));
    unsigned long long st[6];
    CK(cudaMemcpy(st, d.stats, sizeof st, cudaMemcpyDeviceToHost));
    int32_t e = 0;
    CK(cudaMemcpy(&e, d.err, 4, cudaMemcpyDeviceToHost));
    std::memset(out, 0, sizeof *out);
    out->steps = host_step;
    out->capped = (int64_t)st[0];
    out->events = (int64_t)st[1];
    out->events_dropped = (int64_t)st[2];
    out->reorders = (int64_t)st[4];
    out->kernel_launches = launches;
    out->list_overflows = (int64_t)st[5];
    out->device_error = e | (st[3] ? 1 : 0);
    return DEM_OK;
}

}  // namespace demgb

// dem_server.cu -- continuous batching of scene requests on one GPU
// (include/dem.h, "Serving").
//
// Requests (a scene, its settings and a horizon in steps) queue on the host.
// dem_server_advance() retires the scenes that reached their horizon (their
// final state is copied to host memory and their device ranges freed), admits
// queued requests first-come first-served while the device arenas -- sized
// once from the memory budget -- have room, and then steps every admitted
// scene together.  A scene admitted while others run joins the same launches
// from its next step on; each scene stops exactly at its horizon (a device
// countdown), so its result is the result of running it alone.
#include <chrono>
#include <cstring>
#include <algorithm>
#include <deque>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "dem.h"
#include "dem_world_host.h"

namespace {

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// an owned copy of a scene in the reference layouts
struct SceneCopy {
    std::vector<float> pos, radii, vel, acc, rot, rot_vel, rot_acc, forces, del_pos, del_rot, materials, data;
    std::vector<int32_t> fixity, bonds, contacts, material_pointers;
    dem_scene view{};

    void from(const dem_scene &s, bool with_contents) {
        const size_t n = (size_t)s.n_particles;
        auto cp = [&](auto &dst, const auto *src, size_t cnt) {
            dst.assign(cnt, 0);
            if (with_contents && src && cnt) std::memcpy(dst.data(), src, cnt * sizeof(dst[0]));
        };
        cp(pos, s.pos, 2 * n);
        cp(radii, s.radii, n);
        cp(vel, s.vel, 2 * n);
        cp(acc, s.acc, 2 * n);
        cp(rot, s.rot, n);
        cp(rot_vel, s.rot_vel, n);
        cp(rot_acc, s.rot_acc, n);
        cp(forces, s.forces, 6 * n);
        cp(del_pos, s.del_pos, 2 * n);
        cp(del_rot, s.del_rot, n);
        cp(materials, s.materials, 6 * (size_t)s.n_materials);
        cp(data, s.data, 7 * n);
        cp(fixity, s.fixity, 6 * n);
        cp(bonds, s.bonds, 3 * (size_t)s.n_bonds);
        cp(contacts, s.contacts, 6 * (size_t)DEM_MAX_CONTACTS * n);
        cp(material_pointers, s.material_pointers, n);
        view = s;
        view.pos = pos.data(); view.radii = radii.data(); view.vel = vel.data(); view.acc = acc.data();
        view.rot = rot.data(); view.rot_vel = rot_vel.data(); view.rot_acc = rot_acc.data();
        view.forces = forces.data(); view.del_pos = del_pos.data(); view.del_rot = del_rot.data();
        view.materials = materials.data(); view.data = data.data(); view.fixity = fixity.data();
        view.bonds = bonds.empty() ? nullptr : bonds.data(); view.contacts = contacts.data();
        view.material_pointers = material_pointers.data();
    }
};

struct Request {
    int64_t id = 0;
    SceneCopy in, out;
    dem_params params{};
    dem_ext ext{};
    std::vector<float> sn, ss;
    int64_t horizon = 0;
    int64_t steps_done = 0;
    int slot = -1;
    int state = 0;  // 0 queued, 1 running, 2 done, 3 failed (can never be admitted)
    int fail_code = 0;
    std::string fail_msg;
    double t_submit = 0, t_admit = 0, t_done = 0;
    std::vector<dem_break_event> events;
};

}  // namespace

struct dem_server {
    demgb::World world;
    std::string msg;
    dem_server_config cfg{};
    int64_t next_id = 1;
    std::map<int64_t, std::unique_ptr<Request>> reqs;
    std::deque<int64_t> queue;
    std::vector<int64_t> slot_req;  // slot -> running request id
    std::vector<int64_t> done_unpolled;
    int64_t active_particles = 0;
    int64_t particle_steps = 0;
    int64_t completed = 0;
    int64_t waits_active = 0, waits_memory = 0;
};

namespace {
thread_local std::string g_server_create_error;

int sset(dem_server *sv, int code, const std::string &m) {
    if (sv) sv->msg = m;
    else g_server_create_error = m;
    return code;
}
int src_(dem_server *sv, int rc) {
    if (rc < 0) sv->msg = sv->world.err;
    return rc;
}

int retire_finished(dem_server *sv) {
    for (size_t s = 0; s < sv->slot_req.size(); ++s) {
        int64_t id = sv->slot_req[s];
        if (id == 0) continue;
        Request &r = *sv->reqs[id];
        if (r.steps_done < r.horizon) continue;
        r.out.from(r.in.view, false);
        r.out.view.n_particles = r.in.view.n_particles;
        int rc = sv->world.download_scene((int)s, &r.out.view);
        if (rc) return src_(sv, rc);
        rc = sv->world.retire((int)s);
        if (rc) return src_(sv, rc);
        sv->slot_req[s] = 0;
        sv->active_particles -= r.in.view.n_particles;
        r.state = 2;
        r.slot = -1;
        r.t_done = now_s();
        r.in = SceneCopy();  // the input is no longer needed
        sv->done_unpolled.push_back(id);
        sv->completed++;
    }
    return DEM_OK;
}

// a queued request that cannot be admitted even into empty arenas is failed
// (reported by poll, its error returned by fetch) so that the queue moves on
void fail_request(dem_server *sv, Request &r, int code, const std::string &msg) {
    r.state = 3;
    r.fail_code = code;
    r.fail_msg = msg;
    r.t_done = now_s();
    r.in = SceneCopy();
    sv->done_unpolled.push_back(r.id);
}

int admit_queued(dem_server *sv) {
    // first come, first served; a request that does not fit waits at the head
    while (!sv->queue.empty()) {
        Request &r = *sv->reqs[sv->queue.front()];
        if (sv->cfg.max_active_particles > 0 &&
            sv->active_particles + r.in.view.n_particles > sv->cfg.max_active_particles &&
            sv->active_particles > 0) {
            sv->waits_active++;
            break;
        }
        dem_ext e = r.ext;
        e.bond_normal_strength = r.sn.empty() ? nullptr : r.sn.data();
        e.bond_shear_strength = r.ss.empty() ? nullptr : r.ss.data();
        int slot = sv->world.admit(&r.in.view, r.params, e, r.horizon);
        if (slot == DEM_E_CAPACITY && sv->active_particles > 0) {  // waits for ranges to free
            sv->waits_memory++;
            break;
        }
        if (slot == DEM_E_CAPACITY || slot == DEM_E_INVALID || slot == DEM_E_UNSUPPORTED) {
            // the request itself cannot run here: fail it, keep serving the rest
            fail_request(sv, r, slot, sv->world.err);
            sv->queue.pop_front();
            continue;
        }
        if (slot < 0) return src_(sv, slot);
        r.slot = slot;
        r.state = 1;
        r.t_admit = now_s();
        sv->slot_req[slot] = r.id;
        sv->active_particles += r.in.view.n_particles;
        sv->queue.pop_front();
    }
    return DEM_OK;
}

int collect_events(dem_server *sv) {
    std::vector<dem_break_event> ev;
    int rc = sv->world.drain_events(ev);
    if (rc) return src_(sv, rc);
    for (auto &e : ev) {
        if (e.scene < 0 || e.scene >= (int)sv->slot_req.size()) continue;
        int64_t id = sv->slot_req[e.scene];
        if (!id) continue;
        dem_break_event x = e;
        x.step = (int32_t)(e.step - sv->world.sh[e.scene].step0);  // steps since admission
        x.scene = 0;
        sv->reqs[id]->events.push_back(x);
    }
    return DEM_OK;
}

}  // namespace

#define SERVER_GUARD(sv)                     \
    do {                                     \
        if (!(sv)) return DEM_E_INVALID;     \
        cudaSetDevice((sv)->world.device);   \
    } while (0)

extern "C" {

const char *dem_server_last_error(const dem_server *sv) {
    return sv ? sv->msg.c_str() : g_server_create_error.c_str();
}

void dem_server_config_defaults(dem_server_config *c) {
    if (!c) return;
    std::memset(c, 0, sizeof *c);
    c->memory_budget_bytes = 150LL << 30;
    c->max_active_particles = 16 << 20;
    c->max_scenes = 4096;
    c->cells_per_particle = 4.0f;
    c->bonds_per_particle = 1.0f;
    dem_ext_defaults(&c->ext);
}

int dem_server_create(const dem_server_config *cfg, int device, dem_server **out) {
    if (!out) return sset(nullptr, DEM_E_INVALID, "out is NULL");
    *out = nullptr;
    dem_server_config c;
    if (cfg) c = *cfg;
    else dem_server_config_defaults(&c);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return sset(nullptr, DEM_E_CUDA, "no CUDA device available");
    if (device >= 0 && (device >= ndev || cudaSetDevice(device) != cudaSuccess))
        return sset(nullptr, DEM_E_INVALID, "bad device index");
    if (c.memory_budget_bytes <= 0 || c.max_scenes <= 0 || !(c.cells_per_particle > 0.0f) ||
        c.bonds_per_particle < 0.0f)
        return sset(nullptr, DEM_E_INVALID, "bad server configuration");
    dem_server *sv = new (std::nothrow) dem_server();
    if (!sv) return sset(nullptr, DEM_E_OOM, "host allocation failed");
    sv->cfg = c;
    cudaGetDevice(&sv->world.device);
    if (cudaStreamCreateWithFlags(&sv->world.stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete sv;
        return sset(nullptr, DEM_E_CUDA, "stream creation failed");
    }
    // the arenas: particles, with cells and bonds in the configured ratios,
    // within the memory budget and at most max_active_particles
    const double per = (double)sv->world.bytes_per_particle() + 8.0 * c.cells_per_particle +
                       32.0 * c.bonds_per_particle;
    long long np = (long long)((double)c.memory_budget_bytes / per);
    if (c.max_active_particles > 0) np = std::min<long long>(np, (long long)(c.max_active_particles * 1.25) + 65536);
    np = std::max<long long>(std::min<long long>(np, demgb::MAX_WORLD_PARTICLES), 1024);
    long long nc = std::min<long long>((long long)(np * (double)c.cells_per_particle) + 4096, 1LL << 30);
    long long nb = std::min<long long>((long long)(np * (double)c.bonds_per_particle) + 1024, 1LL << 30);
    int rc = sv->world.build_capacity(np, nc, nb, c.max_scenes, 4 * c.max_scenes, c.ext);
    if (rc) {
        std::string m = sv->world.err;
        cudaStream_t st = sv->world.stream;
        delete sv;
        cudaStreamDestroy(st);
        return sset(nullptr, rc, m);
    }
    sv->slot_req.assign(sv->world.sh.size(), 0);
    *out = sv;
    return DEM_OK;
}

void dem_server_destroy(dem_server *sv) {
    if (!sv) return;
    cudaSetDevice(sv->world.device);
    cudaStream_t st = sv->world.stream;
    if (st) cudaStreamSynchronize(st);
    delete sv;
    if (st) cudaStreamDestroy(st);
}

}  // extern "C"

namespace {
// a request queued with its own copy of the scene (borrow = false) or
// referring to the caller's arrays until it is done (borrow = true)
int submit(dem_server *sv, const dem_scene *scene, const dem_params *params, const dem_ext *ext,
           int64_t horizon_steps, int64_t *request_id, bool borrow) {
    if (!scene || !params || horizon_steps <= 0) return sset(sv, DEM_E_INVALID, "bad request");
    if (scene->n_particles < 0 || (long long)scene->n_particles > sv->world.a_part.capacity())
        return sset(sv, DEM_E_CAPACITY, "request has more particles than the server's arena (" +
                                            std::to_string(sv->world.a_part.capacity()) + ")");
    auto r = std::make_unique<Request>();
    r->id = sv->next_id++;
    if (borrow) r->in.view = *scene;
    else r->in.from(*scene, true);
    r->params = *params;
    if (ext) r->ext = *ext;
    else dem_ext_defaults(&r->ext);
    if (r->ext.bond_normal_strength && scene->n_bonds > 0)
        r->sn.assign(r->ext.bond_normal_strength, r->ext.bond_normal_strength + scene->n_bonds);
    if (r->ext.bond_shear_strength && scene->n_bonds > 0)
        r->ss.assign(r->ext.bond_shear_strength, r->ext.bond_shear_strength + scene->n_bonds);
    r->ext.bond_normal_strength = nullptr;
    r->ext.bond_shear_strength = nullptr;
    r->horizon = horizon_steps;
    r->t_submit = now_s();
    if (request_id) *request_id = r->id;
    sv->queue.push_back(r->id);
    sv->reqs[r->id] = std::move(r);
    return DEM_OK;
}
}  // namespace

extern "C" {

int dem_server_submit(dem_server *sv, const dem_scene *scene, const dem_params *params, const dem_ext *ext,
                      int64_t horizon_steps, int64_t *request_id) {
    SERVER_GUARD(sv);
    return submit(sv, scene, params, ext, horizon_steps, request_id, false);
}

int dem_server_submit_borrowed(dem_server *sv, const dem_scene *scene, const dem_params *params,
                               const dem_ext *ext, int64_t horizon_steps, int64_t *request_id) {
    SERVER_GUARD(sv);
    return submit(sv, scene, params, ext, horizon_steps, request_id, true);
}

int dem_server_advance(dem_server *sv, int32_t n_steps) {
    SERVER_GUARD(sv);
    if (n_steps < 0) return sset(sv, DEM_E_INVALID, "n_steps < 0");
    int rc = retire_finished(sv);
    if (rc) return rc;
    rc = admit_queued(sv);
    if (rc) return rc;
    if (sv->active_particles == 0 || n_steps == 0) return DEM_OK;
    rc = sv->world.step(n_steps);
    if (rc) return src_(sv, rc);
    for (size_t s = 0; s < sv->slot_req.size(); ++s) {
        int64_t id = sv->slot_req[s];
        if (!id) continue;
        Request &r = *sv->reqs[id];
        int64_t k = std::min<int64_t>(n_steps, r.horizon - r.steps_done);
        r.steps_done += k;
        sv->particle_steps += k * r.in.view.n_particles;
    }
    rc = sv->world.sync();
    if (rc) return src_(sv, rc);
    return collect_events(sv);
}

int dem_server_poll(dem_server *sv, int64_t *done_ids, int32_t cap, int32_t *n) {
    SERVER_GUARD(sv);
    if (cap < 0 || (cap > 0 && !done_ids)) return sset(sv, DEM_E_INVALID, "bad buffer");
    int32_t k = (int32_t)std::min<size_t>(sv->done_unpolled.size(), (size_t)cap);
    for (int32_t i = 0; i < k; ++i) done_ids[i] = sv->done_unpolled[i];
    sv->done_unpolled.erase(sv->done_unpolled.begin(), sv->done_unpolled.begin() + k);
    if (n) *n = k;
    return DEM_OK;
}

int dem_server_fetch(dem_server *sv, int64_t id, dem_scene *out, double times[3]) {
    SERVER_GUARD(sv);
    auto it = sv->reqs.find(id);
    if (it == sv->reqs.end()) return sset(sv, DEM_E_INVALID, "unknown request id");
    Request &r = *it->second;
    if (r.state == 3) return sset(sv, r.fail_code, "request failed at admission: " + r.fail_msg);
    if (r.state != 2) return sset(sv, DEM_E_STATE, "request not completed");
    if (times) {
        times[0] = r.t_submit;
        times[1] = r.t_admit;
        times[2] = r.t_done;
    }
    if (out) {
        const dem_scene &s = r.out.view;
        if (out->n_particles != s.n_particles) return sset(sv, DEM_E_INVALID, "n_particles mismatch");
        const size_t n = (size_t)s.n_particles;
        auto cp = [&](auto *dst, const auto &src) {
            if (dst && !src.empty()) std::memcpy(dst, src.data(), src.size() * sizeof(src[0]));
        };
        cp(out->pos, r.out.pos); cp(out->radii, r.out.radii); cp(out->vel, r.out.vel); cp(out->acc, r.out.acc);
        cp(out->rot, r.out.rot); cp(out->rot_vel, r.out.rot_vel); cp(out->rot_acc, r.out.rot_acc);
        cp(out->forces, r.out.forces); cp(out->del_pos, r.out.del_pos); cp(out->del_rot, r.out.del_rot);
        cp(out->data, r.out.data); cp(out->fixity, r.out.fixity); cp(out->contacts, r.out.contacts);
        cp(out->material_pointers, r.out.material_pointers);
        if (out->n_materials == s.n_materials) cp(out->materials, r.out.materials);
        if (out->n_bonds == s.n_bonds) cp(out->bonds, r.out.bonds);
        std::memcpy(out->coll_cont, s.coll_cont, sizeof s.coll_cont);
        out->grid = s.grid;
        (void)n;
    }
    return DEM_OK;
}

int dem_server_events(dem_server *sv, int64_t id, dem_break_event *buf, int32_t cap, int32_t *n) {
    SERVER_GUARD(sv);
    auto it = sv->reqs.find(id);
    if (it == sv->reqs.end()) return sset(sv, DEM_E_INVALID, "unknown request id");
    auto &ev = it->second->events;
    int32_t k = (int32_t)std::min<size_t>(ev.size(), (size_t)std::max(cap, 0));
    if (k && buf) std::memcpy(buf, ev.data(), sizeof(dem_break_event) * k);
    if (n) *n = (int32_t)ev.size();
    return DEM_OK;
}

int dem_server_release(dem_server *sv, int64_t id) {
    SERVER_GUARD(sv);
    auto it = sv->reqs.find(id);
    if (it == sv->reqs.end()) return sset(sv, DEM_E_INVALID, "unknown request id");
    if (it->second->state < 2) return sset(sv, DEM_E_STATE, "request not completed");
    sv->reqs.erase(it);
    return DEM_OK;
}

int dem_server_cancel(dem_server *sv, int64_t id) {
    SERVER_GUARD(sv);
    auto it = sv->reqs.find(id);
    if (it == sv->reqs.end()) return sset(sv, DEM_E_INVALID, "unknown request id");
    Request &r = *it->second;
    if (r.state == 0) {
        sv->queue.erase(std::find(sv->queue.begin(), sv->queue.end(), id));
    } else if (r.state == 1) {
        // between advances nothing of the scene is in flight: free its ranges
        int rc = sv->world.retire(r.slot);
        if (rc) return src_(sv, rc);
        sv->slot_req[r.slot] = 0;
        sv->active_particles -= r.in.view.n_particles;
    }
    sv->done_unpolled.erase(std::remove(sv->done_unpolled.begin(), sv->done_unpolled.end(), id),
                            sv->done_unpolled.end());
    sv->reqs.erase(it);
    return DEM_OK;
}

int dem_server_get_stats(dem_server *sv, dem_server_stats *out) {
    SERVER_GUARD(sv);
    if (!out) return sset(sv, DEM_E_INVALID, "out is NULL");
    std::memset(out, 0, sizeof *out);
    out->queued = (int64_t)sv->queue.size();
    int64_t running = 0;
    for (auto id : sv->slot_req) running += id ? 1 : 0;
    out->running = running;
    out->completed = sv->completed;
    out->active_particles = sv->active_particles;
    out->particle_steps = sv->particle_steps;
    out->capacity_particles = sv->world.a_part.capacity();
    out->used_particles = sv->world.a_part.used();
    out->device_bytes = (int64_t)(sv->world.a_part.capacity() * sv->world.bytes_per_particle());
    out->steps = sv->world.host_step;
    out->waits_active = sv->waits_active;
    out->waits_memory = sv->waits_memory;
    return DEM_OK;
}

void *dem_server_stream(dem_server *sv) { return sv ? (void *)sv->world.stream : nullptr; }

}  // extern "C"

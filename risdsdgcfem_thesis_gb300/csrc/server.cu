// server.cu -- a step-request server over device-resident scenes: admission
// by a device-memory budget, shards of scenes stepped as batches, continuous
// batching across shards.
//
// The reference steps each solid when its owner asks (bs::Solid3D::Update,
// Saphyre2 bs/Solid3D.cpp:61-104, one command per solid through the MoP
// channel) and steps several solids one after another
// (SS_AggregateDSH_Basic::MultiDSH_Solid3D_Update,
// SS_AggregateDSH_Basic.cpp:229-300). Here a request asks for one FixedStep
// of one resident scene and many requests share the GPU:
//
//  * Admission. Scenes are registered on the host and wait. fem_server_admit
//    packs waiting scenes, sorted by size, into shards of at most
//    shard_max_tets tets / shard_max_scenes scenes, while the device bytes of
//    the shards built so far plus an estimate of the next one stay within
//    the budget; a shard whose actual bytes would break the budget is taken
//    down again and its scenes keep waiting. Removing every scene of a shard
//    frees its memory for waiting scenes.
//  * Shards. A shard is one batch (batch.cu): its scenes stay resident; a
//    launch of the shard is one CUDA-graph launch on the shard's own stream
//    that runs at most slice_iterations CG iterations (the batch's
//    iteration budget; shards of FIE scenes, whose Newton steps take no
//    budget, run whole steps). Scenes whose step is running continue (mask 2),
//    scenes with a request waiting start a step (mask 1), the others sit
//    out (mask 0).
//  * Continuous batching. fem_server_pump never blocks: it harvests every
//    shard whose launch has finished (a CUDA event), completes the requests
//    whose CG loop ended in it, and at once relaunches every idle shard that
//    has steps running or requests waiting. A request waits at most one
//    slice before its step starts, whatever else runs in the shard; shards
//    run concurrently on their streams, so work of different requests
//    overlaps on the device. Requests for one scene are served in order.
//
// A scene's result does not depend on which other scenes share its shard or
// step (every sum in the batch kernels has a fixed order), so a request
// gives the same bits alone and in the mix.
//
// Threading: a server is used from one host thread at a time.
#include "../../include/fem_tet.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <new>
#include <vector>

namespace femgb {
int batch_fail(int code, const char* fmt, ...);
int batch_enqueue_readback(fem_batch b);
unsigned batch_host_err(fem_batch b);
}  // namespace femgb

using femgb::batch_fail;

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    uint64_t tag;
    Clock::time_point t_submit;
};

enum SceneState : uint32_t { SCENE_WAITING = 0, SCENE_RESIDENT = 1, SCENE_REMOVED = 2 };

struct Scene {
    // host copy until admitted
    std::vector<double> rest, E, nu, knc_targets;
    std::vector<uint32_t> tets, knc_nodes;
    fem_params params{};
    uint32_t N = 0, T = 0;
    SceneState state = SCENE_WAITING;
    int shard = -1;
    uint32_t mesh = 0;  // index inside its shard's batch
    std::deque<Request> queue;
    bool inflight = false;       // its front request's step is running
    Clock::time_point t_start;   // launch that started that step
    double device_us = 0.0;      // device time of the launches it took part in
};

struct Shard {
    fem_batch b = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t start = nullptr, done = nullptr;
    std::vector<uint32_t> scenes;  // server scene id of each batch mesh
    std::vector<uint8_t> mask, flags;
    std::vector<uint32_t> inflight;  // scene ids taking part in the launch in flight
    Clock::time_point t_launch;
    uint64_t bytes = 0;
    uint32_t live = 0;
    bool busy = false;
};

// Upper estimate of a shard's device bytes (the batch layout: per tet the
// FP64 and element-type element data, tile CSR and mixed blob; per node the
// FP64 state vectors, element-type CG vectors and about 2.5 partial slots).
uint64_t estimate_bytes(uint32_t precision, uint64_t T, uint64_t N, uint64_t M)
{
    const bool fp64 = precision == FEM_PRECISION_FP64;
    const uint64_t per_tet = fp64 ? 300 : 310;
    const uint64_t per_node = fp64 ? 400 : 330;
    return per_tet * T + per_node * N + 512 * M + (1u << 20);
}

}  // namespace

struct fem_server_s {
    fem_server_options opt{};
    std::vector<Scene> scenes;
    std::vector<Shard> shards;  // a taken-down shard keeps its slot with b == nullptr
    uint64_t used_bytes = 0;
    uint64_t pending = 0;  // requests submitted and not completed
    uint32_t max_busy = 0;

    ~fem_server_s()
    {
        for (auto& sh : shards) take_down(sh);
    }

    void take_down(Shard& sh)
    {
        if (sh.b) {
            if (sh.busy) cudaEventSynchronize(sh.done);
            fem_batch_destroy(sh.b);
            sh.b = nullptr;
        }
        if (sh.start) cudaEventDestroy(sh.start);
        if (sh.done) cudaEventDestroy(sh.done);
        sh.start = sh.done = nullptr;
        sh.busy = false;
        used_bytes -= std::min(used_bytes, sh.bytes);
        sh.bytes = 0;
    }
};

namespace {

int check_server(fem_server s)
{
    if (!s) return batch_fail(FEM_E_ARG, "null server");
    return FEM_OK;
}

// Builds one shard from the scenes in `ids` (all waiting). Returns FEM_OK and
// fills `out`, or an error (nothing is left allocated).
int build_shard(fem_server srv, const std::vector<uint32_t>& ids, Shard& out)
{
    fem_batch_options o;
    fem_batch_options_default(&o);
    o.precision = srv->opt.precision;
    if (srv->opt.chunk_nodes) o.chunk_nodes = srv->opt.chunk_nodes;
    o.fuse_alpha = srv->opt.fuse_alpha;
    o.persistent_loop = srv->opt.persistent_loop;
    fem_batch b = nullptr;
    if (int e = fem_batch_create(&o, &b)) return e;
    for (uint32_t k = 0; k < ids.size(); k++) {
        Scene& sc = srv->scenes[ids[k]];
        fem_params p = sc.params;
        p.precision = srv->opt.precision;
        uint32_t mi = 0;
        int e = fem_batch_add_mesh(b, sc.rest.data(), sc.N, sc.tets.data(), sc.T, &p,
                                   sc.E.empty() ? nullptr : sc.E.data(), sc.nu.empty() ? nullptr : sc.nu.data(), &mi);
        if (!e && !sc.knc_nodes.empty())
            e = fem_batch_set_knc(b, mi, sc.knc_nodes.data(), sc.knc_targets.data(), (uint32_t)sc.knc_nodes.size());
        if (e) {
            fem_batch_destroy(b);
            return e;
        }
    }
    int e = fem_batch_finalize(b);
    // FIE shards step whole (a Newton step takes no iteration budget)
    const bool newton = srv->scenes[ids[0]].params.integrator != FEM_INTEGRATOR_QIE_V;
    if (!e) e = fem_batch_set_slice(b, newton ? 0u : srv->opt.slice_iterations);
    if (e) {
        fem_batch_destroy(b);
        return e;
    }
    uint64_t bytes = 0;
    fem_batch_info(b, nullptr, nullptr, nullptr, nullptr, &bytes);
    void* st = nullptr;
    fem_batch_stream(b, &st);
    out = Shard{};
    out.b = b;
    out.stream = static_cast<cudaStream_t>(st);
    if (cudaEventCreate(&out.start) != cudaSuccess || cudaEventCreate(&out.done) != cudaSuccess) {
        if (out.start) cudaEventDestroy(out.start);
        fem_batch_destroy(b);
        out = Shard{};
        return batch_fail(FEM_E_CUDA, "event creation failed");
    }
    out.scenes = ids;
    out.mask.assign(ids.size(), 0);
    out.flags.assign(ids.size(), 0);
    out.bytes = bytes;
    out.live = (uint32_t)ids.size();
    return FEM_OK;
}

// One launch of a shard: running steps continue, waiting requests start.
int launch_shard(fem_server srv, Shard& sh)
{
    sh.inflight.clear();
    const Clock::time_point now = Clock::now();
    for (uint32_t k = 0; k < sh.scenes.size(); k++) {
        Scene& sc = srv->scenes[sh.scenes[k]];
        uint8_t m = 0;
        if (sc.state == SCENE_RESIDENT) {
            if (sc.inflight) {
                m = 2;
            } else if (!sc.queue.empty()) {
                m = 1;
                sc.inflight = true;
                sc.t_start = now;
                sc.device_us = 0.0;
            }
        }
        sh.mask[k] = m;
        if (m) sh.inflight.push_back(sh.scenes[k]);
    }
    if (sh.inflight.empty()) return FEM_OK;
    if (int e = fem_batch_set_active(sh.b, sh.mask.data())) return e;
    if (cudaEventRecord(sh.start, sh.stream) != cudaSuccess) return batch_fail(FEM_E_CUDA, "event record failed");
    if (int e = fem_batch_step_async(sh.b, 1)) return e;
    if (int e = femgb::batch_enqueue_readback(sh.b)) return e;
    if (cudaEventRecord(sh.done, sh.stream) != cudaSuccess) return batch_fail(FEM_E_CUDA, "event record failed");
    sh.t_launch = now;
    sh.busy = true;
    return FEM_OK;
}

}  // namespace

extern "C" {

int fem_server_options_default(fem_server_options* o)
{
    if (!o) return batch_fail(FEM_E_ARG, "null options");
    std::memset(o, 0, sizeof(*o));
    o->precision = FEM_PRECISION_MIXED;
    o->hbm_budget_bytes = 120ull << 30;
    o->shard_max_tets = 32000000;
    o->shard_max_scenes = 2048;
    o->slice_iterations = 32;
    o->chunk_nodes = 256;
    return FEM_OK;
}

int fem_server_create(const fem_server_options* opt, fem_server* out)
{
    if (!out) return batch_fail(FEM_E_ARG, "null output handle");
    *out = nullptr;
    fem_server_options o;
    fem_server_options_default(&o);
    if (opt) o = *opt;
    if (o.precision != FEM_PRECISION_FP64 && o.precision != FEM_PRECISION_MIXED)
        return batch_fail(FEM_E_ARG, "unknown precision %u", o.precision);
    if (o.chunk_nodes && (o.chunk_nodes < 32 || o.chunk_nodes > 8192))
        return batch_fail(FEM_E_ARG, "chunk_nodes must be 0 or in [32, 8192]");
    if (o.shard_max_tets == 0 || o.shard_max_scenes == 0)
        return batch_fail(FEM_E_ARG, "shard limits must be > 0");
    fem_server s = new (std::nothrow) fem_server_s;
    if (!s) return batch_fail(FEM_E_OOM, "host allocation failed");
    s->opt = o;
    *out = s;
    return FEM_OK;
}

int fem_server_destroy(fem_server s)
{
    if (int e = check_server(s)) return e;
    delete s;
    return FEM_OK;
}

int fem_server_add_scene(fem_server s, const double* rest, uint32_t N, const uint32_t* tets, uint32_t T,
                         const fem_params* p, const double* young_per_elem, const double* poisson_per_elem,
                         const uint32_t* knc_nodes, const double* knc_targets, uint32_t knc_count, uint32_t* scene)
{
    if (int e = check_server(s)) return e;
    if (!rest || !tets || !p) return batch_fail(FEM_E_ARG, "null rest/tets/params");
    if (N == 0 || T == 0) return batch_fail(FEM_E_ARG, "empty mesh (N=%u, T=%u)", N, T);
    if (p->integrator > FEM_INTEGRATOR_FIE_DX_QUASISTATIC)
        return batch_fail(FEM_E_ARG, "unknown integrator %u", p->integrator);
    if (p->integrator != FEM_INTEGRATOR_QIE_V && s->opt.persistent_loop)
        return batch_fail(FEM_E_ARG, "the persistent loop takes QIE_V scenes only");
    if (p->rotation != FEM_ROTATION_MSVD && p->rotation != FEM_ROTATION_DAPD)
        return batch_fail(FEM_E_ARG, "unknown rotation %u", p->rotation);
    if (p->ls_solver != FEM_LS_CG && p->ls_solver != FEM_LS_MINRES)
        return batch_fail(FEM_E_ARG, "unknown ls_solver %u", p->ls_solver);
    if (p->material > FEM_MATERIAL_C_CCM) return batch_fail(FEM_E_ARG, "unknown material %u", p->material);
    if (p->material == FEM_MATERIAL_C_CCM && s->opt.precision != FEM_PRECISION_FP64)
        return batch_fail(FEM_E_ARG, "C_CCM runs in FP64 (its differential is not symmetric)");
    if (s->opt.persistent_loop && (p->ls_solver != FEM_LS_CG || p->material != FEM_MATERIAL_C_WRP))
        return batch_fail(FEM_E_ARG, "the persistent loop takes CG meshes of C_WRP only");
    if (knc_count && (!knc_nodes || !knc_targets)) return batch_fail(FEM_E_ARG, "null constraint arrays");
    for (size_t i = 0; i < 4 * (size_t)T; i++)
        if (tets[i] >= N) return batch_fail(FEM_E_INDEX, "tet %zu names node %u >= N=%u", i / 4, tets[i], N);
    for (uint32_t k = 0; k < knc_count; k++)
        if (knc_nodes[k] >= N) return batch_fail(FEM_E_INDEX, "constraint %u names node %u >= N=%u", k, knc_nodes[k], N);
    Scene sc;
    sc.rest.assign(rest, rest + 3 * (size_t)N);
    sc.tets.assign(tets, tets + 4 * (size_t)T);
    if (young_per_elem) sc.E.assign(young_per_elem, young_per_elem + T);
    if (poisson_per_elem) sc.nu.assign(poisson_per_elem, poisson_per_elem + T);
    if (knc_count) {
        sc.knc_nodes.assign(knc_nodes, knc_nodes + knc_count);
        sc.knc_targets.assign(knc_targets, knc_targets + 3 * (size_t)knc_count);
    }
    sc.params = *p;
    sc.N = N;
    sc.T = T;
    s->scenes.push_back(std::move(sc));
    if (scene) *scene = (uint32_t)(s->scenes.size() - 1);
    return FEM_OK;
}

int fem_server_admit(fem_server s, uint32_t* admitted)
{
    if (int e = check_server(s)) return e;
    if (admitted) *admitted = 0;
    std::vector<uint32_t> wait;
    for (uint32_t i = 0; i < s->scenes.size(); i++)
        if (s->scenes[i].state == SCENE_WAITING) wait.push_back(i);
    // similar sizes share a shard (a shard's step lasts as long as its
    // slowest scene's CG loop); FIE scenes, whose Newton steps run whole,
    // get shards of their own, so QIE shards keep their slices
    auto newton = [&](uint32_t i) { return s->scenes[i].params.integrator != FEM_INTEGRATOR_QIE_V; };
    std::stable_sort(wait.begin(), wait.end(), [&](uint32_t a, uint32_t b) {
        if (newton(a) != newton(b)) return !newton(a);
        return s->scenes[a].T < s->scenes[b].T;
    });
    size_t k = 0;
    uint32_t count = 0;
    while (k < wait.size()) {
        std::vector<uint32_t> ids;
        uint64_t T = 0, N = 0;
        while (k < wait.size() && ids.size() < s->opt.shard_max_scenes &&
               (ids.empty() || (T + s->scenes[wait[k]].T <= s->opt.shard_max_tets &&
                                newton(wait[k]) == newton(ids[0])))) {
            T += s->scenes[wait[k]].T;
            N += s->scenes[wait[k]].N;
            ids.push_back(wait[k++]);
        }
        if (s->used_bytes + estimate_bytes(s->opt.precision, T, N, ids.size()) > s->opt.hbm_budget_bytes) break;
        Shard sh;
        if (int e = build_shard(s, ids, sh)) return e;
        if (s->used_bytes + sh.bytes > s->opt.hbm_budget_bytes) {  // estimate was short: undo
            sh.bytes = 0;  // not counted yet
            s->take_down(sh);
            break;
        }
        s->used_bytes += sh.bytes;
        const int si = (int)s->shards.size();
        for (uint32_t m = 0; m < ids.size(); m++) {
            Scene& sc = s->scenes[ids[m]];
            sc.state = SCENE_RESIDENT;
            sc.shard = si;
            sc.mesh = m;
            std::vector<double>().swap(sc.rest);
            std::vector<uint32_t>().swap(sc.tets);
            std::vector<double>().swap(sc.E);
            std::vector<double>().swap(sc.nu);
        }
        s->shards.push_back(std::move(sh));
        count += (uint32_t)ids.size();
    }
    if (admitted) *admitted = count;
    return FEM_OK;
}

int fem_server_set_params(fem_server s, uint32_t scene, const fem_params* params)
{
    if (int e = check_server(s)) return e;
    if (scene >= s->scenes.size() || !params) return batch_fail(FEM_E_ARG, "bad scene index or null params");
    Scene& sc = s->scenes[scene];
    if (sc.state == SCENE_REMOVED) return batch_fail(FEM_E_ARG, "scene %u was removed", scene);
    if (!sc.queue.empty() || sc.inflight)
        return batch_fail(FEM_E_ARG, "scene %u has requests pending or in flight", scene);
    fem_params p = *params;
    p.precision = s->opt.precision;
    if (sc.state == SCENE_RESIDENT) {
        // the shard's batch takes it (its restrictions hold: an FIE scene
        // in a sliced shard is refused; remove and add it again)
        const bool newton_old = sc.params.integrator != FEM_INTEGRATOR_QIE_V;
        const bool newton_new = p.integrator != FEM_INTEGRATOR_QIE_V;
        if (newton_old != newton_new)
            return batch_fail(FEM_E_ARG, "scene %u: an integrator change moves it between shard kinds; remove and "
                                         "add it again", scene);
        if (int e = fem_batch_set_params(s->shards[sc.shard].b, sc.mesh, &p)) return e;
    }
    sc.params = p;
    return FEM_OK;
}

int fem_server_remove_scene(fem_server s, uint32_t scene)
{
    if (int e = check_server(s)) return e;
    if (scene >= s->scenes.size()) return batch_fail(FEM_E_ARG, "scene %u out of range", scene);
    Scene& sc = s->scenes[scene];
    if (sc.state == SCENE_REMOVED) return FEM_OK;
    if (!sc.queue.empty() || sc.inflight)
        return batch_fail(FEM_E_ARG, "scene %u has requests pending or in flight", scene);
    if (sc.state == SCENE_RESIDENT) {
        Shard& sh = s->shards[sc.shard];
        if (--sh.live == 0) s->take_down(sh);
    }
    sc.state = SCENE_REMOVED;
    std::vector<double>().swap(sc.rest);
    std::vector<uint32_t>().swap(sc.tets);
    return FEM_OK;
}

int fem_server_submit(fem_server s, uint32_t scene, uint64_t tag)
{
    if (int e = check_server(s)) return e;
    if (scene >= s->scenes.size()) return batch_fail(FEM_E_ARG, "scene %u out of range", scene);
    Scene& sc = s->scenes[scene];
    if (sc.state != SCENE_RESIDENT)
        return batch_fail(FEM_E_ARG, "scene %u is not resident (admit it first)", scene);
    sc.queue.push_back(Request{tag, Clock::now()});
    s->pending++;
    return FEM_OK;
}

int fem_server_pump(fem_server s, fem_server_completion* out, uint32_t cap, uint32_t* n_out)
{
    if (int e = check_server(s)) return e;
    if (n_out) *n_out = 0;
    if (cap && !out) return batch_fail(FEM_E_ARG, "null completion array");
    uint32_t n = 0;
    // harvest finished shard launches (leave a shard unharvested when its
    // completions might not fit into `out`)
    for (auto& sh : s->shards) {
        if (!sh.b || !sh.busy) continue;
        if (n + sh.inflight.size() > cap) continue;
        const cudaError_t q = cudaEventQuery(sh.done);
        if (q == cudaErrorNotReady) continue;
        if (q != cudaSuccess) return batch_fail(FEM_E_CUDA, "shard launch: %s", cudaGetErrorString(q));
        const Clock::time_point now = Clock::now();
        float dev_ms = 0.f;
        cudaEventElapsedTime(&dev_ms, sh.start, sh.done);
        const unsigned err = femgb::batch_host_err(sh.b);
        fem_batch_finished(sh.b, sh.flags.data());
        for (uint32_t id : sh.inflight) {
            Scene& sc = s->scenes[id];
            sc.device_us += 1e3 * (double)dev_ms;
            if (sh.flags[sc.mesh] == 2 && !err) continue;  // still iterating: next launch
            fem_step_stats st{};
            fem_batch_get_stats(sh.b, sc.mesh, &st);
            const Request r = sc.queue.front();
            sc.queue.pop_front();
            sc.inflight = false;
            s->pending--;
            fem_server_completion& c = out[n++];
            c.tag = r.tag;
            c.scene = id;
            c.status = err ? (uint32_t)FEM_E_TIMEOUT : st.status;
            c.cg_iterations = st.cg_iterations;
            c.fp64_resolved = st.fp64_resolved;
            c.latency_us = std::chrono::duration<double, std::micro>(now - r.t_submit).count();
            c.queue_us = std::chrono::duration<double, std::micro>(sc.t_start - r.t_submit).count();
            if (c.queue_us < 0) c.queue_us = 0;
            c.device_us = sc.device_us;
        }
        sh.inflight.clear();
        sh.busy = false;
    }
    // relaunch every idle shard with steps running or requests waiting
    uint32_t busy = 0;
    for (auto& sh : s->shards) {
        if (!sh.b) continue;
        if (!sh.busy)
            if (int e = launch_shard(s, sh)) return e;
        busy += sh.busy ? 1u : 0u;
    }
    s->max_busy = std::max(s->max_busy, busy);
    if (n_out) *n_out = n;
    return FEM_OK;
}

int fem_server_get_state(fem_server s, uint32_t scene, double* x, double* v)
{
    if (int e = check_server(s)) return e;
    if (scene >= s->scenes.size()) return batch_fail(FEM_E_ARG, "scene %u out of range", scene);
    Scene& sc = s->scenes[scene];
    if (sc.state != SCENE_RESIDENT) return batch_fail(FEM_E_ARG, "scene %u is not resident", scene);
    Shard& sh = s->shards[sc.shard];
    if (sh.busy && cudaEventSynchronize(sh.done) != cudaSuccess)
        return batch_fail(FEM_E_CUDA, "waiting for the shard's step failed");
    return fem_batch_get_state(sh.b, sc.mesh, x, v);
}

int fem_server_set_state(fem_server s, uint32_t scene, const double* x, const double* v)
{
    if (int e = check_server(s)) return e;
    if (scene >= s->scenes.size()) return batch_fail(FEM_E_ARG, "scene %u out of range", scene);
    Scene& sc = s->scenes[scene];
    if (sc.state != SCENE_RESIDENT) return batch_fail(FEM_E_ARG, "scene %u is not resident", scene);
    Shard& sh = s->shards[sc.shard];
    if (sh.busy && cudaEventSynchronize(sh.done) != cudaSuccess)
        return batch_fail(FEM_E_CUDA, "waiting for the shard's step failed");
    return fem_batch_set_state(sh.b, sc.mesh, x, v);
}

int fem_server_scene_info(fem_server s, uint32_t scene, uint32_t* state, uint32_t* shard, uint32_t* pending)
{
    if (int e = check_server(s)) return e;
    if (scene >= s->scenes.size()) return batch_fail(FEM_E_ARG, "scene %u out of range", scene);
    const Scene& sc = s->scenes[scene];
    if (state) *state = (uint32_t)sc.state;
    if (shard) *shard = sc.shard < 0 ? 0xffffffffu : (uint32_t)sc.shard;
    if (pending) *pending = (uint32_t)sc.queue.size();
    return FEM_OK;
}

int fem_server_get_status(fem_server s, fem_server_status* info)
{
    if (int e = check_server(s)) return e;
    if (!info) return batch_fail(FEM_E_ARG, "null info");
    std::memset(info, 0, sizeof(*info));
    for (const auto& sc : s->scenes) {
        info->resident_scenes += sc.state == SCENE_RESIDENT ? 1u : 0u;
        info->waiting_scenes += sc.state == SCENE_WAITING ? 1u : 0u;
    }
    for (const auto& sh : s->shards) {
        info->shards += sh.b ? 1u : 0u;
        info->busy_shards += (sh.b && sh.busy) ? 1u : 0u;
    }
    info->max_busy_shards = s->max_busy;
    info->device_bytes = s->used_bytes;
    info->pending_requests = s->pending;
    return FEM_OK;
}

}  // extern "C"

// Scene server: many independent scenes advanced together on one GPU.
//
// No counterpart in the reference, which runs one scene per process.  A
// request is a scene (deep-copied at submission), its options and a step
// count.  Requests are admitted first come, first served while the estimated
// device memory of the admitted scenes (demsph_estimate_bytes, with a margin
// for list growth) stays inside the configured budget; each admitted scene
// gets its own engine, hence its own CUDA stream and stream-ordered memory.
// Worker threads take turns advancing the scenes in chunks of steps
// (demsph_update), so the kernels of different scenes overlap on the device.
// A scene replays CUDA graphs while it is the only active one; in a mix it
// launches its kernels directly (graph capture and instantiation next to
// other scenes' work cost hundreds of times more than on an idle GPU, more
// than the graphs save).  In batch mode one thread advances every active
// scene together instead, a round of steps per scene in one graph launch
// (demsph_batch_update); the workers then create engines (and run each
// scene's first step) and download finished scenes.  A scene that arrives while others run is
// admitted as soon as memory frees up (continuous batching).  A finished
// scene's final state is downloaded, its engine destroyed and its memory
// released before the next admission.
//
// Per-step latency is the wall time of a chunk on the host divided by its
// steps: the time a scene waits for its share of the GPU is included.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/demsph_gb300.h"

namespace {

using Clock = std::chrono::steady_clock;

double seconds(Clock::time_point a, Clock::time_point b) { return std::chrono::duration<double>(b - a).count(); }

// A demsph_scene whose arrays this object owns.
struct OwnedScene {
    demsph_scene s{};
    std::vector<std::vector<double>> d;
    std::vector<std::vector<int>> i;

    const double* keep(const double* p, size_t n)
    {
        if (!p || n == 0) return nullptr;
        d.emplace_back(p, p + n);
        return d.back().data();
    }
    const int* keep(const int* p, size_t n)
    {
        if (!p || n == 0) return nullptr;
        i.emplace_back(p, p + n);
        return i.back().data();
    }
    explicit OwnedScene(const demsph_scene& src)
    {
        s = src;
        d.reserve(40);
        i.reserve(10);
        const size_t nf = src.n_fluid, ns = src.n_solid, nc = src.n_clump, nw = src.n_wall;
        const size_t slots = (size_t)src.n_material * (src.n_material + 1) / 2;
        s.fluid_position = keep(src.fluid_position, 3 * nf);
        s.fluid_velocity = keep(src.fluid_velocity, 3 * nf);
        s.fluid_acceleration = keep(src.fluid_acceleration, 3 * nf);
        s.fluid_smoothing_length = keep(src.fluid_smoothing_length, nf);
        s.fluid_rho0 = keep(src.fluid_rho0, nf);
        s.fluid_drho = keep(src.fluid_drho, nf);
        s.fluid_sound_speed = keep(src.fluid_sound_speed, nf);
        s.fluid_nu = keep(src.fluid_nu, nf);
        s.solid_position = keep(src.solid_position, 3 * ns);
        s.solid_velocity = keep(src.solid_velocity, 3 * ns);
        s.solid_acceleration = keep(src.solid_acceleration, 3 * ns);
        s.solid_normal = keep(src.solid_normal, 3 * ns);
        s.solid_torque = keep(src.solid_torque, 3 * ns);
        s.solid_angular_velocity = keep(src.solid_angular_velocity, 3 * ns);
        s.solid_effective_radius = keep(src.solid_effective_radius, ns);
        s.solid_radius = keep(src.solid_radius, ns);
        s.solid_inverse_mass = keep(src.solid_inverse_mass, ns);
        s.solid_material = keep(src.solid_material, ns);
        s.solid_cluster = keep(src.solid_cluster, ns);
        s.solid_clump = keep(src.solid_clump, ns);
        s.solid_is_dummy = keep(src.solid_is_dummy, ns);
        s.clump_centroid = keep(src.clump_centroid, 3 * nc);
        s.clump_velocity = keep(src.clump_velocity, 3 * nc);
        s.clump_acceleration = keep(src.clump_acceleration, 3 * nc);
        s.clump_angular_velocity = keep(src.clump_angular_velocity, 3 * nc);
        s.clump_torque = keep(src.clump_torque, 3 * nc);
        s.clump_orientation = keep(src.clump_orientation, 4 * nc);
        s.clump_inverse_inertia = keep(src.clump_inverse_inertia, 6 * nc);
        s.clump_inverse_mass = keep(src.clump_inverse_mass, nc);
        s.clump_pebble_start = keep(src.clump_pebble_start, nc);
        s.clump_pebble_end = keep(src.clump_pebble_end, nc);
        s.wall_point = keep(src.wall_point, 3 * nw);
        s.wall_normal = keep(src.wall_normal, 3 * nw);
        s.wall_material = keep(src.wall_material, nw);
        s.hertzian = keep(src.hertzian, 8 * slots);
        s.linear = keep(src.linear, 11 * slots);
        s.bonded = keep(src.bonded, 6 * slots);
    }
};

enum class State { Pending, Active, Done, Failed };

struct Request {
    long long id = 0;
    std::unique_ptr<OwnedScene> scene;
    demsph_options opt{};
    int steps = 0, next = 1, gap = 1;
    double dt = 0;
    long long mobile = 0;          // solids with mass: updated every step
    long long reserved = 0;        // bytes held against the budget
    State state = State::Pending;
    bool busy = false;             // a worker is advancing it
    demsph_engine* eng = nullptr;
    Clock::time_point submitted, admitted, finished, lastRun;
    std::string error;
    int status = DEMSPH_OK;
    std::vector<double> fpos, fvel, facc, fdrho, spos, svel, sacc, snormal, storque, sangvel;
};

}  // namespace

struct demsph_server {
    demsph_server_config cfg{};
    std::mutex m;
    std::condition_variable cv;   // work available, or a request finished
    std::map<long long, std::unique_ptr<Request>> reqs;
    std::deque<long long> pending;
    long long nextId = 1;
    long long used = 0, peak = 0;
    bool stop = false;
    std::vector<std::thread> workers;
    // statistics
    std::vector<double> stepMs;   // per chunk: milliseconds per step
    long long updates = 0, completed = 0, failed = 0, submittedN = 0, admittedN = 0, stepsRun = 0;
    long long activeN = 0;        // admitted requests not yet finished
    double createS = 0, stepS = 0, downloadS = 0;   // worker time by activity
    std::map<int, int> lanesByClass;   // autotuned threads per fluid particle by log2(fluid count)
    std::thread batcher;               // batch mode: the thread launching the rounds
    long long batchRounds = 0;
    demsph_batch_info batchInfo{};     // batch mode: the batch's figures (refreshed after each round)
    Clock::time_point lastJoin;        // batch mode: when the batch's membership last grew
    bool anyAdmitted = false;
    Clock::time_point firstAdmit, lastFinish;

    // Admits pending requests in arrival order while they fit (lock held).
    void admit()
    {
        while (!pending.empty()) {
            Request& r = *reqs[pending.front()];
            if (used + r.reserved > cfg.hbm_budget_bytes && used > 0) break;  // an empty server takes anything
            pending.pop_front();
            r.state = State::Active;
            r.admitted = Clock::now();
            used += r.reserved;
            peak = std::max(peak, used);
            ++admittedN;
            ++activeN;
            if (!anyAdmitted) {
                anyAdmitted = true;
                firstAdmit = r.admitted;
            }
        }
    }

    // The active request not being advanced that waited longest (lock held).
    // In batch mode the workers take only requests without an engine and
    // requests whose steps are all done.
    Request* pick()
    {
        Request* best = nullptr;
        for (auto& kv : reqs) {
            Request& r = *kv.second;
            if (r.state != State::Active || r.busy) continue;
            if (cfg.batch && r.eng && r.next <= r.steps) continue;
            if (!best || r.lastRun < best->lastRun) best = &r;
        }
        return best;
    }

    // Batch mode: steps of a scene's round - whole Shepard periods (5 gap
    // steps with fluid), an even count (the contact-list parity repeats), about
    // batch_round_steps - so that its captured round repeats.
    int roundSteps(const Request& r) const
    {
        const int per = r.scene->s.n_fluid > 0 ? 5 * r.gap : 1;
        const int target = cfg.batch_round_steps;
        int n = per * std::max(1, (target + per / 2) / per);
        if (n & 1) n *= 2;
        return std::min(n, r.steps - r.next + 1);
    }

    void batchLoop()
    {
        demsph_batch* b = nullptr;
        const int brc = demsph_batch_create(cfg.device, &b);
        std::unique_lock<std::mutex> lock(m);
        std::vector<Request*> mem;
        std::vector<demsph_engine*> eng;
        std::vector<int> first, n, gap, st;
        std::vector<double> dt;
        std::vector<long long> ids;  // the members of the last round
        while (true) {
            auto ready = [&](const Request& r) {
                return r.state == State::Active && !r.busy && r.eng && r.next <= r.steps;
            };
            auto creating = [&] {
                for (auto& kv : reqs)
                    if (kv.second->state == State::Active && !kv.second->eng) return true;
                return false;
            };
            cv.wait(lock, [&] {
                if (stop) return true;
                for (auto& kv : reqs)
                    if (ready(*kv.second)) return true;
                return false;
            });
            if (stop) break;
            if (brc != DEMSPH_OK) {  // no batch: the requests fail
                for (auto& kv : reqs) {
                    Request& r = *kv.second;
                    if (!ready(r)) continue;
                    r.status = brc;
                    r.error = "demsph_batch_create failed";
                    demsph_destroy(r.eng);
                    r.eng = nullptr;
                    finish(r, State::Failed);
                }
                continue;
            }
            // members: last round's members still running, plus newcomers -
            // newcomers join when no engine is being created, or 1 s after the
            // membership last grew (each change instantiates a new graph; the
            // first round waits the same way for the engines being created)
            if (ids.empty() && lastJoin == Clock::time_point{}) lastJoin = Clock::now();
            const bool admitNew = !creating() || seconds(lastJoin, Clock::now()) > 1.0;
            mem.clear();
            bool grew = false;
            for (auto& kv : reqs) {
                Request& r = *kv.second;
                if (!ready(r)) continue;
                const bool old = std::find(ids.begin(), ids.end(), r.id) != ids.end();
                if (!old && !admitNew) continue;
                grew |= !old;
                mem.push_back(&r);
            }
            if (mem.empty()) {  // only newcomers, held back: wait for them briefly
                cv.wait_for(lock, std::chrono::milliseconds(10));
                continue;
            }
            if (grew) lastJoin = Clock::now();
            const size_t k = mem.size();
            eng.resize(k);
            first.resize(k);
            n.resize(k);
            gap.resize(k);
            st.resize(k);
            dt.resize(k);
            ids.clear();
            for (size_t q = 0; q < k; ++q) {
                Request& r = *mem[q];
                r.busy = true;
                eng[q] = r.eng;
                first[q] = r.next;
                n[q] = roundSteps(r);
                gap[q] = r.gap;
                dt[q] = r.dt;
                ids.push_back(r.id);
            }
            lock.unlock();
            const auto t0 = Clock::now();
            const int rc = demsph_batch_update(b, eng.data(), (int)k, first.data(), n.data(), dt.data(), gap.data(),
                                               st.data());
            const double wall = seconds(t0, Clock::now());
            lock.lock();
            ++batchRounds;
            stepS += wall;
            demsph_batch_get_info(b, &batchInfo);
            for (size_t q = 0; q < k; ++q) {
                Request& r = *mem[q];
                r.busy = false;
                r.lastRun = Clock::now();
                const int code = rc != DEMSPH_OK ? rc : st[q];
                if (code != DEMSPH_OK) {
                    r.status = code;
                    r.error = demsph_last_error(r.eng);
                    demsph_destroy(r.eng);
                    r.eng = nullptr;
                    finish(r, State::Failed);
                    continue;
                }
                long long fluidSteps = 0;
                for (int s2 = r.next; s2 < r.next + n[q]; ++s2) fluidSteps += (s2 % r.gap == 0);
                updates += fluidSteps * r.scene->s.n_fluid + (long long)n[q] * r.mobile;
                stepsRun += n[q];
                stepMs.push_back(1e3 * wall / std::max(1, n[q]));
                r.next += n[q];
            }
            cv.notify_all();  // finished scenes go to the workers
        }
        if (b) demsph_batch_get_info(b, &batchInfo);
        lock.unlock();
        if (b) demsph_batch_destroy(b);
    }

    void finish(Request& r, State s)
    {
        r.state = s;
        r.finished = Clock::now();
        lastFinish = r.finished;
        used -= r.reserved;
        --activeN;
        if (s == State::Done) ++completed;
        else ++failed;
        admit();
        cv.notify_all();
    }

    void work()
    {
        std::unique_lock<std::mutex> lock(m);
        while (true) {
            Request* r = nullptr;
            cv.wait(lock, [&] { return stop || (r = pick()) != nullptr; });
            if (stop) return;
            r->busy = true;
            const int useGraph = cfg.graphs > 0 || (cfg.graphs == 0 && activeN == 1) ? 1 : 0;
            lock.unlock();
            int rc = DEMSPH_OK;
            std::string err;
            double tCreate = 0, tStep = 0, tDown = 0;
            if (!r->eng) {
                const auto t0 = Clock::now();
                int cls = -1, known = 0;
                if (cfg.autotune && r->scene->s.n_fluid > 0) {
                    cls = 0;
                    while ((2LL << cls) <= r->scene->s.n_fluid) ++cls;
                    std::lock_guard<std::mutex> g(m);
                    auto it = lanesByClass.find(cls);
                    if (it != lanesByClass.end()) known = it->second;
                }
                if (known) r->opt.fluid_lanes = known;
                rc = demsph_create(&r->scene->s, &r->opt, &r->eng);
                if (rc == DEMSPH_OK) rc = demsph_initialize(r->eng);
                if (rc == DEMSPH_OK && cls >= 0 && !known) {
                    int lanes = 0;
                    rc = demsph_autotune(r->eng, &lanes);
                    std::lock_guard<std::mutex> g(m);
                    if (rc == DEMSPH_OK) lanesByClass.emplace(cls, lanes);
                }
                tCreate = seconds(t0, Clock::now());
            }
            int n = 0;
            long long upd = 0;
            double ms = 0;
            if (rc == DEMSPH_OK && cfg.batch && r->next == 1) {
                // the first step alone (it stores the Shepard reference sums),
                // so that the batch's rounds all start past it
                const auto t0 = Clock::now();
                rc = demsph_update(r->eng, r->dt, 1, 1, r->gap, 0);
                tStep = seconds(t0, Clock::now());
                n = 1;
                ms = 1e3 * tStep;
                upd = (1 % r->gap == 0 ? r->scene->s.n_fluid : 0) + r->mobile;
            } else if (rc == DEMSPH_OK && !cfg.batch) {
                n = std::min(cfg.chunk_steps, r->steps - r->next + 1);
                const auto t0 = Clock::now();
                rc = demsph_update(r->eng, r->dt, r->next, n, r->gap, useGraph);
                tStep = seconds(t0, Clock::now());
                ms = 1e3 * tStep / std::max(1, n);
                long long fluidSteps = 0;
                for (int k = r->next; k < r->next + n; ++k) fluidSteps += (k % r->gap == 0);
                upd = fluidSteps * r->scene->s.n_fluid + (long long)n * r->mobile;
            }
            bool done = rc == DEMSPH_OK && r->next + n > r->steps;
            if (rc == DEMSPH_OK && done) {
                const auto t0 = Clock::now();
                rc = download(*r);
                tDown = seconds(t0, Clock::now());
            }
            if (rc != DEMSPH_OK) err = r->eng ? demsph_last_error(r->eng) : demsph_status_string(rc);
            if ((done || rc != DEMSPH_OK) && r->eng) {
                demsph_destroy(r->eng);
                r->eng = nullptr;
            }
            lock.lock();
            createS += tCreate;
            stepS += tStep;
            downloadS += tDown;
            r->busy = false;
            r->lastRun = Clock::now();
            if (rc != DEMSPH_OK) {
                r->status = rc;
                r->error = err;
                finish(*r, State::Failed);
                continue;
            }
            r->next += n;
            if (n > 0) stepMs.push_back(ms);
            updates += upd;
            stepsRun += n;
            if (done) finish(*r, State::Done);
            else cv.notify_all();
        }
    }

    static int download(Request& r)
    {
        const size_t nf = r.scene->s.n_fluid, ns = r.scene->s.n_solid;
        r.fpos.resize(3 * nf);
        r.fvel.resize(3 * nf);
        r.facc.resize(3 * nf);
        r.fdrho.resize(nf);
        r.spos.resize(3 * ns);
        r.svel.resize(3 * ns);
        r.sacc.resize(3 * ns);
        r.snormal.resize(3 * ns);
        r.storque.resize(3 * ns);
        r.sangvel.resize(3 * ns);
        int rc = DEMSPH_OK;
        if (nf) rc = demsph_download_fluids(r.eng, r.fpos.data(), r.fvel.data(), r.facc.data(), r.fdrho.data());
        if (rc == DEMSPH_OK && ns)
            rc = demsph_download_solids(r.eng, r.spos.data(), r.svel.data(), r.sacc.data(), r.snormal.data(),
                                        r.storque.data(), r.sangvel.data());
        return rc;
    }
};

extern "C" {

int demsph_server_create(const demsph_server_config* cfg, demsph_server** out)
{
    if (!out) return DEMSPH_ERR_ARGUMENT;
    *out = nullptr;
    demsph_server_config c{};
    if (cfg) c = *cfg;
    if (c.hbm_budget_bytes <= 0) c.hbm_budget_bytes = 150LL << 30;
    if (c.workers <= 0) c.workers = 8;  // the mix measured fastest with 8 to 16 (16 host cores)
    if (c.chunk_steps <= 0) c.chunk_steps = 100;
    if (c.batch_round_steps <= 0) c.batch_round_steps = 20;
    if (c.workers > 256 || c.graphs < -1 || c.graphs > 1) return DEMSPH_ERR_ARGUMENT;
    auto* s = new demsph_server;
    s->cfg = c;
    for (int k = 0; k < c.workers; ++k) s->workers.emplace_back([s] { s->work(); });
    if (c.batch) s->batcher = std::thread([s] { s->batchLoop(); });
    *out = s;
    return DEMSPH_OK;
}

int demsph_server_destroy(demsph_server* s)
{
    if (!s) return DEMSPH_ERR_ARGUMENT;
    {
        std::lock_guard<std::mutex> lock(s->m);
        s->stop = true;
    }
    s->cv.notify_all();
    for (auto& t : s->workers) t.join();
    if (s->batcher.joinable()) s->batcher.join();
    for (auto& kv : s->reqs)
        if (kv.second->eng) demsph_destroy(kv.second->eng);
    delete s;
    return DEMSPH_OK;
}

int demsph_server_submit(demsph_server* s, const demsph_scene* scene, const demsph_options* opts, int n_steps,
                         long long* request_id)
{
    if (!s || !scene || n_steps < 1 || !request_id) return DEMSPH_ERR_ARGUMENT;
    if (scene->time_step <= 0 || scene->fluid_integrate_gap < 1) return DEMSPH_ERR_ARGUMENT;
    const long long est = demsph_estimate_bytes(scene, opts);
    if (est < 0) return DEMSPH_ERR_ARGUMENT;
    auto r = std::make_unique<Request>();
    r->scene = std::make_unique<OwnedScene>(*scene);
    if (opts) r->opt = *opts;
    r->opt.device = s->cfg.device;
    r->steps = n_steps;
    r->dt = scene->time_step;
    r->gap = scene->fluid_integrate_gap;
    r->reserved = est + est / 4;  // margin for list growth and bonds
    for (int i = 0; i < scene->n_solid; ++i) r->mobile += scene->solid_inverse_mass[i] > 0;
    r->submitted = Clock::now();
    std::lock_guard<std::mutex> lock(s->m);
    if (r->reserved > s->cfg.hbm_budget_bytes) return DEMSPH_ERR_CAPACITY;  // never fits
    r->id = s->nextId++;
    *request_id = r->id;
    s->pending.push_back(r->id);
    s->reqs[r->id] = std::move(r);
    ++s->submittedN;
    s->admit();
    s->cv.notify_all();
    return DEMSPH_OK;
}

int demsph_server_wait(demsph_server* s, long long id, double timeout_s)
{
    if (!s) return DEMSPH_ERR_ARGUMENT;
    std::unique_lock<std::mutex> lock(s->m);
    auto done = [&] {
        if (id < 0) return s->pending.empty() && s->completed + s->failed == s->submittedN;
        auto it = s->reqs.find(id);
        return it == s->reqs.end() || it->second->state == State::Done || it->second->state == State::Failed;
    };
    if (timeout_s < 0) s->cv.wait(lock, done);
    else if (!s->cv.wait_for(lock, std::chrono::duration<double>(timeout_s), done)) return DEMSPH_ERR_TIMEOUT;
    if (id >= 0) {
        auto it = s->reqs.find(id);
        if (it == s->reqs.end()) return DEMSPH_ERR_ARGUMENT;
        if (it->second->state == State::Failed) return it->second->status;
    }
    return DEMSPH_OK;
}

int demsph_server_fetch(demsph_server* s, long long id, double* fluid_position, double* fluid_velocity,
                        double* fluid_drho, double* solid_position, double* solid_velocity,
                        double* solid_angular_velocity)
{
    if (!s) return DEMSPH_ERR_ARGUMENT;
    std::lock_guard<std::mutex> lock(s->m);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return DEMSPH_ERR_ARGUMENT;
    const Request& r = *it->second;
    if (r.state == State::Failed) return r.status;
    if (r.state != State::Done) return DEMSPH_ERR_STATE;
    auto put = [](double* dst, const std::vector<double>& v) {
        if (dst && !v.empty()) std::memcpy(dst, v.data(), sizeof(double) * v.size());
    };
    put(fluid_position, r.fpos);
    put(fluid_velocity, r.fvel);
    put(fluid_drho, r.fdrho);
    put(solid_position, r.spos);
    put(solid_velocity, r.svel);
    put(solid_angular_velocity, r.sangvel);
    return DEMSPH_OK;
}

int demsph_server_release(demsph_server* s, long long id)
{
    if (!s) return DEMSPH_ERR_ARGUMENT;
    std::lock_guard<std::mutex> lock(s->m);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return DEMSPH_ERR_ARGUMENT;
    if (it->second->state != State::Done && it->second->state != State::Failed) return DEMSPH_ERR_STATE;
    s->reqs.erase(it);
    return DEMSPH_OK;
}

int demsph_server_request_info(demsph_server* s, long long id, demsph_request_info* info)
{
    if (!s || !info) return DEMSPH_ERR_ARGUMENT;
    std::lock_guard<std::mutex> lock(s->m);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return DEMSPH_ERR_ARGUMENT;
    const Request& r = *it->second;
    *info = demsph_request_info{};
    info->state = (int)r.state;
    info->steps_done = r.next - 1;
    info->reserved_bytes = r.reserved;
    const auto now = Clock::now();
    const bool admitted = r.state != State::Pending;
    const bool ended = r.state == State::Done || r.state == State::Failed;
    info->queued_s = seconds(r.submitted, admitted ? r.admitted : now);
    info->run_s = admitted ? seconds(r.admitted, ended ? r.finished : now) : 0.0;
    return DEMSPH_OK;
}

int demsph_server_stats(demsph_server* s, demsph_server_summary* st)
{
    if (!s || !st) return DEMSPH_ERR_ARGUMENT;
    std::lock_guard<std::mutex> lock(s->m);
    *st = demsph_server_summary{};
    st->submitted = s->submittedN;
    st->admitted = s->admittedN;
    st->completed = s->completed;
    st->failed = s->failed;
    st->pending = (long long)s->pending.size();
    st->steps = s->stepsRun;
    st->particle_updates = s->updates;
    st->bytes_in_use = s->used;
    st->create_s = s->createS;
    st->step_s = s->stepS;
    st->download_s = s->downloadS;
    st->peak_bytes = s->peak;
    st->batch_rounds = s->batchInfo.launches;
    st->batch_graph_builds = s->batchInfo.graph_builds;
    st->batch_capture_s = s->batchInfo.capture_s;
    st->batch_instantiate_s = s->batchInfo.instantiate_s;
    st->batch_launch_s = s->batchInfo.launch_s;
    if (s->anyAdmitted) {
        const auto end = (s->completed + s->failed == s->admittedN && s->pending.empty()) ? s->lastFinish : Clock::now();
        st->busy_s = seconds(s->firstAdmit, end);
        if (st->busy_s > 0) st->updates_per_s = (double)s->updates / st->busy_s;
    }
    if (!s->stepMs.empty()) {
        std::vector<double> v = s->stepMs;
        std::sort(v.begin(), v.end());
        auto q = [&](double f) { return v[std::min(v.size() - 1, (size_t)(f * (v.size() - 1) + 0.5))]; };
        st->p50_step_ms = q(0.50);
        st->p99_step_ms = q(0.99);
        st->chunks = (long long)v.size();
    }
    return DEMSPH_OK;
}

}  // extern "C"

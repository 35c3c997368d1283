// server.cpp -- continuous-batching request loop over batched arenas.
//
// Requests are laid out (build_instance) on host worker threads as they arrive.  The
// scheduling thread runs rounds: wait for the previous round's device work, retire
// stopped instances (final state copied to the host), free arenas with no instance
// left, enqueue the next chunk of iterations on every arena's own stream, and only
// then admit waiting requests into new arenas, so that host-side assembly and
// uploads overlap with device work already queued.  Admission is oldest-first: the
// oldest waiting request opens an arena and takes along waiting requests of the same
// physics whose cell counts are within size_ratio of its own, as long as the arena's
// exact device bytes fit what the budget has left.  With escalation on, a request
// whose split-precision solve stops with an error is solved again from its initial
// state in plain FP64 (same id; the result says so).  With FP64 finishing on (the
// default), a split-precision solve with a residual drop whose density residual has
// levelled off -- fallen 1000-fold from its first iteration, then no new minimum for
// stall_steps iterations: its increments are down to the FP32 rounding of the flux
// arithmetic -- continues in plain FP64 from its
// current state, keeping its iteration count, time and first-iteration residual, so
// that it retires at the residual drop like an FP64 solve.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>

#include "solver_impl.hpp"

using namespace ebb;

namespace {

struct Request {
    int64_t id = 0;
    std::unique_ptr<ebb_mesh> mesh;
    ebb_config cfg;
    int64_t max_steps = 0;
    double resid_drop = 0;
    double submit_s = 0, admit_s = -1;
    int32_t precision = EBB_PREC_SPLIT;
    int32_t escalated = 0;  // 1: re-solved in FP64 after a split-precision error; 2: finished in FP64
    int64_t split_iterations = 0;
    // a continuation starts from this state (reference cell order) and time-loop state
    std::vector<double> resume_q;
    ebb_instance_status resume{};
    bool resuming = false;
    InstLayout L;
    int status = EBB_OK;
    std::string err;
    size_t bytes = 0;  // device bytes of an arena holding this request alone
};

struct ArenaRun {
    ebb_solver *s = nullptr;
    std::vector<std::shared_ptr<Request>> reqs;
    std::vector<char> retired;
    std::vector<int64_t> iter_seen, cells;
    std::vector<ebb_instance_status> st;  // as of the last harvest
    size_t bytes = 0;
    int left = 0;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    int64_t steps_queued = 0;
    double ms_per_step = 0;  // measured on this arena's stream, smoothed
};

double now_s(std::chrono::steady_clock::time_point t0)
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

bool same_group(const ebb_config &a, const ebb_config &b)
{
    return a.flux == b.flux && a.integrator == b.integrator && a.limited == b.limited && a.order == b.order &&
           a.viscosity == b.viscosity && a.local_timestep == b.local_timestep &&
           a.multistage_limiting == b.multistage_limiting && (a.lp_thresh > 0) == (b.lp_thresh > 0) &&
           (!(a.lp_thresh > 0) || a.lp_thresh == b.lp_thresh) && a.mms == b.mms && a.pr == b.pr && a.r_gas == b.r_gas;
}

}  // namespace

struct ebb_server {
    ebb_server_options opt;
    std::chrono::steady_clock::time_point t0;
    int device = 0;
    std::mutex mu;
    std::condition_variable cv;
    bool stopping = false;
    std::deque<std::shared_ptr<Request>> to_build;     // guarded by mu
    std::vector<std::shared_ptr<Request>> built;       // guarded by mu
    int building = 0;                                  // guarded by mu
    int64_t next_id = 0, submitted = 0;                // guarded by mu
    std::vector<std::thread> workers;
    // scheduling thread only
    std::vector<std::shared_ptr<Request>> waiting;
    std::vector<std::unique_ptr<ArenaRun>> arenas;
    std::deque<ebb_request_result> results;
    std::map<int64_t, std::vector<double>> states;
    uint64_t bytes_in_use = 0, bytes_peak = 0;
    int64_t finished = 0, cell_updates = 0, escalations = 0;
};

namespace {

void worker(ebb_server *sv)
{
    for (;;) {
        std::shared_ptr<Request> r;
        {
            std::unique_lock<std::mutex> lk(sv->mu);
            sv->cv.wait(lk, [&] { return sv->stopping || !sv->to_build.empty(); });
            if (sv->stopping) return;
            r = sv->to_build.front();
            sv->to_build.pop_front();
            sv->building++;
        }
        r->status = build_instance(r->mesh.get(), &r->cfg, r->L, r->err);
        const bool finishing = sv->opt.finish_fp64 && r->resid_drop > 0 && sv->opt.stall_steps > 0;
        // the mesh is kept only while an FP64 re-solve or continuation may still need it
        if (!((sv->opt.escalate || finishing) && r->precision == EBB_PREC_SPLIT)) r->mesh.reset();
        if (r->status == EBB_OK) {
            r->L.st0.max_steps = r->max_steps;
            r->L.st0.stop_drop = r->resid_drop;
            if (finishing && r->precision == EBB_PREC_SPLIT) r->L.st0.stall_steps = sv->opt.stall_steps;
            if (r->resuming) {
                // continue the stopped split solve: its state (local device order) and
                // the time-loop quantities the stop conditions and the records use
                DState &h = r->L.st0;
                for (int64_t i = 0; i < r->L.C; i++)
                    for (int c = 0; c < 4; c++) r->L.q[4 * i + c] = r->resume_q[4 * (size_t)r->L.perm[i] + c];
                h.t = r->resume.t;
                set_step(h, r->resume.dt);
                h.cfl = r->resume.cfl;
                h.cflf = (float)h.cfl;
                h.iter = r->resume.iterations;
                h.resid_first = r->resume.resid_first;
                h.done = !(h.t < h.t_end) || (h.max_steps > 0 && h.iter >= h.max_steps);
                r->resume_q.clear();
                r->resume_q.shrink_to_fit();
            }
            std::vector<InstLayout> one(1);
            one[0].C = r->L.C;  // sizes only
            one[0].G = r->L.G;
            one[0].Eint = r->L.Eint;
            one[0].maxJ = r->L.maxJ;
            one[0].cfg = r->L.cfg;
            one[0].force.resize(r->L.force.size());
            r->bytes = arena_bytes(one, r->precision);
        }
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->building--;
        sv->built.push_back(r);
    }
}

void finish(ebb_server *sv, Request &r, int status, const std::string &msg, const ebb_instance_status *st)
{
    ebb_request_result o;
    std::memset(&o, 0, sizeof o);
    o.id = r.id;
    o.status = status;
    o.err_index = -1;
    o.submit_s = r.submit_s;
    o.admit_s = r.admit_s;
    o.finish_s = now_s(sv->t0);
    o.n_cells = r.L.C;
    o.precision = r.precision;
    o.escalated = r.escalated;
    o.split_iterations = r.split_iterations;
    std::snprintf(o.msg, sizeof o.msg, "%s", msg.c_str());
    if (st) {
        o.err_index = st->err_index;
        o.iterations = st->iterations;
        o.t = st->t;
        o.drag = st->drag;
        o.lift = st->lift;
        for (int k = 0; k < 4; k++) o.resid[k] = st->resid[k];
        o.resid_first = st->resid_first;
        if (status != EBB_OK)
            o.done_reason = 0;
        else if (!(st->t < r.cfg.t_end))
            o.done_reason = 1;
        else if (r.max_steps > 0 && st->iterations >= r.max_steps)
            o.done_reason = 2;
        else
            o.done_reason = 3;
    }
    sv->results.push_back(o);
    sv->finished++;
}

int steps_for(const ebb_server *sv, const ArenaRun &a, const std::vector<ebb_instance_status> &st)
{
    // remaining iterations of the longest-running live instance with a step limit
    int64_t remain = 0;
    bool unbounded = false;
    for (size_t k = 0; k < a.reqs.size(); k++) {
        if (a.retired[k] || st[k].done) continue;
        if (a.reqs[k]->max_steps > 0)
            remain = std::max<int64_t>(remain, a.reqs[k]->max_steps - st[k].iterations);
        else
            unbounded = true;
    }
    int64_t n = a.ms_per_step > 0 ? (int64_t)(sv->opt.tick_ms / a.ms_per_step) : 64;
    n = std::max<int64_t>(16, std::min<int64_t>(n, 4096));
    n = (n + 15) / 16 * 16;
    if (!unbounded) n = std::min(n, remain);
    return (int)std::max<int64_t>(n, 0);
}

int enqueue(ArenaRun &a, int64_t n)
{
    if (n <= 0) {
        a.steps_queued = 0;
        return EBB_OK;
    }
    cudaEventRecord(a.ev[0], a.s->stream);
    int r = ebb_launch_steps(a.s, n);
    cudaEventRecord(a.ev[1], a.s->stream);
    a.steps_queued = n;
    return r;
}

void drop_arena(ebb_server *sv, size_t i)
{
    ArenaRun &a = *sv->arenas[i];
    if (a.ev[0]) cudaEventDestroy(a.ev[0]);
    if (a.ev[1]) cudaEventDestroy(a.ev[1]);
    ebb_solver_destroy(a.s);
    sv->bytes_in_use -= a.bytes;
    sv->arenas.erase(sv->arenas.begin() + i);
}

// wait for the arena's queued chunk, account and retire what has stopped
int harvest(ebb_server *sv, ArenaRun &a)
{
    int r = ebb_sync(a.s);
    if (r) return r;
    if (a.steps_queued > 0) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, a.ev[0], a.ev[1]) == cudaSuccess) {
            const double per = ms / (double)a.steps_queued;
            a.ms_per_step = a.ms_per_step > 0 ? 0.5 * (a.ms_per_step + per) : per;
        }
        a.steps_queued = 0;
    }
    const int n = (int)a.reqs.size();
    std::vector<ebb_instance_status> &st = a.st;
    if ((r = ebb_batch_status(a.s, 0, n, st.data()))) return r;
    for (int k = 0; k < n; k++) {
        if (a.retired[k]) continue;
        sv->cell_updates += a.cells[k] * (st[k].iterations - a.iter_seen[k]);
        a.iter_seen[k] = st[k].iterations;
        if (!st[k].done) continue;
        Request &rq = *a.reqs[k];
        if (rq.precision == EBB_PREC_SPLIT) rq.split_iterations = st[k].iterations;
        const bool stalled = st[k].status == EBB_OK && st[k].t < rq.cfg.t_end &&
                             !(rq.max_steps > 0 && st[k].iterations >= rq.max_steps) &&
                             !(rq.resid_drop > 0 && st[k].resid[0] <= rq.resid_drop * st[k].resid_first);
        if (stalled && sv->opt.finish_fp64 && rq.precision == EBB_PREC_SPLIT && rq.mesh) {
            // continue in the finishing form (plain FP64 or double-float) from the
            // current state (same id)
            auto next = std::make_shared<Request>();
            next->id = rq.id;
            next->mesh = std::move(rq.mesh);
            next->cfg = rq.cfg;
            next->max_steps = rq.max_steps;
            next->resid_drop = rq.resid_drop;
            next->submit_s = rq.submit_s;
            next->admit_s = rq.admit_s;
            next->precision = sv->opt.finish_precision;
            next->escalated = 2;
            next->split_iterations = st[k].iterations;
            next->resume = st[k];
            next->resuming = true;
            next->resume_q.resize(4 * (size_t)a.cells[k]);
            if ((r = ebb_batch_get_state(a.s, k, next->resume_q.data()))) return r;
            {
                std::lock_guard<std::mutex> lk(sv->mu);
                sv->to_build.push_back(next);
            }
            sv->cv.notify_one();
            a.retired[k] = 1;
            a.left--;
            continue;
        }
        if (st[k].status != EBB_OK && sv->opt.escalate && rq.precision == EBB_PREC_SPLIT && rq.mesh) {
            // solve it again in plain FP64, from the start
            auto again = std::make_shared<Request>();
            again->id = rq.id;
            again->mesh = std::move(rq.mesh);
            again->cfg = rq.cfg;
            again->max_steps = rq.max_steps;
            again->resid_drop = rq.resid_drop;
            again->submit_s = rq.submit_s;
            again->precision = EBB_PREC_FP64;
            again->escalated = 1;
            again->split_iterations = rq.split_iterations;
            {
                std::lock_guard<std::mutex> lk(sv->mu);
                sv->to_build.push_back(again);
            }
            sv->cv.notify_one();
            sv->escalations++;
            a.retired[k] = 1;
            a.left--;
            continue;
        }
        rq.mesh.reset();
        std::vector<double> q(4 * (size_t)a.cells[k]);
        if ((r = ebb_batch_get_state(a.s, k, q.data()))) return r;
        sv->states[a.reqs[k]->id] = std::move(q);
        finish(sv, *a.reqs[k], st[k].status, st[k].status ? "stopped by an error" : "", &st[k]);
        a.retired[k] = 1;
        a.left--;
    }
    return EBB_OK;
}

int admit(ebb_server *sv)
{
    const double now = now_s(sv->t0);
    while ((int)sv->arenas.size() < sv->opt.max_arenas && !sv->waiting.empty()) {
        std::shared_ptr<Request> head = sv->waiting.front();
        if (head->bytes > sv->opt.hbm_budget) {
            sv->waiting.erase(sv->waiting.begin());
            finish(sv, *head, EBB_ERR_LIMIT, "solve larger than the device budget", nullptr);
            continue;
        }
        std::vector<size_t> pick{0};
        int64_t cells = head->L.C;
        uint64_t est = head->bytes;
        const uint64_t room = sv->opt.hbm_budget - sv->bytes_in_use;
        for (size_t i = 1; i < sv->waiting.size() && (int)pick.size() < sv->opt.max_batch; i++) {
            const Request &r = *sv->waiting[i];
            const double ratio = (double)std::max(r.L.C, head->L.C) / (double)std::max<int64_t>(1, std::min(r.L.C, head->L.C));
            if (!same_group(r.cfg, head->cfg) || r.precision != head->precision || ratio > sv->opt.size_ratio)
                continue;
            if (cells + r.L.C > sv->opt.arena_cells || est + r.bytes > room) continue;
            pick.push_back(i);
            cells += r.L.C;
            est += r.bytes;
        }
        if (est > room) break;  // the oldest request waits for memory
        std::vector<InstLayout> Ls;
        std::vector<std::shared_ptr<Request>> group;
        for (size_t i : pick) {
            group.push_back(sv->waiting[i]);
            Ls.push_back(std::move(sv->waiting[i]->L));
        }
        for (size_t j = pick.size(); j-- > 0;) sv->waiting.erase(sv->waiting.begin() + pick[j]);
        auto a = std::make_unique<ArenaRun>();
        a->s = new ebb_solver();
        std::string e;
        const uint64_t exact = arena_bytes(Ls, head->precision);
        std::vector<int64_t> cl(Ls.size());
        for (size_t k = 0; k < Ls.size(); k++) cl[k] = Ls[k].C;
        int r = (exact > room) ? EBB_ERR_OOM : assemble(a->s, Ls, head->precision, e);
        for (size_t k = 0; k < group.size(); k++) {
            group[k]->L.C = cl[k];  // keep the size for the result record
            if (group[k]->admit_s < 0) group[k]->admit_s = now;  // a continuation keeps its first admission
        }
        if (r) {
            ebb_solver_destroy(a->s);
            for (auto &g : group) finish(sv, *g, r, e.empty() ? "arena could not be created" : e, nullptr);
            continue;
        }
        a->reqs = group;
        a->retired.assign(group.size(), 0);
        a->iter_seen.assign(group.size(), 0);
        for (size_t k = 0; k < group.size(); k++)
            if (group[k]->resuming) a->iter_seen[k] = group[k]->resume.iterations;
        a->cells = cl;
        a->left = (int)group.size();
        a->bytes = a->s->dbytes;
        cudaEventCreate(&a->ev[0]);
        cudaEventCreate(&a->ev[1]);
        sv->bytes_in_use += a->bytes;
        sv->bytes_peak = std::max(sv->bytes_peak, sv->bytes_in_use);
        a->st.resize(group.size());
        std::memset(a->st.data(), 0, a->st.size() * sizeof(a->st[0]));
        if ((r = enqueue(*a, steps_for(sv, *a, a->st)))) return r;
        sv->arenas.push_back(std::move(a));
    }
    return EBB_OK;
}

}  // namespace

extern "C" {

void ebb_server_options_defaults(ebb_server_options *o)
{
    if (!o) return;
    std::memset(o, 0, sizeof *o);
    o->precision = EBB_PREC_SPLIT;
    o->max_arenas = 32;
    o->max_batch = 512;
    o->build_threads = 4;
    o->tick_ms = 25.0;
    o->size_ratio = 4.0;
    o->arena_cells = 8 << 20;
    o->hbm_budget = 150000000000ull;
    o->finish_fp64 = 1;
    o->stall_steps = 1000;
    o->finish_precision = EBB_PREC_FP64;
}

int ebb_server_create(const ebb_server_options *o, ebb_server **out, char *err, size_t err_len)
{
    if (!out) return EBB_ERR_ARG;
    *out = nullptr;
    int nd = 0;
    if (ebb_device_count(&nd) != EBB_OK) {
        set_err(err, err_len, "no CUDA device available");
        return EBB_ERR_NO_DEVICE;
    }
    auto *sv = new ebb_server();
    if (o)
        sv->opt = *o;
    else
        ebb_server_options_defaults(&sv->opt);
    ebb_server_options &p = sv->opt;
    if ((p.precision != EBB_PREC_FP64 && p.precision != EBB_PREC_SPLIT && p.precision != EBB_PREC_DF) ||
        (p.finish_precision != EBB_PREC_FP64 && p.finish_precision != EBB_PREC_DF) || p.max_arenas <= 0 || p.max_batch <= 0 ||
        p.build_threads <= 0 || !(p.tick_ms > 0) || !(p.size_ratio >= 1) || p.arena_cells <= 0) {
        delete sv;
        set_err(err, err_len, "invalid server options");
        return EBB_ERR_ARG;
    }
    cudaGetDevice(&sv->device);
    sv->t0 = std::chrono::steady_clock::now();
    for (int k = 0; k < p.build_threads; k++) sv->workers.emplace_back(worker, sv);
    *out = sv;
    return EBB_OK;
}

int ebb_server_submit(ebb_server *sv, const ebb_mesh *mesh, const ebb_config *cfg, int64_t max_steps,
                      double resid_drop, int64_t *id)
{
    if (!sv || !mesh || !cfg) return EBB_ERR_ARG;
    auto r = std::make_shared<Request>();
    r->mesh = std::make_unique<ebb_mesh>(*mesh);
    r->cfg = *cfg;
    r->max_steps = max_steps;
    r->resid_drop = resid_drop;
    r->precision = sv->opt.precision;
    r->submit_s = now_s(sv->t0);
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        r->id = sv->next_id++;
        sv->submitted++;
        sv->to_build.push_back(r);
    }
    sv->cv.notify_one();
    if (id) *id = r->id;
    return EBB_OK;
}

int ebb_server_tick(ebb_server *sv, int32_t *n_active, int32_t *n_waiting)
{
    if (!sv) return EBB_ERR_ARG;
    cudaSetDevice(sv->device);
    int r;
    for (size_t i = 0; i < sv->arenas.size(); i++)
        if ((r = harvest(sv, *sv->arenas[i]))) return r;
    for (size_t i = sv->arenas.size(); i-- > 0;)
        if (sv->arenas[i]->left == 0) drop_arena(sv, i);
    int building;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        std::sort(sv->built.begin(), sv->built.end(), [](const auto &a, const auto &b) { return a->id < b->id; });
        for (auto &b : sv->built) {
            if (b->status)
                finish(sv, *b, b->status, b->err, nullptr);
            else
                sv->waiting.push_back(b);
        }
        sv->built.clear();
        building = sv->building + (int)sv->to_build.size();
    }
    std::sort(sv->waiting.begin(), sv->waiting.end(), [](const auto &a, const auto &b) { return a->id < b->id; });
    for (auto &a : sv->arenas)
        if ((r = enqueue(*a, steps_for(sv, *a, a->st)))) return r;
    if ((r = admit(sv))) return r;
    if (n_active) *n_active = (int32_t)sv->arenas.size();
    if (n_waiting) *n_waiting = (int32_t)sv->waiting.size() + building;
    return EBB_OK;
}

int ebb_server_results(ebb_server *sv, ebb_request_result *out, int32_t cap, int32_t *n)
{
    if (!sv || !n || cap < 0 || (cap && !out)) return EBB_ERR_ARG;
    int32_t k = 0;
    while (k < cap && !sv->results.empty()) {
        out[k++] = sv->results.front();
        sv->results.pop_front();
    }
    *n = k;
    return EBB_OK;
}

int ebb_server_take_state(ebb_server *sv, int64_t id, double *q)
{
    if (!sv || !q) return EBB_ERR_ARG;
    auto it = sv->states.find(id);
    if (it == sv->states.end()) return EBB_ERR_ARG;
    std::memcpy(q, it->second.data(), it->second.size() * sizeof(double));
    sv->states.erase(it);
    return EBB_OK;
}

int ebb_server_stats_get(ebb_server *sv, ebb_server_stats *st)
{
    if (!sv || !st) return EBB_ERR_ARG;
    std::memset(st, 0, sizeof *st);
    st->bytes_in_use = sv->bytes_in_use;
    st->bytes_peak = sv->bytes_peak;
    st->arenas = (int32_t)sv->arenas.size();
    st->waiting = (int32_t)sv->waiting.size();
    std::lock_guard<std::mutex> lk(sv->mu);
    st->building = sv->building + (int32_t)sv->to_build.size() + (int32_t)sv->built.size();
    st->submitted = sv->submitted;
    st->finished = sv->finished;
    st->cell_updates = sv->cell_updates;
    st->escalations = sv->escalations;
    return EBB_OK;
}

void ebb_server_destroy(ebb_server *sv)
{
    if (!sv) return;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stopping = true;
    }
    sv->cv.notify_all();
    for (auto &t : sv->workers) t.join();
    cudaSetDevice(sv->device);
    while (!sv->arenas.empty()) drop_arena(sv, sv->arenas.size() - 1);
    delete sv;
}

}  // extern "C"

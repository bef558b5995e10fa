// xtg_server.cpp — request server with admission by HBM budget and
// continuous batching (no counterpart in xtensor, which evaluates one
// expression at a time on the calling thread).
//
// Threads: callers submit (never blocking on the GPU); one scheduler thread
// admits and dispatches; a completion thread polls CUDA events and completes
// requests.
//   admission — in arrival order, a pending request is admitted when the
//     in-flight count is below the limit and its cost (declared workspace +
//     the split-reduction scratch its plan may take) fits the remaining HBM
//     budget; a request that waited longer than the aging limit blocks later
//     ones from overtaking it.  Requests larger than the whole budget are
//     rejected at submit.
//   dispatch — admitted small requests (at most batch_max_elems elements,
//     2-D, elementwise or last-axis reductions) with the same tree shape and
//     immediates form a group launched as ONE batched kernel; everything else
//     goes out individually.  A batchable request waits up to
//     "server.batch_window_us" (default 200) for others of its shape while
//     other work is on the device; a group leaves at once when it reaches
//     "server.batch_max_group" (default 64) or the device has nothing else.  The scheduler hands each wave's groups and
//     requests round-robin to dispatch threads (option
//     "server.dispatch_threads", default 1), each owning a share of the
//     stream pool, so that several cores can pay the host cost of launching
//     (planning or plan-cache replay, kernel launches); the work overlaps on
//     the device across the streams.
//   completion — an event recorded after each unit; the completion thread
//     polls the events, marks the unit's requests done with a host
//     timestamp and releases their budget; the scheduler frees batch work
//     lists once their units completed.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "xtg_plan.h"

using namespace xtgh;
using Clock = std::chrono::steady_clock;

namespace {

struct Req {
    uint64_t id = 0;
    xtg_request r;
    int64_t cost = 0;
    int64_t elems = 0;
    bool batchable = false;
    std::string sig;
    Clock::time_point t_submit, t_dispatch, t_done;
    int status = XTG_OK;
    bool finished = false;
    bool dispatched = false;
    bool batched = false;
};

struct Unit;

// Work handed to one dispatch thread: whole batch groups and single requests.
struct Work {
    std::vector<std::vector<Req*>> groups;
    std::vector<Req*> singles;
};
struct Disp {
    std::thread th;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Work> q;
    std::vector<cudaStream_t> streams;  // this thread's share of the pool
    size_t next_stream = 0;
    bool stop = false;
};
// Completion by events: a unit's event is recorded on its stream after its
// launches; the completion thread polls the recorded events and completes
// the units whose events have passed.  (A host callback per unit would stop
// its stream until CUDA's single callback thread ran it.)
struct Completer {
    std::thread th;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<std::pair<cudaEvent_t, Unit*>> q;
    std::vector<cudaEvent_t> spare;
    bool stop = false;
};

}  // namespace

struct xtg_server {
    xtg_server_config cfg;
    std::vector<cudaStream_t> streams;
    std::vector<std::unique_ptr<Disp>> disp;
    size_t next_disp = 0;
    std::set<std::string> warmed;  // batchable shapes whose batch kernel build has started
    std::mutex mu;
    std::condition_variable cv_sched, cv_done;
    std::deque<Req*> pending;
    std::unordered_map<uint64_t, std::unique_ptr<Req>> reqs;
    std::vector<Unit*> finished_units;
    Completer comp;
    uint64_t next_id = 1;
    uint64_t events = 0;  // submits + completions + cancels: admission retries only when it changes
    int64_t budget = 0, reserved = 0, inflight = 0;
    bool stop = false;
    std::thread sched;
    xtg_server_stats st{};
    std::vector<double> lat;
};

namespace {

struct Unit {
    xtg_server* srv;
    std::vector<Req*> reqs;
    xtg_batch* batch = nullptr;
};

void CUDART_CB on_unit_done(void* p) {
    Unit* u = (Unit*)p;
    xtg_server* s = u->srv;
    const auto now = Clock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    for (Req* r : u->reqs) {
        r->t_done = now;
        r->finished = true;
        s->inflight--;
        s->reserved -= r->cost;
        s->st.completed++;
        s->lat.push_back(std::chrono::duration<double, std::milli>(now - r->t_submit).count());
    }
    s->finished_units.push_back(u);
    s->events++;
    s->cv_done.notify_all();
    s->cv_sched.notify_all();
}

// Completion of a unit once the stream reaches this point (inline in dry-run
// mode, where nothing runs on a device): an event the completion thread
// polls, or with option "server.host_callbacks" a stream host callback.
void complete_after(cudaStream_t st, Unit* u) {
    if (dry_run()) {
        on_unit_done(u);
        return;
    }
    xtg_server* s = u->srv;
    if (opt("server.host_callbacks", 0)) {
        if (cudaLaunchHostFunc(st, on_unit_done, u) != cudaSuccess) {
            cudaGetLastError();
            cudaStreamSynchronize(st);
            on_unit_done(u);
        }
        return;
    }
    cudaEvent_t e = nullptr;
    {
        std::lock_guard<std::mutex> lk(s->comp.mu);
        if (!s->comp.spare.empty()) {
            e = s->comp.spare.back();
            s->comp.spare.pop_back();
        }
    }
    if ((!e && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) ||
        cudaEventRecord(e, st) != cudaSuccess) {
        cudaGetLastError();
        cudaStreamSynchronize(st);
        if (e) cudaEventDestroy(e);
        on_unit_done(u);
        return;
    }
    {
        std::lock_guard<std::mutex> lk(s->comp.mu);
        s->comp.q.emplace_back(e, u);
    }
    s->comp.cv.notify_one();
}

// The completion thread: polls the pending units' events (in any order: the
// streams run independently), completes those that passed, and naps a few
// microseconds when none did.
void completer(xtg_server* s) {
    ensure_device(nullptr);
    Completer& C = s->comp;
    std::vector<std::pair<cudaEvent_t, Unit*>> mine;
    for (;;) {
        {
            std::unique_lock<std::mutex> lk(C.mu);
            if (mine.empty()) C.cv.wait(lk, [&] { return C.stop || !C.q.empty(); });
            while (!C.q.empty()) {
                mine.push_back(C.q.front());
                C.q.pop_front();
            }
            if (mine.empty() && C.stop) break;
        }
        bool progress = false;
        std::vector<cudaEvent_t> passed;
        for (size_t i = 0; i < mine.size();) {
            const cudaError_t r = cudaEventQuery(mine[i].first);
            if (r == cudaErrorNotReady) {
                ++i;
                continue;
            }
            if (r != cudaSuccess) cudaGetLastError();  // completed with an error: the unit still ends
            on_unit_done(mine[i].second);
            passed.push_back(mine[i].first);
            mine[i] = mine.back();
            mine.pop_back();
            progress = true;
        }
        if (!passed.empty()) {
            std::lock_guard<std::mutex> lk(C.mu);
            C.spare.insert(C.spare.end(), passed.begin(), passed.end());
        }
        if (!progress && !mine.empty()) std::this_thread::sleep_for(std::chrono::microseconds(5));
    }
}

int64_t elems_of(const xtg_expr& e, int64_t* shape_rank = nullptr) {
    int32_t rank = 0;
    int64_t sh[XTG_MAX_RANK];
    if (xtg_broadcast_shape(&e, &rank, sh) != XTG_OK) return -1;
    int64_t n = 1;
    for (int d = 0; d < rank; ++d) n *= sh[d];
    if (shape_rank) *shape_rank = rank;
    return n;
}

std::string signature(const xtg_request& r) {
    std::string s = std::to_string(r.kind) + ":" + std::to_string(r.out.dtype) + ":";
    if (r.kind == XTG_REQ_REDUCE)
        s += std::to_string(r.rd.op) + "," + std::to_string(r.rd.acc_dtype) + "," + std::to_string(r.rd.precision) + "," +
             std::to_string(r.rd.has_initial) + "," + std::to_string(r.rd.initial.i) + ":";
    for (int i = 0; i < r.expr.n_nodes; ++i) {
        const xtg_node& n = r.expr.nodes[i];
        s += std::to_string(n.op) + "/" + std::to_string(n.dtype) + "/" + std::to_string(n.arg) + "/" +
             std::to_string(n.aux) + "/" + std::to_string(n.imm.u) + ";";
    }
    for (int i = 0; i < r.expr.n_leaves; ++i)
        s += "L" + std::to_string(r.expr.leaves[i].dtype) + "r" + std::to_string(r.expr.leaves[i].rank);
    return s;
}

void complete_failed(xtg_server* s, const std::vector<Req*>& rs, int status) {
    const auto now = Clock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    for (Req* r : rs) {
        r->status = status;
        r->t_done = now;
        r->finished = true;
        s->inflight--;
        s->reserved -= r->cost;
        s->st.failed++;
    }
    s->events++;
    s->cv_done.notify_all();
    s->cv_sched.notify_all();
}

int dispatch_one(Req* r, cudaStream_t st) {
    const int64_t every = opt("server.inject_fail_every", 0);
    if (every > 0 && (int64_t)(r->id % (uint64_t)every) == 0) {
        fail(XTG_ERR_CUDA, "injected dispatch failure");
        return XTG_ERR_CUDA;
    }
    switch (r->r.kind) {
        case XTG_REQ_ASSIGN: return xtg_assign(&r->r.expr, &r->r.out, st);
        case XTG_REQ_REDUCE: return xtg_reduce(&r->r.expr, &r->r.rd, &r->r.out, st);
        case XTG_REQ_ARGREDUCE:
            return xtg_argreduce(&r->r.expr, r->r.arg_op, r->r.has_axis, r->r.axis, &r->r.out, st);
    }
    return XTG_ERR_INVALID;
}

// Launches one dispatcher's share of a wave on its streams: each group as one
// batched kernel (or, while its batch kernel is not built yet, one request
// at a time), singles round-robin over the streams, and one completion
// callback per stream used.
void dispatch(xtg_server* s, Disp* d, Work& w) {
    std::vector<Req*> singles = std::move(w.singles);
    for (auto& grp : w.groups) {
        cudaStream_t st = d->streams[d->next_stream++ % d->streams.size()];
        const auto now = Clock::now();
        Req* f = grp[0];
        xtg_batch* b = nullptr;
        int rc = xtg_batch_create(&f->r.expr, f->r.kind == XTG_REQ_REDUCE ? &f->r.rd : nullptr, &b);
        for (size_t i = 0; rc == XTG_OK && i < grp.size(); ++i)
            rc = xtg_batch_add(b, grp[i]->r.expr.leaves, grp[i]->r.expr.n_leaves, &grp[i]->r.out);
        if (rc == XTG_OK) {
            // never compile on a dispatch thread: a batch kernel that is not
            // loaded yet is built in the background while this group runs
            // one request at a time
            std::string kname;
            rc = batch_planned_kernel(b, &kname);
            if (rc == XTG_OK && !kernel_ready(kname) && !opt("server.compile_inline", 0)) {
                compile_async(kname, 256);
                rc = XTG_ERR_UNSUPPORTED;
            }
        }
        if (rc == XTG_OK) rc = xtg_batch_build(b, 0, st);
        if (rc == XTG_OK) rc = xtg_batch_run(b, st);
        if (rc != XTG_OK) {
            if (b) xtg_batch_destroy(b);
            // fall back to individual dispatch for this group
            singles.insert(singles.end(), grp.begin(), grp.end());
            continue;
        }
        Unit* u = new Unit{s, grp, b};
        {
            std::lock_guard<std::mutex> lk(s->mu);
            for (Req* r : grp) {
                r->t_dispatch = now;
                r->dispatched = true;
                r->batched = true;
            }
            s->st.batch_launches++;
            s->st.batched_requests += (int64_t)grp.size();
        }
        complete_after(st, u);
    }
    // individual requests: round-robin over the streams, one completion
    // callback per stream for this share of the wave
    std::vector<Unit*> per_stream(d->streams.size(), nullptr);
    for (Req* r : singles) {
        const size_t si = d->next_stream++ % d->streams.size();
        cudaStream_t st = d->streams[si];
        {
            std::lock_guard<std::mutex> lk(s->mu);
            r->t_dispatch = Clock::now();
            r->dispatched = true;
        }
        int rc = dispatch_one(r, st);
        if (rc != XTG_OK) {
            complete_failed(s, {r}, rc);
            continue;
        }
        if (!per_stream[si]) per_stream[si] = new Unit{s, {}, nullptr};
        per_stream[si]->reqs.push_back(r);
    }
    for (size_t si = 0; si < per_stream.size(); ++si)
        if (per_stream[si]) complete_after(d->streams[si], per_stream[si]);
}

void dispatcher(xtg_server* s, Disp* d) {
    ensure_device(nullptr);
    for (;;) {
        std::deque<Work> mine;
        {
            std::unique_lock<std::mutex> lk(d->mu);
            d->cv.wait(lk, [&] { return d->stop || !d->q.empty(); });
            if (d->q.empty() && d->stop) break;
            mine.swap(d->q);
        }
        const auto t0 = Clock::now();
        for (Work& w : mine) dispatch(s, d, w);
        const double ms = std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
        std::lock_guard<std::mutex> lk(s->mu);
        s->st.dispatch_ms += ms;
    }
}

// Splits an admitted wave: batchable requests grouped by signature (groups
// below batch_min_group go out singly), then whole groups and singles
// round-robin over the dispatch threads.
void hand_out(xtg_server* s, std::vector<Req*>& admitted) {
    std::map<std::string, std::vector<Req*>> groups;
    std::vector<Req*> singles;
    for (Req* r : admitted) {
        if (r->batchable) groups[r->sig].push_back(r);
        else singles.push_back(r);
    }
    // the first request of a batchable shape starts building its batch
    // kernel in the background, so that groups of that shape arriving later
    // find it loaded instead of running one request at a time meanwhile
    for (auto& kv : groups) {
        if (!s->warmed.insert(kv.first).second) continue;
        Req* f = kv.second[0];
        xtg_batch* b = nullptr;
        if (xtg_batch_create(&f->r.expr, f->r.kind == XTG_REQ_REDUCE ? &f->r.rd : nullptr, &b) == XTG_OK &&
            xtg_batch_add(b, f->r.expr.leaves, f->r.expr.n_leaves, &f->r.out) == XTG_OK) {
            std::string kname;
            if (batch_planned_kernel(b, &kname) == XTG_OK && !kernel_ready(kname)) compile_async(kname, 256);
        }
        if (b) xtg_batch_destroy(b);
        clear_error();
    }
    const size_t K = s->disp.size();
    std::vector<Work> work(K);
    for (auto& kv : groups) {
        if ((int)kv.second.size() < s->cfg.batch_min_group) {
            singles.insert(singles.end(), kv.second.begin(), kv.second.end());
            continue;
        }
        work[s->next_disp++ % K].groups.push_back(std::move(kv.second));
    }
    for (Req* r : singles) work[s->next_disp++ % K].singles.push_back(r);
    for (size_t i = 0; i < K; ++i) {
        if (work[i].groups.empty() && work[i].singles.empty()) continue;
        Disp* d = s->disp[i].get();
        {
            std::lock_guard<std::mutex> lk(d->mu);
            d->q.push_back(std::move(work[i]));
        }
        d->cv.notify_one();
    }
}

void scheduler(xtg_server* s) {
    ensure_device(nullptr);
    const double aging_ms = (double)opt("server.aging_ms", 50);
    // batchable requests of one shape wait up to this long for others of the
    // same shape (continuous batching's collect window); a group leaves as
    // soon as it is full or nothing else is on the device
    const auto window = std::chrono::microseconds(opt("server.batch_window_us", 200));
    const size_t max_group = (size_t)std::max<int64_t>(2, opt("server.batch_max_group", 64));
    std::map<std::string, std::vector<Req*>> forming;
    size_t n_forming = 0;
    uint64_t seen = ~0ull;
    for (;;) {
        std::vector<Req*> admitted;
        std::vector<Unit*> done;
        bool idle = false;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            // wake for work to clean up, for a change that may let a pending
            // request in, to finish once stopping has drained the device, or
            // when the oldest forming group's window closes
            auto ready = [&] {
                return !s->finished_units.empty() || (!s->pending.empty() && s->events != seen) ||
                       (s->stop && s->inflight == (int64_t)n_forming);
            };
            if (n_forming == 0) {
                s->cv_sched.wait(lk, ready);
            } else {
                auto oldest = Clock::time_point::max();
                for (auto& kv : forming) oldest = std::min(oldest, kv.second[0]->t_submit);
                s->cv_sched.wait_until(lk, oldest + window, ready);
            }
            seen = s->events;
            done.swap(s->finished_units);
            if (s->stop && s->pending.empty() && s->inflight == 0 && done.empty()) break;
            const auto now = Clock::now();
            // option "server.paused": hold admissions (tests of queueing, cancel, timeouts)
            const bool paused = opt("server.paused", 0) != 0;
            for (auto it = s->pending.begin(); !paused && it != s->pending.end();) {
                Req* r = *it;
                if (s->inflight >= s->cfg.max_inflight) break;
                if (s->reserved + r->cost > s->budget) {
                    const double waited = std::chrono::duration<double, std::milli>(now - r->t_submit).count();
                    if (waited > aging_ms) break;  // do not let later requests starve this one
                    ++it;
                    continue;
                }
                s->reserved += r->cost;
                s->inflight++;
                admitted.push_back(r);
                it = s->pending.erase(it);
            }
            if (!admitted.empty()) s->st.waves++;
            // nothing dispatched is still running: forming groups need not wait
            idle = s->inflight - (int64_t)(n_forming + admitted.size()) <= 0 || s->stop;
        }
        for (Unit* u : done) {
            if (u->batch) xtg_batch_destroy(u->batch);
            delete u;
        }
        // batchable requests join their shape's forming group; the rest go out now
        std::vector<Req*> now_out;
        for (Req* r : admitted) {
            if (r->batchable && window.count() > 0) {
                forming[r->sig].push_back(r);
                ++n_forming;
            } else {
                now_out.push_back(r);
            }
        }
        const auto now = Clock::now();
        for (auto it = forming.begin(); it != forming.end();) {
            if (idle || it->second.size() >= max_group || now - it->second[0]->t_submit >= window) {
                n_forming -= it->second.size();
                now_out.insert(now_out.end(), it->second.begin(), it->second.end());
                it = forming.erase(it);
            } else {
                ++it;
            }
        }
        if (!now_out.empty()) hand_out(s, now_out);
    }
}

}  // namespace

extern "C" {

xtg_status xtg_server_create(const xtg_server_config* cfg, xtg_server** out) {
    if (!out) return fail(XTG_ERR_INVALID, "null output");
    XTG_TRY(ensure_device(nullptr));
    std::unique_ptr<xtg_server> s(new xtg_server());
    xtg_server_config c{};
    if (cfg) c = *cfg;
    if (c.streams <= 0) c.streams = 8;
    if (c.max_inflight <= 0) c.max_inflight = 256;
    if (c.batch_max_elems <= 0) c.batch_max_elems = 1 << 20;
    if (c.batch_min_group <= 0) c.batch_min_group = 4;
    s->cfg = c;
    if (c.hbm_budget_bytes > 0) {
        s->budget = c.hbm_budget_bytes;
    } else if (dry_run()) {
        s->budget = (int64_t)1 << 36;
    } else {
        size_t f = 0, t = 0;
        XTG_CUDA(cudaMemGetInfo(&f, &t));
        s->budget = (int64_t)(f * 0.9);
    }
    for (int i = 0; i < c.streams; ++i) {
        cudaStream_t st = nullptr;
        if (!dry_run()) XTG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        s->streams.push_back(st);
    }
    s->st.hbm_budget = s->budget;
    // dispatch threads, each with every K-th stream of the pool
    const int K = (int)std::max<int64_t>(1, std::min<int64_t>(opt("server.dispatch_threads", 1), c.streams));
    for (int i = 0; i < K; ++i) {
        std::unique_ptr<Disp> d(new Disp());
        for (int j = i; j < c.streams; j += K) d->streams.push_back(s->streams[(size_t)j]);
        s->disp.push_back(std::move(d));
    }
    xtg_server* raw = s.release();
    for (auto& d : raw->disp) d->th = std::thread(dispatcher, raw, d.get());
    raw->comp.th = std::thread(completer, raw);
    raw->sched = std::thread(scheduler, raw);
    *out = raw;
    return XTG_OK;
}

xtg_status xtg_server_submit(xtg_server* s, const xtg_request* r, uint64_t* id) {
    if (!s || !r) return fail(XTG_ERR_INVALID, "null argument");
    std::unique_ptr<Req> q(new Req());
    q->r = *r;
    q->t_submit = Clock::now();
    int64_t rank = 0;
    q->elems = elems_of(r->expr, &rank);
    if (q->elems < 0) return fail(XTG_ERR_INVALID, std::string("request expression: ") + xtg_last_error());
    int64_t scratch = 0;
    if (r->kind == XTG_REQ_REDUCE || r->kind == XTG_REQ_ARGREDUCE) {
        int64_t n_out = 1;
        for (int d = 0; d < r->out.rank; ++d) n_out *= r->out.shape[d];
        scratch = (opt("reduce.target_items", kReduceTargetItems) + n_out) * 32;
    }
    q->cost = std::max<int64_t>(0, r->workspace_bytes) + scratch;
    const bool last_axis = r->kind == XTG_REQ_REDUCE && r->rd.n_axes == 1 &&
                           (r->rd.axes[0] == -1 || r->rd.axes[0] == rank - 1) && r->rd.op != XTG_RED_VARIANCE &&
                           r->rd.op != XTG_RED_STDDEV && r->rd.op != XTG_RED_PROD;
    q->batchable = rank >= 1 && rank <= 2 && q->elems <= s->cfg.batch_max_elems &&
                   (r->kind == XTG_REQ_ASSIGN || last_axis);
    for (int i = 0; q->batchable && i < r->expr.n_nodes; ++i)
        if (r->expr.nodes[i].op >= XTG_OP_RSUM) q->batchable = false;
    if (q->batchable) q->sig = signature(*r);
    std::lock_guard<std::mutex> lk(s->mu);
    s->st.submitted++;
    if (q->cost > s->budget) {
        s->st.rejected++;
        return fail(XTG_ERR_REJECTED, "request needs more device memory than the server's HBM budget");
    }
    q->id = s->next_id++;
    if (id) *id = q->id;
    s->pending.push_back(q.get());
    s->reqs.emplace(q->id, std::move(q));
    s->events++;
    s->cv_sched.notify_one();
    return XTG_OK;
}

xtg_status xtg_server_wait(xtg_server* s, uint64_t id, int64_t timeout_ms, xtg_request_result* res) {
    if (!s) return fail(XTG_ERR_INVALID, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return fail(XTG_ERR_NOT_FOUND, "unknown request id");
    Req* r = it->second.get();
    auto pred = [&] { return r->finished; };
    if (timeout_ms < 0) s->cv_done.wait(lk, pred);
    else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred))
        return fail(XTG_ERR_TIMEOUT, "request not finished before the timeout");
    if (res) {
        res->status = r->status;
        res->batched = r->batched ? 1 : 0;
        res->queue_ms = r->dispatched ? std::chrono::duration<double, std::milli>(r->t_dispatch - r->t_submit).count() : 0;
        res->total_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    }
    const int status = r->status;
    s->reqs.erase(it);
    if (status != XTG_OK) return fail((xtg_status)status, "request failed");
    return XTG_OK;
}

xtg_status xtg_server_cancel(xtg_server* s, uint64_t id) {
    if (!s) return fail(XTG_ERR_INVALID, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    for (auto it = s->pending.begin(); it != s->pending.end(); ++it) {
        if ((*it)->id == id) {
            Req* r = *it;
            s->pending.erase(it);
            r->status = XTG_ERR_CANCELLED;
            r->finished = true;
            r->t_done = Clock::now();
            s->st.cancelled++;
            s->events++;
            s->cv_done.notify_all();
            s->cv_sched.notify_all();
            return XTG_OK;
        }
    }
    return fail(XTG_ERR_NOT_FOUND, "request is not pending (unknown, dispatched or finished)");
}

xtg_status xtg_server_drain(xtg_server* s, int64_t timeout_ms) {
    if (!s) return fail(XTG_ERR_INVALID, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto pred = [&] { return s->pending.empty() && s->inflight == 0; };
    if (timeout_ms < 0) s->cv_done.wait(lk, pred);
    else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred))
        return fail(XTG_ERR_TIMEOUT, "server did not drain before the timeout");
    return XTG_OK;
}

xtg_status xtg_server_get_stats(xtg_server* s, xtg_server_stats* out) {
    if (!s || !out) return fail(XTG_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->st;
    out->inflight = s->inflight;
    out->pending = (int64_t)s->pending.size();
    out->hbm_reserved = s->reserved;
    std::vector<double> l = s->lat;
    if (!l.empty()) {
        std::sort(l.begin(), l.end());
        auto q = [&](double f) { return l[std::min(l.size() - 1, (size_t)(f * (double)(l.size() - 1) + 0.5))]; };
        out->p50_ms = q(0.50);
        out->p99_ms = q(0.99);
        double sum = 0;
        for (double v : l) sum += v;
        out->mean_ms = sum / (double)l.size();
    }
    return XTG_OK;
}

xtg_status xtg_server_reset_stats(xtg_server* s) {
    if (!s) return fail(XTG_ERR_INVALID, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    const int64_t budget = s->st.hbm_budget;
    s->st = xtg_server_stats{};
    s->st.hbm_budget = budget;
    s->lat.clear();
    return XTG_OK;
}

xtg_status xtg_server_destroy(xtg_server* s) {
    if (!s) return XTG_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        // requests never dispatched are cancelled
        for (Req* r : s->pending) {
            r->status = XTG_ERR_CANCELLED;
            r->finished = true;
        }
        s->pending.clear();
        s->cv_sched.notify_all();
    }
    if (s->sched.joinable()) s->sched.join();
    // every admitted request has completed once the scheduler is done, so
    // the dispatch threads' queues are empty
    for (auto& d : s->disp) {
        {
            std::lock_guard<std::mutex> lk(d->mu);
            d->stop = true;
        }
        d->cv.notify_one();
    }
    for (auto& d : s->disp)
        if (d->th.joinable()) d->th.join();
    // every unit has completed: the completion thread has nothing left
    {
        std::lock_guard<std::mutex> lk(s->comp.mu);
        s->comp.stop = true;
    }
    s->comp.cv.notify_one();
    if (s->comp.th.joinable()) s->comp.th.join();
    for (cudaEvent_t e : s->comp.spare) cudaEventDestroy(e);
    wait_background_compiles(60000);  // batch kernels it started building
    for (cudaStream_t st : s->streams) {
        if (!st) continue;
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
    }
    for (Unit* u : s->finished_units) {
        if (u->batch) xtg_batch_destroy(u->batch);
        delete u;
    }
    delete s;
    return XTG_OK;
}

}  // extern "C"

// Serving loop: continuous batching of threading requests on one GPU (no counterpart in the
// reference, whose arg-sample threads one sequence at a time on the CPU).
//
// Requests arrive through awg_server_submit from any thread and wait in a FIFO queue. A
// worker thread forms batches ("waves") led by the oldest request — with it, queued requests
// of one precision, one set of wanted outputs and a like number of columns (within the
// options' length_ratio: a batch lasts as long as its longest chain), as many as fit the
// free device memory and max_batch — and
// launches each on an execution context of its own (streams, staging, a region of the
// server's device pool) and a thread of its own that plans, launches and completes it. Up
// to max_inflight waves are on the GPU at once, so requests that
// arrive while others run are admitted as soon as a context and memory free up and their
// kernels overlap on the device with the running ones. Device memory is one pool allocated
// at creation and handed out first-fit, so serving never calls cudaMalloc or cudaFree.
//
// A request submitted as resident keeps its device data (trees, sequences, forward tables,
// FP32 bin sums) after it completes: awg_server_resample draws new paths from it with only
// the traceback, as an MCMC loop re-sampling one thread does, until awg_server_release.
//
// Results do not depend on the company a request keeps: every kernel's sums have an order
// fixed by the problem alone (tested: each result alone equals the one in the mix).

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "argweaver_gb300.h"
#include "engine.h"
#include "plan.h"

namespace {

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Req {
    long long id = 0;
    std::vector<int> ptrees, ages, sprs, blocklens, mapping, rc0;
    std::vector<double> times, pops, uniforms;
    std::vector<char> seqs;
    awg_problem p{};
    awg_outputs out{};  // the caller's buffers; uniforms point at this request's copy
    int precision = AWG_FP32;
    bool resident = false;
    bool want_path = false, want_post = false;
    long long cells = 0, bytes = 0;
    double t_submit = 0, t_start = 0, t_done = 0;
    int status = 0;  // 0 waiting or running, 1 done, < 0 failed
    std::string err;
    int slot = -1;  // resident and done: the slot holding its data
};

// A batch slot: an execution context and the thread that plans, launches and completes the
// batches assigned to it, so host-side planning of different batches runs in parallel.
struct Slot {
    enum State { IDLE, ASSIGNED, HELD };
    awg::Ctx *ctx = nullptr;
    std::vector<Req *> reqs;
    size_t off = 0, bytes = 0;  // pool region
    State state = IDLE;         // ASSIGNED: a batch being launched or on the GPU; HELD: keeps
                                // a resident request's data
    std::thread th;
    std::condition_variable cv;
};

// First-fit allocator over the device pool, in 256-byte units.
struct Pool {
    size_t cap = 0;
    std::map<size_t, size_t> free_;  // offset -> bytes
    void init(size_t c) {
        cap = c;
        free_.clear();
        free_[0] = c;
    }
    bool alloc(size_t bytes, size_t &off) {
        bytes = (bytes + 255) & ~(size_t)255;
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                off = it->first;
                const size_t rest = it->second - bytes;
                free_.erase(it);
                if (rest) free_[off + bytes] = rest;
                return true;
            }
        }
        return false;
    }
    void release(size_t off, size_t bytes) {
        bytes = (bytes + 255) & ~(size_t)255;
        auto it = free_.emplace(off, bytes).first;
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
    size_t largest() const {
        size_t m = 0;
        for (auto &kv : free_) m = std::max(m, kv.second);
        return m;
    }
};

}  // namespace

struct awg_server {
    awg_server_options opt{};
    char *pool_dev = nullptr;
    Pool pool;
    std::vector<std::unique_ptr<Slot>> slots;
    bool stop_slots = false;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Req *> queue;
    std::unordered_map<long long, std::unique_ptr<Req>> reqs;
    long long next_id = 1;
    bool stop = false;
    std::thread worker;
    // statistics
    std::vector<double> lat_ms, queue_ms, service_ms;  // per completed request
    long long submitted = 0, completed = 0, failed = 0, cells_done = 0;
    double t_first = -1.0, t_last = 0.0;
    int inflight = 0, inflight_max = 0;
    double busy_since = -1.0, busy_s = 0.0;  // time with at least one wave on the GPU
    double launch_s = 0.0;                   // worker time spent planning and launching
    std::string create_err;
};

namespace {

thread_local std::string g_srv_err;

void note_busy(awg_server *S, int delta, double t) {
    if (S->inflight == 0 && delta > 0) S->busy_since = t;
    S->inflight += delta;
    S->inflight_max = std::max(S->inflight_max, S->inflight);
    if (S->inflight == 0 && delta < 0 && S->busy_since >= 0) S->busy_s += t - S->busy_since;
}

// A slot's thread: launches each batch assigned to it, waits for it on its own streams,
// hands the results over and frees the slot (or holds it for a resident request).
void slot_main(awg_server *S, int si) {
    Slot &sl = *S->slots[si];
    // the host's cores shared among the slots planning batches at once
    const int hw = (int)std::thread::hardware_concurrency();
    awg::set_plan_threads(std::max(2, hw / std::max(1, (int)S->slots.size() / 2)));
    std::unique_lock<std::mutex> lk(S->mu);
    for (;;) {
        sl.cv.wait(lk, [&] { return sl.state == Slot::ASSIGNED || S->stop_slots; });
        if (sl.state != Slot::ASSIGNED) break;
        const std::vector<Req *> wave = sl.reqs;
        std::vector<awg_problem> probs(wave.size());
        std::vector<awg_outputs> outs(wave.size());
        for (size_t q = 0; q < wave.size(); q++) {
            probs[q] = wave[q]->p;
            outs[q] = wave[q]->out;
        }
        const int precision = wave[0]->precision;
        lk.unlock();
        std::string err;
        const double t0 = now_s();
        int rc = awg::ctx_launch_async(sl.ctx, probs.data(), outs.data(), (int)wave.size(),
                                       precision, err);
        const double t1 = now_s();
        if (rc == 0) rc = awg::ctx_finish(sl.ctx, err);
        else awg::ctx_sync(sl.ctx);  // whatever of the batch was enqueued has finished
        lk.lock();
        const double t = now_s();
        S->launch_s += t1 - t0;
        for (Req *r : wave) {
            r->t_done = t;
            if (rc == 0) {
                r->status = 1;
                S->completed++;
                S->cells_done += r->cells;
                S->lat_ms.push_back(1e3 * (r->t_done - r->t_submit));
                S->queue_ms.push_back(1e3 * (r->t_start - r->t_submit));
                S->service_ms.push_back(1e3 * (r->t_done - r->t_start));
            } else {
                r->status = rc;
                r->err = err;
                S->failed++;
            }
        }
        S->t_last = t;
        note_busy(S, -1, t);
        if (rc == 0 && wave.size() == 1 && wave[0]->resident) {
            sl.state = Slot::HELD;
            wave[0]->slot = si;
        } else {
            S->pool.release(sl.off, sl.bytes);
            sl.reqs.clear();
            sl.state = Slot::IDLE;
        }
        S->cv_done.notify_all();
        S->cv_work.notify_one();
    }
}

// The admitter: forms batches from the queue and assigns them to idle slots.
void serve(awg_server *S) {
    std::unique_lock<std::mutex> lk(S->mu);
    for (;;) {
        while (!S->queue.empty()) {
            int free_slot = -1;
            for (size_t si = 0; si < S->slots.size(); si++)
                if (S->slots[si]->state == Slot::IDLE) {
                    free_slot = (int)si;
                    break;
                }
            if (free_slot < 0) break;
            Req *first = S->queue.front();
            if ((size_t)first->bytes > S->pool.cap) {
                S->queue.pop_front();
                first->status = -5;
                first->err = "the request needs " + std::to_string(first->bytes) +
                             " bytes of device memory; the server's pool holds " +
                             std::to_string(S->pool.cap);
                S->failed++;
                S->cv_done.notify_all();
                continue;
            }
            // the oldest request, then queued requests of like length: a batch lasts as long
            // as its longest chain of columns, so short requests ride with short ones and
            // are not held back by long ones (length within the options' factor of the
            // head's, 2 by default)
            const size_t avail = S->pool.largest();
            const double ratio = S->opt.length_ratio > 1.0 ? S->opt.length_ratio : 2.0;
            std::vector<Req *> wave;
            std::vector<size_t> taken;
            size_t bytes = 0;
            const long long L0 = first->p.seqlen;
            for (size_t qi = 0; qi < S->queue.size(); qi++) {
                Req *r = S->queue[qi];
                if ((int)wave.size() >= S->opt.max_batch) break;
                if (!wave.empty()) {
                    if (first->resident) break;
                    if (r->resident || r->precision != first->precision ||
                        r->want_path != first->want_path || r->want_post != first->want_post)
                        continue;
                    if (ratio * r->p.seqlen < (double)L0 || r->p.seqlen > ratio * L0) continue;
                }
                if (bytes + (size_t)r->bytes > avail) {
                    if (wave.empty()) break;
                    continue;
                }
                wave.push_back(r);
                taken.push_back(qi);
                bytes += (size_t)r->bytes;
            }
            if (wave.empty()) break;  // the head waits for memory to free up
            Slot &sl = *S->slots[free_slot];
            if (!S->pool.alloc(bytes, sl.off)) break;
            for (size_t q = taken.size(); q-- > 0;) S->queue.erase(S->queue.begin() + taken[q]);
            sl.bytes = bytes;
            sl.reqs = wave;
            sl.state = Slot::ASSIGNED;
            const double t = now_s();
            for (Req *r : wave) r->t_start = t;
            note_busy(S, +1, t);
            awg::ctx_set_region(sl.ctx, S->pool_dev + sl.off, bytes);
            sl.cv.notify_one();
        }
        bool any_busy = false;
        for (const auto &sl : S->slots) any_busy |= sl->state == Slot::ASSIGNED;
        if (S->stop && S->queue.empty() && !any_busy) break;
        S->cv_work.wait(lk);
    }
}

template <typename T>
void copy_arr(std::vector<T> &dst, const T *src, size_t n) {
    if (src) dst.assign(src, src + n);
    else dst.clear();
}

}  // namespace

extern "C" {

awg_server *awg_server_create(const awg_server_options *opt) {
    g_srv_err.clear();
    if (!opt || opt->device_bytes < (1 << 20) || opt->max_inflight < 1 || opt->max_batch < 1) {
        g_srv_err = "awg_server_create: device_bytes >= 1 MiB, max_inflight >= 1, max_batch >= 1";
        return nullptr;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        g_srv_err = "no CUDA device: the threading HMM runs on the GPU only";
        return nullptr;
    }
    std::unique_ptr<awg_server> S(new awg_server());
    S->opt = *opt;
    const cudaError_t rc = cudaMalloc(&S->pool_dev, opt->device_bytes);
    if (rc != cudaSuccess) {
        g_srv_err = std::string("awg_server_create: device pool: ") + cudaGetErrorString(rc);
        return nullptr;
    }
    S->pool.init(opt->device_bytes);
    awg_server *raw = S.get();
    // each slot's page-locked staging, sized up front from its share of the pool (inputs
    // and downloaded outputs are a small part of a batch's device footprint)
    const size_t stage = std::min<size_t>(
        256 << 20, std::max<size_t>(64 << 20, opt->device_bytes / opt->max_inflight / 32));
    for (int i = 0; i < opt->max_inflight; i++) {
        S->slots.emplace_back(new Slot());
        S->slots.back()->ctx = awg::ctx_create();
        if (awg::ctx_reserve_host(S->slots.back()->ctx, stage, stage / 2) != 0) {
            g_srv_err = "awg_server_create: page-locked staging";
            for (auto &sl : S->slots) awg::ctx_destroy(sl->ctx);
            cudaFree(S->pool_dev);
            return nullptr;
        }
    }
    for (int i = 0; i < opt->max_inflight; i++) S->slots[i]->th = std::thread(slot_main, raw, i);
    S->worker = std::thread(serve, raw);
    return S.release();
}

void awg_server_destroy(awg_server *S) {
    if (!S) return;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv_work.notify_all();
    if (S->worker.joinable()) S->worker.join();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop_slots = true;
        for (auto &sl : S->slots) sl->cv.notify_all();
    }
    for (auto &sl : S->slots) {
        if (sl->th.joinable()) sl->th.join();
        awg::ctx_destroy(sl->ctx);
    }
    if (S->pool_dev) cudaFree(S->pool_dev);
    delete S;
}

long long awg_server_submit(awg_server *S, const awg_problem *p, const awg_outputs *out,
                            int precision, int resident) {
    g_srv_err.clear();
    if (!S || !p || !out) {
        g_srv_err = "awg_server_submit: NULL argument";
        return -1;
    }
    if (precision != AWG_FP32 && precision != AWG_FP64) {
        g_srv_err = "precision must be AWG_FP64 or AWG_FP32";
        return -1;
    }
    std::unique_ptr<Req> r(new Req());
    r->t_submit = now_s();  // latency counts this call's copying and sizing too
    const size_t tn = (size_t)p->ntrees * p->nnodes;
    copy_arr(r->ptrees, p->ptrees, tn);
    copy_arr(r->ages, p->ages, tn);
    copy_arr(r->sprs, p->sprs, (size_t)p->ntrees * 4);
    copy_arr(r->blocklens, p->blocklens, (size_t)p->ntrees);
    copy_arr(r->mapping, p->mapping, tn);
    copy_arr(r->rc0, p->root_child0, (size_t)p->ntrees);
    copy_arr(r->times, p->times, (size_t)p->ntimes);
    copy_arr(r->pops, p->popsizes, (size_t)p->ntimes);
    copy_arr(r->seqs, p->seqs, (size_t)p->nseqs * p->seqlen);
    if (!p->ptrees || !p->ages || !p->sprs || !p->blocklens || !p->times || !p->popsizes || !p->seqs) {
        g_srv_err = "awg_server_submit: the problem has a NULL array";
        return -1;
    }
    r->p = *p;
    r->p.ptrees = r->ptrees.data();
    r->p.ages = r->ages.data();
    r->p.sprs = r->sprs.data();
    r->p.blocklens = r->blocklens.data();
    r->p.mapping = p->mapping ? r->mapping.data() : nullptr;
    r->p.root_child0 = p->root_child0 ? r->rc0.data() : nullptr;
    r->p.times = r->times.data();
    r->p.popsizes = r->pops.data();
    r->p.seqs = r->seqs.data();
    r->out = *out;
    if (out->uniforms) {
        copy_arr(r->uniforms, out->uniforms, (size_t)p->seqlen);
        r->out.uniforms = r->uniforms.data();
    }
    r->precision = precision;
    r->resident = resident != 0;
    r->want_path = out->path != nullptr;
    r->want_post = out->posterior != nullptr;
    if (r->resident && !r->want_path) {
        g_srv_err = "awg_server_submit: a resident request must want a path";
        return -1;
    }
    // validation and footprint, on the caller's thread
    r->cells = awg_problem_cells(&r->p);
    if (r->cells < 0) {
        g_srv_err = awg_last_error();
        return -1;
    }
    std::string err;
    r->bytes = awg::batch_device_bytes(&r->p, 1, precision, r->want_path, r->want_post, err);
    if (r->bytes < 0) {
        g_srv_err = err;
        return -1;
    }
    std::lock_guard<std::mutex> lk(S->mu);
    r->id = S->next_id++;
    if (S->t_first < 0 || r->t_submit < S->t_first) S->t_first = r->t_submit;
    S->submitted++;
    const long long id = r->id;
    S->queue.push_back(r.get());
    S->reqs[id] = std::move(r);
    S->cv_work.notify_one();
    return id;
}

int awg_server_wait(awg_server *S, long long id, int timeout_ms) {
    g_srv_err.clear();
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) {
        g_srv_err = "awg_server_wait: unknown request";
        return -1;
    }
    Req *r = it->second.get();
    auto done = [&] { return r->status != 0; };
    if (timeout_ms < 0) S->cv_done.wait(lk, done);
    else S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done);
    if (r->status == 0) return 0;
    if (r->status < 0) {
        g_srv_err = r->err;
        return r->status;
    }
    return 1;
}

int awg_server_request_times(awg_server *S, long long id, double *times3) {
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) return -1;
    const Req *r = it->second.get();
    times3[0] = r->t_submit;
    times3[1] = r->t_start;
    times3[2] = r->t_done;
    return 0;
}

int awg_server_forget(awg_server *S, long long id) {
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end() || it->second->status == 0 || it->second->slot >= 0) return -1;
    S->reqs.erase(it);
    return 0;
}

int awg_server_stats_get(awg_server *S, awg_server_stats *out) {
    std::lock_guard<std::mutex> lk(S->mu);
    memset(out, 0, sizeof(*out));
    out->submitted = S->submitted;
    out->completed = S->completed;
    out->failed = S->failed;
    out->cells = S->cells_done;
    out->inflight_max = S->inflight_max;
    out->busy_s = S->busy_s + (S->inflight > 0 && S->busy_since >= 0 ? now_s() - S->busy_since : 0.0);
    out->span_s = S->t_first >= 0 ? S->t_last - S->t_first : 0.0;
    out->launch_s = S->launch_s;
    auto pct = [](std::vector<double> v, double q) {
        std::sort(v.begin(), v.end());
        const double x = q * (v.size() - 1);
        const size_t i = (size_t)x;
        const double f = x - i;
        return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
    };
    if (!S->lat_ms.empty()) {
        out->p50_ms = pct(S->lat_ms, 0.50);
        out->p99_ms = pct(S->lat_ms, 0.99);
        out->max_ms = *std::max_element(S->lat_ms.begin(), S->lat_ms.end());
        double s = 0;
        for (double x : S->lat_ms) s += x;
        out->mean_ms = s / S->lat_ms.size();
        out->queue_p50_ms = pct(S->queue_ms, 0.50);
        out->queue_p99_ms = pct(S->queue_ms, 0.99);
        out->service_p50_ms = pct(S->service_ms, 0.50);
        out->service_p99_ms = pct(S->service_ms, 0.99);
    }
    return 0;
}

int awg_server_resample(awg_server *S, long long id, const double *uniforms, int *path) {
    g_srv_err.clear();
    Slot *sl = nullptr;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        auto it = S->reqs.find(id);
        if (it == S->reqs.end() || it->second->slot < 0) {
            g_srv_err = "awg_server_resample: not a completed resident request";
            return -1;
        }
        sl = S->slots[it->second->slot].get();
    }
    // the slot is held: the worker does not touch its context until it is released
    std::string err;
    const double *u[1] = {uniforms};
    int *pp[1] = {path};
    const int rc = awg::ctx_resample(sl->ctx, u, pp, err);
    if (rc != 0) g_srv_err = err;
    return rc;
}

int awg_server_release(awg_server *S, long long id) {
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end() || it->second->slot < 0) return -1;
    Slot &sl = *S->slots[it->second->slot];
    S->pool.release(sl.off, sl.bytes);
    sl.reqs.clear();
    sl.state = Slot::IDLE;
    it->second->slot = -1;
    S->cv_work.notify_one();
    return 0;
}

const char *awg_server_last_error(void) { return g_srv_err.c_str(); }

}  // extern "C"

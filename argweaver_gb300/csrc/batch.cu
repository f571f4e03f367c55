// Batch engine: arena, upload, kernel sequence, downloads.
//
// Device memory is one grow-only arena per process (no allocation per call once warm);
// inputs travel in one pinned staging buffer and one host-to-device copy. The kernel
// sequence is K1 tables -> K2 variant emissions -> K3 forward -> K4 traceback (when a path
// is wanted) -> K5 backward+posterior (when posteriors are wanted), all on one stream.

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "engine.h"
#include "kernels.h"
#include "plan.h"

namespace awg {

namespace {

std::atomic<long long> g_launches{0};

struct Timings {
    float plan_ms = 0, h2d_ms = 0, tables_ms = 0, emit_ms = 0, forward_ms = 0,
          traceback_ms = 0, backward_ms = 0, d2h_ms = 0, compute_ms = 0;
};

constexpr int MAXG = 12;  // instance groups of the pipelined schedule

struct Engine {
    std::mutex mu;
    bool init = false;
    int device = -1;
    cudaStream_t stream = nullptr;       // uploads, per-tree kernels, downloads
    cudaStream_t gstream[MAXG] = {};     // per group: forward, traceback, backward (high
                                         // priority, so their CTAs are placed first)
    char *dev = nullptr;
    size_t dev_cap = 0;
    char *host = nullptr;
    size_t host_cap = 0;
    cudaEvent_t ev[8];
    cudaEvent_t gev[2 * MAXG + 2];
    Timings last;
    int timing = 0;  // 0 off; 1 on (overlapped schedule: one compute time); 2 serial phases
    int group_div = [] {  // the largest instance group holds n / group_div instances
        const char *e = getenv("AWG_GROUP_DIV");
        return e && atoi(e) > 0 ? atoi(e) : 8;
    }();
};

Engine &engine() {
    static Engine e;
    return e;
}

#define CK(x)                                                                         \
    do {                                                                              \
        cudaError_t rc_ = (x);                                                        \
        if (rc_ != cudaSuccess) {                                                     \
            err = std::string(#x) + ": " + cudaGetErrorString(rc_);                   \
            return -3;                                                                \
        }                                                                             \
    } while (0)

#define CKL(what)                                                                     \
    do {                                                                              \
        cudaError_t rc_ = cudaGetLastError();                                         \
        if (rc_ != cudaSuccess) {                                                     \
            char b_[256];                                                             \
            snprintf(b_, sizeof(b_), "%s launch (maxS %d, maxM %d, nodes %d): %s", what, \
                     plan.maxS, plan.maxM, plan.maxnodes, cudaGetErrorString(rc_));   \
            err = b_;                                                                 \
            return -3;                                                                \
        }                                                                             \
    } while (0)

struct Layout {
    size_t total = 0;
    size_t add(size_t bytes) {
        size_t off = total;
        total += (bytes + 255) & ~size_t(255);
        return off;
    }
};

}  // namespace

long long kernel_launch_count() { return g_launches.load(); }
void note_launch() { g_launches.fetch_add(1); }

int run_batch(const awg_problem *probs, awg_outputs *outs, int n, const RunOptions &opt,
              std::string &err) {
    Engine &E = engine();
    std::lock_guard<std::mutex> lock(E.mu);
    const bool fp32 = opt.precision == AWG_FP32;
    if (!fp32 && opt.precision != AWG_FP64) { err = "precision must be AWG_FP64 or AWG_FP32"; return -1; }

    HostPlan plan;
    if (!plan_layout(probs, n, plan, err, true)) return -1;

    bool want_path = false, want_post = false, want_bw = false;
    for (int q = 0; q < n; q++) {
        want_path |= outs[q].path != nullptr;
        want_post |= outs[q].posterior != nullptr;
        if (opt.backward && opt.backward[q]) want_bw = true;
    }
    want_post |= want_bw;

    if (!E.init) {
        int dc = 0;
        if (cudaGetDeviceCount(&dc) != cudaSuccess || dc == 0) {
            err = "no CUDA device: the threading HMM runs on the GPU only";
            return -2;
        }
        CK(cudaGetDevice(&E.device));
        CK(cudaStreamCreateWithFlags(&E.stream, cudaStreamNonBlocking));
        int lo = 0, hi = 0;
        CK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        for (int g = 0; g < MAXG; g++)
            CK(cudaStreamCreateWithPriority(&E.gstream[g], cudaStreamNonBlocking, hi));
        for (int i = 0; i < 8; i++) CK(cudaEventCreate(&E.ev[i]));
        for (int i = 0; i < 2 * MAXG + 2; i++)
            CK(cudaEventCreateWithFlags(&E.gev[i], cudaEventDisableTiming));
        E.init = true;
    }
    cudaStream_t s = E.stream;

    // ---------------- layout
    const long long ST = std::max(plan.total_states, 1LL);
    const long long CELLS = std::max(plan.total_cells, 1LL);
    const long long COLS = std::max(plan.total_cols, 1LL);
    Layout in;
    const size_t o_inst = in.add(sizeof(InstDev) * plan.ninst);
    const size_t o_blocks = in.add(sizeof(BlockDev) * plan.nblocks);
    const size_t o_model = in.add(sizeof(double) * plan.model.size());
    const size_t o_nodes = in.add(sizeof(int) * 4 * (size_t)plan.total_nodes);
    const size_t o_map = in.add(sizeof(int) * (size_t)std::max(plan.total_map, 1LL));
    const size_t o_seq = in.add((size_t)std::max(plan.total_seq, 1LL));
    const size_t o_cls = in.add((size_t)plan.total_cols);
    const size_t o_cvar = in.add(sizeof(int) * (size_t)plan.total_cols);
    const size_t o_order = in.add(sizeof(int) * plan.ninst);
    const size_t o_blkmap = in.add(sizeof(int) * plan.nblocks);
    const size_t o_u = in.add(want_path ? sizeof(double) * COLS : 0);
    const size_t in_bytes = in.total;

    if (in_bytes > E.host_cap) {
        if (E.host) cudaFreeHost(E.host);
        E.host = nullptr;
        E.host_cap = 0;
        const size_t cap = in_bytes + in_bytes / 8;
        CK(cudaMallocHost(&E.host, cap));
        E.host_cap = cap;
    }

    // ---------------- stage inputs
    char *h = E.host;
    // per-node, per-column and sequence arrays straight into the staging buffer
    plan_fill(probs, n, plan, PlanDst{(int *)(h + o_nodes), (int *)(h + o_map),
                                      (uint8_t *)(h + o_seq), (uint8_t *)(h + o_cls),
                                      (int *)(h + o_cvar)});
    memcpy(h + o_inst, plan.inst.data(), sizeof(InstDev) * plan.ninst);
    memcpy(h + o_blocks, plan.blocks.data(), sizeof(BlockDev) * plan.nblocks);
    memcpy(h + o_model, plan.model.data(), sizeof(double) * plan.model.size());

    Layout w;  // work region follows the inputs
    w.total = in_bytes;
    const size_t o_sinfo = w.add(sizeof(StateInfo) * ST);
    const size_t o_t2off = w.add(sizeof(int) * ST);
    const size_t o_btptr = w.add(sizeof(int) * (size_t)plan.nblocks * (MAXT + 1));
    const size_t o_btperm = w.add(sizeof(int) * ST);
    const size_t o_tm = w.add(sizeof(double) * (size_t)plan.nblocks * MAXT * MAXT);
    const size_t o_gts = w.add(sizeof(double) * std::max(plan.total_M, 1LL));
    const size_t o_inv = w.add(sizeof(double) * ST);
    const size_t o_det = w.add(sizeof(int) * ST);
    const size_t o_detp = w.add(sizeof(double) * ST);
    const size_t o_srcs = w.add(sizeof(int2) * plan.nblocks);
    const size_t o_rrow = w.add(sizeof(double) * ST);
    const size_t o_crow = w.add(sizeof(double) * ST);
    const size_t o_gptr = w.add(sizeof(int) * (ST + plan.nblocks + 1));
    const size_t o_gidx = w.add(sizeof(int) * ST);
    const size_t o_var = w.add(sizeof(double) * std::max(plan.total_var, 1LL));
    size_t o_tm32 = 0, o_t2d32 = 0, o_inv32 = 0, o_var32 = 0, o_detp32 = 0, o_rrow32 = 0,
           o_crow32 = 0, o_rstay32 = 0, o_lneref = 0, o_lnvref = 0,
           o_blkext = 0;
    if (fp32) {
        o_tm32 = w.add(sizeof(float) * (size_t)plan.nblocks * MAXT * MAXT);
        o_t2d32 = w.add(sizeof(float) * std::max(plan.total_M, 1LL));
        o_inv32 = w.add(sizeof(float) * ST);
        o_var32 = w.add(sizeof(float) * std::max(plan.total_var, 1LL));
        o_detp32 = w.add(sizeof(float) * ST);
        o_rrow32 = w.add(sizeof(float) * ST);
        o_crow32 = w.add(sizeof(float) * ST);
        o_rstay32 = w.add(sizeof(float) * (size_t)plan.nblocks * MAXT);
        o_lneref = w.add(sizeof(double) * plan.nblocks);
        o_lnvref = w.add(sizeof(double) * std::max(plan.total_vcols, 1LL));
        o_blkext = w.add(sizeof(double) * plan.nblocks);
    }
    const size_t o_fw = w.add((fp32 ? sizeof(float) : sizeof(double)) * CELLS);
    const size_t o_lnl = w.add(sizeof(double) * plan.ninst);
    const size_t o_post = w.add(want_post ? sizeof(double) * CELLS : 0);
    const size_t o_bw = w.add(want_bw ? sizeof(double) * CELLS : 0);
    const size_t o_path = w.add(want_path ? sizeof(int) * COLS : 0);
    // FP32 traceback: the forward columns' time-bin sums
    const bool want_bins = fp32 && want_path && forward_writes_bins(plan.maxS);
    const size_t o_bins = w.add(want_bins ? sizeof(float) * MAXT * COLS : 0);
    const size_t o_err = w.add(4 * sizeof(int));
    const size_t total = w.total;

    if (total > E.dev_cap) {
        if (E.dev) cudaFree(E.dev);
        E.dev = nullptr;
        E.dev_cap = 0;
        const size_t cap = total + total / 8;
        CK(cudaMalloc(&E.dev, cap));
        E.dev_cap = cap;
    }

    {
        // per-instance kernels take the largest instances first: their time is a chain of
        // columns, so the batch ends when its longest chain does
        int *ord = (int *)(h + o_order);
        std::vector<long long> cost(plan.ninst);
        for (int q = 0; q < plan.ninst; q++) {
            const long long cells =
                (q + 1 < plan.ninst ? plan.inst[q + 1].cell0 : plan.total_cells) - plan.inst[q].cell0;
            cost[q] = 256LL * plan.inst[q].seqlen + cells;
            ord[q] = q;
        }
        std::stable_sort(ord, ord + plan.ninst, [&](int a, int b) { return cost[a] > cost[b]; });
        // trees of the instances in that order, so a group of instances is a range
        int *bm = (int *)(h + o_blkmap);
        int k = 0;
        for (int j = 0; j < plan.ninst; j++) {
            const InstDev &I = plan.inst[ord[j]];
            for (int b = 0; b < I.ntrees; b++) bm[k++] = I.block0 + b;
        }
    }
    if (want_path) {
        double *u = (double *)(h + o_u);
        for (int q = 0; q < n; q++) {
            const InstDev &I = plan.inst[q];
            if (outs[q].uniforms) {
                memcpy(u + I.col0, outs[q].uniforms, sizeof(double) * I.seqlen);
            } else {
                // the reference's draws: rand()/RAND_MAX, last column first (common.h:103-110)
                for (int c = I.seqlen - 1; c >= 0; c--) u[I.col0 + c] = rand() / double(RAND_MAX);
            }
        }
    }

    BatchDev d;
    memset(&d, 0, sizeof(d));
    char *D = E.dev;
    d.ninst = plan.ninst; d.nblocks = plan.nblocks; d.maxS = plan.maxS; d.maxT = plan.maxT;
    d.maxnodes = plan.maxnodes;
    d.maxM = plan.maxM;
    d.inst = (const InstDev *)(D + o_inst);
    d.order = (const int *)(D + o_order);
    d.blocks = (BlockDev *)(D + o_blocks);
    d.model = (const double *)(D + o_model);
    d.nodes = (const int4 *)(D + o_nodes);
    d.mapping = (const int *)(D + o_map);
    d.seqT = (const uint8_t *)(D + o_seq);
    d.colclass = (const uint8_t *)(D + o_cls);
    d.colvar = (const int *)(D + o_cvar);
    d.sinfo = (StateInfo *)(D + o_sinfo);
    d.t2off = (int *)(D + o_t2off);
    d.bt_ptr = (int *)(D + o_btptr);
    d.bt_perm = (int *)(D + o_btperm);
    d.tm = (double *)(D + o_tm);
    d.gts = (double *)(D + o_gts);
    d.inv_lk = (double *)(D + o_inv);
    d.determ = (int *)(D + o_det);
    d.determprob = (double *)(D + o_detp);
    d.srcs = (int2 *)(D + o_srcs);
    d.recombrow = (double *)(D + o_rrow);
    d.recoalrow = (double *)(D + o_crow);
    d.gptr = (int *)(D + o_gptr);
    d.gidx = (int *)(D + o_gidx);
    d.varemit = (double *)(D + o_var);
    if (fp32) {
        d.tm32 = (float *)(D + o_tm32);
        d.t2d32 = (float *)(D + o_t2d32);
        d.inv32 = (float *)(D + o_inv32);
        d.var32 = (float *)(D + o_var32);
        d.determprob32 = (float *)(D + o_detp32);
        d.recombrow32 = (float *)(D + o_rrow32);
        d.recoalrow32 = (float *)(D + o_crow32);
        d.rstay32 = (float *)(D + o_rstay32);
        d.lneref = (double *)(D + o_lneref);
        d.lnvref = (double *)(D + o_lnvref);
        d.blkext = (double *)(D + o_blkext);
        d.fw32 = (float *)(D + o_fw);
    } else {
        d.fw64 = (double *)(D + o_fw);
    }
    d.lnl = (double *)(D + o_lnl);
    d.post = want_post ? (double *)(D + o_post) : nullptr;
    d.uniforms = want_path ? (const double *)(D + o_u) : nullptr;
    d.path = want_path ? (int *)(D + o_path) : nullptr;
    d.bins32 = want_bins ? (float *)(D + o_bins) : nullptr;
    d.err = (int *)(D + o_err);

    // Schedule. Serial: per-tree kernels over the batch, then per-instance kernels. Pipelined
    // (larger batches): instances in groups, largest first; a group's per-tree kernels run
    // on the main stream and its forward (then traceback/backward) on high-priority streams
    // as soon as they are done, so the long per-instance chains start early and the
    // per-tree work of later groups fills the SMs they leave idle.
    const bool pipelined = n >= 16 && !opt.tables_only && !opt.priors && E.timing != 2;
    const bool T = E.timing != 0;
    if (T) CK(cudaEventRecord(E.ev[0], s));
    CK(cudaMemcpyAsync(D, h, in_bytes, cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(d.err, 0, 4 * sizeof(int), s));
    if (T) CK(cudaEventRecord(E.ev[1], s));
    if (pipelined) {
        // group sizes n/32, doubling up to n/div; the last takes the rest
        int bounds[MAXG + 1];
        int ng = 0, q0 = 0, sz = std::max(1, n / 32);
        const int cap = std::max(1, n / std::max(1, E.group_div));
        bounds[0] = 0;
        while (q0 < n) {
            const int q1 = (ng == MAXG - 1) ? n : std::min(n, q0 + sz);
            bounds[++ng] = q1;
            q0 = q1;
            sz = std::min(2 * sz, std::max(cap, sz));
        }
        const int *ord = (const int *)(h + o_order);
        int boff = 0;
        for (int g = 0; g < ng; g++) {
            BatchDev dg = d;
            int nb = 0;
            for (int j = bounds[g]; j < bounds[g + 1]; j++) nb += plan.inst[ord[j]].ntrees;
            dg.order = d.order + bounds[g];
            dg.ninst = bounds[g + 1] - bounds[g];
            dg.blkmap = (const int *)(D + o_blkmap) + boff;
            dg.nblocks = nb;
            boff += nb;
            launch_tables(dg, fp32, s);
            CKL("table kernel");
            launch_varemit(dg, fp32, s);
            CKL("emission kernel");
            cudaStream_t gs = E.gstream[g];
            CK(cudaEventRecord(E.gev[2 * g], s));
            CK(cudaStreamWaitEvent(gs, E.gev[2 * g], 0));
            launch_forward(dg, fp32, gs);
            CKL("forward kernel");
            if (want_path) {
                launch_traceback(dg, fp32, gs);
                CKL("traceback kernel");
            }
            if (want_post) {
                launch_backward(dg, fp32, want_bw ? (double *)(D + o_bw) : nullptr, gs);
                CKL("backward kernel");
            }
            CK(cudaEventRecord(E.gev[2 * g + 1], gs));
        }
        for (int g = 0; g < ng; g++) CK(cudaStreamWaitEvent(s, E.gev[2 * g + 1], 0));
        if (T) CK(cudaEventRecord(E.ev[6], s));
    } else {
        launch_tables(d, fp32, s);
        CKL("table kernel");
        if (opt.priors) {
            for (int q = 0; q < n; q++) {
                if (!opt.priors[q]) continue;
                const InstDev &I = plan.inst[q];
                const int S0 = std::max(plan.blocks[I.block0].S, 1);
                if (fp32) {
                    std::vector<float> tmp(opt.priors[q], opt.priors[q] + S0);
                    CK(cudaMemcpyAsync(d.fw32 + I.cell0, tmp.data(), sizeof(float) * S0,
                                       cudaMemcpyHostToDevice, s));
                    CK(cudaStreamSynchronize(s));
                } else {
                    CK(cudaMemcpyAsync(d.fw64 + I.cell0, opt.priors[q], sizeof(double) * S0,
                                       cudaMemcpyHostToDevice, s));
                }
            }
        }
        if (opt.tables_only) {
            const InstDev &I = plan.inst[0];
            std::vector<double> tmall((size_t)plan.nblocks * MAXT * MAXT);
            CK(cudaMemcpyAsync(tmall.data(), d.tm, sizeof(double) * tmall.size(),
                               cudaMemcpyDeviceToHost, s));
            if (opt.dbg_gts)
                CK(cudaMemcpyAsync(opt.dbg_gts, d.gts, sizeof(double) * plan.total_M,
                                   cudaMemcpyDeviceToHost, s));
            if (opt.dbg_inv)
                CK(cudaMemcpyAsync(opt.dbg_inv, d.inv_lk, sizeof(double) * plan.total_states,
                                   cudaMemcpyDeviceToHost, s));
            if (opt.dbg_btptr)
                CK(cudaMemcpyAsync(opt.dbg_btptr, d.bt_ptr, sizeof(int) * plan.nblocks * (MAXT + 1),
                                   cudaMemcpyDeviceToHost, s));
            if (opt.dbg_btperm)
                CK(cudaMemcpyAsync(opt.dbg_btperm, d.bt_perm, sizeof(int) * plan.total_states,
                                   cudaMemcpyDeviceToHost, s));
            if (opt.dbg_prior)
                CK(cudaMemcpyAsync(opt.dbg_prior, d.fw64 + I.cell0,
                                   sizeof(double) * std::max(plan.blocks[0].S, 1),
                                   cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            if (opt.dbg_tm) {
                const int T = I.T;
                for (int b = 0; b < plan.nblocks; b++)
                    for (int a = 0; a < T - 1; a++)
                        for (int c = 0; c < T - 1; c++)
                            opt.dbg_tm[((size_t)b * (T - 1) + a) * (T - 1) + c] =
                                tmall[((size_t)b * MAXT + a) * MAXT + c];
            }
            return 0;
        }
        if (T) CK(cudaEventRecord(E.ev[2], s));
        launch_varemit(d, fp32, s);
        CKL("emission kernel");
        if (T) CK(cudaEventRecord(E.ev[3], s));
        launch_forward(d, fp32, s);
        CKL("forward kernel");
        if (T) CK(cudaEventRecord(E.ev[4], s));
        if (want_path) {
            launch_traceback(d, fp32, s);
            CKL("traceback kernel");
        }
        if (T) CK(cudaEventRecord(E.ev[5], s));
        if (want_post) {
            launch_backward(d, fp32, want_bw ? (double *)(D + o_bw) : nullptr, s);
            CKL("backward kernel");
        }
        if (T) CK(cudaEventRecord(E.ev[6], s));
    }

    // ---------------- downloads
    for (int q = 0; q < n; q++) {
        const InstDev &I = plan.inst[q];
        const long long cells = (q + 1 < n ? plan.inst[q + 1].cell0 : plan.total_cells) - I.cell0;
        const awg_outputs &o = outs[q];
        if (o.forward && !fp32)
            CK(cudaMemcpyAsync(o.forward, d.fw64 + I.cell0, sizeof(double) * cells,
                               cudaMemcpyDeviceToHost, s));
        if (o.forward32 && fp32)
            CK(cudaMemcpyAsync(o.forward32, d.fw32 + I.cell0, sizeof(float) * cells,
                               cudaMemcpyDeviceToHost, s));
        if (o.posterior)
            CK(cudaMemcpyAsync(o.posterior, d.post + I.cell0, sizeof(double) * cells,
                               cudaMemcpyDeviceToHost, s));
        if (opt.backward && opt.backward[q])
            CK(cudaMemcpyAsync(opt.backward[q], (double *)(D + o_bw) + I.cell0,
                               sizeof(double) * cells, cudaMemcpyDeviceToHost, s));
        if (o.path)
            CK(cudaMemcpyAsync(o.path, d.path + I.col0, sizeof(int) * I.seqlen,
                               cudaMemcpyDeviceToHost, s));
        if (o.loglik)
            CK(cudaMemcpyAsync(o.loglik, d.lnl + q, sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    int dev_err[4] = {0, 0, 0, 0};
    CK(cudaMemcpyAsync(dev_err, d.err, 4 * sizeof(int), cudaMemcpyDeviceToHost, s));
    if (T) CK(cudaEventRecord(E.ev[7], s));
    CK(cudaStreamSynchronize(s));
    if (T) {
        Timings t;
        cudaEventElapsedTime(&t.h2d_ms, E.ev[0], E.ev[1]);
        cudaEventElapsedTime(&t.compute_ms, E.ev[1], E.ev[6]);
        cudaEventElapsedTime(&t.d2h_ms, E.ev[6], E.ev[7]);
        if (!pipelined) {
            float ms[5];
            for (int i = 0; i < 5; i++) cudaEventElapsedTime(&ms[i], E.ev[i + 1], E.ev[i + 2]);
            t.tables_ms = ms[0]; t.emit_ms = ms[1]; t.forward_ms = ms[2];
            t.traceback_ms = ms[3]; t.backward_ms = ms[4];
        }
        E.last = t;
    }
    if (dev_err[0] != 0) {
        static const char *what[] = {"", "switch from a fully specified tree found no state",
                                     "shared-memory plan exceeded", "a forward column summed to "
                                     "zero or NaN", "device state count differs from the plan",
                                     "an index derived from the inputs is out of range",
                                     "a bounded wait for an asynchronous copy ran out"};
        char buf[256];
        snprintf(buf, sizeof(buf), "device error %d (%s) at problem %d, tree %d, column %d",
                 dev_err[0], dev_err[0] < 7 ? what[dev_err[0]] : "?", dev_err[1], dev_err[2],
                 dev_err[3]);
        err = buf;
        return -4;
    }
    return 0;
}

}  // namespace awg

extern "C" {

// Device times (ms) of the last batch when timing is on: h2d, tables, emissions, forward,
// traceback, backward, d2h, compute (the kernels from the end of the upload to the start of
// the downloads). mode 1 keeps the overlapped schedule (phases read 0 when it ran); mode 2
// runs the kernels one phase after another to time each.
void awg_set_timing(int mode) { awg::engine().timing = mode; }
void awg_last_timings(double *out8) {
    const auto &t = awg::engine().last;
    const float v[8] = {t.h2d_ms, t.tables_ms, t.emit_ms, t.forward_ms, t.traceback_ms,
                        t.backward_ms, t.d2h_ms, t.compute_ms};
    for (int i = 0; i < 8; i++) out8[i] = v[i];
}

}  // extern "C"

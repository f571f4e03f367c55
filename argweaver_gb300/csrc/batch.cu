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
#include <map>
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
    // schedule defaults (environment overrides for experiments) and the tuned ones by class
    TuneCfg defaults = [] {
        TuneCfg c;
        if (const char *e = getenv("AWG_GROUP_DIV")) c.group_div = std::max(1, atoi(e));
        if (const char *e = getenv("AWG_FORWARD_KPT")) c.kpt = atoi(e);
        if (const char *e = getenv("AWG_PERSISTENT")) c.persistent = atoi(e) != 0;
        return c;
    }();
    std::map<long long, TuneCfg> tuned;
    // the captured step of the last batch (kernels, memsets, cross-stream events) and the
    // launch parameters it was captured with; replayed while they match
    bool graphs = [] {
        const char *e = getenv("AWG_GRAPHS");
        return !(e && atoi(e) == 0);
    }();
    cudaGraphExec_t gexec = nullptr;
    std::vector<long long> gsig;
    long long gkernels = 0;
    long long graph_replays = 0, graph_captures = 0;
    long long last_key = -1;  // shape class of the last batch
};

// Shape class of a batch for the tuned schedules: precision, path or not, ntimes, and the
// binary orders of magnitude of the largest state count and of the instance count.
long long shape_key(const HostPlan &plan, bool fp32, bool path) {
    auto lg = [](long long v) {
        int k = 0;
        while ((1LL << (k + 1)) <= v && k < 30) k++;
        return (long long)k;
    };
    return (long long)fp32 | (long long)path << 1 | (long long)plan.maxT << 2 |
           lg(std::max(plan.maxS, 1)) << 8 | lg(std::max(plan.ninst, 1)) << 14;
}

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
    TuneCfg cfg = E.defaults;
    E.last_key = shape_key(plan, fp32, want_path);
    if (opt.cfg) {
        cfg = *opt.cfg;
    } else {
        auto it = E.tuned.find(shape_key(plan, fp32, want_path));
        if (it != E.tuned.end()) cfg = it->second;
    }

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
    const bool want_bins = fp32 && want_path && forward_writes_bins(plan.maxS, cfg.kpt);
    const size_t o_bins = w.add(want_bins ? sizeof(float) * MAXT * COLS : 0);
    const size_t o_err = w.add(4 * sizeof(int));
    const size_t o_queue = w.add(sizeof(int) * 2 * MAXG);  // work counters of the groups
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
    // per-tree work of later groups fills the SMs they leave idle. The per-tree kernels are
    // persistent, work-stealing over units of trees; the device part of a step is captured
    // once as a CUDA graph and replayed while its launch parameters repeat.
    const bool special = opt.tables_only || opt.priors;
    const bool serial_timing = E.timing == 2;
    const bool pipelined = n >= 16 && !special && !serial_timing;
    const bool T = E.timing != 0;
    int *queues = (int *)(D + o_queue);
    if (T) CK(cudaEventRecord(E.ev[0], s));
    CK(cudaMemcpyAsync(D, h, in_bytes, cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(d.err, 0, 4 * sizeof(int), s));
    if (T) CK(cudaEventRecord(E.ev[1], s));

    // groups of the pipelined schedule: sizes n/32, doubling up to n/group_div, the last
    // takes the rest
    int bounds[MAXG + 1];
    int ng = 1;
    bounds[0] = 0;
    bounds[1] = n;
    if (pipelined) {
        int q0 = 0, sz = std::max(1, n / 32);
        const int cap = std::max(1, n / std::max(1, cfg.group_div));
        ng = 0;
        while (q0 < n) {
            const int q1 = (ng == MAXG - 1) ? n : std::min(n, q0 + sz);
            bounds[++ng] = q1;
            q0 = q1;
            sz = std::min(2 * sz, std::max(cap, sz));
        }
    }
    int *qk = cfg.persistent ? queues : nullptr;
    auto qp = [&](int i) { return qk ? qk + i : nullptr; };
    // the device part of the step (no host synchronisation: it is also what is captured)
    auto enqueue = [&]() -> cudaError_t {
        cudaError_t rc;
#define EQ(x)                                                                         \
    do {                                                                              \
        if ((rc = (x)) != cudaSuccess) return rc;                                     \
    } while (0)
        if (qk) EQ(cudaMemsetAsync(queues, 0, sizeof(int) * 2 * MAXG, s));
        if (pipelined) {
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
                launch_tables(dg, fp32, s, qp(2 * g), cfg.chunk);
                EQ(cudaGetLastError());
                launch_varemit(dg, fp32, s, qp(2 * g + 1), cfg.chunk);
                EQ(cudaGetLastError());
                cudaStream_t gs = E.gstream[g];
                EQ(cudaEventRecord(E.gev[2 * g], s));
                EQ(cudaStreamWaitEvent(gs, E.gev[2 * g], 0));
                launch_forward(dg, fp32, gs, cfg.kpt);
                EQ(cudaGetLastError());
                if (want_path) {
                    launch_traceback(dg, fp32, gs);
                    EQ(cudaGetLastError());
                }
                if (want_post) {
                    launch_backward(dg, fp32, want_bw ? (double *)(D + o_bw) : nullptr, gs);
                    EQ(cudaGetLastError());
                }
                EQ(cudaEventRecord(E.gev[2 * g + 1], gs));
            }
            for (int g = 0; g < ng; g++) EQ(cudaStreamWaitEvent(s, E.gev[2 * g + 1], 0));
        } else {
            launch_tables(d, fp32, s, qp(0), cfg.chunk);
            EQ(cudaGetLastError());
            launch_varemit(d, fp32, s, qp(1), cfg.chunk);
            EQ(cudaGetLastError());
            launch_forward(d, fp32, s, cfg.kpt);
            EQ(cudaGetLastError());
            if (want_path) {
                launch_traceback(d, fp32, s);
                EQ(cudaGetLastError());
            }
            if (want_post) {
                launch_backward(d, fp32, want_bw ? (double *)(D + o_bw) : nullptr, s);
                EQ(cudaGetLastError());
            }
        }
#undef EQ
        return cudaSuccess;
    };
    auto cuda_fail = [&](cudaError_t rc, const char *what) {
        char b[320];
        snprintf(b, sizeof(b), "%s (maxS %d, maxM %d, nodes %d): %s", what, plan.maxS, plan.maxM,
                 plan.maxnodes, cudaGetErrorString(rc));
        err = b;
        return -3;
    };

    if (!special && !serial_timing) {
        if (E.graphs) {
            // everything a launch depends on: buffers, counts, groups and schedule knobs
            std::vector<long long> sig = {(long long)(uintptr_t)D, (long long)fp32, want_path,
                                          want_post, want_bw, want_bins, plan.ninst, plan.nblocks,
                                          plan.maxS, plan.maxT, plan.maxnodes, plan.maxM,
                                          cfg.kpt, cfg.chunk, cfg.group_div, cfg.persistent, ng,
                                          (long long)total};
            for (size_t o : {o_inst, o_blocks, o_model, o_nodes, o_map, o_seq, o_cls, o_cvar,
                             o_order, o_blkmap, o_u, o_sinfo, o_t2off, o_btptr, o_btperm, o_tm,
                             o_gts, o_inv, o_det, o_detp, o_srcs, o_rrow, o_crow, o_gptr, o_gidx,
                             o_var, o_tm32, o_t2d32, o_inv32, o_var32, o_detp32, o_rrow32,
                             o_crow32, o_rstay32, o_lneref, o_lnvref, o_blkext, o_fw, o_lnl,
                             o_post, o_bw, o_path, o_bins, o_err, o_queue})
                sig.push_back((long long)o);
            for (int g = 0; g <= ng; g++) sig.push_back(bounds[g]);
            const int *ord = (const int *)(h + o_order);
            for (int j = 0; j < n && pipelined; j++) sig.push_back(plan.inst[ord[j]].ntrees);
            if (!(E.gexec && sig == E.gsig)) {
                if (E.gexec) cudaGraphExecDestroy(E.gexec);
                E.gexec = nullptr;
                E.gsig.clear();
                const long long before = kernel_launch_count();
                CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
                const cudaError_t rc = enqueue();
                cudaGraph_t graph = nullptr;
                const cudaError_t rc2 = cudaStreamEndCapture(s, &graph);
                if (rc != cudaSuccess || rc2 != cudaSuccess) {
                    if (graph) cudaGraphDestroy(graph);
                    return cuda_fail(rc != cudaSuccess ? rc : rc2, "capturing the step");
                }
                const cudaError_t rc3 =
                    cudaGraphInstantiateWithFlags(&E.gexec, graph, cudaGraphInstantiateFlagUseNodePriority);
                cudaGraphDestroy(graph);
                if (rc3 != cudaSuccess) {
                    E.gexec = nullptr;
                    return cuda_fail(rc3, "instantiating the step's graph");
                }
                E.gsig = std::move(sig);
                E.gkernels = kernel_launch_count() - before;
                E.graph_captures++;
            } else {
                for (long long q = 0; q < E.gkernels; q++) note_launch();
                E.graph_replays++;
            }
            CK(cudaGraphLaunch(E.gexec, s));
        } else {
            const cudaError_t rc = enqueue();
            if (rc != cudaSuccess) return cuda_fail(rc, "kernel launch");
        }
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
        launch_forward(d, fp32, s, cfg.kpt);
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
        if (serial_timing || special) {
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

int autotune(const awg_problem *probs, awg_outputs *outs, int n, int precision, int trials,
             TuneCfg &best, double &best_ms, std::string &err) {
    Engine &E = engine();
    const int saved_timing = E.timing;
    E.timing = 1;
    trials = std::max(trials, 1);
    auto measure = [&](const TuneCfg &c, double &ms) -> int {
        RunOptions o;
        o.cfg = &c;
        o.precision = precision;
        ms = 1e300;
        for (int t = 0; t < trials; t++) {
            const int rc = run_batch(probs, outs, n, o, err);
            if (rc != 0) return rc;
            ms = std::min(ms, (double)E.last.compute_ms);
        }
        return 0;
    };
    // coordinate descent from the defaults: forward CTA size (states per owner thread),
    // group cap of the pipelined schedule, unit length of the per-tree work queue, and
    // persistent versus one-CTA-per-tree per-tree kernels
    best = E.defaults;
    int rc = measure(best, best_ms);
    const long long key = E.last_key;
    const std::vector<std::pair<int TuneCfg::*, std::vector<int>>> knobs = {
        {&TuneCfg::kpt, {0, 2, 4}},
        {&TuneCfg::group_div, {4, 8, 16}},
        {&TuneCfg::chunk, {1, 4}},
        {&TuneCfg::persistent, {1, 0}},
    };
    for (const auto &k : knobs) {
        if (rc != 0) break;
        const TuneCfg base = best;
        for (int v : k.second) {
            if (base.*(k.first) == v) continue;
            TuneCfg c = base;
            c.*(k.first) = v;
            double ms;
            rc = measure(c, ms);
            if (rc != 0) break;
            if (ms < best_ms) {
                best_ms = ms;
                best = c;
            }
        }
    }
    E.timing = saved_timing;
    if (rc != 0) return rc;
    {
        std::lock_guard<std::mutex> lock(E.mu);
        E.tuned[key] = best;
    }
    return 0;
}

}  // namespace awg

extern "C" {

// Whether steps are captured as CUDA graphs and replayed (1, the default) or launched
// kernel by kernel (0); and how many steps were replayed / captured so far.
void awg_set_graphs(int on) { awg::engine().graphs = on != 0; }

// Default schedule (kpt 0 = by state count; group_div, chunk >= 1; persistent 0/1); clears
// the autotuner's choices so the defaults apply to every shape class.
void awg_set_schedule(int kpt, int group_div, int chunk, int persistent) {
    awg::Engine &E = awg::engine();
    std::lock_guard<std::mutex> lock(E.mu);
    E.defaults.kpt = (kpt == 1 || kpt == 2 || kpt == 4 || kpt == 8) ? kpt : 0;
    E.defaults.group_div = std::max(1, group_div);
    E.defaults.chunk = std::max(1, chunk);
    E.defaults.persistent = persistent != 0;
    E.tuned.clear();
}
long long awg_graph_replays(void) { return awg::engine().graph_replays; }
long long awg_graph_captures(void) { return awg::engine().graph_captures; }

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

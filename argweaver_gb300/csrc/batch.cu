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
#include <set>
#include <vector>

#include "engine.h"
#include "kernels.h"
#include "plan.h"

namespace awg {

struct Timings {
    float plan_ms = 0, h2d_ms = 0, tables_ms = 0, emit_ms = 0, forward_ms = 0,
          traceback_ms = 0, backward_ms = 0, d2h_ms = 0, compute_ms = 0;
};

constexpr int MAXG = 12;  // instance groups of the pipelined schedule

// One execution context: streams, device arena, page-locked staging and the captured graph
// of its last step. The engine owns one; a server owns one per in-flight batch.
struct Ctx {
    bool init = false;
    int device = -1;
    cudaStream_t stream = nullptr;       // uploads, per-tree kernels, downloads
    cudaStream_t gstream[MAXG] = {};     // per group: forward, traceback, backward (high
                                         // priority, so their CTAs are placed first)
    char *dev = nullptr;
    size_t dev_cap = 0;
    char *host = nullptr;                // inputs staging (page-locked)
    size_t host_cap = 0;
    char *ext = nullptr;                 // device region given by the owner (a server's
    size_t ext_cap = 0;                  // pool), used instead of the grow-only arena
    char *hout = nullptr;                // outputs staging of an asynchronous batch
    size_t hout_cap = 0;
    cudaEvent_t ev[8];
    cudaEvent_t gev[2 * MAXG + 2];
    cudaEvent_t done = nullptr;          // end of the last batch's downloads
    Timings last;
    // the captured step of the last batch (kernels, memsets, cross-stream events) and the
    // launch parameters it was captured with; replayed while they match
    cudaGraphExec_t gexec = nullptr;
    std::vector<long long> gsig;
    long long gkernels = 0;
    // an asynchronous batch's outputs: (caller buffer, staging offset, bytes)
    struct Copy {
        void *dst;
        size_t off, bytes;
    };
    std::vector<Copy> copies;
    size_t err_off = 0;
    bool timed = false, serial_phases = false;
    bool graphs = true;  // capture and replay steps (off for one-shot batches: a server's)
    // Page-locked buffers outgrown while other batches run are kept until the context is
    // destroyed: cudaFreeHost would wait for the whole device, stalling every batch in flight.
    bool defer_free = false;
    std::vector<char *> stale;
    HostPlan plan;
    // the last batch's device view, for draws from its resident forward tables
    BatchDev d{};
    bool have_d = false, d_fp32 = false;
    size_t o_u = 0;
};

namespace {

std::atomic<long long> g_launches{0};

void drop_host(Ctx &C, char *p) {
    if (C.defer_free) C.stale.push_back(p);
    else cudaFreeHost(p);
}

struct Engine {
    std::mutex mu;
    Ctx ctx;
    int timing = 0;  // 0 off; 1 on (overlapped schedule: one compute time); 2 serial phases
    // schedule defaults (environment overrides for experiments) and the tuned ones by class
    TuneCfg defaults = [] {
        TuneCfg c;
        if (const char *e = getenv("AWG_GROUP_DIV")) c.group_div = std::max(1, atoi(e));
        if (const char *e = getenv("AWG_FORWARD_KPT")) c.kpt = atoi(e);
        if (const char *e = getenv("AWG_PERSISTENT")) c.persistent = atoi(e) != 0;
        return c;
    }();
    std::mutex tune_mu;  // the tuned table, read by every context
    std::map<long long, TuneCfg> tuned;
    bool graphs = [] {
        const char *e = getenv("AWG_GRAPHS");
        return !(e && atoi(e) == 0);
    }();
    std::atomic<long long> graph_replays{0}, graph_captures{0};
    long long last_key = -1;  // shape class of the engine's last batch
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

namespace {
std::mutex g_attr_mu;
std::map<const void *, size_t> g_smem_limit;  // kernel -> dynamic shared memory opted in
std::set<const void *> g_carveout;            // kernels given the largest carveout
}  // namespace

void prefer_shared_fn(const void *kernel) {
    std::lock_guard<std::mutex> lock(g_attr_mu);
    if (g_carveout.insert(kernel).second)
        cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
}

bool raise_dynamic_smem_fn(const void *kernel, size_t bytes) {
    std::lock_guard<std::mutex> lock(g_attr_mu);
    size_t &cur = g_smem_limit[kernel];
    if (bytes <= cur) return true;
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) !=
        cudaSuccess)
        return false;
    cur = bytes;
    return true;
}

// Plans, uploads and enqueues one batch on context C. Synchronous (async false): outputs go
// straight to the caller's buffers and the call returns when they are there. Asynchronous:
// outputs go to C's page-locked staging, C.done marks their arrival, and ctx_complete (on
// the same thread, before C's next batch) checks the device error record and hands them
// over. timing: 0 off, 1 one compute time, 2 kernels one phase after another. Returns 0,
// 1 when a debug or dense-table call finished inside it (nothing left for ctx_complete), or
// a negative code with err set.
int ctx_launch(Ctx &C, const awg_problem *probs, awg_outputs *outs, int n, const RunOptions &opt,
               bool async, int timing, long long *key_out, std::string &err,
               size_t *dry_bytes) {
    const bool dry = dry_bytes != nullptr;  // only the device bytes the batch needs
    Engine &E = engine();
    const bool fp32 = opt.precision == AWG_FP32;
    if (!fp32 && opt.precision != AWG_FP64) { err = "precision must be AWG_FP64 or AWG_FP32"; return -1; }
    if (fp32 && opt.last_states) { err = "a given last traceback state needs AWG_FP64"; return -1; }
    if (fp32 && opt.dense) { err = "the dense forward step needs AWG_FP64"; return -1; }
    if (fp32 && opt.dense_kind) { err = "the dense helper matrices need AWG_FP64"; return -1; }

    HostPlan &plan = C.plan;
    plan = HostPlan();
    if (!plan_layout(probs, n, plan, err, false)) return -1;  // bytes: checked by plan_fill

    bool want_path = false, want_post = false, want_bw = false;
    for (int q = 0; q < n; q++) {
        want_path |= outs[q].path != nullptr;
        want_post |= outs[q].posterior != nullptr;
        if (opt.backward && opt.backward[q]) want_bw = true;
    }
    want_post |= want_bw;
    TuneCfg cfg = E.defaults;
    const long long key = shape_key(plan, fp32, want_path);
    if (key_out) *key_out = key;
    if (opt.cfg) {
        cfg = *opt.cfg;
    } else {
        std::lock_guard<std::mutex> lock(E.tune_mu);
        auto it = E.tuned.find(key);
        if (it != E.tuned.end()) cfg = it->second;
    }

    if (!dry && !C.init) {
        int dc = 0;
        if (cudaGetDeviceCount(&dc) != cudaSuccess || dc == 0) {
            err = "no CUDA device: the threading HMM runs on the GPU only";
            return -2;
        }
        CK(cudaGetDevice(&C.device));
        CK(cudaStreamCreateWithFlags(&C.stream, cudaStreamNonBlocking));
        int lo = 0, hi = 0;
        CK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        for (int g = 0; g < MAXG; g++)
            CK(cudaStreamCreateWithPriority(&C.gstream[g], cudaStreamNonBlocking, hi));
        for (int i = 0; i < 8; i++) CK(cudaEventCreate(&C.ev[i]));
        for (int i = 0; i < 2 * MAXG + 2; i++)
            CK(cudaEventCreateWithFlags(&C.gev[i], cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&C.done, cudaEventDisableTiming));
        C.init = true;
    }
    cudaStream_t s = C.stream;

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
    const size_t o_last = in.add(want_path && opt.last_states ? sizeof(int) * plan.ninst : 0);
    const size_t in_bytes = in.total;

    char *h = C.host;
    std::vector<char> dry_stage;  // a dry run still fills the plan (variant counts) on the host
    if (dry) {
        dry_stage.resize(in_bytes);
        h = dry_stage.data();
        if (!plan_fill(probs, n, plan, PlanDst{(int *)(h + o_nodes), (int *)(h + o_map),
                                               (uint8_t *)(h + o_seq), (uint8_t *)(h + o_cls),
                                               (int *)(h + o_cvar)},
                       &err))
            return -1;
    } else {
        if (in_bytes > C.host_cap) {
            if (C.host) drop_host(C, C.host);
            C.host = nullptr;
            C.host_cap = 0;
            const size_t cap = in_bytes + in_bytes / 8;
            CK(cudaMallocHost(&C.host, cap));
            C.host_cap = cap;
        }

        // ---------------- stage inputs
        h = C.host;
        // per-node, per-column and sequence arrays straight into the staging buffer
        if (!plan_fill(probs, n, plan, PlanDst{(int *)(h + o_nodes), (int *)(h + o_map),
                                               (uint8_t *)(h + o_seq), (uint8_t *)(h + o_cls),
                                               (int *)(h + o_cvar)},
                       &err))
            return -1;
        memcpy(h + o_inst, plan.inst.data(), sizeof(InstDev) * plan.ninst);
        memcpy(h + o_blocks, plan.blocks.data(), sizeof(BlockDev) * plan.nblocks);
        memcpy(h + o_model, plan.model.data(), sizeof(double) * plan.model.size());
    }

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
           o_crow32 = 0, o_rstay32 = 0, o_lneref = 0, o_vref = 0,
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
        o_vref = w.add(sizeof(double) * std::max(plan.total_vcols, 1LL));
        o_blkext = w.add(sizeof(double) * plan.nblocks);
    }
    const size_t o_fw = w.add((fp32 ? sizeof(float) : sizeof(double)) * CELLS);
    const size_t o_lnl = w.add(sizeof(double) * plan.ninst);
    const size_t o_post = w.add(want_post ? sizeof(double) * CELLS : 0);
    const size_t o_bw = w.add(want_bw ? sizeof(double) * CELLS : 0);
    const size_t o_path = w.add(want_path ? sizeof(int) * COLS : 0);
    // FP32 traceback: the forward columns' time-bin sums
    const bool want_bins = fp32 && want_path && forward_writes_bins(plan.maxS, plan.maxM, plan.maxT, cfg.kpt);
    const size_t o_bins = w.add(want_bins ? sizeof(float) * MAXT * COLS : 0);
    const size_t o_err = w.add(4 * sizeof(int));
    const size_t o_queue = w.add(sizeof(int) * 2 * MAXG);  // work counters of the groups
    const size_t total = w.total;
    if (dry) {
        *dry_bytes = total;
        return 0;
    }

    if (C.ext) {
        if (total > C.ext_cap) {
            char b[200];
            snprintf(b, sizeof(b), "the batch needs %zu bytes of device memory; its region holds %zu",
                     total, C.ext_cap);
            err = b;
            return -5;
        }
    } else if (total > C.dev_cap) {
        if (C.dev) cudaFree(C.dev);
        C.dev = nullptr;
        C.dev_cap = 0;
        const size_t cap = total + total / 8;
        CK(cudaMalloc(&C.dev, cap));
        C.dev_cap = cap;
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
    if (want_path && opt.last_states) memcpy(h + o_last, opt.last_states, sizeof(int) * n);
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
    char *D = C.ext ? C.ext : C.dev;
    d.ninst = plan.ninst; d.nblocks = plan.nblocks; d.maxS = plan.maxS; d.maxT = plan.maxT;
    d.maxnodes = plan.maxnodes;
    d.maxM = plan.maxM;
    d.emit64 = 0;
    d.vardf = fp32 && varemit_full_carve_fits(plan.maxnodes, plan.maxS) ? 1 : 0;
    if (d.vardf) d.emit64 = 1;
    for (int i = 0; i < plan.ninst; i++)
        if (plan.inst[i].internal || plan.model[(size_t)i * MODEL_STRIDE + M_CONST + 3] < 1.0)
            d.emit64 = 1;
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
        d.vref = (double *)(D + o_vref);
        d.blkext = (double *)(D + o_blkext);
        d.fw32 = (float *)(D + o_fw);
    } else {
        d.fw64 = (double *)(D + o_fw);
    }
    d.lnl = (double *)(D + o_lnl);
    d.post = want_post ? (double *)(D + o_post) : nullptr;
    d.uniforms = want_path ? (const double *)(D + o_u) : nullptr;
    d.last_state = want_path && opt.last_states ? (const int *)(D + o_last) : nullptr;
    d.path = want_path ? (int *)(D + o_path) : nullptr;
    d.bins32 = want_bins ? (float *)(D + o_bins) : nullptr;
    d.err = (int *)(D + o_err);
    C.d = d;
    C.have_d = true;
    C.d_fp32 = fp32;
    C.o_u = o_u;

    // Schedule. Serial: per-tree kernels over the batch, then per-instance kernels. Pipelined
    // (larger batches): instances in groups, largest first; a group's per-tree kernels run
    // on the main stream and its forward (then traceback/backward) on high-priority streams
    // as soon as they are done, so the long per-instance chains start early and the
    // per-tree work of later groups fills the SMs they leave idle. The per-tree kernels are
    // persistent, work-stealing over units of trees; the device part of a step is captured
    // once as a CUDA graph and replayed while its launch parameters repeat.
    const bool special =
        opt.tables_only || opt.priors || opt.last_states || opt.dense || opt.dense_kind;
    const bool serial_timing = timing == 2;
    const bool pipelined = n >= 16 && !special && !serial_timing;
    const bool T = timing != 0;
    int *queues = (int *)(D + o_queue);
    if (T) CK(cudaEventRecord(C.ev[0], s));
    CK(cudaMemcpyAsync(D, h, in_bytes, cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(d.err, 0, 4 * sizeof(int), s));
    if (T) CK(cudaEventRecord(C.ev[1], s));

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
                cudaStream_t gs = C.gstream[g];
                EQ(cudaEventRecord(C.gev[2 * g], s));
                EQ(cudaStreamWaitEvent(gs, C.gev[2 * g], 0));
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
                EQ(cudaEventRecord(C.gev[2 * g + 1], gs));
            }
            for (int g = 0; g < ng; g++) EQ(cudaStreamWaitEvent(s, C.gev[2 * g + 1], 0));
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
        if (E.graphs && C.graphs) {
            // everything a launch depends on: buffers, counts, groups and schedule knobs
            std::vector<long long> sig = {(long long)(uintptr_t)D, (long long)fp32, want_path,
                                          want_post, want_bw, want_bins, plan.ninst, plan.nblocks,
                                          plan.maxS, plan.maxT, plan.maxnodes, plan.maxM,
                                          cfg.kpt, cfg.chunk, cfg.group_div, cfg.persistent, ng,
                                          (long long)total, d.emit64, d.vardf};
            for (size_t o : {o_inst, o_blocks, o_model, o_nodes, o_map, o_seq, o_cls, o_cvar,
                             o_order, o_blkmap, o_u, o_sinfo, o_t2off, o_btptr, o_btperm, o_tm,
                             o_gts, o_inv, o_det, o_detp, o_srcs, o_rrow, o_crow, o_gptr, o_gidx,
                             o_var, o_tm32, o_t2d32, o_inv32, o_var32, o_detp32, o_rrow32,
                             o_crow32, o_rstay32, o_lneref, o_vref, o_blkext, o_fw, o_lnl,
                             o_post, o_bw, o_path, o_bins, o_err, o_queue})
                sig.push_back((long long)o);
            for (int g = 0; g <= ng; g++) sig.push_back(bounds[g]);
            const int *ord = (const int *)(h + o_order);
            for (int j = 0; j < n && pipelined; j++) sig.push_back(plan.inst[ord[j]].ntrees);
            if (!(C.gexec && sig == C.gsig)) {
                if (C.gexec) cudaGraphExecDestroy(C.gexec);
                C.gexec = nullptr;
                C.gsig.clear();
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
                    cudaGraphInstantiateWithFlags(&C.gexec, graph, cudaGraphInstantiateFlagUseNodePriority);
                cudaGraphDestroy(graph);
                if (rc3 != cudaSuccess) {
                    C.gexec = nullptr;
                    return cuda_fail(rc3, "instantiating the step's graph");
                }
                C.gsig = std::move(sig);
                C.gkernels = kernel_launch_count() - before;
                E.graph_captures++;
            } else {
                for (long long q = 0; q < C.gkernels; q++) note_launch();
                E.graph_replays++;
            }
            CK(cudaGraphLaunch(C.gexec, s));
        } else {
            const cudaError_t rc = enqueue();
            if (rc != cudaSuccess) return cuda_fail(rc, "kernel launch");
        }
        if (T) CK(cudaEventRecord(C.ev[6], s));
    } else {
        launch_tables(d, fp32, s);
        CKL("table kernel");
        if (opt.dense_kind) {
            if (opt.dense_kind == DENSE_EMISSIONS) {
                launch_varemit(d, fp32, s);
                CKL("emission kernel");
            }
            const int rc = dense_tables(d, opt.dense_kind, opt.dense_rows, opt.dense_nrows,
                                        opt.dense_cols, opt.dense_ncols, opt.dense_ncolumns,
                                        opt.dense_out, s, err);
            return rc != 0 ? rc : 1;  // finished: nothing left for ctx_complete
        }
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
            return 1;  // finished: nothing left for ctx_complete
        }
        if (T) CK(cudaEventRecord(C.ev[2], s));
        launch_varemit(d, fp32, s);
        CKL("emission kernel");
        if (T) CK(cudaEventRecord(C.ev[3], s));
        if (opt.dense) launch_forward_dense(d, s);
        else launch_forward(d, fp32, s, cfg.kpt);
        CKL("forward kernel");
        if (T) CK(cudaEventRecord(C.ev[4], s));
        if (want_path) {
            launch_traceback(d, fp32, s);
            CKL("traceback kernel");
        }
        if (T) CK(cudaEventRecord(C.ev[5], s));
        if (want_post) {
            launch_backward(d, fp32, want_bw ? (double *)(D + o_bw) : nullptr, s);
            CKL("backward kernel");
        }
        if (T) CK(cudaEventRecord(C.ev[6], s));
    }

    // ---------------- downloads (asynchronous: into the page-locked output staging)
    C.copies.clear();
    size_t hout_bytes = 0;
    auto out_slot = [&](size_t bytes) {
        const size_t off = hout_bytes;
        hout_bytes += (bytes + 15) & ~(size_t)15;
        return off;
    };
    struct Pending {
        void *dst;
        const void *src;
        size_t bytes;
    };
    std::vector<Pending> pend;
    for (int q = 0; q < n; q++) {
        const InstDev &I = plan.inst[q];
        const long long cells = (q + 1 < n ? plan.inst[q + 1].cell0 : plan.total_cells) - I.cell0;
        const awg_outputs &o = outs[q];
        if (o.forward && !fp32) pend.push_back({o.forward, d.fw64 + I.cell0, sizeof(double) * cells});
        if (o.forward32 && fp32) pend.push_back({o.forward32, d.fw32 + I.cell0, sizeof(float) * cells});
        if (o.posterior) pend.push_back({o.posterior, d.post + I.cell0, sizeof(double) * cells});
        if (opt.backward && opt.backward[q])
            pend.push_back({opt.backward[q], (double *)(D + o_bw) + I.cell0, sizeof(double) * cells});
        if (o.path) pend.push_back({o.path, d.path + I.col0, sizeof(int) * I.seqlen});
        if (o.loglik) pend.push_back({o.loglik, d.lnl + q, sizeof(double)});
    }
    if (async) {
        for (const Pending &pd : pend) C.copies.push_back({pd.dst, out_slot(pd.bytes), pd.bytes});
    }
    C.err_off = out_slot(4 * sizeof(int));
    if (hout_bytes > C.hout_cap) {
        if (C.hout) drop_host(C, C.hout);
        C.hout = nullptr;
        C.hout_cap = 0;
        const size_t cap = std::max(hout_bytes + hout_bytes / 8, (size_t)256);
        CK(cudaMallocHost(&C.hout, cap));
        C.hout_cap = cap;
    }
    for (size_t i = 0; i < pend.size(); i++)
        CK(cudaMemcpyAsync(async ? (void *)(C.hout + C.copies[i].off) : pend[i].dst, pend[i].src,
                           pend[i].bytes, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(C.hout + C.err_off, d.err, 4 * sizeof(int), cudaMemcpyDeviceToHost, s));
    if (T) CK(cudaEventRecord(C.ev[7], s));
    CK(cudaEventRecord(C.done, s));
    C.timed = T;
    C.serial_phases = serial_timing || special;
    return 0;
}

// Waits for context C's last batch, records its timings, checks its device error record
// and (asynchronous batches) hands the outputs to the caller's buffers.
int ctx_complete(Ctx &C, std::string &err) {
    CK(cudaEventSynchronize(C.done));
    if (C.timed) {
        Timings t;
        cudaEventElapsedTime(&t.h2d_ms, C.ev[0], C.ev[1]);
        cudaEventElapsedTime(&t.compute_ms, C.ev[1], C.ev[6]);
        cudaEventElapsedTime(&t.d2h_ms, C.ev[6], C.ev[7]);
        if (C.serial_phases) {
            float ms[5];
            for (int i = 0; i < 5; i++) cudaEventElapsedTime(&ms[i], C.ev[i + 1], C.ev[i + 2]);
            t.tables_ms = ms[0]; t.emit_ms = ms[1]; t.forward_ms = ms[2];
            t.traceback_ms = ms[3]; t.backward_ms = ms[4];
        }
        C.last = t;
    }
    int dev_err[4];
    memcpy(dev_err, C.hout + C.err_off, sizeof(dev_err));
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
        C.copies.clear();
        return -4;
    }
    for (const Ctx::Copy &c : C.copies) memcpy(c.dst, C.hout + c.off, c.bytes);
    C.copies.clear();
    return 0;
}

Ctx *ctx_create() {
    Ctx *C = new Ctx();
    C->graphs = false;      // a server's batches rarely repeat a shape
    C->defer_free = true;   // and other batches are in flight when its staging grows
    return C;
}

int ctx_reserve_host(Ctx *C, size_t in_bytes, size_t out_bytes) {
    if (in_bytes > C->host_cap) {
        if (C->host) drop_host(*C, C->host);
        C->host = nullptr;
        C->host_cap = 0;
        if (cudaMallocHost(&C->host, in_bytes) != cudaSuccess) return -3;
        C->host_cap = in_bytes;
    }
    if (out_bytes > C->hout_cap) {
        if (C->hout) drop_host(*C, C->hout);
        C->hout = nullptr;
        C->hout_cap = 0;
        if (cudaMallocHost(&C->hout, out_bytes) != cudaSuccess) return -3;
        C->hout_cap = out_bytes;
    }
    return 0;
}

void ctx_destroy(Ctx *C) {
    if (!C) return;
    if (C->init) {
        cudaStreamSynchronize(C->stream);
        for (int g = 0; g < MAXG; g++) cudaStreamSynchronize(C->gstream[g]);
        if (C->gexec) cudaGraphExecDestroy(C->gexec);
        for (int g = 0; g < MAXG; g++) cudaStreamDestroy(C->gstream[g]);
        cudaStreamDestroy(C->stream);
        for (int i = 0; i < 8; i++) cudaEventDestroy(C->ev[i]);
        for (int i = 0; i < 2 * MAXG + 2; i++) cudaEventDestroy(C->gev[i]);
        cudaEventDestroy(C->done);
    }
    if (C->dev) cudaFree(C->dev);
    if (C->host) cudaFreeHost(C->host);
    if (C->hout) cudaFreeHost(C->hout);
    for (char *p : C->stale) cudaFreeHost(p);
    delete C;
}

void ctx_set_graphs(Ctx *C, bool on) { C->graphs = on; }

void ctx_set_region(Ctx *C, char *dev, size_t bytes) {
    C->ext = dev;
    C->ext_cap = bytes;
}

bool ctx_ready(Ctx *C) { return cudaEventQuery(C->done) == cudaSuccess; }

void ctx_sync(Ctx *C) {
    if (!C->init) return;
    cudaStreamSynchronize(C->stream);
    for (int g = 0; g < MAXG; g++) cudaStreamSynchronize(C->gstream[g]);
}

int ctx_launch_async(Ctx *C, const awg_problem *probs, awg_outputs *outs, int n, int precision,
                     std::string &err) {
    RunOptions opt;
    opt.precision = precision;
    return ctx_launch(*C, probs, outs, n, opt, true, 0, nullptr, err, nullptr);
}

int ctx_finish(Ctx *C, std::string &err) { return ctx_complete(*C, err); }

long long batch_device_bytes(const awg_problem *probs, int n, int precision, bool path,
                             bool posterior, std::string &err) {
    Ctx tmp;
    std::vector<awg_outputs> outs(n);
    static double sink;
    for (auto &o : outs) {
        memset(&o, 0, sizeof(o));
        if (path) o.path = (int *)&sink;  // never written: only the wanted outputs count
        if (posterior) o.posterior = &sink;
    }
    RunOptions opt;
    opt.precision = precision;
    size_t bytes = 0;
    const int rc = ctx_launch(tmp, probs, outs.data(), n, opt, false, 0, nullptr, err, &bytes);
    return rc != 0 ? rc : (long long)bytes;
}

// Draws new paths from context C's last batch: its forward tables (and FP32 bin sums) are
// still on the device, so only the uniforms go up and only the traceback runs.
int ctx_resample(Ctx *C, const double *const *uniforms, int *const *paths, std::string &err) {
    if (!C->have_d || !C->d.path || !C->d.uniforms) {
        err = "the context's last batch drew no paths";
        return -1;
    }
    const HostPlan &plan = C->plan;
    cudaStream_t s = C->stream;
    CK(cudaEventSynchronize(C->done));  // the staging buffers are free
    double *u = (double *)(C->host + C->o_u);
    for (int q = 0; q < plan.ninst; q++) {
        const InstDev &I = plan.inst[q];
        if (uniforms && uniforms[q]) {
            memcpy(u + I.col0, uniforms[q], sizeof(double) * I.seqlen);
        } else {
            for (int c = I.seqlen - 1; c >= 0; c--) u[I.col0 + c] = rand() / double(RAND_MAX);
        }
    }
    CK(cudaMemcpyAsync((void *)C->d.uniforms, u, sizeof(double) * std::max(plan.total_cols, 1LL),
                       cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(C->d.err, 0, 4 * sizeof(int), s));
    launch_traceback(C->d, C->d_fp32, s);
    CK(cudaGetLastError());
    C->copies.clear();
    size_t off = 16;  // the error record first
    for (int q = 0; q < plan.ninst; q++) {
        const InstDev &I = plan.inst[q];
        if (!paths || !paths[q]) continue;
        const size_t bytes = sizeof(int) * I.seqlen;
        C->copies.push_back({paths[q], off, bytes});
        off += (bytes + 15) & ~(size_t)15;
    }
    if (off > C->hout_cap) {
        if (C->hout) drop_host(*C, C->hout);
        C->hout = nullptr;
        C->hout_cap = 0;
        CK(cudaMallocHost(&C->hout, off + off / 8));
        C->hout_cap = off + off / 8;
    }
    C->err_off = 0;
    CK(cudaMemcpyAsync(C->hout, C->d.err, 4 * sizeof(int), cudaMemcpyDeviceToHost, s));
    int k = 0;
    for (int q = 0; q < plan.ninst; q++) {
        if (!paths || !paths[q]) continue;
        CK(cudaMemcpyAsync(C->hout + C->copies[k].off, C->d.path + plan.inst[q].col0,
                           C->copies[k].bytes, cudaMemcpyDeviceToHost, s));
        k++;
    }
    CK(cudaEventRecord(C->done, s));
    C->timed = false;
    return ctx_complete(*C, err);
}

int run_batch(const awg_problem *probs, awg_outputs *outs, int n, const RunOptions &opt,
              std::string &err) {
    Engine &E = engine();
    std::lock_guard<std::mutex> lock(E.mu);
    long long key = -1;
    const int rc = ctx_launch(E.ctx, probs, outs, n, opt, false, E.timing, &key, err, nullptr);
    E.last_key = key;
    if (rc == 1) return 0;  // a debug or dense-table call that finished inside the launch
    if (rc != 0) {
        if (E.ctx.init) cudaStreamSynchronize(E.ctx.stream);  // nothing left in flight
        return rc;
    }
    return ctx_complete(E.ctx, err);
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
            ms = std::min(ms, (double)E.ctx.last.compute_ms);
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
        std::lock_guard<std::mutex> lock(E.tune_mu);
        E.tuned[key] = best;
    }
    return 0;
}

}  // namespace awg

extern "C" {

// Frees the engine's device arena, page-locked staging and captured graph (the next batch
// allocates again); returns 0.
int awg_release_memory(void) {
    awg::Engine &E = awg::engine();
    std::lock_guard<std::mutex> lock(E.mu);
    awg::Ctx &C = E.ctx;
    if (C.init) cudaStreamSynchronize(C.stream);
    if (C.gexec) cudaGraphExecDestroy(C.gexec);
    C.gexec = nullptr;
    C.gsig.clear();
    if (C.dev) cudaFree(C.dev);
    C.dev = nullptr;
    C.dev_cap = 0;
    if (C.host) cudaFreeHost(C.host);
    C.host = nullptr;
    C.host_cap = 0;
    if (C.hout) cudaFreeHost(C.hout);
    C.hout = nullptr;
    C.hout_cap = 0;
    C.have_d = false;
    return 0;
}

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
    std::lock_guard<std::mutex> tl(E.tune_mu);
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
    const auto &t = awg::engine().ctx.last;
    const float v[8] = {t.h2d_ms, t.tables_ms, t.emit_ms, t.forward_ms, t.traceback_ms,
                        t.backward_ms, t.d2h_ms, t.compute_ms};
    for (int i = 0; i < 8; i++) out8[i] = v[i];
}

}  // extern "C"

// Forward algorithm of one problem with every device buffer carved out of one file-scope
// device array: no cudaMalloc, no cudaFree, no page-locked host memory, no memory pool.
//
// The kernels are the batch engine's (K1 tables, K2 variant emissions, K3 forward), launched
// unchanged over a one-problem plan; only where their buffers live differs. The array sits
// in this translation unit alone, so a process that never calls awg_forward_static never
// loads it (the CUDA runtime loads modules lazily by default).

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "engine.h"
#include "kernels.h"
#include "plan.h"

namespace awg {

namespace {

constexpr size_t SCRATCH_BYTES = AWG_STATIC_SCRATCH_BYTES;
constexpr int MAX_DEVICES = 64;

__device__ __align__(256) unsigned char g_scratch[SCRATCH_BYTES];

// Device address of g_scratch. The first call on a device (that device current) loads the
// module holding the array; every call then resolves the address again, because a context
// destroyed and recreated in between (cudaDeviceReset) reloads the module and may move it.
std::mutex g_setup_mu;

struct Carve {
    size_t total = 0;
    size_t add(size_t bytes) {
        const size_t off = total;
        total += (bytes + 255) & ~size_t(255);
        return off;
    }
};

}  // namespace

int run_static(const awg_problem *p, awg_outputs *out, int precision, cudaStream_t s,
               std::string &err) {
    const bool fp32 = precision == AWG_FP32;
    if (!fp32 && precision != AWG_FP64) { err = "precision must be AWG_FP64 or AWG_FP32"; return -1; }
    if (!p || !out) { err = "NULL problem or outputs"; return -1; }
    if (out->path || out->posterior) {
        err = "awg_forward_static computes the forward table and log-likelihood only: "
              "path and posterior must be NULL";
        return -1;
    }
    if ((out->forward && fp32) || (out->forward32 && !fp32)) {
        err = "forward is the AWG_FP64 table and forward32 the AWG_FP32 one";
        return -1;
    }

    HostPlan plan;
    if (!build_plan(p, 1, plan, err)) return -1;

    // ---------------- carve the scratch (same regions as the batch engine's arena)
    const long long ST = std::max(plan.total_states, 1LL);
    const long long CELLS = std::max(plan.total_cells, 1LL);
    Carve c;
    const size_t o_inst = c.add(sizeof(InstDev) * plan.ninst);
    const size_t o_blocks = c.add(sizeof(BlockDev) * plan.nblocks);
    const size_t o_model = c.add(sizeof(double) * plan.model.size());
    const size_t o_nodes = c.add(sizeof(int) * plan.nodes.size());
    const size_t o_map = c.add(sizeof(int) * plan.mapping.size());
    const size_t o_seq = c.add(plan.seqT.size());
    const size_t o_cls = c.add(plan.colclass.size());
    const size_t o_cvar = c.add(sizeof(int) * plan.colvar.size());
    const size_t o_sinfo = c.add(sizeof(StateInfo) * ST);
    const size_t o_t2off = c.add(sizeof(int) * ST);
    const size_t o_btptr = c.add(sizeof(int) * (size_t)plan.nblocks * (MAXT + 1));
    const size_t o_btperm = c.add(sizeof(int) * ST);
    const size_t o_tm = c.add(sizeof(double) * (size_t)plan.nblocks * MAXT * MAXT);
    const size_t o_gts = c.add(sizeof(double) * std::max(plan.total_M, 1LL));
    const size_t o_inv = c.add(sizeof(double) * ST);
    const size_t o_det = c.add(sizeof(int) * ST);
    const size_t o_detp = c.add(sizeof(double) * ST);
    const size_t o_srcs = c.add(sizeof(int2) * plan.nblocks);
    const size_t o_rrow = c.add(sizeof(double) * ST);
    const size_t o_crow = c.add(sizeof(double) * ST);
    const size_t o_gptr = c.add(sizeof(int) * (ST + plan.nblocks + 1));
    const size_t o_gidx = c.add(sizeof(int) * ST);
    const size_t o_var = c.add(sizeof(double) * std::max(plan.total_var, 1LL));
    size_t o_tm32 = 0, o_t2d32 = 0, o_inv32 = 0, o_var32 = 0, o_detp32 = 0, o_rrow32 = 0,
           o_crow32 = 0, o_rstay32 = 0, o_lneref = 0, o_vref = 0,
           o_blkext = 0;
    if (fp32) {
        o_tm32 = c.add(sizeof(float) * (size_t)plan.nblocks * MAXT * MAXT);
        o_t2d32 = c.add(sizeof(float) * std::max(plan.total_M, 1LL));
        o_inv32 = c.add(sizeof(float) * ST);
        o_var32 = c.add(sizeof(float) * std::max(plan.total_var, 1LL));
        o_detp32 = c.add(sizeof(float) * ST);
        o_rrow32 = c.add(sizeof(float) * ST);
        o_crow32 = c.add(sizeof(float) * ST);
        o_rstay32 = c.add(sizeof(float) * (size_t)plan.nblocks * MAXT);
        o_lneref = c.add(sizeof(double) * plan.nblocks);
        o_vref = c.add(sizeof(double) * std::max(plan.total_vcols, 1LL));
        o_blkext = c.add(sizeof(double) * plan.nblocks);
    }
    const size_t o_fw = c.add((fp32 ? sizeof(float) : sizeof(double)) * CELLS);
    const size_t o_lnl = c.add(sizeof(double));
    const size_t o_err = c.add(4 * sizeof(int));
    if (c.total > SCRATCH_BYTES) {
        char b[256];
        snprintf(b, sizeof(b),
                 "awg_forward_static: the problem needs %zu bytes of device scratch (%lld "
                 "forward cells, %d trees); the static scratch holds %zu bytes",
                 c.total, plan.total_cells, plan.nblocks, SCRATCH_BYTES);
        err = b;
        return -5;
    }

    // ---------------- the scratch's device address in the current context
    int dev = -1, ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        err = "no CUDA device: the threading HMM runs on the GPU only";
        return -2;
    }
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) {
        err = "awg_forward_static: no usable current device";
        return -2;
    }
    char *D;
    {
        std::lock_guard<std::mutex> lock(g_setup_mu);
        void *ptr = nullptr;
        const cudaError_t rc = cudaGetSymbolAddress(&ptr, g_scratch);
        if (rc != cudaSuccess || !ptr) {
            err = std::string("awg_forward_static: cudaGetSymbolAddress of the static "
                              "scratch failed: ") + cudaGetErrorString(rc);
            return -3;
        }
        D = (char *)ptr;
    }

    BatchDev d;
    memset(&d, 0, sizeof(d));
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
    d.err = (int *)(D + o_err);

    // On an error after work was enqueued, the stream is drained before returning, so no
    // work of this call is left running on the shared array.
#define SCK(x)                                                                        \
    do {                                                                              \
        const cudaError_t rc_ = (x);                                                  \
        if (rc_ != cudaSuccess) {                                                     \
            err = std::string("awg_forward_static: " #x ": ") + cudaGetErrorString(rc_); \
            (void)cudaStreamSynchronize(s);                                           \
            return -3;                                                                \
        }                                                                             \
    } while (0)

    // inputs straight from the plan's (pageable) host arrays; only the error record must
    // start at zero, every other region is written before it is read
    auto up = [&](size_t off, const void *src, size_t bytes) {
        return bytes ? cudaMemcpyAsync(D + off, src, bytes, cudaMemcpyHostToDevice, s)
                     : cudaSuccess;
    };
    SCK(up(o_inst, plan.inst.data(), sizeof(InstDev) * plan.ninst));
    SCK(up(o_blocks, plan.blocks.data(), sizeof(BlockDev) * plan.nblocks));
    SCK(up(o_model, plan.model.data(), sizeof(double) * plan.model.size()));
    SCK(up(o_nodes, plan.nodes.data(), sizeof(int) * plan.nodes.size()));
    SCK(up(o_map, plan.mapping.data(), sizeof(int) * plan.mapping.size()));
    SCK(up(o_seq, plan.seqT.data(), plan.seqT.size()));
    SCK(up(o_cls, plan.colclass.data(), plan.colclass.size()));
    SCK(up(o_cvar, plan.colvar.data(), sizeof(int) * plan.colvar.size()));
    SCK(cudaMemsetAsync(d.err, 0, 4 * sizeof(int), s));

    launch_tables(d, fp32, s);
    SCK(cudaGetLastError());
    launch_varemit(d, fp32, s);
    SCK(cudaGetLastError());
    launch_forward(d, fp32, s);
    SCK(cudaGetLastError());

    const long long cells = plan.total_cells;
    if (out->forward)
        SCK(cudaMemcpyAsync(out->forward, d.fw64, sizeof(double) * cells, cudaMemcpyDeviceToHost, s));
    if (out->forward32)
        SCK(cudaMemcpyAsync(out->forward32, d.fw32, sizeof(float) * cells, cudaMemcpyDeviceToHost, s));
    double lnl = 0.0;
    int dev_err[4] = {0, 0, 0, 0};
    SCK(cudaMemcpyAsync(&lnl, d.lnl, sizeof(double), cudaMemcpyDeviceToHost, s));
    SCK(cudaMemcpyAsync(dev_err, d.err, 4 * sizeof(int), cudaMemcpyDeviceToHost, s));
    SCK(cudaStreamSynchronize(s));
#undef SCK
    if (dev_err[0] != 0) {
        char b[160];
        snprintf(b, sizeof(b), "awg_forward_static: device error %d at tree %d, column %d",
                 dev_err[0], dev_err[2], dev_err[3]);
        err = b;
        return -4;
    }
    if (out->loglik) *out->loglik = lnl;
    return 0;
}

}  // namespace awg

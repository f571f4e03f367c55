// The batch engine: plan -> one upload -> table, emission, forward, traceback and backward
// kernels -> downloads. One engine per process and device; calls are serialised.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "argweaver_gb300.h"

namespace awg {

// Schedule knobs of a batch, chosen by the autotuner (awg_autotune) per shape class.
struct TuneCfg {
    int kpt = 0;         // forward: states per owner thread (0: chosen by the state count)
    int chunk = 1;       // trees per work unit of the persistent per-tree kernels
    int group_div = 8;   // pipelined schedule: the largest instance group holds n / group_div
    int persistent = 1;  // per-tree kernels as persistent work-stealing kernels
};

struct RunOptions {
    const TuneCfg *cfg = nullptr;  // explicit schedule (the autotuner's trials), else tuned
    int precision = AWG_FP64;
    const double *const *priors = nullptr;  // per problem: given column-0 prior, or NULL
    bool dense = false;                     // forward by the dense S x S step (FP64)
    const int *last_states = nullptr;       // per problem: the traceback's given last state
                                            // (FP64 only), or -1 to sample it
    double *const *backward = nullptr;      // per problem: backward table output, or NULL
    // Dense helper matrices (dense_tables, kernels.h) of problem 0, FP64: kind 1-3, the
    // state indices of the rows and columns, the columns of an emission matrix, the host
    // output; the batch stops after them
    int dense_kind = 0;
    const int *dense_rows = nullptr, *dense_cols = nullptr;
    int dense_nrows = 0, dense_ncols = 0, dense_ncolumns = 0;
    double *dense_out = nullptr;
    // Debug: stop after the table kernel and copy its FP64 tables of problem 0 out:
    // tmatrix [ntrees][T-1][T-1], same-branch rows [sum M], invariant emissions
    // [sum max(S,1)], column-0 prior [max(S0,1)].
    bool tables_only = false;
    double *dbg_tm = nullptr, *dbg_gts = nullptr, *dbg_inv = nullptr, *dbg_prior = nullptr;
    int *dbg_btptr = nullptr, *dbg_btperm = nullptr;  // [ntrees][MAXT+1], [sum max(S,1)]
};

// Runs a batch; returns 0 or a negative code with err set.
int run_batch(const awg_problem *probs, awg_outputs *outs, int n, const RunOptions &opt,
              std::string &err);

// Times the candidate schedules on this batch (each run `trials` times, the fastest kept)
// and records the best for the batch's shape class; later batches of the class use it.
int autotune(const awg_problem *probs, awg_outputs *outs, int n, int precision, int trials,
             TuneCfg &best, double &best_ms, std::string &err);

// Execution contexts for callers that keep several batches in flight (the server): each
// has its own streams, page-locked staging and either a grow-only device arena or a region
// the owner hands it. A context runs one batch at a time: launch, then finish (which waits).
struct Ctx;
Ctx *ctx_create();
void ctx_destroy(Ctx *C);
void ctx_set_region(Ctx *C, char *dev, size_t bytes);
// Capture each step as a CUDA graph and replay it while its shape repeats (off by default
// for contexts made here: a server's batches rarely repeat a shape).
void ctx_set_graphs(Ctx *C, bool on);
// Page-locked input and output staging of at least these sizes, allocated now.
int ctx_reserve_host(Ctx *C, size_t in_bytes, size_t out_bytes);
int ctx_launch_async(Ctx *C, const awg_problem *probs, awg_outputs *outs, int n, int precision,
                     std::string &err);
bool ctx_ready(Ctx *C);  // the launched batch's outputs have arrived
void ctx_sync(Ctx *C);   // everything enqueued on the context has finished
int ctx_finish(Ctx *C, std::string &err);
// New paths from the context's last batch (paths wanted), its forward tables still resident:
// uniforms[q] per problem (NULL: libc rand()), paths[q] per problem (NULL: not wanted).
int ctx_resample(Ctx *C, const double *const *uniforms, int *const *paths, std::string &err);
// Device bytes a batch needs (the engine's layout), or a negative code with err set.
long long batch_device_bytes(const awg_problem *probs, int n, int precision, bool path,
                             bool posterior, std::string &err);

// Forward table and log-likelihood of one problem with every device buffer in a static
// device array (no allocation); returns 0 or a negative code with err set.
int run_static(const awg_problem *p, awg_outputs *out, int precision, cudaStream_t s,
               std::string &err);

}  // namespace awg

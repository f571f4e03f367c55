// The batch engine: plan -> one upload -> table, emission, forward, traceback and backward
// kernels -> downloads. One engine per process and device; calls are serialised.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "argweaver_gb300.h"

namespace awg {

struct RunOptions {
    int precision = AWG_FP64;
    const double *const *priors = nullptr;  // per problem: given column-0 prior, or NULL
    double *const *backward = nullptr;      // per problem: backward table output, or NULL
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

// Forward table and log-likelihood of one problem with every device buffer in a static
// device array (no allocation); returns 0 or a negative code with err set.
int run_static(const awg_problem *p, awg_outputs *out, int precision, cudaStream_t s,
               std::string &err);

}  // namespace awg

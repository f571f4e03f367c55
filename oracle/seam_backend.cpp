// Test infrastructure: the C-ABI entry points the C++ seam (argweaver_gb300/seam/
// sample_thread_gpu.cpp) calls, served by the oracle (awg_oracle.cpp) on the CPU, so that a
// relinked arg-sample can run where there is no GPU. It checks the seam's marshalling of the
// reference's objects and its rand() order; the CUDA path is held to the oracle by the GPU
// parity tests on the same problems.
//
// awg_run_batch here: FP64 only, forward table and/or sampled path; NULL uniforms draw
// rand()/RAND_MAX for columns L-1 down to 0, as the library does (stochastic_traceback,
// sample_thread.cpp:522-569, draws one rand() per column, last column first).

#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "argweaver_gb300.h"
#include "awg_oracle.h"

namespace {

thread_local std::string g_err;

oracle_problem to_oracle(const awg_problem *p) {
    oracle_problem o;
    std::memset(&o, 0, sizeof(o));
    o.ntrees = p->ntrees;
    o.nnodes = p->nnodes;
    o.ntimes = p->ntimes;
    o.nseqs = p->nseqs;
    o.seqlen = p->seqlen;
    o.internal = p->internal;
    o.start_coord = p->start_coord;
    o.minage = p->minage;
    o.ptrees = p->ptrees;
    o.ages = p->ages;
    o.sprs = p->sprs;
    o.blocklens = p->blocklens;
    o.mapping = p->mapping;
    o.root_child0 = p->root_child0;
    o.times = p->times;
    o.popsizes = p->popsizes;
    o.rho = p->rho;
    o.mu = p->mu;
    o.seqs = p->seqs;
    o.infsites_penalty = p->infsites_penalty;
    return o;
}

}  // namespace

extern "C" {

const char *awg_last_error(void) { return g_err.c_str(); }

long long awg_problem_cells(const awg_problem *p) {
    const oracle_problem o = to_oracle(p);
    return oracle_cells(&o);
}

int awg_run_batch(const awg_problem *problems, awg_outputs *outputs, int n, int precision) {
    g_err.clear();
    if (precision != AWG_FP64) {
        g_err = "the oracle backend computes in FP64 only";
        return -1;
    }
    for (int q = 0; q < n; q++) {
        const oracle_problem o = to_oracle(&problems[q]);
        const long long cells = oracle_cells(&o);
        if (cells < 0) {
            g_err = "the oracle rejected the problem";
            return -1;
        }
        std::vector<double> fw((size_t)cells);
        double lnl = 0.0;
        if (oracle_forward(&o, fw.data(), &lnl) != 0) {
            g_err = "oracle forward failed";
            return -2;
        }
        awg_outputs &out = outputs[q];
        if (out.forward) std::memcpy(out.forward, fw.data(), sizeof(double) * cells);
        if (out.loglik) *out.loglik = lnl;
        if (out.path) {
            const int L = o.seqlen;
            std::vector<double> u(L);
            if (out.uniforms) {
                std::memcpy(u.data(), out.uniforms, sizeof(double) * L);
            } else {
                for (int i = L - 1; i >= 0; i--) u[i] = rand() / (double)RAND_MAX;
            }
            if (oracle_traceback(&o, fw.data(), u.data(), out.path) != 0) {
                g_err = "oracle traceback failed";
                return -2;
            }
        }
    }
    return 0;
}

int awg_sample_path_conditioned(const awg_problem *p, const double *prior, int last_state,
                                const double *uniforms, int *path, double *loglik) {
    g_err.clear();
    const oracle_problem o = to_oracle(p);
    const long long cells = oracle_cells(&o);
    if (cells < 0) {
        g_err = "the oracle rejected the problem";
        return -1;
    }
    std::vector<double> fw((size_t)cells);
    double lnl = 0.0;
    if (oracle_forward_prior(&o, prior, fw.data(), &lnl) != 0) {
        g_err = "oracle forward failed";
        return -2;
    }
    if (loglik) *loglik = lnl;
    const int L = o.seqlen;
    std::vector<double> u(L, 0.0);
    if (uniforms) {
        std::memcpy(u.data(), uniforms, sizeof(double) * L);
    } else {
        for (int i = L - (last_state >= 0 ? 2 : 1); i >= 0; i--) u[i] = rand() / (double)RAND_MAX;
    }
    if (oracle_traceback_last(&o, fw.data(), u.data(), nullptr, last_state, path) != 0) {
        g_err = "oracle traceback failed";
        return -2;
    }
    return 0;
}

}  // extern "C"

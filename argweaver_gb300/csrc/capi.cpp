// The C ABI: the reference's threading-HMM entry points (sample_thread.cpp:883-1046,
// states.cpp:209, local_tree.cpp:1817-1895) re-hosted on the GPU engine, and the flat
// batch API. Results of the reference-compatible calls are host memory allocated with
// new[], as the reference's are, and are freed by this library's delete_* exports.

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "argweaver_gb300.h"
#include "engine.h"
#include "kernels.h"
#include "plan.h"
#include "arg_surgery.h"
#include "formats.h"

struct awg_local_trees {
    int ntrees = 0, nnodes = 0, start_coord = 0;
    // mapping: from the previous tree (empty: the default); c0, c1: children in the order
    // the trees keep them after surgery (empty: index order); seqids: the sequence each
    // leaf holds (LocalTrees::seqids, local_tree.h:673; empty: leaf i holds sequence i)
    std::vector<int> ptrees, ages, sprs, blocklens, mapping, c0, c1, seqids;
};

namespace {

thread_local std::string g_err;

void set_error(const std::string &msg) {
    g_err = msg;
    fprintf(stderr, "argweaver_gb300: %s\n", msg.c_str());
}

// Trees + model + sequences of a reference-style call as one awg_problem.
struct ProblemView {
    awg_problem p;
    std::vector<char> seqs;
    std::vector<int> root_child0;
};

// The leaf names the reference's exports show (get_local_trees_ptrees, local_tree.cpp:
// 1847-1857): leaf i is named seqids[i], internal nodes keep theirs. False when the names
// are the stored ones (default ids, or ids that are no permutation of the leaves, which the
// reference cannot show either).
bool leaf_perm(const awg_local_trees *t, std::vector<int> &perm) {
    const int n = t->nnodes, nleaves = (n + 1) / 2;
    if (t->seqids.empty() || (int)t->seqids.size() != nleaves) return false;
    perm.assign(n, 0);
    std::vector<char> seen(nleaves, 0);
    bool identity = true;
    for (int i = 0; i < nleaves; i++) {
        const int s = t->seqids[i];
        if (s < 0 || s >= nleaves || seen[s]) return false;
        seen[s] = 1;
        perm[i] = s;
        identity = identity && s == i;
    }
    for (int i = nleaves; i < n; i++) perm[i] = i;
    return !identity;
}

bool make_view(const awg_local_trees *t, double *times, int ntimes, double *popsizes,
               double rho, double mu, char **seqs, int nseqs, int seqlen, bool internal,
               ProblemView &v, const std::vector<int> *row_list = nullptr) {
    if (!t || !times || !popsizes || !seqs) { set_error("NULL argument"); return false; }
    // leaf i reads sequence seqids[i] (matrices.cpp:34, total_prob.cpp:32); the rows after
    // the leaves are the last sequences, in order (the thread's new_chrom = nseqs - 1)
    const int nleaves = (t->nnodes + 1) / 2;
    std::vector<int> rows(nseqs);
    for (int i = 0; i < nseqs; i++) rows[i] = i;
    if (!t->seqids.empty() && nseqs >= nleaves) {
        for (int i = 0; i < nleaves; i++) {
            if (t->seqids[i] < 0 || t->seqids[i] >= nseqs) {
                set_error("a leaf's sequence id is past the sequences given");
                return false;
            }
            rows[i] = t->seqids[i];
        }
    }
    if (row_list) {  // the caller's rows (sequence ids), in leaf order then the new one
        rows = *row_list;
        nseqs = (int)rows.size();
    }
    v.seqs.resize((size_t)nseqs * seqlen);
    for (int i = 0; i < nseqs; i++) memcpy(&v.seqs[(size_t)i * seqlen], seqs[rows[i]], seqlen);
    awg_problem &p = v.p;
    memset(&p, 0, sizeof(p));
    p.ntrees = t->ntrees; p.nnodes = t->nnodes; p.ntimes = ntimes; p.nseqs = nseqs;
    p.seqlen = seqlen; p.internal = internal ? 1 : 0; p.start_coord = t->start_coord;
    p.minage = 0;
    p.ptrees = t->ptrees.data(); p.ages = t->ages.data(); p.sprs = t->sprs.data();
    p.blocklens = t->blocklens.data();
    p.mapping = t->mapping.empty() ? nullptr : t->mapping.data();
    p.root_child0 = nullptr;
    if (internal && !t->c0.empty()) {  // each root's child[0] is the cut subtree
        const int n = t->nnodes;
        v.root_child0.assign(t->ntrees, -1);
        for (int b = 0; b < t->ntrees; b++)
            for (int i = 0; i < n; i++)
                if (t->ptrees[(size_t)b * n + i] == -1) v.root_child0[b] = t->c0[(size_t)b * n + i];
        p.root_child0 = v.root_child0.data();
    }
    p.times = times; p.popsizes = popsizes; p.rho = rho; p.mu = mu;
    p.seqs = v.seqs.data();
    return true;
}

// seqlen rows of max(nstates,1) doubles over one new[] block; the block pointer is kept in
// a hidden slot before the row array so delete_forward_matrix can free it.
double **make_rows(const std::vector<int> &nstates, double **block_out) {
    const int L = (int)nstates.size();
    long long cells = 0;
    for (int i = 0; i < L; i++) cells += std::max(nstates[i], 1);
    double *block = new double[std::max(cells, 1LL)];
    double **rows = new double *[L + 1];
    rows[0] = block;
    long long off = 0;
    for (int i = 0; i < L; i++) {
        rows[i + 1] = block + off;
        off += std::max(nstates[i], 1);
    }
    *block_out = block;
    return rows + 1;
}

std::vector<int> column_nstates(const awg_problem &p) {
    std::vector<int> ns(p.seqlen, 0);
    int pos = 0;
    for (int b = 0; b < p.ntrees; b++) {
        int S = awg::count_states(p.ptrees + (size_t)b * p.nnodes, p.ages + (size_t)b * p.nnodes,
                                  p.nnodes, p.ntimes, p.internal != 0, p.minage,
                                  p.root_child0 ? p.root_child0[b] : -1, nullptr);
        for (int i = 0; i < p.blocklens[b]; i++) ns[pos + i] = S;
        pos += p.blocklens[b];
    }
    return ns;
}

double **table_call(awg_local_trees *trees, double *times, int ntimes, double *popsizes,
                    double rho, double mu, char **seqs, int nseqs, int seqlen, bool internal,
                    const double *prior, int kind, bool dense = false) {
    g_err.clear();
    ProblemView v;
    if (!make_view(trees, times, ntimes, popsizes, rho, mu, seqs, nseqs, seqlen, internal, v))
        return nullptr;
    if (awg_problem_cells(&v.p) < 0) return nullptr;
    std::vector<int> ns = column_nstates(v.p);
    double *block = nullptr;
    double **rows = make_rows(ns, &block);
    awg_outputs o;
    memset(&o, 0, sizeof(o));
    awg::RunOptions opt;
    opt.precision = AWG_FP64;
    const double *priors[1] = {prior};
    double *bws[1] = {block};
    if (kind == 0) o.forward = block;
    if (kind == 1) { opt.backward = bws; }
    if (kind == 2) o.posterior = block;
    if (prior) opt.priors = priors;
    opt.dense = dense;
    std::string err;
    if (awg::run_batch(&v.p, &o, 1, opt, err) != 0) {
        set_error(err);
        delete[] block;
        delete[] (rows - 1);
        return nullptr;
    }
    return rows;
}

}  // namespace

extern "C" {

const char *awg_last_error(void) { return g_err.c_str(); }

int awg_sample_path_conditioned(const awg_problem *p, const double *prior, int last_state,
                                const double *uniforms, int *path, double *loglik) {
    g_err.clear();
    if (!p || !path) {
        g_err = "awg_sample_path_conditioned: NULL problem or path";
        return -1;
    }
    if (awg_problem_cells(p) < 0) return -1;
    if (last_state >= 0) {
        const int b = p->ntrees - 1;
        const int S = awg::count_states(p->ptrees + (size_t)b * p->nnodes,
                                        p->ages + (size_t)b * p->nnodes, p->nnodes, p->ntimes,
                                        p->internal != 0, p->minage,
                                        p->root_child0 ? p->root_child0[b] : -1, nullptr);
        if (last_state >= std::max(S, 1)) {
            g_err = "awg_sample_path_conditioned: last_state " + std::to_string(last_state) +
                    " is not a state of the last tree (" + std::to_string(std::max(S, 1)) + ")";
            return -1;
        }
    }
    awg_outputs o;
    memset(&o, 0, sizeof(o));
    o.path = path;
    o.loglik = loglik;
    std::vector<double> u;
    if (uniforms) {
        o.uniforms = uniforms;
    } else {
        // the reference's draws: one rand() per column, last column first; a given last
        // state takes none (stochastic_traceback, sample_thread.cpp:532-539)
        u.assign(p->seqlen, 0.0);
        for (int c = p->seqlen - (last_state >= 0 ? 2 : 1); c >= 0; c--) u[c] = rand() / double(RAND_MAX);
        o.uniforms = u.data();
    }
    awg::RunOptions opt;
    opt.precision = AWG_FP64;
    const double *priors[1] = {prior};
    if (prior) opt.priors = priors;
    const int last[1] = {last_state};
    opt.last_states = last;
    std::string err;
    const int rc = awg::run_batch(p, &o, 1, opt, err);
    if (rc != 0) set_error(err);
    return rc;
}

long long awg_kernel_launches(void) { return awg::kernel_launch_count(); }

int awg_device_name(char *buf, int len) {
    int dev = 0;
    cudaDeviceProp prop;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess)
        return -1;
    snprintf(buf, len, "%s", prop.name);
    return 0;
}

long long awg_problem_cells(const awg_problem *p) {
    g_err.clear();
    awg::HostPlan plan;
    std::string err;
    if (!p || !awg::plan_layout(p, 1, plan, err, true)) {
        set_error(err.empty() ? "NULL problem" : err);
        return -1;
    }
    return plan.total_cells;
}

int awg_problems_cells(const awg_problem *problems, int n, long long *cells) {
    g_err.clear();
    awg::HostPlan plan;
    std::string err;
    if (!problems || !cells || !awg::plan_layout(problems, n, plan, err, false)) {
        set_error(err.empty() ? "NULL argument" : err);
        return -1;
    }
    for (int q = 0; q < n; q++)
        cells[q] = (q + 1 < n ? plan.inst[q + 1].cell0 : plan.total_cells) - plan.inst[q].cell0;
    return 0;
}

int awg_run_batch(const awg_problem *problems, awg_outputs *outputs, int n, int precision) {
    g_err.clear();
    if (!problems || !outputs || n <= 0) { set_error("empty batch"); return -1; }
    awg::RunOptions opt;
    opt.precision = precision;
    std::string err;
    int rc = awg::run_batch(problems, outputs, n, opt, err);
    if (rc != 0) set_error(err);
    return rc;
}

}  // extern "C"

struct awg_batch_ctx {
    awg::Ctx *ctx = nullptr;
    bool pending = false;
};

extern "C" {

awg_batch_ctx *awg_batch_ctx_create(void) {
    g_err.clear();
    awg_batch_ctx *c = new awg_batch_ctx();
    c->ctx = awg::ctx_create();
    awg::ctx_set_graphs(c->ctx, true);
    return c;
}

int awg_batch_launch(awg_batch_ctx *c, const awg_problem *problems, awg_outputs *outputs, int n,
                     int precision) {
    g_err.clear();
    if (!c || !problems || !outputs || n < 1) {
        set_error("awg_batch_launch: bad arguments");
        return -1;
    }
    if (c->pending) {
        set_error("awg_batch_launch: the context's last batch is not finished");
        return -1;
    }
    std::string err;
    const int rc = awg::ctx_launch_async(c->ctx, problems, outputs, n, precision, err);
    if (rc != 0) {
        awg::ctx_sync(c->ctx);  // nothing of the failed launch left in flight
        set_error(err);
        return rc;
    }
    c->pending = true;
    return 0;
}

int awg_batch_finish(awg_batch_ctx *c) {
    g_err.clear();
    if (!c || !c->pending) {
        set_error("awg_batch_finish: no batch in flight");
        return -1;
    }
    c->pending = false;
    std::string err;
    const int rc = awg::ctx_finish(c->ctx, err);
    if (rc != 0) set_error(err);
    return rc;
}

void awg_batch_ctx_destroy(awg_batch_ctx *c) {
    if (!c) return;
    if (c->ctx) {
        awg::ctx_sync(c->ctx);
        awg::ctx_destroy(c->ctx);
    }
    delete c;
}

long long awg_batch_device_bytes(const awg_problem *problems, int n, int precision, int want_path,
                                 int want_posterior) {
    g_err.clear();
    if (!problems || n <= 0) { set_error("empty batch"); return -1; }
    std::string err;
    const long long b = awg::batch_device_bytes(problems, n, precision, want_path != 0,
                                                want_posterior != 0, err);
    if (b < 0) set_error(err);
    return b;
}

int awg_autotune(const awg_problem *problems, awg_outputs *outputs, int n, int precision,
                 int trials, char *report, int report_len) {
    g_err.clear();
    if (!problems || !outputs || n <= 0) { set_error("empty batch"); return -1; }
    awg::TuneCfg best;
    double ms = 0.0;
    std::string err;
    const int rc = awg::autotune(problems, outputs, n, precision, trials, best, ms, err);
    if (rc != 0) {
        set_error(err);
        return rc;
    }
    if (report && report_len > 0)
        snprintf(report, report_len, "kpt=%d group_div=%d chunk=%d persistent=%d ms=%.3f", best.kpt,
                 best.group_div, best.chunk, best.persistent, ms);
    return 0;
}

int awg_forward_static(const awg_problem *problem, awg_outputs *output, int precision,
                       void *stream) {
    g_err.clear();
    std::string err;
    const int rc = awg::run_static(problem, output, precision, (cudaStream_t)stream, err);
    if (rc != 0) set_error(err);
    return rc;
}

awg_local_trees *arghmm_new_trees(int **ptrees, int **ages, int **sprs, int *blocklens,
                                  int ntrees, int nnodes, int start_coord) {
    if (!ptrees || !ages || !sprs || !blocklens || ntrees < 1 || nnodes < 1) {
        set_error("arghmm_new_trees: bad arguments");
        return nullptr;
    }
    awg_local_trees *t = new awg_local_trees();
    t->ntrees = ntrees; t->nnodes = nnodes; t->start_coord = start_coord;
    t->ptrees.resize((size_t)ntrees * nnodes);
    t->ages.resize((size_t)ntrees * nnodes);
    t->sprs.resize((size_t)ntrees * 4);
    t->blocklens.assign(blocklens, blocklens + ntrees);
    for (int i = 0; i < ntrees; i++) {
        memcpy(&t->ptrees[(size_t)i * nnodes], ptrees[i], sizeof(int) * nnodes);
        memcpy(&t->ages[(size_t)i * nnodes], ages[i], sizeof(int) * nnodes);
        memcpy(&t->sprs[(size_t)i * 4], sprs[i], sizeof(int) * 4);
    }
    return t;
}

void delete_local_trees(awg_local_trees *trees) { delete trees; }

void get_local_trees_ptrees(awg_local_trees *trees, int **ptrees, int **ages, int **sprs,
                            int *blocklens) {
    if (!trees) return;
    const int n = trees->nnodes;
    std::vector<int> perm;
    if (leaf_perm(trees, perm)) {  // leaves named by their sequence (local_tree.cpp:1862-1890)
        for (int b = 0; b < trees->ntrees; b++) {
            const int *par = &trees->ptrees[(size_t)b * n], *age = &trees->ages[(size_t)b * n];
            for (int j = 0; j < n; j++) {
                if (ptrees) ptrees[b][perm[j]] = par[j] != -1 ? perm[par[j]] : -1;
                if (ages) ages[b][perm[j]] = age[j];
            }
            if (sprs) {
                const int *s = &trees->sprs[(size_t)b * 4];
                const bool null = s[0] == -1;
                sprs[b][0] = null ? s[0] : perm[s[0]];
                sprs[b][1] = s[1];
                sprs[b][2] = null ? s[2] : perm[s[2]];
                sprs[b][3] = s[3];
            }
            if (blocklens) blocklens[b] = trees->blocklens[b];
        }
        return;
    }
    for (int b = 0; b < trees->ntrees; b++) {
        if (ptrees) memcpy(ptrees[b], &trees->ptrees[(size_t)b * n], sizeof(int) * n);
        if (ages) memcpy(ages[b], &trees->ages[(size_t)b * n], sizeof(int) * n);
        if (sprs) memcpy(sprs[b], &trees->sprs[(size_t)b * 4], sizeof(int) * 4);
        if (blocklens) blocklens[b] = trees->blocklens[b];
    }
}

int awg_local_trees_seqids(awg_local_trees *trees, int *seqids) {
    g_err.clear();
    if (!trees) {
        set_error("awg_local_trees_seqids: NULL trees");
        return -1;
    }
    const int nleaves = (trees->nnodes + 1) / 2;
    if (seqids)
        for (int i = 0; i < nleaves; i++)
            seqids[i] = trees->seqids.empty() ? i : trees->seqids[i];
    return nleaves;
}

int awg_local_trees_mapping(awg_local_trees *trees, int *mapping) {
    g_err.clear();
    if (!trees || !mapping) {
        set_error("awg_local_trees_mapping: NULL argument");
        return -1;
    }
    const int n = trees->nnodes;
    for (int b = 0; b < trees->ntrees; b++) {
        int *m = mapping + (size_t)b * n;
        if (b == 0) {
            for (int j = 0; j < n; j++) m[j] = -1;
        } else if (!trees->mapping.empty()) {
            memcpy(m, &trees->mapping[(size_t)b * n], sizeof(int) * n);
        } else {  // make_node_mapping (local_tree.h:767-776)
            for (int j = 0; j < n; j++) m[j] = j;
            const int broken = trees->ptrees[(size_t)(b - 1) * n + trees->sprs[(size_t)b * 4]];
            if (broken >= 0) m[broken] = -1;
        }
    }
    std::vector<int> perm, tmp(n);
    if (leaf_perm(trees, perm)) {  // in the names get_local_trees_ptrees shows
        for (int b = 1; b < trees->ntrees; b++) {
            int *m = mapping + (size_t)b * n;
            for (int j = 0; j < n; j++) tmp[perm[j]] = m[j] != -1 ? perm[m[j]] : -1;
            memcpy(m, tmp.data(), sizeof(int) * n);
        }
    }
    return 0;
}

int awg_local_trees_children(awg_local_trees *trees, int *c0, int *c1) {
    g_err.clear();
    if (!trees || !c0 || !c1) {
        set_error("awg_local_trees_children: NULL argument");
        return -1;
    }
    const int n = trees->nnodes;
    std::vector<int> perm;
    const bool named = leaf_perm(trees, perm);
    for (int b = 0; b < trees->ntrees; b++) {
        int *d0 = c0 + (size_t)b * n, *d1 = c1 + (size_t)b * n;
        std::vector<int> a0(n, -1), a1(n, -1);
        if (!trees->c0.empty()) {
            for (int j = 0; j < n; j++) {
                a0[j] = trees->c0[(size_t)b * n + j];
                a1[j] = trees->c1[(size_t)b * n + j];
            }
        } else {
            for (int j = 0; j < n; j++) {
                const int p = trees->ptrees[(size_t)b * n + j];
                if (p < 0 || p >= n) continue;
                if (a0[p] == -1) a0[p] = j;
                else a1[p] = j;
            }
        }
        for (int j = 0; j < n; j++) {
            const int v = named ? perm[j] : j;
            d0[v] = a0[j] != -1 && named ? perm[a0[j]] : a0[j];
            d1[v] = a1[j] != -1 && named ? perm[a1[j]] : a1[j];
        }
    }
    return 0;
}

int awg_local_trees_set_structure(awg_local_trees *trees, const int *mapping,
                                  const int *root_child0) {
    g_err.clear();
    if (!trees) {
        set_error("awg_local_trees_set_structure: NULL trees");
        return -1;
    }
    const int n = trees->nnodes, B = trees->ntrees;
    if (mapping) {
        for (size_t i = (size_t)n; i < (size_t)B * n; i++)
            if (mapping[i] < -1 || mapping[i] >= n) {
                set_error("awg_local_trees_set_structure: mapping out of range");
                return -1;
            }
        trees->mapping.assign(mapping, mapping + (size_t)B * n);
        for (int j = 0; j < n; j++) trees->mapping[j] = -1;
    } else {
        trees->mapping.clear();
    }
    trees->c0.clear();
    trees->c1.clear();
    if (root_child0) {  // children in index order, each root's child[0] named (set_ptree)
        trees->c0.assign((size_t)B * n, -1);
        trees->c1.assign((size_t)B * n, -1);
        for (int b = 0; b < B; b++) {
            int *c0 = &trees->c0[(size_t)b * n], *c1 = &trees->c1[(size_t)b * n];
            const int *par = &trees->ptrees[(size_t)b * n];
            int root = -1;
            for (int i = 0; i < n; i++) {
                const int p = par[i];
                if (p == -1) root = i;
                else if (p < 0 || p >= n || c1[p] != -1) {
                    set_error("awg_local_trees_set_structure: malformed tree");
                    trees->c0.clear();
                    trees->c1.clear();
                    return -1;
                } else if (c0[p] == -1) c0[p] = i;
                else c1[p] = i;
            }
            const int want = root_child0[b];
            if (root >= 0 && want != -1 && c0[root] != want) {
                if (c1[root] != want) {
                    set_error("awg_local_trees_set_structure: root_child0 is no child of the root");
                    trees->c0.clear();
                    trees->c1.clear();
                    return -1;
                }
                std::swap(c0[root], c1[root]);
            }
        }
    }
    return 0;
}

int awg_add_arg_thread(awg_local_trees *trees, int ntimes, const int *path, int seqlen,
                       const int *rec_pos, const int *rec_node, const int *rec_time, int nrec) {
    g_err.clear();
    if (!trees || !path || nrec < 0 || (nrec > 0 && (!rec_pos || !rec_node || !rec_time)) ||
        ntimes < 3 || ntimes > awg::MAXT) {
        set_error("awg_add_arg_thread: bad arguments");
        return -1;
    }
    if ((trees->nnodes + 2 + 1) / 2 > awg::MAXNODES / 2 || trees->nnodes + 2 > awg::MAXNODES) {
        set_error("awg_add_arg_thread: the grown trees exceed the node limit");
        return -1;
    }
    awg::ThreadTrees a;
    a.ntrees = trees->ntrees; a.nnodes = trees->nnodes; a.start_coord = trees->start_coord;
    a.ptrees = trees->ptrees; a.ages = trees->ages; a.sprs = trees->sprs;
    a.blocklens = trees->blocklens; a.mapping = trees->mapping; a.c0 = trees->c0;
    a.c1 = trees->c1;
    std::string err;
    if (!awg::add_arg_thread(a, ntimes, path, seqlen, rec_pos, rec_node, rec_time, nrec, err)) {
        set_error(err);
        return -1;
    }
    trees->ntrees = a.ntrees; trees->nnodes = a.nnodes;
    trees->ptrees = std::move(a.ptrees); trees->ages = std::move(a.ages);
    trees->sprs = std::move(a.sprs); trees->blocklens = std::move(a.blocklens);
    trees->mapping = std::move(a.mapping); trees->c0 = std::move(a.c0);
    trees->c1 = std::move(a.c1);
    if (!trees->seqids.empty()) {  // the new leaf holds the smallest sequence id not in use
        std::vector<char> used(trees->seqids.size() + 1, 0);
        for (int s : trees->seqids)
            if (s >= 0 && s < (int)used.size()) used[s] = 1;
        int id = 0;
        while (used[id]) id++;
        trees->seqids.push_back(id);
    }
    return 0;
}

static awg::ThreadTrees thread_trees(const awg_local_trees *t) {
    awg::ThreadTrees a;
    a.ntrees = t->ntrees; a.nnodes = t->nnodes; a.start_coord = t->start_coord;
    a.ptrees = t->ptrees; a.ages = t->ages; a.sprs = t->sprs; a.blocklens = t->blocklens;
    a.mapping = t->mapping; a.c0 = t->c0; a.c1 = t->c1; a.seqids = t->seqids;
    return a;
}

static void store_trees(awg_local_trees *t, awg::ThreadTrees &a) {
    t->ntrees = a.ntrees; t->nnodes = a.nnodes;
    t->ptrees = std::move(a.ptrees); t->ages = std::move(a.ages); t->sprs = std::move(a.sprs);
    t->blocklens = std::move(a.blocklens); t->mapping = std::move(a.mapping);
    t->c0 = std::move(a.c0); t->c1 = std::move(a.c1); t->seqids = std::move(a.seqids);
}

void arghmm_get_thread_times(awg_local_trees *trees, int ntimes, int *path, int *path_times) {
    g_err.clear();
    std::string err;
    if (!trees || !path || !path_times) set_error("arghmm_get_thread_times: NULL argument");
    else if (!awg::thread_times(thread_trees(trees), ntimes, path, path_times, err))
        set_error(err);
}

int awg_add_arg_thread_path(awg_local_trees *trees, int ntimes, int minage, const int *path,
                            int seqlen, const int *rec_pos, const int *rec_node,
                            const int *rec_time, int nrec) {
    g_err.clear();
    if (!trees || !path || nrec < 0 || (nrec > 0 && (!rec_pos || !rec_node || !rec_time)) ||
        ntimes < 3 || minage < 0) {
        set_error("awg_add_arg_thread_path: bad arguments");
        return -1;
    }
    awg::ThreadTrees a = thread_trees(trees);
    std::string err;
    if (!awg::add_thread_path(a, ntimes, minage, path, seqlen, rec_pos, rec_node, rec_time, nrec,
                              err)) {
        set_error(err);
        return -1;
    }
    store_trees(trees, a);
    return 0;
}

// Removal paths and the internal-branch cut (thread.cpp:1681-1716). Paths hold one node
// per tree in the trees' own node names; draws come from libc rand(), as the reference's.
void arghmm_sample_arg_removal_path(awg_local_trees *trees, int node, int *path) {
    g_err.clear();
    std::string err;
    if (!trees || !path) set_error("arghmm_sample_arg_removal_path: NULL argument");
    else if (!awg::sample_removal_path(thread_trees(trees), node, -1, rand, path, err))
        set_error(err);
}

void arghmm_sample_arg_removal_path2(awg_local_trees *trees, int node, int pos, int *path) {
    g_err.clear();
    std::string err;
    if (!trees || !path) set_error("arghmm_sample_arg_removal_path2: NULL argument");
    else if (!awg::sample_removal_path(thread_trees(trees), node, pos, rand, path, err))
        set_error(err);
}

void arghmm_sample_arg_removal_leaf_path(awg_local_trees *trees, int node, int *path) {
    g_err.clear();
    std::string err;
    if (!trees || !path) set_error("arghmm_sample_arg_removal_leaf_path: NULL argument");
    else if (!awg::sample_removal_path(thread_trees(trees), node, -1, nullptr, path, err))
        set_error(err);
}

void arghmm_sample_arg_removal_path_recomb(awg_local_trees *trees, double recomb_preference,
                                           int *path) {
    g_err.clear();
    std::string err;
    if (!trees || !path) set_error("arghmm_sample_arg_removal_path_recomb: NULL argument");
    else if (!awg::sample_removal_path_recomb(thread_trees(trees), recomb_preference, rand, path,
                                              err))
        set_error(err);
}

double awg_sample_arg_removal_path_uniform(awg_local_trees *trees, int *path) {
    g_err.clear();
    std::string err;
    double lntotal = NAN;
    if (!trees || !path) set_error("awg_sample_arg_removal_path_uniform: NULL argument");
    else if (!awg::sample_removal_path_uniform(thread_trees(trees), rand, path, &lntotal, err))
        set_error(err);
    return lntotal;
}

void arghmm_remove_arg_thread_path(awg_local_trees *trees, int *removal_path, int maxtime) {
    g_err.clear();
    if (!trees || !removal_path) {
        set_error("arghmm_remove_arg_thread_path: NULL argument");
        return;
    }
    awg::ThreadTrees a = thread_trees(trees);
    std::string err;
    if (!awg::remove_thread_path(a, removal_path, maxtime, nullptr, err)) set_error(err);
    else store_trees(trees, a);
}

void arghmm_remove_arg_thread_path2(awg_local_trees *trees, int *removal_path, int maxtime,
                                    int *original_thread) {
    g_err.clear();
    if (!trees || !removal_path || !original_thread) {
        set_error("arghmm_remove_arg_thread_path2: NULL argument");
        return;
    }
    awg::ThreadTrees a = thread_trees(trees);
    std::string err;
    if (!awg::remove_thread_path(a, removal_path, maxtime, original_thread, err)) set_error(err);
    else store_trees(trees, a);
}

// remove_arg_thread (thread.cpp:425-556) on the host: the leaf holding sequence `seqid`
// leaves every tree; the last leaf takes its name (its sequence id moves with it).
int awg_remove_arg_thread(awg_local_trees *trees, int seqid) {
    g_err.clear();
    if (!trees) {
        set_error("awg_remove_arg_thread: NULL trees");
        return -1;
    }
    awg::ThreadTrees a = thread_trees(trees);
    std::string err;
    if (!awg::remove_arg_thread(a, seqid, err)) {
        set_error(err);
        return -1;
    }
    store_trees(trees, a);
    return 0;
}
// get_state_spaces (states.cpp:228-251): each tree's (node, time) states in new[] rows. As
// the reference's, it lists external states (get_coal_states with its default, states.cpp:
// 53-74) whatever `internal` says: node index order, times from the node's age up to its
// parent's (the root's up to ntimes - 2).
awg_intstate **get_state_spaces(awg_local_trees *trees, int ntimes, bool internal) {
    (void)internal;
    g_err.clear();
    if (!trees) {
        set_error("get_state_spaces: NULL trees");
        return nullptr;
    }
    const int n = trees->nnodes;
    awg_intstate **all = new awg_intstate *[trees->ntrees];
    for (int b = 0; b < trees->ntrees; b++) {
        const int *par = &trees->ptrees[(size_t)b * n], *age = &trees->ages[(size_t)b * n];
        std::vector<int> st;
        for (int i = 0; i < n; i++) {
            const int top = par[i] == -1 ? ntimes - 2 : age[par[i]];
            for (int t = age[i]; t <= top; t++) {
                st.push_back(i);
                st.push_back(t);
            }
        }
        all[b] = new awg_intstate[st.size() / 2 + 1];
        for (size_t j = 0; j < st.size() / 2; j++) {
            all[b][j][0] = st[2 * j];
            all[b][j][1] = st[2 * j + 1];
        }
    }
    return all;
}

void delete_state_spaces(awg_intstate **all_states, int ntrees) {
    if (!all_states) return;
    for (int i = 0; i < ntrees; i++) delete[] all_states[i];
    delete[] all_states;
}

// read_local_trees (local_tree.cpp:1908-1932): a trees handle from an SMC file (gzip read
// through a pipe when the name ends in .gz); NULL and awg_last_error() on failure.
awg_local_trees *read_local_trees(const char *filename, const double *times, int ntimes) {
    g_err.clear();
    awg::SmcArrays a;
    std::string err;
    if (!awg::read_smc_arrays(filename, times, ntimes, a, err)) {
        set_error(err);
        return nullptr;
    }
    awg_local_trees *t = new awg_local_trees();
    t->ntrees = a.ntrees; t->nnodes = a.nnodes; t->start_coord = a.start_coord;
    t->ptrees = std::move(a.ptrees); t->ages = std::move(a.ages); t->sprs = std::move(a.sprs);
    t->blocklens = std::move(a.blocklens);
    t->c0 = std::move(a.c0); t->c1 = std::move(a.c1);  // newick child order
    return t;
}

// arghmm_copy_trees (local_tree.cpp:1827-1832)
awg_local_trees *arghmm_copy_trees(awg_local_trees *trees) {
    g_err.clear();
    if (!trees) {
        set_error("arghmm_copy_trees: NULL trees");
        return nullptr;
    }
    return new awg_local_trees(*trees);
}

// get_local_trees_blocks (local_tree.cpp:1946-1958): each tree's [start, end) coordinates
void get_local_trees_blocks(awg_local_trees *trees, int *starts, int *ends) {
    if (!trees || !starts || !ends) return;
    int end = trees->start_coord;
    for (int b = 0; b < trees->ntrees; b++) {
        starts[b] = end;
        end += trees->blocklens[b];
        ends[b] = end;
    }
}

// get_treelens (local_tree.cpp:1935-1943): each tree's branch length without the basal stub
// (get_treelen, local_tree.cpp:136-155), summed in node order as there
void get_treelens(awg_local_trees *trees, const double *times, int ntimes, double *treelens) {
    (void)ntimes;
    if (!trees || !times || !treelens) return;
    const int n = trees->nnodes;
    for (int b = 0; b < trees->ntrees; b++) {
        const int *par = &trees->ptrees[(size_t)b * n], *age = &trees->ages[(size_t)b * n];
        double len = 0.0;
        for (int i = 0; i < n; i++)
            if (par[i] != -1) len += times[age[par[i]]] - times[age[i]];
        treelens[b] = len;
    }
}

int get_local_trees_ntrees(awg_local_trees *trees) { return trees ? trees->ntrees : 0; }
int get_local_trees_nnodes(awg_local_trees *trees) { return trees ? trees->nnodes : 0; }

void arghmm_get_nstates(awg_local_trees *trees, int ntimes, bool internal, int *nstates) {
    if (!trees || !nstates) return;
    int pos = 0;
    const int n = trees->nnodes;
    for (int b = 0; b < trees->ntrees; b++) {
        // internal: the cut subtree is the root's child[0] as the trees keep it
        int rc0 = -1;
        if (!trees->c0.empty())
            for (int i = 0; i < n; i++)
                if (trees->ptrees[(size_t)b * n + i] == -1) rc0 = trees->c0[(size_t)b * n + i];
        int S = awg::count_states(&trees->ptrees[(size_t)b * n], &trees->ages[(size_t)b * n], n,
                                  ntimes, internal, 0, rc0, nullptr);
        for (int i = 0; i < trees->blocklens[b]; i++) nstates[pos + i] = S;
        pos += trees->blocklens[b];
    }
}

double **arghmm_forward_alg(awg_local_trees *trees, double *times, int ntimes,
                            double *popsizes, double rho, double mu, char **seqs, int nseqs,
                            int seqlen, bool prior_given, double *prior, bool internal,
                            bool slow) {
    // slow: the reference's dense S x S step (arghmm_forward_block_slow,
    // sample_thread.cpp:301-337), its test path
    return table_call(trees, times, ntimes, popsizes, rho, mu, seqs, nseqs, seqlen, internal,
                      prior_given ? prior : nullptr, 0, slow);
}

double **arghmm_backward_alg(awg_local_trees *trees, double *times, int ntimes,
                             double *popsizes, double rho, double mu, char **seqs, int nseqs,
                             int seqlen, bool internal) {
    return table_call(trees, times, ntimes, popsizes, rho, mu, seqs, nseqs, seqlen, internal,
                      nullptr, 1);
}

double **arghmm_posterior_marginals(awg_local_trees *trees, double *times, int ntimes,
                                    double *popsizes, double rho, double mu, char **seqs,
                                    int nseqs, int seqlen, bool internal) {
    return table_call(trees, times, ntimes, popsizes, rho, mu, seqs, nseqs, seqlen, internal,
                      nullptr, 2);
}

awg_intstate *arghmm_sample_posterior(int **ptrees, int **ages, int **sprs, int *blocklens,
                                      int ntrees, int nnodes, double *times, int ntimes,
                                      double *popsizes, double rho, double mu, char **seqs,
                                      int nseqs, int seqlen, awg_intstate *path) {
    g_err.clear();
    awg_local_trees *t = arghmm_new_trees(ptrees, ages, sprs, blocklens, ntrees, nnodes, 0);
    if (!t) return nullptr;
    ProblemView v;
    if (!make_view(t, times, ntimes, popsizes, rho, mu, seqs, nseqs, seqlen, false, v)) {
        delete t;
        return nullptr;
    }
    std::vector<int> ipath(seqlen);
    awg_outputs o;
    memset(&o, 0, sizeof(o));
    o.path = ipath.data();
    awg::RunOptions opt;
    std::string err;
    if (awg::run_batch(&v.p, &o, 1, opt, err) != 0) {
        set_error(err);
        delete t;
        return nullptr;
    }
    if (!path) path = (awg_intstate *)new int[2 * (size_t)seqlen];
    // state index -> (node, time) with each column's own state space (states.cpp:53-74)
    int pos = 0;
    for (int b = 0; b < ntrees; b++) {
        const int *par = &t->ptrees[(size_t)b * nnodes];
        const int *age = &t->ages[(size_t)b * nnodes];
        std::vector<int> first(nnodes), t0(nnodes);
        int S = 0;
        for (int v2 = 0; v2 < nnodes; v2++) {
            const int top = par[v2] == -1 ? ntimes - 2 : age[par[v2]];
            first[v2] = S;
            t0[v2] = age[v2];
            S += std::max(0, top - age[v2] + 1);
        }
        for (int i = pos; i < pos + blocklens[b]; i++) {
            const int k = ipath[i];
            int node = nnodes - 1;
            for (int v2 = 0; v2 < nnodes; v2++)
                if (first[v2] <= k && (v2 + 1 == nnodes || k < first[v2 + 1])) { node = v2; break; }
            path[i][0] = node;
            path[i][1] = t0[node] + (k - first[node]);
        }
        pos += blocklens[b];
    }
    delete t;
    return path;
}

void arghmm_sample_arg_thread_internal(awg_local_trees *trees, double *times, int ntimes,
                                       double *popsizes, double rho, double mu, char **seqs,
                                       int nseqs, int seqlen, int *thread_path) {
    g_err.clear();
    ProblemView v;
    if (!make_view(trees, times, ntimes, popsizes, rho, mu, seqs, nseqs, seqlen, true, v)) return;
    awg_outputs o;
    memset(&o, 0, sizeof(o));
    o.path = thread_path;
    awg::RunOptions opt;
    std::string err;
    if (awg::run_batch(&v.p, &o, 1, opt, err) != 0) set_error(err);
}

// arghmm_sample_thread (sample_thread.cpp:1010-1023, sample_arg_thread :575-625): the last
// sequence threaded into the trees in place: forward and traceback on the device (draws
// from rand(), last column first), recombinations along the thread on the device (draws
// continuing rand(): 2 * seqlen + 2 are taken up front, of which the sampler uses the
// reference's number), then the thread added on the host.
awg_local_trees *arghmm_sample_thread(awg_local_trees *trees, double *times, int ntimes,
                                      double *popsizes, double rho, double mu, char **seqs,
                                      int nseqs, int seqlen) {
    g_err.clear();
    if (!trees) {
        set_error("arghmm_sample_thread: NULL trees");
        return trees;
    }
    if (nseqs != (trees->nnodes + 1) / 2 + 1) {
        set_error("arghmm_sample_thread: the new sequence must follow the trees' leaves "
                  "(nseqs = leaves + 1)");
        return trees;
    }
    ProblemView v;
    if (!make_view(trees, times, ntimes, popsizes, rho, mu, seqs, nseqs, seqlen, false, v))
        return trees;
    std::vector<int> path(seqlen);
    awg_outputs o;
    memset(&o, 0, sizeof(o));
    o.path = path.data();
    awg::RunOptions opt;
    std::string err;
    if (awg::run_batch(&v.p, &o, 1, opt, err) != 0) {
        set_error(err);
        return trees;
    }
    const int nu = 2 * seqlen + 2;
    std::vector<double> u(nu);
    for (double &x : u) x = rand() / double(RAND_MAX);  // frand (common.h:103-110)
    std::vector<int> pos(seqlen), node(seqlen), time(seqlen);
    int used = 0;
    const int nrec = awg::sample_recombinations(&v.p, path.data(), u.data(), nu, pos.data(),
                                                node.data(), time.data(), seqlen, &used, err);
    if (nrec < 0) {
        set_error(err);
        return trees;
    }
    if (awg_add_arg_thread(trees, ntimes, path.data(), seqlen, pos.data(), node.data(),
                           time.data(), nrec) == 0 && !trees->seqids.empty())
        trees->seqids.back() = nseqs - 1;  // the new leaf holds new_chrom (thread.cpp:292)
    return trees;
}

// sample_arg_thread (sample_thread.cpp:575-625) for sequence new_chrom of the caller's full
// sequence set: the leaves read their sequence ids' rows, the thread is new_chrom's; the
// step as in arghmm_sample_thread, and the new leaf holds new_chrom.
int awg_sample_arg_thread(awg_local_trees *trees, double *times, int ntimes, double *popsizes,
                          double rho, double mu, char **seqs, int nseqs, int seqlen,
                          int new_chrom) {
    g_err.clear();
    if (!trees || !seqs) {
        set_error("awg_sample_arg_thread: NULL argument");
        return -1;
    }
    const int nleaves = (trees->nnodes + 1) / 2;
    std::vector<int> rows(nleaves + 1);
    for (int i = 0; i < nleaves; i++) rows[i] = trees->seqids.empty() ? i : trees->seqids[i];
    rows[nleaves] = new_chrom;
    for (int i = 0; i <= nleaves; i++)
        if (rows[i] < 0 || rows[i] >= nseqs || (i < nleaves && rows[i] == new_chrom)) {
            set_error("awg_sample_arg_thread: new_chrom must be a sequence no leaf holds");
            return -1;
        }
    ProblemView v;
    if (!make_view(trees, times, ntimes, popsizes, rho, mu, seqs, nseqs, seqlen, false, v, &rows))
        return -1;
    std::vector<int> path(seqlen);
    awg_outputs o;
    memset(&o, 0, sizeof(o));
    o.path = path.data();
    awg::RunOptions opt;
    std::string err;
    if (awg::run_batch(&v.p, &o, 1, opt, err) != 0) {
        set_error(err);
        return -1;
    }
    const int nu = 2 * seqlen + 2;
    std::vector<double> u(nu);
    for (double &x : u) x = rand() / double(RAND_MAX);  // frand (common.h:103-110)
    std::vector<int> pos(seqlen), node(seqlen), time(seqlen);
    int used = 0;
    const int nrec = awg::sample_recombinations(&v.p, path.data(), u.data(), nu, pos.data(),
                                                node.data(), time.data(), seqlen, &used, err);
    if (nrec < 0) {
        set_error(err);
        return -1;
    }
    std::vector<int> ids(rows.begin(), rows.end());  // the leaves' ids after the step
    if (awg_add_arg_thread(trees, ntimes, path.data(), seqlen, pos.data(), node.data(),
                           time.data(), nrec) != 0)
        return -1;
    trees->seqids = ids;  // the new leaf holds new_chrom (thread.cpp:292)
    return 0;
}

// sample_arg_thread_internal (sample_thread.cpp:635-692): the cut subtree of an internal
// problem re-threaded in place: forward and traceback on the device (draws from rand(), last
// column first), recombinations along the thread on the device (2 * seqlen + 2 draws taken up
// front, as in arghmm_sample_thread), then the regraft on the host. The path goes to
// thread_path when given. 0, or -1 (awg_last_error).
int awg_sample_arg_thread_internal(awg_local_trees *trees, double *times, int ntimes,
                                   double *popsizes, double rho, double mu, char **seqs,
                                   int nseqs, int seqlen, int minage, int *thread_path) {
    g_err.clear();
    if (!trees || minage < 0) {
        set_error("awg_sample_arg_thread_internal: bad arguments");
        return -1;
    }
    ProblemView v;
    if (!make_view(trees, times, ntimes, popsizes, rho, mu, seqs, nseqs, seqlen, true, v))
        return -1;
    v.p.minage = minage;
    std::vector<int> path(seqlen);
    awg_outputs o;
    memset(&o, 0, sizeof(o));
    o.path = path.data();
    awg::RunOptions opt;
    std::string err;
    if (awg::run_batch(&v.p, &o, 1, opt, err) != 0) {
        set_error(err);
        return -1;
    }
    const int nu = 2 * seqlen + 2;
    std::vector<double> u(nu);
    for (double &x : u) x = rand() / double(RAND_MAX);  // frand (common.h:103-110)
    std::vector<int> pos(seqlen), node(seqlen), time(seqlen);
    int used = 0;
    const int nrec = awg::sample_recombinations(&v.p, path.data(), u.data(), nu, pos.data(),
                                                node.data(), time.data(), seqlen, &used, err);
    if (nrec < 0) {
        set_error(err);
        return -1;
    }
    if (awg_add_arg_thread_path(trees, ntimes, minage, path.data(), seqlen, pos.data(),
                                node.data(), time.data(), nrec) != 0)
        return -1;
    if (thread_path) memcpy(thread_path, path.data(), sizeof(int) * seqlen);
    return 0;
}

void delete_path(int *path) { delete[] path; }

// Debug export: the FP64 tables the table kernel builds for one problem (layouts in
// engine.h). Returns 0 or a negative code.
int awg_debug_tables(const awg_problem *p, double *tm, double *gts, double *inv, double *prior,
                     int *btptr, int *btperm) {
    g_err.clear();
    awg_outputs o;
    memset(&o, 0, sizeof(o));
    awg::RunOptions opt;
    opt.tables_only = true;
    opt.dbg_tm = tm; opt.dbg_gts = gts; opt.dbg_inv = inv; opt.dbg_prior = prior;
    opt.dbg_btptr = btptr; opt.dbg_btperm = btperm;
    std::string err;
    int rc = awg::run_batch(p, &o, 1, opt, err);
    if (rc != 0) set_error(err);
    return rc;
}

void delete_double_matrix(double **mat, int nrows) {
    (void)nrows;
    if (!mat) return;
    delete[] mat[0];
    delete[] mat;
}

}  // extern "C"

// ---- the reference's dense helper matrices (its ctypes layer's test and plotting aids)

namespace {

// state index of (node, time) in a tree's external state list (get_coal_states,
// states.cpp:53-74: nodes in index order, times from the node's age to its parent's, the
// root's to ntimes - 2), or -1
struct StateIndex {
    std::vector<int> first, lo, hi;
    StateIndex(const int *ptree, const int *ages, int nnodes, int ntimes)
        : first(nnodes), lo(nnodes), hi(nnodes) {
        int S = 0;
        for (int v = 0; v < nnodes; v++) {
            lo[v] = ages[v];
            hi[v] = ptree[v] == -1 ? ntimes - 2 : ages[ptree[v]];
            first[v] = S;
            S += std::max(0, hi[v] - lo[v] + 1);
        }
    }
    int operator()(int node, int time) const {
        if (node < 0 || node >= (int)first.size() || time < lo[node] || time > hi[node]) return -1;
        return first[node] + time - lo[node];
    }
};

bool map_states(const awg_intstate *istates, int n, const StateIndex &ix, std::vector<int> &out,
                const char *who) {
    out.resize(std::max(n, 0));
    for (int i = 0; i < n; i++) {
        out[i] = ix(istates[i][0], istates[i][1]);
        if (out[i] < 0) {
            set_error(std::string(who) + ": state " + std::to_string(i) + " (node " +
                      std::to_string(istates[i][0]) + ", time " + std::to_string(istates[i][1]) +
                      ") is not a coalescence state of its tree");
            return false;
        }
    }
    return true;
}

// nrows row pointers into one block of nrows * ncols doubles (freed by delete_double_matrix
// and its aliases)
double **new_dense(int nrows, int ncols) {
    double **m = new double *[std::max(nrows, 1)];
    double *blk = new double[std::max((size_t)nrows * ncols, (size_t)1)];
    for (int i = 0; i < nrows; i++) m[i] = blk + (size_t)i * ncols;
    if (nrows == 0) m[0] = blk;
    return m;
}

double **dense_call(const awg_problem &p, int kind, const std::vector<int> &rows,
                    const std::vector<int> &cols, int ncolumns, const char *who) {
    const int nr = kind == awg::DENSE_EMISSIONS ? ncolumns : (int)rows.size();
    double **m = new_dense(nr, (int)cols.size());
    awg_outputs o;
    memset(&o, 0, sizeof(o));
    awg::RunOptions opt;
    opt.dense_kind = kind;
    opt.dense_rows = rows.data();
    opt.dense_nrows = (int)rows.size();
    opt.dense_cols = cols.data();
    opt.dense_ncols = (int)cols.size();
    opt.dense_ncolumns = ncolumns;
    opt.dense_out = m[0];
    std::string err;
    if (awg::run_batch(&p, &o, 1, opt, err) != 0) {
        set_error(std::string(who) + ": " + err);
        delete[] m[0];
        delete[] m;
        return nullptr;
    }
    return m;
}

}  // namespace

extern "C" {

double **new_transition_probs(int nnodes, int *ptree, int *ages, double treelen,
                              awg_intstate *istates, int nstates, int ntimes, double *times,
                              double *time_steps, int *nbranches, int *nrecombs, int *ncoals,
                              double *popsizes, double rho) {
    // treelen, time_steps and the lineage counts are the caller's copies of what the table
    // kernel derives from the tree and the times (the reference recomputes them too)
    (void)treelen; (void)time_steps; (void)nbranches; (void)nrecombs; (void)ncoals;
    g_err.clear();
    if (!ptree || !ages || !times || !popsizes || (nstates > 0 && !istates) || nnodes < 1) {
        set_error("new_transition_probs: bad arguments");
        return nullptr;
    }
    std::vector<int> idx;
    if (!map_states(istates, nstates, StateIndex(ptree, ages, nnodes, ntimes), idx,
                    "new_transition_probs"))
        return nullptr;
    const int nseqs = (nnodes + 1) / 2 + 1;
    std::vector<char> seqs(nseqs, 'N');
    int sprs[4] = {-1, -1, -1, -1}, blocklen = 1;
    awg_problem p;
    memset(&p, 0, sizeof(p));
    p.ntrees = 1; p.nnodes = nnodes; p.ntimes = ntimes; p.nseqs = nseqs; p.seqlen = 1;
    p.ptrees = ptree; p.ages = ages; p.sprs = sprs; p.blocklens = &blocklen;
    p.times = times; p.popsizes = popsizes; p.rho = rho; p.mu = 0.0; p.seqs = seqs.data();
    return dense_call(p, awg::DENSE_TRANSITION, idx, idx, 0, "new_transition_probs");
}

double **new_transition_probs_switch(int *ptree, int *last_ptree, int nnodes, int recomb_node,
                                     int recomb_time, int coal_node, int coal_time,
                                     int *ages_index, int *last_ages_index, double treelen,
                                     double last_treelen, awg_intstate *istates1, int nstates1,
                                     awg_intstate *istates2, int nstates2, int ntimes,
                                     double *times, double *time_steps, int *nbranches,
                                     int *nrecombs, int *ncoals, double *popsizes, double rho) {
    (void)treelen; (void)last_treelen; (void)time_steps; (void)nbranches; (void)nrecombs;
    (void)ncoals;
    g_err.clear();
    if (!ptree || !last_ptree || !ages_index || !last_ages_index || !times || !popsizes ||
        (nstates1 > 0 && !istates1) || (nstates2 > 0 && !istates2) || nnodes < 1) {
        set_error("new_transition_probs_switch: bad arguments");
        return nullptr;
    }
    std::vector<int> rows, cols;
    if (!map_states(istates1, nstates1, StateIndex(last_ptree, last_ages_index, nnodes, ntimes),
                    rows, "new_transition_probs_switch") ||
        !map_states(istates2, nstates2, StateIndex(ptree, ages_index, nnodes, ntimes), cols,
                    "new_transition_probs_switch"))
        return nullptr;
    // two trees of one column each; the node mapping is make_node_mapping's (local_tree.h:
    // 767-778), as the reference builds it here
    std::vector<int> pt(2 * (size_t)nnodes), ag(2 * (size_t)nnodes);
    std::copy(last_ptree, last_ptree + nnodes, pt.begin());
    std::copy(ptree, ptree + nnodes, pt.begin() + nnodes);
    std::copy(last_ages_index, last_ages_index + nnodes, ag.begin());
    std::copy(ages_index, ages_index + nnodes, ag.begin() + nnodes);
    int sprs[8] = {-1, -1, -1, -1, recomb_node, recomb_time, coal_node, coal_time};
    int blocklens[2] = {1, 1};
    const int nseqs = (nnodes + 1) / 2 + 1;
    std::vector<char> seqs(2 * (size_t)nseqs, 'N');
    awg_problem p;
    memset(&p, 0, sizeof(p));
    p.ntrees = 2; p.nnodes = nnodes; p.ntimes = ntimes; p.nseqs = nseqs; p.seqlen = 2;
    p.ptrees = pt.data(); p.ages = ag.data(); p.sprs = sprs; p.blocklens = blocklens;
    p.times = times; p.popsizes = popsizes; p.rho = rho; p.mu = 0.0; p.seqs = seqs.data();
    return dense_call(p, awg::DENSE_SWITCH, rows, cols, 0, "new_transition_probs_switch");
}

void delete_transition_probs(double **transmat, int nstates) {
    delete_double_matrix(transmat, nstates);
}

double **new_emissions(awg_intstate *istates, int nstates, int *ptree, int nnodes,
                       int *ages_index, char **seqs, int nseqs, int seqlen, double *times,
                       int ntimes, double mu) {
    g_err.clear();
    if (!ptree || !ages_index || !seqs || !times || (nstates > 0 && !istates) || nnodes < 1 ||
        seqlen < 0 || nseqs < 1) {
        set_error("new_emissions: bad arguments");
        return nullptr;
    }
    std::vector<int> idx;
    if (!map_states(istates, nstates, StateIndex(ptree, ages_index, nnodes, ntimes), idx,
                    "new_emissions"))
        return nullptr;
    // one tree over a masked column (the forward's first column, which has no emission)
    // followed by the caller's columns
    const int L = seqlen + 1;
    std::vector<char> sq((size_t)nseqs * L);
    for (int j = 0; j < nseqs; j++) {
        sq[(size_t)j * L] = 'N';
        memcpy(&sq[(size_t)j * L + 1], seqs[j], seqlen);
    }
    std::vector<double> pops(ntimes, 1.0);  // the model's popsizes do not enter emissions
    int sprs[4] = {-1, -1, -1, -1};
    awg_problem p;
    memset(&p, 0, sizeof(p));
    p.ntrees = 1; p.nnodes = nnodes; p.ntimes = ntimes; p.nseqs = nseqs; p.seqlen = L;
    p.ptrees = ptree; p.ages = ages_index; p.sprs = sprs; p.blocklens = &L;
    p.times = times; p.popsizes = pops.data(); p.rho = 0.0; p.mu = mu; p.seqs = sq.data();
    return dense_call(p, awg::DENSE_EMISSIONS, {}, idx, seqlen, "new_emissions");
}

void delete_emissions(double **emit, int seqlen) { delete_double_matrix(emit, seqlen); }

void delete_forward_matrix(double **mat, int nrows) {
    (void)nrows;
    if (!mat) return;
    double **base = mat - 1;
    delete[] base[0];
    delete[] base;
}

// The dense HMM (hmm.cpp:27-85, bound by argweaver/argweaverc.py:42-56): the first column of
// fw (last of bw, last entry of path) is the caller's, as in the reference.
void forward_alg(int n, int nstates, double **trans, double **emit, double **fw) {
    g_err.clear();
    std::string err;
    if (!awg::dense_hmm(0, n, nstates, trans, emit, fw, nullptr, err)) set_error(err);
}

void backward_alg(int n, int nstates, double **trans, double **emit, double **bw) {
    g_err.clear();
    std::string err;
    if (!awg::dense_hmm(1, n, nstates, trans, emit, bw, nullptr, err)) set_error(err);
}

void sample_hmm_posterior(int n, int nstates, double **trans, double **fw, int *path) {
    g_err.clear();
    std::string err;
    if (!awg::dense_hmm(2, n, nstates, trans, nullptr, fw, path, err)) set_error(err);
}

// ARG probabilities (total_prob.cpp:315-382): computed on the device; NaN and
// awg_last_error() on failure (the reference asserts).
static double arg_prob_call(const awg_local_trees *t, const double *times, int ntimes,
                            const double *popsizes, double rho, double mu, char **seqs,
                            int nseqs, int seqlen, int what, int which) {
    g_err.clear();
    if (!t) {
        set_error("ARG probability: NULL trees");
        return NAN;
    }
    double out[3] = {0, 0, 0};
    std::string err;
    if (awg::arg_probabilities(t->ptrees.data(), t->ages.data(), t->sprs.data(),
                               t->blocklens.data(), t->ntrees, t->nnodes, t->start_coord, times,
                               ntimes, popsizes, rho, mu, seqs, nseqs, seqlen, what, out,
                               err) != 0) {
        set_error(err);
        return NAN;
    }
    return which < 0 ? out[0] + out[1] : out[which];
}

double arghmm_likelihood(awg_local_trees *trees, double *times, int ntimes, double mu,
                         char **seqs, int nseqs, int seqlen) {
    if (trees && trees->nnodes < 3) return log(.25) * seqlen;  // total_prob.cpp:27-28
    return arg_prob_call(trees, times, ntimes, nullptr, 0.0, mu, seqs, nseqs, seqlen, 1, 0);
}

double arghmm_prior_prob(awg_local_trees *trees, double *times, int ntimes, double *popsizes,
                         double rho) {
    return arg_prob_call(trees, times, ntimes, popsizes, rho, 0.0, nullptr, 0, 0, 2, 1);
}

double arghmm_tree_prior_prob(awg_local_trees *trees, double *times, int ntimes,
                              double *popsizes) {
    return arg_prob_call(trees, times, ntimes, popsizes, 0.0, 0.0, nullptr, 0, 0, 4, 2);
}

double arghmm_joint_prob(awg_local_trees *trees, double *times, int ntimes, double *popsizes,
                         double mu, double rho, char **seqs, int nseqs, int seqlen) {
    if (trees && trees->nnodes < 3)
        return log(.25) * seqlen +
               arg_prob_call(trees, times, ntimes, popsizes, rho, mu, nullptr, 0, 0, 2, 1);
    return arg_prob_call(trees, times, ntimes, popsizes, rho, mu, seqs, nseqs, seqlen, 3, -1);
}

int awg_sample_recombinations(const awg_problem *problem, const int *path,
                              const double *uniforms, int n_uniforms, int *pos, int *node,
                              int *time, int cap, int *used) {
    g_err.clear();
    std::string err;
    const int rc = awg::sample_recombinations(problem, path, uniforms, n_uniforms, pos, node,
                                              time, cap, used, err);
    if (rc < 0) set_error(err);
    return rc;
}

}  // extern "C"


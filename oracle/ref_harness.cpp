// Fixture harness around the compiled reference library (oracle/_ref/libargweaver.a).
//
// Test infrastructure only, run where the reference checkout exists. It reads a
// problem file (format below, written by argweaver_gb300/problem.py), runs the
// reference's own C++ threading HMM on it and writes the results as golden data:
//
//   forward <problem> <out> <seed> [penalty]
//                                    forward table (arghmm_forward_alg, sample_thread.cpp:394)
//                                    + stochastic_traceback (sample_thread.cpp:522) after
//                                    srand(seed); per-column nstates (states.cpp:209); with
//                                    penalty, the model's infsites_penalty (emit.cpp:847-862)
//   tables  <problem> <out>          per-block TransMatrix terms (trans.cpp:26),
//                                    TransMatrixSwitch (trans.cpp:538), emissions (emit.cpp:650)
//   dense   <problem> <out> <seed>   single-block problems: the reference's dense log-space
//                                    backward_alg (hmm.cpp:48) on calc_transition_probs
//                                    (trans.cpp:136) + calc_emissions, for the backward oracle;
//                                    its forward_alg (hmm.cpp:26) and sample_hmm_posterior
//                                    (hmm.cpp:76) after srand(seed)
//   densernd <S> <n> <seed> <out>    the dense HMM (hmm.cpp:27-85) on a random S-state
//                                    matrix (about a tenth of the entries zero) and random
//                                    emissions, inputs from a fixed integer hash: forward_alg,
//                                    backward_alg, then a path after srand(seed)
//   argprob <problem> <out>          the ARG's probabilities through the reference's C
//                                    exports (total_prob.cpp:315-382): likelihood, prior,
//                                    first-tree prior, joint (4 doubles)
//   recomb  <problem> <path> <seed> <out>
//                                    sample_recombinations (recomb.cpp:151-235) along the
//                                    int32 state path after srand(seed): count, positions,
//                                    nodes, times, then the next rand() value
//   addthread <problem> <path> <recombs> <out>
//                                    add_arg_thread (thread.cpp:272-422): the new leaf's
//                                    thread (int32 state path) and its recombinations (int32
//                                    triples column, node, time) added to the problem's
//                                    trees; writes the grown ARG as a problem
//   samplethread <problem> <seed> <out>
//   removethread <problem> <out-prefix> <seqid>...
//   addthreadpath <internal problem> <path> <recombs> <out>
//   samplethreadinternal <internal problem> <seed> <out>
//   resampleleaf <problem> <seqid> <seed> <out>
//   removalpaths <problem> <seed> <node> <pos> <out-prefix>
//                                    arghmm_sample_thread (sample_thread.cpp:1010-1023)
//                                    after srand(seed): the last sequence threaded into the
//                                    trees; writes the grown ARG as a problem
//   ingest  <sites> <smc> <c> <out>  reads a sites file + SMC ARG the way arg-sample does
//                                    (read_sites, find_compress_cols, compress_sites,
//                                    make_sequences_from_sites, read_local_trees, set_seqids,
//                                    compress_local_trees) and writes the full ARG problem
//   sim1    <sites> <smc> <c> <out>  reads a sites file + SMC ARG the way arg-sample does
//                                    (arg-sample.cpp:996-1155), removes the last sequence's
//                                    thread (thread.cpp:425) and writes the external problem
//   cut     <problem> <seed> <out>   samples a uniform removal path (thread.h:130) and cuts it
//                                    (remove_arg_thread_path, thread.h:43): internal problem
//
// Problem file (little endian): "AWGPROB1"; int32 ntrees,nnodes,ntimes,nseqs,seqlen,
// internal,start_coord,pad; f64 rho,mu; f64 times[T]; f64 popsizes[T];
// i32 ptrees[ntrees*nnodes]; i32 ages[ntrees*nnodes]; i32 sprs[ntrees*4];
// i32 blocklens[ntrees]; u8 seqs[nseqs*seqlen]. The header's last int32 holds flags:
// bit 0: i32 mapping[ntrees*nnodes] follows: LocalTreeSpr::mapping (previous tree node ->
//        this tree node, -1 for the broken node; row 0 unused). Without it the mapping is
//        the reference's make_node_mapping (local_tree.h:767).
// bit 1: i32 root_child0[ntrees] follows: child[0] of each tree's root. The reference
//        names the cut subtree of an internal-branch tree child[0] of the virtual root
//        (states.cpp:121); parent arrays alone order children by index
//        (local_tree.h:216-229), which cannot express every cut.

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "argweaver/common.h"
#include "argweaver/compress.h"
#include "argweaver/emit.h"
#include "argweaver/hmm.h"
#include "argweaver/local_tree.h"
#include "argweaver/matrices.h"
#include "argweaver/model.h"
#include "argweaver/recomb.h"
#include "argweaver/sample_thread.h"
#include "argweaver/sequences.h"
#include "argweaver/states.h"
#include "argweaver/thread.h"
#include "argweaver/trans.h"

// an export of thread.cpp (:1718) that no header declares
namespace argweaver {
extern "C" void arghmm_get_thread_times(LocalTrees *trees, int ntimes, int *path,
                                        int *path_times);
}

using namespace argweaver;
using std::vector;

// extern "C" entry points the reference defines without a header declaration
namespace argweaver {
extern "C" {
void get_local_trees_ptrees(LocalTrees *trees, int **ptrees, int **ages, int **sprs,
                            int *blocklens);          // local_tree.cpp:1846
void arghmm_get_nstates(LocalTrees *trees, int ntimes, bool internal,
                        int *nstates);                // states.cpp:209
LocalTrees *arghmm_sample_thread(LocalTrees *trees, double *times, int ntimes,
                                 double *popsizes, double rho, double mu, char **seqs,
                                 int nseqs, int seqlen);       // sample_thread.cpp:1010
double arghmm_likelihood(LocalTrees *trees, double *times, int ntimes, double mu,
                         char **seqs, int nseqs, int seqlen);          // total_prob.cpp:317
double arghmm_prior_prob(LocalTrees *trees, double *times, int ntimes, double *popsizes,
                         double rho);                                  // total_prob.cpp:345
double arghmm_tree_prior_prob(LocalTrees *trees, double *times, int ntimes,
                              double *popsizes);                       // total_prob.cpp:355
double arghmm_joint_prob(LocalTrees *trees, double *times, int ntimes, double *popsizes,
                         double mu, double rho, char **seqs, int nseqs,
                         int seqlen);                                  // total_prob.cpp:369
double **new_transition_probs(int nnodes, int *ptree, int *ages, double treelen,
                              intstate *istates, int nstates, int ntimes, double *times,
                              double *time_steps, int *nbranches, int *nrecombs, int *ncoals,
                              double *popsizes, double rho);           // trans.cpp:1190
double **new_transition_probs_switch(
    int *ptree, int *last_ptree, int nnodes, int recomb_node, int recomb_time, int coal_node,
    int coal_time, int *ages_index, int *last_ages_index, double treelen, double last_treelen,
    intstate *istates1, int nstates1, intstate *istates2, int nstates2, int ntimes,
    double *times, double *time_steps, int *nbranches, int *nrecombs, int *ncoals,
    double *popsizes, double rho);                                     // trans.cpp:1212
void delete_transition_probs(double **transmat, int nstates);         // trans.cpp:1248
bool arghmm_assert_transmat(int nnodes, int *ptree, int *ages, int ntimes, double *times,
                            double *popsizes, double rho);             // trans.cpp:1254
bool arghmm_assert_transmat_switch(int nnodes, int *ptree, int *ages, int recomb_node,
                                   int recomb_time, int coal_node, int coal_time, int ntimes,
                                   double *times, double *popsizes,
                                   double rho);                        // trans.cpp:1275
bool arghmm_assert_emit(LocalTrees *trees, int ntimes, double *times, double mu, char **seqs,
                        int nseqs, int seqlen);                        // emit.cpp:1312
}
}

struct Problem {
    int ntrees = 0, nnodes = 0, ntimes = 0, nseqs = 0, seqlen = 0;
    int internal = 0, start_coord = 0;
    double rho = 0, mu = 0;
    vector<double> times, popsizes;
    vector<int> ptrees, ages, sprs, blocklens;
    vector<char> seqs;
    vector<int> mapping;      // empty: make_node_mapping default
    vector<int> root_child0;  // empty: children ordered by index
};

static void die(const char *msg) { fprintf(stderr, "ref_harness: %s\n", msg); exit(1); }

template <class T> static void rd(FILE *f, T *p, size_t n) {
    if (n && fread(p, sizeof(T), n, f) != n) die("short read");
}
template <class T> static void wr(FILE *f, const T *p, size_t n) {
    if (n && fwrite(p, sizeof(T), n, f) != n) die("short write");
}

static Problem read_problem(const char *path) {
    FILE *f = fopen(path, "rb");
    if (!f) die("cannot open problem");
    char magic[8];
    rd(f, magic, 8);
    if (memcmp(magic, "AWGPROB1", 8) != 0) die("bad problem magic");
    Problem p;
    int hdr[8];
    rd(f, hdr, 8);
    p.ntrees = hdr[0]; p.nnodes = hdr[1]; p.ntimes = hdr[2]; p.nseqs = hdr[3];
    p.seqlen = hdr[4]; p.internal = hdr[5]; p.start_coord = hdr[6];
    rd(f, &p.rho, 1); rd(f, &p.mu, 1);
    p.times.resize(p.ntimes); p.popsizes.resize(p.ntimes);
    rd(f, p.times.data(), p.ntimes); rd(f, p.popsizes.data(), p.ntimes);
    size_t tn = (size_t)p.ntrees * p.nnodes;
    p.ptrees.resize(tn); p.ages.resize(tn); p.sprs.resize(p.ntrees * 4);
    p.blocklens.resize(p.ntrees);
    rd(f, p.ptrees.data(), tn); rd(f, p.ages.data(), tn);
    rd(f, p.sprs.data(), p.sprs.size()); rd(f, p.blocklens.data(), p.ntrees);
    p.seqs.resize((size_t)p.nseqs * p.seqlen);
    rd(f, p.seqs.data(), p.seqs.size());
    if (hdr[7] & 1) {
        p.mapping.resize(tn);
        rd(f, p.mapping.data(), tn);
    }
    if (hdr[7] & 2) {
        p.root_child0.resize(p.ntrees);
        rd(f, p.root_child0.data(), p.ntrees);
    }
    fclose(f);
    return p;
}

static void write_problem(const char *path, const Problem &p) {
    FILE *f = fopen(path, "wb");
    if (!f) die("cannot write problem");
    wr(f, "AWGPROB1", 8);
    int hdr[8] = {p.ntrees, p.nnodes, p.ntimes, p.nseqs, p.seqlen, p.internal,
                  p.start_coord,
                  (p.mapping.empty() ? 0 : 1) | (p.root_child0.empty() ? 0 : 2)};
    wr(f, hdr, 8);
    wr(f, &p.rho, 1); wr(f, &p.mu, 1);
    wr(f, p.times.data(), p.ntimes); wr(f, p.popsizes.data(), p.ntimes);
    wr(f, p.ptrees.data(), p.ptrees.size()); wr(f, p.ages.data(), p.ages.size());
    wr(f, p.sprs.data(), p.sprs.size()); wr(f, p.blocklens.data(), p.blocklens.size());
    wr(f, p.seqs.data(), p.seqs.size());
    if (!p.mapping.empty()) wr(f, p.mapping.data(), p.mapping.size());
    if (!p.root_child0.empty()) wr(f, p.root_child0.data(), p.root_child0.size());
    fclose(f);
}

// Build the reference's LocalTrees from the flat arrays (local_tree.cpp:321).
static LocalTrees *make_trees(Problem &p) {
    vector<int *> pt(p.ntrees), ag(p.ntrees), sp(p.ntrees);
    for (int i = 0; i < p.ntrees; i++) {
        pt[i] = &p.ptrees[(size_t)i * p.nnodes];
        ag[i] = &p.ages[(size_t)i * p.nnodes];
        sp[i] = &p.sprs[(size_t)i * 4];
    }
    LocalTrees *trees = new LocalTrees(pt.data(), ag.data(), sp.data(), p.blocklens.data(),
                                       p.ntrees, p.nnodes, -1, p.start_coord);
    if (!p.mapping.empty()) {
        int i = 0;
        for (LocalTrees::iterator it = trees->begin(); it != trees->end(); ++it, ++i)
            if (it->mapping)
                for (int j = 0; j < p.nnodes; j++)
                    it->mapping[j] = p.mapping[(size_t)i * p.nnodes + j];
    }
    if (!p.root_child0.empty()) {
        int i = 0;
        for (LocalTrees::iterator it = trees->begin(); it != trees->end(); ++it, ++i) {
            LocalNode &r = it->tree->nodes[it->tree->root];
            if (r.child[0] != p.root_child0[i]) std::swap(r.child[0], r.child[1]);
        }
    }
    return trees;
}

// Flatten a LocalTrees back to arrays (get_local_trees_ptrees, local_tree.cpp:1846).
static void trees_to_problem(LocalTrees *trees, Problem &p) {
    p.ntrees = trees->get_num_trees();
    p.nnodes = trees->nnodes;
    p.start_coord = trees->start_coord;
    size_t tn = (size_t)p.ntrees * p.nnodes;
    p.ptrees.assign(tn, 0); p.ages.assign(tn, 0);
    p.sprs.assign(p.ntrees * 4, 0); p.blocklens.assign(p.ntrees, 0);
    vector<int *> pt(p.ntrees), ag(p.ntrees), sp(p.ntrees);
    for (int i = 0; i < p.ntrees; i++) {
        pt[i] = &p.ptrees[(size_t)i * p.nnodes];
        ag[i] = &p.ages[(size_t)i * p.nnodes];
        sp[i] = &p.sprs[(size_t)i * 4];
    }
    get_local_trees_ptrees(trees, pt.data(), ag.data(), sp.data(), p.blocklens.data());
    // mappings, in the same leaf permutation get_local_trees_ptrees applies
    const int nleaves = trees->get_num_leaves();
    vector<int> perm(p.nnodes);
    for (int j = 0; j < p.nnodes; j++) perm[j] = j < nleaves ? trees->seqids[j] : j;
    p.mapping.assign(tn, -1);
    int i = 0;
    for (LocalTrees::iterator it = trees->begin(); it != trees->end(); ++it, ++i)
        if (it->mapping)
            for (int j = 0; j < p.nnodes; j++) {
                int m = it->mapping[j];
                p.mapping[(size_t)i * p.nnodes + perm[j]] = m == -1 ? -1 : perm[m];
            }
    p.root_child0.assign(p.ntrees, -1);
    i = 0;
    for (LocalTrees::iterator it = trees->begin(); it != trees->end(); ++it, ++i) {
        LocalTree *t = it->tree;
        int c0 = t->nodes[t->root].child[0];
        p.root_child0[i] = c0 == -1 ? -1 : perm[c0];
    }
}

static vector<char *> seq_ptrs(Problem &p) {
    vector<char *> s(p.nseqs);
    for (int i = 0; i < p.nseqs; i++) s[i] = &p.seqs[(size_t)i * p.seqlen];
    return s;
}

static int cmd_forward(const char *in, const char *out, int seed, double penalty) {
    Problem p = read_problem(in);
    LocalTrees *trees = make_trees(p);
    ArgModel model(p.ntimes, p.times.data(), p.popsizes.data(), p.rho, p.mu);
    model.infsites_penalty = penalty;  // 1: off (the model's default, model.h:53)
    vector<char *> sp = seq_ptrs(p);
    Sequences sequences(sp.data(), p.nseqs, p.seqlen);
    const bool internal = p.internal != 0;

    ArgHmmMatrixList matrix_list(&model, &sequences, trees);
    matrix_list.set_internal(internal);
    matrix_list.setup();
    ArgHmmForwardTable forward(trees->start_coord, trees->length());
    arghmm_forward_alg(trees, &model, &sequences, &matrix_list, &forward, NULL,
                       false, internal, false);
    double **fw = forward.get_table();

    vector<int> nstates(p.seqlen);
    arghmm_get_nstates(trees, p.ntimes, internal, nstates.data());

    srand(seed);
    vector<int> path(p.seqlen);
    stochastic_traceback(trees, &model, &matrix_list, fw, path.data() - trees->start_coord,
                         false, internal);

    FILE *f = fopen(out, "wb");
    if (!f) die("cannot write output");
    wr(f, "AWGREF01", 8);
    long long ncells = 0;
    for (int i = 0; i < p.seqlen; i++) ncells += std::max(nstates[i], 1);
    int hdr[2] = {p.seqlen, 0};
    wr(f, hdr, 2);
    wr(f, &ncells, 1);
    wr(f, nstates.data(), p.seqlen);
    for (int i = 0; i < p.seqlen; i++)
        wr(f, fw[trees->start_coord + i], std::max(nstates[i], 1));
    wr(f, path.data(), p.seqlen);
    fclose(f);
    delete trees;
    return 0;
}

static int cmd_tables(const char *in, const char *out) {
    Problem p = read_problem(in);
    LocalTrees *trees = make_trees(p);
    ArgModel model(p.ntimes, p.times.data(), p.popsizes.data(), p.rho, p.mu);
    vector<char *> sp = seq_ptrs(p);
    Sequences sequences(sp.data(), p.nseqs, p.seqlen);
    const bool internal = p.internal != 0;
    const int T = p.ntimes;

    ArgHmmMatrixList matrix_list(&model, &sequences, trees);
    matrix_list.set_internal(internal);
    matrix_list.setup();

    FILE *f = fopen(out, "wb");
    if (!f) die("cannot write output");
    wr(f, "AWGTAB01", 8);
    int nblocks = 0;
    for (matrix_list.begin(); matrix_list.more(); matrix_list.next()) nblocks++;
    wr(f, &nblocks, 1);
    for (matrix_list.begin(); matrix_list.more(); matrix_list.next()) {
        ArgHmmMatrices &m = matrix_list.ref_matrices();
        int hdr[6] = {matrix_list.get_block_start(), m.blocklen, m.nstates1, m.nstates2,
                      m.transmat_switch ? 1 : 0, m.transmat->minage};
        wr(f, hdr, 6);
        const TransMatrix *tm = m.transmat;
        // entries [0, T-2] are the ones calc_transition_probs writes
        const double *arrs[9] = {tm->D, tm->E, tm->lnB, tm->lnE2, tm->lnNegG1,
                                 tm->G2, tm->G3, tm->lnG4, tm->norecombs};
        for (int a = 0; a < 9; a++) wr(f, arrs[a], T - 1);
        if (m.transmat_switch) {
            const TransMatrixSwitch *sw = m.transmat_switch;
            int n1 = std::max(sw->nstates1, 1), n2 = std::max(sw->nstates2, 1);
            int src[2] = {sw->recombsrc, sw->recoalsrc};
            wr(f, src, 2);
            wr(f, sw->determ, n1);
            wr(f, sw->determprob, n1);
            // rows are only defined when their source exists
            vector<double> zero(n2, 0.0);
            wr(f, sw->recombsrc != -1 ? sw->recombrow : zero.data(), n2);
            wr(f, sw->recoalsrc != -1 ? sw->recoalrow : zero.data(), n2);
        }
        int S = std::max(m.nstates2, 1);
        for (int i = 0; i < m.blocklen; i++) wr(f, m.emit[i], S);
    }
    fclose(f);
    delete trees;
    return 0;
}

// Dense log-space backward of the reference's generic HMM on one block.
static int cmd_dense(const char *in, const char *out, int seed) {
    Problem p = read_problem(in);
    if (p.ntrees != 1 || p.internal) die("dense: single external tree only");
    LocalTrees *trees = make_trees(p);
    ArgModel model(p.ntimes, p.times.data(), p.popsizes.data(), p.rho, p.mu);
    LocalTree *tree = trees->front().tree;
    States states;
    get_coal_states(tree, p.ntimes, states, false);
    int S = states.size();
    LineageCounts lineages(p.ntimes);
    lineages.count(tree);
    double **trans = new_matrix<double>(S, S);
    calc_transition_probs(tree, &model, states, &lineages, trans);  // log values
    double **emit = new_matrix<double>(p.seqlen, S);
    vector<char *> sp = seq_ptrs(p);
    calc_emissions_external(states, tree, sp.data(), p.nseqs, p.seqlen, &model, emit, NULL);
    for (int i = 0; i < p.seqlen; i++)
        for (int k = 0; k < S; k++) emit[i][k] = log(emit[i][k]);
    double **bw = new_matrix<double>(p.seqlen, S);
    for (int k = 0; k < S; k++) bw[p.seqlen - 1][k] = 0.0;
    backward_alg(p.seqlen, S, trans, emit, bw);
    // the dense forward (first column: the log emissions) and a path drawn from it after
    // srand(seed): the last column from its normalised weights, the rest by
    // sample_hmm_posterior (hmm.cpp:76-95), one rand() per column, last column first
    double **fw = new_matrix<double>(p.seqlen, S);
    for (int k = 0; k < S; k++) fw[0][k] = emit[0][k];
    forward_alg(p.seqlen, S, trans, emit, fw);
    srand(seed);
    vector<int> path(p.seqlen);
    {
        vector<double> A(S);
        const double total = logsum(fw[p.seqlen - 1], S);
        for (int k = 0; k < S; k++) A[k] = exp(fw[p.seqlen - 1][k] - total);
        path[p.seqlen - 1] = sample(A.data(), S);
    }
    sample_hmm_posterior(p.seqlen, S, trans, fw, path.data());
    FILE *f = fopen(out, "wb");
    if (!f) die("cannot write output");
    wr(f, "AWGDNS03", 8);
    int hdr[2] = {p.seqlen, S};
    wr(f, hdr, 2);
    for (int i = 0; i < p.seqlen; i++) wr(f, bw[i], S);
    for (int i = 0; i < S; i++) wr(f, trans[i], S);      // log transition matrix
    for (int i = 0; i < p.seqlen; i++) wr(f, emit[i], S); // log emissions
    for (int i = 0; i < p.seqlen; i++) wr(f, fw[i], S);   // dense forward
    wr(f, path.data(), p.seqlen);
    fclose(f);
    delete_matrix(trans, S); delete_matrix(emit, p.seqlen); delete_matrix(bw, p.seqlen);
    delete_matrix(fw, p.seqlen);
    delete trees;
    return 0;
}

// The reference's dense helper exports on a problem's trees, states in get_coal_states
// order: new_transition_probs of tree 0, new_emissions of tree 0's columns, and
// new_transition_probs_switch into trees 1..maxb; then the reference's own brute-force
// self-checks on the same trees (arghmm_assert_transmat on tree 0, arghmm_assert_transmat_
// switch on each boundary, arghmm_assert_emit over every tree). Output "AWGHLP01",
// i32 {S0, L0, nsw}, f64 trans[S0][S0], f64 emit[L0][S0], per switch i32 {S1, S2} and
// f64 [S1][S2], then i32 checks[nsw + 2] (1: passed).
static int cmd_helpers(const char *in, const char *out, int maxb) {
    Problem p = read_problem(in);
    const int n = p.nnodes;
    if (p.internal) die("helpers: external trees only");
    // new_transition_probs_switch maps nodes by make_node_mapping (local_tree.h:767)
    for (int b = 1; b < p.ntrees && !p.mapping.empty(); b++)
        for (int j = 0; j < n; j++) {
            const int broken = p.ptrees[(size_t)(b - 1) * n + p.sprs[(size_t)b * 4]];
            if (p.mapping[(size_t)b * n + j] != (j == broken ? -1 : j))
                die("helpers: node mappings other than make_node_mapping's");
        }
    auto states_of = [&](int b) {
        LocalTree tree(&p.ptrees[(size_t)b * n], n, &p.ages[(size_t)b * n]);
        States st;
        get_coal_states(&tree, p.ntimes, st, false);
        vector<int> flat(2 * st.size());
        for (size_t i = 0; i < st.size(); i++) {
            flat[2 * i] = st[i].node;
            flat[2 * i + 1] = st[i].time;
        }
        return flat;
    };
    FILE *f = fopen(out, "wb");
    if (!f) die("cannot write output");
    wr(f, "AWGHLP01", 8);
    vector<int> s0 = states_of(0);
    const int S0 = (int)s0.size() / 2, L0 = p.blocklens[0];
    const int nsw = std::min(maxb, p.ntrees - 1);
    int hdr[3] = {S0, L0, nsw};
    wr(f, hdr, 3);
    double **tr = new_transition_probs(n, &p.ptrees[0], &p.ages[0], 0.0, (intstate *)s0.data(),
                                       S0, p.ntimes, p.times.data(), NULL, NULL, NULL, NULL,
                                       p.popsizes.data(), p.rho);
    for (int i = 0; i < S0; i++) wr(f, tr[i], S0);
    delete_transition_probs(tr, S0);
    vector<char *> sp = seq_ptrs(p);  // tree 0's columns are the first L0
    double **em = new_emissions((intstate *)s0.data(), S0, &p.ptrees[0], n, &p.ages[0],
                                sp.data(), p.nseqs, L0, p.times.data(), p.ntimes, p.mu);
    for (int i = 0; i < L0; i++) wr(f, em[i], S0);
    delete_emissions(em, L0);
    for (int b = 1; b <= nsw; b++) {
        vector<int> s1 = states_of(b - 1), s2 = states_of(b);
        const int S1 = (int)s1.size() / 2, S2 = (int)s2.size() / 2;
        const int *spr = &p.sprs[(size_t)b * 4];
        double **sw = new_transition_probs_switch(
            &p.ptrees[(size_t)b * n], &p.ptrees[(size_t)(b - 1) * n], n, spr[0], spr[1], spr[2],
            spr[3], &p.ages[(size_t)b * n], &p.ages[(size_t)(b - 1) * n], 0.0, 0.0,
            (intstate *)s1.data(), S1, (intstate *)s2.data(), S2, p.ntimes, p.times.data(), NULL,
            NULL, NULL, NULL, p.popsizes.data(), p.rho);
        int sz[2] = {S1, S2};
        wr(f, sz, 2);
        for (int i = 0; i < S1; i++) wr(f, sw[i], S2);
        delete_transition_probs(sw, S1);
    }
    vector<int> checks;
    checks.push_back(arghmm_assert_transmat(n, &p.ptrees[0], &p.ages[0], p.ntimes,
                                            p.times.data(), p.popsizes.data(), p.rho));
    for (int b = 1; b <= nsw; b++) {
        const int *spr = &p.sprs[(size_t)b * 4];
        checks.push_back(arghmm_assert_transmat_switch(
            n, &p.ptrees[(size_t)(b - 1) * n], &p.ages[(size_t)(b - 1) * n], spr[0], spr[1],
            spr[2], spr[3], p.ntimes, p.times.data(), p.popsizes.data(), p.rho));
    }
    LocalTrees *trees = make_trees(p);
    checks.push_back(arghmm_assert_emit(trees, p.ntimes, p.times.data(), p.mu, sp.data(),
                                        p.nseqs, p.seqlen));
    delete trees;
    wr(f, checks.data(), checks.size());
    fclose(f);
    return 0;
}

static int cmd_argprob(const char *in, const char *out) {
    Problem p = read_problem(in);
    LocalTrees *trees = make_trees(p);
    vector<char *> sp = seq_ptrs(p);
    double v[4];
    v[0] = arghmm_likelihood(trees, p.times.data(), p.ntimes, p.mu, sp.data(), p.nseqs, p.seqlen);
    v[1] = arghmm_prior_prob(trees, p.times.data(), p.ntimes, p.popsizes.data(), p.rho);
    v[2] = arghmm_tree_prior_prob(trees, p.times.data(), p.ntimes, p.popsizes.data());
    v[3] = arghmm_joint_prob(trees, p.times.data(), p.ntimes, p.popsizes.data(), p.mu, p.rho,
                             sp.data(), p.nseqs, p.seqlen);
    FILE *f = fopen(out, "wb");
    if (!f) die("cannot write output");
    wr(f, v, 4);
    fclose(f);
    delete trees;
    return 0;
}

// uniform in [0, 1) from an integer hash of (a, b, c): the random fixture's inputs
static double hash01(unsigned a, unsigned b, unsigned c) {
    unsigned long long x = 0x9E3779B97F4A7C15ull * (a + 1) ^ 0xC2B2AE3D27D4EB4Full * (b + 7) ^
                           0x165667B19E3779F9ull * (c + 13);
    x ^= x >> 31; x *= 0xBF58476D1CE4E5B9ull; x ^= x >> 27; x *= 0x94D049BB133111EBull;
    x ^= x >> 33;
    return (double)(x >> 11) / 9007199254740992.0;
}

static int cmd_densernd(int S, int n, int seed, const char *out) {
    if (S < 1 || n < 2) die("densernd: S >= 1 and n >= 2");
    double **trans = new_matrix<double>(S, S);
    for (int j = 0; j < S; j++) {
        double tot = 0.0;
        vector<double> w(S);
        for (int k = 0; k < S; k++) {
            const double h = hash01(seed, j, k);
            w[k] = (k != j && h < 0.1) ? 0.0 : 0.05 + h;
            tot += w[k];
        }
        for (int k = 0; k < S; k++) trans[j][k] = log(w[k] / tot);
    }
    double **emit = new_matrix<double>(n, S);
    for (int i = 0; i < n; i++)
        for (int k = 0; k < S; k++) emit[i][k] = log(0.01 + hash01(seed + 1000, i, k));
    double **fw = new_matrix<double>(n, S), **bw = new_matrix<double>(n, S);
    for (int k = 0; k < S; k++) {
        fw[0][k] = emit[0][k] - log((double)S);
        bw[n - 1][k] = 0.0;
    }
    forward_alg(n, S, trans, emit, fw);
    backward_alg(n, S, trans, emit, bw);
    srand(seed);
    vector<int> path(n);
    {
        vector<double> A(S);
        const double total = logsum(fw[n - 1], S);
        for (int k = 0; k < S; k++) A[k] = exp(fw[n - 1][k] - total);
        path[n - 1] = sample(A.data(), S);
    }
    sample_hmm_posterior(n, S, trans, fw, path.data());
    FILE *f = fopen(out, "wb");
    if (!f) die("cannot write output");
    wr(f, "AWGDNS03", 8);
    int hdr[2] = {n, S};
    wr(f, hdr, 2);
    for (int i = 0; i < n; i++) wr(f, bw[i], S);
    for (int i = 0; i < S; i++) wr(f, trans[i], S);
    for (int i = 0; i < n; i++) wr(f, emit[i], S);
    for (int i = 0; i < n; i++) wr(f, fw[i], S);
    wr(f, path.data(), n);
    fclose(f);
    delete_matrix(trans, S); delete_matrix(emit, n); delete_matrix(bw, n);
    delete_matrix(fw, n);
    return 0;
}

static int cmd_sim1(const char *sites_file, const char *smc_file, int compress,
                    const char *out) {
    const int ntimes = 20;
    const double maxtime = 200e3, popsize = 1e4, rho = 1.6e-8, mu = 1.8e-8;
    Sites sites;
    CompressStream stream(sites_file);
    if (!stream.stream || !read_sites(stream.stream, &sites, -1, -1)) die("cannot read sites");
    stream.close();
    SitesMapping mapping;
    if (!find_compress_cols(&sites, compress, &mapping)) die("cannot compress");
    compress_sites(&sites, &mapping);
    Sequences sequences;
    make_sequences_from_sites(&sites, &sequences);

    ArgModel model(ntimes, maxtime, popsize, rho, mu);
    LocalTrees *trees = new LocalTrees();
    vector<std::string> seqnames;
    CompressStream smc(smc_file, "r");
    if (!smc.stream || !read_local_trees(smc.stream, model.times, model.ntimes, trees, seqnames))
        die("cannot read smc");
    if (!trees->set_seqids(seqnames, sequences.names)) die("seqids");
    compress_local_trees(trees, &mapping, true);

    // remove the thread of the last sequence (the one to re-thread)
    const int nseqs = sequences.get_num_seqs();
    remove_arg_thread(trees, nseqs - 1);

    Problem p;
    p.ntimes = ntimes;
    p.rho = rho * compress;
    p.mu = mu * compress;
    p.times.assign(model.times, model.times + ntimes);
    p.popsizes.assign(model.popsizes, model.popsizes + ntimes);
    p.internal = 0;
    trees_to_problem(trees, p);
    // sequences in leaf order (seqids) followed by the new sequence
    const int nleaves = trees->get_num_leaves();
    p.nseqs = nleaves + 1;
    p.seqlen = sequences.length();
    p.seqs.resize((size_t)p.nseqs * p.seqlen);
    // get_local_trees_ptrees writes leaf j at position seqids[j], so problem row r is
    // sequence r; the re-threaded sequence comes last
    for (int r = 0; r < nleaves; r++)
        memcpy(&p.seqs[(size_t)r * p.seqlen], sequences.seqs[r], p.seqlen);
    memcpy(&p.seqs[(size_t)nleaves * p.seqlen], sequences.seqs[nseqs - 1], p.seqlen);
    write_problem(out, p);
    delete trees;
    return 0;
}

static int cmd_ingest(const char *sites_file, const char *smc_file, int compress,
                      const char *out) {
    const int ntimes = 20;
    const double maxtime = 200e3, popsize = 1e4, rho = 1.5e-8, mu = 2.5e-8;
    Sites sites;
    CompressStream stream(sites_file);
    if (!stream.stream || !read_sites(stream.stream, &sites, -1, -1)) die("cannot read sites");
    stream.close();
    SitesMapping mapping;
    if (!find_compress_cols(&sites, compress, &mapping)) die("cannot compress");
    compress_sites(&sites, &mapping);
    Sequences sequences;
    make_sequences_from_sites(&sites, &sequences);
    ArgModel model(ntimes, maxtime, popsize, rho, mu);
    LocalTrees *trees = new LocalTrees();
    vector<std::string> seqnames;
    CompressStream smc(smc_file, "r");
    if (!smc.stream || !read_local_trees(smc.stream, model.times, model.ntimes, trees, seqnames))
        die("cannot read smc");
    if (!trees->set_seqids(seqnames, sequences.names)) die("seqids");
    compress_local_trees(trees, &mapping, true);
    Problem p;
    p.ntimes = ntimes;
    p.rho = rho * compress;
    p.mu = mu * compress;
    p.times.assign(model.times, model.times + ntimes);
    p.popsizes.assign(model.popsizes, model.popsizes + ntimes);
    p.internal = 0;
    trees_to_problem(trees, p);
    p.nseqs = sequences.get_num_seqs();
    p.seqlen = sequences.length();
    p.seqs.resize((size_t)p.nseqs * p.seqlen);
    for (int r = 0; r < p.nseqs; r++)
        memcpy(&p.seqs[(size_t)r * p.seqlen], sequences.seqs[r], p.seqlen);
    write_problem(out, p);
    delete trees;
    return 0;
}

static int cmd_recomb(const char *in, const char *path_file, int seed, const char *out) {
    Problem p = read_problem(in);
    LocalTrees *trees = make_trees(p);
    ArgModel model(p.ntimes, p.times.data(), p.popsizes.data(), p.rho, p.mu);
    vector<char *> sp = seq_ptrs(p);
    Sequences sequences(sp.data(), p.nseqs, p.seqlen);
    const bool internal = p.internal != 0;
    ArgHmmMatrixList matrix_list(&model, &sequences, trees);
    matrix_list.set_internal(internal);
    matrix_list.setup();
    vector<int> path(p.seqlen);
    FILE *pf = fopen(path_file, "rb");
    if (!pf) die("cannot read path");
    rd(pf, path.data(), p.seqlen);
    fclose(pf);
    srand(seed);
    vector<int> pos;
    vector<NodePoint> recombs;
    sample_recombinations(trees, &model, &matrix_list, path.data() - trees->start_coord, pos,
                          recombs, internal);
    const int next = rand();
    FILE *f = fopen(out, "wb");
    if (!f) die("cannot write output");
    wr(f, "AWGREC01", 8);
    int hdr[2] = {(int)pos.size(), next};
    wr(f, hdr, 2);
    for (size_t k = 0; k < pos.size(); k++) {
        int v[3] = {pos[k] - trees->start_coord, recombs[k].node, recombs[k].time};
        wr(f, v, 3);
    }
    fclose(f);
    delete trees;
    return 0;
}

static int cmd_addthread(const char *in, const char *path_file, const char *rec_file,
                         const char *out) {
    Problem p = read_problem(in);
    if (p.internal) die("addthread: external problems only");
    LocalTrees *trees = make_trees(p);
    vector<int> path(p.seqlen);
    FILE *pf = fopen(path_file, "rb");
    if (!pf) die("cannot read path");
    rd(pf, path.data(), p.seqlen);
    fclose(pf);
    FILE *rf = fopen(rec_file, "rb");
    if (!rf) die("cannot read recombinations");
    vector<int> pos;
    vector<NodePoint> recombs;
    int v[3];
    while (fread(v, sizeof(int), 3, rf) == 3) {
        pos.push_back(v[0] + trees->start_coord);
        recombs.push_back(NodePoint(v[1], v[2]));
    }
    fclose(rf);
    StatesModel states_model(p.ntimes, false, 0);
    add_arg_thread(trees, states_model, p.ntimes, path.data() - trees->start_coord,
                   p.nseqs - 1, pos, recombs);
    Problem q = p;
    trees_to_problem(trees, q);
    write_problem(out, q);
    delete trees;
    return 0;
}

// add_arg_thread_path (thread.cpp:1314-1449): an internal problem's thread path and its
// recombinations (pos, node, time triples) regrafted into the cut ARG
static int cmd_addthreadpath(const char *in, const char *path_file, const char *rec_file,
                             const char *out) {
    Problem p = read_problem(in);
    if (!p.internal) die("addthreadpath: internal problems only");
    LocalTrees *trees = make_trees(p);
    vector<int> path(p.seqlen);
    FILE *pf = fopen(path_file, "rb");
    if (!pf) die("cannot read path");
    rd(pf, path.data(), p.seqlen);
    fclose(pf);
    FILE *rf = fopen(rec_file, "rb");
    if (!rf) die("cannot read recombinations");
    vector<int> pos;
    vector<NodePoint> recombs;
    int v[3];
    while (fread(v, sizeof(int), 3, rf) == 3) {
        pos.push_back(v[0] + trees->start_coord);
        recombs.push_back(NodePoint(v[1], v[2]));
    }
    fclose(rf);
    // the path's state times first (arghmm_get_thread_times, indexed by coordinate), when
    // every tree has states (the reference reads past an empty state list otherwise)
    bool all_partial = true;
    for (LocalTrees::iterator it = trees->begin(); it != trees->end(); ++it)
        all_partial = all_partial && it->tree->nodes[it->tree->root].age >= p.ntimes;
    if (all_partial) {
        vector<int> pabs(trees->start_coord + p.seqlen, 0), tabs(trees->start_coord + p.seqlen, 0);
        std::copy(path.begin(), path.end(), pabs.begin() + trees->start_coord);
        arghmm_get_thread_times(trees, p.ntimes, pabs.data(), tabs.data());
        FILE *tf = fopen((std::string(out) + ".times").c_str(), "wb");
        if (!tf) die("cannot write thread times");
        wr(tf, tabs.data() + trees->start_coord, p.seqlen);
        fclose(tf);
    }
    StatesModel states_model(p.ntimes, true, 0);
    add_arg_thread_path(trees, states_model, p.ntimes, path.data() - trees->start_coord, pos,
                        recombs);
    Problem q = p;
    q.internal = 0;
    trees_to_problem(trees, q);
    write_problem(out, q);
    delete trees;
    return 0;
}

// sample_arg_thread_internal (sample_thread.cpp:635-692) after srand(seed): the whole ARG
static int cmd_samplethreadinternal(const char *in, int seed, const char *out) {
    Problem p = read_problem(in);
    if (!p.internal) die("samplethreadinternal: internal problems only");
    LocalTrees *trees = make_trees(p);
    vector<char *> sp = seq_ptrs(p);
    ArgModel model(p.ntimes, p.times.data(), p.popsizes.data(), p.rho, p.mu);
    Sequences sequences(sp.data(), p.nseqs, p.seqlen);
    srand(seed);
    sample_arg_thread_internal(&model, &sequences, trees, 0, NULL);
    Problem q = p;
    q.internal = 0;
    trees_to_problem(trees, q);
    write_problem(out, q);
    delete trees;
    return 0;
}

// resample_arg_leaf's move (sample_arg.cpp:66-86) after srand(seed): sequence `seqid`
// removed from the full ARG and threaded back in; the ARG with leaves named by sequence
static int cmd_resampleleaf(const char *in, int seqid, int seed, const char *out) {
    Problem p = read_problem(in);
    if (p.internal) die("resampleleaf: full ARGs only");
    LocalTrees *trees = make_trees(p);
    vector<char *> sp = seq_ptrs(p);
    ArgModel model(p.ntimes, p.times.data(), p.popsizes.data(), p.rho, p.mu);
    Sequences sequences(sp.data(), p.nseqs, p.seqlen);
    srand(seed);
    remove_arg_thread(trees, seqid);
    sample_arg_thread(&model, &sequences, trees, seqid);
    Problem q = p;
    trees_to_problem(trees, q);
    write_problem(out, q);
    delete trees;
    return 0;
}

static int cmd_samplethread(const char *in, int seed, const char *out) {
    Problem p = read_problem(in);
    if (p.internal) die("samplethread: external problems only");
    LocalTrees *trees = make_trees(p);
    vector<char *> sp = seq_ptrs(p);
    srand(seed);
    arghmm_sample_thread(trees, p.times.data(), p.ntimes, p.popsizes.data(), p.rho, p.mu,
                         sp.data(), p.nseqs, p.seqlen);
    Problem q = p;
    trees_to_problem(trees, q);
    write_problem(out, q);
    delete trees;
    return 0;
}

// trees_to_problem when the leaves' sequence ids are a permutation of the leaves (the
// names get_local_trees_ptrees gives), else in the trees' own leaf names; no sequences
static void trees_to_problem_named(LocalTrees *trees, Problem &p) {
    const int nleaves = trees->get_num_leaves();
    vector<int> saved = trees->seqids;
    vector<char> seen(nleaves, 0);
    bool perm = (int)saved.size() == nleaves;
    for (int i = 0; perm && i < nleaves; i++) {
        perm = saved[i] >= 0 && saved[i] < nleaves && !seen[saved[i]];
        if (perm) seen[saved[i]] = 1;
    }
    if (!perm) trees->set_default_seqids();
    trees_to_problem(trees, p);
    trees->seqids = saved;
    p.nseqs = 0;
    p.seqs.clear();
}

// remove_arg_thread (thread.cpp:425-556) of each listed sequence in turn; after removal i
// the trees go to <prefix>.<i>.prob and the leaves' sequence ids to <prefix>.<i>.seqids
static int cmd_removethread(const char *in, const char *prefix, int nrm, char **ids) {
    Problem p = read_problem(in);
    if (p.internal) die("removethread: full ARGs only");
    LocalTrees *trees = make_trees(p);
    for (int i = 0; i < nrm; i++) {
        remove_arg_thread(trees, atoi(ids[i]));
        Problem q = p;
        trees_to_problem_named(trees, q);
        std::string base = std::string(prefix) + "." + std::to_string(i);
        write_problem((base + ".prob").c_str(), q);
        FILE *f = fopen((base + ".seqids").c_str(), "wb");
        if (!f) die("cannot write seqids");
        wr(f, trees->seqids.data(), trees->seqids.size());
        fclose(f);
    }
    delete trees;
    return 0;
}

// After srand(seed): a uniform removal path (sample_arg_removal_path_uniform), a forward
// path from `node` (sample_arg_removal_path), one through `node` at coordinate `pos`
// (sample_arg_removal_path2), the leaf path of leaf 0 and a path preferring recombinations
// (sample_arg_removal_path_recomb, .9), as <prefix>.paths (5 x ntrees
// ints) and the log path count as <prefix>.lntotal; then the ARG cut along the uniform path
// (remove_arg_thread_path, maxtime ntimes + 1) as <prefix>.cut.prob, with the removed thread
// as states of the cut trees as <prefix>.orig
static int cmd_removalpaths(const char *in, int seed, int node, int pos, const char *prefix) {
    Problem p = read_problem(in);
    if (p.internal) die("removalpaths: full ARGs only");
    LocalTrees *trees = make_trees(p);
    const int B = trees->get_num_trees();
    vector<int> paths((size_t)5 * B);
    srand(seed);
    double lntotal = sample_arg_removal_path_uniform(trees, &paths[0]);
    sample_arg_removal_path(trees, node, &paths[B]);
    sample_arg_removal_path(trees, node, pos, &paths[2 * B], .5);
    sample_arg_removal_leaf_path(trees, 0, &paths[3 * B]);
    sample_arg_removal_path_recomb(trees, .9, &paths[4 * B]);
    std::string base(prefix);
    FILE *f = fopen((base + ".paths").c_str(), "wb");
    if (!f) die("cannot write paths");
    wr(f, paths.data(), paths.size());
    fclose(f);
    f = fopen((base + ".lntotal").c_str(), "wb");
    if (!f) die("cannot write lntotal");
    wr(f, &lntotal, 1);
    fclose(f);
    vector<int> orig(p.seqlen);
    remove_arg_thread_path(trees, &paths[0], p.ntimes + 1, orig.data());
    f = fopen((base + ".orig").c_str(), "wb");
    if (!f) die("cannot write the original thread");
    wr(f, orig.data(), orig.size());
    fclose(f);
    Problem q = p;
    q.internal = 1;
    trees_to_problem_named(trees, q);
    write_problem((base + ".cut.prob").c_str(), q);
    delete trees;
    return 0;
}

static int cmd_cut(const char *in, int seed, const char *out) {
    Problem p = read_problem(in);
    if (p.internal) die("cut: input must be a full (external-format) ARG");
    LocalTrees *trees = make_trees(p);
    srand(seed);
    vector<int> path(trees->get_num_trees());
    sample_arg_removal_path_uniform(trees, path.data());
    remove_arg_thread_path(trees, path.data(), p.ntimes + 1);
    Problem q = p;
    q.internal = 1;
    trees_to_problem(trees, q);
    write_problem(out, q);
    delete trees;
    return 0;
}

int main(int argc, char **argv) {
    if (argc < 2) die("usage: ref_harness forward|tables|dense|sim1|cut ...");
    std::string cmd = argv[1];
    if (cmd == "forward" && argc == 5) return cmd_forward(argv[2], argv[3], atoi(argv[4]), 1.0);
    if (cmd == "forward" && argc == 6)
        return cmd_forward(argv[2], argv[3], atoi(argv[4]), atof(argv[5]));
    if (cmd == "tables" && argc == 4) return cmd_tables(argv[2], argv[3]);
    if (cmd == "dense" && argc == 5) return cmd_dense(argv[2], argv[3], atoi(argv[4]));
    if (cmd == "densernd" && argc == 6)
        return cmd_densernd(atoi(argv[2]), atoi(argv[3]), atoi(argv[4]), argv[5]);
    if (cmd == "argprob" && argc == 4) return cmd_argprob(argv[2], argv[3]);
    if (cmd == "helpers" && argc == 5) return cmd_helpers(argv[2], argv[3], atoi(argv[4]));
    if (cmd == "samplethread" && argc == 5)
        return cmd_samplethread(argv[2], atoi(argv[3]), argv[4]);
    if (cmd == "removethread" && argc >= 5)
        return cmd_removethread(argv[2], argv[3], argc - 4, argv + 4);
    if (cmd == "addthreadpath" && argc == 6)
        return cmd_addthreadpath(argv[2], argv[3], argv[4], argv[5]);
    if (cmd == "samplethreadinternal" && argc == 5)
        return cmd_samplethreadinternal(argv[2], atoi(argv[3]), argv[4]);
    if (cmd == "resampleleaf" && argc == 6)
        return cmd_resampleleaf(argv[2], atoi(argv[3]), atoi(argv[4]), argv[5]);
    if (cmd == "addthread" && argc == 6)
        return cmd_addthread(argv[2], argv[3], argv[4], argv[5]);
    if (cmd == "recomb" && argc == 6)
        return cmd_recomb(argv[2], argv[3], atoi(argv[4]), argv[5]);
    if (cmd == "ingest" && argc == 6)
        return cmd_ingest(argv[2], argv[3], atoi(argv[4]), argv[5]);
    if (cmd == "sim1" && argc == 6) return cmd_sim1(argv[2], argv[3], atoi(argv[4]), argv[5]);
    if (cmd == "removalpaths" && argc == 7)
        return cmd_removalpaths(argv[2], atoi(argv[3]), atoi(argv[4]), atoi(argv[5]), argv[6]);
    if (cmd == "cut" && argc == 5) return cmd_cut(argv[2], atoi(argv[3]), argv[4]);
    die("bad arguments");
    return 1;
}

// The in-process C++ seam of the threading HMM, for programs that link the reference's
// library (arg-sample): this file replaces the reference's sample_thread.o. It defines the
// functions sample_thread.h declares (sample_thread.h:130-160) with the same signatures and
// meaning, and runs the forward pass and the stochastic traceback through this library's
// C ABI (awg_run_batch, FP64: the drop-in path, its forward table within 1e-12 relative of
// the reference's and its sampled path the reference's given the same rand() draws). The
// rest of a threading step stays the reference's own code, called as the reference calls
// it: sample_recombinations (recomb.cpp:151) and add_arg_thread / add_arg_thread_path
// (thread.cpp:272,1314).
//
// It compiles against the reference's headers (sample_thread.h and what it includes) and
// links with the reference's other objects; oracle/Makefile target `seam` builds arg-sample
// that way. Randomness is unchanged: the traceback draws one rand() per column, last column
// first, as stochastic_traceback does, so arg-sample's srand(seed) gives the same ARGs.
//
// The conditioned samplers (cond_sample_arg_thread[_internal], arg-sample's MCMC moves over
// regions) run through awg_sample_path_conditioned: a given first forward column and a given
// last state, drawing as the reference does. Not carried over (the call aborts with a
// message): unphased sequences (PhaseProbs), rates that change along the genome
// (ArgModel::mutmap / recombmap holding more than one value; constant maps, arg-sample's
// default, are accepted), and arghmm_forward_alg's prior_given / stochastic_traceback's
// last_state_given when called on their own.

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "sample_thread.h"  // the reference's declarations

#include "argweaver_gb300.h"

namespace argweaver {

namespace {

// new_chrom of an ArgHmmMatrixIter (a protected member): a pointer to member taken in a
// derived class's scope names the base member and may be applied to any base object.
struct MatrixIterAccess : ArgHmmMatrixIter {
    static int new_chrom_of(const ArgHmmMatrixIter *m) {
        return m->*(&MatrixIterAccess::new_chrom);
    }
};

[[noreturn]] void fail(const char *what, const char *detail) {
    fprintf(stderr, "argweaver_gb300 seam: %s%s%s\n", what, detail && *detail ? ": " : "",
            detail ? detail : "");
    abort();
}

// One threading problem of the reference's objects as this library's flat arrays.
struct Flat {
    std::vector<int> ptrees, ages, sprs, blocklens, mapping, rc0;
    std::vector<char> seqs;
    awg_problem p{};
    std::vector<int> nstates;  // states of each tree (the forward table's row lengths)
};

// The rate of a map that holds one value over the whole region (arg-sample builds constant
// maps from --mutrate / --recombrate when no map file is given), else the model's own rate
// when there is no map; a map whose rate changes along the region is refused.
double constant_rate(const Track<double> &map, double rate, const char *what) {
    if (map.size() == 0) return rate;
    const double v = map[0].value;
    for (unsigned int i = 1; i < map.size(); i++)
        if (map[i].value != v) fail(what, "a rate that changes along the region is not supported "
                                          "by the GPU path");
    return v;
}

void flatten(const LocalTrees *trees, const ArgModel *model, const Sequences *sequences,
             int new_chrom, bool internal, int minage, Flat &f) {
    if (model->unphased) fail("unphased sequences are not supported by the GPU path", nullptr);
    const double mu = constant_rate(model->mutmap, model->mu, "mutation map");
    const double rho = constant_rate(model->recombmap, model->rho, "recombination map");
    const int nn = trees->nnodes, B = trees->get_num_trees(), L = trees->length();
    f.ptrees.assign((size_t)B * nn, -1);
    f.ages.assign((size_t)B * nn, 0);
    f.sprs.assign((size_t)B * 4, -1);
    f.blocklens.assign(B, 0);
    f.mapping.assign((size_t)B * nn, -1);
    f.rc0.assign(B, -1);
    f.nstates.assign(B, 0);
    StatesModel states_model(model->ntimes, internal, minage);
    States states;
    int b = 0;
    for (LocalTrees::const_iterator it = trees->begin(); it != trees->end(); ++it, ++b) {
        const LocalTree *t = it->tree;
        for (int i = 0; i < nn; i++) {
            f.ptrees[(size_t)b * nn + i] = t->nodes[i].parent;
            f.ages[(size_t)b * nn + i] = t->nodes[i].age;
            if (b > 0 && it->mapping) f.mapping[(size_t)b * nn + i] = it->mapping[i];
        }
        f.rc0[b] = t->nodes[t->root].child[0];
        f.sprs[(size_t)b * 4 + 0] = it->spr.recomb_node;
        f.sprs[(size_t)b * 4 + 1] = it->spr.recomb_time;
        f.sprs[(size_t)b * 4 + 2] = it->spr.coal_node;
        f.sprs[(size_t)b * 4 + 3] = it->spr.coal_time;
        f.blocklens[b] = it->blocklen;
        states_model.get_coal_states(t, states);
        f.nstates[b] = (int)states.size();
    }
    // leaf i reads the sequence it holds (LocalTrees::seqids); an external problem adds the
    // sequence being threaded as the last row
    const int nleaves = trees->get_num_leaves();
    const int nrows = nleaves + (internal ? 0 : 1);
    const char *const *rows = sequences->get_seqs();
    f.seqs.resize((size_t)nrows * L);
    for (int r = 0; r < nrows; r++) {
        const int sid = r < nleaves ? ((int)trees->seqids.size() > r ? trees->seqids[r] : r)
                                    : new_chrom;
        if (sid < 0 || sid >= sequences->get_num_seqs()) fail("a leaf names no sequence", nullptr);
        const char *src = rows[sid] + trees->start_coord;
        std::copy(src, src + L, f.seqs.begin() + (size_t)r * L);
    }
    awg_problem &p = f.p;
    p.ntrees = B;
    p.nnodes = nn;
    p.ntimes = model->ntimes;
    p.nseqs = nrows;
    p.seqlen = L;
    p.internal = internal ? 1 : 0;
    p.start_coord = trees->start_coord;
    p.minage = minage;
    p.ptrees = f.ptrees.data();
    p.ages = f.ages.data();
    p.sprs = f.sprs.data();
    p.blocklens = f.blocklens.data();
    p.mapping = f.mapping.data();
    p.root_child0 = f.rc0.data();
    p.times = model->times;
    p.popsizes = model->popsizes;
    p.rho = rho;
    p.mu = mu;
    p.seqs = f.seqs.data();
    p.infsites_penalty = model->infsites_penalty;
}

// Forward pass (FP64) and, when path is not NULL, the traceback drawing from rand() in the
// reference's order; the packed table into `table` when not NULL.
void run(const Flat &f, std::vector<double> *table, int *path) {
    awg_outputs out{};
    if (table) {
        const long long cells = awg_problem_cells(&f.p);
        if (cells < 0) fail("awg_problem_cells", awg_last_error());
        table->resize((size_t)cells);
        out.forward = table->data();
    }
    out.path = path;
    out.uniforms = nullptr;  // libc rand(), one per column, last column first
    if (awg_run_batch(&f.p, &out, 1, AWG_FP64) != 0) fail("awg_run_batch", awg_last_error());
}

// The packed table into the reference's forward table, one block per local tree.
void fill_table(const LocalTrees *trees, const Flat &f, const std::vector<double> &table,
                ArgHmmForwardTable *forward) {
    double **fw = forward->get_table();
    size_t off = 0;
    int start = trees->start_coord, b = 0;
    for (LocalTrees::const_iterator it = trees->begin(); it != trees->end(); ++it, ++b) {
        const int end = start + it->blocklen;
        const int S = std::max(f.nstates[b], 1);
        forward->new_block(start, end, S);
        for (int i = start; i < end; i++) {
            std::copy(table.begin() + off, table.begin() + off + S, fw[i]);
            off += S;
        }
        start = end;
    }
}

// A threading step after the path is known: recombinations and the new thread, with the
// reference's own code (sample_thread.cpp:610-622, 675-688).
void finish_external(const ArgModel *model, Sequences *sequences, LocalTrees *trees,
                     int new_chrom, int *thread_path) {
    ArgHmmMatrixIter matrix_iter(model, sequences, trees, new_chrom);
    ArgHmmMatrixIter matrix_iter2(model, NULL, trees, new_chrom);
    vector<int> recomb_pos;
    vector<NodePoint> recombs;
    sample_recombinations(trees, model, &matrix_iter2, thread_path, recomb_pos, recombs);
    add_arg_thread(trees, matrix_iter.states_model, model->ntimes, thread_path, new_chrom,
                   recomb_pos, recombs);
}

}  // namespace

void arghmm_forward_alg(const LocalTrees *trees, const ArgModel *model,
                        const Sequences *sequences, ArgHmmMatrixIter *matrix_iter,
                        ArgHmmForwardTable *forward, PhaseProbs *phase_pr, bool prior_given,
                        bool internal, bool slow) {
    (void)slow;  // the dense step gives the same table; the structured one runs
    if (phase_pr) fail("unphased sequences are not supported by the GPU path", nullptr);
    if (prior_given) fail("a given first forward column is not supported by the GPU path", nullptr);
    Flat f;
    flatten(trees, model, sequences, MatrixIterAccess::new_chrom_of(matrix_iter), internal,
            matrix_iter->states_model.minage, f);
    std::vector<double> table;
    run(f, &table, nullptr);
    fill_table(trees, f, table, forward);
}

double stochastic_traceback(const LocalTrees *trees, const ArgModel *model,
                            ArgHmmMatrixIter *matrix_iter, double **fw, int *path,
                            bool last_state_given, bool internal) {
    (void)fw;  // the device recomputes the forward table it samples from (the same values)
    if (last_state_given)
        fail("a given last traceback state is not supported by the GPU path", nullptr);
    // the traceback iterator carries no sequences; the forward pass needs the ones the
    // forward call used, which the reference's callers pass through the same trees and
    // model: this entry point is served by the threading steps below, which run forward
    // and traceback in one call
    (void)trees;
    (void)model;
    (void)matrix_iter;
    (void)path;
    (void)internal;
    fail("stochastic_traceback alone is not supported by the GPU path (the threading steps "
         "run forward and traceback together)", nullptr);
}

void sample_arg_thread(const ArgModel *model, Sequences *sequences, LocalTrees *trees,
                       int new_chrom) {
    Flat f;
    flatten(trees, model, sequences, new_chrom, false, 0, f);
    std::vector<int> alloc(trees->length());
    run(f, nullptr, alloc.data());
    finish_external(model, sequences, trees, new_chrom, alloc.data() - trees->start_coord);
}

void sample_arg_thread_internal(const ArgModel *model, const Sequences *sequences,
                                LocalTrees *trees, int minage, PhaseProbs *phase_pr) {
    if (phase_pr) fail("unphased sequences are not supported by the GPU path", nullptr);
    Flat f;
    flatten(trees, model, sequences, -1, true, minage, f);
    std::vector<int> alloc(trees->length());
    run(f, nullptr, alloc.data());
    int *thread_path = alloc.data() - trees->start_coord;
    ArgHmmMatrixIter matrix_iter(model, sequences, trees);
    matrix_iter.set_internal(true, minage);
    ArgHmmMatrixIter matrix_iter2(model, NULL, trees);
    matrix_iter2.set_internal(true, minage);
    vector<int> recomb_pos;
    vector<NodePoint> recombs;
    sample_recombinations(trees, model, &matrix_iter2, thread_path, recomb_pos, recombs, true);
    add_arg_thread_path(trees, matrix_iter.states_model, model->ntimes, thread_path,
                        recomb_pos, recombs);
}

void resample_arg_thread(const ArgModel *model, Sequences *sequences, LocalTrees *trees,
                         int chrom) {
    remove_arg_thread(trees, chrom);
    sample_arg_thread(model, sequences, trees, chrom);
}

namespace {

// The conditioned threading step's path (cond_sample_arg_thread[_internal],
// sample_thread.cpp:708-865): the first forward column holds 1 at start_state (the state
// priors when start_state is null and the tree has states; 1 for a tree without states),
// the last column's state is end_state (drawn when null and the tree has states; 0 for a
// tree without states, with no draw).
void conditioned_path(const Flat &f, const LocalTrees *trees, const StatesModel &states_model,
                      const State &start_state, const State &end_state, int *thread_path) {
    States states;
    std::vector<double> prior;
    bool prior_given = true;
    states_model.get_coal_states(trees->front().tree, states);
    if (states.size() > 0) {
        if (!start_state.is_null()) {
            const int j = find_vector(states, start_state);
            if (j == -1) fail("the start state is not a state of the first tree", nullptr);
            prior.assign(states.size(), 0.0);
            prior[j] = 1.0;
        } else {
            prior_given = false;
        }
    } else {
        prior.assign(1, 1.0);
    }
    states_model.get_coal_states(trees->back().tree, states);
    int last = -1;
    if (states.size() > 0) {
        if (!end_state.is_null()) {
            last = find_vector(states, end_state);
            if (last == -1) fail("the end state is not a state of the last tree", nullptr);
        }
    } else {
        last = 0;
    }
    if (awg_sample_path_conditioned(&f.p, prior_given ? prior.data() : nullptr, last, nullptr,
                                    thread_path + trees->start_coord, nullptr) != 0)
        fail("awg_sample_path_conditioned", awg_last_error());
}

}  // namespace

void cond_sample_arg_thread(const ArgModel *model, const Sequences *sequences,
                            LocalTrees *trees, int new_chrom, State start_state,
                            State end_state) {
    Flat f;
    flatten(trees, model, sequences, new_chrom, false, 0, f);
    std::vector<int> alloc(trees->length());
    int *thread_path = alloc.data() - trees->start_coord;
    StatesModel states_model(model->ntimes, false, 0);
    conditioned_path(f, trees, states_model, start_state, end_state, thread_path);
    // recombinations and the new thread (sample_thread.cpp:758-770): the reference's code
    ArgHmmMatrixList matrix_list(model, sequences, trees, new_chrom);
    matrix_list.setup();
    vector<int> recomb_pos;
    vector<NodePoint> recombs;
    sample_recombinations(trees, model, &matrix_list, thread_path, recomb_pos, recombs);
    add_arg_thread(trees, matrix_list.states_model, model->ntimes, thread_path, new_chrom,
                   recomb_pos, recombs);
}

void cond_sample_arg_thread_internal(const ArgModel *model, const Sequences *sequences,
                                     LocalTrees *trees, State start_state, State end_state) {
    Flat f;
    flatten(trees, model, sequences, -1, true, 0, f);
    std::vector<int> alloc(trees->length());
    int *thread_path = alloc.data() - trees->start_coord;
    StatesModel states_model(model->ntimes, true, 0);
    conditioned_path(f, trees, states_model, start_state, end_state, thread_path);
    // recombinations and the regraft (sample_thread.cpp:848-860): the reference's code
    ArgHmmMatrixIter matrix_iter(model, sequences, trees);
    matrix_iter.set_internal(true);
    ArgHmmMatrixIter matrix_iter2(model, NULL, trees);
    matrix_iter2.set_internal(true);
    vector<int> recomb_pos;
    vector<NodePoint> recombs;
    sample_recombinations(trees, model, &matrix_iter2, thread_path, recomb_pos, recombs, true);
    add_arg_thread_path(trees, matrix_iter.states_model, model->ntimes, thread_path,
                        recomb_pos, recombs);
}

}  // namespace argweaver

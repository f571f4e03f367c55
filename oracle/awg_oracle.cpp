// CPU restatement of the reference's chromosome-threading HMM (ARGweaver).
//
// TEST INFRASTRUCTURE, NOT PRODUCT: the checker for the CUDA path and the timed CPU port
// of the reference (bench.py's CPU leg). Nothing under argweaver_gb300/ links it. It
// follows the reference's algorithm step by step, in the same floating-point operation
// order, so that on the same host it reproduces the reference's numbers; it is pinned
// against the compiled reference by the fixtures in tests/golden/.
//
// Reference map (paths inside the reference project):
//   model time grid            src/argweaver/model.h:21-32, 322-333; model.cpp:9-23
//   local trees                src/argweaver/local_tree.h:190-230 (set_ptree), 767 (mapping)
//   lineage counts             src/argweaver/local_tree.cpp:34-131
//   tree lengths               src/argweaver/local_tree.cpp:136-219
//   state spaces               src/argweaver/states.cpp:53-167; states.h:53-131 (lookup)
//   transition matrix          src/argweaver/trans.cpp:13-115; trans.h:64-128
//   switch matrix              src/argweaver/trans.cpp:156-739; trans.h:207-219
//   state priors               src/argweaver/trans.cpp:785-831
//   emissions                  src/argweaver/emit.cpp:86-93, 97-116, 151-324, 620-869
//   forward                    src/argweaver/sample_thread.cpp:186-296, 345-460
//   traceback                  src/argweaver/sample_thread.cpp:470-569; common.h:272-290
// The backward pass and posterior marginals have no counterpart in the reference; they
// use the reference's transition semantics (TransMatrix::get, TransMatrixSwitch::get).

#include "awg_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace {

using std::vector;

struct Tree {
    int n = 0, root = -1;
    vector<int> parent, c0, c1, age;
    bool leaf(int v) const { return c0[v] == -1; }
    int sibling(int v) const {
        int p = parent[v];
        if (p == -1) return -1;
        return c0[p] == v ? c1[p] : c0[p];
    }
    double dist(int v, const double *times) const {
        int p = parent[v];
        return p != -1 ? times[age[p]] - times[age[v]] : 0.0;
    }
    int nleaves() const { return (n + 1) / 2; }
};

struct Model {
    int T = 0;
    vector<double> times, time_steps, coal_time_steps, popsizes;
    double rho = 0, mu = 0;
    double infsites_penalty = 1.0;  // model.h:53 (1: off)
    double mintime() const { return times[1] * .1; }
    int removed_root_time() const { return T + 1; }
};

struct States {
    vector<int> node, time;
    int size() const { return (int)node.size(); }
    void clear() { node.clear(); time.clear(); }
    void push(int v, int t) { node.push_back(v); time.push_back(t); }
};

// NodeStateLookup (states.h:53-131): states of a node are contiguous, time increasing.
struct Lookup {
    vector<int> first, t0, count;
    const States *st = nullptr;
    void build(const States &s, int nnodes) {
        st = &s;
        first.assign(nnodes, -1); t0.assign(nnodes, 0); count.assign(nnodes, 0);
        for (int i = 0; i < s.size(); i++) {
            int v = s.node[i];
            if (count[v] == 0) { first[v] = i; t0[v] = s.time[i]; }
            count[v]++;
        }
    }
    int lookup(int v, int t) const {
        if (v < 0 || count[v] == 0) return -1;
        int d = t - t0[v];
        if (d < 0 || d >= count[v]) return -1;
        int i = first[v] + d;
        if (st->node[i] != v || st->time[i] != t) return -1;
        return i;
    }
};

struct Lineages {
    vector<int> nbranches, nrecombs, ncoals;
};

struct TransMatrix {
    int nstates = 0;
    bool internal = false;
    int minage = 0;
    vector<double> D, E, lnB, lnE2, lnNegG1, G2, G3, lnG4, norecombs;

    double get_time(int a, int b, int c, int minage_, bool same_node) const {
        if (a < minage_ || b < minage_) return 0.0;
        double term1 = D[a] * E[b];
        double minage_term = 0.0;
        if (minage_ > 0) minage_term = exp(lnG4[b] + lnB[minage_ - 1]);
        if (!same_node) {
            if (a < b) {
                return term1 * (exp(lnE2[b] + lnB[a]) - exp(lnE2[b] + lnNegG1[a]) - minage_term);
            } else if (a == b) {
                return term1 * ((b > 0 ? exp(lnE2[b] + lnB[b - 1]) : 0.0) + G3[b] - minage_term);
            } else {
                return term1 * ((b > 0 ? exp(lnE2[b] + lnB[b - 1]) : 0.0) + G2[b] - minage_term);
            }
        } else {
            double c_term = (c > 0 ? exp(lnG4[b] + lnB[c - 1]) : 0.0);
            if (a < b) {
                return term1 * (2 * (exp(lnE2[b] + lnB[a]) - exp(lnE2[b] + lnNegG1[a])) -
                                c_term - minage_term);
            } else if (a == b) {
                return term1 * ((2 * ((b > 0 ? exp(lnE2[b] + lnB[b - 1]) : 0.0) + G3[b])) -
                                c_term - minage_term) +
                       norecombs[a];
            } else {
                return term1 * ((2 * ((b > 0 ? exp(lnE2[b] + lnB[b - 1]) : 0.0) + G2[b])) -
                                c_term - minage_term);
            }
        }
    }

    // TransMatrix::get (trans.h:64-83)
    double get(const Tree &t, const States &s, int i, int j) const {
        int ma = 0;
        if (internal) {
            if (nstates == 0) return 1.0;
            ma = t.age[t.c0[t.root]];
        }
        const int a = s.time[i], b = s.time[j], c = t.age[s.node[j]];
        return get_time(a, b, c, ma, s.node[i] == s.node[j]);
    }
};

struct SwitchMatrix {
    int nstates1 = 0, nstates2 = 0, recoalsrc = -1, recombsrc = -1;
    vector<int> determ;
    vector<double> determprob, recoalrow, recombrow;
    void allocate(int n1, int n2) {
        nstates1 = n1; nstates2 = n2;
        determ.assign(std::max(n1, 1), -1);
        determprob.assign(std::max(n1, 1), 0.0);
        recoalrow.assign(std::max(n2, 1), 0.0);
        recombrow.assign(std::max(n2, 1), 0.0);
    }
    double get(int i, int j) const {  // trans.h:207-219
        if (i == recoalsrc) return recoalrow[j];
        if (i == recombsrc) return recombrow[j];
        return determ[i] == j ? determprob[i] : 0.0;
    }
};

struct Spr { int recomb_node, recomb_time, coal_node, coal_time; };

// ---------------------------------------------------------------------------------------
// problem → model, trees

int dna2int(char c) {
    switch (c) {
        case 'A': case 'a': return 0;
        case 'C': case 'c': return 1;
        case 'G': case 'g': return 2;
        case 'T': case 't': return 3;
        default: return -1;
    }
}

bool build_model(const oracle_problem *p, Model &m) {
    const int T = p->ntimes;
    if (T < 3) return false;
    m.T = T;
    m.times.assign(p->times, p->times + T);
    m.popsizes.assign(p->popsizes, p->popsizes + T);
    m.rho = p->rho;
    m.mu = p->mu;
    m.infsites_penalty =
        (p->infsites_penalty > 0.0 && p->infsites_penalty < 1.0) ? p->infsites_penalty : 1.0;
    m.time_steps.assign(T, 0.0);
    for (int i = 0; i < T - 1; i++) m.time_steps[i] = m.times[i + 1] - m.times[i];
    m.time_steps[T - 1] = INFINITY;
    // get_coal_time_steps (model.cpp:9-23); entries the reference leaves unset are never
    // read on the HMM path and are given their natural values here.
    vector<double> times2(2 * T + 1, 0.0);
    for (int i = 0; i < T - 1; i++) {
        times2[2 * i] = m.times[i];
        times2[2 * i + 1] = sqrt((m.times[i + 1] + 1.0) * (m.times[i] + 1.0));
    }
    times2[2 * T - 2] = m.times[T - 1];
    times2[2 * T - 1] = m.times[T - 1];
    times2[2 * T] = m.times[T - 1];
    m.coal_time_steps.assign(2 * T, 0.0);
    for (int i = 0; i < 2 * T - 2; i++)
        m.coal_time_steps[i] = times2[std::min(i + 1, 2 * T)] - times2[i];
    m.coal_time_steps[2 * T - 2] = INFINITY;
    m.coal_time_steps[2 * T - 1] = INFINITY;
    return true;
}

struct Arg {
    vector<Tree> trees;
    vector<Spr> sprs;
    vector<vector<int>> mapping;
    vector<int> blocklen, start;
};

bool build_arg(const oracle_problem *p, Arg &arg) {
    const int n = p->nnodes, B = p->ntrees, T = p->ntimes;
    if (n < 1 || B < 1) return false;
    arg.trees.resize(B);
    arg.sprs.resize(B);
    arg.mapping.assign(B, vector<int>());
    arg.blocklen.resize(B);
    arg.start.resize(B);
    int pos = 0;
    for (int b = 0; b < B; b++) {
        Tree &t = arg.trees[b];
        t.n = n;
        t.parent.assign(p->ptrees + (size_t)b * n, p->ptrees + (size_t)(b + 1) * n);
        t.age.assign(p->ages + (size_t)b * n, p->ages + (size_t)(b + 1) * n);
        t.c0.assign(n, -1);
        t.c1.assign(n, -1);
        t.root = -1;
        for (int i = 0; i < n; i++) {  // set_ptree (local_tree.h:216-229)
            int par = t.parent[i];
            if (par < -1 || par >= n) return false;
            if (par != -1) {
                if (t.c0[par] == -1) t.c0[par] = i;
                else if (t.c1[par] == -1) t.c1[par] = i;
                else return false;
            } else {
                t.root = i;
            }
            if (t.age[i] < 0 || t.age[i] > T + 1) return false;
        }
        if (t.root < 0) return false;
        if (p->root_child0 && p->root_child0[b] != -1 && t.c0[t.root] != p->root_child0[b]) {
            if (t.c1[t.root] != p->root_child0[b]) return false;
            std::swap(t.c0[t.root], t.c1[t.root]);
        }
        const int *s = p->sprs + (size_t)b * 4;
        arg.sprs[b] = Spr{s[0], s[1], s[2], s[3]};
        arg.blocklen[b] = p->blocklens[b];
        if (p->blocklens[b] < 1) return false;
        arg.start[b] = pos;
        pos += p->blocklens[b];
        if (b > 0) {
            vector<int> &mp = arg.mapping[b];
            if (p->mapping) {
                mp.assign(p->mapping + (size_t)b * n, p->mapping + (size_t)(b + 1) * n);
            } else {  // make_node_mapping (local_tree.h:767-776)
                if (s[0] < 0 || s[0] >= n) return false;
                mp.resize(n);
                for (int j = 0; j < n; j++) mp[j] = j;
                int broken = p->ptrees[(size_t)(b - 1) * n + s[0]];
                if (broken < 0) return false;
                mp[broken] = -1;
            }
            if (s[0] < 0 || s[0] >= n || s[2] < 0 || s[2] >= n) return false;
        }
    }
    if (pos != p->seqlen) return false;
    for (int i = 0; i < p->nseqs * p->seqlen; i++) {
        char c = p->seqs[i];
        if (c != 'N' && dna2int(c) < 0) return false;
    }
    const int nleaves = (n + 1) / 2;
    if (p->internal ? p->nseqs < nleaves : p->nseqs < nleaves + 1) return false;
    return true;
}

// ---------------------------------------------------------------------------------------
// state spaces, lineages, tree lengths

void coal_states_external(const Tree &t, int T, States &s) {  // states.cpp:53-74
    s.clear();
    for (int i = 0; i < t.n; i++) {
        int time = t.age[i];
        const int parent = t.parent[i];
        if (parent == -1) {
            for (; time < T - 1; time++) s.push(i, time);
        } else {
            const int parent_age = t.age[parent];
            for (; time <= parent_age; time++) s.push(i, time);
        }
    }
}

void coal_states_internal(const Tree &t, int T, States &s, int minage) {  // states.cpp:109-167
    s.clear();
    if (t.age[t.root] < T) return;  // fully specified tree
    const int subtree_root = t.c0[t.root];
    minage = std::max(minage, t.age[subtree_root]);
    vector<char> ignore(t.n, 0);
    ignore[t.root] = 1;
    vector<int> stack{subtree_root};
    while (!stack.empty()) {
        int v = stack.back();
        stack.pop_back();
        ignore[v] = 1;
        if (!t.leaf(v)) { stack.push_back(t.c0[v]); stack.push_back(t.c1[v]); }
    }
    for (int i = 0; i < t.n; i++) {
        int time = std::max(t.age[i], minage);
        const int parent = t.parent[i];
        if (ignore[i]) continue;
        if (parent == t.root) {
            for (; time < T - 1; time++) s.push(i, time);
        } else {
            const int parent_age = t.age[parent];
            for (; time <= parent_age; time++) s.push(i, time);
        }
    }
}

void coal_states(const Tree &t, int T, bool internal, int minage, States &s) {
    if (internal) coal_states_internal(t, T, s, minage);
    else coal_states_external(t, T, s);
}

void count_lineages(const Tree &t, int T, Lineages &l) {  // local_tree.cpp:34-69
    l.nbranches.assign(T, 0); l.nrecombs.assign(T, 0); l.ncoals.assign(T, 0);
    for (int i = 0; i < t.n; i++) {
        const int parent = t.parent[i];
        const int parent_age = (parent == -1) ? T - 2 : t.age[parent];
        for (int j = t.age[i]; j < parent_age; j++) {
            l.nbranches[j]++; l.nrecombs[j]++; l.ncoals[j]++;
        }
        l.nrecombs[parent_age]++;
        l.ncoals[parent_age]++;
        if (parent == -1) l.nbranches[parent_age]++;
    }
    l.nbranches[T - 1] = 1;
}

void count_lineages_internal(const Tree &t, int T, Lineages &l) {  // local_tree.cpp:82-131
    const int subtree_root = t.c0[t.root];
    const int minage = t.age[subtree_root];
    l.nbranches.assign(T, 0); l.nrecombs.assign(T, 0); l.ncoals.assign(T, 0);
    for (int i = 0; i < t.n; i++) {
        if (i == subtree_root || i == t.root) continue;
        const int parent = t.parent[i];
        const int parent_age = (parent == t.root) ? T - 2 : t.age[parent];
        for (int j = t.age[i]; j < parent_age; j++) {
            l.nbranches[j]++; l.nrecombs[j]++; l.ncoals[j]++;
        }
        l.nrecombs[parent_age]++;
        l.ncoals[parent_age]++;
        if (parent == t.root) l.nbranches[parent_age]++;
    }
    for (int i = 0; i < minage; i++) {
        l.nbranches[i]--; l.ncoals[i]--; l.nrecombs[i]--;
    }
    l.nbranches[T - 1] = 1;
}

void count(const Tree &t, int T, bool internal, Lineages &l) {
    if (internal) count_lineages_internal(t, T, l);
    else count_lineages(t, T, l);
}

double get_treelen(const Tree &t, const double *times, bool use_basal) {
    double treelen = 0.0;
    for (int i = 0; i < t.n; i++) {
        int parent = t.parent[i], age = t.age[i];
        if (parent == -1) {
            if (use_basal) treelen += times[age + 1] - times[age];
        } else {
            treelen += times[t.age[parent]] - times[age];
        }
    }
    return treelen;
}

double get_treelen_internal(const Tree &t, const double *times) {
    double treelen = 0.0;
    for (int i = 0; i < t.n; i++) {
        int parent = t.parent[i], age = t.age[i];
        if (parent == t.root || parent == -1) {
        } else {
            treelen += times[t.age[parent]] - times[age];
        }
    }
    return treelen;
}

double get_treelen_branch(const Tree &t, const double *times, int node, int time,
                          double treelen, bool use_basal) {
    double root_time;
    int rooti = t.age[t.root];
    if (treelen < 0.0) treelen = get_treelen(t, times, false);
    double blen = times[time];
    double treelen2 = treelen + blen;
    if (node == t.root) {
        treelen2 += blen - times[t.age[t.root]];
        root_time = times[time + 1] - times[time];
    } else {
        rooti = t.age[t.root];
        root_time = times[rooti + 1] - times[rooti];
    }
    return use_basal ? treelen2 + root_time : treelen2;
}

double get_basal_branch(const Tree &t, const double *times, int node, int time) {
    if (node == t.root) return times[time + 1] - times[time];
    int rooti = t.age[t.root];
    return times[rooti + 1] - times[rooti];
}

inline double logadd(double lna, double lnb) {  // common.h:157-163
    if (lna == -INFINITY) return lnb;
    if (lnb == -INFINITY) return lna;
    return std::max(lna, lnb) + log1p(exp(-fabs(lna - lnb)));
}

// ---------------------------------------------------------------------------------------
// transition matrices

void calc_transition_probs(const Tree &t, const Model &m, const States &states,
                           const Lineages &l, TransMatrix &mat, bool internal, int minage) {
    const int T = m.T;
    const double *times = m.times.data();
    const double *time_steps = m.time_steps.data();
    const double rho = m.rho;
    const int *nbranches = l.nbranches.data();
    const int *nrecombs = l.nrecombs.data();
    const int *ncoals = l.ncoals.data();
    mat.nstates = states.size();
    mat.internal = internal;
    mat.minage = minage;
    mat.D.assign(T, 0); mat.E.assign(T, 0); mat.lnB.assign(T, 0); mat.lnE2.assign(T, 0);
    mat.lnNegG1.assign(T, 0); mat.G2.assign(T, 0); mat.G3.assign(T, 0);
    mat.lnG4.assign(T, 0); mat.norecombs.assign(T, 0);

    // calc_coal_rates_partial_tree (trans.cpp:13-21)
    vector<double> coal_rates_alloc(2 * T + 1);
    double *coal_rates = &coal_rates_alloc[1];
    coal_rates[-1] = 0.0;
    for (int i = 0; i < 2 * T; i++)
        coal_rates[i] = m.coal_time_steps[i] * nbranches[i / 2] / (2.0 * m.popsizes[i / 2]);
    vector<double> C_alloc(2 * T + 2);
    double *C = &C_alloc[2];
    C[-2] = 0.0;
    C[-1] = 0.0;
    for (int b = 0; b < 2 * T - 1; b++) C[b] = C[b - 1] + coal_rates[b];

    int root_age_index;
    double root_age, treelen;
    if (internal) {
        const int subtree_root = t.c0[t.root];
        const int maintree_root = t.c1[t.root];
        const double subtree_age = times[t.age[subtree_root]];
        root_age_index = t.age[maintree_root];
        root_age = times[root_age_index];
        treelen = get_treelen_internal(t, times) - subtree_age;
        mat.minage = std::max(mat.minage, t.age[subtree_root]);
    } else {
        root_age_index = t.age[t.root];
        root_age = times[root_age_index];
        treelen = get_treelen(t, times, false);
    }

    for (int b = 0; b < T - 1; b++) {
        double treelen2 = treelen + times[b];
        double treelen2_b;
        if (b > root_age_index) {
            treelen2 += times[b] - root_age;
            treelen2_b = treelen2 + time_steps[b];
        } else {
            treelen2_b = treelen2 + time_steps[root_age_index];
        }
        double term = C[2 * b - 1] + log(time_steps[b] * (nbranches[b] + 1.0) / (nrecombs[b] + 1.0));
        if (b == 0) mat.lnB[b] = term;
        else mat.lnB[b] = logadd(mat.lnB[b - 1], term);
        mat.lnE2[b] = -C[2 * b - 2] +
            (b < T - 2 ? log(1 - exp(-coal_rates[2 * b] - coal_rates[2 * b - 1])) : 0.0);
        mat.lnNegG1[b] = C[2 * b - 1] + log(-time_steps[b] *
            ((nbranches[b] / (nrecombs[b] + 1.0 + int(b < root_age_index))) -
             (nbranches[b] + 1.0) / (nrecombs[b] + 1.0)));
        mat.G2[b] = (b < T - 2 ? 1.0 - exp(-coal_rates[2 * b]) : 1.0) * time_steps[b] *
                    (nbranches[b] + 1.0) / (nrecombs[b] + 1.0);
        mat.G3[b] = (b < T - 2 ? 1.0 - exp(-coal_rates[2 * b]) : 1.0) * time_steps[b] *
                    (nbranches[b] / (nrecombs[b] + 1.0 + int(b < root_age_index)));
        mat.lnG4[b] = -C[2 * b - 2] +
            (b < T - 2 ? log(1.0 - exp(-coal_rates[2 * b] - coal_rates[2 * b - 1])) : 0.0);
        mat.D[b] = (1.0 - exp(-rho * treelen2)) / treelen2_b;
        mat.E[b] = 1.0 / ncoals[b];
        mat.norecombs[b] = exp(-std::max(rho * treelen2, rho));
    }
    mat.E[T - 2] = 1.0 / ncoals[T - 2];
}

// get_deterministic_transitions (trans.cpp:156-275)
void deterministic_transitions(const Tree &last, const Tree &t, const Spr &spr,
                               const vector<int> &mapping, const States &states1,
                               const Lookup &lk2, int *next_states, bool internal) {
    const int nstates1 = states1.size();
    for (int i = 0; i < nstates1; i++) {
        const int node1 = states1.node[i];
        const int time1 = states1.time[i];
        if ((node1 == spr.coal_node && time1 == spr.coal_time) ||
            (node1 == spr.recomb_node && time1 == spr.recomb_time)) {
            next_states[i] = -1;
        } else if (node1 != spr.recomb_node) {
            int node2;
            bool disrupt = false;
            if (last.c0[node1] == -1) {
                node2 = node1;
            } else {
                const int child1 = last.c0[node1], child2 = last.c1[node1];
                if (spr.recomb_node == child1) { node2 = mapping[child2]; disrupt = true; }
                else if (spr.recomb_node == child2) { node2 = mapping[child1]; disrupt = true; }
                else node2 = mapping[node1];
            }
            const int mcoal = mapping[spr.coal_node];
            if ((spr.coal_node == node1 && spr.coal_time < time1) ||
                (mcoal == node2 && spr.coal_time < time1) ||
                (disrupt && mcoal == node2 && spr.coal_time <= time1)) {
                node2 = t.parent[node2];
            }
            if (internal && t.age[node2] > time1) { next_states[i] = -1; continue; }
            const int p = t.parent[node2];
            if (p != -1) {
                if (internal && time1 > t.age[p]) { next_states[i] = -1; continue; }
            }
            next_states[i] = lk2.lookup(node2, time1);
        } else {
            if (spr.recomb_time > time1) {
                next_states[i] = lk2.lookup(mapping[spr.recomb_node], time1);
            } else {
                const int parent = last.parent[spr.recomb_node];
                const int time2 = last.age[parent];
                const int other = (last.c1[parent] == spr.recomb_node ? last.c0[parent]
                                                                         : last.c1[parent]);
                const int node2 = (other == spr.coal_node ? t.parent[mapping[other]]
                                                          : mapping[other]);
                next_states[i] = lk2.lookup(node2, time2);
            }
        }
    }
}

// calc_recomb (trans.cpp:317-413)
double calc_recomb(const Tree &last, const Model &m, const Lineages &l, const Spr &spr,
                   int state_node, int state_time, int recomb_parent_age, double last_treelen,
                   bool internal) {
    (void)recomb_parent_age;
    const int a = state_time;
    const int k = spr.recomb_time;
    double last_treelen_b;
    int root_age;
    if (internal) {
        const int subtree_root = last.c0[last.root];
        const int maintree_root = last.c1[last.root];
        root_age = last.age[maintree_root];
        if (spr.coal_node == subtree_root) {
            if (a < spr.coal_time) return 0.0;
            if (spr.recomb_node == maintree_root && state_node != maintree_root) return 0.0;
        }
        int ptr = spr.coal_node, ptr2 = -1, ptr3 = -1;
        while (ptr != last.root) { ptr2 = ptr; ptr = last.parent[ptr]; }
        ptr = spr.recomb_node;
        while (ptr != last.root) { ptr3 = ptr; ptr = last.parent[ptr]; }
        if (ptr2 == subtree_root && ptr3 == maintree_root && state_time == spr.recomb_time) {
            ptr = last.parent[state_node];
            while (ptr != last.root) {
                if (ptr == spr.recomb_node) return 0.0;
                ptr = last.parent[ptr];
            }
        }
        last_treelen += m.times[a] - m.times[last.age[subtree_root]];
        if (a > root_age) {
            last_treelen += m.times[a] - m.times[root_age];
            last_treelen_b = last_treelen + m.time_steps[a];
        } else {
            last_treelen_b = last_treelen + m.time_steps[root_age];
        }
    } else {
        root_age = last.age[last.root];
        last_treelen = get_treelen_branch(last, m.times.data(), state_node, state_time,
                                          last_treelen, false);
        last_treelen_b = last_treelen + get_basal_branch(last, m.times.data(), state_node,
                                                         state_time);
    }
    int nbranches_k = l.nbranches[k] + int(k < a);
    int nrecombs_k = l.nrecombs[k] + int(k <= a) + int(k == a) - int(k >= std::max(root_age, a));
    double p = nbranches_k * m.time_steps[k] / (nrecombs_k * last_treelen_b) *
               (1.0 - exp(-std::max(m.rho * last_treelen, m.rho)));
    return p;
}

void calc_recoal_sums(const Model &m, const Lineages &l, const Spr &spr,
                      int recomb_parent_age, double *sums, double *sums2) {
    const int k = spr.recomb_time, j = spr.coal_time;
    double sum = 0.0;
    for (int mm = 2 * k; mm < 2 * j - 1; mm++) {
        int nbranches_m = l.nbranches[mm / 2] - int(mm / 2 < recomb_parent_age);
        sum += m.coal_time_steps[mm] * nbranches_m / (2.0 * m.popsizes[mm / 2]);
    }
    *sums = sum;
    sum = 0.0;
    sums2[2 * k] = sum;
    for (int mm = 2 * k; mm < 2 * j - 1; mm++) {
        sum += m.coal_time_steps[mm] / (2.0 * m.popsizes[mm / 2]);
        sums2[mm + 1] = sum;
    }
}

double calc_recoal(const Tree &last, const Model &m, const Lineages &l, const Spr &spr,
                   int state1_time, int recomb_parent_age, bool internal) {
    const int a = state1_time, k = spr.recomb_time, j = spr.coal_time;
    int nbranches_j = l.nbranches[j] - int(j < recomb_parent_age) + int(j < a);
    int ncoals_j = l.ncoals[j] - int(j <= recomb_parent_age) - int(j == recomb_parent_age) +
                   int(j <= a) + int(j == a);
    bool over = false;
    if (internal) {
        const int subtree_root = last.c0[last.root];
        const int maintree_root = last.c1[last.root];
        if (spr.recomb_node == maintree_root) {
            if (spr.coal_time >= last.age[subtree_root]) {
                over = true;
                nbranches_j = 1;
                ncoals_j++;
            }
        }
    }
    double p = 1.0 / ncoals_j;
    if (j < m.T - 2) {
        double Z = 0.0;
        if (j > k) {
            int b1 = l.nbranches[j - 1] - int(j - 1 < recomb_parent_age) + int(j - 1 < a);
            if (over) b1 = 1;
            Z = m.coal_time_steps[2 * j - 1] * b1 / (2.0 * m.popsizes[j - 1]);
        }
        p *= 1.0 - exp(-m.coal_time_steps[2 * j] * nbranches_j / (2.0 * m.popsizes[j]) - Z);
    }
    return p;
}

double calc_recomb_recoal(const Tree &last, const Model &m, const Lineages &l, const Spr &spr,
                          int state_node, int state_time, int recomb_parent_age,
                          double last_treelen, bool internal) {
    const int a = state_time, k = spr.recomb_time, j = spr.coal_time;
    double p = calc_recomb(last, m, l, spr, state_node, state_time, recomb_parent_age,
                           last_treelen, internal);
    double sum = 0.0;
    for (int mm = 2 * k; mm < 2 * j - 1; mm++) {
        int nbranches_m = l.nbranches[mm / 2] - int(mm / 2 < recomb_parent_age) + int(mm / 2 < a);
        sum += m.coal_time_steps[mm] * nbranches_m / (2.0 * m.popsizes[mm / 2]);
    }
    p *= exp(-sum);
    p *= calc_recoal(last, m, l, spr, state_time, recomb_parent_age, internal);
    return p;
}

// calc_transition_probs_switch (trans.cpp:538-739)
bool calc_transition_probs_switch(const Tree &t, const Tree &last, const Spr &spr,
                                  const vector<int> &mapping, const States &states1,
                                  const States &states2, const Model &m, const Lineages &l,
                                  SwitchMatrix &sw, bool internal) {
    const int nstates1 = states1.size(), nstates2 = states2.size();
    sw.allocate(nstates1, nstates2);
    int recomb_parent_age;
    double last_treelen = internal ? get_treelen_internal(last, m.times.data())
                                   : get_treelen(last, m.times.data(), false);
    if (internal) {
        if (nstates1 == 0) {
            if (nstates2 == 0) {
                sw.determ[0] = 0; sw.determprob[0] = 1.0;
                sw.recoalsrc = -1; sw.recombsrc = -1;
                return true;
            }
            const int maintree_root = t.c1[t.root];
            for (int j = 0; j < nstates2; j++) {
                if (states2.node[j] == maintree_root && states2.time[j] == spr.coal_time) {
                    sw.determ[0] = j; sw.determprob[0] = 1.0;
                    sw.recoalsrc = -1; sw.recombsrc = -1;
                    return true;
                }
            }
            return false;
        }
        if (nstates2 == 0) {
            std::fill(sw.determ.begin(), sw.determ.begin() + nstates1, 0);
            for (int i = 0; i < nstates1; i++) {
                if (states1.node[i] == spr.recomb_node && states1.time[i] > spr.recomb_time)
                    recomb_parent_age = states1.time[i];
                else
                    recomb_parent_age = last.age[last.parent[spr.recomb_node]];
                sw.determprob[i] = calc_recomb_recoal(last, m, l, spr, states1.node[i],
                                                      states1.time[i], recomb_parent_age,
                                                      last_treelen, internal);
            }
            sw.recoalsrc = -1; sw.recombsrc = -1;
            return true;
        }
    }

    Lookup lk2;
    lk2.build(states2, t.n);
    deterministic_transitions(last, t, spr, mapping, states1, lk2, sw.determ.data(), internal);

    recomb_parent_age = last.age[last.parent[spr.recomb_node]];
    double sums;
    vector<double> sums2(m.T * 2 + 1, 0.0);
    calc_recoal_sums(m, l, spr, recomb_parent_age, &sums, sums2.data());
    vector<double> recoals(m.T);
    for (int a = 0; a < m.T; a++)
        recoals[a] = calc_recoal(last, m, l, spr, a, recomb_parent_age, false);

    for (int i = 0; i < nstates1; i++) {
        int j = sw.determ[i];
        if (j >= 0) {
            if (states1.node[i] == spr.recomb_node && states1.time[i] > spr.recomb_time) {
                recomb_parent_age = states1.time[i];
                sw.determprob[i] = calc_recomb_recoal(last, m, l, spr, states1.node[i],
                                                      states1.time[i], recomb_parent_age,
                                                      last_treelen, internal);
            } else {
                recomb_parent_age = last.age[last.parent[spr.recomb_node]];
                sw.determprob[i] =
                    calc_recomb(last, m, l, spr, states1.node[i], states1.time[i],
                                recomb_parent_age, last_treelen, internal) *
                    exp(-sums - sums2[std::max(std::min(2 * spr.coal_time - 1, 2 * states1.time[i]),
                                               2 * spr.recomb_time)]) *
                    recoals[states1.time[i]];
            }
        }
    }

    int recoalsrc = -1, recombsrc = -1;
    for (int i = 0; i < nstates1; i++) {
        if (states1.node[i] == spr.recomb_node && states1.time[i] == spr.recomb_time)
            recombsrc = i;
        else if (states1.node[i] == spr.coal_node && states1.time[i] == spr.coal_time)
            recoalsrc = i;
    }
    sw.recoalsrc = recoalsrc;
    sw.recombsrc = recombsrc;

    if (recombsrc != -1) {
        // get_recomb_transition_switch (trans.cpp:278-313)
        const int parent = last.parent[spr.recomb_node];
        const int time2 = last.age[parent];
        const int other = last.sibling(spr.recomb_node);
        const int node2 = (other == spr.coal_node ? t.parent[mapping[other]] : mapping[other]);
        int next0 = lk2.lookup(mapping[spr.recomb_node], spr.recomb_time);
        int next1 = lk2.lookup(node2, time2);
        for (int j = 0; j < nstates2; j++) sw.recombrow[j] = 0.0;
        if (next0 != -1) {
            recomb_parent_age = last.age[last.parent[spr.recomb_node]];
            sw.recombrow[next0] = calc_recomb_recoal(last, m, l, spr, states1.node[recombsrc],
                                                     states1.time[recombsrc], recomb_parent_age,
                                                     last_treelen, internal);
        }
        if (next1 != -1) {
            recomb_parent_age = states1.time[recombsrc];
            sw.recombrow[next1] = calc_recomb_recoal(last, m, l, spr, states1.node[recombsrc],
                                                     states1.time[recombsrc], recomb_parent_age,
                                                     last_treelen, internal);
        }
    }

    if (recoalsrc == -1) {
        for (int j = 0; j < nstates2; j++) sw.recoalrow[j] = 0.0;
        return true;
    }

    const int node1 = states1.node[recoalsrc];
    const int time1 = states1.time[recoalsrc];
    int node3;
    const int last_parent = last.parent[spr.recomb_node];
    if (last_parent == node1) {
        node3 = mapping[last.c1[last_parent] == spr.recomb_node ? last.c0[last_parent]
                                                                 : last.c1[last_parent]];
    } else {
        node3 = mapping[node1];
    }
    const int parent = t.parent[mapping[spr.recomb_node]];
    for (int j = 0; j < nstates2; j++) {
        const int node2 = states2.node[j];
        const int time2 = states2.time[j];
        sw.recoalrow[j] = 0.0;
        if (!((node2 == mapping[spr.recomb_node] && time2 >= spr.recomb_time) ||
              (node2 == node3 && time2 == time1) || (node2 == parent && time2 == time1)))
            continue;
        recomb_parent_age = last.age[last.parent[spr.recomb_node]];
        Spr spr2 = spr;
        spr2.coal_time = time2;
        sw.recoalrow[j] = calc_recomb_recoal(last, m, l, spr2, states1.node[recoalsrc],
                                             states1.time[recoalsrc], recomb_parent_age,
                                             last_treelen, internal);
    }
    return true;
}

// calc_state_priors (trans.cpp:785-831)
void calc_state_priors(const States &states, const Lineages &l, const Model &m, double *priors,
                       int minage) {
    const int nstates = states.size();
    if (nstates == 0) { priors[0] = 1.0; return; }
    for (int i = 0; i < nstates; i++) {
        const int b = states.time[i];
        if (b < minage) { priors[i] = 0.0; continue; }
        double sum = 0.0;
        for (int mm = 2 * minage; mm < 2 * b - 1; mm++)
            sum += m.coal_time_steps[mm] * l.nbranches[mm / 2] / (2.0 * m.popsizes[mm / 2]);
        double p = exp(-sum) / l.ncoals[b];
        if (b < m.T - 2) {
            double Z = 0.0;
            if (b > minage)
                Z = m.coal_time_steps[2 * b - 1] * l.nbranches[b - 1] / (2.0 * m.popsizes[b - 1]);
            p *= 1.0 - exp(-m.coal_time_steps[2 * b] * l.nbranches[b] / (2.0 * m.popsizes[b]) - Z);
        }
        priors[i] = p;
    }
}

// ---------------------------------------------------------------------------------------
// emissions

inline double prob_branch(double t, double mu, bool mut) {  // emit.cpp:86-93
    const double f = 4. / 3.;
    if (!mut) return .25 * (1.0 + 3. * exp(-f * mu * t));
    return .25 * (1.0 - exp(-f * mu * t));
}

typedef double lk_row[4];

// calc_emissions (emit.cpp:650-869) for one block: emit[i*S + j], S = max(nstates,1)
// parsimony_ancestral_set (emit.cpp:898-953): Fitch sets over `order` (children before
// parents, the root last), then refined from the root down.
void parsimony_sets(const Tree &t, const char *const *seqs, int pos, const vector<int> &order,
                    vector<char> &anc) {
    vector<char> sets(t.n, 0);
    for (int node : order) {
        if (t.leaf(node)) {
            const char c = seqs[node][pos];
            sets[node] = c == 'N' ? 0 : (char)(1 << dna2int(c));
        } else {
            const char l = sets[t.c0[node]], r = sets[t.c1[node]];
            const char x = l & r;
            sets[node] = x ? x : (char)(l | r);
        }
    }
    const int root = order.back();
    anc[root] = sets[root];
    for (int i = (int)order.size() - 2; i >= 0; i--) {
        const int node = order[i];
        const char pset = anc[t.parent[node]] & sets[node];
        anc[node] = pset ? pset : sets[node];
    }
}

// get_infinite_sites_states (emit.cpp:454-589): whether each state of a non-invariant
// column keeps the infinite-sites model (the threaded base needs no second mutation).
void infsites_valid(const States &states, const Tree &t, const char *const *seqs, int pos,
                    bool internal, vector<char> &valid) {
    const int nstates = states.size();
    const int n = t.n;
    valid.assign(nstates, 1);
    auto preorder = [&](int top) {  // LocalTree::get_preorder (local_tree.h:305-322)
        vector<int> out, stack{top};
        while (!stack.empty()) {
            const int v = stack.back();
            stack.pop_back();
            out.push_back(v);
            if (!t.leaf(v)) { stack.push_back(t.c0[v]); stack.push_back(t.c1[v]); }
        }
        return out;
    };
    vector<char> anc(n, 0), vnode(n, 0);
    if (internal) {
        const int mainr = t.c1[t.root], subr = t.c0[t.root];
        vector<int> sub = preorder(subr), main = preorder(mainr);
        std::reverse(sub.begin(), sub.end());
        std::reverse(main.begin(), main.end());
        char subset = 0, mainset = 0;
        for (int j : sub)
            if (t.leaf(j) && seqs[j][pos] != 'N') subset |= (char)(1 << dna2int(seqs[j][pos]));
        for (int j : main)
            if (t.leaf(j) && seqs[j][pos] != 'N') mainset |= (char)(1 << dna2int(seqs[j][pos]));
        if (!(subset & mainset)) return;
        parsimony_sets(t, seqs, pos, sub, anc);
        const char cset = anc[subr];
        parsimony_sets(t, seqs, pos, main, anc);
        for (int j : main)
            vnode[j] = (cset & anc[j]) || (j != mainr && (cset & anc[t.parent[j]]));
    } else {
        const int newleaf = t.nleaves();
        char set = 0;
        for (int j = 0; j < newleaf; j++)
            if (seqs[j][pos] != 'N') set |= (char)(1 << dna2int(seqs[j][pos]));
        const char c = seqs[newleaf][pos];
        const char cset = c != 'N' ? (char)(1 << dna2int(c)) : 0;
        if (!(cset & set)) return;
        vector<int> order(n);  // LocalTree::get_postorder (local_tree.h:274-304)
        {
            vector<char> visit(n, 0);
            int i;
            for (i = 0; i < n; i++) {
                if (!t.leaf(i)) break;
                order[i] = i;
            }
            int end = i;
            for (i = 0; i < n; i++) {
                const int parent = t.parent[order[i]];
                if (parent != -1 && ++visit[parent] == 2) order[end++] = parent;
            }
        }
        parsimony_sets(t, seqs, pos, order, anc);
        for (int j = 0; j < n; j++)
            vnode[j] = (cset & anc[j]) || (t.parent[j] != -1 && (cset & anc[t.parent[j]]));
    }
    for (int k = 0; k < nstates; k++) valid[k] = vnode[states.node[k]];
}

void calc_emissions(const States &states, const Tree &t, const char *const *seqs, int nseqs,
                    int seqlen, const Model &m, bool internal, double *emit) {
    const int nstates = states.size();
    const int S = std::max(nstates, 1);
    const double mintime = m.mintime();
    const double *times = m.times.data();
    const int newleaf = t.nleaves();
    const int maintree_root = internal ? t.c1[t.root] : t.root;
    const int subtree_root = internal ? t.c0[t.root] : t.root;
    const int n = t.n;

    if (internal && nstates == 0) {
        for (int i = 0; i < seqlen; i++) emit[(size_t)i * S] = 1.0;
        return;
    }

    vector<char> invariant(seqlen), masked(seqlen);
    for (int i = 0; i < seqlen; i++) {  // find_invariant_sites / find_masked_sites (emit.cpp:30-58)
        char c = seqs[0][i];
        bool mut = false;
        for (int j = 1; j < nseqs; j++)
            if (seqs[j][i] != c) { mut = true; break; }
        invariant[i] = !mut;
        masked[i] = (seqs[0][i] == 'N' && invariant[i]);
    }

    // mutation probabilities per branch (prob_tree_mutation, emit.cpp:97-116)
    vector<double> muts(n, 0.0), nomuts(n, 0.0);
    for (int i = 0; i < n; i++) {
        if (i == t.root) continue;
        int parent_age = t.age[t.parent[i]];
        if (parent_age == m.removed_root_time()) continue;
        double tt = std::max(times[parent_age] - times[t.age[i]], mintime);
        muts[i] = prob_branch(tt, m.mu, true);
        nomuts[i] = prob_branch(tt, m.mu, false);
    }

    // postorder (LocalTree::get_postorder, local_tree.h:274-304)
    vector<int> order(n);
    {
        vector<char> visit(n, 0);
        int i;
        for (i = 0; i < n; i++) {
            if (!t.leaf(i)) break;
            order[i] = i;
        }
        int end = i;
        for (i = 0; i < n; i++) {
            int parent = t.parent[order[i]];
            if (parent != -1) {
                visit[parent]++;
                if (visit[parent] == 2) order[end++] = parent;
            }
        }
    }

    vector<lk_row> inner((size_t)seqlen * n), outer((size_t)seqlen * n);
    for (int i = 0; i < seqlen; i++) {
        if (invariant[i]) continue;
        lk_row *in = &inner[(size_t)i * n];
        for (int oi = 0; oi < n; oi++) {  // likelihood_site_node_inner (emit.cpp:151-196)
            const int j = order[oi];
            if (t.leaf(j)) {
                const char c = seqs[j][i];
                if (c == 'N') { in[j][0] = in[j][1] = in[j][2] = in[j][3] = 1.0; }
                else {
                    in[j][0] = in[j][1] = in[j][2] = in[j][3] = 0.0;
                    in[j][dna2int(c)] = 1.0;
                }
            } else {
                int c1 = t.c0[j], c2 = t.c1[j];
                for (int a = 0; a < 4; a++) {
                    double p1 = 0.0, p2 = 0.0;
                    for (int b = 0; b < 4; b++) {
                        if (a == b) { p1 += in[c1][b] * nomuts[c1]; p2 += in[c2][b] * nomuts[c2]; }
                        else { p1 += in[c1][b] * muts[c1]; p2 += in[c2][b] * muts[c2]; }
                    }
                    in[j][a] = p1 * p2;
                }
            }
        }
        lk_row *out = &outer[(size_t)i * n];
        vector<int> queue;  // likelihood_site_outer (emit.cpp:199-296), preorder
        queue.push_back(maintree_root);
        while (!queue.empty()) {
            int j = queue.back();
            queue.pop_back();
            if (j == maintree_root) {
                out[j][0] = out[j][1] = out[j][2] = out[j][3] = 1.0;
            } else {
                int sib = t.sibling(j), parent = t.parent[j];
                if (parent != maintree_root) {
                    for (int a = 0; a < 4; a++) {
                        double p1 = 0.0, p2 = 0.0;
                        for (int b = 0; b < 4; b++) {
                            if (a == b) { p1 += in[sib][b] * nomuts[sib]; p2 += out[parent][b] * nomuts[parent]; }
                            else { p1 += in[sib][b] * muts[sib]; p2 += out[parent][b] * muts[parent]; }
                        }
                        out[j][a] = p1 * p2;
                    }
                } else {
                    for (int a = 0; a < 4; a++) {
                        double p1 = 0.0;
                        for (int b = 0; b < 4; b++) {
                            if (a == b) p1 += in[sib][b] * nomuts[sib];
                            else p1 += in[sib][b] * muts[sib];
                        }
                        out[j][a] = p1;
                    }
                }
            }
            if (!t.leaf(j)) { queue.push_back(t.c0[j]); queue.push_back(t.c1[j]); }
        }
    }

    vector<lk_row> inner_subtree(internal ? 0 : seqlen);
    if (!internal) {
        for (int i = 0; i < seqlen; i++) {
            const char c = seqs[newleaf][i];
            if (c == 'N') { for (int a = 0; a < 4; a++) inner_subtree[i][a] = 1.0; }
            else {
                for (int a = 0; a < 4; a++) inner_subtree[i][a] = 0.0;
                inner_subtree[i][dna2int(c)] = 1.0;
            }
        }
    }

    // tree lengths by preorder stacks (emit.cpp:744-774)
    double maintreelen = 0.0, subtreelen = 0.0;
    {
        vector<int> queue{maintree_root};
        while (!queue.empty()) {
            int node = queue.back(); queue.pop_back();
            if (node != maintree_root) maintreelen += std::max(t.dist(node, times), mintime);
            if (!t.leaf(node)) { queue.push_back(t.c0[node]); queue.push_back(t.c1[node]); }
        }
        if (internal) {
            queue.push_back(subtree_root);
            while (!queue.empty()) {
                int node = queue.back(); queue.pop_back();
                if (node != subtree_root) subtreelen += std::max(t.dist(node, times), mintime);
                if (!t.leaf(node)) { queue.push_back(t.c0[node]); queue.push_back(t.c1[node]); }
            }
        }
    }

    for (int j = 0; j < nstates; j++) {
        const int node1 = internal ? subtree_root : 0;
        const int node2 = states.node[j];
        const int parent = t.parent[node2];
        double time1 = internal ? times[t.age[node1]] : 0.0;
        double time2 = times[t.age[node2]];
        double parent_time = (parent != -1) ? times[std::min(t.age[parent], m.T - 1)] : 0.0;
        double coal_time = times[states.time[j]];
        double dist[3], mut[3], nomut[3];
        dist[0] = std::max(coal_time - time1, mintime);
        dist[1] = std::max(coal_time - time2, mintime);
        dist[2] = std::max(parent_time - coal_time, mintime);
        for (int x = 0; x < 3; x++) mut[x] = prob_branch(dist[x], m.mu, true);
        for (int x = 0; x < 3; x++) nomut[x] = prob_branch(dist[x], m.mu, false);
        double treelen;
        if (node2 == maintree_root)
            treelen = maintreelen + subtreelen + std::max(coal_time - time1, mintime) +
                      std::max(coal_time - times[t.age[maintree_root]], mintime);
        else
            treelen = maintreelen + subtreelen + std::max(coal_time - time1, mintime);
        double invariant_lk = .25 * exp(-m.mu * std::max(treelen, mintime));

        for (int i = 0; i < seqlen; i++) {
            double e;
            if (masked[i]) e = 1.0;
            else if (invariant[i]) e = invariant_lk;
            else {
                const lk_row *in = &inner[(size_t)i * n];
                const lk_row *out = &outer[(size_t)i * n];
                const double *in2 = internal ? in[node1] : inner_subtree[i];
                e = 0.0;  // calc_emit (emit.cpp:620-645)
                for (int a = 0; a < 4; a++) {
                    double p1 = 0.0, p2 = 0.0, p3 = 0.0;
                    for (int b = 0; b < 4; b++) {
                        if (a == b) {
                            p1 += in2[b] * nomut[0]; p2 += in[node2][b] * nomut[1];
                            p3 += out[node2][b] * nomut[2];
                        } else {
                            p1 += in2[b] * mut[0]; p2 += in[node2][b] * mut[1];
                            p3 += out[node2][b] * mut[2];
                        }
                    }
                    if (node2 != maintree_root) e += p1 * p2 * p3 * .25;
                    else e += p1 * p2 * .25;
                }
            }
            emit[(size_t)i * S + j] = e;
        }
    }

    // optionally the infinite-sites model (calc_emissions, emit.cpp:847-862)
    if (m.infsites_penalty < 1.0) {
        vector<char> valid;
        for (int i = 0; i < seqlen; i++) {
            if (invariant[i]) continue;
            infsites_valid(states, t, seqs, i, internal, valid);
            for (int j = 0; j < nstates; j++)
                if (!valid[j]) emit[(size_t)i * S + j] *= m.infsites_penalty;
        }
    }
}

// ---------------------------------------------------------------------------------------
// per-block matrices (ArgHmmMatrixIter / calc_arghmm_matrices, matrices.cpp:8-175)

struct Block {
    int start = 0, len = 0;
    States states;
    Lineages lineages;
    TransMatrix tm;
    bool has_switch = false;
    SwitchMatrix sw;
};

struct Hmm {
    Model m;
    Arg arg;
    bool internal = false;
    int minage = 0;
    vector<const char *> subseq_base;  // sequence rows for emissions
    int nseqs_emit = 0;
};

bool setup(const oracle_problem *p, Hmm &h) {
    if (!p || !build_model(p, h.m)) return false;
    if (!build_arg(p, h.arg)) return false;
    h.internal = p->internal != 0;
    h.minage = p->minage;
    const int nleaves = (p->nnodes + 1) / 2;
    h.nseqs_emit = h.internal ? nleaves : nleaves + 1;
    h.subseq_base.resize(h.nseqs_emit);
    for (int i = 0; i < h.nseqs_emit; i++) h.subseq_base[i] = p->seqs + (size_t)i * p->seqlen;
    return true;
}

bool make_block(const Hmm &h, int b, Block &blk, bool with_switch) {
    const Tree &t = h.arg.trees[b];
    blk.start = h.arg.start[b];
    blk.len = h.arg.blocklen[b];
    coal_states(t, h.m.T, h.internal, h.minage, blk.states);
    blk.has_switch = false;
    if (with_switch && b > 0) {
        const Tree &last = h.arg.trees[b - 1];
        States last_states;
        coal_states(last, h.m.T, h.internal, h.minage, last_states);
        Lineages ll;
        count(last, h.m.T, h.internal, ll);
        if (!calc_transition_probs_switch(t, last, h.arg.sprs[b], h.arg.mapping[b], last_states,
                                          blk.states, h.m, ll, blk.sw, h.internal))
            return false;
        blk.has_switch = true;
    }
    count(t, h.m.T, h.internal, blk.lineages);
    calc_transition_probs(t, h.m, blk.states, blk.lineages, blk.tm, h.internal, h.minage);
    return true;
}

void block_emissions(const Hmm &h, const Block &blk, int b, vector<double> &emit) {
    const int S = std::max(blk.states.size(), 1);
    emit.assign((size_t)blk.len * S, 0.0);
    vector<const char *> sub(h.nseqs_emit);
    for (int i = 0; i < h.nseqs_emit; i++) sub[i] = h.subseq_base[i] + blk.start;
    calc_emissions(blk.states, h.arg.trees[b], sub.data(), h.nseqs_emit, blk.len, h.m,
                   h.internal, emit.data());
}

// Column offsets of the packed table.
vector<long long> column_offsets(const Hmm &h, vector<int> &nst) {
    const int L = h.arg.start.back() + h.arg.blocklen.back();
    vector<long long> off(L + 1, 0);
    nst.assign(L, 0);
    States s;
    for (size_t b = 0; b < h.arg.trees.size(); b++) {
        coal_states(h.arg.trees[b], h.m.T, h.internal, h.minage, s);
        for (int i = 0; i < h.arg.blocklen[b]; i++) nst[h.arg.start[b] + i] = s.size();
    }
    for (int i = 0; i < L; i++) off[i + 1] = off[i] + std::max(nst[i], 1);
    return off;
}

// arghmm_forward_switch (sample_thread.cpp:345-389)
double forward_switch(const double *col1, double *col2, const SwitchMatrix &sw,
                      const double *emit) {
    const int nstates1 = std::max(sw.nstates1, 1), nstates2 = std::max(sw.nstates2, 1);
    for (int k = 0; k < nstates2; k++) col2[k] = 0.0;
    for (int j = 0; j < nstates1; j++) {
        int k = sw.determ[j];
        if (j != sw.recombsrc && j != sw.recoalsrc && k != -1) col2[k] += col1[j] * sw.determprob[j];
    }
    double norm = 0.0;
    for (int k = 0; k < nstates2; k++) {
        if (sw.recombsrc != -1 && sw.recombrow[k] > 0.0) col2[k] += col1[sw.recombsrc] * sw.recombrow[k];
        if (sw.recoalsrc != -1 && sw.recoalrow[k] > 0.0) col2[k] += col1[sw.recoalsrc] * sw.recoalrow[k];
        col2[k] *= emit[k];
        norm += col2[k];
    }
    for (int k = 0; k < nstates2; k++) col2[k] /= norm;
    return norm;
}

// Structured per-block tables of arghmm_forward_block (sample_thread.cpp:209-247).
struct BlockSteps {
    int T = 0, S = 0;
    vector<double> tmatrix, tmatrix2;  // [T*T], [T*S]
    vector<int> ages1, ages2, indexes;
};

void block_steps(const Tree &t, int T, const States &states, const TransMatrix &tm,
                 bool internal, BlockSteps &bs) {
    const int nstates = states.size();
    const int minage = tm.minage;
    bs.T = T;
    bs.S = nstates;
    bs.tmatrix.assign((size_t)T * T, 0.0);
    bs.tmatrix2.assign((size_t)T * std::max(nstates, 1), 0.0);
    for (int a = 0; a < T - 1; a++) {
        for (int b = 0; b < T - 1; b++) bs.tmatrix[a * T + b] = tm.get_time(a, b, 0, minage, false);
        for (int k = 0; k < nstates; k++) {
            const int b = states.time[k];
            const int c = t.age[states.node[k]];
            bs.tmatrix2[(size_t)a * nstates + k] =
                tm.get_time(a, b, c, minage, true) - tm.get_time(a, b, 0, minage, false);
        }
    }
    int maxtime = 0;
    for (int k = 0; k < nstates; k++) maxtime = std::max(maxtime, states.time[k]);
    Lookup lk;
    lk.build(states, t.n);
    const int maintree_root = internal ? t.c1[t.root] : 0;
    bs.ages1.assign(t.n, 0); bs.ages2.assign(t.n, 0); bs.indexes.assign(t.n, -1);
    for (int i = 0; i < t.n; i++) {
        bs.ages1[i] = std::max(t.age[i], minage);
        bs.indexes[i] = lk.lookup(i, bs.ages1[i]);
        if (internal)
            bs.ages2[i] = (i == maintree_root || i == t.root) ? maxtime : t.age[t.parent[i]];
        else
            bs.ages2[i] = (i == t.root) ? maxtime : t.age[t.parent[i]];
    }
}

// arghmm_forward_block (sample_thread.cpp:186-296); fw points at the block's first column
// (already filled), cols at the packed column offsets; returns sum of log norms.
double forward_block(const Tree &t, const States &states, const BlockSteps &bs, int blocklen,
                     const double *emit, int S, double *fw, bool internal) {
    const int nstates = states.size();
    const int T = bs.T;
    double lnl = 0.0;
    if (internal && nstates == 0) {
        for (int i = 1; i < blocklen; i++) fw[i] = fw[i - 1];
        return 0.0;
    }
    vector<double> tf(T), fgroups(T);
    for (int i = 1; i < blocklen; i++) {
        const double *col1 = fw + (size_t)(i - 1) * S;
        double *col2 = fw + (size_t)i * S;
        const double *emit2 = emit + (size_t)i * S;
        std::fill(fgroups.begin(), fgroups.end(), 0.0);
        for (int j = 0; j < nstates; j++) fgroups[states.time[j]] += col1[j];
        for (int b = 0; b < T - 1; b++) {
            double sum = 0.0;
            for (int a = 0; a < T - 1; a++) sum += bs.tmatrix[a * T + b] * fgroups[a];
            tf[b] = sum;
        }
        double norm = 0.0;
        for (int k = 0; k < nstates; k++) {
            const int b = states.time[k];
            const int node2 = states.node[k];
            const int age1 = bs.ages1[node2], age2 = bs.ages2[node2];
            double sum = tf[b];
            const int j1 = bs.indexes[node2];
            for (int j = j1, a = age1; a <= age2; j++, a++)
                sum += bs.tmatrix2[(size_t)a * nstates + k] * col1[j];
            col2[k] = sum * emit2[k];
            norm += col2[k];
        }
        for (int k = 0; k < nstates; k++) col2[k] /= norm;
        lnl += log(norm);
    }
    return lnl;
}

// sample (common.h:272-290) with an explicit uniform
int sample(const double *w, int n, double u) {
    double total = 0.0;
    for (int i = 0; i < n; i++) total += w[i];
    double pick = u * total;
    double x = 0.0;
    for (int i = 0; i < n; i++) {
        x += w[i];
        if (x >= pick) return i;
    }
    return n - 1;
}

}  // namespace

extern "C" {

long long oracle_cells(const oracle_problem *p) {
    Hmm h;
    if (!setup(p, h)) return -1;
    vector<int> nst;
    return column_offsets(h, nst).back();
}

int oracle_nstates(const oracle_problem *p, int *nstates) {
    Hmm h;
    if (!setup(p, h)) return -1;
    vector<int> nst;
    column_offsets(h, nst);
    std::copy(nst.begin(), nst.end(), nstates);
    return 0;
}

int oracle_forward(const oracle_problem *p, double *fw, double *loglik) {
    return oracle_forward_prior(p, nullptr, fw, loglik);
}

// With prior non-NULL, column 0 holds those max(S0,1) values instead of the state priors
// (the given first column of arghmm_forward_alg's prior_given, sample_thread.cpp:425-429).
int oracle_forward_prior(const oracle_problem *p, const double *prior, double *fw,
                         double *loglik) {
    Hmm h;
    if (!setup(p, h)) return -1;
    vector<int> nst;
    vector<long long> off = column_offsets(h, nst);
    double lnl = 0.0;
    vector<double> emit;
    BlockSteps bs;
    for (size_t b = 0; b < h.arg.trees.size(); b++) {
        Block blk;
        if (!make_block(h, (int)b, blk, true)) return -2;
        block_emissions(h, blk, (int)b, emit);
        const int S = std::max(blk.states.size(), 1);
        double *col = fw + off[blk.start];
        if (b == 0) {
            calc_state_priors(blk.states, blk.lineages, h.m, col, h.minage);
            if (prior) std::copy(prior, prior + S, col);
        } else {
            const int S1 = std::max(nst[blk.start - 1], 1);
            (void)S1;
            lnl += log(forward_switch(fw + off[blk.start - 1], col, blk.sw, emit.data()));
        }
        block_steps(h.arg.trees[b], h.m.T, blk.states, blk.tm, h.internal, bs);
        lnl += forward_block(h.arg.trees[b], blk.states, bs, blk.len, emit.data(), S, col,
                             h.internal);
    }
    if (loglik) *loglik = lnl;
    return 0;
}

// With `given` non-NULL each column draws conditioned on given[i + 1] instead of the path
// drawn so far (a per-column check of another sampler's draws on its own table).
int oracle_traceback_given(const oracle_problem *p, const double *fw, const double *u,
                           const int *given, int *path) {
    return oracle_traceback_last(p, fw, u, given, -1, path);
}

// last_state >= 0: the last column's state is given (stochastic_traceback with
// last_state_given, sample_thread.cpp:532-539) and takes no draw.
int oracle_traceback_last(const oracle_problem *p, const double *fw, const double *u,
                          const int *given, int last_state, int *path) {
    Hmm h;
    if (!setup(p, h)) return -1;
    vector<int> nst;
    vector<long long> off = column_offsets(h, nst);
    const int L = p->seqlen;
    const int B = (int)h.arg.trees.size();
    path[L - 1] = last_state >= 0 ? last_state
                                  : sample(fw + off[L - 1], std::max(nst[L - 1], 1), u[L - 1]);
    vector<double> A, trans;
    for (int b = B - 1; b >= 0; b--) {
        Block blk;
        if (!make_block(h, b, blk, true)) return -2;
        const Tree &t = h.arg.trees[b];
        const int nstates = std::max(blk.states.size(), 1);
        A.assign(nstates, 0.0);
        trans.assign(nstates, 0.0);
        int last_k = -1;
        for (int i = blk.len - 2; i >= 0; i--) {  // sample_hmm_posterior (sample_thread.cpp:470-503)
            const int col = blk.start + i;
            int k = given ? given[col + 1] : path[col + 1];
            if (k != last_k) {
                for (int j = 0; j < nstates; j++) trans[j] = blk.tm.get(t, blk.states, j, k);
                last_k = k;
            }
            for (int j = 0; j < nstates; j++) A[j] = fw[off[col] + j] * trans[j];
            path[col] = sample(A.data(), nstates, u[col]);
        }
        if (blk.start > 0) {  // sample_hmm_posterior_step (sample_thread.cpp:506-519)
            const int col = blk.start - 1;
            const int n1 = std::max(blk.sw.nstates1, 1);
            A.assign(n1, 0.0);
            const int k = given ? given[col + 1] : path[col + 1];
            for (int j = 0; j < n1; j++) A[j] = fw[off[col] + j] * blk.sw.get(j, k);
            path[col] = sample(A.data(), n1, u[col]);
        }
    }
    return 0;
}

int oracle_traceback(const oracle_problem *p, const double *fw, const double *u, int *path) {
    return oracle_traceback_given(p, fw, u, nullptr, path);
}

// The FP32 path's decomposed draw, restated in FP64 (no counterpart in the reference; it
// draws from the same distribution as sample_hmm_posterior, sample_thread.cpp:470-503, with
// the uniform mapped to states in another order). Inside a tree the weights
// fw[i][j] P(j -> k) split into the same-branch part over the states of k's node
// (tmatrix2 of arghmm_forward_block, sample_thread.cpp:215-226) and a background part
// that depends on j only through its time (tmatrix, :211-213). With t = u (V + W): t <= V
// picks the first same-branch state (times ascending) whose running sum reaches t; else
// the first time bin whose running background sum reaches t - V, then the first state of
// that bin (state order) whose running fw sum reaches the remainder over tmatrix[a][b_k].
// Tree switches and the last column draw as the reference does. With `given` non-NULL each
// column draws conditioned on given[i + 1] instead of the path drawn so far (a per-column
// check of another sampler's draws).
int oracle_traceback_split(const oracle_problem *p, const double *fw, const double *u,
                           const int *given, int *path) {
    Hmm h;
    if (!setup(p, h)) return -1;
    vector<int> nst;
    vector<long long> off = column_offsets(h, nst);
    const int L = p->seqlen;
    const int B = (int)h.arg.trees.size();
    const int T = h.m.T;
    path[L - 1] = sample(fw + off[L - 1], std::max(nst[L - 1], 1), u[L - 1]);
    vector<double> A, V, W, bins(T);
    for (int b = B - 1; b >= 0; b--) {
        Block blk;
        if (!make_block(h, b, blk, true)) return -2;
        const Tree &t = h.arg.trees[b];
        const int nstates = blk.states.size();
        const int ma = blk.tm.minage;
        for (int i = blk.len - 2; i >= 0; i--) {
            const int col = blk.start + i;
            if (nstates == 0) { path[col] = 0; continue; }
            const double *f = fw + off[col];
            const int k = given ? given[col + 1] : path[col + 1];
            const int bk = blk.states.time[k], nk = blk.states.node[k];
            const int ck = t.age[nk];
            int j1 = k;
            while (j1 > 0 && blk.states.node[j1 - 1] == nk) j1--;
            int j2 = k;
            while (j2 + 1 < nstates && blk.states.node[j2 + 1] == nk) j2++;
            V.assign(j2 - j1 + 1, 0.0);
            double vt = 0.0;
            for (int j = j1; j <= j2; j++) {
                const int a = blk.states.time[j];
                V[j - j1] = f[j] * (blk.tm.get_time(a, bk, ck, ma, true) -
                                    blk.tm.get_time(a, bk, 0, ma, false));
                vt += V[j - j1];
            }
            std::fill(bins.begin(), bins.end(), 0.0);
            for (int j = 0; j < nstates; j++) bins[blk.states.time[j]] += f[j];
            W.assign(T - 1, 0.0);
            double wt = 0.0;
            for (int a = 0; a < T - 1; a++) {
                W[a] = bins[a] * blk.tm.get_time(a, bk, 0, ma, false);
                wt += W[a];
            }
            const double pick = u[col] * (vt + wt);
            int x = -1;
            if (pick <= vt) {
                double run = 0.0;
                for (int y = 0; y <= j2 - j1 && x < 0; y++) {
                    run += V[y];
                    if (run >= pick) x = j1 + y;
                }
                if (x < 0) x = j2;
            } else {
                const double p2 = pick - vt;
                double run = 0.0;
                int a = -1;
                for (int q = 0; q < T - 1 && a < 0; q++) {
                    if (run + W[q] >= p2) a = q;
                    else run += W[q];
                }
                if (a < 0)
                    for (int q = T - 2; q >= 0 && a < 0; q--)
                        if (W[q] > 0.0) a = q;
                const double r = (p2 - run) / blk.tm.get_time(a, bk, 0, ma, false);
                double fr = 0.0;
                int last = -1;
                for (int j = 0; j < nstates && x < 0; j++) {
                    if (blk.states.time[j] != a) continue;
                    fr += f[j];
                    if (f[j] > 0.0) last = j;
                    if (fr >= r) x = j;
                }
                if (x < 0) x = last;
            }
            path[col] = x;
        }
        if (blk.start > 0) {  // sample_hmm_posterior_step (sample_thread.cpp:506-519)
            const int col = blk.start - 1;
            const int n1 = std::max(blk.sw.nstates1, 1);
            A.assign(n1, 0.0);
            const int k = given ? given[col + 1] : path[col + 1];
            for (int j = 0; j < n1; j++) A[j] = fw[off[col] + j] * blk.sw.get(j, k);
            path[col] = sample(A.data(), n1, u[col]);
        }
    }
    return 0;
}

int oracle_backward(const oracle_problem *p, double *bw) {
    Hmm h;
    if (!setup(p, h)) return -1;
    vector<int> nst;
    vector<long long> off = column_offsets(h, nst);
    const int L = p->seqlen;
    const int B = (int)h.arg.trees.size();
    {
        const int S = std::max(nst[L - 1], 1);
        for (int k = 0; k < S; k++) bw[off[L - 1] + k] = 1.0 / S;
    }
    vector<double> emit, g, G;
    BlockSteps bs;
    for (int b = B - 1; b >= 0; b--) {
        Block blk;
        if (!make_block(h, b, blk, true)) return -2;
        block_emissions(h, blk, b, emit);
        const Tree &t = h.arg.trees[b];
        const int nstates = blk.states.size();
        const int S = std::max(nstates, 1);
        const int T = h.m.T;
        block_steps(t, T, blk.states, blk.tm, h.internal, bs);
        g.assign(S, 0.0);
        G.assign(T, 0.0);
        // within the block: column col -> col+1, both inside this block
        for (int i = blk.len - 2; i >= 0; i--) {
            const int col = blk.start + i;
            const double *next = bw + off[col + 1];
            double *cur = bw + off[col];
            const double *e = emit.data() + (size_t)(i + 1) * S;
            for (int k = 0; k < S; k++) g[k] = e[k] * next[k];
            if (h.internal && nstates == 0) {
                cur[0] = g[0];
            } else {
                std::fill(G.begin(), G.end(), 0.0);
                for (int k = 0; k < nstates; k++) G[blk.states.time[k]] += g[k];
                for (int j = 0; j < nstates; j++) {
                    const int a = blk.states.time[j];
                    double sum = 0.0;
                    for (int bb = 0; bb < T - 1; bb++) sum += bs.tmatrix[a * T + bb] * G[bb];
                    // same-branch part: sum over k of this node, tmatrix2[a][k]
                    const int node = blk.states.node[j];
                    const int j1 = bs.indexes[node];
                    for (int kk = j1, bb = bs.ages1[node]; bb <= bs.ages2[node]; kk++, bb++)
                        sum += bs.tmatrix2[(size_t)a * nstates + kk] * g[kk];
                    cur[j] = sum;
                }
            }
            double norm = 0.0;
            for (int k = 0; k < S; k++) norm += cur[k];
            for (int k = 0; k < S; k++) cur[k] /= norm;
        }
        // into this block's first column from the previous block's last column
        if (blk.start > 0) {
            const int col = blk.start - 1;
            const double *next = bw + off[blk.start];
            double *cur = bw + off[col];
            const double *e = emit.data();
            for (int k = 0; k < S; k++) g[k] = e[k] * next[k];
            const SwitchMatrix &sw = blk.sw;
            const int n1 = std::max(sw.nstates1, 1), n2 = std::max(sw.nstates2, 1);
            for (int j = 0; j < n1; j++) {
                double sum = 0.0;
                if (j == sw.recoalsrc || j == sw.recombsrc) {
                    const double *row = (j == sw.recoalsrc) ? sw.recoalrow.data() : sw.recombrow.data();
                    for (int k = 0; k < n2; k++)
                        if (row[k] > 0.0) sum += row[k] * g[k];
                    // a state that is both sources takes both rows in the forward step
                    if (j == sw.recoalsrc && j == sw.recombsrc)
                        for (int k = 0; k < n2; k++)
                            if (sw.recombrow[k] > 0.0) sum += sw.recombrow[k] * g[k];
                } else if (sw.determ[j] != -1) {
                    sum = sw.determprob[j] * g[sw.determ[j]];
                }
                cur[j] = sum;
            }
            double norm = 0.0;
            for (int k = 0; k < n1; k++) norm += cur[k];
            for (int k = 0; k < n1; k++) cur[k] /= norm;
        }
    }
    return 0;
}

int oracle_posterior(const oracle_problem *p, const double *fw, const double *bw,
                     double *post) {
    Hmm h;
    if (!setup(p, h)) return -1;
    vector<int> nst;
    vector<long long> off = column_offsets(h, nst);
    for (int i = 0; i < p->seqlen; i++) {
        const int S = std::max(nst[i], 1);
        double norm = 0.0;
        for (int k = 0; k < S; k++) norm += fw[off[i] + k] * bw[off[i] + k];
        for (int k = 0; k < S; k++) post[off[i] + k] = fw[off[i] + k] * bw[off[i] + k] / norm;
    }
    return 0;
}

int oracle_block_terms(const oracle_problem *p, double *out_terms, int *out_minage) {
    Hmm h;
    if (!setup(p, h)) return -1;
    const int T = h.m.T;
    for (size_t b = 0; b < h.arg.trees.size(); b++) {
        Block blk;
        if (!make_block(h, (int)b, blk, false)) return -2;
        const vector<double> *arrs[9] = {&blk.tm.D, &blk.tm.E, &blk.tm.lnB, &blk.tm.lnE2,
                                         &blk.tm.lnNegG1, &blk.tm.G2, &blk.tm.G3, &blk.tm.lnG4,
                                         &blk.tm.norecombs};
        for (int a = 0; a < 9; a++)
            for (int t = 0; t < T; t++)
                out_terms[(b * 9 + a) * T + t] = t < T - 1 ? (*arrs[a])[t] : 0.0;
        if (out_minage) out_minage[b] = blk.tm.minage;
    }
    return 0;
}

int oracle_debug_tables(const oracle_problem *p, double *tm_out, double *gts_out,
                        double *inv_out, double *prior_out) {
    Hmm h;
    if (!setup(p, h)) return -1;
    const int T = h.m.T;
    long long goff = 0, ioff = 0;
    BlockSteps bs;
    for (size_t b = 0; b < h.arg.trees.size(); b++) {
        Block blk;
        if (!make_block(h, (int)b, blk, false)) return -2;
        const Tree &t = h.arg.trees[b];
        block_steps(t, T, blk.states, blk.tm, h.internal, bs);
        for (int a = 0; a < T - 1; a++)
            for (int c = 0; c < T - 1; c++)
                tm_out[(b * (T - 1) + a) * (T - 1) + c] = bs.tmatrix[a * T + c];
        const int S = blk.states.size();
        // rows in node order: node v's states j1..j1+m-1, each row over the node's times
        int k = 0;
        while (k < S) {
            const int v = blk.states.node[k];
            int m = 0;
            while (k + m < S && blk.states.node[k + m] == v) m++;
            const int t0 = blk.states.time[k];
            for (int y = 0; y < m; y++)      // source-major: entry (x, y) at y * m + x
                for (int x = 0; x < m; x++)
                    gts_out[goff++] = blk.tm.get_time(t0 + y, t0 + x, t.age[v], blk.tm.minage, true);
            k += m;
        }
        // invariant-site emission per state: the emission of an all-equal column
        vector<double> emit;
        Block one = blk;
        one.len = 1;
        vector<char> col(h.nseqs_emit, 'A');
        vector<const char *> rows(h.nseqs_emit);
        for (int i = 0; i < h.nseqs_emit; i++) rows[i] = &col[i];
        vector<double> e(std::max(S, 1));
        calc_emissions(blk.states, t, rows.data(), h.nseqs_emit, 1, h.m, h.internal, e.data());
        for (int j = 0; j < std::max(S, 1); j++) inv_out[ioff + j] = e[j];
        ioff += std::max(S, 1);
        if (b == 0) calc_state_priors(blk.states, blk.lineages, h.m, prior_out, h.minage);
    }
    return 0;
}

// Dense log matrices of tree b: trans [S][S] = log TransMatrix::get (get_transition_probs,
// trans.cpp:119-130) and, for b > 0 with sw non-NULL, sw [S1][S2] = log
// TransMatrixSwitch::get from tree b - 1 (get_transition_probs_switch, trans.cpp:756-764);
// states in coal_states order.
int oracle_dense_matrices(const oracle_problem *p, int b, double *trans, double *sw) {
    Hmm h;
    if (!setup(p, h)) return -1;
    if (b < 0 || b >= (int)h.arg.trees.size() || (sw && b == 0)) return -1;
    Block blk;
    if (!make_block(h, b, blk, sw != nullptr)) return -2;
    const Tree &t = h.arg.trees[b];
    const int S = blk.states.size();
    if (trans)
        for (int i = 0; i < S; i++)
            for (int j = 0; j < S; j++)
                trans[(size_t)i * S + j] = log(blk.tm.get(t, blk.states, i, j));
    if (sw)
        for (int i = 0; i < blk.sw.nstates1; i++)
            for (int j = 0; j < blk.sw.nstates2; j++)
                sw[(size_t)i * blk.sw.nstates2 + j] = log(blk.sw.get(i, j));
    return 0;
}

int oracle_emissions(const oracle_problem *p, double *emit_out) {
    Hmm h;
    if (!setup(p, h)) return -1;
    vector<int> nst;
    vector<long long> off = column_offsets(h, nst);
    vector<double> emit;
    for (size_t b = 0; b < h.arg.trees.size(); b++) {
        Block blk;
        if (!make_block(h, (int)b, blk, false)) return -2;
        block_emissions(h, blk, (int)b, emit);
        std::copy(emit.begin(), emit.end(), emit_out + off[blk.start]);
    }
    return 0;
}

// ----------------------------------------------------------------------------- dense HMM
// The reference's generic HMM over a full log transition matrix (hmm.cpp:27-85), tables
// row-major n x S. Each entry is a logsum over one row or column, as common.h:182-202:
// the maximum, then the terms within e^-15 of it summed in index order.

static double dense_logsum(const double *v, int n) {
    double mx = v[0];
    for (int i = 1; i < n; i++) mx = v[i] > mx ? v[i] : mx;
    double s = 0.0;
    for (int i = 0; i < n; i++)
        if (v[i] - mx > -15.0) s += std::exp(v[i] - mx);
    return mx + std::log(s);
}

int oracle_dense_forward(int n, int S, const double *trans, const double *emit, double *fw) {
    if (n < 1 || S < 1) return -1;
    vector<double> v(S);
    for (int i = 1; i < n; i++)
        for (int k = 0; k < S; k++) {
            for (int j = 0; j < S; j++) v[j] = fw[(size_t)(i - 1) * S + j] + trans[(size_t)j * S + k];
            fw[(size_t)i * S + k] = dense_logsum(v.data(), S) + emit[(size_t)i * S + k];
        }
    return 0;
}

int oracle_dense_backward(int n, int S, const double *trans, const double *emit, double *bw) {
    if (n < 1 || S < 1) return -1;
    vector<double> v(S);
    for (int i = n - 2; i >= 0; i--)
        for (int j = 0; j < S; j++) {
            for (int k = 0; k < S; k++)
                v[k] = trans[(size_t)j * S + k] + bw[(size_t)(i + 1) * S + k] +
                       emit[(size_t)(i + 1) * S + k];
            bw[(size_t)i * S + j] = dense_logsum(v.data(), S);
        }
    return 0;
}

// path[n-1] is given; u[i] is the uniform of column i (the reference draws them from n-2
// down to 0). The pick is the first index whose running weight reaches u[i] times the
// weights' sum (common.h:272-290).
int oracle_dense_sample(int n, int S, const double *trans, const double *fw, const double *u,
                        int *path) {
    if (n < 1 || S < 1) return -1;
    vector<double> a(S);
    for (int i = n - 2; i >= 0; i--) {
        const int k = path[i + 1];
        if (k < 0 || k >= S) return -2;
        for (int j = 0; j < S; j++) a[j] = fw[(size_t)i * S + j] + trans[(size_t)j * S + k];
        const double total = dense_logsum(a.data(), S);
        double sum = 0.0;
        for (int j = 0; j < S; j++) sum += (a[j] = std::exp(a[j] - total));
        const double pick = u[i] * sum;
        double run = 0.0;
        int pickj = S - 1;
        for (int j = 0; j < S; j++) {
            run += a[j];
            if (run >= pick) { pickj = j; break; }
        }
        path[i] = pickj;
    }
    return 0;
}

// ----------------------------------------------------------------------------- ARG probabilities
// calc_arg_likelihood (total_prob.cpp:19-45, likelihood_tree emit.cpp:399-446),
// calc_arg_prior (total_prob.cpp:262-300, calc_spr_prob :210-259) and calc_tree_prior
// (total_prob.cpp:132-165, prob_coal_counts :108-127), in the reference's order. The
// problem's sequences are one per leaf (more are allowed: the invariance test reads all),
// columns = the trees' sites. out: likelihood, prior, first-tree prior.

static double oracle_prob_coal_counts(int a, int b, double t, double n) {
    double C = 1.0;
    for (int y = 0; y < b; y++) C *= (b + y) * (a - y) / double(a + y);
    double s = exp(-b * (b - 1) * t / 2.0 / n) * C;
    for (int k = b + 1; k < a + 1; k++) {
        const double k1 = double(k - 1);
        C *= double(b + k1) * (a - k1) / (a + k1) / (b - k);
        s += exp(-k * k1 * t / 2.0 / n) * (2 * k - 1) / double(k1 + b) * C;
    }
    for (int i = 1; i <= b; i++) s /= i;
    return s;
}

int oracle_arg_prob(const oracle_problem *p, double *out) {
    Model m;
    if (!build_model(p, m)) return -1;
    const int n = p->nnodes, B = p->ntrees, T = p->ntimes;
    vector<Tree> trees(B);
    for (int b = 0; b < B; b++) {  // set_ptree (local_tree.h:216-229)
        Tree &t = trees[b];
        t.n = n;
        t.parent.assign(p->ptrees + (size_t)b * n, p->ptrees + (size_t)(b + 1) * n);
        t.age.assign(p->ages + (size_t)b * n, p->ages + (size_t)(b + 1) * n);
        t.c0.assign(n, -1);
        t.c1.assign(n, -1);
        for (int i = 0; i < n; i++) {
            const int par = t.parent[i];
            if (par < -1 || par >= n) return -2;
            if (par == -1) t.root = i;
            else if (t.c0[par] == -1) t.c0[par] = i;
            else if (t.c1[par] == -1) t.c1[par] = i;
            else return -2;
        }
        if (t.root < 0) return -2;
    }
    const double *times = m.times.data();
    const double mintime = m.mintime();
    // likelihood
    double lik = 0.0;
    if (n < 3) {
        lik = log(.25) * p->seqlen;
    } else {
        int end = 0;
        for (int b = 0; b < B; b++) {
            const Tree &t = trees[b];
            const int start = end;
            end = start + p->blocklens[b];
            vector<double> muts(n), nomuts(n);
            for (int i = 0; i < n; i++)
                if (i != t.root) {
                    const double tt = std::max(times[t.age[t.parent[i]]] - times[t.age[i]], mintime);
                    muts[i] = prob_branch(tt, m.mu, true);
                    nomuts[i] = prob_branch(tt, m.mu, false);
                }
            vector<int> order(n);  // LocalTree::get_postorder (local_tree.h:274-304)
            {
                vector<char> visit(n, 0);
                int i;
                for (i = 0; i < n; i++) {
                    if (!t.leaf(i)) break;
                    order[i] = i;
                }
                int e = i;
                for (i = 0; i < n; i++) {
                    const int parent = t.parent[order[i]];
                    if (parent != -1 && ++visit[parent] == 2) order[e++] = parent;
                }
            }
            double invariant_lk = -1, tree_lnl = 0.0;  // a tree's sum, then the total
            vector<lk_row> in(n);
            for (int i = start; i < end; i++) {
                bool inv = true;
                const char c0 = p->seqs[(size_t)0 * p->seqlen + i];
                for (int j = 1; j < p->nseqs && inv; j++) inv = p->seqs[(size_t)j * p->seqlen + i] == c0;
                double lk;
                if (inv && invariant_lk > 0) {
                    lk = invariant_lk;
                } else {
                    for (int oi = 0; oi < n; oi++) {  // likelihood_site_node_inner (emit.cpp:151-196)
                        const int j = order[oi];
                        if (t.leaf(j)) {
                            const char c = p->seqs[(size_t)j * p->seqlen + i];
                            if (c == 'N') { in[j][0] = in[j][1] = in[j][2] = in[j][3] = 1.0; }
                            else {
                                in[j][0] = in[j][1] = in[j][2] = in[j][3] = 0.0;
                                in[j][dna2int(c)] = 1.0;
                            }
                        } else {
                            const int c1 = t.c0[j], c2 = t.c1[j];
                            for (int a = 0; a < 4; a++) {
                                double p1 = 0.0, p2 = 0.0;
                                for (int bb = 0; bb < 4; bb++) {
                                    if (a == bb) { p1 += in[c1][bb] * nomuts[c1]; p2 += in[c2][bb] * nomuts[c2]; }
                                    else { p1 += in[c1][bb] * muts[c1]; p2 += in[c2][bb] * muts[c2]; }
                                }
                                in[j][a] = p1 * p2;
                            }
                        }
                    }
                    lk = 0.0;
                    for (int a = 0; a < 4; a++) lk += in[t.root][a] * .25;
                    if (inv) invariant_lk = lk;
                }
                tree_lnl += log(lk);
            }
            lik += tree_lnl;
        }
    }
    // prior
    double prior = 0.0;
    {
        long long total = 0;
        for (int b = 0; b < B; b++) total += p->blocklens[b];
        long long end = 0;
        for (int b = 0; b < B; b++) {
            const Tree &t = trees[b];
            end += p->blocklens[b];
            const int blocklen = p->blocklens[b];
            const double treelen = get_treelen(t, times, false);
            const double recomb_rate = std::max(m.rho * treelen, m.rho);
            if (end < total) {
                prior += log(recomb_rate) - recomb_rate * blocklen;
                const int *s = p->sprs + (size_t)(b + 1) * 4;
                const Spr spr{s[0], s[1], s[2], s[3]};
                // calc_spr_prob
                const int root_age = t.age[t.root];
                const double treelen_b = treelen + m.time_steps[t.age[t.root]];
                Lineages l;
                count_lineages(t, T, l);
                l.nrecombs[root_age]--;
                double lnl = 0.0;
                const int k = spr.recomb_time;
                lnl += log(l.nbranches[k] * m.time_steps[k] / (l.nrecombs[k] * treelen_b));
                const int broken_age = t.age[t.parent[spr.recomb_node]];
                vector<double> coal_rates(2 * T);
                for (int i = 0; i < 2 * T; i++) {  // calc_coal_rates_full_tree
                    const int nb = l.nbranches[i / 2] - int(i / 2 < broken_age);
                    coal_rates[i] = m.coal_time_steps[i] * nb / (2.0 * m.popsizes[i / 2]);
                }
                const int j = spr.coal_time;
                const int ncoals_j = l.ncoals[j] - int(j <= broken_age) - int(j == broken_age);
                lnl -= log(ncoals_j);
                if (j < T - 2)
                    lnl += log(1.0 - exp(-coal_rates[2 * j] - (j > k ? coal_rates[2 * j - 1] : 0.0)));
                for (int mm = 2 * k; mm < 2 * j - 1; mm++) lnl -= coal_rates[mm];
                prior += lnl;
            } else {
                prior += -recomb_rate * blocklen;
            }
        }
    }
    // first tree's prior
    double tprior = 0.0;
    {
        const Tree &t = trees[0];
        Lineages l;
        count_lineages(t, T, l);
        vector<double> tm(T), pm(T);
        tm[0] = m.coal_time_steps[0];
        pm[0] = m.popsizes[0];
        for (int i = 1; i < T - 1; i++) {
            const double t1 = m.coal_time_steps[2 * i - 1], t2 = m.coal_time_steps[2 * i];
            const double n1 = m.popsizes[i - 1], n2 = m.popsizes[i];
            tm[i] = t1 + t2;
            pm[i] = (t1 + t2) / (t1 / n1 + t2 / n2);
        }
        for (int i = 0; i < T - 1; i++) {
            const int a = (i == 0 ? t.nleaves() : l.nbranches[i - 1]);
            const int b = l.nbranches[i];
            tprior += log(oracle_prob_coal_counts(a, b, tm[i], 2.0 * pm[i]));
        }
    }
    out[0] = lik;
    out[1] = prior;
    out[2] = tprior;
    return 0;
}

// ----------------------------------------------------------------------------- recombinations
// sample_recombinations (recomb.cpp:151-235) with recomb_prob_unnormalized (:14-125) and
// get_possible_recomb (:128-148), over the oracle's blocks (states, lineage counts and
// TransMatrix as the reference builds them). u: the draws in order (frand() values).

static double oracle_recomb_prob(const Tree &t, const Model &m, const Lineages &l,
                                 int last_node, int last_time, int state_time, int rnode,
                                 int k, bool internal) {
    const int j = state_time;
    int root_time, recomb_parent_age;
    if (internal) {
        const int subtree_root = t.c0[t.root], maintree_root = t.c1[t.root];
        root_time = std::max(t.age[maintree_root], last_time);
        recomb_parent_age = (rnode == subtree_root || t.parent[rnode] == -1 ||
                             rnode == last_node) ? last_time : t.age[t.parent[rnode]];
    } else {
        root_time = std::max(t.age[t.root], last_time);
        recomb_parent_age = (rnode == -1 || t.parent[rnode] == -1 || rnode == last_node)
                                ? last_time : t.age[t.parent[rnode]];
    }
    const int nbranches_k = l.nbranches[k] + int(k < last_time);
    const int nrecombs_k = l.nrecombs[k] + int(k <= last_time) + int(k == last_time) -
                           int(k == root_time);
    const double precomb = nbranches_k * m.time_steps[k] / nrecombs_k;
    double sum = 0.0;
    for (int q = k; q < j - 1; q++) {
        const int nb = l.nbranches[q] + int(q < last_time) - int(q < recomb_parent_age);
        sum += (m.time_steps[q] * nb / (2.0 * m.popsizes[q]));
    }
    double pcoal = 1.0;
    const int nbranches_j = l.nbranches[j] + int(j < last_time) - int(j < recomb_parent_age);
    if (k == j) {
        if (j < m.T - 2)
            pcoal = 1.0 - exp(-m.coal_time_steps[2 * j] * nbranches_j / (2.0 * m.popsizes[j]));
    } else {
        const int q = j - 1;
        const int nb = l.nbranches[q] + int(q < last_time) - int(q < recomb_parent_age);
        sum += (m.coal_time_steps[2 * q] * nb / (2.0 * m.popsizes[q]));
        if (j < m.T - 2)
            pcoal = 1.0 - exp(-m.coal_time_steps[2 * j - 1] * nb / (2.0 * m.popsizes[q]) -
                              m.coal_time_steps[2 * j] * nbranches_j / (2.0 * m.popsizes[j]));
    }
    const int ncoals_j = l.ncoals[j] - int(j <= recomb_parent_age) -
                         int(j == recomb_parent_age) + int(j <= last_time) +
                         int(j == last_time);
    pcoal /= ncoals_j;
    return precomb * exp(-sum) * pcoal;
}

int oracle_sample_recombinations(const oracle_problem *p, const int *path, const double *u,
                                 int nu, int *pos, int *node, int *time, int cap, int *used) {
    Hmm h;
    if (!setup(p, h)) return -10;
    int count = 0, cu = 0;
    for (size_t b = 0; b < h.arg.trees.size(); b++) {
        Block blk;
        if (!make_block(h, (int)b, blk, false)) return -11;
        const Tree &t = h.arg.trees[b];
        if (h.internal && blk.states.size() == 0) continue;
        const int S = blk.states.size();
        const int start = blk.start + 1;  // every block: the region's start or a switch
        const int end = blk.start + blk.len;
        int next_recomb = -1;
        for (int i = start; i < end; i++) {
            const int ia = p->start_coord + i;
            if (path[i] < 0 || path[i] >= S || path[i - 1] < 0 || path[i - 1] >= S) return -1;
            if (path[i] == path[i - 1]) {
                if (ia > next_recomb) {
                    const int last = path[i - 1];
                    const int a = blk.states.time[last];
                    const double self_trans = blk.tm.get(t, blk.states, last, last);
                    const double rate = 1.0 - (blk.tm.norecombs[a] / self_trans);
                    if (cu >= nu) return -2;
                    const double e = -log(u[cu++]) / rate;  // expovariate (common.h:124)
                    next_recomb = int(std::min(double(p->start_coord + end), ia + e));
                }
                if (ia < next_recomb) continue;
            }
            next_recomb = -1;
            const int sn = blk.states.node[path[i]], st = blk.states.time[path[i]];
            const int ln = blk.states.node[path[i - 1]], lt = blk.states.time[path[i - 1]];
            vector<int> cn, ct;
            const int end_time = std::min(st, lt);
            if (sn == ln)
                for (int k = t.age[sn]; k <= end_time; k++) { cn.push_back(sn); ct.push_back(k); }
            if (h.internal) {
                const int sub = t.c0[t.root];
                for (int k = t.age[sub]; k <= end_time; k++) { cn.push_back(sub); ct.push_back(k); }
            } else {
                for (int k = 0; k <= end_time; k++) { cn.push_back(-1); ct.push_back(k); }
            }
            vector<double> probs(cn.size());
            for (size_t c = 0; c < cn.size(); c++)
                probs[c] = oracle_recomb_prob(t, h.m, blk.lineages, ln, lt, st, cn[c], ct[c],
                                              h.internal);
            // sample (common.h:272-290)
            double total = 0.0;
            for (double w : probs) total += w;
            if (cu >= nu) return -2;
            const double pick = u[cu++] * total;
            int pickc = (int)probs.size() - 1;
            double x = 0.0;
            for (size_t c = 0; c < probs.size(); c++) {
                x += probs[c];
                if (x >= pick) { pickc = (int)c; break; }
            }
            if (count >= cap) return -3;
            pos[count] = i;
            node[count] = cn[pickc];
            time[count] = ct[pickc];
            count++;
        }
    }
    *used = cu;
    return count;
}

}  // extern "C"


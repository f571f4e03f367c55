// Recombination sampling along a sampled thread (sample_recombinations, recomb.cpp:151-235)
// for one instance, external or internal-branch: plain sequential code, compiled for the device (one
// thread per instance, recomb.cu) and, by the tests, for the host, to check its logic
// against the reference's outputs before it runs on a GPU.
//
// Per local tree the routine needs the tree's lineage counts (count_lineages,
// local_tree.cpp:34-69) and, where it draws an optional recombination, the tree's
// transition terms (calc_transition_probs, trans.cpp:26-115) for the state's stay
// probability get(i, i) (trans.h:64-128) and norecombs. Both are computed the first time a
// tree needs them, in the reference's expressions and order.
//
// Randomness: the caller's uniforms, consumed in order, one per draw; the reference draws
// frand() = rand() / RAND_MAX at the same points (expovariate, common.h:124; sample,
// common.h:272-290), so the uniforms rand() gives after srand(seed) reproduce its result.
#pragma once

#include <cmath>

#include "awg_internal.h"

namespace awg {

// Node {parent, child0, child1, age} records of one tree; for an internal-branch tree the
// root is the virtual root, child0 the cut subtree's root (sub), child1 the main tree's
// (mainr), and states start at minage (the problem's, at least the subtree's age).
struct RsTree {
    const int4 *nd;
    int n, root;
    bool internal;
    int sub, mainr, minage;
};

// v lies in the cut subtree (walks bounded by n steps)
AWG_HD inline bool rs_in_sub(const RsTree &t, int v) {
    for (int s = 0; s <= t.n && v != -1; s++) {
        if (v == t.sub) return true;
        if (v == t.root) return false;
        v = t.nd[v].x;
    }
    return false;
}

struct RsModel {
    int T;
    const double *times, *tsteps, *csteps, *pops;
    double rho;
};

// count_lineages / count_lineages_internal (local_tree.cpp:34-131)
AWG_HD inline void rs_lineages(const RsTree &t, int T, int *nb, int *nr, int *nc) {
    for (int i = 0; i < T; i++) nb[i] = nr[i] = nc[i] = 0;
    if (t.internal) {
        for (int i = 0; i < t.n; i++) {
            if (i == t.sub || i == t.root) continue;
            const int parent = t.nd[i].x;
            const int parent_age = parent == t.root ? T - 2 : t.nd[parent].w;
            for (int j = t.nd[i].w; j < parent_age; j++) {
                nb[j]++;
                nr[j]++;
                nc[j]++;
            }
            nr[parent_age]++;
            nc[parent_age]++;
            if (parent == t.root) nb[parent_age]++;
        }
        for (int i = 0; i < t.nd[t.sub].w; i++) {
            nb[i]--;
            nc[i]--;
            nr[i]--;
        }
        nb[T - 1] = 1;
        return;
    }
    for (int i = 0; i < t.n; i++) {
        const int parent = t.nd[i].x;
        const int parent_age = parent == -1 ? T - 2 : t.nd[parent].w;
        for (int j = t.nd[i].w; j < parent_age; j++) {
            nb[j]++;
            nr[j]++;
            nc[j]++;
        }
        nr[parent_age]++;
        nc[parent_age]++;
        if (parent == -1) nb[parent_age]++;
    }
    nb[T - 1] = 1;
}

// logadd (common.h:157-163)
AWG_HD inline double rs_logadd(double lna, double lnb) {
    if (lna == -INFINITY) return lnb;
    if (lnb == -INFINITY) return lna;
    return fmax(lna, lnb) + log1p(exp(-fabs(lna - lnb)));
}

// The transition terms of an external tree (calc_transition_probs, trans.cpp:26-115).
struct RsTerms {
    double D[MAXT], E[MAXT], lnB[MAXT], lnE2[MAXT], G3[MAXT], lnG4[MAXT], norecombs[MAXT];
};

AWG_HD inline void rs_terms(const RsTree &t, const RsModel &m, const int *nb, const int *nr,
                            const int *nc, RsTerms &tr) {
    const int T = m.T;
    double coal_alloc[2 * MAXT + 1], C_alloc[2 * MAXT + 2];
    double *coal_rates = coal_alloc + 1, *C = C_alloc + 2;
    coal_rates[-1] = 0.0;  // calc_coal_rates_partial_tree (trans.cpp:13-21)
    for (int i = 0; i < 2 * T; i++)
        coal_rates[i] = m.csteps[i] * nb[i / 2] / (2.0 * m.pops[i / 2]);
    C[-2] = 0.0;
    C[-1] = 0.0;
    for (int b = 0; b < 2 * T - 1; b++) C[b] = C[b - 1] + coal_rates[b];
    // root, root age and tree length (trans.cpp:56-76): internal trees use the main tree's
    // root and get_treelen_internal minus the subtree's age; external ones get_treelen
    // without the basal branch (local_tree.cpp:136-176)
    const int root_age_index = t.internal ? t.nd[t.mainr].w : t.nd[t.root].w;
    const double root_age = m.times[root_age_index];
    double treelen = 0.0;
    for (int i = 0; i < t.n; i++) {
        const int parent = t.nd[i].x;
        if (parent == -1 || (t.internal && parent == t.root)) continue;
        treelen += m.times[t.nd[parent].w] - m.times[t.nd[i].w];
    }
    if (t.internal) treelen -= m.times[t.nd[t.sub].w];
    for (int b = 0; b < T - 1; b++) {
        double treelen2 = treelen + m.times[b];
        double treelen2_b;
        if (b > root_age_index) {
            treelen2 += m.times[b] - root_age;
            treelen2_b = treelen2 + m.tsteps[b];
        } else {
            treelen2_b = treelen2 + m.tsteps[root_age_index];
        }
        const double term = C[2 * b - 1] + log(m.tsteps[b] * (nb[b] + 1.0) / (nr[b] + 1.0));
        tr.lnB[b] = b == 0 ? term : rs_logadd(tr.lnB[b - 1], term);
        tr.lnE2[b] = -C[2 * b - 2] +
            (b < T - 2 ? log(1 - exp(-coal_rates[2 * b] - coal_rates[2 * b - 1])) : 0.0);
        tr.G3[b] = (b < T - 2 ? 1.0 - exp(-coal_rates[2 * b]) : 1.0) * m.tsteps[b] *
                   (nb[b] / (nr[b] + 1.0 + int(b < root_age_index)));
        tr.lnG4[b] = -C[2 * b - 2] +
            (b < T - 2 ? log(1.0 - exp(-coal_rates[2 * b] - coal_rates[2 * b - 1])) : 0.0);
        tr.D[b] = (1.0 - exp(-m.rho * treelen2)) / treelen2_b;
        tr.E[b] = 1.0 / nc[b];
        tr.norecombs[b] = exp(-fmax(m.rho * treelen2, m.rho));
    }
    tr.E[T - 2] = 1.0 / nc[T - 2];
}

// get(i, i) of a state at time a on a node of age c (trans.h:64-128: same node, a == b;
// minage 0, or the subtree's age for an internal tree)
AWG_HD inline double rs_stay(const RsTerms &tr, int a, int c, int minage) {
    if (a < minage) return 0.0;
    const double term1 = tr.D[a] * tr.E[a];
    double minage_term = 0.0;
    if (minage > 0) minage_term = exp(tr.lnG4[a] + tr.lnB[minage - 1]);
    const double eb = a > 0 ? exp(tr.lnE2[a] + tr.lnB[a - 1]) : 0.0;
    const double c_term = c > 0 ? exp(tr.lnG4[a] + tr.lnB[c - 1]) : 0.0;
    return term1 * ((2 * (eb + tr.G3[a])) - c_term - minage_term) + tr.norecombs[a];
}

// The states of one node: first time and count (get_coal_states_external /
// get_coal_states_internal, states.cpp:53-167): external, from the node's age up to its
// parent's (the root up to T - 2); internal, nodes of the main tree only, from
// max(age, minage) up to the parent's age (children of the virtual root up to T - 2), none
// at all when the tree is fully specified (virtual root below T).
AWG_HD inline int rs_node_states(const RsTree &t, int T, int v, int &t0) {
    if (!t.internal) {
        const int top = t.nd[v].x == -1 ? T - 2 : t.nd[t.nd[v].x].w;
        t0 = t.nd[v].w;
        return top - t0 + 1 > 0 ? top - t0 + 1 : 0;
    }
    if (t.nd[t.root].w < T || v == t.root || rs_in_sub(t, v)) return 0;
    t0 = t.nd[v].w > t.minage ? t.nd[v].w : t.minage;
    const int top = t.nd[v].x == t.root ? T - 2 : t.nd[t.nd[v].x].w;
    return top - t0 + 1 > 0 ? top - t0 + 1 : 0;
}

// State k: nodes in index order, times ascending. False if k is not a state.
AWG_HD inline bool rs_state(const RsTree &t, int T, int k, int &node, int &time) {
    if (k < 0) return false;
    for (int v = 0; v < t.n; v++) {
        int t0;
        const int m = rs_node_states(t, T, v, t0);
        if (k < m) {
            node = v;
            time = t0 + k;
            return true;
        }
        k -= m;
    }
    return false;
}

AWG_HD inline bool rs_has_states(const RsTree &t, int T) {
    for (int v = 0; v < t.n; v++) {
        int t0;
        if (rs_node_states(t, T, v, t0) > 0) return true;
    }
    return false;
}

// recomb_prob_unnormalized (recomb.cpp:14-125): recombination at (rnode, k) on the
// thread's branch (rnode -1; the subtree's root when internal) or the state's node, given
// the move last -> state
AWG_HD inline double rs_recomb_prob(const RsTree &t, const RsModel &m, const int *nb,
                                    const int *nr, const int *nc, int last_node, int last_time,
                                    int state_time, int rnode, int k) {
    const int j = state_time;
    const int top = t.internal ? t.nd[t.mainr].w : t.nd[t.root].w;
    const int root_time = top > last_time ? top : last_time;
    const bool own = t.internal ? rnode == t.sub : rnode == -1;
    const int recomb_parent_age =
        (own || t.nd[rnode].x == -1 || rnode == last_node) ? last_time : t.nd[t.nd[rnode].x].w;
    const int nbranches_k = nb[k] + int(k < last_time);
    const int nrecombs_k = nr[k] + int(k <= last_time) + int(k == last_time) - int(k == root_time);
    const double precomb = nbranches_k * m.tsteps[k] / nrecombs_k;
    double sum = 0.0;
    for (int q = k; q < j - 1; q++) {
        const int nbranches_m = nb[q] + int(q < last_time) - int(q < recomb_parent_age);
        sum += (m.tsteps[q] * nbranches_m / (2.0 * m.pops[q]));
    }
    double pcoal = 1.0;
    const int nbranches_j = nb[j] + int(j < last_time) - int(j < recomb_parent_age);
    if (k == j) {
        if (j < m.T - 2)
            pcoal = 1.0 - exp(-m.csteps[2 * j] * nbranches_j / (2.0 * m.pops[j]));
    } else {
        const int q = j - 1;
        const int nbranches_m = nb[q] + int(q < last_time) - int(q < recomb_parent_age);
        sum += (m.csteps[2 * q] * nbranches_m / (2.0 * m.pops[q]));
        if (j < m.T - 2)
            pcoal = 1.0 - exp(-m.csteps[2 * j - 1] * nbranches_m / (2.0 * m.pops[q]) -
                              m.csteps[2 * j] * nbranches_j / (2.0 * m.pops[j]));
    }
    const int ncoals_j = nc[j] - int(j <= recomb_parent_age) - int(j == recomb_parent_age) +
                         int(j <= last_time) + int(j == last_time);
    pcoal /= ncoals_j;
    return precomb * exp(-sum) * pcoal;
}

// One instance's inputs and outputs.
struct RsInstance {
    const int4 *nodes;        // [ntrees][nnodes]
    const int *blocklens;     // [ntrees]
    const int *path;          // [seqlen] state index per column
    const double *u;          // [nu] uniforms, consumed in order
    int ntrees, nnodes, nu, start_coord;
    bool internal;            // internal-branch problem (virtual root, cut subtree)
    int minage;               // the problem's minimum state age (internal)
    int *pos, *node, *time;   // [cap] recombinations: column, node (-1: the thread), time
    int cap;
};

enum : int { RS_OK = 0, RS_BAD_STATE = -1, RS_OUT_OF_UNIFORMS = -2, RS_FULL = -3 };

// sample_recombinations (recomb.cpp:151-235): the recombinations of one thread path;
// returns their count (or an RS_ code) and the uniforms used in *used
AWG_HD inline int rs_sample(const RsInstance &in, const RsModel &m, int *used) {
    int nb[MAXT], nr[MAXT], nc[MAXT];
    RsTerms tr;
    double probs[2 * MAXT + 2];
    int cnode[2 * MAXT + 2], ctime[2 * MAXT + 2];
    int count = 0, cu = 0, end = 0;
    for (int b = 0; b < in.ntrees; b++) {
        RsTree t{in.nodes + (size_t)b * in.nnodes, in.nnodes, -1, in.internal, -1, -1, 0};
        for (int v = 0; v < t.n; v++)
            if (t.nd[v].x == -1) t.root = v;
        if (t.root < 0) return RS_BAD_STATE;
        if (t.internal) {
            t.sub = t.nd[t.root].y;
            t.mainr = t.nd[t.root].z;
            if (t.sub < 0 || t.mainr < 0) return RS_BAD_STATE;
            t.minage = in.minage > t.nd[t.sub].w ? in.minage : t.nd[t.sub].w;
        }
        const int start = end;
        end = start + in.blocklens[b];
        if (t.internal && !rs_has_states(t, m.T)) continue;  // no state space: no sampling
        bool have_lineages = false, have_terms = false;
        int next_recomb = -1;  // absolute coordinate
        // a block's first column takes no new recombination: the first block starts the
        // region, every later one begins with a switch
        for (int i = start + 1; i < end; i++) {
            const int ia = in.start_coord + i;
            if (in.path[i] == in.path[i - 1]) {
                if (ia > next_recomb) {  // draw the distance to the next optional one
                    int ln, lt;
                    if (!rs_state(t, m.T, in.path[i - 1], ln, lt)) return RS_BAD_STATE;
                    if (!have_lineages) {
                        rs_lineages(t, m.T, nb, nr, nc);
                        have_lineages = true;
                    }
                    if (!have_terms) {
                        rs_terms(t, m, nb, nr, nc, tr);
                        have_terms = true;
                    }
                    const double self_trans =
                        rs_stay(tr, lt, t.nd[ln].w, t.internal ? t.nd[t.sub].w : 0);
                    const double rate = 1.0 - (tr.norecombs[lt] / self_trans);
                    if (cu >= in.nu) return RS_OUT_OF_UNIFORMS;
                    const double e = -log(in.u[cu++]) / rate;  // expovariate
                    const double endd = double(in.start_coord + end), to = ia + e;
                    next_recomb = int(endd < to ? endd : to);
                }
                if (ia < next_recomb) continue;
            }
            next_recomb = -1;
            int sn, st, ln, lt;
            if (!rs_state(t, m.T, in.path[i], sn, st) || !rs_state(t, m.T, in.path[i - 1], ln, lt))
                return RS_BAD_STATE;
            if (!have_lineages) {
                rs_lineages(t, m.T, nb, nr, nc);
                have_lineages = true;
            }
            // get_possible_recomb (recomb.cpp:128-148)
            int nc_ = 0;
            const int end_time = st < lt ? st : lt;
            if (sn == ln)
                for (int k = t.nd[sn].w; k <= end_time; k++) {
                    cnode[nc_] = sn;
                    ctime[nc_++] = k;
                }
            if (t.internal) {
                for (int k = t.nd[t.sub].w; k <= end_time; k++) {
                    cnode[nc_] = t.sub;
                    ctime[nc_++] = k;
                }
            } else {
                for (int k = 0; k <= end_time; k++) {
                    cnode[nc_] = -1;
                    ctime[nc_++] = k;
                }
            }
            double total = 0.0;
            for (int c = 0; c < nc_; c++) {
                probs[c] = rs_recomb_prob(t, m, nb, nr, nc, ln, lt, st, cnode[c], ctime[c]);
                total += probs[c];
            }
            // sample (common.h:272-290)
            if (cu >= in.nu) return RS_OUT_OF_UNIFORMS;
            const double pick = in.u[cu++] * total;
            int pickc = nc_ - 1;
            double x = 0.0;
            for (int c = 0; c < nc_; c++) {
                x += probs[c];
                if (x >= pick) {
                    pickc = c;
                    break;
                }
            }
            if (count >= in.cap) return RS_FULL;
            in.pos[count] = i;
            in.node[count] = cnode[pickc];
            in.time[count] = ctime[pickc];
            count++;
        }
    }
    *used = cu;
    return count;
}

}  // namespace awg

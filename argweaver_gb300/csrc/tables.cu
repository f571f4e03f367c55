// K1 (block tables) and K2 (variant-column emissions), FP64.
//
// One CTA per local tree. Each table is a device restatement of the reference's builder
// and keeps its operation order, so the plain FP64 path differs from the reference only by
// the last-bit differences between CUDA's and the host's exp/log:
//   states / lookups            states.cpp:53-167, states.h:53-131
//   lineage counts              local_tree.cpp:34-131
//   tree lengths                local_tree.cpp:136-219
//   transition terms            trans.cpp:13-115;  entries trans.h:89-128
//   tmatrix / same-branch rows  sample_thread.cpp:209-226
//   switch matrix               trans.cpp:156-739
//   state priors                trans.cpp:785-831
//   emissions                   emit.cpp:86-116, 151-324, 620-845
// The switch step's deterministic scatter (sample_thread.cpp:357-362) is inverted here into
// a gather list per target state, sources in ascending order, so the forward kernel adds
// them in the reference's order without atomics.

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>

#include "kernels.h"

namespace awg {

namespace {

constexpr int TAB_THREADS = 128;

struct Terms {
    double D[MAXT], E[MAXT], lnB[MAXT], lnE2[MAXT], lnNegG1[MAXT], G2[MAXT], G3[MAXT],
        lnG4[MAXT], norecombs[MAXT];
    // the exponentials get_time needs, each evaluated once per tree:
    double EB[MAXT];              // exp(lnE2[b] + lnB[b-1]), b > 0
    double E2B[MAXT][MAXT];       // [a][b] exp(lnE2[b] + lnB[a])
    double E2N[MAXT][MAXT];       // [a][b] exp(lnE2[b] + lnNegG1[a])
    double CT[MAXT][MAXT];        // [b][c] exp(lnG4[b] + lnB[c-1]), c > 0
};

// Fill the exponential tables (the same arguments get_time exponentiates), only the
// entries get_time reads: E2B/E2N[a][b] for a < b (the a < b branch), CT[b][c] for
// 1 <= c <= b (c_term and minage_term: a state's time is at least its node's age and minage).
__device__ void exp_tables(Terms &t, int T) {
    for (int e = threadIdx.x; e < (T - 1) * (T - 1); e += blockDim.x) {
        const int a = e / (T - 1), b = e % (T - 1);
        if (a < b) {
            t.E2B[a][b] = exp(t.lnE2[b] + t.lnB[a]);
            t.E2N[a][b] = exp(t.lnE2[b] + t.lnNegG1[a]);
        } else if (b < a) {
            t.CT[a][b + 1] = exp(t.lnG4[a] + t.lnB[b]);  // [b=a][c=b+1]
        }
    }
    for (int b = threadIdx.x; b < T - 1; b += blockDim.x)
        t.EB[b] = b > 0 ? exp(t.lnE2[b] + t.lnB[b - 1]) : 0.0;
}

// TransMatrix::get_time (trans.h:89-128) over the precomputed exponentials: every value is
// the one the reference computes, in the same order.
__device__ double get_time(const Terms &t, int a, int b, int c, int minage, bool same_node) {
    if (a < minage || b < minage) return 0.0;
    double term1 = __dmul_rn(t.D[a], t.E[b]);
    double minage_term = 0.0;
    if (minage > 0) minage_term = t.CT[b][minage];
    const double eb = t.EB[b];
    if (!same_node) {
        if (a < b) return term1 * (t.E2B[a][b] - t.E2N[a][b] - minage_term);
        if (a == b) return term1 * (eb + t.G3[b] - minage_term);
        return term1 * (eb + t.G2[b] - minage_term);
    }
    double c_term = (c > 0 ? t.CT[b][c] : 0.0);
    if (a < b) return term1 * (2 * (t.E2B[a][b] - t.E2N[a][b]) - c_term - minage_term);
    if (a == b) return term1 * ((2 * (eb + t.G3[b])) - c_term - minage_term) + t.norecombs[a];
    return term1 * ((2 * (eb + t.G2[b])) - c_term - minage_term);
}

__device__ __forceinline__ double logadd(double lna, double lnb) {  // common.h:157-163
    if (lna == -INFINITY) return lnb;
    if (lnb == -INFINITY) return lna;
    return fmax(lna, lnb) + log1p(exp(-fabs(lna - lnb)));
}

// State ranges of every node of one tree (states.cpp:53-167): first state, first time,
// count, and (optionally) the offset of the node's same-branch rows. Thread 0 only.
__device__ int node_ranges(const int4 *nd, int n, int root, int T, bool internal,
                           int minage_param, int *first, int *t0, int *cnt, int *t2base,
                           int *stack, char *ignore) {
    int S = 0, M = 0;
    for (int v = 0; v < n; v++) ignore[v] = 0;
    int minage = 0;
    bool none = false;
    if (internal) {
        if (nd[root].w < T) {
            none = true;
        } else {
            const int sub = nd[root].y;
            minage = max(minage_param, nd[sub].w);
            ignore[root] = 1;
            int sp = 0;
            stack[sp++] = sub;
            while (sp > 0) {
                int v = stack[--sp];
                ignore[v] = 1;
                if (nd[v].y != -1) { stack[sp++] = nd[v].y; stack[sp++] = nd[v].z; }
            }
        }
    }
    for (int v = 0; v < n; v++) {
        int m = 0, start = nd[v].w;
        if (!none && !ignore[v]) {
            const int p = nd[v].x;
            start = internal ? max(nd[v].w, minage) : nd[v].w;
            const bool top_branch = internal ? (p == root) : (p == -1);
            const int top = top_branch ? T - 2 : nd[p].w;
            m = max(0, top - start + 1);
        }
        first[v] = S;
        t0[v] = start;
        cnt[v] = m;
        if (t2base) t2base[v] = M;
        S += m;
        M += m * m;
    }
    return S;
}

__device__ __forceinline__ int lookup(const int *first, const int *t0, const int *cnt, int v,
                                      int t) {
    if (v < 0 || cnt[v] == 0) return -1;
    int d = t - t0[v];
    if (d < 0 || d >= cnt[v]) return -1;
    return first[v] + d;
}

// Lineage counts of one tree (count_lineages[_internal], local_tree.cpp:34-131); thread t
// fills time slice t.
__device__ void lineage_counts(const int4 *nd, int n, int root, int T, bool internal, int *nb,
                               int *nr, int *nc) {
    for (int t = threadIdx.x; t < T; t += blockDim.x) {
        int b = 0, r = 0, c = 0;
        const int sub = internal ? nd[root].y : -1;
        for (int i = 0; i < n; i++) {
            if (internal && (i == sub || i == root)) continue;
            const int p = nd[i].x;
            const bool top_branch = internal ? (p == root) : (p == -1);
            const int pa = top_branch ? T - 2 : nd[p].w;
            if (nd[i].w <= t && t < pa) { b++; r++; c++; }
            if (t == pa) { r++; c++; if (top_branch) b++; }
        }
        if (internal && t < nd[sub].w) { b--; c--; r--; }
        if (t == T - 1) b = 1;
        nb[t] = b; nr[t] = r; nc[t] = c;
    }
}

// get_treelen (use_basal=false) / get_treelen_internal; node order as the reference.
__device__ double treelen_of(const int4 *nd, int n, int root, const double *times,
                             bool internal) {
    double s = 0.0;
    for (int i = 0; i < n; i++) {
        const int p = nd[i].x;
        if (p == -1) continue;
        if (internal && p == root) continue;
        s += times[nd[p].w] - times[nd[i].w];
    }
    return s;
}

struct SwitchCtx {
    const int4 *last, *cur;
    int last_root, cur_root, T;
    const int *mapping;
    const double *times, *tsteps, *csteps, *pops;
    const int *nb, *nr, *nc;  // lineages of the previous tree
    double rho, last_treelen;
    bool internal;
};

__device__ __forceinline__ int sibling(const int4 *nd, int v) {
    const int p = nd[v].x;
    if (p == -1) return -1;
    return nd[p].y == v ? nd[p].z : nd[p].y;
}

// calc_recomb (trans.cpp:317-413)
__device__ double calc_recomb(const SwitchCtx &c, const int *spr, int state_node, int state_time,
                              double last_treelen) {
    const int a = state_time, k = spr[1];
    const int4 *last = c.last;
    double last_treelen_b;
    int root_age;
    if (c.internal) {
        const int sub = last[c.last_root].y, mainr = last[c.last_root].z;
        root_age = last[mainr].w;
        if (spr[2] == sub) {
            if (a < spr[3]) return 0.0;
            if (spr[0] == mainr && state_node != mainr) return 0.0;
        }
        int ptr = spr[2], ptr2 = -1, ptr3 = -1;
        while (ptr != c.last_root) { ptr2 = ptr; ptr = last[ptr].x; }
        ptr = spr[0];
        while (ptr != c.last_root) { ptr3 = ptr; ptr = last[ptr].x; }
        if (ptr2 == sub && ptr3 == mainr && state_time == spr[1]) {
            ptr = last[state_node].x;
            while (ptr != c.last_root) {
                if (ptr == spr[0]) return 0.0;
                ptr = last[ptr].x;
            }
        }
        last_treelen += c.times[a] - c.times[last[sub].w];
        if (a > root_age) {
            last_treelen += c.times[a] - c.times[root_age];
            last_treelen_b = last_treelen + c.tsteps[a];
        } else {
            last_treelen_b = last_treelen + c.tsteps[root_age];
        }
    } else {
        root_age = last[c.last_root].w;
        // get_treelen_branch (local_tree.cpp:179-203), use_basal = false
        double blen = c.times[a];
        double treelen2 = last_treelen + blen;
        if (state_node == c.last_root) treelen2 += blen - c.times[last[c.last_root].w];
        last_treelen = treelen2;
        // get_basal_branch (local_tree.cpp:206-219)
        double root_time;
        if (state_node == c.last_root) root_time = c.times[a + 1] - c.times[a];
        else root_time = c.times[root_age + 1] - c.times[root_age];
        last_treelen_b = last_treelen + root_time;
    }
    int nbranches_k = c.nb[k] + int(k < a);
    int nrecombs_k = c.nr[k] + int(k <= a) + int(k == a) - int(k >= max(root_age, a));
    return nbranches_k * c.tsteps[k] / (nrecombs_k * last_treelen_b) *
           (1.0 - exp(-fmax(c.rho * last_treelen, c.rho)));
}

// calc_recoal (trans.cpp:443-502)
__device__ double calc_recoal(const SwitchCtx &c, const int *spr, int state1_time,
                              int recomb_parent_age, bool internal) {
    const int a = state1_time, k = spr[1], j = spr[3];
    int nbranches_j = c.nb[j] - int(j < recomb_parent_age) + int(j < a);
    int ncoals_j = c.nc[j] - int(j <= recomb_parent_age) - int(j == recomb_parent_age) +
                   int(j <= a) + int(j == a);
    bool over = false;
    if (internal) {
        const int sub = c.last[c.last_root].y, mainr = c.last[c.last_root].z;
        if (spr[0] == mainr && spr[3] >= c.last[sub].w) {
            over = true;
            nbranches_j = 1;
            ncoals_j++;
        }
    }
    double p = 1.0 / ncoals_j;
    if (j < c.T - 2) {
        double Z = 0.0;
        if (j > k) {
            int b1 = c.nb[j - 1] - int(j - 1 < recomb_parent_age) + int(j - 1 < a);
            if (over) b1 = 1;
            Z = c.csteps[2 * j - 1] * b1 / (2.0 * c.pops[j - 1]);
        }
        p *= 1.0 - exp(-c.csteps[2 * j] * nbranches_j / (2.0 * c.pops[j]) - Z);
    }
    return p;
}

// calc_recomb_recoal (trans.cpp:505-534)
__device__ double calc_recomb_recoal(const SwitchCtx &c, const int *spr, int state_node,
                                     int state_time, int recomb_parent_age) {
    const int a = state_time, k = spr[1], j = spr[3];
    double p = calc_recomb(c, spr, state_node, state_time, c.last_treelen);
    double sum = 0.0;
    for (int m = 2 * k; m < 2 * j - 1; m++) {
        int nbm = c.nb[m / 2] - int(m / 2 < recomb_parent_age) + int(m / 2 < a);
        sum += c.csteps[m] * nbm / (2.0 * c.pops[m / 2]);
    }
    p *= exp(-sum);
    p *= calc_recoal(c, spr, state_time, recomb_parent_age, c.internal);
    return p;
}

__device__ __forceinline__ double prob_branch(double t, double mu, bool mut) {  // emit.cpp:86
    const double f = 4. / 3.;
    if (!mut) return .25 * (1.0 + 3. * exp(-f * mu * t));
    return .25 * (1.0 - exp(-f * mu * t));
}


// ---------------------------------------------------------------------------------------
// K1

__global__ void __launch_bounds__(TAB_THREADS) k_tables(BatchDev d, int want32) {
    extern __shared__ int4 dyn[];
    const int blk = cta_block(d);
    BlockDev &Bg = d.blocks[blk];
    const BlockDev B = Bg;
    const InstDev I = d.inst[B.inst];
    const int T = I.T, n = I.nnodes;
    const bool internal = I.internal != 0;
    const int tid = threadIdx.x;

    int4 *cur = dyn;
    int4 *prv = cur + n;
    int *first = (int *)(prv + n);
    int *t0 = first + n;
    int *cnt = t0 + n;
    int *t2base = cnt + n;
    int *pfirst = t2base + n;
    int *pt0 = pfirst + n;
    int *pcnt = pt0 + n;
    int *stack = pcnt + n;
    char *ignore = (char *)(stack + n);
    int *s1node = (int *)(ignore + ((n + 15) & ~15));  // prev states [S1]
    int *s1time = s1node + imax(B.S1, 1);
    int *gcnt = s1time + imax(B.S1, 1);                 // [S+1]

    __shared__ double times[MAXT], tsteps[MAXT], csteps[2 * MAXT], pops[MAXT];
    __shared__ double coal_rates_alloc[2 * MAXT + 1], C_alloc[2 * MAXT + 2], lnBterm[MAXT];
    __shared__ Terms tr;
    __shared__ int nb[MAXT], nr[MAXT], nc[MAXT], pnb[MAXT], pnr[MAXT], pnc[MAXT];
    __shared__ double sums2[2 * MAXT + 1], recoals[MAXT];
    __shared__ double sh_treelen, sh_sums, sh_maintreelen, sh_subtreelen, sh_tlmin;
    __shared__ double wmin[TAB_THREADS / 32];
    __shared__ double tl_tab[2 * MAXT], inv_tab[2 * MAXT], dp_tab[3 * MAXT];
    __shared__ int sh_S, sh_S1, sh_minage, sh_rootage, sh_src[2];

    const double *model = d.model + I.model0;
    for (int i = tid; i < T; i += blockDim.x) {
        times[i] = model[M_TIMES + i];
        tsteps[i] = model[M_TIMESTEPS + i];
        pops[i] = model[M_POPSIZES + i];
    }
    for (int i = tid; i < 2 * T; i += blockDim.x) csteps[i] = model[M_COALSTEPS + i];
    const double rho = model[M_CONST + 0], mu = model[M_CONST + 1], mintime = model[M_CONST + 2];
    for (int i = tid; i < n; i += blockDim.x) {
        cur[i] = d.nodes[B.nodes0 + i];
        if (B.b > 0) prv[i] = d.nodes[B.prev_nodes0 + i];
    }
    __syncthreads();

    const int root = B.root;
    if (tid == 0) {
        sh_S = node_ranges(cur, n, root, T, internal, I.minage, first, t0, cnt, t2base, stack,
                           ignore);
        if (B.b > 0)
            sh_S1 = node_ranges(prv, n, B.prev_root, T, internal, I.minage, pfirst, pt0, pcnt,
                                nullptr, stack, ignore);
        // TransMatrix::minage: max(StatesModel::minage, subtree age) when internal
        sh_minage = internal ? max(I.minage, cur[cur[root].y].w) : 0;
    }
    __syncthreads();
    const int S = sh_S;
    const int Sm = imax(S, 1);
    const int minage = sh_minage;
    if (S != B.S || (B.b > 0 && sh_S1 != B.S1)) {
        if (tid == 0) report_error(d.err, ERR_PLAN_MISMATCH, B.inst, B.b, B.start);
        return;
    }
    if (tid == 0) Bg.minage = minage;

    // per-state metadata and same-branch row offsets
    StateInfo *sinfo = d.sinfo + B.state0;
    int *t2off = d.t2off + B.state0;
    for (int v = tid; v < n; v += blockDim.x) {
        const int m = cnt[v];
        for (int y = 0; y < m; y++) {
            const int k = first[v] + y;
            sinfo[k] = StateInfo{v, t0[v] + y, first[v], m};
            t2off[k] = t2base[v] + y;  // entry (k, source y') at t2off[k] + y' * m
        }
    }
    if (S == 0 && tid == 0) {
        sinfo[0] = StateInfo{-1, 0, 0, 1};
        t2off[0] = 0;
    }

    // lineage counts of this tree, and of the previous tree for the switch
    lineage_counts(cur, n, root, T, internal, nb, nr, nc);
    if (B.b > 0) lineage_counts(prv, n, B.prev_root, T, internal, pnb, pnr, pnc);
    __syncthreads();

    // transition terms (calc_transition_probs, trans.cpp:26-115)
    if (tid == 0) {
        double *coal_rates = &coal_rates_alloc[1];
        coal_rates[-1] = 0.0;
        for (int i = 0; i < 2 * T; i++) coal_rates[i] = csteps[i] * nb[i / 2] / (2.0 * pops[i / 2]);
        double *C = &C_alloc[2];
        C[-2] = 0.0;
        C[-1] = 0.0;
        for (int b = 0; b < 2 * T - 1; b++) C[b] = C[b - 1] + coal_rates[b];
        double treelen;
        int root_age_index;
        if (internal) {
            const int sub = cur[root].y, mainr = cur[root].z;
            root_age_index = cur[mainr].w;
            treelen = treelen_of(cur, n, root, times, true) - times[cur[sub].w];
        } else {
            root_age_index = cur[root].w;
            treelen = treelen_of(cur, n, root, times, false);
        }
        sh_treelen = treelen;
        sh_rootage = root_age_index;
    }
    __syncthreads();
    {
        const double *coal_rates = &coal_rates_alloc[1];
        const double *C = &C_alloc[2];
        const int root_age_index = sh_rootage;
        const double root_age = times[root_age_index];
        for (int b = tid; b < T - 1; b += blockDim.x) {
            double treelen2 = sh_treelen + times[b];
            double treelen2_b;
            if (b > root_age_index) {
                treelen2 += times[b] - root_age;
                treelen2_b = treelen2 + tsteps[b];
            } else {
                treelen2_b = treelen2 + tsteps[root_age_index];
            }
            lnBterm[b] = C[2 * b - 1] + log(tsteps[b] * (nb[b] + 1.0) / (nr[b] + 1.0));
            tr.lnE2[b] = -C[2 * b - 2] +
                (b < T - 2 ? log(1 - exp(-coal_rates[2 * b] - coal_rates[2 * b - 1])) : 0.0);
            tr.lnNegG1[b] = C[2 * b - 1] + log(-tsteps[b] *
                ((nb[b] / (nr[b] + 1.0 + int(b < root_age_index))) - (nb[b] + 1.0) / (nr[b] + 1.0)));
            tr.G2[b] = (b < T - 2 ? 1.0 - exp(-coal_rates[2 * b]) : 1.0) * tsteps[b] *
                       (nb[b] + 1.0) / (nr[b] + 1.0);
            tr.G3[b] = (b < T - 2 ? 1.0 - exp(-coal_rates[2 * b]) : 1.0) * tsteps[b] *
                       (nb[b] / (nr[b] + 1.0 + int(b < root_age_index)));
            tr.lnG4[b] = -C[2 * b - 2] +
                (b < T - 2 ? log(1.0 - exp(-coal_rates[2 * b] - coal_rates[2 * b - 1])) : 0.0);
            tr.D[b] = (1.0 - exp(-rho * treelen2)) / treelen2_b;
            tr.E[b] = 1.0 / nc[b];
            tr.norecombs[b] = exp(-fmax(rho * treelen2, rho));
            if (want32) d.rstay32[(size_t)blk * MAXT + b] = (float)(-expm1(-fmax(rho * treelen2, rho)));
        }
    }
    __syncthreads();
    if (tid == 0) {
        tr.lnB[0] = lnBterm[0];
        for (int b = 1; b < T - 1; b++) tr.lnB[b] = logadd(tr.lnB[b - 1], lnBterm[b]);
        tr.E[T - 2] = 1.0 / nc[T - 2];
    }
    __syncthreads();
    exp_tables(tr, T);
    __syncthreads();

    // tmatrix[a][b] = get_time(a, b, 0, minage, false) (sample_thread.cpp:212-216)
    double *tm = d.tm + (size_t)blk * MAXT * MAXT;
    for (int e = tid; e < (T - 1) * (T - 1); e += blockDim.x) {
        const int a = e / (T - 1), b = e % (T - 1);
        const double v = get_time(tr, a, b, 0, minage, false);
        tm[a * MAXT + b] = v;
        if (want32) d.tm32[(size_t)blk * MAXT * MAXT + a * MAXT + b] = (float)v;
    }
    __syncthreads();

    // same-branch rows: get_time(a, b_k, c_k, minage, true) for the node's times a; a node's
    // m x m block is stored source-major (entry (k, y) at t2off[k] + y * m) so lanes holding
    // consecutive states of one node read consecutive words
    if (!want32) {
        double *gts = d.gts + B.t2_0;
        for (int k = tid; k < S; k += blockDim.x) {
            const StateInfo si = sinfo[k];
            const int b = si.time, c = cur[si.node].w;
            const int base = t2off[k];
            for (int y = 0; y < si.m; y++) {
                const int a = t0[si.node] + y;
                gts[base + y * si.m] = get_time(tr, a, b, c, minage, true);
            }
        }
    } else {
        // FP32 path: only the moving part, get_time(a, b, c, true) - get_time(a, b, 0, false)
        // - [a == b] norecombs[a], which in exact arithmetic is D[a] E[b] (X[a][b] - c_term)
        // (X the different-node bracket without its minage term); formed from that product
        // it keeps its relative accuracy where the two get_time values nearly cancel.
        // X and D[a] E[b] overwrite E2B and E2N, which nothing reads after this point.
        for (int e = tid; e < (T - 1) * (T - 1); e += blockDim.x) {
            const int a = e / (T - 1), b = e % (T - 1);
            const double x = a < b ? tr.E2B[a][b] - tr.E2N[a][b]
                                   : tr.EB[b] + (a == b ? tr.G3[b] : tr.G2[b]);
            tr.E2N[a][b] = __dmul_rn(tr.D[a], tr.E[b]);
            tr.E2B[a][b] = x;
        }
        __syncthreads();
        float *t2d = d.t2d32 + B.t2_0;
        for (int k = tid; k < S; k += blockDim.x) {
            const StateInfo si = sinfo[k];
            const int b = si.time, c = cur[si.node].w;
            const int base = t2off[k];
            const double ct = c > 0 ? tr.CT[b][c] : 0.0;
            for (int y = 0; y < si.m; y++) {
                const int a = t0[si.node] + y;
                t2d[base + y * si.m] =
                    (a < minage || b < minage) ? 0.0f : (float)(tr.E2N[a][b] * (tr.E2B[a][b] - ct));
            }
        }
    }

    // states grouped by time, ascending state index within a time
    int *bt_ptr = d.bt_ptr + (size_t)blk * (MAXT + 1);
    int *bt_perm = d.bt_perm + B.state0;
    for (int a = tid; a < MAXT; a += blockDim.x) {
        int c = 0;
        for (int v = 0; v < n; v++)
            if (cnt[v] && t0[v] <= a && a < t0[v] + cnt[v]) c++;
        gcnt[a] = c;
    }
    __syncthreads();
    if (tid == 0) {
        int acc = 0;
        for (int a = 0; a < MAXT; a++) {
            bt_ptr[a] = acc;
            int c = gcnt[a];
            gcnt[a] = acc;
            acc += c;
        }
        bt_ptr[MAXT] = acc;
    }
    __syncthreads();
    for (int a = tid; a < MAXT; a += blockDim.x) {
        int pos = gcnt[a];
        for (int v = 0; v < n; v++)
            if (cnt[v] && t0[v] <= a && a < t0[v] + cnt[v]) bt_perm[pos++] = first[v] + a - t0[v];
    }

    // invariant-site emission per state (emit.cpp:744-819)
    if (tid == 0) {
        const int mainr = internal ? cur[root].z : root;
        const int sub = internal ? cur[root].y : root;
        double mt = 0.0, st = 0.0;
        int sp = 0;
        stack[sp++] = mainr;
        while (sp > 0) {
            int v = stack[--sp];
            if (v != mainr) {
                const int p = cur[v].x;
                const double dist = p != -1 ? times[cur[p].w] - times[cur[v].w] : 0.0;
                mt += fmax(dist, mintime);
            }
            if (cur[v].y != -1) { stack[sp++] = cur[v].y; stack[sp++] = cur[v].z; }
        }
        if (internal) {
            stack[sp++] = sub;
            while (sp > 0) {
                int v = stack[--sp];
                if (v != sub) {
                    const int p = cur[v].x;
                    const double dist = p != -1 ? times[cur[p].w] - times[cur[v].w] : 0.0;
                    st += fmax(dist, mintime);
                }
                if (cur[v].y != -1) { stack[sp++] = cur[v].y; stack[sp++] = cur[v].z; }
            }
        }
        sh_maintreelen = mt;
        sh_subtreelen = st;
    }
    __syncthreads();
    {
        double *inv = d.inv_lk + B.state0;
        const int mainr = internal ? cur[root].z : root;
        const int node1 = internal ? cur[root].y : 0;
        const double time1 = internal ? times[cur[node1].w] : 0.0;
        // tree length seen by each state (emit.cpp:807-816), floored at mintime
        // the tree length depends on the state only through (node == main root, time):
        // one value per pair, then a lookup per state
        for (int e = tid; e < 2 * T; e += blockDim.x) {
            const int t = e % T;
            const double coal_time = times[t];
            double treelen;
            if (e >= T)
                treelen = sh_maintreelen + sh_subtreelen + fmax(coal_time - time1, mintime) +
                          fmax(coal_time - times[cur[mainr].w], mintime);
            else
                treelen = sh_maintreelen + sh_subtreelen + fmax(coal_time - time1, mintime);
            tl_tab[e] = fmax(treelen, mintime);
            inv_tab[e] = .25 * exp(-mu * tl_tab[e]);
        }
        __syncthreads();
        auto pair = [&](int k) {
            const StateInfo si = sinfo[k];
            return (si.node == mainr ? T : 0) + si.time;
        };
        double lmin = INFINITY;
        for (int k = tid; k < S; k += blockDim.x) {
            const int e = pair(k);
            inv[k] = inv_tab[e];
            lmin = fmin(lmin, tl_tab[e]);
        }
        if (want32) {
            for (int o = 16; o > 0; o >>= 1) lmin = fmin(lmin, __shfl_xor_sync(0xffffffffu, lmin, o));
            if ((tid & 31) == 0) wmin[tid >> 5] = lmin;
            __syncthreads();
            if (tid == 0) {
                double m = INFINITY;
                for (int w = 0; w < (int)(blockDim.x >> 5); w++) m = fmin(m, wmin[w]);
                sh_tlmin = m;
                d.lneref[blk] = S == 0 ? 0.0 : log(.25) - mu * m;
            }
            __syncthreads();
            for (int e = tid; e < 2 * T; e += blockDim.x)
                inv_tab[e] = -expm1(-mu * (tl_tab[e] - sh_tlmin));
            __syncthreads();
            for (int k = tid; k < S; k += blockDim.x) d.inv32[B.state0 + k] = (float)inv_tab[pair(k)];
        }
        if (S == 0 && tid == 0) {
            inv[0] = 1.0;
            if (want32) d.inv32[B.state0] = 0.0f;
        }
    }

    // state priors into forward column 0 (calc_state_priors, trans.cpp:785-831)
    if (B.b == 0) {
        for (int k = tid; k < Sm; k += blockDim.x) {
            double p;
            if (S == 0) {
                p = 1.0;
            } else {
                const int b = sinfo[k].time;
                const int ma = I.minage;
                if (b < ma) {
                    p = 0.0;
                } else {
                    double sum = 0.0;
                    for (int m = 2 * ma; m < 2 * b - 1; m++)
                        sum += csteps[m] * nb[m / 2] / (2.0 * pops[m / 2]);
                    p = exp(-sum) / nc[b];
                    if (b < T - 2) {
                        double Z = 0.0;
                        if (b > ma) Z = csteps[2 * b - 1] * nb[b - 1] / (2.0 * pops[b - 1]);
                        p *= 1.0 - exp(-csteps[2 * b] * nb[b] / (2.0 * pops[b]) - Z);
                    }
                }
            }
            if (d.fw64) d.fw64[B.cell0 + k] = p;
            if (d.fw32) d.fw32[B.cell0 + k] = (float)p;
        }
    }

    if (B.b == 0) return;

    // ---------------- switch matrix from the previous tree (trans.cpp:538-739)
    const int S1 = B.S1;
    int *determ = d.determ + B.prev_state0;
    double *determprob = d.determprob + B.prev_state0;
    double *recombrow = d.recombrow + B.state0;
    double *recoalrow = d.recoalrow + B.state0;
    int *gptr = d.gptr + B.gptr0;
    int *gidx = d.gidx + B.prev_state0;
    for (int v = tid; v < n; v += blockDim.x)
        for (int y = 0; y < pcnt[v]; y++) {
            s1node[pfirst[v] + y] = v;
            s1time[pfirst[v] + y] = pt0[v] + y;
        }
    for (int k = tid; k < Sm; k += blockDim.x) {
        recombrow[k] = 0.0;
        recoalrow[k] = 0.0;
    }
    if (tid == 0) {
        sh_src[0] = -1;
        sh_src[1] = -1;
        const double lt = internal ? treelen_of(prv, n, B.prev_root, times, true)
                                   : treelen_of(prv, n, B.prev_root, times, false);
        sh_treelen = lt;
    }
    __syncthreads();

    SwitchCtx c;
    c.last = prv; c.cur = cur; c.last_root = B.prev_root; c.cur_root = root; c.T = T;
    c.mapping = d.mapping + B.map0;
    c.times = times; c.tsteps = tsteps; c.csteps = csteps; c.pops = pops;
    c.nb = pnb; c.nr = pnr; c.nc = pnc; c.rho = rho; c.last_treelen = sh_treelen;
    c.internal = internal;
    const int *spr = B.spr;
    const int *mapping = c.mapping;

    bool special = false;
    if (internal) {
        if (S1 == 0) {
            special = true;
            if (tid == 0) {
                determprob[0] = 1.0;
                if (S == 0) {
                    determ[0] = 0;
                } else {
                    const int mainr = cur[root].z;
                    int j = lookup(first, t0, cnt, mainr, spr[3]);
                    determ[0] = j;
                    if (j < 0) report_error(d.err, ERR_SWITCH_NO_TARGET, B.inst, B.b, B.start);
                }
            }
        } else if (S == 0) {
            special = true;
            for (int i = tid; i < S1; i += blockDim.x) {
                determ[i] = 0;
                int rpa;
                if (s1node[i] == spr[0] && s1time[i] > spr[1]) rpa = s1time[i];
                else rpa = prv[prv[spr[0]].x].w;
                determprob[i] = calc_recomb_recoal(c, spr, s1node[i], s1time[i], rpa);
            }
        }
    }

    if (!special) {
        // get_deterministic_transitions (trans.cpp:156-275)
        for (int i = tid; i < S1; i += blockDim.x) {
            const int node1 = s1node[i], time1 = s1time[i];
            int next;
            if ((node1 == spr[2] && time1 == spr[3]) || (node1 == spr[0] && time1 == spr[1])) {
                next = -1;
            } else if (node1 != spr[0]) {
                int node2;
                bool disrupt = false;
                if (prv[node1].y == -1) {
                    node2 = node1;
                } else {
                    const int child1 = prv[node1].y, child2 = prv[node1].z;
                    if (spr[0] == child1) { node2 = mapping[child2]; disrupt = true; }
                    else if (spr[0] == child2) { node2 = mapping[child1]; disrupt = true; }
                    else node2 = mapping[node1];
                }
                const int mcoal = mapping[spr[2]];
                if ((spr[2] == node1 && spr[3] < time1) || (mcoal == node2 && spr[3] < time1) ||
                    (disrupt && mcoal == node2 && spr[3] <= time1))
                    node2 = cur[node2].x;
                next = -2;
                if (internal && cur[node2].w > time1) next = -1;
                if (next == -2) {
                    const int p = cur[node2].x;
                    if (p != -1 && internal && time1 > cur[p].w) next = -1;
                }
                if (next == -2) next = lookup(first, t0, cnt, node2, time1);
            } else {
                if (spr[1] > time1) {
                    next = lookup(first, t0, cnt, mapping[spr[0]], time1);
                } else {
                    const int parent = prv[spr[0]].x;
                    const int time2 = prv[parent].w;
                    const int other = (prv[parent].z == spr[0] ? prv[parent].y : prv[parent].z);
                    const int node2 = (other == spr[2] ? cur[mapping[other]].x : mapping[other]);
                    next = lookup(first, t0, cnt, node2, time2);
                }
            }
            determ[i] = next;
        }
        // recoalescence sums (calc_recoal_sums, trans.cpp:417-440)
        const int rpa0 = prv[prv[spr[0]].x].w;
        if (tid == 0) {
            const int k = spr[1], j = spr[3];
            double sum = 0.0;
            for (int m = 2 * k; m < 2 * j - 1; m++) {
                int nbm = pnb[m / 2] - int(m / 2 < rpa0);
                sum += csteps[m] * nbm / (2.0 * pops[m / 2]);
            }
            sh_sums = sum;
            sum = 0.0;
            sums2[2 * k] = sum;
            for (int m = 2 * k; m < 2 * j - 1; m++) {
                sum += csteps[m] / (2.0 * pops[m / 2]);
                sums2[m + 1] = sum;
            }
        }
        for (int a = tid; a < T; a += blockDim.x) recoals[a] = calc_recoal(c, spr, a, rpa0, false);
        __syncthreads();
        auto dprob = [&](int node, int a) {
            if (node == spr[0] && a > spr[1]) return calc_recomb_recoal(c, spr, node, a, a);
            const int idx = max(min(2 * spr[3] - 1, 2 * a), 2 * spr[1]);
            return calc_recomb(c, spr, node, a, c.last_treelen) * exp(-sh_sums - sums2[idx]) *
                   recoals[a];
        };
        if (!internal) {
            // external trees: the value depends on the source state only through its time
            // and whether its node is the root (calc_recomb) or the recombining node above
            // the recombination (calc_recomb_recoal); one evaluation per case. Node -1
            // stands for any other node (the external calc_recomb only compares it with the
            // root; the recombining node is never the root).
            for (int e = tid; e < 3 * (T - 1); e += blockDim.x) {
                const int f = e / (T - 1), a = e % (T - 1);
                const int node = f == 0 ? -1 : f == 1 ? B.prev_root : spr[0];
                dp_tab[f * MAXT + a] = dprob(node, a);
            }
            __syncthreads();
            for (int i = tid; i < S1; i += blockDim.x) {
                if (determ[i] < 0) continue;
                const int node = s1node[i], a = s1time[i];
                const int f = (node == spr[0] && a > spr[1]) ? 2 : node == B.prev_root ? 1 : 0;
                determprob[i] = dp_tab[f * MAXT + a];
            }
        } else {
            for (int i = tid; i < S1; i += blockDim.x) {
                if (determ[i] < 0) continue;
                determprob[i] = dprob(s1node[i], s1time[i]);
            }
        }
        // probabilistic sources (each state at most once: states are distinct)
        for (int i = tid; i < S1; i += blockDim.x) {
            if (s1node[i] == spr[0] && s1time[i] == spr[1]) sh_src[0] = i;
            else if (s1node[i] == spr[2] && s1time[i] == spr[3]) sh_src[1] = i;
        }
        __syncthreads();
        if (tid == 0) {
            const int recombsrc = sh_src[0];
            if (recombsrc != -1) {  // get_recomb_transition_switch (trans.cpp:278-313)
                const int parent = prv[spr[0]].x;
                const int time2 = prv[parent].w;
                const int other = sibling(prv, spr[0]);
                const int node2 = (other == spr[2] ? cur[mapping[other]].x : mapping[other]);
                const int next0 = lookup(first, t0, cnt, mapping[spr[0]], spr[1]);
                const int next1 = lookup(first, t0, cnt, node2, time2);
                if (next0 != -1)
                    recombrow[next0] = calc_recomb_recoal(c, spr, s1node[recombsrc],
                                                          s1time[recombsrc], rpa0);
                if (next1 != -1)
                    recombrow[next1] = calc_recomb_recoal(c, spr, s1node[recombsrc],
                                                          s1time[recombsrc], s1time[recombsrc]);
            }
        }
        __syncthreads();
        const int recoalsrc = sh_src[1];
        if (recoalsrc != -1) {
            const int node1 = s1node[recoalsrc], time1 = s1time[recoalsrc];
            const int last_parent = prv[spr[0]].x;
            int node3;
            if (last_parent == node1)
                node3 = mapping[prv[last_parent].z == spr[0] ? prv[last_parent].y : prv[last_parent].z];
            else
                node3 = mapping[node1];
            const int parent = cur[mapping[spr[0]]].x;
            for (int j = tid; j < S; j += blockDim.x) {
                const int node2 = sinfo[j].node, time2 = sinfo[j].time;
                if (!((node2 == mapping[spr[0]] && time2 >= spr[1]) ||
                      (node2 == node3 && time2 == time1) || (node2 == parent && time2 == time1)))
                    continue;
                int spr2[4] = {spr[0], spr[1], spr[2], time2};
                recoalrow[j] = calc_recomb_recoal(c, spr2, node1, time1, rpa0);
            }
        }
    }
    __syncthreads();

    // gather lists: sources of every target, ascending (sample_thread.cpp:357-362), by a
    // counting sort: counts (integer atomics), a scan, then warp 0 places 32 sources at a
    // time, each after the earlier sources of its target in the same batch of 32
    {
        const int n1 = imax(S1, 1);
        const int rs = sh_src[0], cs = sh_src[1];
        if (tid == 0) d.srcs[blk] = make_int2(rs, cs);
        for (int k = tid; k <= Sm; k += blockDim.x) gcnt[k] = 0;
        __syncthreads();
        for (int j = tid; j < n1; j += blockDim.x) {
            const int k = determ[j];
            if (j != rs && j != cs && k >= 0) atomicAdd(&gcnt[k + 1], 1);
        }
        __syncthreads();
        if (tid < 32) {
            const int lane = tid;
            const int per = (Sm + 1 + 31) / 32;
            const int lo = imin(lane * per, Sm + 1), hi = imin(lo + per, Sm + 1);
            int run = 0;
            for (int i = lo; i < hi; i++) {
                run += gcnt[i];
                gcnt[i] = run;
            }
            int incl = run;
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            for (int i = lo; i < hi; i++) {
                gcnt[i] += incl - run;  // gcnt[k]: first slot of target k
                gptr[i] = gcnt[i];
            }
            __syncwarp();
            for (int jb = 0; jb < n1; jb += 32) {
                const int j = jb + lane;
                const int k = j < n1 ? determ[j] : -1;
                const bool ok = j < n1 && j != rs && j != cs && k >= 0;
                const unsigned peers = __match_any_sync(0xffffffffu, ok ? k : -1 - lane);
                if (ok) gidx[gcnt[k] + __popc(peers & ((1u << lane) - 1))] = j;
                __syncwarp();
                if (ok && lane == 31 - __clz(peers)) gcnt[k] += __popc(peers);
                __syncwarp();
            }
        }
    }
    if (want32) {
        __syncthreads();
        for (int j = tid; j < imax(S1, 1); j += blockDim.x)
            d.determprob32[B.prev_state0 + j] = (float)determprob[j];
        for (int k = tid; k < Sm; k += blockDim.x) {
            d.recombrow32[B.state0 + k] = (float)recombrow[k];
            d.recoalrow32[B.state0 + k] = (float)recoalrow[k];
        }
    }
}

// ---------------------------------------------------------------------------------------
// K2: emissions of variant columns (calc_emissions' non-invariant branch, emit.cpp:822-844)
//
// One CTA per local tree. The per-state branch factors (prob_branch of the three split
// branches, emit.cpp:787-805) are computed once per tree in FP64; each warp then takes
// every nwarps-th variant column of the tree: lane 0 runs the inner (postorder) and outer
// (preorder) partial likelihoods, the warp evaluates calc_emit for all states. F is the
// arithmetic type of the partials and emissions (FP64 plain path / FP32 chosen path).

template <typename F>
__global__ void k_varemit(BatchDev d, int nwarps, int maxS) {
    extern __shared__ int4 dyn[];
    const int blk = cta_block(d);
    const BlockDev B = d.blocks[blk];
    if (B.nvar == 0 || B.S == 0) return;
    const InstDev I = d.inst[B.inst];
    const int T = I.T, n = I.nnodes;
    const bool internal = I.internal != 0;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int S = B.S;

    auto align16 = [](void *p) {
        return (char *)(((uintptr_t)p + 15) & ~(uintptr_t)15);
    };
    int4 *nd = dyn;
    F *muts = (F *)align16(nd + n);
    F *nomuts = muts + n;
    F *pm = (F *)align16(nomuts + n);            // [S][6]: mut0..2, nomut0..2 per state
    int *order = (int *)align16(pm + (size_t)6 * maxS);
    int *visit = order + n;
    int *snode = visit + n;                      // [maxS]
    F *scratch = (F *)align16(snode + maxS);     // per warp: inner[n][4], outer[n][4]
    int *stacks = (int *)align16(scratch + (size_t)nwarps * n * 8);
    __shared__ double times[MAXT];

    const double *model = d.model + I.model0;
    for (int i = tid; i < T; i += blockDim.x) times[i] = model[M_TIMES + i];
    const double mu = model[M_CONST + 1], mintime = model[M_CONST + 2];
    for (int i = tid; i < n; i += blockDim.x) nd[i] = d.nodes[B.nodes0 + i];
    __syncthreads();
    const int root = B.root;
    for (int i = tid; i < n; i += blockDim.x) {  // prob_tree_mutation (emit.cpp:97-116)
        double m1 = 0.0, m0 = 0.0;
        if (i != root) {
            const int pa = nd[nd[i].x].w;
            if (pa != T + 1) {
                const double t = fmax(times[pa] - times[nd[i].w], mintime);
                m1 = prob_branch(t, mu, true);
                m0 = prob_branch(t, mu, false);
            }
        }
        muts[i] = (F)m1;
        nomuts[i] = (F)m0;
    }
    const int mainr = internal ? nd[root].z : root;
    const int node1 = internal ? nd[root].y : 0;
    const double time1 = internal ? times[nd[node1].w] : 0.0;
    const StateInfo *sinfo = d.sinfo + B.state0;
    for (int k = tid; k < S; k += blockDim.x) {  // per-state split branches (emit.cpp:782-805)
        const int node2 = sinfo[k].node;
        snode[k] = node2;
        const int parent = nd[node2].x;
        const double time2 = times[nd[node2].w];
        const double parent_time = (parent != -1) ? times[min(nd[parent].w, T - 1)] : 0.0;
        const double coal_time = times[sinfo[k].time];
        double dist[3];
        dist[0] = fmax(coal_time - time1, mintime);
        dist[1] = fmax(coal_time - time2, mintime);
        dist[2] = fmax(parent_time - coal_time, mintime);
        for (int x = 0; x < 3; x++) {
            pm[6 * k + x] = (F)prob_branch(dist[x], mu, true);
            pm[6 * k + 3 + x] = (F)prob_branch(dist[x], mu, false);
        }
    }
    if (tid == 0) {  // postorder (local_tree.h:274-304)
        int i;
        for (i = 0; i < n; i++) visit[i] = 0;
        for (i = 0; i < n; i++) {
            if (nd[i].y != -1) break;
            order[i] = i;
        }
        int end = i;
        for (i = 0; i < n; i++) {
            const int p = nd[order[i]].x;
            if (p != -1) {
                visit[p]++;
                if (visit[p] == 2) order[end++] = p;
            }
        }
    }
    __syncthreads();

    F (*in)[4] = (F (*)[4])(scratch + (size_t)warp * n * 8);
    F (*out)[4] = in + n;
    int *stack = stacks + warp * n;
    const uint8_t *cls = d.colclass + I.col0 + B.start;
    const int ns = I.nseqs;
    F *vout = (sizeof(F) == 4) ? (F *)d.var32 : (F *)d.varemit;

    // the block's variant columns in order; warp w takes every nwarps-th
    int seen = 0;
    for (int base = 0; base < B.len; base += 32) {
        const int i = base + lane;
        const bool isvar = i < B.len && cls[i] == COL_VARIANT;
        unsigned mm = __ballot_sync(0xffffffffu, isvar);
        while (mm) {
            const int bit = __ffs(mm) - 1;
            mm &= mm - 1;
            const int vslot = seen++;
            if (vslot % nwarps != warp) continue;
            const uint8_t *chars = d.seqT + I.seq0 + (size_t)(B.start + base + bit) * ns;
            if (lane == 0) {
                for (int oi = 0; oi < n; oi++) {  // likelihood_site_node_inner (emit.cpp:151-196)
                    const int j = order[oi];
                    if (nd[j].y == -1) {
                        const uint8_t ch = chars[j];
                        if (ch == 'N') { in[j][0] = in[j][1] = in[j][2] = in[j][3] = F(1); }
                        else {
                            in[j][0] = in[j][1] = in[j][2] = in[j][3] = F(0);
                            const int x = (ch == 'A' || ch == 'a') ? 0 : (ch == 'C' || ch == 'c') ? 1
                                        : (ch == 'G' || ch == 'g') ? 2 : 3;
                            in[j][x] = F(1);
                        }
                    } else {
                        const int c1 = nd[j].y, c2 = nd[j].z;
                        for (int a = 0; a < 4; a++) {
                            F p1 = 0, p2 = 0;
                            for (int b = 0; b < 4; b++) {
                                if (a == b) { p1 += in[c1][b] * nomuts[c1]; p2 += in[c2][b] * nomuts[c2]; }
                                else { p1 += in[c1][b] * muts[c1]; p2 += in[c2][b] * muts[c2]; }
                            }
                            in[j][a] = p1 * p2;
                        }
                    }
                }
                int sp = 0;  // likelihood_site_outer (emit.cpp:273-296), preorder
                stack[sp++] = mainr;
                while (sp > 0) {
                    const int j = stack[--sp];
                    if (j == mainr) {
                        out[j][0] = out[j][1] = out[j][2] = out[j][3] = F(1);
                    } else {
                        const int p = nd[j].x;
                        const int sib = nd[p].y == j ? nd[p].z : nd[p].y;
                        if (p != mainr) {
                            for (int a = 0; a < 4; a++) {
                                F p1 = 0, p2 = 0;
                                for (int b = 0; b < 4; b++) {
                                    if (a == b) { p1 += in[sib][b] * nomuts[sib]; p2 += out[p][b] * nomuts[p]; }
                                    else { p1 += in[sib][b] * muts[sib]; p2 += out[p][b] * muts[p]; }
                                }
                                out[j][a] = p1 * p2;
                            }
                        } else {
                            for (int a = 0; a < 4; a++) {
                                F p1 = 0;
                                for (int b = 0; b < 4; b++) {
                                    if (a == b) p1 += in[sib][b] * nomuts[sib];
                                    else p1 += in[sib][b] * muts[sib];
                                }
                                out[j][a] = p1;
                            }
                        }
                    }
                    if (nd[j].y != -1) { stack[sp++] = nd[j].y; stack[sp++] = nd[j].z; }
                }
            }
            __syncwarp();
            // leaf partial of the threaded sequence (external) or the subtree root (internal)
            F in2[4];
            if (internal) {
                for (int a = 0; a < 4; a++) in2[a] = in[node1][a];
            } else {
                const uint8_t ch = chars[I.nleaves];
                if (ch == 'N') { in2[0] = in2[1] = in2[2] = in2[3] = F(1); }
                else {
                    in2[0] = in2[1] = in2[2] = in2[3] = F(0);
                    const int x = (ch == 'A' || ch == 'a') ? 0 : (ch == 'C' || ch == 'c') ? 1
                                : (ch == 'G' || ch == 'g') ? 2 : 3;
                    in2[x] = F(1);
                }
            }
            F *row = vout + B.var0 + (size_t)d.colvar[I.col0 + B.start + base + bit] * S;
            for (int k = lane; k < S; k += 32) {
                const int node2 = snode[k];
                const F *q = pm + 6 * k;
                F e = 0;  // calc_emit (emit.cpp:620-645)
                for (int a = 0; a < 4; a++) {
                    F p1 = 0, p2 = 0, p3 = 0;
                    for (int b = 0; b < 4; b++) {
                        if (a == b) {
                            p1 += in2[b] * q[3]; p2 += in[node2][b] * q[4]; p3 += out[node2][b] * q[5];
                        } else {
                            p1 += in2[b] * q[0]; p2 += in[node2][b] * q[1]; p3 += out[node2][b] * q[2];
                        }
                    }
                    if (node2 != mainr) e += p1 * p2 * p3 * F(.25);
                    else e += p1 * p2 * F(.25);
                }
                row[k] = e;
            }
            __syncwarp();
        }
    }
}

size_t tables_smem(int n, int S, int S1) {
    size_t b = 2 * (size_t)n * sizeof(int4) + 8 * (size_t)n * sizeof(int);
    b += ((n + 15) & ~15);
    b += 2 * (size_t)imax(S1, 1) * sizeof(int);
    b += (size_t)(imax(imax(S, 1), MAXT) + 2) * sizeof(int);
    return b;
}

}  // namespace

void launch_tables(const BatchDev &d, bool want32, cudaStream_t s) {
    size_t smem = tables_smem(d.maxnodes, d.maxS, d.maxS);
    static size_t configured = 0;
    if (smem > configured) {  // opt in; static shared memory counts against 48 KB too
        if (cudaFuncSetAttribute(k_tables, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return;
        configured = smem;
    }
    k_tables<<<d.nblocks, TAB_THREADS, smem, s>>>(d, want32 ? 1 : 0);
    note_launch();
}

template <typename F>
void launch_varemit_t(const BatchDev &d, cudaStream_t s) {
    const int n = d.maxnodes, maxS = imax(d.maxS, 1);
    int nwarps = 4;
    auto need = [&](int w) {
        return (size_t)n * sizeof(int4) + (2 * (size_t)n + 6 * (size_t)maxS) * sizeof(F) +
               (2 * (size_t)n + maxS + 4) * sizeof(int) + (size_t)w * n * 8 * sizeof(F) +
               (size_t)w * n * sizeof(int) + 6 * 16;
    };
    while (nwarps > 1 && need(nwarps) > 200 * 1024) nwarps--;
    const size_t smem = need(nwarps);
    static size_t configured = 0;
    if (smem > configured) {  // opt in; static shared memory counts against 48 KB too
        if (cudaFuncSetAttribute(k_varemit<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return;
        configured = smem;
    }
    k_varemit<F><<<d.nblocks, nwarps * 32, smem, s>>>(d, nwarps, maxS);
    note_launch();
}

void launch_varemit(const BatchDev &d, bool fp32, cudaStream_t s) {
    if (fp32) launch_varemit_t<float>(d, s);
    else launch_varemit_t<double>(d, s);
}

}  // namespace awg

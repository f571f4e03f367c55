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

#include <type_traits>

#include <cmath>
#include <cstdio>

#include "kernels.h"
#include "tree_util.cuh"

namespace awg {

namespace {

constexpr int TAB_THREADS = 128;

struct Terms {
    double D[MAXT], E[MAXT], lnB[MAXT], lnE2[MAXT], lnNegG1[MAXT], G2[MAXT], G3[MAXT],
        lnG4[MAXT], norecombs[MAXT];
    // the exponentials get_time needs, each evaluated once per tree:
    double EB[MAXT];              // exp(lnE2[b] + lnB[b-1]), b > 0
    // T x T tables in dynamic shared memory (row length ld = T), sized by the instance's T:
    double *E2B;                  // [a][b] exp(lnE2[b] + lnB[a])
    double *E2N;                  // [a][b] exp(lnE2[b] + lnNegG1[a])
    double *CT;                   // [b][c] exp(lnG4[b] + lnB[c-1]), c > 0 (FP64 path only)
    int ld;
    // FP32 path: the exponentials factor, exp(lnE2[b] + lnB[a]) = exp(lnE2[b]) exp(lnB[a])
    // and so on, so T of each are enough; dBN[a] = exp(lnB[a]) - exp(lnNegG1[a]) formed
    // without cancellation as exp(lnB[a]) (-expm1(lnNegG1[a] - lnB[a]))
    double eE2[MAXT], eB[MAXT], eG4[MAXT], dBN[MAXT];
};

// Doubles of K1's exponential tables in dynamic shared memory (kept a multiple of two, so
// the int4 arrays after them stay 16-byte aligned).
__host__ __device__ inline int exp_table_doubles(int T, bool want32) {
    return ((want32 ? 2 : 3) * T * T + 1) & ~1;
}

// Fill the exponential tables (the same arguments get_time exponentiates), only the
// entries get_time reads: E2B/E2N[a][b] for a < b (the a < b branch), CT[b][c] for
// 1 <= c <= b (c_term and minage_term: a state's time is at least its node's age and minage).
__device__ void exp_tables(Terms &t, int T) {
    for (int e = threadIdx.x; e < (T - 1) * (T - 1); e += blockDim.x) {
        const int a = e / (T - 1), b = e % (T - 1);
        if (a < b) {
            t.E2B[a * t.ld + b] = exp(t.lnE2[b] + t.lnB[a]);
            t.E2N[a * t.ld + b] = exp(t.lnE2[b] + t.lnNegG1[a]);
        } else if (b < a) {
            t.CT[a * t.ld + b + 1] = exp(t.lnG4[a] + t.lnB[b]);  // [b=a][c=b+1]
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
    if (minage > 0) minage_term = t.CT[b * t.ld + minage];
    const double eb = t.EB[b];
    if (!same_node) {
        if (a < b) return term1 * (t.E2B[a * t.ld + b] - t.E2N[a * t.ld + b] - minage_term);
        if (a == b) return term1 * (eb + t.G3[b] - minage_term);
        return term1 * (eb + t.G2[b] - minage_term);
    }
    double c_term = (c > 0 ? t.CT[b * t.ld + c] : 0.0);
    if (a < b)
        return term1 * (2 * (t.E2B[a * t.ld + b] - t.E2N[a * t.ld + b]) - c_term - minage_term);
    if (a == b) return term1 * ((2 * (eb + t.G3[b])) - c_term - minage_term) + t.norecombs[a];
    return term1 * ((2 * (eb + t.G2[b])) - c_term - minage_term);
}

__device__ __forceinline__ double logadd(double lna, double lnb) {  // common.h:157-163
    if (lna == -INFINITY) return lnb;
    if (lnb == -INFINITY) return lna;
    return fmax(lna, lnb) + log1p(exp(-fabs(lna - lnb)));
}

// State ranges of every node of one tree (states.cpp:53-167): first state, first time,
// count, and the offset of the node's same-branch rows (node_ranges_par below).

__device__ __forceinline__ int lookup(const int *first, const int *t0, const int *cnt, int v,
                                      int t) {
    if (v < 0 || cnt[v] == 0) return -1;
    int d = t - t0[v];
    if (d < 0 || d >= cnt[v]) return -1;
    return first[v] + d;
}

// Whether v lies strictly below `top` (walks up the parents, at most n steps).
__device__ __forceinline__ bool below(const int4 *nd, int v, int top, int n) {
    int u = nd[v].x;
    for (int s = 0; u != -1 && s < n; s++, u = nd[u].x)
        if (u == top) return true;
    return false;
}

// node_ranges by the whole CTA (the same outputs): per node its state count and first time
// in parallel, then exclusive prefix sums over node order for the first state and the
// same-branch row offset (integers: exact in any order). Returns S.
__device__ int node_ranges_par(const int4 *nd, int n, int root, int T, bool internal,
                               int minage_param, int *first, int *t0, int *cnt, int *t2base) {
    __shared__ int part[TAB_THREADS], part2[TAB_THREADS];
    __shared__ int sh_tot;
    const int tid = threadIdx.x, nt = blockDim.x;
    bool none = false;
    int minage = 0, sub = -1;
    if (internal) {
        if (nd[root].w < T) {
            none = true;
        } else {
            sub = nd[root].y;
            minage = max(minage_param, nd[sub].w);
        }
    }
    for (int v = tid; v < n; v += nt) {
        int m = 0, start = nd[v].w;
        const bool ign = internal && !none && (v == root || v == sub || below(nd, v, sub, n));
        if (!none && !ign) {
            const int p = nd[v].x;
            start = internal ? max(nd[v].w, minage) : nd[v].w;
            const bool top_branch = internal ? (p == root) : (p == -1);
            const int top = top_branch ? T - 2 : nd[p].w;
            m = max(0, top - start + 1);
        }
        t0[v] = start;
        cnt[v] = m;
    }
    __syncthreads();
    const int c = (n + nt - 1) / nt;
    const int lo = min(tid * c, n), hi = min(lo + c, n);
    int s1 = 0, s2 = 0;
    for (int v = lo; v < hi; v++) {
        s1 += cnt[v];
        s2 += cnt[v] * cnt[v];
    }
    part[tid] = s1;
    part2[tid] = s2;
    __syncthreads();
    if (tid == 0) {
        int a = 0, b = 0;
        for (int t = 0; t < nt; t++) {
            const int x = part[t], y = part2[t];
            part[t] = a;
            part2[t] = b;
            a += x;
            b += y;
        }
        sh_tot = a;
    }
    __syncthreads();
    int a = part[tid], b = part2[tid];
    for (int v = lo; v < hi; v++) {
        first[v] = a;
        if (t2base) t2base[v] = b;
        a += cnt[v];
        b += cnt[v] * cnt[v];
    }
    const int S = sh_tot;
    __syncthreads();
    return S;
}

// Sum of one double per thread in a fixed order (warp trees, then the warps in order);
// every thread gets the total.
__device__ double block_sum(double v) {
    __shared__ double red[TAB_THREADS / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w];
    __syncthreads();
    return s;
}

// Lineage counts of one tree (count_lineages[_internal], local_tree.cpp:34-131) by the
// whole CTA: each node adds its branch to the time slices it spans (integer shared-memory
// atomics: exact in any order), then the per-slice corrections. Ends with a barrier.
__device__ void lineage_counts_par(const int4 *nd, int n, int root, int T, bool internal,
                                   int *nb, int *nr, int *nc) {
    const int tid = threadIdx.x;
    for (int t = tid; t < T; t += blockDim.x) nb[t] = nr[t] = nc[t] = 0;
    __syncthreads();
    const int sub = internal ? nd[root].y : -1;
    for (int i = tid; i < n; i += blockDim.x) {
        if (internal && (i == sub || i == root)) continue;
        const int p = nd[i].x;
        const bool top_branch = internal ? (p == root) : (p == -1);
        const int pa = top_branch ? T - 2 : nd[p].w;
        for (int t = max(nd[i].w, 0); t < pa && t < T; t++) {
            atomicAdd(&nb[t], 1);
            atomicAdd(&nr[t], 1);
            atomicAdd(&nc[t], 1);
        }
        if (pa >= 0 && pa < T) {
            atomicAdd(&nr[pa], 1);
            atomicAdd(&nc[pa], 1);
            if (top_branch) atomicAdd(&nb[pa], 1);
        }
    }
    __syncthreads();
    for (int t = tid; t < T; t += blockDim.x) {
        if (internal && t < nd[sub].w) { nb[t]--; nc[t]--; nr[t]--; }
        if (t == T - 1) nb[t] = 1;
    }
    __syncthreads();
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
    // q[m][1 + d] = csteps[m] * (nb[m / 2] + d) / (2.0 * pops[m / 2]) for d in {-1, 0, 1}:
    // every coalescence-rate term of the switch formulas, the reference's expression with
    // the lineage count it uses, evaluated once per tree
    const double (*q)[3];
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
            if (over) Z = c.csteps[2 * j - 1] * 1 / (2.0 * c.pops[j - 1]);
            else Z = c.q[2 * j - 1][1 - int(j - 1 < recomb_parent_age) + int(j - 1 < a)];
        }
        // -(x * n) / y is -(x * n / y) exactly
        const double r = over ? c.csteps[2 * j] * nbranches_j / (2.0 * c.pops[j])
                              : c.q[2 * j][1 - int(j < recomb_parent_age) + int(j < a)];
        p *= 1.0 - exp(-r - Z);
    }
    return p;
}

// calc_recomb_recoal (trans.cpp:505-534)
__device__ double calc_recomb_recoal(const SwitchCtx &c, const int *spr, int state_node,
                                     int state_time, int recomb_parent_age) {
    const int a = state_time, k = spr[1], j = spr[3];
    double p = calc_recomb(c, spr, state_node, state_time, c.last_treelen);
    double sum = 0.0;
    for (int m = 2 * k; m < 2 * j - 1; m++)  // nb[m / 2] - [m / 2 < rpa] + [m / 2 < a]
        sum += c.q[m][1 - int(m / 2 < recomb_parent_age) + int(m / 2 < a)];
    p *= exp(-sum);
    p *= calc_recoal(c, spr, state_time, recomb_parent_age, c.internal);
    return p;
}



// ---------------------------------------------------------------------------------------
// K1

// The tables of one local tree, by the whole CTA (TAB_THREADS threads).
__device__ __forceinline__ void tables_tree(const BatchDev &d, int blk, int want32) {
    extern __shared__ int4 dyn[];
    BlockDev &Bg = d.blocks[blk];
    const BlockDev B = Bg;
    const InstDev I = d.inst[B.inst];
    const int T = I.T, n = I.nnodes;
    const bool internal = I.internal != 0;
    const int tid = threadIdx.x;

    double *dtab = (double *)dyn;  // the T x T exponential tables, then the tree arrays
    int4 *cur = (int4 *)(dtab + exp_table_doubles(T, want32 != 0));
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

    if (tid == 0) {
        tr.ld = T;
        tr.E2B = dtab;
        tr.E2N = dtab + T * T;
        tr.CT = want32 ? nullptr : dtab + 2 * T * T;
    }
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
    {
        const int S0 = node_ranges_par(cur, n, root, T, internal, I.minage, first, t0, cnt, t2base);
        const int S10 = B.b > 0 ? node_ranges_par(prv, n, B.prev_root, T, internal, I.minage,
                                                  pfirst, pt0, pcnt, nullptr)
                                : 0;
        if (tid == 0) {
            sh_S = S0;
            sh_S1 = S10;
            // TransMatrix::minage: max(StatesModel::minage, subtree age) when internal
            sh_minage = internal ? max(I.minage, cur[cur[root].y].w) : 0;
        }
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
    lineage_counts_par(cur, n, root, T, internal, nb, nr, nc);
    if (B.b > 0) lineage_counts_par(prv, n, B.prev_root, T, internal, pnb, pnr, pnc);

    // transition terms (calc_transition_probs, trans.cpp:26-115)
    for (int i = tid; i < 2 * T; i += blockDim.x)
        coal_rates_alloc[1 + i] = csteps[i] * nb[i / 2] / (2.0 * pops[i / 2]);
    double tl_par = 0.0;
    if (want32) {
        // FP32 path: the tree length summed by the CTA (the FP64 path keeps node order)
        double part = 0.0;
        for (int i = tid; i < n; i += blockDim.x) {
            const int p = cur[i].x;
            if (p == -1 || (internal && p == root)) continue;
            part += times[cur[p].w] - times[cur[i].w];
        }
        tl_par = block_sum(part);
    }
    __syncthreads();
    if (tid == 0) {
        double *coal_rates = &coal_rates_alloc[1];
        coal_rates[-1] = 0.0;
        double *C = &C_alloc[2];
        C[-2] = 0.0;
        C[-1] = 0.0;
        for (int b = 0; b < 2 * T - 1; b++) C[b] = C[b - 1] + coal_rates[b];
        double treelen;
        int root_age_index;
        if (internal) {
            const int sub = cur[root].y, mainr = cur[root].z;
            root_age_index = cur[mainr].w;
            treelen = (want32 ? tl_par : treelen_of(cur, n, root, times, true)) - times[cur[sub].w];
        } else {
            root_age_index = cur[root].w;
            treelen = want32 ? tl_par : treelen_of(cur, n, root, times, false);
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
        // one (term, time) pair per thread, each term's expression as the reference writes
        // it (lnE2 and lnG4 are the same expression, trans.cpp:80-86); D and norecombs on
        // separate threads
        for (int e = tid; e < 6 * (T - 1); e += blockDim.x) {
            const int f = e / (T - 1), b = e % (T - 1);
            if (f == 0) {
                lnBterm[b] = C[2 * b - 1] + log(tsteps[b] * (nb[b] + 1.0) / (nr[b] + 1.0));
                tr.E[b] = 1.0 / nc[b];
            } else if (f == 1) {
                const double v = -C[2 * b - 2] +
                    (b < T - 2 ? log(1 - exp(-coal_rates[2 * b] - coal_rates[2 * b - 1])) : 0.0);
                tr.lnE2[b] = v;
                tr.lnG4[b] = v;
            } else if (f == 2) {
                tr.lnNegG1[b] = C[2 * b - 1] + log(-tsteps[b] *
                    ((nb[b] / (nr[b] + 1.0 + int(b < root_age_index))) - (nb[b] + 1.0) / (nr[b] + 1.0)));
            } else if (f == 3) {
                const double g = b < T - 2 ? 1.0 - exp(-coal_rates[2 * b]) : 1.0;
                tr.G2[b] = g * tsteps[b] * (nb[b] + 1.0) / (nr[b] + 1.0);
                tr.G3[b] = g * tsteps[b] * (nb[b] / (nr[b] + 1.0 + int(b < root_age_index)));
            } else {
                double treelen2 = sh_treelen + times[b];
                double treelen2_b;
                if (b > root_age_index) {
                    treelen2 += times[b] - root_age;
                    treelen2_b = treelen2 + tsteps[b];
                } else {
                    treelen2_b = treelen2 + tsteps[root_age_index];
                }
                if (f == 4) {
                    tr.D[b] = (1.0 - exp(-rho * treelen2)) / treelen2_b;
                } else {
                    tr.norecombs[b] = exp(-fmax(rho * treelen2, rho));
                    if (want32)
                        d.rstay32[(size_t)blk * MAXT + b] = (float)(-expm1(-fmax(rho * treelen2, rho)));
                }
            }
        }
    }
    __syncthreads();
    if (!want32) {
        if (tid == 0) {
            tr.lnB[0] = lnBterm[0];
            for (int b = 1; b < T - 1; b++) tr.lnB[b] = logadd(tr.lnB[b - 1], lnBterm[b]);
            tr.E[T - 2] = 1.0 / nc[T - 2];
        }
    } else {
        // FP32 path: the log-sum-exp prefix lnB[b] = log(sum_{i <= b} exp(lnBterm[i])) as T
        // exponentials shifted by the largest term, one prefix sum and T logarithms, by one
        // warp (the reference adds one term at a time with logadd)
        if (tid < 32) {
            const int b = tid;
            const double x = b < T - 1 ? lnBterm[b] : -INFINITY;
            double mx = x;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            double w = b < T - 1 ? exp(x - mx) : 0.0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const double y = __shfl_up_sync(0xffffffffu, w, o);
                if (b >= o) w += y;
            }
            if (b < T - 1) tr.lnB[b] = mx + log(w);
            if (b == 0) tr.E[T - 2] = 1.0 / nc[T - 2];
        }
    }
    __syncthreads();
    if (!want32) {
        exp_tables(tr, T);
        __syncthreads();
        // tmatrix[a][b] = get_time(a, b, 0, minage, false) (sample_thread.cpp:212-216)
        double *tm = d.tm + (size_t)blk * MAXT * MAXT;
        for (int e = tid; e < (T - 1) * (T - 1); e += blockDim.x) {
            const int a = e / (T - 1), b = e % (T - 1);
            tm[a * MAXT + b] = get_time(tr, a, b, 0, minage, false);
        }
    } else {
        // FP32 path: 4 (T-1) exponentials instead of 1.5 (T-1)^2; tmatrix = D[a] E[b] (X[a][b]
        // - minage_term[b]), X the different-node bracket (get_time, trans.h:101-109), kept
        // with D[a] E[b] for the same-branch rows below
        for (int e = tid; e < 4 * (T - 1); e += blockDim.x) {  // one exponential per thread
            const int f = e / (T - 1), i = e % (T - 1);
            if (f == 0) tr.eE2[i] = exp(tr.lnE2[i]);
            else if (f == 1) tr.eB[i] = exp(tr.lnB[i]);
            else if (f == 2) tr.eG4[i] = exp(tr.lnG4[i]);
            else tr.dBN[i] = exp(tr.lnB[i]) * -expm1(tr.lnNegG1[i] - tr.lnB[i]);
        }
        __syncthreads();
        float *tm32 = d.tm32 + (size_t)blk * MAXT * MAXT;
        for (int e = tid; e < (T - 1) * (T - 1); e += blockDim.x) {
            const int a = e / (T - 1), b = e % (T - 1);
            const double eb = b > 0 ? tr.eE2[b] * tr.eB[b - 1] : 0.0;
            const double x = a < b ? tr.eE2[b] * tr.dBN[a] : eb + (a == b ? tr.G3[b] : tr.G2[b]);
            const double de = __dmul_rn(tr.D[a], tr.E[b]);
            const double mt = minage > 0 ? tr.eG4[b] * tr.eB[minage - 1] : 0.0;
            tr.E2B[a * T + b] = x;
            tr.E2N[a * T + b] = de;
            tm32[a * MAXT + b] = (a < minage || b < minage) ? 0.0f : (float)(de * (x - mt));
        }
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
        // (X the different-node bracket without its minage term; both in E2B / E2N above);
        // formed from that product it keeps its relative accuracy where the two get_time
        // values nearly cancel.
        float *t2d = d.t2d32 + B.t2_0;
        for (int k = tid; k < S; k += blockDim.x) {
            const StateInfo si = sinfo[k];
            const int b = si.time, c = cur[si.node].w;
            const int base = t2off[k];
            const double ct = c > 0 ? tr.eG4[b] * tr.eB[c - 1] : 0.0;
            for (int y = 0; y < si.m; y++) {
                const int a = t0[si.node] + y;
                t2d[base + y * si.m] =
                    (a < minage || b < minage) ? 0.0f
                                               : (float)(tr.E2N[a * T + b] * (tr.E2B[a * T + b] - ct));
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
    if (want32) {
        // FP32 path: the main tree's and the subtree's lengths (branches floored at mintime)
        // summed by the CTA; the FP64 path keeps the reference's walk order
        const int mainr = internal ? cur[root].z : root;
        const int sub = internal ? cur[root].y : root;
        double pm = 0.0, ps = 0.0;
        for (int v = tid; v < n; v += blockDim.x) {
            const int p = cur[v].x;
            const double w = fmax(p != -1 ? times[cur[p].w] - times[cur[v].w] : 0.0, mintime);
            // every node of an external tree is below its root
            if (v != mainr && (!internal || below(cur, v, mainr, n))) pm += w;
            if (internal && v != sub && below(cur, v, sub, n)) ps += w;
        }
        const double mt = block_sum(pm);
        const double st = internal ? block_sum(ps) : 0.0;
        if (tid == 0) {
            sh_maintreelen = mt;
            sh_subtreelen = st;
        }
    } else if (tid == 0) {
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
    // the switch's coalescence-rate terms, each once per tree (SwitchCtx::q), and the same
    // without the lineage count
    __shared__ double qrate[2 * MAXT][3], rrate[2 * MAXT];
    for (int e = tid; e < 6 * T; e += blockDim.x) {
        const int m = e / 3, dl = e % 3 - 1;
        qrate[m][dl + 1] = csteps[m] * (pnb[m / 2] + dl) / (2.0 * pops[m / 2]);
    }
    for (int m = tid; m < 2 * T; m += blockDim.x) rrate[m] = csteps[m] / (2.0 * pops[m / 2]);
    // the previous tree's length: FP64 path in node order (local_tree.cpp:136-176), FP32
    // path summed by the CTA
    double lt_part = 0.0;
    if (want32)
        for (int i = tid; i < n; i += blockDim.x) {
            const int p = prv[i].x;
            if (p == -1 || (internal && p == B.prev_root)) continue;
            lt_part += times[prv[p].w] - times[prv[i].w];
        }
    const double lt32 = want32 ? block_sum(lt_part) : 0.0;
    if (tid == 0) {
        sh_src[0] = -1;
        sh_src[1] = -1;
        sh_treelen = want32 ? lt32 : treelen_of(prv, n, B.prev_root, times, internal);
    }
    __syncthreads();

    SwitchCtx c;
    c.last = prv; c.cur = cur; c.last_root = B.prev_root; c.cur_root = root; c.T = T;
    c.mapping = d.mapping + B.map0;
    c.times = times; c.tsteps = tsteps; c.csteps = csteps; c.pops = pops;
    c.nb = pnb; c.nr = pnr; c.nc = pnc; c.q = qrate; c.rho = rho; c.last_treelen = sh_treelen;
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
            for (int m = 2 * k; m < 2 * j - 1; m++) sum += qrate[m][1 - int(m / 2 < rpa0)];
            sh_sums = sum;
            sum = 0.0;
            sums2[2 * k] = sum;
            for (int m = 2 * k; m < 2 * j - 1; m++) {
                sum += rrate[m];
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
        if (tid == 0 || tid == 32) {  // the two entries on two warps
            const int recombsrc = sh_src[0];
            if (recombsrc != -1) {  // get_recomb_transition_switch (trans.cpp:278-313)
                const int parent = prv[spr[0]].x;
                const int time2 = prv[parent].w;
                const int other = sibling(prv, spr[0]);
                const int node2 = (other == spr[2] ? cur[mapping[other]].x : mapping[other]);
                const int next0 = lookup(first, t0, cnt, mapping[spr[0]], spr[1]);
                const int next1 = lookup(first, t0, cnt, node2, time2);
                // where both entries are one state the reference's second write wins
                if (tid == 0 && next0 != -1 && next0 != next1)
                    recombrow[next0] = calc_recomb_recoal(c, spr, s1node[recombsrc],
                                                          s1time[recombsrc], rpa0);
                if (tid == 32 && next1 != -1)
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

__global__ void __launch_bounds__(TAB_THREADS) k_tables(BatchDev d, int want32) {
    tables_tree(d, cta_block(d), want32);
}

// Work queue of a persistent per-tree kernel: units of `chunk` consecutive trees in the
// batch's tree order (largest instances first), taken by CTAs with an atomic counter.
struct WorkQueue {
    int *counter;
    int nunits, chunk;
};

// Takes the next unit for the whole CTA; -1 when the queue is empty.
__device__ __forceinline__ int next_unit(const WorkQueue &q) {
    __shared__ int unit;
    __syncthreads();  // the previous unit's reads of `unit` are done
    if (threadIdx.x == 0) unit = atomicAdd(q.counter, 1);
    __syncthreads();
    const int u = unit;
    return u < q.nunits ? u : -1;
}

// K1 as a persistent kernel: as many CTAs as fit on the GPU at once, each taking units of
// trees until the queue is empty (work-stealing over (instance, tree-chunk) units).
__global__ void __launch_bounds__(TAB_THREADS) k_tables_ws(BatchDev d, int want32, WorkQueue q) {
    for (int u = next_unit(q); u >= 0; u = next_unit(q)) {
        const int t1 = imin((u + 1) * q.chunk, d.nblocks);
        for (int t = u * q.chunk; t < t1; t++) {
            tables_tree(d, d.blkmap ? d.blkmap[t] : t, want32);
            __syncthreads();
        }
    }
}

// ---------------------------------------------------------------------------------------
// K2: emissions of variant columns (calc_emissions' non-invariant branch, emit.cpp:822-844)
//
// One CTA per local tree. Once per tree: the branch mutation probabilities, the per-state
// factors of the three split branches (prob_branch, emit.cpp:787-805, FP64), and two level
// schedules of the tree: nodes by height (children before parents) for the inner partials
// and nodes below the main root by depth for the outer ones. Each warp then takes every
// nwarps-th variant column of the tree: its lanes compute one level of inner partials
// (likelihood_site_node_inner, emit.cpp:151-196), then one level of outer partials
// (likelihood_site_outer, emit.cpp:273-296) at a time, and calc_emit (emit.cpp:620-645) for
// the states.
//
// Plain path (FP64): the reference's order of operations, emissions written as they are.
// FP32 path: a column whose observed calls agree except for missing ones has emissions that
// agree to a few digits, which FP32 values would lose. The partials are therefore carried
// relative to the column's first observed base X: component 0 holds 1 - P(.. | X), the
// others P(.. | Y) for the bases after X, and the JC69 step P x = mut * sum(x) +
// (nomut - mut) * x is written for that form (1 - nomut = 3 mut). Each state's emission
// comes out as D_k = 1 - 4 e_k, exact to FP32 relative precision even when tiny. Per column
// the kernel writes log(e_ref) of the largest emission and, per state, either the
// complement 1 - e_k / e_ref when it is at most 1/2, or -e_k / e_ref: the forward and
// backward steps apply x - x * c or x * r, both without cancellation.

// FP32 path: leaf partial relative to base X (component 0: 1 - P(X), then X+1, X+2, X+3)
template <typename R>
__device__ __forceinline__ void leaf_partial_x(uint8_t ch, int X, R *v) {
    if (ch == 'N') { v[0] = R(0); v[1] = v[2] = v[3] = R(1); return; }
    const int b = (ch == 'A' || ch == 'a') ? 0 : (ch == 'C' || ch == 'c') ? 1
                : (ch == 'G' || ch == 'g') ? 2 : 3;
    v[0] = v[1] = v[2] = v[3] = R(0);
    if (b != X) {
        v[0] = R(1);
        v[(b - X) & 3] = R(1);
    }
}
// JC69 step in that form: off-diagonal m, diagonal 1 - 3m
template <typename R>
__device__ __forceinline__ void jc_apply_x(const R *x, R m, R nm, R *y) {
    const R s3 = (x[1] + x[2]) + x[3];
    const R u = R(1) - x[0];
    y[0] = fma(nm, x[0], fma(-m, s3, R(3) * m));
#pragma unroll
    for (int a = 1; a < 4; a++) y[a] = fma(m, (u + s3) - x[a], nm * x[a]);
}
// complement of a product: 1 - (1 - a)(1 - b)
template <typename R>
__device__ __forceinline__ R cprod(R a, R b) { return (a + b) - a * b; }

// Double-float: value = hi + lo, |lo| <= ulp(hi) / 2, about 48 significant bits, from
// FP32 error-free transforms (Knuth's two-sum; the product's error by fused multiply-add).
// The FP32 path's variant-column emissions are formed in it: the forward posterior amplifies
// an error of those emissions thousands-fold on the columns where they differ little between
// states, so they must reach FP32 as correctly rounded ratios to the column's largest. FP32
// forms left the posterior up to 6.6e-5 from FP64's (9.1e-5 with only the partials in
// double-float); double-float, 3.1e-6 (k = 64, 100,000 columns).
struct df {
    float hi, lo;
    __device__ __forceinline__ df() : hi(0.f), lo(0.f) {}
    __device__ __forceinline__ df(double x) : hi((float)x), lo((float)(x - (double)(float)x)) {}
    // small integer constants (0, 1, 4 in the emission forms) without the FP64 split
    __device__ __forceinline__ df(int x) : hi((float)x), lo(0.0f) {}
    __device__ __forceinline__ df(float h, float l) : hi(h), lo(l) {}
    __device__ __forceinline__ explicit operator double() const { return (double)hi + (double)lo; }
};
__device__ __forceinline__ df df_fast2(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return df(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ df operator+(df a, df b) {
    const float s = __fadd_rn(a.hi, b.hi);
    const float bb = __fsub_rn(s, a.hi);
    const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
    return df_fast2(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ df operator-(df a) { return df(-a.hi, -a.lo); }
__device__ __forceinline__ df operator-(df a, df b) { return a + (-b); }
__device__ __forceinline__ df operator*(df a, df b) {
    const float p = __fmul_rn(a.hi, b.hi);
    const float e = __fmaf_rn(a.hi, b.hi, -p);
    return df_fast2(p, __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e)));
}
__device__ __forceinline__ df &operator+=(df &a, df b) { return a = a + b; }
__device__ __forceinline__ bool operator<(df a, df b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
// a + b for a, b >= 0 (every sum of the emission passes: partials, branch probabilities and
// their products): the larger high part first makes Dekker's fast two-sum exact, three adds
// where the two-sum of arbitrary signs takes six
__device__ __forceinline__ df df_addp(df a, df b) {
    const float big = fmaxf(a.hi, b.hi), small = fminf(a.hi, b.hi);
    const float s = __fadd_rn(big, small);
    const float e = __fsub_rn(small, __fsub_rn(s, big));
    return df_fast2(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}
// a * b + c, a, b, c >= 0 (the JC69 steps of the emission passes)
__device__ __forceinline__ df fma(df a, df b, df c) { return df_addp(a * b, c); }
__device__ __forceinline__ df fmax(df a, df b) { return a < b ? b : a; }
__device__ __forceinline__ df __shfl_xor_sync(unsigned mask, df v, int o) {
    return df(::__shfl_xor_sync(mask, v.hi, o), ::__shfl_xor_sync(mask, v.lo, o));
}
// the built-in overloads stay visible beside the double-float ones
using ::fmax;
using ::fma;
using ::__shfl_xor_sync;

// Per-tree context of K2 shared by the column passes.
struct EmitCtx {
    const int4 *nd;
    const double *muts, *nomuts, *pm;  // branch and per-state split-branch probabilities
    const float *muts32, *nomuts32;    // FP32 copies (converted once per tree)
    const float *pm32;                 // [S][8]: mut0..2, nomut0..2, 1 - 4 mut0, unused
    const int *snode, *inl, *inp, *outl, *outp;
    const uint8_t *sfloor;  // per state: a split branch of it was raised to mintime
    int nlev_in, nlev_out, mainr, node1, S, ns, nleaves, n;
    bool internal;
    // The FP32 path's double-float forms (BatchDev::vardf): muts, nomuts and pm then hold
    // double-float values, 8 bytes each in the same slots, so that the steps read them with
    // no conversion (a conversion from double runs on the FP64 pipe, in every step)
    __device__ __forceinline__ df dmut(int j) const { return ((const df *)muts)[j]; }
    __device__ __forceinline__ df dnomut(int j) const { return ((const df *)nomuts)[j]; }
    __device__ __forceinline__ df dpm(size_t i) const { return ((const df *)pm)[i]; }
};

__device__ __forceinline__ int base_bit(uint8_t ch) {
    if (ch == 'N') return 0;
    return 1 << ((ch == 'A' || ch == 'a') ? 0 : (ch == 'C' || ch == 'c') ? 1
                 : (ch == 'G' || ch == 'g') ? 2 : 3);
}

// Infinite-sites validity of one variant column's nodes (get_infinite_sites_states,
// emit.cpp:454-589, with parsimony_ancestral_set :898-953) by one warp over the level
// schedules: Fitch sets by height, then refined from the main root down (any order with
// children first, then parents first, gives the reference's sets). A state on node j keeps
// the model when the threaded base (the cut subtree's set) meets the set of j or of its
// parent. Node j's flag is bit j / 32 of lane j % 32's word; all flags are 1 when the
// column cannot break the model. sets, anc: n bytes each of the warp's scratch.
__device__ unsigned infsites_nodes(const EmitCtx &c, const uint8_t *chars, uint8_t *sets,
                                   uint8_t *anc) {
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int4 *nd = c.nd;
    int all = 0, subset = 0, mainset = 0;
    for (int x = lane; x < c.inp[1]; x += 32) {
        const int j = c.inl[x];
        const int b = base_bit(chars[j]);
        sets[j] = (uint8_t)b;
        if (!c.internal) {
            all |= b;
        } else {
            int u = j;
            for (int s = 0; u != -1 && u != c.node1 && s < c.n; s++) u = nd[u].x;
            if (u == c.node1) subset |= b;
            else mainset |= b;
        }
    }
    all = __reduce_or_sync(FULL, all);
    subset = __reduce_or_sync(FULL, subset);
    mainset = __reduce_or_sync(FULL, mainset);
    __syncwarp();
    for (int h = 1; h < c.nlev_in; h++) {
        for (int x = c.inp[h] + lane; x < c.inp[h + 1]; x += 32) {
            const int j = c.inl[x];
            const int l = sets[nd[j].y], r = sets[nd[j].z];
            sets[j] = (uint8_t)((l & r) ? (l & r) : (l | r));
        }
        __syncwarp();
    }
    const int cset = c.internal ? sets[c.node1] : base_bit(chars[c.nleaves]);
    if (c.internal ? !(subset & mainset) : !(cset & all)) return FULL;
    for (int h = 0; h < c.nlev_out; h++) {
        for (int x = c.outp[h] + lane; x < c.outp[h + 1]; x += 32) {
            const int j = c.outl[x];
            if (j == c.mainr) {
                anc[j] = sets[j];
            } else {
                const int ps = anc[nd[j].x] & sets[j];
                anc[j] = (uint8_t)(ps ? ps : sets[j]);
            }
        }
        __syncwarp();
    }
    unsigned word = FULL;
    for (int w = 0; w * 32 + lane < c.n && w < 32; w++) {
        const int j = w * 32 + lane;
        int u = j;  // in the main tree (the only nodes with states)
        for (int s = 0; u != -1 && u != c.mainr && s < c.n; s++) u = nd[u].x;
        if (u != c.mainr) continue;
        const bool ok = (cset & anc[j]) || (j != c.mainr && (cset & anc[nd[j].x]));
        if (!ok) word &= ~(1u << w);
    }
    __syncwarp();
    return word;
}

// Whether state k's node keeps the infinite-sites model (all lanes call it).
__device__ __forceinline__ bool state_ok(unsigned word, int node) {
    return (__shfl_sync(0xffffffffu, word, node & 31) >> (node >> 5)) & 1;
}

// Column forms of the partials and emissions:
//   REF  FP64, the reference's order of operations (plain path)
//   F64  FP64, JC69 structure (FP32 path: internal-branch columns with two or more
//        observed bases)
//   REL  FP32 relative to base X (FP32 path, columns whose observed calls agree)
//   SNP  FP32 (FP32 path: external columns with two or more observed bases). With u, v the
//        partials either side of the attachment point and b the threaded base,
//        4 e_k = sum_a p1_a u_a v_a = W_k (m1 + (1 - 4 m1) P_k(b)), P_k(b) = u_b v_b / W_k,
//        W_k = sum_a u_a v_a. W_k is the likelihood of the tree's own calls: the same W for
//        every state, except where the reference raises a split branch to mintime (the
//        lowest and highest state of a branch), which lengthens that branch. The column
//        keeps one W (sum of the main root's inner partial); such states their own W_k / W;
//        and every state its bracket, written as 1 - bracket = 3 m1 + (1 - 4 m1)(1 - P_k(b))
//        when P_k(b) >= 1/2, else the bracket itself: sums of positive terms, so FP32 keeps
//        the small differences between states that decide the posterior.
enum { EM_REF = 0, EM_F64 = 1, EM_REL = 2, EM_SNP = 3 };

// One variant column by one warp: inner partials by height level, outer partials by
// depth, then the states' emissions (4 e_k, or D_k = 1 - 4 e_k in the relative form) into
// eb[S]. Returns, over the warp, the reference value: the largest 4 e_k, or the smallest D_k.
template <typename R, int MODE>
__device__ R emit_column(const EmitCtx &c, const uint8_t *chars, int X, R (*in)[4], R (*out)[4],
                         R *eb) {
    const int lane = threadIdx.x & 31;
    const int4 *nd = c.nd;
    auto leaf = [&](uint8_t ch, R *v) {
        if constexpr (MODE == EM_REL) leaf_partial_x<R>(ch, X, v);
        else leaf_partial<R>(ch, v);
    };
    constexpr bool F32 = std::is_same<R, float>::value;
    constexpr bool DF = std::is_same<R, df>::value;
    auto bm = [&](int j) -> R {
        if constexpr (F32) return c.muts32[j];
        else if constexpr (DF) return c.dmut(j);
        else return (R)c.muts[j];
    };
    auto bn = [&](int j) -> R {
        if constexpr (F32) return c.nomuts32[j];
        else if constexpr (DF) return c.dnomut(j);
        else return (R)c.nomuts[j];
    };
    auto step = [&](const R *x, R m, R nm, R *y) {
        const double m64 = (double)m, nm64 = (double)nm;
        if constexpr (MODE == EM_REL) {
            jc_apply_x<R>(x, m, nm, y);
        } else if constexpr (MODE == EM_F64 || MODE == EM_SNP) {
            const R sum = (x[0] + x[1]) + (x[2] + x[3]);
#pragma unroll
            for (int a = 0; a < 4; a++) y[a] = fma(nm - m, x[a], m * sum);
        } else {
            jc_apply<false>((const double *)x, m64, nm64, (double *)y);
        }
    };
    auto mul = [&](const R *a, const R *b, R *z) {
        z[0] = MODE == EM_REL ? cprod<R>(a[0], b[0]) : a[0] * b[0];
#pragma unroll
        for (int t = 1; t < 4; t++) z[t] = a[t] * b[t];
    };
    // inner partials, one height level at a time (level 0: the leaves)
    for (int x = lane; x < c.inp[1]; x += 32) leaf(chars[c.inl[x]], in[c.inl[x]]);
    __syncwarp();
    for (int h = 1; h < c.nlev_in; h++) {
        for (int x = c.inp[h] + lane; x < c.inp[h + 1]; x += 32) {
            const int j = c.inl[x];
            const int c1 = nd[j].y, c2 = nd[j].z;
            R p1[4], p2[4];
            step(in[c1], bm(c1), bn(c1), p1);
            step(in[c2], bm(c2), bn(c2), p2);
            mul(p1, p2, in[j]);
        }
        __syncwarp();
    }
    // outer partials from the main root down, one depth level at a time
    for (int h = 0; h < c.nlev_out; h++) {
        for (int x = c.outp[h] + lane; x < c.outp[h + 1]; x += 32) {
            const int j = c.outl[x];
            if (j == c.mainr) {
                out[j][0] = MODE == EM_REL ? R(0) : R(1);
                out[j][1] = out[j][2] = out[j][3] = R(1);
                continue;
            }
            const int p = nd[j].x;
            const int sib = nd[p].y == j ? nd[p].z : nd[p].y;
            R p1[4];
            step(in[sib], bm(sib), bn(sib), p1);
            if (p != c.mainr) {
                R p2[4];
                step(out[p], bm(p), bn(p), p2);
                mul(p1, p2, out[j]);
            } else {
#pragma unroll
                for (int a = 0; a < 4; a++) out[j][a] = p1[a];
            }
        }
        __syncwarp();
    }
    // leaf partial of the threaded sequence (external) or the subtree root (internal)
    R in2[4];
    if (c.internal) {
        for (int a = 0; a < 4; a++) in2[a] = in[c.node1][a];
    } else {
        leaf(chars[c.nleaves], in2);
    }
    R ref = MODE == EM_REL || MODE == EM_SNP ? R(4) : R(0);
    R vmax = R(0);  // SNP: the largest bracket among states in the plain form
    R wcol = R(1);  // SNP: the column's W, sum over the main root's inner partial
    if constexpr (MODE == EM_SNP) {
        const R *im = in[c.mainr];
        wcol = (im[0] + im[1]) + (im[2] + im[3]);
    }
    // SNP: the threaded base (external trees), 4 for a missing call
    const uint8_t chb = MODE == EM_SNP ? chars[c.nleaves] : 'N';
    const int bnew = chb == 'N' ? 4 : (chb == 'A' || chb == 'a') ? 0 : (chb == 'C' || chb == 'c') ? 1
                   : (chb == 'G' || chb == 'g') ? 2 : 3;
    for (int k = lane; k < c.S; k += 32) {
        const int node2 = c.snode[k];
        R q[7];
        if constexpr (F32) {
            const float4 qa = *(const float4 *)(c.pm32 + 8 * k);
            const float4 qb = *(const float4 *)(c.pm32 + 8 * k + 4);
            q[0] = qa.x; q[1] = qa.y; q[2] = qa.z; q[3] = qa.w; q[4] = qb.x; q[5] = qb.y; q[6] = qb.z;
        } else {
            for (int t = 0; t < 6; t++) {
                if constexpr (DF) q[t] = c.dpm(6 * (size_t)k + t);
                else q[t] = (R)c.pm[6 * k + t];
            }
            q[6] = R(1) - R(4) * q[0];
        }
        R p1[4], p2[4], p3[4];
        if constexpr (MODE != EM_SNP) step(in2, q[0], q[3], p1);
        step(in[node2], q[1], q[4], p2);
        if (node2 != c.mainr) step(out[node2], q[2], q[5], p3);
        else p3[0] = p3[1] = p3[2] = p3[3] = R(1);
        R v;  // calc_emit (emit.cpp:620-645)
        if constexpr (MODE == EM_SNP) {
            // 4 e_k / (4 e of a state with W and bracket 1), as D = 1 - value (>= 0) or,
            // stored negated, the value itself
            R w = 0, rest = 0;
#pragma unroll
            for (int a = 0; a < 4; a++) {
                const R t = p2[a] * p3[a];
                w += t;
                if (a != bnew) rest += t;
            }
            // omega = W_k / W - 1: 0 unless a split branch was raised to mintime (states on
            // the main root's branch always have W_k = W: the JC69 rows sum to one)
            const R omega = (c.sfloor[k] && node2 != c.mainr) ? (w - wcol) / wcol : R(0);
            if (bnew == 4) {
                v = -(R(1) + omega);  // missing threaded call: bracket 1
                vmax = fmax(vmax, -v);
            } else {
                const R m1 = q[0], a41 = q[6];
                const R pb = (p2[bnew] * p3[bnew]) / w;
                if (pb >= R(0.5)) {
                    const R dd = fma(a41, rest / w, R(3) * m1);  // 1 - bracket
                    v = dd - omega * (R(1) - dd);                // 1 - (1 + omega) bracket
                    if (v >= R(0)) ref = fmin(ref, v);
                    else { v = -(R(1) - v); vmax = fmax(vmax, -v); }
                } else {
                    v = -((R(1) + omega) * fma(a41, pb, m1));
                    vmax = fmax(vmax, -v);
                }
            }
        } else if constexpr (MODE == EM_REL) {
            if (node2 != c.mainr) {
                v = cprod<R>(p1[0], cprod<R>(p2[0], p3[0]));
#pragma unroll
                for (int a = 1; a < 4; a++) v -= p1[a] * p2[a] * p3[a];
            } else {
                v = cprod<R>(p1[0], p2[0]);
#pragma unroll
                for (int a = 1; a < 4; a++) v -= p1[a] * p2[a];
            }
            ref = fmin(ref, v);
        } else if constexpr (MODE == EM_F64) {
            v = 0;
#pragma unroll
            for (int a = 0; a < 4; a++) v += node2 != c.mainr ? p1[a] * p2[a] * p3[a] : p1[a] * p2[a];
            ref = fmax(ref, v);
        } else {
            v = 0;
#pragma unroll
            for (int a = 0; a < 4; a++) {
                if (node2 != c.mainr) v += p1[a] * p2[a] * p3[a] * R(.25);
                else v += p1[a] * p2[a] * R(.25);
            }
        }
        eb[k] = v;
    }
    if constexpr (MODE == EM_SNP) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            ref = fmin(ref, __shfl_xor_sync(0xffffffffu, ref, o));
            vmax = fmax(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
        }
        // the largest bracket: 1 - min D, or the largest plain one (returned negated)
        if (ref != R(4) && R(1) - ref >= vmax) return ref;
        return -vmax;
    }
    if constexpr (MODE == EM_REL) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) ref = fmin(ref, __shfl_xor_sync(0xffffffffu, ref, o));
    } else if constexpr (MODE == EM_F64) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) ref = fmax(ref, __shfl_xor_sync(0xffffffffu, ref, o));
    }
    __syncwarp();
    return ref;
}

// A column whose observed calls all show one base X (it varies only through missing calls),
// in double-float by one warp: 4 e_k into eb[S], returns the largest. Every partial is then
// symmetric in the other three bases (the leaves' are (1, 0) or, missing, (1, 1); JC69 treats
// the three alike), so it is kept as the pair (x_X, x_other): half the work of the four-base
// form, the same sums. The FP32 path's columns of this kind (about 26% of all columns at
// 0.5% missing calls, 87% of the variant ones) are where the forward posterior amplifies an
// emission error most: their emissions differ little between states.
__device__ df emit_near_df(const EmitCtx &c, const uint8_t *chars, int X, df (*in)[2],
                           df (*out)[2], df *eb) {
    const int lane = threadIdx.x & 31;
    const int4 *nd = c.nd;
    // JC69 over a branch with m (to each other base), nm (no change)
    auto step = [](const df *x, df m, df nm, df *y) {
        const df dd = nm - m, ms = m * df_addp(x[0], df(3.0f, 0.0f) * x[1]);
        y[0] = df_addp(dd * x[0], ms);
        y[1] = df_addp(dd * x[1], ms);
    };
    auto leaf = [](uint8_t ch, df *v) {  // observed calls are X here
        v[0] = df(1.0f, 0.0f);
        v[1] = ch == 'N' ? df(1.0f, 0.0f) : df();
    };
    (void)X;
    for (int x = lane; x < c.inp[1]; x += 32) leaf(chars[c.inl[x]], in[c.inl[x]]);
    __syncwarp();
    for (int h = 1; h < c.nlev_in; h++) {
        for (int x = c.inp[h] + lane; x < c.inp[h + 1]; x += 32) {
            const int j = c.inl[x];
            const int c1 = nd[j].y, c2 = nd[j].z;
            df p1[2], p2[2];
            step(in[c1], c.dmut(c1), c.dnomut(c1), p1);
            step(in[c2], c.dmut(c2), c.dnomut(c2), p2);
            in[j][0] = p1[0] * p2[0];
            in[j][1] = p1[1] * p2[1];
        }
        __syncwarp();
    }
    for (int h = 0; h < c.nlev_out; h++) {
        for (int x = c.outp[h] + lane; x < c.outp[h + 1]; x += 32) {
            const int j = c.outl[x];
            if (j == c.mainr) {
                out[j][0] = out[j][1] = df(1.0f, 0.0f);
                continue;
            }
            const int p = nd[j].x;
            const int sib = nd[p].y == j ? nd[p].z : nd[p].y;
            df p1[2];
            step(in[sib], c.dmut(sib), c.dnomut(sib), p1);
            if (p != c.mainr) {
                df p2[2];
                step(out[p], c.dmut(p), c.dnomut(p), p2);
                out[j][0] = p1[0] * p2[0];
                out[j][1] = p1[1] * p2[1];
            } else {
                out[j][0] = p1[0];
                out[j][1] = p1[1];
            }
        }
        __syncwarp();
    }
    df in2[2];
    if (c.internal) {
        in2[0] = in[c.node1][0];
        in2[1] = in[c.node1][1];
    } else {
        leaf(chars[c.nleaves], in2);
    }
    auto state_v = [&](int k) -> df {
        const int node2 = c.snode[k];
        const size_t q = 6 * (size_t)k;  // mut0..2, nomut0..2
        df p1[2], p2[2], t[2];
        step(in2, c.dpm(q), c.dpm(q + 3), p1);
        step(in[node2], c.dpm(q + 1), c.dpm(q + 4), p2);
        if (node2 != c.mainr) {
            df p3[2];
            step(out[node2], c.dpm(q + 2), c.dpm(q + 5), p3);
            t[0] = p2[0] * p3[0];
            t[1] = p2[1] * p3[1];
        } else {
            t[0] = p2[0];
            t[1] = p2[1];
        }
        return df_addp(p1[0] * t[0], df(3.0f, 0.0f) * (p1[1] * t[1]));
    };
    // two states per lane at a time: independent chains the scheduler can interleave (the
    // second one repeats the last state where it would run past S)
    df ref = df();
    for (int k0 = lane; k0 < c.S; k0 += 64) {
        const int k1 = k0 + 32 < c.S ? k0 + 32 : k0;
        const df v0 = state_v(k0), v1 = state_v(k1);
        eb[k0] = v0;
        eb[k1] = v1;
        ref = fmax(ref, fmax(v0, v1));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ref = fmax(ref, __shfl_xor_sync(0xffffffffu, ref, o));
    __syncwarp();
    return ref;
}

// FP32 path: a tree's share of the log-likelihood's emission references, lneref per
// invariant column and log(vref) per variant column (the instance's column 0, the prior, has
// none), summed by one warp in a fixed order. The logarithms are taken here, a lane per
// column, not by one lane per column in the emission passes: there an FP64 log holds the
// warp's FP64 pipe for a few thousand cycles per column.
__device__ void block_log_offset(const BatchDev &d, const BlockDev &B, const InstDev &I, int blk,
                                 int lane) {
    const uint8_t *cls = d.colclass + I.col0 + B.start;
    const int *cvar = d.colvar + I.col0 + B.start;
    const double lner = d.lneref[blk];
    double s = 0.0;
    if (B.S > 0) {
        for (int i = lane; i < B.len; i += 32) {
            if (B.b == 0 && i == 0) continue;
            const uint8_t c = cls[i];
            if (c == COL_INVARIANT) s += lner;
            else if (c == COL_VARIANT) s += log(d.vref[B.vrow0 + cvar[i]]);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) d.blkext[blk] = s;
}

// Variant-column emissions of one local tree, by the whole CTA (nwarps warps).
// The branch exponentials of one instance: every branch length K2 forms is a difference
// of two time points (or of a time point and 0) floored at mintime, so the exponentials
// are tabulated once per instance, not once per state: e[i][j] for max(times[j] -
// times[i], mintime), e0[j] for max(times[j] - 0, mintime), ez[j] for max(0 - times[j],
// mintime). A persistent CTA keeps the table of the instance it last served.
struct BranchCache {
    int inst;
    double e[MAXT][MAXT], e0[MAXT], ez[MAXT];
};

template <bool FP32OUT>
__device__ __forceinline__ void varemit_tree(const BatchDev &d, int blk, int nwarps, int maxS,
                                             int smem_bytes, BranchCache *bc) {
    extern __shared__ int4 dyn[];
    const BlockDev B = d.blocks[blk];
    if (B.nvar == 0 || B.S == 0) {
        if (FP32OUT && threadIdx.x < 32) block_log_offset(d, B, d.inst[B.inst], blk, threadIdx.x);
        return;
    }
    const InstDev I = d.inst[B.inst];
    const int T = I.T, n = I.nnodes;
    const bool internal = I.internal != 0;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int S = B.S;
    if (S > maxS || n > d.maxnodes || n < 1) {
        if (tid == 0) report_error(d.err, ERR_PLAN_MISMATCH, B.inst, B.b, B.start);
        return;
    }

    auto align16 = [](void *p) {
        return (char *)(((uintptr_t)p + 15) & ~(uintptr_t)15);
    };
    // lean: an FP32 batch with no internal-branch or infinite-sites problem needs no FP64
    // emission partials, so neither the FP64 per-state factors nor FP64-sized scratch
    const bool lean = FP32OUT && !d.emit64;
    int4 *nd = dyn;
    double *muts = (double *)align16(nd + n);
    double *nomuts = muts + n;
    double *pm = lean ? nullptr : (double *)align16(nomuts + n);  // [S][6]: mut0..2, nomut0..2
    int *order = (int *)align16(lean ? (void *)(nomuts + n) : (void *)(pm + (size_t)6 * maxS));
    int *hgt = order + n;                        // height, then depth scratch
    int *snode = hgt + n;                        // [maxS]
    int *inl = snode + maxS;                     // nodes by height
    int *inp = inl + n;                          // [n + 2] level starts
    int *outl = inp + n + 2;                     // nodes below the main root by depth
    int *outp = outl + n;                        // [n + 2]
    uint8_t *sfloor = (uint8_t *)(outp + n + 2);  // [maxS]
    float *muts32 = (float *)align16(sfloor + maxS);     // FP32 path copies
    float *nomuts32 = muts32 + n;
    float *pm32 = (float *)align16(nomuts32 + n);        // [maxS][8]
    // per warp: inner[n][4], outer[n][4] partials, then the column's emissions (float-sized
    // when lean)
    const int esz = lean ? 4 : 8;
    double *scratch = (double *)align16(pm32 + (size_t)8 * maxS);
    char *ebuf = (char *)scratch + (size_t)nwarps * n * 8 * esz;
    __shared__ double times[MAXT];
    __shared__ int nlev_in, nlev_out;
    if (ebuf + (size_t)nwarps * maxS * esz - (char *)dyn > smem_bytes) {
        if (tid == 0) report_error(d.err, ERR_SMEM_LIMIT, B.inst, B.b, B.start);
        return;
    }
    // tree and state indices the passes use as addresses
    {
        bool bad = false;
        for (int i = tid; i < n; i += blockDim.x) {
            const int4 v = d.nodes[B.nodes0 + i];
            if (v.x < -1 || v.x >= n || v.y < -1 || v.y >= n || v.z < -1 || v.z >= n ||
                v.w < 0 || v.w > T + 1)
                bad = true;
        }
        for (int k = tid; k < S; k += blockDim.x) {
            const StateInfo si = d.sinfo[B.state0 + k];
            if (si.node < 0 || si.node >= n || si.time < 0 || si.time >= T) bad = true;
        }
        if (B.root < 0 || B.root >= n) bad = true;
        if (__syncthreads_or(bad)) {
            if (tid == 0) report_error(d.err, ERR_BOUNDS, B.inst, B.b, B.start);
            return;
        }
    }

    const double *model = d.model + I.model0;
    for (int i = tid; i < T; i += blockDim.x) times[i] = model[M_TIMES + i];
    const double mu = model[M_CONST + 1], mintime = model[M_CONST + 2];
    const double penalty = model[M_CONST + 3];  // infinite-sites penalty, 1: off
    if (lean && (internal || penalty < 1.0)) {  // the batch flag says otherwise
        if (tid == 0) report_error(d.err, ERR_PLAN_MISMATCH, B.inst, B.b, B.start);
        return;
    }
    for (int i = tid; i < n; i += blockDim.x) nd[i] = d.nodes[B.nodes0 + i];
    // FP32 path with double-float variant columns: every variant column takes that form
    // (penalised ones too), so the split-branch factors are stored as double-float and no
    // FP32 form's copies are made
    const bool f32forms = FP32OUT && !d.vardf;
    const bool dfpm = FP32OUT && d.vardf;
    const bool refill = bc->inst != B.inst;  // read by all before anyone rewrites it
    __syncthreads();
    if (refill) {
        for (int e = tid; e < T * T; e += blockDim.x) {
            const int i = e / T, j = e % T;
            bc->e[i][j] = branch_exp(fmax(times[j] - times[i], mintime), mu);
        }
        for (int j = tid; j < T; j += blockDim.x) {
            bc->e0[j] = branch_exp(fmax(times[j] - 0.0, mintime), mu);
            bc->ez[j] = branch_exp(fmax(0.0 - times[j], mintime), mu);
        }
        if (tid == 0) bc->inst = B.inst;
        __syncthreads();
    }
    const int root = B.root;
    for (int i = tid; i < n; i += blockDim.x) {  // prob_tree_mutation (emit.cpp:97-116)
        double m1 = 0.0, m0 = 0.0;
        if (i != root) {
            const int pa = nd[nd[i].x].w, ag = nd[i].w;
            if (pa != T + 1) {
                const double e = (pa < T && ag < T)
                                     ? bc->e[ag][pa]
                                     : branch_exp(fmax(times[pa] - times[ag], mintime), mu);
                m1 = branch_mut(e);
                m0 = branch_nomut(e);
            }
        }
        if (dfpm) {
            ((df *)muts)[i] = df(m1);
            ((df *)nomuts)[i] = df(m0);
        } else {
            muts[i] = m1;
            nomuts[i] = m0;
        }
        if (f32forms) {
            muts32[i] = (float)m1;
            nomuts32[i] = (float)m0;
        }
    }
    const int mainr = internal ? nd[root].z : root;
    const int node1 = internal ? nd[root].y : 0;
    const int age1 = nd[node1].w;
    const double time1 = internal ? times[age1] : 0.0;
    const StateInfo *sinfo = d.sinfo + B.state0;
    for (int k = tid; k < S; k += blockDim.x) {  // per-state split branches (emit.cpp:782-805)
        const int node2 = sinfo[k].node, a = sinfo[k].time;
        snode[k] = node2;
        const int parent = nd[node2].x, age2 = nd[node2].w;
        const int pidx = parent != -1 ? min(nd[parent].w, T - 1) : -1;
        const double time2 = times[age2];
        const double parent_time = (parent != -1) ? times[pidx] : 0.0;
        const double coal_time = times[a];
        sfloor[k] = (coal_time - time2 < mintime) || (parent_time - coal_time < mintime);
        // the three branch exponentials, each the table entry of the same difference
        double e[3];
        e[0] = !internal ? bc->e0[a]
             : age1 < T  ? bc->e[age1][a]
                         : branch_exp(fmax(coal_time - time1, mintime), mu);
        e[1] = age2 < T ? bc->e[age2][a] : branch_exp(fmax(coal_time - time2, mintime), mu);
        e[2] = parent != -1 ? bc->e[a][pidx] : bc->ez[a];
        if (dfpm) {  // branch_mut / branch_nomut in double-float: one FP64 split each
            const df quarter(0.25f, 0.0f), one(1.0f, 0.0f), three(3.0f, 0.0f);
            for (int x = 0; x < 3; x++) {
                const df ex(e[x]);
                ((df *)pm)[6 * k + x] = quarter * (one - ex);
                ((df *)pm)[6 * k + 3 + x] = quarter * (one + three * ex);
            }
        } else if (!lean) {
            for (int x = 0; x < 3; x++) {
                pm[6 * k + x] = branch_mut(e[x]);
                pm[6 * k + 3 + x] = branch_nomut(e[x]);
            }
        }
        if (f32forms) {
            for (int x = 0; x < 3; x++) {
                pm32[8 * k + x] = (float)branch_mut(e[x]);
                pm32[8 * k + 3 + x] = (float)branch_nomut(e[x]);
            }
            pm32[8 * k + 6] = (float)(1.0 - 4.0 * branch_mut(e[0]));
            pm32[8 * k + 7] = 0.f;
        }
    }
    // level schedules: heights (longest path down to a leaf; leaves 0), then the depth below
    // the main root (-1 outside its subtree), each bucketed by one warp. Walks are bounded
    // by n steps.
    for (int i = tid; i < n; i += blockDim.x) hgt[i] = 0;
    __syncthreads();
    for (int i = tid; i < n; i += blockDim.x) {
        if (nd[i].y != -1) continue;
        int v = i;
        for (int dd = 1; dd <= n && nd[v].x != -1; dd++) {
            v = nd[v].x;
            atomicMax(&hgt[v], dd);
        }
    }
    __syncthreads();
    if (warp == 0) {
        const int nl = warp_levels(hgt, n, inl, inp, order, lane);
        if (lane == 0) nlev_in = nl;
    }
    __syncthreads();
    for (int i = tid; i < n; i += blockDim.x) {
        int v = i, dd = 0;
        while (v != mainr && v != -1 && dd <= n) {
            v = nd[v].x;
            dd++;
        }
        hgt[i] = v == mainr ? dd : -1;
    }
    __syncthreads();
    if (warp == 0) {
        const int nl = warp_levels(hgt, n, outl, outp, order, lane);
        if (lane == 0) nlev_out = nl;
    }
    __syncthreads();

    const EmitCtx ctx{nd,      muts,     nomuts,   pm,   muts32,  nomuts32, pm32, snode,
                      inl,     inp,      outl,     outp, sfloor,  nlev_in,  nlev_out,
                      mainr,   node1,    S,        I.nseqs, I.nleaves, n,   internal};
    double *wscr = (double *)((char *)scratch + (size_t)warp * n * 8 * esz);
    double *eb = (double *)(ebuf + (size_t)warp * maxS * esz);  // read as float when lean
    const uint8_t *cls = d.colclass + I.col0 + B.start;
    const int ns = I.nseqs;

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
            const int vrow = d.colvar[I.col0 + B.start + base + bit];
            if (vrow < 0 || vrow >= B.nvar) {
                if (lane == 0) report_error(d.err, ERR_BOUNDS, B.inst, B.b, B.start + base + bit);
                continue;
            }
            // infinite-sites model (calc_emissions, emit.cpp:847-862): states whose node
            // breaks it have their emission multiplied by the penalty
            unsigned vword = 0xffffffffu;
            bool penalised = false;
            if (penalty < 1.0) {
                vword = infsites_nodes(ctx, chars, (uint8_t *)wscr, (uint8_t *)wscr + n);
                bool bad = false;
                for (int kb = 0; kb < S; kb += 32) {
                    const int k = kb + lane;
                    bad |= !state_ok(vword, k < S ? snode[k] : 0) && k < S;
                }
                penalised = __any_sync(0xffffffffu, bad);
                __syncwarp();
            }
            auto penalise = [&](double *e) {  // e[k] *= penalty where state k breaks it
                for (int kb = 0; kb < S; kb += 32) {
                    const int k = kb + lane;
                    const bool ok = state_ok(vword, k < S ? snode[k] : 0);
                    if (k < S && !ok) e[k] *= penalty;
                }
                __syncwarp();
            };
            if constexpr (!FP32OUT) {
                emit_column<double, EM_REF>(ctx, chars, 0, (double (*)[4])wscr,
                                            (double (*)[4])wscr + n, eb);
                if (penalised) penalise(eb);
                double *row = d.varemit + B.var0 + (size_t)vrow * S;
                for (int k = lane; k < S; k += 32) row[k] = eb[k];
            } else if (penalised && !d.vardf) {
                // FP64 emissions, penalised, then relative to the column's largest
                const int X0 = 0;
                emit_column<double, EM_F64>(ctx, chars, X0, (double (*)[4])wscr,
                                            (double (*)[4])wscr + n, eb);
                penalise(eb);
                double eref = 0.0;
                for (int k = lane; k < S; k += 32) eref = fmax(eref, eb[k]);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) eref = fmax(eref, __shfl_xor_sync(0xffffffffu, eref, o));
                float *row = d.var32 + B.var0 + (size_t)vrow * S;
                const double inv1 = 1.0 / eref;  // 1 / (4 e_ref)
                for (int k = lane; k < S; k += 32) {
                    const double r = eb[k] * inv1;  // e_k / e_ref
                    float v = (float)(r >= 0.5 ? 1.0 - r : -r);
                    // a ratio below FP32's range (a penalised state) stays a ratio: -0
                    // would read as the complement 0, i.e. the largest emission
                    if (r < 0.5 && v == 0.0f) v = -__int_as_float(1);
                    row[k] = v;
                }
                if (lane == 0) d.vref[B.vrow0 + vrow] = .25 * eref;
            } else {
                // X = the column's first observed base; near = every observed call (the
                // threaded sequence's too) is X
                int jfirst = ns;
                for (int j = lane; j < ns; j += 32)
                    if (chars[j] != 'N') { jfirst = j; break; }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) jfirst = min(jfirst, __shfl_xor_sync(0xffffffffu, jfirst, o));
                int X = 0;
                bool near = false;
                if (jfirst < ns) {
                    const uint8_t ch = chars[jfirst];
                    X = (ch == 'A' || ch == 'a') ? 0 : (ch == 'C' || ch == 'c') ? 1
                      : (ch == 'G' || ch == 'g') ? 2 : 3;
                    bool other = false;
                    for (int j = lane; j < ns; j += 32) {
                        const uint8_t c = chars[j];
                        if (c != 'N' && (c & 0xDF) != (ch & 0xDF)) other = true;
                    }
                    near = !__any_sync(0xffffffffu, other);
                }
                float *row = d.var32 + B.var0 + (size_t)vrow * S;
                if (near && !d.vardf) {
                    float *fs = (float *)wscr, *fe = (float *)eb;
                    const float dref = emit_column<float, EM_REL>(ctx, chars, X, (float (*)[4])fs,
                                                                  (float (*)[4])fs + n, fe);
                    const float inv1 = 1.f / (1.f - dref);  // 1 / (4 e_ref)
                    for (int k = lane; k < S; k += 32) {
                        const float c = (fe[k] - dref) * inv1;  // 1 - e_k / e_ref
                        row[k] = c <= 0.5f ? c : -((1.f - fe[k]) * inv1);
                    }
                    if (lane == 0) d.vref[B.vrow0 + vrow] = .25 * (1.0 - (double)dref);
                } else if (d.vardf) {
                    // the forward posterior amplifies an error of a variant column's
                    // emissions thousands-fold where they differ little between states (the
                    // columns that vary only through missing calls): the partials and every
                    // state's split-branch steps are formed in double-float and each ratio
                    // to the column's largest is rounded once
                    // (FP64 arithmetic only once per column: per state it would hold the
                    // FP64 pipe, 64 cycles a warp instruction)
                    df *ed = (df *)eb;
                    df eref =
                        near ? emit_near_df(ctx, chars, X, (df (*)[2])wscr, (df (*)[2])wscr + n, ed)
                             : emit_column<df, EM_F64>(ctx, chars, 0, (df (*)[4])wscr,
                                                       (df (*)[4])wscr + n, ed);
                    if (penalised) {
                        // states that break the infinite-sites model times the penalty
                        // (emit.cpp:847-862); below FP32's range that leaves the ratio 0,
                        // written as the smallest negative value below, as the FP64 form
                        // writes it
                        const df pen(penalty);
                        df mx;
                        for (int kb = 0; kb < S; kb += 32) {
                            const int k = kb + lane;
                            const bool ok = state_ok(vword, k < S ? snode[k] : 0);
                            if (k < S) {
                                if (!ok) ed[k] = ed[k] * pen;
                                mx = fmax(mx, ed[k]);
                            }
                        }
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
                        eref = mx;
                        __syncwarp();
                    }
                    // 1 / (4 e_ref): the FP32 reciprocal and one Newton step in double-float
                    const df one(1.0f, 0.0f);
                    const df y0(1.0f / eref.hi, 0.0f);
                    const df inv1 = y0 + y0 * (one - eref * y0);
                    for (int k = lane; k < S; k += 32) {
                        // e_k / e_ref; the largest state's r can round a hair above 1, so its
                        // complement is clamped at +0 (a negative value would read as a
                        // ratio, i.e. an emission near zero)
                        const df r = ed[k] * inv1;
                        float v = r.hi >= 0.5f ? fmaxf((one - r).hi, 0.0f) : -r.hi;
                        if (r.hi < 0.5f && v == 0.0f) v = -__int_as_float(1);  // stays a ratio
                        row[k] = v;
                    }
                    if (lane == 0) d.vref[B.vrow0 + vrow] = .25 * (double)eref;
                } else if (!internal) {
                    // brackets against the column's largest: D form x / plain form y
                    float *fs = (float *)wscr, *fe = (float *)eb;
                    const float ref = emit_column<float, EM_SNP>(ctx, chars, X, (float (*)[4])fs,
                                                                 (float (*)[4])fs + n, fe);
                    const float bref = ref >= 0.f ? 1.f - ref : -ref;  // the largest bracket
                    const float inv1 = 1.f / bref;
                    for (int k = lane; k < S; k += 32) {
                        const float v = fe[k];
                        if (v >= 0.f && ref >= 0.f) {
                            const float cc = (v - ref) * inv1;  // 1 - e_k / e_ref
                            row[k] = cc <= 0.5f ? cc : -((1.f - v) * inv1);
                        } else {
                            const float r = (v >= 0.f ? 1.f - v : -v) * inv1;  // e_k / e_ref
                            row[k] = r >= 0.5f ? 1.f - r : -r;
                        }
                    }
                    if (lane == 0) {
                        // W: the tree's own likelihood, sum over the main root's inner partial
                        const float *im = fs + 4 * mainr;
                        const double w = (double)((im[0] + im[1]) + (im[2] + im[3]));
                        d.vref[B.vrow0 + vrow] = .25 * w * (double)bref;
                    }
                } else {
                    const double eref = emit_column<double, EM_F64>(ctx, chars, X, (double (*)[4])wscr,
                                                                    (double (*)[4])wscr + n, eb);
                    const double inv1 = 1.0 / eref;  // 1 / (4 e_ref)
                    for (int k = lane; k < S; k += 32) {
                        const double r = eb[k] * inv1;  // e_k / e_ref
                        row[k] = (float)(r >= 0.5 ? 1.0 - r : -r);
                    }
                    if (lane == 0) d.vref[B.vrow0 + vrow] = .25 * eref;
                }
            }
            __syncwarp();
        }
    }
    if constexpr (FP32OUT) {
        __syncthreads();  // every variant column's vref written
        if (warp == 0) block_log_offset(d, B, I, blk, lane);
    }
}

template <bool FP32OUT>
__global__ void k_varemit(BatchDev d, int nwarps, int maxS, int smem_bytes) {
    __shared__ BranchCache bc;
    if (threadIdx.x == 0) bc.inst = -1;
    __syncthreads();
    varemit_tree<FP32OUT>(d, cta_block(d), nwarps, maxS, smem_bytes, &bc);
}

// K2 as a persistent kernel over the same units as k_tables_ws.
template <bool FP32OUT>
__global__ void k_varemit_ws(BatchDev d, int nwarps, int maxS, int smem_bytes, WorkQueue q) {
    __shared__ BranchCache bc;
    if (threadIdx.x == 0) bc.inst = -1;
    __syncthreads();
    for (int u = next_unit(q); u >= 0; u = next_unit(q)) {
        const int t1 = imin((u + 1) * q.chunk, d.nblocks);
        for (int t = u * q.chunk; t < t1; t++) {
            varemit_tree<FP32OUT>(d, d.blkmap ? d.blkmap[t] : t, nwarps, maxS, smem_bytes, &bc);
            __syncthreads();
        }
    }
}

size_t tables_smem(int n, int S, int S1, int T, bool want32) {
    size_t b = sizeof(double) * (size_t)exp_table_doubles(T, want32);
    b += 2 * (size_t)n * sizeof(int4) + 8 * (size_t)n * sizeof(int);
    b += ((n + 15) & ~15);
    b += 2 * (size_t)imax(S1, 1) * sizeof(int);
    b += (size_t)(imax(imax(S, 1), MAXT) + 2) * sizeof(int);
    return b;
}

}  // namespace

// CTAs of a persistent kernel: as many as are resident on the GPU at once, at most one per
// unit of work.
template <typename K>
int persistent_grid(K kernel, int threads, size_t smem, int nunits) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    return imax(1, imin(nunits, per_sm * sms));
}

void launch_tables(const BatchDev &d, bool want32, cudaStream_t s, int *queue, int chunk) {
    size_t smem = tables_smem(d.maxnodes, d.maxS, d.maxS, d.maxT, want32);
    if (!queue) {
        prefer_shared(k_tables);
        // opt in; static shared memory counts against 48 KB too
        if (!raise_dynamic_smem(k_tables, smem)) return;
        k_tables<<<d.nblocks, TAB_THREADS, smem, s>>>(d, want32 ? 1 : 0);
    } else {
        prefer_shared(k_tables_ws);
        if (!raise_dynamic_smem(k_tables_ws, smem)) return;
        chunk = imax(chunk, 1);
        const WorkQueue q{queue, (d.nblocks + chunk - 1) / chunk, chunk};
        const int grid = persistent_grid(k_tables_ws, TAB_THREADS, smem, q.nunits);
        k_tables_ws<<<grid, TAB_THREADS, smem, s>>>(d, want32 ? 1 : 0, q);
    }
    note_launch();
}

// K2's shared-memory carve for w warps, offset by offset (16-byte alignment where it aligns);
// lean: an FP32 batch with FP32 per-state factors and 4-byte scratch only.
size_t varemit_need(int n, int maxS, bool lean, int w) {
    const size_t esz = lean ? sizeof(float) : sizeof(double);
    auto a16 = [](size_t o) { return (o + 15) & ~(size_t)15; };
    size_t o = (size_t)n * sizeof(int4);                              // nd
    o = a16(o) + 2 * (size_t)n * sizeof(double);                      // muts, nomuts
    if (!lean) o = a16(o) + 6 * (size_t)maxS * sizeof(double);        // pm
    o = a16(o) + (6 * (size_t)n + 4 + maxS) * sizeof(int);            // order .. outp
    o += (size_t)maxS;                                                // sfloor
    o = a16(o) + 2 * (size_t)n * sizeof(float);                       // muts32, nomuts32
    o = a16(o) + 8 * (size_t)maxS * sizeof(float);                    // pm32
    o = a16(o) + (size_t)w * n * 8 * esz;                             // scratch
    o += (size_t)w * maxS * esz;                                      // ebuf
    return o + 16;
}

bool varemit_full_carve_fits(int maxnodes, int maxS) {
    return varemit_need(maxnodes, imax(maxS, 1), false, 1) <= 200 * 1024;
}

template <bool FP32OUT>
void launch_varemit_t(const BatchDev &d, cudaStream_t s, int *queue, int chunk) {
    const int n = d.maxnodes, maxS = imax(d.maxS, 1);
    const bool lean = FP32OUT && !d.emit64;
    int nwarps = 4;
    auto need = [&](int w) { return varemit_need(n, maxS, lean, w); };
    while (nwarps > 1 && need(nwarps) > 200 * 1024) nwarps--;
    const size_t smem = need(nwarps);
    if (!queue) {
        prefer_shared(k_varemit<FP32OUT>);
        // opt in; static shared memory counts against 48 KB too
        if (!raise_dynamic_smem(k_varemit<FP32OUT>, smem)) return;
        k_varemit<FP32OUT><<<d.nblocks, nwarps * 32, smem, s>>>(d, nwarps, maxS, (int)smem);
    } else {
        prefer_shared(k_varemit_ws<FP32OUT>);
        if (!raise_dynamic_smem(k_varemit_ws<FP32OUT>, smem)) return;
        chunk = imax(chunk, 1);
        const WorkQueue q{queue, (d.nblocks + chunk - 1) / chunk, chunk};
        const int grid = persistent_grid(k_varemit_ws<FP32OUT>, nwarps * 32, smem, q.nunits);
        k_varemit_ws<FP32OUT><<<grid, nwarps * 32, smem, s>>>(d, nwarps, maxS, (int)smem, q);
    }
    note_launch();
}

void launch_varemit(const BatchDev &d, bool fp32, cudaStream_t s, int *queue, int chunk) {
    if (fp32) launch_varemit_t<true>(d, s, queue, chunk);
    else launch_varemit_t<false>(d, s, queue, chunk);
}

}  // namespace awg

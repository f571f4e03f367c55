// Host plan of a batch of threading problems.
//
// The host does only O(nodes) work per local tree and one pass over the sequences:
// validation, child arrays (the reference's set_ptree, local_tree.h:190-230), state-space
// sizes (states.cpp:53-199) for the memory layout, node mappings (make_node_mapping,
// local_tree.h:767), the model's time grid (model.h:322-333, model.cpp:9-23) and the
// column classes of the emission step (emit.cpp:30-58). Everything numeric runs on the GPU.

#include "plan.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <atomic>
#include <thread>

namespace awg {

// An instance's model block (model.h:322-333, model.cpp:9-23): times, popsizes (zeros when
// NULL), time_steps, coal_time_steps, rho, mu, mintime and the infinite-sites penalty.
void model_arrays(const double *times, const double *popsizes, int T, double rho, double mu,
                  double penalty, double *m) {
    for (int i = 0; i < MODEL_STRIDE; i++) m[i] = 0.0;
    for (int i = 0; i < T; i++) {
        m[M_TIMES + i] = times[i];
        m[M_POPSIZES + i] = popsizes ? popsizes[i] : 0.0;
    }
    for (int i = 0; i < T - 1; i++) m[M_TIMESTEPS + i] = times[i + 1] - times[i];
    m[M_TIMESTEPS + T - 1] = INFINITY;
    std::vector<double> times2(2 * T + 1, 0.0);
    for (int i = 0; i < T - 1; i++) {
        times2[2 * i] = times[i];
        times2[2 * i + 1] = std::sqrt((times[i + 1] + 1.0) * (times[i] + 1.0));
    }
    times2[2 * T - 2] = times2[2 * T - 1] = times2[2 * T] = times[T - 1];
    for (int i = 0; i < 2 * T - 2; i++)
        m[M_COALSTEPS + i] = times2[std::min(i + 1, 2 * T)] - times2[i];
    m[M_COALSTEPS + 2 * T - 2] = INFINITY;
    m[M_COALSTEPS + 2 * T - 1] = INFINITY;
    m[M_CONST + 0] = rho;
    m[M_CONST + 1] = mu;
    m[M_CONST + 2] = times[1] * .1;
    m[M_CONST + 3] = (penalty > 0.0 && penalty < 1.0) ? penalty : 1.0;
}


namespace {

bool valid_base(char c) {
    switch (c) {
        case 'A': case 'C': case 'G': case 'T': case 'N':
        case 'a': case 'c': case 'g': case 't':
            return true;
        default:
            return false;
    }
}

struct TreeScratch {
    int c0[MAXNODES], c1[MAXNODES];
};

// Children in index order (set_ptree), root, optional child[0] override of the root.
bool make_children(const int *parent, int n, int rc0, TreeScratch &ts, int &root) {
    for (int i = 0; i < n; i++) ts.c0[i] = ts.c1[i] = -1;
    root = -1;
    for (int i = 0; i < n; i++) {
        int p = parent[i];
        if (p < -1 || p >= n) return false;
        if (p == -1) {
            if (root != -1) return false;
            root = i;
        } else if (ts.c0[p] == -1) {
            ts.c0[p] = i;
        } else if (ts.c1[p] == -1) {
            ts.c1[p] = i;
        } else {
            return false;
        }
    }
    if (root < 0) return false;
    if (rc0 != -1 && ts.c0[root] != rc0) {
        if (ts.c1[root] != rc0) return false;
        std::swap(ts.c0[root], ts.c1[root]);
    }
    return true;
}

}  // namespace

int count_states(const int *parent, const int *age, int n, int T, bool internal, int minage,
                 int root_child0, int *M_out) {
    TreeScratch ts;
    int root;
    if (!make_children(parent, n, root_child0, ts, root)) return -1;
    long long S = 0, M = 0;
    if (!internal) {
        for (int i = 0; i < n; i++) {
            int top = parent[i] == -1 ? T - 2 : age[parent[i]];
            int m = std::max(0, top - age[i] + 1);
            S += m;
            M += (long long)m * m;
        }
    } else {
        if (age[root] < T) {
            if (M_out) *M_out = 0;
            return 0;
        }
        const int sub = ts.c0[root];
        minage = std::max(minage, age[sub]);
        for (int i = 0; i < n; i++) {
            if (i == root) continue;
            bool in_sub = false;
            for (int v = i; v != -1; v = parent[v])
                if (v == sub) { in_sub = true; break; }
            if (in_sub) continue;
            int t0 = std::max(age[i], minage);
            int top = parent[i] == root ? T - 2 : age[parent[i]];
            int m = std::max(0, top - t0 + 1);
            S += m;
            M += (long long)m * m;
        }
    }
    if (M_out) *M_out = (int)M;
    return (int)S;
}

thread_local int g_plan_threads = 0;
void set_plan_threads(int n) { g_plan_threads = std::max(0, n); }

namespace {

// Runs f(q) for q < n on up to hardware_concurrency threads (or the calling thread's cap).
// Threads take problems from a shared counter, the costliest first (cost(q): sequence
// bytes plus tree nodes), so a few large problems do not leave the other threads idle.
template <typename Fn>
void parallel_for(const awg_problem *probs, int n, Fn f) {
    const int hw = g_plan_threads > 0 ? g_plan_threads : (int)std::thread::hardware_concurrency();
    const int nthreads = std::max(1, std::min<int>(n, hw));
    if (nthreads <= 1 || n < 4) {
        for (int q = 0; q < n; q++) f(q);
        return;
    }
    std::vector<int> order(n);
    std::vector<long long> cost(n);
    for (int q = 0; q < n; q++) {
        order[q] = q;
        const awg_problem &p = probs[q];
        cost[q] = (long long)std::max(p.seqlen, 0) * std::max(p.nseqs, 0) +
                  (long long)std::max(p.ntrees, 0) * std::max(p.nnodes, 0) * 4;
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
    std::atomic<int> next(0);
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; t++)
        pool.emplace_back([&]() {
            for (int k = next.fetch_add(1); k < n; k = next.fetch_add(1)) f(order[k]);
        });
    for (auto &th : pool) th.join();
}

// 1 for a byte outside A, C, G, T, N (either case of ACGT)
inline uint8_t bad_base(uint8_t c) {
    const uint8_t u = c & 0xDF;  // ACGT upper-cased; 'n' stays apart from 'N'
    return !((u == 'A') | (u == 'C') | (u == 'G') | (u == 'T') | (c == 'N'));
}

// An 8 x 8 byte block transposed in registers: x[k] holds row k, byte j (little endian)
// column j; afterwards x[j] holds column j. Three rounds swap 4x4, 2x2 and 1x1 sub-blocks.
inline void transpose8x8(uint64_t x[8]) {
    for (int k = 0; k < 4; k++) {
        const uint64_t t = ((x[k] >> 32) ^ x[k + 4]) & 0x00000000FFFFFFFFull;
        x[k] ^= t << 32;
        x[k + 4] ^= t;
    }
    for (int a : {0, 1, 4, 5}) {
        const uint64_t t = ((x[a] >> 16) ^ x[a + 2]) & 0x0000FFFF0000FFFFull;
        x[a] ^= t << 16;
        x[a + 2] ^= t;
    }
    for (int a : {0, 2, 4, 6}) {
        const uint64_t t = ((x[a] >> 8) ^ x[a + 1]) & 0x00FF00FF00FF00FFull;
        x[a] ^= t << 8;
        x[a + 1] ^= t;
    }
}

// Validation and per-tree state counts of one problem; "" or the failure.
std::string check_problem(const awg_problem &p, int q, bool check_seqs, std::vector<int> &S_of,
                          std::vector<int> &M_of) {
    {
        char buf[256];
        auto fail = [&](const char *what) {
            snprintf(buf, sizeof(buf), "problem %d: %s", q, what);
            return std::string(buf);
        };
        if (p.ntrees < 1) return fail("ntrees < 1");
        if (p.nnodes < 1 || p.nnodes > MAXNODES) return fail("nnodes out of range [1, 1024]");
        if (p.ntimes < 3 || p.ntimes > MAXT) return fail("ntimes out of range [3, 32]");
        if (!p.ptrees || !p.ages || !p.sprs || !p.blocklens || !p.times || !p.popsizes || !p.seqs)
            return fail("missing input array");
        const int nleaves = (p.nnodes + 1) / 2;
        const int nemit = p.internal ? nleaves : nleaves + 1;
        if (p.nseqs < nemit) return fail("fewer sequences than leaves (+1 when external)");
        if (p.minage < 0) return fail("negative minage");
        long long L = 0;
        for (int b = 0; b < p.ntrees; b++) {
            if (p.blocklens[b] < 1) return fail("block length < 1");
            L += p.blocklens[b];
        }
        if (L != p.seqlen) return fail("block lengths do not add up to seqlen");
        if (p.seqlen < 1) return fail("seqlen < 1");
        for (int i = 0; i < p.ntimes; i++)
            if (!(p.times[i] >= 0) || !(p.popsizes[i] > 0)) return fail("bad times or popsizes");
        for (int i = 1; i < p.ntimes; i++)
            if (!(p.times[i] > p.times[i - 1])) return fail("times not increasing");
        S_of.resize(p.ntrees);
        M_of.resize(p.ntrees);
        for (int b = 0; b < p.ntrees; b++) {
            const int *par = p.ptrees + (size_t)b * p.nnodes;
            const int *age = p.ages + (size_t)b * p.nnodes;
            for (int i = 0; i < p.nnodes; i++) {
                const int maxage = p.internal ? p.ntimes + 1 : p.ntimes - 2;
                if (age[i] < 0 || age[i] > maxage) return fail("node age out of range");
            }
            int M = 0;
            int rc0 = p.root_child0 ? p.root_child0[b] : -1;
            int S = count_states(par, age, p.nnodes, p.ntimes, p.internal != 0, p.minage, rc0, &M);
            if (S < 0) return fail("malformed tree (parents/children)");
            if (!p.internal && S == 0) return fail("external tree with no states");
            S_of[b] = S;
            M_of[b] = M;
            if (b > 0) {
                const int *s = p.sprs + (size_t)b * 4;
                if (s[0] < 0 || s[0] >= p.nnodes || s[2] < 0 || s[2] >= p.nnodes)
                    return fail("SPR nodes out of range");
                if (s[1] < 0 || s[1] >= p.ntimes || s[3] < 0 || s[3] >= p.ntimes)
                    return fail("SPR times out of range");
                const int *prev = p.ptrees + (size_t)(b - 1) * p.nnodes;
                if (prev[s[0]] < 0) return fail("SPR recombines the root");
            }
        }
        if (check_seqs)
            for (long long c = 0; c < (long long)nemit * p.seqlen; c++)
                if (!valid_base(p.seqs[c])) return fail("sequence byte outside A,C,G,T,N");
    }
    return std::string();
}

}  // namespace

bool plan_layout(const awg_problem *probs, int n, HostPlan &plan, std::string &err,
                 bool check_seqs) {
    plan = HostPlan();
    if (n <= 0) { err = "empty batch"; return false; }
    plan.ninst = n;
    plan.inst.resize(n);

    // pass 1: validation and sizes, problems in parallel, with each problem's totals
    struct Tot {
        long long cells = 0, states = 0, t2 = 0;
        int maxS = 1, maxM = 1, maxlen = 1;
    };
    std::vector<std::vector<int>> S_of(n), M_of(n);
    std::vector<Tot> tot(n);
    std::vector<std::string> errs(n);
    parallel_for(probs, n, [&](int q) {
        errs[q] = check_problem(probs[q], q, check_seqs, S_of[q], M_of[q]);
        if (!errs[q].empty()) return;
        Tot &t = tot[q];
        for (int b = 0; b < probs[q].ntrees; b++) {
            const int S = S_of[q][b], len = probs[q].blocklens[b];
            t.cells += (long long)len * std::max(S, 1);
            t.states += std::max(S, 1);  // a zero-state space still takes one slot
            t.t2 += M_of[q][b];
            t.maxS = std::max(t.maxS, S);
            t.maxM = std::max(t.maxM, M_of[q][b]);
            t.maxlen = std::max(t.maxlen, len);
        }
    });
    // offsets of every problem: a prefix over the problems
    struct Off {
        long long cell, col, st, t2, nodes, map, seq;
        int blk;
    };
    std::vector<Off> off(n);
    long long cell = 0, col = 0, st = 0, t2 = 0, nodes = 0, map = 0, seq = 0;
    long long nblocks = 0;
    for (int q = 0; q < n; q++) {
        if (!errs[q].empty()) { err = errs[q]; return false; }
        const awg_problem &p = probs[q];
        const int nleaves = (p.nnodes + 1) / 2;
        const int nemit = p.internal ? nleaves : nleaves + 1;
        off[q] = Off{cell, col, st, t2, nodes, map, seq, (int)nblocks};
        plan.maxS = std::max(plan.maxS, tot[q].maxS);
        plan.maxM = std::max(plan.maxM, tot[q].maxM);
        plan.maxlen = std::max(plan.maxlen, tot[q].maxlen);
        plan.maxnodes = std::max(plan.maxnodes, p.nnodes);
        plan.maxT = std::max(plan.maxT, p.ntimes);
        cell += tot[q].cells;
        st += tot[q].states;
        t2 += tot[q].t2;
        nodes += (long long)p.ntrees * p.nnodes;
        map += (long long)(p.ntrees - 1) * p.nnodes;
        col += p.seqlen;
        seq += (long long)p.seqlen * nemit;
        nblocks += p.ntrees;
    }
    plan.nblocks = (int)nblocks;
    plan.blocks.resize(nblocks);
    plan.model.assign((size_t)n * MODEL_STRIDE, 0.0);

    // pass 2: instance and block descriptors, problems in parallel
    parallel_for(probs, n, [&](int q) {
        const awg_problem &p = probs[q];
        const Off &o = off[q];
        const int nleaves = (p.nnodes + 1) / 2;
        const int nemit = p.internal ? nleaves : nleaves + 1;
        InstDev &I = plan.inst[q];
        I.T = p.ntimes; I.internal = p.internal ? 1 : 0; I.minage = p.minage;
        I.nleaves = nleaves; I.nnodes = p.nnodes; I.nseqs = nemit; I.seqlen = p.seqlen;
        I.ntrees = p.ntrees; I.block0 = o.blk; I.pad = 0;
        I.cell0 = o.cell; I.col0 = o.col; I.seq0 = o.seq; I.model0 = (long long)q * MODEL_STRIDE;

        model_arrays(p.times, p.popsizes, p.ntimes, p.rho, p.mu, p.infsites_penalty,
                     &plan.model[(size_t)q * MODEL_STRIDE]);

        long long cellq = o.cell, stq = o.st, t2q = o.t2, nodesq = o.nodes, mapq = o.map;
        int pos = 0, blk = o.blk;
        for (int b = 0; b < p.ntrees; b++, blk++) {
            BlockDev &B = plan.blocks[blk];
            memset(&B, 0, sizeof(B));
            B.inst = q; B.b = b; B.start = pos; B.len = p.blocklens[b];
            B.S = S_of[q][b];
            B.S1 = b > 0 ? S_of[q][b - 1] : 0;
            B.nodes0 = (int)nodesq;
            B.prev_nodes0 = b > 0 ? (int)(nodesq - p.nnodes) : -1;
            const int *s = p.sprs + (size_t)b * 4;
            for (int k = 0; k < 4; k++) B.spr[k] = b > 0 ? s[k] : -1;
            B.map0 = b > 0 ? (int)mapq : -1;
            B.M = M_of[q][b];
            B.cell0 = cellq;
            B.state0 = stq;
            B.prev_state0 = b > 0 ? plan.blocks[blk - 1].state0 : -1;
            B.gptr0 = stq + blk;
            B.t2_0 = t2q;
            cellq += (long long)B.len * std::max(B.S, 1);
            stq += std::max(B.S, 1);
            t2q += B.M;
            nodesq += p.nnodes;
            if (b > 0) mapq += p.nnodes;
            pos += B.len;
        }
    });
    plan.total_cells = cell; plan.total_cols = col; plan.total_states = st;
    plan.total_M = t2; plan.total_nodes = nodes; plan.total_map = map; plan.total_seq = seq;
    return true;
}

bool plan_fill(const awg_problem *probs, int n, HostPlan &plan, const PlanDst &out,
               std::string *err) {
    // pass 3: arrays (instances in parallel), straight into the caller's buffers
    std::vector<std::string> errs(n);
    auto fill = [&](int q) {
        const awg_problem &p = probs[q];
        const InstDev &I = plan.inst[q];
        TreeScratch ts;
        for (int b = 0; b < p.ntrees; b++) {
            BlockDev &B = plan.blocks[I.block0 + b];
            const int *par = p.ptrees + (size_t)b * p.nnodes;
            const int *age = p.ages + (size_t)b * p.nnodes;
            int root;
            int rc0 = p.root_child0 ? p.root_child0[b] : -1;
            make_children(par, p.nnodes, rc0, ts, root);
            B.root = root;
            int *nd = out.nodes + (size_t)B.nodes0 * 4;
            for (int i = 0; i < p.nnodes; i++) {
                nd[4 * i + 0] = par[i];
                nd[4 * i + 1] = ts.c0[i];
                nd[4 * i + 2] = ts.c1[i];
                nd[4 * i + 3] = age[i];
            }
            if (b > 0) {
                B.prev_root = plan.blocks[I.block0 + b - 1].root;
                int *mp = out.mapping + B.map0;
                if (p.mapping) {
                    memcpy(mp, p.mapping + (size_t)b * p.nnodes, sizeof(int) * p.nnodes);
                } else {
                    const int *prev = p.ptrees + (size_t)(b - 1) * p.nnodes;
                    for (int j = 0; j < p.nnodes; j++) mp[j] = j;
                    mp[prev[B.spr[0]]] = -1;
                }
            } else {
                B.prev_root = -1;
            }
        }
        // column-major sequences, column classes and byte checks, a tile of columns at a
        // time: the tile's transposed columns are classified and checked while in cache
        const int ns = I.nseqs, L = p.seqlen;
        uint8_t *dst = out.seqT + I.seq0;
        uint8_t *cls = out.colclass + I.col0;
        int *cv = out.colvar + I.col0;
        constexpr int TILE = 256;
        unsigned bad = 0;
        int b = 0, bend = p.blocklens[0], nv = 0;
        const uint8_t *src = (const uint8_t *)p.seqs;
        const int r8 = ns & ~7;
        for (int i0 = 0; i0 < L; i0 += TILE) {
            const int i1 = std::min(L, i0 + TILE);
            const int i8 = i0 + ((i1 - i0) & ~7);
            // groups of 8 rows: 8 x 8 blocks through registers, 8-byte stores per column
            for (int r = 0; r < r8; r += 8) {
                const uint8_t *rows = src + (size_t)r * L;
                for (int i = i0; i < i8; i += 8) {
                    uint64_t x[8];
                    for (int k = 0; k < 8; k++) memcpy(&x[k], rows + (size_t)k * L + i, 8);
                    transpose8x8(x);
                    for (int j = 0; j < 8; j++) memcpy(dst + (size_t)(i + j) * ns + r, &x[j], 8);
                }
                for (int i = i8; i < i1; i++)
                    for (int k = 0; k < 8; k++) dst[(size_t)i * ns + r + k] = rows[(size_t)k * L + i];
            }
            for (int r = r8; r < ns; r++) {
                const uint8_t *row = src + (size_t)r * L;
                for (int i = i0; i < i1; i++) dst[(size_t)i * ns + r] = row[i];
            }
            for (int i = i0; i < i1; i++) {
                while (i >= bend) {  // the block ends: its variant count
                    plan.blocks[I.block0 + b].nvar = nv;
                    b++;
                    bend += p.blocklens[b];
                    nv = 0;
                }
                const uint8_t *c = dst + (size_t)i * ns;
                uint8_t diff = 0;
                for (int r = 1; r < ns; r++) diff |= (uint8_t)(c[r] ^ c[0]);
                // bytes checked here, in cache: an invariant column's bytes all equal c[0]
                if (!diff) {
                    bad |= bad_base(c[0]);
                    cls[i] = (c[0] == 'N') ? COL_MASKED : COL_INVARIANT;
                    cv[i] = -1;
                } else {
                    for (int r = 0; r < ns; r++) bad |= bad_base(c[r]);
                    cls[i] = COL_VARIANT;
                    cv[i] = nv++;
                }
            }
        }
        plan.blocks[I.block0 + b].nvar = nv;
        if (bad) {
            char buf[96];
            snprintf(buf, sizeof(buf), "problem %d: sequence byte outside A,C,G,T,N", q);
            errs[q] = buf;
        }
    };
    parallel_for(probs, n, fill);
    for (int q = 0; q < n; q++)
        if (!errs[q].empty()) {
            if (err) *err = errs[q];
            return false;
        }
    long long var = 0, vcols = 0;
    for (auto &B : plan.blocks) {
        B.var0 = var;
        B.vrow0 = vcols;
        var += (long long)B.nvar * std::max(B.S, 1);
        vcols += B.nvar;
    }
    plan.total_var = var;
    plan.total_vcols = vcols;
    return true;
}

bool build_plan(const awg_problem *probs, int n, HostPlan &plan, std::string &err) {
    if (!plan_layout(probs, n, plan, err, false)) return false;
    plan.nodes.assign((size_t)plan.total_nodes * 4, -1);
    plan.mapping.assign((size_t)std::max(plan.total_map, 1LL), -1);
    plan.seqT.assign((size_t)std::max(plan.total_seq, 1LL), 'N');
    plan.colclass.assign((size_t)plan.total_cols, COL_INVARIANT);
    plan.colvar.assign((size_t)plan.total_cols, -1);
    return plan_fill(probs, n, plan,
                     PlanDst{plan.nodes.data(), plan.mapping.data(), plan.seqT.data(),
                             plan.colclass.data(), plan.colvar.data()},
                     &err);
}

}  // namespace awg

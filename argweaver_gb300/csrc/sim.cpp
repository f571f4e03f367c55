// Seeded input generator for the threading HMM: a discrete-time SMC (DSMC) ARG in the
// reference's LocalTrees layout, an infinite-sites mutation drop on its local trees, and
// (optionally) one extra haplotype threaded onto the ARG, which the HMM then re-threads.
//
// The ARG process restates the reference's Python simulator (argweaver/sim.py):
//   sample_tree            sim.py:31-63    coalescent tree with piecewise-constant sizes
//   discretize_arg         __init__.py:210 ages rounded to the closer time point (top excluded)
//   sample_dsmc_sprs       sim.py:132-262  recombination time/branch, re-coalescence time/branch
//   sample_arg_mutations   sim.py:297-323  mutations per branch with minimum length times[1]/10
// It works directly in compressed columns: rho and mu are per column (rate * compress), which
// is how the reference's sampler sees them after compress_model (arg-sample.cpp:428-436).
// Trees are stored the way the reference's C API takes them (arghmm_new_trees,
// local_tree.cpp:1817): per tree a parent array and age indices with leaves first; the SPR
// to the left of each tree; each tree equals the previous one with apply_spr
// (local_tree.cpp:223-314) applied, which reuses the broken node as the re-coalescence node.
//
// The extra haplotype is not part of the reference's simulator: its lineage attaches to the
// local tree at a (branch, time) point drawn from the single-lineage coalescent, moves to a
// fresh point after a recombination on its own branch (rate rho * its height) or when an SPR
// invalidates its point, inherits every mutation above its attachment point and gets its own
// mutations on its branch. Missing calls ('N') are dropped uniformly on every sequence.
//
// Host-only C++; compiled into libawg_sim.so by argweaver_gb300/build.py.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <new>

namespace {

struct Rng {  // xoshiro256** seeded by splitmix64: identical streams on every host
    uint64_t s[4];
    explicit Rng(uint64_t seed) {
        uint64_t z = seed + 0x9E3779B97F4A7C15ull;
        for (int i = 0; i < 4; i++) {
            z += 0x9E3779B97F4A7C15ull;
            uint64_t x = z;
            x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
            x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
            s[i] = x ^ (x >> 31);
        }
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3]; s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    double uniform() { return (next() >> 11) * (1.0 / 9007199254740992.0); }
    double uniform_open() {  // (0, 1]
        return ((next() >> 11) + 1) * (1.0 / 9007199254740992.0);
    }
    double expovariate(double rate) { return -std::log(uniform_open()) / rate; }
    int below(int n) { return (int)(uniform() * n) % n; }
};

struct Tree {
    int n = 0, root = -1;
    std::vector<int> parent, c0, c1, age;
    void resize(int nn) {
        n = nn;
        parent.assign(nn, -1); c0.assign(nn, -1); c1.assign(nn, -1); age.assign(nn, 0);
    }
    bool leaf(int v) const { return c0[v] == -1; }
    int sibling(int v) const { int p = parent[v]; return c0[p] == v ? c1[p] : c0[p]; }
    int top(int v, int ntimes) const {  // last time index a state on branch v may use
        return parent[v] == -1 ? ntimes - 2 : age[parent[v]];
    }
};

struct Spr { int rn, rt, cn, ct; };

// apply_spr (local_tree.cpp:223-314): prune recomb_node, reuse its old parent as the
// re-coalescence node on the coal branch.
void apply_spr(Tree &t, const Spr &spr) {
    if (spr.rn == t.root) return;
    int recoal = t.parent[spr.rn];
    int other = (t.c0[recoal] == spr.rn) ? 1 : 0;
    int recomb_sib = other ? t.c1[recoal] : t.c0[recoal];
    int broke_parent = t.parent[recoal];
    t.parent[recomb_sib] = broke_parent;
    int x = 0;
    if (broke_parent != -1) {
        x = (t.c0[broke_parent] == recoal) ? 0 : 1;
        (x ? t.c1 : t.c0)[broke_parent] = recomb_sib;
    }
    if (spr.cn == recoal) {
        (other ? t.c1 : t.c0)[recoal] = recomb_sib;
        t.parent[recoal] = t.parent[recomb_sib];
        t.parent[recomb_sib] = recoal;
        if (broke_parent != -1) (x ? t.c1 : t.c0)[broke_parent] = recoal;
    } else {
        (other ? t.c1 : t.c0)[recoal] = spr.cn;
        t.parent[recoal] = t.parent[spr.cn];
        t.parent[spr.cn] = recoal;
        int p = t.parent[recoal];
        if (p != -1) {
            if (t.c0[p] == spr.cn) t.c0[p] = recoal; else t.c1[p] = recoal;
        }
    }
    t.age[recoal] = spr.ct;
    int root;
    if (spr.cn == t.root) root = recoal;
    else if (recoal == t.root) root = (spr.cn == recomb_sib) ? recoal : recomb_sib;
    else root = t.root;
    t.root = root;
}

struct Model {
    int ntimes;
    std::vector<double> times, time_steps, times2, popsize_hap;
    double mintime;
};

// Coalescent tree (sim.py:31-63) with leaves 0..k-1, internal nodes k..2k-2 in order of
// their (continuous) coalescence times, then ages rounded to the closer of the time points
// times[0..T-2] (discretize_arg with ignore_top).
void sample_tree(Rng &rng, const Model &m, int k, Tree &t) {
    const int T = m.ntimes;
    t.resize(2 * k - 1);
    std::vector<int> lineages(k);
    for (int i = 0; i < k; i++) lineages[i] = i;
    std::vector<double> ctime(2 * k - 1, 0.0);
    int timei = 0, next = k;
    double tt = 0.0;
    while ((int)lineages.size() > 1) {
        int k2 = (int)lineages.size();
        double rate = (k2 * (k2 - 1) / 2) / m.popsize_hap[timei];
        double t2 = rng.expovariate(rate);
        if (timei < T - 2 && tt + t2 > m.times[timei + 1]) {
            timei++;
            tt = m.times[timei];
            continue;
        }
        tt += t2;
        int a = rng.below(k2);
        int va = lineages[a];
        lineages[a] = lineages.back(); lineages.pop_back();
        int b = rng.below(k2 - 1);
        int vb = lineages[b];
        int v = next++;
        t.c0[v] = va; t.c1[v] = vb; t.parent[va] = v; t.parent[vb] = v;
        ctime[v] = tt;
        lineages[b] = v;
    }
    t.root = lineages[0];
    for (int v = 0; v < t.n; v++) {
        double a = ctime[v];
        int i = 0;  // largest time point <= a among times[0..T-2]
        while (i + 1 <= T - 2 && m.times[i + 1] <= a) i++;
        int j = std::min(i + 1, T - 2);
        if (a >= m.times[T - 2]) { i = j = T - 2; }
        t.age[v] = (a - m.times[i] < m.times[j] - a) ? i : j;
    }
    // discretized ages must stay monotone along every root path
    for (int v = k; v < t.n; v++) {  // internal nodes are in increasing continuous time
        int a0 = t.age[t.c0[v]], a1 = t.age[t.c1[v]];
        if (t.age[v] < std::max(a0, a1)) t.age[v] = std::max(a0, a1);
    }
}

void count_lineages(const Tree &t, int T, std::vector<int> &nbranches) {
    nbranches.assign(T, 0);
    for (int v = 0; v < t.n; v++) {
        int top = t.top(v, T);
        for (int j = t.age[v]; j < top; j++) nbranches[j]++;
        if (t.parent[v] == -1) nbranches[top]++;
    }
    nbranches[T - 1] = 1;
}

double tree_length(const Tree &t, const Model &m) {  // sim.py: sum of branch lengths
    double s = 0.0;
    for (int v = 0; v < t.n; v++)
        if (t.parent[v] != -1) s += m.times[t.age[t.parent[v]]] - m.times[t.age[v]];
    return s;
}

// One DSMC recombination + re-coalescence on tree t (sim.py:178-230).
Spr sample_spr(Rng &rng, const Model &m, const Tree &t, std::vector<int> &nbranches) {
    const int T = m.ntimes;
    count_lineages(t, T, nbranches);
    const int root_age = t.age[t.root];

    std::vector<double> probs(root_age + 1);
    double tot = 0.0;
    for (int i = 0; i <= root_age; i++) {
        probs[i] = nbranches[i] * (m.times[i + 1] - m.times[i]);
        tot += probs[i];
    }
    double u = rng.uniform() * tot, acc = 0.0;
    int rt = root_age;
    for (int i = 0; i <= root_age; i++) { acc += probs[i]; if (u < acc) { rt = i; break; } }

    std::vector<int> cand;
    for (int v = 0; v < t.n; v++)
        if (v != t.root && t.age[v] <= rt && rt <= t.top(v, T)) cand.push_back(v);
    const int rn = cand[rng.below((int)cand.size())];

    int j = rt;
    int last_kj = nbranches[std::max(j - 1, 0)];
    while (j < T - 2) {
        int kj = nbranches[j];
        if (t.age[rn] <= j && j <= t.top(rn, T) && t.age[t.parent[rn]] > j) kj -= 1;
        double A = (m.times2[2 * j + 1] - m.times2[2 * j]) * kj;
        if (j > rt) A += (m.times2[2 * j] - m.times2[2 * j - 1]) * last_kj;
        double coal_prob = 1.0 - std::exp(-A / m.popsize_hap[j]);
        if (rng.uniform() < coal_prob) break;
        j++;
        last_kj = kj;
    }
    const int ct = j;

    std::vector<char> exclude(t.n, 0);
    std::vector<int> stack{rn};
    while (!stack.empty()) {
        int v = stack.back(); stack.pop_back();
        exclude[v] = 1;
        if (t.age[v] == ct && !t.leaf(v)) { stack.push_back(t.c0[v]); stack.push_back(t.c1[v]); }
    }
    const int bp = t.parent[rn];
    cand.clear();
    for (int v = 0; v < t.n; v++) {
        if (exclude[v]) continue;
        if (!(t.age[v] <= ct && ct <= t.top(v, T))) continue;
        if (v == bp && ct == t.age[bp]) continue;
        cand.push_back(v);
    }
    const int cn = cand[rng.below((int)cand.size())];
    return Spr{rn, rt, cn, ct};
}

bool is_ancestor_or_self(const Tree &t, int anc, int v) {
    for (; v != -1; v = t.parent[v]) if (v == anc) return true;
    return false;
}

struct Thread { int node, time; };

// Attachment point for one new lineage from the discretized single-lineage coalescent.
Thread sample_attach(Rng &rng, const Model &m, const Tree &t, std::vector<int> &nbranches) {
    const int T = m.ntimes;
    count_lineages(t, T, nbranches);
    int j = 0;
    while (j < T - 2) {
        double A = (m.times2[2 * j + 1] - m.times2[2 * j]) * nbranches[j];
        if (j > 0) A += (m.times2[2 * j] - m.times2[2 * j - 1]) * nbranches[j - 1];
        if (rng.uniform() < 1.0 - std::exp(-A / m.popsize_hap[j])) break;
        j++;
    }
    std::vector<int> cand;
    for (int v = 0; v < t.n; v++)
        if (t.age[v] <= j && j <= t.top(v, T)) cand.push_back(v);
    return Thread{cand[rng.below((int)cand.size())], j};
}

}  // namespace

extern "C" {

// Parameters of one simulated instance (all rates per base pair; columns are `compress` bp).
struct awg_sim_params {
    int nleaves;          // leaves of the simulated ARG (the re-threaded haplotype is extra)
    int seqlen;           // compressed columns
    int compress;         // bp per column
    int ntimes;           // time points
    int add_thread;       // 1: add one threaded haplotype after the ARG's leaves
    int pad;
    double maxtime, popsize, rho, mu;   // popsize is the diploid N the HMM uses
    double missing;       // per-call probability of 'N'
    unsigned long long seed;
};

struct awg_sim_result {
    int ntrees, nnodes, nseqs, seqlen, ntimes;
    int *ptrees, *ages, *sprs, *blocklens, *mapping;  // [ntrees*nnodes], ..., [ntrees*4]
    char *seqs;                                       // [nseqs*seqlen]
    int *path_node, *path_time;                       // true thread per column (add_thread)
    double *times, *popsizes;                         // [ntimes]
    double rho, mu;                                   // per column
};

void awg_sim_free(awg_sim_result *r) {
    if (!r) return;
    delete[] r->ptrees; delete[] r->ages; delete[] r->sprs; delete[] r->blocklens;
    delete[] r->mapping; delete[] r->seqs; delete[] r->path_node; delete[] r->path_time;
    delete[] r->times; delete[] r->popsizes;
    delete r;
}

// Returns NULL on invalid parameters.
awg_sim_result *awg_sim_run(const awg_sim_params *p) {
    if (!p || p->nleaves < 2 || p->seqlen < 2 || p->ntimes < 4 || p->compress < 1)
        return nullptr;
    Rng rng(p->seed);
    const int T = p->ntimes;
    Model m;
    m.ntimes = T;
    m.times.resize(T);
    const double delta = 0.01;
    for (int i = 0; i < T; i++)  // get_time_points (model.h:21-32)
        m.times[i] = (std::exp(i / double(T - 1) * std::log(1.0 + delta * p->maxtime)) - 1) / delta;
    m.times2.assign(2 * T + 1, 0.0);
    for (int i = 0; i < T - 1; i++) {
        m.times2[2 * i] = m.times[i];
        m.times2[2 * i + 1] = std::sqrt((m.times[i + 1] + 1.0) * (m.times[i] + 1.0));
    }
    m.times2[2 * (T - 1)] = m.times[T - 1];
    m.popsize_hap.assign(T, 2.0 * p->popsize);
    m.mintime = m.times[1] * 0.1;
    const double rho_c = p->rho * p->compress, mu_c = p->mu * p->compress;

    const int k = p->nleaves;
    const int L = p->seqlen;
    Tree tree;
    sample_tree(rng, m, k, tree);
    const int n = tree.n;

    std::vector<Tree> trees;
    std::vector<Spr> sprs;
    std::vector<int> starts;
    trees.push_back(tree);
    sprs.push_back(Spr{-1, -1, -1, -1});
    starts.push_back(0);
    std::vector<int> nb;
    int pos = 0;
    while (true) {
        double tl = tree_length(tree, m);
        double bl = 0.0;
        while (bl < 1.0) bl = rng.expovariate(std::max(tl * rho_c, rho_c));
        pos += (int)bl;
        if (pos >= L - 1) break;
        Spr s = sample_spr(rng, m, tree, nb);
        apply_spr(tree, s);
        trees.push_back(tree);
        sprs.push_back(s);
        starts.push_back(pos);
    }
    const int ntrees = (int)trees.size();

    const int nseqs = k + (p->add_thread ? 1 : 0);
    std::vector<char> seqs((size_t)nseqs * L, 'A');
    std::vector<int> pnode(L, -1), ptime(L, -1);

    Thread th{-1, -1};
    for (int b = 0; b < ntrees; b++) {
        const Tree &t = trees[b];
        const int start = starts[b], end = (b + 1 < ntrees) ? starts[b + 1] : L;
        if (p->add_thread) {
            bool valid = th.node >= 0 && th.node < n && t.age[th.node] <= th.time &&
                         th.time <= t.top(th.node, T);
            if (b > 0 && valid) {  // the broken node moved: its points are re-drawn
                int broken = trees[b - 1].parent[sprs[b].rn];
                if (th.node == broken) valid = false;
            }
            if (!valid) th = sample_attach(rng, m, t, nb);
        }
        // branch lengths for the mutation drop (sim.py:312-321)
        std::vector<double> blen(n, 0.0);
        double total = 0.0;
        for (int v = 0; v < n; v++)
            if (t.parent[v] != -1) {
                blen[v] = std::max(m.times[t.age[t.parent[v]]] - m.times[t.age[v]], m.mintime);
                total += blen[v];
            }
        double next_mut = start + rng.expovariate(total * mu_c);
        for (int i = start; i < end; i++) {
            if (p->add_thread) {
                double h = std::max(m.times[th.time], m.mintime);
                if (i > start && rng.uniform() < 1.0 - std::exp(-rho_c * h))
                    th = sample_attach(rng, m, t, nb);
                pnode[i] = th.node;
                ptime[i] = th.time;
                if (rng.uniform() < 1.0 - std::exp(-mu_c * h)) {  // own-branch mutation
                    char &c = seqs[(size_t)k * L + i];
                    c = (c == 'A') ? 'G' : 'A';
                }
            }
            while (next_mut < i + 1) {
                // branch proportional to length, time uniform along it
                double u = rng.uniform() * total, acc = 0.0;
                int x = -1;
                for (int v = 0; v < n; v++) {
                    if (t.parent[v] == -1) continue;
                    acc += blen[v];
                    x = v;
                    if (u < acc) break;
                }
                double tm = m.times[t.age[x]] + rng.uniform() * blen[x];
                for (int leaf = 0; leaf < k; leaf++)
                    if (is_ancestor_or_self(t, x, leaf)) {
                        char &c = seqs[(size_t)leaf * L + i];
                        c = (c == 'A') ? 'G' : 'A';
                    }
                if (p->add_thread && is_ancestor_or_self(t, x, th.node) &&
                    (x != th.node || tm > m.times[th.time])) {
                    char &c = seqs[(size_t)k * L + i];
                    c = (c == 'A') ? 'G' : 'A';
                }
                next_mut += rng.expovariate(total * mu_c);
            }
        }
    }
    if (p->missing > 0.0)
        for (size_t c = 0; c < seqs.size(); c++)
            if (rng.uniform() < p->missing) seqs[c] = 'N';

    awg_sim_result *r = new (std::nothrow) awg_sim_result();
    if (!r) return nullptr;
    r->ntrees = ntrees; r->nnodes = n; r->nseqs = nseqs; r->seqlen = L; r->ntimes = T;
    r->ptrees = new int[(size_t)ntrees * n];
    r->ages = new int[(size_t)ntrees * n];
    r->mapping = new int[(size_t)ntrees * n];
    r->sprs = new int[(size_t)ntrees * 4];
    r->blocklens = new int[ntrees];
    for (int b = 0; b < ntrees; b++) {
        for (int v = 0; v < n; v++) {
            r->ptrees[(size_t)b * n + v] = trees[b].parent[v];
            r->ages[(size_t)b * n + v] = trees[b].age[v];
            r->mapping[(size_t)b * n + v] = v;  // make_node_mapping (local_tree.h:767)
        }
        if (b > 0) r->mapping[(size_t)b * n + trees[b - 1].parent[sprs[b].rn]] = -1;
        else for (int v = 0; v < n; v++) r->mapping[v] = -1;
        r->sprs[b * 4 + 0] = sprs[b].rn; r->sprs[b * 4 + 1] = sprs[b].rt;
        r->sprs[b * 4 + 2] = sprs[b].cn; r->sprs[b * 4 + 3] = sprs[b].ct;
        r->blocklens[b] = ((b + 1 < ntrees) ? starts[b + 1] : L) - starts[b];
    }
    r->seqs = new char[seqs.size()];
    memcpy(r->seqs, seqs.data(), seqs.size());
    r->path_node = new int[L];
    r->path_time = new int[L];
    memcpy(r->path_node, pnode.data(), sizeof(int) * L);
    memcpy(r->path_time, ptime.data(), sizeof(int) * L);
    r->times = new double[T];
    r->popsizes = new double[T];
    for (int i = 0; i < T; i++) { r->times[i] = m.times[i]; r->popsizes[i] = p->popsize; }
    r->rho = rho_c;
    r->mu = mu_c;
    return r;
}

}  // extern "C"

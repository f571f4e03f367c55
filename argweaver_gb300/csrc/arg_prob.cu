// Probabilities of a whole ARG (total_prob.cpp; C exports at total_prob.cpp:315-382, bound
// by argweaver/argweaverc.py:219-245) on the device:
//
//   likelihood   calc_arg_likelihood (total_prob.cpp:19-45): per local tree, the sum over
//                its sites of log P(site | tree) by Felsenstein's pruning
//                (likelihood_tree, emit.cpp:399-446; likelihood_site_inner, emit.cpp:151-269)
//   prior        calc_arg_prior (total_prob.cpp:262-300): per tree, the recombination
//                spacing and the SPR's probability (calc_spr_prob, total_prob.cpp:210-259)
//   tree prior   calc_tree_prior (total_prob.cpp:132-165): the first tree's coalescent prior
//
// Likelihood: one CTA per local tree. Its warps take the tree's sites in turn; a site that
// varies runs the pruning one height level of the tree at a time (lanes over the level's
// nodes), in the reference's arithmetic per node. As in the reference, every invariant
// site of a tree (all sequences equal, 'N' included) gets the likelihood of the tree's
// first invariant site. Prior: one warp per tree; lineage counts with a lane per time
// point. Per-tree values land in an array and are summed in tree order by one thread, so
// a result does not depend on scheduling.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "kernels.h"
#include "plan.h"
#include "tree_util.cuh"

namespace awg {

namespace {

constexpr int LIK_THREADS = 128;
constexpr int LIK_WARPS = LIK_THREADS / 32;
constexpr unsigned FULLMASK = 0xffffffffu;

struct ArgDev {
    int ntrees, nnodes, nleaves, nseqs, T;
    const int4 *nodes;     // [ntrees][nnodes] {parent, child0, child1, age}
    const int *bounds;     // [ntrees + 1] first site of each tree (relative), then the end
    const int *last;       // [ntrees] 1 where the reference treats the tree as the last
    const int4 *sprs;      // [ntrees] the SPR into each tree
    const double *model;   // MODEL_STRIDE doubles
    const uint8_t *seqT;   // [sites][nseqs] sequences, site-major
    double *lik, *prior;   // [ntrees] per-tree terms
    double *out;           // [4]: likelihood, prior, tree prior, (unused)
    int *err;              // [2]: code, tree
};

enum : int { AP_OK = 0, AP_BAD_TREE = 1, AP_ZERO = 2 };

__device__ void ap_error(const ArgDev &a, int code, int tree) {
    if (atomicCAS(a.err, 0, code) == 0) a.err[1] = tree;
}

// ---------------------------------------------------------------------------------------
// likelihood

template <int W>
__global__ void __launch_bounds__(LIK_THREADS) k_arg_likelihood(ArgDev a) {
    extern __shared__ double lk_dyn[];
    const int b = blockIdx.x, n = a.nnodes, T = a.T;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    double *muts = lk_dyn;                             // [n]
    double *nomuts = muts + n;                         // [n]
    double *part = nomuts + n;                         // [W][n][4] inner partials per warp
    int4 *nd = (int4 *)(part + (size_t)W * n * 4);    // [n]
    int *hgt = (int *)(nd + n);                        // [n]
    int *lvl = hgt + n;                                // [n] nodes by height
    int *lptr = lvl + n;                               // [n + 2]
    int *cursor = lptr + n + 2;                        // [n]
    __shared__ double times[32], acc[W], sh_inv;
    __shared__ int sh_root, sh_nlev, sh_first, ninv[W];

    const double *model = a.model;
    const double mu = model[M_CONST + 1], mintime = model[M_CONST + 2];
    for (int i = tid; i < T; i += blockDim.x) times[i] = model[M_TIMES + i];
    const int4 *gnd = a.nodes + (size_t)b * n;
    bool bad = false;
    for (int i = tid; i < n; i += blockDim.x) {
        const int4 v = gnd[i];
        nd[i] = v;
        hgt[i] = 0;
        if (v.x < -1 || v.x >= n || v.y < -1 || v.y >= n || v.z < -1 || v.z >= n || v.w < 0 ||
            v.w >= T || (v.y == -1) != (i < a.nleaves))
            bad = true;
        if (v.x == -1) sh_root = i;
    }
    if (__syncthreads_or(bad)) {
        if (tid == 0) ap_error(a, AP_BAD_TREE, b);
        return;
    }
    const int root = sh_root;
    // branch probabilities (likelihood_tree, emit.cpp:411-421)
    for (int i = tid; i < n; i += blockDim.x) {
        if (i == root) continue;
        const double e = branch_exp(fmax(times[nd[nd[i].x].w] - times[nd[i].w], mintime), mu);
        muts[i] = branch_mut(e);
        nomuts[i] = branch_nomut(e);
    }
    // heights: longest path down to a leaf; walks bounded by n steps
    for (int i = tid; i < a.nleaves; i += blockDim.x) {
        int v = i;
        for (int dd = 1; dd <= n && nd[v].x != -1; dd++) {
            v = nd[v].x;
            atomicMax(&hgt[v], dd);
        }
    }
    __syncthreads();
    const int s0 = a.bounds[b], s1 = a.bounds[b + 1], ns = a.nseqs;
    if (warp == 0) {
        const int nl = warp_levels(hgt, n, lvl, lptr, cursor, lane);
        // the tree's first invariant site (is_invariant_site, emit.cpp:16-26)
        int first = -1;
        for (int base = s0; base < s1 && first < 0; base += 32) {
            const int s = base + lane;
            bool inv = s < s1;
            if (inv) {
                const uint8_t *ch = a.seqT + (size_t)s * ns;
                const uint8_t c0 = ch[0];
                for (int j = 1; j < ns && inv; j++) inv = ch[j] == c0;
            }
            const unsigned m = __ballot_sync(FULLMASK, inv);
            if (m) first = base + __ffs(m) - 1;
        }
        if (lane == 0) {
            sh_nlev = nl;
            sh_first = first;
        }
    }
    __syncthreads();
    const int nlev = sh_nlev;
    double (*in)[4] = (double (*)[4])(part + (size_t)warp * n * 4);

    // P(site | tree) by the warp: leaves, then one height level at a time
    // (likelihood_site_node_inner, emit.cpp:151-196; likelihood_site_inner, :252-269)
    auto site_lk = [&](int s) -> double {
        const uint8_t *ch = a.seqT + (size_t)s * ns;
        for (int x = lane; x < lptr[1]; x += 32) {
            const int j = lvl[x];
            leaf_partial<double>(ch[j], in[j]);
        }
        __syncwarp();
        for (int h = 1; h < nlev; h++) {
            for (int x = lptr[h] + lane; x < lptr[h + 1]; x += 32) {
                const int j = lvl[x];
                const int c1 = nd[j].y, c2 = nd[j].z;
                double p1[4], p2[4];
                jc_apply<false>(in[c1], muts[c1], nomuts[c1], p1);
                jc_apply<false>(in[c2], muts[c2], nomuts[c2], p2);
#pragma unroll
                for (int q = 0; q < 4; q++) in[j][q] = p1[q] * p2[q];
            }
            __syncwarp();
        }
        double p = 0.0;
#pragma unroll
        for (int q = 0; q < 4; q++) p += in[root][q] * .25;
        __syncwarp();
        return p;
    };

    if (warp == 0 && sh_first >= 0) {
        const double v = site_lk(sh_first);
        if (lane == 0) sh_inv = v;
    }
    __syncthreads();
    double sum = 0.0;
    int cinv = 0;
    for (int s = s0 + warp; s < s1; s += W) {
        const uint8_t *ch = a.seqT + (size_t)s * ns;
        const uint8_t c0 = ch[0];
        bool diff = false;
        for (int j = 1 + lane; j < ns; j += 32) diff |= ch[j] != c0;
        if (!__any_sync(FULLMASK, diff)) {
            cinv++;
            continue;
        }
        const double v = site_lk(s);
        if (lane == 0) {
            if (!(v > 0.0)) ap_error(a, AP_ZERO, b);
            sum += log(v);
        }
    }
    if (lane == 0) {
        acc[warp] = sum;
        ninv[warp] = cinv;
    }
    __syncthreads();
    if (tid == 0) {
        double t = 0.0;
        int ci = 0;
        for (int w = 0; w < W; w++) {
            t += acc[w];
            ci += ninv[w];
        }
        if (ci > 0) t += ci * log(sh_inv);
        a.lik[b] = t;
    }
}

// ---------------------------------------------------------------------------------------
// prior

// Lineage counts of one tree at time t = lane (count_lineages, local_tree.cpp:34-68).
__device__ void lane_lineages(const int4 *nd, int n, int T, int t, int &nb, int &nr, int &nc) {
    nb = nr = nc = 0;
    if (t >= T) return;
    for (int i = 0; i < n; i++) {
        const int4 v = nd[i];
        const int pa = v.x == -1 ? T - 2 : nd[v.x].w;
        const int span = (v.w <= t && t < pa) ? 1 : 0;
        nb += span + ((v.x == -1 && t == pa) ? 1 : 0);
        nr += span + (t == pa ? 1 : 0);
        nc += span + (t == pa ? 1 : 0);
    }
    if (t == T - 1) nb = 1;
}

// One warp per tree: the tree's term of calc_arg_prior (total_prob.cpp:262-300).
__global__ void k_arg_prior(ArgDev a) {
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (b >= a.ntrees) return;
    const int n = a.nnodes, T = a.T;
    const int4 *nd = a.nodes + (size_t)b * n;
    const double *times = a.model + M_TIMES, *tsteps = a.model + M_TIMESTEPS;
    const double *csteps = a.model + M_COALSTEPS, *pops = a.model + M_POPSIZES;
    const double rho = a.model[M_CONST + 0];
    // tree length without the basal stub (get_treelen, local_tree.cpp:136-153)
    double part = 0.0;
    int root = -1;
    for (int i = lane; i < n; i += 32) {
        const int4 v = nd[i];
        if (v.x == -1) root = i;
        else part += times[nd[v.x].w] - times[v.w];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        part += __shfl_xor_sync(FULLMASK, part, o);
        root = max(root, __shfl_xor_sync(FULLMASK, root, o));
    }
    const double treelen = part;
    const double recomb_rate = fmax(rho * treelen, rho);
    const int blocklen = a.bounds[b + 1] - a.bounds[b];
    if (a.last[b]) {  // probability of not recombining after blocklen
        if (lane == 0) a.prior[b] = -recomb_rate * blocklen;
        return;
    }
    // probability of recombining after blocklen, then of the SPR into the next tree
    // (calc_spr_prob, total_prob.cpp:210-259)
    const int4 spr = a.sprs[b + 1];
    const int root_age = nd[root].w;
    const double treelen_b = treelen + tsteps[root_age];
    int nb, nr, nc;
    lane_lineages(nd, n, T, lane, nb, nr, nc);
    if (lane == root_age) nr--;
    const int k = spr.y, j = spr.w;
    const int broken_age = nd[nd[spr.x].x].w;
    const int nb_k = __shfl_sync(FULLMASK, nb, k), nr_k = __shfl_sync(FULLMASK, nr, k);
    const int nc_j = __shfl_sync(FULLMASK, nc, j);
    // coalescence rates (calc_coal_rates_full_tree, total_prob.cpp:196-207): rate m on
    // lane m / 2; the sum of those in [2k, 2j - 1)
    auto rate = [&](int m) {
        const int nbm = __shfl_sync(FULLMASK, nb, m / 2) - int(m / 2 < broken_age);
        return csteps[m] * nbm / (2.0 * pops[m / 2]);
    };
    double below = 0.0;
    for (int m0 = 0; m0 < 2 * T; m0 += 32) {
        const int m = m0 + lane;
        const double r = rate(m < 2 * T ? m : 0);
        if (m >= 2 * k && m < 2 * j - 1 && m < 2 * T) below += r;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) below += __shfl_xor_sync(FULLMASK, below, o);
    const double r2j = rate(2 * j < 2 * T ? 2 * j : 0);
    const double r2j1 = rate(j > 0 ? 2 * j - 1 : 0);
    if (lane == 0) {
        double lnl = log(recomb_rate) - recomb_rate * blocklen;
        double sp = 0.0;
        sp += log(nb_k * tsteps[k] / (nr_k * treelen_b));
        const int ncoals_j = nc_j - int(j <= broken_age) - int(j == broken_age);
        sp -= log((double)ncoals_j);
        if (j < T - 2) sp += log(1.0 - exp(-r2j - (j > k ? r2j1 : 0.0)));
        sp -= below;
        a.prior[b] = lnl + sp;
    }
}

// P(a lineages -> b lineages in time t, population n) (prob_coal_counts, total_prob.cpp:108-127)
__device__ double prob_coal_counts(int a, int b, double t, double n) {
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

// One warp: the first tree's prior (calc_tree_prior, total_prob.cpp:132-165), terms on
// lanes, summed in order; then the sums of the per-tree terms, in tree order.
__global__ void k_arg_totals(ArgDev a, int want_lik, int want_prior, int want_tree) {
    const int lane = threadIdx.x;
    const int n = a.nnodes, T = a.T;
    if (want_tree) {
        const double *csteps = a.model + M_COALSTEPS, *pops = a.model + M_POPSIZES;
        int nb, nr, nc;
        lane_lineages(a.nodes, n, T, lane, nb, nr, nc);
        const int nb_prev = __shfl_up_sync(FULLMASK, nb, 1);
        double term = 0.0;
        if (lane < T - 1) {
            double tm, pm;
            if (lane == 0) {
                tm = csteps[0];
                pm = pops[0];
            } else {
                const double t1 = csteps[2 * lane - 1], t2 = csteps[2 * lane];
                const double n1 = pops[lane - 1], n2 = pops[lane];
                tm = t1 + t2;
                pm = (t1 + t2) / (t1 / n1 + t2 / n2);
            }
            const int from = lane == 0 ? a.nleaves : nb_prev;
            term = log(prob_coal_counts(from, nb, tm, 2.0 * pm));
        }
        double terms[32];
#pragma unroll
        for (int i = 0; i < 32; i++) terms[i] = __shfl_sync(FULLMASK, term, i);
        if (lane == 0) {
            double lnl = 0.0;
            for (int i = 0; i < T - 1; i++) lnl += terms[i];
            a.out[2] = lnl;
        }
    }
    if (lane == 0) {
        if (want_lik) {
            double s = 0.0;
            for (int b = 0; b < a.ntrees; b++) s += a.lik[b];
            a.out[0] = s;
        }
        if (want_prior) {
            double s = 0.0;
            for (int b = 0; b < a.ntrees; b++) s += a.prior[b];
            a.out[1] = s;
        }
    }
}

}  // namespace

int arg_probabilities(const int *ptrees, const int *ages, const int *sprs, const int *blocklens,
                      int ntrees, int nnodes, int start_coord, const double *times, int T,
                      const double *popsizes, double rho, double mu, char *const *seqs,
                      int nseqs, int seqlen, int what, double *out, std::string &err) {
    if (!ptrees || !ages || !blocklens || !times || ntrees < 1 || nnodes < 1 || T < 3 ||
        T > MAXT) {
        err = "ARG probability: bad trees or time points (3 <= ntimes <= 32)";
        return -1;
    }
    const int nleaves = (nnodes + 1) / 2;
    const bool want_lik = what & 1, want_prior = what & 2, want_tree = what & 4;
    long long total = 0;
    for (int b = 0; b < ntrees; b++) {
        if (blocklens[b] < 0) { err = "ARG probability: negative block length"; return -1; }
        total += blocklens[b];
    }
    if (want_lik) {
        if (!seqs || nseqs < nleaves || seqlen < start_coord + total || start_coord < 0) {
            err = "ARG probability: the likelihood needs one sequence per leaf covering the trees";
            return -1;
        }
    }
    if ((want_prior || want_tree) && !popsizes) {
        err = "ARG probability: the prior needs popsizes";
        return -1;
    }
    if (want_prior && ntrees > 1 && !sprs) {
        err = "ARG probability: the prior needs the SPRs";
        return -1;
    }
    // trees as {parent, child0, child1, age}, children in index order (local_tree.h:216-229)
    std::vector<int4> nodes((size_t)ntrees * nnodes);
    for (int b = 0; b < ntrees; b++) {
        const int *par = ptrees + (size_t)b * nnodes, *age = ages + (size_t)b * nnodes;
        int4 *nd = &nodes[(size_t)b * nnodes];
        for (int i = 0; i < nnodes; i++) nd[i] = make_int4(par[i], -1, -1, age[i]);
        int nroot = 0;
        for (int i = 0; i < nnodes; i++) {
            const int p = par[i];
            if (p == -1) { nroot++; continue; }
            if (p < 0 || p >= nnodes) { err = "ARG probability: parent out of range"; return -1; }
            if (nd[p].y == -1) nd[p].y = i;
            else if (nd[p].z == -1) nd[p].z = i;
            else { err = "ARG probability: a node with more than two children"; return -1; }
        }
        if (nroot != 1) { err = "ARG probability: a tree without exactly one root"; return -1; }
        for (int i = 0; i < nnodes; i++) {
            if ((nd[i].y == -1) != (i < nleaves) || (nd[i].y != -1 && nd[i].z == -1)) {
                err = "ARG probability: leaves must come first and other nodes have two children";
                return -1;
            }
            int v = i, steps = 0;  // every node reaches the root
            while (par[v] != -1 && steps <= nnodes) { v = par[v]; steps++; }
            if (steps > nnodes) { err = "ARG probability: a tree with a cycle"; return -1; }
        }
    }
    std::vector<int> bounds(ntrees + 1), last(ntrees);
    long long pos = 0;
    for (int b = 0; b < ntrees; b++) {
        bounds[b] = (int)pos;
        pos += blocklens[b];
        last[b] = (start_coord + pos < start_coord + total) ? 0 : 1;  // total_prob.cpp:276
    }
    bounds[ntrees] = (int)pos;
    std::vector<int4> spr4(ntrees, make_int4(-1, -1, -1, -1));
    if (sprs)
        for (int b = 1; b < ntrees; b++)
            spr4[b] = make_int4(sprs[4 * b], sprs[4 * b + 1], sprs[4 * b + 2], sprs[4 * b + 3]);
    if (want_prior)
        for (int b = 0; b + 1 < ntrees; b++) {
            const int4 s = spr4[b + 1];
            if (last[b]) continue;
            if (s.x < 0 || s.x >= nnodes || s.z < 0 || s.z >= nnodes || s.y < 0 || s.y >= T ||
                s.w < 0 || s.w >= T || ptrees[(size_t)b * nnodes + s.x] == -1) {
                err = "ARG probability: an SPR out of range";
                return -1;
            }
        }
    std::vector<double> model(MODEL_STRIDE);
    model_arrays(times, popsizes, T, rho, mu, 1.0, model.data());
    // site-major sequences of the trees' span
    std::vector<uint8_t> seqT;
    if (want_lik) {
        seqT.resize((size_t)total * nseqs);
        for (int j = 0; j < nseqs; j++) {
            const uint8_t *row = (const uint8_t *)seqs[j] + start_coord;
            for (long long s = 0; s < total; s++) seqT[(size_t)s * nseqs + j] = row[s];
        }
    }

    // one device allocation
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    size_t off = 0;
    const size_t o_nodes = off; off += al(sizeof(int4) * nodes.size());
    const size_t o_bounds = off; off += al(sizeof(int) * bounds.size());
    const size_t o_last = off; off += al(sizeof(int) * last.size());
    const size_t o_sprs = off; off += al(sizeof(int4) * spr4.size());
    const size_t o_model = off; off += al(sizeof(double) * model.size());
    const size_t o_seq = off; off += al(std::max<size_t>(seqT.size(), 1));
    const size_t o_lik = off; off += al(sizeof(double) * ntrees);
    const size_t o_prior = off; off += al(sizeof(double) * ntrees);
    const size_t o_out = off; off += al(sizeof(double) * 4);
    const size_t o_err = off; off += al(sizeof(int) * 2);
    char *D = nullptr;
    cudaError_t rc = cudaMalloc(&D, off);
    if (rc != cudaSuccess) {
        err = std::string("ARG probability: cudaMalloc: ") + cudaGetErrorString(rc);
        return -2;
    }
    ArgDev a;
    a.ntrees = ntrees; a.nnodes = nnodes; a.nleaves = nleaves; a.nseqs = nseqs; a.T = T;
    a.nodes = (const int4 *)(D + o_nodes);
    a.bounds = (const int *)(D + o_bounds);
    a.last = (const int *)(D + o_last);
    a.sprs = (const int4 *)(D + o_sprs);
    a.model = (const double *)(D + o_model);
    a.seqT = (const uint8_t *)(D + o_seq);
    a.lik = (double *)(D + o_lik);
    a.prior = (double *)(D + o_prior);
    a.out = (double *)(D + o_out);
    a.err = (int *)(D + o_err);
    auto up = [&](size_t o, const void *p, size_t bytes) {
        return bytes ? cudaMemcpy(D + o, p, bytes, cudaMemcpyHostToDevice) : cudaSuccess;
    };
    const size_t lik_smem = sizeof(double) * ((size_t)2 * nnodes + (size_t)LIK_WARPS * nnodes * 4) +
                            sizeof(int4) * nnodes + sizeof(int) * ((size_t)4 * nnodes + 2);
    int dev_err[2] = {0, 0};
    double res[4] = {0, 0, 0, 0};
    do {
        if ((rc = up(o_nodes, nodes.data(), sizeof(int4) * nodes.size())) != cudaSuccess) break;
        if ((rc = up(o_bounds, bounds.data(), sizeof(int) * bounds.size())) != cudaSuccess) break;
        if ((rc = up(o_last, last.data(), sizeof(int) * last.size())) != cudaSuccess) break;
        if ((rc = up(o_sprs, spr4.data(), sizeof(int4) * spr4.size())) != cudaSuccess) break;
        if ((rc = up(o_model, model.data(), sizeof(double) * model.size())) != cudaSuccess) break;
        if ((rc = up(o_seq, seqT.data(), seqT.size())) != cudaSuccess) break;
        if ((rc = cudaMemset(D + o_err, 0, sizeof(int) * 2)) != cudaSuccess) break;
        if ((rc = cudaMemset(D + o_out, 0, sizeof(double) * 4)) != cudaSuccess) break;
        if (want_lik) {
            if (lik_smem > 48 * 1024 &&
                (rc = cudaFuncSetAttribute(k_arg_likelihood<LIK_WARPS>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)lik_smem)) != cudaSuccess)
                break;
            k_arg_likelihood<LIK_WARPS><<<ntrees, LIK_THREADS, lik_smem>>>(a);
            note_launch();
            if ((rc = cudaGetLastError()) != cudaSuccess) break;
        }
        if (want_prior) {
            k_arg_prior<<<(ntrees + 3) / 4, 128>>>(a);
            note_launch();
            if ((rc = cudaGetLastError()) != cudaSuccess) break;
        }
        k_arg_totals<<<1, 32>>>(a, want_lik, want_prior, want_tree);
        note_launch();
        if ((rc = cudaGetLastError()) != cudaSuccess) break;
        if ((rc = cudaMemcpy(res, D + o_out, sizeof(res), cudaMemcpyDeviceToHost)) != cudaSuccess) break;
        rc = cudaMemcpy(dev_err, D + o_err, sizeof(dev_err), cudaMemcpyDeviceToHost);
    } while (false);
    cudaFree(D);
    if (rc != cudaSuccess) {
        err = std::string("ARG probability: ") + cudaGetErrorString(rc);
        return -3;
    }
    if (dev_err[0] != 0) {
        char b[160];
        snprintf(b, sizeof(b), "ARG probability: %s in tree %d",
                 dev_err[0] == AP_BAD_TREE ? "malformed tree (leaves must come first)"
                                           : "a site of likelihood zero",
                 dev_err[1]);
        err = b;
        return -4;
    }
    out[0] = res[0];
    out[1] = res[1];
    out[2] = res[2];
    return 0;
}

}  // namespace awg

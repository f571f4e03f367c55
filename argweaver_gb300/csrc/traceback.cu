// K4: stochastic traceback, one warp per instance (stochastic_traceback,
// sample_thread.cpp:522-569; sample_hmm_posterior :470-503; sample_hmm_posterior_step
// :506-519; sample, common.h:272-290).
//
// Column i draws path[i] from A[j] = fw[i][j] * P(j -> path[i+1]) with the uniform u[i]:
// the first j whose running sum reaches u[i] * sum(A). The warp splits the states into 32
// contiguous chunks (lane t sums chunk t with two accumulators, even and odd states); chunk
// sums are scanned across lanes and the chunk that holds the pick is rescanned by all
// lanes at once.
//
// Speculation over columns: the transition row P(. -> k) changes only when the sampled
// state does, which is rare inside a local tree. The warp therefore samples G columns at
// once under the current row, every column's sums computed exactly as if it were alone,
// and keeps the draws up to and including the first one that leaves state k; the rest are
// redone under the new row. The path is the same as one column at a time, draw for draw.
//
// The forward table is read from HBM once, newest column first: columns stream into a
// shared-memory ring DEPTH columns ahead of the sampler with 16-byte cp.async (a column's
// start is rounded down to 16 bytes and the slot keeps the offset), each column's uniform
// beside it, so HBM latency overlaps the sampling of earlier groups.

#include <cuda_runtime.h>

#include "kernels.h"

namespace awg {

namespace {

template <typename F> struct TTab;
template <> struct TTab<double> {
    static constexpr bool split = false;
    const float *rstay = nullptr;
    const double *tm, *gts, *dprob, *rrow, *crow, *fw;
    __device__ explicit TTab(const BatchDev &d)
        : tm(d.tm), gts(d.gts), dprob(d.determprob), rrow(d.recombrow), crow(d.recoalrow),
          fw(d.fw64) {}
    // same-node entry: get_time(a, b, c, minage, true)
    __device__ double same(long long idx, double) const { return gts[idx]; }
};
template <> struct TTab<float> {
    static constexpr bool split = true;  // t2d32 excludes the diagonal's stay term
    const float *rstay;
    const float *tm, *t2d, *dprob, *rrow, *crow, *fw;
    __device__ explicit TTab(const BatchDev &d)
        : rstay(d.rstay32), tm(d.tm32), t2d(d.t2d32), dprob(d.determprob32),
          rrow(d.recombrow32), crow(d.recoalrow32), fw(d.fw32) {}
    __device__ float same(long long idx, float tmab) const { return t2d[idx] + tmab; }
};

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

// Elements between a column's 16-byte-aligned start and the column itself.
template <typename F>
__device__ __forceinline__ int col_offset(const F *p) {
    return (int)(((uintptr_t)p & 15) / sizeof(F));
}

// Inclusive lane scan.
template <typename F>
__device__ __forceinline__ F lane_scan(F x, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const F v = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += v;
    }
    return x;
}

// Given the chunk sums' inclusive scan, the pick and lane t's chunk [lo, hi): the index
// the running sum first reaches the pick at (sample(), common.h:272-290), rescanning the
// chunk that holds it 32 states at a time.
template <typename F, typename W>
__device__ __forceinline__ int finish_sample(int n, int chunk, F incl, F pick, int lo, int hi,
                                             int lane, W w) {
    F excl = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) excl = 0;
    const unsigned hit = __ballot_sync(0xffffffffu, incl >= pick && hi > lo);
    if (!hit) return n - 1;
    const int src = __ffs(hit) - 1;
    const int slo = imin(src * chunk, n), shi = imin(slo + chunk, n);
    F carry = __shfl_sync(0xffffffffu, excl, src);
    int result = shi - 1;
    for (int b0 = slo; b0 < shi; b0 += 32) {
        const int jj = b0 + lane;
        const F x = lane_scan(jj < shi ? w(jj) : F(0), lane);
        const F run = carry + x;
        const unsigned got = __ballot_sync(0xffffffffu, jj < shi && run >= pick);
        if (got) {
            result = b0 + __ffs(got) - 1;
            break;
        }
        carry += __shfl_sync(0xffffffffu, x, 31);
    }
    return result;
}

// One column on its own: weights w(j), j < n.
template <typename F, typename W>
__device__ int warp_sample(int n, double u, W w) {
    const int lane = threadIdx.x & 31;
    const int chunk = (n + 31) >> 5;
    const int lo = imin(lane * chunk, n), hi = imin(lo + chunk, n);
    F l0 = 0, l1 = 0;
    int j = lo;
    for (; j + 1 < hi; j += 2) {
        l0 += w(j);
        l1 += w(j + 1);
    }
    if (j < hi) l0 += w(j);
    const F incl = lane_scan(l0 + l1, lane);
    const F total = __shfl_sync(0xffffffffu, incl, 31);
    return finish_sample<F>(n, chunk, incl, (F)u * total, lo, hi, lane, w);
}

template <typename F, int G, int DEPTH>
__global__ void k_traceback(BatchDev d, int maxS, int slot_elems) {
    extern __shared__ double dyn_d[];
    F *ring = (F *)dyn_d;                                   // [DEPTH][slot_elems], 16-B slots
    double *uring = (double *)(ring + (size_t)DEPTH * slot_elems);  // [DEPTH] uniforms
    F *trans = (F *)(uring + DEPTH);                        // [maxS]
    int *stime = (int *)(trans + maxS + (maxS & 1));        // [maxS] state times of the tree
    int *snode = stime + maxS;                              // [maxS]
    __shared__ F tmS[MAXT * MAXT];
    const TTab<F> tab(d);
    const int qi = cta_instance(d);
    const InstDev I = d.inst[qi];
    const int lane = threadIdx.x;
    int *path = d.path + I.col0;
    const double *u = d.uniforms + I.col0;
    const int L = I.seqlen;

    // prefetch cursor: next column to copy (descending), its tree's fields in registers
    int pcol = L - 1, pblk = I.ntrees - 1;
    int pS = imax(d.blocks[I.block0 + pblk].S, 1), pstart = d.blocks[I.block0 + pblk].start;
    long long pcell = d.blocks[I.block0 + pblk].cell0;
    auto issue = [&]() {
        if (pcol >= 0) {
            const F *src = tab.fw + pcell + (size_t)(pcol - pstart) * pS;
            const char *a16 = (const char *)((uintptr_t)src & ~(uintptr_t)15);
            const int nbytes = (int)((const char *)(src + pS) - a16);
            char *dst = (char *)(ring + (size_t)(pcol % DEPTH) * slot_elems);
            for (int q = lane; q * 16 < nbytes; q += 32) cp_async16(dst + q * 16, a16 + q * 16);
            if (lane == 0) cp_async8(uring + pcol % DEPTH, u + pcol);
            pcol--;
            if (pblk > 0 && pcol < pstart) {
                pblk--;
                pS = imax(d.blocks[I.block0 + pblk].S, 1);
                pstart = d.blocks[I.block0 + pblk].start;
                pcell = d.blocks[I.block0 + pblk].cell0;
            }
        }
        cp_commit();  // one group per column, empty ones included
    };
    // Invariant: before a group starting at column c0 is sampled, columns c0 .. c0-DEPTH+1
    // have been issued, one commit group each, oldest first.
    for (int q = 0; q < DEPTH; q++) issue();

    // a column's values in its ring slot
    auto column = [&](const BlockDev &B, int col) -> const F * {
        const int Sm = imax(B.S, 1);
        const F *g = tab.fw + B.cell0 + (size_t)(col - B.start) * Sm;
        return ring + (size_t)(col % DEPTH) * slot_elems + col_offset(g);
    };

    int col = L - 1;
    int state;  // path[col + 1] of the column being sampled
    // last column (sample_thread.cpp:534-539)
    {
        const BlockDev &Bl = d.blocks[I.block0 + I.ntrees - 1];
        cp_wait<DEPTH - 1>();
        __syncwarp();
        const F *c = column(Bl, col);
        const int x = warp_sample<F>(imax(Bl.S, 1), uring[col % DEPTH], [&](int j) { return c[j]; });
        if (lane == 0) path[col] = x;
        state = x;
        __syncwarp();
        issue();
    }
    for (int bi = I.ntrees - 1; bi >= 0; bi--) {
        const int blk = I.block0 + bi;
        const BlockDev B = d.blocks[blk];
        const int S = B.S, Sm = imax(S, 1);
        const int chunk = (Sm + 31) >> 5;
        const int lo = imin(lane * chunk, Sm), hi = imin(lo + chunk, Sm);
        // stage the tree's state times/nodes and tmatrix
        for (int j = lane; j < S; j += 32) {
            const StateInfo si = d.sinfo[B.state0 + j];
            stime[j] = si.time;
            snode[j] = si.node;
        }
        const F *tmg = tab.tm + (size_t)blk * MAXT * MAXT;
        for (int e = lane; e < (I.T - 1) * MAXT; e += 32) tmS[e] = tmg[e];
        __syncwarp();
        // trans[j] = TransMatrix::get(j, k) (trans.h:64-83)
        auto build_row = [&](int k) {
            if (S == 0) {
                if (lane == 0) trans[0] = F(1);
            } else {
                const StateInfo sk = d.sinfo[B.state0 + k];
                const long long row = B.t2_0 + d.t2off[B.state0 + k];
                const F stay = TTab<F>::split ? F(1) - tab.rstay[(size_t)blk * MAXT + sk.time] : F(0);
                for (int j = lane; j < S; j += 32) {
                    const F tmab = tmS[stime[j] * MAXT + sk.time];
                    F t = tmab;
                    if (snode[j] == sk.node) {
                        t = tab.same(row + (long long)(j - sk.j1) * sk.m, tmab);
                        if (j == k) t += stay;
                    }
                    trans[j] = t;
                }
            }
            __syncwarp();
        };
        build_row(state);

        // within the tree: columns B.start + B.len - 2 down to B.start, G at a time
        int c0 = B.start + B.len - 2;
        while (c0 >= B.start) {
            const int ng = imin(G, c0 - B.start + 1);
            cp_wait<DEPTH - G>();
            __syncwarp();
            const F *cg[G];
#pragma unroll
            for (int g = 0; g < G; g++) cg[g] = column(B, c0 - imin(g, ng - 1));
            // every column's chunk sums under the current row, as warp_sample forms them
            F l0[G], l1[G];
#pragma unroll
            for (int g = 0; g < G; g++) l0[g] = l1[g] = F(0);
            int j = lo;
            for (; j + 1 < hi; j += 2) {
                const F t0 = trans[j], t1 = trans[j + 1];
#pragma unroll
                for (int g = 0; g < G; g++) {
                    l0[g] += cg[g][j] * t0;
                    l1[g] += cg[g][j + 1] * t1;
                }
            }
            if (j < hi) {
                const F t0 = trans[j];
#pragma unroll
                for (int g = 0; g < G; g++) l0[g] += cg[g][j] * t0;
            }
            F incl[G];
#pragma unroll
            for (int g = 0; g < G; g++) incl[g] = l0[g] + l1[g];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
                for (int g = 0; g < G; g++) {
                    const F v = __shfl_up_sync(0xffffffffu, incl[g], o);
                    if (lane >= o) incl[g] += v;
                }
            }
            // every column's draw, all G interleaved (finish_sample's steps, column-wise)
            F pick[G], carry[G];
            int slo[G], shi[G], res[G];
#pragma unroll
            for (int g = 0; g < G; g++) {
                F excl = __shfl_up_sync(0xffffffffu, incl[g], 1);
                if (lane == 0) excl = 0;
                const F total = __shfl_sync(0xffffffffu, incl[g], 31);
                pick[g] = (F)uring[(c0 - imin(g, ng - 1)) % DEPTH] * total;
                const unsigned hit = __ballot_sync(0xffffffffu, incl[g] >= pick[g] && hi > lo);
                const int src = hit ? __ffs(hit) - 1 : 0;
                slo[g] = imin(src * chunk, Sm);
                shi[g] = hit ? imin(slo[g] + chunk, Sm) : slo[g];  // empty: no rescan
                carry[g] = __shfl_sync(0xffffffffu, excl, src);
                res[g] = hit ? shi[g] - 1 : Sm - 1;
            }
            unsigned open = 0;  // columns whose pick is not found yet
#pragma unroll
            for (int g = 0; g < G; g++)
                if (shi[g] > slo[g]) open |= 1u << g;
            for (int b = 0; open; b += 32) {
                F x[G];
#pragma unroll
                for (int g = 0; g < G; g++) {
                    const int jj = slo[g] + b + lane;
                    x[g] = ((open >> g) & 1) && jj < shi[g] ? cg[g][jj] * trans[jj] : F(0);
                }
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
                    for (int g = 0; g < G; g++) {
                        const F v = __shfl_up_sync(0xffffffffu, x[g], o);
                        if (lane >= o) x[g] += v;
                    }
                }
#pragma unroll
                for (int g = 0; g < G; g++) {
                    if (!((open >> g) & 1)) continue;
                    const int jj = slo[g] + b + lane;
                    const unsigned got =
                        __ballot_sync(0xffffffffu, jj < shi[g] && carry[g] + x[g] >= pick[g]);
                    if (got) {
                        res[g] = slo[g] + b + __ffs(got) - 1;
                        open &= ~(1u << g);
                    } else {
                        carry[g] += __shfl_sync(0xffffffffu, x[g], 31);
                        if (slo[g] + b + 32 >= shi[g]) open &= ~(1u << g);
                    }
                }
            }
            // keep the draws in column order up to the first that leaves the current state
            int r = 0, x = state;
#pragma unroll
            for (int g = 0; g < G; g++) {
                if (g < ng && x == state) {
                    x = res[g];
                    if (lane == 0) path[c0 - g] = x;
                    r = g + 1;
                }
            }
            __syncwarp();
            for (int q = 0; q < r; q++) issue();
            c0 -= r;
            if (x != state) {
                state = x;
                build_row(state);
            }
        }
        if (bi > 0) {
            // switch into this tree (sample_hmm_posterior_step)
            col = B.start - 1;
            const BlockDev &P = d.blocks[blk - 1];
            const int k = state;
            const int n1 = imax(B.S1, 1);
            const int2 src = d.srcs[blk];
            const int *determ = d.determ + B.prev_state0;
            const F *dp = tab.dprob + B.prev_state0;
            const F rr = tab.rrow[B.state0 + k], cr = tab.crow[B.state0 + k];
            cp_wait<DEPTH - 1>();
            __syncwarp();
            const F *c = column(P, col);
            auto w = [&](int j) -> F {
                F g;
                if (j == src.y) g = cr;
                else if (j == src.x) g = rr;
                else g = (determ[j] == k) ? dp[j] : F(0);
                return c[j] * g;
            };
            const int x = warp_sample<F>(n1, uring[col % DEPTH], w);
            if (lane == 0) path[col] = x;
            state = x;
            __syncwarp();
            issue();
        }
    }
    cp_wait<0>();
}

template <typename F, int G, int DEPTH>
bool launch_cfg(const BatchDev &d, cudaStream_t s, size_t budget) {
    const int maxS = imax(d.maxS, 1);
    const int slot_elems = (int)(((size_t)maxS * sizeof(F) + 32 + 15) / 16 * 16 / sizeof(F));
    const size_t smem = (size_t)DEPTH * slot_elems * sizeof(F) + DEPTH * sizeof(double) +
                        (size_t)(maxS + 1) * sizeof(F) + 2 * (size_t)maxS * sizeof(int) + 16;
    if (smem > budget) return false;
    static size_t configured = 0;
    if (smem > configured) {  // opt in; static shared memory counts against 48 KB too
        if (cudaFuncSetAttribute(k_traceback<F, G, DEPTH>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return true;  // the launch reports the error
        configured = smem;
    }
    k_traceback<F, G, DEPTH><<<d.ninst, 32, smem, s>>>(d, maxS, slot_elems);
    note_launch();
    return true;
}

template <typename F>
void launch(const BatchDev &d, cudaStream_t s) {
    // the deepest speculation whose ring leaves room for two CTAs per SM, else one
    constexpr size_t two = 100 * 1024, one = 200 * 1024;
    if (launch_cfg<F, 8, 24>(d, s, two)) return;
    if (launch_cfg<F, 4, 12>(d, s, two)) return;
    if (launch_cfg<F, 4, 12>(d, s, one)) return;
    if (launch_cfg<F, 2, 6>(d, s, one)) return;
    launch_cfg<F, 1, 3>(d, s, 227 * 1024);
}

}  // namespace

void launch_traceback(const BatchDev &d, bool fp32, cudaStream_t s) {
    if (fp32) launch<float>(d, s);
    else launch<double>(d, s);
}

}  // namespace awg

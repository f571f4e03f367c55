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

// QL: four lanes per column (G = 8): lane 4g + q runs quarter q of column g's states in
// order, keeping each running sum in shared memory, so that a column's draw needs a 4-lane
// scan and a binary search of the stored sums instead of a 32-lane scan and a rescan; the
// fewer warp-wide FP64 instructions suit the FP64 path, whose every warp instruction holds
// the sub-partition's FP64 pipe for about 64 cycles. For trees of up to QL_MAXS states.
constexpr int QL_MAXS = 256;

// The order of non-negative values as integers (their bit patterns order the same way).
__device__ __forceinline__ long long order_key(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ long long order_key(float x) { return __float_as_int(x); }

template <typename F, int G, int DEPTH, bool QL>
__global__ void k_traceback(BatchDev d, int maxS, int slot_elems) {
    extern __shared__ double dyn_d[];
    F *ring = (F *)dyn_d;                                   // [DEPTH][slot_elems], 16-B slots
    double *uring = (double *)(ring + (size_t)DEPTH * slot_elems);  // [DEPTH] uniforms
    F *trans = (F *)(uring + DEPTH);                        // [maxS]
    int *stime = (int *)(trans + maxS + (maxS & 1));        // [maxS] state times of the tree
    int *snode = stime + maxS;                              // [maxS]
    // QL: [G][maxS + 1] running sums (after the ints, 8-byte aligned)
    F *pre = (F *)((char *)dyn_d + (((char *)(snode + maxS) - (char *)dyn_d + 15) & ~(size_t)15));
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
        // a given last state (conditioned sampling) takes no draw
        const int given = d.last_state ? d.last_state[qi] : -1;
        const int x = given >= 0 ? given
                                 : warp_sample<F>(imax(Bl.S, 1), uring[col % DEPTH], [&](int j) { return c[j]; });
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
            int res[G];
            if constexpr (QL) {
                static_assert(G == 8, "four lanes per column of eight");
                const int g = lane >> 2, q = lane & 3;
                const int qs = (Sm + 3) >> 2;
                const int qlo = imin(q * qs, Sm), qhi = imin(qlo + qs, Sm);
                const int mycol = c0 - imin(g, ng - 1);
                const F *cp = column(B, mycol);
                F *pg = pre + g * (maxS + 1);
                F run = 0;
                for (int j = qlo; j < qhi; j++) {
                    run = fma(cp[j], trans[j], run);
                    pg[j] = run;
                }
                // inclusive scan of the quarters' sums within the column's four lanes
                F incl = run;
                F v = __shfl_up_sync(0xffffffffu, incl, 1);
                if (q >= 1) incl += v;
                v = __shfl_up_sync(0xffffffffu, incl, 2);
                if (q >= 2) incl += v;
                F excl = __shfl_up_sync(0xffffffffu, incl, 1);
                if (q == 0) excl = 0;
                const F total = __shfl_sync(0xffffffffu, incl, lane | 3);
                const F pick = (F)uring[mycol % DEPTH] * total;
                const unsigned hit = __ballot_sync(0xffffffffu, incl >= pick && qhi > qlo);
                __syncwarp();  // the running sums are stored
                int mine = Sm - 1;
                const unsigned gh = (hit >> (4 * g)) & 15u;
                if (gh && q == __ffs(gh) - 1) {
                    // the first state whose running sum reaches the pick: stored sum >=
                    // pick - (the sums of the quarters before); none (rounding): the
                    // quarter's last state
                    const long long key = order_key(pick - excl);
                    int a = qlo, b = qhi - 1;
                    if (order_key(pg[b]) >= key) {
                        while (a < b) {
                            const int mid = (a + b) >> 1;
                            if (order_key(pg[mid]) >= key) b = mid;
                            else a = mid + 1;
                        }
                    }
                    mine = b;
                }
#pragma unroll
                for (int gg = 0; gg < G; gg++) {
                    const unsigned hq = (hit >> (4 * gg)) & 15u;
                    const int src = hq ? 4 * gg + __ffs(hq) - 1 : 4 * gg;
                    const int r = __shfl_sync(0xffffffffu, mine, src);
                    res[gg] = hq ? r : Sm - 1;
                }
            } else {
            // every column's chunk sums under the current row, as warp_sample forms them
            F l0[G], l1[G];
#pragma unroll
            for (int g = 0; g < G; g++) l0[g] = l1[g] = F(0);
            int j = lo;
            for (; j + 1 < hi; j += 2) {
                const F t0 = trans[j], t1 = trans[j + 1];
#pragma unroll
                for (int g = 0; g < G; g++) {
                    l0[g] = fma(cg[g][j], t0, l0[g]);
                    l1[g] = fma(cg[g][j + 1], t1, l1[g]);
                }
            }
            if (j < hi) {
                const F t0 = trans[j];
#pragma unroll
                for (int g = 0; g < G; g++) l0[g] = fma(cg[g][j], t0, l0[g]);
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
            int slo[G], shi[G];
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
            if (chunk <= 16) {
                // short chunks: lane g rescans column g's chosen chunk in order, one product
                // and one add per state, the G columns side by side (a 32-lane scan per column
                // costs five warp-wide adds however few states the chunk holds: on the FP64
                // path each holds the sub-partition's FP64 pipe for about 64 cycles)
                int mine = 0;
                if (lane < G) {
                    F mpick = 0, run = 0;
                    int mslo = 0, mshi = 0;
                    const F *mc = cg[0];
#pragma unroll
                    for (int g = 0; g < G; g++)
                        if (lane == g) {
                            mpick = pick[g];
                            run = carry[g];
                            mslo = slo[g];
                            mshi = (open >> g) & 1 ? shi[g] : slo[g];
                            mine = res[g];
                            mc = cg[g];
                        }
                    for (int jj = mslo; jj < mshi; jj++) {
                        run += mc[jj] * trans[jj];
                        if (run >= mpick) {
                            mine = jj;
                            break;
                        }
                    }
                }
#pragma unroll
                for (int g = 0; g < G; g++) res[g] = __shfl_sync(0xffffffffu, mine, g);
                open = 0;
            }
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

// ---------------------------------------------------------------------------------------
// FP32 path: the draw decomposed by the structure of the transition.
//
// Inside a tree P(j -> k) = tm[a_j][b_k] + [node_j = node_k] tm2[a_j][k] (the structured
// step of arghmm_forward_block, sample_thread.cpp:255-290; tm2 >= 0 is the same-branch
// excess, the no-recombination stay included on the diagonal). Column i's weights
// fw[i][j] P(j -> k) thus split into the same-branch part V_y = fw[i][j1 + y] tm2[a_y][k]
// over the m states of k's node, and a background part whose total over the states of
// time bin a is W_a = bins[i][a] tm[a][b_k], bins[i] being the stored column's time-bin
// sums that the forward kernel writes. With t = u (V + W): if t <= V the draw is the first
// y whose running V sum reaches t; else the first bin whose running W sum reaches t - V,
// then the first state of that bin (states of a bin in time-sorted order) whose running
// fw sum reaches the remainder over tm[a][b_k]. This draws from exactly the distribution
// of the reference's scan over all states (sample(), common.h:272-290), mapping the
// uniform to states in another order, with O(T + m) work per column instead of O(S).
// At a tree switch only the sources with a nonzero switch probability into the drawn
// state carry weight (its gather list plus the recombination and recoalescence sources),
// so the switch draw runs over those, in state order.
//
// Speculation: the warp tests 8 columns at once for the common case, the draw staying at
// the current state k: lanes 4g .. 4g+3 take column g, each a quarter of the node's states
// and of the bins, and combine V before k, V at k, V and W by two butterfly steps. The
// first column whose draw leaves k (if any) is drawn exactly by the whole warp; the
// columns after it are tested again under the new state.
//
// Data movement is TMA bulk copies (cp.async.bulk) completing on mbarriers, issued by one
// lane: the forward table streams into a ring of NCH chunks of up to 8 consecutive columns
// of one tree (one copy for the chunk's columns, one for their bins, one for their
// uniforms), and each tree's tables (tmatrix, stay complements, time-bin CSR, state info,
// row offsets, switch gather lists and probabilities) into one of two buffers one tree
// ahead. Every wait is bounded; one that runs out records ERR_WAIT_LIMIT and the kernel
// returns after its copies have landed.

__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
// Global -> shared bulk copy: both addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
constexpr int WAIT_TRIES = 1 << 22;  // try_wait rounds before a wait gives up
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity) {
    for (int it = 0; it < WAIT_TRIES; it++)
        if (mbar_test(bar, parity)) return true;
    return false;
}

// count elements of ESZ bytes at p, copied from the 16-byte boundary below p: the bytes to
// copy (a multiple of 16) and the element offset of p inside the copy.
template <int ESZ>
struct Rounded {
    const char *a16;
    unsigned bytes;
    int off;
    __device__ __forceinline__ Rounded(const void *p, long long count) {
        a16 = (const char *)((uintptr_t)p & ~(uintptr_t)15);
        off = (int)(((uintptr_t)p & 15) / ESZ);
        bytes = count > 0 ? (unsigned)(((const char *)p + ESZ * count - a16 + 15) & ~(long long)15) : 0u;
    }
};

// Fields of a tree the traceback needs, in registers.
struct TreeRef {
    int blk, start, len, S, S1;
    long long cell0, state0, prev_state0, t2_0, gptr0;
};
__device__ __forceinline__ TreeRef tree_ref(const BatchDev &d, int blk) {
    const BlockDev &B = d.blocks[blk];
    return TreeRef{blk, B.start, B.len, B.S, B.S1, B.cell0, B.state0, B.prev_state0, B.t2_0, B.gptr0};
}

// Layout of one tree buffer (bytes from its start; every part 16-byte aligned).
struct TreeBufLayout {
    int tm, rstay, bptr, sinfo, t2off, perm, gptr, gidx, dp, total;
    __host__ __device__ explicit TreeBufLayout(int maxS) {
        const int arr = (4 * maxS + 32 + 15) & ~15;  // a 4-byte array copied from its 16-B start
        tm = 0;
        rstay = tm + 4 * MAXT * MAXT;
        bptr = rstay + 4 * MAXT;
        sinfo = bptr + 160;
        t2off = sinfo + 16 * maxS;
        perm = t2off + arr;
        gptr = perm + arr;
        gidx = gptr + arr;
        dp = gidx + arr;
        total = dp + arr;
    }
};

constexpr int CW = 8;  // columns per ring chunk (= the speculation group)

// Bytes of one ring chunk's table part.
__host__ __device__ inline int chunk_tab_bytes(int maxS) { return (4 * CW * maxS + 32 + 15) & ~15; }

template <int NCH>
__global__ void __launch_bounds__(32) k_traceback_split(BatchDev d, int maxS) {
    constexpr int G = CW;
    constexpr unsigned FULL = 0xffffffffu;
    extern __shared__ __align__(16) unsigned char dyn_b[];
    const int tab_bytes = chunk_tab_bytes(maxS);
    unsigned char *rtab = dyn_b;                                     // [NCH] table chunks
    float *rbins = (float *)(rtab + (size_t)NCH * tab_bytes);        // [NCH][CW][MAXT]
    double *ru = (double *)(rbins + NCH * CW * MAXT);                // [NCH][CW + 2]
    unsigned char *tbuf = (unsigned char *)(ru + NCH * (CW + 2));    // [2] tree buffers
    __shared__ uint64_t cbar[NCH];                                   // chunk barriers
    __shared__ uint64_t tbar[2];                                     // tree buffer barriers
    __shared__ int ch_lo[NCH], ch_cnt[NCH], ch_off[NCH], ch_uoff[NCH], ch_S[NCH];
    __shared__ float t2row[32], tmcol[32];                           // the state's V, W factors
    const TreeBufLayout TL(maxS);
    const TTab<float> tab(d);
    const int qi = cta_instance(d);
    const InstDev I = d.inst[qi];
    const int lane = threadIdx.x;
    const int NB = I.T - 1;
    int *path = d.path + I.col0;
    const double *u = d.uniforms + I.col0;
    const float *bins = d.bins32 + (size_t)I.col0 * MAXT;
    const int L = I.seqlen;
    bool failed = false;

    if (lane == 0) {
        for (int q = 0; q < NCH; q++) mbar_init(&cbar[q], 1);
        mbar_init(&tbar[0], 1);
        mbar_init(&tbar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncwarp();

    // ---- chunk ring: chunk m in slot m % NCH, phase (m / NCH) & 1; chunks hold columns in
    // descending order of their highest column, never across a tree start
    int pcol = L - 1, pblk = I.ntrees - 1;
    TreeRef pc = tree_ref(d, I.block0 + pblk);
    TreeRef pn = pblk > 0 ? tree_ref(d, I.block0 + pblk - 1) : pc;  // the cursor's next tree
    int issued = 0, waited = 0, mc = 0;  // chunks issued, complete, oldest in use
    auto issue = [&]() {
        if (pcol < 0) return;
        const int cnt = imin(CW, pcol - pc.start + 1), lo = pcol - cnt + 1;
        const int slot = issued % NCH;
        const int Sm = imax(pc.S, 1);
        __syncwarp();  // the slot's previous chunk is no longer read
        if (lane == 0) {
            const Rounded<4> rt(tab.fw + pc.cell0 + (size_t)(lo - pc.start) * Sm, (long long)cnt * Sm);
            const Rounded<8> ru8(u + lo, cnt);
            ch_lo[slot] = lo;
            ch_cnt[slot] = cnt;
            ch_off[slot] = rt.off;
            ch_uoff[slot] = ru8.off;
            ch_S[slot] = Sm;
            mbar_expect_tx(&cbar[slot], rt.bytes + 4u * MAXT * cnt + ru8.bytes);
            bulk_g2s(rtab + (size_t)slot * tab_bytes, rt.a16, rt.bytes, &cbar[slot]);
            bulk_g2s(rbins + slot * CW * MAXT, bins + (size_t)lo * MAXT, 4u * MAXT * cnt, &cbar[slot]);
            bulk_g2s(ru + slot * (CW + 2), ru8.a16, ru8.bytes, &cbar[slot]);
        }
        __syncwarp();
        issued++;
        pcol = lo - 1;
        if (pblk > 0 && pcol < pc.start) {
            pblk--;
            pc = pn;
            if (pblk > 0) pn = tree_ref(d, I.block0 + pblk - 1);
        }
    };
    // chunk index of column c: mc, or mc + 1 when c lies below chunk mc
    auto chunk_of = [&](int c) { return c >= ch_lo[mc % NCH] ? mc : mc + 1; };
    auto ensure = [&](int m) -> bool {  // chunks up to m have landed
        bool ok = true;
        while (waited <= m && ok) {
            ok = mbar_wait(&cbar[waited % NCH], (unsigned)((waited / NCH) & 1));
            waited++;
        }
        return ok;
    };
    auto column = [&](int c) -> const float * {
        const int s = chunk_of(c) % NCH;
        return (const float *)(rtab + (size_t)s * tab_bytes) + ch_off[s] + (size_t)(c - ch_lo[s]) * ch_S[s];
    };
    auto colbins = [&](int c) -> const float * {
        const int s = chunk_of(c) % NCH;
        return rbins + (s * CW + (c - ch_lo[s])) * MAXT;
    };
    auto uniform = [&](int c) -> double {
        const int s = chunk_of(c) % NCH;
        return ru[s * (CW + 2) + ch_uoff[s] + (c - ch_lo[s])];
    };
    // columns >= c consumed: release the chunks wholly above c (each landed first, so its
    // barrier phase is complete before the slot is issued again) and issue new ones
    auto consumed_to = [&](int c) {
        while (mc < issued && ch_lo[mc % NCH] >= c) {
            failed |= !ensure(mc);
            mc++;
            issue();
        }
    };

    // ---- tree buffers: tree x in buffer x & 1
    unsigned tphase[2] = {0u, 0u};
    bool tpend[2] = {false, false};  // staged, not yet waited for
    __shared__ int o_t2off[2], o_perm[2], o_gptr[2], o_gidx[2], o_dp[2], o_bptr[2];
    auto stage = [&](const TreeRef &X) {
        const int b = X.blk & 1;
        unsigned char *base = tbuf + (size_t)b * TL.total;
        const int S = X.S, S1 = imax(X.S1, 1);
        const bool sw = X.start > 0;  // a switch into this tree exists
        const Rounded<4> rb(d.bt_ptr + (size_t)X.blk * (MAXT + 1), MAXT + 1);
        const Rounded<4> rt(d.t2off + X.state0, S);
        const Rounded<4> rp(d.bt_perm + X.state0, S);
        const Rounded<4> rg(d.gptr + X.gptr0, imax(S, 1) + 1);
        const Rounded<4> ri(d.gidx + X.prev_state0, S1);
        const Rounded<4> rq(tab.dprob + X.prev_state0, S1);
        tpend[b] = true;
        __syncwarp();
        if (lane == 0) {
            o_bptr[b] = rb.off;
            o_t2off[b] = rt.off;
            o_perm[b] = rp.off;
            o_gptr[b] = rg.off;
            o_gidx[b] = ri.off;
            o_dp[b] = rq.off;
            const unsigned tmb = 4u * MAXT * (unsigned)NB;
            const unsigned tx = (S > 0 ? tmb + 4 * MAXT + rb.bytes + 16u * S + rt.bytes + rp.bytes : 0u) +
                                (sw ? rg.bytes + ri.bytes + rq.bytes : 0u);
            mbar_expect_tx(&tbar[b], tx);
            if (S > 0) {
                bulk_g2s(base + TL.tm, tab.tm + (size_t)X.blk * MAXT * MAXT, tmb, &tbar[b]);
                bulk_g2s(base + TL.rstay, tab.rstay + (size_t)X.blk * MAXT, 4 * MAXT, &tbar[b]);
                bulk_g2s(base + TL.bptr, rb.a16, rb.bytes, &tbar[b]);
                bulk_g2s(base + TL.sinfo, d.sinfo + X.state0, 16u * S, &tbar[b]);
                bulk_g2s(base + TL.t2off, rt.a16, rt.bytes, &tbar[b]);
                bulk_g2s(base + TL.perm, rp.a16, rp.bytes, &tbar[b]);
            }
            if (sw) {
                bulk_g2s(base + TL.gptr, rg.a16, rg.bytes, &tbar[b]);
                bulk_g2s(base + TL.gidx, ri.a16, ri.bytes, &tbar[b]);
                bulk_g2s(base + TL.dp, rq.a16, rq.bytes, &tbar[b]);
            }
        }
        __syncwarp();
    };
    auto wait_tree = [&](int blk) -> bool {
        const int b = blk & 1;
        const bool ok = mbar_wait(&tbar[b], tphase[b]);
        tphase[b] ^= 1u;
        tpend[b] = false;
        return ok;
    };

    for (int q = 0; q < NCH; q++) issue();
    TreeRef cur = tree_ref(d, I.block0 + I.ntrees - 1);
    TreeRef nx1 = I.ntrees > 1 ? tree_ref(d, I.block0 + I.ntrees - 2) : cur;
    stage(cur);

    int state;
    {
        const int col = L - 1;
        failed |= !ensure(chunk_of(col));
        __syncwarp();
        const float *c = column(col);
        const int x = warp_sample<float>(imax(cur.S, 1), uniform(col), [&](int j) { return c[j]; });
        if (lane == 0) path[col] = x;
        state = x;
        __syncwarp();
        consumed_to(col);
    }
    const int g = lane >> 2, sub = lane & 3;  // fast path: column g of a group, quarter sub
    for (int bi = I.ntrees - 1; bi >= 0 && !failed; bi--) {
        const TreeRef B = cur;
        const int b = B.blk & 1;
        const unsigned char *base = tbuf + (size_t)b * TL.total;
        failed |= !wait_tree(B.blk);
        __syncwarp();
        // tables of the next tree, while this one is sampled
        TreeRef nx2 = nx1;
        if (bi > 0) {
            stage(nx1);
            if (bi > 1) nx2 = tree_ref(d, I.block0 + bi - 2);
        }
        const float *tmS = (const float *)(base + TL.tm);
        const float *rst = (const float *)(base + TL.rstay);
        const int *bptr = (const int *)(base + TL.bptr) + o_bptr[b];
        const StateInfo *sinfo = (const StateInfo *)(base + TL.sinfo);
        const int *t2off = (const int *)(base + TL.t2off) + o_t2off[b];
        const int *perm = (const int *)(base + TL.perm) + o_perm[b];
        const int S = B.S;
        int c0 = B.start + B.len - 2;
        if (S == 0) {
            // fully specified tree: its single state carries over
            for (; c0 >= B.start; c0--)
                if (lane == 0) path[c0] = 0;
            if (B.len > 1) consumed_to(B.start);
        } else {
            int kj1 = 0, km = 0, ys = 0;
            float t2r[8], tmr[8];
            auto set_state = [&](int k) {
                const StateInfo sk = sinfo[k];
                kj1 = sk.j1;
                km = sk.m;
                ys = k - sk.j1;
                const long long row = B.t2_0 + t2off[k];
                const float stay = 1.0f - rst[sk.time];
                __syncwarp();
                t2row[lane] = lane < km ? tab.t2d[row + (long long)lane * km] + (lane == ys ? stay : 0.0f) : 0.0f;
                tmcol[lane] = lane < NB ? tmS[lane * MAXT + sk.time] : 0.0f;
                __syncwarp();
#pragma unroll
                for (int q = 0; q < 8; q++) {
                    t2r[q] = t2row[8 * sub + q];
                    tmr[q] = tmcol[8 * sub + q];
                }
            };
            set_state(state);
            while (c0 >= B.start && !failed) {
                const int ng = imin(G, c0 - B.start + 1);
                const int cg = c0 - imin(g, ng - 1);
                failed |= !ensure(chunk_of(c0 - ng + 1));
                __syncwarp();
                if (failed) break;
                // fast path: does column g's draw stay at the current state?
                const float *cp = column(cg);
                const float *bp = colbins(cg);
                float sb = 0.0f, ss = 0.0f, sa = 0.0f, sw = 0.0f;
#pragma unroll
                for (int q = 0; q < 8; q++) {
                    const int y = 8 * sub + q;
                    const float v = y < km ? cp[kj1 + y] * t2r[q] : 0.0f;
                    sa += v;
                    sb += y < ys ? v : 0.0f;
                    ss += y == ys ? v : 0.0f;
                    sw += y < NB ? bp[y] * tmr[q] : 0.0f;
                }
#pragma unroll
                for (int o = 1; o < 4; o <<= 1) {
                    sb += __shfl_xor_sync(FULL, sb, o);
                    ss += __shfl_xor_sync(FULL, ss, o);
                    sa += __shfl_xor_sync(FULL, sa, o);
                    sw += __shfl_xor_sync(FULL, sw, o);
                }
                const float t = (float)uniform(cg) * (sa + sw);
                const bool stay = (ys == 0 || sb < t) && t <= sb + ss;
                const unsigned leave = __ballot_sync(FULL, sub == 0 && g < ng && !stay);
                const int nstay = leave ? (__ffs(leave) - 1) >> 2 : ng;
                if (sub == 0 && g < nstay) path[c0 - g] = state;
                int x = state;
                if (leave) {
                    // exact draw of the first column that leaves, by the whole warp
                    const int cs = c0 - nstay;
                    const float *cq = column(cs);
                    const float *bq = colbins(cs);
                    const float v = lane < km ? cq[kj1 + lane] * t2row[lane] : 0.0f;
                    const float w = lane < NB ? bq[lane] * tmcol[lane] : 0.0f;
                    const float vin = lane_scan(v, lane), win = lane_scan(w, lane);
                    const float vt = __shfl_sync(FULL, vin, 31), wt = __shfl_sync(FULL, win, 31);
                    const float tt = (float)uniform(cs) * (vt + wt);
                    if (tt <= vt) {
                        const unsigned hit = __ballot_sync(FULL, lane < km && vin >= tt);
                        x = kj1 + (hit ? __ffs(hit) - 1 : km - 1);
                    } else {
                        const float t2 = tt - vt;
                        const unsigned hit = __ballot_sync(FULL, lane < NB && win >= t2);
                        const unsigned pos = __ballot_sync(FULL, w > 0.0f);
                        const int a = hit ? __ffs(hit) - 1 : (pos ? 31 - __clz(pos) : 0);
                        const float excl = __shfl_sync(FULL, win - w, a);
                        const float r = (t2 - excl) / tmcol[a];  // threshold on the fw scale
                        const int p0 = bptr[a], p1 = bptr[a + 1];
                        float carry = 0.0f;
                        int res = -1, last = p0;
                        for (int pb = p0; pb < p1; pb += 32) {
                            const int pp = pb + lane;
                            const float f = pp < p1 ? cq[perm[pp]] : 0.0f;
                            const float fin = lane_scan(f, lane);
                            const unsigned got = __ballot_sync(FULL, pp < p1 && carry + fin >= r);
                            const unsigned nz = __ballot_sync(FULL, pp < p1 && f > 0.0f);
                            if (nz) last = pb + 31 - __clz(nz);
                            if (got) {
                                res = pb + __ffs(got) - 1;
                                break;
                            }
                            carry += __shfl_sync(FULL, fin, 31);
                        }
                        // past the bin's sum by rounding: its last state of positive weight
                        x = res >= 0 ? perm[res] : (p1 > p0 ? perm[last] : state);
                    }
                    if (lane == 0) path[cs] = x;
                }
                __syncwarp();
                const int r = leave ? nstay + 1 : nstay;
                c0 -= r;
                consumed_to(c0 + 1);
                if (x != state) {
                    state = x;
                    set_state(state);
                }
            }
        }
        if (bi > 0 && !failed) {
            // switch into this tree (sample_hmm_posterior_step): sources in state order,
            // the gather list of the drawn state merged with the recombination and
            // recoalescence sources
            const int col = B.start - 1;
            const int k = state;
            const int2 src = d.srcs[B.blk];
            const int *gp = (const int *)(base + TL.gptr) + o_gptr[b];
            const int *gi = (const int *)(base + TL.gidx) + o_gidx[b];
            const float *dp = (const float *)(base + TL.dp) + o_dp[b];
            const float rr = tab.rrow[B.state0 + k], cr = tab.crow[B.state0 + k];
            failed |= !ensure(chunk_of(col));
            __syncwarp();
            if (!failed) {
                const float *c = column(col);
                const int p0 = gp[k], ng2 = gp[k + 1] - p0;
                int x = 0;
                if (lane == 0) {
                    // the two extra sources in state order (get(): recoalescence wins a tie)
                    int e0 = -1, e1 = -1;
                    float w0 = 0.0f, w1 = 0.0f;
                    if (src.x >= 0 && src.x != src.y) { e0 = src.x; w0 = rr; }
                    if (src.y >= 0) {
                        if (e0 < 0) { e0 = src.y; w0 = cr; }
                        else if (src.y < e0) { e1 = e0; w1 = w0; e0 = src.y; w0 = cr; }
                        else { e1 = src.y; w1 = cr; }
                    }
                    // merged walk of the gather list and the extras: pass 0 sums, pass 1 draws
                    float tot = 0.0f, run = 0.0f, pick = 0.0f;
                    int last = -1;
                    x = -1;
                    for (int pass = 0; pass < 2 && x < 0; pass++) {
                        int p = 0, q = 0;
                        while ((p < ng2 || q < 2) && x < 0) {
                            const int eq = q == 0 ? e0 : (q == 1 ? e1 : -1);
                            if (eq < 0 && q < 2) { q++; continue; }
                            int j;
                            float wv;
                            if (q < 2 && (p >= ng2 || eq < gi[p0 + p])) {
                                j = eq;
                                wv = c[j] * (q == 0 ? w0 : w1);
                                q++;
                            } else {
                                j = gi[p0 + p];
                                wv = c[j] * dp[j];
                                p++;
                            }
                            if (pass == 0) {
                                tot += wv;
                            } else {
                                run += wv;
                                if (wv > 0.0f) last = j;
                                if (run >= pick) x = j;
                            }
                        }
                        if (pass == 0) pick = (float)uniform(col) * tot;
                    }
                    if (x < 0) x = last >= 0 ? last : 0;
                }
                x = __shfl_sync(FULL, x, 0);
                if (lane == 0) path[col] = x;
                state = x;
                __syncwarp();
                consumed_to(col);
            }
        }
        cur = nx1;
        nx1 = nx2;
    }
    if (failed && lane == 0) report_error(d.err, ERR_WAIT_LIMIT, qi, -1, -1);
    // every copy issued has landed before the CTA's shared memory is released
    if (lane == 0) {
        for (int m = waited; m < issued; m++) mbar_wait(&cbar[m % NCH], (unsigned)((m / NCH) & 1));
        for (int q = 0; q < 2; q++)
            if (tpend[q]) mbar_wait(&tbar[q], tphase[q]);
    }
    __syncwarp();
}

template <int NCH>
bool launch_split(const BatchDev &d, cudaStream_t s, size_t budget) {
    const int maxS = imax(d.maxS, 1);
    const size_t smem = (size_t)NCH * chunk_tab_bytes(maxS) + (size_t)NCH * CW * MAXT * sizeof(float) +
                        (size_t)NCH * (CW + 2) * sizeof(double) + 2 * (size_t)TreeBufLayout(maxS).total;
    if (smem > budget) return false;
    prefer_shared(k_traceback_split<NCH>);
    if (!raise_dynamic_smem(k_traceback_split<NCH>, smem)) return true;  // the launch reports it
    k_traceback_split<NCH><<<d.ninst, 32, smem, s>>>(d, maxS);
    note_launch();
    return true;
}

template <typename F, int G, int DEPTH, bool QL = false>
bool launch_cfg(const BatchDev &d, cudaStream_t s, size_t budget) {
    const int maxS = imax(d.maxS, 1);
    if (QL && maxS > QL_MAXS) return false;
    const int slot_elems = (int)(((size_t)maxS * sizeof(F) + 32 + 15) / 16 * 16 / sizeof(F));
    size_t smem = (size_t)DEPTH * slot_elems * sizeof(F) + DEPTH * sizeof(double) +
                  (size_t)(maxS + 1) * sizeof(F) + 2 * (size_t)maxS * sizeof(int) + 16;
    if (QL) smem = (smem + 15) / 16 * 16 + (size_t)G * (maxS + 1) * sizeof(F);
    if (smem > budget) return false;
    // opt in; static shared memory counts against 48 KB too
    if (!raise_dynamic_smem(k_traceback<F, G, DEPTH, QL>, smem)) return true;  // the launch reports it
    k_traceback<F, G, DEPTH, QL><<<d.ninst, 32, smem, s>>>(d, maxS, slot_elems);
    note_launch();
    return true;
}

template <typename F>
void launch(const BatchDev &d, cudaStream_t s) {
    // the deepest speculation whose ring leaves room for two CTAs per SM, else one
    constexpr size_t two = 100 * 1024, one = 200 * 1024;
    if constexpr (sizeof(F) == 4) {
        if (d.bins32) {
            if (launch_split<4>(d, s, 112 * 1024)) return;
            if (launch_split<3>(d, s, 112 * 1024)) return;
            if (launch_split<4>(d, s, 224 * 1024)) return;
            if (launch_split<3>(d, s, 224 * 1024)) return;
        }
    }
    if constexpr (sizeof(F) == 8) {
        if (launch_cfg<F, 8, 24, true>(d, s, two)) return;
    }
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

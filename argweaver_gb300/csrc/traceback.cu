// K4: stochastic traceback, one warp per instance (stochastic_traceback,
// sample_thread.cpp:522-569; sample_hmm_posterior :470-503; sample_hmm_posterior_step
// :506-519; sample, common.h:272-290).
//
// Column i draws path[i] from A[j] = fw[i][j] * P(j -> path[i+1]) with the uniform u[i]:
// the first j whose running sum reaches u[i] * sum(A). The warp splits the states into 32
// contiguous chunks; chunk sums are scanned across lanes and the lane whose chunk holds the
// pick rescans it in state order. Transition rows P(. -> k) are rebuilt only when k or the
// local tree changes, as in the reference.
//
// The forward table is read from HBM once, newest column first; columns stream into a
// shared-memory ring DEPTH columns ahead of the sampler with cp.async, so HBM latency
// overlaps the sampling of earlier columns.

#include <cuda_runtime.h>

#include "kernels.h"

namespace awg {

namespace {

constexpr int DEPTH = 8;

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

__device__ __forceinline__ void cp_async(void *smem, const void *gmem, int bytes) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    if (bytes == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem));
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

// Draw an index from weights w(j), j < n, with uniform u (sample(), common.h:272-290).
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
    F incl = l0 + l1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const F v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    F excl = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) excl = 0;
    const F total = __shfl_sync(0xffffffffu, incl, 31);
    const F pick = (F)u * total;
    const unsigned hit = __ballot_sync(0xffffffffu, incl >= pick && hi > lo);
    if (!hit) return n - 1;
    // rescan the chunk that holds the pick, all lanes at once: lane t takes element
    // lo_src + t, a lane scan gives the running sums in state order
    const int src = __ffs(hit) - 1;
    const int slo = __shfl_sync(0xffffffffu, lo, src), shi = __shfl_sync(0xffffffffu, hi, src);
    F carry = __shfl_sync(0xffffffffu, excl, src);
    int result = shi - 1;
    for (int b0 = slo; b0 < shi; b0 += 32) {
        const int jj = b0 + lane;
        F x = jj < shi ? w(jj) : F(0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const F v = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += v;
        }
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

template <typename F>
__global__ void k_traceback(BatchDev d, int maxS) {
    extern __shared__ double dyn_d[];
    F *ring = (F *)dyn_d;                       // [DEPTH][maxS]
    F *trans = ring + (size_t)DEPTH * maxS;      // [maxS]
    int *stime = (int *)(trans + maxS + 1);      // [maxS] state times of the current tree
    int *snode = stime + maxS;                   // [maxS]
    __shared__ F tmS[MAXT * MAXT];
    const TTab<F> tab(d);
    const InstDev I = d.inst[blockIdx.x];
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
            F *dst = ring + (size_t)(pcol % DEPTH) * maxS;
            for (int j = lane; j < pS; j += 32) cp_async(dst + j, src + j, sizeof(F));
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
    for (int q = 0; q < DEPTH; q++) issue();

    // uniforms for the next 32 columns (descending), read back by shuffles
    double ucache = 0.0;
    int ubase = -1;  // ucache holds u[ubase - 1 - lane]; empty until the first call
    auto uni = [&](int c) -> double {
        if (ubase - c > 32 || c >= ubase) {
            ubase = c + 1;
            const int q = ubase - 1 - lane;
            ucache = q >= 0 ? u[q] : 0.0;
        }
        return __shfl_sync(0xffffffffu, ucache, ubase - 1 - c);
    };
    int col = L - 1;
    int state;  // path[col + 1] of the column being sampled
    // last column (sample_thread.cpp:534-539)
    {
        cp_wait<DEPTH - 1>();
        __syncwarp();
        const int Slast = d.blocks[I.block0 + I.ntrees - 1].S;
        const F *c = ring + (size_t)(col % DEPTH) * maxS;
        const int x = warp_sample<F>(imax(Slast, 1), uni(col), [&](int j) { return c[j]; });
        if (lane == 0) path[col] = x;
        state = x;
        __syncwarp();
        issue();
    }
    for (int bi = I.ntrees - 1; bi >= 0; bi--) {
        const int blk = I.block0 + bi;
        const BlockDev B = d.blocks[blk];
        const int S = B.S, Sm = imax(S, 1);
        // stage the tree's state times/nodes and tmatrix
        for (int j = lane; j < S; j += 32) {
            const StateInfo si = d.sinfo[B.state0 + j];
            stime[j] = si.time;
            snode[j] = si.node;
        }
        const F *tmg = tab.tm + (size_t)blk * MAXT * MAXT;
        for (int e = lane; e < (I.T - 1) * MAXT; e += 32) tmS[e] = tmg[e];
        __syncwarp();
        int last_k = -1;
        for (int i = B.len - 2; i >= 0; i--) {
            col = B.start + i;
            const int k = state;
            if (k != last_k) {
                // trans[j] = TransMatrix::get(j, k) (trans.h:64-83)
                if (S == 0) {
                    if (lane == 0) trans[0] = F(1);
                } else {
                    const StateInfo sk = d.sinfo[B.state0 + k];
                    const long long row = B.t2_0 + d.t2off[B.state0 + k];
                    const F stay = TTab<F>::split
                                       ? F(1) - tab.rstay[(size_t)blk * MAXT + sk.time] : F(0);
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
                last_k = k;
            }
            cp_wait<DEPTH - 1>();
            __syncwarp();
            const F *c = ring + (size_t)(col % DEPTH) * maxS;
            const int x = warp_sample<F>(Sm, uni(col), [&](int j) { return c[j] * trans[j]; });
            if (lane == 0) path[col] = x;
            state = x;
            __syncwarp();
            issue();
        }
        if (bi > 0) {
            // switch into this tree (sample_hmm_posterior_step)
            col = B.start - 1;
            const int k = state;
            const int n1 = imax(B.S1, 1);
            const int2 src = d.srcs[blk];
            const int *determ = d.determ + B.prev_state0;
            const F *dp = tab.dprob + B.prev_state0;
            const F rr = tab.rrow[B.state0 + k], cr = tab.crow[B.state0 + k];
            cp_wait<DEPTH - 1>();
            __syncwarp();
            const F *c = ring + (size_t)(col % DEPTH) * maxS;
            auto w = [&](int j) -> F {
                F g;
                if (j == src.y) g = cr;
                else if (j == src.x) g = rr;
                else g = (determ[j] == k) ? dp[j] : F(0);
                return c[j] * g;
            };
            const int x = warp_sample<F>(n1, uni(col), w);
            if (lane == 0) path[col] = x;
            state = x;
            __syncwarp();
            issue();
        }
    }
    cp_wait<0>();
}

template <typename F>
void launch(const BatchDev &d, cudaStream_t s) {
    const int maxS = imax(d.maxS, 1);
    const size_t smem = (size_t)(DEPTH + 1) * maxS * sizeof(F) + sizeof(F) +
                        2 * (size_t)maxS * sizeof(int) + 16;
    static size_t configured = 0;
    if (smem > configured) {  // opt in; static shared memory counts against 48 KB too
        if (cudaFuncSetAttribute(k_traceback<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return;
        configured = smem;
    }
    k_traceback<F><<<d.ninst, 32, smem, s>>>(d, maxS);
    note_launch();
}

}  // namespace

void launch_traceback(const BatchDev &d, bool fp32, cudaStream_t s) {
    if (fp32) launch<float>(d, s);
    else launch<double>(d, s);
}

}  // namespace awg

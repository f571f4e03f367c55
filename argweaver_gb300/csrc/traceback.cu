// K4: stochastic traceback, one warp per instance (stochastic_traceback,
// sample_thread.cpp:522-569; sample_hmm_posterior :470-503; sample_hmm_posterior_step
// :506-519; sample, common.h:272-290).
//
// Column i draws path[i] from A[j] = fw[i][j] * P(j -> path[i+1]) with the uniform u[i]:
// the first j whose running sum reaches u[i] * sum(A). The warp splits the states into 32
// contiguous chunks; chunk sums are scanned across lanes, and the lane whose chunk holds
// the pick rescans it in state order. Transition rows P(. -> k) are rebuilt only when k
// changes, as in the reference.

#include <cuda_runtime.h>

#include "kernels.h"

namespace awg {

namespace {

template <typename F> struct TTab;
template <> struct TTab<double> {
    const double *tm, *gts, *dprob, *rrow, *crow, *fw;
    __device__ explicit TTab(const BatchDev &d)
        : tm(d.tm), gts(d.gts), dprob(d.determprob), rrow(d.recombrow), crow(d.recoalrow),
          fw(d.fw64) {}
    // same-node entry: get_time(a, b, c, minage, true)
    __device__ double same(long long t2_0, int off, int y, double) const { return gts[t2_0 + off + y]; }
};
template <> struct TTab<float> {
    const float *tm, *t2d, *dprob, *rrow, *crow, *fw;
    __device__ explicit TTab(const BatchDev &d)
        : tm(d.tm32), t2d(d.t2d32), dprob(d.determprob32), rrow(d.recombrow32),
          crow(d.recoalrow32), fw(d.fw32) {}
    __device__ float same(long long t2_0, int off, int y, float tmab) const {
        return t2d[t2_0 + off + y] + tmab;
    }
};

// Draw an index from weights w(j), j < n, with uniform u (sample(), common.h:272-290).
template <typename F, typename W>
__device__ int warp_sample(int n, double u, W w) {
    const int lane = threadIdx.x & 31;
    const int chunk = (n + 31) >> 5;
    const int lo = imin(lane * chunk, n), hi = imin(lo + chunk, n);
    F ls = 0;
    for (int j = lo; j < hi; j++) ls += w(j);
    F incl = ls;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const F v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    F excl = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) excl = 0;
    const F total = __shfl_sync(0xffffffffu, incl, 31);
    const F pick = (F)(u * (double)total);
    const unsigned hit = __ballot_sync(0xffffffffu, incl >= pick && hi > lo);
    int result = n - 1;
    if (hit) {
        const int src = __ffs(hit) - 1;
        int found = -1;
        if (lane == src) {
            F x = excl;
            for (int j = lo; j < hi; j++) {
                x += w(j);
                if (x >= pick) { found = j; break; }
            }
            if (found < 0) found = hi - 1;
        }
        result = __shfl_sync(0xffffffffu, found, src);
    }
    return result;
}

template <typename F>
__global__ void k_traceback(BatchDev d, int maxS) {
    extern __shared__ double dyn_d[];
    F *trans = (F *)dyn_d;
    const TTab<F> tab(d);
    const InstDev I = d.inst[blockIdx.x];
    const int lane = threadIdx.x;
    int *path = d.path + I.col0;
    const double *u = d.uniforms + I.col0;
    const int L = I.seqlen;

    // last column (sample_thread.cpp:534-539)
    const BlockDev &Blast = d.blocks[I.block0 + I.ntrees - 1];
    {
        const int Sm = imax(Blast.S, 1);
        const F *col = tab.fw + Blast.cell0 + (size_t)(Blast.len - 1) * Sm;
        const int x = warp_sample<F>(Sm, u[L - 1], [&](int j) { return col[j]; });
        if (lane == 0) path[L - 1] = x;
    }
    __syncwarp();
    for (int bi = I.ntrees - 1; bi >= 0; bi--) {
        const BlockDev &B = d.blocks[I.block0 + bi];
        const int S = B.S, Sm = imax(S, 1);
        const F *tm = tab.tm + (size_t)(I.block0 + bi) * MAXT * MAXT;
        const StateInfo *si = d.sinfo + B.state0;
        const int *t2off = d.t2off + B.state0;
        int last_k = -1;
        for (int i = B.len - 2; i >= 0; i--) {
            const int col = B.start + i;
            const int k = path[col + 1];
            if (k != last_k) {
                // trans[j] = TransMatrix::get(j, k) (trans.h:64-83)
                if (S == 0) {
                    if (lane == 0) trans[0] = F(1);
                } else {
                    const StateInfo sk = si[k];
                    const int b = sk.time;
                    for (int j = lane; j < S; j += 32) {
                        const int a = si[j].time;
                        const F tmab = tm[a * MAXT + b];
                        trans[j] = (si[j].node == sk.node)
                                       ? tab.same(B.t2_0, t2off[k], j - sk.j1, tmab)
                                       : tmab;
                    }
                }
                last_k = k;
                __syncwarp();
            }
            const F *fcol = tab.fw + B.cell0 + (size_t)i * Sm;
            const int x = warp_sample<F>(Sm, u[col], [&](int j) { return fcol[j] * trans[j]; });
            if (lane == 0) path[col] = x;
            __syncwarp();
        }
        if (bi > 0) {
            // switch into this block (sample_hmm_posterior_step)
            const BlockDev &P = d.blocks[I.block0 + bi - 1];
            const int col = B.start - 1;
            const int k = path[B.start];
            const int n1 = imax(B.S1, 1);
            const int2 src = d.srcs[I.block0 + bi];
            const int *determ = d.determ + B.prev_state0;
            const F *dp = tab.dprob + B.prev_state0;
            const F rr = tab.rrow[B.state0 + k], cr = tab.crow[B.state0 + k];
            const F *fcol = tab.fw + P.cell0 + (size_t)(P.len - 1) * imax(P.S, 1);
            auto w = [&](int j) -> F {
                F g;
                if (j == src.y) g = cr;
                else if (j == src.x) g = rr;
                else g = (determ[j] == k) ? dp[j] : F(0);
                return fcol[j] * g;
            };
            const int x = warp_sample<F>(n1, u[col], w);
            if (lane == 0) path[col] = x;
            __syncwarp();
        }
    }
}

template <typename F>
void launch(const BatchDev &d, cudaStream_t s) {
    const int maxS = imax(d.maxS, 1);
    const size_t smem = (size_t)maxS * sizeof(F);
    static size_t configured = 0;
    if (smem > 48 * 1024 && smem > configured) {
        cudaFuncSetAttribute(k_traceback<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
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

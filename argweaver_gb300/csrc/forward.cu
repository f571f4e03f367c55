// K3: the forward pass of the threading HMM, one CTA per instance, column in shared memory.
//
// Per column (arghmm_forward_block, sample_thread.cpp:252-295):
//   fgroups[a] = sum of col1 over states of time a
//   tf[b]      = sum_a tmatrix[a][b] * fgroups[a]
//   col2[k]    = (tf[b_k] + sum over the states j of k's node of tmatrix2[a_j][k]*col1[j]) * e_k
//   col2      /= sum(col2)
// At a local-tree boundary the first column comes from the switch matrix
// (arghmm_forward_switch, sample_thread.cpp:345-389), gathered per target state.
// All reductions use a fixed order (per-warp shuffle trees combined in warp order), so a
// result is the same in every run and in every batch composition.
//
// FP64 (plain path): tmatrix2 is formed as gts - tmatrix, the reference's own subtraction.
// FP32 (chosen path): tables were rounded to FP32 by the table kernels; the column is
// rescaled every column as above and log(norm) is accumulated in FP64.

#include <cuda_runtime.h>

#include "kernels.h"

namespace awg {

namespace {

template <typename F> struct Tab;

template <> struct Tab<double> {
    const double *tm, *inv, *var, *dprob, *rrow, *crow, *gts;
    double *fw;
    __device__ explicit Tab(const BatchDev &d)
        : tm(d.tm), inv(d.inv_lk), var(d.varemit), dprob(d.determprob), rrow(d.recombrow),
          crow(d.recoalrow), gts(d.gts), fw(d.fw64) {}
    // tmatrix2[a][k] (sample_thread.cpp:223-224)
    __device__ double t2(long long t2_0, int off, int y, double tmab) const {
        return gts[t2_0 + off + y] - tmab;
    }
};

template <> struct Tab<float> {
    const float *tm, *inv, *var, *dprob, *rrow, *crow, *t2d;
    float *fw;
    __device__ explicit Tab(const BatchDev &d)
        : tm(d.tm32), inv(d.inv32), var(d.var32), dprob(d.determprob32), rrow(d.recombrow32),
          crow(d.recoalrow32), t2d(d.t2d32), fw(d.fw32) {}
    __device__ float t2(long long t2_0, int off, int y, float) const { return t2d[t2_0 + off + y]; }
};

template <typename F>
__device__ __forceinline__ F warp_sum(F v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

struct Meta {  // per-state metadata in shared memory
    int time, j1, m, off;
};

template <typename F>
__global__ void k_forward(BatchDev d, int maxS) {
    extern __shared__ double dyn_d[];
    const Tab<F> tab(d);
    const InstDev I = d.inst[blockIdx.x];
    const int T = I.T;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nwarps = blockDim.x >> 5;

    F *colA = (F *)dyn_d;
    F *colB = colA + maxS;
    Meta *meta = (Meta *)(colB + maxS + (maxS & 1));
    int *perm = (int *)(meta + maxS);
    __shared__ F tm[MAXT * MAXT];
    __shared__ F fg[MAXT], tf[MAXT], red[32];
    __shared__ int bptr[MAXT + 1];

    F *cur = colA, *nxt = colB;
    double lnl = 0.0;
    int prevS = 0;

    for (int bi = 0; bi < I.ntrees; bi++) {
        const BlockDev &B = d.blocks[I.block0 + bi];
        const int S = B.S, Sm = imax(S, 1);
        const bool empty = (S == 0);  // fully specified internal tree: one state of prob 1
        // block tables
        for (int k = tid; k < S; k += blockDim.x) {
            const StateInfo si = d.sinfo[B.state0 + k];
            meta[k] = Meta{si.time, si.j1, si.m, d.t2off[B.state0 + k]};
            perm[k] = d.bt_perm[B.state0 + k];
        }
        const F *tmg = tab.tm + (size_t)(I.block0 + bi) * MAXT * MAXT;
        for (int e = tid; e < (T - 1) * MAXT; e += blockDim.x) tm[e] = tmg[e];
        for (int a = tid; a <= MAXT; a += blockDim.x)
            bptr[a] = d.bt_ptr[(size_t)(I.block0 + bi) * (MAXT + 1) + a];
        const uint8_t *cls = d.colclass + I.col0 + B.start;
        const int *cvar = d.colvar + I.col0 + B.start;
        const F *inv = tab.inv + B.state0;
        const F *var = tab.var + B.var0;
        F *fw = tab.fw + B.cell0;
        __syncthreads();

        auto emit = [&](int i, int k) -> F {
            const uint8_t c = cls[i];
            if (c == COL_MASKED) return F(1);
            if (c == COL_INVARIANT) return inv[k];
            return var[(size_t)cvar[i] * S + k];
        };

        // first column of the block
        if (bi == 0) {
            for (int k = tid; k < Sm; k += blockDim.x) cur[k] = fw[k];  // priors (K1)
            __syncthreads();  // the first step reads every thread's entries
        } else {
            const int2 src = d.srcs[I.block0 + bi];
            const int *gp = d.gptr + B.gptr0;
            const int *gi = d.gidx + B.prev_state0;
            const F *dp = tab.dprob + B.prev_state0;
            const F *rr = tab.rrow + B.state0;
            const F *cr = tab.crow + B.state0;
            F part = 0;
            for (int k = tid; k < Sm; k += blockDim.x) {
                F s = 0;
                for (int p = gp[k]; p < gp[k + 1]; p++) {
                    const int j = gi[p];
                    s += cur[j] * dp[j];
                }
                if (src.x != -1 && rr[k] > F(0)) s += cur[src.x] * rr[k];
                if (src.y != -1 && cr[k] > F(0)) s += cur[src.y] * cr[k];
                s *= empty ? F(1) : emit(0, k);
                nxt[k] = s;
                part += s;
            }
            part = warp_sum(part);
            if (lane == 0) red[warp] = part;
            __syncthreads();
            F norm = 0;
            for (int w = 0; w < nwarps; w++) norm += red[w];
            for (int k = tid; k < Sm; k += blockDim.x) {
                const F v = nxt[k] / norm;
                nxt[k] = v;
                fw[k] = v;
            }
            if (tid == 0) {
                lnl += log((double)norm);
                if (!(norm > F(0))) report_error(d.err, ERR_ZERO_NORM, blockIdx.x, bi, B.start);
            }
            F *t = cur; cur = nxt; nxt = t;
            __syncthreads();
        }
        (void)prevS;
        prevS = S;

        if (empty) {
            // fully specified tree: the single state carries over (sample_thread.cpp:201-206)
            for (int i = 1; i < B.len; i++)
                if (tid == 0) fw[(size_t)i] = cur[0];
            __syncthreads();
            continue;
        }

        for (int i = 1; i < B.len; i++) {
            // fgroups
            for (int a = warp; a < T - 1; a += nwarps) {
                F s = 0;
                for (int p = bptr[a] + lane; p < bptr[a + 1]; p += 32) s += cur[perm[p]];
                s = warp_sum(s);
                if (lane == 0) fg[a] = s;
            }
            __syncthreads();
            if (warp == 0 && lane < T - 1) {
                F s = 0;
                for (int a = 0; a < T - 1; a++) s += tm[a * MAXT + lane] * fg[a];
                tf[lane] = s;
            }
            __syncthreads();
            F part = 0;
            for (int k = tid; k < S; k += blockDim.x) {
                const Meta mk = meta[k];
                const int a0 = mk.time - (k - mk.j1);
                F s = tf[mk.time];
                for (int y = 0; y < mk.m; y++)
                    s += tab.t2(B.t2_0, mk.off, y, tm[(a0 + y) * MAXT + mk.time]) * cur[mk.j1 + y];
                s *= emit(i, k);
                nxt[k] = s;
                part += s;
            }
            part = warp_sum(part);
            if (lane == 0) red[warp] = part;
            __syncthreads();
            F norm = 0;
            for (int w = 0; w < nwarps; w++) norm += red[w];
            F *out = fw + (size_t)i * S;
            for (int k = tid; k < S; k += blockDim.x) {
                const F v = nxt[k] / norm;
                nxt[k] = v;
                out[k] = v;
            }
            if (tid == 0) {
                lnl += log((double)norm);
                if (!(norm > F(0)))
                    report_error(d.err, ERR_ZERO_NORM, blockIdx.x, bi, B.start + i);
            }
            F *t = cur; cur = nxt; nxt = t;
            __syncthreads();
        }
    }
    if (tid == 0 && d.lnl) d.lnl[blockIdx.x] = lnl;
}

int forward_threads(int maxS) {
    if (maxS > 768) return 512;
    if (maxS > 256) return 256;
    return 128;
}

template <typename F>
size_t forward_smem(int maxS) {
    return 2 * (size_t)maxS * sizeof(F) + 8 + (size_t)maxS * (sizeof(Meta) + sizeof(int));
}

template <typename F>
void launch(const BatchDev &d, cudaStream_t s) {
    const int maxS = imax(d.maxS, 1);
    const size_t smem = forward_smem<F>(maxS);
    static size_t configured = 0;
    if (smem > 48 * 1024 && smem > configured) {
        cudaFuncSetAttribute(k_forward<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        configured = smem;
    }
    k_forward<F><<<d.ninst, forward_threads(maxS), smem, s>>>(d, maxS);
    note_launch();
}

}  // namespace

void launch_forward(const BatchDev &d, bool fp32, cudaStream_t s) {
    if (fp32) launch<float>(d, s);
    else launch<double>(d, s);
}

}  // namespace awg

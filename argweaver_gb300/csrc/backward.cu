// K5: backward pass fused with the posterior marginals, one CTA per instance.
//
// The reference has no backward pass for the threading HMM. This one uses the forward
// pass's transition semantics (TransMatrix::get, trans.h:64-83; TransMatrixSwitch::get,
// trans.h:207-219) transposed, over the same structure:
//   g[k]     = e_{i+1}[k] * bw_{i+1}[k]
//   G[b]     = sum of g over states of time b
//   bw_i[j]  = sum_b tmatrix[a_j][b] * G[b] + sum over states k of j's node of
//              tmatrix2[a_j][k] * g[k]
// normalised per column. At a tree boundary bw of the previous tree's last column is
// gathered through the switch matrix. Posterior marginals are fw[i] * bw[i] renormalised;
// the backward column never leaves shared memory unless the caller asks for the table.

#include <cuda_runtime.h>

#include "kernels.h"

namespace awg {

namespace {

template <typename F> struct BTab;
template <> struct BTab<double> {
    static constexpr bool split = false;
    const float *rstay = nullptr;
    const double *tm, *inv, *var, *dprob, *rrow, *crow, *gts, *fw;
    __device__ explicit BTab(const BatchDev &d)
        : tm(d.tm), inv(d.inv_lk), var(d.varemit), dprob(d.determprob), rrow(d.recombrow),
          crow(d.recoalrow), gts(d.gts), fw(d.fw64) {}
    __device__ double t2(long long idx, double tmab) const { return gts[idx] - tmab; }
};
template <> struct BTab<float> {
    // complements of the stay probability and of the invariant emissions, as in the forward
    static constexpr bool split = true;
    const float *rstay;
    const float *tm, *inv, *var, *dprob, *rrow, *crow, *t2d, *fw;
    __device__ explicit BTab(const BatchDev &d)
        : rstay(d.rstay32), tm(d.tm32), inv(d.inv32), var(d.var32), dprob(d.determprob32),
          rrow(d.recombrow32), crow(d.recoalrow32), t2d(d.t2d32), fw(d.fw32) {}
    __device__ float t2(long long idx, float) const { return t2d[idx]; }
};

// FP32 pair arithmetic for the dominant path of the FP32 backward step (the same reason
// and transforms as the forward's: the column's fixed point within a tree would otherwise
// move by the step's rounding over one minus the chain's contraction).
struct F2 {
    float hi, lo;
};
__device__ __forceinline__ F2 f2_renorm(float a, float b) {  // |a| >= |b|
    const float s = a + b;
    return F2{s, b - (s - a)};
}
__device__ __forceinline__ F2 f2_keep(F2 x, float r) {  // x * (1 - r), 0 <= r < 1
    const float t = x.hi * r;
    const float h = x.hi - t;
    return f2_renorm(h, ((x.hi - h) - t) + x.lo);
}
__device__ __forceinline__ F2 f2_mul(F2 x, float e) {
    const float p = x.hi * e;
    return f2_renorm(p, fmaf(x.hi, e, -p) + x.lo * e);
}
__device__ __forceinline__ F2 f2_add(F2 x, float s) {
    const float h = x.hi + s;
    const float bb = h - x.hi;
    const float err = (x.hi - (h - bb)) + (s - bb);
    return f2_renorm(h, err + x.lo);
}

template <typename F>
__device__ __forceinline__ F warp_sum(F v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

struct Meta {
    int time, j1, m, off;
};

// Block-wide sum of fn(k), k < n, in an order fixed by n alone (groups of 32 consecutive
// k, then the group sums), so results do not depend on the block size. Every thread gets
// the result; gs holds ceil(n / 32) group sums.
template <typename F, typename Fn>
__device__ F fixed_sum(int n, Fn fn, F *gs) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int ng = (n + 31) >> 5;
    __syncthreads();  // gs free, inputs complete
    for (int g = warp; g < ng; g += nw) {
        const int k = g * 32 + lane;
        const F x = warp_sum(k < n ? fn(k) : F(0));
        if (lane == 0) gs[g] = x;
    }
    __syncthreads();
    F s = 0;
    for (int g = lane; g < ng; g += 32) s += gs[g];
    return warp_sum(s);
}

template <typename F>
__global__ void k_backward(BatchDev d, int maxS, double *bw_out) {
    extern __shared__ double dyn_d[];
    const BTab<F> tab(d);
    const int qi = cta_instance(d);
    const InstDev I = d.inst[qi];
    const int T = I.T;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nwarps = blockDim.x >> 5;

    F *bwA = (F *)dyn_d;
    F *bwB = bwA + maxS;
    F *g = bwB + maxS;
    float *loA = (float *)(g + maxS);           // FP32 path: low parts of bwA / bwB
    float *loB = loA + maxS;
    float *glo = loB + maxS;                    // FP32 path: low parts of g at a switch
    Meta *meta = (Meta *)(((uintptr_t)(glo + maxS) + 15) & ~(uintptr_t)15);
    int *perm = (int *)(meta + maxS);
    F *gs = (F *)(perm + maxS + 1) + 1;     // [maxS / 32 + 1] group sums, 8-byte aligned
    gs = (F *)(((uintptr_t)gs + 7) & ~(uintptr_t)7);
    __shared__ F tm[MAXT * MAXT];
    __shared__ F G[MAXT], H[MAXT], rS[MAXT];
    __shared__ int bptr[MAXT + 1];

    F *cur = bwA, *nxt = bwB;  // cur: bw of column i+1, nxt: bw of column i
    float *curlo = loA, *nxtlo = loB;
    {
        const BlockDev &B = d.blocks[I.block0 + I.ntrees - 1];
        const int Sm = imax(B.S, 1);
        for (int k = tid; k < Sm; k += blockDim.x) {
            cur[k] = F(1) / F(Sm);
            curlo[k] = 0.0f;
        }
    }
    __syncthreads();

    for (int bi = I.ntrees - 1; bi >= 0; bi--) {
        const BlockDev &B = d.blocks[I.block0 + bi];
        const int S = B.S, Sm = imax(S, 1);
        for (int k = tid; k < S; k += blockDim.x) {
            const StateInfo si = d.sinfo[B.state0 + k];
            meta[k] = Meta{si.time, si.j1, si.m, d.t2off[B.state0 + k]};
            perm[k] = d.bt_perm[B.state0 + k];
        }
        const F *tmg = tab.tm + (size_t)(I.block0 + bi) * MAXT * MAXT;
        for (int e = tid; e < (T - 1) * MAXT; e += blockDim.x) tm[e] = tmg[e];
        for (int a = tid; a <= MAXT; a += blockDim.x)
            bptr[a] = d.bt_ptr[(size_t)(I.block0 + bi) * (MAXT + 1) + a];
        if (BTab<F>::split)
            for (int a = tid; a < MAXT; a += blockDim.x)
                rS[a] = tab.rstay[(size_t)(I.block0 + bi) * MAXT + a];
        const uint8_t *cls = d.colclass + I.col0 + B.start;
        const int *cvar = d.colvar + I.col0 + B.start;
        const F *inv = tab.inv + B.state0;
        const F *var = tab.var + B.var0;
        const F *fw = tab.fw + B.cell0;
        __syncthreads();

        // emission times a backward value (the common factor e_ref dropped in FP32)
        auto emitx = [&](int i, int k, F x) -> F {
            const uint8_t c = cls[i];
            if (c == COL_MASKED || S == 0) return x;
            if (c == COL_INVARIANT) return BTab<F>::split ? x - x * inv[k] : x * inv[k];
            const F e = var[(size_t)cvar[i] * S + k];
            if (!BTab<F>::split) return x * e;
            return e >= F(0) ? x - x * e : x * -e;  // FP32: 1 - e_k / e_ref, or -e_k / e_ref
        };
        // posterior of one column from its bw (in `bw`) and fw
        auto posterior = [&](int i, const F *bw) {
            const F *f = fw + (size_t)i * Sm;
            const F z = fixed_sum<F>(Sm, [&](int k) { return f[k] * bw[k]; }, gs);
            const long long c0 = B.cell0 + (long long)i * Sm;
            for (int k = tid; k < Sm; k += blockDim.x) {
                if (d.post) d.post[c0 + k] = (double)(f[k] * bw[k] / z);
                if (bw_out) bw_out[c0 + k] = (double)bw[k];
            }
        };

        posterior(B.len - 1, cur);
        for (int i = B.len - 2; i >= 0; i--) {
            for (int k = tid; k < Sm; k += blockDim.x) g[k] = emitx(i + 1, k, cur[k]);
            __syncthreads();
            if (S == 0) {
                if (tid == 0) nxt[0] = g[0];
            } else {
                for (int a = warp; a < T - 1; a += nwarps) {
                    F s = 0;
                    for (int p = bptr[a] + lane; p < bptr[a + 1]; p += 32) s += g[perm[p]];
                    s = warp_sum(s);
                    if (lane == 0) G[a] = s;
                }
                __syncthreads();
                if (warp == 0 && lane < T - 1) {
                    F s = 0;
                    for (int b = 0; b < T - 1; b++) s += tm[lane * MAXT + b] * G[b];
                    H[lane] = s;
                }
                __syncthreads();
                for (int j = tid; j < S; j += blockDim.x) {
                    const Meta mj = meta[j];
                    const int y = j - mj.j1;  // position of j's time among its node's times
                    const int a = mj.time;
                    const int a0 = a - y;
                    F s = H[a];
                    for (int x = 0; x < mj.m; x++) {
                        const int k = mj.j1 + x;  // target on the same node, time a0 + x
                        s += tab.t2(B.t2_0 + meta[k].off + y * mj.m, tm[a * MAXT + a0 + x]) * g[k];
                    }
                    if constexpr (BTab<F>::split) {
                        // pairs: (e * bw) of state j kept with (1 - rs), plus the inflow
                        F2 gj = F2{cur[j], curlo[j]};
                        const uint8_t c = cls[i + 1];
                        if (c == COL_INVARIANT) gj = f2_keep(gj, inv[j]);
                        else if (c != COL_MASKED) {
                            const float e = var[(size_t)cvar[i + 1] * S + j];
                            gj = e >= 0.0f ? f2_keep(gj, e) : f2_mul(gj, -e);
                        }
                        const F2 x = f2_add(f2_keep(gj, rS[a]), s);
                        nxt[j] = x.hi;
                        nxtlo[j] = x.lo;
                    } else {
                        nxt[j] = s;
                    }
                }
            }
            const F z = fixed_sum<F>(Sm, [&](int k) { return nxt[k]; }, gs);
            if constexpr (BTab<F>::split) {
                const float iz = 1.0f / z;
                for (int k = tid; k < Sm; k += blockDim.x) {
                    const F2 x = f2_mul(F2{nxt[k], S == 0 ? 0.0f : nxtlo[k]}, iz);
                    nxt[k] = x.hi;
                    nxtlo[k] = x.lo;
                }
            } else {
                for (int k = tid; k < Sm; k += blockDim.x) nxt[k] /= z;
            }
            __syncthreads();
            posterior(i, nxt);
            F *t = cur; cur = nxt; nxt = t;
            float *tl = curlo; curlo = nxtlo; nxtlo = tl;
        }
        if (bi > 0) {
            // into the previous tree's last column through the switch matrix
            const BlockDev &P = d.blocks[I.block0 + bi - 1];
            const int n1 = imax(B.S1, 1);
            if constexpr (BTab<F>::split) {
                // pairs through the switch: e * bw of the tree's first column with its low
                // parts; a deterministic move by its FP64 probability (a complement near 1)
                for (int k = tid; k < Sm; k += blockDim.x) {
                    F2 x = F2{cur[k], S == 0 ? 0.0f : curlo[k]};
                    const uint8_t c = cls[0];
                    if (S > 0 && c == COL_INVARIANT) x = f2_keep(x, inv[k]);
                    else if (S > 0 && c != COL_MASKED) {
                        const float e = var[(size_t)cvar[0] * S + k];
                        x = e >= 0.0f ? f2_keep(x, e) : f2_mul(x, -e);
                    }
                    g[k] = x.hi;
                    glo[k] = x.lo;
                }
            } else {
                for (int k = tid; k < Sm; k += blockDim.x) g[k] = emitx(0, k, cur[k]);
            }
            __syncthreads();
            const int2 src = d.srcs[I.block0 + bi];
            const int *determ = d.determ + B.prev_state0;
            const F *dp = tab.dprob + B.prev_state0;
            const double *dp64 = d.determprob + B.prev_state0;
            const F *rr = tab.rrow + B.state0;
            const F *cr = tab.crow + B.state0;
            for (int j = tid; j < n1; j += blockDim.x) {
                F s = 0;
                float slo = 0.0f;
                if (j == src.y || j == src.x) {
                    const F *row = (j == src.y) ? cr : rr;
                    for (int k = 0; k < Sm; k++)
                        if (row[k] > F(0)) s += row[k] * g[k];
                } else if (determ[j] >= 0) {
                    if constexpr (BTab<F>::split) {
                        const double pj = dp64[j];
                        const F2 x{g[determ[j]], glo[determ[j]]};
                        const F2 y = pj >= 0.5 ? f2_keep(x, (float)(1.0 - pj)) : f2_mul(x, (float)pj);
                        s = y.hi;
                        slo = y.lo;
                    } else {
                        s = dp[j] * g[determ[j]];
                    }
                }
                nxt[j] = s;
                nxtlo[j] = slo;
            }
            const F z = fixed_sum<F>(n1, [&](int k) { return nxt[k]; }, gs);
            if constexpr (BTab<F>::split) {
                const float iz = 1.0f / z;
                for (int k = tid; k < n1; k += blockDim.x) {
                    const F2 x = f2_mul(F2{nxt[k], nxtlo[k]}, iz);
                    nxt[k] = x.hi;
                    nxtlo[k] = x.lo;
                }
            } else {
                for (int k = tid; k < n1; k += blockDim.x) {
                    nxt[k] /= z;
                    nxtlo[k] = 0.0f;
                }
            }
            __syncthreads();
            (void)P;
            F *t = cur; cur = nxt; nxt = t;
            float *tl = curlo; curlo = nxtlo; nxtlo = tl;
        }
    }
}

int backward_threads(int maxS) {
    if (maxS > 768) return 512;
    if (maxS > 256) return 256;
    return 128;
}

template <typename F>
void launch(const BatchDev &d, double *bw_out, cudaStream_t s) {
    const int maxS = imax(d.maxS, 1);
    const size_t smem = 3 * (size_t)maxS * sizeof(F) + 3 * (size_t)maxS * sizeof(float) + 16 +
                        (size_t)maxS * (sizeof(Meta) + sizeof(int)) + sizeof(int) + 16 +
                        ((size_t)maxS / 32 + 1) * sizeof(F);
    // opt in; static shared memory counts against 48 KB too
    if (!raise_dynamic_smem(k_backward<F>, smem)) return;
    k_backward<F><<<d.ninst, backward_threads(maxS), smem, s>>>(d, maxS, bw_out);
    note_launch();
}

}  // namespace

void launch_backward(const BatchDev &d, bool fp32, double *bw_out, cudaStream_t s) {
    if (fp32) launch<float>(d, bw_out, s);
    else launch<double>(d, bw_out, s);
}

}  // namespace awg

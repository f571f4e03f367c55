// K3: the forward pass of the threading HMM, one CTA per instance, column in shared memory.
//
// Per column (arghmm_forward_block, sample_thread.cpp:252-295):
//   fgroups[a] = sum of col1 over states of time a
//   tf[b]      = sum_a tmatrix[a][b] * fgroups[a]
//   col2[k]    = (tf[b_k] + sum over the states j of k's node of tmatrix2[a_j][k]*col1[j]) * e_k
//   col2      /= sum(col2)
// At a local-tree boundary the first column comes from the switch matrix
// (arghmm_forward_switch, sample_thread.cpp:345-389), gathered per target state.
//
// Schedule per column, two CTA barriers:
//   A  the previous column is complete, in state order (for same-branch neighbours) and in
//      time-sorted order (each time bin a contiguous range);
//      warps split the bins; a warp sums a bin with coalesced, conflict-free loads
//   B  every thread reads the bins: the previous column's norm and tf (lane b); then each
//      thread writes its entries of the previous column, divided by that norm, to HBM and
//      computes its entries of the new column scaled by 1/norm (the reference's
//      normalise-then-step, reordered; the normalised values are the same).
// Reductions have a fixed order, so results do not depend on the run or the batch.
// log(norm) goes into an FP64 mantissa product plus an integer exponent (one FP64 log
// every 64 columns instead of one per column).
//
// FP64 (plain path): tmatrix2 = gts - tmatrix, the reference's own subtraction, formed when
// the block's rows are staged. FP32 (chosen path): tables rounded to FP32 by the table
// kernels; columns rescaled every column; the log-likelihood accumulates in FP64. Values
// next to 1 keep their information as complements (built with expm1 in FP64):
//   stay:     x_k * norecombs[b]   ->  x_k - rstay[b] * x_k
//   emission: x_k * e_k            ->  (x_k - inv32[k] * x_k) * e_ref, e_ref into the FP64
//                                      log-likelihood once per invariant column
// so the moving probability mass and the emission contrasts, not their rounding, drive
// the chain over thousands of columns.

#include <cuda_runtime.h>

#include <cstdlib>

#include "kernels.h"

namespace awg {

namespace {

template <typename F> struct Tab;

template <> struct Tab<double> {
    static constexpr bool split = false;
    const double *tm, *inv, *var, *dprob, *rrow, *crow, *gts;
    const float *rstay = nullptr;
    const double *lneref = nullptr, *vref = nullptr;
    double *fw;
    __device__ explicit Tab(const BatchDev &d)
        : tm(d.tm), inv(d.inv_lk), var(d.varemit), dprob(d.determprob), rrow(d.recombrow),
          crow(d.recoalrow), gts(d.gts), fw(d.fw64) {}
    // tmatrix2[a][k] (sample_thread.cpp:223-224)
    __device__ double t2(long long idx, double tmab) const { return gts[idx] - tmab; }
    __device__ const double *t2rows() const { return gts; }
};

template <> struct Tab<float> {
    static constexpr bool split = true;
    const float *tm, *inv, *var, *dprob, *rrow, *crow, *t2d;
    const float *rstay;
    const double *lneref, *vref;
    float *fw;
    __device__ explicit Tab(const BatchDev &d)
        : tm(d.tm32), inv(d.inv32), var(d.var32), dprob(d.determprob32), rrow(d.recombrow32),
          crow(d.recoalrow32), t2d(d.t2d32), rstay(d.rstay32), lneref(d.lneref), vref(d.vref),
          fw(d.fw32) {}
    __device__ float t2(long long idx, float) const { return t2d[idx]; }
    __device__ const float *t2rows() const { return t2d; }
};

// A hint that moves [p, p + bytes) (the whole 16-byte granules inside it) from HBM into L2
// (cp.async.bulk.prefetch.L2): no result, no fault, no effect on any value.
__device__ __forceinline__ void l2_prefetch(const void *p, size_t bytes) {
    const uintptr_t a = ((uintptr_t)p + 15) & ~(uintptr_t)15;
    const uintptr_t e = ((uintptr_t)p + bytes) & ~(uintptr_t)15;
    if (e > a)
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a), "r"((unsigned)(e - a))
                     : "memory");
}

// The tables a tree's staging and columns read (the register kernel's per-tree staging:
// state metadata, tmatrix, same-branch rows, invariant emissions, time bins, the switch
// column's gather lists and rows; then its column classes and variant emission rows), for
// tree blk of instance I, prefetched into L2 while the tree before it runs: its staging then
// waits on L2 instead of HBM.
template <typename F>
__device__ __forceinline__ void prefetch_tree(const BatchDev &d, const Tab<F> &tab, const InstDev &I,
                                              int blk) {
    const BlockDev &N = d.blocks[blk];
    const size_t S = (size_t)imax(N.S, 1), S1 = (size_t)imax(N.S1, 1);
    l2_prefetch(d.sinfo + N.state0, sizeof(StateInfo) * S);
    l2_prefetch(d.t2off + N.state0, sizeof(int) * S);
    l2_prefetch(d.bt_perm + N.state0, sizeof(int) * S);
    l2_prefetch(tab.inv + N.state0, sizeof(F) * S);
    l2_prefetch(tab.rrow + N.state0, sizeof(F) * S);
    l2_prefetch(tab.crow + N.state0, sizeof(F) * S);
    l2_prefetch(tab.tm + (size_t)blk * MAXT * MAXT, sizeof(F) * MAXT * MAXT);
    l2_prefetch(d.bt_ptr + (size_t)blk * (MAXT + 1), sizeof(int) * (MAXT + 1));
    l2_prefetch(d.gptr + N.gptr0, sizeof(int) * (S + 1));
    l2_prefetch(d.gidx + N.prev_state0, sizeof(int) * S1);
    l2_prefetch(d.determprob + N.prev_state0, sizeof(double) * S1);
    l2_prefetch(d.colclass + I.col0 + N.start, (size_t)N.len);
    l2_prefetch(d.colvar + I.col0 + N.start, sizeof(int) * N.len);
    if (N.M > 0) l2_prefetch(tab.t2rows() + N.t2_0, sizeof(F) * N.M);
    if (N.nvar > 0 && N.S > 0) l2_prefetch(tab.var + N.var0, sizeof(F) * N.nvar * (size_t)N.S);
}

template <typename F>
__device__ __forceinline__ F warp_sum(F v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Running sum of log(norm): mantissa product in FP64 and binary exponent in an integer.
struct LogAcc {
    double prod = 1.0;
    long long e = 0;
    int n = 0;
    double lnl = 0.0;
    double extra = 0.0;  // log(e_ref) of invariant columns (FP32 path)
    __device__ void add(double norm) {
        int ex;
        prod *= frexp(norm, &ex);
        e += ex;
        if (++n == 64) flush();
    }
    __device__ void flush() {
        lnl += extra;
        extra = 0.0;
        if (n) {
            lnl += log(prod) + (double)e * 0.69314718055994530942;
            prod = 1.0;
            e = 0;
            n = 0;
        }
    }
};

struct Meta {
    int time, j1, m, off;
};

template <typename F>
__global__ void __launch_bounds__(512) k_forward(BatchDev d, int maxS, int maxM, int t2_in_smem) {
    extern __shared__ double dyn_d[];
    const Tab<F> tab(d);
    const int qi = cta_instance(d);
    const InstDev I = d.inst[qi];
    const int T = I.T, NB = T - 1;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int NT = blockDim.x, NW = NT >> 5;

    F *col = (F *)dyn_d;                       // [2][maxS] columns in state order
    F *colT = col + 2 * maxS;                  // [maxS] newest column, time-sorted
    F *t2s = colT + maxS;                      // [maxM] tmatrix2 entries of the block
    F *invS = t2s + maxM;                      // [maxS] invariant-site emissions
    Meta *meta = (Meta *)(((uintptr_t)(invS + maxS) + 15) & ~(uintptr_t)15);
    int *rank = (int *)(meta + maxS);          // time-sorted position of each state
    __shared__ F tmS[MAXT * MAXT];
    __shared__ F rS[MAXT];
    __shared__ F tfrow[MAXT - 1][32];          // per bin b: tm[b][lane] * sum_b, sum_b (lane 31)
    __shared__ int bptr[MAXT + 1];

    LogAcc acc;
    int c = 0;                                 // buffer holding the current column

    for (int bi = 0; bi < I.ntrees; bi++) {
        const int blk = I.block0 + bi;
        const BlockDev B = d.blocks[blk];
        const int S = B.S;
        F *fw = tab.fw + B.cell0;

        if (S == 0) {
            // fully specified tree: one state that carries over (sample_thread.cpp:201-206)
            F v;
            if (bi == 0) {
                v = fw[0];
                if (tid == 0) col[c * maxS] = v;
            } else {
                // switch into the single state: every source maps to it
                const int2 src = d.srcs[blk];
                const int *gp = d.gptr + B.gptr0;
                const int *gi = d.gidx + B.prev_state0;
                const F *dp = tab.dprob + B.prev_state0;
                const F *rr = tab.rrow + B.state0;
                const F *cr = tab.crow + B.state0;
                F part = 0;
                if (tid < 32) {
                    for (int p = gp[0] + lane; p < gp[1]; p += 32) part += col[c * maxS + gi[p]] * dp[gi[p]];
                    part = warp_sum(part);
                }
                if (tid == 0) {
                    if (src.x != -1 && rr[0] > F(0)) part += col[c * maxS + src.x] * rr[0];
                    if (src.y != -1 && cr[0] > F(0)) part += col[c * maxS + src.y] * cr[0];
                    acc.add((double)part);
                    col[c * maxS] = F(1);
                    fw[0] = F(1);
                }
                v = F(1);
            }
            for (int i = 1 + tid; i < B.len; i += NT) fw[i] = v;
            __syncthreads();
            continue;
        }

        // ---- stage the block's tables
        for (int k = tid; k < S; k += NT) {
            const StateInfo si = d.sinfo[B.state0 + k];
            meta[k] = Meta{si.time, si.j1, si.m, d.t2off[B.state0 + k]};
            rank[d.bt_perm[B.state0 + k]] = k;  // k as sorted position: rank[state] = position
            invS[k] = tab.inv[B.state0 + k];
        }
        const F *tmg = tab.tm + (size_t)blk * MAXT * MAXT;
        for (int e = tid; e < NB * MAXT; e += NT) tmS[e] = tmg[e];
        for (int a = tid; a <= MAXT; a += NT) bptr[a] = d.bt_ptr[(size_t)blk * (MAXT + 1) + a];
        if (Tab<F>::split)
            for (int a = tid; a < MAXT; a += NT) rS[a] = tab.rstay[(size_t)blk * MAXT + a];
        __syncthreads();
        if (t2_in_smem)
            for (int k = tid; k < S; k += NT) {  // same-branch entries, node blocks source-major
                const Meta mk = meta[k];
                const int a0 = mk.time - (k - mk.j1);
                for (int y = 0; y < mk.m; y++)
                    t2s[mk.off + y * mk.m] =
                        tab.t2(B.t2_0 + mk.off + y * mk.m, tmS[(a0 + y) * MAXT + mk.time]);
            }
        const uint8_t *cls = d.colclass + I.col0 + B.start;
        const int *cvar = d.colvar + I.col0 + B.start;
        const F *inv = invS;
        const F *var = tab.var + B.var0;
        // FP32: the tree's emission references, added once the tree is done
        const double blkx = Tab<F>::split && tid == 0 ? d.blkext[blk] : 0.0;
        // column classes and variant rows, 32 columns per load, read back by shuffles
        int ccache = 0, vcache = 0, cbase = -32;
        auto colinfo = [&](int i, uint8_t &ci, int &vi) {
            if (i - cbase >= 32) {
                cbase = i;
                const int q = i + lane;
                ccache = q < B.len ? cls[q] : 0;
                vcache = q < B.len ? cvar[q] : 0;
            }
            ci = (uint8_t)__shfl_sync(0xffffffffu, ccache, i - cbase);
            vi = __shfl_sync(0xffffffffu, vcache, i - cbase);
        };
        __syncthreads();  // rank[] complete

        // ---- first column of the block
        if (bi == 0) {
            for (int k = tid; k < S; k += NT) {
                const F v = fw[k];  // priors (K1)
                col[c * maxS + k] = v;
                colT[rank[k]] = v;
            }
        } else {
            // previous column is normalised in col[c] (S1 entries)
            const int2 src = d.srcs[blk];
            const int *gp = d.gptr + B.gptr0;
            const int *gi = d.gidx + B.prev_state0;
            const F *dp = tab.dprob + B.prev_state0;
            const F *rr = tab.rrow + B.state0;
            const F *cr = tab.crow + B.state0;
            uint8_t c0;
            int v0;
            colinfo(0, c0, v0);
            const F *prev = col + c * maxS;
            for (int k = tid; k < S; k += NT) {
                F s = 0;
                for (int p = gp[k]; p < gp[k + 1]; p++) {
                    const int j = gi[p];
                    s += prev[j] * dp[j];
                }
                if (src.x != -1 && rr[k] > F(0)) s += prev[src.x] * rr[k];
                if (src.y != -1 && cr[k] > F(0)) s += prev[src.y] * cr[k];
                F v;
                if (c0 == COL_MASKED) v = s;
                else if (c0 == COL_INVARIANT) v = Tab<F>::split ? s - s * inv[k] : s * inv[k];
                else {
                    const F e = var[(size_t)v0 * S + k];
                    v = !Tab<F>::split ? s * e : e >= F(0) ? s - s * e : s * -e;
                }
                col[(c ^ 1) * maxS + k] = v;
                colT[rank[k]] = v;
            }
            c ^= 1;
        }

        // ---- remaining columns; iteration i also finalises column i-1
        for (int i = 1; i <= B.len; i++) {
            __syncthreads();  // A: column i-1 complete
            // each bin's sum, and its terms of tf[a] = sum_b tm[b][a] sum_b (lane a); the
            // terms are added in bin order below, so the result does not depend on NT
            for (int b = warp; b < NB; b += NW) {
                F s = 0;
                for (int p = bptr[b] + lane; p < bptr[b + 1]; p += 32) s += colT[p];
                s = warp_sum(s);
                tfrow[b][lane] = lane == 31 ? s : (lane < NB ? tmS[b * MAXT + lane] : F(0)) * s;
            }
            __syncthreads();  // B: bin rows of column i-1
            F norm = 0, tf = 0;
            for (int b = 0; b < NB; b++) {
                tf += tfrow[b][lane];
                norm += tfrow[b][31];
            }
            const F inv_norm = F(1) / norm;
            const F *cur = col + c * maxS;
            if (tid == 0) {
                acc.add((double)norm);
                if (!(norm > F(0))) report_error(d.err, ERR_ZERO_NORM, qi, bi, B.start + i - 1);
            }
            // finalise column i-1: normalised into the table (the instance's column 0
            // keeps the unnormalised prior, as the reference's table does)
            const bool write_prev = !(bi == 0 && i == 1);
            F *outp = fw + (size_t)(i - 1) * S;
            if (i == B.len) {
                for (int k = tid; k < S; k += NT) {
                    const F v = cur[k] * inv_norm;
                    if (write_prev) outp[k] = v;
                    col[c * maxS + k] = v;  // normalised, for the next switch
                }
                break;
            }
            uint8_t ci;
            int vrow;
            colinfo(i, ci, vrow);
            F *nxt = col + (c ^ 1) * maxS;
            for (int k0 = 0; k0 < S; k0 += NT) {
                const int k = k0 + tid;
                const bool valid = k < S;
                const Meta mk = meta[valid ? k : 0];
                const F tfb = __shfl_sync(0xffffffffu, tf, mk.time);
                if (valid) {
                    const F xk = cur[k];
                    if (write_prev) outp[k] = xk * inv_norm;
                    const F *nb = cur + mk.j1;
                    F s = tfb;
                    if (t2_in_smem) {
                        const F *row = t2s + mk.off;
                        const int m = mk.m;
                        int y = 0;
                        F s1 = 0;
                        for (; y + 1 < m; y += 2) {
                            s += row[0] * nb[y];
                            s1 += row[m] * nb[y + 1];
                            row += 2 * m;
                        }
                        if (y < m) s += row[0] * nb[y];
                        s += s1;
                    } else {
                        const int a0 = mk.time - (k - mk.j1);
                        for (int y = 0; y < mk.m; y++)
                            s += tab.t2(B.t2_0 + mk.off + y * mk.m, tmS[(a0 + y) * MAXT + mk.time]) * nb[y];
                    }
                    F v;
                    if (Tab<F>::split) {
                        s = xk + (s - rS[mk.time] * xk);  // stay term apart
                        if (ci == COL_MASKED) v = s;
                        else if (ci == COL_INVARIANT) v = s - s * inv[k];
                        else {
                            const F e = var[(size_t)vrow * S + k];
                            v = e >= F(0) ? s - s * e : s * -e;
                        }
                    } else {
                        const F e = ci == COL_MASKED ? F(1)
                                  : ci == COL_INVARIANT ? inv[k] : var[(size_t)vrow * S + k];
                        v = s * e;
                    }
                    v *= inv_norm;
                    nxt[k] = v;
                    colT[rank[k]] = v;
                }
            }
            c ^= 1;
        }
        if (Tab<F>::split && tid == 0) acc.extra += blkx;
        __syncthreads();
    }
    if (tid == 0 && d.lnl) {
        acc.flush();
        d.lnl[qi] = acc.lnl;
    }
}

// ---------------------------------------------------------------------------------------
// Register-resident variant for trees of up to KPT * (blockDim.x - 32 NRW) states.
//
// Warps 0 .. NRW-1 are reduction warps; the other threads own states
// k = (t - 32 NRW) + q * NTS (q < KPT), in state order, so lanes holding one node's states
// read the same neighbours and consecutive same-branch entries. A state's time, node span,
// row offset, time-sorted rank and invariant emission stay in registers for the tree's
// columns, and the next variant column's emissions are loaded a column ahead. Per column,
// two CTA barriers:
//   A  column i-1 complete in state order and time-sorted (each time bin a contiguous
//      range of the sorted copy). In parallel:
//        reduction warp r: the time bins of its share (FP32: a quarter of the bins; FP64:
//                whole bins holding about a quarter of the states) summed from the sorted
//                copy, then lane a forms its share of tf[a] = sum_b tm[b][a] bin[b] by
//                shuffles, lane 31 (tmatrix column of ones) its share of the norm
//        owners: the same-branch dot sum_y tmatrix2[a_y][k] col[j1 + y] of their states
//   B  the shares published: owners add them for their state's time and finish column i
//      (dot, stay, emission, rescaling). FP32 divides by the norm and writes column i-1;
//      FP64 scales by a power of two and reduction warp NRW-1 divides and writes the
//      previous column into the table.
// Every sum has an order fixed by the tree alone, so results do not depend on the block
// size or on the other problems of the batch. Products are summed with fused multiply-adds
// (explicit: this file compiles without FMA contraction): on GB300 a warp's FP64 instruction
// holds its sub-partition's FP64 pipe for about 64 cycles and a dependent FP64 step costs a
// few hundred cycles, so the plain FP64 path is shaped to issue few FP64 instructions in
// short dependent chains.
// FP32 pair arithmetic (value = hi + lo, |lo| <= ulp(hi) / 2) for the dominant path of
// the FP32 forward step. Within a tree the normalised column converges to the fixed point
// of the step; a rounding error of the step shifts that fixed point by about the error
// divided by (1 - the chain's contraction), and with stay probabilities near 1 the
// contraction is slow. The stay, emission and rescaling factors, which carry almost all of
// a state's mass from column to column, therefore run on pairs built from error-free
// transforms (Fast2Sum, and products split by FMA); the mass moving in from other states
// (a few percent) stays plain FP32.
struct F2 {
    float hi, lo;
};
__device__ __forceinline__ F2 f2_renorm(float a, float b) {  // |a| >= |b|
    const float s = a + b;
    return F2{s, b - (s - a)};
}
// (x.hi + x.lo) * (1 - r), 0 <= r < 1 (x.lo * r dropped: below the pair's precision)
__device__ __forceinline__ F2 f2_keep(F2 x, float r) {
    const float t = x.hi * r;
    const float h = x.hi - t;
    return f2_renorm(h, ((x.hi - h) - t) + x.lo);
}
// x * e
__device__ __forceinline__ F2 f2_mul(F2 x, float e) {
    const float p = x.hi * e;
    return f2_renorm(p, fmaf(x.hi, e, -p) + x.lo * e);
}
// x + s (any magnitudes: two-sum)
__device__ __forceinline__ F2 f2_add(F2 x, float s) {
    const float h = x.hi + s;
    const float bb = h - x.hi;
    const float err = (x.hi - (h - bb)) + (s - bb);
    return f2_renorm(h, err + x.lo);
}
// x + y, both pairs
__device__ __forceinline__ F2 f2_add2(F2 x, F2 y) {
    const F2 s = f2_add(x, y.hi);
    return f2_renorm(s.hi, s.lo + y.lo);
}

constexpr int NRW = 4;                      // reduction warps of the register variant
constexpr int RBINS = (MAXT - 1 + NRW - 1) / NRW;  // time bins per reduction warp (<= 8)

// FP64: the first time bin of reduction warp r (r = NRW: NB), the bins split by their
// states (positions of the time-sorted column) rather than by count; whole bins, at most
// RBINS per warp.
__device__ __forceinline__ int fp64_bin_split(const int *bptr, int NB, int r) {
    if (r >= NRW) return NB;
    const int S = bptr[NB];
    int prev = 0;
    for (int q = 1; q <= r; q++) {
        const int target = (q * S + NRW - 1) / NRW;
        int b = prev;
        while (b < NB && bptr[b] < target) b++;
        b = imax(b, NB - (NRW - q) * RBINS);
        prev = imin(b, prev + RBINS);
    }
    return prev;
}

template <typename F, int KPT>
__global__ void __launch_bounds__(512) k_forward_reg(BatchDev d, int maxS, int maxM, int t2_in_smem) {
    extern __shared__ double dyn_d[];
    const Tab<F> tab(d);
    const int qi = cta_instance(d);
    const InstDev I = d.inst[qi];
    const int T = I.T, NB = T - 1;
    const int tid = threadIdx.x, lane = tid & 31;
    const int NT = blockDim.x, NTS = NT - 32 * NRW;  // state owners: threads 32 NRW ..
    const int st = tid - 32 * NRW;                   // owner index (negative in reducers)
    const bool reducer = tid < 32 * NRW;
    const int rw = tid >> 5;                         // reducer warp: bins [blo, bhi)

    F *col = (F *)dyn_d;                       // [2][maxS] columns in state order
    F *colT = col + 2 * maxS;                  // [maxS] newest column, time-sorted
    F *t2s = colT + maxS;                      // [maxM] same-branch entries of the block
    float *lastlo = (float *)(t2s + maxM);     // FP32: low parts of a tree's last column
    __shared__ F tmS[MAXT * MAXT];             // [b][a] tmatrix; column 31 holds ones
    __shared__ F part[NRW][32][RBINS];         // reducers: per lane, its chunk's bin sums
    __shared__ F tfp[NRW][32];                 // each reducer's share of tf; [31]: of the norm
    __shared__ int bptr[MAXT + 1];
    __shared__ int fbin[NRW][32];              // reducers: first bin of each lane's chunk

    // the log-likelihood accumulates on one thread of reduction warp 1: after barrier B its
    // warp has nothing else to do before barrier A, so the FP64 frexp, product and periodic
    // log stay off the column's critical path (on warp 0 they delayed barrier A by about a
    // fifth of a column). Thread 0 keeps a second accumulator for the rare switch into a
    // fully specified tree; the two are summed at the end.
    LogAcc acc, acc0;
    const bool acc_thread = tid == 32;
    __shared__ double lnl0;
    int c = 0;                                 // buffer holding the current column
    // FP64: a column is computed from the previous one scaled by a power of two (the
    // exponent of its largest norm partial: exact, no division on the column's path) rather
    // than divided by its norm. Reduction warp NRW-1 (its own sub-partition where the owners
    // fill at most three warps) divides while the owners form the next column (fin_inv) and
    // writes the column normalised into the table at the start of the column after. A
    // tree's last column is normalised exactly for the switch, as before.
    constexpr bool pow2 = !Tab<F>::split;
    const bool finalizer = reducer && rw == NRW - 1;
    F fin_inv = F(0);
    bool fin_pending = false;

    for (int bi = 0; bi < I.ntrees; bi++) {
        const int blk = I.block0 + bi;
        const BlockDev &B = d.blocks[blk];
        const int S = B.S, len = B.len;
        F *fw = tab.fw + B.cell0;
        if (tid == NT - 32 && bi + 1 < I.ntrees) prefetch_tree<F>(d, tab, I, blk + 1);

        if (S == 0) {
            // fully specified tree: one state that carries over (sample_thread.cpp:201-206)
            F v;
            if (bi == 0) {
                v = fw[0];
                if (tid == 0) col[c * maxS] = v;
            } else {
                const int2 src = d.srcs[blk];
                const int *gp = d.gptr + B.gptr0;
                const int *gi = d.gidx + B.prev_state0;
                const F *dp = tab.dprob + B.prev_state0;
                const F *rr = tab.rrow + B.state0;
                const F *cr = tab.crow + B.state0;
                F sum = 0;
                if (tid < 32) {
                    for (int p = gp[0] + lane; p < gp[1]; p += 32) sum += col[c * maxS + gi[p]] * dp[gi[p]];
                    sum = warp_sum(sum);
                }
                if (tid == 0) {
                    if (src.x != -1 && rr[0] > F(0)) sum += col[c * maxS + src.x] * rr[0];
                    if (src.y != -1 && cr[0] > F(0)) sum += col[c * maxS + src.y] * cr[0];
                    acc0.add((double)sum);
                    col[c * maxS] = F(1);
                    fw[0] = F(1);
                }
                v = F(1);
            }
            if (Tab<F>::split && tid == 0) lastlo[0] = 0.0f;
            for (int i = 1 + tid; i < len; i += NT) fw[i] = v;
            __syncthreads();
            continue;
        }

        // ---- stage the tree: tmatrix, bins, owned states, reducer chunks
        const long long s0 = B.state0;
        const F *tmg = tab.tm + (size_t)blk * MAXT * MAXT;
        for (int e = tid; e < NB * MAXT; e += NT) {
            const int a = e & (MAXT - 1);
            tmS[e] = a == MAXT - 1 ? F(1) : tmg[e];
        }
        for (int a = tid; a <= MAXT; a += NT) bptr[a] = d.bt_ptr[(size_t)blk * (MAXT + 1) + a];
        int st_time[KPT], st_j1[KPT], st_m[KPT], st_off[KPT], st_rank[KPT];
        F st_inv[KPT], st_rs[KPT], x_own[KPT], e_next[KPT], dq[KPT];
        float x_lo[KPT];  // FP32 path: low parts of the owned states (pairs x_own + x_lo)
        auto owned = [&](int q) { return reducer ? -1 : st + q * NTS; };  // the reducer owns none
        auto valid = [&](int k) { return k >= 0 && k < S; };
#pragma unroll
        for (int q = 0; q < KPT; q++) {
            const int k = owned(q);
            const int kk = valid(k) ? k : 0;
            const StateInfo si = d.sinfo[s0 + kk];
            st_time[q] = si.time;
            st_j1[q] = si.j1;
            st_m[q] = valid(k) ? si.m : 0;
            st_off[q] = d.t2off[s0 + kk];
            st_inv[q] = tab.inv[s0 + kk];
            st_rs[q] = Tab<F>::split ? (F)tab.rstay[(size_t)blk * MAXT + si.time] : F(0);
            x_own[q] = F(0);
            x_lo[q] = 0.0f;
            e_next[q] = F(0);
            dq[q] = F(0);
        }
        // time-sorted rank of each state: bt_perm lists the states of each time in order
        for (int p = tid; p < S; p += NT) col[(c ^ 1) * maxS + d.bt_perm[s0 + p]] = (F)p;
        __syncthreads();  // tmS, bptr, ranks (parked in the free column buffer)
#pragma unroll
        for (int q = 0; q < KPT; q++) {
            const int k = owned(q);
            st_rank[q] = valid(k) ? (int)col[(c ^ 1) * maxS + k] : 0;
        }
        // reducer warp rw: bins [blo, bhi), sorted positions [plo, phi); lane l sums its
        // chunk of ceil((phi - plo) / 32) positions, lane b - blo adds bin b's chunk sums
        const int blo = !reducer ? 0 : sizeof(F) == 8 ? fp64_bin_split(bptr, NB, rw) : rw * NB / NRW;
        const int bhi = !reducer ? 0 : sizeof(F) == 8 ? fp64_bin_split(bptr, NB, rw + 1) : (rw + 1) * NB / NRW;
        const int plo = reducer ? bptr[blo] : 0, phi = reducer ? bptr[bhi] : 0;
        const int chunk = imax((phi - plo + 31) >> 5, 1);
        const int clo = imin(plo + lane * chunk, phi), chi = imin(clo + chunk, phi);
        int l0 = 0, l1 = -1;
        int o1 = 0, o2 = 0, nbc = 0;  // bin boundaries inside the chunk, bins it spans
        // FP64, one position per lane: the lane's bin starts at lane seg0, the warp's largest
        // bin holds segmax positions, bin blo + lane ends at lane blast (-1: empty or none)
        int seg0 = 0, segmax = 0, blast = -1;
        if (reducer) {
            int fb = blo;
            while (fb < bhi - 1 && bptr[fb + 1] <= clo) fb++;
            fbin[rw][lane] = fb;
            seg0 = bptr[fb] - plo;
            const int bl = blo + lane;
            const int bsize = bl < bhi ? bptr[bl + 1] - bptr[bl] : 0;
            segmax = __reduce_max_sync(0xffffffffu, bsize);
            blast = bsize > 0 ? bptr[bl + 1] - 1 - plo : -1;
            const int b = blo + lane;
            if (b < bhi && bptr[b + 1] > bptr[b]) {
                l0 = (bptr[b] - plo) / chunk;
                l1 = (bptr[b + 1] - 1 - plo) / chunk;
            }
            if (chi > clo) {
                int bb = fb;
                nbc = 1;
                o1 = o2 = chi - clo;
                while (bb < bhi - 1 && bptr[bb + 1] < chi) {
                    if (nbc == 1) o1 = bptr[bb + 1] - clo;
                    else if (nbc == 2) o2 = bptr[bb + 1] - clo;
                    nbc++;
                    bb++;
                }
            }
        }
        // the fast chunk sum handles chunks of up to 32 positions spanning up to 3 bins, eight
        // loads and three predicated sums at a time: FP32 only, where the adds are cheap. On
        // GB300 a warp's FP64 add occupies the FP64 pipe of its SM sub-partition for about 64
        // cycles whether its lanes are live or not, so FP64 sums each lane's positions in turn
        const bool fast_chunk =
            sizeof(F) == 4 && __all_sync(0xffffffffu, !reducer || (chunk <= 32 && nbc <= 3));
        if (t2_in_smem) {
#pragma unroll
            for (int q = 0; q < KPT; q++) {
                const int k = owned(q);
                if (!valid(k)) continue;
                const int m = st_m[q], off = st_off[q];
                const int a0 = st_time[q] - (k - st_j1[q]);
                for (int y = 0; y < m; y++)
                    t2s[off + y * m] = tab.t2(B.t2_0 + off + y * m, tmS[(a0 + y) * MAXT + st_time[q]]);
            }
        }
        const uint8_t *cls = d.colclass + I.col0 + B.start;
        const int *cvar = d.colvar + I.col0 + B.start;
        const F *var = tab.var + B.var0;
        // FP32: the tree's emission references, added once the tree is done
        const double blkx = Tab<F>::split && acc_thread ? d.blkext[blk] : 0.0;
        // reducers: the tree's rows of the stored time-bin sums (the address formed once per
        // tree: a per-column read of the tree's descriptor from global memory sat on the
        // reducers' path to barrier A)
        float *const bins_row = Tab<F>::split && reducer && d.bins32
                                    ? d.bins32 + (size_t)(I.col0 + B.start) * MAXT
                                    : nullptr;
        // column classes and variant rows, 32 columns per lane-window; the next window is
        // loaded when the current one is entered, so its loads overlap 32 columns of work
        int ccache, vcache, ncc, nvc, cbase = 0;
        {
            const int q = lane, q2 = 32 + lane;
            ccache = q < len ? cls[q] : 0;
            vcache = q < len ? cvar[q] : 0;
            ncc = q2 < len ? cls[q2] : 0;
            nvc = q2 < len ? cvar[q2] : 0;
        }
        auto colinfo = [&](int i, uint8_t &ci, int &vi) {  // i never decreases, steps <= 1
            if (i - cbase >= 32) {
                cbase += 32;
                ccache = ncc;
                vcache = nvc;
                const int q2 = cbase + 32 + lane;
                ncc = q2 < len ? cls[q2] : 0;
                nvc = q2 < len ? cvar[q2] : 0;
            }
            ci = (uint8_t)__shfl_sync(0xffffffffu, ccache, i - cbase);
            vi = __shfl_sync(0xffffffffu, vcache, i - cbase);
        };
        auto emit = [&](F sv, uint8_t ci, int vrow, int q, bool prefetched) -> F {
            if (ci == COL_MASKED) return sv;
            if (ci == COL_INVARIANT) return Tab<F>::split ? sv - sv * st_inv[q] : sv * st_inv[q];
            const F e = prefetched ? e_next[q] : var[(size_t)vrow * S + owned(q)];
            if (!Tab<F>::split) return sv * e;
            return e >= F(0) ? sv - sv * e : sv * -e;  // FP32: 1 - e_k / e_ref, or -e_k / e_ref
        };
        auto prefetch = [&](int i) {  // emissions of column i, if variant
            uint8_t c1;
            int v1;
            colinfo(i, c1, v1);
            if (c1 == COL_VARIANT)
#pragma unroll
                for (int q = 0; q < KPT; q++)
                    if (valid(owned(q))) e_next[q] = var[(size_t)v1 * S + owned(q)];
        };
        __syncthreads();  // t2s, fbin; the rank scratch is read
        // reducers: bin blo + lane's slot among the partials of chunk l0 (the chunk holding
        // its first position); every later chunk of the bin starts inside it (slot 0)
        const int slot0 = reducer && l0 <= l1 ? blo + lane - fbin[rw][l0] : 0;

        // ---- first column of the block
        if (bi == 0) {
#pragma unroll
            for (int q = 0; q < KPT; q++) {
                const int k = owned(q);
                if (!valid(k)) continue;
                const F v = fw[k];  // priors (K1)
                col[c * maxS + k] = v;
                colT[st_rank[q]] = v;
                x_own[q] = v;
            }
        } else {
            const int2 src = d.srcs[blk];
            const int *gp = d.gptr + B.gptr0;
            const int *gi = d.gidx + B.prev_state0;
            const F *dp = tab.dprob + B.prev_state0;
            const F *rr = tab.rrow + s0;
            const F *cr = tab.crow + s0;
            uint8_t c0;
            int v0;
            colinfo(0, c0, v0);
            const F *prev = col + c * maxS;
#pragma unroll
            for (int q = 0; q < KPT; q++) {
                const int k = owned(q);
                if (!valid(k)) continue;
                if constexpr (Tab<F>::split) {
                    // pairs: the previous column's values with their low parts, each
                    // deterministic move by its FP64 probability (kept as a complement near
                    // 1), the recombination rows (a small inflow) plain, then the emission
                    const double *dp64 = d.determprob + B.prev_state0;
                    F2 a{0.0f, 0.0f};
                    for (int p = gp[k]; p < gp[k + 1]; p++) {
                        const int j = gi[p];
                        const double pj = dp64[j];
                        const F2 xj{prev[j], lastlo[j]};
                        a = f2_add2(a, pj >= 0.5 ? f2_keep(xj, (float)(1.0 - pj)) : f2_mul(xj, (float)pj));
                    }
                    if (src.x != -1 && rr[k] > F(0)) a = f2_add(a, prev[src.x] * rr[k]);
                    if (src.y != -1 && cr[k] > F(0)) a = f2_add(a, prev[src.y] * cr[k]);
                    if (c0 == COL_INVARIANT) a = f2_keep(a, st_inv[q]);
                    else if (c0 != COL_MASKED) {
                        const F e = var[(size_t)v0 * S + k];
                        a = e >= F(0) ? f2_keep(a, e) : f2_mul(a, -e);
                    }
                    col[(c ^ 1) * maxS + k] = a.hi;
                    colT[st_rank[q]] = a.hi;
                    x_own[q] = a.hi;
                    x_lo[q] = a.lo;
                } else {
                    F sv = 0;
                    for (int p = gp[k]; p < gp[k + 1]; p++) {
                        const int j = gi[p];
                        sv = fma(prev[j], dp[j], sv);
                    }
                    if (src.x != -1 && rr[k] > F(0)) sv += prev[src.x] * rr[k];
                    if (src.y != -1 && cr[k] > F(0)) sv += prev[src.y] * cr[k];
                    const F v = emit(sv, c0, v0, q, false);
                    col[(c ^ 1) * maxS + k] = v;
                    colT[st_rank[q]] = v;
                    x_own[q] = v;
                    x_lo[q] = 0.0f;
                }
            }
            c ^= 1;
        }
        if (len > 1 && !reducer) prefetch(1);

        // ---- remaining columns; iteration i also finalises column i-1
        for (int i = 1; i <= len; i++) {
            __syncthreads();  // A: column i-1 complete
            const F *cur = col + c * maxS;
            F binv = F(0);  // reducers, lane b - blo: bin b of column i-1
            if (reducer) {
                if (pow2 && finalizer && fin_pending) {
                    // column i-2 (the other column buffer) normalised into the table
                    const F *x = col + (c ^ 1) * maxS;
                    F *o = fw + (size_t)(i - 2) * S;
                    for (int k = lane; k < S; k += 32) o[k] = x[k] * fin_inv;
                    fin_pending = false;
                }
                F bin = 0;  // lane b - blo: bin b
                if (sizeof(F) == 8 && chunk == 1) {
                    // FP64, one position per lane: an inclusive scan within each bin's lanes
                    // (log2 of the largest bin's size dependent adds, where a sum in order
                    // takes its size: each dependent FP64 step costs hundreds of cycles),
                    // then lane b - blo takes bin b's total from the bin's last lane
                    F v = plo + lane < phi ? colT[plo + lane] : F(0);
                    for (int o = 1; o < segmax; o <<= 1) {
                        const F x = __shfl_up_sync(0xffffffffu, v, o);
                        if (lane - o >= seg0) v += x;
                    }
                    const F t = __shfl_sync(0xffffffffu, v, blast & 31);
                    bin = blast >= 0 ? t : F(0);
                } else {
                    // chunk sums by bin (positions sorted by time)
                    if (fast_chunk) {
                        // eight loads at a time; three independent sums over the chunk's bin ranges
                        F a0 = 0, a1 = 0, a2 = 0;
                        const int len_c = chi - clo;
                        for (int j0 = 0; j0 < len_c; j0 += 8) {
                            F v[8];
#pragma unroll
                            for (int j = 0; j < 8; j++) v[j] = j0 + j < len_c ? colT[clo + j0 + j] : F(0);
#pragma unroll
                            for (int j = 0; j < 8; j++) {
                                const int jj = j0 + j;
                                a0 += jj < o1 ? v[j] : F(0);
                                a1 += (jj >= o1 && jj < o2) ? v[j] : F(0);
                                a2 += jj >= o2 ? v[j] : F(0);
                            }
                        }
                        if (nbc >= 1) part[rw][lane][0] = a0;
                        if (nbc >= 2) part[rw][lane][1] = a1;
                        if (nbc >= 3) part[rw][lane][2] = a2;
                    } else {
                        int bcur = fbin[rw][lane], j = 0, nextb = bptr[bcur + 1];
                        F a = 0;
                        for (int p = clo; p < chi; p++) {
                            while (p >= nextb) {
                                part[rw][lane][j++] = a;
                                a = F(0);
                                bcur++;
                                nextb = bptr[bcur + 1];
                            }
                            a += colT[p];
                        }
                        if (chi > clo) part[rw][lane][j] = a;
                    }
                    __syncwarp();
                    // the chunk partials of bin b, eight loads issued together, then added in
                    // order (the same additions as one at a time; the partials are >= 0, so
                    // the zeros past l1 change nothing)
                    for (int l = l0; l <= l1; l += 8) {
                        F v[8];
#pragma unroll
                        for (int t = 0; t < 8; t++)
                            v[t] = l + t <= l1 ? part[rw][l + t][l + t == l0 ? slot0 : 0] : F(0);
#pragma unroll
                        for (int t = 0; t < 8; t++) bin += v[t];
                    }
                }
                binv = bin;
                // this warp's share of tf[a] = sum_b tm[b][a] bin[b], its bins in order
                F tf = 0;
                if constexpr (sizeof(F) == 8) {
                    // two independent chains (even and odd bins)
                    F ta = 0, tb = 0;
#pragma unroll
                    for (int j = 0; j < RBINS; j++) {
                        const F g = __shfl_sync(0xffffffffu, bin, j);
                        if (blo + j < bhi) {
                            if (j & 1) tb = fma(tmS[(blo + j) * MAXT + lane], g, tb);
                            else ta = fma(tmS[(blo + j) * MAXT + lane], g, ta);
                        }
                    }
                    tf = ta + tb;
                } else {
#pragma unroll
                    for (int j = 0; j < RBINS; j++) {
                        const F g = __shfl_sync(0xffffffffu, bin, j);
                        if (blo + j < bhi) tf = fma(tmS[(blo + j) * MAXT + lane], g, tf);
                    }
                }
                tfp[rw][lane] = tf;
            } else {
                // same-branch dot of the owned states: sum_y tmatrix2[a_y][k] col[j1 + y]
#pragma unroll
                for (int q = 0; q < KPT; q++) {
                    const int k = owned(q);
                    F sv = 0;
                    if (valid(k)) {
                        const F *nb = cur + st_j1[q];
                        const int m = st_m[q];
                        if (t2_in_smem && sizeof(F) == 8) {
                            // FP64: four independent chains, four loads ahead
                            const F *row = t2s + st_off[q];
                            F a0 = 0, a1 = 0, a2 = 0, a3 = 0;
                            int y = 0;
                            for (; y + 3 < m; y += 4) {
                                const F r0 = row[0], r1 = row[m], r2 = row[2 * m], r3 = row[3 * m];
                                const F n0 = nb[y], n1 = nb[y + 1], n2 = nb[y + 2], n3 = nb[y + 3];
                                a0 = fma(r0, n0, a0);
                                a1 = fma(r1, n1, a1);
                                a2 = fma(r2, n2, a2);
                                a3 = fma(r3, n3, a3);
                                row += 4 * m;
                            }
                            if (y < m) a0 = fma(row[0], nb[y], a0);
                            if (y + 1 < m) a1 = fma(row[m], nb[y + 1], a1);
                            if (y + 2 < m) a2 = fma(row[2 * m], nb[y + 2], a2);
                            sv = (a0 + a1) + (a2 + a3);
                        } else if (t2_in_smem) {
                            // even terms into sv, odd into s1, four loads ahead
                            const F *row = t2s + st_off[q];
                            int y = 0;
                            F s1 = 0;
                            for (; y + 3 < m; y += 4) {
                                const F r0 = row[0], r1 = row[m], r2 = row[2 * m], r3 = row[3 * m];
                                const F n0 = nb[y], n1 = nb[y + 1], n2 = nb[y + 2], n3 = nb[y + 3];
                                sv = fma(r0, n0, sv);
                                s1 = fma(r1, n1, s1);
                                sv = fma(r2, n2, sv);
                                s1 = fma(r3, n3, s1);
                                row += 4 * m;
                            }
                            for (; y + 1 < m; y += 2) {
                                sv = fma(row[0], nb[y], sv);
                                s1 = fma(row[m], nb[y + 1], s1);
                                row += 2 * m;
                            }
                            if (y < m) sv = fma(row[0], nb[y], sv);
                            sv += s1;
                        } else {
                            const int a0 = st_time[q] - (k - st_j1[q]);
                            for (int y = 0; y < m; y++)
                                sv = fma(tab.t2(B.t2_0 + st_off[q] + y * m, tmS[(a0 + y) * MAXT + st_time[q]]), nb[y], sv);
                        }
                    }
                    dq[q] = sv;
                }
            }
            __syncthreads();  // B: tf and the norm of column i-1
            // the column's norm and its reciprocal where they are used: the owners, the
            // accumulator thread and (FP32) the reducers storing bin sums; on the FP64 path
            // the other reduction warps skip them, whose division held the FP64 pipe of the
            // sub-partitions the owners share
            F norm = 0, inv_norm = 0, scale = 0;
            if (!pow2 || i == len) {
                if (!reducer || acc_thread || Tab<F>::split) {
                    norm = tfp[0][MAXT - 1];
#pragma unroll
                    for (int r = 1; r < NRW; r++) norm += tfp[r][MAXT - 1];
                    inv_norm = F(1) / norm;
                }
                if (acc_thread) {
                    acc.add((double)norm);
                    if (!(norm > F(0))) report_error(d.err, ERR_ZERO_NORM, qi, bi, B.start + i - 1);
                }
            } else if constexpr (pow2) {
                // 2^(1023 - E), E the largest biased exponent of the partials: the scaled
                // column sums to [1, 8). The tree's log-likelihood is log(norm of its last
                // column) plus ln 2 times the sum of E - 1023 over its other columns
                // (column i's norm is the reference's norm times the scaled sum of column
                // i-1, so the sum of the reference's log norms telescopes).
                int E = 1;
#pragma unroll
                for (int r = 0; r < NRW; r++)
                    E = imax(E, (__double2hiint((double)tfp[r][MAXT - 1]) >> 20) & 0x7ff);
                E = imin(E, 2045);
                scale = (F)__hiloint2double((2046 - E) << 20, 0);
                if (acc_thread) acc.e += E - 1023;
                if (finalizer) {
                    // the reciprocal norm of column i-1, written into the table next column
                    static_assert(NRW == 4, "the FP64 norm sum is written for four warps");
                    const F nrm = (tfp[0][MAXT - 1] + tfp[1][MAXT - 1]) + (tfp[2][MAXT - 1] + tfp[3][MAXT - 1]);
                    fin_inv = F(1) / nrm;
                    fin_pending = !(bi == 0 && i == 1);
                    if (lane == 0 && !(nrm > F(0)))
                        report_error(d.err, ERR_ZERO_NORM, qi, bi, B.start + i - 1);
                }
            }
            // finalise column i-1: normalised into the table (the instance's column 0
            // keeps the unnormalised prior, as the reference's table does)
            const bool write_prev = !(bi == 0 && i == 1);
            if constexpr (Tab<F>::split) {
                // the stored column's time-bin sums, on the stored column's scale
                if (bins_row && blo + lane < bhi)
                    bins_row[(size_t)(i - 1) * MAXT + blo + lane] = write_prev ? binv * inv_norm : binv;
            }
            F *outp = fw + (size_t)(i - 1) * S;
            if (i == len) {
#pragma unroll
                for (int q = 0; q < KPT; q++) {
                    const int k = owned(q);
                    if (!valid(k)) continue;
                    F v = x_own[q] * inv_norm;
                    if constexpr (Tab<F>::split) {
                        const F2 x = f2_mul(F2{x_own[q], x_lo[q]}, inv_norm);
                        v = x.hi;
                        lastlo[k] = x.lo;  // the pair's low part, for the next switch
                    }
                    if (write_prev) outp[k] = v;
                    col[c * maxS + k] = v;  // normalised, for the next switch
                }
                break;
            }
            uint8_t ci;
            int vrow;
            colinfo(i, ci, vrow);
            F *nxt = col + (c ^ 1) * maxS;
            if (!reducer) {
#pragma unroll
                for (int q = 0; q < KPT; q++) {
                    const int k = owned(q);
                    if (!valid(k)) continue;
                    const F xk = x_own[q];
                    if (!pow2 && write_prev) outp[k] = xk * inv_norm;
                    const int tq = st_time[q];
                    F tfk;
                    if constexpr (pow2) {
                        static_assert(NRW == 4, "the FP64 share sum is written for four warps");
                        tfk = (tfp[0][tq] + tfp[1][tq]) + (tfp[2][tq] + tfp[3][tq]);
                    } else {
                        tfk = tfp[0][tq];
#pragma unroll
                        for (int r = 1; r < NRW; r++) tfk += tfp[r][tq];
                    }
                    const F sv = tfk + dq[q];
                    F v;
                    if constexpr (Tab<F>::split) {
                        // pairs: stay (1 - rs), plus the inflow, times the emission, rescaled
                        F2 x = f2_keep(F2{xk, x_lo[q]}, st_rs[q]);
                        x = f2_add(x, sv);
                        if (ci == COL_INVARIANT) x = f2_keep(x, st_inv[q]);
                        else if (ci != COL_MASKED)
                            x = e_next[q] >= 0.0f ? f2_keep(x, e_next[q]) : f2_mul(x, -e_next[q]);
                        x = f2_mul(x, inv_norm);
                        v = x.hi;
                        x_lo[q] = x.lo;
                    } else {
                        // the emission times the power of two (exact) off the chain of sv
                        const F f = ci == COL_MASKED ? scale
                                                     : (ci == COL_INVARIANT ? st_inv[q] : e_next[q]) * scale;
                        v = sv * f;
                    }
                    nxt[k] = v;
                    colT[st_rank[q]] = v;
                    x_own[q] = v;
                }
                if (i + 1 < len) prefetch(i + 1);
            }
            c ^= 1;
        }
        if (Tab<F>::split && acc_thread) acc.extra += blkx;
        __syncthreads();
    }
    if (tid == 0) {
        acc0.flush();
        lnl0 = acc0.lnl;
    }
    __syncthreads();
    if (acc_thread && d.lnl) {
        acc.flush();
        d.lnl[qi] = acc.lnl + lnl0;
    }
}

// ---------------------------------------------------------------------------------------
// The reference's dense test step (arghmm_forward_block_slow, sample_thread.cpp:301-337),
// FP64, one CTA per instance: every column of a local tree from the full S x S transition
// matrix, col2[k] = (sum_j col1[j] transmat[j][k]) emit[i][k], normalised by division. The
// matrix entries are TransMatrix::get (trans.h:64-83) formed where they are read from the
// table kernel's FP64 tables: the different-node entry tmatrix[a_j][b_k] for states on
// other nodes, the same-node row get_time(a, b, c, minage, true) on k's own node. Thread k
// sums over j in the reference's order. Tree switches, priors and the log-likelihood are
// the structured path's (arghmm_forward_switch, sample_thread.cpp:345-389).
__device__ double dense_block_sum(const double *v, int n, double *red) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
    double s = 0.0;
    for (int k = tid; k < n; k += blockDim.x) s += v[k];
    s = warp_sum(s);
    __syncthreads();  // red free
    if (lane == 0) red[warp] = s;
    __syncthreads();
    double t = 0.0;
    for (int w = 0; w < nw; w++) t += red[w];
    return t;
}

__global__ void __launch_bounds__(512) k_forward_dense(BatchDev d, int maxS) {
    extern __shared__ double dyn_d[];
    const int qi = cta_instance(d);
    const InstDev I = d.inst[qi];
    const int tid = threadIdx.x, lane = tid & 31, NT = blockDim.x;
    double *col = dyn_d;                         // [2][maxS]
    int *snode = (int *)(col + 2 * maxS);        // [maxS] node of each state
    int *stime = snode + maxS;                   // [maxS] time of each state
    __shared__ double tmS[MAXT * MAXT];
    __shared__ double red[16];
    LogAcc acc;
    int c = 0;  // buffer holding the current (normalised) column

    for (int bi = 0; bi < I.ntrees; bi++) {
        const int blk = I.block0 + bi;
        const BlockDev B = d.blocks[blk];
        const int S = B.S;
        double *fw = d.fw64 + B.cell0;
        if (S == 0) {
            // fully specified tree: one state that carries over (sample_thread.cpp:201-206)
            double v;
            if (bi == 0) {
                v = fw[0];
                if (tid == 0) col[c * maxS] = v;
            } else {
                const int2 src = d.srcs[blk];
                const int *gp = d.gptr + B.gptr0;
                const int *gi = d.gidx + B.prev_state0;
                const double *dp = d.determprob + B.prev_state0;
                const double *rr = d.recombrow + B.state0;
                const double *cr = d.recoalrow + B.state0;
                double sum = 0.0;
                if (tid < 32) {
                    for (int p = gp[0] + lane; p < gp[1]; p += 32) sum += col[c * maxS + gi[p]] * dp[gi[p]];
                    sum = warp_sum(sum);
                }
                if (tid == 0) {
                    if (src.x != -1 && rr[0] > 0.0) sum += col[c * maxS + src.x] * rr[0];
                    if (src.y != -1 && cr[0] > 0.0) sum += col[c * maxS + src.y] * cr[0];
                    acc.add(sum);
                    col[c * maxS] = 1.0;
                    fw[0] = 1.0;
                }
                v = 1.0;
            }
            for (int i = 1 + tid; i < B.len; i += NT) fw[i] = v;
            __syncthreads();
            continue;
        }
        for (int k = tid; k < S; k += NT) {
            const StateInfo si = d.sinfo[B.state0 + k];
            snode[k] = si.node;
            stime[k] = si.time;
        }
        const double *tmg = d.tm + (size_t)blk * MAXT * MAXT;
        for (int e = tid; e < MAXT * MAXT; e += NT) tmS[e] = tmg[e];
        __syncthreads();
        const uint8_t *cls = d.colclass + I.col0 + B.start;
        const int *cvar = d.colvar + I.col0 + B.start;
        auto emit = [&](int i, int k) -> double {
            const uint8_t ci = cls[i];
            if (ci == COL_MASKED) return 1.0;
            if (ci == COL_INVARIANT) return d.inv_lk[B.state0 + k];
            return d.varemit[B.var0 + (size_t)cvar[i] * S + k];
        };
        // first column: the priors, or the switch from the previous tree's last column
        double *cur = col + (c ^ 1) * maxS;
        if (bi == 0) {
            for (int k = tid; k < S; k += NT) cur[k] = fw[k];
        } else {
            const double *prev = col + c * maxS;
            const int2 src = d.srcs[blk];
            const int *gp = d.gptr + B.gptr0;
            const int *gi = d.gidx + B.prev_state0;
            const double *dp = d.determprob + B.prev_state0;
            const double *rr = d.recombrow + B.state0;
            const double *cr = d.recoalrow + B.state0;
            for (int k = tid; k < S; k += NT) {
                double s = 0.0;
                for (int p = gp[k]; p < gp[k + 1]; p++) s += prev[gi[p]] * dp[gi[p]];
                if (src.x != -1 && rr[k] > 0.0) s += prev[src.x] * rr[k];
                if (src.y != -1 && cr[k] > 0.0) s += prev[src.y] * cr[k];
                cur[k] = s * emit(0, k);
            }
            __syncthreads();
            const double norm = dense_block_sum(cur, S, red);
            if (tid == 0) {
                acc.add(norm);
                if (!(norm > 0.0)) report_error(d.err, ERR_ZERO_NORM, qi, bi, B.start);
            }
            for (int k = tid; k < S; k += NT) {
                cur[k] /= norm;
                fw[k] = cur[k];
            }
        }
        c ^= 1;
        for (int i = 1; i < B.len; i++) {
            __syncthreads();  // column i-1 complete
            const double *c1 = col + c * maxS;
            double *c2 = col + (c ^ 1) * maxS;
            for (int k = tid; k < S; k += NT) {
                const StateInfo sk = d.sinfo[B.state0 + k];
                const double *grow = d.gts + B.t2_0 + d.t2off[B.state0 + k];
                double s = 0.0;
                for (int j = 0; j < S; j++) {
                    const double p = snode[j] == sk.node ? grow[(j - sk.j1) * sk.m]
                                                         : tmS[stime[j] * MAXT + sk.time];
                    s += c1[j] * p;
                }
                c2[k] = s * emit(i, k);
            }
            __syncthreads();
            const double norm = dense_block_sum(c2, S, red);
            if (tid == 0) {
                acc.add(norm);
                if (!(norm > 0.0)) report_error(d.err, ERR_ZERO_NORM, qi, bi, B.start + i);
            }
            double *outp = fw + (size_t)i * S;
            for (int k = tid; k < S; k += NT) {
                c2[k] /= norm;
                outp[k] = c2[k];
            }
            c ^= 1;
        }
        __syncthreads();
    }
    if (tid == 0 && d.lnl) {
        acc.flush();
        d.lnl[qi] = acc.lnl;
    }
}

int forward_threads(int maxS) {
    if (maxS > 256) return 512;
    if (maxS > 128) return 256;
    return 128;
}


template <typename F>
size_t forward_smem(int maxS, int maxM) {
    return (size_t)(4 * maxS + maxM) * sizeof(F) + 16 + (size_t)maxS * (sizeof(Meta) + sizeof(int));
}

template <typename F>
void launch_old(const BatchDev &d, int maxM, cudaStream_t s) {
    const int maxS = imax(d.maxS, 1);
    maxM = imax(maxM, 1);
    // stage the same-branch rows in shared memory when they fit, else read them from L1/L2
    int t2_in_smem = forward_smem<F>(maxS, maxM) <= 200 * 1024;
    if (!t2_in_smem) maxM = 1;
    const size_t smem = forward_smem<F>(maxS, maxM);
    // opt in; static shared memory counts against 48 KB too
    if (!raise_dynamic_smem(k_forward<F>, smem)) return;
    k_forward<F><<<d.ninst, forward_threads(maxS), smem, s>>>(d, maxS, maxM, t2_in_smem);
    note_launch();
}

template <typename F, int KPT>
void launch_reg(const BatchDev &d, int nt, cudaStream_t s) {
    const int maxS = imax(d.maxS, 1);
    int maxM = imax(d.maxM, 1);
    auto bytes = [&](int m) { return (size_t)(3 * maxS + m) * sizeof(F) + (size_t)maxS * sizeof(float) + 16; };
    const int t2_in_smem = bytes(maxM) <= 200 * 1024;
    if (!t2_in_smem) maxM = 1;
    const size_t smem = bytes(maxM);
    if (!raise_dynamic_smem(k_forward_reg<F, KPT>, smem)) return;
    k_forward_reg<F, KPT><<<d.ninst, nt, smem, s>>>(d, maxS, maxM, t2_in_smem);
    note_launch();
}

// States per owner thread of the register variant (1, 2, 4 or 8; AWG_FORWARD_KPT overrides
// it for tuning); the CTA then has the reduction warp plus ceil(maxS / KPT) owners rounded
// up to whole warps. FP64 takes one state a thread while the CTA allows it: a warp's FP64
// instruction holds its sub-partition's FP64 pipe for about 64 cycles, so the same-branch
// dots run faster spread over more warps (config 0, 74 states: forward 28.6 -> 24.9 ms).
int reg_kpt(int maxS, int want, bool fp64 = false) {
    static const int env = [] {
        const char *e = getenv("AWG_FORWARD_KPT");
        return e ? atoi(e) : 0;
    }();
    if (!(want == 1 || want == 2 || want == 4 || want == 8)) want = env;
    int k = (want == 1 || want == 2 || want == 4 || want == 8) ? want
          : fp64 && maxS <= 32 * (16 - NRW) ? 1
          : maxS <= 64 ? 1 : maxS <= 768 ? 2 : maxS <= 1536 ? 4 : 8;
    while (k < 8 && (maxS + k - 1) / k > 384) k *= 2;
    return k;
}

template <typename F>
void launch(const BatchDev &d, cudaStream_t s, int want_kpt) {
    const int maxS = imax(d.maxS, 1);
    const int kpt = reg_kpt(maxS, want_kpt, sizeof(F) == 8);
    // the reduction warps plus ceil(maxS / KPT) owners in whole warps
    const int nt = 32 * NRW + imax(32, ((maxS + kpt - 1) / kpt + 31) / 32 * 32);
    if (nt > 512) launch_old<F>(d, d.maxM, s);
    else if (kpt == 1) launch_reg<F, 1>(d, nt, s);
    else if (kpt == 2) launch_reg<F, 2>(d, nt, s);
    else if (kpt == 4) launch_reg<F, 4>(d, nt, s);
    else launch_reg<F, 8>(d, nt, s);
}

}  // namespace

bool forward_writes_bins(int maxS, int maxM, int maxT, int kpt) {
    (void)maxM;
    (void)maxT;
    const int k = reg_kpt(imax(maxS, 1), kpt);
    return 32 * NRW + imax(32, ((imax(maxS, 1) + k - 1) / k + 31) / 32 * 32) <= 512;
}

void launch_forward_dense(const BatchDev &d, cudaStream_t s) {
    const int maxS = imax(d.maxS, 1);
    const size_t smem = 2 * (size_t)maxS * sizeof(double) + 2 * (size_t)maxS * sizeof(int);
    if (!raise_dynamic_smem(k_forward_dense, smem)) return;  // the launch reports it
    const int nt = imin(512, imax(32, (maxS + 31) / 32 * 32));
    k_forward_dense<<<d.ninst, nt, smem, s>>>(d, maxS);
    note_launch();
}

void launch_forward(const BatchDev &d, bool fp32, cudaStream_t s, int kpt) {
    if (fp32) launch<float>(d, s, kpt);
    else launch<double>(d, s, kpt);
}

}  // namespace awg

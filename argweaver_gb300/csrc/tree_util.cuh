// Device helpers shared by the emission kernel (tables.cu) and the ARG probability
// kernels (arg_prob.cu): JC69 branch probabilities, Felsenstein leaf partials and steps,
// and a warp-level bucketing of tree nodes into levels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace awg {
namespace {

// exp(-4/3 mu t), the exponential of prob_branch (emit.cpp:86-93), and the branch
// probabilities formed from it exactly as prob_branch forms them
__device__ __forceinline__ double branch_exp(double t, double mu) { return exp(-(4. / 3.) * mu * t); }
__device__ __forceinline__ double branch_mut(double e) { return .25 * (1.0 - e); }
__device__ __forceinline__ double branch_nomut(double e) { return .25 * (1.0 + 3. * e); }

template <typename F>
__device__ __forceinline__ void leaf_partial(uint8_t ch, F *v) {
    if (ch == 'N') { v[0] = v[1] = v[2] = v[3] = F(1); return; }
    v[0] = v[1] = v[2] = v[3] = F(0);
    const int x = (ch == 'A' || ch == 'a') ? 0 : (ch == 'C' || ch == 'c') ? 1
                : (ch == 'G' || ch == 'g') ? 2 : 3;
    v[x] = F(1);
}

// (P x)[a] for the JC69 matrix with off-diagonal m and diagonal nm: the reference's order
// (FAST false) or the structured form
template <bool FAST>
__device__ __forceinline__ void jc_apply(const double *x, double m, double nm, double *y) {
    if constexpr (FAST) {
        const double sum = (x[0] + x[1]) + (x[2] + x[3]);
        const double dlt = nm - m;
#pragma unroll
        for (int a = 0; a < 4; a++) y[a] = fma(dlt, x[a], m * sum);
    } else {
#pragma unroll
        for (int a = 0; a < 4; a++) {
            double p = 0;
#pragma unroll
            for (int b = 0; b < 4; b++) p += x[b] * (a == b ? nm : m);
            y[a] = p;
        }
    }
}

// Nodes bucketed by key (key < 0: left out), by one warp: list holds the nodes level by
// level, ascending node index within a level; ptr[l] is the start of level l and
// ptr[nlev] the end (nlev = largest key + 1, returned). cursor: n ints of scratch.
__device__ int warp_levels(const int *key, int n, int *list, int *ptr, int *cursor, int lane) {
    int kmax = -1;
    for (int i = lane; i < n; i += 32) kmax = max(kmax, key[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) kmax = max(kmax, __shfl_xor_sync(0xffffffffu, kmax, o));
    const int nlev = kmax + 1;
    for (int l = lane; l <= nlev; l += 32) ptr[l] = 0;
    __syncwarp();
    const unsigned lt = (1u << lane) - 1u;
    for (int base = 0; base < n; base += 32) {  // counts of level l into ptr[l + 1]
        const int k = base + lane < n ? key[base + lane] : -1;
        const unsigned m = __match_any_sync(0xffffffffu, k);
        if (k >= 0 && (m & lt) == 0) ptr[k + 1] += __popc(m);
        __syncwarp();
    }
    int carry = 0;  // prefix sums: ptr[l] = nodes on levels below l
    for (int b = 0; b <= nlev; b += 32) {
        const int l = b + lane;
        int v = l <= nlev ? ptr[l] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += y;
        }
        if (l <= nlev) ptr[l] = v + carry;
        if (l < nlev) cursor[l] = v + carry;
        carry += __shfl_sync(0xffffffffu, v, 31);
    }
    __syncwarp();
    for (int base = 0; base < n; base += 32) {
        const int i = base + lane;
        const int k = i < n ? key[i] : -1;
        const unsigned m = __match_any_sync(0xffffffffu, k);
        const int leader = __ffs(m) - 1;
        int pos = 0;
        if (k >= 0 && lane == leader) {
            pos = cursor[k];
            cursor[k] = pos + __popc(m);
        }
        pos = __shfl_sync(0xffffffffu, pos, leader);
        if (k >= 0) list[pos + __popc(m & lt)] = i;
        __syncwarp();
    }
    return nlev;
}

}  // namespace
}  // namespace awg

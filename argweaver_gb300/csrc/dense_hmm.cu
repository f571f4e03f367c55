// The dense HMM of the reference's ctypes layer (hmm.cpp:13-105): log-space forward,
// backward and posterior path sampling over a full transition matrix. Not the threading
// HMM (whose transitions are structured), but the same C ABI the reference exports for
// its Python layer (argweaver/argweaverc.py:42-56), so that layer finds every HMM entry
// point here.
//
// One CTA per call. Per column each output is a logsum (common.h:182-202) over one row or
// column of the matrix: a warp per output, the maximum first, then the sum of exp(v - max)
// over the terms within e^-15 of it (the reference's threshold), lane partials in index
// order and a butterfly, so every result has an order fixed by the sizes. The sampler is
// one warp walking the columns from the end, one uniform per column drawn on the host from
// libc rand() in the reference's order.

#include <cuda_runtime.h>

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "kernels.h"

namespace awg {

namespace {

constexpr unsigned FULL = 0xffffffffu;

template <typename V>
__device__ double warp_logsum(int n, V v) {
    const int lane = threadIdx.x & 31;
    double mx = -INFINITY;
    for (int j = lane; j < n; j += 32) mx = fmax(mx, v(j));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(FULL, mx, o));
    double s = 0.0;
    for (int j = lane; j < n; j += 32) {
        const double x = v(j) - mx;
        if (x > -15.0) s += exp(x);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
    return mx + log(s);
}

// forward_alg (hmm.cpp:26-43): fw[i][k] = logsum_j(fw[i-1][j] + trans[j][k]) + emit[i][k];
// transT[k][j] = trans[j][k] (a warp reads one output's terms contiguously)
__global__ void k_dense_forward(int n, int S, const double *transT, const double *emit,
                                double *fw) {
    const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5, lane = threadIdx.x & 31;
    for (int i = 1; i < n; i++) {
        const double *col1 = fw + (size_t)(i - 1) * S;
        for (int k = warp; k < S; k += nw) {
            const double *tk = transT + (size_t)k * S;
            const double v = warp_logsum(S, [&](int j) { return col1[j] + tk[j]; });
            if (lane == 0) fw[(size_t)i * S + k] = v + emit[(size_t)i * S + k];
        }
        __syncthreads();
    }
}

// backward_alg (hmm.cpp:48-64): bw[i][j] = logsum_k(trans[j][k] + bw[i+1][k] + emit[i+1][k])
__global__ void k_dense_backward(int n, int S, const double *trans, const double *emit,
                                 double *bw) {
    const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5, lane = threadIdx.x & 31;
    for (int i = n - 2; i >= 0; i--) {
        const double *col2 = bw + (size_t)(i + 1) * S;
        const double *e2 = emit + (size_t)(i + 1) * S;
        for (int j = warp; j < S; j += nw) {
            const double *tj = trans + (size_t)j * S;
            const double v = warp_logsum(S, [&](int k) { return tj[k] + col2[k] + e2[k]; });
            if (lane == 0) bw[(size_t)i * S + j] = v;
        }
        __syncthreads();
    }
}

// sample_hmm_posterior (hmm.cpp:76-95): path[i] drawn from exp(fw[i][j] + trans[j][k] -
// total), k = path[i+1], with the uniform u[i] (the first index whose running weight
// reaches u[i] times the weights' sum, as sample(), common.h:272-290). One warp.
__global__ void k_dense_sample(int n, int S, const double *transT, const double *fw,
                               const double *u, int *path) {
    const int lane = threadIdx.x & 31;
    const int chunk = (S + 31) / 32;
    const int lo = min(lane * chunk, S), hi = min(lo + chunk, S);
    for (int i = n - 2; i >= 0; i--) {
        const int k = path[i + 1];
        const double *tk = transT + (size_t)k * S;
        const double *col = fw + (size_t)i * S;
        const double total = warp_logsum(S, [&](int j) { return col[j] + tk[j]; });
        // each lane's contiguous chunk of weights, scanned across lanes
        double part = 0.0;
        for (int j = lo; j < hi; j++) part += exp(col[j] + tk[j] - total);
        double incl = part;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double y = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += y;
        }
        const double wsum = __shfl_sync(FULL, incl, 31);
        const double pick = u[i] * wsum;
        const unsigned hit = __ballot_sync(FULL, incl >= pick && hi > lo);
        int x = S - 1;
        if (hit) {
            const int src = __ffs(hit) - 1;
            const double excl = __shfl_sync(FULL, incl - part, src);
            if (lane == src) {
                double run = excl;
                int r = hi - 1;
                for (int j = lo; j < hi; j++) {
                    run += exp(col[j] + tk[j] - total);
                    if (run >= pick) { r = j; break; }
                }
                x = r;
            }
            x = __shfl_sync(FULL, x, src);
        }
        if (lane == 0) path[i] = x;
        __syncwarp();
    }
}

}  // namespace

bool dense_hmm(int which, int n, int S, double **trans, double **emit, double **tab, int *path,
               std::string &err) {
    if (n < 1 || S < 1 || !trans || !tab || (which != 2 && !emit) || (which == 2 && !path)) {
        err = "dense HMM: n and nstates must be positive and no table may be NULL";
        return false;
    }
    if (n < 2) return true;  // nothing to fill: the first (last) column is the caller's
    const size_t SS = (size_t)S * S, nS = (size_t)n * S;
    std::vector<double> t(SS), e(emit ? nS : 0), f(nS);
    for (int j = 0; j < S; j++)
        for (int k = 0; k < S; k++)
            t[which == 1 ? (size_t)j * S + k : (size_t)k * S + j] = trans[j][k];  // T for fwd/sample
    if (emit)
        for (int i = 0; i < n; i++) memcpy(&e[(size_t)i * S], emit[i], sizeof(double) * S);
    for (int i = 0; i < n; i++) memcpy(&f[(size_t)i * S], tab[i], sizeof(double) * S);
    std::vector<double> u;
    if (which == 2) {  // the reference's draws: rand()/RAND_MAX, last column first
        u.assign(n, 0.0);
        for (int i = n - 2; i >= 0; i--) u[i] = rand() / double(RAND_MAX);
    }
    double *dt = nullptr, *de = nullptr, *df = nullptr, *du = nullptr;
    int *dp = nullptr;
    bool ok = cudaMalloc(&dt, sizeof(double) * SS) == cudaSuccess &&
              cudaMalloc(&df, sizeof(double) * nS) == cudaSuccess &&
              (!emit || cudaMalloc(&de, sizeof(double) * nS) == cudaSuccess) &&
              (which != 2 || (cudaMalloc(&du, sizeof(double) * n) == cudaSuccess &&
                              cudaMalloc(&dp, sizeof(int) * n) == cudaSuccess));
    if (ok) {
        cudaMemcpy(dt, t.data(), sizeof(double) * SS, cudaMemcpyHostToDevice);
        cudaMemcpy(df, f.data(), sizeof(double) * nS, cudaMemcpyHostToDevice);
        if (emit) cudaMemcpy(de, e.data(), sizeof(double) * nS, cudaMemcpyHostToDevice);
        if (which == 0) {
            k_dense_forward<<<1, 512>>>(n, S, dt, de, df);
        } else if (which == 1) {
            k_dense_backward<<<1, 512>>>(n, S, dt, de, df);
        } else {
            cudaMemcpy(du, u.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
            cudaMemcpy(dp, path, sizeof(int) * n, cudaMemcpyHostToDevice);
            k_dense_sample<<<1, 32>>>(n, S, dt, df, du, dp);
        }
        note_launch();
        cudaError_t rc = cudaGetLastError();
        if (rc == cudaSuccess) rc = cudaDeviceSynchronize();
        if (rc != cudaSuccess) err = std::string("dense HMM kernel: ") + cudaGetErrorString(rc);
        ok = rc == cudaSuccess;
        if (ok && which == 2) {
            ok = cudaMemcpy(path, dp, sizeof(int) * n, cudaMemcpyDeviceToHost) == cudaSuccess;
        } else if (ok) {
            ok = cudaMemcpy(f.data(), df, sizeof(double) * nS, cudaMemcpyDeviceToHost) == cudaSuccess;
            if (ok)
                for (int i = 0; i < n; i++) memcpy(tab[i], &f[(size_t)i * S], sizeof(double) * S);
        }
    }
    cudaFree(dt);
    cudaFree(de);
    cudaFree(df);
    cudaFree(du);
    cudaFree(dp);
    if (!ok && err.empty()) err = "dense HMM: device allocation or copy failed";
    return ok;
}

}  // namespace awg

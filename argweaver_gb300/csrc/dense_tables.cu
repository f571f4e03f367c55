// Dense matrices of the reference's ctypes helpers, read out of the table kernel's (K1) and
// the emission kernel's (K2) FP64 outputs for one tree or one tree boundary:
//   transition  new_transition_probs (trans.cpp:1190-1208): log P(i -> j) within a tree,
//               TransMatrix::get (trans.h:64-83) over the caller's states;
//   switch      new_transition_probs_switch (trans.cpp:1212-1245): log P(i -> j) from the
//               previous tree's states to the next tree's, TransMatrixSwitch::get
//               (trans.h:207-219);
//   emissions   new_emissions (emit.cpp:1288-1301): P(column i | state j), every column
//               of the tree.
// K1 and K2 have already formed every number (the exponentials, the switch rows, the
// Felsenstein passes); these kernels gather them into the caller's state order, one thread
// per matrix entry, and take the logarithm where the reference does.

#include <cmath>
#include <string>

#include "awg_internal.h"
#include "kernels.h"

namespace awg {
namespace {

// block blk, states rows[r] -> cols[c] of the same tree
__global__ void k_dense_transition(BatchDev d, int blk, const int *rows, const int *cols,
                                   int nr, int nc, double *out) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)nr * nc) return;
    const int r = (int)(e / nc), c = (int)(e % nc);
    const BlockDev B = d.blocks[blk];
    const int j = rows[r], k = cols[c];
    const StateInfo sj = d.sinfo[B.state0 + j], sk = d.sinfo[B.state0 + k];
    double p;
    if (sj.node == sk.node)  // same branch: the row of target k, stride m over its sources
        p = d.gts[B.t2_0 + d.t2off[B.state0 + k] + (long long)(j - sk.j1) * sk.m];
    else
        p = d.tm[(size_t)blk * MAXT * MAXT + sj.time * MAXT + sk.time];
    out[e] = log(p);
}

// boundary into block blk: previous tree's state rows[r] -> this tree's state cols[c]
__global__ void k_dense_switch(BatchDev d, int blk, const int *rows, const int *cols, int nr,
                               int nc, double *out) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)nr * nc) return;
    const int r = (int)(e / nc), c = (int)(e % nc);
    const BlockDev B = d.blocks[blk];
    const int j = rows[r], k = cols[c];
    const int2 src = d.srcs[blk];  // {recombsrc, recoalsrc}
    double p;
    if (j == src.y) p = d.recoalrow[B.state0 + k];
    else if (j == src.x) p = d.recombrow[B.state0 + k];
    else p = d.determ[B.prev_state0 + j] == k ? d.determprob[B.prev_state0 + j] : 0.0;
    out[e] = log(p);
}

// block blk's columns first_col .. first_col + L - 1, states cols[c]
__global__ void k_dense_emissions(BatchDev d, int blk, int first_col, const int *cols, int nc,
                                  int L, double *out) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)L * nc) return;
    const int i = (int)(e / nc), c = (int)(e % nc);
    const BlockDev B = d.blocks[blk];
    const InstDev I = d.inst[B.inst];
    const long long col = I.col0 + B.start + first_col + i;
    const int k = cols[c];
    const uint8_t cls = d.colclass[col];
    double v;
    if (cls == COL_MASKED) v = 1.0;
    else if (cls == COL_INVARIANT) v = d.inv_lk[B.state0 + k];
    else v = d.varemit[B.var0 + (long long)d.colvar[col] * B.S + k];
    out[e] = v;
}

}  // namespace

int dense_tables(const BatchDev &d, int kind, const int *rows, int nr, const int *cols, int nc,
                 int ncolumns, double *out, cudaStream_t s, std::string &err) {
    const long long n = kind == DENSE_EMISSIONS ? (long long)ncolumns * nc : (long long)nr * nc;
    int *didx = nullptr;
    double *dout = nullptr;
    int derr[4] = {0, 0, 0, 0};
    auto fail = [&](const char *what, cudaError_t rc) {
        err = std::string(what) + ": " + cudaGetErrorString(rc);
        (void)cudaStreamSynchronize(s);
        if (didx) cudaFree(didx);
        if (dout) cudaFree(dout);
        return -3;
    };
    cudaError_t rc;
    if ((rc = cudaMalloc(&didx, sizeof(int) * (size_t)(nr + nc + 1))) != cudaSuccess)
        return fail("dense tables: index buffer", rc);
    if ((rc = cudaMalloc(&dout, sizeof(double) * (size_t)std::max(n, 1LL))) != cudaSuccess)
        return fail("dense tables: output buffer", rc);
    if (nr > 0 && (rc = cudaMemcpyAsync(didx, rows, sizeof(int) * nr, cudaMemcpyHostToDevice, s)) !=
                      cudaSuccess)
        return fail("dense tables: upload", rc);
    if (nc > 0 && (rc = cudaMemcpyAsync(didx + nr, cols, sizeof(int) * nc, cudaMemcpyHostToDevice,
                                        s)) != cudaSuccess)
        return fail("dense tables: upload", rc);
    if (n > 0) {
        const int nt = 256;
        const unsigned grid = (unsigned)((n + nt - 1) / nt);
        if (kind == DENSE_TRANSITION)
            k_dense_transition<<<grid, nt, 0, s>>>(d, 0, didx, didx + nr, nr, nc, dout);
        else if (kind == DENSE_SWITCH)
            k_dense_switch<<<grid, nt, 0, s>>>(d, 1, didx, didx + nr, nr, nc, dout);
        else
            k_dense_emissions<<<grid, nt, 0, s>>>(d, 0, 1, didx + nr, nc, ncolumns, dout);
        note_launch();
        if ((rc = cudaGetLastError()) != cudaSuccess) return fail("dense tables: kernel", rc);
        if ((rc = cudaMemcpyAsync(out, dout, sizeof(double) * n, cudaMemcpyDeviceToHost, s)) !=
            cudaSuccess)
            return fail("dense tables: download", rc);
    }
    if ((rc = cudaMemcpyAsync(derr, d.err, sizeof(derr), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return fail("dense tables: error record", rc);
    if ((rc = cudaStreamSynchronize(s)) != cudaSuccess) return fail("dense tables", rc);
    cudaFree(didx);
    cudaFree(dout);
    if (derr[0] != 0) {
        err = "dense tables: the table kernels recorded device error " + std::to_string(derr[0]) +
              " at tree " + std::to_string(derr[2]) + ", column " + std::to_string(derr[3]);
        return -3;
    }
    return 0;
}

}  // namespace awg

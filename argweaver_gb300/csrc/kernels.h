// Kernel launchers (all asynchronous on the given stream).
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "argweaver_gb300.h"
#include "awg_internal.h"

namespace awg {

// K1: per-block tables (states, transition matrix, same-branch rows, switch matrix,
// priors into forward column 0, invariant emissions); one CTA per local tree, or with a
// work counter (zeroed) a persistent kernel whose CTAs take units of `chunk` trees.
void launch_tables(const BatchDev &d, bool want32, cudaStream_t s, int *queue = nullptr,
                   int chunk = 1);
// K2: emissions of variant columns (Felsenstein pruning); as K1.
void launch_varemit(const BatchDev &d, bool want32, cudaStream_t s, int *queue = nullptr,
                    int chunk = 1);
// Whether K2's carve with FP64 per-state factors and 8-byte scratch (needed for FP64 and
// double-float emissions) fits this largest tree.
bool varemit_full_carve_fits(int maxnodes, int maxS);
// K3: forward pass, one CTA per instance; kpt: states per owner thread of the
// register-resident variant (0: chosen by the state count).
void launch_forward(const BatchDev &d, bool fp32, cudaStream_t s, int kpt = 0);
// K3 with the reference's dense test step (arghmm_forward_block_slow), FP64.
void launch_forward_dense(const BatchDev &d, cudaStream_t s);

// The reference's dense helper matrices of one tree (or one boundary) from the table and
// emission kernels' FP64 outputs, into out (host, row-major): DENSE_TRANSITION log P(rows[r]
// -> cols[c]) in tree 0; DENSE_SWITCH log P(rows[r] of tree 0 -> cols[c] of tree 1);
// DENSE_EMISSIONS P(column 1 + i | cols[c]) of tree 0 for i < ncolumns. Synchronous;
// 0 or -3 with err set (also when the table kernels recorded a device error).
enum { DENSE_TRANSITION = 1, DENSE_SWITCH = 2, DENSE_EMISSIONS = 3 };
int dense_tables(const BatchDev &d, int kind, const int *rows, int nr, const int *cols, int nc,
                 int ncolumns, double *out, cudaStream_t s, std::string &err);
// Whether K3 writes the FP32 columns' time-bin sums (BatchDev::bins32) for a batch of these
// largest sizes (the register-resident variant does; the fallback for the largest trees
// does not).
bool forward_writes_bins(int maxS, int maxM, int maxT, int kpt = 0);
// K4: stochastic traceback, one warp per instance; FP32 with bins32 set: the decomposed draw.
void launch_traceback(const BatchDev &d, bool fp32, cudaStream_t s);
// K5: backward pass fused with the posterior marginals, one CTA per instance.
void launch_backward(const BatchDev &d, bool fp32, double *bw_out, cudaStream_t s);

// Kernel attributes, set once per kernel and safe to call from several host threads (the
// serving loop launches from one thread per batch slot).
// Asks for the largest shared-memory carveout for a kernel: the default carveout can leave
// room for fewer CTAs per SM than the registers and threads allow.
void prefer_shared_fn(const void *kernel);
template <typename K>
inline void prefer_shared(K kernel) {
    prefer_shared_fn((const void *)kernel);
}
// Raises a kernel's dynamic shared-memory limit to at least `bytes` (the limit only grows).
// False when the runtime refuses (the launch then reports the error).
bool raise_dynamic_smem_fn(const void *kernel, size_t bytes);
template <typename K>
inline bool raise_dynamic_smem(K kernel, size_t bytes) {
    return raise_dynamic_smem_fn((const void *)kernel, bytes);
}

// Count of kernels launched by this library (process-wide).
long long kernel_launch_count();
void note_launch();

// The dense HMM of hmm.cpp:27-85 on the device: which 0 = forward_alg, 1 = backward_alg,
// 2 = sample_hmm_posterior (uniforms from libc rand(), last column first). Tables are the
// reference's row pointers; false with err set on failure.
bool dense_hmm(int which, int n, int nstates, double **trans, double **emit, double **tab,
               int *path, std::string &err);

// sample_recombinations (recomb.cpp:151-235) along a state path, on the device: the
// recombinations' columns, nodes (-1: the thread) and times in pos/node/time
// (cap entries); the count, or < 0 with err set. *used: the uniforms consumed.
int sample_recombinations(const awg_problem *p, const int *path, const double *u, int nu,
                          int *pos, int *node, int *time, int cap, int *used, std::string &err);

// Probabilities of a whole ARG (total_prob.cpp) on the device: what = 1 likelihood, 2 prior,
// 4 first-tree prior (bits combine); out[0..2] in that order. Trees as the reference's
// arrays (ntrees x nnodes parents and ages, ntrees x 4 SPRs, block lengths). 0, or < 0 with
// err set.
int arg_probabilities(const int *ptrees, const int *ages, const int *sprs, const int *blocklens,
                      int ntrees, int nnodes, int start_coord, const double *times, int T,
                      const double *popsizes, double rho, double mu, char *const *seqs,
                      int nseqs, int seqlen, int what, double *out, std::string &err);

}  // namespace awg

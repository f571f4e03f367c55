// Internal layout shared by the host plan (host_plan.cpp) and the kernels.
//
// A batch holds any number of threading problems ("instances"). Every local tree of every
// instance is one block. All per-block and per-state data live in batch-wide flat arrays
// in HBM; descriptors carry offsets into them.
//
// Forward-table layout (both precisions): per instance, column after column, max(S,1)
// entries per column (S = states of the column's local tree), exactly the packed layout of
// the reference's ArgHmmForwardTable rows (sample_thread.h:35-97).
#pragma once

#include <cstdint>

#include <vector_types.h>  // int2 / int4

#if defined(__CUDACC__)
#define AWG_HD __host__ __device__
#else
#define AWG_HD
#endif

namespace awg {

constexpr int MAXT = 32;        // time points supported (16, 20 and 32 in use)
constexpr int MAXNODES = 1024;  // nodes per local tree (512 leaves)
constexpr int MODEL_STRIDE = 6 * MAXT;  // doubles of model data per instance

// Offsets inside an instance's model block (doubles).
constexpr int M_TIMES = 0;              // times[T]
constexpr int M_POPSIZES = MAXT;        // popsizes[T]
constexpr int M_TIMESTEPS = 2 * MAXT;   // time_steps[T] (model.h:322-329)
constexpr int M_COALSTEPS = 3 * MAXT;   // coal_time_steps[2T] (model.cpp:9-23)
constexpr int M_CONST = 5 * MAXT;       // rho, mu, mintime, infinite-sites penalty (1: off)

// Column classes (find_invariant_sites / find_masked_sites, emit.cpp:30-58).
enum : uint8_t { COL_INVARIANT = 0, COL_MASKED = 1, COL_VARIANT = 2 };

struct InstDev {
    int T, internal, minage, nleaves, nnodes, nseqs, seqlen, ntrees;
    int block0;           // first block of this instance in the batch
    int pad;
    long long cell0;      // forward-table offset of column 0
    long long col0;       // offset into per-column arrays
    long long seq0;       // offset of the column-major sequences [seqlen][nseqs]
    long long model0;     // offset into the model array (MODEL_STRIDE per instance)
};

struct BlockDev {
    int inst, b, start, len;  // instance, tree index within it, first column, columns
    int S, S1;                // states of this tree and of the previous tree (b > 0)
    int nodes0, prev_nodes0;  // offsets of this / previous tree in the node array
    int root, prev_root;
    int spr[4];               // recomb_node, recomb_time, coal_node, coal_time
    int map0;                 // offset of this tree's node mapping (b > 0), else -1
    int nvar;                 // variant columns in the block
    int M;                    // same-branch row entries: sum over states of the node's states
    int minage;               // TransMatrix::minage of the block (filled by the table kernel)
    long long cell0;          // forward-table offset of the block's first column
    long long state0;         // offset of per-state arrays (max(S,1) slots per block)
    long long prev_state0;    // previous block's state0 (switch arrays sized S1 live there)
    long long gptr0;          // offset of the switch gather pointers [max(S,1)+1]
    long long t2_0;           // offset of the same-branch rows
    long long var0;           // offset of the block's variant emission rows
    long long vrow0;          // index of the block's first variant column among the batch's
};

// Per-state metadata: node, time, first state of the node (block-relative), node states.
struct StateInfo {
    int node, time, j1, m;
};

// Device views of a batch (all pointers are device memory).
struct BatchDev {
    int ninst, nblocks, maxS, maxT, maxnodes, maxM;
    int vardf;                   // FP32 path: variant columns formed in double-float and
                                 // rounded once (needs emit64's carve; off where that carve
                                 // does not fit: FP32 forms)
    int emit64;                  // some instance forms FP64 emission partials even on the
                                 // FP32 path (internal-branch or infinite-sites problems)
    const InstDev *inst;
    const int *order;            // [ninst] or NULL: CTA x of a per-instance kernel runs
                                 // instance order[x] (largest work first)
    const int *blkmap;           // [nblocks] or NULL: CTA x of a per-tree kernel builds
                                 // tree blkmap[x]
    BlockDev *blocks;
    const double *model;         // [ninst * MODEL_STRIDE]
    const int4 *nodes;           // {parent, child0, child1, age} per tree node
    const int *mapping;          // node maps
    const uint8_t *seqT;         // column-major sequences
    const uint8_t *colclass;     // per column
    const int *colvar;           // per column: variant row within its block, -1 otherwise

    // table kernel outputs
    StateInfo *sinfo;            // [total states]
    int *t2off;                  // [total states] block-relative offset of the node row
    int *bt_ptr;                 // [nblocks * (MAXT+1)] states grouped by time
    int *bt_perm;                // [total states] block-relative state indices
    double *tm;                  // [nblocks * MAXT * MAXT] tmatrix[a][b]
    double *gts;                 // [total M] get_time(a, b, c, same_node=true) rows
    double *inv_lk;              // [total states] invariant-site emission per state
    int *determ;                 // [total states] switch: target of state j of prev tree
    double *determprob;          // [total states]
    int2 *srcs;                  // [nblocks] {recombsrc, recoalsrc}
    double *recombrow, *recoalrow;  // [total states] dense rows over this block's states
    int *gptr;                   // [total states + nblocks] gather CSR pointers
    int *gidx;                   // [total states] gather sources (prev-tree state indices)
    double *varemit;             // [total variant cells] emissions of variant columns

    // FP32 tables of the chosen path. Quantities next to 1 are stored as their complements,
    // computed with expm1 in FP64, so FP32 keeps their information:
    //   t2d32    tmatrix2 without the no-recombination term of the diagonal
    //   rstay32  [nblocks * MAXT] 1 - norecombs[b]
    //   inv32    1 - e_k / e_ref for invariant sites, e_ref the block's largest emission
    //   lneref   [nblocks] log(e_ref), added to the log-likelihood per invariant column
    //   var32    1 - e_k / e_ref for variant columns too, e_ref the column's largest
    //            emission (formed in double-float: a column that varies only through
    //            missing calls has emissions equal to a few digits, which FP32 values lose)
    //   vref     [variant columns] e_ref / 4 of each variant column (its log is taken when
    //            the tree's share is summed)
    //   blkext   [nblocks] a tree's sum of those references over its columns (lneref per
    //            invariant column, log(vref) per variant column; not the instance's column 0),
    //            added to the log-likelihood once per tree
    float *tm32, *t2d32, *inv32, *var32, *determprob32, *recombrow32, *recoalrow32, *rstay32;
    double *lneref, *vref, *blkext;
    // [total columns * MAXT] or NULL: per stored FP32 forward column, its time-bin sums
    // (the fgroups of arghmm_forward_block, sample_thread.cpp:258-263), written by the
    // forward kernel for the traceback's decomposed draw
    float *bins32;

    // outputs
    double *fw64;                // forward table (FP64 path)
    float *fw32;                 // forward table (FP32 path)
    double *lnl;                 // [ninst] sum of log column norms
    double *post;                // posterior marginals (optional)
    const double *uniforms;      // [total columns] traceback draws
    const int *last_state;       // [ninst] or NULL: FP64 traceback's given last state (-1:
                                 // sampled as usual)
    int *path;                   // [total columns]
    int *err;                    // [4] first failure: code, instance, block, column
};

// Records the first failure (code, instance, block, column); later ones are dropped.
#if defined(__CUDACC__)
// Instance run by this CTA of a per-instance kernel.
__device__ __forceinline__ int cta_instance(const BatchDev &d) {
    return d.order ? d.order[blockIdx.x] : (int)blockIdx.x;
}

// Local tree built by this CTA of a per-tree kernel.
__device__ __forceinline__ int cta_block(const BatchDev &d) {
    return d.blkmap ? d.blkmap[blockIdx.x] : (int)blockIdx.x;
}

__device__ inline void report_error(int *err, int code, int inst, int blk, int col) {
    if (atomicCAS(err, 0, code) == 0) {
        err[1] = inst;
        err[2] = blk;
        err[3] = col;
    }
}
#endif

AWG_HD inline int imax(int a, int b) { return a > b ? a : b; }
AWG_HD inline int imin(int a, int b) { return a < b ? a : b; }

// Device error codes (written once into BatchDev::err, never trap).
enum : int {
    ERR_NONE = 0,
    ERR_SWITCH_NO_TARGET = 1,   // internal switch from a fully specified tree found no state
    ERR_SMEM_LIMIT = 2,         // a block exceeded the kernel's shared-memory plan
    ERR_ZERO_NORM = 3,          // a forward column summed to zero (reference asserts top > 0)
    ERR_PLAN_MISMATCH = 4,      // device state count disagrees with the host plan
    ERR_BOUNDS = 5,             // an index derived from the inputs fell outside its array
    ERR_WAIT_LIMIT = 6,         // a bounded wait for an asynchronous copy ran out
};

}  // namespace awg

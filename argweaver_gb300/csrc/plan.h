// Host-side plan of a batch: validated inputs packed into the flat arrays the kernels read.
#pragma once

#include <string>
#include <vector>

#include "argweaver_gb300.h"
#include "awg_internal.h"

namespace awg {

struct HostPlan {
    int ninst = 0, nblocks = 0, maxS = 1, maxnodes = 1, maxT = 0, maxlen = 1, maxM = 1;
    long long total_states = 0;  // sum of S over blocks
    long long total_cells = 0;   // forward-table cells of the batch
    long long total_cols = 0;    // columns of the batch
    long long total_M = 0;       // same-branch row entries
    long long total_var = 0;     // variant emission cells
    long long total_vcols = 0;   // variant columns
    long long total_nodes = 0;   // tree nodes (int4 each)
    long long total_map = 0;     // mapping ints
    long long total_seq = 0;     // sequence bytes
    std::vector<InstDev> inst;
    std::vector<BlockDev> blocks;
    std::vector<double> model;
    std::vector<int> nodes;      // 4 ints per node
    std::vector<int> mapping;
    std::vector<uint8_t> seqT;
    std::vector<uint8_t> colclass;
    std::vector<int> colvar;
};

// Where plan_fill writes the per-node, per-column and sequence arrays.
struct PlanDst {
    int *nodes;          // [total_nodes * 4]
    int *mapping;        // [max(total_map, 1)]
    uint8_t *seqT;       // [total_seq]
    uint8_t *colclass;   // [total_cols]
    int *colvar;         // [total_cols]
};

// Passes 1-2: validates the problems (sequence bytes too when check_seqs; plan_fill checks
// them anyway) and sizes the plan: instances, blocks and every offset except the
// variant-emission ones.
bool plan_layout(const awg_problem *probs, int n, HostPlan &plan, std::string &err,
                 bool check_seqs);
// Pass 3: fills the arrays into dst, the trees' roots and the variant-emission offsets,
// and checks every sequence byte (A, C, G, T or N); false with *err set on a bad byte.
bool plan_fill(const awg_problem *probs, int n, HostPlan &plan, const PlanDst &dst,
               std::string *err);
// Both, into the plan's own vectors; returns false with a message on bad input.
bool build_plan(const awg_problem *probs, int n, HostPlan &plan, std::string &err);

// The MODEL_STRIDE doubles of one instance's model (model.h:322-333, model.cpp:9-23).
void model_arrays(const double *times, const double *popsizes, int T, double rho, double mu,
                  double penalty, double *m);

// Threads the calling thread's planning may use (0: all hardware threads); callers that
// plan several batches at once share the cores this way.
void set_plan_threads(int n);

// Number of states of a local tree given by parent/age arrays (states.cpp:53-199).
int count_states(const int *parent, const int *age, int n, int T, bool internal, int minage,
                 int root_child0, int *M_out);

}  // namespace awg

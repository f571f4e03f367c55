// Host-side ARG surgery: adding a sampled thread to local trees (add_arg_thread,
// thread.cpp:272-422) and removing a leaf's thread (remove_arg_thread, thread.cpp:425-556).
#pragma once

#include <string>
#include <vector>

namespace awg {

// Local trees as flat arrays: parents and ages per tree (ntrees x nnodes), the SPR into
// each tree (ntrees x 4; row 0 unused), block lengths, node mappings from the previous
// tree (ntrees x nnodes, -1 rows for the first tree; empty: the default mapping), and the
// children in the order the trees keep them (empty: index order).
struct ThreadTrees {
    int ntrees = 0, nnodes = 0, start_coord = 0;
    std::vector<int> ptrees, ages, sprs, blocklens, mapping, c0, c1;
    std::vector<int> seqids;  // sequence of each leaf (empty: leaf i is sequence i)
};

// Adds the thread of a new leaf (state path over the trees' columns, external trees) and
// its recombinations (columns, nodes (-1: the new branch), times) to `a`, which grows by
// two nodes and one tree per recombination. False with err set on inconsistent input.
bool add_arg_thread(ThreadTrees &a, int T, const int *path, int seqlen, const int *rec_pos,
                    const int *rec_node, const int *rec_time, int nrec, std::string &err);

// Removes the thread of the leaf holding sequence `seqid` (remove_arg_thread,
// thread.cpp:425-556): every tree loses that leaf and its coalescence node, the last leaf
// and the two last nodes move into the holes, SPRs on the removed branch vanish and trees
// left without an SPR merge with their neighbour (remove_null_sprs, local_tree.cpp:409-469).
bool remove_arg_thread(ThreadTrees &a, int seqid, std::string &err);

}  // namespace awg

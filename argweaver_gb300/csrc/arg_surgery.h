// Host-side ARG surgery (thread.cpp): adding a sampled leaf thread (add_arg_thread,
// :272-422) and removing one (remove_arg_thread, :425-556); removal paths (:562-1002); the
// internal-branch cut (remove_arg_thread_path, :1481-1668) and regraft (add_arg_thread_path,
// :1204-1449); the times of an internal thread (arghmm_get_thread_times, :1718-1733).
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

// A removal path (one branch per tree) through the trees: from `node` of the block holding
// `pos` forward and backward (pos >= 0: sample_arg_removal_path, thread.cpp:772-790), or from
// `node` of the first tree forward (pos < 0: thread.cpp:793-799). rnd draws the branch at
// each split as the reference does (rand() < .5); rnd NULL (forward only) always keeps the
// passive branch, which is the leaf path (sample_arg_removal_leaf_path, thread.cpp:672-700).
bool sample_removal_path(const ThreadTrees &a, int node, long long pos, int (*rnd)(), int *path,
                         std::string &err);

// A removal path that prefers branches carrying recombinations (sample_arg_removal_path_recomb,
// thread.cpp:800-912): forward over branches with weight `pref` where the SPR's recombination
// node is, 1 - pref elsewhere, then a stochastic traceback; draws from rnd as the reference's.
bool sample_removal_path_recomb(const ThreadTrees &a, double pref, int (*rnd)(), int *path,
                                std::string &err);

// A removal path drawn uniformly from all paths by counting them back to front
// (sample_arg_removal_path_uniform, thread.cpp:914-1002); lntotal: the log path count.
bool sample_removal_path_uniform(const ThreadTrees &a, int (*rnd)(), int *path, double *lntotal,
                                 std::string &err);

// Cuts the ARG along a removal path (remove_arg_thread_path, thread.cpp:1481-1668): in every
// tree the path's branch is pruned and regrafted above the root at maxtime (the subtree the
// root's first child), SPRs and mappings follow, trees left without an SPR merge. With
// original_thread (one int per column), the removed thread as state indices of the cut trees
// (internal states with ntimes = maxtime - 1; 0 where a tree has none).
bool remove_thread_path(ThreadTrees &a, const int *removal_path, int maxtime,
                        int *original_thread, std::string &err);

// Regrafts the cut subtree of every partial tree (add_arg_thread_path, thread.cpp:1314-1449)
// at the state its internal thread path takes at the tree's first column (internal states,
// states.cpp:109-155, with minage), splits trees at the sampled recombinations, and renames
// the SPRs and mappings between neighbouring trees (thread.cpp:1204-1311). Node count stays.
// The time of each column's state of an internal thread path (arghmm_get_thread_times,
// thread.cpp:1718-1733); path and path_times are indexed by coordinate, from start_coord.
// Columns of a whole tree (no states) get -1.
bool thread_times(const ThreadTrees &a, int T, const int *path, int *path_times,
                  std::string &err);

bool add_thread_path(ThreadTrees &a, int T, int minage, const int *path, int seqlen,
                     const int *rec_pos, const int *rec_node, const int *rec_time, int nrec,
                     std::string &err);

}  // namespace awg

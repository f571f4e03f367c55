// Internal interface of the format readers (formats.cpp) for the trees handle.
#pragma once

#include <string>
#include <vector>

namespace awg {

// The local trees of an SMC file as read_local_trees (local_tree.cpp:1422-1540) keeps them:
// leaves in the file's NAMES order, children in newick order, block lengths uncompressed.
struct SmcArrays {
    int ntrees = 0, nnodes = 0, start_coord = 0;
    std::vector<int> ptrees, ages, sprs, blocklens, c0, c1;
};

bool read_smc_arrays(const char *path, const double *times, int ntimes, SmcArrays &out,
                     std::string &err);

}  // namespace awg

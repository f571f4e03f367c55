// Test-only: the device recombination sampler's per-instance routine (recomb_sampler.cuh)
// compiled for the host, so the CPU suite checks its logic against the reference's
// recombinations; the product runs it only on the device (recomb.cu).
#include <string>

#include "plan.h"
#include "recomb_sampler.cuh"

extern "C" int rs_host(const awg_problem *p, const int *path, const double *u, int nu, int *pos,
                       int *node, int *time, int cap, int *used) {
    awg::HostPlan plan;
    std::string err;
    if (!awg::build_plan(p, 1, plan, err)) return -100;
    awg::RsInstance in{(const int4 *)plan.nodes.data(), p->blocklens, path, u, p->ntrees,
                       p->nnodes, nu, p->start_coord, p->internal != 0, p->minage,
                       pos, node, time, cap};
    const double *m = plan.model.data();
    const awg::RsModel mm{p->ntimes, m + awg::M_TIMES, m + awg::M_TIMESTEPS,
                          m + awg::M_COALSTEPS, m + awg::M_POPSIZES, m[awg::M_CONST]};
    return awg::rs_sample(in, mm, used);
}

// Recombination sampling along a sampled thread (sample_recombinations, recomb.cpp:151-235)
// on the device: one thread per instance runs the sequential walk of recomb_sampler.cuh
// over the instance's columns (a walk of draws whose number depends on the draws; it
// consumes the caller's uniforms in order).

#include <cuda_runtime.h>

#include <cstdio>
#include <string>
#include <vector>

#include "kernels.h"
#include "plan.h"
#include "recomb_sampler.cuh"

namespace awg {

namespace {

__global__ void k_recomb_sample(RsInstance in, RsModel m, int *result) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int used = 0;
    const int rc = rs_sample(in, m, &used);
    result[0] = rc;
    result[1] = used;
}

}  // namespace

int sample_recombinations(const awg_problem *p, const int *path, const double *u, int nu,
                          int *pos, int *node, int *time, int cap, int *used, std::string &err) {
    if (!p || !path || (!u && nu > 0) || nu < 0 || cap < 0 || (cap > 0 && (!pos || !node || !time))) {
        err = "sample_recombinations: bad arguments";
        return -1;
    }
    HostPlan plan;
    if (!build_plan(p, 1, plan, err)) return -1;
    const int L = p->seqlen;

    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    size_t off = 0;
    const size_t o_nodes = off; off += al(sizeof(int) * plan.nodes.size());
    const size_t o_bl = off; off += al(sizeof(int) * p->ntrees);
    const size_t o_path = off; off += al(sizeof(int) * L);
    const size_t o_u = off; off += al(sizeof(double) * std::max(nu, 1));
    const size_t o_model = off; off += al(sizeof(double) * MODEL_STRIDE);
    const size_t o_out = off; off += al(sizeof(int) * 3 * std::max(cap, 1));
    const size_t o_res = off; off += al(sizeof(int) * 2);
    char *D = nullptr;
    cudaError_t rc = cudaMalloc(&D, off);
    if (rc != cudaSuccess) {
        err = std::string("sample_recombinations: cudaMalloc: ") + cudaGetErrorString(rc);
        return -2;
    }
    RsInstance in;
    in.nodes = (const int4 *)(D + o_nodes);
    in.blocklens = (const int *)(D + o_bl);
    in.path = (const int *)(D + o_path);
    in.u = (const double *)(D + o_u);
    in.ntrees = p->ntrees;
    in.nnodes = p->nnodes;
    in.nu = nu;
    in.start_coord = p->start_coord;
    in.internal = p->internal != 0;
    in.minage = p->minage;
    int *dout = (int *)(D + o_out);
    in.pos = dout;
    in.node = dout + std::max(cap, 1);
    in.time = dout + 2 * std::max(cap, 1);
    in.cap = cap;
    const double *dm = (const double *)(D + o_model);
    const RsModel m{p->ntimes, dm + M_TIMES, dm + M_TIMESTEPS, dm + M_COALSTEPS, dm + M_POPSIZES,
                    plan.model[M_CONST + 0]};
    int res[2] = {0, 0};
    do {
        if ((rc = cudaMemcpy(D + o_nodes, plan.nodes.data(), sizeof(int) * plan.nodes.size(),
                             cudaMemcpyHostToDevice)) != cudaSuccess) break;
        if ((rc = cudaMemcpy(D + o_bl, p->blocklens, sizeof(int) * p->ntrees,
                             cudaMemcpyHostToDevice)) != cudaSuccess) break;
        if ((rc = cudaMemcpy(D + o_path, path, sizeof(int) * L, cudaMemcpyHostToDevice)) != cudaSuccess) break;
        if (nu > 0 && (rc = cudaMemcpy(D + o_u, u, sizeof(double) * nu,
                                       cudaMemcpyHostToDevice)) != cudaSuccess) break;
        if ((rc = cudaMemcpy(D + o_model, plan.model.data(), sizeof(double) * MODEL_STRIDE,
                             cudaMemcpyHostToDevice)) != cudaSuccess) break;
        k_recomb_sample<<<1, 32>>>(in, m, (int *)(D + o_res));
        note_launch();
        if ((rc = cudaGetLastError()) != cudaSuccess) break;
        if ((rc = cudaMemcpy(res, D + o_res, sizeof(res), cudaMemcpyDeviceToHost)) != cudaSuccess) break;
        if (res[0] > 0) {
            if ((rc = cudaMemcpy(pos, in.pos, sizeof(int) * res[0], cudaMemcpyDeviceToHost)) != cudaSuccess) break;
            if ((rc = cudaMemcpy(node, in.node, sizeof(int) * res[0], cudaMemcpyDeviceToHost)) != cudaSuccess) break;
            rc = cudaMemcpy(time, in.time, sizeof(int) * res[0], cudaMemcpyDeviceToHost);
        }
    } while (false);
    cudaFree(D);
    if (rc != cudaSuccess) {
        err = std::string("sample_recombinations: ") + cudaGetErrorString(rc);
        return -3;
    }
    if (res[0] < 0) {
        err = res[0] == RS_BAD_STATE ? "sample_recombinations: a path entry is not a state of its tree"
            : res[0] == RS_OUT_OF_UNIFORMS ? "sample_recombinations: the uniforms ran out"
                                            : "sample_recombinations: more recombinations than cap";
        return -4;
    }
    if (used) *used = res[1];
    return res[0];
}

}  // namespace awg

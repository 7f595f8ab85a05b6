// sor_batch.cuh -- many Poisson solves in one persistent cluster launch (internal).
#pragma once

#include <map>
#include <vector>

#include "solver.cuh"

namespace pcd {

// Device descriptor of one instance (inputs filled by the host, statistics
// written back by the cluster that solved it).
struct BatchInst {
    int W, H, ld, khp;
    const double *b;
    double *phi;
    float w32[5];
    int in_smem;
    double tol;
    int max_iter;
    int sweeps, converged, cycles;
    double rel;
};

struct BatchArgs {
    BatchInst *inst;
    int count;
    unsigned *counter;            // work queue position, zeroed before the launch
    float *gscratch;              // planes of instances too large for shared memory
    size_t gscratch_per_cluster;  // floats per cluster
    int check_every, cycle_cap, warm_start;
    double drop;
};

struct BatchWorkspace {
    BatchInst *d_inst = nullptr;
    BatchInst *h_inst = nullptr;  // pinned
    int cap = 0;
    float *gscratch = nullptr;
    size_t gscratch_floats = 0;
    unsigned *counter = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    std::map<std::vector<long long>, cudaGraphExec_t> graphs;
    TileBatchWorkspace tiles;   // the batched tile form
    int reserve_inst(int count);
    void release();
};

// Grids whose widths are all multiples of 8 (ld of 4) run on batched tile
// passes unless the schedule is PCD_SCHED_CLUSTER or a cluster size is given;
// the others on clusters.  cluster: CTAs per cluster (16 or 8; 0 = 16)
int batch_solve_device(BatchWorkspace &ws, int dev, const pcd_instance *inst, int count, const pcd_solve_opts &o,
                       pcd_instance_stats *stats, pcd_batch_stats *bstats, cudaStream_t s, int cluster = 0);

}  // namespace pcd

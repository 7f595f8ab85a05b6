// sor_persist.cuh -- persistent shared-memory-resident red-black SOR (internal).
#pragma once

#include "solver.cuh"

namespace pcd {

constexpr int kPersistThreads = 512;

struct PersistArgs {
    int W, H, ld, G;
    const double *b;      // right-hand side (FP64 form)
    double *phi;          // solution, in/out
    const double *r64;    // initial FP64 residual (mixed form)
    double *xbuf;         // exchange rows: G x 2 slots x 2 rows x W (doubles)
    unsigned *flags;      // per-CTA epoch flags (G)
    unsigned *bar;        // grid barrier counter
    double *part;         // check partials: 2 x G x 3
    Ctl *ctl;
    int stop, max_iter, check_every;
    double tol;
    double w64[5];
    float w32[5];
    long long spin_limit;
    int withhold;         // failure test: CTA 0 never raises its epoch flag, so its
                          // neighbour's wait runs out (PCD_TIMEOUT); 0 in normal use
};

size_t persist_smem_bytes(int W, int H, int G, bool mixed);
// Picks the cooperative grid (one CTA per SM, >= 2 rows per band) and the
// dynamic shared memory; PCD_BAD_ARG when the bands do not fit on chip.
int persist_grid(int dev, int W, int H, bool mixed, int *G_out, size_t *smem_out);
int launch_persist(PersistArgs &a, bool mixed, size_t smem, cudaStream_t s);

}  // namespace pcd

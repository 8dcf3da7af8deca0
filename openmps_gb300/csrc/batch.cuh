// batch.cuh - many independent scenes advanced together.
//
// The scenes of a batch share one parameter set (tank, l0, physics) and live in one
// handle: their particles are concatenated, each scene padded with disabled particles to
// whole SELL chunks of 32 rows, and each scene owns its own block of search cells
// (cell index + scene * cells_per_scene), so every stage kernel runs over all scenes at
// once and produces, per scene, exactly what a single-scene handle produces.  The PPE of
// the batch is block diagonal; it is solved by one persistent kernel in which a thread
// block takes one scene at a time from a queue and runs the whole mixed-precision
// multigrid-preconditioned CG of that scene (hierarchy in shared memory, FP64 reliable
// updates and FP64 CG fallback) with block-level synchronisation only.
#pragma once

#include "mg.cuh"

namespace mpsgb {

struct BatchScene {
    int32_t row0, rows;  // first row and row count (multiple of kSellRows)
};

struct BatchSolveStats {
    int32_t iterations, updates, fallback, converged;
    int32_t fb_iterations, stalled, aborted, pad;
    double rr0, true_rr, bb, pad2;
};

struct BatchOps {
    CgOperands o;                // matrix and FP32/FP64 vectors of all scenes (global rows)
    const BatchScene* scenes;
    const int32_t* order;        // processing order of the scenes
    int32_t* queue;              // work counter (zero before each launch)
    int32_t nscenes;
    int32_t cells_per_scene;
    const int32_t* cell_count;
    const int32_t* cell_slot;
    int32_t max_per_cell;
    int32_t levels;              // cell levels of one scene (level 1 = its search cells)
    MgLevel lv[kMgMaxLevels + 1];  // level sizes (device pointers unused: shared memory)
    const int32_t* cell_xz;      // scene-local cell coordinates of each particle
    double* bins;                // 9 x n scratch of the level-1 products
    float* dinv0;                // omega_0 / a_ii per row
    double *r64, *p64, *Ap64;    // FP64 vectors of the CG fallback
    BatchSolveStats* stats;      // per scene
    int32_t* all_ok;             // 1 when every scene converged (stages after the solve)
    const DevStatus* status;
    double eps, delta2;
    int32_t criterion, max_iter;
};

// Shared memory of the batched solve for `threads` threads per block (0 if the scene
// hierarchy does not fit one block).
size_t batch_smem_bytes(const BatchOps& B, int threads);
// One launch: all scenes of the batch, `blocks` persistent blocks of `threads` threads.
cudaError_t launch_batch_solve(const BatchOps& B, int blocks, int threads, cudaStream_t s);
cudaError_t batch_prepare_device(size_t smem_bytes);
// Resident blocks per SM of the batched solve (0 if it cannot launch).
int batch_blocks_per_sm(int threads, size_t smem);

}  // namespace mpsgb

// mg.cuh - cell-aggregation multigrid preconditioner of the PPE solve.
//
// The unknowns are aggregated by the cells of the neighbour search (side NeighborLength
// >= the Laplacian radius), so two particles coupled by the PPE always sit in the same or
// in adjacent cells: the Galerkin operator P^T A P of the piecewise-constant aggregation
// is a 9-point stencil on the cell grid.  Coarser levels merge 2 x 2 cells and stay
// 9-point, so every level below the particles is a small structured grid held as nine
// coefficient planes (L2-resident).
//
// Preconditioner (symmetric, negative definite like A on the rows it acts on):
//   u = s_i * omega_0 * r_i / a_ii  +  P_1 V_1(P_1^T r)
// i.e. a (learned-)scaled Jacobi term on the particles plus a V(1,1) cycle with damped
// Jacobi on the cell levels.  The coarsest levels run inside one thread block from
// shared memory, and the coarsest of all (at most kMgDenseCells cells) is solved with
// its dense inverse.  Identity rows of the PPE (dummy, disabled and free-surface rows)
// get u = 0.
#pragma once

#include "cg.cuh"

namespace mpsgb {

constexpr int kMgMaxLevels = 14;
constexpr int kMgDenseCells = 128;     // the coarsest level, solved with its dense inverse
// The single-block kernel takes the coarsest levels whose planes, vectors and the dense
// inverse fit this much shared memory.
constexpr size_t kMgBottomBytes = 200 * 1024;
constexpr int kMgBottomThreads = 1024;
// Cycle levels between the particles and the bottom block that one down-sweep or one
// up-sweep kernel covers (deeper hierarchies run the remaining levels one kernel each).
constexpr int kMgFuseLevels = 3;
constexpr float kMgOmegaFine = 0.5f;   // Jacobi weight of the particle level
constexpr float kMgOmegaCoarse = 0.9f; // Jacobi weight of the cell levels (best of 0.6-0.9 measured)
// Weight of the coarse-grid correction at every cell level: piecewise-constant aggregation
// underestimates the smooth error components, and over-weighting their correction is the
// usual remedy for unsmoothed aggregation.  A CPU model of this cycle on the 320k
// dam break's PPE system gave 62 PCG iterations to 1e-8 at weight 1, 41-42 at 1.5-1.7 and
// 48 at 1.9 (84k tank: 41 -> 39).  The cycle stays symmetric, so CG applies.
constexpr float kMgCoarseWeight = 1.6f;

// Floats a cycle array of n values is allocated with (a multiple of four), so the bottom
// kernel can stage every array with 16-byte loads.
__host__ __device__ constexpr int64_t mg_round4(int64_t n) { return (n + 3) & ~static_cast<int64_t>(3); }

// One cell level: nine coefficient planes K[d * cells + c], d = 3 (dx + 1) + (dz + 1).
struct MgLevel {
    int32_t nx, nz, cells, pad;
    double* k64;  // FP64 Galerkin coefficients (setup)
    float* k32;   // the same in FP32 (cycle)
    float* dinv;  // omega / K_centre, 0 for cells without unknowns
    float* r;     // restricted residual
    float* e;     // correction
};

struct MgHierarchy {
    int32_t levels = 0;  // cell levels; level 1 = neighbour-search cells
    int32_t bottom = 0;  // first level of the single-block kernel
    MgLevel lv[kMgMaxLevels + 1] = {};  // lv[1..levels]
    float* dense = nullptr;             // inverse of the coarsest operator, cells^2
    // particle level (PPE rows in cell order: the rows of level-1 cell c are
    // cell_start[c] .. cell_start[c + 1] - 1)
    int32_t n = 0;
    const int32_t* cell_xz = nullptr;   // (cx << 16) | cz of each row's cell, -1: none
    const int32_t* cell_start = nullptr;
    float* dinv0 = nullptr;             // omega_0 / a_ii on active rows, 0 on identity rows
    const float* scale = nullptr;       // per-row scale of the Jacobi term (null: 1)
    double* bins = nullptr;             // 9 * n FP64 scratch of the level-1 product
    int32_t* active = nullptr;          // level-1 cells holding particles, ascending (per solve)
    int2* active_rows = nullptr;        // their row ranges [cell_start[c], cell_start[c + 1])
    int32_t* n_active = nullptr;        // their count (the total of the flag scan)
    int32_t* active_flag = nullptr;     // per level-1 cell: 1 with particles
    int32_t* active_pos = nullptr;      // exclusive prefix sum of active_flag (cells + 1)
    int32_t* scan_scratch = nullptr;
    DevStatus* status = nullptr;
};

// Level sizes for a gnx x gnz search grid (returns the level count, 0 if the grid is
// too large for the 16-bit cell coordinates or the level count).
int mg_plan(int gnx, int gnz, MgLevel* lv, int* bottom);
// Setup of one solve: level-1 operator from the FP64 matrix, the coarser Galerkin
// operators and the dense inverse.  Skips itself when the step already failed.
void mg_setup(const MgHierarchy& mg, const CgOperands& o, cudaStream_t s);
// The two halves of mg_setup: the level-1 operator (reads the matrix), then the coarser
// Galerkin operators and the dense inverse (read only the level-1 operator), which can
// run beside other work that does not use the hierarchy.
void mg_setup_level1(const MgHierarchy& mg, const CgOperands& o, cudaStream_t s);
void mg_setup_coarse(const MgHierarchy& mg, cudaStream_t s);
int mg_setup_launches(const MgHierarchy& mg);
// u = M r.  `mode` gates the kernels on the solve state like the PCG kernels: 0 init,
// 1 iteration, 2 after a reliable update (see pcg_skip).  With `fuse_axpy` (mode 1) the
// iteration's vector updates run in the restriction kernel, which then produces r.
void mg_apply(const MgHierarchy& mg, const CgScalars* S, int mode, const float* r, float* u,
              cudaStream_t s, const CgOperands* fuse_axpy = nullptr);
int mg_apply_launches(const MgHierarchy& mg);
// Shared-memory bytes the single-block kernels need (opt-in set once per device).
cudaError_t mg_prepare_device();

// ------------------------------------------------------ 9-point cell stencils
// The 9-point gathers are branchless: a neighbour outside the grid is clamped to a valid
// cell, and its coefficient is zero (no particle can sit outside the grid), so all the
// loads of a cell issue at once.
__device__ __forceinline__ int clampi(int v, int hi) { return min(max(v, 0), hi); }


// Residual of level f after the pre-smoothing x = dinv * r, summed over the children of
// coarse cell (X, Z) (the restriction of the piecewise-constant aggregation).
__device__ __forceinline__ float child_residuals(int nx, int nz, int cells, const float* k,
                                                 const float* dinv, const float* r, int X, int Z) {
    float sum = 0.0f;
#pragma unroll
    for (int a = 0; a < 2; a++) {
#pragma unroll
        for (int b = 0; b < 2; b++) {
            const int cx = 2 * X + a, cz = 2 * Z + b;
            const bool valid = cx < nx && cz < nz;
            const int ccx = min(cx, nx - 1), ccz = min(cz, nz - 1);
            const int ch = ccx * nz + ccz;
            float res = r[ch];
#pragma unroll
            for (int dx = -1; dx <= 1; dx++) {
#pragma unroll
                for (int dz = -1; dz <= 1; dz++) {
                    const int nb = clampi(ccx + dx, nx - 1) * nz + clampi(ccz + dz, nz - 1);
                    res -= k[((dx + 1) * 3 + dz + 1) * cells + ch] * (dinv[nb] * r[nb]);
                }
            }
            sum += valid ? res : 0.0f;
        }
    }
    return sum;
}

// Residual of fine cell (cx, cz) after the pre-smoothing x = dinv * r (0 outside the grid):
// one child's share of child_residuals.
__device__ __forceinline__ float child_residual(int nx, int nz, int cells, const float* k,
                                                const float* dinv, const float* r, int cx, int cz) {
    const bool valid = cx < nx && cz < nz;
    const int ccx = min(cx, nx - 1), ccz = min(cz, nz - 1);
    const int ch = ccx * nz + ccz;
    float res = r[ch];
#pragma unroll
    for (int dx = -1; dx <= 1; dx++) {
#pragma unroll
        for (int dz = -1; dz <= 1; dz++) {
            const int nb = clampi(ccx + dx, nx - 1) * nz + clampi(ccz + dz, nz - 1);
            res -= k[((dx + 1) * 3 + dz + 1) * cells + ch] * (dinv[nb] * r[nb]);
        }
    }
    return valid ? res : 0.0f;
}

// Post-smoothed correction of fine cell (cx, cz): x = dinv r + w e_parent (w the coarse
// weight), then one Jacobi step; ce(px, pz) returns the coarse correction of parent cell
// (px, pz).
template <class CoarseE>
__device__ __forceinline__ float smoothed_correction_at(int nx, int nz, int cells, const float* k,
                                                        const float* dinv, const float* r, int cx, int cz,
                                                        CoarseE ce) {
    const int ch = cx * nz + cz;
    const float rc = r[ch];
    const float xc = dinv[ch] * rc + kMgCoarseWeight * ce(cx >> 1, cz >> 1);
    float res = rc;
#pragma unroll
    for (int dx = -1; dx <= 1; dx++) {
#pragma unroll
        for (int dz = -1; dz <= 1; dz++) {
            const int nx_ = clampi(cx + dx, nx - 1), nz_ = clampi(cz + dz, nz - 1);
            const int nb = nx_ * nz + nz_;
            const float xn = dinv[nb] * r[nb] + kMgCoarseWeight * ce(nx_ >> 1, nz_ >> 1);
            res -= k[((dx + 1) * 3 + dz + 1) * cells + ch] * xn;
        }
    }
    return xc + dinv[ch] * res;
}

// The same with the coarse corrections in a plane of row length cnz.
__device__ __forceinline__ float smoothed_correction(int nx, int nz, int cells, const float* k,
                                                     const float* dinv, const float* r, int cnz,
                                                     const float* ce, int ch) {
    const int cx = ch / nz, cz = ch - (ch / nz) * nz;
    return smoothed_correction_at(nx, nz, cells, k, dinv, r, cx, cz,
                                  [&](int px, int pz) { return ce[px * cnz + pz]; });
}

// Gate of a preconditioned-solve kernel: mode 0 after init, 1 an iteration, 2 after a
// reliable update.
__device__ __forceinline__ bool pcg_skip(const CgScalars* S, int mode) {
    if (S->converged || S->aborted) return true;
    if (mode == 1) return S->iter >= S->max_iter || S->stalled;
    if (mode == 2) return !S->do_update;
    return false;
}

}  // namespace mpsgb

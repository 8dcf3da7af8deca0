// common.cuh - device-side layout and helpers of the GB300 MPS time step.
//
// Data layout in HBM (one scene, N particles, original particle order):
//   state   SoA FP64 x, z, u, w, p, n (+ int32 type), wall targets, nWithoutSpp,
//           ecs, originalX, du scratch.
//   cells   dense buckets cell_count[nx*nz], cell_slot[nx*nz*maxPerCell] like the
//           reference Grid (src/OpenMps/Grid.hpp:76, :140-150); each bucket is sorted
//           to ascending particle index after the parallel fill.
//   lists   neighbour lists in transposed padded ELL form: entry k of row i lives at
//           [k * N + i], so consecutive threads (rows) touch consecutive addresses.
//           Row capacity is the reference's own bound 9 * maxPerCell
//           (Computer.hpp:1763-1765).
//   PPE     the matrix in compact sliced ELL "SELL-32": rows grouped in chunks of 32
//           (one warp, one lane per row), each chunk column-major, so a warp reads 32
//           consecutive entries per load; chunk c starts at off[c] (prefix sum of the
//           chunk sizes), so the whole matrix is a dense stream of about nnz entries.
//           Columns are ascending within a row next to FP64 values, and the FP32
//           solver reads {column, FP32 value} pairs from one 8-byte array.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/mps.h"

namespace mpsgb {

constexpr int kBlock = 256;

// device status bits
constexpr int kStatusCellOverflow = 1;
constexpr int kStatusDeviceCheck = 2;
constexpr int kStatusCgNotConverged = 4;
constexpr int kStatusNonFinite = 8;

// Per-scene constants (Environment.hpp:129-216, Grid.hpp:137-150), passed by value.
struct SceneConst {
    int32_t n;
    uint32_t flags;
    int32_t gnx, gnz, max_per_cell;
    int32_t nb_stride;   // neighbour row capacity (9 * max_per_cell)
    int32_t ppe_stride;  // PPE row capacity (nb_stride + 1)
    int32_t guard;       // 1 inside a full step: stages skip themselves after a failure
    int32_t nchunks;     // PPE chunks of kSellRows rows
    int32_t cells_per_scene;  // gnx * gnz: cells of one scene
    int32_t nscenes;          // scenes of a batch (1 for a single scene)
    int32_t pad1;
    double l0, re, re2, re_lap, rl2;
    double nl, nl2_lo, nl2_hi;  // neighbour length and a guard band around nl^2
    double n0, lambda, n0_lap, lambda_lap;
    double rho, nu, g, surface_ratio, max_dt, max_dx;
    double min_x, min_z;
};

// Time of the step in flight (Environment::t, ::dt); lives in device memory so that
// the CFL time step (DetermineDt) needs no host round trip.
struct StepScalars {
    double t;
    double dt;
    unsigned long long max_u2_bits;  // max |u|^2 of DetermineDt (bit pattern of a non-negative double)
    double pad;
};

struct DevStatus {
    int flags;
    int disabled;
    int check_index;
    int pad;
    unsigned long long nb_total;  // neighbour-list entries of the last search
    unsigned long long ppe_nnz;   // nonzeros of the last PPE assembly
};

// Adds v over the warp and lets lane 0 add it to *dst (few atomics per kernel).
__device__ __forceinline__ void warp_add_u64(unsigned long long* dst, unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(dst, v);
}

struct DeviceState {
    int32_t* type;
    double *x, *z, *u, *w, *p, *nd;
    double *wall_x, *wall_z;
    double *n_wo_spp, *ecs, *ox, *oz, *dux, *duz;
    int32_t *cell_count, *cell_slot;
    int32_t* cell_xz;  // (cx << 16) | cz of each particle's cell at the last search, -1: none
    const int32_t* scene_of;  // batch: scene of each particle (its cells start at
                              // scene * cells_per_scene); null for a single scene
    int32_t *nb_count, *nb;
    int32_t *ppe_len, *ppe_col_tmp;
    double *ppe_val_tmp, *ppe_b, *ppe_x;
    int32_t *ppe_chunk, *ppe_off, *scan_scratch;  // chunk sizes, chunk offsets
    int32_t* ppe_col;                              // SELL-32 columns
    double* ppe_val;                               // SELL-32 FP64 values
    uint2* ppe_cv32;                               // SELL-32 {column, FP32 value}
    StepScalars* step;
    DevStatus* status;
    const int32_t* solve_ok;  // converged flag of the last PPE solve
};

// --------------------------------------------------------------- helpers
// uBLAS inner_prod of 2-vectors: t = 0; t += a0*b0; t += a1*b1, each op rounded.
__device__ __forceinline__ double dot2(double a0, double a1, double b0, double b1) {
    return __dadd_rn(__dadd_rn(0.0, __dmul_rn(a0, b0)), __dmul_rn(a1, b1));
}

// Particle::W (Particle.hpp:71-75)
__device__ __forceinline__ double weight(double r, double re) {
    return ((0 < r) && (r < re)) ? __dadd_rn(__ddiv_rn(re, r), -1.0) : 0.0;
}

__device__ __forceinline__ bool has_flag(uint32_t flags, uint32_t f) { return (flags & f) != 0u; }

// A cell overflow or a failed bounds check ends the step after the search
// (the reference throws from Grid::Store, Grid.hpp:314-318).
__device__ __forceinline__ bool step_failed(const SceneConst& sc, const DeviceState& st) {
    return sc.guard && (st.status->flags & (kStatusCellOverflow | kStatusDeviceCheck)) != 0;
}

// A failed PPE solve ends the step before the pressure is assigned (Computer.hpp:1424-1428).
__device__ __forceinline__ bool solve_failed(const SceneConst& sc, const DeviceState& st) {
    return sc.guard && (step_failed(sc, st) || *st.solve_ok == 0);
}

__device__ __forceinline__ int64_t ell(int k, int n, int i) {
    return static_cast<int64_t>(k) * n + i;
}

// SELL-32: rows in chunks of 32 (one warp, one lane per row); entry k of the chunk's row
// r sits at chunk_off + 32 k + r, so a warp's load at step k reads 32 consecutive
// entries.  A chunk reserves 32 x (its longest row) entries.
constexpr int kSellRows = 32;

__host__ __device__ __forceinline__ int64_t sell_index(int64_t chunk_off, int r, int k) {
    return chunk_off + static_cast<int64_t>(k) * kSellRows + r;
}

__host__ __device__ __forceinline__ int64_t sell_chunk_size(int maxlen) {
    return static_cast<int64_t>(maxlen) * kSellRows;
}

__host__ __device__ __forceinline__ int64_t sell_chunks(int64_t n) {
    return (n + kSellRows - 1) / kSellRows;
}

inline int grid_for(int64_t n, int block = kBlock) {
    return static_cast<int>((n + block - 1) / block);
}

// ------------------------------------------------------ launchers (host side)
// grid.cu
void launch_bucket(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
void launch_cell_sort(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
void launch_neighbors(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
void launch_status_counters_reset(DevStatus* st, cudaStream_t s);
// stages.cu
void launch_set_dt(const SceneConst& sc, const DeviceState& st, double dt, cudaStream_t s);
void launch_cfl_dt(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
void launch_density(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
void launch_error_correction(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
void launch_density_variation(const SceneConst& sc, const DeviceState& st, double* out,
                              cudaStream_t s);
void launch_explicit(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
void launch_save_x(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
void launch_set_ppe(const SceneConst& sc, const DeviceState& st, bool want_fp32, cudaStream_t s);
void launch_assign_pressure(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
void launch_pressure_gradient(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
void launch_dynamic_stabilize(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
// scan.cu
int scan_scratch_ints(int m);
void launch_exclusive_scan(const int* in, int* out, int m, int* scratch, cudaStream_t s);
// number of kernels each launcher issues (for the launch counter)
constexpr int kLaunchesSearch = 3, kLaunchesDensity = 1, kLaunchesEcs = 1, kLaunchesExplicit = 2,
              kLaunchesSaveX = 1, kLaunchesSetPpe = 6, kLaunchesAssign = 1, kLaunchesGradient = 2,
              kLaunchesDs = 2, kLaunchesDt = 1, kLaunchesCfl = 2;

}  // namespace mpsgb

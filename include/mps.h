/*
 * mps.h - C ABI of the GB300-native MPS (Moving Particle Semi-implicit) time step.
 *
 * This is the drop-in boundary for OpenMps's compute class
 * `Computer<POSITION_WALL, POSITION_WALL_PRE>` (src/OpenMps/Computer.hpp:434-1790).
 * Particle arrays go in, one time step is advanced on one GPU, and the same
 * fields (Type, x, z, u, w, p, n) come back in the caller's original order.
 *
 * Every entry point returns an int status (MPS_OK == 0).  Nothing throws across
 * this boundary; the message of the last failure is kept per handle
 * (mps_last_error).  One handle owns one CUDA stream and all device buffers of
 * one scene; handles share no global state, so separate host threads may drive
 * separate handles.  A handle is not re-entrant (like Computer::ForwardTime).
 *
 * Arrays passed with a `_host` meaning are plain host memory of `n` elements;
 * the library copies them (the caller keeps ownership), as AddParticles copies
 * the particles into Computer::particles (Computer.hpp:1754-1777).
 */
#ifndef OPENMPS_GB300_MPS_H
#define OPENMPS_GB300_MPS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define MPS_OK 0
#define MPS_ERR_INVALID_ARGUMENT 1
#define MPS_ERR_CUDA 2
#define MPS_ERR_OUT_OF_MEMORY 3
/* Grid::Exception "Too many particle in a block" (src/OpenMps/Grid.hpp:314-318) */
#define MPS_ERR_CELL_OVERFLOW 4
/* Computer::Exception "Conjugate Gradient method couldn't solve ..." (Computer.hpp:1424-1428) */
#define MPS_ERR_CG_NOT_CONVERGED 5
#define MPS_ERR_NOT_SUPPORTED 6
#define MPS_ERR_STATE 7
#define MPS_ERR_NONFINITE 8
/* a bounded device-side wait ran out of iterations (never a hang) */
#define MPS_ERR_TIMEOUT 9
/* a device-side bounds check fired (index recorded, access skipped) */
#define MPS_ERR_DEVICE_CHECK 10
/* the system is larger than the allocation-free solve's fixed scratch (MPS_NOALLOC_MAX_ROWS) */
#define MPS_ERR_NOALLOC_TOO_LARGE 11

/* ------------------------------------------------- particle types (Particle.hpp:16-29) */
#define MPS_TYPE_FLUID 0    /* Particle::Type::IncompressibleNewton */
#define MPS_TYPE_WALL 1     /* Particle::Type::Wall */
#define MPS_TYPE_DUMMY 2    /* Particle::Type::Dummy */
#define MPS_TYPE_DISABLED 3 /* Particle::Type::Disabled */

/* ------------------------------------- method flags: runtime form of defines.hpp:9-56 */
#define MPS_FLAG_HS 0x01u  /* MPS_HS   higher-order source term        (defines.hpp:31) */
#define MPS_FLAG_HL 0x02u  /* MPS_HL   higher-order Laplacian          (defines.hpp:36) */
#define MPS_FLAG_ECS 0x04u /* MPS_ECS  error-compensating source       (defines.hpp:41) */
#define MPS_FLAG_DS 0x08u  /* MPS_DS   dynamic stabilisation           (defines.hpp:51) */
#define MPS_FLAG_SPP 0x10u /* MPS_SPP  space-potential (surface) particle (defines.hpp:56) */
/* MPS_GC gradient corrective matrix (defines.hpp:46): the pressure gradient of a fluid
 * particle is multiplied by C_i = (sum_j W/r^2 dx dx^T)^-1 (Computer.hpp:1457-1499). */
#define MPS_FLAG_GC 0x20u
/* PRESSURE_EXPLICIT (defines.hpp:26): no PPE; p = c^2 (rho0/n0 n - rho0) where that is
 * positive, from the second number density (Computer.hpp:1046-1067), and MaxDt =
 * min(maxDt, courant l0 / c) (Environment.hpp:131-135).  Needs mps_params.sound_speed. */
#define MPS_FLAG_PRESSURE_EXPLICIT 0x40u
/* CENTRAL_GRAVITY (a switch of Computer.hpp that defines.hpp does not list): gravity
 * points to the origin, a += G_z x / |x|, and vanishes within l0 / 100 of it
 * (Computer.hpp:925-932, :981-988). */
#define MPS_FLAG_CENTRAL_GRAVITY 0x80u
/* PRESSURE_GRADIENT_MIDPOINT (defines.hpp:21) is always on: the other branch does
 * not compile in the reference (Computer.hpp:1522-1537).  ARTIFICIAL_COLLISION_FORCE
 * (defines.hpp:16) has no flag: its stage calls a Particle member that does not exist
 * (Computer.hpp:1104-1134), so no build of the reference can enable it. */
/* Every method flag. */
#define MPS_FLAGS_ALL (MPS_FLAG_HS | MPS_FLAG_HL | MPS_FLAG_ECS | MPS_FLAG_DS | MPS_FLAG_SPP | \
                       MPS_FLAG_GC | MPS_FLAG_PRESSURE_EXPLICIT | MPS_FLAG_CENTRAL_GRAVITY)
/* The stock build of the reference (defines.hpp as shipped). */
#define MPS_PRESET_REFERENCE (MPS_FLAG_HS | MPS_FLAG_HL | MPS_FLAG_ECS | MPS_FLAG_DS | MPS_FLAG_SPP)
/* Plain MPS: standard source/Laplacian, free-surface flag n/n0 < surface_ratio. */
#define MPS_PRESET_PLAIN 0u

/* ----------------------------------------------------------- PPE solver */
#define MPS_SOLVER_CG64 0   /* FP64 CG, the reference algorithm (Computer.hpp:1359-1429) */
#define MPS_SOLVER_MIXED 1  /* FP32 inner CG + FP64 true residual / iterative refinement; the
                               FP64 CG finishes the solve if the true residual stops halving */
#define MPS_SOLVER_LEARNED 2 /* MIXED_MG with the learned initial guess + diagonal scale */
/* MIXED preconditioned by a cell-aggregation multigrid (Jacobi on the particles plus a
 * V-cycle on the neighbour-search cells), FP64 CG fallback when it stalls.  Not in the
 * reference, whose CG is unpreconditioned. */
#define MPS_SOLVER_MIXED_MG 3

/* How the CG loop is launched: one CUDA graph with a device-driven while loop, or
 * host-launched kernel batches (the same kernels; for profilers that cannot see
 * kernels inside conditional graphs). */
#define MPS_CG_LAUNCH_GRAPH 0   /* one CUDA graph per solve, every phase its own kernel */
#define MPS_CG_LAUNCH_HOST 1
#define MPS_CG_LAUNCH_GRAPH_KERNELS 0  /* the same as MPS_CG_LAUNCH_GRAPH */
#define MPS_CG_LAUNCH_PERSISTENT 2     /* MIXED_MG / LEARNED: the iterations in one persistent
                                          cooperative kernel (grid barriers between phases);
                                          per-phase kernels if the device cannot launch it */

/* CG stopping rule */
#define MPS_CRIT_INITIAL_RESIDUAL 0 /* reference: r_k.r_k < eps^2 r_0.r_0 (Computer.hpp:1386, :1408) */
#define MPS_CRIT_RHS 1              /* |b - A x| <= eps |b| */

/*
 * Parameters of Environment (src/OpenMps/Environment.hpp:101-128) and
 * ComputingCondition::Eps (src/OpenMps/ComputingCondition.hpp:13-16), plus the
 * runtime method flags and solver controls.
 */
typedef struct mps_params {
    double max_dt;        /* Environment(maxDt, ...) */
    double courant;       /* courant */
    double g;             /* gravity magnitude, G = (0, -g) (Environment.hpp:149) */
    double rho;           /* density */
    double nu;            /* kinematic viscosity */
    double surface_ratio; /* free-surface threshold beta; used only without MPS_FLAG_SPP */
    double re_by_l0;      /* r_eByl_0: radius of density, source and gradient */
    double re_lap_by_l0;  /* Laplacian radius / l0 (viscosity, PPE matrix); <= 0 means re_by_l0.
                             A second radius is an extension: the reference has one R_e. */
    double l0;            /* l_0 */
    double min_x, min_z, max_x, max_z; /* computational domain */
    double eps;           /* CG allowable residual (ComputingCondition::Eps) */
    uint32_t flags;       /* MPS_FLAG_* */
    int32_t solver;       /* MPS_SOLVER_* */
    int32_t criterion;    /* MPS_CRIT_* */
    int32_t max_cg_iters; /* <= 0: number of unknowns, as the reference (Computer.hpp:1392) */
    double inner_tol;     /* MIXED: relative residual reduction of one FP32 inner solve */
    int32_t max_refinements; /* MIXED: maximum FP64 refinement passes */
    int32_t cg_launch;       /* MPS_CG_LAUNCH_GRAPH (default), _HOST or _PERSISTENT */
    double sound_speed;      /* Environment(..., c, ...): used only with MPS_FLAG_PRESSURE_EXPLICIT */
    int32_t dim;             /* 2 (default; 0 means 2) or 3 (DIM3, defines.hpp:9-11): three-
                                dimensional scenes take the *3 particle calls below and the
                                MPS_SOLVER_CG64 or MPS_SOLVER_MIXED solver; no batches */
    int32_t pad0;
    double min_y, max_y;     /* domain along y (DIM3: Environment(..., minY, ..., maxY, ...)) */
    double reserved[2];
} mps_params;

/* Derived constants of Environment (Environment.hpp:129-216) and Grid (Grid.hpp:137-150). */
typedef struct mps_environment {
    double t, dt;
    double n0, lambda;         /* at r_e (Environment::N0, ::Lambda) */
    double n0_lap, lambda_lap; /* at the Laplacian radius (equal to the above with one radius) */
    double max_dt, max_dx, l0, re, re_lap, neighbor_length;
    double rho, nu, g;
    double min_x, min_z, max_x, max_z;
    int64_t grid_nx, grid_nz, grid_max_per_cell;
    double min_y, max_y;  /* DIM3 */
    int64_t grid_ny;      /* 1 in 2D */
    int64_t dim;
} mps_environment;

/* Per-step solver statistics and counters. */
typedef struct mps_stats {
    int64_t steps;            /* ForwardTime calls completed */
    int64_t kernel_launches;  /* cumulative kernels launched by this handle */
    int64_t neighbor_total;   /* neighbour-list entries of the last search */
    int64_t ppe_nnz;          /* nonzeros of the last PPE matrix */
    int32_t cg_iterations;    /* inner iterations of the last solve (all passes) */
    int32_t cg_refinements;   /* FP64 outer passes of the last solve (1 for CG64) */
    int32_t disabled;         /* particles of type Disabled after the last search */
    int32_t fallback;         /* 1 if the last mixed-precision solve (MIXED, MIXED_MG, LEARNED)
                                 stalled and the plain FP64 CG finished it */
    double cg_rr0;            /* r_0.r_0 of the last solve */
    double cg_rr;             /* final (recursive) r.r of the last solve */
    double cg_true_relres;    /* |b - A x| / |b| recomputed in FP64 after the last solve */
    double stage_ms[12];      /* last step, if stage timing is enabled: search, density,
                                 ecs, explicit, density2, ppe, solve, pressure, gradient,
                                 ds, other, total */
} mps_stats;

typedef struct mps_handle mps_handle;

/* ------------------------------------------------------------ lifecycle */
/* Fills the defaults: the stock reference preset and Sample.xml constants. */
void mps_default_params(mps_params* prm);
size_t mps_params_size(void);
size_t mps_stats_size(void);
size_t mps_environment_size(void);
const char* mps_status_string(int status);
/* Message of the last failure on `h` ("" if none).  Valid until the next call on h. */
const char* mps_last_error(const mps_handle* h);
/* Version string of the library build. */
const char* mps_version(void);

/* CreateComputer(allowableResidual, env, posWall, posWallPre) (Computer.hpp:1800-1815)
 * and the Environment constructor (Environment.hpp:101-216). Selects CUDA device
 * `device` (the caller's current device if < 0). */
int mps_create(const mps_params* prm, int device, mps_handle** out);
int mps_destroy(mps_handle* h);

/* AddParticles(std::vector<Particle>&&) (Computer.hpp:1754-1777): appends particles.
 * The wall target of each added particle is its position here, as the reference
 * driver's static-wall callback returns the initial position (Main.cpp:303-318). */
int mps_add_particles(mps_handle* h, int64_t n, const int32_t* type, const double* x,
                      const double* z, const double* u, const double* w, const double* p,
                      const double* nd);
int64_t mps_particle_count(const mps_handle* h);

/* Particles() (Computer.hpp:1780-1783): copies the state to host arrays (any may be NULL). */
int mps_get_particles(mps_handle* h, int32_t* type, double* x, double* z, double* u, double* w,
                      double* p, double* nd);
/* Overwrites the state of all particles from host arrays (count unchanged). */
int mps_set_particles(mps_handle* h, const int32_t* type, const double* x, const double* z,
                      const double* u, const double* w, const double* p, const double* nd);
/* Same, with device pointers (stream-ordered on the handle's stream). */
int mps_get_particles_device(mps_handle* h, int32_t* type, double* x, double* z, double* u,
                             double* w, double* p, double* nd);
int mps_set_particles_device(mps_handle* h, const int32_t* type, const double* x,
                             const double* z, const double* u, const double* w,
                             const double* p, const double* nd);

/* positionWall(i, t, dt) targets (Computer.hpp:1015): the position every non-fluid
 * particle takes in the explicit step.  Host arrays of n elements. */
int mps_set_wall_positions(mps_handle* h, const double* wx, const double* wz);

/* Three-dimensional scenes (mps_params.dim = 3): the same calls with the y axis, in the
 * reference's DIM3 argument order (position x, y, z; velocity u, v, w).  The
 * two-dimensional particle calls return MPS_ERR_STATE on such a handle, and these on a
 * two-dimensional one. */
int mps_add_particles3(mps_handle* h, int64_t n, const int32_t* type, const double* x,
                       const double* y, const double* z, const double* u, const double* v,
                       const double* w, const double* p, const double* nd);
int mps_get_particles3(mps_handle* h, int32_t* type, double* x, double* y, double* z, double* u,
                       double* v, double* w, double* p, double* nd);
int mps_set_particles3(mps_handle* h, const int32_t* type, const double* x, const double* y,
                       const double* z, const double* u, const double* v, const double* w,
                       const double* p, const double* nd);
int mps_set_wall_positions3(mps_handle* h, const double* wx, const double* wy, const double* wz);

/* ForwardTime(double dt) (Computer.hpp:1700-1742); dt <= 0 selects ForwardTime()
 * (Computer.hpp:1745-1751) with the CFL time step of DetermineDt (:759-777). */
int mps_forward_time(mps_handle* h, double dt);
/* DetermineDt (Computer.hpp:759-777): the CFL time step mps_forward_time(h, 0) would take
 * from the current state, without advancing.  A caller that evaluates moving-wall
 * positions on the host for the step (positionWall(i, t, dt), Computer.hpp:1015) needs
 * dt first; mps_forward_time(h, *dt) then takes exactly that step. */
int mps_determine_dt(mps_handle* h, double* dt);
/* nsteps calls of mps_forward_time(h, dt). */
int mps_forward_steps(mps_handle* h, double dt, int32_t nsteps);

/* GetEnvironment() (Computer.hpp:1786-1789). */
int mps_get_environment(const mps_handle* h, mps_environment* env);
int mps_get_stats(const mps_handle* h, mps_stats* st);
/* Solver controls may change between steps. */
int mps_set_solver(mps_handle* h, int32_t solver, int32_t criterion, double eps);
/* Enables per-stage CUDA-event timing (stats.stage_ms). */
int mps_set_stage_timing(mps_handle* h, int32_t enable);
/* Bounds of the handle's device-side waits, in SM clock cycles (negative: the default).
 * No counterpart in the reference, which has no device waits.  barrier_clocks bounds
 * each grid-barrier wait of the persistent preconditioned solve (MPS_CG_LAUNCH_PERSISTENT;
 * default 4e9, about two seconds); mma_clocks bounds each tensor-core completion wait of
 * the learned solve's network inference (default 2e9).  A wait that runs out sets an
 * error word and lets its kernel return: the step still completes (the network's
 * output is not used, or the FP64 CG finishes the solve), and mps_forward_time returns
 * MPS_ERR_TIMEOUT.  The handle stays usable.  0 makes every such wait give up at its
 * first check, which tests use to exercise this path. */
int mps_set_wait_limits(mps_handle* h, int64_t barrier_clocks, int64_t mma_clocks);

/* ------------------------------------------------- timing on the handle's stream */
int mps_synchronize(mps_handle* h);
/* Records CUDA event `slot` (0..15) on the handle's stream. */
int mps_event_record(mps_handle* h, int32_t slot);
/* Milliseconds between two recorded events (synchronizes on `end`). */
int mps_event_elapsed(mps_handle* h, int32_t begin, int32_t end, float* ms);
/* Writes `bytes` of scratch on the handle's stream, then reads it back: evicts L2 between
 * timed runs and leaves it holding clean lines, so the timed work writes nothing back. */
int mps_flush_l2(mps_handle* h, int64_t bytes);
/* Times the PPE solver's SpMV kernel alone on the last assembled matrix: `reps`
 * back-to-back launches (FP64 values for MPS_SOLVER_CG64, FP32 for MPS_SOLVER_MIXED);
 * *ms_per_launch receives the mean CUDA-event time of one launch.  When flush_bytes
 * > 0, L2 is flushed before every launch and only the launch is timed. */
int mps_bench_spmv(mps_handle* h, int32_t solver, int32_t reps, int64_t flush_bytes,
                   float* ms_per_launch);
/* Algorithmic bytes of one launch of that SpMV on the last assembled matrix (nnz entries,
 * n rows): every matrix entry and row length read once, each vector read or written once
 * per row.  FP64 CG: 12 nnz + 4 (n + 1) + 16 n; MIXED: 8 nnz + 4 (n + 1) + 8 n; MIXED_MG:
 * 8 nnz + 4 (n + 1) + 12 n (an FP32 entry is {column, value}). */
int mps_spmv_bytes(mps_handle* h, int32_t solver, int64_t* bytes);

/* ------------------------------------------------------------------------
 * Stage hooks.  They mirror the reference's friend-class test access to the
 * private stages of Computer (Computer.hpp:437-460) and run exactly one stage.
 * ---------------------------------------------------------------------- */
int mps_stage_search_neighbor(mps_handle* h);        /* SearchNeighbor          :698-756 */
int mps_stage_density(mps_handle* h);                /* ComputeNeighborDensities :780-833 */
int mps_stage_error_correction(mps_handle* h);       /* ComputeErrorCorrection  :877-910 */
int mps_stage_explicit(mps_handle* h);               /* ComputeExplicitForces   :914-1021 */
int mps_stage_save_x(mps_handle* h);                 /* SaveX                   :1025-1039 */
int mps_stage_set_ppe(mps_handle* h);                /* SetPressurePoissonEquation :1145-1356 */
int mps_stage_solve_ppe(mps_handle* h);              /* SolvePressurePoissonEquation :1359-1429 */
int mps_stage_assign_pressure(mps_handle* h);        /* ComputeImplicitForces   :1076-1097 */
int mps_stage_pressure_gradient(mps_handle* h);      /* ModifyByPressureGradient :1433-1564 */
int mps_stage_dynamic_stabilize(mps_handle* h);      /* DynamicStabilize        :1568-1656 */
/* Sets t and dt as ForwardTime does before its stages (Computer.hpp:1703-1706). */
int mps_stage_begin_step(mps_handle* h, double dt);
/* NeighborDensityVariationSpeed(i) for every particle (Computer.hpp:838-872). */
int mps_stage_density_variation(mps_handle* h, double* speed_host);

/* Neighbour lists of the last search in reference order (Computer.hpp:720-755):
 * counts[n]; list receives the concatenated rows (capacity entries).  *total gets
 * the number of entries. */
int mps_debug_get_neighbors(mps_handle* h, int32_t* counts, int32_t* list, int64_t capacity,
                            int64_t* total);
/* PPE system of the last assembly: CSR with ascending columns (uBLAS compressed_matrix
 * semantics, Computer.hpp:1330-1354), b and x.  Any pointer may be NULL. */
int mps_debug_get_ppe(mps_handle* h, int64_t* row_ptr, int32_t* col, double* val, double* b,
                      double* x, int64_t capacity, int64_t* nnz);
/* Auxiliary per-particle state: nWithoutSpp (:553-556), ecs (:543-546),
 * originalX (:548-551).  Any pointer may be NULL. */
int mps_debug_get_aux(mps_handle* h, double* n_without_spp, double* ecs, double* ox, double* oz);
int mps_debug_set_aux(mps_handle* h, const double* n_without_spp, const double* ecs,
                      const double* ox, const double* oz);
/* The same with originalX's y component (DIM3 handles). */
int mps_debug_get_aux3(mps_handle* h, double* n_without_spp, double* ecs, double* ox, double* oy,
                       double* oz);
int mps_debug_set_aux3(mps_handle* h, const double* n_without_spp, const double* ecs,
                       const double* ox, const double* oy, const double* oz);

/* The stage kernels' FP64 division and square root (computed on the FP32 and integer
 * pipes, rounded like IEEE division and square root) on host arrays of n values, run on
 * `device`: quot[i] = a[i] / b[i], root[i] = sqrt(a[i]).  No counterpart in the
 * reference; tests compare them with the host's IEEE arithmetic. */
int mps_debug_exact_arith(int32_t device, int64_t n, const double* a, const double* b, double* quot,
                          double* root);

/* SolvePressurePoissonEquation on a caller-supplied CSR system (host arrays), the
 * entry the reference's CG tests drive (test_ComputerConjugateGradient.cpp).
 * x holds the initial guess on entry and the solution on return. */
int mps_cg_solve_csr(mps_handle* h, int64_t n, const int64_t* row_ptr, const int32_t* col,
                     const double* val, const double* b, double* x, double eps,
                     int32_t criterion, int32_t max_iters, int32_t solver, int32_t* iterations,
                     double* true_relres);

/* ------------------------------------------------------------------------
 * Allocation-free PPE solve.  No counterpart in the reference: the reference owns all
 * its memory.  For callers that cannot allocate device memory -- an application whose
 * device memory is already reserved by its own caching allocator or arena, or code on
 * a latency-critical path where cudaMalloc/cudaFree would synchronize the device --
 * this solves A x = b with the FP64 CG of the reference (Computer.hpp:1359-1429) on a
 * CSR system that already lives in the caller's device memory, and allocates nothing:
 * its scratch vectors sit in one static device array sized for MPS_NOALLOC_MAX_ROWS
 * rows (about 6 MiB, held by every GPU that loads the library until the process
 * exits).  Larger systems return MPS_ERR_NOALLOC_TOO_LARGE.
 *
 * All pointers are device pointers on the current device; `stream` is a
 * cudaStream_t (NULL: the default stream); x holds the initial guess on entry and the
 * solution on return.  Every call looks up the scratch array's address in the current
 * context (cudaGetSymbolAddress, which allocates nothing), so a device reset or another
 * context on the same device never leaves it a stale address; the first call in a
 * context may load the library's module and should come before any stream capture.
 * Every call shares the one array: calls that overlap on the GPU (other streams or
 * host threads at the same time) race.  The call returns when the solve is complete.
 * NULL pointers return MPS_ERR_INVALID_ARGUMENT.
 * ---------------------------------------------------------------------- */
#define MPS_NOALLOC_MAX_ROWS 262144
int mps_cg_solve_csr_device_noalloc(int64_t n, const int64_t* row_ptr, const int32_t* col,
                                    const double* val, const double* b, double* x, double eps,
                                    int32_t criterion, int32_t max_iters, void* stream,
                                    int32_t* iterations, double* true_relres);

/* ------------------------------------------------------------ learned solve
 * No counterpart in the reference (its CG is unpreconditioned and starts from the
 * previous pressure).  MPS_SOLVER_LEARNED is MPS_SOLVER_MIXED_MG started from a
 * network-predicted initial guess and with a network-predicted scale of each particle's
 * Jacobi term; the FP64 CG fallback and the FP64 true residual judge its result.
 *
 * Weight blob (FP32, MPS_MLP_BLOB_FLOATS): feature mean[16], feature std[16],
 * W1[64][16], b1[64], W2[64][64], b2[64], W3[64][64], b3[64], W4[2][64], b4[2]
 * (W[out][in], GELU after the three hidden layers).
 * Outputs: out0 = correction of the initial guess (units of the RMS Jacobi-scaled
 * residual), s = 1 + 0.25 tanh(out1) = scale of the particle's Jacobi term.
 * Sample (FP32, MPS_MLP_SAMPLE_FLOATS): features[16], target y, Jacobi term g. */
#define MPS_MLP_BLOB_FLOATS 9570
#define MPS_MLP_SAMPLE_FLOATS 18

/* Loads the network used by MPS_SOLVER_LEARNED (converted to the tensor-core image). */
int mps_learned_set_weights(mps_handle* h, const float* blob, int64_t count);
/* When enabled, every solve also records one training sample per particle: the
 * features of the step and the targets from the solution (any solver).  Two-dimensional
 * scenes only (MPS_ERR_NOT_SUPPORTED on a DIM3 handle). */
int mps_learned_collect(mps_handle* h, int32_t enable);
/* The last step's samples (n x MPS_MLP_SAMPLE_FLOATS) and active-row flags (n);
 * with both pointers null only *count (= n) is returned. */
int mps_learned_samples(mps_handle* h, float* samples, int32_t* active, int64_t capacity,
                        int64_t* count);
/* Network inference on the tensor cores (BF16 operands, FP32 accumulation) for n
 * feature rows (n x 16, residual features already in units of sigma): out n x 2. */
int mps_mlp_infer(int32_t device, const float* blob, const float* features, int64_t n, float* out);
/* Mean loss over n samples and its gradient (FP32 training kernels); grad has
 * MPS_MLP_BLOB_FLOATS entries, the first 32 (feature mean/std) are zero. */
int mps_mlp_loss_grad(int32_t device, const float* blob, const float* samples, int64_t n,
                      float* grad, double* loss);
/* Adam training on the GPU: `epochs` passes over the samples in seeded shuffled order,
 * minibatches of `batch`; blob holds the initial weights in and the trained ones out;
 * epoch_loss (optional, `epochs` entries) the mean loss of each pass. */
int mps_mlp_train(int32_t device, float* blob, const float* samples, int64_t n, int32_t epochs,
                  int32_t batch, float lr, uint64_t seed, double* epoch_loss);

/* ------------------------------------------------------------ batched scenes
 * No counterpart in the reference (one Computer per scene there).  A batch handle holds
 * `nscenes` independent scenes that share one mps_params (tank, l0, physics); each
 * scene behaves as a separate Computer (no interaction), all advance together with a
 * fixed dt: the stages run over all scenes at once and the PPEs are solved by one
 * persistent kernel, a thread block per scene (mixed-precision multigrid-preconditioned
 * CG, FP64 CG fallback).  The first mps_batch_forward step runs an autotuner (threads
 * per block and scene order of the solve, timed on the assembled step); later steps
 * replay one captured CUDA graph per step.  Limits: dt > 0; the scene's cell hierarchy
 * must fit one block's shared memory (MPS_ERR_NOT_SUPPORTED otherwise). */
typedef struct mps_batch_scene_stats {
    int32_t iterations;          /* PPE iterations of the last step (incl. fallback) */
    int32_t reliable_updates;
    int32_t fallback;            /* 1 if the FP64 CG finished the solve */
    int32_t converged;
    int32_t fallback_iterations;
    int32_t pad;
    double true_relres;          /* |b - A x| / |b| in FP64 after the solve */
    double initial_relres;       /* |b - A x0| / |b| */
} mps_batch_scene_stats;

typedef struct mps_batch_tuning {
    int32_t threads, blocks, order;  /* chosen launch; order 0 = scene index, 1 = largest first */
    int32_t candidates;
    float candidate_ms[16];
    int32_t candidate_threads[16];
    int32_t candidate_order[16];
} mps_batch_tuning;

int mps_batch_create(const mps_params* prm, int device, int32_t nscenes, const int64_t* counts,
                     mps_handle** out);
/* Particles of one scene (counts[scene] of each array, the scene's own order). */
int mps_batch_set_scene(mps_handle* h, int32_t scene, const int32_t* type, const double* x,
                        const double* z, const double* u, const double* w, const double* p,
                        const double* nd);
int mps_batch_get_scene(mps_handle* h, int32_t scene, int32_t* type, double* x, double* z,
                        double* u, double* w, double* p, double* nd);
int mps_batch_forward(mps_handle* h, double dt, int32_t nsteps);
int mps_batch_get_scene_stats(mps_handle* h, int32_t scene, mps_batch_scene_stats* st);
int mps_batch_tuning_info(const mps_handle* h, mps_batch_tuning* t);

#ifdef __cplusplus
}
#endif

#endif /* OPENMPS_GB300_MPS_H */

// cg.cuh - pressure Poisson solvers on the SELL-32 matrix.
#pragma once

#include "common.cuh"

namespace mpsgb {

// A {column, FP32 value} pair of the SELL stream, loaded without allocating in L1: each
// pair is read once per SpMV, so L1 stays with the gathered entries of the vector, which
// neighbouring rows share.  The L2 policy stays the default (the FP32 matrix is read
// every iteration and may stay resident).  The matrix is read-only while a solve runs.
__device__ __forceinline__ uint2 ld_sell_pair(const uint2* p) {
    uint2 e;
    asm("ld.global.nc.L1::no_allocate.v2.u32 {%0, %1}, [%2];" : "=r"(e.x), "=r"(e.y) : "l"(p));
    return e;
}

// Scalars of one solve, in device memory (read back once per step).
struct CgScalars {
    double rr;        // r.r of the current direction update
    double rr_new;    // r.r after the last update
    double pAp;
    double alpha;
    double beta;
    double thr;       // convergence threshold on r.r
    double rr0;       // r_0.r_0
    double bb;        // b.b
    double eps;
    double rr_upd;    // MIXED: true r.r at the last reliable update
    double delta2;    // MIXED: reliable-update trigger (rr_new < delta2 * rr_upd)
    double true_rr;   // last true residual r.r (FP64)
    int32_t iter;
    int32_t max_iter;
    int32_t converged;
    int32_t do_update;  // MIXED: a reliable update is due / was just made
    int32_t criterion;
    int32_t updates;    // MIXED: reliable updates made (parity selects the x buffer)
    uint32_t counter;   // last-block ticket
    int32_t aborted;    // the step failed before the solve: nothing runs
    // preconditioned solve (MIXED_MG, LEARNED)
    int32_t stalled;      // breakdown or a reliable update that did not halve |r|
    int32_t fallback;     // the plain FP64 CG ran after the preconditioned solve
    int32_t fb_iter;      // iterations of that fallback
    int32_t iter_upd;     // MIXED: iteration of the last reliable update
    double prev_true_rr;  // true r.r at the previous reliable update
};

struct CgOperands {
    int32_t n;          // rows
    int32_t nchunks;    // chunks of kSellRows rows
    int32_t grid_vec;   // blocks of the vector kernels (one thread per row)
    int32_t grid_spmv;  // blocks of the SpMV kernels (one warp per chunk)
    int32_t grid_staged;  // blocks of the staged SpMV kernels (one per SM; 0: not used)
    const int32_t* len; // row lengths, kSellRows * nchunks (rows >= n have length 0)
    const int32_t* off; // chunk offsets, nchunks + 1
    const int32_t* chunk;  // entries of each chunk (32 x its widest row): chunks may sit
                           // farther apart than their width (rows assembled in place)
    const int32_t* col; // SELL-32 columns
    const double* val;  // SELL-32 FP64 values
    const uint2* cv32;  // SELL-32 {column, FP32 value}
    const double* b;
    double* x;          // initial guess in, solution out
    // CG64
    double *r, *p, *Ap;
    // MIXED (Chronopoulos-Gear CG in FP32): r, w = A r, s = A p, p, correction d
    double* x2;         // second FP64 solution buffer (reliable updates alternate)
    float *r32, *w32, *s32, *p32, *d32;
    float* u32;         // preconditioned residual u = M r (MIXED_MG, LEARNED)
    double* partials;   // reduction partials (cg_partials doubles)
    uint32_t* tickets;  // per-group reduction counters (cg_tickets, zero between kernels)
    CgScalars* S;
    const DevStatus* status;  // step status (may be null): a failed search aborts the solve
};

// Row i (lane of a chunk at `at`) times v in FP64, ascending columns.  The FP64 matrix
// streams with evict-first hints: on big scenes it exceeds L2 and the solver's vectors
// should stay resident instead.  Software-pipelined: the next D entries are loaded
// before this batch's gathers, so a lane keeps both kinds of loads in flight.  The
// row's last step is predicated (slots past L load nothing and add nothing): a row costs
// ceil(L / D) dependent round trips, and the sum is the same sequence of fma as one
// entry at a time.
template <int D = 8, class V>
__device__ __forceinline__ double row64(const CgOperands& o, int64_t at, int L, V v) {
    double acc = 0.0;
    int c[D];
    double a[D];
#pragma unroll
    for (int u = 0; u < D; u++) {
        c[u] = u < L ? __ldcs(o.col + at + u * kSellRows) : 0;
        a[u] = u < L ? __ldcs(o.val + at + u * kSellRows) : 0.0;
    }
    for (int k0 = 0; k0 < L; k0 += D) {
        double xv[D];
#pragma unroll
        for (int u = 0; u < D; u++) xv[u] = k0 + u < L ? v(c[u]) : 0.0;
        int cn[D];
        double an[D];
        const int64_t nx = at + static_cast<int64_t>(k0 + D) * kSellRows;
#pragma unroll
        for (int u = 0; u < D; u++) {
            const bool in = k0 + D + u < L;
            cn[u] = in ? __ldcs(o.col + nx + u * kSellRows) : 0;
            an[u] = in ? __ldcs(o.val + nx + u * kSellRows) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < D; u++)
            if (k0 + u < L) acc = fma(a[u], xv[u], acc);
#pragma unroll
        for (int u = 0; u < D; u++) {
            c[u] = cn[u];
            a[u] = an[u];
        }
    }
    return acc;
}

// Lane's row of the FP32 matrix times v, FP32 accumulation, ascending columns.
// Software-pipelined: row32_first loads the first D entries (they may be loaded before
// the vector v is ready), row32_rest gathers and sums the row D entries per step while
// the next step's entries load.  The row's last step is predicated (slots past L load
// nothing and add nothing), so a row costs ceil(L / D) dependent round trips and the
// sum is the same sequence of fmaf as one entry at a time.
template <int D>
__device__ __forceinline__ void row32_first(const CgOperands& o, int64_t at, int L, uint2 (&e)[D]) {
#pragma unroll
    for (int u = 0; u < D; u++)
        e[u] = u < L ? ld_sell_pair(o.cv32 + at + u * kSellRows) : make_uint2(0u, 0u);
}

template <int D>
__device__ __forceinline__ float row32_rest(const CgOperands& o, int64_t at, int L, const float* __restrict__ v,
                                            uint2 (&e)[D]) {
    float acc = 0.0f;
    for (int k0 = 0; k0 < L; k0 += D) {
        float xv[D];
#pragma unroll
        for (int u = 0; u < D; u++) xv[u] = k0 + u < L ? v[e[u].x] : 0.0f;
        uint2 f[D];
        const int64_t nx = at + static_cast<int64_t>(k0 + D) * kSellRows;
#pragma unroll
        for (int u = 0; u < D; u++)
            f[u] = k0 + D + u < L ? ld_sell_pair(o.cv32 + nx + u * kSellRows) : make_uint2(0u, 0u);
#pragma unroll
        for (int u = 0; u < D; u++)
            if (k0 + u < L) acc = fmaf(__uint_as_float(e[u].y), xv[u], acc);
#pragma unroll
        for (int u = 0; u < D; u++) e[u] = f[u];
    }
    return acc;
}

// The same row product for the plain mixed solve: whole steps of D entries pipelined,
// the last L mod D entries one at a time (the same sum).  On the 3D dam break's PPE
// (104k rows, 70 % of them single-entry dummy rows) this form took 8.33 ms per step
// against 8.9 ms with the predicated last step, which the 340k 2D PPE prefers (234
// against 243 ms for the same mixed solve).
template <int D = 8>
__device__ __forceinline__ float row32(const CgOperands& o, int64_t at, int L, const float* __restrict__ v) {
    float acc = 0.0f;
    const int nb = L / D;
    uint2 e[D];
    if (nb > 0) {
#pragma unroll
        for (int u = 0; u < D; u++) e[u] = ld_sell_pair(o.cv32 + at + u * kSellRows);
    }
    for (int bt = 0; bt < nb; bt++) {
        float xv[D];
#pragma unroll
        for (int u = 0; u < D; u++) xv[u] = v[e[u].x];
        uint2 f[D];
        if (bt + 1 < nb) {
            const int64_t nx = at + static_cast<int64_t>(bt + 1) * D * kSellRows;
#pragma unroll
            for (int u = 0; u < D; u++) f[u] = ld_sell_pair(o.cv32 + nx + u * kSellRows);
        }
#pragma unroll
        for (int u = 0; u < D; u++) acc = fmaf(__uint_as_float(e[u].y), xv[u], acc);
#pragma unroll
        for (int u = 0; u < D; u++) e[u] = f[u];
    }
    at += static_cast<int64_t>(nb) * D * kSellRows;
    for (int k = nb * D; k < L; k++, at += kSellRows) {
        const uint2 t = ld_sell_pair(o.cv32 + at);
        acc = fmaf(__uint_as_float(t.y), v[t.x], acc);
    }
    return acc;
}

struct MgHierarchy;
struct LearnedOps;

// Bounds of the device-side waits, in SM clock cycles, kept in device memory per handle
// so that captured graphs read the current values.  A wait gives up once this many
// cycles have passed since it began (0: at its first check), sets an error word and
// lets its kernel return; the host turns the word into MPS_ERR_TIMEOUT.
struct WaitLimits {
    long long barrier_clocks;  // grid barrier of the persistent preconditioned solve
    long long mma_clocks;      // tensor-core completion wait of the network inference
};
constexpr long long kDefaultBarrierClocks = 4000000000LL;  // about two seconds
constexpr long long kDefaultMmaClocks = 2000000000LL;      // about one second
// After a tensor-core wait gave up, the MMAs it waited for may still write TMEM: the
// kernel waits this long again for their completion before it frees TMEM.
constexpr long long kMmaDrainClocks = 2000000000LL;

// Device words of the persistent solve's grid barrier, and its grid size.
constexpr int kPersistentCounters = 513;  // barrier group counters + the top one

struct PersistentSync {
    unsigned* count;  // kPersistentCounters counters, zero between launches
    unsigned* gen;
    int32_t* err;     // set when a barrier wait runs out
    int blocks;
    const WaitLimits* limits;  // null: the defaults
};

// The learned start of a solve: its device state and the scalars its kernels gate on.
struct LearnedRun {
    const LearnedOps* L;
    CgScalars* S;
};

// A CUDA graph running one whole solve: init kernels + device-driven while loop (+ for
// the preconditioned solvers the FP64 CG fallback loop, which runs only after a failure).
// Side stream and events of a fork/join inside a captured graph.
struct SetupFork {
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};

class CgGraph {
public:
    ~CgGraph();
    // `mg` and `fb` (operands of the FP64 fallback, own scalars) are required for
    // MPS_SOLVER_MIXED_MG and MPS_SOLVER_LEARNED and ignored otherwise.
    cudaError_t build(int solver, const CgOperands& ops, cudaStream_t s,
                      const MgHierarchy* mg = nullptr, const CgOperands* fb = nullptr,
                      const LearnedRun* lrn = nullptr);
    // MIXED_MG / LEARNED with the whole iteration loop in one cooperative kernel
    cudaError_t build_persistent(int solver, const CgOperands& ops, cudaStream_t s, const MgHierarchy* mg,
                                 const CgOperands* fb, const LearnedRun* lrn, const PersistentSync& ps);
    cudaError_t launch(cudaStream_t s);
    void reset();
    bool persistent() const { return persistent_; }
    bool valid() const { return exec_ != nullptr; }
    int solver() const { return solver_; }
    const CgOperands& operands() const { return ops_; }
    // kernels per iteration, and per reliable update when it runs under its IF node
    int kernels_per_iteration() const { return nested_ ? kpi_ : kpi_ + kri_; }
    int kernels_per_update() const { return nested_ ? kri_ : 0; }
    bool nested() const { return nested_; }

private:
    cudaError_t build_impl(int solver, const CgOperands& ops, cudaStream_t s, bool nested,
                           const MgHierarchy* mg, const CgOperands* fb, const LearnedRun* lrn);
    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t exec_ = nullptr;
    int solver_ = -1;
    bool nested_ = false;
    bool persistent_ = false;
    int kpi_ = 0, kri_ = 0;
    CgOperands ops_{};
    SetupFork fork_;  // created at the first build, kept across rebuilds
};

// The same solve with host-launched kernels: `chunk` iterations per launch batch, the
// device status read back between batches (kernels past convergence return at once).
// Used when kernels must be visible one by one (profilers) and as a fallback.
cudaError_t cg_run_direct(int solver, const CgOperands& ops, CgScalars* host_S, int chunk,
                          cudaStream_t s, int64_t* launches, const MgHierarchy* mg = nullptr,
                          const CgOperands* fb = nullptr, const LearnedRun* lrn = nullptr);
// Grid size of the persistent solve on the current device (0: cooperative launch unavailable).
int persistent_blocks();
// Kernels of one iteration of the solver, and of one reliable update.
int cg_kernels_per_iteration(int solver, const MgHierarchy* mg);
int cg_kernels_per_update(int solver, const MgHierarchy* mg, const CgOperands& ops);

// Sets eps / criterion / max_iter / delta for the next solve (stream-ordered).
void launch_cg_configure(CgScalars* S, double eps, int criterion, int max_iter, double delta2,
                         cudaStream_t s);
// One launch of the solver's SpMV kernel (the CG iteration's dominant kernel) alone.
void launch_spmv_only(int solver, const CgOperands& ops, cudaStream_t s);
// Shared-memory opt-in of the staged SpMV kernels (once per device, before they launch).
cudaError_t cg_prepare_device();
// Launch shapes of the solver kernels for n rows, and the partials they need.
int cg_grid_vec(int64_t n);
int cg_grid_spmv(int64_t n);
int64_t cg_partials(int64_t n);
int64_t cg_tickets(int64_t n);

}  // namespace mpsgb

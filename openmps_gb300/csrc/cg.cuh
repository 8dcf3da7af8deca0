// cg.cuh - pressure Poisson solvers on the transposed ELL matrix.
#pragma once

#include "common.cuh"

namespace mpsgb {

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
    double true_rr;   // MIXED: last true residual r.r
    int32_t iter;
    int32_t max_iter;
    int32_t converged;
    int32_t do_update;
    int32_t criterion;
    int32_t updates;
    uint32_t counter;  // last-block ticket
    int32_t aborted;   // the step failed before the solve: nothing runs
};

struct CgOperands {
    int32_t n;
    const int32_t* len;
    const int32_t* col;
    const double* val;
    const float* val32;
    const double* b;
    double* x;
    // FP64 CG
    double *r, *p, *Ap;
    // MIXED
    float *r32, *p32, *q32, *d32;
    double* partials;  // 2 * grid doubles
    CgScalars* S;
    const DevStatus* status;  // step status (may be null): a failed search aborts the solve
};

// A CUDA graph running one whole solve: init kernel + device-driven while loop.
class CgGraph {
public:
    ~CgGraph();
    cudaError_t build(int solver, const CgOperands& ops, cudaStream_t s);
    cudaError_t launch(cudaStream_t s);
    void reset();
    bool valid() const { return exec_ != nullptr; }
    int solver() const { return solver_; }
    const CgOperands& operands() const { return ops_; }
    int kernels_per_iteration() const { return solver_ == MPS_SOLVER_CG64 ? 3 : 4; }

private:
    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t exec_ = nullptr;
    int solver_ = -1;
    CgOperands ops_{};
};

// Sets eps / criterion / max_iter / delta for the next solve (stream-ordered).
void launch_cg_configure(CgScalars* S, double eps, int criterion, int max_iter, double delta2,
                         cudaStream_t s);
// r.r of b - A x in FP64 (true residual) into *out (device), stream-ordered.
void launch_true_residual(const CgOperands& ops, double* out2, cudaStream_t s);

}  // namespace mpsgb

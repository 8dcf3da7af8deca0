// cg.cu - pressure Poisson solvers (Computer::SolvePressurePoissonEquation,
// Computer.hpp:1359-1429) on the transposed ELL matrix, each run as one CUDA graph:
// an init kernel, then a conditional WHILE node whose body is a few kernels; the last
// block of each reduction decides the next step and sets the graph condition, so a
// solve of thousands of iterations needs no host round trip.
//
// Reductions: each block sums its rows with warp shuffles, writes one partial, and
// the last block to finish (atomic ticket, no waiting) sums the partials in a fixed
// order.  Results are deterministic run to run.
//
// MPS_SOLVER_CG64: the reference CG in FP64.
// MPS_SOLVER_MIXED: CG whose iterations run in FP32 (FP32 matrix, FP32 SpMV and
// axpy with FP32 accumulation, dot products accumulated in FP64) with reliable
// updates (Sleijpen & van der Vorst 1996): when the recursive residual has dropped by
// `delta` since the last update, the FP32 correction is folded into the FP64
// solution and the true residual b - A x is recomputed in FP64 (FP64 matrix), which
// also decides convergence.
#include "cg.cuh"

namespace mpsgb {

namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
    return v;
}

// Sum over the block; valid in thread 0.
__device__ double block_sum(double v, double* ws) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    v = warp_sum(v);
    if (lane == 0) ws[wid] = v;
    __syncthreads();
    const int nw = blockDim.x >> 5;
    v = (static_cast<int>(threadIdx.x) < nw) ? ws[threadIdx.x] : 0.0;
    if (wid == 0) v = warp_sum(v);
    __syncthreads();
    return v;
}

// Writes this block's partials; true in the last block to finish.
__device__ bool publish(double s0, double s1, double* partials, uint32_t* counter) {
    __shared__ bool last;
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = s0;
        partials[gridDim.x + blockIdx.x] = s1;
        __threadfence();
        const uint32_t t = atomicAdd(counter, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    return last;
}

// In the last block: fixed-order sum of the partials (valid in thread 0).
__device__ double gather_sum(const double* partials, int nparts, double* ws) {
    double v = 0.0;
    for (int k = threadIdx.x; k < nparts; k += blockDim.x) v += __ldcg(partials + k);
    return block_sum(v, ws);
}

// Row i of the FP64 matrix times v (ascending columns, FMA).  The matrix is read
// with streaming hints: in FP64 it is larger than L2 on big scenes, and evicting it
// first keeps the solver's vectors resident.
__device__ __forceinline__ double row64(const CgOperands& o, int i, const double* v) {
    const int L = o.len[i];
    const int n = o.n;
    double s = 0.0;
    int k = 0;
    for (; k + 4 <= L; k += 4) {
        const int c0 = __ldcs(o.col + ell(k, n, i)), c1 = __ldcs(o.col + ell(k + 1, n, i));
        const int c2 = __ldcs(o.col + ell(k + 2, n, i)), c3 = __ldcs(o.col + ell(k + 3, n, i));
        const double a0 = __ldcs(o.val + ell(k, n, i)), a1 = __ldcs(o.val + ell(k + 1, n, i));
        const double a2 = __ldcs(o.val + ell(k + 2, n, i)), a3 = __ldcs(o.val + ell(k + 3, n, i));
        const double v0 = v[c0], v1 = v[c1], v2 = v[c2], v3 = v[c3];
        s = fma(a0, v0, s);
        s = fma(a1, v1, s);
        s = fma(a2, v2, s);
        s = fma(a3, v3, s);
    }
    for (; k < L; k++) s = fma(__ldcs(o.val + ell(k, n, i)), v[__ldcs(o.col + ell(k, n, i))], s);
    return s;
}

// Row i of the FP64 matrix times (x + d) with d the FP32 correction (MIXED true residual).
__device__ __forceinline__ double row64_xd(const CgOperands& o, int i) {
    const int L = o.len[i];
    const int n = o.n;
    double s = 0.0;
    for (int k = 0; k < L; k++) {
        const int c = __ldcs(o.col + ell(k, n, i));
        const double xc = o.x[c] + static_cast<double>(o.d32[c]);
        s = fma(__ldcs(o.val + ell(k, n, i)), xc, s);
    }
    return s;
}

// Row i of the FP32 matrix times v, FP32 accumulation.  Kept cacheable: the FP32
// matrix is meant to stay in L2 across iterations.
__device__ __forceinline__ float row32(const CgOperands& o, int i, const float* v) {
    const int L = o.len[i];
    const int n = o.n;
    float s = 0.0f;
    int k = 0;
    for (; k + 4 <= L; k += 4) {
        const int c0 = __ldg(o.col + ell(k, n, i)), c1 = __ldg(o.col + ell(k + 1, n, i));
        const int c2 = __ldg(o.col + ell(k + 2, n, i)), c3 = __ldg(o.col + ell(k + 3, n, i));
        const float a0 = __ldg(o.val32 + ell(k, n, i)), a1 = __ldg(o.val32 + ell(k + 1, n, i));
        const float a2 = __ldg(o.val32 + ell(k + 2, n, i)), a3 = __ldg(o.val32 + ell(k + 3, n, i));
        const float v0 = v[c0], v1 = v[c1], v2 = v[c2], v3 = v[c3];
        s = fmaf(a0, v0, s);
        s = fmaf(a1, v1, s);
        s = fmaf(a2, v2, s);
        s = fmaf(a3, v3, s);
    }
    for (; k < L; k++) s = fmaf(__ldg(o.val32 + ell(k, n, i)), v[__ldg(o.col + ell(k, n, i))], s);
    return s;
}

// Threshold and first convergence test (Computer.hpp:1382-1389).
__device__ void init_scalars(CgScalars* S, double rr, double bb, cudaGraphConditionalHandle h,
                             int use_cond) {
    S->counter = 0;
    S->rr = rr;
    S->rr0 = rr;
    S->rr_new = rr;
    S->rr_upd = rr;
    S->true_rr = rr;
    S->bb = bb;
    double thr = rr * S->eps * S->eps;
    if (S->criterion == MPS_CRIT_RHS && bb > 0) thr = bb * S->eps * S->eps;
    S->thr = thr;
    const int conv = (S->criterion == MPS_CRIT_RHS) ? ((rr < thr) || (rr == 0)) : (thr == 0);
    S->converged = conv;
    S->iter = 0;
    S->do_update = 0;
    S->updates = 0;
    S->aborted = 0;
    if (use_cond) cudaGraphSetConditional(h, (!conv && S->max_iter > 0) ? 1u : 0u);
}

// ------------------------------------------------------------- CG64 kernels
// Ap = A x; r = b - Ap; p = r; rr = r.r (Computer.hpp:1382-1385)
__global__ void k_cg_init(CgOperands o, cudaGraphConditionalHandle h, int use_cond) {
    __shared__ double ws[32];
    if (o.status && (o.status->flags & (kStatusCellOverflow | kStatusDeviceCheck))) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            o.S->aborted = 1;
            o.S->converged = 0;
            o.S->iter = 0;
            if (use_cond) cudaGraphSetConditional(h, 0u);
        }
        return;
    }
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double vrr = 0.0, vbb = 0.0;
    if (i < o.n) {
        const double bi = o.b[i];
        const double ri = bi - row64(o, i, o.x);
        o.r[i] = ri;
        o.p[i] = ri;
        vrr = ri * ri;
        vbb = bi * bi;
    }
    const double s0 = block_sum(vrr, ws);
    const double s1 = block_sum(vbb, ws);
    if (publish(s0, s1, o.partials, &o.S->counter)) {
        const double rr = gather_sum(o.partials, gridDim.x, ws);
        const double bb = gather_sum(o.partials + gridDim.x, gridDim.x, ws);
        if (threadIdx.x == 0) init_scalars(o.S, rr, bb, h, use_cond);
    }
}

// Ap = A p; alpha = rr / (p.Ap)
__global__ void k_cg_spmv_dot(CgOperands o) {
    __shared__ double ws[32];
    if (o.S->converged) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (i < o.n) {
        const double s = row64(o, i, o.p);
        o.Ap[i] = s;
        v = o.p[i] * s;
    }
    const double s0 = block_sum(v, ws);
    if (publish(s0, 0.0, o.partials, &o.S->counter)) {
        const double pap = gather_sum(o.partials, gridDim.x, ws);
        if (threadIdx.x == 0) {
            o.S->counter = 0;
            o.S->pAp = pap;
            o.S->alpha = o.S->rr / pap;
        }
    }
}

// x += alpha p; r -= alpha Ap; rrNew = r.r; convergence; beta (Computer.hpp:1402-1420)
__global__ void k_cg_update(CgOperands o, cudaGraphConditionalHandle h, int use_cond) {
    __shared__ double ws[32];
    if (o.S->converged) return;
    const double alpha = o.S->alpha;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (i < o.n) {
        o.x[i] = fma(alpha, o.p[i], o.x[i]);
        const double ri = fma(-alpha, o.Ap[i], o.r[i]);
        o.r[i] = ri;
        v = ri * ri;
    }
    const double s0 = block_sum(v, ws);
    if (publish(s0, 0.0, o.partials, &o.S->counter)) {
        const double rr_new = gather_sum(o.partials, gridDim.x, ws);
        if (threadIdx.x == 0) {
            CgScalars* S = o.S;
            S->counter = 0;
            S->rr_new = rr_new;
            const int conv = rr_new < S->thr;
            S->converged = conv;
            if (!conv) {
                S->beta = rr_new / S->rr;
                S->rr = rr_new;
            }
            S->iter += 1;
            if (use_cond) cudaGraphSetConditional(h, (!conv && S->iter < S->max_iter) ? 1u : 0u);
        }
    }
}

// p = r + beta p
__global__ void k_cg_pupdate(CgOperands o) {
    if (o.S->converged) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < o.n) o.p[i] = fma(o.S->beta, o.p[i], o.r[i]);
}

// |b - A x|^2 in FP64 into S->true_rr (reported as the true relative residual)
__global__ void k_true_residual(CgOperands o) {
    __shared__ double ws[32];
    if (o.S->aborted) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (i < o.n) {
        const double ri = o.b[i] - row64(o, i, o.x);
        v = ri * ri;
    }
    const double s0 = block_sum(v, ws);
    if (publish(s0, 0.0, o.partials, &o.S->counter)) {
        const double rr = gather_sum(o.partials, gridDim.x, ws);
        if (threadIdx.x == 0) {
            o.S->counter = 0;
            o.S->true_rr = rr;
        }
    }
}

// ------------------------------------------------------------ MIXED kernels
// r = b - A x (FP64); r32 = r; p32 = r32; d32 = 0
__global__ void k_mx_init(CgOperands o, cudaGraphConditionalHandle h, int use_cond) {
    __shared__ double ws[32];
    if (o.status && (o.status->flags & (kStatusCellOverflow | kStatusDeviceCheck))) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            o.S->aborted = 1;
            o.S->converged = 0;
            o.S->iter = 0;
            if (use_cond) cudaGraphSetConditional(h, 0u);
        }
        return;
    }
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double vrr = 0.0, vbb = 0.0;
    if (i < o.n) {
        const double bi = o.b[i];
        const double ri = bi - row64(o, i, o.x);
        const float r32 = __double2float_rn(ri);
        o.r32[i] = r32;
        o.p32[i] = r32;
        o.d32[i] = 0.0f;
        vrr = ri * ri;
        vbb = bi * bi;
    }
    const double s0 = block_sum(vrr, ws);
    const double s1 = block_sum(vbb, ws);
    if (publish(s0, s1, o.partials, &o.S->counter)) {
        const double rr = gather_sum(o.partials, gridDim.x, ws);
        const double bb = gather_sum(o.partials + gridDim.x, gridDim.x, ws);
        if (threadIdx.x == 0) {
            init_scalars(o.S, rr, bb, h, use_cond);
            // the recursion runs on the FP32 copy of r
        }
    }
}

// q = A32 p32 (FP32); alpha = rr / (p.q) with the dot in FP64
__global__ void k_mx_spmv_dot(CgOperands o) {
    __shared__ double ws[32];
    if (o.S->converged) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (i < o.n) {
        const float q = row32(o, i, o.p32);
        o.q32[i] = q;
        v = static_cast<double>(o.p32[i]) * static_cast<double>(q);
    }
    const double s0 = block_sum(v, ws);
    if (publish(s0, 0.0, o.partials, &o.S->counter)) {
        const double pq = gather_sum(o.partials, gridDim.x, ws);
        if (threadIdx.x == 0) {
            o.S->counter = 0;
            o.S->pAp = pq;
            o.S->alpha = o.S->rr / pq;
        }
    }
}

// d += alpha p; r -= alpha q (FP32); rr_new in FP64; decides a reliable update
__global__ void k_mx_update(CgOperands o, cudaGraphConditionalHandle h, int use_cond) {
    __shared__ double ws[32];
    if (o.S->converged) return;
    const float a = __double2float_rn(o.S->alpha);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (i < o.n) {
        o.d32[i] = fmaf(a, o.p32[i], o.d32[i]);
        const float ri = fmaf(-a, o.q32[i], o.r32[i]);
        o.r32[i] = ri;
        v = static_cast<double>(ri) * static_cast<double>(ri);
    }
    const double s0 = block_sum(v, ws);
    if (publish(s0, 0.0, o.partials, &o.S->counter)) {
        const double rr_new = gather_sum(o.partials, gridDim.x, ws);
        if (threadIdx.x == 0) {
            CgScalars* S = o.S;
            S->counter = 0;
            S->rr_new = rr_new;
            const int reliable = (rr_new < S->delta2 * S->rr_upd) || (rr_new < S->thr);
            S->do_update = reliable;
            if (!reliable) {
                S->beta = rr_new / S->rr;
                S->rr = rr_new;
                S->iter += 1;
                if (use_cond) cudaGraphSetConditional(h, (S->iter < S->max_iter) ? 1u : 0u);
            }
        }
    }
}

// reliable update: r = b - A (x + d) in FP64; r32 = r; convergence on the true residual
__global__ void k_mx_true(CgOperands o, cudaGraphConditionalHandle h, int use_cond) {
    __shared__ double ws[32];
    if (o.S->converged || !o.S->do_update) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (i < o.n) {
        const double ri = o.b[i] - row64_xd(o, i);
        o.r32[i] = __double2float_rn(ri);
        v = ri * ri;
    }
    const double s0 = block_sum(v, ws);
    if (publish(s0, 0.0, o.partials, &o.S->counter)) {
        const double rr = gather_sum(o.partials, gridDim.x, ws);
        if (threadIdx.x == 0) {
            CgScalars* S = o.S;
            S->counter = 0;
            S->true_rr = rr;
            S->rr_upd = rr;
            S->rr_new = rr;
            S->updates += 1;
            const int conv = rr < S->thr;
            S->converged = conv;
            if (!conv) {
                S->beta = rr / S->rr;
                S->rr = rr;
            }
            S->iter += 1;
            if (use_cond) cudaGraphSetConditional(h, (!conv && S->iter < S->max_iter) ? 1u : 0u);
        }
    }
}

// fold d into x after a reliable update; p32 = r32 + beta p32
__global__ void k_mx_pupdate(CgOperands o) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= o.n) return;
    if (o.S->do_update) {
        o.x[i] = o.x[i] + static_cast<double>(o.d32[i]);
        o.d32[i] = 0.0f;
    }
    if (o.S->converged) return;
    o.p32[i] = fmaf(__double2float_rn(o.S->beta), o.p32[i], o.r32[i]);
}

// after the loop: fold any remaining correction (iteration limit reached)
__global__ void k_mx_finish(CgOperands o) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= o.n || o.S->aborted) return;
    const float d = o.d32[i];
    if (d != 0.0f) {
        o.x[i] = o.x[i] + static_cast<double>(d);
        o.d32[i] = 0.0f;
    }
}

__global__ void k_cg_configure(CgScalars* S, double eps, int criterion, int max_iter,
                               double delta2) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        S->eps = eps;
        S->criterion = criterion;
        S->max_iter = max_iter;
        S->delta2 = delta2;
        S->counter = 0;
        S->converged = 0;
        S->iter = 0;
        S->aborted = 0;
    }
}

}  // namespace

void launch_cg_configure(CgScalars* S, double eps, int criterion, int max_iter, double delta2,
                         cudaStream_t s) {
    k_cg_configure<<<1, 32, 0, s>>>(S, eps, criterion, max_iter, delta2);
}

void launch_true_residual(const CgOperands& ops, double*, cudaStream_t s) {
    k_true_residual<<<grid_for(ops.n), kBlock, 0, s>>>(ops);
}

CgGraph::~CgGraph() { reset(); }

void CgGraph::reset() {
    if (exec_) cudaGraphExecDestroy(exec_);
    if (graph_) cudaGraphDestroy(graph_);
    exec_ = nullptr;
    graph_ = nullptr;
    solver_ = -1;
}

cudaError_t CgGraph::build(int solver, const CgOperands& ops, cudaStream_t s) {
    reset();
    ops_ = ops;
    solver_ = solver;
    const int grid = grid_for(ops.n);
    cudaError_t e = cudaGraphCreate(&graph_, 0);
    if (e != cudaSuccess) return e;
    cudaGraphConditionalHandle h;
    e = cudaGraphConditionalHandleCreate(&h, graph_, 0, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) return e;

    // init kernel
    e = cudaStreamBeginCaptureToGraph(s, graph_, nullptr, nullptr, 0,
                                      cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    if (solver == MPS_SOLVER_CG64)
        k_cg_init<<<grid, kBlock, 0, s>>>(ops, h, 1);
    else
        k_mx_init<<<grid, kBlock, 0, s>>>(ops, h, 1);
    cudaGraph_t captured = nullptr;
    e = cudaStreamEndCapture(s, &captured);
    if (e != cudaSuccess) return e;

    size_t nn = 0;
    e = cudaGraphGetNodes(graph_, nullptr, &nn);
    if (e != cudaSuccess || nn != 1) return e != cudaSuccess ? e : cudaErrorInvalidValue;
    cudaGraphNode_t init_node;
    e = cudaGraphGetNodes(graph_, &init_node, &nn);
    if (e != cudaSuccess) return e;

    // while (cond) { body }
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t while_node;
    e = cudaGraphAddNode(&while_node, graph_, &init_node, nullptr, 1, &cp);
    if (e != cudaSuccess) return e;
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    e = cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0,
                                      cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    if (solver == MPS_SOLVER_CG64) {
        k_cg_spmv_dot<<<grid, kBlock, 0, s>>>(ops);
        k_cg_update<<<grid, kBlock, 0, s>>>(ops, h, 1);
        k_cg_pupdate<<<grid, kBlock, 0, s>>>(ops);
    } else {
        k_mx_spmv_dot<<<grid, kBlock, 0, s>>>(ops);
        k_mx_update<<<grid, kBlock, 0, s>>>(ops, h, 1);
        k_mx_true<<<grid, kBlock, 0, s>>>(ops, h, 1);
        k_mx_pupdate<<<grid, kBlock, 0, s>>>(ops);
    }
    e = cudaStreamEndCapture(s, &captured);
    if (e != cudaSuccess) return e;

    // tail: fold the last correction (MIXED) and measure the true residual
    e = cudaStreamBeginCaptureToGraph(s, graph_, &while_node, nullptr, 1,
                                      cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    if (solver != MPS_SOLVER_CG64) k_mx_finish<<<grid, kBlock, 0, s>>>(ops);
    k_true_residual<<<grid, kBlock, 0, s>>>(ops);
    e = cudaStreamEndCapture(s, &captured);
    if (e != cudaSuccess) return e;

    return cudaGraphInstantiate(&exec_, graph_, 0);
}

cudaError_t CgGraph::launch(cudaStream_t s) {
    if (!exec_) return cudaErrorInvalidValue;
    return cudaGraphLaunch(exec_, s);
}

}  // namespace mpsgb

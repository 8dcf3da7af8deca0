// noalloc.cu - the PPE conjugate-gradient solve for callers that cannot allocate device
// memory.
//
// Some callers of this library do not own the device allocator: a host application
// whose device memory is already reserved by its own caching allocator or arena (a
// deep-learning framework that pre-reserves the pool, an embedded solver inside a
// larger simulation that hands out fixed buffers), or code on a latency-critical path
// where cudaMalloc/cudaFree would implicitly synchronize the device.  Such callers keep
// their CSR system in their own device buffers and need a solve that allocates
// nothing.  This file provides that solve: the reference's FP64 CG
// (Computer::SolvePressurePoissonEquation, src/OpenMps/Computer.hpp:1359-1429) whose
// scratch vectors r, p, Ap, block partials and scalars live in one file-scope static
// device array of fixed size (kNoallocMaxRows rows).  Every GPU that loads the library
// holds that array until the process exits.
//
// In host code the array's name stands for a host-side shadow, not a device address.
// Each call therefore asks the runtime for the array's address in the current device's
// context (cudaGetSymbolAddress, a lookup that allocates nothing) and passes it to the
// kernels.  The address is not cached: after cudaDeviceReset, or with another context
// current on the same device, the module is loaded again and the array can move, so a
// cached address would point at memory this context does not own.  The first call in a
// context may load the library's module (lazy module loading), so make that first call
// before any stream capture.  Every call shares the array and finds the previous
// call's contents; the parts that must start at zero are cleared at the start of each
// call.  Calls that overlap on the GPU (different streams or host threads at the same
// time) race on the array.
#include <cmath>

#include "common.cuh"

namespace mpsgb {

namespace {

constexpr int64_t kNoallocMaxRows = MPS_NOALLOC_MAX_ROWS;
constexpr int kNoallocMaxBlocks = static_cast<int>((kNoallocMaxRows + kBlock - 1) / kBlock);
constexpr int kNoallocScalars = 16;  // doubles reserved for NoallocScalars
constexpr int64_t kNoallocDoubles = 3 * kNoallocMaxRows + 2 * kNoallocMaxBlocks + kNoallocScalars;

struct NoallocScalars {
    double rr, rr_new, alpha, beta, thr, bb, rr0, true_rr;
    unsigned int counter;
    int iter, converged, max_iter;
};
static_assert(sizeof(NoallocScalars) <= kNoallocScalars * sizeof(double), "scalars do not fit");

// The solver's whole scratch: r, p, Ap, partials, scalars.
static __device__ __align__(256) double g_noalloc_scratch[kNoallocDoubles];

struct Scratch {
    double *r, *p, *Ap, *partials;
    NoallocScalars* S;
};

__device__ __forceinline__ Scratch carve(double* base, int64_t n) {
    (void)n;
    Scratch s;
    s.r = base;
    s.p = base + kNoallocMaxRows;
    s.Ap = base + 2 * kNoallocMaxRows;
    s.partials = base + 3 * kNoallocMaxRows;
    s.S = reinterpret_cast<NoallocScalars*>(base + 3 * kNoallocMaxRows + 2 * kNoallocMaxBlocks);
    return s;
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ double block_sum(double v, double* ws) {
    ws[threadIdx.x] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x < 32) {
        for (int k = threadIdx.x; k < static_cast<int>(blockDim.x); k += 32) s += ws[k];
        s = warp_sum(s);
    }
    __syncthreads();
    return s;
}

// Block partials s0, s1; true in the last block to finish (atomic ticket, no waiting).
__device__ bool publish(double s0, double s1, const Scratch& sc) {
    __shared__ bool last;
    if (threadIdx.x == 0) {
        sc.partials[blockIdx.x] = s0;
        sc.partials[gridDim.x + blockIdx.x] = s1;
        __threadfence();
        last = atomicAdd(&sc.S->counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    return last;
}

__device__ double gather(const double* partials, double* ws) {
    double v = 0.0;
    for (int k = threadIdx.x; k < static_cast<int>(gridDim.x); k += blockDim.x) v += __ldcg(partials + k);
    return block_sum(v, ws);
}

__device__ __forceinline__ double csr_row(int64_t i, const int64_t* rp, const int32_t* col,
                                          const double* val, const double* v) {
    double s = 0.0;
    for (int64_t k = rp[i]; k < rp[i + 1]; k++) s = fma(val[k], v[col[k]], s);
    return s;
}

// r = b - A x; p = r; rr, bb; threshold (Computer.hpp:1382-1389)
__global__ void k_na_init(double* base, int64_t n, const int64_t* rp, const int32_t* col,
                          const double* val, const double* b, const double* x, double eps,
                          int criterion, int max_iter) {
    __shared__ double ws[kBlock];
    const Scratch sc = carve(base, n);
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    double vr = 0.0, vb = 0.0;
    if (i < n) {
        const double bi = b[i];
        const double ri = bi - csr_row(i, rp, col, val, x);
        sc.r[i] = ri;
        sc.p[i] = ri;
        vr = ri * ri;
        vb = bi * bi;
    }
    const double s0 = block_sum(vr, ws);
    const double s1 = block_sum(vb, ws);
    if (publish(s0, s1, sc)) {
        const double rr = gather(sc.partials, ws);
        const double bb = gather(sc.partials + gridDim.x, ws);
        if (threadIdx.x == 0) {
            NoallocScalars* S = sc.S;
            S->counter = 0;
            S->rr = rr;
            S->rr0 = rr;
            S->rr_new = rr;
            S->bb = bb;
            double thr = rr * eps * eps;
            if (criterion == MPS_CRIT_RHS && bb > 0) thr = bb * eps * eps;
            S->thr = thr;
            S->converged = (criterion == MPS_CRIT_RHS) ? ((rr < thr) || (rr == 0)) : (thr == 0);
            S->iter = 0;
            S->max_iter = max_iter;
        }
    }
}

__device__ __forceinline__ bool na_done(const NoallocScalars* S) {
    return S->converged || S->iter >= S->max_iter;
}

// Ap = A p; alpha = rr / p.Ap
__global__ void k_na_spmv_dot(double* base, int64_t n, const int64_t* rp, const int32_t* col,
                              const double* val) {
    __shared__ double ws[kBlock];
    const Scratch sc = carve(base, n);
    if (na_done(sc.S)) return;
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    double v = 0.0;
    if (i < n) {
        const double s = csr_row(i, rp, col, val, sc.p);
        sc.Ap[i] = s;
        v = sc.p[i] * s;
    }
    const double s0 = block_sum(v, ws);
    if (publish(s0, 0.0, sc)) {
        const double pap = gather(sc.partials, ws);
        if (threadIdx.x == 0) {
            sc.S->counter = 0;
            sc.S->alpha = sc.S->rr / pap;
        }
    }
}

// x += alpha p; r -= alpha Ap; rrNew; convergence; beta (Computer.hpp:1402-1420)
__global__ void k_na_update(double* base, int64_t n, double* x) {
    __shared__ double ws[kBlock];
    const Scratch sc = carve(base, n);
    if (na_done(sc.S)) return;
    const double alpha = sc.S->alpha;
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    double v = 0.0;
    if (i < n) {
        x[i] = fma(alpha, sc.p[i], x[i]);
        const double ri = fma(-alpha, sc.Ap[i], sc.r[i]);
        sc.r[i] = ri;
        v = ri * ri;
    }
    const double s0 = block_sum(v, ws);
    if (publish(s0, 0.0, sc)) {
        const double rr_new = gather(sc.partials, ws);
        if (threadIdx.x == 0) {
            NoallocScalars* S = sc.S;
            S->counter = 0;
            S->rr_new = rr_new;
            S->converged = rr_new < S->thr;
            if (!S->converged) {
                S->beta = rr_new / S->rr;
                S->rr = rr_new;
            }
            S->iter += 1;
        }
    }
}

// p = r + beta p
__global__ void k_na_pupdate(double* base, int64_t n) {
    const Scratch sc = carve(base, n);
    if (na_done(sc.S)) return;
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i < n) sc.p[i] = fma(sc.S->beta, sc.p[i], sc.r[i]);
}

// |b - A x|^2 into S->true_rr
__global__ void k_na_true(double* base, int64_t n, const int64_t* rp, const int32_t* col,
                          const double* val, const double* b, const double* x) {
    __shared__ double ws[kBlock];
    const Scratch sc = carve(base, n);
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    double v = 0.0;
    if (i < n) {
        const double ri = b[i] - csr_row(i, rp, col, val, x);
        v = ri * ri;
    }
    const double s0 = block_sum(v, ws);
    if (publish(s0, 0.0, sc)) {
        const double rr = gather(sc.partials, ws);
        if (threadIdx.x == 0) {
            sc.S->counter = 0;
            sc.S->true_rr = rr;
        }
    }
}

// Device address of g_noalloc_scratch in the current context, looked up on every call.
int scratch_for_current_context(double** out) {
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) {
        cudaGetLastError();
        return MPS_ERR_CUDA;
    }
    *out = static_cast<double*>(ptr);
    return MPS_OK;
}

}  // namespace

}  // namespace mpsgb

extern "C" int mps_cg_solve_csr_device_noalloc(int64_t n, const int64_t* row_ptr,
                                               const int32_t* col, const double* val,
                                               const double* b, double* x, double eps,
                                               int32_t criterion, int32_t max_iters,
                                               void* stream, int32_t* iterations,
                                               double* true_relres) {
    using namespace mpsgb;
    if (n <= 0 || !row_ptr || !col || !val || !b || !x) return MPS_ERR_INVALID_ARGUMENT;
    if (n > kNoallocMaxRows) return MPS_ERR_NOALLOC_TOO_LARGE;
    if (criterion != MPS_CRIT_INITIAL_RESIDUAL && criterion != MPS_CRIT_RHS) return MPS_ERR_INVALID_ARGUMENT;
    double* base = nullptr;
    const int rc = scratch_for_current_context(&base);
    if (rc != MPS_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int grid = static_cast<int>((n + kBlock - 1) / kBlock);
    const int max_iter = max_iters > 0 ? max_iters : static_cast<int>(n);
    // the ticket counter and the scalars start from zero on every call
    double* scalars = base + 3 * kNoallocMaxRows + 2 * kNoallocMaxBlocks;
    if (cudaMemsetAsync(scalars, 0, kNoallocScalars * sizeof(double), s) != cudaSuccess) return MPS_ERR_CUDA;
    k_na_init<<<grid, kBlock, 0, s>>>(base, n, row_ptr, col, val, b, x, eps, criterion, max_iter);
    NoallocScalars S{};
    const int kCheck = 16;  // iterations between host reads of the convergence flag
    for (;;) {
        if (cudaGetLastError() != cudaSuccess) return MPS_ERR_CUDA;
        if (cudaMemcpyAsync(&S, scalars, sizeof(S), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return MPS_ERR_CUDA;
        if (S.converged || S.iter >= S.max_iter) break;
        for (int c = 0; c < kCheck; c++) {
            k_na_spmv_dot<<<grid, kBlock, 0, s>>>(base, n, row_ptr, col, val);
            k_na_update<<<grid, kBlock, 0, s>>>(base, n, x);
            k_na_pupdate<<<grid, kBlock, 0, s>>>(base, n);
        }
    }
    k_na_true<<<grid, kBlock, 0, s>>>(base, n, row_ptr, col, val, b, x);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(&S, scalars, sizeof(S), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return MPS_ERR_CUDA;
    if (iterations) *iterations = S.iter;
    if (true_relres) *true_relres = (S.bb > 0) ? std::sqrt(S.true_rr / S.bb) : std::sqrt(S.true_rr);
    return S.converged ? MPS_OK : MPS_ERR_CG_NOT_CONVERGED;
}

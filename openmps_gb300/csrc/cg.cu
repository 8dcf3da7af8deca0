// cg.cu - pressure Poisson solvers (Computer::SolvePressurePoissonEquation,
// Computer.hpp:1359-1429) on the SELL-32 matrix, each run as one CUDA graph: an init
// kernel, then a conditional WHILE node whose body is a few kernels; the last block of
// each reduction decides the next step and sets the graph condition, so a solve of
// thousands of iterations needs no host round trip.
//
// Work layout: vector kernels run one thread per row, SpMV kernels one warp per chunk of
// 32 rows (one lane per row, as many warps as chunks, so the block scheduler balances
// uneven chunks);
// each warp load reads 32 consecutive matrix entries and a row is summed by its own lane
// in ascending column order (no cross-lane reduction: in FP64 every instruction counts,
// the FP64 pipe bounds this kernel on GB300).  Row loads are software-pipelined (eight
// entries per step for the FP64 rows, four for the preconditioned FP32 SpMV) so that each
// lane keeps matrix loads and gathers in flight.
//
// Reductions (grid_sum): lanes park their values in shared memory and the block's last
// warp adds them; blocks publish partials in groups of 32, the last block of a group adds
// the group's, and the last group adds the group sums (atomic tickets, no waiting).  Every
// addition has a fixed order, so results are deterministic run to run.
//
// MPS_SOLVER_CG64: the reference CG in FP64 (3 kernels per iteration).
// MPS_SOLVER_MIXED: CG whose iterations run in FP32 (FP32 matrix, FP32 SpMV and axpy with
// FP32 accumulation, dot products accumulated in FP64) with reliable updates (Sleijpen &
// van der Vorst 1996): when the recursive residual has dropped by `delta` since the last
// update, the FP32 correction is folded into the FP64 solution and the true residual
// b - A x is recomputed with the FP64 matrix, which also decides convergence.  The
// direction update p = r + beta p is folded into the next SpMV (each lane forms
// beta p_j + r_j while gathering), so an iteration is two kernels; the reliable update
// runs under a conditional IF node only when due.
// MPS_SOLVER_MIXED_MG / LEARNED: the same FP32 iteration preconditioned by the cell
// multigrid (mg.cu), three dot products per reduction; if it stalls or runs out of
// iterations the plain FP64 CG continues from the solution it reached, inside the same
// graph (a second WHILE node that runs zero times after a converged solve).
#include <cmath>
#include <vector>

#include "learned.cuh"

namespace mpsgb {

namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
    return v;
}

// Grid-wide sums of up to three values without block barriers: every lane parks its
// values in shared memory; the last warp of the block to arrive (shared-memory ticket)
// adds the block's values in a fixed order and publishes one partial per block; groups
// of blocks and then the groups are summed the same way (global tickets).  Warps that
// finish their rows early leave at once instead of waiting at __syncthreads for the
// block's longest row.  The order of every addition is fixed, so the sums are the same
// run to run.
struct BlockTicket {
    unsigned count;
    double lanes[3][kBlock];
};

// Must run in every thread of the block before the first grid_sum (uniform code path).
__device__ __forceinline__ void ticket_init(BlockTicket& t) {
    if (threadIdx.x == 0) t.count = 0;
    __syncthreads();
}

// True in exactly one thread of the grid, which then holds the totals in out[0..2].
// Blocks publish partials in groups of 32: the last block of a group adds its group's
// partials (one load per lane) and the last group adds the group sums, so the final sum
// costs a few L2 round trips however many blocks the grid has.  `partials` holds
// 3 * (blocks + groups) doubles, `tickets` one counter per group, `counter` the last one.
__device__ bool grid_sum(double a, double b, double c, double* partials, uint32_t* tickets,
                         uint32_t* counter, BlockTicket& T, double* out) {
    const int lane = threadIdx.x & 31;
    const int nwarps = static_cast<int>(blockDim.x >> 5);
    // FP64 instructions are scarce on GB300: lanes park raw values in shared memory and
    // only the block's last warp adds them (8 adds + one 5-level tree per value)
    T.lanes[0][threadIdx.x] = a;
    T.lanes[1][threadIdx.x] = b;
    T.lanes[2][threadIdx.x] = c;
    __threadfence_block();
    unsigned last = 0;
    if (lane == 0) last = atomicAdd(&T.count, 1u) == static_cast<unsigned>(nwarps - 1);
    if (!__shfl_sync(kFull, last, 0)) return false;
    __threadfence_block();
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int w = 0; w < nwarps; w++) {
        s0 += T.lanes[0][32 * w + lane];
        s1 += T.lanes[1][32 * w + lane];
        s2 += T.lanes[2][32 * w + lane];
    }
    s0 = warp_sum(s0);
    s1 = warp_sum(s1);
    s2 = warp_sum(s2);
    const int G = static_cast<int>(gridDim.x);
    const int NG = (G + 31) / 32;
    const int group = static_cast<int>(blockIdx.x) / 32;
    const int gsize = min(32, G - group * 32);
    unsigned group_last = 0;
    if (lane == 0) {
        partials[blockIdx.x] = s0;
        partials[G + blockIdx.x] = s1;
        partials[2 * G + blockIdx.x] = s2;
        __threadfence();
        group_last = atomicAdd(tickets + group, 1u) == static_cast<unsigned>(gsize - 1);
    }
    if (!__shfl_sync(kFull, group_last, 0)) return false;
    __threadfence();
    double x = 0.0, y = 0.0, z = 0.0;
    if (lane < gsize) {
        const int k = group * 32 + lane;
        x = __ldcg(partials + k);
        y = __ldcg(partials + G + k);
        z = __ldcg(partials + 2 * G + k);
    }
    x = warp_sum(x);
    y = warp_sum(y);
    z = warp_sum(z);
    double* gp = partials + 3 * G;
    unsigned all_last = 0;
    if (lane == 0) {
        tickets[group] = 0;
        gp[group] = x;
        gp[NG + group] = y;
        gp[2 * NG + group] = z;
        __threadfence();
        all_last = atomicAdd(counter, 1u) == static_cast<unsigned>(NG - 1);
    }
    if (!__shfl_sync(kFull, all_last, 0)) return false;
    __threadfence();
    x = y = z = 0.0;
    for (int k = lane; k < NG; k += 32) {
        x += __ldcg(gp + k);
        y += __ldcg(gp + NG + k);
        z += __ldcg(gp + 2 * NG + k);
    }
    x = warp_sum(x);
    y = warp_sum(y);
    z = warp_sum(z);
    if (lane != 0) return false;
    out[0] = x;
    out[1] = y;
    out[2] = z;
    *counter = 0;
    return true;
}

__device__ __forceinline__ bool cg_done(const CgScalars* S) {
    return S->converged || S->aborted || S->iter >= S->max_iter;
}

// One warp per chunk of kSellRows rows (lane = row within the chunk).  The SpMV kernels
// launch as many warps as chunks so the block scheduler balances uneven chunks.
struct ChunkLoop {
    int lane, warp, nwarps;
    __device__ ChunkLoop() {
        lane = threadIdx.x & 31;
        warp = static_cast<int>((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
        nwarps = static_cast<int>((gridDim.x * blockDim.x) >> 5);
    }
};

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
    S->beta = 0.0;
    double thr = rr * S->eps * S->eps;
    if (S->criterion == MPS_CRIT_RHS && bb > 0) thr = bb * S->eps * S->eps;
    S->thr = thr;
    const int conv = (S->criterion == MPS_CRIT_RHS) ? ((rr < thr) || (rr == 0)) : (thr == 0);
    S->converged = conv;
    S->iter = 0;
    S->do_update = 0;
    S->updates = 0;
    S->aborted = 0;
    S->stalled = 0;
    S->prev_true_rr = rr;
    S->iter_upd = 0;
    if (use_cond) cudaGraphSetConditional(h, (!conv && S->max_iter > 0) ? 1u : 0u);
}

__device__ __forceinline__ bool aborted_before_solve(const CgOperands& o,
                                                     cudaGraphConditionalHandle h, int use_cond) {
    if (o.status && (o.status->flags & (kStatusCellOverflow | kStatusDeviceCheck))) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            o.S->aborted = 1;
            o.S->converged = 0;
            o.S->iter = 0;
            if (use_cond) cudaGraphSetConditional(h, 0u);
        }
        return true;
    }
    return false;
}

// ------------------------------------------------------------- CG64 kernels
// Ap = A x; r = b - Ap; p = r; rr = r.r (Computer.hpp:1382-1385).  With `gate` (the
// fallback after a preconditioned solve) nothing runs unless that solve failed.
__global__ void __launch_bounds__(kBlock) k_cg_init(CgOperands o, cudaGraphConditionalHandle h,
                                                   int use_cond, const CgScalars* gate) {
    __shared__ BlockTicket tk;
    if (gate && (gate->converged || gate->aborted)) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            o.S->converged = gate->converged;
            o.S->aborted = gate->aborted;
            o.S->iter = 0;
            if (use_cond) cudaGraphSetConditional(h, 0u);
        }
        return;
    }
    if (aborted_before_solve(o, h, use_cond)) return;
    ticket_init(tk);
    const ChunkLoop cl;
    const double* x = o.x;
    double vrr = 0.0, vbb = 0.0;
    for (int c = cl.warp; c < o.nchunks; c += cl.nwarps) {
        const int i = kSellRows * c + cl.lane;
        const int L = o.len[i];
        const double ax = row64(o, sell_index(o.off[c], cl.lane, 0), L, [&](int j) { return x[j]; });
        if (i < o.n) {
            const double bi = o.b[i];
            const double ri = bi - ax;
            o.r[i] = ri;
            o.p[i] = ri;
            vrr += ri * ri;
            vbb += bi * bi;
        }
    }
    double tot[3];
    if (grid_sum(vrr, vbb, 0.0, o.partials, o.tickets, &o.S->counter, tk, tot)) init_scalars(o.S, tot[0], tot[1], h, use_cond);
}

// Ap = A p; alpha = rr / (p.Ap)
__global__ void __launch_bounds__(kBlock) k_cg_spmv_dot(CgOperands o) {
    __shared__ BlockTicket tk;
    if (cg_done(o.S)) return;
    ticket_init(tk);
    const ChunkLoop cl;
    const double* p = o.p;
    double v = 0.0;
    for (int c = cl.warp; c < o.nchunks; c += cl.nwarps) {
        const int i = kSellRows * c + cl.lane;
        const int L = o.len[i];
        const double s = row64(o, sell_index(o.off[c], cl.lane, 0), L, [&](int j) { return p[j]; });
        if (i < o.n) {
            o.Ap[i] = s;
            v += p[i] * s;
        }
    }
    double tot[3];
    if (grid_sum(v, 0.0, 0.0, o.partials, o.tickets, &o.S->counter, tk, tot)) {
        const double pap = tot[0];
        {
            o.S->counter = 0;
            o.S->pAp = pap;
            o.S->alpha = o.S->rr / pap;
        }
    }
}

// x += alpha p; r -= alpha Ap; rrNew = r.r; convergence; beta (Computer.hpp:1402-1420)
__global__ void __launch_bounds__(kBlock) k_cg_update(CgOperands o, cudaGraphConditionalHandle h,
                                                     int use_cond) {
    __shared__ BlockTicket tk;
    if (cg_done(o.S)) return;
    ticket_init(tk);
    const double alpha = o.S->alpha;
    double v = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < o.n; i += gridDim.x * blockDim.x) {
        o.x[i] = fma(alpha, o.p[i], o.x[i]);
        const double ri = fma(-alpha, o.Ap[i], o.r[i]);
        o.r[i] = ri;
        v += ri * ri;
    }
    double tot[3];
    if (grid_sum(v, 0.0, 0.0, o.partials, o.tickets, &o.S->counter, tk, tot)) {
        const double rr_new = tot[0];
        {
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
__global__ void __launch_bounds__(kBlock) k_cg_pupdate(CgOperands o) {
    if (cg_done(o.S)) return;
    const double beta = o.S->beta;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < o.n; i += gridDim.x * blockDim.x)
        o.p[i] = fma(beta, o.p[i], o.r[i]);
}

// |b - A x|^2 in FP64 into S->true_rr (reported as the true relative residual)
// |b - A x|^2 in FP64 for the statistics.  With `after_update` (the mixed-precision
// solves) a solve that converged on its own already holds it: convergence is only ever
// declared by a reliable update, on the true residual of the x it leaves.
__global__ void __launch_bounds__(kBlock) k_true_residual(CgOperands o, int after_update) {
    __shared__ BlockTicket tk;
    if (o.S->aborted) return;
    if (after_update && o.S->converged && !o.S->fallback) return;
    ticket_init(tk);
    const ChunkLoop cl;
    const double* x = o.x;
    double v = 0.0;
    for (int c = cl.warp; c < o.nchunks; c += cl.nwarps) {
        const int i = kSellRows * c + cl.lane;
        const int L = o.len[i];
        const double ax = row64(o, sell_index(o.off[c], cl.lane, 0), L, [&](int j) { return x[j]; });
        if (i < o.n) {
            const double ri = o.b[i] - ax;
            v += ri * ri;
        }
    }
    double tot[3];
    if (grid_sum(v, 0.0, 0.0, o.partials, o.tickets, &o.S->counter, tk, tot)) {
        const double rr = tot[0];
        {
            o.S->counter = 0;
            o.S->true_rr = rr;
        }
    }
}

// ------------------------------------------------------------ MIXED kernels
// Chronopoulos-Gear CG (Chronopoulos & Gear 1989): with s = A p and w = A r kept as
// vectors, both dot products of an iteration (gamma = r.r, delta = w.r) come out of one
// reduction.  An iteration is an elementwise kernel (s, p, d, r updates, no reduction)
// followed by the SpMV w = A r that also forms gamma and delta and the next step sizes.

// init: r_0 = b - A x (FP64); r32 = r_0; d = 0; p = 0; s = 0; rr, bb
__global__ void __launch_bounds__(kBlock) k_mx_init(CgOperands o, cudaGraphConditionalHandle h,
                                                   int use_cond) {
    __shared__ BlockTicket tk;
    if (aborted_before_solve(o, h, use_cond)) return;
    ticket_init(tk);
    const ChunkLoop cl;
    const double* x = o.x;
    double vrr = 0.0, vbb = 0.0;
    for (int c = cl.warp; c < o.nchunks; c += cl.nwarps) {
        const int i = kSellRows * c + cl.lane;
        const int L = o.len[i];
        const double ax = row64(o, sell_index(o.off[c], cl.lane, 0), L, [&](int j) { return x[j]; });
        if (i < o.n) {
            const double bi = o.b[i];
            const double ri = bi - ax;
            o.r32[i] = __double2float_rn(ri);
            o.s32[i] = 0.0f;
            o.p32[i] = 0.0f;
            o.d32[i] = 0.0f;
            if (o.u32) o.u32[i] = 0.0f;  // rows outside every cell keep u = 0
            vrr += ri * ri;
            vbb += bi * bi;
        }
    }
    double tot[3];
    if (grid_sum(vrr, vbb, 0.0, o.partials, o.tickets, &o.S->counter, tk, tot)) init_scalars(o.S, tot[0], tot[1], h, use_cond);
}

// s = w + beta s; p = r + beta p; d += alpha p; r -= alpha s (FP32, no reduction)
__global__ void __launch_bounds__(kBlock) k_mx_axpy(CgOperands o) {
    if (cg_done(o.S)) return;
    const float alpha = __double2float_rn(o.S->alpha);
    const float beta = __double2float_rn(o.S->beta);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < o.n; i += gridDim.x * blockDim.x) {
        const float ri = o.r32[i];
        const float si = fmaf(beta, o.s32[i], o.w32[i]);
        const float pi = fmaf(beta, o.p32[i], ri);
        o.s32[i] = si;
        o.p32[i] = pi;
        o.d32[i] = fmaf(alpha, pi, o.d32[i]);
        o.r32[i] = fmaf(-alpha, si, ri);
    }
}

// w = A r (FP32); gamma = r.r and delta = w.r in FP64; the next Chronopoulos-Gear step
// sizes; decides a reliable update.  mode 0: after init (beta = 0); mode 1: an
// iteration; mode 2: after a reliable update (also clears d, folded into x).
// Iterations the plain mixed solver may run without a reliable update (a tenfold drop of
// its recursive residual norm takes a few hundred iterations on the PPEs of the
// workloads when the FP32 recursion makes progress).
constexpr int kMixedStallIter = 2000;

__global__ void __launch_bounds__(kBlock) k_mx_spmv(CgOperands o, int mode,
                                                   cudaGraphConditionalHandle h,
                                                   cudaGraphConditionalHandle h_true, int use_cond) {
    __shared__ BlockTicket tk;
    CgScalars* S = o.S;
    if (mode == 2) {
        if (S->converged || S->aborted || !S->do_update) return;
    } else if (mode == 1) {
        if (cg_done(S)) return;
    } else if (S->converged || S->aborted) {
        return;
    }
    ticket_init(tk);
    const ChunkLoop cl;
    const float* __restrict__ r = o.r32;
    double vg = 0.0, vd = 0.0;
    for (int c = cl.warp; c < o.nchunks; c += cl.nwarps) {
        const int i = kSellRows * c + cl.lane;
        const int L = o.len[i];
        const float wi = row32(o, sell_index(o.off[c], cl.lane, 0), L, r);
        if (i < o.n) {
            const double ri = static_cast<double>(r[i]);
            o.w32[i] = wi;
            if (mode == 2) o.d32[i] = 0.0f;
            vg += ri * ri;
            vd += static_cast<double>(wi) * ri;
        }
    }
    double tot[3];
    if (grid_sum(vg, vd, 0.0, o.partials, o.tickets, &o.S->counter, tk, tot)) {
        const double gam = tot[0];
        const double del = tot[1];
        {
            S->counter = 0;
            S->rr_new = gam;
            int reliable = 0;
            if (mode == 1) {
                reliable = (gam < S->delta2 * S->rr_upd) || (gam < S->thr);
                S->do_update = reliable;
                if (use_cond && h_true) cudaGraphSetConditional(h_true, reliable ? 1u : 0u);
            }
            if (!reliable) {
                if (mode == 0) {
                    S->beta = 0.0;
                    S->alpha = gam / del;
                } else {
                    const double beta = gam / S->rr;
                    S->beta = beta;
                    S->alpha = gam / (del - beta * gam / S->alpha);
                    S->iter += 1;
                    // no tenfold drop of the recursive residual for kMixedStallIter
                    // iterations: the FP32 iteration has stalled (the FP64 CG takes over)
                    const int stuck = S->iter - S->iter_upd > kMixedStallIter;
                    if (stuck) S->stalled = 1;
                    if (use_cond) cudaGraphSetConditional(h, (!stuck && S->iter < S->max_iter) ? 1u : 0u);
                }
                S->rr = gam;
                S->pAp = del;
            }
            if (mode == 2) {
                // after a reliable update: the true residual must at least halve in norm
                // between updates, or the FP32 iteration has stalled (the FP64 CG takes over)
                const int stalled = S->true_rr > 0.25 * S->prev_true_rr;
                S->prev_true_rr = S->true_rr;
                S->stalled = stalled;
                S->do_update = 0;
                if (use_cond && stalled) cudaGraphSetConditional(h, 0u);
            }
        }
    }
}

// Reliable update, part 1: x' = x + d and r = b - A x' in FP64 (FP64 matrix), written
// over the r the iteration produced; convergence on this true residual.
// The scalars after a reliable update's true residual r.r: the new reference for the
// next update, and convergence (which ends the loop).
__device__ __forceinline__ void true_residual_done(CgScalars* S, double rr, cudaGraphConditionalHandle h,
                                                   int use_cond) {
    S->true_rr = rr;
    S->rr_upd = rr;
    S->rr_new = rr;
    S->updates += 1;
    S->iter_upd = S->iter;
    const int conv = rr < S->thr;
    S->converged = conv;
    if (conv) {
        S->iter += 1;
        if (use_cond) cudaGraphSetConditional(h, 0u);
    }
}

__global__ void __launch_bounds__(kBlock) k_mx_true(CgOperands o, cudaGraphConditionalHandle h,
                                                   int use_cond) {
    __shared__ BlockTicket tk;
    if (o.S->converged || o.S->aborted || o.S->stalled || !o.S->do_update) return;
    ticket_init(tk);
    const ChunkLoop cl;
    const bool odd = (o.S->updates & 1) != 0;
    const double* __restrict__ xc = odd ? o.x2 : o.x;
    double* __restrict__ xn = odd ? o.x : o.x2;
    const float* __restrict__ d = o.d32;
    float* __restrict__ rslot = o.r32;
    double v = 0.0;
    for (int c = cl.warp; c < o.nchunks; c += cl.nwarps) {
        const int i = kSellRows * c + cl.lane;
        const int L = o.len[i];
        const double ax = row64(o, sell_index(o.off[c], cl.lane, 0), L,
                                [&](int j) { return xc[j] + static_cast<double>(d[j]); });
        if (i < o.n) {
            const double ri = o.b[i] - ax;
            xn[i] = xc[i] + static_cast<double>(d[i]);
            rslot[i] = __double2float_rn(ri);
            v += ri * ri;
        }
    }
    double tot[3];
    if (grid_sum(v, 0.0, 0.0, o.partials, o.tickets, &o.S->counter, tk, tot)) {
        o.S->counter = 0;
        true_residual_done(o.S, tot[0], h, use_cond);
    }
}

// After the loop: the solution into x (fold a pending correction, leave the x2 buffer).
__global__ void __launch_bounds__(kBlock) k_mx_finish(CgOperands o) {
    if (o.S->aborted) return;
    const bool odd = (o.S->updates & 1) != 0;
    const bool folded = o.S->do_update != 0;
    const double* xc = odd ? o.x2 : o.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < o.n; i += gridDim.x * blockDim.x) {
        const float di = o.d32[i];
        o.x[i] = folded ? xc[i] : xc[i] + static_cast<double>(di);
        o.d32[i] = 0.0f;
    }
}

// -------------------------------------------------- preconditioned MIXED kernels
// Preconditioned Chronopoulos-Gear CG with u = M r, w = A u and s = A p kept as vectors:
// gamma = r.u, delta = w.u and rho = r.r (convergence and reliable updates) come out of
// one reduction.  A and M are both negative definite on the rows the solve acts on, so
// this is CG on the SPD pair (-A, -M).

// The last block's step of the preconditioned SpMV: the dot products gamma = r.u,
// delta = w.u, rho = r.r decide the next step sizes, a reliable update (mode 1) or a
// stall (mode 2), and the loop's condition.
__device__ __forceinline__ void pmx_finish(CgScalars* S, int mode, const double* tot, cudaGraphConditionalHandle h,
                                           cudaGraphConditionalHandle h_true, int use_cond) {
    const double gam = tot[0];
    const double del = tot[1];
    const double rho = tot[2];
    S->counter = 0;
    S->rr_new = rho;
    int reliable = 0;
    int stalled = 0;
    if (mode == 1) {
        reliable = (rho < S->delta2 * S->rr_upd) || (rho < S->thr);
        S->do_update = reliable;
        if (use_cond && h_true) cudaGraphSetConditional(h_true, reliable ? 1u : 0u);
    } else if (mode == 2) {
        stalled = S->true_rr > 0.25 * S->prev_true_rr;
        S->prev_true_rr = S->true_rr;
    }
    if (!reliable && !stalled) {
        double alpha, beta = 0.0;
        if (mode == 0) {
            alpha = gam / del;
        } else {
            beta = gam / S->rr;
            alpha = gam / (del - beta * gam / S->alpha);
            S->iter += 1;
        }
        stalled = !(std::isfinite(alpha) && std::isfinite(beta) && alpha != 0.0);
        S->alpha = alpha;
        S->beta = beta;
        S->rr = gam;
        S->pAp = del;
    }
    if (mode == 2) S->do_update = 0;
    S->stalled = stalled;
    if (use_cond && (mode != 1 || !reliable))
        cudaGraphSetConditional(h, (!stalled && S->iter < S->max_iter) ? 1u : 0u);
}

// w = A u (FP32); gamma, delta, rho in FP64; next step sizes; reliable-update decision
// (mode 1) or stall check (mode 2: the true residual must at least halve between updates).
// Five entries per pipeline step at 48 registers and five blocks per SM (measured on the
// 340k PPE, alone after an L2 flush: 37.7 us against 39.0 for four entries, 38.8 for six,
// 42-43 for eight at three or four blocks, 39.6-41.0 at six blocks and 40 registers).
constexpr int kPmxDepth = 5;

__global__ void __launch_bounds__(kBlock, 5) k_pmx_spmv(CgOperands o, int mode,
                                                    cudaGraphConditionalHandle h,
                                                    cudaGraphConditionalHandle h_true, int use_cond) {
    __shared__ BlockTicket tk;
    CgScalars* S = o.S;
    const ChunkLoop cl;
    // Before the wait for u: the first chunk's row length and first stream entries (the
    // matrix is fixed for the solve) and the row's residual (written by the vector
    // updates or the reliable update, three or more kernels back).
    int L0 = 0;
    uint2 e0[kPmxDepth];
    float r0 = 0.0f;
    if (cl.warp < o.nchunks) {
        const int i = kSellRows * cl.warp + cl.lane;
        L0 = o.len[i];
        row32_first(o, sell_index(o.off[cl.warp], cl.lane, 0), L0, e0);
        if (i < o.n) r0 = o.r32[i];
    }
    pdl_begin();
    if (pcg_skip(S, mode)) return;
    ticket_init(tk);
    const float* __restrict__ u = o.u32;
    double vg = 0.0, vd = 0.0, vr = 0.0;
    auto row_done = [&](int i, float wi, float rf) {
        if (i < o.n) {
            const double ri = static_cast<double>(rf);
            const double ui = static_cast<double>(u[i]);
            o.w32[i] = wi;
            if (mode == 2) o.d32[i] = 0.0f;
            vg += ri * ui;
            vd += static_cast<double>(wi) * ui;
            vr += ri * ri;
        }
    };
    if (cl.warp < o.nchunks) {
        const int i = kSellRows * cl.warp + cl.lane;
        row_done(i, row32_rest(o, sell_index(o.off[cl.warp], cl.lane, 0), L0, u, e0), r0);
    }
    // further chunks (the launch gives every warp one chunk; kept for other grids)
    for (int c = cl.warp + cl.nwarps; c < o.nchunks; c += cl.nwarps) {
        const int i = kSellRows * c + cl.lane;
        const int L = o.len[i];
        const int64_t at = sell_index(o.off[c], cl.lane, 0);
        uint2 e[kPmxDepth];
        row32_first(o, at, L, e);
        const float wi = row32_rest(o, at, L, u, e);
        row_done(i, wi, i < o.n ? o.r32[i] : 0.0f);
    }
    double tot[3];
    if (grid_sum(vg, vd, vr, o.partials, o.tickets, &o.S->counter, tk, tot)) pmx_finish(S, mode, tot, h, h_true, use_cond);
}

// ------------------------------------------------ staged SELL stream
// A slice of a chunk, entries [k0, k0 + m) of its 32 rows, is one contiguous block of the
// SELL stream (entry k of lane r sits at off[c] + 32 k + r).  The staged FP64 SpMV
// copies slices into a per-warp ring of shared-memory stages with bulk copies
// (cp.async.bulk, global to this CTA's shared memory, completion counted in bytes on one
// mbarrier per stage) issued STAGES slices ahead of the warp's arithmetic.  The stream's
// DRAM latency then leaves the lanes' dependency chain: a lane reads its entries from
// shared memory and issues only the gathers of the vector and its FP64 multiply-adds.
// The grid has a few blocks per SM (as many as the ring's shared memory allows) and
// every warp walks the chunks gw, gw + nw, ... (nw = warps in the grid).
constexpr int kStgWarps = 8;
constexpr int kStgThreads = kStgWarps * 32;
// a stage wait that runs this long gives up: the kernel flags kStatusWaitTimeout, waits
// (bounded again) for the copies it issued, and skips its remaining rows
constexpr long long kStageWaitClocks = 2000000000LL;

__device__ __forceinline__ uint32_t stg_smem(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void stg_bar_init(uint64_t* b) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(stg_smem(b)) : "memory");
}

__device__ __forceinline__ void stg_expect(uint64_t* b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(stg_smem(b)), "r"(bytes) : "memory");
}

// global -> shared bulk copy; dst, src 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void stg_copy(void* dst, const void* src, uint32_t bytes, uint64_t* b) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     stg_smem(dst)),
                 "l"(src), "r"(bytes), "r"(stg_smem(b))
                 : "memory");
}

__device__ __forceinline__ bool stg_test(uint64_t* b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(stg_smem(b)), "r"(parity)
        : "memory");
    return ok != 0;
}

// true once the stage's copy has landed; false after kStageWaitClocks (warp-uniform)
__device__ __forceinline__ bool stg_wait(uint64_t* b, uint32_t parity) {
    const long long t0 = clock64();
    bool ok = true;
    while (!stg_test(b, parity)) {
        if (clock64() - t0 > kStageWaitClocks) {
            ok = false;
            break;
        }
    }
    return __all_sync(kFull, ok);
}

// The producer side of a warp's ring: which slice goes next, and its bulk copies.
// NARR arrays stream side by side (the FP64 matrix has columns and values apart); a
// stage holds SLICE * 32 entries of each.
template <int SLICE, int STAGES, int NARR>
struct StageRing {
    static constexpr int kEntries = SLICE * kSellRows;
    unsigned char* buf;  // this warp's stages
    uint64_t* bar;       // this warp's STAGES mbarriers
    const void* src[NARR];
    int esize[NARR];
    int stage_bytes;
    int pc, ps, issued;  // next chunk and slice to copy; slices copied so far

    __device__ void init(unsigned char* base, uint64_t* bars, int gw) {
        buf = base;
        bar = bars;
        stage_bytes = 0;
        for (int a = 0; a < NARR; a++) stage_bytes += kEntries * esize[a];
        pc = gw;
        ps = 0;
        issued = 0;
        if ((threadIdx.x & 31) == 0) {
            for (int k = 0; k < STAGES; k++) stg_bar_init(bar + k);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        __syncwarp();
    }
    __device__ __forceinline__ unsigned char* stage(int item, int a) const {
        unsigned char* p = buf + (item % STAGES) * stage_bytes;
        for (int k = 0; k < a; k++) p += kEntries * esize[k];
        return p;
    }
    // copies the next slice of the warp's chunks into stage `issued % STAGES`
    __device__ void issue(const CgOperands& o, int nw) {
        while (pc < o.nchunks) {
            const int off = o.off[pc];
            const int width = o.chunk[pc] / kSellRows;
            if (ps * SLICE < width) {
                const int m = min(SLICE, width - ps * SLICE);
                if ((threadIdx.x & 31) == 0) {
                    uint64_t* b = bar + issued % STAGES;
                    uint32_t bytes = 0;
                    for (int a = 0; a < NARR; a++) bytes += static_cast<uint32_t>(m * kSellRows * esize[a]);
                    stg_expect(b, bytes);
                    const int64_t first = static_cast<int64_t>(off) + static_cast<int64_t>(ps) * kEntries;
                    for (int a = 0; a < NARR; a++)
                        stg_copy(stage(issued, a), static_cast<const unsigned char*>(src[a]) + first * esize[a],
                                 static_cast<uint32_t>(m * kSellRows * esize[a]), b);
                }
                issued++;
                ps++;
                return;
            }
            pc += nw;
            ps = 0;
        }
    }
    // after a failed wait: the copies still in flight land before the CTA can exit
    __device__ void drain(int consumed) {
        for (int k = consumed; k < issued; k++) stg_wait(bar + k % STAGES, (k / STAGES) & 1);
    }
};

// What a staged FP64 SpMV computes: the CG's A p (with p.Ap and the step size alpha =
// rr / p.Ap, as k_cg_spmv_dot), or the mixed solves' true residual r = b - A x' after a
// reliable update folded the FP32 correction into x' (with r.r and the update's decisions).
enum StagedKind { kStagedCgAp = 0, kStagedTrueResidual = 1 };

// k_cg_spmv_dot with the staged stream.  A lane sums its row from the stages in
// ascending column order with one accumulator (the order of row64), so the row sums are
// those of the per-chunk kernel.
template <int SLICE, int STAGES, int MINB, int KIND>
__global__ void __launch_bounds__(kStgThreads, MINB) k_cg_spmv_dot_staged(CgOperands o, cudaGraphConditionalHandle h,
                                                                          int use_cond) {
    extern __shared__ __align__(128) unsigned char stg_sm[];
    __shared__ BlockTicket tk;
    if (KIND == kStagedCgAp) {
        if (cg_done(o.S)) return;
    } else if (o.S->converged || o.S->aborted || o.S->stalled || !o.S->do_update) {
        return;
    }
    ticket_init(tk);
    using Ring = StageRing<SLICE, STAGES, 2>;
    constexpr int kStageBytes = Ring::kEntries * 12;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int gw = blockIdx.x * kStgWarps + w, nw = gridDim.x * kStgWarps;
    Ring R;
    R.src[0] = o.val;  // values first: 8-byte entries keep both arrays 16-byte aligned
    R.esize[0] = 8;
    R.src[1] = o.col;
    R.esize[1] = 4;
    R.init(stg_sm + static_cast<size_t>(w) * STAGES * kStageBytes,
           reinterpret_cast<uint64_t*>(stg_sm + static_cast<size_t>(kStgWarps) * STAGES * kStageBytes) + w * STAGES,
           gw);
    for (int k = 0; k < STAGES; k++) R.issue(o, nw);
    // the gathered vector: p, or the folded solution x' (the buffer the update writes)
    const double* __restrict__ p = KIND == kStagedCgAp ? o.p : ((o.S->updates & 1) != 0 ? o.x : o.x2);
    double v = 0.0;
    int item = 0;
    bool ok = true;
    for (int c = gw; c < o.nchunks && ok; c += nw) {
        const int i = kSellRows * c + lane;
        const int L = o.len[i];
        const int width = o.chunk[c] / kSellRows;
        double acc = 0.0;
        for (int k0 = 0; k0 < width; k0 += SLICE, item++) {
            if (!stg_wait(R.bar + item % STAGES, (item / STAGES) & 1)) {
                if (lane == 0 && o.status) atomicOr(&const_cast<DevStatus*>(o.status)->flags, kStatusWaitTimeout);
                R.drain(item);
                ok = false;
                break;
            }
            // the lane's entries of this slice into registers, then the stage is refilled
            // at once: the copy then overlaps this slice's gathers and multiply-adds
            const int m = min(SLICE, L - k0);
            const int32_t* sc = reinterpret_cast<const int32_t*>(R.stage(item, 1));
            const double* sv = reinterpret_cast<const double*>(R.stage(item, 0));
            int cc[SLICE];
            double av[SLICE];
#pragma unroll
            for (int t = 0; t < SLICE; t++) {
                cc[t] = t < m ? sc[t * kSellRows + lane] : 0;
                av[t] = t < m ? sv[t * kSellRows + lane] : 0.0;
            }
            // the values must have arrived before the copy may overwrite the stage
#pragma unroll
            for (int t = 0; t < SLICE; t++) asm volatile("" ::"r"(cc[t]), "d"(av[t]));
            __syncwarp();
            if (lane == 0) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            R.issue(o, nw);
            double xv[SLICE];
#pragma unroll
            for (int t = 0; t < SLICE; t++) xv[t] = t < m ? __ldg(p + cc[t]) : 0.0;
#pragma unroll
            for (int t = 0; t < SLICE; t++)
                if (t < m) acc = fma(av[t], xv[t], acc);
        }
        if (!ok) break;
        if (i < o.n) {
            if (KIND == kStagedCgAp) {
                o.Ap[i] = acc;
                v += p[i] * acc;
            } else {
                const double ri = o.b[i] - acc;
                o.r32[i] = __double2float_rn(ri);
                v += ri * ri;
            }
        }
    }
    double tot[3];
    if (grid_sum(v, 0.0, 0.0, o.partials, o.tickets, &o.S->counter, tk, tot)) {
        CgScalars* S = o.S;
        S->counter = 0;
        if (KIND == kStagedCgAp) {
            S->pAp = tot[0];
            S->alpha = S->rr / tot[0];
        } else {
            true_residual_done(S, tot[0], h, use_cond);
        }
        if (o.status && (o.status->flags & kStatusWaitTimeout)) S->aborted = 1;
    }
}

// The reliable update's first half: x' = x + d in FP64, into the other solution buffer
// (the staged true-residual SpMV then gathers x').
__global__ void __launch_bounds__(kBlock) k_mx_fold(CgOperands o) {
    if (o.S->converged || o.S->aborted || o.S->stalled || !o.S->do_update) return;
    const bool odd = (o.S->updates & 1) != 0;
    const double* __restrict__ xc = odd ? o.x2 : o.x;
    double* __restrict__ xn = odd ? o.x : o.x2;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < o.n; i += gridDim.x * blockDim.x)
        xn[i] = xc[i] + static_cast<double>(o.d32[i]);
}

// The staged FP64 SpMV: 8-entry slices, two stages per warp, three blocks of eight warps
// per SM (a sweep over slices of 4-32 entries, 2-4 stages and 1-6 blocks per SM measured
// 57 us at 340k particles against 63 us for the per-chunk kernel; the staged FP32 SpMV
// of the preconditioned solve measured no faster than k_pmx_spmv and is not used).
constexpr int kStgSlice64 = 8, kStgStages64 = 2, kStgBlocks64 = 3;
constexpr size_t kStgSmem64 = static_cast<size_t>(kStgWarps) * kStgStages64 * (kStgSlice64 * kSellRows * 12 + 8);

// blocks per SM of the staged kernel (occupancy with its shared memory), set by
// cg_prepare_device before any launch or capture
int g_stg_per_sm64 = 1;

// the FP64 CG's SpMV (Ap = A p, p.Ap, alpha): staged when the handle gives an SM count
void launch_cg_spmv(const CgOperands& o, cudaStream_t s) {
    if (o.grid_staged > 0) {
        const int cap = o.grid_staged * g_stg_per_sm64;
        const int need = (o.nchunks + kStgWarps - 1) / kStgWarps;
        const int g = need < cap ? (need > 0 ? need : 1) : cap;
        k_cg_spmv_dot_staged<kStgSlice64, kStgStages64, kStgBlocks64, kStagedCgAp>
            <<<g, kStgThreads, kStgSmem64, s>>>(o, 0, 0);
        return;
    }
    k_cg_spmv_dot<<<o.grid_spmv, kBlock, 0, s>>>(o);
}

// A reliable update's true residual: the fold x' = x + d and the staged FP64 SpMV
// r = b - A x' (about 50 us at 340k), or, without an SM count, one per-chunk kernel that
// gathers x + d on the fly.
void launch_mx_true(const CgOperands& o, cudaGraphConditionalHandle h, int use_cond, cudaStream_t s) {
    if (o.grid_staged > 0) {
        const int cap = o.grid_staged * g_stg_per_sm64;
        const int need = (o.nchunks + kStgWarps - 1) / kStgWarps;
        const int g = need < cap ? (need > 0 ? need : 1) : cap;
        k_mx_fold<<<o.grid_vec, kBlock, 0, s>>>(o);
        k_cg_spmv_dot_staged<kStgSlice64, kStgStages64, kStgBlocks64, kStagedTrueResidual>
            <<<g, kStgThreads, kStgSmem64, s>>>(o, h, use_cond);
        return;
    }
    k_mx_true<<<o.grid_spmv, kBlock, 0, s>>>(o, h, use_cond);
}

int mx_true_launches(const CgOperands& o) { return o.grid_staged > 0 ? 2 : 1; }

// the preconditioned FP32 SpMV (w = A u, three dot products)
void launch_pmx_spmv(const CgOperands& o, int mode, cudaGraphConditionalHandle h, cudaGraphConditionalHandle h_true,
                     int use_cond, cudaStream_t s, bool pdl) {
    if (pdl)
        launch_pdl(k_pmx_spmv, o.grid_spmv, kBlock, 0, s, o, mode, h, h_true, use_cond);
    else
        k_pmx_spmv<<<o.grid_spmv, kBlock, 0, s>>>(o, mode, h, h_true, use_cond);
}

// After the fallback: report it in the primary scalars.
__global__ void k_fb_merge(CgScalars* S, const CgScalars* F) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (S->converged || S->aborted) return;
    S->fallback = 1;
    S->fb_iter = F->iter;
    S->converged = F->converged;
    S->iter += F->iter;
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
        S->do_update = 0;
        S->updates = 0;
        S->stalled = 0;
        S->fallback = 0;
        S->fb_iter = 0;
    }
}

// ------------------------------------------------ persistent preconditioned solve
// The whole preconditioned iteration loop in one cooperative launch: every phase of an
// iteration (vector updates + level-1 restriction, each cycle level, the dense coarsest
// solve, the prolongation, the SpMV with its dot products, the reliable update) runs
// grid-stride over all resident blocks, and phases are separated by a grid barrier
// instead of a kernel boundary.  The barrier spins with a clock bound: a wait that
// exceeds it sets the error word and every block leaves the loop at its next barrier.
struct GridSync {
    unsigned* count;
    unsigned* gen;
    int32_t* err;
    const WaitLimits* limits;  // null: kDefaultBarrierClocks
};

// Two-level arrival: blocks count in groups of kBarrierGroup, the last block of a group
// counts at the top, and the last group releases everyone by advancing the generation.
// `count` holds one counter per group plus the top one (all zero between barriers).
constexpr int kBarrierGroup = 16;

__device__ __forceinline__ bool grid_barrier(const GridSync& g, unsigned& gen, long long limit) {
    __shared__ int err_s;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned target = gen + 1;
        const int G = static_cast<int>(gridDim.x);
        const int NG = (G + kBarrierGroup - 1) / kBarrierGroup;
        const int grp = static_cast<int>(blockIdx.x) / kBarrierGroup;
        const int gsize = min(kBarrierGroup, G - grp * kBarrierGroup);
        __threadfence();
        if (atomicAdd(g.count + grp, 1u) == static_cast<unsigned>(gsize - 1)) {
            atomicExch(g.count + grp, 0u);
            __threadfence();
            if (atomicAdd(g.count + NG, 1u) == static_cast<unsigned>(NG - 1)) {
                atomicExch(g.count + NG, 0u);
                __threadfence();
                atomicExch(g.gen, target);
            }
        }
        const long long t0 = clock64();
        while (*reinterpret_cast<volatile unsigned*>(g.gen) != target) {
            if (clock64() - t0 >= limit) {
                atomicExch(g.err, 1);
                break;
            }
        }
        __threadfence();
        err_s = *reinterpret_cast<volatile int32_t*>(g.err);
    }
    gen++;
    __syncthreads();
    return err_s == 0;
}

struct PersistentState {
    unsigned gen;
    long long limit;  // barrier wait bound in SM clocks
    int gtid, nthreads, gwarp, nwarps, lane;
};

// block sums of three values (lanes park values, warp 0 adds), then one partial per block
// and, after a barrier, the same fixed-order total in every block (thread 0 valid)
__device__ __noinline__ bool persistent_sum3(double a, double b, double c, const CgOperands& o, const GridSync& g,
                                PersistentState& P, double* red, double* out) {
    red[threadIdx.x] = a;
    red[kBlock + threadIdx.x] = b;
    red[2 * kBlock + threadIdx.x] = c;
    __syncthreads();
    if (threadIdx.x < 32) {
        double s0 = 0.0, s1 = 0.0, s2 = 0.0;
        for (int w = 0; w < kBlock / 32; w++) {
            s0 += red[32 * w + threadIdx.x];
            s1 += red[kBlock + 32 * w + threadIdx.x];
            s2 += red[2 * kBlock + 32 * w + threadIdx.x];
        }
        s0 = warp_sum(s0);
        s1 = warp_sum(s1);
        s2 = warp_sum(s2);
        if (threadIdx.x == 0) {
            o.partials[blockIdx.x] = s0;
            o.partials[gridDim.x + blockIdx.x] = s1;
            o.partials[2 * gridDim.x + blockIdx.x] = s2;
        }
    }
    if (!grid_barrier(g, P.gen, P.limit)) return false;
    if (threadIdx.x < 32) {
        double x = 0.0, y = 0.0, z = 0.0;
        for (int k = threadIdx.x; k < static_cast<int>(gridDim.x); k += 32) {
            x += __ldcg(o.partials + k);
            y += __ldcg(o.partials + gridDim.x + k);
            z += __ldcg(o.partials + 2 * gridDim.x + k);
        }
        x = warp_sum(x);
        y = warp_sum(y);
        z = warp_sum(z);
        if (threadIdx.x == 0) {
            out[0] = x;
            out[1] = y;
            out[2] = z;
        }
    }
    __syncthreads();
    return true;
}

// u = M r; with `axpy` the iteration's vector updates run in the restriction
__device__ __noinline__ bool persistent_cycle(const CgOperands& o, const MgHierarchy& mg, const GridSync& g,
                                 PersistentState& P, bool axpy, float alpha, float beta) {
    const MgLevel& L1 = mg.lv[1];
    const int nact = *mg.n_active;
    for (int a = P.gwarp; a < nact; a += P.nwarps) {
        const int c = mg.active[a];
        const int end = mg.cell_start[c + 1];
        float sum = 0.0f;
        for (int i = mg.cell_start[c] + P.lane; i < end; i += 32) {
            float ri = o.r32[i];
            if (axpy) {
                const float si = fmaf(beta, o.s32[i], o.w32[i]);
                const float pi = fmaf(beta, o.p32[i], o.u32[i]);
                ri = fmaf(-alpha, si, ri);
                o.s32[i] = si;
                o.p32[i] = pi;
                o.d32[i] = fmaf(alpha, pi, o.d32[i]);
                o.r32[i] = ri;
            }
            sum += ri;
        }
        for (int k = 16; k > 0; k >>= 1) sum += __shfl_down_sync(kFull, sum, k);
        if (P.lane == 0) L1.r[c] = sum;
    }
    if (!grid_barrier(g, P.gen, P.limit)) return false;
    for (int l = 1; l < mg.levels; l++) {
        const MgLevel& f = mg.lv[l];
        const MgLevel& cl = mg.lv[l + 1];
        for (int I = P.gtid; I < cl.cells; I += P.nthreads)
            cl.r[I] = child_residuals(f.nx, f.nz, f.cells, f.k32, f.dinv, f.r, I / cl.nz, I - (I / cl.nz) * cl.nz);
        if (!grid_barrier(g, P.gen, P.limit)) return false;
    }
    {
        const MgLevel& Lc = mg.lv[mg.levels];
        const int m = Lc.cells;
        for (int row = P.gwarp; row < m; row += P.nwarps) {
            float v = 0.0f;
            for (int k = P.lane; k < m; k += 32) v += mg.dense[row * m + k] * Lc.r[k];
            for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(kFull, v, off);
            if (P.lane == 0) Lc.e[row] = v;
        }
        if (!grid_barrier(g, P.gen, P.limit)) return false;
    }
    for (int l = mg.levels - 1; l >= 2; l--) {
        const MgLevel& f = mg.lv[l];
        for (int ch = P.gtid; ch < f.cells; ch += P.nthreads)
            f.e[ch] = smoothed_correction(f.nx, f.nz, f.cells, f.k32, f.dinv, f.r, mg.lv[l + 1].nz, mg.lv[l + 1].e, ch);
        if (!grid_barrier(g, P.gen, P.limit)) return false;
    }
    if (mg.levels > 1) {
        const MgLevel& c2 = mg.lv[2];
        for (int a = P.gwarp; a < nact; a += P.nwarps) {
            const int c = mg.active[a];
            const int end = mg.cell_start[c + 1];
            const float e = smoothed_correction(L1.nx, L1.nz, L1.cells, L1.k32, L1.dinv, L1.r, c2.nz, c2.e, c);
            for (int i = mg.cell_start[c] + P.lane; i < end; i += 32) {
                const float d = mg.dinv0[i];
                const float scl = mg.scale ? mg.scale[i] : 1.0f;
                o.u32[i] = d != 0.0f ? scl * d * o.r32[i] + e : 0.0f;
            }
        }
    } else {
        for (int c = P.gwarp; c < L1.cells; c += P.nwarps) {
            const int end = mg.cell_start[c + 1];
            const float e = L1.e[c];
            for (int i = mg.cell_start[c] + P.lane; i < end; i += 32) {
                const float d = mg.dinv0[i];
                const float scl = mg.scale ? mg.scale[i] : 1.0f;
                o.u32[i] = d != 0.0f ? scl * d * o.r32[i] + e : 0.0f;
            }
        }
    }
    return grid_barrier(g, P.gen, P.limit);
}

// w = A u; gamma = r.u, delta = w.u, rho = r.r (FP64), the same in every block
__device__ __noinline__ bool persistent_spmv(const CgOperands& o, const GridSync& g, PersistentState& P, double* red,
                                double* sums) {
    double vg = 0.0, vd = 0.0, vr = 0.0;
    for (int c = P.gwarp; c < o.nchunks; c += P.nwarps) {
        const int i = kSellRows * c + P.lane;
        const int L = o.len[i];
        const float wi = row32(o, sell_index(o.off[c], P.lane, 0), L, o.u32);
        if (i < o.n) {
            const double ri = o.r32[i], ui = o.u32[i];
            o.w32[i] = wi;
            vg += ri * ui;
            vd += static_cast<double>(wi) * ui;
            vr += ri * ri;
        }
    }
    return persistent_sum3(vg, vd, vr, o, g, P, red, sums);
}

// x += d (FP64), d = 0; then r = b - A x with the FP64 matrix into r32; returns r.r
__device__ __noinline__ bool persistent_true(const CgOperands& o, const GridSync& g, PersistentState& P, double* red,
                                double* sums) {
    for (int i = P.gtid; i < o.n; i += P.nthreads) {
        o.x[i] += static_cast<double>(o.d32[i]);
        o.d32[i] = 0.0f;
    }
    if (!grid_barrier(g, P.gen, P.limit)) return false;
    double v = 0.0;
    for (int c = P.gwarp; c < o.nchunks; c += P.nwarps) {
        const int i = kSellRows * c + P.lane;
        const int L = o.len[i];
        const double* x = o.x;
        const double ax = row64(o, sell_index(o.off[c], P.lane, 0), L, [&](int j) { return x[j]; });
        if (i < o.n) {
            const double ri = o.b[i] - ax;
            o.r32[i] = static_cast<float>(ri);
            v += ri * ri;
        }
    }
    return persistent_sum3(v, 0.0, 0.0, o, g, P, red, sums);
}

__global__ void __launch_bounds__(kBlock, 4) k_pcg_persistent(CgOperands o, MgHierarchy mg, GridSync g) {
    __shared__ double red[3 * kBlock];
    __shared__ double sums[3];
    __shared__ unsigned gen0;
    CgScalars* S = o.S;
    if (S->converged || S->aborted || S->stalled) return;
    if (threadIdx.x == 0) gen0 = *reinterpret_cast<volatile unsigned*>(g.gen);
    __syncthreads();
    PersistentState P;
    P.gen = gen0;
    P.limit = g.limits ? g.limits->barrier_clocks : kDefaultBarrierClocks;
    P.gtid = static_cast<int>(blockIdx.x * blockDim.x + threadIdx.x);
    P.nthreads = static_cast<int>(gridDim.x * blockDim.x);
    P.gwarp = P.gtid >> 5;
    P.nwarps = P.nthreads >> 5;
    P.lane = threadIdx.x & 31;
    double alpha = S->alpha, beta = S->beta, gam_old = S->rr;
    double rr_upd = S->rr_upd, prev_true = S->prev_true_rr, rho = S->rr_new;
    const double thr = S->thr, delta2 = S->delta2;
    int iter = S->iter, updates = S->updates;
    const int max_iter = S->max_iter;
    bool conv = false, stalled = false, ok = true;
    while (iter < max_iter) {
        ok = persistent_cycle(o, mg, g, P, true, static_cast<float>(alpha), static_cast<float>(beta));
        if (!ok) break;
        ok = persistent_spmv(o, g, P, red, sums);
        if (!ok) break;
        double gam = sums[0], del = sums[1];
        rho = sums[2];
        if (rho < delta2 * rr_upd || rho < thr) {
            ok = persistent_true(o, g, P, red, sums);
            if (!ok) break;
            const double tr = sums[0];
            updates++;
            rr_upd = tr;
            rho = tr;
            if (tr < thr) {
                conv = true;
                iter++;
                break;
            }
            if (tr > 0.25 * prev_true) {
                stalled = true;
                break;
            }
            prev_true = tr;
            ok = persistent_cycle(o, mg, g, P, false, 0.0f, 0.0f) && persistent_spmv(o, g, P, red, sums);
            if (!ok) break;
            gam = sums[0];
            del = sums[1];
            rho = sums[2];
        }
        beta = gam / gam_old;
        alpha = gam / (del - beta * gam / alpha);
        gam_old = gam;
        iter++;
        if (!(isfinite(alpha) && isfinite(beta) && alpha != 0.0)) {
            stalled = true;
            break;
        }
    }
    // the pending FP32 correction into x (no reader follows inside this kernel)
    for (int i = P.gtid; i < o.n; i += P.nthreads) {
        o.x[i] += static_cast<double>(o.d32[i]);
        o.d32[i] = 0.0f;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        S->iter = iter;
        S->updates = updates;
        S->converged = conv ? 1 : 0;
        S->stalled = (stalled || !ok) ? 1 : 0;
        S->rr_new = rho;
        S->rr_upd = rr_upd;
        S->alpha = alpha;
        S->beta = beta;
        S->rr = gam_old;
        S->do_update = 1;  // x is current: nothing left to fold
    }
}

bool is_pcg(int solver) { return solver == MPS_SOLVER_MIXED_MG || solver == MPS_SOLVER_LEARNED; }

void cg64_body(const CgOperands& ops, cudaGraphConditionalHandle h, int use_cond, cudaStream_t s) {
    launch_cg_spmv(ops, s);
    k_cg_update<<<ops.grid_vec, kBlock, 0, s>>>(ops, h, use_cond);
    k_cg_pupdate<<<ops.grid_vec, kBlock, 0, s>>>(ops);
}

void reliable_kernels(int solver, const CgOperands& ops, const MgHierarchy* mg,
                      cudaGraphConditionalHandle h, int use_cond, cudaStream_t s) {
    launch_mx_true(ops, h, use_cond, s);
    if (is_pcg(solver)) {
        mg_apply(*mg, ops.S, 2, ops.r32, ops.u32, s);
        launch_pmx_spmv(ops, 2, h, 0, use_cond, s, false);
    } else {
        k_mx_spmv<<<ops.grid_spmv, kBlock, 0, s>>>(ops, 2, h, 0, use_cond);
    }
}

void body_kernels(int solver, const CgOperands& ops, const MgHierarchy* mg,
                  cudaGraphConditionalHandle h, cudaGraphConditionalHandle h_true, int use_cond,
                  bool with_true, cudaStream_t s) {
    const int gv = ops.grid_vec, gs = ops.grid_spmv;
    if (solver == MPS_SOLVER_CG64) {
        cg64_body(ops, h, use_cond, s);
        return;
    }
    if (is_pcg(solver)) {
        mg_apply(*mg, ops.S, 1, ops.r32, ops.u32, s, &ops);  // vector updates + u = M r
        launch_pmx_spmv(ops, 1, h, h_true, use_cond, s, true);
    } else {
        k_mx_axpy<<<gv, kBlock, 0, s>>>(ops);
        k_mx_spmv<<<gs, kBlock, 0, s>>>(ops, 1, h, h_true, use_cond);
    }
    if (with_true) reliable_kernels(solver, ops, mg, h, use_cond, s);
}

// The learned start in two parts: r0 of the previous pressure and the per-particle
// feature quantities (no use of the hierarchy), then the first preconditioned step,
// the features, the network and the warm start.
void learned_prep_head(const LearnedOps& L, const CgOperands& o, CgScalars* S, cudaStream_t s) {
    CgOperands p = o;
    p.S = S;
    k_mx_init<<<o.grid_spmv, kBlock, 0, s>>>(p, 0, 0);  // r0 = b - A x0 in FP64, into r32
    launch_learned_q(L, p, S, s);
}

void learned_prep_tail(const LearnedOps& L, const CgOperands& o, const MgHierarchy& mg, CgScalars* S,
                       bool infer, cudaStream_t s) {
    CgOperands p = o;
    p.S = S;
    MgHierarchy plain = mg;
    plain.scale = nullptr;
    mg_apply(plain, S, 0, o.r32, o.u32, s);
    launch_pmx_spmv(p, 0, 0, 0, 0, s, false);  // alpha0 = r0.u0 / (A u0).u0
    launch_learned_feature_rows(L, p, S, s);
    if (infer) {
        launch_mlp_infer(L.packed, L.feat, L.n, L.sigma, L.out, L.error, s, L.limits);
        launch_learned_apply(L, p, S, s);
    }
}

// With `fk` (graph capture), the coarse half of the multigrid setup runs on a side
// stream beside the initial residual (and the learned start's first kernels), joining
// before the first use of the hierarchy.  The two branches share no buffers.
void init_kernels(int solver, const CgOperands& ops, const MgHierarchy* mg,
                  cudaGraphConditionalHandle h, int use_cond, cudaStream_t s,
                  const LearnedRun* lrn, const SetupFork* fk = nullptr) {
    const int gs = ops.grid_spmv;
    if (solver == MPS_SOLVER_CG64) {
        k_cg_init<<<gs, kBlock, 0, s>>>(ops, h, use_cond, nullptr);
        return;
    }
    const bool pcg = is_pcg(solver);
    const bool forked = pcg && fk != nullptr;
    if (pcg) {
        mg_setup_level1(*mg, ops, s);
        if (forked) {
            cudaEventRecord(fk->fork, s);
            cudaStreamWaitEvent(fk->side, fk->fork, 0);
            mg_setup_coarse(*mg, fk->side);
            cudaEventRecord(fk->join, fk->side);
        } else {
            mg_setup_coarse(*mg, s);
        }
    }
    if (solver == MPS_SOLVER_LEARNED && lrn) {
        k_cg_configure<<<1, 32, 0, s>>>(lrn->S, 0.0, MPS_CRIT_RHS, 1, 0.0);
        learned_prep_head(*lrn->L, ops, lrn->S, s);
        if (forked) cudaStreamWaitEvent(s, fk->join, 0);
        learned_prep_tail(*lrn->L, ops, *mg, lrn->S, true, s);
        k_mx_init<<<gs, kBlock, 0, s>>>(ops, h, use_cond);
    } else {
        k_mx_init<<<gs, kBlock, 0, s>>>(ops, h, use_cond);
        if (forked) cudaStreamWaitEvent(s, fk->join, 0);
    }
    if (pcg) {
        mg_apply(*mg, ops.S, 0, ops.r32, ops.u32, s);
        launch_pmx_spmv(ops, 0, h, 0, use_cond, s, false);
    } else {
        k_mx_spmv<<<gs, kBlock, 0, s>>>(ops, 0, h, 0, use_cond);
    }
}

}  // namespace

int cg_grid_vec(int64_t n) { return grid_for(n); }
int cg_grid_spmv(int64_t n) { return grid_for(sell_chunks(n) * 32); }

cudaError_t cg_prepare_device() {
    auto k = k_cg_spmv_dot_staged<kStgSlice64, kStgStages64, kStgBlocks64, kStagedCgAp>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kStgSmem64));
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_cg_spmv_dot_staged<kStgSlice64, kStgStages64, kStgBlocks64, kStagedTrueResidual>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kStgSmem64));
    if (e != cudaSuccess) return e;
    int b = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k, kStgThreads, kStgSmem64);
    if (e != cudaSuccess) return e;
    g_stg_per_sm64 = b > 0 ? b : 1;
    return cudaSuccess;
}

int64_t cg_partials(int64_t n) {
    const int64_t g = cg_grid_vec(n) > cg_grid_spmv(n) ? cg_grid_vec(n) : cg_grid_spmv(n);
    return 3 * (g + (g + 31) / 32) + 64;
}

int64_t cg_tickets(int64_t n) {
    const int64_t g = cg_grid_vec(n) > cg_grid_spmv(n) ? cg_grid_vec(n) : cg_grid_spmv(n);
    return (g + 31) / 32 + 1;
}

void launch_cg_configure(CgScalars* S, double eps, int criterion, int max_iter, double delta2,
                         cudaStream_t s) {
    k_cg_configure<<<1, 32, 0, s>>>(S, eps, criterion, max_iter, delta2);
}


void launch_spmv_only(int solver, const CgOperands& ops, cudaStream_t s) {
    if (solver == MPS_SOLVER_CG64)
        launch_cg_spmv(ops, s);
    else if (is_pcg(solver))
        launch_pmx_spmv(ops, 1, 0, 0, 0, s, false);
    else
        k_mx_spmv<<<ops.grid_spmv, kBlock, 0, s>>>(ops, 1, 0, 0, 0);
}

void learned_prep(const LearnedOps& L, const CgOperands& o, const MgHierarchy& mg, CgScalars* S,
                  bool infer, cudaStream_t s) {
    learned_prep_head(L, o, S, s);
    learned_prep_tail(L, o, mg, S, infer, s);
}

int learned_prep_launches(const MgHierarchy& mg, bool infer) {
    return 1 + mg_apply_launches(mg) + 1 + 2 + (infer ? 2 : 0);
}

int cg_kernels_per_iteration(int solver, const MgHierarchy* mg) {
    if (solver == MPS_SOLVER_CG64) return 3;
    return is_pcg(solver) && mg ? 1 + mg_apply_launches(*mg) : 2;
}

int cg_kernels_per_update(int solver, const MgHierarchy* mg, const CgOperands& ops) {
    if (solver == MPS_SOLVER_CG64) return 0;
    const int t = mx_true_launches(ops);
    return is_pcg(solver) && mg ? t + 1 + mg_apply_launches(*mg) : t + 1;
}

CgGraph::~CgGraph() {
    reset();
    if (fork_.fork) cudaEventDestroy(fork_.fork);
    if (fork_.join) cudaEventDestroy(fork_.join);
    if (fork_.side) cudaStreamDestroy(fork_.side);
}

void CgGraph::reset() {
    if (exec_) cudaGraphExecDestroy(exec_);
    if (graph_) cudaGraphDestroy(graph_);
    exec_ = nullptr;
    graph_ = nullptr;
    solver_ = -1;
    nested_ = false;
    persistent_ = false;
}

cudaError_t CgGraph::build(int solver, const CgOperands& ops, cudaStream_t s, const MgHierarchy* mg,
                           const CgOperands* fb, const LearnedRun* lrn) {
    if (is_pcg(solver) && (!mg || !fb)) return cudaErrorInvalidValue;
    if (solver == MPS_SOLVER_LEARNED && !lrn) return cudaErrorInvalidValue;
    if (solver != MPS_SOLVER_CG64) {
        // preferred: the reliable update under an IF node nested in the WHILE body
        if (build_impl(solver, ops, s, true, mg, fb, lrn) == cudaSuccess) return cudaSuccess;
        cudaGetLastError();
    }
    return build_impl(solver, ops, s, false, mg, fb, lrn);
}

namespace {
// The one node of a linear chain that has no successor.
cudaError_t sink_node(cudaGraph_t g, cudaGraphNode_t* out) {
    size_t nn = 0, ne = 0;
    cudaError_t e = cudaGraphGetNodes(g, nullptr, &nn);
    if (e != cudaSuccess) return e;
    std::vector<cudaGraphNode_t> nodes(nn);
    e = cudaGraphGetNodes(g, nodes.data(), &nn);
    if (e != cudaSuccess) return e;
    e = cudaGraphGetEdges(g, nullptr, nullptr, nullptr, &ne);
    if (e != cudaSuccess) return e;
    // edge data is requested too: programmatic (PDL) edges cannot be listed without it
    std::vector<cudaGraphNode_t> from(ne), to(ne);
    std::vector<cudaGraphEdgeData> data(ne);
    if (ne > 0) {
        e = cudaGraphGetEdges(g, from.data(), to.data(), data.data(), &ne);
        if (e != cudaSuccess) return e;
    }
    int found = 0;
    for (cudaGraphNode_t node : nodes) {
        bool has_succ = false;
        for (size_t k = 0; k < ne; k++) has_succ = has_succ || from[k] == node;
        if (!has_succ) {
            *out = node;
            found++;
        }
    }
    return found == 1 ? cudaSuccess : cudaErrorInvalidValue;
}

// Adds a WHILE node after `dep` (or as a root) and returns its body graph.
cudaError_t add_while(cudaGraph_t g, cudaGraphNode_t* dep, cudaGraphConditionalHandle h,
                      cudaGraphNode_t* node, cudaGraph_t* body) {
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaError_t e = cudaGraphAddNode(node, g, dep, nullptr, dep ? 1 : 0, &cp);
    if (e != cudaSuccess) return e;
    *body = cp.conditional.phGraph_out[0];
    return cudaSuccess;
}
}  // namespace

cudaError_t CgGraph::build_impl(int solver, const CgOperands& ops, cudaStream_t s, bool nested,
                                const MgHierarchy* mg, const CgOperands* fb, const LearnedRun* lrn) {
    reset();
    ops_ = ops;
    solver_ = solver;
    nested_ = nested;
    kpi_ = cg_kernels_per_iteration(solver, mg);
    kri_ = cg_kernels_per_update(solver, mg, ops);
    const int gv = ops.grid_vec, gs = ops.grid_spmv;
    cudaError_t e = cudaGraphCreate(&graph_, 0);
    if (e != cudaSuccess) return e;
    cudaGraphConditionalHandle h, h_fb = 0;
    e = cudaGraphConditionalHandleCreate(&h, graph_, 0, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) return e;
    // the mixed-precision solvers end with the plain FP64 CG when they stall
    const bool with_fb = solver != MPS_SOLVER_CG64 && fb != nullptr;
    if (with_fb) {
        e = cudaGraphConditionalHandleCreate(&h_fb, graph_, 0, cudaGraphCondAssignDefault);
        if (e != cudaSuccess) return e;
    }
    cudaGraph_t captured = nullptr;

    // init chain (the multigrid's coarse setup on a side branch)
    if (!fork_.side) {
        e = cudaStreamCreateWithFlags(&fork_.side, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&fork_.fork, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&fork_.join, cudaEventDisableTiming);
        if (e != cudaSuccess) return e;
    }
    e = cudaStreamBeginCaptureToGraph(s, graph_, nullptr, nullptr, 0,
                                      cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    init_kernels(solver, ops, mg, h, 1, s, lrn, &fork_);
    e = cudaStreamEndCapture(s, &captured);
    if (e != cudaSuccess) return e;
    cudaGraphNode_t init_node;
    e = sink_node(graph_, &init_node);
    if (e != cudaSuccess) return e;

    // while (cond) { body }
    cudaGraphNode_t while_node;
    cudaGraph_t body;
    e = add_while(graph_, &init_node, h, &while_node, &body);
    if (e != cudaSuccess) return e;
    cudaGraphConditionalHandle h_true = 0;
    if (nested) {
        e = cudaGraphConditionalHandleCreate(&h_true, body, 0, 0);
        if (e != cudaSuccess) return e;
    }
    e = cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    body_kernels(solver, ops, mg, h, h_true, 1, !nested, s);
    e = cudaStreamEndCapture(s, &captured);
    if (e != cudaSuccess) return e;

    if (nested) {
        // if (reliable update due) { true residual; [u = M r]; w = A u } after the SpMV
        cudaGraphNode_t last;
        e = sink_node(body, &last);
        if (e != cudaSuccess) return e;
        cudaGraphNodeParams ip = {};
        ip.type = cudaGraphNodeTypeConditional;
        ip.conditional.handle = h_true;
        ip.conditional.type = cudaGraphCondTypeIf;
        ip.conditional.size = 1;
        cudaGraphNode_t if_node;
        e = cudaGraphAddNode(&if_node, body, &last, nullptr, 1, &ip);
        if (e != cudaSuccess) return e;
        cudaGraph_t if_body = ip.conditional.phGraph_out[0];
        e = cudaStreamBeginCaptureToGraph(s, if_body, nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return e;
        reliable_kernels(solver, ops, mg, h, 1, s);
        e = cudaStreamEndCapture(s, &captured);
        if (e != cudaSuccess) return e;
    }

    // tail: the solution into x, [plain FP64 CG fallback], the true residual
    e = cudaStreamBeginCaptureToGraph(s, graph_, &while_node, nullptr, 1,
                                      cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    if (solver != MPS_SOLVER_CG64) k_mx_finish<<<gv, kBlock, 0, s>>>(ops);
    if (with_fb) {
        k_cg_init<<<gs, kBlock, 0, s>>>(*fb, h_fb, 1, ops.S);
    } else {
        k_true_residual<<<gs, kBlock, 0, s>>>(ops, solver != MPS_SOLVER_CG64 ? 1 : 0);
    }
    e = cudaStreamEndCapture(s, &captured);
    if (e != cudaSuccess) return e;
    if (with_fb) {
        cudaGraphNode_t fb_init;
        e = sink_node(graph_, &fb_init);
        if (e != cudaSuccess) return e;
        cudaGraphNode_t fb_while;
        cudaGraph_t fb_body;
        e = add_while(graph_, &fb_init, h_fb, &fb_while, &fb_body);
        if (e != cudaSuccess) return e;
        e = cudaStreamBeginCaptureToGraph(s, fb_body, nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return e;
        cg64_body(*fb, h_fb, 1, s);
        e = cudaStreamEndCapture(s, &captured);
        if (e != cudaSuccess) return e;
        e = cudaStreamBeginCaptureToGraph(s, graph_, &fb_while, nullptr, 1,
                                          cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return e;
        k_fb_merge<<<1, 32, 0, s>>>(ops.S, fb->S);
        k_true_residual<<<gs, kBlock, 0, s>>>(ops, 1);
        e = cudaStreamEndCapture(s, &captured);
        if (e != cudaSuccess) return e;
    }

    e = cudaGraphInstantiate(&exec_, graph_, 0);
    if (e != cudaSuccess) {
        exec_ = nullptr;
        return e;
    }
    return cudaSuccess;
}

cudaError_t CgGraph::build_persistent(int solver, const CgOperands& ops, cudaStream_t s,
                                      const MgHierarchy* mg, const CgOperands* fb, const LearnedRun* lrn,
                                      const PersistentSync& ps) {
    reset();
    if (!is_pcg(solver) || !mg || !fb || ps.blocks <= 0) return cudaErrorInvalidValue;
    ops_ = ops;
    solver_ = solver;
    nested_ = false;
    persistent_ = true;
    kpi_ = 0;
    kri_ = 0;
    const int gs = ops.grid_spmv;
    cudaError_t e = cudaGraphCreate(&graph_, 0);
    if (e != cudaSuccess) return e;
    cudaGraphConditionalHandle h_fb;
    e = cudaGraphConditionalHandleCreate(&h_fb, graph_, 0, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) return e;
    cudaGraph_t captured = nullptr;
    e = cudaStreamBeginCaptureToGraph(s, graph_, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    init_kernels(solver, ops, mg, 0, 0, s, lrn);
    cudaMemsetAsync(ps.err, 0, sizeof(int32_t), s);
    cudaMemsetAsync(ps.count, 0, sizeof(unsigned) * kPersistentCounters, s);  // a timed-out barrier leaves them non-zero
    {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(ps.blocks);
        cfg.blockDim = dim3(kBlock);
        cfg.dynamicSmemBytes = 0;
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        GridSync g{ps.count, ps.gen, ps.err, ps.limits};
        cudaLaunchKernelEx(&cfg, k_pcg_persistent, ops, *mg, g);
    }
    k_cg_init<<<gs, kBlock, 0, s>>>(*fb, h_fb, 1, ops.S);
    e = cudaStreamEndCapture(s, &captured);
    if (e != cudaSuccess) return e;
    cudaGraphNode_t fb_init;
    e = sink_node(graph_, &fb_init);
    if (e != cudaSuccess) return e;
    cudaGraphNode_t fb_while;
    cudaGraph_t fb_body;
    e = add_while(graph_, &fb_init, h_fb, &fb_while, &fb_body);
    if (e != cudaSuccess) return e;
    e = cudaStreamBeginCaptureToGraph(s, fb_body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    cg64_body(*fb, h_fb, 1, s);
    e = cudaStreamEndCapture(s, &captured);
    if (e != cudaSuccess) return e;
    e = cudaStreamBeginCaptureToGraph(s, graph_, &fb_while, nullptr, 1, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    k_fb_merge<<<1, 32, 0, s>>>(ops.S, fb->S);
    k_true_residual<<<gs, kBlock, 0, s>>>(ops, 0);  // the persistent loop does not record it
    e = cudaStreamEndCapture(s, &captured);
    if (e != cudaSuccess) return e;
    e = cudaGraphInstantiate(&exec_, graph_, 0);
    if (e != cudaSuccess) {
        exec_ = nullptr;
        return e;
    }
    return cudaSuccess;
}

static_assert(kPersistentCounters * kBarrierGroup >= 8 * 1024, "barrier counters for 8192 blocks");

int persistent_blocks() {
    int dev = 0, sms = 0, coop = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg_persistent, kBlock, 0) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return per_sm * sms;
}

cudaError_t CgGraph::launch(cudaStream_t s) {
    if (!exec_) return cudaErrorInvalidValue;
    return cudaGraphLaunch(exec_, s);
}

namespace {
// Host loop: `chunk` iterations per batch, the scalars read back between batches.
cudaError_t host_loop(int solver, const CgOperands& ops, const MgHierarchy* mg, CgScalars* host_S,
                      int chunk, cudaStream_t s, int64_t* k) {
    const cudaGraphConditionalHandle none = 0;
    cudaError_t e = cudaGetLastError();
    for (;;) {
        if (e != cudaSuccess) return e;
        e = cudaMemcpyAsync(host_S, ops.S, sizeof(CgScalars), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return e;
        if (host_S->converged || host_S->aborted || host_S->stalled || host_S->iter >= host_S->max_iter)
            return cudaSuccess;
        for (int c = 0; c < chunk; c++) {
            body_kernels(solver, ops, mg, none, none, 0, true, s);
            // every kernel of the iteration and of the reliable update is launched
            *k += cg_kernels_per_iteration(solver, mg) + cg_kernels_per_update(solver, mg, ops);
        }
        e = cudaGetLastError();
    }
}
}  // namespace

cudaError_t cg_run_direct(int solver, const CgOperands& ops, CgScalars* host_S, int chunk,
                          cudaStream_t s, int64_t* launches, const MgHierarchy* mg,
                          const CgOperands* fb, const LearnedRun* lrn) {
    if (is_pcg(solver) && (!mg || !fb)) return cudaErrorInvalidValue;
    if (solver == MPS_SOLVER_LEARNED && !lrn) return cudaErrorInvalidValue;
    const int gv = ops.grid_vec, gs = ops.grid_spmv;
    const cudaGraphConditionalHandle none = 0;
    int64_t k = 0;
    init_kernels(solver, ops, mg, none, 0, s, lrn);
    k += solver == MPS_SOLVER_CG64 ? 1 : 2;
    if (is_pcg(solver)) k += mg_setup_launches(*mg) + mg_apply_launches(*mg);
    if (solver == MPS_SOLVER_LEARNED) k += 1 + learned_prep_launches(*mg, true);
    cudaError_t e = host_loop(solver, ops, mg, host_S, chunk, s, &k);
    if (e != cudaSuccess) return e;
    if (solver != MPS_SOLVER_CG64) {
        k_mx_finish<<<gv, kBlock, 0, s>>>(ops);
        k++;
    }
    if (solver != MPS_SOLVER_CG64 && fb) {
        k_cg_init<<<gs, kBlock, 0, s>>>(*fb, none, 0, ops.S);
        k++;
        e = host_loop(MPS_SOLVER_CG64, *fb, nullptr, host_S, chunk, s, &k);
        if (e != cudaSuccess) return e;
        k_fb_merge<<<1, 32, 0, s>>>(ops.S, fb->S);
        k++;
    }
    k_true_residual<<<gs, kBlock, 0, s>>>(ops, solver != MPS_SOLVER_CG64 ? 1 : 0);
    k++;
    if (launches) *launches = k;
    return cudaGetLastError();
}

}  // namespace mpsgb

// mg.cu - cell-aggregation multigrid preconditioner (setup and cycle kernels).
//
// Setup, once per solve (the matrix changes every step):
//   k_mg_bins    one pass over the FP64 SELL-32 matrix: for every active row the sums of
//                its entries per neighbouring cell (9 bins, FP64, in shared memory) and
//                the Jacobi factor omega_0 / a_ii;
//   k_mg_cells   level-1 operator: per cell, the bins of its particles in slot order
//                (deterministic, no atomics);
//   k_mg_coarsen Galerkin product of a 2 x 2 aggregation, FP64;
//   k_mg_dense   dense inverse of the coarsest level (banded L U and one substitution
//                per column, FP32 in shared memory, symmetrised).
// Cycle, once per iteration (FP32, reads L2-resident planes):
//   k_mg_axpy_restrict (the iteration's vector updates + level-1 restriction; after init
//   and after a reliable update k_mg_restrict0), k_mg_down_fused (the coarse residuals of
//   levels 2 .. bottom, tiles with halos in shared memory), k_mg_bottom (the coarsest
//   levels in one block, all in shared memory, __syncthreads between levels),
//   k_mg_up_fused (post-smoothing of levels bottom-1 .. 1 and the prolongation to the
//   particles, tiles again; k_mg_prolong0 when the bottom block covers level 1).
//   Hierarchies deeper than kMgFuseLevels levels above the bottom run the extra levels
//   with k_mg_down / k_mg_up, one kernel per level.
// A 16-block cluster kernel for levels 2 .. coarsest (cluster barriers between levels)
// was measured slower: about 4 us per level against well under 1 us per level for one
// block with __syncthreads, and the grid-wide kernels for the larger levels.
// Every kernel reads only what the previous kernel wrote, so the sequence captures into
// the solver's CUDA graph unchanged.
#include <algorithm>

#include "mg.cuh"

namespace mpsgb {

namespace {

__device__ __forceinline__ bool setup_failed(const DevStatus* st) {
    return st && (st->flags & (kStatusCellOverflow | kStatusDeviceCheck)) != 0;
}

// --------------------------------------------------------------------- setup
// Row i of the FP64 matrix binned by the cell offset of each column.  One warp per SELL
// chunk, one lane per row (coalesced matrix reads); the nine FP64 accumulators of a
// lane live in shared memory (one FP64 add per matrix entry).
__global__ void __launch_bounds__(kBlock) k_mg_bins(CgOperands o, const int32_t* cell_xz,
                                                    double* bins, float* dinv0, float omega,
                                                    DevStatus* status) {
    if (setup_failed(status)) return;
    __shared__ double acc[9 * kBlock];
    const int t = threadIdx.x;
    const int lane = t & 31;
    const int warp = static_cast<int>((blockIdx.x * blockDim.x + t) >> 5);
    const int nwarps = static_cast<int>((gridDim.x * blockDim.x) >> 5);
    for (int c = warp; c < o.nchunks; c += nwarps) {
        const int i = kSellRows * c + lane;
        if (i >= o.n) continue;
#pragma unroll
        for (int q = 0; q < 9; q++) acc[q * kBlock + t] = 0.0;
        const int ci = cell_xz[i];
        double aii = 0.0;
        bool bad = false;
        if (ci >= 0) {
            // four entries per step: their columns and values, then their cells, load
            // together; the bins then take them in row order (the same sums)
            constexpr int D = 4;
            const int L = o.len[i];
            int64_t at = sell_index(o.off[c], lane, 0);
            for (int k0 = 0; k0 < L; k0 += D, at += D * kSellRows) {
                int jj[D], cc[D];
                double aa[D];
#pragma unroll
                for (int u = 0; u < D; u++) {
                    jj[u] = k0 + u < L ? o.col[at + u * kSellRows] : 0;
                    aa[u] = k0 + u < L ? o.val[at + u * kSellRows] : 0.0;
                }
#pragma unroll
                for (int u = 0; u < D; u++) cc[u] = k0 + u < L ? cell_xz[jj[u]] : -1;
#pragma unroll
                for (int u = 0; u < D; u++) {
                    if (k0 + u >= L) continue;
                    if (jj[u] == i) aii = aa[u];
                    const int cj = cc[u];
                    const int dx = (cj >> 16) - (ci >> 16);
                    const int dz = (cj & 0xffff) - (ci & 0xffff);
                    if (cj < 0 || dx < -1 || dx > 1 || dz < -1 || dz > 1) {
                        bad = true;
                        continue;
                    }
                    acc[((dx + 1) * 3 + dz + 1) * kBlock + t] += aa[u];
                }
            }
        }
        if (bad) {
            atomicOr(&status->flags, kStatusDeviceCheck);
            status->check_index = i;
        }
        const bool active = ci >= 0 && aii < 0.0;
#pragma unroll
        for (int q = 0; q < 9; q++) bins[static_cast<int64_t>(q) * o.n + i] = active ? acc[q * kBlock + t] : 0.0;
        dinv0[i] = active ? omega / static_cast<float>(aii) : 0.0f;
    }
}

__device__ __forceinline__ void store_level(const MgLevel& L, int c, const double* k, float omega) {
#pragma unroll
    for (int q = 0; q < 9; q++) {
        L.k64[q * L.cells + c] = k[q];
        L.k32[q * L.cells + c] = static_cast<float>(k[q]);
    }
    L.dinv[c] = k[4] < 0.0 ? omega / static_cast<float>(k[4]) : 0.0f;
}

// Level-1 operator: per search cell, the bins of its rows in order.
__global__ void k_mg_cells(MgLevel L1, const int32_t* cell_start, const double* bins, int n, float omega,
                           const DevStatus* status, int32_t* active_flag) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= L1.cells) return;
    const int b = cell_start[c], e = cell_start[c + 1];
    active_flag[c] = (e > b && !setup_failed(status)) ? 1 : 0;
    if (setup_failed(status)) return;
    double k[9];
#pragma unroll
    for (int q = 0; q < 9; q++) k[q] = 0.0;
    for (int i = b; i < e; i++) {
#pragma unroll
        for (int q = 0; q < 9; q++) k[q] += bins[static_cast<int64_t>(q) * n + i];
    }
    store_level(L1, c, k, omega);
}

// The list of level-1 cells holding particles, in ascending cell order (neighbouring
// warps of the cycle kernels then work on neighbouring cells).
__global__ void k_mg_active(int cells, const int32_t* flag, const int32_t* pos, const int32_t* cell_start,
                            int32_t* active, int2* active_rows) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < cells && flag[c]) {
        active[pos[c]] = c;
        active_rows[pos[c]] = make_int2(cell_start[c], cell_start[c + 1]);
    }
}

// Galerkin product of the 2 x 2 aggregation of level f into level c (FP64).
__global__ void k_mg_coarsen(MgLevel f, MgLevel c, float omega, const DevStatus* status) {
    if (setup_failed(status)) return;
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= c.cells) return;
    const int X = I / c.nz, Z = I - (I / c.nz) * c.nz;
    double k[9];
#pragma unroll
    for (int q = 0; q < 9; q++) k[q] = 0.0;
    for (int a = 0; a < 2; a++) {
        const int cx = 2 * X + a;
        if (cx >= f.nx) continue;
        for (int b = 0; b < 2; b++) {
            const int cz = 2 * Z + b;
            if (cz >= f.nz) continue;
            const int child = cx * f.nz + cz;
            for (int dx = -1; dx <= 1; dx++) {
                const int nx = cx + dx;
                if (nx < 0 || nx >= f.nx) continue;
                for (int dz = -1; dz <= 1; dz++) {
                    const int nz = cz + dz;
                    if (nz < 0 || nz >= f.nz) continue;
                    const double v = f.k64[((dx + 1) * 3 + dz + 1) * f.cells + child];
                    const int DX = (nx >> 1) - X, DZ = (nz >> 1) - Z;
                    k[(DX + 1) * 3 + DZ + 1] += v;
                }
            }
        }
    }
    store_level(c, I, k, omega);
}

// Dense inverse of the coarsest level, FP32 in shared memory, symmetrised on output.  The
// 9-point operator is banded in the level's cell order c = X nz + Z (a row couples cells
// at most nz + 1 apart), so one warp factors it as L U inside the band without pivoting
// (the operator is negative definite on its non-empty cells; empty cells get a unit
// diagonal and a zero row and column in the inverse), and then thread c solves
// L U x = e_c for column c.  The substitutions need no barrier, and all threads run them
// in step: their reads of L and U are broadcasts, their columns sit in distinct banks.
__global__ void __launch_bounds__(kMgBottomThreads) k_mg_dense(MgLevel L, float* dense,
                                                               const DevStatus* status) {
    if (setup_failed(status)) return;
    extern __shared__ float A[];  // m * m operator, then its L U factors in place
    const int m = L.cells;
    float* W = A + m * m;         // m * m: column c of the inverse in W[i m + c]
    float* rd = W + m * m;        // m: 1 / U_ii
    const int b = min(L.nz + 1, m - 1);
    for (int idx = threadIdx.x; idx < m * m; idx += blockDim.x) A[idx] = 0.0f;
    __syncthreads();
    for (int c = threadIdx.x; c < m; c += blockDim.x) {
        const int X = c / L.nz, Z = c - (c / L.nz) * L.nz;
        if (L.k64[4 * m + c] == 0.0) {
            A[c * m + c] = 1.0f;
            continue;
        }
        for (int dx = -1; dx <= 1; dx++) {
            const int nx = X + dx;
            if (nx < 0 || nx >= L.nx) continue;
            for (int dz = -1; dz <= 1; dz++) {
                const int nz = Z + dz;
                if (nz < 0 || nz >= L.nz) continue;
                A[c * m + nx * L.nz + nz] = static_cast<float>(L.k64[((dx + 1) * 3 + dz + 1) * m + c]);
            }
        }
    }
    __syncthreads();
    if (threadIdx.x < 32) {  // banded L U (Doolittle), one warp
        const int lane = threadIdx.x;
        for (int p = 0; p < m; p++) {
            const int last = min(m - 1, p + b);
            const float ip = 1.0f / A[p * m + p];
            for (int i = p + 1 + lane; i <= last; i += 32) A[i * m + p] *= ip;
            __syncwarp();
            const int w = last - p;  // rows and columns p + 1 .. last
            for (int t = lane; t < w * w; t += 32) {
                const int i = p + 1 + t / w, j = p + 1 + (t - (t / w) * w);
                A[i * m + j] -= A[i * m + p] * A[p * m + j];
            }
            __syncwarp();
        }
        for (int i = lane; i < m; i += 32) rd[i] = 1.0f / A[i * m + i];
    }
    __syncthreads();
    for (int c = threadIdx.x; c < m; c += blockDim.x) {
        // forward: L y = e_c (unit lower), rows in order
        for (int i = 0; i < m; i++) {
            float y = (i == c) ? 1.0f : 0.0f;
            for (int k = max(0, i - b); k < i; k++) y -= A[i * m + k] * W[k * m + c];
            W[i * m + c] = y;
        }
        // backward: U x = y
        for (int i = m - 1; i >= 0; i--) {
            float x = W[i * m + c];
            for (int k = i + 1; k <= min(m - 1, i + b); k++) x -= A[i * m + k] * W[k * m + c];
            W[i * m + c] = x * rd[i];
        }
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < m * m; idx += blockDim.x) {
        const int i = idx / m, j = idx - (idx / m) * m;
        const bool live = L.k64[4 * m + i] != 0.0 && L.k64[4 * m + j] != 0.0;
        dense[idx] = live ? 0.5f * (W[i * m + j] + W[j * m + i]) : 0.0f;
    }
}

// --------------------------------------------------------------------- cycle
// The level-1 kernels walk the active cells with half a warp per cell (a cell holds at
// most max_per_cell rows, 25 in 2D at r_e = 4 l0): a warp takes two cells, their row
// ranges come from the per-solve list, and the sixteen lanes of a cell sum their rows
// with a fixed shuffle tree.
__device__ __forceinline__ float half_warp_sum(float v) {
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Level-1 residual: per search cell, the sum of its rows' residuals.
__global__ void __launch_bounds__(kBlock) k_mg_restrict0(MgLevel L1, const int2* active_rows,
                                                         const float* r, const CgScalars* S, int mode,
                                                         const int32_t* active, const int32_t* n_active) {
    pdl_begin();
    if (pcg_skip(S, mode)) return;
    const int lane = threadIdx.x & 31, half = lane >> 4, hl = lane & 15;
    const int nact = *n_active;
    const int nwarps = static_cast<int>((gridDim.x * blockDim.x) >> 5);
    for (int base = 2 * static_cast<int>((blockIdx.x * blockDim.x + threadIdx.x) >> 5); base < nact;
         base += 2 * nwarps) {
        const int a = base + half;
        float sum = 0.0f;
        int c = -1;
        if (a < nact) {
            const int2 rr = active_rows[a];
            c = active[a];
            for (int i = rr.x + hl; i < rr.y; i += 16) sum += r[i];
        }
        sum = half_warp_sum(sum);
        if (hl == 0 && c >= 0) L1.r[c] = sum;
    }
}

// An iteration's vector updates fused with the level-1 restriction of the new residual:
// s = w + beta s; p = u + beta p; d += alpha p; r -= alpha s for the particles of each
// cell (particles outside every cell are identity rows whose vectors stay zero).
__global__ void __launch_bounds__(kBlock) k_mg_axpy_restrict(CgOperands o, MgLevel L1, const int2* active_rows,
                                                             const int32_t* active, const int32_t* n_active) {
    const int lane = threadIdx.x & 31, half = lane >> 4, hl = lane & 15;
    const int nwarps = static_cast<int>((gridDim.x * blockDim.x) >> 5);
    const int base0 = 2 * static_cast<int>((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    // the first cell's row range (the active list is fixed for the solve)
    const int nact = *n_active;
    int2 rr0 = make_int2(0, 0);
    int c0 = -1;
    if (base0 + half < nact) {
        rr0 = active_rows[base0 + half];
        c0 = active[base0 + half];
    }
    pdl_begin();  // the step sizes and the vectors come from the SpMV just before
    if (pcg_skip(o.S, 1)) return;
    const float alpha = __double2float_rn(o.S->alpha);
    const float beta = __double2float_rn(o.S->beta);
    for (int base = base0; base < nact; base += 2 * nwarps) {
        const int a = base + half;
        float sum = 0.0f;
        int c = -1;
        if (a < nact) {
            const int2 rr = base == base0 ? rr0 : active_rows[a];
            c = base == base0 ? c0 : active[a];
            for (int i = rr.x + hl; i < rr.y; i += 16) {
                const float si = fmaf(beta, o.s32[i], o.w32[i]);
                const float pi = fmaf(beta, o.p32[i], o.u32[i]);
                const float ri = fmaf(-alpha, si, o.r32[i]);
                o.s32[i] = si;
                o.p32[i] = pi;
                o.d32[i] = fmaf(alpha, pi, o.d32[i]);
                o.r32[i] = ri;
                sum += ri;
            }
        }
        sum = half_warp_sum(sum);
        if (hl == 0 && c >= 0) L1.r[c] = sum;
    }
}

// Coarse residuals, four threads per coarse cell (one per child, adjacent lanes, summed
// with two shuffles in a fixed order): four times the parallelism of a thread per cell
// for these latency-bound stencils.
__global__ void __launch_bounds__(kBlock) k_mg_down(MgLevel f, MgLevel c, const CgScalars* S, int mode) {
    pdl_begin();
    if (pcg_skip(S, mode)) return;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int I = t >> 2;
    const int cell = min(I, c.cells - 1);  // whole groups of four stay in the shuffles
    const int X = cell / c.nz, Z = cell - (cell / c.nz) * c.nz;
    const int a = (t >> 1) & 1, b = t & 1;
    float v = child_residual(f.nx, f.nz, f.cells, f.k32, f.dinv, f.r, 2 * X + a, 2 * Z + b);
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    v += __shfl_xor_sync(0xffffffffu, v, 2);
    if ((t & 3) == 0 && I < c.cells) c.r[I] = v;
}

// Post-smoothed correction of the level-f cells (levels 2 .. above the bottom block), four
// threads per cell: each takes a share of the nine stencil terms (3, 2, 2, 2), summed with
// two shuffles in a fixed order.
__global__ void __launch_bounds__(kBlock) k_mg_up(MgLevel f, MgLevel c, const CgScalars* S, int mode) {
    pdl_begin();
    if (pcg_skip(S, mode)) return;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int ch0 = t >> 2;
    const int ch = min(ch0, f.cells - 1);  // whole groups of four stay in the shuffles
    const int q = t & 3;
    const int cx = ch / f.nz, cz = ch - (ch / f.nz) * f.nz;
    const int first = q == 0 ? 0 : 1 + 2 * q, count = q == 0 ? 3 : 2;  // terms 0-2, 3-4, 5-6, 7-8
    float part = 0.0f;
    for (int k = first; k < first + count; k++) {
        const int dx = k / 3 - 1, dz = k - (k / 3) * 3 - 1;
        const int nx_ = clampi(cx + dx, f.nx - 1), nz_ = clampi(cz + dz, f.nz - 1);
        const int nb = nx_ * f.nz + nz_;
        const float xn = f.dinv[nb] * f.r[nb] + kMgCoarseWeight * c.e[(nx_ >> 1) * c.nz + (nz_ >> 1)];
        part += f.k32[k * f.cells + ch] * xn;
    }
    part += __shfl_xor_sync(0xffffffffu, part, 1);
    part += __shfl_xor_sync(0xffffffffu, part, 2);
    if (q == 0 && ch0 < f.cells) {
        const float rc = f.r[ch];
        const float xc = f.dinv[ch] * rc + kMgCoarseWeight * c.e[(cx >> 1) * c.nz + (cz >> 1)];
        f.e[ch] = xc + f.dinv[ch] * (rc - part);
    }
}

struct MgBottom {
    int32_t first, last;
    MgLevel lv[kMgMaxLevels + 1];
    const float* dense;
};

// The bottom kernel's shared-memory copies: every array it stages, as one list.  Each
// thread issues eight independent 16-byte loads before it stores any of them, so the
// whole stage takes about one round trip to L2 rather than one per array (arrays and
// shared-memory segments both start on 16 bytes and hold a multiple of four floats).
struct StageSeg {
    float* dst;
    const float* src;
    int32_t n4;  // float4s
};
constexpr int kMaxStageSegs = 2 * kMgMaxLevels + 2;

__device__ __forceinline__ void stage_segments(const StageSeg* segs, const int* pre4, int nseg, int tid, int nt) {
    constexpr int kU = 8;
    const int tot4 = pre4[nseg];
    for (int base = 0; base < tot4; base += kU * nt) {
        float4 v[kU];
        float4* d[kU];
        int s = 0;
#pragma unroll
        for (int u = 0; u < kU; u++) {
            const int g = base + u * nt + tid;
            d[u] = nullptr;
            if (g < tot4) {
                while (pre4[s + 1] <= g) s++;
                const int o = g - pre4[s];
                v[u] = __ldg(reinterpret_cast<const float4*>(segs[s].src) + o);
                d[u] = reinterpret_cast<float4*>(segs[s].dst) + o;
            }
        }
#pragma unroll
        for (int u = 0; u < kU; u++)
            if (d[u]) *d[u] = v[u];
    }
}

// Levels first..last in one block, everything in shared memory: per level the nine
// coefficient planes, dinv, r and e, then the dense inverse of the last level.  The
// places of the arrays in shared memory are one table in shared memory (thread 0 lays
// them out): per-thread pointer arrays indexed by level would live in local memory,
// which a 1024-thread block with 130 KB of shared memory cannot keep in L1.
__global__ void __launch_bounds__(kMgBottomThreads) k_mg_bottom(MgBottom B, const CgScalars* S,
                                                                int mode) {
    __shared__ StageSeg segs[kMaxStageSegs];
    __shared__ int pre4[kMaxStageSegs + 1];
    __shared__ int place[4][kMgMaxLevels + 2];  // float offsets of K, dinv, r, e; [0][last + 1]: dense
    if (pcg_skip(S, mode)) return;  // no kernel of the cycle writes the scalars
    extern __shared__ float4 sm4[];
    float* sm = reinterpret_cast<float*>(sm4);
    const int tid = threadIdx.x, nt = blockDim.x;
    const int m = B.lv[B.last].cells;
    if (tid == 0) {
        int at = 0, nseg = 0;
        for (int l = B.first; l <= B.last; l++) {
            const int cells = B.lv[l].cells;
            const int c4 = static_cast<int>(mg_round4(cells));
            const int k4 = static_cast<int>(mg_round4(9 * static_cast<int64_t>(cells)));
            place[0][l] = at;
            place[1][l] = at + k4;
            place[2][l] = place[1][l] + c4;
            place[3][l] = place[2][l] + c4;
            at = place[3][l] + c4;
            segs[nseg++] = StageSeg{sm + place[0][l], B.lv[l].k32, k4 / 4};
            segs[nseg++] = StageSeg{sm + place[1][l], B.lv[l].dinv, c4 / 4};
        }
        place[0][B.last + 1] = at;
        segs[nseg++] = StageSeg{sm + at, B.dense, static_cast<int32_t>(mg_round4(static_cast<int64_t>(m) * m) / 4)};
        segs[nseg++] = StageSeg{sm + place[2][B.first], B.lv[B.first].r,
                                static_cast<int32_t>(mg_round4(B.lv[B.first].cells) / 4)};
        pre4[0] = 0;
        for (int k = 0; k < nseg; k++) pre4[k + 1] = pre4[k] + segs[k].n4;
    }
    __syncthreads();
    // the planes and the dense inverse are fixed for the solve: staged while the down
    // sweep still runs; the residuals of the first level (the last segment) after it
    const int nconst = 2 * (B.last - B.first + 1) + 1;
    stage_segments(segs, pre4, nconst, tid, nt);
    pdl_begin();
    {
        const float4* src = reinterpret_cast<const float4*>(segs[nconst].src);
        float4* dst = reinterpret_cast<float4*>(segs[nconst].dst);
        for (int k = tid; k < segs[nconst].n4; k += nt) dst[k] = __ldg(src + k);
    }
    __syncthreads();
    for (int l = B.first; l < B.last; l++) {
        const MgLevel& f = B.lv[l];
        const MgLevel& c = B.lv[l + 1];
        const float* k = sm + place[0][l];
        const float* d = sm + place[1][l];
        const float* r = sm + place[2][l];
        float* rc = sm + place[2][l + 1];
        for (int I = tid; I < c.cells; I += nt)
            rc[I] = child_residuals(f.nx, f.nz, f.cells, k, d, r, I / c.nz, I - (I / c.nz) * c.nz);
        __syncthreads();
    }
    {
        const int lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
        const float* dn = sm + place[0][B.last + 1];
        const float* rl = sm + place[2][B.last];
        float* el = sm + place[3][B.last];
        for (int row = warp; row < m; row += nwarps) {
            float v = 0.0f;
            for (int k = lane; k < m; k += 32) v += dn[row * m + k] * rl[k];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if (lane == 0) el[row] = v;
        }
        __syncthreads();
    }
    for (int l = B.last - 1; l >= B.first; l--) {
        const MgLevel& f = B.lv[l];
        const int cnz = B.lv[l + 1].nz;
        const float* k = sm + place[0][l];
        const float* d = sm + place[1][l];
        const float* r = sm + place[2][l];
        float* e = sm + place[3][l];
        const float* ec = sm + place[3][l + 1];
        for (int ch = tid; ch < f.cells; ch += nt) e[ch] = smoothed_correction(f.nx, f.nz, f.cells, k, d, r, cnz, ec, ch);
        __syncthreads();
    }
    const float* e1 = sm + place[3][B.first];
    for (int c = tid; c < B.lv[B.first].cells; c += nt) B.lv[B.first].e[c] = e1[c];
}

// u = s_i dinv0_i r_i + e_1[cell(i)] on active rows, 0 on identity rows (used when the
// bottom kernel covers level 1).
__global__ void __launch_bounds__(kBlock) k_mg_prolong0(int n, const int32_t* cell_xz, int gnz,
                                                        const float* dinv0, const float* scale,
                                                        const float* r, const float* e1, float* u,
                                                        const CgScalars* S, int mode) {
    pdl_begin();
    if (pcg_skip(S, mode)) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float d = dinv0[i];
        float v = 0.0f;
        if (d != 0.0f) {
            const int c = cell_xz[i];
            const float sc = scale ? scale[i] : 1.0f;
            v = sc * d * r[i] + (c >= 0 ? e1[(c >> 16) * gnz + (c & 0xffff)] : 0.0f);
        }
        u[i] = v;
    }
}

// ------------------------------------------------------------- fused sweeps
// The levels between the particles and the bottom block as two kernels instead of one
// per level.  A block owns a tile of one level and computes, level by level in shared
// memory, every cell of the other levels that its tile depends on: the tile's children
// or parents plus a ring of one cell per level.  So no grid-wide dependency separates
// the levels.  A ring cell is computed by every block that needs it, with the arithmetic
// of its owner, so all blocks see the same value; only owned cells are written.
// Each thread of a block owns one cell of one level and issues every global load its
// cell needs (stencil coefficients, residuals, the coarse correction) when the kernel
// starts, so a sweep waits for one round trip to L2, not one per level; the levels then
// run from registers and shared memory with a block barrier between them.
//
// Down sweep over levels 0 .. depth of a chain (level 0 is read, levels 1 .. depth are
// written): a block owns kMgDownTile x kMgDownTile cells of level depth.  Its region at
// level d starts at o_d = 2 o_{d+1} - 1 and spans n_d = 2 n_{d+1} + 2 cells per side
// (the children of level d+1's region and their stencil ring).
constexpr int kMgDownTile = 2;
constexpr int kMgUpTile = 8;  // level-1 cells per side of an up-sweep tile (one warp per column)
static_assert(kMgUpTile * 32 == kBlock, "one warp per tile column");

// region side at the level `steps` levels below the tile's level
__host__ __device__ constexpr int down_side(int steps) {
    return steps == 0 ? kMgDownTile : 2 * down_side(steps - 1) + 2;
}
constexpr int kDownSide0 = down_side(kMgFuseLevels);      // level 0 at the deepest chain
constexpr int kDownSide1 = down_side(kMgFuseLevels - 1);
constexpr int kDownSide2 = down_side(kMgFuseLevels - 2);
static_assert(kMgFuseLevels == 3, "the down sweep keeps three region planes");
static_assert(down_side(2) * down_side(2) + down_side(1) * down_side(1) + down_side(0) * down_side(0) <= kBlock,
              "one thread per computed cell");
constexpr int kDownPer0 = (kDownSide0 * kDownSide0 + kBlock - 1) / kBlock;  // level-0 cells per thread

struct MgChain {
    int32_t depth;                   // 1 .. kMgFuseLevels
    MgLevel lv[kMgFuseLevels + 1];   // lv[0]: finest
};

__global__ void __launch_bounds__(kBlock) k_mg_down_fused(MgChain C, const CgScalars* S, int mode) {
    __shared__ float R0[kDownSide0 * kDownSide0], X0[kDownSide0 * kDownSide0];
    __shared__ float R1[kDownSide1 * kDownSide1], X1[kDownSide1 * kDownSide1];
    __shared__ float R2[kDownSide2 * kDownSide2], X2[kDownSide2 * kDownSide2];
    if (pcg_skip(S, mode)) return;  // no kernel of the cycle writes the scalars
    const int D = C.depth;
    const int TX = blockIdx.x * kMgDownTile, TZ = blockIdx.y * kMgDownTile;
    const int tid = threadIdx.x;
    // this thread's cell: threads [0, n_1^2) take level 1, the next n_2^2 level 2, ...
    int my_d = 0, my_t = 0;
    {
        int t = tid;
        for (int d = 1; d <= D; d++) {
            const int sh = D - d;
            const int n = (kMgDownTile << sh) + (2 << sh) - 2;
            if (t < n * n) {
                my_d = d;
                my_t = t;
                break;
            }
            t -= n * n;
        }
    }
    int gx = 0, gz = 0, n = 0, fn = 1, fox = 0, foz = 0;
    bool in = false;
    float kk[4][9];
    float my_dinv = 0.0f;
    if (my_d > 0) {
        const MgLevel& L = C.lv[my_d];
        const MgLevel& F = C.lv[my_d - 1];
        const int sh = D - my_d;
        n = (kMgDownTile << sh) + (2 << sh) - 2;
        fn = (kMgDownTile << (sh + 1)) + (2 << (sh + 1)) - 2;
        fox = (TX << (sh + 1)) - ((1 << (sh + 1)) - 1);
        foz = (TZ << (sh + 1)) - ((1 << (sh + 1)) - 1);
        gx = (TX << sh) - ((1 << sh) - 1) + my_t / n;
        gz = (TZ << sh) - ((1 << sh) - 1) + (my_t - (my_t / n) * n);
        in = gx >= 0 && gx < L.nx && gz >= 0 && gz < L.nz;
        if (in) {
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int ccx = min(2 * gx + (q >> 1), F.nx - 1), ccz = min(2 * gz + (q & 1), F.nz - 1);
                const int ch = ccx * F.nz + ccz;
#pragma unroll
                for (int k = 0; k < 9; k++) kk[q][k] = F.k32[k * F.cells + ch];
            }
            if (my_d < D) my_dinv = L.dinv[gx * L.nz + gz];
        }
    }
    pdl_begin();  // the level-0 residuals come from the kernel just before
    // level-0 region: r (written by the kernel just before) and dinv (cells outside the
    // grid are never read by the stencil of a cell inside it: neighbours are clamped)
    const MgLevel& F0 = C.lv[0];
    const int n0 = (kMgDownTile << D) + (2 << D) - 2;
    const int o0x = (TX << D) - ((1 << D) - 1), o0z = (TZ << D) - ((1 << D) - 1);
    float r0[kDownPer0], d0[kDownPer0];
#pragma unroll
    for (int k = 0; k < kDownPer0; k++) {
        const int t = tid + k * kBlock;
        r0[k] = 0.0f;
        d0[k] = 0.0f;
        if (t < n0 * n0) {
            const int gx = o0x + t / n0, gz = o0z + (t - (t / n0) * n0);
            if (gx >= 0 && gx < F0.nx && gz >= 0 && gz < F0.nz) {
                const int c = gx * F0.nz + gz;
                r0[k] = F0.r[c];
                d0[k] = F0.dinv[c];
            }
        }
    }
#pragma unroll
    for (int k = 0; k < kDownPer0; k++) {
        const int t = tid + k * kBlock;
        if (t < n0 * n0) {
            R0[t] = r0[k];
            X0[t] = d0[k] * r0[k];
        }
    }
    __syncthreads();
    for (int d = 1; d <= D; d++) {
        if (my_d == d) {
            const MgLevel& F = C.lv[d - 1];
            const MgLevel& L = C.lv[d];
            const float* fr = d == 1 ? R0 : (d == 2 ? R1 : R2);
            const float* fx = d == 1 ? X0 : (d == 2 ? X1 : X2);
            float v = 0.0f;
            if (in) {
                float part[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int cx = 2 * gx + (q >> 1), cz = 2 * gz + (q & 1);
                    const bool valid = cx < F.nx && cz < F.nz;
                    const int ccx = min(cx, F.nx - 1), ccz = min(cz, F.nz - 1);
                    float res = fr[(ccx - fox) * fn + (ccz - foz)];
#pragma unroll
                    for (int dx = -1; dx <= 1; dx++) {
#pragma unroll
                        for (int dz = -1; dz <= 1; dz++) {
                            const int lx = clampi(ccx + dx, F.nx - 1) - fox, lz = clampi(ccz + dz, F.nz - 1) - foz;
                            res -= kk[q][(dx + 1) * 3 + dz + 1] * fx[lx * fn + lz];
                        }
                    }
                    part[q] = valid ? res : 0.0f;
                }
                // the order of the four-thread kernel's shuffles: (00 + 01) + (10 + 11)
                v = (part[0] + part[1]) + (part[2] + part[3]);
                const int sh = D - d;
                if (gx >= (TX << sh) && gx < ((TX + kMgDownTile) << sh) && gz >= (TZ << sh) &&
                    gz < ((TZ + kMgDownTile) << sh))
                    L.r[gx * L.nz + gz] = v;
            }
            if (d < D) {
                float* cr = d == 1 ? R1 : R2;
                float* cx_ = d == 1 ? X1 : X2;
                cr[my_t] = v;
                cx_[my_t] = my_dinv * v;
            }
        }
        __syncthreads();
    }
}

// Up sweep: post-smoothed corrections of chain levels depth-1 .. 0 (the coarse correction
// of level depth is read from memory) and the prolongation to the rows of level 0, which
// is level 1 of the hierarchy.  A block owns kMgUpTile x kMgUpTile level-1 cells and
// writes u for their rows; the region of level d+1 is the parents of level d's region
// widened by one cell.
struct MgUpChain {
    int32_t depth;                   // 1 .. kMgFuseLevels
    int32_t n;                       // rows
    MgLevel lv[kMgFuseLevels + 1];
    const int32_t* cell_start;
    const int32_t* row_cell;
    const float* dinv0;
    const float* scale;
    const float* r;
    float* u;
};

// rows of a tile column a lane prefetches (a column of eight cells holds about 130 rows
// in the dam break, so longer columns take a second pass)
constexpr int kUpRowsPre = 4;

__global__ void __launch_bounds__(kBlock) k_mg_up_fused(MgUpChain C, const CgScalars* S, int mode) {
    constexpr int kSide = kMgUpTile;  // every coarser region is at most this wide
    __shared__ float E[kMgFuseLevels][kSide * kSide];
    if (pcg_skip(S, mode)) return;  // no kernel of the cycle writes the scalars
    const int D = C.depth;
    const MgLevel& L0 = C.lv[0];
    const int x0 = blockIdx.x * kMgUpTile, z0 = blockIdx.y * kMgUpTile;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // the rows of tile column `warp` (cells x0 + warp, z0 .. z0 + 7 are contiguous rows)
    const int gxw = x0 + warp;
    int rb = 0, re = 0;
    if (gxw < L0.nx) {
        rb = C.cell_start[gxw * L0.nz + z0];
        re = C.cell_start[gxw * L0.nz + min(z0 + kMgUpTile, L0.nz)];
    }
    // rows without a cell (after every cell's rows) are identity rows: u = 0
    {
        const int tail = C.cell_start[L0.cells];
        const int stride = gridDim.x * gridDim.y * blockDim.x;
        for (int i = tail + (blockIdx.y * gridDim.x + blockIdx.x) * blockDim.x + tid; i < C.n; i += stride)
            C.u[i] = 0.0f;
    }
    if (!__syncthreads_or(re > rb)) return;
    // region bounds per level (inclusive), from level 0 (the tile) upwards
    int lox[kMgFuseLevels + 1], loz[kMgFuseLevels + 1], hix[kMgFuseLevels + 1], hiz[kMgFuseLevels + 1];
    lox[0] = x0;
    loz[0] = z0;
    hix[0] = x0 + kMgUpTile - 1;
    hiz[0] = z0 + kMgUpTile - 1;
#pragma unroll
    for (int d = 1; d <= kMgFuseLevels; d++) {
        lox[d] = (lox[d - 1] - 1) >> 1;
        loz[d] = (loz[d - 1] - 1) >> 1;
        hix[d] = (hix[d - 1] + 1) >> 1;
        hiz[d] = (hiz[d - 1] + 1) >> 1;
    }
    // this thread's cell: threads take the cells of level depth-1 first, then depth-2, ...
    int my_d = -1, my_t = 0;
    {
        int t = tid;
#pragma unroll
        for (int d = kMgFuseLevels - 1; d >= 0; d--) {
            if (d >= D || my_d >= 0) continue;
            const int cnt = (hix[d] - lox[d] + 1) * (hiz[d] - loz[d] + 1);
            if (t < cnt) {
                my_d = d;
                my_t = t;
            } else {
                t -= cnt;
            }
        }
    }
    // the stencil of this thread's cell: r, dinv and K of the nine neighbours (all final
    // before the kernel just before this one), and the coarse corrections of their parents
    // when the coarse level is read from memory (written by the kernel just before)
    float rn[9], dn[9], kn[9], cn[9];
    int gx = 0, gz = 0;
    bool in = false;
    if (my_d >= 0) {
        const MgLevel& F = C.lv[my_d];
        int lx = 0, lz = 0, w = 1;
#pragma unroll
        for (int d = 0; d < kMgFuseLevels; d++)
            if (d == my_d) {
                lx = lox[d];
                lz = loz[d];
                w = hiz[d] - loz[d] + 1;
            }
        gx = lx + my_t / w;
        gz = lz + (my_t - (my_t / w) * w);
        in = gx >= 0 && gx < F.nx && gz >= 0 && gz < F.nz;
        if (in) {
            const int ch = gx * F.nz + gz;
#pragma unroll
            for (int dx = -1; dx <= 1; dx++) {
#pragma unroll
                for (int dz = -1; dz <= 1; dz++) {
                    const int k = (dx + 1) * 3 + dz + 1;
                    const int ax = clampi(gx + dx, F.nx - 1), az = clampi(gz + dz, F.nz - 1);
                    const int nb = ax * F.nz + az;
                    rn[k] = F.r[nb];
                    dn[k] = F.dinv[nb];
                    kn[k] = F.k32[k * F.cells + ch];
                    cn[k] = 0.0f;
                }
            }
        }
    }
    // the rows of this lane: dinv0, scale, r and the cell of up to kUpRowsPre rows
    float rd[kUpRowsPre], rs[kUpRowsPre], rr[kUpRowsPre];
    int rc[kUpRowsPre];
#pragma unroll
    for (int k = 0; k < kUpRowsPre; k++) {
        const int i = rb + lane + 32 * k;
        rd[k] = 0.0f;
        rs[k] = 1.0f;
        rr[k] = 0.0f;
        rc[k] = 0;
        if (i < re) {
            rd[k] = C.dinv0[i];
            if (C.scale) rs[k] = C.scale[i];
            rr[k] = C.r[i];
            rc[k] = C.row_cell[i];
        }
    }
    pdl_begin();  // the coarse corrections of level `depth`
    if (in && my_d + 1 == D) {
        const MgLevel& F = C.lv[my_d];
        const MgLevel& Cl = C.lv[my_d + 1];
#pragma unroll
        for (int dx = -1; dx <= 1; dx++) {
#pragma unroll
            for (int dz = -1; dz <= 1; dz++) {
                const int ax = clampi(gx + dx, F.nx - 1), az = clampi(gz + dz, F.nz - 1);
                cn[(dx + 1) * 3 + dz + 1] = Cl.e[(ax >> 1) * Cl.nz + (az >> 1)];
            }
        }
    }
#pragma unroll
    for (int d = kMgFuseLevels - 1; d >= 0; d--) {
        if (d >= D) continue;
        if (my_d == d) {
            float e = 0.0f;
            if (in) {
                const int cwz = hiz[d + 1] - loz[d + 1] + 1;
                const int clx = lox[d + 1], clz = loz[d + 1];
                const bool top = d + 1 == D;
                const MgLevel& F = C.lv[d];
                const float* ce = top ? nullptr : E[d + 1];
                // smoothed_correction_at with the stencil's values from registers
                float cen[9];
#pragma unroll
                for (int dx = -1; dx <= 1; dx++) {
#pragma unroll
                    for (int dz = -1; dz <= 1; dz++) {
                        const int k = (dx + 1) * 3 + dz + 1;
                        const int ax = clampi(gx + dx, F.nx - 1), az = clampi(gz + dz, F.nz - 1);
                        cen[k] = kMgCoarseWeight * (top ? cn[k] : ce[((ax >> 1) - clx) * cwz + ((az >> 1) - clz)]);
                    }
                }
                const float rc0 = rn[4];
                const float xc = dn[4] * rc0 + cen[4];
                float res = rc0;
#pragma unroll
                for (int k = 0; k < 9; k++) res -= kn[k] * (dn[k] * rn[k] + cen[k]);
                e = xc + dn[4] * res;
            }
            E[d][my_t] = e;
        }
        __syncthreads();
    }
    // u = s_i dinv0_i r_i + e_1[cell(i)] on active rows, 0 on identity rows
#pragma unroll
    for (int k = 0; k < kUpRowsPre; k++) {
        const int i = rb + lane + 32 * k;
        if (i < re) {
            const float d = rd[k];
            C.u[i] = d != 0.0f ? rs[k] * d * rr[k] + E[0][warp * kMgUpTile + ((rc[k] & 0xffff) - z0)] : 0.0f;
        }
    }
    for (int i = rb + lane + 32 * kUpRowsPre; i < re; i += 32) {
        const float d = C.dinv0[i];
        float v = 0.0f;
        if (d != 0.0f) {
            const float sc = C.scale ? C.scale[i] : 1.0f;
            v = sc * d * C.r[i] + E[0][warp * kMgUpTile + ((C.row_cell[i] & 0xffff) - z0)];
        }
        C.u[i] = v;
    }
}

size_t bottom_bytes(const MgLevel* lv, int first, int last) {
    int64_t floats = 0;
    for (int l = first; l <= last; l++) floats += mg_round4(9 * static_cast<int64_t>(lv[l].cells)) + 3 * mg_round4(lv[l].cells);
    const int64_t m = lv[last].cells;
    return static_cast<size_t>(floats + mg_round4(m * m)) * sizeof(float);
}

size_t dense_smem(const MgHierarchy& mg) {
    const size_t m = static_cast<size_t>(mg.lv[mg.levels].cells);
    return (2 * m * m + m) * sizeof(float);
}

int warp_grid(int cells) { return grid_for(static_cast<int64_t>(cells) * 32); }

// grid of the kernels that walk the active level-1 cells (warp per cell, grid-stride)
int active_grid(int cells) { return std::min(warp_grid(cells), 2048); }

}  // namespace

int mg_plan(int gnx, int gnz, MgLevel* lv, int* bottom) {
    if (gnx <= 0 || gnz <= 0 || gnx >= 32768 || gnz >= 32768) return 0;
    int l = 1;
    lv[1] = MgLevel{gnx, gnz, gnx * gnz, 0, nullptr, nullptr, nullptr, nullptr, nullptr};
    while (lv[l].cells > kMgDenseCells) {
        if (l == kMgMaxLevels) return 0;
        const int nx = (lv[l].nx + 1) / 2, nz = (lv[l].nz + 1) / 2;
        lv[l + 1] = MgLevel{nx, nz, nx * nz, 0, nullptr, nullptr, nullptr, nullptr, nullptr};
        l++;
    }
    int b = l;
    while (b > 1 && bottom_bytes(lv, b - 1, l) <= kMgBottomBytes) b--;
    if (bottom_bytes(lv, b, l) > kMgBottomBytes) return 0;
    *bottom = b;
    return l;
}

cudaError_t mg_prepare_device() {
    const int dense_max = (2 * kMgDenseCells * kMgDenseCells + kMgDenseCells) * static_cast<int>(sizeof(float));
    cudaError_t e = cudaFuncSetAttribute(k_mg_dense, cudaFuncAttributeMaxDynamicSharedMemorySize, dense_max);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_mg_bottom, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                static_cast<int>(kMgBottomBytes));
}

void mg_setup_level1(const MgHierarchy& mg, const CgOperands& o, cudaStream_t s) {
    // cells without particles keep a zero residual through the solve
    cudaMemsetAsync(mg.lv[1].r, 0, sizeof(float) * mg.lv[1].cells, s);
    k_mg_bins<<<o.grid_spmv, kBlock, 0, s>>>(o, mg.cell_xz, mg.bins, mg.dinv0, kMgOmegaFine, mg.status);
    k_mg_cells<<<grid_for(mg.lv[1].cells), kBlock, 0, s>>>(mg.lv[1], mg.cell_start, mg.bins, mg.n,
                                                          kMgOmegaCoarse, mg.status, mg.active_flag);
    launch_exclusive_scan(mg.active_flag, mg.active_pos, mg.lv[1].cells, mg.scan_scratch, s);
    k_mg_active<<<grid_for(mg.lv[1].cells), kBlock, 0, s>>>(mg.lv[1].cells, mg.active_flag, mg.active_pos,
                                                           mg.cell_start, mg.active, mg.active_rows);
}

void mg_setup_coarse(const MgHierarchy& mg, cudaStream_t s) {
    for (int l = 1; l < mg.levels; l++)
        k_mg_coarsen<<<grid_for(mg.lv[l + 1].cells), kBlock, 0, s>>>(mg.lv[l], mg.lv[l + 1],
                                                                    kMgOmegaCoarse, mg.status);
    k_mg_dense<<<1, kMgBottomThreads, dense_smem(mg), s>>>(mg.lv[mg.levels], mg.dense, mg.status);
}

void mg_setup(const MgHierarchy& mg, const CgOperands& o, cudaStream_t s) {
    mg_setup_level1(mg, o, s);
    mg_setup_coarse(mg, s);
}

int mg_setup_launches(const MgHierarchy& mg) { return 2 + 3 + 1 + (mg.levels - 1) + 1; }

void mg_apply(const MgHierarchy& mg, const CgScalars* S, int mode, const float* r, float* u,
              cudaStream_t s, const CgOperands* fuse_axpy) {
    const MgLevel& L1 = mg.lv[1];
    const int g1 = active_grid(L1.cells);
    if (fuse_axpy)
        launch_pdl(k_mg_axpy_restrict, g1, kBlock, 0, s, *fuse_axpy, L1, mg.active_rows, mg.active, mg.n_active);
    else
        launch_pdl(k_mg_restrict0, g1, kBlock, 0, s, L1, mg.active_rows, r, S, mode, mg.active, mg.n_active);
    MgBottom B{};
    B.first = mg.bottom;
    B.last = mg.levels;
    for (int l = 1; l <= mg.levels; l++) B.lv[l] = mg.lv[l];
    B.dense = mg.dense;
    const size_t bottom_smem = bottom_bytes(mg.lv, mg.bottom, mg.levels);
    if (mg.bottom == 1) {
        launch_pdl(k_mg_bottom, 1, kMgBottomThreads, bottom_smem, s, B, S, mode);
        launch_pdl(k_mg_prolong0, grid_for(mg.n), kBlock, 0, s, mg.n, mg.cell_xz, L1.nz, mg.dinv0, mg.scale,
                   r, L1.e, u, S, mode);
        return;
    }
    // down: levels 1 .. bottom, the last kMgFuseLevels steps in one kernel
    const int fuse = std::min(mg.bottom - 1, kMgFuseLevels);
    for (int l = 1; l < mg.bottom - fuse; l++)
        launch_pdl(k_mg_down, grid_for(4 * static_cast<int64_t>(mg.lv[l + 1].cells)), kBlock, 0, s, mg.lv[l],
                   mg.lv[l + 1], S, mode);
    MgChain dc{};
    dc.depth = fuse;
    for (int d = 0; d <= fuse; d++) dc.lv[d] = mg.lv[mg.bottom - fuse + d];
    const MgLevel& Lb = mg.lv[mg.bottom];
    launch_pdl(k_mg_down_fused, dim3((Lb.nx + kMgDownTile - 1) / kMgDownTile, (Lb.nz + kMgDownTile - 1) / kMgDownTile),
               kBlock, 0, s, dc, S, mode);
    launch_pdl(k_mg_bottom, 1, kMgBottomThreads, bottom_smem, s, B, S, mode);
    // up: levels bottom - 1 .. 1, the last kMgFuseLevels with the prolongation in one kernel
    for (int l = mg.bottom - 1; l > fuse; l--)
        launch_pdl(k_mg_up, grid_for(4 * static_cast<int64_t>(mg.lv[l].cells)), kBlock, 0, s, mg.lv[l], mg.lv[l + 1],
                   S, mode);
    MgUpChain uc{};
    uc.depth = fuse;
    uc.n = mg.n;
    for (int d = 0; d <= fuse; d++) uc.lv[d] = mg.lv[1 + d];
    uc.cell_start = mg.cell_start;
    uc.row_cell = mg.cell_xz;
    uc.dinv0 = mg.dinv0;
    uc.scale = mg.scale;
    uc.r = r;
    uc.u = u;
    launch_pdl(k_mg_up_fused, dim3((L1.nx + kMgUpTile - 1) / kMgUpTile, (L1.nz + kMgUpTile - 1) / kMgUpTile), kBlock,
               0, s, uc, S, mode);
}

int mg_apply_launches(const MgHierarchy& mg) {
    if (mg.bottom == 1) return 3;
    return 4 + 2 * (mg.bottom - 1 - std::min(mg.bottom - 1, kMgFuseLevels));
}

}  // namespace mpsgb

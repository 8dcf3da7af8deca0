// batch.cu - the PPE solve of a batch of independent scenes: one persistent kernel, one
// scene per thread block at a time (dynamic queue), every phase of the scene's solve
// separated by __syncthreads only.
//
// Per scene:
//   setup   per-row 9-cell bins of the FP64 matrix, the level-1 operator of the scene's
//           search cells (slot order), 2 x 2 Galerkin coarsening and the dense inverse of
//           the coarsest level, all levels in shared memory;
//   solve   Chronopoulos-Gear CG in FP32 preconditioned by Jacobi on the particles plus a
//           V(1,1) cycle on the cells (the same preconditioner as the single-scene
//           multigrid solver), dot products in FP64, reliable updates with the FP64 matrix;
//   fallback if the preconditioned iteration stalls or runs out of iterations, the plain
//           FP64 CG continues from the solution reached (at most as many iterations as
//           unknowns, like the reference), and the FP64 true residual is reported.
// Block reductions sum warp partials in a fixed order, so a scene's result does not
// depend on which block solved it.
#include <cmath>

#include "batch.cuh"

namespace mpsgb {

namespace {

constexpr unsigned kMask = 0xffffffffu;

struct Smem {
    double* red;  // 3 x 32
    float* k[kMgMaxLevels + 1];
    float* d[kMgMaxLevels + 1];
    float* r[kMgMaxLevels + 1];
    float* e[kMgMaxLevels + 1];
    float* dense;
    float* colp;
    float* piv;
};

__device__ Smem carve(const BatchOps& B, float* base) {
    Smem S;
    S.red = reinterpret_cast<double*>(base);
    float* at = base + 2 * 3 * 32;
    for (int l = 1; l <= B.levels; l++) {
        const int c = B.lv[l].cells;
        S.k[l] = at;
        S.d[l] = at + 9 * c;
        S.r[l] = S.d[l] + c;
        S.e[l] = S.r[l] + c;
        at = S.e[l] + c;
    }
    const int m = B.lv[B.levels].cells;
    S.dense = at;
    S.colp = at + m * m;
    S.piv = S.colp + m;
    return S;
}

__device__ __forceinline__ double warp_sum_d(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kMask, v, o);
    return v;
}

// Block sums of three values, the same in every thread (warp partials in order).
template <int T>
__device__ void block_sum3(double& a, double& b, double& c, double* red) {
    a = warp_sum_d(a);
    b = warp_sum_d(b);
    c = warp_sum_d(c);
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        red[w] = a;
        red[32 + w] = b;
        red[64 + w] = c;
    }
    __syncthreads();
    double x = 0.0, y = 0.0, z = 0.0;
    for (int k = 0; k < T / 32; k++) {
        x += red[k];
        y += red[32 + k];
        z += red[64 + k];
    }
    __syncthreads();
    a = x;
    b = y;
    c = z;
}

__device__ __forceinline__ bool step_failed_batch(const DevStatus* st) {
    return st && (st->flags & (kStatusCellOverflow | kStatusDeviceCheck)) != 0;
}

// ------------------------------------------------------------------ setup
template <int T>
__device__ void setup_scene(const BatchOps& B, const Smem& S, const BatchScene& sc, int cellbase) {
    const CgOperands& o = B.o;
    for (int t = threadIdx.x; t < sc.rows; t += T) {
        const int i = sc.row0 + t;
        const int lane = i & 31;
        float b9[9];
#pragma unroll
        for (int q = 0; q < 9; q++) b9[q] = 0.0f;
        double aii = 0.0;
        const int ci = B.cell_xz[i];
        if (ci >= 0) {
            const int L = o.len[i];
            int64_t at = sell_index(o.off[i >> 5], lane, 0);
            for (int k = 0; k < L; k++, at += kSellRows) {
                const int j = o.col[at];
                const double a = o.val[at];
                if (j == i) aii = a;
                const int cj = B.cell_xz[j];
                const int dx = (cj >> 16) - (ci >> 16), dz = (cj & 0xffff) - (ci & 0xffff);
                const bool ok = cj >= 0 && dx >= -1 && dx <= 1 && dz >= -1 && dz <= 1;
                const int q = (dx + 1) * 3 + dz + 1;
                const float af = static_cast<float>(a);
#pragma unroll
                for (int u = 0; u < 9; u++) b9[u] += (ok && u == q) ? af : 0.0f;
            }
        }
        const bool active = ci >= 0 && aii < 0.0;
#pragma unroll
        for (int q = 0; q < 9; q++) B.bins[static_cast<int64_t>(q) * o.n + i] = active ? b9[q] : 0.0;
        B.dinv0[i] = active ? kMgOmegaFine / static_cast<float>(aii) : 0.0f;
    }
    __syncthreads();
    const MgLevel& L1 = B.lv[1];
    for (int c = threadIdx.x; c < L1.cells; c += T) {
        const int cnt = min(B.cell_count[cellbase + c], B.max_per_cell);
        const int32_t* slots = B.cell_slot + static_cast<int64_t>(cellbase + c) * B.max_per_cell;
        float kk[9];
#pragma unroll
        for (int q = 0; q < 9; q++) kk[q] = 0.0f;
        for (int s = 0; s < cnt; s++) {
            const int i = slots[s];
#pragma unroll
            for (int q = 0; q < 9; q++) kk[q] += static_cast<float>(B.bins[static_cast<int64_t>(q) * o.n + i]);
        }
#pragma unroll
        for (int q = 0; q < 9; q++) S.k[1][q * L1.cells + c] = kk[q];
        S.d[1][c] = kk[4] < 0.0f ? kMgOmegaCoarse / kk[4] : 0.0f;
    }
    __syncthreads();
    for (int l = 1; l < B.levels; l++) {
        const MgLevel& f = B.lv[l];
        const MgLevel& cc = B.lv[l + 1];
        for (int I = threadIdx.x; I < cc.cells; I += T) {
            const int X = I / cc.nz, Z = I - (I / cc.nz) * cc.nz;
            float kk[9];
#pragma unroll
            for (int q = 0; q < 9; q++) kk[q] = 0.0f;
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
                            const int DX = (nx >> 1) - X, DZ = (nz >> 1) - Z;
                            kk[(DX + 1) * 3 + DZ + 1] += S.k[l][((dx + 1) * 3 + dz + 1) * f.cells + child];
                        }
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < 9; q++) S.k[l + 1][q * cc.cells + I] = kk[q];
            S.d[l + 1][I] = kk[4] < 0.0f ? kMgOmegaCoarse / kk[4] : 0.0f;
        }
        __syncthreads();
    }
    // dense inverse of the last level: Gauss-Jordan (FP32), symmetrised; cells without
    // unknowns are unit rows of the matrix and zero rows/columns of the inverse
    const MgLevel& Lc = B.lv[B.levels];
    const int m = Lc.cells;
    const float* kc = S.k[B.levels];
    float* A = S.dense;
    for (int idx = threadIdx.x; idx < m * m; idx += T) A[idx] = 0.0f;
    __syncthreads();
    for (int c = threadIdx.x; c < m; c += T) {
        const int X = c / Lc.nz, Z = c - (c / Lc.nz) * Lc.nz;
        if (kc[4 * m + c] == 0.0f) {
            A[c * m + c] = 1.0f;
            continue;
        }
        for (int dx = -1; dx <= 1; dx++) {
            const int nx = X + dx;
            if (nx < 0 || nx >= Lc.nx) continue;
            for (int dz = -1; dz <= 1; dz++) {
                const int nz = Z + dz;
                if (nz < 0 || nz >= Lc.nz) continue;
                A[c * m + nx * Lc.nz + nz] = kc[((dx + 1) * 3 + dz + 1) * m + c];
            }
        }
    }
    for (int p = 0; p < m; p++) {
        __syncthreads();
        if (threadIdx.x == 0) S.piv[0] = 1.0f / A[p * m + p];
        for (int i = threadIdx.x; i < m; i += T) S.colp[i] = A[i * m + p];
        __syncthreads();
        const float ip = S.piv[0];
        for (int j = threadIdx.x; j < m; j += T) A[p * m + j] = (j == p ? 1.0f : A[p * m + j]) * ip;
        __syncthreads();
        for (int idx = threadIdx.x; idx < m * m; idx += T) {
            const int i = idx / m, j = idx - (idx / m) * m;
            if (i == p) continue;
            A[idx] = (j == p ? 0.0f : A[idx]) - S.colp[i] * A[p * m + j];
        }
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < m * m; idx += T) {
        const int i = idx / m, j = idx - (idx / m) * m;
        if (i > j) continue;
        const bool live = kc[4 * m + i] != 0.0f && kc[4 * m + j] != 0.0f;
        const float v = live ? 0.5f * (A[i * m + j] + A[j * m + i]) : 0.0f;
        A[i * m + j] = v;
        A[j * m + i] = v;
    }
    __syncthreads();
}

// ------------------------------------------------------------------ solve
// u = M r for the scene's rows (r in o.r32, u into o.u32)
template <int T>
__device__ void apply_m(const BatchOps& B, const Smem& S, const BatchScene& sc, int cellbase) {
    const CgOperands& o = B.o;
    const MgLevel& L1 = B.lv[1];
    for (int c = threadIdx.x; c < L1.cells; c += T) {
        const int cnt = min(B.cell_count[cellbase + c], B.max_per_cell);
        const int32_t* slots = B.cell_slot + static_cast<int64_t>(cellbase + c) * B.max_per_cell;
        float sum = 0.0f;
        for (int s = 0; s < cnt; s++) sum += o.r32[slots[s]];
        S.r[1][c] = sum;
    }
    __syncthreads();
    for (int l = 1; l < B.levels; l++) {
        const MgLevel& f = B.lv[l];
        const MgLevel& c = B.lv[l + 1];
        for (int I = threadIdx.x; I < c.cells; I += T)
            S.r[l + 1][I] = child_residuals(f.nx, f.nz, f.cells, S.k[l], S.d[l], S.r[l], I / c.nz,
                                            I - (I / c.nz) * c.nz);
        __syncthreads();
    }
    {
        const int m = B.lv[B.levels].cells;
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        const float* rl = S.r[B.levels];
        for (int row = warp; row < m; row += T / 32) {
            float v = 0.0f;
            for (int k = lane; k < m; k += 32) v += S.dense[row * m + k] * rl[k];
            for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(kMask, v, off);
            if (lane == 0) S.e[B.levels][row] = v;
        }
        __syncthreads();
    }
    for (int l = B.levels - 1; l >= 1; l--) {
        const MgLevel& f = B.lv[l];
        for (int ch = threadIdx.x; ch < f.cells; ch += T)
            S.e[l][ch] = smoothed_correction(f.nx, f.nz, f.cells, S.k[l], S.d[l], S.r[l], B.lv[l + 1].nz,
                                             S.e[l + 1], ch);
        __syncthreads();
    }
    for (int t = threadIdx.x; t < sc.rows; t += T) {
        const int i = sc.row0 + t;
        const float d = B.dinv0[i];
        const int ci = B.cell_xz[i];
        o.u32[i] = (d != 0.0f && ci >= 0) ? d * o.r32[i] + S.e[1][(ci >> 16) * L1.nz + (ci & 0xffff)] : 0.0f;
    }
    __syncthreads();
}

// w = A u (FP32 matrix); returns gamma = r.u, delta = w.u, rho = r.r (FP64 sums)
template <int T>
__device__ void spmv_dots(const BatchOps& B, const Smem& S, const BatchScene& sc, double& gam, double& del,
                          double& rho) {
    const CgOperands& o = B.o;
    double g = 0.0, d = 0.0, r = 0.0;
    for (int t = threadIdx.x; t < sc.rows; t += T) {
        const int i = sc.row0 + t;
        const int L = o.len[i];
        int64_t at = sell_index(o.off[i >> 5], i & 31, 0);
        float acc = 0.0f;
        for (int k = 0; k < L; k++, at += kSellRows) {
            const uint2 e = ld_sell_pair(o.cv32 + at);
            acc = fmaf(__uint_as_float(e.y), o.u32[e.x], acc);
        }
        o.w32[i] = acc;
        const double ri = o.r32[i], ui = o.u32[i];
        g += ri * ui;
        d += static_cast<double>(acc) * ui;
        r += ri * ri;
    }
    block_sum3<T>(g, d, r, S.red);
    gam = g;
    del = d;
    rho = r;
}

// r = b - A x with the FP64 matrix (into r32 and, for the fallback, r64); returns r.r, b.b
template <int T>
__device__ void residual64(const BatchOps& B, const Smem& S, const BatchScene& sc, bool to64, double& rr,
                           double& bb) {
    const CgOperands& o = B.o;
    double a = 0.0, b = 0.0, z = 0.0;
    for (int t = threadIdx.x; t < sc.rows; t += T) {
        const int i = sc.row0 + t;
        const int L = o.len[i];
        int64_t at = sell_index(o.off[i >> 5], i & 31, 0);
        double acc = 0.0;
        for (int k = 0; k < L; k++, at += kSellRows) acc = fma(o.val[at], o.x[o.col[at]], acc);
        const double ri = o.b[i] - acc;
        o.r32[i] = static_cast<float>(ri);
        if (to64) {
            B.r64[i] = ri;
            B.p64[i] = ri;
        }
        a += ri * ri;
        b += o.b[i] * o.b[i];
    }
    block_sum3<T>(a, b, z, S.red);
    rr = a;
    bb = b;
}

template <int T>
__device__ void solve_scene(const BatchOps& B, const Smem& S, int k) {
    const CgOperands& o = B.o;
    const BatchScene sc = B.scenes[k];
    const int cellbase = k * B.cells_per_scene;
    BatchSolveStats st = {};
    if (step_failed_batch(B.status)) {
        st.aborted = 1;
        if (threadIdx.x == 0) B.stats[k] = st;
        return;
    }
    setup_scene<T>(B, S, sc, cellbase);
    for (int t = threadIdx.x; t < sc.rows; t += T) {
        const int i = sc.row0 + t;
        o.s32[i] = 0.0f;
        o.p32[i] = 0.0f;
        o.d32[i] = 0.0f;
        o.u32[i] = 0.0f;
    }
    __syncthreads();
    double rr, bb;
    residual64<T>(B, S, sc, false, rr, bb);
    const double eps2 = B.eps * B.eps;
    const double thr = (B.criterion == MPS_CRIT_RHS && bb > 0.0) ? bb * eps2 : rr * eps2;
    bool conv = (B.criterion == MPS_CRIT_RHS) ? (rr < thr || rr == 0.0) : (thr == 0.0);
    st.rr0 = rr;
    st.bb = bb;
    int iter = 0, updates = 0;
    bool stalled = false;
    if (!conv) {
        double rr_upd = rr, prev_true = rr;
        double gam, del, rho;
        apply_m<T>(B, S, sc, cellbase);
        spmv_dots<T>(B, S, sc, gam, del, rho);
        double alpha = gam / del, beta = 0.0, gam_old = gam;
        stalled = !(std::isfinite(alpha) && alpha != 0.0);
        while (!conv && !stalled && iter < B.max_iter) {
            const float fa = static_cast<float>(alpha), fb = static_cast<float>(beta);
            for (int t = threadIdx.x; t < sc.rows; t += T) {
                const int i = sc.row0 + t;
                const float si = fmaf(fb, o.s32[i], o.w32[i]);
                const float pi = fmaf(fb, o.p32[i], o.u32[i]);
                o.s32[i] = si;
                o.p32[i] = pi;
                o.d32[i] = fmaf(fa, pi, o.d32[i]);
                o.r32[i] = fmaf(-fa, si, o.r32[i]);
            }
            __syncthreads();
            apply_m<T>(B, S, sc, cellbase);
            spmv_dots<T>(B, S, sc, gam, del, rho);
            if (rho < B.delta2 * rr_upd || rho < thr) {
                // reliable update: fold the FP32 correction into x, FP64 true residual
                for (int t = threadIdx.x; t < sc.rows; t += T) {
                    const int i = sc.row0 + t;
                    o.x[i] += static_cast<double>(o.d32[i]);
                    o.d32[i] = 0.0f;
                }
                __syncthreads();
                double tr, dummy;
                residual64<T>(B, S, sc, false, tr, dummy);
                updates++;
                rr_upd = tr;
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
                apply_m<T>(B, S, sc, cellbase);
                spmv_dots<T>(B, S, sc, gam, del, rho);
            }
            beta = gam / gam_old;
            alpha = gam / (del - beta * gam / alpha);
            gam_old = gam;
            iter++;
            if (!(std::isfinite(alpha) && std::isfinite(beta) && alpha != 0.0)) stalled = true;
        }
        for (int t = threadIdx.x; t < sc.rows; t += T) {
            const int i = sc.row0 + t;
            o.x[i] += static_cast<double>(o.d32[i]);
            o.d32[i] = 0.0f;
        }
        __syncthreads();
    }
    st.iterations = iter;
    st.updates = updates;
    st.stalled = stalled ? 1 : 0;
    if (!conv) {
        // plain FP64 CG from the solution reached (at most as many iterations as rows)
        st.fallback = 1;
        double r2, b2;
        residual64<T>(B, S, sc, true, r2, b2);
        const double thr64 = (B.criterion == MPS_CRIT_RHS && b2 > 0.0) ? b2 * eps2 : r2 * eps2;
        conv = (B.criterion == MPS_CRIT_RHS) ? (r2 < thr64 || r2 == 0.0) : (thr64 == 0.0);
        int fit = 0;
        while (!conv && fit < sc.rows) {
            double pap = 0.0, z1 = 0.0, z2 = 0.0;
            for (int t = threadIdx.x; t < sc.rows; t += T) {
                const int i = sc.row0 + t;
                const int L = o.len[i];
                int64_t at = sell_index(o.off[i >> 5], i & 31, 0);
                double acc = 0.0;
                for (int kk = 0; kk < L; kk++, at += kSellRows) acc = fma(o.val[at], B.p64[o.col[at]], acc);
                B.Ap64[i] = acc;
                pap += B.p64[i] * acc;
            }
            block_sum3<T>(pap, z1, z2, S.red);
            const double a = r2 / pap;
            double rn = 0.0;
            for (int t = threadIdx.x; t < sc.rows; t += T) {
                const int i = sc.row0 + t;
                o.x[i] = fma(a, B.p64[i], o.x[i]);
                const double ri = fma(-a, B.Ap64[i], B.r64[i]);
                B.r64[i] = ri;
                rn += ri * ri;
            }
            z1 = z2 = 0.0;
            block_sum3<T>(rn, z1, z2, S.red);
            fit++;
            if (rn < thr64) {
                conv = true;
                break;
            }
            const double bt = rn / r2;
            r2 = rn;
            for (int t = threadIdx.x; t < sc.rows; t += T) {
                const int i = sc.row0 + t;
                B.p64[i] = fma(bt, B.p64[i], B.r64[i]);
            }
            __syncthreads();
        }
        st.fb_iterations = fit;
        st.iterations += fit;
    }
    double tr, dummy;
    residual64<T>(B, S, sc, false, tr, dummy);
    st.true_rr = tr;
    st.converged = conv ? 1 : 0;
    if (threadIdx.x == 0) {
        B.stats[k] = st;
        if (!conv) atomicExch(B.all_ok, 0);
    }
}

template <int T>
__global__ void __launch_bounds__(T) k_batch_solve(BatchOps B) {
    extern __shared__ __align__(16) float smem[];
    __shared__ int s_next;
    const Smem S = carve(B, smem);
    for (;;) {
        if (threadIdx.x == 0) s_next = atomicAdd(B.queue, 1);
        __syncthreads();
        const int q = s_next;
        __syncthreads();
        if (q >= B.nscenes) break;
        solve_scene<T>(B, S, B.order[q]);
        __syncthreads();
    }
}

}  // namespace

size_t batch_smem_bytes(const BatchOps& B, int threads) {
    (void)threads;
    size_t floats = 2 * 3 * 32;
    for (int l = 1; l <= B.levels; l++) floats += 12 * static_cast<size_t>(B.lv[l].cells);
    const size_t m = static_cast<size_t>(B.lv[B.levels].cells);
    floats += m * m + m + 1;
    const size_t bytes = (floats * sizeof(float) + 15) / 16 * 16;
    return bytes <= 220 * 1024 ? bytes : 0;
}

cudaError_t batch_prepare_device(size_t smem_bytes) {
    const int b = static_cast<int>(smem_bytes);
    cudaError_t e = cudaFuncSetAttribute(k_batch_solve<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_batch_solve<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_batch_solve<512>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_batch_solve<1024>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    return e;
}

int batch_blocks_per_sm(int threads, size_t smem) {
    int b = 0;
    cudaError_t e = cudaErrorInvalidValue;
    switch (threads) {
        case 128: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch_solve<128>, 128, smem); break;
        case 256: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch_solve<256>, 256, smem); break;
        case 512: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch_solve<512>, 512, smem); break;
        case 1024: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch_solve<1024>, 1024, smem); break;
        default: break;
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return b;
}

cudaError_t launch_batch_solve(const BatchOps& B, int blocks, int threads, cudaStream_t s) {
    const size_t smem = batch_smem_bytes(B, threads);
    if (smem == 0 || blocks <= 0) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(B.queue, 0, sizeof(int32_t), s);
    if (e != cudaSuccess) return e;
    switch (threads) {
        case 128: k_batch_solve<128><<<blocks, 128, smem, s>>>(B); break;
        case 256: k_batch_solve<256><<<blocks, 256, smem, s>>>(B); break;
        case 512: k_batch_solve<512><<<blocks, 512, smem, s>>>(B); break;
        case 1024: k_batch_solve<1024><<<blocks, 1024, smem, s>>>(B); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace mpsgb

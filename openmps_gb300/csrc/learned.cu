// learned.cu - learned warm start / preconditioner scale: features, tensor-core
// inference (tcgen05, BF16 x BF16 -> FP32 in TMEM), warm start, training samples, and
// the FP32 forward/backward training kernels with Adam.
//
// Tensor-core inference (k_mlp_tc): one CTA of 128 threads per tile of 128 particles
// (persistent over tiles).  The four weight matrices live in shared memory in the
// canonical K-major no-swizzle layout of tcgen05 (8-row x 16-byte core matrices; LBO =
// byte distance of K-adjacent core matrices, SBO = distance of M/N-adjacent 8-row
// groups).  Per layer one thread issues the K/16 MMAs (M = 128, N = 64, or 16 for the
// padded output layer) into 64 TMEM columns and commits them to an mbarrier; every
// thread then reads its own row of the accumulator (tcgen05.ld 32x32b: warp w owns TMEM
// lanes 32w..32w+31), adds the bias, applies GELU, rounds to BF16 and writes the row
// back as the next layer's A operand.  Waits are bounded (WaitLimits::mma_clocks): a
// wait that gives up waits once more, within kMmaDrainClocks, for the MMAs it issued to
// complete, sets an error word, frees its TMEM and returns; the solve then uses no
// network output.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>

#include "learned.cuh"

namespace mpsgb {

namespace {

constexpr int kTile = 128;
constexpr int kTmemCols = 64;

// tensor-core weight image (bytes)
constexpr int kImgW1 = 0;                       // N 64 x K 16
constexpr int kImgW2 = kImgW1 + 64 * 16 * 2;    // N 64 x K 64
constexpr int kImgW3 = kImgW2 + 64 * 64 * 2;
constexpr int kImgW4 = kImgW3 + 64 * 64 * 2;    // N 16 (2 used) x K 64
constexpr int kImgBias = kImgW4 + 16 * 64 * 2;  // b1[64] b2[64] b3[64] b4[16] FP32
constexpr int kImgNorm = kImgBias + (64 * 3 + 16) * 4;  // mean[16] std[16]
constexpr int kImgBytes = ((kImgNorm + 32 * 4) + 15) / 16 * 16;

// shared-memory map of the inference kernel (the tail is slack: every address any
// descriptor can form stays inside the allocation)
constexpr int kSmA0 = 0;                        // 128 x 16 BF16
constexpr int kSmA = kSmA0 + kTile * 16 * 2;    // 128 x 64 BF16
constexpr int kSmImg = kSmA + kTile * 64 * 2;
constexpr int kSmBar = (kSmImg + kImgBytes + 15) / 16 * 16;
constexpr int kSmBytes = 48 * 1024;  // four CTAs per SM: the whole grid is resident

// byte offset of element (r, k) of a K-major operand with `rows` rows
__host__ __device__ constexpr int core_offset(int r, int k, int rows) {
    return ((k >> 3) * (rows >> 3) + (r >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// tcgen05 shared-memory matrix descriptor, no swizzle
__device__ __forceinline__ uint64_t sm_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= static_cast<uint64_t>((addr >> 4) & 0x3FFFu);
    d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
    d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
    d |= static_cast<uint64_t>(1) << 46;  // descriptor version of tcgen05
    return d;                             // base offset 0, no swizzle
}

// instruction descriptor of kind::f16: BF16 A and B (K-major), FP32 D, M = 128
__host__ __device__ constexpr uint32_t idesc_bf16(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(n >> 3) << 17) |
           (static_cast<uint32_t>(kTile >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ bool bar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void proxy_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive FP32 accumulator columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z) {
    return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    const uint32_t lo = __bfloat16_as_ushort(__float2bfloat16_rn(a));
    const uint32_t hi = __bfloat16_as_ushort(__float2bfloat16_rn(b));
    return lo | (hi << 16);
}

// writes 8 consecutive K values of row r of a K-major operand (one 16-byte store)
__device__ __forceinline__ void store_row8(unsigned char* base, int rows, int r, int kc, const float* v) {
    uint4 q;
    q.x = pack_bf16(v[0], v[1]);
    q.y = pack_bf16(v[2], v[3]);
    q.z = pack_bf16(v[4], v[5]);
    q.w = pack_bf16(v[6], v[7]);
    *reinterpret_cast<uint4*>(base + core_offset(r, kc * 8, rows)) = q;
}

// ------------------------------------------------------------ inference (tcgen05)
__global__ void __launch_bounds__(kTile) k_mlp_tc(const unsigned char* __restrict__ image,
                                                  const float* __restrict__ feat, int n,
                                                  const double* sigma, float* __restrict__ out,
                                                  int32_t* error, const WaitLimits* limits) {
    extern __shared__ __align__(1024) unsigned char sm[];
    const int t = threadIdx.x, warp = t >> 5;
    unsigned char* A0 = sm + kSmA0;
    unsigned char* A = sm + kSmA;
    unsigned char* img = sm + kSmImg;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + kSmBar);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + kSmBar + 8);

    for (int k = t; k < kImgBytes / 16; k += kTile)
        reinterpret_cast<uint4*>(img)[k] = reinterpret_cast<const uint4*>(image)[k];
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    const uint32_t lane_addr = tmem + (static_cast<uint32_t>(warp * 32) << 16);
    const float* bias = reinterpret_cast<const float*>(img + kImgBias);
    const float* mu = reinterpret_cast<const float*>(img + kImgNorm);
    const float* sd = mu + 16;
    const float inv_sigma = sigma ? static_cast<float>(1.0 / sigma[0]) : 1.0f;
    const long long wait_clocks = limits ? limits->mma_clocks : kDefaultMmaClocks;
    const uint32_t aA0 = smem_u32(A0), aA = smem_u32(A), aImg = smem_u32(img);
    uint32_t phase = 0;
    bool bad = false;
    const int ntiles = (n + kTile - 1) / kTile;

    // features of the CTA's next tile are loaded while the current tile runs its layers
    float4 nxt[4];
    auto load_tile = [&](int tile) {
        const int r = tile * kTile + t;
        if (tile < ntiles && r < n) {
            const float4* f4 = reinterpret_cast<const float4*>(feat + static_cast<int64_t>(r) * kMlpIn);
#pragma unroll
            for (int q = 0; q < 4; q++) nxt[q] = __ldg(f4 + q);
        }
    };
    load_tile(blockIdx.x);
    for (int tile = blockIdx.x; tile < ntiles && !bad; tile += gridDim.x) {
        const int row = tile * kTile + t;
        float x[16];
        if (row < n) {
#pragma unroll
            for (int q = 0; q < 4; q++) {
                x[4 * q] = nxt[q].x;
                x[4 * q + 1] = nxt[q].y;
                x[4 * q + 2] = nxt[q].z;
                x[4 * q + 3] = nxt[q].w;
            }
            x[8] *= inv_sigma;
            x[9] *= inv_sigma;
            x[10] *= inv_sigma;
#pragma unroll
            for (int k = 0; k < 16; k++) x[k] = (x[k] - mu[k]) / sd[k];
        } else {
#pragma unroll
            for (int k = 0; k < 16; k++) x[k] = 0.0f;
        }
        load_tile(tile + gridDim.x);
        store_row8(A0, kTile, t, 0, x);
        store_row8(A0, kTile, t, 1, x + 8);
        proxy_fence();
        tc_fence_before();
        __syncthreads();

        for (int layer = 0; layer < 4 && !bad; layer++) {
            if (t == 0) {
                tc_fence_after();
                if (layer == 0) {
                    mma_bf16(tmem, sm_desc(aA0, (kTile / 8) * 128, 128),
                             sm_desc(aImg + kImgW1, 64 / 8 * 128, 128), idesc_bf16(64), 0);
                } else {
                    const int nb = layer == 3 ? 16 : 64;
                    const uint32_t wb = aImg + (layer == 1 ? kImgW2 : layer == 2 ? kImgW3 : kImgW4);
                    const uint32_t lbo_a = (kTile / 8) * 128, lbo_b = (nb / 8) * 128;
#pragma unroll
                    for (int s = 0; s < 4; s++)
                        mma_bf16(tmem, sm_desc(aA + 2 * s * lbo_a, lbo_a, 128),
                                 sm_desc(wb + 2 * s * lbo_b, lbo_b, 128), idesc_bf16(nb), s > 0 ? 1u : 0u);
                }
                mma_commit(bar);
            }
            // the bound is checked before each poll, so a bound of 0 gives up at once
            const long long t0 = clock64();
            for (;;) {
                if (clock64() - t0 >= wait_clocks) {
                    bad = true;
                    break;
                }
                if (bar_try_wait(bar, phase)) break;
            }
            if (bad) {
                // the layer's MMAs may still be writing TMEM: wait for their commit
                // (bounded) before the CTA frees TMEM below
                const long long t1 = clock64();
                while (!bar_try_wait(bar, phase) && clock64() - t1 < kMmaDrainClocks) {
                }
            }
            phase ^= 1u;
            tc_fence_after();
            if (!bad) {
                if (layer < 3) {
                    const float* b = bias + 64 * layer;
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        float v[16];
                        tmem_ld16(lane_addr + 16 * q, v);
#pragma unroll
                        for (int k = 0; k < 16; k++) v[k] = gelu(v[k] + b[16 * q + k]);
                        store_row8(A, kTile, t, 2 * q, v);
                        store_row8(A, kTile, t, 2 * q + 1, v + 8);
                    }
                    proxy_fence();
                } else {
                    float v[16];
                    tmem_ld16(lane_addr, v);
                    if (row < n) {
                        out[2 * static_cast<int64_t>(row)] = v[0] + bias[192];
                        out[2 * static_cast<int64_t>(row) + 1] = v[1] + bias[193];
                    }
                }
            }
            tc_fence_before();
            bad = __syncthreads_or(bad) != 0;
        }
    }
    if (bad && t == 0) atomicExch(error, 1);
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols)
                     : "memory");
}

// ------------------------------------------------------------------ features
// Nothing to learn from when the step failed or the initial guess already solves it.
__device__ __forceinline__ bool lrn_skip(const CgScalars* S) { return S->aborted != 0 || S->converged != 0; }

// Per particle: density deviation, source term, free-surface deficiency, wall flag
// (neighbour-averaged below), the Jacobi term g = omega r0 / a_ii and the scaled p.
__global__ void __launch_bounds__(kBlock) k_lrn_q(LearnedOps L, CgOperands o, const float* dinv0,
                                                  const StepScalars* step, const CgScalars* S,
                                                  float4* q4, float2* q2) {
    // each solve starts with a clear tensor-core error word (read by the host after it)
    if (blockIdx.x == 0 && threadIdx.x == 0) *L.error = 0;
    if (lrn_skip(S)) return;
    const double dt = step->dt;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < L.n; i += gridDim.x * blockDim.x) {
        const int q = L.particle_of ? L.particle_of[i] : i;  // row i holds particle q
        const double dev = (L.nd[q] - L.n0) / L.n0;
        double surf;
        if (L.flags & MPS_FLAG_SPP) {
            surf = (L.n0 - L.n_wo_spp[q]) / L.n0;
        } else {
            surf = (L.n0 - L.nd[q]) / L.n0;
        }
        surf = surf > 0.0 ? surf : 0.0;
        const float src = static_cast<float>(o.b[i] * dt * dt / L.rho);
        const float wall = L.type[q] == MPS_TYPE_WALL ? 1.0f : 0.0f;
        q4[i] = make_float4(static_cast<float>(dev), src, static_cast<float>(surf), wall);
        const float g = dinv0[i] * o.r32[i];
        q2[i] = make_float2(g, static_cast<float>(L.p[q] * dt * dt / L.rho_l02));
    }
}

__device__ double block_sum_d(double v, double* ws) {
    ws[threadIdx.x] = v;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (static_cast<int>(threadIdx.x) < s) ws[threadIdx.x] += ws[threadIdx.x + s];
        __syncthreads();
    }
    const double r = ws[0];
    __syncthreads();
    return r;
}

// Features (one warp per SELL chunk, lane per row; neighbour averages weighted by the
// FP32 PPE coefficients a_ij, j != i), the first preconditioned step c = alpha0 u0, FP64
// copy of x0, and sigma = RMS of g over active rows (last block).
__global__ void __launch_bounds__(kBlock) k_lrn_features(LearnedOps L, CgOperands o, const float* dinv0,
                                                         const StepScalars* step, const CgScalars* S,
                                                         const float4* q4, const float2* q2, float len_ref) {
    __shared__ double ws[kBlock];
    __shared__ bool last;
    if (lrn_skip(S)) return;
    const int lane = threadIdx.x & 31;
    const int warp = static_cast<int>((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int nwarps = static_cast<int>((gridDim.x * blockDim.x) >> 5);
    const double dt = step->dt;
    const float alpha0 = static_cast<float>(S->alpha);
    double g2 = 0.0, cnt = 0.0;
    for (int c = warp; c < o.nchunks; c += nwarps) {
        const int i = kSellRows * c + lane;
        if (i >= o.n) continue;
        const float d0 = dinv0[i];
        const bool active = d0 != 0.0f;
        L.active[i] = active ? 1 : 0;
        L.x0d[i] = o.x[i];
        float f[16];
#pragma unroll
        for (int k = 0; k < 16; k++) f[k] = 0.0f;
        float cc = 0.0f;
        if (active) {
            const int len = o.len[i];
            int64_t at = sell_index(o.off[c], lane, 0);
            float wsum = 0.0f, s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, s3 = 0.0f, s4 = 0.0f, s5 = 0.0f;
            for (int k = 0; k < len; k++, at += kSellRows) {
                const uint2 e = o.cv32[at];
                const int j = static_cast<int>(e.x);
                if (j == i) continue;
                const float w = __uint_as_float(e.y);
                const float4 a = q4[j];
                const float2 b = q2[j];
                wsum += w;
                s0 += w * a.x;
                s1 += w * a.y;
                s2 += w * a.z;
                s3 += w * a.w;
                s4 += w * b.x;
                s5 += w * b.y;
            }
            const float inv = wsum > 0.0f ? 1.0f / wsum : 0.0f;
            const float4 a = q4[i];
            const float2 b = q2[i];
            cc = alpha0 * o.u32[i];
            f[0] = a.x;
            f[1] = s0 * inv;
            f[2] = a.y;
            f[3] = s1 * inv;
            f[4] = a.z;
            f[5] = s2 * inv;
            f[6] = a.w;
            f[7] = s3 * inv;
            f[8] = b.x;
            f[9] = s4 * inv;
            f[10] = cc;
            f[11] = static_cast<float>((kMgOmegaFine / d0) / L.a_ref) - 1.0f;
            f[12] = static_cast<float>(len) / len_ref - 1.0f;
            f[13] = b.y;
            f[14] = s5 * inv - b.y;
            f[15] = static_cast<float>(L.ecs[L.particle_of ? L.particle_of[i] : i] * dt);
            g2 += static_cast<double>(b.x) * b.x;
            cnt += 1.0;
        }
        float4* dst = reinterpret_cast<float4*>(L.feat + static_cast<int64_t>(i) * kMlpIn);
#pragma unroll
        for (int q = 0; q < 4; q++) dst[q] = make_float4(f[4 * q], f[4 * q + 1], f[4 * q + 2], f[4 * q + 3]);
        L.coarse[i] = cc;
    }
    const double sg = block_sum_d(g2, ws);
    const double sc = block_sum_d(cnt, ws);
    if (threadIdx.x == 0) {
        L.partials[2 * blockIdx.x] = sg;
        L.partials[2 * blockIdx.x + 1] = sc;
        __threadfence();
        last = atomicAdd(L.counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    double a = 0.0, b = 0.0;
    for (int k = threadIdx.x; k < static_cast<int>(gridDim.x); k += blockDim.x) {
        a += __ldcg(L.partials + 2 * k);
        b += __ldcg(L.partials + 2 * k + 1);
    }
    a = block_sum_d(a, ws);
    b = block_sum_d(b, ws);
    if (threadIdx.x == 0) {
        *L.counter = 0;
        const double s = b > 0.0 ? sqrt(a / b) : 0.0;
        L.sigma[0] = s > 0.0 ? s : 1.0;
    }
}

// x += c + sigma out0 on active rows; scale = 1 + 0.25 tanh(out1) (1 without a usable output).
__global__ void __launch_bounds__(kBlock) k_lrn_apply(LearnedOps L, CgOperands o, const CgScalars* S) {
    if (lrn_skip(S)) return;
    const bool ok = *L.error == 0;
    const double sg = L.sigma[0];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < L.n; i += gridDim.x * blockDim.x) {
        float s = 1.0f;
        if (ok && L.active[i]) {
            const float o0 = L.out[2 * static_cast<int64_t>(i)], o1 = L.out[2 * static_cast<int64_t>(i) + 1];
            if (isfinite(o0) && isfinite(o1)) {
                o.x[i] += static_cast<double>(L.coarse[i]) + sg * static_cast<double>(o0);
                s = 1.0f + kMlpScaleRange * tanhf(o1);
            }
        }
        L.scale[i] = s;
    }
}

// Training sample of each row after the solve: features (residual features in units of
// sigma), y = (x* - x0 - c) / sigma, g / sigma.
__global__ void __launch_bounds__(kBlock) k_lrn_targets(LearnedOps L, CgOperands o, const CgScalars* S) {
    if (lrn_skip(S)) {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < L.n; i += gridDim.x * blockDim.x)
            L.active[i] = 0;
        return;
    }
    const double sg = L.sigma[0];
    const float inv = static_cast<float>(1.0 / sg);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < L.n; i += gridDim.x * blockDim.x) {
        float* dst = L.sample + static_cast<int64_t>(i) * kMlpSampleFloats;
        const float* f = L.feat + static_cast<int64_t>(i) * kMlpIn;
        for (int k = 0; k < kMlpIn; k++) dst[k] = (k >= 8 && k <= 10) ? f[k] * inv : f[k];
        dst[16] = L.active[i] ? static_cast<float>((o.x[i] - L.x0d[i] - static_cast<double>(L.coarse[i])) / sg) : 0.0f;
        dst[17] = f[8] * inv;
    }
}

// ------------------------------------------------------------------ training
constexpr int kTrainThreads = 256;
constexpr int kTrainS = 64;  // samples per block pass
// shared-memory floats of the training kernel
constexpr int kTrWt1 = 0;                        // [16][64]
constexpr int kTrB1 = kTrWt1 + 16 * 64;
constexpr int kTrWt2 = kTrB1 + 64;               // [64][64] transposed (forward)
constexpr int kTrW2 = kTrWt2 + 4096;             // [64][64] (backward)
constexpr int kTrB2 = kTrW2 + 4096;
constexpr int kTrWt3 = kTrB2 + 64;
constexpr int kTrW3 = kTrWt3 + 4096;
constexpr int kTrB3 = kTrW3 + 4096;
constexpr int kTrW4 = kTrB3 + 64;                // [2][64]
constexpr int kTrB4 = kTrW4 + 128;
constexpr int kTrG = kTrB4 + 2;                  // gradient, blob order from W1 (kMlpParams)
constexpr int kTrX = kTrG + kMlpParams;          // [64][16]
constexpr int kTrZ1 = kTrX + kTrainS * 16;       // [64][64] x 6
constexpr int kTrA1 = kTrZ1 + kTrainS * 64;
constexpr int kTrZ2 = kTrA1 + kTrainS * 64;
constexpr int kTrA2 = kTrZ2 + kTrainS * 64;
constexpr int kTrZ3 = kTrA2 + kTrainS * 64;
constexpr int kTrA3 = kTrZ3 + kTrainS * 64;
constexpr int kTrO = kTrA3 + kTrainS * 64;       // [64][2]
constexpr int kTrD4 = kTrO + kTrainS * 2;        // [64][2]
constexpr int kTrY = kTrD4 + kTrainS * 2;        // [64][2]: y, g
constexpr int kTrFloats = kTrY + kTrainS * 2;
constexpr size_t kTrBytes = kTrFloats * sizeof(float);

// gradient offsets (relative to blob W1)
constexpr int gW1 = 0, gB1 = gW1 + 1024, gW2 = gB1 + 64, gB2 = gW2 + 4096, gW3 = gB2 + 64,
              gB3 = gW3 + 4096, gW4 = gB3 + 64, gB4 = gW4 + 128;

// Z = A W^T + b (64 outputs per sample), then the activation
__device__ __forceinline__ void dense_fwd(const float* Wt, const float* b, const float* Ain, int kin,
                                          float* Z, float* Aout) {
    const int j = threadIdx.x & 63, s0 = threadIdx.x >> 6;
    for (int s = s0; s < kTrainS; s += kTrainThreads / 64) {
        float acc = b[j];
        for (int k = 0; k < kin; k++) acc = fmaf(Wt[k * 64 + j], Ain[s * kin + k], acc);
        Z[s * 64 + j] = acc;
        Aout[s * 64 + j] = gelu(acc);
    }
}

// G[j][k] += sum_s delta[s][j] A[s][k]; Gb[j] += sum_s delta[s][j]
__device__ __forceinline__ void dense_wgrad(const float* delta, const float* Ain, int kin, float* G, float* Gb) {
    for (int e = threadIdx.x; e < 64 * kin; e += kTrainThreads) {
        const int j = e / kin, k = e - (e / kin) * kin;
        float acc = 0.0f;
        for (int s = 0; s < kTrainS; s++) acc = fmaf(delta[s * 64 + j], Ain[s * kin + k], acc);
        G[e] += acc;
    }
    if (threadIdx.x < 64) {
        float acc = 0.0f;
        for (int s = 0; s < kTrainS; s++) acc += delta[s * 64 + threadIdx.x];
        Gb[threadIdx.x] += acc;
    }
}

// delta_prev[s][k] = (sum_j W[j][k] delta[s][j]) * gelu'(Zprev[s][k]), in place in Zprev
__device__ __forceinline__ void dense_back(const float* W, const float* delta, float* Zprev) {
    const int k = threadIdx.x & 63, s0 = threadIdx.x >> 6;
    for (int s = s0; s < kTrainS; s += kTrainThreads / 64) {
        float acc = 0.0f;
        for (int j = 0; j < 64; j++) acc = fmaf(W[j * 64 + k], delta[s * 64 + j], acc);
        Zprev[s * 64 + k] = acc * gelu_grad(Zprev[s * 64 + k]);
    }
}

// Loss and gradient of the mean loss over `total` samples; one partial per block.
__global__ void __launch_bounds__(kTrainThreads) k_mlp_grad(const float* __restrict__ w,
                                                           const float* __restrict__ samples, int64_t n,
                                                           int64_t total, float* partials) {
    extern __shared__ float sh[];
    const int t = threadIdx.x;
    const float* W1 = w + kMlpOffW1;
    const float* W2 = w + kMlpOffW2;
    const float* W3 = w + kMlpOffW3;
    for (int e = t; e < 1024; e += kTrainThreads) {
        const int j = e >> 4, k = e & 15;
        sh[kTrWt1 + k * 64 + j] = W1[e];
    }
    for (int e = t; e < 4096; e += kTrainThreads) {
        const int j = e >> 6, k = e & 63;
        sh[kTrWt2 + k * 64 + j] = W2[e];
        sh[kTrW2 + e] = W2[e];
        sh[kTrWt3 + k * 64 + j] = W3[e];
        sh[kTrW3 + e] = W3[e];
    }
    for (int e = t; e < 64; e += kTrainThreads) {
        sh[kTrB1 + e] = w[kMlpOffB1 + e];
        sh[kTrB2 + e] = w[kMlpOffB2 + e];
        sh[kTrB3 + e] = w[kMlpOffB3 + e];
    }
    for (int e = t; e < 128; e += kTrainThreads) sh[kTrW4 + e] = w[kMlpOffW4 + e];
    if (t < 2) sh[kTrB4 + t] = w[kMlpOffB4 + t];
    for (int e = t; e < kMlpParams; e += kTrainThreads) sh[kTrG + e] = 0.0f;
    __shared__ float lsum[kTrainS];
    float loss_acc = 0.0f;
    const float inv_total = 1.0f / static_cast<float>(total);
    const float* mu = w + kMlpOffMu;
    const float* sd = w + kMlpOffSd;
    __syncthreads();
    for (int64_t base = static_cast<int64_t>(blockIdx.x) * kTrainS; base < n;
         base += static_cast<int64_t>(gridDim.x) * kTrainS) {
        for (int e = t; e < kTrainS * 16; e += kTrainThreads) {
            const int s = e >> 4, k = e & 15;
            const int64_t idx = base + s;
            sh[kTrX + e] = idx < n ? (samples[idx * kMlpSampleFloats + k] - mu[k]) / sd[k] : 0.0f;
        }
        if (t < kTrainS) {
            const int64_t idx = base + t;
            sh[kTrY + 2 * t] = idx < n ? samples[idx * kMlpSampleFloats + 16] : 0.0f;
            sh[kTrY + 2 * t + 1] = idx < n ? samples[idx * kMlpSampleFloats + 17] : 0.0f;
        }
        __syncthreads();
        dense_fwd(sh + kTrWt1, sh + kTrB1, sh + kTrX, 16, sh + kTrZ1, sh + kTrA1);
        __syncthreads();
        dense_fwd(sh + kTrWt2, sh + kTrB2, sh + kTrA1, 64, sh + kTrZ2, sh + kTrA2);
        __syncthreads();
        dense_fwd(sh + kTrWt3, sh + kTrB3, sh + kTrA2, 64, sh + kTrZ3, sh + kTrA3);
        __syncthreads();
        if (t < 2 * kTrainS) {
            const int s = t >> 1, o = t & 1;
            float acc = sh[kTrB4 + o];
            for (int k = 0; k < 64; k++) acc = fmaf(sh[kTrW4 + o * 64 + k], sh[kTrA3 + s * 64 + k], acc);
            sh[kTrO + 2 * s + o] = acc;
        }
        __syncthreads();
        if (t < kTrainS) {
            const bool valid = base + t < n;
            const float o0 = sh[kTrO + 2 * t], o1 = sh[kTrO + 2 * t + 1];
            const float y = sh[kTrY + 2 * t], g = sh[kTrY + 2 * t + 1];
            const float th = tanhf(o1);
            const float sc = 1.0f + kMlpScaleRange * th;
            const float r0 = o0 - y, r1 = y - sc * g;
            lsum[t] = valid ? r0 * r0 + r1 * r1 : 0.0f;
            sh[kTrD4 + 2 * t] = valid ? 2.0f * r0 * inv_total : 0.0f;
            sh[kTrD4 + 2 * t + 1] = valid ? -2.0f * r1 * g * kMlpScaleRange * (1.0f - th * th) * inv_total : 0.0f;
        }
        __syncthreads();
        if (t == 0)
            for (int s = 0; s < kTrainS; s++) loss_acc += lsum[s];
        // output layer
        if (t < 128) {
            const int o = t >> 6, k = t & 63;
            float acc = 0.0f;
            for (int s = 0; s < kTrainS; s++) acc = fmaf(sh[kTrD4 + 2 * s + o], sh[kTrA3 + s * 64 + k], acc);
            sh[kTrG + gW4 + t] += acc;
        }
        if (t < 2) {
            float acc = 0.0f;
            for (int s = 0; s < kTrainS; s++) acc += sh[kTrD4 + 2 * s + t];
            sh[kTrG + gB4 + t] += acc;
        }
        {
            const int k = t & 63, s0 = t >> 6;
            for (int s = s0; s < kTrainS; s += kTrainThreads / 64) {
                const float d = sh[kTrW4 + k] * sh[kTrD4 + 2 * s] + sh[kTrW4 + 64 + k] * sh[kTrD4 + 2 * s + 1];
                sh[kTrZ3 + s * 64 + k] = d * gelu_grad(sh[kTrZ3 + s * 64 + k]);
            }
        }
        __syncthreads();
        dense_wgrad(sh + kTrZ3, sh + kTrA2, 64, sh + kTrG + gW3, sh + kTrG + gB3);
        dense_back(sh + kTrW3, sh + kTrZ3, sh + kTrZ2);
        __syncthreads();
        dense_wgrad(sh + kTrZ2, sh + kTrA1, 64, sh + kTrG + gW2, sh + kTrG + gB2);
        dense_back(sh + kTrW2, sh + kTrZ2, sh + kTrZ1);
        __syncthreads();
        dense_wgrad(sh + kTrZ1, sh + kTrX, 16, sh + kTrG + gW1, sh + kTrG + gB1);
        __syncthreads();
    }
    float* dst = partials + static_cast<int64_t>(blockIdx.x) * (kMlpParams + 1);
    for (int e = t; e < kMlpParams; e += kTrainThreads) dst[e] = sh[kTrG + e];
    if (t == 0) dst[kMlpParams] = loss_acc;
}

// grad = sum of the block partials in block order; loss likewise
__global__ void k_mlp_reduce(const float* partials, int blocks, float* grad, double* loss) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e > kMlpParams) return;
    double acc = 0.0;
    for (int b = 0; b < blocks; b++) acc += partials[static_cast<int64_t>(b) * (kMlpParams + 1) + e];
    if (e < kMlpParams)
        grad[kMlpOffW1 + e] = static_cast<float>(acc);
    else
        *loss = acc;
}

__global__ void k_mlp_adam(float* w, float* m, float* v, const float* grad, float lr, float bc1, float bc2) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x + kMlpOffW1;
    if (e >= kMlpBlobFloats) return;
    const float g = grad[e];
    const float mm = 0.9f * m[e] + 0.1f * g;
    const float vv = 0.999f * v[e] + 0.001f * g * g;
    m[e] = mm;
    v[e] = vv;
    w[e] -= lr * (mm / bc1) / (sqrtf(vv / bc2) + 1e-8f);
}

}  // namespace

size_t mlp_packed_bytes() { return kImgBytes; }

void mlp_pack_weights(const float* blob, void* image) {
    unsigned char* img = static_cast<unsigned char*>(image);
    std::memset(img, 0, kImgBytes);
    auto bf16 = [](float f) -> uint16_t {  // round to nearest even
        uint32_t u;
        std::memcpy(&u, &f, 4);
        if ((u & 0x7f800000u) == 0x7f800000u) return static_cast<uint16_t>(u >> 16);
        u += 0x7fffu + ((u >> 16) & 1u);
        return static_cast<uint16_t>(u >> 16);
    };
    auto put = [&](int off, int rows, int kdim, const float* W, int used_rows) {
        for (int r = 0; r < used_rows; r++)
            for (int k = 0; k < kdim; k++) {
                const uint16_t h = bf16(W[r * kdim + k]);
                std::memcpy(img + off + core_offset(r, k, rows), &h, 2);
            }
    };
    put(kImgW1, 64, 16, blob + kMlpOffW1, 64);
    put(kImgW2, 64, 64, blob + kMlpOffW2, 64);
    put(kImgW3, 64, 64, blob + kMlpOffW3, 64);
    put(kImgW4, 16, 64, blob + kMlpOffW4, 2);
    float* bias = reinterpret_cast<float*>(img + kImgBias);
    std::memcpy(bias, blob + kMlpOffB1, 64 * 4);
    std::memcpy(bias + 64, blob + kMlpOffB2, 64 * 4);
    std::memcpy(bias + 128, blob + kMlpOffB3, 64 * 4);
    std::memcpy(bias + 192, blob + kMlpOffB4, 2 * 4);
    std::memcpy(img + kImgNorm, blob + kMlpOffMu, 32 * 4);
}

cudaError_t mlp_prepare_device() {
    return cudaFuncSetAttribute(k_mlp_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmBytes);
}

cudaError_t mlp_train_prepare_device() {
    return cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                static_cast<int>(kTrBytes));
}

void launch_learned_q(const LearnedOps& L, const CgOperands& o, const CgScalars* S, cudaStream_t s) {
    k_lrn_q<<<grid_for(L.n), kBlock, 0, s>>>(L, o, L.dinv0, L.step, S, L.q4, L.q2);
}

void launch_learned_feature_rows(const LearnedOps& L, const CgOperands& o, const CgScalars* S, cudaStream_t s) {
    k_lrn_features<<<o.grid_spmv, kBlock, 0, s>>>(L, o, L.dinv0, L.step, S, L.q4, L.q2, L.len_ref);
}

void launch_learned_features(const LearnedOps& L, const CgOperands& o, const CgScalars* S,
                             cudaStream_t s) {
    launch_learned_q(L, o, S, s);
    launch_learned_feature_rows(L, o, S, s);
}

void launch_learned_apply(const LearnedOps& L, const CgOperands& o, const CgScalars* S, cudaStream_t s) {
    k_lrn_apply<<<grid_for(L.n), kBlock, 0, s>>>(L, o, S);
}

void launch_learned_targets(const LearnedOps& L, const CgOperands& o, const CgScalars* S,
                            cudaStream_t s) {
    k_lrn_targets<<<grid_for(L.n), kBlock, 0, s>>>(L, o, S);
}

void launch_mlp_infer(const void* packed, const float* feat, int n, const double* sigma, float* out,
                      int32_t* error, cudaStream_t s, const WaitLimits* limits) {
    const int tiles = (n + kTile - 1) / kTile;
    const int grid = tiles < 4 * 152 ? (tiles > 0 ? tiles : 1) : 4 * 152;
    k_mlp_tc<<<grid, kTile, kSmBytes, s>>>(static_cast<const unsigned char*>(packed), feat, n, sigma, out, error,
                                           limits);
}

int mlp_train_blocks(int64_t n) {
    const int64_t b = (n + kTrainS - 1) / kTrainS;
    return static_cast<int>(b < 148 ? (b > 0 ? b : 1) : 148);
}

void launch_mlp_loss_grad(const MlpTrainer& T, const float* samples, int64_t n, cudaStream_t s) {
    const int blocks = mlp_train_blocks(n);
    k_mlp_grad<<<blocks, kTrainThreads, kTrBytes, s>>>(T.w, samples, n, n, T.partials);
    k_mlp_reduce<<<(kMlpParams + 1 + 255) / 256, 256, 0, s>>>(T.partials, blocks, T.grad, T.loss);
}

void launch_mlp_adam(const MlpTrainer& T, float lr, int step, cudaStream_t s) {
    const float bc1 = 1.0f - std::pow(0.9f, static_cast<float>(step));
    const float bc2 = 1.0f - std::pow(0.999f, static_cast<float>(step));
    k_mlp_adam<<<(kMlpParams + 255) / 256, 256, 0, s>>>(T.w, T.m, T.v, T.grad, lr, bc1, bc2);
}

}  // namespace mpsgb

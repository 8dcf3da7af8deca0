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
constexpr int kReCache = 48;  // cached weights per particle (entries beyond are recomputed)

// device status bits
constexpr int kStatusCellOverflow = 1;
constexpr int kStatusDeviceCheck = 2;
constexpr int kStatusCgNotConverged = 4;
constexpr int kStatusNonFinite = 8;
constexpr int kStatusWaitTimeout = 16;  // a bounded device wait gave up (MPS_ERR_TIMEOUT)

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
    // FP32 bounds of the FP64 range tests (range_class below): r^2 surely below nl2_lo
    // under f32_in_nl, surely above nl2_hi / re^2 / re_lap^2 / d^2 over the f32_out_*
    // values (d = l0 - max_dx, the collision distance of DynamicStabilize)
    float f32_in_nl;
    float f32_out_nl, f32_out_re, f32_out_rl, f32_out_ds;
    double l0, re, re2, re_lap, rl2;
    double nl, nl2_lo, nl2_hi;  // neighbour length and a guard band around nl^2
    double n0, lambda, n0_lap, lambda_lap;
    double rho, nu, g, surface_ratio, max_dt, max_dx;
    double min_x, min_z;
    double sound_speed;  // c of the explicit pressure (MPS_FLAG_PRESSURE_EXPLICIT)
    // three-dimensional scenes (DIM3): cells (x, y, z) at ((cx gny) + cy) gnz + cz
    int32_t dim;  // 2 or 3
    int32_t gny;  // cells along y (1 in 2D)
    double min_y;
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
    float *x32, *z32;  // positions rounded to FP32 (range prefilter), rewritten with x, z
    // PPE row order of a single scene: particles sorted by search cell (slot order within
    // a cell, particles without a cell slot last in index order), so the rows of a cell
    // are contiguous: coalesced level-1 multigrid work and local SpMV gathers.  Null for a
    // batch, whose rows stay in particle order.
    int32_t* row_of;       // particle -> row
    int32_t* particle_of;  // row -> particle
    int32_t* row_cell;     // row -> (cx << 16) | cz of its cell, -1: none
    int32_t* cell_fill;    // per cell: particles stored (count clipped to maxPerCell)
    int32_t* cell_start;   // exclusive prefix sum of cell_fill (cells + 1 entries)
    int32_t* unplaced;     // per particle: 1 without a cell slot
    int32_t* unplaced_pos; // exclusive prefix sum of unplaced (n + 1 entries)
    int32_t* row_scratch;  // scan scratch of the two prefix sums
    // W(r, r_e) of the first kReCache list entries within r_e of each particle, in list
    // order ([m n + i]), written by the fused density + assembly walk and read by the
    // pressure gradient on the same positions
    double* w_re;
    // the SPP sums sum W(r, r_e^lap) dx and dz of the fused density + assembly walk
    // ([i], [n + i]), read by the pressure gradient on the same positions when r_e^lap =
    // r_e (the same pairs in the same order: the sums are the gradient's own)
    double* spp_g;
    const int32_t* scene_of;  // batch: scene of each particle (its cells start at
                              // scene * cells_per_scene); null for a single scene
    int32_t *nb_count, *nb;
    int32_t *ppe_len, *ppe_col_tmp;
    double *ppe_val_tmp, *ppe_b, *ppe_x;
    int32_t *ppe_chunk, *ppe_off, *scan_scratch;  // chunk sizes, chunk offsets
    int32_t* ppe_col;                              // SELL-32 columns
    double* ppe_val;                               // SELL-32 FP64 values
    uint2* ppe_cv32;                               // SELL-32 {column, FP32 value}
    // 1: PPE rows in cell order, SELL chunks at a fixed stride of ppe_stride entries per
    // row, written in place by the assembly walk; 0: rows through the ELL scratch and
    // k_ppe_sort into the compact layout
    int32_t ppe_direct;
    int32_t ppe_fp32;  // the assembly also writes ppe_cv32 (set per launch)
    StepScalars* step;
    DevStatus* status;
    const int32_t* solve_ok;  // converged flag of the last PPE solve
    // the y axis of three-dimensional scenes (null in 2D): position, velocity, wall
    // target, SaveX copy and velocity change
    double *y, *v, *wall_y, *oy, *duy;
    float* y32;  // FP32 copy of y (range prefilter), rewritten with y
};

// ------------------------------- FP64 division and square root off the FP64 pipe
// GB300 issues FP64 arithmetic at a small fraction of its FP32 rate, and a correctly
// rounded FP64 division or square root costs about as much as eight FP64 fused
// multiply-adds there.  The stage kernels need both for every pair in range, with the
// IEEE result bit for bit.  ddiv_rn / dsqrt_rn below compute that result on the FP32
// and integer pipes:
//   1. the 53-bit significands are split into float-float pairs (hi: the top 24 bits,
//      exact; lo: the next 29 bits, rounded), and the quotient ma / mb or the root of
//      the significand is approximated as q1 + q2 in FP32 (one Newton correction with
//      an error-free product for q1 * hi), to about 2^-44;
//   2. the estimate, scaled to a 53-bit integer Q', gives the exact integer remainder
//      R = N - Q' mb (or N - S'^2) in 64-bit modular arithmetic: |Q - Q'| < 2^9 by the
//      error bound of step 1, so |R| < 2^62 and the low 64 bits hold it exactly;
//   3. R's top bits give the correction d ~ R / mb (off by at most one), two compares
//      each way bring 0 <= R < mb (0 <= R <= 2S for the root), and the quotient or root
//      rounds up when 2R > mb (R > S); ties cannot occur for a quotient or a root of
//      53-bit significands.
// Operands that are zero, subnormal, infinite or NaN, and results outside the normal
// range, take __ddiv_rn / __dsqrt_rn, so every input gives the IEEE result.
namespace exact {

constexpr unsigned long long kM52 = (1ull << 52) - 1ull, kH52 = 1ull << 52;

// the float of a 24-bit integer in [2^23, 2^24) (exact)
__device__ __forceinline__ float f24(unsigned int v) { return __int_as_float((150 << 23) | (v & 0x7FFFFFu)); }

// f * 2^s as an integer for |f| 2^s < 2^63 (truncated below the float's last bit)
__device__ __forceinline__ long long fscale(float f, int s) {
    const unsigned int u = static_cast<unsigned int>(__float_as_int(f));
    const int e = static_cast<int>((u >> 23) & 0xFFu) - 150 + s;
    const long long m = static_cast<long long>((u & 0x7FFFFFu) | 0x800000u);
    long long v = e >= 0 ? (m << min(e, 63)) : (m >> min(-e, 63));
    if ((u & 0x7FFFFFFFu) == 0u) v = 0;
    return (u >> 31) ? -v : v;
}

}  // namespace exact

// a / b, rounded to nearest even (the IEEE quotient)
__device__ __forceinline__ double ddiv_rn(double a, double b) {
    using namespace exact;
    const unsigned long long ua = static_cast<unsigned long long>(__double_as_longlong(a));
    const unsigned long long ub = static_cast<unsigned long long>(__double_as_longlong(b));
    const int ea = static_cast<int>((ua >> 52) & 0x7FFu), eb = static_cast<int>((ub >> 52) & 0x7FFu);
    const unsigned long long ma = (ua & kM52) | kH52, mb = (ub & kM52) | kH52;
    const int ge = ma >= mb;
    int e = ea - eb + 1022 + ge;
    const int s = ge ? 52 : 53;
    const float ah = f24(static_cast<unsigned int>(ma >> 29)), bh = f24(static_cast<unsigned int>(mb >> 29));
    const float al = __fmul_rn(__uint2float_rn(static_cast<unsigned int>(ma & 0x1FFFFFFFu)), 0x1p-29f);
    const float bl = __fmul_rn(__uint2float_rn(static_cast<unsigned int>(mb & 0x1FFFFFFFu)), 0x1p-29f);
    float y = __fdividef(1.0f, bh);
    y = __fmaf_rn(y, __fmaf_rn(-bh, y, 1.0f), y);
    const float q1 = __fmul_rn(ah, y);
    const float p = __fmul_rn(q1, bh);
    const float pe = __fmaf_rn(q1, bh, -p);
    const float rho = __fadd_rn(__fsub_rn(__fsub_rn(ah, p), pe), __fmaf_rn(-q1, bl, al));
    const float q2 = __fmul_rn(rho, y);
    long long Q = fscale(q1, s) + fscale(q2, s);
    const long long B = static_cast<long long>(mb);
    long long R = static_cast<long long>((ma << s) - static_cast<unsigned long long>(Q) * mb);
    const int d = __float2int_rd(__fmul_rn(__fmul_rn(__int2float_rn(static_cast<int>(R >> 32)), 8.0f), y));
    Q += d;
    R -= static_cast<long long>(d) * B;
    if (R < 0) { Q--; R += B; }
    if (R < 0) { Q--; R += B; }
    if (R >= B) { Q++; R -= B; }
    if (R >= B) { Q++; R -= B; }
    const bool in_range = R >= 0 && R < B;
    if (2ull * static_cast<unsigned long long>(R) > mb) Q++;
    if (Q == (1ll << 53)) {
        Q = static_cast<long long>(kH52);
        e++;
    }
    const bool fast = ea != 0 && ea != 2047 && eb != 0 && eb != 2047 && e >= 1 && e <= 2046 && in_range;
    if (!fast) return __ddiv_rn(a, b);
    return __longlong_as_double(static_cast<long long>(((ua ^ ub) & (1ull << 63)) |
                                                       (static_cast<unsigned long long>(e) << 52) |
                                                       (static_cast<unsigned long long>(Q) & kM52)));
}

// sqrt(x), rounded to nearest even (the IEEE square root)
__device__ __forceinline__ double dsqrt_rn(double x) {
    using namespace exact;
    const unsigned long long ux = static_cast<unsigned long long>(__double_as_longlong(x));
    const int ex = static_cast<int>(ux >> 52);  // >= 2048 for a set sign bit
    const unsigned long long m = (ux & kM52) | kH52;
    const int E = ex - 1023;
    const int odd = E & 1;
    int e = ((E - odd) >> 1) + 1023;
    // X = m 2^t with S = floor(sqrt(X)) in [2^52, 2^53); v = X / 2^80 = (xh + xl) in
    // float-float, sqrt(X) = sqrt(v) 2^40
    const int t = odd ? 53 : 52;
    const float f = odd ? 4.0f : 2.0f;
    const float xh = __fmul_rn(f24(static_cast<unsigned int>(m >> 29)), f);
    const float xl = __fmul_rn(__fmul_rn(__uint2float_rn(static_cast<unsigned int>(m & 0x1FFFFFFFu)), 0x1p-29f), f);
    const float rs = rsqrtf(xh);
    const float s1 = __fmul_rn(xh, rs);
    const float p = __fmul_rn(s1, s1);
    const float pe = __fmaf_rn(s1, s1, -p);
    const float rho = __fadd_rn(__fsub_rn(__fsub_rn(xh, p), pe), xl);
    const float h = __fmul_rn(0.5f, rs);
    const float s2 = __fmul_rn(rho, h);
    long long S = fscale(s1, 40) + fscale(s2, 40);
    const unsigned long long X = m << t;
    long long R = static_cast<long long>(X - static_cast<unsigned long long>(S) * static_cast<unsigned long long>(S));
    // d ~ R / (2 S) with S ~ s1 2^40: (R >> 32) 2^-9 / s1 = (R >> 32) 2^-8 h
    S += __float2int_rd(__fmul_rn(__fmul_rn(__int2float_rn(static_cast<int>(R >> 32)), 0x1p-8f), h));
    R = static_cast<long long>(X - static_cast<unsigned long long>(S) * static_cast<unsigned long long>(S));
    if (R < 0) { S--; R += 2 * S + 1; }
    if (R < 0) { S--; R += 2 * S + 1; }
    if (R > 2 * S) { R -= 2 * S + 1; S++; }
    if (R > 2 * S) { R -= 2 * S + 1; S++; }
    const bool fast = ex != 0 && ex < 2047 && R >= 0 && R <= 2 * S;
    if (R > S) S++;
    if (S == (1ll << 53)) {
        S = static_cast<long long>(kH52);
        e++;
    }
    if (!fast) return __dsqrt_rn(x);
    return __longlong_as_double(static_cast<long long>((static_cast<unsigned long long>(e) << 52) |
                                                       (static_cast<unsigned long long>(S) & kM52)));
}

// --------------------------------------------------------------- helpers
// uBLAS inner_prod of 2-vectors: t = 0; t += a0*b0; t += a1*b1, each op rounded.
__device__ __forceinline__ double dot2(double a0, double a1, double b0, double b1) {
    return __dadd_rn(__dadd_rn(0.0, __dmul_rn(a0, b0)), __dmul_rn(a1, b1));
}

// The stage kernels are bound by GB300's FP64 pipe, so exact FP64 comparisons against a
// positive finite bound run on the integer pipe: for b > 0 finite, a < b exactly when
// the bit pattern of a, read as an unsigned integer, is below that of b (non-negative
// doubles order like their bit patterns; -0, negative values and NaN of either sign
// compare false, as in IEEE).
__device__ __forceinline__ bool below(double a, double b) {
    return static_cast<unsigned long long>(__double_as_longlong(a)) <
           static_cast<unsigned long long>(__double_as_longlong(b));
}

// sums_from_zero: where the reference adds a zero term to an accumulator of a neighbour
// walk (a dummy neighbour's zero vector, a pair outside the collision distance), the
// stage kernels add nothing.  Each such accumulator starts at +0, and a round-to-nearest
// sum that starts at +0 never holds -0 (x + y is -0 only when both are -0), so x + 0 is
// x bit for bit; only the payload of a NaN could differ (it stays a NaN).  On GB300 that
// saves two FP64 additions per pair in range of the dynamic stabilisation walk.

// dot2 without its leading 0 +: the two differ only in the sign of a zero result, so
// dot2_term serves where that sign cannot reach the result: the HS term dot / r^3 (r > 0)
// added to a sum that starts at +0 (sums_from_zero above).
__device__ __forceinline__ double dot2_term(double a0, double a1, double b0, double b1) {
    return __dadd_rn(__dmul_rn(a0, b0), __dmul_rn(a1, b1));
}

// Squared distance: the reference's inner_prod(r, r) = (0 + dx dx) + dz dz.  The 0 + is
// the identity here (a square is never -0), so it is left out.
__device__ __forceinline__ double dist2(double dx, double dz) {
    return __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dz, dz));
}

// Particle::W (Particle.hpp:71-75); the test 0 < r < re on the integer pipe: bits(r) - 1
// wraps for +0 and lands at or above bits(re) - 1 for r >= re, -0, negatives and NaN.
__device__ __forceinline__ double weight(double r, double re) {
    const unsigned long long br = static_cast<unsigned long long>(__double_as_longlong(r));
    const unsigned long long be = static_cast<unsigned long long>(__double_as_longlong(re));
    return (br - 1ull < be - 1ull) ? __dadd_rn(ddiv_rn(re, r), -1.0) : 0.0;
}

__device__ __forceinline__ bool has_flag(uint32_t flags, uint32_t f) { return (flags & f) != 0u; }

// ------------------------------------------------- FP32 prefilter of the range tests
// GB300 issues FP64 arithmetic at a small fraction of its FP32 rate, and most entries
// of a neighbour row fail the r^2 < r_e^2 test of a stage.  A test on the FP32 copies of
// the positions settles the clear cases with certainty and leaves only pairs in a thin
// band around the threshold (its width set by the FP32 rounding of the coordinates) and
// non-finite positions to the exact FP64 test, so every decision equals the FP64 one.
//
// Bound: with u = 2^-24 and x~ = fl32(x), |x - x~| <= u |x~| / (1 - u), and a = fl32(x~j -
// x~i) gives |(xj - xi)| in [|a|(1 - u) - e, |a| / (1 - u) + e], e = 1.01 u (|x~i| + |x~j|).
// E = 2^-22 (|x~i| + |z~i| + |x~j| + |z~j|) + 1e-36 covers e + u|a| for both axes (the
// 1e-36 covers FP32 subnormal rounding), so r^2 lies in [ (|a| - E)+^2 + (|b| - E)+^2,
// (|a| + E)^2 + (|b| + E)^2 ] up to four FP32 roundings (4 u relative).  The FP64 r^2 of
// the stages (dx = xj - xi, dot2) is within 2^-50 of the exact value.  With FP32 bounds
// set 2^-20 inside (in) or outside (out) of the FP64 threshold, "in" implies FP64 r^2 <
// threshold and "out" implies FP64 r^2 > threshold.  NaN and infinity fall through to
// the FP64 test (comparisons false, fmaxf drops NaN).
__device__ __forceinline__ float range_slack(float sum_abs) {
    return sum_abs * 2.384185791015625e-07f + 1e-36f;  // 2^-22
}

// Lower bound of r^2 (FP32) for the pair; `out` when it exceeds `out_thr`.
__device__ __forceinline__ bool surely_out(float xi, float zi, float si, float xj, float zj,
                                           float out_thr) {
    const float e = range_slack(si + (fabsf(xj) + fabsf(zj)));
    const float lx = fmaxf(fabsf(xj - xi) - e, 0.0f);
    const float lz = fmaxf(fabsf(zj - zi) - e, 0.0f);
    return lx * lx + lz * lz > out_thr;
}

// 1: FP64 r^2 < the lower threshold for sure; 0: FP64 r^2 > the upper threshold for
// sure; 2: undecided (exact FP64 test).
__device__ __forceinline__ int range_class(float xi, float zi, float si, float xj, float zj,
                                           float in_thr, float out_thr) {
    const float e = range_slack(si + (fabsf(xj) + fabsf(zj)));
    const float ax = fabsf(xj - xi), az = fabsf(zj - zi);
    const float hx = ax + e, hz = az + e;
    if (hx * hx + hz * hz < in_thr) return 1;
    const float lx = fmaxf(ax - e, 0.0f), lz = fmaxf(az - e, 0.0f);
    return (lx * lx + lz * lz > out_thr) ? 0 : 2;
}

// The same for three coordinates.  Each axis's error bound above only grows with the
// sum of absolute coordinates, so E = 2^-22 (sum of the six |coordinates|) + 1e-36
// covers every axis; the bounds of r^2 take six FP32 roundings (6 u relative), still
// inside the 2^-20 margin of the thresholds, and the FP64 r^2 of dist3 is within 2^-50.
__device__ __forceinline__ bool surely_out3(float xi, float yi, float zi, float si, float xj, float yj,
                                            float zj, float out_thr) {
    const float e = range_slack(si + ((fabsf(xj) + fabsf(yj)) + fabsf(zj)));
    const float lx = fmaxf(fabsf(xj - xi) - e, 0.0f);
    const float ly = fmaxf(fabsf(yj - yi) - e, 0.0f);
    const float lz = fmaxf(fabsf(zj - zi) - e, 0.0f);
    return (lx * lx + ly * ly) + lz * lz > out_thr;
}
__device__ __forceinline__ int range_class3(float xi, float yi, float zi, float si, float xj, float yj,
                                            float zj, float in_thr, float out_thr) {
    const float e = range_slack(si + ((fabsf(xj) + fabsf(yj)) + fabsf(zj)));
    const float ax = fabsf(xj - xi), ay = fabsf(yj - yi), az = fabsf(zj - zi);
    const float hx = ax + e, hy = ay + e, hz = az + e;
    if ((hx * hx + hy * hy) + hz * hz < in_thr) return 1;
    const float lx = fmaxf(ax - e, 0.0f), ly = fmaxf(ay - e, 0.0f), lz = fmaxf(az - e, 0.0f);
    return ((lx * lx + ly * ly) + lz * lz > out_thr) ? 0 : 2;
}

// Calls f(j) for the entries of row i that may pass the FP64 range test whose FP32
// upper bound is `out_thr`, in list order.  Entries are screened 128 at a time into a
// bit mask first (two 64-bit words: a whole row of the usual radii), so the FP64 work of
// a warp runs once per candidate of its busiest lane rather than once per list entry.
template <class F>
__device__ __forceinline__ void for_near(const SceneConst& sc, const DeviceState& st, int i,
                                         float out_thr, F f) {
    const float xi = st.x32[i], zi = st.z32[i];
    const float si = fabsf(xi) + fabsf(zi);
    const int cnt = st.nb_count[i];
    for (int base = 0; base < cnt; base += 128) {
        const int m = min(128, cnt - base);
        unsigned long long lo = 0ull, hi = 0ull;
        for (int t = 0; t < m; t++) {
            const int j = st.nb[static_cast<int64_t>(base + t) * sc.n + i];
            if (!surely_out(xi, zi, si, st.x32[j], st.z32[j], out_thr)) {
                if (t < 64) lo |= 1ull << t;
                else hi |= 1ull << (t - 64);
            }
        }
        while (lo | hi) {
            int t;
            if (lo) {
                t = __ffsll(static_cast<long long>(lo)) - 1;
                lo &= lo - 1ull;
            } else {
                t = 63 + __ffsll(static_cast<long long>(hi));
                hi &= hi - 1ull;
            }
            f(st.nb[static_cast<int64_t>(base + t) * sc.n + i]);
        }
    }
}

// for_near for three-dimensional scenes (surely_out3 on x32, y32, z32).
template <class F>
__device__ __forceinline__ void for_near3(const SceneConst& sc, const DeviceState& st, int i,
                                          float out_thr, F f) {
    const float xi = st.x32[i], yi = st.y32[i], zi = st.z32[i];
    const float si = (fabsf(xi) + fabsf(yi)) + fabsf(zi);
    const int cnt = st.nb_count[i];
    for (int base = 0; base < cnt; base += 128) {
        const int m = min(128, cnt - base);
        unsigned long long lo = 0ull, hi = 0ull;
        for (int t = 0; t < m; t++) {
            const int j = st.nb[static_cast<int64_t>(base + t) * sc.n + i];
            if (!surely_out3(xi, yi, zi, si, st.x32[j], st.y32[j], st.z32[j], out_thr)) {
                if (t < 64) lo |= 1ull << t;
                else hi |= 1ull << (t - 64);
            }
        }
        while (lo | hi) {
            int t;
            if (lo) {
                t = __ffsll(static_cast<long long>(lo)) - 1;
                lo &= lo - 1ull;
            } else {
                t = 63 + __ffsll(static_cast<long long>(hi));
                hi &= hi - 1ull;
            }
            f(st.nb[static_cast<int64_t>(base + t) * sc.n + i]);
        }
    }
}

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

// PPE row of particle i.
__device__ __forceinline__ int ppe_row(const DeviceState& st, int i) { return st.row_of ? st.row_of[i] : i; }

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

// Block size of the neighbour walks (a thread per particle, 60-90 registers): small blocks
// fill an SM's register file in finer steps and leave a shorter tail of partly idle SMs
// than 256-thread blocks, whose launch of a few hundred blocks is barely over one wave.
constexpr int kWalkBlock = 64;

inline int grid_for(int64_t n, int block = kBlock) {
    return static_cast<int>((n + block - 1) / block);
}

// ------------------------------------------- programmatic dependent launch
// The solver's kernel chains are short kernels back to back; launched with programmatic
// stream serialization, a kernel's blocks are scheduled while its predecessor drains.
// Every kernel launched that way starts with pdl_begin(): it waits until the predecessor
// grid has completed and its writes are visible (griddepcontrol.wait), then lets its own
// successor start launching (griddepcontrol.launch_dependents).  Both are no-ops for a
// kernel launched without the attribute.
__device__ __forceinline__ void pdl_begin() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
// A kernel may read, before pdl_begin(), what no kernel still running can write: data
// fixed for the whole solve (matrix, cycle planes, row ranges) and what kernels two or
// more launches back wrote (every kernel of a chain waits for its predecessor before it
// lets its own successor launch, so those have completed and flushed).  Such loads then
// overlap the predecessor's tail instead of following it.

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<Args&&>(args)...);
}

// ------------------------------------------------------ launchers (host side)
// grid.cu
void launch_bucket(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
void launch_cell_sort(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
void launch_neighbors(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
// PPE row order from the sorted cells (no-op for a batch); returns the kernels launched.
int launch_rows(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
void launch_status_counters_reset(DevStatus* st, cudaStream_t s);
// FP32 position copies of particles [first, first + count) (count < 0: to the end)
void launch_positions_f32(const SceneConst& sc, const DeviceState& st, cudaStream_t s, int first = 0,
                          int count = -1);
// stages.cu
void launch_set_dt(const SceneConst& sc, const DeviceState& st, double dt, cudaStream_t s);
void launch_cfl_dt(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
void launch_density(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
void launch_error_correction(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
void launch_density_variation(const SceneConst& sc, const DeviceState& st, double* out,
                              cudaStream_t s);
void launch_explicit(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
// density + ECS (when flagged) + explicit accelerations in one neighbour walk; then the
// explicit move (the second loop of ComputeExplicitForces)
void launch_pre_pressure(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
void launch_explicit_update(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
void launch_save_x(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
void launch_set_ppe(const SceneConst& sc, const DeviceState& st, bool want_fp32, cudaStream_t s);
// the second number density and the PPE assembly in one neighbour walk (SPP method set:
// the assembly then needs no neighbour density); same launch count as launch_set_ppe
bool density_ppe_fusable(const SceneConst& sc);
void launch_density_set_ppe(const SceneConst& sc, const DeviceState& st, bool want_fp32, cudaStream_t s);
void launch_assign_pressure(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
// the explicit pressure of every particle from its number density; sets *ok (the solve
// flag the later stages test) to 1 when given
void launch_explicit_pressure(const SceneConst& sc, const DeviceState& st, int32_t* ok, cudaStream_t s);
// the second number density and the explicit pressure in one walk, caching W(r, r_e) for
// launch_pressure_gradient_cached (one launch)
void launch_density_explicit_pressure(const SceneConst& sc, const DeviceState& st, int32_t* ok,
                                      cudaStream_t s);
// the midpoint gradient, or with MPS_FLAG_GC the corrected one (two walks of each row)
void launch_pressure_gradient(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
// the same reading the weights launch_density_set_ppe or launch_density_explicit_pressure
// cached (positions unchanged since)
void launch_pressure_gradient_cached(const SceneConst& sc, const DeviceState& st, bool spp_sums, cudaStream_t s);
void launch_dynamic_stabilize(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
// part 2 of the CFL step (dt from the max |u|^2 a launch before it gathered)
void launch_cfl_dt_finish(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
// dim3.cu: the stages of a three-dimensional scene (same names and counts as above)
void launch_search3(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
void launch_cfl_dt3(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
void launch_density3(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
void launch_error_correction3(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
void launch_density_variation3(const SceneConst& sc, const DeviceState& st, double* out, cudaStream_t s);
void launch_explicit3(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
void launch_save_x3(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
void launch_set_ppe3(const SceneConst& sc, const DeviceState& st, bool want_fp32, cudaStream_t s);
void launch_pressure_gradient3(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
void launch_dynamic_stabilize3(const SceneConst& sc, const DeviceState& st, cudaStream_t s);
// the PPE layout kernels (stages.cu) after a row assembly: chunk sizes, offsets, SELL sort
void launch_ppe_layout(const SceneConst& sc, const DeviceState& st, bool want_fp32, cudaStream_t s);
// kernels the PPE assembly's layout step launches (direct rows skip the scan and the sort)
int set_ppe_launches(const DeviceState& st);
constexpr int kLaunchesSearch3 = 3;
// scan.cu
int scan_scratch_ints(int m);
void launch_exclusive_scan(const int* in, int* out, int m, int* scratch, cudaStream_t s);
// number of kernels each launcher issues (for the launch counter)
constexpr int kLaunchesSearch = 3, kLaunchesDensity = 1, kLaunchesEcs = 1, kLaunchesExplicit = 2,
              kLaunchesSaveX = 1, kLaunchesSetPpe = 6, kLaunchesAssign = 1, kLaunchesGradient = 2,
              kLaunchesDs = 2, kLaunchesDt = 1, kLaunchesCfl = 2, kLaunchesPrePressure = 1,
              kLaunchesExplicitUpdate = 1;

}  // namespace mpsgb

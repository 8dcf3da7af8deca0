// learned.cuh - the learned warm start and preconditioner scale of the PPE solve.
//
// A per-particle MLP 16 -> 64 -> 64 -> 64 -> 2 (GELU) maps neighbour-weighted features
// of the step to
//   out0: the part of the solution error that the first preconditioned CG step
//         c = alpha0 M r0 misses, in units of sigma (RMS of the Jacobi-scaled initial
//         residual): the initial guess becomes x0 = p_prev + c + sigma * out0 (a network
//         with zero output starts the solve one preconditioned step ahead);
//   out1: the scale s = 1 + 0.25 tanh(out1) in (0.75, 1.25) of the particle's Jacobi
//         term inside the multigrid preconditioner (positive: the preconditioner stays
//         definite; the band keeps the damping where the method is insensitive to it).
// Inference runs on the tensor cores (tcgen05, BF16 operands, FP32 accumulators in
// TMEM); training runs in FP32 with hand-written forward/backward kernels and Adam.
//
// Weight blob (FP32, kMlpBlobFloats): feature mean[16], feature std[16], W1[64][16], b1[64],
// W2[64][64], b2[64], W3[64][64], b3[64], W4[2][64], b4[2] (W[out][in]).
// Training sample (FP32, kMlpSampleFloats): features[16], target y, Jacobi term g
// (both in units of sigma); loss (out0 - y)^2 + (y - s g)^2 with s as above.
#pragma once

#include "mg.cuh"

namespace mpsgb {

constexpr int kMlpIn = 16, kMlpHidden = 64, kMlpOut = 2;
constexpr int kMlpOffMu = 0, kMlpOffSd = 16, kMlpOffW1 = 32;
constexpr int kMlpOffB1 = kMlpOffW1 + kMlpHidden * kMlpIn;
constexpr int kMlpOffW2 = kMlpOffB1 + kMlpHidden;
constexpr int kMlpOffB2 = kMlpOffW2 + kMlpHidden * kMlpHidden;
constexpr int kMlpOffW3 = kMlpOffB2 + kMlpHidden;
constexpr int kMlpOffB3 = kMlpOffW3 + kMlpHidden * kMlpHidden;
constexpr int kMlpOffW4 = kMlpOffB3 + kMlpHidden;
constexpr int kMlpOffB4 = kMlpOffW4 + kMlpOut * kMlpHidden;
constexpr int kMlpBlobFloats = kMlpOffB4 + kMlpOut;  // 9570
constexpr int kMlpParams = kMlpBlobFloats - kMlpOffW1;  // trainable (mean/std fixed)
constexpr int kMlpSampleFloats = kMlpIn + 2;
constexpr float kMlpScaleRange = 0.25f;  // s = 1 + kMlpScaleRange tanh(out1)

// Per-solve learned state on the device.
struct LearnedOps {
    int32_t n = 0;
    const void* packed = nullptr;  // tensor-core weight image (mlp_pack_weights)
    float* feat = nullptr;         // n x 16 raw features
    float* out = nullptr;          // n x 2 network outputs
    float* scale = nullptr;        // n preconditioner scales
    float* coarse = nullptr;       // n first preconditioned step c = alpha0 M r0
    float* sample = nullptr;       // n x 18 last step's training samples
    int32_t* active = nullptr;     // n 1 for PPE rows the solve acts on
    double* sigma = nullptr;       // [0] sigma, [1] partial scratch count
    double* partials = nullptr;    // per-block partial sums
    uint32_t* counter = nullptr;   // last-block ticket
    int32_t* error = nullptr;      // tensor-core wait timed out (1), cleared by each solve
    const WaitLimits* limits = nullptr;  // the handle's wait bounds (null: defaults)
    float4* q4 = nullptr;          // n per-particle quantities averaged over neighbours
    float2* q2 = nullptr;
    double* x0d = nullptr;         // n FP64 copy of the assembled initial guess
    // scene: rho l0^2 (pressure and source scales), n0 of the Laplacian radius, the
    // interior lattice diagonal and row length of the PPE
    double rho_l02 = 0, rho = 0, n0 = 0, a_ref = 0;
    float len_ref = 1;
    const double *nd = nullptr, *n_wo_spp = nullptr, *ecs = nullptr, *p = nullptr;
    const int32_t* type = nullptr;
    const int32_t* particle_of = nullptr;  // PPE row -> particle (null: the same index)
    const StepScalars* step = nullptr;
    const float* dinv0 = nullptr;  // the multigrid's omega_0 / a_ii
    uint32_t flags = 0;
};

// Bytes of the tensor-core weight image; builds it from an FP32 blob (host).
size_t mlp_packed_bytes();
void mlp_pack_weights(const float* blob, void* image);

// The step's features (after the assembly, the initial residual r0 in o.r32, the first
// preconditioner application u0 = M r0 in o.u32 and its step size alpha0 in S):
// raw features, c = alpha0 u0, sigma.
void launch_learned_features(const LearnedOps& L, const CgOperands& o, const CgScalars* S,
                             cudaStream_t s);
// its two kernels: per-particle quantities (need r0 only), then the per-row features
// (need the first preconditioned step)
void launch_learned_q(const LearnedOps& L, const CgOperands& o, const CgScalars* S, cudaStream_t s);
void launch_learned_feature_rows(const LearnedOps& L, const CgOperands& o, const CgScalars* S, cudaStream_t s);
// Network inference on the tensor cores: out = MLP(features).  The residual features
// (8, 9, 10) are divided by sigma[0] (sigma null: used as given).
void launch_mlp_infer(const void* packed, const float* feat, int n, const double* sigma,
                      float* out, int32_t* error, cudaStream_t s, const WaitLimits* limits = nullptr);
// The whole learned start of a solve: r0 (FP64, into o.r32 with S as scratch scalars),
// u0 = M r0 without learned scales, the CG step size alpha0 of u0, features, and with
// `infer` the network, the warm start and the scales.
void learned_prep(const LearnedOps& L, const CgOperands& o, const MgHierarchy& mg, CgScalars* S,
                  bool infer, cudaStream_t s);
int learned_prep_launches(const MgHierarchy& mg, bool infer);
// Warm start and scales from the outputs: x += c + sigma out0 on active rows; scale.
void launch_learned_apply(const LearnedOps& L, const CgOperands& o, const CgScalars* S,
                          cudaStream_t s);
// Training samples of the solved step (x holds the solution).
void launch_learned_targets(const LearnedOps& L, const CgOperands& o, const CgScalars* S,
                            cudaStream_t s);
cudaError_t mlp_prepare_device();

// FP32 training: loss and gradient of `n` samples (partials per block, then summed in
// a fixed order); Adam step.
struct MlpTrainer {
    int64_t cap = 0;
    float* samples = nullptr;   // cap x 18
    float* w = nullptr;         // blob
    float* m = nullptr;         // Adam moments (kMlpBlobFloats each)
    float* v = nullptr;
    float* grad = nullptr;      // kMlpBlobFloats
    float* partials = nullptr;  // blocks x (kMlpParams + 1)
    double* loss = nullptr;
    int blocks_cap = 0;
};
int mlp_train_blocks(int64_t n);
void launch_mlp_loss_grad(const MlpTrainer& T, const float* samples, int64_t n, cudaStream_t s);
void launch_mlp_adam(const MlpTrainer& T, float lr, int step, cudaStream_t s);
cudaError_t mlp_train_prepare_device();

}  // namespace mpsgb

#pragma once
// Learned block-Jacobi correction for the mixed-form PCG.
//
// Per camera c, a 3-layer MLP (inputs 49 -> 128 -> 128 -> 45; BF16 weights,
// FP32 accumulation on the tensor cores, FP32 master weights for training)
// maps features of the damped diagonal block S_cc to a lower-triangular factor
// F_c with positive diagonal. The preconditioner block becomes
//   M_c = (L_c F_c F_c^T L_c^T)^-1,   L_c = chol(S_cc),
// which is SPD for any network output and equals block-Jacobi when F_c = I
// (a zero last layer). Parametrisation of the 45 outputs o:
//   F_ij = 0.5 tanh(o_ij) (i > j),   F_ii = exp(0.5 tanh(o_ii)).
// Features (in the Jacobi-scaled space S^ = D^-1/2 S_cc D^-1/2, padded to 64):
//   [0,36)  off-diagonal S^_ij, i > j (row order)
//   [36,45) S_ii / (U_ii + lambda max(U_ii, 1e-12))   (share of the diagonal left after
//           eliminating the points)
//   45 log1p(observations of c) / 10, 46 log1p(sum over c's observations of (track length - 1)) / 15,
//   47 mean track length / 10, 48 log10(lambda) / 10.
// Training loss per camera (the block's step error in its own norm):
//   l = (y - x*)^T S^ (y - x*) / (x*^T S^ x*),  y = M^_c g^_c,
// with g the Schur right-hand side and x* the exact (dense FP64) step, both in
// the scaled space.

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

namespace gba {

class Solver;

constexpr int kMlpIn = 64;   // 49 features padded for the K = 16 MMA steps
constexpr int kMlpH = 128;
constexpr int kMlpOut = 48;  // 45 outputs padded to a multiple of 16
constexpr int kMlpUsedIn = 49;
constexpr int kMlpUsedOut = 45;

// Flat FP32 parameter vector: W1[128x64] b1[128] W2[128x128] b2[128] W3[48x128] b3[48].
constexpr long long kMlpParams =
    1ll * kMlpH * kMlpIn + kMlpH + 1ll * kMlpH * kMlpH + kMlpH + 1ll * kMlpOut * kMlpH + kMlpOut;

class Mlp {
public:
    Mlp(int capacity, uint64_t seed);               // random init, zero last layer
    Mlp(const std::string& path, int capacity);     // load a saved model
    // Inference only (forward): a saved model whose parameters, BF16 weights
    // and activations are allocated stream-ordered on `stream` (the device's
    // memory pool: no driver allocation or device-wide synchronisation per
    // solve) and uploaded on that stream; training calls throw.
    Mlp(const std::string& path, cudaStream_t stream);
    ~Mlp();
    Mlp(const Mlp&) = delete;
    Mlp& operator=(const Mlp&) = delete;

    void save(const std::string& path) const;
    void get_params(float* host) const;
    void set_params(const float* host);
    int capacity() const { return cap_; }
    void ensure_capacity(int B);

    // out[B x 48] (FP32) = network(feat[B x 64]); device pointers.
    void forward(const float* feat, int B, float* out, cudaStream_t s);
    // Forward + loss + backward on a batch (device pointers: Shat, Lhat packed
    // lower 45 per sample, g and x 9 per sample). Gradients kept for adam_step;
    // returns the mean loss. If baseline_loss is non-null it receives the mean
    // loss of F = I (plain block-Jacobi) on the same batch.
    double loss_grad(const float* feat, const double* Shat, const double* Lhat, const double* g, const double* x,
                     int B, cudaStream_t s, double* baseline_loss = nullptr);
    void grads(float* host) const;  // flat gradient of the last loss_grad
    void adam_step(float lr, float beta1, float beta2, float eps, cudaStream_t s);

    float* params_dev() const { return p_; }

private:
    void alloc();
    void refresh_bf16(cudaStream_t s);
    void require_training() const;
    int cap_ = 0;
    cudaStream_t pool_stream_ = nullptr;  // inference mode: allocations are stream-ordered on this stream
    bool inference_ = false;
    std::vector<float> host_params_;      // inference mode: the uploaded parameters (kept until the copy ends)
    long long step_ = 0;
    float* p_ = nullptr;   // FP32 masters (flat)
    float* g_ = nullptr;   // gradients (flat)
    float* m_ = nullptr;   // Adam moments
    float* v_ = nullptr;
    void* wb_ = nullptr;   // BF16 copies of W1, W2, W3
    float* h1_ = nullptr;  // activations [cap x 128]
    float* h2_ = nullptr;
    float* o_ = nullptr;   // [cap x 48]
    float* do_ = nullptr;
    float* dh2_ = nullptr;
    float* dh1_ = nullptr;
    double* loss_ = nullptr;  // [cap x 2] per-sample loss, baseline loss
};

class LearnedPreconditioner {
public:
    // The model's buffers are allocated stream-ordered on the solver's stream.
    LearnedPreconditioner(const std::string& path, cudaStream_t stream);
    ~LearnedPreconditioner();
    // Replaces the block-Jacobi factors in s.Pfac_ by the corrected factors
    // L_c F_c; S_cc (s.Sdiag_) and the factors must be current.
    void correct_factors(Solver& s, double lambda);

private:
    Mlp mlp_;
    cudaStream_t stream_;
    float* feat_ = nullptr;
    float* out_ = nullptr;
    int cap_ = 0;
};

// Per-camera features of the current damped diagonal blocks (s.Sdiag_) into
// feat[C x 64] (device).
void mlp_features(Solver& s, double lambda, float* feat);

}  // namespace gba

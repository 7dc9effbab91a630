#pragma once
// Learned coarse-space correction of the block-Jacobi preconditioner (mixed-form PCG).
//
// Block-Jacobi PCG on the reduced camera system converges slowly because of a
// handful of very small eigenvalues of the Jacobi-preconditioned S: the
// 7-dimensional similarity gauge of bundle adjustment (global rotation,
// translation, scale: only the LM damping holds it) and a few soft
// rotation/translation/focal modes. No block-diagonal correction reaches them
// (they are global), so the learned part is a low-rank correction: per camera
// c, a 3-layer MLP (inputs 58 -> 128 -> 128 -> 81; BF16 weights, FP32
// accumulation on the tensor cores, FP32 master weights for training) maps the
// camera's features to its 9 x kCoarse rows Z_c of a coarse basis Z (9C x
// kCoarse). The preconditioner is the balancing two-level form
//   M = P^T B^-1 P + Z E^-1 Z^T,   P = I - S Z E^-1 Z^T,   E = Z^T S Z,
// with B the block-Jacobi blocks: SPD for any Z of full rank, and B^-1 itself
// (block-Jacobi) when the coarse solve is disabled (E not SPD).
// Output parametrisation: Z_c(i, j) = o[9 i + j] * unit_i, unit = 1 except the
// focal-length row (f_c), so that every output is O(1).
// Features (padded to 64):
//   [0,36)  off-diagonal entries of the Jacobi-scaled block D^-1/2 S_cc D^-1/2, i > j (row order)
//   [36,45) S_ii / (U_ii + lambda max(U_ii, 1e-12))
//   45 log1p(observations of c) / 10, 46 log1p(sum over c's observations of (track length - 1)) / 15,
//   47 mean track length / 10, 48 log10(lambda) / 10,
//   [49,52) 3 x angle-axis, [52,55) translation / 2, 55 (f - 500) / 100, 56 10 k1, 57 100 k2.
// Training objective (train_preconditioner.py): the share of the lowest
// eigenvectors of the block-Jacobi-preconditioned S (from systems the plain
// solver assembles) that lies outside span(B^T Z).

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

namespace gba {

class Solver;

constexpr int kMlpIn = 64;   // 58 features padded for the K = 16 MMA steps
constexpr int kMlpH = 128;
constexpr int kCoarse = 9;   // coarse basis columns
constexpr int kMlpOut = 96;  // 81 outputs padded to a multiple of 16
constexpr int kMlpUsedIn = 58;
constexpr int kMlpUsedOut = 9 * kCoarse;

// Flat FP32 parameter vector: W1[128x64] b1[128] W2[128x128] b2[128] W3[96x128] b3[96].
constexpr long long kMlpParams =
    1ll * kMlpH * kMlpIn + kMlpH + 1ll * kMlpH * kMlpH + kMlpH + 1ll * kMlpOut * kMlpH + kMlpOut;

class Mlp {
public:
    Mlp(int capacity, uint64_t seed);               // random init (He; small last layer), zero biases
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

    // out[B x 96] (FP32) = network(feat[B x 64]); device pointers. Keeps the
    // hidden activations for a following backward() on the same batch.
    void forward(const float* feat, int B, float* out, cudaStream_t s);
    // Gradient of a loss w.r.t. the parameters, given its gradient dO[B x 96]
    // w.r.t. the outputs of the last forward() on feat (device pointers).
    // Gradients kept for adam_step.
    void backward(const float* feat, const float* dO, int B, cudaStream_t s);
    void grads(float* host) const;  // flat gradient of the last backward
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
    float* dh2_ = nullptr;
    float* dh1_ = nullptr;
};

class LearnedPreconditioner {
public:
    // The model's buffers are allocated stream-ordered on the solver's stream.
    LearnedPreconditioner(const std::string& path, cudaStream_t stream);
    ~LearnedPreconditioner();
    // The coarse basis Z (kCoarse columns of 9C, column-major, FP64) at the
    // solver's current cameras; S_cc (s.Sdiag_) must be current.
    void coarse_basis(Solver& s, double lambda, double* Z);

private:
    Mlp mlp_;
    cudaStream_t stream_;
    float* feat_ = nullptr;
    float* out_ = nullptr;
    int cap_ = 0;
};

// Per-camera features of the current damped diagonal blocks (s.Sdiag_) and
// cameras into feat[C x 64] (device).
void mlp_features(Solver& s, double lambda, float* feat);

}  // namespace gba

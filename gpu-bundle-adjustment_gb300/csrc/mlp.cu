// Learned coarse-space correction: MLP training and inference kernels.
//
//   GEMMs      mma.sync.m16n8k16 BF16 x BF16 -> FP32 (BF16 weights and
//              activations in shared memory, FP32 accumulation and storage);
//              one kernel with strided operand loads serves the forward
//              (X W^T), input-gradient (dY W) and weight-gradient (dY^T X) shapes.
//   backward   from the loss gradient w.r.t. the outputs (the loss, the
//              eigenvector share outside the coarse space, is a global function
//              of all cameras' outputs; the training script forms its gradient).
//   Adam       FP32 masters, BF16 copies refreshed after each step.
//   inference  features of S_cc and the camera -> MLP -> coarse basis rows Z_c.
// No reference counterpart (the reference has no iterative solver).

#include <cuda_bf16.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <random>
#include <stdexcept>
#include <vector>

#include "blocks.cuh"
#include "common.cuh"
#include "mlp.hpp"
#include "solver.hpp"

namespace gba {
namespace {

constexpr int kGT = 128;  // GEMM threads (4 warps, 2 x 2 warp grid of 32 x 32)
constexpr long long kW1 = 0, kB1 = kW1 + 1ll * kMlpH * kMlpIn, kW2 = kB1 + kMlpH, kB2 = kW2 + 1ll * kMlpH * kMlpH,
                    kW3 = kB2 + kMlpH, kB3 = kW3 + 1ll * kMlpOut * kMlpH;
constexpr long long kBf16Count = 1ll * kMlpH * kMlpIn + 1ll * kMlpH * kMlpH + 1ll * kMlpOut * kMlpH;

__device__ __forceinline__ __nv_bfloat16 to_bf16(float v) { return __float2bfloat16_rn(v); }
__device__ __forceinline__ __nv_bfloat16 to_bf16(__nv_bfloat16 v) { return v; }

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// C(m, n) = epilogue( sum_k A(m, k) B(k, n) ), A(m,k) = A[m*sam + k*sak],
// B(k,n) = B[k*sbk + n*sbn]; epilogue: + bias[n], ReLU, * (mask(m,n) > 0).
template <typename TA, typename TB>
__global__ void __launch_bounds__(kGT) gemm_bf16_kernel(int M, int N, int K, const TA* __restrict__ A, long long sam,
                                                       long long sak, const TB* __restrict__ B, long long sbk,
                                                       long long sbn, float* __restrict__ Cm, int ldc,
                                                       const float* __restrict__ bias, int relu,
                                                       const float* __restrict__ mask, int ldm) {
    __shared__ __align__(16) __nv_bfloat16 As[64][24];
    __shared__ __align__(16) __nv_bfloat16 Bs[64][24];
    const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int wm = (warp & 1) * 32, wn = (warp >> 1) * 32;
    const int g = lane >> 2, t = lane & 3;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.f;
    for (int k0 = 0; k0 < K; k0 += 16) {
        for (int idx = tid; idx < 64 * 16; idx += kGT) {
            const int r = idx >> 4, kk = idx & 15;
            const int k = k0 + kk;
            const int m = m0 + r, n = n0 + r;
            As[r][kk] = (m < M && k < K) ? to_bf16(A[m * sam + k * sak]) : __float2bfloat16_rn(0.f);
            Bs[r][kk] = (n < N && k < K) ? to_bf16(B[k * sbk + n * sbn]) : __float2bfloat16_rn(0.f);
        }
        __syncthreads();
        uint32_t af[2][4], bfr[4][2];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            const int r = wm + 16 * mt + g;
            af[mt][0] = *reinterpret_cast<const uint32_t*>(&As[r][2 * t]);
            af[mt][1] = *reinterpret_cast<const uint32_t*>(&As[r + 8][2 * t]);
            af[mt][2] = *reinterpret_cast<const uint32_t*>(&As[r][2 * t + 8]);
            af[mt][3] = *reinterpret_cast<const uint32_t*>(&As[r + 8][2 * t + 8]);
        }
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            const int r = wn + 8 * nt + g;
            bfr[nt][0] = *reinterpret_cast<const uint32_t*>(&Bs[r][2 * t]);
            bfr[nt][1] = *reinterpret_cast<const uint32_t*>(&Bs[r][2 * t + 8]);
        }
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) mma_bf16(acc[mt][nt], af[mt], bfr[nt]);
        __syncthreads();
    }
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int m = m0 + wm + 16 * mt + g + ((q >= 2) ? 8 : 0);
                const int n = n0 + wn + 8 * nt + 2 * t + (q & 1);
                if (m >= M || n >= N) continue;
                float v = acc[mt][nt][q];
                if (bias) v += bias[n];
                if (relu) v = fmaxf(v, 0.f);
                if (mask && !(mask[(long long)m * ldm + n] > 0.f)) v = 0.f;
                Cm[(long long)m * ldc + n] = v;
            }
}

template <typename TA, typename TB>
void gemm(int M, int N, int K, const TA* A, long long sam, long long sak, const TB* B, long long sbk, long long sbn,
          float* Cm, int ldc, const float* bias, bool relu, const float* mask, int ldm, cudaStream_t s) {
    dim3 grid(ceil_div(N, 64), ceil_div(M, 64));
    gemm_bf16_kernel<TA, TB><<<grid, kGT, 0, s>>>(M, N, K, A, sam, sak, B, sbk, sbn, Cm, ldc, bias, relu ? 1 : 0,
                                                  mask, ldm);
    GBA_LAUNCH_CHECK();
}

// db[n] = sum_m dY[m][n] (ordered, deterministic); one CTA per column.
__global__ void __launch_bounds__(256) colsum_kernel(const float* __restrict__ dY, int M, int ld, float* __restrict__ db) {
    __shared__ double sh[8];
    double s = 0.0;
    for (int m = threadIdx.x; m < M; m += 256) s += dY[(long long)m * ld + blockIdx.x];
    const double v = block_sum<256>(s, sh);
    if (threadIdx.x == 0) db[blockIdx.x] = static_cast<float>(v);
}

__global__ void to_bf16_kernel(const float* __restrict__ src, __nv_bfloat16* __restrict__ dst, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = __float2bfloat16_rn(src[i]);
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, long long n, float lr, float b1, float b2, float eps, float c1,
                            float c2) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

// ---- inference-side kernels

// Per-camera track statistics: observations, sum of (track length - 1), mean track length.
__global__ void camera_stats_kernel(const int* __restrict__ cam_off, const int* __restrict__ cam_slots,
                                    const int* __restrict__ s_pt, const int* __restrict__ pt_off, int C,
                                    float* __restrict__ stats) {
    const int c = blockIdx.x;
    __shared__ double sh[8];
    double s1 = 0.0;
    for (int i = cam_off[c] + threadIdx.x; i < cam_off[c + 1]; i += 256) {
        const int p = s_pt[cam_slots[i]];
        s1 += pt_off[p + 1] - pt_off[p];
    }
    const double sk = block_sum<256>(s1, sh);
    if (threadIdx.x == 0) {
        const double n = cam_off[c + 1] - cam_off[c];
        stats[3 * c] = static_cast<float>(log1p(n) / 10.0);
        stats[3 * c + 1] = static_cast<float>(log1p(sk - n) / 15.0);
        stats[3 * c + 2] = static_cast<float>(n > 0 ? sk / n / 10.0 : 0.0);
    }
}

// Per-camera FP64 kernels (features, factor correction): one camera per
// thread in warp-sized blocks, so that C cameras spread over all SMs' FP64
// pipes.
constexpr int kCamT = 32;

__global__ void features_kernel(const double* __restrict__ Sdiag, const double* __restrict__ U,
                                const float* __restrict__ stats, const double* __restrict__ cams, double lambda,
                                int C, float* __restrict__ feat) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    const double* S = Sdiag + 81ll * c;
    const double* Uc = U + 81ll * c;
    double isd[9];
    float* f = feat + 64ll * c;
    for (int i = 0; i < 9; ++i) {
        const double d = S[10 * i];
        isd[i] = d > 1e-300 ? 1.0 / sqrt(d) : 0.0;
        const double u = Uc[10 * i];
        const double ud = u + lambda * (u > 0.0 ? u : 1e-12);
        f[36 + i] = static_cast<float>(ud > 0.0 ? d / ud : 0.0);
    }
    int k = 0;
    for (int i = 1; i < 9; ++i)
        for (int j = 0; j < i; ++j) f[k++] = static_cast<float>(S[9 * i + j] * isd[i] * isd[j]);
    f[45] = stats[3 * c];
    f[46] = stats[3 * c + 1];
    f[47] = stats[3 * c + 2];
    f[48] = static_cast<float>(log10(lambda > 1e-300 ? lambda : 1e-300) / 10.0);
    const double* cam = cams + 9ll * c;
    for (int i = 0; i < 3; ++i) f[49 + i] = static_cast<float>(3.0 * cam[i]);
    for (int i = 0; i < 3; ++i) f[52 + i] = static_cast<float>(0.5 * cam[3 + i]);
    f[55] = static_cast<float>((cam[6] - 500.0) / 100.0);
    f[56] = static_cast<float>(10.0 * cam[7]);
    f[57] = static_cast<float>(100.0 * cam[8]);
    for (int i = kMlpUsedIn; i < 64; ++i) f[i] = 0.f;
}

// Coarse basis rows of camera c from the network outputs:
// Z[j][9c + i] = o[9 i + j] * unit_i (unit 1, the focal-length row f_c). A camera
// without observations gets zero rows: its block of S is decoupled (only the
// damping's 1e-12 floor), its right-hand side zero, and its step must stay zero.
__global__ void basis_kernel(const float* __restrict__ O, const double* __restrict__ cams,
                             const int* __restrict__ cam_off, int C, double* __restrict__ Z) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    const double f = cams[9ll * c + 6];
    const bool observed = cam_off[c + 1] > cam_off[c];
    const long long n = 9ll * C;
    for (int i = 0; i < 9; ++i) {
        const double unit = !observed ? 0.0 : i == 6 ? f : 1.0;
        for (int j = 0; j < kCoarse; ++j) Z[j * n + 9ll * c + i] = unit * O[static_cast<long long>(kMlpOut) * c + 9 * i + j];
    }
}

template <typename T>
T* dalloc(long long n) {
    T* p = nullptr;
    GBA_CUDA_CHECK(cudaMalloc(reinterpret_cast<void**>(&p), sizeof(T) * n));
    return p;
}

// Stream-ordered allocation from the device's memory pool (inference mode).
template <typename T>
T* palloc(long long n, cudaStream_t s) {
    T* p = nullptr;
    GBA_CUDA_CHECK(cudaMallocAsync(reinterpret_cast<void**>(&p), sizeof(T) * n, s));
    return p;
}

const char kMagic[8] = {'G', 'B', 'A', 'M', 'L', 'P', '0', '2'};

std::vector<float> read_model(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open model " + path);
    char magic[8];
    int32_t dims[3];
    f.read(magic, 8);
    f.read(reinterpret_cast<char*>(dims), sizeof dims);
    if (!f || std::memcmp(magic, kMagic, 8) != 0 || dims[0] != kMlpIn || dims[1] != kMlpH || dims[2] != kMlpOut)
        throw std::runtime_error("not a gba MLP model: " + path);
    std::vector<float> h(kMlpParams);
    f.read(reinterpret_cast<char*>(h.data()), sizeof(float) * kMlpParams);
    if (!f) throw std::runtime_error("truncated model " + path);
    return h;
}

}  // namespace

// ------------------------------------------------------------------ Mlp

void Mlp::alloc() {
    p_ = dalloc<float>(kMlpParams);
    g_ = dalloc<float>(kMlpParams);
    m_ = dalloc<float>(kMlpParams);
    v_ = dalloc<float>(kMlpParams);
    wb_ = dalloc<__nv_bfloat16>(kBf16Count);
    GBA_CUDA_CHECK(cudaMemset(g_, 0, sizeof(float) * kMlpParams));
    GBA_CUDA_CHECK(cudaMemset(m_, 0, sizeof(float) * kMlpParams));
    GBA_CUDA_CHECK(cudaMemset(v_, 0, sizeof(float) * kMlpParams));
    ensure_capacity(cap_);
}

void Mlp::ensure_capacity(int B) {
    if (B <= cap_ && h1_) return;
    cap_ = std::max(B, std::max(cap_, 1));
    if (inference_) {  // forward activations only
        for (float* q : {h1_, h2_})
            if (q) GBA_CUDA_CHECK(cudaFreeAsync(q, pool_stream_));
        h1_ = palloc<float>(1ll * cap_ * kMlpH, pool_stream_);
        h2_ = palloc<float>(1ll * cap_ * kMlpH, pool_stream_);
        return;
    }
    for (void* q : {static_cast<void*>(h1_), static_cast<void*>(h2_), static_cast<void*>(dh2_),
                    static_cast<void*>(dh1_)})
        if (q) cudaFree(q);
    h1_ = dalloc<float>(1ll * cap_ * kMlpH);
    h2_ = dalloc<float>(1ll * cap_ * kMlpH);
    dh2_ = dalloc<float>(1ll * cap_ * kMlpH);
    dh1_ = dalloc<float>(1ll * cap_ * kMlpH);
}

Mlp::Mlp(int capacity, uint64_t seed) : cap_(capacity) {
    alloc();
    std::vector<float> h(kMlpParams, 0.f);
    std::mt19937_64 rng(seed);
    std::normal_distribution<float> nd(0.f, 1.f);
    const float s1 = std::sqrt(2.f / kMlpUsedIn), s2 = std::sqrt(2.f / kMlpH);
    for (int r = 0; r < kMlpH; ++r)
        for (int c = 0; c < kMlpUsedIn; ++c) h[kW1 + 1ll * r * kMlpIn + c] = s1 * nd(rng);
    for (long long i = 0; i < 1ll * kMlpH * kMlpH; ++i) h[kW2 + i] = s2 * nd(rng);
    const float s3 = 0.1f * s2;  // a small random last layer: a full-rank basis to start from
    for (int r = 0; r < kMlpUsedOut; ++r)
        for (int c = 0; c < kMlpH; ++c) h[kW3 + 1ll * r * kMlpH + c] = s3 * nd(rng);
    set_params(h.data());
}

Mlp::Mlp(const std::string& path, int capacity) : cap_(capacity) {
    const std::vector<float> h = read_model(path);
    alloc();
    set_params(h.data());
}

Mlp::Mlp(const std::string& path, cudaStream_t stream)
    : pool_stream_(stream), inference_(true), host_params_(read_model(path)) {
    p_ = palloc<float>(kMlpParams, stream);
    wb_ = palloc<__nv_bfloat16>(kBf16Count, stream);
    GBA_CUDA_CHECK(cudaMemcpyAsync(p_, host_params_.data(), sizeof(float) * kMlpParams, cudaMemcpyHostToDevice,
                                   stream));
    refresh_bf16(stream);
}

void Mlp::require_training() const {
    if (inference_) throw std::logic_error("this MLP was loaded for inference only");
}

Mlp::~Mlp() {
    if (inference_) {
        for (void* q : {static_cast<void*>(p_), wb_, static_cast<void*>(h1_), static_cast<void*>(h2_)})
            if (q) cudaFreeAsync(q, pool_stream_);
        return;
    }
    for (void* q : {static_cast<void*>(p_), static_cast<void*>(g_), static_cast<void*>(m_), static_cast<void*>(v_), wb_,
                    static_cast<void*>(h1_), static_cast<void*>(h2_), static_cast<void*>(dh2_),
                    static_cast<void*>(dh1_)})
        if (q) cudaFree(q);
}

void Mlp::save(const std::string& path) const {
    std::vector<float> h(kMlpParams);
    get_params(h.data());
    std::ofstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot write model " + path);
    const int32_t dims[3] = {kMlpIn, kMlpH, kMlpOut};
    f.write(kMagic, 8);
    f.write(reinterpret_cast<const char*>(dims), sizeof dims);
    f.write(reinterpret_cast<const char*>(h.data()), sizeof(float) * kMlpParams);
    if (!f) throw std::runtime_error("write failed for " + path);
}

void Mlp::get_params(float* host) const {
    GBA_CUDA_CHECK(cudaMemcpy(host, p_, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost));
}

void Mlp::set_params(const float* host) {
    GBA_CUDA_CHECK(cudaMemcpy(p_, host, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice));
    refresh_bf16(nullptr);
    GBA_CUDA_CHECK(cudaStreamSynchronize(nullptr));
}

void Mlp::grads(float* host) const {
    require_training();
    GBA_CUDA_CHECK(cudaDeviceSynchronize());
    GBA_CUDA_CHECK(cudaMemcpy(host, g_, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost));
}

void Mlp::refresh_bf16(cudaStream_t s) {
    __nv_bfloat16* wb = static_cast<__nv_bfloat16*>(wb_);
    to_bf16_kernel<<<64, 256, 0, s>>>(p_ + kW1, wb, 1ll * kMlpH * kMlpIn);
    GBA_LAUNCH_CHECK();
    to_bf16_kernel<<<64, 256, 0, s>>>(p_ + kW2, wb + 1ll * kMlpH * kMlpIn, 1ll * kMlpH * kMlpH);
    GBA_LAUNCH_CHECK();
    to_bf16_kernel<<<64, 256, 0, s>>>(p_ + kW3, wb + 1ll * kMlpH * kMlpIn + 1ll * kMlpH * kMlpH, 1ll * kMlpOut * kMlpH);
    GBA_LAUNCH_CHECK();
}

void Mlp::forward(const float* feat, int B, float* out, cudaStream_t s) {
    ensure_capacity(B);
    const __nv_bfloat16* wb = static_cast<const __nv_bfloat16*>(wb_);
    const __nv_bfloat16* w1 = wb;
    const __nv_bfloat16* w2 = wb + 1ll * kMlpH * kMlpIn;
    const __nv_bfloat16* w3 = w2 + 1ll * kMlpH * kMlpH;
    // H1 = relu(X W1^T + b1): A = X [B x 64], B(k, n) = W1[n][k]
    gemm(B, kMlpH, kMlpIn, feat, kMlpIn, 1, w1, 1, kMlpIn, h1_, kMlpH, p_ + kB1, true, nullptr, 0, s);
    gemm(B, kMlpH, kMlpH, h1_, kMlpH, 1, w2, 1, kMlpH, h2_, kMlpH, p_ + kB2, true, nullptr, 0, s);
    gemm(B, kMlpOut, kMlpH, h2_, kMlpH, 1, w3, 1, kMlpH, out, kMlpOut, p_ + kB3, false, nullptr, 0, s);
}

void Mlp::backward(const float* feat, const float* dO, int B, cudaStream_t s) {
    require_training();
    if (B <= 0 || B > cap_) throw std::invalid_argument("backward: batch must be the last forward's (<= capacity)");
    const __nv_bfloat16* wb = static_cast<const __nv_bfloat16*>(wb_);
    const __nv_bfloat16* w2 = wb + 1ll * kMlpH * kMlpIn;
    const __nv_bfloat16* w3 = w2 + 1ll * kMlpH * kMlpH;
    // layer 3: dW3[n][k] = sum_m dO[m][n] H2[m][k]; db3; dH2 = (dO W3) * (H2 > 0)
    gemm(kMlpOut, kMlpH, B, dO, 1, kMlpOut, h2_, kMlpH, 1, g_ + kW3, kMlpH, nullptr, false, nullptr, 0, s);
    colsum_kernel<<<kMlpOut, 256, 0, s>>>(dO, B, kMlpOut, g_ + kB3);
    GBA_LAUNCH_CHECK();
    gemm(B, kMlpH, kMlpOut, dO, kMlpOut, 1, w3, kMlpH, 1, dh2_, kMlpH, nullptr, false, h2_, kMlpH, s);
    // layer 2
    gemm(kMlpH, kMlpH, B, dh2_, 1, kMlpH, h1_, kMlpH, 1, g_ + kW2, kMlpH, nullptr, false, nullptr, 0, s);
    colsum_kernel<<<kMlpH, 256, 0, s>>>(dh2_, B, kMlpH, g_ + kB2);
    GBA_LAUNCH_CHECK();
    gemm(B, kMlpH, kMlpH, dh2_, kMlpH, 1, w2, kMlpH, 1, dh1_, kMlpH, nullptr, false, h1_, kMlpH, s);
    // layer 1 (input features need no gradient)
    gemm(kMlpH, kMlpIn, B, dh1_, 1, kMlpH, feat, kMlpIn, 1, g_ + kW1, kMlpIn, nullptr, false, nullptr, 0, s);
    colsum_kernel<<<kMlpH, 256, 0, s>>>(dh1_, B, kMlpH, g_ + kB1);
    GBA_LAUNCH_CHECK();
}

void Mlp::adam_step(float lr, float beta1, float beta2, float eps, cudaStream_t s) {
    require_training();
    ++step_;
    const float c1 = 1.f - std::pow(beta1, static_cast<float>(step_));
    const float c2 = 1.f - std::pow(beta2, static_cast<float>(step_));
    adam_kernel<<<120, 256, 0, s>>>(p_, g_, m_, v_, kMlpParams, lr, beta1, beta2, eps, c1, c2);
    GBA_LAUNCH_CHECK();
    refresh_bf16(s);
}

// ------------------------------------------------------------------ solver side

void mlp_features(Solver& s, double lambda, float* feat) {
    if (!s.mlp_stats_.get()) {
        StreamAllocScope scope(s.stream_);
        s.mlp_stats_.alloc(3ull * s.C_);
        camera_stats_kernel<<<s.C_, 256, 0, s.stream_>>>(s.cam_off_.get(), s.cam_slots_.get(), s.s_pt_.get(),
                                                          s.pt_off_.get(), s.C_, s.mlp_stats_.get());
        GBA_LAUNCH_CHECK();
    }
    features_kernel<<<ceil_div(s.C_, kCamT), kCamT, 0, s.stream_>>>(s.Sdiag_.get(), s.U_.get(), s.mlp_stats_.get(),
                                                                 s.cams_.get(), lambda, s.C_, feat);
    GBA_LAUNCH_CHECK();
}

LearnedPreconditioner::LearnedPreconditioner(const std::string& path, cudaStream_t stream)
    : mlp_(path, stream), stream_(stream) {}

LearnedPreconditioner::~LearnedPreconditioner() {
    if (feat_) cudaFreeAsync(feat_, stream_);
    if (out_) cudaFreeAsync(out_, stream_);
}

void LearnedPreconditioner::coarse_basis(Solver& s, double lambda, double* Z) {
    if (cap_ < s.C_) {
        if (feat_) GBA_CUDA_CHECK(cudaFreeAsync(feat_, stream_));
        if (out_) GBA_CUDA_CHECK(cudaFreeAsync(out_, stream_));
        feat_ = palloc<float>(64ll * s.C_, stream_);
        out_ = palloc<float>(1ll * kMlpOut * s.C_, stream_);
        cap_ = s.C_;
    }
    mlp_features(s, lambda, feat_);
    cudaEvent_t ev = s.prof_start();
    mlp_.forward(feat_, s.C_, out_, s.stream_);
    s.prof_stop("mlp_forward", ev);
    basis_kernel<<<ceil_div(s.C_, kCamT), kCamT, 0, s.stream_>>>(out_, s.cams_.get(), s.cam_off_.get(), s.C_, Z);
    GBA_LAUNCH_CHECK();
}

Solver::~Solver() {
    prof_reset();
    delete model_;
    if (sync_ev_) cudaEventDestroy(sync_ev_);
}

void Solver::load_model(const std::string& path) {
    if (form_ == SolverForm::Plain) throw std::invalid_argument("the learned preconditioner needs a mixed form");
    if (path.empty()) throw std::invalid_argument("learned form: empty model path");
    auto* m = new LearnedPreconditioner(path, stream_);
    delete model_;
    model_ = m;
}

}  // namespace gba

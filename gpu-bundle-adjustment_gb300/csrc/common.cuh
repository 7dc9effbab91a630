#pragma once
// Shared device/host utilities: error handling, launch helpers and the
// deterministic reduction primitives used by every kernel in this library.

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>

namespace gba {

// Floats per camera of the FP32 camera-vector copies read by the point-side
// passes: 9 used, padded to 48 B so that a gather is two float4 and a float.
constexpr int kX32 = 12;

// The mixed forms' FP32 Jacobian rows are stored in component groups: the 18
// Jc components (row 0 then row 1 of the 2 x 9 camera block) as four float4
// planes and a float2 plane, Jc32[(q js + s) 4 + i] = Jc[4q + i] (q < 4) and
// Jc32[16 js + 2 s + i] = Jc[16 + i]; the 6 Jp components as a float4 plane
// and a float2 plane, Jp32[4 s + i] = Jp[i], Jp32[4 js + 2 s + i] = Jp[4 + i];
// js = the slot count rounded up to 32. A warp's access to one plane is 512 or
// 256 contiguous bytes, and a slot's rows are 7 vector accesses (the
// row-major 72- and 24-byte records cost 4x the L1 wavefronts).
inline long long jacobian_stride(long long E) { return (E + 31) / 32 * 32; }

__device__ __forceinline__ void store_jacobian_rows(float* __restrict__ Jc32, float* __restrict__ Jp32, long long js,
                                                    long long s, const float* J) {
    float4* c4 = reinterpret_cast<float4*>(Jc32);
#pragma unroll
    for (int q = 0; q < 4; ++q) c4[q * js + s] = make_float4(J[4 * q], J[4 * q + 1], J[4 * q + 2], J[4 * q + 3]);
    reinterpret_cast<float2*>(Jc32 + 16 * js)[s] = make_float2(J[16], J[17]);
    reinterpret_cast<float4*>(Jp32)[s] = make_float4(J[18], J[19], J[20], J[21]);
    reinterpret_cast<float2*>(Jp32 + 4 * js)[s] = make_float2(J[22], J[23]);
}
__device__ __forceinline__ void load_jc_rows(const float* __restrict__ Jc32, long long js, long long s, float* Jc) {
    const float4* c4 = reinterpret_cast<const float4*>(Jc32);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const float4 v = c4[q * js + s];
        Jc[4 * q] = v.x;
        Jc[4 * q + 1] = v.y;
        Jc[4 * q + 2] = v.z;
        Jc[4 * q + 3] = v.w;
    }
    const float2 v = reinterpret_cast<const float2*>(Jc32 + 16 * js)[s];
    Jc[16] = v.x;
    Jc[17] = v.y;
}
__device__ __forceinline__ void load_jp_rows(const float* __restrict__ Jp32, long long js, long long s, float* jp) {
    const float4 a = reinterpret_cast<const float4*>(Jp32)[s];
    const float2 b = reinterpret_cast<const float2*>(Jp32 + 4 * js)[s];
    jp[0] = a.x;
    jp[1] = a.y;
    jp[2] = a.z;
    jp[3] = a.w;
    jp[4] = b.x;
    jp[5] = b.y;
}

// Thrown by the host driver on CUDA failure (the C-ABI layer converts it to a
// status code; nothing throws across the ABI).
struct CudaError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

#define GBA_CUDA_CHECK(call)                                                            \
    do {                                                                                \
        cudaError_t err_ = (call);                                                      \
        if (err_ != cudaSuccess)                                                        \
            throw ::gba::CudaError(std::string("CUDA error at ") + __FILE__ + ":" +     \
                                   std::to_string(__LINE__) + ": " +                    \
                                   cudaGetErrorString(err_));                           \
    } while (0)

// Every kernel launch of this library is followed by GBA_LAUNCH_CHECK(), which
// also counts it (gba_launch_count() in the C ABI reports the total).
void count_launch();
unsigned long long launch_count();
#define GBA_LAUNCH_CHECK()                          \
    do {                                            \
        ::gba::count_launch();                      \
        GBA_CUDA_CHECK(cudaGetLastError());         \
    } while (0)

inline int ceil_div(long long a, long long b) { return static_cast<int>((a + b - 1) / b); }

// Number of SMs of the current device (152 on GB300), cached per process.
int device_sm_count();

#ifdef __CUDACC__
// Programmatic dependent launch (sm_90 and later). A kernel launched with the
// programmatic stream serialization attribute may start while the kernel
// before it in the stream is still finishing; pdl_wait() blocks until that
// kernel has completed and its memory is visible, so every chained kernel
// calls it before its first access to memory. pdl_trigger() lets the next
// chained kernel be scheduled now (it then waits in its own pdl_wait()). In a
// kernel launched without the attribute both are no-ops.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Deterministic block-wide sum of one double per thread. Fixed shuffle tree
// within each warp, then warp partials summed in warp order by warp 0.
// `shared` holds at least blockDim.x/32 doubles. Result valid in thread 0.
template <int kThreads>
__device__ __forceinline__ double block_sum(double v, double* shared) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) shared[warp] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int w = 0; w < kThreads / 32; ++w) r += shared[w];
    }
    __syncthreads();
    return r;
}

// The same for one float per thread: FP32 shuffle tree within each warp, the
// warp sums widened to FP64 and added in warp order by thread 0 (one FP64 add
// per warp: on GB300 the FP64 pipe is 1/64 of the FP32 one).
template <int kThreads>
__device__ __forceinline__ double block_sum_f(float v, double* shared) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) shared[warp] = static_cast<double>(v);
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int w = 0; w < kThreads / 32; ++w) r += shared[w];
    }
    __syncthreads();
    return r;
}

// Deterministic sum of part[0, n) by one block of kThreads threads (result in
// thread 0): four interleaved accumulators per thread keep four independent
// loads in flight instead of one dependent load per add; they are combined in
// a fixed order, then summed over the block.
template <int kThreads>
__device__ __forceinline__ double wide_block_sum(const double* __restrict__ part, int n, double* shared) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int i = threadIdx.x;
    for (; i + 3 * kThreads < n; i += 4 * kThreads) {
        s0 += part[i];
        s1 += part[i + kThreads];
        s2 += part[i + 2 * kThreads];
        s3 += part[i + 3 * kThreads];
    }
    if (i < n) s0 += part[i];
    if (i + kThreads < n) s1 += part[i + kThreads];
    if (i + 2 * kThreads < n) s2 += part[i + 2 * kThreads];
    return block_sum<kThreads>((s0 + s1) + (s2 + s3), shared);
}

template <int kThreads>
__device__ __forceinline__ unsigned long long block_sum_u64(unsigned long long v,
                                                            unsigned long long* shared) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) shared[warp] = v;
    __syncthreads();
    unsigned long long r = 0;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int w = 0; w < kThreads / 32; ++w) r += shared[w];
    }
    __syncthreads();
    return r;
}

// Huber loss of a squared residual norm s (delta <= 0: no loss): rho(s) and
// the square root of its weight rho'(s) = min(1, delta / sqrt(s)), the factor
// that scales an observation's residual and Jacobian rows.
__device__ __forceinline__ double robust_rho(double s, double delta) {
    return (delta > 0.0 && s > delta * delta) ? 2.0 * delta * sqrt(s) - delta * delta : s;
}
__device__ __forceinline__ double robust_sqrt_weight(double s, double delta) {
    return (delta > 0.0 && s > delta * delta) ? sqrt(delta / sqrt(s)) : 1.0;
}
__device__ __forceinline__ float robust_sqrt_weight(float s, float delta) {
    return (delta > 0.f && s > delta * delta) ? sqrtf(delta / sqrtf(s)) : 1.f;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
#endif

}  // namespace gba

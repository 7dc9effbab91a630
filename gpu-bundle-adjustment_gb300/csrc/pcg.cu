// Mixed form: the reduced camera system S dc = rhs is never formed.
//
//   S x   = U_lambda x - sum_p W_p V'_p^-1 W_p^T x,   W_e = Jc_e^T Jp_e
//   rhs   = bc - sum_p W_p V'_p^-1 bp_p
//
// computed implicitly from the per-slot FP32 Jacobian rows (Jc32, Jp32, slot
// order, component-major):
//   point pass   (slots sorted by point)  w_p = V'^-1 (a bp_p + sum_e Jp_e^T (Jc_e x_c)),
//                                         u_e = Jp_e w_p          (2 values per slot)
//   camera pass  (camera-major chunks)    partial_c = sum_e Jc_e^T u_e
//   finalize                              y = U_lambda x - sum partials   (or rhs = bc - ...)
// templated on the arithmetic type: FP32 inside PCG, float-float (ff.cuh) for
// the right-hand side and the refinement residual when the Schur target is
// tight. Chunk partials are summed in FP64 in a fixed order, so these products
// are deterministic. The right-hand side pass also produces the block-Jacobi
// diagonal-block sums (G = Jp V'^-1 Jp^T per slot, summed by the camera pass).
// The FP32 product inside PCG runs by default as one pass (schur_matvec_warp,
// schur_matvec_long): the point pass adds Jc_e^T u_e into per-camera
// accumulators with device atomics instead of storing u_e, so each slot's
// Jacobian rows are read once; its sums are then ordered only up to the
// atomics (gba_solver_set_matvec selects the two-pass product).
//
// Solve: iterative refinement (dc += e, r = rhs - S dc with float-float
// products, until ||r|| <= refine_tol ||rhs||) around inner block-Jacobi PCG
// solves on the FP32 operator; with refine_tol >= kLooseTol the right-hand side
// is FP32 and a converged inner solve is its own check. The block-Jacobi blocks
// are the 9x9 diagonal blocks S_cc (FP32 products, FP64 sums, FP64 Cholesky,
// explicit inverses); the learned form adds a coarse-space correction whose
// basis the MLP predicts (mlp.cu; the balancing two-level preconditioner
// below). The PCG vectors are FP32; its scalars and the sums of block
// partials are FP64, reduced in a fixed order; all PCG control scalars live on
// the device and the host polls a convergence flag after batches of
// iterations. The kernels of an iteration are chained with programmatic
// dependent launch. The last refinement check of a trial (float-float
// targets) runs the back-substitution's point pass, which the trial then
// reuses.
//
// No reference counterpart: the reference solves S densely on the host.

#include <cuda_bf16.h>

#include "blocks.cuh"
#include "common.cuh"
#include "ff.cuh"
#include "mlp.hpp"
#include "solver.hpp"

namespace gba {
namespace {

constexpr int kPT = 256;
constexpr int kCT = 128;
constexpr int kVT = 256;  // vector-kernel threads
constexpr int kCB = 32;   // thread-per-camera kernels: one warp per block spreads C cameras over the SMs
constexpr int kCamChunk = 1024;
constexpr int kCheck = 8;       // most PCG iterations launched between host checks of the convergence flag
constexpr long long kJudgeMin = 8;  // inner iterations a judged solve needs to be decisive
constexpr int kJudgeAttempts = 2;    // indecisive judgements before block-Jacobi is kept for the solve
constexpr double kShortInnerTol = 1e-2;  // inner tolerances this loose end every solve in a few iterations
// The learned factors serve the solve only if they reach the judged inner
// tolerance in at most this fraction of block-Jacobi's iterations: on workload
// 5 at strict targets a 10% win on the judged system (18 vs 20 iterations)
// turned into 625 vs 472 iterations over the whole solve.
constexpr long long kLearnedWinNum = 4, kLearnedWinDen = 5;
constexpr double kLooseTol = 1e-3;   // refinement targets at or above this run the fast (FP32) path

constexpr int kUC = 32;        // cameras per block of the 9-threads-per-camera kernels
constexpr int kUT = 9 * kUC;   // their block size

// Device scalar slots (pcg_s_). Within one PCG iteration each slot is written
// by one kernel (block 0, thread 0) and read only by later kernels, except
// S_DONE, whose value every block of the writing kernel derives itself:
//   pcg_update         reads S_RZ;            writes S_RZPREV, S_ITERS (and S_DONE on breakdown)
//   pcg_direction      reads S_RZPREV, S_ITERS; writes S_RZ, S_RR, S_BETA, S_DONE
enum { S_RZ = 0, S_ALPHA, S_BETA, S_RR, S_BB, S_DONE, S_ITERS, S_TOL2, S_NORM, S_RZPREV, S_BTX0, S_BTX1 };

using ffa::ff;

// Arithmetic of the implicit product: FP32 (PCG) or float-float (right-hand
// side and refinement residual). The Jacobian records are FP32 either way and
// enter every product exactly.
template <typename T> __device__ __forceinline__ T zero();
template <> __device__ __forceinline__ float zero<float>() { return 0.f; }
template <> __device__ __forceinline__ ff zero<ff>() { return {0.f, 0.f}; }

// FP32 forms; the float-float overloads (ffa::madd, add, norm, shfl_up) are
// found by argument-dependent lookup.
__device__ __forceinline__ void madd(float& acc, float a, float b) { acc = fmaf(a, b, acc); }
__device__ __forceinline__ float add(float a, float b) { return a + b; }
__device__ __forceinline__ float norm(float a) { return a; }
__device__ __forceinline__ float shfl_up(float a, int d) { return __shfl_up_sync(0xffffffffu, a, d); }
__device__ __forceinline__ double as_double(float a) { return a; }
__device__ __forceinline__ double as_double(ff a) { return ffa::to_double(a); }
template <typename T> __device__ __forceinline__ T from_double(double d);
template <> __device__ __forceinline__ float from_double<float>(double d) { return static_cast<float>(d); }
template <> __device__ __forceinline__ ff from_double<ff>(double d) { return ffa::from_double(d); }
__device__ __forceinline__ float hi_of(float x) { return x; }
__device__ __forceinline__ float hi_of(ff x) { return x.hi; }
__device__ __forceinline__ ff to_ff(float x) { return {x, 0.f}; }
__device__ __forceinline__ ff to_ff(ff x) { return x; }
__device__ __forceinline__ float warp_total(float v) { return warp_sum(v); }
__device__ __forceinline__ ff warp_total(ff v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = ffa::add(v, ffa::shfl_xor(v, o));
    return v;
}

// V'^-1 of a point (6 packed): FP32 copy, or FP32 copy + low parts.
// A point's packed V'^-1 (6 floats, 24 B: 8-byte aligned) as three float2 loads.
__device__ __forceinline__ void load_vinv(const float* __restrict__ hi, const float* __restrict__, long long p,
                                          float* v) {
    const float2* h = reinterpret_cast<const float2*>(hi + 6 * p);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float2 t = h[k];
        v[2 * k] = t.x;
        v[2 * k + 1] = t.y;
    }
}
__device__ __forceinline__ void load_vinv(const float* __restrict__ hi, const float* __restrict__ lo, long long p,
                                          ff* v) {
    const float2* h = reinterpret_cast<const float2*>(hi + 6 * p);
    const float2* l = reinterpret_cast<const float2*>(lo + 6 * p);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float2 a = h[k], b = l[k];
        v[2 * k] = {a.x, b.x};
        v[2 * k + 1] = {a.y, b.y};
    }
}

// u_e: two values per slot (8 B in FP32, 16 B in float-float).
__device__ __forceinline__ void store_u(float* u, long long q, float a, float b) {
    reinterpret_cast<float2*>(u)[q] = make_float2(a, b);
}
__device__ __forceinline__ void store_u(ff* u, long long q, ff a, ff b) {
    reinterpret_cast<float4*>(u)[q] = make_float4(a.hi, a.lo, b.hi, b.lo);
}
__device__ __forceinline__ void load_u(const float* u, long long q, float& a, float& b) {
    const float2 v = reinterpret_cast<const float2*>(u)[q];
    a = v.x;
    b = v.y;
}
__device__ __forceinline__ void load_u(const ff* u, long long q, ff& a, ff& b) {
    const float4 v = reinterpret_cast<const float4*>(u)[q];
    a = {v.x, v.y};
    b = {v.z, v.w};
}

// The nine entries of a camera's x: FP32 copies are padded to kX32 floats per
// camera and read as two float4 and a float (a third of the gather requests of
// nine scalar loads); float-float copies are dense (9 per camera).
__device__ __forceinline__ void load_x(const float* __restrict__ x, int c, float* xv) {
    const float* xc = x + static_cast<long long>(kX32) * c;
    const float4 a = reinterpret_cast<const float4*>(xc)[0], b = reinterpret_cast<const float4*>(xc)[1];
    xv[0] = a.x; xv[1] = a.y; xv[2] = a.z; xv[3] = a.w;
    xv[4] = b.x; xv[5] = b.y; xv[6] = b.z; xv[7] = b.w;
    xv[8] = xc[8];
}
__device__ __forceinline__ void load_x(const ff* __restrict__ x, int c, ff* xv) {
#pragma unroll
    for (int k = 0; k < 9; ++k) xv[k] = x[9ll * c + k];
}

// 8-byte asynchronous global -> shared copy (no register holds the data) and
// the wait for this thread's copies.
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// J = [Jc(18), Jp(6)] of slot s (component planes, stride js)
__device__ __forceinline__ void load_j(const float* __restrict__ Jc32, const float* __restrict__ Jp32, long long js,
                                       long long s, float* J) {
    load_jc_rows(Jc32, js, s, J);
    load_jp_rows(Jp32, js, s, J + 18);
}
__device__ __forceinline__ void load_jp(const float* __restrict__ Jp32, long long js, long long s, float* jp) {
    load_jp_rows(Jp32, js, s, jp);
}

// w = V'^-1 z (3x3 packed symmetric)
template <typename T>
__device__ __forceinline__ void apply_vinv(const T* v, T z0, T z1, T z2, T& w0, T& w1, T& w2) {
    z0 = norm(z0);
    z1 = norm(z1);
    z2 = norm(z2);
    w0 = zero<T>();
    w1 = zero<T>();
    w2 = zero<T>();
    madd(w0, v[0], z0);
    madd(w0, v[1], z1);
    madd(w0, v[3], z2);
    madd(w1, v[1], z0);
    madd(w1, v[2], z1);
    madd(w1, v[4], z2);
    madd(w2, v[3], z0);
    madd(w2, v[4], z1);
    madd(w2, v[5], z2);
    w0 = norm(w0);
    w1 = norm(w1);
    w2 = norm(w2);
}

// u = Jp w (Jp row-major 2x3, FP32)
template <typename T>
__device__ __forceinline__ void jp_times(const float* jp, T w0, T w1, T w2, T& u0, T& u1) {
    u0 = zero<T>();
    u1 = zero<T>();
    madd(u0, jp[0], w0);
    madd(u0, jp[1], w1);
    madd(u0, jp[2], w2);
    madd(u1, jp[3], w0);
    madd(u1, jp[4], w1);
    madd(u1, jp[5], w2);
}

// G = Jp V'^-1 Jp^T (2x2 symmetric, FP32: g00, g01, g11) of one slot, for the
// block-Jacobi diagonal blocks; vi: the point's FP32 V'^-1 (packed lower).
__device__ __forceinline__ float4 jp_vinv_jpt(const float* j, const float* vi) {
    float m[6];
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const float a0 = j[3 * r], a1 = j[3 * r + 1], a2 = j[3 * r + 2];
        m[3 * r] = a0 * vi[0] + a1 * vi[1] + a2 * vi[3];
        m[3 * r + 1] = a0 * vi[1] + a1 * vi[2] + a2 * vi[4];
        m[3 * r + 2] = a0 * vi[3] + a1 * vi[4] + a2 * vi[5];
    }
    return make_float4(m[0] * j[0] + m[1] * j[1] + m[2] * j[2], m[0] * j[3] + m[1] * j[4] + m[2] * j[5],
                       m[3] * j[3] + m[4] * j[4] + m[5] * j[5], 0.f);
}

// y += Jc^T u for one slot (FP32, device-memory atomics: two float4 and one
// float into a 12-float accumulator of the slot's camera). The slot's Jacobian
// rows are re-read here; the point pass loaded them moments before, so they
// come from L1 or L2, not HBM.
template <typename T>
__device__ __forceinline__ void accumulate_jct_u(const float* __restrict__ Jc32, long long js, long long s, T u0,
                                                 T u1, T* y) {
    if constexpr (sizeof(T) == 4) {
        float Jc[18];
        load_jc_rows(Jc32, js, s, Jc);
        float r[9];
#pragma unroll
        for (int t = 0; t < 9; ++t) r[t] = fmaf(Jc[t], u0, Jc[9 + t] * u1);
        atomicAdd(reinterpret_cast<float4*>(y), make_float4(r[0], r[1], r[2], r[3]));
        atomicAdd(reinterpret_cast<float4*>(y) + 1, make_float4(r[4], r[5], r[6], r[7]));
        atomicAdd(y + 8, r[8]);
    }
}

// Back-substitution outputs of the point pass (kBack): dp = V'^-1 (bp - W^T dc),
// trial points, and per-chunk partials of the gain denominator's point terms.
struct BacksubOut {
    const double* V;
    const double* pts;
    float2 lambda;  // float-float
    double* dp;
    double* tpts;
    float2* tpts_ff;  // float-float split of the trial points (for the trial cost)
    double* part;
};

// Point pass of the implicit product. xt: the camera vector in the arithmetic
// type (an FP32 copy inside PCG, a float-float copy of dc in refinement), or
// null for the right-hand side; z = sum_e Jp^T Jc x + a bp. V'^-1 from its FP32
// copy (+ low parts for float-float). u is written at the slot's camera-major
// position so that the camera pass reads it contiguously. With kBack (a = -1,
// xt = dc): w = -dp, and the pass ends with the back-substitution outputs
// (and, when u_cm is given, also stores u = Jp w = -Jp dp).
// kRhs: the right-hand side instantiation (xt = null, a = 1, also G).
template <typename T, bool kBack = false, bool kRhs = false, bool kAcc = false>
__global__ void __launch_bounds__(kPT, sizeof(T) == 4 ? (kBack ? 6 : 8) : (kBack ? 4 : 5)) schur_point_pass(const int4* __restrict__ prange, const int* __restrict__ pchunk, const int* __restrict__ pt_off,
                                                       const int* __restrict__ s_cam, const int* __restrict__ s_pt,
                                                       const int* __restrict__ cam_pos, const float* __restrict__ Jc32,
                                                       const float* __restrict__ Jp32, long long js,
                                                       const float* __restrict__ vinv_hi,
                                                       const float* __restrict__ vinv_lo,
                                                       const double* __restrict__ bp, const T* __restrict__ xt,
                                                       double a, T* __restrict__ u_cm,
                                                       const double* __restrict__ done, BacksubOut bk,
                                                       float4* __restrict__ g_cm) {
    __shared__ T seg[kPT][3];  // warp-segment partial sums, at each segment's last slot
    __shared__ T wsh[kPT][3];
    __shared__ __align__(16) float vsh[kPT][6];  // FP32 V'^-1 of the chunk's points
    __shared__ float bsum[kPT / 32][2];
    __shared__ double bout[kBack ? 9 * kPT : 1];  // back-substitution outputs of the chunk's points
    if (done && *done != 0.0) return;
    const int chunk = blockIdx.x;
    // the chunk's points and slots: one 16-byte load from the range table (a
    // null table: the chunk starts and the CSR offsets)
    int p0, p1, s0, s1;
    if (prange) {
        const int4 rg = prange[chunk];
        p0 = rg.x, p1 = rg.y, s0 = rg.z, s1 = rg.w;
    } else {
        p0 = pchunk[chunk], p1 = pchunk[chunk + 1];
        s0 = pt_off[p0], s1 = pt_off[p1];
    }
    const int my_p = p0 + threadIdx.x;
    const int lane = threadIdx.x & 31;
    int my_b = 0, my_e = 0;
    if (my_p < p1) {
        my_b = pt_off[my_p];
        my_e = pt_off[my_p + 1];
    }
    T z0 = zero<T>(), z1 = zero<T>(), z2 = zero<T>();
    // V'^-1 of the chunk's (contiguous) points, fetched first so that its
    // latency overlaps the slot loads and the scan. FP32: the block copies it
    // into shared memory with asynchronous 8-byte copies (coalesced runs
    // instead of six strided loads per owner, no registers held), waited for
    // before the first barrier that precedes its use (233 instead of 269 us per
    // matvec on 8.8M observations). Float-float, and the back-substitution
    // (where the copy measured slower: 329-364 against 306 us): the owners
    // load it.
    constexpr bool kSharedVinv = sizeof(T) == 4 && !kBack;
    T vinv[6];
    if constexpr (kSharedVinv) {
        const float2* src = reinterpret_cast<const float2*>(vinv_hi + 6ll * p0);
        float2* dst = reinterpret_cast<float2*>(&vsh[0][0]);
        for (int i = threadIdx.x; i < 3 * (p1 - p0); i += kPT) cp_async8(dst + i, src + i);
    } else {
        if (my_p < p1) load_vinv(vinv_hi, vinv_lo, my_p, vinv);
    }
    // Single-pass chunks (the usual case) keep the slot's Jp, point and
    // camera-major position in registers for the u phase.
    const bool single = (s1 - s0) <= kPT;
    float jp[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    int key = -1;  // point of the slot (slots past the chunk end share key -1, value 0)
    long long q = 0;
    if (!kRhs && xt) {
        for (int base = s0; base < s1; base += kPT) {
            const int s = base + threadIdx.x;
            T v0 = zero<T>(), v1 = zero<T>(), v2 = zero<T>();
            key = -1;
            if (s < s1) {
                key = s_pt[s];
                const int cam = s_cam[s];
                q = cam_pos[s];  // kAcc: the slot's accumulator
                float J[24];
                load_j(Jc32, Jp32, js, s, J);
#pragma unroll
                for (int k = 0; k < 6; ++k) jp[k] = J[18 + k];
                T xv[9];
                load_x(xt, cam, xv);
                T t0 = zero<T>(), t1 = zero<T>();
#pragma unroll
                for (int k = 0; k < 9; ++k) {
                    madd(t0, J[k], xv[k]);
                    madd(t1, J[9 + k], xv[k]);
                }
                t0 = norm(t0);
                t1 = norm(t1);
                madd(v0, J[18], t0);
                madd(v0, J[21], t1);
                madd(v1, J[19], t0);
                madd(v1, J[22], t1);
                madd(v2, J[20], t0);
                madd(v2, J[23], t1);
            }
            // inclusive segmented scan over the warp (slots of a point are contiguous)
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const T u0 = shfl_up(v0, d);
                const T u1 = shfl_up(v1, d);
                const T u2 = shfl_up(v2, d);
                const int kd = __shfl_up_sync(0xffffffffu, key, d);
                if (lane >= d && kd == key) {
                    v0 = add(v0, u0);
                    v1 = add(v1, u1);
                    v2 = add(v2, u2);
                }
            }
            const int knext = __shfl_down_sync(0xffffffffu, key, 1);
            if (lane == 31 || knext != key) {
                seg[threadIdx.x][0] = v0;
                seg[threadIdx.x][1] = v1;
                seg[threadIdx.x][2] = v2;
            }
            if constexpr (kSharedVinv) cp_async_wait_all();
            __syncthreads();
            // owner: add the point's warp-segment partials of this pass, warps in order
            if (my_p < p1) {
                const int b = max(my_b, base) - base, e = min(my_e, base + kPT) - base;
                for (int w = b >> 5; b < e && w <= (e - 1) >> 5; ++w) {
                    const int t = min(e - 1, 32 * w + 31);
                    z0 = add(z0, seg[t][0]);
                    z1 = add(z1, seg[t][1]);
                    z2 = add(z2, seg[t][2]);
                }
            }
            __syncthreads();
        }
    }
    if (kRhs && single) {
        // right-hand side: the slot's point, Jp and camera-major position are
        // loaded before the barrier, so their latency overlaps the owners' bp
        // and V'^-1 loads
        const int s = s0 + threadIdx.x;
        if (s < s1) {
            key = s_pt[s];
            q = cam_pos[s];
            load_jp(Jp32, js, s, jp);
        }
    }
    if constexpr (kSharedVinv) {
        if (kRhs || !xt || s0 == s1) {  // no slot pass has waited and synchronised
            cp_async_wait_all();
            __syncthreads();
        }
        if (my_p < p1) {
#pragma unroll
            for (int k = 0; k < 6; ++k) vinv[k] = vsh[threadIdx.x][k];
        }
    }
    T w0 = zero<T>(), w1 = zero<T>(), w2 = zero<T>();
    if (my_p < p1) {
        if (a != 0.0) {
            z0 = add(z0, from_double<T>(a * bp[3ll * my_p]));
            z1 = add(z1, from_double<T>(a * bp[3ll * my_p + 1]));
            z2 = add(z2, from_double<T>(a * bp[3ll * my_p + 2]));
        }
        apply_vinv(vinv, z0, z1, z2, w0, w1, w2);
        wsh[threadIdx.x][0] = w0;
        wsh[threadIdx.x][1] = w1;
        wsh[threadIdx.x][2] = w2;
        if (!kSharedVinv && g_cm) {
#pragma unroll
            for (int k = 0; k < 6; ++k) vsh[threadIdx.x][k] = hi_of(vinv[k]);
        }
    }
    if constexpr (kBack) {
        // dp (FP64 out), trial points (FP64 sum), and the gain denominator's
        // point terms dp_k (lambda max(V_kk, 1e-12) dp_k + bp_k) in float-float;
        // V and bp hold FP32 sums here, exact in FP32.
        ff den = {0.f, 0.f};
        if (my_p < p1) {
            const long long p = my_p;
            const ff lam = {bk.lambda.x, bk.lambda.y};
            const ff d[3] = {ffa::neg(to_ff(w0)), ffa::neg(to_ff(w1)), ffa::neg(to_ff(w2))};
            const int diag[3] = {0, 2, 5};
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const double dk = ffa::to_double(d[k]);
                const double tp = bk.pts[3 * p + k] + dk;
                const ff tf = ffa::from_double(tp);
                bout[3 * threadIdx.x + k] = dk;
                bout[3 * kPT + 3 * threadIdx.x + k] = tp;
                reinterpret_cast<float2*>(bout + 6 * kPT)[3 * threadIdx.x + k] = make_float2(tf.hi, tf.lo);
                const float vk = static_cast<float>(bk.V[6 * p + diag[k]]);
                ff t = {static_cast<float>(bp[3 * p + k]), 0.f};
                ffa::madd(t, ffa::mul(lam, ff{vk > 0.f ? vk : 1e-12f, 0.f}), d[k]);
                ffa::madd(den, ffa::norm(t), d[k]);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) den = ffa::add(den, ffa::shfl_xor(den, o));
        if (lane == 0) {
            bsum[threadIdx.x >> 5][0] = den.hi;
            bsum[threadIdx.x >> 5][1] = den.lo;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
#pragma unroll
            for (int w = 0; w < kPT / 32; ++w) t += static_cast<double>(bsum[w][0]) + static_cast<double>(bsum[w][1]);
            bk.part[chunk] = t;
        }
        // dp, trial points and their split for the chunk's contiguous points, as
        // contiguous runs
        const int np = p1 - p0;
        const float2* bff = reinterpret_cast<const float2*>(bout + 6 * kPT);
        for (int i = threadIdx.x; i < 3 * np; i += kPT) {
            bk.dp[3ll * p0 + i] = bout[i];
            bk.tpts[3ll * p0 + i] = bout[3 * kPT + i];
            bk.tpts_ff[3ll * p0 + i] = bff[i];
        }
        if (!u_cm) return;
    }
    __syncthreads();
    // u_e = Jp_e w_p for every slot of the chunk, stored camera-major (kAcc:
    // Jc_e^T u_e added into the camera's accumulators)
    if (single) {
        if (s0 + static_cast<int>(threadIdx.x) < s1) {
            T u0, u1;
            jp_times(jp, wsh[key - p0][0], wsh[key - p0][1], wsh[key - p0][2], u0, u1);
            if constexpr (kAcc)
                accumulate_jct_u(Jc32, js, s0 + threadIdx.x, u0, u1, u_cm + static_cast<long long>(kX32) * q);
            else
                store_u(u_cm, q, u0, u1);
            if (g_cm) g_cm[q] = jp_vinv_jpt(jp, vsh[key - p0]);
        }
        return;
    }
    for (int s = s0 + threadIdx.x; s < s1; s += kPT) {
        const int p = s_pt[s];
        float j[6];
        load_jp(Jp32, js, s, j);
        T u0, u1;
        jp_times(j, wsh[p - p0][0], wsh[p - p0][1], wsh[p - p0][2], u0, u1);
        if constexpr (kAcc) {
            accumulate_jct_u(Jc32, js, s, u0, u1, u_cm + static_cast<long long>(kX32) * cam_pos[s]);
        } else {
            const long long q = cam_pos[s];
            store_u(u_cm, q, u0, u1);
            if (g_cm) g_cm[q] = jp_vinv_jpt(j, vsh[p - p0]);
        }
    }
}

// Camera pass: partial_c = sum over the chunk's camera-major positions of Jc^T u
// (Jc from the camera records J32c = [Jc(18), r(2)] per position; both contiguous).
// Partials at part[kStride * chunk]. kDiag (the right-hand side pass): also the
// chunk's part of sum Jc^T G Jc (lower triangle, 45, FP32 sums) from the slots'
// G = Jp V'^-1 Jp^T, at part[54 chunk + 9 ..], for the block-Jacobi blocks.
template <typename T, bool kDiag = false>
__global__ void __launch_bounds__(kCT) schur_camera_pass(const int* __restrict__ cchunk_begin,
                                                        const int* __restrict__ cchunk_cam,
                                                        const int* __restrict__ cam_off,
                                                        const float* __restrict__ J32c, const T* __restrict__ u_cm,
                                                        double* __restrict__ part, const double* __restrict__ done,
                                                        const float4* __restrict__ g_cm) {
    constexpr int kStride = kDiag ? 54 : 9;
    __shared__ double wpart[kCT / 32][9];
    __shared__ float dpart[kDiag ? kCT / 32 : 1][kDiag ? 45 : 1];
    float dacc[kDiag ? 45 : 1];
    if constexpr (kDiag) {
#pragma unroll
        for (int i = 0; i < 45; ++i) dacc[i] = 0.f;
    }
    if (done && *done != 0.0) return;
    const int k = blockIdx.x;
    const int b = cchunk_begin[k], c = cchunk_cam[k];
    const int e = min(b + kCamChunk, cam_off[c + 1]);
    T acc[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) acc[i] = zero<T>();
    for (int i = b + threadIdx.x; i < e; i += kCT) {
        const float4* q = reinterpret_cast<const float4*>(J32c + 20ll * i);
        float Jc[20];
#pragma unroll
        for (int t = 0; t < 5; ++t) {
            const float4 v = q[t];
            Jc[4 * t] = v.x;
            Jc[4 * t + 1] = v.y;
            Jc[4 * t + 2] = v.z;
            Jc[4 * t + 3] = v.w;
        }
        T u0, u1;
        load_u(u_cm, i, u0, u1);
#pragma unroll
        for (int t = 0; t < 9; ++t) {
            madd(acc[t], Jc[t], u0);
            madd(acc[t], Jc[9 + t], u1);
        }
        if constexpr (kDiag) {
            const float4 g = g_cm[i];
            float H0[9], H1[9];  // G Jc
#pragma unroll
            for (int t = 0; t < 9; ++t) {
                H0[t] = g.x * Jc[t] + g.y * Jc[9 + t];
                H1[t] = g.y * Jc[t] + g.z * Jc[9 + t];
            }
            int idx = 0;
#pragma unroll
            for (int a = 0; a < 9; ++a)
#pragma unroll
                for (int bb = 0; bb <= a; ++bb) {
                    dacc[idx] += Jc[a] * H0[bb] + Jc[9 + a] * H1[bb];
                    ++idx;
                }
        }
    }
    // Warp sums in the arithmetic type (FP32 shuffles stay off GB300's narrow
    // FP64 pipe); the four warp partials are added in FP64.
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int t = 0; t < 9; ++t) {
        const T v = warp_total(acc[t]);
        if (lane == 0) wpart[warp][t] = as_double(v);
    }
    if constexpr (kDiag) {
#pragma unroll
        for (int t = 0; t < 45; ++t) {
            const float v = warp_sum(dacc[t]);
            if (lane == 0) dpart[warp][t] = v;
        }
    }
    __syncthreads();
    if (threadIdx.x < 9) {
        double v = 0.0;
#pragma unroll
        for (int w = 0; w < kCT / 32; ++w) v += wpart[w][threadIdx.x];
        part[static_cast<long long>(kStride) * k + threadIdx.x] = v;
    }
    if constexpr (kDiag) {
        if (threadIdx.x >= 32 && threadIdx.x < 32 + 45) {
            const int t = threadIdx.x - 32;
            double v = 0.0;
#pragma unroll
            for (int w = 0; w < kCT / 32; ++w) v += static_cast<double>(dpart[w][t]);
            part[54ll * k + 9 + t] = v;
        }
    }
}

// ---------------------------------------------------------------- one-pass product, warp chunks
// The one-pass FP32 product over warp chunks: whole points packed into runs of
// at most 32 slots, one run per warp, so that a point's slots never leave the
// warp. Per slot (lane): v = Jp^T (Jc x), an inclusive segmented scan over the
// warp gives each point's sum z at its last lane, which applies V'^-1 (loaded
// by every lane of the point up front: one request per point), and every lane
// takes its point's w from that lane (match + shuffle); then Jc^T (Jp w) goes
// into the slot's accumulator. No shared memory and no barrier: a warp's
// chain is loads -> shuffles -> atomics, and 64 warps per SM hide it. Points
// with more than 32 observations go through the chunked point pass.
constexpr int kMWarps = 8;  // warps per CTA
__global__ void __launch_bounds__(32 * kMWarps) schur_matvec_warp(
    const int2* __restrict__ wchunk, int n_wchunk, const int* __restrict__ s_cam, const int* __restrict__ s_pt,
    const int* __restrict__ acc_id, const float* __restrict__ Jc32, const float* __restrict__ Jp32, long long js,
    const float* __restrict__ vinv, const float* __restrict__ x, float* __restrict__ y,
    const double* __restrict__ done) {
    pdl_wait();  // x: the previous kernel's direction
    if (done && *done != 0.0) return;
    const int wid = blockIdx.x * kMWarps + (threadIdx.x >> 5);
    if (wid >= n_wchunk) return;  // whole warps leave together
    const int lane = threadIdx.x & 31;
    const int2 r = wchunk[wid];
    const int s = r.x + lane;
    const bool has = s < r.y;
    int key = -1, aid = 0;
    float J[24], vi[6];
    float v0 = 0.f, v1 = 0.f, v2 = 0.f;
    if (has) {
        key = s_pt[s];
        aid = acc_id[s];
        float xv[9];
        load_x(x, s_cam[s], xv);
        load_vinv(vinv, nullptr, key, vi);
        load_j(Jc32, Jp32, js, s, J);
        float t0 = 0.f, t1 = 0.f;
#pragma unroll
        for (int c = 0; c < 9; ++c) {
            t0 = fmaf(J[c], xv[c], t0);
            t1 = fmaf(J[9 + c], xv[c], t1);
        }
        v0 = fmaf(J[18], t0, J[21] * t1);
        v1 = fmaf(J[19], t0, J[22] * t1);
        v2 = fmaf(J[20], t0, J[23] * t1);
    }
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const float u0 = __shfl_up_sync(0xffffffffu, v0, d);
        const float u1 = __shfl_up_sync(0xffffffffu, v1, d);
        const float u2 = __shfl_up_sync(0xffffffffu, v2, d);
        const int kd = __shfl_up_sync(0xffffffffu, key, d);
        if (lane >= d && kd == key) {
            v0 += u0;
            v1 += u1;
            v2 += u2;
        }
    }
    float w0 = 0.f, w1 = 0.f, w2 = 0.f;
    if (has) apply_vinv(vi, v0, v1, v2, w0, w1, w2);  // meaningful at the point's last lane
    const unsigned grp = __match_any_sync(0xffffffffu, key);
    const int last = 31 - __clz(grp);
    w0 = __shfl_sync(0xffffffffu, w0, last);
    w1 = __shfl_sync(0xffffffffu, w1, last);
    w2 = __shfl_sync(0xffffffffu, w2, last);
    if (has) {
        float u0, u1;
        jp_times(J + 18, w0, w1, w2, u0, u1);
        float q[9];
#pragma unroll
        for (int c = 0; c < 9; ++c) q[c] = fmaf(J[c], u0, J[9 + c] * u1);
        float* ya = y + static_cast<long long>(kX32) * aid;
        atomicAdd(reinterpret_cast<float4*>(ya), make_float4(q[0], q[1], q[2], q[3]));
        atomicAdd(reinterpret_cast<float4*>(ya) + 1, make_float4(q[4], q[5], q[6], q[7]));
        atomicAdd(ya + 8, q[8]);
    }
}

// The one-pass product for points with 33 to 256 observations: a CTA takes
// a list of such points (not consecutive) whose slots total at most 256 and
// lays them out as one virtual chunk (thread t: the t-th slot of the list);
// the point pass of schur_point_pass follows, then Jc^T u into the slot's
// accumulator. lchunk[k] = {first entry in lpts, entries}.
__global__ void __launch_bounds__(kPT) schur_matvec_long(
    const int2* __restrict__ lchunk, const int* __restrict__ lpts, const int* __restrict__ pt_off,
    const int* __restrict__ s_cam, const int* __restrict__ acc_id, const float* __restrict__ Jc32,
    const float* __restrict__ Jp32, long long js, const float* __restrict__ vinv, const float* __restrict__ x,
    float* __restrict__ y, const double* __restrict__ done) {
    constexpr int kMaxPts = kPT / 33 + 1;  // points of more than 32 slots in 256
    __shared__ int pb[kMaxPts + 1], ps[kMaxPts], pid[kMaxPts];  // virtual begin, first real slot, point
    __shared__ float seg[kPT][3];
    __shared__ float wsh[kMaxPts][3];
    pdl_wait();
    if (done && *done != 0.0) return;
    const int2 lc = lchunk[blockIdx.x];
    const int tid = threadIdx.x, lane = tid & 31;
    if (tid < lc.y) {  // the list's points in parallel, then their prefix
        const int p = lpts[lc.x + tid];
        const int o0 = pt_off[p], o1 = pt_off[p + 1];
        pid[tid] = p;
        ps[tid] = o0;
        pb[tid + 1] = o1 - o0;
    }
    __syncwarp();
    if (tid == 0) {
        pb[0] = 0;
        for (int j = 1; j <= lc.y; ++j) pb[j] += pb[j - 1];
    }
    __syncthreads();
    const int n = pb[lc.y];
    int key = -1, aid = 0;
    long long sl = 0;
    float J[24];
    float v0 = 0.f, v1 = 0.f, v2 = 0.f;
    if (tid < n) {
        int j = 0;
        while (tid >= pb[j + 1]) ++j;
        key = j;
        sl = ps[j] + (tid - pb[j]);
        aid = acc_id[sl];
        float xv[9];
        load_x(x, s_cam[sl], xv);
        load_j(Jc32, Jp32, js, sl, J);
        float t0 = 0.f, t1 = 0.f;
#pragma unroll
        for (int c = 0; c < 9; ++c) {
            t0 = fmaf(J[c], xv[c], t0);
            t1 = fmaf(J[9 + c], xv[c], t1);
        }
        v0 = fmaf(J[18], t0, J[21] * t1);
        v1 = fmaf(J[19], t0, J[22] * t1);
        v2 = fmaf(J[20], t0, J[23] * t1);
    }
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const float u0 = __shfl_up_sync(0xffffffffu, v0, d);
        const float u1 = __shfl_up_sync(0xffffffffu, v1, d);
        const float u2 = __shfl_up_sync(0xffffffffu, v2, d);
        const int kd = __shfl_up_sync(0xffffffffu, key, d);
        if (lane >= d && kd == key) {
            v0 += u0;
            v1 += u1;
            v2 += u2;
        }
    }
    const int knext = __shfl_down_sync(0xffffffffu, key, 1);
    if (lane == 31 || knext != key) {
        seg[tid][0] = v0;
        seg[tid][1] = v1;
        seg[tid][2] = v2;
    }
    __syncthreads();
    if (tid < lc.y) {  // owner of point entry tid: its warp segments in order
        const int b = pb[tid], e = pb[tid + 1];
        float z0 = 0.f, z1 = 0.f, z2 = 0.f;
        for (int w = b >> 5; w <= (e - 1) >> 5; ++w) {
            const int q = min(e - 1, 32 * w + 31);
            z0 += seg[q][0];
            z1 += seg[q][1];
            z2 += seg[q][2];
        }
        float vi[6], w0, w1, w2;
        load_vinv(vinv, nullptr, pid[tid], vi);
        apply_vinv(vi, z0, z1, z2, w0, w1, w2);
        wsh[tid][0] = w0;
        wsh[tid][1] = w1;
        wsh[tid][2] = w2;
    }
    __syncthreads();
    if (tid < n) {
        float u0, u1;
        jp_times(J + 18, wsh[key][0], wsh[key][1], wsh[key][2], u0, u1);
        float q[9];
#pragma unroll
        for (int c = 0; c < 9; ++c) q[c] = fmaf(J[c], u0, J[9 + c] * u1);
        float* ya = y + static_cast<long long>(kX32) * aid;
        atomicAdd(reinterpret_cast<float4*>(ya), make_float4(q[0], q[1], q[2], q[3]));
        atomicAdd(reinterpret_cast<float4*>(ya) + 1, make_float4(q[4], q[5], q[6], q[7]));
        atomicAdd(ya + 8, q[8]);
    }
}

__device__ __forceinline__ double damped_u_row_dot(const double* __restrict__ Uc, int k, double lambda,
                                                   const double* __restrict__ xc) {
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 9; ++j) s += Uc[9 * k + j] * xc[j];
    const double d = Uc[10 * k];
    return s + lambda * (d > 0.0 ? d : 1e-12) * xc[k];
}

__device__ __forceinline__ double chunk_sum(const int* __restrict__ cam_chunk_off, const double* __restrict__ part,
                                            int c, int k, int stride = 9) {
    double s = 0.0;
    for (int q = cam_chunk_off[c]; q < cam_chunk_off[c + 1]; ++q) s += part[static_cast<long long>(stride) * q + k];
    return s;
}

// rhs = bc - sum partials; partial ||rhs||^2 per block.
// rhs = bc - (chunk partials of the right-hand side pass), also copied to the
// refinement's reference residual ref_r; dc (the refined step) starts at zero.
__global__ void __launch_bounds__(kVT) rhs_finalize(const int* __restrict__ cam_chunk_off,
                                                   const double* __restrict__ part, const double* __restrict__ bc,
                                                   int C, double* __restrict__ rhs, double* __restrict__ ref_r,
                                                   double* __restrict__ dc, double* __restrict__ red) {
    __shared__ double sh[kVT / 32];
    const int i = blockIdx.x * kVT + threadIdx.x;
    double v = 0.0;
    if (i < 9 * C) {
        v = bc[i] - chunk_sum(cam_chunk_off, part, i / 9, i % 9, 54);  // the right-hand side pass writes 54 per chunk
        rhs[i] = v;
        ref_r[i] = v;
        dc[i] = 0.0;
    }
    const double t = block_sum<kVT>(v * v, sh);
    if (threadIdx.x == 0) red[blockIdx.x] = t;
}

// r = rhs - (U_lambda x - sum partials); partial ||r||^2 per block (FP64 refinement residual).
__global__ void __launch_bounds__(kVT) residual_finalize(const int* __restrict__ cam_chunk_off,
                                                        const double* __restrict__ part, const double* __restrict__ U,
                                                        double lambda, const double* __restrict__ x,
                                                        const double* __restrict__ rhs, int C, double* __restrict__ r,
                                                        double* __restrict__ red) {
    __shared__ double sh[kVT / 32];
    const int i = blockIdx.x * kVT + threadIdx.x;
    double v = 0.0;
    if (i < 9 * C) {
        const int c = i / 9, k = i % 9;
        const double Sx = damped_u_row_dot(U + 81ll * c, k, lambda, x + 9ll * c) - chunk_sum(cam_chunk_off, part, c, k);
        v = rhs[i] - Sx;
        r[i] = v;
    }
    const double t = block_sum<kVT>(v * v, sh);
    if (threadIdx.x == 0) red[blockIdx.x] = t;
}

// Row k of the damped camera block times the camera's FP32 direction: Ul holds
// U_lambda = U + lambda max(diag U, 1e-12) in FP32 (81 per camera), p32 the
// padded direction (kX32 per camera).
__device__ __forceinline__ float damped_u_row_dot32(const float* __restrict__ Ul, const float* __restrict__ pc, int k) {
    const float* u = Ul + 9 * k;
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < 9; ++j) s = fmaf(u[j], pc[j], s);
    return s;
}

// q = S p (finalize of the two-pass product) and partial p.q: FP32 vectors,
// the chunk partials summed in FP64.
__global__ void __launch_bounds__(kVT) pcg_q_finalize(const int* __restrict__ cam_chunk_off,
                                                     const double* __restrict__ part, const float* __restrict__ Ul,
                                                     const float* __restrict__ p32, int C, float* __restrict__ q,
                                                     double* __restrict__ red, const double* __restrict__ sc) {
    __shared__ double sh[kVT / 32];
    if (sc[S_DONE] != 0.0) return;
    const int i = blockIdx.x * kVT + threadIdx.x;
    float v = 0.f;
    if (i < 9 * C) {
        const int c = i / 9, k = i % 9;
        const float* pc = p32 + static_cast<long long>(kX32) * c;
        const float qi = damped_u_row_dot32(Ul + 81ll * c, pc, k) -
                         static_cast<float>(chunk_sum(cam_chunk_off, part, c, k));
        q[i] = qi;
        v = pc[k] * qi;
    }
    const double t = block_sum_f<kVT>(v, sh);
    if (threadIdx.x == 0) red[blockIdx.x] = t;
}

// pcg_q_finalize for the one-pass product: q = U_lambda p - the sum of the
// camera's accumulators (12 floats each, 9 used; camera c's at [acc_off[c],
// acc_off[c + 1])), which it clears for the next product. One warp per camera
// (the grid has ceil(C / 8) blocks of 8 warps): lanes take the accumulators in
// turn as float4 runs, two per lane per round with both loads issued before
// the stores, then a warp reduction; one p.q partial per block. The loads that
// do not depend on the product (offsets, U_lambda row, p) go out with the done
// flag's, so that a warp waits for two memory round trips, not five. All FP32
// but the block partial.
__global__ void __launch_bounds__(kVT) pcg_q_finalize_acc(float* __restrict__ y, const int* __restrict__ acc_off,
                                                         const float* __restrict__ Ul,
                                                         const float* __restrict__ p32, int C,
                                                         float* __restrict__ q, double* __restrict__ red,
                                                         const double* __restrict__ sc) {
    __shared__ double sh[kVT / 32];
    pdl_wait();
    pdl_trigger();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c = blockIdx.x * (kVT / 32) + warp;
    const bool cam = c < C;
    const double done = sc[S_DONE];
    int r0 = 0, r1 = 0;
    float u[9], pc[9], pown = 0.f;
#pragma unroll
    for (int j = 0; j < 9; ++j) u[j] = pc[j] = 0.f;
    if (cam) {
        r0 = acc_off[c];
        r1 = acc_off[c + 1];
        if (lane < 9) {
            const float* ur = Ul + 81ll * c + 9 * lane;
            const float* pr = p32 + static_cast<long long>(kX32) * c;
#pragma unroll
            for (int j = 0; j < 9; ++j) {
                u[j] = ur[j];
                pc[j] = pr[j];
            }
            pown = pr[lane];
        }
    }
    if (done != 0.0) return;  // the same value in every thread of the grid
    float a[9];
#pragma unroll
    for (int t = 0; t < 9; ++t) a[t] = 0.f;
    // a lane's accumulators (r, r + 32, r + 64, ... in order), then the warp
    // tree: as few terms per sum as the two-pass camera pass
    for (int r = r0 + lane; r < r1; r += 64) {
        const bool two = r + 32 < r1;
        float4* ya = reinterpret_cast<float4*>(y + static_cast<long long>(kX32) * r);
        float4* yb = reinterpret_cast<float4*>(y + static_cast<long long>(kX32) * (r + 32));
        const float4 A0 = ya[0], B0 = ya[1];
        const float e0 = reinterpret_cast<const float*>(ya)[8];
        float4 A1 = make_float4(0.f, 0.f, 0.f, 0.f), B1 = A1;
        float e1 = 0.f;
        if (two) {
            A1 = yb[0];
            B1 = yb[1];
            e1 = reinterpret_cast<const float*>(yb)[8];
        }
        a[0] += A0.x;
        a[1] += A0.y;
        a[2] += A0.z;
        a[3] += A0.w;
        a[4] += B0.x;
        a[5] += B0.y;
        a[6] += B0.z;
        a[7] += B0.w;
        a[8] += e0;
        a[0] += A1.x;
        a[1] += A1.y;
        a[2] += A1.z;
        a[3] += A1.w;
        a[4] += B1.x;
        a[5] += B1.y;
        a[6] += B1.z;
        a[7] += B1.w;
        a[8] += e1;
        const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
        ya[0] = z4;
        ya[1] = z4;
        reinterpret_cast<float*>(ya)[8] = 0.f;
        if (two) {
            yb[0] = z4;
            yb[1] = z4;
            reinterpret_cast<float*>(yb)[8] = 0.f;
        }
    }
    float mine = 0.f;
#pragma unroll
    for (int t = 0; t < 9; ++t) {
        const float v = warp_sum(a[t]);
        if (lane == t) mine = v;
    }
    float pq = 0.f;
    if (cam && lane < 9) {
        float s = 0.f;
#pragma unroll
        for (int j = 0; j < 9; ++j) s = fmaf(u[j], pc[j], s);
        const float qi = s - mine;
        q[9ll * c + lane] = qi;
        pq = pown * qi;
    }
    const double t = block_sum_f<kVT>(pq, sh);
    if (threadIdx.x == 0) red[blockIdx.x] = t;
}

__device__ __forceinline__ double ordered_block_sum(const double* __restrict__ red, int n, double* sh) {
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += 256) s += red[i];
    return block_sum<256>(s, sh);
}

// One read of a device flag per block, shared by all its threads: block 0 of
// the same kernel may write the flag, and every thread of a block must take
// the same branch before the block's barriers.
__device__ __forceinline__ double block_flag(const double* flag, double* sh) {
    if (threadIdx.x == 0) *sh = *flag;
    __syncthreads();
    const double v = *sh;
    __syncthreads();
    return v;
}

// Fixed-order sum of n partials in two phases, so that a kernel can issue the
// loads of the first together with its other independent loads: this
// thread's share (elements threadIdx.x + m kThreads, in order), then the block
// sum, result in every thread of the block.
template <int kThreads>
__device__ __forceinline__ double thread_partial_sum(const double* __restrict__ red, int n) {
    double s = 0.0;
#pragma unroll 4
    for (int i = threadIdx.x; i < n; i += kThreads) s += red[i];
    return s;
}
template <int kThreads>
__device__ __forceinline__ double finish_sum_all(double s, double* sh, double* out) {
    s = block_sum<kThreads>(s, sh);
    if (threadIdx.x == 0) *out = s;
    __syncthreads();
    return *out;
}

// Explicit block-Jacobi inverse M_c = (L L^T)^-1 from the packed factor L
// (45 per camera): thread (camera, j) forms column j of L^-1 by forward
// substitution, then row a of M = L^-T L^-1. Once per inner solve; the PCG
// update then applies M_c as a 9x9 product without divisions.
// z_i = (M_c r_c)_k for entry i = 9c + k; rs holds the block's r entries.
__device__ __forceinline__ float apply_minv_row(const float* __restrict__ Minv, long long c, int k, const float* rs) {
    const float* m = Minv + 81 * c + 9 * k;
    float z = 0.f;
#pragma unroll
    for (int j = 0; j < 9; ++j) z = fmaf(m[j], rs[j], z);
    return z;
}

// ---- balancing two-level preconditioner with the learned coarse basis Z
// (kCoarse columns of n = 9C, column-major): z = M r with
//   c1 = E^-1 Z^T r,  w = B^-1 (r - SZ c1),  c2 = E^-1 SZ^T w,  z = w + Z (c1 - c2),
// E = Z^T S Z, SZ = S Z (both formed once per trial by coarse_prepare). E^-1 and
// its SPD flag live in einv[0, kCoarse^2) and einv[kCoarse^2]; a flag of 0 (E not
// SPD) zeroes c1 and c2, which leaves block-Jacobi.

// Block partials of V^T v for the kCoarse columns of V (FP32): col holds this
// thread's row of V (zeros past the end), vi its entry of v;
// red[block * kCoarse + j] in FP64.
__device__ __forceinline__ void coarse_partials(const float (&col)[kCoarse], float vi, double* __restrict__ red) {
    // the nine block sums at once: warp shuffle trees (independent, so they
    // interleave), one barrier, then the warps' sums in warp order
    __shared__ float wpart[kUT / 32][kCoarse];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float v[kCoarse];
#pragma unroll
    for (int j = 0; j < kCoarse; ++j) v[j] = col[j] * vi;
#pragma unroll
    for (int j = 0; j < kCoarse; ++j) v[j] = warp_sum(v[j]);
    if (lane == 0) {
#pragma unroll
        for (int j = 0; j < kCoarse; ++j) wpart[warp][j] = v[j];
    }
    __syncthreads();
    if (threadIdx.x < kCoarse) {
        float t = 0.f;
#pragma unroll
        for (int w = 0; w < kUT / 32; ++w) t += wpart[w][threadIdx.x];
        red[static_cast<long long>(blockIdx.x) * kCoarse + threadIdx.x] = static_cast<double>(t);
    }
}

// Row i of the kCoarse columns of V (entry i = 9c + k of camera c; zeros for c >= C).
__device__ __forceinline__ void coarse_row(const float* __restrict__ V, long long n, long long i, bool in,
                                           float (&col)[kCoarse]) {
#pragma unroll
    for (int j = 0; j < kCoarse; ++j) col[j] = in ? V[j * n + i] : 0.f;
}

// c = E^-1 (sum over nb blocks of red[b * kCoarse + j]) in shared cs[kCoarse],
// every block in the same order (warp j sums column j); 0 if E is not SPD.
// Also an FP32 copy in csf[kCoarse] when given. Needs kUT / 32 == kCoarse warps.
// Two phases: the loads (coarse_coeff_loads: this lane's share of its warp's
// column, and for threads < kCoarse their row of E^-1 and the SPD flag), then
// the sums (coarse_coeffs).
struct CoarseLoads {
    double v;
    double e[kCoarse];
    bool spd;
};
__device__ __forceinline__ CoarseLoads coarse_coeff_loads(const double* __restrict__ red, int nb,
                                                          const double* __restrict__ einv) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    CoarseLoads L;
    L.v = 0.0;
#pragma unroll 4
    for (int b = lane; b < nb; b += 32) L.v += red[static_cast<long long>(b) * kCoarse + warp];
    const bool row = threadIdx.x < kCoarse;
    L.spd = row && einv[kCoarse * kCoarse] != 0.0;
#pragma unroll
    for (int k = 0; k < kCoarse; ++k) L.e[k] = row ? einv[threadIdx.x * kCoarse + k] : 0.0;
    return L;
}
__device__ __forceinline__ void coarse_coeffs(const CoarseLoads& L, double* tsum, double* cs, float* csf) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const double v = warp_sum(L.v);
    if (lane == 0) tsum[warp] = v;
    __syncthreads();
    if (threadIdx.x < kCoarse) {
        double c = 0.0;
        if (L.spd) {
#pragma unroll
            for (int k = 0; k < kCoarse; ++k) c += L.e[k] * tsum[k];
        }
        cs[threadIdx.x] = c;
        if (csf) csf[threadIdx.x] = static_cast<float>(c);
    }
    __syncthreads();
}

// w = B^-1 (r - SZ c1) into w; block partials of SZ^T w. c1 from the Z^T r
// partials (block 0 also stores it for coarse_z). At init (init != 0) the PCG
// done flag is not consulted (it is set afterwards by pcg_init_finalize).
// Vectors and SZ in FP32; the coarse coefficients in FP64. Every load is
// issued before the flag test and the coefficient sums.
__global__ void __launch_bounds__(kUT) coarse_w(const float* __restrict__ r, const float* __restrict__ SZ,
                                               const float* __restrict__ Minv, const double* __restrict__ einv,
                                               int C, const double* __restrict__ red_zr, int nb,
                                               double* __restrict__ c1_out, float* __restrict__ w,
                                               double* __restrict__ red_szw, const double* __restrict__ sc, int init) {
    static_assert(kUT / 32 == kCoarse, "one warp per coarse column");
    __shared__ float rs[kUT];
    __shared__ double tsum[kCoarse], c1[kCoarse];
    __shared__ float c1f[kCoarse];
    __shared__ double bc;
    pdl_wait();
    pdl_trigger();
    const int cl = threadIdx.x / 9, k = threadIdx.x % 9;
    const long long c = static_cast<long long>(blockIdx.x) * kUC + cl;
    const long long n = 9ll * C, i = 9 * c + k;
    const bool in = c < C;
    const CoarseLoads L = coarse_coeff_loads(red_zr, nb, einv);
    float sz[kCoarse], m[9], rv = 0.f;
    coarse_row(SZ, n, i, in, sz);
#pragma unroll
    for (int j = 0; j < 9; ++j) m[j] = in ? Minv[81 * c + 9 * k + j] : 0.f;
    if (in) rv = r[i];
    if (!init && block_flag(sc + S_DONE, &bc) != 0.0) return;
    coarse_coeffs(L, tsum, c1, c1f);
    if (blockIdx.x == 0 && threadIdx.x < kCoarse) c1_out[threadIdx.x] = c1[threadIdx.x];
    float yi = rv;
#pragma unroll
    for (int j = 0; j < kCoarse; ++j) yi = fmaf(-sz[j], c1f[j], yi);
    rs[threadIdx.x] = in ? yi : 0.f;
    __syncthreads();
    float wi = 0.f;
    if (in) {
        const float* y9 = rs + 9 * cl;
#pragma unroll
        for (int j = 0; j < 9; ++j) wi = fmaf(m[j], y9[j], wi);
        w[i] = wi;
    }
    coarse_partials(sz, wi, red_szw);
}

// z = w + Z (c1 - c2) in place of w, c2 = E^-1 SZ^T w from the partials; the
// partials of r.z; at init also p = z (FP32 padded direction). Every load is
// issued before the flag test and the coefficient sums.
__global__ void __launch_bounds__(kUT) coarse_z(const float* __restrict__ r, const float* __restrict__ Zc,
                                               const double* __restrict__ einv, int C,
                                               const double* __restrict__ red_szw, int nb,
                                               const double* __restrict__ c1_in, float* __restrict__ z,
                                               float* __restrict__ p32, double* __restrict__ red_rz,
                                               const double* __restrict__ sc, int init) {
    __shared__ double sh[kUT / 32];
    __shared__ double tsum[kCoarse], c2[kCoarse];
    __shared__ float d[kCoarse];
    __shared__ double bc;
    pdl_wait();
    pdl_trigger();
    const int cl = threadIdx.x / 9, k = threadIdx.x % 9;
    const long long c = static_cast<long long>(blockIdx.x) * kUC + cl;
    const long long n = 9ll * C, i = 9 * c + k;
    const bool in = c < C;
    const CoarseLoads L = coarse_coeff_loads(red_szw, nb, einv);
    const double c1v = threadIdx.x < kCoarse ? c1_in[threadIdx.x] : 0.0;
    float zc[kCoarse], zv = 0.f, rv = 0.f;
    coarse_row(Zc, n, i, in, zc);
    if (in) {
        zv = z[i];
        rv = r[i];
    }
    if (!init && block_flag(sc + S_DONE, &bc) != 0.0) return;
    coarse_coeffs(L, tsum, c2, nullptr);
    if (threadIdx.x < kCoarse) d[threadIdx.x] = static_cast<float>(c1v - c2[threadIdx.x]);
    __syncthreads();
    float rz = 0.f;
    if (in) {
        float zi = zv;
#pragma unroll
        for (int j = 0; j < kCoarse; ++j) zi = fmaf(zc[j], d[j], zi);
        z[i] = zi;
        if (init) p32[kX32 * c + k] = zi;
        rz = rv * zi;
    }
    const double t = block_sum_f<kUT>(rz, sh);
    if (threadIdx.x == 0) red_rz[blockIdx.x] = t;
}

// ---- S Z for all kCoarse basis columns in one implicit product (instead of
// kCoarse single products): the Jacobian rows are read once per slot.

constexpr int kZs = 88;  // BF16 values per camera of the basis copy Zb (9 x 9, padded to 16-byte multiples)
constexpr int kU9 = 20;  // floats per u record of the coarse product (18 used; 80 B, 16-byte aligned)

// u_j = Jp w_j for the nine columns, stored as one kU9 record: four float4
// and a float2 (the records are scattered to camera-major positions, so fewer,
// wider stores).
__device__ __forceinline__ void store_u9(float* __restrict__ rec, const float* jp, const float* w) {
    float u[18];
#pragma unroll
    for (int j = 0; j < kCoarse; ++j) {
        u[2 * j] = fmaf(jp[0], w[3 * j], fmaf(jp[1], w[3 * j + 1], jp[2] * w[3 * j + 2]));
        u[2 * j + 1] = fmaf(jp[3], w[3 * j], fmaf(jp[4], w[3 * j + 1], jp[5] * w[3 * j + 2]));
    }
    float4* r4 = reinterpret_cast<float4*>(rec);
#pragma unroll
    for (int m = 0; m < 4; ++m) r4[m] = make_float4(u[4 * m], u[4 * m + 1], u[4 * m + 2], u[4 * m + 3]);
    reinterpret_cast<float2*>(rec)[8] = make_float2(u[16], u[17]);
}

// The basis is used at BF16 precision: Zb[c][i][j] = bf16(Z[j][9c + i]), the
// per-camera rows the point pass gathers (176 B per camera), and Z itself (and
// its FP32 copy Zc32, for the PCG) is overwritten by the same rounded values,
// so that S Z, E = Z^T S Z and the preconditioner all use one basis (any full-rank basis is valid; the rounding
// moves its span by ~4e-3 relative).
__global__ void __launch_bounds__(kVT) coarse_zb_kernel(double* __restrict__ Zc, int C,
                                                       __nv_bfloat16* __restrict__ Zb, float* __restrict__ Zc32) {
    const int t = blockIdx.x * kVT + threadIdx.x;
    if (t >= 81 * C) return;
    const int c = t / 81, r = t - 81 * c, i = r / 9, j = r - 9 * i;
    const long long at = static_cast<long long>(j) * 9 * C + 9ll * c + i;
    const __nv_bfloat16 b = __float2bfloat16_rn(static_cast<float>(Zc[at]));
    Zb[static_cast<long long>(kZs) * c + r] = b;
    const float v = __bfloat162float(b);
    Zc[at] = static_cast<double>(v);
    Zc32[at] = v;
}

// Point pass of S Z (FP32, as schur_point_pass for one vector): per slot,
// a_j = Jc Z_c(:, j) for all columns (the camera's 9 x 9 rows read as float4
// runs) and v_j = Jp^T a_j (27 values); per point t_j = sum over its slots (one
// warp segmented scan of the 27 values and ordered segment sums), w_j = V'^-1 t_j;
// per slot u_j = Jp w_j, one kU9 record at the slot's camera-major position.
__global__ void __launch_bounds__(kPT, 2) coarse_point_pass9(const int4* __restrict__ prange,
                                                            const int* __restrict__ pt_off,
                                                            const int* __restrict__ s_cam,
                                                            const int* __restrict__ s_pt,
                                                            const int* __restrict__ cam_pos,
                                                            const float* __restrict__ Jc32,
                                                            const float* __restrict__ Jp32, long long js,
                                                            const float* __restrict__ vinv_hi,
                                                            const __nv_bfloat16* __restrict__ Zb,
                                                            float* __restrict__ u9) {
    constexpr int KV = 3 * kCoarse;
    __shared__ float seg[kPT][KV + 1];  // warp-segment sums (27 per slot), at each segment's last slot
    float* wsh = &seg[0][0];            // reused for w (27 per point) once the sums are taken
    const int4 rg = prange[blockIdx.x];
    const int p0 = rg.x, p1 = rg.y, s0 = rg.z, s1 = rg.w;
    const int my_p = p0 + threadIdx.x;
    const int lane = threadIdx.x & 31;
    int my_b = 0, my_e = 0;
    if (my_p < p1) {
        my_b = pt_off[my_p];
        my_e = pt_off[my_p + 1];
    }
    float t[KV];
#pragma unroll
    for (int k = 0; k < KV; ++k) t[k] = 0.f;
    for (int base = s0; base < s1; base += kPT) {
        const int s = base + threadIdx.x;
        int key = -1;
        float v[KV];
#pragma unroll
        for (int k = 0; k < KV; ++k) v[k] = 0.f;
        if (s < s1) {
            key = s_pt[s];
            float J[24];
            load_j(Jc32, Jp32, js, s, J);
            const uint4* z4 = reinterpret_cast<const uint4*>(Zb + static_cast<long long>(kZs) * s_cam[s]);
            float Z[kZs];
#pragma unroll
            for (int q = 0; q < kZs / 8; ++q) {
                const uint4 z = __ldg(z4 + q);
                const uint32_t w[4] = {z.x, z.y, z.z, z.w};
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    Z[8 * q + 2 * h] = __uint_as_float(w[h] << 16);             // low BF16 of the word
                    Z[8 * q + 2 * h + 1] = __uint_as_float(w[h] & 0xffff0000u);  // high BF16
                }
            }
#pragma unroll
            for (int j = 0; j < kCoarse; ++j) {
                float a0 = 0.f, a1 = 0.f;
#pragma unroll
                for (int i = 0; i < 9; ++i) {
                    a0 = fmaf(J[i], Z[9 * i + j], a0);
                    a1 = fmaf(J[9 + i], Z[9 * i + j], a1);
                }
                v[3 * j] = J[18] * a0 + J[21] * a1;
                v[3 * j + 1] = J[19] * a0 + J[22] * a1;
                v[3 * j + 2] = J[20] * a0 + J[23] * a1;
            }
        }
        const int knext = __shfl_down_sync(0xffffffffu, key, 1);
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int kd = __shfl_up_sync(0xffffffffu, key, d);
            const bool take = lane >= d && kd == key;
#pragma unroll
            for (int k = 0; k < KV; ++k) {
                const float u = __shfl_up_sync(0xffffffffu, v[k], d);
                if (take) v[k] += u;
            }
        }
        if (lane == 31 || knext != key) {
#pragma unroll
            for (int k = 0; k < KV; ++k) seg[threadIdx.x][k] = v[k];
        }
        __syncthreads();
        if (my_p < p1) {
            const int b = max(my_b, base) - base, e = min(my_e, base + kPT) - base;
            for (int w = b >> 5; b < e && w <= (e - 1) >> 5; ++w) {
                const int q = min(e - 1, 32 * w + 31);
#pragma unroll
                for (int k = 0; k < KV; ++k) t[k] += seg[q][k];
            }
        }
        __syncthreads();
    }
    if (my_p < p1) {
        float vi[6];
        load_vinv(vinv_hi, nullptr, my_p, vi);
#pragma unroll
        for (int j = 0; j < kCoarse; ++j) {
            float w0, w1, w2;
            apply_vinv(vi, t[3 * j], t[3 * j + 1], t[3 * j + 2], w0, w1, w2);
            wsh[threadIdx.x * (KV + 1) + 3 * j] = w0;
            wsh[threadIdx.x * (KV + 1) + 3 * j + 1] = w1;
            wsh[threadIdx.x * (KV + 1) + 3 * j + 2] = w2;
        }
    }
    __syncthreads();
    for (int s = s0 + threadIdx.x; s < s1; s += kPT) {
        const int pl = s_pt[s] - p0;
        float jp[6];
        load_jp(Jp32, js, s, jp);
        store_u9(u9 + static_cast<long long>(kU9) * cam_pos[s], jp, wsh + pl * (KV + 1));
    }
}

// a_j = Jc Z_c(:, j) for the nine columns, from the camera's BF16 rows (Zb,
// kZs values per camera) read as 16-byte runs and consumed as they arrive, and
// v_j = Jp^T a_j (27 values: v[3 j + k]).
__device__ __forceinline__ void coarse_slot_v(const float* J, const __nv_bfloat16* __restrict__ Zb, int cam,
                                              float* v) {
    float a0[kCoarse], a1[kCoarse];
#pragma unroll
    for (int j = 0; j < kCoarse; ++j) a0[j] = a1[j] = 0.f;
    const uint4* z4 = reinterpret_cast<const uint4*>(Zb + static_cast<long long>(kZs) * cam);
#pragma unroll
    for (int q = 0; q < kZs / 8; ++q) {
        const uint4 z = __ldg(z4 + q);
        const uint32_t w[4] = {z.x, z.y, z.z, z.w};
#pragma unroll
        for (int h = 0; h < 8; ++h) {
            const int r = 8 * q + h;  // entry (i, j) = (r / 9, r % 9) of the camera's 9 x 9 rows
            if (r < 81) {
                const float zv = (h & 1) ? __uint_as_float(w[h >> 1] & 0xffff0000u) : __uint_as_float(w[h >> 1] << 16);
                a0[r % 9] = fmaf(J[r / 9], zv, a0[r % 9]);
                a1[r % 9] = fmaf(J[9 + r / 9], zv, a1[r % 9]);
            }
        }
    }
#pragma unroll
    for (int j = 0; j < kCoarse; ++j) {
        v[3 * j] = fmaf(J[18], a0[j], J[21] * a1[j]);
        v[3 * j + 1] = fmaf(J[19], a0[j], J[22] * a1[j]);
        v[3 * j + 2] = fmaf(J[20], a0[j], J[23] * a1[j]);
    }
}

// Point pass of S Z over warp chunks (whole points of at most 32 slots per
// warp; as schur_matvec_warp): per slot v_j = Jp^T Jc Z_c(:, j), a segmented
// scan of the 27 values over the warp, w_j = V'^-1 t_j at each point's last
// lane, every lane takes its point's w (match + shuffle) and stores u_j = Jp w_j
// (18 floats) at its camera-major position for coarse_camera_pass9.
__global__ void __launch_bounds__(32 * kMWarps) coarse_point_pass9_warp(
    const int2* __restrict__ wchunk, int n_wchunk, const int* __restrict__ s_cam, const int* __restrict__ s_pt,
    const int* __restrict__ cam_pos, const float* __restrict__ Jc32, const float* __restrict__ Jp32, long long js,
    const float* __restrict__ vinv, const __nv_bfloat16* __restrict__ Zb, float* __restrict__ u9) {
    constexpr int KV = 3 * kCoarse;
    const int wid = blockIdx.x * kMWarps + (threadIdx.x >> 5);
    if (wid >= n_wchunk) return;  // whole warps leave together
    const int lane = threadIdx.x & 31;
    const int2 r = wchunk[wid];
    const int s = r.x + lane;
    const bool has = s < r.y;
    int key = -1;
    long long q = 0;
    float J[24], vi[6], v[KV];
#pragma unroll
    for (int k = 0; k < KV; ++k) v[k] = 0.f;
    if (has) {
        key = s_pt[s];
        q = cam_pos[s];
        load_j(Jc32, Jp32, js, s, J);
        load_vinv(vinv, nullptr, key, vi);
        coarse_slot_v(J, Zb, s_cam[s], v);
    }
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int kd = __shfl_up_sync(0xffffffffu, key, d);
        const bool take = lane >= d && kd == key;
#pragma unroll
        for (int k = 0; k < KV; ++k) {
            const float u = __shfl_up_sync(0xffffffffu, v[k], d);
            if (take) v[k] += u;
        }
    }
    if (has) {  // meaningful at the point's last lane
#pragma unroll
        for (int j = 0; j < kCoarse; ++j) apply_vinv(vi, v[3 * j], v[3 * j + 1], v[3 * j + 2], v[3 * j], v[3 * j + 1],
                                                    v[3 * j + 2]);
    }
    const int last = 31 - __clz(__match_any_sync(0xffffffffu, key));
#pragma unroll
    for (int k = 0; k < KV; ++k) v[k] = __shfl_sync(0xffffffffu, v[k], last);
    if (has) store_u9(u9 + kU9 * q, J + 18, v);
}

// Point pass of S Z for points with 33 to 256 observations: a CTA takes a
// list of them as one virtual chunk (as schur_matvec_long); per point the
// warps' segment sums in order (shared memory), then u_j = Jp w_j per slot.
__global__ void __launch_bounds__(kPT) coarse_point_pass9_list(
    const int2* __restrict__ lchunk, const int* __restrict__ lpts, const int* __restrict__ pt_off,
    const int* __restrict__ s_cam, const int* __restrict__ cam_pos, const float* __restrict__ Jc32,
    const float* __restrict__ Jp32, long long js, const float* __restrict__ vinv,
    const __nv_bfloat16* __restrict__ Zb, float* __restrict__ u9) {
    constexpr int KV = 3 * kCoarse;
    constexpr int kMaxPts = kPT / 33 + 1;
    __shared__ int pb[kMaxPts + 1], ps[kMaxPts], pid[kMaxPts];
    __shared__ float seg[kPT][KV + 1];
    __shared__ float wsh[kMaxPts][KV];
    const int2 lc = lchunk[blockIdx.x];
    const int tid = threadIdx.x, lane = tid & 31;
    if (tid < lc.y) {
        const int p = lpts[lc.x + tid];
        const int o0 = pt_off[p], o1 = pt_off[p + 1];
        pid[tid] = p;
        ps[tid] = o0;
        pb[tid + 1] = o1 - o0;
    }
    __syncwarp();
    if (tid == 0) {
        pb[0] = 0;
        for (int j = 1; j <= lc.y; ++j) pb[j] += pb[j - 1];
    }
    __syncthreads();
    const int n = pb[lc.y];
    int key = -1;
    long long sl = 0;
    float J[24], v[KV];
#pragma unroll
    for (int k = 0; k < KV; ++k) v[k] = 0.f;
    if (tid < n) {
        int j = 0;
        while (tid >= pb[j + 1]) ++j;
        key = j;
        sl = ps[j] + (tid - pb[j]);
        load_j(Jc32, Jp32, js, sl, J);
        coarse_slot_v(J, Zb, s_cam[sl], v);
    }
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int kd = __shfl_up_sync(0xffffffffu, key, d);
        const bool take = lane >= d && kd == key;
#pragma unroll
        for (int k = 0; k < KV; ++k) {
            const float u = __shfl_up_sync(0xffffffffu, v[k], d);
            if (take) v[k] += u;
        }
    }
    const int knext = __shfl_down_sync(0xffffffffu, key, 1);
    if (lane == 31 || knext != key) {
#pragma unroll
        for (int k = 0; k < KV; ++k) seg[tid][k] = v[k];
    }
    __syncthreads();
    // the points' sums, one thread per (point, value): the warps' segment
    // ends in order
    if (tid < KV * lc.y) {
        const int j = tid / KV, k = tid - KV * j;
        const int b = pb[j], e = pb[j + 1];
        float t = 0.f;
        for (int w = b >> 5; w <= (e - 1) >> 5; ++w) t += seg[min(e - 1, 32 * w + 31)][k];
        wsh[j][k] = t;
    }
    __syncthreads();
    // w = V'^-1 t, one thread per (point, column)
    if (tid < kCoarse * lc.y) {
        const int j = tid / kCoarse, c = tid - kCoarse * j;
        float vi[6];
        load_vinv(vinv, nullptr, pid[j], vi);
        float* w = wsh[j] + 3 * c;
        apply_vinv(vi, w[0], w[1], w[2], w[0], w[1], w[2]);
    }
    __syncthreads();
    if (tid < n) {
        store_u9(u9 + static_cast<long long>(kU9) * cam_pos[sl], J + 18, wsh[key]);
    }
}

// Camera pass of S Z: per camera chunk, the partials sum_e Jc_e^T u_e,j for all
// columns (81 per chunk at part[81 chunk + 9 i + j]); thread (g, j): positions
// g, g + 16, ... of the chunk for column j, FP32 sums, groups added in FP64.
constexpr int kC9 = 16 * kCoarse;
__global__ void __launch_bounds__(kC9) coarse_camera_pass9(const int* __restrict__ cchunk_begin,
                                                          const int* __restrict__ cchunk_cam,
                                                          const int* __restrict__ cam_off,
                                                          const float* __restrict__ J32c,
                                                          const float* __restrict__ u9, double* __restrict__ part) {
    __shared__ float sh[16][81];
    const int k = blockIdx.x;
    const int b = cchunk_begin[k], c = cchunk_cam[k];
    const int e = min(b + kCamChunk, cam_off[c + 1]);
    const int g = threadIdx.x / kCoarse, j = threadIdx.x - kCoarse * g;
    float acc[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) acc[i] = 0.f;
    for (int q = b + g; q < e; q += 16) {
        const float* rec = J32c + 20ll * q;
        const float2 u = reinterpret_cast<const float2*>(u9 + static_cast<long long>(kU9) * q)[j];
#pragma unroll
        for (int i = 0; i < 9; ++i) acc[i] = fmaf(__ldg(rec + i), u.x, fmaf(__ldg(rec + 9 + i), u.y, acc[i]));
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) sh[g][9 * i + j] = acc[i];
    __syncthreads();
    if (threadIdx.x < 81) {
        double v = 0.0;
#pragma unroll
        for (int gg = 0; gg < 16; ++gg) v += static_cast<double>(sh[gg][threadIdx.x]);
        part[81ll * k + threadIdx.x] = v;
    }
}

// SZ[j][9c + i] = (U_lambda Z_j)_(c, i) - sum over the camera's chunks of part[81 q + 9 i + j] (FP64),
// and its FP32 copy SZ32 (for the PCG).
__global__ void __launch_bounds__(kVT) coarse_sz_finalize(const int* __restrict__ cam_chunk_off,
                                                         const double* __restrict__ part,
                                                         const double* __restrict__ U, double lambda,
                                                         const double* __restrict__ Zc, int C,
                                                         double* __restrict__ SZ, float* __restrict__ SZ32) {
    const int t = blockIdx.x * kVT + threadIdx.x;
    if (t >= 81 * C) return;
    const int c = t / 81, r = t - 81 * c, i = r / 9, j = r - 9 * i;
    const long long n = 9ll * C;
    double sum = 0.0;
    for (int q = cam_chunk_off[c]; q < cam_chunk_off[c + 1]; ++q) sum += part[81ll * q + r];
    const double v = damped_u_row_dot(U + 81ll * c, i, lambda, Zc + j * n + 9ll * c) - sum;
    SZ[j * n + 9ll * c + i] = v;
    SZ32[j * n + 9ll * c + i] = static_cast<float>(v);
}

// Block partials of E = Z^T SZ: red[block * kCoarse^2 + a kCoarse + b] over the
// block's entries (one per thread): warp shuffle sums per pair, then the warps'
// sums in warp order (one barrier).
__global__ void __launch_bounds__(kVT) coarse_gram_partials(const double* __restrict__ Zc,
                                                           const double* __restrict__ SZ, long long n,
                                                           double* __restrict__ red) {
    constexpr int KK = kCoarse * kCoarse;
    __shared__ double wsum[kVT / 32][KK];
    const long long i = static_cast<long long>(blockIdx.x) * kVT + threadIdx.x;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double zv[kCoarse], sv[kCoarse];
#pragma unroll
    for (int j = 0; j < kCoarse; ++j) {
        zv[j] = i < n ? Zc[j * n + i] : 0.0;
        sv[j] = i < n ? SZ[j * n + i] : 0.0;
    }
#pragma unroll
    for (int a = 0; a < kCoarse; ++a)
#pragma unroll
        for (int b = 0; b < kCoarse; ++b) {
            const double t = warp_sum(zv[a] * sv[b]);
            if (lane == 0) wsum[warp][a * kCoarse + b] = t;
        }
    __syncthreads();
    if (threadIdx.x < KK) {
        double v = 0.0;
#pragma unroll
        for (int w = 0; w < kVT / 32; ++w) v += wsum[w][threadIdx.x];
        red[static_cast<long long>(blockIdx.x) * KK + threadIdx.x] = v;
    }
}

// E from the partials (fixed order), symmetrised; FP64 Cholesky and inverse by
// one thread. einv[kCoarse^2] = 1 if E is SPD (relative pivot floor 1e-13), else 0.
constexpr int kEinvT = 1024;
__global__ void __launch_bounds__(kEinvT) coarse_einv_kernel(const double* __restrict__ red, int nb,
                                                            double* __restrict__ einv) {
    constexpr int K = kCoarse, KK = kCoarse * kCoarse;
    __shared__ double E[KK], L[KK];
    __shared__ int ok;
    // entry t of E: one warp sums the nb block partials (lanes strided, then a shuffle tree)
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int t = warp; t < KK; t += kEinvT / 32) {
        double v = 0.0;
        for (int b = lane; b < nb; b += 32) v += red[static_cast<long long>(b) * KK + t];
        v = warp_sum(v);
        if (lane == 0) E[t] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {  // Cholesky of the symmetrised E (9 x 9)
        double dmax = 0.0;
        for (int a = 0; a < K; ++a)
            for (int b = 0; b < K; ++b) L[a * K + b] = 0.5 * (E[a * K + b] + E[b * K + a]);
        for (int a = 0; a < K; ++a) dmax = fmax(dmax, L[a * K + a]);
        bool good = dmax > 0.0 && isfinite(dmax);
        for (int k = 0; k < K && good; ++k) {
            double d = L[k * K + k];
            for (int m = 0; m < k; ++m) d -= L[k * K + m] * L[k * K + m];
            if (!(d > 1e-13 * dmax)) {
                good = false;
                break;
            }
            const double l = sqrt(d);
            L[k * K + k] = l;
            for (int a = k + 1; a < K; ++a) {
                double v = L[a * K + k];
                for (int m = 0; m < k; ++m) v -= L[a * K + m] * L[k * K + m];
                L[a * K + k] = v / l;
            }
        }
        ok = good;
    }
    __syncthreads();
    if (!ok) {
        for (int t = threadIdx.x; t <= KK; t += kEinvT) einv[t] = 0.0;
        return;
    }
    // E^-1 = L^-T L^-1, one column of the identity per thread
    if (threadIdx.x < K) {
        const int col = threadIdx.x;
        double y[K];
#pragma unroll
        for (int a = 0; a < K; ++a) {
            double v = a == col ? 1.0 : 0.0;
            for (int m = 0; m < a; ++m) v -= L[a * K + m] * y[m];
            y[a] = v / L[a * K + a];
        }
#pragma unroll
        for (int a = K - 1; a >= 0; --a) {
            double v = y[a];
            for (int m = a + 1; m < K; ++m) v -= L[m * K + a] * y[m];
            y[a] = v / L[a * K + a];
        }
#pragma unroll
        for (int a = 0; a < K; ++a) einv[a * K + col] = y[a];
    }
    if (threadIdx.x == 0) einv[KK] = 1.0;
}

// Block partials of a . b, a FP64 and b FP32 (b . x of the inner solution).
__global__ void __launch_bounds__(kVT) dot_partials(const double* __restrict__ a, const float* __restrict__ b, int n,
                                                   double* __restrict__ red) {
    __shared__ double sh[kVT / 32];
    const int i = blockIdx.x * kVT + threadIdx.x;
    const double t = block_sum<kVT>(i < n ? a[i] * static_cast<double>(b[i]) : 0.0, sh);
    if (threadIdx.x == 0) red[blockIdx.x] = t;
}

// The inner PCG's vectors are FP32 (x, r, z, q: 9 per camera; the direction p
// in the padded product layout p32, kX32 per camera): it solves the FP32
// operator's system to a relative residual of 1e-4 or looser, and the
// refinement around it carries the accuracy. Its scalars (p.q, r.r, r.z, alpha,
// beta) and the sums of block partials stay FP64.

// alpha = rz / p.q (every block sums the p.q partials in the same order);
// x += alpha p, r -= alpha q, z = M r; partials r.r and r.z. Nine threads per camera.
// With a coarse basis Z (learned form; Zc non-null) z is left to coarse_w /
// coarse_z: this kernel writes the partials of Z^T r (kCoarse per block) instead.
// Every load (partials, scalars, vectors, the M_c row or Z row) is issued
// before the flag test.
__global__ void __launch_bounds__(kUT) pcg_update(float* __restrict__ x, float* __restrict__ r,
                                                 float* __restrict__ z, const float* __restrict__ p32,
                                                 const float* __restrict__ q, const float* __restrict__ Minv, int C,
                                                 const double* __restrict__ red_pq, int n_pq,
                                                 double* __restrict__ red_rr, double* __restrict__ red_rz,
                                                 double* __restrict__ sc, const float* __restrict__ Zc,
                                                 double* __restrict__ red_zr) {
    __shared__ double sh[kUT / 32];
    __shared__ float rs[kUT];
    __shared__ double bc;
    pdl_wait();
    pdl_trigger();
    const int cl = threadIdx.x / 9, k = threadIdx.x % 9;
    const long long c = static_cast<long long>(blockIdx.x) * kUC + cl;
    const long long n = 9ll * C, i = 9 * c + k;
    const bool in = c < C;
    const double pq_part = thread_partial_sum<kUT>(red_pq, n_pq);
    const double rz_old = sc[S_RZ];
    float m[9], xv = 0.f, pv = 0.f, qv = 0.f, rv = 0.f;
    if (Zc) {
        coarse_row(Zc, n, i, in, m);
    } else {
#pragma unroll
        for (int j = 0; j < 9; ++j) m[j] = in ? Minv[81 * c + 9 * k + j] : 0.f;
    }
    if (in) {
        xv = x[i];
        pv = p32[kX32 * c + k];
        qv = q[i];
        rv = r[i];
    }
    if (block_flag(sc + S_DONE, &bc) != 0.0) return;
    const double pq = finish_sum_all<kUT>(pq_part, sh, &bc);
    const bool first = blockIdx.x == 0 && threadIdx.x == 0;
    if (!(pq > 0.0) || !isfinite(pq)) {
        if (first) sc[S_DONE] = 2.0;  // breakdown: keep the current iterate
        return;
    }
    const double alpha = rz_old / pq;
    if (first) {
        sc[S_ALPHA] = alpha;
        sc[S_RZPREV] = rz_old;
        sc[S_ITERS] += 1.0;
    }
    const float af = static_cast<float>(alpha);
    float ri = 0.f;
    if (in) {
        x[i] = fmaf(af, pv, xv);
        ri = fmaf(-af, qv, rv);
        r[i] = ri;
    }
    if (Zc) {
        coarse_partials(m, ri, red_zr);
        const double a = block_sum_f<kUT>(ri * ri, sh);
        if (threadIdx.x == 0) red_rr[blockIdx.x] = a;
        return;
    }
    rs[threadIdx.x] = ri;
    __syncthreads();
    float rz = 0.f;
    if (in) {
        const float* r9 = rs + 9 * cl;
        float zi = 0.f;
#pragma unroll
        for (int j = 0; j < 9; ++j) zi = fmaf(m[j], r9[j], zi);
        z[i] = zi;
        rz = ri * zi;
    }
    const double a = block_sum_f<kUT>(ri * ri, sh);
    const double b = block_sum_f<kUT>(rz, sh);
    if (threadIdx.x == 0) {
        red_rr[blockIdx.x] = a;
        red_rz[blockIdx.x] = b;
    }
}

// Convergence test and beta = rz / rz_prev (every block sums the partials in
// the same order), then p = z + beta p (FP32, padded layout). Every load is
// issued before the flag test.
__global__ void __launch_bounds__(kVT) pcg_direction(float* __restrict__ p32, const float* __restrict__ z, int n,
                                                    const double* __restrict__ red_rr,
                                                    const double* __restrict__ red_rz, int n_red, int max_iters,
                                                    double* __restrict__ sc) {
    __shared__ double sh[kVT / 32];
    __shared__ double bc;
    pdl_wait();
    pdl_trigger();
    const double rr_part = thread_partial_sum<kVT>(red_rr, n_red);
    const double rz_part = thread_partial_sum<kVT>(red_rz, n_red);
    const double tol2 = sc[S_TOL2], bb = sc[S_BB], iters = sc[S_ITERS], rz_prev = sc[S_RZPREV];
    const int i = blockIdx.x * kVT + threadIdx.x;
    float* pp = nullptr;
    float zv = 0.f, pv = 0.f;
    if (i < n) {
        const int c = i / 9;
        pp = p32 + static_cast<long long>(kX32) * c + (i - 9 * c);
        zv = z[i];
        pv = *pp;
    }
    if (block_flag(sc + S_DONE, &bc) != 0.0) return;
    const double rr = finish_sum_all<kVT>(rr_part, sh, &bc);
    const double rz = finish_sum_all<kVT>(rz_part, sh, &bc);
    double done = 0.0;
    if (rr <= tol2 * bb || iters >= max_iters) {
        done = 1.0;
    } else if (!(rz > 0.0) || !isfinite(rz)) {
        done = 2.0;
    }
    const double beta = rz / rz_prev;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        sc[S_RR] = rr;
        if (done != 0.0) {
            sc[S_DONE] = done;
        } else {
            sc[S_BETA] = beta;
            sc[S_RZ] = rz;
        }
    }
    if (done != 0.0) return;
    if (i < n) *pp = fmaf(static_cast<float>(beta), pv, zv);
}

// x = 0, r = b (rounded to FP32), z = M r, p = z; partials b.b and r.z. Nine
// threads per camera. With a coarse basis (Zc non-null): x = 0, r = b and the
// partials b.b and Z^T b; coarse_w / coarse_z then form z = p and the r.z partials.
__global__ void __launch_bounds__(kUT) pcg_init(float* __restrict__ x, float* __restrict__ r, float* __restrict__ z,
                                               float* __restrict__ p32, const double* __restrict__ b,
                                               const float* __restrict__ Minv, int C, double* __restrict__ red_rr,
                                               double* __restrict__ red_rz, const float* __restrict__ Zc,
                                               double* __restrict__ red_zr) {
    __shared__ double sh[kUT / 32];
    __shared__ float rs[kUT];
    const int cl = threadIdx.x / 9, k = threadIdx.x % 9;
    const long long c = static_cast<long long>(blockIdx.x) * kUC + cl;
    const long long i = 9 * c + k;
    float ri = 0.f;
    if (c < C) {
        ri = static_cast<float>(b[i]);
        x[i] = 0.f;
        r[i] = ri;
    }
    if (Zc) {
        float zc[kCoarse];
        coarse_row(Zc, 9ll * C, i, c < C, zc);
        coarse_partials(zc, ri, red_zr);
        const double a = block_sum_f<kUT>(ri * ri, sh);
        if (threadIdx.x == 0) red_rr[blockIdx.x] = a;
        return;
    }
    rs[threadIdx.x] = ri;
    __syncthreads();
    float rz = 0.f;
    if (c < C) {
        const float zi = apply_minv_row(Minv, c, k, rs + 9 * cl);
        z[i] = zi;
        p32[kX32 * c + k] = zi;
        rz = ri * zi;
    }
    const double a = block_sum_f<kUT>(ri * ri, sh);
    const double bb = block_sum_f<kUT>(rz, sh);
    if (threadIdx.x == 0) {
        red_rr[blockIdx.x] = a;
        red_rz[blockIdx.x] = bb;
    }
}

__global__ void __launch_bounds__(256) pcg_init_finalize(const double* __restrict__ red_rr,
                                                        const double* __restrict__ red_rz, int n, double tol,
                                                        double* __restrict__ sc) {
    __shared__ double sh[8];
    const double bb = ordered_block_sum(red_rr, n, sh);
    const double rz = ordered_block_sum(red_rz, n, sh);
    if (threadIdx.x == 0) {
        sc[S_BB] = bb;
        sc[S_RR] = bb;
        sc[S_RZ] = rz;
        sc[S_TOL2] = tol * tol;
        sc[S_ITERS] = 0.0;
        sc[S_DONE] = (bb == 0.0) ? 1.0 : ((rz > 0.0 && isfinite(rz)) ? 0.0 : 2.0);
    }
}

// Sum of block partials -> sc[slot].
__global__ void __launch_bounds__(256) sum_to_scalar(const double* __restrict__ red, int n, double* __restrict__ sc,
                                                    int slot) {
    __shared__ double sh[8];
    const double v = ordered_block_sum(red, n, sh);
    if (threadIdx.x == 0) sc[slot] = v;
}

// Float-float split of y (hi, lo interleaved).
__global__ void __launch_bounds__(kVT) split_kernel(const double* __restrict__ y, long long n,
                                                   float* __restrict__ yff) {
    const long long i = static_cast<long long>(blockIdx.x) * kVT + threadIdx.x;
    if (i < n) {
        const ff f = ffa::from_double(y[i]);
        reinterpret_cast<float2*>(yff)[i] = make_float2(f.hi, f.lo);
    }
}

// y += x (x: the inner PCG's FP32 solution), and the float-float split of the
// new y (hi, lo interleaved).
__global__ void __launch_bounds__(kVT) axpy_split_kernel(double* __restrict__ y, const float* __restrict__ x, int n,
                                                        float* __restrict__ yff) {
    const int i = blockIdx.x * kVT + threadIdx.x;
    if (i < n) {
        const double v = y[i] + static_cast<double>(x[i]);
        y[i] = v;
        const ff f = ffa::from_double(v);
        reinterpret_cast<float2*>(yff)[i] = make_float2(f.hi, f.lo);
    }
}

// Ul = U + lambda max(diag U, 1e-12) in FP32 (81 per camera): the camera
// blocks of the inner PCG's operator, once per Schur solve.
__global__ void __launch_bounds__(kVT) damped_u32_kernel(const double* __restrict__ U, double lambda, int C,
                                                        float* __restrict__ Ul) {
    const long long t = static_cast<long long>(blockIdx.x) * kVT + threadIdx.x;
    if (t >= 81ll * C) return;
    const long long c = t / 81;
    const int r = static_cast<int>(t - 81 * c), k = r / 9, j = r - 9 * k;
    double v = U[t];
    if (k == j) {
        const double d = U[81 * c + 10 * k];
        v += lambda * (d > 0.0 ? d : 1e-12);
    }
    Ul[t] = static_cast<float>(v);
}

// ---- block-Jacobi blocks S_cc = U_lambda,c - sum_{e in c} Jc^T (Jp V'^-1 Jp^T) Jc
// (the sums come from the right-hand side camera pass)

// Block-Jacobi factor of one camera block: right-looking FP64 Cholesky of the
// 9x9 block. FP64, because even Jacobi-scaled the camera blocks' condition
// numbers make an FP32 factor a visibly weaker preconditioner. A block that is
// not SPD in FP64 (round-off with tiny damping) falls back to the square root
// of its diagonal.
//
// One camera per lane: the 45 packed entries live in registers (fully
// unrolled, constant indices), so every FP64 instruction serves 32 cameras.
// GB300's FP64 pipe takes the same time for a warp instruction whatever its
// active lanes: a CTA per camera (one thread per entry, 1-8 active lanes per
// step) took 80 us per launch on 5,000 cameras, this 37 us. The pivot
// reciprocal scales the column.
constexpr int kSL = 32;  // threads (= cameras) per block of the per-lane kernels

__device__ __forceinline__ void chol9_lane(double (&a)[45]) {
    double d0[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) d0[i] = a[blk::tri(i, i)];
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        const double d = a[blk::tri(k, k)];
        ok = ok && d > 0.0;
        const double l = sqrt(d > 0.0 ? d : 1.0);
        a[blk::tri(k, k)] = l;
        const double r = 1.0 / l;
#pragma unroll
        for (int i = k + 1; i < 9; ++i) a[blk::tri(i, k)] *= r;
#pragma unroll
        for (int j = k + 1; j < 9; ++j)
#pragma unroll
            for (int i = j; i < 9; ++i) a[blk::tri(i, j)] -= a[blk::tri(i, k)] * a[blk::tri(j, k)];
    }
    if (!ok) {
#pragma unroll
        for (int i = 0; i < 9; ++i)
#pragma unroll
            for (int j = 0; j <= i; ++j)
                a[blk::tri(i, j)] = i == j ? sqrt(d0[i] > 1e-300 ? d0[i] : 1e-300) : 0.0;
    }
}

// Explicit block inverse M_c = (L L^T)^-1 = X^T X with X = L^-1, from the
// factor in registers (one camera per lane). X overwrites L column by column
// (column j of X needs L_ij only for its own entry X_ij, and L's later
// columns); sums run in increasing k. M is stored in FP32: it is the inner
// PCG's block-Jacobi preconditioner, applied to FP32 vectors.
__device__ __forceinline__ void inverse_from_factor_lane(double (&x)[45], float* __restrict__ M) {
    double rd[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) rd[i] = 1.0 / x[blk::tri(i, i)];
#pragma unroll
    for (int j = 0; j < 9; ++j) {
        x[blk::tri(j, j)] = rd[j];
#pragma unroll
        for (int i = j + 1; i < 9; ++i) {
            double t = -(x[blk::tri(i, j)] * x[blk::tri(j, j)]);
#pragma unroll
            for (int k = j + 1; k < i; ++k) t -= x[blk::tri(i, k)] * x[blk::tri(k, j)];
            x[blk::tri(i, j)] = t * rd[i];
        }
    }
#pragma unroll
    for (int a = 0; a < 9; ++a)
#pragma unroll
        for (int b = 0; b <= a; ++b) {
            double m = 0.0;
#pragma unroll
            for (int k = a; k < 9; ++k) m += x[blk::tri(k, a)] * x[blk::tri(k, b)];
            M[9 * a + b] = static_cast<float>(m);
            M[9 * b + a] = static_cast<float>(m);
        }
}

// One camera per lane: S_cc = U_lambda,c - (chunk sums from the right-hand
// side pass, in chunk order), stored full FP64, its block-Jacobi factor and
// the explicit inverse (FP32).
__global__ void __launch_bounds__(kSL) sdiag_finalize_lane(const int* __restrict__ cam_chunk_off,
                                                          const double* __restrict__ part,
                                                          const double* __restrict__ U, double lambda, int C,
                                                          double* __restrict__ Sdiag, double* __restrict__ L,
                                                          float* __restrict__ Minv) {
    const int c = blockIdx.x * kSL + threadIdx.x;
    if (c >= C) return;
    const double* Uc = U + 81ll * c;
    double a[45];
#pragma unroll
    for (int t = 0; t < 45; ++t) a[t] = 0.0;
    const int q1 = cam_chunk_off[c + 1];
    for (int q = cam_chunk_off[c]; q < q1; ++q) {
        const double* pq = part + 54ll * q + 9;
#pragma unroll
        for (int t = 0; t < 45; ++t) a[t] += pq[t];
    }
#pragma unroll
    for (int i = 0; i < 9; ++i)
#pragma unroll
        for (int j = 0; j <= i; ++j) {
            double v = Uc[9 * i + j] - a[blk::tri(i, j)];
            if (i == j) v += lambda * (Uc[10 * i] > 0.0 ? Uc[10 * i] : 1e-12);
            a[blk::tri(i, j)] = v;
        }
    double* Sc = Sdiag + 81ll * c;
#pragma unroll
    for (int i = 0; i < 9; ++i)
#pragma unroll
        for (int j = 0; j < 9; ++j) Sc[9 * i + j] = a[i >= j ? blk::tri(i, j) : blk::tri(j, i)];
    chol9_lane(a);
    double* Lc = L + 45ll * c;
#pragma unroll
    for (int t = 0; t < 45; ++t) Lc[t] = a[t];
    inverse_from_factor_lane(a, Minv + 81ll * c);
}

}  // namespace

// Launch of a kernel of the PCG iteration chain with programmatic stream
// serialization: it may be scheduled while the kernel before it finishes, and
// waits for it in pdl_wait().
template <typename... KArgs, typename... Args>
static void launch_chained(void (*kernel)(KArgs...), int grid, int block, cudaStream_t stream, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(static_cast<unsigned>(grid));
    cfg.blockDim = dim3(static_cast<unsigned>(block));
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    GBA_CUDA_CHECK(cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...));
    count_launch();
}

// Implicit product partials for a given x (FP32 or float-float arithmetic). x
// is in the arithmetic type (FP32: the PCG direction copy; float-float: dc) or
// null (then a = 1: the right-hand side). Partials in cam_part_ (9 per chunk).
template <typename T>
static void implicit_parts(Solver& s, const T* x, double a, const double* done) {
    T* u = reinterpret_cast<T*>(s.u_.get());
    const bool f32 = sizeof(T) == 4;
    const bool rhs = x == nullptr;  // right-hand side: also the block-Jacobi diagonal-block partials
    float4* g = rhs ? reinterpret_cast<float4*>(s.g_cm_.get()) : nullptr;
    cudaEvent_t ev = s.prof_start();
    (rhs ? schur_point_pass<T, false, true> : schur_point_pass<T, false, false>)<<<s.n_pchunk_, kPT, 0, s.stream_>>>(reinterpret_cast<const int4*>(s.pchunk4_.get()), s.pchunk_.get(), s.pt_off_.get(), s.s_cam_.get(),
                                                           s.s_pt_.get(), s.cam_pos_.get(), s.Jc32_.get(), s.Jp32_.get(), s.js_,
                                                           s.Vinv32_.get(), s.Vinv32lo_.get(), s.bp_.get(), x, a,
                                                           u, done, BacksubOut{}, g);
    GBA_LAUNCH_CHECK();
    s.prof_stop(rhs ? "schur_rhs_point_pass" : f32 ? "schur_point_pass_f32" : "schur_point_pass_ff", ev);
    if (s.n_cchunk_ > 0) {
        ev = s.prof_start();
        if (rhs) {
            schur_camera_pass<T, true><<<s.n_cchunk_, kCT, 0, s.stream_>>>(
                s.cchunk_begin_.get(), s.cchunk_cam_.get(), s.cam_off_.get(), s.J32c_.get(), u, s.cam_part_.get(),
                done, g);
        } else {
            schur_camera_pass<T><<<s.n_cchunk_, kCT, 0, s.stream_>>>(s.cchunk_begin_.get(), s.cchunk_cam_.get(),
                                                                     s.cam_off_.get(), s.J32c_.get(), u,
                                                                     s.cam_part_.get(), done, nullptr);
        }
        GBA_LAUNCH_CHECK();
        s.prof_stop(rhs ? "schur_rhs_camera_pass" : f32 ? "schur_camera_pass_f32" : "schur_camera_pass_ff", ev);
    }
}

// Camera pass of a float-float product whose u the point pass has stored:
// partials of sum Jc^T u per camera chunk in cam_part_.
static void camera_parts_ff(Solver& s) {
    if (s.n_cchunk_ == 0) return;
    cudaEvent_t ev = s.prof_start();
    schur_camera_pass<ff><<<s.n_cchunk_, kCT, 0, s.stream_>>>(s.cchunk_begin_.get(), s.cchunk_cam_.get(),
                                                             s.cam_off_.get(), s.J32c_.get(),
                                                             reinterpret_cast<const ff*>(s.u_.get()),
                                                             s.cam_part_.get(), nullptr, nullptr);
    GBA_LAUNCH_CHECK();
    s.prof_stop("schur_camera_pass_ff", ev);
}

// The one-pass FP32 product (schur_point_pass with kAcc): y = sum over slots of
// Jc^T u, accumulated in device memory (acc_id_: the slot's accumulator).
static void implicit_parts_acc(Solver& s, const float* x, const double* done) {
    cudaEvent_t ev = s.prof_start();
    if (s.n_wchunk_ > 0) {
        launch_chained(schur_matvec_warp, ceil_div(s.n_wchunk_, kMWarps), 32 * kMWarps, s.stream_,
                       reinterpret_cast<const int2*>(s.wchunk_.get()), s.n_wchunk_, s.s_cam_.get(), s.s_pt_.get(),
                       s.acc_id_.get(), s.Jc32_.get(), s.Jp32_.get(), s.js_, s.Vinv32_.get(), x, s.y_acc_.get(),
                       done);
    }
    if (s.n_lchunk_ > 0) {  // points with 33 to 256 observations, packed per CTA
        launch_chained(schur_matvec_long, s.n_lchunk_, kPT, s.stream_,
                       reinterpret_cast<const int2*>(s.lchunk_.get()), s.lpts_.get(), s.pt_off_.get(),
                       s.s_cam_.get(), s.acc_id_.get(), s.Jc32_.get(), s.Jp32_.get(), s.js_, s.Vinv32_.get(), x,
                       s.y_acc_.get(), done);
    }
    if (s.n_huge_ > 0) {  // points with more than 256 observations, one range each
        schur_point_pass<float, false, false, true><<<s.n_huge_, kPT, 0, s.stream_>>>(
            reinterpret_cast<const int4*>(s.huge_range_.get()), nullptr, s.pt_off_.get(), s.s_cam_.get(),
            s.s_pt_.get(), s.acc_id_.get(), s.Jc32_.get(), s.Jp32_.get(), s.js_, s.Vinv32_.get(), nullptr,
            s.bp_.get(), x, 0.0, s.y_acc_.get(), done, BacksubOut{}, nullptr);
        GBA_LAUNCH_CHECK();
    }
    s.prof_stop("schur_matvec_f32", ev);
}

void launch_split_ff(const double* x, long long n, float* out, cudaStream_t s) {
    if (n <= 0) return;
    split_kernel<<<ceil_div(n, kVT), kVT, 0, s>>>(x, n, out);
    GBA_LAUNCH_CHECK();
}

// Mixed-form back-substitution: the point pass in back-substitution mode (dp,
// trial points and their float-float split, denominator partials per chunk),
// in the arithmetic of the last Schur solve: FP32 after a loose solve,
// float-float otherwise. dc is in that arithmetic (pcg_p32_ padded FP32, or
// dcff_). with_u (float-float only): also u = -Jp dp per slot into u_, for the
// camera pass of the refinement check.
void mixed_back_substitute(Solver& s, double lambda, double* part, bool with_u) {
    const BacksubOut bk{s.V_.get(), s.pts_.get(),
                        make_float2(static_cast<float>(lambda), static_cast<float>(lambda - static_cast<float>(lambda))),
                        s.dp_.get(), s.tpts_.get(), reinterpret_cast<float2*>(s.pts_ff_.get()), part};
    if (s.fast_solve_) {
        schur_point_pass<float, true><<<s.n_pchunk_, kPT, 0, s.stream_>>>(
            reinterpret_cast<const int4*>(s.pchunk4_.get()), s.pchunk_.get(), s.pt_off_.get(), s.s_cam_.get(), s.s_pt_.get(), s.cam_pos_.get(), s.Jc32_.get(), s.Jp32_.get(), s.js_,
            s.Vinv32_.get(), nullptr, s.bp_.get(), s.pcg_p32_.get(), -1.0, nullptr, nullptr, bk, nullptr);
    } else {
        schur_point_pass<ff, true><<<s.n_pchunk_, kPT, 0, s.stream_>>>(
            reinterpret_cast<const int4*>(s.pchunk4_.get()), s.pchunk_.get(), s.pt_off_.get(), s.s_cam_.get(), s.s_pt_.get(), s.cam_pos_.get(), s.Jc32_.get(), s.Jp32_.get(), s.js_,
            s.Vinv32_.get(), s.Vinv32lo_.get(), s.bp_.get(), reinterpret_cast<const ff*>(s.dcff_.get()), -1.0,
            with_u ? reinterpret_cast<ff*>(s.u_.get()) : nullptr, nullptr, bk, nullptr);
    }
    GBA_LAUNCH_CHECK();
    s.ff_holds_ = Solver::kFfNone;  // pts_ff_ holds the trial points now
    s.pts_ff_trial_ = true;
}

PcgStats Solver::schur_pcg(double lambda, const LMOptions& opts, bool learned) {
    return schur_pcg(lambda, opts, learned, nullptr);
}

PcgStats Solver::schur_pcg(double lambda, const LMOptions& opts, bool learned, unsigned long long* nonspd_out) {
    PcgStats st;
    const int n = 9 * C_;
    const int nvb = ceil_div(n, kVT);   // vector blocks (element-wise kernels)
    const int ncb = ceil_div(C_, kCB);  // camera blocks (thread-per-camera kernels)
    const int nub = ceil_div(C_, kUC);  // camera blocks (nine-threads-per-camera kernels)
    double* red = red_part_.get();
    double* red2 = red_part_.get() + std::max(nvb, ncb) + 1;
    double* sc = pcg_s_.get();
    const double* done = sc + S_DONE;

    // Loose targets (refine_tol >= kLooseTol) are far above the FP32 operator's
    // rounding (~1e-6 relative): the right-hand side and back-substitution run
    // in FP32 and a converged inner solve is its own residual check. Tighter
    // targets use float-float products for both and an explicit residual.
    const bool fast = opts.refine_tol >= kLooseTol;
    fast_solve_ = fast;
    backsub_ready_ = false;
    if (fast) {
        implicit_parts<float>(*this, static_cast<const float*>(nullptr), 1.0, nullptr);
    } else {
        implicit_parts<ff>(*this, static_cast<const ff*>(nullptr), 1.0, nullptr);
    }
    rhs_finalize<<<nvb, kVT, 0, stream_>>>(cam_chunk_off_.get(), cam_part_.get(), bc_.get(), C_, rhs_.get(),
                                           ref_r_.get(), dc_.get(), red);
    GBA_LAUNCH_CHECK();
    sum_to_scalar<<<1, 256, 0, stream_>>>(red, nvb, sc, S_NORM);
    GBA_LAUNCH_CHECK();

    // block-Jacobi blocks (partials from the right-hand side pass), factors and
    // explicit inverses
    cudaEvent_t bj_ev = prof_start();
    sdiag_finalize_lane<<<ceil_div(C_, kSL), kSL, 0, stream_>>>(cam_chunk_off_.get(), cam_part_.get(), U_.get(), lambda,
                                                               C_, Sdiag_.get(), Pfac_.get(), Pinv_.get());
    GBA_LAUNCH_CHECK();
    damped_u32_kernel<<<ceil_div(81ll * C_, kVT), kVT, 0, stream_>>>(U_.get(), lambda, C_, ul32_.get());
    GBA_LAUNCH_CHECK();
    prof_stop("bj_blocks", bj_ev);
    if (learned && !model_) throw std::invalid_argument("learned form: no model loaded");
    if (learned && precond_force_ != 0) learned_choice_ = precond_force_;

    double bnorm2 = 0.0;
    unsigned long long nonspd = 0;
    read_back({{&bnorm2, sc + S_NORM, sizeof bnorm2}, {&nonspd, counters_.get() + 3, sizeof nonspd}});
    if (nonspd_out) *nonspd_out = nonspd;
    if (nonspd_out && *nonspd_out) {  // a non-SPD damped point block: the trial is rejected
        st.rel_residual = NAN;
        return st;
    }
    if (!std::isfinite(bnorm2)) {
        st.rel_residual = NAN;
        return st;
    }
    if (bnorm2 == 0.0) {
        st.converged = true;
        return st;
    }
    double rnorm2 = bnorm2;
    const double tol2 = opts.refine_tol * opts.refine_tol * bnorm2;
    // The learned coarse space (basis, S Z, E^-1) is formed once per trial, when
    // an inner solve first needs it.
    bool coarse_ready = false;
    // Inner PCG on the FP32 operator, S32 e = r (e in pcg_e_, FP32), preconditioned by
    // block-Jacobi, or by the balancing two-level form with the learned coarse
    // basis (coarse). Returns the iteration count; *ok = reached the inner
    // tolerance without breakdown; inner_rel2 = its final ||r||^2 / ||b||^2.
    double inner_rel2 = 0.0;
    auto inner_pcg = [&](bool* ok, bool coarse, int max_iters) -> long long {
        if (coarse && !coarse_ready) {
            coarse_prepare(lambda);
            coarse_ready = true;
        }
        const float* Zc = coarse ? cz32_.get() : nullptr;
        double* red_zr = cred_.get();
        double* red_szw = red_zr + 1ll * nub * kCoarse;
        double* c1 = red_szw + 1ll * nub * kCoarse;
        pcg_init<<<nub, kUT, 0, stream_>>>(pcg_e_.get(), pcg_r_.get(), pcg_z_.get(), pcg_p32_.get(), ref_r_.get(),
                                           Pinv_.get(), C_, red, red2, Zc, red_zr);
        GBA_LAUNCH_CHECK();
        if (coarse) {
            coarse_w<<<nub, kUT, 0, stream_>>>(pcg_r_.get(), csz32_.get(), Pinv_.get(), ceinv_.get(), C_, red_zr, nub,
                                               c1, pcg_z_.get(), red_szw, sc, 1);
            GBA_LAUNCH_CHECK();
            coarse_z<<<nub, kUT, 0, stream_>>>(pcg_r_.get(), Zc, ceinv_.get(), C_, red_szw, nub, c1, pcg_z_.get(),
                                               pcg_p32_.get(), red2, sc, 1);
            GBA_LAUNCH_CHECK();
        }
        pcg_init_finalize<<<1, 256, 0, stream_>>>(red, red2, nub, opts.pcg_tol, sc);
        GBA_LAUNCH_CHECK();
        // p.q partials (nvb) and r.r / r.z partials (nub) in disjoint ranges
        double* red_pq = red2 + nub + 1;
        // p.q partials: one per finalize block (one warp per camera for the
        // one-pass product's accumulators)
        const int npq = one_pass_ ? ceil_div(C_, kVT / 32) : nvb;
        // Launch batches sized from the previous inner solve's iteration count
        // (then 1, 2, 4, 8, 8, ...): a launch after convergence returns at once
        // but still dispatches its whole grid (tens of microseconds for the
        // point pass), so overshooting costs more than one extra check.
        int batch = std::max(1, std::min(prev_inner_ - 1, std::min(kCheck, max_iters)));
        double h[9];
        if (max_iters <= 0) read_back({{h, sc, sizeof h}});  // the state pcg_init_finalize left
        for (int it = 0, next = 1; it < max_iters; it += batch, batch = std::min(next, kCheck), next *= 2) {
            for (int j = 0; j < batch; ++j) {
                if (one_pass_) {
                    implicit_parts_acc(*this, pcg_p32_.get(), done);
                    cudaEvent_t fev = prof_start();
                    launch_chained(pcg_q_finalize_acc, npq, kVT, stream_, y_acc_.get(), acc_off_.get(),
                                   ul32_.get(), pcg_p32_.get(), C_, pcg_q_.get(), red_pq, sc);
                    prof_stop("pcg_q_finalize", fev);
                } else {
                    implicit_parts<float>(*this, pcg_p32_.get(), 0.0, done);
                    cudaEvent_t fev = prof_start();
                    pcg_q_finalize<<<nvb, kVT, 0, stream_>>>(cam_chunk_off_.get(), cam_part_.get(), ul32_.get(),
                                                             pcg_p32_.get(), C_, pcg_q_.get(), red_pq, sc);
                    GBA_LAUNCH_CHECK();
                    prof_stop("pcg_q_finalize", fev);
                }
                launch_chained(pcg_update, nub, kUT, stream_, pcg_e_.get(), pcg_r_.get(), pcg_z_.get(),
                               pcg_p32_.get(), pcg_q_.get(), Pinv_.get(), C_, red_pq, npq, red, red2, sc, Zc, red_zr);
                if (coarse) {
                    cudaEvent_t cev = prof_start();
                    launch_chained(coarse_w, nub, kUT, stream_, pcg_r_.get(), csz32_.get(), Pinv_.get(),
                                   ceinv_.get(), C_, red_zr, nub, c1, pcg_z_.get(), red_szw, sc, 0);
                    launch_chained(coarse_z, nub, kUT, stream_, pcg_r_.get(), Zc, ceinv_.get(), C_, red_szw, nub,
                                   c1, pcg_z_.get(), static_cast<float*>(nullptr), red2, sc, 0);
                    prof_stop("coarse_apply", cev);
                }
                launch_chained(pcg_direction, nvb, kVT, stream_, pcg_p32_.get(), pcg_z_.get(), n, red, red2, nub,
                               max_iters, sc);
            }
            read_back({{h, sc, sizeof h}});
            if (h[S_DONE] != 0.0) break;
        }
        *ok = h[S_DONE] != 2.0 && h[S_RR] <= h[S_TOL2] * h[S_BB];
        inner_rel2 = h[S_BB] > 0.0 ? h[S_RR] / h[S_BB] : 0.0;
        prev_inner_ = static_cast<int>(h[S_ITERS]);
        return static_cast<long long>(h[S_ITERS]);
    };
    // b . x of the inner solution pcg_e_ (b = ref_r_, the inner right-hand side) into sc[slot]
    auto btx = [&](int slot) {
        dot_partials<<<nvb, kVT, 0, stream_>>>(ref_r_.get(), pcg_e_.get(), n, red);
        GBA_LAUNCH_CHECK();
        sum_to_scalar<<<1, 256, 0, stream_>>>(red, nvb, sc, slot);
        GBA_LAUNCH_CHECK();
    };
    bool use_learned = learned && learned_choice_ == 1;
    for (int step = 0; step < opts.refine_max_steps && rnorm2 > tol2; ++step) {
        bool ok = false;
        long long it_count = 0;
        if (learned && learned_choice_ == 0) {
            // Block-Jacobi judges the learned correction on the first inner solve
            // of the LM solve: both preconditioners solve it; the learned one
            // serves the rest of the solve if it needed at most 4/5 of
            // block-Jacobi's iterations and its step is no worse in the S-norm.
            // For PCG iterates from x = 0, ||x* - x||_S^2 = b.x* - b.x, so the
            // step with the larger b.x has the smaller S-norm error. The learned
            // solve runs first; block-Jacobi then stops once it has used 5/4 of
            // the learned iterations, past which it cannot win. Both solves
            // count in pcg_iterations.
            bool ok_bj = false, ok_l = false;
            const long long it_l = inner_pcg(&ok_l, true, opts.pcg_max_iters);
            const double rel2_l = inner_rel2;
            btx(S_BTX1);
            GBA_CUDA_CHECK(cudaMemcpyAsync(judge_e_.get(), pcg_e_.get(), n * sizeof(float),
                                           cudaMemcpyDeviceToDevice, stream_));
            const long long cap =
                ok_l ? std::min<long long>(opts.pcg_max_iters, (it_l * kLearnedWinDen + kLearnedWinNum - 1) / kLearnedWinNum)
                     : opts.pcg_max_iters;
            const long long it_bj = inner_pcg(&ok_bj, false, static_cast<int>(cap));
            btx(S_BTX0);
            double bx[2];
            read_back({{bx, sc + S_BTX0, sizeof bx}});
            judge_iters_[0] = it_bj;
            judge_iters_[1] = it_l;
            judge_btx_[0] = bx[0];
            judge_btx_[1] = bx[1];
            // Solves shorter than kJudgeMin iterations are too short to compare:
            // keep block-Jacobi for now and judge again at the next inner solve.
            // After kJudgeAttempts indecisive judgements block-Jacobi is kept:
            // judging costs a second solve each time. With an inner tolerance of
            // kShortInnerTol or looser every later solve is as short, so one
            // indecisive judgement settles it.
            ++judge_attempts_;
            const int attempts = opts.pcg_tol >= kShortInnerTol ? 1 : kJudgeAttempts;
            const bool decisive = std::max(it_bj, it_l) >= kJudgeMin || !ok_bj || !ok_l;
            const bool no_worse = bx[1] >= bx[0] * (1.0 - opts.pcg_tol * opts.pcg_tol);
            if (decisive && ok_l && (!ok_bj || (it_l * kLearnedWinDen <= it_bj * kLearnedWinNum && no_worse))) {
                learned_choice_ = 1;
                use_learned = true;
                inner_rel2 = rel2_l;
                GBA_CUDA_CHECK(cudaMemcpyAsync(pcg_e_.get(), judge_e_.get(), n * sizeof(float),
                                               cudaMemcpyDeviceToDevice, stream_));
                st.pcg_iterations += it_bj;
                it_count = it_l;
                ok = ok_l;
            } else {
                // block-Jacobi's solve is in pcg_e_ (it ran last, and was not
                // stopped early: a stopped run leaves ok_bj false, and the
                // learned solve, converged, wins then)
                learned_choice_ = (decisive || judge_attempts_ >= attempts) ? 2 : 0;
                st.pcg_iterations += it_l;
                it_count = it_bj;
                ok = ok_bj;
            }
        } else {
            it_count = inner_pcg(&ok, use_learned, opts.pcg_max_iters);
        }
        if (use_learned && !ok && precond_force_ != 1) {
            // Block-Jacobi is the fallback: an inner solve with the coarse
            // correction that breaks down or misses its tolerance is redone with
            // block-Jacobi alone, which then serves for the rest of this trial
            // (not when the caller forced the learned correction on).
            use_learned = false;
            ++st.fallbacks;
            st.pcg_iterations += it_count;
            it_count = inner_pcg(&ok, false, opts.pcg_max_iters);
        }
        const double iters = static_cast<double>(it_count);
        if (fast && step == 0 && ok && inner_rel2 <= tol2 / bnorm2) {
            // dc = e (dc is 0 before the first step), with the inner solve's
            // residual as the check
            axpy_split_kernel<<<nvb, kVT, 0, stream_>>>(dc_.get(), pcg_e_.get(), n, dcff_.get());
            GBA_LAUNCH_CHECK();
            rnorm2 = inner_rel2 * bnorm2;
            st.pcg_iterations += static_cast<long long>(iters);
            ++st.refine_steps;
            break;
        }
        // dc += e; residual r = rhs - S dc in float-float products, FP64 sums
        axpy_split_kernel<<<nvb, kVT, 0, stream_>>>(dc_.get(), pcg_e_.get(), n, dcff_.get());
        GBA_LAUNCH_CHECK();
        if (step == 0 || fast) {
            implicit_parts<ff>(*this, reinterpret_cast<const ff*>(dcff_.get()), 0.0, nullptr);
            residual_finalize<<<nvb, kVT, 0, stream_>>>(cam_chunk_off_.get(), cam_part_.get(), U_.get(), lambda,
                                                        dc_.get(), rhs_.get(), C_, ref_r_.get(), red);
            GBA_LAUNCH_CHECK();
            backsub_ready_ = false;
        } else {
            // A later step usually ends the refinement (float-float targets),
            // so its check runs the back-substitution: with
            // dp = V'^-1 (bp - W^T dc) the residual rhs - S dc equals
            // bc - U_lambda dc - W dp, and the point pass of the
            // back-substitution (dp, trial points, denominator partials) also
            // stores u = -Jp dp, whose camera pass sums are -W dp. The
            // back-substitution of the trial then reuses this pass.
            cudaEvent_t bev = prof_start();
            mixed_back_substitute(*this, lambda, backsub_part(), true);
            prof_stop("backsub", bev);
            camera_parts_ff(*this);
            residual_finalize<<<nvb, kVT, 0, stream_>>>(cam_chunk_off_.get(), cam_part_.get(), U_.get(), lambda,
                                                        dc_.get(), bc_.get(), C_, ref_r_.get(), red);
            GBA_LAUNCH_CHECK();
            backsub_ready_ = true;
        }
        sum_to_scalar<<<1, 256, 0, stream_>>>(red, nvb, sc, S_NORM);
        GBA_LAUNCH_CHECK();
        read_back({{&rnorm2, sc + S_NORM, sizeof rnorm2}});
        st.pcg_iterations += static_cast<long long>(iters);
        ++st.refine_steps;
        if (!std::isfinite(rnorm2)) break;
    }
    st.rel_residual = std::sqrt(rnorm2 / bnorm2);
    st.converged = rnorm2 <= tol2;
    return st;
}

// Learned coarse space for this trial: the basis Z from the network at the
// current cameras, SZ = S Z (one FP32 implicit product for all kCoarse columns,
// FP64 finalize; Z and SZ also in FP32 for the PCG), and
// E^-1 = (Z^T S Z)^-1 (FP64 Cholesky on the device; flagged off if E is not SPD).
void Solver::coarse_prepare(double lambda) {
    const int n = 9 * C_;
    const int nvb = ceil_div(n, kVT);
    const int nub = ceil_div(C_, kUC);
    const size_t need_red = 2ull * nub * kCoarse + kCoarse + 1ull * nvb * kCoarse * kCoarse;
    if (!cz_.get()) {
        StreamAllocScope scope(stream_);
        cz_.alloc(1ull * kCoarse * n);
        csz_.alloc(1ull * kCoarse * n);
        cz32_.alloc(1ull * kCoarse * n);
        csz32_.alloc(1ull * kCoarse * n);
        ceinv_.alloc(kCoarse * kCoarse + 1);
        cred_.alloc(need_red);
        czb_.alloc(1ull * kZs * C_);
        cu9_.alloc(static_cast<size_t>(kU9) * E_);
        cpart9_.alloc(81ull * std::max(n_cchunk_, 1));
    }
    cudaEvent_t ev = prof_start();
    cudaEvent_t ev1 = prof_start();
    model_->coarse_basis(*this, lambda, cz_.get());
    coarse_zb_kernel<<<ceil_div(81ll * C_, kVT), kVT, 0, stream_>>>(cz_.get(), C_, czb_.get(), cz32_.get());
    GBA_LAUNCH_CHECK();
    prof_stop("coarse_basis", ev1);
    ev1 = prof_start();
    if (n_wchunk_ > 0) {
        coarse_point_pass9_warp<<<ceil_div(n_wchunk_, kMWarps), 32 * kMWarps, 0, stream_>>>(
            reinterpret_cast<const int2*>(wchunk_.get()), n_wchunk_, s_cam_.get(), s_pt_.get(), cam_pos_.get(),
            Jc32_.get(), Jp32_.get(), js_, Vinv32_.get(), czb_.get(), cu9_.get());
        GBA_LAUNCH_CHECK();
    }
    if (n_lchunk_ > 0) {
        coarse_point_pass9_list<<<n_lchunk_, kPT, 0, stream_>>>(
            reinterpret_cast<const int2*>(lchunk_.get()), lpts_.get(), pt_off_.get(), s_cam_.get(), cam_pos_.get(),
            Jc32_.get(), Jp32_.get(), js_, Vinv32_.get(), czb_.get(), cu9_.get());
        GBA_LAUNCH_CHECK();
    }
    if (n_huge_ > 0) {
        coarse_point_pass9<<<n_huge_, kPT, 0, stream_>>>(reinterpret_cast<const int4*>(huge_range_.get()),
                                                         pt_off_.get(), s_cam_.get(), s_pt_.get(), cam_pos_.get(),
                                                         Jc32_.get(), Jp32_.get(), js_, Vinv32_.get(), czb_.get(),
                                                         cu9_.get());
        GBA_LAUNCH_CHECK();
    }
    prof_stop("coarse_point_pass9", ev1);
    if (n_cchunk_ > 0) {
        ev1 = prof_start();
        coarse_camera_pass9<<<n_cchunk_, kC9, 0, stream_>>>(cchunk_begin_.get(), cchunk_cam_.get(), cam_off_.get(),
                                                            J32c_.get(), cu9_.get(), cpart9_.get());
        GBA_LAUNCH_CHECK();
        prof_stop("coarse_camera_pass9", ev1);
    }
    ev1 = prof_start();
    coarse_sz_finalize<<<ceil_div(81ll * C_, kVT), kVT, 0, stream_>>>(cam_chunk_off_.get(), cpart9_.get(), U_.get(),
                                                                      lambda, cz_.get(), C_, csz_.get(),
                                                                      csz32_.get());
    GBA_LAUNCH_CHECK();
    double* gram = cred_.get() + 2ll * nub * kCoarse + kCoarse;
    coarse_gram_partials<<<nvb, kVT, 0, stream_>>>(cz_.get(), csz_.get(), n, gram);
    GBA_LAUNCH_CHECK();
    coarse_einv_kernel<<<1, kEinvT, 0, stream_>>>(gram, nvb, ceinv_.get());
    GBA_LAUNCH_CHECK();
    prof_stop("coarse_gram", ev1);
    prof_stop("coarse_prepare", ev);
}

void Solver::set_matvec(int mode) {
    if (form_ == SolverForm::Plain) throw std::invalid_argument("the PCG product belongs to the mixed forms");
    if (mode < 0 || mode > 2) throw std::invalid_argument("matvec mode: 0 auto, 1 two-pass, 2 one-pass");
    one_pass_ = mode != 1;
    if (one_pass_ && !y_acc_.get()) {
        const size_t n = static_cast<size_t>(kX32) * std::max(n_acc_, 1);
        y_acc_.alloc(n);
        GBA_CUDA_CHECK(cudaMemsetAsync(y_acc_.get(), 0, n * sizeof(float), stream_));
    }
}

// Point groups of the warp-level point passes (the one-pass product and the
// coarse S Z): whole points packed greedily into runs of at most 32 slots
// (wchunk_), points with 33 to 256 observations into lists of at most 256
// slots (lchunk_, lpts_), longer points as single ranges (huge_range_).
void Solver::build_point_groups() {
    // warp chunks: whole points packed greedily into runs of at most 32
    // slots; points with more observations get a range of their own
    std::vector<int> off(P_ + 1);
    GBA_CUDA_CHECK(cudaMemcpyAsync(off.data(), pt_off_.get(), (P_ + 1ull) * sizeof(int), cudaMemcpyDeviceToHost,
                                   stream_));
    sync();
    std::vector<int2> wc, lc;
    std::vector<int> lp;
    std::vector<int4> hr;
    int b = -1, e = -1, lsum = 0;
    for (int p = 0; p < P_; ++p) {
        const int n = off[p + 1] - off[p];
        if (n == 0) continue;
        if (n > kPT) {
            hr.push_back(make_int4(p, p + 1, off[p], off[p + 1]));
            continue;
        }
        if (n > 32) {  // into the current long-point CTA list, or a new one
            if (lc.empty() || lsum + n > kPT) {
                lc.push_back(make_int2(static_cast<int>(lp.size()), 0));
                lsum = 0;
            }
            lp.push_back(p);
            ++lc.back().y;
            lsum += n;
            continue;
        }
        if (b >= 0 && (off[p] != e || off[p + 1] - b > 32)) {
            wc.push_back(make_int2(b, e));
            b = -1;
        }
        if (b < 0) b = off[p];
        e = off[p + 1];
    }
    if (b >= 0) wc.push_back(make_int2(b, e));
    n_wchunk_ = static_cast<int>(wc.size());
    n_lchunk_ = static_cast<int>(lc.size());
    n_huge_ = static_cast<int>(hr.size());
    wchunk_.alloc(2 * std::max<size_t>(wc.size(), 1));
    lchunk_.alloc(2 * std::max<size_t>(lc.size(), 1));
    lpts_.alloc(std::max<size_t>(lp.size(), 1));
    huge_range_.alloc(4 * std::max<size_t>(hr.size(), 1));
    if (!wc.empty())
        GBA_CUDA_CHECK(cudaMemcpyAsync(wchunk_.get(), wc.data(), wc.size() * sizeof(int2), cudaMemcpyHostToDevice,
                                       stream_));
    if (!lc.empty()) {
        GBA_CUDA_CHECK(cudaMemcpyAsync(lchunk_.get(), lc.data(), lc.size() * sizeof(int2), cudaMemcpyHostToDevice,
                                       stream_));
        GBA_CUDA_CHECK(cudaMemcpyAsync(lpts_.get(), lp.data(), lp.size() * sizeof(int), cudaMemcpyHostToDevice,
                                       stream_));
    }
    if (!hr.empty())
        GBA_CUDA_CHECK(cudaMemcpyAsync(huge_range_.get(), hr.data(), hr.size() * sizeof(int4),
                                       cudaMemcpyHostToDevice, stream_));
    sync();
}

}  // namespace gba

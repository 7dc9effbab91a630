// Normal-equation accumulation (edge kernels) and the trial-cost kernels.
//
// Replaces the reference edge_kernel / cost_kernel (src/lm.cu:205-281), which
// accumulate U, V, bc, bp and the SSE with global FP64 atomics in file order.
// Here every sum is atomic-free and deterministic:
//   point pass   one CTA per point chunk (whole points, <= 256 slots, slots
//                sorted by point): Jacobian per slot, per-edge W (plain form) or
//                the FP32 Jacobian rows and camera records (mixed forms), and
//                V / bp as in-CTA ordered sums.
//   camera pass  one CTA per camera chunk (<= 1024 slots of one camera, from the
//                camera-major view): U / bc partial sums per chunk, then a
//                finalize kernel adds the chunk partials of each camera in order.
//   cost         FP64 per slot (plain form); float-float per camera-major
//                position with the camera's constants in shared memory (mixed
//                forms), FP64 for positions outside FP32's range.
// Non-finite edges contribute nothing, bump counters[0] and get W = 0
// (reference semantics src/lm.cu:219-225; the reference leaves W stale).

#include "camera_model.cuh"
#include "common.cuh"
#include "ff.cuh"
#include "solver.hpp"

namespace gba {
namespace {

constexpr int kPT = 256;       // point-pass threads (= max slots per chunk)
constexpr int kCT = 128;       // camera-pass threads
constexpr int kCamChunk = 1024;
constexpr int kCamRec = 28;    // floats per camera record of the FP32 Jacobian pass

template <typename T>
__device__ __forceinline__ bool all_finite(const T* v, int n) {
    bool ok = true;
#pragma unroll
    for (int i = 0; i < n; ++i) ok = ok && isfinite(v[i]);
    return ok;
}

// ---------------------------------------------------------------- FP64 path

__global__ void __launch_bounds__(kPT) point_pass_f64(
    const int* __restrict__ pchunk, const int* __restrict__ pt_off, const int* __restrict__ s_cam,
    const int* __restrict__ s_pt, const double2* __restrict__ s_px, const double* __restrict__ cams,
    const double* __restrict__ pts, double* __restrict__ W, double* __restrict__ JcR, double* __restrict__ V,
    double* __restrict__ bp, double* __restrict__ sse_part, unsigned long long* __restrict__ counters,
    double delta) {
    __shared__ double contrib[9][kPT];
    __shared__ double red[kPT / 32];
    __shared__ unsigned long long redu[kPT / 32];
    const int chunk = blockIdx.x;
    const int p0 = pchunk[chunk], p1 = pchunk[chunk + 1];
    const int s0 = pt_off[p0], s1 = pt_off[p1];
    const int my_p = p0 + threadIdx.x;
    int my_b = 0, my_e = 0;
    if (my_p < p1) {
        my_b = pt_off[my_p];
        my_e = pt_off[my_p + 1];
    }
    double acc[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) acc[k] = 0.0;
    double sse = 0.0;
    unsigned long long anom = 0;

    for (int base = s0; base < s1; base += kPT) {
        const int s = base + threadIdx.x;
        double v[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) v[k] = 0.0;
        if (s < s1) {
            const int c = s_cam[s], p = s_pt[s];
            double cam[9], X[3], obs[2], r[2], Jc[18], Jp[6];
#pragma unroll
            for (int k = 0; k < 9; ++k) cam[k] = __ldg(cams + 9 * c + k);
#pragma unroll
            for (int k = 0; k < 3; ++k) X[k] = __ldg(pts + 3 * p + k);
            const double2 o = s_px[s];
            obs[0] = o.x;
            obs[1] = o.y;
            model::residual_jacobian(cam, X, obs, r, Jc, Jp);
            const bool fin = all_finite(r, 2) && all_finite(Jc, 18) && all_finite(Jp, 6);
            double* Ws = W + 27ll * s;
            double* Qs = JcR + 20ll * s;
            if (fin) {
                const double sq = r[0] * r[0] + r[1] * r[1];
                sse += robust_rho(sq, delta);
                if (delta > 0.0) {  // robust loss: rows scaled by sqrt(rho'(s))
                    const double sw = robust_sqrt_weight(sq, delta);
                    r[0] *= sw;
                    r[1] *= sw;
#pragma unroll
                    for (int k = 0; k < 18; ++k) Jc[k] *= sw;
#pragma unroll
                    for (int k = 0; k < 6; ++k) Jp[k] *= sw;
                }
#pragma unroll
                for (int i = 0; i < 9; ++i)
#pragma unroll
                    for (int j = 0; j < 3; ++j) Ws[3 * i + j] = Jc[i] * Jp[j] + Jc[9 + i] * Jp[3 + j];
#pragma unroll
                for (int k = 0; k < 18; ++k) Qs[k] = Jc[k];
                Qs[18] = r[0];
                Qs[19] = r[1];
                v[0] = Jp[0] * Jp[0] + Jp[3] * Jp[3];
                v[1] = Jp[1] * Jp[0] + Jp[4] * Jp[3];
                v[2] = Jp[1] * Jp[1] + Jp[4] * Jp[4];
                v[3] = Jp[2] * Jp[0] + Jp[5] * Jp[3];
                v[4] = Jp[2] * Jp[1] + Jp[5] * Jp[4];
                v[5] = Jp[2] * Jp[2] + Jp[5] * Jp[5];
#pragma unroll
                for (int i = 0; i < 3; ++i) v[6 + i] = -(Jp[i] * r[0] + Jp[3 + i] * r[1]);
            } else {
                ++anom;
#pragma unroll
                for (int k = 0; k < 27; ++k) Ws[k] = 0.0;
#pragma unroll
                for (int k = 0; k < 20; ++k) Qs[k] = 0.0;
            }
        }
#pragma unroll
        for (int k = 0; k < 9; ++k) contrib[k][threadIdx.x] = v[k];
        __syncthreads();
        if (my_p < p1) {
            const int b = max(my_b, base), e = min(my_e, base + kPT);
            for (int t = b; t < e; ++t)
#pragma unroll
                for (int k = 0; k < 9; ++k) acc[k] += contrib[k][t - base];
        }
        __syncthreads();
    }
    if (my_p < p1) {
#pragma unroll
        for (int k = 0; k < 6; ++k) V[6ll * my_p + k] = acc[k];
#pragma unroll
        for (int k = 0; k < 3; ++k) bp[3ll * my_p + k] = acc[6 + k];
    }
    const double tot = block_sum<kPT>(sse, red);
    const unsigned long long na = block_sum_u64<kPT>(anom, redu);
    if (threadIdx.x == 0) {
        sse_part[chunk] = tot;
        if (na) atomicAdd(counters, na);
    }
}

// Lower-triangle (a >= b) index of a 9x9 block in row order: a*(a+1)/2 + b.
__device__ __forceinline__ void reduce_store54(double (&u)[54], double* __restrict__ out) {
    __shared__ double wpart[kCT / 32][54];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < 54; ++k) {
        const double t = warp_sum(u[k]);
        if (lane == 0) wpart[warp][k] = t;
    }
    __syncthreads();
    if (threadIdx.x < 54) {
        double t = 0.0;
#pragma unroll
        for (int w = 0; w < kCT / 32; ++w) t += wpart[w][threadIdx.x];
        out[threadIdx.x] = t;
    }
}

__global__ void __launch_bounds__(kCT) camera_pass_f64(const int* __restrict__ cchunk_begin,
                                                       const int* __restrict__ cchunk_cam,
                                                       const int* __restrict__ cam_off,
                                                       const int* __restrict__ cam_slots,
                                                       const double* __restrict__ JcR, double* __restrict__ part) {
    const int k = blockIdx.x;
    const int b = cchunk_begin[k], c = cchunk_cam[k];
    const int e = min(b + kCamChunk, cam_off[c + 1]);
    double u[54];
#pragma unroll
    for (int i = 0; i < 54; ++i) u[i] = 0.0;
    for (int i = b + threadIdx.x; i < e; i += kCT) {
        const double* q = JcR + 20ll * cam_slots[i];
        double J[20];
#pragma unroll
        for (int t = 0; t < 20; ++t) J[t] = q[t];
        int idx = 0;
#pragma unroll
        for (int a = 0; a < 9; ++a)
#pragma unroll
            for (int bb = 0; bb <= a; ++bb) {
                u[idx] += J[a] * J[bb] + J[9 + a] * J[9 + bb];
                ++idx;
            }
#pragma unroll
        for (int a = 0; a < 9; ++a) u[45 + a] -= J[a] * J[18] + J[9 + a] * J[19];
    }
    reduce_store54(u, part + 54ll * k);
}

// ---------------------------------------------------------------- FP32 path

// Point pass, FP32 arithmetic: per-slot Jacobian rows Jc32 (18) and Jp32 (6),
// in slot order, and, at the slot's camera-major position, the camera record [Jc(18), r(2)]
// (80 B) for the camera passes; all three go out through a per-warp staging
// buffer in shared memory. V / bp are summed per point in FP32 by a segmented
// scan over each warp (slots of a point are contiguous) and the warps' segment
// sums, and stored FP64. The residuals
// come from r_cur (camera-major): the float-float cost pass at these parameters
// (run anyway to drive accept/reject) stores them rounded to FP32, which keeps the gradient
// accurate to FP32 rounding of r instead of FP32 rounding of f d u. With a
// robust loss, J and r are scaled by sqrt(rho'(s)) before anything is stored.
constexpr int kStg = 28;  // floats per slot in the store-staging buffer: Jc(18), r(2), Jp(6), q, pad

__global__ void __launch_bounds__(kPT) point_pass_f32(
    const int4* __restrict__ prange, const int* __restrict__ pt_off, const int* __restrict__ s_cam,
    const int* __restrict__ s_pt, const float* __restrict__ cams32,
    const float2* __restrict__ ptsff, const float2* __restrict__ r_cur, const int* __restrict__ cam_pos,
    float* __restrict__ Jc32, float* __restrict__ Jp32, long long js, float* __restrict__ J32c,
    double* __restrict__ V, double* __restrict__ bp, unsigned long long* __restrict__ counters, float delta) {
    __shared__ float seg[9][kPT];  // warp-segment sums, at each segment's last slot
    __shared__ unsigned long long redu[kPT / 32];
    __shared__ __align__(16) float stg[kPT * kStg];  // this pass's rows, per slot (kStg floats)
    const int chunk = blockIdx.x;
    const int4 rg = prange[chunk];
    const int p0 = rg.x, p1 = rg.y, s0 = rg.z, s1 = rg.w;
    const int my_p = p0 + threadIdx.x;
    const int lane = threadIdx.x & 31;
    int my_b = 0, my_e = 0;
    if (my_p < p1) {
        my_b = pt_off[my_p];
        my_e = pt_off[my_p + 1];
    }
    float acc[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) acc[k] = 0.f;
    unsigned long long anom = 0;
    for (int base = s0; base < s1; base += kPT) {
        const int s = base + threadIdx.x;
        float v[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) v[k] = 0.f;
        int key = -1;  // point of the slot; slots past the chunk end share key -1 and add zeros
        if (s < s1) {
            const int c = s_cam[s], p = s_pt[s];
            key = p;
            float cam[kCamRec], X[3], obs[2], r[2], J[24];
            const float4* c4 = reinterpret_cast<const float4*>(cams32 + static_cast<long long>(kCamRec) * c);
#pragma unroll
            for (int k = 0; k < kCamRec / 4; ++k) {
                const float4 t = __ldg(c4 + k);
                cam[4 * k] = t.x;
                cam[4 * k + 1] = t.y;
                cam[4 * k + 2] = t.z;
                cam[4 * k + 3] = t.w;
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) X[k] = __ldg(&ptsff[3ll * p + k].x);
            // The Jacobian does not depend on the observation, and the residual
            // comes from the cost pass: the model's own residual is not used.
            obs[0] = obs[1] = 0.f;
            model::residual_jacobian_pre(cam, X, obs, r, J, J + 18);
            const long long q = cam_pos[s];
            const float2 rf = r_cur[q];  // float-float evaluated residual, stored FP32 (camera-major)
            r[0] = rf.x;
            r[1] = rf.y;
            const bool fin = all_finite(r, 2) && all_finite(J, 24);
            if (fin && delta > 0.f) {  // robust loss: rows scaled by sqrt(rho'(s)); the records hold the scaled rows
                const float sw = robust_sqrt_weight(r[0] * r[0] + r[1] * r[1], delta);
                r[0] *= sw;
                r[1] *= sw;
#pragma unroll
                for (int q = 0; q < 24; ++q) J[q] *= sw;
            }
            if (!fin) {
                ++anom;
#pragma unroll
                for (int q = 0; q < 24; ++q) J[q] = 0.f;
                r[0] = r[1] = 0.f;
            }
            // component planes: lane-contiguous vector stores
            store_jacobian_rows(Jc32, Jp32, js, s, J);
            float4* st = reinterpret_cast<float4*>(stg + kStg * threadIdx.x);
#pragma unroll
            for (int k = 0; k < 4; ++k) st[k] = make_float4(J[4 * k], J[4 * k + 1], J[4 * k + 2], J[4 * k + 3]);
            st[4] = make_float4(J[16], J[17], r[0], r[1]);
            st[5] = make_float4(J[18], J[19], J[20], J[21]);
            st[6] = make_float4(J[22], J[23], __int_as_float(static_cast<int>(q)), 0.f);
            const float* Jp = J + 18;
            v[0] = Jp[0] * Jp[0] + Jp[3] * Jp[3];
            v[1] = Jp[1] * Jp[0] + Jp[4] * Jp[3];
            v[2] = Jp[1] * Jp[1] + Jp[4] * Jp[4];
            v[3] = Jp[2] * Jp[0] + Jp[5] * Jp[3];
            v[4] = Jp[2] * Jp[1] + Jp[5] * Jp[4];
            v[5] = Jp[2] * Jp[2] + Jp[5] * Jp[5];
#pragma unroll
            for (int i = 0; i < 3; ++i) v[6 + i] = -(Jp[i] * r[0] + Jp[3 + i] * r[1]);
        }
        {
            // Each camera record (camera-major) is written by five adjacent
            // lanes from the staging buffer, instead of one 16-byte piece per
            // lane (4x fewer L2 store requests).
            __syncwarp();
            const int w0 = base + (threadIdx.x & ~31);
            const int n = max(0, min(32, s1 - w0));
            const float* ws = stg + kStg * (threadIdx.x & ~31);
            for (int t = lane; t < 5 * n; t += 32) {
                const int j = t / 5, k = t - 5 * j;
                const long long qj = __float_as_int(ws[kStg * j + 26]);
                reinterpret_cast<float4*>(J32c + 20ll * qj)[k] = *reinterpret_cast<const float4*>(ws + kStg * j + 4 * k);
            }
        }
        // inclusive segmented scan over the warp
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int kd = __shfl_up_sync(0xffffffffu, key, d);
            const bool take = lane >= d && kd == key;
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                const float t = __shfl_up_sync(0xffffffffu, v[k], d);
                if (take) v[k] += t;
            }
        }
        const int knext = __shfl_down_sync(0xffffffffu, key, 1);
        if (lane == 31 || knext != key) {
#pragma unroll
            for (int k = 0; k < 9; ++k) seg[k][threadIdx.x] = v[k];
        }
        __syncthreads();
        // owner: add the point's warp-segment sums of this pass, warps in order
        if (my_p < p1) {
            const int b = max(my_b, base) - base, e = min(my_e, base + kPT) - base;
            for (int w = b >> 5; b < e && w <= (e - 1) >> 5; ++w) {
                const int t = min(e - 1, 32 * w + 31);
#pragma unroll
                for (int k = 0; k < 9; ++k) acc[k] += seg[k][t];
            }
        }
        __syncthreads();
    }
    if (my_p < p1) {
#pragma unroll
        for (int k = 0; k < 6; ++k) V[6ll * my_p + k] = static_cast<double>(acc[k]);
#pragma unroll
        for (int k = 0; k < 3; ++k) bp[3ll * my_p + k] = static_cast<double>(acc[6 + k]);
    }
    const unsigned long long na = block_sum_u64<kPT>(anom, redu);
    if (threadIdx.x == 0 && na) atomicAdd(counters, na);
}

// Camera pass, FP32 arithmetic: streams the camera records [Jc(18), r(2)] the
// point pass wrote (robust-scaled), sums U and bc products per thread and per
// warp in FP32, and adds the four warp partials in FP64.
__global__ void __launch_bounds__(kCT) camera_pass_f32(const int* __restrict__ cchunk_begin,
                                                      const int* __restrict__ cchunk_cam,
                                                      const int* __restrict__ cam_off, const float* __restrict__ J32c,
                                                      double* __restrict__ part) {
    __shared__ float wpart[kCT / 32][54];
    const int k = blockIdx.x;
    const int b = cchunk_begin[k], c = cchunk_cam[k];
    const int e = min(b + kCamChunk, cam_off[c + 1]);
    float u[54];
#pragma unroll
    for (int i = 0; i < 54; ++i) u[i] = 0.f;
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
        const float2 r = make_float2(Jc[18], Jc[19]);
        int idx = 0;
#pragma unroll
        for (int a = 0; a < 9; ++a)
#pragma unroll
            for (int bb = 0; bb <= a; ++bb) {
                u[idx] += Jc[a] * Jc[bb] + Jc[9 + a] * Jc[9 + bb];
                ++idx;
            }
#pragma unroll
        for (int a = 0; a < 9; ++a) u[45 + a] -= Jc[a] * r.x + Jc[9 + a] * r.y;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int t = 0; t < 54; ++t) {
        const float v = warp_sum(u[t]);
        if (lane == 0) wpart[warp][t] = v;
    }
    __syncthreads();
    if (threadIdx.x < 54) {
        double t = 0.0;
#pragma unroll
        for (int w = 0; w < kCT / 32; ++w) t += static_cast<double>(wpart[w][threadIdx.x]);
        part[54ll * k + threadIdx.x] = t;
    }
}

// U (full symmetric 9x9) and bc from the chunk partials, chunks in order.
__global__ void camera_finalize(const int* __restrict__ cam_chunk_off, const double* __restrict__ part, int C,
                                double* __restrict__ U, double* __restrict__ bc) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 54 * C) return;
    const int c = t / 54, j = t % 54;
    double s = 0.0;
    for (int k = cam_chunk_off[c]; k < cam_chunk_off[c + 1]; ++k) s += part[54ll * k + j];
    if (j < 45) {
        int a = 0;
        while ((a + 1) * (a + 2) / 2 <= j) ++a;
        const int b = j - a * (a + 1) / 2;
        U[81ll * c + 9 * a + b] = s;
        U[81ll * c + 9 * b + a] = s;
    } else {
        bc[9ll * c + (j - 45)] = s;
    }
}

__global__ void add_counter_kernel(unsigned long long* __restrict__ dst, const unsigned long long* __restrict__ src) {
    *dst += *src;
}

// Sum of n partials in a fixed order (single CTA) -> *out.
constexpr int kSumT = 1024;  // threads of the single-block partial sums

__global__ void __launch_bounds__(kSumT) ordered_sum(const double* __restrict__ part, int n, double* __restrict__ out) {
    __shared__ double red[kSumT / 32];
    const double t = wide_block_sum<kSumT>(part, n, red);
    if (threadIdx.x == 0) *out = t;
}

// Per-camera FP64 rotation matrix (Rodrigues, or I + [a]x on the first-order
// branch, the same model as model::residual), translation and intrinsics:
// 15 doubles per camera, so the cost kernel evaluates R X + t per observation
// instead of a sin / cos / sqrt per observation on GB300's narrow FP64 pipe.
constexpr int kCamPre = 16;
// Per-camera constants of the residual: rotation matrix (Rodrigues), t, f, k1,
// k2 (kCamPre doubles); preff (may be null): the same as float-float pairs;
// cams32 (may be null): the FP32 Jacobian pass's per-camera record
// (model::camera_constants, 28 floats: R, J_l, t, f, k1, k2, branch flag),
// computed in FP64 and rounded.
// One camera per thread in warp-sized blocks: the FP64 trigonometry of C
// cameras spreads over all SMs' FP64 pipes (blocks of 128 used C / 128 SMs).
constexpr int kPreT = 32;

__global__ void camera_precompute_kernel(const double* __restrict__ cams, int C, double* __restrict__ pre,
                                         float2* __restrict__ preff, float* __restrict__ cams32) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    const double* a = cams + 9ll * c;
    double* o = pre + static_cast<long long>(kCamPre) * c;
    const double th2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
    if (th2 > 1e-24) {
        const double th = sqrt(th2);
        const double w0 = a[0] / th, w1 = a[1] / th, w2 = a[2] / th;
        double s, cth;
        sincos(th, &s, &cth);
        const double sh = sin(0.5 * th);
        const double omc = 2.0 * sh * sh;
        o[0] = cth + omc * w0 * w0;  o[1] = -s * w2 + omc * w0 * w1;  o[2] = s * w1 + omc * w0 * w2;
        o[3] = s * w2 + omc * w1 * w0;  o[4] = cth + omc * w1 * w1;  o[5] = -s * w0 + omc * w1 * w2;
        o[6] = -s * w1 + omc * w2 * w0;  o[7] = s * w0 + omc * w2 * w1;  o[8] = cth + omc * w2 * w2;
    } else {
        o[0] = 1.0;  o[1] = -a[2]; o[2] = a[1];
        o[3] = a[2]; o[4] = 1.0;   o[5] = -a[0];
        o[6] = -a[1]; o[7] = a[0]; o[8] = 1.0;
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) o[9 + i] = a[3 + i];
    o[15] = 0.0;
    if (cams32) {
        double k[kCamRec];
        model::camera_constants(a, k);
        float4* o4 = reinterpret_cast<float4*>(cams32 + static_cast<long long>(kCamRec) * c);
#pragma unroll
        for (int i = 0; i < kCamRec / 4; ++i)
            o4[i] = make_float4(static_cast<float>(k[4 * i]), static_cast<float>(k[4 * i + 1]),
                                static_cast<float>(k[4 * i + 2]), static_cast<float>(k[4 * i + 3]));
    }
    if (preff) {
#pragma unroll
        for (int i = 0; i < kCamPre; ++i) {
            const ffa::ff f = ffa::from_double(o[i]);
            preff[static_cast<long long>(kCamPre) * c + i] = make_float2(f.hi, f.lo);
        }
    }
}

__device__ __forceinline__ void residual_pre(const double* __restrict__ pc, const double* X, const double* obs,
                                             double* r) {
    const double P0 = pc[0] * X[0] + pc[1] * X[1] + pc[2] * X[2] + pc[9];
    const double P1 = pc[3] * X[0] + pc[4] * X[1] + pc[5] * X[2] + pc[10];
    const double P2 = pc[6] * X[0] + pc[7] * X[1] + pc[8] * X[2] + pc[11];
    const double iz = 1.0 / P2;
    const double u = -P0 * iz, v = -P1 * iz;
    const double r2 = u * u + v * v;
    const double d = 1.0 + r2 * (pc[13] + pc[14] * r2);
    r[0] = pc[12] * d * u - obs[0];
    r[1] = pc[12] * d * v - obs[1];
}

// FP64 SSE of all slots at (cams, pts), one CTA per point chunk. If r_out is
// set, each slot's residual is also stored (FP32; NaN where not finite).
__global__ void __launch_bounds__(kPT) cost_f64(const int* __restrict__ pchunk, const int* __restrict__ pt_off,
                                               const int* __restrict__ s_cam, const int* __restrict__ s_pt,
                                               const double2* __restrict__ s_px, const double* __restrict__ pre,
                                               const double* __restrict__ pts, double* __restrict__ sse_part,
                                               unsigned long long* __restrict__ counters, float2* __restrict__ r_out,
                                               double delta) {
    __shared__ double red[kPT / 32];
    __shared__ unsigned long long redu[kPT / 32];
    const int chunk = blockIdx.x;
    const int s0 = pt_off[pchunk[chunk]], s1 = pt_off[pchunk[chunk + 1]];
    double sse = 0.0;
    unsigned long long anom = 0;
    for (int s = s0 + threadIdx.x; s < s1; s += kPT) {
        const int c = s_cam[s], p = s_pt[s];
        double X[3], obs[2], r[2];
#pragma unroll
        for (int k = 0; k < 3; ++k) X[k] = __ldg(pts + 3 * p + k);
        const double2 o = s_px[s];
        obs[0] = o.x;
        obs[1] = o.y;
        residual_pre(pre + static_cast<long long>(kCamPre) * c, X, obs, r);
        const bool fin = isfinite(r[0]) && isfinite(r[1]);
        if (r_out) r_out[s] = fin ? make_float2(static_cast<float>(r[0]), static_cast<float>(r[1])) : make_float2(NAN, NAN);
        if (!fin) {
            ++anom;
            continue;
        }
        sse += robust_rho(r[0] * r[0] + r[1] * r[1], delta);
    }
    const double tot = block_sum<kPT>(sse, red);
    const unsigned long long na = block_sum_u64<kPT>(anom, redu);
    if (threadIdx.x == 0) {
        sse_part[chunk] = tot;
        if (na) atomicAdd(counters, na);
    }
}

// Residual from float-float camera constants (R, t, f, k1, k2), point and
// observation: the FP64 formula of residual_pre with every operation in
// float-float (relative error about 1e-14 before the cancellation against the
// observation).
__device__ __forceinline__ void residual_ff(const float2* __restrict__ pc, const ffa::ff* X, ffa::ff o0, ffa::ff o1,
                                            ffa::ff& r0, ffa::ff& r1) {
    using ffa::ff;
    ff P[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float2 t = pc[9 + i];
        P[i] = {t.x, t.y};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float2 R = pc[3 * i + k];
            ffa::madd(P[i], ff{R.x, R.y}, X[k]);
        }
        P[i] = ffa::norm(P[i]);
    }
    const ff iz = ffa::div(ff{1.f, 0.f}, P[2]);
    const ff u = ffa::neg(ffa::mul(P[0], iz)), v = ffa::neg(ffa::mul(P[1], iz));
    ff r2 = {0.f, 0.f};
    ffa::madd(r2, u, u);
    ffa::madd(r2, v, v);
    r2 = ffa::norm(r2);
    const float2 fk = pc[12], k1 = pc[13], k2 = pc[14];
    ff t = {k1.x, k1.y};
    ffa::madd(t, ff{k2.x, k2.y}, r2);
    ff d = {1.f, 0.f};
    ffa::madd(d, r2, ffa::norm(t));
    const ff fd = ffa::mul(ff{fk.x, fk.y}, ffa::norm(d));
    r0 = ffa::norm(ffa::sub(ffa::mul(fd, u), o0));
    r1 = ffa::norm(ffa::sub(ffa::mul(fd, v), o1));
}

// Mixed-form cost, camera-major: one CTA per camera chunk holds the camera's
// float-float constants in shared memory and streams the chunk's positions
// (camera-major point index and float-float observation), gathering only the
// point. rho(|r|^2) is summed in float-float per thread and per warp, warps
// combined in FP64; the residuals are stored FP32 at the camera-major position
// (NaN where not finite, counted as anomalies). A position whose float-float
// residual leaves FP32's safe range (|r| >= kFfSafe or not finite: a wild trial
// step, e.g. a point near the camera plane) is evaluated again in FP64 from
// the FP64 constants (pre64), point (pts64) and observation, so the cost and
// the anomaly count follow FP64 semantics; its rho is summed in FP64 (warps
// that met such a position only).
constexpr float kFfSafe = 1e12f;
constexpr int kCostT = 256;

__global__ void __launch_bounds__(kCostT, 4) cost_ff(const int* __restrict__ cchunk_begin,
                                                 const int* __restrict__ cchunk_cam, const int* __restrict__ cam_off,
                                                 const int* __restrict__ cm_pt, const float4* __restrict__ cm_pxff,
                                                 const float2* __restrict__ preff, const float2* __restrict__ ptsff,
                                                 const int* __restrict__ cam_slots, const double2* __restrict__ s_px,
                                                 const double* __restrict__ pre64, const double* __restrict__ pts64,
                                                 double* __restrict__ sse_part,
                                                 unsigned long long* __restrict__ counters,
                                                 float2* __restrict__ r_out, double delta, float2 delta_ff,
                                                 float2 delta2_ff) {
    using ffa::ff;
    __shared__ float2 pc[kCamPre];
    __shared__ float red[kCostT / 32][2];
    __shared__ double red64[kCostT / 32];
    __shared__ unsigned long long redu[kCostT / 32];
    const int k = blockIdx.x;
    const int b = cchunk_begin[k], c = cchunk_cam[k];
    const int e = min(b + kCamChunk, cam_off[c + 1]);
    if (threadIdx.x < kCamPre) pc[threadIdx.x] = preff[static_cast<long long>(kCamPre) * c + threadIdx.x];
    __syncthreads();
    const bool robust = delta_ff.x > 0.f;
    const ff dl = {delta_ff.x, delta_ff.y}, dl2 = {delta2_ff.x, delta2_ff.y};
    ff sse = {0.f, 0.f};
    double sse64 = 0.0;
    int fallback = 0;
    unsigned long long anom = 0;
    for (int i = b + threadIdx.x; i < e; i += kCostT) {
        const int p = cm_pt[i];
        ff X[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const float2 x = ptsff[3ll * p + q];
            X[q] = {x.x, x.y};
        }
        const float4 o = cm_pxff[i];
        ff r0, r1;
        residual_ff(pc, X, ff{o.x, o.y}, ff{o.z, o.w}, r0, r1);
        if (!(fabsf(r0.hi) < kFfSafe && fabsf(r1.hi) < kFfSafe)) {
            double X64[3], obs[2], r[2];
#pragma unroll
            for (int q = 0; q < 3; ++q) X64[q] = pts64[3ll * p + q];
            const double2 ob = s_px[cam_slots[i]];
            obs[0] = ob.x;
            obs[1] = ob.y;
            residual_pre(pre64 + static_cast<long long>(kCamPre) * c, X64, obs, r);
            const bool fin = isfinite(r[0]) && isfinite(r[1]);
            r_out[i] = fin ? make_float2(static_cast<float>(r[0]), static_cast<float>(r[1])) : make_float2(NAN, NAN);
            if (!fin) {
                ++anom;
                continue;
            }
            sse64 += robust_rho(r[0] * r[0] + r[1] * r[1], delta);
            fallback = 1;
            continue;
        }
        r_out[i] = make_float2(r0.hi, r1.hi);
        ff sq = {0.f, 0.f};
        ffa::madd(sq, r0, r0);
        ffa::madd(sq, r1, r1);
        sq = ffa::norm(sq);
        if (robust && (sq.hi > dl2.hi || (sq.hi == dl2.hi && sq.lo > dl2.lo))) {
            // 2 delta sqrt(s) - delta^2
            sq = ffa::norm(ffa::sub(ffa::mul(ff{2.f * dl.hi, 2.f * dl.lo}, ffa::sqrt(sq)), dl2));
        }
        sse = ffa::add(sse, sq);
    }
    // warp sums in float-float, then FP64 across warps
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sse = ffa::add(sse, ffa::shfl_xor(sse, o));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (__any_sync(0xffffffffu, fallback)) sse64 = warp_sum(sse64);  // else every lane holds 0
    if (lane == 0) {
        red[warp][0] = sse.hi;
        red[warp][1] = sse.lo;
        red64[warp] = sse64;
    }
    const unsigned long long na = block_sum_u64<kCostT>(anom, redu);  // synchronises the block
    if (threadIdx.x == 0) {
        double tot = 0.0;
#pragma unroll
        for (int w = 0; w < kCostT / 32; ++w)
            tot += static_cast<double>(red[w][0]) + static_cast<double>(red[w][1]) + red64[w];
        sse_part[k] = tot;
        if (na) atomicAdd(counters, na);
    }
}

template <typename T>
__global__ void eval_edges_kernel(const double* __restrict__ cams, const double* __restrict__ pts,
                                  const int* __restrict__ oc, const int* __restrict__ op,
                                  const double* __restrict__ px, int E, T* __restrict__ r, T* __restrict__ Jc,
                                  T* __restrict__ Jp) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
        T cam[9], X[3], obs[2], rr[2], jc[18], jp[6];
        for (int k = 0; k < 9; ++k) cam[k] = static_cast<T>(cams[9ll * oc[e] + k]);
        for (int k = 0; k < 3; ++k) X[k] = static_cast<T>(pts[3ll * op[e] + k]);
        obs[0] = static_cast<T>(px[2ll * e]);
        obs[1] = static_cast<T>(px[2ll * e + 1]);
        model::residual_jacobian(cam, X, obs, rr, jc, jp);
        r[2ll * e] = rr[0];
        r[2ll * e + 1] = rr[1];
        if (Jc)
            for (int k = 0; k < 18; ++k) Jc[18ll * e + k] = jc[k];
        if (Jp)
            for (int k = 0; k < 6; ++k) Jp[6ll * e + k] = jp[k];
    }
}

}  // namespace

double Solver::accumulate() {
    accumulate_launch();
    double sse = 0.0;
    read_back({{&sse, scal_.get(), sizeof sse}});
    return sse;
}

// The normal-equation passes without the host read of the SSE (scal_[0]).
void Solver::accumulate_launch() {
    const double2* spx = reinterpret_cast<const double2*>(s_px_.get());
    if (form_ == SolverForm::Plain) {
        cudaEvent_t ev = prof_start();
        point_pass_f64<<<n_pchunk_, kPT, 0, stream_>>>(pchunk_.get(), pt_off_.get(), s_cam_.get(), s_pt_.get(),
                                                       spx, cams_.get(), pts_.get(), W_.get(), JcR_.get(),
                                                       V_.get(), bp_.get(), sse_part_.get(), counters_.get(),
                                                       huber_delta_);
        GBA_LAUNCH_CHECK();
        prof_stop("point_pass_f64", ev);
        if (n_cchunk_ > 0) {
            ev = prof_start();
            camera_pass_f64<<<n_cchunk_, kCT, 0, stream_>>>(cchunk_begin_.get(), cchunk_cam_.get(),
                                                            cam_off_.get(), cam_slots_.get(), JcR_.get(),
                                                            cam_part_.get());
            GBA_LAUNCH_CHECK();
            prof_stop("camera_pass_f64", ev);
        }
        ordered_sum<<<1, kSumT, 0, stream_>>>(sse_part_.get(), n_pchunk_, scal_.get());
        GBA_LAUNCH_CHECK();
    } else {
        // The mixed form keeps the cost at FP64 accuracy: SSE and residuals come
        // from the float-float residual pass. After an accepted trial they are already there
        // (the trial evaluation at these parameters). Its non-finite count goes
        // to a scratch counter: the FP32 pass counts this evaluation's anomalies.
        if (!resid_valid_) {
            cost_mixed(cams_.get(), pts_.get(), counters_.get() + 2, reinterpret_cast<float2*>(r_cur_.get()));
            ordered_sum<<<1, kSumT, 0, stream_>>>(sse_part_.get(), n_cchunk_, scal_.get());
            GBA_LAUNCH_CHECK();
            resid_valid_ = true;
        }
        if (ff_holds_ != kFfCurrent) prepare_ff(cams_.get(), pts_.get());
        const float2* rc = reinterpret_cast<const float2*>(r_cur_.get());
        cudaEvent_t ev = prof_start();
        point_pass_f32<<<n_pchunk_, kPT, 0, stream_>>>(
            reinterpret_cast<const int4*>(pchunk4_.get()), pt_off_.get(), s_cam_.get(), s_pt_.get(), cams32_.get(), reinterpret_cast<const float2*>(pts_ff_.get()), rc, cam_pos_.get(), Jc32_.get(), Jp32_.get(),
            js_, J32c_.get(), V_.get(), bp_.get(), counters_.get(), static_cast<float>(huber_delta_));
        GBA_LAUNCH_CHECK();
        prof_stop("point_pass_f32", ev);
        if (n_cchunk_ > 0) {
            ev = prof_start();
            camera_pass_f32<<<n_cchunk_, kCT, 0, stream_>>>(cchunk_begin_.get(), cchunk_cam_.get(),
                                                            cam_off_.get(), J32c_.get(), cam_part_.get());
            GBA_LAUNCH_CHECK();
            prof_stop("camera_pass_f32", ev);
        }
    }
    camera_finalize<<<ceil_div(54ll * C_, 256), 256, 0, stream_>>>(cam_chunk_off_.get(), cam_part_.get(), C_,
                                                                 U_.get(), bc_.get());
    GBA_LAUNCH_CHECK();
}

// Mixed-form cost at (cams, pts): camera constants and points split to
// float-float, then the float-float residual pass (SSE partials per chunk in
// sse_part_, residuals in r_out).
void Solver::cost_mixed(const double* cams, const double* pts, unsigned long long* anomalies, float2* r_out) {
    cudaEvent_t ev = prof_start();
    prepare_ff(cams, pts);
    // Huber threshold and its square as float-float pairs (host-split: no
    // per-thread FP64 conversions)
    const double d2 = huber_delta_ * huber_delta_;
    const float dh = static_cast<float>(huber_delta_), d2h = static_cast<float>(d2);
    const float2 dl = huber_delta_ > 0.0 ? make_float2(dh, static_cast<float>(huber_delta_ - dh)) : make_float2(0.f, 0.f);
    const float2 dl2 = make_float2(d2h, static_cast<float>(d2 - d2h));
    if (n_cchunk_ > 0) {
        cost_ff<<<n_cchunk_, kCostT, 0, stream_>>>(
            cchunk_begin_.get(), cchunk_cam_.get(), cam_off_.get(), cm_pt_.get(),
            reinterpret_cast<const float4*>(cm_pxff_.get()), reinterpret_cast<const float2*>(cam_pre_ff_.get()),
            reinterpret_cast<const float2*>(pts_ff_.get()), cam_slots_.get(),
            reinterpret_cast<const double2*>(s_px_.get()), cam_pre_.get(), pts, sse_part_.get(), anomalies, r_out,
            huber_delta_, dl, dl2);
    }
    GBA_LAUNCH_CHECK();
    prof_stop("cost_ff", ev);
}

// Float-float camera constants, FP32 cameras and float-float points of
// (cams, pts), for the cost pass and the FP32 Jacobian pass.
void Solver::prepare_ff(const double* cams, const double* pts) {
    camera_precompute_kernel<<<ceil_div(C_, kPreT), kPreT, 0, stream_>>>(
        cams, C_, cam_pre_.get(), reinterpret_cast<float2*>(cam_pre_ff_.get()), cams32_.get());
    GBA_LAUNCH_CHECK();
    if (!(pts == tpts_.get() && pts_ff_trial_)) launch_split_ff(pts, 3ll * P_, pts_ff_.get(), stream_);
    pts_ff_trial_ = pts == tpts_.get();
    ff_holds_ = (cams == cams_.get() && pts == pts_.get()) ? kFfCurrent
                : (cams == tcams_.get() && pts == tpts_.get()) ? kFfTrial
                                                                : kFfNone;
}

double Solver::trial_cost() {
    trial_cost_launch(counters_.get());
    double sse = 0.0;
    read_back({{&sse, scal_.get() + 1, sizeof sse}});
    return sse;
}

void Solver::read_trial(double* denom, double* sse, unsigned long long* cost_anomalies) {
    read_back({{denom, scal_.get() + 2, sizeof(double)},
               {sse, scal_.get() + 1, sizeof(double)},
               {cost_anomalies, counters_.get() + 2, sizeof(unsigned long long)}});
}

void Solver::zero_cost_scratch() {
    GBA_CUDA_CHECK(cudaMemsetAsync(counters_.get() + 2, 0, sizeof(unsigned long long), stream_));
}

void Solver::commit_cost_anomalies() {
    add_counter_kernel<<<1, 1, 0, stream_>>>(counters_.get(), counters_.get() + 2);
    GBA_LAUNCH_CHECK();
}

// Trial SSE into scal_[1] (non-finite residual count added to *anomalies), without a host read.
void Solver::trial_cost_launch(unsigned long long* anomalies) {
    if (form_ == SolverForm::Plain) {
        const double2* spx = reinterpret_cast<const double2*>(s_px_.get());
        cudaEvent_t ev = prof_start();
        camera_precompute_kernel<<<ceil_div(C_, kPreT), kPreT, 0, stream_>>>(tcams_.get(), C_, cam_pre_.get(), nullptr,
                                                                         nullptr);
        GBA_LAUNCH_CHECK();
        cost_f64<<<n_pchunk_, kPT, 0, stream_>>>(pchunk_.get(), pt_off_.get(), s_cam_.get(), s_pt_.get(), spx,
                                                 cam_pre_.get(), tpts_.get(), sse_part_.get(), anomalies,
                                                 nullptr, huber_delta_);
        GBA_LAUNCH_CHECK();
        prof_stop("cost_f64", ev);
    } else {
        cost_mixed(tcams_.get(), tpts_.get(), anomalies, reinterpret_cast<float2*>(r_trial_.get()));
    }
    ordered_sum<<<1, kSumT, 0, stream_>>>(sse_part_.get(), form_ == SolverForm::Plain ? n_pchunk_ : n_cchunk_,
                                        scal_.get() + 1);
    GBA_LAUNCH_CHECK();
}

void launch_eval_edges_f64(const double* cams, const double* pts, const int* oc, const int* op, const double* px,
                           int E, double* r, double* Jc, double* Jp, cudaStream_t s) {
    eval_edges_kernel<double><<<ceil_div(E, 128), 128, 0, s>>>(cams, pts, oc, op, px, E, r, Jc, Jp);
    GBA_LAUNCH_CHECK();
}

void launch_eval_edges_f32(const double* cams, const double* pts, const int* oc, const int* op, const double* px,
                           int E, float* r, float* Jc, float* Jp, cudaStream_t s) {
    eval_edges_kernel<float><<<ceil_div(E, 128), 128, 0, s>>>(cams, pts, oc, op, px, E, r, Jc, Jp);
    GBA_LAUNCH_CHECK();
}

}  // namespace gba

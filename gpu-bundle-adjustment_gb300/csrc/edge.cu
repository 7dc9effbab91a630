// Normal-equation accumulation (edge kernels) and the FP64 trial-cost kernel.
//
// Replaces the reference edge_kernel / cost_kernel (src/lm.cu:205-281), which
// accumulate U, V, bc, bp and the SSE with global FP64 atomics in file order.
// Here every sum is atomic-free and deterministic:
//   point pass   one CTA per point chunk (whole points, <= 256 slots, slots
//                sorted by point): residual + Jacobian per slot, per-edge W (or the
//                FP32 Jacobian record), and V / bp as in-CTA ordered sums.
//   camera pass  one CTA per camera chunk (<= 1024 slots of one camera, from the
//                camera-major view): U / bc partial sums per chunk, then a
//                finalize kernel adds the chunk partials of each camera in order.
// Non-finite edges contribute nothing, bump counters[0] and get W = 0
// (reference semantics src/lm.cu:219-225; the reference leaves W stale).

#include "camera_model.cuh"
#include "common.cuh"
#include "solver.hpp"

namespace gba {
namespace {

constexpr int kPT = 256;       // point-pass threads (= max slots per chunk)
constexpr int kCT = 128;       // camera-pass threads
constexpr int kCamChunk = 1024;

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

// Point pass, FP32 arithmetic: per-slot Jacobian record J32 = [Jc(18), Jp(6)];
// V / bp summed per point in FP32 and stored FP64 (one FP64 conversion per point).
// The residuals come from r_cur: the FP64 cost pass at these parameters (run
// anyway to drive accept/reject) stores them rounded to FP32, which keeps the
// gradient accurate to FP32 rounding of r instead of FP32 rounding of f d u.
__global__ void __launch_bounds__(kPT) point_pass_f32(
    const int* __restrict__ pchunk, const int* __restrict__ pt_off, const int* __restrict__ s_cam,
    const int* __restrict__ s_pt, const double2* __restrict__ s_px, const double* __restrict__ cams,
    const double* __restrict__ pts, const float2* __restrict__ r_cur, const int* __restrict__ cam_pos,
    float* __restrict__ J32, float* __restrict__ J32c, double* __restrict__ V, double* __restrict__ bp,
    unsigned long long* __restrict__ counters, float delta) {
    __shared__ float contrib[9][kPT];
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
    float acc[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) acc[k] = 0.f;
    unsigned long long anom = 0;
    for (int base = s0; base < s1; base += kPT) {
        const int s = base + threadIdx.x;
        float v[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) v[k] = 0.f;
        if (s < s1) {
            const int c = s_cam[s], p = s_pt[s];
            float cam[9], X[3], obs[2], r[2], J[24];
#pragma unroll
            for (int k = 0; k < 9; ++k) cam[k] = static_cast<float>(__ldg(cams + 9 * c + k));
#pragma unroll
            for (int k = 0; k < 3; ++k) X[k] = static_cast<float>(__ldg(pts + 3 * p + k));
            const double2 o = s_px[s];
            obs[0] = static_cast<float>(o.x);
            obs[1] = static_cast<float>(o.y);
            model::residual_jacobian(cam, X, obs, r, J, J + 18);
            const float2 rf = r_cur[s];  // FP64-evaluated residual, stored FP32
            r[0] = rf.x;
            r[1] = rf.y;
            const bool fin = all_finite(r, 2) && all_finite(J, 24);
            float4* out = reinterpret_cast<float4*>(J32 + 24ll * s);
            float2* outc = reinterpret_cast<float2*>(J32c + 18ll * cam_pos[s]);  // camera-major Jc copy
            if (fin && delta > 0.f) {  // robust loss: rows scaled by sqrt(rho'(s)); J32 holds the scaled rows
                const float sw = robust_sqrt_weight(r[0] * r[0] + r[1] * r[1], delta);
                r[0] *= sw;
                r[1] *= sw;
#pragma unroll
                for (int q = 0; q < 24; ++q) J[q] *= sw;
            }
            if (fin) {
#pragma unroll
                for (int q = 0; q < 6; ++q) out[q] = make_float4(J[4 * q], J[4 * q + 1], J[4 * q + 2], J[4 * q + 3]);
#pragma unroll
                for (int q = 0; q < 9; ++q) outc[q] = make_float2(J[2 * q], J[2 * q + 1]);
                const float* Jp = J + 18;
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
                for (int q = 0; q < 6; ++q) out[q] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                for (int q = 0; q < 9; ++q) outc[q] = make_float2(0.f, 0.f);
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
        for (int k = 0; k < 6; ++k) V[6ll * my_p + k] = static_cast<double>(acc[k]);
#pragma unroll
        for (int k = 0; k < 3; ++k) bp[3ll * my_p + k] = static_cast<double>(acc[6 + k]);
    }
    const unsigned long long na = block_sum_u64<kPT>(anom, redu);
    if (threadIdx.x == 0 && na) atomicAdd(counters, na);
}

// Camera pass, FP32 arithmetic: recomputes Jc and r for the chunk's slots
// (cheaper than re-reading the Jacobian records), sums products per thread in
// FP32, then reduces the per-thread partials in FP64.
__global__ void __launch_bounds__(kCT) camera_pass_f32(
    const int* __restrict__ cchunk_begin, const int* __restrict__ cchunk_cam, const int* __restrict__ cam_off,
    const int* __restrict__ cam_slots, const int* __restrict__ s_pt, const double2* __restrict__ s_px,
    const double* __restrict__ cams, const double* __restrict__ pts, const float2* __restrict__ r_cur,
    double* __restrict__ part, float delta) {
    const int k = blockIdx.x;
    const int b = cchunk_begin[k], c = cchunk_cam[k];
    const int e = min(b + kCamChunk, cam_off[c + 1]);
    float cam[9];
#pragma unroll
    for (int t = 0; t < 9; ++t) cam[t] = static_cast<float>(__ldg(cams + 9 * c + t));
    float u[54];
#pragma unroll
    for (int i = 0; i < 54; ++i) u[i] = 0.f;
    for (int i = b + threadIdx.x; i < e; i += kCT) {
        const int s = cam_slots[i];
        const int p = s_pt[s];
        float X[3], obs[2], r[2], Jc[18], Jp[6];
#pragma unroll
        for (int t = 0; t < 3; ++t) X[t] = static_cast<float>(__ldg(pts + 3 * p + t));
        const double2 o = s_px[s];
        obs[0] = static_cast<float>(o.x);
        obs[1] = static_cast<float>(o.y);
        model::residual_jacobian(cam, X, obs, r, Jc, Jp);
        const float2 rf = r_cur[s];
        r[0] = rf.x;
        r[1] = rf.y;
        const bool fin = all_finite(r, 2) && all_finite(Jc, 18) && all_finite(Jp, 6);
        if (!fin) continue;
        if (delta > 0.f) {
            const float sw = robust_sqrt_weight(r[0] * r[0] + r[1] * r[1], delta);
            r[0] *= sw;
            r[1] *= sw;
#pragma unroll
            for (int q = 0; q < 18; ++q) Jc[q] *= sw;
        }
        int idx = 0;
#pragma unroll
        for (int a = 0; a < 9; ++a)
#pragma unroll
            for (int bb = 0; bb <= a; ++bb) {
                u[idx] += Jc[a] * Jc[bb] + Jc[9 + a] * Jc[9 + bb];
                ++idx;
            }
#pragma unroll
        for (int a = 0; a < 9; ++a) u[45 + a] -= Jc[a] * r[0] + Jc[9 + a] * r[1];
    }
    double ud[54];
#pragma unroll
    for (int i = 0; i < 54; ++i) ud[i] = static_cast<double>(u[i]);
    reduce_store54(ud, part + 54ll * k);
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

// Sum of n partials in a fixed order (single CTA) -> *out.
__global__ void __launch_bounds__(256) ordered_sum(const double* __restrict__ part, int n, double* __restrict__ out) {
    __shared__ double red[8];
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += 256) s += part[i];
    const double t = block_sum<256>(s, red);
    if (threadIdx.x == 0) *out = t;
}

// Per-camera FP64 rotation matrix (Rodrigues, or I + [a]x on the first-order
// branch, the same model as model::residual), translation and intrinsics:
// 15 doubles per camera, so the cost kernel evaluates R X + t per observation
// instead of a sin / cos / sqrt per observation on GB300's narrow FP64 pipe.
constexpr int kCamPre = 16;
__global__ void camera_precompute_kernel(const double* __restrict__ cams, int C, double* __restrict__ pre) {
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
        ordered_sum<<<1, 256, 0, stream_>>>(sse_part_.get(), n_pchunk_, scal_.get());
        GBA_LAUNCH_CHECK();
    } else {
        // The mixed form keeps the cost FP64: SSE and residuals come from the
        // FP64 residual pass. After an accepted trial they are already there
        // (the trial evaluation at these parameters). Its non-finite count goes
        // to a scratch counter: the FP32 pass counts this evaluation's anomalies.
        if (!resid_valid_) {
            camera_precompute_kernel<<<ceil_div(C_, 128), 128, 0, stream_>>>(cams_.get(), C_, cam_pre_.get());
            GBA_LAUNCH_CHECK();
            cost_f64<<<n_pchunk_, kPT, 0, stream_>>>(pchunk_.get(), pt_off_.get(), s_cam_.get(), s_pt_.get(), spx,
                                                     cam_pre_.get(), pts_.get(), sse_part_.get(), counters_.get() + 2,
                                                     reinterpret_cast<float2*>(r_cur_.get()), huber_delta_);
            GBA_LAUNCH_CHECK();
            ordered_sum<<<1, 256, 0, stream_>>>(sse_part_.get(), n_pchunk_, scal_.get());
            GBA_LAUNCH_CHECK();
            resid_valid_ = true;
        }
        const float2* rc = reinterpret_cast<const float2*>(r_cur_.get());
        cudaEvent_t ev = prof_start();
        point_pass_f32<<<n_pchunk_, kPT, 0, stream_>>>(pchunk_.get(), pt_off_.get(), s_cam_.get(), s_pt_.get(),
                                                       spx, cams_.get(), pts_.get(), rc, cam_pos_.get(), J32_.get(),
                                                       J32c_.get(), V_.get(), bp_.get(), counters_.get(),
                                                       static_cast<float>(huber_delta_));
        GBA_LAUNCH_CHECK();
        prof_stop("point_pass_f32", ev);
        if (n_cchunk_ > 0) {
            ev = prof_start();
            camera_pass_f32<<<n_cchunk_, kCT, 0, stream_>>>(cchunk_begin_.get(), cchunk_cam_.get(),
                                                            cam_off_.get(), cam_slots_.get(), s_pt_.get(), spx,
                                                            cams_.get(), pts_.get(), rc, cam_part_.get(),
                                                            static_cast<float>(huber_delta_));
            GBA_LAUNCH_CHECK();
            prof_stop("camera_pass_f32", ev);
        }
    }
    camera_finalize<<<ceil_div(54ll * C_, 256), 256, 0, stream_>>>(cam_chunk_off_.get(), cam_part_.get(), C_,
                                                                 U_.get(), bc_.get());
    GBA_LAUNCH_CHECK();
    double sse = 0.0;
    GBA_CUDA_CHECK(cudaMemcpyAsync(&sse, scal_.get(), sizeof(double), cudaMemcpyDeviceToHost, stream_));
    sync();
    return sse;
}

double Solver::trial_cost() {
    const double2* spx = reinterpret_cast<const double2*>(s_px_.get());
    cudaEvent_t ev = prof_start();
    camera_precompute_kernel<<<ceil_div(C_, 128), 128, 0, stream_>>>(tcams_.get(), C_, cam_pre_.get());
    GBA_LAUNCH_CHECK();
    cost_f64<<<n_pchunk_, kPT, 0, stream_>>>(pchunk_.get(), pt_off_.get(), s_cam_.get(), s_pt_.get(), spx,
                                             cam_pre_.get(), tpts_.get(), sse_part_.get(), counters_.get(),
                                             reinterpret_cast<float2*>(r_trial_.get()), huber_delta_);
    GBA_LAUNCH_CHECK();
    prof_stop("cost_f64", ev);
    ordered_sum<<<1, 256, 0, stream_>>>(sse_part_.get(), n_pchunk_, scal_.get() + 1);
    GBA_LAUNCH_CHECK();
    double sse = 0.0;
    GBA_CUDA_CHECK(cudaMemcpyAsync(&sse, scal_.get() + 1, sizeof(double), cudaMemcpyDeviceToHost, stream_));
    sync();
    return sse;
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

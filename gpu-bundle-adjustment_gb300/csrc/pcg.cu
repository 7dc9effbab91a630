// Mixed form: the reduced camera system S dc = rhs is never formed.
//
//   S x   = U_lambda x - sum_p W_p V'_p^-1 W_p^T x,   W_e = Jc_e^T Jp_e
//   rhs   = bc - sum_p W_p V'_p^-1 bp_p
//
// computed implicitly from the per-slot FP32 Jacobian records (J32 = Jc, Jp):
//   point pass   (slots sorted by point)  w_p = V'^-1 (a bp_p + sum_e Jp_e^T (Jc_e x_c)),
//                                         u_e = Jp_e w_p          (2 values per slot)
//   camera pass  (camera-major chunks)    partial_c = sum_e Jc_e^T u_e
//   finalize                              y = U_lambda x - sum partials   (or rhs = bc - ...)
// templated on the arithmetic type: FP32 inside PCG, FP64 for the right-hand
// side and the iterative-refinement residual. Chunk partials are summed in
// FP64 in a fixed order, so every product is deterministic.
//
// Solve: FP64 iterative refinement (dc += e, r = rhs - S64 dc, until
// ||r|| <= refine_tol ||rhs||) around inner block-Jacobi PCG solves on the FP32
// operator. The block-Jacobi blocks are the 9x9 diagonal blocks S_cc (FP32
// products, FP64 sums, FP64 Cholesky); the learned form replaces their
// factors by the MLP-corrected ones (mlp.cu). PCG vectors and dot products are
// FP64 with deterministic reductions; all PCG control scalars live on the
// device and the host polls a convergence flag every kCheck iterations.
//
// No reference counterpart: the reference solves S densely on the host.

#include "blocks.cuh"
#include "common.cuh"
#include "mlp.hpp"
#include "solver.hpp"

namespace gba {
namespace {

constexpr int kPT = 256;
constexpr int kCT = 128;
constexpr int kVT = 256;  // vector-kernel threads
constexpr int kCamChunk = 1024;
constexpr int kCheck = 8;
constexpr long long kJudgeMin = 8;  // inner iterations a judged solve needs to be decisive

// device scalar slots (pcg_s_)
enum { S_RZ = 0, S_ALPHA, S_BETA, S_RR, S_BB, S_DONE, S_ITERS, S_TOL2, S_NORM };

template <typename T>
__device__ __forceinline__ void load_j(const float* __restrict__ J32, long long s, T* J) {
    const float4* q = reinterpret_cast<const float4*>(J32 + 24 * s);
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const float4 v = q[k];
        J[4 * k] = static_cast<T>(v.x);
        J[4 * k + 1] = static_cast<T>(v.y);
        J[4 * k + 2] = static_cast<T>(v.z);
        J[4 * k + 3] = static_cast<T>(v.w);
    }
}

// Point pass of the implicit product. xt: the camera vector in the arithmetic
// type (an FP32 copy inside PCG), Vinv_t: V'^-1 in the arithmetic type (6 per
// point); u is written at the slot's camera-major position so that the camera
// pass reads it contiguously.
template <typename T>
__global__ void __launch_bounds__(kPT) schur_point_pass(const int* __restrict__ pchunk, const int* __restrict__ pt_off,
                                                       const int* __restrict__ s_cam, const int* __restrict__ s_pt,
                                                       const int* __restrict__ cam_pos, const float* __restrict__ J32,
                                                       const T* __restrict__ Vinv_t, const double* __restrict__ bp,
                                                       const T* __restrict__ xt, double a, T* __restrict__ u_cm,
                                                       const double* __restrict__ done) {
    __shared__ T seg[kPT][3];  // warp-segment partial sums, at each segment's last slot
    __shared__ T wsh[kPT][3];
    if (done && *done != 0.0) return;
    const int chunk = blockIdx.x;
    const int p0 = pchunk[chunk], p1 = pchunk[chunk + 1];
    const int s0 = pt_off[p0], s1 = pt_off[p1];
    const int my_p = p0 + threadIdx.x;
    const int lane = threadIdx.x & 31;
    int my_b = 0, my_e = 0;
    if (my_p < p1) {
        my_b = pt_off[my_p];
        my_e = pt_off[my_p + 1];
    }
    T z0 = T(0), z1 = T(0), z2 = T(0);
    // Single-pass chunks (the usual case) keep the slot's Jp, point and
    // camera-major position in registers for the u phase.
    const bool single = (s1 - s0) <= kPT;
    T jp[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
    int key = -1;  // point of the slot (slots past the chunk end share key -1, value 0)
    long long q = 0;
    if (xt) {
        for (int base = s0; base < s1; base += kPT) {
            const int s = base + threadIdx.x;
            T v0 = T(0), v1 = T(0), v2 = T(0);
            key = -1;
            if (s < s1) {
                key = s_pt[s];
                q = cam_pos[s];
                T J[24];
                load_j(J32, s, J);
#pragma unroll
                for (int k = 0; k < 6; ++k) jp[k] = J[18 + k];
                const T* xc = xt + 9ll * s_cam[s];
                T t0 = T(0), t1 = T(0);
#pragma unroll
                for (int k = 0; k < 9; ++k) {
                    const T xk = xc[k];
                    t0 += J[k] * xk;
                    t1 += J[9 + k] * xk;
                }
                v0 = J[18] * t0 + J[21] * t1;
                v1 = J[19] * t0 + J[22] * t1;
                v2 = J[20] * t0 + J[23] * t1;
            }
            // inclusive segmented scan over the warp (slots of a point are contiguous)
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const T u0 = __shfl_up_sync(0xffffffffu, v0, d);
                const T u1 = __shfl_up_sync(0xffffffffu, v1, d);
                const T u2 = __shfl_up_sync(0xffffffffu, v2, d);
                const int kd = __shfl_up_sync(0xffffffffu, key, d);
                if (lane >= d && kd == key) {
                    v0 += u0;
                    v1 += u1;
                    v2 += u2;
                }
            }
            const int knext = __shfl_down_sync(0xffffffffu, key, 1);
            if (lane == 31 || knext != key) {
                seg[threadIdx.x][0] = v0;
                seg[threadIdx.x][1] = v1;
                seg[threadIdx.x][2] = v2;
            }
            __syncthreads();
            // owner: add the point's warp-segment partials of this pass, warps in order
            if (my_p < p1) {
                const int b = max(my_b, base) - base, e = min(my_e, base + kPT) - base;
                for (int w = b >> 5; b < e && w <= (e - 1) >> 5; ++w) {
                    const int t = min(e - 1, 32 * w + 31);
                    z0 += seg[t][0];
                    z1 += seg[t][1];
                    z2 += seg[t][2];
                }
            }
            __syncthreads();
        }
    }
    if (my_p < p1) {
        if (a != 0.0) {
            z0 += static_cast<T>(a * bp[3ll * my_p]);
            z1 += static_cast<T>(a * bp[3ll * my_p + 1]);
            z2 += static_cast<T>(a * bp[3ll * my_p + 2]);
        }
        const T* Vi = Vinv_t + 6ll * my_p;
        const T v00 = Vi[0], v10 = Vi[1], v11 = Vi[2], v20 = Vi[3], v21 = Vi[4], v22 = Vi[5];
        wsh[threadIdx.x][0] = v00 * z0 + v10 * z1 + v20 * z2;
        wsh[threadIdx.x][1] = v10 * z0 + v11 * z1 + v21 * z2;
        wsh[threadIdx.x][2] = v20 * z0 + v21 * z1 + v22 * z2;
    }
    __syncthreads();
    // u_e = Jp_e w_p for every slot of the chunk, stored camera-major
    if (single && xt) {
        if (s0 + static_cast<int>(threadIdx.x) < s1) {
            const T w0 = wsh[key - p0][0], w1 = wsh[key - p0][1], w2 = wsh[key - p0][2];
            u_cm[2 * q] = jp[0] * w0 + jp[1] * w1 + jp[2] * w2;
            u_cm[2 * q + 1] = jp[3] * w0 + jp[4] * w1 + jp[5] * w2;
        }
        return;
    }
    for (int s = s0 + threadIdx.x; s < s1; s += kPT) {
        const int p = s_pt[s];
        const T w0 = wsh[p - p0][0], w1 = wsh[p - p0][1], w2 = wsh[p - p0][2];
        const float2* Jp2 = reinterpret_cast<const float2*>(J32 + 24ll * s + 18);
        const float2 j01 = Jp2[0], j23 = Jp2[1], j45 = Jp2[2];
        const long long qs = cam_pos[s];
        u_cm[2 * qs] = static_cast<T>(j01.x) * w0 + static_cast<T>(j01.y) * w1 + static_cast<T>(j23.x) * w2;
        u_cm[2 * qs + 1] = static_cast<T>(j23.y) * w0 + static_cast<T>(j45.x) * w1 + static_cast<T>(j45.y) * w2;
    }
}

// Camera pass: partial_c = sum over the chunk's camera-major positions of Jc^T u
// (Jc from the camera-major copy J32c, 20 floats per position; both contiguous).
template <typename T>
__global__ void __launch_bounds__(kCT) schur_camera_pass(const int* __restrict__ cchunk_begin,
                                                        const int* __restrict__ cchunk_cam,
                                                        const int* __restrict__ cam_off,
                                                        const float* __restrict__ J32c, const T* __restrict__ u_cm,
                                                        double* __restrict__ part, const double* __restrict__ done) {
    __shared__ double wpart[kCT / 32][9];
    if (done && *done != 0.0) return;
    const int k = blockIdx.x;
    const int b = cchunk_begin[k], c = cchunk_cam[k];
    const int e = min(b + kCamChunk, cam_off[c + 1]);
    T acc[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) acc[i] = T(0);
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
        const T u0 = u_cm[2ll * i], u1 = u_cm[2ll * i + 1];
#pragma unroll
        for (int t = 0; t < 9; ++t) acc[t] += static_cast<T>(Jc[t]) * u0 + static_cast<T>(Jc[9 + t]) * u1;
    }
    // Warp sums in the arithmetic type (FP32 shuffles stay off GB300's narrow
    // FP64 pipe); the four warp partials are added in FP64.
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int t = 0; t < 9; ++t) {
        const T v = warp_sum(acc[t]);
        if (lane == 0) wpart[warp][t] = static_cast<double>(v);
    }
    __syncthreads();
    if (threadIdx.x < 9) {
        double v = 0.0;
#pragma unroll
        for (int w = 0; w < kCT / 32; ++w) v += wpart[w][threadIdx.x];
        part[9ll * k + threadIdx.x] = v;
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
                                            int c, int k) {
    double s = 0.0;
    for (int q = cam_chunk_off[c]; q < cam_chunk_off[c + 1]; ++q) s += part[9ll * q + k];
    return s;
}

// rhs = bc - sum partials; partial ||rhs||^2 per block.
__global__ void __launch_bounds__(kVT) rhs_finalize(const int* __restrict__ cam_chunk_off,
                                                   const double* __restrict__ part, const double* __restrict__ bc,
                                                   int C, double* __restrict__ rhs, double* __restrict__ red) {
    __shared__ double sh[kVT / 32];
    const int i = blockIdx.x * kVT + threadIdx.x;
    double v = 0.0;
    if (i < 9 * C) {
        v = bc[i] - chunk_sum(cam_chunk_off, part, i / 9, i % 9);
        rhs[i] = v;
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

// q = S p (finalize) and partial p.q.
__global__ void __launch_bounds__(kVT) pcg_q_finalize(const int* __restrict__ cam_chunk_off,
                                                     const double* __restrict__ part, const double* __restrict__ U,
                                                     double lambda, const double* __restrict__ p, int C,
                                                     double* __restrict__ q, double* __restrict__ red,
                                                     const double* __restrict__ sc) {
    __shared__ double sh[kVT / 32];
    if (sc[S_DONE] != 0.0) return;
    const int i = blockIdx.x * kVT + threadIdx.x;
    double v = 0.0;
    if (i < 9 * C) {
        const int c = i / 9, k = i % 9;
        const double qi = damped_u_row_dot(U + 81ll * c, k, lambda, p + 9ll * c) - chunk_sum(cam_chunk_off, part, c, k);
        q[i] = qi;
        v = p[i] * qi;
    }
    const double t = block_sum<kVT>(v, sh);
    if (threadIdx.x == 0) red[blockIdx.x] = t;
}

__device__ __forceinline__ double ordered_block_sum(const double* __restrict__ red, int n, double* sh) {
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += 256) s += red[i];
    return block_sum<256>(s, sh);
}

__global__ void __launch_bounds__(256) pcg_alpha(const double* __restrict__ red, int n, double* __restrict__ sc) {
    __shared__ double sh[8];
    if (sc[S_DONE] != 0.0) return;
    const double pq = ordered_block_sum(red, n, sh);
    if (threadIdx.x == 0) {
        if (!(pq > 0.0) || !isfinite(pq)) {
            sc[S_DONE] = 2.0;  // breakdown: keep the current iterate
        } else {
            sc[S_ALPHA] = sc[S_RZ] / pq;
        }
    }
}

// z = M r with M = (L L^T)^-1 per camera (packed factor, 45 per camera).
__device__ __forceinline__ void precond_apply(const double* __restrict__ L, const double* r, double* z) {
    blk::chol9_solve(L, r, z);
}

// Thread per camera: x += alpha p, r -= alpha q, z = M r; partials r.r, r.z.
__global__ void __launch_bounds__(kVT) pcg_update(double* __restrict__ x, double* __restrict__ r,
                                                 double* __restrict__ z, const double* __restrict__ p,
                                                 const double* __restrict__ q, const double* __restrict__ L, int C,
                                                 double* __restrict__ red_rr, double* __restrict__ red_rz,
                                                 const double* __restrict__ sc) {
    __shared__ double sh[kVT / 32];
    if (sc[S_DONE] != 0.0) return;
    const int c = blockIdx.x * kVT + threadIdx.x;
    double rr = 0.0, rz = 0.0;
    if (c < C) {
        const double alpha = sc[S_ALPHA];
        double rc[9], zc[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            const long long i = 9ll * c + k;
            x[i] += alpha * p[i];
            rc[k] = r[i] - alpha * q[i];
            r[i] = rc[k];
            rr += rc[k] * rc[k];
        }
        precond_apply(L + 45ll * c, rc, zc);
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            z[9ll * c + k] = zc[k];
            rz += rc[k] * zc[k];
        }
    }
    const double a = block_sum<kVT>(rr, sh);
    const double b = block_sum<kVT>(rz, sh);
    if (threadIdx.x == 0) {
        red_rr[blockIdx.x] = a;
        red_rz[blockIdx.x] = b;
    }
}

__global__ void __launch_bounds__(256) pcg_beta(const double* __restrict__ red_rr, const double* __restrict__ red_rz,
                                               int n, int max_iters, double* __restrict__ sc) {
    __shared__ double sh[8];
    if (sc[S_DONE] != 0.0) return;
    const double rr = ordered_block_sum(red_rr, n, sh);
    const double rz = ordered_block_sum(red_rz, n, sh);
    if (threadIdx.x == 0) {
        sc[S_ITERS] += 1.0;
        sc[S_RR] = rr;
        if (rr <= sc[S_TOL2] * sc[S_BB] || sc[S_ITERS] >= max_iters) {
            sc[S_DONE] = 1.0;
        } else if (!(rz > 0.0) || !isfinite(rz)) {
            sc[S_DONE] = 2.0;
        } else {
            sc[S_BETA] = rz / sc[S_RZ];
            sc[S_RZ] = rz;
        }
    }
}

__global__ void __launch_bounds__(kVT) pcg_p_update(double* __restrict__ p, float* __restrict__ p32,
                                                   const double* __restrict__ z, int n, const double* __restrict__ sc) {
    if (sc[S_DONE] != 0.0) return;
    const int i = blockIdx.x * kVT + threadIdx.x;
    if (i < n) {
        const double v = z[i] + sc[S_BETA] * p[i];
        p[i] = v;
        p32[i] = static_cast<float>(v);
    }
}

// x = 0, r = b, z = M b, p = z; partials b.b and r.z.
__global__ void __launch_bounds__(kVT) pcg_init(double* __restrict__ x, double* __restrict__ r, double* __restrict__ z,
                                               double* __restrict__ p, float* __restrict__ p32,
                                               const double* __restrict__ b,
                                               const double* __restrict__ L, int C, double* __restrict__ red_rr,
                                               double* __restrict__ red_rz) {
    __shared__ double sh[kVT / 32];
    const int c = blockIdx.x * kVT + threadIdx.x;
    double rr = 0.0, rz = 0.0;
    if (c < C) {
        double rc[9], zc[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            rc[k] = b[9ll * c + k];
            x[9ll * c + k] = 0.0;
            r[9ll * c + k] = rc[k];
            rr += rc[k] * rc[k];
        }
        precond_apply(L + 45ll * c, rc, zc);
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            z[9ll * c + k] = zc[k];
            p[9ll * c + k] = zc[k];
            p32[9ll * c + k] = static_cast<float>(zc[k]);
            rz += rc[k] * zc[k];
        }
    }
    const double a = block_sum<kVT>(rr, sh);
    const double bb = block_sum<kVT>(rz, sh);
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

__global__ void __launch_bounds__(kVT) axpy_kernel(double* __restrict__ y, const double* __restrict__ x, int n) {
    const int i = blockIdx.x * kVT + threadIdx.x;
    if (i < n) y[i] += x[i];
}

// ---- block-Jacobi blocks S_cc = U_lambda,c - sum_{e in c} Jc^T (Jp V'^-1 Jp^T) Jc
__global__ void __launch_bounds__(kCT) sdiag_camera_pass(const int* __restrict__ cchunk_begin,
                                                        const int* __restrict__ cchunk_cam,
                                                        const int* __restrict__ cam_off,
                                                        const int* __restrict__ cam_slots, const int* __restrict__ s_pt,
                                                        const float* __restrict__ J32, const double* __restrict__ Vinv,
                                                        double* __restrict__ part) {
    __shared__ double wpart[kCT / 32][45];
    const int k = blockIdx.x;
    const int b = cchunk_begin[k], c = cchunk_cam[k];
    const int e = min(b + kCamChunk, cam_off[c + 1]);
    float acc[45];
#pragma unroll
    for (int i = 0; i < 45; ++i) acc[i] = 0.f;
    for (int i = b + threadIdx.x; i < e; i += kCT) {
        const long long s = cam_slots[i];
        float J[24];
        load_j(J32, s, J);
        const double* Vi = Vinv + 6ll * s_pt[s];
        const float v00 = Vi[0], v10 = Vi[1], v11 = Vi[2], v20 = Vi[3], v21 = Vi[4], v22 = Vi[5];
        const float* Jp = J + 18;
        // M = Jp V^-1 (2x3), G = M Jp^T (2x2 symmetric)
        float M[6];
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            const float a0 = Jp[3 * r], a1 = Jp[3 * r + 1], a2 = Jp[3 * r + 2];
            M[3 * r] = a0 * v00 + a1 * v10 + a2 * v20;
            M[3 * r + 1] = a0 * v10 + a1 * v11 + a2 * v21;
            M[3 * r + 2] = a0 * v20 + a1 * v21 + a2 * v22;
        }
        const float g00 = M[0] * Jp[0] + M[1] * Jp[1] + M[2] * Jp[2];
        const float g01 = M[0] * Jp[3] + M[1] * Jp[4] + M[2] * Jp[5];
        const float g11 = M[3] * Jp[3] + M[4] * Jp[4] + M[5] * Jp[5];
        // H = G Jc (2x9)
        float H0[9], H1[9];
#pragma unroll
        for (int t = 0; t < 9; ++t) {
            H0[t] = g00 * J[t] + g01 * J[9 + t];
            H1[t] = g01 * J[t] + g11 * J[9 + t];
        }
        int idx = 0;
#pragma unroll
        for (int a = 0; a < 9; ++a)
#pragma unroll
            for (int bb = 0; bb <= a; ++bb) {
                acc[idx] += J[a] * H0[bb] + J[9 + a] * H1[bb];
                ++idx;
            }
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int t = 0; t < 45; ++t) {
        const double v = warp_sum(static_cast<double>(acc[t]));
        if (lane == 0) wpart[warp][t] = v;
    }
    __syncthreads();
    if (threadIdx.x < 45) {
        double v = 0.0;
#pragma unroll
        for (int w = 0; w < kCT / 32; ++w) v += wpart[w][threadIdx.x];
        part[54ll * k + threadIdx.x] = v;
    }
}

// Packed Cholesky factor of a full 9x9 block; a block that is not SPD in FP64
// (round-off with tiny damping) falls back to the square root of its diagonal.
__device__ void factor_block(const double* A, double* Lc) {
    double f[45];
    if (!blk::chol9_factor(A, f)) {
#pragma unroll
        for (int i = 0; i < 45; ++i) f[i] = 0.0;
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const double d = A[10 * i];
            f[blk::tri(i, i)] = sqrt(d > 1e-300 ? d : 1e-300);
        }
    }
#pragma unroll
    for (int i = 0; i < 45; ++i) Lc[i] = f[i];
}

// Thread per camera: S_cc (full, FP64) and its packed Cholesky factor.
__global__ void __launch_bounds__(kVT) sdiag_finalize(const int* __restrict__ cam_chunk_off,
                                                     const double* __restrict__ part, const double* __restrict__ U,
                                                     double lambda, int C, double* __restrict__ Sdiag,
                                                     double* __restrict__ L) {
    const int c = blockIdx.x * kVT + threadIdx.x;
    if (c >= C) return;
    double A[81];
    const double* Uc = U + 81ll * c;
#pragma unroll
    for (int i = 0; i < 81; ++i) A[i] = Uc[i];
#pragma unroll
    for (int i = 0; i < 9; ++i) A[10 * i] += lambda * (Uc[10 * i] > 0.0 ? Uc[10 * i] : 1e-12);
    int idx = 0;
    for (int a = 0; a < 9; ++a)
        for (int b = 0; b <= a; ++b) {
            double s = 0.0;
            for (int q = cam_chunk_off[c]; q < cam_chunk_off[c + 1]; ++q) s += part[54ll * q + idx];
            A[9 * a + b] -= s;
            if (a != b) A[9 * b + a] = A[9 * a + b];
            ++idx;
        }
    double* Sd = Sdiag + 81ll * c;
#pragma unroll
    for (int i = 0; i < 81; ++i) Sd[i] = A[i];
    factor_block(A, L + 45ll * c);
}

// Block-Jacobi factors from stored diagonal blocks (the learned form's fallback).
__global__ void __launch_bounds__(kVT) factor_blocks_kernel(const double* __restrict__ Sdiag, int C,
                                                           double* __restrict__ L) {
    const int c = blockIdx.x * kVT + threadIdx.x;
    if (c >= C) return;
    double A[81];
#pragma unroll
    for (int i = 0; i < 81; ++i) A[i] = Sdiag[81ll * c + i];
    factor_block(A, L + 45ll * c);
}

}  // namespace

// Implicit product partials for a given x (FP32 or FP64 arithmetic). x is in
// the arithmetic type (FP32: the PCG direction copy; FP64: dc) or null (then
// a = 1: the right-hand side). Partials in cam_part_ (9 per chunk).
template <typename T>
static void implicit_parts(Solver& s, const T* x, double a, const double* done) {
    T* u = reinterpret_cast<T*>(s.u_.get());
    const bool f32 = sizeof(T) == 4;
    const T* vinv = f32 ? reinterpret_cast<const T*>(s.Vinv32_.get()) : reinterpret_cast<const T*>(s.Vinv_.get());
    cudaEvent_t ev = s.prof_start();
    schur_point_pass<T><<<s.n_pchunk_, kPT, 0, s.stream_>>>(s.pchunk_.get(), s.pt_off_.get(), s.s_cam_.get(),
                                                           s.s_pt_.get(), s.cam_pos_.get(), s.J32_.get(), vinv,
                                                           s.bp_.get(), x, a, u, done);
    GBA_LAUNCH_CHECK();
    s.prof_stop(f32 ? "schur_point_pass_f32" : "schur_point_pass_f64", ev);
    if (s.n_cchunk_ > 0) {
        ev = s.prof_start();
        schur_camera_pass<T><<<s.n_cchunk_, kCT, 0, s.stream_>>>(s.cchunk_begin_.get(), s.cchunk_cam_.get(),
                                                                 s.cam_off_.get(), s.J32c_.get(), u,
                                                                 s.cam_part_.get(), done);
        GBA_LAUNCH_CHECK();
        s.prof_stop(f32 ? "schur_camera_pass_f32" : "schur_camera_pass_f64", ev);
    }
}

PcgStats Solver::schur_pcg(double lambda, const LMOptions& opts, bool learned) {
    PcgStats st;
    const int n = 9 * C_;
    const int nvb = ceil_div(n, kVT);   // vector blocks (element-wise kernels)
    const int ncb = ceil_div(C_, kVT);  // camera blocks (per-camera kernels)
    double* red = red_part_.get();
    double* red2 = red_part_.get() + std::max(nvb, ncb) + 1;
    double* sc = pcg_s_.get();
    const double* done = sc + S_DONE;

    // right-hand side, FP64 arithmetic
    implicit_parts<double>(*this, static_cast<const double*>(nullptr), 1.0, nullptr);
    rhs_finalize<<<nvb, kVT, 0, stream_>>>(cam_chunk_off_.get(), cam_part_.get(), bc_.get(), C_, rhs_.get(), red);
    GBA_LAUNCH_CHECK();
    sum_to_scalar<<<1, 256, 0, stream_>>>(red, nvb, sc, S_NORM);
    GBA_LAUNCH_CHECK();

    // block-Jacobi blocks and factors (+ learned correction)
    if (n_cchunk_ > 0) {
        sdiag_camera_pass<<<n_cchunk_, kCT, 0, stream_>>>(cchunk_begin_.get(), cchunk_cam_.get(), cam_off_.get(),
                                                          cam_slots_.get(), s_pt_.get(), J32_.get(), Vinv_.get(),
                                                          cam_part_.get());
        GBA_LAUNCH_CHECK();
    }
    sdiag_finalize<<<ncb, kVT, 0, stream_>>>(cam_chunk_off_.get(), cam_part_.get(), U_.get(), lambda, C_,
                                             Sdiag_.get(), Pfac_.get());
    GBA_LAUNCH_CHECK();
    if (learned && !model_) throw std::invalid_argument("learned form: no model loaded");
    // Learned factors are used once they have won the judged solve (below).
    if (learned && learned_choice_ == 1) model_->correct_factors(*this, lambda);

    double bnorm2 = 0.0;
    GBA_CUDA_CHECK(cudaMemcpyAsync(&bnorm2, sc + S_NORM, sizeof(double), cudaMemcpyDeviceToHost, stream_));
    GBA_CUDA_CHECK(cudaMemsetAsync(dc_.get(), 0, n * sizeof(double), stream_));
    GBA_CUDA_CHECK(cudaMemcpyAsync(ref_r_.get(), rhs_.get(), n * sizeof(double), cudaMemcpyDeviceToDevice, stream_));
    sync();
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
    // Inner PCG on the FP32 operator, S32 e = r (e in pcg_x_). Returns the
    // iteration count; *ok = reached the inner tolerance without breakdown.
    auto inner_pcg = [&](bool* ok) -> long long {
        pcg_init<<<ncb, kVT, 0, stream_>>>(pcg_x_.get(), pcg_r_.get(), pcg_z_.get(), pcg_p_.get(), pcg_p32_.get(),
                                           ref_r_.get(),
                                           Pfac_.get(), C_, red, red2);
        GBA_LAUNCH_CHECK();
        pcg_init_finalize<<<1, 256, 0, stream_>>>(red, red2, ncb, opts.pcg_tol, sc);
        GBA_LAUNCH_CHECK();
        for (int it = 0; it < opts.pcg_max_iters; it += kCheck) {
            for (int j = 0; j < kCheck; ++j) {
                implicit_parts<float>(*this, pcg_p32_.get(), 0.0, done);
                pcg_q_finalize<<<nvb, kVT, 0, stream_>>>(cam_chunk_off_.get(), cam_part_.get(), U_.get(), lambda,
                                                         pcg_p_.get(), C_, pcg_q_.get(), red, sc);
                GBA_LAUNCH_CHECK();
                pcg_alpha<<<1, 256, 0, stream_>>>(red, nvb, sc);
                GBA_LAUNCH_CHECK();
                pcg_update<<<ncb, kVT, 0, stream_>>>(pcg_x_.get(), pcg_r_.get(), pcg_z_.get(), pcg_p_.get(),
                                                     pcg_q_.get(), Pfac_.get(), C_, red, red2, sc);
                GBA_LAUNCH_CHECK();
                pcg_beta<<<1, 256, 0, stream_>>>(red, red2, ncb, opts.pcg_max_iters, sc);
                GBA_LAUNCH_CHECK();
                pcg_p_update<<<nvb, kVT, 0, stream_>>>(pcg_p_.get(), pcg_p32_.get(), pcg_z_.get(), n, sc);
                GBA_LAUNCH_CHECK();
            }
            double flag = 0.0;
            GBA_CUDA_CHECK(cudaMemcpyAsync(&flag, done, sizeof(double), cudaMemcpyDeviceToHost, stream_));
            sync();
            if (flag != 0.0) break;
        }
        double h[9];
        GBA_CUDA_CHECK(cudaMemcpyAsync(h, sc, sizeof h, cudaMemcpyDeviceToHost, stream_));
        sync();
        *ok = h[S_DONE] != 2.0 && h[S_RR] <= h[S_TOL2] * h[S_BB];
        return static_cast<long long>(h[S_ITERS]);
    };
    bool use_learned = learned && learned_choice_ == 1;
    for (int step = 0; step < opts.refine_max_steps && rnorm2 > tol2; ++step) {
        bool ok = false;
        long long it_count = 0;
        if (learned && learned_choice_ == 0) {
            // Block-Jacobi judges the learned factors on the first inner solve of
            // the LM solve: both preconditioners solve it, and the one that
            // reaches the inner tolerance in fewer iterations serves for the rest
            // of the solve. Both solves count in pcg_iterations.
            bool ok_bj = false, ok_l = false;
            const long long it_bj = inner_pcg(&ok_bj);
            GBA_CUDA_CHECK(cudaMemcpyAsync(judge_x_.get(), pcg_x_.get(), n * sizeof(double),
                                           cudaMemcpyDeviceToDevice, stream_));
            model_->correct_factors(*this, lambda);
            const long long it_l = inner_pcg(&ok_l);
            judge_iters_[0] = it_bj;
            judge_iters_[1] = it_l;
            // Solves shorter than kJudgeMin iterations are too short to compare:
            // keep block-Jacobi for now and judge again at the next inner solve.
            const bool decisive = std::max(it_bj, it_l) >= kJudgeMin || !ok_bj || !ok_l;
            if (decisive && ok_l && (!ok_bj || it_l < it_bj)) {
                learned_choice_ = 1;
                use_learned = true;
                st.pcg_iterations += it_bj;
                it_count = it_l;
                ok = ok_l;
            } else {
                learned_choice_ = decisive ? 2 : 0;
                GBA_CUDA_CHECK(cudaMemcpyAsync(pcg_x_.get(), judge_x_.get(), n * sizeof(double),
                                               cudaMemcpyDeviceToDevice, stream_));
                factor_blocks_kernel<<<ncb, kVT, 0, stream_>>>(Sdiag_.get(), C_, Pfac_.get());
                GBA_LAUNCH_CHECK();
                st.pcg_iterations += it_l;
                it_count = it_bj;
                ok = ok_bj;
            }
        } else {
            it_count = inner_pcg(&ok);
        }
        if (use_learned && !ok) {
            // Block-Jacobi judges the learned factors: an inner solve that breaks
            // down or misses its tolerance is redone with the plain blocks, which
            // then serve for the rest of this trial.
            factor_blocks_kernel<<<ncb, kVT, 0, stream_>>>(Sdiag_.get(), C_, Pfac_.get());
            GBA_LAUNCH_CHECK();
            use_learned = false;
            ++st.fallbacks;
            st.pcg_iterations += it_count;
            it_count = inner_pcg(&ok);
        }
        const double iters = static_cast<double>(it_count);
        // dc += e; FP64 residual r = rhs - S64 dc
        axpy_kernel<<<nvb, kVT, 0, stream_>>>(dc_.get(), pcg_x_.get(), n);
        GBA_LAUNCH_CHECK();
        implicit_parts<double>(*this, static_cast<const double*>(dc_.get()), 0.0, nullptr);
        residual_finalize<<<nvb, kVT, 0, stream_>>>(cam_chunk_off_.get(), cam_part_.get(), U_.get(), lambda,
                                                    dc_.get(), rhs_.get(), C_, ref_r_.get(), red);
        GBA_LAUNCH_CHECK();
        sum_to_scalar<<<1, 256, 0, stream_>>>(red, nvb, sc, S_NORM);
        GBA_LAUNCH_CHECK();
        GBA_CUDA_CHECK(cudaMemcpyAsync(&rnorm2, sc + S_NORM, sizeof(double), cudaMemcpyDeviceToHost, stream_));
        sync();
        st.pcg_iterations += static_cast<long long>(iters);
        ++st.refine_steps;
        if (!std::isfinite(rnorm2)) break;
    }
    st.rel_residual = std::sqrt(rnorm2 / bnorm2);
    st.converged = rnorm2 <= tol2;
    return st;
}

}  // namespace gba

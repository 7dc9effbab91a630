// Batched small-block linear algebra (9x9 camera and 3x3 point blocks), the
// damped point-block inverse, the point back-substitution, the LM gain
// denominator and the trial-parameter update.
//
// Reference counterparts: schur.cuh:23-116 (chol9 factor/solve, inverse3_spd,
// batch kernels), src/lm.cu:289-302 (damp_invert_v_kernel) and the host loops
// src/lm.cu:606-654 (back-substitution, denominator, trial parameters), which
// here run on the device with deterministic reductions.

#include "blocks.cuh"
#include "common.cuh"
#include "ff.cuh"
#include "solver.hpp"

namespace gba {
namespace {

constexpr int kTB = 256;

// V' = V + lambda * max(diag V, 1e-12) on the diagonal; Vinv = V'^-1 (packed),
// FP64 (plain form).
__global__ void __launch_bounds__(kTB) damp_invert_v_kernel(const double* __restrict__ V, double lambda, int P,
                                                           double* __restrict__ Vinv,
                                                           unsigned long long* __restrict__ nonspd) {
    __shared__ unsigned long long redu[kTB / 32];
    unsigned long long bad = 0;
    for (int p = blockIdx.x * kTB + threadIdx.x; p < P; p += gridDim.x * kTB) {
        double a[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) a[k] = V[6ll * p + k];
        a[0] += lambda * (a[0] > 0.0 ? a[0] : 1e-12);
        a[2] += lambda * (a[2] > 0.0 ? a[2] : 1e-12);
        a[5] += lambda * (a[5] > 0.0 ? a[5] : 1e-12);
        double inv[6];
        if (!blk::inverse3_packed(a, inv)) {
            ++bad;
#pragma unroll
            for (int k = 0; k < 6; ++k) inv[k] = 0.0;
        }
#pragma unroll
        for (int k = 0; k < 6; ++k) Vinv[6ll * p + k] = inv[k];
    }
    const unsigned long long nb = block_sum_u64<kTB>(bad, redu);
    if (threadIdx.x == 0 && nb) atomicAdd(nonspd, nb);
}

// Mixed forms: the same damping and inverse in float-float arithmetic (V's
// entries are FP32 sums, exact in FP32), V'^-1 written as its FP32 rounding
// (Vinv32) and the FP32-rounded remainder (Vinv32lo). Cholesky L of the packed
// 3x3, M = L^-1, V'^-1 = M^T M; a non-positive pivot marks the block non-SPD.
__device__ __forceinline__ bool ff_gt0(ffa::ff a) { return a.hi > 0.f || (a.hi == 0.f && a.lo > 0.f); }

__global__ void __launch_bounds__(kTB) damp_invert_v_ff_kernel(const double* __restrict__ V, float2 lambda_ff,
                                                              int P, float* __restrict__ Vinv32,
                                                              float* __restrict__ Vinv32lo,
                                                              unsigned long long* __restrict__ nonspd) {
    using ffa::ff;
    __shared__ unsigned long long redu[kTB / 32];
    const ff lam = {lambda_ff.x, lambda_ff.y}, one = {1.f, 0.f};
    unsigned long long bad = 0;
    for (int p = blockIdx.x * kTB + threadIdx.x; p < P; p += gridDim.x * kTB) {
        ff a[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) a[k] = {static_cast<float>(V[6ll * p + k]), 0.f};
#pragma unroll
        for (int k : {0, 2, 5}) {
            const float d = a[k].hi > 0.f ? a[k].hi : 1e-12f;
            float pr, e;
            ffa::two_prod(d, lam.hi, pr, e);
            a[k] = ffa::norm(ffa::add(a[k], ff{pr, __fmaf_rn(d, lam.lo, e)}));
        }
        float h[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, l[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        bool ok = ff_gt0(a[0]);
        if (ok) {
            const ff l00 = ffa::sqrt(a[0]);
            const ff l10 = ffa::div(a[1], l00), l20 = ffa::div(a[3], l00);
            const ff t1 = ffa::norm(ffa::sub(a[2], ffa::mul(l10, l10)));
            ok = ff_gt0(t1);
            if (ok) {
                const ff l11 = ffa::sqrt(t1);
                const ff l21 = ffa::div(ffa::norm(ffa::sub(a[4], ffa::mul(l20, l10))), l11);
                const ff t2 = ffa::norm(ffa::sub(ffa::sub(a[5], ffa::mul(l20, l20)), ffa::mul(l21, l21)));
                ok = ff_gt0(t2);
                if (ok) {
                    const ff l22 = ffa::sqrt(t2);
                    const ff m00 = ffa::div(one, l00), m11 = ffa::div(one, l11), m22 = ffa::div(one, l22);
                    const ff m10 = ffa::neg(ffa::mul(ffa::mul(l10, m00), m11));
                    const ff m21 = ffa::neg(ffa::mul(ffa::mul(l21, m11), m22));
                    const ff m20 = ffa::neg(
                        ffa::mul(ffa::norm(ffa::add(ffa::mul(l20, m00), ffa::mul(l21, m10))), m22));
                    ff inv[6];
                    inv[0] = ffa::norm(ffa::add(ffa::add(ffa::mul(m00, m00), ffa::mul(m10, m10)), ffa::mul(m20, m20)));
                    inv[1] = ffa::norm(ffa::add(ffa::mul(m10, m11), ffa::mul(m20, m21)));
                    inv[2] = ffa::norm(ffa::add(ffa::mul(m11, m11), ffa::mul(m21, m21)));
                    inv[3] = ffa::mul(m20, m22);
                    inv[4] = ffa::mul(m21, m22);
                    inv[5] = ffa::mul(m22, m22);
#pragma unroll
                    for (int k = 0; k < 6; ++k) {
                        h[k] = inv[k].hi;
                        l[k] = inv[k].lo;
                    }
                }
            }
        }
        if (!ok) ++bad;
        float2* o = reinterpret_cast<float2*>(Vinv32 + 6ll * p);
        float2* ol = reinterpret_cast<float2*>(Vinv32lo + 6ll * p);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            o[k] = make_float2(h[2 * k], h[2 * k + 1]);
            ol[k] = make_float2(l[2 * k], l[2 * k + 1]);
        }
    }
    const unsigned long long nb = block_sum_u64<kTB>(bad, redu);
    if (threadIdx.x == 0 && nb) atomicAdd(nonspd, nb);
}

__global__ void batch_chol9_kernel(const double* __restrict__ A, const double* __restrict__ b, double* __restrict__ x,
                                   int* __restrict__ ok, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double L[45];
    const bool good = blk::chol9_factor(A + 81ll * i, L);
    ok[i] = good ? 1 : 0;
    if (good) {
        double xi[9], bi[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) bi[k] = b[9ll * i + k];
        blk::chol9_solve(L, bi, xi);
#pragma unroll
        for (int k = 0; k < 9; ++k) x[9ll * i + k] = xi[k];
    }
}

__global__ void batch_inverse3_kernel(const double* __restrict__ A, double* __restrict__ Ainv, int* __restrict__ ok,
                                      int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* a = A + 9ll * i;
    const double pk[6] = {a[0], a[3], a[4], a[6], a[7], a[8]};  // lower triangle, row-major
    double inv[6];
    const bool good = blk::inverse3_packed(pk, inv);
    ok[i] = good ? 1 : 0;
    if (good) {
        double* o = Ainv + 9ll * i;
        o[0] = inv[0]; o[1] = inv[1]; o[2] = inv[3];
        o[3] = inv[1]; o[4] = inv[2]; o[5] = inv[4];
        o[6] = inv[3]; o[7] = inv[4]; o[8] = inv[5];
    }
}

// Plain-form point back-substitution, one CTA per point chunk (slots sorted by
// point): dp_p = V'^-1_p (bp_p - sum_{e in p} W_e^T dc_{c(e)}), tpts = pts + dp,
// and the chunk's part of the gain denominator sum dp (lambda d dp + bp), all
// FP64 from the W records. (The mixed form runs the float-float point pass in
// its back-substitution mode instead.)
__global__ void __launch_bounds__(kTB) backsub_chunk_kernel(
    const int* __restrict__ pchunk, const int* __restrict__ pt_off, const int* __restrict__ s_cam,
    const double* __restrict__ W, const double* __restrict__ dc, const double* __restrict__ V,
    const double* __restrict__ Vinv, const double* __restrict__ bp, const double* __restrict__ pts, double lambda,
    double* __restrict__ dp, double* __restrict__ tpts, double* __restrict__ part) {
    __shared__ double contrib[3][kTB];
    __shared__ double red[kTB / 32];
    const int chunk = blockIdx.x;
    const int p0 = pchunk[chunk], p1 = pchunk[chunk + 1];
    const int s0 = pt_off[p0], s1 = pt_off[p1];
    const int my_p = p0 + threadIdx.x;
    int my_b = 0, my_e = 0;
    if (my_p < p1) {
        my_b = pt_off[my_p];
        my_e = pt_off[my_p + 1];
    }
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for (int base = s0; base < s1; base += kTB) {
        const int s = base + threadIdx.x;
        double v0 = 0.0, v1 = 0.0, v2 = 0.0;
        if (s < s1) {
            const double* We = W + 27ll * s;
            const double* d = dc + 9ll * s_cam[s];
#pragma unroll
            for (int i = 0; i < 9; ++i) {
                const double di = d[i];
                v0 += We[3 * i] * di;
                v1 += We[3 * i + 1] * di;
                v2 += We[3 * i + 2] * di;
            }
        }
        contrib[0][threadIdx.x] = v0;
        contrib[1][threadIdx.x] = v1;
        contrib[2][threadIdx.x] = v2;
        __syncthreads();
        if (my_p < p1) {
            const int b = max(my_b, base), e = min(my_e, base + kTB);
            for (int t = b; t < e; ++t) {
                a0 += contrib[0][t - base];
                a1 += contrib[1][t - base];
                a2 += contrib[2][t - base];
            }
        }
        __syncthreads();
    }
    double den = 0.0;
    if (my_p < p1) {
        const long long p = my_p;
        const double b0 = bp[3 * p], b1 = bp[3 * p + 1], b2 = bp[3 * p + 2];
        const double m0 = b0 - a0, m1 = b1 - a1, m2 = b2 - a2;
        const double* Vi = Vinv + 6 * p;  // packed (00,10,11,20,21,22)
        const double d0 = Vi[0] * m0 + Vi[1] * m1 + Vi[3] * m2;
        const double d1 = Vi[1] * m0 + Vi[2] * m1 + Vi[4] * m2;
        const double d2 = Vi[3] * m0 + Vi[4] * m1 + Vi[5] * m2;
        dp[3 * p] = d0;
        dp[3 * p + 1] = d1;
        dp[3 * p + 2] = d2;
        tpts[3 * p] = pts[3 * p] + d0;
        tpts[3 * p + 1] = pts[3 * p + 1] + d1;
        tpts[3 * p + 2] = pts[3 * p + 2] + d2;
        const double v0 = V[6 * p], v1 = V[6 * p + 2], v2 = V[6 * p + 5];
        den = d0 * (lambda * (v0 > 0.0 ? v0 : 1e-12) * d0 + b0) + d1 * (lambda * (v1 > 0.0 ? v1 : 1e-12) * d1 + b1) +
              d2 * (lambda * (v2 > 0.0 ? v2 : 1e-12) * d2 + b2);
    }
    const double t = block_sum<kTB>(den, red);
    if (threadIdx.x == 0) part[chunk] = t;
}

// Camera part of the denominator and the trial cameras (tcams = cams + dc);
// for the mixed back-substitution also dc's FP32 copy in the padded layout
// (dc32, kX32 per camera) or its float-float split (dcff), when given.
__global__ void __launch_bounds__(kTB) camera_step_kernel(const double* __restrict__ dc, const double* __restrict__ U,
                                                         const double* __restrict__ bc,
                                                         const double* __restrict__ cams, double lambda, int C,
                                                         double* __restrict__ tcams, double* __restrict__ part,
                                                         float* __restrict__ dc32, float2* __restrict__ dcff) {
    __shared__ double red[kTB / 32];
    double den = 0.0;
    const int i = blockIdx.x * kTB + threadIdx.x;
    if (i < 9 * C) {
        const int c = i / 9, k = i % 9;
        const double dg = U[81ll * c + 10 * k];
        const double d = dc[i];
        den = d * (lambda * (dg > 0.0 ? dg : 1e-12) * d + bc[i]);
        tcams[i] = cams[i] + d;
        if (dc32) dc32[kX32 * c + k] = static_cast<float>(d);
        if (dcff) {
            const ffa::ff f = ffa::from_double(d);
            dcff[i] = make_float2(f.hi, f.lo);
        }
    }
    const double t = block_sum<kTB>(den, red);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// denom = (camera partials in order) + (point partials in order).
constexpr int kSumT = 1024;

__global__ void __launch_bounds__(kSumT) denom_finalize(const double* __restrict__ part, int ncam, int npt,
                                                       double* __restrict__ out) {
    __shared__ double red[kSumT / 32];
    const double a = wide_block_sum<kSumT>(part, ncam, red);
    const double b = wide_block_sum<kSumT>(part + ncam, npt, red);
    if (threadIdx.x == 0) *out = a + b;
}

}  // namespace

unsigned long long Solver::damp_invert_v(double lambda) {
    damp_launch(lambda);
    unsigned long long bad = 0;
    read_back({{&bad, counters_.get() + 3, sizeof bad}});
    if (bad) add_nonspd(bad);
    return bad;
}

// keep the cumulative non-SPD count (reference counters[1])
void Solver::add_nonspd(unsigned long long n) {
    unsigned long long h[2];
    read_back({{h, counters_.get(), sizeof h}});
    h[1] += n;
    GBA_CUDA_CHECK(cudaMemcpyAsync(counters_.get(), h, sizeof h, cudaMemcpyHostToDevice, stream_));
    sync();
}

void Solver::damp_launch(double lambda) {
    GBA_CUDA_CHECK(cudaMemsetAsync(counters_.get() + 3, 0, sizeof(unsigned long long), stream_));
    const int grid = std::min(ceil_div(P_, kTB), 8 * device_sm_count());
    if (form_ == SolverForm::Plain) {
        damp_invert_v_kernel<<<grid, kTB, 0, stream_>>>(V_.get(), lambda, P_, Vinv_.get(), counters_.get() + 3);
    } else {
        const float lh = static_cast<float>(lambda);
        damp_invert_v_ff_kernel<<<grid, kTB, 0, stream_>>>(V_.get(), make_float2(lh, static_cast<float>(lambda - lh)),
                                                           P_, Vinv32_.get(), Vinv32lo_.get(), counters_.get() + 3);
    }
    GBA_LAUNCH_CHECK();
}

double Solver::back_substitute(double lambda) {
    backsub_launch(lambda);
    double denom = 0.0;
    read_back({{&denom, scal_.get() + 2, sizeof denom}});
    return denom;
}

double* Solver::backsub_part() { return red_part_.get() + ceil_div(9ll * C_, kTB); }

// dp, trial parameters and the gain denominator into scal_[2], without a host read.
void Solver::backsub_launch(double lambda, bool reuse) {
    const int ncam = ceil_div(9ll * C_, kTB);
    double* part = red_part_.get();
    const bool mixed = form_ != SolverForm::Plain;
    camera_step_kernel<<<ncam, kTB, 0, stream_>>>(dc_.get(), U_.get(), bc_.get(), cams_.get(), lambda, C_,
                                                  tcams_.get(), part, mixed && fast_solve_ ? pcg_p32_.get() : nullptr,
                                                  mixed && !fast_solve_ ? reinterpret_cast<float2*>(dcff_.get())
                                                                        : nullptr);
    GBA_LAUNCH_CHECK();
    cudaEvent_t ev = prof_start();
    if (form_ == SolverForm::Plain) {
        backsub_chunk_kernel<<<n_pchunk_, kTB, 0, stream_>>>(pchunk_.get(), pt_off_.get(), s_cam_.get(), W_.get(),
                                                             dc_.get(), V_.get(), Vinv_.get(), bp_.get(), pts_.get(),
                                                             lambda, dp_.get(), tpts_.get(), part + ncam);
        GBA_LAUNCH_CHECK();
        pts_ff_trial_ = false;
    } else if (!(reuse && backsub_ready_ && !fast_solve_)) {
        mixed_back_substitute(*this, lambda, part + ncam);
    }  // else: the last refinement check ran the point pass at this dc (dp, trial points, partials)
    backsub_ready_ = false;
    prof_stop("backsub", ev);
    denom_finalize<<<1, kSumT, 0, stream_>>>(part, ncam, n_pchunk_, scal_.get() + 2);
    GBA_LAUNCH_CHECK();
}

void launch_batch_chol9_factor_solve(const double* A, const double* b, double* x, int* ok, int n, cudaStream_t s) {
    if (n <= 0) return;
    batch_chol9_kernel<<<ceil_div(n, 128), 128, 0, s>>>(A, b, x, ok, n);
    GBA_LAUNCH_CHECK();
}

void launch_batch_inverse3_spd(const double* A, double* Ainv, int* ok, int n, cudaStream_t s) {
    if (n <= 0) return;
    batch_inverse3_kernel<<<ceil_div(n, 128), 128, 0, s>>>(A, Ainv, ok, n);
    GBA_LAUNCH_CHECK();
}

}  // namespace gba

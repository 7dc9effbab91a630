#pragma once
// Device routines for one small SPD block per thread (FP64 or FP32):
// 9x9 Cholesky factor / solve with the factor packed as a lower triangle
// (index i*(i+1)/2 + j, j <= i), and the 3x3 SPD inverse on packed storage
// (00, 10, 11, 20, 21, 22). Non-SPD input (a pivot that is not > 0, NaN
// included) returns false and leaves the output undefined.
// Reference: schur.cuh:23-96 (row-major 9x9 / 3x3 variants of the same
// textbook Cholesky-Banachiewicz recurrence).

namespace gba {
namespace blk {

template <typename T>
__device__ __forceinline__ T bsqrt(T x) { return sqrt(x); }
template <>
__device__ __forceinline__ float bsqrt<float>(float x) { return sqrtf(x); }

__host__ __device__ constexpr int tri(int i, int j) { return i * (i + 1) / 2 + j; }

// A: row-major 9x9, lower triangle read. L: packed lower (45).
template <typename T>
__device__ __forceinline__ bool chol9_factor(const T* A, T* L) {
#pragma unroll
    for (int i = 0; i < 9; ++i) {
#pragma unroll
        for (int j = 0; j <= i; ++j) {
            T s = A[9 * i + j];
#pragma unroll
            for (int k = 0; k < j; ++k) s -= L[tri(i, k)] * L[tri(j, k)];
            if (i == j) {
                if (!(s > T(0))) return false;
                L[tri(i, i)] = bsqrt(s);
            } else {
                L[tri(i, j)] = s / L[tri(j, j)];
            }
        }
    }
    return true;
}

// Same, from a packed symmetric lower triangle (45).
template <typename T>
__device__ __forceinline__ bool chol9_factor_packed(const T* A, T* L) {
#pragma unroll
    for (int i = 0; i < 9; ++i) {
#pragma unroll
        for (int j = 0; j <= i; ++j) {
            T s = A[tri(i, j)];
#pragma unroll
            for (int k = 0; k < j; ++k) s -= L[tri(i, k)] * L[tri(j, k)];
            if (i == j) {
                if (!(s > T(0))) return false;
                L[tri(i, i)] = bsqrt(s);
            } else {
                L[tri(i, j)] = s / L[tri(j, j)];
            }
        }
    }
    return true;
}

// Solve L L^T x = b.
template <typename T>
__device__ __forceinline__ void chol9_solve(const T* L, const T* b, T* x) {
    T y[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        T s = b[i];
#pragma unroll
        for (int k = 0; k < i; ++k) s -= L[tri(i, k)] * y[k];
        y[i] = s / L[tri(i, i)];
    }
#pragma unroll
    for (int i = 8; i >= 0; --i) {
        T s = y[i];
#pragma unroll
        for (int k = i + 1; k < 9; ++k) s -= L[tri(k, i)] * x[k];
        x[i] = s / L[tri(i, i)];
    }
}

// Inverse of a packed SPD 3x3 through its Cholesky factor: A^-1 = M^T M, M = L^-1.
template <typename T>
__device__ __forceinline__ bool inverse3_packed(const T* a, T* inv) {
    if (!(a[0] > T(0))) return false;
    const T l00 = bsqrt(a[0]);
    const T l10 = a[1] / l00, l20 = a[3] / l00;
    const T t1 = a[2] - l10 * l10;
    if (!(t1 > T(0))) return false;
    const T l11 = bsqrt(t1);
    const T l21 = (a[4] - l20 * l10) / l11;
    const T t2 = a[5] - l20 * l20 - l21 * l21;
    if (!(t2 > T(0))) return false;
    const T l22 = bsqrt(t2);
    const T m00 = T(1) / l00, m11 = T(1) / l11, m22 = T(1) / l22;
    const T m10 = -l10 * m00 * m11;
    const T m21 = -l21 * m11 * m22;
    const T m20 = -(l20 * m00 + l21 * m10) * m22;
    inv[0] = m00 * m00 + m10 * m10 + m20 * m20;
    inv[1] = m10 * m11 + m20 * m21;
    inv[2] = m11 * m11 + m21 * m21;
    inv[3] = m20 * m22;
    inv[4] = m21 * m22;
    inv[5] = m22 * m22;
    return true;
}

}  // namespace blk
}  // namespace gba

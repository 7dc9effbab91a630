#pragma once
// Snavely camera model: residual and analytic Jacobian of one observation,
// shared by the host (FP64 finite-difference entry point) and by the device
// edge kernels (FP64 plain form, FP32 mixed form).
//
// Model (BAL; reference src/lm.cu:58-82 and 93-191 evaluate the same function):
//   X_c = R(a) X + t,  u = -X_c.x / X_c.z,  v = -X_c.y / X_c.z,
//   d   = 1 + k1 r2 + k2 r2^2  (r2 = u^2 + v^2),  pred = f d (u, v),
//   residual = pred - obs.
// Rotation branch: the Rodrigues formula when |a|^2 > 1e-24 (FP64 threshold of
// the reference edge kernel, src/lm.cu:62-63), else the first-order model
// R(a) X = X + a x X with dR X/da = -[X]x and R = I (src/lm.cu:72-76,141-149).
//
// Jacobian derivation used here (own derivation, mathematically equal to the
// reference's): for a rotation vector a, R(a + da) X = R(a) X - [R X]x J_l(a) da,
// with the left Jacobian of SO(3)
//   J_l(a) = (s/th) I + ((1-c)/th) [w]x + (1 - s/th) w w^T,  w = a/th,
// so dX_c/da = -[R X]x J_l(a). (1 - c) is formed as 2 sin^2(th/2), which avoids
// cancellation at small th.
//   d(u,v)/dX_c = [[-1/z, 0, x/z^2], [0, -1/z, y/z^2]]
//   d pred/d(u,v) = f (d I + 2 L (u,v)^T (u,v)),  L = k1 + 2 k2 r2.

#ifdef __CUDACC__
#define GBA_HD __host__ __device__ __forceinline__
#else
#define GBA_HD inline
#endif

#include <cmath>

namespace gba {
namespace model {

template <typename T>
GBA_HD T msqrt(T x) { return sqrt(x); }
template <>
GBA_HD float msqrt<float>(float x) { return sqrtf(x); }
template <typename T>
GBA_HD void msincos(T x, T* s, T* c) { *s = sin(x); *c = cos(x); }
template <>
GBA_HD void msincos<float>(float x, float* s, float* c) { *s = sinf(x); *c = cosf(x); }
template <typename T>
GBA_HD T msin(T x) { return sin(x); }
template <>
GBA_HD float msin<float>(float x) { return sinf(x); }

// Rotated point R(a) X (without translation) and the pieces the Jacobian needs.
template <typename T>
struct Rotation {
    T RX[3];
    T R[9];    // row-major rotation matrix (dRX/dX)
    T Jl[9];   // row-major left Jacobian J_l(a); identity on the first-order branch
    bool first_order;
};

template <typename T>
GBA_HD void rotate(const T* a, const T* X, Rotation<T>& o) {
    const T th2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
    if (th2 > T(1e-24)) {
        const T th = msqrt(th2);
        const T inv = T(1) / th;
        const T w0 = a[0] * inv, w1 = a[1] * inv, w2 = a[2] * inv;
        T s, c;
        msincos(th, &s, &c);
        const T sh = msin(T(0.5) * th);
        const T omc = T(2) * sh * sh;  // 1 - cos th
        const T wX = w0 * X[0] + w1 * X[1] + w2 * X[2];
        const T cx0 = w1 * X[2] - w2 * X[1];
        const T cx1 = w2 * X[0] - w0 * X[2];
        const T cx2 = w0 * X[1] - w1 * X[0];
        o.RX[0] = c * X[0] + s * cx0 + omc * wX * w0;
        o.RX[1] = c * X[1] + s * cx1 + omc * wX * w1;
        o.RX[2] = c * X[2] + s * cx2 + omc * wX * w2;
        // R = c I + s [w]x + (1-c) w w^T
        o.R[0] = c + omc * w0 * w0;  o.R[1] = -s * w2 + omc * w0 * w1;  o.R[2] = s * w1 + omc * w0 * w2;
        o.R[3] = s * w2 + omc * w1 * w0;  o.R[4] = c + omc * w1 * w1;  o.R[5] = -s * w0 + omc * w1 * w2;
        o.R[6] = -s * w1 + omc * w2 * w0;  o.R[7] = s * w0 + omc * w2 * w1;  o.R[8] = c + omc * w2 * w2;
        // J_l = (s/th) I + ((1-c)/th) [w]x + (1 - s/th) w w^T
        const T p = s * inv, q = omc * inv, g = T(1) - p;
        o.Jl[0] = p + g * w0 * w0;  o.Jl[1] = -q * w2 + g * w0 * w1;  o.Jl[2] = q * w1 + g * w0 * w2;
        o.Jl[3] = q * w2 + g * w1 * w0;  o.Jl[4] = p + g * w1 * w1;  o.Jl[5] = -q * w0 + g * w1 * w2;
        o.Jl[6] = -q * w1 + g * w2 * w0;  o.Jl[7] = q * w0 + g * w2 * w1;  o.Jl[8] = p + g * w2 * w2;
        o.first_order = false;
    } else {
        o.RX[0] = X[0] + (a[1] * X[2] - a[2] * X[1]);
        o.RX[1] = X[1] + (a[2] * X[0] - a[0] * X[2]);
        o.RX[2] = X[2] + (a[0] * X[1] - a[1] * X[0]);
        for (int i = 0; i < 9; ++i) o.R[i] = (i % 4 == 0) ? T(1) : T(0);
        for (int i = 0; i < 9; ++i) o.Jl[i] = (i % 4 == 0) ? T(1) : T(0);
        o.first_order = true;
    }
}

// Residual only.
template <typename T>
GBA_HD void residual(const T* cam, const T* X, const T* obs, T* r) {
    T P[3];
    const T* a = cam;
    const T th2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
    if (th2 > T(1e-24)) {
        const T th = msqrt(th2);
        const T inv = T(1) / th;
        const T w0 = a[0] * inv, w1 = a[1] * inv, w2 = a[2] * inv;
        T s, c;
        msincos(th, &s, &c);
        const T sh = msin(T(0.5) * th);
        const T omc = T(2) * sh * sh;
        const T wX = w0 * X[0] + w1 * X[1] + w2 * X[2];
        P[0] = c * X[0] + s * (w1 * X[2] - w2 * X[1]) + omc * wX * w0 + cam[3];
        P[1] = c * X[1] + s * (w2 * X[0] - w0 * X[2]) + omc * wX * w1 + cam[4];
        P[2] = c * X[2] + s * (w0 * X[1] - w1 * X[0]) + omc * wX * w2 + cam[5];
    } else {
        P[0] = X[0] + (a[1] * X[2] - a[2] * X[1]) + cam[3];
        P[1] = X[1] + (a[2] * X[0] - a[0] * X[2]) + cam[4];
        P[2] = X[2] + (a[0] * X[1] - a[1] * X[0]) + cam[5];
    }
    const T iz = T(1) / P[2];
    const T u = -P[0] * iz, v = -P[1] * iz;
    const T r2 = u * u + v * v;
    const T d = T(1) + r2 * (cam[7] + cam[8] * r2);
    r[0] = cam[6] * d * u - obs[0];
    r[1] = cam[6] * d * v - obs[1];
}

// Residual + analytic Jacobian. Jc: 2x9 row-major (a[3], t[3], f, k1, k2);
// Jp: 2x3 row-major.
template <typename T>
GBA_HD void residual_jacobian(const T* cam, const T* X, const T* obs, T* r, T* Jc, T* Jp) {
    Rotation<T> rot;
    rotate(cam, X, rot);
    const T P0 = rot.RX[0] + cam[3], P1 = rot.RX[1] + cam[4], P2 = rot.RX[2] + cam[5];
    const T iz = T(1) / P2;
    const T u = -P0 * iz, v = -P1 * iz;
    const T r2 = u * u + v * v;
    const T f = cam[6], k1 = cam[7], k2 = cam[8];
    const T d = T(1) + r2 * (k1 + k2 * r2);
    const T L = k1 + T(2) * k2 * r2;
    r[0] = f * d * u - obs[0];
    r[1] = f * d * v - obs[1];

    // D = f (d I + 2 L [u v]^T [u v]), symmetric 2x2
    const T D00 = f * (d + T(2) * L * u * u);
    const T D01 = f * (T(2) * L * u * v);
    const T D11 = f * (d + T(2) * L * v * v);
    // M = d(u,v)/dX_c = [[-iz, 0, -u iz], [0, -iz, -v iz]]
    const T m02 = -u * iz, m12 = -v * iz;
    // DM = D M (2x3) = derivative of pred w.r.t. X_c
    T DM[6];
    DM[0] = -D00 * iz;  DM[1] = -D01 * iz;  DM[2] = D00 * m02 + D01 * m12;
    DM[3] = -D01 * iz;  DM[4] = -D11 * iz;  DM[5] = D01 * m02 + D11 * m12;

    // B = DM * (-[y]x) (2x3), y = R X (main branch) or X (first-order branch,
    // where dRX/da = -[X]x); [y]x = [[0,-y2,y1],[y2,0,-y0],[-y1,y0,0]].
    const T y0 = rot.first_order ? X[0] : rot.RX[0];
    const T y1 = rot.first_order ? X[1] : rot.RX[1];
    const T y2 = rot.first_order ? X[2] : rot.RX[2];
    T B[6];
    for (int row = 0; row < 2; ++row) {
        const T g0 = DM[row * 3 + 0], g1 = DM[row * 3 + 1], g2 = DM[row * 3 + 2];
        // (-[y]x) = [[0,y2,-y1],[-y2,0,y0],[y1,-y0,0]]
        B[row * 3 + 0] = -g1 * y2 + g2 * y1;
        B[row * 3 + 1] = g0 * y2 - g2 * y0;
        B[row * 3 + 2] = -g0 * y1 + g1 * y0;
    }
    for (int row = 0; row < 2; ++row) {
        // rotation columns: B * J_l
        for (int j = 0; j < 3; ++j)
            Jc[row * 9 + j] = B[row * 3 + 0] * rot.Jl[0 * 3 + j] + B[row * 3 + 1] * rot.Jl[1 * 3 + j] +
                              B[row * 3 + 2] * rot.Jl[2 * 3 + j];
        for (int j = 0; j < 3; ++j) Jc[row * 9 + 3 + j] = DM[row * 3 + j];
        const T p = row == 0 ? u : v;
        Jc[row * 9 + 6] = d * p;
        Jc[row * 9 + 7] = f * r2 * p;
        Jc[row * 9 + 8] = f * r2 * r2 * p;
        for (int j = 0; j < 3; ++j)
            Jp[row * 3 + j] = DM[row * 3 + 0] * rot.R[0 * 3 + j] + DM[row * 3 + 1] * rot.R[1 * 3 + j] +
                              DM[row * 3 + 2] * rot.R[2 * 3 + j];
    }
}

// Residual + Jacobian from per-camera constants precomputed once per camera
// (in FP64, stored in T): pre = [R (9, row-major), J_l (9), t (3), f, k1, k2,
// first_order (0 / 1)]. On the first-order branch R = I + [a]x (so R X is the
// branch's X + a x X), J_l = I, and the branch's dRX/da = -[X]x and dX_c/dX = I
// are applied here; otherwise the same formulas as residual_jacobian.
template <typename T>
GBA_HD void residual_jacobian_pre(const T* pre, const T* X, const T* obs, T* r, T* Jc, T* Jp) {
    const T* R = pre;
    const T* Jl = pre + 9;
    const bool first_order = pre[24] != T(0);
    T RX[3];
    for (int i = 0; i < 3; ++i) RX[i] = R[3 * i] * X[0] + R[3 * i + 1] * X[1] + R[3 * i + 2] * X[2];
    const T P0 = RX[0] + pre[18], P1 = RX[1] + pre[19], P2 = RX[2] + pre[20];
    const T iz = T(1) / P2;
    const T u = -P0 * iz, v = -P1 * iz;
    const T r2 = u * u + v * v;
    const T f = pre[21], k1 = pre[22], k2 = pre[23];
    const T d = T(1) + r2 * (k1 + k2 * r2);
    const T L = k1 + T(2) * k2 * r2;
    r[0] = f * d * u - obs[0];
    r[1] = f * d * v - obs[1];
    const T D00 = f * (d + T(2) * L * u * u);
    const T D01 = f * (T(2) * L * u * v);
    const T D11 = f * (d + T(2) * L * v * v);
    const T m02 = -u * iz, m12 = -v * iz;
    T DM[6];
    DM[0] = -D00 * iz;  DM[1] = -D01 * iz;  DM[2] = D00 * m02 + D01 * m12;
    DM[3] = -D01 * iz;  DM[4] = -D11 * iz;  DM[5] = D01 * m02 + D11 * m12;
    const T y0 = first_order ? X[0] : RX[0];
    const T y1 = first_order ? X[1] : RX[1];
    const T y2 = first_order ? X[2] : RX[2];
    for (int row = 0; row < 2; ++row) {
        const T g0 = DM[row * 3 + 0], g1 = DM[row * 3 + 1], g2 = DM[row * 3 + 2];
        const T b0 = -g1 * y2 + g2 * y1, b1 = g0 * y2 - g2 * y0, b2 = -g0 * y1 + g1 * y0;
        for (int j = 0; j < 3; ++j) Jc[row * 9 + j] = b0 * Jl[j] + b1 * Jl[3 + j] + b2 * Jl[6 + j];
        for (int j = 0; j < 3; ++j) Jc[row * 9 + 3 + j] = DM[row * 3 + j];
        const T p = row == 0 ? u : v;
        Jc[row * 9 + 6] = d * p;
        Jc[row * 9 + 7] = f * r2 * p;
        Jc[row * 9 + 8] = f * r2 * r2 * p;
        for (int j = 0; j < 3; ++j)
            Jp[row * 3 + j] = first_order ? DM[row * 3 + j]
                                          : g0 * R[j] + g1 * R[3 + j] + g2 * R[6 + j];
    }
}

// The per-camera constants of residual_jacobian_pre, in FP64 (28 slots; the
// last three are padding).
GBA_HD void camera_constants(const double* a, double* o) {
    const double th2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
    if (th2 > 1e-24) {
        const double th = sqrt(th2);
        const double inv = 1.0 / th;
        const double w0 = a[0] * inv, w1 = a[1] * inv, w2 = a[2] * inv;
        const double s = sin(th), c = cos(th), sh = sin(0.5 * th);
        const double omc = 2.0 * sh * sh;
        o[0] = c + omc * w0 * w0;  o[1] = -s * w2 + omc * w0 * w1;  o[2] = s * w1 + omc * w0 * w2;
        o[3] = s * w2 + omc * w1 * w0;  o[4] = c + omc * w1 * w1;  o[5] = -s * w0 + omc * w1 * w2;
        o[6] = -s * w1 + omc * w2 * w0;  o[7] = s * w0 + omc * w2 * w1;  o[8] = c + omc * w2 * w2;
        const double p = s * inv, q = omc * inv, g = 1.0 - p;
        o[9] = p + g * w0 * w0;  o[10] = -q * w2 + g * w0 * w1;  o[11] = q * w1 + g * w0 * w2;
        o[12] = q * w2 + g * w1 * w0;  o[13] = p + g * w1 * w1;  o[14] = -q * w0 + g * w1 * w2;
        o[15] = -q * w1 + g * w2 * w0;  o[16] = q * w0 + g * w2 * w1;  o[17] = p + g * w2 * w2;
        o[24] = 0.0;
    } else {
        o[0] = 1.0;   o[1] = -a[2]; o[2] = a[1];
        o[3] = a[2];  o[4] = 1.0;   o[5] = -a[0];
        o[6] = -a[1]; o[7] = a[0];  o[8] = 1.0;
        for (int i = 0; i < 9; ++i) o[9 + i] = (i % 4 == 0) ? 1.0 : 0.0;
        o[24] = 1.0;
    }
    for (int i = 0; i < 6; ++i) o[18 + i] = a[3 + i];
    o[25] = o[26] = o[27] = 0.0;
}

}  // namespace model
}  // namespace gba

// Small dense linear algebra and SE(3) helpers used on the device (in the
// solve step of the tracking kernels) and on the host (covariance).
//
// Restates the arithmetic of the reference host loop
// (src/odom/RGBDOdometryef.cpp:292-595, src/odom/utils.h:16-74) and of the
// Eigen 3.3 routines it calls (Eigen is a third-party dependency of the
// reference and is not vendored):
//  - LDLT with symmetric pivoting on the largest remaining |diagonal| and a
//    pseudo-inverse of D (|d| <= the smallest normal number -> 0);
//  - 3x3 inverse by cofactors, 4x4 rigid inverse, 6x6 LU inverse with
//    partial pivoting;
//  - Transform::rotation() = polar factor of the linear part, computed with
//    Newton iterations X <- (X + X^-T) / 2 in FP64.
#pragma once
#include <cfloat>
#include <cmath>

#if defined(__CUDACC__)
#define SE3_HD __host__ __device__ __forceinline__
#else
#define SE3_HD inline
#endif

namespace slamgb {
namespace se3 {

template <typename T>
SE3_HD T tiny();
template <>
SE3_HD double tiny<double>() { return DBL_MIN; }
template <>
SE3_HD float tiny<float>() { return FLT_MIN; }

template <typename T>
SE3_HD T tabs(T v) { return v < T(0) ? -v : v; }

// x = A^-1 b for symmetric A (row-major n x n, n <= 6).
template <typename T, int n>
SE3_HD void ldlt_solve(const T *Ain, const T *b, T *x) {
    T A[n * n];
    int perm[n];
    for (int i = 0; i < n * n; ++i) A[i] = Ain[i];
    for (int i = 0; i < n; ++i) perm[i] = i;
    for (int k = 0; k < n; ++k) {
        int p = k;
        T best = tabs(A[k * n + k]);
        for (int i = k + 1; i < n; ++i)
            if (tabs(A[i * n + i]) > best) {
                best = tabs(A[i * n + i]);
                p = i;
            }
        if (p != k) {
            for (int j = 0; j < n; ++j) { T t = A[k * n + j]; A[k * n + j] = A[p * n + j]; A[p * n + j] = t; }
            for (int i = 0; i < n; ++i) { T t = A[i * n + k]; A[i * n + k] = A[i * n + p]; A[i * n + p] = t; }
            int t = perm[k]; perm[k] = perm[p]; perm[p] = t;
        }
        T t[n];
        for (int j = 0; j < k; ++j) t[j] = A[k * n + j] * A[j * n + j];
        T s = 0;
        for (int j = 0; j < k; ++j) s += A[k * n + j] * t[j];
        A[k * n + k] -= s;
        const T akk = A[k * n + k];
        for (int i = k + 1; i < n; ++i) {
            T r = 0;
            for (int j = 0; j < k; ++j) r += A[i * n + j] * t[j];
            A[i * n + k] -= r;
            if (tabs(akk) > T(0)) A[i * n + k] /= akk;
        }
    }
    T y[n];
    for (int i = 0; i < n; ++i) y[i] = b[perm[i]];
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < i; ++j) y[i] -= A[i * n + j] * y[j];
    for (int i = 0; i < n; ++i) y[i] = tabs(A[i * n + i]) > tiny<T>() ? y[i] / A[i * n + i] : T(0);
    for (int i = n - 1; i >= 0; --i)
        for (int j = i + 1; j < n; ++j) y[i] -= A[j * n + i] * y[j];
    for (int i = 0; i < n; ++i) x[perm[i]] = y[i];
}

template <typename T>
SE3_HD void inv33(const T *m, T *o) {
    T c00 = m[4] * m[8] - m[5] * m[7], c01 = m[5] * m[6] - m[3] * m[8], c02 = m[3] * m[7] - m[4] * m[6];
    T det = m[0] * c00 + m[1] * c01 + m[2] * c02;
    T id = T(1) / det;
    o[0] = c00 * id; o[1] = (m[2] * m[7] - m[1] * m[8]) * id; o[2] = (m[1] * m[5] - m[2] * m[4]) * id;
    o[3] = c01 * id; o[4] = (m[0] * m[8] - m[2] * m[6]) * id; o[5] = (m[2] * m[3] - m[0] * m[5]) * id;
    o[6] = c02 * id; o[7] = (m[1] * m[6] - m[0] * m[7]) * id; o[8] = (m[0] * m[4] - m[1] * m[3]) * id;
}

template <typename T>
SE3_HD void mm33(const T *a, const T *b, T *o) {
    T t[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) t[i * 3 + j] = a[i * 3] * b[j] + a[i * 3 + 1] * b[3 + j] + a[i * 3 + 2] * b[6 + j];
    for (int k = 0; k < 9; ++k) o[k] = t[k];
}

// OdometryProvider::rodrigues, src/odom/utils.h:16-52.
SE3_HD void rodrigues(const double *src, double *R) {
    for (int k = 0; k < 9; ++k) R[k] = (k % 4 == 0) ? 1.0 : 0.0;
    double rx = src[0], ry = src[1], rz = src[2];
    double theta = sqrt(rx * rx + ry * ry + rz * rz);
    if (theta >= DBL_EPSILON) {
        double c = cos(theta), s = sin(theta), c1 = 1. - c, it = theta ? 1. / theta : 0.;
        rx *= it; ry *= it; rz *= it;
        const double I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        const double rrt[9] = {rx * rx, rx * ry, rx * rz, rx * ry, ry * ry, ry * rz, rx * rz, ry * rz, rz * rz};
        const double rx_[9] = {0, -rz, ry, rz, 0, -rx, -ry, rx, 0};
        for (int k = 0; k < 9; ++k) R[k] = c * I[k] + c1 * rrt[k] + s * rx_[k];
    }
}

// Polar factor of a float 3x3 (the rotation() of an Eigen 3.3 Isometry).
SE3_HD void polar33(const float *Min, float *Rout) {
    double X[9];
    for (int k = 0; k < 9; ++k) X[k] = (double)Min[k];
    for (int it = 0; it < 2; ++it) {
        double Xi[9];
        inv33(X, Xi);
        double Y[9];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) Y[i * 3 + j] = 0.5 * (X[i * 3 + j] + Xi[j * 3 + i]);
        for (int k = 0; k < 9; ++k) X[k] = Y[k];
    }
    for (int k = 0; k < 9; ++k) Rout[k] = (float)X[k];
}

// One Gauss-Newton pose update (src/odom/RGBDOdometryef.cpp:533-575 and
// computeUpdateSE3, src/odom/utils.h:54-74): solve A x = b, left-compose
// [R(x[3:6]) | x[0:3]] onto resultRt (FP64 4x4 row-major), then
// currentT = [Rprev | tprev] * rgbOdom^-1 in FP32.
#if defined(__CUDA_ARCH__)
#define SE3_MARK(i) \
    if (marks) asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(marks[i]))
#else
#define SE3_MARK(i)
#endif
SE3_HD void gn_update(const double *A, const double *b, double *resultRt, const float *Rprev, const float *tprev,
                      float *Rcurr, float *tcurr, double *x_out = nullptr, unsigned long long *marks = nullptr) {
    double x[6];
    SE3_MARK(0);
    ldlt_solve<double, 6>(A, b, x);
    SE3_MARK(1);
    if (x_out)
        for (int k = 0; k < 6; ++k) x_out[k] = x[k];
    double Rinc[9];
    rodrigues(x + 3, Rinc);
    const double Rt4[16] = {Rinc[0], Rinc[1], Rinc[2], x[0], Rinc[3], Rinc[4], Rinc[5], x[1],
                            Rinc[6], Rinc[7], Rinc[8], x[2], 0, 0, 0, 1};
    double nr[16];
    for (int a = 0; a < 4; ++a)
        for (int c = 0; c < 4; ++c) {
            double s = 0;
            for (int k = 0; k < 4; ++k) s += Rt4[a * 4 + k] * resultRt[k * 4 + c];
            nr[a * 4 + c] = s;
        }
    for (int k = 0; k < 16; ++k) resultRt[k] = nr[k];
    SE3_MARK(2);
    float oR[9], ot[3];
    for (int a = 0; a < 3; ++a) {
        for (int c = 0; c < 3; ++c) oR[a * 3 + c] = (float)resultRt[a * 4 + c];
        ot[a] = (float)resultRt[a * 4 + 3];
    }
    float iR[9], it[3];
    for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c) iR[a * 3 + c] = oR[c * 3 + a];
    for (int a = 0; a < 3; ++a) it[a] = -(iR[a * 3] * ot[0] + iR[a * 3 + 1] * ot[1] + iR[a * 3 + 2] * ot[2]);
    float cR[9];
    mm33(Rprev, iR, cR);
    for (int a = 0; a < 3; ++a)
        tcurr[a] = (Rprev[a * 3] * it[0] + Rprev[a * 3 + 1] * it[1] + Rprev[a * 3 + 2] * it[2]) + tprev[a];
    polar33(cR, Rcurr);
    SE3_MARK(3);
}

// K R K^-1 and K t of resultRt^-1 for the photometric warp
// (src/odom/RGBDOdometryef.cpp:422-432).
SE3_HD void warp_params(const double *resultRt, double fx, double fy, double cx, double cy, float *krkinv, float *kt) {
    double R[9], t[3];
    for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c) R[a * 3 + c] = resultRt[c * 4 + a];
    for (int a = 0; a < 3; ++a) t[a] = -(R[a * 3] * resultRt[3] + R[a * 3 + 1] * resultRt[7] + R[a * 3 + 2] * resultRt[11]);
    const double K[9] = {fx, 0, cx, 0, fy, cy, 0, 0, 1};
    double Ki[9], KR[9], KRKi[9];
    inv33(K, Ki);
    mm33(K, R, KR);
    mm33(KR, Ki, KRKi);
    for (int k = 0; k < 9; ++k) krkinv[k] = (float)KRKi[k];
    for (int a = 0; a < 3; ++a) kt[a] = (float)(K[a * 3] * t[0] + K[a * 3 + 1] * t[1] + K[a * 3 + 2] * t[2]);
}

// 6x6 inverse by LU with partial pivoting (getCovariance,
// src/odom/RGBDOdometryef.cpp:597-600).
SE3_HD void inverse6(const double *Ain, double *inv) {
    double A[36];
    for (int i = 0; i < 36; ++i) { A[i] = Ain[i]; inv[i] = (i % 7 == 0) ? 1.0 : 0.0; }
    for (int k = 0; k < 6; ++k) {
        int p = k;
        for (int i = k + 1; i < 6; ++i)
            if (tabs(A[i * 6 + k]) > tabs(A[p * 6 + k])) p = i;
        if (p != k)
            for (int j = 0; j < 6; ++j) {
                double t = A[k * 6 + j]; A[k * 6 + j] = A[p * 6 + j]; A[p * 6 + j] = t;
                t = inv[k * 6 + j]; inv[k * 6 + j] = inv[p * 6 + j]; inv[p * 6 + j] = t;
            }
        double d = A[k * 6 + k];
        for (int j = 0; j < 6; ++j) { A[k * 6 + j] /= d; inv[k * 6 + j] /= d; }
        for (int i = 0; i < 6; ++i)
            if (i != k) {
                double f = A[i * 6 + k];
                for (int j = 0; j < 6; ++j) { A[i * 6 + j] -= f * A[k * 6 + j]; inv[i * 6 + j] -= f * inv[k * 6 + j]; }
            }
    }
}

}  // namespace se3
}  // namespace slamgb

// arap_device.cuh -- device helpers shared by the single-pose and batched
// kernels: precision traits and the 3x3 rotation fit of the local step
// (inc/deform/arap.h:376-382).
#pragma once

#include <cuda_runtime.h>

#include "arap_kernels.h"

namespace arapgpu {
namespace dev {

template <typename T> __device__ __forceinline__ T tsqrt(T x);
template <> __device__ __forceinline__ float tsqrt(float x) { return sqrtf(x); }
template <> __device__ __forceinline__ double tsqrt(double x) { return sqrt(x); }

template <typename T> struct Eps;
template <> struct Eps<float> { static constexpr float v = 1.1920929e-07f; };
template <> struct Eps<double> { static constexpr double v = 2.220446049250313e-16; };

// One-sided (Hestenes) Jacobi on a 3x3 matrix (Golub & Van Loan, Sec. 8.6.3;
// Demmel & Veselic 1992): plane rotations from the right orthogonalise the
// columns of B = S J1 J2 ..., V accumulates the rotations. On exit the columns
// of B are sigma_i u_i and those of V the right singular vectors. Working on S
// itself, not on S^T S, keeps the small singular directions accurate in FP32
// (the one-rings stretched close to rank one in the first iterations of a
// large handle move).
template <typename T>
__device__ __forceinline__ void hestenes3(T B[3][3], T V[3][3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) V[i][j] = (i == j) ? (T)1 : (T)0;
    const int sweeps = sizeof(T) == 4 ? 8 : 12;
    for (int sw = 0; sw < sweeps; ++sw) {
        bool rotated = false;
#pragma unroll
        for (int pq = 0; pq < 3; ++pq) {
            const int p = pq == 2 ? 1 : 0;
            const int q = pq == 0 ? 1 : 2;
            const T a = B[0][p] * B[0][p] + B[1][p] * B[1][p] + B[2][p] * B[2][p];
            const T b = B[0][q] * B[0][q] + B[1][q] * B[1][q] + B[2][q] * B[2][q];
            const T g = B[0][p] * B[0][q] + B[1][p] * B[1][q] + B[2][p] * B[2][q];
            if (fabs(g) <= Eps<T>::v * tsqrt(a * b)) continue;  // columns orthogonal to working precision
            rotated = true;
            // t = tan of the angle that makes the new columns orthogonal, the
            // root of t^2 + 2 zeta t - 1 = 0 of smaller magnitude
            const T zeta = (b - a) / ((T)2 * g);
            const T az = fabs(zeta);
            const T r = az > (T)1 ? az * tsqrt((T)1 + (T)1 / (az * az)) : tsqrt((T)1 + az * az);
            const T t = (zeta < (T)0 ? (T)-1 : (T)1) / (az + r);
            const T c = (T)1 / tsqrt((T)1 + t * t);
            const T sn = c * t;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const T bp = B[i][p], bq = B[i][q];
                B[i][p] = c * bp - sn * bq;
                B[i][q] = sn * bp + c * bq;
                const T vp = V[i][p], vq = V[i][q];
                V[i][p] = c * vp - sn * vq;
                V[i][q] = sn * vp + c * vq;
            }
        }
        if (!rotated) break;
    }
}

// Best rotation R = V diag(1,1,det(V U^T)) U^T for cov = U S V^T (arap.h:376-382),
// from the one-sided Jacobi SVD of cov: the right singular vectors v1, v2 of
// the two largest singular values and v3 = v1 x v2 (proper), the left ones
// u1 = b1/|b1|, u2 = Gram-Schmidt(b2) and u3 = u1 x u2 (proper). With both
// factors proper the sign of det(V U^T) lands on the smallest singular value,
// as the reference's reflection fix puts it.
// spread (optional): (sigma_2 + sigma_3) / sigma_1 of cov, which bounds how
// well R is determined by it (the polar factor's condition number is about
// its inverse); 0 for a zero covariance.
template <typename T>
__device__ __forceinline__ void rotation_from_cov(const T S_in[3][3], T R[3][3], T *spread = nullptr) {
    if (spread) *spread = (T)0;
    T f2 = (T)0;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) f2 += S_in[i][j] * S_in[i][j];
    if (!(f2 > (T)0)) {
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) R[i][j] = (i == j) ? (T)1 : (T)0;
        return;
    }
    const T sc = (T)1 / tsqrt(f2);
    T B[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) B[i][j] = S_in[i][j] * sc;
    T Vm[3][3];
    hestenes3(B, Vm);
    // singular values (column norms of B), ordered descending
    T nrm[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) nrm[j] = B[0][j] * B[0][j] + B[1][j] * B[1][j] + B[2][j] * B[2][j];
    // indices of the largest and second largest (ties keep the lower index)
    const int o0 = (nrm[1] > nrm[0]) ? ((nrm[2] > nrm[1]) ? 2 : 1) : ((nrm[2] > nrm[0]) ? 2 : 0);
    const int lo = o0 == 0 ? 1 : 0, hi = o0 == 2 ? 1 : 2;  // the other two, lo < hi
    const T nlo = lo == 0 ? nrm[0] : nrm[1], nhi = hi == 1 ? nrm[1] : nrm[2];
    const int o1 = (nhi > nlo) ? hi : lo;
    if (spread) {
        const T n0 = o0 == 0 ? nrm[0] : (o0 == 1 ? nrm[1] : nrm[2]);
        *spread = (tsqrt(nlo) + tsqrt(nhi)) / tsqrt(n0);
    }
    T v1[3], v2[3], v3[3];
    T u1[3], u2[3], u3[3];
    // columns picked by selects, not by indexing with o0/o1 (keeps every
    // array in registers)
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        v1[i] = o0 == 0 ? Vm[i][0] : (o0 == 1 ? Vm[i][1] : Vm[i][2]);
        v2[i] = o1 == 0 ? Vm[i][0] : (o1 == 1 ? Vm[i][1] : Vm[i][2]);
        u1[i] = o0 == 0 ? B[i][0] : (o0 == 1 ? B[i][1] : B[i][2]);
        u2[i] = o1 == 0 ? B[i][0] : (o1 == 1 ? B[i][1] : B[i][2]);
    }
    v3[0] = v1[1] * v2[2] - v1[2] * v2[1];
    v3[1] = v1[2] * v2[0] - v1[0] * v2[2];
    v3[2] = v1[0] * v2[1] - v1[1] * v2[0];
    const T n1 = tsqrt(u1[0] * u1[0] + u1[1] * u1[1] + u1[2] * u1[2]);
#pragma unroll
    for (int i = 0; i < 3; ++i) u1[i] /= n1;
    const T dp = u1[0] * u2[0] + u1[1] * u2[1] + u1[2] * u2[2];
#pragma unroll
    for (int i = 0; i < 3; ++i) u2[i] -= dp * u1[i];
    T n2 = tsqrt(u2[0] * u2[0] + u2[1] * u2[1] + u2[2] * u2[2]);
    if (!(n2 > (T)64 * Eps<T>::v * n1)) {
        // rank one: any unit vector orthogonal to u1
        const T a0 = fabs(u1[0]), a1 = fabs(u1[1]), a2 = fabs(u1[2]);
        const int mi = (a1 < a0) ? ((a2 < a1) ? 2 : 1) : ((a2 < a0) ? 2 : 0);
        const T d2 = mi == 0 ? u1[0] : (mi == 1 ? u1[1] : u1[2]);
#pragma unroll
        for (int i = 0; i < 3; ++i) u2[i] = (i == mi ? (T)1 : (T)0) - d2 * u1[i];
        n2 = tsqrt(u2[0] * u2[0] + u2[1] * u2[1] + u2[2] * u2[2]);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) u2[i] /= n2;
    u3[0] = u1[1] * u2[2] - u1[2] * u2[1];
    u3[1] = u1[2] * u2[0] - u1[0] * u2[2];
    u3[2] = u1[0] * u2[1] - u1[1] * u2[0];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) R[i][j] = v1[i] * u1[j] + v2[i] * u2[j] + v3[i] * u3[j];
}


// The mixed form's rotation fit runs in FP32. Where the one-ring's covariance
// is close to rank one ((sigma_2 + sigma_3) / sigma_1 below this bound, which
// happens where a large handle move stretches a one-ring in the first
// iterations), the FP32 rounding of the covariance is amplified by about the
// inverse of that ratio, so the fit is redone in FP64 from the FP64 rest and
// current positions: the FP64 arithmetic goes only where the stability needs
// it (a fraction of a percent of the vertices).
constexpr float kPolarFallback = 0.1f;

// FP64 covariance of vertex i's one-ring (estimateRotations, arap.h:358-374)
// and its rotation, from the rest positions p, current positions pc (element
// k of vertex k's pose at k * stride + off) and the FP64 weights.
__device__ __forceinline__ void rotation_fp64(int i, int e0, int e1, const int32_t *__restrict__ dcol,
                                              const double *__restrict__ w64, const Vec4<double> *__restrict__ p,
                                              const Vec4<double> *__restrict__ pc, int64_t stride, int64_t off,
                                              float Rm[3][3]) {
    const Vec4<double> pi = p[i], ci = pc[(int64_t)i * stride + off];
    double S[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int e = e0; e < e1; ++e) {
        const int j = dcol[e];
        const double wj = w64[e];
        const Vec4<double> pj = p[j], cj = pc[(int64_t)j * stride + off];
        const double ex = wj * (pi.x - pj.x), ey = wj * (pi.y - pj.y), ez = wj * (pi.z - pj.z);
        const double fx = ci.x - cj.x, fy = ci.y - cj.y, fz = ci.z - cj.z;
        S[0][0] += ex * fx; S[0][1] += ex * fy; S[0][2] += ex * fz;
        S[1][0] += ey * fx; S[1][1] += ey * fy; S[1][2] += ey * fz;
        S[2][0] += ez * fx; S[2][1] += ez * fy; S[2][2] += ez * fz;
    }
    double R[3][3];
    rotation_from_cov<double>(S, R);
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) Rm[a][b] = (float)R[a][b];
}

}  // namespace dev
}  // namespace arapgpu

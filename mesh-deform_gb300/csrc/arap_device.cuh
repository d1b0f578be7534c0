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

// Newton steps towards the rotation R of rotation_from_cov (the maximiser of
// tr(R S) over proper rotations, so V diag(1,1,det) U^T for S = U Sigma V^T)
// from a nearby R. With R = R0 exp([w]x) the objective's gradient at w = 0
// is g, the axial vector of the skew part of Q = (S R0)^T, and its Hessian
// -(tr(Q) I - sym(Q)); the step w = (tr(Q) I - sym(Q))^-1 g is applied
// through the Cayley map, which keeps R orthogonal. Quadratic convergence:
// from an FP32 fit (error e), one step leaves about e^2, two reach FP64
// accuracy.
template <typename T>
__device__ __forceinline__ void polar_newton(const T S[3][3], T R[3][3], int ns_iters, int iters) {
    // R orthogonal to working precision first (the Cayley steps keep R's
    // deviation from orthogonality): Newton-Schulz, R <- R (3 I - R^T R) / 2,
    // which squares the deviation (1e-7 of an FP32 fit -> 1e-14 -> 1e-28)
    for (int it = 0; it < ns_iters; ++it) {
        T G[3][3];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b)
                G[a][b] = (a == b ? (T)1.5 : (T)0) - (T)0.5 * (R[0][a] * R[0][b] + R[1][a] * R[1][b] + R[2][a] * R[2][b]);
        T Rn[3][3];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) Rn[a][b] = R[a][0] * G[0][b] + R[a][1] * G[1][b] + R[a][2] * G[2][b];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) R[a][b] = Rn[a][b];
    }
    for (int it = 0; it < iters; ++it) {
        T Q[3][3];  // Q = (S R)^T: Q[a][b] = sum_k S[b][k] R[k][a]
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) Q[a][b] = S[b][0] * R[0][a] + S[b][1] * R[1][a] + S[b][2] * R[2][a];
        const T g0 = Q[2][1] - Q[1][2], g1 = Q[0][2] - Q[2][0], g2 = Q[1][0] - Q[0][1];
        const T tr = Q[0][0] + Q[1][1] + Q[2][2];
        // H = tr I - sym(Q), symmetric
        const T h00 = tr - Q[0][0], h11 = tr - Q[1][1], h22 = tr - Q[2][2];
        const T h01 = -(T)0.5 * (Q[0][1] + Q[1][0]), h02 = -(T)0.5 * (Q[0][2] + Q[2][0]),
                h12 = -(T)0.5 * (Q[1][2] + Q[2][1]);
        // w = adj(H) g / det(H)
        const T c00 = h11 * h22 - h12 * h12, c01 = h02 * h12 - h01 * h22, c02 = h01 * h12 - h02 * h11;
        const T c11 = h00 * h22 - h02 * h02, c12 = h01 * h02 - h00 * h12, c22 = h00 * h11 - h01 * h01;
        const T det = h00 * c00 + h01 * c01 + h02 * c02;
        const T scale = fabs(h00) + fabs(h11) + fabs(h22);
        if (!(det > Eps<T>::v * scale * scale * scale)) break;  // not a maximum's neighbourhood: keep R
        const T id = (T)1 / det;
        const T w0 = (c00 * g0 + c01 * g1 + c02 * g2) * id, w1 = (c01 * g0 + c11 * g1 + c12 * g2) * id,
                w2 = (c02 * g0 + c12 * g1 + c22 * g2) * id;
        // Cayley: C = I + 2/(1+|a|^2) ([a]x + [a]x^2), a = w/2
        const T a0 = (T)0.5 * w0, a1 = (T)0.5 * w1, a2 = (T)0.5 * w2;
        const T f = (T)2 / ((T)1 + a0 * a0 + a1 * a1 + a2 * a2);
        const T C[3][3] = {{(T)1 - f * (a1 * a1 + a2 * a2), f * (a0 * a1 - a2), f * (a0 * a2 + a1)},
                           {f * (a0 * a1 + a2), (T)1 - f * (a0 * a0 + a2 * a2), f * (a1 * a2 - a0)},
                           {f * (a0 * a2 - a1), f * (a1 * a2 + a0), (T)1 - f * (a0 * a0 + a1 * a1)}};
        T Rn[3][3];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) Rn[a][b] = R[a][0] * C[0][b] + R[a][1] * C[1][b] + R[a][2] * C[2][b];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) R[a][b] = Rn[a][b];
    }
}

// FP64 covariance of vertex i's one-ring (estimateRotations, arap.h:358-374)
// and its rotation refined from the FP32 fit Rm (in place), from the rest
// positions p, current positions pc (element k of vertex k's pose at
// k * stride + off) and the FP64 weights.
// NEWTON: the refinement below; else the FP64 one-sided Jacobi fit of the
// FP64 covariance (measured faster in the batched local step, where the 32
// lanes of a warp are 32 poses of one vertex, slower for one request).
template <bool NEWTON>
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
    // Newton's method on the rotation group from the FP32 fit, which is close
    // (a few 1e-6 at worst): one orthonormalisation and one Newton step leave
    // an error of about 1e-12, far below what the mixed form's FP32 rotations
    // carry anyway, for ~300 FP64 instructions (the scarce kind on this GPU).
    double R[3][3];
    if constexpr (NEWTON) {
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) R[a][b] = (double)Rm[a][b];
        polar_newton(S, R, 1, 1);
    } else {
        rotation_from_cov<double>(S, R);
    }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) Rm[a][b] = (float)R[a][b];
}

// FP64 rotation fit of the FP64 form: the FP32 fit of the covariance
// (scaled to unit Frobenius norm before rounding), orthonormalised (one
// Newton-Schulz step: 1e-7 -> 1e-14) and refined to FP64 accuracy by two
// Newton steps on the rotation group (polar_newton); near rank-one
// covariances, where the FP32 fit is a poor
// seed, take the FP64 one-sided Jacobi fit. About a quarter of the FP64
// instructions of the FP64 Jacobi fit, the same rotation to FP64 accuracy.
__device__ __forceinline__ void rotation_fit_fp64(const double S[3][3], double R[3][3]) {
    double f2 = 0.0;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) f2 += S[a][b] * S[a][b];
    if (f2 > 0.0 && f2 < 1e300) {
        const double sc = 1.0 / sqrt(f2);
        float Sf[3][3], Rf[3][3], spread;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) Sf[a][b] = (float)(S[a][b] * sc);
        rotation_from_cov<float>(Sf, Rf, &spread);
        if (spread >= kPolarFallback) {
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int b = 0; b < 3; ++b) R[a][b] = (double)Rf[a][b];
            polar_newton(S, R, 1, 2);
            return;
        }
    }
    rotation_from_cov<double>(S, R);
}

}  // namespace dev
}  // namespace arapgpu

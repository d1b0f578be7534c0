// arap_device.cuh -- device helpers shared by the single-pose and batched
// kernels: precision traits and the 3x3 rotation fit of the local step
// (inc/deform/arap.h:376-382).
#pragma once

#include <cuda_runtime.h>

namespace arapgpu {
namespace dev {

template <typename T> __device__ __forceinline__ T tsqrt(T x);
template <> __device__ __forceinline__ float tsqrt(float x) { return sqrtf(x); }
template <> __device__ __forceinline__ double tsqrt(double x) { return sqrt(x); }

template <typename T> struct Eps;
template <> struct Eps<float> { static constexpr float v = 1.1920929e-07f; };
template <> struct Eps<double> { static constexpr double v = 2.220446049250313e-16; };

// Classical cyclic Jacobi on a symmetric 3x3 (Golub & Van Loan, Alg. 8.5.3):
// a -> diag(lambda), v = eigenvectors (columns).
template <typename T>
__device__ __forceinline__ void jacobi_eig3(T a[3][3], T v[3][3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) v[i][j] = (i == j) ? (T)1 : (T)0;
    const int sweeps = sizeof(T) == 4 ? 6 : 10;
    for (int sw = 0; sw < sweeps; ++sw) {
        const T off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
        const T dia = a[0][0] * a[0][0] + a[1][1] * a[1][1] + a[2][2] * a[2][2];
        if (off <= Eps<T>::v * Eps<T>::v * dia) break;
#pragma unroll
        for (int pq = 0; pq < 3; ++pq) {
            const int p = pq == 2 ? 1 : 0;
            const int q = pq == 0 ? 1 : 2;
            const int r = 3 - p - q;
            const T apq = a[p][q];
            if (apq == (T)0) continue;
            const T theta = (a[q][q] - a[p][p]) / ((T)2 * apq);
            T t = (T)1 / (fabs(theta) + tsqrt(theta * theta + (T)1));
            if (theta < (T)0) t = -t;
            const T c = (T)1 / tsqrt(t * t + (T)1);
            const T s = t * c;
            const T tau = s / ((T)1 + c);
            a[p][p] -= t * apq;
            a[q][q] += t * apq;
            a[p][q] = a[q][p] = (T)0;
            const T arp = a[r][p], arq = a[r][q];
            a[r][p] = a[p][r] = arp - s * (arq + tau * arp);
            a[r][q] = a[q][r] = arq + s * (arp - tau * arq);
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const T vip = v[i][p], viq = v[i][q];
                v[i][p] = vip - s * (viq + tau * vip);
                v[i][q] = viq + s * (vip - tau * viq);
            }
        }
    }
}

// Best rotation R = V diag(1,1,det(V U^T)) U^T for cov = U S V^T (arap.h:376-382),
// from the eigenvectors V of cov^T cov (proper, v3 = v1 x v2) and the proper
// left factor u1 = cov v1/|.|, u2 = Gram-Schmidt(cov v2), u3 = u1 x u2.
template <typename T>
__device__ __forceinline__ void rotation_from_cov(const T S_in[3][3], T R[3][3]) {
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
    T S[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) S[i][j] = S_in[i][j] * sc;
    T C[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) C[i][j] = S[0][i] * S[0][j] + S[1][i] * S[1][j] + S[2][i] * S[2][j];
    T Vm[3][3];
    jacobi_eig3(C, Vm);
    // order eigenpairs descending
    T lam[3] = {C[0][0], C[1][1], C[2][2]};
    int o0 = 0, o1 = 1, o2 = 2;
    if (lam[o1] > lam[o0]) { int t = o0; o0 = o1; o1 = t; }
    if (lam[o2] > lam[o0]) { int t = o0; o0 = o2; o2 = t; }
    if (lam[o2] > lam[o1]) { int t = o1; o1 = o2; o2 = t; }
    T v1[3], v2[3], v3[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) { v1[i] = Vm[i][o0]; v2[i] = Vm[i][o1]; }
    v3[0] = v1[1] * v2[2] - v1[2] * v2[1];
    v3[1] = v1[2] * v2[0] - v1[0] * v2[2];
    v3[2] = v1[0] * v2[1] - v1[1] * v2[0];
    T u1[3], u2[3], u3[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        u1[i] = S[i][0] * v1[0] + S[i][1] * v1[1] + S[i][2] * v1[2];
        u2[i] = S[i][0] * v2[0] + S[i][1] * v2[1] + S[i][2] * v2[2];
    }
    const T n1 = tsqrt(u1[0] * u1[0] + u1[1] * u1[1] + u1[2] * u1[2]);
#pragma unroll
    for (int i = 0; i < 3; ++i) u1[i] /= n1;
    const T dp = u1[0] * u2[0] + u1[1] * u2[1] + u1[2] * u2[2];
#pragma unroll
    for (int i = 0; i < 3; ++i) u2[i] -= dp * u1[i];
    T n2 = tsqrt(u2[0] * u2[0] + u2[1] * u2[1] + u2[2] * u2[2]);
    if (!(n2 > (T)64 * Eps<T>::v * n1)) {
        // rank one: any unit vector orthogonal to u1
        int mi = 0;
        if (fabs(u1[1]) < fabs(u1[mi])) mi = 1;
        if (fabs(u1[2]) < fabs(u1[mi])) mi = 2;
        T e[3] = {(T)0, (T)0, (T)0};
        e[mi] = (T)1;
        const T d2 = u1[mi];
#pragma unroll
        for (int i = 0; i < 3; ++i) u2[i] = e[i] - d2 * u1[i];
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


}  // namespace dev
}  // namespace arapgpu

// arap_kernels.cu -- sm_103a kernels of the ARAP hot path.
//
// Reference: cheind/mesh-deform inc/deform/arap.h. Each kernel names the lines
// it replaces. Layouts are described in arap_kernels.h.
#include "arap_kernels.h"
#include "arap_device.cuh"

#include <cooperative_groups.h>

#include <algorithm>
#include <cstdio>
#include <map>
#include <mutex>

namespace arapgpu {

namespace {

using dev::tsqrt;
using dev::Eps;
using dev::rotation_from_cov;

constexpr int NB = kDiagBlock;  // diagonal block width (32)

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Arrival count: old value of *p, incremented with acquire-release semantics
// at device scope (the caller's CTA barrier orders its threads' writes before
// it, cumulatively; the CTA that reads the final count sees every writer's).
__device__ __forceinline__ unsigned atom_add_acq_rel(unsigned *p, unsigned v) {
    unsigned old;
    asm volatile("atom.add.acq_rel.gpu.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ void st_release(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Bounded wait until *p >= target; on expiry records kErrTimeout and returns.
__device__ __forceinline__ void wait_flag(const unsigned *p, unsigned target, int *err) {
    const unsigned lim = flag_wait_limit(err);
    for (unsigned it = 0;; ++it) {
        if (ld_acquire(p) >= target) return;
        if (it >= lim) break;
        __nanosleep(it < 64 ? 20 : 200);
    }
    atomicOr(err, kErrTimeout);
}

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialization may start once every CTA of the kernel before it has called
// pdl_trigger (or exited); pdl_wait then blocks until that kernel has
// finished and its memory is visible. Without the launch attribute pdl_wait
// returns at once.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename T> __device__ __forceinline__ Vec4<T> ldcg4(const Vec4<T> *p);
template <> __device__ __forceinline__ Vec4<float> ldcg4(const Vec4<float> *p) {
    float4 v = __ldcg(reinterpret_cast<const float4 *>(p));
    return {v.x, v.y, v.z, v.w};
}
template <> __device__ __forceinline__ Vec4<double> ldcg4(const Vec4<double> *p) {
    const double2 *q = reinterpret_cast<const double2 *>(p);
    double2 a = __ldcg(q), b = __ldcg(q + 1);
    return {a.x, a.y, b.x, b.y};
}

// ---------------------------------------------------------------------------
// cotan weights

// computeCotanWeights, arap.h:189-222, per face: the three clamped cotangents
// times 1/2, rounded exactly as the FP64 CPU code (no fused multiply-adds).
__global__ void k_face_cots(int F, const int32_t *__restrict__ faces, const double *__restrict__ xyz,
                            double *__restrict__ hc) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= F) return;
    const int i0 = faces[3 * f], i1 = faces[3 * f + 1], i2 = faces[3 * f + 2];
    const double *v0 = xyz + 3 * (int64_t)i0, *v1 = xyz + 3 * (int64_t)i1, *v2 = xyz + 3 * (int64_t)i2;
    double l0 = 0.0, l1 = 0.0, l2 = 0.0, d;
#pragma unroll
    for (int c = 0; c < 3; ++c) { d = __dsub_rn(v1[c], v0[c]); l0 = __dadd_rn(l0, __dmul_rn(d, d)); }
#pragma unroll
    for (int c = 0; c < 3; ++c) { d = __dsub_rn(v2[c], v1[c]); l1 = __dadd_rn(l1, __dmul_rn(d, d)); }
#pragma unroll
    for (int c = 0; c < 3; ++c) { d = __dsub_rn(v0[c], v2[c]); l2 = __dadd_rn(l2, __dmul_rn(d, d)); }
    // std::max<Scalar>(1e-8, x) = (1e-8 < x) ? x : 1e-8
    l0 = (1e-8 < l0) ? l0 : 1e-8;
    l1 = (1e-8 < l1) ? l1 : 1e-8;
    l2 = (1e-8 < l2) ? l2 : 1e-8;
    l0 = __dsqrt_rn(l0);
    l1 = __dsqrt_rn(l1);
    l2 = __dsqrt_rn(l2);
    const double semip = __dmul_rn(0.5, __dadd_rn(__dadd_rn(l0, l1), l2));
    double h = __dmul_rn(__dmul_rn(__dmul_rn(semip, __dsub_rn(semip, l0)), __dsub_rn(semip, l1)),
                         __dsub_rn(semip, l2));
    double area = __dsqrt_rn(h);
    area = (1e-8 < area) ? area : 1e-8;  // NaN from a negative product also gives 1e-8
    const double denom = __ddiv_rn(1.0, __dmul_rn(4.0, area));
    const double s0 = __dmul_rn(l0, l0), s1 = __dmul_rn(l1, l1), s2 = __dmul_rn(l2, l2);
    double c0 = __dmul_rn(__dadd_rn(__dadd_rn(-s0, s1), s2), denom);
    double c1 = __dmul_rn(__dadd_rn(__dsub_rn(s0, s1), s2), denom);
    double c2 = __dmul_rn(__dsub_rn(__dadd_rn(s0, s1), s2), denom);
    c0 = (1e-10 < c0) ? c0 : 1e-10;
    c1 = (1e-10 < c1) ? c1 : 1e-10;
    c2 = (1e-10 < c2) ? c2 : 1e-10;
    hc[3 * (int64_t)f + 0] = __dmul_rn(c0, 0.5);
    hc[3 * (int64_t)f + 1] = __dmul_rn(c1, 0.5);
    hc[3 * (int64_t)f + 2] = __dmul_rn(c2, 0.5);
}

// setFromTriplets (arap.h:238): contributions of an edge summed in face order.
__device__ __forceinline__ double edge_weight(const int32_t *ent_ptr, const int32_t *ent_fc, const double *hc,
                                              int e) {
    const int b = ent_ptr[e], t = ent_ptr[e + 1];
    double w = hc[ent_fc[b]];
    for (int q = b + 1; q < t; ++q) w = __dadd_rn(w, hc[ent_fc[q]]);
    return w;
}

__global__ void k_edge_weights(int nnz, const int32_t *__restrict__ dent, const int32_t *__restrict__ ent_ptr,
                               const int32_t *__restrict__ ent_fc, const double *__restrict__ hc,
                               double *__restrict__ w64, float *__restrict__ w32, double *__restrict__ w_orig) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nnz) return;
    const int o = dent[e];
    const double w = edge_weight(ent_ptr, ent_fc, hc, o);
    if (w64) w64[e] = w;
    if (w32) w32[e] = (float)w;
    if (w_orig) w_orig[o] = w;
}

__global__ void k_edge_weights_orig(int nnz, const int32_t *__restrict__ ent_ptr, const int32_t *__restrict__ ent_fc,
                                    const double *__restrict__ hc, double *__restrict__ w_orig) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nnz) return;
    w_orig[e] = edge_weight(ent_ptr, ent_fc, hc, e);
}

// ---------------------------------------------------------------------------
// per-vertex setup

template <typename T>
__global__ void k_setup_vertices(int V, int m, const int32_t *__restrict__ oldidx, const double *__restrict__ rest,
                                 const double *__restrict__ targets, Vec4<double> *p64, Vec4<double> *pc64,
                                 Vec4<T> *p_t, Vec4<T> *pc_t, Vec4<T> *R) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= V) return;
    const int v = oldidx[k];
    const Vec4<double> pr = {rest[3 * (int64_t)v], rest[3 * (int64_t)v + 1], rest[3 * (int64_t)v + 2], 0.0};
    Vec4<double> pc = pr;
    if (k >= m) {  // constrained vertex: snapped to its target (arap.h:277-281)
        const double *t = targets + 3 * (int64_t)(k - m);
        pc = {t[0], t[1], t[2], 0.0};
    }
    p64[k] = pr;
    pc64[k] = pc;
    p_t[k] = {(T)pr.x, (T)pr.y, (T)pr.z, (T)0};
    pc_t[k] = {(T)pc.x, (T)pc.y, (T)pc.z, (T)0};
    R[3 * (int64_t)k + 0] = {(T)1, (T)0, (T)0, (T)0};
    R[3 * (int64_t)k + 1] = {(T)0, (T)1, (T)0, (T)0};
    R[3 * (int64_t)k + 2] = {(T)0, (T)0, (T)1, (T)0};
}

// setupLinearSystem, arap.h:310-336: L_kk = sum_j w_kj, L_lk = -w_kl for free
// l > k (written into the supernodal panel of column k), bFixed_k = sum over
// constrained neighbours of w_kj * c_j, all summed in adjacency order.
template <typename TF>
__global__ void k_assemble(int m, const int32_t *__restrict__ drow, const int32_t *__restrict__ dcol,
                           const double *__restrict__ w64, const int64_t *__restrict__ amap,
                           const int64_t *__restrict__ dmap, const Vec4<double> *__restrict__ pc64,
                           TF *__restrict__ Lval, double *__restrict__ diag64, Vec4<double> *__restrict__ bfixed) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    double diag = 0.0, bx = 0.0, by = 0.0, bz = 0.0;
    for (int e = drow[k]; e < drow[k + 1]; ++e) {
        const int l = dcol[e];
        if (l == k) continue;
        const double w = w64[e];
        diag = __dadd_rn(diag, w);
        if (l >= m) {
            const Vec4<double> c = pc64[l];
            bx = __dadd_rn(bx, __dmul_rn(w, c.x));
            by = __dadd_rn(by, __dmul_rn(w, c.y));
            bz = __dadd_rn(bz, __dmul_rn(w, c.z));
        } else if (l > k) {
            Lval[amap[e]] = (TF)(-w);
        }
    }
    Lval[dmap[k]] = (TF)diag;
    diag64[k] = diag;
    bfixed[k] = {bx, by, bz, 0.0};
}

// bFixed alone (arap.h:325-327), for a re-pose that keeps the factor
__global__ void k_bfixed(int m, const int32_t *__restrict__ drow, const int32_t *__restrict__ dcol,
                         const double *__restrict__ w64, const Vec4<double> *__restrict__ pc64,
                         Vec4<double> *__restrict__ bfixed) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    double bx = 0.0, by = 0.0, bz = 0.0;
    for (int e = drow[k]; e < drow[k + 1]; ++e) {
        const int l = dcol[e];
        if (l < m) continue;
        const double w = w64[e];
        const Vec4<double> c = pc64[l];
        bx = __dadd_rn(bx, __dmul_rn(w, c.x));
        by = __dadd_rn(by, __dmul_rn(w, c.y));
        bz = __dadd_rn(bz, __dmul_rn(w, c.z));
    }
    bfixed[k] = {bx, by, bz, 0.0};
}

// Rest edge vectors p_k - p_l per adjacency entry, differenced in FP64 and
// stored in FP32: exact to FP32 rounding of the (short) edge itself, where
// differencing FP32 positions would lose the digits the positions' magnitude
// takes.
__global__ void k_rest_edges(int V, const int32_t *__restrict__ drow, const int32_t *__restrict__ dcol,
                             const Vec4<double> *__restrict__ p64, Vec4<float> *__restrict__ redge) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= V) return;
    const Vec4<double> pk = p64[k];
    for (int e = drow[k]; e < drow[k + 1]; ++e) {
        const Vec4<double> pl = p64[dcol[e]];
        redge[e] = {(float)(pk.x - pl.x), (float)(pk.y - pl.y), (float)(pk.z - pl.z), 0.f};
    }
}

// ---------------------------------------------------------------------------
// multifrontal Cholesky, level by level, many CTAs per front

constexpr int kFactorThreads = 256;
// Tile shapes of the factorisation plan (arap_symbolic.cpp builds the items
// with the same sizes): rows of a block-column update tile, rows of a tile of
// the solve below a diagonal block, and the square tiles of the Schur
// complement. Small tiles spread a front's work over many CTAs, which the
// FP64 factor needs: a GB300 SM issues about two FP64 FMAs per clock.
constexpr int kUpdRows = kFactorUpdRows;
constexpr int kRowsTile = kFactorRowsTile;
constexpr int kSyrkTile = kFactorSyrkTile;
static_assert(kUpdRows == 32 && kRowsTile == 64 && kSyrkTile == 32, "thread mappings below assume these sizes");

// Front of supernode d: the nrow x ncol panel P (column-major, ld nrow; rows are
// the supernode's columns then its struct rows) and the nb x nb update matrix U.
// Element (row i, column k) of the front, k <= i.
template <typename TF>
__device__ __forceinline__ TF &front(TF *P, TF *U, int n, int nc, int nb, int i, int k) {
    return k < nc ? P[(int64_t)k * n + i] : U[(int64_t)(k - nc) * nb + (i - nc)];
}

// Extend-add: the parent columns [a, b) of a front receive the matching
// columns of every child's update matrix, children in order. Parent columns
// are split between CTAs, so no two CTAs touch the same entry.
template <typename TF>
__global__ void __launch_bounds__(kFactorThreads)
k_fea(const FItem *__restrict__ items, const SnInfo *__restrict__ sn, const int32_t *__restrict__ child,
      const int32_t *__restrict__ relind, TF *__restrict__ Lval, TF *__restrict__ Upd) {
    __shared__ int s_k0, s_k1;
    const FItem it = items[blockIdx.x];
    const SnInfo d = sn[it.sn];
    const int n = d.nrow, nc = d.ncol, nb = n - nc;
    TF *P = Lval + d.panel_off;
    TF *U = Upd + d.upd_off;
    const int tid = threadIdx.x;
    for (int ci = d.child_begin; ci < d.child_end; ++ci) {
        const SnInfo c = sn[child[ci]];
        const int nbc = c.nrow - c.ncol;
        const int32_t *ri = relind + c.relind_off;
        // child columns whose parent column lies in [a, b): ri increases, so
        // they are [k0, k1) with k0 = #{ri < a}, k1 = #{ri < b}, counted by all threads
        if (tid == 0) s_k0 = s_k1 = 0;
        __syncthreads();
        int n0 = 0, n1 = 0;
        for (int m = tid; m < nbc; m += kFactorThreads) {
            const int v = ri[m];
            n0 += v < it.a;
            n1 += v < it.b;
        }
        if (n0) atomicAdd(&s_k0, n0);
        if (n1) atomicAdd(&s_k1, n1);
        __syncthreads();
        const int k0 = s_k0, k1 = s_k1;
        const TF *Uc = Upd + c.upd_off;
        // every (column k, row i >= k) pair of the slice in one sweep: distinct
        // targets within one child, so no two threads meet. A thread takes
        // kEa pairs at a time and issues all their loads (child entries, row
        // maps, front entries) before its stores, so the round trips of a
        // batch overlap instead of queueing behind each other's stores.
        constexpr int kEa = 8;
        const int64_t cnt = (int64_t)(k1 - k0) * nbc;
        for (int64_t q0 = tid; q0 < cnt; q0 += (int64_t)kEa * kFactorThreads) {
            TF val[kEa];
            TF *dst[kEa];
#pragma unroll
            for (int u = 0; u < kEa; ++u) {
                const int64_t q = q0 + (int64_t)u * kFactorThreads;
                dst[u] = nullptr;
                if (q < cnt) {
                    const int k = k0 + (int)(q / nbc), i = (int)(q % nbc);
                    if (i >= k) {
                        val[u] = Uc[(int64_t)k * nbc + i];
                        dst[u] = &front(P, U, n, nc, nb, ri[i], ri[k]);
                    }
                }
            }
            TF cur[kEa];
#pragma unroll
            for (int u = 0; u < kEa; ++u)
                if (dst[u]) cur[u] = *dst[u];
#pragma unroll
            for (int u = 0; u < kEa; ++u)
                if (dst[u]) *dst[u] = cur[u] + val[u];
        }
        __syncthreads();
    }
}

// The entries of a factor tile of vr rows x vc columns that are needed
// (tri: only rows r >= c, the tile on the diagonal), column by column, dealt
// to the CTA's threads in turn: at most four per thread, all lanes of a warp
// busy but in the last one. Factor kernels built on it issue no FP64
// instruction for padding or for the upper triangle (GB300 issues about two
// FP64 FMAs per clock per SM, so every wasted lane costs).
// acc[q] += sum_t A(t, er[q]) B(t, ec[q]) over t < kw for the thread's ne
// entries (A, B row-major in shared memory, rows t). One branch per count,
// so a warp whose lanes all hold fewer entries issues fewer FP64
// instructions (predicated-off instructions still take issue slots).
template <int NE, typename TF>
__device__ __forceinline__ void tile_fma_n(int kw, const TF *A, int lda, const TF *B, int ldb, const int er[4],
                                           const int ec[4], TF acc[4]) {
    for (int t = 0; t < kw; ++t)
#pragma unroll
        for (int q = 0; q < NE; ++q) acc[q] += A[t * lda + er[q]] * B[t * ldb + ec[q]];
}
template <typename TF>
__device__ __forceinline__ void tile_fma(int ne, int kw, const TF *A, int lda, const TF *B, int ldb, const int er[4],
                                         const int ec[4], TF acc[4]) {
    switch (ne) {
    case 4: tile_fma_n<4>(kw, A, lda, B, ldb, er, ec, acc); break;
    case 3: tile_fma_n<3>(kw, A, lda, B, ldb, er, ec, acc); break;
    case 2: tile_fma_n<2>(kw, A, lda, B, ldb, er, ec, acc); break;
    case 1: tile_fma_n<1>(kw, A, lda, B, ldb, er, ec, acc); break;
    default: break;
    }
}

__device__ __forceinline__ int tile_entries(int vr, int vc, bool tri, int er[4], int ec[4]) {
    int ne = 0;
    if (vr <= 0 || vc <= 0) return 0;
    if (!tri) {
        const int tot = vr * vc;
        for (int e = threadIdx.x; e < tot && ne < 4; e += blockDim.x) {
            er[ne] = e % vr;
            ec[ne] = e / vr;
            ++ne;
        }
    } else {
        int tot = 0;
        for (int c = 0; c < vc; ++c) tot += max(vr - c, 0);
        for (int e = threadIdx.x; e < tot && ne < 4; e += blockDim.x) {
            // column c holds rows c..vr-1 (vr - c entries)
            int c = 0, base = 0;
            while (e >= base + (vr - c)) {
                base += vr - c;
                ++c;
            }
            er[ne] = c + (e - base);
            ec[ne] = c;
            ++ne;
        }
    }
    return ne;
}

// Left-looking update of block column jb: rows [j0 + 32 rt, +32) of columns
// [j0, j0+w) lose sum_{k < j0} P(r, k) P(j0+c, k).
template <typename TF>
__global__ void __launch_bounds__(kFactorThreads)
k_fupd(const FItem *__restrict__ items, int jb, const SnInfo *__restrict__ sn, TF *__restrict__ Lval) {
    __shared__ TF As[NB][kUpdRows];
    __shared__ TF Bs[NB][NB + 1];
    const FItem it = items[blockIdx.x];
    const SnInfo d = sn[it.sn];
    const int n = d.nrow, nc = d.ncol;
    const int j0 = jb * NB, w = min(NB, nc - j0);
    const int r0 = j0 + it.a * kUpdRows;
    TF *P = Lval + d.panel_off;
    const int tid = threadIdx.x;
    // the tile's entries: rows r0.. (at most kUpdRows, inside the front),
    // columns of the block; the first row tile is the diagonal block, of
    // which the lower triangle is needed
    int er[4], ec[4];
    const int ne = tile_entries(min(kUpdRows, n - r0), w, it.a == 0, er, ec);
    TF acc[4] = {0, 0, 0, 0};
    // the next k-slice is loaded into registers while the current one is
    // multiplied, so its global round trip overlaps the products
    constexpr int kPa = NB * kUpdRows / kFactorThreads, kPb = NB * NB / kFactorThreads;
    TF pa[kPa], pb[kPb];
    auto load_slice = [&](int k0) {
#pragma unroll
        for (int u = 0; u < kPa; ++u) {
            const int q = tid + u * kFactorThreads, t = q / kUpdRows, r = q % kUpdRows;
            pa[u] = (r0 + r < n) ? P[(int64_t)(k0 + t) * n + r0 + r] : (TF)0;
        }
#pragma unroll
        for (int u = 0; u < kPb; ++u) {
            const int q = tid + u * kFactorThreads, t = q / NB, c = q % NB;
            pb[u] = (c < w) ? P[(int64_t)(k0 + t) * n + j0 + c] : (TF)0;
        }
    };
    if (j0 > 0) load_slice(0);
    for (int k0 = 0; k0 < j0; k0 += NB) {
#pragma unroll
        for (int u = 0; u < kPa; ++u) {
            const int q = tid + u * kFactorThreads;
            As[q / kUpdRows][q % kUpdRows] = pa[u];
        }
#pragma unroll
        for (int u = 0; u < kPb; ++u) {
            const int q = tid + u * kFactorThreads;
            Bs[q / NB][q % NB] = pb[u];
        }
        __syncthreads();
        if (k0 + NB < j0) load_slice(k0 + NB);
        tile_fma(ne, NB, &As[0][0], kUpdRows, &Bs[0][0], NB + 1, er, ec, acc);
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
        if (q < ne) P[(int64_t)(j0 + ec[q]) * n + r0 + er[q]] -= acc[q];
}

// 1/sqrt(a) for the pivots: an FP32 seed refined by two Newton steps in the
// working precision (a double's 53 bits from the seed's 22), which on GB300
// costs far fewer FP64 instructions than a correctly rounded sqrt and a
// division. Pivots outside the FP32 range take the plain route.
template <typename TF> __device__ __forceinline__ TF pivot_rsqrt(TF a);
template <> __device__ __forceinline__ float pivot_rsqrt(float a) { return rsqrtf(a); }
template <> __device__ __forceinline__ double pivot_rsqrt(double a) {
    if (!(a > 1e-30 && a < 1e30)) return 1.0 / sqrt(a);
    double r = (double)rsqrtf((float)a);
    r = r * (1.5 - 0.5 * a * r * r);
    r = r * (1.5 - 0.5 * a * r * r);
    return r;
}

constexpr int kFdtThreads = 128;
constexpr int kTri = NB * (NB + 1) / 2;  // entries of a block's lower triangle

// Diagonal block jb of a front: its Cholesky factor and that factor's inverse
// (written to Dinv for k_frows, which solves the rows below, and for k_fx).
// Four warps share each step through shared memory, every lane with a useful
// entry, so the FP64 form's arithmetic uses all four schedulers of the SM (a
// GB300 SM issues about two FP64 FMAs per clock; a single warp's FP64 chain
// runs at a quarter of that). Right-looking: step k takes the pivot, scales
// column k and updates the trailing lower triangle, the operations of a
// column-by-column Cholesky in the same order. The trailing entries of step k
// are the first (31-k)(32-k)/2 of a table of the triangle ordered by column,
// last column first. The inverse X = inv(L) is formed row by row: row i is
// -rinv(i) times row i of L times the rows above, with the sum over k split
// in four quarters (one per warp) added in a fixed order.
template <typename TF>
__global__ void __launch_bounds__(kFdtThreads)
k_fdt(const FItem *__restrict__ items, int jb, const SnInfo *__restrict__ sn, TF *__restrict__ Lval,
      TF *__restrict__ Dinv, int *err) {
    __shared__ TF A[NB][NB + 1];   // the block, A[r][c] = L(r, c) once factored
    __shared__ TF X[NB][NB + 1];   // its inverse, X[r][c]
    __shared__ TF part[4][NB];     // quarter sums of the inverse's current row
    __shared__ TF rinv[NB];        // 1 / L(r, r)
    __shared__ uint8_t tri_i[kTri], tri_j[kTri];
    __shared__ int s_bad;
    const SnInfo d = sn[items[blockIdx.x].sn];
    const int n = d.nrow, nc = d.ncol;
    const int j0 = jb * NB, w = min(NB, nc - j0);
    TF *P = Lval + d.panel_off;
    const int tid = threadIdx.x;
    if (tid == 0) s_bad = 0;
    for (int q = tid; q < NB * NB; q += kFdtThreads) {
        const int r = q % NB, c = q / NB;
        A[r][c] = (r < w && c <= r) ? P[(int64_t)(j0 + c) * n + j0 + r] : (TF)0;
        X[r][c] = (TF)0;
    }
    // triangle table of the block's w columns: column jj from w-1 down to 0,
    // rows jj..w-1 (a narrow block issues no FP64 work for absent rows)
    for (int t = tid; t < w * (w + 1) / 2; t += kFdtThreads) {
        int jj = w - 1, base = 0;
        while (t >= base + (w - jj)) {
            base += w - jj;
            --jj;
        }
        tri_j[t] = (uint8_t)jj;
        tri_i[t] = (uint8_t)(jj + (t - base));
    }
    __syncthreads();
    for (int k = 0; k < w; ++k) {
        if (tid == 0) {
            TF a = A[k][k];
            if (!(a > (TF)0)) {
                s_bad = 1;
                a = (TF)1;
            }
            const TF r = pivot_rsqrt(a);
            A[k][k] = a * r;
            rinv[k] = r;
        }
        __syncthreads();
        const TF r = rinv[k];
        for (int i = k + 1 + tid; i < w; i += kFdtThreads) A[i][k] *= r;
        __syncthreads();
        const int T = (w - 1 - k) * (w - k) / 2;  // entries of columns k+1..w-1
        for (int t = tid; t < T; t += kFdtThreads) {
            const int i = tri_i[t], jj = tri_j[t];
            A[i][jj] -= A[i][k] * A[jj][k];
        }
        __syncthreads();
    }
    if (s_bad && tid == 0) atomicOr(err, kErrNotSpd);
    // the factored block back into the panel
    for (int q = tid; q < NB * NB; q += kFdtThreads) {
        const int r = q % NB, c = q / NB;
        if (r < w && c <= r) P[(int64_t)(j0 + c) * n + j0 + r] = A[r][c];
    }
    // X row by row: X(i, c) = -rinv(i) sum_{c <= k < i} L(i, k) X(k, c), X(i, i) = rinv(i)
    const int c = tid & 31, qk = tid >> 5;  // column, quarter of the k range
    for (int i = 0; i < w; ++i) {
        TF acc = (TF)0;
        for (int k = c + ((qk - c) & 3); k < i; k += 4) acc += A[i][k] * X[k][c];  // k >= c, k = qk mod 4
        part[qk][c] = acc;
        __syncthreads();
        if (tid < NB && c <= i) {
            const TF sum = (part[0][c] + part[1][c]) + (part[2][c] + part[3][c]);
            X[i][c] = (c == i) ? rinv[i] : -sum * rinv[i];
        }
        __syncthreads();
    }
    TF *D = Dinv + d.dinv_off + (int64_t)jb * NB * NB;  // column-major: D[c * NB + r] = X(r, c)
    for (int q = tid; q < NB * NB; q += kFdtThreads) D[q] = X[q % NB][q / NB];
}

// The rows below diagonal block jb of a front, 64 rows per CTA, when the plan
// takes them out of k_fdt (fronts with many rows): L(i, j0 + c) =
// sum_k A(i, j0 + k) X(c, k) with X = inv(L_bb) from Dinv, written in place.
// One matrix product per tile, so the rows spread over many CTAs instead of
// one CTA's forward substitution.
template <typename TF>
__global__ void __launch_bounds__(kFactorThreads)
k_frows(const FItem *__restrict__ items, int jb, const SnInfo *__restrict__ sn, TF *__restrict__ Lval,
        const TF *__restrict__ Dinv) {
    __shared__ TF As[NB][kRowsTile];
    __shared__ TF Bs[NB][NB + 1];
    const FItem it = items[blockIdx.x];
    const SnInfo d = sn[it.sn];
    const int n = d.nrow, nc = d.ncol;
    const int j0 = jb * NB, w = min(NB, nc - j0);
    const int r0 = j0 + w + it.a * kRowsTile;
    TF *P = Lval + d.panel_off;
    const TF *D = Dinv + d.dinv_off + (int64_t)jb * NB * NB;  // column-major: D[k * NB + c] = X(c, k)
    // warp wp: columns 4wp..4wp+3; lane: rows lane and lane + 32. X is lower
    // triangular, so column c needs k <= c only: a warp's k range ends at its
    // last column (the same bound for all its lanes), and warps past the
    // block's columns or rows skip their work, which saves FP64 instructions,
    // the scarce kind on this GPU
    const int tid = threadIdx.x, wp = tid >> 5, lane = tid & 31;
    for (int q = tid; q < NB * kRowsTile; q += kFactorThreads) {
        const int t = q / kRowsTile, r = q % kRowsTile;
        As[t][r] = (t < w && r0 + r < n) ? P[(int64_t)(j0 + t) * n + r0 + r] : (TF)0;
    }
    for (int q = tid; q < NB * NB; q += kFactorThreads) Bs[q / NB][q % NB] = D[q];
    __syncthreads();
    const int c0 = 4 * wp;
    if (c0 >= w) return;
    const int kend = min(c0 + 4, w);
    const bool two = r0 + 32 < n;  // rows lane + 32 hold entries for some lane
    TF acc[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}};
    for (int t = 0; t < kend; ++t) {
        const TF a0 = As[t][lane];
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) acc[0][cc] += a0 * Bs[t][c0 + cc];
        if (two) {
            const TF a1 = As[t][lane + 32];
#pragma unroll
            for (int cc = 0; cc < 4; ++cc) acc[1][cc] += a1 * Bs[t][c0 + cc];
        }
    }
#pragma unroll
    for (int rr = 0; rr < 2; ++rr) {
        const int r = r0 + lane + 32 * rr;
        if (r >= n) continue;
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) {
            const int c = c0 + cc;
            if (c < w) P[(int64_t)(j0 + c) * n + r] = acc[rr][cc];
        }
    }
}

// Schur complement of a front: the 32x32 tile (rt, ct), rt >= ct, of U loses
// sum_{k < nc} L21(r, k) L21(c, k); each entry is read and written once.
template <typename TF>
__global__ void __launch_bounds__(kFactorThreads)
k_fsyrk(const FItem *__restrict__ items, const SnInfo *__restrict__ sn, const TF *__restrict__ Lval,
        TF *__restrict__ Upd) {
    __shared__ TF As[NB][kSyrkTile];
    __shared__ TF Bs[NB][kSyrkTile];
    const FItem it = items[blockIdx.x];
    const SnInfo d = sn[it.sn];
    const int n = d.nrow, nc = d.ncol, nb = n - nc;
    const TF *P = Lval + d.panel_off;
    TF *U = Upd + d.upd_off;
    const int rb = it.a * kSyrkTile, cb = it.b * kSyrkTile;  // within U
    const int vr = min(kSyrkTile, nb - rb), vc = min(kSyrkTile, nb - cb);
    const bool diag = rb == cb;
    const int tid = threadIdx.x;
    // only the tile's entries inside U and its lower triangle are computed
    int er[4], ec[4];
    const int ne = tile_entries(vr, vc, diag, er, ec);
    TF acc[4] = {(TF)0, (TF)0, (TF)0, (TF)0};
    // the next k-slice is loaded into registers while the current one is
    // multiplied, so its global round trip overlaps the products
    constexpr int kPer = NB * kSyrkTile / kFactorThreads;
    TF pa[kPer], pb[kPer];
    auto load_slice = [&](int k0) {
        const int kw = min(NB, nc - k0);
#pragma unroll
        for (int u = 0; u < kPer; ++u) {
            const int q = tid + u * kFactorThreads, t = q / kSyrkTile, r = q % kSyrkTile;
            pa[u] = pb[u] = (TF)0;
            if (t < kw) {
                const TF *col = P + (int64_t)(k0 + t) * n + nc;
                if (rb + r < nb) pa[u] = col[rb + r];
                if (cb + r < nb) pb[u] = col[cb + r];
            }
        }
    };
    if (nc > 0) load_slice(0);
    for (int k0 = 0; k0 < nc; k0 += NB) {
        const int kw = min(NB, nc - k0);
#pragma unroll
        for (int u = 0; u < kPer; ++u) {
            const int q = tid + u * kFactorThreads;
            As[q / kSyrkTile][q % kSyrkTile] = pa[u];
            Bs[q / kSyrkTile][q % kSyrkTile] = pb[u];
        }
        __syncthreads();
        if (k0 + NB < nc) load_slice(k0 + NB);
        tile_fma(ne, kw, &As[0][0], kSyrkTile, &Bs[0][0], kSyrkTile, er, ec, acc);
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
        if (q < ne) U[(int64_t)(cb + ec[q]) * nb + rb + er[q]] -= acc[q];
}

// Solve block of a level-1 supernode s and its leaf children (SolveBlocks):
// X_b = inv(L_bb) of the subtree and L21_b = L(rows below s, subtree columns),
// with their transposes, from the supernodes' inverses (k_fx) and panels. With
// leaves l_i (columns at o_i) and s (at o_s), L_bb has the leaves' diagonal
// blocks, s's diagonal block and A_i = L(s columns, l_i columns), so X_b has
// X_{l_i} and X_s on its diagonal, -X_s A_i X_{l_i} below them and zeros
// elsewhere (written too: the sweeps stream whole columns). One CTA per block;
// the products are small (s has a few dozen columns), staged in shared memory
// kBlkRows rows at a time.
constexpr int kBlkCols = 64;  // leaf columns per pass of the products
template <typename TF>
__global__ void __launch_bounds__(kFactorThreads)
k_fx_block(const int32_t *__restrict__ items, const int32_t *__restrict__ members, const SnInfo *__restrict__ sn,
           const SnInfo *__restrict__ bsn, const int32_t *__restrict__ relind, const TF *__restrict__ Lval,
           TF *__restrict__ X, TF *__restrict__ L21, TF *__restrict__ L21T) {
    __shared__ TF Ms[kBlkCols][kBlkCols + 1];  // M = A X_l for up to 64 rows of s x 64 leaf columns
    __shared__ int tmap[kMaxSolveBlock];        // per column of s: the leaf's row below landing there (-1: none)
    const int node = items[3 * blockIdx.x], mb = items[3 * blockIdx.x + 1], me = items[3 * blockIdx.x + 2];
    const SnInfo ns = sn[node], b = bsn[node];
    const int nb = ns.nrow - ns.ncol, nbk = b.ncol, ldb = b.ldx, ld21 = b.ld21;
    const int os = ns.first - b.first;
    TF *Xb = X + b.x_off, *XbT = X + b.xt_off, *Lb = L21 + b.l21_off, *LbT = L21T + b.l21t_off;
    const int tid = threadIdx.x;
    // zeros, then the diagonal blocks and s's rows below
    for (int64_t q = tid; q < (int64_t)ldb * nbk; q += kFactorThreads) Xb[q] = (TF)0;
    for (int64_t q = tid; q < (int64_t)ld21 * nbk; q += kFactorThreads) Lb[q] = (TF)0;
    __syncthreads();
    for (int m = mb; m < me; ++m) {
        const SnInfo d = sn[members[m]];
        const int o = d.first - b.first;
        const TF *Xd = X + d.x_off;
        for (int q = tid; q < d.ncol * d.ncol; q += kFactorThreads) {
            const int r = q % d.ncol, c = q / d.ncol;
            if (r >= c) Xb[(int64_t)(o + c) * ldb + o + r] = Xd[(int64_t)c * d.ldx + r];
        }
    }
    {
        const TF *P = Lval + ns.panel_off;
        for (int q = tid; q < nb * ns.ncol; q += kFactorThreads) {
            const int r = q % nb, c = q / nb;
            Lb[(int64_t)(os + c) * ld21 + r] = P[(int64_t)c * ns.nrow + ns.ncol + r];
        }
    }
    __syncthreads();
    // per leaf: its rows below go to s's columns (A_i) or below s (L21_b)
    const TF *Xs = X + ns.x_off;
    for (int m = mb; m < me - 1; ++m) {
        const SnInfo d = sn[members[m]];
        const int o = d.first - b.first, nbl = d.nrow - d.ncol;
        const TF *P = Lval + d.panel_off;
        const int32_t *ri = relind + d.relind_off;
        for (int q = tid; q < nbl * d.ncol; q += kFactorThreads) {
            const int t = q % nbl, c = q / nbl, pos = ri[t];
            if (pos >= ns.ncol) Lb[(int64_t)(o + c) * ld21 + pos - ns.ncol] = P[(int64_t)c * d.nrow + d.ncol + t];
        }
        for (int k = tid; k < ns.ncol; k += kFactorThreads) tmap[k] = -1;
        __syncthreads();
        for (int t = tid; t < nbl; t += kFactorThreads)
            if (ri[t] < ns.ncol) tmap[ri[t]] = t;
        __syncthreads();
        // X_b(s rows, leaf columns) = -X_s (A_i X_l), in tiles of kBlkCols
        // rows of s x kBlkCols leaf columns
        for (int r0 = 0; r0 < ns.ncol; r0 += kBlkCols)
            for (int c0 = 0; c0 < d.ncol; c0 += kBlkCols) {
                const int rn = min(kBlkCols, ns.ncol - r0), cn = min(kBlkCols, d.ncol - c0);
                // M(r, c) = sum_t A(r0 + r, t) X_l(t, c0 + c), A(k, t) = the leaf's row
                // below that lands on s's column k
                for (int q = tid; q < kBlkCols * kBlkCols; q += kFactorThreads) Ms[q / kBlkCols][q % kBlkCols] = (TF)0;
                __syncthreads();
                for (int q = tid; q < rn * cn; q += kFactorThreads) {
                    const int r = q % rn, c = q / rn, t = tmap[r0 + r];
                    TF acc = (TF)0;
                    if (t >= 0) {
                        // row t of the leaf's rows below, times column c0 + c of X_l (rows k >= c0 + c)
                        const TF *Pt = P + d.ncol + t;
                        for (int k = c0 + c; k < d.ncol; ++k)
                            acc += Pt[(int64_t)k * d.nrow] * X[d.x_off + (int64_t)(c0 + c) * d.ldx + k];
                    }
                    Ms[r][c] = acc;
                }
                __syncthreads();
                // rows r0.. of -X_s M: X_s(i, k) for k <= i
                for (int q = tid; q < ns.ncol * cn; q += kFactorThreads) {
                    const int i = q % ns.ncol, c = q / ns.ncol;
                    TF acc = (TF)0;
                    for (int k = r0; k < r0 + rn && k <= i; ++k) acc += Xs[(int64_t)k * ns.ldx + i] * Ms[k - r0][c];
                    Xb[(int64_t)(o + c0 + c) * ldb + os + i] -= acc;
                }
                __syncthreads();
            }
    }
    __syncthreads();
    // transposes: X^T (nbk columns of ldb rows) and L21^T (nb columns of ldb rows)
    for (int64_t q = tid; q < (int64_t)ldb * nbk; q += kFactorThreads) {
        const int r = (int)(q % ldb), c = (int)(q / ldb);  // XbT(r, c) = Xb(c, r)
        XbT[q] = (r < nbk && c < nbk) ? Xb[(int64_t)r * ldb + c] : (TF)0;
    }
    for (int64_t q = tid; q < (int64_t)ldb * nb; q += kFactorThreads) {
        const int r = (int)(q % ldb), c = (int)(q / ldb);  // LbT(r, c) = Lb(c, r)
        LbT[q] = r < nbk ? Lb[(int64_t)r * ld21 + c] : (TF)0;
    }
}

// Column block jb of X = inv(L11): X_jj = inv(L_jj) and, block row by block
// row, X_ij = -inv(L_ii) sum_{k=j..i-1} L_ik X_kj. Each block row is written
// to X (and X^T) as soon as it is known; later block rows read the rows above
// back from X (the CTA's own writes, visible after a barrier), staged with the
// matching columns of L through shared memory KC rows at a time, so the front
// may have any number of columns. Also writes the aligned L21 / L21^T copies
// of the block's columns.
template <typename TF>
__global__ void __launch_bounds__(kFactorThreads)
k_fx(const FItem *__restrict__ items, const SnInfo *__restrict__ sn, const TF *__restrict__ Lval,
     const TF *__restrict__ Dinv, TF *__restrict__ Xall, TF *__restrict__ L21all, TF *__restrict__ L21Tall) {
    constexpr int KC = sizeof(TF) == 4 ? 64 : 32;  // rows of the sum staged per pass
    __shared__ TF Ts[NB][NB + 1];
    __shared__ TF Ds[NB][NB + 1];  // inverse of the current diagonal block, [t][r]
    __shared__ TF Ls[NB][KC + 1];  // L(i0 + r, k0 + kk)
    __shared__ TF Xs[KC][NB + 1];  // X(k0 + kk, j0 + c)
    const FItem it = items[blockIdx.x];
    const SnInfo d = sn[it.sn];
    const int n = d.nrow, nc = d.ncol, nb = n - nc;
    const int jb = it.a, j0 = jb * NB, wj = min(NB, nc - j0);
    const TF *P = Lval + d.panel_off;
    TF *X = Xall + d.x_off, *XT = Xall + d.xt_off;
    const int ldx = d.ldx;
    const int tid = threadIdx.x;
    const int nblk = (nc + NB - 1) / NB;
    const int r = tid % NB, cg = tid / NB;  // row in block, group of 4 columns
    // X(i0 + r, j0 + c) for c < wj into X and X^T (X^T keeps the lower part)
    auto store_rows = [&](int i0, int wi, const TF v[4]) {
        if (r >= wi) return;
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) {
            const int c = cg * 4 + cc, i = i0 + r;
            if (c >= wj) continue;
            X[(int64_t)(j0 + c) * ldx + i] = v[cc];
            if (i >= j0 + c) XT[(int64_t)i * ldx + j0 + c] = v[cc];
        }
    };
    {
        const TF *Djj = Dinv + d.dinv_off + (int64_t)jb * NB * NB;  // column-major
        TF v[4];
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) v[cc] = Djj[(int64_t)(cg * 4 + cc) * NB + r];
        store_rows(j0, wj, v);
    }
    for (int ib = jb + 1; ib < nblk; ++ib) {
        const int i0 = ib * NB, wi = min(NB, nc - i0);
        {
            // the block's inverse into shared memory (read 32 times per column below)
            const TF *Dii = Dinv + d.dinv_off + (int64_t)ib * NB * NB;
            for (int q = tid; q < NB * NB; q += kFactorThreads) Ds[q / NB][q % NB] = Dii[q];
        }
        // sum_k L(i0 + r, k) X(k, j0 + c) over k in [j0, i0), in increasing k
        TF acc[4] = {(TF)0, (TF)0, (TF)0, (TF)0};
        for (int k0 = j0; k0 < i0; k0 += KC) {
            const int kw = min(KC, i0 - k0);
            __syncthreads();  // the rows of X read below were written before it
            for (int q = tid; q < NB * KC; q += kFactorThreads) {
                const int rr = q % NB, kk = q / NB;
                Ls[rr][kk] = (rr < wi && kk < kw) ? P[(int64_t)(k0 + kk) * n + i0 + rr] : (TF)0;
            }
            for (int q = tid; q < KC * NB; q += kFactorThreads) {
                const int kk = q % KC, c = q / KC;
                Xs[kk][c] = (kk < kw && c < wj) ? X[(int64_t)(j0 + c) * ldx + k0 + kk] : (TF)0;
            }
            __syncthreads();
            if (r < wi) {
#pragma unroll 8
                for (int kk = 0; kk < kw; ++kk) {
                    const TF l = Ls[r][kk];
#pragma unroll
                    for (int cc = 0; cc < 4; ++cc) acc[cc] += l * Xs[kk][cg * 4 + cc];
                }
            }
        }
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) Ts[cg * 4 + cc][r] = acc[cc];
        __syncthreads();
        // X(i0 + r, c) = -sum_{t <= r} inv(L_ii)(r, t) T(t, c), in increasing t
        // (a fixed-length loop with the bound as a predicate: the loads of
        // all terms issue ahead of the sums)
        TF v[4] = {(TF)0, (TF)0, (TF)0, (TF)0};
#pragma unroll
        for (int t = 0; t < NB; ++t) {
            const TF dt = Ds[t][r];
#pragma unroll
            for (int cc = 0; cc < 4; ++cc)
                if (t <= r) v[cc] += dt * Ts[cg * 4 + cc][t];
        }
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) v[cc] = -v[cc];
        store_rows(i0, wi, v);
        __syncthreads();  // Ts and Ds are rewritten by the next block row
    }
    // rows of X above the block column stay as set up: zero (X is lower triangular)
    TF *L21 = L21all + d.l21_off, *L21T = L21Tall + d.l21t_off;
    const int ld21 = d.ld21;
    for (int q = tid; q < wj * nb; q += kFactorThreads) {
        const int c = j0 + q / nb, i = q % nb;
        const TF v = P[(int64_t)c * n + nc + i];
        L21[(int64_t)c * ld21 + i] = v;
        L21T[(int64_t)i * ldx + c] = v;
    }
}

// ---------------------------------------------------------------------------
// local step: estimateRotations, arap.h:354-384

template <typename T>
__global__ void __launch_bounds__(256)
k_local_step(int V, const int32_t *__restrict__ drow, const int32_t *__restrict__ dcol, const T *__restrict__ w,
             const Vec4<T> *__restrict__ p, const Vec4<T> *__restrict__ pc, Vec4<T> *__restrict__ R) {
    pdl_wait();  // the positions of the kernels before (an overlapped launch)
    pdl_trigger();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    const Vec4<T> pi = p[i], ci = pc[i];
    T S[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) S[a][b] = (T)0;
    const int e1 = drow[i + 1];
    for (int e = drow[i]; e < e1; ++e) {
        const int j = dcol[e];
        const T wj = w[e];
        const Vec4<T> pj = p[j], cj = pc[j];
        const T ex = wj * (pi.x - pj.x), ey = wj * (pi.y - pj.y), ez = wj * (pi.z - pj.z);
        const T fx = ci.x - cj.x, fy = ci.y - cj.y, fz = ci.z - cj.z;
        S[0][0] += ex * fx; S[0][1] += ex * fy; S[0][2] += ex * fz;
        S[1][0] += ey * fx; S[1][1] += ey * fy; S[1][2] += ey * fz;
        S[2][0] += ez * fx; S[2][1] += ez * fy; S[2][2] += ez * fz;
    }
    T Rm[3][3];
    if constexpr (sizeof(T) == 8) dev::rotation_fit_fp64(S, Rm);
    else rotation_from_cov(S, Rm);
    R[3 * (int64_t)i + 0] = {Rm[0][0], Rm[0][1], Rm[0][2], (T)0};
    R[3 * (int64_t)i + 1] = {Rm[1][0], Rm[1][1], Rm[1][2], (T)0};
    R[3 * (int64_t)i + 2] = {Rm[2][0], Rm[2][1], Rm[2][2], (T)0};
}

// Local step of the mixed form: the covariance in FP32 from the FP32 rest
// edges and the current edges differenced in FP64 (the positions are kept in
// FP64), then the FP32 rotation fit.
template <int G>
__device__ __forceinline__ float group_sum(float v) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
template <int G>
__device__ __forceinline__ double group_sum(double v) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Threads per vertex: a group of G lanes of one warp takes a vertex, lane l
// its adjacency entries l, l + G, ...; the partial sums meet by shuffles
// (G = 1: one thread per vertex). Every lane of a warp reaches the shuffles.
template <int G>
__global__ void __launch_bounds__(kLocalMaxBlock)
k_local_step_mixed(int V, const int32_t *__restrict__ drow, const int32_t *__restrict__ dcol,
                   const float *__restrict__ w, const Vec4<float> *__restrict__ redge,
                   const Vec4<double> *__restrict__ pc64, Vec4<float> *__restrict__ R,
                   const double *__restrict__ w64, const Vec4<double> *__restrict__ p64) {
    pdl_wait();  // the positions of the kernels before (an overlapped launch)
    pdl_trigger();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = t / G, l = t % G;
    const bool live = i < V;
    float S[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    int e1 = 0;
    if (live) {
        const Vec4<double> ci = pc64[i];
        e1 = drow[i + 1];
        for (int e = drow[i] + l; e < e1; e += G) {
            const float wj = w[e];
            const Vec4<float> re = redge[e];
            const Vec4<double> cj = pc64[dcol[e]];
            const float ex = wj * re.x, ey = wj * re.y, ez = wj * re.z;
            const float fx = (float)(ci.x - cj.x), fy = (float)(ci.y - cj.y), fz = (float)(ci.z - cj.z);
            S[0][0] += ex * fx; S[0][1] += ex * fy; S[0][2] += ex * fz;
            S[1][0] += ey * fx; S[1][1] += ey * fy; S[1][2] += ey * fz;
            S[2][0] += ez * fx; S[2][1] += ez * fy; S[2][2] += ez * fz;
        }
    }
    if (G > 1) {
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) S[a][b] = group_sum<G>(S[a][b]);
    }
    if (!live || l != 0) return;
    float Rm[3][3], spread;
    rotation_from_cov(S, Rm, &spread);
    if (!(spread >= dev::kPolarFallback)) dev::rotation_fp64<true>(i, drow[i], e1, dcol, w64, p64, pc64, 1, 0, Rm);
    R[3 * (int64_t)i + 0] = {Rm[0][0], Rm[0][1], Rm[0][2], 0.f};
    R[3 * (int64_t)i + 1] = {Rm[1][0], Rm[1][1], Rm[1][2], 0.f};
    R[3 * (int64_t)i + 2] = {Rm[2][0], Rm[2][1], Rm[2][2], 0.f};
}



// RHS of the mixed form without bFixed (added in FP64 by the residual):
// sum_j 1/2 w (R_i + R_j)(p_i - p_j) over the FP32 rest edges.
template <int G>
__global__ void __launch_bounds__(1024)
k_rhs_mixed(int m, const int32_t *__restrict__ drow, const int32_t *__restrict__ dcol, const float *__restrict__ w,
            const Vec4<float> *__restrict__ redge, const Vec4<float> *__restrict__ R, Vec4<float> *__restrict__ b) {
    pdl_wait();  // the rotations of the local step (an overlapped launch)
    pdl_trigger();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = t / G, l = t % G;
    const bool live = i < m;
    float ax = 0.f, ay = 0.f, az = 0.f;
    if (live) {
        const Vec4<float> r0 = R[3 * (int64_t)i], r1 = R[3 * (int64_t)i + 1], r2 = R[3 * (int64_t)i + 2];
        const int e1 = drow[i + 1];
        for (int e = drow[i] + l; e < e1; e += G) {
            const int j = dcol[e];
            if (j == i) continue;
            const float h = w[e] * 0.5f;
            const Vec4<float> d = redge[e];
            const Vec4<float> q0 = R[3 * (int64_t)j], q1 = R[3 * (int64_t)j + 1], q2 = R[3 * (int64_t)j + 2];
            ax += ((r0.x + q0.x) * d.x + (r0.y + q0.y) * d.y + (r0.z + q0.z) * d.z) * h;
            ay += ((r1.x + q1.x) * d.x + (r1.y + q1.y) * d.y + (r1.z + q1.z) * d.z) * h;
            az += ((r2.x + q2.x) * d.x + (r2.y + q2.y) * d.y + (r2.z + q2.z) * d.z) * h;
        }
    }
    if (G > 1) {
        ax = group_sum<G>(ax);
        ay = group_sum<G>(ay);
        az = group_sum<G>(az);
    }
    if (live && l == 0) b[i] = {ax, ay, az, 0.f};
}

// estimatePositions RHS, arap.h:395-414
template <typename T>
__global__ void __launch_bounds__(256)
k_rhs(int m, const int32_t *__restrict__ drow, const int32_t *__restrict__ dcol, const T *__restrict__ w,
      const Vec4<T> *__restrict__ p, const Vec4<T> *__restrict__ R, const Vec4<T> *__restrict__ bfixed,
      Vec4<T> *__restrict__ b) {
    pdl_wait();     // the positions and rotations of the kernels before
    pdl_trigger();  // the forward sweep may take its first tasks meanwhile
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const Vec4<T> pi = p[i];
    const Vec4<T> r0 = R[3 * (int64_t)i], r1 = R[3 * (int64_t)i + 1], r2 = R[3 * (int64_t)i + 2];
    Vec4<T> acc = bfixed[i];
    const int e1 = drow[i + 1];
    for (int e = drow[i]; e < e1; ++e) {
        const int j = dcol[e];
        if (j == i) continue;
        const T h = w[e] * (T)0.5;
        const Vec4<T> pj = p[j];
        const Vec4<T> q0 = R[3 * (int64_t)j], q1 = R[3 * (int64_t)j + 1], q2 = R[3 * (int64_t)j + 2];
        const T dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
        acc.x += ((r0.x + q0.x) * dx + (r0.y + q0.y) * dy + (r0.z + q0.z) * dz) * h;
        acc.y += ((r1.x + q1.x) * dx + (r1.y + q1.y) * dy + (r1.z + q1.z) * dz) * h;
        acc.z += ((r2.x + q2.x) * dx + (r2.y + q2.y) * dy + (r2.z + q2.z) * dz) * h;
    }
    b[i] = acc;
}

// r = b - A x in FP64 over the free vertices (A = constrained Laplacian)
template <int G>
__global__ void __launch_bounds__(1024)
k_residual(int m, const int32_t *__restrict__ drow, const int32_t *__restrict__ dcol, const double *__restrict__ w64,
           const double *__restrict__ diag64, const Vec4<double> *__restrict__ bfixed,
           const Vec4<float> *__restrict__ b, const Vec4<double> *__restrict__ x, Vec4<float> *__restrict__ r) {
    pdl_wait();     // x and b of the kernels before
    pdl_trigger();  // the forward sweep may take its first tasks meanwhile
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = t / G, l = t % G;
    const bool live = i < m;
    double ax = 0.0, ay = 0.0, az = 0.0;
    if (live) {
        const int e1 = drow[i + 1];
        for (int e = drow[i] + l; e < e1; e += G) {
            const int j = dcol[e];
            if (j == i || j >= m) continue;
            const double wj = w64[e];
            const Vec4<double> xj = x[j];
            ax -= wj * xj.x;
            ay -= wj * xj.y;
            az -= wj * xj.z;
        }
    }
    if (G > 1) {
        ax = group_sum<G>(ax);
        ay = group_sum<G>(ay);
        az = group_sum<G>(az);
    }
    if (!live || l != 0) return;
    const Vec4<double> xi = x[i];
    const double d = diag64[i];
    ax += d * xi.x;
    ay += d * xi.y;
    az += d * xi.z;
    const Vec4<float> bi = b[i];
    const Vec4<double> bf = bfixed[i];
    r[i] = {(float)((bf.x + (double)bi.x) - ax), (float)((bf.y + (double)bi.y) - ay),
            (float)((bf.z + (double)bi.z) - az), 0.f};
}

// ---------------------------------------------------------------------------
// supernodal triangular solves
//
// One CTA per supernode, one launch per sweep. The CTA's matrices (forward: X
// then L21; backward: L21^T then X^T, all column-major with 16-byte aligned
// columns) are streamed through two shared-memory buffers by TMA bulk copies
// (cp.async.bulk + mbarrier). The first two chunks are requested before the
// CTA waits for the supernodes it depends on, so the copies overlap the wait.
// Threads own 4-row quads of the result; G groups of threads split each
// chunk's columns and are reduced once at the end of a matrix.

#ifndef ARAP_SOLVE_CHUNK_KB
#define ARAP_SOLVE_CHUNK_KB 16
#endif
#ifndef ARAP_SOLVE_BUFS
#define ARAP_SOLVE_BUFS 2
#endif
constexpr int kSolveThreads = 256;
constexpr int kChunkBytes = ARAP_SOLVE_CHUNK_KB * 1024;  // bytes per TMA chunk buffer
constexpr int kSolveBufs = ARAP_SOLVE_BUFS;  // chunk buffers of a lower-level solve CTA (a ring)
static_assert((kSolveBufs & (kSolveBufs - 1)) == 0 && kSolveBufs >= 2, "ring of 2, 4 or 8 buffers");
constexpr int kRedRows = 4 * kSolveThreads;  // G * 4 * NQ <= 4 * threads

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bulk copy global -> shared (both 16-byte aligned, bytes a multiple of 16),
// completion counted on `bar`.
__device__ __forceinline__ void tma_load_1d(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// The chunks of one task: matrix A (columns [0, CA), leading dimension ldA)
// then matrix B (columns [0, CB), ldB), each cut into column ranges of at most
// kChunkBytes (fronts of one pass: a column has at most kSolveBlockRows rows).
// Fronts of several passes stream segments instead: segment j of pass rb
// holds rows [rb * kSolveBlockRows, +kSolveBlockRows) of kSegCols columns,
// packed with the segment's row count as leading dimension, so a column may
// have any length and each pass reads only its own rows.
template <typename T>
struct ChunkPlan {
    static constexpr int kSegCols = kChunkBytes / (kSolveBlockRows * (int)sizeof(T));
    const T *A, *B;
    int ldA, ldB, CA, CB, cwA, cwB, nA, nB, sA, sB;
    __device__ void init(const T *a, int lda, int ca, const T *b, int ldb, int cb) {
        A = a; B = b; ldA = lda; ldB = ldb; CA = ca; CB = cb;
        cwA = max(1, kChunkBytes / (lda * (int)sizeof(T)));
        cwB = ldb > 0 ? max(1, kChunkBytes / (ldb * (int)sizeof(T))) : 1;
        nA = (CA + cwA - 1) / cwA;
        nB = CB > 0 ? (CB + cwB - 1) / cwB : 0;
        sA = (CA + kSegCols - 1) / kSegCols;
        sB = CB > 0 ? (CB + kSegCols - 1) / kSegCols : 0;
    }
    // segment j (j < sA: of A, else of B) of pass rb: first column, columns,
    // source of its first column's rows, the matrix's leading dimension and
    // the segment's rows
    __device__ void seg(int j, int rb, int &c0, int &cn, const T *&src, int &ld, int &rows) const {
        const bool a = j < sA;
        const int jj = a ? j : j - sA, C = a ? CA : CB, row0 = rb * kSolveBlockRows;
        ld = a ? ldA : ldB;
        c0 = jj * kSegCols;
        cn = min(kSegCols, C - c0);
        rows = min(kSolveBlockRows, ld - row0);
        src = (a ? A : B) + (int64_t)c0 * ld + row0;
    }
    __device__ int total() const { return nA + nB; }
    // first column, number of columns and source of chunk k
    __device__ void chunk(int k, int &c0, int &cn, const T *&src, int &ld) const {
        if (k < nA) { c0 = k * cwA; cn = min(cwA, CA - c0); src = A + (int64_t)c0 * ldA; ld = ldA; }
        else { const int j = k - nA; c0 = j * cwB; cn = min(cwB, CB - c0); src = B + (int64_t)c0 * ldB; ld = ldB; }
    }
};

// Asks the TMA unit to pull chunk k into L2 (no shared memory involved).
template <typename T>
__device__ __forceinline__ void prefetch_chunk_l2(const ChunkPlan<T> &pl, int k) {
    int c0, cn, ld;
    const T *src;
    pl.chunk(k, c0, cn, src, ld);
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"((unsigned)(cn * ld * (int)sizeof(T)))
                 : "memory");
}

template <typename T>
__device__ __forceinline__ void issue_chunk(const ChunkPlan<T> &pl, int k, T *buf, uint64_t *bar) {
    int c0, cn, ld;
    const T *src;
    pl.chunk(k, c0, cn, src, ld);
    const unsigned bytes = (unsigned)(cn * ld * (int)sizeof(T));
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // buffer reads done before the async write
    mbar_expect_tx(bar, bytes);
    tma_load_1d(buf, src, bytes, bar);
}

// Segment j of pass rb into buf: one bulk copy per column (16-byte aligned:
// leading dimensions are multiples of 4 and passes start at multiples of
// kSolveBlockRows), all counted on `bar`.
template <typename T>
__device__ __forceinline__ void issue_seg(const ChunkPlan<T> &pl, int j, int rb, T *buf, uint64_t *bar) {
    int c0, cn, ld, rows;
    const T *src;
    pl.seg(j, rb, c0, cn, src, ld, rows);
    const unsigned bytes = (unsigned)(rows * (int)sizeof(T));
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // buffer reads done before the async write
    mbar_expect_tx(bar, bytes * (unsigned)cn);
    for (int i = 0; i < cn; ++i) tma_load_1d(buf + i * rows, src + (int64_t)i * ld, bytes, bar);
}

// Both matrices of a task of several passes into L2, in pieces of at most 1 MiB.
template <typename T>
__device__ __forceinline__ void prefetch_mats_l2(const ChunkPlan<T> &pl) {
    for (int m = 0; m < 2; ++m) {
        const char *p = reinterpret_cast<const char *>(m == 0 ? pl.A : pl.B);
        const int64_t total = (int64_t)(m == 0 ? pl.CA * pl.ldA : pl.CB * pl.ldB) * (int64_t)sizeof(T);
        for (int64_t o = 0; o < total; o += (1 << 20)) {
            const unsigned n = (unsigned)min((int64_t)(1 << 20), total - o);
            asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p + o), "r"(n) : "memory");
        }
    }
}

// Chunk buffer b of a lower-level solve CTA (the ring at the start of its
// dynamic shared memory).
template <typename T>
__device__ __forceinline__ T *sbuf(unsigned char *raw, int b) {
    return reinterpret_cast<T *>(raw + b * kChunkBytes);
}

// A task's chunk stream when a GEMV phase has more rows than one pass covers
// (kSolveBlockRows, one 4-row quad per thread): phase A's chunks once per row
// block of its rows, then phase B's chunks once per row block of theirs (B's
// chunks follow A's in the ChunkPlan). With fronts of at most kSolveBlockRows
// rows this is the plain chunk sequence.
struct VPlan {
    int nA, nB, rbA, rbB;
    __device__ int total() const { return nA * rbA + nB * rbB; }
};

__device__ __forceinline__ int row_blocks(int rows) { return (rows + kSolveBlockRows - 1) / kSolveBlockRows; }

// Walks a VPlan's stream one chunk at a time without divisions: k is the
// chunk's index in the ChunkPlan, phase and rb its phase and row block.
struct VCursor {
    int k, phase, rb;
    __device__ void start(const VPlan &v) {
        rb = 0;
        phase = v.nA * v.rbA > 0 ? 0 : 1;
        k = phase == 0 ? 0 : v.nA;
    }
    __device__ void step(const VPlan &v) {
        ++k;
        if (phase == 0) {
            if (k == v.nA) {
                k = 0;
                if (++rb == v.rbA) {
                    phase = 1;
                    rb = 0;
                    k = v.nA;
                }
            }
        } else if (k == v.nA + v.nB) {
            k = v.nA;
            ++rb;
        }
    }
    __device__ bool first_of_pass(const VPlan &v) const { return k == (phase == 0 ? 0 : v.nA); }
};

// Bounded wait for a buffer's bytes. On expiry it records kErrTimeout and
// waits once more (bounded) so that no copy is still writing into shared
// memory when the CTA moves on.
__device__ __forceinline__ void wait_chunk(uint64_t *bar, unsigned parity, int *err) {
    for (unsigned it = 0; it < kSpinLimit; ++it)
        if (mbar_try_wait(bar, parity)) return;
    if (threadIdx.x == 0) atomicOr(err, kErrTimeout);
    for (unsigned it = 0; it < kSpinLimit; ++it)
        if (mbar_try_wait(bar, parity)) return;
}

// acc[k] += sum over this thread's columns of the chunk of M(4q+k, c) v[c0+c]
template <typename T>
__device__ __forceinline__ void chunk_axpy(const T *buf, int ld, int cn, int c0, int q, int g, int G,
                                           const Vec4<T> *v, T ax[4], T ay[4], T az[4]) {
    for (int c = g; c < cn; c += G) {
        const Vec4<T> m = *reinterpret_cast<const Vec4<T> *>(buf + (int64_t)c * ld + 4 * q);
        const Vec4<T> vc = v[c0 + c];
        ax[0] += m.x * vc.x; ay[0] += m.x * vc.y; az[0] += m.x * vc.z;
        ax[1] += m.y * vc.x; ay[1] += m.y * vc.y; az[1] += m.y * vc.z;
        ax[2] += m.z * vc.x; ay[2] += m.z * vc.y; az[2] += m.z * vc.z;
        ax[3] += m.w * vc.x; ay[3] += m.w * vc.y; az[3] += m.w * vc.z;
    }
}

// Work split of a GEMV phase over the CTA: thread t owns the 4-row quad q of
// the result (NQ = ceil(rows / 4) quads, at most 256) for the columns g,
// g + G, ... Below 32 quads, q = t mod NQp and g = t div NQp with NQp the next
// power of two (a warp's partial sums then meet by shuffles); from 32 quads
// on, q = t mod NQ and g = t div NQ with G = 256 div NQ groups, so that all
// but 256 mod NQ threads work. Inactive threads only take part in the
// reductions.
struct Quads {
    int NQ, NQp, G, q, g;
    __device__ bool active() const { return q < NQ && g < G; }
};

__device__ __forceinline__ Quads quads_for(int rows) {
    Quads Q;
    Q.NQ = (rows + 3) >> 2;
    Q.NQp = 1;
    while (Q.NQp < Q.NQ) Q.NQp <<= 1;
    if (Q.NQ < 32) {
        Q.G = kSolveThreads / Q.NQp;
        Q.q = threadIdx.x & (Q.NQp - 1);
        Q.g = threadIdx.x / Q.NQp;
    } else {
        Q.G = kSolveThreads / Q.NQ;
        Q.q = threadIdx.x % Q.NQ;
        Q.g = threadIdx.x / Q.NQ;
    }
    return Q;
}

// Sums the G partial results of every quad into out (SUB: out -= sum): first
// across the lanes of a warp that share a quad (shuffles; only when NQp < 32),
// then over at most 8 partials per quad through shared memory, in a fixed
// order. Ends with a barrier.
template <typename T, bool SUB>
__device__ __forceinline__ void reduce_quads(const Quads &Q, T ax[4], T ay[4], T az[4], T *red, Vec4<T> *out) {
    // scratch: three arrays of kRedRows scalars (x, y, z)
    T *rx = red, *ry = red + kRedRows, *rz = red + 2 * kRedRows;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int slot, nslots;
    bool writer;
    if (Q.NQp < 32) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            if (off < Q.NQp) break;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                ax[k] += __shfl_xor_sync(0xffffffffu, ax[k], off);
                ay[k] += __shfl_xor_sync(0xffffffffu, ay[k], off);
                az[k] += __shfl_xor_sync(0xffffffffu, az[k], off);
            }
        }
        slot = warp;
        nslots = kSolveThreads / 32;
        writer = lane < Q.NQp;
    } else {
        slot = Q.g;
        nslots = Q.G;
        writer = true;
    }
    if (writer && Q.active())
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int i = (slot * Q.NQ + Q.q) * 4 + k;
            rx[i] = ax[k];
            ry[i] = ay[k];
            rz[i] = az[k];
        }
    __syncthreads();
    for (int rr = tid; rr < 4 * Q.NQ; rr += kSolveThreads) {
        const int qq = rr >> 2, k = rr & 3;
        T sx = 0, sy = 0, sz = 0;
        for (int s = 0; s < nslots; ++s) {
            const int i = (s * Q.NQ + qq) * 4 + k;
            sx += rx[i]; sy += ry[i]; sz += rz[i];
        }
        Vec4<T> &o = out[rr];
        if (SUB) { o.x -= sx; o.y -= sy; o.z -= sz; }
        else o = {sx, sy, sz, (T)0};
    }
    __syncthreads();
}

// Ticket of the calling CTA's next task (thread 0 only). A launch of G CTAs
// over S tasks consumes exactly Z = S + G tickets: S tasks, then one ticket
// per CTA that finds no task left and leaves the loop. Launch e (counted from
// the last reset of the counter) owns tickets [e*Z, (e+1)*Z) and publishes
// its flags with epoch e + 1. Once any wait of the context expired, every CTA
// leaves at its next ticket. `reverse`: tasks in reverse `order`.
__device__ __forceinline__ void next_task(unsigned long long *ticket, int S, int Z, const int32_t *order,
                                          bool reverse, const int *err, int &task, unsigned &epoch) {
    const unsigned long long t = atomicAdd(ticket, 1ull);
    const int r = (int)(t % (unsigned long long)Z);
    const bool stop = (*(volatile const int *)err & kErrTimeout) != 0;
    task = (r < S && !stop) ? order[reverse ? S - 1 - r : r] : -1;
    epoch = (unsigned)(t / (unsigned long long)Z) + 1u;
}

#include "arap_wsolve.cuh"

// Shared memory of a solve CTA (dynamic): two chunk buffers, three vectors
// (two of max_ldx rows, one of max_ld21 rows) and the reduction scratch.
struct SolveSmem {
    int ldx_max, ld21_max;
};

// Forward: for supernode s (children first), f = [b(cols); 0] plus the
// children's update vectors; y = X f(cols); u_s = f(struct) - L21 y goes to
// the parent. Tickets follow `order` (level by level, leaves first), so a CTA
// only waits for CTAs that started before it.
template <typename T>
__global__ void __launch_bounds__(kSolveThreads, 3)
k_solve_fwd(int S, int Z, int lbeg, SolveSmem lay, const int32_t *__restrict__ order, const SnInfo *__restrict__ sn,
            const int32_t *__restrict__ child, const int32_t *__restrict__ relind, const T *__restrict__ Xall,
            const T *__restrict__ L21all, Vec4<T> *__restrict__ sol, Vec4<T> *__restrict__ uvec,
            unsigned long long *ticket, unsigned *flags, int *err) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    Vec4<T> *fc = reinterpret_cast<Vec4<T> *>(smem_raw + kSolveBufs * kChunkBytes);
    // y takes f's place once phase A's sums are reduced, unless a front needs
    // several passes (later passes still read all of f)
    const bool y_in_f = lay.ldx_max <= kSolveBlockRows;
    Vec4<T> *yv = y_in_f ? fc : fc + lay.ldx_max;
    Vec4<T> *fb = yv + lay.ldx_max;
    T *red = reinterpret_cast<T *>(fb + lay.ld21_max);
    __shared__ __align__(8) uint64_t bars[kSolveBufs];
    __shared__ int s_task[2];  // this task's and the next one's ticket (taken early)
    __shared__ unsigned s_epoch[2];
    const int tid = threadIdx.x;
    // the dense top's product may start its copies on SMs this grid leaves
    pdl_trigger();
    if (tid == 0) {
        for (int b = 0; b < kSolveBufs; ++b) mbar_init(&bars[b], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        next_task(ticket, S, Z, order, false, err, s_task[0], s_epoch[0]);
    }
    __syncthreads();
    unsigned ph[kSolveBufs];  // phases each chunk buffer completed in earlier tasks
#pragma unroll
    for (int b = 0; b < kSolveBufs; ++b) ph[b] = 0u;
    for (int slot = 0;; slot ^= 1) {
    const int s = s_task[slot];
    if (s < 0) break;
    const unsigned epoch = s_epoch[slot];
    const SnInfo d = sn[s];
    const int nc = d.ncol, nb = d.nrow - d.ncol;
    ChunkPlan<T> pl;
    pl.init(Xall + d.x_off, d.ldx, nc, L21all + d.l21_off, d.ld21, nb > 0 ? nc : 0);
    const int ntot = pl.total();
    // one pass (chunks of whole columns) or several (segments of each pass's rows)
    const int rbA = row_blocks(nc), rbB = pl.nB > 0 ? row_blocks(nb) : 0;
    const bool multi = rbA > 1 || rbB > 1;
    const VPlan vp = multi ? VPlan{pl.sA, pl.sB, rbA, rbB} : VPlan{pl.nA, pl.nB, rbA, rbB};
    const int vtot = vp.total();
    VCursor iss;  // next stream position to issue (thread 0)
    iss.start(vp);
    if (tid == 0) {
        for (int e = 0; e < vtot && e < kSolveBufs; ++e, iss.step(vp)) {
            if (multi) issue_seg(pl, iss.k, iss.rb, sbuf<T>(smem_raw, e), &bars[e]);
            else issue_chunk(pl, iss.k, sbuf<T>(smem_raw, e), &bars[e]);
        }
        if (multi) prefetch_mats_l2(pl);
        else for (int k = kSolveBufs; k < ntot; ++k) prefetch_chunk_l2(pl, k);
    }
    // the ticket, the task's description and its first copies (the factor does
    // not change between factorisations) came before the kernel this launch
    // may overlap had finished; the right-hand side and the flags come after
    pdl_wait();
    for (int i = tid; i < d.ldx; i += kSolveThreads)
        fc[i] = (i < nc) ? sol[d.first + i] : Vec4<T>{(T)0, (T)0, (T)0, (T)0};
    for (int i = tid; i < d.ld21; i += kSolveThreads) fb[i] = {(T)0, (T)0, (T)0, (T)0};
    // the children's entries of this thread (child-major list, kPull per thread):
    // positions are read before waiting, update vectors in one round trip after
    constexpr int kPull = 4;
    int pci[kPull], ppos[kPull], puo[kPull];
    {
        int base = 0, u = 0;
        for (int ci = d.child_begin; ci < d.child_end && u < kPull; ++ci) {
            const SnInfo c = sn[child[ci]];
            const int nbc = c.nrow - c.ncol;
            for (int i = tid - base; i < nbc && u < kPull; i += kSolveThreads) {
                if (i < 0) continue;
                pci[u] = ci;
                ppos[u] = relind[c.relind_off + i];
                puo[u] = (int)c.uvec_off + i;
                ++u;
            }
            base += nbc;
        }
        for (; u < kPull; ++u) pci[u] = -1;
    }
    int total_children_rows = 0;
    for (int ci = d.child_begin; ci < d.child_end; ++ci) {
        const SnInfo c = sn[child[ci]];
        total_children_rows += c.nrow - c.ncol;
    }
    if (tid == 0)
        for (int ci = d.child_begin; ci < d.child_end; ++ci)
            if (sn[child[ci]].level >= lbeg) wait_flag(flags + child[ci], epoch, err);  // lower: an earlier launch
    // the next ticket is taken once this task is ready to run, so its round
    // trip overlaps the work below
    if (tid == 32) next_task(ticket, S, Z, order, false, err, s_task[slot ^ 1], s_epoch[slot ^ 1]);
    __syncthreads();
    if (total_children_rows <= kPull * kSolveThreads) {
        Vec4<T> pu[kPull];
#pragma unroll
        for (int u = 0; u < kPull; ++u)
            if (pci[u] >= 0) pu[u] = ldcg4(uvec + puo[u]);
        for (int ci = d.child_begin; ci < d.child_end; ++ci) {  // children in order
#pragma unroll
            for (int u = 0; u < kPull; ++u) {
                if (pci[u] != ci) continue;
                Vec4<T> &t = ppos[u] < nc ? fc[ppos[u]] : fb[ppos[u] - nc];
                t.x += pu[u].x;
                t.y += pu[u].y;
                t.z += pu[u].z;
            }
            __syncthreads();
        }
    } else {
        for (int ci = d.child_begin; ci < d.child_end; ++ci) {
            const SnInfo c = sn[child[ci]];
            const int nbc = c.nrow - c.ncol;
            const int32_t *ri = relind + c.relind_off;
            for (int i = tid; i < nbc; i += kSolveThreads) {
                const Vec4<T> u = ldcg4(uvec + c.uvec_off + i);
                const int pos = ri[i];
                Vec4<T> &t = pos < nc ? fc[pos] : fb[pos - nc];
                t.x += u.x;
                t.y += u.y;
                t.z += u.z;
            }
            __syncthreads();
        }
    }
    // phase A: y = X fc (rows nc), phase B: fb -= L21 y (rows nb), each in
    // passes of at most kSolveBlockRows rows
    T ax[4] = {0, 0, 0, 0}, ay[4] = {0, 0, 0, 0}, az[4] = {0, 0, 0, 0};
    if (!multi) {
        // every phase in one pass: the plain chunk sequence
        const Quads Qa = quads_for(nc), Qb = quads_for(nb);
        for (int k = 0; k < ntot; ++k) {
            const int kb = k & (kSolveBufs - 1);
            T *buf = sbuf<T>(smem_raw, kb);
            wait_chunk(&bars[kb], (ph[kb] + (unsigned)(k / kSolveBufs)) & 1u, err);
            int c0, cn, ld;
            const T *src;
            pl.chunk(k, c0, cn, src, ld);
            if (k < pl.nA) {
                if (Qa.active()) chunk_axpy(buf, ld, cn, c0, Qa.q, Qa.g, Qa.G, fc, ax, ay, az);
            } else {
                if (Qb.active()) chunk_axpy(buf, ld, cn, c0, Qb.q, Qb.g, Qb.G, yv, ax, ay, az);
            }
            __syncthreads();
            if (tid == 0 && k + kSolveBufs < ntot) issue_chunk(pl, k + kSolveBufs, buf, &bars[kb]);
            if (k == pl.nA - 1) {
                reduce_quads<T, false>(Qa, ax, ay, az, red, yv);
#pragma unroll
                for (int z = 0; z < 4; ++z) ax[z] = ay[z] = az[z] = (T)0;
            }
        }
        if (pl.nB > 0) reduce_quads<T, true>(Qb, ax, ay, az, red, fb);
    } else {
        VCursor cur;
        cur.start(vp);
        Quads Q;
        for (int e = 0; e < vtot; ++e, cur.step(vp)) {
            const int k = cur.k, phase = cur.phase, row0 = cur.rb * kSolveBlockRows;
            if (cur.first_of_pass(vp)) Q = quads_for(min(kSolveBlockRows, (phase == 0 ? nc : nb) - row0));
            const int kb = e & (kSolveBufs - 1);
            T *buf = sbuf<T>(smem_raw, kb);
            wait_chunk(&bars[kb], (ph[kb] + (unsigned)(e / kSolveBufs)) & 1u, err);
            int c0, cn, ld, rows;
            const T *src;
            pl.seg(k, cur.rb, c0, cn, src, ld, rows);
            if (Q.active()) chunk_axpy(buf, rows, cn, c0, Q.q, Q.g, Q.G, phase == 0 ? fc : yv, ax, ay, az);
            __syncthreads();
            if (tid == 0 && e + kSolveBufs < vtot) {
                issue_seg(pl, iss.k, iss.rb, buf, &bars[kb]);
                iss.step(vp);
            }
            if (k == (phase == 0 ? vp.nA - 1 : vp.nA + vp.nB - 1)) {
                if (phase == 0) reduce_quads<T, false>(Q, ax, ay, az, red, yv + row0);
                else reduce_quads<T, true>(Q, ax, ay, az, red, fb + row0);
#pragma unroll
                for (int z = 0; z < 4; ++z) ax[z] = ay[z] = az[z] = (T)0;
            }
        }
    }
    for (int i = tid; i < nb; i += kSolveThreads) uvec[d.uvec_off + i] = fb[i];
    // the barrier orders every thread's writes before thread 0's release,
    // which is cumulative: a CTA that acquires the flag sees them all
    __syncthreads();
    if (tid == 0) st_release(flags + s, epoch);
    // y of this supernode's columns is read only by the backward sweep (a
    // later launch): stored after the release, off the parent's critical
    // path.
    for (int i = tid; i < nc; i += kSolveThreads) sol[d.first + i] = yv[i];
    if (y_in_f) __syncthreads();  // the next task loads its f over y
#pragma unroll
    for (int b = 0; b < kSolveBufs; ++b) ph[b] += (unsigned)((vtot - b + kSolveBufs - 1) / kSolveBufs);
    }
    pdl_wait();  // a CTA without tasks still ends after the kernel it may overlap
}

// Backward: for supernode s (root first), z = y - L21^T x(struct) and
// x(cols) = X^T z, streaming the stored transposes (L21^T: nb columns of ldx
// rows; X^T: nc columns of ldx rows). mode 0: pc64[k] = x_k;
// mode 1: pc64[k] += x_k, pc32[k] = float(pc64[k]).
template <typename T>
__global__ void __launch_bounds__(kSolveThreads, 3)
k_solve_bwd(int S, int Z, int ltop, SolveSmem lay, const int32_t *__restrict__ order, const SnInfo *__restrict__ sn,
            const int32_t *__restrict__ rows, const T *__restrict__ Xall, const T *__restrict__ L21Tall,
            Vec4<T> *__restrict__ sol, Vec4<double> *__restrict__ pc64, Vec4<float> *__restrict__ pc32, int mode,
            unsigned long long *ticket, unsigned *flags, int *err) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    Vec4<T> *zv = reinterpret_cast<Vec4<T> *>(smem_raw + kSolveBufs * kChunkBytes);
    Vec4<T> *gb = zv + lay.ldx_max;
    Vec4<T> *xv = gb;  // x takes the place of the gathered rows, read by phase A only
    T *red = reinterpret_cast<T *>(gb + max(lay.ldx_max, lay.ld21_max));
    __shared__ __align__(8) uint64_t bars[kSolveBufs];
    __shared__ int s_task[2];  // this task's and the next one's ticket (taken early)
    __shared__ unsigned s_epoch[2];
    const int tid = threadIdx.x;
    if (tid == 0) {
        for (int b = 0; b < kSolveBufs; ++b) mbar_init(&bars[b], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        next_task(ticket, S, Z, order, true, err, s_task[0], s_epoch[0]);
    }
    __syncthreads();
    unsigned ph[kSolveBufs];  // phases each chunk buffer completed in earlier tasks
#pragma unroll
    for (int b = 0; b < kSolveBufs; ++b) ph[b] = 0u;
    for (int slot = 0;; slot ^= 1) {
    const int s = s_task[slot];
    if (s < 0) break;
    const unsigned epoch = s_epoch[slot];
    const SnInfo d = sn[s];
    const int nc = d.ncol, nb = d.nrow - d.ncol;
    ChunkPlan<T> pl;
    if (nb > 0) pl.init(L21Tall + d.l21t_off, d.ldx, nb, Xall + d.xt_off, d.ldx, nc);
    else pl.init(Xall + d.xt_off, d.ldx, nc, nullptr, 0, 0);
    const int ntot = pl.total();
    const int nA = nb > 0 ? pl.nA : 0;  // chunks of L21^T
    // one pass (chunks of whole columns) or several (segments of each pass's rows)
    const int rbs = row_blocks(nc);
    const bool multi = rbs > 1;
    const int sAv = nb > 0 ? pl.sA : 0;
    const VPlan vp = multi ? VPlan{sAv, pl.sA + pl.sB - sAv, rbs, rbs} : VPlan{nA, ntot - nA, rbs, rbs};
    const int vtot = vp.total();
    VCursor iss;  // next stream position to issue (thread 0)
    iss.start(vp);
    if (tid == 0) {
        for (int e = 0; e < vtot && e < kSolveBufs; ++e, iss.step(vp)) {
            if (multi) issue_seg(pl, iss.k, iss.rb, sbuf<T>(smem_raw, e), &bars[e]);
            else issue_chunk(pl, iss.k, sbuf<T>(smem_raw, e), &bars[e]);
        }
        if (multi) prefetch_mats_l2(pl);
        else for (int k = kSolveBufs; k < ntot; ++k) prefetch_chunk_l2(pl, k);
    }
    pdl_wait();  // as in the forward sweep
    const int32_t *rs = rows + d.rows_off;
    for (int i = tid; i < d.ldx; i += kSolveThreads)
        zv[i] = (i < nc) ? sol[d.first + i] : Vec4<T>{(T)0, (T)0, (T)0, (T)0};
    int myrow[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) myrow[u] = (tid + u * kSolveThreads < nb) ? rs[tid + u * kSolveThreads] : 0;
    // a parent in the top levels was finished by the launch before this one
    if (tid == 0 && d.parent >= 0 && sn[d.parent].level < ltop) wait_flag(flags + d.parent, epoch, err);
    if (tid == 32) next_task(ticket, S, Z, order, true, err, s_task[slot ^ 1], s_epoch[slot ^ 1]);
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 4; ++u)
        if (tid + u * kSolveThreads < nb) gb[tid + u * kSolveThreads] = ldcg4(sol + myrow[u]);
    for (int i = tid + 4 * kSolveThreads; i < nb; i += kSolveThreads) gb[i] = ldcg4(sol + rs[i]);
    __syncthreads();
    // phase A (nb > 0): z -= L21^T g; phase B: x = X^T z; both have nc rows,
    // in passes of at most kSolveBlockRows rows
    T ax[4] = {0, 0, 0, 0}, ay[4] = {0, 0, 0, 0}, az[4] = {0, 0, 0, 0};
    if (!multi) {
        // both phases in one pass: the plain chunk sequence
        const Quads Q = quads_for(nc);
        for (int k = 0; k < ntot; ++k) {
            const int kb = k & (kSolveBufs - 1);
            T *buf = sbuf<T>(smem_raw, kb);
            wait_chunk(&bars[kb], (ph[kb] + (unsigned)(k / kSolveBufs)) & 1u, err);
            int c0, cn, ld;
            const T *src;
            pl.chunk(k, c0, cn, src, ld);
            const Vec4<T> *v = (k < nA) ? gb : zv;
            if (Q.active()) chunk_axpy(buf, ld, cn, c0, Q.q, Q.g, Q.G, v, ax, ay, az);
            __syncthreads();
            if (tid == 0 && k + kSolveBufs < ntot) issue_chunk(pl, k + kSolveBufs, buf, &bars[kb]);
            if (k == nA - 1) {
                reduce_quads<T, true>(Q, ax, ay, az, red, zv);
#pragma unroll
                for (int z = 0; z < 4; ++z) ax[z] = ay[z] = az[z] = (T)0;
            }
        }
        reduce_quads<T, false>(Q, ax, ay, az, red, xv);
    } else {
        VCursor cur;
        cur.start(vp);
        Quads Q;
        for (int e = 0; e < vtot; ++e, cur.step(vp)) {
            const int k = cur.k, phase = cur.phase, row0 = cur.rb * kSolveBlockRows;
            if (cur.first_of_pass(vp)) Q = quads_for(min(kSolveBlockRows, nc - row0));
            const int kb = e & (kSolveBufs - 1);
            T *buf = sbuf<T>(smem_raw, kb);
            wait_chunk(&bars[kb], (ph[kb] + (unsigned)(e / kSolveBufs)) & 1u, err);
            int c0, cn, ld, rows;
            const T *src;
            pl.seg(k, cur.rb, c0, cn, src, ld, rows);
            if (Q.active()) chunk_axpy(buf, rows, cn, c0, Q.q, Q.g, Q.G, phase == 0 ? gb : zv, ax, ay, az);
            __syncthreads();
            if (tid == 0 && e + kSolveBufs < vtot) {
                issue_seg(pl, iss.k, iss.rb, buf, &bars[kb]);
                iss.step(vp);
            }
            if (k == (phase == 0 ? vp.nA - 1 : vp.nA + vp.nB - 1)) {
                if (phase == 0) reduce_quads<T, true>(Q, ax, ay, az, red, zv + row0);
                else reduce_quads<T, false>(Q, ax, ay, az, red, xv + row0);
#pragma unroll
                for (int z = 0; z < 4; ++z) ax[z] = ay[z] = az[z] = (T)0;
            }
        }
    }
    for (int i = tid; i < nc; i += kSolveThreads) sol[d.first + i] = xv[i];
    // the barrier orders every thread's writes before thread 0's release,
    // which is cumulative: a CTA that acquires the flag sees them all
    __syncthreads();
    if (tid == 0) st_release(flags + s, epoch);
    // the positions are read by no other task of this sweep: updated after
    // the release, off the children's critical path. xv is next written
    // after a barrier of the next task.
    for (int i = tid; i < nc; i += kSolveThreads) {
        const Vec4<T> x = xv[i];
        const int k = d.first + i;
        if (mode == 0) {
            pc64[k] = {(double)x.x, (double)x.y, (double)x.z, 0.0};
        } else {
            Vec4<double> v = pc64[k];
            v.x += (double)x.x;
            v.y += (double)x.y;
            v.z += (double)x.z;
            pc64[k] = v;
            pc32[k] = {(float)v.x, (float)v.y, (float)v.z, 0.f};
        }
    }
#pragma unroll
    for (int b = 0; b < kSolveBufs; ++b) ph[b] += (unsigned)((vtot - b + kSolveBufs - 1) / kSolveBufs);
    }
    pdl_wait();  // a CTA without tasks still ends after the kernel it may overlap
}


// ---------------------------------------------------------------------------
// Top levels of the elimination tree: few supernodes with large fronts, where
// one CTA streaming its matrices is the critical path. A cluster of CL CTAs
// takes each such supernode: CTA r streams the chunks k = r, r+CL, ... of the
// task's matrices into its own shared memory and forms a partial product;
// the partials are summed through distributed shared memory in rank order
// (same order every run). Rank 0 takes the tickets (same S + G scheme, G =
// clusters) and publishes the flags. These launches run after (forward) or
// before (backward) the launch of the lower levels, so dependencies that cross
// the boundary are already met by stream order.

constexpr int kTopCluster = 8;

template <typename T, int CL>
struct TopSmem {
    // byte offsets of the vectors after the two chunk buffers
    __device__ static Vec4<T> *vec(unsigned char *raw, int k, int ldx_max, int ld21_max) {
        Vec4<T> *base = reinterpret_cast<Vec4<T> *>(raw + 2 * kChunkBytes);
        // 0: fc/zv (ldx)  1: yv/xfull (ldx)  2: fb/gb (ld21)  3: red (kRedRows)  4: part A (ldx)  5: part B (ld21 or ldx)
        const int off[6] = {0, ldx_max, 2 * ldx_max, 2 * ldx_max + ld21_max, 2 * ldx_max + ld21_max + kRedRows,
                            3 * ldx_max + ld21_max + kRedRows};
        return base + off[k];
    }
};

size_t top_smem_bytes_impl(int ldx_max, int ld21_max, int scalar_bytes) {
    return (size_t)2 * kChunkBytes +
           (size_t)(3 * ldx_max + ld21_max + kRedRows + std::max(ldx_max, ld21_max)) * 4 * scalar_bytes;
}

// my chunks are k = rank + j*CL, j = 0, 1, ...
template <typename T, int CL>
__device__ __forceinline__ void top_issue(const ChunkPlan<T> &pl, int rank, int j, T *buf0, T *buf1, uint64_t *bars) {
    const int k = rank + j * CL;
    if (k < pl.total()) issue_chunk(pl, k, (j & 1) ? buf1 : buf0, &bars[j & 1]);
}

template <typename T, int CL>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(kSolveThreads, 1)
k_solve_fwd_top(int S, int Z, int ltop, SolveSmem lay, const int32_t *__restrict__ order,
                const SnInfo *__restrict__ sn, const int32_t *__restrict__ child, const int32_t *__restrict__ relind,
                const T *__restrict__ Xall, const T *__restrict__ L21all, Vec4<T> *__restrict__ sol,
                Vec4<T> *__restrict__ uvec, unsigned long long *ticket, unsigned *flags, int *err) {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T *buf0 = reinterpret_cast<T *>(smem_raw);
    T *buf1 = reinterpret_cast<T *>(smem_raw + kChunkBytes);
    Vec4<T> *fc = TopSmem<T, CL>::vec(smem_raw, 0, lay.ldx_max, lay.ld21_max);
    Vec4<T> *yv = TopSmem<T, CL>::vec(smem_raw, 1, lay.ldx_max, lay.ld21_max);
    Vec4<T> *fb = TopSmem<T, CL>::vec(smem_raw, 2, lay.ldx_max, lay.ld21_max);
    T *red = reinterpret_cast<T *>(TopSmem<T, CL>::vec(smem_raw, 3, lay.ldx_max, lay.ld21_max));
    Vec4<T> *ypart = TopSmem<T, CL>::vec(smem_raw, 4, lay.ldx_max, lay.ld21_max);
    Vec4<T> *upart = TopSmem<T, CL>::vec(smem_raw, 5, lay.ldx_max, lay.ld21_max);
    __shared__ __align__(8) uint64_t bars[2];
    __shared__ int s_task[2];  // rank 0 holds this task's and the next one's ticket
    __shared__ unsigned s_epoch[2];
    const int tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        if (rank == 0) next_task(ticket, S, Z, order, false, err, s_task[0], s_epoch[0]);
    }
    cluster.sync();
    unsigned ph[2] = {0u, 0u};
    for (int slot = 0;; slot ^= 1) {
        const int s = cluster.map_shared_rank(s_task, 0)[slot];
        const unsigned epoch = cluster.map_shared_rank(s_epoch, 0)[slot];
        if (s < 0) {
            cluster.sync();  // rank 0 leaves only after every rank read its shared memory
            break;
        }
        const SnInfo d = sn[s];
        const int nc = d.ncol, nb = d.nrow - d.ncol;
        ChunkPlan<T> pl;
        pl.init(Xall + d.x_off, d.ldx, nc, L21all + d.l21_off, d.ld21, nb > 0 ? nc : 0);
        const int ntot = pl.total();
        const int mine = rank < ntot ? (ntot - rank + CL - 1) / CL : 0;
        if (tid == 0) {
            top_issue<T, CL>(pl, rank, 0, buf0, buf1, bars);
            top_issue<T, CL>(pl, rank, 1, buf0, buf1, bars);
            for (int j = 2; j < mine; ++j) prefetch_chunk_l2(pl, rank + j * CL);
        }
        for (int i = tid; i < d.ldx; i += kSolveThreads)
            fc[i] = (i < nc) ? sol[d.first + i] : Vec4<T>{(T)0, (T)0, (T)0, (T)0};
        for (int i = tid; i < d.ld21; i += kSolveThreads) fb[i] = {(T)0, (T)0, (T)0, (T)0};
        if (rank == 0 && tid == 0)
            for (int ci = d.child_begin; ci < d.child_end; ++ci) {
                const int c = child[ci];
                if (sn[c].level >= ltop) wait_flag(flags + c, epoch, err);
            }
        if (rank == 0 && tid == 32) next_task(ticket, S, Z, order, false, err, s_task[slot ^ 1], s_epoch[slot ^ 1]);
        cluster.sync();  // the children's update vectors are complete for every rank
        for (int ci = d.child_begin; ci < d.child_end; ++ci) {
            const SnInfo c = sn[child[ci]];
            const int nbc = c.nrow - c.ncol;
            const int32_t *ri = relind + c.relind_off;
            for (int i = tid; i < nbc; i += kSolveThreads) {
                const Vec4<T> u = ldcg4(uvec + c.uvec_off + i);
                const int pos = ri[i];
                Vec4<T> &t = pos < nc ? fc[pos] : fb[pos - nc];
                t.x += u.x;
                t.y += u.y;
                t.z += u.z;
            }
            __syncthreads();
        }
        const Quads Qa = quads_for(nc), Qb = quads_for(nb);
        T ax[4] = {0, 0, 0, 0}, ay[4] = {0, 0, 0, 0}, az[4] = {0, 0, 0, 0};
        bool a_done = false;
        for (int j = 0; j <= mine; ++j) {
            const int k = rank + j * CL;
            if (!a_done && (j == mine || k >= pl.nA)) {
                // my part of y = X fc, then the sum over the ranks
                reduce_quads<T, false>(Qa, ax, ay, az, red, ypart);
#pragma unroll
                for (int z = 0; z < 4; ++z) ax[z] = ay[z] = az[z] = (T)0;
                cluster.sync();
                for (int i = tid; i < nc; i += kSolveThreads) {
                    Vec4<T> a = {(T)0, (T)0, (T)0, (T)0};
                    for (int r = 0; r < CL; ++r) {
                        const Vec4<T> p = cluster.map_shared_rank(ypart, r)[i];
                        a.x += p.x;
                        a.y += p.y;
                        a.z += p.z;
                    }
                    yv[i] = a;
                }
                __syncthreads();
                a_done = true;
            }
            if (j == mine) break;
            T *buf = (j & 1) ? buf1 : buf0;
            wait_chunk(&bars[j & 1], (ph[j & 1] + (unsigned)(j >> 1)) & 1u, err);
            int c0, cn, ld;
            const T *src;
            pl.chunk(k, c0, cn, src, ld);
            if (k < pl.nA) {
                if (Qa.active()) chunk_axpy(buf, ld, cn, c0, Qa.q, Qa.g, Qa.G, fc, ax, ay, az);
            } else {
                if (Qb.active()) chunk_axpy(buf, ld, cn, c0, Qb.q, Qb.g, Qb.G, yv, ax, ay, az);
            }
            __syncthreads();
            if (tid == 0) top_issue<T, CL>(pl, rank, j + 2, buf0, buf1, bars);
        }
        if (nb > 0) reduce_quads<T, false>(Qb, ax, ay, az, red, upart);
        cluster.sync();  // every rank's part of L21 y is in its shared memory
        for (int i = rank * kSolveThreads + tid; i < nb; i += CL * kSolveThreads) {
            Vec4<T> u = fb[i];
            for (int r = 0; r < CL; ++r) {
                const Vec4<T> p = cluster.map_shared_rank(upart, r)[i];
                u.x -= p.x;
                u.y -= p.y;
                u.z -= p.z;
            }
            uvec[d.uvec_off + i] = u;
        }
        for (int i = rank * kSolveThreads + tid; i < nc; i += CL * kSolveThreads) sol[d.first + i] = yv[i];
        // the cluster barrier orders every rank's writes before rank 0's
        // (cumulative) release
        cluster.sync();
        if (rank == 0 && tid == 0) st_release(flags + s, epoch);
        ph[0] += (unsigned)(mine + 1) / 2u;
        ph[1] += (unsigned)mine / 2u;
    }
}

// Backward counterpart: z = y - L21^T g (g: the solution at the struct rows),
// x = X^T z, both split over the ranks by chunks and summed in rank order.
template <typename T, int CL>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(kSolveThreads, 1)
k_solve_bwd_top(int S, int Z, SolveSmem lay, const int32_t *__restrict__ order, const SnInfo *__restrict__ sn,
                const int32_t *__restrict__ rows, const T *__restrict__ Xall, const T *__restrict__ L21Tall,
                Vec4<T> *__restrict__ sol, Vec4<double> *__restrict__ pc64, Vec4<float> *__restrict__ pc32,
                int mode, unsigned long long *ticket, unsigned *flags, int *err) {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T *buf0 = reinterpret_cast<T *>(smem_raw);
    T *buf1 = reinterpret_cast<T *>(smem_raw + kChunkBytes);
    Vec4<T> *zv = TopSmem<T, CL>::vec(smem_raw, 0, lay.ldx_max, lay.ld21_max);
    Vec4<T> *zf = TopSmem<T, CL>::vec(smem_raw, 1, lay.ldx_max, lay.ld21_max);
    Vec4<T> *gb = TopSmem<T, CL>::vec(smem_raw, 2, lay.ldx_max, lay.ld21_max);
    T *red = reinterpret_cast<T *>(TopSmem<T, CL>::vec(smem_raw, 3, lay.ldx_max, lay.ld21_max));
    Vec4<T> *zpart = TopSmem<T, CL>::vec(smem_raw, 4, lay.ldx_max, lay.ld21_max);
    Vec4<T> *xpart = TopSmem<T, CL>::vec(smem_raw, 5, lay.ldx_max, lay.ld21_max);
    __shared__ __align__(8) uint64_t bars[2];
    __shared__ int s_task[2];  // rank 0 holds this task's and the next one's ticket
    __shared__ unsigned s_epoch[2];
    const int tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        if (rank == 0) next_task(ticket, S, Z, order, true, err, s_task[0], s_epoch[0]);
    }
    cluster.sync();
    unsigned ph[2] = {0u, 0u};
    for (int slot = 0;; slot ^= 1) {
        const int s = cluster.map_shared_rank(s_task, 0)[slot];
        const unsigned epoch = cluster.map_shared_rank(s_epoch, 0)[slot];
        if (s < 0) {
            cluster.sync();
            break;
        }
        const SnInfo d = sn[s];
        const int nc = d.ncol, nb = d.nrow - d.ncol;
        ChunkPlan<T> pl;
        if (nb > 0) pl.init(L21Tall + d.l21t_off, d.ldx, nb, Xall + d.xt_off, d.ldx, nc);
        else pl.init(Xall + d.xt_off, d.ldx, nc, nullptr, 0, 0);
        const int ntot = pl.total();
        const int nA = nb > 0 ? pl.nA : 0;  // chunks of L21^T
        const int mine = rank < ntot ? (ntot - rank + CL - 1) / CL : 0;
        if (tid == 0) {
            top_issue<T, CL>(pl, rank, 0, buf0, buf1, bars);
            top_issue<T, CL>(pl, rank, 1, buf0, buf1, bars);
            for (int j = 2; j < mine; ++j) prefetch_chunk_l2(pl, rank + j * CL);
        }
        for (int i = tid; i < d.ldx; i += kSolveThreads)
            zv[i] = (i < nc) ? sol[d.first + i] : Vec4<T>{(T)0, (T)0, (T)0, (T)0};
        if (rank == 0 && tid == 0 && d.parent >= 0) wait_flag(flags + d.parent, epoch, err);
        if (rank == 0 && tid == 32) next_task(ticket, S, Z, order, true, err, s_task[slot ^ 1], s_epoch[slot ^ 1]);
        cluster.sync();  // the parent's solution is complete for every rank
        const int32_t *rs = rows + d.rows_off;
        for (int i = tid; i < nb; i += kSolveThreads) gb[i] = ldcg4(sol + rs[i]);
        __syncthreads();
        const Quads Q = quads_for(nc);
        T ax[4] = {0, 0, 0, 0}, ay[4] = {0, 0, 0, 0}, az[4] = {0, 0, 0, 0};
        bool a_done = false;
        for (int j = 0; j <= mine; ++j) {
            const int k = rank + j * CL;
            if (!a_done && (j == mine || k >= nA)) {
                // z = y - sum over the ranks of their part of L21^T g
                if (nb > 0) {
                    reduce_quads<T, false>(Q, ax, ay, az, red, zpart);
#pragma unroll
                    for (int z = 0; z < 4; ++z) ax[z] = ay[z] = az[z] = (T)0;
                    cluster.sync();
                }
                for (int i = tid; i < nc; i += kSolveThreads) {
                    Vec4<T> a = zv[i];
                    if (nb > 0)
                        for (int r = 0; r < CL; ++r) {
                            const Vec4<T> p = cluster.map_shared_rank(zpart, r)[i];
                            a.x -= p.x;
                            a.y -= p.y;
                            a.z -= p.z;
                        }
                    zf[i] = a;
                }
                __syncthreads();
                a_done = true;
            }
            if (j == mine) break;
            T *buf = (j & 1) ? buf1 : buf0;
            wait_chunk(&bars[j & 1], (ph[j & 1] + (unsigned)(j >> 1)) & 1u, err);
            int c0, cn, ld;
            const T *src;
            pl.chunk(k, c0, cn, src, ld);
            const Vec4<T> *v = (k < nA) ? gb : zf;
            if (Q.active()) chunk_axpy(buf, ld, cn, c0, Q.q, Q.g, Q.G, v, ax, ay, az);
            __syncthreads();
            if (tid == 0) top_issue<T, CL>(pl, rank, j + 2, buf0, buf1, bars);
        }
        reduce_quads<T, false>(Q, ax, ay, az, red, xpart);
        cluster.sync();  // every rank's part of X^T z is in its shared memory
        for (int i = rank * kSolveThreads + tid; i < nc; i += CL * kSolveThreads) {
            Vec4<T> x = {(T)0, (T)0, (T)0, (T)0};
            for (int r = 0; r < CL; ++r) {
                const Vec4<T> p = cluster.map_shared_rank(xpart, r)[i];
                x.x += p.x;
                x.y += p.y;
                x.z += p.z;
            }
            const int kk = d.first + i;
            sol[kk] = x;
            if (mode == 0) {
                pc64[kk] = {(double)x.x, (double)x.y, (double)x.z, 0.0};
            } else {
                Vec4<double> v = pc64[kk];
                v.x += (double)x.x;
                v.y += (double)x.y;
                v.z += (double)x.z;
                pc64[kk] = v;
                pc32[kk] = {(float)v.x, (float)v.y, (float)v.z, 0.f};
            }
        }
        // the cluster barrier orders every rank's writes before rank 0's
        // (cumulative) release
        cluster.sync();
        if (rank == 0 && tid == 0) st_release(flags + s, epoch);
        ph[0] += (unsigned)(mine + 1) / 2u;
        ph[1] += (unsigned)mine / 2u;
    }
}

// ---------------------------------------------------------------------------
// Dense top of the elimination tree. The top levels hold few supernodes, and
// each is one CTA's task on the sweeps' critical path. For them the factor's
// restriction L_top (n_top <= a few thousand columns, in elimination order)
// is inverted once per factorisation, T = inv(L_top) dense; a sweep then
// solves the top in one wide launch: forward y_top = T f_top, where f_top is
// the top columns' right-hand side plus the update vectors of their children
// in the lower levels, and backward x_top = T^T y_top.

// Column block [c0, c0 + 16) of supernode j's columns of T: the forward solve
// of L_top Y = E (E the identity columns) restricted to j and its ancestors,
// supernode by supernode: Y_a = X_a F_a, U_a = F_b - L21_a Y_a, with F the
// update rows scattered into the parent's front (Y_j = X_j at the start).
template <typename T, int RC>
__global__ void __launch_bounds__(256)
k_top_inverse(const int32_t *__restrict__ items, const SnInfo *__restrict__ sn, const int32_t *__restrict__ relind,
              const int32_t *__restrict__ tdpos, const T *__restrict__ Xall, const T *__restrict__ L21all, int ldt,
              int ldx_max, int ld21_max, T *__restrict__ Tt, T *__restrict__ TTt) {
    extern __shared__ __align__(16) unsigned char top_raw[];
    // the item's kTopRhs columns in passes of RC (fewer columns per pass for
    // fronts whose buffers would not fit shared memory otherwise)
    for (int pass = 0; pass < kTopRhs / RC; ++pass) {
    T *Y = reinterpret_cast<T *>(top_raw);  // [row][RC], rows of the current supernode's columns
    T *U = Y + (size_t)ldx_max * RC;       // [row][RC], its struct rows
    T *F = U + (size_t)ld21_max * RC;      // the parent's front: columns
    T *Fb = F + (size_t)ldx_max * RC;      // and struct rows
    const int tid = threadIdx.x;
    const int j = items[2 * blockIdx.x], c0 = items[2 * blockIdx.x + 1] + pass * RC;
    const SnInfo dj = sn[j];
    if (c0 >= dj.ncol) break;
    const int w = min(RC, dj.ncol - c0);
    const int64_t dcol0 = (int64_t)tdpos[j] + c0;  // dense column of the block's first column
    // supernode j: Y = X_j[:, c0 + c]
    {
        const T *X = Xall + dj.x_off;
        for (int q = tid; q < dj.ncol * RC; q += 256) {
            const int r = q / RC, c = q % RC;
            const T v = c < w ? X[(int64_t)(c0 + c) * dj.ldx + r] : (T)0;
            Y[q] = v;
            if (c < w) {
                Tt[((int64_t)tdpos[j] + r) * ldt + dcol0 + c] = v;
                TTt[(dcol0 + c) * ldt + tdpos[j] + r] = v;
            }
        }
    }
    __syncthreads();
    int node = j;
    SnInfo dn = dj;
    for (;;) {
        // U = -L21 Y (or F_b - L21 Y below), the update rows of `node`
        const int nbn = dn.nrow - dn.ncol;
        const T *L21 = L21all + dn.l21_off;
        const bool first = node == j;
        for (int r = tid; r < nbn; r += 256) {
            T acc[RC];
#pragma unroll
            for (int c = 0; c < RC; ++c) acc[c] = first ? (T)0 : Fb[r * RC + c];
            for (int k = 0; k < dn.ncol; ++k) {
                const T l = L21[(int64_t)k * dn.ld21 + r];
#pragma unroll
                for (int c = 0; c < RC; ++c) acc[c] -= l * Y[k * RC + c];
            }
#pragma unroll
            for (int c = 0; c < RC; ++c) U[r * RC + c] = acc[c];
        }
        __syncthreads();
        if (dn.parent < 0) break;
        const int a = dn.parent;
        const SnInfo da = sn[a];
        const int nca = da.ncol, nba = da.nrow - da.ncol;
        for (int q = tid; q < (nca + nba) * RC; q += 256) (q < nca * RC ? F[q] : Fb[q - nca * RC]) = (T)0;
        __syncthreads();
        const int32_t *ri = relind + dn.relind_off;
        for (int q = tid; q < nbn * RC; q += 256) {
            const int i = q / RC, c = q % RC;
            const int pos = ri[i];
            (pos < nca ? F[pos * RC + c] : Fb[(pos - nca) * RC + c]) = U[q];
        }
        __syncthreads();
        // Y = X_a F
        const T *X = Xall + da.x_off;
        for (int r = tid; r < nca; r += 256) {
            T acc[RC];
#pragma unroll
            for (int c = 0; c < RC; ++c) acc[c] = (T)0;
            for (int k = 0; k <= r; ++k) {  // X_a is lower triangular
                const T x = X[(int64_t)k * da.ldx + r];
#pragma unroll
                for (int c = 0; c < RC; ++c) acc[c] += x * F[k * RC + c];
            }
            T *trow = Tt + ((int64_t)tdpos[a] + r) * ldt + dcol0;
#pragma unroll
            for (int c = 0; c < RC; ++c) {
                Y[r * RC + c] = acc[c];
                if (c < w) {
                    trow[c] = acc[c];
                    TTt[(dcol0 + c) * ldt + tdpos[a] + r] = acc[c];
                }
            }
        }
        __syncthreads();
        node = a;
        dn = da;
    }
    __syncthreads();  // the buffers are reused by the next pass
    }
}

// The dense top's products with T = inv(L_top) (row-major, leading dimension
// ldt, zeros above the diagonal and in the padding columns) run over
// kTopTile x kTopTile tiles of T's lower triangle, (rb, cb) with rb >= cb,
// whose partial products are stored at tile index t = rb (rb + 1) / 2 + cb.
// A CTA takes two tiles of one block column, (rb0, cb) and (rb0 + 1, cb)
// (the pairs of column cb start at rb0 = cb, cb + 2, ...; the last may be a
// single tile), so one wave covers a top of 4,096 columns. Each tile counts
// its arrival on its block's counter; the CTA that brings a block's last tile
// sums the block's partials in tile order (a fixed order: results repeat bit
// for bit) and resets the counter for the next launch. No CTA waits on
// another. When the launch overlaps the kernel before it (pdl_wait), a CTA
// loads its tiles of T and the gather's indices first (both change only with
// the factorisation) and the vectors after.

// pairs of the block columns before cb: sum over c < cb of ceil((nb - c) / 2)
__device__ __forceinline__ int top_pairs_before(int nb, int cb) {
    auto S = [](int x) { return (x + 1) * (x + 1) / 4; };  // sum_{k=1..x} ceil(k / 2)
    return S(nb) - S(nb - cb);
}
__device__ __forceinline__ void top_pair_coords(int t, int nb, int &cb, int &rb0) {
    int lo = 0, hi = nb - 1;  // the last cb with top_pairs_before(nb, cb) <= t
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (top_pairs_before(nb, mid) <= t) lo = mid;
        else hi = mid - 1;
    }
    cb = lo;
    rb0 = cb + 2 * (t - top_pairs_before(nb, cb));
}

__device__ __forceinline__ void top_tile_coords(int t, int &rb, int &cb) {
    int r = (int)((sqrtf(8.f * (float)t + 1.f) - 1.f) * 0.5f);
    while ((r + 1) * (r + 2) / 2 <= t) ++r;
    while (r * (r + 1) / 2 > t) --r;
    rb = r;
    cb = t - r * (r + 1) / 2;
}

template <typename T> __device__ __forceinline__ Vec4<T> ldg4(const T *p);
template <> __device__ __forceinline__ Vec4<float> ldg4(const float *p) {
    const float4 v = __ldg(reinterpret_cast<const float4 *>(p));
    return {v.x, v.y, v.z, v.w};
}
template <> __device__ __forceinline__ Vec4<double> ldg4(const double *p) {
    const double2 *q = reinterpret_cast<const double2 *>(p);
    const double2 a = __ldg(q), b = __ldg(q + 1);
    return {a.x, a.y, b.x, b.y};
}

template <typename T> __device__ __forceinline__ void quad_sum(T &x, T &y, T &z) {
    // the four lanes of an aligned quad end with the same sum, (a0 + a1) + (a2 + a3)
#pragma unroll
    for (int off = 1; off <= 2; off <<= 1) {
        x += __shfl_xor_sync(0xffffffffu, x, off);
        y += __shfl_xor_sync(0xffffffffu, y, off);
        z += __shfl_xor_sync(0xffffffffu, z, off);
    }
}

// p[j kTopTile] over j = q, q + 4, ... < ntiles, in order, loads eight at a time
template <typename T>
__device__ __forceinline__ void top_partial_sum(const Vec4<T> *p, int q, int ntiles, T &sx, T &sy, T &sz) {
    for (int j = q; j < ntiles; j += 32) {
        Vec4<T> u[8];
#pragma unroll
        for (int i = 0; i < 8; ++i)
            u[i] = j + 4 * i < ntiles ? ldcg4(p + (int64_t)(j + 4 * i) * kTopTile) : Vec4<T>{(T)0, (T)0, (T)0, (T)0};
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            sx += u[i].x;
            sy += u[i].y;
            sz += u[i].z;
        }
    }
}

// The pair's 2 x kTopTile rows of T, columns [c0, c0 + kTopTile) clipped to
// ldt, into shared memory by bulk copies (a thread per row, rows of kTopRow
// words: 16-byte aligned, 4 banks apart), counted on `bar`. Thread 0 has
// initialised `bar`; rows at or past n are not copied.
constexpr int kTopRow = kTopTile + 4;
template <typename T>
__device__ __forceinline__ void top_pair_copy(const T *M, int ldt, int n, int rb0, int nsub, int c0, T *Ms,
                                              uint64_t *bar) {
    const int tid = threadIdx.x, w = min(kTopTile, ldt - c0);
    const int nr = max(0, min(nsub * kTopTile, n - rb0 * kTopTile));
    if (tid == 0) mbar_expect_tx(bar, (unsigned)(nr * w * (int)sizeof(T)));
    __syncthreads();  // the expected bytes are set before any copy can complete
    if (tid < nr)
        tma_load_1d(Ms + (size_t)tid * kTopRow, M + (int64_t)(rb0 * kTopTile + tid) * ldt + c0,
                    (unsigned)(w * (int)sizeof(T)), bar);
}

// Forward, y_top = T f_top: the pair gathers f of its columns (four threads
// per column over every fourth update vector), each of its tiles multiplies
// its rows (four threads per row, 16 columns each) and adds the row sums into
// its block row (rb + 1 tiles).
template <typename T>
__global__ void __launch_bounds__(256)
k_top_pair_fwd(int n, int ldt, int nb, const T *__restrict__ M, const int32_t *__restrict__ col,
               const int32_t *__restrict__ gptr, const int64_t *__restrict__ gidx, const Vec4<T> *__restrict__ sol,
               const Vec4<T> *__restrict__ uvec, Vec4<T> *__restrict__ part, unsigned *__restrict__ cnt,
               Vec4<T> *__restrict__ ytop, int *err) {
    extern __shared__ __align__(128) unsigned char top_raw[];
    T *Ms = reinterpret_cast<T *>(top_raw);  // 2 kTopTile rows of kTopRow
    __shared__ Vec4<T> f[kTopTile];
    __shared__ __align__(8) uint64_t bar;
    __shared__ int last[2];
    pdl_trigger();
    int cb, rb0;
    top_pair_coords(blockIdx.x, nb, cb, rb0);
    const int nsub = min(2, nb - rb0);
    const int tid = threadIdx.x, q = tid & 3, c0 = cb * kTopTile, row = tid >> 2;
    const Vec4<T> zero{(T)0, (T)0, (T)0, (T)0};
    if (tid == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    top_pair_copy(M, ldt, n, rb0, nsub, c0, Ms, &bar);
    {
        // column d: thread q takes the right-hand side (q = 0) and the update
        // vectors k0 + q, k0 + q + 4, ... in order; the first two indices early
        const int d = c0 + (tid >> 2);
        int kc = -1, k0 = 0, k1 = 0;
        int64_t g0 = -1, g1 = -1;
        if (d < n) {
            if (q == 0) kc = col[d];
            k0 = gptr[d] + q;
            k1 = gptr[d + 1];
            if (k0 < k1) g0 = gidx[k0];
            if (k0 + 4 < k1) g1 = gidx[k0 + 4];
        }
        pdl_wait();
        T vx = 0, vy = 0, vz = 0;
        if (kc >= 0) {
            const Vec4<T> v = sol[kc];
            vx = v.x;
            vy = v.y;
            vz = v.z;
        }
        const Vec4<T> u0 = g0 >= 0 ? ldcg4(uvec + g0) : zero, u1 = g1 >= 0 ? ldcg4(uvec + g1) : zero;
        vx += u0.x;
        vy += u0.y;
        vz += u0.z;
        vx += u1.x;
        vy += u1.y;
        vz += u1.z;
        for (int k = k0 + 8; k < k1; k += 4) {
            const Vec4<T> u = ldcg4(uvec + gidx[k]);
            vx += u.x;
            vy += u.y;
            vz += u.z;
        }
        quad_sum(vx, vy, vz);
        if (q == 0) f[tid >> 2] = {vx, vy, vz, (T)0};
    }
    __syncthreads();
    wait_chunk(&bar, 0, err);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const T *mr = Ms + (size_t)(h * kTopTile + row) * kTopRow;
        T ax = 0, ay = 0, az = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int cl = 4 * q + 16 * k;
            if (c0 + cl >= ldt) continue;  // not copied: past the matrix
            const Vec4<T> m = *reinterpret_cast<const Vec4<T> *>(mr + cl);
            const Vec4<T> f0 = f[cl], f1 = f[cl + 1], f2 = f[cl + 2], f3 = f[cl + 3];
            ax += m.x * f0.x + m.y * f1.x + m.z * f2.x + m.w * f3.x;
            ay += m.x * f0.y + m.y * f1.y + m.z * f2.y + m.w * f3.y;
            az += m.x * f0.z + m.y * f1.z + m.z * f2.z + m.w * f3.z;
        }
        quad_sum(ax, ay, az);
        const int rb = rb0 + h;
        // rows at or past n were not copied: their sums are never read
        if (q == 0 && h < nsub) part[((int64_t)rb * (rb + 1) / 2 + cb) * kTopTile + row] = {ax, ay, az, (T)0};
    }
    __syncthreads();
    if (tid == 0)
        for (int h = 0; h < 2; ++h)
            last[h] = h < nsub && atom_add_acq_rel(cnt + rb0 + h, 1u) == (unsigned)(rb0 + h);
    __syncthreads();
    for (int h = 0; h < nsub; ++h) {
        if (!last[h]) continue;
        const int rb = rb0 + h, r = rb * kTopTile + row;
        const Vec4<T> *p = part + (int64_t)(rb * (rb + 1) / 2) * kTopTile + row;
        T sx = 0, sy = 0, sz = 0;
        top_partial_sum(p, q, rb + 1, sx, sy, sz);
        quad_sum(sx, sy, sz);
        if (q == 0 && r < n) ytop[r] = {sx, sy, sz, (T)0};
        if (tid == 0) cnt[rb] = 0;
    }
}

// Backward, x_top = T^T y_top, T read by columns: each tile of the pair adds
// sum_r T(r, c) y_r over its rows into block column cb (nb - cb tiles), a
// thread per column and row quarter (16 rows), the quarters combined in
// shared memory in a fixed order; x into the solution and the positions
// (mode 0: pc64 = x; mode 1: pc64 += x, pc32 = float(pc64)).
template <typename T>
__global__ void __launch_bounds__(256)
k_top_pair_bwd(int n, int ldt, int nb, const T *__restrict__ M, const Vec4<T> *__restrict__ ytop,
               Vec4<T> *__restrict__ part, unsigned *__restrict__ cnt, const int32_t *__restrict__ col,
               Vec4<T> *__restrict__ sol, Vec4<double> *__restrict__ pc64, Vec4<float> *__restrict__ pc32,
               int mode, int *err) {
    extern __shared__ __align__(128) unsigned char top_raw[];
    T *Ms = reinterpret_cast<T *>(top_raw);  // 2 kTopTile rows of kTopRow
    __shared__ Vec4<T> y[2][kTopTile];
    __shared__ Vec4<T> red[4][kTopTile];
    __shared__ __align__(8) uint64_t bar;
    __shared__ int last;
    pdl_trigger();
    int cb, rb0;
    top_pair_coords(blockIdx.x, nb, cb, rb0);
    const int nsub = min(2, nb - rb0);
    const int tid = threadIdx.x, c0 = cb * kTopTile;
    const int cl = tid & (kTopTile - 1), q = tid >> 6, c = c0 + cl;
    if (tid == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    top_pair_copy(M, ldt, n, rb0, nsub, c0, Ms, &bar);
    const int oc = tid >> 2, j4 = tid & 3;  // the final sum's column and tile phase (see below)
    const int kout = (j4 == 0 && c0 + oc < n) ? col[c0 + oc] : -1;
    pdl_wait();
    if (tid < 2 * kTopTile) {
        const int r = rb0 * kTopTile + tid;
        y[tid / kTopTile][tid % kTopTile] =
            (tid < nsub * kTopTile && r < n) ? ytop[r] : Vec4<T>{(T)0, (T)0, (T)0, (T)0};
    }
    __syncthreads();
    wait_chunk(&bar, 0, err);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        T ax = 0, ay = 0, az = 0;
        if (c < n) {
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const int rl = h * kTopTile + 16 * q + i;
                if (rb0 * kTopTile + rl >= n) break;  // not copied: past the matrix
                const T m = Ms[(size_t)rl * kTopRow + cl];
                const Vec4<T> v = y[h][16 * q + i];
                ax += m * v.x;
                ay += m * v.y;
                az += m * v.z;
            }
        }
        red[q][cl] = {ax, ay, az, (T)0};
        __syncthreads();
        if (tid < kTopTile && h < nsub) {
            Vec4<T> v = red[0][tid];
#pragma unroll
            for (int j = 1; j < 4; ++j) {
                v.x += red[j][tid].x;
                v.y += red[j][tid].y;
                v.z += red[j][tid].z;
            }
            const int rb = rb0 + h;
            part[((int64_t)rb * (rb + 1) / 2 + cb) * kTopTile + tid] = v;
        }
        __syncthreads();
    }
    if (tid == 0) last = atom_add_acq_rel(cnt + cb, (unsigned)nsub) + (unsigned)nsub == (unsigned)(nb - cb);
    __syncthreads();
    if (!last) return;
    // four threads per column (an aligned quad), thread j4 over the block
    // column's tiles j4, j4 + 4, ... of block rows cb, cb + 1, ..., nb - 1
    T sx = 0, sy = 0, sz = 0;
    for (int j = j4; j < nb - cb; j += 32) {
        Vec4<T> u[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int rr = cb + j + 4 * i;
            u[i] = j + 4 * i < nb - cb ? ldcg4(part + ((int64_t)rr * (rr + 1) / 2 + cb) * kTopTile + oc)
                                       : Vec4<T>{(T)0, (T)0, (T)0, (T)0};
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            sx += u[i].x;
            sy += u[i].y;
            sz += u[i].z;
        }
    }
    quad_sum(sx, sy, sz);
    if (kout >= 0) {
        const int k = kout;
        sol[k] = {sx, sy, sz, (T)0};
        if (mode == 0) {
            pc64[k] = {(double)sx, (double)sy, (double)sz, 0.0};
        } else {
            Vec4<double> p = pc64[k];
            p.x += (double)sx;
            p.y += (double)sy;
            p.z += (double)sz;
            pc64[k] = p;
            pc32[k] = {(float)p.x, (float)p.y, (float)p.z, 0.f};
        }
    }
    if (tid == 0) cnt[cb] = 0;
}

// One tile per CTA (tops whose tiles fit one wave), tile t = rb (rb + 1) / 2 + cb.
// Forward, y_top = T f_top: tile (rb, cb) gathers f of its columns (four
// threads per column over every fourth update vector), multiplies its rows
// (four threads per row, 16 columns each) and adds the row sums into block
// row rb (rb + 1 tiles).
template <typename T>
__global__ void __launch_bounds__(256)
k_top_tile_fwd(int n, int ldt, const T *__restrict__ M, const int32_t *__restrict__ col,
               const int32_t *__restrict__ gptr, const int64_t *__restrict__ gidx, const Vec4<T> *__restrict__ sol,
               const Vec4<T> *__restrict__ uvec, Vec4<T> *__restrict__ part, unsigned *__restrict__ cnt,
               Vec4<T> *__restrict__ ytop) {
    __shared__ Vec4<T> f[kTopTile];
    __shared__ int last;
    pdl_trigger();
    int rb, cb;
    top_tile_coords(blockIdx.x, rb, cb);
    const int tid = threadIdx.x, q = tid & 3, r0 = rb * kTopTile, c0 = cb * kTopTile;
    const int row = tid >> 2, r = r0 + row;
    const Vec4<T> zero{(T)0, (T)0, (T)0, (T)0};
    Vec4<T> m[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int c = c0 + 4 * q + 16 * k;  // ldt is a multiple of 4: c < ldt covers c + 3
        m[k] = (r < n && c < ldt) ? ldg4(M + (int64_t)r * ldt + c) : zero;
    }
    {
        // column d: thread q takes the right-hand side (q = 0) and the update
        // vectors k0 + q, k0 + q + 4, ... in order; the first two indices early
        const int d = c0 + (tid >> 2);
        int kc = -1, k0 = 0, k1 = 0;
        int64_t g0 = -1, g1 = -1;
        if (d < n) {
            if (q == 0) kc = col[d];
            k0 = gptr[d] + q;
            k1 = gptr[d + 1];
            if (k0 < k1) g0 = gidx[k0];
            if (k0 + 4 < k1) g1 = gidx[k0 + 4];
        }
        pdl_wait();
        T vx = 0, vy = 0, vz = 0;
        if (kc >= 0) {
            const Vec4<T> v = sol[kc];
            vx = v.x;
            vy = v.y;
            vz = v.z;
        }
        const Vec4<T> u0 = g0 >= 0 ? ldcg4(uvec + g0) : zero, u1 = g1 >= 0 ? ldcg4(uvec + g1) : zero;
        vx += u0.x;
        vy += u0.y;
        vz += u0.z;
        vx += u1.x;
        vy += u1.y;
        vz += u1.z;
        for (int k = k0 + 8; k < k1; k += 4) {
            const Vec4<T> u = ldcg4(uvec + gidx[k]);
            vx += u.x;
            vy += u.y;
            vz += u.z;
        }
        quad_sum(vx, vy, vz);
        if (q == 0) f[tid >> 2] = {vx, vy, vz, (T)0};
    }
    __syncthreads();
    T ax = 0, ay = 0, az = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int cl = 4 * q + 16 * k;
        const Vec4<T> f0 = f[cl], f1 = f[cl + 1], f2 = f[cl + 2], f3 = f[cl + 3];
        ax += m[k].x * f0.x + m[k].y * f1.x + m[k].z * f2.x + m[k].w * f3.x;
        ay += m[k].x * f0.y + m[k].y * f1.y + m[k].z * f2.y + m[k].w * f3.y;
        az += m[k].x * f0.z + m[k].y * f1.z + m[k].z * f2.z + m[k].w * f3.z;
    }
    quad_sum(ax, ay, az);
    if (q == 0) part[(int64_t)blockIdx.x * kTopTile + row] = {ax, ay, az, (T)0};
    __syncthreads();
    if (tid == 0) last = atom_add_acq_rel(cnt + rb, 1u) == (unsigned)rb;
    __syncthreads();
    if (!last) return;
    {
        const Vec4<T> *p = part + (int64_t)(rb * (rb + 1) / 2) * kTopTile + row;
        T sx = 0, sy = 0, sz = 0;
        top_partial_sum(p, q, rb + 1, sx, sy, sz);
        quad_sum(sx, sy, sz);
        if (q == 0 && r < n) ytop[r] = {sx, sy, sz, (T)0};
    }
    if (tid == 0) cnt[rb] = 0;
}

// Backward, x_top = T^T y_top, T read by columns: tile (rb, cb) adds
// sum_r T(r, c) y_r over its rows into block column cb (nb - cb tiles), a
// thread per column and row quarter (16 rows), the quarters combined in shared
// memory in a fixed order; x into the solution and the positions as above.
template <typename T>
__global__ void __launch_bounds__(256)
k_top_tile_bwd(int n, int ldt, int nb, const T *__restrict__ M, const Vec4<T> *__restrict__ ytop,
               Vec4<T> *__restrict__ part, unsigned *__restrict__ cnt, const int32_t *__restrict__ col,
               Vec4<T> *__restrict__ sol, Vec4<double> *__restrict__ pc64, Vec4<float> *__restrict__ pc32,
               int mode) {
    __shared__ Vec4<T> y[kTopTile];
    __shared__ Vec4<T> red[4][kTopTile];
    __shared__ int last;
    pdl_trigger();
    int rb, cb;
    top_tile_coords(blockIdx.x, rb, cb);
    const int tid = threadIdx.x, r0 = rb * kTopTile, c0 = cb * kTopTile;
    const int cl = tid & (kTopTile - 1), q = tid >> 6, c = c0 + cl;
    T mv[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const int r = r0 + 16 * q + i;
        mv[i] = (r < n && c < n) ? __ldg(M + (int64_t)r * ldt + c) : (T)0;
    }
    const int oc = tid >> 2, j4 = tid & 3;  // the final sum's column and tile phase (see below)
    const int kout = (j4 == 0 && c0 + oc < n) ? col[c0 + oc] : -1;
    pdl_wait();
    if (tid < kTopTile) y[tid] = (r0 + tid < n) ? ytop[r0 + tid] : Vec4<T>{(T)0, (T)0, (T)0, (T)0};
    __syncthreads();
    T ax = 0, ay = 0, az = 0;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const Vec4<T> v = y[16 * q + i];
        ax += mv[i] * v.x;
        ay += mv[i] * v.y;
        az += mv[i] * v.z;
    }
    red[q][cl] = {ax, ay, az, (T)0};
    __syncthreads();
    if (tid < kTopTile) {
        Vec4<T> v = red[0][tid];
#pragma unroll
        for (int j = 1; j < 4; ++j) {
            v.x += red[j][tid].x;
            v.y += red[j][tid].y;
            v.z += red[j][tid].z;
        }
        part[(int64_t)blockIdx.x * kTopTile + tid] = v;
    }
    __syncthreads();
    if (tid == 0) last = atom_add_acq_rel(cnt + cb, 1u) == (unsigned)(nb - cb - 1);
    __syncthreads();
    if (!last) return;
    // four threads per column (an aligned quad), thread j4 over the block
    // column's tiles j4, j4 + 4, ... of block rows cb, cb + 1, ..., nb - 1
    T sx = 0, sy = 0, sz = 0;
    for (int j = j4; j < nb - cb; j += 32) {
        Vec4<T> u[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int rr = cb + j + 4 * i;
            u[i] = j + 4 * i < nb - cb ? ldcg4(part + ((int64_t)rr * (rr + 1) / 2 + cb) * kTopTile + oc)
                                       : Vec4<T>{(T)0, (T)0, (T)0, (T)0};
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            sx += u[i].x;
            sy += u[i].y;
            sz += u[i].z;
        }
    }
    quad_sum(sx, sy, sz);
    if (kout >= 0) {
        const int k = kout;
        sol[k] = {sx, sy, sz, (T)0};
        if (mode == 0) {
            pc64[k] = {(double)sx, (double)sy, (double)sz, 0.0};
        } else {
            Vec4<double> p = pc64[k];
            p.x += (double)sx;
            p.y += (double)sy;
            p.z += (double)sz;
            pc64[k] = p;
            pc32[k] = {(float)p.x, (float)p.y, (float)p.z, 0.f};
        }
    }
    if (tid == 0) cnt[cb] = 0;
}

// ---------------------------------------------------------------------------
// ARAP energy (FP64): per vertex the rotation the local step would fit to its
// one-ring now, then sum over its entries of w |(p'_k - p'_l) - R_k (p_k - p_l)|^2.
// One partial sum per block (warp shuffles, then the warps in order), summed
// by k_sum_partials in a fixed order: the result does not depend on timing.

constexpr int kEnergyThreads = 256;

__global__ void __launch_bounds__(kEnergyThreads)
k_energy(int V, const int32_t *__restrict__ drow, const int32_t *__restrict__ dcol, const double *__restrict__ w,
         const Vec4<double> *__restrict__ p, const Vec4<double> *__restrict__ pc, double *__restrict__ partial) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double ev = 0.0;
    if (i < V) {
        const Vec4<double> pi = p[i], ci = pc[i];
        double S[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        const int e0 = drow[i], e1 = drow[i + 1];
        for (int e = e0; e < e1; ++e) {
            const int j = dcol[e];
            const double wj = w[e];
            const Vec4<double> pj = p[j], cj = pc[j];
            const double ex = wj * (pi.x - pj.x), ey = wj * (pi.y - pj.y), ez = wj * (pi.z - pj.z);
            const double fx = ci.x - cj.x, fy = ci.y - cj.y, fz = ci.z - cj.z;
            S[0][0] += ex * fx; S[0][1] += ex * fy; S[0][2] += ex * fz;
            S[1][0] += ey * fx; S[1][1] += ey * fy; S[1][2] += ey * fz;
            S[2][0] += ez * fx; S[2][1] += ez * fy; S[2][2] += ez * fz;
        }
        double R[3][3];
        rotation_from_cov(S, R);
        for (int e = e0; e < e1; ++e) {
            const int j = dcol[e];
            const Vec4<double> pj = p[j], cj = pc[j];
            const double dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            const double rx = (ci.x - cj.x) - (R[0][0] * dx + R[0][1] * dy + R[0][2] * dz);
            const double ry = (ci.y - cj.y) - (R[1][0] * dx + R[1][1] * dy + R[1][2] * dz);
            const double rz = (ci.z - cj.z) - (R[2][0] * dx + R[2][1] * dy + R[2][2] * dz);
            ev += w[e] * (rx * rx + ry * ry + rz * rz);
        }
    }
    __shared__ double warp_sum[kEnergyThreads / 32];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) ev += __shfl_down_sync(0xffffffffu, ev, off);
    if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = ev;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < kEnergyThreads / 32; ++k) t += warp_sum[k];
        partial[blockIdx.x] = t;
    }
}

// out[0] = sum of n partial sums (one block; strided per-thread sums, then a
// fixed tree)
__global__ void __launch_bounds__(kEnergyThreads) k_sum_partials(int n, const double *__restrict__ partial,
                                                                 double *__restrict__ out) {
    __shared__ double buf[kEnergyThreads];
    double t = 0.0;
    for (int k = threadIdx.x; k < n; k += kEnergyThreads) t += partial[k];
    buf[threadIdx.x] = t;
    __syncthreads();
    for (int h = kEnergyThreads / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) buf[threadIdx.x] += buf[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = buf[0];
}

// Vertex normals of a triangle mesh as OpenMesh's update_normals computes them
// for display after a deform (examples/osg_viewer.cpp:53,60-62): face normal
// = normalised (p1 - p0) x (p2 - p0), vertex normal = normalised sum of the
// normals of the faces around the vertex (summed in face order). Degenerate
// faces and vertices without faces give zero vectors.
__device__ __forceinline__ void normalize3(double &x, double &y, double &z) {
    const double n = sqrt(x * x + y * y + z * z);
    if (n > 0.0) {
        x /= n;
        y /= n;
        z /= n;
    }
}

__global__ void k_face_normals(int F, const int32_t *__restrict__ faces, const double *__restrict__ xyz,
                               double *__restrict__ fn) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= F) return;
    const double *a = xyz + 3 * (int64_t)faces[3 * f], *b = xyz + 3 * (int64_t)faces[3 * f + 1],
                 *c = xyz + 3 * (int64_t)faces[3 * f + 2];
    const double ux = b[0] - a[0], uy = b[1] - a[1], uz = b[2] - a[2];
    const double vx = c[0] - a[0], vy = c[1] - a[1], vz = c[2] - a[2];
    double nx = uy * vz - uz * vy, ny = uz * vx - ux * vz, nz = ux * vy - uy * vx;
    normalize3(nx, ny, nz);
    fn[3 * (int64_t)f] = nx;
    fn[3 * (int64_t)f + 1] = ny;
    fn[3 * (int64_t)f + 2] = nz;
}

__global__ void k_vertex_normals(int V, const int32_t *__restrict__ vf_ptr, const int32_t *__restrict__ vf_face,
                                 const double *__restrict__ fn, double *__restrict__ vn) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    double x = 0.0, y = 0.0, z = 0.0;
    for (int q = vf_ptr[v]; q < vf_ptr[v + 1]; ++q) {
        const double *n = fn + 3 * (int64_t)vf_face[q];
        x += n[0];
        y += n[1];
        z += n[2];
    }
    normalize3(x, y, z);
    vn[3 * (int64_t)v] = x;
    vn[3 * (int64_t)v + 1] = y;
    vn[3 * (int64_t)v + 2] = z;
}

__global__ void k_gather_positions(int V, const int32_t *__restrict__ oldidx, const Vec4<double> *__restrict__ pc64,
                                   double *__restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= V) return;
    const int v = oldidx[k];
    const Vec4<double> x = pc64[k];
    out[3 * (int64_t)v] = x.x;
    out[3 * (int64_t)v + 1] = x.y;
    out[3 * (int64_t)v + 2] = x.z;
}

template <typename T>
__global__ void k_gather_rotations(int V, const int32_t *__restrict__ oldidx, const Vec4<T> *__restrict__ R,
                                   double *__restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= V) return;
    const int v = oldidx[k];
    for (int r = 0; r < 3; ++r) {
        const Vec4<T> q = R[3 * (int64_t)k + r];
        out[9 * (int64_t)v + 3 * r + 0] = (double)q.x;
        out[9 * (int64_t)v + 3 * r + 1] = (double)q.y;
        out[9 * (int64_t)v + 3 * r + 2] = (double)q.z;
    }
}

inline int blocks_for(int64_t n, int t) { return (int)((n + t - 1) / t); }

// FP64 factor outputs rounded to FP32 for the solves: up to four arrays in
// one launch, four elements per thread and step (32-byte loads, 16-byte
// stores; the allocations are 256-byte aligned), grid-stride over each array.
struct DemoteJob {
    const double *src[4];
    float *dst[4];
    int64_t n[4];
};

__global__ void __launch_bounds__(256) k_demote(DemoteJob job) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
#pragma unroll 1
    for (int a = 0; a < 4; ++a) {
        const double *__restrict__ src = job.src[a];
        float *__restrict__ dst = job.dst[a];
        const int64_t n = job.n[a], n4 = n / 4;
        for (int64_t q = t0; q < n4; q += stride) {
            const Vec4<double> v = reinterpret_cast<const Vec4<double> *>(src)[q];
            reinterpret_cast<float4 *>(dst)[q] = make_float4((float)v.x, (float)v.y, (float)v.z, (float)v.w);
        }
        for (int64_t i = 4 * n4 + t0; i < n; i += stride) dst[i] = (float)src[i];
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// launch wrappers

void launch_face_cots(const DevTopo &t, const double *rest_xyz, double *hc, cudaStream_t st) {
    if (t.F == 0) return;
    k_face_cots<<<blocks_for(t.F, 256), 256, 0, st>>>(t.F, t.faces, rest_xyz, hc);
}

void launch_edge_weights(const DevTopo &t, const DevSym &s, const double *hc, double *w64, float *w32,
                         double *w_orig, cudaStream_t st) {
    if (s.nnz == 0) return;
    k_edge_weights<<<blocks_for(s.nnz, 256), 256, 0, st>>>(s.nnz, s.dent, t.ent_ptr, t.ent_fc, hc, w64, w32, w_orig);
}

void launch_edge_weights_orig(const DevTopo &t, const double *hc, double *w_orig, cudaStream_t st) {
    if (t.nnz == 0) return;
    k_edge_weights_orig<<<blocks_for(t.nnz, 256), 256, 0, st>>>(t.nnz, t.ent_ptr, t.ent_fc, hc, w_orig);
}

template <typename T>
void launch_setup_vertices(const DevSym &s, const double *rest_xyz, const double *targets_xyz,
                           Vec4<double> *p64, Vec4<double> *pc64, Vec4<T> *p_t, Vec4<T> *pc_t, Vec4<T> *R,
                           cudaStream_t st) {
    if (s.V == 0) return;
    k_setup_vertices<T><<<blocks_for(s.V, 256), 256, 0, st>>>(s.V, s.m, s.oldidx, rest_xyz, targets_xyz, p64, pc64,
                                                              p_t, pc_t, R);
}

template <typename TF>
void launch_assemble(const DevSym &s, const double *w64, const Vec4<double> *pc64, TF *Lval, double *diag64,
                     Vec4<double> *bfixed, cudaStream_t st) {
    if (s.m == 0) return;
    k_assemble<TF><<<blocks_for(s.m, 256), 256, 0, st>>>(s.m, s.drow, s.dcol, w64, s.amap, s.dmap, pc64, Lval,
                                                         diag64, bfixed);
}

void launch_bfixed(const DevSym &s, const double *w64, const Vec4<double> *pc64, Vec4<double> *bfixed,
                   cudaStream_t st) {
    if (s.m == 0) return;
    k_bfixed<<<blocks_for(s.m, 256), 256, 0, st>>>(s.m, s.drow, s.dcol, w64, pc64, bfixed);
}

void launch_rest_edges(const DevSym &s, const Vec4<double> *p64, Vec4<float> *redge, cudaStream_t st) {
    if (s.V == 0) return;
    k_rest_edges<<<blocks_for(s.V, 256), 256, 0, st>>>(s.V, s.drow, s.dcol, p64, redge);
}

// A launch with programmatic stream serialization when `overlap` is set: the
// kernel may then start while the kernel before it in the stream still runs
// (see pdl_wait); otherwise an ordinary launch.
template <typename... KArgs, typename... Args>
static void launch_pdl(void (*kern)(KArgs...), bool overlap, int grid, int block, size_t smem, cudaStream_t st,
                       Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = overlap ? 1 : 0;
    cudaLaunchKernelEx(&cfg, kern, args...);
}

void launch_local_step_mixed(const DevSym &s, const float *w32, const Vec4<float> *redge, const Vec4<double> *pc64,
                             Vec4<float> *R, const double *w64, const Vec4<double> *p64, cudaStream_t st) {
    if (s.V == 0) return;
    const VertexLaunch vl = s.vlaunch[kVertexLocal];
    const int grid = (int)(((int64_t)s.V * vl.tpv + vl.block - 1) / vl.block);
#define ARAP_LOCAL(G)                                                                                  \
    launch_pdl(k_local_step_mixed<G>, s.overlap != 0, grid, vl.block, 0, st, s.V, (const int32_t *)s.drow,  \
               (const int32_t *)s.dcol, w32, redge, pc64, R, w64, p64)
    switch (vl.tpv) {
    case 2: ARAP_LOCAL(2); break;
    case 4: ARAP_LOCAL(4); break;
    case 8: ARAP_LOCAL(8); break;
    case 32: ARAP_LOCAL(32); break;
    default: ARAP_LOCAL(1); break;
    }
#undef ARAP_LOCAL
}

void launch_rhs_mixed(const DevSym &s, const float *w32, const Vec4<float> *redge, const Vec4<float> *R,
                      Vec4<float> *b, cudaStream_t st) {
    if (s.m == 0) return;
    const VertexLaunch vl = s.vlaunch[kVertexRhs];
    const int grid = (int)(((int64_t)s.m * vl.tpv + vl.block - 1) / vl.block);
#define ARAP_RHS(G)                                                                                    \
    launch_pdl(k_rhs_mixed<G>, s.overlap != 0, grid, vl.block, 0, st, s.m, (const int32_t *)s.drow,         \
               (const int32_t *)s.dcol, w32, redge, (const Vec4<float> *)R, b)
    switch (vl.tpv) {
    case 2: ARAP_RHS(2); break;
    case 4: ARAP_RHS(4); break;
    case 8: ARAP_RHS(8); break;
    case 32: ARAP_RHS(32); break;
    default: ARAP_RHS(1); break;
    }
#undef ARAP_RHS
}

template <typename TF>
void launch_factor_step(const DevSym &s, const FactorLaunch &fl, const FItem *items, TF *Lval, TF *Upd, TF *Dinv,
                        TF *X, TF *L21, TF *L21T, int *err, cudaStream_t st) {
    if (fl.count == 0) return;
    const FItem *it = items + fl.item_off;
    switch (fl.kind) {
    case kFea: k_fea<TF><<<fl.count, kFactorThreads, 0, st>>>(it, s.sn, s.child, s.relind, Lval, Upd); break;
    case kFupd: k_fupd<TF><<<fl.count, kFactorThreads, 0, st>>>(it, fl.jb, s.sn, Lval); break;
    case kFdt: k_fdt<TF><<<fl.count, kFdtThreads, 0, st>>>(it, fl.jb, s.sn, Lval, Dinv, err); break;
    case kFrows: k_frows<TF><<<fl.count, kFactorThreads, 0, st>>>(it, fl.jb, s.sn, Lval, Dinv); break;
    case kFsyrk: k_fsyrk<TF><<<fl.count, kFactorThreads, 0, st>>>(it, s.sn, Lval, Upd); break;
    case kFx: k_fx<TF><<<fl.count, kFactorThreads, 0, st>>>(it, s.sn, Lval, Dinv, X, L21, L21T); break;
    }
}

template <typename TF>
void launch_solve_blocks(int nblocks, const int32_t *items, const int32_t *members, const SnInfo *sn,
                         const SnInfo *bsn, const int32_t *relind, const TF *Lval, TF *X, TF *L21, TF *L21T,
                         cudaStream_t st) {
    if (nblocks > 0)
        k_fx_block<TF><<<nblocks, kFactorThreads, 0, st>>>(items, members, sn, bsn, relind, Lval, X, L21, L21T);
}
template void launch_solve_blocks<float>(int, const int32_t *, const int32_t *, const SnInfo *, const SnInfo *,
                                         const int32_t *, const float *, float *, float *, float *, cudaStream_t);
template void launch_solve_blocks<double>(int, const int32_t *, const int32_t *, const SnInfo *, const SnInfo *,
                                          const int32_t *, const double *, double *, double *, double *, cudaStream_t);

template <typename T>
void launch_local_step(const DevSym &s, const T *w, const Vec4<T> *p, const Vec4<T> *pc, Vec4<T> *R,
                       cudaStream_t st) {
    if (s.V == 0) return;
    launch_pdl(k_local_step<T>, s.overlap != 0, blocks_for(s.V, 256), 256, 0, st, s.V, (const int32_t *)s.drow,
               (const int32_t *)s.dcol, w, p, pc, R);
}

template <typename T>
void launch_rhs(const DevSym &s, const T *w, const Vec4<T> *p, const Vec4<T> *R, const Vec4<T> *bfixed,
                Vec4<T> *b, cudaStream_t st) {
    if (s.m == 0) return;
    launch_pdl(k_rhs<T>, s.overlap != 0, blocks_for(s.m, 256), 256, 0, st, s.m, (const int32_t *)s.drow,
               (const int32_t *)s.dcol, w, p, R, bfixed, b);
}

void launch_residual(const DevSym &s, const double *w64, const double *diag64, const Vec4<double> *bfixed,
                     const Vec4<float> *b, const Vec4<double> *x64, Vec4<float> *r, cudaStream_t st) {
    if (s.m == 0) return;
    const VertexLaunch vl = s.vlaunch[kVertexResidual];
    const int grid = (int)(((int64_t)s.m * vl.tpv + vl.block - 1) / vl.block);
#define ARAP_RES(G)                                                                                    \
    launch_pdl(k_residual<G>, s.overlap != 0, grid, vl.block, 0, st, s.m, (const int32_t *)s.drow,          \
               (const int32_t *)s.dcol, w64, diag64, bfixed, b, x64, r)
    switch (vl.tpv) {
    case 2: ARAP_RES(2); break;
    case 4: ARAP_RES(4); break;
    case 8: ARAP_RES(8); break;
    case 32: ARAP_RES(32); break;
    default: ARAP_RES(1); break;
    }
#undef ARAP_RES
}

void launch_demote(int count, const double *const *src, float *const *dst, const int64_t *n, cudaStream_t st) {
    DemoteJob job{};
    int64_t most = 0;
    for (int a = 0; a < 4; ++a) {
        const bool use = a < count && n[a] > 0 && src[a] && dst[a];
        job.src[a] = use ? src[a] : nullptr;
        job.dst[a] = use ? dst[a] : nullptr;
        job.n[a] = use ? n[a] : 0;
        most = std::max(most, job.n[a]);
    }
    if (most == 0) return;
    static const int sms = [] {  // initialised once, thread-safe
        int dev = 0, v = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return 1;
        return v;
    }();
    const int grid = std::max(1, std::min(blocks_for((most + 3) / 4, 256), 8 * sms));
    k_demote<<<grid, 256, 0, st>>>(job);
}

size_t wsolve_smem_bytes(int scalar_bytes) { return (size_t)kWarpsPerCta * kWarpRows * 4 * scalar_bytes; }
int wsolve_max_rows() { return kWarpRows; }

cudaError_t configure_wsolve() {
    cudaError_t e = raise_smem_limit((const void *)k_wsolve_fwd<float>, (int)wsolve_smem_bytes(4));
    if (e == cudaSuccess) e = raise_smem_limit((const void *)k_wsolve_bwd<float>, (int)wsolve_smem_bytes(4));
    if (e == cudaSuccess) e = raise_smem_limit((const void *)k_wsolve_fwd<double>, (int)wsolve_smem_bytes(8));
    if (e == cudaSuccess) e = raise_smem_limit((const void *)k_wsolve_bwd<double>, (int)wsolve_smem_bytes(8));
    return e;
}

int wsolve_resident_ctas(int scalar_bytes) {
    int dev = 0, sms = 0, a = 0, b = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return 1;
    const size_t smem = wsolve_smem_bytes(scalar_bytes);
    if (scalar_bytes == 4) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_wsolve_fwd<float>, kWarpThreads, smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_wsolve_bwd<float>, kWarpThreads, smem);
    } else {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_wsolve_fwd<double>, kWarpThreads, smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_wsolve_bwd<double>, kWarpThreads, smem);
    }
    return std::max(1, std::min(a, b)) * sms;
}

int solve_chunk_bytes() { return kChunkBytes; }

size_t solve_smem_bytes(int ldx_max, int ld21_max, int scalar_bytes) {
    // forward: f [y] f_b; backward: z, then g and x in one place; then the
    // reduction scratch (3 x kRedRows scalars)
    const size_t fwd = (size_t)ldx_max + (ldx_max > kSolveBlockRows ? ldx_max : 0) + ld21_max;
    const size_t bwd = (size_t)ldx_max + std::max(ldx_max, ld21_max);
    return (size_t)kSolveBufs * kChunkBytes + (std::max(fwd, bwd) * 4 + 3 * (size_t)kRedRows) * scalar_bytes;
}


template <typename T>
void launch_solve_fwd(const DevSym &s, const T *X, const T *L21, Vec4<T> *sol, Vec4<T> *uvec,
                      unsigned long long *ticket, unsigned *flags, int *err, cudaStream_t st, const T *Ttop,
                      Vec4<T> *ytop) {
    if (s.S == 0) return;
    const SolveSmem lay{s.max_ldx, s.max_ld21};
    const size_t smem = solve_smem_bytes(s.max_ldx, s.max_ld21, sizeof(T));
    const int G = sizeof(T) == 4 ? s.solve_grid32 : s.solve_grid64;
    if (s.s_warp > 0) {
        const int WG = sizeof(T) == 4 ? s.wgrid32 : s.wgrid64;
        const int W = WG * kWarpsPerCta;
        k_wsolve_fwd<T><<<WG, kWarpThreads, wsolve_smem_bytes(sizeof(T)), st>>>(
            s.s_warp, s.s_warp + W, s.level_sn, s.sn, s.child, s.relind, X, L21, sol, uvec, ticket + 4, flags, err);
    }
    const int sb = s.s_low - s.s_warp;  // supernodes of the CTA sweep
    if (sb > 0 && s.level_launch) {
        // one launch per level: every child was solved by an earlier launch,
        // so no task waits (lbeg = l)
        for (int l = s.lwarp; l < s.ltop; ++l) {
            const int b = s.lev_ptr[l], n = s.lev_ptr[l + 1] - b;
            if (n == 0) continue;
            const SolveSmem ll{s.lev_ldx[l], s.lev_ld21[l]};
            const int Gl = sizeof(T) == 4 ? s.lev_grid32[l] : s.lev_grid64[l];
            k_solve_fwd<T><<<Gl, kSolveThreads, solve_smem_bytes(ll.ldx_max, ll.ld21_max, sizeof(T)), st>>>(
                n, n + Gl, l, ll, s.level_sn + b, s.sn, s.child, s.relind, X, L21, sol, uvec,
                ticket + kLevelTicket0 + 2 * l, flags, err);
        }
    } else if (sb > 0) {
        launch_pdl(k_solve_fwd<T>, s.overlap != 0, G, kSolveThreads, smem, st, sb, sb + G, s.lwarp, lay, (const int32_t *)(s.level_sn + s.s_warp),
                   (const SnInfo *)s.sn, (const int32_t *)s.child, (const int32_t *)s.relind, X, L21, sol, uvec,
                   ticket, flags, err);
    }
    if (s.s_top > 0) {
        const SolveSmem tlay{s.top_ldx, s.top_ld21};
        const size_t tsmem = top_smem_bytes_impl(s.top_ldx, s.top_ld21, sizeof(T));
        k_solve_fwd_top<T, kTopCluster><<<s.top_clusters * kTopCluster, kSolveThreads, tsmem, st>>>(
            s.s_top, s.s_top + s.top_clusters, s.ltop, tlay, s.level_sn + s.s_low, s.sn, s.child, s.relind, X, L21,
            sol, uvec, ticket + 2, flags, err);
    }
    if (s.n_top > 0) {
        // y_top = T f_top, f_top gathered by the tiles: one tile per CTA while
        // they fit one wave, else two (the same sums either way)
        const int ldt = dense_ld(s.n_top);
        Vec4<T> *part = ytop + ldt;
        unsigned *cnt = reinterpret_cast<unsigned *>(part + top_tiles(s.n_top) * kTopTile);
        if ((sizeof(T) == 4 ? s.top_pair32 : s.top_pair64) != 0)
            launch_pdl(k_top_pair_fwd<T>, s.overlap != 0, (int)top_pairs(s.n_top), 256, top_pair_smem(sizeof(T)),
                       st, s.n_top, ldt, top_blocks(s.n_top), Ttop, (const int32_t *)s.top_col,
                       (const int32_t *)s.top_gptr, (const int64_t *)s.top_gidx, (const Vec4<T> *)sol,
                       (const Vec4<T> *)uvec, part, cnt, ytop, err);
        else
            launch_pdl(k_top_tile_fwd<T>, s.overlap != 0, (int)top_tiles(s.n_top), 256, 0, st, s.n_top, ldt, Ttop,
                       (const int32_t *)s.top_col, (const int32_t *)s.top_gptr, (const int64_t *)s.top_gidx,
                       (const Vec4<T> *)sol, (const Vec4<T> *)uvec, part, cnt, ytop);
    }
}

template <typename T>
void launch_solve_bwd(const DevSym &s, const T *X, const T *L21T, Vec4<T> *sol, Vec4<double> *pc64,
                      Vec4<float> *pc32, int mode, unsigned long long *ticket, unsigned *flags, int *err,
                      cudaStream_t st, const T *Ttop, const Vec4<T> *ytop) {
    if (s.S == 0) return;
    const SolveSmem lay{s.max_ldx, s.max_ld21};
    if (s.n_top > 0) {
        // x_top = T^T y_top, T read by columns
        const int ldt = dense_ld(s.n_top);
        Vec4<T> *part = const_cast<Vec4<T> *>(ytop) + ldt;
        unsigned *cnt = reinterpret_cast<unsigned *>(part + top_tiles(s.n_top) * kTopTile);
        if ((sizeof(T) == 4 ? s.top_pair32 : s.top_pair64) != 0)
            launch_pdl(k_top_pair_bwd<T>, s.overlap != 0, (int)top_pairs(s.n_top), 256, top_pair_smem(sizeof(T)),
                       st, s.n_top, ldt, top_blocks(s.n_top), Ttop, ytop, part, cnt, (const int32_t *)s.top_col, sol,
                       pc64, pc32, mode, err);
        else
            launch_pdl(k_top_tile_bwd<T>, s.overlap != 0, (int)top_tiles(s.n_top), 256, 0, st, s.n_top, ldt,
                       top_blocks(s.n_top), Ttop, ytop, part, cnt, (const int32_t *)s.top_col, sol, pc64, pc32, mode);
    }
    const size_t smem = solve_smem_bytes(s.max_ldx, s.max_ld21, sizeof(T));
    const int G = sizeof(T) == 4 ? s.solve_grid32 : s.solve_grid64;
    if (s.s_top > 0) {
        const SolveSmem tlay{s.top_ldx, s.top_ld21};
        const size_t tsmem = top_smem_bytes_impl(s.top_ldx, s.top_ld21, sizeof(T));
        k_solve_bwd_top<T, kTopCluster><<<s.top_clusters * kTopCluster, kSolveThreads, tsmem, st>>>(
            s.s_top, s.s_top + s.top_clusters, tlay, s.level_sn + s.s_low, s.sn, s.rows, X, L21T, sol, pc64, pc32,
            mode, ticket + 2, flags, err);
    }
    const int sb = s.s_low - s.s_warp;
    if (sb > 0 && s.level_launch) {
        // one launch per level, root side first: every parent was solved by
        // an earlier launch, so no task waits (ltop = l + 1)
        for (int l = s.ltop - 1; l >= s.lwarp; --l) {
            const int b = s.lev_ptr[l], n = s.lev_ptr[l + 1] - b;
            if (n == 0) continue;
            const SolveSmem ll{s.lev_ldx[l], s.lev_ld21[l]};
            const int Gl = sizeof(T) == 4 ? s.lev_grid32[l] : s.lev_grid64[l];
            k_solve_bwd<T><<<Gl, kSolveThreads, solve_smem_bytes(ll.ldx_max, ll.ld21_max, sizeof(T)), st>>>(
                n, n + Gl, l + 1, ll, s.level_sn + b, s.sn, s.rows, X, L21T, sol, pc64, pc32, mode,
                ticket + kLevelTicket0 + 2 * l, flags, err);
        }
    } else if (sb > 0) {
        launch_pdl(k_solve_bwd<T>, s.overlap != 0, G, kSolveThreads, smem, st, sb, sb + G, s.ltop, lay, (const int32_t *)(s.level_sn + s.s_warp),
                   (const SnInfo *)s.sn, (const int32_t *)s.rows, X, L21T, sol, pc64, pc32, mode, ticket, flags, err);
    }
    if (s.s_warp > 0) {
        const int WG = sizeof(T) == 4 ? s.wgrid32 : s.wgrid64;
        const int W = WG * kWarpsPerCta;
        k_wsolve_bwd<T><<<WG, kWarpThreads, wsolve_smem_bytes(sizeof(T)), st>>>(
            s.s_warp, s.s_warp + W, s.lwarp, s.level_sn, s.sn, s.rows, X, L21T, sol, pc64, pc32, mode, ticket + 5,
            flags, err);
    }
}

template <typename T>
void launch_top_inverse(const DevSym &s, const T *X, const T *L21, T *Tt, cudaStream_t st) {
    if (s.n_top == 0) return;
    const int ldt = dense_ld(s.n_top);
    cudaMemsetAsync(Tt, 0, dense_top_elems(s.n_top) * sizeof(T), st);
    const int rc = dense_inverse_rhs(s.dense_ldx, s.dense_ld21, sizeof(T));
    const size_t smem = dense_inverse_smem_bytes(s.dense_ldx, s.dense_ld21, sizeof(T), rc);
    T *TT = Tt + (size_t)ldt * s.n_top;
#define ARAP_TOPINV(R)                                                                                               \
    k_top_inverse<T, R><<<s.n_top_items, 256, smem, st>>>(s.top_items, s.sn, s.relind, s.tdpos, X, L21, ldt,       \
                                                          s.dense_ldx, s.dense_ld21, Tt, TT)
    switch (rc) {
    case 16: ARAP_TOPINV(16); break;
    case 8: ARAP_TOPINV(8); break;
    case 4: ARAP_TOPINV(4); break;
    default: ARAP_TOPINV(2); break;
    }
#undef ARAP_TOPINV
}

int dense_inverse_rhs(int ldx_max, int ld21_max, int scalar_bytes) {
    for (int rc = kTopRhs; rc >= 2; rc /= 2)
        if (dense_inverse_smem_bytes(ldx_max, ld21_max, scalar_bytes, rc) <= 227 * 1024) return rc;
    return 0;
}

int dense_ld(int n) { return (n + 3) & ~3; }
int top_blocks(int n) { return (n + kTopTile - 1) / kTopTile; }
size_t top_tiles(int n) { return (size_t)top_blocks(n) * (top_blocks(n) + 1) / 2; }
size_t top_pairs(int n) { return (size_t)(top_blocks(n) + 1) * (top_blocks(n) + 1) / 4; }
size_t top_pair_smem(int scalar_bytes) { return (size_t)2 * kTopTile * kTopRow * scalar_bytes; }
size_t top_vec_bytes(int n, int scalar_bytes) {
    if (n <= 0) return 0;
    const size_t v = (size_t)4 * scalar_bytes;
    return (dense_ld(n) + top_tiles(n) * kTopTile) * v + (((size_t)top_blocks(n) * 4 + 15) & ~(size_t)15);
}
size_t dense_top_elems(int n) { return (size_t)2 * dense_ld(n) * n; }

size_t dense_inverse_smem_bytes(int ldx_max, int ld21_max, int scalar_bytes, int rc) {
    return (size_t)2 * (ldx_max + ld21_max) * rc * scalar_bytes;
}

template <typename T>
static cudaError_t raise_inverse(int bytes) {
    cudaError_t e = raise_smem_limit((const void *)k_top_inverse<T, 16>, bytes);
    if (e == cudaSuccess) e = raise_smem_limit((const void *)k_top_inverse<T, 8>, bytes);
    if (e == cudaSuccess) e = raise_smem_limit((const void *)k_top_inverse<T, 4>, bytes);
    if (e == cudaSuccess) e = raise_smem_limit((const void *)k_top_inverse<T, 2>, bytes);
    return e;
}

cudaError_t configure_dense_smem(int inv32, int inv64) {
    cudaError_t e = raise_inverse<float>(inv32);
    if (e == cudaSuccess) e = raise_inverse<double>(inv64);
    if (e == cudaSuccess) e = raise_smem_limit((const void *)k_top_pair_fwd<float>, (int)top_pair_smem(4));
    if (e == cudaSuccess) e = raise_smem_limit((const void *)k_top_pair_bwd<float>, (int)top_pair_smem(4));
    if (e == cudaSuccess) e = raise_smem_limit((const void *)k_top_pair_fwd<double>, (int)top_pair_smem(8));
    if (e == cudaSuccess) e = raise_smem_limit((const void *)k_top_pair_bwd<double>, (int)top_pair_smem(8));
    return e;
}

int energy_partials(int V) { return std::max(1, blocks_for(V, kEnergyThreads)); }

void launch_energy(const DevSym &s, const double *w64, const Vec4<double> *p64, const Vec4<double> *pc64,
                   double *partial, double *out, cudaStream_t st) {
    const int nb = energy_partials(s.V);
    k_energy<<<nb, kEnergyThreads, 0, st>>>(s.V, s.drow, s.dcol, w64, p64, pc64, partial);
    k_sum_partials<<<1, kEnergyThreads, 0, st>>>(nb, partial, out);
}

void launch_vertex_normals(int V, int F, const int32_t *faces, const int32_t *vf_ptr, const int32_t *vf_face,
                           const double *xyz, double *face_n, double *vertex_n, cudaStream_t st) {
    if (F > 0) k_face_normals<<<blocks_for(F, 256), 256, 0, st>>>(F, faces, xyz, face_n);
    if (V > 0) k_vertex_normals<<<blocks_for(V, 256), 256, 0, st>>>(V, vf_ptr, vf_face, face_n, vertex_n);
}

void launch_gather_positions(const DevSym &s, const Vec4<double> *pc64, double *out_xyz, cudaStream_t st) {
    if (s.V == 0) return;
    k_gather_positions<<<blocks_for(s.V, 256), 256, 0, st>>>(s.V, s.oldidx, pc64, out_xyz);
}

template <typename T>
void launch_gather_rotations(const DevSym &s, const Vec4<T> *R, double *out9, cudaStream_t st) {
    if (s.V == 0) return;
    k_gather_rotations<T><<<blocks_for(s.V, 256), 256, 0, st>>>(s.V, s.oldidx, R, out9);
}

// Raises, never lowers, a kernel's dynamic shared-memory limit on the current
// device. The limit belongs to the kernel, not to a context: contexts of
// different sizes in one process must not lower each other's.
cudaError_t raise_smem_limit(const void *func, int bytes) {
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, int> current;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    int &cur = current[{dev, func}];
    if (bytes <= cur) return cudaSuccess;
    e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) cur = bytes;
    return e;
}


// CTAs of the solve kernels that fit on the device at once for this dynamic
// shared memory (precision T), at least 1.
int solve_resident_ctas(int smem_bytes, int scalar_bytes) {
    int dev = 0, sms = 0, a = 0, b = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess)
        return 1;
    if (scalar_bytes == 4) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_solve_fwd<float>, kSolveThreads, smem_bytes);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_solve_bwd<float>, kSolveThreads, smem_bytes);
    } else {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_solve_fwd<double>, kSolveThreads, smem_bytes);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_solve_bwd<double>, kSolveThreads, smem_bytes);
    }
    return std::max(1, std::min(a, b) * sms);
}

int top_tile_resident_ctas(int scalar_bytes) {
    int dev = 0, sms = 0, a = 0, b = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess)
        return 1;
    if (scalar_bytes == 4) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_top_tile_fwd<float>, 256, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_top_tile_bwd<float>, 256, 0);
    } else {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_top_tile_fwd<double>, 256, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_top_tile_bwd<double>, 256, 0);
    }
    return std::max(1, std::min(a, b) * sms);
}

// Raises the dynamic shared-memory limit of the solve kernels (bytes per CTA).
cudaError_t configure_solve_smem(int bytes_f32, int bytes_f64) {
    cudaError_t e = raise_smem_limit((const void *)k_solve_fwd<float>, bytes_f32);
    if (e != cudaSuccess) return e;
    e = raise_smem_limit((const void *)k_solve_bwd<float>, bytes_f32);
    if (e != cudaSuccess || bytes_f64 <= 0) return e;
    e = raise_smem_limit((const void *)k_solve_fwd<double>, bytes_f64);
    if (e != cudaSuccess) return e;
    return raise_smem_limit((const void *)k_solve_bwd<double>, bytes_f64);
}

size_t top_smem_bytes(int ldx_max, int ld21_max, int scalar_bytes) {
    return top_smem_bytes_impl(ldx_max, ld21_max, scalar_bytes);
}

cudaError_t configure_top_smem(int bytes_f32, int bytes_f64) {
    cudaError_t e = raise_smem_limit((const void *)k_solve_fwd_top<float, kTopCluster>, bytes_f32);
    if (e != cudaSuccess) return e;
    e = raise_smem_limit((const void *)k_solve_bwd_top<float, kTopCluster>, bytes_f32);
    if (e != cudaSuccess || bytes_f64 <= 0) return e;
    e = raise_smem_limit((const void *)k_solve_fwd_top<double, kTopCluster>, bytes_f64);
    if (e != cudaSuccess) return e;
    return raise_smem_limit((const void *)k_solve_bwd_top<double, kTopCluster>, bytes_f64);
}

// explicit instantiations
template void launch_setup_vertices<float>(const DevSym &, const double *, const double *, Vec4<double> *,
                                           Vec4<double> *, Vec4<float> *, Vec4<float> *, Vec4<float> *,
                                           cudaStream_t);
template void launch_setup_vertices<double>(const DevSym &, const double *, const double *, Vec4<double> *,
                                            Vec4<double> *, Vec4<double> *, Vec4<double> *, Vec4<double> *,
                                            cudaStream_t);
template void launch_assemble<float>(const DevSym &, const double *, const Vec4<double> *, float *, double *,
                                     Vec4<double> *, cudaStream_t);
template void launch_assemble<double>(const DevSym &, const double *, const Vec4<double> *, double *, double *,
                                      Vec4<double> *, cudaStream_t);
template void launch_factor_step<float>(const DevSym &, const FactorLaunch &, const FItem *, float *, float *,
                                        float *, float *, float *, float *, int *, cudaStream_t);
template void launch_factor_step<double>(const DevSym &, const FactorLaunch &, const FItem *, double *, double *,
                                         double *, double *, double *, double *, int *, cudaStream_t);
template void launch_local_step<float>(const DevSym &, const float *, const Vec4<float> *, const Vec4<float> *,
                                       Vec4<float> *, cudaStream_t);
template void launch_local_step<double>(const DevSym &, const double *, const Vec4<double> *, const Vec4<double> *,
                                        Vec4<double> *, cudaStream_t);
template void launch_rhs<float>(const DevSym &, const float *, const Vec4<float> *, const Vec4<float> *,
                                const Vec4<float> *, Vec4<float> *, cudaStream_t);
template void launch_rhs<double>(const DevSym &, const double *, const Vec4<double> *, const Vec4<double> *,
                                 const Vec4<double> *, Vec4<double> *, cudaStream_t);
template void launch_solve_fwd<float>(const DevSym &, const float *, const float *, Vec4<float> *, Vec4<float> *,
                                      unsigned long long *, unsigned *, int *, cudaStream_t, const float *,
                                      Vec4<float> *);
template void launch_solve_fwd<double>(const DevSym &, const double *, const double *, Vec4<double> *,
                                       Vec4<double> *, unsigned long long *, unsigned *, int *, cudaStream_t,
                                       const double *, Vec4<double> *);
template void launch_solve_bwd<float>(const DevSym &, const float *, const float *, Vec4<float> *, Vec4<double> *,
                                      Vec4<float> *, int, unsigned long long *, unsigned *, int *, cudaStream_t,
                                      const float *, const Vec4<float> *);
template void launch_solve_bwd<double>(const DevSym &, const double *, const double *, Vec4<double> *,
                                       Vec4<double> *, Vec4<float> *, int, unsigned long long *, unsigned *, int *,
                                       cudaStream_t, const double *, const Vec4<double> *);
template void launch_top_inverse<float>(const DevSym &, const float *, const float *, float *, cudaStream_t);
template void launch_top_inverse<double>(const DevSym &, const double *, const double *, double *, cudaStream_t);
template void launch_gather_rotations<float>(const DevSym &, const Vec4<float> *, double *, cudaStream_t);
template void launch_gather_rotations<double>(const DevSym &, const Vec4<double> *, double *, cudaStream_t);

}  // namespace arapgpu

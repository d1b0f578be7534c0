// arap_batch.cu -- many handle poses of one mesh and constraint set in one
// pass: the mixed-precision iteration of inc/deform/arap.h:122-129 for P poses
// that share the cotan weights, the constrained Laplacian and its Cholesky
// factor (the use pattern of inc/deform/deformation_util.h:48-57, where every
// pose moves the same handles).
//
// Layout: per-vertex-per-pose arrays are vertex-major, element (k, p) at
// k * P + p, so that a supernode's rows for a tile of poses are contiguous.
// The triangular solves run one CTA per (supernode, tile of PT poses); every
// 16 KB chunk of a supernode's matrices streamed into shared memory (TMA bulk
// copies) serves PT poses.
#include "arap_kernels.h"

#include <algorithm>
#include <climits>
#include "arap_btop.cuh"
#include "arap_device.cuh"

namespace arapgpu {

namespace {

constexpr int kThreads = 256;
constexpr int kChunkBytes = 16 * 1024;
constexpr int kMaxItems = 4;  // (row quad, pose) items per thread

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void wait_flag(const unsigned *p, unsigned target, int *err) {
    const unsigned lim = flag_wait_limit(err);
    for (unsigned it = 0;; ++it) {
        if (ld_acquire(p) >= target) return;
        if (it >= lim) break;
        __nanosleep(it < 64 ? 20 : 200);
    }
    atomicOr(err, kErrTimeout);
}
__device__ __forceinline__ Vec4<float> ldcg4(const Vec4<float> *p) {
    const float4 v = __ldcg(reinterpret_cast<const float4 *>(p));
    return {v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t *bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
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
// Bounded wait; on expiry records kErrTimeout and waits once more (bounded) so
// that no copy still writes into shared memory afterwards.
__device__ __forceinline__ void wait_chunk(uint64_t *bar, unsigned parity, int *err) {
    for (unsigned it = 0; it < kSpinLimit; ++it)
        if (mbar_try_wait(bar, parity)) return;
    if (threadIdx.x == 0) atomicOr(err, kErrTimeout);
    for (unsigned it = 0; it < kSpinLimit; ++it)
        if (mbar_try_wait(bar, parity)) return;
}

// Next task of a persistent batched solve (thread 0): tasks are (supernode,
// pose tile) pairs, supernodes in `order` (reversed for the backward sweep),
// tiles inner. A launch of G CTAs over N = S*T tasks consumes exactly
// Z = N + G tickets (one per task, one per CTA that finds none left); launch e
// owns [e*Z, (e+1)*Z) and publishes epoch e + 1. After an expired wait every
// CTA leaves at its next ticket.
__device__ __forceinline__ void next_btask(unsigned long long *ticket, int S, int T, unsigned long long Z,
                                           const int32_t *order, bool reverse, const int *err, int &task,
                                           int &tile, unsigned &epoch) {
    const unsigned long long n = (unsigned long long)S * T;
    const unsigned long long t = atomicAdd(ticket, 1ull);
    const unsigned long long r = t % Z;
    const bool stop = (*(volatile const int *)err & kErrTimeout) != 0;
    if (r < n && !stop) {
        const int idx = (int)(reverse ? n - 1 - r : r);
        task = order[idx / T];
        tile = idx % T;
    } else {
        task = -1;
        tile = 0;
    }
    epoch = (unsigned)(t / Z) + 1u;
}

// Column chunks of matrix A then matrix B (both column-major, 16-byte aligned
// columns), each chunk at most kChunkBytes.
struct Chunks {
    const float *A, *B;
    int ldA, ldB, CA, CB, cwA, cwB, nA, nB;
    __device__ void init(const float *a, int lda, int ca, const float *b, int ldb, int cb) {
        A = a; B = b; ldA = lda; ldB = ldb; CA = ca; CB = cb;
        cwA = max(1, kChunkBytes / (lda * 4));
        cwB = ldb > 0 ? max(1, kChunkBytes / (ldb * 4)) : 1;
        nA = (CA + cwA - 1) / cwA;
        nB = CB > 0 ? (CB + cwB - 1) / cwB : 0;
    }
    __device__ void chunk(int k, int &c0, int &cn, const float *&src, int &ld) const {
        if (k < nA) { c0 = k * cwA; cn = min(cwA, CA - c0); src = A + (int64_t)c0 * ldA; ld = ldA; }
        else { const int j = k - nA; c0 = j * cwB; cn = min(cwB, CB - c0); src = B + (int64_t)c0 * ldB; ld = ldB; }
    }
    __device__ void issue(int k, float *buf, uint64_t *bar) const {
        int c0, cn, ld;
        const float *src;
        chunk(k, c0, cn, src, ld);
        const unsigned bytes = (unsigned)(cn * ld * 4);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                     : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_u32(buf)),
                     "l"(src), "r"(bytes), "r"(smem_u32(bar))
                     : "memory");
    }
    __device__ void prefetch(int k) const {
        int c0, cn, ld;
        const float *src;
        chunk(k, c0, cn, src, ld);
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"((unsigned)(cn * ld * 4)) : "memory");
    }
};

// acc[it][k] += sum_c M(4q+k, c) v[(c0+c)*PT + p] for the thread's items
// (item w = tid + i*kThreads -> q = w / PT, p = w % PT, w < NQ*PT).
template <int PT>
__device__ __forceinline__ void chunk_gemm(const float *buf, int ld, int cn, int c0, int NQ, const Vec4<float> *v,
                                           float acc[kMaxItems][4][3]) {
#pragma unroll
    for (int i = 0; i < kMaxItems; ++i) {
        const int w = threadIdx.x + i * kThreads;
        if (w >= NQ * PT) break;
        const int q = w / PT, p = w % PT;
        for (int c = 0; c < cn; ++c) {
            const float4 m = *reinterpret_cast<const float4 *>(buf + c * ld + 4 * q);
            const Vec4<float> f = v[(c0 + c) * PT + p];
            acc[i][0][0] += m.x * f.x; acc[i][0][1] += m.x * f.y; acc[i][0][2] += m.x * f.z;
            acc[i][1][0] += m.y * f.x; acc[i][1][1] += m.y * f.y; acc[i][1][2] += m.y * f.z;
            acc[i][2][0] += m.z * f.x; acc[i][2][1] += m.z * f.y; acc[i][2][2] += m.z * f.z;
            acc[i][3][0] += m.w * f.x; acc[i][3][1] += m.w * f.y; acc[i][3][2] += m.w * f.z;
        }
    }
}

// out[(4q+k)*PT + p] = acc (MODE 0), -= acc (MODE 1); zeroes acc.
template <int PT, int MODE>
__device__ __forceinline__ void store_items(int NQ, float acc[kMaxItems][4][3], Vec4<float> *out) {
#pragma unroll
    for (int i = 0; i < kMaxItems; ++i) {
        const int w = threadIdx.x + i * kThreads;
        if (w < NQ * PT) {
            const int q = w / PT, p = w % PT;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                Vec4<float> &o = out[(4 * q + k) * PT + p];
                if (MODE == 0) o = {acc[i][k][0], acc[i][k][1], acc[i][k][2], 0.f};
                else { o.x -= acc[i][k][0]; o.y -= acc[i][k][1]; o.z -= acc[i][k][2]; }
            }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) acc[i][k][0] = acc[i][k][1] = acc[i][k][2] = 0.f;
    }
}

struct BLayout {
    int ldx_max, ld21_max;
};

// Forward solve for a tile of PT poses of one supernode (children first).
template <int PT>
__global__ void __launch_bounds__(kThreads)
k_bsolve_fwd(int S, int T, int P, unsigned long long nz, BLayout lay, const int32_t *__restrict__ order, const SnInfo *__restrict__ sn,
             const int32_t *__restrict__ child, const int32_t *__restrict__ relind, const float *__restrict__ Xall,
             const float *__restrict__ L21all, Vec4<float> *__restrict__ sol, Vec4<float> *__restrict__ uvec,
             unsigned long long *ticket, unsigned *flags, int *err) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float *buf[2] = {reinterpret_cast<float *>(smem_raw), reinterpret_cast<float *>(smem_raw + kChunkBytes)};
    Vec4<float> *F = reinterpret_cast<Vec4<float> *>(smem_raw + 2 * kChunkBytes);
    Vec4<float> *Y = F + lay.ldx_max * PT;
    Vec4<float> *Fb = Y + lay.ldx_max * PT;
    __shared__ __align__(8) uint64_t bars[2];
    __shared__ int s_task[2], s_tile[2];  // this task's and the next one's ticket
    __shared__ unsigned s_epoch[2];
    const int tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(&bars[0]);
        mbar_init(&bars[1]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        next_btask(ticket, S, T, nz, order, false, err, s_task[0], s_tile[0], s_epoch[0]);
    }
    __syncthreads();
    unsigned ph[2] = {0u, 0u};  // phases each chunk buffer completed in earlier tasks
    for (int slot = 0;; slot ^= 1) {
    const int s = s_task[slot], tile = s_tile[slot], p0 = tile * PT;
    if (s < 0) break;
    const unsigned epoch = s_epoch[slot];
    const SnInfo d = sn[s];
    const int nc = d.ncol, nb = d.nrow - d.ncol;
    Chunks pl;
    pl.init(Xall + d.x_off, d.ldx, nc, L21all + d.l21_off, d.ld21, nb > 0 ? nc : 0);
    const int ntot = pl.nA + pl.nB;
    if (tid == 0) {
        pl.issue(0, buf[0], &bars[0]);
        if (ntot > 1) pl.issue(1, buf[1], &bars[1]);
        for (int k = 2; k < ntot; ++k) pl.prefetch(k);
    }
    for (int e = tid; e < d.ldx * PT; e += kThreads) {
        const int i = e / PT, p = e % PT;
        F[e] = (i < nc && p0 + p < P) ? sol[(int64_t)(d.first + i) * P + p0 + p] : Vec4<float>{0.f, 0.f, 0.f, 0.f};
    }
    for (int e = tid; e < d.ld21 * PT; e += kThreads) Fb[e] = {0.f, 0.f, 0.f, 0.f};
    if (tid == 0)
        for (int ci = d.child_begin; ci < d.child_end; ++ci) wait_flag(flags + (int64_t)child[ci] * T + tile, epoch, err);
    if (tid == 32) next_btask(ticket, S, T, nz, order, false, err, s_task[slot ^ 1], s_tile[slot ^ 1], s_epoch[slot ^ 1]);
    __syncthreads();
    for (int ci = d.child_begin; ci < d.child_end; ++ci) {
        const SnInfo c = sn[child[ci]];
        const int nbc = c.nrow - c.ncol;
        const int32_t *ri = relind + c.relind_off;
        for (int e = tid; e < nbc * PT; e += kThreads) {
            const int i = e / PT, p = e % PT;
            if (p0 + p >= P) continue;
            const Vec4<float> u = ldcg4(uvec + (c.uvec_off + i) * P + p0 + p);
            const int pos = ri[i];
            Vec4<float> &t = pos < nc ? F[pos * PT + p] : Fb[(pos - nc) * PT + p];
            t.x += u.x;
            t.y += u.y;
            t.z += u.z;
        }
        __syncthreads();
    }
    const int NQa = (nc + 3) >> 2, NQb = (nb + 3) >> 2;
    float acc[kMaxItems][4][3];
#pragma unroll
    for (int i = 0; i < kMaxItems; ++i)
#pragma unroll
        for (int k = 0; k < 4; ++k) acc[i][k][0] = acc[i][k][1] = acc[i][k][2] = 0.f;
    for (int k = 0; k < ntot; ++k) {
        wait_chunk(&bars[k & 1], (ph[k & 1] + (unsigned)(k >> 1)) & 1u, err);
        int c0, cn, ld;
        const float *src;
        pl.chunk(k, c0, cn, src, ld);
        if (k < pl.nA) chunk_gemm<PT>(buf[k & 1], ld, cn, c0, NQa, F, acc);
        else chunk_gemm<PT>(buf[k & 1], ld, cn, c0, NQb, Y, acc);
        __syncthreads();
        if (tid == 0 && k + 2 < ntot) pl.issue(k + 2, buf[k & 1], &bars[k & 1]);
        if (k == pl.nA - 1) {
            store_items<PT, 0>(NQa, acc, Y);
            __syncthreads();
        }
    }
    if (pl.nB > 0) {
        store_items<PT, 1>(NQb, acc, Fb);
        __syncthreads();
    }
    for (int e = tid; e < nb * PT; e += kThreads) {
        const int i = e / PT, p = e % PT;
        if (p0 + p < P) uvec[(d.uvec_off + i) * P + p0 + p] = Fb[e];
    }
    // the barrier orders every thread's writes before thread 0's release,
    // which is cumulative: a CTA that acquires the flag sees them all
    __syncthreads();
    if (tid == 0) st_release(flags + (int64_t)s * T + tile, epoch);
    // y of the columns is read only by the backward sweep (a later launch):
    // stored after the release; Y is next written after a barrier
    for (int e = tid; e < nc * PT; e += kThreads) {
        const int i = e / PT, p = e % PT;
        if (p0 + p < P) sol[(int64_t)(d.first + i) * P + p0 + p] = Y[e];
    }
    ph[0] += (unsigned)(ntot + 1) / 2u;
    ph[1] += (unsigned)ntot / 2u;
    }
}

// Backward solve for a tile of PT poses of one supernode (root first); adds the
// correction to the FP64 positions and refreshes their FP32 copy.
template <int PT>
__global__ void __launch_bounds__(kThreads)
k_bsolve_bwd(int S, int T, int P, unsigned long long nz, int lend, BLayout lay, const int32_t *__restrict__ order, const SnInfo *__restrict__ sn,
             const int32_t *__restrict__ rows, const float *__restrict__ Xall, const float *__restrict__ L21Tall,
             Vec4<float> *__restrict__ sol, Vec4<double> *__restrict__ pc64, Vec4<float> *__restrict__ pc32,
             unsigned long long *ticket, unsigned *flags, int *err) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float *buf[2] = {reinterpret_cast<float *>(smem_raw), reinterpret_cast<float *>(smem_raw + kChunkBytes)};
    Vec4<float> *Z = reinterpret_cast<Vec4<float> *>(smem_raw + 2 * kChunkBytes);
    Vec4<float> *Xv = Z + lay.ldx_max * PT;
    Vec4<float> *G = Xv + lay.ldx_max * PT;
    __shared__ __align__(8) uint64_t bars[2];
    __shared__ int s_task[2], s_tile[2];  // this task's and the next one's ticket
    __shared__ unsigned s_epoch[2];
    const int tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(&bars[0]);
        mbar_init(&bars[1]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        next_btask(ticket, S, T, nz, order, true, err, s_task[0], s_tile[0], s_epoch[0]);
    }
    __syncthreads();
    unsigned ph[2] = {0u, 0u};  // phases each chunk buffer completed in earlier tasks
    for (int slot = 0;; slot ^= 1) {
    const int s = s_task[slot], tile = s_tile[slot], p0 = tile * PT;
    if (s < 0) break;
    const unsigned epoch = s_epoch[slot];
    const SnInfo d = sn[s];
    const int nc = d.ncol, nb = d.nrow - d.ncol;
    Chunks pl;
    if (nb > 0) pl.init(L21Tall + d.l21t_off, d.ldx, nb, Xall + d.xt_off, d.ldx, nc);
    else pl.init(Xall + d.xt_off, d.ldx, nc, nullptr, 0, 0);
    const int ntot = pl.nA + pl.nB;
    const int nA = nb > 0 ? pl.nA : 0;
    if (tid == 0) {
        pl.issue(0, buf[0], &bars[0]);
        if (ntot > 1) pl.issue(1, buf[1], &bars[1]);
        for (int k = 2; k < ntot; ++k) pl.prefetch(k);
    }
    for (int e = tid; e < d.ldx * PT; e += kThreads) {
        const int i = e / PT, p = e % PT;
        Z[e] = (i < nc && p0 + p < P) ? sol[(int64_t)(d.first + i) * P + p0 + p] : Vec4<float>{0.f, 0.f, 0.f, 0.f};
    }
    const int32_t *rs = rows + d.rows_off;
    // a parent at level lend or above (the dense top) was solved by the launch before this one
    if (tid == 0 && d.parent >= 0 && sn[d.parent].level < lend) wait_flag(flags + (int64_t)d.parent * T + tile, epoch, err);
    if (tid == 32) next_btask(ticket, S, T, nz, order, true, err, s_task[slot ^ 1], s_tile[slot ^ 1], s_epoch[slot ^ 1]);
    __syncthreads();
    for (int e = tid; e < nb * PT; e += kThreads) {
        const int i = e / PT, p = e % PT;
        G[e] = (p0 + p < P) ? ldcg4(sol + (int64_t)rs[i] * P + p0 + p) : Vec4<float>{0.f, 0.f, 0.f, 0.f};
    }
    __syncthreads();
    const int NQ = (nc + 3) >> 2;
    float acc[kMaxItems][4][3];
#pragma unroll
    for (int i = 0; i < kMaxItems; ++i)
#pragma unroll
        for (int k = 0; k < 4; ++k) acc[i][k][0] = acc[i][k][1] = acc[i][k][2] = 0.f;
    for (int k = 0; k < ntot; ++k) {
        wait_chunk(&bars[k & 1], (ph[k & 1] + (unsigned)(k >> 1)) & 1u, err);
        int c0, cn, ld;
        const float *src;
        pl.chunk(k, c0, cn, src, ld);
        chunk_gemm<PT>(buf[k & 1], ld, cn, c0, NQ, (k < nA) ? G : Z, acc);
        __syncthreads();
        if (tid == 0 && k + 2 < ntot) pl.issue(k + 2, buf[k & 1], &bars[k & 1]);
        if (k == nA - 1) {
            store_items<PT, 1>(NQ, acc, Z);  // z = y - L21^T g
            __syncthreads();
        }
    }
    store_items<PT, 0>(NQ, acc, Xv);  // x = X^T z
    __syncthreads();
    for (int e = tid; e < nc * PT; e += kThreads) {
        const int i = e / PT, p = e % PT;
        if (p0 + p < P) sol[(int64_t)(d.first + i) * P + p0 + p] = Xv[e];
    }
    // the barrier orders every thread's writes before thread 0's release,
    // which is cumulative: a CTA that acquires the flag sees them all
    __syncthreads();
    if (tid == 0) st_release(flags + (int64_t)s * T + tile, epoch);
    // the positions are read by no other task of this sweep: updated after
    // the release; Xv is next written after a barrier
    for (int e = tid; e < nc * PT; e += kThreads) {
        const int i = e / PT, p = e % PT;
        if (p0 + p >= P) continue;
        const int64_t k = (int64_t)(d.first + i) * P + p0 + p;
        const Vec4<float> x = Xv[e];
        Vec4<double> v = pc64[k];
        v.x += (double)x.x;
        v.y += (double)x.y;
        v.z += (double)x.z;
        pc64[k] = v;
        pc32[k] = {(float)v.x, (float)v.y, (float)v.z, 0.f};
    }
    ph[0] += (unsigned)(ntot + 1) / 2u;
    ph[1] += (unsigned)ntot / 2u;
    }
}

// ---------------------------------------------------------------------------
// per (vertex, pose) kernels; thread index = k * P + p

// initializeMeshGeometry + initializeConstraints (arap.h:162-168,277-281) per
// pose: free vertices at rest, constrained ones at the pose's targets
// (targets: P x nc x 3, constrained vertices in ascending order); R = I.
__global__ void k_bsetup(int V, int m, int P, const Vec4<double> *__restrict__ p64,
                         const double *__restrict__ targets, Vec4<double> *__restrict__ pc64,
                         Vec4<float> *__restrict__ pc32, Vec4<float> *__restrict__ R) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)V * P) return;
    const int k = (int)(t / P), p = (int)(t % P);
    Vec4<double> v = p64[k];
    if (k >= m) {
        const double *g = targets + ((int64_t)p * (V - m) + (k - m)) * 3;
        v = {g[0], g[1], g[2], 0.0};
    }
    pc64[t] = v;
    pc32[t] = {(float)v.x, (float)v.y, (float)v.z, 0.f};
    R[3 * t + 0] = {1.f, 0.f, 0.f, 0.f};
    R[3 * t + 1] = {0.f, 1.f, 0.f, 0.f};
    R[3 * t + 2] = {0.f, 0.f, 1.f, 0.f};
}

// bFixed per pose (arap.h:325-327), adjacency order as in k_assemble
__global__ void k_bbfixed(int m, int P, const int32_t *__restrict__ drow, const int32_t *__restrict__ dcol,
                          const double *__restrict__ w64, const Vec4<double> *__restrict__ pc64,
                          Vec4<double> *__restrict__ bfixed) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)m * P) return;
    const int k = (int)(t / P), p = (int)(t % P);
    double bx = 0.0, by = 0.0, bz = 0.0;
    for (int e = drow[k]; e < drow[k + 1]; ++e) {
        const int l = dcol[e];
        if (l < m) continue;
        const double w = w64[e];
        const Vec4<double> c = pc64[(int64_t)l * P + p];
        bx = __dadd_rn(bx, __dmul_rn(w, c.x));
        by = __dadd_rn(by, __dmul_rn(w, c.y));
        bz = __dadd_rn(bz, __dmul_rn(w, c.z));
    }
    bfixed[t] = {bx, by, bz, 0.0};
}

// estimateRotations per pose (arap.h:354-384): FP32 covariance from the FP32
// rest edges and the pose's current edges differenced in FP64
__global__ void __launch_bounds__(256)
k_blocal(int V, int P, const int32_t *__restrict__ drow, const int32_t *__restrict__ dcol, const float *__restrict__ w,
         const Vec4<float> *__restrict__ redge, const Vec4<double> *__restrict__ pc64, Vec4<float> *__restrict__ R,
         const double *__restrict__ w64, const Vec4<double> *__restrict__ p64) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)V * P) return;
    const int i = (int)(t / P), p = (int)(t % P);
    const Vec4<double> ci = pc64[t];
    float S[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int e = drow[i]; e < drow[i + 1]; ++e) {
        const float wj = w[e];
        const Vec4<float> re = redge[e];
        const Vec4<double> cj = pc64[(int64_t)dcol[e] * P + p];
        const float ex = wj * re.x, ey = wj * re.y, ez = wj * re.z;
        const float fx = (float)(ci.x - cj.x), fy = (float)(ci.y - cj.y), fz = (float)(ci.z - cj.z);
        S[0][0] += ex * fx; S[0][1] += ex * fy; S[0][2] += ex * fz;
        S[1][0] += ey * fx; S[1][1] += ey * fy; S[1][2] += ey * fz;
        S[2][0] += ez * fx; S[2][1] += ez * fy; S[2][2] += ez * fz;
    }
    float Rm[3][3], spread;
    dev::rotation_from_cov<float>(S, Rm, &spread);
    if (!(spread >= dev::kPolarFallback)) dev::rotation_fp64<false>(i, drow[i], drow[i + 1], dcol, w64, p64, pc64, P, p, Rm);
    R[3 * t + 0] = {Rm[0][0], Rm[0][1], Rm[0][2], 0.f};
    R[3 * t + 1] = {Rm[1][0], Rm[1][1], Rm[1][2], 0.f};
    R[3 * t + 2] = {Rm[2][0], Rm[2][1], Rm[2][2], 0.f};
}

// estimatePositions RHS terms per pose (arap.h:395-414), bFixed added in FP64
// by the residual
__global__ void __launch_bounds__(256)
k_brhs(int m, int P, const int32_t *__restrict__ drow, const int32_t *__restrict__ dcol, const float *__restrict__ w,
       const Vec4<float> *__restrict__ redge, const Vec4<float> *__restrict__ R, Vec4<float> *__restrict__ b) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)m * P) return;
    const int i = (int)(t / P), p = (int)(t % P);
    const Vec4<float> r0 = R[3 * t], r1 = R[3 * t + 1], r2 = R[3 * t + 2];
    float ax = 0.f, ay = 0.f, az = 0.f;
    for (int e = drow[i]; e < drow[i + 1]; ++e) {
        const int j = dcol[e];
        if (j == i) continue;
        const float h = w[e] * 0.5f;
        const Vec4<float> d = redge[e];
        const int64_t tj = (int64_t)j * P + p;
        const Vec4<float> q0 = R[3 * tj], q1 = R[3 * tj + 1], q2 = R[3 * tj + 2];
        ax += ((r0.x + q0.x) * d.x + (r0.y + q0.y) * d.y + (r0.z + q0.z) * d.z) * h;
        ay += ((r1.x + q1.x) * d.x + (r1.y + q1.y) * d.y + (r1.z + q1.z) * d.z) * h;
        az += ((r2.x + q2.x) * d.x + (r2.y + q2.y) * d.y + (r2.z + q2.z) * d.z) * h;
    }
    b[t] = {ax, ay, az, 0.f};
}

// r = b - A x in FP64 per pose
__global__ void __launch_bounds__(256)
k_bresidual(int m, int P, const int32_t *__restrict__ drow, const int32_t *__restrict__ dcol,
            const double *__restrict__ w64, const double *__restrict__ diag64, const Vec4<double> *__restrict__ bfixed,
            const Vec4<float> *__restrict__ b, const Vec4<double> *__restrict__ x, Vec4<float> *__restrict__ r) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)m * P) return;
    const int i = (int)(t / P), p = (int)(t % P);
    const Vec4<double> xi = x[t];
    const double dg = diag64[i];
    double ax = dg * xi.x, ay = dg * xi.y, az = dg * xi.z;
    for (int e = drow[i]; e < drow[i + 1]; ++e) {
        const int j = dcol[e];
        if (j == i || j >= m) continue;
        const double wj = w64[e];
        const Vec4<double> xj = x[(int64_t)j * P + p];
        ax -= wj * xj.x;
        ay -= wj * xj.y;
        az -= wj * xj.z;
    }
    const Vec4<float> bi = b[t];
    const Vec4<double> bf = bfixed[t];
    r[t] = {(float)((bf.x + (double)bi.x) - ax), (float)((bf.y + (double)bi.y) - ay),
            (float)((bf.z + (double)bi.z) - az), 0.f};
}

// positions of every pose back to vertex order: out[p][v][3]
__global__ void k_bgather(int V, int P, const int32_t *__restrict__ oldidx, const Vec4<double> *__restrict__ pc64,
                          double *__restrict__ out) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)V * P) return;
    const int k = (int)(t / P), p = (int)(t % P);
    const Vec4<double> x = pc64[t];
    double *o = out + ((int64_t)p * V + oldidx[k]) * 3;
    o[0] = x.x;
    o[1] = x.y;
    o[2] = x.z;
}

inline int nblocks(int64_t n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

// ---------------------------------------------------------------------------

bool batch_pose_tile_fits(int max_ldx, int max_ld21, int pt) {
    if (pt != 1 && pt != 2 && pt != 4 && pt != 8 && pt != 16) return false;
    const int rows = max_ldx > max_ld21 ? max_ldx : max_ld21;
    const size_t smem = batch_solve_smem_bytes(max_ldx, max_ld21, pt);
    return ((rows + 3) / 4) * pt <= kMaxItems * kThreads && smem <= 200 * 1024;
}

int batch_pose_tile(int max_ldx, int max_ld21) {
    for (int pt = 16; pt >= 1; pt /= 2)
        if (batch_pose_tile_fits(max_ldx, max_ld21, pt)) return pt;
    return 0;
}

size_t batch_solve_smem_bytes(int max_ldx, int max_ld21, int pt) {
    return (size_t)2 * kChunkBytes + (size_t)(2 * max_ldx + max_ld21) * pt * sizeof(Vec4<float>);
}

template <int PT>
static cudaError_t configure_pt(size_t bytes) {
    cudaError_t e = raise_smem_limit((const void *)k_bsolve_fwd<PT>, (int)bytes);
    if (e != cudaSuccess) return e;
    return raise_smem_limit((const void *)k_bsolve_bwd<PT>, (int)bytes);
}

// the tensor-core products of the dense top: shared memory above the default
// (per device)
static cudaError_t configure_btop() {
    const cudaError_t a = raise_smem_limit((const void *)btop::k_btop_mma<false>, btop::kSmemBytes);
    if (a != cudaSuccess) return a;
    return raise_smem_limit((const void *)btop::k_btop_mma<true>, btop::kSmemBytes);
}

cudaError_t configure_batch_smem(int max_ldx, int max_ld21, int pt) {
    const cudaError_t eb = configure_btop();
    if (eb != cudaSuccess) return eb;
    const size_t bytes = batch_solve_smem_bytes(max_ldx, max_ld21, pt);
    switch (pt) {
    case 16: return configure_pt<16>(bytes);
    case 8: return configure_pt<8>(bytes);
    case 4: return configure_pt<4>(bytes);
    case 2: return configure_pt<2>(bytes);
    default: return configure_pt<1>(bytes);
    }
}

// DeformationUtil::updateConstraints (inc/deform/deformation_util.h:48-57) for
// P poses at once: constrained vertex i of pose p (ascending vertex order) is
// tabs_p * rest(v) for a handle, its arap_set_constraints target otherwise.
// tabs_p = origin * t_p * origin^-1 as a row-major 3x4 affine matrix.
__global__ void k_pose_targets(int P, int nc, const int32_t *__restrict__ cidx, const uint8_t *__restrict__ handle,
                               const double *__restrict__ rest, const double *__restrict__ ctgt,
                               const double *__restrict__ tabs, double *__restrict__ out) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (int64_t)P * nc) return;
    const int p = (int)(q / nc), i = (int)(q % nc);
    double *o = out + 3 * q;
    if (!handle[i]) {
        o[0] = ctgt[3 * i];
        o[1] = ctgt[3 * i + 1];
        o[2] = ctgt[3 * i + 2];
        return;
    }
    const double *x = rest + 3 * (int64_t)cidx[i];
    const double *M = tabs + 12 * (int64_t)p;
#pragma unroll
    for (int r = 0; r < 3; ++r)
        o[r] = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(M[4 * r], x[0]), __dmul_rn(M[4 * r + 1], x[1])),
                                   __dmul_rn(M[4 * r + 2], x[2])),
                         M[4 * r + 3]);
}

void launch_pose_targets(int P, int nc, const int32_t *cidx, const uint8_t *handle, const double *rest,
                         const double *ctgt, const double *tabs, double *out, cudaStream_t st) {
    const int64_t n = (int64_t)P * nc;
    if (n) k_pose_targets<<<nblocks(n, 256), 256, 0, st>>>(P, nc, cidx, handle, rest, ctgt, tabs, out);
}

void launch_bsetup(const DevSym &s, int P, const Vec4<double> *p64, const double *targets, Vec4<double> *pc64,
                   Vec4<float> *pc32, Vec4<float> *R, cudaStream_t st) {
    const int64_t n = (int64_t)s.V * P;
    if (n) k_bsetup<<<nblocks(n, 256), 256, 0, st>>>(s.V, s.m, P, p64, targets, pc64, pc32, R);
}

void launch_bbfixed(const DevSym &s, int P, const double *w64, const Vec4<double> *pc64, Vec4<double> *bfixed,
                    cudaStream_t st) {
    const int64_t n = (int64_t)s.m * P;
    if (n) k_bbfixed<<<nblocks(n, 256), 256, 0, st>>>(s.m, P, s.drow, s.dcol, w64, pc64, bfixed);
}

void launch_blocal(const DevSym &s, int P, const float *w32, const Vec4<float> *redge, const Vec4<double> *pc64,
                   Vec4<float> *R, const double *w64, const Vec4<double> *p64, cudaStream_t st) {
    const int64_t n = (int64_t)s.V * P;
    if (n) k_blocal<<<nblocks(n, 256), 256, 0, st>>>(s.V, P, s.drow, s.dcol, w32, redge, pc64, R, w64, p64);
}

void launch_brhs(const DevSym &s, int P, const float *w32, const Vec4<float> *redge, const Vec4<float> *R,
                 Vec4<float> *b, cudaStream_t st) {
    const int64_t n = (int64_t)s.m * P;
    if (n) k_brhs<<<nblocks(n, 256), 256, 0, st>>>(s.m, P, s.drow, s.dcol, w32, redge, R, b);
}

void launch_bresidual(const DevSym &s, int P, const double *w64, const double *diag64, const Vec4<double> *bfixed,
                      const Vec4<float> *b, const Vec4<double> *x, Vec4<float> *r, cudaStream_t st) {
    const int64_t n = (int64_t)s.m * P;
    if (n) k_bresidual<<<nblocks(n, 256), 256, 0, st>>>(s.m, P, s.drow, s.dcol, w64, diag64, bfixed, b, x, r);
}

void launch_bgather(const DevSym &s, int P, const Vec4<double> *pc64, double *out, cudaStream_t st) {
    const int64_t n = (int64_t)s.V * P;
    if (n) k_bgather<<<nblocks(n, 256), 256, 0, st>>>(s.V, P, s.oldidx, pc64, out);
}

// CTAs of a persistent batched solve: the tasks, at most what fits on the
// device at once (both sweeps' occupancy at this pose tile's shared memory).
template <int PT>
static int resident_bsolve(size_t smem) {
    int dev = 0, sms = 0, a = 0, b = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess)
        return 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_bsolve_fwd<PT>, kThreads, smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_bsolve_bwd<PT>, kThreads, smem);
    return std::max(1, std::min(a, b) * sms);
}

int batch_grid(const DevSym &s, int P, int pt) {
    const size_t smem = batch_solve_smem_bytes(s.max_ldx, s.max_ld21, pt);
    const int T = (P + pt - 1) / pt;
    int res = 1;
    switch (pt) {
    case 16: res = resident_bsolve<16>(smem); break;
    case 8: res = resident_bsolve<8>(smem); break;
    case 4: res = resident_bsolve<4>(smem); break;
    case 2: res = resident_bsolve<2>(smem); break;
    default: res = resident_bsolve<1>(smem); break;
    }
    const long long ntask = (long long)batch_tasks(s) * T;
    return (int)std::max(1LL, std::min<long long>(ntask, res));
}

template <int PT>
static void bsolve(const DevSym &s, int P, int grid, const float *X, const float *L21, const float *L21T, Vec4<float> *sol,
                   Vec4<float> *uvec, Vec4<double> *pc64, Vec4<float> *pc32, unsigned long long *ticket,
                   unsigned *flags, int *err, bool forward, cudaStream_t st) {
    const int T = (P + PT - 1) / PT;
    const int Sb = batch_tasks(s);
    if (Sb == 0) return;
    const BLayout lay{s.max_ldx, s.max_ld21};
    const size_t smem = batch_solve_smem_bytes(s.max_ldx, s.max_ld21, PT);
    const unsigned long long Z = (unsigned long long)Sb * T + grid;
    if (forward)
        k_bsolve_fwd<PT><<<grid, kThreads, smem, st>>>(Sb, T, P, Z, lay, s.level_sn, s.sn, s.child, s.relind, X,
                                                       L21, sol, uvec, ticket, flags, err);
    else
        k_bsolve_bwd<PT><<<grid, kThreads, smem, st>>>(Sb, T, P, Z, s.n_top > 0 ? s.ltop : INT_MAX, lay, s.level_sn,
                                                       s.sn, s.rows, X, L21T, sol, pc64, pc32, ticket, flags, err);
}

// ---------------------------------------------------------------------------
// dense top for many poses (arap_btop.cuh)

size_t btop_workspace_floats(int n, int P) { return (size_t)btop::ws_floats(n, P); }

size_t btop_matrix_floats(int n, int P) { return (size_t)btop::b_tile_floats(n, btop::ldb_of(P)); }
size_t btop_atile_floats(int n) { return (size_t)btop::a_tile_floats(n); }

void launch_btop_pack(const DevSym &s, const float *Ttop, float *atiles, cudaStream_t st) {
    const int n = s.n_top;
    if (n <= 0) return;
    const int ldt = dense_ld(n), nrt = btop::row_tiles(n);
    const unsigned max_stages = (unsigned)((n + btop::kDepth - 1) / btop::kDepth);
    btop::k_btop_pack<false><<<dim3(max_stages, nrt), 256, 0, st>>>(n, ldt, Ttop, atiles);
    btop::k_btop_pack<true><<<dim3(max_stages, nrt), 256, 0, st>>>(
        n, ldt, Ttop + (size_t)ldt * n, atiles + (size_t)btop::stages_before(false, n, nrt) * btop::kATileFloats);
}

int batch_tasks(const DevSym &s) { return s.n_top > 0 ? s.s_low : s.s_sched; }

int batch_top_launches(const DevSym &s) { return s.n_top > 0 ? 5 : 0; }

void launch_bsolve(const DevSym &s, int P, int pt, int grid, const float *X, const float *L21, const float *L21T,
                   Vec4<float> *sol, Vec4<float> *uvec, Vec4<double> *pc64, Vec4<float> *pc32,
                   unsigned long long *ticket, unsigned *flags, int *err, bool forward, cudaStream_t st,
                   const float *atiles, float *bftop, float *bytop, float *bws) {
    if (s.S == 0) return;
    const int n = s.n_top, ldb = btop::ldb_of(P);
    const int nrt = btop::row_tiles(n), nct = (ldb + btop::kCols - 1) / btop::kCols;
    const unsigned rblocks = (unsigned)(((int64_t)n * (ldb / 4) + 255) / 256);
    const unsigned pblocks = (unsigned)(((int64_t)n * P + 255) / 256);
    if (!forward && n > 0) {
        btop::k_btop_mma<true><<<dim3(nct, btop::tasks(true, n, nrt)), btop::kThreads, btop::kSmemBytes, st>>>(
            n, ldb, atiles, bytop, bws, btop::kCoreK, btop::kCoreMN, err);
        btop::k_btop_reduce_bwd<<<pblocks, 256, 0, st>>>(n, P, ldb, bws, s.top_col, sol, pc64, pc32);
    }
    switch (pt) {
    case 16: bsolve<16>(s, P, grid, X, L21, L21T, sol, uvec, pc64, pc32, ticket, flags, err, forward, st); break;
    case 8: bsolve<8>(s, P, grid, X, L21, L21T, sol, uvec, pc64, pc32, ticket, flags, err, forward, st); break;
    case 4: bsolve<4>(s, P, grid, X, L21, L21T, sol, uvec, pc64, pc32, ticket, flags, err, forward, st); break;
    case 2: bsolve<2>(s, P, grid, X, L21, L21T, sol, uvec, pc64, pc32, ticket, flags, err, forward, st); break;
    default: bsolve<1>(s, P, grid, X, L21, L21T, sol, uvec, pc64, pc32, ticket, flags, err, forward, st); break;
    }
    if (forward && n > 0) {
        btop::k_btop_gather<<<pblocks, 256, 0, st>>>(n, P, ldb, s.top_col, s.top_gptr, s.top_gidx, sol, uvec, bftop);
        btop::k_btop_mma<false><<<dim3(nct, btop::tasks(false, n, nrt)), btop::kThreads, btop::kSmemBytes, st>>>(
            n, ldb, atiles, bftop, bws, btop::kCoreK, btop::kCoreMN, err);
        btop::k_btop_reduce_fwd<<<rblocks, 256, 0, st>>>(n, ldb, bws, bytop);
    }
}

}  // namespace arapgpu

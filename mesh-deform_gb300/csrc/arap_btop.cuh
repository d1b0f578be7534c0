// arap_btop.cuh -- the dense top of the elimination tree for many poses at
// once (the top levels of the triangular solves of inc/deform/arap.h:417-429,
// solved through T = inv(L_top)).
//
// The top's right-hand sides form an n x 3P matrix (row d: the xyz of every
// pose, packed; rows padded to ldb floats, a multiple of 4). The forward
// sweep's Y = T F and the backward sweep's X = T^T Y are products with the
// triangular T on the 5th-generation tensor cores (tcgen05, kind::tf32, the
// accumulator in tensor memory). FP32 accuracy is kept by splitting every
// operand into a TF32 head and the TF32 rest (x = hi + lo) and summing
// lo*hi + hi*lo + hi*hi (the lo*lo term, below 2^-22 of the product, is left
// out). Each row tile of 128 rows reads only T's triangle, cut into splits of
// kSplit columns; one CTA computes one (row tile, split, 256 columns) partial
// product, and a second kernel sums a row's partials in split order (the same
// order for every run, pose tile and pose count) and applies the sweep's
// epilogue.
#pragma once

#include <cstdint>

#include "arap_btop_plan.h"
#include "arap_kernels.h"

namespace arapgpu {
namespace btop {

constexpr int kThreads = 256;
constexpr uint32_t kTmemCols = 256;  // the fp32 accumulator: 128 lanes x 256 columns

// Operands in shared memory, K-major without swizzle: core matrices of 8 rows
// x 16 bytes (4 floats) stored as 128 contiguous bytes; the core matrices of
// one 8-row group follow each other along k (kCoreK bytes apart), the 8-row
// groups are kCoreMN bytes apart.
constexpr uint32_t kCoreK = 128, kCoreMN = (kDepth / 4) * 128;
constexpr int kAFloats = kRows * kDepth, kBFloats = kCols * kDepth;
constexpr int kSmemBytes = (2 * kAFloats + 2 * kBFloats) * 4 + 1024;  // hi and lo of each, alignment slack

// byte offset of element (r, k) of an operand tile (r: row of M or column of
// the right-hand sides, k: column of T within the stage)
__device__ __forceinline__ uint32_t tile_off(int r, int k) {
    return (uint32_t)(r >> 3) * kCoreMN + (uint32_t)(k >> 2) * kCoreK + (uint32_t)(r & 7) * 16u + (uint32_t)(k & 3) * 4u;
}

__device__ __forceinline__ uint32_t s_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start address, leading-dimension byte
// offset (between core matrices along k), stride byte offset (between 8-row
// groups), descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor of kind::tf32: fp32 accumulator, TF32 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(s_addr(bar))
                 : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ bool bar_try_wait(uint64_t *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(s_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for a phase of the MMA barrier; false after kSpinLimit tries.
__device__ __forceinline__ bool bar_wait(uint64_t *bar, unsigned parity) {
    for (unsigned it = 0; it < kSpinLimit; ++it)
        if (bar_try_wait(bar, parity)) return true;
    return false;
}

// 16 consecutive accumulator columns of this thread's lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// x = hi + lo, hi = x with the low 13 mantissa bits cleared (exact in TF32)
__device__ __forceinline__ void split_tf32(float x, float &hi, float &lo) {
    hi = __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
    lo = x - hi;
}

// F[d][3p + c] = the top's right-hand side of pose p: its solution entry plus
// the update vectors of the lower children (gptr/gidx, a CSR per top row)
__global__ void __launch_bounds__(256)
k_btop_gather(int n, int P, int ldb, const int32_t *__restrict__ col, const int32_t *__restrict__ gptr,
              const int64_t *__restrict__ gidx, const Vec4<float> *__restrict__ sol,
              const Vec4<float> *__restrict__ uvec, float *__restrict__ F) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (int64_t)n * P) return;
    const int d = (int)(q / P), p = (int)(q % P);
    Vec4<float> v = sol[(int64_t)col[d] * P + p];
    for (int k = gptr[d]; k < gptr[d + 1]; ++k) {
        const Vec4<float> u = uvec[gidx[k] * P + p];
        v.x += u.x;
        v.y += u.y;
        v.z += u.z;
    }
    float *row = F + (int64_t)d * ldb;
    row[3 * p] = v.x;
    row[3 * p + 1] = v.y;
    row[3 * p + 2] = v.z;
    if (p == P - 1)
        for (int c = 3 * P; c < ldb; ++c) row[c] = 0.f;
}

// One partial product: rows [i0, i0+128) of M (n x n, row-major, leading
// dimension ldt, a multiple of 4, zero past column n) times rows [k_lo, k_hi)
// of B (n x ldb), columns [c0, c0+256), into ws[task] (128 x ldb, ws_at). Per stage
// of 32 columns of M: all threads load and split the tiles into shared
// memory, thread 0 issues 12 MMAs (4 steps of K = 8, three products each)
// and commits them to an mbarrier; the next stage is loaded into registers
// meanwhile, and the tiles are rewritten once that phase completes.
// lbo / sbo: kCoreK / kCoreMN. Waits are bounded: on expiry the CTA records
// kErrTimeout, writes nothing, frees its tensor memory and returns.
template <bool UPPER>
__global__ void __launch_bounds__(kThreads, 2)
k_btop_mma(int n, int ldt, int ldb, const float *__restrict__ M, const float *__restrict__ B, float *__restrict__ ws,
           uint32_t lbo, uint32_t sbo, int *err) {
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_slot;
    unsigned char *base = smem_raw + ((1024u - (s_addr(smem_raw) & 1023u)) & 1023u);
    float *Ahi = reinterpret_cast<float *>(base), *Alo = Ahi + kAFloats;
    float *Bhi = Alo + kAFloats, *Blo = Bhi + kBFloats;
    const int task = blockIdx.y;
    int rt, k_lo, k_hi;
    task_of(UPPER, n, task, rt, k_lo, k_hi);
    const int i0 = rt * kRows, c0 = blockIdx.x * kCols;
    const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(s_addr(&tmem_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(s_addr(&bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = tmem_slot;
    constexpr uint32_t idesc = idesc_tf32(kRows, kCols);

    // the next stage's tiles are loaded into registers while the tensor cores
    // multiply the current one
    constexpr int kAU = kAFloats / 4 / kThreads, kBU = kBFloats / 4 / kThreads;
    float4 ra[kAU], rb[kBU];
    auto gload = [&](int k0) {
        // M: 8 rows x 4 float4 per warp and step (64 contiguous bytes per row)
#pragma unroll
        for (int u = 0; u < kAU; ++u) {
            const int idx = tid + u * kThreads, wc = idx / 32, ln = idx % 32;
            const int r = (wc % (kRows / 8)) * 8 + (ln % 8), k4 = ln / 8 + 4 * (wc / (kRows / 8));
            const int i = i0 + r, ka = k0 + 4 * k4;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (i < n && ka < k_hi) {  // ka + 3 < ldt: ka and ldt are multiples of 4
                v = *reinterpret_cast<const float4 *>(M + (int64_t)i * ldt + ka);
                if (ka + 1 >= k_hi) v.y = 0.f;
                if (ka + 2 >= k_hi) v.z = 0.f;
                if (ka + 3 >= k_hi) v.w = 0.f;
            }
            ra[u] = v;
        }
        // B: column c0 + tid, 4 rows per step (coalesced along the columns)
        const int c = c0 + tid;
#pragma unroll
        for (int u = 0; u < kBU; ++u) {
            const int kr = k0 + 4 * u;
            const float *src = B + (int64_t)kr * ldb + c;
            const bool cin = c < ldb;
            rb[u].x = (cin && kr < k_hi) ? src[0] : 0.f;
            rb[u].y = (cin && kr + 1 < k_hi) ? src[ldb] : 0.f;
            rb[u].z = (cin && kr + 2 < k_hi) ? src[2 * (int64_t)ldb] : 0.f;
            rb[u].w = (cin && kr + 3 < k_hi) ? src[3 * (int64_t)ldb] : 0.f;
        }
    };
    // split into TF32 heads and rests, stored in the MMA layout (a quarter
    // warp stores one 128-byte core matrix)
    auto sstore = [&] {
#pragma unroll
        for (int u = 0; u < kAU; ++u) {
            const int idx = tid + u * kThreads, wc = idx / 32, ln = idx % 32;
            const int r = (wc % (kRows / 8)) * 8 + (ln % 8), k4 = ln / 8 + 4 * (wc / (kRows / 8));
            float4 h, l;
            split_tf32(ra[u].x, h.x, l.x);
            split_tf32(ra[u].y, h.y, l.y);
            split_tf32(ra[u].z, h.z, l.z);
            split_tf32(ra[u].w, h.w, l.w);
            const uint32_t o = tile_off(r, 4 * k4);
            *reinterpret_cast<float4 *>(reinterpret_cast<unsigned char *>(Ahi) + o) = h;
            *reinterpret_cast<float4 *>(reinterpret_cast<unsigned char *>(Alo) + o) = l;
        }
#pragma unroll
        for (int u = 0; u < kBU; ++u) {
            float4 h, l;
            split_tf32(rb[u].x, h.x, l.x);
            split_tf32(rb[u].y, h.y, l.y);
            split_tf32(rb[u].z, h.z, l.z);
            split_tf32(rb[u].w, h.w, l.w);
            const uint32_t o = tile_off(tid, 4 * u);
            *reinterpret_cast<float4 *>(reinterpret_cast<unsigned char *>(Bhi) + o) = h;
            *reinterpret_cast<float4 *>(reinterpret_cast<unsigned char *>(Blo) + o) = l;
        }
    };

    bool ok = true;
    int stage = 0;
    gload(k_lo);
    for (int k0 = k_lo; k0 < k_hi; k0 += kDepth, ++stage) {
        sstore();
        // the tensor cores read shared memory through the async proxy
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            fence_after_sync();
            const uint32_t ah = s_addr(Ahi), al = s_addr(Alo), bh = s_addr(Bhi), bl = s_addr(Blo);
#pragma unroll
            for (int j = 0; j < kDepth / 8; ++j) {
                const uint32_t o = (uint32_t)j * 2u * kCoreK;  // K = 8: two core matrices along k
                mma_tf32(tmem, smem_desc(al + o, lbo, sbo), smem_desc(bh + o, lbo, sbo), idesc,
                         (stage > 0 || j > 0) ? 1u : 0u);
                mma_tf32(tmem, smem_desc(ah + o, lbo, sbo), smem_desc(bl + o, lbo, sbo), idesc, 1u);
                mma_tf32(tmem, smem_desc(ah + o, lbo, sbo), smem_desc(bh + o, lbo, sbo), idesc, 1u);
            }
            mma_commit(&bar);
        }
        if (k0 + kDepth < k_hi) gload(k0 + kDepth);
        // every thread waits for this stage's products before the tiles are
        // rewritten (or the accumulator read)
        const bool done = bar_wait(&bar, (unsigned)stage & 1u);
        if (__syncthreads_or(!done)) {
            ok = false;
            break;
        }
    }
    fence_after_sync();
    if (ok) {
        const int lane_base = 32 * (warp % 4), cbase = (warp / 4) * (kCols / 2), r = lane_base + lane;
#pragma unroll 1
        for (int ch = 0; ch < kCols / 2 / 16; ++ch) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)lane_base << 16) + (uint32_t)(cbase + ch * 16), v);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int c = c0 + cbase + ch * 16 + 4 * q;
                if (c < ldb)
                    *reinterpret_cast<float4 *>(ws + ws_at(task, r, c, ldb)) =
                        make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
            }
        }
    } else {
        if (tid == 0) atomicOr(err, kErrTimeout);
        // one more bounded wait, so that no product is still running when the
        // tensor memory is freed
        if (tid == 0) bar_wait(&bar, (unsigned)(stage & 1));
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        fence_after_sync();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
    }
}

// Sums a row's partial products in split order. Forward: Y (n x ldb), one
// float4 per thread, consecutive threads on consecutive rows (the partials'
// order).
__global__ void __launch_bounds__(256)
k_btop_reduce_fwd(int n, int ldb, const float *__restrict__ ws, float *__restrict__ Y) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (int64_t)n * (ldb / 4)) return;
    const int c = (int)(q / n) * 4, i = (int)(q % n), rt = i / kRows, r = i - rt * kRows;
    const int t0 = tasks(false, n, rt), ns = splits(false, n, rt);
    float4 acc = *reinterpret_cast<const float4 *>(ws + ws_at(t0, r, c, ldb));
    for (int k = 1; k < ns; ++k) {
        const float4 v = *reinterpret_cast<const float4 *>(ws + ws_at(t0 + k, r, c, ldb));
        acc.x += v.x;
        acc.y += v.y;
        acc.z += v.z;
        acc.w += v.w;
    }
    *reinterpret_cast<float4 *>(Y + (int64_t)i * ldb + c) = acc;
}

// Backward, one (top row, pose) per thread, consecutive threads on
// consecutive rows: x of that top column stored into the solution and added
// to the positions (pc32 = float(pc64)).
__global__ void __launch_bounds__(256)
k_btop_reduce_bwd(int n, int P, int ldb, const float *__restrict__ ws, const int32_t *__restrict__ col,
                  Vec4<float> *__restrict__ sol, Vec4<double> *__restrict__ pc64, Vec4<float> *__restrict__ pc32) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (int64_t)n * P) return;
    const int p = (int)(q / n), i = (int)(q % n), rt = i / kRows, r = i - rt * kRows;
    const int t0 = tasks(true, n, rt), ns = splits(true, n, rt);
    float x = ws[ws_at(t0, r, 3 * p, ldb)], y = ws[ws_at(t0, r, 3 * p + 1, ldb)], z = ws[ws_at(t0, r, 3 * p + 2, ldb)];
    for (int k = 1; k < ns; ++k) {
        x += ws[ws_at(t0 + k, r, 3 * p, ldb)];
        y += ws[ws_at(t0 + k, r, 3 * p + 1, ldb)];
        z += ws[ws_at(t0 + k, r, 3 * p + 2, ldb)];
    }
    const int64_t e = (int64_t)col[i] * P + p;
    sol[e] = {x, y, z, 0.f};
    Vec4<double> v = pc64[e];
    v.x += (double)x;
    v.y += (double)y;
    v.z += (double)z;
    pc64[e] = v;
    pc32[e] = {(float)v.x, (float)v.y, (float)v.z, 0.f};
}

}  // namespace btop
}  // namespace arapgpu

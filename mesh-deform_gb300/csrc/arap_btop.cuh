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
//
// Both operands reach shared memory by TMA bulk copies, already split and in
// the MMA's layout: T's tiles are split and laid out once per batched deform
// (k_btop_pack, T changes only with the factorisation), the right-hand sides
// are written split and tiled by the kernels that produce them (the gather
// and the forward reduction). A CTA's stages go through two buffers: the copy
// of stage s + 1 runs while the tensor cores multiply stage s.
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
constexpr int kStageBytes = (kATileFloats + kBTileFloats) * 4;  // A and B tiles, head and rest of each
constexpr int kSmemBytes = 2 * kStageBytes + 1024;                // two stage buffers, alignment slack

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

__device__ __forceinline__ void bar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(s_addr(bar)), "r"(bytes) : "memory");
}

// bulk copy global -> shared (16-byte aligned, bytes a multiple of 16) counted on bar
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     s_addr(dst)),
                 "l"(src), "r"(bytes), "r"(s_addr(bar))
                 : "memory");
}

// x = hi + lo, hi = x with the low 13 mantissa bits cleared (exact in TF32)
__device__ __forceinline__ void split_tf32(float x, float &hi, float &lo) {
    hi = __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
    lo = x - hi;
}

// Entry (d, c) of an n x ldb right-hand side matrix into its B tile, split:
// head at the MMA layout's offset, rest kBFloats further. Entries never
// written (rows past n, columns past 3P) stay zero from the buffer's clearing.
__device__ __forceinline__ void put_b(float *Bt, int ldb, int d, int c, float x) {
    float *tile = Bt + b_tile_at(d / kDepth, c / kCols, ldb);
    const uint32_t o = tile_off(c % kCols, d % kDepth) / 4u;
    float h, l;
    split_tf32(x, h, l);
    tile[o] = h;
    tile[kBFloats + o] = l;
}

// F[d][3p + c] = the top's right-hand side of pose p: its solution entry plus
// the update vectors of the lower children (gptr/gidx, a CSR per top row),
// written split into F's B tiles
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
    put_b(F, ldb, d, 3 * p, v.x);
    put_b(F, ldb, d, 3 * p + 1, v.y);
    put_b(F, ldb, d, 3 * p + 2, v.z);
}

// T (UPPER: T^T) split and laid out as A tiles, row tile by row tile, the
// stages of a row tile in column order: CTA (stage, row tile), columns past
// the row tile's range zero.
template <bool UPPER>
__global__ void __launch_bounds__(256)
k_btop_pack(int n, int ldt, const float *__restrict__ M, float *__restrict__ At) {
    const int rt = blockIdx.y;
    int kb, ke;
    krange(UPPER, n, rt, kb, ke);
    const int st = blockIdx.x;
    if (kb + st * kDepth >= ke) return;
    const int k0 = kb + st * kDepth;
    float *tile = At + (int64_t)(stages_before(UPPER, n, rt) + st) * kATileFloats;
    for (int q = threadIdx.x; q < kRows * (kDepth / 4); q += blockDim.x) {
        const int r = q / (kDepth / 4), k4 = q % (kDepth / 4);
        const int i = rt * kRows + r, ka = k0 + 4 * k4;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (i < n && ka < ke) {  // ka + 3 < ldt: ka and ldt are multiples of 4
            v = *reinterpret_cast<const float4 *>(M + (int64_t)i * ldt + ka);
            if (ka + 1 >= ke) v.y = 0.f;
            if (ka + 2 >= ke) v.z = 0.f;
            if (ka + 3 >= ke) v.w = 0.f;
        }
        float4 h, l;
        split_tf32(v.x, h.x, l.x);
        split_tf32(v.y, h.y, l.y);
        split_tf32(v.z, h.z, l.z);
        split_tf32(v.w, h.w, l.w);
        const uint32_t o = tile_off(r, 4 * k4) / 4u;
        *reinterpret_cast<float4 *>(tile + o) = h;
        *reinterpret_cast<float4 *>(tile + kAFloats + o) = l;
    }
}

// One partial product: rows [i0, i0+128) of T (UPPER: T^T) times rows
// [k_lo, k_hi) of B, columns [c0, c0+256), into ws[task] (128 x ldb, ws_at).
// Thread 0 drives the pipeline: the bulk copies of each stage's A tile
// (32 KB) and B tile (64 KB) into one of two buffers, counted on that
// buffer's `full` barrier; once they land, 12 MMAs (4 steps of K = 8, three
// products each) committed to the buffer's `done` barrier, whose completion
// frees the buffer for the stage after next. At: both directions' A tiles
// (forward first); Bt: B's tiles. lbo / sbo: kCoreK / kCoreMN. Waits are
// bounded: on expiry the CTA records kErrTimeout, waits (bounded) for its
// copies and products in flight, writes nothing, frees its tensor memory and
// returns.
template <bool UPPER>
__global__ void __launch_bounds__(kThreads, 1)
k_btop_mma(int n, int ldb, const float *__restrict__ At, const float *__restrict__ Bt, float *__restrict__ ws,
           uint32_t lbo, uint32_t sbo, int *err) {
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full[2], done[2], drain;
    __shared__ uint32_t tmem_slot;
    __shared__ int s_ok;
    unsigned char *base = smem_raw + ((1024u - (s_addr(smem_raw) & 1023u)) & 1023u);
    const int task = blockIdx.y;
    int rt, k_lo, k_hi;
    task_of(UPPER, n, task, rt, k_lo, k_hi);
    int kb_rt, ke_rt;
    krange(UPPER, n, rt, kb_rt, ke_rt);
    const int ns = (k_hi - k_lo + kDepth - 1) / kDepth;
    const int ct = blockIdx.x, c0 = ct * kCols;
    const float *Ad = At + (UPPER ? (int64_t)stages_before(false, n, row_tiles(n)) * kATileFloats : 0) +
                      (int64_t)(stages_before(UPPER, n, rt) + (k_lo - kb_rt) / kDepth) * kATileFloats;
    const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(s_addr(&tmem_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (uint64_t *b : {&full[0], &full[1], &done[0], &done[1], &drain})
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(s_addr(b)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = tmem_slot;

    if (tid == 0) {
        constexpr uint32_t idesc = idesc_tf32(kRows, kCols);
        auto load = [&](int st, int b) {
            unsigned char *buf = base + b * kStageBytes;
            bar_expect_tx(&full[b], (uint32_t)kStageBytes);
            bulk_load(buf, Ad + (int64_t)st * kATileFloats, kATileFloats * 4u, &full[b]);
            bulk_load(buf + kATileFloats * 4, Bt + b_tile_at(k_lo / kDepth + st, ct, ldb), kBTileFloats * 4u,
                      &full[b]);
        };
        bool ok = true;
        int loaded = 0, multiplied = 0;  // stages whose copies / products were issued
        load(0, 0);
        loaded = 1;
        if (ns > 1) {
            load(1, 1);
            loaded = 2;
        }
        for (int st = 0; st < ns; ++st) {
            const int b = st & 1;
            if (!bar_wait(&full[b], (unsigned)(st >> 1) & 1u)) {
                ok = false;
                break;
            }
            fence_after_sync();
            const uint32_t ah = s_addr(base + b * kStageBytes), al = ah + kAFloats * 4u;
            const uint32_t bh = ah + kATileFloats * 4u, bl = bh + kBFloats * 4u;
#pragma unroll
            for (int j = 0; j < kDepth / 8; ++j) {
                const uint32_t o = (uint32_t)j * 2u * kCoreK;  // K = 8: two core matrices along k
                mma_tf32(tmem, smem_desc(al + o, lbo, sbo), smem_desc(bh + o, lbo, sbo), idesc,
                         (st > 0 || j > 0) ? 1u : 0u);
                mma_tf32(tmem, smem_desc(ah + o, lbo, sbo), smem_desc(bl + o, lbo, sbo), idesc, 1u);
                mma_tf32(tmem, smem_desc(ah + o, lbo, sbo), smem_desc(bh + o, lbo, sbo), idesc, 1u);
            }
            mma_commit(&done[b]);
            multiplied = st + 1;
            if (st + 2 < ns) {
                // the buffer is free once this stage's products are done
                if (!bar_wait(&done[b], (unsigned)(st >> 1) & 1u)) {
                    ok = false;
                    break;
                }
                load(st + 2, b);
                loaded = st + 3;
            }
        }
        // the last stage's products (a commit covers every earlier MMA too)
        if (ok && !bar_wait(&done[(ns - 1) & 1], (unsigned)((ns - 1) >> 1) & 1u)) ok = false;
        if (!ok) {
            atomicOr(err, kErrTimeout);
            // no copy or product may still run when the CTA leaves: wait
            // (bounded) for every copy issued and for all products issued
            for (int st = multiplied; st < loaded; ++st) bar_wait(&full[st & 1], (unsigned)(st >> 1) & 1u);
            if (multiplied > 0) {
                mma_commit(&drain);
                bar_wait(&drain, 0u);
            }
        }
        s_ok = ok ? 1 : 0;
    }
    __syncthreads();
    fence_after_sync();
    if (s_ok) {
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
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        fence_after_sync();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
    }
}

// Sums a row's partial products in split order. Forward: Y (n x ldb, the
// backward product's right-hand sides, written split into its B tiles), one
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
    put_b(Y, ldb, i, c, acc.x);
    put_b(Y, ldb, i, c + 1, acc.y);
    put_b(Y, ldb, i, c + 2, acc.z);
    put_b(Y, ldb, i, c + 3, acc.w);
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

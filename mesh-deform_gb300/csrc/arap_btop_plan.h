// arap_btop_plan.h -- the task plan of the dense top's products for many
// poses (arap_btop.cuh): how the triangle of T = inv(L_top) is cut into
// (row tile, split) tasks, and where a task's partial product lives. Plain
// C++ shared by the kernels, the host launch code and the host tests.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define ARAP_BTOP_HD __host__ __device__
#else
#define ARAP_BTOP_HD
#endif

#ifndef ARAP_BTOP_SPLIT
#define ARAP_BTOP_SPLIT 256
#endif

namespace arapgpu {
namespace btop {

constexpr int kRows = 128;               // rows of T per task: the MMA's M
constexpr int kCols = 256;               // columns of the right-hand sides per CTA: the MMA's N
constexpr int kDepth = 32;               // columns of T per stage: 4 MMAs of K = 8
constexpr int kSplit = ARAP_BTOP_SPLIT;  // columns of T per task (a multiple of kDepth)
static_assert(kSplit % kDepth == 0, "a split is a whole number of stages");

// floats per row of the packed right-hand sides: xyz of P poses, padded to 4
ARAP_BTOP_HD inline int ldb_of(int P) { return (3 * P + 3) & ~3; }

ARAP_BTOP_HD inline int row_tiles(int n) { return (n + kRows - 1) / kRows; }

// columns [kb, ke) of T's rows in row tile rt that the product reads: the
// lower triangle up to the tile's last row (forward, T) or the upper one from
// its first row (backward, T^T)
ARAP_BTOP_HD inline void krange(bool upper, int n, int rt, int &kb, int &ke) {
    kb = upper ? rt * kRows : 0;
    ke = upper ? n : ((rt + 1) * kRows < n ? (rt + 1) * kRows : n);
}

ARAP_BTOP_HD inline int splits(bool upper, int n, int rt) {
    int kb, ke;
    krange(upper, n, rt, kb, ke);
    return (ke - kb + kSplit - 1) / kSplit;
}

// tasks (row tile, split) of the row tiles before rt_end, row tile by row
// tile, splits in increasing column order
ARAP_BTOP_HD inline int tasks(bool upper, int n, int rt_end) {
    int t = 0;
    for (int rt = 0; rt < rt_end && rt * kRows < n; ++rt) t += splits(upper, n, rt);
    return t;
}

// the row tile and split of task `task`, and the columns [k_lo, k_hi) of T
// it reads
ARAP_BTOP_HD inline void task_of(bool upper, int n, int task, int &rt, int &k_lo, int &k_hi) {
    rt = 0;
    int t = task;
    for (int c = splits(upper, n, 0); t >= c; c = splits(upper, n, rt)) {
        t -= c;
        ++rt;
    }
    int kb, ke;
    krange(upper, n, rt, kb, ke);
    k_lo = kb + t * kSplit;
    k_hi = ke < k_lo + kSplit ? ke : k_lo + kSplit;
}

// A task's partial product (kRows x ldb) is stored column-quad-major: the 4
// columns [4q, 4q+4) of all 128 rows, then the next quad, so that a warp's
// accumulator rows (one per lane) leave as 512 contiguous bytes.
ARAP_BTOP_HD inline int64_t ws_at(int task, int r, int c, int ldb) {
    return (int64_t)task * kRows * ldb + ((int64_t)(c >> 2) * kRows + r) * 4 + (c & 3);
}

// Operand tiles, stored in global memory exactly as the MMA reads them from
// shared memory (K-major core matrices, arap_btop.cuh's tile_off), TF32 head
// then rest, so that one bulk copy moves a stage's tile. A tile: 128 rows of
// T x 32 of its columns (kRows x kDepth floats per part); B tile: 32 rows of
// the right-hand sides x 256 of their columns (kCols x kDepth per part).
constexpr int kAFloats = kRows * kDepth, kBFloats = kCols * kDepth;
constexpr int kATileFloats = 2 * kAFloats, kBTileFloats = 2 * kBFloats;

// A tiles of direction `upper` for the row tiles before rt: each row tile's
// columns [kb, ke) in stages of kDepth
ARAP_BTOP_HD inline int stages_before(bool upper, int n, int rt) {
    int t = 0;
    for (int r = 0; r < rt && r * kRows < n; ++r) {
        int kb, ke;
        krange(upper, n, r, kb, ke);
        t += (ke - kb + kDepth - 1) / kDepth;
    }
    return t;
}

// floats of both directions' A tiles of an n-column top
inline int64_t a_tile_floats(int n) {
    if (n <= 0) return 0;
    const int nrt = row_tiles(n);
    return (int64_t)(stages_before(false, n, nrt) + stages_before(true, n, nrt)) * kATileFloats;
}

// B tile (stage kb, column tile ct) of an n x ldb right-hand side matrix
ARAP_BTOP_HD inline int col_tiles(int ldb) { return (ldb + kCols - 1) / kCols; }
ARAP_BTOP_HD inline int64_t b_tile_at(int kb, int ct, int ldb) {
    return ((int64_t)kb * col_tiles(ldb) + ct) * kBTileFloats;
}
inline int64_t b_tile_floats(int n, int ldb) {
    return n <= 0 ? 0 : (int64_t)((n + kDepth - 1) / kDepth) * col_tiles(ldb) * kBTileFloats;
}

// floats of the partial products of one sweep (the larger of the two
// directions' task counts)
inline int64_t ws_floats(int n, int P) {
    if (n <= 0) return 0;
    const int nrt = row_tiles(n), a = tasks(false, n, nrt), b = tasks(true, n, nrt);
    return (int64_t)(a > b ? a : b) * kRows * ldb_of(P);
}

}  // namespace btop
}  // namespace arapgpu

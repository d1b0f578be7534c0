// Host checks of the dense top's task plan (mesh-deform_gb300/csrc/arap_btop_plan.h):
// every row tile's part of the triangle of T is cut into whole, disjoint,
// ordered splits; the kernel's task decoding matches the reduction's task
// numbering; the partial-product layout is a bijection inside its task block
// with 16-byte quads and warp rows 512 contiguous bytes apart per quad.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "arap_btop_plan.h"

using namespace arapgpu::btop;

static int fails = 0;
#define CHECK(c)                                                                  \
    do {                                                                          \
        if (!(c)) {                                                               \
            if (fails++ < 20) std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #c); \
        }                                                                         \
    } while (0)

static void check_plan(int n) {
    for (int up = 0; up < 2; ++up) {
        const bool upper = up != 0;
        const int nrt = row_tiles(n), total = tasks(upper, n, nrt);
        CHECK(total >= nrt);
        int task = 0;
        for (int rt = 0; rt < nrt; ++rt) {
            int kb, ke;
            krange(upper, n, rt, kb, ke);
            CHECK(0 <= kb && kb < ke && ke <= n);
            // the triangle of every row of the tile lies inside [kb, ke)
            const int r0 = rt * kRows, r1 = (rt + 1) * kRows < n ? (rt + 1) * kRows : n;
            if (upper) CHECK(kb <= r0);
            else CHECK(ke >= r1);
            CHECK(tasks(upper, n, rt) == task);
            const int ns = splits(upper, n, rt);
            int next = kb;
            for (int s = 0; s < ns; ++s, ++task) {
                int rt2, lo, hi;
                task_of(upper, n, task, rt2, lo, hi);
                CHECK(rt2 == rt);
                CHECK(lo == next);  // disjoint, ordered, no gap
                CHECK(lo < hi && hi - lo <= kSplit);
                CHECK(lo % 4 == 0);  // float4 loads of T's rows start on a quad
                next = hi;
            }
            CHECK(next == ke);
        }
        CHECK(task == total);
        CHECK(ws_floats(n, 7) >= (int64_t)total * kRows * ldb_of(7));
    }
}

// The operand tiles the products copy: every (task, stage) A tile lies inside
// its direction's part of a_tile_floats, distinct stages of a row tile are
// distinct tiles, and every B tile a task reads (and every entry the
// producers write) lies inside b_tile_floats; copy offsets are 16-byte aligned.
static void check_tiles(int n, int P) {
    const int ldb = ldb_of(P), nrt = row_tiles(n);
    const int64_t fwd = (int64_t)stages_before(false, n, nrt) * kATileFloats;
    CHECK(a_tile_floats(n) == fwd + (int64_t)stages_before(true, n, nrt) * kATileFloats);
    for (int up = 0; up < 2; ++up) {
        const bool upper = up != 0;
        const int total = tasks(upper, n, nrt);
        std::vector<char> used(a_tile_floats(n) / kATileFloats + 1, 0);
        for (int task = 0; task < total; ++task) {
            int rt, lo, hi, kb, ke;
            task_of(upper, n, task, rt, lo, hi);
            krange(upper, n, rt, kb, ke);
            CHECK((lo - kb) % kDepth == 0 && lo % kDepth == 0);
            const int ns = (hi - lo + kDepth - 1) / kDepth;
            for (int st = 0; st < ns; ++st) {
                const int64_t a = (upper ? fwd : 0) +
                                  (int64_t)(stages_before(upper, n, rt) + (lo - kb) / kDepth + st) * kATileFloats;
                const int64_t part_end = upper ? a_tile_floats(n) : fwd;
                CHECK(a >= (upper ? fwd : 0) && a + kATileFloats <= part_end);
                CHECK((a * 4) % 16 == 0);
                const size_t t = (size_t)(a / kATileFloats);
                if (t < used.size()) {
                    CHECK(!used[t]);
                    used[t] = 1;
                }
                for (int ct = 0; ct < col_tiles(ldb); ++ct) {
                    const int64_t b = b_tile_at(lo / kDepth + st, ct, ldb);
                    CHECK(b >= 0 && b + kBTileFloats <= b_tile_floats(n, ldb));
                    CHECK((b * 4) % 16 == 0);
                }
            }
        }
    }
    // every entry the gather and the forward reduction write
    for (int d = 0; d < n; d += (n > 64 ? 7 : 1))
        for (int c = 0; c < ldb; ++c) {
            const int64_t b = b_tile_at(d / kDepth, c / kCols, ldb);
            CHECK(b >= 0 && b + kBTileFloats <= b_tile_floats(n, ldb));
        }
}

static void check_layout(int P) {
    const int ldb = ldb_of(P);
    CHECK(ldb % 4 == 0 && ldb >= 3 * P && ldb < 3 * P + 4);
    for (int task = 0; task < 3; ++task) {
        std::vector<char> seen((size_t)kRows * ldb, 0);
        const int64_t base = (int64_t)task * kRows * ldb;
        for (int r = 0; r < kRows; ++r)
            for (int c = 0; c < ldb; ++c) {
                const int64_t e = ws_at(task, r, c, ldb) - base;
                CHECK(e >= 0 && e < (int64_t)kRows * ldb);
                if (e >= 0 && e < (int64_t)kRows * ldb) {
                    CHECK(!seen[(size_t)e]);
                    seen[(size_t)e] = 1;
                }
                if (c % 4 == 0) CHECK(ws_at(task, r, c, ldb) % 4 == 0);
                else CHECK(ws_at(task, r, c, ldb) == ws_at(task, r, c - 1, ldb) + 1);
                if (r % 32 != 0 && c % 4 == 0) CHECK(ws_at(task, r, c, ldb) == ws_at(task, r - 1, c, ldb) + 4);
            }
    }
}

int main() {
    for (int n = 1; n <= 1200; ++n) check_plan(n);
    for (int n : {1457, 1868, 2047, 2048, 2049, 3000, 4095, 4096}) check_plan(n);
    for (int P : {1, 2, 3, 4, 5, 7, 19, 85, 86, 256, 1000}) check_layout(P);
    for (int n : {1, 31, 32, 33, 127, 128, 129, 300, 1457, 2048, 3072, 4096})
        for (int P : {1, 5, 85, 86, 256}) check_tiles(n, P);
    if (fails) {
        std::printf("%d failures\n", fails);
        return 1;
    }
    std::printf("ALL PASSED\n");
    return 0;
}

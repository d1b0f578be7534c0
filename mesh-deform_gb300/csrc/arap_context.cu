// arap_context.cu -- the C ABI (include/arap_gpu.h): context state, setup and
// the local/global iteration loop of deform() (inc/deform/arap.h:101-138).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/arap_gpu.h"
#include "arap_kernels.h"
#include "arap_symbolic.h"

namespace arapgpu {
cudaError_t configure_solve_smem(int bytes_f32, int bytes_f64);
}

using namespace arapgpu;

namespace {

// ticket counters of the single-request solves: forward / backward of the CTA
// sweep (0, 1), of the cluster sweep (2, 3), of the warp sweep (4, 6), then
// forward / backward per tree level of the level schedule
// (kLevelTicket0 + 2 l, kLevelTicket0 + 2 l + 1)
constexpr int kTickets = kLevelTicket0 + 2 * kMaxLevelLaunch;
// schedule of the single-CTA solve levels (arap_set_solve_schedule)
constexpr int kSolveScheduleDefault = ARAP_SOLVE_PERSISTENT;
// largest subtree (columns) of a level-1 supernode solved as one block by the
// single-request sweeps (arap_set_solve_blocks; 0: none). Measured on the
// twisted bar: iterations of one request 13.3 -> 9.7 ms, 16 requests in flight
// 91 -> 86 ms per step.
constexpr int kSolveBlocksDefault = 512;
// fronts of at most this many rows at the bottom of the tree are solved one
// warp per supernode (arap_set_warp_rows; 0: none)
constexpr int kWarpRowsDefault = 0;

// Device buffer from the device's stream-ordered memory pool, allocated and
// freed on the owning context's stream: growing or dropping a buffer never
// waits for work on other streams (a plain cudaFree would wait for the whole
// device).
struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaStream_t st = nullptr;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap && p) return cudaSuccess;
        if (p) cudaFreeAsync(p, st);
        p = nullptr;
        cap = 0;
        const size_t want = std::max<size_t>(bytes, 256);
        cudaError_t e = cudaMallocAsync(&p, want, st);
        if (e == cudaSuccess) cap = want;
        else p = nullptr;
        return e;
    }
    void release() {
        if (p) cudaFreeAsync(p, st);
        p = nullptr;
        cap = 0;
    }
    template <typename T> T *as() const { return reinterpret_cast<T *>(p); }
};

// Freed pool memory stays with the process (release threshold at its
// maximum), so contexts created after others were destroyed reuse it without
// a trip to the driver. Set once per device.
cudaError_t keep_pool_memory(int device) {
    static std::mutex mu;
    static std::vector<int> done;
    std::lock_guard<std::mutex> lk(mu);
    if (std::find(done.begin(), done.end(), device) != done.end()) return cudaSuccess;
    cudaMemPool_t pool;
    cudaError_t e = cudaDeviceGetDefaultMemPool(&pool, device);
    if (e != cudaSuccess) return e;
    uint64_t thr = ~0ull;
    e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    if (e == cudaSuccess) done.push_back(device);
    return e;
}

// 64-byte words of pinned host memory for the per-context error word, handed
// out from pages that live as long as the process (freeing pinned memory can
// wait for the device).
struct PinnedWords {
    std::mutex mu;
    std::vector<int *> free_words;
    int *get() {
        std::lock_guard<std::mutex> lk(mu);
        if (free_words.empty()) {
            char *page = nullptr;
            if (cudaMallocHost(&page, 4096) != cudaSuccess) return nullptr;
            for (int i = 0; i < 4096 / 64; ++i) free_words.push_back(reinterpret_cast<int *>(page + 64 * i));
        }
        int *w = free_words.back();
        free_words.pop_back();
        return w;
    }
    void put(int *w) {
        std::lock_guard<std::mutex> lk(mu);
        free_words.push_back(w);
    }
};

PinnedWords &pinned_words() {
    static PinnedWords *pw = new PinnedWords();  // never destroyed: pages outlive every context
    return *pw;
}

thread_local std::string g_create_error;

}  // namespace

namespace arapgpu {
// Message returned by arap_last_error(NULL) for context-free entry points.
void set_global_error(const std::string &msg) { g_create_error = msg; }
}  // namespace arapgpu

struct arap_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr;
    std::string err;
    Topology topo;
    // inputs
    bool have_rest = false;
    std::vector<int32_t> cidx;    // sorted unique constrained vertices
    std::vector<double> ctgt;     // 3 per constrained vertex (sorted order)
    std::vector<uint8_t> cmask;   // V
    int precision = ARAP_PRECISION_FP64;
    int refine = 1;
    // numeric factorisation of the mixed form: 64 (FP64 factor, rounded to FP32
    // copies for the solves) or 32 (FP32 factor)
    int factor_bits = 64;
    bool dirty = true;
    bool retarget = false;  // same constrained set, new targets: reuse weights and factor
    bool sym_cache = true;  // keep the symbolic analysis while the constrained set is unchanged
    // symbolic cache (keyed by the constrained-vertex mask)
    bool sym_valid = false;  // analysed and uploaded
    bool sym_host = false;   // analysed (host only)
    Symbolic sym;
    size_t smem_f32 = 0, smem_f64 = 0;  // dynamic shared memory the solve kernels are configured for
    bool fp64_solves = true;             // the FP64 solves fit this symbolic analysis's fronts
    size_t top_smem_f32 = 0, top_smem_f64 = 0;
    // which precision the iteration state was set up for
    int state_prec = -1;
    bool have_rotations = false;
    // device buffers
    DevBuf faces, ent_ptr, ent_fc, hc, w_orig;
    DevBuf rest, targets, out;
    DevBuf drow, dcol, dent, oldidx, amap, dmap, sn, rows, relind, child, level_sn, fitems;
    DevBuf w64, w32, p64, pc64, p32, pc32, R, diag64, bfixed, b, sol, uvec, Lval, Dinv, Upd, Xinv, L21, L21T, redge;
    DevBuf Lval32, Dinv32;  // the mixed form's FP64 factor rounded to FP32 (the inverses for the solves are formed from it)
    DevBuf errw, ticket, flags, energy;
    DevBuf cidx_dev, handle_dev, tabs_dev;  // arap_pose_targets inputs
    DevBuf vf_ptr, vf_face, fnorm, vnorm;    // vertex normals
    // many-pose state (arap_deform_poses)
    DevBuf btargets, bpc64, bpc32, bR, bbfixed, bb, bsol, buvec, bout, bticket, bflags, bftop, bytop, bws, batile;
    int bP = 0, bT = 0, bpt = 0, bgrid = 0, bntop = -1;
    int64_t bgen = -1;  // gen the many-pose buffers and counters were set up for (-1: redo)
    int pose_tile = 0;  // poses per batched-solve task (0: the largest that fits)
    int tP = -1;  // poses whose targets btargets holds (-1: none)
    int model_P = 1, model_T = 1;  // poses / pose tiles of the last deform (cost model)
    bool model_batched = false;    // the last deform was arap_deform_poses (its solves cover the whole tree)
    // CUDA graphs of the setup and of 2^k iterations (k < kIterGraphs); a deform
    // of n iterations replays the graphs of n's binary digits, so any count
    // reuses them. Replayed while nothing they reference changes (direct
    // launches when profiling).
    static constexpr int kIterGraphs = 8;
    cudaGraphExec_t g_setup = nullptr, g_iter[kIterGraphs] = {}, g_biter[kIterGraphs] = {};
    int64_t g_setup_key[4] = {0, 0, 0, 0}, g_iter_key[kIterGraphs][4] = {}, g_biter_key[kIterGraphs][4] = {};
    int64_t g_setup_launches = 0, g_iter_launches[kIterGraphs] = {}, g_biter_launches[kIterGraphs] = {};
    int64_t gen = 1;  // bumped when the symbolic analysis or any device buffer changes
    bool use_graphs = true;
    int solve_cap = 0;  // most CTAs per triangular-solve launch (0: as many as fit the device)
    int top_bytes = 0;  // supernode size from which tree levels go to the cluster solves (0: default, <0: never)
    int dense_cols = 0;  // most columns of the dense top of the tree (0: default, <0: none)
    int warp_rows = kWarpRowsDefault;  // largest front of the warp-per-supernode solves (0: none)
    int solve_schedule = kSolveScheduleDefault;  // ARAP_SOLVE_PERSISTENT or ARAP_SOLVE_LEVELS
    int solve_blocks = kSolveBlocksDefault;      // largest solve block (columns), 0: none
    SolveBlocks sb;                              // the blocks of the current analysis (use_sb)
    bool use_sb = false;
    DevSym dss;                                  // the single-request sweeps' layout with the blocks
    DevBuf ssn, slevel_sn, sbitems, sbmembers;
    // launch shape of the local step, RHS and residual (arap_set_vertex_launch)
    VertexLaunch vlaunch[kVertexKernels] = {{1, 256}, {1, 256}, {1, 256}};
    size_t dense_inv_smem[2] = {0, 0};  // configured limits (FP32, FP64)
    DevBuf top_col, top_gptr, top_gidx, tdpos, top_items, Ttop, ytop;
    int ordering = ARAP_ORDER_PER_CONSTRAINT_SET;
    arap_done_fn done_fn = nullptr;  // called from a CUDA thread when an async deform finished
    void *done_user = nullptr;
    // host time of the last arap_deform_async, ms: analysis + uploads,
    // allocation, set-up enqueue, iteration enqueue, rest
    double host_ms[5] = {0, 0, 0, 0, 0};
    // asynchronous deform (arap_deform_async / arap_wait)
    bool in_flight = false;    // a deform was enqueued and not waited for
    int *herr_host = nullptr;  // pinned copy of the device error word
    bool poses_in_flight = false;  // the pending deform is an arap_deform_poses_async
    cudaEvent_t ev_done = nullptr;  // recorded after the last copy of an async deform
    size_t bsmem = 0;
    DevTopo dt{};
    DevSym ds{};
    int64_t launches = 0;
    double setup_ms = 0.0, iter_ms = 0.0;
    // optional per-launch profiler
    bool profiling = false;
    std::vector<cudaEvent_t> evpool;
    size_t evused = 0;
    struct Pending { int cls; cudaEvent_t a, b; };
    std::vector<Pending> pending;
    double kms[ARAP_K_NUM_CLASSES] = {0};
    int64_t kcnt[ARAP_K_NUM_CLASSES] = {0};

    std::vector<DevBuf *> buffers() {
        return {&faces, &ent_ptr, &ent_fc, &hc, &w_orig, &rest, &targets, &out, &drow, &dcol, &dent, &oldidx,
                &amap, &dmap, &sn, &rows, &relind, &child, &level_sn, &fitems, &w64, &w32, &p64, &pc64, &p32,
                &pc32, &R, &diag64, &bfixed, &b, &sol, &uvec, &Lval, &Dinv, &Upd, &Xinv, &L21, &L21T, &redge,
                &errw, &ticket, &flags, &energy, &cidx_dev, &handle_dev, &tabs_dev, &vf_ptr, &vf_face, &fnorm,
                &vnorm, &btargets, &bpc64, &bpc32, &bR, &bbfixed, &bb, &bsol, &buvec, &bout, &bftop, &bytop, &bws,
                &batile,
                &bticket, &bflags, &top_col, &top_gptr, &top_gidx, &tdpos, &top_items, &Ttop, &ytop, &Lval32,
                &Dinv32, &ssn, &slevel_sn, &sbitems, &sbmembers};
    }
};

#define CK(call)                                                                       \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess) {                                                       \
            ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);             \
            return e_ == cudaErrorMemoryAllocation ? ARAP_ERR_OUT_OF_MEMORY : ARAP_ERR_CUDA; \
        }                                                                              \
    } while (0)

namespace {

cudaEvent_t pool_event(arap_ctx *ctx) {
    if (ctx->evused == ctx->evpool.size()) {
        cudaEvent_t e = nullptr;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        ctx->evpool.push_back(e);
    }
    return ctx->evpool[ctx->evused++];
}

// Brackets one launch with events when profiling is on.
struct Prof {
    arap_ctx *ctx;
    int cls;
    cudaEvent_t a = nullptr;
    Prof(arap_ctx *c, int k) : ctx(c), cls(k) {
        if (ctx->profiling && (a = pool_event(ctx))) cudaEventRecord(a, ctx->stream);
    }
    ~Prof() {
        if (!a) return;
        cudaEvent_t b = pool_event(ctx);
        if (!b) return;
        cudaEventRecord(b, ctx->stream);
        ctx->pending.push_back({cls, a, b});
    }
};

// Adds the device time of completed bracketed launches (stream synchronized).
void collect_profile(arap_ctx *ctx) {
    for (const auto &p : ctx->pending) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            ctx->kms[p.cls] += ms;
            ctx->kcnt[p.cls] += 1;
        }
    }
    ctx->pending.clear();
    ctx->evused = 0;
}

template <typename T>
cudaError_t upload(DevBuf &buf, const std::vector<T> &v, cudaStream_t st) {
    cudaError_t e = buf.ensure(v.size() * sizeof(T));
    if (e != cudaSuccess || v.empty()) return e;
    return cudaMemcpyAsync(buf.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st);
}

int fail(arap_ctx *ctx, int code, const std::string &msg) {
    ctx->err = msg;
    return code;
}

// Builds (or reuses) the symbolic analysis for the current constraint mask and
// uploads it.
// Host part of prepare_symbolic: the analysis of the current mask, kept until
// the mask changes.
int analyze_symbolic(arap_ctx *ctx) {
    if (ctx->sym_host && ctx->sym.constrained == ctx->cmask) return ARAP_OK;
    ctx->sym_valid = false;
    ctx->sym_host = false;
    std::string err;
    bool singular = false;
    if (!build_symbolic(ctx->topo, ctx->cmask, ctx->sym, err, singular, ctx->ordering == ARAP_ORDER_MESH))
        return fail(ctx, singular ? ARAP_ERR_NOT_SPD : ARAP_ERR_CUDA, err);
    ctx->use_sb = ctx->solve_blocks > 0 && build_solve_blocks(ctx->sym, ctx->solve_blocks, ctx->sb);
    if (!ctx->use_sb) ctx->sb = SolveBlocks();
    ctx->sym_host = true;
    return ARAP_OK;
}

// The dense top of the tree: the most top levels whose supernodes hold at most
// `cap` columns together (at least two levels, or none). Returns its first
// level (nlev when empty) and its column count.
struct DenseTopChoice {
    int level = 0, ncols = 0;
};
DenseTopChoice choose_dense_top(const Symbolic &s, int cap) {
    const int nlev = (int)s.level_ptr.size() - 1;
    DenseTopChoice t;
    t.level = std::max(nlev, 0);
    if (cap <= 0 || nlev <= 0) return t;
    int cols = 0, level = nlev;
    for (int l = nlev - 1; l >= 0; --l) {
        int c = 0;
        for (int q = s.level_ptr[l]; q < s.level_ptr[l + 1]; ++q) c += s.sn[s.level_sn[q]].ncol;
        if (cols + c > cap) break;
        cols += c;
        level = l;
    }
    if (nlev - level >= 2) {
        t.level = level;
        t.ncols = cols;
    }
    return t;
}

int dense_cap(const arap_ctx *ctx) {
    if (ctx->dense_cols < 0) return 0;
    if (ctx->dense_cols > 0) return std::min(ctx->dense_cols, kDenseTopCols);
    // a request that owns the device takes more levels into T (fewer sweep
    // levels, one wider product); under a CTA cap the product's SM time is
    // shared with other requests
    return ctx->solve_cap <= 0 ? kDenseTopOwned : kDenseTopDefault;
}

// Bytes of every device buffer the setup of precision T (and, for n_poses > 0,
// arap_deform_poses with that many poses) holds, buffer by buffer.
template <typename T>
void planned_sizes(arap_ctx *ctx, int n_poses, std::vector<std::pair<DevBuf *, size_t>> &out) {
    const Symbolic &s = ctx->sym;
    const size_t V = (size_t)s.V, m1 = (size_t)std::max(s.m, 1), nnz = s.dcol.size(), S1 = (size_t)std::max(s.S, 1);
    out.clear();
    auto add = [&](DevBuf &b, size_t bytes) { out.push_back({&b, bytes}); };
    // symbolic uploads and solve scheduling state
    add(ctx->drow, s.drow.size() * 4);
    add(ctx->dcol, s.dcol.size() * 4);
    add(ctx->dent, s.dent.size() * 4);
    add(ctx->oldidx, s.oldidx.size() * 4);
    add(ctx->amap, s.amap.size() * 8);
    add(ctx->dmap, s.dmap.size() * 8);
    add(ctx->sn, s.sn.size() * sizeof(SnInfo));
    add(ctx->rows, s.rows.size() * 4);
    add(ctx->relind, s.relind.size() * 4);
    add(ctx->child, s.child.size() * 4);
    add(ctx->level_sn, s.level_sn.size() * 4);
    add(ctx->fitems, s.fitems.size() * sizeof(FItem));
    add(ctx->ticket, kTickets * sizeof(unsigned long long));
    add(ctx->flags, 2 * sizeof(unsigned) * S1);
    // iteration state and factor (setup_alloc)
    const bool f32 = sizeof(T) == 4;
    add(ctx->w64, nnz * sizeof(double));
    if (f32) add(ctx->w32, nnz * sizeof(float));
    add(ctx->p64, V * sizeof(Vec4<double>));
    add(ctx->pc64, V * sizeof(Vec4<double>));
    if (f32) {
        add(ctx->p32, V * sizeof(Vec4<float>));
        add(ctx->pc32, V * sizeof(Vec4<float>));
    }
    add(ctx->R, V * 3 * sizeof(Vec4<T>));
    add(ctx->diag64, m1 * sizeof(double));
    add(ctx->bfixed, m1 * sizeof(Vec4<double>));
    if (f32) add(ctx->redge, std::max<size_t>(nnz, 1) * sizeof(Vec4<float>));
    add(ctx->b, m1 * sizeof(Vec4<T>));
    add(ctx->sol, m1 * sizeof(Vec4<T>));
    add(ctx->uvec, (size_t)std::max<int64_t>(s.uvec_size, 1) * sizeof(Vec4<T>));
    // the factor's working arrays in the factor's precision; an FP64 factor of
    // the mixed form also keeps FP64 solve arrays, rounded into the FP32 ones
    const bool f64f = f32 && ctx->factor_bits == 64;
    const size_t fs = f64f ? sizeof(double) : sizeof(T);
    add(ctx->Lval, (size_t)std::max<int64_t>(s.panel_size, 1) * fs);
    add(ctx->Dinv, (size_t)std::max<int64_t>(s.dinv_size, 1) * fs);
    add(ctx->Upd, (size_t)std::max<int64_t>(s.upd_size, 1) * fs);
    // the solve arrays, with the solve blocks after the supernodes' own
    const int64_t xs = ctx->use_sb ? ctx->sb.x_size : s.x_size, l21s = ctx->use_sb ? ctx->sb.l21_size : s.l21_size,
                  l21ts = ctx->use_sb ? ctx->sb.l21t_size : s.l21t_size;
    add(ctx->Xinv, (size_t)std::max<int64_t>(xs, 1) * sizeof(T));
    add(ctx->L21, (size_t)std::max<int64_t>(l21s, 1) * sizeof(T));
    add(ctx->L21T, (size_t)std::max<int64_t>(l21ts, 1) * sizeof(T));
    const int nt = choose_dense_top(s, dense_cap(ctx)).ncols;
    add(ctx->Ttop, std::max<size_t>(nt > 0 ? dense_top_elems(nt) : 0, 1) * sizeof(T));
    if (f64f) {
        add(ctx->Lval32, (size_t)std::max<int64_t>(s.panel_size, 1) * sizeof(float));
        add(ctx->Dinv32, (size_t)std::max<int64_t>(s.dinv_size, 1) * sizeof(float));
    }
    add(ctx->ytop, std::max<size_t>(top_vec_bytes(nt, sizeof(T)), 16));  // y_top, the tiles' partials, counters
    if (n_poses > 0) {
        const size_t P = (size_t)n_poses, VP = V * P, MP = m1 * P, nc = V - (size_t)s.m;
        const int pt = std::max(batch_pose_tile(ctx->use_sb ? std::max(s.max_ldx, ctx->sb.max_ldx) : s.max_ldx,
                                                ctx->use_sb ? std::max(s.max_ld21, ctx->sb.max_ld21) : s.max_ld21), 1);
        const size_t T_ = (P + pt - 1) / pt;
        add(ctx->bpc64, VP * sizeof(Vec4<double>));
        add(ctx->bpc32, VP * sizeof(Vec4<float>));
        add(ctx->bR, VP * 3 * sizeof(Vec4<float>));
        add(ctx->bbfixed, MP * sizeof(Vec4<double>));
        add(ctx->bb, MP * sizeof(Vec4<float>));
        add(ctx->bsol, MP * sizeof(Vec4<float>));
        add(ctx->buvec, (size_t)std::max<int64_t>(s.uvec_size, 1) * P * sizeof(Vec4<float>));
        add(ctx->bout, VP * 3 * sizeof(double));
        add(ctx->btargets, P * nc * 3 * sizeof(double));
        add(ctx->bticket, 2 * sizeof(unsigned long long));
        add(ctx->bflags, 2 * S1 * T_ * sizeof(unsigned));
        add(ctx->bftop, std::max<size_t>(btop_matrix_floats(nt, (int)P), 1) * sizeof(float));
        add(ctx->bytop, std::max<size_t>(btop_matrix_floats(nt, (int)P), 1) * sizeof(float));
        add(ctx->bws, std::max<size_t>(btop_workspace_floats(nt, (int)P), 1) * sizeof(float));
        add(ctx->batile, std::max<size_t>(btop_atile_floats(nt), 1) * sizeof(float));
    }
}

// Index maps of the dense top (levels >= level, n columns) uploaded to the
// device: each top supernode's dense offset, each dense index's device column,
// the update-vector entries of the top supernodes' children in the lower
// levels that land on each dense row (children in child-list order), and the
// work items of the inversion (supernode, first of 16 columns).
int prepare_dense_top(arap_ctx *ctx, int level, int n) {
    const Symbolic &s = ctx->sym;
    DevSym &d = ctx->ds;
    cudaStream_t st = ctx->stream;
    const int nlev = (int)s.level_ptr.size() - 1;
    std::vector<int32_t> tdpos(std::max(s.S, 1), -1), col(n), items;
    std::vector<int32_t> col2d(std::max(s.m, 1), -1);
    int off = 0;
    for (int j = 0; j < s.S; ++j) {  // supernode order is the elimination order
        const SnInfo &x = s.sn[j];
        if (x.level < level) continue;
        tdpos[j] = off;
        for (int c = 0; c < x.ncol; ++c) {
            col[off + c] = x.first + c;
            col2d[x.first + c] = off + c;
        }
        for (int c0 = 0; c0 < x.ncol; c0 += kTopRhs) items.insert(items.end(), {j, c0});
        off += x.ncol;
    }
    if (off != n) return fail(ctx, ARAP_ERR_CUDA, "dense top: column count mismatch");
    std::vector<int32_t> cnt(n + 1, 0);
    std::vector<std::pair<int32_t, int64_t>> entries;
    for (int q = s.level_ptr[level]; q < s.level_ptr[nlev]; ++q) {
        const SnInfo &a = s.sn[s.level_sn[q]];
        for (int ci = a.child_begin; ci < a.child_end; ++ci) {
            const SnInfo &c = s.sn[s.child[ci]];
            if (c.level >= level) continue;
            for (int i = 0; i < c.nrow - c.ncol; ++i) {
                const int dd = col2d[s.rows[c.rows_off + i]];
                if (dd < 0) return fail(ctx, ARAP_ERR_CUDA, "dense top: update row outside the top");
                entries.push_back({dd, c.uvec_off + i});
            }
        }
    }
    for (const auto &e : entries) ++cnt[e.first + 1];
    for (int i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
    std::vector<int64_t> gidx(std::max<size_t>(entries.size(), 1), 0);
    {
        std::vector<int32_t> fill(cnt.begin(), cnt.end() - 1);
        for (const auto &e : entries) gidx[fill[e.first]++] = e.second;  // stable: entries keep their order per row
    }
    CK(upload(ctx->tdpos, tdpos, st));
    CK(upload(ctx->top_col, col, st));
    CK(upload(ctx->top_gptr, cnt, st));
    CK(upload(ctx->top_gidx, gidx, st));
    CK(upload(ctx->top_items, items, st));
    d.n_top = n;
    d.top_pair32 = (int64_t)top_tiles(n) > top_tile_resident_ctas(4);
    d.top_pair64 = (int64_t)top_tiles(n) > top_tile_resident_ctas(8);
    d.n_top_items = (int)items.size() / 2;
    return ARAP_OK;
}

// The single-request sweeps' layout with the solve blocks (SolveBlocks): the
// supernodal layout ds with the blocks' array and solve levels. Every level of
// the solve tree is one below the supernodal level, so the top's split moves
// down by one; the blocks need the top to start at supernodal level 2 or
// above (else they are not used).
int prepare_solve_blocks(arap_ctx *ctx) {
    const SolveBlocks &b = ctx->sb;
    const DevSym &f = ctx->ds;
    cudaStream_t st = ctx->stream;
    if (f.ltop < 2) {
        ctx->use_sb = false;
        return ARAP_OK;
    }
    CK(upload(ctx->ssn, b.sn, st));
    CK(upload(ctx->slevel_sn, b.level_sn, st));
    CK(upload(ctx->sbitems, b.items, st));
    CK(upload(ctx->sbmembers, b.members, st));
    DevSym d = f;
    d.sn = ctx->ssn.as<SnInfo>();
    d.level_sn = ctx->slevel_sn.as<int32_t>();
    const int nlev = (int)b.level_ptr.size() - 1;
    d.ltop = f.ltop - 1;
    d.s_low = b.level_ptr[d.ltop];
    d.max_ldx = std::max(f.max_ldx, b.max_ldx);
    d.max_ld21 = std::max(f.max_ld21, b.max_ld21);
    d.max_ncol = std::max(f.max_ncol, b.max_ncol);
    const size_t b32 = solve_smem_bytes(d.max_ldx, d.max_ld21, 4), b64 = solve_smem_bytes(d.max_ldx, d.max_ld21, 8);
    constexpr size_t kSmemMax = 227 * 1024;
    if (b32 > kSmemMax || (ctx->fp64_solves && b64 > kSmemMax)) {
        ctx->use_sb = false;
        return ARAP_OK;
    }
    if (b32 > ctx->smem_f32 || (ctx->fp64_solves && b64 > ctx->smem_f64)) {
        CK(configure_solve_smem((int)b32, ctx->fp64_solves ? (int)b64 : 0));
        ctx->smem_f32 = std::max(ctx->smem_f32, b32);
        if (ctx->fp64_solves) ctx->smem_f64 = std::max(ctx->smem_f64, b64);
    }
    // warp-per-supernode levels at the bottom of the solve tree
    int lwarp = 0;
    const int wrows = std::min(ctx->warp_rows, wsolve_max_rows());
    while (wrows > 0 && lwarp < d.ltop) {
        int mx = 0;
        for (int q = b.level_ptr[lwarp]; q < b.level_ptr[lwarp + 1]; ++q) mx = std::max(mx, (int)b.sn[b.level_sn[q]].nrow);
        if (mx > wrows) break;
        ++lwarp;
    }
    d.lwarp = lwarp;
    d.s_warp = b.level_ptr[lwarp];
    const int cap = ctx->solve_cap;
    if (d.s_warp > 0) {
        CK(configure_wsolve());
        const int need = (d.s_warp + 7) / 8;
        const int r32 = wsolve_resident_ctas(4), r64 = wsolve_resident_ctas(8);
        d.wgrid32 = std::max(1, std::min(need, cap > 0 ? std::min(cap, r32) : r32));
        d.wgrid64 = std::max(1, std::min(need, cap > 0 ? std::min(cap, r64) : r64));
    }
    d.s_sched = b.level_ptr[nlev];  // the absorbed leaves are not scheduled
    d.s_top = f.n_top > 0 ? 0 : b.level_ptr[nlev] - d.s_low;
    const int res32 = solve_resident_ctas((int)b32, 4), res64 = solve_resident_ctas((int)b64, 8);
    const int nl = std::max(d.s_low - d.s_warp, 1);
    d.solve_grid32 = std::max(1, std::min(nl, cap > 0 ? std::min(cap, res32) : res32));
    d.solve_grid64 = std::max(1, std::min(nl, cap > 0 ? std::min(cap, res64) : res64));
    d.overlap = cap <= 0;
    d.level_launch = ctx->solve_schedule == ARAP_SOLVE_LEVELS && nlev <= kMaxLevelLaunch;
    for (int l = 0; l <= kMaxLevelLaunch; ++l) d.lev_ptr[l] = nlev > 0 ? b.level_ptr[std::min(l, nlev)] : 0;
    for (int l = 0; l < kMaxLevelLaunch; ++l) {
        int lx = 0, l21 = 0;
        for (int q = d.lev_ptr[l]; q < d.lev_ptr[l + 1]; ++q) {
            const SnInfo &x = b.sn[b.level_sn[q]];
            lx = std::max(lx, (int)x.ldx);
            l21 = std::max(l21, (int)x.ld21);
        }
        d.lev_ldx[l] = lx;
        d.lev_ld21[l] = l21;
        const int n = std::max(d.lev_ptr[l + 1] - d.lev_ptr[l], 1);
        const int r32 = solve_resident_ctas((int)solve_smem_bytes(lx, l21, 4), 4);
        const int r64 = solve_resident_ctas((int)solve_smem_bytes(lx, l21, 8), 8);
        d.lev_grid32[l] = std::max(1, std::min(n, cap > 0 ? std::min(cap, r32) : r32));
        d.lev_grid64[l] = std::max(1, std::min(n, cap > 0 ? std::min(cap, r64) : r64));
    }
    ctx->dss = d;
    return ARAP_OK;
}

int prepare_symbolic(arap_ctx *ctx) {
    if (ctx->sym_valid && ctx->sym.constrained == ctx->cmask) return ARAP_OK;
    const int rc = analyze_symbolic(ctx);
    if (rc != ARAP_OK) return rc;
    Symbolic &s = ctx->sym;
    cudaStream_t st = ctx->stream;
    ctx->gen++;
    CK(upload(ctx->drow, s.drow, st));
    CK(upload(ctx->dcol, s.dcol, st));
    CK(upload(ctx->dent, s.dent, st));
    CK(upload(ctx->oldidx, s.oldidx, st));
    CK(upload(ctx->amap, s.amap, st));
    CK(upload(ctx->dmap, s.dmap, st));
    CK(upload(ctx->sn, s.sn, st));
    CK(upload(ctx->rows, s.rows, st));
    CK(upload(ctx->relind, s.relind, st));
    CK(upload(ctx->child, s.child, st));
    CK(upload(ctx->level_sn, s.level_sn, st));
    CK(upload(ctx->fitems, s.fitems, st));
    // solve scheduling state: ticket counters and per-supernode flags start at 0
    // counters: forward / backward of the lower levels, then of the top levels
    CK(ctx->ticket.ensure(kTickets * sizeof(unsigned long long)));
    CK(ctx->flags.ensure(2 * sizeof(unsigned) * (size_t)std::max(s.S, 1)));
    CK(cudaMemsetAsync(ctx->ticket.p, 0, kTickets * sizeof(unsigned long long), st));
    CK(cudaMemsetAsync(ctx->flags.p, 0, 2 * sizeof(unsigned) * (size_t)std::max(s.S, 1), st));
    // the solve kernels stream a front's matrices through chunk buffers
    // (whole columns for fronts of one pass, row segments of each pass for
    // larger ones, so columns may have any length) and keep the front's
    // vectors in shared memory. The FP64 form needs twice the bytes: when
    // only the mixed form fits, FP64 deforms are refused.
    const int max_rows = std::max(s.max_ldx, s.max_ld21);
    const size_t b32 = solve_smem_bytes(s.max_ldx, s.max_ld21, 4), b64 = solve_smem_bytes(s.max_ldx, s.max_ld21, 8);
    constexpr size_t kSmemMax = 227 * 1024;
    if (b32 > kSmemMax)
        return fail(ctx, ARAP_ERR_UNSUPPORTED,
                    "supernode front of " + std::to_string(max_rows) + " rows (" + std::to_string(s.max_ncol) +
                        " columns) exceeds the solve kernels' shared memory");
    ctx->fp64_solves = b64 <= kSmemMax;
    if (b32 > ctx->smem_f32 || (ctx->fp64_solves && b64 > ctx->smem_f64)) {
        CK(configure_solve_smem((int)b32, ctx->fp64_solves ? (int)b64 : 0));
        ctx->smem_f32 = b32;
        if (ctx->fp64_solves) ctx->smem_f64 = b64;
    }
    DevSym &d = ctx->ds;
    {
        // split of the tree between the single-CTA and the cluster solves
        const int nlev = (int)s.level_ptr.size() - 1;
        std::vector<char> big(std::max(nlev, 1), 0);
        for (const SnInfo &q : s.sn) {
            const int64_t bytes = ((int64_t)q.ldx * q.ncol + (int64_t)q.ld21 * q.ncol) * 4;
            const int64_t thr = ctx->top_bytes == 0 ? kTopTaskBytes : ctx->top_bytes;
            if (ctx->top_bytes >= 0 && bytes >= thr) big[q.level] = 1;
        }
        int ltop = nlev;
        while (ltop > 0 && big[ltop - 1]) --ltop;
        // the cluster solves take fronts of at most kSolveBlockRows rows
        for (const SnInfo &q : s.sn)
            if (q.level >= ltop && std::max(q.ldx, q.ld21) > kSolveBlockRows) ltop = std::max(ltop, q.level + 1);
        // the dense top, where its inversion's and its solves' shared memory
        // fit, takes the top levels instead of the clusters
        d.n_top = d.n_top_items = d.dense_ldx = d.dense_ld21 = 0;
        const DenseTopChoice dtop = choose_dense_top(s, dense_cap(ctx));
        if (dtop.ncols > 0) {
            int ldxm = 0, ld21m = 0;
            for (int q = s.level_ptr[dtop.level]; q < s.level_ptr[nlev]; ++q) {
                const SnInfo &x = s.sn[s.level_sn[q]];
                ldxm = std::max(ldxm, (int)x.ldx);
                ld21m = std::max(ld21m, (int)x.ld21);
            }
            const int rc32 = dense_inverse_rhs(ldxm, ld21m, 4), rc64 = dense_inverse_rhs(ldxm, ld21m, 8);
            const size_t i32 = rc32 > 0 ? dense_inverse_smem_bytes(ldxm, ld21m, 4, rc32) : 0;
            const size_t i64 = rc64 > 0 ? dense_inverse_smem_bytes(ldxm, ld21m, 8, rc64) : 0;
            if (rc32 > 0 && rc64 > 0) {
                const int rc_d = prepare_dense_top(ctx, dtop.level, dtop.ncols);
                if (rc_d != ARAP_OK) return rc_d;
                if (i32 > ctx->dense_inv_smem[0] || i64 > ctx->dense_inv_smem[1]) {
                    CK(configure_dense_smem((int)i32, (int)i64));
                    ctx->dense_inv_smem[0] = std::max(ctx->dense_inv_smem[0], i32);
                    ctx->dense_inv_smem[1] = std::max(ctx->dense_inv_smem[1], i64);
                }
                d.dense_ldx = ldxm;
                d.dense_ld21 = ld21m;
                ltop = dtop.level;
            }
        }
        d.ltop = ltop;
        d.s_low = nlev > 0 ? s.level_ptr[ltop] : 0;
        // the bottom levels whose fronts all fit a warp task
        int lwarp = 0;
        const int wrows = std::min(ctx->warp_rows, wsolve_max_rows());
        while (wrows > 0 && lwarp < ltop) {
            int mx = 0;
            for (int q = s.level_ptr[lwarp]; q < s.level_ptr[lwarp + 1]; ++q) mx = std::max(mx, (int)s.sn[s.level_sn[q]].nrow);
            if (mx > wrows) break;
            ++lwarp;
        }
        d.lwarp = lwarp;
        d.s_warp = nlev > 0 ? s.level_ptr[lwarp] : 0;
        if (d.s_warp > 0) {
            CK(configure_wsolve());
            const int cap = ctx->solve_cap;
            const int need = (d.s_warp + 7) / 8;
            const int r32 = wsolve_resident_ctas(4), r64 = wsolve_resident_ctas(8);
            d.wgrid32 = std::max(1, std::min(need, cap > 0 ? std::min(cap, r32) : r32));
            d.wgrid64 = std::max(1, std::min(need, cap > 0 ? std::min(cap, r64) : r64));
        } else {
            d.wgrid32 = d.wgrid64 = 0;
        }
        d.s_top = d.n_top > 0 ? 0 : s.S - d.s_low;
        int width = 0;
        for (int l = ltop; l < nlev; ++l) width = std::max(width, s.level_ptr[l + 1] - s.level_ptr[l]);
        d.top_clusters = std::max(1, std::min(width, kTopMaxClusters));
        const int res32 = solve_resident_ctas((int)b32, 4), res64 = solve_resident_ctas((int)b64, 8);
        const int cap = ctx->solve_cap;
        const int nl = std::max(d.s_low - d.s_warp, 1);
        d.solve_grid32 = std::max(1, std::min(nl, cap > 0 ? std::min(cap, res32) : res32));
        d.solve_grid64 = std::max(1, std::min(nl, cap > 0 ? std::min(cap, res64) : res64));
        d.overlap = cap <= 0;
        // level schedule: per level its supernodes, the shared memory its
        // largest front needs and a grid of at most one CTA per supernode
        d.level_launch = ctx->solve_schedule == ARAP_SOLVE_LEVELS && nlev <= kMaxLevelLaunch;
        for (int l = 0; l <= kMaxLevelLaunch; ++l) d.lev_ptr[l] = nlev > 0 ? s.level_ptr[std::min(l, nlev)] : 0;
        for (int l = 0; l < kMaxLevelLaunch; ++l) {
            int lx = 0, l21 = 0;
            for (int q = d.lev_ptr[l]; q < d.lev_ptr[l + 1]; ++q) {
                const SnInfo &x = s.sn[s.level_sn[q]];
                lx = std::max(lx, (int)x.ldx);
                l21 = std::max(l21, (int)x.ld21);
            }
            d.lev_ldx[l] = lx;
            d.lev_ld21[l] = l21;
            const int n = std::max(d.lev_ptr[l + 1] - d.lev_ptr[l], 1);
            const int r32 = solve_resident_ctas((int)solve_smem_bytes(lx, l21, 4), 4);
            const int r64 = solve_resident_ctas((int)solve_smem_bytes(lx, l21, 8), 8);
            d.lev_grid32[l] = std::max(1, std::min(n, cap > 0 ? std::min(cap, r32) : r32));
            d.lev_grid64[l] = std::max(1, std::min(n, cap > 0 ? std::min(cap, r64) : r64));
        }
        // the cluster solves size their shared memory by the largest front of
        // the cluster levels
        d.top_ldx = d.top_ld21 = 0;
        for (const SnInfo &q : s.sn)
            if (q.level >= ltop && d.s_top > 0) {
                d.top_ldx = std::max(d.top_ldx, (int)q.ldx);
                d.top_ld21 = std::max(d.top_ld21, (int)q.ld21);
            }
        if (d.s_top > 0) {
            const size_t t32 = top_smem_bytes(d.top_ldx, d.top_ld21, 4), t64 = top_smem_bytes(d.top_ldx, d.top_ld21, 8);
            if (t32 > kSmemMax)
                return fail(ctx, ARAP_ERR_UNSUPPORTED, "top supernode fronts exceed the cluster solve's shared memory");
            if (t64 > kSmemMax) ctx->fp64_solves = false;
            if (t32 > ctx->top_smem_f32 || (t64 <= kSmemMax && t64 > ctx->top_smem_f64)) {
                CK(configure_top_smem((int)t32, t64 <= kSmemMax ? (int)t64 : 0));
                ctx->top_smem_f32 = t32;
                if (t64 <= kSmemMax) ctx->top_smem_f64 = t64;
            }
        }
    }
    d.V = s.V;
    d.m = s.m;
    d.S = s.S;
    d.s_sched = s.S;
    for (int k = 0; k < kVertexKernels; ++k) d.vlaunch[k] = ctx->vlaunch[k];
    d.nnz = (int)s.dcol.size();
    d.max_ldx = s.max_ldx;
    d.max_ld21 = s.max_ld21;
    d.max_ncol = s.max_ncol;
    d.drow = ctx->drow.as<int32_t>();
    d.dcol = ctx->dcol.as<int32_t>();
    d.dent = ctx->dent.as<int32_t>();
    d.oldidx = ctx->oldidx.as<int32_t>();
    d.amap = ctx->amap.as<int64_t>();
    d.dmap = ctx->dmap.as<int64_t>();
    d.sn = ctx->sn.as<SnInfo>();
    d.rows = ctx->rows.as<int32_t>();
    d.relind = ctx->relind.as<int32_t>();
    d.child = ctx->child.as<int32_t>();
    d.level_sn = ctx->level_sn.as<int32_t>();
    d.top_col = ctx->top_col.as<int32_t>();
    d.top_gptr = ctx->top_gptr.as<int32_t>();
    d.top_gidx = ctx->top_gidx.as<int64_t>();
    d.tdpos = ctx->tdpos.as<int32_t>();
    d.top_items = ctx->top_items.as<int32_t>();
    if (ctx->use_sb) {
        const int rc_b = prepare_solve_blocks(ctx);
        if (rc_b != ARAP_OK) return rc_b;
    }
    ctx->sym_valid = true;
    return ARAP_OK;
}


// Allocates (or keeps) every buffer the setup and the iterations of precision
// T use. Any reallocation bumps ctx->gen so captured graphs are rebuilt.
template <typename T>
int setup_alloc(arap_ctx *ctx) {
    std::vector<std::pair<DevBuf *, size_t>> plan;
    planned_sizes<T>(ctx, 0, plan);
    bool moved = false;
    for (auto &pb : plan) {
        void *before = pb.first->p;
        CK(pb.first->ensure(pb.second));
        moved |= before != pb.first->p;
    }
    if (moved) ctx->gen++;
    return ARAP_OK;
}

// Enqueues the numeric factorisation in precision TF: the constrained
// Laplacian assembled into the supernodal panels (and bFixed) and the
// multifrontal Cholesky plan level by level (every launch but the inverses').
template <typename TF>
int factor_numeric(arap_ctx *ctx, TF *Lval, TF *Upd, TF *Dinv) {
    const Symbolic &s = ctx->sym;
    const DevSym &d = ctx->ds;
    cudaStream_t st = ctx->stream;
    CK(cudaMemsetAsync(Lval, 0, (size_t)s.panel_size * sizeof(TF), st));
    if (s.upd_size > 0) CK(cudaMemsetAsync(Upd, 0, (size_t)s.upd_size * sizeof(TF), st));
    {
        Prof pr(ctx, ARAP_K_ASSEMBLE);
        launch_assemble<TF>(d, ctx->w64.as<double>(), ctx->pc64.as<Vec4<double>>(), Lval, ctx->diag64.as<double>(),
                            ctx->bfixed.as<Vec4<double>>(), st);
    }
    ctx->launches += 1;
    for (const FactorLaunch &fl : s.fplan) {
        if (fl.kind == kFx) continue;
        Prof pr(ctx, ARAP_K_FACTOR);
        launch_factor_step<TF>(d, fl, ctx->fitems.as<FItem>(), Lval, Upd, Dinv, nullptr, nullptr, nullptr,
                               ctx->errw.as<int>(), st);
        ctx->launches += 1;
    }
    CK(cudaGetLastError());
    return ARAP_OK;
}

// Enqueues the arrays the triangular solves multiply by, in precision TI,
// from a factor (panels and inverted diagonal blocks) in that precision:
// X = inv(L11) and X^T per supernode, the aligned L21 / L21^T copies, and the
// dense top's T = inv(L_top). The factor no longer changes when they run.
template <typename TI>
int factor_inverses(arap_ctx *ctx, const TI *Lval, const TI *Dinv, TI *X, TI *L21, TI *L21T, TI *Ttop) {
    const Symbolic &s = ctx->sym;
    const DevSym &d = ctx->ds;
    cudaStream_t st = ctx->stream;
    CK(cudaMemsetAsync(X, 0, (size_t)s.x_size * sizeof(TI), st));
    if (s.l21_size > 0) CK(cudaMemsetAsync(L21, 0, (size_t)s.l21_size * sizeof(TI), st));
    if (s.l21t_size > 0) CK(cudaMemsetAsync(L21T, 0, (size_t)s.l21t_size * sizeof(TI), st));
    // (the solve blocks' arrays after them are written whole by their kernel)
    for (const FactorLaunch &fl : s.fplan) {
        if (fl.kind != kFx) continue;
        Prof pr(ctx, ARAP_K_FACTOR);
        launch_factor_step<TI>(d, fl, ctx->fitems.as<FItem>(), const_cast<TI *>(Lval), nullptr, const_cast<TI *>(Dinv),
                               X, L21, L21T, ctx->errw.as<int>(), st);
        ctx->launches += 1;
    }
    if (ctx->use_sb) {
        Prof pr(ctx, ARAP_K_FACTOR);
        launch_solve_blocks<TI>(ctx->sb.nblocks, ctx->sbitems.as<int32_t>(), ctx->sbmembers.as<int32_t>(), d.sn,
                                ctx->ssn.as<SnInfo>(), d.relind, Lval, X, L21, L21T, st);
        ctx->launches += 1;
    }
    if (d.n_top > 0) {
        Prof pr(ctx, ARAP_K_FACTOR);
        launch_top_inverse<TI>(d, X, L21, Ttop, st);
        ctx->launches += 1;
    }
    CK(cudaGetLastError());
    return ARAP_OK;
}

// Enqueues the dirty-deform setup in precision T (FP64: T = double for
// everything; MIXED: T = float for the local step, RHS and solves, with the
// factor in FP64 unless factor_bits is 32):
// cotan weights, geometry and constraint snap, rotations reset, Laplacian and
// bFixed assembly, the factorisation plan. No host synchronisation; a failed
// pivot shows up in the device error word.
template <typename T>
int setup_enqueue(arap_ctx *ctx) {
    const Symbolic &s = ctx->sym;
    const DevSym &d = ctx->ds;
    cudaStream_t st = ctx->stream;
    const int m = s.m;
    // the solves' scheduling counters and flags restart with every set-up: a
    // launch consumes tickets in proportion to its grid, which differs
    // between the precisions
    CK(cudaMemsetAsync(ctx->ticket.p, 0, kTickets * sizeof(unsigned long long), st));
    CK(cudaMemsetAsync(ctx->flags.p, 0, 2 * sizeof(unsigned) * (size_t)std::max(s.S, 1), st));
    // and the dense top's arrival counters
    if (ctx->ytop.p) CK(cudaMemsetAsync(ctx->ytop.p, 0, ctx->ytop.cap, st));
    // cotan weights (arap.h:182-239)
    {
        Prof pr(ctx, ARAP_K_WEIGHTS);
        launch_edge_weights(ctx->dt, d, ctx->hc.as<double>(), ctx->w64.as<double>(),
                            sizeof(T) == 4 ? ctx->w32.as<float>() : nullptr, ctx->w_orig.as<double>(), st);
    }
    // geometry, constraint snap, rotations = I
    Vec4<T> *p_t = sizeof(T) == 4 ? ctx->p32.as<Vec4<T>>() : ctx->p64.as<Vec4<T>>();
    Vec4<T> *pc_t = sizeof(T) == 4 ? ctx->pc32.as<Vec4<T>>() : ctx->pc64.as<Vec4<T>>();
    {
        Prof pr(ctx, ARAP_K_ASSEMBLE);
        launch_setup_vertices<T>(d, ctx->rest.as<double>(), ctx->targets.as<double>(), ctx->p64.as<Vec4<double>>(),
                                 ctx->pc64.as<Vec4<double>>(), p_t, pc_t, ctx->R.as<Vec4<T>>(), st);
        if (sizeof(T) == 4) launch_rest_edges(d, ctx->p64.as<Vec4<double>>(), ctx->redge.as<Vec4<float>>(), st);
    }
    ctx->launches += sizeof(T) == 4 ? 3 : 2;
    if (m > 0) {
        int rc;
        if (sizeof(T) == 4 && ctx->factor_bits == 64) {
            // FP64 numeric factorisation (arap.h:337 factors in double); the
            // factor is then rounded to FP32, and the arrays the FP32 solves
            // multiply by (the supernodes' X = inv(L11), the dense top's T)
            // are formed from it in FP32: they carry FP32 accuracy either way,
            // and the FP64 residual refinement restores the rest
            rc = factor_numeric<double>(ctx, ctx->Lval.as<double>(), ctx->Upd.as<double>(), ctx->Dinv.as<double>());
            if (rc != ARAP_OK) return rc;
            {
                const double *src[2] = {ctx->Lval.as<double>(), ctx->Dinv.as<double>()};
                float *dst[2] = {ctx->Lval32.as<float>(), ctx->Dinv32.as<float>()};
                const int64_t n[2] = {s.panel_size, s.dinv_size};
                Prof pr(ctx, ARAP_K_FACTOR);
                launch_demote(2, src, dst, n, st);
                ctx->launches += 1;
            }
            rc = factor_inverses<float>(ctx, ctx->Lval32.as<float>(), ctx->Dinv32.as<float>(), ctx->Xinv.as<float>(),
                                        ctx->L21.as<float>(), ctx->L21T.as<float>(), ctx->Ttop.as<float>());
            if (rc != ARAP_OK) return rc;
        } else {
            rc = factor_numeric<T>(ctx, ctx->Lval.as<T>(), ctx->Upd.as<T>(), ctx->Dinv.as<T>());
            if (rc != ARAP_OK) return rc;
            rc = factor_inverses<T>(ctx, ctx->Lval.as<T>(), ctx->Dinv.as<T>(), ctx->Xinv.as<T>(), ctx->L21.as<T>(),
                                    ctx->L21T.as<T>(), ctx->Ttop.as<T>());
            if (rc != ARAP_OK) return rc;
        }
    }
    CK(cudaGetLastError());
    return ARAP_OK;
}

// Enqueues a re-pose of the set-up problem (arap_set_targets): positions back
// to the rest pose with the constrained vertices at their new targets,
// rotations reset, bFixed recomputed; weights and factor stay.
template <typename T>
int retarget_enqueue(arap_ctx *ctx) {
    const DevSym &d = ctx->ds;
    cudaStream_t st = ctx->stream;
    Vec4<T> *p_t = sizeof(T) == 4 ? ctx->p32.as<Vec4<T>>() : ctx->p64.as<Vec4<T>>();
    Vec4<T> *pc_t = sizeof(T) == 4 ? ctx->pc32.as<Vec4<T>>() : ctx->pc64.as<Vec4<T>>();
    {
        Prof pr(ctx, ARAP_K_ASSEMBLE);
        launch_setup_vertices<T>(d, ctx->rest.as<double>(), ctx->targets.as<double>(), ctx->p64.as<Vec4<double>>(),
                                 ctx->pc64.as<Vec4<double>>(), p_t, pc_t, ctx->R.as<Vec4<T>>(), st);
        launch_bfixed(d, ctx->w64.as<double>(), ctx->pc64.as<Vec4<double>>(), ctx->bfixed.as<Vec4<double>>(), st);
    }
    ctx->launches += 2;
    CK(cudaGetLastError());
    return ARAP_OK;
}

// Runs `enqueue` directly, or through a CUDA graph captured from it and kept
// while `key` stays the same.
template <class F>
int graph_or_direct(arap_ctx *ctx, cudaGraphExec_t &exec, int64_t key_store[4], const int64_t key[4],
                    int64_t &nlaunch, F enqueue) {
    cudaStream_t st = ctx->stream;
    if (!ctx->use_graphs || ctx->profiling) return enqueue();
    const bool same_key = key_store[0] == key[0] && key_store[1] == key[1] && key_store[2] == key[2] &&
                          key_store[3] == key[3];
    if (!same_key) {
        // first use of this key: launch directly and only remember the key; a
        // graph is captured when the same sequence comes again (one-shot
        // contexts never pay for capture and instantiation)
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        for (int i = 0; i < 4; ++i) key_store[i] = key[i];
        return enqueue();
    }
    if (!exec) {
        const int64_t before = ctx->launches;
        CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        const int rc = enqueue();
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(st, &g);
        if (rc != ARAP_OK) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        CK(e);
        const cudaError_t ei = cudaGraphInstantiate(&exec, g, 0);
        cudaGraphDestroy(g);
        CK(ei);
        nlaunch = ctx->launches - before;
        ctx->launches = before;
    }
    CK(cudaGraphLaunch(exec, st));
    ctx->launches += nlaunch;
    return ARAP_OK;
}

template <typename T>
int run_iterations(arap_ctx *ctx, int iterations);

// kernels of one forward + backward sweep (lower levels and cluster levels)
int solve_launches(const DevSym &d) {
    int cta = d.s_low > d.s_warp;
    if (cta && d.level_launch) {
        cta = 0;
        for (int l = d.lwarp; l < d.ltop; ++l) cta += d.lev_ptr[l + 1] > d.lev_ptr[l];
    }
    // the dense top: one tiled product each way
    return 2 * ((d.s_warp > 0) + cta + (d.s_top > 0)) + (d.n_top > 0 ? 2 : 0);
}

template <>
int run_iterations<double>(arap_ctx *ctx, int iterations) {
    const Symbolic &s = ctx->sym;
    const DevSym &d = ctx->ds;
    const DevSym &dv = ctx->use_sb ? ctx->dss : d;  // the sweeps' layout (with the solve blocks)
    cudaStream_t st = ctx->stream;
    unsigned long long *tk = ctx->ticket.as<unsigned long long>();
    unsigned *fl = ctx->flags.as<unsigned>();
    for (int it = 0; it < iterations; ++it) {
        {
            Prof pr(ctx, ARAP_K_LOCAL);
            launch_local_step<double>(d, ctx->w64.as<double>(), ctx->p64.as<Vec4<double>>(),
                                      ctx->pc64.as<Vec4<double>>(), ctx->R.as<Vec4<double>>(), st);
        }
        ctx->launches += 1;
        if (s.m == 0) continue;
        {
            Prof pr(ctx, ARAP_K_RHS);
            launch_rhs<double>(d, ctx->w64.as<double>(), ctx->p64.as<Vec4<double>>(), ctx->R.as<Vec4<double>>(),
                               ctx->bfixed.as<Vec4<double>>(), ctx->sol.as<Vec4<double>>(), st);
        }
        {
            Prof pr(ctx, ARAP_K_SOLVE_FWD);
            launch_solve_fwd<double>(dv, ctx->Xinv.as<double>(), ctx->L21.as<double>(),
                                     ctx->sol.as<Vec4<double>>(), ctx->uvec.as<Vec4<double>>(), tk, fl,
                                     ctx->errw.as<int>(), st, ctx->Ttop.as<double>(), ctx->ytop.as<Vec4<double>>());
        }
        {
            Prof pr(ctx, ARAP_K_SOLVE_BWD);
            launch_solve_bwd<double>(dv, ctx->Xinv.as<double>(), ctx->L21T.as<double>(),
                                     ctx->sol.as<Vec4<double>>(), ctx->pc64.as<Vec4<double>>(), nullptr, 0, tk + 1,
                                     fl + s.S, ctx->errw.as<int>(), st, ctx->Ttop.as<double>(),
                                     ctx->ytop.as<Vec4<double>>());
        }
        ctx->launches += solve_launches(dv) + 1;
    }
    CK(cudaGetLastError());
    return ARAP_OK;
}

template <>
int run_iterations<float>(arap_ctx *ctx, int iterations) {
    const Symbolic &s = ctx->sym;
    const DevSym &d = ctx->ds;
    const DevSym &dv = ctx->use_sb ? ctx->dss : d;  // the sweeps' layout (with the solve blocks)
    cudaStream_t st = ctx->stream;
    unsigned long long *tk = ctx->ticket.as<unsigned long long>();
    unsigned *fl = ctx->flags.as<unsigned>();
    for (int it = 0; it < iterations; ++it) {
        {
            Prof pr(ctx, ARAP_K_LOCAL);
            launch_local_step_mixed(d, ctx->w32.as<float>(), ctx->redge.as<Vec4<float>>(),
                                    ctx->pc64.as<Vec4<double>>(), ctx->R.as<Vec4<float>>(), ctx->w64.as<double>(),
                                    ctx->p64.as<Vec4<double>>(), st);
        }
        ctx->launches += 1;
        if (s.m == 0) continue;
        {
            Prof pr(ctx, ARAP_K_RHS);
            launch_rhs_mixed(d, ctx->w32.as<float>(), ctx->redge.as<Vec4<float>>(), ctx->R.as<Vec4<float>>(),
                             ctx->b.as<Vec4<float>>(), st);
        }
        ctx->launches += 1;
        for (int r = 0; r <= ctx->refine; ++r) {
            {
                Prof pr(ctx, ARAP_K_RESIDUAL);
                launch_residual(d, ctx->w64.as<double>(), ctx->diag64.as<double>(), ctx->bfixed.as<Vec4<double>>(),
                                ctx->b.as<Vec4<float>>(), ctx->pc64.as<Vec4<double>>(), ctx->sol.as<Vec4<float>>(), st);
            }
            {
                Prof pr(ctx, ARAP_K_SOLVE_FWD);
                launch_solve_fwd<float>(dv, ctx->Xinv.as<float>(), ctx->L21.as<float>(),
                                        ctx->sol.as<Vec4<float>>(), ctx->uvec.as<Vec4<float>>(), tk, fl,
                                        ctx->errw.as<int>(), st, ctx->Ttop.as<float>(), ctx->ytop.as<Vec4<float>>());
            }
            {
                Prof pr(ctx, ARAP_K_SOLVE_BWD);
                launch_solve_bwd<float>(dv, ctx->Xinv.as<float>(), ctx->L21T.as<float>(),
                                        ctx->sol.as<Vec4<float>>(), ctx->pc64.as<Vec4<double>>(),
                                        ctx->pc32.as<Vec4<float>>(), 1, tk + 1, fl + s.S, ctx->errw.as<int>(), st,
                                        ctx->Ttop.as<float>(), ctx->ytop.as<Vec4<float>>());
            }
            ctx->launches += solve_launches(dv) + 1;
        }
    }
    CK(cudaGetLastError());
    return ARAP_OK;
}

// `iterations` local/global iterations of P poses at once (the loop of
// arap.h:122-129 per pose), the two triangular solves each one persistent
// launch over all (supernode, pose tile) tasks.
int run_batch_iterations(arap_ctx *ctx, int P, int iterations) {
    const Symbolic &s = ctx->sym;
    const DevSym &d = ctx->ds;
    const DevSym &dv = ctx->use_sb ? ctx->dss : d;  // the batched sweeps' layout (with the solve blocks)
    cudaStream_t st = ctx->stream;
    const int m = s.m;
    unsigned long long *tk = ctx->bticket.as<unsigned long long>();
    unsigned *fl = ctx->bflags.as<unsigned>();
    const size_t fhalf = (size_t)std::max(s.S, 1) * ctx->bT;
    if (d.n_top > 0 && m > 0 && iterations > 0) {
        // T of this factorisation as the tensor-core products' operand tiles
        launch_btop_pack(d, ctx->Ttop.as<float>(), ctx->batile.as<float>(), st);
        ctx->launches += 2;
    }
    for (int it = 0; it < iterations; ++it) {
        {
            Prof pr(ctx, ARAP_K_LOCAL);
            launch_blocal(d, P, ctx->w32.as<float>(), ctx->redge.as<Vec4<float>>(), ctx->bpc64.as<Vec4<double>>(),
                          ctx->bR.as<Vec4<float>>(), ctx->w64.as<double>(), ctx->p64.as<Vec4<double>>(), st);
        }
        ctx->launches += 1;
        if (m == 0) continue;
        {
            Prof pr(ctx, ARAP_K_RHS);
            launch_brhs(d, P, ctx->w32.as<float>(), ctx->redge.as<Vec4<float>>(), ctx->bR.as<Vec4<float>>(),
                        ctx->bb.as<Vec4<float>>(), st);
        }
        ctx->launches += 1;
        for (int r = 0; r <= ctx->refine; ++r) {
            {
                Prof pr(ctx, ARAP_K_RESIDUAL);
                launch_bresidual(d, P, ctx->w64.as<double>(), ctx->diag64.as<double>(),
                                 ctx->bbfixed.as<Vec4<double>>(), ctx->bb.as<Vec4<float>>(),
                                 ctx->bpc64.as<Vec4<double>>(), ctx->bsol.as<Vec4<float>>(), st);
            }
            {
                Prof pr(ctx, ARAP_K_SOLVE_FWD);
                launch_bsolve(dv, P, ctx->bpt, ctx->bgrid, ctx->Xinv.as<float>(), ctx->L21.as<float>(), ctx->L21T.as<float>(),
                              ctx->bsol.as<Vec4<float>>(), ctx->buvec.as<Vec4<float>>(), nullptr, nullptr, tk, fl,
                              ctx->errw.as<int>(), true, st, ctx->batile.as<float>(), ctx->bftop.as<float>(),
                              ctx->bytop.as<float>(), ctx->bws.as<float>());
            }
            {
                Prof pr(ctx, ARAP_K_SOLVE_BWD);
                launch_bsolve(dv, P, ctx->bpt, ctx->bgrid, ctx->Xinv.as<float>(), ctx->L21.as<float>(), ctx->L21T.as<float>(),
                              ctx->bsol.as<Vec4<float>>(), ctx->buvec.as<Vec4<float>>(), ctx->bpc64.as<Vec4<double>>(),
                              ctx->bpc32.as<Vec4<float>>(), tk + 1, fl + fhalf, ctx->errw.as<int>(), false, st,
                              ctx->batile.as<float>(), ctx->bftop.as<float>(), ctx->bytop.as<float>(),
                              ctx->bws.as<float>());
            }
            ctx->launches += 1 + (batch_tasks(dv) > 0 ? 2 : 0) + batch_top_launches(dv);
        }
    }
    CK(cudaGetLastError());
    return ARAP_OK;
}

int check_ctx(const arap_ctx *ctx) { return ctx ? ARAP_OK : ARAP_ERR_INVALID_ARGUMENT; }

}  // namespace

extern "C" {

const char *arap_status_string(int status) {
    switch (status) {
    case ARAP_OK: return "ARAP_OK";
    case ARAP_ERR_INVALID_ARGUMENT: return "ARAP_ERR_INVALID_ARGUMENT";
    case ARAP_ERR_BAD_INDEX: return "ARAP_ERR_BAD_INDEX";
    case ARAP_ERR_NOT_SPD: return "ARAP_ERR_NOT_SPD";
    case ARAP_ERR_OUT_OF_MEMORY: return "ARAP_ERR_OUT_OF_MEMORY";
    case ARAP_ERR_CUDA: return "ARAP_ERR_CUDA";
    case ARAP_ERR_TIMEOUT: return "ARAP_ERR_TIMEOUT";
    case ARAP_ERR_ADMISSION_REFUSED: return "ARAP_ERR_ADMISSION_REFUSED";
    case ARAP_ERR_NO_DEVICE: return "ARAP_ERR_NO_DEVICE";
    case ARAP_ERR_UNSUPPORTED: return "ARAP_ERR_UNSUPPORTED";
    case ARAP_PENDING: return "ARAP_PENDING";
    default: return "ARAP_ERR_UNKNOWN";
    }
}

const char *arap_last_error(const arap_ctx *ctx) {
    return ctx ? ctx->err.c_str() : g_create_error.c_str();
}

namespace {
// Everything arap_create does after the topology is built: stream, events,
// device copies of the topology (uploaded, or copied from src's), the
// per-mesh buffers. On failure the context is destroyed.
int finish_create(arap_ctx *ctx, int device, const arap_ctx *src, arap_ctx **out) {
    const int n_vertices = ctx->topo.V, n_faces = ctx->topo.F;
    ctx->cmask.assign(n_vertices, 0);
    auto bail = [&](cudaError_t e, const char *what) {
        g_create_error = std::string(what) + ": " + cudaGetErrorString(e);
        arap_destroy(ctx);
        return e == cudaErrorMemoryAllocation ? ARAP_ERR_OUT_OF_MEMORY : ARAP_ERR_CUDA;
    };
    cudaError_t e;
    if ((e = cudaSetDevice(device)) != cudaSuccess) return bail(e, "cudaSetDevice");
    if ((e = keep_pool_memory(device)) != cudaSuccess) return bail(e, "memory pool");
    if ((e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess)
        return bail(e, "cudaStreamCreate");
    for (DevBuf *b : ctx->buffers()) b->st = ctx->stream;
    if ((e = cudaEventCreateWithFlags(&ctx->ev_done, cudaEventDisableTiming)) != cudaSuccess)
        return bail(e, "cudaEventCreate");
    if ((e = cudaEventCreate(&ctx->ev0)) != cudaSuccess) return bail(e, "cudaEventCreate");
    if ((e = cudaEventCreate(&ctx->ev1)) != cudaSuccess) return bail(e, "cudaEventCreate");
    if ((e = cudaEventCreate(&ctx->ev2)) != cudaSuccess) return bail(e, "cudaEventCreate");
    const Topology &t = ctx->topo;
    if (!src) {
        if ((e = upload(ctx->faces, t.faces, ctx->stream)) != cudaSuccess) return bail(e, "upload faces");
        if ((e = upload(ctx->ent_ptr, t.ent_ptr, ctx->stream)) != cudaSuccess) return bail(e, "upload adjacency");
        if ((e = upload(ctx->ent_fc, t.ent_fc, ctx->stream)) != cudaSuccess) return bail(e, "upload adjacency");
    } else {
        const std::pair<DevBuf *, const DevBuf *> copies[] = {
            {&ctx->faces, &src->faces}, {&ctx->ent_ptr, &src->ent_ptr}, {&ctx->ent_fc, &src->ent_fc}};
        for (const auto &c : copies) {
            if ((e = c.first->ensure(c.second->cap)) != cudaSuccess) return bail(e, "alloc");
            if ((e = cudaMemcpyAsync(c.first->p, c.second->p, c.second->cap, cudaMemcpyDeviceToDevice,
                                     ctx->stream)) != cudaSuccess)
                return bail(e, "copy topology");
        }
    }
    if ((e = ctx->hc.ensure((size_t)3 * std::max(n_faces, 1) * sizeof(double))) != cudaSuccess)
        return bail(e, "alloc");
    if ((e = ctx->w_orig.ensure((size_t)std::max(t.nnz(), 1) * sizeof(double))) != cudaSuccess)
        return bail(e, "alloc");
    if ((e = ctx->rest.ensure((size_t)3 * std::max(n_vertices, 1) * sizeof(double))) != cudaSuccess)
        return bail(e, "alloc");
    if ((e = ctx->targets.ensure((size_t)3 * std::max(n_vertices, 1) * sizeof(double))) != cudaSuccess)
        return bail(e, "alloc");
    if ((e = ctx->out.ensure((size_t)9 * std::max(n_vertices, 1) * sizeof(double))) != cudaSuccess)
        return bail(e, "alloc");
    // status word: error bits, then the flag-wait poll limit (0: the default)
    if ((e = ctx->errw.ensure(2 * sizeof(int))) != cudaSuccess) return bail(e, "alloc");
    if ((e = cudaMemsetAsync(ctx->errw.p, 0, 2 * sizeof(int), ctx->stream)) != cudaSuccess) return bail(e, "memset");
    if (!(ctx->herr_host = pinned_words().get())) return bail(cudaErrorMemoryAllocation, "pinned error word");
    *ctx->herr_host = 0;
    if (src && src->have_rest) {
        if ((e = cudaMemcpyAsync(ctx->rest.p, src->rest.p, (size_t)3 * n_vertices * sizeof(double),
                                 cudaMemcpyDeviceToDevice, ctx->stream)) != cudaSuccess)
            return bail(e, "copy rest positions");
        ctx->have_rest = true;
    }
    if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) return bail(e, "sync");
    ctx->dt.V = n_vertices;
    ctx->dt.F = n_faces;
    ctx->dt.nnz = t.nnz();
    ctx->dt.faces = ctx->faces.as<int32_t>();
    ctx->dt.ent_ptr = ctx->ent_ptr.as<int32_t>();
    ctx->dt.ent_fc = ctx->ent_fc.as<int32_t>();
    *out = ctx;
    return ARAP_OK;
}

}  // namespace

int arap_create(int32_t n_vertices, int32_t n_faces, const int32_t *faces, int32_t device, arap_ctx **out) {
    g_create_error.clear();
    if (!out || n_vertices < 0 || n_faces < 0 || (n_faces > 0 && !faces)) {
        g_create_error = "arap_create: invalid argument";
        return ARAP_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        g_create_error = "no CUDA device visible";
        return ARAP_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= ndev) {
        g_create_error = "device ordinal out of range";
        return ARAP_ERR_INVALID_ARGUMENT;
    }
    arap_ctx *ctx = new arap_ctx();
    ctx->device = device;
    std::string err;
    if (!build_topology(n_vertices, n_faces, faces, ctx->topo, err)) {
        g_create_error = err;
        delete ctx;
        return ARAP_ERR_BAD_INDEX;
    }
    return finish_create(ctx, device, nullptr, out);
}

int arap_create_like(const arap_ctx *src, arap_ctx **out) {
    g_create_error.clear();
    if (!out || !src) {
        g_create_error = "arap_create_like: invalid argument";
        return ARAP_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    arap_ctx *ctx = new arap_ctx();
    ctx->device = src->device;
    ctx->topo = src->topo;
    ctx->precision = src->precision;
    ctx->refine = src->refine;
    ctx->factor_bits = src->factor_bits;
    ctx->sym_cache = src->sym_cache;
    ctx->use_graphs = src->use_graphs;
    ctx->solve_cap = src->solve_cap;
    ctx->top_bytes = src->top_bytes;
    ctx->dense_cols = src->dense_cols;
    ctx->warp_rows = src->warp_rows;
    ctx->solve_schedule = src->solve_schedule;
    ctx->solve_blocks = src->solve_blocks;
    for (int k = 0; k < kVertexKernels; ++k) ctx->vlaunch[k] = src->vlaunch[k];
    ctx->ordering = src->ordering;
    return finish_create(ctx, src->device, src, out);
}

void arap_destroy(arap_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (DevBuf *b : ctx->buffers()) b->release();
    for (cudaEvent_t e : ctx->evpool) cudaEventDestroy(e);
    if (ctx->g_setup) cudaGraphExecDestroy(ctx->g_setup);
    for (cudaGraphExec_t g : ctx->g_iter)
        if (g) cudaGraphExecDestroy(g);
    for (cudaGraphExec_t g : ctx->g_biter)
        if (g) cudaGraphExecDestroy(g);
    if (ctx->herr_host) pinned_words().put(ctx->herr_host);
    if (ctx->ev_done) cudaEventDestroy(ctx->ev_done);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->ev2) cudaEventDestroy(ctx->ev2);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

int arap_set_precision(arap_ctx *ctx, int32_t precision, int32_t refine_steps) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    if (ctx->in_flight) {
        const int rc_ = arap_wait(ctx);
        if (rc_ != ARAP_OK) return rc_;
    }
    if (precision != ARAP_PRECISION_FP64 && precision != ARAP_PRECISION_MIXED)
        return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "unknown precision");
    if (refine_steps < 0 || refine_steps > 8) return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "refine_steps outside 0..8");
    ctx->precision = precision;
    ctx->refine = refine_steps;
    ctx->dirty = true;
    return ARAP_OK;
}

int arap_set_factor_precision(arap_ctx *ctx, int32_t bits) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    if (ctx->in_flight) {
        const int rc_ = arap_wait(ctx);
        if (rc_ != ARAP_OK) return rc_;
    }
    if (bits != 32 && bits != 64) return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "factor precision must be 32 or 64 bits");
    if (bits != ctx->factor_bits) {
        ctx->factor_bits = bits;
        ctx->dirty = true;
    }
    return ARAP_OK;
}

int arap_set_rest_positions(arap_ctx *ctx, const double *xyz) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    if (ctx->in_flight) {
        const int rc_ = arap_wait(ctx);
        if (rc_ != ARAP_OK) return rc_;
    }
    if (!xyz && ctx->topo.V > 0) return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "null positions");
    cudaSetDevice(ctx->device);
    if (ctx->topo.V > 0)
        CK(cudaMemcpyAsync(ctx->rest.p, xyz, (size_t)3 * ctx->topo.V * sizeof(double), cudaMemcpyHostToDevice,
                           ctx->stream));
    ctx->have_rest = true;
    ctx->dirty = true;
    ctx->tP = -1;
    return ARAP_OK;
}

int arap_set_constraints(arap_ctx *ctx, int32_t n, const int32_t *indices, const double *xyz) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    if (ctx->in_flight) {
        const int rc_ = arap_wait(ctx);
        if (rc_ != ARAP_OK) return rc_;
    }
    if (n < 0 || (n > 0 && (!indices || !xyz))) return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "invalid constraint arrays");
    const int V = ctx->topo.V;
    for (int i = 0; i < n; ++i)
        if (indices[i] < 0 || indices[i] >= V)
            return fail(ctx, ARAP_ERR_BAD_INDEX,
                        "constraint index " + std::to_string(indices[i]) + " outside [0, " + std::to_string(V) + ")");
    // map semantics: the last target given for a vertex wins
    std::vector<int32_t> last(V, -1);
    for (int i = 0; i < n; ++i) last[indices[i]] = i;
    ctx->cidx.clear();
    ctx->ctgt.clear();
    std::fill(ctx->cmask.begin(), ctx->cmask.end(), 0);
    for (int v = 0; v < V; ++v) {
        if (last[v] < 0) continue;
        ctx->cidx.push_back(v);
        ctx->cmask[v] = 1;
        const double *t = xyz + 3 * (size_t)last[v];
        ctx->ctgt.insert(ctx->ctgt.end(), t, t + 3);
    }
    cudaSetDevice(ctx->device);
    if (!ctx->ctgt.empty())
        CK(cudaMemcpyAsync(ctx->targets.p, ctx->ctgt.data(), ctx->ctgt.size() * sizeof(double),
                           cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));  // the host vector may change on the next call
    ctx->dirty = true;
    ctx->tP = -1;
    return ARAP_OK;
}

int arap_deform_poses_async(arap_ctx *ctx, int32_t n_poses, const double *targets, int32_t iterations,
                            double *out_xyz) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    if (ctx->in_flight) {
        const int rc_ = arap_wait(ctx);
        if (rc_ != ARAP_OK) return rc_;
    }
    std::fill(ctx->host_ms, ctx->host_ms + 5, 0.0);  // phases are timed for arap_deform_async only
    if (n_poses <= 0 || iterations < 0) return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "n_poses must be positive");
    if (ctx->precision != ARAP_PRECISION_MIXED)
        return fail(ctx, ARAP_ERR_UNSUPPORTED, "arap_deform_poses runs the mixed-precision form only");
    if (!ctx->have_rest) return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "rest positions not set");
    if (ctx->cidx.empty()) return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "no constrained vertex");
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    if (ctx->profiling) {
        CK(cudaStreamSynchronize(st));
        collect_profile(ctx);
    }
    ctx->launches = 0;
    ctx->setup_ms = ctx->iter_ms = 0.0;
    CK(cudaEventRecord(ctx->ev0, st));
    CK(cudaMemsetAsync(ctx->errw.p, 0, sizeof(int), st));
    if (ctx->dirty || ctx->state_prec != ARAP_PRECISION_MIXED) {
        {
            Prof pr(ctx, ARAP_K_WEIGHTS);
            launch_face_cots(ctx->dt, ctx->rest.as<double>(), ctx->hc.as<double>(), st);
        }
        ctx->launches += 1;
        if (!ctx->sym_cache) ctx->sym_host = ctx->sym_valid = false;  // analyse again, as SimplicialLDLT::compute
        int rc = prepare_symbolic(ctx);
        if (rc != ARAP_OK) return rc;
        rc = setup_alloc<float>(ctx);
        if (rc != ARAP_OK) return rc;
        rc = setup_enqueue<float>(ctx);
        if (rc != ARAP_OK) return rc;
        // a failed pivot is reported by arap_wait (the device error word)
        ctx->retarget = false;
        ctx->state_prec = ARAP_PRECISION_MIXED;
        ctx->have_rotations = true;
        ctx->dirty = false;
    }
    const Symbolic &s = ctx->sym;
    const DevSym &d = ctx->use_sb ? ctx->dss : ctx->ds;  // the batched sweeps' layout (with the solve blocks)
    const int V = s.V, m = s.m, P = n_poses, nc = V - m;
    int pt = ctx->pose_tile;
    if (pt == 0) pt = batch_pose_tile(d.max_ldx, d.max_ld21);
    else if (!batch_pose_tile_fits(d.max_ldx, d.max_ld21, pt))
        return fail(ctx, ARAP_ERR_UNSUPPORTED,
                    "pose tile " + std::to_string(pt) + " does not fit this mesh's largest supernode");
    if (pt == 0) return fail(ctx, ARAP_ERR_UNSUPPORTED, "supernode fronts too large for the batched solves");
    if (ctx->bgen != ctx->gen || ctx->bP != P || ctx->bpt != pt || ctx->bntop != d.n_top) {
        const size_t smem = batch_solve_smem_bytes(d.max_ldx, d.max_ld21, pt);
        if (pt != ctx->bpt || smem > ctx->bsmem) {
            CK(configure_batch_smem(d.max_ldx, d.max_ld21, pt));
            ctx->bsmem = smem;
        }
        const int T = (P + pt - 1) / pt;
        const size_t VP = (size_t)V * P, MP = (size_t)std::max(m, 1) * P;
        const size_t nflags = (size_t)2 * std::max(s.S, 1) * T;
        const std::pair<DevBuf *, size_t> plan[] = {
            {&ctx->bpc64, VP * sizeof(Vec4<double>)},
            {&ctx->bpc32, VP * sizeof(Vec4<float>)},
            {&ctx->bR, VP * 3 * sizeof(Vec4<float>)},
            {&ctx->bbfixed, MP * sizeof(Vec4<double>)},
            {&ctx->bb, MP * sizeof(Vec4<float>)},
            {&ctx->bsol, MP * sizeof(Vec4<float>)},
            {&ctx->buvec, (size_t)std::max<int64_t>(s.uvec_size, 1) * P * sizeof(Vec4<float>)},
            {&ctx->bout, VP * 3 * sizeof(double)},
            {&ctx->btargets, (size_t)P * nc * 3 * sizeof(double)},
            {&ctx->bticket, 2 * sizeof(unsigned long long)},
            {&ctx->bflags, nflags * sizeof(unsigned)},
            {&ctx->bftop, std::max<size_t>(btop_matrix_floats(d.n_top, P), 1) * sizeof(float)},
            {&ctx->bytop, std::max<size_t>(btop_matrix_floats(d.n_top, P), 1) * sizeof(float)},
            {&ctx->bws, std::max<size_t>(btop_workspace_floats(d.n_top, P), 1) * sizeof(float)},
            {&ctx->batile, std::max<size_t>(btop_atile_floats(d.n_top), 1) * sizeof(float)}};
        bool moved = false;
        void *const old_targets = ctx->btargets.p;
        for (const auto &pb : plan) {
            void *before = pb.first->p;
            CK(pb.first->ensure(pb.second));
            moved |= before != pb.first->p;
        }
        if (moved) ctx->gen++;  // captured graphs hold the old addresses
        if (ctx->btargets.p != old_targets) ctx->tP = -1;
        // scheduling counters restart: each launch then consumes a fixed
        // number of tickets (tasks + CTAs), so the grid is fixed with them
        CK(cudaMemsetAsync(ctx->bticket.p, 0, 2 * sizeof(unsigned long long), st));
        CK(cudaMemsetAsync(ctx->bflags.p, 0, nflags * sizeof(unsigned), st));
        // the products' B tiles: entries past the top's rows and the poses'
        // columns are never written and must read as zero
        CK(cudaMemsetAsync(ctx->bftop.p, 0, ctx->bftop.cap, st));
        CK(cudaMemsetAsync(ctx->bytop.p, 0, ctx->bytop.cap, st));
        int grid = batch_grid(d, P, pt);
        if (ctx->solve_cap > 0) grid = std::min(grid, ctx->solve_cap);
        ctx->bpt = pt;
        ctx->bT = T;
        ctx->bgrid = grid;
        ctx->bP = P;
        ctx->bntop = d.n_top;
        ctx->bgen = ctx->gen;
    }
    if (!targets && ctx->tP < 0) return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "no targets on the device yet");
    if (!targets && ctx->tP != P)
        return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "the targets on the device are for another pose count");
    if (targets) {
        CK(cudaMemcpyAsync(ctx->btargets.p, targets, (size_t)P * nc * 3 * sizeof(double), cudaMemcpyHostToDevice,
                           st));
        ctx->tP = P;
    }
    {
        Prof pr(ctx, ARAP_K_ASSEMBLE);
        launch_bsetup(d, P, ctx->p64.as<Vec4<double>>(), ctx->btargets.as<double>(), ctx->bpc64.as<Vec4<double>>(),
                      ctx->bpc32.as<Vec4<float>>(), ctx->bR.as<Vec4<float>>(), st);
        launch_bbfixed(d, P, ctx->w64.as<double>(), ctx->bpc64.as<Vec4<double>>(), ctx->bbfixed.as<Vec4<double>>(),
                       st);
    }
    ctx->launches += 2;
    CK(cudaEventRecord(ctx->ev1, st));
    ctx->model_P = P;
    ctx->model_T = ctx->bT;
    ctx->model_batched = true;
    for (int left = iterations; left > 0;) {
        int k = 0;
        while (k + 1 < arap_ctx::kIterGraphs && (2 << k) <= left) ++k;
        const int n = 1 << k;
        const int64_t key[4] = {ctx->gen, P, n + ((int64_t)ctx->refine << 32),
                                ctx->bpt + ((int64_t)ctx->bgrid << 32)};
        const int rc = graph_or_direct(ctx, ctx->g_biter[k], ctx->g_biter_key[k], key, ctx->g_biter_launches[k],
                                       [&] { return run_batch_iterations(ctx, P, n); });
        if (rc != ARAP_OK) return rc;
        left -= n;
    }
    CK(cudaGetLastError());
    CK(cudaEventRecord(ctx->ev2, st));
    if (out_xyz) {
        {
            Prof pr(ctx, ARAP_K_GATHER);
            launch_bgather(d, P, ctx->bpc64.as<Vec4<double>>(), ctx->bout.as<double>(), st);
        }
        ctx->launches += 1;
        CK(cudaMemcpyAsync(out_xyz, ctx->bout.p, (size_t)P * V * 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
    }
    CK(cudaMemcpyAsync(ctx->herr_host, ctx->errw.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaEventRecord(ctx->ev_done, st));
    if (ctx->done_fn) CK(cudaLaunchHostFunc(st, ctx->done_fn, ctx->done_user));
    CK(cudaGetLastError());
    ctx->in_flight = true;
    ctx->poses_in_flight = true;
    return ARAP_OK;
}

int arap_deform_poses(arap_ctx *ctx, int32_t n_poses, const double *targets, int32_t iterations,
                      double *out_xyz) {
    const int rc = arap_deform_poses_async(ctx, n_poses, targets, iterations, out_xyz);
    if (rc != ARAP_OK) return rc;
    return arap_wait(ctx);
}

namespace {
// a = b * c for row-major 3x4 affine matrices (implicit last row 0 0 0 1)
void affine_mul(const double *b, const double *c, double *a) {
    for (int r = 0; r < 3; ++r) {
        for (int k = 0; k < 4; ++k) {
            double v = b[4 * r] * c[k] + b[4 * r + 1] * c[4 + k] + b[4 * r + 2] * c[8 + k];
            if (k == 3) v += b[4 * r + 3];
            a[4 * r + k] = v;
        }
    }
}
}  // namespace

int arap_pose_targets(arap_ctx *ctx, int32_t n_handles, const int32_t *handles, const double *origin,
                      int32_t n_poses, const double *transforms) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    if (ctx->in_flight) {
        const int rc_ = arap_wait(ctx);
        if (rc_ != ARAP_OK) return rc_;
    }
    if (n_poses <= 0 || n_handles < 0 || !transforms || (n_handles > 0 && !handles))
        return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "invalid pose arrays");
    if (!ctx->have_rest) return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "rest positions not set");
    const int nc = (int)ctx->cidx.size();
    if (nc == 0) return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "no constrained vertex");
    std::vector<uint8_t> is_handle(nc, 0);
    for (int h = 0; h < n_handles; ++h) {
        const auto it = std::lower_bound(ctx->cidx.begin(), ctx->cidx.end(), handles[h]);
        if (it == ctx->cidx.end() || *it != handles[h])
            return fail(ctx, ARAP_ERR_BAD_INDEX,
                        "handle " + std::to_string(handles[h]) + " is not a constrained vertex");
        is_handle[it - ctx->cidx.begin()] = 1;
    }
    // tabs = origin * t * origin^-1, the inverse taken as an isometry's
    // ([R^T | -R^T x]), as Transform::inverse(Eigen::Isometry) does
    static const double identity[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
    const double *O = origin ? origin : identity;
    double Oinv[12];
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) Oinv[4 * r + c] = O[4 * c + r];
        Oinv[4 * r + 3] = -(O[r] * O[3] + O[4 + r] * O[7] + O[8 + r] * O[11]);
    }
    std::vector<double> tabs((size_t)12 * n_poses);
    for (int p = 0; p < n_poses; ++p) {
        double tmp[12];
        affine_mul(O, transforms + 12 * (size_t)p, tmp);
        affine_mul(tmp, Oinv, tabs.data() + 12 * (size_t)p);
    }
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    CK(upload(ctx->cidx_dev, ctx->cidx, st));
    CK(upload(ctx->handle_dev, is_handle, st));
    CK(upload(ctx->tabs_dev, tabs, st));
    CK(ctx->btargets.ensure((size_t)n_poses * nc * 3 * sizeof(double)));
    launch_pose_targets(n_poses, nc, ctx->cidx_dev.as<int32_t>(), ctx->handle_dev.as<uint8_t>(), ctx->rest.as<double>(),
                        ctx->targets.as<double>(), ctx->tabs_dev.as<double>(), ctx->btargets.as<double>(), st);
    CK(cudaGetLastError());
    ctx->tP = n_poses;
    return ARAP_OK;
}

int arap_set_targets(arap_ctx *ctx, int32_t n, const double *xyz) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    if (ctx->in_flight) {
        const int rc_ = arap_wait(ctx);
        if (rc_ != ARAP_OK) return rc_;
    }
    if (n != (int32_t)ctx->cidx.size() || (n > 0 && !xyz))
        return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "arap_set_targets needs one target per constrained vertex");
    std::memcpy(ctx->ctgt.data(), xyz, sizeof(double) * 3 * (size_t)n);
    CK(cudaSetDevice(ctx->device));
    // a copy from pageable memory returns once the source is staged, so the
    // host vector may change right after
    if (n > 0)
        CK(cudaMemcpyAsync(ctx->targets.p, ctx->ctgt.data(), ctx->ctgt.size() * sizeof(double),
                           cudaMemcpyHostToDevice, ctx->stream));
    if (!ctx->dirty) ctx->retarget = true;
    return ARAP_OK;
}

int64_t arap_device_bytes(const arap_ctx *ctx);

int arap_invalidate(arap_ctx *ctx) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    ctx->dirty = true;
    return ARAP_OK;
}

int arap_deform_async(arap_ctx *ctx, int32_t iterations, double *out_xyz) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    if (iterations < 0) return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "negative iteration count");
    if (!ctx->have_rest) return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "rest positions not set");
    if (ctx->in_flight) {
        const int rc = arap_wait(ctx);
        if (rc != ARAP_OK) return rc;
    }
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    if (ctx->profiling) {
        CK(cudaStreamSynchronize(st));
        collect_profile(ctx);
    }
    ctx->launches = 0;
    ctx->setup_ms = ctx->iter_ms = 0.0;
    ctx->model_P = ctx->model_T = 1;
    ctx->model_batched = false;
    const bool fp64 = ctx->precision == ARAP_PRECISION_FP64;
    using HClock = std::chrono::steady_clock;
    auto hms = [](HClock::time_point a, HClock::time_point b) {
        return std::chrono::duration<double, std::milli>(b - a).count();
    };
    const auto h0 = HClock::now();
    auto h1 = h0, h2 = h0, h3 = h0, h4 = h0;
    CK(cudaEventRecord(ctx->ev0, st));
    CK(cudaMemsetAsync(ctx->errw.p, 0, sizeof(int), st));
    if (ctx->dirty) {
        {
            Prof pr(ctx, ARAP_K_WEIGHTS);
            launch_face_cots(ctx->dt, ctx->rest.as<double>(), ctx->hc.as<double>(), st);
        }
        ctx->launches += 1;
        if (ctx->cidx.empty()) {
            // arap.h:113-114: no constrained vertex -> weights only, no write-back
            launch_edge_weights_orig(ctx->dt, ctx->hc.as<double>(), ctx->w_orig.as<double>(), st);
            ctx->launches += 1;
            CK(cudaGetLastError());
            CK(cudaStreamSynchronize(st));
            ctx->have_rotations = false;
            return ARAP_OK;
        }
        if (!ctx->sym_cache) ctx->sym_host = ctx->sym_valid = false;  // analyse again, as SimplicialLDLT::compute
        int rc = prepare_symbolic(ctx);
        if (rc != ARAP_OK) return rc;
        if (fp64 && !ctx->fp64_solves)
            return fail(ctx, ARAP_ERR_UNSUPPORTED,
                        "supernode fronts too large for the FP64 solves' shared memory (the mixed form handles them)");
        h1 = HClock::now();
        rc = fp64 ? setup_alloc<double>(ctx) : setup_alloc<float>(ctx);
        if (rc != ARAP_OK) return rc;
        h2 = HClock::now();
        const int64_t key[4] = {ctx->gen, fp64 ? 1 : 2, fp64 ? 64 : ctx->factor_bits, 0};
        rc = graph_or_direct(ctx, ctx->g_setup, ctx->g_setup_key, key, ctx->g_setup_launches, [&] {
            return fp64 ? setup_enqueue<double>(ctx) : setup_enqueue<float>(ctx);
        });
        if (rc != ARAP_OK) return rc;
        ctx->state_prec = fp64 ? ARAP_PRECISION_FP64 : ARAP_PRECISION_MIXED;
        ctx->have_rotations = true;
        ctx->dirty = false;
        ctx->retarget = false;
    } else if (ctx->retarget) {
        const int rc = ctx->state_prec == ARAP_PRECISION_FP64 ? retarget_enqueue<double>(ctx)
                                                               : retarget_enqueue<float>(ctx);
        if (rc != ARAP_OK) return rc;
        ctx->retarget = false;
    }
    h1 = std::max(h1, h0);
    h2 = std::max(h2, h1);
    h3 = HClock::now();
    CK(cudaEventRecord(ctx->ev1, st));
    for (int left = iterations; left > 0;) {
        const bool it64 = ctx->state_prec == ARAP_PRECISION_FP64;
        int k = 0;
        while (k + 1 < arap_ctx::kIterGraphs && (2 << k) <= left) ++k;
        const int n = 1 << k;
        const int64_t key[4] = {ctx->gen, it64 ? 1 : 2, n, ctx->refine};
        const int rc = graph_or_direct(ctx, ctx->g_iter[k], ctx->g_iter_key[k], key, ctx->g_iter_launches[k], [&] {
            return it64 ? run_iterations<double>(ctx, n) : run_iterations<float>(ctx, n);
        });
        if (rc != ARAP_OK) return rc;
        left -= n;
    }
    h4 = HClock::now();
    CK(cudaEventRecord(ctx->ev2, st));
    if (out_xyz) {
        {
            Prof pr(ctx, ARAP_K_GATHER);
            launch_gather_positions(ctx->ds, ctx->pc64.as<Vec4<double>>(), ctx->out.as<double>(), st);
        }
        ctx->launches += 1;
        CK(cudaMemcpyAsync(out_xyz, ctx->out.p, (size_t)3 * ctx->topo.V * sizeof(double), cudaMemcpyDeviceToHost,
                           st));
    }
    CK(cudaMemcpyAsync(ctx->herr_host, ctx->errw.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaEventRecord(ctx->ev_done, st));
    if (ctx->done_fn) CK(cudaLaunchHostFunc(st, ctx->done_fn, ctx->done_user));
    CK(cudaGetLastError());
    ctx->in_flight = true;
    ctx->poses_in_flight = false;
    const auto h5 = HClock::now();
    ctx->host_ms[0] = hms(h0, h1);
    ctx->host_ms[1] = hms(h1, h2);
    ctx->host_ms[2] = hms(h2, h3);
    ctx->host_ms[3] = hms(h3, h4);
    ctx->host_ms[4] = hms(h4, h5);
    return ARAP_OK;
}

int arap_get_host_timing(arap_ctx *ctx, double *ms5) {
    if (check_ctx(ctx) || !ms5) return ARAP_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < 5; ++i) ms5[i] = ctx->host_ms[i];
    return ARAP_OK;
}

int arap_wait(arap_ctx *ctx) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    if (!ctx->in_flight) return ARAP_OK;
    ctx->in_flight = false;
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    collect_profile(ctx);
    float a = 0.f, b = 0.f;
    cudaEventElapsedTime(&a, ctx->ev0, ctx->ev1);
    cudaEventElapsedTime(&b, ctx->ev1, ctx->ev2);
    ctx->setup_ms = a;
    ctx->iter_ms = b;
    const int herr = *ctx->herr_host;
    if (herr & kErrNotSpd) {
        ctx->dirty = true;  // as the reference: the next deform sets the problem up again
        return fail(ctx, ARAP_ERR_NOT_SPD, "Cholesky factorisation met a non-positive pivot");
    }
    if (herr & kErrTimeout) {
        // scheduling counters may be inconsistent now: rebuild them next time
        ctx->sym_valid = false;
        ctx->dirty = true;
        ctx->bgen = -1;
        return fail(ctx, ARAP_ERR_TIMEOUT, "a bounded in-kernel wait expired");
    }
    return ARAP_OK;
}

int arap_set_done_callback(arap_ctx *ctx, arap_done_fn fn, void *user) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    if (ctx->in_flight) {
        const int rc_ = arap_wait(ctx);
        if (rc_ != ARAP_OK) return rc_;
    }
    ctx->done_fn = fn;
    ctx->done_user = user;
    return ARAP_OK;
}

int arap_query(arap_ctx *ctx, int32_t *done) {
    if (check_ctx(ctx) || !done) return ARAP_ERR_INVALID_ARGUMENT;
    *done = 1;
    if (!ctx->in_flight) return ARAP_OK;
    CK(cudaSetDevice(ctx->device));
    const cudaError_t q = cudaEventQuery(ctx->ev_done);
    if (q == cudaErrorNotReady) {
        *done = 0;
        return ARAP_OK;
    }
    if (q != cudaSuccess) CK(q);
    return arap_wait(ctx);
}

int arap_deform(arap_ctx *ctx, int32_t iterations, double *out_xyz) {
    const int rc = arap_deform_async(ctx, iterations, out_xyz);
    if (rc != ARAP_OK) return rc;
    return arap_wait(ctx);
}

int arap_set_solve_ctas(arap_ctx *ctx, int32_t max_ctas) {
    if (check_ctx(ctx) || max_ctas < 0) return ARAP_ERR_INVALID_ARGUMENT;
    if (ctx->in_flight) {
        const int rc_ = arap_wait(ctx);
        if (rc_ != ARAP_OK) return rc_;
    }
    if (max_ctas != ctx->solve_cap) {
        ctx->solve_cap = max_ctas;
        ctx->sym_valid = false;  // new launch shape: scheduling counters restart with the next setup
        ctx->dirty = true;
    }
    return ARAP_OK;
}

int arap_set_pose_tile(arap_ctx *ctx, int32_t poses) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    if (poses != 0 && poses != 1 && poses != 2 && poses != 4 && poses != 8 && poses != 16)
        return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "pose tile must be 0, 1, 2, 4, 8 or 16");
    if (ctx->in_flight) {
        const int rc_ = arap_wait(ctx);
        if (rc_ != ARAP_OK) return rc_;
    }
    ctx->pose_tile = poses;  // a changed tile resets the batched solves' counters at the next call
    return ARAP_OK;
}

int arap_set_ordering(arap_ctx *ctx, int32_t mode) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    if (mode != ARAP_ORDER_PER_CONSTRAINT_SET && mode != ARAP_ORDER_MESH)
        return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "unknown ordering mode");
    if (ctx->in_flight) {
        const int rc_ = arap_wait(ctx);
        if (rc_ != ARAP_OK) return rc_;
    }
    if (mode != ctx->ordering) {
        ctx->ordering = mode;
        ctx->sym_host = false;
        ctx->sym_valid = false;
        ctx->dirty = true;
    }
    return ARAP_OK;
}

int arap_set_warp_rows(arap_ctx *ctx, int32_t rows) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    if (rows < 0) return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "negative row count");
    if (ctx->in_flight) {
        const int rc_ = arap_wait(ctx);
        if (rc_ != ARAP_OK) return rc_;
    }
    if (rows != ctx->warp_rows) {
        ctx->warp_rows = rows;
        ctx->sym_valid = false;  // new launch shape: scheduling counters restart with the next setup
        ctx->dirty = true;
    }
    return ARAP_OK;
}

int arap_set_vertex_launch(arap_ctx *ctx, int32_t kernel, int32_t threads_per_vertex, int32_t block_threads) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    const int k = kernel == ARAP_K_LOCAL ? kVertexLocal
                  : kernel == ARAP_K_RHS ? kVertexRhs
                  : kernel == ARAP_K_RESIDUAL ? kVertexResidual : -1;
    if (k < 0) return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "kernel class without a vertex launch shape");
    const int t = threads_per_vertex, b = block_threads;
    if (t != 1 && t != 2 && t != 4 && t != 8 && t != 32)
        return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "threads per vertex must be 1, 2, 4, 8 or 32");
    if (b < 32 || b % 32 != 0 || b > (k == kVertexLocal ? kLocalMaxBlock : 1024))
        return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "block threads must be a multiple of 32 up to the kernel's limit");
    if (ctx->in_flight) {
        const int rc_ = arap_wait(ctx);
        if (rc_ != ARAP_OK) return rc_;
    }
    if (ctx->vlaunch[k].tpv != t || ctx->vlaunch[k].block != b) {
        ctx->vlaunch[k] = {t, b};
        ctx->ds.vlaunch[k] = ctx->vlaunch[k];
        ctx->gen++;  // captured iteration graphs hold the old launch shape
    }
    return ARAP_OK;
}

int arap_set_solve_blocks(arap_ctx *ctx, int32_t max_columns) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    if (max_columns < 0 || max_columns > kMaxSolveBlock)
        return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "solve block columns out of range (0..1024)");
    if (ctx->in_flight) {
        const int rc_ = arap_wait(ctx);
        if (rc_ != ARAP_OK) return rc_;
    }
    if (max_columns != ctx->solve_blocks) {
        ctx->solve_blocks = max_columns;
        ctx->sym_host = ctx->sym_valid = false;  // the analysis decides the blocks
        ctx->dirty = true;
    }
    return ARAP_OK;
}

int arap_set_solve_schedule(arap_ctx *ctx, int32_t schedule) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    if (schedule != ARAP_SOLVE_PERSISTENT && schedule != ARAP_SOLVE_LEVELS)
        return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "unknown solve schedule");
    if (ctx->in_flight) {
        const int rc_ = arap_wait(ctx);
        if (rc_ != ARAP_OK) return rc_;
    }
    if (schedule != ctx->solve_schedule) {
        ctx->solve_schedule = schedule;
        ctx->sym_valid = false;  // new launch shape: scheduling counters restart with the next setup
        ctx->dirty = true;
    }
    return ARAP_OK;
}

int arap_set_cluster_threshold(arap_ctx *ctx, int32_t bytes) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    if (ctx->in_flight) {
        const int rc_ = arap_wait(ctx);
        if (rc_ != ARAP_OK) return rc_;
    }
    if (bytes != ctx->top_bytes) {
        ctx->top_bytes = bytes;
        ctx->sym_valid = false;  // new launch shape: scheduling counters restart with the next setup
        ctx->dirty = true;
    }
    return ARAP_OK;
}

int arap_set_dense_top(arap_ctx *ctx, int32_t max_columns) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    if (ctx->in_flight) {
        const int rc_ = arap_wait(ctx);
        if (rc_ != ARAP_OK) return rc_;
    }
    if (max_columns != ctx->dense_cols) {
        ctx->dense_cols = max_columns;
        ctx->sym_valid = false;  // new launch shape: scheduling counters restart with the next setup
        ctx->dirty = true;
    }
    return ARAP_OK;
}

int arap_set_wait_limit(arap_ctx *ctx, int32_t polls) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    if (polls < 0) return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "negative poll limit");
    if (ctx->in_flight) {
        const int rc_ = arap_wait(ctx);
        if (rc_ != ARAP_OK) return rc_;
    }
    CK(cudaSetDevice(ctx->device));
    const int v = polls;
    CK(cudaMemcpyAsync(ctx->errw.as<int>() + 1, &v, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return ARAP_OK;
}

int arap_set_symbolic_cache(arap_ctx *ctx, int32_t enable) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    if (ctx->in_flight) {
        const int rc_ = arap_wait(ctx);
        if (rc_ != ARAP_OK) return rc_;
    }
    ctx->sym_cache = enable != 0;
    return ARAP_OK;
}

int arap_set_graphs(arap_ctx *ctx, int32_t enable) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    ctx->use_graphs = enable != 0;
    return ARAP_OK;
}

int arap_get_positions(arap_ctx *ctx, double *out_xyz) {
    if (check_ctx(ctx) || !out_xyz) return ARAP_ERR_INVALID_ARGUMENT;
    if (ctx->in_flight) {
        const int rc_ = arap_wait(ctx);
        if (rc_ != ARAP_OK) return rc_;
    }
    if (!ctx->sym_valid || ctx->state_prec < 0) return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "no deformed state yet");
    CK(cudaSetDevice(ctx->device));
    launch_gather_positions(ctx->ds, ctx->pc64.as<Vec4<double>>(), ctx->out.as<double>(), ctx->stream);
    CK(cudaMemcpyAsync(out_xyz, ctx->out.p, (size_t)3 * ctx->topo.V * sizeof(double), cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return ARAP_OK;
}

int arap_energy(arap_ctx *ctx, double *energy) {
    if (check_ctx(ctx) || !energy) return ARAP_ERR_INVALID_ARGUMENT;
    if (ctx->in_flight) {
        const int rc_ = arap_wait(ctx);
        if (rc_ != ARAP_OK) return rc_;
    }
    if (!ctx->sym_valid || ctx->state_prec < 0) return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "no deformed state yet");
    CK(cudaSetDevice(ctx->device));
    // scratch: the partial sums, then the total
    CK(ctx->energy.ensure(((size_t)energy_partials(ctx->ds.V) + 1) * sizeof(double)));
    double *scratch = ctx->energy.as<double>();
    const int np = energy_partials(ctx->ds.V);
    launch_energy(ctx->ds, ctx->w64.as<double>(), ctx->p64.as<Vec4<double>>(), ctx->pc64.as<Vec4<double>>(), scratch,
                  scratch + np, ctx->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(energy, scratch + np, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return ARAP_OK;
}

namespace {
// Deformed positions (vertex order) into ctx->out and their vertex normals into
// ctx->vnorm, on the context's stream.
int enqueue_positions_normals(arap_ctx *ctx, bool normals) {
    cudaStream_t st = ctx->stream;
    launch_gather_positions(ctx->ds, ctx->pc64.as<Vec4<double>>(), ctx->out.as<double>(), st);
    if (normals) {
        const Topology &t = ctx->topo;
        if (!ctx->vf_ptr.p || ctx->vf_ptr.cap < t.vf_ptr.size() * sizeof(int32_t)) {
            CK(upload(ctx->vf_ptr, t.vf_ptr, st));
            CK(upload(ctx->vf_face, t.vf_face, st));
        }
        CK(ctx->fnorm.ensure((size_t)3 * std::max(t.F, 1) * sizeof(double)));
        CK(ctx->vnorm.ensure((size_t)3 * std::max(t.V, 1) * sizeof(double)));
        launch_vertex_normals(t.V, t.F, ctx->faces.as<int32_t>(), ctx->vf_ptr.as<int32_t>(),
                              ctx->vf_face.as<int32_t>(), ctx->out.as<double>(), ctx->fnorm.as<double>(),
                              ctx->vnorm.as<double>(), st);
    }
    CK(cudaGetLastError());
    return ARAP_OK;
}
}  // namespace

int arap_vertex_normals(arap_ctx *ctx, double *normals_xyz) {
    if (check_ctx(ctx) || !normals_xyz) return ARAP_ERR_INVALID_ARGUMENT;
    if (ctx->in_flight) {
        const int rc_ = arap_wait(ctx);
        if (rc_ != ARAP_OK) return rc_;
    }
    if (!ctx->sym_valid || ctx->state_prec < 0) return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "no deformed state yet");
    CK(cudaSetDevice(ctx->device));
    const int rc = enqueue_positions_normals(ctx, true);
    if (rc != ARAP_OK) return rc;
    CK(cudaMemcpyAsync(normals_xyz, ctx->vnorm.p, (size_t)3 * ctx->topo.V * sizeof(double), cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return ARAP_OK;
}

int arap_device_positions(arap_ctx *ctx, int32_t with_normals, const double **positions_device,
                          const double **normals_device) {
    if (check_ctx(ctx) || !positions_device) return ARAP_ERR_INVALID_ARGUMENT;
    if (ctx->in_flight) {
        const int rc_ = arap_wait(ctx);
        if (rc_ != ARAP_OK) return rc_;
    }
    if (!ctx->sym_valid || ctx->state_prec < 0) return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "no deformed state yet");
    CK(cudaSetDevice(ctx->device));
    const int rc = enqueue_positions_normals(ctx, with_normals != 0);
    if (rc != ARAP_OK) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    *positions_device = ctx->out.as<double>();
    if (normals_device) *normals_device = with_normals ? ctx->vnorm.as<double>() : nullptr;
    return ARAP_OK;
}

int arap_edge_weights_nnz(arap_ctx *ctx, int32_t *nnz) {
    if (check_ctx(ctx) || !nnz) return ARAP_ERR_INVALID_ARGUMENT;
    *nnz = ctx->topo.nnz();
    return ARAP_OK;
}

int arap_get_edge_weights(arap_ctx *ctx, int32_t *rowptr, int32_t *col, double *val) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    if (ctx->in_flight) {
        const int rc_ = arap_wait(ctx);
        if (rc_ != ARAP_OK) return rc_;
    }
    const Topology &t = ctx->topo;
    if (rowptr) std::memcpy(rowptr, t.rowptr.data(), t.rowptr.size() * sizeof(int32_t));
    if (col && t.nnz()) std::memcpy(col, t.col.data(), t.col.size() * sizeof(int32_t));
    if (val && t.nnz()) {
        CK(cudaSetDevice(ctx->device));
        CK(cudaMemcpyAsync(val, ctx->w_orig.p, (size_t)t.nnz() * sizeof(double), cudaMemcpyDeviceToHost,
                           ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    return ARAP_OK;
}

int arap_get_rotations(arap_ctx *ctx, double *R9) {
    if (check_ctx(ctx) || !R9) return ARAP_ERR_INVALID_ARGUMENT;
    if (ctx->in_flight) {
        const int rc_ = arap_wait(ctx);
        if (rc_ != ARAP_OK) return rc_;
    }
    const int V = ctx->topo.V;
    if (!ctx->have_rotations || !ctx->sym_valid) {
        for (int v = 0; v < V; ++v)
            for (int a = 0; a < 9; ++a) R9[9 * v + a] = (a % 4 == 0) ? 1.0 : 0.0;
        return ARAP_OK;
    }
    CK(cudaSetDevice(ctx->device));
    if (ctx->state_prec == ARAP_PRECISION_FP64)
        launch_gather_rotations<double>(ctx->ds, ctx->R.as<Vec4<double>>(), ctx->out.as<double>(), ctx->stream);
    else
        launch_gather_rotations<float>(ctx->ds, ctx->R.as<Vec4<float>>(), ctx->out.as<double>(), ctx->stream);
    CK(cudaMemcpyAsync(R9, ctx->out.p, (size_t)9 * V * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return ARAP_OK;
}

int arap_get_symbolic_sizes(arap_ctx *ctx, int32_t *n_free, int32_t *n_blocks, int64_t *factor_nnz) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    if (!ctx->sym_valid) return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "no symbolic analysis yet");
    if (n_free) *n_free = ctx->sym.m;
    if (n_blocks) *n_blocks = ctx->sym.S;
    if (factor_nnz) *factor_nnz = symbolic_factor_nnz(ctx->sym);
    return ARAP_OK;
}

int arap_get_symbolic(arap_ctx *ctx, int32_t *perm, int32_t *etree, int32_t *block_ptr) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    if (!ctx->sym_valid) return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "no symbolic analysis yet");
    const Symbolic &s = ctx->sym;
    if (perm && s.m) std::memcpy(perm, s.perm.data(), (size_t)s.m * sizeof(int32_t));
    if (etree && s.m) std::memcpy(etree, s.etree.data(), (size_t)s.m * sizeof(int32_t));
    if (block_ptr) std::memcpy(block_ptr, s.block_ptr.data(), s.block_ptr.size() * sizeof(int32_t));
    return ARAP_OK;
}

int arap_analyze_pattern(int32_t n_vertices, int32_t n_faces, const int32_t *faces, int32_t n_constrained,
                         const int32_t *constrained, int32_t *n_free, int32_t *n_blocks, int64_t *factor_nnz,
                         int32_t *perm, int32_t *etree, int32_t *block_ptr) {
    g_create_error.clear();
    if (n_vertices < 0 || n_faces < 0 || n_constrained < 0 || (n_faces > 0 && !faces) ||
        (n_constrained > 0 && !constrained)) {
        g_create_error = "arap_analyze_pattern: invalid argument";
        return ARAP_ERR_INVALID_ARGUMENT;
    }
    Topology topo;
    std::string err;
    if (!build_topology(n_vertices, n_faces, faces, topo, err)) {
        g_create_error = err;
        return ARAP_ERR_BAD_INDEX;
    }
    std::vector<uint8_t> mask(n_vertices, 0);
    for (int i = 0; i < n_constrained; ++i) {
        if (constrained[i] < 0 || constrained[i] >= n_vertices) {
            g_create_error = "constraint index outside the mesh";
            return ARAP_ERR_BAD_INDEX;
        }
        mask[constrained[i]] = 1;
    }
    Symbolic s;
    bool singular = false;
    if (!build_symbolic(topo, mask, s, err, singular)) {
        g_create_error = err;
        return singular ? ARAP_ERR_NOT_SPD : ARAP_ERR_UNSUPPORTED;
    }
    if (n_free) *n_free = s.m;
    if (n_blocks) *n_blocks = s.S;
    if (factor_nnz) *factor_nnz = symbolic_factor_nnz(s);
    if (perm && s.m) std::memcpy(perm, s.perm.data(), (size_t)s.m * sizeof(int32_t));
    if (etree && s.m) std::memcpy(etree, s.etree.data(), (size_t)s.m * sizeof(int32_t));
    if (block_ptr) std::memcpy(block_ptr, s.block_ptr.data(), s.block_ptr.size() * sizeof(int32_t));
    return ARAP_OK;
}

int arap_get_timing(arap_ctx *ctx, double *setup_ms, double *iterations_ms) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    if (setup_ms) *setup_ms = ctx->setup_ms;
    if (iterations_ms) *iterations_ms = ctx->iter_ms;
    return ARAP_OK;
}

int arap_get_launch_count(arap_ctx *ctx, int64_t *launches) {
    if (check_ctx(ctx) || !launches) return ARAP_ERR_INVALID_ARGUMENT;
    *launches = ctx->launches;
    return ARAP_OK;
}

int arap_plan_bytes(arap_ctx *ctx, int32_t n_poses, int64_t *bytes) {
    if (check_ctx(ctx) || !bytes || n_poses < 0) return ARAP_ERR_INVALID_ARGUMENT;
    if (ctx->in_flight) {
        const int rc_ = arap_wait(ctx);
        if (rc_ != ARAP_OK) return rc_;
    }
    *bytes = 0;
    int64_t total = 0;
    std::vector<std::pair<DevBuf *, size_t>> plan;
    if (!ctx->cidx.empty()) {
        const int rc = analyze_symbolic(ctx);
        if (rc != ARAP_OK) return rc;
        if (ctx->precision == ARAP_PRECISION_FP64 && n_poses == 0) planned_sizes<double>(ctx, 0, plan);
        else planned_sizes<float>(ctx, n_poses, plan);
    }
    for (DevBuf *b : ctx->buffers()) {
        size_t want = b->cap;
        for (auto &pb : plan)
            if (pb.first == b) want = std::max(want, std::max<size_t>(pb.second, 256));
        total += (int64_t)want;
    }
    *bytes = total;
    return ARAP_OK;
}

int64_t arap_device_bytes(const arap_ctx *ctx) {
    if (!ctx) return 0;
    int64_t total = 0;
    for (const DevBuf *b : const_cast<arap_ctx *>(ctx)->buffers()) total += (int64_t)b->cap;
    return total;
}

int arap_get_stream(arap_ctx *ctx, void **stream) {
    if (check_ctx(ctx) || !stream) return ARAP_ERR_INVALID_ARGUMENT;
    *stream = (void *)ctx->stream;
    return ARAP_OK;
}

int arap_set_profiling(arap_ctx *ctx, int32_t enable) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    ctx->profiling = enable != 0;
    return ARAP_OK;
}

int arap_reset_kernel_stats(arap_ctx *ctx) {
    if (check_ctx(ctx)) return ARAP_ERR_INVALID_ARGUMENT;
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    collect_profile(ctx);
    for (int k = 0; k < ARAP_K_NUM_CLASSES; ++k) {
        ctx->kms[k] = 0.0;
        ctx->kcnt[k] = 0;
    }
    return ARAP_OK;
}

int arap_get_kernel_model(arap_ctx *ctx, int32_t kernel_class, double *bytes, double *flops) {
    if (check_ctx(ctx) || kernel_class < 0 || kernel_class >= ARAP_K_NUM_CLASSES) return ARAP_ERR_INVALID_ARGUMENT;
    if (!ctx->sym_valid || ctx->state_prec < 0) return fail(ctx, ARAP_ERR_INVALID_ARGUMENT, "no problem set up yet");
    const Symbolic &s = ctx->sym;
    const double sz = ctx->state_prec == ARAP_PRECISION_FP64 ? 8.0 : 4.0;  // scalar of the iteration
    const double V = s.V, m = s.m, nnz = (double)s.dcol.size(), F = ctx->topo.F;
    // panel entries below the diagonal blocks and lower-triangular entries of the
    // inverted diagonal blocks, read once per solve sweep
    // per solve sweep: the lower triangle of X = inv(L11) and L21, once each
    // (the levels below the dense top, where there is one: the _lo sums)
    double xlow = 0.0, l21 = 0.0, xlow_lo = 0.0, l21_lo = 0.0, nbsum_lo = 0.0;
    // the supernodes (or, with solve blocks, the blocks and the supernodes
    // above them) the single-request sweeps read
    const std::vector<int32_t> &sched = ctx->use_sb ? ctx->sb.level_sn : s.level_sn;
    const std::vector<SnInfo> &snv = ctx->use_sb ? ctx->sb.sn : s.sn;
    const int ltop_m = ctx->use_sb ? ctx->dss.ltop : ctx->ds.ltop;
    for (const int32_t q : sched) {
        const SnInfo &d = snv[q];
        xlow += (double)d.ncol * (d.ncol + 1) / 2;
        l21 += (double)(d.nrow - d.ncol) * d.ncol;
        if (ctx->ds.n_top == 0 || d.level < ltop_m) {
            xlow_lo += (double)d.ncol * (d.ncol + 1) / 2;
            l21_lo += (double)(d.nrow - d.ncol) * d.ncol;
            nbsum_lo += d.nrow - d.ncol;
        }
    }
    // one sweep: the lower levels' matrices, then the dense top's triangle of
    // T (or T^T); per pose the solution, the update vectors and the top's
    // vector, each written and read once
    const double nt = ctx->ds.n_top;
    const double tri = nt * (nt + 1) / 2;
    const double vec = m * 3 * sz * 2 + nbsum_lo * 3 * sz * 2 + nt * 3 * sz * 2;
    double B = 0.0, FL = 0.0;
    const double P = ctx->model_P, T = ctx->model_T;  // poses, pose tiles of the last deform
    switch (kernel_class) {
    case ARAP_K_WEIGHTS:  // faces + rest positions + weights out (two precisions)
        B = F * 12 + V * 24 + F * 24 + nnz * (4 + 8 + sz);
        FL = F * 40;
        break;
    case ARAP_K_ASSEMBLE:
        B = V * (24 + 24 + 3 * sz * 2 + 9 * sz) + m * (8 + 3 * sz) + nnz * (4 + 8 + 8);
        FL = nnz * 4;
        break;
    case ARAP_K_FACTOR: {
        // in the factor's precision; an FP64 factor of the mixed form also
        // writes the FP32 solve copies (and reads the FP64 ones back once)
        const bool f64f = ctx->state_prec == ARAP_PRECISION_MIXED && ctx->factor_bits == 64;
        const double fz = f64f ? 8.0 : sz;
        B = (double)s.panel_size * fz * 2 + (double)s.upd_size * fz * 2 + (double)s.dinv_size * fz +
            (xlow + l21) * sz;
        if (f64f) B += (double)(s.panel_size + s.dinv_size) * (8 + 4);  // rounded to FP32 for the inverses
        FL = s.factor_flops;
        break;
    }
    case ARAP_K_LOCAL:
        if (sz == 8.0)  // rest + current positions, rotations out, adjacency + weights
            B = V * 3 * sz + P * V * (3 * sz + 9 * sz) + 4 * (V + 1) + nnz * (4 + sz);
        else  // FP32 rest edges + weights per entry; FP64 current positions, FP32 rotations per vertex and pose
            B = nnz * (4 + 4 + 12) + 4 * (V + 1) + P * V * (24 + 36);
        FL = P * (nnz * 24 + V * 600);
        break;
    case ARAP_K_RHS:
        if (sz == 8.0)
            B = m * 3 * sz + P * m * (9 * sz + 3 * sz + 3 * sz) + 4 * (m + 1) + nnz * (4 + sz);
        else  // rest edges + weights per entry; rotations of every vertex, b of the free ones, per pose
            B = nnz * (4 + 4 + 12) + 4 * (m + 1) + P * (V * 36 + m * 12);
        FL = P * nnz * 24;
        break;
    case ARAP_K_RESIDUAL:  // x, bFixed (FP64), b in, r out per free vertex and pose
        B = P * m * (24 + 24 + 12 + 12) + m * 8 + 4 * (m + 1) + nnz * (4 + 8);
        FL = P * nnz * 6;
        break;
    case ARAP_K_SOLVE_FWD:
    case ARAP_K_SOLVE_BWD:
        if (ctx->model_batched) {  // lower matrices once per pose tile, T once, vectors once per pose
            B = (T * (xlow_lo + l21_lo) + tri) * sz + P * vec;
            FL = P * (xlow_lo + l21_lo + tri) * 6;
        } else {
            B = (xlow_lo + l21_lo + tri) * sz + vec;
            FL = (xlow_lo + l21_lo + tri) * 6;
        }
        if (kernel_class == ARAP_K_SOLVE_BWD && ctx->state_prec != ARAP_PRECISION_FP64) B += P * m * (24 * 2 + 12);
        break;
    case ARAP_K_GATHER:
        B = P * V * (24 + 24) + V * 4;
        FL = 0;
        break;
    }
    if (bytes) *bytes = B;
    if (flops) *flops = FL;
    return ARAP_OK;
}

int arap_get_kernel_stats(arap_ctx *ctx, int32_t kernel_class, double *total_ms, int64_t *launches) {
    if (check_ctx(ctx) || kernel_class < 0 || kernel_class >= ARAP_K_NUM_CLASSES) return ARAP_ERR_INVALID_ARGUMENT;
    if (total_ms) *total_ms = ctx->kms[kernel_class];
    if (launches) *launches = ctx->kcnt[kernel_class];
    return ARAP_OK;
}

}  // extern "C"

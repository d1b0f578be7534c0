// arap_symbolic.cpp -- host-side symbolic analysis for the GPU ARAP solver.
//
// Covers the integer part of inc/deform/arap.h:
//   - the sparsity of _edgeWeights built by computeCotanWeights (arap.h:182-239,
//     undirectedEdge arap.h:435-440), which doubles as the one-ring adjacency;
//   - the free-variable map (initializeFreeVariableMapping, arap.h:261-272);
//   - the pattern of the constrained Laplacian L (setupLinearSystem, arap.h:292-336)
//     and the symbolic part of its factorisation (SimplicialLDLT::compute,
//     arap.h:337), here a nested-dissection ordering, the elimination tree and a
//     supernodal partition for a multifrontal Cholesky on the GPU.
//
// Nested dissection (George 1973) with level-structure separators: a set of at
// most kNdLeaf vertices is one leaf block; a disconnected set is ordered one
// component at a time (components in order of their smallest vertex); a
// connected set is split by the BFS level of a pseudo-peripheral vertex
// (George & Liu) whose two sides both hold >= 4/10 of the set, smallest level
// first, then most balanced, then lowest level; level vertices with no
// neighbour in the next level move to the near side. Order: near side, far
// side, separator. Every emitted leaf or separator is one supernode.
#include "arap_symbolic.h"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <numeric>
#include <thread>

namespace arapgpu {

bool build_topology(int V, int F, const int32_t *faces, Topology &topo, std::string &err) {
    topo = Topology();
    topo.V = V;
    topo.F = F;
    topo.faces.assign(faces, faces + (size_t)3 * F);
    for (int64_t i = 0; i < (int64_t)3 * F; ++i) {
        if (faces[i] < 0 || faces[i] >= V) {
            err = "face index " + std::to_string(faces[i]) + " outside [0, " + std::to_string(V) + ")";
            return false;
        }
    }
    // Directed contributions in the order computeCotanWeights pushes them
    // (arap.h:225-232): per face e0,e1,e2 as (min,max), then as (max,min).
    // A counting sort by row, then a stable insertion sort by column inside
    // each row (a handful of entries), orders them as a stable sort by
    // (row, column) would.
    struct Contrib { int32_t c, fc; };
    std::vector<int32_t> rstart((size_t)V + 1, 0);
    for (int64_t i = 0; i < (int64_t)3 * F; ++i) rstart[faces[i] + 1] += 2;
    for (int v = 0; v < V; ++v) rstart[v + 1] += rstart[v];
    std::vector<int32_t> fillp(rstart.begin(), rstart.end() - 1);
    std::vector<Contrib> t((size_t)6 * F);
    for (int f = 0; f < F; ++f) {
        const int32_t v[3] = {faces[3 * f], faces[3 * f + 1], faces[3 * f + 2]};
        int32_t a[3], b[3];
        for (int k = 0; k < 3; ++k) {
            a[k] = std::min(v[k], v[(k + 1) % 3]);
            b[k] = std::max(v[k], v[(k + 1) % 3]);
        }
        for (int k = 0; k < 3; ++k) t[fillp[a[k]]++] = {b[k], 3 * f + k};
        for (int k = 0; k < 3; ++k) t[fillp[b[k]]++] = {a[k], 3 * f + k};
    }
    for (int v = 0; v < V; ++v)
        for (int32_t i = rstart[v] + 1; i < rstart[v + 1]; ++i) {
            const Contrib x = t[i];
            int32_t j = i - 1;
            while (j >= rstart[v] && t[j].c > x.c) { t[j + 1] = t[j]; --j; }
            t[j + 1] = x;
        }
    topo.rowptr.assign((size_t)V + 1, 0);
    topo.ent_ptr.clear();
    topo.ent_ptr.reserve((size_t)3 * F + 1);
    topo.ent_ptr.push_back(0);
    topo.ent_fc.reserve((size_t)6 * F);
    topo.col.reserve((size_t)3 * F);
    for (int v = 0; v < V; ++v) {
        for (int32_t i = rstart[v]; i < rstart[v + 1];) {
            int32_t j = i;
            while (j < rstart[v + 1] && t[j].c == t[i].c) {
                topo.ent_fc.push_back(t[j].fc);
                ++j;
            }
            topo.col.push_back(t[i].c);
            topo.rowptr[v + 1]++;
            topo.ent_ptr.push_back((int32_t)topo.ent_fc.size());
            i = j;
        }
    }
    for (int v = 0; v < V; ++v) topo.rowptr[v + 1] += topo.rowptr[v];
    // faces around each vertex (a face whose corners repeat is listed once per corner)
    topo.vf_ptr.assign((size_t)V + 1, 0);
    for (int64_t i = 0; i < (int64_t)3 * F; ++i) topo.vf_ptr[faces[i] + 1]++;
    for (int v = 0; v < V; ++v) topo.vf_ptr[v + 1] += topo.vf_ptr[v];
    topo.vf_face.resize((size_t)3 * F);
    {
        std::vector<int32_t> fill(topo.vf_ptr.begin(), topo.vf_ptr.end() - 1);
        for (int f = 0; f < F; ++f)
            for (int k = 0; k < 3; ++k) topo.vf_face[fill[faces[3 * f + k]]++] = f;
    }
    return true;
}

// ---------------------------------------------------------------------------
// nested dissection

namespace {

// State shared by every worker of one dissection: the graph and the arrays
// indexed by vertex. A worker only writes the entries of the vertices of its
// own set; it reads `inset` of neighbours outside the set, which another
// worker may be writing at the same time, so those accesses are relaxed
// atomics. Stamps come from one atomic counter, so a set's stamp is never
// seen on a vertex outside the set: the result does not depend on timing.
struct NdShared {
    const int32_t *rowptr, *col;
    int n;
    std::vector<int32_t> inset, seen, lev_buf[2];
    std::atomic<int32_t> stamp{0};
    int32_t next_stamp() { return stamp.fetch_add(1, std::memory_order_relaxed) + 1; }
};

inline int32_t load_rlx(const int32_t *p) { return __atomic_load_n(p, __ATOMIC_RELAXED); }
inline void store_rlx(int32_t *p, int32_t v) { __atomic_store_n(p, v, __ATOMIC_RELAXED); }

// Output of a recursion: the vertices in elimination order and the sizes of
// the blocks (leaves and separators) they form.
struct NdOut {
    std::vector<int32_t> perm, sizes;
    void emit(const std::vector<int32_t> &S) {
        perm.insert(perm.end(), S.begin(), S.end());
        sizes.push_back((int32_t)S.size());
    }
    void append(const NdOut &o) {
        perm.insert(perm.end(), o.perm.begin(), o.perm.end());
        sizes.insert(sizes.end(), o.sizes.begin(), o.sizes.end());
    }
};

// Sets of at least this many vertices dissect their two sides on two threads
// (down to a depth of kNdParallelDepth: at most 2^depth threads at once).
constexpr int kNdParallelMin = 16384;
constexpr int kNdParallelDepth = 3;

struct NdWorker {
    NdShared *sh;
    // two BFS queues (indexed by position): a trial BFS from a new root
    // fills the spare one, which becomes current when the trial is kept
    std::vector<int32_t> queue_buf[2];
    int cur = 0;

    NdWorker(NdShared *s, size_t cap) : sh(s) {
        queue_buf[0].resize(cap);
        queue_buf[1].resize(cap);
    }

    // BFS inside the stamped set into buffer `buf`; neighbours visited in CSR
    // order. Returns the number of levels, level offsets into the queue in levptr.
    int bfs(int32_t setstamp, int32_t root, std::vector<int32_t> &levptr, int buf) {
        const int32_t *rowptr = sh->rowptr, *col = sh->col;
        int32_t *queue = queue_buf[buf].data(), *lev = sh->lev_buf[buf].data();
        int32_t *inset = sh->inset.data(), *seen = sh->seen.data();
        const int32_t bs = sh->next_stamp();
        int head = 0, tail = 0;
        queue[tail++] = root;
        seen[root] = bs;
        lev[root] = 0;
        levptr.clear();
        while (head < tail) {
            const int32_t v = queue[head];
            if (lev[v] == (int32_t)levptr.size()) levptr.push_back(head);
            ++head;
            for (int32_t q = rowptr[v]; q < rowptr[v + 1]; ++q) {
                const int32_t u = col[q];
                if (load_rlx(inset + u) != setstamp || seen[u] == bs) continue;
                seen[u] = bs;
                lev[u] = lev[v] + 1;
                queue[tail++] = u;
            }
        }
        levptr.push_back(tail);
        return (int)levptr.size() - 1;
    }

    // S arrives in any order; only the blocks emitted are sorted, and the
    // smallest vertex of S is the first BFS root, so the result is that of
    // recursing on sorted sets.
    void recurse(std::vector<int32_t> S, NdOut &out, int depth) {
        const int ns = (int)S.size();
        if (ns <= kNdLeaf) {
            std::sort(S.begin(), S.end());
            out.emit(S);
            return;
        }
        int32_t *inset = sh->inset.data();
        const int32_t *rowptr = sh->rowptr, *col = sh->col;
        const int32_t setstamp = sh->next_stamp();
        int32_t smin = S[0];
        for (int32_t v : S) {
            store_rlx(inset + v, setstamp);
            smin = std::min(smin, v);
        }
        std::vector<int32_t> levptr;
        int h = bfs(setstamp, smin, levptr, cur);
        if (levptr[h] < ns) {
            // several components, each in order of its smallest vertex
            std::sort(S.begin(), S.end());
            std::vector<std::vector<int32_t>> comps;
            for (int32_t v : S) {
                if (load_rlx(inset + v) != setstamp) continue;
                const int hl = bfs(setstamp, v, levptr, cur);
                comps.emplace_back(queue_buf[cur].begin(), queue_buf[cur].begin() + levptr[hl]);
                const int32_t cs = sh->next_stamp();
                for (int32_t u : comps.back()) store_rlx(inset + u, cs);
            }
            const int nt = std::min<int>((int)comps.size(), (int)std::max(1u, std::thread::hardware_concurrency()));
            if (ns < kNdParallelMin || depth >= kNdParallelDepth || nt < 2) {
                for (auto &c : comps) recurse(std::move(c), out, depth);
                return;
            }
            // components (the meshes of a batch) on a pool of threads, output
            // in component order; with many components each recursion stays
            // on its thread
            const int sub_depth = (int)comps.size() >= nt ? kNdParallelDepth : depth + 1;
            std::vector<NdOut> outs(comps.size());
            std::atomic<int> next{0};
            auto work = [&]() {
                for (int c = next.fetch_add(1); c < (int)comps.size(); c = next.fetch_add(1)) {
                    NdWorker w(sh, comps[c].size() + 1);
                    w.recurse(std::move(comps[c]), outs[c], sub_depth);
                }
            };
            std::vector<std::thread> pool;
            for (int t = 1; t < nt; ++t) pool.emplace_back(work);
            work();
            for (auto &t : pool) t.join();
            for (const NdOut &o : outs) out.append(o);
            return;
        }
        // pseudo-peripheral vertex
        std::vector<int32_t> lp2;
        for (int it = 0; it < kNdPseudoPeripheralRounds; ++it) {
            const int32_t *queue = queue_buf[cur].data();
            int32_t best = -1, bestdeg = 0;
            for (int q = levptr[h - 1]; q < levptr[h]; ++q) {
                const int32_t v = queue[q];
                int32_t deg = 0;
                for (int32_t e = rowptr[v]; e < rowptr[v + 1]; ++e) deg += (load_rlx(inset + col[e]) == setstamp);
                if (best < 0 || deg < bestdeg || (deg == bestdeg && v < best)) { best = v; bestdeg = deg; }
            }
            const int h2 = bfs(setstamp, best, lp2, cur ^ 1);
            if (h2 > h) { h = h2; levptr.swap(lp2); cur ^= 1; }
            else break;
        }
        const int32_t *queue = queue_buf[cur].data(), *lev = sh->lev_buf[cur].data();
        if (h < 3) {
            std::sort(S.begin(), S.end());
            out.emit(S);
            return;
        }
        int bestk = -1;
        int64_t bsz = 0, bdiff = 0;
        for (int k = 1; k <= h - 2; ++k) {
            const int64_t a = levptr[k], sz = levptr[k + 1] - levptr[k], b = (int64_t)ns - a - sz;
            const int64_t mn = std::min(a, b);
            if (mn * kNdBalDen < (int64_t)kNdBalNum * ns) continue;
            const int64_t d = a > b ? a - b : b - a;
            if (bestk < 0 || sz < bsz || (sz == bsz && d < bdiff)) { bestk = k; bsz = sz; bdiff = d; }
        }
        if (bestk < 0) {
            bestk = h - 2;
            for (int k = 1; k <= h - 2; ++k)
                if (2LL * levptr[k + 1] >= ns) { bestk = k; break; }
        }
        const int k = bestk;
        std::vector<int32_t> A, B, Sep;
        A.assign(queue, queue + levptr[k]);
        for (int q = levptr[k]; q < levptr[k + 1]; ++q) {
            const int32_t v = queue[q];
            bool touches = false;
            for (int32_t e = rowptr[v]; e < rowptr[v + 1] && !touches; ++e) {
                const int32_t u = col[e];
                touches = (load_rlx(inset + u) == setstamp && lev[u] == k + 1);
            }
            (touches ? Sep : A).push_back(v);
        }
        B.assign(queue + levptr[k + 1], queue + levptr[h]);
        std::sort(Sep.begin(), Sep.end());
        if (ns >= kNdParallelMin && depth < kNdParallelDepth) {
            // the near side on a second thread, the far side here; blocks are
            // emitted in the sequential order (near, far, separator)
            NdOut outA, outB;
            const size_t capA = A.size() + 1;
            std::thread th([this, &outA, capA, depth](std::vector<int32_t> a) {
                NdWorker w(sh, capA);
                w.recurse(std::move(a), outA, depth + 1);
            }, std::move(A));
            recurse(std::move(B), outB, depth + 1);
            th.join();
            out.append(outA);
            out.append(outB);
        } else {
            recurse(std::move(A), out, depth);
            recurse(std::move(B), out, depth);
        }
        out.emit(Sep);
    }
};

}  // namespace

void nd_order(int n, const int32_t *rowptr, const int32_t *col, std::vector<int32_t> &perm,
              std::vector<int32_t> &block_ptr) {
    perm.clear();
    block_ptr.assign(1, 0);
    if (n <= 0) return;
    NdShared sh;
    sh.rowptr = rowptr;
    sh.col = col;
    sh.n = n;
    sh.inset.assign(n, 0);
    sh.seen.assign(n, 0);
    for (int b = 0; b < 2; ++b) sh.lev_buf[b].assign(n, 0);
    NdWorker w(&sh, (size_t)n);
    std::vector<int32_t> S(n);
    std::iota(S.begin(), S.end(), 0);
    NdOut out;
    out.perm.reserve(n);
    w.recurse(std::move(S), out, 0);
    perm.swap(out.perm);
    block_ptr.reserve(out.sizes.size() + 1);
    for (int32_t sz : out.sizes) block_ptr.push_back(block_ptr.back() + sz);
}

// ---------------------------------------------------------------------------

bool build_solve_blocks(const Symbolic &sym, int max_cols, SolveBlocks &out) {
    out = SolveBlocks();
    const int S = sym.S;
    if (S == 0) return false;
    SolveBlocks b;
    b.sn = sym.sn;
    b.x_size = sym.x_size;
    b.l21_size = sym.l21_size;
    b.l21t_size = sym.l21t_size;
    std::vector<char> absorbed(S, 0);
    for (int s = 0; s < S; ++s) {
        const SnInfo &d = sym.sn[s];
        if (d.level != 1) continue;
        // the subtree: the leaf children (all leaves, the node being of level
        // 1), contiguous before the node in the elimination order
        int first = d.first, cols = d.ncol;
        for (int ci = d.child_begin; ci < d.child_end; ++ci) {
            const SnInfo &c = sym.sn[sym.child[ci]];
            first = std::min(first, (int)c.first);
            cols += c.ncol;
        }
        if (first + cols != d.first + d.ncol || cols > max_cols) return false;
        b.items.push_back(s);
        b.items.push_back((int32_t)b.members.size());
        for (int ci = d.child_begin; ci < d.child_end; ++ci) {
            b.members.push_back(sym.child[ci]);
            absorbed[sym.child[ci]] = 1;
        }
        b.members.push_back(s);
        b.items.push_back((int32_t)b.members.size());
        SnInfo &e = b.sn[s];
        const int nb = d.nrow - d.ncol;
        e.first = first;
        e.ncol = cols;
        e.nrow = cols + nb;
        e.child_begin = e.child_end = d.child_begin;  // no children left
        e.ldx = (cols + 3) & ~3;
        e.x_off = b.x_size;
        b.x_size += (int64_t)e.ldx * cols;
        e.xt_off = b.x_size;
        b.x_size += (int64_t)e.ldx * cols;
        e.l21t_off = b.l21t_size;
        b.l21t_size += (int64_t)e.ldx * nb;
        e.l21_off = b.l21_size;
        b.l21_size += (int64_t)e.ld21 * cols;
        ++b.nblocks;
    }
    if (b.nblocks == 0) return false;
    // levels of the solve tree (children come before parents in the array)
    int maxlev = 0;
    for (int s = 0; s < S; ++s) {
        SnInfo &e = b.sn[s];
        int lv = 0;
        for (int ci = e.child_begin; ci < e.child_end; ++ci) lv = std::max(lv, b.sn[sym.child[ci]].level + 1);
        e.level = lv;
        if (!absorbed[s]) maxlev = std::max(maxlev, lv);
    }
    b.level_ptr.assign(maxlev + 2, 0);
    for (int s = 0; s < S; ++s)
        if (!absorbed[s]) b.level_ptr[b.sn[s].level + 1]++;
    for (int l = 0; l <= maxlev; ++l) b.level_ptr[l + 1] += b.level_ptr[l];
    b.level_sn.assign(b.level_ptr.back(), 0);
    std::vector<int32_t> fill(b.level_ptr.begin(), b.level_ptr.end() - 1);
    for (int s = 0; s < S; ++s)
        if (!absorbed[s]) b.level_sn[fill[b.sn[s].level]++] = s;
    for (int s = 0; s < S; ++s) {
        if (absorbed[s]) continue;
        b.max_ldx = std::max(b.max_ldx, (int)b.sn[s].ldx);
        b.max_ld21 = std::max(b.max_ld21, (int)b.sn[s].ld21);
        b.max_ncol = std::max(b.max_ncol, (int)b.sn[s].ncol);
    }
    out = std::move(b);
    return true;
}

int64_t symbolic_factor_nnz(Symbolic &sym) {
    if (sym.factor_nnz >= 0) return sym.factor_nnz;
    // row subtrees of the elimination tree: row k of L holds column i < k for
    // every i on the tree path from a neighbour of k (in the permuted free
    // graph, which is the device-order adjacency restricted to [0, m)) up to k
    const int m = sym.m;
    std::vector<int32_t> mark(m, -1);
    int64_t nz = m;
    for (int k = 0; k < m; ++k) {
        mark[k] = k;
        for (int32_t e = sym.drow[k]; e < sym.drow[k + 1]; ++e) {
            int32_t i = sym.dcol[e];
            if (i >= k) continue;
            while (mark[i] != k) { mark[i] = k; ++nz; i = sym.etree[i]; }
        }
    }
    sym.factor_nnz = nz;
    return nz;
}

namespace {
// a thread joined when it goes out of scope (also on early returns)
struct JoinOnExit {
    std::thread t;
    ~JoinOnExit() {
        if (t.joinable()) t.join();
    }
};

// analyses running in this process (several requests prepared at once fill
// the cores already; one alone splits its row loops over threads)
std::atomic<int> g_analyses{0};
struct AnalysisCount {
    AnalysisCount() { g_analyses.fetch_add(1); }
    ~AnalysisCount() { g_analyses.fetch_sub(1); }
};

// body(lo, hi) over [0, n): in up to four contiguous chunks on threads when
// the range is large and no other analysis runs, else in one call
template <typename F>
void row_chunks(int n, F &&body) {
    const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    const int parts = (n >= 32768 && g_analyses.load() == 1) ? std::min(4, hw) : 1;
    if (parts <= 1) {
        body(0, n);
        return;
    }
    std::vector<std::thread> th;
    for (int p = 1; p < parts; ++p)
        th.emplace_back([&body, n, p, parts] { body((int)((int64_t)n * p / parts), (int)((int64_t)n * (p + 1) / parts)); });
    body(0, (int)((int64_t)n / parts));
    for (auto &t : th) t.join();
}
}  // namespace

bool build_symbolic(const Topology &topo, const std::vector<uint8_t> &constrained, Symbolic &sym,
                    std::string &err, bool &singular, bool mesh_order) {
    const AnalysisCount counted;
    singular = false;
    sym = Symbolic();
    const int V = topo.V;
    sym.V = V;
    sym.constrained = constrained;
    // free-variable map (arap.h:261-272)
    std::vector<int32_t> fidx(V, -1), fvert;
    for (int v = 0; v < V; ++v)
        if (!constrained[v]) { fidx[v] = (int32_t)fvert.size(); fvert.push_back(v); }
    const int m = (int)fvert.size();
    sym.m = m;
    // graph of L's off-diagonal pattern over free indices (arap.h:319-330):
    // row lengths, offsets, then the rows
    std::vector<int32_t> grow(m + 1, 0), gcol;
    std::vector<uint8_t> touches_c(m, 0);
    row_chunks(m, [&](int lo, int hi) {
        for (int a = lo; a < hi; ++a) {
            const int v = fvert[a];
            int32_t c = 0;
            for (int32_t q = topo.rowptr[v]; q < topo.rowptr[v + 1]; ++q) {
                const int u = topo.col[q];
                if (u == v) continue;
                if (constrained[u]) { touches_c[a] = 1; continue; }
                ++c;
            }
            grow[a + 1] = c;
        }
    });
    for (int a = 0; a < m; ++a) grow[a + 1] += grow[a];
    gcol.resize(grow[m]);
    row_chunks(m, [&](int lo, int hi) {
        for (int a = lo; a < hi; ++a) {
            const int v = fvert[a];
            int32_t e = grow[a];
            for (int32_t q = topo.rowptr[v]; q < topo.rowptr[v + 1]; ++q) {
                const int u = topo.col[q];
                if (u != v && !constrained[u]) gcol[e++] = fidx[u];
            }
        }
    });
    if (!mesh_order) {
        nd_order(m, grow.data(), gcol.data(), sym.perm, sym.block_ptr);
    } else {
        MeshOrder &mo = *topo.mesh_order;
        {
            std::lock_guard<std::mutex> lk(mo.mu);
            if (!mo.ready) {
                // the mesh graph without self entries
                std::vector<int32_t> mrow(V + 1, 0), mcol;
                mcol.reserve(topo.col.size());
                for (int v = 0; v < V; ++v) {
                    for (int32_t q = topo.rowptr[v]; q < topo.rowptr[v + 1]; ++q)
                        if (topo.col[q] != v) mcol.push_back(topo.col[q]);
                    mrow[v + 1] = (int32_t)mcol.size();
                }
                nd_order(V, mrow.data(), mcol.data(), mo.perm, mo.block_ptr);
                mo.ready = true;
            }
        }
        sym.perm.clear();
        sym.perm.reserve(m);
        sym.block_ptr.assign(1, 0);
        for (size_t b = 0; b + 1 < mo.block_ptr.size(); ++b) {
            for (int32_t k = mo.block_ptr[b]; k < mo.block_ptr[b + 1]; ++k)
                if (!constrained[mo.perm[k]]) sym.perm.push_back(fidx[mo.perm[k]]);
            if ((int32_t)sym.perm.size() > sym.block_ptr.back()) sym.block_ptr.push_back((int32_t)sym.perm.size());
        }
    }
    std::vector<int32_t> iperm(m);
    for (int k = 0; k < m; ++k) iperm[sym.perm[k]] = k;
    // device order: free vertices in elimination order, then constrained ascending
    sym.newidx.assign(V, -1);
    sym.oldidx.assign(V, -1);
    for (int a = 0; a < m; ++a) sym.newidx[fvert[a]] = iperm[a];
    int nc = m;
    for (int v = 0; v < V; ++v)
        if (constrained[v]) sym.newidx[v] = nc++;
    for (int v = 0; v < V; ++v) sym.oldidx[sym.newidx[v]] = v;
    // adjacency in device order, on a second thread while the elimination
    // tree and the supernodes are built (it only writes drow, dcol, dent)
    const int nnz = topo.nnz();
    JoinOnExit adj;
    adj.t = std::thread([&sym, &topo, V, nnz] {
        sym.drow.assign(V + 1, 0);
        sym.dcol.resize(nnz);
        sym.dent.resize(nnz);
        int32_t e = 0;
        for (int k = 0; k < V; ++k) {
            const int v = sym.oldidx[k];
            for (int32_t q = topo.rowptr[v]; q < topo.rowptr[v + 1]; ++q) {
                sym.dcol[e] = sym.newidx[topo.col[q]];
                sym.dent[e] = q;
                ++e;
            }
            sym.drow[k + 1] = e;
        }
    });
    // permuted free graph: adjacency of device index k < m (neighbours < m)
    std::vector<int32_t> prow(m + 1, 0), pcol(gcol.size());
    for (int k = 0; k < m; ++k) prow[k + 1] = prow[k] + (grow[sym.perm[k] + 1] - grow[sym.perm[k]]);
    row_chunks(m, [&](int lo, int hi) {
        for (int k = lo; k < hi; ++k) {
            const int a = sym.perm[k];
            int32_t e = prow[k];
            for (int32_t q = grow[a]; q < grow[a + 1]; ++q) pcol[e++] = iperm[gcol[q]];
        }
    });
    // elimination tree (Liu, with path compression), on a helper thread while
    // the supernodes' rows are built (they follow from the dissection's blocks)
    JoinOnExit et;
    et.t = std::thread([&sym, &prow, &pcol, m] {
        sym.etree.assign(m, -1);
        std::vector<int32_t> anc(m, -1);
        for (int k = 0; k < m; ++k) {
            for (int32_t q = prow[k]; q < prow[k + 1]; ++q) {
                int32_t i = pcol[q];
                while (i != -1 && i < k) {
                    const int32_t next = anc[i];
                    anc[i] = k;
                    if (next == -1) { sym.etree[i] = k; break; }
                    i = next;
                }
            }
        }
    });
    // the factor's nonzero count is only reported, so it is counted on demand
    // (symbolic_factor_nnz) rather than on every analysis
    sym.factor_nnz = -1;
    // supernodes = the dissection's blocks
    const int S = (int)sym.block_ptr.size() - 1;
    sym.S = S;
    sym.sn.assign(S, SnInfo());
    std::vector<int32_t> owner(m);
    for (int s = 0; s < S; ++s)
        for (int k = sym.block_ptr[s]; k < sym.block_ptr[s + 1]; ++k) owner[k] = s;
    // struct rows of each supernode (its columns' rows below it and its
    // children's struct rows below it, sorted), written straight into
    // sym.rows; children as linked lists in increasing order
    std::vector<int32_t> mark(m, -1), st, chead(S, -1), ctail(S, -1), cnext(S, -1);
    st.reserve(1024);
    sym.rows.clear();
    sym.rows.reserve(prow[m]);
    for (int s = 0; s < S; ++s) {
        const int f = sym.block_ptr[s], l = sym.block_ptr[s + 1];
        st.clear();
        for (int k = f; k < l; ++k)
            for (int32_t q = prow[k]; q < prow[k + 1]; ++q) {
                const int32_t r = pcol[q];
                if (r >= l && mark[r] != s) { mark[r] = s; st.push_back(r); }
            }
        for (int32_t c = chead[s]; c >= 0; c = cnext[c]) {
            const SnInfo &cd = sym.sn[c];
            const int32_t *cr = sym.rows.data() + cd.rows_off;
            for (int i = 0; i < cd.nrow - cd.ncol; ++i) {
                const int32_t r = cr[i];
                if (r >= l && mark[r] != s) { mark[r] = s; st.push_back(r); }
            }
        }
        std::sort(st.begin(), st.end());
        const int p = st.empty() ? -1 : owner[st[0]];
        SnInfo &d = sym.sn[s];
        d.first = f;
        d.ncol = l - f;
        d.nrow = d.ncol + (int32_t)st.size();
        d.parent = p;
        d.rows_off = (int32_t)sym.rows.size();
        sym.rows.insert(sym.rows.end(), st.begin(), st.end());
        if (p >= 0) {
            if (chead[p] < 0) chead[p] = s;
            else cnext[ctail[p]] = s;
            ctail[p] = s;
        }
    }
    et.t.join();
    // every free component must reach a constrained vertex, else L is
    // singular; each component of the free graph is one tree of the
    // elimination forest, so "touches a constrained vertex" is carried up to
    // the roots (children come before their parents)
    {
        std::vector<uint8_t> anchored(m, 0);
        for (int k = 0; k < m; ++k) anchored[k] = touches_c[sym.perm[k]];
        for (int k = 0; k < m; ++k) {
            const int32_t p = sym.etree[k];
            if (p >= 0) anchored[p] |= anchored[k];
            else if (!anchored[k]) {
                singular = true;
                err = "free vertex " + std::to_string(fvert[sym.perm[k]]) +
                      " belongs to a mesh component without constrained vertices (singular Laplacian)";
                return false;
            }
        }
    }
    // levels, offsets, struct rows, children, relative indices
    int maxlev = 0;
    int64_t poff = 0, doff = 0, uoff = 0, voff = 0, xoff = 0, loff = 0, ltoff = 0;
    double flops = 0.0;
    for (int s = 0; s < S; ++s) {
        SnInfo &d = sym.sn[s];
        int lv = 0, nch = 0;
        for (int32_t c = chead[s]; c >= 0; c = cnext[c], ++nch) lv = std::max(lv, sym.sn[c].level + 1);
        d.level = lv;
        maxlev = std::max(maxlev, lv);
        const int nb = d.nrow - d.ncol;
        d.panel_off = poff;
        poff += (int64_t)d.nrow * d.ncol;
        d.dinv_off = doff;
        doff += (int64_t)((d.ncol + kDiagBlock - 1) / kDiagBlock) * kDiagBlock * kDiagBlock;
        d.upd_off = uoff;
        uoff += (int64_t)nb * nb;
        d.uvec_off = voff;
        voff += nb;
        // solve-time copies with 16-byte aligned columns (offsets and leading
        // dimensions are multiples of 4 elements)
        d.ldx = (d.ncol + 3) & ~3;
        d.ld21 = (nb + 3) & ~3;
        d.x_off = xoff;
        xoff += (int64_t)d.ldx * d.ncol;
        d.xt_off = xoff;  // X and X^T side by side in the same array
        xoff += (int64_t)d.ldx * d.ncol;
        d.l21t_off = ltoff;
        ltoff += (int64_t)d.ldx * nb;
        d.l21_off = loff;
        loff += (int64_t)d.ld21 * d.ncol;
        sym.max_ldx = std::max(sym.max_ldx, (int)d.ldx);
        sym.max_ld21 = std::max(sym.max_ld21, (int)d.ld21);
        d.child_begin = (int32_t)sym.child.size();
        for (int32_t c = chead[s]; c >= 0; c = cnext[c]) sym.child.push_back(c);
        d.child_end = (int32_t)sym.child.size();
        sym.max_nrow = std::max(sym.max_nrow, (int)d.nrow);
        sym.max_ncol = std::max(sym.max_ncol, (int)d.ncol);
        sym.max_children = std::max(sym.max_children, nch);
        const double nc_ = d.ncol, nb_ = nb;
        flops += nc_ * nc_ * nc_ / 3.0 + nc_ * nc_ * nb_ + nc_ * nb_ * nb_;
    }
    sym.factor_flops = flops;
    sym.panel_size = poff;
    sym.dinv_size = doff;
    sym.upd_size = uoff;
    sym.uvec_size = voff;
    sym.x_size = xoff;
    sym.l21_size = loff;
    sym.l21t_size = ltoff;
    // front position of every row of supernode s's front: its columns, then
    // its struct rows; filled for one supernode at a time (stamped by s), so
    // lookups below are direct
    auto map_front = [&sym](int s, std::vector<int32_t> &fpos, std::vector<int32_t> &fstamp) {
        const SnInfo &d = sym.sn[s];
        for (int c = 0; c < d.ncol; ++c) {
            fpos[d.first + c] = c;
            fstamp[d.first + c] = s;
        }
        const int32_t *rs = sym.rows.data() + d.rows_off;
        for (int i = 0; i < d.nrow - d.ncol; ++i) {
            fpos[rs[i]] = d.ncol + i;
            fstamp[rs[i]] = s;
        }
    };
    // assembly maps (L_kk and L_lk = -w_kl, l > k, both free, into the
    // panels) on a second thread, with their own front map, while the
    // relative indices and the launch plan are built here
    adj.t.join();
    bool amap_ok = true;
    JoinOnExit amap_th;
    amap_th.t = std::thread([&sym, &map_front, &amap_ok, m, S, nnz] {
        std::vector<int32_t> fpos(m, 0), fstamp(m, -1);
        sym.amap.assign(nnz, -1);
        sym.dmap.assign(m, -1);
        for (int s = 0; s < S; ++s) {
            const SnInfo &d = sym.sn[s];
            map_front(s, fpos, fstamp);
            for (int k = d.first; k < d.first + d.ncol; ++k) {
                const int cidx = k - d.first;
                sym.dmap[k] = d.panel_off + (int64_t)cidx * d.nrow + cidx;
                for (int32_t e = sym.drow[k]; e < sym.drow[k + 1]; ++e) {
                    const int32_t l = sym.dcol[e];
                    if (l >= m || l <= k) continue;
                    if (fstamp[l] != s) {
                        amap_ok = false;
                        return;
                    }
                    sym.amap[e] = d.panel_off + (int64_t)cidx * d.nrow + fpos[l];
                }
            }
        }
    });
    std::vector<int32_t> fpos(m, 0), fstamp(m, -1);
    // relind: where each struct row of s sits in its parent's front
    sym.relind.reserve(sym.rows.size());
    for (int s = 0; s < S; ++s) sym.sn[s].relind_off = -1;
    for (int p = 0; p < S; ++p) {
        const SnInfo &pd = sym.sn[p];
        if (pd.child_begin == pd.child_end) continue;
        map_front(p, fpos, fstamp);
        for (int ci = pd.child_begin; ci < pd.child_end; ++ci) {
            SnInfo &d = sym.sn[sym.child[ci]];
            d.relind_off = (int32_t)sym.relind.size();
            const int32_t *cr = sym.rows.data() + d.rows_off;
            for (int i = 0; i < d.nrow - d.ncol; ++i) {
                const int32_t r = cr[i];
                if (fstamp[r] != p) {
                    err = "internal: struct row missing from parent front";
                    return false;
                }
                sym.relind.push_back(fpos[r]);
            }
        }
    }
    for (int s = 0; s < S; ++s)
        if (sym.sn[s].relind_off < 0) sym.sn[s].relind_off = (int32_t)sym.relind.size();
    // supernodes grouped by level
    sym.level_ptr.assign(maxlev + 2, 0);
    for (int s = 0; s < S; ++s) sym.level_ptr[sym.sn[s].level + 1]++;
    for (int l = 0; l <= maxlev; ++l) sym.level_ptr[l + 1] += sym.level_ptr[l];
    sym.level_sn.assign(S, 0);
    {
        std::vector<int32_t> fill(sym.level_ptr.begin(), sym.level_ptr.end() - 1);
        for (int s = 0; s < S; ++s) sym.level_sn[fill[sym.sn[s].level]++] = s;
    }
    if (S == 0) sym.level_ptr.assign(1, 0);
    // factorisation launch plan
    {
        const int nlev = (int)sym.level_ptr.size() - 1;
        auto add = [&](int kind, int jb, const std::vector<FItem> &items) {
            if (items.empty()) return;
            sym.fplan.push_back({kind, jb, (int32_t)sym.fitems.size(), (int32_t)items.size()});
            sym.fitems.insert(sym.fitems.end(), items.begin(), items.end());
        };
        constexpr int kSlice = 32, kRowTile = kFactorUpdRows, kTileU = kFactorSyrkTile;
        for (int l = 0; l < nlev; ++l) {
            std::vector<FItem> it;
            int nblk_max = 0;
            for (int q = sym.level_ptr[l]; q < sym.level_ptr[l + 1]; ++q) {
                const int sidx = sym.level_sn[q];
                const SnInfo &d = sym.sn[sidx];
                nblk_max = std::max(nblk_max, (d.ncol + kDiagBlock - 1) / kDiagBlock);
                if (d.child_begin == d.child_end) continue;
                for (int lo = 0; lo < d.nrow; lo += kSlice) it.push_back({sidx, lo, std::min(d.nrow, lo + kSlice), 0});
            }
            add(kFea, 0, it);
            for (int jb = 0; jb < nblk_max; ++jb) {
                std::vector<FItem> up, dt, rw;
                for (int q = sym.level_ptr[l]; q < sym.level_ptr[l + 1]; ++q) {
                    const int sidx = sym.level_sn[q];
                    const SnInfo &d = sym.sn[sidx];
                    const int j0 = jb * kDiagBlock;
                    if (j0 >= d.ncol) continue;
                    const int below = d.nrow - std::min(d.ncol, j0 + kDiagBlock);
                    dt.push_back({sidx, 0, 0, 0});
                    for (int rt = 0; rt * kFactorRowsTile < below; ++rt) rw.push_back({sidx, rt, 0, 0});
                    if (jb > 0)
                        for (int rt = 0; j0 + rt * kRowTile < d.nrow; ++rt) up.push_back({sidx, rt, 0, 0});
                }
                add(kFupd, jb, up);
                add(kFdt, jb, dt);
                add(kFrows, jb, rw);
            }
            std::vector<FItem> sy, fx;
            for (int q = sym.level_ptr[l]; q < sym.level_ptr[l + 1]; ++q) {
                const int sidx = sym.level_sn[q];
                const SnInfo &d = sym.sn[sidx];
                const int nb = d.nrow - d.ncol;
                const int nt = (nb + kTileU - 1) / kTileU;
                for (int rt = 0; rt < nt; ++rt)
                    for (int ct = 0; ct <= rt; ++ct) sy.push_back({sidx, rt, ct, 0});
                for (int jb = 0; jb * kDiagBlock < d.ncol; ++jb) fx.push_back({sidx, jb, 0, 0});
            }
            add(kFsyrk, 0, sy);
            add(kFx, 0, fx);
        }
    }
    amap_th.t.join();
    if (!amap_ok) {
        err = "internal: matrix entry outside its supernode's front";
        return false;
    }
    return true;
}

}  // namespace arapgpu

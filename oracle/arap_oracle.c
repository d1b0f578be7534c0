/*
 * arap_oracle.c -- FP64 CPU restatement of the ARAP hot path of cheind/mesh-deform.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA library and the timed CPU
 * baseline. The product never includes, links or calls this file.
 *
 * Every function names the lines of inc/deform/arap.h it restates. Third-party
 * arithmetic the reference takes from Eigen (version not pinned by the
 * reference: cmake/FindEigen3.cmake:4-10 only locates headers) is restated from
 * the published algorithms:
 *   - Eigen::JacobiSVD (arap.h:376)            -> one-sided (Hestenes) Jacobi SVD,
 *                                                 Demmel & Veselic 1992, with the
 *                                                 singular values sorted descending.
 *   - Eigen::SimplicialLDLT (arap.h:337,420)   -> up-looking sparse LDL^T driven by
 *                                                 the elimination tree (T. Davis,
 *                                                 ACM TOMS Algorithm 849, 2005),
 *                                                 with a nested-dissection ordering
 *                                                 (George 1973) in place of Eigen's AMD;
 *                                                 any ordering gives the same solution
 *                                                 up to rounding.
 *   - SparseMatrix::setFromTriplets            -> duplicates summed in insertion order.
 *
 * Compile with -ffp-contract=off so that the results do not depend on whether
 * the host compiler fuses multiply-adds (x86-64 vs aarch64).
 *
 * Parity status: cotan weights pinned by the reference's known-answer test
 * (tests/test_cotan.cpp:26-53); end-to-end positions "parity unpinned" against
 * the reference binary (no Eigen here), cross-checked against an independent
 * numpy/scipy restatement instead.
 */
#include "arap_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* std::max<Scalar>(a, b) as written in arap.h: (a < b) ? b : a. NaN in b yields a. */
#define REF_MAX(a, b) (((a) < (b)) ? (b) : (a))

#define ND_LEAF 64
/* A level separator is accepted when both sides hold at least 4/10 of the set. */
#define ND_BAL_NUM 4
#define ND_BAL_DEN 10
#define ND_PP_ROUNDS 8

struct oracle_arap {
    int V, F;
    int *faces;    /* 3F, _faces (arap.h:151-154) */
    double *mesh;  /* 3V, the adapter's vertex locations */
    double *p;     /* 3V, _p (arap.h:163-166) */
    double *pp;    /* 3V, _pprime (arap.h:167) */
    /* _edgeWeights, RowMajor CSR with sorted columns (arap.h:235-238) */
    int *wrow, *wcol;
    double *wval;
    int wnnz;
    double *R; /* 9V row-major, _rotations (arap.h:246-249) */
    int *free_idx; /* _freeIdxMap (arap.h:261-272) */
    int nfree;
    unsigned char *has_c; /* _constrainedLocations keys */
    double *ctarget;      /* 3V, _constrainedLocations values */
    /* L over free indices (arap.h:292-336): CSR rows incl. diagonal */
    int *arow, *acol;
    double *aval;
    double *bfixed, *b; /* 3m each, row-major m x 3 */
    /* solver: ordering, elimination tree and LDL^T factor */
    int *perm, *iperm;
    int nblocks, *block_ptr;
    int *parent, *Lp, *Li, *Lnz;
    double *Lx, *D;
    long long lnnz;
    int dirty;
};

static void *xcalloc(size_t n, size_t s) {
    void *p = calloc(n ? n : 1, s ? s : 1);
    if (!p) abort();
    return p;
}

static void free_solver(oracle_arap *oa) {
    free(oa->arow); free(oa->acol); free(oa->aval);
    free(oa->bfixed); free(oa->b);
    free(oa->perm); free(oa->iperm); free(oa->block_ptr);
    free(oa->parent); free(oa->Lp); free(oa->Li); free(oa->Lnz);
    free(oa->Lx); free(oa->D);
    oa->arow = oa->acol = NULL; oa->aval = NULL;
    oa->bfixed = oa->b = NULL;
    oa->perm = oa->iperm = oa->block_ptr = NULL;
    oa->parent = oa->Lp = oa->Li = oa->Lnz = NULL;
    oa->Lx = oa->D = NULL;
    oa->nblocks = 0;
    oa->lnnz = 0;
}

oracle_arap *oa_create(int n_vertices, int n_faces, const int *faces, const double *positions) {
    oracle_arap *oa = (oracle_arap *)xcalloc(1, sizeof(oracle_arap));
    oa->V = n_vertices;
    oa->F = n_faces;
    oa->faces = (int *)xcalloc((size_t)3 * n_faces, sizeof(int));
    memcpy(oa->faces, faces, sizeof(int) * 3 * (size_t)n_faces);
    oa->mesh = (double *)xcalloc((size_t)3 * n_vertices, sizeof(double));
    if (positions) memcpy(oa->mesh, positions, sizeof(double) * 3 * (size_t)n_vertices);
    oa->p = (double *)xcalloc((size_t)3 * n_vertices, sizeof(double));
    oa->pp = (double *)xcalloc((size_t)3 * n_vertices, sizeof(double));
    oa->R = (double *)xcalloc((size_t)9 * n_vertices, sizeof(double));
    oa->free_idx = (int *)xcalloc((size_t)n_vertices, sizeof(int));
    oa->has_c = (unsigned char *)xcalloc((size_t)n_vertices, 1);
    oa->ctarget = (double *)xcalloc((size_t)3 * n_vertices, sizeof(double));
    oa->dirty = 1; /* arap.h:67 */
    return oa;
}

void oa_destroy(oracle_arap *oa) {
    if (!oa) return;
    free_solver(oa);
    free(oa->faces); free(oa->mesh); free(oa->p); free(oa->pp);
    free(oa->wrow); free(oa->wcol); free(oa->wval);
    free(oa->R); free(oa->free_idx); free(oa->has_c); free(oa->ctarget);
    free(oa);
}

void oa_set_mesh_positions(oracle_arap *oa, const double *xyz) {
    memcpy(oa->mesh, xyz, sizeof(double) * 3 * (size_t)oa->V);
}

void oa_get_mesh_positions(const oracle_arap *oa, double *xyz) {
    memcpy(xyz, oa->mesh, sizeof(double) * 3 * (size_t)oa->V);
}

/* arap.h:81-85 */
int oa_set_constraint(oracle_arap *oa, int vidx, double x, double y, double z) {
    if (vidx < 0 || vidx >= oa->V) return -1;
    oa->has_c[vidx] = 1;
    oa->ctarget[3 * vidx + 0] = x;
    oa->ctarget[3 * vidx + 1] = y;
    oa->ctarget[3 * vidx + 2] = z;
    oa->dirty = 1;
    return 0;
}

/* initializeMeshGeometry, arap.h:162-168 */
static void initialize_mesh_geometry(oracle_arap *oa) {
    memcpy(oa->p, oa->mesh, sizeof(double) * 3 * (size_t)oa->V);
    memcpy(oa->pp, oa->p, sizeof(double) * 3 * (size_t)oa->V);
}

/* ---- triplet accumulation with setFromTriplets semantics ----------------- */

typedef struct { int r, c; double v; } triplet;

/* Builds a CSR matrix (sorted columns) from triplets; duplicates are summed in
   insertion order (Eigen's collapseDuplicates), as arap.h:224,238,336 rely on. */
static void triplets_to_csr(int nrows, const triplet *t, size_t nt,
                            int **rowptr_out, int **col_out, double **val_out, int *nnz_out) {
    int *cnt = (int *)xcalloc((size_t)nrows + 1, sizeof(int));
    for (size_t k = 0; k < nt; ++k) cnt[t[k].r + 1]++;
    for (int i = 0; i < nrows; ++i) cnt[i + 1] += cnt[i];
    int *pos = (int *)xcalloc((size_t)nrows + 1, sizeof(int));
    memcpy(pos, cnt, sizeof(int) * ((size_t)nrows + 1));
    int *tc = (int *)xcalloc(nt, sizeof(int));
    double *tv = (double *)xcalloc(nt, sizeof(double));
    for (size_t k = 0; k < nt; ++k) { /* insertion order within each row */
        int q = pos[t[k].r]++;
        tc[q] = t[k].c;
        tv[q] = t[k].v;
    }
    /* collapse duplicates in insertion order, then sort columns of each row */
    int *rowptr = (int *)xcalloc((size_t)nrows + 1, sizeof(int));
    int *col = (int *)xcalloc(nt, sizeof(int));
    double *val = (double *)xcalloc(nt, sizeof(double));
    int nnz = 0;
    for (int i = 0; i < nrows; ++i) {
        int start = nnz;
        for (int q = cnt[i]; q < cnt[i + 1]; ++q) {
            int found = -1;
            for (int z = start; z < nnz; ++z)
                if (col[z] == tc[q]) { found = z; break; }
            if (found >= 0) {
                val[found] = val[found] + tv[q];
            } else {
                col[nnz] = tc[q];
                val[nnz] = tv[q];
                nnz++;
            }
        }
        /* insertion sort by column (rows are short) */
        for (int a = start + 1; a < nnz; ++a) {
            int c = col[a];
            double v = val[a];
            int b = a - 1;
            while (b >= start && col[b] > c) { col[b + 1] = col[b]; val[b + 1] = val[b]; --b; }
            col[b + 1] = c;
            val[b + 1] = v;
        }
        rowptr[i + 1] = nnz;
    }
    free(cnt); free(pos); free(tc); free(tv);
    *rowptr_out = rowptr;
    *col_out = col;
    *val_out = val;
    *nnz_out = nnz;
}

/* computeCotanWeights, arap.h:182-239 (clamped Heron cotangents, 1/2 factor,
   both directions, duplicates summed). */
static void compute_cotan_weights(oracle_arap *oa) {
    size_t nt = (size_t)6 * oa->F;
    triplet *t = (triplet *)xcalloc(nt, sizeof(triplet));
    size_t k = 0;
    for (int f = 0; f < oa->F; ++f) {
        const int i0 = oa->faces[3 * f + 0], i1 = oa->faces[3 * f + 1], i2 = oa->faces[3 * f + 2];
        const double *v0 = oa->p + 3 * i0, *v1 = oa->p + 3 * i1, *v2 = oa->p + 3 * i2;
        double d;
        double l0 = 0.0, l1 = 0.0, l2 = 0.0;
        for (int c = 0; c < 3; ++c) { d = v1[c] - v0[c]; l0 = l0 + d * d; }
        for (int c = 0; c < 3; ++c) { d = v2[c] - v1[c]; l1 = l1 + d * d; }
        for (int c = 0; c < 3; ++c) { d = v0[c] - v2[c]; l2 = l2 + d * d; }
        l0 = REF_MAX(1e-8, l0); /* arap.h:199-201 */
        l1 = REF_MAX(1e-8, l1);
        l2 = REF_MAX(1e-8, l2);
        l0 = sqrt(l0);
        l1 = sqrt(l1);
        l2 = sqrt(l2);
        const double semip = 0.5 * (l0 + l1 + l2);
        const double area = REF_MAX(1e-8, sqrt(semip * (semip - l0) * (semip - l1) * (semip - l2)));
        const double denom = 1.0 / (4.0 * area);
        double cot0 = (-l0 * l0 + l1 * l1 + l2 * l2) * denom;
        double cot1 = (l0 * l0 - l1 * l1 + l2 * l2) * denom;
        double cot2 = (l0 * l0 + l1 * l1 - l2 * l2) * denom;
        cot0 = REF_MAX(1e-10, cot0); /* arap.h:216-218 */
        cot1 = REF_MAX(1e-10, cot1);
        cot2 = REF_MAX(1e-10, cot2);
        /* undirectedEdge, arap.h:435-440 */
        int e0a = i0 < i1 ? i0 : i1, e0b = i0 < i1 ? i1 : i0;
        int e1a = i1 < i2 ? i1 : i2, e1b = i1 < i2 ? i2 : i1;
        int e2a = i2 < i0 ? i2 : i0, e2b = i2 < i0 ? i0 : i2;
        if (i0 == i1) { e0a = i0; e0b = i1; }
        if (i1 == i2) { e1a = i1; e1b = i2; }
        if (i2 == i0) { e2a = i2; e2b = i0; }
        const double h0 = cot0 * 0.5, h1 = cot1 * 0.5, h2 = cot2 * 0.5;
        t[k++] = (triplet){e0a, e0b, h0}; /* arap.h:225-232 */
        t[k++] = (triplet){e1a, e1b, h1};
        t[k++] = (triplet){e2a, e2b, h2};
        t[k++] = (triplet){e0b, e0a, h0};
        t[k++] = (triplet){e1b, e1a, h1};
        t[k++] = (triplet){e2b, e2a, h2};
    }
    free(oa->wrow); free(oa->wcol); free(oa->wval);
    triplets_to_csr(oa->V, t, nt, &oa->wrow, &oa->wcol, &oa->wval, &oa->wnnz);
    free(t);
}

/* initializeRotations, arap.h:246-249 */
static void initialize_rotations(oracle_arap *oa) {
    for (int v = 0; v < oa->V; ++v)
        for (int a = 0; a < 9; ++a) oa->R[9 * v + a] = (a % 4 == 0) ? 1.0 : 0.0;
}

/* initializeFreeVariableMapping, arap.h:261-272 */
static void initialize_free_variable_mapping(oracle_arap *oa) {
    int fi = 0;
    for (int i = 0; i < oa->V; ++i) oa->free_idx[i] = oa->has_c[i] ? -1 : fi++;
    oa->nfree = fi;
}

/* initializeConstraints, arap.h:277-281 */
static void initialize_constraints(oracle_arap *oa) {
    for (int i = 0; i < oa->V; ++i)
        if (oa->has_c[i])
            for (int c = 0; c < 3; ++c) oa->pp[3 * i + c] = oa->ctarget[3 * i + c];
}

/* ---- nested dissection ordering ------------------------------------------- */

typedef struct {
    int n;
    const int *rowptr, *col;
    int *inset;   /* membership stamp */
    int *seen;    /* BFS stamp */
    int *lev;     /* BFS level */
    int *queue;
    int stamp;
    int *perm;    /* output order */
    int nout;
    int *block_ptr;
    int nblocks;
} nd_state;

static int cmp_int(const void *a, const void *b) {
    int x = *(const int *)a, y = *(const int *)b;
    return (x > y) - (x < y);
}

static void nd_emit(nd_state *st, const int *S, int n) {
    for (int i = 0; i < n; ++i) st->perm[st->nout++] = S[i];
    st->block_ptr[++st->nblocks] = st->nout;
}

/* BFS from root within the stamped set; neighbours in CSR (ascending) order.
   Fills queue with the BFS order, returns the number of levels and writes the
   level start offsets (levptr, capacity n+1). */
static int nd_bfs(nd_state *st, int setstamp, int root, int *levptr) {
    int bstamp = ++st->stamp;
    int head = 0, tail = 0;
    st->queue[tail++] = root;
    st->seen[root] = bstamp;
    st->lev[root] = 0;
    int nlev = 0;
    levptr[0] = 0;
    while (head < tail) {
        int v = st->queue[head];
        if (st->lev[v] == nlev) levptr[nlev++] = head; /* first vertex of a new level */
        head++;
        for (int q = st->rowptr[v]; q < st->rowptr[v + 1]; ++q) {
            int u = st->col[q];
            if (st->inset[u] != setstamp || st->seen[u] == bstamp) continue;
            st->seen[u] = bstamp;
            st->lev[u] = st->lev[v] + 1;
            st->queue[tail++] = u;
        }
    }
    levptr[nlev] = tail;
    return nlev;
}

static void nd_recurse(nd_state *st, int *S, int n) {
    if (n <= ND_LEAF) { nd_emit(st, S, n); return; }
    int setstamp = ++st->stamp;
    for (int i = 0; i < n; ++i) st->inset[S[i]] = setstamp;

    /* connected components, each found by BFS from its smallest vertex */
    int *levptr = (int *)xcalloc((size_t)n + 1, sizeof(int));
    int nlev = nd_bfs(st, setstamp, S[0], levptr);
    int reached = levptr[nlev];
    if (reached < n) {
        /* more than one component: order each one separately, in order of its
           smallest vertex; no separator is needed between them */
        for (int i = 0; i < n; ++i) {
            int v = S[i];
            if (st->inset[v] != setstamp) continue; /* already in an earlier component */
            int nl = nd_bfs(st, setstamp, v, levptr);
            int cnt = levptr[nl];
            int *chunk = (int *)xcalloc((size_t)cnt, sizeof(int));
            memcpy(chunk, st->queue, sizeof(int) * (size_t)cnt);
            int cstamp = ++st->stamp;
            for (int j = 0; j < cnt; ++j) st->inset[chunk[j]] = cstamp;
            qsort(chunk, (size_t)cnt, sizeof(int), cmp_int);
            nd_recurse(st, chunk, cnt);
            free(chunk);
        }
        free(levptr);
        return;
    }

    /* pseudo-peripheral root (George & Liu) */
    int root = S[0];
    int h = nlev;
    for (int it = 0; it < ND_PP_ROUNDS; ++it) {
        int best = -1, bestdeg = 0;
        for (int q = levptr[h - 1]; q < levptr[h]; ++q) {
            int v = st->queue[q];
            int deg = 0;
            for (int e = st->rowptr[v]; e < st->rowptr[v + 1]; ++e)
                if (st->inset[st->col[e]] == setstamp) deg++;
            if (best < 0 || deg < bestdeg || (deg == bestdeg && v < best)) { best = v; bestdeg = deg; }
        }
        int *lp2 = (int *)xcalloc((size_t)n + 1, sizeof(int));
        int h2 = nd_bfs(st, setstamp, best, lp2);
        if (h2 > h) {
            root = best;
            h = h2;
            memcpy(levptr, lp2, sizeof(int) * ((size_t)h2 + 1));
            free(lp2);
        } else {
            free(lp2);
            break;
        }
    }
    /* the queue/levels must describe BFS(root) */
    h = nd_bfs(st, setstamp, root, levptr);
    if (h < 3) { nd_emit(st, S, n); free(levptr); return; }

    /* separator level */
    int bestk = -1;
    long long bs = 0, bd = 0;
    for (int k = 1; k <= h - 2; ++k) {
        long long a = levptr[k], s = levptr[k + 1] - levptr[k], b = (long long)n - a - s;
        long long mn = a < b ? a : b;
        if (mn * ND_BAL_DEN < (long long)ND_BAL_NUM * n) continue;
        long long dd = a > b ? a - b : b - a;
        if (bestk < 0 || s < bs || (s == bs && dd < bd)) { bestk = k; bs = s; bd = dd; }
    }
    if (bestk < 0) {
        bestk = h - 2;
        for (int k = 1; k <= h - 2; ++k)
            if (2LL * levptr[k + 1] >= n) { bestk = k; break; }
    }
    const int k = bestk;
    int *A = (int *)xcalloc((size_t)n, sizeof(int));
    int *B = (int *)xcalloc((size_t)n, sizeof(int));
    int *Sep = (int *)xcalloc((size_t)n, sizeof(int));
    int na = 0, nb = 0, ns = 0;
    for (int q = 0; q < levptr[k]; ++q) A[na++] = st->queue[q];
    for (int q = levptr[k]; q < levptr[k + 1]; ++q) {
        int v = st->queue[q];
        int touches = 0;
        for (int e = st->rowptr[v]; e < st->rowptr[v + 1]; ++e) {
            int u = st->col[e];
            if (st->inset[u] == setstamp && st->lev[u] == k + 1) { touches = 1; break; }
        }
        if (touches) Sep[ns++] = v; else A[na++] = v;
    }
    for (int q = levptr[k + 1]; q < levptr[h]; ++q) B[nb++] = st->queue[q];
    free(levptr);
    qsort(A, (size_t)na, sizeof(int), cmp_int);
    qsort(B, (size_t)nb, sizeof(int), cmp_int);
    qsort(Sep, (size_t)ns, sizeof(int), cmp_int);
    nd_recurse(st, A, na);
    nd_recurse(st, B, nb);
    nd_emit(st, Sep, ns);
    free(A); free(B); free(Sep);
}

int oa_nd_order(int n, const int *rowptr, const int *col, int *perm, int *block_ptr) {
    nd_state st;
    memset(&st, 0, sizeof(st));
    st.n = n;
    st.rowptr = rowptr;
    st.col = col;
    st.inset = (int *)xcalloc((size_t)n, sizeof(int));
    st.seen = (int *)xcalloc((size_t)n, sizeof(int));
    st.lev = (int *)xcalloc((size_t)n, sizeof(int));
    st.queue = (int *)xcalloc((size_t)n, sizeof(int));
    st.perm = perm;
    st.block_ptr = block_ptr;
    block_ptr[0] = 0;
    if (n > 0) {
        int *S = (int *)xcalloc((size_t)n, sizeof(int));
        for (int i = 0; i < n; ++i) S[i] = i;
        nd_recurse(&st, S, n);
        free(S);
    }
    free(st.inset); free(st.seen); free(st.lev); free(st.queue);
    return st.nblocks;
}

/* ---- setupLinearSystem, arap.h:292-340 ------------------------------------ */

static int setup_linear_system(oracle_arap *oa) {
    free_solver(oa);
    const int m = oa->nfree;
    oa->bfixed = (double *)xcalloc((size_t)3 * m, sizeof(double));
    oa->b = (double *)xcalloc((size_t)3 * m, sizeof(double));
    /* triplets in the order arap.h:310-334 pushes them */
    size_t cap = (size_t)2 * oa->wnnz + 1;
    triplet *t = (triplet *)xcalloc(cap, sizeof(triplet));
    size_t nt = 0;
    for (int vi = 0; vi < oa->V; ++vi) {
        int iidx = oa->free_idx[vi];
        if (iidx == -1) continue;
        for (int q = oa->wrow[vi]; q < oa->wrow[vi + 1]; ++q) {
            int vj = oa->wcol[q];
            int jidx = oa->free_idx[vj];
            double wij = oa->wval[q];
            if (jidx == -1) {
                for (int c = 0; c < 3; ++c)
                    oa->bfixed[3 * iidx + c] = oa->bfixed[3 * iidx + c] + wij * oa->ctarget[3 * vj + c];
            } else {
                t[nt++] = (triplet){iidx, jidx, -wij};
            }
            t[nt++] = (triplet){iidx, iidx, wij};
        }
    }
    int annz;
    triplets_to_csr(m, t, nt, &oa->arow, &oa->acol, &oa->aval, &annz);
    free(t);

    /* ordering: nested dissection on the off-diagonal pattern of L */
    int *grow = (int *)xcalloc((size_t)m + 1, sizeof(int));
    int *gcol = (int *)xcalloc((size_t)annz + 1, sizeof(int));
    int gn = 0;
    for (int i = 0; i < m; ++i) {
        for (int q = oa->arow[i]; q < oa->arow[i + 1]; ++q)
            if (oa->acol[q] != i) gcol[gn++] = oa->acol[q];
        grow[i + 1] = gn;
    }
    oa->perm = (int *)xcalloc((size_t)m + 1, sizeof(int));
    oa->iperm = (int *)xcalloc((size_t)m + 1, sizeof(int));
    oa->block_ptr = (int *)xcalloc((size_t)m + 2, sizeof(int));
    oa->nblocks = oa_nd_order(m, grow, gcol, oa->perm, oa->block_ptr);
    free(grow); free(gcol);
    for (int k = 0; k < m; ++k) oa->iperm[oa->perm[k]] = k;

    /* upper-triangular columns of C = P L P^T: column k holds C(i,k), i <= k */
    int *cp = (int *)xcalloc((size_t)m + 1, sizeof(int));
    for (int a = 0; a < m; ++a) {
        int k = oa->iperm[a];
        for (int q = oa->arow[a]; q < oa->arow[a + 1]; ++q)
            if (oa->iperm[oa->acol[q]] <= k) cp[k + 1]++;
    }
    for (int k = 0; k < m; ++k) cp[k + 1] += cp[k];
    int *ci = (int *)xcalloc((size_t)cp[m] + 1, sizeof(int));
    double *cx = (double *)xcalloc((size_t)cp[m] + 1, sizeof(double));
    int *fill = (int *)xcalloc((size_t)m + 1, sizeof(int));
    memcpy(fill, cp, sizeof(int) * (size_t)m);
    for (int a = 0; a < m; ++a) {
        int k = oa->iperm[a];
        for (int q = oa->arow[a]; q < oa->arow[a + 1]; ++q) {
            int i = oa->iperm[oa->acol[q]];
            if (i <= k) { ci[fill[k]] = i; cx[fill[k]] = oa->aval[q]; fill[k]++; }
        }
    }
    free(fill);

    /* symbolic: elimination tree and column counts (Davis, Algorithm 849) */
    oa->parent = (int *)xcalloc((size_t)m + 1, sizeof(int));
    oa->Lnz = (int *)xcalloc((size_t)m + 1, sizeof(int));
    oa->Lp = (int *)xcalloc((size_t)m + 1, sizeof(int));
    int *flag = (int *)xcalloc((size_t)m + 1, sizeof(int));
    for (int k = 0; k < m; ++k) {
        oa->parent[k] = -1;
        flag[k] = k;
        oa->Lnz[k] = 0;
        for (int q = cp[k]; q < cp[k + 1]; ++q) {
            int i = ci[q];
            if (i < k) {
                for (; flag[i] != k; i = oa->parent[i]) {
                    if (oa->parent[i] == -1) oa->parent[i] = k;
                    oa->Lnz[i]++;
                    flag[i] = k;
                }
            }
        }
    }
    oa->Lp[0] = 0;
    for (int k = 0; k < m; ++k) oa->Lp[k + 1] = oa->Lp[k] + oa->Lnz[k];
    oa->lnnz = oa->Lp[m];
    oa->Li = (int *)xcalloc((size_t)oa->lnnz + 1, sizeof(int));
    oa->Lx = (double *)xcalloc((size_t)oa->lnnz + 1, sizeof(double));
    oa->D = (double *)xcalloc((size_t)m + 1, sizeof(double));

    /* numeric: up-looking LDL^T, row k of L from a sparse triangular solve */
    double *Y = (double *)xcalloc((size_t)m + 1, sizeof(double));
    int *pattern = (int *)xcalloc((size_t)m + 1, sizeof(int));
    int ok = 1;
    for (int k = 0; k < m; ++k) {
        Y[k] = 0.0;
        int top = m;
        flag[k] = k;
        oa->Lnz[k] = 0;
        for (int q = cp[k]; q < cp[k + 1]; ++q) {
            int i = ci[q];
            Y[i] = Y[i] + cx[q];
            int len = 0;
            for (; flag[i] != k; i = oa->parent[i]) {
                pattern[len++] = i;
                flag[i] = k;
            }
            while (len > 0) pattern[--top] = pattern[--len];
        }
        oa->D[k] = Y[k];
        Y[k] = 0.0;
        for (; top < m; ++top) {
            int i = pattern[top];
            double yi = Y[i];
            Y[i] = 0.0;
            int p2 = oa->Lp[i] + oa->Lnz[i];
            for (int q = oa->Lp[i]; q < p2; ++q) Y[oa->Li[q]] = Y[oa->Li[q]] - oa->Lx[q] * yi;
            double lki = yi / oa->D[i];
            oa->D[k] = oa->D[k] - lki * yi;
            oa->Li[p2] = k;
            oa->Lx[p2] = lki;
            oa->Lnz[i]++;
        }
        if (oa->D[k] == 0.0) { ok = 0; break; } /* SimplicialLDLT: NumericalIssue */
    }
    free(Y); free(pattern); free(flag); free(cp); free(ci); free(cx);
    return ok;
}

/* solve C y = P b, then x = P^T y (SimplicialLDLT::solve, arap.h:420) */
static void ldl_solve(const oracle_arap *oa, const double *bin, double *xout, double *work) {
    const int m = oa->nfree;
    for (int k = 0; k < m; ++k) work[k] = bin[oa->perm[k]];
    for (int j = 0; j < m; ++j) { /* L y = b */
        double yj = work[j];
        for (int q = oa->Lp[j]; q < oa->Lp[j + 1]; ++q) work[oa->Li[q]] = work[oa->Li[q]] - oa->Lx[q] * yj;
    }
    for (int j = 0; j < m; ++j) work[j] = work[j] / oa->D[j];
    for (int j = m - 1; j >= 0; --j) { /* L^T x = y */
        double s = work[j];
        for (int q = oa->Lp[j]; q < oa->Lp[j + 1]; ++q) s = s - oa->Lx[q] * work[oa->Li[q]];
        work[j] = s;
    }
    for (int k = 0; k < m; ++k) xout[oa->perm[k]] = work[k];
}

/* ---- one-sided Jacobi SVD of a 3x3 matrix --------------------------------- */

/* A = U diag(s) V^T with s sorted descending, U and V orthogonal (A, U, V
   row-major). Columns of U that belong to zero singular values are completed
   to an orthonormal basis. */
static void svd3_jacobi(const double *Ain, double *U, double *s, double *Vm) {
    double A[9], V[9];
    memcpy(A, Ain, sizeof(A));
    for (int i = 0; i < 9; ++i) V[i] = (i % 4 == 0) ? 1.0 : 0.0;
    double f2 = 0.0; /* squared Frobenius norm: pairs whose coupling is below
                        eps relative to the whole matrix are left alone */
    for (int i = 0; i < 9; ++i) f2 = f2 + A[i] * A[i];
    for (int sweep = 0; sweep < 60; ++sweep) {
        int rotated = 0;
        for (int p = 0; p < 2; ++p) {
            for (int q = p + 1; q < 3; ++q) {
                double alpha = 0.0, beta = 0.0, gamma = 0.0;
                for (int r = 0; r < 3; ++r) {
                    alpha = alpha + A[3 * r + p] * A[3 * r + p];
                    beta = beta + A[3 * r + q] * A[3 * r + q];
                    gamma = gamma + A[3 * r + p] * A[3 * r + q];
                }
                if (gamma == 0.0 || fabs(gamma) <= 1e-15 * sqrt(alpha * beta) || fabs(gamma) <= 1e-16 * f2) continue;
                rotated = 1;
                double zeta = (beta - alpha) / (2.0 * gamma);
                double tt = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                double c = 1.0 / sqrt(1.0 + tt * tt);
                double sn = c * tt;
                for (int r = 0; r < 3; ++r) {
                    double ap = A[3 * r + p], aq = A[3 * r + q];
                    A[3 * r + p] = c * ap - sn * aq;
                    A[3 * r + q] = sn * ap + c * aq;
                    double vp = V[3 * r + p], vq = V[3 * r + q];
                    V[3 * r + p] = c * vp - sn * vq;
                    V[3 * r + q] = sn * vp + c * vq;
                }
            }
        }
        if (!rotated) break;
    }
    double nrm[3];
    for (int k = 0; k < 3; ++k)
        nrm[k] = sqrt(A[k] * A[k] + A[3 + k] * A[3 + k] + A[6 + k] * A[6 + k]);
    int ord[3] = {0, 1, 2};
    for (int a = 0; a < 3; ++a)
        for (int b = a + 1; b < 3; ++b)
            if (nrm[ord[b]] > nrm[ord[a]]) { int t = ord[a]; ord[a] = ord[b]; ord[b] = t; }
    double Uc[3][3] = {{0}}, Vc[3][3];
    for (int k = 0; k < 3; ++k) {
        int o = ord[k];
        s[k] = nrm[o];
        for (int r = 0; r < 3; ++r) Vc[k][r] = V[3 * r + o];
    }
    const double tiny = 1e-300;
    const double rel = (s[0] > 0.0 ? s[0] : 1.0) * 1e-14;
    int have = 0;
    for (int k = 0; k < 3; ++k) {
        int o = ord[k];
        if (s[k] > tiny && s[k] > rel) {
            for (int r = 0; r < 3; ++r) Uc[k][r] = A[3 * r + o] / s[k];
            have = k + 1;
        } else {
            break;
        }
    }
    if (have == 0) { Uc[0][0] = 1.0; Uc[0][1] = 0.0; Uc[0][2] = 0.0; have = 1; }
    if (have == 1) { /* any unit vector orthogonal to u0 */
        const double *u = Uc[0];
        double e[3] = {0, 0, 0};
        int m = 0;
        if (fabs(u[1]) < fabs(u[m])) m = 1;
        if (fabs(u[2]) < fabs(u[m])) m = 2;
        e[m] = 1.0;
        double d = e[0] * u[0] + e[1] * u[1] + e[2] * u[2];
        double w[3] = {e[0] - d * u[0], e[1] - d * u[1], e[2] - d * u[2]};
        double n = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
        for (int r = 0; r < 3; ++r) Uc[1][r] = w[r] / n;
        have = 2;
    }
    if (have == 2) { /* u2 = u0 x u1 */
        Uc[2][0] = Uc[0][1] * Uc[1][2] - Uc[0][2] * Uc[1][1];
        Uc[2][1] = Uc[0][2] * Uc[1][0] - Uc[0][0] * Uc[1][2];
        Uc[2][2] = Uc[0][0] * Uc[1][1] - Uc[0][1] * Uc[1][0];
    }
    for (int r = 0; r < 3; ++r)
        for (int k = 0; k < 3; ++k) {
            U[3 * r + k] = Uc[k][r];
            Vm[3 * r + k] = Vc[k][r];
        }
}

static double det3(const double *M) {
    return M[0] * (M[4] * M[8] - M[5] * M[7]) - M[1] * (M[3] * M[8] - M[5] * M[6]) +
           M[2] * (M[3] * M[7] - M[4] * M[6]);
}

/* arap.h:376-382: R = V diag(1, 1, det(V U^T)) U^T */
void oa_rotation_from_covariance(const double *cov, double *R) {
    double U[9], s[3], V[9], VUt[9];
    svd3_jacobi(cov, U, s, V);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double a = 0.0;
            for (int k = 0; k < 3; ++k) a = a + V[3 * i + k] * U[3 * j + k];
            VUt[3 * i + j] = a;
        }
    double d = det3(VUt);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            R[3 * i + j] = V[3 * i + 0] * U[3 * j + 0] + V[3 * i + 1] * U[3 * j + 1] + d * V[3 * i + 2] * U[3 * j + 2];
}

/* estimateRotations, arap.h:354-384 */
static void estimate_rotations(oracle_arap *oa) {
    for (int vi = 0; vi < oa->V; ++vi) {
        const double *pi = oa->p + 3 * vi, *ppi = oa->pp + 3 * vi;
        double cov[9] = {0};
        for (int q = oa->wrow[vi]; q < oa->wrow[vi + 1]; ++q) {
            const int vj = oa->wcol[q];
            const double wij = oa->wval[q];
            const double *pj = oa->p + 3 * vj, *ppj = oa->pp + 3 * vj;
            double e[3], f[3];
            for (int c = 0; c < 3; ++c) { e[c] = pi[c] - pj[c]; f[c] = ppi[c] - ppj[c]; }
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) cov[3 * r + c] = cov[3 * r + c] + wij * e[r] * f[c];
        }
        oa_rotation_from_covariance(cov, oa->R + 9 * vi);
    }
}

/* ARAP energy of the current positions (not computed by the reference; the
   quantity its local/global iteration decreases, Sorkine & Alexa 2007 eq. 3
   with the cotan weights of arap.h:182-239): for every vertex the rotation
   estimate_rotations would fit to its one-ring now, then
   sum_i sum_j w_ij |(p'_i - p'_j) - R_i (p_i - p_j)|^2 over all adjacency
   entries. Vertices in ascending order, entries in CSR order. */
double oa_energy(const oracle_arap *oa) {
    double total = 0.0;
    for (int vi = 0; vi < oa->V; ++vi) {
        const double *pi = oa->p + 3 * vi, *ppi = oa->pp + 3 * vi;
        double cov[9] = {0}, R[9];
        for (int q = oa->wrow[vi]; q < oa->wrow[vi + 1]; ++q) {
            const int vj = oa->wcol[q];
            const double wij = oa->wval[q];
            const double *pj = oa->p + 3 * vj, *ppj = oa->pp + 3 * vj;
            double e[3], f[3];
            for (int c = 0; c < 3; ++c) { e[c] = pi[c] - pj[c]; f[c] = ppi[c] - ppj[c]; }
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) cov[3 * r + c] = cov[3 * r + c] + wij * e[r] * f[c];
        }
        oa_rotation_from_covariance(cov, R);
        double ev = 0.0;
        for (int q = oa->wrow[vi]; q < oa->wrow[vi + 1]; ++q) {
            const int vj = oa->wcol[q];
            const double *pj = oa->p + 3 * vj, *ppj = oa->pp + 3 * vj;
            double d[3], r2 = 0.0;
            for (int c = 0; c < 3; ++c) d[c] = pi[c] - pj[c];
            for (int c = 0; c < 3; ++c) {
                const double rc = (ppi[c] - ppj[c]) - (R[3 * c + 0] * d[0] + R[3 * c + 1] * d[1] + R[3 * c + 2] * d[2]);
                r2 = r2 + rc * rc;
            }
            ev = ev + oa->wval[q] * r2;
        }
        total = total + ev;
    }
    return total;
}

/* estimatePositions, arap.h:393-430 */
static void estimate_positions(oracle_arap *oa, double *work, double *rhs, double *u) {
    const int m = oa->nfree;
    memcpy(oa->b, oa->bfixed, sizeof(double) * 3 * (size_t)m);
    for (int vi = 0; vi < oa->V; ++vi) {
        int iidx = oa->free_idx[vi];
        if (iidx == -1) continue;
        for (int q = oa->wrow[vi]; q < oa->wrow[vi + 1]; ++q) {
            const int vj = oa->wcol[q];
            const double wij = oa->wval[q];
            double r[9], d[3];
            for (int a = 0; a < 9; ++a) r[a] = oa->R[9 * vi + a] + oa->R[9 * vj + a];
            for (int c = 0; c < 3; ++c) d[c] = oa->p[3 * vi + c] - oa->p[3 * vj + c];
            for (int c = 0; c < 3; ++c) {
                double pt = r[3 * c + 0] * d[0] + r[3 * c + 1] * d[1] + r[3 * c + 2] * d[2];
                pt = pt * wij * 0.5;
                oa->b[3 * iidx + c] = oa->b[3 * iidx + c] + pt;
            }
        }
    }
    for (int c = 0; c < 3; ++c) {
        for (int i = 0; i < m; ++i) rhs[i] = oa->b[3 * i + c];
        ldl_solve(oa, rhs, u, work);
        int idx = 0;
        for (int vi = 0; vi < oa->V; ++vi)
            if (oa->free_idx[vi] != -1) oa->pp[3 * vi + c] = u[idx++];
    }
}

/* deform, arap.h:101-138 */
int oa_deform(oracle_arap *oa, int iterations) {
    if (oa->dirty) {
        initialize_mesh_geometry(oa);
        compute_cotan_weights(oa);
        initialize_rotations(oa);
        initialize_free_variable_mapping(oa);
        initialize_constraints(oa);
        if (oa->nfree == oa->V) return 1; /* arap.h:113-114: no write-back */
        if (!setup_linear_system(oa)) return 0;
        oa->dirty = 0;
    }
    const int m = oa->nfree;
    double *work = (double *)xcalloc((size_t)m + 1, sizeof(double));
    double *rhs = (double *)xcalloc((size_t)m + 1, sizeof(double));
    double *u = (double *)xcalloc((size_t)m + 1, sizeof(double));
    for (int i = 0; i < iterations; ++i) {
        estimate_rotations(oa);
        estimate_positions(oa, work, rhs, u);
    }
    free(work); free(rhs); free(u);
    memcpy(oa->mesh, oa->pp, sizeof(double) * 3 * (size_t)oa->V); /* arap.h:133-135 */
    return 1;
}

/* ---- introspection ---------------------------------------------------------- */

int oa_num_free(const oracle_arap *oa) { return oa->nfree; }
int oa_weights_nnz(const oracle_arap *oa) { return oa->wnnz; }

void oa_get_weights(const oracle_arap *oa, int *rowptr, int *col, double *val) {
    if (!oa->wrow) return;
    memcpy(rowptr, oa->wrow, sizeof(int) * ((size_t)oa->V + 1));
    memcpy(col, oa->wcol, sizeof(int) * (size_t)oa->wnnz);
    memcpy(val, oa->wval, sizeof(double) * (size_t)oa->wnnz);
}

void oa_get_rotations(const oracle_arap *oa, double *R9) {
    memcpy(R9, oa->R, sizeof(double) * 9 * (size_t)oa->V);
}

void oa_get_free_map(const oracle_arap *oa, int *free_idx) {
    memcpy(free_idx, oa->free_idx, sizeof(int) * (size_t)oa->V);
}

void oa_get_bfixed(const oracle_arap *oa, double *b) {
    if (oa->bfixed) memcpy(b, oa->bfixed, sizeof(double) * 3 * (size_t)oa->nfree);
}

void oa_get_ordering(const oracle_arap *oa, int *perm) {
    if (oa->perm) memcpy(perm, oa->perm, sizeof(int) * (size_t)oa->nfree);
}

void oa_get_etree(const oracle_arap *oa, int *parent) {
    if (oa->parent) memcpy(parent, oa->parent, sizeof(int) * (size_t)oa->nfree);
}

int oa_num_blocks(const oracle_arap *oa) { return oa->nblocks; }

void oa_get_blocks(const oracle_arap *oa, int *block_ptr) {
    if (oa->block_ptr) memcpy(block_ptr, oa->block_ptr, sizeof(int) * ((size_t)oa->nblocks + 1));
}

long long oa_factor_nnz(const oracle_arap *oa) { return oa->lnnz; }

// arap_wsolve.cuh -- triangular solves of the small supernodes at the bottom
// of the elimination tree, one warp per supernode (inc/deform/arap.h:417-429,
// the L^-1 and L^-T halves of SimplicialLDLT::solve, for the levels whose
// fronts hold at most kWarpRows rows).
//
// The bottom levels hold most of the tree's supernodes (the twisted bar: 1,077
// leaves of at most 121 rows, 2,063 supernodes in its five lowest levels) and
// each of them is a small matrix-vector product. A warp per supernode, with
// its front in a private slice of shared memory and no CTA barrier, keeps
// every leaf of a level in flight at once (16 warps per SM) where a CTA per
// supernode runs them in waves. Tasks are taken from a ticket counter in the
// order of `order` (leaves first for the forward sweep, reversed for the
// backward one); a warp waits (bounded) for the completion flags of the tasks
// it depends on, which always hold smaller tickets and so belong to running
// warps. Included by arap_kernels.cu inside its anonymous namespace, after
// the flag and load helpers.

constexpr int kWarpRows = 256;        // largest front (rows) a warp task holds
constexpr int kWarpThreads = 256;     // 8 warps per CTA
constexpr int kWarpsPerCta = kWarpThreads / 32;

// Next task of the calling warp (all lanes): lane 0 takes the ticket. A launch
// of W warps over S tasks consumes exactly Z = S + W tickets, as the CTA
// solves do per CTA.
__device__ __forceinline__ void next_wtask(unsigned long long *ticket, int S, int Z, const int32_t *order,
                                           bool reverse, const int *err, int &task, unsigned &epoch) {
    int tk = -1;
    unsigned ep = 0;
    if ((threadIdx.x & 31) == 0) next_task(ticket, S, Z, order, reverse, err, tk, ep);
    task = __shfl_sync(0xffffffffu, tk, 0);
    epoch = __shfl_sync(0xffffffffu, ep, 0);
}

// out_r = sum_c M(r, c) v_c for r < rows, c < cols (M column-major, leading
// dimension ld a multiple of 4, columns 16-byte aligned), by one warp. Rows
// go in quads of four (one vector load per quad and column). With at least 32
// quads each lane takes the quads lane, lane + 32, ...; with fewer the quads
// are replicated over G = 32 / NQp column groups (NQp: quads rounded up to a
// power of two) and the groups' partial sums meet by shuffles. TRI: M is
// lower (1) or upper (2) triangular and the zero quads of a column are
// skipped. Every lane returns the sums of its quads (lanes of group 0 hold
// the totals when the columns are split).
template <typename T, int TRI>
__device__ __forceinline__ void warp_gemv(const T *__restrict__ M, int ld, int rows, int cols, const Vec4<T> *v,
                                          T ax[2][4], T ay[2][4], T az[2][4], int &q0, int &nq, int &g) {
    const int lane = threadIdx.x & 31;
    const int NQ = (rows + 3) >> 2;
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int k = 0; k < 4; ++k) ax[a][k] = ay[a][k] = az[a][k] = (T)0;
    int G, NQp = 1;
    if (NQ >= 32) {
        G = 1;
        g = 0;
        q0 = lane;
        nq = NQ > 32 + lane ? 2 : 1;
    } else {
        while (NQp < NQ) NQp <<= 1;
        G = 32 / NQp;
        q0 = lane & (NQp - 1);
        g = lane / NQp;
        nq = q0 < NQ ? 1 : 0;
    }
#pragma unroll 4
    for (int c = g; c < cols; c += G) {
        const Vec4<T> vc = v[c];
        const T *col = M + (int64_t)c * ld;
#pragma unroll
        for (int a = 0; a < 2; ++a) {
            const int q = q0 + 32 * a;
            if (a >= nq) continue;
            if (TRI == 1 && 4 * q + 3 < c) continue;  // rows above the diagonal: zero
            if (TRI == 2 && 4 * q > c) continue;      // rows below the diagonal: zero
            const Vec4<T> m = *reinterpret_cast<const Vec4<T> *>(col + 4 * q);
            ax[a][0] += m.x * vc.x; ay[a][0] += m.x * vc.y; az[a][0] += m.x * vc.z;
            ax[a][1] += m.y * vc.x; ay[a][1] += m.y * vc.y; az[a][1] += m.y * vc.z;
            ax[a][2] += m.z * vc.x; ay[a][2] += m.z * vc.y; az[a][2] += m.z * vc.z;
            ax[a][3] += m.w * vc.x; ay[a][3] += m.w * vc.y; az[a][3] += m.w * vc.z;
        }
    }
    if (G > 1) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            if (off < NQp) break;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                ax[0][k] += __shfl_xor_sync(0xffffffffu, ax[0][k], off);
                ay[0][k] += __shfl_xor_sync(0xffffffffu, ay[0][k], off);
                az[0][k] += __shfl_xor_sync(0xffffffffu, az[0][k], off);
            }
        }
    }
}

// Forward sweep over the supernodes order[0, S): f = [b(cols); 0] plus the
// children's update vectors (children in order), y = X f(cols), u = f(struct)
// - L21 y for the parent. Children at levels >= lend belong to another launch
// (never the case for the bottom levels this kernel takes).
template <typename T>
__global__ void __launch_bounds__(kWarpThreads)
k_wsolve_fwd(int S, int Z, const int32_t *__restrict__ order, const SnInfo *__restrict__ sn,
             const int32_t *__restrict__ child, const int32_t *__restrict__ relind, const T *__restrict__ Xall,
             const T *__restrict__ L21all, Vec4<T> *__restrict__ sol, Vec4<T> *__restrict__ uvec,
             unsigned long long *ticket, unsigned *flags, int *err) {
    extern __shared__ __align__(32) unsigned char wsmem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    Vec4<T> *f = reinterpret_cast<Vec4<T> *>(wsmem) + (size_t)warp * kWarpRows;
    for (;;) {
        int s;
        unsigned epoch;
        next_wtask(ticket, S, Z, order, false, err, s, epoch);
        if (s < 0) return;
        const SnInfo d = sn[s];
        const int nc = d.ncol, nb = d.nrow - d.ncol;
        if (lane == 0)
            for (int ci = d.child_begin; ci < d.child_end; ++ci) wait_flag(flags + child[ci], epoch, err);
        for (int i = lane; i < d.nrow; i += 32) f[i] = i < nc ? sol[d.first + i] : Vec4<T>{(T)0, (T)0, (T)0, (T)0};
        __syncwarp();
        for (int ci = d.child_begin; ci < d.child_end; ++ci) {  // children in order
            const SnInfo c = sn[child[ci]];
            const int nbc = c.nrow - c.ncol;
            const int32_t *ri = relind + c.relind_off;
            for (int i = lane; i < nbc; i += 32) {
                const Vec4<T> u = ldcg4(uvec + c.uvec_off + i);
                Vec4<T> &t = f[ri[i]];
                t.x += u.x;
                t.y += u.y;
                t.z += u.z;
            }
            __syncwarp();
        }
        T ax[2][4], ay[2][4], az[2][4];
        int q0, nq, g;
        // y = X f(cols), X lower triangular
        warp_gemv<T, 1>(Xall + d.x_off, d.ldx, nc, nc, f, ax, ay, az, q0, nq, g);
        __syncwarp();  // every lane has read f(cols)
        if (g == 0)
#pragma unroll
            for (int a = 0; a < 2; ++a)
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int r = 4 * (q0 + 32 * a) + k;
                    if (a < nq && r < nc) f[r] = {ax[a][k], ay[a][k], az[a][k], (T)0};
                }
        __syncwarp();
        // u = f(struct) - L21 y
        if (nb > 0) {
            warp_gemv<T, 0>(L21all + d.l21_off, d.ld21, nb, nc, f, ax, ay, az, q0, nq, g);
            if (g == 0)
#pragma unroll
                for (int a = 0; a < 2; ++a)
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const int r = 4 * (q0 + 32 * a) + k;
                        if (a < nq && r < nb) {
                            const Vec4<T> fb = f[nc + r];
                            uvec[d.uvec_off + r] = {fb.x - ax[a][k], fb.y - ay[a][k], fb.z - az[a][k], (T)0};
                        }
                    }
        }
        // the warp barrier orders every lane's writes before lane 0's release,
        // which is cumulative: a warp or CTA that acquires the flag sees them
        __syncwarp();
        if (lane == 0) st_release(flags + s, epoch);
        // y is read only by the backward sweep (a later launch)
        for (int i = lane; i < nc; i += 32) sol[d.first + i] = f[i];
        __syncwarp();  // the next task rewrites f
    }
}

// Backward sweep over order[0, S) reversed (roots of the bottom levels
// first): z = y - L21^T g with g the solution at the struct rows, x = X^T z.
// A parent at a level >= lend was finished by an earlier launch.
// mode 0: pc64 = x; mode 1: pc64 += x, pc32 = float(pc64).
template <typename T>
__global__ void __launch_bounds__(kWarpThreads)
k_wsolve_bwd(int S, int Z, int lend, const int32_t *__restrict__ order, const SnInfo *__restrict__ sn,
             const int32_t *__restrict__ rows, const T *__restrict__ Xall, const T *__restrict__ L21Tall,
             Vec4<T> *__restrict__ sol, Vec4<double> *__restrict__ pc64, Vec4<float> *__restrict__ pc32, int mode,
             unsigned long long *ticket, unsigned *flags, int *err) {
    extern __shared__ __align__(32) unsigned char wsmem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    Vec4<T> *zv = reinterpret_cast<Vec4<T> *>(wsmem) + (size_t)warp * kWarpRows;  // z then x: ncol rows
    for (;;) {
        int s;
        unsigned epoch;
        next_wtask(ticket, S, Z, order, true, err, s, epoch);
        if (s < 0) return;
        const SnInfo d = sn[s];
        const int nc = d.ncol, nb = d.nrow - d.ncol;
        Vec4<T> *gv = zv + nc;  // g: the struct rows' solution
        if (lane == 0 && d.parent >= 0 && sn[d.parent].level < lend) wait_flag(flags + d.parent, epoch, err);
        __syncwarp();
        const int32_t *rs = rows + d.rows_off;
        for (int i = lane; i < nc; i += 32) zv[i] = sol[d.first + i];
        for (int i = lane; i < nb; i += 32) gv[i] = ldcg4(sol + rs[i]);
        __syncwarp();
        T ax[2][4], ay[2][4], az[2][4];
        int q0, nq, g;
        if (nb > 0) {
            // z -= L21^T g (L21^T: nb columns of ldx rows)
            warp_gemv<T, 0>(L21Tall + d.l21t_off, d.ldx, nc, nb, gv, ax, ay, az, q0, nq, g);
            if (g == 0)
#pragma unroll
                for (int a = 0; a < 2; ++a)
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const int r = 4 * (q0 + 32 * a) + k;
                        if (a < nq && r < nc) {
                            Vec4<T> &z = zv[r];
                            z.x -= ax[a][k];
                            z.y -= ay[a][k];
                            z.z -= az[a][k];
                        }
                    }
            __syncwarp();
        }
        // x = X^T z (X^T upper triangular)
        warp_gemv<T, 2>(Xall + d.xt_off, d.ldx, nc, nc, zv, ax, ay, az, q0, nq, g);
        __syncwarp();  // every lane has read z
        if (g == 0)
#pragma unroll
            for (int a = 0; a < 2; ++a)
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int r = 4 * (q0 + 32 * a) + k;
                    if (a < nq && r < nc) {
                        const Vec4<T> x = {ax[a][k], ay[a][k], az[a][k], (T)0};
                        zv[r] = x;
                        sol[d.first + r] = x;
                    }
                }
        __syncwarp();
        if (lane == 0) st_release(flags + s, epoch);
        // the positions are read by no other task of this sweep
        for (int i = lane; i < nc; i += 32) {
            const Vec4<T> x = zv[i];
            const int k = d.first + i;
            if (mode == 0) {
                pc64[k] = {(double)x.x, (double)x.y, (double)x.z, 0.0};
            } else {
                Vec4<double> p = pc64[k];
                p.x += (double)x.x;
                p.y += (double)x.y;
                p.z += (double)x.z;
                pc64[k] = p;
                pc32[k] = {(float)p.x, (float)p.y, (float)p.z, 0.f};
            }
        }
        __syncwarp();  // the next task rewrites zv
    }
}

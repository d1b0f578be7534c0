// arap_kernels.h -- launch interface of the sm_103a ARAP kernels.
//
// Device data layout (all arrays in device order: free vertices in
// nested-dissection elimination order [0, m), constrained vertices [m, V) in
// ascending vertex order):
//   positions   V x {x,y,z,0} in Vec4<T> (16 B for float, 32 B for double)
//   rotations   V x 3 rows of Vec4<T> (row-major R, 4th lane unused)
//   adjacency   CSR drow/dcol with weights w (per device entry)
//   factor      per supernode an nrow x ncol column-major panel (L11 lower
//               triangle, then L21) and the inverses of its 32x32 diagonal blocks
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "arap_symbolic.h"

namespace arapgpu {

template <typename T> struct __align__(4 * sizeof(T)) Vec4 { T x, y, z, w; };

// error bits written by kernels into the context's device status word
constexpr int kErrNotSpd = 1;
constexpr int kErrTimeout = 2;

// Bound on the polls of one in-kernel wait (each poll sleeps 20-200 ns, so
// the bound is a few seconds).
constexpr unsigned kSpinLimit = 1u << 24;

// The context's device status word is two ints: err[0] collects the error
// bits of a deform, err[1] is the poll limit of the waits for another task's
// flag (0: kSpinLimit), set by arap_set_wait_limit. The waits for a CTA's own
// bulk copies always use kSpinLimit, so that no copy is left in flight.
#ifdef __CUDACC__
__device__ __forceinline__ unsigned flag_wait_limit(const int *err) {
    const unsigned v = (unsigned)__ldcg(err + 1);
    return v == 0u ? kSpinLimit : v;
}
#endif

// level schedule of the single-request solves: at most this many tree levels
// (deeper trees keep the persistent schedule). The forward sweep's launch for
// level l takes its tickets from counter kLevelTicket0 + 2 l of the counter
// array it is given, the backward sweep's from the same index of its array
// (the backward sweeps are given the array one counter further on).
constexpr int kMaxLevelLaunch = 48;
constexpr int kLevelTicket0 = 8;

// launch shape of a per-vertex kernel of the single-request iterations
// (arap_set_vertex_launch): tpv lanes of one warp per vertex (1, 2, 4, 8 or
// 32), block threads a multiple of 32 (and of tpv) up to 1024
struct VertexLaunch {
    int tpv, block;
};
enum { kVertexLocal = 0, kVertexRhs = 1, kVertexResidual = 2, kVertexKernels = 3 };
// largest block of the local step (its FP64 refit needs the registers of at
// most 256 threads per block); the RHS and the residual take up to 1024
constexpr int kLocalMaxBlock = 256;

struct DevTopo {
    int V, F, nnz;
    const int32_t *faces;    // 3F (original vertex ids)
    const int32_t *ent_ptr;  // nnz+1 (original CSR entries)
    const int32_t *ent_fc;   // face*3+k
};

struct DevSym {
    int V, m, S, nnz;
    int s_sched;  // entries of level_sn (the supernodes the sweeps schedule; below S with solve blocks)
    int max_ldx, max_ld21, max_ncol;
    int solve_grid32, solve_grid64;  // CTAs per lower-level solve launch (each loops over tickets)
    // the solves split the tree: levels [0, ltop) by single CTAs (s_low tasks),
    // levels [ltop, top) by clusters (s_top tasks, top_clusters clusters)
    int ltop, s_low, s_top, top_clusters;
    // the bottom levels [0, lwarp) (s_warp supernodes, fronts of at most
    // wsolve_max_rows() rows) are solved one warp per supernode, in wgrid
    // CTAs, before (forward) / after (backward) the CTA sweep of the levels
    // [lwarp, ltop)
    int lwarp, s_warp, wgrid32, wgrid64;
    int top_ldx, top_ld21;  // largest front of the cluster levels (their shared-memory layout)
    // level schedule (arap_set_solve_schedule): the CTA sweep of the levels
    // [lwarp, ltop) as one launch per level instead of one persistent launch;
    // level l holds the supernodes level_sn[lev_ptr[l], lev_ptr[l+1]), its
    // fronts fit lev_ldx[l] / lev_ld21[l] rows, lev_grid32/64[l] CTAs
    VertexLaunch vlaunch[kVertexKernels];
    // the persistent sweeps and the dense top's products start while the
    // kernel before them finishes (programmatic dependent launch): set when
    // the sweeps' grids fill the device (no CTA cap); with a cap, requests
    // share the SMs and early-resident waiting CTAs would hold them
    int overlap;
    int level_launch;
    int lev_ptr[kMaxLevelLaunch + 1], lev_ldx[kMaxLevelLaunch], lev_ld21[kMaxLevelLaunch];
    int lev_grid32[kMaxLevelLaunch], lev_grid64[kMaxLevelLaunch];
    // dense top (levels [ltop, top) when n_top > 0, instead of cluster levels):
    // n_top columns, T = inv(L_top) formed by n_top_items CTAs
    int n_top, n_top_items, dense_ldx, dense_ld21;
    // the top's products take two tiles per CTA (T staged in shared memory)
    // when one tile per CTA would need more than one wave (FP32 / FP64)
    int top_pair32, top_pair64;
    const int32_t *top_col;    // n_top: device column of each dense index
    const int32_t *top_gptr;   // n_top + 1: update-vector entries added to each dense row
    const int64_t *top_gidx;   // their offsets in the update-vector array
    const int32_t *tdpos;      // S: dense index of a top supernode's first column (-1 elsewhere)
    const int32_t *top_items;  // 2 per CTA: supernode, first column
    const int32_t *drow, *dcol, *dent, *oldidx;
    const int64_t *amap, *dmap;
    const SnInfo *sn;
    const int32_t *rows, *relind, *child, *level_sn;
};

// raises (never lowers) a kernel's dynamic shared-memory limit on the current device
cudaError_t raise_smem_limit(const void *func, int bytes);
// cotangent halves per face (computeCotanWeights arap.h:189-222), FP64
void launch_face_cots(const DevTopo &t, const double *rest_xyz, double *hc, cudaStream_t st);
// edge weights per device entry (w64/w32) and per original entry (w_orig); any
// output may be null. arap.h:224-238
void launch_edge_weights(const DevTopo &t, const DevSym &s, const double *hc, double *w64, float *w32,
                         double *w_orig, cudaStream_t st);
// weights per original entry only (no symbolic analysis yet)
void launch_edge_weights_orig(const DevTopo &t, const double *hc, double *w_orig, cudaStream_t st);
// rest / current positions in device order (initializeMeshGeometry arap.h:162-168,
// initializeConstraints arap.h:277-281), rotations reset (arap.h:246-249)
template <typename T>
void launch_setup_vertices(const DevSym &s, const double *rest_xyz, const double *targets_xyz,
                           Vec4<double> *p64, Vec4<double> *pc64, Vec4<T> *p_t, Vec4<T> *pc_t, Vec4<T> *R,
                           cudaStream_t st);
// constrained Laplacian into the supernodal panels + bFixed (arap.h:292-336)
template <typename TF>
void launch_assemble(const DevSym &s, const double *w64, const Vec4<double> *pc64, TF *Lval, double *diag64,
                     Vec4<double> *bfixed, cudaStream_t st);
// bFixed alone for a re-pose with the same constrained set
void launch_bfixed(const DevSym &s, const double *w64, const Vec4<double> *pc64, Vec4<double> *bfixed,
                   cudaStream_t st);
// FP32 rest edge vectors per adjacency entry, differenced in FP64
void launch_rest_edges(const DevSym &s, const Vec4<double> *p64, Vec4<float> *redge, cudaStream_t st);
// mixed form: FP32 covariance from FP32 rest edges and FP64-differenced current edges;
// one-rings whose covariance is close to rank one are fitted again in FP64
// from the FP64 weights and rest positions p64
void launch_local_step_mixed(const DevSym &s, const float *w32, const Vec4<float> *redge, const Vec4<double> *pc64,
                             Vec4<float> *R, const double *w64, const Vec4<double> *p64, cudaStream_t st);
// mixed form: the RHS terms sum 1/2 w (Ri+Rj)(pi-pj) without bFixed
void launch_rhs_mixed(const DevSym &s, const float *w32, const Vec4<float> *redge, const Vec4<float> *R,
                      Vec4<float> *b, cudaStream_t st);
// one launch of the multifrontal Cholesky plan (Symbolic::fplan); the last
// launches of a level also write X = inverse of L11 and the aligned copies of
// L21 and L21^T that the solves read
template <typename TF>
void launch_factor_step(const DevSym &s, const FactorLaunch &fl, const FItem *items, TF *Lval, TF *Upd, TF *Dinv,
                        TF *X, TF *L21, TF *L21T, int *err, cudaStream_t st);
// largest solve block (columns; arap_set_solve_blocks)
constexpr int kMaxSolveBlock = 1024;
// the solve blocks (SolveBlocks: a level-1 supernode with its leaf children)
// from the supernodes' inverses X (k_fx) and the panels: X_b, X_b^T, L21_b,
// L21_b^T at the blocks' offsets of the same arrays (bsn: the solve array)
template <typename TF>
void launch_solve_blocks(int nblocks, const int32_t *items, const int32_t *members, const SnInfo *sn,
                         const SnInfo *bsn, const int32_t *relind, const TF *Lval, TF *X, TF *L21, TF *L21T,
                         cudaStream_t st);
// FP64 factor outputs (X, L21, L21^T, the dense top's T) rounded to the FP32
// copies the mixed form's solves read: count <= 4 arrays of n[a] elements
void launch_demote(int count, const double *const *src, float *const *dst, const int64_t *n, cudaStream_t st);
// local step: covariance + rotation fit (estimateRotations arap.h:354-384)
template <typename T>
void launch_local_step(const DevSym &s, const T *w, const Vec4<T> *p, const Vec4<T> *pc, Vec4<T> *R,
                       cudaStream_t st);
// RHS (estimatePositions arap.h:395-414): b = bFixed + sum 1/2 w (Ri+Rj)(pi-pj)
template <typename T>
void launch_rhs(const DevSym &s, const T *w, const Vec4<T> *p, const Vec4<T> *R, const Vec4<T> *bfixed,
                Vec4<T> *b, cudaStream_t st);
// FP64 residual of the global system: r = (bFixed + b) - A x over the free vertices
void launch_residual(const DevSym &s, const double *w64, const double *diag64, const Vec4<double> *bfixed,
                     const Vec4<float> *b, const Vec4<double> *x64, Vec4<float> *r, cudaStream_t st);
// supernodal triangular solves L y = b (forward) and L^T x = y (backward),
// one launch each, supernodes scheduled by a ticket counter with bounded waits.
// mode 0: pc64[k] = x_k; mode 1: pc64[k] += x_k and pc32[k] = float(pc64[k]).
// rows of one pass of a solve GEMV phase (one 4-row quad per thread); the
// single-CTA solves take larger fronts in several passes, the cluster solves
// take fronts of at most this many rows
constexpr int kSolveBlockRows = 1024;
// bytes of one chunk buffer of the solves (a matrix column must fit one)
int solve_chunk_bytes();
// warp-per-supernode solves of the bottom levels: largest front, dynamic shared
// memory per CTA, shared-memory limits, CTAs resident on the device
int wsolve_max_rows();
size_t wsolve_smem_bytes(int scalar_bytes);
cudaError_t configure_wsolve();
int wsolve_resident_ctas(int scalar_bytes);
size_t solve_smem_bytes(int ldx_max, int ld21_max, int scalar_bytes);
// solve CTAs resident on the device at once (occupancy x SMs) for that shared memory
int solve_resident_ctas(int smem_bytes, int scalar_bytes);
// shared memory of the cluster solves of the top levels, and its limit
size_t top_smem_bytes(int ldx_max, int ld21_max, int scalar_bytes);
cudaError_t configure_top_smem(int bytes_f32, int bytes_f64);
// a tree level goes to the cluster solves when one of its supernodes holds at
// least this many bytes of X and L21 (FP32), and every level above does too
#ifndef ARAP_TOP_TASK_KB
#define ARAP_TOP_TASK_KB 128
#endif
constexpr int kTopTaskBytes = ARAP_TOP_TASK_KB * 1024;
constexpr int kTopMaxClusters = 16;
template <typename T>
void launch_solve_fwd(const DevSym &s, const T *X, const T *L21, Vec4<T> *sol, Vec4<T> *uvec,
                      unsigned long long *ticket, unsigned *flags, int *err, cudaStream_t st, const T *Ttop,
                      Vec4<T> *ytop);
template <typename T>
void launch_solve_bwd(const DevSym &s, const T *X, const T *L21T, Vec4<T> *sol, Vec4<double> *pc64,
                      Vec4<float> *pc32, int mode, unsigned long long *ticket, unsigned *flags, int *err,
                      cudaStream_t st, const T *Ttop, const Vec4<T> *ytop);
// T = inv(L_top) of the dense top (n_top rows of dense_ld(n_top), row-major, zero
// above the diagonal), followed by T^T in the same layout
template <typename T>
void launch_top_inverse(const DevSym &s, const T *X, const T *L21, T *Tt, cudaStream_t st);
size_t dense_inverse_smem_bytes(int ldx_max, int ld21_max, int scalar_bytes, int rc);
// columns per pass of the inversion whose buffers fit shared memory (0: none)
int dense_inverse_rhs(int ldx_max, int ld21_max, int scalar_bytes);
// leading dimension of the dense top's T and T^T rows, and the elements of both
int dense_ld(int n);
size_t dense_top_elems(int n);
// the products with T (forward) and T^T (backward, T read by columns) run
// over kTopTile x kTopTile tiles of T's lower triangle, two per CTA; the
// vector buffer (ytop) holds y_top, the tiles' partial products and one
// arrival counter per block of kTopTile rows (zero between launches)
constexpr int kTopTile = 64;
int top_blocks(int n);
size_t top_tiles(int n);
size_t top_pairs(int n);  // CTAs of one product: tile pairs of a block column
size_t top_pair_smem(int scalar_bytes);  // dynamic shared memory of a pair's rows of T
int top_tile_resident_ctas(int scalar_bytes);  // one-tile CTAs resident at once on the device
size_t top_vec_bytes(int n, int scalar_bytes);
cudaError_t configure_dense_smem(int inv32, int inv64);
// most columns of the dense top (its T must fit the device)
constexpr int kDenseTopCols = 4096;
constexpr int kDenseTopDefault = 2048;  // the default column cap under a solve-CTA cap
constexpr int kDenseTopOwned = 4096;    // the default with an uncapped solve grid (the device is the request's)
constexpr int kTopRhs = 8;   // columns of T one CTA of the inversion forms
// ---- many poses of one mesh and constraint set (arap_batch.cu); arrays of
// (vertex, pose) pairs are vertex-major, element (k, p) at k * P + p
size_t batch_solve_smem_bytes(int max_ldx, int max_ld21, int pt);
// largest pose tile (16, 8, 4, 2, 1) the batched solves support for these
// front sizes, 0 when none fits
int batch_pose_tile(int max_ldx, int max_ld21);
// whether tiles of pt poses (1, 2, 4, 8 or 16) fit the batched solve kernels
bool batch_pose_tile_fits(int max_ldx, int max_ld21, int pt);
cudaError_t configure_batch_smem(int max_ldx, int max_ld21, int pt);
// CTAs of one persistent batched solve launch for P poses in tiles of pt
int batch_grid(const DevSym &s, int P, int pt);
void launch_bsetup(const DevSym &s, int P, const Vec4<double> *p64, const double *targets, Vec4<double> *pc64,
                   Vec4<float> *pc32, Vec4<float> *R, cudaStream_t st);
void launch_bbfixed(const DevSym &s, int P, const double *w64, const Vec4<double> *pc64, Vec4<double> *bfixed,
                    cudaStream_t st);
void launch_blocal(const DevSym &s, int P, const float *w32, const Vec4<float> *redge, const Vec4<double> *pc64,
                   Vec4<float> *R, const double *w64, const Vec4<double> *p64, cudaStream_t st);
void launch_brhs(const DevSym &s, int P, const float *w32, const Vec4<float> *redge, const Vec4<float> *R,
                 Vec4<float> *b, cudaStream_t st);
void launch_bresidual(const DevSym &s, int P, const double *w64, const double *diag64, const Vec4<double> *bfixed,
                      const Vec4<float> *b, const Vec4<double> *x, Vec4<float> *r, cudaStream_t st);
// one persistent launch of `grid` CTAs (batch_grid) over all (supernode, pose
// tile) tasks; the grid must stay fixed while the ticket counter is not reset
void launch_bsolve(const DevSym &s, int P, int pt, int grid, const float *X, const float *L21, const float *L21T,
                   Vec4<float> *sol, Vec4<float> *uvec, Vec4<double> *pc64, Vec4<float> *pc32,
                   unsigned long long *ticket, unsigned *flags, int *err, bool forward, cudaStream_t st,
                   const float *atiles, float *bftop, float *bytop, float *bws);
// the dense top's T and T^T (row-major, FP32) split into TF32 head and rest
// and laid out as the tensor-core products' A tiles (btop_atile_floats)
void launch_btop_pack(const DevSym &s, const float *Ttop, float *atiles, cudaStream_t st);
// supernode tasks of the batched sweeps (the dense top's levels excluded)
int batch_tasks(const DevSym &s);
// launches of the dense top in one forward + backward pair of batched sweeps
int batch_top_launches(const DevSym &s);
// the dense top's n x 3P right-hand sides as the products' B tiles (split,
// zero padding: clear them when allocated), its A tiles and the partial
// products of one sweep, in floats
size_t btop_matrix_floats(int n, int P);
size_t btop_atile_floats(int n);
size_t btop_workspace_floats(int n, int P);
void launch_bgather(const DevSym &s, int P, const Vec4<double> *pc64, double *out, cudaStream_t st);
// handle targets of P rigid poses (P x nc x 3, ascending constrained order)
void launch_pose_targets(int P, int nc, const int32_t *cidx, const uint8_t *handle, const double *rest,
                         const double *ctgt, const double *tabs, double *out, cudaStream_t st);

// ARAP energy of the current positions in FP64 (best rotation per vertex for
// its one-ring): energy_partials(V) doubles of scratch, the sum in out[0]
int energy_partials(int V);
void launch_energy(const DevSym &s, const double *w64, const Vec4<double> *p64, const Vec4<double> *pc64,
                   double *partial, double *out, cudaStream_t st);

// vertex normals of positions xyz (V x 3, vertex order): face normals into
// face_n (F x 3), then vertex_n (V x 3)
void launch_vertex_normals(int V, int F, const int32_t *faces, const int32_t *vf_ptr, const int32_t *vf_face,
                           const double *xyz, double *face_n, double *vertex_n, cudaStream_t st);

// deformed positions back to the original vertex order as doubles (arap.h:133-135)
void launch_gather_positions(const DevSym &s, const Vec4<double> *pc64, double *out_xyz, cudaStream_t st);
template <typename T>
void launch_gather_rotations(const DevSym &s, const Vec4<T> *R, double *out9, cudaStream_t st);

}  // namespace arapgpu

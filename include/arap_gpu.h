/*
 * arap_gpu.h -- C ABI of the GB300 ARAP deformation library (libarap_gb300.so).
 *
 * Drop-in boundary for the hot path of cheind/mesh-deform's
 * deform::AsRigidAsPossibleDeformation (inc/deform/arap.h). The header-only
 * C++ template in mesh-deform_gb300/deform/arap.h gathers the mesh adapter's
 * data into flat arrays, calls these entry points and scatters the result back
 * through the adapter. Any other host language binds the same symbols
 * (ctypes, cgo, JNI, N-API).
 *
 * Conventions: plain pointers to HOST memory unless a name ends in _device;
 * int32 indices; positions as V x 3 doubles (x,y,z per vertex); every entry
 * point returns an arap_status (0 = ARAP_OK). A context is used by one host
 * thread at a time; distinct contexts are independent.
 */
#ifndef ARAP_GPU_H
#define ARAP_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum arap_status {
    ARAP_OK = 0,
    ARAP_ERR_INVALID_ARGUMENT = 1, /* null pointer, negative size, bad option */
    ARAP_ERR_BAD_INDEX = 2,        /* face or constraint index outside [0, V) */
    ARAP_ERR_NOT_SPD = 3,          /* constrained Laplacian singular / not positive definite */
    ARAP_ERR_OUT_OF_MEMORY = 4,    /* device allocation failed */
    ARAP_ERR_CUDA = 5,             /* CUDA runtime error (message in arap_last_error) */
    ARAP_ERR_TIMEOUT = 6,          /* a bounded in-kernel wait expired */
    ARAP_ERR_ADMISSION_REFUSED = 7,/* request does not fit the device memory budget */
    ARAP_ERR_NO_DEVICE = 8,        /* no CUDA device visible */
    ARAP_ERR_UNSUPPORTED = 9,      /* input outside the implemented limits */
    ARAP_PENDING = 10              /* (arap_srv_poll / arap_srv_wait) not finished yet */
} arap_status;

typedef enum arap_precision {
    /* Everything in FP64 on the GPU: cotan weights, local step, RHS, Cholesky
       factor, triangular solves. Matches the FP64 CPU path to <= 1e-10 of the
       bounding-box diagonal. */
    ARAP_PRECISION_FP64 = 0,
    /* FP32 local step, RHS and triangular solves; the Cholesky factor is
       computed in FP64 and rounded to FP32 for the solves
       (arap_set_factor_precision); every solve corrects the positions from
       the global system's residual taken in FP64, 1 + refine_steps such
       refinement solves per iteration. */
    ARAP_PRECISION_MIXED = 1
} arap_precision;

/* Fill-reducing ordering of the free vertices (arap_set_ordering). */
typedef enum arap_ordering {
    /* nested dissection of each constraint set's free vertices (default) */
    ARAP_ORDER_PER_CONSTRAINT_SET = 0,
    /* the mesh's own nested dissection (computed once per mesh and shared by
       contexts made with arap_create_like) restricted to the free vertices:
       cheaper for a new constraint set, the factor may hold more fill */
    ARAP_ORDER_MESH = 1
} arap_ordering;

typedef struct arap_ctx arap_ctx;

/* Human-readable name of a status code. */
const char *arap_status_string(int status);
/* Message of the last error raised on ctx (or of the last failed arap_create
   when ctx is NULL). Valid until the next call on the same context. */
const char *arap_last_error(const arap_ctx *ctx);

/* Replaces AsRigidAsPossibleDeformation(Mesh &mesh) and initializeMeshTopology
   (inc/deform/arap.h:66-70,149-155): copies the triangle list (3*n_faces ints,
   counter-clockwise) and builds the vertex adjacency once. device = CUDA
   ordinal. */
int arap_create(int32_t n_vertices, int32_t n_faces, const int32_t *faces, int32_t device,
                arap_ctx **out);
void arap_destroy(arap_ctx *ctx);
/* A new context for the same mesh as src (same device, topology, precision
   and rest positions, copied on the device; no constraints): skips the
   adjacency build of arap_create. src is only read. */
int arap_create_like(const arap_ctx *src, arap_ctx **out);

/* Precision form and number of FP64-residual refinement solves per iteration
   (MIXED only; 0..8). The default is ARAP_PRECISION_FP64. Marks the context
   dirty. */
int arap_set_precision(arap_ctx *ctx, int32_t precision, int32_t refine_steps);

/* Numeric factorisation of the MIXED form: bits = 64 (the default) factors
   the constrained Laplacian in FP64, as SimplicialLDLT<SparseMatrix<double>>
   does (arap.h:337,462), rounds the factor to FP32 and forms from it, in
   FP32, the inverted blocks the FP32 triangular solves multiply by; bits = 32
   factors in FP32 (cheaper set-up; the FP64 residual refinement still
   carries the accuracy). The FP64 form always factors in FP64. Marks the
   context dirty. */
int arap_set_factor_precision(arap_ctx *ctx, int32_t bits);

/* Replaces initializeMeshGeometry (arap.h:162-168): the rest pose _p, read
   from the mesh on every dirty deform. 3*V doubles. Marks the context dirty. */
int arap_set_rest_positions(arap_ctx *ctx, const double *xyz);

/* Replaces the constraint map filled by setConstraint (arap.h:81-85,443,458):
   the complete set of constrained vertices and their target locations
   (3*n doubles). A vertex listed twice keeps its last target, as a map
   overwrite does. n = 0 clears the set. Marks the context dirty. */
int arap_set_constraints(arap_ctx *ctx, int32_t n, const int32_t *indices, const double *xyz);

/* Replaces deform(numberOfIterations) (arap.h:101-138). When the context is
   dirty it first rebuilds the problem from the rest pose and the constraints
   (cotan weights arap.h:182-239, rotations reset arap.h:246-249, free-variable
   map arap.h:261-272, constraint snap arap.h:277-281, constrained Laplacian
   and its Cholesky factor arap.h:292-340); then it runs the local/global
   iterations (arap.h:122-129) and, when out_xyz is not NULL, copies the
   deformed positions (3*V doubles, all vertices) to it (arap.h:133-135).
   As in the reference, with no constrained vertex it computes the weights,
   leaves the context dirty, does not touch out_xyz and returns ARAP_OK.
   A singular constrained Laplacian (a free vertex without faces, or a mesh
   component without a constrained vertex) returns ARAP_ERR_NOT_SPD, where
   the reference's deform returns false. */
int arap_deform(arap_ctx *ctx, int32_t iterations, double *out_xyz);

/* Many handle poses of one mesh and one constrained-vertex set in one pass,
   the pattern of DeformationUtil::updateConstraints
   (inc/deform/deformation_util.h:48-57), where every pose moves the same
   handles. For each pose p: a dirty deform from the rest pose with the
   constrained vertices at targets[p], `iterations` local/global iterations
   (arap.h:102-129). targets: n_poses x n_constrained x 3 doubles, the
   constrained vertices (as given to arap_set_constraints) in ascending vertex
   order; NULL reuses the targets of the previous call, already on the device.
   All poses share the cotan weights and the Cholesky factor of the current
   rest pose and constraint set; the constraint targets given to
   arap_set_constraints are not used. MIXED precision only. out_xyz:
   n_poses x V x 3 doubles (NULL keeps the result on the device). */
int arap_deform_poses(arap_ctx *ctx, int32_t n_poses, const double *targets, int32_t iterations,
                      double *out_xyz);

/* DeformationUtil::updateConstraints (inc/deform/deformation_util.h:48-57) for
   n_poses rigid poses at once, computed on the device into the targets
   arap_deform_poses(ctx, n_poses, NULL, ...) then uses. For pose p and
   constrained vertex v (ascending order): a handle (listed in handles, which
   must all be constrained) goes to tabs_p * rest(v) with
   tabs_p = origin * transforms[p] * origin^-1 (the inverse taken as an
   isometry's, as Transform::inverse(Eigen::Isometry)); any other constrained
   vertex keeps its arap_set_constraints target. origin and each transform are
   row-major 3x4 affine matrices (12 doubles; origin NULL: identity). Uploads
   12 doubles per pose instead of 3 per constrained vertex and pose. */
int arap_pose_targets(arap_ctx *ctx, int32_t n_handles, const int32_t *handles, const double *origin,
                      int32_t n_poses, const double *transforms);

/* arap_deform split in two: arap_deform_async enqueues the whole deform on
   the context's stream and returns at once (out_xyz must stay valid, and is
   best pinned, until arap_wait returns); arap_wait waits for it and returns
   its status. Any other call on the context first waits for a pending
   deform. Contexts on one device run concurrently, so one host thread can
   keep several requests in flight. Each context has its own stream; with more
   contexts in flight than CUDA's hardware queues (CUDA_DEVICE_MAX_CONNECTIONS,
   8 unless set), streams share queues and wait on each other, so set it (to
   32) in the environment before the process's first CUDA call. */
int arap_deform_async(arap_ctx *ctx, int32_t iterations, double *out_xyz);
int arap_wait(arap_ctx *ctx);
/* arap_deform_poses split the same way (completed by arap_wait or
   arap_query). */
int arap_deform_poses_async(arap_ctx *ctx, int32_t n_poses, const double *targets, int32_t iterations,
                            double *out_xyz);
/* Completion notification: fn(user) is called on a CUDA runtime thread once
   each later asynchronous deform has finished on the device (its results
   copied). fn must return quickly and call neither CUDA nor arap_*; the
   caller then collects the status with arap_wait or arap_query. NULL removes
   it. */
typedef void (*arap_done_fn)(void *user);
int arap_set_done_callback(arap_ctx *ctx, arap_done_fn fn, void *user);

/* Non-blocking completion check of a pending asynchronous deform: *done = 0
   while it runs (returns ARAP_OK); otherwise *done = 1 and the return value
   is what arap_wait returns. */
int arap_query(arap_ctx *ctx, int32_t *done);

/* Most CTAs one triangular-solve launch uses (0, the default: as many as fit
   on the device). Each CTA works through the supernodes in schedule order, so
   any count gives the same result; a smaller count leaves room for the
   launches of other contexts running at the same time. With 0 the context
   assumes it owns the device: its sweeps and dense-top products start while
   the kernel before them finishes (programmatic dependent launch); with a cap
   every launch waits for the previous one as usual. Takes effect at the next
   deform (which sets the problem up again). */
int arap_set_solve_ctas(arap_ctx *ctx, int32_t max_ctas);

/* Poses per task of the batched triangular solves of arap_deform_poses: 1, 2,
   4, 8 or 16 (0, the default: the largest the mesh's biggest supernode
   allows). A larger tile streams each factor block once for more poses; a
   smaller one gives more tasks to run at once. Any value gives the same
   result. ARAP_ERR_UNSUPPORTED at the next arap_deform_poses when the tile
   does not fit; ARAP_ERR_INVALID_ARGUMENT for other values. */
int arap_set_pose_tile(arap_ctx *ctx, int32_t poses);

/* The triangular solves take the top levels of the elimination tree (large
   fronts, one or a few supernodes per level) with clusters of 8 CTAs that
   split each supernode's matrices, and the levels below with one CTA per
   supernode. A level goes to the clusters when one of its supernodes holds at
   least `bytes` of X = inv(L11) and L21 (as FP32) and every level above it does
   too. 0 (the default): 128 KiB; negative: no cluster levels. The split changes
   only the order of some sums. Takes effect at the next deform (which sets the
   problem up again). */
int arap_set_cluster_threshold(arap_ctx *ctx, int32_t bytes);

/* The bottom levels of the elimination tree whose supernode fronts all have
   at most `rows` rows (0, the default: none; at most 256) are solved one warp
   per supernode, many supernodes per CTA, before the CTA-per-supernode sweep
   of the levels above (after it, backward). Any value gives a correct
   result; it changes the order of some sums. Takes effect at the next deform
   (which sets the problem up again). On the measured meshes a warp's task
   takes longer than a CTA's, so the default leaves it off. */
int arap_set_warp_rows(arap_ctx *ctx, int32_t rows);

/* Schedule of the CTA-per-supernode levels of a single request's triangular
   solves (arap.h:417-429). ARAP_SOLVE_PERSISTENT: one launch of persistent
   CTAs per sweep that take supernodes in dependency order and wait (bounded)
   for their children's or parent's completion flags. ARAP_SOLVE_LEVELS: one
   launch per level of the elimination tree, sized to the level, in which no
   task waits; CTAs only occupy SMs while they have work, so concurrent
   requests share the device better. Trees of more than 48 levels keep the
   persistent schedule. Both give identical results. Takes effect at the next
   deform (which sets the problem up again). */
/* Launch shape of a per-vertex kernel of a single request's iterations:
   kernel = ARAP_K_LOCAL (covariance + rotation fit, arap.h:354-384), ARAP_K_RHS
   (arap.h:395-414) or ARAP_K_RESIDUAL (the FP64 residual of the mixed form).
   threads_per_vertex = 1, 2, 4, 8 or 32 lanes of one warp per vertex, which
   split the vertex's adjacency entries and sum by shuffles (32: a warp per
   vertex); block_threads a multiple of 32, at most 256 for ARAP_K_LOCAL and
   1024 for the others. Default 1 and 256 for all three. Any shape gives the
   same result up to the order of sums. The batched kernels of
   arap_deform_poses take one thread per (vertex, pose) and keep their shape.
   mesh-deform_gb300/arap_tune.py measures the best shape per kernel. */
int arap_set_vertex_launch(arap_ctx *ctx, int32_t kernel, int32_t threads_per_vertex, int32_t block_threads);

/* Solve blocks of a single request's triangular sweeps (arap.h:417-429):
   every supernode of level 1 of the elimination tree is solved together with
   its leaf children as one task, through the dense inverse of the subtree's
   diagonal block (formed once per factorisation) and the subtree's rows
   below, when every such subtree has at most `max_columns` columns (default
   512; 0: none; at most 1,024). Half the tasks of a sweep and one level less on its chain,
   for more bytes per task. Results equal up to the order of sums. Takes
   effect at the next deform (which analyses the problem again). */
int arap_set_solve_blocks(arap_ctx *ctx, int32_t max_columns);

#define ARAP_SOLVE_PERSISTENT 0
#define ARAP_SOLVE_LEVELS 1
int arap_set_solve_schedule(arap_ctx *ctx, int32_t schedule);

/* The top levels of the elimination tree, up to `max_columns` columns in all
   (0, the default: 4,096 when the solve grid is uncapped, i.e. the request
   owns the device, and 2,048 under an arap_set_solve_ctas cap, where the
   wider product's SM time competes with other requests; at most 4,096;
   negative: none), are solved through the explicit
   inverse of the factor restricted to them: formed once per factorisation
   (n x n dense), it turns the top of each triangular sweep, a chain of
   single-supernode steps, into one wide matrix-vector product (in
   arap_deform_poses: one matrix product over all poses). Takes effect at the
   next deform (which sets the problem up again); it changes the order of
   sums. */
int arap_set_dense_top(arap_ctx *ctx, int32_t max_columns);

/* arap_ordering of the next symbolic analysis (marks the context dirty). */
int arap_set_ordering(arap_ctx *ctx, int32_t mode);

/* Failure detection: the most polls a triangular-solve task makes while it
   waits for another task's completion flag (0, the default: 2^24 polls of
   20-200 ns, a few seconds). When a wait runs out, the kernel records it,
   every CTA of the launch leaves at its next task, the rest of the deform's
   solve launches leave at once, and arap_wait (arap_deform) returns
   ARAP_ERR_TIMEOUT; the context rebuilds its scheduling state, so the next
   deform is correct. Waits of a CTA for its own bulk copies are not limited
   by this value. No counterpart in the reference (whose solves are
   sequential). */
int arap_set_wait_limit(arap_ctx *ctx, int32_t polls);

/* enable != 0 (the default) keeps the symbolic analysis (ordering,
   elimination tree, supernodes, factorisation plan) of a constrained-vertex
   set for later dirty deforms of the same set, which then only refactor
   numerically. 0 redoes and re-uploads it on every dirty deform, as the
   reference's SimplicialLDLT::compute (arap.h:337) analyses the pattern on
   every call; the CUDA graphs are then captured anew too. */
int arap_set_symbolic_cache(arap_ctx *ctx, int32_t enable);

/* enable != 0 (the default) runs the setup and the iteration sequence as CUDA
   graphs captured on first use and replayed while the problem's size,
   precision and iteration count stay the same; 0 launches every kernel
   directly. Profiling (arap_set_profiling) always launches directly. */
int arap_set_graphs(arap_ctx *ctx, int32_t enable);

/* New targets for the SAME constrained vertices (3*n doubles, n = the number
   of vertices of the last arap_set_constraints, in ascending vertex order).
   Unlike arap_set_constraints it keeps the rest pose, the cotan weights and
   the Cholesky factor: the next arap_deform starts from the rest pose with
   the constrained vertices at the new targets and rotations reset, as a dirty
   deform of the reference would on an unchanged rest pose, without the
   factorisation (an extension: the reference always refactors after
   setConstraint). */
int arap_set_targets(arap_ctx *ctx, int32_t n, const double *xyz);

/* ARAP energy of the current positions, in FP64 on the device:
   sum_i sum_j w_ij |(p'_i - p'_j) - R_i (p_i - p_j)|^2 over every adjacency
   entry (cotan weights of arap.h:182-239, rest pose p, current positions p'),
   with R_i the rotation the local step (arap.h:354-384) fits to vertex i's
   one-ring for the current positions (not stored). The quantity the
   local/global iteration decreases; the reference does not compute it. */
int arap_energy(arap_ctx *ctx, double *energy);

/* Host time of the last arap_deform_async, in ms, by phase: symbolic
   analysis and its upload, device allocation, set-up enqueue, iteration
   enqueue, the rest (gather, copies). The phases of a non-dirty deform are 0
   but for the last two; after an arap_deform_poses_async all five are 0. */
int arap_get_host_timing(arap_ctx *ctx, double *ms5);

/* Vertex normals of the current deformed positions, computed on the device
   as OpenMesh's update_normals does before display
   (examples/osg_viewer.cpp:53,60-62): face normal = normalised
   (p1 - p0) x (p2 - p0), vertex normal = normalised sum of the normals of its
   faces. normals_xyz: V x 3 doubles (host). */
int arap_vertex_normals(arap_ctx *ctx, double *normals_xyz);

/* The current deformed positions (and, with_normals != 0, their vertex
   normals) in vertex order, V x 3 doubles each, left in device memory owned
   by the context: the pointers stay valid until the next call on the context.
   For consumers on the same device (rendering, further kernels) that need no
   host copy. Ready when the call returns. */
int arap_device_positions(arap_ctx *ctx, int32_t with_normals, const double **positions_device,
                          const double **normals_device);

/* Device memory held by the context, in bytes. */
int64_t arap_device_bytes(const arap_ctx *ctx);
/* Device memory the context will hold after its next arap_deform
   (n_poses = 0) or arap_deform_poses with n_poses poses, in bytes. Runs the
   host-side symbolic analysis of the current constraint set if it has not
   run yet (kept for the deform); launches nothing and allocates nothing on
   the device. */
int arap_plan_bytes(arap_ctx *ctx, int32_t n_poses, int64_t *bytes);

/* Marks the context dirty without uploading anything: the next arap_deform
   rebuilds the problem from the rest pose and targets already on the device.
   Used to time a dirty deform with its inputs resident in device memory. */
int arap_invalidate(arap_ctx *ctx);

/* Current positions _pprime (3*V doubles). */
int arap_get_positions(arap_ctx *ctx, double *out_xyz);

/* _edgeWeights as CSR over all vertices (tests/accessor.h:19-21 exposes it
   through PrivateAccessor). rowptr: V+1, col/val: nnz entries. */
int arap_edge_weights_nnz(arap_ctx *ctx, int32_t *nnz);
int arap_get_edge_weights(arap_ctx *ctx, int32_t *rowptr, int32_t *col, double *val);

/* _rotations of the last local step (arap.h:382), V x 9 row-major doubles. */
int arap_get_rotations(arap_ctx *ctx, double *R9);

/* Symbolic analysis of the constrained Laplacian built by the last dirty
   deform: m free vertices, perm[k] = free index (rank among free vertices in
   ascending vertex order) eliminated k-th, etree of the permuted matrix, and
   the supernode partition block_ptr (n_blocks+1 entries). Any pointer may be
   NULL. */
int arap_get_symbolic_sizes(arap_ctx *ctx, int32_t *n_free, int32_t *n_blocks, int64_t *factor_nnz);
int arap_get_symbolic(arap_ctx *ctx, int32_t *perm, int32_t *etree, int32_t *block_ptr);

/* Host-only symbolic analysis, no device needed: the same ordering, elimination
   tree and supernode partition arap_deform builds for this mesh and
   constrained-vertex set (the symbolic half of SimplicialLDLT::compute,
   arap.h:337, over the pattern of setupLinearSystem, arap.h:292-336).
   perm and etree need V entries, block_ptr V+1. Returns ARAP_ERR_NOT_SPD when
   a free mesh component has no constrained vertex. */
int arap_analyze_pattern(int32_t n_vertices, int32_t n_faces, const int32_t *faces, int32_t n_constrained,
                         const int32_t *constrained, int32_t *n_free, int32_t *n_blocks, int64_t *factor_nnz,
                         int32_t *perm, int32_t *etree, int32_t *block_ptr);

/* Timing of the last arap_deform in milliseconds (device events): setup
   (weights, assembly, factor) and iterations. */
int arap_get_timing(arap_ctx *ctx, double *setup_ms, double *iterations_ms);

/* Number of kernel launches issued by the last arap_deform. */
int arap_get_launch_count(arap_ctx *ctx, int64_t *launches);

/* The CUDA stream (cudaStream_t) every kernel of this context runs on, so a
   caller can order its own work or record events on it. */
int arap_get_stream(arap_ctx *ctx, void **stream);

/* Kernel classes timed by the optional per-launch profiler. */
typedef enum arap_kernel_class {
    ARAP_K_WEIGHTS = 0,   /* cotan weights (face cotangents + edge sums) */
    ARAP_K_ASSEMBLE = 1,  /* vertex setup + Laplacian/bFixed assembly */
    ARAP_K_FACTOR = 2,    /* multifrontal Cholesky levels */
    ARAP_K_LOCAL = 3,     /* local step: covariance + rotation fit */
    ARAP_K_RHS = 4,       /* right-hand side assembly */
    ARAP_K_RESIDUAL = 5,  /* FP64 residual of the global system */
    ARAP_K_SOLVE_FWD = 6, /* forward supernodal triangular solve */
    ARAP_K_SOLVE_BWD = 7, /* backward supernodal triangular solve */
    ARAP_K_GATHER = 8,    /* positions back to vertex order */
    ARAP_K_NUM_CLASSES = 9
} arap_kernel_class;

/* enable != 0 brackets every launch with CUDA events on the context's stream
   and accumulates the device time per kernel class until reset. */
int arap_set_profiling(arap_ctx *ctx, int32_t enable);
int arap_reset_kernel_stats(arap_ctx *ctx);
int arap_get_kernel_stats(arap_ctx *ctx, int32_t kernel_class, double *total_ms, int64_t *launches);

/* Algorithmic DRAM bytes and flops of ONE launch of a kernel class for the
   current problem and precision (the minimum traffic: every input read once,
   every output written once, unpadded 3-vectors; for FACTOR the sum over all
   of its level launches). Used for roofline fractions. */
int arap_get_kernel_model(arap_ctx *ctx, int32_t kernel_class, double *bytes, double *flops);

/* Cotan edge weights (the values of _edgeWeights, inc/deform/arap.h:182-239)
   for callers that cannot allocate device memory when they need them: a
   per-frame callback of an interactive viewer must not stall the device on
   cudaMalloc, and a host application that manages all device memory through
   its own pool forbids driver allocations. This entry point has no counterpart
   in the reference. It allocates nothing: its only scratch, three doubles per
   face, is a file-scope __device__ array of at most 524,288 faces (12 MiB,
   held on every device that loads the library until the process exits).
   All pointers are DEVICE pointers owned by the caller: faces (3*n_faces),
   xyz (3*n_vertices doubles), the weight pattern rowptr (n_vertices+1) / col
   (nnz, columns sorted in each row, every mesh edge present in both
   directions -- the pattern arap_get_edge_weights returns), and the output
   val (nnz doubles, overwritten). The kernels run on `stream` (a
   cudaStream_t; NULL = default stream) of the calling thread's current
   device and the call returns without waiting for them. The first call on a
   device looks up the scratch array's device address, which under CUDA's
   default lazy module loading also loads the library's device code on that
   device: a one-time driver allocation of the 12 MiB array that may
   synchronise the device. Make that first call at start-up, before any stream
   capture and before the callbacks that must not stall; later calls allocate
   nothing. All calls on one device share the scratch array, which keeps the
   last call's contents: calls whose kernels overlap on the GPU race and must
   be ordered by the caller. More than 524,288 faces returns
   ARAP_ERR_UNSUPPORTED. The device-resident inputs are checked by the
   kernels: a face with an index outside [0, n_vertices) is skipped (it adds
   nothing) and an edge missing from the pattern adds nothing; both are
   counted for arap_cotan_weights_static_status, and no kernel reads outside
   the given arrays. A face whose corners repeat a vertex adds both halves of
   that edge to the diagonal entry (the reference's two (a, a) triplets) when
   the pattern holds it. Values equal arap_get_edge_weights bit for bit when no
   entry receives more than two contributions (every edge on at most two
   faces, no diagonal shared by two degenerate corners); otherwise the
   additions' order, and so the last bit, may differ. */
int arap_cotan_weights_static(int32_t n_vertices, int32_t n_faces, const int32_t *faces, const double *xyz,
                              const int32_t *rowptr, const int32_t *col, int32_t nnz, double *val, void *stream);
/* Input-check result of the last arap_cotan_weights_static on the current
   device: waits for `stream` (the stream that call used), stores in *skipped
   (may be NULL) the number of faces it skipped for an out-of-range index plus
   the edges it found missing from the pattern, and returns ARAP_ERR_BAD_INDEX
   when that number is not zero, else ARAP_OK. Allocates nothing. */
int arap_cotan_weights_static_status(void *stream, int32_t *skipped);

/* ------------------------------------------------------------------------
   Deform server: a request loop over resident contexts (no counterpart in the
   reference, whose deform() is a synchronous call on one object).

   Requests (mesh, constraint set with targets, iteration count) are queued as
   they arrive. One context per (mesh, constraint set) stays resident on the
   device with its cotan weights and Cholesky factor; a request whose
   constraint set is resident re-poses it (arap_set_targets) instead of
   refactoring. New constraint sets are analysed on host worker threads and
   admitted when their planned device footprint fits the budget, evicting
   the least recently used idle contexts. Requests of one resident constraint
   set with the same iteration count that wait together run as one
   multi-pose launch (arap_deform_poses, MIXED precision). Up to
   max_in_flight launches run concurrently on their own streams. Each result
   equals that of a lone arap_deform of the same request on a fresh context,
   within the precision form's tolerance. Thread-safe. */
typedef struct arap_server arap_server;

typedef struct arap_server_config {
    int32_t device;
    int32_t precision;           /* arap_precision of every request (ARAP_PRECISION_MIXED) */
    int32_t refine_steps;        /* MIXED refinement solves per iteration (1) */
    int32_t max_in_flight;       /* launches on the device at once (0: 8; beyond that the measured
                                    serving stream got no faster) */
    int64_t device_budget_bytes; /* resident device memory limit (0: 80% of the free memory) */
    int32_t prep_threads;        /* host threads for analysis and first launches (0: 4) */
    int32_t max_batch;           /* most requests per multi-pose launch (0: 64; 1: no batching) */
    int32_t max_queue;           /* waiting requests before submit refuses (0: 65536) */
    int32_t poll_us;             /* completion polling interval of the scheduler (0: 20) */
    int32_t solve_ctas;          /* arap_set_solve_ctas of every context (0: as many as fit) */
    int32_t per_set_ordering;    /* 1: ARAP_ORDER_PER_CONSTRAINT_SET; 0 (default): ARAP_ORDER_MESH */
} arap_server_config;

typedef struct arap_request {
    int32_t mesh;             /* id from arap_srv_add_mesh */
    int32_t n_constraints;
    const int32_t *indices;   /* copied by submit; a vertex listed twice keeps its last target */
    const double *targets;    /* 3 per constraint, copied by submit */
    int32_t iterations;
    int32_t pad;
    double *out_xyz;          /* V x 3, written before the request completes; must stay valid until then */
} arap_request;

typedef struct arap_request_info {
    int32_t status;           /* ARAP_OK or the error of this request */
    int32_t factor_reused;    /* 1: served by a resident factor of the same constraint set */
    int32_t batch_size;       /* requests in the launch that served it */
    int32_t pad;
    double queue_ms;          /* submit -> launch */
    double latency_ms;        /* submit -> result in out_xyz */
} arap_request_info;

typedef struct arap_server_stats {
    int64_t submitted, completed, failed, refused;
    int64_t factor_hits, factor_misses, evictions, launches, batched_launches, batched_requests;
    int64_t iterations_done;  /* iterations of completed requests */
    int64_t resident_bytes, peak_resident_bytes, budget_bytes;
    int32_t resident_factors, queue_depth, in_flight, pad;
    double scheduler_busy_ms;  /* scheduler thread time outside its waits */
    double worker_busy_ms;     /* prep-thread time in analyses and first launches */
    double analyze_ms;         /* of which: contexts created, constraint sets analysed */
    double staging_ms;         /* scheduler time allocating pinned result buffers */
    double device_ms;          /* sum over launches of their device time (set-up + iterations) */
    double launch_ms;          /* host time in the launch calls (arap_deform[_poses]_async and the
                                  re-pose before it) */
    double launch_host_ms[5];  /* of which, summed arap_get_host_timing phases: analysis and uploads,
                                  allocation, set-up enqueue, iteration enqueue, rest */
} arap_server_stats;

int arap_srv_create(const arap_server_config *cfg, arap_server **out);
/* Finishes every submitted request, then frees everything. */
void arap_srv_destroy(arap_server *srv);
/* Registers a mesh (faces and rest positions are copied; one context holds
   its topology on the device). */
int arap_srv_add_mesh(arap_server *srv, int32_t n_vertices, int32_t n_faces, const int32_t *faces,
                      const double *rest_xyz, int32_t *mesh_id);
/* Queues a request; ARAP_ERR_BAD_INDEX / INVALID_ARGUMENT for malformed ones,
   ARAP_ERR_ADMISSION_REFUSED when max_queue requests already wait. */
int arap_srv_submit(arap_server *srv, const arap_request *req, int64_t *ticket);
/* ARAP_PENDING while the request runs; otherwise its final status, with info
   filled in (when non-NULL) and the ticket released. */
int arap_srv_poll(arap_server *srv, int64_t ticket, arap_request_info *info);
/* As arap_srv_poll, waiting up to timeout_ms (negative: no limit). */
int arap_srv_wait(arap_server *srv, int64_t ticket, int32_t timeout_ms, arap_request_info *info);
int arap_srv_stats(arap_server *srv, arap_server_stats *stats);
/* Message of the last failed arap_srv_* call on this server. */
const char *arap_srv_last_error(const arap_server *srv);

#ifdef __cplusplus
}
#endif
#endif

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
    ARAP_ERR_UNSUPPORTED = 9       /* input outside the implemented limits */
} arap_status;

typedef enum arap_precision {
    /* Everything in FP64 on the GPU: cotan weights, local step, RHS, Cholesky
       factor, triangular solves. Matches the FP64 CPU path to <= 1e-10 of the
       bounding-box diagonal. */
    ARAP_PRECISION_FP64 = 0,
    /* FP32 local step, RHS and triangular solves on an FP32 Cholesky factor;
       the global system's residual is taken in FP64 and refined
       (refine_steps extra solves per iteration). */
    ARAP_PRECISION_MIXED = 1
} arap_precision;

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

/* Precision form and number of FP64-residual refinement solves per iteration
   (MIXED only; 0..8). The default is ARAP_PRECISION_FP64. Marks the context
   dirty. */
int arap_set_precision(arap_ctx *ctx, int32_t precision, int32_t refine_steps);

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

/* arap_deform split in two: arap_deform_async enqueues the whole deform on
   the context's stream and returns at once (out_xyz must stay valid, and is
   best pinned, until arap_wait returns); arap_wait waits for it and returns
   its status. Any other call on the context first waits for a pending
   deform. Contexts on one device run concurrently, so one host thread can
   keep several requests in flight. */
int arap_deform_async(arap_ctx *ctx, int32_t iterations, double *out_xyz);
int arap_wait(arap_ctx *ctx);

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

/* Device memory held by the context, in bytes. */
int64_t arap_device_bytes(const arap_ctx *ctx);

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
   device looks up the scratch array's device address; make that first call
   before any stream capture. All calls on one device share the scratch array,
   which keeps the last call's contents: calls whose kernels overlap on the GPU
   race and must be ordered by the caller. More than 524,288 faces returns
   ARAP_ERR_UNSUPPORTED. Values equal arap_get_edge_weights bit for bit when
   every edge lies on at most two faces. */
int arap_cotan_weights_static(int32_t n_vertices, int32_t n_faces, const int32_t *faces, const double *xyz,
                              const int32_t *rowptr, const int32_t *col, int32_t nnz, double *val, void *stream);

#ifdef __cplusplus
}
#endif
#endif

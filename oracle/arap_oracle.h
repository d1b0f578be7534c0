/*
 * arap_oracle.h -- FP64 CPU restatement of the ARAP hot path of cheind/mesh-deform.
 *
 * TEST INFRASTRUCTURE ONLY. This is the oracle the CUDA path is checked against
 * and the CPU baseline the benchmark times beside it. Nothing in the product
 * (the CUDA library, the drop-in header) includes, links or calls it.
 *
 * Parity status: the cotan weights are pinned by the reference's own known-answer
 * test (tests/test_cotan.cpp:26-53, reproduced in tests/golden/). The reference
 * cannot be compiled here (it needs Eigen, which is absent), so rotations, RHS,
 * solves and end-to-end positions are pinned only by this restatement, by an
 * independent numpy/scipy restatement (tests/np_arap.py) and by exact-answer
 * properties of ARAP (rigid motions, deform(0)) -- end-to-end parity is
 * therefore "parity unpinned" against the reference binary itself.
 *
 * The handle mirrors deform::AsRigidAsPossibleDeformation<Mesh, double>
 * (inc/deform/arap.h:49-466): it owns a copy of the mesh positions (the adapter's
 * vertexLocation get/set, inc/deform/openmesh_adapter.h:74-83), a constraint map
 * with overwrite semantics (arap.h:81-85,443,458) and a dirty flag (arap.h:464).
 */
#ifndef ARAP_ORACLE_H
#define ARAP_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_arap oracle_arap;

/* Construction: arap.h:66-70 (stores the faces, initializeMeshTopology arap.h:149-155).
   positions: 3*V doubles, the mesh's current vertex locations. */
oracle_arap *oa_create(int n_vertices, int n_faces, const int *faces, const double *positions);
void oa_destroy(oracle_arap *oa);

/* Overwrite the mesh's vertex locations (what a caller does through the adapter). */
void oa_set_mesh_positions(oracle_arap *oa, const double *xyz);
/* Read the mesh's vertex locations (written back by oa_deform, arap.h:133-135). */
void oa_get_mesh_positions(const oracle_arap *oa, double *xyz);

/* setConstraint, arap.h:81-85. Returns 0, or -1 for an index outside [0, V). */
int oa_set_constraint(oracle_arap *oa, int vidx, double x, double y, double z);

/* deform, arap.h:101-138. Returns 1 on success, 0 when the factorisation fails
   (SimplicialLDLT::info() != Success, arap.h:116-117,339). */
int oa_deform(oracle_arap *oa, int iterations);

/* Introspection for tests (the reference exposes _edgeWeights through
   PrivateAccessor, tests/accessor.h:19-21). */
int oa_num_free(const oracle_arap *oa);
int oa_weights_nnz(const oracle_arap *oa);
void oa_get_weights(const oracle_arap *oa, int *rowptr, int *col, double *val);
void oa_get_rotations(const oracle_arap *oa, double *R9);      /* V x 9, row-major */
void oa_get_free_map(const oracle_arap *oa, int *free_idx);     /* V */
void oa_get_bfixed(const oracle_arap *oa, double *b);           /* m x 3 */
/* Symbolic analysis of the constrained Laplacian (over free indices):
   perm[k] = free index eliminated k-th; parent = elimination tree of the
   permuted matrix; blocks = supernode partition of the elimination order
   (block_ptr has n_blocks+1 entries). */
void oa_get_ordering(const oracle_arap *oa, int *perm);
void oa_get_etree(const oracle_arap *oa, int *parent);
int oa_num_blocks(const oracle_arap *oa);
void oa_get_blocks(const oracle_arap *oa, int *block_ptr);
long long oa_factor_nnz(const oracle_arap *oa);
/* ARAP energy of the current positions with the best rotation per vertex. */
double oa_energy(const oracle_arap *oa);

/* Pure helpers. */
void oa_rotation_from_covariance(const double *cov9, double *R9);
/* Nested-dissection ordering of an arbitrary graph given as CSR (n vertices,
   symmetric pattern, no self loops). perm: n, block_ptr: n+1 capacity.
   Returns the number of blocks. */
int oa_nd_order(int n, const int *rowptr, const int *col, int *perm, int *block_ptr);

#ifdef __cplusplus
}
#endif
#endif

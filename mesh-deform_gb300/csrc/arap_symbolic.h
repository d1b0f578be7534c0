// arap_symbolic.h -- host-side symbolic analysis for the GPU ARAP solver.
//
// Everything here is integer work done once per mesh (adjacency) or once per
// constrained-vertex set (ordering, elimination tree, supernodes, assembly
// maps). It is deterministic: the same mesh and constraint set give the same
// arrays on every machine.
#pragma once

#include <cstdint>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

namespace arapgpu {

// Nested-dissection parameters (must match the oracle's ND_LEAF / ND_BAL_*).
constexpr int kNdLeaf = 64;
constexpr int kNdBalNum = 4;
constexpr int kNdBalDen = 10;
constexpr int kNdPseudoPeripheralRounds = 8;

// Block width of the dense diagonal blocks inside a supernode.
constexpr int kDiagBlock = 32;

// Vertex adjacency of a triangle mesh: the sparsity pattern of _edgeWeights
// (inc/deform/arap.h:224-238), sorted columns, one entry per undirected edge
// direction (a face whose corners repeat contributes a self entry, as in the
// reference). For every CSR entry, the faces that contribute to its weight, in
// face order (setFromTriplets sums duplicates in insertion order).
// Nested dissection of the whole mesh (constrained vertices included), made
// once on first use and shared by every context of the mesh (copies of a
// Topology share it).
struct MeshOrder {
    std::mutex mu;
    bool ready = false;
    std::vector<int32_t> perm;       // V: vertex eliminated k-th
    std::vector<int32_t> block_ptr;  // blocks of the dissection
};

struct Topology {
    int V = 0, F = 0;
    std::shared_ptr<MeshOrder> mesh_order = std::make_shared<MeshOrder>();
    std::vector<int32_t> faces;      // 3F
    std::vector<int32_t> rowptr;     // V+1
    std::vector<int32_t> col;        // nnz
    std::vector<int32_t> ent_ptr;    // nnz+1
    std::vector<int32_t> ent_fc;     // face*3 + k (k: which cotangent of the face)
    std::vector<int32_t> vf_ptr;     // V+1: faces around each vertex, in face order
    std::vector<int32_t> vf_face;    // 3F
    int nnz() const { return (int)col.size(); }
};

bool build_topology(int V, int F, const int32_t *faces, Topology &topo, std::string &err);

// Per-supernode description used by the kernels (plain data, copied to the device).
struct SnInfo {
    int32_t first;       // first column (device / elimination order)
    int32_t ncol;        // columns in the supernode
    int32_t nrow;        // rows of the front: ncol + |struct|
    int32_t parent;      // parent supernode or -1
    int64_t panel_off;   // nrow x ncol column-major panel in the factor array
    int64_t dinv_off;    // ceil(ncol/kDiagBlock) blocks of kDiagBlock^2 inverse diagonal blocks
    int64_t upd_off;     // nb x nb update matrix (nb = nrow - ncol)
    int64_t uvec_off;    // nb rows of the forward-solve update vectors
    int32_t rows_off;    // offset of the struct row list (nb entries, device indices)
    int32_t relind_off;  // offset of this supernode's struct positions in its parent's front
    int32_t child_begin; // children [child_begin, child_end) in the child list
    int32_t child_end;
    int32_t level;       // height in the supernodal tree (leaves = 0)
    int32_t ldx;         // leading dimension of X (ncol rounded up to 4)
    int64_t x_off;       // X = inverse of L11, ncol columns of ldx rows (lower, zero above)
    int64_t l21_off;     // L21 copy, ncol columns of ld21 rows
    int32_t ld21;        // leading dimension of L21 (nb rounded up to 4)
    int32_t pad;
    int64_t xt_off;      // X^T, ncol columns of ldx rows (upper, zero below)
    int64_t l21t_off;    // L21^T, nb columns of ldx rows
};

// One CTA's share of a factorisation launch: supernode and sub-range (meaning
// depends on the launch kind, see FactorLaunch).
struct FItem {
    int32_t sn, a, b, c;
};

// Factorisation launch plan, level by level (leaves first):
//   kFea   extend-add, item = (sn, first parent column, end parent column)
//   kFupd  left-looking update of block column jb, item = (sn, row tile)
//   kFdt   diagonal block jb: factor and invert, item = (sn)
//   kFsyrk Schur complement U -= L21 L21^T, item = (sn, row tile, column tile)
//   kFx    X = inv(L11) column block jb and the solve copies, item = (sn, jb)
//   kFrows the rows below diagonal block jb, item = (sn, row tile)
enum FactorKind { kFea = 0, kFupd = 1, kFdt = 2, kFsyrk = 3, kFx = 4, kFrows = 5 };
// Tile sizes of the plan's items: rows of a kFupd tile, rows of a kFrows
// tile, side of a kFsyrk tile
constexpr int kFactorUpdRows = 32;
constexpr int kFactorRowsTile = 64;
constexpr int kFactorSyrkTile = 32;
struct FactorLaunch {
    int32_t kind, jb, item_off, count;
};

struct Symbolic {
    int V = 0, m = 0;                 // vertices, free vertices
    std::vector<uint8_t> constrained; // V
    std::vector<int32_t> perm;        // m: free index eliminated k-th
    std::vector<int32_t> etree;       // m: elimination tree of the permuted matrix
    std::vector<int32_t> block_ptr;   // S+1: supernode partition of [0, m)
    std::vector<int32_t> newidx;      // V: vertex -> device index
    std::vector<int32_t> oldidx;      // V: device index -> vertex
    // adjacency in device order (row k = vertex oldidx[k]; entries keep the
    // original neighbour order)
    std::vector<int32_t> drow, dcol;  // V+1, nnz
    std::vector<int32_t> dent;        // nnz: original CSR entry of each device entry
    // supernodes
    int S = 0;
    std::vector<SnInfo> sn;
    std::vector<int32_t> rows;        // concatenated struct rows
    std::vector<int32_t> relind;      // concatenated positions in the parent's front
    std::vector<int32_t> child;       // concatenated children lists
    std::vector<int32_t> level_ptr;   // levels+1
    std::vector<int32_t> level_sn;    // supernodes grouped by level (leaves first)
    int max_nrow = 0, max_ncol = 0, max_children = 0, max_ldx = 0, max_ld21 = 0;
    int64_t panel_size = 0, dinv_size = 0, upd_size = 0, uvec_size = 0, x_size = 0, l21_size = 0;
    int64_t l21t_size = 0;
    int64_t factor_nnz = -1;          // nonzeros of the scalar factor (-1: not counted yet)
    double factor_flops = 0.0;        // dense flops of the supernodal factorisation
    std::vector<FItem> fitems;
    std::vector<FactorLaunch> fplan;
    // assembly maps into the factor array
    std::vector<int64_t> amap;        // per device entry: destination of -w (or -1)
    std::vector<int64_t> dmap;        // per free device row: destination of the diagonal
};

// Builds the symbolic analysis for a constrained-vertex set. Returns false and
// sets err when the free graph has a component that touches no constrained
// vertex (the constrained Laplacian is then singular).
// mesh_order: order the free vertices by the mesh's own dissection restricted
// to them (one dissection per mesh instead of one per constraint set; blocks
// left empty are dropped) instead of dissecting the free graph.
bool build_symbolic(const Topology &topo, const std::vector<uint8_t> &constrained, Symbolic &sym,
                    std::string &err, bool &singular, bool mesh_order = false);

// Solve-time amalgamation: every supernode of level 1 (whose children are all
// leaves) is solved together with its leaf children as one block, the subtree's
// columns being contiguous in the elimination order. A block keeps its node's
// index, parent, rows below, relative indices and update vector, so the rest of
// the tree sees no difference; it has no children, ncol = the subtree's
// columns, a dense X = inv(L) of the subtree and L21 = L(rows below, subtree
// columns), stored after the supernodes' solve arrays. Every level of the
// solve tree is then one below the supernodal level (uniform shift). The
// factorisation keeps the supernodal tree.
struct SolveBlocks {
    std::vector<SnInfo> sn;               // S entries: sym.sn with the blocks in place of their nodes
    std::vector<int32_t> level_ptr;       // solve levels (leaves and blocks = 0)
    std::vector<int32_t> level_sn;        // scheduled entries by level (absorbed leaves left out)
    std::vector<int32_t> items;           // per block: node, first member, end member (into members)
    std::vector<int32_t> members;         // leaf children in order, then the node
    int64_t x_size = 0, l21_size = 0, l21t_size = 0;  // solve arrays with the blocks
    int max_ldx = 0, max_ld21 = 0, max_ncol = 0, nblocks = 0;
};

// Builds the solve blocks; false (and out empty) when the tree has no level-1
// supernode or a subtree has more than max_cols columns.
bool build_solve_blocks(const Symbolic &sym, int max_cols, SolveBlocks &out);

// Nonzeros of the scalar Cholesky factor (diagonal included), counted from the
// elimination tree on first use and kept in sym.factor_nnz.
int64_t symbolic_factor_nnz(Symbolic &sym);

// Nested-dissection order of a symmetric graph (no self loops); exposed for tests.
void nd_order(int n, const int32_t *rowptr, const int32_t *col, std::vector<int32_t> &perm,
              std::vector<int32_t> &block_ptr);

}  // namespace arapgpu

/*
 * deform/arap.h -- drop-in for cheind/mesh-deform's inc/deform/arap.h.
 *
 * Same class template, same mesh adapter concept, same setConstraint/deform
 * semantics; the hot path runs on the GPU through the C ABI of
 * include/arap_gpu.h (link libarap_gb300.so). Header-only C++17, no Eigen
 * dependency: vertex and face values are read with operator()(int) and vertex
 * values are written back by constructing the adapter's vertex type from three
 * scalars, which Eigen::Matrix<S,3,1> and deform::Vec3 both support.
 *
 * Behaviour kept from the reference (inc/deform/arap.h):
 *   - the constructor reads the faces once (arap.h:66-70,149-155);
 *   - setConstraint stores the target cast to Scalar in a map and marks the
 *     object dirty; a second call for the same vertex overwrites (arap.h:81-85);
 *   - a dirty deform re-captures the rest pose from the mesh's current
 *     positions, recomputes weights, resets rotations, rebuilds and refactors
 *     the constrained Laplacian (arap.h:102-120); a clean deform continues
 *     from the current solution with the same factor (arap.h:122-129);
 *   - with no constraint deform returns true, writes nothing back and stays
 *     dirty (arap.h:113-114); a failed factorisation returns false (arap.h:116-117);
 *   - the result is written back through the adapter, cast to Mesh::Scalar
 *     (arap.h:133-135).
 * Precision: PrecisionType = double runs the FP64 GPU form; float runs the
 * mixed form (FP64 factor, FP32 local step and solves with FP64-residual
 * refinement), which is more accurate than the reference's all-float path.
 *
 * Test access: as in the reference (arap.h:28,141,445,453), the private
 * typedef SparseMatrix and the member _edgeWeights are reachable from the
 * friend template PrivateAccessor<ARAP>, so an accessor that returns
 * `typename ARAP::SparseMatrix` from `a._edgeWeights` works unchanged.
 * SparseMatrix is Eigen::SparseMatrix<Scalar, Eigen::RowMajor> when Eigen's
 * headers are on the include path (define DEFORM_NO_EIGEN to opt out), else
 * deform::SparseRowMatrix<Scalar>. _edgeWeights reads the weights from the
 * device when it is converted to SparseMatrix; before the first deform it is
 * an empty matrix, as the reference's member is.
 *
 * No device: the constructor does not throw (the reference's cannot fail);
 * deform then returns false and lastError() says why.
 */
#ifndef DEFORM_ARAP_H
#define DEFORM_ARAP_H

#include <arap_gpu.h>

#include <algorithm>
#include <cstdint>
#include <map>
#include <string>
#include <type_traits>
#include <vector>

#if !defined(DEFORM_NO_EIGEN) && defined(__has_include)
#if __has_include(<Eigen/Sparse>)
#include <Eigen/Sparse>
#define DEFORM_HAVE_EIGEN 1
#endif
#endif

namespace deform {

/** Forward declaration of a class with access to internals (tests), as arap.h:28. */
template <class T> class PrivateAccessor;

/** Row-major compressed sparse matrix: the form of _edgeWeights when Eigen is
    not available. Columns are sorted within each row. */
template <class S>
struct SparseRowMatrix {
    typedef S Scalar;
    int32_t n = 0;
    std::vector<int32_t> rowptr{0}, col;
    std::vector<S> val;
    int rows() const { return n; }
    int cols() const { return n; }
    int nonZeros() const { return (int)col.size(); }
    /** Entry (r, c), zero where the pattern has none. */
    S coeff(int r, int c) const {
        const auto b = col.begin() + rowptr[r], e = col.begin() + rowptr[r + 1];
        const auto it = std::lower_bound(b, e, c);
        return (it != e && *it == c) ? val[it - col.begin()] : S(0);
    }
};

template <class MeshType, class PrecisionType = typename MeshType::Scalar>
class AsRigidAsPossibleDeformation {
public:
    /** Floating point precision used in calculations. */
    typedef PrecisionType Scalar;
    /** Mesh type we are working on. */
    typedef MeshType Mesh;
    /** Type for indices. */
    typedef int Index;

    /** Construct from mesh; the mesh must outlive this object. device: CUDA ordinal. */
    AsRigidAsPossibleDeformation(Mesh &mesh, int device = 0) : _mesh(mesh), _edgeWeights(this), _dirty(true) {
        initializeMeshTopology(device);
    }

    ~AsRigidAsPossibleDeformation() { arap_destroy(_ctx); }

    AsRigidAsPossibleDeformation(const AsRigidAsPossibleDeformation &) = delete;
    AsRigidAsPossibleDeformation &operator=(const AsRigidAsPossibleDeformation &) = delete;

    /** Set the positional constraint of a vertex (arap.h:81-85). */
    template <class V>
    void setConstraint(Index vidx, const V &loc) {
        _constrainedLocations[vidx] = {Scalar(loc(0)), Scalar(loc(1)), Scalar(loc(2))};
        _dirty = true;
    }

    /** Run numberOfIterations local/global iterations (arap.h:101-138). */
    bool deform(Index numberOfIterations) {
        const Index V = _mesh.numberOfVertices();
        if (!_ctx) return false;  // no device (lastError() says why)
        const bool was_dirty = _dirty;
        if (_dirty) {
            std::vector<double> xyz((size_t)3 * V);
            for (Index v = 0; v < V; ++v) {
                auto p = _mesh.vertexLocation(v);
                for (int c = 0; c < 3; ++c) xyz[(size_t)3 * v + c] = static_cast<double>(Scalar(p(c)));
            }
            if (arap_set_rest_positions(_ctx, xyz.data()) != ARAP_OK) return false;
            std::vector<int32_t> idx;
            std::vector<double> tgt;
            idx.reserve(_constrainedLocations.size());
            tgt.reserve(3 * _constrainedLocations.size());
            for (const auto &kv : _constrainedLocations) {
                idx.push_back(kv.first);
                for (int c = 0; c < 3; ++c) tgt.push_back(static_cast<double>(kv.second.v[c]));
            }
            if (arap_set_constraints(_ctx, (int32_t)idx.size(), idx.data(), tgt.data()) != ARAP_OK) return false;
        }
        std::vector<double> out((size_t)3 * V);
        const int rc = arap_deform(_ctx, numberOfIterations, out.data());
        if (rc != ARAP_OK) {
            _lastError = arap_last_error(_ctx);
            return false;
        }
        if (was_dirty) _weightsValid = true;
        if (_constrainedLocations.empty()) return true;  // arap.h:113-114
        _dirty = false;
        typedef typename std::decay<decltype(_mesh.vertexLocation(0))>::type VertexType;
        typedef typename Mesh::Scalar MS;
        for (Index v = 0; v < V; ++v)
            _mesh.vertexLocation(v, VertexType(static_cast<MS>(out[(size_t)3 * v]),
                                               static_cast<MS>(out[(size_t)3 * v + 1]),
                                               static_cast<MS>(out[(size_t)3 * v + 2])));
        return true;
    }

    /** Message of the last failed deform (empty when none). */
    const std::string &lastError() const { return _lastError; }

    /** Extension: refinement solves per iteration of the mixed form beyond the
        first (default 2). */
    void setRefinementSteps(int steps) {
        if (_ctx) arap_set_precision(_ctx, precision(), steps);
        _dirty = true;
    }

private:
    template <class> friend class PrivateAccessor;

    struct Point { Scalar v[3]; };

#ifdef DEFORM_HAVE_EIGEN
    typedef Eigen::SparseMatrix<Scalar, Eigen::RowMajor> SparseMatrix;
#else
    typedef SparseRowMatrix<Scalar> SparseMatrix;
#endif

    /** _edgeWeights: the cotan weights of the last dirty deform
        (computeCotanWeights, arap.h:182-239), read from the device when
        converted to SparseMatrix. */
    class EdgeWeights {
    public:
        explicit EdgeWeights(const AsRigidAsPossibleDeformation *owner) : _owner(owner) {}
        operator SparseMatrix() const {
            const int n = _owner->_weightsValid ? _owner->_mesh.numberOfVertices() : 0;
            std::vector<int32_t> rowptr((size_t)n + 1, 0), col;
            std::vector<double> val;
            if (n > 0) {
                int32_t nnz = 0;
                arap_edge_weights_nnz(_owner->_ctx, &nnz);
                col.resize(nnz);
                val.resize(nnz);
                arap_get_edge_weights(_owner->_ctx, rowptr.data(), col.data(), val.data());
            }
#ifdef DEFORM_HAVE_EIGEN
            SparseMatrix m(n, n);
            std::vector<Eigen::Triplet<Scalar>> t;
            t.reserve(col.size());
            for (int r = 0; r < n; ++r)
                for (int q = rowptr[r]; q < rowptr[r + 1]; ++q) t.emplace_back(r, col[q], Scalar(val[q]));
            m.setFromTriplets(t.begin(), t.end());
            return m;
#else
            SparseMatrix m;
            m.n = n;
            m.rowptr = rowptr;
            m.col = col;
            m.val.assign(val.begin(), val.end());
            return m;
#endif
        }

    private:
        const AsRigidAsPossibleDeformation *_owner;
    };

    static int precision() {
        return std::is_same<Scalar, double>::value ? ARAP_PRECISION_FP64 : ARAP_PRECISION_MIXED;
    }

    void initializeMeshTopology(int device) {
        const Index F = _mesh.numberOfFaces();
        std::vector<int32_t> faces((size_t)3 * F);
        for (Index f = 0; f < F; ++f) {
            auto t = _mesh.face(f);
            for (int c = 0; c < 3; ++c) faces[(size_t)3 * f + c] = static_cast<int32_t>(t(c));
        }
        const int rc = arap_create(_mesh.numberOfVertices(), F, faces.data(), device, &_ctx);
        if (rc != ARAP_OK) {
            _ctx = nullptr;
            _lastError = std::string("arap_create: ") + arap_status_string(rc) + ": " + arap_last_error(nullptr);
            return;
        }
        arap_set_precision(_ctx, precision(), 2);
    }

    Mesh &_mesh;
    EdgeWeights _edgeWeights;
    bool _weightsValid = false;
    arap_ctx *_ctx = nullptr;
    std::map<Index, Point> _constrainedLocations;
    bool _dirty;
    std::string _lastError;
};

}  // namespace deform

#endif

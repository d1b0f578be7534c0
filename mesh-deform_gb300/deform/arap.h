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
 * mixed form (FP32 local step and solves with FP64-residual refinement), which
 * is more accurate than the reference's all-float path.
 */
#ifndef DEFORM_ARAP_H
#define DEFORM_ARAP_H

#include <arap_gpu.h>

#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

namespace deform {

/** Forward declaration of a class with access to internals (tests), as arap.h:28. */
template <class T> class PrivateAccessor;

/** Compressed sparse rows of _edgeWeights. */
struct EdgeWeightsCSR {
    std::vector<int32_t> rowptr, col;
    std::vector<double> val;
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
    AsRigidAsPossibleDeformation(Mesh &mesh, int device = 0) : _mesh(mesh), _dirty(true) {
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

    /** Extension: refinement solves per iteration of the mixed form (default 2). */
    void setRefinementSteps(int steps) {
        arap_set_precision(_ctx, precision(), steps);
        _dirty = true;
    }

private:
    template <class> friend class PrivateAccessor;

    struct Point { Scalar v[3]; };

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
        if (rc != ARAP_OK)
            throw std::runtime_error(std::string("arap_create: ") + arap_status_string(rc) + ": " +
                                     arap_last_error(nullptr));
        arap_set_precision(_ctx, precision(), 2);
    }

    /** _edgeWeights (arap.h:453) as CSR, for PrivateAccessor. */
    EdgeWeightsCSR edgeWeights() const {
        EdgeWeightsCSR w;
        int32_t nnz = 0;
        arap_edge_weights_nnz(_ctx, &nnz);
        w.rowptr.resize((size_t)_mesh.numberOfVertices() + 1);
        w.col.resize(nnz);
        w.val.resize(nnz);
        arap_get_edge_weights(_ctx, w.rowptr.data(), w.col.data(), w.val.data());
        return w;
    }

    Mesh &_mesh;
    arap_ctx *_ctx = nullptr;
    std::map<Index, Point> _constrainedLocations;
    bool _dirty;
    std::string _lastError;
};

}  // namespace deform

#endif

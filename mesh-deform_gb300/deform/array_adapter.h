/*
 * deform/array_adapter.h -- a mesh adapter over plain arrays.
 *
 * Provides the five accessors of the adapter concept that
 * deform::AsRigidAsPossibleDeformation needs (the reference's OpenMeshAdapter,
 * inc/deform/openmesh_adapter.h:54-113), for callers that keep their mesh in
 * flat arrays instead of OpenMesh. Vec3 mirrors the small part of
 * Eigen::Matrix<S,3,1> the template uses: operator()(int) and a three-scalar
 * constructor.
 */
#ifndef DEFORM_ARRAY_ADAPTER_H
#define DEFORM_ARRAY_ADAPTER_H

#include <array>
#include <vector>

namespace deform {

template <class S>
struct Vec3 {
    S v[3];
    Vec3() : v{S(0), S(0), S(0)} {}
    Vec3(S x, S y, S z) : v{x, y, z} {}
    S &operator()(int i) { return v[i]; }
    const S &operator()(int i) const { return v[i]; }
};

struct Face3 {
    int v[3];
    int operator()(int i) const { return v[i]; }
};

template <class S>
class ArrayMeshAdapter {
public:
    /** Floating point precision type of the mesh. Required. */
    typedef S Scalar;
    typedef Vec3<S> VertexType;
    typedef Face3 FaceType;

    ArrayMeshAdapter() = default;
    ArrayMeshAdapter(std::vector<std::array<S, 3>> positions, std::vector<std::array<int, 3>> faces)
        : _positions(std::move(positions)), _faces(std::move(faces)) {}

    int addVertex(S x, S y, S z) {
        _positions.push_back({x, y, z});
        return (int)_positions.size() - 1;
    }
    int addFace(int a, int b, int c) {
        _faces.push_back({a, b, c});
        return (int)_faces.size() - 1;
    }

    /** Retrieve a vertex position. Required. */
    VertexType vertexLocation(int idx) const {
        const auto &p = _positions[idx];
        return VertexType(p[0], p[1], p[2]);
    }
    /** Set a vertex position. Required. */
    void vertexLocation(int idx, const VertexType &v) { _positions[idx] = {v(0), v(1), v(2)}; }
    /** Triangle corners, counter-clockwise. Required. */
    FaceType face(int idx) const { return FaceType{{_faces[idx][0], _faces[idx][1], _faces[idx][2]}}; }
    /** Number of faces. Required. */
    int numberOfFaces() const { return (int)_faces.size(); }
    /** Number of vertices. Required. */
    int numberOfVertices() const { return (int)_positions.size(); }

    const std::vector<std::array<S, 3>> &positions() const { return _positions; }

private:
    std::vector<std::array<S, 3>> _positions;
    std::vector<std::array<int, 3>> _faces;
};

}  // namespace deform

#endif

// deform/obj_io.h -- Wavefront OBJ reading and writing for the array adapter.
//
// The reference's examples and tests load their meshes (etc/sphere.obj,
// etc/bar.obj, etc/plane.obj) through OpenMesh's reader; this header reads the
// same files without OpenMesh: `v x y z` lines and `f` lines whose corners may
// be `i`, `i/t`, `i//n` or `i/t/n` (1-based, negative = relative to the end);
// polygons are split into a triangle fan. Other lines are ignored. The writer
// emits `v` and `f` lines, so a deformed mesh can be inspected or reloaded.
#ifndef DEFORM_OBJ_IO_H
#define DEFORM_OBJ_IO_H

#include <cstdint>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace deform {
namespace obj {

struct Mesh {
    std::vector<double> positions;  // 3 per vertex
    std::vector<int32_t> faces;     // 3 per triangle, 0-based
    int numberOfVertices() const { return (int)(positions.size() / 3); }
    int numberOfFaces() const { return (int)(faces.size() / 3); }
};

inline Mesh read(const std::string &path) {
    std::ifstream in(path);
    if (!in) throw std::runtime_error("cannot open " + path);
    Mesh m;
    std::string line;
    int lineno = 0;
    while (std::getline(in, line)) {
        ++lineno;
        std::istringstream ls(line);
        std::string tag;
        if (!(ls >> tag)) continue;
        if (tag == "v") {
            double x, y, z;
            if (!(ls >> x >> y >> z)) throw std::runtime_error(path + ":" + std::to_string(lineno) + ": bad vertex");
            m.positions.insert(m.positions.end(), {x, y, z});
        } else if (tag == "f") {
            std::vector<int32_t> corner;
            std::string tok;
            const int nv = m.numberOfVertices();
            while (ls >> tok) {
                const long i = std::stol(tok.substr(0, tok.find('/')));
                const long idx = i > 0 ? i - 1 : nv + i;
                if (i == 0 || idx < 0 || idx >= nv)
                    throw std::runtime_error(path + ":" + std::to_string(lineno) + ": bad face index " + tok);
                corner.push_back((int32_t)idx);
            }
            if (corner.size() < 3) throw std::runtime_error(path + ":" + std::to_string(lineno) + ": face with <3 corners");
            for (size_t k = 1; k + 1 < corner.size(); ++k)
                m.faces.insert(m.faces.end(), {corner[0], corner[k], corner[k + 1]});
        }
    }
    return m;
}

inline void write(const std::string &path, const double *positions, int n_vertices, const int32_t *faces,
                  int n_faces) {
    FILE *f = std::fopen(path.c_str(), "w");
    if (!f) throw std::runtime_error("cannot write " + path);
    for (int v = 0; v < n_vertices; ++v)
        std::fprintf(f, "v %.17g %.17g %.17g\n", positions[3 * v], positions[3 * v + 1], positions[3 * v + 2]);
    for (int t = 0; t < n_faces; ++t)
        std::fprintf(f, "f %d %d %d\n", faces[3 * t] + 1, faces[3 * t + 1] + 1, faces[3 * t + 2] + 1);
    std::fclose(f);
}

}  // namespace obj
}  // namespace deform

#endif

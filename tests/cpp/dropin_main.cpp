// dropin_main.cpp -- exercises the header-only drop-in (deform/arap.h) the way
// the reference's own tests and examples use inc/deform/arap.h.
//
//   dropin_main kat                      the cotan known-answer test of
//                                        tests/test_cotan.cpp:20-54 (unit square, deform(0))
//   dropin_main run <in> <out> <float|double>
//                                        reads a mesh + constraints + iteration count,
//                                        deforms through the template, writes positions
#include <deform/arap.h>
#include <deform/array_adapter.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

namespace deform {
template <class ARAP>
class PrivateAccessor {
public:
    static EdgeWeightsCSR cotanWeights(const ARAP &a) { return a.edgeWeights(); }
};
}  // namespace deform

static int kat() {
    typedef deform::ArrayMeshAdapter<float> Mesh;
    Mesh m;
    m.addVertex(0.f, 0.f, 0.f);
    m.addVertex(1.f, 0.f, 0.f);
    m.addVertex(1.f, 1.f, 0.f);
    m.addVertex(0.f, 1.f, 0.f);
    m.addFace(0, 1, 2);
    m.addFace(0, 2, 3);
    typedef deform::AsRigidAsPossibleDeformation<Mesh> ARAP;
    ARAP arap(m);
    if (!arap.deform(0)) { std::printf("deform(0) failed\n"); return 1; }
    deform::EdgeWeightsCSR w = deform::PrivateAccessor<ARAP>::cotanWeights(arap);
    if (w.rowptr.size() != 5) { std::printf("rows %zu\n", w.rowptr.size()); return 1; }
    double sp[4][4] = {{0}};
    for (int i = 0; i < 4; ++i)
        for (int q = w.rowptr[i]; q < w.rowptr[i + 1]; ++q) sp[i][w.col[q]] = w.val[q];
    const double expected[4][4] = {{0, .5, 0, .5}, {.5, 0, .5, 0}, {0, .5, 0, .5}, {.5, 0, .5, 0}};
    double d2 = 0, a2 = 0, b2 = 0;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            d2 += (sp[i][j] - expected[i][j]) * (sp[i][j] - expected[i][j]);
            a2 += sp[i][j] * sp[i][j];
            b2 += expected[i][j] * expected[i][j];
        }
    // Eigen's isApprox(expected, 1e-4)
    const bool ok = std::sqrt(d2) <= 1e-4 * std::sqrt(a2 < b2 ? a2 : b2);
    std::printf("kat %s\n", ok ? "ok" : "FAILED");
    return ok ? 0 : 1;
}

template <class S>
static int run(const char *in, const char *out) {
    FILE *f = std::fopen(in, "rb");
    if (!f) return 2;
    int32_t hdr[4];  // V, F, n constraints, iterations
    if (std::fread(hdr, 4, 4, f) != 4) return 2;
    const int V = hdr[0], F = hdr[1], nc = hdr[2], iters = hdr[3];
    std::vector<double> pos((size_t)3 * V), tgt((size_t)3 * nc);
    std::vector<int32_t> faces((size_t)3 * F), cidx(nc);
    bool okr = std::fread(pos.data(), 8, pos.size(), f) == pos.size() &&
               std::fread(faces.data(), 4, faces.size(), f) == faces.size() &&
               std::fread(cidx.data(), 4, cidx.size(), f) == cidx.size() &&
               std::fread(tgt.data(), 8, tgt.size(), f) == tgt.size();
    std::fclose(f);
    if (!okr) return 2;
    typedef deform::ArrayMeshAdapter<double> Mesh;  // mesh scalar double, compute scalar S
    Mesh m;
    for (int v = 0; v < V; ++v) m.addVertex(pos[3 * v], pos[3 * v + 1], pos[3 * v + 2]);
    for (int t = 0; t < F; ++t) m.addFace(faces[3 * t], faces[3 * t + 1], faces[3 * t + 2]);
    deform::AsRigidAsPossibleDeformation<Mesh, S> arap(m);
    for (int i = 0; i < nc; ++i)
        arap.setConstraint(cidx[i], deform::Vec3<double>(tgt[3 * i], tgt[3 * i + 1], tgt[3 * i + 2]));
    if (!arap.deform(iters)) { std::printf("deform failed: %s\n", arap.lastError().c_str()); return 1; }
    f = std::fopen(out, "wb");
    for (const auto &p : m.positions()) std::fwrite(p.data(), 8, 3, f);
    std::fclose(f);
    return 0;
}

int main(int argc, char **argv) {
    if (argc >= 2 && std::strcmp(argv[1], "kat") == 0) return kat();
    if (argc >= 5 && std::strcmp(argv[1], "run") == 0)
        return std::strcmp(argv[4], "float") == 0 ? run<float>(argv[2], argv[3]) : run<double>(argv[2], argv[3]);
    std::printf("usage: dropin_main kat | run <in> <out> <float|double>\n");
    return 2;
}

// dropin_main.cpp -- exercises the header-only drop-in (deform/arap.h) the way
// the reference's own tests and examples use inc/deform/arap.h.
//
//   dropin_main kat                      the cotan known-answer test of
//                                        tests/test_cotan.cpp:20-54 (unit square, deform(0))
//   dropin_main run <in> <out> <float|double>
//                                        reads a mesh + constraints + iteration count,
//                                        deforms through the template, writes positions
//   dropin_main nodevice                 construction and the accessor without a GPU:
//                                        no exception, an empty weight matrix before the
//                                        first deform, deform() false with a message
//
// The weights are read through PrivateAccessor<ARAP>::cotanWeights, which
// returns `typename ARAP::SparseMatrix` from `a._edgeWeights`, the contract of
// the reference's tests/accessor.h. Built with -DDEFORM_REFERENCE_ACCESSOR and
// the reference's tests/ directory on the include path, that file itself is
// used; otherwise an accessor of the same shape is defined here.
#include <deform/arap.h>
#include <deform/array_adapter.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#ifdef DEFORM_REFERENCE_ACCESSOR
#include <accessor.h>
#else
namespace deform {
template <class ARAP>
class PrivateAccessor {
public:
    static typename ARAP::SparseMatrix cotanWeights(const ARAP &a) { return a._edgeWeights; }
};
}  // namespace deform
#endif

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
    const auto w = deform::PrivateAccessor<ARAP>::cotanWeights(arap);
    if (w.rows() != 4 || w.cols() != 4) { std::printf("size %d x %d\n", (int)w.rows(), (int)w.cols()); return 1; }
    double sp[4][4] = {{0}};
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) sp[i][j] = w.coeff(i, j);
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

static int nodevice() {
    typedef deform::ArrayMeshAdapter<double> Mesh;
    Mesh m;
    m.addVertex(0., 0., 0.);
    m.addVertex(1., 0., 0.);
    m.addVertex(0., 1., 0.);
    m.addFace(0, 1, 2);
    typedef deform::AsRigidAsPossibleDeformation<Mesh> ARAP;
    ARAP arap(m);  // must not throw
    const auto w = deform::PrivateAccessor<ARAP>::cotanWeights(arap);
    if (w.rows() != 0 || w.nonZeros() != 0) { std::printf("weights before deform not empty\n"); return 1; }
    arap.setConstraint(0, deform::Vec3<double>(0., 0., 1.));
    const bool ok = arap.deform(1);
    std::printf("nodevice deform=%d error=%s\n", ok ? 1 : 0, arap.lastError().c_str());
    return ok ? 3 : 0;
}

int main(int argc, char **argv) {
    if (argc >= 2 && std::strcmp(argv[1], "kat") == 0) return kat();
    if (argc >= 2 && std::strcmp(argv[1], "nodevice") == 0) return nodevice();
    if (argc >= 5 && std::strcmp(argv[1], "run") == 0)
        return std::strcmp(argv[4], "float") == 0 ? run<float>(argv[2], argv[3]) : run<double>(argv[2], argv[3]);
    std::printf("usage: dropin_main kat | run <in> <out> <float|double>\n");
    return 2;
}

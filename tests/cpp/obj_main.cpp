// Reads an OBJ with deform/obj_io.h and writes it back (v and f lines only).
#include <cstdio>
#include "deform/obj_io.h"
int main(int argc, char **argv) {
    if (argc < 3) return 2;
    try {
        deform::obj::Mesh m = deform::obj::read(argv[1]);
        deform::obj::write(argv[2], m.positions.data(), m.numberOfVertices(), m.faces.data(), m.numberOfFaces());
        std::printf("%d %d\n", m.numberOfVertices(), m.numberOfFaces());
    } catch (const std::exception &e) {
        std::printf("error: %s\n", e.what());
        return 1;
    }
    return 0;
}

// Prints TrajectorySE3 samples (deform/trajectory.h) of the key poses given
// on stdin: n, then n row-major 3x4 matrices; then m times; output: m lines of
// 12 numbers.
#include <cstdio>
#include <vector>
#include "deform/trajectory.h"
int main() {
    typedef deform::TrajectorySE3<double> Traj;
    Traj path;
    int n = 0;
    if (std::scanf("%d", &n) != 1) return 2;
    for (int i = 0; i < n; ++i) {
        Traj::Transform T;
        for (int k = 0; k < 12; ++k)
            if (std::scanf("%lf", &T[k]) != 1) return 2;
        path.addKeyPose(T);
    }
    int m = 0;
    if (std::scanf("%d", &m) != 1) return 2;
    for (int j = 0; j < m; ++j) {
        double t;
        if (std::scanf("%lf", &t) != 1) return 2;
        const Traj::Transform T = path(t);
        for (int k = 0; k < 12; ++k) std::printf("%.17g%c", T[k], k == 11 ? '\n' : ' ');
    }
    return 0;
}

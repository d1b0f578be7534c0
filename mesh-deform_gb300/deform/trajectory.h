// deform/trajectory.h -- TrajectorySE3 without Eigen or Sophus.
//
// Same behaviour as the reference's deform::TrajectorySE3
// (inc/deform/trajectory.h:33-83): key poses are mapped to se(3) by the SE3
// logarithm (tangent = (upsilon, omega), translation part first, as Sophus
// orders it), a cubic B-spline interpolates the tangents (chord-length
// parameters in [0, 1], knots by averaging, as Eigen's
// SplineFitting::Interpolate(points, 3) chooses them), and a time t in [0, 1]
// maps back through the SE3 exponential. Poses are row-major 3x4 affine
// matrices [R | t].
//
// The spline interpolation follows the textbook global interpolation method
// (Piegl & Tiller, The NURBS Book, 2nd ed., section 9.2.1: eqs. 9.5 and 9.8,
// algorithms A2.1 FindSpan and A2.2 BasisFuns); the SE(3) maps are the
// closed forms of Barfoot, State Estimation for Robotics, section 7.1.
#ifndef DEFORM_TRAJECTORY_H
#define DEFORM_TRAJECTORY_H

#include <array>
#include <cmath>
#include <stdexcept>
#include <vector>

namespace deform {

template <class PrecisionType>
class TrajectorySE3 {
  public:
    typedef PrecisionType Scalar;
    typedef std::array<Scalar, 12> Transform;  // row-major [R | t]
    typedef std::array<Scalar, 6> Tangent;     // (upsilon, omega)

    TrajectorySE3() : _dirty(false) {}

    Transform addKeyPose(const Transform &transform) {
        _poses.push_back(transform);
        _dirty = true;
        return transform;
    }

    Transform operator()(Scalar time) {
        if (_dirty) {
            fit();
            _dirty = false;
        }
        return exp(evaluate(time));
    }

    // SE(3) logarithm and exponential (Barfoot sec. 7.1.4 / 7.1.3)
    static Tangent log(const Transform &T) {
        const Scalar R[9] = {T[0], T[1], T[2], T[4], T[5], T[6], T[8], T[9], T[10]};
        const Scalar tr = R[0] + R[4] + R[8];
        const Scalar c = std::max(Scalar(-1), std::min(Scalar(1), (tr - 1) / 2));
        const Scalar theta = std::acos(c);
        Scalar w[3] = {R[7] - R[5], R[2] - R[6], R[3] - R[1]};  // 2 sin(theta) * axis
        Scalar f;                                                // omega = f * w
        if (theta < Scalar(1e-6)) {
            f = Scalar(0.5) + theta * theta / 12;
        } else if (Scalar(M_PI) - theta < Scalar(1e-4)) {
            // near pi: the axis from the symmetric part, R = 2 a a^T - I
            Scalar a[3];
            const int k = (R[0] >= R[4] && R[0] >= R[8]) ? 0 : (R[4] >= R[8] ? 1 : 2);
            a[k] = std::sqrt(std::max(Scalar(0), (R[4 * k] + 1) / 2));
            for (int j = 0; j < 3; ++j)
                if (j != k) a[j] = (R[3 * k + j] + R[3 * j + k]) / (4 * a[k]);
            // sign from the antisymmetric part when it is not lost to rounding
            const Scalar s = a[0] * w[0] + a[1] * w[1] + a[2] * w[2];
            const Scalar sg = s < 0 ? Scalar(-1) : Scalar(1);
            for (int j = 0; j < 3; ++j) w[j] = sg * a[j] * theta;
            f = 1;
        } else {
            f = theta / (2 * std::sin(theta));
        }
        const Scalar om[3] = {f * w[0], f * w[1], f * w[2]};
        Scalar Vinv[9];
        left_jacobian(om, true, Vinv);
        Tangent x;
        for (int i = 0; i < 3; ++i) x[i] = Vinv[3 * i] * T[3] + Vinv[3 * i + 1] * T[7] + Vinv[3 * i + 2] * T[11];
        x[3] = om[0];
        x[4] = om[1];
        x[5] = om[2];
        return x;
    }

    static Transform exp(const Tangent &x) {
        const Scalar om[3] = {x[3], x[4], x[5]};
        const Scalar th2 = om[0] * om[0] + om[1] * om[1] + om[2] * om[2], th = std::sqrt(th2);
        Scalar A, B;  // R = I + A W + B W^2
        if (th < Scalar(1e-6)) {
            A = 1 - th2 / 6;
            B = Scalar(0.5) - th2 / 24;
        } else {
            A = std::sin(th) / th;
            B = (1 - std::cos(th)) / th2;
        }
        Scalar W[9], W2[9];
        hat(om, W);
        mul3(W, W, W2);
        Scalar V[9];
        left_jacobian(om, false, V);
        Transform T;
        for (int i = 0; i < 3; ++i) {
            for (int j = 0; j < 3; ++j) T[4 * i + j] = (i == j ? 1 : 0) + A * W[3 * i + j] + B * W2[3 * i + j];
            T[4 * i + 3] = V[3 * i] * x[0] + V[3 * i + 1] * x[1] + V[3 * i + 2] * x[2];
        }
        return T;
    }

  private:
    static void hat(const Scalar *w, Scalar *W) {
        W[0] = 0; W[1] = -w[2]; W[2] = w[1];
        W[3] = w[2]; W[4] = 0; W[5] = -w[0];
        W[6] = -w[1]; W[7] = w[0]; W[8] = 0;
    }
    static void mul3(const Scalar *a, const Scalar *b, Scalar *c) {
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) c[3 * i + j] = a[3 * i] * b[j] + a[3 * i + 1] * b[3 + j] + a[3 * i + 2] * b[6 + j];
    }
    // left Jacobian of SO(3) (the V of the SE(3) exponential) or its inverse
    static void left_jacobian(const Scalar *om, bool inverse, Scalar *J) {
        const Scalar th2 = om[0] * om[0] + om[1] * om[1] + om[2] * om[2], th = std::sqrt(th2);
        Scalar W[9], W2[9];
        hat(om, W);
        mul3(W, W, W2);
        Scalar a, b;
        if (!inverse) {  // V = I + (1 - cos)/th^2 W + (th - sin)/th^3 W^2
            if (th < Scalar(1e-6)) {
                a = Scalar(0.5) - th2 / 24;
                b = Scalar(1) / 6 - th2 / 120;
            } else {
                a = (1 - std::cos(th)) / th2;
                b = (th - std::sin(th)) / (th2 * th);
            }
        } else {  // V^-1 = I - W/2 + (1 - th sin / (2 (1 - cos))) / th^2 W^2
            a = Scalar(-0.5);
            if (th < Scalar(1e-6)) b = Scalar(1) / 12 + th2 / 720;
            else b = (1 - th * std::sin(th) / (2 * (1 - std::cos(th)))) / th2;
        }
        for (int i = 0; i < 9; ++i) J[i] = ((i % 4) == 0 ? 1 : 0) + a * W[i] + b * W2[i];
    }

    // cubic B-spline through the key tangents
    void fit() {
        const int n = (int)_poses.size();
        if (n == 0) throw std::runtime_error("TrajectorySE3: no key pose");
        std::vector<Tangent> pts(n);
        for (int i = 0; i < n; ++i) pts[i] = log(_poses[i]);
        _p = std::min(3, n - 1);  // degree (lower with fewer than 4 poses)
        // chord-length parameters (eq. 9.5)
        _u.assign(n, 0);
        for (int i = 1; i < n; ++i) {
            Scalar d = 0;
            for (int k = 0; k < 6; ++k) d += (pts[i][k] - pts[i - 1][k]) * (pts[i][k] - pts[i - 1][k]);
            _u[i] = _u[i - 1] + std::sqrt(d);
        }
        for (int i = 1; i < n; ++i) _u[i] = _u[n - 1] > 0 ? _u[i] / _u[n - 1] : Scalar(i) / (n - 1);
        // knots by averaging (eq. 9.8)
        _knots.assign(n + _p + 1, 0);
        for (int i = n; i < n + _p + 1; ++i) _knots[i] = 1;
        for (int j = 1; j < n - _p; ++j) {
            Scalar s = 0;
            for (int i = j; i < j + _p; ++i) s += _u[i];
            _knots[j + _p] = s / _p;
        }
        // A c = pts, A[i][j] = N_j(u_i); solved by Gaussian elimination with partial pivoting
        _ctrl = pts;  // right-hand sides, solved in place (find_span needs the count)
        std::vector<Scalar> A((size_t)n * n, 0);
        std::vector<Scalar> N(_p + 1);
        for (int i = 0; i < n; ++i) {
            const int span = find_span(_u[i]);
            basis(span, _u[i], N.data());
            for (int k = 0; k <= _p; ++k) A[(size_t)i * n + span - _p + k] = N[k];
        }
        for (int c = 0; c < n; ++c) {
            int piv = c;
            for (int r = c + 1; r < n; ++r)
                if (std::abs(A[(size_t)r * n + c]) > std::abs(A[(size_t)piv * n + c])) piv = r;
            if (piv != c) {
                for (int k = 0; k < n; ++k) std::swap(A[(size_t)c * n + k], A[(size_t)piv * n + k]);
                std::swap(_ctrl[c], _ctrl[piv]);
            }
            for (int r = c + 1; r < n; ++r) {
                const Scalar f = A[(size_t)r * n + c] / A[(size_t)c * n + c];
                if (f == 0) continue;
                for (int k = c; k < n; ++k) A[(size_t)r * n + k] -= f * A[(size_t)c * n + k];
                for (int k = 0; k < 6; ++k) _ctrl[r][k] -= f * _ctrl[c][k];
            }
        }
        for (int c = n - 1; c >= 0; --c) {
            for (int k = c + 1; k < n; ++k)
                for (int d = 0; d < 6; ++d) _ctrl[c][d] -= A[(size_t)c * n + k] * _ctrl[k][d];
            for (int d = 0; d < 6; ++d) _ctrl[c][d] /= A[(size_t)c * n + c];
        }
    }

    int find_span(Scalar u) const {  // A2.1
        const int n = (int)_ctrl.size() - 1;
        if (u >= _knots[n + 1]) return n;
        if (u <= _knots[_p]) return _p;
        int lo = _p, hi = n + 1, mid = (lo + hi) / 2;
        while (u < _knots[mid] || u >= _knots[mid + 1]) {
            if (u < _knots[mid]) hi = mid;
            else lo = mid;
            mid = (lo + hi) / 2;
        }
        return mid;
    }

    void basis(int i, Scalar u, Scalar *N) const {  // A2.2
        Scalar left[4], right[4];
        N[0] = 1;
        for (int j = 1; j <= _p; ++j) {
            left[j] = u - _knots[i + 1 - j];
            right[j] = _knots[i + j] - u;
            Scalar saved = 0;
            for (int r = 0; r < j; ++r) {
                const Scalar tmp = N[r] / (right[r + 1] + left[j - r]);
                N[r] = saved + right[r + 1] * tmp;
                saved = left[j - r] * tmp;
            }
            N[j] = saved;
        }
    }

    Tangent evaluate(Scalar t) const {
        const Scalar u = std::max(Scalar(0), std::min(Scalar(1), t));
        Tangent x{};
        if (_ctrl.size() == 1) return _ctrl[0];
        const int span = find_span(u);
        Scalar N[4];
        basis(span, u, N);
        for (int k = 0; k <= _p; ++k)
            for (int d = 0; d < 6; ++d) x[d] += N[k] * _ctrl[span - _p + k][d];
        return x;
    }

    bool _dirty;
    int _p = 3;
    std::vector<Transform> _poses;
    std::vector<Tangent> _ctrl;
    std::vector<Scalar> _u, _knots;
};

}  // namespace deform

#endif

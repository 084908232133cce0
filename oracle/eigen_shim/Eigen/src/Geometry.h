// Oracle (test infrastructure only): AngleAxis of the Eigen-API shim.
#pragma once

namespace Eigen {

template <typename T>
class AngleAxis {
public:
    AngleAxis() : angle_(0), axis_(Matrix<T, 3, 1>(T(1), T(0), T(0))) {}
    AngleAxis(T angle, const Matrix<T, 3, 1>& axis) : angle_(angle), axis_(axis) {}
    // From a rotation matrix: the angle from the trace, the axis from the
    // skew part (or, near pi, from the largest diagonal of (R + I) / 2).
    explicit AngleAxis(const Matrix<T, 3, 3>& R) {
        const double r00 = R(0, 0), r11 = R(1, 1), r22 = R(2, 2);
        const double c = std::max(-1.0, std::min(1.0, ((r00 + r11) + r22 - 1.0) * 0.5));
        const double a = std::acos(c);
        double x = R(2, 1) - R(1, 2), y = R(0, 2) - R(2, 0), z = R(1, 0) - R(0, 1);
        double n = std::sqrt(x * x + y * y + z * z);
        if (n < 1e-6) {
            if (a < 1e-3) {
                x = 1.0; y = 0.0; z = 0.0; n = 1.0;
            } else {
                const double xx = std::sqrt(std::max(0.0, (r00 + 1.0) * 0.5));
                const double yy = std::sqrt(std::max(0.0, (r11 + 1.0) * 0.5));
                const double zz = std::sqrt(std::max(0.0, (r22 + 1.0) * 0.5));
                if (xx >= yy && xx >= zz) {
                    x = xx; y = (R(0, 1) + R(1, 0)) / (4.0 * xx); z = (R(0, 2) + R(2, 0)) / (4.0 * xx);
                } else if (yy >= zz) {
                    y = yy; x = (R(0, 1) + R(1, 0)) / (4.0 * yy); z = (R(1, 2) + R(2, 1)) / (4.0 * yy);
                } else {
                    z = zz; x = (R(0, 2) + R(2, 0)) / (4.0 * zz); y = (R(1, 2) + R(2, 1)) / (4.0 * zz);
                }
                n = std::sqrt(x * x + y * y + z * z);
            }
        }
        angle_ = static_cast<T>(a);
        axis_ = Matrix<T, 3, 1>(static_cast<T>(x / n), static_cast<T>(y / n), static_cast<T>(z / n));
    }
    T angle() const { return angle_; }
    const Matrix<T, 3, 1>& axis() const { return axis_; }
    // Rodrigues, in the restatement's expression order (oracle/orc_icp.cpp angleAxis)
    Matrix<T, 3, 3> toRotationMatrix() const {
        const T s = std::sin(angle_), c = std::cos(angle_);
        const Matrix<T, 3, 1> sa = axis_ * s;
        const Matrix<T, 3, 1> ca = axis_ * (T(1) - c);
        Matrix<T, 3, 3> r;
        T tmp = ca.x() * axis_.y();
        r(0, 1) = tmp - sa.z();
        r(1, 0) = tmp + sa.z();
        tmp = ca.x() * axis_.z();
        r(0, 2) = tmp + sa.y();
        r(2, 0) = tmp - sa.y();
        tmp = ca.y() * axis_.z();
        r(1, 2) = tmp - sa.x();
        r(2, 1) = tmp + sa.x();
        r(0, 0) = ca.x() * axis_.x() + c;
        r(1, 1) = ca.y() * axis_.y() + c;
        r(2, 2) = ca.z() * axis_.z() + c;
        return r;
    }

private:
    T angle_;
    Matrix<T, 3, 1> axis_;
};

typedef AngleAxis<float> AngleAxisf;
typedef AngleAxis<double> AngleAxisd;

}  // namespace Eigen

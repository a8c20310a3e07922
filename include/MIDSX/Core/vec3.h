// vec3.h - the 3-vector of the MIDSX C++ API.
//
// The reference uses Eigen::Vector3d throughout its public API (e.g. include/MIDSX/Core/
// source.h, surface_tally.h, volume_tally.h).  This build has no Eigen dependency: Vec3 is a
// plain value type with the same construction and accessor forms (Vec3(x, y, z), v.x(),
// v(i), v.dot(w), v.cross(w), v.norm(), v.normalized()).  It converts from any type with
// x(), y(), z() accessors, so real Eigen vectors are accepted where Eigen is present; when
// Eigen is absent, Eigen::Vector3d names Vec3 so that reference-style code compiles as is.
#pragma once
#include <cmath>
#include <type_traits>
#include <utility>

namespace midsx {

class Vec3 {
public:
    Vec3() = default;
    Vec3(double x, double y, double z) : v_{x, y, z} {}
    template <typename V, typename = decltype(std::declval<const V&>().x()),
              typename = std::enable_if_t<!std::is_same<std::decay_t<V>, Vec3>::value>>
    Vec3(const V& o) : v_{double(o.x()), double(o.y()), double(o.z())} {}

    double x() const { return v_[0]; }
    double y() const { return v_[1]; }
    double z() const { return v_[2]; }
    double operator()(int i) const { return v_[i]; }
    double& operator()(int i) { return v_[i]; }
    double operator[](int i) const { return v_[i]; }
    double& operator[](int i) { return v_[i]; }
    const double* data() const { return v_; }

    Vec3 operator+(const Vec3& o) const { return {v_[0] + o.v_[0], v_[1] + o.v_[1], v_[2] + o.v_[2]}; }
    Vec3 operator-(const Vec3& o) const { return {v_[0] - o.v_[0], v_[1] - o.v_[1], v_[2] - o.v_[2]}; }
    Vec3 operator*(double s) const { return {v_[0] * s, v_[1] * s, v_[2] * s}; }
    Vec3 operator/(double s) const { return {v_[0] / s, v_[1] / s, v_[2] / s}; }
    Vec3& operator+=(const Vec3& o) {
        for (int i = 0; i < 3; ++i) v_[i] += o.v_[i];
        return *this;
    }
    bool operator==(const Vec3& o) const { return v_[0] == o.v_[0] && v_[1] == o.v_[1] && v_[2] == o.v_[2]; }
    double dot(const Vec3& o) const { return v_[0] * o.v_[0] + v_[1] * o.v_[1] + v_[2] * o.v_[2]; }
    Vec3 cross(const Vec3& o) const {
        return {v_[1] * o.v_[2] - v_[2] * o.v_[1], v_[2] * o.v_[0] - v_[0] * o.v_[2],
                v_[0] * o.v_[1] - v_[1] * o.v_[0]};
    }
    double norm() const { return std::sqrt(dot(*this)); }
    double squaredNorm() const { return dot(*this); }
    Vec3 normalized() const {
        double n = norm();
        return n > 0 ? *this / n : *this;
    }
    static Vec3 Zero() { return {0, 0, 0}; }
    static Vec3 UnitX() { return {1, 0, 0}; }
    static Vec3 UnitY() { return {0, 1, 0}; }
    static Vec3 UnitZ() { return {0, 0, 1}; }

private:
    double v_[3] = {0, 0, 0};
};

inline Vec3 operator*(double s, const Vec3& v) { return v * s; }

}  // namespace midsx

#if !defined(EIGEN_WORLD_VERSION) && !defined(MIDSX_NO_EIGEN_ALIAS)
namespace Eigen {
using Vector3d = ::midsx::Vec3;
}
#endif

using midsx::Vec3;

/*
 * TEST INFRASTRUCTURE — the two parsers CameraCalibration::deserialize and
 * StereoCameraCalibration::deserialize reference (defined in
 * cvt/math/Matrix.cpp, which needs Eigen's SVD and is not compiled).  The
 * rectification harness never deserializes; these only satisfy the linker.
 */
#include <cstring>
#include <stdexcept>

#include <cvt/math/Matrix.h>

namespace cvt {
template <>
Matrix3<float> Matrix3<float>::fromString(const String&) {
    throw std::runtime_error("Matrix3f::fromString is not part of the rectification harness");
}
template <>
Matrix4<float> Matrix4<float>::fromString(const String&) {
    throw std::runtime_error("Matrix4f::fromString is not part of the rectification harness");
}
}  // namespace cvt

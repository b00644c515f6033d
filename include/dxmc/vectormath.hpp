// dxmc/vectormath.hpp -- the 3-vector helpers OpenDXMC calls
// (dxmc_specialization.cpp:80-88, beamactorcontainer.cpp:44-67).
#pragma once

#include <array>
#include <cmath>

namespace dxmc::vectormath {

template <typename T>
std::array<T, 3> add(const std::array<T, 3>& a, const std::array<T, 3>& b) { return { a[0] + b[0], a[1] + b[1], a[2] + b[2] }; }

template <typename T>
std::array<T, 3> subtract(const std::array<T, 3>& a, const std::array<T, 3>& b) { return { a[0] - b[0], a[1] - b[1], a[2] - b[2] }; }

template <typename T>
std::array<T, 3> scale(const std::array<T, 3>& a, T s) { return { a[0] * s, a[1] * s, a[2] * s }; }

template <typename T>
T dot(const std::array<T, 3>& a, const std::array<T, 3>& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

template <typename T>
std::array<T, 3> cross(const std::array<T, 3>& a, const std::array<T, 3>& b)
{
    return { a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0] };
}

template <typename T>
T lenght_sqr(const std::array<T, 3>& a) { return dot(a, a); }

template <typename T>
T lenght(const std::array<T, 3>& a) { return std::sqrt(dot(a, a)); }

template <typename T>
std::array<T, 3> normalized(const std::array<T, 3>& a)
{
    const T n = lenght(a);
    return n > T { 0 } ? scale(a, T { 1 } / n) : a;
}

template <typename T>
void normalize(std::array<T, 3>& a) { a = normalized(a); }

// Rodrigues rotation of v about the unit vector k by `angle` radians (right-handed)
template <typename T>
std::array<T, 3> rotate(const std::array<T, 3>& v, const std::array<T, 3>& k, T angle)
{
    const T c = std::cos(angle), s = std::sin(angle);
    const auto kv = cross(k, v);
    const T kd = dot(k, v);
    return { v[0] * c + kv[0] * s + k[0] * kd * (1 - c), v[1] * c + kv[1] * s + k[1] * kd * (1 - c),
        v[2] * c + kv[2] * s + k[2] * kd * (1 - c) };
}

} // namespace dxmc::vectormath

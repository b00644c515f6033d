// dxmc/floating.hpp -- angle constants used by OpenDXMC (dxmc_specialization.cpp:62-76).
// Part of the header-only dxmc:: layer over the GB300 engine's C ABI (dxmcg.h).
#pragma once

namespace dxmc {

template <typename T = double>
constexpr T PI_VAL() { return T { 3.14159265358979323846264338327950288 }; }

template <typename T = double>
constexpr T DEG_TO_RAD() { return PI_VAL<T>() / T { 180 }; }

template <typename T = double>
constexpr T RAD_TO_DEG() { return T { 180 } / PI_VAL<T>(); }

} // namespace dxmc

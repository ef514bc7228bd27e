#pragma once
#include <cmath>
#include "ext/scalar_constants.hpp"
namespace glm {
template<typename T> inline T cos(T v) { return std::cos(v); }
template<typename T> inline T sin(T v) { return std::sin(v); }
template<typename T> constexpr T radians(T deg) { return deg * static_cast<T>(0.01745329251994329576923690768489); }
}

#pragma once
#include "shim_func.hpp"
#include <cmath>
#include "ext/scalar_constants.hpp"
namespace glm {
template<typename T> GLM_SHIM_FUNC inline T cos(T v) { return std::cos(v); }
template<typename T> GLM_SHIM_FUNC inline T sin(T v) { return std::sin(v); }
template<typename T> GLM_SHIM_FUNC constexpr T radians(T deg) { return deg * static_cast<T>(0.01745329251994329576923690768489); }
}

#pragma once
#include "shim_func.hpp"
#include "detail_vec.hpp"
#include "exponential.hpp"
#include "common.hpp"
// glm::dot and glm::length for two components as glm defines them
// (func_geometric: the products summed in component order; length = sqrt(dot))
namespace glm {
template<typename T> GLM_SHIM_FUNC inline T dot(const tvec2<T>& a, const tvec2<T>& b) { return a.x * b.x + a.y * b.y; }
template<typename T> GLM_SHIM_FUNC inline T length(const tvec2<T>& v) { return sqrt(dot(v, v)); }
}

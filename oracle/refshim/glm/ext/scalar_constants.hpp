#pragma once
#include "../shim_func.hpp"
namespace glm {
template<typename T> GLM_SHIM_FUNC constexpr T pi() { return static_cast<T>(3.14159265358979323846264338327950288); }
}

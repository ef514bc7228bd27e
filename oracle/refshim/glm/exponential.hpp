#pragma once
#include "shim_func.hpp"
#include <cmath>
namespace glm {
template<typename T> GLM_SHIM_FUNC inline T sqrt(T v) { return std::sqrt(v); }
}

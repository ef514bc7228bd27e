#pragma once
#include <cmath>
namespace glm {
template<typename T> inline T sqrt(T v) { return std::sqrt(v); }
}

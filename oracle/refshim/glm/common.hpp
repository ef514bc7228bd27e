#pragma once
#include "detail_vec.hpp"
// glm::mix as glm defines it (func_common: x * (1 - a) + y * a, per component
// for vectors with a scalar weight)
namespace glm {
template<typename T> inline T mix(T x, T y, T a) { return x * (static_cast<T>(1) - a) + y * a; }
template<typename T> inline tvec2<T> mix(const tvec2<T>& x, const tvec2<T>& y, T a) {
	return x * (static_cast<T>(1) - a) + y * a;
}
}

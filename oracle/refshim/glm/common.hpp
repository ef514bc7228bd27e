#pragma once
#include "shim_func.hpp"
#include "detail_vec.hpp"
// glm::mix as glm defines it (func_common: x * (1 - a) + y * a, per component
// for vectors with a scalar weight)
namespace glm {
template<typename T> GLM_SHIM_FUNC inline T mix(T x, T y, T a) { return x * (static_cast<T>(1) - a) + y * a; }
template<typename T> GLM_SHIM_FUNC inline tvec2<T> mix(const tvec2<T>& x, const tvec2<T>& y, T a) {
	return x * (static_cast<T>(1) - a) + y * a;
}
}
// glm::max of a vector and a scalar, per component (named by the reference's
// launch-configuration helper, STPDeviceLaunchSetup.inl)
namespace glm {
template<typename T> GLM_SHIM_FUNC inline tvec2<T> max(const tvec2<T>& v, T s) {
	return tvec2<T>(v.x < s ? s : v.x, v.y < s ? s : v.y);
}
template<typename T> GLM_SHIM_FUNC inline tvec3<T> max(const tvec3<T>& v, T s) {
	return tvec3<T>(v.x < s ? s : v.x, v.y < s ? s : v.y, v.z < s ? s : v.z);
}
}

// Minimal vector subset written for compiling a few SuperTerrain+ host sources
// without the glm library (test infrastructure for the oracle only).
#pragma once
#include "shim_func.hpp"
#include <cmath>
#include <cstddef>

// glm defines its version here; code that adapts to glm tests this macro
#ifndef GLM_VERSION
#define GLM_VERSION 0
#endif

namespace glm {

template<typename T> struct tvec2 {
	T x, y;
	GLM_SHIM_FUNC constexpr tvec2() : x(0), y(0) {}
	GLM_SHIM_FUNC constexpr explicit tvec2(T s) : x(s), y(s) {}
	GLM_SHIM_FUNC constexpr tvec2(T a, T b) : x(a), y(b) {}
	template<typename U> GLM_SHIM_FUNC constexpr explicit tvec2(const tvec2<U>& o) : x(static_cast<T>(o.x)), y(static_cast<T>(o.y)) {}
	GLM_SHIM_FUNC constexpr T& operator[](std::size_t i) { return i == 0 ? x : y; }
	GLM_SHIM_FUNC constexpr const T& operator[](std::size_t i) const { return i == 0 ? x : y; }
	GLM_SHIM_FUNC tvec2& operator+=(const tvec2& o) { x += o.x; y += o.y; return *this; }
	GLM_SHIM_FUNC tvec2& operator-=(const tvec2& o) { x -= o.x; y -= o.y; return *this; }
	GLM_SHIM_FUNC tvec2& operator*=(T s) { x *= s; y *= s; return *this; }
	GLM_SHIM_FUNC tvec2& operator/=(T s) { x /= s; y /= s; return *this; }
	template<typename U> GLM_SHIM_FUNC tvec2& operator+=(const tvec2<U>& o) { x += static_cast<T>(o.x); y += static_cast<T>(o.y); return *this; }
	template<typename U> GLM_SHIM_FUNC tvec2& operator*=(const tvec2<U>& o) { x *= static_cast<T>(o.x); y *= static_cast<T>(o.y); return *this; }
};
template<typename T> GLM_SHIM_FUNC constexpr tvec2<T> operator+(const tvec2<T>& a, const tvec2<T>& b) { return tvec2<T>(a.x + b.x, a.y + b.y); }
template<typename T> GLM_SHIM_FUNC constexpr tvec2<T> operator-(const tvec2<T>& a, const tvec2<T>& b) { return tvec2<T>(a.x - b.x, a.y - b.y); }
template<typename T> GLM_SHIM_FUNC constexpr tvec2<T> operator*(const tvec2<T>& a, const tvec2<T>& b) { return tvec2<T>(a.x * b.x, a.y * b.y); }
template<typename T> GLM_SHIM_FUNC constexpr tvec2<T> operator/(const tvec2<T>& a, const tvec2<T>& b) { return tvec2<T>(a.x / b.x, a.y / b.y); }
template<typename T> GLM_SHIM_FUNC constexpr tvec2<T> operator*(const tvec2<T>& a, T s) { return tvec2<T>(a.x * s, a.y * s); }
template<typename T> GLM_SHIM_FUNC constexpr tvec2<T> operator*(T s, const tvec2<T>& a) { return tvec2<T>(a.x * s, a.y * s); }
template<typename T> GLM_SHIM_FUNC constexpr tvec2<T> operator/(const tvec2<T>& a, T s) { return tvec2<T>(a.x / s, a.y / s); }
template<typename T> GLM_SHIM_FUNC constexpr tvec2<T> operator-(const tvec2<T>& a, T s) { return tvec2<T>(a.x - s, a.y - s); }
template<typename T> GLM_SHIM_FUNC constexpr tvec2<T> operator&(const tvec2<T>& a, const tvec2<T>& b) { return tvec2<T>(a.x & b.x, a.y & b.y); }
template<typename T> GLM_SHIM_FUNC constexpr bool operator==(const tvec2<T>& a, const tvec2<T>& b) { return a.x == b.x && a.y == b.y; }
template<typename T> GLM_SHIM_FUNC constexpr bool operator!=(const tvec2<T>& a, const tvec2<T>& b) { return !(a == b); }
template<typename T> GLM_SHIM_FUNC constexpr tvec2<T> operator-(const tvec2<T>& a) { return tvec2<T>(-a.x, -a.y); }

template<typename T> struct tvec3 {
	T x, y, z;
	GLM_SHIM_FUNC constexpr tvec3() : x(0), y(0), z(0) {}
	GLM_SHIM_FUNC constexpr explicit tvec3(T s) : x(s), y(s), z(s) {}
	GLM_SHIM_FUNC constexpr tvec3(T a, T b, T c) : x(a), y(b), z(c) {}
};

template<typename T> struct tvec4 {
	T x, y, z, w;
	GLM_SHIM_FUNC constexpr tvec4() : x(0), y(0), z(0), w(0) {}
	GLM_SHIM_FUNC constexpr explicit tvec4(T s) : x(s), y(s), z(s), w(s) {}
	GLM_SHIM_FUNC constexpr tvec4(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
};

typedef tvec2<float> vec2;
typedef tvec2<double> dvec2;
typedef tvec2<unsigned int> uvec2;
typedef tvec2<int> ivec2;
typedef tvec3<float> vec3;
typedef tvec3<double> dvec3;
typedef tvec3<unsigned int> uvec3;
typedef tvec3<int> ivec3;
typedef tvec4<float> vec4;

} // namespace glm

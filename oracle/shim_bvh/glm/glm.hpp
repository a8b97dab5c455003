/*
 * glm stand-in for compiling the reference's source/bvh.cpp on the host
 * (TEST INFRASTRUCTURE; glm is an empty submodule in the reference
 * checkout).  What bvh.cpp computes with is real: vec3 and vec4 with
 * component access, glm::min / glm::max componentwise as glm defines them
 * ((y < x) ? y : x and (x < y) ? y : x).  The rest -- matrices, quaternions,
 * the transform helpers -- only has to compile, because include/transform.hpp
 * (included by include/bbox.hpp) names them in inline members the builder
 * never calls; those return zeros.
 */
#pragma once

#include <cmath>
#include <string>

namespace glm {

struct vec4;

struct vec3 {
	float x, y, z;
	vec3() : x(0), y(0), z(0) {}
	explicit vec3(float s) : x(s), y(s), z(s) {}
	vec3(float a, float b, float c) : x(a), y(b), z(c) {}
	vec3(const vec4 &v);
	float &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
	float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
	vec3 &operator+=(const vec3 &o)
	{
		x += o.x;
		y += o.y;
		z += o.z;
		return *this;
	}
	bool operator==(const vec3 &o) const { return x == o.x && y == o.y && z == o.z; }
};

struct vec4 {
	float x, y, z, w;
	vec4() : x(0), y(0), z(0), w(0) {}
	explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
	vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
	vec4(const vec3 &v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
	float &operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
	float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};

inline vec3::vec3(const vec4 &v) : x(v.x), y(v.y), z(v.z) {}

struct uvec4 {
	unsigned x, y, z, w;
};

struct mat4 {
	vec4 c[4];
	mat4() {}
	explicit mat4(float) {}
	vec4 &operator[](int i) { return c[i]; }
	const vec4 &operator[](int i) const { return c[i]; }
};

struct quat {
	float x, y, z, w;
	quat() : x(0), y(0), z(0), w(1) {}
	explicit quat(const vec3 &) : x(0), y(0), z(0), w(1) {}
};

inline vec3 min(const vec3 &a, const vec3 &b)
{
	return vec3(b.x < a.x ? b.x : a.x, b.y < a.y ? b.y : a.y, b.z < a.z ? b.z : a.z);
}
inline vec3 max(const vec3 &a, const vec3 &b)
{
	return vec3(a.x < b.x ? b.x : a.x, a.y < b.y ? b.y : a.y, a.z < b.z ? b.z : a.z);
}

/* compiled, never called by the builder */
inline float length(const vec3 &) { return 0.0f; }
inline vec3 normalize(const vec3 &) { return vec3(); }
inline vec3 degrees(const vec3 &) { return vec3(); }
inline vec3 radians(const vec3 &) { return vec3(); }
inline mat4 translate(const mat4 &, const vec3 &) { return mat4(); }
inline mat4 scale(const mat4 &, const vec3 &) { return mat4(); }
inline mat4 mat4_cast(const quat &) { return mat4(); }
inline vec3 eulerAngles(const quat &) { return vec3(); }
inline quat quatLookAt(const vec3 &, const vec3 &) { return quat(); }
inline std::string to_string(const mat4 &) { return std::string(); }
inline mat4 operator*(const mat4 &, const mat4 &) { return mat4(); }
inline vec4 operator*(const mat4 &, const vec4 &) { return vec4(); }
inline vec4 operator*(const quat &, const vec4 &) { return vec4(); }

} /* namespace glm */

/*
 * glm stand-in for compiling the reference's path-tracer programs on the
 * host (TEST INFRASTRUCTURE; glm is an empty submodule in the reference
 * checkout).  It restates what glm publishes for the operations those
 * programs and their headers evaluate, in glm's order of operations:
 *   vector +, -, +=, * and / componentwise, with a scalar on either side;
 *   isnan and any componentwise;
 *   dot(a, b) = (a.x * b.x + a.y * b.y) + a.z * b.z (the product vector
 *     summed left to right; two components for vec2);
 *   cross(x, y) = (x.y y.z - y.y x.z, x.z y.x - y.z x.x, x.x y.y - y.x x.y);
 *   normalize(v) = v * (1 / sqrt(dot(v, v)))  (inversesqrt is 1 / sqrt);
 *   length(v) = sqrt(dot(v, v));
 *   min / max componentwise as (y < x) ? y : x and (x < y) ? y : x;
 *   mat4 * vec4 = (m[0] v.x + m[1] v.y) + (m[2] v.z + m[3] v.w), columns
 *     m[i], each m[i] v_i componentwise.
 * Matrices hold columns.  The quaternion, transform and string helpers
 * that include/transform.hpp names in inline members the programs never
 * call return zeros.
 */
#pragma once

#include <cmath>
#include <string>

namespace glm {

struct vec4;

struct vec2 {
	float x, y;
	vec2() : x(0), y(0) {}
	explicit vec2(float s) : x(s), y(s) {}
	vec2(float a, float b) : x(a), y(b) {}
	float &operator[](int i) { return i == 0 ? x : y; }
	float operator[](int i) const { return i == 0 ? x : y; }
};

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
	vec4 &operator+=(const vec4 &o)
	{
		x += o.x;
		y += o.y;
		z += o.z;
		w += o.w;
		return *this;
	}
};

struct bvec4 {
	bool x, y, z, w;
};
inline bvec4 isnan(const vec4 &v) { return bvec4{std::isnan(v.x), std::isnan(v.y), std::isnan(v.z), std::isnan(v.w)}; }
inline bool any(const bvec4 &b) { return b.x || b.y || b.z || b.w; }

inline vec3::vec3(const vec4 &v) : x(v.x), y(v.y), z(v.z) {}

struct uvec3 {
	unsigned x, y, z;
};
struct uvec4 {
	unsigned x, y, z, w;
};
struct ivec2 {
	int x, y;
};

inline vec2 operator+(const vec2 &a, const vec2 &b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator-(const vec2 &a, const vec2 &b) { return vec2(a.x - b.x, a.y - b.y); }
inline vec2 operator*(float s, const vec2 &a) { return vec2(s * a.x, s * a.y); }
inline vec2 operator*(const vec2 &a, float s) { return vec2(a.x * s, a.y * s); }

inline vec3 operator+(const vec3 &a, const vec3 &b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3 &a, const vec3 &b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator-(const vec3 &a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3 operator*(float s, const vec3 &a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator*(const vec3 &a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(const vec3 &a, const vec3 &b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator/(const vec3 &a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }

inline vec4 operator+(const vec4 &a, const vec4 &b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline vec4 operator*(const vec4 &a, float s) { return vec4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline vec4 operator*(float s, const vec4 &a) { return vec4(s * a.x, s * a.y, s * a.z, s * a.w); }
inline vec4 operator/(const vec4 &a, float s) { return vec4(a.x / s, a.y / s, a.z / s, a.w / s); }

inline float dot(const vec2 &a, const vec2 &b) { return a.x * b.x + a.y * b.y; }
inline float length(const vec2 &v) { return std::sqrt(dot(v, v)); }

inline float dot(const vec3 &a, const vec3 &b)
{
	vec3 t = a * b;
	return t.x + t.y + t.z;
}
inline vec3 cross(const vec3 &x, const vec3 &y)
{
	return vec3(x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y);
}
inline float inversesqrt(float x) { return 1.0f / std::sqrt(x); }
inline vec3 normalize(const vec3 &v) { return v * inversesqrt(dot(v, v)); }
inline float length(const vec3 &v) { return std::sqrt(dot(v, v)); }
inline vec3 min(const vec3 &a, const vec3 &b)
{
	return vec3(b.x < a.x ? b.x : a.x, b.y < a.y ? b.y : a.y, b.z < a.z ? b.z : a.z);
}
inline vec3 max(const vec3 &a, const vec3 &b)
{
	return vec3(a.x < b.x ? b.x : a.x, a.y < b.y ? b.y : a.y, a.z < b.z ? b.z : a.z);
}

struct mat4 {
	vec4 c[4];
	mat4() {}
	explicit mat4(float s)
	{
		c[0] = vec4(s, 0, 0, 0);
		c[1] = vec4(0, s, 0, 0);
		c[2] = vec4(0, 0, s, 0);
		c[3] = vec4(0, 0, 0, s);
	}
	vec4 &operator[](int i) { return c[i]; }
	const vec4 &operator[](int i) const { return c[i]; }
};

inline vec4 operator*(const mat4 &m, const vec4 &v)
{
	vec4 add0 = m[0] * v.x + m[1] * v.y;
	vec4 add1 = m[2] * v.z + m[3] * v.w;
	return add0 + add1;
}

struct quat {
	float x, y, z, w;
	quat() : x(0), y(0), z(0), w(1) {}
	explicit quat(const vec3 &) : x(0), y(0), z(0), w(1) {}
};

/* compiled, never called by the programs */
inline vec3 degrees(const vec3 &) { return vec3(); }
inline vec3 radians(const vec3 &) { return vec3(); }
inline mat4 translate(const mat4 &, const vec3 &) { return mat4(); }
inline mat4 scale(const mat4 &, const vec3 &) { return mat4(); }
inline mat4 mat4_cast(const quat &) { return mat4(); }
inline vec3 eulerAngles(const quat &) { return vec3(); }
inline quat quatLookAt(const vec3 &, const vec3 &) { return quat(); }
inline std::string to_string(const mat4 &) { return std::string(); }
inline mat4 operator*(const mat4 &, const mat4 &) { return mat4(); }
inline vec4 operator*(const quat &, const vec4 &) { return vec4(); }

} /* namespace glm */

/*
 * ref_glsl.cpp -- the reference's GLSL traversal compiled as C++, for
 * known-answer vectors of the threaded-BVH walk.
 *
 * TEST INFRASTRUCTURE.  Compiled by oracle/Makefile (target `ref`) against
 * the reference sources where they lie (REFERENCE=<path>), into
 * oracle/_ref/ref_glsl, with g++ -std=c++20 -fsingle-precision-constant
 * -ffp-contract=off.  It includes, unmodified:
 *   shaders/rt/modules/ray.glsl         Ray
 *   shaders/rt/modules/primitives.glsl  Triangle, Sphere
 *   shaders/rt/modules/bbox.glsl        BoundingBox, intersect_box, in_box
 *   shaders/rt/modules/intersect.glsl   _intersect_t, intersect_shape,
 *                                       ray_intersect (and include/types.hpp)
 *   shaders/rt/modules/bvh.glsl         hit/miss/object/id/leaf/bbox, trace
 * The GLSL built-ins they use are supplied here as plain C++ (vector types
 * with the swizzles the files read, dot, cross, normalize, lessThan, any,
 * floatBitsToInt/Uint); so are the declarations of layouts.glsl that
 * cannot compile as C++ (the storage buffers, Material and def_mat(),
 * AreaLight), a zero area-light count, and stand-ins for the texture
 * lookups of material and environment, which the traversal's hit does not
 * depend on.  -fsingle-precision-constant keeps GLSL's float literals
 * (1.0 / divisor is a float division there).  GLSL leaves the order of
 * dot's additions to the implementation; here it is (x + y) + z.
 *
 * Input on stdin (little endian): uint32 vertex_count, triangle_count,
 * bvh_vec4_count, ray_count; float positions[3 * V]; uint32 tris[4 * T];
 * float bvh[4 * B]; float rays[6 * R] ({origin, direction}).  Output on
 * stdout: one line per ray, "object time_bits" (time as the hex bits of
 * the float).
 */
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

typedef unsigned int uint;

struct vec2 {
	float x, y;
	vec2() = default;
	explicit vec2(float s) : x(s), y(s) {}
	vec2(float a, float b) : x(a), y(b) {}
};

struct vec3 {
	float x, y, z;
	vec3() = default;
	explicit vec3(float s) : x(s), y(s), z(s) {}
	vec3(float a, float b, float c) : x(a), y(b), z(c) {}
};

/* swizzle views of a vec4 (members of its union, so without constructors) */
struct vec3_view {
	float x, y, z;
	operator vec3() const { return vec3(x, y, z); }
};
struct vec2_view {
	float x, y;
	operator vec2() const { return vec2(x, y); }
};

struct vec4 {
	union {
		struct {
			float x, y, z, w;
		};
		struct {
			vec3_view xyz;
			float w_;
		};
		struct {
			vec3_view rgb;
			float a_;
		};
		struct {
			vec2_view xy;
			vec2_view zw;
		};
	};
	vec4() : x(0), y(0), z(0), w(0) {}
	explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
};

struct uvec4 {
	uint x, y, z, w;
};

struct bvec3 {
	bool x, y, z;
};

inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator-(vec3 a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3 operator*(vec3 a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, vec3 a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator*(int s, vec3 a) { return (float)s * a; }
inline vec3 operator-(vec3 a, int s) { return vec3(a.x - (float)s, a.y - (float)s, a.z - (float)s); }
inline vec2 operator*(vec2 a, float s) { return vec2(a.x * s, a.y * s); }
inline vec2 operator+(vec2 a, vec2 b) { return vec2(a.x + b.x, a.y + b.y); }
inline float dot(vec3 a, vec3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline vec3 cross(vec3 a, vec3 b)
{
	return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline float length(vec3 a) { return sqrtf(dot(a, a)); }
inline vec3 normalize(vec3 a) { return a * (1.0f / length(a)); }
inline bvec3 lessThan(vec3 a, vec3 b) { return bvec3{a.x < b.x, a.y < b.y, a.z < b.z}; }
inline bvec3 greaterThan(vec3 a, vec3 b) { return bvec3{a.x > b.x, a.y > b.y, a.z > b.z}; }
inline bool any(bvec3 b) { return b.x || b.y || b.z; }
inline int floatBitsToInt(float f)
{
	int i;
	memcpy(&i, &f, 4);
	return i;
}
inline uvec4 floatBitsToUint(vec4 v)
{
	uvec4 u;
	memcpy(&u, &v, 16);
	return u;
}
inline float atan(float y, float x) { return atan2f(y, x); }
/* GLSL min/max of floats: y < x ? y : x, x < y ? y : x */
inline float min(float x, float y) { return y < x ? y : x; }
inline float max(float x, float y) { return x < y ? y : x; }

struct mat3 {
	vec3 c0, c1, c2;
	mat3(vec3 a, vec3 b, vec3 c) : c0(a), c1(b), c2(c) {}
};
inline vec3 operator*(mat3 m, vec3 v) { return m.c0 * v.x + m.c1 * v.y + m.c2 * v.z; }

const float PI = 3.14159265358979323846f;
const int SHADING_EMISSIVE = 1 << 5;

/* layouts.glsl's declarations, as C++ */
struct Material {
	vec3 diffuse;
	vec3 specular;
	vec3 emission;
	vec3 ambient;
	float shininess;
	float roughness;
	float refraction;
	int albedo;
	int normal;
	int type;
};

Material def_mat()
{
	Material m;
	m.diffuse = vec3(0.0);
	m.specular = vec3(0.0);
	m.emission = vec3(0.0);
	m.ambient = vec3(0.0);
	m.shininess = 0.0;
	m.roughness = 0.0;
	m.refraction = 0.0;
	m.albedo = 0;
	m.normal = 0;
	m.type = 0;
	return m;
}

struct AreaLight {
	vec3 a;
	vec3 ab;
	vec3 ac;
	vec3 color;
	float power;
};

struct Buffer {
	vec4 *data;
};
Buffer vertices, triangles, bvh;
struct {
	int count;
	AreaLight data[1];
} area_lights = {0, {}};
struct {
	int triangles;
} pc = {0};

/* texture lookups: material and environment colours (not part of the hit) */
struct sampler2D {
	int unused;
};
sampler2D s2_albedo[1], s2_normals[1];
inline vec4 texture(sampler2D, vec2) { return vec4(0.0); }
inline Material get_material(uint, vec2) { return def_mat(); }

#include "shaders/rt/modules/ray.glsl"
#include "shaders/rt/modules/primitives.glsl"
#include "shaders/rt/modules/bbox.glsl"

inline vec3 sample_environment(Ray) { return vec3(0.0); }

#include "shaders/rt/modules/intersect.glsl"
#include "shaders/rt/modules/bvh.glsl"

int main()
{
	uint32_t h[4];
	if (fread(h, 4, 4, stdin) != 4)
		return 1;
	uint32_t V = h[0], T = h[1], B = h[2], R = h[3];
	std::vector<float> pos(3 * (size_t)V), rays(6 * (size_t)R);
	std::vector<uint32_t> tris(4 * (size_t)T);
	std::vector<vec4> vbuf(5 * (size_t)V), tbuf(T), bbuf(B);
	std::vector<float> braw(4 * (size_t)B);
	if (fread(pos.data(), 4, pos.size(), stdin) != pos.size() || fread(tris.data(), 4, tris.size(), stdin) != tris.size()
		|| fread(braw.data(), 4, braw.size(), stdin) != braw.size() || fread(rays.data(), 4, rays.size(), stdin) != rays.size())
		return 1;
	/* vertices.data[5 i] = position (VERTEX_STRIDE = 5, include/types.hpp) */
	for (uint32_t i = 0; i < V; i++) {
		vbuf[5 * (size_t)i].x = pos[3 * (size_t)i];
		vbuf[5 * (size_t)i].y = pos[3 * (size_t)i + 1];
		vbuf[5 * (size_t)i].z = pos[3 * (size_t)i + 2];
	}
	for (uint32_t t = 0; t < T; t++)
		memcpy(&tbuf[t], &tris[4 * (size_t)t], 16);
	for (uint32_t b = 0; b < B; b++)
		memcpy(&bbuf[b], &braw[4 * (size_t)b], 16);
	vertices.data = vbuf.data();
	triangles.data = tbuf.data();
	bvh.data = bbuf.data();
	for (uint32_t r = 0; r < R; r++) {
		const float *q = &rays[6 * (size_t)r];
		Ray ray = Ray(vec3(q[0], q[1], q[2]), vec3(q[3], q[4], q[5]), 1.0, 1.0);
		Hit hit = trace(ray);
		uint32_t bits;
		memcpy(&bits, &hit.time, 4);
		printf("%d %08x\n", hit.object, bits);
	}
	return 0;
}

/*
 * ref_optix_host.h -- what the host harnesses of the reference's OptiX
 * programs share (TEST INFRASTRUCTURE; oracle/ref_pt.cpp for the path
 * tracer, oracle/ref_restir.cpp for ReSTIR DI).
 *
 * Include order: this header, then the harness's launch-parameter struct
 * (with the reference's member names and types), then the program file
 * under source/optix; then define program_closesthit() and
 * program_miss(index), and call host_scene_build() before the first trace.
 *
 * What stands in for what a host cannot compile:
 *   - the OptiX device calls.  optixTrace finds the hit with the oracle's
 *     walk (itself checked against shaders/rt/modules/bvh.glsl compiled on
 *     the host) and then runs the closest-hit program, or the miss program
 *     of the call's miss index; the shadow rays (no closest-hit program)
 *     run only their miss program.  The getters read a stack of per-call
 *     states, so that the recursive closest-hit program sees its own ray;
 *   - glm (an empty submodule in the checkout): oracle/shim_pt restates
 *     glm's published formulas;
 *   - include/amadeus/armada.cuh and include/vertex.hpp pull in the Vulkan
 *     engine: their include guards are defined here, and Vertex is
 *     declared with the reference's member names and types;
 *   - __sinf, __cosf, __tanf, sinf, cosf, sin, cos, tanf, atanf, acosf,
 *     asinf and powf map to the oracle's specification of the reference's
 *     fast intrinsics (oracle/ref_math.h; powf with exponent 2, 4 or 5 as
 *     repeated multiplication), the same functions the oracle and the
 *     kernels use, so that the images can agree to rounding; printf is
 *     silenced (the reference's ray-generation programs print);
 *   - tex2D: the texture unit's read of the environment map (normalised
 *     coordinates, wrap addressing, the given filter) is the oracle's
 *     reading of the CUDA texture rules (oracle_env_lookup); the scenes
 *     have no material textures.
 */
#ifndef KGR_ORACLE_REF_OPTIX_HOST_H_
#define KGR_ORACLE_REF_OPTIX_HOST_H_

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include <texture_types.h>
#include <vector_functions.h>
#include <vector_types.h>

#include "oracle.h"
#include "ref_math.h"

using std::abs;
using std::fmax;
using std::fmaxf;
using std::fminf;
using std::sqrt;

/* CUDA qualifiers on the host */
#define __forceinline__ inline
#define __device__
#define __global__
#define __constant__
#define __host__
#define __align__(n) alignas(n)

/* the oracle's specification of the fast intrinsics */
inline float ref_powf(float x, float y)
{
	if (y == 2.0f)
		return oref::kpow2(x);
	if (y == 4.0f)
		return oref::kpow4(x);
	if (y == 5.0f)
		return oref::kpow5(x);
	return powf(x, y);
}
#define __sinf oref::ksin
#define __cosf oref::kcos
#define __tanf oref::ktan
#define sinf oref::ksin
#define cosf oref::kcos
#define sin oref::ksin
#define cos oref::kcos
#define tanf oref::ktan
#define atanf oref::katan
#define acosf oref::kacos
#define asinf oref::kasin
#define powf ref_powf

inline float min(float a, float b) { return a < b ? a : b; }

/* the environment map, read through the texture rules of the oracle */
static std::vector<float> g_env;
static uint32_t g_env_w = 0, g_env_h = 0;
static int g_env_filter = 0;

template <class T>
T tex2D(cudaTextureObject_t, float u, float v)
{
	float uv[2] = {u, v}, rgb[3] = {0.0f, 0.0f, 0.0f};
	if (g_env_w)
		oracle_env_lookup(g_env.data(), g_env_w, g_env_h, g_env_filter, uv, 1, rgb);
	T t = T();
	t.x = rgb[0];
	t.y = rgb[1];
	t.z = rgb[2];
	return t;
}

/* the OptiX host header: types, flags and the host API */
#include <optix.h>
#include <optix_function_table_definition.h>

/* the OptiX device calls the programs make, over a stack of per-call states */
struct TraceCall {
	float3 direction;
	unsigned int p0, p1;
	unsigned int prim;
	float2 bary;
	const void *sbt;
};
static std::vector<TraceCall> g_calls;
static uint3 g_launch;

inline uint3 optixGetLaunchIndex() { return g_launch; }
inline unsigned int optixGetPayload_0() { return g_calls.back().p0; }
inline unsigned int optixGetPayload_1() { return g_calls.back().p1; }
inline float3 optixGetWorldRayDirection() { return g_calls.back().direction; }
inline float2 optixGetTriangleBarycentrics() { return g_calls.back().bary; }
inline unsigned int optixGetPrimitiveIndex() { return g_calls.back().prim; }
inline CUdeviceptr optixGetSbtDataPointer() { return (CUdeviceptr)(uintptr_t)g_calls.back().sbt; }
void optixTrace(OptixTraversableHandle handle, float3 origin, float3 direction, float tmin, float tmax, float time,
		OptixVisibilityMask mask, unsigned int flags, unsigned int sbt_offset, unsigned int sbt_stride,
		unsigned int miss_index, unsigned int &p0, unsigned int &p1);

/* the harness's programs (defined after it includes the program file) */
void program_closesthit();
void program_miss(unsigned int miss_index);

/* printf of the reference's ray-generation programs */
#define printf(...) ((void)0)

/* the reference's own headers the programs include */
#include "include/cuda/cast.cuh"
#include "include/cuda/material.cuh"
#include "include/optix/lighting.cuh"

/* include/vertex.hpp (Vulkan vertex descriptions around it): the vertex */
#define VERTEX_H_
namespace kobra {
struct Vertex {
	glm::vec3 position;
	glm::vec3 normal;
	glm::vec2 tex_coords;
	glm::vec3 tangent;
	glm::vec3 bitangent;
};
} /* namespace kobra */

/* include/amadeus/armada.cuh: its launch information is restated by each
 * harness in its parameter struct */
#define KOBRA_AMADEUS_ARMADA_H_

/* the hit records (OptiX's shader-binding-table data) */
#include "include/optix/sbt.cuh"

/* ---------------------------------------------------------- the scene -- */

/* The oracle's scene (its generator, SAH BVH with leaves of 4, lights), and
 * the reference's view of it: vertices, one hit record a material with the
 * identity model (OptiX's submeshes), materials and triangle lights. */
struct HostScene {
	oracle_generated *gen = nullptr;
	oracle_scene_arrays a;
	std::vector<uint32_t> tris;
	std::vector<float> bvh;
	std::vector<kgr_triangle_light> lights;
	std::vector<kobra::Vertex> vertices;
	std::vector<std::vector<glm::uvec3>> tri_lists;
	std::vector<kobra::cuda::_material> materials;
	std::vector<kobra::optix::TriangleLight> tri_lights;
	float center[3], ax_u[3], ax_v[3], ax_w[3];
};

static oracle_scene g_scene;
static std::vector<kobra::optix::Hit> g_records;
static std::vector<std::pair<uint32_t, uint32_t>> g_where;

void optixTrace(OptixTraversableHandle, float3 origin, float3 direction, float tmin, float tmax, float,
		OptixVisibilityMask, unsigned int flags, unsigned int, unsigned int, unsigned int miss_index,
		unsigned int &p0, unsigned int &p1)
{
	(void)tmin; /* 0 in every call the programs make, the walk's own lower bound */
	float ray[8] = {origin.x, origin.y, origin.z, 0.0f, direction.x, direction.y, direction.z, tmax};
	TraceCall call = {direction, p0, p1, 0, make_float2(0.0f, 0.0f), nullptr};
	if (flags & OPTIX_RAY_FLAG_DISABLE_CLOSESTHIT) {
		uint32_t occluded = 0;
		oracle_trace_any(&g_scene, ray, 1, &occluded, nullptr, 1);
		if (!occluded) {
			g_calls.push_back(call);
			program_miss(miss_index);
			g_calls.pop_back();
		}
		return;
	}
	kgr_hit h;
	oracle_trace_closest(&g_scene, ray, 1, &h, nullptr, 1);
	if (h.prim >= 0) {
		call.prim = g_where[(uint32_t)h.prim].second;
		call.bary = make_float2(h.b1, h.b2);
		call.sbt = &g_records[g_where[(uint32_t)h.prim].first];
		g_calls.push_back(call);
		program_closesthit();
	} else {
		g_calls.push_back(call);
		program_miss(miss_index);
	}
	g_calls.pop_back();
}

/* Read an environment file: uint32 width, height, then width * height RGBA
 * float32 texels, row 0 first. */
inline bool host_load_environment(const char *path, int filter)
{
	FILE *f = fopen(path, "rb");
	uint32_t wh[2];
	if (!f || fread(wh, 4, 2, f) != 2)
		return false;
	g_env.resize(4 * (size_t)wh[0] * wh[1]);
	bool ok = fread(g_env.data(), 4, g_env.size(), f) == g_env.size();
	fclose(f);
	g_env_w = wh[0];
	g_env_h = wh[1];
	g_env_filter = filter;
	return ok;
}

/* quad lights, in the oracle's form and the reference's */
static std::vector<kgr_quad_light> g_quads;
static std::vector<kobra::optix::QuadLight> g_quad_lights;

/* Read a quad-light file: uint32 count, then count x 12 float32 {a, ab, ac,
 * intensity}. */
inline bool host_load_quads(const char *path)
{
	FILE *f = fopen(path, "rb");
	uint32_t n;
	if (!f || fread(&n, 4, 1, f) != 1)
		return false;
	g_quads.resize(n);
	bool ok = fread(g_quads.data(), sizeof(kgr_quad_light), n, f) == n;
	fclose(f);
	g_quad_lights.resize(n);
	for (uint32_t i = 0; i < n; i++) {
		const kgr_quad_light &q = g_quads[i];
		g_quad_lights[i].a = make_float3(q.a[0], q.a[1], q.a[2]);
		g_quad_lights[i].ab = make_float3(q.ab[0], q.ab[1], q.ab[2]);
		g_quad_lights[i].ac = make_float3(q.ac[0], q.ac[1], q.ac[2]);
		g_quad_lights[i].intensity = make_float3(q.intensity[0], q.intensity[1], q.intensity[2]);
	}
	return ok;
}

/* Options after the positional arguments: --env <file> <filter> (uint32
 * width, height, then width * height RGBA float32 texels, row 0 first;
 * filter 0 linear, 1 point) and --quads <file>.  Returns false on a bad
 * option or file. */
inline bool host_options(int argc, char **argv, int first)
{
	for (int i = first; i < argc; i++) {
		if (!strcmp(argv[i], "--env") && i + 2 < argc) {
			if (!host_load_environment(argv[i + 1], atoi(argv[i + 2])))
				return false;
			i += 2;
		} else if (!strcmp(argv[i], "--quads") && i + 1 < argc) {
			if (!host_load_quads(argv[i + 1]))
				return false;
			i += 1;
		} else {
			return false;
		}
	}
	return true;
}

inline bool host_scene_build(HostScene &hs, const char *name, uint64_t seed, uint32_t W, uint32_t H)
{
	if (oracle_generate_scene(name, seed, &hs.gen) != 0)
		return false;
	oracle_scene_arrays &a = hs.a;
	oracle_generated_view(hs.gen, &a);
	hs.tris.resize(4 * (size_t)a.triangle_count);
	for (uint32_t t = 0; t < a.triangle_count; t++) {
		for (int k = 0; k < 3; k++)
			hs.tris[4 * (size_t)t + k] = a.indices[3 * (size_t)t + k];
		hs.tris[4 * (size_t)t + 3] = a.material_indices[t];
	}
	int64_t nb = oracle_build_sah(a.positions, a.indices, a.triangle_count, 4, nullptr, 0);
	hs.bvh.resize(4 * (size_t)nb);
	oracle_build_sah(a.positions, a.indices, a.triangle_count, 4, hs.bvh.data(), (uint64_t)nb);
	uint32_t nl = oracle_scene_lights(a.positions, a.indices, a.material_indices, a.triangle_count, a.materials,
		nullptr);
	hs.lights.resize(nl);
	oracle_scene_lights(a.positions, a.indices, a.material_indices, a.triangle_count, a.materials, hs.lights.data());
	memset(&g_scene, 0, sizeof(g_scene));
	g_scene.positions = a.positions;
	g_scene.normals = a.normals;
	g_scene.tris = hs.tris.data();
	g_scene.materials = a.materials;
	g_scene.lights = hs.lights.data();
	g_scene.bvh = hs.bvh.data();
	g_scene.vertex_count = a.vertex_count;
	g_scene.triangle_count = a.triangle_count;
	g_scene.material_count = a.material_count;
	g_scene.light_count = nl;
	g_scene.bvh_vec4_count = (uint32_t)nb;
	if (g_env_w) {
		g_scene.env = g_env.data();
		g_scene.env_width = g_env_w;
		g_scene.env_height = g_env_h;
		g_scene.env_filter = g_env_filter;
	}
	if (!g_quads.empty()) {
		g_scene.quads = g_quads.data();
		g_scene.quad_count = (uint32_t)g_quads.size();
	}

	hs.vertices.resize(a.vertex_count);
	for (uint32_t v = 0; v < a.vertex_count; v++) {
		const float *p = a.positions + 3 * (size_t)v, *n = a.normals + 3 * (size_t)v;
		hs.vertices[v].position = glm::vec3(p[0], p[1], p[2]);
		hs.vertices[v].normal = glm::vec3(n[0], n[1], n[2]);
	}
	hs.tri_lists.assign(a.material_count, {});
	g_where.resize(a.triangle_count);
	for (uint32_t t = 0; t < a.triangle_count; t++) {
		uint32_t m = a.material_indices[t];
		g_where[t] = {m, (uint32_t)hs.tri_lists[m].size()};
		hs.tri_lists[m].push_back(glm::uvec3{a.indices[3 * (size_t)t], a.indices[3 * (size_t)t + 1],
			a.indices[3 * (size_t)t + 2]});
	}
	g_records.resize(a.material_count);
	for (uint32_t m = 0; m < a.material_count; m++) {
		memset(&g_records[m], 0, sizeof(kobra::optix::Hit));
		g_records[m].vertices = hs.vertices.data();
		g_records[m].model = glm::mat4(1.0f);
		g_records[m].triangles = hs.tri_lists[m].data();
		g_records[m].light_index = -1;
		g_records[m].material_index = m;
	}
	hs.materials.resize(a.material_count);
	for (uint32_t m = 0; m < a.material_count; m++) {
		const kgr_material &s = a.materials[m];
		kobra::cuda::_material &d = hs.materials[m];
		d.diffuse = make_float3(s.diffuse[0], s.diffuse[1], s.diffuse[2]);
		d.specular = make_float3(s.specular[0], s.specular[1], s.specular[2]);
		d.emission = make_float3(s.emission[0], s.emission[1], s.emission[2]);
		d.ambient = make_float3(s.ambient[0], s.ambient[1], s.ambient[2]);
		d.shininess = s.shininess;
		d.roughness = s.roughness;
		d.refraction = s.refraction;
		d.type = (Shading)s.type;
	}
	hs.tri_lights.resize(nl);
	for (uint32_t l = 0; l < nl; l++) {
		const kgr_triangle_light &s = hs.lights[l];
		hs.tri_lights[l].a = make_float3(s.a[0], s.a[1], s.a[2]);
		hs.tri_lights[l].ab = make_float3(s.ab[0], s.ab[1], s.ab[2]);
		hs.tri_lights[l].ac = make_float3(s.ac[0], s.ac[1], s.ac[2]);
		hs.tri_lights[l].intensity = make_float3(s.intensity[0], s.intensity[1], s.intensity[2]);
	}
	const float up[3] = {0.0f, 1.0f, 0.0f};
	oracle_camera(a.eye, a.target, up, a.fov_deg, (float)W / (float)H, hs.center, hs.ax_u, hs.ax_v, hs.ax_w);
	return true;
}

/* the logger that include/logger.hpp declares, as a plain stream */
#include "include/logger.hpp"
namespace kobra {
namespace detail {
std::map<void *, LogHandler> log_handlers;
}
detail::LogStream &logger(const std::string &, Log, const std::string &, bool)
{
	static detail::LogStream stream(std::cerr);
	return stream;
}
} /* namespace kobra */

#endif

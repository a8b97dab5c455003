/*
 * ref_pt.cpp -- the reference's path-tracer programs compiled on the host,
 * for known-answer images of the integrator.
 *
 * TEST INFRASTRUCTURE.  Compiled by oracle/Makefile (target `ref`) against
 * the reference sources where they lie (REFERENCE=<path>) and the oracle
 * library, into oracle/_ref/ref_pt.  It includes, unmodified,
 * source/optix/amadeus_path_tracer.cu -- the closest-hit and miss programs,
 * make_ray and the ray packet -- and through it
 * source/optix/amadeus_common.cuh (Ld, is_occluded, trace, the hit's normal,
 * position and material, the LOAD_RAYPACKET and LOAD_INTERSECTION_DATA
 * blocks), include/cuda/{brdf,material,math,matrix,random}.cuh,
 * include/cuda/cast.cuh, include/optix/{core,lighting,sbt}.cuh and
 * include/bbox.hpp with the headers they include.  What stands in for what
 * a host cannot compile:
 *   - the OptiX device calls.  optixTrace finds the hit with the oracle's
 *     walk (itself checked against shaders/rt/modules/bvh.glsl compiled on
 *     the host) and then runs the closest-hit program, or the miss program
 *     of the call's miss index; the shadow rays (no closest-hit program)
 *     run only their miss program.  The getters read a stack of per-call
 *     states, so that the recursive closest-hit program sees its own ray;
 *   - glm (an empty submodule in the checkout): oracle/shim_pt restates
 *     glm's published formulas;
 *   - include/amadeus/{armada,path_tracer}.cuh and include/vertex.hpp pull
 *     in the Vulkan engine: their include guards are defined here, and the
 *     launch parameters (ArmadaLaunchInfo's members and the traversable) and
 *     Vertex are declared with the reference's member names and types;
 *   - the ray-generation program: the reference's __raygen__ seeds a path
 *     from sinf(x - y), the sample count and the time
 *     (amadeus_path_tracer.cu:90-108), where the benchmark configurations
 *     seed each pixel's PCG stream from the pixel index and the frame.  The
 *     raygen here takes that seed (the oracle's pixel_seed) and then runs the
 *     reference's own make_ray and trace, so everything past the seed is the
 *     reference's code;
 *   - __sinf, __cosf, __tanf, sinf, cosf, tanf, atanf, acosf, asinf and
 *     powf map to the oracle's specification of the reference's fast
 *     intrinsics (oracle/ref_math.h; powf with exponent 2, 4 or 5 as
 *     repeated multiplication), the same functions the oracle and the
 *     kernels use, so that the images can agree to rounding; printf is
 *     silenced (the reference's raygen prints every pixel);
 *   - tex2D: the texture unit's read of the environment map (normalised
 *     coordinates, wrap addressing, the given filter) is the oracle's
 *     reading of the CUDA texture rules (oracle_env_lookup); the scenes
 *     have no material textures.
 *
 * Usage: ref_pt <scene> <seed> <width> <height> <max_depth> <frame>
 *               [<environment file> <filter>]
 * The environment file holds uint32 width, height, then width * height
 * RGBA float32 texels, row 0 first; filter 0 is linear, 1 point.
 * Output on stdout: width * height * 3 float32 (the radiance of one sample
 * of each pixel, row 0 first).
 */
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

/* printf of the reference's raygen */
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

/* include/amadeus/{armada,path_tracer}.cuh: the launch parameters */
#define KOBRA_AMADEUS_ARMADA_H_
#define KOBRA_AMADEUS_PATH_TRACER_H_
namespace kobra {
namespace amadeus {
struct PathTracerParameters {
	glm::vec2 resolution;
	struct Camera {
		glm::vec3 center;
		glm::vec3 ax_u;
		glm::vec3 ax_v;
		glm::vec3 ax_w;
		glm::mat4 projection;
		glm::mat4 view;
	} camera;
	struct {
		optix::QuadLight *quad_lights;
		optix::TriangleLight *tri_lights;
		int quad_count;
		int tri_count;
	} lights;
	struct {
		glm::vec4 *color;
		glm::vec4 *normal;
		glm::vec4 *albedo;
		glm::vec4 *position;
	} buffers;
	cuda::_material *materials;
	cudaTextureObject_t environment_map;
	bool has_environment_map;
	bool accumulate;
	float time;
	int max_depth;
	int samples;
	OptixTraversableHandle traversable;
};
} /* namespace amadeus */
} /* namespace kobra */

#include "source/optix/amadeus_path_tracer.cu"

#undef printf

/* ------------------------------------------------------------- harness -- */

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

static oracle_scene g_scene;
/* one hit record a material (a submesh of OptiX's scene), and where each
 * triangle of the scene sits in them */
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
			if (miss_index == 1)
				__miss__shadow();
			else
				__miss__();
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
		__closesthit__();
	} else {
		g_calls.push_back(call);
		if (miss_index == 1)
			__miss__shadow();
		else
			__miss__();
	}
	g_calls.pop_back();
}

/* The ray-generation program with the pixel's PCG seed (see the header):
 * the reference's make_ray and trace, then its NaN rule. */
static float3 raygen(uint32_t ix, uint32_t iy, uint32_t frame)
{
	g_launch = make_uint3(ix, iy, 0);
	const uint3 idx = optixGetLaunchIndex();
	RayPacket rp{
		.value = make_float3(0.0f),
		.position = make_float4(0),
		.ior = 1.0f,
		.depth = 0,
	};
	uint32_t pix = ix + iy * (uint32_t)parameters.resolution.x;
	oref::f3 s = oref::pixel_seed(pix, frame, 0);
	rp.seed = make_float3(s.x, s.y, s.z);
	unsigned int i0, i1;
	pack_pointer(&rp, i0, i1);
	float3 origin, direction;
	make_ray(idx, origin, direction, rp.seed);
	trace(parameters.traversable, 0, 1, origin, direction, i0, i1);
	float3 c = rp.value;
	if (std::isnan(c.x) || std::isnan(c.y) || std::isnan(c.z))
		c = make_float3(1.0f, 0.0f, 1.0f);
	return c;
}

int main(int argc, char **argv)
{
	if (argc != 7 && argc != 9) {
		fprintf(stderr, "usage: ref_pt <scene> <seed> <width> <height> <max_depth> <frame> [<env> <filter>]\n");
		return 2;
	}
	if (argc == 9) {
		FILE *f = fopen(argv[7], "rb");
		uint32_t wh[2];
		if (!f || fread(wh, 4, 2, f) != 2)
			return 1;
		g_env.resize(4 * (size_t)wh[0] * wh[1]);
		if (fread(g_env.data(), 4, g_env.size(), f) != g_env.size())
			return 1;
		fclose(f);
		g_env_w = wh[0];
		g_env_h = wh[1];
		g_env_filter = atoi(argv[8]);
	}
	uint32_t W = (uint32_t)atoi(argv[3]), H = (uint32_t)atoi(argv[4]), frame = (uint32_t)atoi(argv[6]);
	oracle_generated *gen = nullptr;
	if (oracle_generate_scene(argv[1], strtoull(argv[2], nullptr, 10), &gen) != 0)
		return 1;
	oracle_scene_arrays a;
	oracle_generated_view(gen, &a);

	/* the oracle's scene: its SAH BVH (leaves of 4) and its lights */
	std::vector<uint32_t> tris(4 * (size_t)a.triangle_count);
	for (uint32_t t = 0; t < a.triangle_count; t++) {
		for (int k = 0; k < 3; k++)
			tris[4 * (size_t)t + k] = a.indices[3 * (size_t)t + k];
		tris[4 * (size_t)t + 3] = a.material_indices[t];
	}
	int64_t nb = oracle_build_sah(a.positions, a.indices, a.triangle_count, 4, nullptr, 0);
	std::vector<float> bvh(4 * (size_t)nb);
	oracle_build_sah(a.positions, a.indices, a.triangle_count, 4, bvh.data(), (uint64_t)nb);
	uint32_t nl = oracle_scene_lights(a.positions, a.indices, a.material_indices, a.triangle_count, a.materials,
		nullptr);
	std::vector<kgr_triangle_light> lights(nl);
	oracle_scene_lights(a.positions, a.indices, a.material_indices, a.triangle_count, a.materials, lights.data());
	memset(&g_scene, 0, sizeof(g_scene));
	g_scene.positions = a.positions;
	g_scene.normals = a.normals;
	g_scene.tris = tris.data();
	g_scene.materials = a.materials;
	g_scene.lights = lights.data();
	g_scene.bvh = bvh.data();
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

	/* the reference's view of it: vertices, one hit record a material with
	 * the identity model, materials, triangle lights */
	std::vector<kobra::Vertex> vertices(a.vertex_count);
	for (uint32_t v = 0; v < a.vertex_count; v++) {
		const float *p = a.positions + 3 * (size_t)v, *n = a.normals + 3 * (size_t)v;
		vertices[v].position = glm::vec3(p[0], p[1], p[2]);
		vertices[v].normal = glm::vec3(n[0], n[1], n[2]);
	}
	std::vector<std::vector<glm::uvec3>> tri_lists(a.material_count);
	g_where.resize(a.triangle_count);
	for (uint32_t t = 0; t < a.triangle_count; t++) {
		uint32_t m = a.material_indices[t];
		g_where[t] = {m, (uint32_t)tri_lists[m].size()};
		tri_lists[m].push_back(glm::uvec3{a.indices[3 * (size_t)t], a.indices[3 * (size_t)t + 1],
			a.indices[3 * (size_t)t + 2]});
	}
	g_records.resize(a.material_count);
	for (uint32_t m = 0; m < a.material_count; m++) {
		memset(&g_records[m], 0, sizeof(kobra::optix::Hit));
		g_records[m].vertices = vertices.data();
		g_records[m].model = glm::mat4(1.0f);
		g_records[m].triangles = tri_lists[m].data();
		g_records[m].light_index = -1;
		g_records[m].material_index = m;
	}
	std::vector<kobra::cuda::_material> materials(a.material_count);
	for (uint32_t m = 0; m < a.material_count; m++) {
		const kgr_material &s = a.materials[m];
		kobra::cuda::_material &d = materials[m];
		d.diffuse = make_float3(s.diffuse[0], s.diffuse[1], s.diffuse[2]);
		d.specular = make_float3(s.specular[0], s.specular[1], s.specular[2]);
		d.emission = make_float3(s.emission[0], s.emission[1], s.emission[2]);
		d.ambient = make_float3(s.ambient[0], s.ambient[1], s.ambient[2]);
		d.shininess = s.shininess;
		d.roughness = s.roughness;
		d.refraction = s.refraction;
		d.type = (Shading)s.type;
	}
	std::vector<kobra::optix::TriangleLight> tri_lights(nl);
	for (uint32_t l = 0; l < nl; l++) {
		const kgr_triangle_light &s = lights[l];
		tri_lights[l].a = make_float3(s.a[0], s.a[1], s.a[2]);
		tri_lights[l].ab = make_float3(s.ab[0], s.ab[1], s.ab[2]);
		tri_lights[l].ac = make_float3(s.ac[0], s.ac[1], s.ac[2]);
		tri_lights[l].intensity = make_float3(s.intensity[0], s.intensity[1], s.intensity[2]);
	}

	float cam[12];
	const float up[3] = {0.0f, 1.0f, 0.0f};
	oracle_camera(a.eye, a.target, up, a.fov_deg, (float)W / (float)H, cam, cam + 3, cam + 6, cam + 9);
	memset(&parameters, 0, sizeof(parameters));
	parameters.resolution = glm::vec2((float)W, (float)H);
	parameters.camera.center = glm::vec3(cam[0], cam[1], cam[2]);
	parameters.camera.ax_u = glm::vec3(cam[3], cam[4], cam[5]);
	parameters.camera.ax_v = glm::vec3(cam[6], cam[7], cam[8]);
	parameters.camera.ax_w = glm::vec3(cam[9], cam[10], cam[11]);
	parameters.lights.quad_lights = nullptr;
	parameters.lights.tri_lights = tri_lights.data();
	parameters.lights.quad_count = 0;
	parameters.lights.tri_count = (int)nl;
	parameters.materials = materials.data();
	parameters.has_environment_map = g_env_w != 0;
	parameters.environment_map = 1; /* any handle: tex2D reads g_env */
	parameters.accumulate = false;
	parameters.max_depth = atoi(argv[5]);
	parameters.samples = 0;

	std::vector<float> out(3 * (size_t)W * H);
	for (uint32_t iy = 0; iy < H; iy++)
		for (uint32_t ix = 0; ix < W; ix++) {
			float3 c = raygen(ix, iy, frame);
			size_t i = 3 * ((size_t)iy * W + ix);
			out[i] = c.x;
			out[i + 1] = c.y;
			out[i + 2] = c.z;
		}
	fwrite(out.data(), sizeof(float), out.size(), stdout);
	oracle_generated_destroy(gen);
	return 0;
}

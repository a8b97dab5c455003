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
 * include/bbox.hpp with the headers they include.  The OptiX device calls,
 * glm, the Vulkan-bound headers, the fast intrinsics and the texture reads
 * are stood in for as oracle/ref_optix_host.h states; include/amadeus/
 * path_tracer.cuh is replaced by its launch parameters, declared here with
 * the reference's member names and types.  The ray-generation program: the
 * reference's __raygen__ seeds a path from sinf(x - y), the sample count
 * and the time (amadeus_path_tracer.cu:90-108), where the benchmark
 * configurations seed each pixel's PCG stream from the pixel index and the
 * frame.  The raygen here takes that seed (the oracle's pixel_seed) and
 * then runs the reference's own make_ray and trace, so everything past the
 * seed is the reference's code.
 *
 * Usage: ref_pt <scene> <seed> <width> <height> <max_depth> <frame>
 *               [--env <file> <filter>] [--quads <file>]
 * (oracle/ref_optix_host.h gives the file formats).
 * Output on stdout: width * height * 3 float32 (the radiance of one sample
 * of each pixel, row 0 first).
 */
#include "ref_optix_host.h"

/* include/amadeus/path_tracer.cuh: the launch parameters (its
 * PathTracerParameters, ArmadaLaunchInfo's members and the traversable) */
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

void program_closesthit() { __closesthit__(); }

void program_miss(unsigned int miss_index)
{
	if (miss_index == 1)
		__miss__shadow();
	else
		__miss__();
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
	if (argc < 7 || !host_options(argc, argv, 7)) {
		fprintf(stderr, "usage: ref_pt <scene> <seed> <width> <height> <max_depth> <frame> [--env <file> <filter>] "
			"[--quads <file>]\n");
		return 2;
	}
	uint32_t W = (uint32_t)atoi(argv[3]), H = (uint32_t)atoi(argv[4]), frame = (uint32_t)atoi(argv[6]);
	HostScene hs;
	if (!host_scene_build(hs, argv[1], strtoull(argv[2], nullptr, 10), W, H))
		return 1;
	memset(&parameters, 0, sizeof(parameters));
	parameters.resolution = glm::vec2((float)W, (float)H);
	parameters.camera.center = glm::vec3(hs.center[0], hs.center[1], hs.center[2]);
	parameters.camera.ax_u = glm::vec3(hs.ax_u[0], hs.ax_u[1], hs.ax_u[2]);
	parameters.camera.ax_v = glm::vec3(hs.ax_v[0], hs.ax_v[1], hs.ax_v[2]);
	parameters.camera.ax_w = glm::vec3(hs.ax_w[0], hs.ax_w[1], hs.ax_w[2]);
	parameters.lights.quad_lights = g_quad_lights.data();
	parameters.lights.tri_lights = hs.tri_lights.data();
	parameters.lights.quad_count = (int)g_quad_lights.size();
	parameters.lights.tri_count = (int)hs.tri_lights.size();
	parameters.materials = hs.materials.data();
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
	oracle_generated_destroy(hs.gen);
	return 0;
}

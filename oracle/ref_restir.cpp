/*
 * ref_restir.cpp -- the reference's ReSTIR DI programs compiled on the host,
 * for known-answer images and reservoirs of the resampling.
 *
 * TEST INFRASTRUCTURE.  Compiled by oracle/Makefile (target `ref`) against
 * the reference sources where they lie (REFERENCE=<path>) and the oracle
 * library, into oracle/_ref/ref_restir.  It includes, unmodified,
 * source/optix/amadeus_restir.cu -- __closesthit__initial (RIS over 32
 * candidates at the primary vertex, the path beyond it), __raygen__temporal,
 * __raygen__spatial, the miss programs, make_ray, target, occluded_target,
 * reproject and sample_spatial_neighborhood -- with
 * include/amadeus/reservoir.cuh (Reservoir, DirectLightingSample) and
 * source/optix/amadeus_common.cuh.  The OptiX device calls, glm, the
 * Vulkan-bound headers, the fast intrinsics and the texture reads are stood
 * in for as oracle/ref_optix_host.h states; include/amadeus/restir.cuh is
 * replaced by its launch parameters (ReSTIR_Parameters), declared here with
 * the reference's member names and types.
 *
 * A frame follows ReSTIR::render (include/amadeus/restir.cuh:254-303), a
 * host method around optixLaunch, restated here: the initial pass, the
 * temporal pass, two spatial passes each followed by the swap of the
 * current and previous reservoirs, the final swap, and the camera kept as
 * the previous camera.  Two inputs are set here:
 *   - the initial pass's ray generation (__raygen__initial,
 *     amadeus_restir.cu:82-144) seeds a path from sinf(x - y), the sample
 *     count and the time, where the benchmark configurations seed each
 *     pixel's PCG stream from the pixel index and the frame; the raygen
 *     here takes that seed and otherwise does what the reference's does
 *     (make_ray, trace, the intermediate colour, the auxiliary seed, the
 *     AOVs);
 *   - the RIS reservoir's own seed, which the reference draws once, when
 *     the reservoirs are allocated, from std::random_device
 *     (reservoir.cuh:27-34), is set before every initial pass to the
 *     oracle's per-frame seed pixel_seed(pixel, frame, 0x9E3779B9).
 *
 * Usage: ref_restir <scene> <seed> <width> <height> <max_depth> <frames>
 *                   [--env <file> <filter>] [--quads <file>]
 * (oracle/ref_optix_host.h gives the file formats).
 * Output on stdout: for each frame the colour buffer after it (width *
 * height RGBA float32, accumulated over the frames, row 0 first); then the
 * reservoirs the next frame would reuse, six float32 a pixel: the selected
 * point xyz, w, W and M.
 */
#include "ref_optix_host.h"

#include "include/amadeus/reservoir.cuh"

/* include/amadeus/restir.cuh: the launch parameters (its ReSTIR_Parameters,
 * ArmadaLaunchInfo's members and its own) */
#define KOBRA_AMADEUS_RESTIR_H_
namespace kobra {
namespace amadeus {
struct ReSTIR_Parameters {
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
	Reservoir<DirectLightingSample> *current;
	Reservoir<DirectLightingSample> *previous;
	cuda::Material *materials_buffer;
	glm::vec4 *intermediate;
	glm::vec4 *auxiliary;
	Camera previous_camera;
};
} /* namespace amadeus */
} /* namespace kobra */

#include "source/optix/amadeus_restir.cu"

#undef printf

void program_closesthit() { __closesthit__initial(); }

void program_miss(unsigned int miss_index)
{
	if (miss_index == 1)
		__miss__shadow();
	else
		__miss__();
}

/* the oracle's salt of the RIS reservoir's per-frame seed */
static const uint32_t RIS_SALT = 0x9E3779B9u;

/* The initial pass's ray generation with the pixel's PCG seeds (see the
 * header). */
static void raygen_initial(uint32_t ix, uint32_t iy, uint32_t frame)
{
	g_launch = make_uint3(ix, iy, 0);
	const uint3 idx = optixGetLaunchIndex();
	const int index = idx.x + idx.y * parameters.resolution.x;
	parameters.current[index].reset();
	oref::f3 rs = oref::pixel_seed((uint32_t)index, frame, RIS_SALT);
	parameters.current[index].seed = make_float3(rs.x, rs.y, rs.z);
	RayPacket rp{
		.value = make_float3(0.0f),
		.position = make_float4(0),
		.ior = 1.0f,
		.depth = 0,
		.index = index,
	};
	oref::f3 s = oref::pixel_seed((uint32_t)index, frame, 0);
	rp.seed = make_float3(s.x, s.y, s.z);
	unsigned int i0, i1;
	pack_pointer(&rp, i0, i1);
	float3 origin, direction;
	make_ray(idx, origin, direction, rp.seed);
	trace(parameters.traversable, 0, 1, origin, direction, i0, i1);
	glm::vec4 color = {rp.value.x, rp.value.y, rp.value.z, 1.0f};
	glm::vec3 normal = {rp.normal.x, rp.normal.y, rp.normal.z};
	glm::vec3 albedo = {rp.albedo.x, rp.albedo.y, rp.albedo.z};
	glm::vec3 position = {rp.position.x, rp.position.y, rp.position.z};
	if (std::isnan(color.x) || std::isnan(color.y) || std::isnan(color.z))
		color = {1, 0, 1, 1};
	parameters.intermediate[index] = color;
	parameters.auxiliary[index] = {rp.seed.x, rp.seed.y, rp.seed.z, 1.0f};
	auto &buffers = parameters.buffers;
	accumulate(buffers.normal[index], {normal, 0.0f});
	accumulate(buffers.albedo[index], {albedo, 0.0f});
	buffers.position[index] = {position, 0.0f};
}

template <class F>
static void each_pixel(uint32_t W, uint32_t H, F f)
{
	for (uint32_t iy = 0; iy < H; iy++)
		for (uint32_t ix = 0; ix < W; ix++) {
			g_launch = make_uint3(ix, iy, 0);
			f(ix, iy);
		}
}

int main(int argc, char **argv)
{
	if (argc < 7 || !host_options(argc, argv, 7)) {
		fprintf(stderr, "usage: ref_restir <scene> <seed> <width> <height> <max_depth> <frames> "
			"[--env <file> <filter>] [--quads <file>]\n");
		return 2;
	}
	uint32_t W = (uint32_t)atoi(argv[3]), H = (uint32_t)atoi(argv[4]), frames = (uint32_t)atoi(argv[6]);
	HostScene hs;
	if (!host_scene_build(hs, argv[1], strtoull(argv[2], nullptr, 10), W, H))
		return 1;
	size_t npix = (size_t)W * H;
	std::vector<glm::vec4> color(npix), normal(npix), albedo(npix), position(npix), intermediate(npix),
		auxiliary(npix);
	std::vector<kobra::cuda::Material> material_buffer(npix);
	/* the reference allocates the reservoirs with the default constructor,
	 * whose seed is overwritten before each initial pass here */
	std::vector<Reservoir<DirectLightingSample>> A(npix), B(npix);

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
	parameters.buffers.color = color.data();
	parameters.buffers.normal = normal.data();
	parameters.buffers.albedo = albedo.data();
	parameters.buffers.position = position.data();
	parameters.materials = hs.materials.data();
	parameters.has_environment_map = g_env_w != 0;
	parameters.environment_map = 1; /* any handle: tex2D reads g_env */
	parameters.max_depth = atoi(argv[5]);
	parameters.current = A.data();
	parameters.previous = B.data();
	parameters.materials_buffer = material_buffer.data();
	parameters.intermediate = intermediate.data();
	parameters.auxiliary = auxiliary.data();

	for (uint32_t f = 0; f < frames; f++) {
		/* frame f of a still camera: f samples accumulated before it */
		parameters.samples = (int)f;
		parameters.accumulate = f > 0;
		each_pixel(W, H, [&](uint32_t ix, uint32_t iy) { raygen_initial(ix, iy, f); });
		each_pixel(W, H, [&](uint32_t, uint32_t) { __raygen__temporal(); });
		for (int i = 0; i < 2; i++) {
			each_pixel(W, H, [&](uint32_t, uint32_t) { __raygen__spatial(); });
			std::swap(parameters.current, parameters.previous);
		}
		std::swap(parameters.current, parameters.previous);
		parameters.previous_camera = parameters.camera;
		fwrite(color.data(), sizeof(glm::vec4), npix, stdout);
	}
	for (size_t i = 0; i < npix; i++) {
		const Reservoir<DirectLightingSample> &r = parameters.previous[i];
		float v[6] = {r.data.point.x, r.data.point.y, r.data.point.z, r.w, r.W, (float)r.M};
		fwrite(v, sizeof(float), 6, stdout);
	}
	oracle_generated_destroy(hs.gen);
	return 0;
}

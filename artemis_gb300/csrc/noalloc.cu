/*
 * noalloc.cu -- a path-traced frame that allocates nothing.
 *
 * kgr_render_pt_noalloc runs the same wavefront kernels as the path-tracer
 * attachment, but its per-path scratch (rays, throughput, radiance, RNG
 * state, hit records, pending NEE terms, AOVs, the three path-id queues and
 * the queue counters) lives in one file-scope __device__ array instead of
 * buffers the attachment allocates in kgr_load.  It is meant for callers that
 * cannot call cudaMalloc at render time: a host that fixes its device memory
 * at start-up and owns the allocator (a real-time loop with a hard memory
 * budget, a plugin host that hands out device memory itself), where an
 * allocation inside the plugin would break the host's accounting or fail.
 *
 * Limits and sharing:
 *  - at most KGR_NOALLOC_MAX_PATHS (65536) paths per call, i.e.
 *    width * height * spp <= 65536 (256x256 at 1 spp, 128x128 at 4 spp);
 *    larger requests fail with KGR_ERR_INVALID_ARGUMENT before any launch;
 *  - the array (about 12.8 MiB) is part of the library image: every GPU the
 *    library is loaded on holds it until the process exits;
 *  - every call on a device uses the same array, and it keeps the previous
 *    call's contents.  The kernels overwrite every path slot they read and
 *    the queue counters are cleared at the start of each call, so nothing
 *    leaks between calls -- but two calls whose work overlaps on the GPU
 *    (different streams, no ordering between them) race on the array and
 *    give wrong images.  Serialise them on one stream or with events.
 *  - the first call on a device looks up the array's device address with
 *    cudaGetSymbolAddress (once per device, with that device current); make
 *    that first call before any stream capture begins.
 */
#include <math.h>
#include <string.h>

#include <cmath>

#include <mutex>

#include "kgr_wavefront.h"

#define KGR_NOALLOC_MAX_PATHS 65536u
#define KGR_NOALLOC_SLOT_BYTES ((size_t)KGR_NOALLOC_MAX_PATHS * 16u)
#define KGR_NOALLOC_QUEUE_BYTES ((size_t)KGR_NOALLOC_MAX_PATHS * 4u)
/* KGR_PATH_ARRAYS float4 path arrays + 3 uint32 queues + 256 bytes of counters */
#define KGR_NOALLOC_BYTES ((size_t)KGR_PATH_ARRAYS * KGR_NOALLOC_SLOT_BYTES + 3u * KGR_NOALLOC_QUEUE_BYTES + 256u)

static __device__ __align__(256) unsigned char g_noalloc_scratch[KGR_NOALLOC_BYTES];

namespace kgr {
namespace {

#define KGR_NOALLOC_MAX_DEVICES 64
std::mutex g_noalloc_mutex;
unsigned char *g_noalloc_ptr[KGR_NOALLOC_MAX_DEVICES] = {nullptr};

/* Device address of the scratch array on the current device.  The host-side
 * symbol is only a stand-in; the kernels need the address the runtime maps
 * for this device. */
unsigned char *noalloc_scratch(int device)
{
	KGR_REQUIRE(device >= 0 && device < KGR_NOALLOC_MAX_DEVICES, KGR_ERR_UNSUPPORTED, "device ordinal too large");
	std::lock_guard<std::mutex> lock(g_noalloc_mutex);
	if (!g_noalloc_ptr[device]) {
		void *p = nullptr;
		cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
		if (e != cudaSuccess)
			throw Error(KGR_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
		g_noalloc_ptr[device] = static_cast<unsigned char *>(p);
	}
	return g_noalloc_ptr[device];
}

PathBuffers noalloc_buffers(unsigned char *base)
{
	PathBuffers pb;
	float4 **fields[KGR_PATH_ARRAYS];
	path_array_slots(pb, fields);
	for (int k = 0; k < KGR_PATH_ARRAYS; k++)
		*fields[k] = reinterpret_cast<float4 *>(base + (size_t)k * KGR_NOALLOC_SLOT_BYTES);
	unsigned char *q = base + (size_t)KGR_PATH_ARRAYS * KGR_NOALLOC_SLOT_BYTES;
	pb.queue[0] = reinterpret_cast<uint32_t *>(q);
	pb.queue[1] = reinterpret_cast<uint32_t *>(q + KGR_NOALLOC_QUEUE_BYTES);
	pb.shadow_queue = reinterpret_cast<uint32_t *>(q + 2u * KGR_NOALLOC_QUEUE_BYTES);
	pb.counters = reinterpret_cast<uint32_t *>(q + 3u * KGR_NOALLOC_QUEUE_BYTES);
	pb.visits = nullptr;
	pb.capacity = KGR_NOALLOC_MAX_PATHS;
	return pb;
}

} /* namespace */
} /* namespace kgr */

using namespace kgr;

extern "C" kgr_status kgr_render_pt_noalloc(const kgr_scene *sc, const kgr_launch_info *info, int32_t spp,
		int32_t russian_roulette, int32_t rr_start_depth, void *stream)
{
	try {
		KGR_REQUIRE(sc && info, KGR_ERR_INVALID_ARGUMENT, "NULL scene or launch info");
		KGR_REQUIRE(info->buffers.color, KGR_ERR_INVALID_ARGUMENT, "color buffer is NULL");
		KGR_REQUIRE(!info->has_environment_map && info->lights.quad_count == 0, KGR_ERR_UNSUPPORTED,
			"environment maps and quad lights are not supported");
		KGR_REQUIRE(info->max_depth >= 0 && info->max_depth <= 64, KGR_ERR_INVALID_ARGUMENT,
			"max_depth out of range");
		KGR_REQUIRE(spp >= 1, KGR_ERR_INVALID_ARGUMENT, "spp must be at least 1");
		/* validate the float extent before any conversion: a negative, NaN or
		 * huge value has no defined unsigned conversion */
		for (int k = 0; k < 2; k++) {
			float r = info->resolution[k];
			KGR_REQUIRE(std::isfinite(r) && r >= 1.0f && r <= (float)KGR_NOALLOC_MAX_PATHS && r == floorf(r),
				KGR_ERR_INVALID_ARGUMENT, "resolution must hold whole numbers in [1, 65536]");
		}
		uint64_t w = (uint64_t)(uint32_t)info->resolution[0], h = (uint64_t)(uint32_t)info->resolution[1];
		uint64_t paths = w * h * (uint64_t)spp;
		KGR_REQUIRE(paths <= KGR_NOALLOC_MAX_PATHS, KGR_ERR_INVALID_ARGUMENT,
			"width * height * spp = " + std::to_string(paths) + " exceeds the no-allocation limit of "
				+ std::to_string(KGR_NOALLOC_MAX_PATHS) + " paths");
		const void *bufs[4] = {info->buffers.color, info->buffers.normal, info->buffers.albedo,
			info->buffers.position};
		for (const void *b : bufs)
			KGR_REQUIRE(((uintptr_t)b & 15u) == 0, KGR_ERR_INVALID_ARGUMENT, "output buffers must be 16-byte aligned");
		DeviceGuard guard(sc->device);
		PathBuffers pb = noalloc_buffers(noalloc_scratch(sc->device));

		FrameParams fp;
		memset(&fp, 0, sizeof(fp));
		fp.width = (uint32_t)w;
		fp.height = (uint32_t)h;
		fp.npix = (uint32_t)(w * h);
		fp.spp = (uint32_t)spp;
		fp.paths = (uint32_t)paths;
		memcpy(fp.center, info->camera.center, 12);
		memcpy(fp.U, info->camera.ax_u, 12);
		memcpy(fp.V, info->camera.ax_v, 12);
		memcpy(fp.W, info->camera.ax_w, 12);
		fp.max_depth = info->max_depth;
		fp.russian_roulette = russian_roulette ? 1 : 0;
		fp.rr_start_depth = rr_start_depth;
		fp.frame = info->frame;
		fp.accumulate = info->accumulate ? 1 : 0;
		fp.samples = info->samples;
		fp.layout = KGR_LAYOUT_FAST;
		fp.tune = default_trace_tune();
		fp.jitter = 1;

		DeviceScene s = sc->view();
		if (info->lights.tri_lights) {
			s.lights = info->lights.tri_lights;
			s.light_count = (uint32_t)info->lights.tri_count;
		}
		if (info->materials)
			s.materials = info->materials;
		OutputBuffers out = {reinterpret_cast<float4 *>(info->buffers.color),
			reinterpret_cast<float4 *>(info->buffers.normal), reinterpret_cast<float4 *>(info->buffers.albedo),
			reinterpret_cast<float4 *>(info->buffers.position)};
		cudaStream_t st = (cudaStream_t)stream;

		/* the array keeps the last call's contents: clear the counters */
		KGR_CUDA(cudaMemsetAsync(pb.counters, 0, 256, st));
		pt_generate(pb, fp, st);
		for (int d = 0; d <= fp.max_depth; d++) {
			int q = d & 1;
			if (d > 0)
				reset_counters(pb, (1 << (q ^ 1)) | (1 << CNT_SHADOW), st);
			pt_trace_closest(s, pb, q, fp.layout, fp.tune, st);
			pt_shade(s, pb, fp, d, q, st);
			pt_shadow_resolve(s, pb, fp.layout, fp.tune, st);
		}
		pt_accumulate(pb, fp, out, st);
		return KGR_OK;
	} catch (const Error &e) {
		set_last_error(e.what());
		return e.status;
	} catch (const std::exception &e) {
		set_last_error(e.what());
		return KGR_ERR_INTERNAL;
	}
}

/*
 * batch.cu -- the job-aware stages of a batched path-tracer frame.
 *
 * Every path computes exactly what the single-image path tracer computes for
 * it: the seed of sample s of pixel i of a job is pixel_seed(i, frame * spp +
 * s), the camera ray and the shading are the same functions, and samples are
 * blended in sample order.  A job rendered in a batch, or in slices of
 * samples over several batches, therefore gives the same image, bit for bit,
 * as the "path_tracer" attachment with the same spp and frame.
 */
#include "kgr_batch.h"
#include "kgr_device.cuh"
#include "kgr_shade.cuh"

namespace kgr {

namespace {

/* The last job whose `offset` field (path or pixel) is <= x. */
template <bool PIX>
__device__ __forceinline__ uint32_t find_job(const BatchJob *jobs, uint32_t njobs, uint32_t x)
{
	uint32_t lo = 0, hi = njobs - 1;
	while (lo < hi) {
		uint32_t mid = (lo + hi + 1) >> 1;
		uint32_t off = PIX ? jobs[mid].pix_offset : jobs[mid].path_offset;
		if (off <= x)
			lo = mid;
		else
			hi = mid - 1;
	}
	return lo;
}

__global__ void __launch_bounds__(256) batch_generate_kernel(PathBuffers pb, const BatchHeader *hdr,
		const BatchJob *jobs)
{
	const uint32_t total = hdr->total_paths, njobs = hdr->njobs;
	if (blockIdx.x == 0 && threadIdx.x == 0) {
		pb.counters[CNT_Q0] = total;
		pb.counters[CNT_Q1] = 0;
		pb.counters[CNT_SHADOW] = 0;
		pb.counters[CNT_BOUNCE_TOTAL] = 0;
		pb.counters[CNT_SHADOW_TOTAL] = 0;
	}
	for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < total; p += gridDim.x * blockDim.x) {
		const BatchJob &J = jobs[find_job<false>(jobs, njobs, p)];
		uint32_t lp = p - J.path_offset;
		uint32_t srel = lp / J.npix, pix = lp - srel * J.npix;
		uint32_t ix = pix % J.width, iy = pix / J.width;
		uint32_t stream = J.frame * J.spp + J.s0 + srel;
		f3 seed = pixel_seed(pix, stream, 0);
		f3 o, d;
		camera_ray(J.center, J.U, J.V, J.W, J.width, J.height, 1, ix, iy, seed, o, d);
		pb.ray_o[p] = f4_of(o, 0.0f);
		pb.ray_d[p] = f4_of(d, 1e16f);
		pb.beta[p] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
		pb.L[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
		pb.seed[p] = f4_of(seed, 0.0f);
		pb.aov_n[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
		pb.aov_a[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
		pb.aov_p[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
		pb.queue[0][p] = p;
	}
}

__global__ void __launch_bounds__(256) batch_accumulate_kernel(PathBuffers pb, const BatchHeader *hdr,
		const BatchJob *jobs)
{
	const uint32_t total = hdr->total_pix, njobs = hdr->njobs;
	for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
		const BatchJob &J = jobs[find_job<true>(jobs, njobs, q)];
		uint32_t pix = q - J.pix_offset;
		OutputBuffers out = {J.color, J.normal, J.albedo, J.position};
		for (uint32_t sidx = 0; sidx < J.k; sidx++) {
			uint32_t s = J.s0 + sidx;
			bool acc = J.accumulate || s > 0;
			float count = (float)(J.accumulate ? J.samples + (int)s : (int)s);
			accumulate_path(out, pb, J.path_offset + sidx * J.npix + pix, pix, acc, count);
		}
	}
}

/* Fixed grids: the job table, not the launch, carries the sizes. */
inline int fixed_grid() { return device_sm_count() * 8; }

} /* namespace */

void batch_generate(const PathBuffers &pb, const BatchHeader *hdr, const BatchJob *jobs, cudaStream_t st)
{
	batch_generate_kernel<<<fixed_grid(), 256, 0, st>>>(pb, hdr, jobs);
	KGR_CUDA(cudaGetLastError());
}

void batch_accumulate(const PathBuffers &pb, const BatchHeader *hdr, const BatchJob *jobs, cudaStream_t st)
{
	batch_accumulate_kernel<<<fixed_grid(), 256, 0, st>>>(pb, hdr, jobs);
	KGR_CUDA(cudaGetLastError());
}

void batch_frame(const DeviceScene &s, const PathBuffers &pb, const FrameParams &fp, const BatchHeader *hdr,
		const BatchJob *jobs, cudaStream_t st, const StreamPair &side)
{
	batch_generate(pb, hdr, jobs, st);
	if (side.stream) {
		/* the plain tracer's overlap (render_pt): bounce d's shadow rays on
		 * the side stream, bounce d + 1's closest hits here, joined before
		 * the next shade */
		pt_trace_closest(s, pb, 0, fp.layout, fp.tune, st);
		for (int d = 0; d <= fp.max_depth; d++) {
			int q = d & 1;
			if (d > 0)
				reset_counters(pb, (1 << (q ^ 1)) | (1 << CNT_SHADOW), st);
			pt_shade(s, pb, fp, d, q, st);
			KGR_CUDA(cudaEventRecord(side.shaded, st));
			KGR_CUDA(cudaStreamWaitEvent(side.stream, side.shaded, 0));
			pt_shadow_resolve(s, pb, fp.layout, fp.tune, side.stream);
			KGR_CUDA(cudaEventRecord(side.shadowed, side.stream));
			if (d < fp.max_depth)
				pt_trace_closest(s, pb, q ^ 1, fp.layout, fp.tune, st);
			KGR_CUDA(cudaStreamWaitEvent(st, side.shadowed, 0));
		}
	} else {
		for (int d = 0; d <= fp.max_depth; d++) {
			int q = d & 1;
			if (d > 0)
				reset_counters(pb, (1 << (q ^ 1)) | (1 << CNT_SHADOW), st);
			pt_trace_closest(s, pb, q, fp.layout, fp.tune, st);
			pt_shade(s, pb, fp, d, q, st);
			pt_shadow_resolve(s, pb, fp.layout, fp.tune, st);
		}
	}
	batch_accumulate(pb, hdr, jobs, st);
}

} /* namespace kgr */

/*
 * batch_api.cpp -- kgr_batcher: several path-traced jobs per shared
 * wavefront frame, replayed as a captured CUDA graph.
 *
 * A frame is: copy the job table (pinned staging -> device), the frame's
 * kernels (batch.cu), copy the counters back to pinned memory, record the
 * ring slot's event.  The kernels take every size from the device table, so
 * the graph of one (scene, depth, Russian roulette, layout) replays for any
 * mix of jobs.  The first frame of a configuration runs eagerly (it also
 * settles the launchers' one-time occupancy queries); the second is
 * captured on a private stream and every later one replays the graph on
 * the caller's stream.
 */
#include <string.h>

#include <algorithm>
#include <memory>

#include "kgr_batch.h"

using namespace kgr;

kgr::PathBuffers kgr_batcher::path_buffers()
{
	PathBuffers pb;
	float4 **fields[KGR_PATH_ARRAYS];
	path_array_slots(pb, fields);
	for (int k = 0; k < KGR_PATH_ARRAYS; k++)
		*fields[k] = f4[k].ptr;
	pb.queue[0] = queues[0].ptr;
	pb.queue[1] = queues[1].ptr;
	pb.shadow_queue = queues[2].ptr;
	pb.counters = counters.ptr;
	pb.visits = nullptr;
	pb.capacity = capacity;
	return pb;
}

void kgr_batcher::render(const kgr_scene *scene, const kgr_batch_job *jobs, uint32_t n,
		const kgr_batch_options &opt, cudaStream_t st)
{
	KGR_REQUIRE(scene, KGR_ERR_INVALID_ARGUMENT, "NULL scene");
	KGR_REQUIRE(scene->device == device, KGR_ERR_INVALID_ARGUMENT, "scene and batcher on different devices");
	KGR_REQUIRE(n >= 1 && n <= max_jobs, KGR_ERR_INVALID_ARGUMENT, "job count must be 1..max_jobs");
	KGR_REQUIRE(jobs, KGR_ERR_INVALID_ARGUMENT, "NULL job list");
	KGR_REQUIRE(opt.max_depth >= 0 && opt.max_depth <= 64, KGR_ERR_INVALID_ARGUMENT, "max_depth must be 0..64");
	KGR_REQUIRE(opt.layout == KGR_LAYOUT_FAST || opt.layout == KGR_LAYOUT_THREADED || opt.layout == KGR_LAYOUT_WIDE
			|| opt.layout == KGR_LAYOUT_CW8,
		KGR_ERR_INVALID_ARGUMENT,
		"unknown layout");

	/* the staging slot is free once the frame that last used it is done */
	int r = ring;
	ring = (ring + 1) % RING;
	KGR_CUDA(cudaEventSynchronize(done[r]));

	BatchHeader hdr = {0, 0, 0, 0};
	BatchJob *dj = reinterpret_cast<BatchJob *>(staging[r] + 16);
	uint64_t paths = 0, pix = 0;
	for (uint32_t j = 0; j < n; j++) {
		const kgr_batch_job &J = jobs[j];
		KGR_REQUIRE(J.width >= 1 && J.height >= 1 && J.spp >= 1 && J.sample_count >= 1, KGR_ERR_INVALID_ARGUMENT,
			"job sizes and sample counts must be positive");
		KGR_REQUIRE((uint64_t)J.sample_begin + J.sample_count <= J.spp, KGR_ERR_INVALID_ARGUMENT,
			"job samples past its spp");
		uint64_t np = (uint64_t)J.width * J.height;
		uint64_t jp = np * J.sample_count;
		KGR_REQUIRE(paths + jp <= capacity, KGR_ERR_BUDGET, "jobs exceed the batcher's path capacity");
		BatchJob b;
		memset(&b, 0, sizeof(b));
		b.path_offset = (uint32_t)paths;
		b.pix_offset = (uint32_t)pix;
		b.npix = (uint32_t)np;
		b.width = J.width;
		b.height = J.height;
		b.s0 = J.sample_begin;
		b.k = J.sample_count;
		b.spp = J.spp;
		b.frame = J.frame;
		b.accumulate = J.accumulate ? 1 : 0;
		b.samples = J.samples;
		memcpy(b.center, J.center, 12);
		memcpy(b.U, J.ax_u, 12);
		memcpy(b.V, J.ax_v, 12);
		memcpy(b.W, J.ax_w, 12);
		b.color = reinterpret_cast<float4 *>(J.color);
		b.normal = reinterpret_cast<float4 *>(J.normal);
		b.albedo = reinterpret_cast<float4 *>(J.albedo);
		b.position = reinterpret_cast<float4 *>(J.position);
		dj[j] = b;
		paths += jp;
		pix += np;
		KGR_REQUIRE(pix < (1ull << 32), KGR_ERR_BUDGET, "too many pixels in one batch");
	}
	hdr.njobs = n;
	hdr.total_paths = (uint32_t)paths;
	hdr.total_pix = (uint32_t)pix;
	memcpy(staging[r], &hdr, sizeof(hdr));
	paths_in[r] = hdr.total_paths;

	/* frames on different streams stay in order: the table and the path
	 * state are shared */
	if (last >= 0)
		KGR_CUDA(cudaStreamWaitEvent(st, done[last], 0));
	KGR_CUDA(cudaMemcpyAsync(table.ptr, staging[r], 16 + (size_t)n * sizeof(BatchJob), cudaMemcpyHostToDevice, st));

	FrameParams fp;
	memset(&fp, 0, sizeof(fp));
	fp.max_depth = opt.max_depth;
	fp.russian_roulette = opt.russian_roulette ? 1 : 0;
	fp.rr_start_depth = opt.rr_start_depth;
	fp.layout = layout_for(opt.layout, scene);
	fp.tune = tune;
	DeviceScene s = scene->view();
	PathBuffers pb = path_buffers();
	const BatchHeader *dh = reinterpret_cast<const BatchHeader *>(table.ptr);
	const BatchJob *djobs = reinterpret_cast<const BatchJob *>(table.ptr + 16);

	Graph *g = nullptr;
	if (opt.use_graph) {
		for (auto &e : graphs)
			if (e.scene == scene && e.max_depth == fp.max_depth && e.rr == fp.russian_roulette &&
					e.rr_start == fp.rr_start_depth && e.layout == fp.layout &&
					e.tune.shadow == tune.shadow && e.tune.occupancy == tune.occupancy &&
					e.tune.block == tune.block && e.tune.stack == tune.stack)
				g = &e;
		if (!g) {
			graphs.push_back(Graph{scene, fp.max_depth, fp.russian_roulette, fp.rr_start_depth, fp.layout, tune,
				0, nullptr});
			g = &graphs.back();
		}
	}
	last_graph = 0;
	if (g && !g->exec && g->eager_runs >= 1) {
		/* capture on a private stream (the caller's may be the legacy
		 * default stream, which cannot be captured) */
		cudaGraph_t graph = nullptr;
		KGR_CUDA(cudaStreamBeginCapture(capture_stream, cudaStreamCaptureModeThreadLocal));
		try {
			batch_frame(s, pb, fp, dh, djobs, capture_stream, side);
		} catch (...) {
			cudaStreamEndCapture(capture_stream, &graph);
			if (graph)
				cudaGraphDestroy(graph);
			throw;
		}
		KGR_CUDA(cudaStreamEndCapture(capture_stream, &graph));
		cudaError_t e = cudaGraphInstantiate(&g->exec, graph, 0);
		cudaGraphDestroy(graph);
		KGR_CUDA(e);
	}
	if (g && g->exec) {
		KGR_CUDA(cudaGraphLaunch(g->exec, st));
		last_graph = 1;
		graph_replays++;
	} else {
		batch_frame(s, pb, fp, dh, djobs, st, side);
		if (g)
			g->eager_runs++;
	}
	last_launches = 2 + 3 * (uint32_t)(fp.max_depth + 1);
	KGR_CUDA(cudaMemcpyAsync(stats_host[r], counters.ptr, CNT_COUNT * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
	KGR_CUDA(cudaEventRecord(done[r], st));
	last = r;
}

void kgr_batcher::ray_counts(int r, uint64_t counts[3])
{
	KGR_CUDA(cudaEventSynchronize(done[r]));
	counts[0] = paths_in[r];
	counts[1] = stats_host[r][CNT_BOUNCE_TOTAL];
	counts[2] = stats_host[r][CNT_SHADOW_TOTAL];
}

kgr_batcher::~kgr_batcher()
{
	DeviceGuard guard(device);
	for (int r = 0; r < RING; r++) {
		if (done[r]) {
			cudaEventSynchronize(done[r]);
			cudaEventDestroy(done[r]);
		}
		if (staging[r])
			cudaFreeHost(staging[r]);
		if (stats_host[r])
			cudaFreeHost(stats_host[r]);
	}
	for (auto &g : graphs)
		if (g.exec)
			cudaGraphExecDestroy(g.exec);
	if (capture_stream)
		cudaStreamDestroy(capture_stream);
	if (side.stream) {
		cudaStreamSynchronize(side.stream);
		cudaStreamDestroy(side.stream);
	}
	for (cudaEvent_t e : {side.shaded, side.shadowed})
		if (e)
			cudaEventDestroy(e);
}

extern "C" {

kgr_status kgr_batcher_create(int32_t device, uint32_t path_capacity, uint32_t max_jobs, kgr_batcher **out)
{
	return guard_call([&] {
		KGR_REQUIRE(out, KGR_ERR_INVALID_ARGUMENT, "NULL out");
		*out = nullptr;
		KGR_REQUIRE(path_capacity >= 1 && path_capacity <= (1u << 28), KGR_ERR_INVALID_ARGUMENT,
			"path_capacity must be 1..2^28");
		KGR_REQUIRE(max_jobs >= 1 && max_jobs <= 65536, KGR_ERR_INVALID_ARGUMENT, "max_jobs must be 1..65536");
		int dev = pick_device_ordinal(device);
		DeviceGuard guard(dev);
		std::unique_ptr<kgr_batcher> b(new kgr_batcher());
		b->device = dev;
		b->capacity = path_capacity;
		b->max_jobs = max_jobs;
		for (auto &f : b->f4)
			f.alloc(path_capacity);
		for (auto &q : b->queues)
			q.alloc(path_capacity);
		b->counters.alloc(CNT_COUNT);
		KGR_CUDA(cudaMemset(b->counters.ptr, 0, CNT_COUNT * sizeof(uint32_t)));
		b->table.alloc(batch_table_bytes(max_jobs));
		for (int r = 0; r < kgr_batcher::RING; r++) {
			KGR_CUDA(cudaHostAlloc((void **)&b->staging[r], batch_table_bytes(max_jobs), cudaHostAllocDefault));
			KGR_CUDA(cudaHostAlloc((void **)&b->stats_host[r], CNT_COUNT * sizeof(uint32_t), cudaHostAllocDefault));
			memset(b->stats_host[r], 0, CNT_COUNT * sizeof(uint32_t));
			KGR_CUDA(cudaEventCreateWithFlags(&b->done[r], cudaEventDisableTiming));
		}
		KGR_CUDA(cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking));
		KGR_CUDA(cudaStreamCreateWithFlags(&b->side.stream, cudaStreamNonBlocking));
		KGR_CUDA(cudaEventCreateWithFlags(&b->side.shaded, cudaEventDisableTiming));
		KGR_CUDA(cudaEventCreateWithFlags(&b->side.shadowed, cudaEventDisableTiming));
		*out = b.release();
	});
}

kgr_status kgr_batcher_render(kgr_batcher *b, const kgr_scene *scene, const kgr_batch_job *jobs, uint32_t n,
		const kgr_batch_options *options, void *stream)
{
	return guard_call([&] {
		KGR_REQUIRE(b && options, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		DeviceGuard guard(b->device);
		b->render(scene, jobs, n, *options, static_cast<cudaStream_t>(stream));
	});
}

kgr_status kgr_batcher_autotune(kgr_batcher *b, const kgr_scene *scene, const kgr_batch_job *jobs, uint32_t n,
		const kgr_batch_options *options, int32_t frames, void *stream, kgr_autotune_result *result)
{
	return guard_call([&] {
		KGR_REQUIRE(b && options && scene, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		KGR_REQUIRE(frames >= 1 && frames <= 256, KGR_ERR_INVALID_ARGUMENT, "frames must be 1..256");
		DeviceGuard guard(b->device);
		cudaStream_t st = static_cast<cudaStream_t>(stream);
		kgr_batch_options opt = *options;
		TraceTune old = b->tune;
		kgr_autotune_result res;
		memset(&res, 0, sizeof(res));
		try {
			double best = -1.0;
			for (const kgr_trace_tune &c : tune_candidates(scene)) {
				opt.layout = c.layout;
				b->tune.shadow = (int16_t)c.shadow;
				b->tune.block = (int16_t)c.block;
				b->tune.occupancy = (int16_t)c.occupancy;
				b->tune.stack = (int16_t)c.stack;
				double ms = time_frames([&] { b->render(scene, jobs, n, opt, st); }, frames, st);
				if (is_default_shape(c))
					res.default_ms = ms;
				if (best < 0.0 || ms < best) {
					best = ms;
					res.best = c;
				}
				res.candidates++;
			}
			/* second stage: the best shape with a shared-memory short stack */
			const kgr_trace_tune first = res.best;
			for (int k : kTuneStacks) {
				kgr_trace_tune c = first;
				c.stack = k;
				opt.layout = c.layout;
				b->tune.shadow = (int16_t)c.shadow;
				b->tune.block = (int16_t)c.block;
				b->tune.occupancy = (int16_t)c.occupancy;
				b->tune.stack = (int16_t)k;
				double ms = time_frames([&] { b->render(scene, jobs, n, opt, st); }, frames, st);
				res.candidates++;
				if (ms < best) {
					best = ms;
					res.best = c;
				}
			}
			res.best_ms = best;
		} catch (...) {
			b->tune = old;
			throw;
		}
		b->tune.shadow = (int16_t)res.best.shadow;
		b->tune.block = (int16_t)res.best.block;
		b->tune.occupancy = (int16_t)res.best.occupancy;
		b->tune.stack = (int16_t)res.best.stack;
		if (result)
			*result = res;
	});
}

kgr_status kgr_batcher_set_tune(kgr_batcher *b, const kgr_trace_tune *tune)
{
	return guard_call([&] {
		KGR_REQUIRE(b && tune, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		KGR_REQUIRE(tune->shadow == KGR_TRACE_GRID || tune->shadow == KGR_TRACE_PERSISTENT,
			KGR_ERR_INVALID_ARGUMENT, "unknown shadow kernel");
		KGR_REQUIRE(tune->block == 64 || tune->block == 128 || tune->block == 256, KGR_ERR_INVALID_ARGUMENT,
			"block must be 64, 128 or 256");
		KGR_REQUIRE(tune->occupancy == 0 || tune->occupancy == 1, KGR_ERR_INVALID_ARGUMENT, "occupancy is 0 or 1");
		KGR_REQUIRE(tune->stack == 0 || tune->stack == 8 || tune->stack == 16, KGR_ERR_INVALID_ARGUMENT,
			"stack is 0, 8 or 16");
		b->tune.shadow = (int16_t)tune->shadow;
		b->tune.block = (int16_t)tune->block;
		b->tune.occupancy = (int16_t)tune->occupancy;
		b->tune.stack = (int16_t)tune->stack;
	});
}

kgr_status kgr_batcher_ray_counts(kgr_batcher *b, uint64_t counts[3])
{
	return guard_call([&] {
		KGR_REQUIRE(b && counts, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		KGR_REQUIRE(b->last >= 0, KGR_ERR_INVALID_ARGUMENT, "no frame rendered yet");
		DeviceGuard guard(b->device);
		b->ray_counts(b->last, counts);
	});
}

kgr_status kgr_batcher_launch_info(const kgr_batcher *b, uint32_t *launches, int32_t *graph_replayed)
{
	return guard_call([&] {
		KGR_REQUIRE(b, KGR_ERR_INVALID_ARGUMENT, "NULL batcher");
		if (launches)
			*launches = b->last_launches;
		if (graph_replayed)
			*graph_replayed = b->last_graph;
	});
}

kgr_status kgr_batcher_destroy(kgr_batcher *b)
{
	return guard_call([&] { delete b; });
}

} /* extern "C" */

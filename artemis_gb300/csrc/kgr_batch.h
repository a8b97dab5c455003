/*
 * kgr_batch.h -- several path-traced jobs (images of any size, any spp
 * slice, each with its own camera and output buffers) rendered as one
 * wavefront: one generate launch over every job's paths, the shared
 * trace/shade/shadow launches of the path tracer, one accumulate launch.
 * Only generate and accumulate know about jobs; they read the job table from
 * device memory and use fixed grids, so a captured CUDA graph of one frame
 * replays for any mix of jobs that fits the path capacity.
 */
#ifndef KGR_BATCH_H_
#define KGR_BATCH_H_

#include "../../include/kgr_serve.h"
#include "kgr_wavefront.h"

namespace kgr {

/* One job of a batch in device memory (128 bytes).  Paths of the job are
 * path_offset + (s - s0) * npix + pixel for samples s in [s0, s0 + k). */
struct BatchJob {
	uint32_t path_offset, pix_offset, npix, width;
	uint32_t height, s0, k, spp;
	uint32_t frame;
	int32_t accumulate, samples, pad;
	float center[3], U[3], V[3], W[3];
	float4 *color, *normal, *albedo, *position;
};

struct BatchHeader {
	uint32_t njobs, total_paths, total_pix, pad;
};

/* Device table: the header, then max_jobs BatchJob records. */
inline size_t batch_table_bytes(uint32_t max_jobs) { return 16 + (size_t)max_jobs * sizeof(BatchJob); }

void batch_generate(const PathBuffers &pb, const BatchHeader *hdr, const BatchJob *jobs, cudaStream_t st);
void batch_accumulate(const PathBuffers &pb, const BatchHeader *hdr, const BatchJob *jobs, cudaStream_t st);

/* A second stream and two events: with them, batch_frame runs a bounce's
 * shadow rays on `stream` while the next bounce's closest hits run on the
 * frame's stream (forked and joined by events, so a captured frame keeps
 * the fork in its graph).  stream = nullptr: everything in order. */
struct StreamPair {
	cudaStream_t stream;
	cudaEvent_t shaded, shadowed;
};

/* One frame of every job in the table: generate, depth loop, accumulate.
 * fp supplies max_depth, Russian roulette and the layout. */
void batch_frame(const DeviceScene &s, const PathBuffers &pb, const FrameParams &fp, const BatchHeader *hdr,
		const BatchJob *jobs, cudaStream_t st, const StreamPair &side);

} /* namespace kgr */

/* The batcher: path state for `capacity` paths, the device job table, pinned
 * staging copies of the table and of the frame's counters (a ring, so the
 * host can prepare the next frame while one runs), and the captured graphs. */
struct kgr_batcher {
	static const int RING = 4;
	int device = 0;
	uint32_t capacity = 0, max_jobs = 0;
	kgr::DevBuf<float4> f4[KGR_PATH_ARRAYS];
	kgr::DevBuf<uint32_t> queues[3], counters;
	kgr::DevBuf<unsigned char> table;
	unsigned char *staging[RING] = {};
	uint32_t *stats_host[RING] = {};
	uint32_t paths_in[RING] = {};
	cudaEvent_t done[RING] = {};
	int ring = 0, last = -1;
	cudaStream_t capture_stream = nullptr;
	kgr::StreamPair side = {nullptr, nullptr, nullptr};
	/* launch shape of the traversal stages (kgr_batcher_set_tune) */
	kgr::TraceTune tune = kgr::default_trace_tune();
	struct Graph {
		const kgr_scene *scene;
		int max_depth, rr, rr_start, layout;
		kgr::TraceTune tune;
		int eager_runs;
		cudaGraphExec_t exec;
	};
	std::vector<Graph> graphs;
	uint32_t last_launches = 0;
	int last_graph = 0;
	uint64_t graph_replays = 0;

	kgr::PathBuffers path_buffers();
	/* Enqueue one shared frame (see kgr_batcher_render). */
	void render(const kgr_scene *scene, const kgr_batch_job *jobs, uint32_t n, const kgr_batch_options &opt,
			cudaStream_t st);
	/* camera, bounce and shadow rays of ring slot r (waits for it) */
	void ray_counts(int r, uint64_t counts[3]);
	~kgr_batcher();
};

#endif

/*
 * kgr_wavefront.h -- device state of the wavefront integrators (path tracer
 * and ReSTIR DI/GI) and the launchers the attachments call.
 *
 * Paths live in structure-of-arrays buffers of 16-byte records indexed by
 * path id p; stages exchange work through queues of path ids compacted with
 * warp ballots.  Path id p = sample * pixels + pixel, so consecutive threads
 * of the first bounce trace neighbouring pixels.
 */
#ifndef KGR_WAVEFRONT_H_
#define KGR_WAVEFRONT_H_

#include <functional>

#include "kgr_internal.h"

namespace kgr {

enum Counter {
	CNT_Q0 = 0,        /* live paths in queue 0 */
	CNT_Q1 = 1,        /* live paths in queue 1 */
	CNT_SHADOW = 2,    /* shadow rays of this bounce */
	CNT_BOUNCE_TOTAL = 3,
	CNT_SHADOW_TOTAL = 4,
	CNT_FETCH_CLOSEST = 5, /* next queue entry of the persistent closest-hit kernel */
	CNT_FETCH_SHADOW = 6,  /* next queue entry of the persistent shadow kernel */
	CNT_COUNT = 8
};

struct PathBuffers {
	float4 *ray_o;  /* origin xyz */
	float4 *ray_d;  /* direction xyz, tmax */
	float4 *beta;   /* throughput */
	float4 *L;      /* radiance */
	float4 *seed;   /* seed bits xyz */
	float4 *hit;    /* prim bits, t, b1, b2 */
	float4 *sh_o;   /* shadow ray origin */
	float4 *sh_d;   /* shadow ray direction, tmax */
	/* the path radiance with this vertex's NEE term added as if its shadow
	 * ray were unblocked; L already holds it added as if blocked (shade
	 * computes both, the resolve keeps this one when the ray is unblocked) */
	float4 *pend_c;
	float4 *aov_n, *aov_a, *aov_p;
	uint32_t *queue[2];
	uint32_t *shadow_queue;
	uint32_t *counters;
	/* traversal visit counters (nodes, triangles) of the closest and the
	 * any-hit stage; NULL unless visit counting is on */
	unsigned long long *visits;
	uint32_t capacity;
	/* when set, the any-hit walks store each shadow ray's blocked flag
	 * (1 or 0) at its path id instead of resolving the path's pending
	 * light (visibility rays of other passes); with shadow_queue NULL the
	 * walks take rays 0 .. counters[CNT_SHADOW]-1 in order (the id of a
	 * ray is its position) */
	uint32_t *shadow_flags = nullptr;
};

/* The float4 arrays of the path state, in the order their allocators lay
 * them out. */
#define KGR_PATH_ARRAYS 12
inline void path_array_slots(PathBuffers &pb, float4 **slots[KGR_PATH_ARRAYS])
{
	float4 **f[KGR_PATH_ARRAYS] = {&pb.ray_o, &pb.ray_d, &pb.beta, &pb.L, &pb.seed, &pb.hit, &pb.sh_o, &pb.sh_d,
		&pb.pend_c, &pb.aov_n, &pb.aov_a, &pb.aov_p};
	for (int k = 0; k < KGR_PATH_ARRAYS; k++)
		slots[k] = f[k];
}

/* Stage kinds for the per-launch CUDA-event timing of an attachment. */
enum StageKind {
	STAGE_GENERATE = 0,
	STAGE_TRACE_CLOSEST = 1,
	STAGE_SHADE = 2,
	STAGE_SHADOW = 3,
	STAGE_ACCUMULATE = 4,
	STAGE_RESTIR_PRIMARY = 5,
	STAGE_RESTIR_TEMPORAL = 6,
	STAGE_RESTIR_SPATIAL = 7,
	STAGE_RESTIR_FINALIZE = 8,
	STAGE_CACHE_INFER = 9,  /* radiance-cache query + network + apply */
	STAGE_CACHE_TRAIN = 10, /* training paths + targets + gradient + Adam */
	/* the reuse passes' queued visibility rays; stages 6 and 7 then hold
	 * only their resampling kernels (gather, resample/merge, finish) */
	STAGE_RESTIR_TEMPORAL_VIS = 11,
	STAGE_RESTIR_SPATIAL_VIS = 12,
	/* the "mamba" attachment: secondary rays, the probe splat, the probe
	 * upkeep (Sobel, raster, collapse, allocation), the final gather */
	STAGE_MAMBA_SECONDARY = 13,
	STAGE_MAMBA_GATHER = 14,
	STAGE_MAMBA_PROBES = 15,
	STAGE_MAMBA_FINAL = 16,
	STAGE_COUNT = 17
};

/* Called after each launch of a multi-kernel pass with the stage it belongs
 * to (the attachment's per-launch event timing); may be empty. */
typedef std::function<void(int)> StageMark;

/* Streaming read of a buffer with 16-byte loads (bandwidth probe). */
void launch_read_probe(const float4 *buf, size_t n, float4 *sink, int iters, cudaStream_t st);

/* Launch shape of the traversal stages of the fast and wide layouts.  Every
 * shape gives the same hits (the per-ray walk is the same; only the
 * scheduling of rays onto threads differs), so the autotuner may pick any. */
enum TraceKernel {
	TRACE_GRID = 0,      /* one ray per thread, grid-stride loop */
	TRACE_PERSISTENT = 1 /* lanes refill from the queue as their rays end */
};

struct TraceTune {
	int16_t shadow;    /* TraceKernel of the shadow stage (closest hit is always persistent) */
	int16_t block;     /* threads per block: 64, 128 or 256 */
	int16_t occupancy; /* 1: registers capped so that 48 warps fit an SM */
	int16_t stack;     /* traversal stack entries a thread keeps in shared memory: 0, 8 or 16 */
};

/* The shape used when nothing was tuned.  The persistent shadow kernel:
 * with the speculative descent it beats the grid kernel on every scene
 * measured (1080p terrain: 3.4 against 4.8 ms a frame). */
inline TraceTune default_trace_tune()
{
	TraceTune t;
	t.shadow = TRACE_PERSISTENT;
	t.block = 128;
	t.occupancy = 0;
	t.stack = 0;
	return t;
}

/* Whether an autotuner candidate is the untuned shape (the fast layout with
 * default_trace_tune()): its time is reported as default_ms. */
inline bool is_default_shape(const kgr_trace_tune &c)
{
	TraceTune d = default_trace_tune();
	return c.layout == KGR_LAYOUT_FAST && c.shadow == d.shadow && c.block == d.block && c.occupancy == d.occupancy &&
		c.stack == d.stack;
}

struct FrameParams {
	uint32_t width, height, npix, spp, paths;
	float center[3], U[3], V[3], W[3];
	float prev_proj_view[16]; /* previous camera projection * view */
	int32_t max_depth;
	int32_t russian_roulette, rr_start_depth;
	uint32_t frame;
	int32_t accumulate, samples;
	int32_t layout;
	int32_t jitter;
	/* ReSTIR */
	int32_t candidates, temporal, temporal_mcap, spatial_neighbors, spatial_radius;
	/* ReSTIR GI */
	int32_t gi_capture; /* shade records the depth-1 vertex in aov_p/aov_n */
	int32_t gi_mcap, gi_neighbors, gi_radius;
	float gi_jmax;           /* shifts with a Jacobian outside [1 / jmax, jmax] are invalid */
	int32_t gi_confidence_rule; /* a neighbour's confidence is at most the centre's M */
	float prev_center[3];
	TraceTune tune;
};

/* 32-byte reservoir in two 16-byte SoA arrays:
 *   a[i] = {sample point xyz, light index bits}
 *   b[i] = {w, W, M bits, unused} */
struct ReservoirBuffers {
	float4 *a;
	float4 *b;
};

struct RestirFrameBuffers {
	ReservoirBuffers res[2];
	kgr_material *materials; /* per pixel */
	float4 *intermediate;
	float4 *auxiliary;
	/* between the launches of a spatial pass: per neighbour slot (k-major,
	 * k * npix + pixel) {neighbour pixel, M}; targets per slot, then one
	 * row of npix for the lighting rays; the shadow-ray queues of the two
	 * rounds (entries index targets), their counts and (entries 2, 3) the
	 * visibility kernels' fetch counters */
	int2 *neighbours;
	float *targets;
	uint32_t *vis_queue[2];
	/* two counter arrays of CNT_COUNT entries, one per round: the queue
	 * count at CNT_SHADOW, the any-hit walk's fetch counter at
	 * CNT_FETCH_SHADOW */
	uint32_t *vis_count;
	/* per slot of the target array: the queued shadow ray ({origin},
	 * {direction, tmax}) and the walk's blocked flag (per path for the
	 * primary pass's rays); vis_capacity slots, (KGR_MAX_NEIGHBORS + 1) *
	 * npix */
	float4 *vis_o, *vis_d;
	uint32_t *vis_flag;
	uint32_t vis_capacity;
	/* every queued visibility ray also counts here (the frame's shadow-ray
	 * total, CNT_SHADOW_TOTAL of the path counters) */
	uint32_t *ray_total;
};

/* Most neighbours a ReSTIR DI spatial pass takes (spatial_neighbors). */
#define KGR_MAX_NEIGHBORS 16
/* Kernels one ReSTIR DI spatial pass launches: gather, the any-hit walk of
 * the neighbours' rays, resample, the walk of the selection's rays,
 * finish. */
#define KGR_RESTIR_SPATIAL_LAUNCHES 5
/* Kernels the temporal pass launches (gather, walk, merge) and the primary
 * pass (selection, walk, blocked weights). */
#define KGR_RESTIR_TEMPORAL_LAUNCHES 3
#define KGR_RESTIR_PRIMARY_LAUNCHES 3

struct OutputBuffers {
	float4 *color, *normal, *albedo, *position;
};

/* --- path tracer (pt.cu) --- */
void pt_generate(const PathBuffers &pb, const FrameParams &fp, cudaStream_t st);
void pt_trace_closest(const DeviceScene &s, const PathBuffers &pb, int q, int layout, const TraceTune &tune,
		cudaStream_t st);
void pt_shade(const DeviceScene &s, const PathBuffers &pb, const FrameParams &fp, int depth, int q,
		cudaStream_t st);
/* shade that also advances the RNG at the last depth (ReSTIR keeps the
 * path's final seed as its auxiliary seed) */
void pt_shade_final_seed(const DeviceScene &s, const PathBuffers &pb, const FrameParams &fp, int depth,
		int q, cudaStream_t st);
void pt_shadow_resolve(const DeviceScene &s, const PathBuffers &pb, int layout, const TraceTune &tune,
		cudaStream_t st);
void pt_accumulate(const PathBuffers &pb, const FrameParams &fp, const OutputBuffers &out, cudaStream_t st);
void reset_counters(const PathBuffers &pb, int which_mask, cudaStream_t st);

/* --- ReSTIR DI (restir.cu) --- */
void restir_primary(const DeviceScene &s, const PathBuffers &pb, const FrameParams &fp,
		const RestirFrameBuffers &rb, int cur, cudaStream_t st);
void restir_finalize(const PathBuffers &pb, const FrameParams &fp, const RestirFrameBuffers &rb,
		const OutputBuffers &out, cudaStream_t st);
void restir_temporal(const DeviceScene &s, const FrameParams &fp, const RestirFrameBuffers &rb,
		const OutputBuffers &out, int cur, int prev, cudaStream_t st, const StageMark &mark = StageMark());
void restir_spatial(const DeviceScene &s, const FrameParams &fp, const RestirFrameBuffers &rb,
		const OutputBuffers &out, int in, int outbuf, cudaStream_t st, const StageMark &mark = StageMark());

int device_sm_count();

} /* namespace kgr */

#endif

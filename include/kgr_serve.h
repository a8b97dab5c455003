/*
 * kgr_serve.h -- batched path tracing and the render server of libkgr.
 *
 * Neither has a counterpart in the reference, whose attachments render one
 * image per render() call on stream 0 with a device synchronisation after
 * every launch (include/amadeus/path_tracer.cuh:140-166, include/amadeus/
 * restir.cuh:258-303).  They are the serving and batching layers that stand
 * beside the "path_tracer" and "restir_di" attachments of kgr.h and use the
 * same kernels:
 *
 *   kgr_batcher  packs path-traced jobs of any resolution and spp slice into
 *                one shared wavefront per frame, replayed as a CUDA graph;
 *   kgr_server   a request loop (one host thread) that admits render
 *                requests by a device-memory budget, keeps scenes and
 *                per-request accumulation buffers resident, advances every
 *                admitted request a slice of samples per tick through the
 *                batcher (continuous batching), and reports latencies.
 *
 * All functions return a kgr_status and never throw.
 */
#ifndef KGR_SERVE_H_
#define KGR_SERVE_H_

#include "kgr.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------- batching -- */

/* One job of a batch: samples [sample_begin, sample_begin + sample_count)
 * of a width x height image whose whole render has `spp` samples per pixel.
 * After calls that cover samples 0 .. spp-1 in order, the buffers hold what
 * kgr_render of the "path_tracer" attachment writes for the same camera,
 * frame, spp and depth settings (bit for bit). */
typedef struct kgr_batch_job {
	uint32_t width;
	uint32_t height;
	uint32_t spp;
	uint32_t sample_begin;
	uint32_t sample_count;
	uint32_t frame;      /* RNG stream index of the image, as kgr_launch_info.frame */
	int32_t accumulate;  /* blend with `samples` earlier samples, as kgr_launch_info */
	int32_t samples;
	float center[3];     /* camera of kgr_launch_info.camera */
	float ax_u[3];
	float ax_v[3];
	float ax_w[3];
	float *color;        /* device float4 [width * height]; any of the four may be NULL */
	float *normal;
	float *albedo;
	float *position;
} kgr_batch_job;

typedef struct kgr_batch_options {
	int32_t max_depth;
	int32_t russian_roulette;
	int32_t rr_start_depth;
	int32_t layout;    /* KGR_LAYOUT_* */
	int32_t use_graph; /* replay one captured CUDA graph per (scene, options) */
	int32_t reserved[3];
} kgr_batch_options;

typedef struct kgr_batcher kgr_batcher;

/* path_capacity: paths of one shared frame (sum over jobs of
 * width * height * sample_count), 1 .. 2^28; max_jobs: 1 .. 65536. */
kgr_status kgr_batcher_create(int32_t device, uint32_t path_capacity, uint32_t max_jobs, kgr_batcher **out);
/* Enqueue one shared frame of n jobs on `stream` (asynchronous).  The job
 * list is copied; output buffers must stay valid until the stream reaches
 * the frame's end. */
kgr_status kgr_batcher_render(kgr_batcher *b, const kgr_scene *scene, const kgr_batch_job *jobs, uint32_t n,
		const kgr_batch_options *options, void *stream);
/* The autotuner (kgr_autotune) for a batch: times `frames` frames of these
 * jobs with every launch shape the scene admits and keeps the fastest
 * shadow kernel and block size for later frames; result->best.layout is the
 * layout to pass in kgr_batch_options from then on.  The frames are real
 * renders into the jobs' buffers.  Synchronous. */
kgr_status kgr_batcher_autotune(kgr_batcher *b, const kgr_scene *scene, const kgr_batch_job *jobs, uint32_t n,
		const kgr_batch_options *options, int32_t frames, void *stream, kgr_autotune_result *result);
/* Set the shadow kernel and block size directly (layout goes in the options). */
kgr_status kgr_batcher_set_tune(kgr_batcher *b, const kgr_trace_tune *tune);
/* Rays of the last frame: camera, bounce and shadow (waits for the frame). */
kgr_status kgr_batcher_ray_counts(kgr_batcher *b, uint64_t counts[3]);
/* Launches of the last frame and whether it ran as a graph replay. */
kgr_status kgr_batcher_launch_info(const kgr_batcher *b, uint32_t *launches, int32_t *graph_replayed);
kgr_status kgr_batcher_destroy(kgr_batcher *b);

/* -------------------------------------------------------------- serving -- */

enum { KGR_REQUEST_PATH_TRACER = 0, KGR_REQUEST_RESTIR_DI = 1 };

/* Tick composition.  FCFS: the oldest request with samples left picks the
 * tick's scene, then requests of that scene join oldest first, each with as
 * many samples as fit.  FAIR: processor sharing -- the tick goes to the
 * scene of the request served longest ago, its requests share the path
 * capacity equally (a request too large for its share banks the share until
 * a whole sample fits), and capacity left over goes to the requests closest
 * to their next sample; a ReSTIR DI request's tick holds as many frames as
 * cost about a full path-tracer tick on its scene (by the ticks timed so
 * far, at least one frame); latency then grows with a request's size
 * instead of with the size of the requests queued before it. */
enum { KGR_SCHEDULE_FCFS = 0, KGR_SCHEDULE_FAIR = 1 };

typedef struct kgr_server_config {
	int32_t device;
	uint32_t path_capacity;   /* paths of one tick's shared frame */
	uint32_t max_jobs;        /* requests in one tick */
	uint32_t spp_per_tick;    /* samples a request advances per tick; 0 = as many as fit */
	uint64_t memory_budget;   /* bytes of request buffers (accumulation, reservoirs) admitted at once */
	int32_t layout;           /* KGR_LAYOUT_*; with autotune, the layout tuned per scene */
	int32_t use_graph;
	int32_t autotune;         /* tune each scene's traversal launch shape (kgr_batcher_autotune on a
	                           * 1280x720 batch) before its first tick */
	int32_t policy;           /* KGR_SCHEDULE_* */
} kgr_server_config;

typedef struct kgr_request {
	uint32_t scene;      /* id from kgr_server_add_scene */
	int32_t kind;        /* KGR_REQUEST_* */
	uint32_t width;
	uint32_t height;
	uint32_t spp;        /* path tracer: samples per pixel; ReSTIR DI: frames accumulated */
	uint32_t max_depth;
	uint32_t frame;
	int32_t russian_roulette;
	int32_t rr_start_depth;
	float eye[3];
	float target[3];
	float fov_deg;
	float *host_color;   /* width * height * 4 floats written at completion, or NULL */
} kgr_request;

typedef struct kgr_request_result {
	int32_t status;      /* KGR_OK or the request's error */
	int32_t done;
	double queue_ms;     /* submission -> admission */
	double latency_ms;   /* submission -> result in host memory */
	double service_ms;   /* first launch -> result */
	uint32_t ticks;      /* ticks the request took part in */
	uint32_t reserved;
} kgr_request_result;

typedef struct kgr_server_stats {
	uint64_t submitted, completed, failed;
	uint64_t rays;            /* camera + bounce + shadow rays of every tick, the ReSTIR DI reuse
	                           * passes' visibility rays included */
	uint64_t ticks;
	double busy_ms;           /* wall time from the first submission to the last completion */
	double latency_p50_ms, latency_p90_ms, latency_p99_ms, latency_max_ms;
	double mean_jobs_per_tick;
	uint64_t peak_budget_bytes;
	uint64_t graph_replays;
} kgr_server_stats;

typedef struct kgr_server kgr_server;

kgr_status kgr_server_create(const kgr_server_config *config, kgr_server **out);
/* Register a resident scene (it must outlive the server). */
kgr_status kgr_server_add_scene(kgr_server *s, const kgr_scene *scene, uint32_t *id);
/* Queue a request (returns at once); KGR_ERR_INVALID_ARGUMENT for a request
 * that can never run (unknown scene, zero size, more paths per sample than
 * the path capacity, buffers above the whole budget). */
kgr_status kgr_server_submit(kgr_server *s, const kgr_request *request, uint64_t *id);
/* Wait up to timeout_ms (< 0: forever) for a request; KGR_ERR_TIMEOUT if it
 * is not done by then.  A finished request's result stays readable. */
kgr_status kgr_server_wait(kgr_server *s, uint64_t id, double timeout_ms, kgr_request_result *result);
kgr_status kgr_server_stats_get(kgr_server *s, kgr_server_stats *stats);
/* Stop the loop: requests not finished fail with KGR_ERR_NOT_LOADED. */
kgr_status kgr_server_destroy(kgr_server *s);

#ifdef __cplusplus
}
#endif

#endif

/*
 * serve.cpp -- kgr_server: the render request loop.
 *
 * One host thread runs the loop; callers only queue requests and wait.
 *
 *   admission   pending requests, oldest first, are admitted while the sum
 *               of their buffer sizes stays within the memory budget (a
 *               request never overtakes an older one); an admitted request
 *               gets its device accumulation buffer (stream-ordered
 *               allocation from the device pool).
 *   ticks       each tick is one shared wavefront frame of the batcher: the
 *               oldest admitted request with samples left picks the scene
 *               and path settings, then every admitted path-tracer request
 *               with the same ones, oldest first, adds a slice of its
 *               samples (spp_per_tick, or as many as fit the path
 *               capacity).  Up to two ticks are in flight: the host
 *               composes the next while the GPU runs the current, and
 *               requests that arrive meanwhile join the next tick --
 *               continuous batching; behind a tick expected to run longer
 *               than KGR_SHORT_TICK_MS the next is composed only when it
 *               ends, so that a request arriving meanwhile can take it.
 *   ReSTIR DI   requests render their frames (temporal and spatial reuse
 *               inside the request, history reset at its start) through a
 *               resident "restir_di" attachment of their resolution, as a
 *               tick of their own on the same stream; under FAIR a tick
 *               holds as many frames as cost about a full path-tracer tick,
 *               by the scene's measured costs.
 *   costs       every tick is timed by CUDA events on the stream; the ms per
 *               path-traced path and per ReSTIR DI pixel-frame of each scene
 *               are kept as exponential averages.
 *   rays        a tick's rays are counted on the device: camera, bounce and
 *               shadow rays of the path tracer, and for ReSTIR DI also the
 *               reuse passes' visibility rays (read after each frame into
 *               pinned memory).
 *   completion  when a request's last tick is done its image is copied to
 *               the caller's host buffer on a copy stream (directly when the
 *               buffer is pinned, through a pinned staging buffer when it is
 *               not); then its buffers go back to the pool and its bytes to
 *               the budget, and waiters are woken.
 *
 * Scenes and the batcher's path state stay resident for the server's life,
 * and so do the ReSTIR attachments (reservoirs) of each resolution seen.
 * Latency = submission to result in host memory.  Every wait in the loop is
 * bounded (event queries with short sleeps); device work ends on its own.
 */
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "kgr_batch.h"

using namespace kgr;
using Clock = std::chrono::steady_clock;

#define KGR_SERVER_MAX_SCENES 256

namespace {

double ms_between(Clock::time_point a, Clock::time_point b)
{
	return std::chrono::duration<double, std::milli>(b - a).count();
}

enum Phase { PHASE_PENDING = 0, PHASE_ACTIVE = 1, PHASE_COPYING = 2, PHASE_DONE = 3 };

struct Request {
	uint64_t id = 0;
	kgr_request req;
	kgr_launch_info cam; /* camera (center, axes, matrices) of the request */
	Phase phase = PHASE_PENDING;
	int status = KGR_OK;
	Clock::time_point t_submit, t_admit, t_first, t_done;
	bool launched = false;
	uint32_t scheduled = 0, completed = 0, ticks = 0;
	double credit = 0.0;     /* FAIR: paths banked toward the next slice */
	uint64_t last_tick = 0;  /* FAIR: tick number of the last slice (0: none yet) */
	uint64_t bytes = 0;
	float4 *color = nullptr; /* device accumulation, width * height */
	float4 *aov = nullptr;   /* ReSTIR: normal, albedo, position */
	cudaEvent_t copied = nullptr;
	unsigned char *staging = nullptr; /* pinned copy when host_color is pageable */
	size_t staging_bytes = 0;
	uint64_t rays = 0;
};

struct TickJob {
	Request *r;
	uint32_t k;
};

struct Tick {
	std::vector<TickJob> jobs;
	int batch_slot = -1; /* the batcher's ring slot, or -1 for a ReSTIR tick */
	cudaEvent_t start = nullptr, ev = nullptr; /* timing events before and after the tick's work */
	kgr_attachment *restir = nullptr;
	uint32_t scene = 0;
	uint64_t work = 0;             /* paths (path tracer) or pixel-frames (ReSTIR DI) */
	double est_ms = 0.0;           /* expected device time by the scene's costs (0: not known yet) */
	uint32_t *frame_rays = nullptr; /* ReSTIR DI: pinned, bounce and shadow rays of each frame */
	size_t frame_rays_bytes = 0;
};

/* What a tick costs on a scene, from the ticks timed so far (exponential
 * average, 0 until the first): ms per path-traced path and per ReSTIR DI
 * pixel-frame. */
struct SceneCost {
	double pt = 0.0, restir = 0.0;
};

/* The cost of a ReSTIR DI pixel-frame against a path-traced path assumed
 * until a scene has had a tick of each kind (about what depth 8 measures). */
#define KGR_RESTIR_COST_RATIO 4.0
/* A second tick is composed while one runs only when the running one is
 * expected to take at most this long: a request that arrives during a long
 * tick then waits for that tick alone, not for the next one as well. */
#define KGR_SHORT_TICK_MS 4.0

/* A resident "restir_di" attachment of one resolution; `owner` is the
 * request whose frames it renders (its temporal history is that request's),
 * NULL while it waits in the pool. */
struct RestirEntry {
	uint32_t width, height;
	kgr_attachment *att;
	const void *owner;
};

uint64_t request_bytes(const kgr_request &q)
{
	uint64_t npix = (uint64_t)q.width * q.height;
	/* path tracer: the color accumulation; ReSTIR DI: color and three AOVs,
	 * two 32-byte reservoirs, the per-pixel material, intermediate and
	 * auxiliary terms, and the reuse passes' scratch for up to 16
	 * neighbours: {pixel, M} and a target per neighbour slot, a row of
	 * lighting targets, the two shadow-ray queues (16 * 8 + 17 * 4 +
	 * 16 * 4 + 17 * 4 = 328 bytes), and per target slot a shadow ray and
	 * its blocked flag (17 * 36 = 612 bytes) */
	return q.kind == KGR_REQUEST_RESTIR_DI ? npix * (64 + 64 + 64 + 32 + 328 + 612) : npix * 16;
}

} /* namespace */

struct kgr_server {
	kgr_server_config cfg;
	int device = 0;
	kgr_batcher *batcher = nullptr;
	cudaStream_t stream = nullptr, copy_stream = nullptr;
	std::vector<const kgr_scene *> scenes;
	/* per scene: tuned layout and launch shape (autotune), -1 = not yet */
	struct SceneTune {
		int layout = -1;
		kgr_trace_tune tune = {KGR_LAYOUT_FAST, KGR_TRACE_PERSISTENT, 128, 0, 0};
	};
	std::vector<SceneTune> scene_tune;
	std::vector<SceneCost> scene_cost;

	std::mutex mu; /* guards everything callers touch */
	std::condition_variable cv_done, cv_work;
	std::map<uint64_t, std::unique_ptr<Request>> requests;
	std::deque<Request *> pending;
	uint64_t next_id = 1;
	uint64_t budget_used = 0, peak_budget = 0;
	bool stop = false;
	uint64_t submitted = 0, completed = 0, failed = 0, rays = 0, ticks = 0, jobs_in_ticks = 0;
	std::vector<double> latencies;
	bool any_submit = false;
	Clock::time_point t_first_submit, t_last_done;

	/* owned by the loop thread */
	std::vector<Request *> active, copying;
	std::deque<Tick> inflight;
	std::vector<cudaEvent_t> event_pool, timing_pool;
	std::vector<RestirEntry> restir;
	std::multimap<size_t, unsigned char *> pinned_pool;
	std::thread loop;

	cudaEvent_t take_event()
	{
		if (!event_pool.empty()) {
			cudaEvent_t e = event_pool.back();
			event_pool.pop_back();
			return e;
		}
		cudaEvent_t e;
		KGR_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
		return e;
	}

	cudaEvent_t take_timing_event()
	{
		if (!timing_pool.empty()) {
			cudaEvent_t e = timing_pool.back();
			timing_pool.pop_back();
			return e;
		}
		cudaEvent_t e;
		KGR_CUDA(cudaEventCreate(&e));
		return e;
	}

	/* a tick's events and pinned buffer back to their pools */
	void release_tick(Tick &t)
	{
		if (t.start)
			timing_pool.push_back(t.start);
		if (t.ev)
			timing_pool.push_back(t.ev);
		t.start = t.ev = nullptr;
		if (t.frame_rays) {
			pinned_pool.emplace(t.frame_rays_bytes, reinterpret_cast<unsigned char *>(t.frame_rays));
			t.frame_rays = nullptr;
		}
	}

	unsigned char *take_pinned(size_t bytes, size_t &got)
	{
		auto it = pinned_pool.lower_bound(bytes);
		if (it != pinned_pool.end() && it->first <= 2 * bytes) {
			unsigned char *p = it->second;
			got = it->first;
			pinned_pool.erase(it);
			return p;
		}
		unsigned char *p = nullptr;
		KGR_CUDA(cudaHostAlloc((void **)&p, bytes, cudaHostAllocDefault));
		got = bytes;
		return p;
	}

	/* a request leaves the loop: result, budget, buffers */
	void finish(Request *r, int status)
	{
		if (r->staging && status == KGR_OK && r->req.host_color)
			memcpy(r->req.host_color, r->staging, (size_t)r->req.width * r->req.height * 16);
		if (r->staging) {
			pinned_pool.emplace(r->staging_bytes, r->staging);
			r->staging = nullptr;
		}
		if (r->color)
			cudaFreeAsync(r->color, stream);
		if (r->aov)
			cudaFreeAsync(r->aov, stream);
		r->color = r->aov = nullptr;
		for (auto &e : restir)
			if (e.owner == r)
				e.owner = nullptr; /* back to the pool: later work on it is stream-ordered */
		if (r->copied) {
			event_pool.push_back(r->copied);
			r->copied = nullptr;
		}
		std::lock_guard<std::mutex> lk(mu);
		bool admitted = r->phase != PHASE_PENDING;
		r->status = status;
		r->phase = PHASE_DONE;
		r->t_done = Clock::now();
		if (admitted)
			budget_used -= r->bytes;
		if (status == KGR_OK) {
			completed++;
			latencies.push_back(ms_between(r->t_submit, r->t_done));
		} else {
			failed++;
		}
		rays += r->rays;
		t_last_done = r->t_done;
		cv_done.notify_all();
	}

	void fail_active(Request *r, int status)
	{
		active.erase(std::remove(active.begin(), active.end(), r), active.end());
		finish(r, status);
	}

	/* ticks done on the device: count samples, start result copies */
	void retire(Tick &t)
	{
		uint64_t counts[3] = {0, 0, 0};
		if (t.batch_slot >= 0)
			batcher->ray_counts(t.batch_slot, counts);
		uint64_t total_paths = 0;
		for (auto &j : t.jobs)
			total_paths += (uint64_t)j.r->req.width * j.r->req.height * j.k;
		uint64_t tick_rays = counts[0] + counts[1] + counts[2];
		if (t.restir && t.frame_rays) {
			/* camera rays, then the bounce and the shadow and visibility
			 * rays the attachment counted, frame by frame */
			uint64_t npix = (uint64_t)t.jobs[0].r->req.width * t.jobs[0].r->req.height;
			for (uint32_t f = 0; f < t.jobs[0].k; f++)
				tick_rays += npix + t.frame_rays[2 * f] + t.frame_rays[2 * f + 1];
		}
		float ms = 0.0f;
		if (t.start && t.work && cudaEventElapsedTime(&ms, t.start, t.ev) == cudaSuccess && ms > 0.0f) {
			SceneCost &c = scene_cost[t.scene];
			double x = (double)ms / (double)t.work;
			double &v = t.restir ? c.restir : c.pt;
			v = v > 0.0 ? 0.7 * v + 0.3 * x : x;
		}
		cudaGetLastError();
		for (auto &j : t.jobs) {
			Request *r = j.r;
			/* rays shared out by paths */
			uint64_t paths = (uint64_t)r->req.width * r->req.height * j.k;
			r->rays += total_paths ? (uint64_t)((double)tick_rays * paths / total_paths) : 0;
			r->completed += j.k;
			if (r->completed < r->req.spp || r->phase != PHASE_ACTIVE)
				continue;
			/* last tick: copy the image out */
			active.erase(std::remove(active.begin(), active.end(), r), active.end());
			try {
				size_t bytes = (size_t)r->req.width * r->req.height * 16;
				KGR_CUDA(cudaStreamWaitEvent(copy_stream, t.ev, 0));
				if (r->req.host_color) {
					cudaPointerAttributes pa;
					bool pinned = cudaPointerGetAttributes(&pa, r->req.host_color) == cudaSuccess &&
						pa.type == cudaMemoryTypeHost;
					cudaGetLastError();
					void *dst = r->req.host_color;
					if (!pinned) {
						r->staging = take_pinned(bytes, r->staging_bytes);
						dst = r->staging;
					}
					KGR_CUDA(cudaMemcpyAsync(dst, r->color, bytes, cudaMemcpyDeviceToHost, copy_stream));
				}
				r->copied = take_event();
				KGR_CUDA(cudaEventRecord(r->copied, copy_stream));
				{
					std::lock_guard<std::mutex> lk(mu);
					r->phase = PHASE_COPYING;
				}
				copying.push_back(r);
			} catch (const Error &e) {
				set_last_error(e.what());
				finish(r, e.status);
			}
		}
		release_tick(t);
	}

	/* the attachment rendering request r: its own, or a free one of its
	 * resolution from the pool, or a new one */
	kgr_attachment *restir_for(const Request *r, uint32_t w, uint32_t h)
	{
		for (auto &e : restir)
			if (e.owner == r)
				return e.att;
		for (auto &e : restir)
			if (!e.owner && e.width == w && e.height == h) {
				e.owner = r;
				return e.att;
			}
		kgr_attachment *att = nullptr;
		KGR_REQUIRE(kgr_create("restir_di", &att) == KGR_OK, KGR_ERR_INTERNAL, kgr_last_error());
		kgr_context ctx = {w, h, device, 0};
		if (kgr_attach(att, &ctx) != KGR_OK || kgr_load(att) != KGR_OK) {
			std::string msg = kgr_last_error();
			kgr_destroy(att);
			throw Error(KGR_ERR_OUT_OF_MEMORY, "ReSTIR attachment: " + msg);
		}
		restir.push_back(RestirEntry{w, h, att, r});
		return att;
	}

	void set_opt_int(kgr_attachment *att, const char *name, int v, int tag)
	{
		kgr_value val = {tag, v, 0.0f, v, nullptr};
		KGR_REQUIRE(kgr_set_option(att, name, &val) == KGR_OK, KGR_ERR_INTERNAL, kgr_last_error());
	}

	/* frames of one ReSTIR DI request as a tick of their own: all of them
	 * (FCFS), or as many as a path-tracer tick holds paths (FAIR, at least
	 * one), so that other requests run between the frames of a large one */
	void launch_restir(Request *r)
	{
		Tick t;
		const kgr_request &q = r->req;
		kgr_attachment *att = restir_for(r, q.width, q.height);
		uint32_t first = r->scheduled;
		uint32_t count = q.spp - first;
		if (cfg.policy == KGR_SCHEDULE_FAIR) {
			/* as many frames as cost about what a full path-tracer tick
			 * costs on this scene, by the ticks timed so far */
			const SceneCost &c = scene_cost[q.scene];
			double ratio = (c.pt > 0.0 && c.restir > 0.0) ? c.restir / c.pt : KGR_RESTIR_COST_RATIO;
			double fit = (double)cfg.path_capacity / ((double)q.width * q.height * ratio);
			count = (uint32_t)std::max<double>(1.0, std::min<double>((double)count, std::floor(fit)));
		}
		if (first == 0)
			set_opt_int(att, "reset_history", 1, KGR_VALUE_BOOL);
		set_opt_int(att, "russian_roulette", q.russian_roulette ? 1 : 0, KGR_VALUE_BOOL);
		set_opt_int(att, "rr_start_depth", q.rr_start_depth, KGR_VALUE_INT);
		size_t npix = (size_t)q.width * q.height;
		kgr_launch_info info = r->cam;
		info.buffers.color = reinterpret_cast<float *>(r->color);
		info.buffers.normal = reinterpret_cast<float *>(r->aov);
		info.buffers.albedo = reinterpret_cast<float *>(r->aov + npix);
		info.buffers.position = reinterpret_cast<float *>(r->aov + 2 * npix);
		info.max_depth = (int32_t)q.max_depth;
		t.restir = att;
		t.scene = q.scene;
		t.work = (uint64_t)npix * count;
		t.est_ms = (double)t.work * scene_cost[q.scene].restir;
		try {
			t.frame_rays =
				reinterpret_cast<uint32_t *>(take_pinned(2 * sizeof(uint32_t) * count, t.frame_rays_bytes));
			t.start = take_timing_event();
			t.ev = take_timing_event();
			KGR_CUDA(cudaEventRecord(t.start, stream));
			for (uint32_t i = first; i < first + count; i++) {
				info.frame = q.frame + i;
				info.accumulate = i > 0;
				info.samples = (int32_t)i;
				KGR_REQUIRE(kgr_render(att, &info, scenes[q.scene], stream) == KGR_OK, KGR_ERR_CUDA,
					kgr_last_error());
				attachment_ray_totals_async(att, t.frame_rays + 2 * (i - first), stream);
			}
			KGR_CUDA(cudaEventRecord(t.ev, stream));
		} catch (const Error &) {
			/* copies into the pinned buffer may still be queued */
			cudaStreamSynchronize(stream);
			cudaGetLastError();
			release_tick(t);
			throw;
		}
		r->scheduled = first + count;
		r->last_tick = ticks + 1;
		t.jobs.push_back(TickJob{r, count});
		note_launch(t);
		inflight.push_back(std::move(t));
	}

	void note_launch(const Tick &t)
	{
		Clock::time_point now = Clock::now();
		std::lock_guard<std::mutex> lk(mu);
		for (auto &j : t.jobs) {
			if (!j.r->launched) {
				j.r->launched = true;
				j.r->t_first = now;
			}
			j.r->ticks++;
		}
		ticks++;
		jobs_in_ticks += t.jobs.size();
	}

	/* Tune scene `id` (loop thread, nothing in flight): the autotuner over a
	 * 1280x720 batch of a slice of samples into a scratch buffer. */
	void tune_scene(uint32_t id, const kgr_request &like)
	{
		SceneTune &t = scene_tune[id];
		const uint32_t w = 1280, h = 720;
		uint32_t k = cfg.spp_per_tick ? cfg.spp_per_tick : 4;
		while (k > 1 && (uint64_t)w * h * k > cfg.path_capacity)
			k--;
		float4 *buf = nullptr;
		KGR_CUDA(cudaMallocAsync((void **)&buf, (size_t)w * h * sizeof(float4), stream));
		kgr_launch_info cam;
		memset(&cam, 0, sizeof(cam));
		const float up[3] = {0.0f, 1.0f, 0.0f};
		kgr_camera_setup(like.eye, like.target, up, like.fov_deg, (float)w / (float)h, &cam);
		kgr_batch_job j;
		memset(&j, 0, sizeof(j));
		j.width = w;
		j.height = h;
		j.spp = k;
		j.sample_count = k;
		memcpy(j.center, cam.camera.center, 12);
		memcpy(j.ax_u, cam.camera.ax_u, 12);
		memcpy(j.ax_v, cam.camera.ax_v, 12);
		memcpy(j.ax_w, cam.camera.ax_w, 12);
		j.color = reinterpret_cast<float *>(buf);
		kgr_batch_options opt;
		memset(&opt, 0, sizeof(opt));
		opt.max_depth = (int32_t)like.max_depth;
		opt.russian_roulette = like.russian_roulette ? 1 : 0;
		opt.rr_start_depth = like.rr_start_depth;
		opt.use_graph = cfg.use_graph;
		kgr_autotune_result res;
		kgr_status st = kgr_batcher_autotune(batcher, scenes[id], &j, 1, &opt, 2, stream, &res);
		cudaFreeAsync(buf, stream);
		KGR_REQUIRE(st == KGR_OK, st, std::string("autotune: ") + kgr_last_error());
		t.layout = res.best.layout;
		t.tune = res.best;
	}

	/* FAIR composition over the requests of one scene (see KGR_SCHEDULE_FAIR). */
	void compose_fair(const std::vector<Request *> &group, std::vector<uint32_t> &slice)
	{
		size_t n = group.size();
		slice.assign(n, 0);
		double share = (double)cfg.path_capacity / (double)n;
		uint64_t room = cfg.path_capacity;
		for (size_t i = 0; i < n; i++) {
			Request *r = group[i];
			uint64_t npix = (uint64_t)r->req.width * r->req.height;
			uint32_t left = r->req.spp - r->scheduled;
			r->credit = std::min(r->credit + share, (double)npix * left);
			uint64_t k = (uint64_t)(r->credit / (double)npix);
			k = std::min<uint64_t>(k, left);
			if (cfg.spp_per_tick)
				k = std::min<uint64_t>(k, cfg.spp_per_tick);
			k = std::min<uint64_t>(k, room / npix);
			slice[i] = (uint32_t)k;
			room -= k * npix;
			r->credit -= (double)(k * npix);
		}
		/* leftover capacity: requests nearest to a whole sample first */
		std::vector<size_t> order(n);
		for (size_t i = 0; i < n; i++)
			order[i] = i;
		std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
			auto need = [&](size_t i) {
				Request *r = group[i];
				return (double)r->req.width * r->req.height - r->credit;
			};
			return need(a) < need(b);
		});
		for (size_t i : order) {
			Request *r = group[i];
			uint64_t npix = (uint64_t)r->req.width * r->req.height;
			uint32_t left = r->req.spp - r->scheduled - slice[i];
			uint64_t k = std::min<uint64_t>(left, room / npix);
			if (cfg.spp_per_tick)
				k = std::min<uint64_t>(k, cfg.spp_per_tick - std::min(cfg.spp_per_tick, slice[i]));
			if (!k)
				continue;
			slice[i] += (uint32_t)k;
			room -= k * npix;
			r->credit -= (double)(k * npix);
		}
	}

	/* compose and launch one tick; false when nothing is left to schedule */
	bool launch_tick()
	{
		Request *head = nullptr;
		for (Request *r : active)
			if (r->scheduled < r->req.spp) {
				if (cfg.policy != KGR_SCHEDULE_FAIR) {
					head = r;
					break;
				}
				/* FAIR: the request served longest ago (never served first) */
				if (!head || r->last_tick < head->last_tick)
					head = r;
			}
		if (!head)
			return false;
		if (head->req.kind == KGR_REQUEST_RESTIR_DI) {
			try {
				launch_restir(head);
			} catch (const Error &e) {
				set_last_error(e.what());
				fail_active(head, e.status);
			}
			return true;
		}
		const kgr_request &h = head->req;
		if (cfg.autotune && scene_tune[h.scene].layout < 0) {
			if (!inflight.empty())
				return false; /* tune with nothing in flight: its frames reuse the batcher's ring */
			try {
				tune_scene(h.scene, h);
			} catch (const Error &e) {
				set_last_error(e.what());
				scene_tune[h.scene].layout = cfg.layout; /* keep the configured shape */
			}
		}
		std::vector<Request *> group;
		for (Request *r : active) {
			const kgr_request &q = r->req;
			if (q.kind != KGR_REQUEST_PATH_TRACER || r->scheduled >= q.spp || q.scene != h.scene ||
					q.max_depth != h.max_depth || (q.russian_roulette != 0) != (h.russian_roulette != 0) ||
					q.rr_start_depth != h.rr_start_depth)
				continue;
			group.push_back(r);
		}
		if (cfg.policy == KGR_SCHEDULE_FAIR)
			std::stable_sort(group.begin(), group.end(),
				[](const Request *a, const Request *b) { return a->last_tick < b->last_tick; });
		std::vector<uint32_t> fair;
		if (cfg.policy == KGR_SCHEDULE_FAIR)
			compose_fair(group, fair);
		std::vector<kgr_batch_job> jobs;
		Tick t;
		uint64_t paths = 0;
		for (size_t gi = 0; gi < group.size(); gi++) {
			Request *r = group[gi];
			const kgr_request &q = r->req;
			uint64_t npix = (uint64_t)q.width * q.height;
			uint32_t k = q.spp - r->scheduled;
			if (cfg.spp_per_tick)
				k = std::min(k, cfg.spp_per_tick);
			uint64_t fit = (cfg.path_capacity - paths) / npix;
			if (fit < k)
				k = (uint32_t)fit;
			if (cfg.policy == KGR_SCHEDULE_FAIR)
				k = std::min(k, fair[gi]);
			if (k == 0)
				continue;
			kgr_batch_job j;
			memset(&j, 0, sizeof(j));
			j.width = q.width;
			j.height = q.height;
			j.spp = q.spp;
			j.sample_begin = r->scheduled;
			j.sample_count = k;
			j.frame = q.frame;
			memcpy(j.center, r->cam.camera.center, 12);
			memcpy(j.ax_u, r->cam.camera.ax_u, 12);
			memcpy(j.ax_v, r->cam.camera.ax_v, 12);
			memcpy(j.ax_w, r->cam.camera.ax_w, 12);
			j.color = reinterpret_cast<float *>(r->color);
			jobs.push_back(j);
			t.jobs.push_back(TickJob{r, k});
			paths += npix * k;
			if (jobs.size() >= cfg.max_jobs)
				break;
		}
		kgr_batch_options opt;
		memset(&opt, 0, sizeof(opt));
		opt.max_depth = (int32_t)h.max_depth;
		opt.russian_roulette = h.russian_roulette ? 1 : 0;
		opt.rr_start_depth = h.rr_start_depth;
		opt.layout = cfg.layout;
		opt.use_graph = cfg.use_graph;
		if (cfg.autotune) {
			const SceneTune &st = scene_tune[h.scene];
			opt.layout = st.layout;
			batcher->tune.shadow = (int16_t)st.tune.shadow;
			batcher->tune.block = (int16_t)st.tune.block;
			batcher->tune.occupancy = (int16_t)st.tune.occupancy;
			batcher->tune.stack = (int16_t)st.tune.stack;
		}
		if (jobs.empty()) {
			/* FAIR: every share of this scene is still banking toward a
			 * sample; serve the head alone */
			head->last_tick = ticks + 1;
			return true;
		}
		try {
			t.scene = h.scene;
			t.work = paths;
			t.est_ms = (double)paths * scene_cost[h.scene].pt;
			t.start = take_timing_event();
			t.ev = take_timing_event();
			KGR_CUDA(cudaEventRecord(t.start, stream));
			batcher->render(scenes[h.scene], jobs.data(), (uint32_t)jobs.size(), opt, stream);
			t.batch_slot = batcher->last;
			KGR_CUDA(cudaEventRecord(t.ev, stream));
		} catch (const Error &e) {
			set_last_error(e.what());
			release_tick(t);
			for (auto &j : t.jobs)
				fail_active(j.r, e.status);
			return true;
		}
		for (auto &j : t.jobs) {
			j.r->scheduled += j.k;
			j.r->last_tick = ticks + 1;
		}
		note_launch(t);
		inflight.push_back(std::move(t));
		return true;
	}

	void admit()
	{
		std::vector<Request *> admitted;
		{
			std::lock_guard<std::mutex> lk(mu);
			while (!pending.empty()) {
				Request *r = pending.front();
				if (budget_used + r->bytes > cfg.memory_budget)
					break;
				pending.pop_front();
				budget_used += r->bytes;
				peak_budget = std::max(peak_budget, budget_used);
				r->phase = PHASE_ACTIVE;
				r->t_admit = Clock::now();
				admitted.push_back(r);
			}
		}
		for (Request *r : admitted) {
			size_t npix = (size_t)r->req.width * r->req.height;
			cudaError_t e = cudaMallocAsync((void **)&r->color, npix * sizeof(float4), stream);
			if (e == cudaSuccess && r->req.kind == KGR_REQUEST_RESTIR_DI)
				e = cudaMallocAsync((void **)&r->aov, 3 * npix * sizeof(float4), stream);
			if (e != cudaSuccess) {
				cudaGetLastError();
				set_last_error(std::string("request buffers: ") + cudaGetErrorString(e));
				finish(r, KGR_ERR_OUT_OF_MEMORY);
				continue;
			}
			active.push_back(r);
		}
	}

	void run()
	{
		cudaSetDevice(device);
		for (;;) {
			bool worked = false;
			try {
				while (!inflight.empty() && cudaEventQuery(inflight.front().ev) == cudaSuccess) {
					retire(inflight.front());
					inflight.pop_front();
					worked = true;
				}
				for (size_t i = 0; i < copying.size();) {
					if (cudaEventQuery(copying[i]->copied) == cudaSuccess) {
						Request *r = copying[i];
						copying.erase(copying.begin() + i);
						finish(r, KGR_OK);
						worked = true;
					} else {
						i++;
					}
				}
				cudaGetLastError(); /* cudaErrorNotReady of the queries */
				admit();
				bool room = inflight.empty() || (inflight.size() == 1 && inflight.back().est_ms <= KGR_SHORT_TICK_MS);
				if (room && launch_tick())
					worked = true;
			} catch (const Error &e) {
				/* a failed CUDA call in the loop: every request in flight
				 * fails with it; the loop goes on for new requests */
				set_last_error(e.what());
				cudaStreamSynchronize(stream);
				cudaStreamSynchronize(copy_stream);
				cudaGetLastError();
				for (auto &t : inflight)
					release_tick(t);
				inflight.clear();
				std::vector<Request *> left = active;
				left.insert(left.end(), copying.begin(), copying.end());
				active.clear();
				copying.clear();
				for (Request *r : left)
					finish(r, e.status);
				worked = true;
			}
			std::unique_lock<std::mutex> lk(mu);
			if (stop)
				break;
			if (!worked) {
				bool device_busy = !inflight.empty() || !copying.empty();
				if (device_busy || !active.empty())
					cv_work.wait_for(lk, std::chrono::microseconds(50));
				else
					cv_work.wait_for(lk, std::chrono::milliseconds(20), [&] { return stop || !pending.empty(); });
			}
		}
		/* shutdown: let the device finish, fail what is left */
		cudaStreamSynchronize(stream);
		cudaStreamSynchronize(copy_stream);
		cudaGetLastError();
		while (!inflight.empty()) {
			release_tick(inflight.front());
			inflight.pop_front();
		}
		for (Request *r : copying)
			finish(r, KGR_OK);
		copying.clear();
		std::vector<Request *> left = active;
		active.clear();
		for (Request *r : left)
			finish(r, KGR_ERR_NOT_LOADED);
		std::deque<Request *> queued;
		{
			std::lock_guard<std::mutex> lk(mu);
			queued.swap(pending);
		}
		for (Request *r : queued)
			finish(r, KGR_ERR_NOT_LOADED);
	}

	~kgr_server()
	{
		DeviceGuard g(device);
		for (auto &e : restir)
			kgr_destroy(e.att);
		if (batcher)
			kgr_batcher_destroy(batcher);
		for (cudaEvent_t e : event_pool)
			cudaEventDestroy(e);
		for (cudaEvent_t e : timing_pool)
			cudaEventDestroy(e);
		for (auto &p : pinned_pool)
			cudaFreeHost(p.second);
		if (stream)
			cudaStreamDestroy(stream);
		if (copy_stream)
			cudaStreamDestroy(copy_stream);
	}
};

extern "C" {

kgr_status kgr_server_create(const kgr_server_config *config, kgr_server **out)
{
	return guard_call([&] {
		KGR_REQUIRE(config && out, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		*out = nullptr;
		KGR_REQUIRE(config->max_jobs >= 1, KGR_ERR_INVALID_ARGUMENT, "max_jobs must be >= 1");
		KGR_REQUIRE(config->memory_budget >= 1, KGR_ERR_INVALID_ARGUMENT, "memory_budget must be > 0");
		KGR_REQUIRE(config->layout == KGR_LAYOUT_FAST || config->layout == KGR_LAYOUT_THREADED ||
				config->layout == KGR_LAYOUT_WIDE || config->layout == KGR_LAYOUT_CW8,
			KGR_ERR_INVALID_ARGUMENT, "unknown layout");
		KGR_REQUIRE(config->policy == KGR_SCHEDULE_FCFS || config->policy == KGR_SCHEDULE_FAIR,
			KGR_ERR_INVALID_ARGUMENT, "unknown scheduling policy");
		int dev = pick_device_ordinal(config->device);
		DeviceGuard g(dev);
		std::unique_ptr<kgr_server> s(new kgr_server());
		s->cfg = *config;
		s->device = dev;
		/* the loop thread reads these without the lock: no reallocation */
		s->scenes.reserve(KGR_SERVER_MAX_SCENES);
		s->scene_tune.reserve(KGR_SERVER_MAX_SCENES);
		kgr_status st = kgr_batcher_create(dev, config->path_capacity, config->max_jobs, &s->batcher);
		KGR_REQUIRE(st == KGR_OK, st, std::string("batcher: ") + kgr_last_error());
		KGR_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
		KGR_CUDA(cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking));
		/* keep freed request buffers in the pool for the next requests */
		cudaMemPool_t pool;
		KGR_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
		uint64_t keep = UINT64_MAX;
		KGR_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
		kgr_server *raw = s.get();
		s->loop = std::thread([raw] { raw->run(); });
		*out = s.release();
	});
}

kgr_status kgr_server_add_scene(kgr_server *s, const kgr_scene *scene, uint32_t *id)
{
	return guard_call([&] {
		KGR_REQUIRE(s && scene && id, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		KGR_REQUIRE(scene->device == s->device, KGR_ERR_INVALID_ARGUMENT, "scene on another device");
		std::lock_guard<std::mutex> lk(s->mu);
		KGR_REQUIRE(s->scenes.size() < KGR_SERVER_MAX_SCENES, KGR_ERR_INVALID_ARGUMENT, "too many scenes");
		s->scenes.push_back(scene);
		s->scene_tune.emplace_back();
		s->scene_cost.emplace_back();
		*id = (uint32_t)(s->scenes.size() - 1);
	});
}

kgr_status kgr_server_submit(kgr_server *s, const kgr_request *request, uint64_t *id)
{
	return guard_call([&] {
		KGR_REQUIRE(s && request, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		const kgr_request &q = *request;
		KGR_REQUIRE(q.kind == KGR_REQUEST_PATH_TRACER || q.kind == KGR_REQUEST_RESTIR_DI, KGR_ERR_INVALID_ARGUMENT,
			"unknown request kind");
		KGR_REQUIRE(q.width >= 1 && q.height >= 1 && q.spp >= 1 && q.spp <= 65536, KGR_ERR_INVALID_ARGUMENT,
			"request sizes out of range");
		KGR_REQUIRE(q.max_depth <= 64, KGR_ERR_INVALID_ARGUMENT, "max_depth must be 0..64");
		uint64_t npix = (uint64_t)q.width * q.height;
		KGR_REQUIRE(npix < (1ull << 30), KGR_ERR_INVALID_ARGUMENT, "image too large");
		if (q.kind == KGR_REQUEST_PATH_TRACER)
			KGR_REQUIRE(npix <= s->cfg.path_capacity, KGR_ERR_INVALID_ARGUMENT,
				"one sample of the image exceeds the path capacity");
		else
			KGR_REQUIRE(q.max_depth >= 1, KGR_ERR_INVALID_ARGUMENT, "ReSTIR DI needs max_depth >= 1");
		std::unique_ptr<Request> r(new Request());
		r->req = q;
		r->bytes = request_bytes(q);
		KGR_REQUIRE(r->bytes <= s->cfg.memory_budget, KGR_ERR_INVALID_ARGUMENT,
			"request buffers exceed the whole memory budget");
		memset(&r->cam, 0, sizeof(r->cam));
		const float up[3] = {0.0f, 1.0f, 0.0f};
		kgr_status cs = kgr_camera_setup(q.eye, q.target, up, q.fov_deg, (float)q.width / (float)q.height, &r->cam);
		KGR_REQUIRE(cs == KGR_OK, KGR_ERR_INVALID_ARGUMENT, std::string("camera: ") + kgr_last_error());
		r->cam.resolution[0] = (float)q.width;
		r->cam.resolution[1] = (float)q.height;
		std::lock_guard<std::mutex> lk(s->mu);
		KGR_REQUIRE(!s->stop, KGR_ERR_NOT_LOADED, "server is stopping");
		KGR_REQUIRE(q.scene < s->scenes.size(), KGR_ERR_INVALID_ARGUMENT, "unknown scene id");
		r->id = s->next_id++;
		r->t_submit = Clock::now();
		if (!s->any_submit) {
			s->any_submit = true;
			s->t_first_submit = r->t_submit;
		}
		s->submitted++;
		s->pending.push_back(r.get());
		if (id)
			*id = r->id;
		s->requests.emplace(r->id, std::move(r));
		s->cv_work.notify_one();
	});
}

kgr_status kgr_server_wait(kgr_server *s, uint64_t id, double timeout_ms, kgr_request_result *result)
{
	return guard_call([&] {
		KGR_REQUIRE(s, KGR_ERR_INVALID_ARGUMENT, "NULL server");
		std::unique_lock<std::mutex> lk(s->mu);
		auto it = s->requests.find(id);
		KGR_REQUIRE(it != s->requests.end(), KGR_ERR_INVALID_ARGUMENT, "unknown request id");
		Request *r = it->second.get();
		auto done = [&] { return r->phase == PHASE_DONE; };
		if (timeout_ms < 0)
			s->cv_done.wait(lk, done);
		else
			s->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), done);
		if (result) {
			memset(result, 0, sizeof(*result));
			result->done = done() ? 1 : 0;
			result->status = r->status;
			result->ticks = r->ticks;
			if (r->phase != PHASE_PENDING && r->phase != PHASE_DONE)
				result->queue_ms = ms_between(r->t_submit, r->t_admit);
			if (done()) {
				if (r->t_admit.time_since_epoch().count())
					result->queue_ms = ms_between(r->t_submit, r->t_admit);
				result->latency_ms = ms_between(r->t_submit, r->t_done);
				if (r->launched)
					result->service_ms = ms_between(r->t_first, r->t_done);
			}
		}
		KGR_REQUIRE(done(), KGR_ERR_TIMEOUT, "request not finished");
		if (r->status != KGR_OK)
			set_last_error("request failed");
	});
}

kgr_status kgr_server_stats_get(kgr_server *s, kgr_server_stats *st)
{
	return guard_call([&] {
		KGR_REQUIRE(s && st, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		std::lock_guard<std::mutex> lk(s->mu);
		memset(st, 0, sizeof(*st));
		st->submitted = s->submitted;
		st->completed = s->completed;
		st->failed = s->failed;
		st->rays = s->rays;
		st->ticks = s->ticks;
		st->mean_jobs_per_tick = s->ticks ? (double)s->jobs_in_ticks / (double)s->ticks : 0.0;
		st->peak_budget_bytes = s->peak_budget;
		st->graph_replays = s->batcher ? s->batcher->graph_replays : 0;
		if (s->any_submit && s->completed + s->failed > 0)
			st->busy_ms = ms_between(s->t_first_submit, s->t_last_done);
		std::vector<double> l = s->latencies;
		std::sort(l.begin(), l.end());
		auto pct = [&](double p) {
			if (l.empty())
				return 0.0;
			size_t i = (size_t)ceil(p * (double)l.size()) - 1;
			return l[std::min(i, l.size() - 1)];
		};
		st->latency_p50_ms = pct(0.50);
		st->latency_p90_ms = pct(0.90);
		st->latency_p99_ms = pct(0.99);
		st->latency_max_ms = l.empty() ? 0.0 : l.back();
	});
}

kgr_status kgr_server_destroy(kgr_server *s)
{
	return guard_call([&] {
		if (!s)
			return;
		{
			std::lock_guard<std::mutex> lk(s->mu);
			s->stop = true;
		}
		s->cv_work.notify_all();
		if (s->loop.joinable())
			s->loop.join();
		delete s;
	});
}

} /* extern "C" */

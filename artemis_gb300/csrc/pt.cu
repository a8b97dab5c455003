/*
 * pt.cu -- wavefront path tracer: generate -> traverse (closest) -> shade
 * (NEE sample + BSDF sample, emits shadow rays and continuation rays into
 * compacted queues) -> traverse (any) + resolve -> ... -> accumulate.
 *
 * The integrator is the recursion of source/optix/amadeus_path_tracer.cu:
 * 133-201 (emission plus one-light NEE at every vertex, GGX continuation)
 * unrolled forward as L = sum_k beta_k (Le_k + Ld_k), with the Russian
 * roulette of source/optix/naive_path_tracer.cu:294-303 as an option.
 */
#include "kgr_device.cuh"
#include "kgr_shade.cuh"
#include "kgr_wavefront.h"

namespace kgr {

int device_sm_count()
{
	int dev = 0, sms = 152;
	cudaGetDevice(&dev);
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	return sms;
}

namespace {

inline int grid_for(uint32_t n, int block, int per_sm = 16)
{
	long long blocks = ((long long)n + block - 1) / block;
	long long cap = (long long)device_sm_count() * per_sm;
	if (blocks < 1)
		blocks = 1;
	return (int)(blocks < cap ? blocks : cap);
}

__device__ __forceinline__ f3 v3(const float *p) { return mk(p[0], p[1], p[2]); }

__device__ __forceinline__ void make_ray(const FrameParams &fp, uint32_t ix, uint32_t iy, f3 &seed,
		f3 &origin, f3 &direction)
{
	camera_ray(fp.center, fp.U, fp.V, fp.W, fp.width, fp.height, fp.jitter, ix, iy, seed, origin, direction);
}

__global__ void generate_kernel(PathBuffers pb, FrameParams fp)
{
	uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
	if (p == 0) {
		pb.counters[CNT_Q0] = fp.paths;
		pb.counters[CNT_Q1] = 0;
		pb.counters[CNT_SHADOW] = 0;
		pb.counters[CNT_BOUNCE_TOTAL] = 0;
		pb.counters[CNT_SHADOW_TOTAL] = 0;
	}
	if (p >= fp.paths)
		return;
	uint32_t s = p / fp.npix, pix = p - s * fp.npix;
	uint32_t ix = pix % fp.width, iy = pix / fp.width;
	uint32_t stream = fp.frame * fp.spp + s;
	f3 seed = pixel_seed(pix, stream, 0);
	f3 o, d;
	make_ray(fp, ix, iy, seed, o, d);
	pb.ray_o[p] = f4_of(o, 0.0f);
	pb.ray_d[p] = f4_of(d, 1e16f);
	pb.beta[p] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
	pb.L[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
	pb.seed[p] = f4_of(seed, 0.0f);
	pb.aov_n[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
	pb.aov_a[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
	pb.aov_p[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
	/* queue position p takes the path of sample s at the p-th pixel in tile order */
	pb.queue[0][p] = s * fp.npix + tiled_pixel(pix, fp.width, fp.height);
}

/* Sum per-thread visit counts into two 64-bit counters, one atomic per warp. */
__device__ __forceinline__ void add_visits(unsigned long long *dst, const TraceCounters &c)
{
	unsigned long long a = c.nodes, b = c.tris;
	for (int off = 16; off > 0; off >>= 1) {
		a += __shfl_down_sync(0xffffffffu, a, off);
		b += __shfl_down_sync(0xffffffffu, b, off);
	}
	if ((threadIdx.x & 31) == 0) {
		atomicAdd(dst, a);
		atomicAdd(dst + 1, b);
	}
}

template <int LAYOUT, bool COUNT>
__global__ void __launch_bounds__(128) trace_closest_kernel(DeviceScene s, PathBuffers pb, int q)
{
	const uint32_t n = pb.counters[q == 0 ? CNT_Q0 : CNT_Q1];
	const uint32_t *queue = pb.queue[q];
	uint32_t stride = gridDim.x * blockDim.x;
	TraceCounters cnt = {0, 0};
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
		uint32_t p = queue[i];
		float4 a = pb.ray_o[p], b = pb.ray_d[p];
		kgr_hit h;
		if (LAYOUT == KGR_LAYOUT_THREADED)
			trace_threaded<false, COUNT>(s, mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), b.w, h, &cnt);
		else
			trace_fast<false, COUNT>(s, mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), b.w, h, &cnt);
		pb.hit[p] = make_float4(__int_as_float(h.prim), h.t, h.b1, h.b2);
	}
	if (COUNT)
		add_visits(pb.visits, cnt);
}

/* Writes one shaded vertex into the path state of path p. */
struct WavefrontSink {
	const PathBuffers &pb;
	uint32_t p;
	int depth, gi_capture;
	f3 albedo;
	bool shadow = false, cont = false;
	__device__ __forceinline__ void vertex(const f3 &x, const f3 &n, const Material &m)
	{
		if (depth == 0) {
			pb.aov_n[p] = f4_of(n, 0.0f);
			pb.aov_a[p] = f4_of(albedo, 0.0f);
			pb.aov_p[p] = f4_of(x, 0.0f);
		} else if (depth == 1 && gi_capture) {
			/* the secondary vertex of a ReSTIR GI sample; w = 1 when its
			 * radiance may be reused toward other receivers */
			pb.aov_n[p] = f4_of(n, gi_reconnectable(m) ? 1.0f : 0.0f);
			pb.aov_p[p] = f4_of(x, 1.0f);
		}
	}
	__device__ __forceinline__ void emit(const f3 &add)
	{
		float4 Lv = pb.L[p];
		pb.L[p] = f4_of(mk(Lv.x, Lv.y, Lv.z) + add, 0.0f);
	}
	/* L += beta * (Le + Ld) waits for the shadow ray; nothing else changes
	 * L before the ray is resolved, so both outcomes are computed here: L
	 * takes the blocked one, pend_c the unblocked one, and the resolve
	 * copies pend_c into L when the ray is unblocked. */
	__device__ __forceinline__ void nee(float4 c, float4 e, float4 b, float4 o, float4 d)
	{
		float4 L = pb.L[p];
		pb.L[p] = nee_add(L, c, e, b, true);
		pb.pend_c[p] = nee_add(L, c, e, b, false);
		pb.sh_o[p] = o;
		pb.sh_d[p] = d;
		shadow = true;
	}
	__device__ __forceinline__ void next(const f3 &x, const f3 &wi, const f3 &beta)
	{
		pb.ray_o[p] = f4_of(x, 0.0f);
		pb.ray_d[p] = f4_of(wi, 1e16f);
		pb.beta[p] = f4_of(beta, 0.0f);
		cont = true;
	}
};

/* One vertex of amadeus_path_tracer.cu:133-201 for path p, whose ray hit
 * `hv`: the surface, the shading (NEE sample and continuation), then the
 * appends to the next bounce's queue and the shadow queue.  Every active
 * lane of the warp calls it (the appends vote over the active lanes). */
__device__ __forceinline__ void shade_hit(const DeviceScene &s, const PathBuffers &pb, const FrameParams &fp,
		int depth, int final_seed, uint32_t *next_queue, uint32_t *out_counter, uint32_t p, float4 hv)
{
	bool shadow = false, cont = false;
	kgr_hit h;
	h.prim = __float_as_int(hv.x);
	h.t = hv.y;
	h.b1 = hv.z;
	h.b2 = hv.w;
	float4 dv = pb.ray_d[p];
	SurfaceHit sh;
	if (surface(s, h, mk(dv.x, dv.y, dv.z), sh)) {
		WavefrontSink out{pb, p, depth, fp.gi_capture, sh.mat.diffuse};
		float4 sv = pb.seed[p];
		f3 seed = mk(sv.x, sv.y, sv.z);
		float4 bv = pb.beta[p];
		shade_surface(s, fp, depth, final_seed, sh, mk(bv.x, bv.y, bv.z), seed, out);
		shadow = out.shadow;
		cont = out.cont;
		pb.seed[p] = f4_of(seed, 0.0f);
	}
	queue_append(next_queue, out_counter, p, cont, pb.counters + CNT_BOUNCE_TOTAL);
	queue_append(pb.shadow_queue, pb.counters + CNT_SHADOW, p, shadow, pb.counters + CNT_SHADOW_TOTAL);
}

/* One vertex of amadeus_path_tracer.cu:133-201 for every queued path: a
 * miss adds the environment map along the ray (__miss__,
 * amadeus_path_tracer.cu:204-220) in place; the hits are shaded in full
 * warps (for_each_hit). */
#define SHADE_BLOCK 256
__global__ void __launch_bounds__(SHADE_BLOCK) shade_kernel(DeviceScene s, PathBuffers pb, FrameParams fp,
		int depth, int q, int final_seed)
{
	const int qn = q ^ 1;
	const uint32_t n = pb.counters[q == 0 ? CNT_Q0 : CNT_Q1];
	uint32_t *out_counter = pb.counters + (qn == 0 ? CNT_Q0 : CNT_Q1);
	uint32_t *next_queue = pb.queue[qn];
	const uint32_t *queue = pb.queue[q];
	for_each_hit<SHADE_BLOCK>(n,
		[&](uint32_t i, float4 &hv, bool &heavy) {
			uint32_t p = queue[i];
			hv = pb.hit[p];
			if (__float_as_int(hv.x) >= 0) {
				heavy = depth <= fp.max_depth;
			} else if (s.has_env) {
				/* the environment map along the ray, weighted by the path
				 * throughput */
				float4 dv = pb.ray_d[p], bv = pb.beta[p], Lv = pb.L[p];
				f3 add = mk(bv.x, bv.y, bv.z) * env_miss(s, mk(dv.x, dv.y, dv.z));
				pb.L[p] = f4_of(mk(Lv.x, Lv.y, Lv.z) + add, 0.0f);
			}
			return p;
		},
		[&](uint32_t p, float4 hv) { shade_hit(s, pb, fp, depth, final_seed, next_queue, out_counter, p, hv); });
}

/* is_occluded for every queued shadow ray, then Ld = contr / pdf and
 * L += beta * (Le + Ld) in the order of the recursion.  One ray per thread,
 * grid-stride over the queue. */
/* Minimum resident blocks per SM a launch shape asks the compiler for:
 * OCC = 1 caps registers so that 1536 threads (48 warps) fit an SM. */
#define KGR_MIN_BLOCKS(BLOCK, OCC) ((OCC) ? 1536 / (BLOCK) : 1)

/* The traversal stack of a kernel instantiation: SHORT entries a thread in
 * shared memory (the rest in local memory), or all in local memory. */
template <int SHORT, int BLOCK>
struct StackOf {
	typedef ShortStack<SHORT, BLOCK> type;
};
template <int BLOCK>
struct StackOf<0, BLOCK> {
	typedef LocalStack type;
};


template <int LAYOUT, bool COUNT, int BLOCK, int OCC = 0, int SHORT = 0>
__global__ void __launch_bounds__(BLOCK, KGR_MIN_BLOCKS(BLOCK, OCC)) shadow_resolve_kernel(DeviceScene s, PathBuffers pb)
{
	__shared__ int32_t short_stack[SHORT > 0 ? SHORT * BLOCK : 1];
	int32_t local_stack[KGR_STACK_DEPTH - SHORT];
	typename StackOf<SHORT, BLOCK>::type stack(short_stack + threadIdx.x, local_stack);
	const uint32_t n = pb.counters[CNT_SHADOW];
	uint32_t stride = gridDim.x * blockDim.x;
	TraceCounters cnt = {0, 0};
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
		uint32_t p = pb.shadow_queue ? pb.shadow_queue[i] : i;
		float4 a = pb.sh_o[p], b = pb.sh_d[p];
		kgr_hit h;
		bool occ;
		if (LAYOUT == KGR_LAYOUT_THREADED)
			occ = trace_threaded<true, COUNT>(s, mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), b.w, h, &cnt);
		else if (LAYOUT == KGR_LAYOUT_CW8)
			occ = trace_cw<true, COUNT>(s, mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), b.w, h, &cnt);
		else
			occ = trace_fast_stack<true, COUNT, LAYOUT>(s, mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), b.w, h, stack,
				&cnt);
		if (pb.shadow_flags) {
			pb.shadow_flags[p] = occ ? 1u : 0u;
			continue;
		}
		if (!occ)
			pb.L[p] = pb.pend_c[p];
	}
	if (COUNT)
		add_visits(pb.visits + 2, cnt);
}

/* Shadow-ray resolve: L holds L + beta * (Le + 0) already (the blocked
 * outcome, computed at shade); an unblocked ray replaces it with
 * L + beta * (Le + contr / pdf), computed at shade into pend_c. */
__device__ __forceinline__ void resolve_shadow(const PathBuffers &pb, uint32_t p, bool occ)
{
	if (pb.shadow_flags) {
		pb.shadow_flags[p] = occ ? 1u : 0u;
		return;
	}
	if (!occ)
		pb.L[p] = pb.pend_c[p];
}

/* Persistent traversal of the fast or wide layout: each lane takes a new ray
 * from the queue (one atomic per warp) as soon as its current ray is
 * finished, so a lane whose ray ends early does not idle until the longest
 * ray of its warp is done.  One loop iteration descends to a leaf and tests
 * it.  ANY: shadow rays, resolved into the path radiance.  The grid is sized
 * to the resident capacity of the GPU. */
template <bool ANY, bool COUNT, int LAYOUT, int BLOCK, int OCC = 0, int SHORT = 0>
__global__ void __launch_bounds__(BLOCK, KGR_MIN_BLOCKS(BLOCK, OCC)) fast_persistent_kernel(DeviceScene s,
		PathBuffers pb, int q)
{
	__shared__ int32_t short_stack[SHORT > 0 ? SHORT * BLOCK : 1];
	const uint32_t n = ANY ? pb.counters[CNT_SHADOW] : pb.counters[q == 0 ? CNT_Q0 : CNT_Q1];
	const uint32_t *queue = ANY ? pb.shadow_queue : pb.queue[q];
	uint32_t *fetch = pb.counters + (ANY ? CNT_FETCH_SHADOW : CNT_FETCH_CLOSEST);
	const int lane = threadIdx.x & 31;
	TraceCounters cnt = {0, 0};
	uint32_t p = 0;
	bool have = false, exhausted = false;
	FastRay r;
	kgr_hit best;
	int32_t best_rank = 0x7fffffff;
	int32_t local_stack[KGR_STACK_DEPTH - SHORT];
	typename StackOf<SHORT, BLOCK>::type stack(short_stack + threadIdx.x, local_stack);
	int32_t ref = 0;
	for (;;) {
		bool need = !have && !exhausted;
		unsigned m = __ballot_sync(0xffffffffu, need);
		if (m) {
			int leader = __ffs(m) - 1;
			uint32_t base = 0;
			if (lane == leader)
				base = atomicAdd(fetch, (uint32_t)__popc(m));
			base = __shfl_sync(0xffffffffu, base, leader);
			if (need) {
				uint32_t i = base + __popc(m & ((1u << lane) - 1u));
				if (i < n) {
					p = (ANY && !queue) ? i : queue[i];
					float4 a = ANY ? pb.sh_o[p] : pb.ray_o[p];
					float4 b = ANY ? pb.sh_d[p] : pb.ray_d[p];
					r = fast_ray(mk(a.x, a.y, a.z), mk(b.x, b.y, b.z));
					best.prim = -1;
					best.t = b.w;
					best.b1 = 0.0f;
					best.b2 = 0.0f;
					best_rank = 0x7fffffff;
					stack.clear();
					ref = 0;
					have = true;
				} else {
					exhausted = true;
				}
			}
		}
		if (!__any_sync(0xffffffffu, have))
			break;
		if (!have)
			continue;
		/* descend with the postponed-leaf rule (speculative_descend), then
		 * test the leaves the descent collected */
		int32_t leaf = 0;
		speculative_descend<LAYOUT, COUNT>(s, r, ref, leaf, best.t, stack, &cnt);
		bool occ = test_leaves<ANY, COUNT>(s, r, ref, leaf, best, best_rank, stack, &cnt);
		bool done = occ || ref == KGR_REF_NONE;
		if (done) {
			if (ANY)
				resolve_shadow(pb, p, occ);
			else
				pb.hit[p] = make_float4(__int_as_float(best.prim), best.t, best.b1, best.b2);
			have = false;
		}
	}
	if (COUNT)
		add_visits(pb.visits + (ANY ? 2 : 0), cnt);
}

/* The persistent traversal over the compressed eight-child layout: the
 * refill of fast_persistent_kernel, one cw_step (descend with postponed
 * leaves, then test) per iteration. */
template <bool ANY, bool COUNT, int BLOCK, int OCC = 0>
__global__ void __launch_bounds__(BLOCK, KGR_MIN_BLOCKS(BLOCK, OCC)) cw_persistent_kernel(DeviceScene s,
		PathBuffers pb, int q)
{
	const uint32_t n = ANY ? pb.counters[CNT_SHADOW] : pb.counters[q == 0 ? CNT_Q0 : CNT_Q1];
	const uint32_t *queue = ANY ? pb.shadow_queue : pb.queue[q];
	uint32_t *fetch = pb.counters + (ANY ? CNT_FETCH_SHADOW : CNT_FETCH_CLOSEST);
	const int lane = threadIdx.x & 31;
	TraceCounters cnt = {0, 0};
	uint32_t p = 0;
	bool have = false, exhausted = false;
	kgr_hit best;
	int32_t best_rank = 0x7fffffff;
	CwStack stack;
	CwWalk w;
	for (;;) {
		bool need = !have && !exhausted;
		unsigned m = __ballot_sync(0xffffffffu, need);
		if (m) {
			int leader = __ffs(m) - 1;
			uint32_t base = 0;
			if (lane == leader)
				base = atomicAdd(fetch, (uint32_t)__popc(m));
			base = __shfl_sync(0xffffffffu, base, leader);
			if (need) {
				uint32_t i = base + __popc(m & ((1u << lane) - 1u));
				if (i < n) {
					p = (ANY && !queue) ? i : queue[i];
					float4 a = ANY ? pb.sh_o[p] : pb.ray_o[p];
					float4 b = ANY ? pb.sh_d[p] : pb.ray_d[p];
					cw_begin(w, mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), stack);
					best.prim = -1;
					best.t = b.w;
					best.b1 = 0.0f;
					best.b2 = 0.0f;
					best_rank = 0x7fffffff;
					have = true;
				} else {
					exhausted = true;
				}
			}
		}
		if (!__any_sync(0xffffffffu, have))
			break;
		if (!have)
			continue;
		bool done = false;
		bool occ = cw_step<ANY, COUNT>(s, w, best, best_rank, stack, &cnt, done);
		if (occ || done) {
			if (ANY)
				resolve_shadow(pb, p, occ);
			else
				pb.hit[p] = make_float4(__int_as_float(best.prim), best.t, best.b1, best.b2);
			have = false;
		}
	}
	if (COUNT)
		add_visits(pb.visits + (ANY ? 2 : 0), cnt);
}

template <class K>
int resident_grid(K kernel, int block)
{
	int per_sm = 0;
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0) != cudaSuccess || per_sm < 1)
		per_sm = 1;
	return per_sm * device_sm_count();
}

/* One launch of a persistent traversal kernel over a resident grid (the
 * grid of each instantiation is computed once). */
template <bool ANY, bool COUNT, int LAYOUT, int BLOCK, int OCC = 0, int SHORT = 0>
void launch_persistent(const DeviceScene &s, const PathBuffers &pb, int q, cudaStream_t st)
{
	static const int g = resident_grid(fast_persistent_kernel<ANY, COUNT, LAYOUT, BLOCK, OCC, SHORT>, BLOCK);
	fast_persistent_kernel<ANY, COUNT, LAYOUT, BLOCK, OCC, SHORT><<<g, BLOCK, 0, st>>>(s, pb, q);
}

template <bool ANY, int LAYOUT, int OCC, int BLOCK>
void launch_persistent_stack(const DeviceScene &s, const PathBuffers &pb, int q, int stack, cudaStream_t st)
{
	if (stack == 16)
		launch_persistent<ANY, false, LAYOUT, BLOCK, OCC, 16>(s, pb, q, st);
	else if (stack == 8)
		launch_persistent<ANY, false, LAYOUT, BLOCK, OCC, 8>(s, pb, q, st);
	else
		launch_persistent<ANY, false, LAYOUT, BLOCK, OCC, 0>(s, pb, q, st);
}

template <bool ANY, int LAYOUT, int OCC>
void launch_persistent_occ(const DeviceScene &s, const PathBuffers &pb, int q, int block, int stack,
		cudaStream_t st)
{
	if (block == 64)
		launch_persistent_stack<ANY, LAYOUT, OCC, 64>(s, pb, q, stack, st);
	else if (block == 256)
		launch_persistent_stack<ANY, LAYOUT, OCC, 256>(s, pb, q, stack, st);
	else
		launch_persistent_stack<ANY, LAYOUT, OCC, 128>(s, pb, q, stack, st);
}

template <bool ANY, bool COUNT, int BLOCK, int OCC = 0>
void launch_cw_persistent(const DeviceScene &s, const PathBuffers &pb, int q, cudaStream_t st)
{
	static const int g = resident_grid(cw_persistent_kernel<ANY, COUNT, BLOCK, OCC>, BLOCK);
	cw_persistent_kernel<ANY, COUNT, BLOCK, OCC><<<g, BLOCK, 0, st>>>(s, pb, q);
}

/* The compressed layout's stack is per thread (node groups): the stack
 * knob does not apply. */
template <bool ANY>
void launch_cw_persistent_tuned(const DeviceScene &s, const PathBuffers &pb, int q, const TraceTune &t,
		cudaStream_t st)
{
	if (t.occupancy) {
		if (t.block == 64)
			launch_cw_persistent<ANY, false, 64, 1>(s, pb, q, st);
		else if (t.block == 256)
			launch_cw_persistent<ANY, false, 256, 1>(s, pb, q, st);
		else
			launch_cw_persistent<ANY, false, 128, 1>(s, pb, q, st);
	} else {
		if (t.block == 64)
			launch_cw_persistent<ANY, false, 64>(s, pb, q, st);
		else if (t.block == 256)
			launch_cw_persistent<ANY, false, 256>(s, pb, q, st);
		else
			launch_cw_persistent<ANY, false, 128>(s, pb, q, st);
	}
}

template <bool ANY, int LAYOUT>
void launch_persistent_block(const DeviceScene &s, const PathBuffers &pb, int q, const TraceTune &t,
		cudaStream_t st)
{
	if (t.occupancy)
		launch_persistent_occ<ANY, LAYOUT, 1>(s, pb, q, t.block, t.stack, st);
	else
		launch_persistent_occ<ANY, LAYOUT, 0>(s, pb, q, t.block, t.stack, st);
}

template <bool COUNT, int LAYOUT, int BLOCK, int OCC = 0, int SHORT = 0>
void launch_shadow_grid(const DeviceScene &s, const PathBuffers &pb, cudaStream_t st)
{
	static const int g = resident_grid(shadow_resolve_kernel<LAYOUT, COUNT, BLOCK, OCC, SHORT>, BLOCK);
	shadow_resolve_kernel<LAYOUT, COUNT, BLOCK, OCC, SHORT><<<g, BLOCK, 0, st>>>(s, pb);
}

template <int LAYOUT, int OCC, int BLOCK>
void launch_shadow_grid_stack(const DeviceScene &s, const PathBuffers &pb, int stack, cudaStream_t st)
{
	if (stack == 16)
		launch_shadow_grid<false, LAYOUT, BLOCK, OCC, 16>(s, pb, st);
	else if (stack == 8)
		launch_shadow_grid<false, LAYOUT, BLOCK, OCC, 8>(s, pb, st);
	else
		launch_shadow_grid<false, LAYOUT, BLOCK, OCC, 0>(s, pb, st);
}

template <int LAYOUT, int OCC>
void launch_shadow_grid_occ(const DeviceScene &s, const PathBuffers &pb, int block, int stack, cudaStream_t st)
{
	if (block == 64)
		launch_shadow_grid_stack<LAYOUT, OCC, 64>(s, pb, stack, st);
	else if (block == 256)
		launch_shadow_grid_stack<LAYOUT, OCC, 256>(s, pb, stack, st);
	else
		launch_shadow_grid_stack<LAYOUT, OCC, 128>(s, pb, stack, st);
}

template <int LAYOUT>
void launch_shadow_grid_block(const DeviceScene &s, const PathBuffers &pb, const TraceTune &t, cudaStream_t st)
{
	if (t.occupancy)
		launch_shadow_grid_occ<LAYOUT, 1>(s, pb, t.block, t.stack, st);
	else
		launch_shadow_grid_occ<LAYOUT, 0>(s, pb, t.block, t.stack, st);
}

/* accumulate (amadeus_path_tracer.cu:59-70), the frame's samples in order */
__global__ void accumulate_kernel(PathBuffers pb, FrameParams fp, OutputBuffers out)
{
	uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
	if (pix >= fp.npix)
		return;
	for (uint32_t sidx = 0; sidx < fp.spp; sidx++) {
		bool acc = fp.accumulate || sidx > 0;
		float count = (float)(fp.accumulate ? fp.samples + (int)sidx : (int)sidx);
		accumulate_path(out, pb, sidx * fp.npix + pix, pix, acc, count);
	}
}

} /* namespace */

void reset_counters(const PathBuffers &pb, int which_mask, cudaStream_t st)
{
	for (int k = 0; k < CNT_COUNT; k++)
		if (which_mask & (1 << k))
			KGR_CUDA(cudaMemsetAsync(pb.counters + k, 0, sizeof(uint32_t), st));
}

void pt_generate(const PathBuffers &pb, const FrameParams &fp, cudaStream_t st)
{
	generate_kernel<<<(fp.paths + 255) / 256, 256, 0, st>>>(pb, fp);
	KGR_CUDA(cudaGetLastError());
}

void pt_trace_closest(const DeviceScene &s, const PathBuffers &pb, int q, int layout, const TraceTune &tune,
		cudaStream_t st)
{
	bool c = pb.visits != nullptr;
	if (layout == KGR_LAYOUT_THREADED) {
		int grid = grid_for(pb.capacity, 128);
		if (c)
			trace_closest_kernel<KGR_LAYOUT_THREADED, true><<<grid, 128, 0, st>>>(s, pb, q);
		else
			trace_closest_kernel<KGR_LAYOUT_THREADED, false><<<grid, 128, 0, st>>>(s, pb, q);
	} else {
		KGR_CUDA(cudaMemsetAsync(pb.counters + CNT_FETCH_CLOSEST, 0, sizeof(uint32_t), st));
		if (layout == KGR_LAYOUT_CW8) {
			if (c)
				launch_cw_persistent<false, true, 128>(s, pb, q, st);
			else
				launch_cw_persistent_tuned<false>(s, pb, q, tune, st);
		} else if (layout == KGR_LAYOUT_WIDE) {
			if (c)
				launch_persistent<false, true, KGR_LAYOUT_WIDE, 128>(s, pb, q, st);
			else
				launch_persistent_block<false, KGR_LAYOUT_WIDE>(s, pb, q, tune, st);
		} else {
			if (c)
				launch_persistent<false, true, KGR_LAYOUT_FAST, 128>(s, pb, q, st);
			else
				launch_persistent_block<false, KGR_LAYOUT_FAST>(s, pb, q, tune, st);
		}
	}
	KGR_CUDA(cudaGetLastError());
}

void pt_shade(const DeviceScene &s, const PathBuffers &pb, const FrameParams &fp, int depth, int q,
		cudaStream_t st)
{
	int grid = grid_for(pb.capacity, SHADE_BLOCK);
	shade_kernel<<<grid, SHADE_BLOCK, 0, st>>>(s, pb, fp, depth, q, 0);
	KGR_CUDA(cudaGetLastError());
}

void pt_shade_final_seed(const DeviceScene &s, const PathBuffers &pb, const FrameParams &fp, int depth,
		int q, cudaStream_t st)
{
	int grid = grid_for(pb.capacity, SHADE_BLOCK);
	shade_kernel<<<grid, SHADE_BLOCK, 0, st>>>(s, pb, fp, depth, q, 1);
	KGR_CUDA(cudaGetLastError());
}

void pt_shadow_resolve(const DeviceScene &s, const PathBuffers &pb, int layout, const TraceTune &tune,
		cudaStream_t st)
{
	bool c = pb.visits != nullptr;
	if (layout == KGR_LAYOUT_THREADED) {
		int grid = grid_for(pb.capacity, 128);
		if (c)
			shadow_resolve_kernel<KGR_LAYOUT_THREADED, true, 128><<<grid, 128, 0, st>>>(s, pb);
		else
			shadow_resolve_kernel<KGR_LAYOUT_THREADED, false, 128><<<grid, 128, 0, st>>>(s, pb);
	} else if (c) {
		if (layout == KGR_LAYOUT_WIDE)
			launch_shadow_grid<true, KGR_LAYOUT_WIDE, 128>(s, pb, st);
		else if (layout == KGR_LAYOUT_CW8)
			launch_shadow_grid<true, KGR_LAYOUT_CW8, 128>(s, pb, st);
		else
			launch_shadow_grid<true, KGR_LAYOUT_FAST, 128>(s, pb, st);
	} else if (tune.shadow == TRACE_PERSISTENT) {
		KGR_CUDA(cudaMemsetAsync(pb.counters + CNT_FETCH_SHADOW, 0, sizeof(uint32_t), st));
		if (layout == KGR_LAYOUT_CW8)
			launch_cw_persistent_tuned<true>(s, pb, 0, tune, st);
		else if (layout == KGR_LAYOUT_WIDE)
			launch_persistent_block<true, KGR_LAYOUT_WIDE>(s, pb, 0, tune, st);
		else
			launch_persistent_block<true, KGR_LAYOUT_FAST>(s, pb, 0, tune, st);
	} else if (layout == KGR_LAYOUT_WIDE) {
		launch_shadow_grid_block<KGR_LAYOUT_WIDE>(s, pb, tune, st);
	} else if (layout == KGR_LAYOUT_CW8) {
		/* one instantiation per block size; the stack knob does not apply */
		if (tune.block == 64)
			launch_shadow_grid<false, KGR_LAYOUT_CW8, 64>(s, pb, st);
		else if (tune.block == 256)
			launch_shadow_grid<false, KGR_LAYOUT_CW8, 256>(s, pb, st);
		else
			launch_shadow_grid<false, KGR_LAYOUT_CW8, 128>(s, pb, st);
	} else {
		launch_shadow_grid_block<KGR_LAYOUT_FAST>(s, pb, tune, st);
	}
	KGR_CUDA(cudaGetLastError());
}

void pt_accumulate(const PathBuffers &pb, const FrameParams &fp, const OutputBuffers &out, cudaStream_t st)
{
	accumulate_kernel<<<(fp.npix + 255) / 256, 256, 0, st>>>(pb, fp, out);
	KGR_CUDA(cudaGetLastError());
}

} /* namespace kgr */

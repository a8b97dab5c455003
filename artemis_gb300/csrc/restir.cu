/*
 * restir.cu -- ReSTIR DI kernels: RIS at the primary vertex, the per-pixel
 * finalisation of the initial pass, temporal reuse and spatial reuse.
 *
 * Follows source/optix/amadeus_restir.cu: __closesthit__initial (:437-559)
 * for RIS with 32 candidates, __raygen__temporal (:213-291) and
 * __raygen__spatial (:317-434) with the bias-corrected normalisation of
 * :387-399.  Reservoirs are 32 bytes in two 16-byte SoA arrays; a sample is
 * a light index plus the point on it (Le and the light normal are looked up
 * from the light, which gives the same values the reference stores).
 */
#include "kgr_device.cuh"
#include "kgr_wavefront.h"

namespace kgr {

namespace {

/* Salt of the RIS reservoir's own stream (the reference seeds it from
 * std::random_device on the host, reservoir.cuh:29-36). */
#define KGR_RIS_SALT 0x9E3779B9u

/* A light sample: `light` is its place among the launch's quad lights and
 * triangle lights (quads first), -1 for none, or -- for a point on the
 * environment map -- the bits of -u, negative and never -1, with v in
 * env_v: the map is read again at (u, v), which gives the Le the reference
 * stores in DirectLightingSample. */
struct Sample {
	int32_t light;
	f3 point;
	float env_v;
};

__device__ __forceinline__ bool has_light(const Sample &smp) { return smp.light != -1; }

/* Le, light normal and type (0 quad, 1 triangle, 2 environment) of a sample */
__device__ __forceinline__ int emitter(const DeviceScene &s, const Sample &smp, f3 &Le, f3 &normal)
{
	if (smp.light >= 0) {
		if ((uint32_t)smp.light < s.quad_count) {
			QuadLight l = load_quad(s.quads, (uint32_t)smp.light);
			Le = l.intensity;
			normal = l.normal();
			return 0;
		}
		TriLight l = load_light(s.lights, (uint32_t)smp.light - s.quad_count);
		Le = l.intensity;
		normal = l.normal();
		return 1;
	}
	Le = env_fetch(s, -__int_as_float(smp.light), smp.env_v);
	normal = mk(0.0f);
	return 2;
}

/* Reservoir<T>::update/resample (include/amadeus/reservoir.cuh:43-62) */
struct Reservoir {
	Sample data;
	float w, W;
	int32_t M;
	f3 seed;
	__device__ __forceinline__ void init(const f3 &s)
	{
		data.light = -1;
		data.point = mk(0.0f);
		data.env_v = 0.0f;
		w = 0.0f;
		W = 0.0f;
		M = 0;
		seed = s;
	}
	__device__ __forceinline__ bool update(const Sample &sample, float weight)
	{
		w += weight;
		float eta = rand_uniform(seed);
		bool selected = (eta * w) < weight;
		if (selected)
			data = sample;
		M++;
		return selected;
	}
	__device__ __forceinline__ void resample(float target)
	{
		float d = target * M;
		W = (d > 0) ? w / d : 0.0f;
	}
};

__device__ __forceinline__ void load_res(const ReservoirBuffers &rb, uint32_t i, Sample &smp, float &w,
		float &W, int32_t &M)
{
	float4 a = rb.a[i], b = rb.b[i];
	smp.light = __float_as_int(a.w);
	smp.point = mk(a.x, a.y, a.z);
	smp.env_v = b.w;
	w = b.x;
	W = b.y;
	M = __float_as_int(b.z);
}

__device__ __forceinline__ void store_res(const ReservoirBuffers &rb, uint32_t i, const Sample &smp,
		float w, float W, int32_t M)
{
	rb.a[i] = make_float4(smp.point.x, smp.point.y, smp.point.z, __int_as_float(smp.light));
	rb.b[i] = make_float4(w, W, __int_as_float(M), smp.env_v);
}


/* target (amadeus_restir.cu:147-161) */
__device__ __forceinline__ float target(const DeviceScene &s, const Sample &smp, const SurfaceHit &hit)
{
	if (!has_light(smp))
		return 0.0f;
	f3 Le, ln;
	int type = emitter(s, smp, Le, ln);
	f3 D = smp.point - hit.x;
	float d = length(D);
	f3 Li = direct_unoccluded_typed(hit, Le, ln, type, D / d, d);
	return Li.x + Li.y + Li.z;
}

/* occluded_target (amadeus_restir.cu:163-178, via direct_occluded of
 * amadeus_common.cuh:399-421) is target() when the shadow ray from the
 * surface to the sample -- the any-hit walk over D / |D| up to |D| - eps --
 * is unblocked, and 0 when it is blocked.  The reuse kernels compute
 * target() and queue that ray (vis_ray); the path tracer's tuned any-hit
 * walk flags it, and the next kernel reads the target through vis_target. */

__device__ __forceinline__ f3 v3(const float *p) { return mk(p[0], p[1], p[2]); }

/* The reuse passes rebuild the surface from the per-pixel material, the
 * normal and position AOVs and wo = normalize(center - position)
 * (amadeus_restir.cu:226-240, 326-336). */
__device__ __forceinline__ SurfaceHit gbuffer_hit(const FrameParams &fp, const RestirFrameBuffers &rb,
		const OutputBuffers &out, uint32_t pix)
{
	SurfaceHit h;
	float4 pv = out.position[pix];
	float4 nv = out.normal[pix];
	f3 x = mk(pv.x, pv.y, pv.z);
	h.mat = load_material(rb.materials, pix);
	h.entering = false;
	h.n = mk(nv.x, nv.y, nv.z);
	h.wo = normalize(v3(fp.center) - x);
	h.x = x;
	return h;
}

/* The reuse passes' shadow rays.  The kernel that queues an entry (a slot
 * of the target array) also writes the entry's ray there, {origin} and
 * {D / |D|, |D| - eps} -- the ray of occluded_target from `from` towards
 * `to` (amadeus_common.cuh:399-421); the path tracer's tuned any-hit walk
 * takes the queue and stores a blocked flag per entry; the next kernel
 * reads an entry's target as 0 when its flag is set.  The queue count of
 * round q sits in a counter array of its own (vis_count + q * CNT_COUNT),
 * where the walk looks for it. */
__device__ __forceinline__ uint32_t *vis_n(const RestirFrameBuffers &rb, int q)
{
	return rb.vis_count + q * CNT_COUNT + CNT_SHADOW;
}

__device__ __forceinline__ void vis_ray(const RestirFrameBuffers &rb, uint32_t e, const f3 &from, const f3 &to)
{
	f3 D = to - from;
	float d = length(D);
	f3 Dn = D / d;
	rb.vis_o[e] = f4_of(from, 0.0f);
	rb.vis_d[e] = f4_of(Dn, d - KGR_SHADOW_EPS);
}

/* An entry's target after its walk.  An entry that was not queued holds
 * +0, or a target its reader ignores (not above 0), so a flag left from an
 * earlier round does not change what is read. */
__device__ __forceinline__ float vis_target(const RestirFrameBuffers &rb, uint32_t e)
{
	return rb.vis_flag[e] ? 0.0f : rb.targets[e];
}

/* RIS at the primary vertex, then the continuation ray. */
__global__ void __launch_bounds__(128) primary_kernel(DeviceScene s, PathBuffers pb, FrameParams fp,
		RestirFrameBuffers rb, int cur)
{
	const uint32_t n = pb.counters[CNT_Q0];
	uint32_t *out_counter = pb.counters + CNT_Q1;
	uint32_t stride = gridDim.x * blockDim.x;
	uint32_t iters = (n + stride - 1) / stride;
	ReservoirBuffers R = rb.res[cur];
	for (uint32_t it = 0; it < iters; it++) {
		uint32_t i = it * stride + blockIdx.x * blockDim.x + threadIdx.x;
		bool active = i < n;
		uint32_t p = active ? pb.queue[0][i] : 0;
		bool cont = false, shadow = false;
		if (active) {
			float4 hv = pb.hit[p];
			kgr_hit h;
			h.prim = __float_as_int(hv.x);
			h.t = hv.y;
			h.b1 = hv.z;
			h.b2 = hv.w;
			float4 dv = pb.ray_d[p];
			SurfaceHit sh;
			if (h.prim < 0) {
				/* __miss__ (amadeus_restir.cu:561-578): the environment map at
				 * (u, v) becomes the pixel's intermediate colour */
				if (s.has_env)
					pb.L[p] = f4_of(env_miss(s, mk(dv.x, dv.y, dv.z)), 0.0f);
			} else if (surface(s, h, mk(dv.x, dv.y, dv.z), sh)) {
				f3 n3 = sh.n;
				float sgn = sh.mat.type == KGR_SHADING_TRANSMISSION ? -1.0f : 1.0f;
				sh.x = sh.x + sgn * n3 * KGR_OFFSET_EPS;
				pb.aov_n[p] = f4_of(n3, 0.0f);
				pb.aov_a[p] = f4_of(sh.mat.diffuse, 0.0f);
				pb.aov_p[p] = f4_of(sh.x, 0.0f);
				float4 sv = pb.seed[p];
				f3 seed = mk(sv.x, sv.y, sv.z);
				Reservoir res;
				res.init(pixel_seed(p, fp.frame, KGR_RIS_SALT));
				for (int c = 0; c < fp.candidates; c++) {
					/* sample_direct (amadeus_common.cuh:301-377) */
					LightPoint lp;
					int li = sample_direct(s, sh.x, seed, lp);
					Sample smp;
					float pdf = 0.0f, tgt = 0.0f;
					if (li >= 0) {
						smp.light = lp.type == 2 ? __float_as_int(-lp.env_u) : (int32_t)li;
						smp.point = lp.point;
						smp.env_v = lp.env_v;
						pdf = lp.pdf;
						f3 D = smp.point - sh.x;
						float d = length(D);
						f3 Li = direct_unoccluded_typed(sh, lp.Le, lp.normal, lp.type, D / d, d);
						tgt = Li.x + Li.y + Li.z;
					} else {
						smp.light = -1;
						smp.point = mk(0.0f);
						smp.env_v = 0.0f;
					}
					res.update(smp, (pdf > 0) ? tgt / pdf : 0);
				}
				/* direct_occluded of the selection, resample, and the second
				 * visibility test of :522-523 (the same ray, so the same
				 * answer).  The reservoir is stored as if the selection were
				 * visible and its shadow ray queued: a blocked ray makes the
				 * target 0, so resample and the visibility factor give W = +0,
				 * which primary_blocked_kernel writes. */
				float tgt = 0.0f;
				if (has_light(res.data)) {
					f3 Le, ln;
					int type = emitter(s, res.data, Le, ln);
					f3 D = res.data.point - sh.x;
					float d = length(D);
					f3 Dn = D / d;
					f3 Li = direct_unoccluded_typed(sh, Le, ln, type, Dn, d);
					tgt = Li.x + Li.y + Li.z;
					pb.sh_o[p] = f4_of(sh.x, 0.0f);
					pb.sh_d[p] = f4_of(Dn, d - KGR_SHADOW_EPS);
					shadow = true;
				}
				res.resample(tgt); /* the visibility factor of a visible selection is 1 */
				store_res(R, p, res.data, res.w, res.W, res.M);
				/* per-pixel material (:526) */
				uint4 tr = __ldg(&s.tris[h.prim]);
				const float4 *src = reinterpret_cast<const float4 *>(s.materials + tr.w);
				float4 *dst = reinterpret_cast<float4 *>(rb.materials + p);
				for (int k = 0; k < 4; k++)
					dst[k] = __ldg(src + k);
				/* continuation (:531-558) */
				f3 wi;
				float pdf = 0.0f;
				f3 f = eval(sh, wi, pdf, seed);
				if (pdf > 0) {
					f3 T = f * fabsf(dot(wi, n3)) / pdf;
					float4 bv = pb.beta[p];
					f3 beta = mk(bv.x, bv.y, bv.z) * T;
					bool alive = true;
					if (fp.russian_roulette && 0 >= fp.rr_start_depth) {
						float qq = 1.0f - kmin(kmax(0.05f, beta.y), 1.0f);
						if (fract(seed.x) < qq)
							alive = false;
						else
							beta = beta / (1.0f - qq);
					}
					if (alive && 0 < fp.max_depth) {
						pb.ray_o[p] = f4_of(sh.x, 0.0f);
						pb.ray_d[p] = f4_of(wi, 1e16f);
						pb.beta[p] = f4_of(beta, 0.0f);
						cont = true;
					}
				}
				pb.seed[p] = f4_of(seed, 0.0f);
			}
		}
		queue_append(pb.queue[1], out_counter, p, cont, pb.counters + CNT_BOUNCE_TOTAL);
		queue_append(rb.vis_queue[0], vis_n(rb, 0), p, shadow, rb.ray_total);
	}
}

/* The selections' shadow rays queued by primary_kernel (in the shadow-ray
 * arrays, free until the first bounce is shaded) are walked by the tuned
 * any-hit walk, which flags each blocked one at its path; a blocked
 * selection's reservoir gets W = +0. */
__global__ void primary_blocked_kernel(RestirFrameBuffers rb, int cur)
{
	const uint32_t n = *vis_n(rb, 0);
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		uint32_t p = rb.vis_queue[0][i];
		if (rb.vis_flag[p])
			rb.res[cur].b[p].y = 0.0f;
	}
}

__device__ __forceinline__ void accumulate4(float4 *buf, uint32_t i, float4 v, bool acc, float count)
{
	if (acc) {
		float4 d = buf[i];
		d.x = (d.x * count + v.x) / (count + 1);
		d.y = (d.y * count + v.y) / (count + 1);
		d.z = (d.z * count + v.z) / (count + 1);
		d.w = (d.w * count + v.w) / (count + 1);
		buf[i] = d;
	} else {
		buf[i] = v;
	}
}

/* End of __raygen__initial (amadeus_restir.cu:126-143): indirect colour,
 * auxiliary seed, normal/albedo AOVs accumulated, position stored. */
__global__ void finalize_kernel(PathBuffers pb, FrameParams fp, RestirFrameBuffers rb, OutputBuffers out)
{
	uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
	if (pix >= fp.npix)
		return;
	float4 L = pb.L[pix];
	f3 c = mk(L.x, L.y, L.z);
	if (anynan(c))
		c = mk(1.0f, 0.0f, 1.0f);
	rb.intermediate[pix] = f4_of(c, 1.0f);
	float4 sv = pb.seed[pix];
	rb.auxiliary[pix] = make_float4(sv.x, sv.y, sv.z, 1.0f);
	bool acc = fp.accumulate != 0;
	float count = (float)fp.samples;
	accumulate4(out.normal, pix, pb.aov_n[pix], acc, count);
	accumulate4(out.albedo, pix, pb.aov_a[pix], acc, count);
	out.position[pix] = pb.aov_p[pix];
}

/* reproject (amadeus_restir.cu:181-210); out-of-image indices rejected */
__device__ __forceinline__ int reproject(const FrameParams &fp, int index, const f3 &x)
{
	if (fp.samples > 0)
		return index;
	const float *m = fp.prev_proj_view;
	float q[4];
	for (int i = 0; i < 4; i++)
		q[i] = m[0 * 4 + i] * x.x + m[1 * 4 + i] * x.y + m[2 * 4 + i] * x.z + m[3 * 4 + i] * 1.0f;
	float u = q[0] / q[3];
	float v = q[1] / q[3];
	bool in_u = (u >= -1.0f && u <= 1.0f);
	bool in_v = (v >= -1.0f && v <= 1.0f);
	if (!(in_u && in_v))
		return -1;
	u = (u + 1.0f) * 0.5f;
	v = (v + 1.0f) * 0.5f;
	int ix = (int)((double)(u * (float)fp.width) + 0.5);
	int iy = (int)((double)(v * (float)fp.height) + 0.5);
	if (ix < 0 || iy < 0 || ix >= (int)fp.width || iy >= (int)fp.height)
		return -1;
	return iy * (int)fp.width + ix;
}

/* Temporal reuse (amadeus_restir.cu:316-365) in three launches: the two
 * occluded targets -- the current reservoir's and the reprojected previous
 * one's -- are computed unoccluded with their shadow rays queued
 * (temporal_gather_kernel), the rays walked (a blocked ray makes its
 * target 0, occluded_target's result), then the merge
 * (temporal_merge_kernel).  Targets sit in rows 0 (current) and 1
 * (previous) of the spatial pass's target array, the reprojected pixel and
 * its M in the neighbour array: both are free until spatial reuse starts. */
__global__ void __launch_bounds__(128) temporal_gather_kernel(DeviceScene s, FrameParams fp, RestirFrameBuffers rb,
		OutputBuffers out, int cur, int prev)
{
	uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
	if (pix >= fp.npix)
		return;
	ReservoirBuffers C = rb.res[cur], P = rb.res[prev];
	Sample cs;
	float cw, cW;
	int32_t cM;
	load_res(C, pix, cs, cw, cW, cM);
	if (cM <= 0)
		return;
	SurfaceHit hit = gbuffer_hit(fp, rb, out, pix);
	int pindex = reproject(fp, (int)pix, hit.x);
	float t_current = target(s, cs, hit);
	rb.targets[pix] = t_current;
	/* +0 stays +0 whatever the ray; anything else is traced */
	bool ray = __float_as_uint(t_current) != 0u;
	f3 from = f3_of(out.position[pix]);
	if (ray)
		vis_ray(rb, pix, from, cs.point);
	queue_append(rb.vis_queue[0], vis_n(rb, 0), pix, ray, rb.ray_total);
	int32_t pM = 0;
	if (pindex >= 0) {
		Sample ps;
		float pw, pW;
		load_res(P, (uint32_t)pindex, ps, pw, pW, pM);
		if (pM > 0) {
			float t_previous = target(s, ps, hit);
			rb.targets[fp.npix + pix] = t_previous;
			bool pray = __float_as_uint(t_previous) != 0u;
			if (pray)
				vis_ray(rb, fp.npix + pix, from, ps.point);
			queue_append(rb.vis_queue[0], vis_n(rb, 0), fp.npix + pix, pray, rb.ray_total);
		}
	}
	rb.neighbours[pix] = make_int2(pindex, pM);
}

__global__ void __launch_bounds__(128) temporal_merge_kernel(DeviceScene s, FrameParams fp, RestirFrameBuffers rb,
		OutputBuffers out, int cur, int prev)
{
	uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
	if (pix >= fp.npix)
		return;
	ReservoirBuffers C = rb.res[cur], P = rb.res[prev];
	Sample cs;
	float cw, cW;
	int32_t cM;
	load_res(C, pix, cs, cw, cW, cM);
	if (cM <= 0)
		return;
	SurfaceHit hit = gbuffer_hit(fp, rb, out, pix);
	int2 pr = rb.neighbours[pix];
	float4 av = rb.auxiliary[pix];
	Reservoir merged;
	merged.init(mk(av.x, av.y, av.z));
	float t_current = vis_target(rb, pix);
	merged.update(cs, t_current * cW * cM);
	int32_t N = cM;
	if (pr.x >= 0) {
		Sample ps;
		float pw, pW;
		int32_t pM;
		load_res(P, (uint32_t)pr.x, ps, pw, pW, pM);
		if (pM > 0) {
			pM = pM < fp.temporal_mcap ? pM : fp.temporal_mcap;
			float t_previous = vis_target(rb, fp.npix + pix);
			merged.update(ps, t_previous * pW * pM);
			N += (t_previous > 0) * pM;
		}
	}
	merged.M = N;
	float t_merged = target(s, merged.data, hit);
	merged.resample(t_merged);
	store_res(C, pix, merged.data, merged.w, merged.W, merged.M);
}

/* sample_spatial_neighborhood (amadeus_restir.cu:294-314); 2 * M_PI is the
 * double constant of <math.h>, so theta is a double product rounded. */
__device__ __forceinline__ int spatial_neighbor(const FrameParams &fp, int index, f3 &seed)
{
	int width = (int)fp.width, height = (int)fp.height;
	int x = index % width;
	int y = index / width;
	f3 offset = rand_uniform_3f(seed);
	float theta = (float)(2.0 * 3.14159265358979323846 * (double)offset.x);
	float r = (float)fp.spatial_radius * ksqrt(offset.y);
	float st, ct;
	ksincos(theta, st, ct);
	int x0 = (int)((float)x + r * ct);
	int y0 = (int)((float)y + r * st);
	x0 = x0 < 0 ? 0 : (x0 > width - 1 ? width - 1 : x0);
	y0 = y0 < 0 ? 0 : (y0 > height - 1 ? height - 1 : y0);
	return x0 + y0 * width;
}

/* Spatial reuse (amadeus_restir.cu:367-433) as a wavefront of five launches
 * per pass.  Its shadow rays -- one per neighbour reservoir (occluded_target
 * at this pixel), one per neighbour for the bias correction (the selected
 * sample seen from the neighbour's surface) and the final lighting ray --
 * are queued with their rays and walked by the path tracer's tuned any-hit
 * walk, instead of inside the per-pixel loops.  Between the launches: per
 * neighbour slot (k-major, slot = i * npix + pixel) {neighbour pixel, M}
 * and a target value that reads as 0 once its ray is found blocked
 * (occluded_target's result); row KGR_MAX_NEIGHBORS of the target array holds the lighting
 * ray's 1 (visible) or 0; the merged reservoir sits in the output buffer
 * between resample and finish.  Every value is computed by the reference's
 * expressions in its order, and each pixel's random stream is replayed
 * draw for draw, so the result is the single-pass kernel's bit for bit.
 *
 * gather: the neighbours and, for each one with M > 0 and a light, the
 * unoccluded target at this pixel, with its shadow ray queued.  The random
 * stream advances as the resampling will draw it: one uniform for the
 * centre, three for each neighbour's offset, one for each neighbour with
 * M > 0. */
__global__ void __launch_bounds__(128) restir_gather_kernel(DeviceScene s, FrameParams fp, RestirFrameBuffers rb,
		OutputBuffers out, int inb)
{
	uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
	if (pix >= fp.npix)
		return;
	ReservoirBuffers IN = rb.res[inb];
	Sample cs;
	float cw, cW;
	int32_t cM;
	load_res(IN, pix, cs, cw, cW, cM);
	if (cM <= 0)
		return;
	SurfaceHit hit = gbuffer_hit(fp, rb, out, pix);
	f3 from = f3_of(out.position[pix]);
	float4 av = rb.auxiliary[pix];
	f3 seed = mk(av.x, av.y, av.z);
	rand_uniform(seed);
	for (int i = 0; i < fp.spatial_neighbors; i++) {
		int index0 = spatial_neighbor(fp, (int)pix, seed);
		uint32_t slot = (uint32_t)i * fp.npix + pix;
		Sample ns;
		float nw, nW;
		int32_t nM;
		load_res(IN, (uint32_t)index0, ns, nw, nW, nM);
		float t = 0.0f;
		bool ray = false;
		if (nM > 0) {
			if (has_light(ns)) {
				t = target(s, ns, hit);
				/* +0 stays +0 whatever the ray; -0 would become +0 if blocked */
				ray = __float_as_uint(t) != 0u;
			}
			rand_uniform(seed);
		}
		rb.neighbours[slot] = make_int2(index0, nM);
		rb.targets[slot] = t;
		if (ray)
			vis_ray(rb, slot, from, ns.point);
		queue_append(rb.vis_queue[0], vis_n(rb, 0), slot, ray, rb.ray_total);
	}
}

/* resample: the merged reservoir over the centre and the neighbours with
 * their occluded targets (Reservoir::update, the same draws), then the
 * bias correction's targets of the selected sample at each neighbour's
 * surface with their shadow rays queued, and the lighting ray queued. */
__global__ void __launch_bounds__(128) restir_resample_kernel(DeviceScene s, FrameParams fp, RestirFrameBuffers rb,
		OutputBuffers out, int inb, int outb)
{
	uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
	if (pix >= fp.npix)
		return;
	ReservoirBuffers IN = rb.res[inb], OUT = rb.res[outb];
	Sample cs;
	float cw, cW;
	int32_t cM;
	load_res(IN, pix, cs, cw, cW, cM);
	if (cM <= 0)
		return;
	SurfaceHit hit = gbuffer_hit(fp, rb, out, pix);
	float4 av = rb.auxiliary[pix];
	Reservoir merged;
	merged.init(mk(av.x, av.y, av.z));
	float t_current = target(s, cs, hit);
	merged.update(cs, t_current * cW * cM);
	int K = fp.spatial_neighbors;
	int32_t count = 0;
	for (int i = 0; i < K; i++) {
		rand_uniform_3f(merged.seed);
		uint32_t slot = (uint32_t)i * fp.npix + pix;
		int2 nb = rb.neighbours[slot];
		if (nb.y > 0) {
			Sample ns;
			float nw, nW;
			int32_t nM;
			load_res(IN, (uint32_t)nb.x, ns, nw, nW, nM);
			merged.update(ns, vis_target(rb, slot) * nW * nM);
		}
		count += nb.y;
	}
	merged.M = cM + count;
	for (int i = 0; i < K; i++) {
		uint32_t slot = (uint32_t)i * fp.npix + pix;
		int2 nb = rb.neighbours[slot];
		if (nb.y <= 0)
			continue;
		float t = 0.0f;
		if (has_light(merged.data)) {
			SurfaceHit h0 = gbuffer_hit(fp, rb, out, (uint32_t)nb.x);
			h0.wo = hit.wo;
			h0.entering = true;
			t = target(s, merged.data, h0);
		}
		rb.targets[slot] = t;
		if (t > 0.0f)
			vis_ray(rb, slot, f3_of(out.position[nb.x]), merged.data.point);
		queue_append(rb.vis_queue[1], vis_n(rb, 1), slot, t > 0.0f, rb.ray_total);
	}
	uint32_t lit = (uint32_t)KGR_MAX_NEIGHBORS * fp.npix + pix;
	rb.targets[lit] = has_light(merged.data) ? 1.0f : 0.0f;
	if (has_light(merged.data))
		vis_ray(rb, lit, f3_of(out.position[pix]), merged.data.point);
	queue_append(rb.vis_queue[1], vis_n(rb, 1), lit, has_light(merged.data), rb.ray_total);
	store_res(OUT, pix, merged.data, merged.w, 0.0f, merged.M);
}

/* finish: Z = M of the centre and of every neighbour whose surface sees
 * the selected sample, W = w / (p^ Z), the shaded direct light and the
 * blend into the output (amadeus_restir.cu:387-433). */
__global__ void __launch_bounds__(128) restir_finish_kernel(DeviceScene s, FrameParams fp, RestirFrameBuffers rb,
		OutputBuffers out, int inb, int outb)
{
	uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
	if (pix >= fp.npix)
		return;
	ReservoirBuffers IN = rb.res[inb], OUT = rb.res[outb];
	int32_t cM = __float_as_int(IN.b[pix].z);
	f3 direct = mk(0.0f);
	if (cM > 0) {
		SurfaceHit hit = gbuffer_hit(fp, rb, out, pix);
		Sample data;
		float w, W0;
		int32_t M;
		load_res(OUT, pix, data, w, W0, M);
		int32_t Z = cM;
		for (int i = 0; i < fp.spatial_neighbors; i++) {
			uint32_t slot = (uint32_t)i * fp.npix + pix;
			int32_t size = rb.neighbours[slot].y;
			if (size <= 0)
				continue;
			if (vis_target(rb, slot) > 0.0f)
				Z += size;
		}
		float t_merged = target(s, data, hit);
		float denominator = t_merged * Z;
		float W = (denominator > 0.0f) ? w / denominator : 0.0f;
		f3 lighting = mk(0.0f);
		if (has_light(data) && vis_target(rb, (uint32_t)KGR_MAX_NEIGHBORS * fp.npix + pix) > 0.0f) {
			f3 Le, ln;
			int type = emitter(s, data, Le, ln);
			f3 D = data.point - hit.x;
			float d = length(D);
			f3 Dn = D / d;
			lighting = direct_unoccluded_typed(hit, Le, ln, type, Dn, d);
		}
		direct = hit.mat.emission + lighting * W;
		store_res(OUT, pix, data, w, W, M);
	} else {
		float4 b = OUT.b[pix];
		OUT.b[pix] = make_float4(0.0f, 0.0f, __int_as_float(0), b.w);
	}
	float4 iv = rb.intermediate[pix];
	f3 c = direct + mk(iv.x, iv.y, iv.z);
	float cwt = 1.0f + iv.w;
	if (anynan(c) || kisnan(cwt)) {
		c = mk(1.0f, 0.0f, 1.0f);
		cwt = 1.0f;
	}
	accumulate4(out.color, pix, f4_of(c, cwt), fp.accumulate != 0, (float)fp.samples);
}

/* The tuned any-hit walk over the queued entries of round q: their rays
 * (the slots' rays, or the paths' shadow rays for the primary pass), a
 * blocked flag per entry, the round's counter array. */
void vis_walk(const DeviceScene &s, const FrameParams &fp, const RestirFrameBuffers &rb, float4 *o, float4 *d,
		int q, cudaStream_t st)
{
	PathBuffers vb{};
	vb.sh_o = o;
	vb.sh_d = d;
	vb.shadow_queue = rb.vis_queue[q];
	vb.counters = rb.vis_count + q * CNT_COUNT;
	vb.shadow_flags = rb.vis_flag;
	vb.visits = nullptr;
	vb.capacity = rb.vis_capacity;
	pt_shadow_resolve(s, vb, fp.layout, fp.tune, st);
}

/* both rounds' counter arrays to zero */
void vis_clear(const RestirFrameBuffers &rb, cudaStream_t st)
{
	KGR_CUDA(cudaMemsetAsync(rb.vis_count, 0, 2 * CNT_COUNT * sizeof(uint32_t), st));
}

} /* namespace */

void restir_primary(const DeviceScene &s, const PathBuffers &pb, const FrameParams &fp,
		const RestirFrameBuffers &rb, int cur, cudaStream_t st)
{
	int grid = (int)((pb.capacity + 127) / 128);
	int cap = device_sm_count() * 16;
	vis_clear(rb, st);
	primary_kernel<<<grid < cap ? grid : cap, 128, 0, st>>>(s, pb, fp, rb, cur);
	vis_walk(s, fp, rb, pb.sh_o, pb.sh_d, 0, st);
	primary_blocked_kernel<<<device_sm_count() * 8, 128, 0, st>>>(rb, cur);
	KGR_CUDA(cudaGetLastError());
}

void restir_finalize(const PathBuffers &pb, const FrameParams &fp, const RestirFrameBuffers &rb,
		const OutputBuffers &out, cudaStream_t st)
{
	finalize_kernel<<<(fp.npix + 255) / 256, 256, 0, st>>>(pb, fp, rb, out);
	KGR_CUDA(cudaGetLastError());
}

void restir_temporal(const DeviceScene &s, const FrameParams &fp, const RestirFrameBuffers &rb,
		const OutputBuffers &out, int cur, int prev, cudaStream_t st, const StageMark &mark)
{
	unsigned grid = (fp.npix + 127) / 128;
	auto done = [&](int stage) {
		if (mark)
			mark(stage);
	};
	vis_clear(rb, st);
	temporal_gather_kernel<<<grid, 128, 0, st>>>(s, fp, rb, out, cur, prev);
	done(STAGE_RESTIR_TEMPORAL);
	vis_walk(s, fp, rb, rb.vis_o, rb.vis_d, 0, st);
	done(STAGE_RESTIR_TEMPORAL_VIS);
	temporal_merge_kernel<<<grid, 128, 0, st>>>(s, fp, rb, out, cur, prev);
	done(STAGE_RESTIR_TEMPORAL);
	KGR_CUDA(cudaGetLastError());
}

void restir_spatial(const DeviceScene &s, const FrameParams &fp, const RestirFrameBuffers &rb,
		const OutputBuffers &out, int in, int outbuf, cudaStream_t st, const StageMark &mark)
{
	unsigned grid = (fp.npix + 127) / 128;
	auto done = [&](int stage) {
		if (mark)
			mark(stage);
	};
	vis_clear(rb, st);
	restir_gather_kernel<<<grid, 128, 0, st>>>(s, fp, rb, out, in);
	done(STAGE_RESTIR_SPATIAL);
	vis_walk(s, fp, rb, rb.vis_o, rb.vis_d, 0, st);
	done(STAGE_RESTIR_SPATIAL_VIS);
	restir_resample_kernel<<<grid, 128, 0, st>>>(s, fp, rb, out, in, outbuf);
	done(STAGE_RESTIR_SPATIAL);
	vis_walk(s, fp, rb, rb.vis_o, rb.vis_d, 1, st);
	done(STAGE_RESTIR_SPATIAL_VIS);
	restir_finish_kernel<<<grid, 128, 0, st>>>(s, fp, rb, out, in, outbuf);
	done(STAGE_RESTIR_SPATIAL);
	KGR_CUDA(cudaGetLastError());
}

} /* namespace kgr */

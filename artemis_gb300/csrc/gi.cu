/*
 * gi.cu -- ReSTIR GI: reservoir resampling of one-bounce path samples.
 *
 * The reference has no working ReSTIR GI (its PathSample reservoirs in
 * include/optix/parameters.cuh:34-60 are never read by compiled code; a
 * dormant sketch lies in source/layers/optix_rt.cu:670-856).  This follows
 * that sketch where it is specific -- neighbours rejected when their
 * normals differ by more than 10 degrees or their depth by more than 10% --
 * and otherwise the reconnection-shift formulation of ReSTIR GI:
 *
 *  sample     x_s, n_s: the secondary vertex; L_o: radiance leaving x_s
 *             toward the primary vertex x_v (emission + NEE + the rest of
 *             the path, max depth as configured)
 *  target     p^_q(s) = sum_rgb(f_q(w) L_o) |n_q . w|, w = x_s - x_q
 *             normalised: the sample's contribution at receiver q.  The
 *             sketch's target (the largest component of L_o alone) leaves
 *             the receiver's BSDF out, so a neighbour's sample that lands in
 *             a narrow GGX lobe of q gets weight ~1/pdf of another surface
 *             and shades as a firefly; with the BSDF in the target the
 *             shaded value f L_o |n.w| W is w_sum / Z up to colour.
 *  initial    BSDF-sampled direction at x_v, source pdf p;
 *             w = p^_v(s) / p, M = 1
 *  shift      reusing a sample created at receiver x_r for receiver x_q
 *             multiplies its weight by the Jacobian
 *             |J| = (|cos phi_q| / |cos phi_r|) (|x_r - x_s|^2 / |x_q - x_s|^2),
 *             phi the angle at x_s between n_s and the receiver
 *  temporal   previous frame's reservoir at the reprojected pixel, M capped
 *  spatial    k neighbours in a disk, shadow ray to each reused sample
 *  weights    candidates are resampled with w_i = p^_q(y_i) |J_i| W_i M_i;
 *             the selected y (from domain j) gets the balance-heuristic
 *             contribution weight (Bitterli et al. 2020, the MIS form of
 *             their unbiased combination, with confidence weights M):
 *               W = p^<-j(y) w_sum / (p^_q(y) D),
 *               D = sum_i M_i p^<-i(y),  p^<-i(y) = p^_i(y) |J_q->i| v_i(y)
 *             over the centre, and the history or the neighbours; v_i is
 *             a visibility ray from receiver i (taken as 1 for the
 *             history).  A spatial neighbour's confidence M_i is at most
 *             the centre's M (gi_neighbor_confidence).  The uniform 1/Z
 *             weight it replaces keeps W ~
 *             1/p^_q(y), which a neighbour with a much larger p^ for the
 *             same sample turns into an unbounded contribution; here the
 *             small p^_q(y) cancels in the neighbour's weight.  Normalised
 *             in FP64.
 *  shading    f(x_v, w) L_o |n_v . w| W with a visibility ray, plus the
 *             primary vertex's emission and its ReSTIR DI direct light
 *
 *  reconnect  only samples whose secondary vertex is rough (gi_reconnectable)
 *             move to another pixel's receiver: spatial candidates that are
 *             not are skipped, and a selected sample that is not can only
 *             have come from the centre.  The history at the reprojected
 *             pixel is reused whatever its vertex (the receiver moves by
 *             less than a pixel).
 *
 * Reservoirs are 32 bytes in two 16-byte SoA arrays:
 *   a = {x_s.xyz, bits(n_s octahedral 12+12, M 8)},
 *   b = {L_o.rgb, W with its sign bit set when the sample is not
 *        reconnectable}.
 * The G-buffer position's w holds the pixel's material index + 1 (0: no
 * hit), so the history's receiver is known one frame later.
 */
#include "kgr_device.cuh"
#include "kgr_gi.h"

namespace kgr {

namespace {

#define KGR_GI_RIS_SALT 0x9E3779B9u
/* Random streams of the reuse passes: the temporal pass and spatial
 * iteration i draw from pixel_seed(pixel, frame, salt + pass).  Every pass
 * has its own stream; a pass that replayed another pass's uniforms would
 * resample candidates that already depend on those uniforms, and the
 * selection would no longer be independent of the candidates. */
#define KGR_GI_REUSE_SALT 0x47495255u
#define KGR_GI_COS_10DEG 0.984807753f
/* A shift whose Jacobian leaves [1/jmax, jmax] (jmax: option
 * gi_jacobian_max) is invalid: reconnecting to a secondary vertex much
 * nearer one receiver than the other (a crease, a contact) scales the
 * sample's weight without bound.  The range is closed under inversion, so
 * the bias correction -- which shifts the selected sample back to each
 * neighbour -- sees the same domains. */
__device__ __forceinline__ f3 v3(const float *p) { return mk(p[0], p[1], p[2]); }

struct GiSample {
	f3 xs, ns, Lo;
	bool valid;
	bool rc; /* reconnectable */
};

struct GiRes {
	GiSample s;
	float W;
	int32_t M;
};

__device__ __forceinline__ GiRes load_gi(const GiReservoirs &r, uint32_t i)
{
	float4 a = r.a[i], b = r.b[i];
	uint32_t w = __float_as_uint(a.w);
	GiRes g;
	g.s.xs = mk(a.x, a.y, a.z);
	g.s.ns = unpack_normal(w);
	g.s.Lo = mk(b.x, b.y, b.z);
	g.s.valid = true;
	g.s.rc = !signbit(b.w);
	g.W = fabsf(b.w);
	g.M = unpack_m(w);
	return g;
}

__device__ __forceinline__ void store_gi(const GiReservoirs &r, uint32_t i, const GiSample &s, float W, int32_t M)
{
	r.a[i] = make_float4(s.xs.x, s.xs.y, s.xs.z, __uint_as_float(pack_normal_m(s.ns, M)));
	r.b[i] = make_float4(s.Lo.x, s.Lo.y, s.Lo.z, s.rc ? W : -W);
}

/* Weighted reservoir over GI samples (reservoir.cuh:43-56 update rule);
 * src records the domain of the selected sample (-1: the centre). */
struct GiMerge {
	GiSample sel;
	float w;
	int32_t src;
	f3 seed;
	__device__ __forceinline__ void init(const f3 &s)
	{
		sel.xs = sel.ns = sel.Lo = mk(0.0f);
		sel.valid = false;
		sel.rc = true;
		w = 0.0f;
		src = -1;
		seed = s;
	}
	/* the update rule's draw: true when the candidate replaces the selection */
	__device__ __forceinline__ bool take(float weight)
	{
		w += weight;
		float eta = rand_uniform(seed);
		return (eta * w) < weight;
	}
	__device__ __forceinline__ void update(const GiSample &s, float weight, int32_t from)
	{
		if (take(weight)) {
			sel = s;
			src = from;
		}
	}
};

/* W = w_sum / p^ of a single candidate (M = 1), in double precision */
__device__ __forceinline__ float gi_normalise(float w_sum, int32_t Z, float target)
{
	if (!(target > 0.0f) || Z <= 0)
		return 0.0f;
	return (float)((double)w_sum / ((double)Z * (double)target));
}

/* Balance-heuristic contribution weight W = num w_sum / (D p^_q), FP64. */
__device__ __forceinline__ float gi_mis_weight(float w_sum, float num, float D, float target)
{
	if (!(target > 0.0f) || !(D > 0.0f))
		return 0.0f;
	return (float)(((double)num * (double)w_sum) / ((double)D * (double)target));
}

/* Solid-angle Jacobian of moving a sample's receiver from xr to xq; 0 for
 * an invalid shift. */
__device__ __forceinline__ float gi_jacobian(const f3 &xq, const f3 &xr, const GiSample &s, float jmax)
{
	f3 dq = xq - s.xs, dr = xr - s.xs;
	float lq2 = dot(dq, dq), lr2 = dot(dr, dr);
	float cq = fabsf(dot(s.ns, dq)) / ksqrt(lq2);
	float cr = fabsf(dot(s.ns, dr)) / ksqrt(lr2);
	float j = (cq / cr) * (lr2 / lq2);
	return (j >= 1.0f / jmax && j <= jmax) ? j : 0.0f;
}

/* The any-hit test of the visibility ray from `from` to `to`. */
__device__ __forceinline__ bool visible(const DeviceScene &s, int layout, const f3 &from, const f3 &to)
{
	f3 D = to - from;
	float d = length(D);
	kgr_hit h;
	return !trace<true>(s, layout, from, D / d, d - KGR_SHADOW_EPS, h);
}

/* Round q's queue count sits in its own counter array (vis_count +
 * q * CNT_COUNT), where the tuned any-hit walk looks for it; the fetch
 * counter of a one-ray-per-thread round sits in the same array. */
__device__ __forceinline__ uint32_t *gi_vis_n(const GiFrameBuffers &gb, int q)
{
	return gb.vis_count + q * CNT_COUNT + CNT_SHADOW;
}

/* A ray for the tuned any-hit walk at slot e: {from}, {D / |D|, |D| - eps}
 * with D = to - from, the ray visible() walks. */
__device__ __forceinline__ void gi_vis_ray(const GiFrameBuffers &gb, uint32_t e, const f3 &from, const f3 &to)
{
	f3 D = to - from;
	float d = length(D);
	gb.vis_o[e] = f4_of(from, 0.0f);
	gb.vis_d[e] = f4_of(D / d, d - KGR_SHADOW_EPS);
}

struct GBuf {
	f3 x, n;
	bool hit;
	uint32_t mat; /* material index (valid when hit) */
};

__device__ __forceinline__ GBuf gbuf(const float4 *pos, const float4 *nrm, uint32_t i)
{
	float4 p = pos[i], n = nrm[i];
	GBuf g;
	g.x = mk(p.x, p.y, p.z);
	g.n = mk(n.x, n.y, n.z);
	g.hit = p.w > 0.0f;
	g.mat = g.hit ? (uint32_t)p.w - 1u : 0u;
	return g;
}

/* the reference sketch's geometric test: normals within 10 degrees, view
 * depth within 10% (optix_rt.cu:745-752) */
__device__ __forceinline__ bool similar(const GBuf &a, float depth_a, const GBuf &b, float depth_b)
{
	if (!a.hit || !b.hit)
		return false;
	if (dot(a.n, b.n) < KGR_GI_COS_10DEG)
		return false;
	return fabsf(depth_b - depth_a) / depth_a <= 0.1f;
}

__device__ __forceinline__ SurfaceHit receiver(const FrameParams &fp, const GiFrameBuffers &gb, uint32_t pix,
		const GBuf &g)
{
	SurfaceHit h;
	h.mat = load_material(gb.materials, pix);
	h.entering = false;
	h.n = g.n;
	h.wo = normalize(v3(fp.center) - g.x);
	h.x = g.x;
	return h;
}

/* The receiver of the previous frame's pixel: its material by index, the
 * direction toward the previous camera centre. */
__device__ __forceinline__ SurfaceHit receiver_prev(const DeviceScene &s, const FrameParams &fp, const GBuf &g)
{
	SurfaceHit h;
	h.mat = load_material(s.materials, g.mat);
	h.entering = false;
	h.n = g.n;
	h.wo = normalize(v3(fp.prev_center) - g.x);
	h.x = g.x;
	return h;
}

/* Target function of sample s at receiver h: sum_rgb(f L_o) |n.w|. */
__device__ __forceinline__ float gi_target(const SurfaceHit &h, const GiSample &s)
{
	f3 D = s.xs - h.x;
	float d = length(D);
	f3 w = D / d;
	f3 v = brdf(h, w) * s.Lo * fabsf(dot(h.n, w));
	float t = v.x + v.y + v.z;
	return (t > 0.0f && t < 1e30f) ? t : 0.0f;
}

/* Primary vertex: G-buffer, ReSTIR DI candidates for direct light, and the
 * BSDF-sampled direction of the GI sample, after which the path continues
 * with throughput 1 so that it accumulates L_o at the secondary vertex. */
__global__ void __launch_bounds__(128) gi_primary_kernel(DeviceScene s, PathBuffers pb, FrameParams fp,
		GiFrameBuffers gb)
{
	const uint32_t n = pb.counters[CNT_Q0];
	uint32_t *out_counter = pb.counters + CNT_Q1;
	uint32_t stride = gridDim.x * blockDim.x;
	uint32_t iters = (n + stride - 1) / stride;
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
			gb.position[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
			gb.gi_dir[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
			gb.direct[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
			if (h.prim >= 0 && surface(s, h, mk(dv.x, dv.y, dv.z), sh)) {
				f3 n3 = sh.n;
				float sgn = sh.mat.type == KGR_SHADING_TRANSMISSION ? -1.0f : 1.0f;
				sh.x = sh.x + sgn * n3 * KGR_OFFSET_EPS;
				uint4 tr = __ldg(&s.tris[h.prim]);
				gb.position[p] = f4_of(sh.x, (float)(tr.w + 1u));
				gb.normal[p] = f4_of(n3, 0.0f);
				const float4 *src = reinterpret_cast<const float4 *>(s.materials + tr.w);
				float4 *dst = reinterpret_cast<float4 *>(gb.materials + p);
				for (int k = 0; k < 4; k++)
					dst[k] = __ldg(src + k);
				float4 sv = pb.seed[p];
				f3 seed = mk(sv.x, sv.y, sv.z);
				/* ReSTIR DI candidates (amadeus_restir.cu:478-523), shaded directly */
				f3 risseed = pixel_seed(p, fp.frame, KGR_GI_RIS_SALT);
				float wsum = 0.0f;
				int32_t M = 0, sel = -1;
				f3 selp = mk(0.0f);
				unsigned int total = s.light_count;
				for (int c = 0; c < fp.candidates; c++) {
					unsigned int li = (unsigned int)(rand_uniform(seed) * total);
					float weight = 0.0f;
					f3 pt = mk(0.0f);
					if (li < total) {
						TriLight l = load_light(s.lights, li);
						pt = sample_area_light(l, seed);
						float pdf = 1.0f / (l.area() * total);
						f3 D = pt - sh.x;
						float d = length(D);
						f3 Li = direct_unoccluded(sh, l.intensity, l.normal(), D / d, d);
						float tgt = Li.x + Li.y + Li.z;
						weight = (pdf > 0) ? tgt / pdf : 0;
					}
					wsum += weight;
					float eta = rand_uniform(risseed);
					if ((eta * wsum) < weight) {
						sel = (int32_t)li;
						selp = pt;
					}
					M++;
				}
				/* the selected light's contribution, with its shadow ray
				 * queued for the any-hit walk; gi_direct_blocked_kernel
				 * zeroes the contribution when the ray is blocked */
				f3 direct = mk(0.0f);
				if (sel >= 0) {
					TriLight l = load_light(s.lights, (uint32_t)sel);
					f3 D = selp - sh.x;
					float d = length(D);
					f3 Dn = D / d;
					f3 Li = direct_unoccluded(sh, l.intensity, l.normal(), Dn, d);
					float tgt = Li.x + Li.y + Li.z;
					float dd = tgt * M;
					float W = (dd > 0) ? wsum / dd : 0.0f;
					direct = Li * W;
					pb.sh_o[p] = f4_of(sh.x, 0.0f);
					pb.sh_d[p] = f4_of(Dn, d - KGR_SHADOW_EPS);
					shadow = true;
				}
				gb.direct[p] = f4_of(direct, 0.0f);
				/* GI direction (eval, brdf.cuh:573-589) */
				f3 wi;
				float pdf = 0.0f;
				eval(sh, wi, pdf, seed);
				if (pdf > 0 && 0 < fp.max_depth) {
					gb.gi_dir[p] = f4_of(wi, pdf);
					pb.ray_o[p] = f4_of(sh.x, 0.0f);
					pb.ray_d[p] = f4_of(wi, 1e16f);
					pb.beta[p] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
					pb.aov_p[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
					cont = true;
				}
				pb.seed[p] = f4_of(seed, 0.0f);
			}
		}
		queue_append(pb.queue[1], out_counter, p, cont, pb.counters + CNT_BOUNCE_TOTAL);
		queue_append(gb.vis_queue[0], gi_vis_n(gb, 0), p, shadow, gb.ray_total);
	}
}

/* The primary vertices' ReSTIR DI shadow rays (queued by gi_primary_kernel
 * in the shadow-ray arrays, free until the first bounce is shaded) are
 * walked by the tuned any-hit walk, which flags a blocked one at its path:
 * a blocked ray zeroes the pixel's direct light. */
__global__ void gi_direct_blocked_kernel(GiFrameBuffers gb)
{
	const uint32_t n = *gi_vis_n(gb, 0);
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		uint32_t p = gb.vis_queue[0][i];
		if (gb.vis_flag[p])
			gb.direct[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
	}
}

/* Initial reservoir from the finished path: one candidate, W in FP64. */
__global__ void gi_initial_kernel(PathBuffers pb, FrameParams fp, GiFrameBuffers gb, int cur)
{
	uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
	if (pix >= fp.npix)
		return;
	float4 dir = gb.gi_dir[pix];
	float4 xs = pb.aov_p[pix];
	float4 ns = pb.aov_n[pix];
	float4 L = pb.L[pix];
	GiSample smp;
	smp.xs = mk(xs.x, xs.y, xs.z);
	smp.ns = mk(ns.x, ns.y, ns.z);
	smp.Lo = mk(L.x, L.y, L.z);
	smp.rc = ns.w > 0.0f;
	GBuf g = gbuf(gb.position, gb.normal, pix);
	bool valid = g.hit && dir.w > 0.0f && xs.w > 0.0f && !anynan(smp.Lo);
	float W = 0.0f;
	if (valid) {
		float target = gi_target(receiver(fp, gb, pix, g), smp);
		float w = target / dir.w;
		W = gi_normalise(w, 1, target);
	} else {
		smp.xs = smp.Lo = mk(0.0f);
		smp.ns = mk(0.0f, 0.0f, 1.0f);
		smp.rc = true;
	}
	store_gi(gb.res[cur], pix, smp, W, 1);
	float4 sv = pb.seed[pix];
	gb.auxiliary[pix] = make_float4(sv.x, sv.y, sv.z, 1.0f);
}

__device__ __forceinline__ int reproject_gi(const FrameParams &fp, const f3 &x)
{
	const float *m = fp.prev_proj_view;
	float q[4];
	for (int i = 0; i < 4; i++)
		q[i] = m[0 * 4 + i] * x.x + m[1 * 4 + i] * x.y + m[2 * 4 + i] * x.z + m[3 * 4 + i] * 1.0f;
	float u = q[0] / q[3];
	float v = q[1] / q[3];
	if (!(u >= -1.0f && u <= 1.0f && v >= -1.0f && v <= 1.0f))
		return -1;
	u = (u + 1.0f) * 0.5f;
	v = (v + 1.0f) * 0.5f;
	int ix = (int)((double)(u * (float)fp.width) + 0.5);
	int iy = (int)((double)(v * (float)fp.height) + 0.5);
	if (ix < 0 || iy < 0 || ix >= (int)fp.width || iy >= (int)fp.height)
		return -1;
	return iy * (int)fp.width + ix;
}

__global__ void __launch_bounds__(128) gi_temporal_kernel(DeviceScene s, FrameParams fp, GiFrameBuffers gb,
		int cur, int prev)
{
	uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
	if (pix >= fp.npix)
		return;
	GBuf g = gbuf(gb.position, gb.normal, pix);
	if (!g.hit)
		return;
	int pindex = reproject_gi(fp, g.x);
	if (pindex < 0)
		return;
	GBuf gp = gbuf(gb.prev_position, gb.prev_normal, (uint32_t)pindex);
	float depth = length(g.x - v3(fp.center));
	float pdepth = length(gp.x - v3(fp.prev_center));
	if (!similar(g, depth, gp, pdepth))
		return;
	GiRes P = load_gi(gb.res[prev], (uint32_t)pindex);
	if (P.M <= 0)
		return;
	GiRes C = load_gi(gb.res[cur], pix);
	int32_t pM = P.M < fp.gi_mcap ? P.M : fp.gi_mcap;
	SurfaceHit h = receiver(fp, gb, pix, g);
	GiMerge r;
	r.init(pixel_seed(pix, fp.frame, KGR_GI_REUSE_SALT));
	r.update(C.s, gi_target(h, C.s) * C.W * C.M, -1);
	float J = gi_jacobian(g.x, gp.x, P.s, fp.gi_jmax);
	float wp = gi_target(h, P.s) * J * P.W * pM;
	r.update(P.s, wp, 0);
	/* The history counts toward the normalisation whether or not its own
	 * sample carries weight: an empty history reservoir (its GI ray found
	 * nothing) is pM candidates of the same domain that all came out zero.
	 * Dropping it -- the DI rule of counting the previous M only when its
	 * sample's target is positive -- divides by too few candidates and
	 * brightens pixels whose GI samples are often empty. */
	int32_t M = C.M + pM;
	float tq = gi_target(h, r.sel);
	float jp = gi_jacobian(gp.x, g.x, r.sel, fp.gi_jmax);
	float tp = jp > 0.0f ? gi_target(receiver_prev(s, fp, gp), r.sel) * jp : 0.0f;
	float D = (float)C.M * tq + (float)pM * tp;
	float W = gi_mis_weight(r.w, r.src < 0 ? tq : tp, D, tq);
	store_gi(gb.res[cur], pix, r.sel, W, M);
}

/* sample_spatial_neighborhood (amadeus_restir.cu:294-314) */
__device__ __forceinline__ int gi_neighbor(const FrameParams &fp, int index, f3 &seed)
{
	int width = (int)fp.width, height = (int)fp.height;
	int x = index % width;
	int y = index / width;
	f3 offset = rand_uniform_3f(seed);
	float theta = (float)(2.0 * 3.14159265358979323846 * (double)offset.x);
	float r = (float)fp.gi_radius * ksqrt(offset.y);
	float st, ct;
	ksincos(theta, st, ct);
	int x0 = (int)((float)x + r * ct);
	int y0 = (int)((float)y + r * st);
	x0 = x0 < 0 ? 0 : (x0 > width - 1 ? width - 1 : x0);
	y0 = y0 < 0 ? 0 : (y0 > height - 1 ? height - 1 : y0);
	return x0 + y0 * width;
}

/* Spatial reuse as a wavefront of five launches per iteration.  The
 * visibility rays of one resampling step -- one per weighted candidate, one
 * per neighbour domain of the balance-heuristic denominator -- are queued
 * and walked by their own kernel, one ray per thread, instead of inside the
 * per-pixel loops, where a warp's lanes wait on each other's rays and the
 * loops' live state costs occupancy.  The state between the launches is per
 * neighbour slot (k-major, slot = k * npix + pixel): {pixel or -1, M} and a
 * weight; per pixel: {w_sum, bits(domain), bits(M sum), target}.  Every
 * value is computed by the same expressions in the same order as one pass
 * over both loops would, and the random stream is replayed draw for draw,
 * so the reservoirs are those of the single-pass formulation bit for bit.
 *
 * gather: the neighbours that pass the geometric test, their resampling
 * weights w_i = p^_q(y_i) |J_i| W_i M_i, and a visibility ray queued for
 * each positive weight.  The pixel's random stream advances as the
 * resampling will draw it: one uniform for the centre, three for each
 * neighbour's offset, one for each neighbour that is resampled. */
__global__ void __launch_bounds__(128) gi_spatial_gather_kernel(FrameParams fp, GiFrameBuffers gb, int in, int out,
		int iteration)
{
	uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
	if (pix >= fp.npix)
		return;
	GiRes C = load_gi(gb.res[in], pix);
	GBuf g = gbuf(gb.position, gb.normal, pix);
	if (!g.hit) {
		store_gi(gb.res[out], pix, C.s, C.W, C.M);
		return;
	}
	float depth = length(g.x - v3(fp.center));
	SurfaceHit h = receiver(fp, gb, pix, g);
	f3 seed = pixel_seed(pix, fp.frame, KGR_GI_REUSE_SALT + 1u + (uint32_t)iteration);
	float wC = gi_target(h, C.s) * C.W * C.M;
	rand_uniform(seed);
	int32_t Msum = C.M;
	for (int k = 0; k < fp.gi_neighbors; k++) {
		int index0 = gi_neighbor(fp, (int)pix, seed);
		uint32_t slot = (uint32_t)k * fp.npix + pix;
		int2 nb = make_int2(-1, 0);
		float wn = 0.0f;
		GBuf gn = gbuf(gb.position, gb.normal, (uint32_t)index0);
		if (similar(g, depth, gn, length(gn.x - v3(fp.center)))) {
			GiRes N = load_gi(gb.res[in], (uint32_t)index0);
			if (N.M > 0) {
				/* confidence of the neighbour's domain (option
				 * gi_neighbor_confidence, on by default): at most the
				 * centre's M.  Any positive confidences keep the balance
				 * heuristic's weights summing to one; with a neighbour's M
				 * far above the centre's, a sample the centre can barely
				 * see would be shaded with the ratio M_n / M_c (up to 255
				 * where a disocclusion meets reused neighbours) */
				int32_t cn = fp.gi_confidence_rule && C.M < N.M ? C.M : N.M;
				nb = make_int2(index0, cn);
				Msum += cn;
				float J = N.s.rc ? gi_jacobian(g.x, gn.x, N.s, fp.gi_jmax) : 0.0f;
				wn = J > 0.0f ? gi_target(h, N.s) * J * N.W * cn : 0.0f;
				rand_uniform(seed);
			}
		}
		gb.neighbours[slot] = nb;
		gb.weights[slot] = wn;
		queue_append(gb.vis_queue[0], gi_vis_n(gb, 0), slot, wn > 0.0f, gb.ray_total);
	}
	gb.selection[pix] = make_float4(wC, 0.0f, __int_as_float(Msum), 0.0f);
}

/* The receiver of neighbour slot `slot`'s selected sample (second round):
 * the sample the pixel selected, from the centre or a neighbour. */
__device__ __forceinline__ uint32_t selected_from(const GiFrameBuffers &gb, uint32_t npix, uint32_t pix,
		int32_t domain)
{
	return domain < 0 ? pix : (uint32_t)gb.neighbours[(size_t)domain * npix + pix].x;
}

/* visibility of queued slots, one ray per thread; a blocked ray's weight
 * becomes 0.  Round 0: from the pixel's receiver to the neighbour's
 * sample.  Round 1: from the neighbour's receiver to the pixel's selected
 * sample.  (These rays are short and two per neighbour: writing them out
 * for the tuned walk cost more than the walk saved.) */
__global__ void __launch_bounds__(128) gi_visibility_kernel(DeviceScene s, FrameParams fp, GiFrameBuffers gb, int in,
		int round)
{
	const uint32_t *queue = gb.vis_queue[round];
	uint32_t *n = gi_vis_n(gb, round);
	for_each_queued(*n, n + (CNT_FETCH_SHADOW - CNT_SHADOW), [&](uint32_t i) {
		uint32_t slot = queue[i];
		uint32_t pix = slot % fp.npix;
		uint32_t idx = (uint32_t)gb.neighbours[slot].x;
		f3 from, to;
		if (round == 0) {
			from = f3_of(gb.position[pix]);
			to = f3_of(gb.res[in].a[idx]);
		} else {
			int32_t domain = __float_as_int(gb.selection[pix].y);
			from = f3_of(gb.position[idx]);
			to = f3_of(gb.res[in].a[selected_from(gb, fp.npix, pix, domain)]);
		}
		if (!visible(s, fp.layout, from, to))
			gb.weights[slot] = 0.0f;
	});
}

/* resample: the weighted reservoir over the centre and the neighbours with
 * their visibility-tested weights (GiMerge's rule, the same draws), then
 * the selected sample shifted back to every neighbour receiver,
 * p^_i(y) |J_q->i|, with a visibility ray queued for each positive one. */
__global__ void __launch_bounds__(128) gi_spatial_resample_kernel(FrameParams fp, GiFrameBuffers gb, int in,
		int iteration)
{
	uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
	if (pix >= fp.npix)
		return;
	GBuf g = gbuf(gb.position, gb.normal, pix);
	if (!g.hit)
		return;
	float4 st = gb.selection[pix];
	GiMerge r;
	r.init(pixel_seed(pix, fp.frame, KGR_GI_REUSE_SALT + 1u + (uint32_t)iteration));
	bool chosen = r.take(st.x);
	for (int k = 0; k < fp.gi_neighbors; k++) {
		rand_uniform_3f(r.seed);
		uint32_t slot = (uint32_t)k * fp.npix + pix;
		if (gb.neighbours[slot].x < 0)
			continue;
		if (r.take(gb.weights[slot])) {
			r.src = k;
			chosen = true;
		}
	}
	int32_t domain = chosen ? r.src : -2;
	GiSample sel;
	if (chosen) {
		sel = load_gi(gb.res[in], selected_from(gb, fp.npix, pix, domain)).s;
	} else {
		sel.xs = sel.ns = sel.Lo = mk(0.0f);
		sel.valid = false;
		sel.rc = true;
	}
	SurfaceHit h = receiver(fp, gb, pix, g);
	float target = gi_target(h, sel);
	if (target > 0.0f && sel.rc) {
		for (int k = 0; k < fp.gi_neighbors; k++) {
			uint32_t slot = (uint32_t)k * fp.npix + pix;
			int2 nb = gb.neighbours[slot];
			if (nb.x < 0)
				continue;
			GBuf gn = gbuf(gb.position, gb.normal, (uint32_t)nb.x);
			float jn = gi_jacobian(gn.x, g.x, sel, fp.gi_jmax);
			float tn = jn > 0.0f ? gi_target(receiver(fp, gb, (uint32_t)nb.x, gn), sel) * jn : 0.0f;
			gb.weights[slot] = tn;
			queue_append(gb.vis_queue[1], gi_vis_n(gb, 1), slot, tn > 0.0f, gb.ray_total);
		}
	}
	gb.selection[pix] = make_float4(r.w, __int_as_float(domain), st.z, target);
}

/* finish: the balance-heuristic weight W = p^<-j(y) w_sum / (p^_q(y) D),
 * D = sum_i M_i p^<-i(y) with each neighbour's visibility, and the
 * reservoir {y, W, M sum}. */
__global__ void __launch_bounds__(128) gi_spatial_finish_kernel(FrameParams fp, GiFrameBuffers gb, int in, int out)
{
	uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
	if (pix >= fp.npix)
		return;
	if (!(gb.position[pix].w > 0.0f))
		return; /* gather stored the centre reservoir */
	float4 st = gb.selection[pix];
	float w_sum = st.x, target = st.w;
	int32_t domain = __float_as_int(st.y), Msum = __float_as_int(st.z);
	GiSample sel;
	if (domain == -2) {
		sel.xs = sel.ns = sel.Lo = mk(0.0f);
		sel.valid = false;
		sel.rc = true;
	} else {
		sel = load_gi(gb.res[in], selected_from(gb, fp.npix, pix, domain)).s;
	}
	int32_t CM = unpack_m(__float_as_uint(gb.res[in].a[pix].w));
	float D = (float)CM * target;
	float num = domain < 0 ? target : 0.0f;
	if (target > 0.0f && sel.rc) {
		for (int k = 0; k < fp.gi_neighbors; k++) {
			uint32_t slot = (uint32_t)k * fp.npix + pix;
			int2 nb = gb.neighbours[slot];
			if (nb.x < 0)
				continue;
			float tn = gb.weights[slot];
			D += (float)nb.y * tn;
			if (k == domain)
				num = tn;
		}
	}
	float W = gi_mis_weight(w_sum, num, D, target);
	store_gi(gb.res[out], pix, sel, W, Msum);
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

/* The final shading's visibility rays, from the primary vertex to the
 * selected sample of each pixel with W > 0 (slot = pixel). */
__global__ void __launch_bounds__(128) gi_final_rays_kernel(FrameParams fp, GiFrameBuffers gb, int fin)
{
	uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
	if (pix >= fp.npix)
		return;
	GBuf g = gbuf(gb.position, gb.normal, pix);
	bool ray = false;
	if (g.hit) {
		GiRes R = load_gi(gb.res[fin], pix);
		if (R.W > 0.0f) {
			gi_vis_ray(gb, pix, g.x, R.s.xs);
			ray = true;
		}
	}
	queue_append(gb.vis_queue[0], gi_vis_n(gb, 0), pix, ray, gb.ray_total);
}

/* Final shading: emission + direct + f L_o |n.w| W when the visibility ray
 * is unblocked; the G-buffer becomes the history of the next frame. */
__global__ void __launch_bounds__(128) gi_final_kernel(DeviceScene s, FrameParams fp, GiFrameBuffers gb,
		OutputBuffers out, int fin)
{
	uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
	if (pix >= fp.npix)
		return;
	GBuf g = gbuf(gb.position, gb.normal, pix);
	f3 c = mk(0.0f);
	if (g.hit) {
		SurfaceHit h = receiver(fp, gb, pix, g);
		float4 dv = gb.direct[pix];
		f3 gi = mk(0.0f);
		GiRes R = load_gi(gb.res[fin], pix);
		if (R.W > 0.0f) {
			f3 D = R.s.xs - g.x;
			float d = length(D);
			f3 w = D / d;
			if (!gb.vis_flag[pix])
				gi = brdf(h, w) * R.s.Lo * (fabsf(dot(h.n, w)) * R.W);
		}
		c = h.mat.emission + mk(dv.x, dv.y, dv.z) + gi;
	}
	if (anynan(c))
		c = mk(1.0f, 0.0f, 1.0f);
	accumulate4(out.color, pix, f4_of(c, 1.0f), fp.accumulate != 0, (float)fp.samples);
	float4 pv = gb.position[pix];
	if (out.position)
		out.position[pix] = make_float4(pv.x, pv.y, pv.z, 0.0f);
	if (out.normal)
		out.normal[pix] = gb.normal[pix];
	gb.prev_position[pix] = pv;
	gb.prev_normal[pix] = gb.normal[pix];
}

} /* namespace */

namespace {

/* The tuned any-hit walk over round q's queue (the slots' rays, or the
 * paths' shadow rays of the primary vertices), flags per entry. */
void gi_walk(const DeviceScene &s, const FrameParams &fp, const GiFrameBuffers &gb, float4 *o, float4 *d, int q,
		cudaStream_t st)
{
	PathBuffers vb{};
	vb.sh_o = o;
	vb.sh_d = d;
	vb.shadow_queue = gb.vis_queue[q];
	vb.counters = gb.vis_count + q * CNT_COUNT;
	vb.shadow_flags = gb.vis_flag;
	vb.visits = nullptr;
	vb.capacity = gb.vis_capacity;
	pt_shadow_resolve(s, vb, fp.layout, fp.tune, st);
}

void gi_vis_clear(const GiFrameBuffers &gb, cudaStream_t st)
{
	KGR_CUDA(cudaMemsetAsync(gb.vis_count, 0, 2 * CNT_COUNT * sizeof(uint32_t), st));
}

} /* namespace */

void gi_primary(const DeviceScene &s, const PathBuffers &pb, const FrameParams &fp, const GiFrameBuffers &gb,
		cudaStream_t st)
{
	int grid = (int)((pb.capacity + 127) / 128);
	int cap = device_sm_count() * 16;
	gi_vis_clear(gb, st);
	gi_primary_kernel<<<grid < cap ? grid : cap, 128, 0, st>>>(s, pb, fp, gb);
	gi_walk(s, fp, gb, pb.sh_o, pb.sh_d, 0, st);
	gi_direct_blocked_kernel<<<device_sm_count() * 8, 128, 0, st>>>(gb);
	KGR_CUDA(cudaGetLastError());
}

void gi_initial(const PathBuffers &pb, const FrameParams &fp, const GiFrameBuffers &gb, int cur, cudaStream_t st)
{
	gi_initial_kernel<<<(fp.npix + 255) / 256, 256, 0, st>>>(pb, fp, gb, cur);
	KGR_CUDA(cudaGetLastError());
}

void gi_temporal(const DeviceScene &s, const FrameParams &fp, const GiFrameBuffers &gb, int cur, int prev,
		cudaStream_t st)
{
	gi_temporal_kernel<<<(fp.npix + 127) / 128, 128, 0, st>>>(s, fp, gb, cur, prev);
	KGR_CUDA(cudaGetLastError());
}

void gi_spatial(const DeviceScene &s, const FrameParams &fp, const GiFrameBuffers &gb, int in, int out,
		int iteration, cudaStream_t st)
{
	unsigned grid = (fp.npix + 127) / 128;
	gi_vis_clear(gb, st);
	int vis_grid = device_sm_count() * 8;
	gi_spatial_gather_kernel<<<grid, 128, 0, st>>>(fp, gb, in, out, iteration);
	gi_visibility_kernel<<<vis_grid, 128, 0, st>>>(s, fp, gb, in, 0);
	gi_spatial_resample_kernel<<<grid, 128, 0, st>>>(fp, gb, in, iteration);
	gi_visibility_kernel<<<vis_grid, 128, 0, st>>>(s, fp, gb, in, 1);
	gi_spatial_finish_kernel<<<grid, 128, 0, st>>>(fp, gb, in, out);
	KGR_CUDA(cudaGetLastError());
}

void gi_final(const DeviceScene &s, const FrameParams &fp, const GiFrameBuffers &gb, const OutputBuffers &out,
		int fin, cudaStream_t st)
{
	unsigned grid = (fp.npix + 127) / 128;
	gi_vis_clear(gb, st);
	gi_final_rays_kernel<<<grid, 128, 0, st>>>(fp, gb, fin);
	gi_walk(s, fp, gb, gb.vis_o, gb.vis_d, 0, st);
	gi_final_kernel<<<grid, 128, 0, st>>>(s, fp, gb, out, fin);
	KGR_CUDA(cudaGetLastError());
}

} /* namespace kgr */

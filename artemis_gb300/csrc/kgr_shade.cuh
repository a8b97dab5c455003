/*
 * kgr_shade.cuh -- one path vertex of the path tracer: next-event estimation
 * against the triangle lights and the BSDF continuation with Russian
 * roulette.  The wavefront shade kernel (pt.cu) and the per-thread training
 * paths of the radiance cache (cache.cu) share this code, so both estimate
 * the same radiance with the same operations in the same order.
 */
#ifndef KGR_SHADE_CUH_
#define KGR_SHADE_CUH_

#include "kgr_device.cuh"
#include "kgr_wavefront.h"

namespace kgr {

/* Ld (amadeus_common.cuh:256-286) -- a uniform pick over the quad lights,
 * the triangle lights and the environment map -- with Ld_light
 * (lighting.cuh:149-174) or Ld_Environment (amadeus_common.cuh:215-254), and
 * the continuation (eval, brdf.cuh:573-589; Russian roulette as in
 * naive_path_tracer.cu:294-303).  `seed` advances in place.  At the last
 * depth the continuation is sampled only when final_seed is set (ReSTIR
 * keeps that seed).  Results go to `out` as they are produced:
 *   out.vertex(x, n, m)   offset hit point, shading normal and material
 *   out.emit(add)         beta * emission (scene without lights)
 *   out.nee(c, e, b, o, d) NEE record {contribution, pdf}, emission, beta,
 *                         shadow ray origin and {direction, tmax}
 *   out.next(x, wi, beta) the path continues from x along wi */
template <class Sink>
__device__ __forceinline__ void shade_surface(const DeviceScene &s, const FrameParams &fp, int depth, int final_seed,
		SurfaceHit sh, f3 beta, f3 &seed, Sink &out)
{
	f3 n3 = sh.n;
	float sgn = sh.mat.type == KGR_SHADING_TRANSMISSION ? -1.0f : 1.0f;
	sh.x = sh.x + sgn * n3 * KGR_OFFSET_EPS;
	out.vertex(sh.x, n3, sh.mat);
	unsigned int total_count = s.quad_count + s.light_count + (s.has_env ? 1u : 0u);
	if (total_count == 0) {
		f3 direct = sh.mat.emission + mk(0.0f);
		out.emit(beta * direct);
	} else {
		unsigned int li = (unsigned int)(rand_uniform(seed) * total_count);
		float pdf = 1.0f / total_count;
		float light_pdf;
		f3 contr, wi;
		float tmax;
		if (li < s.quad_count + s.light_count || !s.has_env) {
			/* Ld_light (lighting.cuh:149-174) over a quad or a triangle */
			f3 lpos, lnormal, Le;
			if (li < s.quad_count) {
				QuadLight light = load_quad(s.quads, li);
				light_pdf = 1.0f / light.area();
				lpos = sample_area_light(light, seed);
				lnormal = light.normal();
				Le = light.intensity;
			} else {
				uint32_t ti = li - s.quad_count;
				TriLight light = load_light(s.lights, ti < s.light_count ? ti : s.light_count - 1);
				light_pdf = 1.0f / light.area();
				lpos = sample_area_light(light, seed);
				lnormal = light.normal();
				Le = light.intensity;
			}
			wi = normalize(lpos - sh.x);
			float R = length(lpos - sh.x);
			f3 f = brdf(sh, wi);
			float ldot = fabsf(dot(lnormal, wi));
			float geometric = ldot * fabsf(dot(sh.n, wi)) / (R * R);
			contr = f * Le * geometric;
			tmax = R - KGR_SHADOW_EPS;
		} else {
			/* Ld_Environment (amadeus_common.cuh:215-254): the map at (u, v),
			 * a shadow ray to the world radius, pdf 1 / (4 pi) */
			wi = env_direction(seed, false);
			float u, v;
			env_uv(wi, u, v);
			f3 Li = env_fetch(s, u, v);
			light_pdf = (float)(1.0 / (4.0 * KGR_PI_D));
			f3 f = brdf(sh, wi) * fabsf(dot(sh.n, wi));
			contr = f * Li;
			tmax = KGR_WORLD_RADIUS - KGR_SHADOW_EPS;
		}
		pdf *= light_pdf;
		out.nee(f4_of(contr, pdf), f4_of(sh.mat.emission, 0.0f), f4_of(beta, 0.0f), f4_of(sh.x, 0.0f),
			f4_of(wi, tmax));
	}
	/* no ray is cast past the last vertex: the reference's closest-hit and
	 * miss programs both return 0 for a ray at depth > max_depth
	 * (LOAD_RAYPACKET, amadeus_common.cuh:480-488), so its hit adds nothing
	 * and its miss does not see the environment map */
	int last = fp.max_depth;
	if (depth < last || final_seed) {
		f3 wi;
		float pdf = 0.0f;
		f3 f = eval(sh, wi, pdf, seed);
		if (pdf > 0) {
			f3 T = f * fabsf(dot(wi, n3)) / pdf;
			beta = beta * T;
			bool alive = true;
			if (fp.russian_roulette && depth >= fp.rr_start_depth) {
				float qq = 1.0f - kmin(kmax(0.05f, beta.y), 1.0f);
				float r = fract(seed.x);
				if (r < qq)
					alive = false;
				else
					beta = beta / (1.0f - qq);
			}
			if (alive && depth < last)
				out.next(sh.x, wi, beta);
		}
	}
}

/* make_ray (amadeus_path_tracer.cu:25-56): one pcg3f draw for the jitter;
 * the ReSTIR variant (amadeus_restir.cu:30-65) draws it but uses -0.5. */
__device__ __forceinline__ void camera_ray(const float *center, const float *Uc, const float *Vc, const float *Wc,
		uint32_t width, uint32_t height, int jitter, uint32_t ix, uint32_t iy, f3 &seed, f3 &origin,
		f3 &direction)
{
	f3 U = mk(Uc[0], Uc[1], Uc[2]), V = mk(Vc[0], Vc[1], Vc[2]), W = mk(Wc[0], Wc[1], Wc[2]);
	pcg3f(seed);
	float xoffset = jitter ? (fract(seed.x) - 0.5f) : -0.5f;
	float yoffset = jitter ? (fract(seed.y) - 0.5f) : -0.5f;
	float ax = ((float)ix + xoffset) / (float)width;
	float ay = ((float)iy + yoffset) / (float)height;
	float dx = 2.0f * ax - 1.0f;
	float dy = 2.0f * ay - 1.0f;
	origin = mk(center[0], center[1], center[2]);
	direction = normalize(dx * U + dy * V + W);
}

/* Progressive mean dst = (prev * n + s) / (n + 1) (amadeus_path_tracer.cu:59-70). */
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

/* One finished path into the frame's buffers: sample `count` of pixel pix
 * (acc: blend with the previous mean); NaN radiance shows as magenta. */
__device__ __forceinline__ void accumulate_path(const OutputBuffers &out, const PathBuffers &pb, uint32_t p,
		uint32_t pix, bool acc, float count)
{
	float4 L = pb.L[p];
	f3 c = mk(L.x, L.y, L.z);
	if (anynan(c))
		c = mk(1.0f, 0.0f, 1.0f);
	if (out.color)
		accumulate4(out.color, pix, f4_of(c, 1.0f), acc, count);
	if (out.normal)
		accumulate4(out.normal, pix, pb.aov_n[p], acc, count);
	if (out.albedo)
		accumulate4(out.albedo, pix, pb.aov_a[p], acc, count);
	if (out.position)
		out.position[pix] = pb.aov_p[p];
}

/* L += beta * (Le + Ld) once the shadow ray is resolved, in the order of
 * the recursion (Ld = contribution / pdf, zero when occluded). */
__device__ __forceinline__ float4 nee_add(float4 L, float4 c, float4 e, float4 be, bool occ)
{
	f3 contr = occ ? mk(0.0f) : mk(c.x, c.y, c.z);
	f3 direct = mk(e.x, e.y, e.z) + contr / c.w;
	return f4_of(mk(L.x, L.y, L.z) + mk(be.x, be.y, be.z) * direct, 0.0f);
}

} /* namespace kgr */

#endif

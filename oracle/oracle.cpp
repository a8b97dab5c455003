/*
 * oracle.cpp -- CPU restatement of the reference's ray-tracing hot path.
 *
 * TEST INFRASTRUCTURE: the checker the CUDA kernels are compared against.
 * Nothing in the product links or calls this file.  Built by oracle/Makefile
 * with g++ -O2 -ffp-contract=off -fopenmp into oracle/liboracle.so.
 *
 * Floating-point expressions keep the reference's evaluation order; the
 * vector helpers, the RNG and the transcendentals are the oracle's own
 * (ref_math.h), written apart from the kernels' so that a slip on either
 * side fails the parity tests instead of passing on both.
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <memory>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "ref_math.h"

using namespace oref;

namespace {

/* ============================================================ BVH build == */

/* BoundingBox (include/bbox.hpp:9-30) */
struct Box {
	f3 min, max;
	float surface_area() const
	{
		float dx = max.x - min.x;
		float dy = max.y - min.y;
		float dz = max.z - min.z;
		float xy = dx * dy;
		float yz = dy * dz;
		float xz = dx * dz;
		return 2.0f * (xy + yz + xz);
	}
};

/* glm::min / glm::max: (y < x) ? y : x, componentwise */
inline f3 gmin(const f3 &a, const f3 &b)
{
	return mk(b.x < a.x ? b.x : a.x, b.y < a.y ? b.y : a.y, b.z < a.z ? b.z : a.z);
}
inline f3 gmax(const f3 &a, const f3 &b)
{
	return mk(a.x < b.x ? b.x : a.x, a.y < b.y ? b.y : a.y, a.z < b.z ? b.z : a.z);
}

/* BVHNode (include/bvh.hpp:24-38), index-based instead of shared_ptr */
struct Node {
	Box bbox;
	int object = -1;
	int left = -1, right = -1;
};

struct Builder {
	std::vector<Node> nodes;

	/* union_of (source/bvh.cpp:32-43) */
	Box union_of(const std::vector<int> &ids) const
	{
		f3 mn = nodes[ids[0]].bbox.min, mx = nodes[ids[0]].bbox.max;
		for (size_t i = 1; i < ids.size(); i++) {
			mn = gmin(mn, nodes[ids[i]].bbox.min);
			mx = gmax(mx, nodes[ids[i]].bbox.max);
		}
		return Box{mn, mx};
	}

	/* sah_cost (source/bvh.cpp:46-98) */
	float sah_cost(const std::vector<int> &ids, int axis, float split) const
	{
		f3 min_left = mk(FLT_MAX), max_left = mk(-FLT_MAX);
		f3 min_right = mk(FLT_MAX), max_right = mk(-FLT_MAX);
		f3 tmin = nodes[ids[0]].bbox.min, tmax = nodes[ids[0]].bbox.max;
		int prims_left = 0, prims_right = 0;
		for (int id : ids) {
			f3 mn = nodes[id].bbox.min, mx = nodes[id].bbox.max;
			tmin = gmin(tmin, mn);
			tmax = gmax(tmax, mx);
			float value = (comp(mn, axis) + comp(mx, axis)) / 2.0f;
			if (value < split) {
				prims_left++;
				min_left = gmin(min_left, mn);
				max_left = gmax(max_left, mx);
			} else {
				prims_right++;
				min_right = gmin(min_right, mn);
				max_right = gmax(max_right, mx);
			}
		}
		if (prims_left == 0 || prims_right == 0)
			return FLT_MAX;
		float sa_left = Box{min_left, max_left}.surface_area();
		float sa_right = Box{min_right, max_right}.surface_area();
		float sa_total = Box{tmin, tmax}.surface_area();
		return 1 + (prims_left * sa_left + prims_right * sa_right) / sa_total;
	}

	/* partition (source/bvh.cpp:102-195) */
	int partition(const std::vector<int> &ids)
	{
		if (ids.size() == 0)
			return -1;
		if (ids.size() == 1)
			return ids[0];
		if (ids.size() == 2) {
			Node node;
			node.bbox = union_of(ids);
			node.left = ids[0];
			node.right = ids[1];
			nodes.push_back(node);
			return (int)nodes.size() - 1;
		}

		int axis = 0;
		float max_extent = 0.0f;
		float min_value = FLT_MAX;
		float max_value = -FLT_MAX;
		for (size_t n = 0; n < ids.size(); n++) {
			for (int i = 0; i < 3; i++) {
				f3 mn = nodes[ids[n]].bbox.min, mx = nodes[ids[n]].bbox.max;
				float extent = fabsf(comp(mx, i) - comp(mn, i));
				if (extent > max_extent) {
					max_extent = extent;
					min_value = comp(mn, i);
					max_value = comp(mx, i);
					axis = i;
				}
			}
		}

		float min_cost = FLT_MAX;
		float min_split = 0.0f;
		int bins = 10;
		for (int i = 0; i < bins; i++) {
			float split = (max_value - min_value) / bins * i + min_value;
			float cost = sah_cost(ids, axis, split);
			if (cost < min_cost) {
				min_cost = cost;
				min_split = split;
			}
		}

		std::vector<int> left, right;
		if (min_cost == FLT_MAX) {
			for (size_t i = 0; i < ids.size(); i++) {
				if (i % 2 == 0)
					left.push_back(ids[i]);
				else
					right.push_back(ids[i]);
			}
		} else {
			for (int id : ids) {
				f3 mn = nodes[id].bbox.min, mx = nodes[id].bbox.max;
				float value = (comp(mn, axis) + comp(mx, axis)) / 2.0f;
				if (value < min_split)
					left.push_back(id);
				else
					right.push_back(id);
			}
		}

		Box bbox = union_of(ids);
		int l = partition(left);
		int r = partition(right);
		Node node;
		node.bbox = bbox;
		node.left = l;
		node.right = r;
		nodes.push_back(node);
		return (int)nodes.size() - 1;
	}

	/* BVHNode::node_count (source/bvh.cpp:18-22) */
	size_t node_count(int i) const
	{
		if (i < 0)
			return 0;
		return 1 + node_count(nodes[i].left) + node_count(nodes[i].right);
	}

	/* serialize (source/bvh.cpp:213-260) */
	void serialize(std::vector<float> &buf, int bvh, int miss) const
	{
		if (bvh < 0)
			return;
		int size = (int)(buf.size() / 4);
		int after = size + 3;
		int left = nodes[bvh].left, right = nodes[bvh].right;
		int32_t left_index = left >= 0 ? after : -1;
		int32_t left_size = left >= 0 ? 3 * (int32_t)node_count(left) : 0;
		int32_t right_index = right >= 0 ? after + left_size : -1;
		int32_t hit = left_index;
		if (left < 0 && right < 0)
			hit = miss;
		int32_t miss_left = right_index;
		if (right < 0)
			miss_left = miss;
		int32_t object = nodes[bvh].object;
		float leaf = object != -1 ? 1.0f : 0.0f;
		const Box &b = nodes[bvh].bbox;
		float v[12] = {leaf, u2f((uint32_t)object), u2f((uint32_t)hit), u2f((uint32_t)miss),
			b.min.x, b.min.y, b.min.z, 0.0f, b.max.x, b.max.y, b.max.z, 0.0f};
		buf.insert(buf.end(), v, v + 12);
		if (left >= 0)
			serialize(buf, left, miss_left);
		if (right >= 0)
			serialize(buf, right, miss);
	}
};

/* ========================================================== intersection == */

inline f3 ld3(const float *p, uint32_t i) { return mk(p[3 * i + 0], p[3 * i + 1], p[3 * i + 2]); }

/* intersects_triangle (include/optix/lighting.cuh:34-55) == _intersect_t
 * (shaders/rt/modules/intersect.glsl:14-33).  1.0 / divisor is a double
 * division rounded to float; for binary32 operands that equals the float
 * division (double rounding of a quotient is innocuous at 53 >= 2*24+2). */
inline float intersect_triangle(const f3 &v1, const f3 &v2, const f3 &v3,
		const f3 &origin, const f3 &dir, float &b1, float &b2)
{
	f3 e1 = v2 - v1;
	f3 e2 = v3 - v1;
	f3 s1 = cross(dir, e2);
	float divisor = dot(s1, e1);
	if (divisor == 0.0f)
		return -1;
	f3 s = origin - v1;
	float inv_divisor = (float)(1.0 / (double)divisor);
	b1 = dot(s, s1) * inv_divisor;
	if (b1 < 0.0f || b1 > 1.0f)
		return -1;
	f3 s2 = cross(s, e1);
	b2 = dot(dir, s2) * inv_divisor;
	if (b2 < 0.0f || b1 + b2 > 1.0f)
		return -1;
	return dot(e2, s2) * inv_divisor;
}

/* intersect_box (shaders/rt/modules/bbox.glsl:8-58) */
inline float intersect_box(const f3 &o, const f3 &d, const f3 &pmin, const f3 &pmax)
{
	float tmin = (pmin.x - o.x) / d.x;
	float tmax = (pmax.x - o.x) / d.x;
	if (tmin > tmax) { float t = tmin; tmin = tmax; tmax = t; }
	float tymin = (pmin.y - o.y) / d.y;
	float tymax = (pmax.y - o.y) / d.y;
	if (tymin > tymax) { float t = tymin; tymin = tymax; tymax = t; }
	if ((tmin > tymax) || (tymin > tmax))
		return -1.0f;
	if (tymin > tmin)
		tmin = tymin;
	if (tymax < tmax)
		tmax = tymax;
	float tzmin = (pmin.z - o.z) / d.z;
	float tzmax = (pmax.z - o.z) / d.z;
	if (tzmin > tzmax) { float t = tzmin; tzmin = tzmax; tzmax = t; }
	if ((tmin > tzmax) || (tzmin > tmax))
		return -1.0f;
	if (tzmin > tmin)
		tmin = tzmin;
	if (tzmax < tmax)
		tmax = tzmax;
	return tmin;
}

/* in_box (bbox.glsl:61-67) */
inline bool in_box(const f3 &p, const f3 &pmin, const f3 &pmax)
{
	bool lt = p.x < pmin.x || p.y < pmin.y || p.z < pmin.z;
	bool gt = p.x > pmax.x || p.y > pmax.y || p.z > pmax.z;
	return !(lt || gt);
}

inline int32_t bits_i(float f) { return (int32_t)f2u(f); }

struct Tri {
	f3 a, b, c;
};

inline Tri load_tri(const oracle_scene *s, int prim)
{
	const uint32_t *t = s->tris + 4 * (size_t)prim;
	return Tri{ld3(s->positions, t[0]), ld3(s->positions, t[1]), ld3(s->positions, t[2])};
}

/* trace (shaders/rt/modules/bvh.glsl:52-99): threaded walk, a primitive
 * replaces the best hit when 0 < t < best; a box is entered when its entry
 * distance is in (0, best) or the origin lies inside it. */
kgr_hit trace_closest(const oracle_scene *s, const f3 &o, const f3 &d, float tmax,
		uint64_t *internal, uint64_t *leaves)
{
	kgr_hit best = {-1, tmax, 0.0f, 0.0f};
	const float *bvh = s->bvh;
	int node = 0;
	if (s->bvh_vec4_count == 0)
		node = -1;
	while (node != -1) {
		const float *h = bvh + 4 * (size_t)node;
		int object = bits_i(h[1]);
		if (object != -1) {
			(*leaves)++;
			Tri tri = load_tri(s, object);
			float b1 = 0, b2 = 0;
			float t = intersect_triangle(tri.a, tri.b, tri.c, o, d, b1, b2);
			if (t > 0.0f && t < best.t) {
				best.prim = object;
				best.t = t;
				best.b1 = b1;
				best.b2 = b2;
			}
			node = bits_i(h[3]);
		} else {
			(*internal)++;
			f3 pmin = mk(h[4], h[5], h[6]), pmax = mk(h[8], h[9], h[10]);
			float t = intersect_box(o, d, pmin, pmax);
			bool inside = in_box(o, pmin, pmax);
			if ((t > 0.0f && t < best.t) || inside)
				node = bits_i(h[2]);
			else
				node = bits_i(h[3]);
		}
	}
	if (best.prim < 0)
		best.t = tmax;
	return best;
}

/* Occlusion over (0, tmax): the walk of trace() with best = tmax that stops
 * at the first accepted primitive (OPTIX_RAY_FLAG_TERMINATE_ON_FIRST_HIT in
 * is_occluded, source/optix/amadeus_common.cuh:190-212). */
bool trace_any(const oracle_scene *s, const f3 &o, const f3 &d, float tmax,
		uint64_t *internal, uint64_t *leaves)
{
	const float *bvh = s->bvh;
	int node = s->bvh_vec4_count ? 0 : -1;
	while (node != -1) {
		const float *h = bvh + 4 * (size_t)node;
		int object = bits_i(h[1]);
		if (object != -1) {
			(*leaves)++;
			Tri tri = load_tri(s, object);
			float b1 = 0, b2 = 0;
			float t = intersect_triangle(tri.a, tri.b, tri.c, o, d, b1, b2);
			if (t > 0.0f && t < tmax)
				return true;
			node = bits_i(h[3]);
		} else {
			(*internal)++;
			f3 pmin = mk(h[4], h[5], h[6]), pmax = mk(h[8], h[9], h[10]);
			float t = intersect_box(o, d, pmin, pmax);
			bool inside = in_box(o, pmin, pmax);
			if ((t > 0.0f && t < tmax) || inside)
				node = bits_i(h[2]);
			else
				node = bits_i(h[3]);
		}
	}
	return false;
}

/* ================================================================ BSDF == */

struct Material {
	f3 diffuse, specular, emission, ambient;
	float shininess, roughness, refraction;
	int type;
};

inline Material load_material(const kgr_material &m)
{
	Material r;
	r.diffuse = mk(m.diffuse[0], m.diffuse[1], m.diffuse[2]);
	r.specular = mk(m.specular[0], m.specular[1], m.specular[2]);
	r.emission = mk(m.emission[0], m.emission[1], m.emission[2]);
	r.ambient = mk(m.ambient[0], m.ambient[1], m.ambient[2]);
	r.shininess = m.shininess;
	r.roughness = m.roughness;
	r.refraction = m.refraction;
	r.type = m.type;
	return r;
}

/* SurfaceHit (include/cuda/brdf.cuh:67-74) */
struct SurfaceHit {
	Material mat;
	bool entering;
	f3 n, wo, x;
};

const float PI_F = 3.14159265358979323846f; /* brdf.cuh:64 */

/* G1 (brdf.cuh:179-192) */
float G1(f3 n, f3 v, const Material &mat)
{
	if (dot(v, n) <= 0.0f)
		return 0.0f;
	float alpha = mat.roughness;
	float theta = kacos(clampf(dot(n, v), 0.0f, 0.999f));
	float tan_theta = ktan(theta);
	float denom = 1 + ksqrt(1 + alpha * alpha * tan_theta * tan_theta);
	return 2.0f / denom;
}

/* G (brdf.cuh:195-199) */
float G(f3 n, f3 wi, f3 wo, const Material &mat) { return G1(n, wo, mat) * G1(n, wi, mat); }

/* shlick_F (brdf.cuh:202-207) */
f3 shlick_F(f3 wi, f3 h, const Material &mat)
{
	float k = kpow5(1 - dot(wi, h));
	return mat.specular + (1.0f - mat.specular) * k;
}

/* Microfacets::GGX (brdf.cuh:210-220) */
float ggx_D(f3 n, f3 h, const Material &mat)
{
	float alpha = mat.roughness;
	float theta = kacos(clampf(dot(n, h), 0.0f, 1.0f));
	float c, sn;
	ksincos(theta, sn, c);
	float tn = sn / c;
	return (alpha * alpha) / (PI_F * kpow4(c) * kpow2(alpha * alpha + tn * tn));
}

/* GGX::brdf (brdf.cuh:337-353) */
f3 ggx_brdf(const Material &mat, f3 n, f3 wi, f3 wo)
{
	if (dot(wo, n) <= 0.0f)
		n = -n;
	f3 h = normalize(wi + wo);
	f3 f = shlick_F(wi, h, mat);
	float g = G(n, wi, wo, mat);
	float d = ggx_D(n, h, mat);
	f3 num = f * g * d;
	float denom = 4 * dot(wi, n) * dot(wo, n);
	return num / (denom + 1e-6f);
}

/* GGX::pdf (brdf.cuh:356-382) */
float ggx_pdf(const Material &mat, f3 n, f3 wi, f3 wo)
{
	if (dot(wo, n) <= 0.0f)
		n = -n;
	if (dot(wi, n) <= 0.0f)
		return 0.0f;
	f3 h = normalize(wi + wo);
	float avg_Kd = (mat.diffuse.x + mat.diffuse.y + mat.diffuse.z) / 3.0f;
	float avg_Ks = (mat.specular.x + mat.specular.y + mat.specular.z) / 3.0f;
	float t = 1.0f;
	if (avg_Kd + avg_Ks > 0.0f)
		t = kmax(avg_Ks / (avg_Kd + avg_Ks), 0.25f);
	float term1 = dot(n, wi) / PI_F;
	float term2 = ggx_D(n, h, mat) * dot(n, h) / (4.0f * dot(wi, h));
	return (1 - t) * term1 + t * term2;
}

/* GGX::sample (brdf.cuh:385-433) */
f3 ggx_sample(const Material &mat, f3 n, f3 wo, f3 &seed)
{
	if (dot(wo, n) <= 0.0f)
		n = -n;
	float avg_Kd = (mat.diffuse.x + mat.diffuse.y + mat.diffuse.z) / 3.0f;
	float avg_Ks = (mat.specular.x + mat.specular.y + mat.specular.z) / 3.0f;
	float t = 1.0f;
	if (avg_Kd + avg_Ks > 0.0f)
		t = avg_Ks / (avg_Kd + avg_Ks);
	f3 eta = rand_uniform_3f(seed);
	if (eta.x < t) {
		float k = ksqrt(eta.y / (1 - eta.y));
		float theta = katan(k * mat.roughness);
		float phi = 2.0f * PI_F * eta.z;
		float st, ct, sp, cp;
		ksincos(theta, st, ct);
		ksincos(phi, sp, cp);
		f3 h = mk(st * cp, st * sp, ct);
		h = rotate(h, n);
		return reflect(-wo, h);
	}
	float theta = kacos(ksqrt(eta.y));
	float phi = 2.0f * PI_F * eta.z;
	float st, ct, sp, cp;
	ksincos(theta, st, ct);
	ksincos(phi, sp, cp);
	f3 s = mk(st * cp, st * sp, ct);
	return rotate(s, n);
}

/* brdf() (brdf.cuh:437-449) for out = eDiffuse, the only lobe the path uses */
f3 brdf(const SurfaceHit &sh, f3 wi)
{
	return sh.mat.diffuse / PI_F + ggx_brdf(sh.mat, sh.n, wi, sh.wo);
}

/* Glass::sample (brdf.cuh:154-175) */
f3 glass_refract(f3 v, f3 n, float ni_over_nt)
{
	float cos_theta = dot(-v, n);
	f3 r_out_parallel = ni_over_nt * (v + cos_theta * n);
	float r_out_length = length(r_out_parallel);
	float r_out_length_squared = r_out_length * r_out_length;
	f3 r_out_perp = -ksqrt(fabsf(1.0f - r_out_length_squared)) * n;
	return r_out_parallel + r_out_perp;
}

/* eval() (brdf.cuh:573-589 -> eval<GGX> :477-492, Glass :576-583).  pdf is
 * set to 0 when the sampled direction is degenerate (the reference leaves
 * it unset there). */
f3 eval(const SurfaceHit &sh, f3 &wi, float &pdf, f3 &seed)
{
	if (sh.mat.type & KGR_SHADING_TRANSMISSION) {
		float eta = sh.mat.refraction;
		float cos_theta = kmin(dot(-sh.wo, sh.n), 1.0f);
		float sin_theta = ksqrt(1.0f - cos_theta * cos_theta);
		bool reflect_ray = (eta * sin_theta > 1.0f);
		float ni_over_nt = (float)(1.0 / (double)eta);
		if (!sh.entering)
			ni_over_nt = eta;
		wi = reflect_ray ? reflect(sh.wo, sh.n) : glass_refract(sh.wo, sh.n, ni_over_nt);
		pdf = 1.0f;
		return sh.mat.specular;
	}
	wi = ggx_sample(sh.mat, sh.n, sh.wo, seed);
	if (length(wi) < 1e-6f) {
		pdf = 0.0f;
		return mk(0.0f);
	}
	pdf = ggx_pdf(sh.mat, sh.n, wi, sh.wo);
	return brdf(sh, wi);
}

/* ============================================================== lights == */

struct TriLight {
	f3 a, ab, ac, intensity;
	/* TriangleLight::area (lighting.cuh:103-105): length * 0.5 in double */
	float area() const { return (float)((double)length(cross(ab, ac)) * 0.5); }
	f3 normal() const { return normalize(cross(ab, ac)); }
};

inline TriLight load_light(const kgr_triangle_light &l)
{
	return TriLight{mk(l.a[0], l.a[1], l.a[2]), mk(l.ab[0], l.ab[1], l.ab[2]),
		mk(l.ac[0], l.ac[1], l.ac[2]), mk(l.intensity[0], l.intensity[1], l.intensity[2])};
}

/* sample_area_light(TriangleLight) (lighting.cuh:133-146) */
f3 sample_area_light(const TriLight &light, f3 &seed)
{
	f3 r = pcg3f(seed);
	float u = fract(r.x);
	float v = fract(r.y);
	if (u + v > 1.0f) {
		u = 1.0f - u;
		v = 1.0f - v;
	}
	return light.a + u * light.ab + v * light.ac;
}

/* QuadLight (lighting.cuh:57-94): area = |ab x ac| */
struct QuadLight {
	f3 a, ab, ac, intensity;
	float area() const { return length(cross(ab, ac)); }
	f3 normal() const { return normalize(cross(ab, ac)); }
};

inline QuadLight load_quad(const kgr_quad_light &l)
{
	return QuadLight{mk(l.a[0], l.a[1], l.a[2]), mk(l.ab[0], l.ab[1], l.ab[2]),
		mk(l.ac[0], l.ac[1], l.ac[2]), mk(l.intensity[0], l.intensity[1], l.intensity[2])};
}

/* sample_area_light(QuadLight) (lighting.cuh:123-131) */
f3 sample_area_light(const QuadLight &light, f3 &seed)
{
	f3 r = pcg3f(seed);
	float u = fract(r.x);
	float v = fract(r.y);
	return light.a + u * light.ab + v * light.ac;
}

const double PI_D = 3.14159265358979323846; /* M_PI */
const float WORLD_RADIUS = 10000.0f;        /* Ld_Environment, amadeus_common.cuh:218 */

/* u = atan2(d.x, d.z) / (2 M_PI) + 0.5, v = asin(d.y) / M_PI + 0.5
 * (amadeus_path_tracer.cu:209-210): double arithmetic, one rounding. */
inline void env_uv(const f3 &d, float &u, float &v)
{
	u = (float)((double)katan2(d.x, d.z) / (2.0 * PI_D) + 0.5);
	v = (float)((double)kasin(d.y) / PI_D + 0.5);
}

/* tex2D<float4> of the environment map with normalised coordinates and wrap
 * addressing, by the texture-fetching rules of the CUDA C++ Programming
 * Guide: the coordinate's fraction times the extent; point sampling takes
 * the texel it falls in, linear filtering blends the four texels around it
 * (minus half a texel) with weights held in fixed point with 8 fractional
 * bits.  Measured on a GB300 (a sweep of 65,536 coordinates over texels
 * holding their own index): the weights round half up, and the blend of
 * float32 texels is within 6e-8 relative of the exact blend. */
void env_fetch4(const oracle_scene *s, float u, float v, float out[4])
{
	const int W = (int)s->env_width, H = (int)s->env_height;
	/* the wrapped coordinate in fixed point with 24 fractional bits
	 * (truncated), then scaled by the extent: exact in double */
	double fu = (double)u - floor((double)u), fv = (double)v - floor((double)v);
	double x = floor(fu * 16777216.0) / 16777216.0 * W;
	double y = floor(fv * 16777216.0) / 16777216.0 * H;
	auto texel = [&](long i, long j) {
		i %= W;
		j %= H;
		if (i < 0)
			i += W;
		if (j < 0)
			j += H;
		const float *t = s->env + 4 * ((size_t)j * W + i);
		return t;
	};
	if (s->env_filter == KGR_FILTER_POINT) {
		const float *t = texel((long)floor(x), (long)floor(y));
		for (int k = 0; k < 4; k++)
			out[k] = t[k];
		return;
	}
	/* weights: the fraction below the texel centre, rounded half up to
	 * 8 fractional bits; the blend is evaluated in double and rounded once */
	double xb = x - 0.5, yb = y - 0.5;
	double i0 = floor(xb), j0 = floor(yb);
	double a = floor((xb - i0) * 256.0 + 0.5) / 256.0;
	double b = floor((yb - j0) * 256.0 + 0.5) / 256.0;
	long i = (long)i0, j = (long)j0;
	const float *t00 = texel(i, j), *t10 = texel(i + 1, j), *t01 = texel(i, j + 1), *t11 = texel(i + 1, j + 1);
	for (int k = 0; k < 4; k++)
		out[k] = (float)((1.0 - a) * (1.0 - b) * t00[k] + a * (1.0 - b) * t10[k] + (1.0 - a) * b * t01[k]
			+ a * b * t11[k]);
}

f3 env_fetch(const oracle_scene *s, float u, float v)
{
	float c[4];
	env_fetch4(s, u, v, c);
	return mk(c[0], c[1], c[2]);
}

/* The environment light's direction: seed = rand_uniform_3f(seed), theta =
 * acos(sqrt(1 - seed.x)), phi = 2 pi seed.y -- float with brdf.cuh's PI in
 * Ld_Environment (amadeus_common.cuh:215-238), double with M_PI in
 * sample_direct (:343-374). */
f3 env_direction(f3 &seed, bool phi_double)
{
	seed = rand_uniform_3f(seed);
	float theta = kacos(ksqrt(1.0f - fract(seed.x)));
	float phi = phi_double ? (float)(2.0 * PI_D * (double)fract(seed.y))
		: 2.0f * 3.14159265358979323846f * fract(seed.y);
	float st = ksin(theta);
	return mk(st * kcos(phi), st * ksin(phi), kcos(theta));
}

/* FullLightSample of sample_direct (amadeus_common.cuh:289-377) */
struct LightPoint {
	f3 Le, normal, point;
	float pdf;
	int type; /* 0 quad, 1 triangle, 2 environment */
	float env_u, env_v;
};

const float SHADOW_EPS = 0.05f; /* is_occluded, amadeus_common.cuh:193 */
const float OFFSET_EPS = 1e-3f; /* amadeus_common.cuh:22 */

struct Ctx {
	const oracle_scene *s;
	std::vector<TriLight> lights;
	std::vector<QuadLight> quads;
	bool env_flip_v = false; /* the path tracer's miss reads (u, 1 - v) */
	oracle_render_stats stats;
	uint64_t internal = 0, leaves = 0;
	float tmax_closest = 1e16f;

	bool occluded(const f3 &o, const f3 &d, float R)
	{
		stats.shadow_rays++;
		return trace_any(s, o, d, R - SHADOW_EPS, &internal, &leaves);
	}

	bool has_env() const { return s->env != nullptr; }

	/* __miss__ (amadeus_path_tracer.cu:204-220, amadeus_restir.cu:561-578) */
	f3 env_miss(const f3 &d) const
	{
		if (!has_env())
			return mk(0.0f);
		float u, v;
		env_uv(d, u, v);
		return env_fetch(s, u, env_flip_v ? 1.0f - v : v);
	}

	/* Ld (amadeus_common.cuh:256-286): a uniform pick over the quad lights,
	 * the triangle lights and the environment, with Ld_light
	 * (lighting.cuh:149-174) or Ld_Environment (amadeus_common.cuh:215-254). */
	f3 Ld(const SurfaceHit &sh, f3 &seed)
	{
		unsigned int nq = (unsigned int)quads.size(), nt = (unsigned int)lights.size();
		unsigned int total_count = nq + nt + (has_env() ? 1u : 0u);
		if (total_count == 0)
			return mk(0.0f);
		unsigned int i = (unsigned int)(rand_uniform(seed) * total_count);
		f3 contr = mk(0.0f);
		float pdf = 1.0f / total_count;
		float light_pdf = 0.0f;
		if (i < nq + nt) {
			f3 lpos, lnormal, Le;
			if (i < nq) {
				const QuadLight &light = quads[i];
				light_pdf = 1.0f / light.area();
				lpos = sample_area_light(light, seed);
				lnormal = light.normal();
				Le = light.intensity;
			} else {
				const TriLight &light = lights[i - nq];
				light_pdf = 1.0f / light.area();
				lpos = sample_area_light(light, seed);
				lnormal = light.normal();
				Le = light.intensity;
			}
			f3 wi = normalize(lpos - sh.x);
			float R = length(lpos - sh.x);
			if (!occluded(sh.x, wi, R)) {
				f3 f = brdf(sh, wi);
				float ldot = fabsf(dot(lnormal, wi));
				float geometric = ldot * fabsf(dot(sh.n, wi)) / (R * R);
				contr = f * Le * geometric;
			}
		} else {
			f3 wi = env_direction(seed, false);
			float u, v;
			env_uv(wi, u, v);
			f3 Li = env_fetch(s, u, v);
			light_pdf = (float)(1.0 / (4.0 * PI_D));
			if (!occluded(sh.x, wi, WORLD_RADIUS)) {
				f3 f = brdf(sh, wi) * fabsf(dot(sh.n, wi));
				contr = f * Li;
			}
		}
		pdf *= light_pdf;
		return contr / pdf;
	}

	/* sample_direct (amadeus_common.cuh:301-377).  Returns the light's place
	 * among quads + triangles + environment, or -1 with nothing to pick. */
	int sample_direct(const SurfaceHit &sh, f3 &seed, LightPoint &lp)
	{
		unsigned int nq = (unsigned int)quads.size(), nt = (unsigned int)lights.size();
		unsigned int total = nq + nt + (has_env() ? 1u : 0u);
		unsigned int li = (unsigned int)(rand_uniform(seed) * total);
		lp.env_u = lp.env_v = 0.0f;
		if (li < nq) {
			const QuadLight &l = quads[li];
			lp.point = sample_area_light(l, seed);
			lp.Le = l.intensity;
			lp.normal = l.normal();
			lp.pdf = 1.0f / (l.area() * total);
			lp.type = 0;
			return (int)li;
		}
		if (li < nq + nt) {
			const TriLight &l = lights[li - nq];
			lp.point = sample_area_light(l, seed);
			lp.Le = l.intensity;
			lp.normal = l.normal();
			lp.pdf = 1.0f / (l.area() * total);
			lp.type = 1;
			return (int)li;
		}
		if (li < total) {
			f3 wi = env_direction(seed, true);
			lp.point = sh.x + wi * WORLD_RADIUS;
			env_uv(wi, lp.env_u, lp.env_v);
			lp.Le = env_fetch(s, lp.env_u, lp.env_v);
			lp.normal = -wi;
			lp.pdf = (float)(1.0 / (4.0 * PI_D * (double)total));
			lp.type = 2;
			return (int)li;
		}
		lp.point = mk(0.0f);
		lp.pdf = 0.0f;
		lp.type = -1;
		return -1;
	}

	/* direct_unoccluded / direct_occluded (amadeus_common.cuh:380-421): the
	 * environment (type 2) has no light cosine and no 1/d^2 */
	f3 direct_typed(const SurfaceHit &sh, const f3 &Le, const f3 &normal, int type, f3 D, float d, bool test)
	{
		if (test && occluded(sh.x, D, d))
			return mk(0.0f);
		f3 rho = brdf(sh, D);
		float geometric = fabsf(dot(sh.n, D));
		if (type != 2) {
			float ldot = fabsf(dot(normal, D));
			geometric *= ldot / (d * d);
		}
		return rho * Le * geometric;
	}

	/* direct_unoccluded (amadeus_common.cuh:380-397) */
	f3 direct_unoccluded(const SurfaceHit &sh, const f3 &Le, const f3 &normal, f3 D, float d)
	{
		f3 rho = brdf(sh, D);
		float geometric = fabsf(dot(sh.n, D));
		float ldot = fabsf(dot(normal, D));
		geometric *= ldot / (d * d);
		return rho * Le * geometric;
	}

	/* direct_occluded (amadeus_common.cuh:399-421) */
	f3 direct_occluded(const SurfaceHit &sh, const f3 &Le, const f3 &normal, f3 D, float d)
	{
		f3 Li = mk(0.0f);
		if (!occluded(sh.x, D, d)) {
			f3 rho = brdf(sh, D);
			float geometric = fabsf(dot(sh.n, D));
			float ldot = fabsf(dot(normal, D));
			geometric *= ldot / (d * d);
			Li = rho * Le * geometric;
		}
		return Li;
	}
};

/* ============================================================ hit data == */

/* LOAD_INTERSECTION_DATA (amadeus_common.cuh:490-515) with
 * calculate_normal (:74-150), calculate_intersection (:62-71) and
 * calculate_material (:153-187); world-space vertices (identity model).
 * Returns false when the normal is NaN (the path then contributes 0). */
bool surface(const oracle_scene *s, const kgr_hit &h, const f3 &dir, SurfaceHit &sh)
{
	const uint32_t *t = s->tris + 4 * (size_t)h.prim;
	f3 a = ld3(s->positions, t[0]), b = ld3(s->positions, t[1]), c = ld3(s->positions, t[2]);
	f3 e1 = b - a;
	f3 e2 = c - a;
	f3 ng = normalize(cross(e1, e2));
	bool entering;
	if (dot(ng, dir) > 0.0f) {
		ng = -ng;
		entering = false;
	} else {
		entering = true;
	}
	ng = normalize(ng);
	f3 na = ld3(s->normals, t[0]), nb = ld3(s->normals, t[1]), nc = ld3(s->normals, t[2]);
	float w0 = 1.0f - h.b1 - h.b2;
	f3 normal = w0 * na + h.b1 * nb + h.b2 * nc;
	if (dot(normal, ng) < 0.0f)
		normal = -normal;
	normal = normalize(normal);
	f3 x = w0 * a + h.b1 * b + h.b2 * c;
	sh.mat = load_material(s->materials[t[3]]);
	sh.entering = entering;
	sh.n = normal;
	sh.wo = -dir;
	sh.x = x;
	return !anynan(normal);
}

/* make_ray (amadeus_path_tracer.cu:25-56; amadeus_restir.cu:30-65 uses a
 * fixed -0.5 offset but still draws once) */
void make_ray(const oracle_render_params *p, uint32_t ix, uint32_t iy, bool jitter,
		f3 &seed, f3 &origin, f3 &direction)
{
	f3 U = mk(p->ax_u[0], p->ax_u[1], p->ax_u[2]);
	f3 V = mk(p->ax_v[0], p->ax_v[1], p->ax_v[2]);
	f3 W = mk(p->ax_w[0], p->ax_w[1], p->ax_w[2]);
	pcg3f(seed);
	float xoffset = jitter ? (fract(seed.x) - 0.5f) : -0.5f;
	float yoffset = jitter ? (fract(seed.y) - 0.5f) : -0.5f;
	float ax = ((float)ix + xoffset) / (float)p->width;
	float ay = ((float)iy + yoffset) / (float)p->height;
	float dx = 2.0f * ax - 1.0f;
	float dy = 2.0f * ay - 1.0f;
	origin = mk(p->center[0], p->center[1], p->center[2]);
	direction = normalize(dx * U + dy * V + W);
}

struct PathResult {
	f3 L;
	f3 normal, albedo, position;
	bool hit;
};

/* One path of the recursive __closesthit__ (amadeus_path_tracer.cu:133-201)
 * written as a loop: L = sum_k beta_k * (Le_k + Ld_k), beta_{k+1} = beta_k *
 * f |wi.n| / pdf.  Hits at depth > max_depth contribute nothing
 * (LOAD_RAYPACKET, amadeus_common.cuh:480-488), so no ray is cast there.
 * Russian roulette follows naive_path_tracer.cu:294-303.  restir_primary
 * turns the depth-0 vertex into the ReSTIR initial vertex
 * (amadeus_restir.cu:473-526), which adds no direct term; `on_primary` is
 * then called to run RIS. */
template <class OnPrimary>
PathResult trace_path(Ctx &ctx, const oracle_render_params *p, f3 o, f3 d, f3 &seed,
		bool restir_primary, OnPrimary on_primary)
{
	PathResult r;
	r.L = mk(0.0f);
	r.normal = r.albedo = r.position = mk(0.0f);
	r.hit = false;
	f3 beta = mk(1.0f);
	/* no ray past the last vertex: the closest-hit and miss programs both
	 * return 0 for a ray at depth > max_depth (LOAD_RAYPACKET,
	 * amadeus_common.cuh:480-488), so such a ray adds nothing, hit or miss */
	const int last = p->max_depth;
	for (int depth = 0;; depth++) {
		if (depth > last)
			break;
		if (depth == 0)
			ctx.stats.camera_rays++;
		else
			ctx.stats.bounce_rays++;
		kgr_hit h = trace_closest(ctx.s, o, d, ctx.tmax_closest, &ctx.internal, &ctx.leaves);
		if (h.prim < 0) {
			if (ctx.has_env())
				r.L = r.L + beta * ctx.env_miss(d);
			break;
		}
		if (depth > p->max_depth)
			break;
		SurfaceHit sh;
		if (!surface(ctx.s, h, d, sh))
			break;
		f3 n = sh.n;
		float sgn = sh.mat.type == KGR_SHADING_TRANSMISSION ? -1.0f : 1.0f;
		sh.x = sh.x + sgn * n * OFFSET_EPS;
		if (depth == 0) {
			r.hit = true;
			r.normal = n;
			r.albedo = sh.mat.diffuse;
			r.position = sh.x;
		}
		if (restir_primary && depth == 0) {
			on_primary(sh, seed);
		} else {
			f3 direct = sh.mat.emission + ctx.Ld(sh, seed);
			r.L = r.L + beta * direct;
		}
		f3 wi;
		float pdf = 0.0f;
		f3 f = eval(sh, wi, pdf, seed);
		if (!(pdf > 0))
			break;
		f3 T = f * fabsf(dot(wi, n)) / pdf;
		beta = beta * T;
		if (p->russian_roulette && depth >= p->rr_start_depth) {
			float q = 1.0f - kmin(kmax(0.05f, beta.y), 1.0f);
			float rr = fract(seed.x);
			if (rr < q)
				break;
			beta = beta / (1.0f - q);
		}
		o = sh.x;
		d = wi;
	}
	return r;
}

struct NoPrimary {
	void operator()(const SurfaceHit &, f3 &) const {}
};

inline void store4(float *buf, size_t i, const f3 &v, float w)
{
	buf[4 * i + 0] = v.x;
	buf[4 * i + 1] = v.y;
	buf[4 * i + 2] = v.z;
	buf[4 * i + 3] = w;
}

inline f3 load4(const float *buf, size_t i) { return mk(buf[4 * i], buf[4 * i + 1], buf[4 * i + 2]); }

/* accumulate (amadeus_path_tracer.cu:59-70): glm::vec4 divided by a scalar
 * divides each component. */
inline void accumulate4(float *buf, size_t i, const f3 &v, float w, bool acc, float count)
{
	if (acc) {
		float *d = buf + 4 * i;
		float s[4] = {v.x, v.y, v.z, w};
		for (int c = 0; c < 4; c++)
			d[c] = (d[c] * count + s[c]) / (count + 1);
	} else {
		store4(buf, i, v, w);
	}
}

std::vector<QuadLight> load_quads(const oracle_scene *s)
{
	std::vector<QuadLight> q;
	for (uint32_t i = 0; i < s->quad_count; i++)
		q.push_back(load_quad(s->quads[i]));
	return q;
}

std::vector<TriLight> load_lights(const oracle_scene *s)
{
	std::vector<TriLight> v(s->light_count);
	for (uint32_t i = 0; i < s->light_count; i++)
		v[i] = load_light(s->lights[i]);
	return v;
}

void merge_stats(oracle_render_stats *dst, const oracle_render_stats &src)
{
	dst->camera_rays += src.camera_rays;
	dst->bounce_rays += src.bounce_rays;
	dst->shadow_rays += src.shadow_rays;
}

int nthreads(int t)
{
#ifdef _OPENMP
	return t > 0 ? t : omp_get_max_threads();
#else
	(void)t;
	return 1;
#endif
}

/* ============================================================== ReSTIR == */

/* A light sample: `light` is the light's place among quads + triangles,
 * -1 for none, or for the environment the bits of -u (negative, never -1)
 * with v in env_v; the map is read again at (u, v) for its Le. */
struct Sample {
	int light;
	f3 point;
	float env_v;
};

inline bool has_light(const Sample &smp) { return smp.light != -1; }

/* Le, normal and type of a sample's light */
int emitter(const Ctx &ctx, const Sample &smp, f3 &Le, f3 &normal)
{
	if (smp.light >= 0) {
		if ((size_t)smp.light < ctx.quads.size()) {
			const QuadLight &l = ctx.quads[smp.light];
			Le = l.intensity;
			normal = l.normal();
			return 0;
		}
		const TriLight &l = ctx.lights[smp.light - (int)ctx.quads.size()];
		Le = l.intensity;
		normal = l.normal();
		return 1;
	}
	Le = env_fetch(ctx.s, -u2f((uint32_t)smp.light), smp.env_v);
	normal = mk(0.0f);
	return 2;
}

/* Reservoir<T> (include/amadeus/reservoir.cuh:19-75) */
struct Reservoir {
	Sample data = {-1, {0.0f, 0.0f, 0.0f}, 0.0f};
	float w = 0.0f, W = 0.0f;
	int M = 0;
	f3 seed;

	bool update(const Sample &sample, float weight)
	{
		w += weight;
		float eta = rand_uniform(seed);
		bool selected = (eta * w) < weight;
		if (selected)
			data = sample;
		M++;
		return selected;
	}
	void resample(float target)
	{
		float d = target * M;
		W = (d > 0) ? w / d : 0.0f;
	}
	void reset()
	{
		w = 0.0f;
		M = 0;
		W = 0.0f;
	}
};

/* Salt of the RIS reservoir's own stream.  The reference seeds reservoirs
 * from std::random_device on the host (reservoir.cuh:29-36); here the seed
 * is a fixed function of pixel and frame so runs are reproducible. */
const uint32_t RIS_SALT = 0x9E3779B9u;

struct RestirBufs {
	int32_t *light; float *point; float *w; float *W; int32_t *M; float *env_v;
	Reservoir get(size_t i) const
	{
		Reservoir r;
		r.data.light = light[i];
		r.data.point = mk(point[3 * i], point[3 * i + 1], point[3 * i + 2]);
		r.data.env_v = env_v[i];
		r.w = w[i];
		r.W = W[i];
		r.M = M[i];
		return r;
	}
	void set(size_t i, const Reservoir &r) const
	{
		light[i] = r.data.light;
		env_v[i] = r.data.env_v;
		point[3 * i] = r.data.point.x;
		point[3 * i + 1] = r.data.point.y;
		point[3 * i + 2] = r.data.point.z;
		w[i] = r.w;
		W[i] = r.W;
		M[i] = r.M;
	}
	void reset(size_t i) const
	{
		w[i] = 0.0f;
		M[i] = 0;
		W[i] = 0.0f;
	}
};

/* target (amadeus_restir.cu:147-161) */
float target(Ctx &ctx, const Sample &smp, const SurfaceHit &hit)
{
	if (!has_light(smp))
		return 0.0f;
	f3 Le, ln;
	int type = emitter(ctx, smp, Le, ln);
	f3 D = smp.point - hit.x;
	float d = length(D);
	f3 Li = ctx.direct_typed(hit, Le, ln, type, D / d, d, false);
	return Li.x + Li.y + Li.z;
}

/* occluded_target (amadeus_restir.cu:163-178) */
float occluded_target(Ctx &ctx, const Sample &smp, const SurfaceHit &hit)
{
	if (!has_light(smp))
		return 0.0f;
	f3 Le, ln;
	int type = emitter(ctx, smp, Le, ln);
	f3 D = smp.point - hit.x;
	float d = length(D);
	f3 Li = ctx.direct_typed(hit, Le, ln, type, D / d, d, true);
	return Li.x + Li.y + Li.z;
}

/* glm::mat4 * glm::mat4 and mat4 * vec4, column-major, columns summed in
 * order (glm/detail/type_mat4x4.inl). */
void mat4_mul(const float *a, const float *b, float *out)
{
	for (int j = 0; j < 4; j++) {
		for (int i = 0; i < 4; i++) {
			float v = a[0 * 4 + i] * b[j * 4 + 0] + a[1 * 4 + i] * b[j * 4 + 1]
				+ a[2 * 4 + i] * b[j * 4 + 2] + a[3 * 4 + i] * b[j * 4 + 3];
			out[j * 4 + i] = v;
		}
	}
}

/* reproject (amadeus_restir.cu:181-210); indices past the image edge are
 * rejected instead of read out of bounds. */
int reproject(const oracle_render_params *p, int index, const f3 &position)
{
	if (p->samples > 0)
		return index;
	float pv[16];
	mat4_mul(p->prev_projection, p->prev_view, pv);
	float q[4];
	for (int i = 0; i < 4; i++)
		q[i] = pv[0 * 4 + i] * position.x + pv[1 * 4 + i] * position.y
			+ pv[2 * 4 + i] * position.z + pv[3 * 4 + i] * 1.0f;
	float u = q[0] / q[3];
	float v = q[1] / q[3];
	bool in_u = (u >= -1.0f && u <= 1.0f);
	bool in_v = (v >= -1.0f && v <= 1.0f);
	if (!(in_u && in_v))
		return -1;
	u = (u + 1.0f) * 0.5f;
	v = (v + 1.0f) * 0.5f;
	int ix = (int)((double)(u * (float)p->width) + 0.5);
	int iy = (int)((double)(v * (float)p->height) + 0.5);
	if (ix < 0 || iy < 0 || ix >= (int)p->width || iy >= (int)p->height)
		return -1;
	return iy * (int)p->width + ix;
}

/* sample_spatial_neighborhood (amadeus_restir.cu:294-314); 2 * M_PI is the
 * double constant of <math.h>, so theta is computed in double and rounded. */
int spatial_neighbor(const oracle_render_params *p, int index, f3 &seed, int radius)
{
	int width = (int)p->width, height = (int)p->height;
	int x = index % width;
	int y = index / width;
	f3 offset = rand_uniform_3f(seed);
	float theta = (float)(2.0 * 3.14159265358979323846 * (double)offset.x);
	float r = (float)radius * ksqrt(offset.y);
	float st, ct;
	ksincos(theta, st, ct);
	int x0 = (int)((float)x + r * ct);
	int y0 = (int)((float)y + r * st);
	x0 = x0 < 0 ? 0 : (x0 > width - 1 ? width - 1 : x0);
	y0 = y0 < 0 ? 0 : (y0 > height - 1 ? height - 1 : y0);
	return x0 + y0 * width;
}

/* glm::normalize(center - position) for the reuse passes' wo */
inline f3 view_wo(const oracle_render_params *p, const f3 &position)
{
	f3 c = mk(p->center[0], p->center[1], p->center[2]);
	return normalize(c - position);
}

} /* namespace */

/* ================================================================= API == */

extern "C" {

int64_t oracle_build_kobra(const float *boxes, uint32_t n, float *out_vec4, uint64_t capacity)
{
	Builder b;
	b.nodes.reserve(2 * (size_t)n);
	std::vector<int> ids(n);
	for (uint32_t i = 0; i < n; i++) {
		Node node;
		node.bbox.min = mk(boxes[6 * i + 0], boxes[6 * i + 1], boxes[6 * i + 2]);
		node.bbox.max = mk(boxes[6 * i + 3], boxes[6 * i + 4], boxes[6 * i + 5]);
		node.object = (int)i;
		b.nodes.push_back(node);
		ids[i] = (int)i;
	}
	int root = b.partition(ids);
	std::vector<float> buf;
	b.serialize(buf, root, -1);
	uint64_t count = buf.size() / 4;
	if (count > capacity)
		return -1;
	memcpy(out_vec4, buf.data(), buf.size() * sizeof(float));
	return (int64_t)count;
}

void oracle_triangle_boxes(const oracle_scene *s, float *boxes)
{
	for (uint32_t i = 0; i < s->triangle_count; i++) {
		Tri t = load_tri(s, (int)i);
		f3 mn = gmin(t.a, gmin(t.b, t.c));
		f3 mx = gmax(t.a, gmax(t.b, t.c));
		float *o = boxes + 6 * (size_t)i;
		o[0] = mn.x; o[1] = mn.y; o[2] = mn.z;
		o[3] = mx.x; o[4] = mx.y; o[5] = mx.z;
	}
}

void oracle_trace_closest(const oracle_scene *s, const float *rays, uint32_t n,
		kgr_hit *hits, oracle_trace_stats *stats, int threads)
{
	uint64_t internal = 0, leaves = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+:internal, leaves) num_threads(nthreads(threads))
	for (int64_t i = 0; i < (int64_t)n; i++) {
		const float *r = rays + 8 * i;
		hits[i] = trace_closest(s, mk(r[0], r[1], r[2]), mk(r[4], r[5], r[6]), r[7], &internal, &leaves);
	}
	if (stats) {
		stats->internal_visits += internal;
		stats->leaf_visits += leaves;
		stats->rays += n;
	}
}

void oracle_trace_any(const oracle_scene *s, const float *rays, uint32_t n,
		uint32_t *occluded, oracle_trace_stats *stats, int threads)
{
	uint64_t internal = 0, leaves = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+:internal, leaves) num_threads(nthreads(threads))
	for (int64_t i = 0; i < (int64_t)n; i++) {
		const float *r = rays + 8 * i;
		occluded[i] = trace_any(s, mk(r[0], r[1], r[2]), mk(r[4], r[5], r[6]), r[7], &internal, &leaves) ? 1u : 0u;
	}
	if (stats) {
		stats->internal_visits += internal;
		stats->leaf_visits += leaves;
		stats->rays += n;
	}
}

void oracle_trace_closest_brute(const oracle_scene *s, const float *rays, uint32_t n, kgr_hit *hits)
{
	/* rank = order of the leaf records in the threaded buffer */
	std::vector<int> order;
	for (uint32_t v = 0; v < s->bvh_vec4_count; v += 3) {
		int object = bits_i(s->bvh[4 * (size_t)v + 1]);
		if (object != -1)
			order.push_back(object);
	}
#pragma omp parallel for schedule(dynamic, 64)
	for (int64_t i = 0; i < (int64_t)n; i++) {
		const float *r = rays + 8 * i;
		f3 o = mk(r[0], r[1], r[2]), d = mk(r[4], r[5], r[6]);
		kgr_hit best = {-1, r[7], 0, 0};
		for (int prim : order) {
			Tri t = load_tri(s, prim);
			float b1 = 0, b2 = 0;
			float tt = intersect_triangle(t.a, t.b, t.c, o, d, b1, b2);
			if (tt > 0.0f && tt < best.t) {
				best.prim = prim;
				best.t = tt;
				best.b1 = b1;
				best.b2 = b2;
			}
		}
		hits[i] = best;
	}
}

static void render_pt_rows(const oracle_scene *s, const oracle_render_params *p,
		float *color, float *normal, float *albedo, float *position,
		double *out64, oracle_render_stats *stats)
{
	std::vector<TriLight> lights = load_lights(s);
	uint32_t row_end = p->row_end ? p->row_end : p->height;
	int64_t npix = (int64_t)(row_end - p->row_begin) * p->width;
	oracle_render_stats total = {0, 0, 0};
#pragma omp parallel num_threads(nthreads(p->threads))
	{
		Ctx ctx;
		ctx.s = s;
		ctx.lights = lights;
		ctx.quads = load_quads(s);
		ctx.env_flip_v = true;
		ctx.stats = {0, 0, 0};
#pragma omp for schedule(dynamic, 64)
		for (int64_t k = 0; k < npix; k++) {
			uint32_t iy = p->row_begin + (uint32_t)(k / p->width);
			uint32_t ix = (uint32_t)(k % p->width);
			uint32_t pix = ix + iy * p->width;
			double acc[3] = {0, 0, 0};
			for (int sidx = 0; sidx < p->spp; sidx++) {
				uint32_t stream = p->frame * (uint32_t)p->spp + (uint32_t)sidx;
				f3 seed = pixel_seed(pix, stream, 0);
				f3 o, d;
				make_ray(p, ix, iy, true, seed, o, d);
				PathResult r = trace_path(ctx, p, o, d, seed, false, NoPrimary());
				f3 L = r.L;
				if (anynan(L))
					L = mk(1.0f, 0.0f, 1.0f);
				if (out64) {
					acc[0] += L.x;
					acc[1] += L.y;
					acc[2] += L.z;
					continue;
				}
				bool acc_on = p->accumulate || sidx > 0;
				float count = (float)(p->accumulate ? p->samples + sidx : sidx);
				accumulate4(color, pix, L, 1.0f, acc_on, count);
				accumulate4(normal, pix, r.normal, 0.0f, acc_on, count);
				accumulate4(albedo, pix, r.albedo, 0.0f, acc_on, count);
				store4(position, pix, r.position, 0.0f);
			}
			if (out64) {
				for (int c = 0; c < 3; c++)
					out64[3 * (size_t)pix + c] = acc[c] / p->spp;
			}
		}
#pragma omp critical
		merge_stats(&total, ctx.stats);
	}
	if (stats)
		merge_stats(stats, total);
}

void oracle_render_pt(const oracle_scene *s, const oracle_render_params *p,
		float *color, float *normal, float *albedo, float *position,
		oracle_render_stats *stats)
{
	render_pt_rows(s, p, color, normal, albedo, position, nullptr, stats);
}

void oracle_render_pt_f64(const oracle_scene *s, const oracle_render_params *p,
		double *out_rgb, oracle_render_stats *stats)
{
	render_pt_rows(s, p, nullptr, nullptr, nullptr, nullptr, out_rgb, stats);
}

void oracle_render_restir(const oracle_scene *s, const oracle_render_params *p,
		oracle_restir_state *st, float *color, float *normal, float *albedo,
		float *position, oracle_render_stats *stats)
{
	std::vector<TriLight> lights = load_lights(s);
	int64_t npix = (int64_t)p->width * p->height;
	RestirBufs A = {st->cur_light, st->cur_point, st->cur_w, st->cur_W, st->cur_M, st->cur_env_v};
	RestirBufs B = {st->prev_light, st->prev_point, st->prev_w, st->prev_W, st->prev_M, st->prev_env_v};
	oracle_render_stats total = {0, 0, 0};
	float count = (float)p->samples;
	bool acc = p->accumulate != 0;

	/* ---- initial pass (amadeus_restir.cu:82-144, 437-559) ---- */
#pragma omp parallel num_threads(nthreads(p->threads))
	{
		Ctx ctx;
		ctx.s = s;
		ctx.lights = lights;
		ctx.quads = load_quads(s);
		ctx.stats = {0, 0, 0};
#pragma omp for schedule(dynamic, 64)
		for (int64_t k = 0; k < npix; k++) {
			uint32_t ix = (uint32_t)(k % p->width), iy = (uint32_t)(k / p->width);
			uint32_t pix = (uint32_t)k;
			A.reset(pix);
			f3 seed = pixel_seed(pix, p->frame, 0);
			f3 o, d;
			make_ray(p, ix, iy, false, seed, o, d);
			auto ris = [&](const SurfaceHit &sh, f3 &pseed) {
				Reservoir res;
				res.seed = pixel_seed(pix, p->frame, RIS_SALT);
				res.data.light = -1;
				res.data.point = mk(0.0f);
				res.data.env_v = 0.0f;
				for (int i = 0; i < p->candidates; i++) {
					Sample smp;
					LightPoint lp;
					int li = ctx.sample_direct(sh, pseed, lp);
					float pdf = 0.0f, tgt = 0.0f;
					if (li >= 0) {
						smp.light = lp.type == 2 ? (int)f2u(-lp.env_u) : li;
						smp.point = lp.point;
						smp.env_v = lp.env_v;
						pdf = lp.pdf;
						f3 D = smp.point - sh.x;
						float dd = length(D);
						f3 Li = ctx.direct_typed(sh, lp.Le, lp.normal, lp.type, D / dd, dd, false);
						tgt = Li.x + Li.y + Li.z;
					} else {
						smp.light = -1;
						smp.point = mk(0.0f);
						smp.env_v = 0.0f;
					}
					res.update(smp, (pdf > 0) ? tgt / pdf : 0);
				}
				float tgt = 0.0f;
				f3 D = mk(0.0f);
				float dd = 0.0f;
				if (has_light(res.data)) {
					f3 Le, ln;
					int type = emitter(ctx, res.data, Le, ln);
					D = res.data.point - sh.x;
					dd = length(D);
					f3 Li = ctx.direct_typed(sh, Le, ln, type, D / dd, dd, true);
					tgt = Li.x + Li.y + Li.z;
				}
				res.resample(tgt);
				bool occ = ctx.occluded(sh.x, D / dd, dd);
				res.W *= 1.0f - (occ ? 1.0f : 0.0f);
				A.set(pix, res);
				kgr_material m;
				memcpy(m.diffuse, &sh.mat.diffuse, 12);
				memcpy(m.specular, &sh.mat.specular, 12);
				memcpy(m.emission, &sh.mat.emission, 12);
				memcpy(m.ambient, &sh.mat.ambient, 12);
				m.shininess = sh.mat.shininess;
				m.roughness = sh.mat.roughness;
				m.refraction = sh.mat.refraction;
				m.type = sh.mat.type;
				st->materials[pix] = m;
			};
			PathResult r = trace_path(ctx, p, o, d, seed, true, ris);
			f3 L = r.L;
			if (anynan(L))
				L = mk(1.0f, 0.0f, 1.0f);
			store4(st->intermediate, pix, L, 1.0f);
			store4(st->auxiliary, pix, seed, 1.0f);
			accumulate4(normal, pix, r.normal, 0.0f, acc, count);
			accumulate4(albedo, pix, r.albedo, 0.0f, acc, count);
			store4(position, pix, r.position, 0.0f);
		}
#pragma omp critical
		merge_stats(&total, ctx.stats);
	}

	/* ---- temporal pass (amadeus_restir.cu:213-291): current = A, previous = B ---- */
	if (p->temporal) {
#pragma omp parallel num_threads(nthreads(p->threads))
		{
			Ctx ctx;
			ctx.s = s;
			ctx.lights = lights;
			ctx.quads = load_quads(s);
			ctx.stats = {0, 0, 0};
#pragma omp for schedule(dynamic, 64)
			for (int64_t k = 0; k < npix; k++) {
				int pix = (int)k;
				Reservoir cur = A.get(pix);
				if (cur.M <= 0)
					continue;
				f3 xpos = load4(position, pix);
				SurfaceHit hit;
				hit.mat = load_material(st->materials[pix]);
				hit.entering = false;
				hit.n = load4(normal, pix);
				hit.wo = view_wo(p, xpos);
				hit.x = xpos;
				int pindex = reproject(p, pix, xpos);
				Reservoir merged;
				merged.seed = load4(st->auxiliary, pix);
				float t_current = occluded_target(ctx, cur.data, hit);
				merged.update(cur.data, t_current * cur.W * cur.M);
				int N = cur.M;
				if (pindex >= 0) {
					Reservoir prev = B.get(pindex);
					if (prev.M > 0) {
						prev.M = prev.M < p->temporal_mcap ? prev.M : p->temporal_mcap;
						float t_previous = occluded_target(ctx, prev.data, hit);
						merged.update(prev.data, t_previous * prev.W * prev.M);
						N += (t_previous > 0) * prev.M;
					}
				}
				merged.M = N;
				float t_merged = target(ctx, merged.data, hit);
				merged.resample(t_merged);
				A.set(pix, merged);
			}
#pragma omp critical
			merge_stats(&total, ctx.stats);
		}
	}

	/* ---- spatial passes (amadeus_restir.cu:317-434), ping-pong of
	 * restir.cuh:280-300: read `in`, write `out`, then swap ---- */
	RestirBufs in = A, out = B;
	for (int pass = 0; pass < p->spatial_passes; pass++) {
#pragma omp parallel num_threads(nthreads(p->threads))
		{
			Ctx ctx;
			ctx.s = s;
			ctx.lights = lights;
			ctx.quads = load_quads(s);
			ctx.stats = {0, 0, 0};
			const int K = p->spatial_neighbors;
			std::vector<SurfaceHit> hits(K);
			std::vector<int> sizes(K);
#pragma omp for schedule(dynamic, 64)
			for (int64_t k = 0; k < npix; k++) {
				int pix = (int)k;
				f3 xpos = load4(position, pix);
				SurfaceHit hit;
				hit.mat = load_material(st->materials[pix]);
				hit.entering = false;
				hit.n = load4(normal, pix);
				hit.wo = view_wo(p, xpos);
				hit.x = xpos;
				Reservoir current = in.get(pix);
				f3 direct = mk(0.0f);
				if (current.M > 0) {
					Reservoir merged;
					merged.seed = load4(st->auxiliary, pix);
					float t_current = target(ctx, current.data, hit);
					merged.update(current.data, t_current * current.W * current.M);
					int cnt = 0;
					for (int i = 0; i < K; i++) {
						int index0 = spatial_neighbor(p, pix, merged.seed, p->spatial_radius);
						Reservoir nb = in.get(index0);
						if (nb.M > 0) {
							float t_neighbor = occluded_target(ctx, nb.data, hit);
							merged.update(nb.data, t_neighbor * nb.W * nb.M);
						}
						SurfaceHit h0;
						h0.mat = load_material(st->materials[index0]);
						h0.entering = nb.M > 0;
						h0.n = load4(normal, index0);
						h0.wo = hit.wo;
						h0.x = load4(position, index0);
						hits[i] = h0;
						sizes[i] = nb.M;
						cnt += nb.M;
					}
					merged.M = current.M + cnt;
					int Z = current.M;
					for (int i = 0; i < K; i++) {
						float t_neighbor = hits[i].entering ? occluded_target(ctx, merged.data, hits[i]) : 0.0f;
						if (t_neighbor > 0.0f)
							Z += sizes[i];
					}
					float t_merged = target(ctx, merged.data, hit);
					float denominator = t_merged * Z;
					merged.W = (denominator > 0.0f) ? merged.w / denominator : 0.0f;
					f3 lighting = mk(0.0f);
					if (has_light(merged.data)) {
						f3 Le, ln;
						int type = emitter(ctx, merged.data, Le, ln);
						f3 D = merged.data.point - hit.x;
						float dd = length(D);
						lighting = ctx.direct_typed(hit, Le, ln, type, D / dd, dd, true);
					}
					direct = hit.mat.emission + lighting * merged.W;
					out.set(pix, merged);
				} else {
					out.reset(pix);
				}
				f3 c = direct + load4(st->intermediate, pix);
				float cw = 1.0f + st->intermediate[4 * (size_t)pix + 3];
				if (anynan(c) || kisnan(cw)) {
					c = mk(1.0f, 0.0f, 1.0f);
					cw = 1.0f;
				}
				accumulate4(color, pix, c, cw, acc, count);
			}
#pragma omp critical
			merge_stats(&total, ctx.stats);
		}
		std::swap(in, out);
	}
	/* restir.cuh:300: the final swap makes `previous` the last spatial
	 * output.  With the pass loop's swaps, that output is now `in`; copy it
	 * into the caller's prev buffers if it lives in the cur buffers. */
	if (p->spatial_passes > 0 && in.light == A.light) {
		for (int64_t k = 0; k < npix; k++)
			B.set(k, A.get(k));
	}
	if (stats)
		merge_stats(stats, total);
}

/* ================================================================== GI == */

namespace {

const float GI_COS_10DEG = 0.984807753f;
const uint32_t GI_REUSE_SALT = 0x47495255u; /* streams of the reuse passes (gi.cu) */
/* shifts with a Jacobian outside [1/4, 4] are invalid (gi.cu with its
 * default gi_jacobian_max of 4) */
#define KGR_GI_JACOBIAN_MIN 0.25f
#define KGR_GI_JACOBIAN_MAX 4.0f

struct GiS {
	f3 xs, ns, Lo;
	bool rc = true; /* reconnectable: W is stored with its sign bit set when not */
};

/* gi_reconnectable (kgr_device.cuh): no transmission, roughness >= 0.3 */
inline bool gi_rc(const Material &m)
{
	return m.type != KGR_SHADING_TRANSMISSION && m.roughness >= 0.3f;
}

inline void gi_load(const float *a, const float *b, size_t i, GiS &s, float &W, int &M)
{
	uint32_t w = f2u(a[4 * i + 3]);
	s.xs = mk(a[4 * i], a[4 * i + 1], a[4 * i + 2]);
	s.ns = unpack_normal(w);
	s.Lo = mk(b[4 * i], b[4 * i + 1], b[4 * i + 2]);
	s.rc = !std::signbit(b[4 * i + 3]);
	W = fabsf(b[4 * i + 3]);
	M = unpack_m(w);
}

inline void gi_store(float *a, float *b, size_t i, const GiS &s, float W, int M)
{
	a[4 * i] = s.xs.x; a[4 * i + 1] = s.xs.y; a[4 * i + 2] = s.xs.z;
	a[4 * i + 3] = u2f(pack_normal_m(s.ns, M));
	b[4 * i] = s.Lo.x; b[4 * i + 1] = s.Lo.y; b[4 * i + 2] = s.Lo.z; b[4 * i + 3] = s.rc ? W : -W;
}

inline float gi_norm(float w_sum, int Z, float target)
{
	if (!(target > 0.0f) || Z <= 0)
		return 0.0f;
	return (float)((double)w_sum / ((double)Z * (double)target));
}

inline float gi_jac(const f3 &xq, const f3 &xr, const GiS &s)
{
	f3 dq = xq - s.xs, dr = xr - s.xs;
	float lq2 = dot(dq, dq), lr2 = dot(dr, dr);
	float cq = fabsf(dot(s.ns, dq)) / ksqrt(lq2);
	float cr = fabsf(dot(s.ns, dr)) / ksqrt(lr2);
	float j = (cq / cr) * (lr2 / lq2);
	return (j >= KGR_GI_JACOBIAN_MIN && j <= KGR_GI_JACOBIAN_MAX) ? j : 0.0f;
}

/* src: domain of the selected sample (-1 the centre) */
struct GiMergeO {
	GiS sel;
	float w = 0.0f;
	int src = -1;
	f3 seed;
	void update(const GiS &s, float weight, int from)
	{
		w += weight;
		float eta = rand_uniform(seed);
		if ((eta * w) < weight) {
			sel = s;
			src = from;
		}
	}
};

/* balance-heuristic contribution weight W = num w_sum / (D p^_q) (gi.cu) */
inline float gi_mis(float w_sum, float num, float D, float target)
{
	if (!(target > 0.0f) || !(D > 0.0f))
		return 0.0f;
	return (float)(((double)num * (double)w_sum) / ((double)D * (double)target));
}

/* G-buffer entry; position.w = material index + 1 (0: no hit) */
struct GB {
	f3 x, n;
	bool hit;
	uint32_t mat;
};

inline GB gb_at(const float *pos, const float *nrm, size_t i)
{
	GB g;
	g.x = mk(pos[4 * i], pos[4 * i + 1], pos[4 * i + 2]);
	g.n = mk(nrm[4 * i], nrm[4 * i + 1], nrm[4 * i + 2]);
	g.hit = pos[4 * i + 3] > 0.0f;
	g.mat = g.hit ? (uint32_t)pos[4 * i + 3] - 1u : 0u;
	return g;
}

inline bool gi_similar(const GB &a, float da, const GB &b, float db)
{
	if (!a.hit || !b.hit)
		return false;
	if (dot(a.n, b.n) < GI_COS_10DEG)
		return false;
	return fabsf(db - da) / da <= 0.1f;
}

inline bool gi_visible(Ctx &ctx, const f3 &from, const f3 &to)
{
	f3 D = to - from;
	float d = length(D);
	return !ctx.occluded(from, D / d, d);
}

int gi_neighbor(const oracle_render_params *p, int index, f3 &seed, int radius)
{
	return spatial_neighbor(p, index, seed, radius);
}

/* The receiver of a GI sample at a pixel: its material, shading normal and
 * the direction toward the camera centre. */
inline SurfaceHit gi_receiver(const kgr_material &m, const GB &g, const f3 &center)
{
	SurfaceHit h;
	h.mat = load_material(m);
	h.entering = false;
	h.n = g.n;
	h.wo = normalize(center - g.x);
	h.x = g.x;
	return h;
}

/* Target function of sample s at receiver h: sum_rgb(f L_o) |n.w|. */
inline float gi_target(const SurfaceHit &h, const GiS &s)
{
	f3 D = s.xs - h.x;
	float d = length(D);
	f3 w = D / d;
	f3 v = brdf(h, w) * s.Lo * fabsf(dot(h.n, w));
	float t = v.x + v.y + v.z;
	return (t > 0.0f && t < 1e30f) ? t : 0.0f;
}

} /* namespace */

extern "C" void oracle_render_gi(const oracle_scene *s, const oracle_render_params *p, oracle_gi_state *st,
		float *color, float *direct_out, oracle_render_stats *stats)
{
	std::vector<TriLight> lights = load_lights(s);
	size_t npix = (size_t)p->width * p->height;
	std::vector<float> pos(4 * npix, 0.0f), nrm(4 * npix, 0.0f), dir(4 * npix, 0.0f), direct(4 * npix, 0.0f);
	std::vector<float> aux(4 * npix, 0.0f);
	std::vector<kgr_material> mats(npix);
	std::vector<float> cur_a(4 * npix), cur_b(4 * npix), tmp_a(4 * npix), tmp_b(4 * npix);
	oracle_render_stats total = {0, 0, 0};
	f3 center = mk(p->center[0], p->center[1], p->center[2]);
	f3 pcenter = mk(st->prev_center[0], st->prev_center[1], st->prev_center[2]);

	/* primary vertex, DI candidates, GI path, initial reservoir */
#pragma omp parallel num_threads(nthreads(p->threads))
	{
		Ctx ctx;
		ctx.s = s;
		ctx.lights = lights;
		ctx.stats = {0, 0, 0};
#pragma omp for schedule(dynamic, 64)
		for (int64_t k = 0; k < (int64_t)npix; k++) {
			uint32_t pix = (uint32_t)k;
			uint32_t ix = pix % p->width, iy = pix / p->width;
			f3 seed = pixel_seed(pix, p->frame, 0);
			f3 o, d;
			make_ray(p, ix, iy, true, seed, o, d);
			ctx.stats.camera_rays++;
			kgr_hit h = trace_closest(s, o, d, 1e16f, &ctx.internal, &ctx.leaves);
			SurfaceHit sh;
			GiS smp = {mk(0.0f), mk(0.0f, 0.0f, 1.0f), mk(0.0f), true};
			bool valid = false;
			float gpdf = 0.0f;
			if (h.prim >= 0 && surface(s, h, d, sh)) {
				f3 n3 = sh.n;
				float sgn = sh.mat.type == KGR_SHADING_TRANSMISSION ? -1.0f : 1.0f;
				sh.x = sh.x + sgn * n3 * OFFSET_EPS;
				store4(pos.data(), pix, sh.x, (float)(s->tris[4 * (size_t)h.prim + 3] + 1u));
				store4(nrm.data(), pix, n3, 0.0f);
				mats[pix] = s->materials[s->tris[4 * (size_t)h.prim + 3]];
				/* DI candidates */
				f3 risseed = pixel_seed(pix, p->frame, RIS_SALT);
				float wsum = 0.0f;
				int M = 0, sel = -1;
				f3 selp = mk(0.0f);
				unsigned int tot = (unsigned int)lights.size();
				for (int c = 0; c < p->candidates; c++) {
					unsigned int li = (unsigned int)(rand_uniform(seed) * tot);
					float weight = 0.0f;
					f3 pt = mk(0.0f);
					if (li < tot) {
						const TriLight &l = lights[li];
						pt = sample_area_light(l, seed);
						float pdf = 1.0f / (l.area() * tot);
						f3 D = pt - sh.x;
						float dd = length(D);
						f3 Li = ctx.direct_unoccluded(sh, l.intensity, l.normal(), D / dd, dd);
						float tgt = Li.x + Li.y + Li.z;
						weight = (pdf > 0) ? tgt / pdf : 0;
					}
					wsum += weight;
					float eta = rand_uniform(risseed);
					if ((eta * wsum) < weight) {
						sel = (int)li;
						selp = pt;
					}
					M++;
				}
				f3 dl = mk(0.0f);
				if (sel >= 0) {
					const TriLight &l = lights[sel];
					f3 D = selp - sh.x;
					float dd = length(D);
					f3 Dn = D / dd;
					if (!ctx.occluded(sh.x, Dn, dd)) {
						f3 Li = ctx.direct_unoccluded(sh, l.intensity, l.normal(), Dn, dd);
						float tgt = Li.x + Li.y + Li.z;
						float den = tgt * M;
						float W = (den > 0) ? wsum / den : 0.0f;
						dl = Li * W;
					}
				}
				store4(direct.data(), pix, dl, 0.0f);
				/* GI path from the BSDF-sampled direction, throughput 1 */
				f3 wi;
				float pdf = 0.0f;
				eval(sh, wi, pdf, seed);
				if (pdf > 0 && p->max_depth >= 1) {
					gpdf = pdf;
					store4(dir.data(), pix, wi, pdf);
					f3 L = mk(0.0f), beta = mk(1.0f);
					f3 oo = sh.x, dd3 = wi;
					bool captured = false;
					for (int depth = 1; depth <= p->max_depth; depth++) {
						ctx.stats.bounce_rays++;
						kgr_hit hh = trace_closest(s, oo, dd3, 1e16f, &ctx.internal, &ctx.leaves);
						if (hh.prim < 0)
							break;
						SurfaceHit s2;
						if (!surface(s, hh, dd3, s2))
							break;
						f3 n2 = s2.n;
						float sg = s2.mat.type == KGR_SHADING_TRANSMISSION ? -1.0f : 1.0f;
						s2.x = s2.x + sg * n2 * OFFSET_EPS;
						if (depth == 1) {
							smp.xs = s2.x;
							smp.ns = n2;
							smp.rc = gi_rc(s2.mat);
							captured = true;
						}
						f3 dir2 = s2.mat.emission + ctx.Ld(s2, seed);
						L = L + beta * dir2;
						f3 w2;
						float pdf2 = 0.0f;
						f3 f2 = eval(s2, w2, pdf2, seed);
						if (!(pdf2 > 0))
							break;
						beta = beta * (f2 * fabsf(dot(w2, n2)) / pdf2);
						if (p->russian_roulette && depth >= p->rr_start_depth) {
							float q = 1.0f - kmin(kmax(0.05f, beta.y), 1.0f);
							if (fract(seed.x) < q)
								break;
							beta = beta / (1.0f - q);
						}
						oo = s2.x;
						dd3 = w2;
					}
					smp.Lo = L;
					valid = captured && !anynan(L);
				}
			}
			store4(aux.data(), pix, seed, 1.0f);
			float W = 0.0f;
			if (valid) {
				float target = gi_target(gi_receiver(mats[pix], gb_at(pos.data(), nrm.data(), pix), center), smp);
				W = gi_norm(target / gpdf, 1, target);
			} else {
				smp.xs = smp.Lo = mk(0.0f);
				smp.ns = mk(0.0f, 0.0f, 1.0f);
				smp.rc = true;
			}
			gi_store(cur_a.data(), cur_b.data(), pix, smp, W, 1);
		}
#pragma omp critical
		merge_stats(&total, ctx.stats);
	}

	/* temporal */
	if (st->gi_temporal) {
		float pv[16];
		mat4_mul(p->prev_projection, p->prev_view, pv);
#pragma omp parallel num_threads(nthreads(p->threads))
		{
			Ctx ctx;
			ctx.s = s;
			ctx.lights = lights;
			ctx.stats = {0, 0, 0};
#pragma omp for schedule(dynamic, 64)
			for (int64_t k = 0; k < (int64_t)npix; k++) {
				size_t pix = (size_t)k;
				GB g = gb_at(pos.data(), nrm.data(), pix);
				if (!g.hit)
					continue;
				/* reprojection as reproject() without the samples > 0 shortcut */
				float qv[4];
				for (int i = 0; i < 4; i++)
					qv[i] = pv[0 * 4 + i] * g.x.x + pv[1 * 4 + i] * g.x.y + pv[2 * 4 + i] * g.x.z
						+ pv[3 * 4 + i] * 1.0f;
				float u = qv[0] / qv[3], v = qv[1] / qv[3];
				if (!(u >= -1.0f && u <= 1.0f && v >= -1.0f && v <= 1.0f))
					continue;
				u = (u + 1.0f) * 0.5f;
				v = (v + 1.0f) * 0.5f;
				int ixp = (int)((double)(u * (float)p->width) + 0.5);
				int iyp = (int)((double)(v * (float)p->height) + 0.5);
				if (ixp < 0 || iyp < 0 || ixp >= (int)p->width || iyp >= (int)p->height)
					continue;
				size_t pi = (size_t)iyp * p->width + ixp;
				GB gp = gb_at(st->prev_position, st->prev_normal, pi);
				if (!gi_similar(g, length(g.x - center), gp, length(gp.x - pcenter)))
					continue;
				GiS ps, cs;
				float pW, cW;
				int pM, cM;
				gi_load(st->res_a, st->res_b, pi, ps, pW, pM);
				if (pM <= 0)
					continue;
				gi_load(cur_a.data(), cur_b.data(), pix, cs, cW, cM);
				int pMc = pM < st->gi_mcap ? pM : st->gi_mcap;
				SurfaceHit h = gi_receiver(mats[pix], g, center);
				GiMergeO r;
				r.sel = {mk(0.0f), mk(0.0f), mk(0.0f), true};
				r.seed = pixel_seed((uint32_t)pix, p->frame, GI_REUSE_SALT);
				r.update(cs, gi_target(h, cs) * cW * cM, -1);
				float J = gi_jac(g.x, gp.x, ps);
				float wp = gi_target(h, ps) * J * pW * pMc;
				r.update(ps, wp, 0);
				/* the history counts whether or not its sample carries weight */
				int Mt = cM + pMc;
				float tq = gi_target(h, r.sel);
				float jp = gi_jac(gp.x, g.x, r.sel);
				float tp = jp > 0.0f ? gi_target(gi_receiver(s->materials[gp.mat], gp, pcenter), r.sel) * jp : 0.0f;
				float D = (float)cM * tq + (float)pMc * tp;
				float W = gi_mis(r.w, r.src < 0 ? tq : tp, D, tq);
				gi_store(cur_a.data(), cur_b.data(), pix, r.sel, W, Mt);
			}
#pragma omp critical
			merge_stats(&total, ctx.stats);
		}
	}

	/* spatial iterations, ping-pong */
	float *in_a = cur_a.data(), *in_b = cur_b.data(), *out_a = tmp_a.data(), *out_b = tmp_b.data();
	for (int it = 0; it < st->gi_spatial_iterations; it++) {
#pragma omp parallel num_threads(nthreads(p->threads))
		{
			Ctx ctx;
			ctx.s = s;
			ctx.lights = lights;
			ctx.stats = {0, 0, 0};
			std::vector<int> nidx(st->gi_neighbors), nM(st->gi_neighbors);
#pragma omp for schedule(dynamic, 64)
			for (int64_t k = 0; k < (int64_t)npix; k++) {
				size_t pix = (size_t)k;
				GiS cs;
				float cW;
				int cM;
				gi_load(in_a, in_b, pix, cs, cW, cM);
				GB g = gb_at(pos.data(), nrm.data(), pix);
				if (!g.hit) {
					gi_store(out_a, out_b, pix, cs, cW, cM);
					continue;
				}
				float depth = length(g.x - center);
				SurfaceHit h = gi_receiver(mats[pix], g, center);
				GiMergeO r;
				r.sel = {mk(0.0f), mk(0.0f), mk(0.0f), true};
				r.seed = pixel_seed((uint32_t)pix, p->frame, GI_REUSE_SALT + 1u + (uint32_t)it);
				r.update(cs, gi_target(h, cs) * cW * cM, -1);
				int Msum = cM;
				for (int i = 0; i < st->gi_neighbors; i++) {
					int index0 = gi_neighbor(p, (int)pix, r.seed, st->gi_radius);
					nidx[i] = -1;
					nM[i] = 0;
					GB gn = gb_at(pos.data(), nrm.data(), (size_t)index0);
					if (!gi_similar(g, depth, gn, length(gn.x - center)))
						continue;
					GiS ns;
					float nW;
					int nMi;
					gi_load(in_a, in_b, (size_t)index0, ns, nW, nMi);
					if (nMi <= 0)
						continue;
					/* the neighbour domain's confidence: at most the centre's M */
					int cn = st->gi_confidence_rule && cM < nMi ? cM : nMi;
					nidx[i] = index0;
					nM[i] = cn;
					Msum += cn;
					float J = ns.rc ? gi_jac(g.x, gn.x, ns) : 0.0f;
					float wn = J > 0.0f ? gi_target(h, ns) * J * nW * cn : 0.0f;
					if (wn > 0.0f && !gi_visible(ctx, g.x, ns.xs))
						wn = 0.0f;
					r.update(ns, wn, i);
				}
				/* balance heuristic over the centre and the neighbour domains */
				float target = gi_target(h, r.sel);
				float D = (float)cM * target;
				float num = r.src < 0 ? target : 0.0f;
				if (target > 0.0f && r.sel.rc) {
					for (int i = 0; i < st->gi_neighbors; i++) {
						if (nidx[i] < 0)
							continue;
						GB gn = gb_at(pos.data(), nrm.data(), (size_t)nidx[i]);
						float jn = gi_jac(gn.x, g.x, r.sel);
						float tn = jn > 0.0f
							? gi_target(gi_receiver(mats[(size_t)nidx[i]], gn, center), r.sel) * jn : 0.0f;
						if (tn > 0.0f && !gi_visible(ctx, gn.x, r.sel.xs))
							tn = 0.0f;
						D += (float)nM[i] * tn;
						if (i == r.src)
							num = tn;
					}
				}
				gi_store(out_a, out_b, pix, r.sel, gi_mis(r.w, num, D, target), Msum);
			}
#pragma omp critical
			merge_stats(&total, ctx.stats);
		}
		std::swap(in_a, out_a);
		std::swap(in_b, out_b);
	}

	/* final shading and history */
#pragma omp parallel num_threads(nthreads(p->threads))
	{
		Ctx ctx;
		ctx.s = s;
		ctx.lights = lights;
		ctx.stats = {0, 0, 0};
#pragma omp for schedule(dynamic, 64)
		for (int64_t k = 0; k < (int64_t)npix; k++) {
			size_t pix = (size_t)k;
			GB g = gb_at(pos.data(), nrm.data(), pix);
			f3 c = mk(0.0f);
			if (g.hit) {
				SurfaceHit h;
				h.mat = load_material(mats[pix]);
				h.entering = false;
				h.n = g.n;
				h.wo = normalize(center - g.x);
				h.x = g.x;
				GiS rs;
				float W;
				int M;
				gi_load(in_a, in_b, pix, rs, W, M);
				f3 gi = mk(0.0f);
				if (W > 0.0f) {
					f3 D = rs.xs - g.x;
					float d = length(D);
					f3 w = D / d;
					if (!ctx.occluded(g.x, w, d))
						gi = brdf(h, w) * rs.Lo * (fabsf(dot(h.n, w)) * W);
				}
				c = h.mat.emission + load4(direct.data(), pix) + gi;
			}
			if (anynan(c))
				c = mk(1.0f, 0.0f, 1.0f);
			accumulate4(color, pix, c, 1.0f, p->accumulate != 0, (float)p->samples);
			if (direct_out)
				memcpy(direct_out + 4 * pix, direct.data() + 4 * pix, 16);
		}
#pragma omp critical
		merge_stats(&total, ctx.stats);
	}
	memcpy(st->res_a, in_a, 16 * npix);
	memcpy(st->res_b, in_b, 16 * npix);
	memcpy(st->prev_position, pos.data(), 16 * npix);
	memcpy(st->prev_normal, nrm.data(), 16 * npix);
	memcpy(st->prev_center, p->center, 12);
	if (stats)
		merge_stats(stats, total);
}

/* --------------------------------------------------------- known answers */

void oracle_env_lookup(const float *texels, uint32_t width, uint32_t height, int filter, const float *uv,
		uint32_t n, float *rgb)
{
	oracle_scene s;
	memset(&s, 0, sizeof(s));
	s.env = texels;
	s.env_width = width;
	s.env_height = height;
	s.env_filter = filter;
	for (uint32_t i = 0; i < n; i++) {
		f3 c = env_fetch(&s, uv[2 * i], uv[2 * i + 1]);
		rgb[3 * i] = c.x;
		rgb[3 * i + 1] = c.y;
		rgb[3 * i + 2] = c.z;
	}
}

void oracle_kat_rng(float sx, float sy, float sz, int draws, float *out)
{
	f3 seed = mk(sx, sy, sz);
	for (int i = 0; i < draws; i++) {
		float u = rand_uniform(seed);
		out[4 * i + 0] = u;
		out[4 * i + 1] = seed.x;
		out[4 * i + 2] = seed.y;
		out[4 * i + 3] = seed.z;
	}
}

float oracle_kat_intersect(const float *v1, const float *v2, const float *v3,
		const float *o, const float *d, float *b1b2)
{
	float b1 = 0, b2 = 0;
	float t = intersect_triangle(mk(v1[0], v1[1], v1[2]), mk(v2[0], v2[1], v2[2]),
		mk(v3[0], v3[1], v3[2]), mk(o[0], o[1], o[2]), mk(d[0], d[1], d[2]), b1, b2);
	b1b2[0] = b1;
	b1b2[1] = b2;
	return t;
}

void oracle_kat_sample_light(const kgr_triangle_light *l, const float *seed, float *point, float *area_normal)
{
	TriLight L = load_light(*l);
	f3 sd = mk(seed[0], seed[1], seed[2]);
	f3 pt = sample_area_light(L, sd);
	point[0] = pt.x; point[1] = pt.y; point[2] = pt.z;
	f3 n = L.normal();
	area_normal[0] = L.area();
	area_normal[1] = n.x; area_normal[2] = n.y; area_normal[3] = n.z;
}

void oracle_kat_brdf_eval(const kgr_material *m, const float *n, const float *wo,
		const float *seed_in, float *out)
{
	SurfaceHit sh;
	sh.mat = load_material(*m);
	sh.entering = true;
	sh.n = mk(n[0], n[1], n[2]);
	sh.wo = mk(wo[0], wo[1], wo[2]);
	sh.x = mk(0.0f);
	f3 seed = mk(seed_in[0], seed_in[1], seed_in[2]);
	f3 wi;
	float pdf = 0;
	f3 f = eval(sh, wi, pdf, seed);
	float v[10] = {f.x, f.y, f.z, wi.x, wi.y, wi.z, pdf, seed.x, seed.y, seed.z};
	memcpy(out, v, sizeof(v));
}

void oracle_kat_brdf(const kgr_material *m, const float *n, const float *wo, const float *wi, float *out)
{
	SurfaceHit sh;
	sh.mat = load_material(*m);
	sh.entering = true;
	sh.n = mk(n[0], n[1], n[2]);
	sh.wo = mk(wo[0], wo[1], wo[2]);
	sh.x = mk(0.0f);
	f3 w = mk(wi[0], wi[1], wi[2]);
	f3 f = brdf(sh, w);
	out[0] = f.x; out[1] = f.y; out[2] = f.z;
	out[3] = ggx_pdf(sh.mat, sh.n, w, sh.wo);
}

void oracle_kat_math(const float *x, int n, float *out)
{
	for (int i = 0; i < n; i++) {
		out[5 * i + 0] = ksin(x[i]);
		out[5 * i + 1] = kcos(x[i]);
		out[5 * i + 2] = ktan(x[i]);
		out[5 * i + 3] = katan(x[i]);
		out[5 * i + 4] = kacos(x[i]);
	}
}

void oracle_kat_atan2_asin(const float *y, const float *x, int n, float *out)
{
	for (int i = 0; i < n; i++) {
		out[2 * i + 0] = katan2(y[i], x[i]);
		out[2 * i + 1] = kasin(y[i]);
	}
}

} /* extern "C" */

/* ========================================================== tonemapping == */

namespace {

/* clamp (include/cuda/math.cuh:101-104) */
inline float clamp_ref(float f, float a, float b) { return fmaxf(a, fminf(f, b)); }

/* aces (include/cuda/color.cuh:33-39), one channel */
inline float aces1(float c)
{
	float a = c * (c * 2.51f + 0.03f);
	float b = c * (c * 2.43f + 0.59f) + 0.14f;
	return clamp_ref(a / b, 0.0f, 1.0f);
}

/* srgb (color.cuh:13-30), one channel */
inline float srgb1(float c)
{
	float powed = powf(c, 1.0f / 2.4f);
	float s = c < 0.0031308f ? 12.92f * c : 1.055f * powed - 0.055f;
	return clamp_ref(s, 0.0f, 1.0f);
}

/* quantize_unsigned_8_bits (color.cuh:42-55) */
inline uint32_t quantize8(float x)
{
	x = clamp_ref(x, 0.0f, 1.0f);
	uint32_t q = (uint32_t)(x * 256.0f);
	return q < 255u ? q : 255u;
}

} /* namespace */

/* hdr_to_ldr_kernel (color.cuh:84-103): make_color + to_ui32 (cast.cuh:16-20)
 * of every pixel, rows written bottom to top. */
extern "C" void oracle_tonemap(const float *hdr, uint32_t *ldr, uint32_t width, uint32_t height, int mode)
{
	for (uint32_t y = 0; y < height; y++)
		for (uint32_t x = 0; x < width; x++) {
			const float *c = hdr + 4 * ((size_t)y * width + x);
			float r = mode == 0 ? aces1(c[0]) : srgb1(c[0]);
			float g = mode == 0 ? aces1(c[1]) : srgb1(c[1]);
			float b = mode == 0 ? aces1(c[2]) : srgb1(c[2]);
			ldr[(size_t)(height - y - 1) * width + x] =
				(255u << 24) | (quantize8(b) << 16) | (quantize8(g) << 8) | quantize8(r);
		}
}

/* ================================================================ Mamba == */
/*
 * The editor's Mamba frame (Mamba::render, editor/mamba.cu:941-1312) with
 * the deterministic choices of the GPU build: traced G-buffer at pixel
 * centres, probes allocated in 16x16-block order, bin radiance summed in
 * 64-bit fixed point (2^-20), a bin's depth from the frame's last splat in
 * splat order, every pass reading its inputs as they were when it began.
 * The state is kept in the GPU build's layouts so that every buffer can be
 * compared byte for byte.
 */

namespace {

const int M_BINS = 25;        /* IrradianceProbe::size^2 (probe.cuh:11) */
const int M_SIZE = 5;
const int M_REFS = 32767;     /* MAX_REFS (probe.cuh:78) */
const float M_PI_F = 3.14159265358979323846f;
const double M_PI_DBL = 3.14159265358979323846;
const float M_FIXED = 1048576.0f;
const float M_UNFIXED = 9.5367431640625e-07f;

struct MLut { /* IrradianceProbeLUT header (probe.cuh:80-104) */
	float center[3];
	float size;
	float resolution;
	int32_t level;
	int32_t counter;
	int32_t pad;
};

struct F4 {
	float x, y, z, w;
};
inline F4 f4(const f3 &v, float w) { return F4{v.x, v.y, v.z, w}; }
inline f3 f3of(const F4 &v) { return mk(v.x, v.y, v.z); }

struct MRes4 {
	std::vector<F4> r0, r1, r2, r3;
	void resize(size_t n) { r0.assign(n, F4{0, 0, 0, 0}); r1 = r0; r2 = r0; r3 = r0; }
};

/* LightInfo (mamba_shader.cuh:19-25) */
struct MLight {
	f3 position, normal, emission;
	bool sky;
};

inline MLight m_no_light() { return MLight{mk(0.0f), mk(0.0f), mk(0.0f), false}; }

/* Reservoir<LightInfo> (editor/optix/common.cuh:53-104) */
struct MRes {
	MLight data;
	float w, W;
	int M;
	f3 seed;
	void update(const MLight &sample, float weight)
	{
		w += weight;
		float eta = rand_uniform(seed);
		if ((eta * w) < weight)
			data = sample;
		M++;
	}
	void resample(float target)
	{
		float d = target * (float)M;
		W = (d > 0.0f) ? w / d : 0.0f;
	}
	void reset()
	{
		w = 0.0f;
		M = 0;
		W = 0.0f;
	}
};

inline MRes m_fresh(const f3 &seed) { return MRes{m_no_light(), 0.0f, 0.0f, 0, seed}; }

inline int32_t bits_of(float f) { return (int32_t)f2u(f); }
inline float float_of(int32_t i) { return u2f((uint32_t)i); }

inline MRes m_load(const MRes4 &R, size_t i)
{
	const F4 &a = R.r0[i], &b = R.r1[i], &c = R.r2[i], &d = R.r3[i];
	MRes r;
	r.data.position = mk(a.x, a.y, a.z);
	r.data.normal = mk(b.x, b.y, b.z);
	r.data.sky = b.w != 0.0f;
	r.data.emission = mk(c.x, c.y, c.z);
	r.M = bits_of(c.w);
	r.w = d.x;
	r.W = d.y;
	r.seed = mk(d.z, d.w, a.w);
	return r;
}

inline void m_store(MRes4 &R, size_t i, const MRes &r)
{
	R.r0[i] = F4{r.data.position.x, r.data.position.y, r.data.position.z, r.seed.z};
	R.r1[i] = F4{r.data.normal.x, r.data.normal.y, r.data.normal.z, r.data.sky ? 1.0f : 0.0f};
	R.r2[i] = F4{r.data.emission.x, r.data.emission.y, r.data.emission.z, float_of(r.M)};
	R.r3[i] = F4{r.w, r.W, r.seed.x, r.seed.y};
}

/* ONB (brdf.cuh:77-105) */
struct MOnb {
	f3 u, v, w;
	f3 local(const f3 &a) const { return a.x * u + a.y * v + a.z * w; }
	f3 inv_local(const f3 &a) const { return mk(dot(a, u), dot(a, v), dot(a, w)); }
};

MOnb m_onb(const f3 &n)
{
	MOnb o;
	o.w = normalize(n);
	f3 a = ((double)fabsf(o.w.x) > 0.9) ? mk(0.0f, 1.0f, 0.0f) : mk(1.0f, 0.0f, 0.0f);
	o.v = normalize(cross(o.w, a));
	o.u = cross(o.w, o.v);
	return o;
}

inline f3 m_cleanse(const f3 &v) { return anynan(v) ? mk(0.0f) : v; }
inline float m_luminance(const f3 &v) { return v.x + v.y + v.z; }

/* brdf / pdf (brdf.cuh:436-457) with sh.mat.type: Glass's lobes are zero */
f3 m_brdf(const SurfaceHit &sh, const f3 &wi)
{
	if (sh.mat.type & KGR_SHADING_TRANSMISSION)
		return sh.mat.diffuse / PI_F + mk(0.0f);
	return brdf(sh, wi);
}

float m_pdf(const SurfaceHit &sh, const f3 &wi)
{
	if (sh.mat.type & KGR_SHADING_TRANSMISSION)
		return 0.0f;
	return ggx_pdf(sh.mat, sh.n, wi, sh.wo);
}

/* to_disk / to_index (probe.cuh:36-54); a NaN direction is bin 0 */
void m_to_disk(const f3 &v, float &su, float &sv)
{
	float theta = katan2(v.y, v.x);
	if (theta < 0.0f)
		theta = (float)((double)theta + 2.0 * M_PI_DBL);
	float rp = ksqrt(v.x * v.x + v.y * v.y);
	su = (float)((double)theta / (2.0 * M_PI_DBL));
	sv = rp;
}

int32_t m_bin(const f3 &v)
{
	if (kisnan(v.x) || kisnan(v.y))
		return 0;
	float su, sv;
	m_to_disk(v, su, sv);
	int32_t x = (int32_t)(su * (float)M_SIZE);
	int32_t y = (int32_t)(sv * (float)M_SIZE);
	int32_t i = y * M_SIZE + x;
	return i < 0 ? 0 : (i > M_BINS - 1 ? M_BINS - 1 : i);
}

/* from_index + from_uv (probe.cuh:56-73) of every bin */
void m_bin_dirs(f3 out[M_BINS])
{
	for (int index = 0; index < M_BINS; index++) {
		int x = index % M_SIZE, y = index / M_SIZE;
		float u = (float)x / (float)M_SIZE, v = (float)y / (float)M_SIZE;
		u = u < 0.0f ? 0.0f : (u > 1.0f ? 1.0f : u);
		v = v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v);
		double theta = (double)(2.0f * u) * M_PI_DBL;
		float dx = (float)((double)v * cos(theta));
		float dy = (float)((double)v * sin(theta));
		float dz = sqrtf(1.0f - dx * dx - dy * dy);
		out[index] = mk(dx, dy, dz);
	}
}

struct MambaState {
	uint32_t width, height, npix, sec_w, sec_h, nsec;
	int32_t max_probes, max_luts;
	std::vector<F4> g_position, g_normal;
	std::vector<int32_t> g_index;
	MRes4 res[2], prev[2];
	std::vector<F4> direct_le;
	std::vector<F4> s_wi, s_le, s_ld, s_ld_wi, s_hit_x, s_hit_n, s_hit_wo;
	std::vector<int32_t> s_hit_mat;
	std::vector<float> sobel, raster;
	std::vector<F4> raster_indicator, raster_radiance;
	std::vector<int32_t> probe_ids;
	std::vector<int32_t> group_probes; /* 4 per group */
	std::vector<int32_t> group_sizes;
	/* table */
	std::vector<MLut> luts;
	std::vector<int32_t> refs;
	std::vector<uint32_t> hashes;
	std::vector<F4> lut_positions;
	std::vector<F4> probe_pos, probe_nrm;
	std::vector<uint64_t> bin_le, bin_depth;
	std::vector<uint32_t> bin_n;
	int32_t counters[2];
	int res_in = 0, prev_in = 0;
	uint64_t stamp = 0;
};

void m_clear_table(MambaState &m)
{
	size_t slots = (size_t)m.max_luts * M_REFS, bins = (size_t)m.max_probes * M_BINS;
	m.luts.assign((size_t)m.max_luts, MLut{{0, 0, 0}, 0, 0, 0, 0, 0});
	m.refs.assign(slots, -1);
	m.hashes.assign(slots, 0xFFFFFFFFu);
	m.lut_positions.assign(slots, F4{0, 0, 0, 0});
	m.probe_pos.assign((size_t)m.max_probes, F4{0, 0, 0, 0});
	m.probe_nrm = m.probe_pos;
	m.bin_le.assign(3 * bins, 0);
	m.bin_n.assign(bins, 0);
	m.bin_depth.assign(bins, 0);
	/* IrradianceProbeLUT::alloc of the top table (probe.cuh:106-118) */
	MLut &top = m.luts[0];
	top.level = 2;
	top.size = 250.0f;
	top.resolution = 250.0f / 25.0f;
	m.counters[0] = 0;
	m.counters[1] = 1;
}

struct MambaFrame {
	const oracle_scene *s;
	const oracle_mamba_params *p;
	MambaState *m;
	std::vector<TriLight> lights;
	f3 bin_dir[M_BINS];
	f3 origin, U, V, W;
	float prev_pv[16];
	uint64_t shadow_rays = 0, closest_rays = 0;

	bool has_env() const { return s->env != nullptr; }

	/* sky_at (editor/optix/common.cuh:18-31) */
	void sky_at(const f3 &d, float out[4]) const
	{
		if (!has_env()) {
			out[0] = out[1] = out[2] = out[3] = 0.0f;
			return;
		}
		float theta = kacos(d.y);
		float phi = katan2(d.z, d.x);
		float u = phi / (2.0f * M_PI_F);
		float v = theta / M_PI_F;
		env_fetch4(s, u, 1.0f - v, out);
	}

	/* load_surface_hit (mamba_shader.cu:166-219) */
	bool surface(size_t pix, SurfaceHit &sh) const
	{
		int32_t idx = m->g_index[pix];
		if (idx == -1)
			return false;
		f3 position = f3of(m->g_position[pix]);
		f3 normal = f3of(m->g_normal[pix]);
		f3 ray = position - origin;
		if (dot(ray, normal) > 0.0f)
			normal = -normal;
		sh.x = position;
		sh.wo = normalize(origin - position);
		sh.n = normalize(normal);
		sh.entering = true;
		sh.mat = load_material(s->materials[idx]);
		float sign = (sh.mat.type == KGR_SHADING_TRANSMISSION) ? -1.0f : 1.0f;
		sh.x = sh.x + sign * sh.n * 1e-3f;
		return true;
	}

	/* sample_light (mamba_shader.cu:101-164); an area light is one emissive
	 * triangle with vertices a, a + ab, a + ac */
	float sample_light(MLight &li, f3 &seed) const
	{
		unsigned int nl = (unsigned int)lights.size();
		unsigned int total = nl + (has_env() ? 1u : 0u);
		if (total == 0)
			return -1.0f;
		unsigned int light_index = (unsigned int)(rand_uniform(seed) * total);
		float area;
		if (light_index < nl) {
			(void)rand_uniform(seed);
			const TriLight &l = lights[light_index];
			f3 v0 = l.a, v1 = l.a + l.ab, v2 = l.a + l.ac;
			f3 c = cross(v1 - v0, v2 - v0);
			f3 gnormal = normalize(c);
			f3 bary = pcg3f(seed);
			float u = bary.x, v = bary.y;
			if (u + v > 1.0f) {
				u = 1.0f - u;
				v = 1.0f - v;
			}
			li.sky = false;
			li.position = v0 * (1.0f - u - v) + v1 * u + v2 * v;
			li.normal = gnormal;
			li.emission = l.intensity;
			area = length(c) * 0.5f;
		} else {
			float theta = (2.0f * M_PI_F) * rand_uniform(seed);
			float phi = M_PI_F * rand_uniform(seed);
			f3 dir = mk(ksin(phi) * kcos(theta), kcos(phi), ksin(phi) * ksin(theta));
			float e[4];
			sky_at(dir, e);
			li.sky = true;
			li.position = 1000.0f * dir;
			li.normal = mk(0.0f);
			li.emission = mk(e[0], e[1], e[2]);
			area = 4.0f * M_PI_F;
		}
		return 1.0f / (area * (float)total);
	}

	/* direct_unoccluded (mamba_shader.cu:74-87) */
	f3 direct_unoccluded(const SurfaceHit &sh, const MLight &li) const
	{
		f3 wi = normalize(li.position - sh.x);
		float R = length(li.position - sh.x);
		f3 rho = m_cleanse(m_brdf(sh, wi));
		float ldotn = li.sky ? 1.0f : fabsf(dot(li.normal, wi));
		float ndotwi = fabsf(dot(sh.n, wi));
		float falloff = li.sky ? 1.0f : 1.0f / (R * R);
		return rho * li.emission * ldotn * ndotwi * falloff;
	}

	bool blocked(const f3 &o, const f3 &d, float tmax, uint64_t &rays) const
	{
		uint64_t a = 0, b = 0;
		rays++;
		return trace_any(s, o, d, tmax, &a, &b);
	}

	/* occluded (mamba_shader.cu:38-64) */
	bool occluded(const f3 &origin_, const f3 &target, uint64_t &rays) const
	{
		f3 dir = normalize(target - origin_);
		return blocked(origin_, dir, length(target - origin_) - 1e-3f, rays);
	}

	float target(const SurfaceHit &sh, const MLight &li) const { return m_luminance(direct_unoccluded(sh, li)); }

	float occluded_target(const SurfaceHit &sh, const MLight &li, uint64_t &rays) const
	{
		f3 Li = direct_unoccluded(sh, li);
		return m_luminance(Li * (1.0f - (float)occluded(sh.x, li.position, rays)));
	}

	void accumulate_direct(size_t pix, const SurfaceHit &sh, const f3 &Ld, bool occl, float Wt) const
	{
		f3 new_direct = m_cleanse(Ld * (1.0f - (float)occl) * Wt);
		f3 le = f3of(m->direct_le[pix]);
		le = (le * (float)p->samples + sh.mat.emission + new_direct) / (float)(p->samples + 1);
		m->direct_le[pix] = f4(le, 0.0f);
	}

	/* reproject (mamba_shader.cu:289-321) */
	int reproject(int index, const f3 &x) const
	{
		if (p->samples > 0)
			return index;
		float q[4];
		for (int i = 0; i < 4; i++)
			q[i] = prev_pv[0 * 4 + i] * x.x + prev_pv[1 * 4 + i] * x.y + prev_pv[2 * 4 + i] * x.z
				+ prev_pv[3 * 4 + i] * 1.0f;
		float u = q[0] / q[3];
		float v = q[1] / q[3];
		if (!((u >= -1.0f && u <= 1.0f) && (v >= -1.0f && v <= 1.0f)))
			return -1;
		u = (u + 1.0f) * 0.5f;
		v = (v + 1.0f) * 0.5f;
		int ix = (int)((double)(u * (float)m->width) + 0.5);
		int iy = (int)((double)(v * (float)m->height) + 0.5);
		if (ix < 0 || iy < 0 || ix >= (int)m->width || iy >= (int)m->height)
			return -1;
		return iy * (int)m->width + ix;
	}

	/* sample_spatial_neighborhood (mamba_shader.cu:395-417) */
	int spatial_neighbor(int index, f3 &seed) const
	{
		int width = (int)m->width, height = (int)m->height;
		int x = index % width, y = index / width;
		f3 offset = rand_uniform_3f(seed);
		float theta = (float)(2.0 * M_PI_DBL * (double)offset.x);
		float r = 20.0f * ksqrt(offset.y);
		int x0 = (int)((float)x + r * kcos(theta));
		int y0 = (int)((float)y + r * ksin(theta));
		x0 = x0 < 0 ? 0 : (x0 > width - 1 ? width - 1 : x0);
		y0 = y0 < 0 ? 0 : (y0 > height - 1 ? height - 1 : y0);
		return x0 + y0 * width;
	}

	/* ---- probe tables (probe.cuh) ---- */

	static bool contains(const MLut &L, const f3 &x, bool neighbor)
	{
		float e = L.size / 2.0f + (neighbor ? 1.0f : 0.0f) * L.resolution;
		f3 c = mk(L.center[0], L.center[1], L.center[2]);
		f3 mn = c - mk(e), mx = c + mk(e);
		return (x.x >= mn.x && x.y >= mn.y && x.z >= mn.z) && (x.x <= mx.x && x.y <= mx.y && x.z <= mx.z);
	}

	/* hash (probe.cuh:168-187); the first shuffle shifts a signed value */
	static uint32_t hash(const MLut &L, const f3 &x, int dx, int dy, int dz)
	{
		float cdx = x.x - L.center[0] + L.size / 2.0f;
		float cdy = x.y - L.center[1] + L.size / 2.0f;
		float cdz = x.z - L.center[2] + L.size / 2.0f;
		int32_t ix = (int32_t)((cdx / L.resolution) + (float)dx);
		int32_t iy = (int32_t)((cdy / L.resolution) + (float)dy);
		int32_t iz = (int32_t)((cdz / L.resolution) + (float)dz);
		uint32_t u = (uint32_t)(ix & 0x7FF) | ((uint32_t)(iy & 0x7FF) << 11) | ((uint32_t)(iz & 0x7FF) << 22);
		int32_t h = (int32_t)u;
		h ^= (h >> 11) ^ (h >> 22);
		u = (uint32_t)h;
		u ^= (u << 7) & 0x9D2C5680u;
		u ^= (u << 15) & 0xEFC60000u;
		return u;
	}

	static uint32_t neighbor_hash(const MLut &L, const f3 &x, int ni)
	{
		return hash(L, x, ni % 3 - 1, (ni / 3) % 3 - 1, ni / 9 - 1);
	}

	/* lookup (probe.cuh:256-285) */
	int32_t lookup(int32_t l, const f3 &x, int ni) const
	{
		const MLut &L = m->luts[l];
		if (!contains(L, x, ni != -1))
			return -1;
		uint32_t h = ni == -1 ? hash(L, x, 0, 0, 0) : neighbor_hash(L, x, ni);
		size_t base = (size_t)l * M_REFS;
		int32_t index = -1;
		float closest = FLT_MAX;
		for (int i = 0; i < 2; i++) {
			int32_t j = (int32_t)((h + (uint32_t)(i * i)) % (uint32_t)M_REFS);
			if (m->refs[base + j] == -1)
				break;
			if (m->hashes[base + j] == h) {
				float dist = length(f3of(m->lut_positions[base + j]) - x);
				if (dist < closest) {
					closest = dist;
					index = j;
				}
			}
		}
		return index;
	}

	/* full_lookup (probe.cuh:287-301) */
	int32_t full_lookup(int32_t l, const f3 &x) const
	{
		int32_t r = lookup(l, x, -1);
		for (int ni = 0; r == -1 && ni < 27; ni++)
			r = lookup(l, x, ni);
		return r;
	}

	/* lookup_L2 (probe.cuh:678-712) */
	int32_t top_lookup(const f3 &x) const
	{
		const MLut &L = m->luts[0];
		if (!contains(L, x, false))
			return -1;
		uint32_t h = hash(L, x, 0, 0, 0);
		f3 half = mk(0.5f * L.resolution);
		for (int i = 0; i < M_REFS; i++) {
			uint32_t j = (h + (uint32_t)i) % (uint32_t)M_REFS;
			if (m->refs[j] == -1)
				return -1;
			f3 c = f3of(m->lut_positions[j]);
			f3 mn = c - half, mx = c + half;
			if ((x.x <= mx.x && x.y <= mx.y && x.z <= mx.z) && (x.x >= mn.x && x.y >= mn.y && x.z >= mn.z))
				return (int32_t)j;
		}
		return -1;
	}

	/* lookup_L2 and the guard against an index at or above the probe
	 * counter (mamba.cu:278, 456, 490, 550, 793) */
	int32_t table_of(const f3 &x, int32_t probe_counter) const
	{
		int32_t r = top_lookup(x);
		if (r == -1)
			return -1;
		int32_t l = m->refs[r];
		if (l < 0 || l >= probe_counter)
			return -1;
		return l;
	}

	/* closest<2> (probe.cuh:305-363) */
	void closest2(int32_t l, const f3 &x, int32_t idx[2], float dist[2]) const
	{
		const MLut &L = m->luts[l];
		if (!contains(L, x, true))
			return;
		size_t base = (size_t)l * M_REFS;
		for (int ni = -1; ni < 27; ni++) {
			uint32_t h = ni == -1 ? hash(L, x, 0, 0, 0) : neighbor_hash(L, x, ni);
			for (int i = 0; i < 2; i++) {
				int32_t j = (int32_t)((h + (uint32_t)(i * i)) % (uint32_t)M_REFS);
				if (m->refs[base + j] == -1)
					break;
				float d = length(f3of(m->lut_positions[base + j]) - x);
				for (int k = 0; k < 2; k++) {
					if (d < dist[k]) {
						for (int q = 1; q > k; q--) {
							dist[q] = dist[q - 1];
							idx[q] = idx[q - 1];
						}
						dist[k] = d;
						idx[k] = j;
						break;
					}
				}
			}
		}
	}

	f3 bin_radiance(size_t b) const
	{
		return mk((float)(int64_t)m->bin_le[3 * b + 0] * M_UNFIXED, (float)(int64_t)m->bin_le[3 * b + 1] * M_UNFIXED,
			(float)(int64_t)m->bin_le[3 * b + 2] * M_UNFIXED);
	}

	float bin_depth(size_t b) const { return u2f((uint32_t)(m->bin_depth[b] & 0xFFFFFFFFull)); }

	/* ---- passes ---- */

	void gbuffer()
	{
		const uint32_t width = m->width, height = m->height;
		uint64_t rays = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : rays) num_threads(nthreads(p->threads))
		for (long i = 0; i < (long)m->npix; i++) {
			uint32_t x = (uint32_t)i % width, y = (uint32_t)i / width;
			uint32_t yy = height - (y + 1);
			float u = 2.0f * ((float)x + 0.5f) / (float)width - 1.0f;
			float v = 2.0f * ((float)yy + 0.5f) / (float)height - 1.0f;
			f3 d = normalize(u * U - v * V + W);
			uint64_t a = 0, b = 0;
			kgr_hit h = trace_closest(s, origin, d, 1e16f, &a, &b);
			rays++;
			if (h.prim < 0) {
				m->g_position[i] = F4{0, 0, 0, 0};
				m->g_normal[i] = F4{0, 0, 0, 0};
				m->g_index[i] = -1;
				continue;
			}
			const uint32_t *t = s->tris + 4 * (size_t)h.prim;
			f3 pa = ld3(s->positions, t[0]), pb = ld3(s->positions, t[1]), pc = ld3(s->positions, t[2]);
			f3 na = ld3(s->normals, t[0]), nb = ld3(s->normals, t[1]), nc = ld3(s->normals, t[2]);
			float w0 = 1.0f - h.b1 - h.b2;
			f3 xx = w0 * pa + h.b1 * pb + h.b2 * pc;
			f3 n = normalize(w0 * na + h.b1 * nb + h.b2 * nc);
			m->g_position[i] = f4(xx, 1.0f);
			m->g_normal[i] = f4(n, 1.0f);
			m->g_index[i] = (int32_t)t[3];
		}
		closest_rays += rays;
	}

	/* __raygen__direct_primary (mamba_shader.cu:221-272) */
	void direct_primary()
	{
		MRes4 &R = m->res[m->res_in];
		uint64_t rays = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : rays) num_threads(nthreads(p->threads))
		for (long i = 0; i < (long)m->npix; i++) {
			uint32_t x = (uint32_t)i % m->width, y = (uint32_t)i / m->width;
			MRes r = m_load(R, i);
			r.reset();
			SurfaceHit sh;
			if (!surface(i, sh)) {
				m_store(R, i, r);
				continue;
			}
			f3 seed = mk((float)x, (float)y, p->time);
			for (int k = 0; k < 8; k++) {
				MLight lighting = m_no_light();
				float pdf = sample_light(lighting, seed);
				f3 Ld = direct_unoccluded(sh, lighting);
				float t = Ld.x + Ld.y + Ld.z;
				r.update(lighting, t / pdf > 0.0f ? t / pdf : 0.0f);
			}
			f3 Ld_res = direct_unoccluded(sh, r.data);
			bool occl = occluded(sh.x, r.data.position, rays);
			r.resample(m_luminance(Ld_res * (1.0f - (float)occl)));
			m_store(R, i, r);
			if (!p->temporal_reuse && !p->spatial_reuse)
				accumulate_direct(i, sh, Ld_res, occl, r.W);
		}
		shadow_rays += rays;
	}

	/* __raygen__temporal_reuse (mamba_shader.cu:323-393) */
	void direct_temporal()
	{
		MRes4 &R = m->res[m->res_in];
		const MRes4 &Pin = m->prev[m->prev_in];
		MRes4 &Pout = m->prev[1 - m->prev_in];
		bool end = !p->spatial_reuse;
		uint64_t rays = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : rays) num_threads(nthreads(p->threads))
		for (long i = 0; i < (long)m->npix; i++) {
			uint32_t x = (uint32_t)i % m->width, y = (uint32_t)i / m->width;
			SurfaceHit sh;
			if (!surface(i, sh)) {
				MRes q = m_load(Pin, i);
				q.reset();
				m_store(Pout, i, q);
				continue;
			}
			int pindex = reproject((int)i, sh.x);
			MRes cur = m_load(R, i);
			if (cur.M <= 0) {
				m_store(Pout, i, m_load(Pin, i));
				continue;
			}
			MRes merged = m_fresh(2.0f * mk((float)x, (float)y, p->time));
			float t_current = occluded_target(sh, cur.data, rays);
			merged.update(cur.data, t_current * cur.W * (float)cur.M);
			int N = cur.M;
			if (pindex >= 0) {
				MRes prev = m_load(Pin, (size_t)pindex);
				if (prev.M > 0) {
					prev.M = std::min(prev.M, 200);
					float t_previous = occluded_target(sh, prev.data, rays);
					merged.update(prev.data, t_previous * prev.W * (float)prev.M);
					N += (t_previous > 0.0f) * prev.M;
				}
			}
			merged.M = N;
			merged.resample(target(sh, merged.data));
			m_store(R, i, merged);
			if (end) {
				f3 Ld_res = direct_unoccluded(sh, merged.data);
				bool occl = occluded(sh.x, merged.data.position, rays);
				accumulate_direct(i, sh, Ld_res, occl, merged.W);
				m_store(Pout, i, merged);
			} else {
				m_store(Pout, i, m_load(Pin, i));
			}
		}
		shadow_rays += rays;
	}

	/* __raygen__spatial_reuse (mamba_shader.cu:419-510) */
	void direct_spatial()
	{
		const MRes4 &Rin = m->res[m->res_in];
		MRes4 &Rout = m->res[1 - m->res_in];
		const MRes4 &Pin = m->prev[m->prev_in];
		MRes4 &Pout = m->prev[1 - m->prev_in];
		uint64_t rays = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : rays) num_threads(nthreads(p->threads))
		for (long i = 0; i < (long)m->npix; i++) {
			uint32_t x = (uint32_t)i % m->width, y = (uint32_t)i / m->width;
			MRes cur = m_load(Rin, i);
			SurfaceHit sh;
			if (!surface(i, sh)) {
				m_store(Rout, i, cur);
				MRes q = m_load(Pin, i);
				q.reset();
				m_store(Pout, i, q);
				continue;
			}
			if (cur.M <= 0) {
				m->direct_le[i] = F4{0.0f, 0.0f, 1.0f, 0.0f};
				m_store(Rout, i, cur);
				MRes q = m_load(Pin, i);
				q.reset();
				m_store(Pout, i, q);
				continue;
			}
			MRes merged = m_fresh(2.0f * mk((float)x, (float)y, p->time));
			float t_current = target(sh, cur.data);
			merged.update(cur.data, t_current * cur.W * (float)cur.M);
			SurfaceHit hits[2];
			int sizes[2];
			bool valid[2];
			int count = 0;
			for (int k = 0; k < 2; k++) {
				int index0 = spatial_neighbor((int)i, merged.seed);
				MRes nb = m_load(Rin, (size_t)index0);
				nb.M = std::min(nb.M, 200);
				if (nb.M > 0) {
					float t_neighbor = occluded_target(sh, nb.data, rays);
					merged.update(nb.data, t_neighbor * nb.W * (float)nb.M);
				}
				hits[k].mat = sh.mat;
				hits[k].x = hits[k].n = mk(0.0f);
				surface((size_t)index0, hits[k]);
				hits[k].wo = sh.wo;
				valid[k] = nb.M > 0;
				sizes[k] = nb.M;
				count += nb.M;
			}
			merged.M = cur.M + count;
			int Z = cur.M;
			for (int k = 0; k < 2; k++) {
				float t_neighbor = valid[k] ? occluded_target(hits[k], merged.data, rays) : 0.0f;
				if (t_neighbor > 0.0f)
					Z += sizes[k];
			}
			float t_merged = target(sh, merged.data);
			float denominator = t_merged * (float)Z;
			merged.W = (denominator > 0.0f) ? merged.w / denominator : 0.0f;
			m_store(Rout, i, merged);
			f3 Ld_res = direct_unoccluded(sh, merged.data);
			bool occl = occluded(sh.x, merged.data.position, rays);
			accumulate_direct(i, sh, Ld_res, occl, merged.W);
			m_store(Pout, i, merged);
		}
		shadow_rays += rays;
	}

	/* Ld (mamba_shader.cu:512-561) */
	f3 Ld(const SurfaceHit &sh, f3 &seed, f3 &Le, f3 &wi, float &R, uint64_t &rays) const
	{
		MLight li = m_no_light();
		float light_pdf = sample_light(li, seed);
		if (light_pdf < 0.0f)
			return mk(0.0f);
		f3 direction = normalize(li.position - sh.x);
		f3 o = sh.x;
		bool hit = blocked(o, direction, length(li.position - o) - 1e-3f, rays);
		f3 out = sh.mat.emission;
		if (!hit && length(out) < 1e-3f) {
			wi = normalize(li.position - o);
			R = length(li.position - o);
			f3 f = m_cleanse(m_brdf(sh, wi));
			float ldotn = li.sky ? 1.0f : fabsf(dot(li.normal, wi));
			float ndotwi = fabsf(dot(sh.n, wi));
			float falloff = li.sky ? 1.0f : (R * R) + 1e-3f;
			out = f * li.emission * ldotn * ndotwi / (light_pdf * falloff);
			Le = li.emission;
		}
		return out;
	}

	/* __raygen__secondary (mamba_shader.cu:563-680) with the closest-hit
	 * program (:707-777) */
	void secondary()
	{
		uint64_t rays = 0, crays = 0;
		const int32_t cycle = p->samples % 16;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : rays, crays) num_threads(nthreads(p->threads))
		for (long li = 0; li < (long)m->nsec; li++) {
			uint32_t sx = (uint32_t)li % m->sec_w, sy = (uint32_t)li / m->sec_w;
			int32_t x = 4 * (int32_t)sx + (cycle % 4), y = 4 * (int32_t)sy + (cycle / 4);
			if (x >= (int32_t)m->width || y >= (int32_t)m->height)
				continue;
			size_t pix = (size_t)y * m->width + (size_t)x;
			SurfaceHit sh;
			if (!surface(pix, sh)) {
				m->s_wi[li] = F4{0, 0, 0, 0};
				continue;
			}
			f3 wi;
			float pdf;
			f3 seed = mk((float)sx, (float)sy, p->time);
			(void)eval(sh, wi, pdf, seed);
			if (pdf <= 0.0f) {
				m->s_wi[li] = m->s_hit_x[li] = m->s_hit_n[li] = m->s_hit_wo[li] = F4{0, 0, 0, 0};
				continue;
			}
			uint64_t a = 0, b = 0;
			kgr_hit h = trace_closest(s, sh.x, wi, 1e16f, &a, &b);
			crays++;
			if (h.prim < 0) {
				float e[4];
				sky_at(wi, e);
				m->s_le[li] = f4(mk(e[0], e[1], e[2]) / pdf, 0.0f);
				m->s_wi[li] = f4(wi, 0.0f);
				m->s_hit_x[li] = f4(1000.0f * wi, 0.0f);
				m->s_hit_n[li] = m->s_hit_wo[li] = F4{0, 0, 0, 0};
				continue;
			}
			const uint32_t *t = s->tris + 4 * (size_t)h.prim;
			f3 pa = ld3(s->positions, t[0]), pb = ld3(s->positions, t[1]), pc = ld3(s->positions, t[2]);
			f3 na = ld3(s->normals, t[0]), nb = ld3(s->normals, t[1]), nc = ld3(s->normals, t[2]);
			float bu = h.b1, bv = h.b2;
			float bw = 1.0f - bu - bv;
			f3 hx = bw * pa + bu * pb + bv * pc;
			f3 ng = normalize(cross(pb - pa, pc - pa));
			if (dot(wi, ng) > 0.0f)
				ng = -ng;
			f3 ns = bw * na + bu * nb + bv * nc;
			if (dot(ng, ns) < 0.0f)
				ns = -ns;
			f3 hn = normalize(ns);
			f3 Le = mk(0.0f), Le_wi = mk(0.0f);
			float Le_depth = 0.0f;
			f3 indirect = Ld(sh, seed, Le, Le_wi, Le_depth, rays);
			m->s_wi[li] = f4(wi, 0.0f);
			m->s_ld[li] = f4(Le, 0.0f);
			m->s_ld_wi[li] = f4(Le_wi, Le_depth);
			m->s_le[li] = f4(indirect, 0.0f);
			m->s_hit_x[li] = f4(hx, 0.0f);
			m->s_hit_n[li] = f4(hn, 0.0f);
			m->s_hit_wo[li] = f4(-wi, 0.0f);
			m->s_hit_mat[li] = (int32_t)t[3];
		}
		shadow_rays += rays;
		closest_rays += crays;
	}

	/* secondary_gather (mamba.cu:401-576): the splats against the table as
	 * it stood before the frame's splats, then added in splat order */
	void gather()
	{
		const int32_t cycle = p->samples % 16;
		const int32_t probe_counter = m->counters[0];
		std::vector<int32_t> rec_bin(2 * (size_t)m->nsec, -1);
		std::vector<F4> rec_val(2 * (size_t)m->nsec, F4{0, 0, 0, 0});
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads(p->threads))
		for (long index = 0; index < (long)m->nsec; index++) {
			uint32_t sx = (uint32_t)index % m->sec_w, sy = (uint32_t)index / m->sec_w;
			int32_t tx = 4 * (int32_t)sx + (cycle % 4), ty = 4 * (int32_t)sy + (cycle / 4);
			if (tx >= (int32_t)m->width || ty >= (int32_t)m->height)
				continue;
			f3 hx = f3of(m->s_hit_x[index]), hn = f3of(m->s_hit_n[index]), hwo = f3of(m->s_hit_wo[index]);
			int32_t hmat = m->s_hit_mat[index];
			f3 wi = f3of(m->s_wi[index]);
			f3 Le = f3of(m->s_le[index]);
			F4 ldw = m->s_ld_wi[index];
			f3 Ld_wi = mk(ldw.x, ldw.y, ldw.z);
			float Ld_depth = ldw.w;
			f3 Ldv = f3of(m->s_ld[index]);
			size_t pix = (size_t)ty * m->width + (size_t)tx;
			if (m->g_index[pix] == -1) {
				m->s_le[index] = F4{0, 0, 0, 0};
				continue;
			}
			f3 position = f3of(m->g_position[pix]);
			f3 normal = f3of(m->g_normal[pix]);
			int32_t l = table_of(position, probe_counter);
			if (l != -1) {
				int32_t r2 = full_lookup(l, position);
				if (r2 == -1) {
					m->s_le[index] = F4{0, 0, 0, 0};
				} else {
					MOnb onb = m_onb(normal);
					f3 local_wi = normalize(onb.inv_local(wi));
					int32_t probe = m->refs[(size_t)l * M_REFS + r2];
					int32_t bin = m_bin(local_wi);
					if (!(length(hn) < 1e-6f)) {
						int32_t l2 = table_of(hx, probe_counter);
						int32_t r4 = l2 == -1 ? -1 : full_lookup(l2, hx);
						if (r4 != -1) {
							int32_t p2 = m->refs[(size_t)l2 * M_REFS + r4];
							f3 ppos = f3of(m->probe_pos[p2]);
							MOnb o2 = m_onb(f3of(m->probe_nrm[p2]));
							SurfaceHit sec;
							sec.mat = load_material(s->materials[hmat]);
							sec.entering = true;
							sec.n = hn;
							sec.wo = hwo;
							sec.x = hx;
							f3 sum = mk(0.0f);
							for (int j = 0; j < M_BINS; j++) {
								f3 probe_wo = o2.local(bin_dir[j]);
								size_t b = (size_t)p2 * M_BINS + j;
								float d = bin_depth(b);
								f3 wo = normalize((d * probe_wo + ppos) - hx);
								if (dot(wo, hn) <= 0.0f)
									continue;
								float geometric = kmax(dot(wo, hn), 0.0f);
								f3 f = m_cleanse(m_brdf(sec, wo));
								f3 le = m_cleanse(bin_radiance(b));
								float n = (float)m->bin_n[b];
								sum = sum + (sec.mat.emission + (n > 0.0f ? (le / n) * f * geometric : mk(0.0f)));
							}
							Le = Le + sum / (float)M_BINS;
						}
					}
					rec_bin[2 * index] = probe * M_BINS + bin;
					rec_val[2 * index] = f4(Le, length(position - hx));
				}
			}
			if (length(hn) > 1e-6f) {
				int32_t lb = table_of(hx, probe_counter);
				if (lb == -1)
					continue;
				int32_t r2 = full_lookup(lb, hx);
				if (r2 == -1)
					continue;
				MOnb onb = m_onb(hn);
				f3 local_wi = normalize(onb.inv_local(Ld_wi));
				int32_t probe = m->refs[(size_t)lb * M_REFS + r2];
				rec_bin[2 * index + 1] = probe * M_BINS + m_bin(local_wi);
				rec_val[2 * index + 1] = f4(Ldv, Ld_depth);
			}
		}
		for (size_t r = 0; r < rec_bin.size(); r++) {
			int32_t bin = rec_bin[r];
			if (bin < 0)
				continue;
			const F4 &v = rec_val[r];
			float c[3] = {v.x, v.y, v.z};
			for (int k = 0; k < 3; k++)
				m->bin_le[3 * (size_t)bin + k] += (uint64_t)to_fixed(c[k]);
			m->bin_n[bin] += 1;
			m->bin_depth[bin] = ((uint64_t)(uint32_t)(m->stamp + r + 1) << 32) | f2u(v.w);
		}
	}

	static int64_t to_fixed(float v)
	{
		float sc = v * M_FIXED;
		if (kisnan(sc))
			return 0;
		if (sc >= 4611686018427387904.0f)
			return 4611686018427387904ll;
		if (sc <= -4611686018427387904.0f)
			return -4611686018427387904ll;
		return (int64_t)nearbyintf(sc);
	}

	/* sobel_normal (mamba.cu:169-201) */
	void sobel()
	{
		int W = (int)m->width, H = (int)m->height;
#pragma omp parallel for schedule(static) num_threads(nthreads(p->threads))
		for (long i = 0; i < (long)m->npix; i++) {
			int x = (int)(i % W), y = (int)(i / W);
			int ys = H - (y + 1);
			f3 n = f3of(m->g_normal[i]);
			float acc = 0.0f;
			for (int a = -1; a <= 1; a++)
				for (int b = -1; b <= 1; b++) {
					int x2 = x + a, y2s = ys + b;
					if (x2 < 0 || x2 >= W || y2s < 0 || y2s >= H)
						continue;
					int y2 = H - (y2s + 1);
					acc += length(n - f3of(m->g_normal[(size_t)y2 * W + x2]));
				}
			m->sobel[i] = acc;
		}
	}

	/* raster_probes (mamba.cu:244-369) */
	void raster()
	{
		static const float wheel[12][3] = {{0.910f, 0.490f, 0.490f}, {0.910f, 0.700f, 0.490f},
			{0.910f, 0.910f, 0.490f}, {0.700f, 0.910f, 0.490f}, {0.490f, 0.910f, 0.490f},
			{0.490f, 0.910f, 0.700f}, {0.490f, 0.910f, 0.910f}, {0.490f, 0.700f, 0.910f},
			{0.490f, 0.490f, 0.910f}, {0.700f, 0.490f, 0.910f}, {0.910f, 0.490f, 0.910f},
			{0.910f, 0.490f, 0.700f}};
		const int32_t probe_counter = m->counters[0];
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads(p->threads))
		for (long i = 0; i < (long)m->npix; i++) {
			f3 position = f3of(m->g_position[i]);
			int32_t l = table_of(position, probe_counter);
			if (l == -1)
				continue;
			const MLut &L = m->luts[l];
			size_t base = (size_t)l * M_REFS;
			float closest = FLT_MAX;
			int32_t closest_index = -1;
			for (int ni = -1; ni < 27; ni++) {
				int32_t r = lookup(l, position, ni);
				if (r == -1)
					continue;
				int32_t q = m->refs[base + r];
				float dist = length(position - f3of(m->probe_pos[q]));
				if (dist < closest) {
					closest = dist;
					closest_index = q;
				}
			}
			float v = 0.0f;
			f3 indicator = mk((float)(l % 2)), radiance = mk((float)(l % 2));
			int32_t probe_index = -1;
			if (closest_index != -1) {
				probe_index = closest_index;
				f3 diff = position - f3of(m->probe_pos[probe_index]);
				MOnb onb = m_onb(f3of(m->probe_nrm[probe_index]));
				f3 local = onb.inv_local(diff) / L.resolution;
				local.z = 0.0f;
				if (length(local) < 1.0f) {
					v = 1.0f;
					if (p->render_probes || p->render_probe_radiance) {
						f3 wi = normalize(mk(local.x, local.y, ksqrt(1.0f - local.x * local.x - local.y * local.y)));
						int32_t idx = m_bin(wi);
						if (p->render_probes) {
							float su, sv;
							m_to_disk(wi, su, sv);
							int32_t ix = (int32_t)(su * (float)M_SIZE), iy = (int32_t)(sv * (float)M_SIZE);
							int32_t mod = (ix + iy) % 2;
							int32_t c = probe_index % 12;
							indicator = mk(wheel[c][0], wheel[c][1], wheel[c][2]) * (0.5f + 0.5f * (float)mod);
						} else {
							size_t b = (size_t)probe_index * M_BINS + idx;
							float n = (float)m->bin_n[b];
							radiance = n > 0.0f ? bin_radiance(b) / n : mk(0.0f);
						}
					}
				}
			}
			m->raster[i] = v;
			m->raster_indicator[i] = f4(indicator, 0.0f);
			m->raster_radiance[i] = f4(radiance, 0.0f);
			m->probe_ids[i] = probe_index;
		}
	}

	/* probe_collapse (mamba.cu:889-938) */
	void collapse()
	{
		uint32_t gw = (m->width + 15) / 16, gh = (m->height + 15) / 16;
		for (uint32_t i = 0; i < gw * gh; i++) {
			uint32_t x16 = i % gw, y16 = i / gw;
			int32_t dst[4] = {-1, -1, -1, -1};
			int32_t size = 0;
			for (uint32_t xo = 0; xo < 16; xo++)
				for (uint32_t yo = 0; yo < 16; yo++) {
					if (size >= 4)
						break;
					uint32_t x = x16 * 16 + xo, y = y16 * 16 + yo;
					if (x >= m->width || y >= m->height)
						continue;
					int32_t id = m->probe_ids[(size_t)y * m->width + x];
					bool dup = false;
					for (int32_t j = 0; j < size; j++)
						if (dst[j] == id)
							dup = true;
					if (!dup)
						dst[size++] = id;
				}
			for (int k = 0; k < 4; k++)
				m->group_probes[4 * (size_t)i + k] = dst[k];
			m->group_sizes[i] = size;
		}
	}

	/* probe_allocation (mamba_kernels.cu:5-182) with request_L2, the
	 * second-level table's allocation and request_L1 (probe.cuh:522-676),
	 * one 16x16 block after another */
	void allocate()
	{
		int W = (int)m->width, H = (int)m->height;
		int bw = W / 16, bh = H / 16;
		for (int b = 0; b < bw * bh; b++) {
			int x = b % bw, y = b / bw;
			int x2 = x * 16, y2 = y * 16;
			int misses = 0, best_distance = 0;
			int x_best = x2 + 8, y_best = y2 + 8;
			for (int i = 0; i < 16; i++)
				for (int j = 0; j < 16; j++) {
					int x3 = x2 + i, y3 = y2 + j;
					if (m->raster[(size_t)y3 * W + x3] != 0.0f)
						continue;
					int distance = 0;
					for (int k = -2; k <= 2; k++)
						for (int l = -2; l <= 2; l++) {
							int x4 = x3 + k, y4 = y3 + l;
							if (x4 < 0 || x4 >= W || y4 < 0 || y4 >= H)
								continue;
							if (m->raster[(size_t)y4 * W + x4] == 0.0f)
								continue;
							distance = std::max(abs(k) + abs(l), distance);
						}
					if (distance > best_distance) {
						best_distance = distance;
						x_best = x3;
						y_best = y3;
					}
					misses++;
				}
			if ((double)misses < 0.4 * 16 * 16)
				continue;
			if (misses == 16 * 16) {
				x_best = x2 + 8;
				y_best = y2 + 8;
			}
			size_t pix = (size_t)y_best * W + x_best;
			if (m->g_index[pix] == -1)
				continue;
			f3 position = f3of(m->g_position[pix]);
			f3 normal = f3of(m->g_normal[pix]);
			MLut &top = m->luts[0];
			if (!contains(top, position, false))
				continue;
			/* request_L2 */
			uint32_t h = hash(top, position, 0, 0, 0);
			int32_t idx = -1;
			f3 half = mk(0.5f * top.resolution);
			for (int i = 0; i < M_REFS; i++) {
				uint32_t j = (h + (uint32_t)i) % (uint32_t)M_REFS;
				if (m->refs[j] == -1) {
					if (m->counters[1] >= m->max_luts)
						break;
					float cdx = position.x - top.center[0] + top.size / 2.0f;
					float cdy = position.y - top.center[1] + top.size / 2.0f;
					float cdz = position.z - top.center[2] + top.size / 2.0f;
					int32_t ix = (int32_t)(cdx / top.resolution);
					int32_t iy = (int32_t)(cdy / top.resolution);
					int32_t iz = (int32_t)(cdz / top.resolution);
					f3 c = mk(top.center[0] + ((float)ix + 0.5f) * top.resolution - top.size / 2.0f,
						top.center[1] + ((float)iy + 0.5f) * top.resolution - top.size / 2.0f,
						top.center[2] + ((float)iz + 0.5f) * top.resolution - top.size / 2.0f);
					m->hashes[j] = h;
					m->lut_positions[j] = f4(c, 0.0f);
					top.counter++;
					int32_t l = m->counters[1]++;
					MLut &nl = m->luts[l];
					nl.center[0] = c.x;
					nl.center[1] = c.y;
					nl.center[2] = c.z;
					nl.size = 10.0f;
					nl.resolution = 10.0f / 25.0f;
					nl.level = 1;
					nl.counter = 0;
					nl.pad = 0;
					m->refs[j] = l;
					idx = (int32_t)j;
					break;
				}
				f3 c = f3of(m->lut_positions[j]);
				f3 mn = c - half, mx = c + half;
				if ((position.x <= mx.x && position.y <= mx.y && position.z <= mx.z)
					&& (position.x >= mn.x && position.y >= mn.y && position.z >= mn.z)) {
					idx = (int32_t)j;
					break;
				}
			}
			if (idx == -1 || m->counters[0] >= m->max_probes)
				continue;
			/* request_L1 and the probe */
			int32_t l = m->refs[idx];
			MLut &L = m->luts[l];
			uint32_t h1 = hash(L, position, 0, 0, 0);
			size_t base = (size_t)l * M_REFS;
			int32_t slot = -1;
			for (int t = 0; t < 2; t++) {
				uint32_t j = (h1 + (uint32_t)(t * t)) % (uint32_t)M_REFS;
				if (m->refs[base + j] == -1) {
					slot = (int32_t)j;
					break;
				}
			}
			if (slot == -1)
				continue;
			m->hashes[base + slot] = h1;
			m->lut_positions[base + slot] = f4(position, 0.0f);
			L.counter++;
			int32_t q = m->counters[0]++;
			m->probe_pos[q] = f4(position, 0.0f);
			m->probe_nrm[q] = f4(normal, 0.0f);
			m->refs[base + slot] = q;
		}
	}

	/* final_gather (mamba.cu:686-878) */
	void final_gather(float *color)
	{
		const uint32_t width = m->width;
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads(p->threads))
		for (long i = 0; i < (long)m->npix; i++) {
			uint32_t x = (uint32_t)i % width, y = (uint32_t)i / width;
			SurfaceHit sh;
			if (!surface(i, sh)) {
				uint32_t yy = m->height - (y + 1);
				float u = 2.0f * (float)x / (float)m->width - 1.0f;
				float v = 2.0f * (float)yy / (float)m->height - 1.0f;
				float e[4];
				sky_at(normalize(u * U - v * V + W), e);
				for (int k = 0; k < 4; k++)
					color[4 * i + k] = e[k];
				continue;
			}
			f3 c = sh.mat.emission + (float)(p->direct_lighting != 0) * f3of(m->direct_le[i]) + mk(0.0f);
			f3 covered = mk(0.0f);
			if (p->render_probes || p->render_probe_radiance)
				covered = f3of(p->render_probes ? m->raster_indicator[i] : m->raster_radiance[i]);
			uint32_t sidx = x / 4 + (y / 4) * m->sec_w;
			f3 sec = mk(0.0f);
			if (sidx < m->nsec && p->indirect_lighting) {
				sec = f3of(m->s_le[sidx]);
			} else if (p->irradiance) {
				int32_t l = table_of(sh.x, m->counters[0]);
				if (l != -1) {
					int32_t closest[2] = {-1, -1};
					float distance[2] = {FLT_MAX, FLT_MAX};
					closest2(l, sh.x, closest, distance);
					if (closest[0] != -1) {
						f3 sum = mk(0.0f);
						int32_t count = 0;
						for (int k = 0; k < 2; k++) {
							if (closest[k] == -1)
								break;
							int32_t q = m->refs[(size_t)l * M_REFS + closest[k]];
							f3 ppos = f3of(m->probe_pos[q]), pn = f3of(m->probe_nrm[q]);
							MOnb onb = m_onb(pn);
							for (int j = 0; j < M_BINS; j++) {
								f3 probe_wo = onb.local(bin_dir[j]);
								/* scaled by the bin's index, as the reference does */
								f3 wo = normalize(((float)j * probe_wo + ppos) - sh.x);
								if (dot(wo, sh.n) <= 0.0f)
									continue;
								float geometric = kmax(dot(wo, sh.n), 0.0f);
								f3 f = m_cleanse(m_brdf(sh, wo));
								float pdf = m_pdf(sh, wo);
								f = pdf > 0.0f ? f / pdf : mk(0.0f);
								size_t b = (size_t)q * M_BINS + j;
								f3 le = m_cleanse(bin_radiance(b));
								float n = (float)m->bin_n[b];
								sum = sum
									+ (n > 0.0f ? (le / n) * f * fabsf(dot(wo, pn)) * geometric : mk(0.0f));
							}
							count++;
						}
						sec = sum / (float)(count * M_BINS);
					}
				}
			}
			f3 out = c + sec + covered;
			color[4 * i + 0] = out.x;
			color[4 * i + 1] = out.y;
			color[4 * i + 2] = out.z;
			color[4 * i + 3] = 1.0f;
		}
	}
};

} /* namespace */

struct oracle_mamba {
	MambaState st;
};

extern "C" {

oracle_mamba *oracle_mamba_create(uint32_t width, uint32_t height, int32_t max_probes, int32_t max_luts)
{
	if (width == 0 || height == 0 || max_probes < 1 || max_luts < 2)
		return nullptr;
	oracle_mamba *o = new oracle_mamba();
	MambaState &m = o->st;
	m.width = width;
	m.height = height;
	m.npix = width * height;
	m.sec_w = width / 4 + 1;
	m.sec_h = height / 4 + 1;
	m.nsec = m.sec_w * m.sec_h;
	m.max_probes = max_probes;
	m.max_luts = max_luts;
	F4 z = {0, 0, 0, 0};
	m.g_position.assign(m.npix, z);
	m.g_normal.assign(m.npix, z);
	m.g_index.assign(m.npix, 0);
	for (int k = 0; k < 2; k++) {
		m.res[k].resize(m.npix);
		m.prev[k].resize(m.npix);
	}
	m.direct_le.assign(m.npix, z);
	for (std::vector<F4> *v : {&m.s_wi, &m.s_le, &m.s_ld, &m.s_ld_wi, &m.s_hit_x, &m.s_hit_n, &m.s_hit_wo})
		v->assign(m.nsec, z);
	m.s_hit_mat.assign(m.nsec, 0);
	m.sobel.assign(m.npix, 0.0f);
	m.raster.assign(m.npix, 0.0f);
	m.raster_indicator.assign(m.npix, z);
	m.raster_radiance.assign(m.npix, z);
	m.probe_ids.assign(m.npix, 0);
	size_t groups = (size_t)((width + 15) / 16) * ((height + 15) / 16);
	m.group_probes.assign(4 * groups, 0);
	m.group_sizes.assign(groups, 0);
	m_clear_table(m);
	return o;
}

void oracle_mamba_destroy(oracle_mamba *o)
{
	delete o;
}

void oracle_mamba_frame(oracle_mamba *o, const oracle_scene *s, const oracle_mamba_params *p, float *color,
		oracle_render_stats *stats)
{
	MambaState &m = o->st;
	MambaFrame f;
	f.s = s;
	f.p = p;
	f.m = &m;
	f.lights = load_lights(s);
	m_bin_dirs(f.bin_dir);
	f.origin = mk(p->center[0], p->center[1], p->center[2]);
	f.U = mk(p->ax_u[0], p->ax_u[1], p->ax_u[2]);
	f.V = mk(p->ax_v[0], p->ax_v[1], p->ax_v[2]);
	f.W = mk(p->ax_w[0], p->ax_w[1], p->ax_w[2]);
	mat4_mul(p->prev_projection, p->prev_view, f.prev_pv);
	uint64_t records = 2ull * m.nsec;
	if (m.stamp + records + 1 > 0xFFFFFFFFull) {
		for (uint64_t &k : m.bin_depth)
			k &= 0xFFFFFFFFull;
		m.stamp = 0;
	}
	f.gbuffer();
	if (p->direct_lighting) {
		f.direct_primary();
		if (p->temporal_reuse)
			f.direct_temporal();
		if (p->spatial_reuse)
			f.direct_spatial();
	}
	f.secondary();
	f.gather();
	f.sobel();
	f.raster();
	f.collapse();
	f.allocate();
	f.final_gather(color);
	m.stamp += records;
	if (p->direct_lighting && p->spatial_reuse)
		m.res_in = 1 - m.res_in;
	if (p->direct_lighting && (p->temporal_reuse || p->spatial_reuse))
		m.prev_in = 1 - m.prev_in;
	if (stats) {
		stats->camera_rays = m.npix;
		stats->bounce_rays = f.closest_rays - m.npix;
		stats->shadow_rays = f.shadow_rays;
	}
}

int64_t oracle_mamba_buffer(const oracle_mamba *o, const char *name, void *out, uint64_t bytes)
{
	const MambaState &m = o->st;
	std::string n(name);
	const MRes4 &R = m.res[m.res_in], &P = m.prev[m.prev_in];
	const void *src = nullptr;
	size_t size = 0;
	auto pick = [&](const void *p, size_t b) {
		src = p;
		size = b;
	};
	if (n == "g_position") pick(m.g_position.data(), 16 * m.npix);
	else if (n == "g_normal") pick(m.g_normal.data(), 16 * m.npix);
	else if (n == "g_index") pick(m.g_index.data(), 4 * m.npix);
	else if (n == "direct_le") pick(m.direct_le.data(), 16 * m.npix);
	else if (n == "res_r0") pick(R.r0.data(), 16 * m.npix);
	else if (n == "res_r1") pick(R.r1.data(), 16 * m.npix);
	else if (n == "res_r2") pick(R.r2.data(), 16 * m.npix);
	else if (n == "res_r3") pick(R.r3.data(), 16 * m.npix);
	else if (n == "prev_r0") pick(P.r0.data(), 16 * m.npix);
	else if (n == "prev_r1") pick(P.r1.data(), 16 * m.npix);
	else if (n == "prev_r2") pick(P.r2.data(), 16 * m.npix);
	else if (n == "prev_r3") pick(P.r3.data(), 16 * m.npix);
	else if (n == "s_wi") pick(m.s_wi.data(), 16 * (size_t)m.nsec);
	else if (n == "s_le") pick(m.s_le.data(), 16 * (size_t)m.nsec);
	else if (n == "s_ld") pick(m.s_ld.data(), 16 * (size_t)m.nsec);
	else if (n == "s_ld_wi") pick(m.s_ld_wi.data(), 16 * (size_t)m.nsec);
	else if (n == "s_hit_x") pick(m.s_hit_x.data(), 16 * (size_t)m.nsec);
	else if (n == "s_hit_n") pick(m.s_hit_n.data(), 16 * (size_t)m.nsec);
	else if (n == "s_hit_wo") pick(m.s_hit_wo.data(), 16 * (size_t)m.nsec);
	else if (n == "s_hit_mat") pick(m.s_hit_mat.data(), 4 * (size_t)m.nsec);
	else if (n == "sobel") pick(m.sobel.data(), 4 * m.npix);
	else if (n == "raster") pick(m.raster.data(), 4 * m.npix);
	else if (n == "raster_indicator") pick(m.raster_indicator.data(), 16 * m.npix);
	else if (n == "raster_radiance") pick(m.raster_radiance.data(), 16 * m.npix);
	else if (n == "probe_ids") pick(m.probe_ids.data(), 4 * m.npix);
	else if (n == "group_probes") pick(m.group_probes.data(), 4 * m.group_probes.size());
	else if (n == "group_sizes") pick(m.group_sizes.data(), 4 * m.group_sizes.size());
	else if (n == "counters") pick(m.counters, 8);
	else if (n == "luts") pick(m.luts.data(), sizeof(MLut) * m.luts.size());
	else if (n == "refs") pick(m.refs.data(), 4 * m.refs.size());
	else if (n == "hashes") pick(m.hashes.data(), 4 * m.hashes.size());
	else if (n == "lut_positions") pick(m.lut_positions.data(), 16 * m.lut_positions.size());
	else if (n == "probe_pos") pick(m.probe_pos.data(), 16 * m.probe_pos.size());
	else if (n == "probe_nrm") pick(m.probe_nrm.data(), 16 * m.probe_nrm.size());
	else if (n == "bin_le") pick(m.bin_le.data(), 8 * m.bin_le.size());
	else if (n == "bin_n") pick(m.bin_n.data(), 4 * m.bin_n.size());
	else if (n == "bin_depth") pick(m.bin_depth.data(), 8 * m.bin_depth.size());
	else
		return -1;
	if (out) {
		if (bytes > size)
			return -1;
		memcpy(out, src, bytes);
	}
	return (int64_t)size;
}

} /* extern "C" */

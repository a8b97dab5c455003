/*
 * mamba.cu -- the "mamba" attachment's kernels: G-buffer, ReSTIR DI with 8
 * candidates, the quarter-resolution secondary rays, the irradiance-probe
 * splat, Sobel filter, probe raster, collapse and allocation, and the final
 * gather (Mamba::render, editor/mamba.cu:941-1312).  The state and the
 * choices that make the frame deterministic are described in kgr_mamba.h.
 */
#include "kgr_mamba.h"

#include <float.h>
#include <math.h>
#include <string.h>

#include <string>

#include "kgr_device.cuh"

namespace kgr {

namespace {

#define MAMBA_PI 3.14159265358979323846f  /* brdf.cuh PI, a float */
#define MAMBA_PI_D 3.14159265358979323846 /* M_PI, a double */
#define MAMBA_CANDIDATES 8                /* __raygen__direct_primary, mamba_shader.cu:249 */
#define MAMBA_MCAP 200                    /* mamba_shader.cu:371, :468 */
#define MAMBA_NEIGHBORS 2                 /* mamba_shader.cu:457 */
#define MAMBA_RADIUS 20                   /* mamba_shader.cu:464 */
#define MAMBA_ENV_DISTANCE 1000.0f        /* ENVIRONMENT_DISTANCE, mamba_shader.cu:99 */
#define MAMBA_OCCLUSION_EPS 1e-3f         /* occluded(), mamba_shader.cu:41 */
#define MAMBA_SIZE 5                      /* IrradianceProbe::size */
#define MAMBA_TOP_SIZE 250.0f             /* IrradianceProbeLUT::L2 = L1 * 25 */
#define MAMBA_L1_SIZE 10.0f               /* IrradianceProbeLUT::L1 */
#define MAMBA_DIVISION 25.0f              /* RESOLUTION_DIVISION */
#define MAMBA_FIXED_LIMIT 4611686018427387904.0f /* 2^62: a splat is clamped to +-2^62 */

/* COLOR_WHEEL (mamba.cu:227-241): the probe indicator's colours. */
__constant__ float c_color_wheel[12][3] = {{0.910f, 0.490f, 0.490f}, {0.910f, 0.700f, 0.490f},
	{0.910f, 0.910f, 0.490f}, {0.700f, 0.910f, 0.490f}, {0.490f, 0.910f, 0.490f}, {0.490f, 0.910f, 0.700f},
	{0.490f, 0.910f, 0.910f}, {0.490f, 0.700f, 0.910f}, {0.490f, 0.490f, 0.910f}, {0.700f, 0.490f, 0.910f},
	{0.910f, 0.490f, 0.910f}, {0.910f, 0.490f, 0.700f}};

/* ------------------------------------------------------------ surfaces -- */

/* load_surface_hit (mamba_shader.cu:166-219) over the traced G-buffer: the
 * normal turned toward the camera, the point pushed 1e-3 along it (against
 * it for transmissive materials). */
__device__ __forceinline__ bool load_surface(const MambaParams &mp, const MambaBuffers &mb,
		const kgr_material *mats, uint32_t pix, SurfaceHit &sh)
{
	int32_t idx = mb.g_index[pix];
	if (idx == -1)
		return false;
	f3 position = f3_of(mb.g_position[pix]);
	f3 normal = f3_of(mb.g_normal[pix]);
	f3 origin = mk(mp.origin[0], mp.origin[1], mp.origin[2]);
	f3 ray = position - origin;
	if (dot(ray, normal) > 0.0f)
		normal = -normal;
	sh.x = position;
	sh.wo = normalize(origin - position);
	sh.n = normalize(normal);
	sh.entering = true;
	sh.mat = load_material(mats, (uint32_t)idx);
	float sign = (sh.mat.type == KGR_SHADING_TRANSMISSION) ? -1.0f : 1.0f;
	sh.x = sh.x + sign * sh.n * 1e-3f;
	return true;
}

__device__ __forceinline__ f3 cleanse(const f3 &v)
{
	return anynan(v) ? mk(0.0f) : v;
}

__device__ __forceinline__ float luminance(const f3 &v)
{
	return v.x + v.y + v.z;
}

/* brdf(sh, wi, sh.mat.type) (brdf.cuh:436-447): Glass::brdf is zero. */
__device__ __forceinline__ f3 m_brdf(const SurfaceHit &sh, const f3 &wi)
{
	if (sh.mat.type & KGR_SHADING_TRANSMISSION)
		return sh.mat.diffuse / KGR_PI_DEV + mk(0.0f);
	return brdf(sh, wi);
}

/* pdf(sh, wi, sh.mat.type) (brdf.cuh:450-457): Glass::pdf is zero. */
__device__ __forceinline__ float m_pdf(const SurfaceHit &sh, const f3 &wi)
{
	if (sh.mat.type & KGR_SHADING_TRANSMISSION)
		return 0.0f;
	return ggx_pdf(sh.mat, sh.n, wi, sh.wo);
}

/* m_brdf and m_pdf of one direction, sharing the GGX lobe's terms */
__device__ __forceinline__ void m_brdf_pdf(const SurfaceHit &sh, const f3 &wi, f3 &f, float &pdf)
{
	if (sh.mat.type & KGR_SHADING_TRANSMISSION) {
		f = sh.mat.diffuse / KGR_PI_DEV + mk(0.0f);
		pdf = 0.0f;
		return;
	}
	f3 spec;
	ggx_brdf_pdf(sh.mat, sh.n, wi, sh.wo, spec, pdf);
	f = sh.mat.diffuse / KGR_PI_DEV + spec;
}

/* sky_at (editor/optix/common.cuh:18-31) */
__device__ __forceinline__ float4 sky_at(const DeviceScene &s, const f3 &d)
{
	if (!s.has_env)
		return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
	float theta = kacos(d.y);
	float phi = katan2(d.z, d.x);
	float u = phi / (2.0f * MAMBA_PI);
	float v = theta / MAMBA_PI;
	return tex2D<float4>((cudaTextureObject_t)s.env, u, 1.0f - v);
}

/* ray_at (mamba_shader.cu:89-97): the direction of a pixel's corner */
__device__ __forceinline__ f3 ray_at(const MambaParams &mp, uint32_t x, uint32_t y)
{
	uint32_t yy = mp.height - (y + 1);
	float u = 2.0f * (float)x / (float)mp.width - 1.0f;
	float v = 2.0f * (float)yy / (float)mp.height - 1.0f;
	f3 U = mk(mp.U[0], mp.U[1], mp.U[2]), V = mk(mp.V[0], mp.V[1], mp.V[2]), W = mk(mp.W[0], mp.W[1], mp.W[2]);
	return normalize(u * U - v * V + W);
}

/* ------------------------------------------------------------- lights -- */

/* LightInfo (mamba_shader.cuh:19-25) */
struct LightInfo {
	f3 position, normal, emission;
	bool sky;
};

__device__ __forceinline__ LightInfo no_light()
{
	LightInfo l;
	l.position = l.normal = l.emission = mk(0.0f);
	l.sky = false;
	return l;
}

/* sample_light (mamba_shader.cu:101-164): a uniform pick over the area
 * lights and the sky, then a point.  An area light here is one emissive
 * triangle with vertices a, a + ab, a + ac.  Returns the point's pdf, or
 * -1 with nothing to sample. */
__device__ __forceinline__ float m_sample_light(const DeviceScene &s, LightInfo &li, f3 &seed)
{
	unsigned int total = s.light_count + (s.has_env ? 1u : 0u);
	if (total == 0)
		return -1.0f;
	unsigned int light_index = rand_uniform(total, seed);
	float area;
	if (light_index < s.light_count) {
		(void)rand_uniform(1u, seed); /* the triangle within the light */
		TriLight l = load_light(s.lights, light_index);
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
		float theta = (2.0f * MAMBA_PI) * rand_uniform(seed);
		float phi = MAMBA_PI * rand_uniform(seed);
		f3 dir = mk(ksin(phi) * kcos(theta), kcos(phi), ksin(phi) * ksin(theta));
		float4 e = sky_at(s, dir);
		li.sky = true;
		li.position = MAMBA_ENV_DISTANCE * dir;
		li.normal = mk(0.0f);
		li.emission = mk(e.x, e.y, e.z);
		area = 4.0f * MAMBA_PI;
	}
	return 1.0f / (area * (float)total);
}

/* direct_unoccluded (mamba_shader.cu:74-87) */
__device__ __forceinline__ f3 m_direct_unoccluded(const SurfaceHit &sh, const LightInfo &li)
{
	f3 wi = normalize(li.position - sh.x);
	float R = length(li.position - sh.x);
	f3 rho = cleanse(m_brdf(sh, wi));
	float ldotn = li.sky ? 1.0f : fabsf(dot(li.normal, wi));
	float ndotwi = fabsf(dot(sh.n, wi));
	float falloff = li.sky ? 1.0f : 1.0f / (R * R);
	return rho * li.emission * ldotn * ndotwi * falloff;
}

/* target (mamba_shader.cu:274-279); occluded_target (:281-287) is this
 * times 1 - occluded, with the shadow ray walked by visibility_kernel */
__device__ __forceinline__ float m_target(const SurfaceHit &sh, const LightInfo &li)
{
	return luminance(m_direct_unoccluded(sh, li));
}

/* ---------------------------------------------------------- reservoirs -- */

/* Reservoir<LightInfo> (editor/optix/common.cuh:53-104) */
struct MRes {
	LightInfo data;
	float w, W;
	int M;
	f3 seed;

	__device__ __forceinline__ void update(const LightInfo &sample, float weight)
	{
		w += weight;
		float eta = rand_uniform(seed);
		bool selected = (eta * w) < weight;
		if (selected)
			data = sample;
		M++;
	}
	__device__ __forceinline__ void resample(float target)
	{
		float d = target * (float)M;
		W = (d > 0.0f) ? w / d : 0.0f;
	}
	__device__ __forceinline__ void reset()
	{
		w = 0.0f;
		M = 0;
		W = 0.0f;
	}
};

/* Reservoir(seed): an empty reservoir with a zero sample */
__device__ __forceinline__ MRes fresh_res(const f3 &seed)
{
	MRes r;
	r.data = no_light();
	r.w = r.W = 0.0f;
	r.M = 0;
	r.seed = seed;
	return r;
}

__device__ __forceinline__ MRes load_res(const MambaReservoirs &R, uint32_t i)
{
	float4 a = R.r0[i], b = R.r1[i], c = R.r2[i], d = R.r3[i];
	MRes r;
	r.data.position = mk(a.x, a.y, a.z);
	r.data.normal = mk(b.x, b.y, b.z);
	r.data.sky = b.w != 0.0f;
	r.data.emission = mk(c.x, c.y, c.z);
	r.M = __float_as_int(c.w);
	r.w = d.x;
	r.W = d.y;
	r.seed = mk(d.z, d.w, a.w);
	return r;
}

__device__ __forceinline__ void store_res(const MambaReservoirs &R, uint32_t i, const MRes &r)
{
	R.r0[i] = make_float4(r.data.position.x, r.data.position.y, r.data.position.z, r.seed.z);
	R.r1[i] = make_float4(r.data.normal.x, r.data.normal.y, r.data.normal.z, r.data.sky ? 1.0f : 0.0f);
	R.r2[i] = make_float4(r.data.emission.x, r.data.emission.y, r.data.emission.z, __int_as_float(r.M));
	R.r3[i] = make_float4(r.w, r.W, r.seed.x, r.seed.y);
}

/* direct.Le = (Le * samples + emission + new_direct) / (samples + 1) */
__device__ __forceinline__ void accumulate_direct(const MambaParams &mp, const MambaBuffers &mb, uint32_t pix,
		const SurfaceHit &sh, const f3 &Ld, bool occl, float W)
{
	f3 new_direct = cleanse(Ld * (1.0f - (float)occl) * W);
	f3 le = f3_of(mb.direct_Le[pix]);
	le = (le * (float)mp.samples + sh.mat.emission + new_direct) / (float)(mp.samples + 1);
	mb.direct_Le[pix] = f4_of(le, 0.0f);
}

/* reproject (mamba_shader.cu:289-321): the pixel itself unless the camera
 * moved (samples = 0); indices outside the image are rejected */
__device__ __forceinline__ int m_reproject(const MambaParams &mp, int index, const f3 &x)
{
	if (mp.samples > 0)
		return index;
	const float *m = mp.prev_proj_view;
	float q[4];
	for (int i = 0; i < 4; i++)
		q[i] = m[0 * 4 + i] * x.x + m[1 * 4 + i] * x.y + m[2 * 4 + i] * x.z + m[3 * 4 + i] * 1.0f;
	float u = q[0] / q[3];
	float v = q[1] / q[3];
	if (!((u >= -1.0f && u <= 1.0f) && (v >= -1.0f && v <= 1.0f)))
		return -1;
	u = (u + 1.0f) * 0.5f;
	v = (v + 1.0f) * 0.5f;
	int ix = (int)((double)(u * (float)mp.width) + 0.5);
	int iy = (int)((double)(v * (float)mp.height) + 0.5);
	if (ix < 0 || iy < 0 || ix >= (int)mp.width || iy >= (int)mp.height)
		return -1;
	return iy * (int)mp.width + ix;
}

/* sample_spatial_neighborhood (mamba_shader.cu:395-417) */
__device__ __forceinline__ int m_spatial_neighbor(const MambaParams &mp, int index, f3 &seed, int radius)
{
	int width = (int)mp.width, height = (int)mp.height;
	int x = index % width;
	int y = index / width;
	f3 offset = rand_uniform_3f(seed);
	float theta = (float)(2.0 * MAMBA_PI_D * (double)offset.x);
	float r = (float)radius * ksqrt(offset.y);
	int x0 = (int)((float)x + r * kcos(theta));
	int y0 = (int)((float)y + r * ksin(theta));
	x0 = x0 < 0 ? 0 : (x0 > width - 1 ? width - 1 : x0);
	y0 = y0 < 0 ? 0 : (y0 > height - 1 ? height - 1 : y0);
	return x0 + y0 * width;
}

/* ------------------------------------------------------- probe tables -- */

/* ONB (brdf.cuh:77-105) */
struct Onb {
	f3 u, v, w;
	__device__ __forceinline__ f3 local(const f3 &a) const { return a.x * u + a.y * v + a.z * w; }
	__device__ __forceinline__ f3 inv_local(const f3 &a) const { return mk(dot(a, u), dot(a, v), dot(a, w)); }
};

__device__ __forceinline__ Onb onb_from_normal(const f3 &n)
{
	Onb o;
	o.w = normalize(n);
	/* fabs(w.x) > 0.9 compares in double; for a float, x > 0.9f is the same
	 * test (0.9f is just below 0.9, and the next float is above it) without
	 * the FP64 pipe */
	f3 a = (fabsf(o.w.x) > 0.9f) ? mk(0.0f, 1.0f, 0.0f) : mk(1.0f, 0.0f, 0.0f);
	o.v = normalize(cross(o.w, a));
	o.u = cross(o.w, o.v);
	return o;
}

/* to_disk + to_index (probe.cuh:36-54): the disk bin of a local
 * direction.  A direction with a NaN component falls in bin 0, as the
 * reference's float-to-int conversion of NaN gives 0. */
__device__ __forceinline__ void to_disk(const f3 &v, float &su, float &sv)
{
	float theta = katan2(v.y, v.x);
	if (theta < 0.0f)
		theta = (float)((double)theta + 2.0 * MAMBA_PI_D);
	float rp = ksqrt(v.x * v.x + v.y * v.y);
	su = (float)((double)theta / (2.0 * MAMBA_PI_D));
	sv = rp;
}

__device__ __forceinline__ int32_t bin_of(const f3 &v)
{
	if (kisnan(v.x) || kisnan(v.y))
		return 0;
	float su, sv;
	to_disk(v, su, sv);
	int32_t x = (int32_t)(su * (float)MAMBA_SIZE);
	int32_t y = (int32_t)(sv * (float)MAMBA_SIZE);
	int32_t i = y * MAMBA_SIZE + x;
	return i < 0 ? 0 : (i > KGR_PROBE_BINS - 1 ? KGR_PROBE_BINS - 1 : i);
}

__device__ __forceinline__ bool lut_contains(const MambaLut &L, const f3 &x, bool neighbor)
{
	float e = L.size / 2.0f + (neighbor ? 1.0f : 0.0f) * L.resolution;
	f3 c = mk(L.center[0], L.center[1], L.center[2]);
	f3 mn = c - mk(e), mx = c + mk(e);
	return (x.x >= mn.x && x.y >= mn.y && x.z >= mn.z) && (x.x <= mx.x && x.y <= mx.y && x.z <= mx.z);
}

/* hash (probe.cuh:168-187): cell coordinates in 11 bits each, shuffled;
 * the first shuffle shifts a signed value (arithmetic shift) */
__device__ __forceinline__ uint32_t lut_hash(const MambaLut &L, const f3 &x, int dx, int dy, int dz)
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

__device__ __forceinline__ uint32_t lut_neighbor_hash(const MambaLut &L, const f3 &x, int ni)
{
	return lut_hash(L, x, ni % 3 - 1, (ni / 3) % 3 - 1, ni / 9 - 1);
}

__device__ __forceinline__ MambaLut load_lut(const MambaTable &T, int32_t l)
{
	return T.luts[l];
}

/* lookup (probe.cuh:256-285): of the two slots of x's cell (or of a
 * neighbouring cell ni), the one with the same hash nearest to x */
__device__ __forceinline__ int32_t lut_lookup(const MambaTable &T, int32_t l, const MambaLut &L, const f3 &x,
		int ni)
{
	if (!lut_contains(L, x, ni != -1))
		return -1;
	uint32_t h = (ni == -1) ? lut_hash(L, x, 0, 0, 0) : lut_neighbor_hash(L, x, ni);
	size_t base = (size_t)l * KGR_LUT_REFS;
	int32_t index = -1;
	float closest = FLT_MAX;
	for (int i = 0; i < 2; i++) {
		int32_t j = (int32_t)((h + (uint32_t)(i * i)) % (uint32_t)KGR_LUT_REFS);
		if (T.refs[base + j] == -1)
			break;
		if (T.hashes[base + j] == h) {
			float dist = length(f3_of(T.positions[base + j]) - x);
			if (dist < closest) {
				closest = dist;
				index = j;
			}
		}
	}
	return index;
}

/* full_lookup (probe.cuh:287-301) */
__device__ __forceinline__ int32_t lut_full_lookup(const MambaTable &T, int32_t l, const f3 &x)
{
	MambaLut L = load_lut(T, l);
	int32_t r = lut_lookup(T, l, L, x, -1);
	if (r == -1) {
		for (int ni = 0; ni < 27; ni++) {
			r = lut_lookup(T, l, L, x, ni);
			if (r != -1)
				break;
		}
	}
	return r;
}

/* lookup_L2 (probe.cuh:678-712): linear probing over the top table from
 * the cell's hash to the first empty slot or the slot whose cell holds x */
__device__ __forceinline__ int32_t top_lookup(const MambaTable &T, const f3 &x)
{
	MambaLut L = load_lut(T, 0);
	if (!lut_contains(L, x, false))
		return -1;
	uint32_t h = lut_hash(L, x, 0, 0, 0);
	f3 half = mk(0.5f * L.resolution);
	for (int i = 0; i < KGR_LUT_REFS; i++) {
		uint32_t j = (h + (uint32_t)i) % (uint32_t)KGR_LUT_REFS;
		if (T.refs[j] == -1)
			return -1;
		f3 c = f3_of(T.positions[j]);
		f3 mn = c - half, mx = c + half;
		if ((x.x <= mx.x && x.y <= mx.y && x.z <= mx.z) && (x.x >= mn.x && x.y >= mn.y && x.z >= mn.z))
			return (int32_t)j;
	}
	return -1;
}

/* The second-level table of x, or -1: lookup_L2 and the reference's guard
 * against an index at or above the probe counter (mamba.cu:278, 456, 490, 550, 793) */
__device__ __forceinline__ int32_t table_of(const MambaTable &T, const f3 &x, int32_t probe_counter)
{
	int32_t r = top_lookup(T, x);
	if (r == -1)
		return -1;
	int32_t l = T.refs[r];
	if (l < 0 || l >= probe_counter)
		return -1;
	return l;
}

/* closest<2> (probe.cuh:305-363): the two nearest occupied slots among the
 * two tries of x's cell and of its 27 neighbours (no hash check) */
__device__ __forceinline__ void lut_closest2(const MambaTable &T, int32_t l, const f3 &x, int32_t idx[2],
		float dist[2])
{
	MambaLut L = load_lut(T, l);
	if (!lut_contains(L, x, true))
		return;
	size_t base = (size_t)l * KGR_LUT_REFS;
	for (int ni = -1; ni < 27; ni++) {
		uint32_t h = ni == -1 ? lut_hash(L, x, 0, 0, 0) : lut_neighbor_hash(L, x, ni);
		for (int i = 0; i < 2; i++) {
			int32_t j = (int32_t)((h + (uint32_t)(i * i)) % (uint32_t)KGR_LUT_REFS);
			if (T.refs[base + j] == -1)
				break;
			float d = length(f3_of(T.positions[base + j]) - x);
			for (int k = 0; k < 2; k++) {
				if (d < dist[k]) {
					if (k == 0) {
						dist[1] = dist[0];
						idx[1] = idx[0];
					}
					dist[k] = d;
					idx[k] = j;
					break;
				}
			}
		}
	}
}

__device__ __forceinline__ f3 bin_radiance(const MambaTable &T, size_t bin)
{
	long long a = (long long)T.bin_le[3 * bin + 0], b = (long long)T.bin_le[3 * bin + 1],
		  c = (long long)T.bin_le[3 * bin + 2];
	return mk(__ll2float_rn(a) * KGR_MAMBA_UNFIXED, __ll2float_rn(b) * KGR_MAMBA_UNFIXED,
		__ll2float_rn(c) * KGR_MAMBA_UNFIXED);
}

__device__ __forceinline__ float bin_depth(const MambaTable &T, size_t bin)
{
	return __uint_as_float((uint32_t)(T.bin_depth[bin] & 0xFFFFFFFFull));
}

__device__ __forceinline__ long long to_fixed(float v)
{
	float s = v * KGR_MAMBA_FIXED;
	if (kisnan(s))
		return 0;
	if (s >= MAMBA_FIXED_LIMIT)
		return 4611686018427387904ll;
	if (s <= -MAMBA_FIXED_LIMIT)
		return -4611686018427387904ll;
	return __float2ll_rn(s);
}

/* ============================================================= kernels == */

/* G-buffer rays: one per pixel centre, queued in tile order for the
 * closest-hit walk (the raster pass of the reference) */
__global__ void gbuffer_rays_kernel(PathBuffers pb, MambaParams mp)
{
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i == 0) {
		pb.counters[CNT_Q0] = mp.npix;
		pb.counters[CNT_Q1] = 0;
		pb.counters[CNT_SHADOW] = 0;
	}
	if (i >= mp.npix)
		return;
	uint32_t x = i % mp.width, y = i / mp.width;
	uint32_t yy = mp.height - (y + 1);
	float u = 2.0f * ((float)x + 0.5f) / (float)mp.width - 1.0f;
	float v = 2.0f * ((float)yy + 0.5f) / (float)mp.height - 1.0f;
	f3 U = mk(mp.U[0], mp.U[1], mp.U[2]), V = mk(mp.V[0], mp.V[1], mp.V[2]), W = mk(mp.W[0], mp.W[1], mp.W[2]);
	f3 d = normalize(u * U - v * V + W);
	pb.ray_o[i] = make_float4(mp.origin[0], mp.origin[1], mp.origin[2], 0.0f);
	pb.ray_d[i] = f4_of(d, 1e16f);
	pb.queue[0][i] = tiled_pixel(i, mp.width, mp.height);
}

/* The G-buffer of the raster pass (editor/shaders.cpp gbuffer shaders):
 * interpolated position, normalised interpolated shading normal, material;
 * a miss keeps zero position and normal and index -1. */
__global__ void gbuffer_store_kernel(DeviceScene s, PathBuffers pb, MambaParams mp, MambaBuffers mb)
{
	uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
	if (pix >= mp.npix)
		return;
	float4 hv = pb.hit[pix];
	int32_t prim = __float_as_int(hv.x);
	if (prim < 0) {
		mb.g_position[pix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
		mb.g_normal[pix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
		mb.g_index[pix] = -1;
		return;
	}
	uint4 t = __ldg(&s.tris[prim]);
	f3 a = f3_of(__ldg(&s.positions[t.x])), b = f3_of(__ldg(&s.positions[t.y])), c = f3_of(__ldg(&s.positions[t.z]));
	f3 na = f3_of(__ldg(&s.normals[t.x])), nb = f3_of(__ldg(&s.normals[t.y])), nc = f3_of(__ldg(&s.normals[t.z]));
	float b1 = hv.z, b2 = hv.w;
	float w0 = 1.0f - b1 - b2;
	f3 x = w0 * a + b1 * b + b2 * c;
	f3 n = normalize(w0 * na + b1 * nb + b2 * nc);
	mb.g_position[pix] = f4_of(x, 1.0f);
	mb.g_normal[pix] = f4_of(n, 1.0f);
	mb.g_index[pix] = (int32_t)t.w;
}

/* ------------------------------------------------ direct lighting rays -- */

/* The direct-lighting passes run as wavefronts: a resampling kernel queues
 * its shadow rays -- occluded(origin, target) of mamba_shader.cu:38-64, in
 * slot k * npix + pixel -- the path tracer's any-hit walk (tuned launch
 * shape) takes them all with full warps and stores a blocked flag per slot,
 * and the next kernel reads the flags.  Each kernel redoes the arithmetic
 * and the draws of the one before it, so the results are those of the
 * per-pixel programs. */
__device__ __forceinline__ void queue_ray(const MambaBuffers &mb, uint32_t slot, const f3 &o, const f3 &target,
		bool pred)
{
	if (pred) {
		mb.vis_o[slot] = f4_of(o, 0.0f);
		mb.vis_d[slot] = f4_of(normalize(target - o), length(target - o) - MAMBA_OCCLUSION_EPS);
	}
	queue_append(mb.vis_queue, mb.vis_counters + CNT_SHADOW, slot, pred);
}

__device__ __forceinline__ bool blocked(const MambaBuffers &mb, uint32_t slot)
{
	return mb.vis_flag[slot] != 0u;
}

/* __raygen__direct_primary (mamba_shader.cu:221-272): the eight candidates
 * and the selected sample's shadow ray */
__global__ void __launch_bounds__(128) primary_ris_kernel(DeviceScene s, MambaParams mp, MambaBuffers mb)
{
	uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
	if (pix >= mp.npix)
		return;
	uint32_t x = pix % mp.width, y = pix / mp.width;
	const MambaReservoirs R = mb.res[mp.res_in];
	MRes r = load_res(R, pix);
	r.reset();
	SurfaceHit sh;
	bool hit = load_surface(mp, mb, s.materials, pix, sh);
	if (hit) {
		f3 seed = mk((float)x, (float)y, mp.time);
		for (int i = 0; i < MAMBA_CANDIDATES; i++) {
			LightInfo lighting = no_light();
			float pdf = m_sample_light(s, lighting, seed);
			f3 Ld = m_direct_unoccluded(sh, lighting);
			float target = Ld.x + Ld.y + Ld.z;
			r.update(lighting, target / pdf > 0.0f ? target / pdf : 0.0f);
		}
	}
	store_res(R, pix, r);
	queue_ray(mb, pix, hit ? sh.x : mk(0.0f), r.data.position, hit);
}

/* ... its resample(luminance(Ld * (1 - occluded))) and, when it is the
 * last pass, the accumulated direct light */
__global__ void __launch_bounds__(128) primary_finish_kernel(DeviceScene s, MambaParams mp, MambaBuffers mb)
{
	uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
	if (pix >= mp.npix)
		return;
	SurfaceHit sh;
	if (!load_surface(mp, mb, s.materials, pix, sh))
		return;
	const MambaReservoirs R = mb.res[mp.res_in];
	MRes r = load_res(R, pix);
	f3 Ld_res = m_direct_unoccluded(sh, r.data);
	bool occl = blocked(mb, pix);
	r.resample(luminance(Ld_res * (1.0f - (float)occl)));
	R.r3[pix].y = r.W;
	if (!mp.temporal && !mp.spatial)
		accumulate_direct(mp, mb, pix, sh, Ld_res, occl, r.W);
}

/* __raygen__temporal_reuse (mamba_shader.cu:323-393).  The previous
 * reservoirs are read from prev[prev_in] as the last frame left them and
 * written to prev[1 - prev_in] (every pixel writes its entry).  First
 * launch: the shadow rays of the current and the reprojected previous
 * sample (occluded_target). */
__global__ void __launch_bounds__(128) temporal_gather_kernel(DeviceScene s, MambaParams mp, MambaBuffers mb)
{
	uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
	if (pix >= mp.npix)
		return;
	const MambaReservoirs R = mb.res[mp.res_in], Pin = mb.prev[mp.prev_in], Pout = mb.prev[1 - mp.prev_in];
	SurfaceHit sh;
	if (!load_surface(mp, mb, s.materials, pix, sh)) {
		MRes p = load_res(Pin, pix);
		p.reset();
		store_res(Pout, pix, p);
		return;
	}
	MRes cur = load_res(R, pix);
	if (cur.M <= 0) {
		store_res(Pout, pix, load_res(Pin, pix));
		return;
	}
	int pindex = m_reproject(mp, (int)pix, sh.x);
	bool has_prev = false;
	f3 prev_point = mk(0.0f);
	if (pindex >= 0) {
		MRes prev = load_res(Pin, (uint32_t)pindex);
		has_prev = prev.M > 0;
		prev_point = prev.data.position;
	}
	queue_ray(mb, pix, sh.x, cur.data.position, true);
	queue_ray(mb, mp.npix + pix, sh.x, prev_point, has_prev);
}

/* ... the merge with the occluded targets, and the lighting ray when the
 * temporal pass is the last */
__global__ void __launch_bounds__(128) temporal_merge_kernel(DeviceScene s, MambaParams mp, MambaBuffers mb)
{
	uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
	if (pix >= mp.npix)
		return;
	uint32_t x = pix % mp.width, y = pix / mp.width;
	const MambaReservoirs R = mb.res[mp.res_in], Pin = mb.prev[mp.prev_in], Pout = mb.prev[1 - mp.prev_in];
	SurfaceHit sh;
	if (!load_surface(mp, mb, s.materials, pix, sh))
		return;
	MRes cur = load_res(R, pix);
	if (cur.M <= 0)
		return;
	int pindex = m_reproject(mp, (int)pix, sh.x);
	MRes merged = fresh_res(2.0f * mk((float)x, (float)y, mp.time));
	f3 Li = m_direct_unoccluded(sh, cur.data);
	float t_current = luminance(Li * (1.0f - (float)blocked(mb, pix)));
	merged.update(cur.data, t_current * cur.W * (float)cur.M);
	int N = cur.M;
	if (pindex >= 0) {
		MRes prev = load_res(Pin, (uint32_t)pindex);
		if (prev.M > 0) {
			prev.M = min(prev.M, MAMBA_MCAP);
			f3 Lp = m_direct_unoccluded(sh, prev.data);
			float t_previous = luminance(Lp * (1.0f - (float)blocked(mb, mp.npix + pix)));
			merged.update(prev.data, t_previous * prev.W * (float)prev.M);
			N += (t_previous > 0.0f) * prev.M;
		}
	}
	merged.M = N;
	merged.resample(m_target(sh, merged.data));
	store_res(R, pix, merged);
	if (mp.spatial)
		store_res(Pout, pix, load_res(Pin, pix));
	queue_ray(mb, pix, sh.x, merged.data.position, !mp.spatial);
}

/* ... the direct light of the merged sample and the previous reservoir of
 * the next frame (when the temporal pass is the last) */
__global__ void __launch_bounds__(128) temporal_finish_kernel(DeviceScene s, MambaParams mp, MambaBuffers mb)
{
	uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
	if (pix >= mp.npix)
		return;
	SurfaceHit sh;
	if (!load_surface(mp, mb, s.materials, pix, sh))
		return;
	const MambaReservoirs R = mb.res[mp.res_in], Pout = mb.prev[1 - mp.prev_in];
	MRes merged = load_res(R, pix);
	if (merged.M <= 0)
		return; /* skipped by the merge (no current sample) */
	f3 Ld_res = m_direct_unoccluded(sh, merged.data);
	accumulate_direct(mp, mb, pix, sh, Ld_res, blocked(mb, pix), merged.W);
	store_res(Pout, pix, merged);
}

/* A spatial neighbour's surface as __raygen__spatial_reuse holds it:
 * its G-buffer point and normal (zero for a miss) and the centre's wo. */
__device__ __forceinline__ SurfaceHit neighbour_hit(const MambaParams &mp, const MambaBuffers &mb,
		const kgr_material *mats, uint32_t index0, const SurfaceHit &sh)
{
	SurfaceHit h;
	h.mat = sh.mat;
	h.entering = true;
	h.x = h.n = mk(0.0f);
	load_surface(mp, mb, mats, index0, h);
	h.wo = sh.wo;
	return h;
}

/* __raygen__spatial_reuse (mamba_shader.cu:419-510): neighbours are read
 * from res[res_in], the result written to res[1 - res_in].  First launch:
 * the two neighbours (their draws replayed) and the shadow rays of their
 * samples seen from the centre. */
__global__ void __launch_bounds__(128) spatial_gather_kernel(DeviceScene s, MambaParams mp, MambaBuffers mb)
{
	uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
	if (pix >= mp.npix)
		return;
	uint32_t x = pix % mp.width, y = pix / mp.width;
	const MambaReservoirs Rin = mb.res[mp.res_in], Rout = mb.res[1 - mp.res_in];
	const MambaReservoirs Pin = mb.prev[mp.prev_in], Pout = mb.prev[1 - mp.prev_in];
	MRes cur = load_res(Rin, pix);
	SurfaceHit sh;
	bool hit = load_surface(mp, mb, s.materials, pix, sh);
	if (!hit || cur.M <= 0) {
		if (hit)
			mb.direct_Le[pix] = make_float4(0.0f, 0.0f, 1.0f, 0.0f);
		store_res(Rout, pix, cur);
		MRes p = load_res(Pin, pix);
		p.reset();
		store_res(Pout, pix, p);
		return;
	}
	f3 seed = 2.0f * mk((float)x, (float)y, mp.time);
	(void)rand_uniform(seed); /* the centre's update */
	int i0 = m_spatial_neighbor(mp, (int)pix, seed, MAMBA_RADIUS);
	MRes nb0 = load_res(Rin, (uint32_t)i0);
	if (nb0.M > 0)
		(void)rand_uniform(seed); /* the first neighbour's update */
	int i1 = m_spatial_neighbor(mp, (int)pix, seed, MAMBA_RADIUS);
	MRes nb1 = load_res(Rin, (uint32_t)i1);
	queue_ray(mb, pix, sh.x, nb0.data.position, nb0.M > 0);
	queue_ray(mb, mp.npix + pix, sh.x, nb1.data.position, nb1.M > 0);
}

/* ... the merge over the centre and the neighbours' occluded targets, then
 * the bias correction's shadow rays (the merged sample seen from each
 * neighbour with a sample) and the lighting ray */
__global__ void __launch_bounds__(128) spatial_resample_kernel(DeviceScene s, MambaParams mp, MambaBuffers mb)
{
	uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
	if (pix >= mp.npix)
		return;
	uint32_t x = pix % mp.width, y = pix / mp.width;
	const MambaReservoirs Rin = mb.res[mp.res_in], Rout = mb.res[1 - mp.res_in];
	MRes cur = load_res(Rin, pix);
	SurfaceHit sh;
	if (!load_surface(mp, mb, s.materials, pix, sh) || cur.M <= 0)
		return;
	MRes merged = fresh_res(2.0f * mk((float)x, (float)y, mp.time));
	float t_current = m_target(sh, cur.data);
	merged.update(cur.data, t_current * cur.W * (float)cur.M);
	int index[MAMBA_NEIGHBORS], sizes[MAMBA_NEIGHBORS];
	int count = 0;
	for (int i = 0; i < MAMBA_NEIGHBORS; i++) {
		index[i] = m_spatial_neighbor(mp, (int)pix, merged.seed, MAMBA_RADIUS);
		MRes nb = load_res(Rin, (uint32_t)index[i]);
		nb.M = min(nb.M, MAMBA_MCAP);
		if (nb.M > 0) {
			f3 Li = m_direct_unoccluded(sh, nb.data);
			float t_neighbor = luminance(Li * (1.0f - (float)blocked(mb, (uint32_t)i * mp.npix + pix)));
			merged.update(nb.data, t_neighbor * nb.W * (float)nb.M);
		}
		sizes[i] = nb.M;
		count += nb.M;
	}
	merged.M = cur.M + count;
	store_res(Rout, pix, merged);
	mb.spatial_aux[pix] = make_int4(index[0], index[1], sizes[0], sizes[1]);
	for (int i = 0; i < MAMBA_NEIGHBORS; i++) {
		SurfaceHit h = neighbour_hit(mp, mb, s.materials, (uint32_t)index[i], sh);
		queue_ray(mb, (uint32_t)i * mp.npix + pix, h.x, merged.data.position, sizes[i] > 0);
	}
	queue_ray(mb, 2 * mp.npix + pix, sh.x, merged.data.position, true);
}

/* ... Z over the neighbours whose surface sees the merged sample, W, the
 * direct light, and the previous reservoir of the next frame */
__global__ void __launch_bounds__(128) spatial_finish_kernel(DeviceScene s, MambaParams mp, MambaBuffers mb)
{
	uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
	if (pix >= mp.npix)
		return;
	const MambaReservoirs Rin = mb.res[mp.res_in], Rout = mb.res[1 - mp.res_in];
	const MambaReservoirs Pout = mb.prev[1 - mp.prev_in];
	MRes cur = load_res(Rin, pix);
	SurfaceHit sh;
	if (!load_surface(mp, mb, s.materials, pix, sh) || cur.M <= 0)
		return;
	MRes merged = load_res(Rout, pix);
	int4 aux = mb.spatial_aux[pix];
	int index[MAMBA_NEIGHBORS] = {aux.x, aux.y}, sizes[MAMBA_NEIGHBORS] = {aux.z, aux.w};
	int Z = cur.M;
	for (int i = 0; i < MAMBA_NEIGHBORS; i++) {
		if (sizes[i] <= 0)
			continue;
		SurfaceHit h = neighbour_hit(mp, mb, s.materials, (uint32_t)index[i], sh);
		f3 Li = m_direct_unoccluded(h, merged.data);
		float t_neighbor = luminance(Li * (1.0f - (float)blocked(mb, (uint32_t)i * mp.npix + pix)));
		if (t_neighbor > 0.0f)
			Z += sizes[i];
	}
	float t_merged = m_target(sh, merged.data);
	float denominator = t_merged * (float)Z;
	merged.W = (denominator > 0.0f) ? merged.w / denominator : 0.0f;
	Rout.r3[pix].y = merged.W;
	f3 Ld_res = m_direct_unoccluded(sh, merged.data);
	accumulate_direct(mp, mb, pix, sh, Ld_res, blocked(mb, 2 * mp.npix + pix), merged.W);
	store_res(Pout, pix, merged);
}

/* The closest-hit program of the secondary rays (mamba_shader.cu:707-777):
 * interpolated position, geometric normal against the ray, shading normal
 * on its side. */
__device__ __forceinline__ void m_closest_surface(const DeviceScene &s, const kgr_hit &h, const f3 &dir, f3 &x,
		f3 &n, int32_t &mat)
{
	uint4 t = __ldg(&s.tris[h.prim]);
	f3 a = f3_of(__ldg(&s.positions[t.x])), b = f3_of(__ldg(&s.positions[t.y])), c = f3_of(__ldg(&s.positions[t.z]));
	f3 na = f3_of(__ldg(&s.normals[t.x])), nb = f3_of(__ldg(&s.normals[t.y])), nc = f3_of(__ldg(&s.normals[t.z]));
	float bu = h.b1, bv = h.b2;
	float bw = 1.0f - bu - bv;
	x = bw * a + bu * b + bv * c;
	f3 ng = normalize(cross(b - a, c - a));
	if (dot(dir, ng) > 0.0f)
		ng = -ng;
	f3 ns = bw * na + bu * nb + bv * nc;
	if (dot(ng, ns) < 0.0f)
		ns = -ns;
	n = normalize(ns);
	mat = (int32_t)t.w;
}

/* Ld (mamba_shader.cu:512-561): a light sample seen from the primary
 * vertex; Le, wi and R are set when it is unblocked and the vertex is not
 * emissive. */
__device__ __forceinline__ f3 m_Ld(const DeviceScene &s, int layout, const SurfaceHit &sh, f3 &seed, f3 &Le, f3 &wi,
		float &R)
{
	LightInfo li = no_light();
	float light_pdf = m_sample_light(s, li, seed);
	if (light_pdf < 0.0f)
		return mk(0.0f);
	f3 direction = normalize(li.position - sh.x);
	f3 origin = sh.x;
	kgr_hit h;
	bool blocked = trace<true>(s, layout, origin, direction, length(li.position - origin) - 1e-3f, h);
	f3 out = sh.mat.emission;
	if (!blocked && length(out) < 1e-3f) {
		wi = normalize(li.position - origin);
		R = length(li.position - origin);
		f3 f = cleanse(m_brdf(sh, wi));
		float ldotn = li.sky ? 1.0f : fabsf(dot(li.normal, wi));
		float ndotwi = fabsf(dot(sh.n, wi));
		float falloff = li.sky ? 1.0f : (R * R) + 1e-3f;
		out = f * li.emission * ldotn * ndotwi / (light_pdf * falloff);
		Le = li.emission;
	}
	return out;
}

/* __raygen__secondary (mamba_shader.cu:563-680): pixel (4 sx + c % 4,
 * 4 sy + c / 4) with c = samples % 16 of each 4x4 block */
__global__ void __launch_bounds__(128) secondary_kernel(DeviceScene s, MambaParams mp, MambaBuffers mb)
{
	uint32_t li = blockIdx.x * blockDim.x + threadIdx.x;
	if (li >= mp.sec_w * mp.sec_h)
		return;
	uint32_t sx = li % mp.sec_w, sy = li / mp.sec_w;
	int32_t cycle = mp.samples % 16;
	int32_t x = 4 * (int32_t)sx + (cycle % 4), y = 4 * (int32_t)sy + (cycle / 4);
	if (x >= (int32_t)mp.width || y >= (int32_t)mp.height)
		return;
	uint32_t pix = (uint32_t)y * mp.width + (uint32_t)x;
	SurfaceHit sh;
	if (!load_surface(mp, mb, s.materials, pix, sh)) {
		mb.s_wi[li] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
		return;
	}
	f3 wi;
	float pdf;
	f3 seed = mk((float)sx, (float)sy, mp.time);
	(void)eval(sh, wi, pdf, seed);
	if (pdf <= 0.0f) {
		float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
		mb.s_wi[li] = z;
		mb.s_hit_x[li] = z;
		mb.s_hit_n[li] = z;
		mb.s_hit_wo[li] = z;
		return;
	}
	kgr_hit h;
	trace<false>(s, mp.layout, sh.x, wi, 1e16f, h);
	if (h.prim < 0) {
		float4 e = sky_at(s, wi);
		mb.s_Le[li] = f4_of(mk(e.x, e.y, e.z) / pdf, 0.0f);
		mb.s_wi[li] = f4_of(wi, 0.0f);
		mb.s_hit_x[li] = f4_of(MAMBA_ENV_DISTANCE * wi, 0.0f);
		mb.s_hit_n[li] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
		mb.s_hit_wo[li] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
		return;
	}
	f3 hx, hn;
	int32_t hmat;
	m_closest_surface(s, h, wi, hx, hn, hmat);
	f3 Le = mk(0.0f), Le_wi = mk(0.0f);
	float Le_depth = 0.0f;
	f3 indirect = m_Ld(s, mp.layout, sh, seed, Le, Le_wi, Le_depth);
	mb.s_wi[li] = f4_of(wi, 0.0f);
	mb.s_Ld[li] = f4_of(Le, 0.0f);
	mb.s_Ld_wi[li] = f4_of(Le_wi, Le_depth);
	mb.s_Le[li] = f4_of(indirect, 0.0f);
	mb.s_hit_x[li] = f4_of(hx, 0.0f);
	mb.s_hit_n[li] = f4_of(hn, 0.0f);
	mb.s_hit_wo[li] = f4_of(-wi, 0.0f);
	mb.s_hit_mat[li] = hmat;
}

/* secondary_gather (mamba.cu:401-576), first half: each secondary pixel's
 * two splats -- its radiance (plus what the probe at its hit point sends
 * back) into the probe at the primary vertex, and the light sample's
 * emission into the probe at the hit point -- computed against the table
 * as it stands before any of this frame's splats. */
__global__ void __launch_bounds__(128) gather_splat_kernel(DeviceScene s, MambaParams mp, MambaBuffers mb)
{
	uint32_t index = blockIdx.x * blockDim.x + threadIdx.x;
	if (index >= mp.sec_w * mp.sec_h)
		return;
	mb.rec_bin[2 * index] = -1;
	mb.rec_bin[2 * index + 1] = -1;
	uint32_t sx = index % mp.sec_w, sy = index / mp.sec_w;
	int32_t cycle = mp.samples % 16;
	int32_t true_x = 4 * (int32_t)sx + (cycle % 4), true_y = 4 * (int32_t)sy + (cycle / 4);
	if (true_x >= (int32_t)mp.width || true_y >= (int32_t)mp.height)
		return;
	const MambaTable &T = mb.table;
	f3 hx = f3_of(mb.s_hit_x[index]), hn = f3_of(mb.s_hit_n[index]), hwo = f3_of(mb.s_hit_wo[index]);
	int32_t hmat = mb.s_hit_mat[index];
	f3 wi = f3_of(mb.s_wi[index]);
	f3 Le = f3_of(mb.s_Le[index]);
	float4 ldw = mb.s_Ld_wi[index];
	f3 Ld_wi = mk(ldw.x, ldw.y, ldw.z);
	float Ld_depth = ldw.w;
	f3 Ld = f3_of(mb.s_Ld[index]);
	uint32_t pix = (uint32_t)true_y * mp.width + (uint32_t)true_x;
	if (mb.g_index[pix] == -1) {
		mb.s_Le[index] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
		return;
	}
	f3 position = f3_of(mb.g_position[pix]);
	f3 normal = f3_of(mb.g_normal[pix]);
	int32_t probe_counter = T.counters[0];

	int32_t l = table_of(T, position, probe_counter);
	if (l != -1) {
		int32_t r2 = lut_full_lookup(T, l, position);
		if (r2 == -1) {
			mb.s_Le[index] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
		} else {
			Onb onb = onb_from_normal(normal);
			f3 local_wi = normalize(onb.inv_local(wi));
			int32_t probe = T.refs[(size_t)l * KGR_LUT_REFS + r2];
			int32_t bin = bin_of(local_wi);
			if (!(length(hn) < 1e-6f)) {
				/* what the probe at the hit point sends toward it */
				int32_t l2 = table_of(T, hx, probe_counter);
				int32_t r4 = l2 == -1 ? -1 : lut_full_lookup(T, l2, hx);
				if (r4 != -1) {
					int32_t p2 = T.refs[(size_t)l2 * KGR_LUT_REFS + r4];
					f3 ppos = f3_of(T.probe_pos[p2]);
					Onb o2 = onb_from_normal(f3_of(T.probe_nrm[p2]));
					SurfaceHit sec;
					sec.mat = load_material(s.materials, (uint32_t)hmat);
					sec.entering = true;
					sec.n = hn;
					sec.wo = hwo;
					sec.x = hx;
					f3 sum = mk(0.0f);
					for (int j = 0; j < KGR_PROBE_BINS; j++) {
						f3 probe_wo = o2.local(mk(mp.bin_dir[j][0], mp.bin_dir[j][1], mp.bin_dir[j][2]));
						size_t b = (size_t)p2 * KGR_PROBE_BINS + j;
						float d = bin_depth(T, b);
						f3 wo = normalize((d * probe_wo + ppos) - hx);
						if (dot(wo, hn) <= 0.0f)
							continue;
						uint32_t nb = T.bin_n[b];
						if (nb == 0) {
							sum = sum + (sec.mat.emission + mk(0.0f));
							continue;
						}
						float geometric = kmax(dot(wo, hn), 0.0f);
						f3 f = cleanse(m_brdf(sec, wo));
						f3 le = cleanse(bin_radiance(T, b));
						float n = (float)nb;
						sum = sum + (sec.mat.emission + (le / n) * f * geometric);
					}
					Le = Le + sum / (float)KGR_PROBE_BINS;
				}
			}
			mb.rec_bin[2 * index] = probe * KGR_PROBE_BINS + bin;
			mb.rec_val[2 * index] = f4_of(Le, length(position - hx));
		}
	}

	if (length(hn) > 1e-6f) {
		int32_t lb = table_of(T, hx, probe_counter);
		if (lb == -1)
			return;
		int32_t r2 = lut_full_lookup(T, lb, hx);
		if (r2 == -1)
			return;
		Onb onb = onb_from_normal(hn);
		f3 local_wi = normalize(onb.inv_local(Ld_wi));
		int32_t probe = T.refs[(size_t)lb * KGR_LUT_REFS + r2];
		mb.rec_bin[2 * index + 1] = probe * KGR_PROBE_BINS + bin_of(local_wi);
		mb.rec_val[2 * index + 1] = f4_of(Ld, Ld_depth);
	}
}

/* secondary_gather, second half: the splats added to their bins -- the
 * radiance in fixed point, one count each, and the depth of the last splat
 * in splat order (the largest stamp). */
__global__ void gather_apply_kernel(MambaParams mp, MambaBuffers mb)
{
	uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
	if (r >= 2 * mp.sec_w * mp.sec_h)
		return;
	int32_t bin = mb.rec_bin[r];
	if (bin < 0)
		return;
	float4 v = mb.rec_val[r];
	const MambaTable &T = mb.table;
	atomicAdd(&T.bin_le[3 * (size_t)bin + 0], (unsigned long long)to_fixed(v.x));
	atomicAdd(&T.bin_le[3 * (size_t)bin + 1], (unsigned long long)to_fixed(v.y));
	atomicAdd(&T.bin_le[3 * (size_t)bin + 2], (unsigned long long)to_fixed(v.z));
	atomicAdd(&T.bin_n[bin], 1u);
	unsigned long long key = ((unsigned long long)(mp.stamp_base + r + 1u) << 32) | __float_as_uint(v.w);
	atomicMax(&T.bin_depth[bin], key);
}

/* sobel_normal (mamba.cu:169-201): the sum of |n - n'| over the 3x3
 * neighbourhood, in the reference's loop order (its rows run bottom up) */
__global__ void sobel_kernel(MambaParams mp, MambaBuffers mb)
{
	uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
	if (pix >= mp.npix)
		return;
	int W = (int)mp.width, H = (int)mp.height;
	int x = (int)(pix % mp.width), y = (int)(pix / mp.width);
	int ys = H - (y + 1);
	f3 n = f3_of(mb.g_normal[pix]);
	float acc = 0.0f;
	for (int i = -1; i <= 1; i++) {
		for (int j = -1; j <= 1; j++) {
			int x2 = x + i, y2s = ys + j;
			if (x2 < 0 || x2 >= W || y2s < 0 || y2s >= H)
				continue;
			int y2 = H - (y2s + 1);
			acc += length(n - f3_of(mb.g_normal[(uint32_t)(y2 * W + x2)]));
		}
	}
	mb.sobel[pix] = acc;
}

/* raster_probes (mamba.cu:244-369): the probe nearest each pixel's
 * position and whether the pixel lies within its disk; pixels outside the
 * table keep their values. */
__global__ void __launch_bounds__(128) raster_kernel(MambaParams mp, MambaBuffers mb)
{
	uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
	if (pix >= mp.npix)
		return;
	const MambaTable &T = mb.table;
	f3 position = f3_of(mb.g_position[pix]);
	int32_t l = table_of(T, position, T.counters[0]);
	if (l == -1)
		return;
	MambaLut L = load_lut(T, l);
	size_t base = (size_t)l * KGR_LUT_REFS;
	float closest = FLT_MAX;
	int32_t closest_index = -1;
	for (int ni = -1; ni < 27; ni++) {
		int32_t r = lut_lookup(T, l, L, position, ni);
		if (r == -1)
			continue;
		int32_t p = T.refs[base + r];
		float dist = length(position - f3_of(T.probe_pos[p]));
		if (dist < closest) {
			closest = dist;
			closest_index = p;
		}
	}
	float v = 0.0f;
	f3 indicator = mk((float)(l % 2)), radiance = mk((float)(l % 2));
	int32_t probe_index = -1;
	if (closest_index != -1) {
		probe_index = closest_index;
		f3 diff = position - f3_of(T.probe_pos[probe_index]);
		Onb onb = onb_from_normal(f3_of(T.probe_nrm[probe_index]));
		f3 local = onb.inv_local(diff) / L.resolution;
		local.z = 0.0f;
		float dist = length(local);
		if (dist < 1.0f) {
			v = 1.0f;
			if (mp.render_probes || mp.render_probe_radiance) {
				f3 wi = normalize(mk(local.x, local.y, ksqrt(1.0f - local.x * local.x - local.y * local.y)));
				int32_t idx = bin_of(wi);
				if (mp.render_probes) {
					float su, sv;
					to_disk(wi, su, sv);
					int32_t ix = (int32_t)(su * (float)MAMBA_SIZE), iy = (int32_t)(sv * (float)MAMBA_SIZE);
					int32_t mod = (ix + iy) % 2;
					int32_t c = probe_index % 12;
					indicator = mk(c_color_wheel[c][0], c_color_wheel[c][1], c_color_wheel[c][2])
						* (0.5f + 0.5f * (float)mod);
				} else {
					size_t b = (size_t)probe_index * KGR_PROBE_BINS + idx;
					float n = (float)T.bin_n[b];
					radiance = n > 0.0f ? bin_radiance(T, b) / n : mk(0.0f);
				}
			}
		}
	}
	mb.raster[pix] = v;
	mb.raster_indicator[pix] = f4_of(indicator, 0.0f);
	mb.raster_radiance[pix] = f4_of(radiance, 0.0f);
	mb.probe_ids[pix] = probe_index;
}

/* probe_collapse (mamba.cu:889-938): up to four distinct probe ids per
 * 16x16 group, in column-major scan order */
__global__ void collapse_kernel(MambaParams mp, MambaBuffers mb)
{
	uint32_t gw = (mp.width + 15) / 16, gh = (mp.height + 15) / 16;
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= gw * gh)
		return;
	uint32_t x16 = i % gw, y16 = i / gw;
	int32_t dst[4] = {-1, -1, -1, -1};
	int32_t size = 0;
	for (uint32_t xoff = 0; xoff < 16; xoff++) {
		for (uint32_t yoff = 0; yoff < 16; yoff++) {
			if (size >= 4)
				break;
			uint32_t x = x16 * 16 + xoff, y = y16 * 16 + yoff;
			if (x >= mp.width || y >= mp.height)
				continue;
			int32_t id = mb.probe_ids[y * mp.width + x];
			bool dup = false;
			for (int32_t j = 0; j < size; j++)
				if (dst[j] == id) {
					dup = true;
					break;
				}
			if (!dup)
				dst[size++] = id;
		}
	}
	mb.group_probes[i] = make_int4(dst[0], dst[1], dst[2], dst[3]);
	mb.group_sizes[i] = size;
}

/* probe_allocation (mamba_kernels.cu:5-98), the part that reads only: each
 * 16x16 block less than 60% covered picks the uncovered pixel farthest
 * (within +-2) from a covered one, or its centre.  Blocks whose allocation
 * would change nothing -- a miss, a point outside the top table, or a
 * second-level cell whose two slots were already taken -- drop out here;
 * the rest are allocated in block order by alloc_serial_kernel. */
__global__ void alloc_candidates_kernel(MambaParams mp, MambaBuffers mb)
{
	int W = (int)mp.width, H = (int)mp.height;
	int bw = W / 16, bh = H / 16;
	int b = (int)(blockIdx.x * blockDim.x + threadIdx.x);
	if (b >= bw * bh)
		return;
	int x = b % bw, y = b / bw;
	int x2 = x * 16, y2 = y * 16;
	int misses = 0, best_distance = 0;
	int x_best = x2 + 8, y_best = y2 + 8;
	for (int i = 0; i < 16; i++) {
		for (int j = 0; j < 16; j++) {
			int x3 = x2 + i, y3 = y2 + j;
			if (mb.raster[y3 * W + x3] != 0.0f)
				continue;
			int distance = 0;
			for (int k = -2; k <= 2; k++) {
				for (int l = -2; l <= 2; l++) {
					int x4 = x3 + k, y4 = y3 + l;
					if (x4 < 0 || x4 >= W || y4 < 0 || y4 >= H)
						continue;
					if (mb.raster[y4 * W + x4] == 0.0f)
						continue;
					int m = abs(k) + abs(l);
					distance = m > distance ? m : distance;
				}
			}
			if (distance > best_distance) {
				best_distance = distance;
				x_best = x3;
				y_best = y3;
			}
			misses++;
		}
	}
	mb.cand_flag[b] = 0;
	if ((double)misses < 0.4 * 16 * 16)
		return;
	if (misses == 16 * 16) {
		x_best = x2 + 8;
		y_best = y2 + 8;
	}
	uint32_t pix = (uint32_t)(y_best * W + x_best);
	if (mb.g_index[pix] == -1)
		return;
	const MambaTable &T = mb.table;
	f3 position = f3_of(mb.g_position[pix]);
	MambaLut top = load_lut(T, 0);
	if (!lut_contains(top, position, false))
		return;
	int32_t r = top_lookup(T, position);
	if (r != -1) {
		int32_t l = T.refs[r];
		MambaLut L = load_lut(T, l);
		uint32_t h = lut_hash(L, position, 0, 0, 0);
		size_t base = (size_t)l * KGR_LUT_REFS;
		if (T.refs[base + h % (uint32_t)KGR_LUT_REFS] != -1 && T.refs[base + (h + 1u) % (uint32_t)KGR_LUT_REFS] != -1)
			return;
	}
	mb.cand_flag[b] = 1;
	mb.cand_pixel[b] = make_int2(x_best, y_best);
}

/* request_L2 + lookup-table allocation + request_L1 + probe allocation of
 * one candidate (probe.cuh:560-676, :522-558; mamba_kernels.cu:100-182). */
__device__ void allocate_probe(const MambaParams &mp, const MambaBuffers &mb, int2 px)
{
	const MambaTable &T = mb.table;
	uint32_t pix = (uint32_t)(px.y * (int)mp.width + px.x);
	f3 position = f3_of(mb.g_position[pix]);
	f3 normal = f3_of(mb.g_normal[pix]);
	MambaLut top = T.luts[0];
	uint32_t h = lut_hash(top, position, 0, 0, 0);
	int32_t idx = -1;
	bool created = false;
	f3 half = mk(0.5f * top.resolution);
	for (int i = 0; i < KGR_LUT_REFS; i++) {
		uint32_t j = (h + (uint32_t)i) % (uint32_t)KGR_LUT_REFS;
		if (T.refs[j] == -1) {
			if (T.counters[1] >= T.max_luts)
				break; /* no second-level table left: nothing is claimed */
			float cdx = position.x - top.center[0] + top.size / 2.0f;
			float cdy = position.y - top.center[1] + top.size / 2.0f;
			float cdz = position.z - top.center[2] + top.size / 2.0f;
			int32_t ix = (int32_t)(cdx / top.resolution);
			int32_t iy = (int32_t)(cdy / top.resolution);
			int32_t iz = (int32_t)(cdz / top.resolution);
			f3 c = mk(top.center[0] + ((float)ix + 0.5f) * top.resolution - top.size / 2.0f,
				top.center[1] + ((float)iy + 0.5f) * top.resolution - top.size / 2.0f,
				top.center[2] + ((float)iz + 0.5f) * top.resolution - top.size / 2.0f);
			T.hashes[j] = h;
			T.positions[j] = f4_of(c, 0.0f);
			T.luts[0].counter++;
			int32_t l = T.counters[1]++;
			MambaLut nl;
			nl.center[0] = c.x;
			nl.center[1] = c.y;
			nl.center[2] = c.z;
			nl.size = MAMBA_L1_SIZE;
			nl.resolution = MAMBA_L1_SIZE / MAMBA_DIVISION;
			nl.level = 1;
			nl.counter = 0;
			nl.pad = 0;
			T.luts[l] = nl;
			T.refs[j] = l;
			idx = (int32_t)j;
			created = true;
			break;
		}
		f3 c = f3_of(T.positions[j]);
		f3 mn = c - half, mx = c + half;
		if ((position.x <= mx.x && position.y <= mx.y && position.z <= mx.z)
			&& (position.x >= mn.x && position.y >= mn.y && position.z >= mn.z)) {
			idx = (int32_t)j;
			break;
		}
	}
	(void)created;
	if (idx == -1)
		return;
	if (T.counters[0] >= T.max_probes)
		return;
	int32_t l = T.refs[idx];
	MambaLut L = T.luts[l];
	uint32_t h1 = lut_hash(L, position, 0, 0, 0);
	size_t base = (size_t)l * KGR_LUT_REFS;
	int32_t slot = -1;
	for (int t = 0; t < 2; t++) {
		uint32_t j = (h1 + (uint32_t)(t * t)) % (uint32_t)KGR_LUT_REFS;
		if (T.refs[base + j] == -1) {
			slot = (int32_t)j;
			break;
		}
	}
	if (slot == -1)
		return;
	T.hashes[base + slot] = h1;
	T.positions[base + slot] = f4_of(position, 0.0f);
	T.luts[l].counter++;
	int32_t p = T.counters[0]++;
	T.probe_pos[p] = f4_of(position, 0.0f);
	T.probe_nrm[p] = f4_of(normal, 0.0f);
	T.refs[base + slot] = p;
}

/* One block of 1024 threads: the candidates compacted in block order, then
 * allocated one after another by thread 0 (each allocation may depend on
 * the ones before it). */
__global__ void __launch_bounds__(1024) alloc_serial_kernel(MambaParams mp, MambaBuffers mb, int nblocks)
{
	__shared__ int warp_sums[32];
	__shared__ int base;
	int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	if (tid == 0)
		base = 0;
	__syncthreads();
	for (int start = 0; start < nblocks; start += 1024) {
		int i = start + tid;
		int f = (i < nblocks) ? mb.cand_flag[i] : 0;
		unsigned ballot = __ballot_sync(0xffffffffu, f != 0);
		int before = __popc(ballot & ((1u << lane) - 1u));
		if (lane == 0)
			warp_sums[warp] = __popc(ballot);
		__syncthreads();
		if (warp == 0) {
			int v = warp_sums[lane];
			for (int o = 1; o < 32; o <<= 1) {
				int t = __shfl_up_sync(0xffffffffu, v, o);
				if (lane >= o)
					v += t;
			}
			warp_sums[lane] = v;
		}
		__syncthreads();
		int wbase = warp ? warp_sums[warp - 1] : 0;
		if (f)
			mb.cand_list[base + wbase + before] = i;
		__syncthreads();
		if (tid == 0)
			base += warp_sums[31];
		__syncthreads();
	}
	if (tid != 0)
		return;
	__threadfence();
	for (int c = 0; c < base; c++)
		allocate_probe(mp, mb, mb.cand_pixel[mb.cand_list[c]]);
}

/* final_gather (mamba.cu:686-878) */
__global__ void __launch_bounds__(128) final_gather_kernel(DeviceScene s, MambaParams mp, MambaBuffers mb,
		float4 *color)
{
	uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
	if (pix >= mp.npix)
		return;
	uint32_t x = pix % mp.width, y = pix / mp.width;
	SurfaceHit sh;
	if (!load_surface(mp, mb, s.materials, pix, sh)) {
		color[pix] = sky_at(s, ray_at(mp, x, y));
		return;
	}
	f3 c = sh.mat.emission + (float)(mp.direct_lighting != 0) * f3_of(mb.direct_Le[pix]) + mk(0.0f);
	f3 covered = mk(0.0f);
	if (mp.render_probes || mp.render_probe_radiance)
		covered = f3_of(mp.render_probes ? mb.raster_indicator[pix] : mb.raster_radiance[pix]);
	uint32_t sidx = x / 4 + (y / 4) * mp.sec_w;
	f3 sec = mk(0.0f);
	if (sidx < mp.sec_w * mp.sec_h && mp.indirect_lighting) {
		sec = f3_of(mb.s_Le[sidx]);
	} else if (mp.irradiance) {
		const MambaTable &T = mb.table;
		int32_t l = table_of(T, sh.x, T.counters[0]);
		if (l != -1) {
			int32_t closest[2] = {-1, -1};
			float distance[2] = {FLT_MAX, FLT_MAX};
			lut_closest2(T, l, sh.x, closest, distance);
			if (closest[0] != -1) {
				f3 sum = mk(0.0f);
				int32_t count = 0;
				for (int i = 0; i < 2; i++) {
					if (closest[i] == -1)
						break;
					int32_t p = T.refs[(size_t)l * KGR_LUT_REFS + closest[i]];
					f3 ppos = f3_of(T.probe_pos[p]), pn = f3_of(T.probe_nrm[p]);
					Onb onb = onb_from_normal(pn);
					for (int j = 0; j < KGR_PROBE_BINS; j++) {
						f3 probe_wo = onb.local(mk(mp.bin_dir[j][0], mp.bin_dir[j][1], mp.bin_dir[j][2]));
						/* the reference scales the bin's direction by its index, not its depth */
						f3 wo = normalize(((float)j * probe_wo + ppos) - sh.x);
						if (dot(wo, sh.n) <= 0.0f)
							continue;
						size_t b = (size_t)p * KGR_PROBE_BINS + j;
						uint32_t nb = T.bin_n[b];
						if (nb == 0)
							continue; /* adds an exact zero to a non-negative sum */
						float geometric = kmax(dot(wo, sh.n), 0.0f);
						f3 f;
						float pdf;
						m_brdf_pdf(sh, wo, f, pdf);
						f = cleanse(f);
						f = pdf > 0.0f ? f / pdf : mk(0.0f);
						f3 le = cleanse(bin_radiance(T, b));
						float n = (float)nb;
						sum = sum + (le / n) * f * fabsf(dot(wo, pn)) * geometric;
					}
					count++;
				}
				sec = sum / (float)(count * KGR_PROBE_BINS);
			}
		}
	}
	color[pix] = f4_of(c + sec + covered, 1.0f);
}

__global__ void table_header_kernel(MambaTable t)
{
	MambaLut top;
	top.center[0] = top.center[1] = top.center[2] = 0.0f;
	top.size = MAMBA_TOP_SIZE;
	top.resolution = MAMBA_TOP_SIZE / MAMBA_DIVISION;
	top.level = 2;
	top.counter = 0;
	top.pad = 0;
	t.luts[0] = top;
	t.counters[0] = 0;
	t.counters[1] = 1;
}

__global__ void restamp_kernel(MambaTable t, size_t n)
{
	size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
	if (i < n)
		t.bin_depth[i] &= 0xFFFFFFFFull;
}

inline uint32_t blocks_for(uint32_t n, uint32_t b)
{
	return (n + b - 1) / b;
}

} /* namespace */

void mamba_bin_directions(float out[KGR_PROBE_BINS][3])
{
	for (int index = 0; index < KGR_PROBE_BINS; index++) {
		/* from_index: uv = clamp((x, y) / size, 0, 1); from_uv: theta =
		 * 2 uv.x M_PI (double), x = uv.y cos(theta), y = uv.y sin(theta)
		 * in double, z = sqrt(1 - x^2 - y^2) in float */
		int x = index % MAMBA_SIZE, y = index / MAMBA_SIZE;
		float u = (float)x / (float)MAMBA_SIZE, v = (float)y / (float)MAMBA_SIZE;
		u = u < 0.0f ? 0.0f : (u > 1.0f ? 1.0f : u);
		v = v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v);
		double theta = (double)(2.0f * u) * MAMBA_PI_D;
		float dx = (float)((double)v * cos(theta));
		float dy = (float)((double)v * sin(theta));
		float dz = sqrtf(1.0f - dx * dx - dy * dy);
		out[index][0] = dx;
		out[index][1] = dy;
		out[index][2] = dz;
	}
}

namespace {

struct BufferSizes {
	size_t npix, nsec, groups, blocks, slots, bins;
};

BufferSizes buffer_sizes(uint32_t width, uint32_t height, int32_t max_probes, int32_t max_luts)
{
	BufferSizes z;
	z.npix = (size_t)width * height;
	z.nsec = (size_t)(width / 4 + 1) * (height / 4 + 1);
	z.groups = (size_t)((width + 15) / 16) * ((height + 15) / 16);
	z.blocks = (size_t)(width / 16) * (height / 16);
	if (z.blocks == 0)
		z.blocks = 1;
	z.slots = (size_t)max_luts * KGR_LUT_REFS;
	z.bins = (size_t)max_probes * KGR_PROBE_BINS;
	return z;
}

/* Calls f(pointer-to-member-pointer, bytes) for every per-pixel and
 * per-secondary buffer. */
template <class F>
void for_each_frame_buffer(MambaBuffers &mb, const BufferSizes &z, F f)
{
	f((void **)&mb.g_position, sizeof(float4) * z.npix);
	f((void **)&mb.g_normal, sizeof(float4) * z.npix);
	f((void **)&mb.g_index, sizeof(int32_t) * z.npix);
	for (int k = 0; k < 2; k++) {
		for (MambaReservoirs *r : {&mb.res[k], &mb.prev[k]}) {
			f((void **)&r->r0, sizeof(float4) * z.npix);
			f((void **)&r->r1, sizeof(float4) * z.npix);
			f((void **)&r->r2, sizeof(float4) * z.npix);
			f((void **)&r->r3, sizeof(float4) * z.npix);
		}
	}
	f((void **)&mb.direct_Le, sizeof(float4) * z.npix);
	f((void **)&mb.vis_o, sizeof(float4) * 3 * z.npix);
	f((void **)&mb.vis_d, sizeof(float4) * 3 * z.npix);
	f((void **)&mb.vis_flag, sizeof(uint32_t) * 3 * z.npix);
	f((void **)&mb.vis_queue, sizeof(uint32_t) * 3 * z.npix);
	f((void **)&mb.vis_counters, sizeof(uint32_t) * CNT_COUNT);
	f((void **)&mb.spatial_aux, sizeof(int4) * z.npix);
	for (float4 **b : {&mb.s_wi, &mb.s_Le, &mb.s_Ld, &mb.s_Ld_wi, &mb.s_hit_x, &mb.s_hit_n, &mb.s_hit_wo})
		f((void **)b, sizeof(float4) * z.nsec);
	f((void **)&mb.s_hit_mat, sizeof(int32_t) * z.nsec);
	f((void **)&mb.rec_bin, sizeof(int32_t) * 2 * z.nsec);
	f((void **)&mb.rec_val, sizeof(float4) * 2 * z.nsec);
	f((void **)&mb.sobel, sizeof(float) * z.npix);
	f((void **)&mb.raster, sizeof(float) * z.npix);
	f((void **)&mb.raster_indicator, sizeof(float4) * z.npix);
	f((void **)&mb.raster_radiance, sizeof(float4) * z.npix);
	f((void **)&mb.probe_ids, sizeof(int32_t) * z.npix);
	f((void **)&mb.group_probes, sizeof(int4) * z.groups);
	f((void **)&mb.group_sizes, sizeof(int32_t) * z.groups);
	f((void **)&mb.cand_flag, sizeof(int32_t) * z.blocks);
	f((void **)&mb.cand_pixel, sizeof(int2) * z.blocks);
	f((void **)&mb.cand_list, sizeof(int32_t) * z.blocks);
}

template <class F>
void for_each_table_buffer(MambaTable &t, const BufferSizes &z, F f)
{
	f((void **)&t.luts, sizeof(MambaLut) * (size_t)t.max_luts);
	f((void **)&t.refs, sizeof(int32_t) * z.slots);
	f((void **)&t.hashes, sizeof(uint32_t) * z.slots);
	f((void **)&t.positions, sizeof(float4) * z.slots);
	f((void **)&t.probe_pos, sizeof(float4) * (size_t)t.max_probes);
	f((void **)&t.probe_nrm, sizeof(float4) * (size_t)t.max_probes);
	f((void **)&t.bin_le, sizeof(unsigned long long) * 3 * z.bins);
	f((void **)&t.bin_n, sizeof(uint32_t) * z.bins);
	f((void **)&t.bin_depth, sizeof(unsigned long long) * z.bins);
	f((void **)&t.counters, sizeof(int32_t) * 2);
}

} /* namespace */

void mamba_alloc(MambaBuffers &mb, uint32_t width, uint32_t height, int32_t max_probes, int32_t max_luts)
{
	KGR_REQUIRE(max_probes >= 1 && max_probes <= (1 << 24), KGR_ERR_INVALID_ARGUMENT, "max_probes must be 1..2^24");
	KGR_REQUIRE(max_luts >= 2 && max_luts <= 4096, KGR_ERR_INVALID_ARGUMENT, "max_luts must be 2..4096");
	memset(&mb, 0, sizeof(mb));
	mb.table.max_probes = max_probes;
	mb.table.max_luts = max_luts;
	BufferSizes z = buffer_sizes(width, height, max_probes, max_luts);
	auto grab = [&](void **p, size_t bytes) {
		if (cudaMalloc(p, bytes) != cudaSuccess) {
			cudaGetLastError();
			*p = nullptr;
			mamba_free(mb);
			throw Error(KGR_ERR_OUT_OF_MEMORY, "cudaMalloc of the mamba buffers failed");
		}
	};
	for_each_frame_buffer(mb, z, grab);
	for_each_table_buffer(mb.table, z, grab);
	mamba_reset(mb, width, height, 0);
	KGR_CUDA(cudaStreamSynchronize(0));
}

void mamba_free(MambaBuffers &mb)
{
	BufferSizes z = buffer_sizes(1, 1, 1, 2);
	auto drop = [](void **p, size_t) {
		if (*p)
			cudaFree(*p);
		*p = nullptr;
	};
	for_each_frame_buffer(mb, z, drop);
	for_each_table_buffer(mb.table, z, drop);
}

void mamba_reset(const MambaBuffers &mb0, uint32_t width, uint32_t height, cudaStream_t st)
{
	MambaBuffers mb = mb0;
	BufferSizes z = buffer_sizes(width, height, mb.table.max_probes, mb.table.max_luts);
	auto zero = [&](void **p, size_t bytes) { KGR_CUDA(cudaMemsetAsync(*p, 0, bytes, st)); };
	for_each_frame_buffer(mb, z, zero);
	mamba_table_clear(mb.table, st);
}

bool mamba_buffer(const MambaBuffers &mb0, int res_in, int prev_in, uint32_t width, uint32_t height,
		const char *name, const void **ptr, size_t *bytes)
{
	MambaBuffers mb = mb0;
	BufferSizes z = buffer_sizes(width, height, mb.table.max_probes, mb.table.max_luts);
	std::string n(name);
	const MambaReservoirs &R = mb.res[res_in], &P = mb.prev[prev_in];
	struct Entry {
		const char *name;
		const void *p;
		size_t bytes;
	} entries[] = {
		{"g_position", mb.g_position, sizeof(float4) * z.npix}, {"g_normal", mb.g_normal, sizeof(float4) * z.npix},
		{"g_index", mb.g_index, sizeof(int32_t) * z.npix}, {"direct_le", mb.direct_Le, sizeof(float4) * z.npix},
		{"res_r0", R.r0, sizeof(float4) * z.npix}, {"res_r1", R.r1, sizeof(float4) * z.npix},
		{"res_r2", R.r2, sizeof(float4) * z.npix}, {"res_r3", R.r3, sizeof(float4) * z.npix},
		{"prev_r0", P.r0, sizeof(float4) * z.npix}, {"prev_r1", P.r1, sizeof(float4) * z.npix},
		{"prev_r2", P.r2, sizeof(float4) * z.npix}, {"prev_r3", P.r3, sizeof(float4) * z.npix},
		{"s_wi", mb.s_wi, sizeof(float4) * z.nsec}, {"s_le", mb.s_Le, sizeof(float4) * z.nsec},
		{"s_ld", mb.s_Ld, sizeof(float4) * z.nsec}, {"s_ld_wi", mb.s_Ld_wi, sizeof(float4) * z.nsec},
		{"s_hit_x", mb.s_hit_x, sizeof(float4) * z.nsec}, {"s_hit_n", mb.s_hit_n, sizeof(float4) * z.nsec},
		{"s_hit_wo", mb.s_hit_wo, sizeof(float4) * z.nsec}, {"s_hit_mat", mb.s_hit_mat, sizeof(int32_t) * z.nsec},
		{"sobel", mb.sobel, sizeof(float) * z.npix}, {"raster", mb.raster, sizeof(float) * z.npix},
		{"raster_indicator", mb.raster_indicator, sizeof(float4) * z.npix},
		{"raster_radiance", mb.raster_radiance, sizeof(float4) * z.npix},
		{"probe_ids", mb.probe_ids, sizeof(int32_t) * z.npix},
		{"group_probes", mb.group_probes, sizeof(int4) * z.groups},
		{"group_sizes", mb.group_sizes, sizeof(int32_t) * z.groups},
		{"counters", mb.table.counters, sizeof(int32_t) * 2},
		{"luts", mb.table.luts, sizeof(MambaLut) * (size_t)mb.table.max_luts},
		{"refs", mb.table.refs, sizeof(int32_t) * z.slots}, {"hashes", mb.table.hashes, sizeof(uint32_t) * z.slots},
		{"lut_positions", mb.table.positions, sizeof(float4) * z.slots},
		{"probe_pos", mb.table.probe_pos, sizeof(float4) * (size_t)mb.table.max_probes},
		{"probe_nrm", mb.table.probe_nrm, sizeof(float4) * (size_t)mb.table.max_probes},
		{"bin_le", mb.table.bin_le, sizeof(unsigned long long) * 3 * z.bins},
		{"bin_n", mb.table.bin_n, sizeof(uint32_t) * z.bins},
		{"bin_depth", mb.table.bin_depth, sizeof(unsigned long long) * z.bins},
	};
	for (const Entry &e : entries) {
		if (n == e.name) {
			*ptr = e.p;
			*bytes = e.bytes;
			return true;
		}
	}
	return false;
}

void mamba_table_clear(const MambaTable &t, cudaStream_t st)
{
	size_t slots = (size_t)t.max_luts * KGR_LUT_REFS;
	size_t bins = (size_t)t.max_probes * KGR_PROBE_BINS;
	KGR_CUDA(cudaMemsetAsync(t.luts, 0, sizeof(MambaLut) * (size_t)t.max_luts, st));
	KGR_CUDA(cudaMemsetAsync(t.refs, 0xff, sizeof(int32_t) * slots, st));
	KGR_CUDA(cudaMemsetAsync(t.hashes, 0xff, sizeof(uint32_t) * slots, st));
	KGR_CUDA(cudaMemsetAsync(t.positions, 0, sizeof(float4) * slots, st));
	KGR_CUDA(cudaMemsetAsync(t.probe_pos, 0, sizeof(float4) * (size_t)t.max_probes, st));
	KGR_CUDA(cudaMemsetAsync(t.probe_nrm, 0, sizeof(float4) * (size_t)t.max_probes, st));
	KGR_CUDA(cudaMemsetAsync(t.bin_le, 0, sizeof(unsigned long long) * 3 * bins, st));
	KGR_CUDA(cudaMemsetAsync(t.bin_n, 0, sizeof(uint32_t) * bins, st));
	KGR_CUDA(cudaMemsetAsync(t.bin_depth, 0, sizeof(unsigned long long) * bins, st));
	table_header_kernel<<<1, 1, 0, st>>>(t);
	KGR_CUDA(cudaGetLastError());
}

void mamba_restamp(const MambaTable &t, cudaStream_t st)
{
	size_t n = (size_t)t.max_probes * KGR_PROBE_BINS;
	restamp_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(t, n);
	KGR_CUDA(cudaGetLastError());
}

uint32_t mamba_render(const DeviceScene &s, const PathBuffers &pb, const MambaParams &mp, const MambaBuffers &mb,
		const TraceTune &tune, float4 *color, cudaStream_t st, const StageMark &mark)
{
	auto done = [&](int stage) {
		KGR_CUDA(cudaGetLastError());
		if (mark)
			mark(stage);
	};
	const uint32_t npix = mp.npix, nsec = mp.sec_w * mp.sec_h;
	uint32_t launches = 0;
	gbuffer_rays_kernel<<<blocks_for(npix, 256), 256, 0, st>>>(pb, mp);
	done(STAGE_GENERATE);
	pt_trace_closest(s, pb, 0, mp.layout, tune, st);
	done(STAGE_TRACE_CLOSEST);
	gbuffer_store_kernel<<<blocks_for(npix, 256), 256, 0, st>>>(s, pb, mp, mb);
	done(STAGE_GENERATE);
	launches += 3;
	if (mp.direct_lighting) {
		const unsigned grid = blocks_for(npix, 128);
		PathBuffers vb = pb;
		vb.sh_o = mb.vis_o;
		vb.sh_d = mb.vis_d;
		vb.shadow_queue = mb.vis_queue;
		vb.counters = mb.vis_counters;
		vb.shadow_flags = mb.vis_flag;
		vb.capacity = 3 * npix;
		auto rays = [&](int stage) {
			pt_shadow_resolve(s, vb, mp.layout, tune, st);
			done(stage);
			launches++;
		};
		auto clear_queue = [&]() { KGR_CUDA(cudaMemsetAsync(mb.vis_counters, 0, CNT_COUNT * sizeof(uint32_t), st)); };
		clear_queue();
		primary_ris_kernel<<<grid, 128, 0, st>>>(s, mp, mb);
		done(STAGE_RESTIR_PRIMARY);
		rays(STAGE_RESTIR_PRIMARY);
		primary_finish_kernel<<<grid, 128, 0, st>>>(s, mp, mb);
		done(STAGE_RESTIR_PRIMARY);
		launches += 2;
		if (mp.temporal) {
			clear_queue();
			temporal_gather_kernel<<<grid, 128, 0, st>>>(s, mp, mb);
			done(STAGE_RESTIR_TEMPORAL);
			rays(STAGE_RESTIR_TEMPORAL_VIS);
			clear_queue();
			temporal_merge_kernel<<<grid, 128, 0, st>>>(s, mp, mb);
			done(STAGE_RESTIR_TEMPORAL);
			launches += 2;
			if (!mp.spatial) {
				rays(STAGE_RESTIR_TEMPORAL_VIS);
				temporal_finish_kernel<<<grid, 128, 0, st>>>(s, mp, mb);
				done(STAGE_RESTIR_TEMPORAL);
				launches++;
			}
		}
		if (mp.spatial) {
			clear_queue();
			spatial_gather_kernel<<<grid, 128, 0, st>>>(s, mp, mb);
			done(STAGE_RESTIR_SPATIAL);
			rays(STAGE_RESTIR_SPATIAL_VIS);
			clear_queue();
			spatial_resample_kernel<<<grid, 128, 0, st>>>(s, mp, mb);
			done(STAGE_RESTIR_SPATIAL);
			rays(STAGE_RESTIR_SPATIAL_VIS);
			spatial_finish_kernel<<<grid, 128, 0, st>>>(s, mp, mb);
			done(STAGE_RESTIR_SPATIAL);
			launches += 3;
		}
	}
	secondary_kernel<<<blocks_for(nsec, 128), 128, 0, st>>>(s, mp, mb);
	done(STAGE_MAMBA_SECONDARY);
	gather_splat_kernel<<<blocks_for(nsec, 128), 128, 0, st>>>(s, mp, mb);
	gather_apply_kernel<<<blocks_for(2 * nsec, 256), 256, 0, st>>>(mp, mb);
	done(STAGE_MAMBA_GATHER);
	sobel_kernel<<<blocks_for(npix, 256), 256, 0, st>>>(mp, mb);
	raster_kernel<<<blocks_for(npix, 128), 128, 0, st>>>(mp, mb);
	uint32_t groups = ((mp.width + 15) / 16) * ((mp.height + 15) / 16);
	collapse_kernel<<<blocks_for(groups, 128), 128, 0, st>>>(mp, mb);
	int nblocks = (int)((mp.width / 16) * (mp.height / 16));
	if (nblocks > 0) {
		alloc_candidates_kernel<<<blocks_for((uint32_t)nblocks, 64), 64, 0, st>>>(mp, mb);
		alloc_serial_kernel<<<1, 1024, 0, st>>>(mp, mb, nblocks);
		launches += 2;
	}
	done(STAGE_MAMBA_PROBES);
	final_gather_kernel<<<blocks_for(npix, 128), 128, 0, st>>>(s, mp, mb, color);
	done(STAGE_MAMBA_FINAL);
	launches += 7;
	return launches;
}

} /* namespace kgr */

/*
 * post.cu -- what follows the accumulated frame: HDR -> LDR tonemapping and
 * an AOV-guided denoiser.
 *
 * Tonemapping follows include/cuda/color.cuh of the reference: aces()
 * (:33-39), srgb() (:13-30), quantize_unsigned_8_bits() (:42-55),
 * make_color() (:57-66) and cast.cuh to_ui32() (:16-20), with the vertical
 * flip of hdr_to_ldr_kernel (:84-103).  ACES is plain IEEE arithmetic and
 * matches the reference bit for bit; sRGB calls powf, whose last bit can
 * differ from the host C library's.
 *
 * The reference denoises with the OptiX AI denoiser (source/layers/
 * denoiser.cu:9-149), a closed library; this is a filter of its own: the
 * edge-avoiding a-trous wavelet transform (Dammertz et al., "Edge-Avoiding
 * A-Trous Wavelet Transform for fast Global Illumination Filtering", HPG
 * 2010).  Pass i (i = 0 .. iterations-1) convolves with the 5 x 5 B3-spline
 * kernel (1/16, 1/4, 3/8, 1/4, 1/16 in each direction) spread by a step of
 * 2^i pixels, each tap weighted by three edge-stopping functions between the
 * centre p and the tap q:
 *   colour    exp(-|l_p - l_q| / (sigma_color 2^-i (l_p + l_q) / 2 + 1e-4)),
 *             l = luminance of the demodulated value (relative, so HDR
 *             radiance of any scale filters the same way)
 *   normal    max(0, n_p . n_q) ^ normal_power
 *   position  exp(-d / sigma_position), d = |n_p . (x_q - x_p)| / |x_q - x_p|,
 *             the distance of q off p's tangent plane per unit of separation
 *             (scale free)
 * With the albedo guide the filter works on colour / albedo' (albedo'
 * = albedo where a channel exceeds 1e-3, else 1) and multiplies back at the
 * end, so texture and material detail is not blurred.  Pixels without a hit
 * (zero normal) only average among themselves.
 */
#include "kgr_post.h"

namespace kgr {

namespace {

__device__ __forceinline__ float clamp_ref(float f, float a, float b) { return fmaxf(a, fminf(f, b)); }

/* aces (color.cuh:33-39) */
__device__ __forceinline__ float aces1(float c)
{
	float a = c * (c * 2.51f + 0.03f);
	float b = c * (c * 2.43f + 0.59f) + 0.14f;
	return clamp_ref(a / b, 0.0f, 1.0f);
}

/* srgb (color.cuh:13-30) */
__device__ __forceinline__ float srgb1(float c)
{
	float powed = powf(c, 1.0f / 2.4f);
	float s = c < 0.0031308f ? 12.92f * c : 1.055f * powed - 0.055f;
	return clamp_ref(s, 0.0f, 1.0f);
}

/* quantize_unsigned_8_bits (color.cuh:42-55) */
__device__ __forceinline__ uint32_t quantize8(float x)
{
	x = clamp_ref(x, 0.0f, 1.0f);
	uint32_t q = (uint32_t)(x * 256.0f);
	return q < 255u ? q : 255u;
}

__global__ void tonemap_kernel(const float4 *__restrict__ hdr, uint32_t *__restrict__ ldr, uint32_t width,
		uint32_t height, int mode)
{
	uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
	uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
	if (x >= width || y >= height)
		return;
	float4 c = hdr[(size_t)y * width + x];
	float r, g, b;
	if (mode == KGR_TONEMAP_ACES) {
		r = aces1(c.x);
		g = aces1(c.y);
		b = aces1(c.z);
	} else {
		r = srgb1(c.x);
		g = srgb1(c.y);
		b = srgb1(c.z);
	}
	/* to_ui32 (cast.cuh:16-20): alpha 255 in the top byte, red in the lowest */
	uint32_t v = (255u << 24) | (quantize8(b) << 16) | (quantize8(g) << 8) | quantize8(r);
	ldr[(size_t)(height - y - 1) * width + x] = v;
}

__device__ __forceinline__ float lum(float3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }

__device__ __forceinline__ float3 f3of(float4 v) { return make_float3(v.x, v.y, v.z); }

__device__ __forceinline__ float3 albedo_div(float4 a)
{
	return make_float3(a.x > 1e-3f ? a.x : 1.0f, a.y > 1e-3f ? a.y : 1.0f, a.z > 1e-3f ? a.z : 1.0f);
}

/* One a-trous pass.  first: read colour and demodulate; last: remodulate. */
__global__ void atrous_kernel(const float4 *__restrict__ in, float4 *__restrict__ out,
		const float4 *__restrict__ normal, const float4 *__restrict__ albedo, const float4 *__restrict__ position,
		uint32_t width, uint32_t height, int step, float sigma_color, float normal_power, float sigma_position,
		int guides, int first, int last)
{
	uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
	uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
	if (x >= width || y >= height)
		return;
	const bool use_albedo = (guides & KGR_DENOISE_ALBEDO) != 0;
	const bool use_normal = (guides & KGR_DENOISE_NORMAL) != 0;
	const bool use_pos = (guides & KGR_DENOISE_POSITION) != 0;
	const float h[5] = {1.0f / 16.0f, 1.0f / 4.0f, 3.0f / 8.0f, 1.0f / 4.0f, 1.0f / 16.0f};
	size_t ip = (size_t)y * width + x;
	float3 np = f3of(normal[ip]);
	float3 xp = f3of(position[ip]);
	bool hit_p = np.x != 0.0f || np.y != 0.0f || np.z != 0.0f;
	float3 cp = f3of(in[ip]);
	if (first && use_albedo) {
		float3 d = albedo_div(albedo[ip]);
		cp = make_float3(cp.x / d.x, cp.y / d.y, cp.z / d.z);
	}
	float lp = lum(cp);
	float3 sum = make_float3(0.0f, 0.0f, 0.0f);
	float wsum = 0.0f;
	for (int dy = -2; dy <= 2; dy++) {
		int qy = (int)y + dy * step;
		if (qy < 0 || qy >= (int)height)
			continue;
		for (int dx = -2; dx <= 2; dx++) {
			int qx = (int)x + dx * step;
			if (qx < 0 || qx >= (int)width)
				continue;
			size_t iq = (size_t)qy * width + qx;
			float3 cq = f3of(in[iq]);
			if (first && use_albedo) {
				float3 d = albedo_div(albedo[iq]);
				cq = make_float3(cq.x / d.x, cq.y / d.y, cq.z / d.z);
			}
			float3 nq = f3of(normal[iq]);
			bool hit_q = nq.x != 0.0f || nq.y != 0.0f || nq.z != 0.0f;
			if (hit_p != hit_q)
				continue;
			float w = h[dx + 2] * h[dy + 2];
			float lq = lum(cq);
			w *= expf(-fabsf(lp - lq) / (sigma_color * 0.5f * (lp + lq) + 1e-4f));
			if (hit_p && use_normal) {
				float c = np.x * nq.x + np.y * nq.y + np.z * nq.z;
				w *= powf(fmaxf(c, 0.0f), normal_power);
			}
			if (hit_p && use_pos && (dx != 0 || dy != 0)) {
				float3 xq = f3of(position[iq]);
				float3 v = make_float3(xq.x - xp.x, xq.y - xp.y, xq.z - xp.z);
				float len = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
				float d = len > 0.0f ? fabsf(np.x * v.x + np.y * v.y + np.z * v.z) / len : 0.0f;
				w *= expf(-d / sigma_position);
			}
			sum.x += w * cq.x;
			sum.y += w * cq.y;
			sum.z += w * cq.z;
			wsum += w;
		}
	}
	float3 r = wsum > 0.0f ? make_float3(sum.x / wsum, sum.y / wsum, sum.z / wsum) : cp;
	if (last && use_albedo) {
		float3 d = albedo_div(albedo[ip]);
		r = make_float3(r.x * d.x, r.y * d.y, r.z * d.z);
	}
	out[ip] = make_float4(r.x, r.y, r.z, in[ip].w);
}

} /* namespace */

void tonemap(const float4 *hdr, uint32_t *ldr, uint32_t width, uint32_t height, int mode, cudaStream_t st)
{
	dim3 block(16, 16);
	dim3 grid((width + 15) / 16, (height + 15) / 16);
	tonemap_kernel<<<grid, block, 0, st>>>(hdr, ldr, width, height, mode);
	KGR_CUDA(cudaGetLastError());
}

void denoise(const float4 *color, const float4 *normal, const float4 *albedo, const float4 *position, float4 *out,
		float4 *scratch, uint32_t width, uint32_t height, const kgr_denoise_params &p, int guides, cudaStream_t st)
{
	dim3 block(16, 16);
	dim3 grid((width + 15) / 16, (height + 15) / 16);
	/* passes alternate between out and scratch so that the last one lands in out */
	const float4 *src = color;
	for (int i = 0; i < p.iterations; i++) {
		bool last = i == p.iterations - 1;
		float4 *dst = ((p.iterations - 1 - i) % 2 == 0) ? out : scratch;
		float sc = p.sigma_color * (1.0f / (float)(1 << i));
		atrous_kernel<<<grid, block, 0, st>>>(src, dst, normal, albedo, position, width, height, 1 << i, sc,
			p.normal_power, p.sigma_position, guides, i == 0, last);
		KGR_CUDA(cudaGetLastError());
		src = dst;
	}
}

} /* namespace kgr */

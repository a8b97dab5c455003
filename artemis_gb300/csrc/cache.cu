/*
 * cache.cu -- the radiance cache in the wavefront path tracer.
 *
 * Render paths trace the camera ray, shade the primary vertex (emission +
 * NEE + BSDF sample) and trace the first bounce; at that secondary vertex
 * they query the network for the radiance it scatters toward the path and
 * stop: L += beta_1 (Le_1 + max(0, cache(x_1))).  Training paths -- a
 * rotating subset of pixels traced as plain paths to the full depth --
 * record at every vertex k >= 1 the network input, the throughput beta_k,
 * the radiance accumulated before the vertex, and its emission; when the
 * paths end, target_k = (L_final - L_before_k) / beta_k - Le_k is the
 * radiance the vertex scattered, and up to 2^16 (input, target) pairs train
 * the network for the next frame.  The plain path tracer stays available
 * (cache off) and is the judge of the cache's error.
 *
 * Network input (64 values) at a vertex x with outgoing direction wo,
 * shading normal n and material m, p = (x - scene_min) / scene_extent:
 *   0-35   sin(2^k pi p) for k = 0..11 (12 octaves x 3 axes)
 *   36-47  cos(2^k pi p) for k = 0..3
 *   48-50  wo      51-53  n      54  roughness
 *   55-57  diffuse albedo        58  mean specular
 *   59-61  p       62-63  0
 */
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "kgr_cache.h"
#include "kgr_device.cuh"

namespace kgr {

namespace {

template <class T>
__device__ __forceinline__ T to_half(float v);
template <>
__device__ __forceinline__ __nv_bfloat16 to_half<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }
template <>
__device__ __forceinline__ __half to_half<__half>(float v) { return __float2half_rn(v); }

template <class T>
__device__ __forceinline__ void write_features(T *dst, const f3 &x, const f3 &wo, const f3 &n, const Material &m,
		const CacheParams &cp)
{
	float p[3] = {(x.x - cp.bmin[0]) * cp.binv[0], (x.y - cp.bmin[1]) * cp.binv[1], (x.z - cp.bmin[2]) * cp.binv[2]};
	float f[64];
#pragma unroll
	for (int a = 0; a < 3; a++) {
		float scale = 1.0f;
#pragma unroll
		for (int k = 0; k < 12; k++) {
			float s, c;
			sincospif(p[a] * scale, &s, &c);
			f[3 * k + a] = s;
			if (k < 4)
				f[36 + 3 * k + a] = c;
			scale *= 2.0f;
		}
	}
	f[48] = wo.x; f[49] = wo.y; f[50] = wo.z;
	f[51] = n.x; f[52] = n.y; f[53] = n.z;
	f[54] = m.roughness;
	f[55] = m.diffuse.x; f[56] = m.diffuse.y; f[57] = m.diffuse.z;
	f[58] = (m.specular.x + m.specular.y + m.specular.z) * (1.0f / 3.0f);
	f[59] = p[0]; f[60] = p[1]; f[61] = p[2];
	f[62] = 0.0f; f[63] = 0.0f;
	/* 16-byte stores of 8 halves */
	uint4 *d4 = reinterpret_cast<uint4 *>(dst);
#pragma unroll
	for (int q = 0; q < 8; q++) {
		T h[8];
#pragma unroll
		for (int e = 0; e < 8; e++)
			h[e] = to_half<T>(f[8 * q + e]);
		d4[q] = *reinterpret_cast<uint4 *>(h);
	}
}

/* Query at the first bounce: one feature row per live path of the queue. */
template <class T>
__global__ void __launch_bounds__(128) query_kernel(DeviceScene s, PathBuffers pb, int q, CacheParams cp,
		T *__restrict__ feat, float4 *__restrict__ le)
{
	const uint32_t n = pb.counters[q == 0 ? CNT_Q0 : CNT_Q1];
	uint32_t stride = gridDim.x * blockDim.x;
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
		uint32_t p = pb.queue[q][i];
		float4 hv = pb.hit[p];
		kgr_hit h;
		h.prim = __float_as_int(hv.x);
		h.t = hv.y;
		h.b1 = hv.z;
		h.b2 = hv.w;
		float4 dv = pb.ray_d[p];
		f3 dir = mk(dv.x, dv.y, dv.z);
		SurfaceHit sh;
		if (h.prim >= 0 && surface(s, h, dir, sh)) {
			write_features<T>(feat + (size_t)i * 64, sh.x, sh.wo, sh.n, sh.mat, cp);
			le[i] = f4_of(sh.mat.emission, 1.0f);
		} else {
			le[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
			uint4 *d4 = reinterpret_cast<uint4 *>(feat + (size_t)i * 64);
			for (int k = 0; k < 8; k++)
				d4[k] = make_uint4(0, 0, 0, 0);
		}
	}
}

/* L += beta_1 (Le_1 + max(0, cache)) for every queried path. */
__global__ void apply_kernel(PathBuffers pb, int q, const float4 *__restrict__ out, const float4 *__restrict__ le)
{
	const uint32_t n = pb.counters[q == 0 ? CNT_Q0 : CNT_Q1];
	uint32_t stride = gridDim.x * blockDim.x;
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
		float4 e = le[i];
		if (e.w == 0.0f)
			continue;
		uint32_t p = pb.queue[q][i];
		float4 o = out[i];
		float4 b = pb.beta[p];
		float4 L = pb.L[p];
		L.x += b.x * (e.x + fmaxf(o.x, 0.0f));
		L.y += b.y * (e.y + fmaxf(o.y, 0.0f));
		L.z += b.z * (e.z + fmaxf(o.z, 0.0f));
		pb.L[p] = L;
	}
}

/* Training paths: a pixel subset that rotates with the frame. */
__global__ void train_generate_kernel(PathBuffers pb, FrameParams fp, uint32_t paths)
{
	uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
	if (p == 0) {
		pb.counters[CNT_Q0] = paths;
		pb.counters[CNT_Q1] = 0;
		pb.counters[CNT_SHADOW] = 0;
		pb.counters[CNT_BOUNCE_TOTAL] = 0;
		pb.counters[CNT_SHADOW_TOTAL] = 0;
	}
	if (p >= paths)
		return;
	uint32_t pix = (uint32_t)(((uint64_t)p * 2654435761ull + (uint64_t)fp.frame * 40503ull) % fp.npix);
	uint32_t ix = pix % fp.width, iy = pix / fp.width;
	f3 seed = pixel_seed(pix, fp.frame, 0x7F4A7C15u + p);
	f3 U = mk(fp.U[0], fp.U[1], fp.U[2]), V = mk(fp.V[0], fp.V[1], fp.V[2]), W = mk(fp.W[0], fp.W[1], fp.W[2]);
	pcg3f(seed);
	float ax = ((float)ix + (fract(seed.x) - 0.5f)) / (float)fp.width;
	float ay = ((float)iy + (fract(seed.y) - 0.5f)) / (float)fp.height;
	f3 d = normalize((2.0f * ax - 1.0f) * U + (2.0f * ay - 1.0f) * V + W);
	pb.ray_o[p] = make_float4(fp.center[0], fp.center[1], fp.center[2], 0.0f);
	pb.ray_d[p] = f4_of(d, 1e16f);
	pb.beta[p] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
	pb.L[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
	pb.seed[p] = f4_of(seed, 0.0f);
	pb.aov_n[p] = pb.aov_a[p] = pb.aov_p[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
	pb.queue[0][p] = p;
}

/* Record vertex `depth` of every live training path before it is shaded. */
template <class T>
__global__ void __launch_bounds__(128) record_kernel(DeviceScene s, PathBuffers pb, int q, int depth,
		CacheParams cp, CacheRecords rec)
{
	const uint32_t n = pb.counters[q == 0 ? CNT_Q0 : CNT_Q1];
	uint32_t stride = gridDim.x * blockDim.x;
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
		uint32_t p = pb.queue[q][i];
		size_t slot = (size_t)p * rec.depths + depth;
		float4 hv = pb.hit[p];
		kgr_hit h;
		h.prim = __float_as_int(hv.x);
		h.t = hv.y;
		h.b1 = hv.z;
		h.b2 = hv.w;
		float4 dv = pb.ray_d[p];
		SurfaceHit sh;
		if (h.prim >= 0 && surface(s, h, mk(dv.x, dv.y, dv.z), sh)) {
			write_features<T>(static_cast<T *>(rec.feat) + slot * 64, sh.x, sh.wo, sh.n, sh.mat, cp);
			rec.beta[slot] = pb.beta[p];
			float4 L = pb.L[p];
			rec.lbefore[slot] = L;
			rec.le[slot] = f4_of(sh.mat.emission, 1.0f);
		} else {
			rec.le[slot] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
		}
	}
}

/* Targets of the finished training paths, compacted into the batch. */
template <class T>
__global__ void targets_kernel(PathBuffers pb, uint32_t paths, CacheRecords rec, T *__restrict__ xb,
		float4 *__restrict__ tb, uint32_t *__restrict__ count, uint32_t cap)
{
	uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
	if (p >= paths)
		return;
	float4 Lf = pb.L[p];
	for (int d = 1; d < rec.depths; d++) {
		size_t slot = (size_t)p * rec.depths + d;
		float4 e = rec.le[slot];
		if (e.w == 0.0f)
			break;
		float4 b = rec.beta[slot], Lb = rec.lbefore[slot];
		if (fmaxf(b.x, fmaxf(b.y, b.z)) < 1e-4f)
			break;
		float4 t = make_float4((Lf.x - Lb.x) / b.x - e.x, (Lf.y - Lb.y) / b.y - e.y, (Lf.z - Lb.z) / b.z - e.z,
			0.0f);
		if (!(isfinite(t.x) && isfinite(t.y) && isfinite(t.z)))
			break;
		t.x = fmaxf(t.x, 0.0f);
		t.y = fmaxf(t.y, 0.0f);
		t.z = fmaxf(t.z, 0.0f);
		uint32_t k = atomicAdd(count, 1u);
		if (k >= cap)
			break;
		const uint4 *src = reinterpret_cast<const uint4 *>(static_cast<const T *>(rec.feat) + slot * 64);
		uint4 *dst = reinterpret_cast<uint4 *>(xb + (size_t)k * 64);
		for (int w = 0; w < 8; w++)
			dst[w] = src[w];
		tb[k] = t;
	}
}

inline int grid_for(uint32_t n, int block)
{
	long long b = ((long long)n + block - 1) / block;
	long long cap = (long long)device_sm_count() * 16;
	return (int)(b < 1 ? 1 : (b < cap ? b : cap));
}

} /* namespace */

void cache_query(const DeviceScene &s, const PathBuffers &pb, int q, const CacheParams &cp, void *feat,
		float4 *le, cudaStream_t st)
{
	int g = grid_for(pb.capacity, 128);
	if (cp.dtype == KGR_MLP_BF16)
		query_kernel<__nv_bfloat16><<<g, 128, 0, st>>>(s, pb, q, cp, static_cast<__nv_bfloat16 *>(feat), le);
	else
		query_kernel<__half><<<g, 128, 0, st>>>(s, pb, q, cp, static_cast<__half *>(feat), le);
	KGR_CUDA(cudaGetLastError());
}

void cache_apply(const PathBuffers &pb, int q, const float4 *out, const float4 *le, cudaStream_t st)
{
	apply_kernel<<<grid_for(pb.capacity, 256), 256, 0, st>>>(pb, q, out, le);
	KGR_CUDA(cudaGetLastError());
}

void cache_train_generate(const PathBuffers &pb, const FrameParams &fp, uint32_t paths, cudaStream_t st)
{
	train_generate_kernel<<<(paths + 255) / 256, 256, 0, st>>>(pb, fp, paths);
	KGR_CUDA(cudaGetLastError());
}

void cache_record(const DeviceScene &s, const PathBuffers &pb, int q, int depth, const CacheParams &cp,
		const CacheRecords &rec, cudaStream_t st)
{
	int g = grid_for(pb.capacity, 128);
	if (cp.dtype == KGR_MLP_BF16)
		record_kernel<__nv_bfloat16><<<g, 128, 0, st>>>(s, pb, q, depth, cp, rec);
	else
		record_kernel<__half><<<g, 128, 0, st>>>(s, pb, q, depth, cp, rec);
	KGR_CUDA(cudaGetLastError());
}

void cache_targets(const PathBuffers &pb, uint32_t paths, const CacheRecords &rec, int dtype, void *xb, float4 *tb,
		uint32_t *count, uint32_t cap, cudaStream_t st)
{
	KGR_CUDA(cudaMemsetAsync(count, 0, sizeof(uint32_t), st));
	if (dtype == KGR_MLP_BF16)
		targets_kernel<__nv_bfloat16><<<(paths + 127) / 128, 128, 0, st>>>(pb, paths, rec,
			static_cast<__nv_bfloat16 *>(xb), tb, count, cap);
	else
		targets_kernel<__half><<<(paths + 127) / 128, 128, 0, st>>>(pb, paths, rec, static_cast<__half *>(xb), tb,
			count, cap);
	KGR_CUDA(cudaGetLastError());
}

} /* namespace kgr */

/*
 * cache.cu -- the radiance cache in the wavefront path tracer.
 *
 * Render paths trace the camera ray, shade the primary vertex (emission +
 * NEE + BSDF sample) and trace the first bounce; at that secondary vertex
 * they query the network for the radiance it scatters toward the path and
 * stop: L += beta_1 (Le_1 + max(0, cache(x_1))).  Training paths -- a
 * rotating subset of pixels traced as plain paths to the full depth, one
 * thread per path -- record at every vertex k >= 1 the network input, the throughput beta_k,
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
#include "kgr_shade.cuh"

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

/* Camera ray of training path p: a pixel subset that rotates with the frame. */
__device__ __forceinline__ void train_camera_ray(const FrameParams &fp, uint32_t p, f3 &o, f3 &d, f3 &seed)
{
	uint32_t pix = (uint32_t)(((uint64_t)p * 2654435761ull + (uint64_t)fp.frame * 40503ull) % fp.npix);
	uint32_t ix = pix % fp.width, iy = pix / fp.width;
	seed = pixel_seed(pix, fp.frame, 0x7F4A7C15u + p);
	f3 U = mk(fp.U[0], fp.U[1], fp.U[2]), V = mk(fp.V[0], fp.V[1], fp.V[2]), W = mk(fp.W[0], fp.W[1], fp.W[2]);
	pcg3f(seed);
	float ax = ((float)ix + (fract(seed.x) - 0.5f)) / (float)fp.width;
	float ay = ((float)iy + (fract(seed.y) - 0.5f)) / (float)fp.height;
	d = normalize((2.0f * ax - 1.0f) * U + (2.0f * ay - 1.0f) * V + W);
	o = mk(fp.center[0], fp.center[1], fp.center[2]);
}

/* Keeps one shaded vertex in registers (training paths). */
struct RegisterSink {
	f3 x, L_add, next_d, next_beta;
	float4 pend_c, pend_e, pend_b, sh_o, sh_d;
	bool add_L = false, shadow = false, cont = false;
	__device__ __forceinline__ void vertex(const f3 &xv, const f3 &, const Material &) { x = xv; }
	__device__ __forceinline__ void emit(const f3 &add)
	{
		L_add = add;
		add_L = true;
	}
	__device__ __forceinline__ void nee(float4 c, float4 e, float4 b, float4 o, float4 d)
	{
		pend_c = c;
		pend_e = e;
		pend_b = b;
		sh_o = o;
		sh_d = d;
		shadow = true;
	}
	__device__ __forceinline__ void next(const f3 &, const f3 &wi, const f3 &beta)
	{
		next_d = wi;
		next_beta = beta;
		cont = true;
	}
};

/* Training paths, one thread per path through every depth (closest hit,
 * record, shade, shadow ray) -- a few thousand paths traced as a wavefront
 * would pay one launch latency per stage and depth.  At every vertex k >= 1
 * the record holds the network input, the throughput beta_k, the radiance
 * gathered before the vertex and its emission; pb.L[p] receives the path's
 * final radiance.  Shading is the path tracer's own (shade_surface). */
template <class T>
__global__ void __launch_bounds__(64) train_paths_kernel(DeviceScene s, PathBuffers pb, FrameParams fp,
		uint32_t paths, CacheParams cp, CacheRecords rec)
{
	uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
	if (p >= paths)
		return;
	f3 o, d, seed;
	train_camera_ray(fp, p, o, d, seed);
	f3 beta = mk(1.0f);
	float4 L = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
	for (int depth = 0; depth <= fp.max_depth; depth++) {
		kgr_hit h;
		trace<false>(s, fp.layout, o, d, 1e16f, h);
		SurfaceHit sh;
		bool surf = h.prim >= 0 && surface(s, h, d, sh);
		if (depth >= 1) {
			size_t slot = (size_t)p * rec.depths + depth;
			if (surf) {
				write_features<T>(static_cast<T *>(rec.feat) + slot * 64, sh.x, sh.wo, sh.n, sh.mat, cp);
				rec.beta[slot] = f4_of(beta, 0.0f);
				rec.lbefore[slot] = L;
				rec.le[slot] = f4_of(sh.mat.emission, 1.0f);
			} else {
				rec.le[slot] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
			}
		}
		if (!surf)
			break;
		RegisterSink v;
		shade_surface(s, fp, depth, 0, sh, beta, seed, v);
		if (v.add_L)
			L = f4_of(mk(L.x, L.y, L.z) + v.L_add, 0.0f);
		if (v.shadow) {
			kgr_hit sh_hit;
			bool occ = trace<true>(s, fp.layout, f3_of(v.sh_o), f3_of(v.sh_d), v.sh_d.w, sh_hit);
			L = nee_add(L, v.pend_c, v.pend_e, v.pend_b, occ);
		}
		if (!v.cont)
			break;
		o = v.x;
		d = v.next_d;
		beta = v.next_beta;
	}
	pb.L[p] = L;
}

/* The target of vertex d of path p, or false at the path's first vertex
 * without one (no record, vanishing throughput, non-finite value). */
__device__ __forceinline__ bool vertex_target(const CacheRecords &rec, uint32_t p, int d, float4 Lf, float4 &t)
{
	size_t slot = (size_t)p * rec.depths + d;
	float4 e = rec.le[slot];
	if (e.w == 0.0f)
		return false;
	float4 b = rec.beta[slot], Lb = rec.lbefore[slot];
	if (fmaxf(b.x, fmaxf(b.y, b.z)) < 1e-4f)
		return false;
	t = make_float4((Lf.x - Lb.x) / b.x - e.x, (Lf.y - Lb.y) / b.y - e.y, (Lf.z - Lb.z) / b.z - e.z, 0.0f);
	if (!(isfinite(t.x) && isfinite(t.y) && isfinite(t.z)))
		return false;
	t.x = fmaxf(t.x, 0.0f);
	t.y = fmaxf(t.y, 0.0f);
	t.z = fmaxf(t.z, 0.0f);
	return true;
}

/* Targets of the finished training paths, compacted into the batch (one
 * atomic per warp; slots at or past cap are dropped). */
template <class T>
__global__ void targets_kernel(PathBuffers pb, uint32_t paths, CacheRecords rec, T *__restrict__ xb,
		float4 *__restrict__ tb, uint32_t *__restrict__ count, uint32_t cap)
{
	uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
	const int lane = threadIdx.x & 31;
	bool act = p < paths;
	float4 Lf = act ? pb.L[p] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
	int mine = 0;
	if (act) {
		float4 t;
		for (int d = 1; d < rec.depths && vertex_target(rec, p, d, Lf, t); d++)
			mine++;
	}
	int incl = mine;
	for (int off = 1; off < 32; off <<= 1) {
		int v = __shfl_up_sync(0xffffffffu, incl, off);
		if (lane >= off)
			incl += v;
	}
	int total = __shfl_sync(0xffffffffu, incl, 31);
	uint32_t base = 0;
	if (lane == 31 && total > 0)
		base = atomicAdd(count, (uint32_t)total);
	base = __shfl_sync(0xffffffffu, base, 31);
	uint32_t k = base + (uint32_t)(incl - mine);
	for (int d = 1; d <= mine && k < cap; d++, k++) {
		float4 t;
		vertex_target(rec, p, d, Lf, t);
		size_t slot = (size_t)p * rec.depths + d;
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

void cache_train_paths(const DeviceScene &s, const PathBuffers &tb, const FrameParams &fp, uint32_t paths,
		const CacheParams &cp, const CacheRecords &rec, cudaStream_t st)
{
	if (paths == 0)
		return;
	if (cp.dtype == KGR_MLP_BF16)
		train_paths_kernel<__nv_bfloat16><<<(paths + 63) / 64, 64, 0, st>>>(s, tb, fp, paths, cp, rec);
	else
		train_paths_kernel<__half><<<(paths + 63) / 64, 64, 0, st>>>(s, tb, fp, paths, cp, rec);
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

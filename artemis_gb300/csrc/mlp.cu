/*
 * mlp.cu -- the radiance-cache MLP: 64 inputs -> 5 hidden layers of 64 with
 * ReLU -> 3 outputs (RGB radiance), weights and activations in BF16 or FP16
 * with FP32 accumulation on the tensor cores (mma.sync m16n8k16).
 *
 * The reference has only an unused FP32 forward pass (editor/mlp.cuh:48-154:
 * a 3 -> 4x256 -> 3 RadianceField with a naive GEMM, never compiled); the
 * network here is the one the benchmark configuration describes.
 *
 * Layouts.  Weights of layer l map in -> out as y = x W_l; the host keeps
 * FP32 master weights W[l][in][out] (6 layers; the last has 3 outputs padded
 * to 16) and half-precision copies; kernels stage the transposed copy
 *   wt[l][out][in]  (row stride 72 in shared memory)
 * whose 32-bit words are the B fragments of the forward x W.  The padding of
 * 8 elements makes the fragment loads of a warp hit 32 distinct banks.  The
 * backward delta W^T gathers its B fragments from the same array.
 *
 * Forward (inference): one warp owns 32 rows; the m16n8 accumulators of one
 * layer, after ReLU and rounding to half precision, are exactly the A
 * fragments of the next layer's m16n8k16, so activations never leave the
 * registers.
 *
 * Training: one kernel runs forward and backward for tiles of 64 rows with
 * the activations of all layers in shared memory and the block's FP32
 * weight gradient accumulated there too (213 KB per block, one block per
 * SM); per-block gradients are summed in a fixed order by a second kernel,
 * so training is deterministic.  Loss: relative L2,
 * sum_rows sum_c (y_c - t_c)^2 / (y_c^2 + 0.01) / rows, with y_c^2 in the
 * denominator treated as a constant (as in neural radiance caching).
 */
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "kgr_internal.h"
#include "kgr_mlp.h"

namespace kgr {

namespace {

#define MLP_W 64
#define MLP_OUT_PAD 16
#define MLP_LAYERS 6
#define MLP_STRIDE 72 /* padded row stride of staged weights (elements) */

template <class T>
struct HalfOps;

template <>
struct HalfOps<__nv_bfloat16> {
	__device__ static __forceinline__ uint32_t pack(float lo, float hi)
	{
		__nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
		return *reinterpret_cast<uint32_t *>(&v);
	}
	__device__ static __forceinline__ float to_float(__nv_bfloat16 v) { return __bfloat162float(v); }
	__device__ static __forceinline__ __nv_bfloat16 from_float(float v) { return __float2bfloat16_rn(v); }
	__device__ static __forceinline__ void mma(float *c, const uint32_t *a, const uint32_t *b)
	{
		asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
			     "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
			     : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
			     : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
	}
};

template <>
struct HalfOps<__half> {
	__device__ static __forceinline__ uint32_t pack(float lo, float hi)
	{
		__half2 v = __floats2half2_rn(lo, hi);
		return *reinterpret_cast<uint32_t *>(&v);
	}
	__device__ static __forceinline__ float to_float(__half v) { return __half2float(v); }
	__device__ static __forceinline__ __half from_float(float v) { return __float2half_rn(v); }
	__device__ static __forceinline__ void mma(float *c, const uint32_t *a, const uint32_t *b)
	{
		asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 "
			     "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
			     : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
			     : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
	}
};

/* Stage the half-precision weights in shared memory, transposed (forward)
 * and/or as stored (backward). */
template <class T>
__device__ __forceinline__ void stage_weights(const T *__restrict__ wt_g, T *wt_s, const T *__restrict__ wn_g,
		T *wn_s)
{
	/* global layout: per layer a dense [rows][64] block; layer 5 has 16 rows
	 * in the transposed copy and 64 x 16 in the plain copy */
	for (int l = 0; l < MLP_LAYERS; l++) {
		int rows_t = l == MLP_LAYERS - 1 ? MLP_OUT_PAD : MLP_W;
		const T *src = wt_g + (size_t)l * MLP_W * MLP_W;
		T *dst = wt_s + (size_t)l * MLP_W * MLP_STRIDE;
		for (int i = threadIdx.x; i < rows_t * MLP_W; i += blockDim.x)
			dst[(i / MLP_W) * MLP_STRIDE + (i % MLP_W)] = src[i];
		if (wn_s) {
			int cols_n = l == MLP_LAYERS - 1 ? MLP_OUT_PAD : MLP_W;
			const T *s2 = wn_g + (size_t)l * MLP_W * MLP_W;
			T *d2 = wn_s + (size_t)l * MLP_W * MLP_STRIDE;
			for (int i = threadIdx.x; i < MLP_W * cols_n; i += blockDim.x)
				d2[(i / cols_n) * MLP_STRIDE + (i % cols_n)] = s2[i];
		}
	}
}

/* B fragment of m16n8k16 from a [n][k] array with row stride MLP_STRIDE:
 * b0 = (k = 2t, 2t+1; n = g), b1 = (k = 2t+8, 2t+9; n = g). */
template <class T>
__device__ __forceinline__ void load_b(const T *w, int n0, int k0, int lane, uint32_t *b)
{
	int g = lane >> 2, t = lane & 3;
	const T *row = w + (size_t)(n0 + g) * MLP_STRIDE + k0 + 2 * t;
	b[0] = *reinterpret_cast<const uint32_t *>(row);
	b[1] = *reinterpret_cast<const uint32_t *>(row + 8);
}

/* Forward for one warp's 32 rows: a[mt][kk][4] holds the input fragments. */
template <class T>
__device__ __forceinline__ void warp_forward(const T *wt_s, uint32_t a[2][4][4], float out[2][2][4], int lane)
{
	for (int l = 0; l < MLP_LAYERS - 1; l++) {
		const T *w = wt_s + (size_t)l * MLP_W * MLP_STRIDE;
		float acc[2][8][4];
#pragma unroll
		for (int mt = 0; mt < 2; mt++)
#pragma unroll
			for (int j = 0; j < 8; j++)
#pragma unroll
				for (int r = 0; r < 4; r++)
					acc[mt][j][r] = 0.0f;
#pragma unroll
		for (int kk = 0; kk < 4; kk++)
#pragma unroll
			for (int j = 0; j < 8; j++) {
				uint32_t b[2];
				load_b(w, 8 * j, 16 * kk, lane, b);
				HalfOps<T>::mma(acc[0][j], a[0][kk], b);
				HalfOps<T>::mma(acc[1][j], a[1][kk], b);
			}
		/* ReLU, round, and reuse as the next layer's A fragments */
#pragma unroll
		for (int mt = 0; mt < 2; mt++)
#pragma unroll
			for (int kk = 0; kk < 4; kk++) {
				float *c0 = acc[mt][2 * kk], *c1 = acc[mt][2 * kk + 1];
				a[mt][kk][0] = HalfOps<T>::pack(fmaxf(c0[0], 0.0f), fmaxf(c0[1], 0.0f));
				a[mt][kk][1] = HalfOps<T>::pack(fmaxf(c0[2], 0.0f), fmaxf(c0[3], 0.0f));
				a[mt][kk][2] = HalfOps<T>::pack(fmaxf(c1[0], 0.0f), fmaxf(c1[1], 0.0f));
				a[mt][kk][3] = HalfOps<T>::pack(fmaxf(c1[2], 0.0f), fmaxf(c1[3], 0.0f));
			}
	}
	const T *w = wt_s + (size_t)(MLP_LAYERS - 1) * MLP_W * MLP_STRIDE;
#pragma unroll
	for (int mt = 0; mt < 2; mt++)
#pragma unroll
		for (int j = 0; j < 2; j++)
#pragma unroll
			for (int r = 0; r < 4; r++)
				out[mt][j][r] = 0.0f;
#pragma unroll
	for (int kk = 0; kk < 4; kk++)
#pragma unroll
		for (int j = 0; j < 2; j++) {
			uint32_t b[2];
			load_b(w, 8 * j, 16 * kk, lane, b);
			HalfOps<T>::mma(out[0][j], a[0][kk], b);
			HalfOps<T>::mma(out[1][j], a[1][kk], b);
		}
}

/* A fragments for rows [r0, r0 + 32) of a row-major [rows][64] half array:
 * a0 = (row g, k 2t..), a1 = (row g+8, k 2t..), a2 = (row g, k 2t+8..),
 * a3 = (row g+8, k 2t+8..).  Rows at or past n read as zero. */
template <class T>
__device__ __forceinline__ void load_a_rows(const T *x, size_t r0, uint32_t n, int lane, uint32_t a[2][4][4])
{
	int g = lane >> 2, t = lane & 3;
#pragma unroll
	for (int mt = 0; mt < 2; mt++) {
		size_t ra = r0 + 16 * mt + g, rb = ra + 8;
#pragma unroll
		for (int kk = 0; kk < 4; kk++) {
			int k = 16 * kk + 2 * t;
			a[mt][kk][0] = ra < n ? __ldg(reinterpret_cast<const uint32_t *>(x + ra * MLP_W + k)) : 0u;
			a[mt][kk][1] = rb < n ? __ldg(reinterpret_cast<const uint32_t *>(x + rb * MLP_W + k)) : 0u;
			a[mt][kk][2] = ra < n ? __ldg(reinterpret_cast<const uint32_t *>(x + ra * MLP_W + k + 8)) : 0u;
			a[mt][kk][3] = rb < n ? __ldg(reinterpret_cast<const uint32_t *>(x + rb * MLP_W + k + 8)) : 0u;
		}
	}
}

template <class T>
__global__ void __launch_bounds__(128) mlp_infer_kernel(const T *__restrict__ wt_g, const T *__restrict__ x,
		uint32_t n, float4 *__restrict__ out, const uint32_t *__restrict__ n_dev)
{
	if (n_dev) {
		uint32_t c = *n_dev;
		n = c < n ? c : n;
	}
	extern __shared__ __align__(16) unsigned char smem_raw[];
	T *wt_s = reinterpret_cast<T *>(smem_raw);
	stage_weights<T>(wt_g, wt_s, nullptr, nullptr);
	__syncthreads();
	int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	int g = lane >> 2, t = lane & 3;
	for (size_t base = (size_t)blockIdx.x * 128; base < n; base += (size_t)gridDim.x * 128) {
		size_t r0 = base + 32 * warp;
		uint32_t a[2][4][4];
		load_a_rows<T>(x, r0, n, lane, a);
		float o[2][2][4];
		warp_forward<T>(wt_s, a, o, lane);
		/* output columns 0..2 live in tile j = 0: t = 0 holds cols 0,1 and
		 * t = 1 holds col 2 (and the padded col 3) */
#pragma unroll
		for (int mt = 0; mt < 2; mt++) {
			float lo0 = __shfl_sync(0xffffffffu, o[mt][0][0], (lane & ~3) | 1);
			float hi0 = __shfl_sync(0xffffffffu, o[mt][0][2], (lane & ~3) | 1);
			if (t == 0) {
				size_t ra = r0 + 16 * mt + g, rb = ra + 8;
				if (ra < n)
					out[ra] = make_float4(o[mt][0][0], o[mt][0][1], lo0, 0.0f);
				if (rb < n)
					out[rb] = make_float4(o[mt][0][2], o[mt][0][3], hi0, 0.0f);
			}
		}
	}
}

/* ------------------------------------------------------------- training */

/* Generic warp GEMM over shared memory for the backward pass: C[16*MT x 8*NT]
 * += A[rows m][k] (row-major or transposed) * B[k][n] given as [n][k] with
 * stride ldb (or as [k][n] when b_kn).  Fragments are gathered with 16-bit
 * loads, which handles every transposition. */
template <class T>
__device__ __forceinline__ uint32_t gather2(const T *p0, const T *p1)
{
	T v[2] = {*p0, *p1};
	return *reinterpret_cast<uint32_t *>(v);
}

#define TRAIN_ROWS 64 /* rows per tile: 4 warps x 16 */

/* A fragments of one m16 tile: rows [r0, r0 + 16) of a row-major [rows][64]
 * half array; rows at or past n read as zero. */
template <class T>
__device__ __forceinline__ void load_a_tile(const T *x, size_t r0, uint32_t n, int lane, uint32_t a[4][4])
{
	int g = lane >> 2, t = lane & 3;
	size_t ra = r0 + g, rb = ra + 8;
#pragma unroll
	for (int kk = 0; kk < 4; kk++) {
		int k = 16 * kk + 2 * t;
		a[kk][0] = ra < n ? __ldg(reinterpret_cast<const uint32_t *>(x + ra * MLP_W + k)) : 0u;
		a[kk][1] = rb < n ? __ldg(reinterpret_cast<const uint32_t *>(x + rb * MLP_W + k)) : 0u;
		a[kk][2] = ra < n ? __ldg(reinterpret_cast<const uint32_t *>(x + ra * MLP_W + k + 8)) : 0u;
		a[kk][3] = rb < n ? __ldg(reinterpret_cast<const uint32_t *>(x + rb * MLP_W + k + 8)) : 0u;
	}
}

/* Forward and backward over tiles of 64 rows; the grid is persistent (at
 * most one block per SM) and each block accumulates its weight gradient in
 * shared memory (FP32, every element owned by one lane, so no atomics),
 * then writes it to its own slice of `partial` ([gridDim.x][6][64][64]).
 * reduce_partials sums the slices in block order, so the gradient does not
 * depend on scheduling.
 *
 * Per tile: warp w runs the forward of rows [16w, 16w + 16) with the layer
 * inputs kept in shared memory, writes the output delta of its rows, and in
 * the backward computes for each layer the 16-row block [16w, 16w + 16) of
 * dW = A^T delta over all 64 rows of the tile (an m16n8k16 chain with K =
 * rows), then the delta of its own rows' layer input. */
template <class T>
__global__ void __launch_bounds__(128) mlp_train_kernel(const T *__restrict__ wt_g, const T *__restrict__ x,
		const float4 *__restrict__ target, uint32_t n, float *__restrict__ partial, float *__restrict__ loss_sum,
		const uint32_t *__restrict__ n_dev)
{
	if (n_dev) {
		uint32_t c = *n_dev;
		n = c < n ? c : n;
	}
	extern __shared__ __align__(16) unsigned char smem_raw[];
	T *wt_s = reinterpret_cast<T *>(smem_raw);
	T *act = wt_s + (size_t)MLP_LAYERS * MLP_W * MLP_STRIDE;             /* 6 x [64][72] */
	T *dlt = act + (size_t)MLP_LAYERS * TRAIN_ROWS * MLP_STRIDE;          /* [64][72] */
	float *gacc = reinterpret_cast<float *>(dlt + (size_t)TRAIN_ROWS * MLP_STRIDE); /* [6][64][64] */
	stage_weights<T>(wt_g, wt_s, nullptr, nullptr);
	for (int i = threadIdx.x; i < MLP_LAYERS * MLP_W * MLP_W / 4; i += blockDim.x)
		reinterpret_cast<float4 *>(gacc)[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
	__syncthreads();
	int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	int g = lane >> 2, t = lane & 3;
	const int lr0 = 16 * warp; /* this warp's rows within the tile */
	float lsum = 0.0f;
	for (size_t base = (size_t)blockIdx.x * TRAIN_ROWS; base < n; base += (size_t)gridDim.x * TRAIN_ROWS) {
		/* ---- forward, keeping every layer's input in shared memory ---- */
		uint32_t a[4][4];
		load_a_tile<T>(x, base + lr0, n, lane, a);
		for (int l = 0; l < MLP_LAYERS; l++) {
			T *A = act + (size_t)l * TRAIN_ROWS * MLP_STRIDE;
#pragma unroll
			for (int kk = 0; kk < 4; kk++) {
				int ra = lr0 + g, k = 16 * kk + 2 * t;
				*reinterpret_cast<uint32_t *>(A + ra * MLP_STRIDE + k) = a[kk][0];
				*reinterpret_cast<uint32_t *>(A + (ra + 8) * MLP_STRIDE + k) = a[kk][1];
				*reinterpret_cast<uint32_t *>(A + ra * MLP_STRIDE + k + 8) = a[kk][2];
				*reinterpret_cast<uint32_t *>(A + (ra + 8) * MLP_STRIDE + k + 8) = a[kk][3];
			}
			if (l == MLP_LAYERS - 1)
				break;
			const T *w = wt_s + (size_t)l * MLP_W * MLP_STRIDE;
			float acc[8][4];
#pragma unroll
			for (int j = 0; j < 8; j++)
#pragma unroll
				for (int r = 0; r < 4; r++)
					acc[j][r] = 0.0f;
#pragma unroll
			for (int kk = 0; kk < 4; kk++)
#pragma unroll
				for (int j = 0; j < 8; j++) {
					uint32_t b[2];
					load_b(w, 8 * j, 16 * kk, lane, b);
					HalfOps<T>::mma(acc[j], a[kk], b);
				}
#pragma unroll
			for (int kk = 0; kk < 4; kk++) {
				float *c0 = acc[2 * kk], *c1 = acc[2 * kk + 1];
				a[kk][0] = HalfOps<T>::pack(fmaxf(c0[0], 0.0f), fmaxf(c0[1], 0.0f));
				a[kk][1] = HalfOps<T>::pack(fmaxf(c0[2], 0.0f), fmaxf(c0[3], 0.0f));
				a[kk][2] = HalfOps<T>::pack(fmaxf(c1[0], 0.0f), fmaxf(c1[1], 0.0f));
				a[kk][3] = HalfOps<T>::pack(fmaxf(c1[2], 0.0f), fmaxf(c1[3], 0.0f));
			}
		}
		/* output layer */
		float o[2][4];
		{
			const T *w = wt_s + (size_t)(MLP_LAYERS - 1) * MLP_W * MLP_STRIDE;
#pragma unroll
			for (int j = 0; j < 2; j++)
#pragma unroll
				for (int r = 0; r < 4; r++)
					o[j][r] = 0.0f;
#pragma unroll
			for (int kk = 0; kk < 4; kk++)
#pragma unroll
				for (int j = 0; j < 2; j++) {
					uint32_t b[2];
					load_b(w, 8 * j, 16 * kk, lane, b);
					HalfOps<T>::mma(o[j], a[kk], b);
				}
		}
		/* loss and output delta (columns 0..15, only 0..2 non-zero) */
#pragma unroll
		for (int half = 0; half < 2; half++) {
			int lr = lr0 + g + 8 * half;
			size_t gr = base + lr;
			float4 tg = gr < n ? target[gr] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
			float tv[3] = {tg.x, tg.y, tg.z};
#pragma unroll
			for (int j = 0; j < 2; j++)
#pragma unroll
				for (int e = 0; e < 2; e++) {
					int col = 8 * j + 2 * t + e;
					float y = o[j][2 * half + e];
					float d = 0.0f;
					if (col < 3 && gr < n) {
						float diff = y - tv[col];
						float den = y * y + 0.01f;
						lsum += diff * diff / den;
						d = 2.0f * diff / den / (float)n;
					}
					dlt[lr * MLP_STRIDE + col] = HalfOps<T>::from_float(d);
				}
		}
		__syncthreads();
		/* ---- backward ---- */
		int ncols = MLP_OUT_PAD;
		for (int l = MLP_LAYERS - 1; l >= 0; l--) {
			const T *A = act + (size_t)l * TRAIN_ROWS * MLP_STRIDE; /* layer input [rows][64] */
			/* dW[i][j] += sum over the tile's rows r of A[r][i] dlt[r][j]
			 * for i in this warp's block: M = 16 (i), N = ncols, K = 64 */
			float *gl = gacc + (size_t)l * MLP_W * MLP_W;
			const int i0 = lr0 + g; /* weight row (layer input index) */
			for (int nj = 0; nj < ncols / 8; nj++) {
				float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
				const int jn = 8 * nj + g;
#pragma unroll
				for (int kk = 0; kk < TRAIN_ROWS / 16; kk++) {
					int rr = 16 * kk + 2 * t;
					uint32_t af[4], bf[2];
					af[0] = gather2(A + rr * MLP_STRIDE + i0, A + (rr + 1) * MLP_STRIDE + i0);
					af[1] = gather2(A + rr * MLP_STRIDE + i0 + 8, A + (rr + 1) * MLP_STRIDE + i0 + 8);
					af[2] = gather2(A + (rr + 8) * MLP_STRIDE + i0, A + (rr + 9) * MLP_STRIDE + i0);
					af[3] = gather2(A + (rr + 8) * MLP_STRIDE + i0 + 8, A + (rr + 9) * MLP_STRIDE + i0 + 8);
					bf[0] = gather2(dlt + rr * MLP_STRIDE + jn, dlt + (rr + 1) * MLP_STRIDE + jn);
					bf[1] = gather2(dlt + (rr + 8) * MLP_STRIDE + jn, dlt + (rr + 9) * MLP_STRIDE + jn);
					HalfOps<T>::mma(c, af, bf);
				}
				int j = 8 * nj + 2 * t;
				float2 *p0 = reinterpret_cast<float2 *>(gl + i0 * MLP_W + j);
				float2 *p1 = reinterpret_cast<float2 *>(gl + (i0 + 8) * MLP_W + j);
				float2 v0 = *p0, v1 = *p1;
				v0.x += c[0];
				v0.y += c[1];
				v1.x += c[2];
				v1.y += c[3];
				*p0 = v0;
				*p1 = v1;
			}
			if (l == 0)
				break;
			/* delta of this warp's rows of the layer input: (dlt W^T) *
			 * relu'(A), K = ncols; B[k = out][n = in] = wt[out][in] */
			const T *w = wt_s + (size_t)l * MLP_W * MLP_STRIDE;
			float acc[8][4];
#pragma unroll
			for (int j = 0; j < 8; j++)
#pragma unroll
				for (int r = 0; r < 4; r++)
					acc[j][r] = 0.0f;
			for (int kk = 0; kk < ncols / 16; kk++) {
				uint32_t af[4];
				int ra = lr0 + g, k = 16 * kk + 2 * t;
				af[0] = *reinterpret_cast<const uint32_t *>(dlt + ra * MLP_STRIDE + k);
				af[1] = *reinterpret_cast<const uint32_t *>(dlt + (ra + 8) * MLP_STRIDE + k);
				af[2] = *reinterpret_cast<const uint32_t *>(dlt + ra * MLP_STRIDE + k + 8);
				af[3] = *reinterpret_cast<const uint32_t *>(dlt + (ra + 8) * MLP_STRIDE + k + 8);
#pragma unroll
				for (int j = 0; j < 8; j++) {
					int nn = 8 * j + g;
					uint32_t b[2];
					b[0] = gather2(w + k * MLP_STRIDE + nn, w + (k + 1) * MLP_STRIDE + nn);
					b[1] = gather2(w + (k + 8) * MLP_STRIDE + nn, w + (k + 9) * MLP_STRIDE + nn);
					HalfOps<T>::mma(acc[j], af, b);
				}
			}
			/* every warp has read the whole delta tile for dW */
			__syncthreads();
#pragma unroll
			for (int j = 0; j < 8; j++) {
				int c = 8 * j + 2 * t;
#pragma unroll
				for (int e = 0; e < 4; e++) {
					int rr = lr0 + g + (e >> 1) * 8, cc = c + (e & 1);
					float av = HalfOps<T>::to_float(A[rr * MLP_STRIDE + cc]);
					float d = av > 0.0f ? acc[j][e] : 0.0f;
					dlt[rr * MLP_STRIDE + cc] = HalfOps<T>::from_float(d);
				}
			}
			__syncthreads();
			ncols = MLP_W;
		}
		/* the next tile overwrites act and dlt */
		__syncthreads();
	}
	float *dst = partial + (size_t)blockIdx.x * MLP_LAYERS * MLP_W * MLP_W;
	for (int i = threadIdx.x; i < MLP_LAYERS * MLP_W * MLP_W / 4; i += blockDim.x)
		reinterpret_cast<float4 *>(dst)[i] = reinterpret_cast<const float4 *>(gacc)[i];
	for (int off = 16; off > 0; off >>= 1)
		lsum += __shfl_down_sync(0xffffffffu, lsum, off);
	if (lane == 0)
		atomicAdd(loss_sum, lsum);
}

/* grad[k] = sum over blocks b (in order) of partial[b][k]. */
__global__ void reduce_partials_kernel(const float *__restrict__ partial, int blocks, float *__restrict__ grad)
{
	int k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= MLP_LAYERS * MLP_W * MLP_W)
		return;
	float s = 0.0f;
	for (int b = 0; b < blocks; b++)
		s += partial[(size_t)b * MLP_LAYERS * MLP_W * MLP_W + k];
	grad[k] = s;
}

/* Adam on the FP32 master weights, then the half-precision copies in both
 * layouts (plain [l][in][out] and transposed [l][out][in]). */
template <class T>
__global__ void adam_kernel(float *__restrict__ w, float *__restrict__ m, float *__restrict__ v,
		const float *__restrict__ grad, T *__restrict__ wn, T *__restrict__ wt, float lr, float b1, float b2,
		float eps, float c1, float c2, int update)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= MLP_LAYERS * MLP_W * MLP_W)
		return;
	int l = i / (MLP_W * MLP_W), r = i % (MLP_W * MLP_W);
	int in = r / MLP_W, out = r % MLP_W;
	int outs = l == MLP_LAYERS - 1 ? 3 : MLP_W;
	float wi = w[i];
	if (out >= outs) {
		wi = 0.0f;
	} else if (update) {
		float gi = grad[i];
		float mi = b1 * m[i] + (1.0f - b1) * gi;
		float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
		m[i] = mi;
		v[i] = vi;
		wi -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
		w[i] = wi;
	}
	T h = HalfOps<T>::from_float(wi);
	/* plain copy: layer l block [in][cols], cols = 64 or 16 */
	int cols = l == MLP_LAYERS - 1 ? MLP_OUT_PAD : MLP_W;
	if (out < cols)
		wn[(size_t)l * MLP_W * MLP_W + in * cols + out] = h;
	/* transposed copy: [out][in], rows = 64 or 16 */
	if (out < cols)
		wt[(size_t)l * MLP_W * MLP_W + out * MLP_W + in] = h;
}

size_t infer_smem() { return (size_t)MLP_LAYERS * MLP_W * MLP_STRIDE * 2; }
size_t train_smem()
{
	return (size_t)MLP_LAYERS * MLP_W * MLP_STRIDE * 2 + (size_t)MLP_LAYERS * TRAIN_ROWS * MLP_STRIDE * 2
		+ (size_t)TRAIN_ROWS * MLP_STRIDE * 2 + (size_t)MLP_LAYERS * MLP_W * MLP_W * 4;
}

template <class K>
void set_smem(K kernel, size_t bytes)
{
	KGR_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
}

} /* namespace */

void mlp_infer(const MlpParams &mp, const void *x, uint32_t n, float4 *out, cudaStream_t st, const uint32_t *n_dev)
{
	if (n == 0)
		return;
	if (mp.infer == KGR_MLP_INFER_TCGEN05) {
		mlp_infer_tc(mp, x, n, out, mp.tc_err, st, n_dev);
		return;
	}
	int grid = device_sm_count() * 4;
	size_t sm = infer_smem();
	if (mp.dtype == KGR_MLP_BF16) {
		static bool once = (set_smem(mlp_infer_kernel<__nv_bfloat16>, sm), true);
		(void)once;
		mlp_infer_kernel<__nv_bfloat16><<<grid, 128, sm, st>>>(
			static_cast<const __nv_bfloat16 *>(mp.wt), static_cast<const __nv_bfloat16 *>(x), n, out, n_dev);
	} else {
		static bool once = (set_smem(mlp_infer_kernel<__half>, sm), true);
		(void)once;
		mlp_infer_kernel<__half><<<grid, 128, sm, st>>>(static_cast<const __half *>(mp.wt),
			static_cast<const __half *>(x), n, out, n_dev);
	}
	KGR_CUDA(cudaGetLastError());
}

void mlp_gradients(const MlpParams &mp, const void *x, const float4 *target, uint32_t n, float *grad, float *loss,
		cudaStream_t st, const uint32_t *n_dev, int max_blocks)
{
	KGR_CUDA(cudaMemsetAsync(loss, 0, sizeof(float), st));
	if (n == 0) {
		KGR_CUDA(cudaMemsetAsync(grad, 0, sizeof(float) * MLP_LAYERS * MLP_W * MLP_W, st));
		return;
	}
	size_t sm = train_smem();
	int grid = mp.partial_blocks;
	if (max_blocks > 0 && max_blocks < grid)
		grid = max_blocks;
	const long long rows_per_tile = mp.train == KGR_MLP_TRAIN_TCGEN05 ? 128 : TRAIN_ROWS;
	long long tiles = ((long long)n + rows_per_tile - 1) / rows_per_tile;
	if (tiles < grid)
		grid = (int)tiles;
	KGR_REQUIRE(grid >= 1 && mp.partial, KGR_ERR_INTERNAL, "MLP gradient scratch missing");
	if (mp.train == KGR_MLP_TRAIN_TCGEN05) {
		mlp_train_tc(mp, x, target, n, grid, loss, st, n_dev);
	} else if (mp.dtype == KGR_MLP_BF16) {
		static bool once = (set_smem(mlp_train_kernel<__nv_bfloat16>, sm), true);
		(void)once;
		mlp_train_kernel<__nv_bfloat16><<<grid, 128, sm, st>>>(static_cast<const __nv_bfloat16 *>(mp.wt),
			static_cast<const __nv_bfloat16 *>(x), target, n, mp.partial, loss, n_dev);
	} else {
		static bool once = (set_smem(mlp_train_kernel<__half>, sm), true);
		(void)once;
		mlp_train_kernel<__half><<<grid, 128, sm, st>>>(static_cast<const __half *>(mp.wt),
			static_cast<const __half *>(x), target, n, mp.partial, loss, n_dev);
	}
	KGR_CUDA(cudaGetLastError());
	int np = MLP_LAYERS * MLP_W * MLP_W;
	reduce_partials_kernel<<<(np + 255) / 256, 256, 0, st>>>(mp.partial, grid, grad);
	KGR_CUDA(cudaGetLastError());
}

void mlp_adam(const MlpParams &mp, const float *grad, float lr, int step, cudaStream_t st)
{
	/* step <= 0 only refreshes the half-precision copies from the masters */
	const float b1 = 0.9f, b2 = 0.99f, eps = 1e-8f;
	int update = step > 0;
	float c1 = update ? 1.0f - powf(b1, (float)step) : 1.0f, c2 = update ? 1.0f - powf(b2, (float)step) : 1.0f;
	int n = MLP_LAYERS * MLP_W * MLP_W;
	if (mp.dtype == KGR_MLP_BF16)
		adam_kernel<__nv_bfloat16><<<(n + 255) / 256, 256, 0, st>>>(mp.master, mp.m, mp.v, grad,
			static_cast<__nv_bfloat16 *>(mp.wn), static_cast<__nv_bfloat16 *>(mp.wt), lr, b1, b2, eps, c1, c2,
			update);
	else
		adam_kernel<__half><<<(n + 255) / 256, 256, 0, st>>>(mp.master, mp.m, mp.v, grad,
			static_cast<__half *>(mp.wn), static_cast<__half *>(mp.wt), lr, b1, b2, eps, c1, c2, update);
	KGR_CUDA(cudaGetLastError());
}

} /* namespace kgr */

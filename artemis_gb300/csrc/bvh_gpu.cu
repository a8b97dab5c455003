/*
 * bvh_gpu.cu -- the binned-SAH builder of bvh_build.cpp (build_sah) on the
 * GPU, producing the same tree: the same splits, the same leaves, the same
 * primitive order inside every node.
 *
 * Why the trees agree.  build_sah's decisions depend only on the set of
 * primitives in a node: its bounds and its 32-bin histograms per axis are
 * min/max/count reductions, which are independent of order; the split is
 * chosen by one sequential sweep over the bins in a fixed float order; and
 * the partition is stable.  Here the reductions run as atomics on
 * order-preserving integer encodings of the floats (exact), the sweep runs
 * in one thread per node with the host's expressions (kernels are built
 * with -fmad=false and IEEE division), and the partition is a stable
 * segmented scatter.  Box coordinates are canonical (no -0), so min and max
 * are exact functions of the set.  Node numbering differs (level order
 * here, depth-first on the host); no layout depends on it.
 *
 * Nodes with more than GB_SMALL primitives are processed level by level
 * across blocks of GB_CHUNK primitives; a node at or below GB_SMALL is
 * built, with its whole subtree, by one thread running the host algorithm.
 * The host keeps the per-level bookkeeping (task lists, chunk tables, the
 * segmented scan of left counts, child allocation), a few small copies per
 * level.
 */
#include <float.h>

#include <algorithm>
#include <vector>

#include "kgr_internal.h"

namespace kgr {

namespace {

#define GB_BINS 32
#define GB_SMALL 128
#define GB_CHUNK 2048
#define GB_BLOCK 256
#define GB_STACK 128

__device__ __forceinline__ uint32_t fenc(float f)
{
	uint32_t b = __float_as_uint(f);
	return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

__device__ __forceinline__ float fdec(uint32_t e)
{
	return __uint_as_float((e & 0x80000000u) ? (e & 0x7FFFFFFFu) : ~e);
}

__device__ __forceinline__ float dmin(float a, float b) { return b < a ? b : a; }
__device__ __forceinline__ float dmax(float a, float b) { return a < b ? b : a; }

/* surface_area of bvh_build.cpp, same operations in the same order */
__device__ __forceinline__ float sarea(const float *mn, const float *mx)
{
	float dx = __fsub_rn(mx[0], mn[0]), dy = __fsub_rn(mx[1], mn[1]), dz = __fsub_rn(mx[2], mn[2]);
	float xy = __fmul_rn(dx, dy), yz = __fmul_rn(dy, dz), xz = __fmul_rn(dx, dz);
	return __fmul_rn(2.0f, __fadd_rn(__fadd_rn(xy, yz), xz));
}

__device__ __forceinline__ int bin_of(float c, float c0, float scale)
{
	int b = (int)__fmul_rn(__fsub_rn(c, c0), scale);
	return b < 0 ? 0 : (b >= GB_BINS ? GB_BINS - 1 : b);
}

struct Task {
	int32_t node;
	uint32_t begin, end;
};

/* per large task: encoded bounds of boxes (0..5) and centroids (6..11) */
struct TaskBounds {
	uint32_t v[12];
};

struct Bin {
	uint32_t count;
	uint32_t mn[3], mx[3];
};

struct Decision {
	int32_t axis, split; /* axis -1: no usable axis */
	int32_t leaf;
	uint32_t pad;
	float c0, scale;
};

struct Boxes {
	const float4 *bmin, *bmax, *cen;
};

__global__ void gb_init(const float *boxes6, uint32_t n, float4 *bmin, float4 *bmax, float4 *cen, uint32_t *order)
{
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	const float *b = boxes6 + 6 * (size_t)i;
	float mn[3], mx[3], c[3];
	for (int k = 0; k < 3; k++) {
		mn[k] = __fadd_rn(b[k], 0.0f); /* canonical zero */
		mx[k] = __fadd_rn(b[3 + k], 0.0f);
		c[k] = __fmul_rn(__fadd_rn(mn[k], mx[k]), 0.5f);
	}
	bmin[i] = make_float4(mn[0], mn[1], mn[2], 0.0f);
	bmax[i] = make_float4(mx[0], mx[1], mx[2], 0.0f);
	cen[i] = make_float4(c[0], c[1], c[2], 0.0f);
	order[i] = i;
}

__global__ void gb_reset_bounds(TaskBounds *tb, Bin *bins, uint32_t ntasks)
{
	uint32_t t = blockIdx.x;
	if (t >= ntasks)
		return;
	for (int k = threadIdx.x; k < 12; k += blockDim.x)
		tb[t].v[k] = (k % 6) < 3 ? 0xFFFFFFFFu : 0u; /* min slots high, max slots low */
	for (int k = threadIdx.x; k < 3 * GB_BINS; k += blockDim.x) {
		Bin &b = bins[(size_t)t * 3 * GB_BINS + k];
		b.count = 0;
		for (int a = 0; a < 3; a++) {
			b.mn[a] = 0xFFFFFFFFu;
			b.mx[a] = 0u;
		}
	}
}

/* node bounds and centroid bounds of every large task, one block per chunk */
__global__ void __launch_bounds__(GB_BLOCK) gb_bounds(Boxes bx, const uint32_t *order, const Task *tasks,
		const uint32_t *chunk_task, const uint32_t *chunk_begin, TaskBounds *tb)
{
	uint32_t t = chunk_task[blockIdx.x];
	uint32_t b0 = chunk_begin[blockIdx.x], b1 = min(b0 + GB_CHUNK, tasks[t].end);
	__shared__ uint32_t s[12];
	if (threadIdx.x < 12)
		s[threadIdx.x] = (threadIdx.x % 6) < 3 ? 0xFFFFFFFFu : 0u;
	__syncthreads();
	uint32_t v[12];
	for (int k = 0; k < 12; k++)
		v[k] = (k % 6) < 3 ? 0xFFFFFFFFu : 0u;
	for (uint32_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
		uint32_t p = order[i];
		float4 mn = bx.bmin[p], mx = bx.bmax[p], c = bx.cen[p];
		float a[12] = {mn.x, mn.y, mn.z, mx.x, mx.y, mx.z, c.x, c.y, c.z, c.x, c.y, c.z};
		for (int k = 0; k < 12; k++) {
			uint32_t e = fenc(a[k]);
			v[k] = (k % 6) < 3 ? min(v[k], e) : max(v[k], e);
		}
	}
	for (int k = 0; k < 12; k++) {
		if ((k % 6) < 3)
			atomicMin(&s[k], v[k]);
		else
			atomicMax(&s[k], v[k]);
	}
	__syncthreads();
	if (threadIdx.x < 12) {
		int k = threadIdx.x;
		if ((k % 6) < 3)
			atomicMin(&tb[t].v[k], s[k]);
		else
			atomicMax(&tb[t].v[k], s[k]);
	}
}

/* 32-bin histograms of every axis with extent, one block per chunk */
__global__ void __launch_bounds__(GB_BLOCK) gb_bins(Boxes bx, const uint32_t *order, const Task *tasks,
		const uint32_t *chunk_task, const uint32_t *chunk_begin, const TaskBounds *tb, Bin *bins)
{
	uint32_t t = chunk_task[blockIdx.x];
	uint32_t b0 = chunk_begin[blockIdx.x], b1 = min(b0 + GB_CHUNK, tasks[t].end);
	__shared__ Bin s[3 * GB_BINS];
	for (int k = threadIdx.x; k < 3 * GB_BINS; k += blockDim.x) {
		s[k].count = 0;
		for (int a = 0; a < 3; a++) {
			s[k].mn[a] = 0xFFFFFFFFu;
			s[k].mx[a] = 0u;
		}
	}
	__syncthreads();
	float c0[3], scale[3];
	bool use[3];
	for (int a = 0; a < 3; a++) {
		c0[a] = fdec(tb[t].v[6 + a]);
		float ext = __fsub_rn(fdec(tb[t].v[9 + a]), c0[a]);
		use[a] = ext > 0.0f;
		scale[a] = use[a] ? __fdiv_rn((float)GB_BINS, ext) : 0.0f;
	}
	for (uint32_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
		uint32_t p = order[i];
		float4 mn = bx.bmin[p], mx = bx.bmax[p], c = bx.cen[p];
		float cc[3] = {c.x, c.y, c.z};
		uint32_t emn[3] = {fenc(mn.x), fenc(mn.y), fenc(mn.z)}, emx[3] = {fenc(mx.x), fenc(mx.y), fenc(mx.z)};
		for (int a = 0; a < 3; a++) {
			if (!use[a])
				continue;
			Bin &b = s[a * GB_BINS + bin_of(cc[a], c0[a], scale[a])];
			atomicAdd(&b.count, 1u);
			for (int k = 0; k < 3; k++) {
				atomicMin(&b.mn[k], emn[k]);
				atomicMax(&b.mx[k], emx[k]);
			}
		}
	}
	__syncthreads();
	for (int k = threadIdx.x; k < 3 * GB_BINS; k += blockDim.x) {
		if (!s[k].count)
			continue;
		Bin &g = bins[(size_t)t * 3 * GB_BINS + k];
		atomicAdd(&g.count, s[k].count);
		for (int a = 0; a < 3; a++) {
			atomicMin(&g.mn[a], s[k].mn[a]);
			atomicMax(&g.mx[a], s[k].mx[a]);
		}
	}
}

/* The split of one node from its bins: the host's sweep, one thread. */
__device__ void choose_split(const float *bmn, const float *bmx, const float *cmn, const float *cmx, uint32_t cnt,
		int max_leaf, const Bin *const *axis_bins, Decision &d, float sa_parent)
{
	float best_cost = FLT_MAX;
	int best_axis = -1, best_split = 0;
	for (int axis = 0; axis < 3; axis++) {
		float ext = __fsub_rn(cmx[axis], cmn[axis]);
		if (!(ext > 0.0f))
			continue;
		const Bin *bins = axis_bins[axis];
		float rarea[GB_BINS];
		uint32_t rcount[GB_BINS];
		float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
		uint32_t c = 0;
		for (int b = GB_BINS - 1; b > 0; b--) {
			c += bins[b].count;
			if (bins[b].count)
				for (int k = 0; k < 3; k++) {
					mn[k] = dmin(mn[k], fdec(bins[b].mn[k]));
					mx[k] = dmax(mx[k], fdec(bins[b].mx[k]));
				}
			rcount[b] = c;
			rarea[b] = c ? sarea(mn, mx) : 0.0f;
		}
		for (int k = 0; k < 3; k++) {
			mn[k] = FLT_MAX;
			mx[k] = -FLT_MAX;
		}
		c = 0;
		for (int b = 1; b < GB_BINS; b++) {
			c += bins[b - 1].count;
			if (bins[b - 1].count)
				for (int k = 0; k < 3; k++) {
					mn[k] = dmin(mn[k], fdec(bins[b - 1].mn[k]));
					mx[k] = dmax(mx[k], fdec(bins[b - 1].mx[k]));
				}
			if (c == 0 || rcount[b] == 0)
				continue;
			float cost = __fadd_rn(1.0f, __fdiv_rn(__fadd_rn(__fmul_rn((float)c, sarea(mn, mx)),
				__fmul_rn((float)rcount[b], rarea[b])), sa_parent));
			if (cost < best_cost) {
				best_cost = cost;
				best_axis = axis;
				best_split = b;
			}
		}
	}
	d.axis = best_axis;
	d.split = best_split;
	d.leaf = (cnt <= 1u) || ((int)cnt <= max_leaf && (best_axis < 0 || (float)cnt <= best_cost));
	d.c0 = best_axis >= 0 ? cmn[best_axis] : 0.0f;
	d.scale = best_axis >= 0 ? __fdiv_rn((float)GB_BINS, __fsub_rn(cmx[best_axis], cmn[best_axis])) : 0.0f;
}

/* decisions of the large tasks, one thread per task; node bounds written */
__global__ void gb_decide(const Task *tasks, uint32_t ntasks, const TaskBounds *tb, const Bin *bins, int max_leaf,
		Decision *dec, TreeNode *nodes)
{
	uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= ntasks)
		return;
	float bmn[3], bmx[3], cmn[3], cmx[3];
	for (int k = 0; k < 3; k++) {
		bmn[k] = fdec(tb[t].v[k]);
		bmx[k] = fdec(tb[t].v[3 + k]);
		cmn[k] = fdec(tb[t].v[6 + k]);
		cmx[k] = fdec(tb[t].v[9 + k]);
	}
	TreeNode &nd = nodes[tasks[t].node];
	for (int k = 0; k < 3; k++) {
		nd.bmin[k] = bmn[k];
		nd.bmax[k] = bmx[k];
	}
	const Bin *ab[3] = {bins + (size_t)t * 3 * GB_BINS, bins + (size_t)t * 3 * GB_BINS + GB_BINS,
		bins + (size_t)t * 3 * GB_BINS + 2 * GB_BINS};
	choose_split(bmn, bmx, cmn, cmx, tasks[t].end - tasks[t].begin, max_leaf, ab, dec[t], sarea(bmn, bmx));
}

/* left counts of every chunk of a splitting task */
__global__ void __launch_bounds__(GB_BLOCK) gb_count_left(Boxes bx, const uint32_t *order, const Task *tasks,
		const uint32_t *chunk_task, const uint32_t *chunk_begin, const Decision *dec, uint32_t *chunk_left)
{
	uint32_t t = chunk_task[blockIdx.x];
	const Decision d = dec[t];
	__shared__ uint32_t s;
	if (threadIdx.x == 0)
		s = 0;
	__syncthreads();
	if (d.leaf || d.axis < 0) {
		if (threadIdx.x == 0)
			chunk_left[blockIdx.x] = 0;
		return;
	}
	uint32_t b0 = chunk_begin[blockIdx.x], b1 = min(b0 + GB_CHUNK, tasks[t].end);
	uint32_t c = 0;
	for (uint32_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
		float4 cv = bx.cen[order[i]];
		float cc[3] = {cv.x, cv.y, cv.z};
		c += bin_of(cc[d.axis], d.c0, d.scale) < d.split ? 1u : 0u;
	}
	atomicAdd(&s, c);
	__syncthreads();
	if (threadIdx.x == 0)
		chunk_left[blockIdx.x] = s;
}

/* stable scatter of one chunk: lefts to begin + left_before, rights to
 * mid + right_before (both in input order).  task_mid holds the mid with
 * bit 31 set when the task reorders (a split with lefts and rights); any
 * other task copies its range unchanged. */
__global__ void __launch_bounds__(GB_BLOCK) gb_scatter(Boxes bx, const uint32_t *order, uint32_t *out,
		const Task *tasks, const uint32_t *chunk_task, const uint32_t *chunk_begin, const Decision *dec,
		const uint32_t *chunk_left_before, const uint32_t *task_mid)
{
	uint32_t t = chunk_task[blockIdx.x];
	const Decision d = dec[t];
	const bool reorder = (task_mid[t] & 0x80000000u) != 0u;
	const uint32_t mid = task_mid[t] & 0x7FFFFFFFu;
	uint32_t tb0 = tasks[t].begin;
	uint32_t b0 = chunk_begin[blockIdx.x], b1 = min(b0 + GB_CHUNK, tasks[t].end);
	__shared__ uint32_t warp_sums[GB_BLOCK / 32];
	__shared__ uint32_t base_left;
	if (threadIdx.x == 0)
		base_left = chunk_left_before[blockIdx.x];
	__syncthreads();
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	for (uint32_t i0 = b0; i0 < b1; i0 += blockDim.x) {
		uint32_t i = i0 + threadIdx.x;
		bool in = i < b1;
		uint32_t p = in ? order[i] : 0u;
		bool left = false;
		if (in && reorder) {
			float4 cv = bx.cen[p];
			float cc[3] = {cv.x, cv.y, cv.z};
			left = bin_of(cc[d.axis], d.c0, d.scale) < d.split;
		}
		unsigned m = __ballot_sync(0xffffffffu, left);
		uint32_t rank = __popc(m & ((1u << lane) - 1u));
		if (lane == 0)
			warp_sums[warp] = __popc(m);
		__syncthreads();
		uint32_t before = 0, total = 0;
		for (int w = 0; w < GB_BLOCK / 32; w++) {
			before += w < warp ? warp_sums[w] : 0u;
			total += warp_sums[w];
		}
		if (in) {
			uint32_t lb = base_left + before + rank; /* lefts before i within the task */
			uint32_t dst;
			if (!reorder)
				dst = i;
			else if (left)
				dst = tb0 + lb;
			else
				dst = mid + ((i - tb0) - lb);
			out[dst] = p;
		}
		__syncthreads();
		if (threadIdx.x == 0)
			base_left += total;
		__syncthreads();
	}
}

__global__ void gb_copy(const uint32_t *src, uint32_t *dst, const Task *tasks, const uint32_t *chunk_task,
		const uint32_t *chunk_begin)
{
	uint32_t t = chunk_task[blockIdx.x];
	uint32_t b0 = chunk_begin[blockIdx.x], b1 = min(b0 + GB_CHUNK, tasks[t].end);
	for (uint32_t i = b0 + threadIdx.x; i < b1; i += blockDim.x)
		dst[i] = src[i];
}

/* links of the large tasks' nodes: children or leaf range */
__global__ void gb_link(const Task *tasks, uint32_t ntasks, const Decision *dec, const int32_t *child, TreeNode *nodes)
{
	uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= ntasks)
		return;
	TreeNode &nd = nodes[tasks[t].node];
	if (dec[t].leaf) {
		nd.left = nd.right = -1;
		nd.first = (int32_t)tasks[t].begin;
		nd.count = (int32_t)(tasks[t].end - tasks[t].begin);
	} else {
		nd.left = child[t];
		nd.right = child[t] + 1;
		nd.first = 0;
		nd.count = 0;
	}
}

/* A whole subtree of at most GB_SMALL primitives, one thread: the host
 * algorithm, with node ids drawn from *node_count and a stable partition
 * through `scratch`. */
__global__ void gb_small(Boxes bx, uint32_t *order, uint32_t *scratch, const Task *tasks, uint32_t ntasks,
		int max_leaf, TreeNode *nodes, uint32_t *node_count, uint32_t *overflow)
{
	uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= ntasks)
		return;
	Task stack[GB_STACK];
	int sp = 0;
	stack[sp++] = tasks[t];
	Bin bins[3][GB_BINS];
	while (sp > 0) {
		Task k = stack[--sp];
		TreeNode &nd = nodes[k.node];
		float bmn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, bmx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
		float cmn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, cmx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
		for (uint32_t i = k.begin; i < k.end; i++) {
			uint32_t p = order[i];
			float4 mn = bx.bmin[p], mx = bx.bmax[p], c = bx.cen[p];
			float a[3] = {mn.x, mn.y, mn.z}, b[3] = {mx.x, mx.y, mx.z}, cc[3] = {c.x, c.y, c.z};
			for (int q = 0; q < 3; q++) {
				bmn[q] = dmin(bmn[q], a[q]);
				bmx[q] = dmax(bmx[q], b[q]);
				cmn[q] = dmin(cmn[q], cc[q]);
				cmx[q] = dmax(cmx[q], cc[q]);
			}
		}
		for (int q = 0; q < 3; q++) {
			nd.bmin[q] = bmn[q];
			nd.bmax[q] = bmx[q];
		}
		uint32_t cnt = k.end - k.begin;
		Decision d;
		if (cnt <= 1u) {
			d.leaf = 1;
			d.axis = -1;
		} else {
			for (int a = 0; a < 3; a++) {
				for (int b = 0; b < GB_BINS; b++) {
					bins[a][b].count = 0;
					for (int q = 0; q < 3; q++) {
						bins[a][b].mn[q] = 0xFFFFFFFFu;
						bins[a][b].mx[q] = 0u;
					}
				}
				float ext = __fsub_rn(cmx[a], cmn[a]);
				if (!(ext > 0.0f))
					continue;
				float scale = __fdiv_rn((float)GB_BINS, ext);
				for (uint32_t i = k.begin; i < k.end; i++) {
					uint32_t p = order[i];
					float4 mn = bx.bmin[p], mx = bx.bmax[p], c = bx.cen[p];
					float cc[3] = {c.x, c.y, c.z};
					float a3[3] = {mn.x, mn.y, mn.z}, b3[3] = {mx.x, mx.y, mx.z};
					Bin &bn = bins[a][bin_of(cc[a], cmn[a], scale)];
					bn.count++;
					for (int q = 0; q < 3; q++) {
						bn.mn[q] = min(bn.mn[q], fenc(a3[q]));
						bn.mx[q] = max(bn.mx[q], fenc(b3[q]));
					}
				}
			}
			const Bin *ab[3] = {bins[0], bins[1], bins[2]};
			choose_split(bmn, bmx, cmn, cmx, cnt, max_leaf, ab, d, sarea(bmn, bmx));
		}
		if (d.leaf) {
			nd.left = nd.right = -1;
			nd.first = (int32_t)k.begin;
			nd.count = (int32_t)cnt;
			continue;
		}
		uint32_t mid = k.begin + cnt / 2u;
		if (d.axis >= 0) {
			uint32_t nl = 0;
			for (uint32_t i = k.begin; i < k.end; i++) {
				float4 c = bx.cen[order[i]];
				float cc[3] = {c.x, c.y, c.z};
				nl += bin_of(cc[d.axis], d.c0, d.scale) < d.split ? 1u : 0u;
			}
			if (nl != 0 && nl != cnt) {
				uint32_t li = k.begin, ri = k.begin + nl;
				for (uint32_t i = k.begin; i < k.end; i++) {
					uint32_t p = order[i];
					float4 c = bx.cen[p];
					float cc[3] = {c.x, c.y, c.z};
					if (bin_of(cc[d.axis], d.c0, d.scale) < d.split)
						scratch[li++] = p;
					else
						scratch[ri++] = p;
				}
				for (uint32_t i = k.begin; i < k.end; i++)
					order[i] = scratch[i];
				mid = k.begin + nl;
			}
		}
		int32_t l = (int32_t)atomicAdd(node_count, 2u);
		nd.left = l;
		nd.right = l + 1;
		nd.first = 0;
		nd.count = 0;
		if (sp + 2 > GB_STACK) {
			atomicOr(overflow, 1u);
			return;
		}
		stack[sp++] = Task{l + 1, mid, k.end};
		stack[sp++] = Task{l, k.begin, mid};
	}
}

template <class T>
T *dev_alloc(DevBuf<T> &b, size_t n)
{
	b.alloc(n ? n : 1);
	return b.ptr;
}

} /* namespace */

void build_sah_gpu(const std::vector<PrimBox> &boxes, int max_leaf, Tree &tree, cudaStream_t st)
{
	tree.nodes.clear();
	size_t n = boxes.size();
	tree.prim_order.resize(n);
	if (n == 0)
		return;
	KGR_REQUIRE(n < (1ull << 31), KGR_ERR_UNSUPPORTED, "too many primitives for the GPU builder");
	DevBuf<float> d_boxes;
	DevBuf<float4> d_bmin, d_bmax, d_cen;
	DevBuf<uint32_t> d_order, d_tmp, d_chunk_task, d_chunk_begin, d_chunk_left, d_task_mid, d_node_count,
		d_overflow;
	DevBuf<Task> d_tasks;
	DevBuf<TaskBounds> d_tb;
	DevBuf<Bin> d_bins;
	DevBuf<Decision> d_dec;
	DevBuf<int32_t> d_child;
	DevBuf<TreeNode> d_nodes;
	d_boxes.upload(reinterpret_cast<const float *>(boxes.data()), 6 * n);
	dev_alloc(d_bmin, n);
	dev_alloc(d_bmax, n);
	dev_alloc(d_cen, n);
	dev_alloc(d_order, n);
	dev_alloc(d_tmp, n);
	size_t max_nodes = 2 * n;
	dev_alloc(d_nodes, max_nodes);
	dev_alloc(d_node_count, 1);
	dev_alloc(d_overflow, 1);
	KGR_CUDA(cudaMemsetAsync(d_overflow.ptr, 0, 4, st));
	gb_init<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d_boxes.ptr, (uint32_t)n, d_bmin.ptr, d_bmax.ptr, d_cen.ptr,
		d_order.ptr);
	KGR_CUDA(cudaGetLastError());
	Boxes bx = {d_bmin.ptr, d_bmax.ptr, d_cen.ptr};

	uint32_t node_count = 1;
	std::vector<Task> large, small;
	(n > GB_SMALL ? large : small).push_back(Task{0, 0, (uint32_t)n});
	while (!large.empty()) {
		uint32_t nt = (uint32_t)large.size();
		/* chunk table */
		std::vector<uint32_t> ctask, cbegin;
		for (uint32_t t = 0; t < nt; t++)
			for (uint32_t b = large[t].begin; b < large[t].end; b += GB_CHUNK) {
				ctask.push_back(t);
				cbegin.push_back(b);
			}
		uint32_t nc = (uint32_t)ctask.size();
		d_tasks.upload(large);
		d_chunk_task.upload(ctask);
		d_chunk_begin.upload(cbegin);
		dev_alloc(d_tb, nt);
		dev_alloc(d_bins, (size_t)nt * 3 * GB_BINS);
		dev_alloc(d_dec, nt);
		dev_alloc(d_chunk_left, nc);
		gb_reset_bounds<<<nt, 128, 0, st>>>(d_tb.ptr, d_bins.ptr, nt);
		gb_bounds<<<nc, GB_BLOCK, 0, st>>>(bx, d_order.ptr, d_tasks.ptr, d_chunk_task.ptr, d_chunk_begin.ptr, d_tb.ptr);
		gb_bins<<<nc, GB_BLOCK, 0, st>>>(bx, d_order.ptr, d_tasks.ptr, d_chunk_task.ptr, d_chunk_begin.ptr, d_tb.ptr,
			d_bins.ptr);
		gb_decide<<<(nt + 127) / 128, 128, 0, st>>>(d_tasks.ptr, nt, d_tb.ptr, d_bins.ptr, max_leaf, d_dec.ptr,
			d_nodes.ptr);
		gb_count_left<<<nc, GB_BLOCK, 0, st>>>(bx, d_order.ptr, d_tasks.ptr, d_chunk_task.ptr, d_chunk_begin.ptr,
			d_dec.ptr, d_chunk_left.ptr);
		KGR_CUDA(cudaGetLastError());
		std::vector<Decision> dec(nt);
		std::vector<uint32_t> cleft(nc);
		KGR_CUDA(cudaMemcpyAsync(dec.data(), d_dec.ptr, nt * sizeof(Decision), cudaMemcpyDeviceToHost, st));
		KGR_CUDA(cudaMemcpyAsync(cleft.data(), d_chunk_left.ptr, nc * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
		KGR_CUDA(cudaStreamSynchronize(st));
		/* segmented exclusive scan of left counts; mid of every task */
		std::vector<uint32_t> before(nc), mid(nt);
		std::vector<uint32_t> total(nt, 0);
		for (uint32_t c = 0; c < nc; c++) {
			before[c] = total[ctask[c]];
			total[ctask[c]] += cleft[c];
		}
		std::vector<int32_t> child(nt, -1);
		std::vector<Task> next;
		std::vector<uint32_t> mid_flag(nt);
		for (uint32_t t = 0; t < nt; t++) {
			const Task &k = large[t];
			uint32_t cnt = k.end - k.begin;
			mid[t] = k.begin + cnt / 2u; /* no usable axis, or all on one side: split by index */
			bool reorder = !dec[t].leaf && dec[t].axis >= 0 && total[t] != 0 && total[t] != cnt;
			if (reorder)
				mid[t] = k.begin + total[t];
			mid_flag[t] = mid[t] | (reorder ? 0x80000000u : 0u);
			if (dec[t].leaf)
				continue;
			child[t] = (int32_t)node_count;
			node_count += 2;
			Task lt = {child[t], k.begin, mid[t]}, rt = {child[t] + 1, mid[t], k.end};
			(lt.end - lt.begin > GB_SMALL ? next : small).push_back(lt);
			(rt.end - rt.begin > GB_SMALL ? next : small).push_back(rt);
		}
		d_chunk_left.upload(before);
		d_task_mid.upload(mid_flag);
		d_child.upload(child);
		gb_scatter<<<nc, GB_BLOCK, 0, st>>>(bx, d_order.ptr, d_tmp.ptr, d_tasks.ptr, d_chunk_task.ptr,
			d_chunk_begin.ptr, d_dec.ptr, d_chunk_left.ptr, d_task_mid.ptr);
		gb_copy<<<nc, GB_BLOCK, 0, st>>>(d_tmp.ptr, d_order.ptr, d_tasks.ptr, d_chunk_task.ptr, d_chunk_begin.ptr);
		gb_link<<<(nt + 127) / 128, 128, 0, st>>>(d_tasks.ptr, nt, d_dec.ptr, d_child.ptr, d_nodes.ptr);
		KGR_CUDA(cudaGetLastError());
		KGR_REQUIRE(node_count + 2 <= max_nodes, KGR_ERR_INTERNAL, "GPU builder: node overflow");
		large.swap(next);
	}
	if (!small.empty()) {
		uint32_t ns = (uint32_t)small.size();
		d_tasks.upload(small);
		KGR_CUDA(cudaMemcpyAsync(d_node_count.ptr, &node_count, 4, cudaMemcpyHostToDevice, st));
		gb_small<<<(ns + 63) / 64, 64, 0, st>>>(bx, d_order.ptr, d_tmp.ptr, d_tasks.ptr, ns, max_leaf, d_nodes.ptr,
			d_node_count.ptr, d_overflow.ptr);
		KGR_CUDA(cudaGetLastError());
		KGR_CUDA(cudaMemcpyAsync(&node_count, d_node_count.ptr, 4, cudaMemcpyDeviceToHost, st));
	}
	uint32_t overflow = 0;
	KGR_CUDA(cudaMemcpyAsync(&overflow, d_overflow.ptr, 4, cudaMemcpyDeviceToHost, st));
	KGR_CUDA(cudaStreamSynchronize(st));
	KGR_REQUIRE(!overflow, KGR_ERR_UNSUPPORTED, "GPU builder: subtree deeper than its stack");
	tree.nodes.resize(node_count);
	KGR_CUDA(cudaMemcpyAsync(tree.nodes.data(), d_nodes.ptr, node_count * sizeof(TreeNode), cudaMemcpyDeviceToHost,
		st));
	KGR_CUDA(cudaMemcpyAsync(tree.prim_order.data(), d_order.ptr, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
	KGR_CUDA(cudaStreamSynchronize(st));
}

} /* namespace kgr */

/*
 * kgr_device.cuh -- device functions of the hot path: BVH traversal of both
 * layouts, hit reconstruction, light sampling, the GGX BSDF and reservoirs.
 *
 * Compiled with -fmad=false, -prec-div=true, -prec-sqrt=true and without
 * flush-to-zero, so every expression rounds exactly as written.  The
 * evaluation order of each expression is the reference's (cited per
 * function); that keeps hit ids, bounce directions, Russian-roulette
 * decisions and reservoir selections identical to the CPU restatement.
 * The fast-layout slab test is the one place that uses explicit FMA
 * (__fmaf_rn): its boxes are padded at build time so that culling stays
 * conservative, and it only decides which triangles get tested.
 */
#ifndef KGR_DEVICE_CUH_
#define KGR_DEVICE_CUH_

#include "kgr_internal.h"
#include "kgr_math.h"

namespace kgr {

#define KGR_STACK_DEPTH KGR_STACK_DEPTH_HOST

__device__ __forceinline__ f3 f3_of(float4 v) { return mk(v.x, v.y, v.z); }
__device__ __forceinline__ float4 f4_of(f3 v, float w) { return make_float4(v.x, v.y, v.z, w); }
__device__ __forceinline__ int32_t ibits(float f) { return __float_as_int(f); }
__device__ __forceinline__ float fbits(int32_t i) { return __int_as_float(i); }

/* ----------------------------------------------------------- triangles -- */

/* intersects_triangle (include/optix/lighting.cuh:34-55) with the edges
 * e1 = v2 - v1, e2 = v3 - v1 given (computed by the same float
 * subtraction on the host). 1.0/divisor as a float IEEE division equals the
 * reference's double division rounded to float. */
__device__ __forceinline__ float mt_test(const f3 &v1, const f3 &e1, const f3 &e2,
		const f3 &origin, const f3 &dir, float &b1, float &b2)
{
	f3 s1 = cross(dir, e2);
	float divisor = dot(s1, e1);
	if (divisor == 0.0f)
		return -1.0f;
	f3 s = origin - v1;
	float d1 = dot(s, s1);
	/* Early reject without the division, only where b1 = d1 * (1/divisor)
	 * must fail the reference's test: for a finite divisor, opposite signs
	 * and |d1| >= 2^-60 |divisor| make b1 a normal negative number, and equal
	 * signs with |d1| > (1 + 2^-10) |divisor| make it greater than 1 after
	 * both roundings. */
	{
		float ad = fabsf(divisor), a1 = fabsf(d1);
		if (ad < INFINITY) {
			bool opposite = (d1 < 0.0f) != (divisor < 0.0f);
			if (opposite ? (d1 != 0.0f && a1 >= ad * 8.67361738e-19f) : (a1 > ad * 1.0009765625f))
				return -1.0f;
		}
	}
	float inv_divisor = 1.0f / divisor;
	b1 = d1 * inv_divisor;
	if (b1 < 0.0f || b1 > 1.0f)
		return -1.0f;
	f3 s2 = cross(s, e1);
	b2 = dot(dir, s2) * inv_divisor;
	if (b2 < 0.0f || b1 + b2 > 1.0f)
		return -1.0f;
	return dot(e2, s2) * inv_divisor;
}

/* ---------------------------------------------------- threaded layout -- */

/* intersect_box (shaders/rt/modules/bbox.glsl:8-58), IEEE divisions */
__device__ __forceinline__ float slab_box(const f3 &o, const f3 &d, const f3 &pmin, const f3 &pmax)
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
__device__ __forceinline__ bool origin_in_box(const f3 &p, const f3 &pmin, const f3 &pmax)
{
	bool lt = p.x < pmin.x || p.y < pmin.y || p.z < pmin.z;
	bool gt = p.x > pmax.x || p.y > pmax.y || p.z > pmax.z;
	return !(lt || gt);
}

struct TraceCounters {
	uint32_t nodes, tris;
};

/* trace() (shaders/rt/modules/bvh.glsl:52-99): the stackless threaded walk
 * over 3-vec4 records.  ANY: stop at the first primitive with 0 < t < tmax
 * (is_occluded, amadeus_common.cuh:190-212). */
template <bool ANY, bool COUNT>
__device__ __forceinline__ bool trace_threaded(const DeviceScene &s, const f3 &o, const f3 &d,
		float tmax, kgr_hit &best, TraceCounters *cnt = nullptr)
{
	best.prim = -1;
	best.t = tmax;
	best.b1 = 0.0f;
	best.b2 = 0.0f;
	int32_t node = s.bvh_vec4_count ? 0 : -1;
	while (node != -1) {
		float4 h = __ldg(&s.bvh[node]);
		int32_t object = ibits(h.y);
		if (object != -1) {
			if (COUNT)
				cnt->tris++;
			uint4 t = __ldg(&s.tris[object]);
			f3 v1 = f3_of(__ldg(&s.positions[t.x]));
			f3 v2 = f3_of(__ldg(&s.positions[t.y]));
			f3 v3 = f3_of(__ldg(&s.positions[t.z]));
			float b1 = 0.0f, b2 = 0.0f;
			float tt = mt_test(v1, v2 - v1, v3 - v1, o, d, b1, b2);
			if (tt > 0.0f && tt < best.t) {
				if (ANY)
					return true;
				best.prim = object;
				best.t = tt;
				best.b1 = b1;
				best.b2 = b2;
			}
			node = ibits(h.w);
		} else {
			if (COUNT)
				cnt->nodes++;
			f3 pmin = f3_of(__ldg(&s.bvh[node + 1]));
			f3 pmax = f3_of(__ldg(&s.bvh[node + 2]));
			float tb = slab_box(o, d, pmin, pmax);
			bool inside = origin_in_box(o, pmin, pmax);
			node = ((tb > 0.0f && tb < best.t) || inside) ? ibits(h.z) : ibits(h.w);
		}
	}
	return best.prim >= 0;
}

/* -------------------------------------------------------- fast layout -- */

/* A ray prepared for the slab tests of the fast layout.  A zero direction
 * component would give an infinite reciprocal, and lo * inf - o * inf turns
 * into NaN for the far plane; a tiny stand-in keeps every slab finite and the
 * interval of a parallel ray unbounded (inside the slab) or out of reach
 * (outside it). */
struct FastRay {
	f3 o, d;
	float ix, iy, iz, ox, oy, oz;
};

__device__ __forceinline__ FastRay fast_ray(const f3 &o, const f3 &d)
{
	FastRay r;
	r.o = o;
	r.d = d;
	r.ix = 1.0f / (fabsf(d.x) > 1e-20f ? d.x : copysignf(1e-20f, d.x));
	r.iy = 1.0f / (fabsf(d.y) > 1e-20f ? d.y : copysignf(1e-20f, d.y));
	r.iz = 1.0f / (fabsf(d.z) > 1e-20f ? d.z : copysignf(1e-20f, d.z));
	r.ox = o.x * r.ix;
	r.oy = o.y * r.iy;
	r.oz = o.z * r.iz;
	return r;
}

/* 32-byte load through the read-only path: one 256-bit vector load
 * (ld.global.nc.v8.f32, sm_100 and later) instead of two 128-bit ones.  p
 * must be 32-byte aligned: node arrays come from cudaMalloc (256-byte
 * aligned) and nodes are 64 or 128 bytes, which the scene build checks. */
__device__ __forceinline__ void ldg256(const float4 *p, float4 &a, float4 &b)
{
	asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
		: "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
		: "l"(p));
}

/* One child-pair node: which children the ray reaches within [0, best_t],
 * nearer one first.  Returns the number of children hit (0, 1 or 2). */
__device__ __forceinline__ int fast_node(const DeviceScene &s, const FastRay &r, int32_t ref, float best_t,
		int32_t &first, int32_t &second)
{
	const float4 *np = reinterpret_cast<const float4 *>(s.fast_nodes + ref);
	float4 lxy, rxy, lrz, rv;
	ldg256(np, lxy, rxy);
	ldg256(np + 2, lrz, rv);
	int4 refs = make_int4(__float_as_int(rv.x), __float_as_int(rv.y), __float_as_int(rv.z), __float_as_int(rv.w));
	float l0x = __fmaf_rn(lxy.x, r.ix, -r.ox), l1x = __fmaf_rn(lxy.y, r.ix, -r.ox);
	float l0y = __fmaf_rn(lxy.z, r.iy, -r.oy), l1y = __fmaf_rn(lxy.w, r.iy, -r.oy);
	float l0z = __fmaf_rn(lrz.x, r.iz, -r.oz), l1z = __fmaf_rn(lrz.y, r.iz, -r.oz);
	float r0x = __fmaf_rn(rxy.x, r.ix, -r.ox), r1x = __fmaf_rn(rxy.y, r.ix, -r.ox);
	float r0y = __fmaf_rn(rxy.z, r.iy, -r.oy), r1y = __fmaf_rn(rxy.w, r.iy, -r.oy);
	float r0z = __fmaf_rn(lrz.z, r.iz, -r.oz), r1z = __fmaf_rn(lrz.w, r.iz, -r.oz);
	float ln = fmaxf(fmaxf(fminf(l0x, l1x), fminf(l0y, l1y)), fmaxf(fminf(l0z, l1z), 0.0f));
	float lf = fminf(fminf(fmaxf(l0x, l1x), fmaxf(l0y, l1y)), fmaxf(l0z, l1z));
	float rn = fmaxf(fmaxf(fminf(r0x, r1x), fminf(r0y, r1y)), fmaxf(fminf(r0z, r1z), 0.0f));
	float rf = fminf(fminf(fmaxf(r0x, r1x), fmaxf(r0y, r1y)), fmaxf(r0z, r1z));
	bool hl = ln <= lf && ln <= best_t;
	bool hr = rn <= rf && rn <= best_t;
	if (hl && hr) {
		bool swap = rn < ln;
		first = swap ? refs.y : refs.x;
		second = swap ? refs.x : refs.y;
		return 2;
	}
	first = hl ? refs.x : refs.y;
	return (hl || hr) ? 1 : 0;
}

/* One triangle (record `idx` of the walk-ordered triangle array).  Closest
 * hit: it replaces the best when 0 < t < best, or t == best and its rank
 * (position in the threaded walk) is lower -- the primitive the reference's
 * strict `t < best` walk keeps.  Any hit: returns true when 0 < t < tmax. */
template <bool ANY, bool COUNT>
__device__ __forceinline__ bool fast_triangle(const DeviceScene &s, const FastRay &r, uint32_t idx,
		kgr_hit &best, int32_t &best_rank, TraceCounters *cnt)
{
	if (COUNT)
		cnt->tris++;
	const float4 *tp = s.fast_tris + 3 * (size_t)idx;
	float4 a = __ldg(tp + 0);
	float4 e1 = __ldg(tp + 1);
	float4 e2 = __ldg(tp + 2);
	float b1 = 0.0f, b2 = 0.0f;
	float tt = mt_test(f3_of(a), f3_of(e1), f3_of(e2), r.o, r.d, b1, b2);
	if (ANY) {
		if (tt > 0.0f && tt < best.t) {
			best.prim = ibits(a.w);
			best.t = tt;
			return true;
		}
		return false;
	}
	int32_t rank = (int32_t)idx;
	if (tt > 0.0f && (tt < best.t || (tt == best.t && rank < best_rank))) {
		best.prim = ibits(a.w);
		best.t = tt;
		best.b1 = b1;
		best.b2 = b2;
		best_rank = rank;
	}
	return false;
}

/* The triangles of one leaf (fast_triangle for each).  Any hit: returns true
 * at the first triangle with 0 < t < tmax. */
template <bool ANY, bool COUNT>
__device__ __forceinline__ bool fast_leaf(const DeviceScene &s, const FastRay &r, int32_t ref, kgr_hit &best,
		int32_t &best_rank, TraceCounters *cnt)
{
	uint32_t code = ~(uint32_t)ref;
	uint32_t start = code >> 3, n = (code & 7u) + 1u;
	for (uint32_t k = 0; k < n; k++)
		if (fast_triangle<ANY, COUNT>(s, r, start + k, best, best_rank, cnt))
			return true;
	return false;
}

/* Slab test of one child of a wide node, the arithmetic of fast_node:
 * its near distance when the ray reaches the padded box within
 * [0, best_t], +inf otherwise (or for an unused slot). */
__device__ __forceinline__ float wide_child(const FastRay &r, float lx, float hx, float ly, float hy, float lz,
		float hz, int32_t ref, float best_t)
{
	float x0 = __fmaf_rn(lx, r.ix, -r.ox), x1 = __fmaf_rn(hx, r.ix, -r.ox);
	float y0 = __fmaf_rn(ly, r.iy, -r.oy), y1 = __fmaf_rn(hy, r.iy, -r.oy);
	float z0 = __fmaf_rn(lz, r.iz, -r.oz), z1 = __fmaf_rn(hz, r.iz, -r.oz);
	float tn = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fmaxf(fminf(z0, z1), 0.0f));
	float tf = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fmaxf(z0, z1));
	return (ref != KGR_WIDE_EMPTY && tn <= tf && tn <= best_t) ? tn : __int_as_float(0x7f800000);
}

/* Order two (distance, reference) pairs, nearer first. */
__device__ __forceinline__ void order_pair(float &ta, int32_t &ca, float &tb, int32_t &cb)
{
	bool s = tb < ta;
	float t = s ? tb : ta;
	int32_t c = s ? cb : ca;
	tb = s ? ta : tb;
	cb = s ? ca : cb;
	ta = t;
	ca = c;
}

/* Per-thread traversal stack in local memory: `a` is the caller's array of
 * KGR_STACK_DEPTH entries (the builder rejects trees whose walk could need
 * more).  The object holds only the pointer and the depth, so the depth
 * stays in a register. */
struct LocalStack {
	int32_t *a;
	int sp;
	__device__ __forceinline__ LocalStack(int32_t *shared_column, int32_t *local) : a(local), sp(0)
	{
		(void)shared_column;
	}
	__device__ __forceinline__ bool empty() const { return sp == 0; }
	__device__ __forceinline__ void clear() { sp = 0; }
	__device__ __forceinline__ void push(int32_t v) { a[sp++] = v; }
	__device__ __forceinline__ int32_t pop() { return a[--sp]; }
};

/* Short stack: the first SHORT entries of each thread in shared memory,
 * deeper ones in the caller's local array of KGR_STACK_DEPTH - SHORT.
 * `col` is the thread's column of a SHORT x BLOCK block array: entry k of
 * thread t sits at k * BLOCK + t, so the 32 lanes of a warp touch 32
 * different banks whatever depths they are at. */
template <int SHORT, int BLOCK>
struct ShortStack {
	int32_t *col;
	int32_t *deep;
	int sp;
	__device__ __forceinline__ ShortStack(int32_t *column, int32_t *local) : col(column), deep(local), sp(0) {}
	__device__ __forceinline__ bool empty() const { return sp == 0; }
	__device__ __forceinline__ void clear() { sp = 0; }
	__device__ __forceinline__ void push(int32_t v)
	{
		if (sp < SHORT)
			col[sp * BLOCK] = v;
		else
			deep[sp - SHORT] = v;
		sp++;
	}
	__device__ __forceinline__ int32_t pop()
	{
		--sp;
		return sp < SHORT ? col[sp * BLOCK] : deep[sp - SHORT];
	}
};

/* One interior node of the fast (BVH2) or wide (BVH4) layout: `ref`
 * becomes the nearest child whose padded box the ray reaches within
 * [0, best_t] and the other reached children are pushed, farthest first;
 * with none reached, `ref` is popped.  Returns false when there was nothing
 * to pop: the walk is over. */
template <int LAYOUT, class STACK>
__device__ __forceinline__ bool node_step(const DeviceScene &s, const FastRay &r, int32_t &ref, float best_t,
		STACK &stack)
{
	if (LAYOUT == KGR_LAYOUT_WIDE) {
		const float4 *np = reinterpret_cast<const float4 *>(s.wide_nodes + ref);
		float4 lx, hx, ly, hy, lz, hz, rr, unused;
		ldg256(np + 0, lx, hx);
		ldg256(np + 2, ly, hy);
		ldg256(np + 4, lz, hz);
		ldg256(np + 6, rr, unused);
		int4 rf = make_int4(__float_as_int(rr.x), __float_as_int(rr.y), __float_as_int(rr.z), __float_as_int(rr.w));
		float t0 = wide_child(r, lx.x, hx.x, ly.x, hy.x, lz.x, hz.x, rf.x, best_t);
		float t1 = wide_child(r, lx.y, hx.y, ly.y, hy.y, lz.y, hz.y, rf.y, best_t);
		float t2 = wide_child(r, lx.z, hx.z, ly.z, hy.z, lz.z, hz.z, rf.z, best_t);
		float t3 = wide_child(r, lx.w, hx.w, ly.w, hy.w, lz.w, hz.w, rf.w, best_t);
		int32_t c0 = rf.x, c1 = rf.y, c2 = rf.z, c3 = rf.w;
		order_pair(t0, c0, t1, c1);
		order_pair(t2, c2, t3, c3);
		order_pair(t0, c0, t2, c2);
		order_pair(t1, c1, t3, c3);
		order_pair(t1, c1, t2, c2);
		const float inf = __int_as_float(0x7f800000);
		if (!(t0 < inf)) {
			if (stack.empty())
				return false;
			ref = stack.pop();
			return true;
		}
		if (t3 < inf)
			stack.push(c3);
		if (t2 < inf)
			stack.push(c2);
		if (t1 < inf)
			stack.push(c1);
		ref = c0;
		return true;
	}
	int32_t first, second;
	int hits = fast_node(s, r, ref, best_t, first, second);
	if (hits == 2) {
		stack.push(second);
		ref = first;
	} else if (hits == 1) {
		ref = first;
	} else {
		if (stack.empty())
			return false;
		ref = stack.pop();
	}
	return true;
}

/* Ordered descent over the fast (64-byte child-pair) or wide (128-byte
 * four-child) nodes with a per-thread stack.  Box culling keeps every child
 * whose padded slab interval reaches [0, best]; the build pads boxes so that
 * no triangle the exact test accepts is culled.  Both layouts share the
 * triangle records, so they return the same hit. */
/* A walk with nothing left to visit. */
#define KGR_REF_NONE ((int32_t)0x80000000)

/* Descend until every active lane of the warp holds a leaf, or has no node
 * left (the postponed-leaf traversal of Aila and Laine, "Understanding the
 * Efficiency of Ray Traversal on GPUs", HPG 2009).  A lane that reaches a
 * leaf parks it in `leaf` and keeps descending from the next stacked node
 * while other lanes are still looking for theirs, so the warp then tests
 * leaves together instead of alternating between node steps and triangle
 * tests lane by lane.  On return `leaf` is 0 or a parked leaf, and `ref` is
 * an interior node (the lane ran ahead), a second leaf, or KGR_REF_NONE.
 * The extra nodes a lane visits ahead are culled against a best distance
 * that its parked leaf may still shorten, so the walk tests a superset of
 * the nodes and triangles of the plain order; the closest hit, a minimum
 * over (t, rank), and occlusion are unchanged. */
template <int LAYOUT, bool COUNT, class STACK>
__device__ __forceinline__ void speculative_descend(const DeviceScene &s, const FastRay &r, int32_t &ref,
		int32_t &leaf, float best_t, STACK &stack, TraceCounters *cnt)
{
	for (;;) {
		if (ref >= 0) {
			if (COUNT)
				cnt->nodes++;
			if (!node_step<LAYOUT>(s, r, ref, best_t, stack))
				ref = KGR_REF_NONE;
		}
		if (ref < 0 && ref != KGR_REF_NONE && leaf == 0) {
			leaf = ref;
			ref = stack.empty() ? KGR_REF_NONE : stack.pop();
		}
		/* a lane stops only once it holds a leaf or is out of nodes, so the
		 * vote over the lanes executing here never ends another lane's
		 * search early */
		if (!__any_sync(__activemask(), leaf == 0 && ref >= 0))
			return;
	}
}

/* Test the parked leaf and, when the descent stopped on a second one, that
 * one too (then take the next stacked node).  Returns true on an occluding
 * hit (ANY). */
template <bool ANY, bool COUNT, class STACK>
__device__ __forceinline__ bool test_leaves(const DeviceScene &s, const FastRay &r, int32_t &ref, int32_t leaf,
		kgr_hit &best, int32_t &best_rank, STACK &stack, TraceCounters *cnt)
{
	if (leaf != 0 && fast_leaf<ANY, COUNT>(s, r, leaf, best, best_rank, cnt))
		return true;
	if (ref < 0 && ref != KGR_REF_NONE) {
		if (fast_leaf<ANY, COUNT>(s, r, ref, best, best_rank, cnt))
			return true;
		ref = stack.empty() ? KGR_REF_NONE : stack.pop();
	}
	return false;
}

template <bool ANY, bool COUNT, int LAYOUT, class STACK>
__device__ __forceinline__ bool trace_fast_stack(const DeviceScene &s, const f3 &o, const f3 &d,
		float tmax, kgr_hit &best, STACK &stack, TraceCounters *cnt = nullptr)
{
	best.prim = -1;
	best.t = tmax;
	best.b1 = 0.0f;
	best.b2 = 0.0f;
	int32_t best_rank = 0x7fffffff;
	FastRay r = fast_ray(o, d);
	stack.clear();
	int32_t ref = 0;
	for (;;) {
		int32_t leaf = 0;
		speculative_descend<LAYOUT, COUNT>(s, r, ref, leaf, best.t, stack, cnt);
		if (test_leaves<ANY, COUNT>(s, r, ref, leaf, best, best_rank, stack, cnt))
			return true;
		if (ref == KGR_REF_NONE)
			return best.prim >= 0;
	}
}

/* ------------------------------------------------- compressed layout -- */

/* The walk of the compressed eight-child layout (CwNode), after Ylitie,
 * Karras and Laine (HPG 2017).  A node group {first internal child, bits}
 * holds in bits 24-31 the internal children a node visit found reached, in
 * visiting order (highest bit first), and in bits 0-7 the node's imask;
 * slot j of a node sits at bit 24 + (j ^ oi), oi = 7 ^ octant, so slot
 * `octant` comes first.  A triangle group {first record, mask} holds the
 * reached leaves' triangles.  The stack holds node groups only. */
struct CwStack {
	uint2 a[KGR_CW_STACK];
	int sp;
	__device__ __forceinline__ bool empty() const { return sp == 0; }
	__device__ __forceinline__ void clear() { sp = 0; }
	__device__ __forceinline__ void push(uint2 v) { a[sp++] = v; }
	__device__ __forceinline__ uint2 pop() { return a[--sp]; }
};

struct CwWalk {
	FastRay r;
	uint32_t oi;
	uint2 node;           /* the node group being expanded */
	uint2 park, cur;      /* triangle groups: the postponed one and the one that stopped the descent */
};

__device__ __forceinline__ void cw_begin(CwWalk &w, const f3 &o, const f3 &d, CwStack &stack)
{
	w.r = fast_ray(o, d);
	uint32_t oct = (w.r.ix < 0.0f ? 1u : 0u) | (w.r.iy < 0.0f ? 2u : 0u) | (w.r.iz < 0.0f ? 4u : 0u);
	w.oi = 7u ^ oct;
	/* the root as the only reached child of a group with imask 0: rank 0 */
	w.node = make_uint2(0u, 0x80000000u);
	w.park = make_uint2(0u, 0u);
	w.cur = make_uint2(0u, 0u);
	stack.clear();
}

__device__ __forceinline__ float cw_byte(uint32_t lo4, uint32_t hi4, int j)
{
	uint32_t w = j < 4 ? lo4 : hi4;
	return __uint2float_rn((w >> (8 * (j & 3))) & 0xffu);
}

/* One node: the reached internal children become the node group, the
 * reached leaves' triangles a triangle group.  A child is reached when its
 * quantised box meets [0, best_t]: the slab planes are p + q 2^e, and
 * (p + q 2^e - o) / d is evaluated as q (2^e / d) + (p - o) / d. */
__device__ __forceinline__ void cw_visit(const DeviceScene &s, const CwWalk &w, uint32_t child, float best_t,
		uint2 &node, uint2 &tris)
{
	const float4 *np = reinterpret_cast<const float4 *>(s.cw_nodes + child);
	float4 o4 = __ldg(np);
	float4 b4 = __ldg(np + 1), a4 = __ldg(np + 2), c4 = __ldg(np + 3), d4 = __ldg(np + 4);
	uint4 base = make_uint4(__float_as_uint(b4.x), __float_as_uint(b4.y), __float_as_uint(b4.z), __float_as_uint(b4.w));
	uint4 qa = make_uint4(__float_as_uint(a4.x), __float_as_uint(a4.y), __float_as_uint(a4.z), __float_as_uint(a4.w));
	uint4 qb = make_uint4(__float_as_uint(c4.x), __float_as_uint(c4.y), __float_as_uint(c4.z), __float_as_uint(c4.w));
	uint4 qc = make_uint4(__float_as_uint(d4.x), __float_as_uint(d4.y), __float_as_uint(d4.z), __float_as_uint(d4.w));
	uint32_t eb = __float_as_uint(o4.w);
	uint32_t imask = eb >> 24;
	float scx = __uint_as_float((eb & 0xffu) << 23) * w.r.ix;
	float scy = __uint_as_float(((eb >> 8) & 0xffu) << 23) * w.r.iy;
	float scz = __uint_as_float(((eb >> 16) & 0xffu) << 23) * w.r.iz;
	float adx = (o4.x - w.r.o.x) * w.r.ix;
	float ady = (o4.y - w.r.o.y) * w.r.iy;
	float adz = (o4.z - w.r.o.z) * w.r.iz;
	uint32_t hits = 0u, tmask = 0u;
#pragma unroll
	for (int j = 0; j < 8; j++) {
		uint32_t meta = ((j < 4 ? base.z : base.w) >> (8 * (j & 3))) & 0xffu;
		bool internal = (imask >> j) & 1u;
		if (!internal && meta == 0u)
			continue;
		float x0 = __fmaf_rn(cw_byte(qa.x, qa.y, j), scx, adx), x1 = __fmaf_rn(cw_byte(qb.z, qb.w, j), scx, adx);
		float y0 = __fmaf_rn(cw_byte(qa.z, qa.w, j), scy, ady), y1 = __fmaf_rn(cw_byte(qc.x, qc.y, j), scy, ady);
		float z0 = __fmaf_rn(cw_byte(qb.x, qb.y, j), scz, adz), z1 = __fmaf_rn(cw_byte(qc.z, qc.w, j), scz, adz);
		float tn = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fmaxf(fminf(z0, z1), 0.0f));
		float tf = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fmaxf(z0, z1));
		if (tn <= tf && tn <= best_t) {
			if (internal)
				hits |= 1u << (24u + ((uint32_t)j ^ w.oi));
			else
				tmask |= ((1u << (meta >> 5)) - 1u) << (meta & 31u);
		}
	}
	node = make_uint2(base.x, hits | imask);
	tris = make_uint2(base.y, tmask);
}

/* One triangle record of the compressed layout: fast_triangle with the walk
 * rank read from the record. */
template <bool ANY, bool COUNT>
__device__ __forceinline__ bool cw_triangle(const DeviceScene &s, const FastRay &r, uint32_t idx, kgr_hit &best,
		int32_t &best_rank, TraceCounters *cnt)
{
	if (COUNT)
		cnt->tris++;
	const float4 *tp = s.cw_tris + 3 * (size_t)idx;
	float4 a = __ldg(tp + 0);
	float4 e1 = __ldg(tp + 1);
	float4 e2 = __ldg(tp + 2);
	float b1 = 0.0f, b2 = 0.0f;
	float tt = mt_test(f3_of(a), f3_of(e1), f3_of(e2), r.o, r.d, b1, b2);
	if (ANY) {
		if (tt > 0.0f && tt < best.t) {
			best.prim = ibits(a.w);
			best.t = tt;
			return true;
		}
		return false;
	}
	int32_t rank = __float_as_int(e1.w);
	if (tt > 0.0f && (tt < best.t || (tt == best.t && rank < best_rank))) {
		best.prim = ibits(a.w);
		best.t = tt;
		best.b1 = b1;
		best.b2 = b2;
		best_rank = rank;
	}
	return false;
}

template <bool ANY, bool COUNT>
__device__ __forceinline__ bool cw_triangles(const DeviceScene &s, const FastRay &r, uint2 &g, kgr_hit &best,
		int32_t &best_rank, TraceCounters *cnt)
{
	while (g.y) {
		uint32_t k = (uint32_t)__ffs(g.y) - 1u;
		g.y &= g.y - 1u;
		if (cw_triangle<ANY, COUNT>(s, r, g.x + k, best, best_rank, cnt))
			return true;
	}
	return false;
}

/* One step of the walk: descend with the postponed-leaf rule (a lane parks
 * its first triangle group and keeps descending until it finds a second
 * one, or runs out of nodes, while any lane of the warp is still looking),
 * then test the held triangles.  Returns true on an occluding hit (ANY);
 * `done` when nothing is left to visit. */
template <bool ANY, bool COUNT>
__device__ __forceinline__ bool cw_step(const DeviceScene &s, CwWalk &w, kgr_hit &best, int32_t &best_rank,
		CwStack &stack, TraceCounters *cnt, bool &done)
{
	for (;;) {
		if (w.cur.y == 0u) {
			if (w.node.y & 0xff000000u) {
				uint32_t b = 31u - (uint32_t)__clz(w.node.y);
				uint32_t slot = (b - 24u) ^ w.oi;
				w.node.y &= ~(1u << b);
				uint32_t child = w.node.x + (uint32_t)__popc(w.node.y & 0xffu & ((1u << slot) - 1u));
				if (w.node.y & 0xff000000u)
					stack.push(w.node);
				if (COUNT)
					cnt->nodes++;
				uint2 t;
				cw_visit(s, w, child, best.t, w.node, t);
				if (t.y) {
					if (w.park.y == 0u)
						w.park = t;
					else
						w.cur = t;
				}
			} else if (!stack.empty()) {
				w.node = stack.pop();
			}
		}
		bool looking = w.cur.y == 0u && ((w.node.y & 0xff000000u) || !stack.empty());
		if (!__any_sync(__activemask(), looking))
			break;
	}
	if (cw_triangles<ANY, COUNT>(s, w.r, w.park, best, best_rank, cnt))
		return true;
	if (cw_triangles<ANY, COUNT>(s, w.r, w.cur, best, best_rank, cnt))
		return true;
	done = !(w.node.y & 0xff000000u) && stack.empty();
	return false;
}

template <bool ANY, bool COUNT>
__device__ __forceinline__ bool trace_cw(const DeviceScene &s, const f3 &o, const f3 &d, float tmax, kgr_hit &best,
		TraceCounters *cnt = nullptr)
{
	best.prim = -1;
	best.t = tmax;
	best.b1 = 0.0f;
	best.b2 = 0.0f;
	int32_t best_rank = 0x7fffffff;
	CwStack stack;
	CwWalk w;
	cw_begin(w, o, d, stack);
	for (;;) {
		bool done = false;
		if (cw_step<ANY, COUNT>(s, w, best, best_rank, stack, cnt, done))
			return true;
		if (done)
			return best.prim >= 0;
	}
}

template <bool ANY, bool COUNT, int LAYOUT = KGR_LAYOUT_FAST>
__device__ __forceinline__ bool trace_fast(const DeviceScene &s, const f3 &o, const f3 &d,
		float tmax, kgr_hit &best, TraceCounters *cnt = nullptr)
{
	if (LAYOUT == KGR_LAYOUT_CW8)
		return trace_cw<ANY, COUNT>(s, o, d, tmax, best, cnt);
	int32_t entries[KGR_STACK_DEPTH];
	LocalStack stack(nullptr, entries);
	return trace_fast_stack<ANY, COUNT, LAYOUT>(s, o, d, tmax, best, stack, cnt);
}

template <bool ANY>
__device__ __forceinline__ bool trace(const DeviceScene &s, int layout, const f3 &o, const f3 &d,
		float tmax, kgr_hit &best)
{
	if (layout == KGR_LAYOUT_THREADED)
		return trace_threaded<ANY, false>(s, o, d, tmax, best);
	if (layout == KGR_LAYOUT_WIDE)
		return trace_fast<ANY, false, KGR_LAYOUT_WIDE>(s, o, d, tmax, best);
	if (layout == KGR_LAYOUT_CW8)
		return trace_cw<ANY, false>(s, o, d, tmax, best);
	return trace_fast<ANY, false>(s, o, d, tmax, best);
}

/* -------------------------------------------------------------- shading -- */

struct Material {
	f3 diffuse, specular, emission;
	float roughness, refraction;
	int type;
};

__device__ __forceinline__ Material load_material(const kgr_material *mats, uint32_t i)
{
	const float4 *p = reinterpret_cast<const float4 *>(mats + i);
	float4 a = __ldg(p + 0), b = __ldg(p + 1), c = __ldg(p + 2), e = __ldg(p + 3);
	Material m;
	m.diffuse = mk(a.x, a.y, a.z);
	m.specular = mk(a.w, b.x, b.y);
	m.emission = mk(b.z, b.w, c.x);
	/* c.y..c.w = ambient, e.x = shininess */
	m.roughness = e.y;
	m.refraction = e.z;
	m.type = __float_as_int(e.w);
	return m;
}

/* SurfaceHit (include/cuda/brdf.cuh:67-74) */
struct SurfaceHit {
	Material mat;
	bool entering;
	f3 n, wo, x;
};

#define KGR_PI_DEV 3.14159265358979323846f /* brdf.cuh:64 */

/* G1 (brdf.cuh:179-192) */
__device__ __forceinline__ float G1(const f3 &n, const f3 &v, const Material &mat)
{
	if (dot(v, n) <= 0.0f)
		return 0.0f;
	float alpha = mat.roughness;
	float theta = kacos(clampf(dot(n, v), 0.0f, 0.999f));
	float tan_theta = ktan(theta);
	float denom = 1 + ksqrt(1 + alpha * alpha * tan_theta * tan_theta);
	return 2.0f / denom;
}

/* Microfacets::GGX (brdf.cuh:210-220) */
__device__ __forceinline__ float ggx_D(const f3 &n, const f3 &h, const Material &mat)
{
	float alpha = mat.roughness;
	float theta = kacos(clampf(dot(n, h), 0.0f, 1.0f));
	float sn, c;
	ksincos(theta, sn, c);
	float tn = sn / c;
	return (alpha * alpha) / (KGR_PI_DEV * kpow4(c) * kpow2(alpha * alpha + tn * tn));
}

/* GGX::brdf (brdf.cuh:337-353) with shlick_F (:202-207) and G (:195-199) */
__device__ __forceinline__ f3 ggx_brdf(const Material &mat, f3 n, const f3 &wi, const f3 &wo)
{
	if (dot(wo, n) <= 0.0f)
		n = -n;
	f3 h = normalize(wi + wo);
	float k = kpow5(1 - dot(wi, h));
	f3 f = mat.specular + (1.0f - mat.specular) * k;
	float g = G1(n, wo, mat) * G1(n, wi, mat);
	float d = ggx_D(n, h, mat);
	f3 num = f * g * d;
	float denom = 4 * dot(wi, n) * dot(wo, n);
	return num / (denom + 1e-6f);
}

/* GGX::pdf (brdf.cuh:356-382) */
__device__ __forceinline__ float ggx_pdf(const Material &mat, f3 n, const f3 &wi, const f3 &wo)
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
	float term1 = dot(n, wi) / KGR_PI_DEV;
	float term2 = ggx_D(n, h, mat) * dot(n, h) / (4.0f * dot(wi, h));
	return (1 - t) * term1 + t * term2;
}

/* GGX::sample (brdf.cuh:385-433) */
__device__ __forceinline__ f3 ggx_sample(const Material &mat, f3 n, const f3 &wo, f3 &seed)
{
	if (dot(wo, n) <= 0.0f)
		n = -n;
	float avg_Kd = (mat.diffuse.x + mat.diffuse.y + mat.diffuse.z) / 3.0f;
	float avg_Ks = (mat.specular.x + mat.specular.y + mat.specular.z) / 3.0f;
	float t = 1.0f;
	if (avg_Kd + avg_Ks > 0.0f)
		t = avg_Ks / (avg_Kd + avg_Ks);
	f3 eta = rand_uniform_3f(seed);
	float theta;
	if (eta.x < t) {
		float k = ksqrt(eta.y / (1 - eta.y));
		theta = katan(k * mat.roughness);
	} else {
		theta = kacos(ksqrt(eta.y));
	}
	float phi = 2.0f * KGR_PI_DEV * eta.z;
	float st, ct, sp, cp;
	ksincos(theta, st, ct);
	ksincos(phi, sp, cp);
	f3 v = mk(st * cp, st * sp, ct);
	if (eta.x < t) {
		f3 h = rotate(v, n);
		return reflect(-wo, h);
	}
	return rotate(v, n);
}

/* ggx_brdf and ggx_pdf of one direction pair together: the flipped normal,
 * the half vector and D are the same in both, so they are computed once
 * (the results are those of the two separate calls). */
__device__ __forceinline__ void ggx_brdf_pdf(const Material &mat, f3 n, const f3 &wi, const f3 &wo, f3 &brdf_out,
		float &pdf_out)
{
	if (dot(wo, n) <= 0.0f)
		n = -n;
	f3 h = normalize(wi + wo);
	float d = ggx_D(n, h, mat);
	float k = kpow5(1 - dot(wi, h));
	f3 f = mat.specular + (1.0f - mat.specular) * k;
	float g = G1(n, wo, mat) * G1(n, wi, mat);
	f3 num = f * g * d;
	float denom = 4 * dot(wi, n) * dot(wo, n);
	brdf_out = num / (denom + 1e-6f);
	if (dot(wi, n) <= 0.0f) {
		pdf_out = 0.0f;
		return;
	}
	float avg_Kd = (mat.diffuse.x + mat.diffuse.y + mat.diffuse.z) / 3.0f;
	float avg_Ks = (mat.specular.x + mat.specular.y + mat.specular.z) / 3.0f;
	float t = 1.0f;
	if (avg_Kd + avg_Ks > 0.0f)
		t = kmax(avg_Ks / (avg_Kd + avg_Ks), 0.25f);
	float term1 = dot(n, wi) / KGR_PI_DEV;
	float term2 = d * dot(n, h) / (4.0f * dot(wi, h));
	pdf_out = (1 - t) * term1 + t * term2;
}

/* brdf() (brdf.cuh:437-449), out = eDiffuse */
__device__ __forceinline__ f3 brdf(const SurfaceHit &sh, const f3 &wi)
{
	return sh.mat.diffuse / KGR_PI_DEV + ggx_brdf(sh.mat, sh.n, wi, sh.wo);
}

/* A ReSTIR GI secondary vertex whose outgoing radiance may be reused toward
 * another receiver (the reconnection shift): no transmission and a GGX
 * lobe of roughness >= 0.3, so that the radiance it scatters changes slowly
 * with direction.  A glossier vertex sends its radiance mostly one way, and
 * reusing the value that was bright toward one receiver for another would
 * brighten the image. */
__device__ __forceinline__ bool gi_reconnectable(const Material &m)
{
	return m.type != KGR_SHADING_TRANSMISSION && m.roughness >= 0.3f;
}

/* eval() (brdf.cuh:573-589): GGX, or Glass::sample (:154-175) for
 * transmissive materials; pdf = 0 for a degenerate direction. */
__device__ __forceinline__ f3 eval(const SurfaceHit &sh, f3 &wi, float &pdf, f3 &seed)
{
	if (sh.mat.type & KGR_SHADING_TRANSMISSION) {
		float eta = sh.mat.refraction;
		float cos_theta = kmin(dot(-sh.wo, sh.n), 1.0f);
		float sin_theta = ksqrt(1.0f - cos_theta * cos_theta);
		bool reflect_ray = (eta * sin_theta > 1.0f);
		float ni_over_nt = 1.0f / eta;
		if (!sh.entering)
			ni_over_nt = eta;
		if (reflect_ray) {
			wi = reflect(sh.wo, sh.n);
		} else {
			float c2 = dot(-sh.wo, sh.n);
			f3 par = ni_over_nt * (sh.wo + c2 * sh.n);
			float pl = length(par);
			float pl2 = pl * pl;
			f3 perp = -ksqrt(fabsf(1.0f - pl2)) * sh.n;
			wi = par + perp;
		}
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

/* --------------------------------------------------------------- lights -- */

struct TriLight {
	f3 a, ab, ac, intensity;
	/* TriangleLight::area (lighting.cuh:103-105): `length * 0.5` is a double
	 * product; halving is exact, so the float product is the same value. */
	__device__ __forceinline__ float area() const { return length(cross(ab, ac)) * 0.5f; }
	__device__ __forceinline__ f3 normal() const { return normalize(cross(ab, ac)); }
};

__device__ __forceinline__ TriLight load_light(const kgr_triangle_light *lights, uint32_t i)
{
	const float4 *p = reinterpret_cast<const float4 *>(lights + i);
	float4 a = __ldg(p + 0), b = __ldg(p + 1), c = __ldg(p + 2);
	TriLight l;
	l.a = mk(a.x, a.y, a.z);
	l.ab = mk(a.w, b.x, b.y);
	l.ac = mk(b.z, b.w, c.x);
	l.intensity = mk(c.y, c.z, c.w);
	return l;
}

/* sample_area_light(TriangleLight) (lighting.cuh:133-146) */
__device__ __forceinline__ f3 sample_area_light(const TriLight &light, f3 &seed)
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

#define KGR_SHADOW_EPS 0.05f /* is_occluded, amadeus_common.cuh:193 */
#define KGR_OFFSET_EPS 1e-3f /* amadeus_common.cuh:22 */

/* direct_unoccluded (amadeus_common.cuh:380-397) for a triangle light */
__device__ __forceinline__ f3 direct_unoccluded(const SurfaceHit &sh, const f3 &Le, const f3 &normal,
		const f3 &D, float d)
{
	f3 rho = brdf(sh, D);
	float geometric = fabsf(dot(sh.n, D));
	float ldot = fabsf(dot(normal, D));
	geometric *= ldot / (d * d);
	return rho * Le * geometric;
}

/* ------------------------------------------ quad lights, environment map -- */

/* QuadLight (lighting.cuh:57-94): the parallelogram a + u ab + v ac. */
struct QuadLight {
	f3 a, ab, ac, intensity;
	__device__ __forceinline__ float area() const { return length(cross(ab, ac)); }
	__device__ __forceinline__ f3 normal() const { return normalize(cross(ab, ac)); }
};

__device__ __forceinline__ QuadLight load_quad(const kgr_quad_light *quads, uint32_t i)
{
	const float4 *p = reinterpret_cast<const float4 *>(quads + i);
	float4 a = __ldg(p + 0), b = __ldg(p + 1), c = __ldg(p + 2);
	QuadLight l;
	l.a = mk(a.x, a.y, a.z);
	l.ab = mk(a.w, b.x, b.y);
	l.ac = mk(b.z, b.w, c.x);
	l.intensity = mk(c.y, c.z, c.w);
	return l;
}

/* sample_area_light(QuadLight) (lighting.cuh:123-131): no reflection */
__device__ __forceinline__ f3 sample_area_light(const QuadLight &light, f3 &seed)
{
	f3 r = pcg3f(seed);
	float u = fract(r.x);
	float v = fract(r.y);
	return light.a + u * light.ab + v * light.ac;
}

#define KGR_WORLD_RADIUS 10000.0f /* Ld_Environment, amadeus_common.cuh:218 */
#define KGR_PI_D 3.14159265358979323846 /* M_PI, a double */

/* Texture coordinates of a direction (amadeus_path_tracer.cu:209-210):
 * u = atan2(d.x, d.z) / (2 pi) + 0.5, v = asin(d.y) / pi + 0.5; M_PI is a
 * double, so the division and the offset are double and round once. */
__device__ __forceinline__ void env_uv(const f3 &d, float &u, float &v)
{
	u = (float)((double)katan2(d.x, d.z) / (2.0 * KGR_PI_D) + 0.5);
	v = (float)((double)kasin(d.y) / KGR_PI_D + 0.5);
}

__device__ __forceinline__ f3 env_fetch(const DeviceScene &s, float u, float v)
{
	float4 c = tex2D<float4>((cudaTextureObject_t)s.env, u, v);
	return mk(c.x, c.y, c.z);
}

/* The miss program's radiance along d: the map at (u, 1 - v) for the path
 * tracer, (u, v) for ReSTIR; black without a map. */
__device__ __forceinline__ f3 env_miss(const DeviceScene &s, const f3 &d)
{
	if (!s.has_env)
		return mk(0.0f);
	float u, v;
	env_uv(d, u, v);
	return env_fetch(s, u, s.env_flip_v ? 1.0f - v : v);
}

/* The environment light's direction (Ld_Environment,
 * amadeus_common.cuh:215-238; sample_direct, :343-374): seed =
 * rand_uniform_3f(seed), theta = acos(sqrt(1 - seed.x)), phi = 2 pi
 * seed.y -- in float with brdf.cuh's float PI in Ld_Environment, in double
 * with M_PI in sample_direct. */
__device__ __forceinline__ f3 env_direction(f3 &seed, bool phi_double)
{
	seed = rand_uniform_3f(seed);
	float theta = kacos(ksqrt(1.0f - fract(seed.x)));
	float phi = phi_double ? (float)(2.0 * KGR_PI_D * (double)fract(seed.y)) : 2.0f * KGR_PI_F * fract(seed.y);
	float st = ksin(theta);
	return mk(st * kcos(phi), st * ksin(phi), kcos(theta));
}

/* One light of the launch by its place in [quads | triangles | env]: what
 * sample_direct (amadeus_common.cuh:301-377) records in FullLightSample.
 * type 0 quad, 1 triangle, 2 environment. */
struct LightPoint {
	f3 Le, normal, point;
	float pdf;
	int type;
	float env_u, env_v;
};

/* sample_direct: a uniform pick over quads + triangles + the environment,
 * then a point on it.  index < 0 when there is nothing to pick. */
__device__ __forceinline__ int sample_direct(const DeviceScene &s, const f3 &x, f3 &seed, LightPoint &lp)
{
	unsigned int total = s.quad_count + s.light_count + (s.has_env ? 1u : 0u);
	unsigned int li = (unsigned int)(rand_uniform(seed) * total);
	lp.env_u = lp.env_v = 0.0f;
	if (li < s.quad_count) {
		QuadLight l = load_quad(s.quads, li);
		lp.point = sample_area_light(l, seed);
		lp.Le = l.intensity;
		lp.normal = l.normal();
		lp.pdf = 1.0f / (l.area() * total);
		lp.type = 0;
		return (int)li;
	}
	if (li < s.quad_count + s.light_count) {
		TriLight l = load_light(s.lights, li - s.quad_count);
		lp.point = sample_area_light(l, seed);
		lp.Le = l.intensity;
		lp.normal = l.normal();
		lp.pdf = 1.0f / (l.area() * total);
		lp.type = 1;
		return (int)li;
	}
	if (li < total) {
		f3 wi = env_direction(seed, true);
		lp.point = x + wi * KGR_WORLD_RADIUS;
		env_uv(wi, lp.env_u, lp.env_v);
		lp.Le = env_fetch(s, lp.env_u, lp.env_v);
		lp.normal = -wi;
		lp.pdf = (float)(1.0 / (4.0 * KGR_PI_D * (double)total));
		lp.type = 2;
		return (int)li;
	}
	lp.point = mk(0.0f);
	lp.pdf = 0.0f;
	lp.type = -1;
	return -1;
}

/* direct_unoccluded (amadeus_common.cuh:380-397) for any light type: the
 * environment (type 2) drops the light's cosine and 1/d^2 */
__device__ __forceinline__ f3 direct_unoccluded_typed(const SurfaceHit &sh, const f3 &Le, const f3 &normal,
		int type, const f3 &D, float d)
{
	f3 rho = brdf(sh, D);
	float geometric = fabsf(dot(sh.n, D));
	if (type != 2) {
		float ldot = fabsf(dot(normal, D));
		geometric *= ldot / (d * d);
	}
	return rho * Le * geometric;
}

/* ------------------------------------------------------------ hit data -- */

/* LOAD_INTERSECTION_DATA (amadeus_common.cuh:490-515): geometric normal
 * flipped against the ray (entering), interpolated shading normal made
 * consistent with it, interpolated position; world-space vertices. */
__device__ __forceinline__ bool surface(const DeviceScene &s, const kgr_hit &h, const f3 &dir,
		SurfaceHit &sh)
{
	uint4 t = __ldg(&s.tris[h.prim]);
	f3 a = f3_of(__ldg(&s.positions[t.x])), b = f3_of(__ldg(&s.positions[t.y])),
	   c = f3_of(__ldg(&s.positions[t.z]));
	f3 ng = normalize(cross(b - a, c - a));
	bool entering;
	if (dot(ng, dir) > 0.0f) {
		ng = -ng;
		entering = false;
	} else {
		entering = true;
	}
	ng = normalize(ng);
	f3 na = f3_of(__ldg(&s.normals[t.x])), nb = f3_of(__ldg(&s.normals[t.y])),
	   nc = f3_of(__ldg(&s.normals[t.z]));
	float w0 = 1.0f - h.b1 - h.b2;
	f3 normal = w0 * na + h.b1 * nb + h.b2 * nc;
	if (dot(normal, ng) < 0.0f)
		normal = -normal;
	normal = normalize(normal);
	sh.x = w0 * a + h.b1 * b + h.b2 * c;
	sh.mat = load_material(s.materials, t.w);
	sh.entering = entering;
	sh.n = normal;
	sh.wo = -dir;
	return !anynan(normal);
}

/* Queue position j of a sample's npix camera paths -> its pixel: bands of
 * four rows, each band cut into tiles eight pixels wide (the last band and
 * the last tile of a band may be smaller), a tile's pixels row by row.  A
 * warp's 32 consecutive positions are then an 8x4 tile of the image rather
 * than a 32-pixel strip of one row, so its camera rays, and the bounces the
 * shade kernel queues from them in the same order, stay closer together.
 * A bijection on [0, npix): every path is queued once. */
__device__ __forceinline__ uint32_t tiled_pixel(uint32_t j, uint32_t width, uint32_t height)
{
	uint32_t band = j / (4u * width);
	uint32_t jb = j - band * 4u * width;
	uint32_t rows = height - 4u * band < 4u ? height - 4u * band : 4u;
	uint32_t full = width / 8u;
	uint32_t x, y;
	if (jb < 8u * rows * full) {
		uint32_t c = jb / (8u * rows), local = jb - c * 8u * rows;
		x = 8u * c + local % 8u;
		y = 4u * band + local / 8u;
	} else {
		uint32_t w = width - 8u * full, local = jb - 8u * rows * full;
		x = 8u * full + local % w;
		y = 4u * band + local / w;
	}
	return y * width + x;
}

/* ------------------------------------------------------------- queues -- */

/* Warp-aggregated append: one atomic per warp, lanes write in lane order. */
__device__ __forceinline__ void queue_append(uint32_t *queue, uint32_t *counter, uint32_t value, bool pred,
		uint32_t *total = nullptr)
{
	unsigned mask = __activemask();
	unsigned ballot = __ballot_sync(mask, pred);
	if (!ballot)
		return;
	int lane = threadIdx.x & 31;
	int leader = __ffs(ballot) - 1;
	uint32_t base = 0;
	if (lane == leader) {
		base = atomicAdd(counter, (uint32_t)__popc(ballot));
		if (total)
			atomicAdd(total, (uint32_t)__popc(ballot));
	}
	base = __shfl_sync(mask, base, leader);
	if (pred)
		queue[base + __popc(ballot & ((1u << lane) - 1u))] = value;
}

/* Visit entries 0..n-1 of a queue in batches of 32 a warp: lane 0 takes the
 * next batch from *fetch when the warp is done with its last, so warps that
 * drew short rays take more batches and none is left with a fixed share of
 * long ones at the end.  Every lane of the warp must call it (no lane may
 * have returned). */
template <class F>
__device__ __forceinline__ void for_each_queued(uint32_t n, uint32_t *fetch, F f)
{
	const int lane = threadIdx.x & 31;
	for (;;) {
		uint32_t base = 0;
		if (lane == 0)
			base = atomicAdd(fetch, 32u);
		base = __shfl_sync(0xffffffffu, base, 0);
		if (base >= n)
			return;
		if (base + (uint32_t)lane < n)
			f(base + (uint32_t)lane);
	}
}

/* Visit entries 0..n-1 of a ray queue, grid-stride, and run the heavy work
 * of the entries whose ray hit in full warps.  A missed ray ends its path
 * and needs at most an environment lookup, and on a scene open to the sky a
 * third of the camera rays and about half of each bounce's rays miss, so
 * one path a thread leaves that share of a warp's lanes idle through the
 * shading.  Here each block reads BLOCK entries at a time: look(i, hv)
 * returns entry i's path (hv: its hit record), does what a miss needs in
 * place and sets `heavy` for an entry that needs work(p, hv).  Those are
 * gathered in shared memory (one shared atomic a warp) and, whenever BLOCK
 * of them have gathered, run one per thread; the last fewer than BLOCK run
 * at the end.  Every thread of a block of BLOCK threads calls it with the
 * same n.  Entries reach `work` in another order than the queue's, which
 * changes only the order of the queues that work appends to. */
template <int BLOCK, class Look, class Work>
__device__ __forceinline__ void for_each_hit(uint32_t n, Look look, Work work)
{
	__shared__ uint32_t held_p[2 * BLOCK];
	__shared__ float4 held_hit[2 * BLOCK];
	__shared__ uint32_t held;
	const uint32_t stride = gridDim.x * BLOCK;
	const int lane = threadIdx.x & 31;
	if (threadIdx.x == 0)
		held = 0;
	__syncthreads();
	/* `base` is the same for every thread of the block, so all of them take
	 * the same number of iterations and reach every barrier */
	for (uint32_t base = blockIdx.x * BLOCK; base < n; base += stride) {
		uint32_t i = base + threadIdx.x;
		bool heavy = false;
		uint32_t p = 0;
		float4 hv = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
		if (i < n)
			p = look(i, hv, heavy);
		/* `held` is below BLOCK between iterations, so the slots fit */
		unsigned ballot = __ballot_sync(0xffffffffu, heavy);
		uint32_t slot = 0;
		if (lane == 0 && ballot)
			slot = atomicAdd(&held, (uint32_t)__popc(ballot));
		slot = __shfl_sync(0xffffffffu, slot, 0) + __popc(ballot & ((1u << lane) - 1u));
		if (heavy) {
			held_p[slot] = p;
			held_hit[slot] = hv;
		}
		__syncthreads();
		const uint32_t c = held;
		__syncthreads();
		if (c >= BLOCK) {
			const uint32_t k = c - BLOCK + threadIdx.x;
			work(held_p[k], held_hit[k]);
			if (threadIdx.x == 0)
				held = c - BLOCK;
			__syncthreads();
		}
	}
	const uint32_t c = held;
	if (threadIdx.x < c)
		work(held_p[threadIdx.x], held_hit[threadIdx.x]);
}

} /* namespace kgr */

#endif

/*
 * bvh_build.cpp -- host BVH builders and the two device layouts.
 *
 *  build_kobra       the reference builder, partition() of source/bvh.cpp:
 *                    102-210 (axis and range of the single primitive with the
 *                    largest extent, 10 SAH bins over that range, alternate
 *                    split when every bin leaves a side empty, one primitive
 *                    per leaf).  Same float operations, so the serialised
 *                    buffer is identical to the reference's.
 *  build_sah         binned SAH over centroid bounds (32 bins, 3 axes),
 *                    leaves of at most max_leaf primitives.
 *  serialize_threaded the threaded layout of serialize(), source/bvh.cpp:
 *                    213-260; a leaf of k primitives becomes k consecutive
 *                    one-primitive leaf records chained by their miss links.
 *  parse_threaded    the inverse, for buffers serialised by the caller.
 *  build_fast        64-byte child-pair nodes + leaf-ordered triangles.
 */
#include <float.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <functional>

#include "kgr_cw8.h"
#include "kgr_internal.h"

namespace kgr {

namespace {

inline float fbits(int32_t i)
{
	float f;
	memcpy(&f, &i, 4);
	return f;
}

inline int32_t ibits(float f)
{
	int32_t i;
	memcpy(&i, &f, 4);
	return i;
}

/* glm::min / glm::max semantics: (y < x) ? y : x */
inline float gmin(float a, float b) { return b < a ? b : a; }
inline float gmax(float a, float b) { return a < b ? b : a; }

inline void box_union(float *mn, float *mx, const PrimBox &b)
{
	for (int k = 0; k < 3; k++) {
		mn[k] = gmin(mn[k], b.bmin[k]);
		mx[k] = gmax(mx[k], b.bmax[k]);
	}
}

/* BoundingBox::surface_area (include/bbox.hpp:14-25) */
inline float surface_area(const float *mn, const float *mx)
{
	float dx = mx[0] - mn[0], dy = mx[1] - mn[1], dz = mx[2] - mn[2];
	float xy = dx * dy, yz = dy * dz, xz = dx * dz;
	return 2.0f * (xy + yz + xz);
}

} /* namespace */

/* ======================================================= kobra builder == */

namespace {

struct KobraBuilder {
	const std::vector<PrimBox> &boxes;
	Tree &tree;
	explicit KobraBuilder(const std::vector<PrimBox> &b, Tree &t) : boxes(b), tree(t) {}

	/* An element of a partition list: a primitive (leaf) or a built node. */
	struct Item {
		int32_t node; /* tree node index */
		float bmin[3], bmax[3];
	};

	int32_t make_leaf(uint32_t prim)
	{
		TreeNode n;
		memcpy(n.bmin, boxes[prim].bmin, 12);
		memcpy(n.bmax, boxes[prim].bmax, 12);
		n.first = (int32_t)tree.prim_order.size();
		n.count = 1;
		tree.prim_order.push_back(prim);
		tree.nodes.push_back(n);
		return (int32_t)tree.nodes.size() - 1;
	}

	void union_of(const std::vector<Item> &items, float *mn, float *mx)
	{
		memcpy(mn, items[0].bmin, 12);
		memcpy(mx, items[0].bmax, 12);
		for (size_t i = 1; i < items.size(); i++)
			for (int k = 0; k < 3; k++) {
				mn[k] = gmin(mn[k], items[i].bmin[k]);
				mx[k] = gmax(mx[k], items[i].bmax[k]);
			}
	}

	/* sah_cost, source/bvh.cpp:46-98 */
	float sah_cost(const std::vector<Item> &items, int axis, float split)
	{
		float lmn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, lmx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
		float rmn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, rmx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
		float tmn[3], tmx[3];
		memcpy(tmn, items[0].bmin, 12);
		memcpy(tmx, items[0].bmax, 12);
		int nl = 0, nr = 0;
		for (const Item &it : items) {
			for (int k = 0; k < 3; k++) {
				tmn[k] = gmin(tmn[k], it.bmin[k]);
				tmx[k] = gmax(tmx[k], it.bmax[k]);
			}
			float value = (it.bmin[axis] + it.bmax[axis]) / 2.0f;
			float *mn = value < split ? lmn : rmn, *mx = value < split ? lmx : rmx;
			(value < split ? nl : nr)++;
			for (int k = 0; k < 3; k++) {
				mn[k] = gmin(mn[k], it.bmin[k]);
				mx[k] = gmax(mx[k], it.bmax[k]);
			}
		}
		if (nl == 0 || nr == 0)
			return FLT_MAX;
		float sl = surface_area(lmn, lmx), sr = surface_area(rmn, rmx), st = surface_area(tmn, tmx);
		return 1 + (nl * sl + nr * sr) / st;
	}

	/* partition, source/bvh.cpp:102-195 */
	int32_t partition(const std::vector<Item> &items)
	{
		if (items.empty())
			return -1;
		if (items.size() == 1)
			return items[0].node;
		TreeNode node;
		if (items.size() == 2) {
			union_of(items, node.bmin, node.bmax);
			node.left = items[0].node;
			node.right = items[1].node;
			tree.nodes.push_back(node);
			return (int32_t)tree.nodes.size() - 1;
		}
		int axis = 0;
		float max_extent = 0.0f, min_value = FLT_MAX, max_value = -FLT_MAX;
		for (const Item &it : items)
			for (int k = 0; k < 3; k++) {
				float extent = fabsf(it.bmax[k] - it.bmin[k]);
				if (extent > max_extent) {
					max_extent = extent;
					min_value = it.bmin[k];
					max_value = it.bmax[k];
					axis = k;
				}
			}
		float min_cost = FLT_MAX, min_split = 0.0f;
		const int bins = 10;
		for (int i = 0; i < bins; i++) {
			float split = (max_value - min_value) / bins * i + min_value;
			float cost = sah_cost(items, axis, split);
			if (cost < min_cost) {
				min_cost = cost;
				min_split = split;
			}
		}
		std::vector<Item> left, right;
		if (min_cost == FLT_MAX) {
			for (size_t i = 0; i < items.size(); i++)
				(i % 2 == 0 ? left : right).push_back(items[i]);
		} else {
			for (const Item &it : items) {
				float value = (it.bmin[axis] + it.bmax[axis]) / 2.0f;
				(value < min_split ? left : right).push_back(it);
			}
		}
		union_of(items, node.bmin, node.bmax);
		int32_t l = partition(left);
		int32_t r = partition(right);
		node.left = l;
		node.right = r;
		tree.nodes.push_back(node);
		return (int32_t)tree.nodes.size() - 1;
	}
};

} /* namespace */

void build_kobra(const std::vector<PrimBox> &boxes, Tree &tree)
{
	tree.nodes.clear();
	tree.prim_order.clear();
	if (boxes.empty())
		return;
	KobraBuilder b(boxes, tree);
	std::vector<KobraBuilder::Item> items(boxes.size());
	for (size_t i = 0; i < boxes.size(); i++) {
		items[i].node = b.make_leaf((uint32_t)i);
		memcpy(items[i].bmin, boxes[i].bmin, 12);
		memcpy(items[i].bmax, boxes[i].bmax, 12);
	}
	int32_t root = b.partition(items);
	/* move the root to index 0 */
	if (root != 0) {
		std::swap(tree.nodes[0], tree.nodes[root]);
		for (TreeNode &n : tree.nodes) {
			if (n.count)
				continue;
			for (int32_t *c : {&n.left, &n.right}) {
				if (*c == root)
					*c = 0;
				else if (*c == 0)
					*c = root;
			}
		}
	}
}

/* ========================================================= SAH builder == */

void build_sah(const std::vector<PrimBox> &boxes_in, int max_leaf, Tree &tree)
{
	const int BINS = 32;
	tree.nodes.clear();
	size_t n = boxes_in.size();
	/* canonical zeros (-0 -> +0): every min and max below is then a
	 * function of the set of values, not of their order */
	std::vector<PrimBox> boxes(boxes_in);
	for (PrimBox &b : boxes)
		for (int k = 0; k < 3; k++) {
			b.bmin[k] += 0.0f;
			b.bmax[k] += 0.0f;
		}
	tree.prim_order.resize(n);
	if (n == 0)
		return;
	std::vector<float> cen(3 * n);
	for (size_t i = 0; i < n; i++) {
		tree.prim_order[i] = (uint32_t)i;
		for (int k = 0; k < 3; k++)
			cen[3 * i + k] = (boxes[i].bmin[k] + boxes[i].bmax[k]) * 0.5f;
	}
	tree.nodes.reserve(2 * n / std::max(1, max_leaf / 2) + 8);

	struct Task {
		int32_t node;
		uint32_t begin, end;
	};
	std::vector<Task> stack;
	tree.nodes.push_back(TreeNode());
	stack.push_back({0, 0, (uint32_t)n});
	uint32_t *order = tree.prim_order.data();

	struct Bin {
		float mn[3], mx[3];
		uint32_t count;
	};

	while (!stack.empty()) {
		Task t = stack.back();
		stack.pop_back();
		TreeNode &node = tree.nodes[t.node];
		float bmn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, bmx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
		float cmn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, cmx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
		for (uint32_t i = t.begin; i < t.end; i++) {
			uint32_t p = order[i];
			box_union(bmn, bmx, boxes[p]);
			for (int k = 0; k < 3; k++) {
				cmn[k] = std::min(cmn[k], cen[3 * p + k]);
				cmx[k] = std::max(cmx[k], cen[3 * p + k]);
			}
		}
		memcpy(node.bmin, bmn, 12);
		memcpy(node.bmax, bmx, 12);
		uint32_t cnt = t.end - t.begin;
		if (cnt <= 1) {
			node.first = (int32_t)t.begin;
			node.count = (int32_t)cnt;
			continue;
		}

		float best_cost = FLT_MAX;
		int best_axis = -1, best_split = 0;
		float sa_parent = surface_area(bmn, bmx);
		for (int axis = 0; axis < 3; axis++) {
			float ext = cmx[axis] - cmn[axis];
			if (!(ext > 0.0f))
				continue;
			Bin bins[BINS];
			for (int b = 0; b < BINS; b++) {
				bins[b].count = 0;
				for (int k = 0; k < 3; k++) {
					bins[b].mn[k] = FLT_MAX;
					bins[b].mx[k] = -FLT_MAX;
				}
			}
			float scale = BINS / ext;
			for (uint32_t i = t.begin; i < t.end; i++) {
				uint32_t p = order[i];
				int b = (int)((cen[3 * p + axis] - cmn[axis]) * scale);
				b = b < 0 ? 0 : (b >= BINS ? BINS - 1 : b);
				bins[b].count++;
				box_union(bins[b].mn, bins[b].mx, boxes[p]);
			}
			float rarea[BINS];
			uint32_t rcount[BINS];
			float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
			uint32_t c = 0;
			for (int b = BINS - 1; b > 0; b--) {
				c += bins[b].count;
				for (int k = 0; k < 3; k++) {
					mn[k] = std::min(mn[k], bins[b].mn[k]);
					mx[k] = std::max(mx[k], bins[b].mx[k]);
				}
				rcount[b] = c;
				rarea[b] = c ? surface_area(mn, mx) : 0.0f;
			}
			for (int k = 0; k < 3; k++) {
				mn[k] = FLT_MAX;
				mx[k] = -FLT_MAX;
			}
			c = 0;
			for (int b = 1; b < BINS; b++) {
				c += bins[b - 1].count;
				for (int k = 0; k < 3; k++) {
					mn[k] = std::min(mn[k], bins[b - 1].mn[k]);
					mx[k] = std::max(mx[k], bins[b - 1].mx[k]);
				}
				if (c == 0 || rcount[b] == 0)
					continue;
				float cost = 1.0f + ((float)c * surface_area(mn, mx) + (float)rcount[b] * rarea[b]) / sa_parent;
				if (cost < best_cost) {
					best_cost = cost;
					best_axis = axis;
					best_split = b;
				}
			}
		}

		bool make_leaf = (int)cnt <= max_leaf && (best_axis < 0 || (float)cnt <= best_cost);
		if (make_leaf) {
			node.first = (int32_t)t.begin;
			node.count = (int32_t)cnt;
			continue;
		}
		uint32_t mid;
		if (best_axis < 0) {
			mid = t.begin + cnt / 2; /* identical centroids: split by index */
		} else {
			float scale = BINS / (cmx[best_axis] - cmn[best_axis]);
			float c0 = cmn[best_axis];
			const float *cp = cen.data();
			/* stable: each side keeps the parent's order, so the tree is a
			 * function of the primitive sets alone (the GPU builder in
			 * bvh_gpu.cu reproduces it) */
			uint32_t *m = std::stable_partition(order + t.begin, order + t.end, [&](uint32_t p) {
				int b = (int)((cp[3 * p + best_axis] - c0) * scale);
				b = b < 0 ? 0 : (b >= BINS ? BINS - 1 : b);
				return b < best_split;
			});
			mid = (uint32_t)(m - order);
			if (mid == t.begin || mid == t.end)
				mid = t.begin + cnt / 2;
		}
		int32_t l = (int32_t)tree.nodes.size();
		tree.nodes.push_back(TreeNode());
		tree.nodes.push_back(TreeNode());
		tree.nodes[t.node].left = l;
		tree.nodes[t.node].right = l + 1;
		/* push right first so the left subtree is built first (locality) */
		stack.push_back({l + 1, mid, t.end});
		stack.push_back({l, t.begin, mid});
	}
}

/* ============================================================ threaded == */

namespace {

uint32_t subtree_records(const Tree &tree, int32_t i, std::vector<uint32_t> &memo)
{
	if (memo[i])
		return memo[i];
	const TreeNode &n = tree.nodes[i];
	uint32_t r = n.count ? (uint32_t)n.count
		: 1 + subtree_records(tree, n.left, memo) + subtree_records(tree, n.right, memo);
	memo[i] = r;
	return r;
}

void emit(std::vector<float> &out, float leaf, int32_t object, int32_t hit, int32_t miss,
		const float *mn, const float *mx)
{
	float v[12] = {leaf, fbits(object), fbits(hit), fbits(miss), mn[0], mn[1], mn[2], 0.0f,
		mx[0], mx[1], mx[2], 0.0f};
	out.insert(out.end(), v, v + 12);
}

void serialize_node(const Tree &tree, const std::vector<PrimBox> &boxes, int32_t i, int32_t miss,
		std::vector<uint32_t> &memo, std::vector<float> &out, std::vector<int32_t> *rec_node)
{
	const TreeNode &n = tree.nodes[i];
	int32_t size = (int32_t)(out.size() / 4);
	if (n.count) {
		for (int32_t k = 0; k < n.count; k++) {
			uint32_t prim = tree.prim_order[n.first + k];
			int32_t next = k + 1 < n.count ? size + 3 * (k + 1) : miss;
			emit(out, 1.0f, (int32_t)prim, next, next, boxes[prim].bmin, boxes[prim].bmax);
			if (rec_node)
				rec_node->push_back(~(int32_t)prim);
		}
		return;
	}
	int32_t after = size + 3;
	int32_t right_index = after + 3 * (int32_t)subtree_records(tree, n.left, memo);
	emit(out, 0.0f, -1, after, miss, n.bmin, n.bmax);
	if (rec_node)
		rec_node->push_back(i);
	serialize_node(tree, boxes, n.left, right_index, memo, out, rec_node);
	serialize_node(tree, boxes, n.right, miss, memo, out, rec_node);
}

} /* namespace */

void serialize_threaded(const Tree &tree, const std::vector<PrimBox> &boxes, std::vector<float> &out,
		std::vector<int32_t> *rec_node)
{
	out.clear();
	if (rec_node)
		rec_node->clear();
	if (tree.nodes.empty())
		return;
	std::vector<uint32_t> memo(tree.nodes.size(), 0);
	out.reserve((size_t)subtree_records(tree, 0, memo) * 12);
	serialize_node(tree, boxes, 0, -1, memo, out, rec_node);
}

/* Parse a threaded buffer: the children of an internal record are the
 * records met from its hit link following miss links until its own miss
 * link.  Runs of leaf records become leaves (at most 8 primitives); lists of
 * more than two children become a right-leaning chain of extra nodes, which
 * keeps the walk order of the primitives. */
void parse_threaded(const float *vec4, uint32_t count, uint32_t prim_count,
		const std::vector<PrimBox> &boxes, Tree &tree, std::vector<int32_t> *rec_node)
{
	tree.nodes.clear();
	tree.prim_order.clear();
	KGR_REQUIRE(count % 3 == 0, KGR_ERR_BVH_FORMAT, "bvh buffer length is not a multiple of 3 vec4");
	if (rec_node)
		rec_node->assign(count / 3, KGR_REC_UNREACHED);
	if (count == 0)
		return;
	uint32_t records = count / 3;
	std::vector<uint8_t> seen(prim_count, 0);
	uint64_t steps = 0;
	auto rec = [&](int32_t idx) -> const float * {
		KGR_REQUIRE(idx >= 0 && (uint32_t)idx < count && idx % 3 == 0, KGR_ERR_BVH_FORMAT,
			"bvh link out of range: " + std::to_string(idx));
		KGR_REQUIRE(++steps <= 4ull * records + 16, KGR_ERR_BVH_FORMAT, "bvh links form a cycle");
		return vec4 + 4 * (size_t)idx;
	};
	auto add_leaf_prims = [&](const std::vector<uint32_t> &prims) -> int32_t {
		TreeNode n;
		for (int k = 0; k < 3; k++) {
			n.bmin[k] = FLT_MAX;
			n.bmax[k] = -FLT_MAX;
		}
		n.first = (int32_t)tree.prim_order.size();
		n.count = (int32_t)prims.size();
		for (uint32_t p : prims) {
			tree.prim_order.push_back(p);
			box_union(n.bmin, n.bmax, boxes[p]);
		}
		tree.nodes.push_back(n);
		return (int32_t)tree.nodes.size() - 1;
	};
	auto take_prim = [&](const float *h) -> uint32_t {
		int32_t obj = ibits(h[1]);
		KGR_REQUIRE(obj >= 0 && (uint32_t)obj < prim_count, KGR_ERR_BVH_FORMAT,
			"leaf object out of range: " + std::to_string(obj));
		KGR_REQUIRE(!seen[obj], KGR_ERR_BVH_FORMAT, "primitive referenced twice: " + std::to_string(obj));
		seen[obj] = 1;
		return (uint32_t)obj;
	};
	auto combine = [&](int32_t a, int32_t b) -> int32_t {
		TreeNode n;
		for (int k = 0; k < 3; k++) {
			n.bmin[k] = gmin(tree.nodes[a].bmin[k], tree.nodes[b].bmin[k]);
			n.bmax[k] = gmax(tree.nodes[a].bmax[k], tree.nodes[b].bmax[k]);
		}
		n.left = a;
		n.right = b;
		tree.nodes.push_back(n);
		return (int32_t)tree.nodes.size() - 1;
	};

	auto note = [&](int32_t idx, int32_t v) {
		if (rec_node)
			(*rec_node)[idx / 3] = v;
	};
	std::function<int32_t(int32_t)> parse = [&](int32_t idx) -> int32_t {
		const float *h = rec(idx);
		if (ibits(h[1]) != -1) {
			uint32_t p = take_prim(h);
			note(idx, ~(int32_t)p);
			return add_leaf_prims({p});
		}
		int32_t miss = ibits(h[3]);
		std::vector<int32_t> kids;
		std::vector<uint32_t> run;
		auto flush = [&]() {
			if (!run.empty()) {
				kids.push_back(add_leaf_prims(run));
				run.clear();
			}
		};
		int32_t c = ibits(h[2]);
		while (c != miss) {
			const float *ch = rec(c);
			if (ibits(ch[1]) != -1) {
				run.push_back(take_prim(ch));
				note(c, ~(int32_t)run.back());
				if (run.size() == 8)
					flush();
			} else {
				flush();
				kids.push_back(parse(c));
			}
			c = ibits(ch[3]);
		}
		flush();
		KGR_REQUIRE(!kids.empty(), KGR_ERR_BVH_FORMAT, "internal bvh record without children");
		int32_t acc = kids.back();
		for (int k = (int)kids.size() - 2; k >= 0; k--)
			acc = combine(kids[k], acc);
		/* the internal record's own box is the one the threaded walk tests */
		if (kids.size() >= 1) {
			memcpy(tree.nodes[acc].bmin, h + 4, 12);
			memcpy(tree.nodes[acc].bmax, h + 8, 12);
		}
		note(idx, acc);
		return acc;
	};
	int32_t root = parse(0);
	for (uint32_t p = 0; p < prim_count; p++)
		KGR_REQUIRE(seen[p], KGR_ERR_BVH_FORMAT, "primitive missing from bvh: " + std::to_string(p));
	if (root != 0) {
		/* move root to index 0 */
		std::swap(tree.nodes[0], tree.nodes[root]);
		for (TreeNode &n : tree.nodes) {
			if (n.count)
				continue;
			for (int32_t *c : {&n.left, &n.right}) {
				if (*c == root)
					*c = 0;
				else if (*c == 0)
					*c = root;
			}
		}
		if (rec_node)
			for (int32_t &r : *rec_node) {
				if (r == root)
					r = 0;
				else if (r == 0)
					r = root;
			}
	}
}

/* ================================================================ fast == */

namespace {

/* Outward padding so that slab tests computed with FMA never cull a box
 * whose triangles the exact Moller-Trumbore test would accept. */
inline void pad_box(const float *mn, const float *mx, float *pmn, float *pmx)
{
	const float rel = 1.0f / (1 << 19);
	for (int k = 0; k < 3; k++) {
		float ext = mx[k] - mn[k];
		pmn[k] = mn[k] - ((fabsf(mn[k]) + ext) * rel + 1e-20f);
		pmx[k] = mx[k] + ((fabsf(mx[k]) + ext) * rel + 1e-20f);
	}
}

} /* namespace */

void build_fast(const Tree &tree, const std::vector<PrimBox> &boxes, const float *positions,
		const uint32_t *tris4, std::vector<FastNode> &nodes, std::vector<float4> &tri_records,
		std::vector<int2> *kids)
{
	(void)boxes;
	nodes.clear();
	tri_records.clear();
	if (kids)
		kids->clear();
	if (tree.nodes.empty())
		return;
	tri_records.reserve(3 * tree.prim_order.size());
	auto leaf_ref = [&](const TreeNode &n) -> int32_t {
		uint32_t start = (uint32_t)(tri_records.size() / 3);
		KGR_REQUIRE(n.count >= 1 && n.count <= 8, KGR_ERR_INTERNAL, "leaf size out of range");
		KGR_REQUIRE(start < (1u << 27), KGR_ERR_UNSUPPORTED, "too many triangles for the fast layout");
		for (int32_t k = 0; k < n.count; k++) {
			uint32_t prim = tree.prim_order[n.first + k];
			const uint32_t *t = tris4 + 4 * (size_t)prim;
			const float *a = positions + 3 * (size_t)t[0];
			const float *b = positions + 3 * (size_t)t[1];
			const float *c = positions + 3 * (size_t)t[2];
			tri_records.push_back(make_float4(a[0], a[1], a[2], fbits((int32_t)prim)));
			tri_records.push_back(make_float4(b[0] - a[0], b[1] - a[1], b[2] - a[2], 0.0f));
			tri_records.push_back(make_float4(c[0] - a[0], c[1] - a[1], c[2] - a[2], 0.0f));
		}
		return ~(int32_t)((start << 3) | (uint32_t)(n.count - 1));
	};
	auto set_child = [&](FastNode &fn, int side, const float *mn, const float *mx, int32_t ref) {
		float pmn[3], pmx[3];
		pad_box(mn, mx, pmn, pmx);
		if (side == 0) {
			fn.lxy = make_float4(pmn[0], pmx[0], pmn[1], pmx[1]);
			fn.lrz.x = pmn[2];
			fn.lrz.y = pmx[2];
			fn.refs.x = ref;
		} else {
			fn.rxy = make_float4(pmn[0], pmx[0], pmn[1], pmx[1]);
			fn.lrz.z = pmn[2];
			fn.lrz.w = pmx[2];
			fn.refs.y = ref;
		}
	};

	const TreeNode &root = tree.nodes[0];
	if (root.count) {
		FastNode fn;
		memset(&fn, 0, sizeof(fn));
		set_child(fn, 0, root.bmin, root.bmax, leaf_ref(root));
		/* The right slot is empty.  An inverted box (min +inf, max -inf)
		 * would not do: fast_node's slab test takes the min and max of the
		 * two plane distances, so an inverted box reads as all of space.
		 * NaN planes make the far distance NaN, and `near <= far` is false
		 * for every ray.  The slot names the same leaf, never the root, so
		 * no walk can return to node 0. */
		float nan = NAN;
		fn.rxy = make_float4(nan, nan, nan, nan);
		fn.lrz.z = nan;
		fn.lrz.w = nan;
		fn.refs.y = fn.refs.x;
		nodes.push_back(fn);
		if (kids)
			kids->push_back(make_int2(0, -1));
		return;
	}
	/* depth-first, left child first: the same order serialize_threaded emits
	 * leaf records in, so a triangle's record index is its walk rank */
	std::function<int32_t(int32_t)> emit_node = [&](int32_t i) -> int32_t {
		int32_t me = (int32_t)nodes.size();
		nodes.push_back(FastNode());
		memset(&nodes[me], 0, sizeof(FastNode));
		const TreeNode &n = tree.nodes[i];
		if (kids)
			kids->push_back(make_int2(n.left, n.right));
		for (int side = 0; side < 2; side++) {
			const TreeNode &c = tree.nodes[side == 0 ? n.left : n.right];
			int32_t ref = c.count ? leaf_ref(c) : emit_node(side == 0 ? n.left : n.right);
			set_child(nodes[me], side, c.bmin, c.bmax, ref);
		}
		return me;
	};
	emit_node(0);
}

void build_wide(const Tree &tree, std::vector<WideNode> &nodes, uint32_t &max_stack, std::vector<int4> *kids_out)
{
	nodes.clear();
	max_stack = 0;
	if (kids_out)
		kids_out->clear();
	if (tree.nodes.empty() || tree.nodes[0].count)
		return;
	/* record index of every leaf: the fast layout emits leaves depth-first,
	 * left child first */
	std::vector<uint32_t> first_record(tree.nodes.size(), 0);
	{
		uint32_t next = 0;
		std::vector<int32_t> st(1, 0);
		while (!st.empty()) {
			int32_t i = st.back();
			st.pop_back();
			const TreeNode &n = tree.nodes[i];
			if (n.count) {
				first_record[i] = next;
				next += (uint32_t)n.count;
			} else {
				st.push_back(n.right);
				st.push_back(n.left);
			}
		}
	}
	auto leaf_ref = [&](int32_t i) -> int32_t {
		const TreeNode &n = tree.nodes[i];
		return ~(int32_t)((first_record[i] << 3) | (uint32_t)(n.count - 1));
	};
	/* returns the node index and the stack need of its subtree */
	std::function<int32_t(int32_t, uint32_t &)> emit = [&](int32_t i, uint32_t &need) -> int32_t {
		int32_t kids[4] = {tree.nodes[i].left, tree.nodes[i].right, -1, -1};
		int nk = 2;
		while (nk < 4) {
			int best = -1;
			float best_area = -1.0f;
			for (int k = 0; k < nk; k++) {
				const TreeNode &c = tree.nodes[kids[k]];
				if (c.count)
					continue;
				float a = surface_area(c.bmin, c.bmax);
				if (a > best_area) {
					best_area = a;
					best = k;
				}
			}
			if (best < 0)
				break;
			const TreeNode &c = tree.nodes[kids[best]];
			for (int k = nk; k > best + 1; k--)
				kids[k] = kids[k - 1];
			kids[best] = c.left;
			kids[best + 1] = c.right;
			nk++;
		}
		int32_t me = (int32_t)nodes.size();
		nodes.push_back(WideNode());
		if (kids_out) {
			kids_out->resize(nodes.size());
			(*kids_out)[me] = make_int4(nk > 0 ? kids[0] : -1, nk > 1 ? kids[1] : -1, nk > 2 ? kids[2] : -1,
				nk > 3 ? kids[3] : -1);
		}
		WideNode w;
		float *lo[3] = {&w.lox.x, &w.loy.x, &w.loz.x}, *hi[3] = {&w.hix.x, &w.hiy.x, &w.hiz.x};
		int32_t *refs = &w.refs.x;
		memset(&w, 0, sizeof(w));
		uint32_t child_need = 0;
		for (int k = 0; k < 4; k++) {
			if (k >= nk) {
				for (int a = 0; a < 3; a++) {
					lo[a][k] = 0.0f;
					hi[a][k] = 0.0f;
				}
				refs[k] = KGR_WIDE_EMPTY;
				continue;
			}
			const TreeNode &c = tree.nodes[kids[k]];
			float pmn[3], pmx[3];
			pad_box(c.bmin, c.bmax, pmn, pmx);
			for (int a = 0; a < 3; a++) {
				lo[a][k] = pmn[a];
				hi[a][k] = pmx[a];
			}
			if (c.count) {
				refs[k] = leaf_ref(kids[k]);
			} else {
				uint32_t cn = 0;
				refs[k] = emit(kids[k], cn);
				child_need = cn > child_need ? cn : child_need;
			}
		}
		nodes[me] = w;
		need = (uint32_t)(nk - 1) + child_need;
		return me;
	};
	emit(0, max_stack);
}

/* ======================================================== compressed == */

bool build_cw8(const Tree &tree, const std::vector<float4> &fast_tris, std::vector<CwNode> &nodes,
		std::vector<float4> &cw_tris, uint32_t &depth, std::vector<int32_t> *kids_out)
{
	nodes.clear();
	cw_tris.clear();
	depth = 0;
	if (kids_out)
		kids_out->clear();
	if (tree.nodes.empty())
		return false;
	for (const TreeNode &n : tree.nodes)
		if (n.count > 4)
			return false;
	/* walk rank of every leaf's first triangle: the fast layout emits
	 * leaves depth-first, left child first */
	std::vector<uint32_t> first_record(tree.nodes.size(), 0);
	{
		uint32_t next = 0;
		std::vector<int32_t> st(1, 0);
		while (!st.empty()) {
			int32_t i = st.back();
			st.pop_back();
			const TreeNode &n = tree.nodes[i];
			if (n.count) {
				first_record[i] = next;
				next += (uint32_t)n.count;
			} else {
				st.push_back(n.right);
				st.push_back(n.left);
			}
		}
	}
	struct Job {
		int32_t tree_node; /* a tree node whose children the compressed node gathers (or a root leaf) */
		uint32_t index;
		uint32_t level;
	};
	std::vector<Job> queue;
	queue.push_back({0, 0, 1});
	nodes.push_back(CwNode());
	if (kids_out)
		kids_out->assign(8, -1);
	for (size_t qi = 0; qi < queue.size(); qi++) {
		Job job = queue[qi];
		depth = job.level > depth ? job.level : depth;
		const TreeNode &tn = tree.nodes[job.tree_node];
		/* gather: a root leaf is the node's only child; otherwise open the
		 * largest-area interior child until eight children */
		std::vector<int32_t> kids;
		if (tn.count) {
			kids.push_back(job.tree_node);
		} else {
			kids.push_back(tn.left);
			kids.push_back(tn.right);
			while (kids.size() < 8) {
				int best = -1;
				float best_area = -1.0f;
				for (size_t k = 0; k < kids.size(); k++) {
					const TreeNode &c = tree.nodes[kids[k]];
					if (c.count)
						continue;
					float a = surface_area(c.bmin, c.bmax);
					if (a > best_area) {
						best_area = a;
						best = (int)k;
					}
				}
				if (best < 0)
					break;
				const TreeNode &c = tree.nodes[kids[best]];
				int32_t l = c.left, r = c.right;
				kids[best] = l;
				kids.insert(kids.begin() + best + 1, r);
			}
		}
		int nk = (int)kids.size();
		/* slots: the child whose centroid lies furthest back along an
		 * octant's direction goes to that octant's slot (greedy over the
		 * cheapest (child, slot) pairs), so that a ray of octant o meets
		 * slot o first */
		float cen[8][3], node_c[3] = {0, 0, 0};
		float bmn[3] = {INFINITY, INFINITY, INFINITY}, bmx[3] = {-INFINITY, -INFINITY, -INFINITY};
		for (int k = 0; k < nk; k++) {
			const TreeNode &c = tree.nodes[kids[k]];
			for (int a = 0; a < 3; a++) {
				cen[k][a] = (c.bmin[a] + c.bmax[a]) * 0.5f;
				bmn[a] = c.bmin[a] < bmn[a] ? c.bmin[a] : bmn[a];
				bmx[a] = c.bmax[a] > bmx[a] ? c.bmax[a] : bmx[a];
			}
		}
		for (int a = 0; a < 3; a++)
			node_c[a] = (bmn[a] + bmx[a]) * 0.5f;
		int slot_of[8] = {-1, -1, -1, -1, -1, -1, -1, -1}, kid_in[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
		{
			struct Pair {
				float cost;
				int kid, slot;
			};
			std::vector<Pair> pairs;
			for (int k = 0; k < nk; k++)
				for (int sl = 0; sl < 8; sl++) {
					float dx = (sl & 1) ? -1.0f : 1.0f, dy = (sl & 2) ? -1.0f : 1.0f, dz = (sl & 4) ? -1.0f : 1.0f;
					float cost = (cen[k][0] - node_c[0]) * dx + (cen[k][1] - node_c[1]) * dy
						+ (cen[k][2] - node_c[2]) * dz;
					pairs.push_back({cost, k, sl});
				}
			std::stable_sort(pairs.begin(), pairs.end(), [](const Pair &x, const Pair &y) { return x.cost < y.cost; });
			for (const Pair &pr : pairs)
				if (slot_of[pr.kid] < 0 && kid_in[pr.slot] < 0) {
					slot_of[pr.kid] = pr.slot;
					kid_in[pr.slot] = pr.kid;
				}
		}
		/* internal children: consecutive nodes in slot order; leaves: their
		 * triangle records in slot order */
		uint32_t first_child = (uint32_t)nodes.size(), first_tri = (uint32_t)(cw_tris.size() / 3);
		uint32_t imask = 0, used = 0, meta[8] = {0, 0, 0, 0, 0, 0, 0, 0}, tri_off = 0;
		float lo[8][3], hi[8][3];
		int32_t slot_kids[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
		for (int sl = 0; sl < 8; sl++) {
			int k = kid_in[sl];
			if (k < 0)
				continue;
			int32_t ti = kids[k];
			const TreeNode &c = tree.nodes[ti];
			slot_kids[sl] = ti;
			used |= 1u << sl;
			pad_box(c.bmin, c.bmax, lo[sl], hi[sl]);
			if (c.count) {
				meta[sl] = (uint32_t)c.count << 5 | tri_off;
				for (int32_t t = 0; t < c.count; t++) {
					uint32_t rank = first_record[ti] + (uint32_t)t;
					float4 r0 = fast_tris[3 * (size_t)rank], r1 = fast_tris[3 * (size_t)rank + 1],
					       r2 = fast_tris[3 * (size_t)rank + 2];
					r1.w = fbits((int32_t)rank);
					cw_tris.push_back(r0);
					cw_tris.push_back(r1);
					cw_tris.push_back(r2);
				}
				tri_off += (uint32_t)c.count;
			} else {
				imask |= 1u << sl;
				uint32_t idx = (uint32_t)nodes.size();
				nodes.push_back(CwNode());
				if (kids_out)
					kids_out->insert(kids_out->end(), 8, -1);
				queue.push_back({ti, idx, job.level + 1});
			}
		}
		KGR_REQUIRE(tri_off <= 32, KGR_ERR_INTERNAL, "compressed node with more than 32 triangles");
		KGR_REQUIRE(nodes.size() < (1u << 31) && cw_tris.size() / 3 < (1u << 31), KGR_ERR_UNSUPPORTED,
			"scene too large for the compressed layout");
		CwNode &n = nodes[job.index];
		cw_quantize(lo, hi, used, imask, n.origin, n.qa, n.qb, n.qc);
		n.base = make_uint4(first_child, first_tri, meta[0] | meta[1] << 8 | meta[2] << 16 | meta[3] << 24,
			meta[4] | meta[5] << 8 | meta[6] << 16 | meta[7] << 24);
		if (kids_out)
			for (int sl = 0; sl < 8; sl++)
				(*kids_out)[8 * (size_t)job.index + sl] = slot_kids[sl];
	}
	return true;
}

} /* namespace kgr */

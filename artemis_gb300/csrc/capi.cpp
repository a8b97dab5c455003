/*
 * capi.cpp -- the C ABI of include/kgr.h: scenes, traversal entry points,
 * the path-tracer / ReSTIR attachments and the procedural scene generator.
 *
 * The attachment keeps the life cycle of the reference's AttachmentRTX
 * (include/amadeus/armada.cuh:107-139): attach() learns the extent,
 * load() allocates the per-pixel state (restir.cuh:203-211), unload() frees
 * it, render() launches one frame.  Unlike the reference no render call
 * synchronises the device: every launch is asynchronous on the caller's
 * stream, and the launch sequence has no host round trip, so a frame can be
 * captured into a CUDA graph.
 */
#include <math.h>
#include <string.h>

#include <chrono>
#include <cstdio>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <variant>

#include "kgr_internal.h"
#include "kgr_cache.h"
#include "kgr_gi.h"
#include "kgr_mamba.h"
#include "kgr_wavefront.h"

namespace kgr {
void generate_scene(const std::string &name, uint64_t seed, kgr_generated *g);
}

namespace kgr {

static thread_local std::string g_last_error;

void set_last_error(const std::string &msg) { g_last_error = msg; }

DeviceGuard::DeviceGuard(int device)
{
	if (device < 0)
		return;
	cudaGetDevice(&prev);
	if (prev != device)
		KGR_CUDA(cudaSetDevice(device));
	else
		prev = -1;
}

DeviceGuard::~DeviceGuard()
{
	if (prev >= 0)
		cudaSetDevice(prev);
}

template <class F>
static kgr_status guarded(F &&f)
{
	try {
		f();
		return KGR_OK;
	} catch (const Error &e) {
		set_last_error(e.what());
		return e.status;
	} catch (const std::bad_alloc &) {
		set_last_error("host allocation failed");
		return KGR_ERR_OUT_OF_MEMORY;
	} catch (const std::exception &e) {
		set_last_error(e.what());
		return KGR_ERR_INTERNAL;
	}
}

static int resolve_device(int device);

int pick_device_ordinal(int device) { return resolve_device(device); }

static int resolve_device(int device)
{
	int count = 0;
	cudaError_t e = cudaGetDeviceCount(&count);
	if (e != cudaSuccess || count == 0) {
		cudaGetLastError();
		throw Error(KGR_ERR_NO_DEVICE, "no CUDA device available");
	}
	if (device < 0)
		KGR_CUDA(cudaGetDevice(&device));
	KGR_REQUIRE(device < count, KGR_ERR_INVALID_ARGUMENT, "device ordinal out of range");
	return device;
}

static bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

} /* namespace kgr */

using namespace kgr;

/* ================================================================ scene == */

kgr::DeviceScene kgr_scene::view() const
{
	DeviceScene s;
	s.positions = d_positions.ptr;
	s.normals = d_normals.ptr;
	s.tris = d_tris.ptr;
	s.bvh = d_bvh.ptr;
	s.fast_nodes = d_fast_nodes.ptr;
	s.fast_tris = d_fast_tris.ptr;
	s.wide_nodes = d_wide_nodes.ptr;
	s.materials = d_materials.ptr;
	s.lights = d_lights.ptr;
	s.triangle_count = (uint32_t)(tris4.size() / 4);
	s.light_count = (uint32_t)lights.size();
	s.bvh_vec4_count = (uint32_t)(bvh.size() / 4);
	s.fast_node_count = fast_node_count;
	s.wide_node_count = wide_node_count;
	s.cw_nodes = d_cw_nodes.ptr;
	s.cw_tris = d_cw_tris.ptr;
	s.cw_node_count = cw_node_count;
	s.quads = nullptr;
	s.quad_count = 0;
	s.has_env = 0;
	s.env_flip_v = 0;
	s.env = 0;
	return s;
}

uint64_t kgr_scene::device_bytes() const
{
	return d_positions.bytes() + d_normals.bytes() + d_tris.bytes() + d_bvh.bytes() + d_fast_tris.bytes()
		+ d_fast_nodes.bytes() + d_wide_nodes.bytes() + d_cw_nodes.bytes() + d_cw_tris.bytes() + d_materials.bytes()
		+ d_lights.bytes();
}

namespace {

/* glm::mat4 * vec4(p, w), columns summed in order */
void transform_point(const float *m, const float *p, float w, float *out)
{
	for (int i = 0; i < 3; i++)
		out[i] = m[0 * 4 + i] * p[0] + m[1 * 4 + i] * p[1] + m[2 * 4 + i] * p[2] + m[3 * 4 + i] * w;
}

void gather_meshes(kgr_scene *sc, const kgr_mesh *meshes, uint32_t mesh_count, const kgr_material *materials,
		uint32_t material_count)
{
	KGR_REQUIRE(mesh_count == 0 || meshes, KGR_ERR_INVALID_ARGUMENT, "meshes is NULL");
	KGR_REQUIRE(material_count > 0 && materials, KGR_ERR_INVALID_ARGUMENT, "at least one material is required");
	sc->materials.assign(materials, materials + material_count);
	uint64_t vtotal = 0, ttotal = 0;
	for (uint32_t m = 0; m < mesh_count; m++) {
		vtotal += meshes[m].vertex_count;
		ttotal += meshes[m].triangle_count;
	}
	KGR_REQUIRE(ttotal < (1ull << 27), KGR_ERR_UNSUPPORTED, "more than 2^27 triangles");
	sc->positions.resize(3 * vtotal);
	sc->normals.resize(3 * vtotal);
	sc->tris4.resize(4 * ttotal);
	RefitPlan &pl = sc->plan;
	pl.obj_positions.resize(3 * vtotal);
	pl.obj_normals.assign(3 * vtotal, 0.0f);
	pl.vertex_mesh.resize(vtotal);
	pl.normal_src.assign(vtotal, KGR_NORMAL_ZERO);
	pl.models.assign(16 * (size_t)mesh_count, 0.0f);
	pl.has_model.assign(mesh_count, 0);
	uint64_t vb = 0, tb = 0;
	for (uint32_t m = 0; m < mesh_count; m++) {
		const kgr_mesh &me = meshes[m];
		KGR_REQUIRE(me.vertex_count == 0 || me.positions, KGR_ERR_INVALID_ARGUMENT, "mesh positions are NULL");
		KGR_REQUIRE(me.triangle_count == 0 || me.indices, KGR_ERR_INVALID_ARGUMENT, "mesh indices are NULL");
		if (me.model) {
			memcpy(&pl.models[16 * (size_t)m], me.model, 64);
			pl.has_model[m] = 1;
		}
		if (me.vertex_count)
			memcpy(&pl.obj_positions[3 * vb], me.positions, 12 * (size_t)me.vertex_count);
		if (me.vertex_count && me.normals)
			memcpy(&pl.obj_normals[3 * vb], me.normals, 12 * (size_t)me.vertex_count);
		for (uint32_t v = 0; v < me.vertex_count; v++) {
			pl.vertex_mesh[vb + v] = m;
			if (me.normals)
				pl.normal_src[vb + v] = KGR_NORMAL_OWN;
		}
		for (uint32_t v = 0; v < me.vertex_count; v++) {
			float *pp = &sc->positions[3 * (vb + v)];
			float *nn = &sc->normals[3 * (vb + v)];
			if (me.model) {
				transform_point(me.model, me.positions + 3 * (size_t)v, 1.0f, pp);
				if (me.normals)
					transform_point(me.model, me.normals + 3 * (size_t)v, 0.0f, nn);
			} else {
				memcpy(pp, me.positions + 3 * (size_t)v, 12);
				if (me.normals)
					memcpy(nn, me.normals + 3 * (size_t)v, 12);
			}
		}
		for (uint32_t t = 0; t < me.triangle_count; t++) {
			uint32_t *o = &sc->tris4[4 * (tb + t)];
			for (int k = 0; k < 3; k++) {
				uint32_t idx = me.indices[3 * (size_t)t + k];
				KGR_REQUIRE(idx < me.vertex_count, KGR_ERR_INVALID_ARGUMENT,
					"triangle index out of range in mesh " + std::to_string(m));
				o[k] = (uint32_t)(vb + idx);
			}
			uint32_t mat = me.material_indices ? me.material_indices[t] : 0;
			KGR_REQUIRE(mat < material_count, KGR_ERR_INVALID_ARGUMENT, "material index out of range");
			o[3] = mat;
			if (!me.normals) {
				/* face normal for every vertex of a mesh without normals */
				const float *a = &sc->positions[3 * o[0]], *b = &sc->positions[3 * o[1]],
					    *c = &sc->positions[3 * o[2]];
				float e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
				float e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
				float n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
					e1[0] * e2[1] - e1[1] * e2[0]};
				for (int k = 0; k < 3; k++) {
					memcpy(&sc->normals[3 * o[k]], n, 12);
					pl.normal_src[o[k]] = (int32_t)(tb + t);
				}
			}
		}
		vb += me.vertex_count;
		tb += me.triangle_count;
	}
	/* triangle lights in triangle order (armada.cu:98-212) */
	sc->lights.clear();
	pl.light_tri.clear();
	for (uint64_t t = 0; t < ttotal; t++) {
		const uint32_t *o = &sc->tris4[4 * t];
		const kgr_material &m = sc->materials[o[3]];
		if (!(m.emission[0] > 0 || m.emission[1] > 0 || m.emission[2] > 0))
			continue;
		const float *a = &sc->positions[3 * o[0]], *b = &sc->positions[3 * o[1]], *c = &sc->positions[3 * o[2]];
		kgr_triangle_light l;
		for (int k = 0; k < 3; k++) {
			l.a[k] = a[k];
			l.ab[k] = b[k] - a[k];
			l.ac[k] = c[k] - a[k];
			l.intensity[k] = m.emission[k];
		}
		sc->lights.push_back(l);
		pl.light_tri.push_back((uint32_t)t);
	}
	for (int k = 0; k < 3; k++) {
		sc->bounds_min[k] = INFINITY;
		sc->bounds_max[k] = -INFINITY;
	}
	for (uint64_t v = 0; v < vtotal; v++)
		for (int k = 0; k < 3; k++) {
			sc->bounds_min[k] = fminf(sc->bounds_min[k], sc->positions[3 * v + k]);
			sc->bounds_max[k] = fmaxf(sc->bounds_max[k], sc->positions[3 * v + k]);
		}
}

/* Submesh::bvh boxes (include/mesh.hpp:48-78): min(p1, min(p2, p3)) */
std::vector<PrimBox> prim_boxes(const kgr_scene *sc)
{
	size_t n = sc->tris4.size() / 4;
	std::vector<PrimBox> boxes(n);
	auto gmin = [](float a, float b) { return b < a ? b : a; };
	auto gmax = [](float a, float b) { return a < b ? b : a; };
	for (size_t i = 0; i < n; i++) {
		const float *a = &sc->positions[3 * sc->tris4[4 * i]];
		const float *b = &sc->positions[3 * sc->tris4[4 * i + 1]];
		const float *c = &sc->positions[3 * sc->tris4[4 * i + 2]];
		for (int k = 0; k < 3; k++) {
			boxes[i].bmin[k] = gmin(a[k], gmin(b[k], c[k]));
			boxes[i].bmax[k] = gmax(a[k], gmax(b[k], c[k]));
		}
	}
	return boxes;
}

uint32_t tree_depth(const Tree &t)
{
	if (t.nodes.empty())
		return 0;
	uint32_t best = 0;
	std::vector<std::pair<int32_t, uint32_t>> st = {{0, 1}};
	while (!st.empty()) {
		auto [i, d] = st.back();
		st.pop_back();
		best = d > best ? d : best;
		if (!t.nodes[i].count) {
			st.push_back({t.nodes[i].left, d + 1});
			st.push_back({t.nodes[i].right, d + 1});
		}
	}
	return best;
}

/* The tree half of the refit plan: nodes, primitive order, nodes grouped by
 * depth (deepest first, so a level's children are done before it). */
void plan_tree(RefitPlan &pl, const Tree &tree, std::vector<int32_t> &&rec_node)
{
	size_t n = tree.nodes.size();
	pl.nodes.resize(n);
	for (size_t i = 0; i < n; i++) {
		const TreeNode &t = tree.nodes[i];
		pl.nodes[i] = t.count ? make_int4(-1, -1, t.first, t.count) : make_int4(t.left, t.right, 0, 0);
	}
	pl.prim_order = tree.prim_order;
	pl.rec_node = std::move(rec_node);
	std::vector<std::vector<uint32_t>> levels;
	if (n) {
		std::vector<uint32_t> cur(1, 0u), next;
		while (!cur.empty()) {
			levels.push_back(cur);
			next.clear();
			for (uint32_t i : cur)
				if (!tree.nodes[i].count) {
					next.push_back((uint32_t)tree.nodes[i].left);
					next.push_back((uint32_t)tree.nodes[i].right);
				}
			cur.swap(next);
		}
	}
	pl.level_order.clear();
	pl.level_begin.assign(1, 0u);
	for (size_t l = levels.size(); l-- > 0;) {
		pl.level_order.insert(pl.level_order.end(), levels[l].begin(), levels[l].end());
		pl.level_begin.push_back((uint32_t)pl.level_order.size());
	}
}

void finish_scene(kgr_scene *sc, const Tree &tree, const std::vector<PrimBox> &boxes, std::vector<int32_t> &&rec_node)
{
	KGR_REQUIRE(tree_depth(tree) < KGR_STACK_DEPTH_HOST, KGR_ERR_UNSUPPORTED,
		"BVH deeper than the traversal stack (" + std::to_string(tree_depth(tree)) + " levels)");
	std::vector<FastNode> nodes;
	std::vector<float4> tri_records;
	build_fast(tree, boxes, sc->positions.data(), sc->tris4.data(), nodes, tri_records, &sc->plan.fast_kids);
	sc->fast_node_count = (uint32_t)nodes.size();
	std::vector<WideNode> wide;
	uint32_t wide_stack = 0;
	build_wide(tree, wide, wide_stack, &sc->plan.wide_kids);
	if (wide_stack >= KGR_STACK_DEPTH_HOST) {
		wide.clear(); /* a walk could overflow the stack: fast layout only */
		sc->plan.wide_kids.clear();
	}
	plan_tree(sc->plan, tree, std::move(rec_node));
	sc->wide_node_count = (uint32_t)wide.size();
	sc->wide_max_stack = wide.empty() ? 0 : wide_stack;
	size_t nv = sc->positions.size() / 3, nt = sc->tris4.size() / 4;
	std::vector<float4> p4(nv), n4(nv);
	for (size_t v = 0; v < nv; v++) {
		p4[v] = make_float4(sc->positions[3 * v], sc->positions[3 * v + 1], sc->positions[3 * v + 2], 0.0f);
		n4[v] = make_float4(sc->normals[3 * v], sc->normals[3 * v + 1], sc->normals[3 * v + 2], 0.0f);
	}
	sc->d_positions.upload(p4);
	sc->d_normals.upload(n4);
	sc->d_tris.upload(reinterpret_cast<const uint4 *>(sc->tris4.data()), nt);
	sc->d_bvh.upload(reinterpret_cast<const float4 *>(sc->bvh.data()), sc->bvh.size() / 4);
	sc->d_fast_nodes.upload(nodes);
	if (!wide.empty())
		sc->d_wide_nodes.upload(wide);
	/* the traversal reads nodes with 32-byte vector loads */
	static_assert(sizeof(FastNode) == 64 && sizeof(WideNode) == 128, "node sizes");
	KGR_REQUIRE(((uintptr_t)sc->d_fast_nodes.ptr & 31) == 0 && ((uintptr_t)sc->d_wide_nodes.ptr & 31) == 0,
		KGR_ERR_INTERNAL, "node arrays are not 32-byte aligned");
	sc->d_fast_tris.upload(tri_records);
	std::vector<CwNode> cw;
	std::vector<float4> cw_tris;
	uint32_t cw_depth = 0;
	if (build_cw8(tree, tri_records, cw, cw_tris, cw_depth, &sc->plan.cw_kids) && 2 * cw_depth + 2 <= KGR_CW_STACK) {
		sc->d_cw_nodes.upload(cw);
		sc->d_cw_tris.upload(cw_tris);
		sc->cw_node_count = (uint32_t)cw.size();
		sc->cw_depth = cw_depth;
		static_assert(sizeof(CwNode) == 80, "compressed node size");
		KGR_REQUIRE(((uintptr_t)sc->d_cw_nodes.ptr & 15) == 0, KGR_ERR_INTERNAL, "compressed nodes misaligned");
	} else {
		sc->plan.cw_kids.clear();
	}
	sc->d_materials.upload(sc->materials);
	sc->d_lights.upload(sc->lights);
}

} /* namespace */

extern "C" {

const char *kgr_status_string(kgr_status s)
{
	switch (s) {
	case KGR_OK: return "ok";
	case KGR_ERR_INVALID_ARGUMENT: return "invalid argument";
	case KGR_ERR_OUT_OF_MEMORY: return "out of memory";
	case KGR_ERR_CUDA: return "CUDA error";
	case KGR_ERR_UNSUPPORTED: return "unsupported";
	case KGR_ERR_NOT_ATTACHED: return "attachment not attached";
	case KGR_ERR_NOT_LOADED: return "attachment not loaded";
	case KGR_ERR_BVH_FORMAT: return "malformed BVH";
	case KGR_ERR_BUDGET: return "over memory budget";
	case KGR_ERR_TIMEOUT: return "timed out";
	case KGR_ERR_UNKNOWN_OPTION: return "unknown option";
	case KGR_ERR_TYPE: return "wrong option type";
	case KGR_ERR_INTERNAL: return "internal error";
	case KGR_ERR_NO_DEVICE: return "no CUDA device";
	}
	return "unknown status";
}

const char *kgr_last_error(void) { return g_last_error.c_str(); }

int kgr_abi_version(void) { return KGR_ABI_VERSION; }

kgr_status kgr_scene_create(const kgr_mesh *meshes, uint32_t mesh_count, const kgr_material *materials,
		uint32_t material_count, const kgr_scene_options *options, kgr_scene **out)
{
	return guarded([&] {
		KGR_REQUIRE(out, KGR_ERR_INVALID_ARGUMENT, "out is NULL");
		*out = nullptr;
		kgr_scene_options opt = {KGR_BUILDER_SAH, 4, -1, 0};
		if (options)
			opt = *options;
		int max_leaf = opt.max_leaf_size ? opt.max_leaf_size : 4;
		KGR_REQUIRE(max_leaf >= 1 && max_leaf <= 8, KGR_ERR_INVALID_ARGUMENT, "max_leaf_size must be 1..8");
		KGR_REQUIRE(opt.builder == KGR_BUILDER_SAH || opt.builder == KGR_BUILDER_KOBRA ||
				opt.builder == KGR_BUILDER_SAH_HOST,
			KGR_ERR_INVALID_ARGUMENT, "unknown builder");
		int device = resolve_device(opt.device);
		DeviceGuard guard(device);
		std::unique_ptr<kgr_scene> sc(new kgr_scene());
		sc->device = device;
		gather_meshes(sc.get(), meshes, mesh_count, materials, material_count);
		auto t0 = std::chrono::steady_clock::now();
		std::vector<PrimBox> boxes = prim_boxes(sc.get());
		Tree tree;
		if (opt.builder == KGR_BUILDER_KOBRA)
			build_kobra(boxes, tree);
		else if (opt.builder == KGR_BUILDER_SAH_HOST)
			build_sah(boxes, max_leaf, tree);
		else
			build_sah_gpu(boxes, max_leaf, tree, 0);
		std::vector<int32_t> rec_node;
		serialize_threaded(tree, boxes, sc->bvh, &rec_node);
		sc->build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
		finish_scene(sc.get(), tree, boxes, std::move(rec_node));
		*out = sc.release();
	});
}

kgr_status kgr_scene_create_from_bvh(const kgr_mesh *meshes, uint32_t mesh_count, const kgr_material *materials,
		uint32_t material_count, const float *bvh_vec4, uint32_t bvh_vec4_count, int32_t device,
		kgr_scene **out)
{
	return guarded([&] {
		KGR_REQUIRE(out, KGR_ERR_INVALID_ARGUMENT, "out is NULL");
		*out = nullptr;
		KGR_REQUIRE(bvh_vec4 || bvh_vec4_count == 0, KGR_ERR_INVALID_ARGUMENT, "bvh is NULL");
		int dev = resolve_device(device);
		DeviceGuard guard(dev);
		std::unique_ptr<kgr_scene> sc(new kgr_scene());
		sc->device = dev;
		gather_meshes(sc.get(), meshes, mesh_count, materials, material_count);
		auto t0 = std::chrono::steady_clock::now();
		std::vector<PrimBox> boxes = prim_boxes(sc.get());
		Tree tree;
		std::vector<int32_t> rec_node;
		parse_threaded(bvh_vec4, bvh_vec4_count, (uint32_t)boxes.size(), boxes, tree, &rec_node);
		sc->bvh.assign(bvh_vec4, bvh_vec4 + 4 * (size_t)bvh_vec4_count);
		sc->build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
		finish_scene(sc.get(), tree, boxes, std::move(rec_node));
		*out = sc.release();
	});
}

kgr_status kgr_bvh_build_host(const float *positions, uint32_t vertex_count, const uint32_t *indices,
		uint32_t triangle_count, int32_t builder, int32_t max_leaf_size, float *out_vec4, uint32_t capacity,
		uint32_t *count)
{
	return guarded([&] {
		KGR_REQUIRE(count && (positions || vertex_count == 0) && (indices || triangle_count == 0),
			KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		int max_leaf = max_leaf_size ? max_leaf_size : 4;
		KGR_REQUIRE(max_leaf >= 1 && max_leaf <= 8, KGR_ERR_INVALID_ARGUMENT, "max_leaf_size must be 1..8");
		kgr_scene sc;
		kgr_material m;
		memset(&m, 0, sizeof(m));
		kgr_mesh mesh = {positions, nullptr, vertex_count, indices, nullptr, triangle_count, nullptr};
		gather_meshes(&sc, &mesh, 1, &m, 1);
		std::vector<PrimBox> boxes = prim_boxes(&sc);
		Tree tree;
		if (builder == KGR_BUILDER_KOBRA)
			build_kobra(boxes, tree);
		else
			build_sah(boxes, max_leaf, tree);
		std::vector<float> buf;
		serialize_threaded(tree, boxes, buf);
		*count = (uint32_t)(buf.size() / 4);
		if (out_vec4) {
			KGR_REQUIRE(capacity >= *count, KGR_ERR_INVALID_ARGUMENT, "capacity too small");
			memcpy(out_vec4, buf.data(), buf.size() * sizeof(float));
		}
	});
}

kgr_status kgr_scene_info_get(const kgr_scene *sc, kgr_scene_info *info)
{
	return guarded([&] {
		KGR_REQUIRE(sc && info, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		info->vertex_count = (uint32_t)(sc->positions.size() / 3);
		info->triangle_count = (uint32_t)(sc->tris4.size() / 4);
		info->light_count = (uint32_t)sc->lights.size();
		info->material_count = (uint32_t)sc->materials.size();
		info->bvh_vec4_count = (uint32_t)(sc->bvh.size() / 4);
		info->fast_node_count = sc->fast_node_count;
		info->device_bytes = sc->device_bytes();
		info->build_ms = sc->build_ms;
		memcpy(info->bounds_min, sc->bounds_min, 12);
		memcpy(info->bounds_max, sc->bounds_max, 12);
		info->wide_node_count = sc->wide_node_count;
		info->wide_max_stack = sc->wide_max_stack;
		info->cw8_node_count = sc->cw_node_count;
		info->cw8_depth = sc->cw_depth;
	});
}

/* The host copies of the threaded buffer and the lights hold the scene as
 * created; after a refit the device holds the current ones. */
kgr_status kgr_scene_copy_bvh(const kgr_scene *sc, float *out_vec4, uint32_t capacity, uint32_t *count)
{
	return guarded([&] {
		KGR_REQUIRE(sc && count, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		uint32_t n = (uint32_t)(sc->bvh.size() / 4);
		*count = n;
		if (out_vec4) {
			KGR_REQUIRE(capacity >= n, KGR_ERR_INVALID_ARGUMENT, "capacity too small");
			if (sc->refits && n) {
				DeviceGuard guard(sc->device);
				KGR_CUDA(cudaDeviceSynchronize());
				KGR_CUDA(cudaMemcpy(out_vec4, sc->d_bvh.ptr, (size_t)n * 16, cudaMemcpyDeviceToHost));
			} else {
				memcpy(out_vec4, sc->bvh.data(), sc->bvh.size() * sizeof(float));
			}
		}
	});
}

kgr_status kgr_scene_copy_lights(const kgr_scene *sc, kgr_triangle_light *out, uint32_t capacity, uint32_t *count)
{
	return guarded([&] {
		KGR_REQUIRE(sc && count, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		*count = (uint32_t)sc->lights.size();
		if (out) {
			KGR_REQUIRE(capacity >= sc->lights.size(), KGR_ERR_INVALID_ARGUMENT, "capacity too small");
			if (sc->refits && !sc->lights.empty()) {
				DeviceGuard guard(sc->device);
				KGR_CUDA(cudaDeviceSynchronize());
				KGR_CUDA(cudaMemcpy(out, sc->d_lights.ptr, sc->d_lights.bytes(), cudaMemcpyDeviceToHost));
			} else {
				memcpy(out, sc->lights.data(), sc->lights.size() * sizeof(kgr_triangle_light));
			}
		}
	});
}

kgr_status kgr_scene_copy_vertices(const kgr_scene *sc, float *positions, float *normals)
{
	return guarded([&] {
		KGR_REQUIRE(sc, KGR_ERR_INVALID_ARGUMENT, "NULL scene");
		size_t nv = sc->positions.size() / 3;
		if (!nv)
			return;
		DeviceGuard guard(sc->device);
		KGR_CUDA(cudaDeviceSynchronize());
		std::vector<float4> tmp(nv);
		for (int pass = 0; pass < 2; pass++) {
			float *out = pass == 0 ? positions : normals;
			if (!out)
				continue;
			const float4 *src = pass == 0 ? sc->d_positions.ptr : sc->d_normals.ptr;
			KGR_CUDA(cudaMemcpy(tmp.data(), src, nv * sizeof(float4), cudaMemcpyDeviceToHost));
			for (size_t v = 0; v < nv; v++) {
				out[3 * v] = tmp[v].x;
				out[3 * v + 1] = tmp[v].y;
				out[3 * v + 2] = tmp[v].z;
			}
		}
	});
}

kgr_status kgr_scene_copy_array(const kgr_scene *sc, int32_t which, void *out, uint64_t capacity_bytes,
		uint64_t *bytes)
{
	return guarded([&] {
		KGR_REQUIRE(sc && bytes, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		const void *src = nullptr;
		size_t n = 0;
		switch (which) {
		case KGR_ARRAY_THREADED: src = sc->d_bvh.ptr; n = sc->d_bvh.bytes(); break;
		case KGR_ARRAY_FAST_NODES: src = sc->d_fast_nodes.ptr; n = sc->d_fast_nodes.bytes(); break;
		case KGR_ARRAY_WIDE_NODES: src = sc->d_wide_nodes.ptr; n = sc->d_wide_nodes.bytes(); break;
		case KGR_ARRAY_CW8_NODES: src = sc->d_cw_nodes.ptr; n = sc->d_cw_nodes.bytes(); break;
		case KGR_ARRAY_CW8_TRIANGLES: src = sc->d_cw_tris.ptr; n = sc->d_cw_tris.bytes(); break;
		case KGR_ARRAY_TRIANGLE_RECORDS: src = sc->d_fast_tris.ptr; n = sc->d_fast_tris.bytes(); break;
		default: throw Error(KGR_ERR_INVALID_ARGUMENT, "unknown scene array");
		}
		*bytes = n;
		if (out && n) {
			KGR_REQUIRE(capacity_bytes >= n, KGR_ERR_INVALID_ARGUMENT, "capacity too small");
			DeviceGuard guard(sc->device);
			KGR_CUDA(cudaDeviceSynchronize());
			KGR_CUDA(cudaMemcpy(out, src, n, cudaMemcpyDeviceToHost));
		}
	});
}

kgr_status kgr_scene_set_transforms(kgr_scene *sc, const uint32_t *mesh_ids, const float *models, uint32_t count,
		void *stream)
{
	return guarded([&] {
		KGR_REQUIRE(sc, KGR_ERR_INVALID_ARGUMENT, "NULL scene");
		KGR_REQUIRE(count == 0 || (mesh_ids && models), KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		RefitPlan &pl = sc->plan;
		for (uint32_t i = 0; i < count; i++)
			KGR_REQUIRE(mesh_ids[i] < pl.has_model.size(), KGR_ERR_INVALID_ARGUMENT,
				"mesh index out of range: " + std::to_string(mesh_ids[i]));
		for (uint32_t i = 0; i < count; i++) {
			memcpy(&pl.models[16 * (size_t)mesh_ids[i]], models + 16 * (size_t)i, 64);
			pl.has_model[mesh_ids[i]] = 1;
		}
		DeviceGuard guard(sc->device);
		refit_scene(sc, REFIT_TRANSFORM, nullptr, nullptr, (cudaStream_t)stream);
	});
}

kgr_status kgr_scene_refit(kgr_scene *sc, const float *positions, const float *normals, void *stream)
{
	return guarded([&] {
		KGR_REQUIRE(sc, KGR_ERR_INVALID_ARGUMENT, "NULL scene");
		KGR_REQUIRE(positions || sc->positions.empty(), KGR_ERR_INVALID_ARGUMENT, "positions is NULL");
		DeviceGuard guard(sc->device);
		refit_scene(sc, REFIT_POSITIONS, positions, normals, (cudaStream_t)stream);
	});
}

kgr_status kgr_scene_destroy(kgr_scene *sc)
{
	return guarded([&] {
		if (!sc)
			return;
		DeviceGuard guard(sc->device);
		delete sc;
	});
}

/* ============================================================ traversal == */

namespace {

void check_layout(const kgr_scene *sc, int32_t layout)
{
	KGR_REQUIRE(layout == KGR_LAYOUT_FAST || layout == KGR_LAYOUT_THREADED || layout == KGR_LAYOUT_WIDE
			|| layout == KGR_LAYOUT_CW8,
		KGR_ERR_INVALID_ARGUMENT, "unknown layout");
	KGR_REQUIRE(layout != KGR_LAYOUT_WIDE || sc->wide_node_count, KGR_ERR_UNSUPPORTED,
		"the scene's wide layout was not built (its worst-case walk exceeds the traversal stack)");
	KGR_REQUIRE(layout != KGR_LAYOUT_CW8 || sc->cw_node_count, KGR_ERR_UNSUPPORTED,
		"the scene's compressed layout is not available (leaves over 4 triangles, or dropped by a refit)");
}

} /* namespace */

kgr_status kgr_trace_closest(const kgr_scene *sc, const float *rays, uint32_t n, kgr_hit *hits, int32_t layout,
		void *stream)
{
	return guarded([&] {
		KGR_REQUIRE(sc, KGR_ERR_INVALID_ARGUMENT, "scene is NULL");
		KGR_REQUIRE(n == 0 || (rays && hits), KGR_ERR_INVALID_ARGUMENT, "NULL buffer");
		KGR_REQUIRE(aligned16(rays) && aligned16(hits), KGR_ERR_INVALID_ARGUMENT, "buffers must be 16-byte aligned");
		check_layout(sc, layout);
		DeviceGuard guard(sc->device);
		launch_trace_closest(sc->view(), reinterpret_cast<const float4 *>(rays), n, hits, layout,
			(cudaStream_t)stream);
	});
}

kgr_status kgr_trace_any(const kgr_scene *sc, const float *rays, uint32_t n, uint32_t *occluded, int32_t layout,
		void *stream)
{
	return guarded([&] {
		KGR_REQUIRE(sc, KGR_ERR_INVALID_ARGUMENT, "scene is NULL");
		KGR_REQUIRE(n == 0 || (rays && occluded), KGR_ERR_INVALID_ARGUMENT, "NULL buffer");
		KGR_REQUIRE(aligned16(rays), KGR_ERR_INVALID_ARGUMENT, "rays must be 16-byte aligned");
		check_layout(sc, layout);
		DeviceGuard guard(sc->device);
		launch_trace_any(sc->view(), reinterpret_cast<const float4 *>(rays), n, occluded, layout,
			(cudaStream_t)stream);
	});
}

kgr_status kgr_trace_closest_host(const kgr_scene *sc, const float *rays, uint32_t n, kgr_hit *hits, int32_t layout)
{
	return guarded([&] {
		KGR_REQUIRE(sc, KGR_ERR_INVALID_ARGUMENT, "scene is NULL");
		KGR_REQUIRE(n == 0 || (rays && hits), KGR_ERR_INVALID_ARGUMENT, "NULL buffer");
		check_layout(sc, layout);
		if (n == 0)
			return;
		DeviceGuard guard(sc->device);
		DevBuf<float4> dr;
		DevBuf<kgr_hit> dh;
		dr.upload(reinterpret_cast<const float4 *>(rays), 2 * (size_t)n);
		dh.alloc(n);
		launch_trace_closest(sc->view(), dr.ptr, n, dh.ptr, layout, 0);
		KGR_CUDA(cudaMemcpy(hits, dh.ptr, n * sizeof(kgr_hit), cudaMemcpyDeviceToHost));
	});
}

kgr_status kgr_trace_any_host(const kgr_scene *sc, const float *rays, uint32_t n, uint32_t *occluded, int32_t layout)
{
	return guarded([&] {
		KGR_REQUIRE(sc, KGR_ERR_INVALID_ARGUMENT, "scene is NULL");
		KGR_REQUIRE(n == 0 || (rays && occluded), KGR_ERR_INVALID_ARGUMENT, "NULL buffer");
		check_layout(sc, layout);
		if (n == 0)
			return;
		DeviceGuard guard(sc->device);
		DevBuf<float4> dr;
		DevBuf<uint32_t> dout;
		dr.upload(reinterpret_cast<const float4 *>(rays), 2 * (size_t)n);
		dout.alloc(n);
		launch_trace_any(sc->view(), dr.ptr, n, dout.ptr, layout, 0);
		KGR_CUDA(cudaMemcpy(occluded, dout.ptr, n * sizeof(uint32_t), cudaMemcpyDeviceToHost));
	});
}

kgr_status kgr_trace_counts(const kgr_scene *sc, const float *rays, uint32_t n, int32_t any, uint64_t *counts)
{
	return guarded([&] {
		KGR_REQUIRE(sc && counts, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		KGR_REQUIRE(n == 0 || rays, KGR_ERR_INVALID_ARGUMENT, "rays is NULL");
		DeviceGuard guard(sc->device);
		DevBuf<unsigned long long> dc;
		dc.alloc(4);
		KGR_CUDA(cudaMemset(dc.ptr, 0, 4 * sizeof(unsigned long long)));
		launch_trace_stats(sc->view(), reinterpret_cast<const float4 *>(rays), n, any, dc.ptr, 0);
		KGR_CUDA(cudaMemcpy(counts, dc.ptr, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
	});
}

} /* extern "C" */

/* ========================================================== attachments == */

namespace {

enum Kind { KIND_PT = 0, KIND_RESTIR_DI = 1, KIND_RESTIR_GI = 2, KIND_MAMBA = 3 };

using OptionValue = std::variant<int, float, bool, std::string>;

struct Timing {
	cudaEvent_t ev[2] = {nullptr, nullptr};
};

} /* namespace */

struct kgr_attachment {
	Kind kind;
	std::string name;
	bool attached = false, loaded = false;
	uint32_t width = 0, height = 0;
	int device = 0;
	std::map<std::string, OptionValue> options;
	std::string option_string; /* storage for get_option strings */

	/* path state */
	DevBuf<float4> f4[KGR_PATH_ARRAYS];
	DevBuf<uint32_t> queues[3];
	DevBuf<uint32_t> counters;
	uint32_t capacity = 0;

	/* ReSTIR state */
	DevBuf<float4> res_a[2], res_b[2], intermediate, auxiliary;
	DevBuf<kgr_material> pixel_materials;
	int prev_index = 1;
	bool have_prev_camera = false;
	float prev_projection[16], prev_view[16], prev_center[3];

	/* ReSTIR GI state */
	DevBuf<float4> gi_a[3], gi_b[3], g_pos, g_nrm, g_ppos, g_pnrm, g_direct, g_dir;
	DevBuf<int2> di_neighbours;
	DevBuf<float> di_targets;
	DevBuf<uint32_t> di_vis_queue[2], di_vis_count;
	/* the visibility rounds' rays, blocked flags and walk counters */
	DevBuf<float4> di_vis_o, di_vis_d;
	DevBuf<uint32_t> di_vis_flag;
	DevBuf<float4> gi_selection;
	DevBuf<int2> gi_neighbours;
	DevBuf<float> gi_weights;
	DevBuf<uint32_t> gi_vis_queue[2], gi_vis_count;
	DevBuf<float4> gi_vis_o, gi_vis_d;
	DevBuf<uint32_t> gi_vis_flag;
	int gi_prev = 0;

	/* Mamba state: G-buffer, reservoirs, secondary rays, probe table; which
	 * reservoir and previous sets are current; the next depth stamp */
	MambaBuffers mamba;
	bool mamba_loaded = false;
	int mamba_res_in = 0, mamba_prev_in = 0;
	uint64_t mamba_stamp = 0;

	/* radiance cache: network, query rows, training paths, records, batch */
	kgr_mlp *cache_mlp = nullptr;
	DevBuf<uint16_t> q_feat, r_feat, b_x;
	DevBuf<float4> q_le, q_out, r_beta, r_lb, r_le, b_t;
	DevBuf<uint32_t> b_count;
	DevBuf<float4> t_L; /* final radiance of each training path */
	/* training runs on a side stream, overlapped with the frame:
	 * fork -> (side) training paths, targets, gradient -> wait for the
	 * frame's inference -> Adam -> join */
	cudaStream_t side = nullptr;
	cudaEvent_t ev_fork = nullptr, ev_infer = nullptr, ev_train = nullptr;
	/* the plain tracer's overlap of a bounce's shadow rays with the next
	 * bounce's closest hits (render_pt) */
	cudaEvent_t ev_shaded = nullptr, ev_shadowed = nullptr;
	/* the cached frame's shadow rays, beside the side stream's training */
	cudaStream_t side2 = nullptr;

	kgr_render_stats stats = {0, 0, 0, 0, 0};
	uint32_t last_paths = 0;
	cudaEvent_t ev_start = nullptr, ev_stop = nullptr;

	/* per-launch timing: one event after every launch, tagged by stage */
	std::vector<cudaEvent_t> event_pool;
	std::vector<int> event_kinds; /* kind of the launch that ends at event i; -1 = start */
	std::vector<int> event_prev;  /* the event a span ends after: i - 1 unless given */
	double stage_ms[STAGE_COUNT] = {0};
	uint32_t stage_launches[STAGE_COUNT] = {0};
	DevBuf<unsigned long long> visits;

	bool profiling() const { return opt_int("profile", 0) != 0; }
	/* Record an event on `st` ending a span of stage `kind` (-1: a start)
	 * that began at event `prev` (default: the previous event, which must
	 * then be on the same stream).  Returns the event's index. */
	int mark(int kind, cudaStream_t st, int prev = -1)
	{
		if (!profiling())
			return -1;
		size_t i = event_kinds.size();
		if (i == event_pool.size()) {
			cudaEvent_t e;
			KGR_CUDA(cudaEventCreate(&e));
			event_pool.push_back(e);
		}
		KGR_CUDA(cudaEventRecord(event_pool[i], st));
		event_kinds.push_back(kind);
		event_prev.push_back(prev);
		return (int)i;
	}
	/* fold recorded events into per-stage totals (waits for every event) */
	void collect_times()
	{
		if (event_kinds.empty())
			return;
		for (size_t i = 0; i < event_kinds.size(); i++)
			KGR_CUDA(cudaEventSynchronize(event_pool[i]));
		for (size_t i = 1; i < event_kinds.size(); i++) {
			int k = event_kinds[i];
			if (k < 0)
				continue;
			int j = event_prev[i] >= 0 ? event_prev[i] : (int)i - 1;
			float ms = 0.0f;
			KGR_CUDA(cudaEventElapsedTime(&ms, event_pool[j], event_pool[i]));
			stage_ms[k] += ms;
			stage_launches[k]++;
		}
		event_kinds.clear();
		event_prev.clear();
	}

	int opt_int(const char *k, int def) const
	{
		auto it = options.find(k);
		if (it == options.end())
			return def;
		if (auto p = std::get_if<int>(&it->second))
			return *p;
		if (auto b = std::get_if<bool>(&it->second))
			return *b ? 1 : 0;
		return def;
	}
	float opt_float(const char *k, float def) const
	{
		auto it = options.find(k);
		if (it == options.end())
			return def;
		if (auto p = std::get_if<float>(&it->second))
			return *p;
		if (auto i = std::get_if<int>(&it->second))
			return (float)*i;
		return def;
	}
	std::string opt_str(const char *k, const std::string &def) const
	{
		auto it = options.find(k);
		if (it == options.end())
			return def;
		if (auto p = std::get_if<std::string>(&it->second))
			return *p;
		return def;
	}
	/* The layout option ("fast" | "threaded" | "wide" | "cw8"); unset, the layout
	 * kgr_autotune chose (fast when nothing was tuned). */
	int tuned_layout = KGR_LAYOUT_FAST;
	int layout() const
	{
		std::string l = opt_str("layout", "");
		if (l == "threaded")
			return KGR_LAYOUT_THREADED;
		if (l == "fast")
			return KGR_LAYOUT_FAST;
		if (l == "wide")
			return KGR_LAYOUT_WIDE;
		if (l == "cw8")
			return KGR_LAYOUT_CW8;
		return tuned_layout;
	}

	/* Launch shape of the fast/wide traversal: the shape kgr_autotune chose
	 * (or the default), with any field the options set overriding it:
	 * trace_shadow "grid" | "persistent", trace_block 64 | 128 | 256,
	 * trace_occupancy 0 | 1, trace_stack 0 | 8 | 16. */
	TraceTune tuned = default_trace_tune();
	TraceTune trace_tune() const
	{
		TraceTune t = tuned;
		std::string a = opt_str("trace_shadow", "");
		if (a == "grid")
			t.shadow = TRACE_GRID;
		else if (a == "persistent")
			t.shadow = TRACE_PERSISTENT;
		int b = opt_int("trace_block", 0);
		if (b == 64 || b == 128 || b == 256)
			t.block = (int16_t)b;
		int o = opt_int("trace_occupancy", -1);
		if (o == 0 || o == 1)
			t.occupancy = (int16_t)o;
		int k = opt_int("trace_stack", -1);
		if (k == 0 || k == 8 || k == 16)
			t.stack = (int16_t)k;
		return t;
	}

	PathBuffers path_buffers()
	{
		PathBuffers pb;
		float4 **fields[KGR_PATH_ARRAYS];
		path_array_slots(pb, fields);
		for (int k = 0; k < KGR_PATH_ARRAYS; k++)
			*fields[k] = f4[k].ptr;
		pb.queue[0] = queues[0].ptr;
		pb.queue[1] = queues[1].ptr;
		pb.shadow_queue = queues[2].ptr;
		pb.counters = counters.ptr;
		if (opt_int("count_visits", 0) && !visits.ptr)
			visits.alloc(4);
		pb.visits = opt_int("count_visits", 0) ? visits.ptr : nullptr;
		pb.capacity = capacity;
		return pb;
	}

	void ensure_paths(uint32_t paths)
	{
		if (paths <= capacity)
			return;
		for (auto &b : f4)
			b.alloc(paths);
		for (auto &q : queues)
			q.alloc(paths);
		capacity = paths;
	}

	void release_all()
	{
		if (side)
			cudaStreamSynchronize(side);
		if (side2)
			cudaStreamSynchronize(side2);
		for (auto &b : f4)
			b.release();
		for (auto &q : queues)
			q.release();
		counters.release();
		for (int k = 0; k < 2; k++) {
			res_a[k].release();
			res_b[k].release();
		}
		intermediate.release();
		auxiliary.release();
		pixel_materials.release();
		for (int k = 0; k < 3; k++) {
			gi_a[k].release();
			gi_b[k].release();
		}
		for (DevBuf<float4> *b : {&g_pos, &g_nrm, &g_ppos, &g_pnrm, &g_direct, &g_dir})
			b->release();
		di_neighbours.release();
		di_targets.release();
		di_vis_queue[0].release();
		di_vis_queue[1].release();
		di_vis_count.release();
		di_vis_o.release();
		di_vis_d.release();
		di_vis_flag.release();
		gi_selection.release();
		gi_neighbours.release();
		gi_weights.release();
		gi_vis_queue[0].release();
		gi_vis_queue[1].release();
		gi_vis_count.release();
		gi_vis_o.release();
		gi_vis_d.release();
		gi_vis_flag.release();
		for (DevBuf<uint16_t> *b : {&q_feat, &r_feat, &b_x})
			b->release();
		for (DevBuf<float4> *b : {&q_le, &q_out, &r_beta, &r_lb, &r_le, &b_t})
			b->release();
		b_count.release();
		t_L.release();
		if (mamba_loaded) {
			mamba_free(mamba);
			mamba_loaded = false;
		}
		capacity = 0;
	}

	/* path buffers of the cache's training paths */
	/* Forget the temporal history -- reservoirs, per-pixel materials, the
	 * previous camera -- as load() leaves it (asynchronous on st). */
	void reset_history(cudaStream_t st)
	{
		size_t npix = (size_t)width * height;
		if (kind == KIND_RESTIR_DI && res_a[0].ptr) {
			for (int k = 0; k < 2; k++) {
				KGR_CUDA(cudaMemsetAsync(res_a[k].ptr, 0xff, npix * sizeof(float4), st));
				KGR_CUDA(cudaMemsetAsync(res_b[k].ptr, 0, npix * sizeof(float4), st));
			}
			KGR_CUDA(cudaMemsetAsync(pixel_materials.ptr, 0, npix * sizeof(kgr_material), st));
			prev_index = 1;
		}
		if (kind == KIND_RESTIR_GI && gi_a[0].ptr) {
			for (int k = 0; k < 3; k++) {
				KGR_CUDA(cudaMemsetAsync(gi_a[k].ptr, 0, npix * sizeof(float4), st));
				KGR_CUDA(cudaMemsetAsync(gi_b[k].ptr, 0, npix * sizeof(float4), st));
			}
			for (DevBuf<float4> *b : {&g_pos, &g_nrm, &g_ppos, &g_pnrm, &g_direct, &g_dir, &auxiliary})
				KGR_CUDA(cudaMemsetAsync(b->ptr, 0, npix * sizeof(float4), st));
			KGR_CUDA(cudaMemsetAsync(pixel_materials.ptr, 0, npix * sizeof(kgr_material), st));
			gi_prev = 0;
		}
		if (kind == KIND_MAMBA && mamba_loaded) {
			mamba_reset(mamba, width, height, st);
			mamba_res_in = mamba_prev_in = 0;
			mamba_stamp = 0;
		}
		have_prev_camera = false;
	}

	void ensure_side_stream()
	{
		if (side)
			return;
		KGR_CUDA(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
		KGR_CUDA(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
		KGR_CUDA(cudaEventCreateWithFlags(&ev_infer, cudaEventDisableTiming));
		KGR_CUDA(cudaEventCreateWithFlags(&ev_train, cudaEventDisableTiming));
		KGR_CUDA(cudaEventCreateWithFlags(&ev_shaded, cudaEventDisableTiming));
		KGR_CUDA(cudaEventCreateWithFlags(&ev_shadowed, cudaEventDisableTiming));
		KGR_CUDA(cudaStreamCreateWithFlags(&side2, cudaStreamNonBlocking));
	}

	~kgr_attachment()
	{
		release_all();
		if (cache_mlp)
			kgr_mlp_destroy(cache_mlp);
		for (cudaEvent_t e : {ev_fork, ev_infer, ev_train, ev_shaded, ev_shadowed})
			if (e)
				cudaEventDestroy(e);
		if (side)
			cudaStreamDestroy(side);
		if (side2)
			cudaStreamDestroy(side2);
		visits.release();
		if (ev_start)
			cudaEventDestroy(ev_start);
		if (ev_stop)
			cudaEventDestroy(ev_stop);
		for (cudaEvent_t e : event_pool)
			cudaEventDestroy(e);
	}
};

namespace {

void mat4_mul(const float *a, const float *b, float *out)
{
	for (int j = 0; j < 4; j++)
		for (int i = 0; i < 4; i++)
			out[j * 4 + i] = a[0 * 4 + i] * b[j * 4 + 0] + a[1 * 4 + i] * b[j * 4 + 1]
				+ a[2 * 4 + i] * b[j * 4 + 2] + a[3 * 4 + i] * b[j * 4 + 3];
}

void check_launch(const kgr_attachment *att, const kgr_launch_info *info, const kgr_scene *sc)
{
	KGR_REQUIRE(att, KGR_ERR_INVALID_ARGUMENT, "attachment is NULL");
	KGR_REQUIRE(att->attached, KGR_ERR_NOT_ATTACHED, "attach() was not called");
	KGR_REQUIRE(att->loaded, KGR_ERR_NOT_LOADED, "load() was not called");
	KGR_REQUIRE(info && sc, KGR_ERR_INVALID_ARGUMENT, "NULL launch info or scene");
	KGR_REQUIRE(sc->device == att->device, KGR_ERR_INVALID_ARGUMENT, "scene and attachment are on different devices");
	KGR_REQUIRE((uint32_t)info->resolution[0] == att->width && (uint32_t)info->resolution[1] == att->height,
		KGR_ERR_INVALID_ARGUMENT, "resolution differs from the attached extent");
	KGR_REQUIRE(info->lights.quad_count >= 0 && info->lights.tri_count >= 0, KGR_ERR_INVALID_ARGUMENT,
		"negative light count");
	KGR_REQUIRE(info->lights.quad_count == 0 || (info->lights.quad_lights && aligned16(info->lights.quad_lights)),
		KGR_ERR_INVALID_ARGUMENT, "quad_lights must be a 16-byte aligned device array when quad_count > 0");
	KGR_REQUIRE(!info->has_environment_map || info->environment_map, KGR_ERR_INVALID_ARGUMENT,
		"has_environment_map is set but environment_map is 0");
	KGR_REQUIRE(info->buffers.color, KGR_ERR_INVALID_ARGUMENT, "color buffer is NULL");
	const void *bufs[4] = {info->buffers.color, info->buffers.normal, info->buffers.albedo, info->buffers.position};
	for (const void *b : bufs)
		KGR_REQUIRE(aligned16(b), KGR_ERR_INVALID_ARGUMENT, "output buffers must be 16-byte aligned");
	KGR_REQUIRE(info->max_depth >= 0 && info->max_depth <= 64, KGR_ERR_INVALID_ARGUMENT, "max_depth out of range");
}

FrameParams frame_params(const kgr_attachment *att, const kgr_launch_info *info, const kgr_scene *sc)
{
	FrameParams fp;
	memset(&fp, 0, sizeof(fp));
	fp.width = att->width;
	fp.height = att->height;
	fp.npix = att->width * att->height;
	memcpy(fp.center, info->camera.center, 12);
	memcpy(fp.U, info->camera.ax_u, 12);
	memcpy(fp.V, info->camera.ax_v, 12);
	memcpy(fp.W, info->camera.ax_w, 12);
	int md = att->opt_int("max_depth", -1);
	fp.max_depth = md >= 0 ? md : info->max_depth;
	fp.russian_roulette = att->opt_int("russian_roulette", 0);
	fp.rr_start_depth = att->opt_int("rr_start_depth", 3);
	fp.frame = info->frame;
	fp.accumulate = info->accumulate ? 1 : 0;
	fp.samples = info->samples;
	fp.layout = layout_for(att->layout(), sc);
	fp.tune = att->trace_tune();
	fp.candidates = att->opt_int("candidates", 32);
	fp.temporal = att->opt_int("temporal", 1);
	fp.temporal_mcap = att->opt_int("temporal_mcap", 200);
	fp.spatial_neighbors = att->opt_int("spatial_neighbors", 5);
	fp.spatial_radius = att->opt_int("spatial_radius", 30);
	return fp;
}

/* The scene as a launch sees it: the caller's triangle lights and materials
 * when given, its quad lights and environment map.  flip_v: the miss
 * program's (u, 1 - v) of the path tracer rather than ReSTIR's (u, v). */
DeviceScene scene_for_launch(const kgr_scene *sc, const kgr_launch_info *info, bool flip_v = false)
{
	DeviceScene s = sc->view();
	if (info->lights.tri_lights) {
		s.lights = info->lights.tri_lights;
		s.light_count = (uint32_t)info->lights.tri_count;
	}
	if (info->materials)
		s.materials = info->materials;
	if (info->lights.quad_count > 0) {
		s.quads = info->lights.quad_lights;
		s.quad_count = (uint32_t)info->lights.quad_count;
	}
	if (info->has_environment_map) {
		s.has_env = 1;
		s.env = (unsigned long long)info->environment_map;
		s.env_flip_v = flip_v ? 1 : 0;
	}
	return s;
}

/* Zero the visit counters at the start of a frame when counting is on. */
void prepare_visits(kgr_attachment *att, cudaStream_t st)
{
	if (!att->opt_int("count_visits", 0))
		return;
	if (!att->visits.ptr)
		att->visits.alloc(4);
	KGR_CUDA(cudaMemsetAsync(att->visits.ptr, 0, 4 * sizeof(unsigned long long), st));
}

void render_pt(kgr_attachment *att, const kgr_launch_info *info, const kgr_scene *sc, cudaStream_t st)
{
	FrameParams fp = frame_params(att, info, sc);
	int spp = att->opt_int("spp", 1);
	KGR_REQUIRE(spp >= 1 && spp <= 4096, KGR_ERR_INVALID_ARGUMENT, "spp out of range");
	uint64_t paths = (uint64_t)fp.npix * (uint64_t)spp;
	KGR_REQUIRE(paths < (1ull << 31), KGR_ERR_UNSUPPORTED, "too many paths per frame");
	fp.spp = (uint32_t)spp;
	fp.paths = (uint32_t)paths;
	fp.jitter = 1;
	att->ensure_paths(fp.paths);
	PathBuffers pb = att->path_buffers();
	DeviceScene s = scene_for_launch(sc, info, true);
	OutputBuffers out = {reinterpret_cast<float4 *>(info->buffers.color),
		reinterpret_cast<float4 *>(info->buffers.normal), reinterpret_cast<float4 *>(info->buffers.albedo),
		reinterpret_cast<float4 *>(info->buffers.position)};
	/* bounces 0 .. max_depth; a ray past the last vertex would add nothing,
	 * hit or miss (LOAD_RAYPACKET, amadeus_common.cuh:480-488) */
	const int last = fp.max_depth;
	uint32_t launches = 0;
	prepare_visits(att, st);
	int m = att->mark(-1, st);
	pt_generate(pb, fp, st);
	m = att->mark(STAGE_GENERATE, st, m);
	launches++;
	if (att->opt_int("trace_overlap", 1)) {
		/* bounce d's shadow rays on the side stream while bounce d + 1's
		 * closest hits run here: the two persistent launches share the GPU,
		 * and each fills the SMs the other's tail leaves idle.  They touch
		 * disjoint arrays and counters; the next shade waits for both, so
		 * every path's radiance is still summed in the order of the
		 * recursion. */
		att->ensure_side_stream();
		cudaStream_t side = att->side;
		pt_trace_closest(s, pb, 0, fp.layout, fp.tune, st);
		m = att->mark(STAGE_TRACE_CLOSEST, st, m);
		for (int d = 0; d <= last; d++) {
			int q = d & 1;
			if (d > 0) {
				reset_counters(pb, (1 << (q ^ 1)) | (1 << CNT_SHADOW), st);
				m = att->mark(-1, st);
			}
			pt_shade(s, pb, fp, d, q, st);
			m = att->mark(STAGE_SHADE, st, m);
			KGR_CUDA(cudaEventRecord(att->ev_shaded, st));
			KGR_CUDA(cudaStreamWaitEvent(side, att->ev_shaded, 0));
			int ms = att->mark(-1, side);
			pt_shadow_resolve(s, pb, fp.layout, fp.tune, side);
			att->mark(STAGE_SHADOW, side, ms);
			KGR_CUDA(cudaEventRecord(att->ev_shadowed, side));
			if (d < last) {
				pt_trace_closest(s, pb, q ^ 1, fp.layout, fp.tune, st);
				m = att->mark(STAGE_TRACE_CLOSEST, st, m);
			}
			KGR_CUDA(cudaStreamWaitEvent(st, att->ev_shadowed, 0));
			m = att->mark(-1, st);
			launches += 3;
		}
	} else {
		for (int d = 0; d <= last; d++) {
			int q = d & 1;
			if (d > 0) {
				reset_counters(pb, (1 << (q ^ 1)) | (1 << CNT_SHADOW), st);
				m = att->mark(-1, st);
			}
			pt_trace_closest(s, pb, q, fp.layout, fp.tune, st);
			m = att->mark(STAGE_TRACE_CLOSEST, st, m);
			pt_shade(s, pb, fp, d, q, st);
			m = att->mark(STAGE_SHADE, st, m);
			pt_shadow_resolve(s, pb, fp.layout, fp.tune, st);
			m = att->mark(STAGE_SHADOW, st, m);
			launches += 3;
		}
	}
	pt_accumulate(pb, fp, out, st);
	att->mark(STAGE_ACCUMULATE, st);
	launches++;
	att->stats.kernel_launches = launches;
	att->stats.camera_rays = fp.paths;
	att->last_paths = fp.paths;
}

void render_restir_di(kgr_attachment *att, const kgr_launch_info *info, const kgr_scene *sc, cudaStream_t st)
{
	FrameParams fp = frame_params(att, info, sc);
	fp.spp = 1;
	fp.paths = fp.npix;
	fp.jitter = 0;
	KGR_REQUIRE(fp.spatial_neighbors >= 0 && fp.spatial_neighbors <= KGR_MAX_NEIGHBORS, KGR_ERR_INVALID_ARGUMENT,
		"spatial_neighbors must be 0..16");
	KGR_REQUIRE(fp.candidates >= 1 && fp.candidates <= 1024, KGR_ERR_INVALID_ARGUMENT, "candidates must be 1..1024");
	KGR_REQUIRE(info->buffers.normal && info->buffers.albedo && info->buffers.position, KGR_ERR_INVALID_ARGUMENT,
		"ReSTIR needs the normal, albedo and position buffers");
	if (!att->have_prev_camera) {
		memcpy(att->prev_projection, info->camera.projection, 64);
		memcpy(att->prev_view, info->camera.view, 64);
		att->have_prev_camera = true;
	}
	mat4_mul(att->prev_projection, att->prev_view, fp.prev_proj_view);
	att->ensure_paths(fp.paths);
	PathBuffers pb = att->path_buffers();
	DeviceScene s = scene_for_launch(sc, info);
	OutputBuffers out = {reinterpret_cast<float4 *>(info->buffers.color),
		reinterpret_cast<float4 *>(info->buffers.normal), reinterpret_cast<float4 *>(info->buffers.albedo),
		reinterpret_cast<float4 *>(info->buffers.position)};
	RestirFrameBuffers rb;
	for (int k = 0; k < 2; k++) {
		rb.res[k].a = att->res_a[k].ptr;
		rb.res[k].b = att->res_b[k].ptr;
	}
	rb.materials = att->pixel_materials.ptr;
	rb.intermediate = att->intermediate.ptr;
	rb.auxiliary = att->auxiliary.ptr;
	rb.neighbours = att->di_neighbours.ptr;
	rb.targets = att->di_targets.ptr;
	rb.vis_queue[0] = att->di_vis_queue[0].ptr;
	rb.vis_queue[1] = att->di_vis_queue[1].ptr;
	rb.vis_count = att->di_vis_count.ptr;
	rb.vis_o = att->di_vis_o.ptr;
	rb.vis_d = att->di_vis_d.ptr;
	rb.vis_flag = att->di_vis_flag.ptr;
	rb.vis_capacity = (uint32_t)att->di_vis_o.count;
	rb.ray_total = pb.counters + CNT_SHADOW_TOTAL;
	KGR_REQUIRE(fp.paths <= rb.vis_capacity, KGR_ERR_INTERNAL, "ReSTIR visibility buffers below the path count");
	int prev = att->prev_index, cur = 1 - prev;
	uint32_t launches = 0;

	/* initial pass */
	prepare_visits(att, st);
	KGR_CUDA(cudaMemsetAsync(rb.res[cur].b, 0, sizeof(float4) * fp.npix, st));
	att->mark(-1, st);
	pt_generate(pb, fp, st);
	att->mark(STAGE_GENERATE, st);
	pt_trace_closest(s, pb, 0, fp.layout, fp.tune, st);
	att->mark(STAGE_TRACE_CLOSEST, st);
	restir_primary(s, pb, fp, rb, cur, st);
	att->mark(STAGE_RESTIR_PRIMARY, st);
	launches += 2 + KGR_RESTIR_PRIMARY_LAUNCHES; /* generate, closest hit, primary vertex, its shadow rays */
	/* with an environment map one more bounce is traced for its misses */
	for (int d = 1; d <= fp.max_depth; d++) {
		int q = d & 1;
		reset_counters(pb, (1 << (q ^ 1)) | (1 << CNT_SHADOW), st);
		att->mark(-1, st);
		pt_trace_closest(s, pb, q, fp.layout, fp.tune, st);
		att->mark(STAGE_TRACE_CLOSEST, st);
		pt_shade_final_seed(s, pb, fp, d, q, st);
		att->mark(STAGE_SHADE, st);
		pt_shadow_resolve(s, pb, fp.layout, fp.tune, st);
		att->mark(STAGE_SHADOW, st);
		launches += 3;
	}
	restir_finalize(pb, fp, rb, out, st);
	att->mark(STAGE_RESTIR_FINALIZE, st);
	launches++;
	/* temporal pass */
	if (fp.temporal) {
		restir_temporal(s, fp, rb, out, cur, prev, st, [&](int k) { att->mark(k, st); });
		launches += KGR_RESTIR_TEMPORAL_LAUNCHES;
	}
	/* spatial passes with the ping-pong of restir.cuh:280-300 */
	int passes = att->opt_int("spatial_passes", 2);
	KGR_REQUIRE(passes >= 0 && passes <= 16, KGR_ERR_INVALID_ARGUMENT, "spatial_passes must be 0..16");
	int in = cur, outb = prev;
	for (int k = 0; k < passes; k++) {
		restir_spatial(s, fp, rb, out, in, outb, st, [&](int k) { att->mark(k, st); });
		std::swap(in, outb);
		launches += KGR_RESTIR_SPATIAL_LAUNCHES;
	}
	att->prev_index = in;
	memcpy(att->prev_projection, info->camera.projection, 64);
	memcpy(att->prev_view, info->camera.view, 64);
	att->stats.kernel_launches = launches;
	att->stats.camera_rays = fp.paths;
	att->last_paths = fp.paths;
}

/* The editor's Mamba frame (Mamba::render, editor/mamba.cu:941-1312): see
 * kgr_mamba.h.  Its options are the reference's Mamba switches:
 * direct_lighting, indirect_lighting, irradiance, render_probes and
 * render_probe_radiance (Mamba::options, editor/mamba.cuh:60-67),
 * temporal_reuse and spatial_reuse (:57-58). */
void render_mamba(kgr_attachment *att, const kgr_launch_info *info, const kgr_scene *sc, cudaStream_t st)
{
	KGR_REQUIRE(info->lights.quad_count == 0, KGR_ERR_UNSUPPORTED,
		"the mamba attachment samples the scene's triangle lights and the environment only");
	KGR_REQUIRE(att->mamba_loaded, KGR_ERR_NOT_LOADED, "load() was not called");
	FrameParams fp = frame_params(att, info, sc);
	MambaParams mp;
	memset(&mp, 0, sizeof(mp));
	mp.width = att->width;
	mp.height = att->height;
	mp.npix = att->width * att->height;
	mp.sec_w = att->width / 4 + 1;
	mp.sec_h = att->height / 4 + 1;
	memcpy(mp.origin, info->camera.center, 12);
	memcpy(mp.U, info->camera.ax_u, 12);
	memcpy(mp.V, info->camera.ax_v, 12);
	memcpy(mp.W, info->camera.ax_w, 12);
	if (!att->have_prev_camera) {
		memcpy(att->prev_projection, info->camera.projection, 64);
		memcpy(att->prev_view, info->camera.view, 64);
		att->have_prev_camera = true;
	}
	mat4_mul(att->prev_projection, att->prev_view, mp.prev_proj_view);
	mp.time = info->time;
	mp.samples = info->samples;
	KGR_REQUIRE(mp.samples >= 0, KGR_ERR_INVALID_ARGUMENT, "samples must be >= 0");
	mp.direct_lighting = att->opt_int("direct_lighting", 0);
	mp.indirect_lighting = att->opt_int("indirect_lighting", 0);
	mp.irradiance = att->opt_int("irradiance", 1);
	mp.render_probes = att->opt_int("render_probes", 0);
	mp.render_probe_radiance = att->opt_int("render_probe_radiance", 0);
	mp.temporal = att->opt_int("temporal_reuse", 0);
	mp.spatial = att->opt_int("spatial_reuse", 0);
	mp.layout = fp.layout;
	mp.res_in = att->mamba_res_in;
	mp.prev_in = att->mamba_prev_in;
	uint64_t records = 2ull * mp.sec_w * mp.sec_h;
	if (att->mamba_stamp + records + 1 > 0xFFFFFFFFull) {
		mamba_restamp(att->mamba.table, st);
		att->mamba_stamp = 0;
	}
	mp.stamp_base = (uint32_t)att->mamba_stamp;
	att->mamba_stamp += records;
	mamba_bin_directions(mp.bin_dir);
	att->ensure_paths(mp.npix);
	PathBuffers pb = att->path_buffers();
	prepare_visits(att, st);
	DeviceScene s = scene_for_launch(sc, info);
	att->mark(-1, st);
	uint32_t launches = mamba_render(s, pb, mp, att->mamba, fp.tune, reinterpret_cast<float4 *>(info->buffers.color),
		st, [&](int k) { att->mark(k, st); });
	if (mp.direct_lighting && mp.spatial)
		att->mamba_res_in = 1 - att->mamba_res_in;
	if (mp.direct_lighting && (mp.temporal || mp.spatial))
		att->mamba_prev_in = 1 - att->mamba_prev_in;
	memcpy(att->prev_projection, info->camera.projection, 64);
	memcpy(att->prev_view, info->camera.view, 64);
	att->stats.kernel_launches = launches;
	att->stats.camera_rays = mp.npix;
	att->last_paths = mp.npix;
}

/* Path tracer with the radiance cache: render paths end at the first bounce
 * with a network query; training paths (plain, full depth) train it. */
void render_pt_cached(kgr_attachment *att, const kgr_launch_info *info, const kgr_scene *sc, cudaStream_t st)
{
	FrameParams fp = frame_params(att, info, sc);
	int spp = att->opt_int("spp", 1);
	KGR_REQUIRE(spp >= 1 && spp <= 4096, KGR_ERR_INVALID_ARGUMENT, "spp out of range");
	KGR_REQUIRE(fp.max_depth >= 1, KGR_ERR_INVALID_ARGUMENT, "the cached tracer needs max_depth >= 1");
	uint64_t paths = (uint64_t)fp.npix * (uint64_t)spp;
	KGR_REQUIRE(paths < (1ull << 31), KGR_ERR_UNSUPPORTED, "too many paths per frame");
	fp.spp = (uint32_t)spp;
	fp.paths = (uint32_t)paths;
	fp.jitter = 1;
	att->ensure_paths(fp.paths);
	PathBuffers pb = att->path_buffers();
	DeviceScene s = scene_for_launch(sc, info);
	OutputBuffers out = {reinterpret_cast<float4 *>(info->buffers.color),
		reinterpret_cast<float4 *>(info->buffers.normal), reinterpret_cast<float4 *>(info->buffers.albedo),
		reinterpret_cast<float4 *>(info->buffers.position)};
	int dtype = att->opt_str("cache_dtype", "bf16") == "fp16" ? KGR_MLP_FP16 : KGR_MLP_BF16;
	if (!att->cache_mlp || att->cache_mlp->dtype != dtype) {
		if (att->cache_mlp)
			kgr_mlp_destroy(att->cache_mlp);
		att->cache_mlp = nullptr;
		KGR_REQUIRE(kgr_mlp_create(dtype, 1, att->device, &att->cache_mlp) == KGR_OK, KGR_ERR_CUDA,
			std::string("radiance cache: ") + kgr_last_error());
	}
	att->cache_mlp->infer = att->opt_str("cache_infer", "tcgen05") == "mma" ? KGR_MLP_INFER_MMA : KGR_MLP_INFER_TCGEN05;
	MlpParams mp = att->cache_mlp->params();
	CacheParams cp;
	cp.dtype = dtype;
	for (int k = 0; k < 3; k++) {
		cp.bmin[k] = sc->bounds_min[k];
		float ext = sc->bounds_max[k] - sc->bounds_min[k];
		cp.binv[k] = ext > 0.0f ? 1.0f / ext : 1.0f;
	}
	att->q_feat.alloc((size_t)att->capacity * 64);
	att->q_le.alloc(att->capacity);
	att->q_out.alloc(att->capacity);
	uint32_t launches = 0;
	const bool train = att->opt_int("cache_train", 1) != 0;
	float lr = 1e-3f;
	{
		auto it = att->options.find("cache_lr");
		if (it != att->options.end())
			if (auto f = std::get_if<float>(&it->second))
				lr = *f;
	}

	/* training, forked onto the side stream: paths, targets, gradient with
	 * the weights this frame's inference also reads */
	int train_start = -1;
	if (train) {
		uint32_t tpaths = (uint32_t)att->opt_int("cache_train_paths", 16384);
		KGR_REQUIRE(tpaths >= 128 && tpaths <= (1u << 22), KGR_ERR_INVALID_ARGUMENT, "cache_train_paths out of range");
		const uint32_t cap = 1u << 16;
		int depths = fp.max_depth + 1;
		size_t slots = (size_t)tpaths * depths;
		att->ensure_side_stream();
		att->t_L.alloc(tpaths);
		att->r_feat.alloc(slots * 64);
		att->r_beta.alloc(slots);
		att->r_lb.alloc(slots);
		att->r_le.alloc(slots);
		att->b_x.alloc((size_t)cap * 64);
		att->b_t.alloc(cap);
		att->b_count.alloc(1);
		cudaStream_t side = att->side;
		KGR_CUDA(cudaEventRecord(att->ev_fork, st));
		KGR_CUDA(cudaStreamWaitEvent(side, att->ev_fork, 0));
		train_start = att->mark(-1, side);
		KGR_CUDA(cudaMemsetAsync(att->r_le.ptr, 0, slots * sizeof(float4), side));
		CacheRecords rec = {att->r_feat.ptr, att->r_beta.ptr, att->r_lb.ptr, att->r_le.ptr, depths};
		PathBuffers tb = {};
		tb.L = att->t_L.ptr;
		tb.capacity = tpaths;
		FrameParams tf = fp;
		tf.spp = 1;
		tf.paths = tpaths;
		cache_train_paths(s, tb, tf, tpaths, cp, rec, side);
		cache_targets(tb, tpaths, rec, dtype, att->b_x.ptr, att->b_t.ptr, att->b_count.ptr, cap, side);
		/* a quarter of the SMs: the frame keeps the rest (cached terrain
		 * frame 2.01 -> 1.96 ms against a full grid) */
		mlp_gradients(mp, att->b_x.ptr, att->b_t.ptr, cap, att->cache_mlp->grad.ptr, att->cache_mlp->loss.ptr, side,
			att->b_count.ptr, (device_sm_count() + 3) / 4);
		launches += 4;
	}

	/* render: primary vertex, first bounce, cache.  The primary vertex's
	 * shadow rays run on a second side stream while the first bounce is
	 * traced and queried (the overlap of render_pt); they join before the
	 * cache's radiance is added, so each path's radiance is summed in the
	 * order of the recursion. */
	const bool overlap = att->opt_int("trace_overlap", 1) != 0;
	if (overlap)
		att->ensure_side_stream();
	int m = att->mark(-1, st);
	pt_generate(pb, fp, st);
	m = att->mark(STAGE_GENERATE, st, m);
	pt_trace_closest(s, pb, 0, fp.layout, fp.tune, st);
	m = att->mark(STAGE_TRACE_CLOSEST, st, m);
	pt_shade(s, pb, fp, 0, 0, st);
	m = att->mark(STAGE_SHADE, st, m);
	if (overlap) {
		KGR_CUDA(cudaEventRecord(att->ev_shaded, st));
		KGR_CUDA(cudaStreamWaitEvent(att->side2, att->ev_shaded, 0));
		int ms = att->mark(-1, att->side2);
		pt_shadow_resolve(s, pb, fp.layout, fp.tune, att->side2);
		att->mark(STAGE_SHADOW, att->side2, ms);
		KGR_CUDA(cudaEventRecord(att->ev_shadowed, att->side2));
	} else {
		pt_shadow_resolve(s, pb, fp.layout, fp.tune, st);
		m = att->mark(STAGE_SHADOW, st, m);
	}
	pt_trace_closest(s, pb, 1, fp.layout, fp.tune, st);
	m = att->mark(STAGE_TRACE_CLOSEST, st, m);
	cache_query(s, pb, 1, cp, att->q_feat.ptr, att->q_le.ptr, st);
	mlp_infer(mp, att->q_feat.ptr, att->capacity, att->q_out.ptr, st, pb.counters + CNT_Q1);
	if (train)
		KGR_CUDA(cudaEventRecord(att->ev_infer, st));
	if (overlap)
		KGR_CUDA(cudaStreamWaitEvent(st, att->ev_shadowed, 0));
	reset_counters(pb, (1 << CNT_Q0) | (1 << CNT_SHADOW), st);
	cache_apply(pb, 1, att->q_out.ptr, att->q_le.ptr, st);
	m = att->mark(STAGE_CACHE_INFER, st, m);
	pt_accumulate(pb, fp, out, st);
	att->mark(STAGE_ACCUMULATE, st, m);
	launches += 10;

	/* Adam once this frame's inference is done, then join */
	if (train) {
		cudaStream_t side = att->side;
		KGR_CUDA(cudaStreamWaitEvent(side, att->ev_infer, 0));
		att->cache_mlp->step++;
		mlp_adam(mp, att->cache_mlp->grad.ptr, lr, att->cache_mlp->step, side);
		att->mark(STAGE_CACHE_TRAIN, side, train_start);
		KGR_CUDA(cudaEventRecord(att->ev_train, side));
		KGR_CUDA(cudaStreamWaitEvent(st, att->ev_train, 0));
		launches += 1;
	}
	att->stats.kernel_launches = launches;
	att->stats.camera_rays = fp.paths;
	att->last_paths = fp.paths;
}

/* One ReSTIR GI frame: primary vertex (G-buffer, DI candidates, GI
 * direction), the GI path from the secondary vertex, initial reservoirs,
 * temporal reuse, spatial iterations (ping-pong), final shading. */
void render_restir_gi(kgr_attachment *att, const kgr_launch_info *info, const kgr_scene *sc, cudaStream_t st)
{
	FrameParams fp = frame_params(att, info, sc);
	fp.spp = 1;
	fp.paths = fp.npix;
	fp.jitter = 1;
	fp.gi_capture = 1;
	fp.gi_mcap = att->opt_int("gi_mcap", 30);
	fp.gi_jmax = att->opt_float("gi_jacobian_max", 4.0f);
	KGR_REQUIRE(fp.gi_jmax >= 1.0f, KGR_ERR_INVALID_ARGUMENT, "gi_jacobian_max must be >= 1");
	fp.gi_confidence_rule = att->opt_int("gi_neighbor_confidence", 1);
	fp.gi_neighbors = att->opt_int("gi_neighbors", 8);
	fp.gi_radius = att->opt_int("gi_radius", 30);
	KGR_REQUIRE(fp.gi_neighbors >= 0 && fp.gi_neighbors <= KGR_GI_MAX_NEIGHBORS, KGR_ERR_INVALID_ARGUMENT,
		"gi_neighbors must be 0..16");
	KGR_REQUIRE(fp.candidates >= 1 && fp.candidates <= 1024, KGR_ERR_INVALID_ARGUMENT, "candidates must be 1..1024");
	KGR_REQUIRE(fp.max_depth >= 1, KGR_ERR_INVALID_ARGUMENT, "ReSTIR GI needs max_depth >= 1");
	if (!att->have_prev_camera) {
		memcpy(att->prev_projection, info->camera.projection, 64);
		memcpy(att->prev_view, info->camera.view, 64);
		memcpy(att->prev_center, info->camera.center, 12);
		att->have_prev_camera = true;
	}
	mat4_mul(att->prev_projection, att->prev_view, fp.prev_proj_view);
	memcpy(fp.prev_center, att->prev_center, 12);
	att->ensure_paths(fp.paths);
	PathBuffers pb = att->path_buffers();
	DeviceScene s = scene_for_launch(sc, info);
	OutputBuffers out = {reinterpret_cast<float4 *>(info->buffers.color),
		reinterpret_cast<float4 *>(info->buffers.normal), reinterpret_cast<float4 *>(info->buffers.albedo),
		reinterpret_cast<float4 *>(info->buffers.position)};
	GiFrameBuffers gb;
	for (int k = 0; k < 3; k++) {
		gb.res[k].a = att->gi_a[k].ptr;
		gb.res[k].b = att->gi_b[k].ptr;
	}
	gb.materials = att->pixel_materials.ptr;
	gb.position = att->g_pos.ptr;
	gb.normal = att->g_nrm.ptr;
	gb.prev_position = att->g_ppos.ptr;
	gb.prev_normal = att->g_pnrm.ptr;
	gb.direct = att->g_direct.ptr;
	gb.gi_dir = att->g_dir.ptr;
	gb.auxiliary = att->auxiliary.ptr;
	gb.selection = att->gi_selection.ptr;
	gb.neighbours = att->gi_neighbours.ptr;
	gb.weights = att->gi_weights.ptr;
	gb.vis_queue[0] = att->gi_vis_queue[0].ptr;
	gb.vis_queue[1] = att->gi_vis_queue[1].ptr;
	gb.vis_count = att->gi_vis_count.ptr;
	gb.vis_o = att->gi_vis_o.ptr;
	gb.vis_d = att->gi_vis_d.ptr;
	gb.vis_flag = att->gi_vis_flag.ptr;
	gb.vis_capacity = (uint32_t)att->gi_vis_o.count;
	gb.ray_total = pb.counters + CNT_SHADOW_TOTAL;
	KGR_REQUIRE(fp.paths <= gb.vis_capacity, KGR_ERR_INTERNAL, "GI visibility buffers below the path count");
	int prev = att->gi_prev, cur = (prev + 1) % 3, tmp = (prev + 2) % 3;
	uint32_t launches = 0;

	prepare_visits(att, st);
	att->mark(-1, st);
	pt_generate(pb, fp, st);
	att->mark(STAGE_GENERATE, st);
	pt_trace_closest(s, pb, 0, fp.layout, fp.tune, st);
	att->mark(STAGE_TRACE_CLOSEST, st);
	gi_primary(s, pb, fp, gb, st);
	att->mark(STAGE_RESTIR_PRIMARY, st);
	launches += 2 + KGR_GI_PRIMARY_LAUNCHES; /* generate, closest hit, primary vertex, its shadow rays */
	for (int d = 1; d <= fp.max_depth; d++) {
		int q = d & 1;
		reset_counters(pb, (1 << (q ^ 1)) | (1 << CNT_SHADOW), st);
		att->mark(-1, st);
		pt_trace_closest(s, pb, q, fp.layout, fp.tune, st);
		att->mark(STAGE_TRACE_CLOSEST, st);
		pt_shade_final_seed(s, pb, fp, d, q, st);
		att->mark(STAGE_SHADE, st);
		pt_shadow_resolve(s, pb, fp.layout, fp.tune, st);
		att->mark(STAGE_SHADOW, st);
		launches += 3;
	}
	gi_initial(pb, fp, gb, cur, st);
	att->mark(STAGE_RESTIR_FINALIZE, st);
	launches++;
	if (att->opt_int("gi_temporal", 1)) {
		gi_temporal(s, fp, gb, cur, prev, st);
		att->mark(STAGE_RESTIR_TEMPORAL, st);
		launches++;
	}
	int iters = att->opt_int("gi_spatial_iterations", 3);
	KGR_REQUIRE(iters >= 0 && iters <= 16, KGR_ERR_INVALID_ARGUMENT, "gi_spatial_iterations must be 0..16");
	int in = cur, outb = tmp;
	for (int k = 0; k < iters; k++) {
		gi_spatial(s, fp, gb, in, outb, k, st);
		att->mark(STAGE_RESTIR_SPATIAL, st);
		std::swap(in, outb);
		launches += KGR_GI_SPATIAL_LAUNCHES;
	}
	gi_final(s, fp, gb, out, in, st);
	att->mark(STAGE_ACCUMULATE, st);
	launches += KGR_GI_FINAL_LAUNCHES;
	att->gi_prev = in;
	memcpy(att->prev_projection, info->camera.projection, 64);
	memcpy(att->prev_view, info->camera.view, 64);
	memcpy(att->prev_center, info->camera.center, 12);
	att->stats.kernel_launches = launches;
	att->stats.camera_rays = fp.paths;
	att->last_paths = fp.paths;
}

} /* namespace */

namespace kgr {

void attachment_ray_totals_async(const kgr_attachment *att, uint32_t *dst, cudaStream_t st)
{
	static_assert(CNT_SHADOW_TOTAL == CNT_BOUNCE_TOTAL + 1, "the two totals are adjacent");
	KGR_REQUIRE(att->loaded && att->counters.ptr, KGR_ERR_NOT_LOADED, "attachment is not loaded");
	KGR_CUDA(cudaMemcpyAsync(dst, att->counters.ptr + CNT_BOUNCE_TOTAL, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost,
		st));
}

} /* namespace kgr */

extern "C" {

kgr_status kgr_create(const char *kind, kgr_attachment **out)
{
	return guarded([&] {
		KGR_REQUIRE(kind && out, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		*out = nullptr;
		std::string k(kind);
		Kind kd;
		std::string name;
		if (k == "path_tracer") {
			kd = KIND_PT;
			name = "Path Tracer";
		} else if (k == "restir_di" || k == "restir") {
			kd = KIND_RESTIR_DI;
			name = "ReSTIR";
		} else if (k == "restir_gi") {
			kd = KIND_RESTIR_GI;
			name = "ReSTIR GI";
		} else if (k == "mamba") {
			kd = KIND_MAMBA;
			name = "Mamba";
		} else {
			throw Error(KGR_ERR_INVALID_ARGUMENT, "unknown attachment kind: " + k);
		}
		kgr_attachment *a = new kgr_attachment();
		a->kind = kd;
		a->name = name;
		*out = a;
	});
}

kgr_status kgr_attach(kgr_attachment *att, const kgr_context *ctx)
{
	return guarded([&] {
		KGR_REQUIRE(att && ctx, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		KGR_REQUIRE(ctx->width > 0 && ctx->height > 0, KGR_ERR_INVALID_ARGUMENT, "empty extent");
		KGR_REQUIRE((uint64_t)ctx->width * ctx->height < (1ull << 30), KGR_ERR_UNSUPPORTED, "extent too large");
		int dev = resolve_device(ctx->device);
		if (att->loaded) {
			DeviceGuard g(att->device);
			att->release_all();
			att->loaded = false;
		}
		att->device = dev;
		att->width = ctx->width;
		att->height = ctx->height;
		att->attached = true;
		att->have_prev_camera = false;
	});
}

kgr_status kgr_load(kgr_attachment *att)
{
	return guarded([&] {
		KGR_REQUIRE(att, KGR_ERR_INVALID_ARGUMENT, "attachment is NULL");
		KGR_REQUIRE(att->attached, KGR_ERR_NOT_ATTACHED, "attach() was not called");
		DeviceGuard g(att->device);
		size_t npix = (size_t)att->width * att->height;
		try {
			att->counters.alloc(CNT_COUNT);
			KGR_CUDA(cudaMemset(att->counters.ptr, 0, CNT_COUNT * sizeof(uint32_t)));
			if (att->kind == KIND_RESTIR_DI) {
				for (int k = 0; k < 2; k++) {
					att->res_a[k].alloc(npix);
					att->res_b[k].alloc(npix);
					KGR_CUDA(cudaMemset(att->res_a[k].ptr, 0xff, npix * sizeof(float4)));
					KGR_CUDA(cudaMemset(att->res_b[k].ptr, 0, npix * sizeof(float4)));
				}
				att->intermediate.alloc(npix);
				att->auxiliary.alloc(npix);
				att->pixel_materials.alloc(npix);
				KGR_CUDA(cudaMemset(att->pixel_materials.ptr, 0, npix * sizeof(kgr_material)));
				att->di_neighbours.alloc(npix * KGR_MAX_NEIGHBORS);
				att->di_targets.alloc(npix * (KGR_MAX_NEIGHBORS + 1));
				att->di_vis_queue[0].alloc(npix * KGR_MAX_NEIGHBORS);
				att->di_vis_queue[1].alloc(npix * (KGR_MAX_NEIGHBORS + 1));
				att->di_vis_count.alloc(2 * CNT_COUNT); /* a counter array per visibility round */
				att->di_vis_o.alloc(npix * (KGR_MAX_NEIGHBORS + 1));
				att->di_vis_d.alloc(npix * (KGR_MAX_NEIGHBORS + 1));
				att->di_vis_flag.alloc(npix * (KGR_MAX_NEIGHBORS + 1));
				KGR_CUDA(cudaMemset(att->di_vis_flag.ptr, 0, npix * (KGR_MAX_NEIGHBORS + 1) * sizeof(uint32_t)));
				att->prev_index = 1;
				att->ensure_paths((uint32_t)npix);
			}
			if (att->kind == KIND_RESTIR_GI) {
				for (int k = 0; k < 3; k++) {
					att->gi_a[k].alloc(npix);
					att->gi_b[k].alloc(npix);
					KGR_CUDA(cudaMemset(att->gi_a[k].ptr, 0, npix * sizeof(float4)));
					KGR_CUDA(cudaMemset(att->gi_b[k].ptr, 0, npix * sizeof(float4)));
				}
				for (DevBuf<float4> *b : {&att->g_pos, &att->g_nrm, &att->g_ppos, &att->g_pnrm, &att->g_direct,
					     &att->g_dir, &att->auxiliary}) {
					b->alloc(npix);
					KGR_CUDA(cudaMemset(b->ptr, 0, npix * sizeof(float4)));
				}
				att->pixel_materials.alloc(npix);
				KGR_CUDA(cudaMemset(att->pixel_materials.ptr, 0, npix * sizeof(kgr_material)));
				att->gi_selection.alloc(npix);
				att->gi_neighbours.alloc(npix * KGR_GI_MAX_NEIGHBORS);
				att->gi_weights.alloc(npix * KGR_GI_MAX_NEIGHBORS);
				att->gi_vis_queue[0].alloc(npix * KGR_GI_MAX_NEIGHBORS);
				att->gi_vis_queue[1].alloc(npix * KGR_GI_MAX_NEIGHBORS);
				att->gi_vis_count.alloc(2 * CNT_COUNT); /* a counter array per visibility round */
				att->gi_vis_o.alloc(npix);
				att->gi_vis_d.alloc(npix);
				att->gi_vis_flag.alloc(npix);
				KGR_CUDA(cudaMemset(att->gi_vis_flag.ptr, 0, npix * sizeof(uint32_t)));
				att->gi_prev = 0;
				att->ensure_paths((uint32_t)npix);
			}
			if (att->kind == KIND_MAMBA) {
				mamba_alloc(att->mamba, att->width, att->height, att->opt_int("max_probes", 1 << 20),
					att->opt_int("max_luts", 1024));
				att->mamba_loaded = true;
				att->mamba_res_in = att->mamba_prev_in = 0;
				att->mamba_stamp = 0;
				att->ensure_paths((uint32_t)npix);
			}
			if (!att->ev_start) {
				KGR_CUDA(cudaEventCreate(&att->ev_start));
				KGR_CUDA(cudaEventCreate(&att->ev_stop));
			}
		} catch (...) {
			att->release_all();
			throw;
		}
		att->loaded = true;
	});
}

kgr_status kgr_unload(kgr_attachment *att)
{
	return guarded([&] {
		KGR_REQUIRE(att, KGR_ERR_INVALID_ARGUMENT, "attachment is NULL");
		if (!att->loaded)
			return;
		DeviceGuard g(att->device);
		att->release_all();
		att->loaded = false;
	});
}

kgr_status kgr_destroy(kgr_attachment *att)
{
	return guarded([&] {
		if (!att)
			return;
		DeviceGuard g(att->attached ? att->device : -1);
		delete att;
	});
}

/* Known options, their types and defaults.  Unknown names are ignored, as
 * the reference's attachments ignore them (naive_path_tracer.cu:215-225);
 * a known name with the wrong type is rejected with KGR_ERR_TYPE (the
 * reference logs a warning and keeps the old value). */
static const std::map<std::string, OptionValue> &option_defaults()
{
	static const std::map<std::string, OptionValue> d = {
		{"max_depth", -1}, {"russian_roulette", false}, {"rr_start_depth", 3}, {"spp", 1},
		{"layout", std::string("fast")}, {"candidates", 32}, {"temporal", true}, {"temporal_mcap", 200},
		{"spatial_passes", 2}, {"spatial_neighbors", 5}, {"spatial_radius", 30},
		{"profile", false}, {"count_visits", false},
		{"gi_temporal", true}, {"gi_mcap", 30}, {"gi_spatial_iterations", 3}, {"gi_neighbors", 8},
		{"gi_radius", 30}, {"gi_jacobian_max", 4.0f}, {"gi_neighbor_confidence", true},
		{"cache", false}, {"cache_train", true}, {"cache_train_paths", 16384}, {"cache_lr", 1e-3f},
		{"cache_dtype", std::string("bf16")}, {"cache_infer", std::string("tcgen05")}, {"reset_history", false},
		{"trace_shadow", std::string("")}, {"trace_block", 0}, {"trace_occupancy", -1}, {"trace_stack", -1},
		{"trace_overlap", true},
		{"direct_lighting", false}, {"indirect_lighting", false}, {"irradiance", true}, {"render_probes", false},
		{"render_probe_radiance", false}, {"temporal_reuse", false}, {"spatial_reuse", false},
		{"max_probes", 1 << 20}, {"max_luts", 1024}};
	return d;
}

kgr_status kgr_set_option(kgr_attachment *att, const char *name, const kgr_value *value)
{
	return guarded([&] {
		KGR_REQUIRE(att && name && value, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		auto it = option_defaults().find(name);
		if (it == option_defaults().end())
			return;
		OptionValue v;
		switch (value->tag) {
		case KGR_VALUE_INT: v = (int)value->i; break;
		case KGR_VALUE_FLOAT: v = value->f; break;
		case KGR_VALUE_BOOL: v = value->b != 0; break;
		case KGR_VALUE_STRING:
			KGR_REQUIRE(value->s, KGR_ERR_INVALID_ARGUMENT, "NULL string value");
			v = std::string(value->s);
			break;
		default: throw Error(KGR_ERR_TYPE, "option value has no type");
		}
		KGR_REQUIRE(v.index() == it->second.index(), KGR_ERR_TYPE, std::string("wrong type for option ") + name);
		if (std::string(name) == "layout") {
			const std::string &s = std::get<std::string>(v);
			KGR_REQUIRE(s == "fast" || s == "threaded" || s == "wide" || s == "cw8", KGR_ERR_INVALID_ARGUMENT,
				"layout is fast, threaded, wide or cw8");
		}
		att->options[name] = v;
	});
}

kgr_status kgr_get_option(const kgr_attachment *att, const char *name, kgr_value *value)
{
	return guarded([&] {
		KGR_REQUIRE(att && name && value, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		memset(value, 0, sizeof(*value));
		auto d = option_defaults().find(name);
		if (d == option_defaults().end()) {
			/* AttachmentRTX::get_option returns {} -- a variant holding int 0 */
			value->tag = KGR_VALUE_INT;
			return;
		}
		auto it = att->options.find(name);
		const OptionValue &v = it == att->options.end() ? d->second : it->second;
		if (auto p = std::get_if<int>(&v)) {
			value->tag = KGR_VALUE_INT;
			value->i = *p;
		} else if (auto f = std::get_if<float>(&v)) {
			value->tag = KGR_VALUE_FLOAT;
			value->f = *f;
		} else if (auto b = std::get_if<bool>(&v)) {
			value->tag = KGR_VALUE_BOOL;
			value->b = *b;
		} else {
			const_cast<kgr_attachment *>(att)->option_string = std::get<std::string>(v);
			value->tag = KGR_VALUE_STRING;
			value->s = att->option_string.c_str();
		}
	});
}

namespace {

/* One frame of an attachment on `st` (the body of kgr_render). */
void render_frame(kgr_attachment *att, const kgr_launch_info *info, const kgr_scene *sc, cudaStream_t st)
{
	if (att->opt_int("reset_history", 0)) {
		att->reset_history(st);
		att->options.erase("reset_history");
	}
	/* the radiance cache and ReSTIR GI have no reference counterpart; they
	 * light with the scene's triangles only */
	bool extra_lights = info->lights.quad_count > 0 || info->has_environment_map;
	KGR_REQUIRE(!(extra_lights && (att->kind == KIND_RESTIR_GI || (att->kind == KIND_PT && att->opt_int("cache", 0)))),
		KGR_ERR_UNSUPPORTED, "quad lights and environment maps are supported by the plain path tracer and ReSTIR DI");
	switch (att->kind) {
	case KIND_PT:
		if (att->opt_int("cache", 0))
			render_pt_cached(att, info, sc, st);
		else
			render_pt(att, info, sc, st);
		break;
	case KIND_RESTIR_DI: render_restir_di(att, info, sc, st); break;
	case KIND_RESTIR_GI: render_restir_gi(att, info, sc, st); break;
	case KIND_MAMBA: render_mamba(att, info, sc, st); break;
	default: throw Error(KGR_ERR_UNSUPPORTED, "attachment kind not built");
	}
}

} /* namespace */

kgr_status kgr_render(kgr_attachment *att, const kgr_launch_info *info, const kgr_scene *sc, void *stream)
{
	return guarded([&] {
		check_launch(att, info, sc);
		DeviceGuard g(att->device);
		render_frame(att, info, sc, (cudaStream_t)stream);
	});
}

kgr_status kgr_autotune(kgr_attachment *att, const kgr_launch_info *info, const kgr_scene *sc, int32_t frames,
		void *stream, kgr_autotune_result *result)
{
	return guarded([&] {
		check_launch(att, info, sc);
		KGR_REQUIRE(frames >= 1 && frames <= 256, KGR_ERR_INVALID_ARGUMENT, "frames must be 1..256");
		DeviceGuard g(att->device);
		cudaStream_t st = (cudaStream_t)stream;
		/* the options override the tuned shape: set them aside while tuning */
		std::map<std::string, OptionValue> held;
		for (const char *k : {"layout", "trace_shadow", "trace_block", "trace_occupancy", "trace_stack"}) {
			auto it = att->options.find(k);
			if (it != att->options.end()) {
				held[k] = it->second;
				att->options.erase(it);
			}
		}
		int old_layout = att->tuned_layout;
		TraceTune old_tune = att->tuned;
		kgr_autotune_result res;
		memset(&res, 0, sizeof(res));
		try {
			double best = -1.0;
			for (const kgr_trace_tune &c : tune_candidates(sc)) {
				att->tuned_layout = c.layout;
				att->tuned.shadow = (int16_t)c.shadow;
				att->tuned.block = (int16_t)c.block;
				att->tuned.occupancy = (int16_t)c.occupancy;
				att->tuned.stack = (int16_t)c.stack;
				double ms = time_frames([&] { render_frame(att, info, sc, st); }, frames, st);
				if (is_default_shape(c))
					res.default_ms = ms;
				if (best < 0.0 || ms < best) {
					best = ms;
					res.best = c;
				}
				res.candidates++;
			}
			/* second stage: the best shape with a shared-memory short stack */
			const kgr_trace_tune first = res.best;
			for (int k : kTuneStacks) {
				kgr_trace_tune c = first;
				c.stack = k;
				att->tuned_layout = c.layout;
				att->tuned.shadow = (int16_t)c.shadow;
				att->tuned.block = (int16_t)c.block;
				att->tuned.occupancy = (int16_t)c.occupancy;
				att->tuned.stack = (int16_t)k;
				double ms = time_frames([&] { render_frame(att, info, sc, st); }, frames, st);
				res.candidates++;
				if (ms < best) {
					best = ms;
					res.best = c;
				}
			}
			res.best_ms = best;
			att->tuned_layout = res.best.layout;
			att->tuned.shadow = (int16_t)res.best.shadow;
			att->tuned.block = (int16_t)res.best.block;
			att->tuned.occupancy = (int16_t)res.best.occupancy;
			att->tuned.stack = (int16_t)res.best.stack;
		} catch (...) {
			att->tuned_layout = old_layout;
			att->tuned = old_tune;
			for (auto &kv : held)
				att->options[kv.first] = kv.second;
			throw;
		}
		for (auto &kv : held)
			att->options[kv.first] = kv.second;
		if (result)
			*result = res;
	});
}

kgr_status kgr_get_trace_tune(const kgr_attachment *att, kgr_trace_tune *tune)
{
	return guarded([&] {
		KGR_REQUIRE(att && tune, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		TraceTune t = att->trace_tune();
		tune->layout = att->layout();
		tune->shadow = t.shadow;
		tune->block = t.block;
		tune->occupancy = t.occupancy;
		tune->stack = t.stack;
	});
}

kgr_status kgr_get_render_stats(const kgr_attachment *att, kgr_render_stats *stats)
{
	return guarded([&] {
		KGR_REQUIRE(att && stats, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		*stats = att->stats;
		if (att->loaded && att->counters.ptr) {
			DeviceGuard g(att->device);
			uint32_t c[CNT_COUNT];
			KGR_CUDA(cudaMemcpy(c, att->counters.ptr, sizeof(c), cudaMemcpyDeviceToHost));
			stats->bounce_rays = c[CNT_BOUNCE_TOTAL];
			stats->shadow_rays = c[CNT_SHADOW_TOTAL];
		}
	});
}

kgr_status kgr_get_stage_times(kgr_attachment *att, double *ms, uint32_t *launches, uint32_t count)
{
	return guarded([&] {
		KGR_REQUIRE(att && ms && launches, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		DeviceGuard g(att->device);
		att->collect_times();
		for (uint32_t k = 0; k < count; k++) {
			ms[k] = k < STAGE_COUNT ? att->stage_ms[k] : 0.0;
			launches[k] = k < STAGE_COUNT ? att->stage_launches[k] : 0;
		}
		for (int k = 0; k < STAGE_COUNT; k++) {
			att->stage_ms[k] = 0.0;
			att->stage_launches[k] = 0;
		}
	});
}

kgr_status kgr_get_visit_counts(const kgr_attachment *att, uint64_t counts[4])
{
	return guarded([&] {
		KGR_REQUIRE(att && counts, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		memset(counts, 0, 4 * sizeof(uint64_t));
		if (!att->visits.ptr)
			return;
		DeviceGuard g(att->device);
		KGR_CUDA(cudaMemcpy(counts, att->visits.ptr, 4 * sizeof(uint64_t), cudaMemcpyDeviceToHost));
	});
}

kgr_status kgr_measure_read_bandwidth(int32_t device, uint64_t bytes, int32_t iters, double *gbps)
{
	return guarded([&] {
		KGR_REQUIRE(gbps && bytes >= 16 && iters >= 1, KGR_ERR_INVALID_ARGUMENT, "bad argument");
		int dev = resolve_device(device);
		DeviceGuard g(dev);
		size_t n = (size_t)(bytes / 16);
		DevBuf<float4> buf, sink;
		buf.alloc(n);
		sink.alloc(1);
		KGR_CUDA(cudaMemset(buf.ptr, 0, n * sizeof(float4)));
		launch_read_probe(buf.ptr, n, sink.ptr, 1, 0);
		cudaEvent_t a, b;
		KGR_CUDA(cudaEventCreate(&a));
		KGR_CUDA(cudaEventCreate(&b));
		float best = 1e30f;
		for (int rep = 0; rep < 5; rep++) {
			KGR_CUDA(cudaEventRecord(a, 0));
			launch_read_probe(buf.ptr, n, sink.ptr, iters, 0);
			KGR_CUDA(cudaEventRecord(b, 0));
			KGR_CUDA(cudaEventSynchronize(b));
			float ms = 0.0f;
			KGR_CUDA(cudaEventElapsedTime(&ms, a, b));
			best = ms < best ? ms : best;
		}
		cudaEventDestroy(a);
		cudaEventDestroy(b);
		*gbps = (double)n * 16.0 * iters / (best * 1e-3) / 1e9;
	});
}

kgr_status kgr_debug_copy(const kgr_attachment *att, const char *what, void *host, uint64_t bytes)
{
	return guarded([&] {
		KGR_REQUIRE(att && what && host, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		KGR_REQUIRE(att->loaded, KGR_ERR_NOT_LOADED, "not loaded");
		DeviceGuard g(att->device);
		std::string w(what);
		const void *src = nullptr;
		size_t n = 0;
		int prev = att->prev_index;
		if (w == "reservoir_prev_a") { src = att->res_a[prev].ptr; n = att->res_a[prev].bytes(); }
		else if (w == "reservoir_prev_b") { src = att->res_b[prev].ptr; n = att->res_b[prev].bytes(); }
		else if (w == "intermediate") { src = att->intermediate.ptr; n = att->intermediate.bytes(); }
		else if (w == "auxiliary") { src = att->auxiliary.ptr; n = att->auxiliary.bytes(); }
		else if (w == "materials") { src = att->pixel_materials.ptr; n = att->pixel_materials.bytes(); }
		else if (w == "gi_reservoir_a") { src = att->gi_a[att->gi_prev].ptr; n = att->gi_a[att->gi_prev].bytes(); }
		else if (w == "gi_reservoir_b") { src = att->gi_b[att->gi_prev].ptr; n = att->gi_b[att->gi_prev].bytes(); }
		else if (w == "gi_direct") { src = att->g_direct.ptr; n = att->g_direct.bytes(); }
		else if (w.compare(0, 6, "mamba_") == 0 && att->mamba_loaded) {
			if (!mamba_buffer(att->mamba, att->mamba_res_in, att->mamba_prev_in, att->width, att->height,
				    w.c_str() + 6, &src, &n))
				throw Error(KGR_ERR_INVALID_ARGUMENT, "unknown buffer " + w);
		}
		else throw Error(KGR_ERR_INVALID_ARGUMENT, "unknown buffer " + w);
		KGR_REQUIRE(src && bytes <= n, KGR_ERR_INVALID_ARGUMENT, "buffer missing or too small");
		KGR_CUDA(cudaMemcpy(host, src, bytes, cudaMemcpyDeviceToHost));
	});
}

kgr_plugin_ret kgr_load_attachment(const char *kind)
{
	kgr_attachment *a = nullptr;
	if (kgr_create(kind ? kind : "path_tracer", &a) != KGR_OK)
		return {nullptr, nullptr};
	return {a->name.c_str(), a};
}

/* ====================================================== procedural scenes == */

kgr_status kgr_generate_scene(const char *name, uint64_t seed, kgr_generated **out)
{
	return guarded([&] {
		KGR_REQUIRE(name && out, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		std::unique_ptr<kgr_generated> g(new kgr_generated());
		generate_scene(name, seed, g.get());
		*out = g.release();
	});
}

kgr_status kgr_generated_get(const kgr_generated *g, kgr_generated_view *v)
{
	return guarded([&] {
		KGR_REQUIRE(g && v, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		v->positions = g->positions.data();
		v->normals = g->normals.data();
		v->vertex_count = (uint32_t)(g->positions.size() / 3);
		v->indices = g->indices.data();
		v->material_indices = g->material_indices.data();
		v->triangle_count = (uint32_t)(g->indices.size() / 3);
		v->materials = g->materials.data();
		v->material_count = (uint32_t)g->materials.size();
		memcpy(v->camera_eye, g->eye, 12);
		memcpy(v->camera_target, g->target, 12);
		v->camera_fov_deg = g->fov;
	});
}

kgr_status kgr_generated_destroy(kgr_generated *g)
{
	delete g;
	return KGR_OK;
}

/* uvw_frame (include/camera.hpp:45-63), glm::perspective and glm::lookAt
 * (camera.hpp:20-34) with near 0.1 and far 1000. */
kgr_status kgr_camera_setup(const float eye[3], const float target[3], const float up[3], float fov_deg,
		float aspect, kgr_launch_info *info)
{
	return guarded([&] {
		KGR_REQUIRE(eye && target && up && info, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		auto sub = [](const float *a, const float *b, float *o) { for (int k = 0; k < 3; k++) o[k] = a[k] - b[k]; };
		auto crs = [](const float *a, const float *b, float *o) {
			o[0] = a[1] * b[2] - b[1] * a[2];
			o[1] = a[2] * b[0] - b[2] * a[0];
			o[2] = a[0] * b[1] - b[0] * a[1];
		};
		auto dotp = [](const float *a, const float *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
		auto nrm = [&](float *v) { float inv = 1.0f / sqrtf(dotp(v, v)); for (int k = 0; k < 3; k++) v[k] *= inv; };
		float w[3], u[3], v[3];
		sub(target, eye, w);
		float wlen = sqrtf(dotp(w, w));
		crs(w, up, u);
		nrm(u);
		crs(u, w, v);
		nrm(v);
		/* glm::radians(fov) / 2: a float product with the float constant */
		float half = fov_deg * (float)0.01745329251994329576923690768489 / 2.0f;
		float vlen = wlen * tanf(half);
		for (int k = 0; k < 3; k++)
			v[k] *= vlen;
		float ulen = vlen * aspect;
		for (int k = 0; k < 3; k++)
			u[k] *= ulen;
		memcpy(info->camera.center, eye, 12);
		memcpy(info->camera.ax_u, u, 12);
		memcpy(info->camera.ax_v, v, 12);
		memcpy(info->camera.ax_w, w, 12);
		/* glm::perspective (right-handed, depth -1..1) */
		float *P = info->camera.projection;
		memset(P, 0, 64);
		float tan_half = tanf(half);
		P[0] = 1.0f / (aspect * tan_half);
		P[5] = 1.0f / tan_half;
		float zn = 0.1f, zf = 1000.0f;
		P[10] = -(zf + zn) / (zf - zn);
		P[11] = -1.0f;
		P[14] = -(2.0f * zf * zn) / (zf - zn);
		/* glm::lookAt (right-handed) */
		float f[3], s[3], uu[3];
		sub(target, eye, f);
		nrm(f);
		crs(f, up, s);
		nrm(s);
		crs(s, f, uu);
		float *V = info->camera.view;
		memset(V, 0, 64);
		V[0] = s[0]; V[4] = s[1]; V[8] = s[2];
		V[1] = uu[0]; V[5] = uu[1]; V[9] = uu[2];
		V[2] = -f[0]; V[6] = -f[1]; V[10] = -f[2];
		V[12] = -dotp(s, eye);
		V[13] = -dotp(uu, eye);
		V[14] = dotp(f, eye);
		V[15] = 1.0f;
	});
}

} /* extern "C" */

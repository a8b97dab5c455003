/*
 * kgr_internal.h -- internal structures of libkgr shared by the host C++
 * translation units and the CUDA kernels.
 */
#ifndef KGR_INTERNAL_H_
#define KGR_INTERNAL_H_

#include <cuda_runtime.h>
#include <stdint.h>

#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/kgr.h"

namespace kgr {

/* ---------------------------------------------------------------- errors -- */

struct Error : std::runtime_error {
	kgr_status status;
	Error(kgr_status s, const std::string &msg) : std::runtime_error(msg), status(s) {}
};

void set_last_error(const std::string &msg);

#define KGR_CUDA(call)                                                                 \
	do {                                                                           \
		cudaError_t err_ = (call);                                             \
		if (err_ != cudaSuccess)                                               \
			throw ::kgr::Error(err_ == cudaErrorMemoryAllocation ?          \
				KGR_ERR_OUT_OF_MEMORY : KGR_ERR_CUDA,                  \
				std::string(#call) + ": " + cudaGetErrorString(err_)); \
	} while (0)

#define KGR_REQUIRE(cond, status, msg)                                                 \
	do {                                                                           \
		if (!(cond))                                                           \
			throw ::kgr::Error((status), (msg));                            \
	} while (0)

/* Run f and return its status: a thrown Error becomes its code and message
 * (kgr_last_error); the C ABI never lets an exception out. */
template <class F>
inline kgr_status guard_call(F &&f)
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

/* The CUDA ordinal to use: device, or the current one when device < 0
 * (KGR_ERR_NO_DEVICE without a GPU). */
int pick_device_ordinal(int device);

/* Sets the device for the lifetime of the guard and restores the caller's. */
struct DeviceGuard {
	int prev = -1;
	explicit DeviceGuard(int device);
	~DeviceGuard();
};

/* ------------------------------------------------------- device buffers -- */

template <class T>
struct DevBuf {
	T *ptr = nullptr;
	size_t count = 0;
	DevBuf() = default;
	DevBuf(const DevBuf &) = delete;
	DevBuf &operator=(const DevBuf &) = delete;
	~DevBuf() { release(); }
	void release()
	{
		if (ptr)
			cudaFree(ptr);
		ptr = nullptr;
		count = 0;
	}
	void alloc(size_t n)
	{
		if (n == count && ptr)
			return;
		release();
		if (n == 0)
			return;
		KGR_CUDA(cudaMalloc((void **)&ptr, n * sizeof(T)));
		count = n;
	}
	void upload(const T *host, size_t n)
	{
		alloc(n);
		if (n)
			KGR_CUDA(cudaMemcpy(ptr, host, n * sizeof(T), cudaMemcpyHostToDevice));
	}
	void upload(const std::vector<T> &v) { upload(v.data(), v.size()); }
	size_t bytes() const { return count * sizeof(T); }
};

/* ---------------------------------------------------------- BVH layouts -- */

/* Binary tree produced by the host builders.  Leaves hold a contiguous range
 * of the builder's primitive order. */
struct TreeNode {
	float bmin[3], bmax[3];
	int32_t left = -1, right = -1; /* internal: child node indices */
	int32_t first = 0, count = 0;  /* leaf: range in prim_order */
};

struct Tree {
	std::vector<TreeNode> nodes; /* nodes[0] is the root (if any) */
	std::vector<uint32_t> prim_order;
};

/* 64-byte child-pair node of the fast layout: boxes of both children
 * (x/y of left, x/y of right, z of both) and two child references.  A
 * reference >= 0 is an internal node; < 0 is a leaf ~((start << 3) | (n-1))
 * over the leaf-ordered triangle array. */
struct FastNode {
	float4 lxy;  /* l.min.x, l.max.x, l.min.y, l.max.y */
	float4 rxy;  /* r.min.x, r.max.x, r.min.y, r.max.y */
	float4 lrz;  /* l.min.z, l.max.z, r.min.z, r.max.z */
	int4 refs;   /* left ref, right ref, unused, unused */
};

/* 128-byte four-child node of the wide layout: the padded boxes of up to
 * four children in SoA form (component c of each float4 belongs to child
 * c) and their references, encoded as in FastNode; KGR_WIDE_EMPTY marks an
 * unused slot.  The boxes are the fast layout's, bit for bit, so a slab
 * test of a child here is the slab test of the same child there. */
struct WideNode {
	float4 lox, hix, loy, hiy, loz, hiz;
	int4 refs;
	int4 unused;
};
#define KGR_WIDE_EMPTY ((int32_t)0x80000000)

/* 80-byte eight-child node of the compressed wide layout (after Ylitie,
 * Karras and Laine, "Efficient Incoherent Ray Traversal on GPUs Through
 * Compressed Wide BVHs", HPG 2017).  Child boxes are the fast layout's
 * padded boxes quantised to 8 bits a plane on the node's grid p + q * 2^e,
 * rounded outward by at least half a grid step, so culling stays
 * conservative.  Slot j of a node is internal when bit j of imask is set
 * (its node index: first_child + the number of internal slots before j), a
 * leaf when meta[j] != 0 (meta = count << 5 | offset: `count` triangle
 * records from first_tri + offset), empty otherwise.  Children sit in the
 * slots that order them front to back for rays of each octant: a ray whose
 * direction signs form octant o visits slot o first, then o ^ 1, o ^ 2, ...
 * Triangle records are the fast layout's, copied in node order, each with
 * its walk rank (the fast layout's record index) in e1.w for the tie-break
 * of equal distances. */
struct CwNode {
	float4 origin; /* p.x, p.y, p.z, bits(ex | ey << 8 | ez << 16 | imask << 24); 2^(e - 127) */
	uint4 base;    /* first internal child, first triangle record, meta[0..3], meta[4..7] */
	uint4 qa;      /* lo.x[0..7], lo.y[0..7] */
	uint4 qb;      /* lo.z[0..7], hi.x[0..7] */
	uint4 qc;      /* hi.y[0..7], hi.z[0..7] */
};
/* traversal stack entries of the compressed layout (node groups) */
#define KGR_CW_STACK 32

/* Host builders (bvh_build.cpp). */
struct PrimBox {
	float bmin[3], bmax[3];
};

void build_sah(const std::vector<PrimBox> &boxes, int max_leaf, Tree &tree);
/* The same tree built on the GPU (bvh_gpu.cu): same splits, same leaves,
 * same primitive order; node numbering differs. */
void build_sah_gpu(const std::vector<PrimBox> &boxes, int max_leaf, Tree &tree, cudaStream_t st);
void build_kobra(const std::vector<PrimBox> &boxes, Tree &tree);
/* Threaded bvh.cpp layout, leaves as chains of one-primitive records.
 * rec_node (optional) receives, per record, the tree node whose box the
 * record holds, or ~prim for a leaf record (the refit map). */
void serialize_threaded(const Tree &tree, const std::vector<PrimBox> &boxes,
		std::vector<float> &out_vec4, std::vector<int32_t> *rec_node = nullptr);
/* Parse a threaded buffer back into a tree (for caller-supplied buffers);
 * rec_node as above, KGR_REC_UNREACHED for records no walk reaches. */
#define KGR_REC_UNREACHED ((int32_t)0x80000000)
void parse_threaded(const float *vec4, uint32_t count, uint32_t prim_count,
		const std::vector<PrimBox> &boxes, Tree &tree, std::vector<int32_t> *rec_node = nullptr);
/* Fast layout from a tree: nodes + leaf-ordered triangle records
 * {v0.xyz, prim}, {e1}, {e2}.  Boxes are padded outward so that culling is
 * conservative with respect to the exact triangle test. */
void build_fast(const Tree &tree, const std::vector<PrimBox> &boxes,
		const float *positions, const uint32_t *tris4, std::vector<FastNode> &nodes,
		std::vector<float4> &tri_records, std::vector<int2> *kids = nullptr);
/* Wide layout from the same tree: each node gathers up to four children by
 * repeatedly opening its largest-area interior child (left-to-right order
 * kept), leaf references identical to the fast layout's so both share its
 * triangle records.  max_stack: the most stack entries a walk can hold
 * (over every root-to-node path, the sum of children - 1). */
void build_wide(const Tree &tree, std::vector<WideNode> &nodes, uint32_t &max_stack,
		std::vector<int4> *kids = nullptr);
/* Compressed wide layout from the same tree (leaves of at most 4
 * triangles): each node gathers up to eight children by opening its
 * largest-area interior child; `fast_tris` are the fast layout's records.
 * depth: the most nodes on a root-to-leaf path.  Returns false (nothing
 * built) when a leaf holds more than 4 triangles. */
bool build_cw8(const Tree &tree, const std::vector<float4> &fast_tris, std::vector<CwNode> &nodes,
		std::vector<float4> &cw_tris, uint32_t &depth, std::vector<int32_t> *kids = nullptr);

/* ---------------------------------------------------------------- scene -- */

struct DeviceScene {
	const float4 *positions;  /* xyz */
	const float4 *normals;    /* xyz */
	const uint4 *tris;        /* i0, i1, i2, material */
	const float4 *bvh;        /* threaded layout, 3 per node */
	const FastNode *fast_nodes;
	const float4 *fast_tris;  /* 3 per triangle, leaf order */
	const WideNode *wide_nodes;
	const kgr_material *materials;
	const kgr_triangle_light *lights;
	uint32_t triangle_count;
	uint32_t light_count;
	uint32_t bvh_vec4_count;
	uint32_t fast_node_count;
	uint32_t wide_node_count;
	const CwNode *cw_nodes;
	const float4 *cw_tris; /* 3 per triangle, compressed-layout node order */
	uint32_t cw_node_count;
	/* lights of the launch beyond the scene's triangles: quad lights
	 * (sampled only, never traced) and an environment texture */
	const kgr_quad_light *quads;
	uint32_t quad_count;
	int32_t has_env;
	/* the miss program's v: 1 - v in the path tracer
	 * (amadeus_path_tracer.cu:216), v in ReSTIR (amadeus_restir.cu:574) */
	int32_t env_flip_v;
	unsigned long long env; /* cudaTextureObject_t */
};

} /* namespace kgr */

/* Host arrays of a procedural scene (kgr_generate_scene). */
struct kgr_generated {
	std::vector<float> positions, normals;
	std::vector<uint32_t> indices, material_indices;
	std::vector<kgr_material> materials;
	float eye[3], target[3], fov;
};

#define KGR_STACK_DEPTH_HOST 64

namespace kgr {

/* What a refit needs, recorded when the scene is created; the topology of
 * every layout stays fixed, only coordinates change. */
struct RefitPlan {
	/* vertices, in the concatenated order of kgr_scene_create */
	std::vector<float> obj_positions, obj_normals; /* 3 per vertex, as the meshes gave them */
	std::vector<uint32_t> vertex_mesh;
	/* >= 0: the vertex takes the face normal of that triangle (meshes
	 * without normals; the last triangle that names the vertex);
	 * KGR_NORMAL_OWN: the mesh's own normal; KGR_NORMAL_ZERO: zero */
	std::vector<int32_t> normal_src;
	std::vector<float> models;     /* 16 per mesh, column-major (glm::mat4) */
	std::vector<int32_t> has_model; /* per mesh: 0 = vertices taken as given */
	std::vector<uint32_t> light_tri; /* triangle of each light */
	/* tree: node {left, right, first, count}; count > 0 marks a leaf over
	 * prim_order[first, first + count) */
	std::vector<int4> nodes;
	std::vector<uint32_t> prim_order;
	std::vector<uint32_t> level_order; /* node ids, deepest level first */
	std::vector<uint32_t> level_begin; /* level l = level_order[level_begin[l], level_begin[l + 1]) */
	std::vector<int32_t> rec_node;     /* threaded record -> node, ~prim for leaf records */
	std::vector<int2> fast_kids;       /* fast node -> its two child nodes (-1: none) */
	std::vector<int4> wide_kids;       /* wide node -> its child nodes (-1: empty slot) */
	std::vector<int32_t> cw_kids;      /* compressed node -> 8 child tree nodes by slot (-1: empty) */
};
#define KGR_NORMAL_OWN (-1)
#define KGR_NORMAL_ZERO (-2)

/* The plan on the device, uploaded by the first refit. */
struct RefitDevice {
	bool ready = false;
	DevBuf<float4> obj_positions, obj_normals, boxes;
	DevBuf<uint32_t> vertex_mesh, light_tri, prim_order, level_order;
	DevBuf<int32_t> normal_src, has_model, rec_node;
	DevBuf<float> models;
	DevBuf<int4> nodes, wide_kids;
	DevBuf<int32_t> cw_kids;
	DevBuf<int2> fast_kids;
};

} /* namespace kgr */

struct kgr_scene {
	int device = 0;
	std::vector<float> positions, normals; /* 3 per vertex */
	std::vector<uint32_t> tris4;           /* 4 per triangle */
	std::vector<kgr_material> materials;
	std::vector<kgr_triangle_light> lights;
	std::vector<float> bvh;                /* threaded, 4 floats per vec4 */
	uint32_t fast_node_count = 0;
	uint32_t wide_node_count = 0, wide_max_stack = 0;
	uint32_t cw_node_count = 0, cw_depth = 0;
	float bounds_min[3] = {0, 0, 0}, bounds_max[3] = {0, 0, 0};
	double build_ms = 0.0;

	kgr::DevBuf<float4> d_positions, d_normals, d_bvh, d_fast_tris;
	kgr::DevBuf<uint4> d_tris;
	kgr::DevBuf<kgr::FastNode> d_fast_nodes;
	kgr::DevBuf<kgr::WideNode> d_wide_nodes;
	kgr::DevBuf<kgr::CwNode> d_cw_nodes;
	kgr::DevBuf<float4> d_cw_tris;
	kgr::DevBuf<kgr_material> d_materials;
	kgr::DevBuf<kgr_triangle_light> d_lights;

	kgr::RefitPlan plan;
	kgr::RefitDevice refit;
	uint32_t refits = 0;

	kgr::DeviceScene view() const;
	uint64_t device_bytes() const;
};

namespace kgr {

/* A scene whose wide layout was not built (its worst-case walk would not fit
 * the traversal stack) is walked on the fast layout: the same boxes, the
 * same triangle records, the same hits. */
inline int layout_for(int layout, const kgr_scene *sc)
{
	if (layout == KGR_LAYOUT_WIDE && sc && !sc->wide_node_count)
		return KGR_LAYOUT_FAST;
	if (layout == KGR_LAYOUT_CW8 && sc && !sc->cw_node_count)
		return KGR_LAYOUT_FAST;
	return layout;
}

/* Every launch shape the autotuner tries on a scene. */
inline std::vector<kgr_trace_tune> tune_candidates(const kgr_scene *sc)
{
	std::vector<kgr_trace_tune> c;
	for (int layout : {KGR_LAYOUT_FAST, KGR_LAYOUT_WIDE, KGR_LAYOUT_CW8}) {
		if (layout == KGR_LAYOUT_WIDE && !sc->wide_node_count)
			continue;
		if (layout == KGR_LAYOUT_CW8 && !sc->cw_node_count)
			continue;
		for (int shadow : {KGR_TRACE_GRID, KGR_TRACE_PERSISTENT})
			for (int block : {64, 128, 256})
				for (int occ : {0, 1})
					c.push_back(kgr_trace_tune{layout, shadow, block, occ, 0});
	}
	return c;
}

/* Shared-memory stack sizes the autotuner's second stage tries on the best
 * shape of the first. */
static const int kTuneStacks[2] = {8, 16};

/* Time `frames` calls of `frame` on `st` (one untimed call first): ms per
 * call from CUDA events. */
template <class F>
inline double time_frames(F frame, int frames, cudaStream_t st)
{
	frame();
	cudaEvent_t e0, e1;
	KGR_CUDA(cudaEventCreate(&e0));
	KGR_CUDA(cudaEventCreate(&e1));
	double ms = 0.0;
	try {
		KGR_CUDA(cudaEventRecord(e0, st));
		for (int f = 0; f < frames; f++)
			frame();
		KGR_CUDA(cudaEventRecord(e1, st));
		KGR_CUDA(cudaEventSynchronize(e1));
		float t = 0.0f;
		KGR_CUDA(cudaEventElapsedTime(&t, e0, e1));
		ms = (double)t / frames;
	} catch (...) {
		cudaEventDestroy(e0);
		cudaEventDestroy(e1);
		throw;
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	return ms;
}

/* ------------------------------------------------------ kernel launchers -- */

/* Refit (refit.cu).  REFIT_TRANSFORM: every vertex from the object-space
 * vertices and the current models; REFIT_POSITIONS: world-space positions
 * (and normals, if given) from device arrays of 3 floats per vertex.  Then
 * normals of meshes without normals, triangle lights, and every layout's
 * boxes and triangle records, in place, on st. */
enum { REFIT_TRANSFORM = 0, REFIT_POSITIONS = 1 };
void refit_scene(kgr_scene *sc, int mode, const float *positions, const float *normals, cudaStream_t st);

/* Traversal of a ray buffer (8 floats per ray) into hits or occlusion flags. */
void launch_trace_closest(const DeviceScene &s, const float4 *rays, uint32_t n,
		kgr_hit *hits, int layout, cudaStream_t stream);
void launch_trace_any(const DeviceScene &s, const float4 *rays, uint32_t n,
		uint32_t *occluded, int layout, cudaStream_t stream);

/* Per-ray node/triangle visit counts of the fast layout (diagnostics). */
void launch_trace_stats(const DeviceScene &s, const float4 *rays, uint32_t n, int any,
		unsigned long long *counters, cudaStream_t stream);

/* Enqueue on st a copy of a loaded attachment's ray totals of its last
 * frame -- bounce rays, then shadow and visibility rays -- into dst (two
 * uint32 of pinned host memory), as kgr_get_render_stats reads them but
 * without waiting. */
void attachment_ray_totals_async(const kgr_attachment *att, uint32_t *dst, cudaStream_t st);

} /* namespace kgr */

#endif

/*
 * refit.cu -- moving geometry without rebuilding the BVH.
 *
 * The reference animates instances through OptiX: a changed Transform
 * gives the instance's GAS a new matrix in a rebuilt TLAS
 * (include/amadeus/accelerator.cuh:145-230), and the vertices of emissive
 * submeshes are transformed again for the triangle-light buffer
 * (source/amadeus/armada.cu:160-205, Transform::apply of
 * include/transform.hpp:76-79).  This library traces one world-space BVH,
 * so a moved instance is a refit of that BVH: the same tree, new boxes.
 *
 * One refit, all on the caller's stream:
 *   1. vertices: object-space vertex x model (transform_point's expression,
 *      columns summed in order), or world positions copied from the caller;
 *   2. face normals of meshes created without normals (the triangle that
 *      gathered the vertex last, as scene creation does);
 *   3. triangle lights {a, b - a, c - a} of their triangles;
 *   4. tree-node boxes, one launch per tree level from the deepest: a leaf
 *      is the union of its triangles' boxes (min(p1, min(p2, p3)) per axis,
 *      zeros made +0), an inner node the union of its two children.  With
 *      canonical zeros min and max are functions of the set of values, so
 *      every box equals the one the SAH builders compute for the same tree;
 *   5. the layouts, in place: threaded records (leaf records keep the raw
 *      triangle box of Submesh::bvh, include/mesh.hpp:48-78), the padded
 *      child boxes of the fast and wide nodes, and the walk-ordered
 *      triangle records.  Headers, links and references are not touched.
 * Every kernel is a grid-stride loop over independent items; nothing waits.
 */
#include <float.h>

#include "kgr_cw8.h"
#include "kgr_internal.h"
#include "kgr_wavefront.h"

namespace kgr {

namespace {

constexpr int REFIT_BLOCK = 256;

__device__ __forceinline__ float gmin_d(float a, float b) { return b < a ? b : a; }
__device__ __forceinline__ float gmax_d(float a, float b) { return a < b ? b : a; }

/* glm::mat4 * vec4(p, w), columns summed in order (capi.cpp transform_point) */
__device__ __forceinline__ float4 transform(const float *m, float4 p, float w)
{
	float o[3];
	for (int i = 0; i < 3; i++)
		o[i] = m[0 * 4 + i] * p.x + m[1 * 4 + i] * p.y + m[2 * 4 + i] * p.z + m[3 * 4 + i] * w;
	return make_float4(o[0], o[1], o[2], 0.0f);
}

__global__ void transform_vertices_kernel(const float4 *__restrict__ obj_p, const float4 *__restrict__ obj_n,
		const uint32_t *__restrict__ vertex_mesh, const int32_t *__restrict__ normal_src,
		const float *__restrict__ models, const int32_t *__restrict__ has_model, uint32_t nv, float4 *pos,
		float4 *nrm)
{
	for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
		uint32_t m = vertex_mesh[v];
		const bool xf = has_model[m] != 0;
		const float *M = models + 16 * (size_t)m;
		float4 p = obj_p[v];
		pos[v] = xf ? transform(M, p, 1.0f) : make_float4(p.x, p.y, p.z, 0.0f);
		if (normal_src[v] == KGR_NORMAL_OWN) {
			float4 n = obj_n[v];
			nrm[v] = xf ? transform(M, n, 0.0f) : make_float4(n.x, n.y, n.z, 0.0f);
		}
	}
}

__global__ void copy_vertices_kernel(const float *__restrict__ p3, const float *__restrict__ n3,
		const int32_t *__restrict__ normal_src, uint32_t nv, float4 *pos, float4 *nrm)
{
	for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
		size_t i = 3 * (size_t)v;
		pos[v] = make_float4(p3[i], p3[i + 1], p3[i + 2], 0.0f);
		if (n3 && normal_src[v] == KGR_NORMAL_OWN)
			nrm[v] = make_float4(n3[i], n3[i + 1], n3[i + 2], 0.0f);
	}
}

/* the unnormalised face normal e1 x e2 that scene creation gives vertices
 * of meshes without normals */
__global__ void face_normals_kernel(const int32_t *__restrict__ normal_src, const uint4 *__restrict__ tris,
		const float4 *__restrict__ pos, uint32_t nv, float4 *nrm)
{
	for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
		int32_t s = normal_src[v];
		if (s == KGR_NORMAL_OWN)
			continue;
		if (s == KGR_NORMAL_ZERO) {
			nrm[v] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
			continue;
		}
		uint4 t = tris[s];
		float4 a = pos[t.x], b = pos[t.y], c = pos[t.z];
		float e1[3] = {b.x - a.x, b.y - a.y, b.z - a.z};
		float e2[3] = {c.x - a.x, c.y - a.y, c.z - a.z};
		nrm[v] = make_float4(e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
			e1[0] * e2[1] - e1[1] * e2[0], 0.0f);
	}
}

__global__ void lights_kernel(const uint32_t *__restrict__ light_tri, const uint4 *__restrict__ tris,
		const float4 *__restrict__ pos, uint32_t nl, kgr_triangle_light *lights)
{
	for (uint32_t l = blockIdx.x * blockDim.x + threadIdx.x; l < nl; l += gridDim.x * blockDim.x) {
		uint4 t = tris[light_tri[l]];
		float4 a = pos[t.x], b = pos[t.y], c = pos[t.z];
		kgr_triangle_light &L = lights[l];
		L.a[0] = a.x;
		L.a[1] = a.y;
		L.a[2] = a.z;
		L.ab[0] = b.x - a.x;
		L.ab[1] = b.y - a.y;
		L.ab[2] = b.z - a.z;
		L.ac[0] = c.x - a.x;
		L.ac[1] = c.y - a.y;
		L.ac[2] = c.z - a.z;
	}
}

/* Submesh::bvh box of a triangle: min(p1, min(p2, p3)) per axis */
__device__ __forceinline__ void triangle_box(const uint4 *tris, const float4 *pos, uint32_t prim, float *mn,
		float *mx)
{
	uint4 t = tris[prim];
	float4 a = pos[t.x], b = pos[t.y], c = pos[t.z];
	mn[0] = gmin_d(a.x, gmin_d(b.x, c.x));
	mn[1] = gmin_d(a.y, gmin_d(b.y, c.y));
	mn[2] = gmin_d(a.z, gmin_d(b.z, c.z));
	mx[0] = gmax_d(a.x, gmax_d(b.x, c.x));
	mx[1] = gmax_d(a.y, gmax_d(b.y, c.y));
	mx[2] = gmax_d(a.z, gmax_d(b.z, c.z));
}

__global__ void node_boxes_kernel(const uint32_t *__restrict__ ids, uint32_t n, const int4 *__restrict__ nodes,
		const uint32_t *__restrict__ prim_order, const uint4 *__restrict__ tris, const float4 *__restrict__ pos,
		float4 *boxes)
{
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		uint32_t id = ids[i];
		int4 nd = nodes[id];
		float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
		if (nd.w > 0) {
			for (int k = 0; k < nd.w; k++) {
				float tmn[3], tmx[3];
				triangle_box(tris, pos, prim_order[nd.z + k], tmn, tmx);
				for (int a = 0; a < 3; a++) {
					mn[a] = gmin_d(mn[a], tmn[a] + 0.0f); /* +0.0f: -0 -> +0 */
					mx[a] = gmax_d(mx[a], tmx[a] + 0.0f);
				}
			}
		} else {
			float4 l0 = boxes[2 * (size_t)nd.x], l1 = boxes[2 * (size_t)nd.x + 1];
			float4 r0 = boxes[2 * (size_t)nd.y], r1 = boxes[2 * (size_t)nd.y + 1];
			mn[0] = gmin_d(l0.x, r0.x);
			mn[1] = gmin_d(l0.y, r0.y);
			mn[2] = gmin_d(l0.z, r0.z);
			mx[0] = gmax_d(l1.x, r1.x);
			mx[1] = gmax_d(l1.y, r1.y);
			mx[2] = gmax_d(l1.z, r1.z);
		}
		boxes[2 * (size_t)id] = make_float4(mn[0], mn[1], mn[2], 0.0f);
		boxes[2 * (size_t)id + 1] = make_float4(mx[0], mx[1], mx[2], 0.0f);
	}
}

__global__ void threaded_kernel(const int32_t *__restrict__ rec_node, uint32_t nrec, const float4 *__restrict__ boxes,
		const uint4 *__restrict__ tris, const float4 *__restrict__ pos, float4 *bvh)
{
	for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < nrec; r += gridDim.x * blockDim.x) {
		int32_t v = rec_node[r];
		if (v == KGR_REC_UNREACHED)
			continue;
		float mn[3], mx[3];
		if (v < 0) {
			triangle_box(tris, pos, (uint32_t)~v, mn, mx);
		} else {
			float4 b0 = boxes[2 * (size_t)v], b1 = boxes[2 * (size_t)v + 1];
			mn[0] = b0.x, mn[1] = b0.y, mn[2] = b0.z;
			mx[0] = b1.x, mx[1] = b1.y, mx[2] = b1.z;
		}
		float4 lo = bvh[3 * (size_t)r + 1], hi = bvh[3 * (size_t)r + 2];
		bvh[3 * (size_t)r + 1] = make_float4(mn[0], mn[1], mn[2], lo.w);
		bvh[3 * (size_t)r + 2] = make_float4(mx[0], mx[1], mx[2], hi.w);
	}
}

/* pad_box of bvh_build.cpp: outward by 2^-19 relative plus 1e-20 */
__device__ __forceinline__ void padded(const float4 *boxes, int32_t node, float *pmn, float *pmx)
{
	float4 b0 = boxes[2 * (size_t)node], b1 = boxes[2 * (size_t)node + 1];
	const float mn[3] = {b0.x, b0.y, b0.z}, mx[3] = {b1.x, b1.y, b1.z};
	const float rel = 1.0f / (1 << 19);
	for (int k = 0; k < 3; k++) {
		float ext = mx[k] - mn[k];
		pmn[k] = mn[k] - ((fabsf(mn[k]) + ext) * rel + 1e-20f);
		pmx[k] = mx[k] + ((fabsf(mx[k]) + ext) * rel + 1e-20f);
	}
}

__global__ void fast_nodes_kernel(const int2 *__restrict__ kids, uint32_t nf, const float4 *__restrict__ boxes,
		FastNode *nodes)
{
	for (uint32_t f = blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += gridDim.x * blockDim.x) {
		int2 k = kids[f];
		FastNode n = nodes[f];
		float pmn[3], pmx[3];
		if (k.x >= 0) {
			padded(boxes, k.x, pmn, pmx);
			n.lxy = make_float4(pmn[0], pmx[0], pmn[1], pmx[1]);
			n.lrz.x = pmn[2];
			n.lrz.y = pmx[2];
		}
		if (k.y >= 0) {
			padded(boxes, k.y, pmn, pmx);
			n.rxy = make_float4(pmn[0], pmx[0], pmn[1], pmx[1]);
			n.lrz.z = pmn[2];
			n.lrz.w = pmx[2];
		}
		nodes[f] = n;
	}
}

__global__ void wide_nodes_kernel(const int4 *__restrict__ kids, uint32_t nw, const float4 *__restrict__ boxes,
		WideNode *nodes)
{
	for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < nw; w += gridDim.x * blockDim.x) {
		int4 k4 = kids[w];
		const int32_t kid[4] = {k4.x, k4.y, k4.z, k4.w};
		WideNode n = nodes[w];
		float4 *lo[3] = {&n.lox, &n.loy, &n.loz}, *hi[3] = {&n.hix, &n.hiy, &n.hiz};
		for (int s = 0; s < 4; s++) {
			if (kid[s] < 0)
				continue;
			float pmn[3], pmx[3];
			padded(boxes, kid[s], pmn, pmx);
			for (int a = 0; a < 3; a++) {
				(&lo[a]->x)[s] = pmn[a];
				(&hi[a]->x)[s] = pmx[a];
			}
		}
		nodes[w] = n;
	}
}

/* The compressed nodes requantised from their children's refitted boxes by
 * the host builder's own rules (kgr_cw8.h): same slots, same child and
 * triangle bases, new grid and planes. */
__global__ void cw_nodes_kernel(const int32_t *__restrict__ kids, uint32_t nc, const float4 *__restrict__ boxes,
		CwNode *nodes)
{
	for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
		float lo[8][3], hi[8][3];
		uint32_t used = 0;
		for (int j = 0; j < 8; j++) {
			int32_t k = kids[8 * (size_t)c + j];
			for (int a = 0; a < 3; a++) {
				lo[j][a] = 0.0f;
				hi[j][a] = 0.0f;
			}
			if (k < 0)
				continue;
			used |= 1u << j;
			padded(boxes, k, lo[j], hi[j]);
		}
		CwNode n = nodes[c];
		uint32_t imask = __float_as_uint(n.origin.w) >> 24;
		cw_quantize(lo, hi, used, imask, n.origin, n.qa, n.qb, n.qc);
		nodes[c] = n;
	}
}

/* {v0, prim}, {v1 - v0}, {v2 - v0} in walk order; the primitive id stays */
__global__ void triangle_records_kernel(uint32_t nt, const uint4 *__restrict__ tris, const float4 *__restrict__ pos,
		float4 *rec)
{
	for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nt; k += gridDim.x * blockDim.x) {
		float4 r0 = rec[3 * (size_t)k];
		uint4 t = tris[(uint32_t)__float_as_int(r0.w)];
		float4 a = pos[t.x], b = pos[t.y], c = pos[t.z];
		rec[3 * (size_t)k] = make_float4(a.x, a.y, a.z, r0.w);
		rec[3 * (size_t)k + 1] = make_float4(b.x - a.x, b.y - a.y, b.z - a.z, 0.0f);
		rec[3 * (size_t)k + 2] = make_float4(c.x - a.x, c.y - a.y, c.z - a.z, 0.0f);
	}
}

/* the compressed layout's copies of the records: the rank in e1.w stays */
__global__ void cw_triangle_records_kernel(uint32_t nt, const uint4 *__restrict__ tris,
		const float4 *__restrict__ pos, float4 *rec)
{
	for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nt; k += gridDim.x * blockDim.x) {
		float4 r0 = rec[3 * (size_t)k];
		float rank = rec[3 * (size_t)k + 1].w;
		uint4 t = tris[(uint32_t)__float_as_int(r0.w)];
		float4 a = pos[t.x], b = pos[t.y], c = pos[t.z];
		rec[3 * (size_t)k] = make_float4(a.x, a.y, a.z, r0.w);
		rec[3 * (size_t)k + 1] = make_float4(b.x - a.x, b.y - a.y, b.z - a.z, rank);
		rec[3 * (size_t)k + 2] = make_float4(c.x - a.x, c.y - a.y, c.z - a.z, 0.0f);
	}
}

unsigned grid_for(size_t n)
{
	size_t blocks = (n + REFIT_BLOCK - 1) / REFIT_BLOCK;
	size_t cap = (size_t)device_sm_count() * 8;
	return (unsigned)(blocks < cap ? blocks : cap);
}

template <class T>
void upload_vec(DevBuf<T> &d, const std::vector<T> &h)
{
	d.upload(h);
}

void upload_plan(kgr_scene *sc)
{
	RefitPlan &pl = sc->plan;
	RefitDevice &d = sc->refit;
	size_t nv = pl.vertex_mesh.size();
	std::vector<float4> tmp(nv);
	for (size_t v = 0; v < nv; v++)
		tmp[v] = make_float4(pl.obj_positions[3 * v], pl.obj_positions[3 * v + 1], pl.obj_positions[3 * v + 2], 0.0f);
	d.obj_positions.upload(tmp);
	for (size_t v = 0; v < nv; v++)
		tmp[v] = make_float4(pl.obj_normals[3 * v], pl.obj_normals[3 * v + 1], pl.obj_normals[3 * v + 2], 0.0f);
	d.obj_normals.upload(tmp);
	upload_vec(d.vertex_mesh, pl.vertex_mesh);
	upload_vec(d.normal_src, pl.normal_src);
	d.models.alloc(pl.models.size());
	d.has_model.alloc(pl.has_model.size());
	upload_vec(d.light_tri, pl.light_tri);
	upload_vec(d.nodes, pl.nodes);
	upload_vec(d.prim_order, pl.prim_order);
	upload_vec(d.level_order, pl.level_order);
	upload_vec(d.rec_node, pl.rec_node);
	upload_vec(d.fast_kids, pl.fast_kids);
	upload_vec(d.wide_kids, pl.wide_kids);
	upload_vec(d.cw_kids, pl.cw_kids);
	d.boxes.alloc(2 * pl.nodes.size());
	d.ready = true;
}

} /* namespace */

void refit_scene(kgr_scene *sc, int mode, const float *positions, const float *normals, cudaStream_t st)
{
	RefitPlan &pl = sc->plan;
	RefitDevice &d = sc->refit;
	KGR_REQUIRE(pl.vertex_mesh.size() == sc->positions.size() / 3 && pl.rec_node.size() == sc->bvh.size() / 12 &&
			pl.fast_kids.size() == sc->fast_node_count && pl.wide_kids.size() == sc->wide_node_count &&
			pl.cw_kids.size() == 8 * (size_t)sc->cw_node_count,
		KGR_ERR_INTERNAL, "refit plan does not match the scene");
	if (!d.ready)
		upload_plan(sc);
	const uint32_t nv = (uint32_t)(sc->positions.size() / 3);
	const uint32_t nt = (uint32_t)(sc->tris4.size() / 4);
	const uint32_t nl = (uint32_t)sc->lights.size();
	float4 *pos = sc->d_positions.ptr, *nrm = sc->d_normals.ptr;
	const uint4 *tris = sc->d_tris.ptr;
	if (mode == REFIT_TRANSFORM) {
		if (!pl.models.empty()) {
			KGR_CUDA(cudaMemcpyAsync(d.models.ptr, pl.models.data(), pl.models.size() * sizeof(float),
				cudaMemcpyHostToDevice, st));
			KGR_CUDA(cudaMemcpyAsync(d.has_model.ptr, pl.has_model.data(), pl.has_model.size() * sizeof(int32_t),
				cudaMemcpyHostToDevice, st));
		}
		if (nv)
			transform_vertices_kernel<<<grid_for(nv), REFIT_BLOCK, 0, st>>>(d.obj_positions.ptr,
				d.obj_normals.ptr, d.vertex_mesh.ptr, d.normal_src.ptr, d.models.ptr, d.has_model.ptr, nv, pos,
				nrm);
	} else if (nv) {
		copy_vertices_kernel<<<grid_for(nv), REFIT_BLOCK, 0, st>>>(positions, normals, d.normal_src.ptr, nv, pos,
			nrm);
	}
	if (nv)
		face_normals_kernel<<<grid_for(nv), REFIT_BLOCK, 0, st>>>(d.normal_src.ptr, tris, pos, nv, nrm);
	if (nl)
		lights_kernel<<<grid_for(nl), REFIT_BLOCK, 0, st>>>(d.light_tri.ptr, tris, pos, nl, sc->d_lights.ptr);
	for (size_t l = 0; l + 1 < pl.level_begin.size(); l++) {
		uint32_t b = pl.level_begin[l], e = pl.level_begin[l + 1];
		if (e > b)
			node_boxes_kernel<<<grid_for(e - b), REFIT_BLOCK, 0, st>>>(d.level_order.ptr + b, e - b,
				d.nodes.ptr, d.prim_order.ptr, tris, pos, d.boxes.ptr);
	}
	uint32_t nrec = (uint32_t)pl.rec_node.size();
	if (nrec)
		threaded_kernel<<<grid_for(nrec), REFIT_BLOCK, 0, st>>>(d.rec_node.ptr, nrec, d.boxes.ptr, tris, pos,
			sc->d_bvh.ptr);
	if (sc->fast_node_count)
		fast_nodes_kernel<<<grid_for(sc->fast_node_count), REFIT_BLOCK, 0, st>>>(d.fast_kids.ptr,
			sc->fast_node_count, d.boxes.ptr, sc->d_fast_nodes.ptr);
	if (sc->wide_node_count)
		wide_nodes_kernel<<<grid_for(sc->wide_node_count), REFIT_BLOCK, 0, st>>>(d.wide_kids.ptr,
			sc->wide_node_count, d.boxes.ptr, sc->d_wide_nodes.ptr);
	if (sc->cw_node_count)
		cw_nodes_kernel<<<grid_for(sc->cw_node_count), REFIT_BLOCK, 0, st>>>(d.cw_kids.ptr, sc->cw_node_count,
			d.boxes.ptr, sc->d_cw_nodes.ptr);
	if (nt)
		triangle_records_kernel<<<grid_for(nt), REFIT_BLOCK, 0, st>>>(nt, tris, pos, sc->d_fast_tris.ptr);
	if (nt && sc->cw_node_count)
		cw_triangle_records_kernel<<<grid_for(nt), REFIT_BLOCK, 0, st>>>(nt, tris, pos, sc->d_cw_tris.ptr);
	KGR_CUDA(cudaGetLastError());
	sc->refits++;
}

} /* namespace kgr */

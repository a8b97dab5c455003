/*
 * oracle.h -- CPU oracle for the ray-tracing hot path (TEST INFRASTRUCTURE).
 *
 * This library is the checker, not the product: only tests/, the smoke test
 * of __graft_entry__.py and the cpu_baseline / --impl reference legs of
 * bench.py load it.  It restates, function by function, the reference's
 * algorithms (each definition in oracle.cpp cites the reference file:line it
 * follows) in plain C++ compiled with -O2 -ffp-contract=off, so that its
 * float results can be compared bit for bit with the CUDA kernels.
 *
 * Parity pin: the reference has no tests or golden vectors.  The RNG, the
 * triangle test, the area-light sampler and the GGX BRDF are pinned against
 * known-answer vectors produced by compiling the reference's own headers
 * (include/cuda/random.cuh, include/cuda/math.cuh, include/cuda/brdf.cuh,
 * include/optix/lighting.cuh) on the host (oracle/_ref, tests/golden/).  The
 * BVH builder is pinned against source/bvh.cpp compiled on the host with a
 * glm stand-in (oracle/ref_bvh.cpp), and the threaded walk against the
 * traversal shaders (shaders/rt/modules/bvh.glsl and the modules it uses)
 * compiled as C++ (oracle/ref_glsl.cpp).  The path tracer is pinned
 * against the reference's own path-tracer programs
 * (source/optix/amadeus_path_tracer.cu, amadeus_common.cuh) compiled on the
 * host with the OptiX device calls stood in for (oracle/ref_pt.cpp), and
 * ReSTIR DI against source/optix/amadeus_restir.cu compiled the same way
 * (oracle/ref_restir.cpp).
 */
#ifndef KGR_ORACLE_H_
#define KGR_ORACLE_H_

#include <stdint.h>
#include "../include/kgr.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_scene {
	const float *positions;        /* 3 * vertex_count */
	const float *normals;          /* 3 * vertex_count */
	const uint32_t *tris;          /* 4 * triangle_count: i0, i1, i2, material */
	const kgr_material *materials;
	const kgr_triangle_light *lights;
	const float *bvh;              /* threaded bvh.cpp layout */
	uint32_t vertex_count;
	uint32_t triangle_count;
	uint32_t material_count;
	uint32_t light_count;
	uint32_t bvh_vec4_count;
	uint32_t pad;
	/* quad lights and an environment map (NULL / 0 for none): RGBA float
	 * texels, row 0 first, read with normalised coordinates and wrap
	 * addressing, point-sampled or linearly filtered */
	const kgr_quad_light *quads;
	const float *env;
	uint32_t quad_count;
	uint32_t env_width, env_height;
	int32_t env_filter; /* KGR_FILTER_LINEAR or KGR_FILTER_POINT */
} oracle_scene;

typedef struct oracle_trace_stats {
	uint64_t internal_visits; /* 48 B each: header, min, max */
	uint64_t leaf_visits;     /* 16 B header + 64 B triangle (index + 3 positions) */
	uint64_t rays;
} oracle_trace_stats;

/* Reference builder: partition() + serialize() of source/bvh.cpp.
 * boxes: 6 floats per primitive {min xyz, max xyz}.  Returns the number of
 * vec4 written (3 per node) or -1 if capacity is too small. */
int64_t oracle_build_kobra(const float *boxes, uint32_t n, float *out_vec4, uint64_t capacity);

/* Per-triangle AABBs as Submesh::bvh computes them (include/mesh.hpp:48-78). */
void oracle_triangle_boxes(const oracle_scene *s, float *boxes);

/* GLSL trace() (bvh.glsl:52-99) over the threaded layout; rays are 8 floats
 * {o, unused, d, tmax}.  Multithreaded over rays when threads > 1. */
void oracle_trace_closest(const oracle_scene *s, const float *rays, uint32_t n,
		kgr_hit *hits, oracle_trace_stats *stats, int threads);
void oracle_trace_any(const oracle_scene *s, const float *rays, uint32_t n,
		uint32_t *occluded, oracle_trace_stats *stats, int threads);

/* Brute force closest hit over all triangles: same triangle test, ties to
 * the lower rank (position in the threaded walk), for cross-checking. */
void oracle_trace_closest_brute(const oracle_scene *s, const float *rays, uint32_t n, kgr_hit *hits);

typedef struct oracle_render_params {
	uint32_t width, height;
	float center[3], ax_u[3], ax_v[3], ax_w[3];
	float projection[16], view[16];
	float prev_projection[16], prev_view[16];
	int32_t max_depth;
	int32_t spp;
	int32_t samples;        /* previously accumulated samples (count) */
	int32_t accumulate;
	uint32_t frame;
	int32_t russian_roulette;
	int32_t rr_start_depth;
	int32_t candidates;     /* ReSTIR RIS candidates (32) */
	int32_t temporal;       /* run the temporal pass */
	int32_t temporal_mcap;  /* 200 in the reference */
	int32_t spatial_passes; /* 2 in the reference */
	int32_t spatial_neighbors; /* 5 */
	int32_t spatial_radius;    /* 30 */
	uint32_t row_begin, row_end; /* PT only: rows to render (crop) */
	int32_t threads;
} oracle_render_params;

typedef struct oracle_render_stats {
	uint64_t camera_rays, bounce_rays, shadow_rays;
} oracle_render_stats;

/* Path tracer: amadeus_path_tracer.cu + naive_path_tracer.cu Russian
 * roulette.  Buffers are float4 width*height (color, normal, albedo,
 * position); only rows [row_begin, row_end) are written. */
void oracle_render_pt(const oracle_scene *s, const oracle_render_params *p,
		float *color, float *normal, float *albedo, float *position,
		oracle_render_stats *stats);

/* Same path tracer with double-precision accumulation of the per-pixel
 * sample mean (the "FP64 oracle" image): out is 3 doubles per pixel. */
void oracle_render_pt_f64(const oracle_scene *s, const oracle_render_params *p,
		double *out_rgb, oracle_render_stats *stats);

/* ReSTIR DI state, all width*height: reservoirs in the 32-byte SoA layout
 * (light index, point xyz, w, W, M), the per-pixel material, the indirect
 * "intermediate" colour and the auxiliary seed. */
typedef struct oracle_restir_state {
	int32_t *cur_light; float *cur_point; float *cur_w; float *cur_W; int32_t *cur_M;
	int32_t *prev_light; float *prev_point; float *prev_w; float *prev_W; int32_t *prev_M;
	kgr_material *materials;
	float *intermediate; /* float4 */
	float *auxiliary;    /* float4 */
	/* v of environment samples (light < -1 holds the bits of -u) */
	float *cur_env_v; float *prev_env_v;
} oracle_restir_state;

/* One ReSTIR DI frame: initial (amadeus_restir.cu:82-144,437-559), temporal
 * (:213-291), spatial passes (:294-434) and the buffer swaps of
 * include/amadeus/restir.cuh:258-303.  After the call prev_* holds the
 * reservoirs the next frame's temporal pass reuses. */
void oracle_render_restir(const oracle_scene *s, const oracle_render_params *p,
		oracle_restir_state *st, float *color, float *normal, float *albedo,
		float *position, oracle_render_stats *stats);

/* ReSTIR GI (no working reference; the project's specification restated):
 * state carried between frames -- last frame's GI reservoirs in the 32-byte
 * two-array layout ({x_s, bits(n_s oct | M)}, {L_o, W}) and its G-buffer --
 * plus the previous camera. */
typedef struct oracle_gi_state {
	float *res_a;         /* float4 per pixel */
	float *res_b;         /* float4 per pixel */
	float *prev_position; /* float4 per pixel, w = 1 on a hit */
	float *prev_normal;   /* float4 per pixel */
	float prev_center[3];
	int32_t gi_temporal, gi_mcap, gi_spatial_iterations, gi_neighbors, gi_radius;
	int32_t gi_confidence_rule; /* a neighbour's confidence is at most the centre's M */
} oracle_gi_state;

/* One ReSTIR GI frame (DI candidates + GI reservoir reuse), see gi.cu's
 * header for the algorithm.  color accumulates with p->accumulate; the
 * state is updated for the next frame.  direct (float4 per pixel, may be
 * NULL) receives the DI term. */
void oracle_render_gi(const oracle_scene *s, const oracle_render_params *p, oracle_gi_state *st,
		float *color, float *direct, oracle_render_stats *stats);

/* The editor's Mamba frame (editor/mamba.cu:941-1312), in the GPU build's
 * deterministic form: a G-buffer traced at pixel centres, ReSTIR DI with 8
 * candidates (when direct_lighting), quarter-resolution secondary rays,
 * irradiance probes (splat, Sobel, raster, collapse, allocation in block
 * order) and the final gather.  The state lives in the oracle_mamba, in the
 * GPU build's layouts; oracle_mamba_buffer copies a named buffer (the names
 * of the product's "mamba_" debug buffers without the prefix) and returns
 * its size in bytes, or -1 for an unknown name or a short out. */
typedef struct oracle_mamba oracle_mamba;
typedef struct oracle_mamba_params {
	uint32_t width, height;
	float center[3], ax_u[3], ax_v[3], ax_w[3];
	float prev_projection[16], prev_view[16];
	float time;
	int32_t samples;
	int32_t direct_lighting, indirect_lighting, irradiance, render_probes, render_probe_radiance;
	int32_t temporal_reuse, spatial_reuse;
	int32_t threads;
} oracle_mamba_params;
oracle_mamba *oracle_mamba_create(uint32_t width, uint32_t height, int32_t max_probes, int32_t max_luts);
void oracle_mamba_destroy(oracle_mamba *m);
void oracle_mamba_frame(oracle_mamba *m, const oracle_scene *s, const oracle_mamba_params *p, float *color,
		oracle_render_stats *stats);
int64_t oracle_mamba_buffer(const oracle_mamba *m, const char *name, void *out, uint64_t bytes);

/* The environment map's texture read (normalised coordinates, wrap
 * addressing) at n (u, v) pairs: rgb gets 3 floats per pair. */
void oracle_env_lookup(const float *texels, uint32_t width, uint32_t height, int filter, const float *uv,
		uint32_t n, float *rgb);

/* Known-answer helpers exposed for the golden-vector tests. */
void oracle_kat_rng(float seed_x, float seed_y, float seed_z, int draws, float *out);
float oracle_kat_intersect(const float *v1, const float *v2, const float *v3,
		const float *o, const float *d, float *b1b2);
void oracle_kat_sample_light(const kgr_triangle_light *l, const float *seed, float *point, float *area_normal);
void oracle_kat_brdf_eval(const kgr_material *m, const float *n, const float *wo,
		const float *seed_in, float *f_wi_pdf_seed);
void oracle_kat_brdf(const kgr_material *m, const float *n, const float *wo, const float *wi, float *f_pdf);
void oracle_kat_math(const float *x, int n, float *sin_cos_tan_atan_acos);
void oracle_kat_atan2_asin(const float *y, const float *x, int n, float *atan2_asin);

/* hdr_to_ldr of include/cuda/color.cuh:84-103: mode 0 ACES, 1 sRGB; ldr rows
 * bottom to top, packed as to_ui32 (cast.cuh:16-20). */
void oracle_tonemap(const float *hdr, uint32_t *ldr, uint32_t width, uint32_t height, int mode);

/* ---- scene inputs of the CPU reference arm (scene_ref.cpp) ---- */

/* Seeded procedural scene: "box4k", "box64", "terrain", "terrain_s",
 * "terrain_m", "terrain_l".  Returns 0, or -1 for an unknown name. */
typedef struct oracle_generated oracle_generated;
typedef struct oracle_scene_arrays {
	const float *positions;          /* 3 * vertex_count */
	const float *normals;            /* 3 * vertex_count */
	const uint32_t *indices;         /* 3 * triangle_count */
	const uint32_t *material_indices; /* triangle_count */
	const kgr_material *materials;
	uint32_t vertex_count, triangle_count, material_count;
	float eye[3], target[3], fov_deg;
} oracle_scene_arrays;
int oracle_generate_scene(const char *name, uint64_t seed, oracle_generated **out);
void oracle_generated_view(const oracle_generated *g, oracle_scene_arrays *view);
void oracle_generated_destroy(oracle_generated *g);

/* Binned-SAH BVH with leaves of at most max_leaf triangles, in the threaded
 * bvh.cpp layout (one record per leaf triangle).  With out_vec4 = NULL it
 * returns the vec4 count; else -1 if capacity is too small. */
int64_t oracle_build_sah(const float *positions, const uint32_t *indices, uint32_t triangle_count, int max_leaf,
		float *out_vec4, uint64_t capacity);

/* Triangle lights of the emissive triangles in triangle order; returns the
 * count (out may be NULL to count). */
uint32_t oracle_scene_lights(const float *positions, const uint32_t *indices, const uint32_t *material_indices,
		uint32_t triangle_count, const kgr_material *materials, kgr_triangle_light *out);

/* Pinhole camera frame of uvw_frame (include/camera.hpp:45-63). */
void oracle_camera(const float eye[3], const float target[3], const float up[3], float fov_deg, float aspect,
		float center[3], float ax_u[3], float ax_v[3], float ax_w[3]);

#ifdef __cplusplus
}
#endif

#endif

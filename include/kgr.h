/*
 * kgr.h -- C ABI of the GB300-native ray-tracing hot path for Kobra.
 *
 * This header is the drop-in boundary.  It replaces, for the path-tracer and
 * ReSTIR attachments, the C++ surface of the reference's Armada plugin layer:
 *
 *   class AttachmentRTX          include/amadeus/armada.cuh:107-139
 *   struct ArmadaLaunchInfo      include/amadeus/armada.cuh:43-83
 *   extern "C" load_attachment   source/amadeus/naive_path_tracer.cu:280-348
 *   Accelerator GAS/IAS build    include/amadeus/accelerator.cuh:46-277
 *   software BVH build/layout    source/bvh.cpp:102-260
 *   GLSL trace()/any-hit         shaders/rt/modules/bvh.glsl:52-127,
 *                                source/optix/amadeus_common.cuh:190-212
 *
 * Conventions.  Every function returns a kgr_status and never throws across
 * the ABI (the reference throws from CUDA_CHECK/OPTIX_CHECK,
 * include/cuda/error.cuh:40-123).  The message of the last failure on the
 * calling thread is returned by kgr_last_error().  Pointers documented as
 * "device" are CUDA device pointers on the device the object was created on;
 * streams are cudaStream_t passed as void* (NULL = the legacy default stream,
 * which is what the reference launches on).  No function allocates on the
 * caller's behalf except the *_create functions, which own what they
 * allocate until the matching *_destroy.
 */
#ifndef KGR_H_
#define KGR_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KGR_ABI_VERSION 5

typedef enum kgr_status {
	KGR_OK = 0,
	KGR_ERR_INVALID_ARGUMENT = 1,
	KGR_ERR_OUT_OF_MEMORY = 2,
	KGR_ERR_CUDA = 3,
	KGR_ERR_UNSUPPORTED = 4,
	KGR_ERR_NOT_ATTACHED = 5,
	KGR_ERR_NOT_LOADED = 6,
	KGR_ERR_BVH_FORMAT = 7,
	KGR_ERR_BUDGET = 8,
	KGR_ERR_TIMEOUT = 9,
	KGR_ERR_UNKNOWN_OPTION = 10,
	KGR_ERR_TYPE = 11,
	KGR_ERR_INTERNAL = 12,
	KGR_ERR_NO_DEVICE = 13
} kgr_status;

/* Human-readable name of a status, and the last error message on this thread. */
const char *kgr_status_string(kgr_status status);
const char *kgr_last_error(void);
int kgr_abi_version(void);

/* ------------------------------------------------------------------ data -- */

/* Shading flags, same values as the reference's `enum Shading`
 * (include/types.hpp:17-25). */
enum {
	KGR_SHADING_NONE = 0,
	KGR_SHADING_REFLECTION = 1 << 0,
	KGR_SHADING_TRANSMISSION = 1 << 1,
	KGR_SHADING_DIFFUSE = 1 << 2,
	KGR_SHADING_GLOSSY = 1 << 3,
	KGR_SHADING_SPECULAR = 1 << 4,
	KGR_SHADING_EMISSIVE = 1 << 5
};

/* Material, field for field the reference's cuda::Material
 * (include/cuda/material.cuh:13-23) without the unused light_index; the
 * texture slots of cuda::_material (:26-49) are not supported. 64 bytes. */
typedef struct kgr_material {
	float diffuse[3];
	float specular[3];
	float emission[3];
	float ambient[3];
	float shininess;
	float roughness;
	float refraction;
	int32_t type;
} kgr_material;

/* Triangle area light {a, ab, ac, intensity}: optix::TriangleLight
 * (include/optix/lighting.cuh:96-120).  48 bytes. */
typedef struct kgr_triangle_light {
	float a[3];
	float ab[3];
	float ac[3];
	float intensity[3];
} kgr_triangle_light;

/* Quad area light {a, ab, ac, intensity}: optix::QuadLight
 * (include/optix/lighting.cuh:57-94), the parallelogram a + u ab + v ac for
 * u, v in [0, 1].  Quads are lights only: they are sampled by next-event
 * estimation and are not part of the traced geometry.  48 bytes. */
typedef struct kgr_quad_light {
	float a[3];
	float ab[3];
	float ac[3];
	float intensity[3];
} kgr_quad_light;

/* One mesh of a scene.  Positions and normals are xyz triples; normals may be
 * NULL (the face normal is used).  `model` is an optional column-major 4x4
 * world transform (glm layout, the Hit::model of include/optix/sbt.cuh:14-21);
 * NULL means identity.  Triangles index this mesh's vertices. */
typedef struct kgr_mesh {
	const float *positions;
	const float *normals;
	uint32_t vertex_count;
	const uint32_t *indices;
	const uint32_t *material_indices; /* one per triangle, or NULL = 0 */
	uint32_t triangle_count;
	const float *model;
} kgr_mesh;

/* BVH builders. */
enum {
	/* binned SAH (32 bins) with leaves of at most max_leaf_size triangles,
	 * written as chains of one-triangle leaf records in the bvh.cpp layout;
	 * kgr_scene_create runs it on the GPU */
	KGR_BUILDER_SAH = 0,
	/* the reference builder: partition() of source/bvh.cpp:102-210 (SAH over
	 * 10 bins of the largest primitive's extent, one triangle per leaf) */
	KGR_BUILDER_KOBRA = 1,
	/* KGR_BUILDER_SAH on the host: the same tree, bit for bit */
	KGR_BUILDER_SAH_HOST = 2
};

typedef struct kgr_scene_options {
	int32_t builder;       /* KGR_BUILDER_* */
	int32_t max_leaf_size; /* SAH builder only, 1..8; 0 = 4 */
	int32_t device;        /* CUDA ordinal; -1 = current device */
	int32_t reserved;
} kgr_scene_options;

typedef struct kgr_scene kgr_scene;

typedef struct kgr_scene_info {
	uint32_t vertex_count;
	uint32_t triangle_count;
	uint32_t light_count;
	uint32_t material_count;
	uint32_t bvh_vec4_count;  /* threaded bvh.cpp layout, 3 vec4 per node */
	uint32_t fast_node_count; /* 64-byte child-pair nodes */
	uint64_t device_bytes;
	double build_ms;
	float bounds_min[3];
	float bounds_max[3];
	uint32_t wide_node_count; /* 128-byte four-child nodes; 0 when the wide layout is not built */
	uint32_t wide_max_stack;  /* most traversal stack entries a walk of the wide layout can hold */
	uint32_t cw8_node_count;  /* 80-byte eight-child nodes; 0 when the compressed layout is not built */
	uint32_t cw8_depth;       /* most compressed nodes on a root-to-leaf path */
} kgr_scene_info;

/* Build the BVH on the host and upload the scene to the device.  Emissive
 * triangles (any emission component > 0) become triangle lights in triangle
 * order, as ArmadaRTX::update_triangle_light_buffers does
 * (source/amadeus/armada.cu:98-212).  Triangle i of the concatenated mesh
 * list has primitive id i. */
kgr_status kgr_scene_create(const kgr_mesh *meshes, uint32_t mesh_count,
		const kgr_material *materials, uint32_t material_count,
		const kgr_scene_options *options, kgr_scene **out);

/* Same, but with a caller-serialised BVH in the bvh.cpp layout
 * (source/bvh.cpp:213-260: 3 vec4 per node, header {leaf ? 1.0f : 0.0f,
 * bits(object), bits(hit), bits(miss)}, then bbox min, then bbox max; links
 * count vec4 units).  Leaf objects are primitive ids of the concatenated
 * triangle list.  Both layouts on the device are derived from it. */
kgr_status kgr_scene_create_from_bvh(const kgr_mesh *meshes, uint32_t mesh_count,
		const kgr_material *materials, uint32_t material_count,
		const float *bvh_vec4, uint32_t bvh_vec4_count,
		int32_t device, kgr_scene **out);

kgr_status kgr_scene_info_get(const kgr_scene *scene, kgr_scene_info *info);

/* Host-only BVH build (no device needed): the threaded bvh.cpp-layout
 * buffer kgr_scene_create would build for one mesh.  Call with out_vec4 =
 * NULL to learn the size. */
kgr_status kgr_bvh_build_host(const float *positions, uint32_t vertex_count,
		const uint32_t *indices, uint32_t triangle_count, int32_t builder,
		int32_t max_leaf_size, float *out_vec4, uint32_t capacity, uint32_t *count);

/* Host copy of the threaded bvh.cpp-layout buffer (capacity in vec4 units). */
kgr_status kgr_scene_copy_bvh(const kgr_scene *scene, float *out_vec4,
		uint32_t capacity, uint32_t *count);

/* Host copy of the triangle lights. */
kgr_status kgr_scene_copy_lights(const kgr_scene *scene, kgr_triangle_light *out,
		uint32_t capacity, uint32_t *count);

/* Host copy of the current vertices (3 floats per vertex, concatenated
 * mesh order); either pointer may be NULL. */
kgr_status kgr_scene_copy_vertices(const kgr_scene *scene, float *positions, float *normals);

/* Raw bytes of one device array of the scene (diagnostics and tests). */
enum {
	KGR_ARRAY_THREADED = 0,         /* float4 x 3 per record, bvh.cpp layout */
	KGR_ARRAY_FAST_NODES = 1,       /* 64-byte child-pair nodes */
	KGR_ARRAY_WIDE_NODES = 2,       /* 128-byte four-child nodes */
	KGR_ARRAY_TRIANGLE_RECORDS = 3, /* float4 x 3 per triangle in walk order: {v0, prim}, e1, e2 */
	KGR_ARRAY_CW8_NODES = 4,        /* 80-byte compressed eight-child nodes */
	KGR_ARRAY_CW8_TRIANGLES = 5     /* float4 x 3 per triangle in compressed-node order: {v0, prim}, {e1, rank}, e2 */
};
kgr_status kgr_scene_copy_array(const kgr_scene *scene, int32_t which, void *out,
		uint64_t capacity_bytes, uint64_t *bytes);

/* Animated instances.  The reference moves an instance by giving its GAS a
 * new transform in the TLAS (include/amadeus/accelerator.cuh:145-230) and
 * re-applies Transform::matrix() to the vertices of emissive submeshes for
 * the light buffer (source/amadeus/armada.cu:160-205).  Here the scene is
 * one world-space BVH, so a transform change is a refit: set the model
 * matrix of `count` meshes (16 floats each, column-major like glm::mat4 and
 * kgr_mesh.model; meshes are numbered in kgr_scene_create order), recompute
 * every vertex, normal and triangle light on the device from the meshes'
 * object-space data, then recompute the boxes of every BVH layout and the
 * triangle records in place.  The topology is kept: traversal stays exact,
 * but a tree refitted far from its build shape walks more nodes (create the
 * scene again to rebuild it).  Each box equals what the builder would
 * compute over the same tree from the new vertices.  Asynchronous on
 * `stream`; order refits and renders of one scene on one stream (or with
 * events).  A captured CUDA graph of a frame stays valid: arrays are
 * updated in place.  bounds_min/max of kgr_scene_info keep their values
 * from creation (the radiance cache's input frame). */
kgr_status kgr_scene_set_transforms(kgr_scene *scene, const uint32_t *mesh_ids,
		const float *models, uint32_t count, void *stream);

/* Deformed geometry: new world-space positions for every vertex (DEVICE
 * array, 3 floats per vertex in kgr_scene_create order) and, optionally,
 * normals (NULL keeps the current normals, except that meshes created
 * without normals get their face normals recomputed).  Then the same refit
 * as kgr_scene_set_transforms.  A later kgr_scene_set_transforms starts
 * again from the object-space vertices. */
kgr_status kgr_scene_refit(kgr_scene *scene, const float *positions, const float *normals, void *stream);

kgr_status kgr_scene_destroy(kgr_scene *scene);

/* ------------------------------------------------------------- traversal -- */

/* Hit record: primitive id (-1 = miss), distance and the barycentrics
 * (b1, b2) of the Moller-Trumbore test of include/optix/lighting.cuh:34-55. */
typedef struct kgr_hit {
	int32_t prim;
	float t;
	float b1;
	float b2;
} kgr_hit;

/* Which device layout a traversal walks. */
enum {
	/* child-pair BVH2 with ordered descent and a short stack (default) */
	KGR_LAYOUT_FAST = 0,
	/* the threaded bvh.cpp layout, walked exactly as bvh.glsl:52-99 does */
	KGR_LAYOUT_THREADED = 1,
	/* four-child BVH4 over the same padded boxes and triangle records as the
	 * fast layout: half the dependent node fetches per ray; built when the
	 * walk's worst-case stack fits the traversal stack */
	KGR_LAYOUT_WIDE = 2,
	/* eight-child BVH8 with child boxes quantised to 8 bits a plane (80-byte
	 * nodes, outward rounding) over the same padded boxes and triangles:
	 * a third of the fast layout's dependent node fetches; built when the
	 * leaves hold at most 4 triangles, requantised in place by a refit */
	KGR_LAYOUT_CW8 = 3
};

/* Closest hit for n rays.  `rays` (device) holds 8 floats per ray:
 * {ox, oy, oz, unused, dx, dy, dz, tmax}; a primitive is accepted when
 * 0 < t < best with best starting at tmax (pass INFINITY for the GLSL
 * trace(), 1e16 for the OptiX launches of amadeus_common.cuh:467-478).
 * Equal distances resolve to the primitive the threaded walk meets first.
 * `hits` (device) receives n records.  Asynchronous on `stream`. */
kgr_status kgr_trace_closest(const kgr_scene *scene, const float *rays,
		uint32_t n, kgr_hit *hits, int32_t layout, void *stream);

/* Any hit: occluded[i] = 1 if some primitive has 0 < t < tmax, else 0
 * (is_occluded, source/optix/amadeus_common.cuh:190-212). */
kgr_status kgr_trace_any(const kgr_scene *scene, const float *rays,
		uint32_t n, uint32_t *occluded, int32_t layout, void *stream);

/* Same two calls on HOST buffers: the rays are copied in, the results out,
 * synchronously.  For callers that hold no device memory. */
kgr_status kgr_trace_closest_host(const kgr_scene *scene, const float *rays,
		uint32_t n, kgr_hit *hits, int32_t layout);
kgr_status kgr_trace_any_host(const kgr_scene *scene, const float *rays,
		uint32_t n, uint32_t *occluded, int32_t layout);

/* Visit counts for n device rays (synchronous, diagnostics and roofline
 * accounting): counts[0..1] = internal nodes and triangles visited on the
 * fast layout, counts[2..3] = the same on the threaded layout. */
kgr_status kgr_trace_counts(const kgr_scene *scene, const float *rays, uint32_t n,
		int32_t any, uint64_t counts[4]);

/* ----------------------------------------------------------- attachments -- */

typedef struct kgr_attachment kgr_attachment;

/* Option values: std::variant<int, float, bool, std::string> of
 * AttachmentRTX::OptionValue (armada.cuh:120). */
enum { KGR_VALUE_NONE = 0, KGR_VALUE_INT = 1, KGR_VALUE_FLOAT = 2, KGR_VALUE_BOOL = 3, KGR_VALUE_STRING = 4 };

typedef struct kgr_value {
	int32_t tag;
	int32_t i;
	float f;
	int32_t b;
	const char *s; /* borrowed for set_option; owned by the attachment for get_option */
} kgr_value;

/* What attach() learns from ArmadaRTX: extent() and the device. */
typedef struct kgr_context {
	uint32_t width;
	uint32_t height;
	int32_t device;
	int32_t reserved;
} kgr_context;

/* ArmadaLaunchInfo (armada.cuh:43-83) with POD types: glm::vec2/vec3 become
 * float[2]/float[3], glm::mat4 becomes float[16] column-major.  Buffers are
 * device float4 arrays of width * height owned by the caller. */
typedef struct kgr_launch_info {
	float resolution[2];
	struct {
		float center[3];
		float ax_u[3];
		float ax_v[3];
		float ax_w[3];
		float projection[16];
		float view[16];
	} camera;
	struct {
		const kgr_quad_light *quad_lights;     /* device; may be NULL when quad_count = 0 */
		const kgr_triangle_light *tri_lights; /* device; NULL = the scene's */
		int32_t quad_count;
		int32_t tri_count;
	} lights;
	struct {
		float *color;
		float *normal;
		float *albedo;
		float *position;
	} buffers;
	const kgr_material *materials; /* device; NULL = the scene's */
	/* cudaTextureObject_t of an RGBA float environment map (normalised
	 * coordinates), e.g. from kgr_environment_create; read when
	 * has_environment_map is set.  The "path_tracer" and "restir_di"
	 * attachments light with it; the other consumers refuse it. */
	uint64_t environment_map;
	int32_t has_environment_map;
	int32_t accumulate;
	float time;
	int32_t max_depth;
	int32_t samples;
	uint32_t frame; /* RNG stream index of this frame */
} kgr_launch_info;

/* Environment maps.  ArmadaRTX::set_envmap (source/amadeus/armada.cu:86-96)
 * loads an image and imports it as a CUDA texture object with normalised
 * coordinates and linear filtering (include/cuda/interop.cuh:96-135).  This
 * makes the same kind of texture from host RGBA float texels (row 0 first,
 * width * height * 4 floats): wrap addressing, KGR_FILTER_LINEAR as the
 * reference does or KGR_FILTER_POINT.  The handle is what
 * kgr_launch_info.environment_map takes. */
enum { KGR_FILTER_LINEAR = 0, KGR_FILTER_POINT = 1 };
typedef struct kgr_environment kgr_environment;
kgr_status kgr_environment_create(const float *rgba, uint32_t width, uint32_t height, int32_t filter,
		int32_t device, kgr_environment **out);
kgr_status kgr_environment_texture(const kgr_environment *env, uint64_t *texture);
/* tex2D<float4> of the texture at n (u, v) pairs (device arrays, 2 and 4
 * floats per entry): what the kernels read for those coordinates. */
kgr_status kgr_environment_sample(const kgr_environment *env, const float *uv, uint32_t n, float *rgba,
		void *stream);
kgr_status kgr_environment_destroy(kgr_environment *env);

/* kind: "path_tracer", "restir_di", "restir_gi" or "mamba" (the editor's
 * default GI mode, editor/mamba.cu:941-1312: ReSTIR DI with 8 candidates,
 * quarter-resolution secondary rays and irradiance probes; it lights with
 * the scene's triangles and the environment map, and refuses quad lights). */
kgr_status kgr_create(const char *kind, kgr_attachment **out);
kgr_status kgr_attach(kgr_attachment *att, const kgr_context *ctx);
kgr_status kgr_load(kgr_attachment *att);
kgr_status kgr_unload(kgr_attachment *att);
kgr_status kgr_set_option(kgr_attachment *att, const char *name, const kgr_value *value);
kgr_status kgr_get_option(const kgr_attachment *att, const char *name, kgr_value *value);
kgr_status kgr_render(kgr_attachment *att, const kgr_launch_info *info,
		const kgr_scene *scene, void *stream);
kgr_status kgr_destroy(kgr_attachment *att);

/* One path-traced frame that allocates no device memory.  No counterpart in
 * the reference: it exists for callers that cannot call cudaMalloc when they
 * render: a host that fixes its device memory at start-up and hands it out
 * itself, where an allocation inside the plugin would break the host's
 * accounting or fail.  The same kernels
 * as the "path_tracer" attachment (fast layout) write one frame into the
 * caller's buffers of info->buffers; the per-path scratch is a fixed array of
 * about 12.8 MiB inside the library, so width * height * spp must be at most
 * 65536, and each resolution component a whole number in [1, 65536]
 * (KGR_ERR_INVALID_ARGUMENT otherwise, before anything runs).  All calls on a device share
 * that array: calls that overlap on the GPU race, so order them on one
 * stream.  The first call on a device looks up the array's address
 * (cudaGetSymbolAddress); make it before any stream capture. */
kgr_status kgr_render_pt_noalloc(const kgr_scene *scene, const kgr_launch_info *info,
		int32_t spp, int32_t russian_roulette, int32_t rr_start_depth, void *stream);

/* Counters of the last render: rays traced by kind and kernel launches. */
typedef struct kgr_render_stats {
	uint64_t camera_rays;
	uint64_t bounce_rays;
	uint64_t shadow_rays;
	uint32_t kernel_launches;
	uint32_t reserved;
} kgr_render_stats;
kgr_status kgr_get_render_stats(const kgr_attachment *att, kgr_render_stats *stats);

/* Per-stage device time of the frames rendered since the last call, when
 * the "profile" option is on: a CUDA event is recorded on the render stream
 * after every launch, and the time between consecutive events is charged to
 * the stage that launched.  Stages: 0 generate, 1 closest-hit traversal,
 * 2 shade, 3 shadow rays (any-hit traversal + resolve), 4 accumulate,
 * 5 ReSTIR RIS, 6 temporal resampling (gather and merge kernels),
 * 7 spatial resampling (gather, resample and finish kernels), 8 ReSTIR
 * finalise, 9 radiance-cache inference, 10 radiance-cache training,
 * 11 temporal-reuse visibility rays, 12 spatial-reuse visibility rays,
 * and for the "mamba" attachment 13 secondary rays, 14 probe splat,
 * 15 probe upkeep (Sobel, raster, collapse, allocation), 16 final gather
 * (its G-buffer is charged to 0 and 1, its direct lighting to 5-7).
 * Synchronises on the last event, then resets the totals. */
kgr_status kgr_get_stage_times(kgr_attachment *att, double *ms, uint32_t *launches, uint32_t count);

/* ------------------------------------------------------------- autotuner -- */

/* Launch shape of the traversal stages on the fast and wide layouts.  All
 * shapes return the same hits -- the per-ray walk is the same, only the
 * mapping of rays onto threads and of children onto nodes changes -- so the
 * choice is one of speed alone.  No counterpart in the reference, whose
 * traversal runs inside OptiX. */
enum { KGR_TRACE_GRID = 0, KGR_TRACE_PERSISTENT = 1 };
typedef struct kgr_trace_tune {
	int32_t layout; /* KGR_LAYOUT_FAST or KGR_LAYOUT_WIDE */
	int32_t shadow; /* shadow stage: KGR_TRACE_GRID (a ray per thread, grid-stride)
	                 * or KGR_TRACE_PERSISTENT (lanes refill as their rays end);
	                 * the closest-hit stage is always persistent */
	int32_t block;  /* threads per block of both stages: 64, 128 or 256 */
	int32_t occupancy; /* 0: registers as the compiler chooses; 1: capped so that
	                    * 48 warps fit an SM (more rays in flight per SM) */
	int32_t stack;     /* traversal stack entries a thread keeps in shared memory
	                    * (0, 8 or 16; deeper entries in local memory) */
} kgr_trace_tune;

typedef struct kgr_autotune_result {
	kgr_trace_tune best;
	double best_ms;       /* ms per frame of the chosen shape */
	double default_ms;    /* ms per frame of the untuned shape {fast, persistent, 128, 0, 0} */
	uint32_t candidates;  /* shapes timed */
	uint32_t reserved;
} kgr_autotune_result;

/* The project's autotuner: renders `frames` frames of `info` (after one
 * untimed frame) with every launch shape the scene admits -- layouts fast
 * and wide (when built) x shadow kernel x block size x occupancy -- then the
 * fastest of those with 8 and with 16 stack entries in shared memory, times
 * each on `stream` with CUDA events, and keeps the fastest as this
 * attachment's shape.  The options "layout", "trace_shadow", "trace_block",
 * "trace_occupancy" and "trace_stack" still override it field by field.  The frames are real renders: they write
 * info's buffers and advance ReSTIR history and radiance-cache training.
 * Synchronous. */
kgr_status kgr_autotune(kgr_attachment *att, const kgr_launch_info *info, const kgr_scene *scene,
		int32_t frames, void *stream, kgr_autotune_result *result);
/* The shape an attachment renders with now (tuned or default, options
 * applied). */
kgr_status kgr_get_trace_tune(const kgr_attachment *att, kgr_trace_tune *tune);

/* Traversal visit counts of the last frame rendered with the
 * "count_visits" option: {closest nodes, closest triangles, shadow nodes,
 * shadow triangles} on the layout the frame used. */
kgr_status kgr_get_visit_counts(const kgr_attachment *att, uint64_t counts[4]);

/* Streaming-read bandwidth probe (GB/s, best of 5): a buffer of `bytes`
 * read `iters` times with 16-byte L2-cached loads.  A buffer well below the
 * L2 size measures L2 bandwidth, one well above measures HBM. */
kgr_status kgr_measure_read_bandwidth(int32_t device, uint64_t bytes, int32_t iters, double *gbps);

/* Copy an internal per-pixel buffer of a ReSTIR attachment to the host
 * (synchronous; for inspection and tests): "reservoir_prev_a",
 * "reservoir_prev_b" (the 32-byte reservoirs kept for the next frame, as
 * {point xyz, light index bits} and {w, W, M bits, 0}), "intermediate",
 * "auxiliary" (float4 per pixel) or "materials" (kgr_material per pixel). */
kgr_status kgr_debug_copy(const kgr_attachment *att, const char *what, void *host, uint64_t bytes);

/* The .rtxa plugin export (source/amadeus/naive_path_tracer.cu:280-348),
 * returning a C handle instead of an AttachmentRTX*.  NULL name and ptr on
 * failure, as the reference does. */
typedef struct kgr_plugin_ret {
	const char *name;
	kgr_attachment *ptr;
} kgr_plugin_ret;
kgr_plugin_ret kgr_load_attachment(const char *kind);

/* --------------------------------------------------------- radiance cache -- */

/* The radiance-cache network: 64 inputs -> 5 hidden layers of 64 (ReLU) ->
 * RGB, half-precision weights and activations with FP32 accumulation on the
 * tensor cores, trained with Adam on a relative L2 loss.  The reference's
 * only network is an unused FP32 forward pass (editor/mlp.cuh:48-154). */
enum { KGR_MLP_BF16 = 0, KGR_MLP_FP16 = 1 };
typedef struct kgr_mlp kgr_mlp;

/* Uniform(+-sqrt(6/fan_in)) initialisation from `seed`. */
kgr_status kgr_mlp_create(int32_t dtype, uint64_t seed, int32_t device, kgr_mlp **out);
/* FP32 master weights W[6][64][64] as [layer][in][out] (last layer: out < 3). */
kgr_status kgr_mlp_get_weights(const kgr_mlp *mlp, float *host);
kgr_status kgr_mlp_set_weights(kgr_mlp *mlp, const float *host);
/* out (device, n x 4 floats) = network(x) for x (device, n x 64 halves of the
 * network's type).  Asynchronous on `stream`. */
kgr_status kgr_mlp_forward(kgr_mlp *mlp, const void *x, uint32_t n, float *out, void *stream);
/* Gradient of the loss sum_rows sum_c (y-t)^2/(y^2+0.01) / n over n rows
 * (targets device n x 4) into host memory (6*64*64 floats, may be NULL) and
 * the loss into *loss (may be NULL).  Synchronous. */
kgr_status kgr_mlp_gradients(kgr_mlp *mlp, const void *x, const float *targets, uint32_t n,
		float *grad_host, float *loss);
/* One Adam step (beta 0.9/0.99, eps 1e-8) at learning rate lr on n rows. */
kgr_status kgr_mlp_train_step(kgr_mlp *mlp, const void *x, const float *targets, uint32_t n,
		float lr, void *stream);
kgr_status kgr_mlp_destroy(kgr_mlp *mlp);

/* Inference kernel of kgr_mlp_forward and of the radiance cache:
 * KGR_MLP_INFER_TCGEN05 (the default: tcgen05.mma with the accumulator in
 * tensor memory, operands staged in shared memory) or KGR_MLP_INFER_MMA
 * (warp-level mma.sync, activations kept in registers).  Same network, same rounding points;
 * the results differ only in FP32 summation order.  No counterpart in the
 * reference, whose only network is an unused FP32 forward pass. */
enum { KGR_MLP_INFER_MMA = 0, KGR_MLP_INFER_TCGEN05 = 1 };
kgr_status kgr_mlp_set_inference(kgr_mlp *mlp, int32_t kernel);
/* Gradient kernel of kgr_mlp_gradients, kgr_mlp_train_step and the
 * radiance cache's training: KGR_MLP_TRAIN_TCGEN05 (the default:
 * tcgen05.mma on 128-row tiles, forward and the input deltas at M = 128,
 * the weight gradient at M = 64 accumulated in tensor memory over a block's
 * tiles) or KGR_MLP_TRAIN_MMA (warp-level mma.sync, 64-row tiles, the
 * weight gradient summed in shared memory).  Same network and rounding points;
 * the gradients differ only in FP32 summation order.  A tcgen05 wait that
 * runs out is reported by kgr_mlp_check. */
enum { KGR_MLP_TRAIN_MMA = 0, KGR_MLP_TRAIN_TCGEN05 = 1 };
kgr_status kgr_mlp_set_training(kgr_mlp *mlp, int32_t kernel);
/* Synchronise the device and report a tcgen05 inference whose mbarrier wait
 * ran out (KGR_ERR_CUDA; the flag is then cleared).  KGR_OK otherwise. */
kgr_status kgr_mlp_check(kgr_mlp *mlp);
/* A test of the timeout path: one tcgen05 inference over x (n rows) whose
 * blocks never issue their first tile's load, so each block's wait on it
 * runs out after 65,536 polls; the blocks set the error word, free their
 * tensor memory and return without writing `out`.  kgr_mlp_check then
 * reports KGR_ERR_CUDA, and the network stays usable. */
kgr_status kgr_mlp_test_wait_timeout(kgr_mlp *mlp, const void *x, uint32_t n, float *out, void *stream);

/* ------------------------------------------------------ after the frame -- */

/* HDR -> LDR: hdr_to_ldr (include/cuda/color.cuh:84-118).  hdr is the
 * float4 colour buffer (W x H, row 0 at the top), ldr receives one packed
 * pixel per entry, to_ui32 (include/cuda/cast.cuh:16-20) of make_color
 * (color.cuh:57-66), rows written bottom to top as the reference kernel
 * does.  Asynchronous on `stream`. */
enum { KGR_TONEMAP_ACES = 0, KGR_TONEMAP_SRGB = 1 }; /* eTonemappingACES, eTonemappingSRGB (color.cuh:76-79) */
kgr_status kgr_tonemap(const float *hdr, uint32_t *ldr, uint32_t width, uint32_t height, int32_t mode,
		void *stream);

/* Denoiser: replaces layers::Denoiser (include/layers/denoiser.cuh:14-55,
 * source/layers/denoiser.cu:9-149), whose OptiX AI denoiser is a closed
 * library, with this project's edge-avoiding a-trous filter (post.cu).  The
 * guides are the reference's Guides bits plus a position guide. */
enum {
	KGR_DENOISE_NONE = 0,
	KGR_DENOISE_NORMAL = 1,   /* eNormal */
	KGR_DENOISE_ALBEDO = 2,   /* eAlbedo: filter colour / albedo, multiply back */
	KGR_DENOISE_POSITION = 4  /* this project's: stop at depth and plane changes */
};
typedef struct kgr_denoise_params {
	int32_t iterations;     /* a-trous passes, 1..8 (step 1, 2, 4, ...); default 5 */
	float sigma_color;      /* relative luminance scale of the first pass, halved each pass; default 1 */
	float normal_power;     /* exponent of the normal cosine; default 64 */
	float sigma_position;   /* scale of the off-plane distance per unit separation; default 0.2 */
	int32_t reserved[4];
} kgr_denoise_params;
/* Denoiser::Input (denoiser.cuh:40-45) plus a position buffer; device float4
 * W x H each.  The normal buffer is always required (a zero normal marks a
 * pixel without a hit; hits and misses are never averaged together); the
 * albedo and position buffers are required when their guide is on. */
typedef struct kgr_denoise_input {
	const float *color;
	const float *normal;
	const float *albedo;
	const float *position;
} kgr_denoise_input;
typedef struct kgr_denoiser kgr_denoiser;
/* Denoiser::make (denoiser.cu:9-68): width x height, guides a KGR_DENOISE_*
 * mask; allocates the result and a scratch image. */
kgr_status kgr_denoiser_create(uint32_t width, uint32_t height, int32_t guides, int32_t device, kgr_denoiser **out);
/* denoise (denoiser.cu:71-149): the result lands in the denoiser's own
 * buffer (kgr_denoiser_result), as the reference's layer.result.  params
 * NULL: the defaults.  Asynchronous on `stream`. */
kgr_status kgr_denoise(kgr_denoiser *d, const kgr_denoise_input *input, const kgr_denoise_params *params,
		void *stream);
kgr_status kgr_denoiser_result(const kgr_denoiser *d, float **result);
/* Copy the result to host memory (synchronous; bytes = W x H x 16). */
kgr_status kgr_denoiser_copy_result(const kgr_denoiser *d, float *host, uint64_t bytes);
kgr_status kgr_denoiser_destroy(kgr_denoiser *d);

/* ------------------------------------------------------ procedural scenes -- */

/* Seeded procedural scenes used by the tests and the benchmark.  The
 * generator uses integer hashing and IEEE + - * / sqrt only, so a given
 * (name, seed) gives the same bits on every host.
 *   "box4k"    box [-2,2]^3 (12 tris) + 4096 random tris + 64 ceiling quads
 *   "terrain"  512x512 value-noise height field + 2000 icospheres (320 tris)
 *              + 512 emissive quads (1024 tris)
 *   "terrain_s","terrain_m","terrain_l": 0.25M / 1M / 4M triangle variants
 *   "tiny"     a few triangles, for unit tests                               */
typedef struct kgr_generated kgr_generated;

typedef struct kgr_generated_view {
	const float *positions;   /* 3 * vertex_count */
	const float *normals;     /* 3 * vertex_count */
	uint32_t vertex_count;
	const uint32_t *indices;  /* 3 * triangle_count */
	const uint32_t *material_indices;
	uint32_t triangle_count;
	const kgr_material *materials;
	uint32_t material_count;
	float camera_eye[3];
	float camera_target[3];
	float camera_fov_deg;
} kgr_generated_view;

kgr_status kgr_generate_scene(const char *name, uint64_t seed, kgr_generated **out);
kgr_status kgr_generated_get(const kgr_generated *g, kgr_generated_view *view);
kgr_status kgr_generated_destroy(kgr_generated *g);

/* ------------------------------------------------------ Kobra projects -- */

/* A Kobra project directory as Project::save writes it
 * (source/project.cpp:63-205): project.den lists the scenes; a .kobra scene
 * file lists entities with a transform, submeshes from the .cache mesh
 * cache with .mat materials from assets/, a renderable flag and a camera.
 * kgr_project_open is Project::load_project (include/project.hpp:58-92);
 * kgr_project_read_scene is Project::load_scene (source/project.cpp:
 * 242-560) into host arrays, one kgr_mesh per submesh of a renderable
 * entity with the entity's Transform::matrix() as its model.  Pass the
 * meshes and materials to kgr_scene_create; mesh k of the list is mesh k
 * of the scene, so kgr_scene_set_transforms moves entity e by its
 * [mesh_first, mesh_first + mesh_count) range.  Host only: no device. */
typedef struct kgr_project kgr_project;
typedef struct kgr_project_scene kgr_project_scene;

typedef struct kgr_project_scene_info {
	uint32_t entity_count;
	uint32_t mesh_count;         /* submeshes of renderable entities that were found */
	uint32_t vertex_count;
	uint32_t triangle_count;
	uint32_t material_count;     /* distinct by name, as the material daemon keeps them */
	uint32_t textured_materials; /* materials naming a texture (textures are not sampled) */
	uint32_t missing_meshes;     /* submesh files that were absent: skipped, as the reference skips them */
	int32_t camera_entity;       /* first entity with a camera, -1 if none */
} kgr_project_scene_info;

typedef struct kgr_project_entity {
	const char *name;     /* valid while the kgr_project_scene lives */
	float position[3];
	float rotation[3];    /* degrees, Euler x, y, z */
	float scale[3];
	float model[16];      /* Transform::matrix(), column-major */
	int32_t renderable;
	int32_t has_camera;
	float fov, aspect;    /* Camera component, when has_camera */
	uint32_t mesh_first;  /* its meshes in kgr_project_scene_meshes' list */
	uint32_t mesh_count;
} kgr_project_entity;

kgr_status kgr_project_open(const char *directory, kgr_project **out);
kgr_status kgr_project_scene_count(const kgr_project *p, uint32_t *count);
kgr_status kgr_project_scene_file(const kgr_project *p, uint32_t index, const char **name);
/* index < 0: the default scene (the first) */
kgr_status kgr_project_read_scene(const kgr_project *p, int32_t index, kgr_project_scene **out);
kgr_status kgr_project_scene_info_get(const kgr_project_scene *s, kgr_project_scene_info *info);
/* Pointers into the kgr_project_scene, valid while it lives. */
kgr_status kgr_project_scene_meshes(const kgr_project_scene *s, const kgr_mesh **meshes, uint32_t *mesh_count,
		const kgr_material **materials, uint32_t *material_count);
kgr_status kgr_project_scene_entity(const kgr_project_scene *s, uint32_t index, kgr_project_entity *out);
/* The launch camera of a camera entity: uvw_frame (include/camera.hpp:
 * 45-63) from Transform::forward()/up() (include/transform.hpp:98-112),
 * aspect <= 0 taking the entity's own. */
kgr_status kgr_project_scene_camera(const kgr_project_scene *s, uint32_t entity, float aspect,
		kgr_launch_info *info);
kgr_status kgr_project_scene_destroy(kgr_project_scene *s);
kgr_status kgr_project_close(kgr_project *p);

/* Transform::matrix() (include/transform.hpp:67-72): translate(position) *
 * mat4_cast(quat(radians(rotation))) * scale(scale), column-major. */
kgr_status kgr_transform_matrix(const float position[3], const float rotation_deg[3], const float scale[3],
		float out[16]);

/* Camera helper: uvw_frame of include/camera.hpp:45-63 plus the glm
 * perspective/lookAt matrices of camera.hpp:20-34 (near 0.1, far 1000). */
kgr_status kgr_camera_setup(const float eye[3], const float target[3], const float up[3],
		float fov_deg, float aspect, kgr_launch_info *info);

#ifdef __cplusplus
}
#endif

#endif

/*
 * kgr_mamba.h -- state and launcher of the "mamba" attachment: the editor's
 * default global-illumination mode (Mamba::render, editor/mamba.cu:941-1312).
 *
 * A frame is, in the reference's order:
 *   G-buffer       primary hits of every pixel centre (the reference rasters
 *                  them with Vulkan; here the closest-hit walk traces them)
 *   direct         ReSTIR DI with 8 candidates, temporal reuse and a
 *                  two-neighbour spatial pass (mamba_shader.cu:221-510),
 *                  when "direct_lighting" is set
 *   secondary      one BSDF-sampled ray per 4x4 block of pixels, cycling
 *                  through the block over 16 frames, and a light sample at
 *                  the primary vertex (mamba_shader.cu:512-680)
 *   gather         the secondary radiance splatted into irradiance probes
 *                  (secondary_gather, mamba.cu:401-576)
 *   sobel, raster, collapse, allocation
 *                  normal edges, the probe that covers each pixel, up to
 *                  four probes per 16x16 group, and new probes where a
 *                  16x16 block is less than 60% covered (mamba.cu:169-369,
 *                  889-938, mamba_kernels.cu:5-183)
 *   final gather   emission + direct + the two nearest probes' irradiance
 *                  (mamba.cu:686-878)
 *
 * The probe table is the reference's two-level hash (editor/optix/probe.cuh):
 * a top lookup table of 10-unit cells over a 250-unit cube at the origin,
 * each cell owning a second-level table of 0.4-unit cells that holds up to
 * 32767 probes by double hashing with two tries; a probe keeps 5 x 5 disk
 * bins of radiance sum, sample count and depth.
 *
 * Where the reference's outcome depends on thread timing, this build fixes
 * one of the outcomes its code allows:
 *   - probes are allocated one block at a time in block order (the
 *     reference's atomics allow any order, and its spin-waits on a
 *     neighbour's allocation are replaced by that order);
 *   - a bin's radiance is summed in 64-bit fixed point with 20 fractional
 *     bits, so the sum does not depend on the order of the splats; a bin's
 *     depth is the depth of the frame's last splat in splat order;
 *   - every read of the table, the reservoirs and the previous reservoirs
 *     sees them as they were when the pass began (the reference reads
 *     values other threads are writing).
 */
#ifndef KGR_MAMBA_H_
#define KGR_MAMBA_H_

#include "kgr_wavefront.h"

namespace kgr {

/* IrradianceProbe::size^2 (probe.cuh:11) */
#define KGR_PROBE_BINS 25
/* IrradianceProbeLUT MAX_REFS (probe.cuh:78) */
#define KGR_LUT_REFS 32767
/* fixed-point scale of a bin's radiance sum: 2^20 */
#define KGR_MAMBA_FIXED 1048576.0f
#define KGR_MAMBA_UNFIXED 9.5367431640625e-07f

/* One lookup table's header (IrradianceProbeLUT, probe.cuh:80-104): the
 * top table is level 2 with 10-unit cells, a second-level table level 1
 * with 0.4-unit cells. */
struct MambaLut {
	float center[3];
	float size;
	float resolution;
	int32_t level;
	int32_t counter;
	int32_t pad;
};

/* IrradianceProbeTable (probe.cuh:365-520) in structure-of-arrays form. */
struct MambaTable {
	MambaLut *luts;       /* max_luts */
	int32_t *refs;        /* max_luts * KGR_LUT_REFS: -1 empty, else the LUT (top) or probe index */
	uint32_t *hashes;     /* max_luts * KGR_LUT_REFS */
	float4 *positions;    /* max_luts * KGR_LUT_REFS: cell centre (top) or probe position */
	float4 *probe_pos;    /* max_probes */
	float4 *probe_nrm;    /* max_probes */
	unsigned long long *bin_le;    /* max_probes * 25 * 3, two's-complement fixed point */
	uint32_t *bin_n;               /* max_probes * 25: splats into the bin (pdfs) */
	unsigned long long *bin_depth; /* max_probes * 25: splat stamp << 32 | depth bits */
	int32_t *counters;             /* [0] probes, [1] lookup tables (starts at 1) */
	int32_t max_probes, max_luts;
};

/* Reservoir<LightInfo> (editor/optix/common.cuh:53-104): 64 bytes a pixel.
 *   r0 = {light position xyz, seed.z}
 *   r1 = {light normal xyz, sky ? 1 : 0}
 *   r2 = {emission xyz, M bits}
 *   r3 = {w, W, seed.x, seed.y}
 * (LightInfo::area is read only where it is sampled.) */
struct MambaReservoirs {
	float4 *r0, *r1, *r2, *r3;
};

struct MambaBuffers {
	/* G-buffer: raw interpolated position and shading normal, material (-1 = miss) */
	float4 *g_position, *g_normal;
	int32_t *g_index;
	/* direct lighting: reservoirs (in, out of the spatial pass), previous
	 * (in, out), accumulated direct radiance */
	MambaReservoirs res[2], prev[2];
	float4 *direct_Le;
	/* the direct passes' shadow rays in slots k * npix + pixel (k < 3):
	 * {origin}, {direction, tmax}, blocked flag; the queue of the slots to
	 * walk and its counters (CNT_SHADOW, CNT_FETCH_SHADOW of a path
	 * tracer's counter array); the spatial pass's neighbours and their M
	 * ({index0, index1, M0, M1}) */
	float4 *vis_o, *vis_d;
	uint32_t *vis_flag, *vis_queue, *vis_counters;
	int4 *spatial_aux;
	/* secondary rays at (W/4 + 1) x (H/4 + 1) */
	float4 *s_wi, *s_Le, *s_Ld, *s_Ld_wi; /* s_Ld_wi.w = Ld_depth */
	float4 *s_hit_x, *s_hit_n, *s_hit_wo;
	int32_t *s_hit_mat;
	/* splat records, two per secondary pixel: bin (-1 none), {Le, depth} */
	int32_t *rec_bin;
	float4 *rec_val;
	/* per pixel */
	float *sobel, *raster;
	float4 *raster_indicator, *raster_radiance;
	int32_t *probe_ids;
	/* per 16x16 group (ceil(W/16) x ceil(H/16)) */
	int4 *group_probes;
	int32_t *group_sizes;
	/* allocation candidates per 16x16 block ((W/16) x (H/16)): flag and
	 * pixel; and the ordered candidate list */
	int32_t *cand_flag;
	int2 *cand_pixel;
	int32_t *cand_list;
	MambaTable table;
};

struct MambaParams {
	uint32_t width, height, npix;
	uint32_t sec_w, sec_h;
	float origin[3], U[3], V[3], W[3];
	float prev_proj_view[16];
	float time;
	int32_t samples; /* frames since the camera last moved; 0 = moved */
	int32_t direct_lighting, indirect_lighting, irradiance, render_probes, render_probe_radiance;
	int32_t temporal, spatial;
	int32_t layout;
	int32_t res_in, prev_in; /* which of the two reservoir and previous sets are current */
	uint32_t stamp_base;     /* this frame's depth stamps are stamp_base + record + 1 */
	/* IrradianceProbe::from_index (probe.cuh:56-73) of each bin: a local
	 * direction, computed on the host */
	float bin_dir[KGR_PROBE_BINS][3];
};

/* Device buffers of a width x height attachment and a table of max_probes
 * probes and max_luts lookup tables, all zero (the table cleared as
 * mamba_table_clear leaves it); throws Error(KGR_ERR_OUT_OF_MEMORY). */
void mamba_alloc(MambaBuffers &mb, uint32_t width, uint32_t height, int32_t max_probes, int32_t max_luts);
void mamba_free(MambaBuffers &mb);
/* Every per-pixel and per-secondary buffer back to zero and the table
 * cleared (the state after mamba_alloc). */
void mamba_reset(const MambaBuffers &mb, uint32_t width, uint32_t height, cudaStream_t st);
/* A named device buffer and its size in bytes, for inspection:
 * "g_position", "g_normal", "g_index", "direct_le", "res_r0".."res_r3"
 * (the current reservoirs), "prev_r0".."prev_r3", "s_wi", "s_le", "s_ld",
 * "s_ld_wi", "s_hit_x", "s_hit_n", "s_hit_wo", "s_hit_mat", "sobel",
 * "raster", "raster_indicator", "raster_radiance", "probe_ids",
 * "group_probes", "group_sizes", "counters", "luts", "refs", "hashes",
 * "lut_positions", "probe_pos", "probe_nrm", "bin_le", "bin_n",
 * "bin_depth".  False for an unknown name. */
bool mamba_buffer(const MambaBuffers &mb, int res_in, int prev_in, uint32_t width, uint32_t height,
		const char *name, const void **ptr, size_t *bytes);

/* The local direction of each disk bin (from_index), in float. */
void mamba_bin_directions(float out[KGR_PROBE_BINS][3]);

/* Empty table: every ref -1, hashes all ones, the top table's header
 * (probe.cuh:106-118), counters {0, 1}, bins zero. */
void mamba_table_clear(const MambaTable &t, cudaStream_t st);

/* Resets the depth stamps to 0 keeping the depths (when stamp_base would
 * overflow). */
void mamba_restamp(const MambaTable &t, cudaStream_t st);

/* One frame; returns the launches it made.  pb supplies the closest-hit
 * walk's ray, hit and queue buffers (npix paths). */
uint32_t mamba_render(const DeviceScene &s, const PathBuffers &pb, const MambaParams &mp, const MambaBuffers &mb,
		const TraceTune &tune, float4 *color, cudaStream_t st, const StageMark &mark);

} /* namespace kgr */

#endif

/*
 * kgr_gi.h -- per-pixel state and launchers of ReSTIR GI (gi.cu).
 */
#ifndef KGR_GI_H_
#define KGR_GI_H_

#include "kgr_wavefront.h"

namespace kgr {

/* 32-byte GI reservoirs in two SoA arrays:
 *   a[i] = {x_s.xyz, bits(n_s octahedral 12+12 | M 8)}
 *   b[i] = {L_o.rgb, W} */
struct GiReservoirs {
	float4 *a;
	float4 *b;
};

struct GiFrameBuffers {
	GiReservoirs res[3];    /* previous frame, current, spatial ping-pong */
	kgr_material *materials; /* per pixel */
	float4 *position;       /* primary vertex, w = 1 when there is one */
	float4 *normal;
	float4 *prev_position;  /* last frame's primary vertices (temporal reuse) */
	float4 *prev_normal;
	float4 *direct;         /* ReSTIR DI direct light of the primary vertex */
	float4 *gi_dir;         /* GI direction xyz, source pdf */
	float4 *auxiliary;      /* final path seed (reuse RNG) */
	/* between the launches of a spatial iteration: per pixel {w_sum,
	 * bits(domain), bits(M sum), target}; per neighbour slot (k-major,
	 * k * npix + pixel) {neighbour pixel or -1, its M} and its weight; the
	 * queues of visibility rays (slots) of the two rounds and a counter
	 * array of CNT_COUNT entries per round (the queue count at CNT_SHADOW,
	 * the any-hit walk's fetch counter at CNT_FETCH_SHADOW) */
	float4 *selection;
	int2 *neighbours;
	float *weights;
	uint32_t *vis_queue[2];
	uint32_t *vis_count;
	/* rays for the tuned any-hit walk ({origin}, {direction, tmax}) of the
	 * final shading (slot = pixel), and the walk's blocked flag per slot
	 * (per path for the primary vertices' DI rays); the spatial rounds walk
	 * one ray per thread and zero a blocked slot's weight instead; vis_capacity slots */
	float4 *vis_o, *vis_d;
	uint32_t *vis_flag;
	uint32_t vis_capacity;
	/* every queued visibility ray also counts here (the frame's shadow-ray
	 * total, CNT_SHADOW_TOTAL of the path counters) */
	uint32_t *ray_total;
};

/* Most neighbours a spatial iteration takes (the gi_neighbors option). */
#define KGR_GI_MAX_NEIGHBORS 16
/* Kernels one spatial iteration launches (gather, visibility, resample,
 * visibility, finish), the primary vertex (its kernel, the walk of its DI
 * shadow rays, the blocked direct light) and the final shading (its rays,
 * the walk, the shading). */
#define KGR_GI_SPATIAL_LAUNCHES 5
#define KGR_GI_PRIMARY_LAUNCHES 3
#define KGR_GI_FINAL_LAUNCHES 3

void gi_primary(const DeviceScene &s, const PathBuffers &pb, const FrameParams &fp, const GiFrameBuffers &gb,
		cudaStream_t st);
void gi_initial(const PathBuffers &pb, const FrameParams &fp, const GiFrameBuffers &gb, int cur, cudaStream_t st);
void gi_temporal(const DeviceScene &s, const FrameParams &fp, const GiFrameBuffers &gb, int cur, int prev,
		cudaStream_t st);
void gi_spatial(const DeviceScene &s, const FrameParams &fp, const GiFrameBuffers &gb, int in, int out, int iteration,
		cudaStream_t st);
void gi_final(const DeviceScene &s, const FrameParams &fp, const GiFrameBuffers &gb, const OutputBuffers &out,
		int fin, cudaStream_t st);

} /* namespace kgr */

#endif

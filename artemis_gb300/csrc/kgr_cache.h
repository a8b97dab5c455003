/*
 * kgr_cache.h -- radiance-cache stages of the wavefront path tracer
 * (cache.cu) and their buffers.
 */
#ifndef KGR_CACHE_H_
#define KGR_CACHE_H_

#include "kgr_mlp.h"
#include "kgr_wavefront.h"

namespace kgr {

struct CacheParams {
	int dtype;                 /* KGR_MLP_BF16 or KGR_MLP_FP16 */
	float bmin[3], binv[3];    /* scene bounds: p = (x - bmin) * binv */
};

/* Per training path and depth: network input, throughput, radiance before
 * the vertex, emission (w = 1 when recorded). */
struct CacheRecords {
	void *feat;
	float4 *beta, *lbefore, *le;
	int depths;
};

void cache_query(const DeviceScene &s, const PathBuffers &pb, int q, const CacheParams &cp, void *feat,
		float4 *le, cudaStream_t st);
void cache_apply(const PathBuffers &pb, int q, const float4 *out, const float4 *le, cudaStream_t st);
/* Trace `paths` training paths to the full depth (one thread each), filling
 * `rec` and tb.L (final radiance); rec.le must be zero on entry. */
void cache_train_paths(const DeviceScene &s, const PathBuffers &tb, const FrameParams &fp, uint32_t paths,
		const CacheParams &cp, const CacheRecords &rec, cudaStream_t st);
void cache_targets(const PathBuffers &pb, uint32_t paths, const CacheRecords &rec, int dtype, void *xb, float4 *tb,
		uint32_t *count, uint32_t cap, cudaStream_t st);

} /* namespace kgr */

#endif

/*
 * kgr_post.h -- tonemapping and denoising of a finished frame (post.cu).
 */
#ifndef KGR_POST_H_
#define KGR_POST_H_

#include "kgr_internal.h"

namespace kgr {

/* hdr (float4, W x H, rows top to bottom) -> ldr (packed RGBA8, rows bottom
 * to top, as hdr_to_ldr_kernel writes them) */
void tonemap(const float4 *hdr, uint32_t *ldr, uint32_t width, uint32_t height, int mode, cudaStream_t st);

/* p.iterations a-trous passes from color into out (scratch: W x H float4) */
void denoise(const float4 *color, const float4 *normal, const float4 *albedo, const float4 *position, float4 *out,
		float4 *scratch, uint32_t width, uint32_t height, const kgr_denoise_params &p, int guides, cudaStream_t st);

} /* namespace kgr */

#endif

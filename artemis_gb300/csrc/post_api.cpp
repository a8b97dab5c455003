/*
 * post_api.cpp -- C ABI of the tonemapper and the denoiser (kgr_tonemap,
 * kgr_denoiser_*).
 */
#include <string.h>

#include <memory>

#include "kgr_post.h"

using namespace kgr;

struct kgr_denoiser {
	int device = 0;
	uint32_t width = 0, height = 0;
	int guides = 0;
	DevBuf<float4> result, scratch;
};

namespace {

template <class F>
kgr_status guard(F &&f)
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

bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

int device_of(int device)
{
	int count = 0;
	if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
		cudaGetLastError();
		throw Error(KGR_ERR_NO_DEVICE, "no CUDA device available");
	}
	if (device < 0)
		KGR_CUDA(cudaGetDevice(&device));
	KGR_REQUIRE(device < count, KGR_ERR_INVALID_ARGUMENT, "device ordinal out of range");
	return device;
}

} /* namespace */

extern "C" {

kgr_status kgr_tonemap(const float *hdr, uint32_t *ldr, uint32_t width, uint32_t height, int32_t mode, void *stream)
{
	return guard([&] {
		KGR_REQUIRE(mode == KGR_TONEMAP_ACES || mode == KGR_TONEMAP_SRGB, KGR_ERR_INVALID_ARGUMENT,
			"unknown tonemapping");
		if (width == 0 || height == 0)
			return;
		KGR_REQUIRE(hdr && ldr, KGR_ERR_INVALID_ARGUMENT, "NULL buffer");
		KGR_REQUIRE(aligned16(hdr) && ((uintptr_t)ldr & 3u) == 0, KGR_ERR_INVALID_ARGUMENT, "misaligned buffer");
		tonemap(reinterpret_cast<const float4 *>(hdr), ldr, width, height, mode, (cudaStream_t)stream);
	});
}

kgr_status kgr_denoiser_create(uint32_t width, uint32_t height, int32_t guides, int32_t device, kgr_denoiser **out)
{
	return guard([&] {
		KGR_REQUIRE(out, KGR_ERR_INVALID_ARGUMENT, "NULL out");
		*out = nullptr;
		KGR_REQUIRE(width >= 1 && height >= 1 && (uint64_t)width * height < (1ull << 30), KGR_ERR_INVALID_ARGUMENT,
			"extent out of range");
		KGR_REQUIRE((guides & ~7) == 0, KGR_ERR_INVALID_ARGUMENT, "unknown guide bits");
		int dev = device_of(device);
		DeviceGuard g(dev);
		std::unique_ptr<kgr_denoiser> d(new kgr_denoiser());
		d->device = dev;
		d->width = width;
		d->height = height;
		d->guides = guides;
		d->result.alloc((size_t)width * height);
		d->scratch.alloc((size_t)width * height);
		*out = d.release();
	});
}

kgr_status kgr_denoise(kgr_denoiser *d, const kgr_denoise_input *in, const kgr_denoise_params *params, void *stream)
{
	return guard([&] {
		KGR_REQUIRE(d && in && in->color, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		kgr_denoise_params p;
		memset(&p, 0, sizeof(p));
		p.iterations = 5;
		p.sigma_color = 1.0f;
		p.normal_power = 64.0f;
		p.sigma_position = 0.2f;
		if (params)
			p = *params;
		KGR_REQUIRE(p.iterations >= 1 && p.iterations <= 8, KGR_ERR_INVALID_ARGUMENT, "iterations must be 1..8");
		KGR_REQUIRE(p.sigma_color > 0.0f && p.normal_power >= 0.0f && p.sigma_position > 0.0f,
			KGR_ERR_INVALID_ARGUMENT, "sigmas must be positive");
		KGR_REQUIRE(in->normal, KGR_ERR_INVALID_ARGUMENT, "the normal buffer is required (it tells hits from misses)");
		KGR_REQUIRE(!(d->guides & KGR_DENOISE_ALBEDO) || in->albedo, KGR_ERR_INVALID_ARGUMENT, "albedo guide missing");
		KGR_REQUIRE(!(d->guides & KGR_DENOISE_POSITION) || in->position, KGR_ERR_INVALID_ARGUMENT,
			"position guide missing");
		KGR_REQUIRE(aligned16(in->color) && aligned16(in->normal) && aligned16(in->albedo) &&
				aligned16(in->position), KGR_ERR_INVALID_ARGUMENT, "buffers must be 16-byte aligned");
		DeviceGuard g(d->device);
		/* a guide that is off may have no buffer: the kernel never reads it,
		 * so it points at the colour */
		const float4 *c = reinterpret_cast<const float4 *>(in->color);
		const float4 *n = reinterpret_cast<const float4 *>(in->normal);
		const float4 *a = in->albedo ? reinterpret_cast<const float4 *>(in->albedo) : c;
		const float4 *x = in->position ? reinterpret_cast<const float4 *>(in->position) : c;
		denoise(c, n, a, x, d->result.ptr, d->scratch.ptr, d->width, d->height, p, d->guides, (cudaStream_t)stream);
	});
}

kgr_status kgr_denoiser_result(const kgr_denoiser *d, float **result)
{
	return guard([&] {
		KGR_REQUIRE(d && result, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		*result = reinterpret_cast<float *>(d->result.ptr);
	});
}

kgr_status kgr_denoiser_copy_result(const kgr_denoiser *d, float *host, uint64_t bytes)
{
	return guard([&] {
		KGR_REQUIRE(d && host, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		KGR_REQUIRE(bytes == d->result.bytes(), KGR_ERR_INVALID_ARGUMENT, "size differs from the result's");
		DeviceGuard g(d->device);
		KGR_CUDA(cudaDeviceSynchronize());
		KGR_CUDA(cudaMemcpy(host, d->result.ptr, bytes, cudaMemcpyDeviceToHost));
	});
}

kgr_status kgr_denoiser_destroy(kgr_denoiser *d)
{
	return guard([&] {
		if (!d)
			return;
		DeviceGuard g(d->device);
		delete d;
	});
}

} /* extern "C" */

/*
 * envmap.cu -- environment maps as CUDA texture objects (kgr_environment_*).
 *
 * ArmadaRTX::set_envmap (source/amadeus/armada.cu:86-96) imports the loaded
 * image into CUDA through Vulkan interop as a texture object with normalised
 * coordinates and linear filtering (include/cuda/interop.cuh:96-135; the
 * zero-initialised descriptor leaves every address mode at wrap).  Without
 * Vulkan the texels come from host memory: they are copied into a CUDA array
 * of float4 and wrapped in a texture object with the same descriptor.  The
 * kernels read it with tex2D<float4>, as the reference's programs do.
 */
#include <string.h>

#include <memory>

#include "kgr_internal.h"

struct kgr_environment {
	int device = 0;
	uint32_t width = 0, height = 0;
	cudaArray_t array = nullptr;
	cudaTextureObject_t texture = 0;
	~kgr_environment()
	{
		if (texture)
			cudaDestroyTextureObject(texture);
		if (array)
			cudaFreeArray(array);
	}
};

namespace kgr {
namespace {

__global__ void env_sample_kernel(cudaTextureObject_t tex, const float2 *uv, uint32_t n, float4 *out)
{
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	float2 c = uv[i];
	out[i] = tex2D<float4>(tex, c.x, c.y);
}

} /* namespace */
} /* namespace kgr */

using namespace kgr;

extern "C" {

kgr_status kgr_environment_create(const float *rgba, uint32_t width, uint32_t height, int32_t filter,
		int32_t device, kgr_environment **out)
{
	return guard_call([&] {
		KGR_REQUIRE(out, KGR_ERR_INVALID_ARGUMENT, "NULL out");
		*out = nullptr;
		KGR_REQUIRE(rgba, KGR_ERR_INVALID_ARGUMENT, "NULL texels");
		KGR_REQUIRE(width >= 1 && height >= 1 && width <= 65536 && height <= 65536, KGR_ERR_INVALID_ARGUMENT,
			"environment extent out of range");
		KGR_REQUIRE(filter == KGR_FILTER_LINEAR || filter == KGR_FILTER_POINT, KGR_ERR_INVALID_ARGUMENT,
			"unknown filter");
		int dev = pick_device_ordinal(device);
		DeviceGuard g(dev);
		std::unique_ptr<kgr_environment> env(new kgr_environment());
		env->device = dev;
		env->width = width;
		env->height = height;
		cudaChannelFormatDesc ch = cudaCreateChannelDesc(32, 32, 32, 32, cudaChannelFormatKindFloat);
		KGR_CUDA(cudaMallocArray(&env->array, &ch, width, height));
		KGR_CUDA(cudaMemcpy2DToArray(env->array, 0, 0, rgba, (size_t)width * 16, (size_t)width * 16, height,
			cudaMemcpyHostToDevice));
		cudaResourceDesc res;
		memset(&res, 0, sizeof(res));
		res.resType = cudaResourceTypeArray;
		res.res.array.array = env->array;
		cudaTextureDesc td;
		memset(&td, 0, sizeof(td)); /* address modes: wrap */
		td.readMode = cudaReadModeElementType;
		td.normalizedCoords = 1;
		td.filterMode = filter == KGR_FILTER_POINT ? cudaFilterModePoint : cudaFilterModeLinear;
		KGR_CUDA(cudaCreateTextureObject(&env->texture, &res, &td, nullptr));
		*out = env.release();
	});
}

kgr_status kgr_environment_texture(const kgr_environment *env, uint64_t *texture)
{
	return guard_call([&] {
		KGR_REQUIRE(env && texture, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		*texture = (uint64_t)env->texture;
	});
}

kgr_status kgr_environment_sample(const kgr_environment *env, const float *uv, uint32_t n, float *rgba,
		void *stream)
{
	return guard_call([&] {
		KGR_REQUIRE(env, KGR_ERR_INVALID_ARGUMENT, "NULL environment");
		if (n == 0)
			return;
		KGR_REQUIRE(uv && rgba, KGR_ERR_INVALID_ARGUMENT, "NULL buffer");
		KGR_REQUIRE(((uintptr_t)uv & 7u) == 0 && ((uintptr_t)rgba & 15u) == 0, KGR_ERR_INVALID_ARGUMENT,
			"misaligned buffer");
		DeviceGuard g(env->device);
		env_sample_kernel<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(env->texture,
			reinterpret_cast<const float2 *>(uv), n, reinterpret_cast<float4 *>(rgba));
		KGR_CUDA(cudaGetLastError());
	});
}

kgr_status kgr_environment_destroy(kgr_environment *env)
{
	return guard_call([&] {
		if (!env)
			return;
		DeviceGuard g(env->device);
		delete env;
	});
}

} /* extern "C" */

/*
 * mlp_api.cpp -- C ABI of the radiance-cache network (kgr_mlp_*).
 */
#include <math.h>
#include <string.h>

#include <memory>
#include <vector>

#include "kgr_mlp.h"

using namespace kgr;

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
	} catch (const std::exception &e) {
		set_last_error(e.what());
		return KGR_ERR_INTERNAL;
	}
}

int pick_device(int device)
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

void alloc_all(kgr_mlp *m)
{
	m->master.alloc(KGR_MLP_PARAMS);
	m->m.alloc(KGR_MLP_PARAMS);
	m->v.alloc(KGR_MLP_PARAMS);
	m->grad.alloc(KGR_MLP_PARAMS);
	m->loss.alloc(1);
	m->wn.alloc(KGR_MLP_PARAMS);
	m->wt.alloc(KGR_MLP_PARAMS);
	m->partial_blocks = kgr::device_sm_count();
	m->partial.alloc((size_t)m->partial_blocks * KGR_MLP_PARAMS);
	m->tc_err.alloc(1);
	KGR_CUDA(cudaMemset(m->tc_err.ptr, 0, sizeof(uint32_t)));
	KGR_CUDA(cudaMemset(m->m.ptr, 0, KGR_MLP_PARAMS * 4));
	KGR_CUDA(cudaMemset(m->v.ptr, 0, KGR_MLP_PARAMS * 4));
	KGR_CUDA(cudaMemset(m->wn.ptr, 0, KGR_MLP_PARAMS * 2));
	KGR_CUDA(cudaMemset(m->wt.ptr, 0, KGR_MLP_PARAMS * 2));
}

} /* namespace */

extern "C" {

kgr_status kgr_mlp_create(int32_t dtype, uint64_t seed, int32_t device, kgr_mlp **out)
{
	return guard([&] {
		KGR_REQUIRE(out, KGR_ERR_INVALID_ARGUMENT, "out is NULL");
		KGR_REQUIRE(dtype == KGR_MLP_BF16 || dtype == KGR_MLP_FP16, KGR_ERR_INVALID_ARGUMENT, "unknown dtype");
		*out = nullptr;
		int dev = pick_device(device);
		DeviceGuard g(dev);
		std::unique_ptr<kgr_mlp> m(new kgr_mlp());
		m->device = dev;
		m->dtype = dtype;
		alloc_all(m.get());
		std::vector<float> w(KGR_MLP_PARAMS, 0.0f);
		uint64_t s = seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
		const float a = sqrtf(6.0f / 64.0f);
		for (int l = 0; l < 6; l++)
			for (int i = 0; i < 64; i++)
				for (int o = 0; o < 64; o++) {
					s += 0x9E3779B97F4A7C15ull;
					uint64_t z = s;
					z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
					z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
					z ^= z >> 31;
					float u = (float)(z >> 40) * (1.0f / 16777216.0f);
					if (l < 5 || o < 3)
						w[(size_t)l * 4096 + i * 64 + o] = (2.0f * u - 1.0f) * a;
				}
		KGR_CUDA(cudaMemcpy(m->master.ptr, w.data(), KGR_MLP_PARAMS * 4, cudaMemcpyHostToDevice));
		mlp_adam(m->params(), m->grad.ptr, 0.0f, 0, 0);
		KGR_CUDA(cudaDeviceSynchronize());
		*out = m.release();
	});
}

kgr_status kgr_mlp_get_weights(const kgr_mlp *m, float *host)
{
	return guard([&] {
		KGR_REQUIRE(m && host, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		DeviceGuard g(m->device);
		KGR_CUDA(cudaMemcpy(host, m->master.ptr, KGR_MLP_PARAMS * 4, cudaMemcpyDeviceToHost));
	});
}

kgr_status kgr_mlp_set_weights(kgr_mlp *m, const float *host)
{
	return guard([&] {
		KGR_REQUIRE(m && host, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		DeviceGuard g(m->device);
		KGR_CUDA(cudaMemcpy(m->master.ptr, host, KGR_MLP_PARAMS * 4, cudaMemcpyHostToDevice));
		mlp_adam(m->params(), m->grad.ptr, 0.0f, 0, 0);
		KGR_CUDA(cudaDeviceSynchronize());
	});
}

kgr_status kgr_mlp_forward(kgr_mlp *m, const void *x, uint32_t n, float *out, void *stream)
{
	return guard([&] {
		KGR_REQUIRE(m && (n == 0 || (x && out)), KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		KGR_REQUIRE(((uintptr_t)x & 15u) == 0 && ((uintptr_t)out & 15u) == 0, KGR_ERR_INVALID_ARGUMENT,
			"buffers must be 16-byte aligned");
		DeviceGuard g(m->device);
		mlp_infer(m->params(), x, n, reinterpret_cast<float4 *>(out), (cudaStream_t)stream);
	});
}

kgr_status kgr_mlp_gradients(kgr_mlp *m, const void *x, const float *targets, uint32_t n, float *grad_host,
		float *loss)
{
	return guard([&] {
		KGR_REQUIRE(m && (n == 0 || (x && targets)), KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		DeviceGuard g(m->device);
		mlp_gradients(m->params(), x, reinterpret_cast<const float4 *>(targets), n, m->grad.ptr, m->loss.ptr, 0);
		if (grad_host)
			KGR_CUDA(cudaMemcpy(grad_host, m->grad.ptr, KGR_MLP_PARAMS * 4, cudaMemcpyDeviceToHost));
		if (loss)
			KGR_CUDA(cudaMemcpy(loss, m->loss.ptr, 4, cudaMemcpyDeviceToHost));
		KGR_CUDA(cudaDeviceSynchronize());
	});
}

kgr_status kgr_mlp_train_step(kgr_mlp *m, const void *x, const float *targets, uint32_t n, float lr, void *stream)
{
	return guard([&] {
		KGR_REQUIRE(m && (n == 0 || (x && targets)), KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		DeviceGuard g(m->device);
		cudaStream_t st = (cudaStream_t)stream;
		mlp_gradients(m->params(), x, reinterpret_cast<const float4 *>(targets), n, m->grad.ptr, m->loss.ptr, st);
		m->step++;
		mlp_adam(m->params(), m->grad.ptr, lr, m->step, st);
	});
}

kgr_status kgr_mlp_set_inference(kgr_mlp *m, int32_t kernel)
{
	return guard([&] {
		KGR_REQUIRE(m, KGR_ERR_INVALID_ARGUMENT, "NULL network");
		KGR_REQUIRE(kernel == KGR_MLP_INFER_MMA || kernel == KGR_MLP_INFER_TCGEN05, KGR_ERR_INVALID_ARGUMENT,
			"unknown inference kernel");
		m->infer = kernel;
	});
}

kgr_status kgr_mlp_set_training(kgr_mlp *m, int32_t kernel)
{
	return guard([&] {
		KGR_REQUIRE(m, KGR_ERR_INVALID_ARGUMENT, "NULL network");
		KGR_REQUIRE(kernel == KGR_MLP_TRAIN_MMA || kernel == KGR_MLP_TRAIN_TCGEN05, KGR_ERR_INVALID_ARGUMENT,
			"unknown training kernel");
		m->train = kernel;
	});
}

kgr_status kgr_mlp_test_wait_timeout(kgr_mlp *m, const void *x, uint32_t n, float *out, void *stream)
{
	return guard([&] {
		KGR_REQUIRE(m && n > 0 && x && out, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		KGR_REQUIRE(((uintptr_t)x & 15u) == 0 && ((uintptr_t)out & 15u) == 0, KGR_ERR_INVALID_ARGUMENT,
			"buffers must be 16-byte aligned");
		DeviceGuard g(m->device);
		mlp_infer_tc(m->params(), x, n, reinterpret_cast<float4 *>(out), m->tc_err.ptr, (cudaStream_t)stream,
			nullptr, true);
	});
}

kgr_status kgr_mlp_check(kgr_mlp *m)
{
	return guard([&] {
		KGR_REQUIRE(m, KGR_ERR_INVALID_ARGUMENT, "NULL network");
		DeviceGuard g(m->device);
		uint32_t e = 0;
		KGR_CUDA(cudaDeviceSynchronize());
		KGR_CUDA(cudaMemcpy(&e, m->tc_err.ptr, sizeof(e), cudaMemcpyDeviceToHost));
		if (e) {
			KGR_CUDA(cudaMemset(m->tc_err.ptr, 0, sizeof(uint32_t)));
			throw Error(KGR_ERR_CUDA, "tensor-core inference: an mbarrier wait ran out of its iteration limit");
		}
	});
}

kgr_status kgr_mlp_destroy(kgr_mlp *m)
{
	return guard([&] {
		if (!m)
			return;
		DeviceGuard g(m->device);
		delete m;
	});
}

} /* extern "C" */

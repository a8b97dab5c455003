/*
 * kgr_mlp.h -- the radiance-cache MLP (mlp.cu) and the device buffers of one
 * network: FP32 master weights W[6][64][64] ([in][out]; the last layer's
 * outputs 3..63 unused), Adam moments, and half-precision copies
 * wn[l] = [in][cols] and wt[l] = [cols][in] (cols = 64, or 16 for the last).
 */
#ifndef KGR_MLP_H_
#define KGR_MLP_H_

#include "kgr_internal.h"

namespace kgr {

#define KGR_MLP_PARAMS (6 * 64 * 64)
#define KGR_MLP_INPUTS 64

struct MlpParams {
	int dtype; /* KGR_MLP_BF16 or KGR_MLP_FP16 */
	float *master, *m, *v;
	void *wn, *wt;
	float *partial;     /* per-block gradient slices [partial_blocks][6][64][64] */
	int partial_blocks;
	int infer;          /* KGR_MLP_INFER_MMA or KGR_MLP_INFER_TCGEN05 */
	uint32_t *tc_err;   /* error word of the tcgen05 kernels (bit 0: a wait ran out) */
	int train;          /* KGR_MLP_TRAIN_MMA or KGR_MLP_TRAIN_TCGEN05 */
};

/* out[i] = {r, g, b, 0} for the n rows of x ([n][64] half precision); with
 * n_dev, the row count is min(n, *n_dev) read on the device. */
void mlp_infer(const MlpParams &mp, const void *x, uint32_t n, float4 *out, cudaStream_t st,
		const uint32_t *n_dev = nullptr);
/* The same on the fifth-generation tensor cores (mlp_tc.cu): tcgen05.mma
 * with TMEM accumulators; sets bit 0 of *err if an mbarrier wait ran out.
 * withhold_first: a test of that path (every block's first load is not
 * issued, so its wait runs out; no output row is written). */
void mlp_infer_tc(const MlpParams &mp, const void *x, uint32_t n, float4 *out, uint32_t *err, cudaStream_t st,
		const uint32_t *n_dev = nullptr, bool withhold_first = false);
/* The gradient pass of mlp_gradients on the tensor cores (mlp_tc.cu):
 * grid blocks write their slices of mp.partial (tiles of 128 rows) and add
 * their loss into *loss; sets bit 0 of *mp.tc_err if a wait ran out. */
void mlp_train_tc(const MlpParams &mp, const void *x, const float4 *target, uint32_t n, int grid, float *loss,
		cudaStream_t st, const uint32_t *n_dev);
/* grad (FP32, [6][64][64]) = d loss / d W over n rows; loss = sum of the
 * relative L2 terms (not divided by n).  Uses mp.partial as scratch; the
 * result does not depend on block scheduling.  max_blocks > 0 caps the grid
 * (each block takes one SM's shared memory): training that runs beside a
 * frame leaves the other SMs to the frame. */
void mlp_gradients(const MlpParams &mp, const void *x, const float4 *target, uint32_t n, float *grad, float *loss,
		cudaStream_t st, const uint32_t *n_dev = nullptr, int max_blocks = 0);
/* One Adam step (lr, bias correction for `step`); step <= 0 only refreshes
 * the half-precision copies from the master weights. */
void mlp_adam(const MlpParams &mp, const float *grad, float lr, int step, cudaStream_t st);

int device_sm_count();

} /* namespace kgr */

struct kgr_mlp {
	int device = 0;
	int dtype = 0;
	int step = 0;
	int partial_blocks = 0;
	int infer = KGR_MLP_INFER_TCGEN05;
	int train = KGR_MLP_TRAIN_TCGEN05;
	kgr::DevBuf<float> master, m, v, grad, loss, partial;
	kgr::DevBuf<uint16_t> wn, wt;
	kgr::DevBuf<uint32_t> tc_err;
	kgr::MlpParams params()
	{
		return kgr::MlpParams{dtype, master.ptr, m.ptr, v.ptr, wn.ptr, wt.ptr, partial.ptr, partial_blocks, infer,
			tc_err.ptr, train};
	}
};

#endif

/*
 * mlp_tc.cu -- radiance-cache network inference on the fifth-generation
 * tensor cores: tcgen05.mma with the accumulator in tensor memory (TMEM).
 *
 * The network is the one of mlp.cu (64 inputs -> 5 x 64 ReLU -> 3 outputs,
 * BF16 or FP16 weights and activations, FP32 accumulation); this kernel is
 * an alternative to its mma.sync inference and computes the same function.
 *
 * A CTA of four warpgroups (512 threads) holds the weights once and runs
 * four independent chains, one a warpgroup, each walking tiles of 128 rows
 * (the MMA's M) with its own buffer, barriers and accumulator; two CTAs fit
 * an SM, so eight tiles move through the network on an SM at once and the
 * 512 TMEM columns are all in use:
 *   weights        the six layers (B operands, N x K) in shared memory in
 *                  the canonical K-major layout without swizzle: 8 x 8 core
 *                  matrices of 128 contiguous bytes, K neighbours 128 bytes
 *                  apart (leading byte offset), 8-row groups 1024 bytes apart
 *                  (stride byte offset);
 *   activations    one 128 x 64 tile (A operand) a chain in the K-major
 *                  layout with the 128-byte swizzle: row r at r x 128 bytes,
 *                  its 16-byte chunk c at chunk c ^ (r mod 8).  A tile
 *                  arrives by one TMA load (cp.async.bulk.tensor.2d, the
 *                  tensor map's 128-byte swizzle writes exactly this layout;
 *                  rows past the end read as zero); the chain's next tile is
 *                  loaded into the same buffer as soon as the last layer's
 *                  MMA has read it, while the outputs are read back;
 *   TMEM           a 128-lane x 64-column FP32 accumulator a chain (columns
 *                  64 c .. 64 c + 63), row i in lane i; a warp reads lanes
 *                  32 (warp mod 4) .. +31;
 *   per layer      one thread of the chain issues four tcgen05.mma (K = 16
 *                  each; the A start address advances 32 bytes inside the
 *                  swizzled row) and a tcgen05.commit to the chain's
 *                  mbarrier; after it every warp of the chain reads its 32
 *                  lanes with tcgen05.ld (32x32b, two halves of 32 columns),
 *                  applies ReLU, rounds to half precision and writes the row
 *                  back into the tile, swizzled, as the next layer's A
 *                  operand; the chain's 128 threads meet at a named barrier
 *                  (1 + chain).
 *
 * Every wait on an mbarrier is bounded.  A wait that runs out sets bit 0 of
 * the error word; the chain stops at the next layer boundary (the decision
 * is taken by all its threads together), waits (bounded) for its TMA load in
 * flight, and the block frees its TMEM and returns; the host reads the word with
 * kgr_mlp_check.  kgr_mlp_test_wait_timeout exercises that path: its launch
 * withholds each block's first load, so the wait on it runs out (after
 * TC_WAIT_TEST_LIMIT polls) before any MMA was issued.
 */
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cuda.h>

#include <mutex>
#include <type_traits>

#include "kgr_mlp.h"

namespace kgr {

namespace {

#define TC_ROWS 128                 /* rows per tile: the MMA's M */
#define TC_W 64                     /* hidden width and input width */
#define TC_OUT 16                   /* N of the last layer (3 outputs used) */
#define TC_LAYERS 6
#define TC_LBO 128u                 /* bytes between K-neighbour core matrices */
#define TC_SBO 1024u                /* bytes between 8-row groups (64-wide K) */
#define TC_LAYER_BYTES 8192u        /* 64 x 64 half-precision weights */
#define TC_W_BYTES (5u * TC_LAYER_BYTES + 2048u)
#define TC_CHAINS 4                 /* warpgroups a CTA, each walking tiles of its own */
#define TC_THREADS (128 * TC_CHAINS)
#define TC_X_OFF 43008u             /* = TC_W_BYTES, a multiple of 1024 (swizzle atom) */
#define TC_X_BYTES (TC_ROWS * TC_W * 2u)
#define TC_BAR_OFF (TC_X_OFF + TC_CHAINS * TC_X_BYTES)  /* per chain: MMA barrier, TMA barrier */
#define TC_SLOT_OFF (TC_BAR_OFF + TC_CHAINS * 16u)
#define TC_SMEM (TC_SLOT_OFF + 8u)  /* 108,616 bytes: two CTAs fit an SM */
#define TC_TMEM_COLS 256u           /* 64 columns a chain, rounded up to a power of two */
#define TC_WAIT_LIMIT (1u << 24)    /* mbarrier polls before a wait gives up */
#define TC_WAIT_TEST_LIMIT (1u << 16) /* the same, in a launch that tests the give-up path */

/* Byte offset of element (r, k) of an R x 64 K-major operand without
 * swizzle (the weights). */
__device__ __forceinline__ uint32_t core_off(uint32_t r, uint32_t k)
{
	return (r >> 3) * TC_SBO + (k >> 3) * TC_LBO + (r & 7u) * 16u + (k & 7u) * 2u;
}

/* Byte offset of the 16-byte chunk c of row r of a 128-byte-swizzled tile
 * (the activations). */
__device__ __forceinline__ uint32_t sw128_off(uint32_t r, uint32_t c)
{
	return r * 128u + ((c ^ (r & 7u)) << 4);
}

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
	return (uint32_t)__cvta_generic_to_shared(p);
}

/* Shared-memory matrix descriptor: start address, leading and stride byte
 * offsets (all in 16-byte units), descriptor version 1, layout type (0: no
 * swizzle; 2: 128-byte swizzle, whose leading offset is unused). */
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo, uint32_t layout)
{
	uint64_t d = (uint64_t)((addr >> 4) & 0x3FFFu);
	d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
	d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
	d |= (uint64_t)1u << 46;
	d |= (uint64_t)layout << 61;
	return d;
}

/* Arm a TMA barrier with the bytes of one tile and start the tile's load:
 * rows [row0, row0 + 128) of the [n][64] input, all 64 columns (x = 0). */
__device__ __forceinline__ void tma_tile(const CUtensorMap *map, uint32_t dst, uint32_t bar, int row0)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(bar), "r"(TC_X_BYTES) : "memory");
	asm volatile(
		"cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
		:: "r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(row0), "r"(bar) : "memory");
}

/* Instruction descriptor of kind::f16: FP32 accumulator, A and B both BF16
 * (or both FP16), both K-major, N and M. */
__device__ __forceinline__ uint32_t instr_desc(bool bf16, uint32_t n, uint32_t m)
{
	uint32_t f = bf16 ? 1u : 0u;
	return (1u << 4) | (f << 7) | (f << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

/* Barrier of one chain's 128 threads (named barrier 1 + chain; 0 is the
 * CTA's), and the same with an AND over a flag of every thread. */
__device__ __forceinline__ void chain_sync(int chain)
{
	asm volatile("bar.sync %0, 128;" :: "r"(chain + 1) : "memory");
}

__device__ __forceinline__ bool chain_and(int chain, bool v)
{
	uint32_t r;
	asm volatile(
		"{\n\t.reg .pred p, q;\n\t"
		"setp.ne.u32 q, %1, 0;\n\t"
		"bar.red.and.pred p, %2, 128, q;\n\t"
		"selp.u32 %0, 1, 0, p;\n\t"
		"}"
		: "=r"(r) : "r"((uint32_t)v), "r"(chain + 1) : "memory");
	return r != 0;
}

__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
	asm volatile(
		"{\n\t.reg .pred p;\n\t"
		"setp.ne.b32 p, %4, 0;\n\t"
		"tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t"
		"}"
		:: "r"(tmem), "l"(a), "l"(b), "r"(idesc), "r"(acc) : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t bar)
{
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(bar)
		: "memory");
}

/* Poll the mbarrier for the completion of `parity`, at most `limit` times.
 * Returns false when it gave up. */
__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity, uint32_t limit)
{
	for (uint32_t i = 0; i < limit; i++) {
		uint32_t done;
		asm volatile(
			"{\n\t.reg .pred p;\n\t"
			"mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
			"selp.u32 %0, 1, 0, p;\n\t"
			"}"
			: "=r"(done) : "r"(bar), "r"(parity) : "memory");
		if (done)
			return true;
	}
	return false;
}

#define TC_R8(i) "=r"(v[i]), "=r"(v[i + 1]), "=r"(v[i + 2]), "=r"(v[i + 3]), "=r"(v[i + 4]), "=r"(v[i + 5]), \
	"=r"(v[i + 6]), "=r"(v[i + 7])

/* 64 consecutive FP32 columns of this thread's TMEM lane. */
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, uint32_t (&v)[64])
{
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x64.b32 "
		"{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
		"%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, "
		"%32, %33, %34, %35, %36, %37, %38, %39, %40, %41, %42, %43, %44, %45, %46, %47, "
		"%48, %49, %50, %51, %52, %53, %54, %55, %56, %57, %58, %59, %60, %61, %62, %63}, [%64];"
		: TC_R8(0), TC_R8(8), TC_R8(16), TC_R8(24), TC_R8(32), TC_R8(40), TC_R8(48), TC_R8(56)
		: "r"(taddr) : "memory");
}

/* 32 consecutive FP32 columns of this thread's TMEM lane. */
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32])
{
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
		"{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
		"%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
		: TC_R8(0), TC_R8(8), TC_R8(16), TC_R8(24) : "r"(taddr) : "memory");
}

/* 16 consecutive FP32 columns of this thread's TMEM lane. */
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16])
{
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
		"{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
		: TC_R8(0), TC_R8(8) : "r"(taddr) : "memory");
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

template <class T>
__device__ __forceinline__ uint32_t pack_relu(uint32_t lo, uint32_t hi);

template <>
__device__ __forceinline__ uint32_t pack_relu<__nv_bfloat16>(uint32_t lo, uint32_t hi)
{
	__nv_bfloat162 h = __floats2bfloat162_rn(fmaxf(__uint_as_float(lo), 0.0f), fmaxf(__uint_as_float(hi), 0.0f));
	return *reinterpret_cast<uint32_t *>(&h);
}

template <>
__device__ __forceinline__ uint32_t pack_relu<__half>(uint32_t lo, uint32_t hi)
{
	__half2 h = __floats2half2_rn(fmaxf(__uint_as_float(lo), 0.0f), fmaxf(__uint_as_float(hi), 0.0f));
	return *reinterpret_cast<uint32_t *>(&h);
}

template <class T>
__global__ void __launch_bounds__(TC_THREADS, 2) mlp_infer_tc_kernel(const T *__restrict__ wt_g,
		const __grid_constant__ CUtensorMap xmap, uint32_t n, float4 *__restrict__ out,
		const uint32_t *__restrict__ n_dev, uint32_t *__restrict__ err, uint32_t withhold_first)
{
	const uint32_t limit = withhold_first ? TC_WAIT_TEST_LIMIT : TC_WAIT_LIMIT;
	if (n_dev) {
		uint32_t c = *n_dev;
		n = c < n ? c : n;
	}
	extern __shared__ __align__(1024) unsigned char sm[];
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	/* chain = warpgroup; a warp reads the TMEM lanes 32 (warp mod 4) .. +31 */
	const int chain = warp >> 2, ctid = tid & 127, cwarp = warp & 3;
	/* the 128-byte swizzle repeats every 1024 bytes; the kernel has no static
	 * shared memory, so its dynamic block starts on such a boundary.  If it
	 * did not, report it (bit 1) and do nothing. */
	if (smem_addr(sm) & 1023u) {
		if (tid == 0)
			atomicOr(err, 2u);
		return;
	}
	const bool bf16 = std::is_same<T, __nv_bfloat16>::value;
	const uint32_t mbar = smem_addr(sm + TC_BAR_OFF + 16u * (uint32_t)chain), tbar = mbar + 8u;
	uint32_t *slot = reinterpret_cast<uint32_t *>(sm + TC_SLOT_OFF);
	const uint32_t tiles = (n + TC_ROWS - 1) / TC_ROWS;

	/* weights: global [l][rows][64] row-major -> canonical layout */
	for (int l = 0; l < TC_LAYERS; l++) {
		int rows = l == TC_LAYERS - 1 ? TC_OUT : TC_W;
		const uint4 *src = reinterpret_cast<const uint4 *>(wt_g + (size_t)l * TC_W * TC_W);
		unsigned char *dst = sm + l * TC_LAYER_BYTES;
		for (int c = tid; c < rows * 8; c += TC_THREADS) {
			uint32_t r = (uint32_t)c >> 3, kb = (uint32_t)c & 7u;
			*reinterpret_cast<uint4 *>(dst + core_off(r, kb * 8u)) = __ldg(src + c);
		}
	}
	if (tid == 0) {
		for (int i = 0; i < 2 * TC_CHAINS; i++)
			asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_addr(sm + TC_BAR_OFF) + 8u * i),
				"r"(1u) : "memory");
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	if (warp == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
			:: "r"(smem_addr(slot)), "r"(TC_TMEM_COLS) : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
	}
	fence_async_smem();
	tc_before();
	__syncthreads();
	tc_after();
	const uint32_t tmem_base = *slot;
	const uint32_t tmem = tmem_base + 64u * (uint32_t)chain;
	const uint32_t lane_addr = tmem + ((uint32_t)(cwarp * 32) << 16);
	const uint32_t wbase = smem_addr(sm), xbase = smem_addr(sm + TC_X_OFF + (uint32_t)chain * TC_X_BYTES);
	unsigned char *xs = sm + TC_X_OFF + (uint32_t)chain * TC_X_BYTES;
	const uint32_t id_hidden = instr_desc(bf16, TC_W, TC_ROWS), id_out = instr_desc(bf16, TC_OUT, TC_ROWS);
	uint32_t parity = 0;
	bool ok = true;
	/* a TMA load issued and not yet waited for, and its parity */
	bool pending = false;
	uint32_t pend_parity = 0;

	const uint32_t stride = gridDim.x * TC_CHAINS;
	uint32_t t = blockIdx.x * TC_CHAINS + (uint32_t)chain;
	if (ctid == 0 && t < tiles && !withhold_first)
		tma_tile(&xmap, xbase, tbar, (int)(t * TC_ROWS));
	pending = t < tiles && !withhold_first;
	for (uint32_t i = 0; ok && t < tiles; i++, t += stride) {
		pend_parity = i & 1u;
		bool got = bar_wait(tbar, i & 1u, limit);
		ok = chain_and(chain, got);
		if (!ok)
			break;
		pending = false;
		const uint64_t lo_sw = 2u; /* layout type: 128-byte swizzle */
		for (int l = 0; l < TC_LAYERS; l++) {
			const bool last = l == TC_LAYERS - 1;
			if (ctid == 0) {
				for (uint32_t kc = 0; kc < 4; kc++)
					tc_mma(tmem, smem_desc(xbase + kc * 32u, 16u, 1024u, (uint32_t)lo_sw),
						smem_desc(wbase + l * TC_LAYER_BYTES + kc * 256u, TC_LBO, TC_SBO, 0u),
						last ? id_out : id_hidden, kc > 0 ? 1u : 0u);
				tc_commit(mbar);
			}
			got = bar_wait(mbar, parity, limit);
			parity ^= 1u;
			ok = chain_and(chain, got);
			tc_after();
			if (!ok)
				break;
			uint32_t r = (uint32_t)(cwarp * 32 + lane);
			if (!last) {
				/* two halves of 32 columns: two CTAs of 512 threads leave
				 * 64 registers a thread */
#pragma unroll
				for (uint32_t h = 0; h < 2; h++) {
					uint32_t v[32];
					tmem_ld32(lane_addr + 32u * h, v);
					tmem_wait_ld();
#pragma unroll
					for (uint32_t kb = 0; kb < 4; kb++) {
						uint4 p;
						p.x = pack_relu<T>(v[8 * kb + 0], v[8 * kb + 1]);
						p.y = pack_relu<T>(v[8 * kb + 2], v[8 * kb + 3]);
						p.z = pack_relu<T>(v[8 * kb + 4], v[8 * kb + 5]);
						p.w = pack_relu<T>(v[8 * kb + 6], v[8 * kb + 7]);
						*reinterpret_cast<uint4 *>(xs + sw128_off(r, 4u * h + kb)) = p;
					}
				}
				fence_async_smem();
			} else {
				/* the last MMA has read the tile: the next tile's load into
				 * the same buffer runs while the outputs are read */
				uint32_t tn = t + stride;
				if (ctid == 0 && tn < tiles)
					tma_tile(&xmap, xbase, tbar, (int)(tn * TC_ROWS));
				pending = tn < tiles;
				uint32_t v[16];
				tmem_ld16(lane_addr, v);
				tmem_wait_ld();
				size_t row = (size_t)t * TC_ROWS + r;
				if (row < n)
					out[row] = make_float4(__uint_as_float(v[0]), __uint_as_float(v[1]), __uint_as_float(v[2]), 0.0f);
			}
			tc_before();
			chain_sync(chain);
			tc_after();
		}
	}
	if (!ok) {
		if (ctid == 0)
			atomicOr(err, 1u);
		/* a load may still be in flight: give it its (bounded) time before
		 * the block frees its memory */
		if (pending)
			bar_wait(tbar, pend_parity, limit);
	}
	tc_before();
	__syncthreads();
	tc_after();
	if (warp == 0)
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem_base), "r"(TC_TMEM_COLS)
			: "memory");
}

/* ------------------------------------------------------------ training -- */

/* Training (forward, loss, backward) on the fifth-generation tensor cores.
 * One CTA of 128 threads per SM (225 KB of shared memory, 512 TMEM
 * columns) walks tiles of 128 rows; every operand sits in shared memory in
 * the canonical K-major layout without swizzle (8 x 8 core matrices of 128
 * contiguous bytes, K neighbours 128 bytes apart, 8-row groups K/8 x 128
 * bytes apart):
 *   WT   the six layers' weights as [out][in] (forward B operands, 42 KB)
 *   WN   layers 1..5 as [in][out] (the delta's B operands, 34 KB)
 *   X    the tile's input of the current layer [128][64] (forward A operand)
 *   AT   every layer's input transposed, [64][128] (A operands of dW)
 *   D    the delta of the current layer's output [128][cols] (A operand)
 *   DT   the same transposed, [cols][128] (B operand of dW)
 * Per tile: six forward MMAs (M = 128) whose epilogue applies ReLU, rounds
 * to half precision and writes X and AT; the loss and the output delta;
 * then for each layer from the last, dW += AT^T-shaped MMA (M = 64: the
 * layer's 64 inputs, N = its outputs, K = the 128 rows), accumulated in
 * TMEM over every tile of the block, and the delta of the layer input
 * (M = 128, N = 64, K = outputs) masked by ReLU'.  With M = 64 the
 * accumulator's rows 16q..16q+15 are TMEM lanes 32q..32q+15.  At the end
 * the block writes its dW to its slice of `partial`, which the host sums in
 * block order; the rounding points are those of mlp_train_kernel. */
#define TT_ROWS 128
#define TT_SBO16 256u
#define TT_SBO64 1024u
#define TT_SBO128 2048u
#define TT_WN_OFF TC_W_BYTES                      /* 43,008 */
#define TT_WN_BYTES (4u * TC_LAYER_BYTES + 2048u) /* layers 1..4, then layer 5 (K = 16) */
#define TT_X_OFF (TT_WN_OFF + TT_WN_BYTES)        /* 77,824 */
#define TT_TILE_BYTES (TT_ROWS * TC_W * 2u)       /* 16 KB */
#define TT_AT_OFF (TT_X_OFF + TT_TILE_BYTES)
#define TT_D_OFF (TT_AT_OFF + 6u * TT_TILE_BYTES)
#define TT_DT_OFF (TT_D_OFF + TT_TILE_BYTES)
#define TT_BAR_OFF (TT_DT_OFF + TT_TILE_BYTES)    /* 225,280 */
#define TT_SLOT_OFF (TT_BAR_OFF + 8u)
#define TT_SMEM (TT_SLOT_OFF + 8u)
#define TT_TMEM_COLS 512u
#define TT_DW_COL(l) (64u + 64u * (uint32_t)(l))   /* dW of layer l (layer 5: 16 columns) */

__device__ __forceinline__ uint32_t kmaj_off(uint32_t r, uint32_t k, uint32_t sbo)
{
	return (r >> 3) * sbo + (k >> 3) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

__device__ __forceinline__ uint32_t wn_off(int l)
{
	return TT_WN_OFF + (l < TC_LAYERS - 1 ? (uint32_t)(l - 1) * TC_LAYER_BYTES : 4u * TC_LAYER_BYTES);
}

template <class T>
__device__ __forceinline__ T half_bits(uint16_t b)
{
	T h;
	*reinterpret_cast<uint16_t *>(&h) = b;
	return h;
}

template <class T>
__device__ __forceinline__ uint16_t bits_of(T h)
{
	return *reinterpret_cast<uint16_t *>(&h);
}

template <class T>
__device__ __forceinline__ float half_to_float(T h);
template <>
__device__ __forceinline__ float half_to_float<__nv_bfloat16>(__nv_bfloat16 h) { return __bfloat162float(h); }
template <>
__device__ __forceinline__ float half_to_float<__half>(__half h) { return __half2float(h); }

template <class T>
__device__ __forceinline__ T float_to_half(float f);
template <>
__device__ __forceinline__ __nv_bfloat16 float_to_half<__nv_bfloat16>(float f) { return __float2bfloat16_rn(f); }
template <>
__device__ __forceinline__ __half float_to_half<__half>(float f) { return __float2half_rn(f); }

/* A row of 8 halves (one 16-byte chunk) from 8 values. */
template <class T>
__device__ __forceinline__ uint4 pack8(const uint16_t (&h)[8])
{
	uint4 p;
	p.x = (uint32_t)h[0] | ((uint32_t)h[1] << 16);
	p.y = (uint32_t)h[2] | ((uint32_t)h[3] << 16);
	p.z = (uint32_t)h[4] | ((uint32_t)h[5] << 16);
	p.w = (uint32_t)h[6] | ((uint32_t)h[7] << 16);
	return p;
}

template <class T>
__global__ void __launch_bounds__(128, 1) mlp_train_tc_kernel(const T *__restrict__ wt_g, const T *__restrict__ wn_g,
		const T *__restrict__ x, const float4 *__restrict__ target, uint32_t n, float *__restrict__ partial,
		float *__restrict__ loss_sum, const uint32_t *__restrict__ n_dev, uint32_t *__restrict__ err)
{
	if (n_dev) {
		uint32_t c = *n_dev;
		n = c < n ? c : n;
	}
	extern __shared__ __align__(1024) unsigned char sm[];
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const bool bf16 = std::is_same<T, __nv_bfloat16>::value;
	const uint32_t bar = smem_addr(sm + TT_BAR_OFF);
	uint32_t *slot = reinterpret_cast<uint32_t *>(sm + TT_SLOT_OFF);
	const uint32_t tiles = (n + TT_ROWS - 1) / TT_ROWS;

	/* weights: forward [out][in], then layers 1..5 as [in][out] */
	for (int l = 0; l < TC_LAYERS; l++) {
		int rows = l == TC_LAYERS - 1 ? TC_OUT : TC_W;
		const uint4 *src = reinterpret_cast<const uint4 *>(wt_g + (size_t)l * TC_W * TC_W);
		unsigned char *dst = sm + l * TC_LAYER_BYTES;
		for (int c = tid; c < rows * 8; c += 128) {
			uint32_t r = (uint32_t)c >> 3, kb = (uint32_t)c & 7u;
			*reinterpret_cast<uint4 *>(dst + kmaj_off(r, kb * 8u, TT_SBO64)) = __ldg(src + c);
		}
	}
	for (int l = 1; l < TC_LAYERS; l++) {
		uint32_t cols = l == TC_LAYERS - 1 ? TC_OUT : TC_W, chunks = cols / 8u, sbo = chunks * 128u;
		const uint4 *src = reinterpret_cast<const uint4 *>(wn_g + (size_t)l * TC_W * TC_W);
		unsigned char *dst = sm + wn_off(l);
		for (uint32_t c = (uint32_t)tid; c < TC_W * chunks; c += 128u) {
			uint32_t r = c / chunks, kb = c % chunks;
			*reinterpret_cast<uint4 *>(dst + kmaj_off(r, kb * 8u, sbo)) = __ldg(src + c);
		}
	}
	if (tid == 0) {
		asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(bar), "r"(1u) : "memory");
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	if (warp == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
			:: "r"(smem_addr(slot)), "r"(TT_TMEM_COLS) : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
	}
	fence_async_smem();
	tc_before();
	__syncthreads();
	tc_after();
	const uint32_t tmem = *slot;
	const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
	const uint32_t base = smem_addr(sm);
	const uint32_t id_hidden = instr_desc(bf16, TC_W, TT_ROWS), id_out = instr_desc(bf16, TC_OUT, TT_ROWS);
	const uint32_t id_dw = instr_desc(bf16, TC_W, 64), id_dw_out = instr_desc(bf16, TC_OUT, 64);
	const uint32_t r = (uint32_t)tid; /* this thread's row of the tile, and its TMEM lane */
	unsigned char *xs = sm + TT_X_OFF, *ds = sm + TT_D_OFF, *dts = sm + TT_DT_OFF;
	uint32_t parity = 0;
	bool ok = true, first = true;
	float lsum = 0.0f;

	/* wait for the committed MMAs, then make the epilogue's view current */
	auto mma_wait = [&]() -> bool {
		bool got = bar_wait(bar, parity, TC_WAIT_LIMIT);
		parity ^= 1u;
		bool all = __syncthreads_and(got) != 0;
		tc_after();
		return all;
	};
	/* make this thread's shared-memory writes visible to the MMAs */
	auto publish = [&]() {
		fence_async_smem();
		tc_before();
		__syncthreads();
		tc_after();
	};

	for (uint32_t t = blockIdx.x; ok && t < tiles; t += gridDim.x) {
		const size_t gr = (size_t)t * TT_ROWS + r;
		/* ---- the tile's input: X (row r) and AT[0] (column r) ---- */
		{
			uint4 c[8];
			const uint4 *src = reinterpret_cast<const uint4 *>(x + gr * TC_W);
#pragma unroll
			for (int kb = 0; kb < 8; kb++)
				c[kb] = gr < n ? __ldg(src + kb) : make_uint4(0u, 0u, 0u, 0u);
			unsigned char *at = sm + TT_AT_OFF;
#pragma unroll
			for (int kb = 0; kb < 8; kb++) {
				*reinterpret_cast<uint4 *>(xs + kmaj_off(r, kb * 8u, TT_SBO64)) = c[kb];
				const uint32_t w4[4] = {c[kb].x, c[kb].y, c[kb].z, c[kb].w};
#pragma unroll
				for (int e = 0; e < 8; e++) {
					uint16_t h = (uint16_t)(w4[e >> 1] >> (16 * (e & 1)));
					*reinterpret_cast<uint16_t *>(at + kmaj_off((uint32_t)(kb * 8 + e), r, TT_SBO128)) = h;
				}
			}
		}
		publish();
		/* ---- forward ---- */
		for (int l = 0; l < TC_LAYERS && ok; l++) {
			const bool last = l == TC_LAYERS - 1;
			if (tid == 0) {
				for (uint32_t kc = 0; kc < 4; kc++)
					tc_mma(tmem, smem_desc(base + TT_X_OFF + kc * 256u, TC_LBO, TT_SBO64, 0u),
						smem_desc(base + l * TC_LAYER_BYTES + kc * 256u, TC_LBO, TT_SBO64, 0u),
						last ? id_out : id_hidden, kc > 0 ? 1u : 0u);
				tc_commit(bar);
			}
			ok = mma_wait();
			if (!ok)
				break;
			if (!last) {
				uint32_t v[64];
				tmem_ld64(lane_addr, v);
				tmem_wait_ld();
				unsigned char *at = sm + TT_AT_OFF + (uint32_t)(l + 1) * TT_TILE_BYTES;
#pragma unroll
				for (uint32_t kb = 0; kb < 8; kb++) {
					uint16_t h[8];
#pragma unroll
					for (int e = 0; e < 8; e++) {
						h[e] = bits_of<T>(float_to_half<T>(fmaxf(__uint_as_float(v[8 * kb + e]), 0.0f)));
						*reinterpret_cast<uint16_t *>(at + kmaj_off(8u * kb + (uint32_t)e, r, TT_SBO128)) = h[e];
					}
					*reinterpret_cast<uint4 *>(xs + kmaj_off(r, kb * 8u, TT_SBO64)) = pack8<T>(h);
				}
			} else {
				/* the loss and the output delta (columns 0..15, 0..2 non-zero) */
				uint32_t v[16];
				tmem_ld16(lane_addr, v);
				tmem_wait_ld();
				float4 tg = gr < n ? target[gr] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
				const float tv[3] = {tg.x, tg.y, tg.z};
				uint16_t h[16];
#pragma unroll
				for (int col = 0; col < 16; col++) {
					float d = 0.0f;
					if (col < 3 && gr < n) {
						float y = __uint_as_float(v[col]);
						float diff = y - tv[col];
						float den = y * y + 0.01f;
						lsum += diff * diff / den;
						d = 2.0f * diff / den / (float)n;
					}
					h[col] = bits_of<T>(float_to_half<T>(d));
					*reinterpret_cast<uint16_t *>(dts + kmaj_off((uint32_t)col, r, TT_SBO128)) = h[col];
				}
				uint16_t lo[8], hi[8];
#pragma unroll
				for (int e = 0; e < 8; e++) {
					lo[e] = h[e];
					hi[e] = h[8 + e];
				}
				*reinterpret_cast<uint4 *>(ds + kmaj_off(r, 0u, TT_SBO16)) = pack8<T>(lo);
				*reinterpret_cast<uint4 *>(ds + kmaj_off(r, 8u, TT_SBO16)) = pack8<T>(hi);
			}
			publish();
		}
		/* ---- backward ---- */
		for (int l = TC_LAYERS - 1; l >= 0 && ok; l--) {
			const uint32_t cols = l == TC_LAYERS - 1 ? TC_OUT : TC_W;
			const uint32_t sbo_d = cols / 8u * 128u;
			if (tid == 0) {
				/* dW[l] (+)= AT[l] x DT: M = 64 inputs, N = cols outputs, K = 128 rows */
				for (uint32_t kc = 0; kc < 8; kc++)
					tc_mma(tmem + TT_DW_COL(l),
						smem_desc(base + TT_AT_OFF + (uint32_t)l * TT_TILE_BYTES + kc * 256u, TC_LBO, TT_SBO128, 0u),
						smem_desc(base + TT_DT_OFF + kc * 256u, TC_LBO, TT_SBO128, 0u),
						l == TC_LAYERS - 1 ? id_dw_out : id_dw, (!first || kc > 0) ? 1u : 0u);
				/* the delta of the layer input: D x WN[l], M = 128, N = 64, K = cols */
				if (l > 0)
					for (uint32_t kc = 0; kc < cols / 16u; kc++)
						tc_mma(tmem, smem_desc(base + TT_D_OFF + kc * 256u, TC_LBO, sbo_d, 0u),
							smem_desc(base + wn_off(l) + kc * 256u, TC_LBO, sbo_d, 0u), id_hidden,
							kc > 0 ? 1u : 0u);
				tc_commit(bar);
			}
			ok = mma_wait();
			if (!ok || l == 0)
				break;
			uint32_t v[64];
			tmem_ld64(lane_addr, v);
			tmem_wait_ld();
			const unsigned char *at = sm + TT_AT_OFF + (uint32_t)l * TT_TILE_BYTES;
#pragma unroll
			for (uint32_t kb = 0; kb < 8; kb++) {
				uint16_t h[8];
#pragma unroll
				for (int e = 0; e < 8; e++) {
					uint32_t i = 8u * kb + (uint32_t)e;
					float av = half_to_float<T>(half_bits<T>(*reinterpret_cast<const uint16_t *>(
						at + kmaj_off(i, r, TT_SBO128))));
					float d = av > 0.0f ? __uint_as_float(v[i]) : 0.0f;
					h[e] = bits_of<T>(float_to_half<T>(d));
					*reinterpret_cast<uint16_t *>(dts + kmaj_off(i, r, TT_SBO128)) = h[e];
				}
				*reinterpret_cast<uint4 *>(ds + kmaj_off(r, kb * 8u, TT_SBO64)) = pack8<T>(h);
			}
			publish();
		}
		first = false;
	}
	if (!ok && tid == 0)
		atomicOr(err, 1u);
	tc_before();
	__syncthreads();
	tc_after();
	/* this block's dW: lanes 32w..32w+15 hold rows 16w..16w+15 */
	float *dst = partial + (size_t)blockIdx.x * TC_LAYERS * TC_W * TC_W;
	for (int l = 0; l < TC_LAYERS; l++) {
		const uint32_t cols = l == TC_LAYERS - 1 ? TC_OUT : TC_W;
		const uint32_t i = 16u * (uint32_t)warp + (uint32_t)lane;
		uint32_t v[64];
		if (cols == TC_W) {
			tmem_ld64(lane_addr + TT_DW_COL(l), v);
		} else {
			uint32_t w16[16];
			tmem_ld16(lane_addr + TT_DW_COL(l), w16);
#pragma unroll
			for (int j = 0; j < 16; j++)
				v[j] = w16[j];
#pragma unroll
			for (int j = 16; j < 64; j++)
				v[j] = 0u;
		}
		tmem_wait_ld();
		if (lane < 16) {
			float *row = dst + (size_t)l * TC_W * TC_W + (size_t)i * TC_W;
			const bool valid = ok && !first;
#pragma unroll
			for (int j = 0; j < 64; j += 4)
				*reinterpret_cast<float4 *>(row + j) = valid
					? make_float4(__uint_as_float(v[j]), __uint_as_float(v[j + 1]), __uint_as_float(v[j + 2]),
						__uint_as_float(v[j + 3]))
					: make_float4(0.0f, 0.0f, 0.0f, 0.0f);
		}
	}
	for (int off = 16; off > 0; off >>= 1)
		lsum += __shfl_down_sync(0xffffffffu, lsum, off);
	if (lane == 0)
		atomicAdd(loss_sum, lsum);
	tc_before();
	__syncthreads();
	tc_after();
	if (warp == 0)
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(TT_TMEM_COLS)
			: "memory");
}

template <class K>
void set_tc_smem(K kernel)
{
	KGR_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM));
}

/* cuTensorMapEncodeTiled, looked up once through the runtime (no link
 * against the driver library). */
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
		const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
		CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled()
{
	static EncodeTiledFn fn = nullptr;
	static std::once_flag once;
	std::call_once(once, [] {
		void *p = nullptr;
		cudaDriverEntryPointQueryResult q;
		if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
				cudaSuccess && q == cudaDriverEntryPointSuccess)
			fn = reinterpret_cast<EncodeTiledFn>(p);
		cudaGetLastError();
	});
	KGR_REQUIRE(fn, KGR_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
	return fn;
}

template <class K>
void set_train_smem(K kernel)
{
	KGR_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TT_SMEM));
}

} /* namespace */

void mlp_train_tc(const MlpParams &mp, const void *x, const float4 *target, uint32_t n, int grid, float *loss,
		cudaStream_t st, const uint32_t *n_dev)
{
	KGR_REQUIRE(((uintptr_t)x & 15u) == 0, KGR_ERR_INVALID_ARGUMENT, "inputs must be 16-byte aligned");
	if (mp.dtype == KGR_MLP_BF16) {
		static bool once = (set_train_smem(mlp_train_tc_kernel<__nv_bfloat16>), true);
		(void)once;
		mlp_train_tc_kernel<__nv_bfloat16><<<grid, 128, TT_SMEM, st>>>(static_cast<const __nv_bfloat16 *>(mp.wt),
			static_cast<const __nv_bfloat16 *>(mp.wn), static_cast<const __nv_bfloat16 *>(x), target, n, mp.partial,
			loss, n_dev, mp.tc_err);
	} else {
		static bool once = (set_train_smem(mlp_train_tc_kernel<__half>), true);
		(void)once;
		mlp_train_tc_kernel<__half><<<grid, 128, TT_SMEM, st>>>(static_cast<const __half *>(mp.wt),
			static_cast<const __half *>(mp.wn), static_cast<const __half *>(x), target, n, mp.partial, loss, n_dev,
			mp.tc_err);
	}
	KGR_CUDA(cudaGetLastError());
}

void mlp_infer_tc(const MlpParams &mp, const void *x, uint32_t n, float4 *out, uint32_t *err, cudaStream_t st,
		const uint32_t *n_dev, bool withhold_first)
{
	if (n == 0)
		return;
	KGR_REQUIRE(((uintptr_t)x & 15u) == 0, KGR_ERR_INVALID_ARGUMENT, "inputs must be 16-byte aligned");
	/* the input as a 2-D tensor: 64 elements (128 bytes) per row, n rows;
	 * one box is a 128 x 64 tile, swizzled by 128 bytes on its way in */
	CUtensorMap map;
	cuuint64_t dims[2] = {TC_W, n};
	cuuint64_t strides[1] = {TC_W * 2};
	cuuint32_t box[2] = {TC_W, TC_ROWS};
	cuuint32_t estr[2] = {1, 1};
	CUresult r = encode_tiled()(&map,
		mp.dtype == KGR_MLP_BF16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2,
		const_cast<void *>(x), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
		CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
	KGR_REQUIRE(r == CUDA_SUCCESS, KGR_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
	/* two CTAs fit an SM (106 KB of shared memory, 256 TMEM columns and 512
	 * threads at 64 registers each); a CTA walks TC_CHAINS tiles at a time */
	long long tiles = ((long long)n + TC_ROWS - 1) / TC_ROWS;
	long long blocks = (tiles + TC_CHAINS - 1) / TC_CHAINS;
	long long cap = (long long)device_sm_count() * 2;
	int grid = (int)(blocks < cap ? blocks : cap);
	if (mp.dtype == KGR_MLP_BF16) {
		static bool once = (set_tc_smem(mlp_infer_tc_kernel<__nv_bfloat16>), true);
		(void)once;
		mlp_infer_tc_kernel<__nv_bfloat16><<<grid, TC_THREADS, TC_SMEM, st>>>(
			static_cast<const __nv_bfloat16 *>(mp.wt), map, n, out, n_dev, err, withhold_first ? 1u : 0u);
	} else {
		static bool once = (set_tc_smem(mlp_infer_tc_kernel<__half>), true);
		(void)once;
		mlp_infer_tc_kernel<__half><<<grid, TC_THREADS, TC_SMEM, st>>>(static_cast<const __half *>(mp.wt), map, n, out,
			n_dev, err, withhold_first ? 1u : 0u);
	}
	KGR_CUDA(cudaGetLastError());
}

} /* namespace kgr */

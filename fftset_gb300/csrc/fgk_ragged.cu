/* Ragged batches: many transforms of different sizes in one persistent
 * launch.
 *
 * The host groups the items by size (largest first) into chunks of up to G
 * same-size items; CTAs (512 threads, 227 KB of shared memory, one per SM)
 * claim chunks from an atomic counter. A chunk's items run side by side, one
 * group of threads each, as ping-pong Stockham chains in shared memory: each
 * stage reads one buffer and writes the other, one butterfly per thread at a
 * time (only one radix worth of values is live, so the runtime-dispatched
 * radix costs no spills), one barrier per stage. Plans (chain, twiddles,
 * modulation factors) are the fftset's own plans for each size, so all sizes
 * share the fftset's twiddle tables. Items too large for two shared buffers
 * go through the four-step passes (fgk_fourstep.cu) with an item list. */
#include <cuda_runtime.h>
#include <stdint.h>
#include "fgk.h"
#include "fgk_pingpong.cuh"

namespace fgk {

__global__ void __launch_bounds__(512, 1)
    ragged_kernel(const fgk_plan *__restrict__ plans, const fgk_rg_chunk *__restrict__ chunks, uint32_t nchunks,
                  const fgk_rg_item *__restrict__ items, int *counter, int op, const float *in_base, float *out_base)
{
	extern __shared__ float2 smem[];
	__shared__ uint32_t cur;
	for (;;) {
		if (threadIdx.x == 0)
			cur = (uint32_t)atomicAdd(counter, 1);
		__syncthreads();
		const uint32_t c = cur;
		if (c >= nchunks)
			break;
		const fgk_rg_chunk ch = chunks[c];
		const fgk_plan *pl = plans + ch.plan;
		const int L = (int)pl->L;
		const bool freq = pl->modulation == FGK_MOD_FREQOFF;
		const float2 *mod = (const float2 *)pl->modtw;
		const int T = (int)ch.tg;
		const int g = (int)threadIdx.x / T;
		const int tid = (int)threadIdx.x - g * T;
		const bool active = g < (int)ch.n;
		const int slots = rslots(L);
		float2 *buf0 = smem + (size_t)(active ? g : 0) * 2 * slots;
		float2 *buf1 = buf0 + slots;
		const fgk_rg_item it = active ? items[ch.first + g] : fgk_rg_item{0, 0};
		const float *x = in_base + it.in_off;
		float *y = out_base + it.out_off;

		/* prologue: the sequence to transform, natural order */
		if (active) {
			if (op != FGK_OP_INVERSE) {
				if (freq) {
					for (int i = tid; i < L; i += T)
						buf0[rslot(i)] = cmul(make_float2(__ldcs(x + i), -__ldcs(x + L + i)), __ldg(mod + i));
				} else {
					const float2 *x2 = reinterpret_cast<const float2 *>(x);
					for (int i = tid; i < L; i += T)
						buf0[rslot(i)] = __ldcs(x2 + i);
				}
			} else {
				const float2 *X = reinterpret_cast<const float2 *>(x);
				if (freq) {
					const int half = L >> 1;
					for (int m = tid; m < half; m += T) {
						buf0[rslot(m)] = conjf2(__ldcs(X + 2 * m));
						buf0[rslot(L - 1 - m)] = __ldcs(X + 2 * m + 1);
					}
					if ((L & 1) && tid == 0)
						buf0[rslot(half)] = conjf2(__ldcs(X + L - 1));
				} else {
					for (int i = tid; i < L; i += T)
						buf0[rslot(i)] = conjf2(__ldcs(X + i));
				}
			}
		}
		__syncthreads();
		const float2 *src = rg_chain(pl, buf0, buf1, active, tid, T, [] { __syncthreads(); });
		/* epilogue from src */
		if (active) {
			if (op == FGK_OP_INVERSE) {
				if (freq) {
					for (int i = tid; i < L; i += T) {
						const float2 r = cmul(src[rslot(i)], __ldg(mod + i));
						__stcs(y + i, r.x);
						__stcs(y + L + i, r.y);
					}
				} else {
					float2 *y2 = reinterpret_cast<float2 *>(y);
					for (int i = tid; i < L; i += T)
						__stcs(y2 + i, conjf2(src[rslot(i)]));
				}
			} else if (freq) {
				float2 *y2 = reinterpret_cast<float2 *>(y);
				const int half = L >> 1;
				for (int m = tid; m < half; m += T) {
					__stcs(y2 + 2 * m, src[rslot(m)]);
					__stcs(y2 + 2 * m + 1, conjf2(src[rslot(L - 1 - m)]));
				}
				if ((L & 1) && tid == 0)
					__stcs(y2 + L - 1, src[rslot(half)]);
			} else {
				float2 *y2 = reinterpret_cast<float2 *>(y);
				for (int i = tid; i < L; i += T)
					__stcs(y2 + i, src[rslot(i)]);
			}
		}
		__syncthreads(); /* buffers and `cur` are reused by the next chunk */
	}
}

} /* namespace fgk */

extern "C" size_t fgk_ragged_smem_bytes(void)
{
	return 232448 - 1024; /* the opt-in limit less room for static shared memory */
}

extern "C" int fgk_launch_ragged(const fgk_plan *plans_dev, const fgk_rg_chunk *chunks_dev, uint32_t nchunks,
                                 const fgk_rg_item *items_dev, int *counter_dev, int op, const float *in_base,
                                 float *out_base, int num_sms, void *stream)
{
	using namespace fgk;
	const size_t smem = fgk_ragged_smem_bytes();
	cudaError_t e;
	if (nchunks == 0)
		return 0;
	if ((e = cudaFuncSetAttribute((const void *)ragged_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
	                              (int)smem)) != cudaSuccess)
		return (int)e;
	if ((e = cudaMemsetAsync(counter_dev, 0, sizeof(int), (cudaStream_t)stream)) != cudaSuccess)
		return (int)e;
	const uint32_t grid = (uint32_t)num_sms < nchunks ? (uint32_t)num_sms : nchunks;
	ragged_kernel<<<grid, 512, smem, (cudaStream_t)stream>>>(plans_dev, chunks_dev, nchunks, items_dev, counter_dev, op,
	                                                         in_base, out_base);
	return (int)cudaGetLastError();
}

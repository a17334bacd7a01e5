/* Overlap-add block convolution (fftset_fft_conv_overlap_add): the two
 * gather kernels around one batched fftset_fft_conv.
 *
 * A signal of n samples (real samples for FREQ_OFFSET_REAL, complex ones
 * for COMPLEX) is cut into blocks of B samples; each block is zero-padded to
 * the transform length N (2 complex_bins reals, or complex_bins complex
 * points) and convolved with a kernel of K <= N - B + 1 taps, so the
 * negacyclic (cyclic) wrap of the block convolution only ever meets zeros
 * and each block's result is its linear convolution. Output sample t is the
 * sum over blocks b with 0 <= t - b B < B + K - 1 of block b's result at
 * t - b B: a gather, so every output is written once, with no atomics.
 * Elements are float (E = 1) or float2 (E = 2). */
#include <cuda_runtime.h>
#include <stdint.h>

#include "fgk.h"

namespace fgk {

/* blocks[b][i] = in[b B + i] for i < B and b B + i < n, else 0. A CTA takes
 * whole blocks (rows of N elements), so no element index is divided. */
template <class T>
__global__ void ola_split(const T *__restrict__ in, uint64_t n, uint32_t B, uint32_t N, uint32_t nblocks, T *blocks)
{
	const T zero{};
	for (uint64_t b = blockIdx.x; b < nblocks; b += gridDim.x) {
		const uint64_t base = b * B;
		const uint32_t valid = base + B <= n ? B : (uint32_t)(n - base); /* base < n for every block */
		T *row = blocks + b * N;
		for (uint32_t i = threadIdx.x; i < N; i += blockDim.x)
			__stcs(row + i, i < valid ? __ldcs(in + base + i) : zero);
	}
}

/* out[t] = sum_b ys[b][t - b B] over 0 <= t - b B < span (span = B + K - 1).
 * A CTA takes whole chunks of B outputs (chunk c: t = c B + i0), to which
 * block c contributes element i0, block c - 1 element i0 + B, and so on
 * while the element lies within span. */
template <class T>
__global__ void ola_merge(const T *__restrict__ ys, uint32_t B, uint32_t N, uint32_t span, uint32_t nblocks,
                          uint64_t nout, T *out)
{
	const uint64_t nchunks = (nout + B - 1) / B;
	for (uint64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
		const uint64_t t0 = c * B;
		const uint32_t m = t0 + B <= nout ? B : (uint32_t)(nout - t0);
		for (uint32_t i0 = threadIdx.x; i0 < m; i0 += blockDim.x) {
			uint64_t b = c, i = i0;
			if (b >= nblocks) { /* the tail past the last block's start */
				i += (b - (nblocks - 1)) * (uint64_t)B;
				b = nblocks - 1;
			}
			T acc{};
			while (i < span) {
				const T v = __ldcs(ys + b * N + i);
				if constexpr (sizeof(T) == sizeof(float)) {
					acc += v;
				} else {
					acc.x += v.x;
					acc.y += v.y;
				}
				if (b == 0)
					break;
				b--;
				i += B;
			}
			__stcs(out + t0 + i0, acc);
		}
	}
}

} /* namespace fgk */

/* CTAs for `rows` rows (blocks or output chunks), at most 16 per SM */
static unsigned ola_grid(uint64_t rows, int num_sms)
{
	const uint64_t cap = (uint64_t)num_sms * 16;
	return (unsigned)(rows < cap ? (rows ? rows : 1) : cap);
}

extern "C" int fgk_launch_ola_split(const float *in, uint64_t n, uint32_t B, uint32_t N, uint32_t nblocks,
                                    int complex_samples, float *blocks, int num_sms, void *stream)
{
	using namespace fgk;
	const unsigned grid = ola_grid(nblocks, num_sms);
	if (complex_samples)
		ola_split<float2><<<grid, 256, 0, (cudaStream_t)stream>>>(reinterpret_cast<const float2 *>(in), n, B, N,
		                                                         nblocks, reinterpret_cast<float2 *>(blocks));
	else
		ola_split<float><<<grid, 256, 0, (cudaStream_t)stream>>>(in, n, B, N, nblocks, blocks);
	fgk_count_launch();
	return (int)cudaGetLastError();
}

extern "C" int fgk_launch_ola_merge(const float *ys, uint32_t B, uint32_t N, uint32_t span, uint32_t nblocks,
                                    uint64_t nout, int complex_samples, float *out, int num_sms, void *stream)
{
	using namespace fgk;
	const unsigned grid = ola_grid((nout + B - 1) / B, num_sms);
	if (complex_samples)
		ola_merge<float2><<<grid, 256, 0, (cudaStream_t)stream>>>(reinterpret_cast<const float2 *>(ys), B, N, span,
		                                                         nblocks, nout, reinterpret_cast<float2 *>(out));
	else
		ola_merge<float><<<grid, 256, 0, (cudaStream_t)stream>>>(ys, B, N, span, nblocks, nout, out);
	fgk_count_launch();
	return (int)cudaGetLastError();
}

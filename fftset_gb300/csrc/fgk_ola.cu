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

/* blocks[b][i] = in[b B + i] for i < B and b B + i < n, else 0 */
template <class T>
__global__ void ola_split(const T *__restrict__ in, uint64_t n, uint32_t B, uint32_t N, uint32_t nblocks, T *blocks)
{
	const uint64_t total = (uint64_t)nblocks * N;
	const T zero{};
	for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
	     e += (uint64_t)gridDim.x * blockDim.x) {
		const uint64_t b = e / N;
		const uint32_t i = (uint32_t)(e - b * N);
		const uint64_t src = b * B + i;
		blocks[e] = (i < B && src < n) ? __ldcs(in + src) : zero;
	}
}

/* out[t] = sum_b ys[b][t - b B] over 0 <= t - b B < span (span = B + K - 1) */
template <class T>
__global__ void ola_merge(const T *__restrict__ ys, uint32_t B, uint32_t N, uint32_t span, uint32_t nblocks,
                          uint64_t nout, T *out)
{
	for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nout;
	     t += (uint64_t)gridDim.x * blockDim.x) {
		uint64_t b = t / B;
		if (b >= nblocks)
			b = nblocks - 1;
		T acc{};
		for (;;) {
			const uint64_t i = t - b * B;
			if (i >= span)
				break;
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
		}
		__stcs(out + t, acc);
	}
}

} /* namespace fgk */

static unsigned ola_grid(uint64_t work, int num_sms)
{
	const uint64_t per = 256;
	uint64_t g = (work + per - 1) / per;
	const uint64_t cap = (uint64_t)num_sms * 16;
	return (unsigned)(g < cap ? (g ? g : 1) : cap);
}

extern "C" int fgk_launch_ola_split(const float *in, uint64_t n, uint32_t B, uint32_t N, uint32_t nblocks,
                                    int complex_samples, float *blocks, int num_sms, void *stream)
{
	using namespace fgk;
	const unsigned grid = ola_grid((uint64_t)nblocks * N, num_sms);
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
	const unsigned grid = ola_grid(nout, num_sms);
	if (complex_samples)
		ola_merge<float2><<<grid, 256, 0, (cudaStream_t)stream>>>(reinterpret_cast<const float2 *>(ys), B, N, span,
		                                                         nblocks, nout, reinterpret_cast<float2 *>(out));
	else
		ola_merge<float><<<grid, 256, 0, (cudaStream_t)stream>>>(ys, B, N, span, nblocks, nout, out);
	fgk_count_launch();
	return (int)cudaGetLastError();
}

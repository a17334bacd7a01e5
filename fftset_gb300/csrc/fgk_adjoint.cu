/* Adjoint of the convolution with respect to the kernel taps.
 *
 * For y_b = conv(x_b, K) over a batch (fftset_fft_conv, K the spectrum of
 * taps h from fftset_fft_conv_get_kernel) and upstream gradients g_b =
 * dLoss/dy_b, the gradient with respect to h is
 *     dh = inverse( sum_b G_b conj(X_b) ),
 * G_b and X_b the forward spectra of g_b and x_b (for FREQ_OFFSET_REAL the
 * half-bin-offset spectra; the library's inverse is unnormalised, which is
 * the factor complex_bins the convolution carries). In the time domain this
 * is complex_bins times the sum over b of the negacyclic (FREQ_OFFSET_REAL)
 * or cyclic (COMPLEX) cross-correlation of g_b with x_b.
 *
 * The host runs the plan's batched forward transforms of g and x into
 * scratch (the tuned compiled kernels); kg_spec_partial sums G conj(X) over
 * chunks of blocks (bin-parallel, coalesced over bins), kg_reduce sums the
 * chunk partials, and the plan's inverse turns the sum into dh. On GB300 this
 * beat a kernel that transformed g_b and x_b together in shared memory and
 * accumulated in registers (4096 bins x 2048 blocks: 0.140 ms against
 * 0.215 ms): the batched forward kernels are much faster than that kernel's
 * generic shared-memory chains, and the extra scratch traffic is cheap. */
#include <cuda_runtime.h>
#include <stdint.h>
#include "fgk.h"
#include "fgk_codelets.cuh"

namespace fgk {

/* partials[c][k] = sum over blocks b of chunk c of S[b][k] conj(X[b][k]) */
__global__ void kg_spec_partial(const float2 *__restrict__ S, const float2 *__restrict__ X, size_t stride,
                                uint32_t count, uint32_t L, uint32_t chunk, float2 *partials)
{
	const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= L)
		return;
	const uint64_t b0 = (uint64_t)blockIdx.y * chunk;
	const uint64_t b1 = b0 + chunk < count ? b0 + chunk : count;
	float2 a = make_float2(0.f, 0.f);
	for (uint64_t b = b0; b < b1; b++)
		a = cadd(a, cmulc(__ldcs(S + b * stride + k), __ldcs(X + b * stride + k)));
	partials[(uint64_t)blockIdx.y * L + k] = a;
}

/* out = sum over the P partials, in natural order (pack == 0) or in the
 * FREQ_OFFSET_REAL forward layout from packed-sequence bins (pack == 1).
 * A CTA covers KG_BINS bins with KG_SPLIT threads per bin, each summing every
 * KG_SPLIT-th partial (a warp reads 128-byte runs of two rows), then the
 * KG_SPLIT sums of a bin are added in shared memory in a fixed order.
 * Launched as a programmatic dependent of the kernel that wrote the
 * partials (it waits for it before the first read) and lets the inverse
 * transform after it be scheduled as it starts. */
constexpr int KG_BINS = 16, KG_SPLIT = 32;
__global__ void __launch_bounds__(KG_BINS *KG_SPLIT) kg_reduce(const float2 *__restrict__ partials, uint32_t P,
                                                              uint32_t L, int pack, float2 *out)
{
	__shared__ float2 part[KG_SPLIT][KG_BINS];
	asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
	asm volatile("griddepcontrol.wait;" ::: "memory");
	const uint32_t lane = threadIdx.x % KG_BINS, r0 = threadIdx.x / KG_BINS;
	const uint32_t i = blockIdx.x * KG_BINS + lane;
	float2 a = make_float2(0.f, 0.f);
	if (i < L) {
#pragma unroll 4
		for (uint32_t p = r0; p < P; p += KG_SPLIT)
			a = cadd(a, __ldcg(partials + (uint64_t)p * L + i));
	}
	part[r0][lane] = a;
	__syncthreads();
	if (r0 != 0 || i >= L)
		return;
#pragma unroll
	for (int r = 1; r < KG_SPLIT; r++)
		a = cadd(a, part[r][lane]);
	if (!pack)
		out[i] = a;
	else if (i < ((L + 1) >> 1))
		out[2 * i] = a;
	else
		out[2 * (L - 1 - i) + 1] = conjf2(a);
}

} /* namespace fgk */

extern "C" int fgk_launch_kgrad_spec(const float *S, const float *X, size_t stride, uint32_t count, uint32_t L,
                                     uint32_t chunk, float *partials, void *stream)
{
	using namespace fgk;
	const uint32_t nch = (count + chunk - 1) / chunk;
	dim3 grid((L + 255) / 256, nch);
	kg_spec_partial<<<grid, 256, 0, (cudaStream_t)stream>>>(reinterpret_cast<const float2 *>(S),
	                                                        reinterpret_cast<const float2 *>(X), stride / 2, count, L,
	                                                        chunk, reinterpret_cast<float2 *>(partials));
	fgk_count_launch();
	return (int)cudaGetLastError();
}

extern "C" int fgk_launch_kgrad_reduce(const float *partials, uint32_t P, uint32_t L, int pack, float *out,
                                       void *stream)
{
	using namespace fgk;
	cudaLaunchConfig_t cfg = {};
	cudaLaunchAttribute at[1];
	at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
	at[0].val.programmaticStreamSerializationAllowed = 1;
	cfg.gridDim = dim3((L + KG_BINS - 1) / KG_BINS);
	cfg.blockDim = dim3(KG_BINS * KG_SPLIT);
	cfg.stream = (cudaStream_t)stream;
	cfg.attrs = at;
	cfg.numAttrs = 1;
	const cudaError_t le = cudaLaunchKernelEx(&cfg, kg_reduce, reinterpret_cast<const float2 *>(partials), P, L, pack,
	                                          reinterpret_cast<float2 *>(out));
	fgk_count_launch();
	return le != cudaSuccess ? (int)le : (int)cudaGetLastError();
}

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
 * Fused path (kg_fused): each CTA runs G groups of T threads; a group takes
 * blocks b = group, group + P, ... and for each one transforms g_b and x_b in
 * shared memory (runtime-chain ping-pong stages, three buffers) and adds
 * G_b[i] conj(X_b[i]) into registers (bin i = tid + k T, k < 16). Each
 * block's g_b and x_b cross HBM once; nothing per block is written. At the
 * end every group writes its partial spectrum; kg_reduce sums the P
 * partials into the layout the forward transform writes (the FREQ_OFFSET_REAL
 * packing X[2m] = W[m], X[2m+1] = conj W[L-1-m] included), and the plan's
 * inverse turns that into dh.
 *
 * Sizes whose three buffers do not fit shared memory take the unfused
 * path: batched forward transforms of g and x into scratch, kg_spec_partial
 * (column sums of G conj(X) over chunks of blocks) and kg_reduce. */
#include <cuda_runtime.h>
#include <stdint.h>
#include "fgk.h"
#include "fgk_pingpong.cuh"

namespace fgk {

constexpr int KG_ACC = 16;      /* accumulated bins per thread: L <= 16 T */
constexpr int KG_THREADS = 512; /* threads per CTA at most */

__device__ __forceinline__ void kg_bar(int g, int T)
{
	asm volatile("bar.sync %0, %1;" ::"r"(g + 1), "r"(T) : "memory");
}

/* natural-order input of the plan's forward chain: the block itself
 * (COMPLEX) or conj(x[i] + j x[L+i]) e^{-j pi i/(2L)} (FREQ_OFFSET_REAL);
 * eight loads per thread in flight */
template <bool FREQ>
__device__ __forceinline__ void kg_prologue(const fgk_plan *pl, float2 *buf, const float *x, int L, int tid, int T)
{
	if (FREQ) {
		const float2 *mod = (const float2 *)pl->modtw;
		batched_copy<8>(
		    L, tid, T,
		    [&](int i) { return cmul(make_float2(__ldcs(x + i), -__ldcs(x + L + i)), __ldg(mod + i)); },
		    [&](int i, float2 v) { buf[rslot(i)] = v; });
	} else {
		const float2 *x2 = reinterpret_cast<const float2 *>(x);
		batched_copy<8>(
		    L, tid, T, [&](int i) { return __ldcs(x2 + i); }, [&](int i, float2 v) { buf[rslot(i)] = v; });
	}
}

/* Both blocks of a step (g_b into b0, x_b into b2) are loaded before either
 * transform runs, so their loads overlap; g_b's chain then runs over b0/b1
 * and x_b's over b2 and whichever of b0/b1 does not hold G_b. */
template <bool FREQ>
__global__ void __launch_bounds__(KG_THREADS, 1)
    kg_fused(const fgk_plan *__restrict__ pl, const float *gr, size_t g_stride, const float *x, size_t x_stride,
             uint32_t count, int T, int G, float2 *partials)
{
	extern __shared__ float2 smem[];
	const int L = (int)pl->L;
	const int g = (int)threadIdx.x / T;
	const int tid = (int)threadIdx.x - g * T;
	const int slots = rslots(L);
	float2 *b0 = smem + (size_t)g * 3 * slots;
	float2 *b1 = b0 + slots;
	float2 *b2 = b1 + slots;
	float2 acc[KG_ACC];
#pragma unroll
	for (int k = 0; k < KG_ACC; k++)
		acc[k] = make_float2(0.f, 0.f);
	auto sync = [&] { kg_bar(g, T); };
	const uint64_t P = (uint64_t)gridDim.x * G;
	for (uint64_t b = (uint64_t)blockIdx.x * G + g; b < count; b += P) {
		kg_prologue<FREQ>(pl, b0, gr + b * g_stride, L, tid, T);
		kg_prologue<FREQ>(pl, b2, x + b * x_stride, L, tid, T);
		sync();
		float2 *W = rg_chain(pl, b0, b1, true, tid, T, sync);
		const float2 *X = rg_chain(pl, b2, W == b0 ? b1 : b0, true, tid, T, sync);
#pragma unroll
		for (int k = 0; k < KG_ACC; k++) {
			const int i = tid + k * T;
			if (i < L)
				acc[k] = cadd(acc[k], cmulc(W[rslot(i)], X[rslot(i)]));
		}
		sync(); /* the buffers are reused by the next block */
	}
	float2 *part = partials + ((uint64_t)blockIdx.x * G + g) * L;
#pragma unroll
	for (int k = 0; k < KG_ACC; k++) {
		const int i = tid + k * T;
		if (i < L)
			part[i] = acc[k];
	}
}

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
 * FREQ_OFFSET_REAL forward layout from packed-sequence bins (pack == 1) */
__global__ void kg_reduce(const float2 *__restrict__ partials, uint32_t P, uint32_t L, int pack, float2 *out)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= L)
		return;
	float2 a = make_float2(0.f, 0.f);
	for (uint32_t p = 0; p < P; p++)
		a = cadd(a, partials[(uint64_t)p * L + i]);
	if (!pack)
		out[i] = a;
	else if (i < ((L + 1) >> 1))
		out[2 * i] = a;
	else
		out[2 * (L - 1 - i) + 1] = conjf2(a);
}

} /* namespace fgk */

/* Launch shape of the fused path for plan p (host copy): threads per group,
 * groups per CTA and the dynamic shared memory; 0 when L does not fit. */
extern "C" int fgk_kgrad_fused_shape(const fgk_plan *p, uint32_t *T, uint32_t *G, size_t *smem)
{
	using namespace fgk;
	uint32_t s, w = 32;
	const size_t per = 3 * (size_t)rslots((int)p->L) * sizeof(float2);
	const size_t limit = 232448 - 1024;
	for (s = 0; s < p->fwd.nstages; s++) {
		const uint32_t nbf = p->L / p->fwd.st[s].radix;
		if (nbf > w)
			w = nbf;
	}
	while (w * KG_ACC < p->L)
		w *= 2;
	w = (w + 31) & ~31u;
	if (w > KG_THREADS || per > limit || p->L > (uint32_t)KG_ACC * w)
		return 0;
	uint32_t g = KG_THREADS / w;
	if (g > 15)
		g = 15; /* named barriers 1..15 */
	if (g * per > limit)
		g = (uint32_t)(limit / per);
	*T = w;
	*G = g;
	*smem = g * per;
	return 1;
}

extern "C" int fgk_launch_kgrad_fused(const fgk_plan *p, const float *grad_out, size_t g_stride, const float *x,
                                      size_t x_stride, uint32_t count, uint32_t grid, float *partials, void *stream)
{
	using namespace fgk;
	uint32_t T, G;
	size_t smem;
	cudaError_t e;
	if (!fgk_kgrad_fused_shape(p, &T, &G, &smem))
		return (int)cudaErrorInvalidValue;
	auto k = p->modulation == FGK_MOD_FREQOFF ? kg_fused<true> : kg_fused<false>;
	if ((e = cudaFuncSetAttribute((const void *)k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
	    cudaSuccess)
		return (int)e;
	k<<<grid, T * G, smem, (cudaStream_t)stream>>>(p->dev, grad_out, g_stride, x, x_stride, count, (int)T, (int)G,
	                                               reinterpret_cast<float2 *>(partials));
	return (int)cudaGetLastError();
}

extern "C" int fgk_launch_kgrad_spec(const float *S, const float *X, size_t stride, uint32_t count, uint32_t L,
                                     uint32_t chunk, float *partials, void *stream)
{
	using namespace fgk;
	const uint32_t nch = (count + chunk - 1) / chunk;
	dim3 grid((L + 255) / 256, nch);
	kg_spec_partial<<<grid, 256, 0, (cudaStream_t)stream>>>(reinterpret_cast<const float2 *>(S),
	                                                        reinterpret_cast<const float2 *>(X), stride / 2, count, L,
	                                                        chunk, reinterpret_cast<float2 *>(partials));
	return (int)cudaGetLastError();
}

extern "C" int fgk_launch_kgrad_reduce(const float *partials, uint32_t P, uint32_t L, int pack, float *out,
                                       void *stream)
{
	using namespace fgk;
	kg_reduce<<<(L + 63) / 64, 64, 0, (cudaStream_t)stream>>>(reinterpret_cast<const float2 *>(partials), P, L, pack,
	                                                          reinterpret_cast<float2 *>(out));
	return (int)cudaGetLastError();
}

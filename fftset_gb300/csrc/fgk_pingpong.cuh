/* Runtime-chain Stockham stages between two shared-memory buffers, used by
 * the kernels whose transform size is known only at run time (ragged
 * batches, the convolution adjoint).
 *
 * A stage reads buffer `src` and writes buffer `dst`; each thread runs its
 * butterflies j = tid, tid + T, ... one at a time, so only one radix worth of
 * values is live and the runtime-dispatched radix costs no spills. One
 * barrier per stage (the caller's) separates the stages. Shared-memory slot
 * of element i is i + i/16 (rslot), which spreads the strided accesses of a
 * stage over the banks. */
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "fgk.h"
#include "fgk_codelets.cuh"

namespace fgk {

#define FGKR_RADIX_SWITCH(r, CALL)                                  \
	switch (r) {                                                    \
	case 2: { constexpr int R_ = 2; CALL; } break;                  \
	case 3: { constexpr int R_ = 3; CALL; } break;                  \
	case 4: { constexpr int R_ = 4; CALL; } break;                  \
	case 5: { constexpr int R_ = 5; CALL; } break;                  \
	case 6: { constexpr int R_ = 6; CALL; } break;                  \
	case 8: { constexpr int R_ = 8; CALL; } break;                  \
	case 10: { constexpr int R_ = 10; CALL; } break;                \
	case 12: { constexpr int R_ = 12; CALL; } break;                \
	case 15: { constexpr int R_ = 15; CALL; } break;                \
	default: { constexpr int R_ = 16; CALL; } break;                \
	}

__device__ __forceinline__ int rslot(int i) { return i + (i >> 4); }

/* float2 slots of one padded buffer of L elements */
__host__ __device__ __forceinline__ int rslots(int L) { return L + L / 16 + 1; }

/* one stage, src -> dst, this thread's butterflies j = tid, tid + T, ... */
template <int R>
__device__ __forceinline__ void rg_stage(const float2 *src, float2 *dst, int L, int ns, const float2 *__restrict__ tw,
                                         int tid, int T)
{
	const int nbf = L / R;
	for (int j = tid; j < nbf; j += T) {
		float2 v[R];
#pragma unroll
		for (int p = 0; p < R; p++)
			v[p] = src[rslot(j + p * nbf)];
		const int k = j % ns;
		if (ns > 1) {
			const float2 *t = tw + k * (R - 1);
#pragma unroll
			for (int p = 1; p < R; p++)
				v[p] = cmul(v[p], __ldg(t + p - 1));
		}
		Radix<R>::run(v);
		const int base = (j - k) * R + k;
#pragma unroll
		for (int q = 0; q < R; q++)
			dst[rslot(base + q * ns)] = v[q];
	}
}

/* n elements from ld(i) to st(i, v), this thread's i = tid, tid + T, ...,
 * U loads in flight per thread: HBM needs tens of KB in flight per SM, which
 * one dependent load per loop iteration does not provide. */
template <int U, class Ld, class St>
__device__ __forceinline__ void batched_copy(int n, int tid, int T, Ld &&ld, St &&st)
{
	for (int base = tid; base < n; base += U * T) {
		float2 v[U];
#pragma unroll
		for (int u = 0; u < U; u++) {
			const int i = base + u * T;
			if (i < n)
				v[u] = ld(i);
		}
#pragma unroll
		for (int u = 0; u < U; u++) {
			const int i = base + u * T;
			if (i < n)
				st(i, v[u]);
		}
	}
}

/* The plan's forward chain over buffers a/b, starting from a (which holds
 * the natural-order input). Returns the buffer that holds the natural-order
 * DFT. `sync` is the group's barrier, called after every stage. */
template <class Sync>
__device__ __forceinline__ float2 *rg_chain(const fgk_plan *pl, float2 *a, float2 *b, bool active, int tid, int T,
                                            Sync &&sync)
{
	const int n = (int)pl->fwd.nstages;
	const int L = (int)pl->L;
	const float2 *tw = (const float2 *)pl->tw;
	float2 *src = a, *dst = b;
	for (int s = 0; s < n; s++) {
		const fgk_stage st = pl->fwd.st[s];
		if (active)
			FGKR_RADIX_SWITCH(st.radix, (rg_stage<R_>(src, dst, L, (int)st.ns, tw + st.tw_off, tid, T)));
		sync();
		float2 *t = src;
		src = dst;
		dst = t;
	}
	return src;
}

} /* namespace fgk */

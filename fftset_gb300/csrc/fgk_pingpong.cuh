/* Helpers of the kernels whose transform size is known only at run time
 * (the ragged task kernel, the four-step passes): the runtime radix switch,
 * the padded shared-memory slot of element i (i + i/16, which spreads a
 * stage's strided accesses over the banks) and a copy loop that keeps eight
 * loads per thread in flight. */
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
	case 9: { constexpr int R_ = 9; CALL; } break;                  \
	case 10: { constexpr int R_ = 10; CALL; } break;                \
	case 12: { constexpr int R_ = 12; CALL; } break;                \
	case 15: { constexpr int R_ = 15; CALL; } break;                \
	default: { constexpr int R_ = 16; CALL; } break;                \
	}

__device__ __forceinline__ int rslot(int i) { return i + (i >> 4); }

/* float2 slots of one padded buffer of L elements */
__host__ __device__ __forceinline__ int rslots(int L) { return L + L / 16 + 1; }

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

} /* namespace fgk */

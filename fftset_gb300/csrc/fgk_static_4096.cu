/* Compile-time kernels for FREQ_OFFSET_REAL, 4096 bins (the batched
 * differentiable convolution workload): 16^3, 256 threads per transform.
 * SCfg<modulation, L, T, G, twiddles-from-global, mode, radices...> (mode 0
 * in place, 1 in place with bulk-copy input, 2 ping-pong). The first
 * variant that implements an op is its default: the order is the measured
 * one, fastest first (2048 and 16384 blocks on a GB300: V0 0.056 / 0.342 ms
 * for the convolution, V1 0.064 / 0.375, V3 0.070 / 0.479, V2 0.086 /
 * 0.549); the chain is a palindrome, so its twiddles are staged once. */
#include "fgk_static.cuh"

namespace fgk {
using V0 = SCfg<FGK_MOD_FREQOFF, 4096, 256, 2, 0, 0, 16, 16, 16>;
using V1 = SCfg<FGK_MOD_FREQOFF, 4096, 256, 3, 0, 0, 16, 16, 16>;
using V2 = SCfg<FGK_MOD_FREQOFF, 4096, 256, 2, 1, 1, 16, 16, 16>;
using V3 = SCfg<FGK_MOD_FREQOFF, 4096, 256, 1, 0, 2, 16, 16, 16>;

int static_entries_4096(const StaticEntry **out)
{
	static StaticEntry t[4];
	static bool init = false;
	if (!init) {
		t[0] = make_entry<V0, OPS_ALL>();
		t[1] = make_entry<V1, OPS_CONV_CORR>();
		t[2] = make_entry<V2, OPS_ALL>();
		t[3] = make_entry<V3, OPS_CONV_CORR>();
		init = true;
	}
	*out = t;
	return 4;
}
} /* namespace fgk */

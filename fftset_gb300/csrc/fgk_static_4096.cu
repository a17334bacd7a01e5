/* Compile-time kernels for FREQ_OFFSET_REAL, 4096 bins (the batched
 * differentiable convolution workload): 16^3, 256 threads per transform.
 * SCfg<modulation, L, T, G, twiddles-from-global, TMA, radices...> */
#include "fgk_static.cuh"

namespace fgk {
using V0 = SCfg<FGK_MOD_FREQOFF, 4096, 256, 2, 1, 1, 16, 16, 16>;
using V1 = SCfg<FGK_MOD_FREQOFF, 4096, 256, 2, 0, 0, 16, 16, 16>;
using V2 = SCfg<FGK_MOD_FREQOFF, 4096, 256, 3, 1, 0, 16, 16, 16>;

int static_entries_4096(const StaticEntry **out)
{
	static StaticEntry t[3];
	static bool init = false;
	if (!init) {
		t[0] = make_entry<V0, OPS_ALL>();
		t[1] = make_entry<V1, OPS_ALL>();
		t[2] = make_entry<V2, OPS_CONV_CORR>();
		init = true;
	}
	*out = t;
	return 3;
}
} /* namespace fgk */

/* Compile-time kernels for FREQ_OFFSET_REAL, 1536 bins (the fused
 * convolution workload). Variants differ in radix order, threads per
 * transform (T) and transforms per CTA (G); the autotuner picks one. */
#include "fgk_static.cuh"

namespace fgk {
/* (16,16,6): R16 stages use 96 of 128 threads (one warp idle), R6 stages two
 * butterflies per thread; (16,12,8) one warp per transform with 48 values per
 * thread; (8,8,8,3) 64 threads, 24 values per thread. */
using V0 = SCfg<FGK_MOD_FREQOFF, 1536, 128, 4, 0, 16, 16, 6>;
using V1 = SCfg<FGK_MOD_FREQOFF, 1536, 128, 6, 0, 16, 16, 6>;
using V2 = SCfg<FGK_MOD_FREQOFF, 1536, 96, 8, 0, 16, 16, 6>;
using V3 = SCfg<FGK_MOD_FREQOFF, 1536, 64, 8, 0, 8, 8, 8, 3>;
using V4 = SCfg<FGK_MOD_FREQOFF, 1536, 32, 12, 0, 16, 12, 8>;

int static_entries_1536(const StaticEntry **out)
{
	static StaticEntry t[5];
	static bool init = false;
	if (!init) {
		t[0] = make_entry<V0, OPS_ALL>();
		t[1] = make_entry<V1, OPS_CONV>();
		t[2] = make_entry<V2, OPS_CONV>();
		t[3] = make_entry<V3, OPS_CONV>();
		t[4] = make_entry<V4, OPS_CONV>();
		init = true;
	}
	*out = t;
	return 5;
}
} /* namespace fgk */

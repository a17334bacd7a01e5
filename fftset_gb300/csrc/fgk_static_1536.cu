/* Compile-time kernels for FREQ_OFFSET_REAL, 1536 bins (the fused
 * convolution workload). Variants differ in radix order, threads per
 * transform (T), transforms per CTA (G) and input path (direct loads, or
 * bulk-copy double buffering); the autotuner picks one.
 * SCfg<modulation, L, T, G, twiddles-from-global, TMA, radices...> */
#include "fgk_static.cuh"

namespace fgk {
/* (16,16,6) with 128 threads: R16 stages use 96 of them, R6 stages two
 * butterflies per thread. V0-V2 ping-pong (one butterfly in registers at a
 * time, so 6-12 transforms per CTA fit); V3 in-place with direct loads; V4
 * in-place with bulk-copy input. */
using V0 = SCfg<FGK_MOD_FREQOFF, 1536, 128, 6, 0, 2, 16, 16, 6>;
using V1 = SCfg<FGK_MOD_FREQOFF, 1536, 128, 7, 1, 2, 16, 16, 6>;
using V2 = SCfg<FGK_MOD_FREQOFF, 1536, 64, 7, 1, 2, 16, 12, 8>;
using V3 = SCfg<FGK_MOD_FREQOFF, 1536, 128, 4, 0, 0, 16, 16, 6>;
using V4 = SCfg<FGK_MOD_FREQOFF, 1536, 128, 4, 0, 1, 16, 16, 6>;
/* V5: V0 with the chain (16, 6, 16): both stages that scatter with ns = 1
 * (forward stage 0 and the first reversed stage) are radix 16, whose
 * stride-16 stores the i + i/16 padding makes conflict-free, and the radix-6
 * stage (ns = 16) stores runs of 16 consecutive slots: no shared-memory bank
 * conflicts in the exchange, against 28 % extra wavefronts for (16, 16, 6) */
using V5 = SCfg<FGK_MOD_FREQOFF, 1536, 128, 6, 0, 2, 16, 6, 16>;

int static_entries_1536(const StaticEntry **out)
{
	static StaticEntry t[6];
	static bool init = false;
	if (!init) {
		t[0] = make_entry<V0, OPS_ALL>();
		t[1] = make_entry<V1, OPS_CONV>();
		t[2] = make_entry<V2, OPS_CONV>();
		t[3] = make_entry<V3, OPS_ALL>();
		t[4] = make_entry<V4, OPS_CONV>();
		t[5] = make_entry<V5, OPS_ALL>();
		init = true;
	}
	*out = t;
	return 6;
}
} /* namespace fgk */

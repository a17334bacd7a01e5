/* Compile-time kernels for FREQ_OFFSET_REAL, 1536 bins (the fused
 * convolution workload). Variants differ in radix order, threads per
 * transform (T), transforms per CTA (G) and input path (direct loads, or
 * bulk-copy double buffering); the autotuner picks one, and without it the
 * first variant that implements an op is its default (fastest measured
 * first). SCfg<modulation, L, T, G, twiddles-from-global, mode, radices...>
 * (mode 0 in place, 1 in place with bulk-copy input, 2 ping-pong). */
#include "fgk_static.cuh"

namespace fgk {
/* (16, 6, 16): both stages that scatter with ns = 1 (forward stage 0 and
 * the first reversed stage) are radix 16, whose stride-16 stores the
 * i + i/16 padding makes conflict-free, and the radix-6 stage (ns = 16)
 * stores runs of 16 consecutive slots: no shared-memory bank conflicts in
 * the exchange (against 28 % extra wavefronts for (16, 16, 6)); the chain is
 * a palindrome, so the reversed stages share the forward twiddles.
 * Ping-pong, 16384 blocks on a GB300: convolution V0 (5 groups of 128
 * threads) 0.119 ms, V2 (5 x 96) 0.122, V1 (6 x 128) 0.122; forward V1
 * 0.119 ms. In-place and bulk-copy forms of this chain were slower. */
using V0 = SCfg<FGK_MOD_FREQOFF, 1536, 128, 5, 0, 2, 16, 6, 16>;
using V1 = SCfg<FGK_MOD_FREQOFF, 1536, 128, 6, 0, 2, 16, 6, 16>;
using V2 = SCfg<FGK_MOD_FREQOFF, 1536, 96, 5, 0, 2, 16, 6, 16>;
/* (16, 16, 6): R16 stages use 96 of 128 threads, R6 stages two butterflies
 * per thread. V3 ping-pong (convolution 0.138 ms); V4 in place with direct
 * loads (0.149); V5 in place with bulk-copy input (0.181). */
using V3 = SCfg<FGK_MOD_FREQOFF, 1536, 128, 6, 0, 2, 16, 16, 6>;
using V4 = SCfg<FGK_MOD_FREQOFF, 1536, 128, 4, 0, 0, 16, 16, 6>;
using V5 = SCfg<FGK_MOD_FREQOFF, 1536, 128, 4, 0, 1, 16, 16, 6>;
/* (16, 12, 8), 64 threads, twiddles through L1 (0.158 ms) */
using V6 = SCfg<FGK_MOD_FREQOFF, 1536, 64, 7, 1, 2, 16, 12, 8>;

int static_entries_1536(const StaticEntry **out)
{
	static StaticEntry t[7];
	static bool init = false;
	if (!init) {
		t[0] = make_entry<V0, OPS_CONV_CORR>();
		t[1] = make_entry<V1, OPS_ALL>();
		t[2] = make_entry<V2, OPS_CONV_CORR>();
		t[3] = make_entry<V3, OPS_ALL>();
		t[4] = make_entry<V4, OPS_ALL>();
		t[5] = make_entry<V5, OPS_CONV>();
		t[6] = make_entry<V6, OPS_CONV>();
		init = true;
	}
	*out = t;
	return 7;
}
} /* namespace fgk */

/* Compile-time kernels for FREQ_OFFSET_REAL, 1536 bins (the fused
 * convolution workload). Variants differ in radix order, threads per
 * transform (T), transforms per CTA (G), input path (direct loads, or
 * bulk-copy double buffering), the butterfly-to-thread map and how the
 * twiddle and modulation tables are read; the autotuner picks one, and
 * without it the first variant that implements an op is its default
 * (fastest measured first). SCfg<modulation, L, T, G, table flags, mode,
 * radices...>: table flags | 1 twiddles through L1, | 2 radix-16 twiddles
 * from the entries of p = 1, 2, 4, 8, | 4 modulation factors from one entry
 * per butterfly and constants; mode 0 in place, 1 in place with bulk-copy
 * input, 2 ping-pong, | 4 butterfly-to-thread map rotated by 32 threads per
 * group. */
#include "fgk_static.cuh"

namespace fgk {
/* (16, 6, 16): both stages that scatter with ns = 1 (forward stage 0 and
 * the first reversed stage) are radix 16, whose stride-16 stores the
 * i + i/16 padding makes conflict-free, and the radix-6 stage (ns = 16)
 * stores runs of 16 consecutive slots: no shared-memory bank conflicts in
 * the exchange (against 28 % extra wavefronts for (16, 16, 6)); the chain is
 * a palindrome, so the reversed stages share the forward twiddles.
 * The radix-16 stages have 96 butterflies for 128 threads; with the rotated
 * map the idle warp of each group sits on a different scheduler (warps go
 * to the SM's four schedulers by warp index mod 4), instead of every
 * group's last warp idling on the same one.
 * With the L1/shared-memory pipe the busiest unit (82 % in a profile of V4),
 * the lean-table forms trade shared-memory reads for multiplies: 11 of the
 * 15 twiddle reads of a radix-16 butterfly and 15 of the 16 modulation reads
 * of the first and last stages go.
 * Ping-pong, 16384 blocks on a GB300, convolution (ms): V0 (both table
 * forms, rotated, 6 groups of 128 threads, 80 registers) 0.1125; V1 (both,
 * 5 groups) 0.1149; V2 (twiddles only) 0.1157; V3 (modulation only) 0.1155;
 * V4 (rotated, 5 groups) 0.1164; V5 (rotated, 6 groups) 0.1194; V6
 * (5 groups, plain map) 0.1176; V7 (6 groups, plain) 0.1217; V8 (5 x 96)
 * 0.1219; V9 (5 x 96 rotated) 0.1229. Both table forms at 7 groups (72
 * registers): 0.1235. In-place and bulk-copy forms of this chain were
 * slower. */
using V0 = SCfg<FGK_MOD_FREQOFF, 1536, 128, 6, 6, 2 | 4, 16, 6, 16>;
using V1 = SCfg<FGK_MOD_FREQOFF, 1536, 128, 5, 6, 2 | 4, 16, 6, 16>;
using V2 = SCfg<FGK_MOD_FREQOFF, 1536, 128, 5, 2, 2 | 4, 16, 6, 16>;
using V3 = SCfg<FGK_MOD_FREQOFF, 1536, 128, 5, 4, 2 | 4, 16, 6, 16>;
using V4 = SCfg<FGK_MOD_FREQOFF, 1536, 128, 5, 0, 2 | 4, 16, 6, 16>;
using V5 = SCfg<FGK_MOD_FREQOFF, 1536, 128, 6, 0, 2 | 4, 16, 6, 16>;
using V6 = SCfg<FGK_MOD_FREQOFF, 1536, 128, 5, 0, 2, 16, 6, 16>;
using V7 = SCfg<FGK_MOD_FREQOFF, 1536, 128, 6, 0, 2, 16, 6, 16>;
using V8 = SCfg<FGK_MOD_FREQOFF, 1536, 96, 5, 0, 2, 16, 6, 16>;
using V9 = SCfg<FGK_MOD_FREQOFF, 1536, 96, 5, 0, 2 | 4, 16, 6, 16>;
/* (16, 16, 6): R16 stages use 96 of 128 threads, R6 stages two butterflies
 * per thread. V10 ping-pong (convolution 0.138 ms); V11 in place with direct
 * loads (0.148); V12 in place with bulk-copy input (0.180). */
using V10 = SCfg<FGK_MOD_FREQOFF, 1536, 128, 6, 0, 2, 16, 16, 6>;
using V11 = SCfg<FGK_MOD_FREQOFF, 1536, 128, 4, 0, 0, 16, 16, 6>;
using V12 = SCfg<FGK_MOD_FREQOFF, 1536, 128, 4, 0, 1, 16, 16, 6>;
/* (16, 12, 8), 64 threads, twiddles through L1 (0.157 ms) */
using V13 = SCfg<FGK_MOD_FREQOFF, 1536, 64, 7, 1, 2, 16, 12, 8>;

int static_entries_1536(const StaticEntry **out)
{
	static StaticEntry t[14];
	static bool init = false;
	if (!init) {
		t[0] = with_serve<V0, OPS_ALL>(with_ola<V0>(make_entry<V0, OPS_ALL>()));
		t[1] = make_entry<V1, OPS_CONV_CORR>();
		t[2] = make_entry<V2, OPS_CONV_CORR>();
		t[3] = make_entry<V3, OPS_CONV_CORR>();
		t[4] = make_entry<V4, OPS_CONV_CORR>();
		t[5] = make_entry<V5, OPS_ALL>();
		t[6] = make_entry<V6, OPS_CONV_CORR>();
		t[7] = make_entry<V7, OPS_ALL>();
		t[8] = make_entry<V8, OPS_CONV_CORR>();
		t[9] = make_entry<V9, OPS_CONV_CORR>();
		t[10] = make_entry<V10, OPS_ALL>();
		t[11] = make_entry<V11, OPS_ALL>();
		t[12] = make_entry<V12, OPS_CONV>();
		t[13] = make_entry<V13, OPS_CONV>();
		init = true;
	}
	*out = t;
	return 14;
}
} /* namespace fgk */

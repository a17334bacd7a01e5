/* Compile-time kernels for FREQ_OFFSET_REAL, 4096 bins (the batched
 * differentiable convolution workload): 16^3, 256 threads per transform.
 * SCfg<modulation, L, T, G, table flags, mode, radices...> (table flags
 * | 1 twiddles through L1, | 2 radix-16 twiddles from the entries of
 * p = 1, 2, 4, 8, | 4 modulation factors from one entry per butterfly and
 * constants; mode 0 in place, 1 in place with bulk-copy input, 2 ping-pong).
 * The first variant that implements an op is its default: the order is the
 * measured one, fastest first (GB300, convolution at 2048 / 16384 blocks in
 * ms: V0 0.0553 / 0.341, V1 0.0587 / 0.345, V2 0.0619 / 0.370, V3 0.0624 /
 * 0.371, V4 0.0658 / 0.458, V5 0.0676 / 0.474, V6 0.0848 / 0.542; forward at
 * 16384 blocks: V0 0.245, V1 0.250, V6 0.289; inverse: V1 0.215, V0 0.221).
 * Unlike the 1536-bin kernels, fewer twiddle reads do not pay here: at
 * 4096 bins a thread runs one radix-16 butterfly per stage with all 256
 * threads busy, and the extra multiplies lengthen it. The chain is a
 * palindrome, so its twiddles are staged once. V0 also carries the
 * adjoint's one-pass kernels (static_kernel_adj, static_kernel_kgrad). */
#include "fgk_static.cuh"

namespace fgk {
using V0 = SCfg<FGK_MOD_FREQOFF, 4096, 256, 2, 0, 0, 16, 16, 16>;
using V1 = SCfg<FGK_MOD_FREQOFF, 4096, 256, 2, 2, 0, 16, 16, 16>;
using V2 = SCfg<FGK_MOD_FREQOFF, 4096, 256, 3, 2, 0, 16, 16, 16>;
using V3 = SCfg<FGK_MOD_FREQOFF, 4096, 256, 3, 0, 0, 16, 16, 16>;
using V4 = SCfg<FGK_MOD_FREQOFF, 4096, 256, 1, 6, 2, 16, 16, 16>;
using V5 = SCfg<FGK_MOD_FREQOFF, 4096, 256, 1, 0, 2, 16, 16, 16>;
using V6 = SCfg<FGK_MOD_FREQOFF, 4096, 256, 2, 1, 1, 16, 16, 16>;
/* ping-pong with both table forms and two groups (the constant modulation
 * stages 256 factors, not 4096, which leaves room for the second group):
 * the fastest inverse (2048 / 8192 blocks: 0.0358 / 0.106 ms against V0's
 * 0.0404 / 0.121), listed first for that op only; for conv and forward it
 * measured slower than V0 (0.061 / 0.195 and 0.050 / 0.146 ms). V8: the
 * same with the modulation form only (inverse 0.0364 / 0.109). */
using V7 = SCfg<FGK_MOD_FREQOFF, 4096, 256, 2, 6, 2, 16, 16, 16>;
using V8 = SCfg<FGK_MOD_FREQOFF, 4096, 256, 2, 4, 2, 16, 16, 16>;

int static_entries_4096(const StaticEntry **out)
{
	static StaticEntry t[10];
	static bool init = false;
	if (!init) {
		t[0] = with_serve<V7, 1 << FGK_OP_INVERSE>(make_entry<V7, 1 << FGK_OP_INVERSE>());
		t[1] = with_serve<V0, OPS_ALL>(with_kgrad<V0>(make_entry<V0, OPS_ALL>()));
		t[2] = make_entry<V1, OPS_ALL>();
		t[3] = make_entry<V2, OPS_CONV_CORR>();
		t[4] = make_entry<V3, OPS_CONV_CORR>();
		t[5] = make_entry<V4, OPS_ALL>();
		t[6] = make_entry<V5, OPS_CONV_CORR>();
		t[7] = make_entry<V6, OPS_ALL>();
		t[8] = make_entry<V7, OPS_ALL>();
		t[9] = make_entry<V8, OPS_ALL>();
		init = true;
	}
	*out = t;
	return 10;
}
} /* namespace fgk */

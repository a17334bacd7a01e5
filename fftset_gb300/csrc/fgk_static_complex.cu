/* Compile-time kernels for COMPLEX, 1536 and 4096 bins: the cyclic fused
 * convolution and the plain transforms at the sizes the FREQ_OFFSET_REAL
 * workloads use, with the same chains as their FREQ_OFFSET_REAL kernels
 * (fgk_static_1536.cu, fgk_static_4096.cu). Without these, COMPLEX
 * batches of these sizes run on the generic resident kernel.
 * SCfg<modulation, L, T, G, table flags, mode, radices...>: table flag 2
 * radix-16 twiddles from the entries of p = 1, 2, 4, 8; mode 0 in place,
 * 2 ping-pong, | 4 butterfly-to-thread map rotated by 32 threads per group.
 * Fastest measured first (16384 blocks on a GB300, convolution / forward /
 * inverse in ms): 1536 bins C1536a 0.107 / 0.069 / 0.070, C1536b 0.112 /
 * 0.073 / 0.073, the generic kernel 0.357 / 0.231 / 0.232; 4096 bins C4096a
 * 0.307 / 0.200 / 0.201, C4096b 0.327 / 0.199 / 0.198, the generic kernel
 * 0.846 / 0.471 / 0.474. */
#include "fgk_static.cuh"

namespace fgk {
using C1536a = SCfg<FGK_MOD_COMPLEX, 1536, 128, 6, 2, 2 | 4, 16, 6, 16>;
using C1536b = SCfg<FGK_MOD_COMPLEX, 1536, 128, 5, 0, 2 | 4, 16, 6, 16>;
using C4096a = SCfg<FGK_MOD_COMPLEX, 4096, 256, 2, 0, 0, 16, 16, 16>;
using C4096b = SCfg<FGK_MOD_COMPLEX, 4096, 256, 2, 2, 0, 16, 16, 16>;

int static_entries_c1536(const StaticEntry **out)
{
	static StaticEntry t[2];
	static bool init = false;
	if (!init) {
		t[0] = with_serve<C1536a, OPS_ALL>(make_entry<C1536a, OPS_ALL>());
		t[1] = make_entry<C1536b, OPS_ALL>();
		init = true;
	}
	*out = t;
	return 2;
}

int static_entries_c4096(const StaticEntry **out)
{
	static StaticEntry t[2];
	static bool init = false;
	if (!init) {
		t[0] = with_serve<C4096a, OPS_ALL>(make_entry<C4096a, OPS_ALL>());
		t[1] = make_entry<C4096b, OPS_ALL>();
		init = true;
	}
	*out = t;
	return 2;
}
} /* namespace fgk */

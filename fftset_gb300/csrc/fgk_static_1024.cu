/* Compile-time kernels for COMPLEX, 1024 bins: 16*16*4, 64 threads per
 * transform. SCfg<modulation, L, T, G, table flags, mode, radices...>
 * (table flag 2: radix-16 twiddles from the entries of p = 1, 2, 4, 8;
 * mode 0 in place, 1 in place with bulk-copy input). Fastest first (16384
 * blocks on a GB300, convolution / forward in ms): V0 0.0711 / 0.0479, V1
 * 0.0725 / 0.0480, V2 0.0742 / 0.0511. */
#include "fgk_static.cuh"

namespace fgk {
using V0 = SCfg<FGK_MOD_COMPLEX, 1024, 64, 4, 2, 0, 16, 16, 4>;
using V1 = SCfg<FGK_MOD_COMPLEX, 1024, 64, 4, 0, 0, 16, 16, 4>;
using V2 = SCfg<FGK_MOD_COMPLEX, 1024, 64, 8, 0, 1, 16, 16, 4>;

int static_entries_1024(const StaticEntry **out)
{
	static StaticEntry t[3];
	static bool init = false;
	if (!init) {
		t[0] = with_serve<V0, OPS_ALL>(make_entry<V0, OPS_ALL>());
		t[1] = make_entry<V1, OPS_ALL>();
		t[2] = make_entry<V2, OPS_ALL>();
		init = true;
	}
	*out = t;
	return 3;
}
} /* namespace fgk */

/* Compile-time kernels for COMPLEX, 1024 bins: 16*16*4, 64 threads per
 * transform. SCfg<modulation, L, T, G, twiddles-from-global, TMA, radices...> */
#include "fgk_static.cuh"

namespace fgk {
using V0 = SCfg<FGK_MOD_COMPLEX, 1024, 64, 8, 0, 1, 16, 16, 4>;
using V1 = SCfg<FGK_MOD_COMPLEX, 1024, 64, 4, 0, 0, 16, 16, 4>;

int static_entries_1024(const StaticEntry **out)
{
	static StaticEntry t[2];
	static bool init = false;
	if (!init) {
		t[0] = make_entry<V0, OPS_ALL>();
		t[1] = make_entry<V1, OPS_ALL>();
		init = true;
	}
	*out = t;
	return 2;
}
} /* namespace fgk */

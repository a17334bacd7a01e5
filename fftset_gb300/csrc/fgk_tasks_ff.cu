/* The ragged task kernel (forward, FREQ_OFFSET_REAL); fgk_tasks.cuh. */
#include "fgk_tasks.cuh"

extern "C" int fgk_launch_tasks_ff(FGKT_LAUNCH_ARGS)
{
	return fgk::launch_tasks<false, true>(FGKT_LAUNCH_PASS);
}

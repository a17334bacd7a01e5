/* The ragged task kernel (inverse, FREQ_OFFSET_REAL); fgk_tasks.cuh. */
#include "fgk_tasks.cuh"

extern "C" int fgk_launch_tasks_if(FGKT_LAUNCH_ARGS)
{
	return fgk::launch_tasks<true, true>(FGKT_LAUNCH_PASS);
}

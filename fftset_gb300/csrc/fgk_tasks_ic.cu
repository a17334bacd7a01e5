/* The ragged task kernel (inverse, COMPLEX); fgk_tasks.cuh. */
#include "fgk_tasks.cuh"

extern "C" int fgk_launch_tasks_ic(FGKT_LAUNCH_ARGS)
{
	return fgk::launch_tasks<true, false>(FGKT_LAUNCH_PASS);
}

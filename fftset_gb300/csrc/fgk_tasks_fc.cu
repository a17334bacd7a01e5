/* The ragged task kernel (forward, COMPLEX); fgk_tasks.cuh. */
#include "fgk_tasks.cuh"

extern "C" int fgk_launch_tasks_fc(FGKT_LAUNCH_ARGS)
{
	return fgk::launch_tasks<false, false>(FGKT_LAUNCH_PASS);
}

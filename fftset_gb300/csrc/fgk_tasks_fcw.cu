/* The ragged task kernel (forward, COMPLEX), wide CTAs; fgk_tasks.cuh. */
#include "fgk_tasks.cuh"

extern "C" int fgk_launch_tasks_fcw(FGKT_LAUNCH_ARGS)
{
	return fgk::launch_tasks<false, false, fgk::TK_THREADS_WIDE, fgk::TK_CTAS_WIDE>(FGKT_LAUNCH_PASS);
}

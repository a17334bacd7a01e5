/* The ragged task kernel (inverse, COMPLEX), single-buffer CTAs; fgk_tasks.cuh. */
#include "fgk_tasks.cuh"

extern "C" int fgk_launch_tasks_ics(FGKT_LAUNCH_ARGS)
{
	return fgk::launch_tasks<true, false, fgk::TK_THREADS_SINGLE, fgk::TK_CTAS_SINGLE, 1>(FGKT_LAUNCH_PASS);
}

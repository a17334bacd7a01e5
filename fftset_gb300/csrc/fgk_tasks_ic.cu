/* The ragged task kernel (inverse, COMPLEX), narrow CTAs; fgk_tasks.cuh. */
#include "fgk_tasks.cuh"

extern "C" int fgk_launch_tasks_ic(FGKT_LAUNCH_ARGS)
{
	return fgk::launch_tasks<true, false, fgk::TK_THREADS_NARROW, fgk::TK_CTAS_NARROW>(FGKT_LAUNCH_PASS);
}

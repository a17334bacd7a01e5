/* The ragged task kernel (inverse, FREQ_OFFSET_REAL), narrow CTAs; fgk_tasks.cuh. */
#include "fgk_tasks.cuh"

extern "C" int fgk_launch_tasks_if(FGKT_LAUNCH_ARGS)
{
	return fgk::launch_tasks<true, true, fgk::TK_THREADS_NARROW, fgk::TK_CTAS_NARROW>(FGKT_LAUNCH_PASS);
}

/* The ragged task kernel (inverse, FREQ_OFFSET_REAL), wide CTAs; fgk_tasks.cuh. */
#include "fgk_tasks.cuh"

extern "C" int fgk_launch_tasks_ifw(FGKT_LAUNCH_ARGS)
{
	return fgk::launch_tasks<true, true, fgk::TK_THREADS_WIDE, fgk::TK_CTAS_WIDE>(FGKT_LAUNCH_PASS);
}

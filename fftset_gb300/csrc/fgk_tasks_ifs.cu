/* The ragged task kernel (inverse, FREQ_OFFSET_REAL), single-buffer CTAs; fgk_tasks.cuh. */
#include "fgk_tasks.cuh"

extern "C" int fgk_launch_tasks_ifs(FGKT_LAUNCH_ARGS)
{
	return fgk::launch_tasks<true, true, fgk::TK_THREADS_SINGLE, fgk::TK_CTAS_SINGLE, 1>(FGKT_LAUNCH_PASS);
}

/* The ragged task kernel (forward, COMPLEX), narrow CTAs; fgk_tasks.cuh. */
#include "fgk_tasks.cuh"

extern "C" int fgk_launch_tasks_fc(FGKT_LAUNCH_ARGS)
{
	return fgk::launch_tasks<false, false, fgk::TK_THREADS_NARROW, fgk::TK_CTAS_NARROW>(FGKT_LAUNCH_PASS);
}

/* Host entry points of the ragged task kernel (fgk_tasks.cuh): its tile
 * geometry, and the launch, which zeroes the dependency counters and calls
 * the instantiation for the batch's direction, modulation and CTA shape
 * (fgk_tasks_{fc,ff,ic,if}[w].cu). */
#include "fgk_tasks.cuh"

namespace fgk {
__global__ void spectrum_natural(const float *__restrict__ kern, const int32_t *__restrict__ kidx, int kvw, uint32_t L,
                                 int conj, float2 *spec)
{
	for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < L; m += gridDim.x * blockDim.x) {
		const int o = __ldg(kidx + m);
		const float im = __ldg(kern + o + kvw);
		spec[m] = make_float2(__ldg(kern + o), conj ? -im : im);
	}
}
} /* namespace fgk */

extern "C" int fgk_launch_spectrum_natural(const float *kern, const int32_t *kidx, int kvw, uint32_t L, int conj,
                                           void *spec, void *stream)
{
	const uint32_t grid = (L + 255) / 256 < 1024 ? (L + 255) / 256 : 1024;
	fgk::spectrum_natural<<<grid, 256, 0, (cudaStream_t)stream>>>(kern, kidx, kvw, L, conj, (float2 *)spec);
	fgk_count_launch();
	return (int)cudaGetLastError();
}

extern "C" int fgk_launch_tasks_fc(FGKT_LAUNCH_ARGS);
extern "C" int fgk_launch_tasks_ff(FGKT_LAUNCH_ARGS);
extern "C" int fgk_launch_tasks_ic(FGKT_LAUNCH_ARGS);
extern "C" int fgk_launch_tasks_if(FGKT_LAUNCH_ARGS);
extern "C" int fgk_launch_tasks_fcw(FGKT_LAUNCH_ARGS);
extern "C" int fgk_launch_tasks_ffw(FGKT_LAUNCH_ARGS);
extern "C" int fgk_launch_tasks_icw(FGKT_LAUNCH_ARGS);
extern "C" int fgk_launch_tasks_ifw(FGKT_LAUNCH_ARGS);
extern "C" int fgk_launch_tasks_fcs(FGKT_LAUNCH_ARGS);
extern "C" int fgk_launch_tasks_ffs(FGKT_LAUNCH_ARGS);
extern "C" int fgk_launch_tasks_ics(FGKT_LAUNCH_ARGS);
extern "C" int fgk_launch_tasks_ifs(FGKT_LAUNCH_ARGS);

extern "C" int fgk_tasks_points(void)
{
	return FGKT_POINTS;
}

extern "C" int fgk_tasks_slots(void)
{
	return fgk::TK_SLOTS;
}

extern "C" int fgk_tasks_threads(int shape)
{
	return shape == FGK_SHAPE_WIDE ? fgk::TK_THREADS_WIDE
	       : shape == FGK_SHAPE_SINGLE ? fgk::TK_THREADS_SINGLE
	                                   : fgk::TK_THREADS_NARROW;
}

extern "C" int fgk_tasks_grid(int num_sms, int shape)
{
	return (shape == FGK_SHAPE_WIDE     ? fgk::TK_CTAS_WIDE
	        : shape == FGK_SHAPE_SINGLE ? fgk::TK_CTAS_SINGLE
	                                    : fgk::TK_CTAS_NARROW) *
	       num_sms;
}

extern "C" int fgk_launch_tasks(const fgk_task *tasks_dev, uint32_t ntasks, const fgk_plan *plans_dev,
                                const fgk_rg_item *items_dev, const fgk_big *bigs_dev, uint32_t nbig,
                                const fgk_huge *huges_dev, uint32_t nhcount, int *counters_dev, float *scratch_dev,
                                int op, int modulation, const float *in_base, float *out_base, int num_sms,
                                int shape, int *err_flag, uint32_t spin_limit, fgk_product prod, void *stream)
{
	const bool inv = op == FGK_OP_INVERSE, freq = modulation == FGK_MOD_FREQOFF;
	cudaStream_t s = (cudaStream_t)stream;
	cudaError_t e;
	if (ntasks == 0)
		return 0;
	if ((e = cudaMemsetAsync(counters_dev, 0, sizeof(int) * (1 + (size_t)nbig + (size_t)nhcount), s)) !=
	    cudaSuccess)
		return (int)e;
	uint32_t grid = (uint32_t)fgk_tasks_grid(num_sms, shape);
	if (grid > ntasks)
		grid = ntasks;
	int *hcounters = counters_dev + 1 + nbig;
	float2 *scratch = reinterpret_cast<float2 *>(scratch_dev);
	auto launch = shape == FGK_SHAPE_WIDE
	                  ? (inv ? (freq ? fgk_launch_tasks_ifw : fgk_launch_tasks_icw)
	                         : (freq ? fgk_launch_tasks_ffw : fgk_launch_tasks_fcw))
	              : shape == FGK_SHAPE_SINGLE
	                  ? (inv ? (freq ? fgk_launch_tasks_ifs : fgk_launch_tasks_ics)
	                         : (freq ? fgk_launch_tasks_ffs : fgk_launch_tasks_fcs))
	                  : (inv ? (freq ? fgk_launch_tasks_if : fgk_launch_tasks_ic)
	                         : (freq ? fgk_launch_tasks_ff : fgk_launch_tasks_fc));
	return launch(grid, tasks_dev, ntasks, plans_dev, items_dev, bigs_dev, huges_dev, counters_dev, hcounters, scratch,
	              in_base, out_base, err_flag, spin_limit, prod, s);
}

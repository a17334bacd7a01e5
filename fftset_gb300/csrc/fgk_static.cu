/* Registry and launcher of the compile-time kernels (fgk_static.cuh); the
 * configurations themselves are instantiated in fgk_static_<size>.cu. */
#include "fgk_static.cuh"

namespace fgk {
int static_entries_1536(const StaticEntry **out);
int static_entries_4096(const StaticEntry **out);
int static_entries_1024(const StaticEntry **out);
int static_entries_c1536(const StaticEntry **out);
int static_entries_c4096(const StaticEntry **out);

static int variants(uint32_t mod, uint32_t L, const StaticEntry **out)
{
	const StaticEntry *e = nullptr;
	int n = 0;
	if (mod == FGK_MOD_FREQOFF && L == 1536)
		n = static_entries_1536(&e);
	else if (mod == FGK_MOD_FREQOFF && L == 4096)
		n = static_entries_4096(&e);
	else if (mod == FGK_MOD_COMPLEX && L == 1024)
		n = static_entries_1024(&e);
	else if (mod == FGK_MOD_COMPLEX && L == 1536)
		n = static_entries_c1536(&e);
	else if (mod == FGK_MOD_COMPLEX && L == 4096)
		n = static_entries_c4096(&e);
	*out = e;
	return n;
}
} /* namespace fgk */

extern "C" int fgk_static_count(uint32_t mod, uint32_t L)
{
	const fgk::StaticEntry *e;
	return fgk::variants(mod, L, &e);
}

extern "C" int fgk_static_info(uint32_t mod, uint32_t L, int v, uint32_t *radices, uint32_t *n, uint32_t *threads,
                               uint32_t *groups, uint32_t *opmask, uint32_t *tma)
{
	const fgk::StaticEntry *e;
	int nv = fgk::variants(mod, L, &e);
	if (v < 0 || v >= nv)
		return 0;
	e += v;
	for (uint32_t i = 0; i < e->n; i++)
		radices[i] = e->radices[i];
	*n = e->n;
	*threads = e->T;
	*groups = e->G;
	*tma = e->tma;
	*opmask = 0;
	for (int op = 0; op < FGK_OP_COUNT; op++)
		if (e->fn[op])
			*opmask |= 1u << op;
	return 1;
}

extern "C" int fgk_launch_static(const fgk_plan *p, int v, int op, float *out, const float *in, const float *kern,
                                 uint32_t count, size_t in_stride, size_t out_stride, void *stream, int num_sms,
                                 int *err_flag)
{
	using namespace fgk;
	const StaticEntry *e;
	int nv = variants(p->modulation, p->L, &e);
	if (v < 0 || v >= nv || op < 0 || op >= FGK_OP_COUNT || !e[v].fn[op])
		return -1; /* not handled: caller falls back to the generic kernel */
	e += v;
	/* bulk copies need 16-byte aligned blocks */
	if (e->tma && ((((uintptr_t)in) & 15) || ((in_stride * sizeof(float)) & 15)))
		return -1;
	if (count == 0)
		return 0;
	const size_t smem = e->smem[op];
	cudaError_t err = cudaFuncSetAttribute((const void *)e->fn[op], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (err != cudaSuccess)
		return (int)err;
	int per_sm = 0;
	err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)e->fn[op], (int)(e->T * e->G), smem);
	if (err != cudaSuccess)
		return (int)err;
	if (per_sm < 1)
		return (int)cudaErrorInvalidConfiguration;
	const uint64_t need = ((uint64_t)count + e->G - 1) / e->G;
	uint64_t grid = (uint64_t)per_sm * (uint64_t)num_sms;
	if (grid > need)
		grid = need;
	StaticArgs a{out, in, kern, count, in_stride, out_stride, err_flag};
	e->fn[op]<<<(unsigned)grid, e->T * e->G, smem, (cudaStream_t)stream>>>(*p, a);
	return (int)cudaGetLastError();
}

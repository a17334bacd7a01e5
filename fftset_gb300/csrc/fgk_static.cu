/* Registry and launcher of the compile-time kernels (fgk_static.cuh); the
 * configurations themselves are instantiated in fgk_static_<size>.cu. */
#include <pthread.h>

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

/* The shared-memory attribute and the occupancy of a kernel, set and
 * queried once per (kernel, device) and remembered: a launch of a single
 * small transform then costs no more host calls than the launch itself. */
namespace fgk {
struct SetupEntry {
	const void *fn;
	int         dev, per_sm;
	size_t      smem;
};
static SetupEntry setup_cache[128];
static pthread_mutex_t setup_lock = PTHREAD_MUTEX_INITIALIZER;

static cudaError_t launch_setup(const void *fn, int threads, size_t smem, int *per_sm)
{
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess)
		return e;
	pthread_mutex_lock(&setup_lock);
	for (auto &c : setup_cache)
		if (c.fn == fn && c.dev == dev && c.smem == smem) {
			*per_sm = c.per_sm;
			pthread_mutex_unlock(&setup_lock);
			return cudaSuccess;
		}
	e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e == cudaSuccess)
		e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, fn, threads, smem);
	if (e == cudaSuccess)
		for (auto &c : setup_cache)
			if (c.fn == nullptr) {
				c = SetupEntry{fn, dev, *per_sm, smem};
				break;
			}
	pthread_mutex_unlock(&setup_lock);
	return e;
}
/* a launch with programmatic stream serialisation: the kernel executes
 * griddepcontrol.wait before it reads what earlier launches may have written
 * (stage_tables, static_kernel_adj) */
template <class... Args>
static cudaError_t launch_dependent(void (*fn)(Args...), unsigned grid, unsigned block, size_t smem,
                                    cudaStream_t stream, Args... args)
{
	cudaLaunchConfig_t cfg = {};
	cudaLaunchAttribute at[1];
	at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
	at[0].val.programmaticStreamSerializationAllowed = 1;
	cfg.gridDim = dim3(grid);
	cfg.blockDim = dim3(block);
	cfg.dynamicSmemBytes = smem;
	cfg.stream = stream;
	cfg.attrs = at;
	cfg.numAttrs = 1;
	return cudaLaunchKernelEx(&cfg, fn, args...);
}
} /* namespace fgk */

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
	int per_sm = 0;
	cudaError_t err = launch_setup((const void *)e->fn[op], (int)(e->T * e->G), smem, &per_sm);
	if (err != cudaSuccess)
		return (int)err;
	if (per_sm < 1)
		return (int)cudaErrorInvalidConfiguration;
	const uint64_t need = ((uint64_t)count + e->G - 1) / e->G;
	uint64_t grid = (uint64_t)per_sm * (uint64_t)num_sms;
	if (grid > need)
		grid = need;
	StaticArgs a{out, in, kern, count, in_stride, out_stride, err_flag};
	const cudaError_t le =
	    launch_dependent(e->fn[op], (unsigned)grid, e->T * e->G, smem, (cudaStream_t)stream, *p, a);
	fgk_count_launch();
	return le != cudaSuccess ? (int)le : (int)cudaGetLastError();
}

extern "C" int fgk_static_kgrad_variant(uint32_t mod, uint32_t L)
{
	const fgk::StaticEntry *e;
	const int nv = fgk::variants(mod, L, &e);
	for (int v = 0; v < nv; v++)
		if (e[v].kgrad)
			return v;
	return -1;
}

extern "C" int fgk_launch_static_kgrad(const fgk_plan *p, int v, const float *g, size_t g_stride, const float *x,
                                       size_t x_stride, uint32_t count, float *partials, uint32_t max_rows,
                                       uint32_t *rows, void *stream, int num_sms)
{
	using namespace fgk;
	const StaticEntry *e;
	const int nv = variants(p->modulation, p->L, &e);
	if (v < 0 || v >= nv || !e[v].kgrad)
		return -1;
	e += v;
	int per_sm = 0;
	cudaError_t err = launch_setup((const void *)e->kgrad, (int)(e->T * e->G), e->kgrad_smem, &per_sm);
	if (err != cudaSuccess)
		return (int)err;
	if (per_sm < 1)
		return (int)cudaErrorInvalidConfiguration;
	uint64_t grid = (uint64_t)per_sm * (uint64_t)num_sms;
	const uint64_t need = ((uint64_t)count + e->G - 1) / e->G;
	if (grid > need)
		grid = need;
	if (grid > max_rows)
		grid = max_rows;
	if (grid == 0)
		return (int)cudaErrorInvalidValue;
	KgradArgs a{g, x, g_stride, x_stride, count, reinterpret_cast<float2 *>(partials)};
	const cudaError_t le =
	    launch_dependent(e->kgrad, (unsigned)grid, e->T * e->G, e->kgrad_smem, (cudaStream_t)stream, *p, a);
	fgk_count_launch();
	if (le != cudaSuccess)
		return (int)le;
	*rows = (uint32_t)grid;
	return (int)cudaGetLastError();
}

extern "C" int fgk_launch_static_adj(const fgk_plan *p, int v, const float *g, size_t g_stride, const float *x,
                                     size_t x_stride, float *dx, size_t dx_stride, const float *kern, uint32_t count,
                                     float *partials, uint32_t max_rows, uint32_t *rows, void *stream, int num_sms)
{
	using namespace fgk;
	const StaticEntry *e;
	const int nv = variants(p->modulation, p->L, &e);
	if (v < 0 || v >= nv || !e[v].adj)
		return -1;
	e += v;
	int per_sm = 0;
	cudaError_t err = launch_setup((const void *)e->adj, (int)(e->T * e->G), e->adj_smem, &per_sm);
	if (err != cudaSuccess)
		return (int)err;
	if (per_sm < 1)
		return (int)cudaErrorInvalidConfiguration;
	uint64_t grid = (uint64_t)per_sm * (uint64_t)num_sms;
	const uint64_t need = ((uint64_t)count + e->G - 1) / e->G;
	if (grid > need)
		grid = need;
	if (grid > max_rows)
		grid = max_rows;
	if (grid == 0)
		return (int)cudaErrorInvalidValue;
	AdjArgs a{g, x, kern, dx, g_stride, x_stride, dx_stride, count, reinterpret_cast<float2 *>(partials)};
	const cudaError_t le =
	    launch_dependent(e->adj, (unsigned)grid, e->T * e->G, e->adj_smem, (cudaStream_t)stream, *p, a);
	fgk_count_launch();
	if (le != cudaSuccess)
		return (int)le;
	*rows = (uint32_t)grid;
	return (int)cudaGetLastError();
}

extern "C" int fgk_static_serve_ok(uint32_t mod, uint32_t L, int v, int op)
{
	const fgk::StaticEntry *e;
	const int nv = fgk::variants(mod, L, &e);
	return v >= 0 && v < nv && e[v].serve && op >= 0 && op < FGK_OP_COUNT && ((e[v].serve_ops >> op) & 1u);
}

extern "C" int fgk_launch_static_serve(const fgk_plan *p, int v, fgk_serve_words w, uint64_t seen, uint64_t id,
                                       uint32_t idle_polls, void *stream)
{
	using namespace fgk;
	const StaticEntry *e;
	const int nv = variants(p->modulation, p->L, &e);
	if (v < 0 || v >= nv || !e[v].serve || id == 0 || idle_polls == 0)
		return -1;
	e += v;
	int per_sm = 0;
	cudaError_t err = launch_setup((const void *)e->serve, (int)e->T, e->serve_smem, &per_sm);
	if (err != cudaSuccess)
		return (int)err;
	if (per_sm < 1)
		return (int)cudaErrorInvalidConfiguration;
	e->serve<<<1, e->T, e->serve_smem, (cudaStream_t)stream>>>(*p, w, seen, id, idle_polls);
	fgk_count_launch();
	return (int)cudaGetLastError();
}

extern "C" int fgk_static_ola_variant(uint32_t mod, uint32_t L)
{
	const fgk::StaticEntry *e;
	const int nv = fgk::variants(mod, L, &e);
	for (int v = 0; v < nv; v++)
		if (e[v].ola)
			return v;
	return -1;
}

extern "C" int fgk_launch_static_ola(const fgk_plan *p, int v, const float *in, uint64_t n, uint32_t B, uint32_t span,
                                     uint32_t nblocks, uint64_t nout, const float *kern, float *out, void *stream,
                                     int num_sms)
{
	using namespace fgk;
	const StaticEntry *e;
	const int nv = variants(p->modulation, p->L, &e);
	if (v < 0 || v >= nv || !e[v].ola)
		return -1;
	e += v;
	int per_sm = 0;
	cudaError_t err = launch_setup((const void *)e->ola, (int)(e->T * e->G), e->ola_smem, &per_sm);
	if (err != cudaSuccess)
		return (int)err;
	if (per_sm < 1)
		return (int)cudaErrorInvalidConfiguration;
	uint64_t grid = (uint64_t)per_sm * (uint64_t)num_sms;
	const uint64_t need = ((uint64_t)nblocks + e->G - 1) / e->G;
	if (grid > need)
		grid = need;
	OlaArgs a{in, n, B, span, nblocks, nout, kern, out};
	e->ola<<<(unsigned)grid, e->T * e->G, e->ola_smem, (cudaStream_t)stream>>>(*p, a);
	fgk_count_launch();
	return (int)cudaGetLastError();
}

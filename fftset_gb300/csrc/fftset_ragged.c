/* Ragged batches: transforms of many different sizes in one submission, and
 * the task lists of the plain calls of sizes beyond the shared-memory limit.
 *
 * fsr_create plans every distinct size through the fftset's own plan cache
 * (so all sizes share the fftset's twiddle tables) and builds the task list
 * of one persistent launch (fgk_tasks.cu), every task a tile of at most
 * fgk_tasks_points() points:
 *   - items up to fgk_tasks_points() bins: SMALL tasks of same-size items;
 *   - items up to 65536 bins: their four-step split L = L1 L2 (both <= 256),
 *     COLS tiles (columns into the item's scratch) then ROWS tiles (rows
 *     into the output). The ROWS tiles of item i are listed after the COLS
 *     tiles of item i + D, D chosen so that two full grids of tasks separate
 *     them, so ROWS tiles rarely wait;
 *   - larger items: their three-level split L = L1 L2 L3 (each <= 256),
 *     pass A, B and C tiles through two scratch areas, each pass after the
 *     previous one of the same item.
 * Items run largest first, which balances the tail. fftset_ragged_execute
 * records the launch into a CUDA graph on first use (and when the base
 * pointers change) and replays the graph afterwards. */
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include "fftset.h"
#include "fftset_internal.h"
#include "fgk.h"

#define FSR_THREADS ((uint32_t)fgk_tasks_threads()) /* threads of a task CTA */

struct fftset_ragged {
	struct fs_impl *fs;
	int             op;
	int             modulation; /* FGK_MOD_* */
	unsigned        n;
	fgk_task       *tasks_dev;
	uint32_t        ntasks;
	fgk_plan       *plans_dev;
	fgk_rg_item    *items_dev;
	fgk_big        *bigs_dev;
	uint32_t        nbig;
	fgk_huge       *huges_dev;
	uint32_t        nhuge;
	int            *counters_dev;
	float          *scratch;
	/* graph */
	cudaStream_t    cap_stream;
	cudaGraphExec_t exec;
	const float    *g_in;
	float          *g_out;
	int             use_graph;
	double          bytes;
};

struct fsr_sort {
	unsigned bins;
	unsigned idx;
};

static int fsr_cmp(const void *a, const void *b)
{
	const struct fsr_sort *x = (const struct fsr_sort *)a, *y = (const struct fsr_sort *)b;
	if (x->bins != y->bins)
		return x->bins > y->bins ? -1 : 1;
	return x->idx < y->idx ? -1 : (x->idx > y->idx);
}

static uint32_t fsr_slots(uint32_t L)
{
	return L + L / 16 + 1;
}

/* threads per item of a SMALL task: the butterflies of the narrowest stage
 * (so that every stage keeps all threads busy; wider stages loop), a
 * multiple of 32, at most the CTA */
static uint32_t fsr_item_threads(const fgk_plan *p)
{
	uint32_t s, w = p->L;
	for (s = 0; s < p->fwd.nstages; s++) {
		uint32_t nbf = p->L / p->fwd.st[s].radix;
		if (nbf < w)
			w = nbf;
	}
	w = (w + 31) & ~31u;
	return w > FSR_THREADS ? FSR_THREADS : w;
}

/* log2 of the lanes of a tile of columns (rows) of length lp: as many as
 * a tile holds, no more than the `count` columns (rows) there are */
static uint32_t fsr_lanes_log2(uint32_t lp, uint32_t count)
{
	uint32_t ls = 0;
	while ((lp << (ls + 1)) <= (uint32_t)fgk_tasks_points() && (1u << ls) < count)
		ls++;
	return ls;
}

void fsr_free(struct fftset_ragged *rb)
{
	if (!rb)
		return;
	if (rb->fs)
		cudaStreamSynchronize(rb->fs->stream);
	if (rb->exec)
		cudaGraphExecDestroy(rb->exec);
	if (rb->cap_stream)
		cudaStreamDestroy(rb->cap_stream);
	cudaFree(rb->tasks_dev);
	cudaFree(rb->plans_dev);
	cudaFree(rb->items_dev);
	cudaFree(rb->bigs_dev);
	cudaFree(rb->huges_dev);
	cudaFree(rb->counters_dev);
	cudaFree(rb->scratch);
	free(rb);
}

void fftset_ragged_destroy(struct fftset_ragged *rb)
{
	fsr_free(rb);
}

static struct fftset_ragged *fsr_create(struct fs_impl *fs, const struct fftset_modulation *modulation, int op,
                                        unsigned n, const unsigned *bins, const size_t *in_offsets,
                                        const size_t *out_offsets)
{
	struct fftset_ragged *rb = NULL;
	struct fsr_sort *order = NULL;
	fgk_plan *plans = NULL;
	fgk_rg_item *items = NULL;
	fgk_big *bigs = NULL;
	fgk_huge *huges = NULL;
	fgk_task *tasks = NULL;
	unsigned i, j, nplans = 0, nitems = 0, nbig = 0, nhuge = 0, ntasks = 0, cap_tasks = 0;
	size_t scratch_f2 = 0;
	uint64_t total_cols = 0;
	cudaError_t e;
	int rc = FFTSET_E_NOMEM;

	if (!fs)
		return NULL;
	if (n == 0 || !bins || !in_offsets || !out_offsets || (op != FFTSET_OP_FORWARD && op != FFTSET_OP_INVERSE)) {
		fs_latch(fs, FFTSET_E_INVALID, 0);
		return NULL;
	}
	for (i = 0; i < n; i++)
		if ((in_offsets[i] | out_offsets[i]) & 1) { /* complex values are read in pairs */
			fs_latch(fs, FFTSET_E_INVALID, 0);
			return NULL;
		}
	rb = (struct fftset_ragged *)calloc(1, sizeof(*rb));
	order = (struct fsr_sort *)malloc(sizeof(*order) * n);
	plans = (fgk_plan *)calloc(n, sizeof(*plans));
	items = (fgk_rg_item *)calloc(n, sizeof(*items));
	bigs = (fgk_big *)calloc(n, sizeof(*bigs));
	huges = (fgk_huge *)calloc(n, sizeof(*huges));
	if (!rb || !order || !plans || !items || !bigs || !huges)
		goto fail;
	rb->fs = fs;
	rb->op = op;
	rb->modulation = modulation->freq_offset_real ? FGK_MOD_FREQOFF : FGK_MOD_COMPLEX;
	rb->n = n;
	rb->use_graph = 1;
	for (i = 0; i < n; i++) {
		order[i].bins = bins[i];
		order[i].idx = i;
		rb->bytes += 16.0 * bins[i];
	}
	qsort(order, n, sizeof(*order), fsr_cmp);

	/* plans, items and big items; SMALL tasks are counted here, listed below */
	for (i = 0; i < n; i = j) {
		const unsigned L = order[i].bins;
		struct fftset_fft *f = fs_create_plan(fs, modulation, L);
		for (j = i; j < n && order[j].bins == L; j++)
			;
		if (!f) {
			rc = FFTSET_E_INVALID;
			goto fail;
		}
		if (!f->fourstep && L <= (uint32_t)fgk_tasks_points()) {
			const uint32_t tg = fsr_item_threads(&f->rp);
			uint32_t G = FSR_THREADS / tg;
			if (G * fsr_slots(L) > (uint32_t)fgk_tasks_slots())
				G = (uint32_t)fgk_tasks_slots() / fsr_slots(L);
			plans[nplans] = f->rp;
			cap_tasks += (j - i + G - 1) / G;
			plans[nplans].threads = tg; /* reused below: threads per item */
			plans[nplans].per_cta = G;  /* and items per task */
			nplans++;
		} else if (L > 65536) {
			/* three-level: pass A, B, C tiles, two scratch areas per item */
			uint32_t k;
			const fgk_plan3 *p3;
			if ((rc = fs_ensure_threestep(fs, f)) != 0)
				goto fail;
			p3 = &f->p3;
			for (k = i; k < j; k++) {
				fgk_huge *h = &huges[nhuge++];
				const size_t span = ((size_t)L + 15) & ~(size_t)15;
				h->p3 = p3->dev;
				h->in_off = in_offsets[order[k].idx];
				h->out_off = out_offsets[order[k].idx];
				h->sa = scratch_f2;
				h->sb = scratch_f2 + span;
				scratch_f2 += 2 * span;
				h->na = (p3->L2 * p3->L3 + 15) / 16;
				h->nb3 = (p3->L3 + 3) / 4;
				h->nb = (p3->L1 + 3) / 4 * h->nb3;
				h->nc1 = (p3->L1 + 15) / 16;
				cap_tasks += h->na + h->nb + h->nc1 * p3->L2;
			}
		} else {
			uint32_t L1, L2, k;
			if ((rc = fs_ensure_fourstep(fs, f)) != 0)
				goto fail;
			L1 = f->p4.L1;
			L2 = f->p4.L2;
			/* tiles of 16 or more lanes (the task kernel's Rows layout) */
			if ((L1 << 4) > (uint32_t)fgk_tasks_points() || (L2 << 4) > (uint32_t)fgk_tasks_points()) {
				rc = FFTSET_E_UNSUPPORTED;
				goto fail;
			}
			for (k = i; k < j; k++) {
				fgk_big *b = &bigs[nbig++];
				b->p4 = f->p4.dev;
				b->in_off = in_offsets[order[k].idx];
				b->out_off = out_offsets[order[k].idx];
				b->scratch_off = scratch_f2;
				b->ls1 = fsr_lanes_log2(L1, L2);
				b->ls2 = fsr_lanes_log2(L2, L1);
				b->ncols = (L2 + (1u << b->ls1) - 1) >> b->ls1;
				b->nrows = (L1 + (1u << b->ls2) - 1) >> b->ls2;
				total_cols += b->ncols;
				cap_tasks += b->ncols + b->nrows;
				/* laid out by ROWS tiles (full tiles), 128-byte aligned items */
				scratch_f2 += ((((size_t)b->nrows * L2) << b->ls2) + 15) & ~(size_t)15;
			}
		}
	}
	tasks = (fgk_task *)malloc(sizeof(*tasks) * (cap_tasks ? cap_tasks : 1));
	if (!tasks)
		goto fail;
	/* three-level items: all A tiles, all B tiles, all C tiles */
	for (i = 0; i < nhuge; i++) {
		const struct fftset_fft *f = fs_create_plan(fs, modulation, order[i].bins);
		uint32_t t;
		for (t = 0; t < huges[i].na; t++)
			tasks[ntasks++] = (fgk_task){FGK_TASK_PA, i, t, 0};
		for (t = 0; t < huges[i].nb; t++)
			tasks[ntasks++] = (fgk_task){FGK_TASK_PB, i, t, 0};
		for (t = 0; t < huges[i].nc1 * f->p3.L2; t++)
			tasks[ntasks++] = (fgk_task){FGK_TASK_PC, i, t, 0};
	}
	/* big items: COLS of item b, ROWS of item b - D */
	if (nbig) {
		const uint64_t grid = (uint64_t)fgk_tasks_grid(fs->num_sms);
		const uint64_t avg = (total_cols + nbig - 1) / nbig;
		uint32_t D = (uint32_t)((2 * grid + avg - 1) / avg) + 1, b, t;
		for (b = 0; b < nbig + D; b++) {
			if (b < nbig)
				for (t = 0; t < bigs[b].ncols; t++)
					tasks[ntasks++] = (fgk_task){FGK_TASK_COLS, b, t, 0};
			if (b >= D)
				for (t = 0; t < bigs[b - D].nrows; t++)
					tasks[ntasks++] = (fgk_task){FGK_TASK_ROWS, b - D, t, 0};
		}
	}
	/* small items, largest first */
	{
		uint32_t pi = 0;
		for (i = nhuge + nbig; i < n; i = j) {
			const unsigned L = order[i].bins;
			uint32_t G, tg;
			for (j = i; j < n && order[j].bins == L; j++)
				;
			tg = plans[pi].threads;
			G = plans[pi].per_cta;
			for (; i < j;) {
				const uint32_t m = j - i < G ? j - i : G;
				uint32_t k;
				tasks[ntasks++] = (fgk_task){FGK_TASK_SMALL, pi, nitems, m | (tg << 16)};
				for (k = 0; k < m; k++) {
					items[nitems].in_off = in_offsets[order[i + k].idx];
					items[nitems].out_off = out_offsets[order[i + k].idx];
					nitems++;
				}
				i += m;
			}
			pi++;
		}
	}
	rb->ntasks = ntasks;
	rb->nbig = nbig;
	rb->nhuge = nhuge;
	if ((e = cudaMalloc((void **)&rb->tasks_dev, sizeof(fgk_task) * (ntasks ? ntasks : 1))) != cudaSuccess ||
	    (e = cudaMalloc((void **)&rb->plans_dev, sizeof(fgk_plan) * (nplans ? nplans : 1))) != cudaSuccess ||
	    (e = cudaMalloc((void **)&rb->items_dev, sizeof(fgk_rg_item) * (nitems ? nitems : 1))) != cudaSuccess ||
	    (e = cudaMalloc((void **)&rb->bigs_dev, sizeof(fgk_big) * (nbig ? nbig : 1))) != cudaSuccess ||
	    (e = cudaMalloc((void **)&rb->huges_dev, sizeof(fgk_huge) * (nhuge ? nhuge : 1))) != cudaSuccess ||
	    (e = cudaMalloc((void **)&rb->counters_dev, sizeof(int) * (1 + (size_t)nbig + 2 * (size_t)nhuge))) !=
	        cudaSuccess ||
	    (scratch_f2 && (e = cudaMalloc((void **)&rb->scratch, scratch_f2 * 2 * sizeof(float))) != cudaSuccess))
		goto cuda_fail;
	if ((e = cudaMemcpy(rb->tasks_dev, tasks, sizeof(fgk_task) * ntasks, cudaMemcpyHostToDevice)) != cudaSuccess ||
	    (nplans && (e = cudaMemcpy(rb->plans_dev, plans, sizeof(fgk_plan) * nplans, cudaMemcpyHostToDevice)) !=
	                   cudaSuccess) ||
	    (nitems && (e = cudaMemcpy(rb->items_dev, items, sizeof(fgk_rg_item) * nitems, cudaMemcpyHostToDevice)) !=
	                   cudaSuccess) ||
	    (nbig && (e = cudaMemcpy(rb->bigs_dev, bigs, sizeof(fgk_big) * nbig, cudaMemcpyHostToDevice)) != cudaSuccess) ||
	    (nhuge &&
	     (e = cudaMemcpy(rb->huges_dev, huges, sizeof(fgk_huge) * nhuge, cudaMemcpyHostToDevice)) != cudaSuccess))
		goto cuda_fail;
	if ((e = cudaStreamCreateWithFlags(&rb->cap_stream, cudaStreamNonBlocking)) != cudaSuccess)
		goto cuda_fail;
	free(order);
	free(plans);
	free(items);
	free(bigs);
	free(huges);
	free(tasks);
	return rb;
cuda_fail:
	cudaGetLastError();
	rc = e == cudaErrorMemoryAllocation ? FFTSET_E_NOMEM : FFTSET_E_CUDA;
fail:
	fs_latch(fs, rc, 0);
	free(order);
	free(plans);
	free(items);
	free(bigs);
	free(huges);
	free(tasks);
	fsr_free(rb);
	return NULL;
}

struct fftset_ragged *fftset_ragged_create(struct fftset *fc, const struct fftset_modulation *modulation, int op,
                                           unsigned n, const unsigned *bins, const size_t *in_offsets,
                                           const size_t *out_offsets)
{
	struct fs_impl *fs = fs_impl_of(fc);
	if (!fs)
		return NULL;
	return fsr_create(fs, modulation, op, n, bins, in_offsets, out_offsets);
}

/* the launch sequence, on `s` */
static int fsr_record(struct fftset_ragged *rb, float *out, const float *in, cudaStream_t s)
{
	struct fs_impl *fs = rb->fs;
	return fgk_launch_tasks(rb->tasks_dev, rb->ntasks, rb->plans_dev, rb->items_dev, rb->bigs_dev, rb->nbig,
	                        rb->huges_dev, rb->nhuge, rb->counters_dev, rb->scratch, rb->op, rb->modulation, in, out,
	                        fs->num_sms, fs->dev_flag, s);
}

int fftset_ragged_execute(struct fftset_ragged *rb, float *output_base, const float *input_base)
{
	struct fs_impl *fs;
	int rc;
	cudaError_t e;
	if (!rb || !output_base || !input_base)
		return FFTSET_E_INVALID;
	fs = rb->fs;
	if (!fs_is_device_ptr(output_base) || !fs_is_device_ptr(input_base))
		return fs_latch(fs, FFTSET_E_INVALID, 0); /* ragged batches take device buffers */
	if (!rb->use_graph) {
		rc = fsr_record(rb, output_base, input_base, fs->stream);
		if (rc)
			return fs_latch(fs, FFTSET_E_CUDA, rc);
	} else {
		if (!rb->exec || rb->g_in != input_base || rb->g_out != output_base) {
			cudaGraph_t graph = NULL;
			if (rb->exec) {
				cudaGraphExecDestroy(rb->exec);
				rb->exec = NULL;
			}
			/* an uncaptured run on the caller's stream first (ordered with the
			 * caller's work, same result as the graph): it also sets the
			 * kernels' shared-memory attributes outside the capture */
			if ((rc = fsr_record(rb, output_base, input_base, fs->stream)) != 0)
				return fs_latch(fs, FFTSET_E_CUDA, rc);
			if ((e = cudaStreamBeginCapture(rb->cap_stream, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
				return fs_cuda(fs, e);
			rc = fsr_record(rb, output_base, input_base, rb->cap_stream);
			e = cudaStreamEndCapture(rb->cap_stream, &graph);
			if (rc || e != cudaSuccess) {
				if (graph)
					cudaGraphDestroy(graph);
				return rc ? fs_latch(fs, FFTSET_E_CUDA, rc) : fs_cuda(fs, e);
			}
			e = cudaGraphInstantiate(&rb->exec, graph, 0);
			cudaGraphDestroy(graph);
			if (e != cudaSuccess) {
				rb->exec = NULL;
				return fs_cuda(fs, e);
			}
			rb->g_in = input_base;
			rb->g_out = output_base;
		}
		if ((e = cudaGraphLaunch(rb->exec, fs->stream)) != cudaSuccess)
			return fs_cuda(fs, e);
	}
	if (fs->blocking) {
		if ((rc = fs_cuda(fs, cudaStreamSynchronize(fs->stream))) != 0)
			return rc;
		return fs_check_flag(fs);
	}
	return FFTSET_OK;
}

int fftset_ragged_set_graph(struct fftset_ragged *rb, int enable)
{
	if (!rb)
		return FFTSET_E_INVALID;
	rb->use_graph = enable ? 1 : 0;
	return FFTSET_OK;
}

double fftset_ragged_bytes(const struct fftset_ragged *rb)
{
	return rb ? rb->bytes : 0.0;
}

unsigned fftset_ragged_persistent_items(const struct fftset_ragged *rb)
{
	return rb ? rb->n : 0; /* every item runs in the one persistent launch */
}

/* The plain calls (forward / inverse, device buffers) of a plan beyond the
 * shared-memory limit: `count` items of its size at b * stride, one task
 * launch on `stream`. The task list is kept on the plan for the last (count,
 * strides) seen; the direction is chosen at launch. */
int fs_tasks_batch(struct fftset_fft *f, int op, float *out, size_t out_stride, const float *in, size_t in_stride,
                   unsigned count, cudaStream_t stream)
{
	struct fs_impl *fs = f->fs;
	const size_t nf = 2 * (size_t)f->lfft;
	if (count == 0)
		return 0;
	if (count == 1)
		in_stride = out_stride = nf;
	if (!f->tasks || f->tasks_count != count || f->tasks_in_stride != in_stride ||
	    f->tasks_out_stride != out_stride) {
		unsigned *bins = (unsigned *)malloc(sizeof(unsigned) * count);
		size_t *io = (size_t *)malloc(sizeof(size_t) * count), *oo = (size_t *)malloc(sizeof(size_t) * count);
		unsigned b;
		int err0 = fs->err;
		if (!bins || !io || !oo) {
			free(bins);
			free(io);
			free(oo);
			return -FFTSET_E_NOMEM;
		}
		for (b = 0; b < count; b++) {
			bins[b] = f->lfft;
			io[b] = b * in_stride;
			oo[b] = b * out_stride;
		}
		fsr_free(f->tasks);
		f->tasks = fsr_create(fs, f->modulator, op, count, bins, io, oo);
		free(bins);
		free(io);
		free(oo);
		if (!f->tasks) {
			/* no tile split for this size: the caller falls back; leave the
			 * latched error as it was */
			if (!err0 && fs->err == FFTSET_E_UNSUPPORTED) {
				fs->err = 0;
				fs->cuda_err = 0;
			}
			return -FFTSET_E_UNSUPPORTED;
		}
		f->tasks_count = count;
		f->tasks_in_stride = in_stride;
		f->tasks_out_stride = out_stride;
	}
	f->tasks->op = op; /* the task list does not depend on the direction */
	return fsr_record(f->tasks, out, in, stream);
}

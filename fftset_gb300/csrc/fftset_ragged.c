/* Ragged batches: transforms of many different sizes in one submission, and
 * the task lists of the plain calls of sizes beyond the shared-memory limit.
 *
 * fsr_create plans every distinct size through the fftset's own plan cache
 * (so all sizes share the fftset's twiddle tables) and builds the task list
 * of one persistent launch (fgk_tasks.cuh), every task a tile of at most
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

/* threads of a narrow task CTA: per-size thread counts (tuned or not) stay
 * within it, so they fit every CTA shape */
#define FSR_THREADS ((uint32_t)fgk_tasks_threads(0))

struct fftset_ragged {
	struct fs_impl *fs;
	int             op;
	int             modulation; /* FGK_MOD_* */
	int             shape;      /* CTA shape (enum fgk_task_shape) */
	unsigned        n;
	fgk_task       *tasks_dev;
	uint32_t        ntasks;
	fgk_plan       *plans_dev;
	fgk_rg_item    *items_dev;
	fgk_big        *bigs_dev;
	uint32_t        nbig;
	fgk_huge       *huges_dev;
	uint32_t        nhuge;
	uint32_t        nhcount;    /* the three-level items' counters (fgk_huge.cnt) */
	int            *counters_dev;
	float          *scratch;
	/* graph */
	cudaStream_t    cap_stream;
	cudaGraphExec_t exec;
	const float    *g_in;
	float          *g_out;
	int             use_graph;
	double          bytes;
	/* the creation arguments (a rebuild after autotuning) */
	const struct fftset_modulation *mod;
	unsigned       *bins;
	size_t         *in_offsets, *out_offsets;
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

/* tile counts of a three-level item L1 x L2 x L3 (fgk_huge): A tiles of 16
 * columns, B tiles of 4 x 4 (k1, n3) blocks, C tiles of 16 k1; A and B
 * tiles in L3/16 groups by n3 when 16 divides L3 */
static void fsr_huge_tiles(fgk_huge *h, uint32_t L1, uint32_t L2, uint32_t L3)
{
	h->L1 = L1;
	h->L2 = L2;
	h->L3 = L3;
	h->ngrp = L3 % 16 == 0 ? L3 / 16 : 1;
	h->reserved = 0;
	h->na = (L2 * L3 + 15) / 16;
	h->nb3 = (L3 + 3) / 4;
	h->nb = (L1 + 3) / 4 * h->nb3;
	h->nc1 = (L1 + 15) / 16;
}

/* the k-th of N tiles listed next to its mirror: 0, N-1, 1, N-2, ... */
static uint32_t fsr_zip(int on, uint32_t k, uint32_t N)
{
	return on ? ((k & 1) ? N - 1 - (k >> 1) : k >> 1) : k;
}

/* The tasks of three-level item i (ref i). A tiles slot by slot, a slot
 * being one n3 group of L2 A tiles (tile t = n2 ngrp + u for group u), or
 * with mirror tiles adjacent the pair of groups u and ngrp-1-u (the mirror
 * of tile (u, n2) is (ngrp-1-u, L2-1-n2)). Then the B tiles of the first P
 * slots in the same order: at the A -> B boundary only the groups of the
 * last A tiles are still running, and these B tiles belong to groups
 * finished long before, so they start at once instead of waiting for the
 * whole pass. Then the other slots' B tiles by k1 group of 16 (P slots hold
 * about two grids of B tiles, so every A tile is done by then), and the C
 * tiles by k1 group in the same order: at the B -> C boundary the first C
 * tiles belong to k1 groups finished long before. With one n3 group the B
 * tiles are listed in index order, which is k1 order. The mirror of C tile
 * (k2, g) is (L2-1-k2, nc1-1-g): with mirror tiles adjacent the k1 groups
 * go in pairs g, nc1-1-g. Every tile is listed after the tiles it waits
 * for, so no wait depends on a tile not yet claimed.
 * 15,728,640 bins forward + inverse: 0.535 ms with every A tile before
 * every B tile and every B tile before every C tile; 0.516 with the A -> B
 * boundary opened, 0.496-0.500 with both. group_dist interleaves the A and
 * B passes instead (a test hook sets it), the B tiles of slot s after the
 * A tiles of slot s + D: that measured slower (D = 2: 0.552 ms; D = 9:
 * 0.524 ms), the interleaved B tiles waiting on A tiles still in flight.
 * Returns the tasks written: na + nb + nc1 L2. */
static uint32_t fsr_list_huge(fgk_task *tasks, uint32_t i, const fgk_huge *h, int zip_in, int zip_out, uint32_t grid,
                              uint32_t group_dist)
{
	uint32_t ntasks = 0;
	const uint32_t U = h->ngrp, L2 = h->L2, L1q = h->nb / h->nb3, nc1 = h->nc1;
	const uint32_t nslot = U > 1 && zip_in ? (U + 1) / 2 : U;
	const uint32_t D = group_dist && group_dist < nslot ? group_dist : nslot;
	const uint32_t per_b = (U > 1 && zip_in ? 8 : 4) * L1q; /* B tiles of a slot */
	const uint32_t P = U == 1 ? 0 : D < nslot ? nslot : (2 * grid + per_b - 1) / per_b;
	uint32_t s, t, k, q;
	for (s = 0; s < nslot + D; s++) {
		if (s < nslot) {
			const uint32_t u0 = s, u1 = U - 1 - s;
			if (U == 1)
				for (t = 0; t < h->na; t++)
					tasks[ntasks++] = (fgk_task){FGK_TASK_PA, i, fsr_zip(zip_in, t, h->na), 0};
			else if (!zip_in)
				for (k = 0; k < L2; k++)
					tasks[ntasks++] = (fgk_task){FGK_TASK_PA, i, k * U + u0, 0};
			else if (u0 != u1)
				for (k = 0; k < 2 * L2; k++)
					tasks[ntasks++] = (fgk_task){FGK_TASK_PA, i,
					                             k & 1 ? (L2 - 1 - (k >> 1)) * U + u1 : (k >> 1) * U + u0, 0};
			else
				for (k = 0; k < L2; k++)
					tasks[ntasks++] = (fgk_task){FGK_TASK_PA, i, fsr_zip(1, k, L2) * U + u0, 0};
		}
		if (s >= D && s - D < P) {
			/* the slot's groups, their 4 n3 blocks for every k1 block:
			 * t = k1 block x nb3 + n3 block */
			const uint32_t u0 = s - D, u1 = U - 1 - (s - D);
			for (q = 0; q < (zip_in && u1 != u0 ? 2u : 1u); q++)
				for (k = 0; k < L1q * 4; k++)
					tasks[ntasks++] = (fgk_task){FGK_TASK_PB, i, (k >> 2) * h->nb3 + 4 * (q ? u1 : u0) + (k & 3),
					                             0};
		}
	}
	/* k1 groups in C's order: g = 0, 1, ... or the pairs g, nc1-1-g */
	for (k = 0; k < (zip_out ? (nc1 + 1) / 2 : nc1); k++) {
		const uint32_t g0 = k, g1 = zip_out ? nc1 - 1 - k : k;
		uint32_t g;
		for (g = g0;; g = g1) {
			const uint32_t b1 = 4 * g + 4 < L1q ? 4 * g + 4 : L1q;
			uint32_t b, j;
			if (U == 1) {
				for (b = 4 * g; b < b1; b++)
					for (j = 0; j < h->nb3; j++)
						tasks[ntasks++] = (fgk_task){FGK_TASK_PB, i, b * h->nb3 + j, 0};
			} else {
				for (s = P; s < nslot; s++) {
					const uint32_t u0 = s, u1 = U - 1 - s;
					for (q = 0; q < (zip_in && u1 != u0 ? 2u : 1u); q++)
						for (b = 4 * g; b < b1; b++)
							for (j = 0; j < 4; j++)
								tasks[ntasks++] = (fgk_task){FGK_TASK_PB, i, b * h->nb3 + 4 * (q ? u1 : u0) + j, 0};
				}
			}
			if (g == g1)
				break;
		}
	}
	for (k = 0; k < (zip_out ? (nc1 + 1) / 2 : nc1); k++) {
		const uint32_t g0 = k, g1 = zip_out ? nc1 - 1 - k : k;
		if (g0 == g1)
			for (t = 0; t < L2; t++)
				tasks[ntasks++] = (fgk_task){FGK_TASK_PC, i, fsr_zip(zip_out, t, L2) * nc1 + g0, 0};
		else
			for (t = 0; t < 2 * L2; t++)
				tasks[ntasks++] = (fgk_task){FGK_TASK_PC, i,
				                             t & 1 ? (L2 - 1 - (t >> 1)) * nc1 + g1 : (t >> 1) * nc1 + g0, 0};
	}
	return ntasks;
}

/* Test hook: the task order of one three-level item L1 x L2 x L3 (ref 0),
 * mirror tiles adjacent on the input (zip_in) or the output (zip_out) side,
 * for a grid of `grid` CTAs and A -> B distance group_dist (0: every A tile
 * first); returns the tasks written, 0 when cap is too small. No GPU is
 * involved. */
uint32_t fftset__test_list_huge(uint32_t L1, uint32_t L2, uint32_t L3, int zip_in, int zip_out, uint32_t grid,
                                uint32_t group_dist, fgk_task *out, uint32_t cap)
{
	fgk_huge h;
	memset(&h, 0, sizeof(h));
	fsr_huge_tiles(&h, L1, L2, L3);
	if ((uint64_t)h.na + h.nb + (uint64_t)h.nc1 * L2 > cap)
		return 0;
	return fsr_list_huge(out, 0, &h, zip_in, zip_out, grid, group_dist);
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
	free(rb->bins);
	free(rb->in_offsets);
	free(rb->out_offsets);
	free(rb);
}

void fftset_ragged_destroy(struct fftset_ragged *rb)
{
	fsr_free(rb);
}

/* why the calling thread's last fsr_create returned NULL (FFTSET_E_*) */
static __thread int fsr_why;

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
	unsigned i, j, nplans = 0, nitems = 0, nbig = 0, nhuge = 0, nhcount = 0, ntasks = 0, cap_tasks = 0;
	uint32_t max_stages = 0; /* the longest chain of any tile of the list */
	int three_level = 0;
	size_t scratch_f2 = 0;
	uint64_t total_cols = 0;
	cudaError_t e;
	int rc = FFTSET_E_NOMEM;

	fsr_why = FFTSET_E_INVALID;
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
		if (bins[i] > 65536)
			three_level = 1;
	}
	/* the shape is settled once the plans (their chains) are known below;
	 * the SMALL tasks are packed for 128-thread CTAs meanwhile, which every
	 * shape runs */
	rb->shape = fs->task_shape >= 0 ? fs->task_shape : FGK_SHAPE_NARROW;
	qsort(order, n, sizeof(*order), fsr_cmp);

	/* plans, items and big items; SMALL tasks are counted here, listed below */
	for (i = 0; i < n; i = j) {
		const unsigned L = order[i].bins;
		struct fftset_fft *f = fs_create_plan(fs, modulation, L);
		for (j = i; j < n && order[j].bins == L; j++)
			;
		if (!f) {
			rc = fs_plan_error();
			goto fail;
		}
		if (!f->fourstep && L <= (uint32_t)fgk_tasks_points()) {
			const fgk_plan *pl = f->rg_tuned && f->rg_dmem ? &f->rg_plan : &f->rp;
			const uint32_t tg = f->rg_tuned ? f->rg_tg : fsr_item_threads(pl);
			uint32_t G = (uint32_t)fgk_tasks_threads(rb->shape) / tg;
			if (!pl->fwd.code) { /* tiles take chains of at most 15 stages */
				rc = FFTSET_E_UNSUPPORTED;
				goto fail;
			}
			if (pl->fwd.nstages > max_stages)
				max_stages = pl->fwd.nstages;
			if (G * fsr_slots(L) > (uint32_t)fgk_tasks_slots())
				G = (uint32_t)fgk_tasks_slots() / fsr_slots(L);
			plans[nplans] = *pl;
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
			if (!p3->c1.code || !p3->c2.code || !p3->c3.code) {
				rc = FFTSET_E_UNSUPPORTED;
				goto fail;
			}
			for (k = 0; k < 3; k++) {
				const uint32_t ns = (k == 0 ? p3->c1 : k == 1 ? p3->c2 : p3->c3).nstages;
				if (ns > max_stages)
					max_stages = ns;
			}
			for (k = i; k < j; k++) {
				fgk_huge *h = &huges[nhuge++];
				/* each scratch area in 4 x 4 blocks: L2 ceil(L1/4) ceil(L3/4) x 16 */
				const size_t span = (size_t)p3->L2 * ((p3->L1 + 3) / 4) * ((p3->L3 + 3) / 4) * 16;
				h->p3 = p3->dev;
				fsr_huge_tiles(h, p3->L1, p3->L2, p3->L3);
				h->cnt = nhcount;
				h->code1 = p3->c1.code;
				h->code2 = p3->c2.code;
				h->code3 = p3->c3.code;
				h->in_off = in_offsets[order[k].idx];
				h->out_off = out_offsets[order[k].idx];
				h->sa = scratch_f2;
				h->sb = scratch_f2 + span;
				scratch_f2 += 2 * span;
				nhcount += h->ngrp + h->nc1;
				cap_tasks += h->na + h->nb + h->nc1 * p3->L2;
			}
		} else {
			uint32_t L1, L2, k;
			if ((rc = fs_ensure_fourstep(fs, f)) != 0)
				goto fail;
			L1 = f->p4.L1;
			L2 = f->p4.L2;
			/* tiles of 16 or more lanes (the task kernel's Rows layout) */
			if ((L1 << 4) > (uint32_t)fgk_tasks_points() || (L2 << 4) > (uint32_t)fgk_tasks_points() ||
			    !f->p4.c1.code || !f->p4.c2.code) {
				rc = FFTSET_E_UNSUPPORTED;
				goto fail;
			}
			if (f->p4.c1.nstages > max_stages)
				max_stages = f->p4.c1.nstages;
			if (f->p4.c2.nstages > max_stages)
				max_stages = f->p4.c2.nstages;
			for (k = i; k < j; k++) {
				fgk_big *b = &bigs[nbig++];
				b->p4 = f->p4.dev;
				b->L1 = L1;
				b->L2 = L2;
				b->code1 = f->p4.c1.code;
				b->code2 = f->p4.c2.code;
				b->in_off = in_offsets[order[k].idx];
				b->out_off = out_offsets[order[k].idx];
				b->scratch_off = scratch_f2;
				b->ls1 = f->rg_tuned ? f->rg_ls1 : fsr_lanes_log2(L1, L2);
				b->ls2 = f->rg_tuned ? f->rg_ls2 : fsr_lanes_log2(L2, L1);
				b->ncols = (L2 + (1u << b->ls1) - 1) >> b->ls1;
				b->nrows = (L1 + (1u << b->ls2) - 1) >> b->ls2;
				total_cols += b->ncols;
				cap_tasks += b->ncols + b->nrows;
				/* laid out by ROWS tiles (full tiles), 128-byte aligned items */
				scratch_f2 += ((((size_t)b->nrows * L2) << b->ls2) + 15) & ~(size_t)15;
			}
		}
	}
	/* Chains of two stages at most run on six single-buffer CTAs per SM
	 * (the 15,728,640-bin pair: 0.529 against 0.604 ms on wide CTAs; the
	 * mix's two-stage two-level items: 0.775 against 0.820 ms on narrow
	 * ones); otherwise three-level lists on wide CTAs, the rest on narrow
	 * ones. One tile buffer cannot hold a longer chain. */
	if (fs->task_shape < 0)
		rb->shape = max_stages <= 2 ? FGK_SHAPE_SINGLE : three_level ? FGK_SHAPE_WIDE : FGK_SHAPE_NARROW;
	else if (rb->shape == FGK_SHAPE_SINGLE && max_stages > 2) {
		rc = FFTSET_E_UNSUPPORTED;
		goto fail;
	}
	/* one buffer: the G items of a SMALL task use buffer slots from 2 g
	 * rslots(L) on (g < G), so they reach (2 G - 1) rslots(L); threads per
	 * item are a multiple of 32, so G <= 4, and two-stage sizes have L <=
	 * 256: this always holds, and is checked all the same */
	if (rb->shape == FGK_SHAPE_SINGLE)
		for (j = 0; j < nplans; j++)
			if ((2 * plans[j].per_cta - 1) * fsr_slots(plans[j].L) > (uint32_t)fgk_tasks_slots()) {
				rc = FFTSET_E_UNSUPPORTED;
				goto fail;
			}
	tasks = (fgk_task *)malloc(sizeof(*tasks) * (cap_tasks ? cap_tasks : 1));
	if (!tasks)
		goto fail;
	/* FREQ_OFFSET_REAL keeps bin m and its mirror L-1-m in one 16-byte pair
	 * (X[2m] = W[m], X[2m+1] = conj W[L-1-m]): the tiles writing the
	 * forward's output (ROWS, C) and those reading the inverse's input
	 * (COLS, A) are listed next to their mirror tile, the one holding the
	 * mirrored bins (tile t of N mirrors tile N-1-t), so that both halves
	 * of every pair meet in L2 within microseconds and reach HBM as whole
	 * sectors instead of two partial writes (or reads) far apart. */
	const int zip_in = rb->modulation == FGK_MOD_FREQOFF && op == FFTSET_OP_INVERSE;
	const int zip_out = rb->modulation == FGK_MOD_FREQOFF && op == FFTSET_OP_FORWARD;
	/* three-level items: the order is described at fsr_list_huge */
	for (i = 0; i < nhuge; i++)
		ntasks += fsr_list_huge(tasks + ntasks, i, &huges[i], zip_in, zip_out,
		                        (uint32_t)fgk_tasks_grid(fs->num_sms, rb->shape), fs->group_dist);
	/* big items: COLS of item b, ROWS of item b - D */
	if (nbig) {
		const uint64_t grid = (uint64_t)fgk_tasks_grid(fs->num_sms, rb->shape);
		const uint64_t avg = (total_cols + nbig - 1) / nbig;
		uint32_t D = (uint32_t)((2 * grid + avg - 1) / avg) + 1, b, t;
		for (b = 0; b < nbig + D; b++) {
			if (b < nbig)
				for (t = 0; t < bigs[b].ncols; t++)
					tasks[ntasks++] = (fgk_task){FGK_TASK_COLS, b, fsr_zip(zip_in, t, bigs[b].ncols), 0};
			if (b >= D)
				for (t = 0; t < bigs[b - D].nrows; t++)
					tasks[ntasks++] = (fgk_task){FGK_TASK_ROWS, b - D, fsr_zip(zip_out, t, bigs[b - D].nrows), 0};
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
	rb->nhcount = nhcount;
	if ((e = cudaMalloc((void **)&rb->tasks_dev, sizeof(fgk_task) * (ntasks ? ntasks : 1))) != cudaSuccess ||
	    (e = cudaMalloc((void **)&rb->plans_dev, sizeof(fgk_plan) * (nplans ? nplans : 1))) != cudaSuccess ||
	    (e = cudaMalloc((void **)&rb->items_dev, sizeof(fgk_rg_item) * (nitems ? nitems : 1))) != cudaSuccess ||
	    (e = cudaMalloc((void **)&rb->bigs_dev, sizeof(fgk_big) * (nbig ? nbig : 1))) != cudaSuccess ||
	    (e = cudaMalloc((void **)&rb->huges_dev, sizeof(fgk_huge) * (nhuge ? nhuge : 1))) != cudaSuccess ||
	    (e = cudaMalloc((void **)&rb->counters_dev, sizeof(int) * (1 + (size_t)nbig + (size_t)nhcount))) !=
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
	rb->mod = modulation;
	rb->bins = (unsigned *)malloc(sizeof(unsigned) * n);
	rb->in_offsets = (size_t *)malloc(sizeof(size_t) * n);
	rb->out_offsets = (size_t *)malloc(sizeof(size_t) * n);
	if (!rb->bins || !rb->in_offsets || !rb->out_offsets)
		goto fail;
	memcpy(rb->bins, bins, sizeof(unsigned) * n);
	memcpy(rb->in_offsets, in_offsets, sizeof(size_t) * n);
	memcpy(rb->out_offsets, out_offsets, sizeof(size_t) * n);
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
	fsr_why = rc;
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
	struct fftset_ragged *rb;
	if (!fs)
		return NULL;
	/* plans and their on-demand tables are shared with the execution calls */
	pthread_mutex_lock(&fs->lock);
	rb = fsr_create(fs, modulation, op, n, bins, in_offsets, out_offsets);
	pthread_mutex_unlock(&fs->lock);
	return rb;
}

/* the launch sequence of direction `op`, on `s` (a task list does not
 * depend on the direction) */
static int fsr_record_product(struct fftset_ragged *rb, int op, float *out, const float *in, cudaStream_t s,
                              const fgk_product *prod)
{
	struct fs_impl *fs = rb->fs;
	const fgk_product none = {NULL};
	return fgk_launch_tasks(rb->tasks_dev, rb->ntasks, rb->plans_dev, rb->items_dev, rb->bigs_dev, rb->nbig,
	                        rb->huges_dev, rb->nhcount, rb->counters_dev, rb->scratch, op, rb->modulation, in, out,
	                        fs->num_sms, rb->shape, fs->dev_flag, fs->spin_limit, prod ? *prod : none, s);
}

static int fsr_record(struct fftset_ragged *rb, int op, float *out, const float *in, cudaStream_t s)
{
	return fsr_record_product(rb, op, out, in, s, NULL);
}

/* Test hook: removes the batch's tasks of one kind (FGK_TASK_*), so that
 * the tasks that wait on them run into their bounded waits; the graph is
 * recorded again at the next execute. */
int fftset__test_ragged_drop_kind(struct fftset_ragged *rb, int kind)
{
	fgk_task *t;
	uint32_t i, n = 0;
	cudaError_t e;
	if (!rb)
		return FFTSET_E_INVALID;
	cudaStreamSynchronize(rb->fs->stream);
	t = (fgk_task *)malloc(sizeof(*t) * (rb->ntasks ? rb->ntasks : 1));
	if (!t)
		return FFTSET_E_NOMEM;
	if ((e = cudaMemcpy(t, rb->tasks_dev, sizeof(*t) * rb->ntasks, cudaMemcpyDeviceToHost)) != cudaSuccess) {
		free(t);
		return fs_cuda(rb->fs, e);
	}
	for (i = 0; i < rb->ntasks; i++)
		if ((int)t[i].kind != kind)
			t[n++] = t[i];
	e = cudaMemcpy(rb->tasks_dev, t, sizeof(*t) * n, cudaMemcpyHostToDevice);
	free(t);
	if (e != cudaSuccess)
		return fs_cuda(rb->fs, e);
	rb->ntasks = n;
	if (rb->exec) {
		cudaGraphExecDestroy(rb->exec);
		rb->exec = NULL;
	}
	return FFTSET_OK;
}

static int fsr_execute(struct fftset_ragged *rb, float *output_base, const float *input_base);

/* Several threads may execute batches of one fftset (and the same batch):
 * the launch and the graph it may re-instantiate are made under the
 * fftset's lock; the wait for the results is not. */
int fftset_ragged_execute(struct fftset_ragged *rb, float *output_base, const float *input_base)
{
	struct fs_impl *fs;
	int rc;
	if (!rb || !output_base || !input_base)
		return FFTSET_E_INVALID;
	fs = rb->fs;
	if (!fs_is_device_ptr(output_base) || !fs_is_device_ptr(input_base))
		return fs_latch(fs, FFTSET_E_INVALID, 0); /* ragged batches take device buffers */
	FS_RANGE_PUSH("fftset_ragged_execute");
	pthread_mutex_lock(&fs->lock);
	rc = fsr_execute(rb, output_base, input_base);
	pthread_mutex_unlock(&fs->lock);
	if (rc == 0 && fs->blocking && (rc = fs_cuda(fs, cudaStreamSynchronize(fs->stream))) == 0)
		rc = fs_check_flag(fs);
	FS_RANGE_POP();
	return rc;
}

static int fsr_execute(struct fftset_ragged *rb, float *output_base, const float *input_base)
{
	struct fs_impl *fs = rb->fs;
	int rc;
	cudaError_t e;
	if (!rb->use_graph) {
		rc = fsr_record(rb, rb->op, output_base, input_base, fs->stream);
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
			if ((rc = fsr_record(rb, rb->op, output_base, input_base, fs->stream)) != 0)
				return fs_latch(fs, FFTSET_E_CUDA, rc);
			if ((e = cudaStreamBeginCapture(rb->cap_stream, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
				return fs_cuda(fs, e);
			rc = fsr_record(rb, rb->op, output_base, input_base, rb->cap_stream);
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
 * launch on `stream`. The plan keeps the task lists of the last
 * FS_TASK_LISTS shapes (count, strides) it ran, so that callers alternating
 * between a few shapes (the adjoint's sub-batches, single calls between
 * batches) do not rebuild one per call; the direction is a launch argument.
 * Called with fs->lock held: the lists are shared by all threads calling
 * this plan, and a list being replaced is freed only after the stream's
 * earlier launches, which may use it, have finished (fsr_free). */
int fs_tasks_batch(struct fftset_fft *f, int op, float *out, size_t out_stride, const float *in, size_t in_stride,
                   unsigned count, cudaStream_t stream, const fgk_product *prod)
{
	struct fs_impl *fs = f->fs;
	const size_t nf = 2 * (size_t)f->lfft;
	struct fs_tasklist *t = NULL;
	unsigned k;
	if (count == 0)
		return 0;
	if (count == 1)
		in_stride = out_stride = nf;
	/* FREQ_OFFSET_REAL lists order their tiles for one direction (mirror
	 * pairs, fsr_create); COMPLEX lists serve both */
	const int key_op = f->modulator->freq_offset_real ? op : -1;
	for (k = 0; k < FS_TASK_LISTS && !t; k++)
		if (f->tl[k].rb && f->tl[k].count == count && f->tl[k].in_stride == in_stride &&
		    f->tl[k].out_stride == out_stride && f->tl[k].op == key_op)
			t = &f->tl[k];
	if (!t) {
		unsigned *bins = (unsigned *)malloc(sizeof(unsigned) * count);
		size_t *io = (size_t *)malloc(sizeof(size_t) * count), *oo = (size_t *)malloc(sizeof(size_t) * count);
		struct fftset_ragged *rb;
		unsigned b;
		const int err0 = __atomic_load_n(&fs->err, __ATOMIC_ACQUIRE);
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
		rb = fsr_create(fs, f->modulator, op, count, bins, io, oo);
		free(bins);
		free(io);
		free(oo);
		if (!rb) {
			/* no tile split for this size: the caller falls back; leave the
			 * latched error as it was. Other failures (memory) are the
			 * call's. */
			int unsup = FFTSET_E_UNSUPPORTED;
			if (fsr_why != FFTSET_E_UNSUPPORTED)
				return -(fsr_why ? fsr_why : FFTSET_E_NOMEM);
			if (!err0 && __atomic_compare_exchange_n(&fs->err, &unsup, 0, 0, __ATOMIC_ACQ_REL, __ATOMIC_ACQUIRE))
				__atomic_store_n(&fs->cuda_err, 0, __ATOMIC_RELEASE);
			return -FFTSET_E_UNSUPPORTED;
		}
		/* an empty slot, else the least recently used list */
		t = &f->tl[0];
		for (k = 0; k < FS_TASK_LISTS; k++) {
			if (!f->tl[k].rb) {
				t = &f->tl[k];
				break;
			}
			if (f->tl[k].used < t->used)
				t = &f->tl[k];
		}
		fsr_free(t->rb);
		t->rb = rb;
		t->count = count;
		t->in_stride = in_stride;
		t->out_stride = out_stride;
		t->op = key_op;
	}
	t->used = ++f->tl_clock;
	return fsr_record_product(t->rb, op, out, in, stream, prod);
}

/* ------------------------------------------------------------------------
 * Autotuning the task schedule per size */

/* Device tables of a whole-item chain candidate (the resident plan with a
 * forced radix order); *dmem receives the allocation. */
static int fsr_candidate_plan(struct fs_impl *fs, const struct fftset_fft *f, const uint32_t *rad, uint32_t n,
                              fgk_plan *out, void **dmem)
{
	const uint32_t L = f->lfft;
	size_t ntw;
	float *h;
	cudaError_t e;
	if (fgk_plan_resident(out, L, f->rp.modulation, fs->max_smem, rad, n))
		return FFTSET_E_UNSUPPORTED;
	ntw = fgk_plan_twiddles(out, NULL);
	h = (float *)malloc(sizeof(float) * 2 * (ntw ? ntw : 1));
	if (!h)
		return FFTSET_E_NOMEM;
	fgk_plan_twiddles(out, h);
	if ((e = cudaMalloc(dmem, sizeof(float) * 2 * (ntw ? ntw : 1))) != cudaSuccess) {
		free(h);
		cudaGetLastError();
		return FFTSET_E_NOMEM;
	}
	e = cudaMemcpy(*dmem, h, sizeof(float) * 2 * ntw, cudaMemcpyHostToDevice);
	free(h);
	if (e != cudaSuccess) {
		cudaFree(*dmem);
		*dmem = NULL;
		return FFTSET_E_CUDA;
	}
	out->tw = *dmem;
	out->modtw = f->rp.modtw;
	out->kidx = f->rp.kidx;
	out->kvw = f->rp.kvw;
	out->dev = NULL; /* the task kernel reads the plan from its own array */
	return FFTSET_OK;
}

/* Times one launch schedule of `count` items of f's size (the current
 * rg_* fields), best of a few launches. */
static float fsr_time_size(struct fs_impl *fs, struct fftset_fft *f, int op, unsigned count, float *buf_in,
                           float *buf_out, cudaEvent_t e0, cudaEvent_t e1)
{
	unsigned *bins = (unsigned *)malloc(sizeof(unsigned) * count);
	size_t *offs = (size_t *)malloc(sizeof(size_t) * count);
	struct fftset_ragged *rb;
	float best = -1.f;
	unsigned b;
	int r;
	if (!bins || !offs) {
		free(bins);
		free(offs);
		return -1.f;
	}
	for (b = 0; b < count; b++) {
		bins[b] = f->lfft;
		offs[b] = (size_t)b * 2 * f->lfft;
	}
	rb = fsr_create(fs, f->modulator, op, count, bins, offs, offs);
	free(bins);
	free(offs);
	if (!rb)
		return -1.f;
	if (fsr_record(rb, op, buf_out, buf_in, fs->stream) == 0) {
		for (r = 0; r < 3; r++) {
			float ms = 0.f;
			cudaEventRecord(e0, fs->stream);
			fsr_record(rb, op, buf_out, buf_in, fs->stream);
			cudaEventRecord(e1, fs->stream);
			if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
				break;
			if (best < 0.f || ms < best)
				best = ms;
		}
	}
	cudaStreamSynchronize(fs->stream);
	cudaGetLastError();
	fsr_free(rb);
	return best;
}

/* Applies a saved per-size schedule (fftset_tuning_load): items up to a
 * tile get the chain rad[0..n) (n == 0: the plan's own chain) with tg
 * threads each; two-level items get 2^ls1 / 2^ls2 lanes per COLS / ROWS
 * tile. The same checks as the autotuner's candidates. */
int fsr_apply_schedule(struct fs_impl *fs, struct fftset_fft *f, const uint32_t *rad, uint32_t n, uint32_t tg,
                       uint32_t ls1, uint32_t ls2)
{
	const uint32_t L = f->lfft;
	int rc;
	if (L > 65536)
		return FFTSET_E_UNSUPPORTED;
	if (!f->fourstep && L <= (uint32_t)fgk_tasks_points()) {
		fgk_plan cand = f->rp;
		void *dm = NULL;
		uint32_t k, same = n == f->rp.fwd.nstages;
		if (tg == 0 || tg > FSR_THREADS || (tg & 31))
			return FFTSET_E_INVALID;
		for (k = 0; same && k < n; k++)
			same = rad[k] == f->rp.fwd.st[k].radix;
		if (n && !same && (rc = fsr_candidate_plan(fs, f, rad, n, &cand, &dm)) != FFTSET_OK)
			return rc;
		if (f->rg_dmem)
			cudaFree(f->rg_dmem);
		f->rg_plan = cand;
		f->rg_dmem = dm;
		f->rg_tg = tg;
		f->rg_tuned = 1;
		return FFTSET_OK;
	}
	if ((rc = fs_ensure_fourstep(fs, f)) != FFTSET_OK)
		return rc;
	if (ls1 < 4 || ls2 < 4 || ls1 > fsr_lanes_log2(f->p4.L1, f->p4.L2) || ls2 > fsr_lanes_log2(f->p4.L2, f->p4.L1))
		return FFTSET_E_INVALID;
	f->rg_ls1 = ls1;
	f->rg_ls2 = ls2;
	f->rg_tuned = 1;
	return FFTSET_OK;
}

static int fsr_autotune(struct fftset_ragged *rb);

/* Changes the schedules of the fftset's plans: under the fftset's lock. */
int fftset_ragged_autotune(struct fftset_ragged *rb)
{
	int rc;
	if (!rb || !rb->bins)
		return FFTSET_E_INVALID;
	pthread_mutex_lock(&rb->fs->lock);
	rc = fsr_autotune(rb);
	pthread_mutex_unlock(&rb->fs->lock);
	return rc;
}

static int fsr_autotune(struct fftset_ragged *rb)
{
	struct fs_impl *fs;
	float *bin = NULL, *bout = NULL;
	cudaEvent_t e0 = NULL, e1 = NULL;
	unsigned i, maxL = 0;
	size_t cap;
	struct fftset_ragged *nrb;
	int rc = FFTSET_OK;
	if (!rb || !rb->bins)
		return FFTSET_E_INVALID;
	fs = rb->fs;
	for (i = 0; i < rb->n; i++)
		if (rb->bins[i] > maxL)
			maxL = rb->bins[i];
	/* timing buffers: 32 MB of items, at least two items of the largest size */
	cap = (size_t)8 << 20;
	if (cap < 4 * (size_t)maxL)
		cap = 4 * (size_t)maxL;
	if (cudaMalloc((void **)&bin, cap * sizeof(float)) != cudaSuccess ||
	    cudaMalloc((void **)&bout, cap * sizeof(float)) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
	    cudaEventCreate(&e1) != cudaSuccess) {
		cudaGetLastError();
		rc = fs_latch(fs, FFTSET_E_NOMEM, 0);
		goto out;
	}
	cudaMemsetAsync(bin, 0, cap * sizeof(float), fs->stream);
	for (i = 0; i < rb->n; i++) {
		struct fftset_fft *f = fs_create_plan(fs, rb->mod, rb->bins[i]);
		const uint32_t L = rb->bins[i];
		const unsigned count = (unsigned)(cap / (2 * (size_t)L));
		float best = -1.f, t;
		if (!f || f->rg_tuned || L > 65536)
			continue;
		if (!f->fourstep && L <= (uint32_t)fgk_tasks_points()) {
			/* whole items: radix order x threads per item */
			uint32_t rad[3][FGK_MAX_STAGES], nr[3] = {0, 0, 0}, nc = 0, c, k, tgs[3], ntg, q;
			fgk_plan best_plan = f->rp;
			void *best_dmem = NULL;
			uint32_t best_tg = fsr_item_threads(&f->rp);
			nr[0] = f->rp.fwd.nstages;
			for (k = 0; k < nr[0]; k++)
				rad[0][k] = f->rp.fwd.st[k].radix;
			nc = 1;
			if (nr[0] > 1) { /* reversed order: smallest radix first (unless it is the same chain) */
				uint32_t pal = 1;
				nr[1] = nr[0];
				for (k = 0; k < nr[0]; k++) {
					rad[1][k] = rad[0][nr[0] - 1 - k];
					pal &= rad[1][k] == rad[0][k];
				}
				nc = pal ? 1 : 2;
			}
			for (c = 0; c < nc; c++) {
				fgk_plan cand;
				void *dm = NULL;
				if (c == 0) {
					cand = f->rp;
				} else if (fsr_candidate_plan(fs, f, rad[c], nr[c], &cand, &dm) != FFTSET_OK) {
					continue;
				}
				/* threads per item: narrowest stage, 2x that, widest stage */
				tgs[0] = fsr_item_threads(&cand);
				tgs[1] = tgs[0] * 2 > FSR_THREADS ? FSR_THREADS : tgs[0] * 2;
				{
					uint32_t s2, w = 1;
					for (s2 = 0; s2 < cand.fwd.nstages; s2++)
						if (L / cand.fwd.st[s2].radix > w)
							w = L / cand.fwd.st[s2].radix;
					w = (w + 31) & ~31u;
					tgs[2] = w > FSR_THREADS ? FSR_THREADS : w;
				}
				ntg = 3;
				for (q = 0; q < ntg; q++) {
					if (q > 0 && (tgs[q] == tgs[q - 1] || (q == 2 && tgs[2] == tgs[0])))
						continue;
					f->rg_tuned = 1;
					f->rg_plan = cand;
					f->rg_dmem = c ? dm : NULL;
					f->rg_tg = tgs[q];
					t = fsr_time_size(fs, f, rb->op, count, bin, bout, e0, e1);
					if (t > 0.f && (best < 0.f || t < best)) {
						best = t;
						best_plan = cand;
						best_tg = tgs[q];
						if (best_dmem && best_dmem != dm)
							cudaFree(best_dmem);
						best_dmem = c ? dm : NULL;
					}
				}
				if (dm && dm != best_dmem)
					cudaFree(dm);
			}
			f->rg_plan = best_plan;
			f->rg_dmem = best_dmem;
			f->rg_tg = best_tg;
			f->rg_tuned = 1;
		} else {
			/* two-level items: lanes per COLS / ROWS tile (16 and up) */
			uint32_t da, db, ls1m, ls2m, best1, best2;
			if (fs_ensure_fourstep(fs, f) != FFTSET_OK)
				continue;
			ls1m = fsr_lanes_log2(f->p4.L1, f->p4.L2);
			ls2m = fsr_lanes_log2(f->p4.L2, f->p4.L1);
			best1 = ls1m;
			best2 = ls2m;
			for (da = 0; da < 2; da++)
				for (db = 0; db < 2; db++) {
					if (ls1m < 4 + da || ls2m < 4 + db)
						continue;
					f->rg_tuned = 1;
					f->rg_ls1 = ls1m - da;
					f->rg_ls2 = ls2m - db;
					t = fsr_time_size(fs, f, rb->op, count, bin, bout, e0, e1);
					if (t > 0.f && (best < 0.f || t < best)) {
						best = t;
						best1 = ls1m - da;
						best2 = ls2m - db;
					}
				}
			f->rg_ls1 = best1;
			f->rg_ls2 = best2;
			f->rg_tuned = 1;
		}
	}
	/* rebuild this batch with the chosen schedules */
	nrb = fsr_create(fs, rb->mod, rb->op, rb->n, rb->bins, rb->in_offsets, rb->out_offsets);
	if (!nrb) {
		rc = fs->err ? fs->err : FFTSET_E_NOMEM;
		goto out;
	}
	{
		struct fftset_ragged tmp = *rb;
		nrb->use_graph = rb->use_graph;
		*rb = *nrb;
		*nrb = tmp; /* the old lists go with nrb */
		nrb->exec = tmp.exec;
		fsr_free(nrb);
	}
out:
	if (e0)
		cudaEventDestroy(e0);
	if (e1)
		cudaEventDestroy(e1);
	cudaFree(bin);
	cudaFree(bout);
	return rc;
}

/* Ragged batches: transforms of many different sizes in one submission.
 *
 * fftset_ragged_create plans every distinct size through the fftset's own
 * plan cache (fftset_create_fft, so all sizes share the fftset's twiddle
 * tables), sorts the items by size, and builds the device work list:
 *   - items whose two ping-pong buffers fit one CTA's shared memory go to one
 *     persistent launch (fgk_ragged.cu) as chunks of same-size items, largest
 *     first, claimed by CTAs from an atomic counter;
 *   - larger items run the four-step passes with an item list, by size, in
 *     sub-batches that share one work buffer.
 * fftset_ragged_execute records that sequence into a CUDA graph on first use
 * (and when the base pointers change) and replays the graph afterwards. */
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include "fftset.h"
#include "fftset_internal.h"
#include "fgk.h"

#define FSR_WORK_CAP ((size_t)512 << 20) /* bytes of four-step work buffer */

struct fsr_big {
	const struct fftset_fft *f;
	uint32_t                 first, count; /* into the device item array */
};

struct fftset_ragged {
	struct fs_impl *fs;
	int             op;
	unsigned        n;
	/* persistent part */
	fgk_plan       *plans_dev;
	fgk_rg_chunk   *chunks_dev;
	uint32_t        nchunks;
	fgk_rg_item    *items_dev;
	int            *counter_dev;
	/* four-step part */
	struct fsr_big *big;
	uint32_t        nbig;
	float          *work;
	size_t          work_floats;
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

/* threads per item of a persistent chunk: enough for the widest stage, a
 * multiple of 32, at most the CTA */
static uint32_t fsr_item_threads(const fgk_plan *p)
{
	uint32_t s, w = 1;
	for (s = 0; s < p->fwd.nstages; s++) {
		uint32_t nbf = p->L / p->fwd.st[s].radix;
		if (nbf > w)
			w = nbf;
	}
	w = (w + 31) & ~31u;
	return w > 512 ? 512 : w;
}

void fftset_ragged_destroy(struct fftset_ragged *rb)
{
	if (!rb)
		return;
	if (rb->fs)
		cudaStreamSynchronize(rb->fs->stream);
	if (rb->exec)
		cudaGraphExecDestroy(rb->exec);
	if (rb->cap_stream)
		cudaStreamDestroy(rb->cap_stream);
	cudaFree(rb->plans_dev);
	cudaFree(rb->chunks_dev);
	cudaFree(rb->items_dev);
	cudaFree(rb->counter_dev);
	cudaFree(rb->work);
	free(rb->big);
	free(rb);
}

struct fftset_ragged *fftset_ragged_create(struct fftset *fc, const struct fftset_modulation *modulation, int op,
                                           unsigned n, const unsigned *bins, const size_t *in_offsets,
                                           const size_t *out_offsets)
{
	struct fs_impl *fs = fs_impl_of(fc);
	struct fftset_ragged *rb = NULL;
	struct fsr_sort *order = NULL;
	fgk_plan *plans = NULL;
	fgk_rg_chunk *chunks = NULL;
	fgk_rg_item *items = NULL;
	unsigned i, j, nplans = 0, nchunks = 0, nitems = 0;
	const size_t smem = fgk_ragged_smem_bytes();
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
	chunks = (fgk_rg_chunk *)calloc(n, sizeof(*chunks));
	items = (fgk_rg_item *)calloc(n, sizeof(*items));
	if (!rb || !order || !plans || !chunks || !items)
		goto fail;
	rb->fs = fs;
	rb->op = op;
	rb->n = n;
	rb->use_graph = 1;
	for (i = 0; i < n; i++) {
		order[i].bins = bins[i];
		order[i].idx = i;
		rb->bytes += 16.0 * bins[i];
	}
	qsort(order, n, sizeof(*order), fsr_cmp);

	/* pass 1: persistent chunks for the sizes whose ping-pong buffers fit */
	for (i = 0; i < n;) {
		const unsigned L = order[i].bins;
		const struct fftset_fft *f = fftset_create_fft(fc, modulation, L);
		size_t per_item;
		unsigned G, tg, cnt, m;
		for (j = i; j < n && order[j].bins == L; j++)
			;
		cnt = j - i;
		if (!f) {
			rc = FFTSET_E_INVALID;
			goto fail;
		}
		per_item = 2 * ((size_t)L + L / 16 + 1) * 8;
		if (f->fourstep || per_item > smem) {
			i = j; /* second pass */
			continue;
		}
		plans[nplans] = f->rp;
		tg = fsr_item_threads(&f->rp);
		G = 512 / tg;
		if ((size_t)G * per_item > smem)
			G = (unsigned)(smem / per_item);
		for (; i < j; i += m) {
			unsigned k;
			m = j - i < G ? j - i : G;
			chunks[nchunks].plan = nplans;
			chunks[nchunks].first = nitems;
			chunks[nchunks].n = m;
			chunks[nchunks].tg = tg;
			nchunks++;
			for (k = 0; k < m; k++) {
				items[nitems].in_off = in_offsets[order[i + k].idx];
				items[nitems].out_off = out_offsets[order[i + k].idx];
				nitems++;
			}
		}
		nplans++;
	}
	/* pass 2: four-step items, grouped by size */
	for (i = 0; i < n;) {
		const unsigned L = order[i].bins;
		struct fftset_fft *f = (struct fftset_fft *)fftset_create_fft(fc, modulation, L);
		size_t per_item = 2 * ((size_t)L + L / 16 + 1) * 8;
		for (j = i; j < n && order[j].bins == L; j++)
			;
		if (f->fourstep || per_item > smem) {
			struct fsr_big *nb;
			if ((rc = fs_ensure_fourstep(fs, f)) != 0)
				goto fail;
			nb = (struct fsr_big *)realloc(rb->big, sizeof(*nb) * (rb->nbig + 1));
			if (!nb)
				goto fail;
			rb->big = nb;
			rb->big[rb->nbig].f = f;
			rb->big[rb->nbig].first = nitems;
			rb->big[rb->nbig].count = j - i;
			rb->nbig++;
			for (; i < j; i++) {
				items[nitems].in_off = in_offsets[order[i].idx];
				items[nitems].out_off = out_offsets[order[i].idx];
				nitems++;
			}
			if (2 * (size_t)L > rb->work_floats)
				rb->work_floats = 2 * (size_t)L;
		}
		i = j;
	}
	/* work buffer: as many big items at a time as fit the cap (at least one) */
	if (rb->nbig) {
		size_t per = rb->work_floats; /* floats per item slot (largest size) */
		size_t slots = FSR_WORK_CAP / (per * sizeof(float));
		uint32_t maxc = 0;
		for (i = 0; i < rb->nbig; i++)
			if (rb->big[i].count > maxc)
				maxc = rb->big[i].count;
		if (slots < 1)
			slots = 1;
		if (slots > maxc)
			slots = maxc;
		rb->work_floats = per * slots;
		if ((e = cudaMalloc((void **)&rb->work, rb->work_floats * sizeof(float))) != cudaSuccess)
			goto cuda_fail;
	}
	rb->nchunks = nchunks;
	if ((e = cudaMalloc((void **)&rb->plans_dev, sizeof(fgk_plan) * (nplans ? nplans : 1))) != cudaSuccess ||
	    (e = cudaMalloc((void **)&rb->chunks_dev, sizeof(fgk_rg_chunk) * (nchunks ? nchunks : 1))) != cudaSuccess ||
	    (e = cudaMalloc((void **)&rb->items_dev, sizeof(fgk_rg_item) * n)) != cudaSuccess ||
	    (e = cudaMalloc((void **)&rb->counter_dev, sizeof(int))) != cudaSuccess)
		goto cuda_fail;
	if ((nplans && (e = cudaMemcpy(rb->plans_dev, plans, sizeof(fgk_plan) * nplans, cudaMemcpyHostToDevice)) !=
	                   cudaSuccess) ||
	    (nchunks && (e = cudaMemcpy(rb->chunks_dev, chunks, sizeof(fgk_rg_chunk) * nchunks,
	                                cudaMemcpyHostToDevice)) != cudaSuccess) ||
	    (e = cudaMemcpy(rb->items_dev, items, sizeof(fgk_rg_item) * n, cudaMemcpyHostToDevice)) != cudaSuccess)
		goto cuda_fail;
	if ((e = cudaStreamCreateWithFlags(&rb->cap_stream, cudaStreamNonBlocking)) != cudaSuccess)
		goto cuda_fail;
	free(order);
	free(plans);
	free(chunks);
	free(items);
	return rb;
cuda_fail:
	cudaGetLastError();
	rc = e == cudaErrorMemoryAllocation ? FFTSET_E_NOMEM : FFTSET_E_CUDA;
fail:
	fs_latch(fs, rc, 0);
	free(order);
	free(plans);
	free(chunks);
	free(items);
	fftset_ragged_destroy(rb);
	return NULL;
}

/* the launch sequence, on `s` */
static int fsr_record(struct fftset_ragged *rb, float *out, const float *in, cudaStream_t s)
{
	struct fs_impl *fs = rb->fs;
	uint32_t b;
	int rc = fgk_launch_ragged(rb->plans_dev, rb->chunks_dev, rb->nchunks, rb->items_dev, rb->counter_dev, rb->op, in,
	                           out, fs->num_sms, s);
	if (rc)
		return rc;
	for (b = 0; b < rb->nbig; b++) {
		const struct fftset_fft *f = rb->big[b].f;
		const size_t per = 2 * (size_t)f->lfft;
		const uint32_t slots = (uint32_t)(rb->work_floats / per);
		uint32_t done;
		for (done = 0; done < rb->big[b].count; done += slots) {
			uint32_t m = rb->big[b].count - done < slots ? rb->big[b].count - done : slots;
			rc = fgk_launch_fourstep_items(&f->p4, rb->op, out, in, rb->items_dev + rb->big[b].first + done, rb->work,
			                               m, per, s);
			if (rc)
				return rc;
		}
	}
	return 0;
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
	unsigned i, m = 0;
	if (!rb)
		return 0;
	m = rb->n;
	for (i = 0; i < rb->nbig; i++)
		m -= rb->big[i].count;
	return m;
}

/* Host layer of the fftset C API on GB300: plan registry, device tables,
 * buffer classification and the thin C ABI into the CUDA kernels (fgk.h).
 *
 * Mirrors src/fftset.c of the reference:
 *   fftset_init / fftset_destroy      src/fftset.c:80-95
 *   fftset_create_fft                 src/fftset.c:97-129 (find-or-create in a
 *                                     list sorted by descending size, keyed by
 *                                     (size, modulation))
 *   execution calls                   src/fftset.c:36-78 (one dispatch each)
 *   fftset_recommend_conv_length      src/fftset.c:131-167
 * Twiddles, modulation factors and kernel-layout tables are generated here
 * in FP64, rounded once to FP32 and uploaded once per plan. */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include "fftset.h"
#include "fftset_internal.h"
#include "fftset_layout.h"
#include "fgk.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static const struct fftset_modulation FS_MOD_FREQOFF = {1, "FREQ_OFFSET_REAL"};
static const struct fftset_modulation FS_MOD_COMPLEX = {0, "COMPLEX"};
const struct fftset_modulation *FFTSET_MODULATION_FREQ_OFFSET_REAL = &FS_MOD_FREQOFF;
const struct fftset_modulation *FFTSET_MODULATION_COMPLEX = &FS_MOD_COMPLEX;

static struct fs_impl *fs_of(const struct fftset *fc)
{
	return fc ? (struct fs_impl *)fc->impl : NULL;
}

struct fs_impl *fs_impl_of(struct fftset *fc)
{
	return fs_of(fc);
}

/* The first error is kept until fftset_clear_error; calls on several
 * threads may latch at once, so the slot is claimed with a compare-and-swap. */
int fs_latch(struct fs_impl *fs, int code, int cuda_err)
{
	int zero = 0;
	if (fs && code &&
	    __atomic_compare_exchange_n(&fs->err, &zero, code, 0, __ATOMIC_ACQ_REL, __ATOMIC_ACQUIRE))
		__atomic_store_n(&fs->cuda_err, cuda_err, __ATOMIC_RELEASE);
	return code;
}

int fs_cuda(struct fs_impl *fs, cudaError_t e)
{
	if (e == cudaSuccess)
		return FFTSET_OK;
	return fs_latch(fs, e == cudaErrorMemoryAllocation ? FFTSET_E_NOMEM : FFTSET_E_CUDA, (int)e);
}

/* ------------------------------------------------------------------------ */

int fftset_init(struct fftset *fc)
{
	struct fs_impl *fs;
	int dev = 0, smem = 0, sms = 0;
	if (fc == NULL)
		return -1;
	memset(fc, 0, sizeof(*fc));
	if (cudaGetDevice(&dev) != cudaSuccess) {
		cudaGetLastError();
		return -1;
	}
	if (cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
	    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
		cudaGetLastError();
		return -1;
	}
	fs = (struct fs_impl *)calloc(1, sizeof(*fs));
	if (fs == NULL)
		return -1;
	if (cudaStreamCreateWithFlags(&fs->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
		cudaGetLastError();
		free(fs);
		return -1;
	}
	{
		pthread_mutexattr_t ma;
		int bad = pthread_mutexattr_init(&ma) != 0;
		bad = bad || pthread_mutexattr_settype(&ma, PTHREAD_MUTEX_RECURSIVE) != 0 ||
		      pthread_mutex_init(&fs->lock, &ma) != 0;
		pthread_mutexattr_destroy(&ma);
		if (bad) {
			cudaStreamDestroy(fs->own_stream);
			free(fs);
			return -1;
		}
	}
	if (cudaHostAlloc((void **)&fs->host_flag, sizeof(int), cudaHostAllocMapped) != cudaSuccess ||
	    cudaHostGetDevicePointer((void **)&fs->dev_flag, fs->host_flag, 0) != cudaSuccess) {
		cudaGetLastError();
		if (fs->host_flag)
			cudaFreeHost(fs->host_flag);
		pthread_mutex_destroy(&fs->lock);
		cudaStreamDestroy(fs->own_stream);
		free(fs);
		return -1;
	}
	*fs->host_flag = 0;
	{
		int p, ok = cudaEventCreateWithFlags(&fs->pipe_ev, cudaEventDisableTiming) == cudaSuccess;
		for (p = 0; p < FS_PIPE && ok; p++)
			ok = cudaStreamCreateWithFlags(&fs->pipe[p], cudaStreamNonBlocking) == cudaSuccess;
		if (!ok) {
			cudaGetLastError();
			for (p = 0; p < FS_PIPE; p++)
				if (fs->pipe[p])
					cudaStreamDestroy(fs->pipe[p]);
			if (fs->pipe_ev)
				cudaEventDestroy(fs->pipe_ev);
			cudaFreeHost(fs->host_flag);
			pthread_mutex_destroy(&fs->lock);
			cudaStreamDestroy(fs->own_stream);
			free(fs);
			return -1;
		}
	}
	fs->stream = fs->own_stream;
	fs->spin_limit = 1u << 22; /* about a second */
	fs->task_shape = -1;
	fs->srv.idle_polls = FS_SERVE_IDLE_POLLS;
	fs->srv.last_v = -1;
	fs->blocking = 1;
	fs->layout_vw = 4;
	fs->device = dev;
	fs->max_smem = (unsigned)smem;
	fs->num_sms = sms;
	fc->impl = fs;
	return 0;
}

void fftset_destroy(struct fftset *fc)
{
	struct fs_impl *fs = fs_of(fc);
	struct fftset_fft *p, *n;
	int i;
	if (fs == NULL)
		return;
	cudaStreamSynchronize(fs->stream);
	fs_serve_stop(fs);
	if (fs->srv.stream)
		cudaStreamDestroy(fs->srv.stream);
	if (fs->srv.map)
		cudaFreeHost(fs->srv.map);
	for (p = fs->first; p != NULL; p = n) {
		n = p->next;
		for (i = 0; i < FS_TASK_LISTS; i++)
			fsr_free(p->tl[i].rb);
		cudaFree(p->rg_dmem);
		cudaFree(p->dmem);
		cudaFree(p->dmem4);
		cudaFree(p->dmem3);
		free(p);
	}
	for (i = 0; i < FS_PIPE; i++) {
		cudaStreamSynchronize(fs->pipe[i]);
		cudaStreamDestroy(fs->pipe[i]);
	}
	cudaEventDestroy(fs->pipe_ev);
	for (i = 0; i < FS_NSTAGE; i++)
		cudaFree(fs->stage[i]);
	cudaStreamDestroy(fs->own_stream);
	cudaFreeHost(fs->host_flag);
	pthread_mutex_destroy(&fs->lock);
	free(fs);
	fc->impl = NULL;
}

/* ------------------------------------------------------------------------ */

static int fs_valid_size(unsigned L)
{
	unsigned n = L;
	if (L < 2)
		return 0;
	while (n % 2 == 0)
		n /= 2;
	while (n % 3 == 0)
		n /= 3;
	if (n % 5 == 0)
		n /= 5;
	return n == 1;
}

static size_t fs_align(size_t x)
{
	return (x + 255) & ~(size_t)255;
}

/* Four-step tables (two HBM passes) into their own device allocation:
 * the plan of sizes beyond the shared-memory limit, and on demand for
 * resident sizes that a ragged batch runs through the four-step passes. */
int fs_ensure_fourstep(struct fs_impl *fs, struct fftset_fft *f)
{
	fgk_plan4 *p = &f->p4;
	const unsigned L = f->lfft;
	const uint32_t modulation = f->modulator->freq_offset_real ? FGK_MOD_FREQOFF : FGK_MOD_COMPLEX;
	size_t n1, n2, nhi, nlo, off[11], total, i;
	float *h = NULL;
	char *d = NULL;
	int32_t *kidx = NULL;
	unsigned lanes = 0;
	cudaError_t e;
	int rc = FFTSET_E_NOMEM;

	if (f->dmem4)
		return FFTSET_OK;
	if (fgk_plan_fourstep(p, L, modulation, fs->max_smem))
		return FFTSET_E_UNSUPPORTED;
	n1 = fgk_chain_twiddles(&p->c1, NULL);
	n2 = fgk_chain_twiddles(&p->c2, NULL);
	/* w_L^m = thi[m >> tshift] tlo[m & (2^tshift - 1)], both tables about
	 * sqrt(L) entries so that they stay in L1 */
	p->tshift = 1;
	while (((uint64_t)1 << (2 * p->tshift)) < L)
		p->tshift++;
	nlo = (size_t)1 << p->tshift;
	nhi = (L + nlo - 1) / nlo;
	/* w_{R L2}^m for the task kernel's inter-step twiddle, R the last radix of
	 * the column chain */
	p->nq = p->c1.st[p->c1.nstages - 1].radix * p->L2;
	/* float2 counts: tw1, tw2, thi, tlo, m1, m2, n1, n2, tq; then kidx (int32) and the plan copy */
	{
		const size_t cnt[9] = {n1 ? n1 : 1, n2 ? n2 : 1, nhi, nlo, p->L1, p->L2, p->L1, p->L2, p->nq};
		total = fs_align(sizeof(fgk_plan4));
		for (i = 0; i < 9; i++) {
			off[i] = total;
			total += fs_align(cnt[i] * 2 * sizeof(float));
		}
		off[9] = total;
		total += fs_align(sizeof(int32_t) * L);
	}
	h = (float *)malloc(sizeof(float) * 2 *
	                    (n1 + n2 + nhi + nlo + 2 * (size_t)p->L1 + 2 * (size_t)p->L2 + (size_t)p->nq + 2));
	kidx = (int32_t *)malloc(sizeof(int32_t) * L);
	if (!h || !kidx)
		goto out;
	if (fsl_kernel_offsets(f->modulator->freq_offset_real, L, fs->layout_vw, kidx, &lanes)) {
		rc = FFTSET_E_INVALID;
		goto out;
	}
	f->lanes = lanes;
	if ((e = cudaMalloc((void **)&d, total)) != cudaSuccess) {
		cudaGetLastError();
		goto out;
	}
	{
		float *w = h;
		float *tw1 = w, *tw2, *thi, *tlo, *m1, *m2, *q1, *q2, *tq;
		size_t k;
		fgk_chain_twiddles(&p->c1, tw1);
		tw2 = tw1 + 2 * (n1 ? n1 : 1);
		fgk_chain_twiddles(&p->c2, tw2);
		thi = tw2 + 2 * (n2 ? n2 : 1);
		tlo = thi + 2 * nhi;
		m1 = tlo + 2 * nlo;
		m2 = m1 + 2 * (size_t)p->L1;
		q1 = m2 + 2 * (size_t)p->L2;
		q2 = q1 + 2 * (size_t)p->L1;
		tq = q2 + 2 * (size_t)p->L2;
		for (k = 0; k < p->nq; k++) {
			double a = -2.0 * M_PI * (double)k / (double)p->nq;
			tq[2 * k] = (float)cos(a);
			tq[2 * k + 1] = (float)sin(a);
		}
		for (k = 0; k < nhi; k++) {
			double a = -2.0 * M_PI * (double)(k * nlo) / (double)L;
			thi[2 * k] = (float)cos(a);
			thi[2 * k + 1] = (float)sin(a);
		}
		for (k = 0; k < nlo; k++) {
			double a = -2.0 * M_PI * (double)k / (double)L;
			tlo[2 * k] = (float)cos(a);
			tlo[2 * k + 1] = (float)sin(a);
		}
		for (k = 0; k < p->L1; k++) {
			double a = -M_PI * (double)k / (2.0 * p->L1), b = -M_PI * (double)k / (2.0 * (double)L);
			m1[2 * k] = (float)cos(a);
			m1[2 * k + 1] = (float)sin(a);
			q1[2 * k] = (float)cos(b);
			q1[2 * k + 1] = (float)sin(b);
		}
		for (k = 0; k < p->L2; k++) {
			double a = -M_PI * (double)k / (2.0 * (double)L), b = -M_PI * (double)k / (2.0 * p->L2);
			m2[2 * k] = (float)cos(a);
			m2[2 * k + 1] = (float)sin(a);
			q2[2 * k] = (float)cos(b);
			q2[2 * k + 1] = (float)sin(b);
		}
		{
			float *srcs[9] = {tw1, tw2, thi, tlo, m1, m2, q1, q2, tq};
			const size_t cnt[9] = {n1, n2, nhi, nlo, p->L1, p->L2, p->L1, p->L2, p->nq};
			const void **dst[9] = {&p->tw1, &p->tw2, &p->thi, &p->tlo, &p->m1, &p->m2, &p->n1, &p->n2, &p->tq};
			for (k = 0; k < 9; k++) {
				*dst[k] = d + off[k];
				if (cnt[k] &&
				    (e = cudaMemcpy(d + off[k], srcs[k], cnt[k] * 2 * sizeof(float), cudaMemcpyHostToDevice)) !=
				        cudaSuccess)
					goto cuda_fail;
			}
		}
	}
	p->dev = (const fgk_plan4 *)d;
	if ((e = cudaMemcpy(d + off[9], kidx, sizeof(int32_t) * L, cudaMemcpyHostToDevice)) != cudaSuccess ||
	    (e = cudaMemcpy(d, p, sizeof(fgk_plan4), cudaMemcpyHostToDevice)) != cudaSuccess)
		goto cuda_fail;
	f->kidx4 = (const int32_t *)(d + off[9]);
	f->dmem4 = d;
	rc = FFTSET_OK;
	goto out;
cuda_fail:
	fs_cuda(fs, e);
	cudaFree(d);
	rc = FFTSET_E_CUDA;
out:
	free(h);
	free(kidx);
	return rc;
}

/* Three-level tables (fgk_plan3) in their own device allocation. */
int fs_ensure_threestep(struct fs_impl *fs, struct fftset_fft *f)
{
	fgk_plan3 *p = &f->p3;
	const unsigned L = f->lfft;
	const uint32_t modulation = f->modulator->freq_offset_real ? FGK_MOD_FREQOFF : FGK_MOD_COMPLEX;
	enum { NT = 8 };
	size_t cnt[NT], off[NT + 1], total, i, k, all = 0;
	float *h = NULL, *w[NT];
	char *d = NULL;
	cudaError_t e;
	int rc = FFTSET_E_NOMEM;
	uint32_t L12;

	(void)fs;
	if (f->dmem3)
		return FFTSET_OK;
	if (fgk_plan_threestep(p, L, modulation))
		return FFTSET_E_UNSUPPORTED;
	L12 = p->L1 * p->L2;
	/* tq1 tq2 ma mb mc oa ob oc */
	cnt[0] = p->nq1;
	cnt[1] = p->nq2;
	cnt[2] = cnt[5] = p->L1;
	cnt[3] = cnt[6] = p->L2;
	cnt[4] = cnt[7] = p->L3;
	total = fs_align(sizeof(fgk_plan3));
	for (i = 0; i < NT; i++) {
		off[i] = total;
		total += fs_align((cnt[i] ? cnt[i] : 1) * 2 * sizeof(float));
		all += cnt[i] ? cnt[i] : 1;
	}
	h = (float *)malloc(sizeof(float) * 2 * all);
	if (!h)
		goto out;
	w[0] = h;
	for (i = 1; i < NT; i++)
		w[i] = w[i - 1] + 2 * (cnt[i - 1] ? cnt[i - 1] : 1);
	{
		/* table i, entry k: e^{-j 2 pi num(k) / den} (FP64, rounded once) */
		const double twopi = 2.0 * M_PI;
		for (k = 0; k < cnt[0]; k++) {
			double a = -twopi * (double)k / (double)p->nq1;
			w[0][2 * k] = (float)cos(a), w[0][2 * k + 1] = (float)sin(a);
		}
		for (k = 0; k < cnt[1]; k++) {
			double a = -twopi * (double)k / (double)p->nq2;
			w[1][2 * k] = (float)cos(a), w[1][2 * k + 1] = (float)sin(a);
		}
		/* modulation: in e^{-j pi n1/(2 L1)}, e^{-j pi n2/(2 L1 L2)}, e^{-j pi n3/(2L)};
		 * out e^{-j pi k1/(2L)}, e^{-j pi k2/(2 L2 L3)}, e^{-j pi k3/(2 L3)} */
		{
			const double den[6] = {2.0 * p->L1, 2.0 * L12, 2.0 * L, 2.0 * L, 2.0 * p->L2 * p->L3, 2.0 * p->L3};
			for (i = 0; i < 6; i++)
				for (k = 0; k < cnt[2 + i]; k++) {
					double a = -M_PI * (double)k / den[i];
					w[2 + i][2 * k] = (float)cos(a), w[2 + i][2 * k + 1] = (float)sin(a);
				}
		}
	}
	if ((e = cudaMalloc((void **)&d, total)) != cudaSuccess) {
		cudaGetLastError();
		goto out;
	}
	{
		const void **dst[NT] = {&p->tq1, &p->tq2, &p->ma, &p->mb, &p->mc, &p->oa, &p->ob, &p->oc};
		for (i = 0; i < NT; i++) {
			*dst[i] = d + off[i];
			if (cnt[i] &&
			    (e = cudaMemcpy(d + off[i], w[i], cnt[i] * 2 * sizeof(float), cudaMemcpyHostToDevice)) != cudaSuccess)
				goto cuda_fail;
		}
	}
	p->dev = (const fgk_plan3 *)d;
	if ((e = cudaMemcpy(d, p, sizeof(fgk_plan3), cudaMemcpyHostToDevice)) != cudaSuccess)
		goto cuda_fail;
	f->dmem3 = d;
	rc = FFTSET_OK;
	goto out;
cuda_fail:
	fs_cuda(fs, e);
	cudaFree(d);
	rc = FFTSET_E_CUDA;
out:
	free(h);
	return rc;
}

/* Build the device tables of a plan: the generic resident plan (chain from
 * the GPU planner) plus one twiddle table per compile-time variant (each
 * variant has its own chain); modulation factors and the kernel-layout index
 * table are shared. Everything lives in one device allocation. */
static int fs_build_resident(struct fs_impl *fs, struct fftset_fft *f)
{
	fgk_plan *rp = &f->rp;
	size_t ntw, vtw[FS_MAX_VAR], o_plan, o_tw, o_mod, o_kidx, o_v[FS_MAX_VAR], total;
	float *tw = NULL, *mod = NULL;
	int32_t *kidx = NULL;
	char *d = NULL;
	unsigned L = f->lfft, i, lanes = 0;
	uint32_t modulation = f->modulator->freq_offset_real ? FGK_MOD_FREQOFF : FGK_MOD_COMPLEX;
	int rc = FFTSET_E_NOMEM, v, op, nvar;
	cudaError_t e;

	if (fgk_plan_resident(rp, L, modulation, fs->max_smem, NULL, 0)) {
		f->fourstep = 1;
		f->nvar = 0;
		for (v = 0; v < FGK_OP_COUNT; v++)
			f->sel[v] = -1;
		return fs_ensure_fourstep(fs, f);
	}
	ntw = fgk_plan_twiddles(rp, NULL);
	nvar = fgk_static_count(modulation, L);
	if (nvar > FS_MAX_VAR)
		nvar = FS_MAX_VAR;
	f->nvar = 0;
	for (v = 0; v < nvar; v++) {
		uint32_t rad[FGK_MAX_STAGES], n, threads, groups, ops, tma;
		if (!fgk_static_info(modulation, L, v, rad, &n, &threads, &groups, &ops, &tma) ||
		    fgk_plan_resident(&f->vp[v], L, modulation, fs->max_smem, rad, n))
			return FFTSET_E_UNSUPPORTED;
		f->vops[v] = ops;
		f->vtma[v] = tma;
		vtw[v] = fgk_plan_twiddles(&f->vp[v], NULL);
	}
	f->nvar = nvar;
	for (op = 0; op < FGK_OP_COUNT; op++) {
		f->sel[op] = -1;
		for (v = 0; v < nvar; v++)
			if (f->vops[v] & (1u << op)) {
				f->sel[op] = v;
				break;
			}
	}

	mod = (float *)malloc(sizeof(float) * 2 * L);
	kidx = (int32_t *)malloc(sizeof(int32_t) * L);
	if (!mod || !kidx)
		goto out;
	for (i = 0; i < L; i++) {
		double a = -M_PI * (double)i / (2.0 * (double)L);
		mod[2 * i + 0] = (float)cos(a);
		mod[2 * i + 1] = (float)sin(a);
	}
	if (fsl_kernel_offsets(f->modulator->freq_offset_real, L, fs->layout_vw, kidx, &lanes)) {
		rc = FFTSET_E_INVALID;
		goto out;
	}
	f->lanes = lanes;
	rp->kvw = lanes;

	o_plan = 0;
	o_tw = fs_align(sizeof(fgk_plan));
	o_mod = o_tw + fs_align(sizeof(float) * 2 * (ntw ? ntw : 1));
	o_kidx = o_mod + fs_align(sizeof(float) * 2 * L);
	total = o_kidx + fs_align(sizeof(int32_t) * L);
	for (v = 0; v < nvar; v++) {
		o_v[v] = total;
		total += fs_align(sizeof(float) * 2 * (vtw[v] ? vtw[v] : 1));
	}
	e = cudaMalloc((void **)&d, total);
	if (e != cudaSuccess) {
		cudaGetLastError();
		goto out;
	}
	rp->tw = d + o_tw;
	rp->modtw = d + o_mod;
	rp->kidx = (const int32_t *)(d + o_kidx);
	rp->dev = (const fgk_plan *)(d + o_plan);
	if ((e = cudaMemcpy(d + o_mod, mod, sizeof(float) * 2 * L, cudaMemcpyHostToDevice)) != cudaSuccess ||
	    (e = cudaMemcpy(d + o_kidx, kidx, sizeof(int32_t) * L, cudaMemcpyHostToDevice)) != cudaSuccess ||
	    (e = cudaMemcpy(d + o_plan, rp, sizeof(fgk_plan), cudaMemcpyHostToDevice)) != cudaSuccess)
		goto cuda_fail;
	/* twiddle tables, one host buffer at a time */
	for (v = -1; v < nvar; v++) {
		fgk_plan *pp = v < 0 ? rp : &f->vp[v];
		size_t nt = v < 0 ? ntw : vtw[v];
		tw = (float *)malloc(sizeof(float) * 2 * (nt ? nt : 1));
		if (!tw) {
			cudaFree(d);
			goto out;
		}
		fgk_plan_twiddles(pp, tw);
		if (v >= 0) {
			pp->tw = d + o_v[v];
			pp->modtw = rp->modtw;
			pp->kidx = rp->kidx;
			pp->kvw = lanes;
			pp->dev = NULL;
		}
		e = cudaMemcpy((void *)pp->tw, tw, sizeof(float) * 2 * nt, cudaMemcpyHostToDevice);
		free(tw);
		tw = NULL;
		if (e != cudaSuccess)
			goto cuda_fail;
	}
	f->dmem = d;
	rc = FFTSET_OK;
	goto out;
cuda_fail:
	fs_cuda(fs, e);
	cudaFree(d);
	rc = FFTSET_E_CUDA;
out:
	free(tw);
	free(mod);
	free(kidx);
	return rc;
}

const struct fftset_fft *fftset_create_fft(struct fftset *fc, const struct fftset_modulation *modulation,
                                           unsigned complex_bins)
{
	struct fs_impl *fs = fs_of(fc);
	if (fs == NULL)
		return NULL;
	return fs_create_plan(fs, modulation, complex_bins);
}

/* why the calling thread's last fs_create_plan returned NULL */
static __thread int fs_plan_why;

int fs_plan_error(void)
{
	return fs_plan_why;
}

struct fftset_fft *fs_create_plan(struct fs_impl *fs, const struct fftset_modulation *modulation, unsigned complex_bins)
{
	struct fftset_fft *p, **ipos;
	int rc;
	fs_plan_why = FFTSET_E_INVALID;
	if (modulation != FFTSET_MODULATION_COMPLEX && modulation != FFTSET_MODULATION_FREQ_OFFSET_REAL) {
		fs_latch(fs, FFTSET_E_INVALID, 0);
		return NULL;
	}
	if (!fs_valid_size(complex_bins)) {
		fs_latch(fs, FFTSET_E_INVALID, 0);
		return NULL;
	}
	for (p = fs->first; p != NULL; p = p->next) {
		if (p->lfft == complex_bins && p->modulator == modulation)
			return p;
		if (p->lfft < complex_bins)
			break;
	}
	p = (struct fftset_fft *)calloc(1, sizeof(*p));
	if (p == NULL) {
		fs_plan_why = FFTSET_E_NOMEM;
		fs_latch(fs, FFTSET_E_NOMEM, 0);
		return NULL;
	}
	p->lfft = complex_bins;
	p->modulator = modulation;
	p->fs = fs;
	rc = fs_build_resident(fs, p);
	if (rc) {
		fs_plan_why = rc;
		fs_latch(fs, rc, 0);
		free(p);
		return NULL;
	}
	ipos = &fs->first;
	while (*ipos != NULL && complex_bins < (*ipos)->lfft)
		ipos = &(*ipos)->next;
	p->next = *ipos;
	*ipos = p;
	return p;
}

/* ------------------------------------------------------------------------
 * Execution */

int fs_is_device_ptr(const void *ptr)
{
	struct cudaPointerAttributes a;
	if (ptr == NULL)
		return 1;
	if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
		cudaGetLastError();
		return 0;
	}
	return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

/* What a call's buffer is, from one pointer-attribute query: device or
 * managed memory (used in place), pinned host memory (kernels reach it over
 * the host link at `kaddr`), or pageable host memory (staged). */
struct fs_ptrinfo {
	int         dev;    /* device or managed (NULL counts as device) */
	int         pinned; /* page-locked host memory with a device address */
	const void *kaddr;  /* the address kernels use */
};

static struct fs_ptrinfo fs_classify(const void *ptr)
{
	struct fs_ptrinfo pi = {1, 0, ptr};
	struct cudaPointerAttributes a;
	if (ptr == NULL)
		return pi;
	pi.dev = 0;
	if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
		cudaGetLastError();
		return pi;
	}
	if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged)
		pi.dev = 1;
	else if (a.type == cudaMemoryTypeHost && a.devicePointer != NULL) {
		pi.pinned = 1;
		pi.kaddr = a.devicePointer;
	}
	return pi;
}

int fs_stage_reserve(struct fs_impl *fs, int slot, size_t bytes)
{
	cudaError_t e;
	if (fs->stage_bytes[slot] >= bytes)
		return FFTSET_OK;
	if (fs->stage[slot]) {
		cudaStreamSynchronize(fs->stream);
		cudaFree(fs->stage[slot]);
		fs->stage[slot] = NULL;
		fs->stage_bytes[slot] = 0;
	}
	e = cudaMalloc(&fs->stage[slot], bytes);
	if (e != cudaSuccess) {
		cudaGetLastError();
		fs->stage[slot] = NULL;
		return fs_latch(fs, FFTSET_E_NOMEM, (int)e);
	}
	fs->stage_bytes[slot] = bytes;
	return FFTSET_OK;
}

/* A kernel whose bounded wait gave up wrote 1 to the mapped flag; the
 * thread that takes it latches the timeout. */
int fs_check_flag(struct fs_impl *fs)
{
	if (__atomic_load_n(fs->host_flag, __ATOMIC_ACQUIRE) && __atomic_exchange_n(fs->host_flag, 0, __ATOMIC_ACQ_REL))
		return fs_latch(fs, FFTSET_E_TIMEOUT, 0);
	return FFTSET_OK;
}

/* Kernel choice: the compile-time kernel chosen for the op when one exists,
 * the generic resident kernel otherwise, whatever the batch count. Single
 * transforms gain from it too (one CTA stages the tables at once, where the
 * generic kernel waits on each stage's twiddle reads: 6.1 against 8.2 us of
 * GPU time for one 1024-bin transform), and a block gives the same bits in
 * a batch of any size as in a single call. */
static int fs_pick_variant(const struct fftset_fft *f, int op, unsigned count)
{
	(void)count;
	return f->sel[op];
}

/* no_bulk: the buffers live in host memory, which the library does not read
 * with bulk copies (TMA): variants with bulk-copy input are skipped */
static int fs_launch_variant_ex(const struct fftset_fft *f, int v, int op, float *out, const float *in,
                                const float *kern, unsigned count, size_t in_stride, size_t out_stride,
                                cudaStream_t stream, int no_bulk)
{
	struct fs_impl *fs = f->fs;
	if (v >= 0 && v < f->nvar) {
		int rc = -1;
		if (!(no_bulk && f->vtma[v]))
			rc = fgk_launch_static(&f->vp[v], v, op, out, in, kern, count, in_stride, out_stride, stream,
			                       fs->num_sms, fs->dev_flag);
		if (rc >= 0)
			return rc;
		/* the variant cannot take these buffers (alignment, host memory):
		 * any other compiled variant that can, else the generic kernel */
		for (v = 0; v < f->nvar; v++) {
			if (no_bulk && f->vtma[v])
				continue;
			rc = fgk_launch_static(&f->vp[v], v, op, out, in, kern, count, in_stride, out_stride, stream,
			                       fs->num_sms, fs->dev_flag);
			if (rc >= 0)
				return rc;
		}
	}
	return fgk_launch_resident(&f->rp, op, out, in, kern, count, in_stride, out_stride, stream);
}

static int fs_launch_variant(const struct fftset_fft *f, int v, int op, float *out, const float *in,
                             const float *kern, unsigned count, size_t in_stride, size_t out_stride,
                             cudaStream_t stream)
{
	return fs_launch_variant_ex(f, v, op, out, in, kern, count, in_stride, out_stride, stream, 0);
}

/* Plans beyond the shared-memory limit share state between calls (their
 * cached task lists, the work buffer of staging slot 3, tables built on
 * demand): calls on them hold the fftset's lock from lookup to launch, so
 * that concurrent calls on several threads never launch on a list or a
 * buffer another thread is replacing. */
static int fs_launch_fourstep(const struct fftset_fft *f, int op, float *out, const float *in, const float *kern,
                              unsigned count, size_t in_stride, size_t out_stride)
{
	struct fs_impl *fs = f->fs;
	const size_t nf = 2 * (size_t)f->lfft;
	int rc = -FFTSET_E_UNSUPPORTED;
	pthread_mutex_lock(&fs->lock);
	if (op == FGK_OP_FORWARD || op == FGK_OP_INVERSE) {
		/* tile tasks (fgk_tasks.cuh): two- or three-level split */
		rc = fs_tasks_batch((struct fftset_fft *)f, op, out, out_stride, in, in_stride, count, fs->stream, NULL);
	} else if (op == FGK_OP_CONV || op == FGK_OP_CORR) {
		/* the forward task launch with the spectrum product fused into its
		 * final stores, into the work buffer (natural bins, the forward's
		 * output layout), then the inverse task launch from it: the
		 * convolution theorem in the library's own transforms, inverse(
		 * forward(x) K) = complex_bins x the (negacyclic or cyclic)
		 * convolution, two launches through HBM */
		const size_t is = count > 1 ? in_stride : nf, os = count > 1 ? out_stride : nf;
		if ((rc = fs_stage_reserve(fs, 3, nf * ((size_t)count + 1) * sizeof(float))) != 0) {
			rc = -rc;
		} else {
			/* the work buffer, then the kernel spectrum in natural order */
			float *work = (float *)fs->stage[3], *spec = work + nf * (size_t)count;
			const fgk_product prod = {spec};
			rc = fgk_launch_spectrum_natural(kern, f->kidx4, (int)f->lanes, f->lfft, op == FGK_OP_CORR, spec,
			                                 fs->stream);
			if (rc == 0)
				rc = fs_tasks_batch((struct fftset_fft *)f, FGK_OP_FORWARD, work, nf, in, is, count, fs->stream,
				                    &prod);
			if (rc == 0)
				rc = fs_tasks_batch((struct fftset_fft *)f, FGK_OP_INVERSE, out, os, work, nf, count, fs->stream,
				                    NULL);
		}
	}
	if (rc == -FFTSET_E_UNSUPPORTED) {
		/* two passes through a work buffer of 2L floats per transform (the
		 * library's own scratch: work_buf of the reference API may be host
		 * memory or too small for batches) */
		if ((rc = fs_stage_reserve(fs, 3, nf * count * sizeof(float))) != 0)
			rc = -rc;
		else
			rc = fgk_launch_fourstep(&f->p4, op, out, in, kern, f->kidx4, (int)f->lanes, (float *)fs->stage[3],
			                         count, in_stride ? in_stride : nf, out_stride ? out_stride : nf, nf, fs->stream);
	}
	pthread_mutex_unlock(&fs->lock);
	return rc;
}

int fs_launch(const struct fftset_fft *f, int op, float *out, const float *in, const float *kern,
                     unsigned count, size_t in_stride, size_t out_stride)
{
	if (f->fourstep)
		return fs_launch_fourstep(f, op, out, in, kern, count, in_stride, out_stride);
	return fs_launch_variant(f, fs_pick_variant(f, op, count), op, out, in, kern, count, in_stride, out_stride,
	                         f->fs->stream);
}

/* m rows of nf floats, `stride` floats apart on both sides: only the rows
 * move (the caller's memory between rows is left alone) */
static cudaError_t fs_copy_rows(float *dst, const float *src, size_t stride, size_t nf, size_t m,
                                enum cudaMemcpyKind kind, cudaStream_t st)
{
	if (m == 1 || stride == nf)
		return cudaMemcpyAsync(dst, src, ((m - 1) * stride + nf) * sizeof(float), kind, st);
	return cudaMemcpy2DAsync(dst, stride * sizeof(float), src, stride * sizeof(float), nf * sizeof(float), m, kind,
	                         st);
}

/* Host buffers, many blocks: chunks of about FS_CHUNK_BYTES go round-robin
 * over FS_PIPE streams, each chunk copied in, transformed and copied out on
 * its stream, so that the copies in both directions and the kernels of
 * different chunks overlap. Resident sizes only (the four-step passes share
 * one work buffer). Called with fs->lock held; returns after the results are
 * in `out`. */
#define FS_CHUNK_BYTES ((size_t)16 << 20)

static int fs_exec_pipelined(const struct fftset_fft *f, int op, float *out, size_t out_stride, const float *in,
                             size_t in_stride, const float *dkern, unsigned count, int in_dev, int out_dev)
{
	struct fs_impl *fs = f->fs;
	const size_t nf = 2 * (size_t)f->lfft;
	const size_t cb = FS_CHUNK_BYTES / (nf * sizeof(float)) ? FS_CHUNK_BYTES / (nf * sizeof(float)) : 1;
	const size_t in_span = (cb - 1) * in_stride + nf, out_span = (cb - 1) * out_stride + nf;
	float *sin = NULL, *sout = NULL;
	size_t c, first;
	int rc = FFTSET_OK, p;
	cudaError_t e;

	if (!in_dev) {
		if ((rc = fs_stage_reserve(fs, 0, FS_PIPE * in_span * sizeof(float))) != 0)
			return rc;
		sin = (float *)fs->stage[0];
	}
	if (!out_dev) {
		if ((rc = fs_stage_reserve(fs, 1, FS_PIPE * out_span * sizeof(float))) != 0)
			return rc;
		sout = (float *)fs->stage[1];
	}
	/* after everything already on the fftset's stream (the kernel-buffer copy) */
	if ((e = cudaEventRecord(fs->pipe_ev, fs->stream)) != cudaSuccess)
		return fs_cuda(fs, e);
	for (p = 0; p < FS_PIPE; p++)
		if ((e = cudaStreamWaitEvent(fs->pipe[p], fs->pipe_ev, 0)) != cudaSuccess)
			return fs_cuda(fs, e);
	for (c = 0, first = 0; first < count; c++, first += cb) {
		const unsigned m = (unsigned)(count - first < cb ? count - first : cb);
		cudaStream_t st = fs->pipe[c % FS_PIPE];
		const float *din = in + first * in_stride;
		float *dout = out + first * out_stride;
		const int v = fs_pick_variant(f, op, (unsigned)count); /* the kernel the whole batch would use */
		if (!in_dev) {
			din = sin + (c % FS_PIPE) * in_span;
			if ((e = fs_copy_rows((float *)din, in + first * in_stride, in_stride, nf, m, cudaMemcpyHostToDevice,
			                      st)) != cudaSuccess) {
				rc = fs_cuda(fs, e);
				break;
			}
		}
		if (!out_dev)
			dout = sout + (c % FS_PIPE) * out_span;
		if ((rc = fs_launch_variant(f, v, op, dout, din, dkern, m, in_stride, out_stride, st)) != 0) {
			rc = rc < 0 ? fs_latch(fs, -rc, 0) : fs_latch(fs, FFTSET_E_CUDA, rc);
			break;
		}
		if (!out_dev && (e = fs_copy_rows(out + first * out_stride, dout, out_stride, nf, m, cudaMemcpyDeviceToHost,
		                                  st)) != cudaSuccess) {
			rc = fs_cuda(fs, e);
			break;
		}
	}
	for (p = 0; p < FS_PIPE; p++) {
		const int r = fs_cuda(fs, cudaStreamSynchronize(fs->pipe[p]));
		if (rc == FFTSET_OK)
			rc = r;
	}
	if (rc == FFTSET_OK)
		rc = fs_check_flag(fs);
	return rc;
}

/* ---- the call service ----------------------------------------------------
 * Blocking single calls on device buffers of resident sizes (the op's
 * compiled variant when it has a call service, else the generic kernel's,
 * fgk.h) are answered by one resident CTA instead of a launch and a stream
 * synchronisation: the request goes into a pinned, mapped page,
 * the doorbell is a sequence number, and the call returns when the CTA has
 * published that number in `reply` (its output stores released before it).
 * A launch of the service is made only when the same (plan, variant) is
 * called twice in a row; it exits on its own after FS_SERVE_IDLE_POLLS idle
 * polls, and every host wait here is bounded, ending in a wait for the
 * service's stream and, if the request is still pending, a new launch. */
#define FS_SERVE_SPIN (1u << 26) /* host polls of `reply` before checking on the service the slow way */

static uint64_t fs_ld(const volatile uint64_t *p) { return __atomic_load_n(p, __ATOMIC_ACQUIRE); }

static int fs_serve_init(struct fs_impl *fs)
{
	struct fs_serve *s = &fs->srv;
	char *h = NULL, *d = NULL;
	if (cudaHostAlloc((void **)&h, 4096, cudaHostAllocMapped) != cudaSuccess ||
	    cudaHostGetDevicePointer((void **)&d, h, 0) != cudaSuccess ||
	    cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
		cudaGetLastError();
		if (h)
			cudaFreeHost(h);
		s->stream = NULL;
		return -1;
	}
	memset(h, 0, 4096);
	s->map = h;
	/* one 128-byte line per word */
	s->bell = (volatile uint64_t *)(h + 0);
	s->reply = (volatile uint64_t *)(h + 128);
	s->state = (volatile uint64_t *)(h + 256);
	s->req = (fgk_serve_req *)(h + 384);
	s->dev.bell = (const volatile uint64_t *)(d + 0);
	s->dev.reply = (volatile uint64_t *)(d + 128);
	s->dev.state = (volatile uint64_t *)(d + 256);
	s->dev.req = (const fgk_serve_req *)(d + 384);
	return 0;
}

/* a new launch for (f, v) that has seen every request before `seen` */
static int fs_serve_launch(struct fs_impl *fs, const struct fftset_fft *f, int v, uint64_t seen)
{
	struct fs_serve *s = &fs->srv;
	const uint64_t id = ++s->id;
	int rc;
	__atomic_store_n(s->state, id, __ATOMIC_RELEASE);
	rc = v < 0 ? fgk_launch_resident_serve(&f->rp, s->dev, seen, id, s->idle_polls, s->stream)
	           : fgk_launch_static_serve(&f->vp[v], v, s->dev, seen, id, s->idle_polls, s->stream);
	if (rc != 0) {
		cudaGetLastError();
		__atomic_store_n(s->state, 0, __ATOMIC_RELEASE);
		return -1;
	}
	s->f = f;
	s->v = v;
	return 0;
}

/* the live launch, if any, leaves: a request with op -1, then its stream */
void fs_serve_stop(struct fs_impl *fs)
{
	struct fs_serve *s = &fs->srv;
	if (!s->map || !s->stream)
		return;
	if (fs_ld(s->state) == s->id && s->id) {
		s->req->op = -1;
		__atomic_store_n(s->bell, ++s->seq, __ATOMIC_SEQ_CST);
	}
	cudaStreamSynchronize(s->stream);
	cudaGetLastError();
	s->f = NULL;
}

/* -1: not taken (the caller runs the call the usual way), else the call's
 * FFTSET status */
static int fs_serve_call(const struct fftset_fft *f, int v, int op, float *out, const float *in, const float *kern)
{
	struct fs_impl *fs = f->fs;
	struct fs_serve *s = &fs->srv;
	uint64_t seq;
	unsigned relaunch = 0;
	uint32_t polls;
	cudaError_t e;
	if (!s->idle_polls || s->broken || f->fourstep || op < 0 || op >= FGK_OP_COUNT)
		return -1;
	/* v < 0: the generic kernel, whose service takes every op */
	if (v >= 0 && !fgk_static_serve_ok(f->rp.modulation, f->lfft, v, op))
		return -1;
	pthread_mutex_lock(&fs->lock);
	if (s->last_f != f || s->last_v != v) {
		/* a launch pays off from the second call of the same kind */
		s->last_f = f;
		s->last_v = v;
		pthread_mutex_unlock(&fs->lock);
		return -1;
	}
	if (!s->map && fs_serve_init(fs) != 0) {
		s->broken = 1;
		pthread_mutex_unlock(&fs->lock);
		return -1;
	}
	/* a blocking call runs after the work already queued on the stream */
	if ((e = cudaStreamSynchronize(fs->stream)) != cudaSuccess) {
		pthread_mutex_unlock(&fs->lock);
		return fs_cuda(fs, e);
	}
	if (!(s->f == f && s->v == v && s->id && fs_ld(s->state) == s->id)) {
		fs_serve_stop(fs);
		if (fs_serve_launch(fs, f, v, s->seq) != 0) {
			s->broken = 1;
			pthread_mutex_unlock(&fs->lock);
			return -1;
		}
	}
	s->req->op = op;
	s->req->in = in;
	s->req->out = out;
	s->req->kern = kern;
	seq = ++s->seq;
	__atomic_store_n(s->bell, seq, __ATOMIC_SEQ_CST);
	__atomic_thread_fence(__ATOMIC_SEQ_CST);
	for (polls = 0;; polls++) {
		if (fs_ld(s->reply) == seq)
			break;
		if (fs_ld(s->state) != s->id || polls >= FS_SERVE_SPIN) {
			/* the launch left (or stopped answering): once its stream is
			 * done, either it answered on its way out or the request is
			 * still pending and a new launch takes it */
			if ((e = cudaStreamSynchronize(s->stream)) != cudaSuccess) {
				s->broken = 1;
				pthread_mutex_unlock(&fs->lock);
				return fs_cuda(fs, e);
			}
			if (fs_ld(s->reply) == seq)
				break;
			if (++relaunch > 2 || fs_serve_launch(fs, f, v, seq - 1) != 0) {
				/* the request is void now (no launch is alive): run it the
				 * usual way */
				s->broken = 1;
				s->f = NULL;
				pthread_mutex_unlock(&fs->lock);
				return -1;
			}
			polls = 0;
		}
	}
	s->served++;
	pthread_mutex_unlock(&fs->lock);
	return FFTSET_OK;
}

/* Runs op on `count` blocks. Buffers of any memory kind. */
static int fs_exec(const struct fftset_fft *f, int op, float *out, size_t out_stride, const float *in,
                   size_t in_stride, const float *kern, unsigned count)
{
	struct fs_impl *fs;
	int rc = FFTSET_OK, staged = 0;
	size_t nf = 2 * (size_t)(f ? f->lfft : 0);
	size_t in_span, out_span;
	const float *din = in, *dkern = kern;
	float *dout = out;
	cudaError_t e;

	if (f == NULL)
		return FFTSET_E_INVALID;
	fs = f->fs;
	if (out == NULL || in == NULL || (count > 1 && (in_stride < nf || out_stride < nf)) ||
	    ((op == FGK_OP_CONV || op == FGK_OP_CORR) && kern == NULL))
		return fs_latch(fs, FFTSET_E_INVALID, 0);
	if ((((uintptr_t)in) | ((uintptr_t)out) | ((uintptr_t)kern)) & 7)
		return fs_latch(fs, FFTSET_E_INVALID, 0);
	/* blocks must stay 8-byte aligned (complex values are read as pairs) */
	if (count > 1 && ((in_stride | out_stride) & 1))
		return fs_latch(fs, FFTSET_E_INVALID, 0);
	if (count == 0)
		return FFTSET_OK;
	in_span = (size_t)(count - 1) * in_stride + nf;
	out_span = (size_t)(count - 1) * out_stride + nf;
	/* one query per buffer, whatever path the call takes */
	const struct fs_ptrinfo pin = fs_classify(in), pout = fs_classify(out), pkern = fs_classify(kern);

	if (pin.dev && pout.dev && pkern.dev) {
		if (fs->blocking && count == 1 && !f->fourstep) {
			rc = fs_serve_call(f, fs_pick_variant(f, op, 1), op, out, in, kern);
			if (rc >= 0)
				return rc;
		}
		rc = fs_launch(f, op, out, in, kern, count, in_stride, out_stride);
		if (rc < 0)
			return fs_latch(fs, -rc, 0);
		if (rc)
			return fs_latch(fs, FFTSET_E_CUDA, rc);
		if (fs->blocking) {
			if ((rc = fs_cuda(fs, cudaStreamSynchronize(fs->stream))) != 0)
				return rc;
			return fs_check_flag(fs);
		}
		return FFTSET_OK;
	}

	/* pinned host buffers (and device ones): resident kernels read and write
	 * them in place over the host link, no staging copies */
	if (!f->fourstep && (pin.pinned || pin.dev) && (pout.pinned || pout.dev) && (pkern.pinned || pkern.dev)) {
		rc = fs_launch_variant_ex(f, fs_pick_variant(f, op, count), op, (float *)pout.kaddr,
		                          (const float *)pin.kaddr, (const float *)pkern.kaddr, count, in_stride, out_stride,
		                          fs->stream, 1);
		if (rc)
			return rc < 0 ? fs_latch(fs, -rc, 0) : fs_latch(fs, FFTSET_E_CUDA, rc);
		if ((rc = fs_cuda(fs, cudaStreamSynchronize(fs->stream))) != 0)
			return rc;
		return fs_check_flag(fs);
	}

	/* pageable host buffers: stage through device memory */
	pthread_mutex_lock(&fs->lock);
	staged = 1;
	if (!f->fourstep && count > 1 && count * nf * sizeof(float) >= 2 * FS_CHUNK_BYTES &&
	    in_stride >= nf && out_stride >= nf) {
		if (!pkern.dev) {
			if ((rc = fs_stage_reserve(fs, 2, nf * sizeof(float))))
				goto done;
			dkern = (const float *)fs->stage[2];
			if ((e = cudaMemcpyAsync(fs->stage[2], kern, nf * sizeof(float), cudaMemcpyHostToDevice,
			                         fs->stream)) != cudaSuccess) {
				rc = fs_cuda(fs, e);
				goto done;
			}
		}
		rc = fs_exec_pipelined(f, op, out, out_stride, in, in_stride, dkern, count, pin.dev, pout.dev);
		goto done;
	}
	if (!pin.dev) {
		if ((rc = fs_stage_reserve(fs, 0, in_span * sizeof(float))))
			goto done;
		din = (const float *)fs->stage[0];
		if ((e = fs_copy_rows((float *)fs->stage[0], in, count > 1 ? in_stride : nf, nf, count, cudaMemcpyHostToDevice,
		                      fs->stream)) !=
		    cudaSuccess) {
			rc = fs_cuda(fs, e);
			goto done;
		}
	}
	if (!pkern.dev) {
		if ((rc = fs_stage_reserve(fs, 2, nf * sizeof(float))))
			goto done;
		dkern = (const float *)fs->stage[2];
		if ((e = cudaMemcpyAsync(fs->stage[2], kern, nf * sizeof(float), cudaMemcpyHostToDevice, fs->stream)) !=
		    cudaSuccess) {
			rc = fs_cuda(fs, e);
			goto done;
		}
	}
	if (!pout.dev) {
		if ((rc = fs_stage_reserve(fs, 1, out_span * sizeof(float))))
			goto done;
		dout = (float *)fs->stage[1];
	}
	rc = fs_launch(f, op, dout, din, dkern, count, in_stride, out_stride);
	if (rc) {
		rc = rc < 0 ? fs_latch(fs, -rc, 0) : fs_latch(fs, FFTSET_E_CUDA, rc);
		goto done;
	}
	if (dout != out) {
		if ((e = fs_copy_rows(out, dout, count > 1 ? out_stride : nf, nf, count, cudaMemcpyDeviceToHost, fs->stream)) !=
		    cudaSuccess) {
			rc = fs_cuda(fs, e);
			goto done;
		}
	}
	rc = fs_cuda(fs, cudaStreamSynchronize(fs->stream));
	if (rc == FFTSET_OK)
		rc = fs_check_flag(fs);
done:
	if (staged)
		pthread_mutex_unlock(&fs->lock);
	return rc;
}

void fftset_fft_forward(const struct fftset_fft *first_pass, float *output_buf, const float *input_buf, float *work_buf)
{
	(void)work_buf;
	FS_RANGE_PUSH("fftset_fft_forward");
	fs_exec(first_pass, FGK_OP_FORWARD, output_buf, 0, input_buf, 0, NULL, 1);
	FS_RANGE_POP();
}

void fftset_fft_inverse(const struct fftset_fft *first_pass, float *output_buf, const float *input_buf, float *work_buf)
{
	(void)work_buf;
	FS_RANGE_PUSH("fftset_fft_inverse");
	fs_exec(first_pass, FGK_OP_INVERSE, output_buf, 0, input_buf, 0, NULL, 1);
	FS_RANGE_POP();
}

void fftset_fft_conv_get_kernel(const struct fftset_fft *first_pass, float *output_buf, const float *input_buf)
{
	FS_RANGE_PUSH("fftset_fft_conv_get_kernel");
	fs_exec(first_pass, FGK_OP_KERNEL, output_buf, 0, input_buf, 0, NULL, 1);
	FS_RANGE_POP();
}

void fftset_fft_conv(const struct fftset_fft *first_pass, float *output_buf, const float *input_buf,
                     const float *kernel_buf, float *work_buf)
{
	(void)work_buf;
	FS_RANGE_PUSH("fftset_fft_conv");
	fs_exec(first_pass, FGK_OP_CONV, output_buf, 0, input_buf, 0, kernel_buf, 1);
	FS_RANGE_POP();
}

int fftset_fft_forward_batch(const struct fftset_fft *fft, float *output_buf, size_t out_stride,
                             const float *input_buf, size_t in_stride, unsigned count)
{
	int rc;
	FS_RANGE_PUSH("fftset_fft_forward_batch");
	rc = fs_exec(fft, FGK_OP_FORWARD, output_buf, out_stride, input_buf, in_stride, NULL, count);
	FS_RANGE_POP();
	return rc;
}

int fftset_fft_inverse_batch(const struct fftset_fft *fft, float *output_buf, size_t out_stride,
                             const float *input_buf, size_t in_stride, unsigned count)
{
	int rc;
	FS_RANGE_PUSH("fftset_fft_inverse_batch");
	rc = fs_exec(fft, FGK_OP_INVERSE, output_buf, out_stride, input_buf, in_stride, NULL, count);
	FS_RANGE_POP();
	return rc;
}

int fftset_fft_conv_batch(const struct fftset_fft *fft, float *output_buf, size_t out_stride,
                          const float *input_buf, size_t in_stride, const float *kernel_buf, unsigned count)
{
	int rc;
	FS_RANGE_PUSH("fftset_fft_conv_batch");
	rc = fs_exec(fft, FGK_OP_CONV, output_buf, out_stride, input_buf, in_stride, kernel_buf, count);
	FS_RANGE_POP();
	return rc;
}

int fftset_fft_conv_get_kernel_batch(const struct fftset_fft *fft, float *output_buf, size_t out_stride,
                                     const float *input_buf, size_t in_stride, unsigned count)
{
	int rc;
	FS_RANGE_PUSH("fftset_fft_conv_get_kernel_batch");
	rc = fs_exec(fft, FGK_OP_KERNEL, output_buf, out_stride, input_buf, in_stride, NULL, count);
	FS_RANGE_POP();
	return rc;
}

/* ------------------------------------------------------------------------
 * Helpers and settings */

/* Smallest 2^a 3^b >= min built by the reference's greedy rule: double when
 * that reaches min, else triple when that does, else quadruple
 * (src/fftset.c:131-143). */
static unsigned fs_round_up_23(unsigned min)
{
	unsigned length = 1;
	while (length < min) {
		if (length * 2 >= min)
			length *= 2;
		else if (length * 3 >= min)
			length *= 3;
		else
			length *= 4;
	}
	return length;
}

/* src/fftset.c:145-167: blocks of 8 kernel lengths are the target; the
 * real DFT length is a multiple of 32 reals, so the result (complex bins) is
 * 16 times the rounded-up number of 32-real units. */
unsigned fftset_recommend_conv_length(unsigned kernel_length, unsigned max_block_size)
{
	const unsigned target = 8 * kernel_length;
	const unsigned block = max_block_size > target ? max_block_size : target;
	const unsigned min_real = kernel_length + block - 1;
	return 16u * fs_round_up_23((min_real + 31u) / 32u);
}

int fftset_last_error(const struct fftset *fc)
{
	struct fs_impl *fs = fs_of(fc);
	if (!fs)
		return FFTSET_E_INVALID;
	fs_check_flag(fs); /* picks up kernel reports of non-blocking calls once they finished */
	return __atomic_load_n(&fs->err, __ATOMIC_ACQUIRE);
}

int fftset_clear_error(struct fftset *fc)
{
	struct fs_impl *fs = fs_of(fc);
	int e;
	if (!fs)
		return FFTSET_E_INVALID;
	e = __atomic_exchange_n(&fs->err, 0, __ATOMIC_ACQ_REL);
	__atomic_store_n(&fs->cuda_err, 0, __ATOMIC_RELEASE);
	return e;
}

int fftset_cuda_error(const struct fftset *fc)
{
	struct fs_impl *fs = fs_of(fc);
	return fs ? fs->cuda_err : 0;
}

const char *fftset_error_string(int code)
{
	switch (code) {
	case FFTSET_OK: return "ok";
	case FFTSET_E_INVALID: return "invalid argument or size";
	case FFTSET_E_NOMEM: return "out of memory";
	case FFTSET_E_CUDA: return "CUDA error";
	case FFTSET_E_UNSUPPORTED: return "unsupported operation for this plan";
	case FFTSET_E_TIMEOUT: return "a bounded wait inside a kernel gave up";
	default: return "unknown error";
	}
}

int fftset_set_stream(struct fftset *fc, void *cuda_stream)
{
	struct fs_impl *fs = fs_of(fc);
	if (!fs)
		return FFTSET_E_INVALID;
	fs->stream = (cudaStream_t)cuda_stream;
	return FFTSET_OK;
}

void *fftset_get_stream(const struct fftset *fc)
{
	struct fs_impl *fs = fs_of(fc);
	return fs ? (void *)fs->stream : NULL;
}

void *fftset_own_stream(const struct fftset *fc)
{
	struct fs_impl *fs = fs_of(fc);
	return fs ? (void *)fs->own_stream : NULL;
}

int fftset__test_set_spin_limit(struct fftset *fc, unsigned polls)
{
	struct fs_impl *fs = fs_of(fc);
	if (!fs || polls == 0)
		return FFTSET_E_INVALID;
	fs->spin_limit = polls;
	return FFTSET_OK;
}

int fftset__test_set_call_service(struct fftset *fc, unsigned idle_polls)
{
	struct fs_impl *fs = fs_of(fc);
	if (!fs)
		return FFTSET_E_INVALID;
	pthread_mutex_lock(&fs->lock);
	fs_serve_stop(fs);
	fs->srv.idle_polls = idle_polls;
	fs->srv.broken = 0;
	fs->srv.last_f = NULL;
	pthread_mutex_unlock(&fs->lock);
	return FFTSET_OK;
}

unsigned long long fftset__test_served_calls(struct fftset *fc)
{
	struct fs_impl *fs = fs_of(fc);
	return fs ? fs->srv.served : 0;
}

int fftset__test_set_task_shape(struct fftset *fc, int shape)
{
	struct fs_impl *fs = fs_of(fc);
	if (!fs || shape < -1 || shape > FGK_SHAPE_SINGLE)
		return FFTSET_E_INVALID;
	fs->task_shape = shape;
	return FFTSET_OK;
}

int fftset__test_set_group_distance(struct fftset *fc, unsigned slots)
{
	struct fs_impl *fs = fs_of(fc);
	if (!fs)
		return FFTSET_E_INVALID;
	fs->group_dist = slots;
	return FFTSET_OK;
}

int fftset_set_blocking(struct fftset *fc, int blocking)
{
	struct fs_impl *fs = fs_of(fc);
	if (!fs)
		return FFTSET_E_INVALID;
	fs->blocking = blocking ? 1 : 0;
	return FFTSET_OK;
}

int fftset_set_kernel_layout(struct fftset *fc, unsigned simd_width)
{
	struct fs_impl *fs = fs_of(fc);
	if (!fs || (simd_width != 1 && simd_width != 4 && simd_width != 8))
		return fs_latch(fs, FFTSET_E_INVALID, 0);
	fs->layout_vw = simd_width;
	return FFTSET_OK;
}

unsigned fftset_fft_kernel_lanes(const struct fftset_fft *fft)
{
	return fft ? fft->lanes : 0;
}

unsigned fftset_fft_bins(const struct fftset_fft *fft)
{
	return fft ? fft->lfft : 0;
}

int fftset_kernel_layout(const struct fftset_modulation *modulation, unsigned complex_bins, unsigned simd_width,
                         int *re_offsets, unsigned *lanes)
{
	if ((modulation != FFTSET_MODULATION_COMPLEX && modulation != FFTSET_MODULATION_FREQ_OFFSET_REAL) ||
	    !fs_valid_size(complex_bins) || re_offsets == NULL || lanes == NULL ||
	    (simd_width != 1 && simd_width != 4 && simd_width != 8))
		return FFTSET_E_INVALID;
	if (fsl_kernel_offsets(modulation->freq_offset_real, complex_bins, simd_width, (int32_t *)re_offsets, lanes))
		return FFTSET_E_INVALID;
	return FFTSET_OK;
}

/* ------------------------------------------------------------------------
 * Kernel variants and the autotuner */

int fftset_fft_variants(const struct fftset_fft *fft)
{
	return fft ? fft->nvar : 0;
}

int fftset_fft_variant(const struct fftset_fft *fft, int op)
{
	if (!fft || op < 0 || op >= FGK_OP_COUNT)
		return -1;
	return fft->sel[op];
}

int fftset_fft_set_variant(const struct fftset_fft *fft, int op, int variant)
{
	struct fftset_fft *f = (struct fftset_fft *)fft; /* the plan object is the library's own */
	if (!f || op < 0 || op >= FGK_OP_COUNT || variant < -1 || variant >= f->nvar)
		return FFTSET_E_INVALID;
	if (variant >= 0 && !(f->vops[variant] & (1u << op)))
		return FFTSET_E_UNSUPPORTED;
	f->sel[op] = variant;
	return FFTSET_OK;
}

/* Times every kernel that can run `op` for this plan (the generic resident
 * kernel and each compile-time variant) on `count` blocks of scratch device
 * memory, and selects the fastest for batched calls of that op. */
int fftset_fft_autotune(const struct fftset_fft *fft, int op, unsigned count, float *best_ms)
{
	struct fftset_fft *f = (struct fftset_fft *)fft;
	struct fs_impl *fs;
	float *in = NULL, *out = NULL, *kern = NULL, best = -1.0f;
	size_t nf;
	cudaEvent_t e0 = NULL, e1 = NULL;
	cudaError_t e;
	int v, rep, bestv = -1, rc = FFTSET_OK;
	if (!f || op < 0 || op >= FGK_OP_COUNT || count == 0)
		return FFTSET_E_INVALID;
	fs = f->fs;
	nf = 2 * (size_t)f->lfft;
	if ((e = cudaMalloc((void **)&in, nf * count * sizeof(float))) != cudaSuccess ||
	    (e = cudaMalloc((void **)&out, nf * count * sizeof(float))) != cudaSuccess ||
	    (e = cudaMalloc((void **)&kern, nf * sizeof(float))) != cudaSuccess) {
		cudaGetLastError();
		rc = fs_latch(fs, FFTSET_E_NOMEM, (int)e);
		goto done;
	}
	if ((e = cudaMemsetAsync(in, 0, nf * count * sizeof(float), fs->stream)) != cudaSuccess ||
	    (e = cudaMemsetAsync(kern, 0, nf * sizeof(float), fs->stream)) != cudaSuccess ||
	    (e = cudaEventCreate(&e0)) != cudaSuccess || (e = cudaEventCreate(&e1)) != cudaSuccess) {
		rc = fs_cuda(fs, e);
		goto done;
	}
	for (v = -1; v < f->nvar; v++) {
		float ms = 0, vbest = -1.0f;
		if (v >= 0 && !(f->vops[v] & (1u << op)))
			continue;
		for (rep = 0; rep < 7; rep++) {
			if ((e = cudaEventRecord(e0, fs->stream)) != cudaSuccess) {
				rc = fs_cuda(fs, e);
				goto done;
			}
			if ((rc = fs_launch_variant(f, v, op, out, in, kern, count, nf, nf, fs->stream)) != 0) {
				rc = fs_latch(fs, FFTSET_E_CUDA, rc);
				goto done;
			}
			if ((e = cudaEventRecord(e1, fs->stream)) != cudaSuccess ||
			    (e = cudaEventSynchronize(e1)) != cudaSuccess ||
			    (e = cudaEventElapsedTime(&ms, e0, e1)) != cudaSuccess) {
				rc = fs_cuda(fs, e);
				goto done;
			}
			if (rep >= 2 && (vbest < 0 || ms < vbest))
				vbest = ms;
		}
		if (best < 0 || vbest < best) {
			best = vbest;
			bestv = v;
		}
	}
	f->sel[op] = bestv;
	if (best_ms)
		*best_ms = best;
done:
	if (e0)
		cudaEventDestroy(e0);
	if (e1)
		cudaEventDestroy(e1);
	cudaStreamSynchronize(fs->stream);
	cudaFree(in);
	cudaFree(out);
	cudaFree(kern);
	return rc;
}

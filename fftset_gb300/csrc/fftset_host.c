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
#include "fftset_layout.h"
#include "fgk.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

struct fftset_modulation {
	int         freq_offset_real;
	const char *name;
};

static const struct fftset_modulation FS_MOD_FREQOFF = {1, "FREQ_OFFSET_REAL"};
static const struct fftset_modulation FS_MOD_COMPLEX = {0, "COMPLEX"};
const struct fftset_modulation *FFTSET_MODULATION_FREQ_OFFSET_REAL = &FS_MOD_FREQOFF;
const struct fftset_modulation *FFTSET_MODULATION_COMPLEX = &FS_MOD_COMPLEX;

struct fs_impl;

struct fftset_fft {
	unsigned                        lfft;
	const struct fftset_modulation *modulator;
	struct fftset_fft              *next;
	struct fs_impl                 *fs;
	unsigned                        lanes; /* kernel-buffer lane width */
	fgk_plan                        rp;    /* resident plan (device pointers inside) */
	void                           *dmem;  /* one device block for all tables */
};

#define FS_NSTAGE 3 /* staging buffers: input, output, kernel */

struct fs_impl {
	cudaStream_t       stream;
	cudaStream_t       own_stream;
	int                blocking;
	unsigned           layout_vw;
	int                err;
	int                cuda_err;
	int                device;
	unsigned           max_smem;
	struct fftset_fft *first;
	pthread_mutex_t    lock;
	void              *stage[FS_NSTAGE];
	size_t             stage_bytes[FS_NSTAGE];
};

static struct fs_impl *fs_of(const struct fftset *fc)
{
	return fc ? (struct fs_impl *)fc->impl : NULL;
}

static int fs_latch(struct fs_impl *fs, int code, int cuda_err)
{
	if (fs && code && !fs->err) {
		fs->err = code;
		fs->cuda_err = cuda_err;
	}
	return code;
}

static int fs_cuda(struct fs_impl *fs, cudaError_t e)
{
	if (e == cudaSuccess)
		return FFTSET_OK;
	return fs_latch(fs, e == cudaErrorMemoryAllocation ? FFTSET_E_NOMEM : FFTSET_E_CUDA, (int)e);
}

/* ------------------------------------------------------------------------ */

int fftset_init(struct fftset *fc)
{
	struct fs_impl *fs;
	int dev = 0, smem = 0;
	if (fc == NULL)
		return -1;
	memset(fc, 0, sizeof(*fc));
	if (cudaGetDevice(&dev) != cudaSuccess) {
		cudaGetLastError();
		return -1;
	}
	if (cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
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
	if (pthread_mutex_init(&fs->lock, NULL) != 0) {
		cudaStreamDestroy(fs->own_stream);
		free(fs);
		return -1;
	}
	fs->stream = fs->own_stream;
	fs->blocking = 1;
	fs->layout_vw = 4;
	fs->device = dev;
	fs->max_smem = (unsigned)smem;
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
	for (p = fs->first; p != NULL; p = n) {
		n = p->next;
		cudaFree(p->dmem);
		free(p);
	}
	for (i = 0; i < FS_NSTAGE; i++)
		cudaFree(fs->stage[i]);
	cudaStreamDestroy(fs->own_stream);
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

/* Build the device tables of a resident plan. */
static int fs_build_resident(struct fs_impl *fs, struct fftset_fft *f)
{
	fgk_plan *rp = &f->rp;
	size_t ntw, o_plan, o_tw, o_mod, o_kidx, total;
	float *tw = NULL, *mod = NULL;
	int32_t *kidx = NULL;
	char *d = NULL;
	unsigned L = f->lfft, i, lanes = 0;
	int rc = FFTSET_E_NOMEM;
	cudaError_t e;

	if (fgk_plan_resident(rp, L, f->modulator->freq_offset_real ? FGK_MOD_FREQOFF : FGK_MOD_COMPLEX, fs->max_smem))
		return FFTSET_E_UNSUPPORTED;
	ntw = fgk_plan_twiddles(rp, NULL);
	tw = (float *)malloc(sizeof(float) * 2 * (ntw ? ntw : 1));
	mod = (float *)malloc(sizeof(float) * 2 * L);
	kidx = (int32_t *)malloc(sizeof(int32_t) * L);
	if (!tw || !mod || !kidx)
		goto out;
	fgk_plan_twiddles(rp, tw);
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
	e = cudaMalloc((void **)&d, total);
	if (e != cudaSuccess) {
		cudaGetLastError();
		goto out;
	}
	rp->tw = d + o_tw;
	rp->modtw = d + o_mod;
	rp->kidx = (const int32_t *)(d + o_kidx);
	rp->dev = (const fgk_plan *)(d + o_plan);
	if ((e = cudaMemcpy(d + o_tw, tw, sizeof(float) * 2 * ntw, cudaMemcpyHostToDevice)) != cudaSuccess ||
	    (e = cudaMemcpy(d + o_mod, mod, sizeof(float) * 2 * L, cudaMemcpyHostToDevice)) != cudaSuccess ||
	    (e = cudaMemcpy(d + o_kidx, kidx, sizeof(int32_t) * L, cudaMemcpyHostToDevice)) != cudaSuccess ||
	    (e = cudaMemcpy(d + o_plan, rp, sizeof(fgk_plan), cudaMemcpyHostToDevice)) != cudaSuccess) {
		fs_cuda(fs, e);
		cudaFree(d);
		rc = FFTSET_E_CUDA;
		goto out;
	}
	f->dmem = d;
	rc = FFTSET_OK;
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
	struct fftset_fft *p, **ipos;
	int rc;
	if (fs == NULL)
		return NULL;
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
		fs_latch(fs, FFTSET_E_NOMEM, 0);
		return NULL;
	}
	p->lfft = complex_bins;
	p->modulator = modulation;
	p->fs = fs;
	rc = fs_build_resident(fs, p);
	if (rc) {
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

static int fs_is_device_ptr(const void *ptr)
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

static int fs_stage_reserve(struct fs_impl *fs, int slot, size_t bytes)
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
	if (count == 0)
		return FFTSET_OK;
	in_span = (size_t)(count - 1) * in_stride + nf;
	out_span = (size_t)(count - 1) * out_stride + nf;

	if (fs_is_device_ptr(in) && fs_is_device_ptr(out) && (kern == NULL || fs_is_device_ptr(kern))) {
		rc = fgk_launch_resident(&f->rp, op, out, in, kern, count, in_stride, out_stride, fs->stream);
		if (rc)
			return fs_latch(fs, FFTSET_E_CUDA, rc);
		if (fs->blocking)
			return fs_cuda(fs, cudaStreamSynchronize(fs->stream));
		return FFTSET_OK;
	}

	/* host buffers: stage through device memory */
	pthread_mutex_lock(&fs->lock);
	staged = 1;
	if (!fs_is_device_ptr(in)) {
		if ((rc = fs_stage_reserve(fs, 0, in_span * sizeof(float))))
			goto done;
		din = (const float *)fs->stage[0];
		if ((e = cudaMemcpyAsync(fs->stage[0], in, in_span * sizeof(float), cudaMemcpyHostToDevice, fs->stream)) !=
		    cudaSuccess) {
			rc = fs_cuda(fs, e);
			goto done;
		}
	}
	if (kern != NULL && !fs_is_device_ptr(kern)) {
		if ((rc = fs_stage_reserve(fs, 2, nf * sizeof(float))))
			goto done;
		dkern = (const float *)fs->stage[2];
		if ((e = cudaMemcpyAsync(fs->stage[2], kern, nf * sizeof(float), cudaMemcpyHostToDevice, fs->stream)) !=
		    cudaSuccess) {
			rc = fs_cuda(fs, e);
			goto done;
		}
	}
	if (!fs_is_device_ptr(out)) {
		if ((rc = fs_stage_reserve(fs, 1, out_span * sizeof(float))))
			goto done;
		dout = (float *)fs->stage[1];
	}
	rc = fgk_launch_resident(&f->rp, op, dout, din, dkern, count, in_stride, out_stride, fs->stream);
	if (rc) {
		rc = fs_latch(fs, FFTSET_E_CUDA, rc);
		goto done;
	}
	if (dout != out) {
		if ((e = cudaMemcpyAsync(out, dout, out_span * sizeof(float), cudaMemcpyDeviceToHost, fs->stream)) !=
		    cudaSuccess) {
			rc = fs_cuda(fs, e);
			goto done;
		}
	}
	rc = fs_cuda(fs, cudaStreamSynchronize(fs->stream));
done:
	if (staged)
		pthread_mutex_unlock(&fs->lock);
	return rc;
}

void fftset_fft_forward(const struct fftset_fft *first_pass, float *output_buf, const float *input_buf, float *work_buf)
{
	(void)work_buf;
	fs_exec(first_pass, FGK_OP_FORWARD, output_buf, 0, input_buf, 0, NULL, 1);
}

void fftset_fft_inverse(const struct fftset_fft *first_pass, float *output_buf, const float *input_buf, float *work_buf)
{
	(void)work_buf;
	fs_exec(first_pass, FGK_OP_INVERSE, output_buf, 0, input_buf, 0, NULL, 1);
}

void fftset_fft_conv_get_kernel(const struct fftset_fft *first_pass, float *output_buf, const float *input_buf)
{
	fs_exec(first_pass, FGK_OP_KERNEL, output_buf, 0, input_buf, 0, NULL, 1);
}

void fftset_fft_conv(const struct fftset_fft *first_pass, float *output_buf, const float *input_buf,
                     const float *kernel_buf, float *work_buf)
{
	(void)work_buf;
	fs_exec(first_pass, FGK_OP_CONV, output_buf, 0, input_buf, 0, kernel_buf, 1);
}

int fftset_fft_forward_batch(const struct fftset_fft *fft, float *output_buf, size_t out_stride,
                             const float *input_buf, size_t in_stride, unsigned count)
{
	return fs_exec(fft, FGK_OP_FORWARD, output_buf, out_stride, input_buf, in_stride, NULL, count);
}

int fftset_fft_inverse_batch(const struct fftset_fft *fft, float *output_buf, size_t out_stride,
                             const float *input_buf, size_t in_stride, unsigned count)
{
	return fs_exec(fft, FGK_OP_INVERSE, output_buf, out_stride, input_buf, in_stride, NULL, count);
}

int fftset_fft_conv_batch(const struct fftset_fft *fft, float *output_buf, size_t out_stride,
                          const float *input_buf, size_t in_stride, const float *kernel_buf, unsigned count)
{
	return fs_exec(fft, FGK_OP_CONV, output_buf, out_stride, input_buf, in_stride, kernel_buf, count);
}

int fftset_fft_conv_get_kernel_batch(const struct fftset_fft *fft, float *output_buf, size_t out_stride,
                                     const float *input_buf, size_t in_stride, unsigned count)
{
	return fs_exec(fft, FGK_OP_KERNEL, output_buf, out_stride, input_buf, in_stride, NULL, count);
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
	return fs ? fs->err : FFTSET_E_INVALID;
}

int fftset_clear_error(struct fftset *fc)
{
	struct fs_impl *fs = fs_of(fc);
	int e;
	if (!fs)
		return FFTSET_E_INVALID;
	e = fs->err;
	fs->err = 0;
	fs->cuda_err = 0;
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
	default: return "unknown error";
	}
}

int fftset_set_stream(struct fftset *fc, void *cuda_stream)
{
	struct fs_impl *fs = fs_of(fc);
	if (!fs)
		return FFTSET_E_INVALID;
	fs->stream = cuda_stream ? (cudaStream_t)cuda_stream : fs->own_stream;
	return FFTSET_OK;
}

void *fftset_get_stream(const struct fftset *fc)
{
	struct fs_impl *fs = fs_of(fc);
	return fs ? (void *)fs->stream : NULL;
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

/* The adjoint of fftset_fft_conv (no reference counterpart; the reference
 * computes only the forward convolution, src/fftset_vec.c:1161-1220).
 *
 * For a batch y_b = conv(x_b, K), K = fftset_fft_conv_get_kernel(h), and
 * upstream gradients g_b = dLoss/dy_b:
 *   grad_input_b = the convolution of g_b with the conjugated kernel
 *                  spectrum (FGK_OP_CORR: the same fused DIF -> product ->
 *                  DIT kernels as fftset_fft_conv), i.e. complex_bins times
 *                  the negacyclic (FREQ_OFFSET_REAL) or cyclic (COMPLEX)
 *                  cross-correlation of g_b with h;
 *   grad_taps    = inverse( sum_b G_b conj(X_b) ), the gradient with respect
 *                  to the taps h: where the size has a compiled taps-gradient
 *                  kernel (fgk_static.cuh, static_kernel_kgrad), one pass that
 *                  transforms both blocks of every pair and accumulates the
 *                  product per CTA; otherwise batched forward transforms of
 *                  g and x into scratch and column sums (fgk_adjoint.cu);
 *                  then the row sums and the plan's inverse.
 * For FREQ_OFFSET_REAL (real data) these are the gradients of a real loss;
 * for COMPLEX they are the adjoint linear maps. */
#include <stdint.h>
#include <stdlib.h>

#include <cuda_runtime_api.h>

#include "fftset.h"
#include "fftset_internal.h"
#include "fgk.h"

#define FSA_SLOT 4                       /* staging slot of the adjoint's scratch */
#define FSA_SPEC_CAP ((size_t)256 << 20) /* bytes of spectra per sub-batch */
#define FSA_CHUNKS 64                    /* partial rows per sub-batch */

/* implemented in fgk_adjoint.cu */
int fgk_launch_kgrad_spec(const float *S, const float *X, size_t stride, uint32_t count, uint32_t L, uint32_t chunk,
                          float *partials, void *stream);
int fgk_launch_kgrad_reduce(const float *partials, uint32_t P, uint32_t L, int pack, float *out, void *stream);

static size_t fsa_align(size_t floats)
{
	return (floats + 63) & ~(size_t)63; /* 256-byte boundaries */
}

static int fsa_rc(struct fs_impl *fs, int rc)
{
	if (rc == 0)
		return FFTSET_OK;
	return rc < 0 ? fs_latch(fs, -rc, 0) : fs_latch(fs, FFTSET_E_CUDA, rc);
}

/* grad_taps through the compiled taps-gradient kernel (sizes that have
 * one): every block pair transformed and multiplied in shared memory and
 * registers, one partial row per CTA, the rows summed into the
 * FREQ_OFFSET_REAL forward layout (or natural order), then the inverse.
 * Returns -FFTSET_E_UNSUPPORTED when the size has no such kernel. */
static int fsa_taps_fused(const struct fftset_fft *f, float *grad_taps, const float *g, size_t g_stride,
                          const float *x, size_t x_stride, unsigned count, float *grad_input, size_t gi_stride,
                          const float *kern)
{
	struct fs_impl *fs = f->fs;
	const size_t L = f->lfft, nf = 2 * L;
	const int v = fgk_static_kgrad_variant(f->rp.modulation, (uint32_t)L);
	const uint32_t cap = 4u * (uint32_t)fs->num_sms;
	uint32_t rows = 0;
	float *partials, *S;
	int rc;
	if (v < 0 || v >= f->nvar)
		return -FFTSET_E_UNSUPPORTED;
	if ((rc = fs_stage_reserve(fs, FSA_SLOT, ((size_t)cap + 1) * nf * sizeof(float))) != 0)
		return -rc;
	partials = (float *)fs->stage[FSA_SLOT];
	S = partials + (size_t)cap * nf;
	if (grad_input)
		/* both gradients in one pass: g_b is transformed once for both */
		rc = fgk_launch_static_adj(&f->vp[v], v, g, g_stride, x, x_stride, grad_input, gi_stride, kern, count,
		                           partials, cap, &rows, fs->stream, fs->num_sms);
	else
		rc = fgk_launch_static_kgrad(&f->vp[v], v, g, g_stride, x, x_stride, count, partials, cap, &rows, fs->stream,
		                             fs->num_sms);
	if (rc != 0)
		return rc < 0 ? -FFTSET_E_UNSUPPORTED : rc;
	if ((rc = fgk_launch_kgrad_reduce(partials, rows, (uint32_t)L, f->modulator->freq_offset_real, S, fs->stream)) !=
	    0)
		return rc;
	return fs_launch(f, FGK_OP_INVERSE, grad_taps, S, NULL, 1, 0, 0);
}

/* grad_taps: batched forward transforms into scratch, column sums of
 * G conj(X), then the inverse */
static int fsa_taps(const struct fftset_fft *f, float *grad_taps, const float *g, size_t g_stride,
                            const float *x, size_t x_stride, unsigned count)
{
	struct fs_impl *fs = f->fs;
	const size_t L = f->lfft, nf = 2 * L;
	size_t sub = FSA_SPEC_CAP / (2 * nf * sizeof(float));
	size_t nsub, spec, part_floats, done;
	uint32_t P = 0;
	float *Gs, *Xs, *partials, *S;
	int rc;
	if (sub < 1)
		sub = 1;
	if (sub > count)
		sub = count;
	nsub = (count + sub - 1) / sub;
	spec = fsa_align(sub * nf);
	part_floats = fsa_align(nsub * FSA_CHUNKS * nf);
	if ((rc = fs_stage_reserve(fs, FSA_SLOT, (2 * spec + part_floats + nf) * sizeof(float))) != 0)
		return -rc;
	Gs = (float *)fs->stage[FSA_SLOT];
	Xs = Gs + spec;
	partials = Xs + spec;
	S = partials + part_floats;
	for (done = 0; done < count; done += sub) {
		const unsigned m = (unsigned)(count - done < sub ? count - done : sub);
		const uint32_t chunk = (m + FSA_CHUNKS - 1) / FSA_CHUNKS;
		const uint32_t rows = (m + chunk - 1) / chunk;
		if ((rc = fs_launch(f, FGK_OP_FORWARD, Gs, g + done * g_stride, NULL, m, g_stride, nf)) != 0)
			return rc;
		if ((rc = fs_launch(f, FGK_OP_FORWARD, Xs, x + done * x_stride, NULL, m, x_stride, nf)) != 0)
			return rc;
		if ((rc = fgk_launch_kgrad_spec(Gs, Xs, nf, m, (uint32_t)L, chunk, partials + (size_t)P * nf, fs->stream)) !=
		    0)
			return rc;
		P += rows;
	}
	if ((rc = fgk_launch_kgrad_reduce(partials, P, (uint32_t)L, 0, S, fs->stream)) != 0)
		return rc;
	return fs_launch(f, FGK_OP_INVERSE, grad_taps, S, NULL, 1, 0, 0);
}

int fftset_fft_conv_adjoint_batch(const struct fftset_fft *fft, float *grad_input, size_t gi_stride,
                                  float *grad_taps, const float *grad_output, size_t go_stride, const float *input_buf,
                                  size_t in_stride, const float *kernel_buf, unsigned count)
{
	struct fs_impl *fs;
	size_t nf;
	int rc = 0;

	if (fft == NULL)
		return FFTSET_E_INVALID;
	fs = fft->fs;
	nf = 2 * (size_t)fft->lfft;
	if (count == 0) {
		/* an empty batch: no input gradient, zero taps gradient */
		if (grad_taps == NULL)
			return FFTSET_OK;
		if (((uintptr_t)grad_taps & 7) || !fs_is_device_ptr(grad_taps))
			return fs_latch(fs, FFTSET_E_INVALID, 0);
		if ((rc = fs_cuda(fs, cudaMemsetAsync(grad_taps, 0, nf * sizeof(float), fs->stream))) != 0)
			return rc;
		return fs->blocking ? fs_cuda(fs, cudaStreamSynchronize(fs->stream)) : FFTSET_OK;
	}
	if (grad_output == NULL || (grad_input != NULL && kernel_buf == NULL) ||
	    (grad_taps != NULL && input_buf == NULL))
		return fs_latch(fs, FFTSET_E_INVALID, 0);
	if (count > 1 && (go_stride < nf || (grad_input && gi_stride < nf) || (grad_taps && in_stride < nf) ||
	                  ((go_stride | gi_stride | in_stride) & 1)))
		return fs_latch(fs, FFTSET_E_INVALID, 0);
	if ((((uintptr_t)grad_input) | ((uintptr_t)grad_taps) | ((uintptr_t)grad_output) | ((uintptr_t)input_buf) |
	     ((uintptr_t)kernel_buf)) &
	    7)
		return fs_latch(fs, FFTSET_E_INVALID, 0);
	if (!fs_is_device_ptr(grad_input) || !fs_is_device_ptr(grad_taps) || !fs_is_device_ptr(grad_output) ||
	    !fs_is_device_ptr(input_buf) || !fs_is_device_ptr(kernel_buf))
		return fs_latch(fs, FFTSET_E_INVALID, 0); /* device buffers only */
	if (count == 1) {
		go_stride = nf;
		gi_stride = nf;
		in_stride = nf;
	}

	FS_RANGE_PUSH("fftset_fft_conv_adjoint_batch");
	pthread_mutex_lock(&fs->lock); /* the adjoint's scratch slot */
	rc = -FFTSET_E_UNSUPPORTED;
	if (grad_taps) {
		/* the compiled one-pass kernels where the size has them (both
		 * gradients, or the taps gradient alone) */
		rc = fsa_taps_fused(fft, grad_taps, grad_output, go_stride, input_buf, in_stride, count, grad_input,
		                    gi_stride, kernel_buf);
		if (rc != -FFTSET_E_UNSUPPORTED && (rc = fsa_rc(fs, rc)) != 0)
			goto done;
	}
	if (rc == -FFTSET_E_UNSUPPORTED || (!grad_taps && grad_input)) {
		if (grad_input) {
			rc = fs_launch(fft, FGK_OP_CORR, grad_input, grad_output, kernel_buf, count, go_stride, gi_stride);
			if ((rc = fsa_rc(fs, rc)) != 0)
				goto done;
		}
		if (grad_taps) {
			rc = fsa_taps(fft, grad_taps, grad_output, go_stride, input_buf, in_stride, count);
			if ((rc = fsa_rc(fs, rc)) != 0)
				goto done;
		}
	}
	if (fs->blocking) {
		if ((rc = fs_cuda(fs, cudaStreamSynchronize(fs->stream))) == 0)
			rc = fs_check_flag(fs);
	}
done:
	pthread_mutex_unlock(&fs->lock);
	FS_RANGE_POP();
	return rc;
}

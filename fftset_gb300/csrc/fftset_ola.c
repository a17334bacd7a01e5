/* Overlap-add block convolution on top of the batched convolution: the
 * streaming caller the reference is built for (README.md:3; block and
 * transform lengths from fftset_recommend_conv_length, src/fftset.c:145-167).
 * The reference leaves this loop to its users; here it is one call. Where
 * the size has the compiled fused kernel (static_kernel_ola) and the block
 * results overlap at most pairwise (K - 1 <= B), one launch reads the blocks
 * straight from the signal and adds their results into the zeroed output;
 * otherwise split into zero-padded blocks (fgk_ola.cu), one batched conv,
 * overlap-add gather into the output. */
#include <stdint.h>

#include <cuda_runtime_api.h>

#include "fftset.h"
#include "fftset_internal.h"
#include "fgk.h"

int fgk_launch_ola_split(const float *in, uint64_t n, uint32_t B, uint32_t N, uint32_t nblocks, int complex_samples,
                         float *blocks, int num_sms, void *stream);
int fgk_launch_ola_merge(const float *ys, uint32_t B, uint32_t N, uint32_t span, uint32_t nblocks, uint64_t nout,
                         int complex_samples, float *out, int num_sms, void *stream);

int fftset_fft_conv_overlap_add(const struct fftset_fft *fft, float *output_buf, const float *input_buf,
                                size_t samples, const float *kernel_buf, unsigned kernel_length,
                                unsigned block_length)
{
	struct fs_impl *fs;
	int cplx, rc;
	size_t N, nf, B, nblocks, bytes;
	float *blocks, *ys;

	if (fft == NULL)
		return FFTSET_E_INVALID;
	fs = fft->fs;
	cplx = !fft->modulator->freq_offset_real;
	nf = 2 * (size_t)fft->lfft;     /* floats per block */
	N = cplx ? fft->lfft : nf;       /* samples per block */
	if (!output_buf || !input_buf || !kernel_buf || kernel_length == 0 || kernel_length > N || samples == 0)
		return fs_latch(fs, FFTSET_E_INVALID, 0);
	B = block_length ? block_length : N - kernel_length + 1;
	if (B == 0 || B + kernel_length - 1 > N)
		return fs_latch(fs, FFTSET_E_INVALID, 0); /* the block's convolution would wrap */
	if (!fs_is_device_ptr(output_buf) || !fs_is_device_ptr(input_buf) || !fs_is_device_ptr(kernel_buf))
		return fs_latch(fs, FFTSET_E_INVALID, 0);
	if ((((uintptr_t)output_buf) | ((uintptr_t)input_buf) | ((uintptr_t)kernel_buf)) & (cplx ? 7 : 3))
		return fs_latch(fs, FFTSET_E_INVALID, 0);
	nblocks = (samples + B - 1) / B;
	if (nblocks > 0xffffffffu || N > 0xffffffffu)
		return fs_latch(fs, FFTSET_E_INVALID, 0);
	bytes = nblocks * nf * sizeof(float);

	FS_RANGE_PUSH("fftset_fft_conv_overlap_add");
	pthread_mutex_lock(&fs->lock); /* staging slots 0 and 1 */
	if (!cplx && B + kernel_length - 1 <= 2 * B &&
	    (input_buf + samples <= output_buf || output_buf + samples + kernel_length - 1 <= input_buf)) {
		/* the compiled fused form where the size has it: the blocks are read
		 * from the signal and their results written into the output, added
		 * where two blocks meet (at most two additions per output sample;
		 * those overlap zones, the first K - 1 samples of every B, are
		 * zeroed first, so the output must not overlap the signal) */
		const int v = fgk_static_ola_variant(FGK_MOD_FREQOFF, fft->lfft);
		if (v >= 0 && v < fft->nvar) {
			const size_t nout = samples + kernel_length - 1, ovl = kernel_length - 1;
			if (ovl) {
				/* rows of ovl floats, B apart; the last segment start may
				 * leave fewer than ovl samples before the end */
				const size_t full = nout >= ovl ? (nout - ovl) / B + 1 : 0, last = full * B;
				if (full && (rc = fs_cuda(fs, cudaMemset2DAsync(output_buf, B * sizeof(float), 0, ovl * sizeof(float),
				                                               full, fs->stream))) != 0)
					goto done;
				if (last < nout && (rc = fs_cuda(fs, cudaMemsetAsync(output_buf + last, 0,
				                                                     (nout - last) * sizeof(float), fs->stream))) != 0)
					goto done;
			}
			rc = fgk_launch_static_ola(&fft->vp[v], v, input_buf, samples, (uint32_t)B,
			                           (uint32_t)(B + kernel_length - 1), (uint32_t)nblocks,
			                           samples + kernel_length - 1, kernel_buf, output_buf, fs->stream, fs->num_sms);
			if (rc == 0)
				goto finish;
			if (rc > 0) {
				rc = fs_latch(fs, FFTSET_E_CUDA, rc);
				goto done;
			}
		}
	}
	if ((rc = fs_stage_reserve(fs, 0, bytes)) != 0 || (rc = fs_stage_reserve(fs, 1, bytes)) != 0)
		goto done;
	blocks = (float *)fs->stage[0];
	ys = (float *)fs->stage[1];
	if ((rc = fgk_launch_ola_split(input_buf, samples, (uint32_t)B, (uint32_t)N, (uint32_t)nblocks, cplx, blocks,
	                               fs->num_sms, fs->stream)) != 0) {
		rc = fs_latch(fs, FFTSET_E_CUDA, rc);
		goto done;
	}
	rc = fs_launch(fft, FGK_OP_CONV, ys, blocks, kernel_buf, (unsigned)nblocks, nf, nf);
	if (rc) {
		rc = rc < 0 ? fs_latch(fs, -rc, 0) : fs_latch(fs, FFTSET_E_CUDA, rc);
		goto done;
	}
	if ((rc = fgk_launch_ola_merge(ys, (uint32_t)B, (uint32_t)N, (uint32_t)(B + kernel_length - 1),
	                               (uint32_t)nblocks, samples + kernel_length - 1, cplx, output_buf, fs->num_sms,
	                               fs->stream)) != 0) {
		rc = fs_latch(fs, FFTSET_E_CUDA, rc);
		goto done;
	}
finish:
	rc = FFTSET_OK;
	if (fs->blocking) {
		if ((rc = fs_cuda(fs, cudaStreamSynchronize(fs->stream))) == 0)
			rc = fs_check_flag(fs);
	}
done:
	pthread_mutex_unlock(&fs->lock);
	FS_RANGE_POP();
	return rc;
}

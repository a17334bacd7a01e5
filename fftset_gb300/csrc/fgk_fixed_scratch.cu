/* fftset_fft_execute_fixed_scratch: the four-step passes with their work
 * buffer in a fixed device array instead of memory the library allocates.
 *
 * Who needs it: callers that must not allocate device memory while they run,
 * such as a real-time audio callback that has a deadline every few
 * milliseconds and must not block in the driver's allocator, or a host
 * that set a fixed device-memory budget up front. The regular calls grow
 * the fftset's own work buffer with cudaMalloc the first time a four-step
 * size (one beyond the shared-memory limit) runs with more blocks than
 * before; this entry point never does.
 *
 * The work buffer lives in `fgk_fixed_scratch` below, a file-scope device
 * array of FFTSET_FIXED_SCRATCH_FLOATS floats (32 MiB). Every GPU that
 * loads this library holds it until the process exits. Host code cannot
 * use the array's name as a device address (on the host it names a
 * stand-in object), so the first call on each device looks the address up
 * with cudaGetSymbolAddress while that device is current and keeps it. */
#include <cuda_runtime.h>
#include <pthread.h>
#include <stdint.h>

extern "C" {
#include "fftset_internal.h"
}
#include "fgk.h"

static __device__ __align__(256) float fgk_fixed_scratch[FFTSET_FIXED_SCRATCH_FLOATS];

#define FGK_FIXED_MAX_DEVICES 64

static pthread_mutex_t fgk_fixed_lock = PTHREAD_MUTEX_INITIALIZER;
static float *fgk_fixed_addr[FGK_FIXED_MAX_DEVICES];

/* Device address of the array on device `dev` (the current device). */
static cudaError_t fgk_fixed_scratch_address(int dev, float **addr)
{
	cudaError_t e = cudaSuccess;
	pthread_mutex_lock(&fgk_fixed_lock);
	if (fgk_fixed_addr[dev] == NULL) {
		void *p = NULL;
		e = cudaGetSymbolAddress(&p, fgk_fixed_scratch);
		if (e == cudaSuccess)
			fgk_fixed_addr[dev] = (float *)p;
	}
	*addr = fgk_fixed_addr[dev];
	pthread_mutex_unlock(&fgk_fixed_lock);
	return e;
}

extern "C" int fftset_fft_execute_fixed_scratch(const struct fftset_fft *fft, int op, float *output_buf,
                                                size_t out_stride, const float *input_buf, size_t in_stride,
                                                const float *kernel_buf, unsigned count)
{
	struct fs_impl *fs;
	size_t nf;
	float *scratch = NULL;
	int dev = -1, rc;
	cudaError_t e;

	if (fft == NULL)
		return FFTSET_E_INVALID;
	fs = fft->fs;
	nf = 2 * (size_t)fft->lfft;
	if (op < FFTSET_OP_FORWARD || op > FFTSET_OP_CORR)
		return fs_latch(fs, FFTSET_E_INVALID, 0);
	if (!fft->fourstep)
		return fs_latch(fs, FFTSET_E_UNSUPPORTED, 0); /* resident sizes use no scratch */
	if (output_buf == NULL || input_buf == NULL ||
	    ((op == FFTSET_OP_CONV || op == FFTSET_OP_CORR) && kernel_buf == NULL))
		return fs_latch(fs, FFTSET_E_INVALID, 0);
	if (count == 0)
		return FFTSET_OK;
	if (count > 1 && (in_stride < nf || out_stride < nf || ((in_stride | out_stride) & 1)))
		return fs_latch(fs, FFTSET_E_INVALID, 0);
	if ((((uintptr_t)input_buf) | ((uintptr_t)output_buf) | ((uintptr_t)kernel_buf)) & 7)
		return fs_latch(fs, FFTSET_E_INVALID, 0);
	/* the whole batch's work must fit the fixed array */
	if ((size_t)count > FFTSET_FIXED_SCRATCH_FLOATS / nf)
		return fs_latch(fs, FFTSET_E_INVALID, 0);
	/* device buffers only: host buffers would need staging memory */
	if (!fs_is_device_ptr(input_buf) || !fs_is_device_ptr(output_buf) ||
	    (kernel_buf != NULL && !fs_is_device_ptr(kernel_buf)))
		return fs_latch(fs, FFTSET_E_INVALID, 0);
	if ((e = cudaGetDevice(&dev)) != cudaSuccess)
		return fs_cuda(fs, e);
	if (dev != fs->device || dev < 0 || dev >= FGK_FIXED_MAX_DEVICES)
		return fs_latch(fs, FFTSET_E_INVALID, 0);
	if ((e = fgk_fixed_scratch_address(dev, &scratch)) != cudaSuccess)
		return fs_cuda(fs, e);

	FS_RANGE_PUSH("fftset_fft_execute_fixed_scratch");
	rc = fgk_launch_fourstep(&fft->p4, op, output_buf, input_buf, kernel_buf, fft->kidx4, (int)fft->lanes, scratch,
	                         count, count > 1 ? in_stride : nf, count > 1 ? out_stride : nf, nf, fs->stream);
	FS_RANGE_POP();
	if (rc)
		return fs_latch(fs, FFTSET_E_CUDA, rc);
	if (fs->blocking) {
		if ((rc = fs_cuda(fs, cudaStreamSynchronize(fs->stream))) != 0)
			return rc;
		return fs_check_flag(fs);
	}
	return FFTSET_OK;
}

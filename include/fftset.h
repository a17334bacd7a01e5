/* fftset C API on GB300 (sm_103a).
 *
 * Drop-in for the reference library's public header (fftset.h of
 * templeblock/fftset): same function names, argument order and meaning,
 * buffer layouts and error behaviour, with C linkage. Each declaration cites
 * the reference declaration it replaces. Entry points after "Additions" have
 * no reference counterpart.
 *
 * Buffers may be device, managed or host memory. Device and managed buffers
 * are used in place on the fftset's CUDA stream; host buffers are staged
 * through device memory. Calls block until their results are in the output
 * buffer, like the reference's CPU calls, unless fftset_set_blocking(fc, 0)
 * is used (device buffers only; completion is then ordered on the stream).
 *
 * Threads: the execution calls (forward, inverse, get_kernel, conv, their
 * batched forms, the ragged execute, the adjoint, overlap-add) may be made
 * from several threads at once on one fftset, given distinct output buffers,
 * as the reference promises for its own (README.md:38); all of them are
 * ordered on the fftset's one stream. Creating plans and batches, changing
 * settings and the autotuners are not thread-safe, as in the reference. */
#ifndef FFTSET_H
#define FFTSET_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

struct fftset;             /* defined below so it can be placed on the stack (fftset.h:28-31) */
struct fftset_modulation;  /* opaque (fftset.h:33-35) */
struct fftset_fft;         /* opaque (fftset.h:37-39) */

/* Initialization and Cleanup
 * ------------------------------------------------------------------------ */

/* replaces fftset.h:44-47 (src/fftset.c:80-85): returns zero on success,
 * non-zero when memory (host or device) is exhausted or no CUDA device is
 * usable. */
int fftset_init(struct fftset *fc);

/* replaces fftset.h:49-52 (src/fftset.c:87-95): frees every plan, twiddle
 * table and staging buffer; all fftset_fft objects of fc become invalid. */
void fftset_destroy(struct fftset *fc);

/* Modulator Construction
 * ------------------------------------------------------------------------ */

/* replaces fftset.h:62-73: X[k] = sum_{n<N} x[n] e^{-j 2 pi n (k + 1/2) / N},
 * x real, N = 2 complex_bins reals in, complex_bins interleaved bins out. */
extern const struct fftset_modulation *FFTSET_MODULATION_FREQ_OFFSET_REAL;

/* replaces fftset.h:75-76: the plain complex DFT of complex_bins points. */
extern const struct fftset_modulation *FFTSET_MODULATION_COMPLEX;

/* replaces fftset.h:78 (src/fftset.c:97-129): finds or creates the plan for
 * (modulation, complex_bins); repeated calls return the same pointer.
 * complex_bins must be 2^a 3^b 5^c with c <= 1 and complex_bins >= 2 (the
 * sizes the reference supports, README.md:3); other sizes return NULL (the
 * reference's behaviour for them is undefined), as does memory exhaustion.
 * Not thread-safe, like the reference. */
const struct fftset_fft *fftset_create_fft(struct fftset *fc, const struct fftset_modulation *modulation,
                                           unsigned complex_bins);

/* Modulator Execution
 * ------------------------------------------------------------------------
 * All buffers hold 2*complex_bins floats and must be 8-byte aligned (the
 * reference asks for vector alignment, fftset.h:92-94). Aliasing rules are
 * the reference's (fftset.h:93-96, :103-108). work_buf is accepted for
 * compatibility; its contents are undefined after the call. */

/* replaces fftset.h:109-115 (src/fftset.c:58-67) */
void fftset_fft_forward(const struct fftset_fft *first_pass, float *output_buf, const float *input_buf,
                        float *work_buf);

/* replaces fftset.h:117-123 (src/fftset.c:69-78): unnormalised,
 * inverse(forward(x)) = complex_bins * x. */
void fftset_fft_inverse(const struct fftset_fft *first_pass, float *output_buf, const float *input_buf,
                        float *work_buf);

/* replaces fftset.h:125-130 (src/fftset.c:36-44). The output uses the
 * reference's kernel-buffer layout for the SIMD width selected with
 * fftset_set_kernel_layout (default 4), so kernels prepared here and by a CPU
 * build of the reference are interchangeable. */
void fftset_fft_conv_get_kernel(const struct fftset_fft *first_pass, float *output_buf, const float *input_buf);

/* replaces fftset.h:132-139 (src/fftset.c:46-56): FREQ_OFFSET_REAL gives
 * complex_bins times the negacyclic convolution of length 2 complex_bins;
 * COMPLEX gives complex_bins times the cyclic convolution. */
void fftset_fft_conv(const struct fftset_fft *first_pass, float *output_buf, const float *input_buf,
                     const float *kernel_buf, float *work_buf);

/* Helpful Routines
 * ------------------------------------------------------------------------ */

/* replaces fftset.h:144-151 (src/fftset.c:131-167), same result. */
unsigned fftset_recommend_conv_length(unsigned kernel_length, unsigned max_block_size);

/* Additions (no reference counterpart)
 * ------------------------------------------------------------------------ */

/* Error codes. Execution calls return void like the reference; a failure
 * (bad argument, CUDA error) is latched in the fftset and read here. */
#define FFTSET_OK               0
#define FFTSET_E_INVALID        1  /* bad argument or size */
#define FFTSET_E_NOMEM          2  /* host or device allocation failed */
#define FFTSET_E_CUDA           3  /* a CUDA call failed; see fftset_cuda_error */
#define FFTSET_E_UNSUPPORTED    4  /* plan cannot run this operation */
#define FFTSET_E_TIMEOUT        5  /* a bounded wait inside a kernel gave up (results invalid) */
int         fftset_last_error(const struct fftset *fc);      /* returns and keeps the latched code */
int         fftset_clear_error(struct fftset *fc);           /* returns the code and resets it */
int         fftset_cuda_error(const struct fftset *fc);      /* cudaError_t of the last CUDA failure */
const char *fftset_error_string(int code);

/* CUDA stream (a cudaStream_t) every call of fc is ordered on. The default
 * is a non-blocking stream fftset_init creates (fftset_own_stream); NULL is
 * CUDA's legacy default stream, as everywhere in CUDA. */
int  fftset_set_stream(struct fftset *fc, void *cuda_stream);
void *fftset_get_stream(const struct fftset *fc);
void *fftset_own_stream(const struct fftset *fc);
/* 1 (default): calls return after their results are in place. 0: calls
 * with device buffers only enqueue work on the stream.
 * Blocking single calls on device buffers of sizes up to the shared-memory
 * limit are answered, from the second such call of the same size and kernel
 * in a row, by a resident one-CTA service on a stream of its own: the call waits for the work queued on the fftset's stream,
 * hands the request over through host-mapped memory and returns when the
 * results are in place, with the same bits as the batched kernels and no
 * launch of its own. The service exits after about 50 us without requests
 * (so a device-wide synchronisation may wait that long) and when the
 * fftset is destroyed. */
int  fftset_set_blocking(struct fftset *fc, int blocking);
/* Kernel-buffer layout of fftset_fft_conv_get_kernel / fftset_fft_conv:
 * that of a reference build with SIMD width 1, 4 (default) or 8. Applies to
 * plans created afterwards. */
int  fftset_set_kernel_layout(struct fftset *fc, unsigned simd_width);
/* Kernel-buffer layout without a GPU: re_offsets[bin] (complex_bins
 * entries) receives the float offset of the real part of DFT bin `bin` in
 * the buffer fftset_fft_conv_get_kernel writes for a reference build of SIMD
 * width simd_width; the imaginary part is at re_offsets[bin] + *lanes. */
int fftset_kernel_layout(const struct fftset_modulation *modulation, unsigned complex_bins, unsigned simd_width,
                         int *re_offsets, unsigned *lanes);
/* Lane width of the kernel-buffer layout of one plan (1, 4 or 8). */
unsigned fftset_fft_kernel_lanes(const struct fftset_fft *fft);
unsigned fftset_fft_bins(const struct fftset_fft *fft);

/* Batched forms of the four execution calls: `count` independent blocks,
 * block b at input_buf + b*in_stride and output_buf + b*out_stride floats
 * (strides >= 2*complex_bins). One launch for all blocks. Return an error
 * code (also latched). Aliasing: as for the single-block calls, block by
 * block. */
int fftset_fft_forward_batch(const struct fftset_fft *fft, float *output_buf, size_t out_stride,
                             const float *input_buf, size_t in_stride, unsigned count);
int fftset_fft_inverse_batch(const struct fftset_fft *fft, float *output_buf, size_t out_stride,
                             const float *input_buf, size_t in_stride, unsigned count);
int fftset_fft_conv_batch(const struct fftset_fft *fft, float *output_buf, size_t out_stride,
                          const float *input_buf, size_t in_stride, const float *kernel_buf, unsigned count);
int fftset_fft_conv_get_kernel_batch(const struct fftset_fft *fft, float *output_buf, size_t out_stride,
                                     const float *input_buf, size_t in_stride, unsigned count);

/* Kernel variants and autotuning. Batched calls of `op` (FFTSET_OP_*) with
 * enough blocks run one of several compiled kernels for the plan's size
 * (radix order, threads per transform, transforms per CTA); variant -1 is
 * the generic kernel. fftset_fft_autotune times every candidate on `count`
 * blocks of scratch device memory and keeps the fastest (its time in
 * *best_ms when non-NULL). Not thread-safe with calls on the same plan. */
#define FFTSET_OP_FORWARD     0
#define FFTSET_OP_INVERSE     1
#define FFTSET_OP_GET_KERNEL  2
#define FFTSET_OP_CONV        3
#define FFTSET_OP_CORR        4
int fftset_fft_variants(const struct fftset_fft *fft);
int fftset_fft_variant(const struct fftset_fft *fft, int op);
int fftset_fft_set_variant(const struct fftset_fft *fft, int op, int variant);
int fftset_fft_autotune(const struct fftset_fft *fft, int op, unsigned count, float *best_ms);

/* Ragged batches: n transforms of different sizes (bins[i] complex bins,
 * same modulation, op FFTSET_OP_FORWARD or FFTSET_OP_INVERSE), item i read
 * from input_base + in_offsets[i] and written to output_base + out_offsets[i]
 * (offsets in floats, even; device buffers). All sizes share the fftset's
 * plans and twiddles. Every item runs in one persistent launch of tile tasks
 * (items up to 4096 bins whole; up to 65536 bins as the column and row tiles
 * of their four-step split, through a scratch buffer that L2 serves; larger
 * ones as the three passes of a three-level split), captured
 * in a CUDA graph on the first execute (again when the base pointers change)
 * and replayed. fftset_ragged_execute reports FFTSET_E_TIMEOUT if a tile's
 * bounded wait gave up. */
struct fftset_ragged;
struct fftset_ragged *fftset_ragged_create(struct fftset *fc, const struct fftset_modulation *modulation, int op,
                                           unsigned n, const unsigned *bins, const size_t *in_offsets,
                                           const size_t *out_offsets);
int      fftset_ragged_execute(struct fftset_ragged *rb, float *output_base, const float *input_base);
int      fftset_ragged_set_graph(struct fftset_ragged *rb, int enable);
double   fftset_ragged_bytes(const struct fftset_ragged *rb);  /* one read + one write of every item */
unsigned fftset_ragged_persistent_items(const struct fftset_ragged *rb);
/* Per-size schedule autotuner of the task kernel: for every distinct size of
 * rb up to 65536 bins, times candidate schedules on scratch buffers (whole
 * items: radix order, as planned or reversed, x threads per item, which sets
 * the items per task; two-level items: lanes per column / row tile) and keeps
 * the fastest on the size's plan (later batches of the same fftset reuse
 * it), then rebuilds rb's task list. */
int      fftset_ragged_autotune(struct fftset_ragged *rb);
/* Frees rb. A batch uses its fftset's plans, which fftset_destroy frees
 * (like the reference's plans, fftset.h:49-52): destroy every batch first. */
void     fftset_ragged_destroy(struct fftset_ragged *rb);

/* Adjoint of fftset_fft_conv (the reference has only the forward,
 * src/fftset_vec.c:1161-1220). For count blocks y_b = conv(x_b, K) with
 * K = fftset_fft_conv_get_kernel(h) and upstream gradients g_b (grad_output,
 * strides in floats like the batched calls):
 *   grad_input_b = conv of g_b with the conjugated kernel spectrum, i.e.
 *                  complex_bins times the negacyclic (FREQ_OFFSET_REAL) or
 *                  cyclic (COMPLEX) cross-correlation of g_b with h;
 *   grad_taps    = sum over b of complex_bins times the cross-correlation of
 *                  g_b with x_b: the gradient with respect to the 2L taps h.
 * Either output may be NULL. Device buffers only. For FREQ_OFFSET_REAL these
 * are the gradients of the real loss sum_b <g_b, y_b>. */
int fftset_fft_conv_adjoint_batch(const struct fftset_fft *fft, float *grad_input, size_t gi_stride,
                                  float *grad_taps, const float *grad_output, size_t go_stride,
                                  const float *input_buf, size_t in_stride, const float *kernel_buf, unsigned count);

/* Overlap-add block convolution (the reference leaves this loop to its
 * callers; its README.md:3 use case, block and transform lengths as from
 * fftset_recommend_conv_length, src/fftset.c:145-167): the linear
 * convolution of `samples` input samples (reals for FREQ_OFFSET_REAL,
 * interleaved complex for COMPLEX) with a kernel of kernel_length taps whose
 * spectrum kernel_buf comes from fftset_fft_conv_get_kernel of the taps
 * zero-padded to the plan's length N (2 complex_bins reals, or complex_bins
 * complex points). The input is cut into blocks of block_length samples (0:
 * N - kernel_length + 1, the most that does not wrap), each zero-padded to N;
 * one batched convolution; the results are overlap-added into output_buf,
 * samples + kernel_length - 1 samples, complex_bins times the linear
 * convolution (the scale of fftset_fft_conv). Device buffers. Where the
 * plan has a compiled fused kernel (FREQ_OFFSET_REAL, 1536 bins) and
 * kernel_length - 1 <= block_length, one launch reads the blocks from the
 * signal and adds their results into output_buf (used when output_buf does
 * not overlap input_buf); otherwise the blocks go through 2 x blocks x N
 * samples of the fftset's staging memory. */
int fftset_fft_conv_overlap_add(const struct fftset_fft *fft, float *output_buf, const float *input_buf,
                                size_t samples, const float *kernel_buf, unsigned kernel_length,
                                unsigned block_length);

/* No counterpart in the reference (its planner runs inside
 * fftset_create_fft, src/fftset_vec.c:993-1152, and keeps nothing across
 * processes). Persistent autotune results: fftset_tuning_save writes, for
 * every plan of the fftset, the compiled kernel chosen per operation
 * (fftset_fft_autotune / fftset_fft_set_variant) and the task schedule
 * chosen by fftset_ragged_autotune, as text, with the device model it was
 * measured on; fftset_tuning_load creates those plans in this fftset and
 * applies the choices. Returns FFTSET_OK; FFTSET_E_UNSUPPORTED (nothing
 * applied) for a file from another device model; FFTSET_E_INVALID for an
 * unreadable or malformed file (records before the bad one stay applied). */
int fftset_tuning_save(struct fftset *fs, const char *path);
int fftset_tuning_load(struct fftset *fs, const char *path);

/* No counterpart in the reference. A batched call (op FFTSET_OP_*, the
 * arguments of fftset_fft_*_batch) that allocates nothing, for callers that
 * must not call cudaMalloc while they run: a real-time audio callback with a
 * deadline every few milliseconds cannot block in the driver's allocator,
 * and some hosts fix their device-memory budget up front. It is for sizes
 * beyond the shared-memory limit, whose four-step passes need a work buffer
 * of 2 * complex_bins floats per block; the regular calls grow the fftset's
 * own work buffer with cudaMalloc, this one uses a fixed device array of
 * FFTSET_FIXED_SCRATCH_FLOATS floats (32 MiB, held by every GPU that loads
 * the library until the process exits).
 * - count * 2 * complex_bins above FFTSET_FIXED_SCRATCH_FLOATS returns
 *   FFTSET_E_INVALID; sizes that fit shared memory need no scratch and
 *   return FFTSET_E_UNSUPPORTED (their fftset_fft_*_batch calls serve them).
 * - Device buffers only; the fftset's device must be current.
 * - The first call on a device looks up the array's device address
 *   (cudaGetSymbolAddress); make that first call before any stream capture.
 * - All calls in the process share the one array per device: calls that
 *   overlap on the GPU (other streams, other fftsets, other threads) race
 *   on it and give wrong results; serialise them. Nothing in it needs to
 *   start at zero: the first pass writes all of it before the second reads. */
#define FFTSET_FIXED_SCRATCH_FLOATS (8u << 20)
int fftset_fft_execute_fixed_scratch(const struct fftset_fft *fft, int op, float *output_buf, size_t out_stride,
                                     const float *input_buf, size_t in_stride, const float *kernel_buf,
                                     unsigned count);

/* Private Parts
 * ---------------------------------------------------------------------------
 * Don't touch them. */
struct fftset {
	void *impl;
	void *reserved[7];
};

#ifdef __cplusplus
}
#endif

#endif /* FFTSET_H */

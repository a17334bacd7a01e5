/* Internal structures of the host layer, shared by fftset_host.c and
 * fftset_ragged.c. Not part of the public interface. */
#ifndef FFTSET_INTERNAL_H
#define FFTSET_INTERNAL_H

#include <pthread.h>
#include <stdint.h>
#include <cuda_runtime_api.h>

#include "fftset.h"
#include "fgk.h"

struct fftset_modulation {
	int         freq_offset_real;
	const char *name;
};

struct fs_impl;

#define FS_MAX_VAR 16

struct fftset_fft {
	unsigned                        lfft;
	const struct fftset_modulation *modulator;
	struct fftset_fft              *next;
	struct fs_impl                 *fs;
	unsigned                        lanes; /* kernel-buffer lane width */
	fgk_plan                        rp;    /* generic resident plan (device pointers inside) */
	int                             nvar;  /* compile-time kernel variants for this size */
	fgk_plan                        vp[FS_MAX_VAR]; /* their plans (chain of the variant) */
	uint32_t                        vops[FS_MAX_VAR]; /* ops each variant implements (1 << op) */
	uint32_t                        vtma[FS_MAX_VAR]; /* 1: the variant reads its input with bulk copies */
	int                             sel[FGK_OP_COUNT]; /* chosen variant per op, -1 = generic */
	int                             fourstep; /* 1: sizes beyond shared memory, two HBM passes */
	fgk_plan4                       p4;    /* four-step plan (when dmem4 != NULL) */
	void                           *dmem4; /* its device tables */
	const int32_t                  *kidx4; /* kernel-layout table in dmem4 */
	fgk_plan3                       p3;    /* three-level plan (when dmem3 != NULL) */
	void                           *dmem3; /* its device tables */
	struct fftset_ragged           *tasks; /* cached task list of the plain calls (fftset_ragged.c) */
	/* task-kernel schedule picked by fftset_ragged_autotune (rg_tuned):
	 * whole items run rg_plan's chain (its tables in rg_dmem, NULL for the
	 * default chain) with rg_tg threads each; two-level items use rg_ls1 /
	 * rg_ls2 lanes per COLS / ROWS tile */
	int                             rg_tuned;
	fgk_plan                        rg_plan;
	void                           *rg_dmem;
	uint32_t                        rg_tg, rg_ls1, rg_ls2;
	unsigned                        tasks_count;
	size_t                          tasks_in_stride, tasks_out_stride;
	void                           *dmem;  /* one device block for all tables */
};

#define FS_NSTAGE 5 /* staging buffers: input, output, kernel, four-step work, adjoint scratch */
#define FS_PIPE   3 /* streams of the host-buffer chunk pipeline */

struct fs_impl {
	cudaStream_t       stream;
	cudaStream_t       own_stream;
	int                blocking;
	unsigned           layout_vw;
	int                err;
	int                cuda_err;
	int                device;
	unsigned           max_smem;
	int                num_sms;
	struct fftset_fft *first;
	pthread_mutex_t    lock;
	int               *host_flag; /* mapped pinned int: kernels report a failed bounded wait */
	int               *dev_flag;
	void              *stage[FS_NSTAGE];
	size_t             stage_bytes[FS_NSTAGE];
	cudaStream_t       pipe[FS_PIPE]; /* host-buffer chunk pipeline (fs_exec) */
	cudaEvent_t        pipe_ev;
};


/* helpers implemented in fftset_host.c */
int  fs_latch(struct fs_impl *fs, int code, int cuda_err);
int  fs_cuda(struct fs_impl *fs, cudaError_t e);
int  fs_is_device_ptr(const void *ptr);
int  fs_check_flag(struct fs_impl *fs);
/* four-step tables for a plan (built on demand for resident-size plans too) */
int  fs_ensure_fourstep(struct fs_impl *fs, struct fftset_fft *f);
/* three-level tables for a plan (sizes beyond 65536 bins), on demand */
int  fs_ensure_threestep(struct fs_impl *fs, struct fftset_fft *f);
/* find-or-create a plan (fftset_create_fft without the public wrapper) */
struct fftset_fft *fs_create_plan(struct fs_impl *fs, const struct fftset_modulation *modulation, unsigned bins);
/* forward / inverse of `count` device blocks of a four-step plan as one task
 * launch (fftset_ragged.c); returns 0, a negative FFTSET_E_* code or a
 * positive cudaError_t; FFTSET_E_UNSUPPORTED when the size has no tile split */
int  fs_tasks_batch(struct fftset_fft *f, int op, float *out, size_t out_stride, const float *in, size_t in_stride,
                    unsigned count, cudaStream_t stream);
struct fftset_ragged;
void fsr_free(struct fftset_ragged *rb);
/* applies a saved task-kernel schedule to a plan (fftset_ragged.c) */
int  fsr_apply_schedule(struct fs_impl *fs, struct fftset_fft *f, const uint32_t *rad, uint32_t n, uint32_t tg,
                        uint32_t ls1, uint32_t ls2);
struct fs_impl *fs_impl_of(struct fftset *fc);
/* grows staging slot `slot` to at least `bytes` (cudaMalloc) */
int  fs_stage_reserve(struct fs_impl *fs, int slot, size_t bytes);
/* runs op on `count` device-resident blocks on the fftset's stream;
 * returns 0, a negative FFTSET_E_* code or a positive cudaError_t */
int  fs_launch(const struct fftset_fft *f, int op, float *out, const float *in, const float *kern, unsigned count,
               size_t in_stride, size_t out_stride);

#endif

/* Internal structures of the host layer, shared by fftset_host.c and
 * fftset_ragged.c. Not part of the public interface. */
#ifndef FFTSET_INTERNAL_H
#define FFTSET_INTERNAL_H

#include <pthread.h>
#include <stdint.h>
#include <cuda_runtime_api.h>

#include "fftset.h"
#include "fgk.h"

/* NVTX ranges (header-only NVTX 3; inert unless a profiler is attached)
 * around every public call, named after the call */
#include <nvtx3/nvToolsExt.h>
#define FS_RANGE_PUSH(name) nvtxRangePushA(name)
#define FS_RANGE_POP()      nvtxRangePop()

struct fftset_modulation {
	int         freq_offset_real;
	const char *name;
};

struct fs_impl;
struct fftset_ragged;

#define FS_MAX_VAR 16
#define FS_TASK_LISTS 4 /* cached task lists per plan (shapes of the plain calls) */

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
	/* task lists of the plain calls of this plan (fftset_ragged.c), one per
	 * (count, strides) shape seen, least recently used replaced first; the
	 * direction is a launch argument, so a COMPLEX list serves both (op -1;
	 * FREQ_OFFSET_REAL lists are ordered for one direction, op). Read and
	 * written with fs->lock held. */
	struct fs_tasklist {
		struct fftset_ragged *rb;
		int                   op;
		unsigned              count;
		size_t                in_stride, out_stride;
		uint64_t              used;
	} tl[FS_TASK_LISTS];
	uint64_t                        tl_clock;
	/* task-kernel schedule picked by fftset_ragged_autotune (rg_tuned):
	 * whole items run rg_plan's chain (its tables in rg_dmem, NULL for the
	 * default chain) with rg_tg threads each; two-level items use rg_ls1 /
	 * rg_ls2 lanes per COLS / ROWS tile */
	int                             rg_tuned;
	fgk_plan                        rg_plan;
	void                           *rg_dmem;
	uint32_t                        rg_tg, rg_ls1, rg_ls2;
	void                           *dmem;  /* one device block for all tables */
};

#define FS_NSTAGE 5 /* staging buffers: input, output, kernel, four-step work, adjoint scratch */
#define FS_PIPE   3 /* streams of the host-buffer chunk pipeline */
/* doorbell polls (about 0.8 us each over NVLink-C2C) before an idle call
 * service exits: a caller that waits longer than this between blocking
 * calls pays one launch on its next call */
#define FS_SERVE_IDLE_POLLS 64

/* The call service (fgk.h, fgk_launch_static_serve): one resident CTA that
 * runs blocking single calls of a compiled variant without a launch each. */
struct fs_serve {
	void                  *map;   /* pinned, mapped page: the words and the request */
	volatile uint64_t     *bell, *reply, *state;
	fgk_serve_req         *req;
	fgk_serve_words        dev;   /* the same, as device addresses */
	cudaStream_t           stream;
	const struct fftset_fft *f;   /* what the live launch serves (f, v) */
	int                    v;
	uint64_t               seq;   /* last request sequence number issued */
	uint64_t               id;    /* id of the latest launch (0: none yet) */
	const struct fftset_fft *last_f; /* the previous eligible call's (f, v): a */
	int                    last_v;   /* launch is only worth it on a repeat */
	uint32_t               idle_polls; /* doorbell polls before an idle CTA exits; 0: off */
	int                    broken;     /* a failure turned the service off */
	unsigned long long     served;     /* requests answered */
};

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
	/* recursive: held around everything that touches state shared by the
	 * execution calls of this fftset (staging buffers, the task lists and
	 * on-demand tables of plans beyond the shared-memory limit, the call
	 * service's request page), so that those calls are thread-safe like the
	 * reference's (README.md:38); batched and non-blocking resident-size
	 * calls share nothing and do not take it */
	pthread_mutex_t    lock;
	int               *host_flag; /* mapped pinned int: kernels report a failed bounded wait */
	uint32_t           spin_limit; /* polls of a task kernel's bounded waits (fgk_launch_tasks) */
	int                task_shape; /* ragged task CTAs: -1 by the list, else enum fgk_task_shape */
	uint32_t           group_dist; /* three-level lists: slots from A to B tiles of a group; 0: all A tiles first */
	int               *dev_flag;
	void              *stage[FS_NSTAGE];
	size_t             stage_bytes[FS_NSTAGE];
	cudaStream_t       pipe[FS_PIPE]; /* host-buffer chunk pipeline (fs_exec) */
	cudaEvent_t        pipe_ev;
	struct fs_serve    srv;
};


/* helpers implemented in fftset_host.c */
int  fs_latch(struct fs_impl *fs, int code, int cuda_err);
int  fs_cuda(struct fs_impl *fs, cudaError_t e);
int  fs_is_device_ptr(const void *ptr);
int  fs_check_flag(struct fs_impl *fs);
/* the call service's live launch, if any, exits (fftset_host.c) */
void fs_serve_stop(struct fs_impl *fs);
/* four-step tables for a plan (built on demand for resident-size plans too) */
int  fs_ensure_fourstep(struct fs_impl *fs, struct fftset_fft *f);
/* three-level tables for a plan (sizes beyond 65536 bins), on demand */
int  fs_ensure_threestep(struct fs_impl *fs, struct fftset_fft *f);
/* find-or-create a plan (fftset_create_fft without the public wrapper) */
struct fftset_fft *fs_create_plan(struct fs_impl *fs, const struct fftset_modulation *modulation, unsigned bins);
/* FFTSET_E_* code of the calling thread's last fs_create_plan that returned NULL */
int  fs_plan_error(void);
/* forward / inverse of `count` device blocks of a four-step plan as one task
 * launch (fftset_ragged.c); returns 0, a negative FFTSET_E_* code or a
 * positive cudaError_t; FFTSET_E_UNSUPPORTED when the size has no tile split.
 * prod (forward only, may be NULL): a spectrum product fused into the final
 * stores. Called with fs->lock held. */
int  fs_tasks_batch(struct fftset_fft *f, int op, float *out, size_t out_stride, const float *in, size_t in_stride,
                    unsigned count, cudaStream_t stream, const fgk_product *prod);
void fsr_free(struct fftset_ragged *rb);
/* applies a saved task-kernel schedule to a plan (fftset_ragged.c) */
int  fsr_apply_schedule(struct fs_impl *fs, struct fftset_fft *f, const uint32_t *rad, uint32_t n, uint32_t tg,
                        uint32_t ls1, uint32_t ls2);
struct fs_impl *fs_impl_of(struct fftset *fc);
/* grows staging slot `slot` to at least `bytes` (cudaMalloc); called with
 * fs->lock held */
int  fs_stage_reserve(struct fs_impl *fs, int slot, size_t bytes);
/* runs op on `count` device-resident blocks on the fftset's stream;
 * returns 0, a negative FFTSET_E_* code or a positive cudaError_t. Takes
 * fs->lock itself for plans beyond the shared-memory limit. */
int  fs_launch(const struct fftset_fft *f, int op, float *out, const float *in, const float *kern, unsigned count,
               size_t in_stride, size_t out_stride);


/* Allocation wrappers (fftset_alloc.c): the host layer's allocations are
 * counted, and a test can make one of them fail. */
void       *fs_malloc(size_t n);
void       *fs_calloc(size_t n, size_t m);
void        fs_free(void *p);
cudaError_t fs_cuda_malloc(void **p, size_t n);
cudaError_t fs_cuda_free(void *p);
cudaError_t fs_cuda_host_alloc(void **p, size_t n, unsigned flags);
cudaError_t fs_cuda_free_host(void *p);
/* Test hooks, exported but not part of the public header: the nth host or
 * device allocation from now fails (0: none; returns the previous setting),
 * and the numbers of host and device allocations still held. */
long fftset__test_fail_allocation(long nth);
void fftset__test_live_allocations(long *host, long *device);
/* Test hooks of the bounded waits: the polls of the task kernel's waits
 * (launches made afterwards), and a ragged batch without its tasks of one
 * kind (the tasks that wait on them then time out). */
int  fftset__test_set_spin_limit(struct fftset *fc, unsigned polls);
/* the call service's idle doorbell polls (0 turns it off; the default is
 * FS_SERVE_IDLE_POLLS) and the number of requests it has served */
int  fftset__test_set_call_service(struct fftset *fc, unsigned idle_polls);
unsigned long long fftset__test_served_calls(struct fftset *fc);
/* CTA shape of the task lists of later ragged creates: -1 chosen by the
 * list (three-level items: single-buffer when every chain has two stages
 * at most, else wide; otherwise narrow), or an enum fgk_task_shape (single
 * makes creates of lists with longer chains fail) */
int  fftset__test_set_task_shape(struct fftset *fc, int shape);
/* slots between the A and the B tiles of an n3 group in the three-level
 * lists of later ragged creates (0: the default, every A tile first) */
int  fftset__test_set_group_distance(struct fftset *fc, unsigned slots);
int  fftset__test_ragged_drop_kind(struct fftset_ragged *rb, int kind);
/* the task order of one three-level item L1 x L2 x L3 (fftset_ragged.c,
 * fsr_list_huge), written to out (at most cap tasks; returns the count,
 * 0 when cap is too small); no GPU is involved */
uint32_t fftset__test_list_huge(uint32_t L1, uint32_t L2, uint32_t L3, int zip_in, int zip_out, uint32_t grid,
                                uint32_t group_dist, fgk_task *out, uint32_t cap);
#if !defined(FS_ALLOC_IMPL) && !defined(__cplusplus)
#include <stdlib.h>
#define malloc(n)                 fs_malloc(n)
#define calloc(n, m)              fs_calloc((n), (m))
#define free(p)                   fs_free(p)
#define cudaMalloc(p, n)          fs_cuda_malloc((void **)(p), (n))
#define cudaFree(p)               fs_cuda_free(p)
#define cudaHostAlloc(p, n, f)    fs_cuda_host_alloc((void **)(p), (n), (f))
#define cudaFreeHost(p)           fs_cuda_free_host(p)
#endif

#endif

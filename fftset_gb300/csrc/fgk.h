/* Internal C ABI between the C host layer (fftset_host.c) and the CUDA
 * kernels (fgk_*.cu). Plain C structs of sizes, offsets and device pointers;
 * no torch and no C++ types. Not part of the public interface. */
#ifndef FGK_H
#define FGK_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FGK_MAX_STAGES 24

/* One Stockham stage of a resident transform of length L.
 * Butterfly j (0 <= j < L/radix) reads x[j + p L/radix], multiplies input p
 * by w_{ns*radix}^{p (j mod ns)}, runs DFT_radix and writes output q to
 * (j - j mod ns) radix + (j mod ns) + q ns. After all stages the sequence is
 * the natural-order DFT. */
typedef struct fgk_stage {
	uint32_t radix;
	uint32_t ns;      /* product of the radices of the stages before */
	uint32_t tw_off;  /* float2 offset of this stage's twiddles: (radix-1)*ns entries, [k][p-1] */
	uint32_t nb;      /* butterflies per thread (ceil(L/radix / threads)) */
} fgk_stage;

typedef struct fgk_chain {
	uint32_t  nstages;
	uint32_t  reserved;
	uint64_t  code; /* nstages in bits 0-3, radix of stage s minus 1 in bits 4s+4 .. 4s+7 (chains
	                   of at most 15 stages; 0 otherwise): the whole chain in one load */
	fgk_stage st[FGK_MAX_STAGES];
} fgk_chain;

enum fgk_modulation { FGK_MOD_COMPLEX = 0, FGK_MOD_FREQOFF = 1 };

enum fgk_op {
	FGK_OP_FORWARD = 0,
	FGK_OP_INVERSE = 1,
	FGK_OP_KERNEL  = 2,   /* fftset_fft_conv_get_kernel */
	FGK_OP_CONV    = 3,   /* fftset_fft_conv */
	FGK_OP_CORR    = 4,   /* convolution with the conjugated kernel spectrum (adjoint w.r.t. input) */
	FGK_OP_COUNT
};

/* Device-side plan of one resident (shared-memory) transform. */
typedef struct fgk_plan {
	uint32_t  L;           /* complex bins */
	uint32_t  modulation;  /* enum fgk_modulation */
	uint32_t  threads;     /* threads per transform */
	uint32_t  per_cta;     /* transforms per CTA */
	uint32_t  smem_stride; /* float2 slots of shared memory per transform */
	uint32_t  kvw;         /* kernel-buffer lane width: imag = real offset + kvw */
	uint32_t  pad;         /* 1: shared-memory slot of element i is i + i/16; 0: i */
	uint32_t  emax;        /* register budget (complex elements per thread per stage): 16 or 32 */
	fgk_chain fwd;         /* natural in -> natural out */
	fgk_chain inv;         /* fwd's radices reversed: the chain run after the spectrum product */
	const void    *tw;     /* device float2 twiddles of both chains */
	const void    *modtw;  /* device float2[L] e^{-j pi i/(2L)} (FREQOFF only) */
	const int32_t *kidx;   /* device int32[L]: kernel-buffer float offset of bin m's real part */
	const struct fgk_plan *dev; /* device copy of this struct (kernels index its chains) */
} fgk_plan;

/* Plan of a four-step transform L = L1 * L2 (fgk_fourstep.cu). Pass 1 runs
 * L2 column DFTs of length L1, pass 2 L1 row DFTs of length L2; a CTA holds
 * 1 << lshift transforms lane-interleaved (mirrored passes need >= 2). */
typedef struct fgk_plan4 {
	uint32_t  L1, L2, modulation;
	uint32_t  lshift1, lshift2;
	uint32_t  threads1, threads2;
	uint32_t  slots1, slots2;   /* shared float2 slots of one tile buffer */
	uint32_t  emax1, emax2;     /* 0: ping-pong tile (two buffers, one butterfly per
	                             * thread at a time); else in place, up to emax
	                             * points per thread in registers (one buffer) */
	fgk_chain c1, c2;
	const void *tw1, *tw2;      /* chain twiddles */
	uint32_t  tshift;           /* w_L^m = thi[m >> tshift] * tlo[m & ((1 << tshift) - 1)] */
	const void *thi, *tlo;
	const void *m1, *m2;        /* e^{-j pi n1/(2 L1)}, e^{-j pi n2/(2L)}: input modulation */
	const void *n1, *n2;        /* e^{-j pi k1/(2L)}, e^{-j pi k2/(2 L2)}: output modulation */
	uint32_t    nq;             /* R L2, R the last radix of c1 */
	const void *tq;             /* w_{R L2}^m, m < nq */
	const struct fgk_plan4 *dev;
} fgk_plan4;

/* Plan of a three-level transform L = L1 L2 L3 (each <= 256, L1 >= 16) run
 * as tile tasks (fgk_tasks.cuh): n = (n1 L2 + n2) L3 + n3,
 * k = k1 + L1 (k2 + L2 k3).
 *   pass A: DFT_L1 over n1, times w_{L1 L2}^{n2 k1}, into A[k1][n2 L3 + n3];
 *   pass B: DFT_L2 over n2, times w_L^{n3 (k1 + L1 k2)}, into
 *           B[(k2 L3 + n3) L1 + k1];
 *   pass C: DFT_L3 over n3 into X[k1 + L1 k2 + L1 L2 k3]. */
typedef struct fgk_plan3 {
	uint32_t    L1, L2, L3, modulation;
	uint32_t    nq1, nq2;        /* R1 L2 and R2 L3, R1 / R2 the last radices of c1 / c2 */
	fgk_chain   c1, c2, c3;      /* the passes' chains (their twiddles are computed in the kernel) */
	const void *tq1, *tq2;       /* w_{R1 L2}^m, w_{R2 L3}^m */
	const void *ma, *mb, *mc;    /* e^{-j pi n1/(2 L1)}, e^{-j pi n2/(2 L1 L2)}, e^{-j pi n3/(2L)} */
	const void *oa, *ob, *oc;    /* e^{-j pi k1/(2L)}, e^{-j pi k2/(2 L2 L3)}, e^{-j pi k3/(2 L3)} */
	const struct fgk_plan3 *dev;
} fgk_plan3;

/* Ragged batches: item offsets in floats from the batch's base pointers. */
typedef struct fgk_rg_item {
	uint64_t in_off, out_off;
} fgk_rg_item;

/* Ragged batches as tasks of one persistent launch (fgk_tasks.cuh). Every
 * task is a tile of at most fgk_tasks_points() points:
 *   SMALL  n same-size items (whole transforms, tg threads each);
 *   COLS   lanes of columns of a big item's four-step split L = L1 L2 (DFTs
 *          of length L1 from the input, twiddled, into the item's scratch);
 *   ROWS   lanes of rows of that scratch (DFTs of length L2 into the
 *          output); they start once every COLS tile of the item is done. */

enum fgk_task_kind {
	FGK_TASK_SMALL = 0,
	FGK_TASK_COLS = 1,
	FGK_TASK_ROWS = 2,
	FGK_TASK_PA = 3, /* three-level passes (fgk_plan3) */
	FGK_TASK_PB = 4,
	FGK_TASK_PC = 5
};

typedef struct fgk_task {
	uint32_t kind;
	uint32_t ref;  /* SMALL: plan index; COLS/ROWS: big-item index */
	uint32_t a;    /* SMALL: first item; COLS/ROWS: tile index */
	uint32_t b;    /* SMALL: items | threads per item << 16 */
} fgk_task;

/* A spectrum product fused into the final stores of a forward task launch
 * (ROWS and C tiles): W[m] times spec[m], the kernel spectrum in natural bin
 * order (fgk_launch_spectrum_natural); spec == NULL: no product. The
 * convolution of sizes beyond the shared-memory limit is this forward
 * followed by the inverse task launch. */
typedef struct fgk_product {
	const void *spec; /* float2[L] */
} fgk_product;

/* spec[m] = bin m of a kernel buffer (re at kern[kidx[m]], im kvw floats
 * later), conjugated when conj is set: the natural-order copy the product
 * reads with one coalesced load per bin */
int fgk_launch_spectrum_natural(const float *kern, const int32_t *kidx, int kvw, uint32_t L, int conj, void *spec,
                                void *stream);

/* A three-level item: passes A, B, C through two scratch areas. When 16
 * divides L3 the A and B tiles fall into ngrp = L3/16 groups by n3 (A tile
 * t: t % ngrp; B tile: its n3 / 16) and a B tile waits for the L2 A tiles
 * of its group only; otherwise ngrp = 1 and B tiles wait for every A tile.
 * A C tile (16 k1) waits for the B tiles of its 16 k1 only. The item's
 * counters: hcounters[cnt + u], u < ngrp, A tiles done in n3 group u;
 * hcounters[cnt + ngrp + g], g < nc1, B tiles done in k1 group g. */
typedef struct fgk_huge {
	const struct fgk_plan3 *p3;             /* device copy of the item's plan */
	uint32_t                L1, L2, L3, ngrp;
	uint64_t                code1, code2, code3; /* the passes' chains (fgk_chain.code) */
	uint64_t                in_off, out_off; /* floats from the batch's base pointers */
	uint64_t                sa, sb;          /* float2 offsets of its A and B scratch */
	uint32_t                na, nb;          /* A tiles, B tiles */
	uint32_t                nb3, nc1;        /* B tiles per k1 group (ceil(L3/4)), C tiles per k2 (ceil(L1/16)) */
	uint32_t                cnt, reserved;   /* first counter of the item */
} fgk_huge;

typedef struct fgk_big {
	const struct fgk_plan4 *p4;            /* device copy of the item's four-step plan */
	uint32_t                L1, L2;
	uint64_t                code1, code2;    /* the COLS / ROWS chains (fgk_chain.code) */
	uint64_t                in_off, out_off; /* floats from the batch's base pointers */
	uint64_t                scratch_off;     /* float2 offset of the item's L1 x L2 scratch */
	uint32_t                ncols;           /* COLS tiles */
	uint32_t                ls1, ls2;        /* log2 of the lanes of a COLS / ROWS tile */
	uint32_t                nrows;           /* ROWS tiles */
} fgk_big;

/* Every kernel launch of the library is counted (fgk_resident.cu): the
 * counter lets a profile run map the library's launches to its cases and a
 * benchmark report how many of its own kernels ran. */
void fgk_count_launch(void);
unsigned long long fftset__launch_count(void);

/* Host-side planning helpers implemented in fgk_plan.c */
int  fgk_plan_chain(uint32_t L, uint32_t *radices, uint32_t *nstages);
/* forced_radices: NULL, or the chain a static kernel was compiled for */
int  fgk_plan_resident(fgk_plan *p, uint32_t L, uint32_t modulation, uint32_t max_smem_bytes,
                       const uint32_t *forced_radices, uint32_t forced_n);
/* Number of float2 twiddles both chains of p need; fills them when tw != NULL. */
size_t fgk_plan_twiddles(fgk_plan *p, void *tw_host_float2);
/* Four-step planning: fills sizes, lanes, threads and chains (not the
 * pointers). Returns -1 when L has no two-factor split the kernels take. */
int    fgk_plan_fourstep(fgk_plan4 *p, uint32_t L, uint32_t modulation, uint32_t max_smem_bytes);
/* Three-level split of L (each factor <= 256, L1 >= 16, most balanced);
 * fills sizes and chains. Returns -1 when L has none. */
int    fgk_plan_threestep(fgk_plan3 *p, uint32_t L, uint32_t modulation);
/* twiddles of one chain (the chain's tw_off fields are set) */
size_t fgk_chain_twiddles(fgk_chain *c, void *tw_host_float2);

/* Launchers implemented in fgk_kernels.cu. All return 0 or a cudaError_t. */
int fgk_launch_resident(const fgk_plan *p, int op, float *out, const float *in, const float *kern,
                        uint32_t count, size_t in_stride, size_t out_stride, void *stream);
uint32_t fgk_max_resident_L(void);
/* two launches per DFT (pass 1, pass 2; convolution: two DFTs); work: count
 * transforms of 2L floats at work_stride; kern/kidx/kvw: the kernel buffer and
 * its layout table (get_kernel, conv) */
int fgk_launch_fourstep(const fgk_plan4 *p, int op, float *out, const float *in, const float *kern,
                        const int32_t *kidx, int kvw, float *work, uint32_t count, size_t in_stride,
                        size_t out_stride, size_t work_stride, void *stream);
/* the task launch: counters_dev holds 1 + nbig + nhcount ints (claim
 * counter, the finished COLS tiles of each big item, the three-level items'
 * counters, fgk_huge.cnt) and is reset by the launcher;
 * scratch_dev holds the big items' L1 x L2 intermediates; err_flag is set
 * when a bounded wait gives up, after spin_limit polls (about 256 ns
 * apart); shape selects the CTA shape the list was planned for (enum
 * fgk_task_shape) */
enum fgk_task_shape {
	FGK_SHAPE_NARROW = 0, /* 128 threads, two tile buffers, three CTAs per SM */
	FGK_SHAPE_WIDE = 1,   /* 256 threads, two buffers, three CTAs per SM */
	FGK_SHAPE_SINGLE = 2  /* 128 threads, one buffer, six CTAs per SM: chains of two stages at most */
};
int    fgk_launch_tasks(const fgk_task *tasks_dev, uint32_t ntasks, const fgk_plan *plans_dev,
                        const fgk_rg_item *items_dev, const fgk_big *bigs_dev, uint32_t nbig,
                        const fgk_huge *huges_dev, uint32_t nhcount, int *counters_dev,
                        float *scratch_dev, int op, int modulation, const float *in_base, float *out_base,
                        int num_sms, int shape, int *err_flag, uint32_t spin_limit, fgk_product prod, void *stream);
int    fgk_tasks_grid(int num_sms, int shape);
int    fgk_tasks_threads(int shape);
/* points of a tile (items up to this size run whole) and the shared-memory
 * slots of one of its two buffers */
int    fgk_tasks_points(void);
int    fgk_tasks_slots(void);

/* Static (compile-time) kernels, fgk_static*.cu: `fgk_static_count`
 * variants exist for (modulation, L); fgk_static_info describes variant v
 * (chain, threads per transform, transforms per CTA, compiled ops as a bit
 * mask of 1 << fgk_op). The plan passed to fgk_launch_static must have been
 * made with that variant's chain. fgk_launch_static returns -1 when the
 * variant does not implement op. */
int fgk_static_count(uint32_t modulation, uint32_t L);
int fgk_static_info(uint32_t modulation, uint32_t L, int v, uint32_t *radices, uint32_t *n, uint32_t *threads,
                    uint32_t *groups, uint32_t *opmask, uint32_t *tma);
/* err_flag: device-visible int set to 1 when a bounded wait inside the
 * kernel gives up (may be NULL) */
int fgk_launch_static(const fgk_plan *p, int v, int op, float *out, const float *in, const float *kern,
                      uint32_t count, size_t in_stride, size_t out_stride, void *stream, int num_sms, int *err_flag);

/* The taps-gradient kernel of the adjoint (fgk_static.cuh,
 * static_kernel_kgrad): the first compiled variant of (modulation, L) that
 * has one, or -1; the launch writes *rows <= max_rows partial rows of L
 * float2, P[m] = sum over its blocks of W_g[m] conj(W_x[m]) (natural-order
 * spectra before the FREQ_OFFSET_REAL split). The plan must be the
 * variant's (its chain's twiddles). Returns -1 when the variant has none. */
int fgk_static_kgrad_variant(uint32_t modulation, uint32_t L);
int fgk_launch_static_kgrad(const fgk_plan *p, int v, const float *g, size_t g_stride, const float *x,
                            size_t x_stride, uint32_t count, float *partials, uint32_t max_rows, uint32_t *rows,
                            void *stream, int num_sms);
/* The one-pass adjoint of the same variant (static_kernel_adj): writes dx
 * (the correlation of each g_b with the taps, as FGK_OP_CORR) and the same
 * partial rows as the taps-gradient kernel. */
int fgk_launch_static_adj(const fgk_plan *p, int v, const float *g, size_t g_stride, const float *x,
                          size_t x_stride, float *dx, size_t dx_stride, const float *kern, uint32_t count,
                          float *partials, uint32_t max_rows, uint32_t *rows, void *stream, int num_sms);

/* The fused overlap-add (static_kernel_ola): the first compiled variant of
 * (modulation, L) that has it, or -1; the launch convolves the nblocks
 * zero-padded blocks of B samples of `in` and writes the first span samples
 * of each result into `out` at b B, adding where two blocks meet (output t
 * with t mod B < span - B, which the caller zeroes first). The caller
 * launches it only when span <= 2 B (at most two additions per sample, so
 * the result does not depend on their order). */
int fgk_static_ola_variant(uint32_t modulation, uint32_t L);
int fgk_launch_static_ola(const fgk_plan *p, int v, const float *in, uint64_t n, uint32_t B, uint32_t span,
                          uint32_t nblocks, uint64_t nout, const float *kern, float *out, void *stream, int num_sms);

/* The call service of a compiled variant (static_kernel_serve): one CTA
 * that runs single transforms on request, with the variant's own stages and
 * tables (so its results are the batched kernel's, bit for bit), without a
 * launch per call. Requests and replies go through words in host-mapped
 * memory (coherent over NVLink-C2C): the host writes the request, then the
 * doorbell (a sequence number); thread 0 polls the doorbell, the CTA runs
 * the op, and thread 0 publishes the sequence number in `reply` with a
 * system-scope release once every output store is done. After idle_polls
 * polls with nothing new the CTA writes 0 to `state`, reads the doorbell
 * once more (after a system-scope fence) and exits unless it changed.
 * All words are 64-bit, each in its own 128-byte line. */
typedef struct fgk_serve_req {
	int32_t      op; /* enum fgk_op (FORWARD, INVERSE, CONV or CORR) */
	uint32_t     reserved;
	const float *in;
	float       *out;
	const float *kern; /* CONV / CORR: the kernel buffer */
} fgk_serve_req;

typedef struct fgk_serve_words {
	const volatile uint64_t *bell;  /* request sequence number (host writes) */
	volatile uint64_t       *reply; /* last sequence number served (device writes) */
	volatile uint64_t       *state; /* the live launch's id; 0 once it exits */
	const fgk_serve_req     *req;   /* the pending request (host writes before the doorbell) */
} fgk_serve_words;

/* 1 when variant v of (modulation, L) has a call service that implements
 * op (compiled variants without bulk-copy input) */
int fgk_static_serve_ok(uint32_t modulation, uint32_t L, int v, int op);
/* launches the service: `seen` is the last sequence number already served,
 * `id` the nonzero value it keeps in state while alive */
int fgk_launch_static_serve(const fgk_plan *p, int v, fgk_serve_words w, uint64_t seen, uint64_t id,
                            uint32_t idle_polls, void *stream);
/* the same for the generic resident kernel (any resident plan, every op,
 * the results of fgk_launch_resident bit for bit) */
int fgk_launch_resident_serve(const fgk_plan *p, fgk_serve_words w, uint64_t seen, uint64_t id, uint32_t idle_polls,
                              void *stream);

#ifdef __cplusplus
}
#endif

#endif

/* Ragged batches as one persistent launch of tile tasks.
 *
 * Every task is a tile of at most FGK_TASK_POINTS points held in two padded
 * shared-memory buffers (ping-pong Stockham stages, one butterfly per thread
 * at a time, runtime radix; fgk_pingpong.cuh), so one CTA of 256 threads
 * needs 70 KB and three CTAs share an SM: while one loads its tile from HBM
 * the others compute, which is what keeps enough bytes in flight. Loads are
 * issued eight per thread before any is used.
 *
 *   SMALL  n items of one size L <= FGK_TASK_POINTS, whole transforms side
 *          by side (tg threads each), HBM in, HBM out.
 *   COLS   a big item (L > FGK_TASK_POINTS) split L = L1 L2 (the fftset's
 *          four-step plan: n = L2 n1 + n2, k = k1 + L1 k2): 2^ls1 adjacent
 *          columns n2, each a DFT of length L1 over n1 read straight from
 *          the input (row segments of 2^ls1 elements), multiplied by
 *          w_L^{n2 k1} and written row-major into the item's scratch.
 *   ROWS   2^ls2 adjacent rows k1 of that scratch, DFTs of length L2 over
 *          n2, written to X[k1 + L1 k2] (segments of 2^ls2 elements).
 *
 * A ROWS task waits for all COLS tasks of its item: each COLS task bumps the
 * item's counter after its stores are visible (threadfence), and a ROWS task
 * spins on it with a bounded wait (on timeout it raises the error flag and
 * skips the tile). Tasks are claimed in list order from an atomic counter,
 * and the host lists every COLS task of an item before its ROWS tasks, so a
 * ROWS task only ever waits on tasks already claimed by running CTAs: no
 * deadlock whatever the residency. The scratch of an item is written and
 * read back within a few microseconds, so it is served by L2; the ROWS task
 * discards the lines it has consumed (discard.global.L2) so that they are
 * never written back to HBM.
 *
 * The FREQ_OFFSET_REAL modulation is fused into the loads (pack and
 * e^{-j pi n/(2L)} = m1[n1] m2[n2]) and the final stores (split X[2m] = W[m],
 * X[2(L-1-m)+1] = conj W[m]; inverse: y = Re/Im of u e^{-j pi m/(2L)}). */
#include <cuda_runtime.h>
#include <stdint.h>
#include "fgk.h"
#include "fgk_pingpong.cuh"

namespace fgk {

constexpr int TK_THREADS = 256;
constexpr int TK_SLOTS = FGK_TASK_POINTS + FGK_TASK_POINTS / 16 + 1; /* rslots(FGK_TASK_POINTS) */
constexpr uint32_t TK_SPIN_LIMIT = 1u << 22;                         /* x 256 ns: about a second */

/* q = w / d for 0 <= w < 2^24, inv = 1/d (one correction step) */
__device__ __forceinline__ int tk_div(int w, int d, float inv)
{
	int q = __float2int_rz(__int2float_rn(w) * inv);
	const int r = w - q * d;
	if (r < 0)
		q--;
	else if (r >= d)
		q++;
	return q;
}

/* Stockham stage over a lane-interleaved tile: element i of lane l at
 * rslot((i << ls) + l); work item w = (butterfly j, lane) with the lane
 * fastest, so a warp's accesses are consecutive slots. */
template <int R>
__device__ __forceinline__ void lane_stage(const float2 *src, float2 *dst, int Lp, int ls, int ns,
                                           const float2 *__restrict__ tw, int tid, int T)
{
	const int nbf = Lp / R;
	const int items = nbf << ls;
	const int lm = (1 << ls) - 1;
	for (int w = tid; w < items; w += T) {
		const int j = w >> ls, lane = w & lm;
		float2 v[R];
#pragma unroll
		for (int p = 0; p < R; p++)
			v[p] = src[rslot(((j + p * nbf) << ls) + lane)];
		const int k = j % ns;
		if (ns > 1) {
			const float2 *t = tw + k * (R - 1);
#pragma unroll
			for (int p = 1; p < R; p++)
				v[p] = cmul(v[p], __ldg(t + p - 1));
		}
		Radix<R>::run(v);
		const int base = (j - k) * R + k;
#pragma unroll
		for (int q = 0; q < R; q++)
			dst[rslot(((base + q * ns) << ls) + lane)] = v[q];
	}
}

/* chain `ch` over the tile in a/b (input in a); returns the result buffer */
__device__ __forceinline__ float2 *lane_chain(const fgk_chain *ch, const float2 *tw, int Lp, int ls, float2 *a,
                                              float2 *b, int tid, int T)
{
	const int n = (int)ch->nstages;
	float2 *src = a, *dst = b;
	for (int s = 0; s < n; s++) {
		const fgk_stage st = ch->st[s];
		FGKR_RADIX_SWITCH(st.radix, (lane_stage<R_>(src, dst, Lp, ls, (int)st.ns, tw + st.tw_off, tid, T)));
		__syncthreads();
		float2 *t = src;
		src = dst;
		dst = t;
	}
	return src;
}

/* w_L^m = thi[m >> 12] tlo[m & 4095] */
__device__ __forceinline__ float2 tk_wl(const fgk_plan4 *p, uint64_t m)
{
	return cmul(__ldg((const float2 *)p->thi + (m >> 12)), __ldg((const float2 *)p->tlo + (m & 4095)));
}

/* ---- SMALL: whole items side by side ---------------------------------- */
__device__ __forceinline__ void task_small(const fgk_task &tk, const fgk_plan *__restrict__ plans,
                                           const fgk_rg_item *__restrict__ items, int op, const float *in_base,
                                           float *out_base, float2 *smem)
{
	const fgk_plan *pl = plans + tk.ref;
	const int L = (int)pl->L;
	const bool freq = pl->modulation == FGK_MOD_FREQOFF;
	const float2 *mod = (const float2 *)pl->modtw;
	const int n = (int)(tk.b & 0xffff), T = (int)(tk.b >> 16);
	const int g = (int)threadIdx.x / T;
	const int tid = (int)threadIdx.x - g * T;
	const bool active = g < n;
	const int slots = rslots(L);
	float2 *buf0 = smem + (size_t)(active ? g : 0) * 2 * slots;
	float2 *buf1 = buf0 + slots;
	const fgk_rg_item it = active ? items[tk.a + g] : fgk_rg_item{0, 0};
	const float *x = in_base + it.in_off;
	float *y = out_base + it.out_off;

	if (active) {
		if (op != FGK_OP_INVERSE) {
			if (freq) {
				batched_copy<8>(
				    L, tid, T, [&](int i) { return make_float2(__ldcs(x + i), -__ldcs(x + L + i)); },
				    [&](int i, float2 v) { buf0[rslot(i)] = cmul(v, __ldg(mod + i)); });
			} else {
				const float2 *x2 = reinterpret_cast<const float2 *>(x);
				batched_copy<8>(
				    L, tid, T, [&](int i) { return __ldcs(x2 + i); }, [&](int i, float2 v) { buf0[rslot(i)] = v; });
			}
		} else {
			const float2 *X = reinterpret_cast<const float2 *>(x);
			if (freq) {
				/* conj W[i]: W[i] = X[2i] for i < ceil(L/2), conj X[2(L-1-i)+1] after */
				const int hc = (L + 1) >> 1;
				batched_copy<8>(
				    L, tid, T,
				    [&](int i) { return i < hc ? conjf2(__ldcs(X + 2 * i)) : __ldcs(X + 2 * (L - 1 - i) + 1); },
				    [&](int i, float2 v) { buf0[rslot(i)] = v; });
			} else {
				batched_copy<8>(
				    L, tid, T, [&](int i) { return __ldcs(X + i); },
				    [&](int i, float2 v) { buf0[rslot(i)] = conjf2(v); });
			}
		}
	}
	__syncthreads();
	const float2 *src = rg_chain(pl, buf0, buf1, active, tid, T, [] { __syncthreads(); });
	if (active) {
		float2 *y2 = reinterpret_cast<float2 *>(y);
		if (op == FGK_OP_INVERSE) {
			if (freq) {
				for (int i = tid; i < L; i += T) {
					const float2 r = cmul(src[rslot(i)], __ldg(mod + i));
					__stcs(y + i, r.x);
					__stcs(y + L + i, r.y);
				}
			} else {
				for (int i = tid; i < L; i += T)
					__stcs(y2 + i, conjf2(src[rslot(i)]));
			}
		} else if (freq) {
			const int hc = (L + 1) >> 1;
			for (int i = tid; i < L; i += T) {
				const float2 v = src[rslot(i)];
				if (i < hc)
					__stcs(y2 + 2 * i, v);
				else
					__stcs(y2 + 2 * (L - 1 - i) + 1, conjf2(v));
			}
		} else {
			for (int i = tid; i < L; i += T)
				__stcs(y2 + i, src[rslot(i)]);
		}
	}
}

/* ---- COLS: columns of a big item into its scratch ---------------------- */
__device__ __forceinline__ void task_cols(const fgk_task &tk, const fgk_big &bg, int op, const float *in_base,
                                          float2 *scratch, int *done, float2 *smem)
{
	const fgk_plan4 *p = bg.p4;
	const int L1 = (int)p->L1, L2 = (int)p->L2;
	const uint64_t L = (uint64_t)L1 * L2;
	const int ls = (int)bg.ls1, lm = (1 << ls) - 1;
	const int n2base = (int)(tk.a << ls);
	const bool freq = p->modulation == FGK_MOD_FREQOFF;
	const bool inverse = op == FGK_OP_INVERSE;
	const float *x = in_base + bg.in_off;
	const float2 *x2 = reinterpret_cast<const float2 *>(x);
	const float2 *m1 = (const float2 *)p->m1, *m2 = (const float2 *)p->m2;
	const int tid = (int)threadIdx.x, T = (int)blockDim.x;
	float2 *A = smem, *B = smem + TK_SLOTS;

	batched_copy<8>(
	    L1 << ls, tid, T,
	    [&](int w) {
		    const int n1 = w >> ls, n2 = n2base + (w & lm);
		    if (n2 >= L2)
			    return make_float2(0.f, 0.f);
		    const uint64_t n = (uint64_t)n1 * L2 + n2;
		    if (!inverse) {
			    if (freq)
				    return cmul(make_float2(__ldcs(x + n), -__ldcs(x + L + n)), cmul(__ldg(m1 + n1), __ldg(m2 + n2)));
			    return __ldcs(x2 + n);
		    }
		    if (freq)
			    return n < ((L + 1) >> 1) ? conjf2(__ldcs(x2 + 2 * n)) : __ldcs(x2 + 2 * (L - 1 - n) + 1);
		    return conjf2(__ldcs(x2 + n));
	    },
	    [&](int w, float2 v) { A[rslot(w)] = v; });
	__syncthreads();
	const float2 *R = lane_chain(&p->c1, (const float2 *)p->tw1, L1, ls, A, B, tid, T);
	float2 *S = scratch + bg.scratch_off;
	for (int w = tid; w < (L1 << ls); w += T) {
		const int k1 = w >> ls, n2 = n2base + (w & lm);
		if (n2 < L2)
			__stcg(S + (uint64_t)k1 * L2 + n2, cmul(R[rslot(w)], tk_wl(p, (uint64_t)n2 * (uint32_t)k1)));
	}
	__threadfence();
	__syncthreads();
	if (tid == 0)
		atomicAdd(done, 1);
}

/* ---- ROWS: rows of the scratch into the output -------------------------- */
__device__ __forceinline__ void task_rows(const fgk_task &tk, const fgk_big &bg, int op, float *out_base,
                                          float2 *scratch, const int *done, int *err, float2 *smem)
{
	__shared__ int failed;
	const fgk_plan4 *p = bg.p4;
	const int L1 = (int)p->L1, L2 = (int)p->L2;
	const uint64_t L = (uint64_t)L1 * L2;
	const int ls = (int)bg.ls2, nl = 1 << ls, lm = nl - 1;
	const int k1base = (int)(tk.a << ls);
	const bool freq = p->modulation == FGK_MOD_FREQOFF;
	const bool inverse = op == FGK_OP_INVERSE;
	const int tid = (int)threadIdx.x, T = (int)blockDim.x;
	float2 *A = smem, *B = smem + TK_SLOTS;
	float2 *S = scratch + bg.scratch_off;

	/* every COLS tile of this item, bounded */
	if (tid == 0) {
		int f = 0;
		uint32_t it = 0;
		for (;;) {
			int d;
			asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(d) : "l"(done) : "memory");
			if (d >= (int)bg.ncols)
				break;
			if (++it > TK_SPIN_LIMIT) {
				f = 1;
				if (err)
					atomicExch(err, 1);
				break;
			}
			__nanosleep(256);
		}
		__threadfence();
		failed = f;
	}
	__syncthreads();
	if (failed)
		return; /* the caller's barrier ends the task */

	const int nrow = min(nl, L1 - k1base); /* rows of this tile */
	const float inv = 1.0f / (float)L2;
	const float2 *Srow = S + (uint64_t)k1base * L2;
	batched_copy<8>(
	    nrow * L2, tid, T, [&](int w) { return __ldcg(Srow + w); },
	    [&](int w, float2 v) {
		    const int lane = tk_div(w, L2, inv), n2 = w - lane * L2;
		    A[rslot((n2 << ls) + lane)] = v;
	    });
	if (nrow < nl) /* lanes past the last row hold zeros */
		for (int w = tid; w < (L2 << ls); w += T)
			if ((w & lm) >= nrow)
				A[rslot(w)] = make_float2(0.f, 0.f);
	__syncthreads();
	/* the rows are consumed: drop their L2 lines without writing them back */
	{
		const uintptr_t b0 = (reinterpret_cast<uintptr_t>(Srow) + 127) & ~(uintptr_t)127;
		const uintptr_t b1 = reinterpret_cast<uintptr_t>(Srow + (uint64_t)nrow * L2) & ~(uintptr_t)127;
		for (uintptr_t a = b0 + (uintptr_t)tid * 128; a < b1; a += (uintptr_t)T * 128)
			asm volatile("discard.global.L2 [%0], 128;" ::"l"(a) : "memory");
	}
	const float2 *R = lane_chain(&p->c2, (const float2 *)p->tw2, L2, ls, A, B, tid, T);
	float *o = out_base + bg.out_off;
	float2 *o2 = reinterpret_cast<float2 *>(o);
	const float2 *q1 = (const float2 *)p->n1, *q2 = (const float2 *)p->n2;
	for (int w = tid; w < (L2 << ls); w += T) {
		const int k2 = w >> ls, lane = w & lm;
		if (lane >= nrow)
			continue;
		const int k1 = k1base + lane;
		const uint64_t m = (uint64_t)k1 + (uint64_t)L1 * k2;
		const float2 v = R[rslot(w)];
		if (!inverse) {
			if (!freq)
				__stcs(o2 + m, v);
			else if (m < ((L + 1) >> 1))
				__stcs(o2 + 2 * m, v);
			else
				__stcs(o2 + 2 * (L - 1 - m) + 1, conjf2(v));
		} else if (freq) {
			const float2 r = cmul(v, cmul(__ldg(q1 + k1), __ldg(q2 + k2)));
			__stcs(o + m, r.x);
			__stcs(o + L + m, r.y);
		} else {
			__stcs(o2 + m, conjf2(v));
		}
	}
}

__global__ void __launch_bounds__(TK_THREADS, 3)
    task_kernel(const fgk_task *__restrict__ tasks, uint32_t ntasks, const fgk_plan *__restrict__ plans,
                const fgk_rg_item *__restrict__ items, const fgk_big *__restrict__ bigs, int *counters,
                float2 *scratch, int op, const float *in_base, float *out_base, int *err)
{
	extern __shared__ float2 smem[];
	__shared__ uint32_t cur;
	for (;;) {
		if (threadIdx.x == 0)
			cur = (uint32_t)atomicAdd(counters, 1);
		__syncthreads();
		const uint32_t c = cur;
		if (c >= ntasks)
			break;
		const fgk_task tk = tasks[c];
		if (tk.kind == FGK_TASK_SMALL)
			task_small(tk, plans, items, op, in_base, out_base, smem);
		else if (tk.kind == FGK_TASK_COLS)
			task_cols(tk, bigs[tk.ref], op, in_base, scratch, counters + 1 + tk.ref, smem);
		else
			task_rows(tk, bigs[tk.ref], op, out_base, scratch, counters + 1 + tk.ref, err, smem);
		__syncthreads(); /* buffers and `cur` are reused by the next task */
	}
}

} /* namespace fgk */

extern "C" int fgk_tasks_grid(int num_sms)
{
	return 3 * num_sms;
}

extern "C" int fgk_launch_tasks(const fgk_task *tasks_dev, uint32_t ntasks, const fgk_plan *plans_dev,
                                const fgk_rg_item *items_dev, const fgk_big *bigs_dev, uint32_t nbig,
                                int *counters_dev, float *scratch_dev, int op, const float *in_base, float *out_base,
                                int num_sms, int *err_flag, void *stream)
{
	using namespace fgk;
	const size_t smem = 2 * (size_t)TK_SLOTS * sizeof(float2);
	cudaError_t e;
	(void)bigs_dev;
	if (ntasks == 0)
		return 0;
	if ((e = cudaFuncSetAttribute((const void *)task_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
	    cudaSuccess)
		return (int)e;
	if ((e = cudaMemsetAsync(counters_dev, 0, sizeof(int) * (1 + (size_t)nbig), (cudaStream_t)stream)) != cudaSuccess)
		return (int)e;
	uint32_t grid = (uint32_t)fgk_tasks_grid(num_sms);
	if (grid > ntasks)
		grid = ntasks;
	task_kernel<<<grid, TK_THREADS, smem, (cudaStream_t)stream>>>(tasks_dev, ntasks, plans_dev, items_dev, bigs_dev,
	                                                              counters_dev, reinterpret_cast<float2 *>(scratch_dev),
	                                                              op, in_base, out_base, err_flag);
	return (int)cudaGetLastError();
}

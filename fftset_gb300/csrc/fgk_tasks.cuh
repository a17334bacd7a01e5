/* Ragged batches as one persistent launch of tile tasks.
 *
 * Every task is a tile of at most FGKT_POINTS points held in two padded
 * shared-memory buffers (ping-pong Stockham stages, one butterfly per thread
 * at a time, runtime radix; fgk_pingpong.cuh), 70 KB per CTA, or in one
 * buffer when every chain of the list has two stages; the CTA shapes are
 * described at TK_THREADS_NARROW.
 *
 *   SMALL  n items of one size L <= FGKT_POINTS, whole transforms side
 *          by side (tg threads each), HBM in, HBM out.
 *   COLS   a big item (L > FGKT_POINTS) split L = L1 L2 (the fftset's
 *          four-step plan: n = L2 n1 + n2, k = k1 + L1 k2): 2^ls1 adjacent
 *          columns n2, each a DFT of length L1 over n1 whose first stage
 *          reads the input directly (row segments of 2^ls1 elements) and
 *          whose last stage multiplies by w_L^{n2 k1} and writes the item's
 *          scratch directly, in the order the ROWS tiles read it.
 *   ROWS   2^ls2 adjacent rows k1 of that scratch (one contiguous block),
 *          DFTs of length L2 over n2, the last stage writing X[k1 + L1 k2]
 *          directly (segments of 2^ls2 elements).
 * Only the middle stages of a big-item tile go through shared memory.
 * Big-item tiles have at least 16 lanes (L1, L2 <= 256), which makes the
 * Rows layout below conflict-free.
 *
 * A ROWS task waits for all COLS tasks of its item: each COLS task bumps the
 * item's counter with a gpu-scope release add after a barrier, and a ROWS task
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
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "fgk.h"
#include "fgk_pingpong.cuh"

namespace fgk {

#ifndef FGKT_POINTS
#define FGKT_POINTS 4096 /* points of a tile */
#endif
/* CTA shapes, chosen per task list (fgk.h, enum fgk_task_shape). Narrow
 * and wide have two tile buffers and three CTAs (three tiles) per SM:
 * narrow, 128 threads (up to 168 registers a thread, no spills), for lists
 * with chains of three stages or more (the 20000-item ragged mix: 1.757 ms
 * against 1.851 on two wide CTAs per SM and 1.90 on three); wide, 256
 * threads (80 registers, a few hundred bytes of spills), for such lists
 * with three-level items (the 15,728,640-bin forward + inverse on it: 0.604
 * ms against 0.641 on two wide CTAs per SM, with no spills, and 0.684
 * narrow). */
constexpr int TK_THREADS_NARROW = 128, TK_CTAS_NARROW = 3;
constexpr int TK_THREADS_WIDE = 256, TK_CTAS_WIDE = 3;
/* A third shape for lists whose every chain has at most two stages (the
 * first stage writes buffer A and the last reads it, so B is never used):
 * 128 threads, one buffer, six CTAs (six tiles in flight) per SM, 80
 * registers with a few hundred bytes of spills. The 15,728,640-bin
 * forward + inverse (240 x 256 x 256, all two-stage): 0.53 ms against 0.604
 * on the wide shape; the 65536-bin convolution batch 0.60 against 0.70 ms
 * on the narrow one. A task whose chain is longer is refused (error flag)
 * rather than run on one buffer; the host never lists one. */
constexpr int TK_THREADS_SINGLE = 128, TK_CTAS_SINGLE = 6;
/* float2 slots of one of the two tile buffers: rslots(points), rounded up to 4 */
constexpr int TK_SLOTS = (FGKT_POINTS + FGKT_POINTS / 16 + 1 + 3) & ~3;

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

/* Shared-memory layouts of a tile (element i of lane l):
 *   Pad   (one lane, whole items)  slot i + i/16: the strided accesses of a
 *         stage spread over the banks;
 *   Rows  (16 or more lanes)       slot i (nl + 1) + l: linear in i, so a
 *         stage's R accesses are one base plus multiples of a stride, and
 *         conflict-free whether a warp runs along the lanes or along i. */
struct Pad {
	int ls;
	__device__ __forceinline__ int slot(int i, int lane) const { return rslot((i << ls) + lane); }
};
struct Rows {
	int ls;
	__device__ __forceinline__ int slot(int i, int lane) const { return i * ((1 << ls) + 1) + lane; }
};

/* e^{-j pi x} (x = 2 m / D) by CUDA's sincospif */
__device__ __forceinline__ float2 tk_expi(float x)
{
	float sn, cs;
	sincospif(x, &sn, &cs);
	return make_float2(cs, -sn);
}

/* w_D^m = e^{-2 pi j m / D} for 0 <= m < D, x2 = 2 / D: the angle taken
 * in (-pi, pi] so that its rounding error stays below pi 2^-23 */
__device__ __forceinline__ float2 tk_wm(uint32_t m, uint32_t D, float x2)
{
	const int mm = m > (D >> 1) ? (int)(m - D) : (int)m;
	return tk_expi((float)mm * x2);
}

/* v[p] *= w^{p k} (p = 1..R-1), w = e^{-2 pi j / D}, x2 = 2 / D. The
 * butterfly's base twiddles are computed, not read: w^{k} and (radix 8
 * and above) w^{8k} by sincospif, w^{2k} and w^{4k} as squares, the other
 * powers as products (twiddle_powers, fgk_codelets.cuh). A table read
 * would go through an L1 shared with many sizes' tables and three tiles'
 * shared memory, and its latency sat on every stage's critical path. */
template <int R> __device__ __forceinline__ void tk_twiddle(float2 (&v)[R], int k, float x2)
{
	const float2 w1 = tk_expi((float)k * x2);
	const float2 w2 = cmul(w1, w1);
	float2 w4 = make_float2(1.f, 0.f), w8 = w4;
	if constexpr (R > 4)
		w4 = cmul(w2, w2);
	if constexpr (R > 8)
		w8 = tk_expi((float)(8 * k) * x2);
	float2 w[R];
	twiddle_powers<R>(w, [&](int p) { return p == 1 ? w1 : p == 2 ? w2 : p == 4 ? w4 : w8; });
#pragma unroll
	for (int p = 1; p < R; p++)
		v[p] = cmul(v[p], w[p]);
}

/* Stockham stage over a lane-interleaved tile: element i of lane l at
 * rslot((i << ls) + l); work item w = (butterfly j, lane) with the lane
 * fastest, so a warp's accesses are consecutive slots. */
template <int R, class A>
__device__ __forceinline__ void lane_stage(const float2 *src, float2 *dst, int Lp, int ls, int ns, int tid, int T,
                                           A ad)
{
	const int nbf = Lp / R;
	const float x2 = 2.0f / (float)(ns * R);
	const int items = nbf << ls;
	const int lm = (1 << ls) - 1;
	for (int w = tid; w < items; w += T) {
		const int j = w >> ls, lane = w & lm;
		float2 v[R];
#pragma unroll
		for (int p = 0; p < R; p++)
			v[p] = src[ad.slot(j + p * nbf, lane)];
		const int k = j % ns;
		if (ns > 1)
			tk_twiddle<R>(v, k, x2);
		Radix<R>::run(v);
		const int base = (j - k) * R + k;
#pragma unroll
		for (int q = 0; q < R; q++)
			dst[ad.slot(base + q * ns, lane)] = v[q];
	}
}

/* ---- tiles: first and last stages straight from and to memory ---------- */
/* First stage of a tile (ns = 1, no twiddles) straight from memory:
 * butterfly j of lane l reads ld(j + p nbf, l) (lanes fastest, so a warp
 * reads consecutive lanes of one element: the row segments in memory). */
/* butterflies a thread loads side by side in the first stage, so that
 * 16 loads are in flight for the radices 2, 4 and 8 */
template <int R> struct Batch {
	static constexpr int B = 1;
};

template <int R, class A, class Ld>
__device__ __forceinline__ void lane_first(Ld &&ld, float2 *dst, int Lp, int ls, int tid, int T, A ad)
{
	constexpr int B = Batch<R>::B;
	const int nbf = Lp / R;
	const int items = nbf << ls;
	const int lm = (1 << ls) - 1;
	for (int w0 = tid; w0 < items; w0 += B * T) {
		float2 v[B][R];
#pragma unroll
		for (int b = 0; b < B; b++) {
			const int w = w0 + b * T;
			if (w < items) {
				const int j = w >> ls, lane = w & lm;
#pragma unroll
				for (int p = 0; p < R; p++)
					v[b][p] = ld(j + p * nbf, lane);
			}
		}
#pragma unroll
		for (int b = 0; b < B; b++) {
			const int w = w0 + b * T;
			if (w < items) {
				const int j = w >> ls, lane = w & lm;
				Radix<R>::run(v[b]);
#pragma unroll
				for (int q = 0; q < R; q++)
					dst[ad.slot(j * R + q, lane)] = v[b][q];
			}
		}
	}
}

/* Last stage of a tile (ns = Lp/R: butterfly j twiddled by w^{p j},
 * outputs k = j + q nbf) straight to memory through st(j, q, nbf, lane, v). JF: a warp
 * takes consecutive butterflies j of one lane (consecutive outputs k),
 * otherwise consecutive lanes of one butterfly. */
template <int R, bool JF, class A, class St>
__device__ __forceinline__ void lane_last(const float2 *src, St &&st, int Lp, int ls, int tid, int T, A ad)
{
	const int nbf = Lp / R;
	const float x2 = 2.0f / (float)Lp;
	const int items = nbf << ls;
	const int lm = (1 << ls) - 1;
	const float inv = 1.0f / (float)nbf;
	for (int w = tid; w < items; w += T) {
		int j, lane;
		if (JF) {
			lane = tk_div(w, nbf, inv);
			j = w - lane * nbf;
		} else {
			j = w >> ls;
			lane = w & lm;
		}
		float2 v[R];
#pragma unroll
		for (int p = 0; p < R; p++)
			v[p] = src[ad.slot(j + p * nbf, lane)];
		if (nbf > 1)
			tk_twiddle<R>(v, j, x2);
		Radix<R>::run(v);
#pragma unroll
		for (int q = 0; q < R; q++)
			st(j, q, nbf, lane, v[q]);
	}
}

/* A single-stage chain (Lp = R): memory to memory */
template <int R, class Ld, class St>
__device__ __forceinline__ void lane_single(Ld &&ld, St &&st, int ls, int tid, int T)
{
	const int lanes = 1 << ls;
	for (int lane = tid; lane < lanes; lane += T) {
		float2 v[R];
#pragma unroll
		for (int p = 0; p < R; p++)
			v[p] = ld(p, lane);
		Radix<R>::run(v);
#pragma unroll
		for (int q = 0; q < R; q++)
			st(0, q, 1, lane, v[q]);
	}
}

/* The whole chain of a tile: first stage from ld, middle stages in shared
 * memory (A/B ping-pong), last stage to st. `after_first` runs once the first
 * stage is done (all of its reads have returned). Threads with active ==
 * false only take part in the barriers. */
template <bool JF, class AD, class Ld, class St, class After>
__device__ __forceinline__ void tile_chain(uint64_t code, int Lp, int ls, float2 *A, float2 *B, int tid, int T,
                                           bool active, Ld &&ld, St &&st, After &&after_first)
{
	/* the chain comes packed in one word (fgk_chain.code) from the task's
	 * descriptor: no stage reads global memory for its radix */
	const AD ad{ls};
	const int n = (int)(code & 15);
	const int r0 = (int)((code >> 4) & 15) + 1;
	if (n == 1) {
		if (active)
			FGKR_RADIX_SWITCH(r0, (lane_single<R_>(ld, st, ls, tid, T)));
		__syncthreads();
		after_first();
		return;
	}
	if (active)
		FGKR_RADIX_SWITCH(r0, (lane_first<R_>(ld, A, Lp, ls, tid, T, ad)));
	__syncthreads();
	after_first();
	float2 *src = A, *dst = B;
	int ns = r0;
	for (int s = 1; s < n - 1; s++) {
		const int r = (int)((code >> (4 * s + 4)) & 15) + 1;
		if (active)
			FGKR_RADIX_SWITCH(r, (lane_stage<R_>(src, dst, Lp, ls, ns, tid, T, ad)));
		__syncthreads();
		ns *= r;
		float2 *t = src;
		src = dst;
		dst = t;
	}
	if (active) {
		const int rl = (int)((code >> (4 * n)) & 15) + 1;
		FGKR_RADIX_SWITCH(rl, (lane_last<R_, JF>(src, st, Lp, ls, tid, T, ad)));
	}
}

/* Bounded wait of a whole CTA until *ctr >= need (thread 0 polls with an
 * acquire load, then a barrier), at most spin_limit polls about 256 ns
 * apart (the host's default, 2^22, is about a second). On timeout the error
 * flag is raised and false returned: the caller skips its tile. */
__device__ __forceinline__ bool tk_wait(const int *ctr, int need, int *err, int *failed, uint32_t spin_limit)
{
	if (threadIdx.x == 0) {
		int f = 0;
		uint32_t it = 0;
		for (;;) {
			int d;
			asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(d) : "l"(ctr) : "memory");
			if (d >= need)
				break;
			if (++it > spin_limit) {
				f = 1;
				if (err)
					atomicExch(err, 1);
				break;
			}
			__nanosleep(256);
		}
		/* no fence: the acquire load, then the barrier, order every
		 * thread's later reads after the counted tiles' stores */
		*failed = f;
	}
	__syncthreads();
	return !*failed;
}

/* A tile's count: after the task loop's barrier that follows the tile (so
 * after every thread's scratch stores), thread 0 makes one gpu-scope
 * release add (cumulative: it publishes the whole CTA's stores). Tiles that
 * count return their counter to the loop; the loop's barrier is the only
 * one, and a release add takes no full fence. */
__device__ __forceinline__ void tk_release(int *ctr)
{
	asm volatile("red.release.gpu.global.add.s32 [%0], 1;" ::"l"(ctr) : "memory");
}

/* v times bin m of the product's natural-order spectrum */
__device__ __forceinline__ float2 tk_product(const fgk_product &pr, uint32_t m, float2 v)
{
	return cmul(v, __ldg(reinterpret_cast<const float2 *>(pr.spec) + m));
}

/* ---- SMALL: whole items side by side ---------------------------------- */
/* n items of one size, tg threads each (group g = threadIdx / tg), each
 * group's first stage reading its item and its last stage writing its
 * output directly. */
template <bool inverse, bool freq, class Pre>
__device__ __forceinline__ void task_small(const fgk_task &tk, const fgk_plan *__restrict__ plans,
                                           const fgk_rg_item *__restrict__ items, const float *in_base,
                                           float *out_base, float2 *smem, Pre &&pre)
{
	const fgk_plan *pl = plans + tk.ref;
	const int L = (int)pl->L;
	const int n = (int)(tk.b & 0xffff), T = (int)(tk.b >> 16);
	const int g = (int)threadIdx.x / T;
	const int tid = (int)threadIdx.x - g * T;
	const bool active = g < n;
	float2 *buf0 = smem + (size_t)(active ? g : 0) * 2 * rslots(L);
	const fgk_rg_item it = active ? items[tk.a + g] : fgk_rg_item{0, 0};
	const float *x = in_base + it.in_off;
	const float2 *X = reinterpret_cast<const float2 *>(x);
	float *y = out_base + it.out_off;
	float2 *y2 = reinterpret_cast<float2 *>(y);
	const float2 *mod = (const float2 *)pl->modtw;
	const int hc = (L + 1) >> 1;
	auto ld = [&](int i, int) {
		if (!inverse) {
			if (freq)
				return cmul(make_float2(__ldcs(x + i), -__ldcs(x + L + i)), __ldg(mod + i));
			return __ldcs(X + i);
		}
		/* conj W[i]: W[i] = X[2i] for i < ceil(L/2), conj X[2(L-1-i)+1] after */
		if (freq)
			return i < hc ? conjf2(__ldcs(X + 2 * i)) : __ldcs(X + 2 * (L - 1 - i) + 1);
		return conjf2(__ldcs(X + i));
	};
	auto st = [&](int j, int q, int nbf, int, float2 v) {
		const int k = j + q * nbf;
		if (!inverse) {
			if (!freq)
				__stcs(y2 + k, v);
			else if (k < hc)
				__stcs(y2 + 2 * k, v);
			else
				__stcs(y2 + 2 * (L - 1 - k) + 1, conjf2(v));
		} else if (freq) {
			const float2 r = cmul(v, __ldg(mod + k));
			__stcs(y + k, r.x);
			__stcs(y + L + k, r.y);
		} else {
			__stcs(y2 + k, conjf2(v));
		}
	};
	tile_chain<false, Pad>(pl->fwd.code, L, 0, buf0, buf0 + rslots(L), tid, T, active, ld, st,
	                       pre);
}

/* COLS: columns n2base .. n2base + 2^ls1 - 1, DFTs of length L1 from the
 * input into the item's scratch, which is laid out by ROWS tiles: element
 * (k1, n2) at ((k1 >> ls2) L2 + n2) 2^ls2 + (k1 & (2^ls2 - 1)), so a ROWS
 * tile reads one contiguous block with its lanes fastest. */
template <bool inverse, bool freq, class Pre>
__device__ __forceinline__ int *task_cols(const fgk_task &tk, const fgk_big &bg, const float *in_base,
                                          float2 *scratch, int *done, float2 *smem, Pre &&pre)
{
	const fgk_plan4 *p = bg.p4;
	const int L1 = (int)bg.L1, L2 = (int)bg.L2;
	const uint32_t L = (uint32_t)L1 * (uint32_t)L2;
	const int ls = (int)bg.ls1;
	const int ls2 = (int)bg.ls2, lm2 = (1 << ls2) - 1;
	const int n2base = (int)(tk.a << ls);
	const float *x = in_base + bg.in_off;
	const float2 *x2 = reinterpret_cast<const float2 *>(x);
	const float2 *m1 = (const float2 *)p->m1, *m2 = (const float2 *)p->m2;
	const float xL = 2.0f / (float)L;
	float2 *S = scratch + bg.scratch_off;
	auto ld = [&](int n1, int lane) {
		const int n2 = n2base + lane;
		if (n2 >= L2)
			return make_float2(0.f, 0.f);
		const uint32_t n = (uint32_t)n1 * (uint32_t)L2 + (uint32_t)n2;
		if (!inverse) {
			if (freq)
				return cmul(make_float2(__ldcs(x + n), -__ldcs(x + L + n)), cmul(__ldg(m1 + n1), __ldg(m2 + n2)));
			return __ldcs(x2 + n);
		}
		if (freq)
			return n < ((L + 1) >> 1) ? conjf2(__ldcs(x2 + 2 * n)) : __ldcs(x2 + 2 * (L - 1 - n) + 1);
		return conjf2(__ldcs(x2 + n));
	};
	const float2 *tq = (const float2 *)p->tq;
	/* w_L^{n2 k1}, k1 = j + q nbf: w_L^{n2 j} w_{R L2}^{n2 q} (L = R nbf L2;
	 * n2 q < R L2, so no reduction) */
	auto st = [&](int j, int q, int nbf, int lane, float2 v) {
		const int n2 = n2base + lane;
		if (n2 >= L2)
			return;
		const int k1 = j + q * nbf;
		const uint32_t m = (uint32_t)n2 * (uint32_t)j;
		const float2 a = tk_wm(m, L, xL);
		const float2 w = q ? cmul(a, __ldg(tq + (uint32_t)n2 * (uint32_t)q)) : a;
		__stcg(S + ((((uint32_t)(k1 >> ls2) * (uint32_t)L2 + (uint32_t)n2) << ls2) + (uint32_t)(k1 & lm2)),
		       cmul(v, w));
	};
	tile_chain<true, Rows>(bg.code1, L1, ls, smem, smem + TK_SLOTS, (int)threadIdx.x,
	                       (int)blockDim.x, true, ld, st, pre);
	return done;
}

/* ROWS: rows k1base .. k1base + 2^ls2 - 1 of the scratch, DFTs of length L2
 * into X[k1 + L1 k2] */
template <bool inverse, bool freq, class Pre>
__device__ __forceinline__ void task_rows(const fgk_task &tk, const fgk_big &bg, float *out_base, float2 *scratch,
                                          const int *done, int *err, uint32_t spin_limit, const fgk_product &prod,
                                          float2 *smem, int *failed, Pre &&pre)
{
	const fgk_plan4 *p = bg.p4;
	const int L1 = (int)bg.L1, L2 = (int)bg.L2;
	const uint32_t L = (uint32_t)L1 * (uint32_t)L2;
	const int ls = (int)bg.ls2, nl = 1 << ls;
	const int k1base = (int)(tk.a << ls);
	const int nrow = min(nl, L1 - k1base);
	const int tid = (int)threadIdx.x, T = (int)blockDim.x;

	/* every COLS tile of this item, bounded */
	if (!tk_wait(done, (int)bg.ncols, err, failed, spin_limit))
		return;

	const float2 *Stile = scratch + bg.scratch_off + (uint64_t)tk.a * ((uint64_t)L2 << ls);
	float *o = out_base + bg.out_off;
	float2 *o2 = reinterpret_cast<float2 *>(o);
	const float2 *q1 = (const float2 *)p->n1, *q2 = (const float2 *)p->n2;
	auto ld = [&](int n2, int lane) { return __ldcg(Stile + (((uint32_t)n2 << ls) + (uint32_t)lane)); };
	auto st = [&](int j, int q, int nbf, int lane, float2 v) {
		if (lane >= nrow)
			return;
		const int k2 = j + q * nbf;
		const int k1 = k1base + lane;
		const uint32_t m = (uint32_t)k1 + (uint32_t)L1 * (uint32_t)k2;
		if (!inverse) {
			if (prod.spec)
				v = tk_product(prod, m, v);
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
	};
	/* once the first stage has read the tile, drop its L2 lines without
	 * writing them back */
	auto discard = [&] {
		const uintptr_t b0 = reinterpret_cast<uintptr_t>(Stile);
		const uintptr_t b1 = b0 + ((uintptr_t)L2 << ls) * sizeof(float2);
		for (uintptr_t a = ((b0 + 127) & ~(uintptr_t)127) + (uintptr_t)tid * 128; a + 128 <= b1; a += (uintptr_t)T * 128)
			asm volatile("discard.global.L2 [%0], 128;" ::"l"(a) : "memory");
	};
	tile_chain<false, Rows>(bg.code2, L2, ls, smem, smem + TK_SLOTS, tid, T, true, ld, st,
	                        [&] {
		                        discard();
		                        pre();
	                        });
}

/* ---- three-level items (fgk_plan3): passes A, B, C ------------------- */
/* The two scratch areas are laid out in blocks of 4 k1 x 4 n3 (128 bytes),
 * L1q = ceil(L1/4) and L3q = ceil(L3/4) blocks along k1 and n3:
 *   A (k1, n2, n3) in block ((n2 L3q + n3/4) L1q + k1/4), at (k1%4) 4 + n3%4;
 *   B (k2, n3, k1) in block ((k2 L1q + k1/4) L3q + n3/4), at (n3%4) 4 + k1%4.
 * A pass-B tile (4 k1 x 4 n3 lanes) then reads one whole block of A per n2
 * and writes one whole block of B per k2; a pass-A store of 16 adjacent n3
 * fills four 32-byte sectors, and a pass-C load of 16 adjacent k1 reads four
 * whole sectors. */
__device__ __forceinline__ uint32_t tk_blk_a(uint32_t k1, uint32_t n2, uint32_t n3, uint32_t L1q, uint32_t L3q)
{
	return (((n2 * L3q + (n3 >> 2)) * L1q + (k1 >> 2)) << 4) + ((k1 & 3) << 2) + (n3 & 3);
}
__device__ __forceinline__ uint32_t tk_blk_b(uint32_t k2, uint32_t n3, uint32_t k1, uint32_t L1q, uint32_t L3q)
{
	return (((k2 * L1q + (k1 >> 2)) * L3q + (n3 >> 2)) << 4) + ((n3 & 3) << 2) + (k1 & 3);
}

/* A: 16 adjacent columns c = n2 L3 + n3, DFT_L1 over n1 straight from the
 * input, times w_{L1 L2}^{n2 k1} = w_{L1 L2}^{n2 j} w_{R1 L2}^{n2 q}, into
 * the blocked A. Returns the counter of the tile's group (tile t, columns
 * 16t .. 16t + 15: n3 group t % ngrp when 16 divides L3). */
template <bool inverse, bool freq, class Pre>
__device__ __forceinline__ int *task_pa(const fgk_task &tk, const fgk_huge &hg, const float *in_base,
                                        float2 *scratch, int *hcounters, float2 *smem, Pre &&pre)
{
	const fgk_plan3 *p = hg.p3;
	const int L1 = (int)hg.L1, L3 = (int)hg.L3;
	const uint32_t L23 = hg.L2 * hg.L3, L = (uint32_t)L1 * L23;
	const int cbase = (int)(tk.a << 4);
	const float inv3 = 1.0f / (float)L3;
	const float *x = in_base + hg.in_off;
	const float2 *x2 = reinterpret_cast<const float2 *>(x);
	const float2 *ma = (const float2 *)p->ma, *mb = (const float2 *)p->mb, *mc = (const float2 *)p->mc;
	const float2 *tq = (const float2 *)p->tq1;
	const uint32_t L12 = (uint32_t)L1 * hg.L2;
	const float x12 = 2.0f / (float)L12;
	float2 *A = scratch + hg.sa;
	auto ld = [&](int n1, int lane) {
		const uint32_t c = (uint32_t)(cbase + lane);
		if (c >= L23)
			return make_float2(0.f, 0.f);
		const uint32_t n = (uint32_t)n1 * L23 + c;
		if (!inverse) {
			if (freq) {
				const int n2 = tk_div((int)c, L3, inv3), n3 = (int)c - n2 * L3;
				const float2 m = cmul(__ldg(ma + n1), cmul(__ldg(mb + n2), __ldg(mc + n3)));
				return cmul(make_float2(__ldcs(x + n), -__ldcs(x + L + n)), m);
			}
			return __ldcs(x2 + n);
		}
		if (freq)
			return n < ((L + 1) >> 1) ? conjf2(__ldcs(x2 + 2 * n)) : __ldcs(x2 + 2 * (L - 1 - n) + 1);
		return conjf2(__ldcs(x2 + n));
	};
	const uint32_t L1q = (uint32_t)(L1 + 3) >> 2, L3q = hg.nb3;
	auto st = [&](int j, int q, int nbf, int lane, float2 v) {
		const uint32_t c = (uint32_t)(cbase + lane);
		if (c >= L23)
			return;
		const int n2 = tk_div((int)c, L3, inv3);
		const uint32_t m = (uint32_t)n2 * (uint32_t)j;
		const float2 b = tk_wm(m, L12, x12);
		const float2 w = q ? cmul(b, __ldg(tq + (uint32_t)n2 * (uint32_t)q)) : b;
		__stcg(A + tk_blk_a((uint32_t)(j + q * nbf), (uint32_t)n2, c - (uint32_t)n2 * (uint32_t)L3, L1q, L3q),
		       cmul(v, w));
	};
	tile_chain<false, Rows>(hg.code1, L1, 4, smem, smem + TK_SLOTS, (int)threadIdx.x,
	                        (int)blockDim.x, true, ld, st, pre);
	return hcounters + hg.cnt + tk.a % hg.ngrp;
}

/* B: a block of 4 k1 x 4 n3 (lanes l -> k1b + l/4, n3b + l%4), DFT_L2 over
 * n2 from the blocked A (one block per n2), times w_L^{n3 (k1 + L1 k2)} =
 * w_L^{n3 (k1 + L1 j)} w_{R2 L3}^{n3 q}, into the blocked B (one block per
 * k2). Waits for the A tiles of its n3 group (all A tiles when ngrp = 1)
 * and counts itself in its group of 16 k1 (the C tiles' unit); every A
 * block is read by this tile alone, so once the first stage has read them
 * their L2 lines are dropped without a write-back. */
template <bool inverse, bool freq, class Pre>
__device__ __forceinline__ int *task_pb(const fgk_task &tk, const fgk_huge &hg, float2 *scratch, int *hcounters,
                                        int *err, uint32_t spin_limit, float2 *smem, int *failed, Pre &&pre)
{
	const fgk_plan3 *p = hg.p3;
	const int L1 = (int)hg.L1, L2 = (int)hg.L2, L3 = (int)hg.L3;
	const uint32_t L23 = (uint32_t)L2 * L3;
	const int k1g = (int)(tk.a / hg.nb3);
	const int k1b = k1g * 4, n3b = (int)(tk.a - (uint32_t)k1g * hg.nb3) * 4;
	const float2 *tq = (const float2 *)p->tq2;
	const uint32_t L = (uint32_t)L1 * L23;
	const float xL = 2.0f / (float)L;
	const float2 *A = scratch + hg.sa;
	float2 *B = scratch + hg.sb;
	const uint32_t grp = hg.ngrp > 1 ? (uint32_t)n3b >> 4 : 0;
	if (!tk_wait(hcounters + hg.cnt + grp, (int)(hg.na / hg.ngrp), err, failed, spin_limit))
		return nullptr;
	const uint32_t L1q = hg.nb / hg.nb3, L3q = hg.nb3;
	auto ld = [&](int n2, int lane) {
		const int k1 = k1b + (lane >> 2), n3 = n3b + (lane & 3);
		if (k1 >= L1 || n3 >= L3)
			return make_float2(0.f, 0.f);
		return __ldcg(A + tk_blk_a((uint32_t)k1, (uint32_t)n2, (uint32_t)n3, L1q, L3q));
	};
	auto st = [&](int j, int q, int nbf, int lane, float2 v) {
		const int k1 = k1b + (lane >> 2), n3 = n3b + (lane & 3);
		if (k1 >= L1 || n3 >= L3)
			return;
		const uint32_t m = (uint32_t)n3 * ((uint32_t)k1 + (uint32_t)L1 * (uint32_t)j);
		const float2 b = tk_wm(m, L, xL);
		const float2 w = q ? cmul(b, __ldg(tq + (uint32_t)n3 * (uint32_t)q)) : b;
		__stcg(B + tk_blk_b((uint32_t)(j + q * nbf), (uint32_t)n3, (uint32_t)k1, L1q, L3q), cmul(v, w));
	};
	auto discard = [&] {
		for (int n2 = (int)threadIdx.x; n2 < L2; n2 += (int)blockDim.x) {
			const float2 *a = A + tk_blk_a((uint32_t)k1b, (uint32_t)n2, (uint32_t)n3b, L1q, L3q);
			asm volatile("discard.global.L2 [%0], 128;" ::"l"(a) : "memory");
		}
	};
	tile_chain<false, Rows>(hg.code2, L2, 4, smem, smem + TK_SLOTS, (int)threadIdx.x,
	                        (int)blockDim.x, true, ld, st, [&] {
		                        discard();
		                        pre();
	                        });
	return hcounters + hg.cnt + hg.ngrp + (k1g >> 2);
}

/* C: 16 adjacent k1 of one k2, DFT_L3 over n3 from the blocked B (four
 * 32-byte sectors per n3), into X[k1 + L1 k2 + L1 L2 k3] (the modulation's
 * final step fused). Waits for the B tiles of its 16 k1: their 4 (fewer at
 * the end) k1 blocks times ceil(L3/4) n3 blocks. */
template <bool inverse, bool freq, class Pre>
__device__ __forceinline__ void task_pc(const fgk_task &tk, const fgk_huge &hg, float *out_base, float2 *scratch,
                                        const int *hcounters, int *err, uint32_t spin_limit, const fgk_product &prod,
                                        float2 *smem, int *failed, Pre &&pre)
{
	const fgk_plan3 *p = hg.p3;
	const int L1 = (int)hg.L1, L2 = (int)hg.L2, L3 = (int)hg.L3;
	const uint32_t L = (uint32_t)L1 * L2 * L3;
	const int k2 = (int)(tk.a / hg.nc1);
	const int k1b = (int)(tk.a - (uint32_t)k2 * hg.nc1) * 16;
	const float2 *B = scratch + hg.sb;
	float *o = out_base + hg.out_off;
	float2 *o2 = reinterpret_cast<float2 *>(o);
	const float2 *oa = (const float2 *)p->oa, *ob = (const float2 *)p->ob, *oc = (const float2 *)p->oc;
	const uint32_t L1q = hg.nb / hg.nb3, L3q = hg.nb3;
	const uint32_t kg = (uint32_t)k1b >> 4, nblk = min(4u, L1q - 4 * kg);
	if (!tk_wait(hcounters + hg.cnt + hg.ngrp + kg, (int)(nblk * L3q), err, failed, spin_limit))
		return;
	auto ld = [&](int n3, int lane) {
		const int k1 = k1b + lane;
		if (k1 >= L1)
			return make_float2(0.f, 0.f);
		return __ldcg(B + tk_blk_b((uint32_t)k2, (uint32_t)n3, (uint32_t)k1, L1q, L3q));
	};
	auto st = [&](int j, int q, int nbf, int lane, float2 v) {
		const int k1 = k1b + lane;
		if (k1 >= L1)
			return;
		const int k3 = j + q * nbf;
		const uint32_t m = (uint32_t)k1 + (uint32_t)L1 * ((uint32_t)k2 + (uint32_t)L2 * k3);
		if (!inverse) {
			if (prod.spec)
				v = tk_product(prod, m, v);
			if (!freq)
				__stcs(o2 + m, v);
			else if (m < ((L + 1) >> 1))
				__stcs(o2 + 2 * m, v);
			else
				__stcs(o2 + 2 * (L - 1 - m) + 1, conjf2(v));
		} else if (freq) {
			const float2 r = cmul(v, cmul(__ldg(oa + k1), cmul(__ldg(ob + k2), __ldg(oc + k3))));
			__stcs(o + m, r.x);
			__stcs(o + L + m, r.y);
		} else {
			__stcs(o2 + m, conjf2(v));
		}
	};
	tile_chain<false, Rows>(hg.code3, L3, 4, smem, smem + TK_SLOTS, (int)threadIdx.x,
	                        (int)blockDim.x, true, ld, st, pre);
}

/* One CTA: run tasks in claim order. Thread 0 claims the next task as the
 * current one starts, so the claim's round trip overlaps the work. One
 * instantiation per (direction, modulation): a batch has one of each. */
template <bool inverse, bool freq, int THREADS, int MINB, int BUFS>
__global__ void __launch_bounds__(THREADS, MINB)
    task_kernel(const fgk_task *__restrict__ tasks, uint32_t ntasks, const fgk_plan *__restrict__ plans,
                const fgk_rg_item *__restrict__ items, const fgk_big *__restrict__ bigs,
                const fgk_huge *__restrict__ huges, int *counters, int *hcounters, float2 *scratch,
                const float *in_base, float *out_base, int *err, uint32_t spin_limit, const fgk_product prod)
{
	extern __shared__ float2 smem[];
	__shared__ uint32_t cur;
	__shared__ __align__(16) fgk_task next_task;
	__shared__ int failed;
	uint32_t ahead = 0;
	/* thread 0 copies the record of the task claimed ahead into next_task
	 * (an asynchronous 16-byte copy) once the current task's first stage is
	 * done: the claim has returned by then, every thread has read
	 * next_task at the top of the loop, and the copy's round trip overlaps
	 * the rest of the task */
	bool copying = false;
	auto pre = [&] {
		if (threadIdx.x == 0 && !copying && ahead < ntasks) {
			asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
			                 (uint32_t)__cvta_generic_to_shared(&next_task)),
			             "l"(tasks + ahead)
			             : "memory");
			asm volatile("cp.async.commit_group;" ::: "memory");
			copying = true;
		}
	};
	if (threadIdx.x == 0) {
		cur = (uint32_t)atomicAdd(counters, 1);
		if (cur < ntasks)
			next_task = tasks[cur];
	}
	__syncthreads();
	for (;;) {
		const uint32_t c = cur;
		if (c >= ntasks)
			break;
		const fgk_task tk = next_task;
		int *count = nullptr; /* the tile's counter, released after the barrier below */
		if (threadIdx.x == 0)
			ahead = (uint32_t)atomicAdd(counters, 1);
		bool fits = true;
		if constexpr (BUFS == 1) {
			/* one buffer holds two-stage chains only */
			const uint64_t code = tk.kind == FGK_TASK_SMALL  ? plans[tk.ref].fwd.code
			                      : tk.kind == FGK_TASK_COLS ? bigs[tk.ref].code1
			                      : tk.kind == FGK_TASK_ROWS ? bigs[tk.ref].code2
			                      : tk.kind == FGK_TASK_PA   ? huges[tk.ref].code1
			                      : tk.kind == FGK_TASK_PB   ? huges[tk.ref].code2
			                                                 : huges[tk.ref].code3;
			fits = (code & 15) <= 2;
			if (!fits && threadIdx.x == 0)
				atomicExch(err, 1);
		}
		if (!fits) {
			/* refused, the error flag raised */
		} else if (tk.kind == FGK_TASK_SMALL)
			task_small<inverse, freq>(tk, plans, items, in_base, out_base, smem, pre);
		else if (tk.kind == FGK_TASK_COLS)
			count = task_cols<inverse, freq>(tk, bigs[tk.ref], in_base, scratch, counters + 1 + tk.ref, smem, pre);
		else if (tk.kind == FGK_TASK_ROWS)
			task_rows<inverse, freq>(tk, bigs[tk.ref], out_base, scratch, counters + 1 + tk.ref, err, spin_limit,
			                         prod, smem, &failed, pre);
		else if (tk.kind == FGK_TASK_PA)
			count = task_pa<inverse, freq>(tk, huges[tk.ref], in_base, scratch, hcounters, smem, pre);
		else if (tk.kind == FGK_TASK_PB)
			count = task_pb<inverse, freq>(tk, huges[tk.ref], scratch, hcounters, err, spin_limit, smem, &failed,
			                               pre);
		else
			task_pc<inverse, freq>(tk, huges[tk.ref], out_base, scratch, hcounters, err, spin_limit, prod, smem,
			                       &failed, pre);
		if (threadIdx.x == 0) {
			if (copying) {
				asm volatile("cp.async.wait_all;" ::: "memory");
				/* the next task's descriptor lines into L1 while the other
				 * warps finish this one */
				const fgk_task n = next_task;
				const void *d = n.kind == FGK_TASK_SMALL ? (const void *)(plans + n.ref)
				                : n.kind <= FGK_TASK_ROWS ? (const void *)(bigs + n.ref)
				                                           : (const void *)(huges + n.ref);
				asm volatile("prefetch.global.L1 [%0];" ::"l"(d));
				if (n.kind == FGK_TASK_SMALL)
					asm volatile("prefetch.global.L1 [%0];" ::"l"(items + n.a));
			} else if (ahead < ntasks) {
				next_task = tasks[ahead]; /* a ROWS wait that gave up skipped the copy */
			}
			copying = false;
			cur = ahead;
		}
		__syncthreads(); /* buffers are reused by the next task */
		if (threadIdx.x == 0 && count)
			tk_release(count);
	}
}

/* Launch of one instantiation (each lives in its own translation unit,
 * fgk_tasks_<direction><modulation>[w|s].cu, so that the twelve compile in
 * parallel); counters are already zeroed. */
template <bool inverse, bool freq, int THREADS, int MINB, int BUFS = 2>
int launch_tasks(uint32_t grid, const fgk_task *tasks, uint32_t ntasks, const fgk_plan *plans,
                 const fgk_rg_item *items, const fgk_big *bigs, const fgk_huge *huges, int *counters,
                 int *hcounters, float2 *scratch, const float *in_base, float *out_base, int *err, uint32_t spin_limit,
                 fgk_product prod, cudaStream_t stream)
{
	const size_t smem = (size_t)BUFS * TK_SLOTS * sizeof(float2);
	auto kern = task_kernel<inverse, freq, THREADS, MINB, BUFS>;
	cudaError_t e = cudaFuncSetAttribute((const void *)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e != cudaSuccess)
		return (int)e;
	kern<<<grid, THREADS, smem, stream>>>(tasks, ntasks, plans, items, bigs, huges, counters, hcounters, scratch, in_base,
	                                      out_base, err, spin_limit, prod);
	fgk_count_launch();
	return (int)cudaGetLastError();
}

} /* namespace fgk */

#define FGKT_LAUNCH_ARGS                                                                                 \
	uint32_t grid, const fgk_task *tasks, uint32_t ntasks, const fgk_plan *plans, const fgk_rg_item *items,     \
	    const fgk_big *bigs, const fgk_huge *huges, int *counters, int *hcounters, float2 *scratch,              \
	    const float *in_base, float *out_base, int *err, uint32_t spin_limit, fgk_product prod, cudaStream_t stream
#define FGKT_LAUNCH_PASS                                                                                 \
	grid, tasks, ntasks, plans, items, bigs, huges, counters, hcounters, scratch, in_base, out_base, err, spin_limit, \
	    prod, stream

/* Four-step transforms for sizes beyond the shared-memory limit.
 *
 * L = L1 * L2, input index n = L2 n1 + n2, output index k = k1 + L1 k2:
 *   X[k1 + L1 k2] = sum_n2 w_L2^{n2 k2} [ w_L^{n2 k1} sum_n1 x[L2 n1 + n2] w_L1^{n1 k1} ]
 * Pass 1 (columns): for each n2, DFT_L1 over n1, multiply by w_L^{n2 k1},
 *   store y[k1 L2 + n2] (row-major) in the work buffer.
 * Pass 2 (rows): for each k1, DFT_L2 over n2 of y[k1 L2 + n2], result
 *   X[k1 + L1 k2].
 * Each HBM array is read once and written once per pass (two passes per
 * transform). A CTA owns NL transforms of one
 * pass (NL adjacent columns, or NL adjacent rows) and keeps them lane-
 * interleaved in shared memory (element i of lane l at slot(i NL + l)), so
 * its HBM accesses are NL-element contiguous segments. Two forms, chosen by
 * the planner (fgk_plan4.emax): ping-pong tiles (fourstep_pp1/2: two
 * buffers, the chain run as the task kernel runs it, tile_chain) wherever
 * two buffers fit, else in place (fourstep_pass1/2: one buffer, each
 * stage's points read into registers, a barrier, then written back).
 *
 * The modulation edges of the reference are fused as in the resident path:
 *   FREQ_OFFSET_REAL forward: pass 1 loads c[n] = conj(x[n] + j x[L+n])
 *     e^{-j pi n/(2L)} (factor e^{-j pi n1/(2 L1)} e^{-j pi n2/(2L)});
 *     pass 2 writes the split X[2m] = W[m], X[2m+1] = conj W[L-1-m]: lanes
 *     NL/2..NL-1 hold the mirror rows L1-1-k1 of lanes 0..NL/2-1, so every
 *     output pair is produced by one CTA.
 *   inverse (both): pass 1 loads conj(W), FREQ_OFFSET_REAL mirror columns
 *     L2-1-n2 in the upper lanes; pass 2 applies the final step
 *     (src/fftset_mod_freqoffsetreal.c:974-1010, src/fftset_mod_cplx.c:212-239).
 * The twiddle w_L^{m}, m = n2 k1 < L, is T_hi[m >> s] * T_lo[m & (2^s - 1)]
 * with 2^s about sqrt(L): two FP64-generated tables rounded once to FP32. */
#include <cuda_runtime.h>
#include <stdint.h>
#include "fgk.h"
#include "fgk_codelets.cuh"
#include "fgk_pingpong.cuh"
#include "fgk_tasks.cuh"

namespace fgk {

/* pass-1 input modes and pass-2 output modes */
enum { FGK4_IN_FORWARD = 0, FGK4_IN_INVERSE = 1, FGK4_IN_NATURAL = 2 };
enum { FGK4_OUT_FORWARD = 0, FGK4_OUT_FINAL = 1, FGK4_OUT_KERNEL = 2, FGK4_OUT_PRODUCT = 3, FGK4_OUT_PRODUCT_CONJ = 4 };

#define FGK4_RADIX_SWITCH(r, CALL)                                  \
	switch (r) {                                                    \
	case 2: { constexpr int R_ = 2; CALL; } break;                  \
	case 3: { constexpr int R_ = 3; CALL; } break;                  \
	case 4: { constexpr int R_ = 4; CALL; } break;                  \
	case 5: { constexpr int R_ = 5; CALL; } break;                  \
	case 6: { constexpr int R_ = 6; CALL; } break;                  \
	case 8: { constexpr int R_ = 8; CALL; } break;                  \
	case 9: { constexpr int R_ = 9; CALL; } break;                  \
	case 10: { constexpr int R_ = 10; CALL; } break;                \
	case 12: { constexpr int R_ = 12; CALL; } break;                \
	case 15: { constexpr int R_ = 15; CALL; } break;                \
	default: { constexpr int R_ = 16; CALL; } break;                \
	}

/* A CTA's lane-interleaved tile: Lp points x NL lanes (NL a power of two). */
struct Tile4 {
	int     Lp, lshift, nl, T, tid;
	float2 *sm;
	__device__ __forceinline__ int slot(int i, int lane) const
	{
		const int x = (i << lshift) + lane;
		return x + (x >> 4);
	}
	__device__ __forceinline__ float2 ld(int i, int lane) const { return sm[slot(i, lane)]; }
	__device__ __forceinline__ void st(int i, int lane, float2 v) const { sm[slot(i, lane)] = v; }
};

/* One Stockham stage over all lanes: work item w = j * NL + lane. */
template <int R, int EMAX>
__device__ __forceinline__ void stage4(const Tile4 &t, const fgk_stage &st, const float2 *__restrict__ tw)
{
	constexpr int BM = (EMAX / R) > 0 ? EMAX / R : 1;
	const int nbf = t.Lp / R;
	const int items = nbf << t.lshift;
	const int ns = (int)st.ns;
	float2 v[BM][R];
#pragma unroll
	for (int b = 0; b < BM; b++) {
		const int w = t.tid + b * t.T;
		if (w < items) {
			const int j = w >> t.lshift, lane = w & (t.nl - 1);
#pragma unroll
			for (int p = 0; p < R; p++)
				v[b][p] = t.ld(j + p * nbf, lane);
		}
	}
	__syncthreads();
#pragma unroll
	for (int b = 0; b < BM; b++) {
		const int w = t.tid + b * t.T;
		if (w < items) {
			const int j = w >> t.lshift, lane = w & (t.nl - 1);
			const int k = j % ns;
			if (ns > 1) {
				const float2 *tp = tw + st.tw_off + k * (R - 1);
#pragma unroll
				for (int p = 1; p < R; p++)
					v[b][p] = cmul(v[b][p], __ldg(tp + p - 1));
			}
			Radix<R>::run(v[b]);
			const int base = (j - k) * R + k;
#pragma unroll
			for (int q = 0; q < R; q++)
				t.st(base + q * ns, lane, v[b][q]);
		}
	}
	__syncthreads();
}

template <int EMAX>
__device__ __forceinline__ void run_chain4(const Tile4 &t, const fgk_chain *ch, const float2 *tw)
{
	const int n = (int)ch->nstages;
	for (int s = 0; s < n; s++) {
		const fgk_stage st = ch->st[s];
		FGK4_RADIX_SWITCH(st.radix, (stage4<R_, EMAX>(t, st, tw)));
	}
}

__device__ __forceinline__ float2 wl(const fgk_plan4 &p, uint64_t m)
{
	const float2 hi = __ldg((const float2 *)p.thi + (m >> p.tshift));
	const float2 lo = __ldg((const float2 *)p.tlo + (m & ((1u << p.tshift) - 1)));
	return cmul(hi, lo);
}

/* Which column/row a lane of CTA group `grp` holds. Plain passes: lane l of
 * group g is index g*NL + l. Mirrored passes (FREQ_OFFSET_REAL: forward pass
 * 2, inverse pass 1): lanes l < NL/2 hold index g*NL/2 + l of the first
 * ceil(len/2) indices, lanes l + NL/2 hold their mirrors len-1-index (the
 * middle index of an odd length is its own mirror). valid = false for lanes
 * past the end. */
__device__ __forceinline__ uint32_t lane_index(uint32_t grp, int lane, int nl, bool mirror, uint32_t len, bool &valid)
{
	if (!mirror) {
		const uint32_t i = grp * (uint32_t)nl + (uint32_t)lane;
		valid = i < len;
		return valid ? i : 0;
	}
	const int half = nl >> 1;
	const uint32_t base = grp * (uint32_t)half + (uint32_t)(lane < half ? lane : lane - half);
	valid = base < ((len + 1) >> 1);
	if (!valid)
		return 0;
	return lane < half ? base : len - 1 - base;
}

__host__ __device__ __forceinline__ uint32_t lane_groups(uint32_t len, int nl, bool mirror)
{
	return mirror ? (((len + 1) >> 1) + (nl >> 1) - 1) / (nl >> 1) : (len + nl - 1) / nl;
}

/* Pass 1's input element n = L2 n1 + n2 (mode: FGK4_IN_*), with the
 * FREQ_OFFSET_REAL modulation and pairing fused */
__device__ __forceinline__ float2 pass1_load(const fgk_plan4 &p, int mode, const float *x, uint64_t L, uint64_t n,
                                             uint32_t n1, uint32_t n2)
{
	const bool freq = p.modulation == FGK_MOD_FREQOFF;
	if (mode == FGK4_IN_NATURAL)
		return __ldcs(reinterpret_cast<const float2 *>(x) + n);
	if (mode != FGK4_IN_INVERSE) {
		if (freq) {
			const float2 m = cmul(__ldg((const float2 *)p.m1 + n1), __ldg((const float2 *)p.m2 + n2));
			return cmul(make_float2(__ldcs(x + n), -__ldcs(x + L + n)), m);
		}
		return __ldcs(reinterpret_cast<const float2 *>(x) + n);
	}
	const float2 *X = reinterpret_cast<const float2 *>(x);
	if (freq) /* conj(W[n]): W[n] = X[2n] (n < ceil(L/2)), conj X[2(L-1-n)+1] otherwise */
		return n < ((L + 1) >> 1) ? conjf2(__ldcs(X + 2 * n)) : __ldcs(X + 2 * (L - 1 - n) + 1);
	return conjf2(__ldcs(X + n));
}

/* Pass 2's output of bin m = k1 + L1 k2 in every mode but the FREQ_OFFSET_REAL
 * forward split (mode: FGK4_OUT_*) */
__device__ __forceinline__ void pass2_store(const fgk_plan4 &p, int mode, float *o, uint64_t L, uint64_t m,
                                            uint32_t k1, uint32_t k2, float2 v, const float *__restrict__ kern,
                                            const int32_t *__restrict__ kidx, int kvw)
{
	if (mode == FGK4_OUT_KERNEL) {
		/* spectrum bin m into the reference's kernel-buffer layout */
		const int ko = __ldg(kidx + m);
		o[ko] = v.x;
		o[ko + kvw] = v.y;
	} else if (mode == FGK4_OUT_PRODUCT || mode == FGK4_OUT_PRODUCT_CONJ) {
		/* conj(W K) (or conj(W conj K)), natural order, for the second half of a convolution */
		const int ko = __ldg(kidx + m);
		const float2 k = make_float2(__ldg(kern + ko), __ldg(kern + ko + kvw));
		__stcs(reinterpret_cast<float2 *>(o) + m, conjf2(mode == FGK4_OUT_PRODUCT ? cmul(v, k) : cmulc(v, k)));
	} else if (mode == FGK4_OUT_FORWARD) {
		__stcs(reinterpret_cast<float2 *>(o) + m, v);
	} else if (p.modulation == FGK_MOD_FREQOFF) {
		const float2 md = cmul(__ldg((const float2 *)p.n1 + k1), __ldg((const float2 *)p.n2 + k2));
		const float2 r = cmul(v, md);
		__stcs(o + m, r.x);
		__stcs(o + L + m, r.y);
	} else {
		__stcs(reinterpret_cast<float2 *>(o) + m, conjf2(v));
	}
}

/* Pass 1: columns. */
template <int EMAX>
__global__ void __launch_bounds__(512, 1) fourstep_pass1(const fgk_plan4 p, int mode, const float *in, float2 *work,
                                                          uint32_t count, size_t in_stride, size_t work_stride)
{
	extern __shared__ float2 smem[];
	const fgk_plan4 *dp = p.dev;
	Tile4 t;
	t.Lp = (int)p.L1;
	t.lshift = (int)p.lshift1;
	t.nl = 1 << t.lshift;
	t.T = blockDim.x;
	t.tid = threadIdx.x;
	t.sm = smem;
	const uint32_t L1 = p.L1, L2 = p.L2;
	const uint64_t L = (uint64_t)L1 * L2;
	const bool freq = p.modulation == FGK_MOD_FREQOFF;
	const bool inverse = mode == FGK4_IN_INVERSE;
	const bool mirror = freq && inverse;
	const uint32_t groups = lane_groups(L2, t.nl, mirror);
	const uint64_t tr = blockIdx.x / groups;
	const uint32_t grp = blockIdx.x - (uint32_t)(tr * groups);
	if (tr >= count)
		return;
	const float *x = in + tr * in_stride;
	float2 *y = work + tr * work_stride;

	const int items = (int)L1 << t.lshift;
	batched_copy<8>(items, t.tid, t.T, [&](int w) {
		const int n1 = w >> t.lshift, lane = w & (t.nl - 1);
		bool valid;
		const uint32_t n2 = lane_index(grp, lane, t.nl, mirror, L2, valid);
		return valid ? pass1_load(p, mode, x, L, (uint64_t)L2 * n1 + n2, (uint32_t)n1, n2) : make_float2(0.f, 0.f); },
	    [&](int w, float2 v) { t.st(w >> t.lshift, w & (t.nl - 1), v); });
	__syncthreads();
	run_chain4<EMAX>(t, &dp->c1, (const float2 *)p.tw1);
	for (int w = t.tid; w < items; w += t.T) {
		const int k1 = w >> t.lshift, lane = w & (t.nl - 1);
		bool valid;
		const uint32_t n2 = lane_index(grp, lane, t.nl, mirror, L2, valid);
		if (valid)
			__stcs(y + (uint64_t)k1 * L2 + n2, cmul(t.ld(k1, lane), wl(p, (uint64_t)n2 * (uint32_t)k1)));
	}
}

/* Pass 2: rows. */
template <int EMAX>
__global__ void __launch_bounds__(512, 1) fourstep_pass2(const fgk_plan4 p, int mode, const float2 *work, float *out,
                                                          uint32_t count, size_t work_stride, size_t out_stride,
                                                          const float *__restrict__ kern, const int32_t *__restrict__ kidx,
                                                          int kvw)
{
	extern __shared__ float2 smem[];
	const fgk_plan4 *dp = p.dev;
	Tile4 t;
	t.Lp = (int)p.L2;
	t.lshift = (int)p.lshift2;
	t.nl = 1 << t.lshift;
	t.T = blockDim.x;
	t.tid = threadIdx.x;
	t.sm = smem;
	const uint32_t L1 = p.L1, L2 = p.L2;
	const uint64_t L = (uint64_t)L1 * L2;
	const bool freq = p.modulation == FGK_MOD_FREQOFF;
	const bool forward = mode == FGK4_OUT_FORWARD;
	const bool mirror = freq && forward;
	const uint32_t groups = lane_groups(L1, t.nl, mirror);
	const uint64_t tr = blockIdx.x / groups;
	const uint32_t grp = blockIdx.x - (uint32_t)(tr * groups);
	if (tr >= count)
		return;
	const float2 *yin = work + tr * work_stride;
	float *o = out + tr * out_stride;
	const int half = t.nl >> 1;
	const int items = (int)L2 << t.lshift;
	/* consecutive threads read consecutive n2 of one row */
	batched_copy<8>(
	    items, t.tid, t.T,
	    [&](int w) {
		    const int lane = w / (int)L2, n2 = w - lane * (int)L2;
		    bool valid;
		    const uint32_t k1 = lane_index(grp, lane, t.nl, mirror, L1, valid);
		    return valid ? __ldcs(yin + (uint64_t)k1 * L2 + n2) : make_float2(0.f, 0.f);
	    },
	    [&](int w, float2 v) {
		    const int lane = w / (int)L2, n2 = w - lane * (int)L2;
		    t.st(n2, lane, v);
	    });
	__syncthreads();
	run_chain4<EMAX>(t, &dp->c2, (const float2 *)p.tw2);
	for (int w = t.tid; w < items; w += t.T) {
		const int k2 = w >> t.lshift, lane = w & (t.nl - 1);
		bool valid;
		const uint32_t k1 = lane_index(grp, lane, t.nl, mirror, L1, valid);
		if (!valid)
			continue;
		const uint64_t m = k1 + (uint64_t)L1 * k2;
		if (mirror) {
			if (lane >= half)
				continue;
			/* lane l + half holds row L1-1-k1: W[L-1-m] sits at its position L2-1-k2 */
			const uint64_t mm = L - 1 - m;
			const float2 a = t.ld(k2, lane);
			const float2 b = t.ld(L2 - 1 - k2, lane + half);
			float2 *X = reinterpret_cast<float2 *>(o);
			/* X[2i] = W[i] for i < ceil(L/2); otherwise W[i] = conj X[2(L-1-i)+1] */
			if (m < ((L + 1) >> 1))
				__stcs(X + 2 * m, a);
			else
				__stcs(X + 2 * mm + 1, conjf2(a));
			if (mm < ((L + 1) >> 1))
				__stcs(X + 2 * mm, b);
			else
				__stcs(X + 2 * m + 1, conjf2(b));
			continue;
		}
		pass2_store(p, mode, o, L, m, k1, (uint32_t)k2, t.ld(k2, lane), kern, kidx, kvw);
	}
}

/* ---- ping-pong tiles (plans with emax == 0) ------------------------------
 * The tile's chain runs as in the task kernel (tile_chain, fgk_tasks.cuh):
 * one butterfly per thread at a time between two padded shared-memory
 * buffers, twiddles computed, no register batches and so no spills. */

/* Pass 1: the first stage reads the input directly (the tile's NL columns
 * are NL-element segments of each row), the last stage multiplies by
 * w_L^{n2 k1} and writes the work buffer y[k1 L2 + n2]. */
__global__ void __launch_bounds__(512, 1) fourstep_pp1(const fgk_plan4 p, int mode, const float *in, float2 *work,
                                                        uint32_t count, size_t in_stride, size_t work_stride)
{
	extern __shared__ float2 smem[];
	const int ls = (int)p.lshift1, nl = 1 << ls;
	const uint32_t L1 = p.L1, L2 = p.L2;
	const uint64_t L = (uint64_t)L1 * L2;
	const bool mirror = p.modulation == FGK_MOD_FREQOFF && mode == FGK4_IN_INVERSE;
	const uint32_t groups = lane_groups(L2, nl, mirror);
	const uint64_t tr = blockIdx.x / groups;
	const uint32_t grp = blockIdx.x - (uint32_t)(tr * groups);
	if (tr >= count)
		return;
	const float *x = in + tr * in_stride;
	float2 *y = work + tr * work_stride;
	auto ld = [&](int n1, int lane) {
		bool valid;
		const uint32_t n2 = lane_index(grp, lane, nl, mirror, L2, valid);
		return valid ? pass1_load(p, mode, x, L, (uint64_t)L2 * (uint32_t)n1 + n2, (uint32_t)n1, n2)
		             : make_float2(0.f, 0.f);
	};
	auto st = [&](int j, int q, int nbf, int lane, float2 v) {
		bool valid;
		const uint32_t n2 = lane_index(grp, lane, nl, mirror, L2, valid);
		const uint32_t k1 = (uint32_t)(j + q * nbf);
		if (valid)
			__stcs(y + (uint64_t)k1 * L2 + n2, cmul(v, wl(p, (uint64_t)n2 * k1)));
	};
	tile_chain<false, Pad>(p.c1.code, (int)L1, ls, smem, smem + p.slots1, (int)threadIdx.x, (int)blockDim.x, true,
	                       ld, st, [] {});
}

/* Pass 2: the tile's rows are copied into the second buffer first (a warp
 * reads consecutive n2 of one row of the row-major work buffer), the first
 * stage reads them there and writes the first buffer, the last stage writes
 * the output directly. FREQ_OFFSET_REAL forward: lanes NL/2.. hold the
 * mirror rows, so both halves of every 16-byte bin pair come from this CTA. */
__global__ void __launch_bounds__(512, 1) fourstep_pp2(const fgk_plan4 p, int mode, const float2 *work, float *out,
                                                        uint32_t count, size_t work_stride, size_t out_stride,
                                                        const float *__restrict__ kern,
                                                        const int32_t *__restrict__ kidx, int kvw)
{
	extern __shared__ float2 smem[];
	const int ls = (int)p.lshift2, nl = 1 << ls;
	const uint32_t L1 = p.L1, L2 = p.L2;
	const uint64_t L = (uint64_t)L1 * L2;
	const bool mirror = p.modulation == FGK_MOD_FREQOFF && mode == FGK4_OUT_FORWARD;
	const uint32_t groups = lane_groups(L1, nl, mirror);
	const uint64_t tr = blockIdx.x / groups;
	const uint32_t grp = blockIdx.x - (uint32_t)(tr * groups);
	if (tr >= count)
		return;
	const float2 *yin = work + tr * work_stride;
	float *o = out + tr * out_stride;
	float2 *A = smem, *B = smem + p.slots2;
	const Pad ad{ls};
	batched_copy<8>(
	    (int)L2 << ls, (int)threadIdx.x, (int)blockDim.x,
	    [&](int w) {
		    const int lane = w / (int)L2, n2 = w - lane * (int)L2;
		    bool valid;
		    const uint32_t k1 = lane_index(grp, lane, nl, mirror, L1, valid);
		    return valid ? __ldcs(yin + (uint64_t)k1 * L2 + n2) : make_float2(0.f, 0.f);
	    },
	    [&](int w, float2 v) {
		    const int lane = w / (int)L2, n2 = w - lane * (int)L2;
		    B[ad.slot(n2, lane)] = v;
	    });
	__syncthreads();
	auto ld = [&](int n2, int lane) { return B[ad.slot(n2, lane)]; };
	auto st = [&](int j, int q, int nbf, int lane, float2 v) {
		bool valid;
		const uint32_t k1 = lane_index(grp, lane, nl, mirror, L1, valid);
		if (!valid)
			return;
		const uint32_t k2 = (uint32_t)(j + q * nbf);
		const uint64_t m = k1 + (uint64_t)L1 * k2;
		if (mirror) {
			/* X[2m] = W[m] for m < ceil(L/2); otherwise W[m] = conj X[2(L-1-m)+1] */
			float2 *X = reinterpret_cast<float2 *>(o);
			if (m < ((L + 1) >> 1))
				__stcs(X + 2 * m, v);
			else
				__stcs(X + 2 * (L - 1 - m) + 1, conjf2(v));
		} else {
			pass2_store(p, mode, o, L, m, k1, k2, v, kern, kidx, kvw);
		}
	};
	tile_chain<false, Pad>(p.c2.code, (int)L2, ls, A, B, (int)threadIdx.x, (int)blockDim.x, true, ld, st, [] {});
}

} /* namespace fgk */

static int launch_pass(const fgk_plan4 *p, int in_mode, int out_mode, float *out, const float *in, float *work,
                       uint32_t count, size_t in_stride, size_t out_stride, size_t work_stride, const float *kern,
                       const int32_t *kidx, int kvw, cudaStream_t stream)
{
	using namespace fgk;
	const bool freq = p->modulation == FGK_MOD_FREQOFF;
	const int nl1 = 1 << p->lshift1, nl2 = 1 << p->lshift2;
	const uint32_t g1 = lane_groups(p->L2, nl1, freq && in_mode == FGK4_IN_INVERSE);
	const uint32_t g2 = lane_groups(p->L1, nl2, freq && out_mode == FGK4_OUT_FORWARD);
	/* ping-pong tiles hold two buffers */
	const size_t sm1 = (size_t)p->slots1 * sizeof(float2) * (p->emax1 ? 1 : 2);
	const size_t sm2 = (size_t)p->slots2 * sizeof(float2) * (p->emax2 ? 1 : 2);
	auto k1 = p->emax1 == 0 ? fourstep_pp1 : p->emax1 > 16 ? fourstep_pass1<32> : fourstep_pass1<16>;
	auto k2 = p->emax2 == 0 ? fourstep_pp2 : p->emax2 > 16 ? fourstep_pass2<32> : fourstep_pass2<16>;
	cudaError_t e;
	if ((e = cudaFuncSetAttribute((const void *)k1, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm1)) != cudaSuccess)
		return (int)e;
	if ((e = cudaFuncSetAttribute((const void *)k2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2)) != cudaSuccess)
		return (int)e;
	const uint64_t b1 = (uint64_t)g1 * count, b2 = (uint64_t)g2 * count;
	if (b1 > 0x7fffffffull || b2 > 0x7fffffffull)
		return (int)cudaErrorInvalidValue;
	k1<<<(unsigned)b1, p->threads1, sm1, stream>>>(*p, in_mode, in, reinterpret_cast<float2 *>(work), count, in_stride,
	                                                 work_stride / 2);
	fgk_count_launch();
	if ((e = cudaGetLastError()) != cudaSuccess)
		return (int)e;
	k2<<<(unsigned)b2, p->threads2, sm2, stream>>>(*p, out_mode, reinterpret_cast<const float2 *>(work), out, count,
	                                                 work_stride / 2, out_stride, kern, kidx, kvw);
	fgk_count_launch();
	return (int)cudaGetLastError();
}

extern "C" int fgk_launch_fourstep(const fgk_plan4 *p, int op, float *out, const float *in, const float *kern,
                                   const int32_t *kidx, int kvw, float *work, uint32_t count, size_t in_stride,
                                   size_t out_stride, size_t work_stride, void *stream)
{
	using namespace fgk;
	cudaStream_t s = (cudaStream_t)stream;
	if (count == 0)
		return 0;
	switch (op) {
	case FGK_OP_FORWARD:
		return launch_pass(p, FGK4_IN_FORWARD, FGK4_OUT_FORWARD, out, in, work, count, in_stride, out_stride,
		                   work_stride, kern, kidx, kvw, s);
	case FGK_OP_INVERSE:
		return launch_pass(p, FGK4_IN_INVERSE, FGK4_OUT_FINAL, out, in, work, count, in_stride, out_stride,
		                   work_stride, kern, kidx, kvw, s);
	case FGK_OP_KERNEL:
		return launch_pass(p, FGK4_IN_FORWARD, FGK4_OUT_KERNEL, out, in, work, count, in_stride, out_stride,
		                   work_stride, kern, kidx, kvw, s);
	case FGK_OP_CONV:
	case FGK_OP_CORR: {
		/* DFT, conj(W K) in natural order into out, then a forward DFT of
		 * that (= conj of the inverse) with the final step: four passes */
		int rc = launch_pass(p, FGK4_IN_FORWARD, op == FGK_OP_CONV ? FGK4_OUT_PRODUCT : FGK4_OUT_PRODUCT_CONJ, out,
		                     in, work, count, in_stride, out_stride, work_stride, kern, kidx, kvw, s);
		if (rc)
			return rc;
		return launch_pass(p, FGK4_IN_NATURAL, FGK4_OUT_FINAL, out, out, work, count, out_stride, out_stride,
		                   work_stride, kern, kidx, kvw, s);
	}
	default:
		return (int)cudaErrorInvalidValue;
	}
}

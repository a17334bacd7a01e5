/* Compile-time ("static") resident kernels for the hot sizes (shared
 * templates; one translation unit per size instantiates them).
 *
 * Same algorithm as fgk_resident.cu (a Stockham chain whose first stage reads
 * HBM and whose last stage writes HBM, with the FREQ_OFFSET_REAL modulation
 * and the convolution's spectrum product fused in), but L, the radix chain,
 * the threads per transform T and the transforms per CTA G are template
 * constants, so every index, stride and division folds at compile time and
 * the register tiles are sized exactly.
 *
 * Execution model: a persistent grid; each CTA first stages the twiddles of
 * every stage, the modulation factors e^{-j pi i/(2L)} and (convolution) the
 * kernel spectrum in natural order into shared memory, then its G groups of
 * T threads loop over transforms. A group synchronises with __syncwarp when
 * T == 32 and with its own named barrier otherwise; groups never wait on
 * each other. Inputs are read with streaming loads and outputs written with
 * streaming stores (they are touched once).
 *
 * The host picks a static kernel when one is compiled for (modulation, L)
 * and plans the twiddle tables with the same chain (fgk_static_chain). */
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "fgk.h"
#include "fgk_codelets.cuh"
#include "fgk_serve.cuh"

namespace fgk {

/* MODE (low two bits): 0 in-place exchange buffer, direct HBM loads; 1
 * in-place with inputs double-buffered by bulk copies (TMA); 2 ping-pong
 * exchange buffers (out-of-place stages, one barrier per stage, one
 * butterfly at a time). MODE | 4 (direct-load modes only): group g hands
 * butterfly j to thread (j - 32 g) mod T instead of thread j. Warps go to
 * the SM's four schedulers by warp index mod 4, so when a stage has fewer
 * butterflies than threads (radix 16 of 1536 bins: 96 for 128 threads) the
 * idle warp is a different scheduler's in each group instead of always the
 * last one's. */
/* TWG_ (table flags): | 1 twiddles read from global memory (L1) instead of
 * shared; | 2 radix >= 8 stages read the twiddles of p = 1, 2, 4, 8 only and
 * form the others as products (fewer shared-memory reads, a few more
 * multiplies); | 4 (ping-pong, FREQ_OFFSET_REAL) the modulation factors of
 * the first and last stages from one table entry per butterfly times
 * compile-time constants instead of one entry per point. */
template <int MOD_, int L_, int T_, int G_, int TWG_, int MODE_, int... Rs> struct SCfg {
	static constexpr int MOD = MOD_;
	static constexpr bool TWG = (TWG_ & 1) != 0;
	static constexpr bool TWR = (TWG_ & 2) != 0;
	static constexpr bool MODC = (TWG_ & 4) != 0;
	static_assert(!(MODC && (MODE_ & 3) != 2), "constant modulation is a ping-pong form");
	static constexpr int MODE = MODE_ & 3;
	static constexpr bool TMA = MODE == 1;
	static constexpr bool PP = MODE == 2;
	static constexpr bool ROT = (MODE_ & 4) != 0;
	static_assert(!(ROT && MODE == 1), "rotation is for the direct-load modes");
	/* work index of thread t of group g (a bijection of 0..T-1) */
	static __device__ __forceinline__ int wt(int t, int g) { return ROT ? (t + 32 * g) % T : t; }
	static constexpr int L = L_;
	static constexpr int T = T_;
	static constexpr int G = G_;
	static constexpr int N = sizeof...(Rs);
	static constexpr int R[N] = {Rs...};
	/* forward chain */
	static __host__ __device__ constexpr int fr(int s) { return R[s]; }
	static __host__ __device__ constexpr int fns(int s) { return s == 0 ? 1 : fns(s - 1) * R[s - 1]; }
	/* reversed chain (run after the spectrum product) */
	static __host__ __device__ constexpr int ir(int s) { return R[N - 1 - s]; }
	static __host__ __device__ constexpr int ins(int s) { return s == 0 ? 1 : ins(s - 1) * R[N - s]; }
	/* twiddle entries of a stage, in the host's order: forward stages
	 * 1..N-1, then reversed stages 1..N-1 (stages with ns == 1 have none) */
	static __host__ __device__ constexpr int ftw_size(int s) { return s == 0 ? 0 : (fr(s) - 1) * fns(s); }
	static __host__ __device__ constexpr int itw_size(int s) { return s == 0 ? 0 : (ir(s) - 1) * ins(s); }
	static __host__ __device__ constexpr int ftw_off(int s) { return s == 0 ? 0 : ftw_off(s - 1) + ftw_size(s - 1); }
	/* a palindromic chain is its own reverse: the reversed stages read the
	 * forward stages' twiddles (the host's table holds both; only the
	 * forward half is staged) */
	static __host__ __device__ constexpr bool pal(int s = 0) { return s >= N || (R[s] == R[N - 1 - s] && pal(s + 1)); }
	static constexpr bool PAL = pal();
	static __host__ __device__ constexpr int itw_off_full(int s)
	{
		return s == 0 ? ftw_off(N) : itw_off_full(s - 1) + itw_size(s - 1);
	}
	static __host__ __device__ constexpr int itw_off(int s) { return PAL ? ftw_off(s) : itw_off_full(s); }
	static constexpr int TW_TOTAL = PAL ? ftw_off(N) : itw_off_full(N);
	static constexpr int SLOTS = L + L / 16 + 1; /* padded exchange buffer */
	/* modulation factors staged in shared memory: all L, or with constant
	 * modulation only those of the first and last stages' butterflies
	 * (mods[j], j < L / R for R the first and last radices) */
	static constexpr int NMODS =
	    MOD == FGK_MOD_FREQOFF ? (MODC ? L / (R[0] < R[N - 1] ? R[0] : R[N - 1]) : L) : 0;
	static __host__ __device__ constexpr int slot(int i) { return i + (i >> 4); }
};

template <class C> __device__ __forceinline__ void gsync(int g)
{
	if constexpr (C::T == 32) {
		__syncwarp();
	} else {
		asm volatile("bar.sync %0, %1;" ::"r"(g + 1), "r"(C::T) : "memory");
	}
}

__device__ __forceinline__ float ldcs(const float *p) { return __ldcs(p); }
__device__ __forceinline__ float2 ldcs2(const float2 *p) { return __ldcs(p); }
__device__ __forceinline__ void stcs(float *p, float v) { __stcs(p, v); }
__device__ __forceinline__ void stcs2(float2 *p, float2 v) { __stcs(p, v); }

/* Input twiddles of butterfly k of a stage (R, NS): v[p] *= w^{p k} for
 * p = 1..R-1, the table holding entry (p-1, k) at tws[(p-1) NS + k] (shared)
 * or tws[k (R-1) + p-1] (global, TWG). With TWR and R >= 8 only the entries
 * of p = 1, 2, 4, 8 are read (twiddle_powers, fgk_codelets.cuh). */
template <class C, int R, int NS>
__device__ __forceinline__ void twiddle_in(float2 (&v)[R], const float2 *tws, int k)
{
	auto entry = [&](int p) { return C::TWG ? __ldg(tws + k * (R - 1) + (p - 1)) : tws[(p - 1) * NS + k]; };
	if constexpr (C::TWR && R >= 8) {
		float2 w[R];
		twiddle_powers<R>(w, entry);
#pragma unroll
		for (int p = 1; p < R; p++)
			v[p] = cmul(v[p], w[p]);
	} else {
#pragma unroll
		for (int p = 1; p < R; p++)
			v[p] = cmul(v[p], entry(p));
	}
}

/* Tile of one stage: NB butterflies of radix R per thread. */
template <class C, int R> struct Tile {
	static constexpr int NBF = C::L / R;
	static constexpr int NB = (NBF + C::T - 1) / C::T;
	static constexpr bool FULL = (NBF % C::T) == 0;
	float2 v[NB][R];

	__device__ __forceinline__ static bool live(int tid, int b) { return FULL || tid + b * C::T < NBF; }

	template <class Ld> __device__ __forceinline__ void load(int tid, Ld &&ld)
	{
#pragma unroll
		for (int b = 0; b < NB; b++) {
			const int j = tid + b * C::T;
			if (live(tid, b)) {
#pragma unroll
				for (int p = 0; p < R; p++)
					v[b][p] = ld(j + p * NBF);
			}
		}
	}

	/* twiddle (table [p-1][k] in shared memory, k = j mod NS) + DFT_R */
	template <int NS> __device__ __forceinline__ void butterfly(int tid, const float2 *tws)
	{
#pragma unroll
		for (int b = 0; b < NB; b++) {
			const int j = tid + b * C::T;
			if (live(tid, b)) {
				if constexpr (NS > 1)
					twiddle_in<C, R, NS>(v[b], tws, j % NS);
				Radix<R>::run(v[b]);
			}
		}
	}

	/* Stockham scatter of stage (R, NS): output q of butterfly j goes to
	 * (j - j mod NS) R + j mod NS + q NS */
	template <int NS, class St> __device__ __forceinline__ void store(int tid, St &&st)
	{
#pragma unroll
		for (int b = 0; b < NB; b++) {
			const int j = tid + b * C::T;
			if (live(tid, b)) {
				const int k = j % NS;
				const int base = (j - k) * R + k;
#pragma unroll
				for (int q = 0; q < R; q++)
					st(base + q * NS, v[b][q]);
			}
		}
	}
};

/* shared-memory exchange helpers for one group */
template <class C> struct Ex {
	float2 *sm;
	__device__ __forceinline__ float2 operator()(int i) const { return sm[C::slot(i)]; }
	__device__ __forceinline__ void put(int i, float2 v) const { sm[C::slot(i)] = v; }
};

/* forward-chain stages 1..E-1 (smem -> smem) */
template <class C, int S, int E>
__device__ __forceinline__ void fwd_mid(int tid, int g, const Ex<C> &ex, const float2 *tws)
{
	if constexpr (S < E) {
		constexpr int R = C::fr(S), NS = C::fns(S);
		Tile<C, R> t;
		t.load(tid, ex);
		gsync<C>(g);
		t.template butterfly<NS>(tid, tws + C::ftw_off(S));
		t.template store<NS>(tid, [&](int i, float2 v) { ex.put(i, v); });
		gsync<C>(g);
		fwd_mid<C, S + 1, E>(tid, g, ex, tws);
	}
}

/* reversed-chain stages S..E-1 (smem -> smem) */
template <class C, int S, int E>
__device__ __forceinline__ void inv_mid(int tid, int g, const Ex<C> &ex, const float2 *tws)
{
	if constexpr (S < E) {
		constexpr int R = C::ir(S), NS = C::ins(S);
		Tile<C, R> t;
		t.load(tid, ex);
		gsync<C>(g);
		t.template butterfly<NS>(tid, tws + C::itw_off(S));
		t.template store<NS>(tid, [&](int i, float2 v) { ex.put(i, v); });
		gsync<C>(g);
		inv_mid<C, S + 1, E>(tid, g, ex, tws);
	}
}

/* Copy the twiddles of every stage from the plan's global table (layout
 * [k][p-1] per stage) into shared memory (layout [p-1][k], so that threads
 * with consecutive k read consecutive words). */
template <class C, int S>
__device__ __forceinline__ void stage_twiddles(float2 *tws, const float2 *__restrict__ gtw)
{
	if constexpr (S < (C::PAL ? C::N : 2 * C::N)) {
		constexpr bool FW = S < C::N;
		constexpr int ST = FW ? S : S - C::N;
		if constexpr (ST > 0) {
			constexpr int R = FW ? C::fr(ST) : C::ir(ST);
			constexpr int NS = FW ? C::fns(ST) : C::ins(ST);
			constexpr int OFF = FW ? C::ftw_off(ST) : C::itw_off(ST);
			constexpr int NE = (R - 1) * NS;
			for (int e = threadIdx.x; e < NE; e += blockDim.x) {
				const int k = e / (R - 1), q = e - k * (R - 1);
				tws[OFF + q * NS + k] = __ldg(gtw + OFF + e);
			}
		}
		stage_twiddles<C, S + 1>(tws, gtw);
	}
}

struct StaticArgs {
	float       *out;
	const float *in;
	const float *kern;
	uint32_t     count;
	size_t       in_stride, out_stride;
	int         *err; /* set to 1 when a bounded wait gives up (TMA mode) */
};

/* ---- TMA (cp.async.bulk) + mbarrier helpers ---------------------------- */
#define FGK_SPIN_LIMIT (1u << 20) /* x 1 us suspend hint: about a second */

__device__ __forceinline__ uint32_t smem_u32(const void *ptr) { return (uint32_t)__cvta_generic_to_shared(ptr); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

/* one 1-D bulk copy global -> shared, completion counted on `bar` */
__device__ __forceinline__ void tma_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
	                 smem_u32(dst)),
	             "l"(src), "r"(bytes), "r"(smem_u32(bar))
	             : "memory");
}

/* bounded wait for phase `parity` of `bar`; false when it gave up */
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity)
{
	for (uint32_t it = 0; it < FGK_SPIN_LIMIT; it++) {
		uint32_t ok;
		asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
		             "selp.u32 %0, 1, 0, p;\n\t}"
		             : "=r"(ok)
		             : "r"(smem_u32(bar)), "r"(parity), "r"(1000u)
		             : "memory");
		if (ok)
			return true;
	}
	return false;
}

/* ---- one transform ----------------------------------------------------- */
/* First-stage loader: the modulated sequence (FORWARD/CONV) or conj(W)
 * (INVERSE) at natural index i, from HBM (x is a global pointer) or from the
 * block's shared staging copy (x is a shared pointer). */
template <class C, int OP, bool SHARED_IN> struct FirstLoad {
	const float  *x;
	const float2 *mods;
	__device__ __forceinline__ float ld(int i) const
	{
		if constexpr (SHARED_IN)
			return x[i];
		else
			return ldcs(x + i);
	}
	__device__ __forceinline__ float2 ld2(int i) const
	{
		const float2 *x2 = reinterpret_cast<const float2 *>(x);
		if constexpr (SHARED_IN)
			return x2[i];
		else
			return ldcs2(x2 + i);
	}
	__device__ __forceinline__ float2 operator()(int i) const
	{
		constexpr int L = C::L;
		if constexpr (OP == FGK_OP_INVERSE) {
			if constexpr (C::MOD == FGK_MOD_FREQOFF)
				return i < ((L + 1) >> 1) ? conjf2(ld2(2 * i)) : ld2(2 * (L - 1 - i) + 1);
			else
				return conjf2(ld2(i));
		} else {
			if constexpr (C::MOD == FGK_MOD_FREQOFF)
				return cmul(make_float2(ld(i), -ld(L + i)), mods[i]);
			else
				return ld2(i);
		}
	}
};

/* Runs one transform. `first` feeds stage 0; when stage 0 reads the same
 * shared buffer it writes (TMA mode), IN_PLACE adds the barrier between its
 * loads and stores. Ends with the group barrier that frees `ex`. */
template <class C, int OP, bool IN_PLACE, class First>
__device__ __forceinline__ void transform(int tid, int g, const Ex<C> &ex, const First &first, float *y,
                                          const float2 *tws, const float2 *mods, const float2 *ks)
{
	constexpr int L = C::L, N = C::N;
	constexpr bool FREQ = C::MOD == FGK_MOD_FREQOFF;
	constexpr bool CONV = OP == FGK_OP_CONV || OP == FGK_OP_CORR;
	auto out_final = [&](int i, float2 u) {
		if constexpr (FREQ) {
			const float2 r = cmul(u, mods[i]);
			stcs(y + i, r.x);
			stcs(y + L + i, r.y);
		} else {
			stcs2(reinterpret_cast<float2 *>(y) + i, conjf2(u));
		}
	};
	auto exput = [&](int i, float2 v) { ex.put(i, v); };
	{
		constexpr int R = C::fr(0);
		Tile<C, R> t0;
		t0.load(tid, first);
		if constexpr (IN_PLACE)
			gsync<C>(g);
		t0.template butterfly<1>(tid, tws);
		t0.template store<1>(tid, exput);
		gsync<C>(g);
	}
	fwd_mid<C, 1, N - 1>(tid, g, ex, tws);
	if constexpr (CONV) {
		static_assert(N >= 2, "static conv needs two or more stages");
		{
			/* last forward stage + product + first reversed stage */
			constexpr int R = C::fr(N - 1), NS = C::fns(N - 1);
			Tile<C, R> t;
			t.load(tid, ex);
			gsync<C>(g);
			t.template butterfly<NS>(tid, tws + C::ftw_off(N - 1));
#pragma unroll
			for (int b = 0; b < Tile<C, R>::NB; b++) {
				const int j = tid + b * C::T;
				if (Tile<C, R>::live(tid, b)) {
#pragma unroll
					for (int q = 0; q < R; q++)
						t.v[b][q] = conjf2(cmul(t.v[b][q], ks[j + q * (L / R)]));
					Radix<R>::run(t.v[b]);
				}
			}
			t.template store<1>(tid, exput);
			gsync<C>(g);
		}
		inv_mid<C, 1, N - 1>(tid, g, ex, tws);
		{
			constexpr int R = C::ir(N - 1), NS = C::ins(N - 1);
			Tile<C, R> t;
			t.load(tid, ex);
			t.template butterfly<NS>(tid, tws + C::itw_off(N - 1));
			t.template store<NS>(tid, out_final);
		}
	} else {
		constexpr int R = C::fr(N - 1), NS = C::fns(N - 1);
		Tile<C, R> t;
		t.load(tid, ex);
		if constexpr (OP == FGK_OP_FORWARD && FREQ)
			gsync<C>(g); /* results go back to shared memory */
		t.template butterfly<NS>(tid, tws + C::ftw_off(N - 1));
		if constexpr (OP == FGK_OP_INVERSE) {
			t.template store<NS>(tid, out_final);
		} else if constexpr (!FREQ) {
			t.template store<NS>(tid, [&](int i, float2 v) { stcs2(reinterpret_cast<float2 *>(y) + i, v); });
		} else {
			t.template store<NS>(tid, exput);
			gsync<C>(g);
			/* X[2m] = W[m], X[2m+1] = conj W[L-1-m] */
			if ((reinterpret_cast<uintptr_t>(y) & 15) == 0) {
				float4 *y4 = reinterpret_cast<float4 *>(y);
				for (int m = tid; m < L / 2; m += C::T) {
					const float2 w0 = ex(m), w1 = ex(L - 1 - m);
					__stcs(y4 + m, make_float4(w0.x, w0.y, w1.x, -w1.y));
				}
			} else {
				float2 *y2 = reinterpret_cast<float2 *>(y);
				for (int m = tid; m < L / 2; m += C::T) {
					const float2 w0 = ex(m), w1 = ex(L - 1 - m);
					stcs2(y2 + 2 * m, w0);
					stcs2(y2 + 2 * m + 1, conjf2(w1));
				}
			}
		}
	}
	gsync<C>(g); /* the exchange buffer is reused by the next transform */
}

/* ---- per-CTA tables -----------------------------------------------------
 * The batched kernels are launched with programmatic stream serialisation
 * (fgk_launch_static): a CTA lets the next launch on the stream be
 * scheduled as soon as it starts, stages the plan's twiddles and
 * modulation factors (written when the plan was made, never by a kernel),
 * then waits for the launches before it on the stream to finish
 * (griddepcontrol.wait, which returns at once when there are none) before
 * it reads anything a kernel may have written: the kernel buffer here, the
 * input blocks after. The next step's launch and table staging overlap the
 * tail of this one. */
template <class C, int OP>
__device__ __forceinline__ void stage_tables(const fgk_plan &p, const StaticArgs &a, float2 *smem, float2 *mods,
                                             float2 *ks)
{
	constexpr int L = C::L;
	asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
	if constexpr (!C::TWG)
		stage_twiddles<C, 1>(smem, (const float2 *)p.tw);
	if constexpr (C::MOD == FGK_MOD_FREQOFF) {
		const float2 *gm = (const float2 *)p.modtw;
		for (int i = threadIdx.x; i < C::NMODS; i += blockDim.x)
			mods[i] = __ldg(gm + i);
	}
	asm volatile("griddepcontrol.wait;" ::: "memory");
	if constexpr (OP == FGK_OP_CONV || OP == FGK_OP_CORR) {
		const int32_t *kidx = p.kidx;
		const int kvw = (int)p.kvw;
		for (int i = threadIdx.x; i < L; i += blockDim.x) {
			const int o = __ldg(kidx + i);
			float2 k = make_float2(__ldg(a.kern + o), __ldg(a.kern + o + kvw));
			if (OP == FGK_OP_CORR)
				k.y = -k.y;
			ks[i] = k;
		}
	}
}

template <class C, int OP> struct Layout {
	static constexpr bool FREQ = C::MOD == FGK_MOD_FREQOFF;
	static constexpr bool CONV = OP == FGK_OP_CONV || OP == FGK_OP_CORR;
	static constexpr size_t TW = C::TWG ? 0 : (size_t)C::TW_TOTAL; /* float2 */
	static constexpr size_t MODS = (size_t)C::NMODS;
	static constexpr size_t KS = CONV ? C::L : 0;
	static constexpr size_t TABLES = TW + MODS + KS;
	/* TMA mode: per group two buffers, each holding a raw input block (2L
	 * floats) or the padded exchange buffer, whichever is larger; 16-byte
	 * multiples so every bulk copy lands aligned */
	static constexpr size_t BUF = ((C::SLOTS > C::L ? C::SLOTS : C::L) + 1) & ~(size_t)1; /* float2 */
	static constexpr size_t DIRECT_BYTES = sizeof(float2) * (TABLES + (size_t)C::G * C::SLOTS);
	static constexpr size_t PP_BYTES = sizeof(float2) * (TABLES + 2 * (size_t)C::G * C::SLOTS);
	static constexpr size_t TMA_BYTES = sizeof(float2) * (((TABLES + 1) & ~(size_t)1) + 2 * (size_t)C::G * BUF) +
	                                    2 * (size_t)C::G * sizeof(uint64_t);
};

/* ---- kernels ------------------------------------------------------------ */
template <class C, int OP>
__global__ void __launch_bounds__(C::T *C::G, 1) static_kernel(const fgk_plan p, StaticArgs a)
{
	extern __shared__ float2 smem[];
	using Lay = Layout<C, OP>;
	const float2 *tws = C::TWG ? (const float2 *)p.tw : smem;
	float2 *mods = smem + Lay::TW;
	float2 *ks = mods + Lay::MODS;
	float2 *exb = ks + Lay::KS;
	stage_tables<C, OP>(p, a, smem, mods, ks);
	__syncthreads();

	const int g = threadIdx.x / C::T;
	const int tid = C::wt((int)threadIdx.x - g * C::T, g);
	const Ex<C> ex{exb + (size_t)g * C::SLOTS};
	for (uint64_t t = (uint64_t)blockIdx.x * C::G + g; t < a.count; t += (uint64_t)gridDim.x * C::G) {
		const FirstLoad<C, OP, false> first{a.in + t * a.in_stride, mods};
		transform<C, OP, false>(tid, g, ex, first, a.out + t * a.out_stride, tws, mods, ks);
	}
}

/* TMA mode: each group double-buffers its input blocks with bulk copies
 * (one elected thread issues them), so the next block streams in while the
 * current one is transformed; the block's staging buffer then serves as its
 * exchange buffer. Requires 16-byte aligned blocks. */
template <class C, int OP>
__global__ void __launch_bounds__(C::T *C::G, 1) static_kernel_tma(const fgk_plan p, StaticArgs a)
{
	extern __shared__ float2 smem[];
	using Lay = Layout<C, OP>;
	constexpr uint32_t BYTES = 2u * C::L * sizeof(float);
	const float2 *tws = C::TWG ? (const float2 *)p.tw : smem;
	float2 *mods = smem + Lay::TW;
	float2 *ks = mods + Lay::MODS;
	float2 *bufs = smem + ((Lay::TABLES + 1) & ~(size_t)1);
	uint64_t *bars = reinterpret_cast<uint64_t *>(bufs + 2 * (size_t)C::G * Lay::BUF);
	__shared__ int grp_err[C::G];

	const int g = threadIdx.x / C::T;
	const int tid = threadIdx.x - g * C::T;
	if (threadIdx.x < 2 * C::G)
		mbar_init(bars + threadIdx.x, 1);
	if (threadIdx.x < C::G)
		grp_err[threadIdx.x] = 0;
	mbar_fence_init();
	stage_tables<C, OP>(p, a, smem, mods, ks);
	__syncthreads();

	const uint64_t step = (uint64_t)gridDim.x * C::G;
	uint64_t t = (uint64_t)blockIdx.x * C::G + g;
	/* group g owns buffers 2g, 2g+1 and barriers 2g, 2g+1 (computed, not
	 * held in arrays: a runtime-indexed array would live in local memory) */
	float2 *const gbuf = bufs + (size_t)(2 * g) * Lay::BUF;
	uint64_t *const gbar = bars + 2 * g;
	uint32_t pending = 0; /* bit b: copy into buffer b issued, not yet waited for */
	if (t < a.count) {
		if (tid == 0)
			tma_load(gbuf, a.in + t * a.in_stride, BYTES, gbar);
		pending = 1;
	}
	uint32_t it = 0;
	for (; t < a.count; t += step, it++) {
		const uint32_t b = it & 1;
		const bool ok = mbar_wait(gbar + b, (it >> 1) & 1);
		if (!ok) {
			grp_err[g] = 1;
			if (a.err)
				atomicExch(a.err, 1);
		}
		pending = ok ? (pending & ~(1u << b)) : pending; /* a copy that never signalled is drained below */
		if (t + step < a.count) {
			/* the other buffer served the previous block, released by its final barrier */
			if (tid == 0) {
				fence_proxy_async();
				tma_load(gbuf + (size_t)(b ^ 1) * Lay::BUF, a.in + (t + step) * a.in_stride, BYTES, gbar + (b ^ 1));
			}
			pending |= 1u << (b ^ 1);
		}
		gsync<C>(g);
		if (grp_err[g])
			break;
		float2 *cur = gbuf + (size_t)b * Lay::BUF;
		const Ex<C> ex{cur};
		const FirstLoad<C, OP, true> first{reinterpret_cast<const float *>(cur), mods};
		transform<C, OP, true>(tid, g, ex, first, a.out + t * a.out_stride, tws, mods, ks);
	}
	/* drain copies still in flight (only after a failed wait) */
	for (uint32_t b = 0; b < 2; b++)
		if (pending & (1u << b))
			mbar_wait(gbar + b, ((it + (b != (it & 1))) >> 1) & 1);
}

/* ---- ping-pong mode ------------------------------------------------------
 * One stage = read buffer `src`, write buffer `dst`; butterflies are processed
 * one at a time (register tile = one radix), and the only barrier is the one
 * after the stage's stores. */
template <class C, int R, int NS, class Ld, class St>
__device__ __forceinline__ void pp_stage(int tid, const float2 *tws, Ld &&ld, St &&st)
{
	constexpr int NBF = C::L / R;
	constexpr int NB = (NBF + C::T - 1) / C::T;
	constexpr bool FULL = (NBF % C::T) == 0;
#pragma unroll 2
	for (int b = 0; b < NB; b++) {
		const int j = tid + b * C::T;
		if (FULL || j < NBF) {
			float2 v[R];
#pragma unroll
			for (int p = 0; p < R; p++)
				v[p] = ld(j + p * NBF);
			const int k = j % NS;
			if constexpr (NS > 1)
				twiddle_in<C, R, NS>(v, tws, k);
			Radix<R>::run(v);
			const int base = (j - k) * R + k;
#pragma unroll
			for (int q = 0; q < R; q++)
				st(base + q * NS, v[q]);
		}
	}
}

/* Constant-modulation forms (MODC, FREQ_OFFSET_REAL). The factor of point
 * i is e^{-j pi i / (2L)}; the first stage's butterfly j reads the points
 * j + p L/R and the last stage's butterfly j writes the points j + q L/R
 * (its ns is L/R), so every factor is mods[j] e^{-j pi p / (2R)}: one table
 * read per butterfly and compile-time constants. */
template <class C, int OP, class First, class St>
__device__ __forceinline__ void pp_first_modc(int tid, const First &first, const float2 *mods, St &&st)
{
	constexpr int L = C::L, R = C::fr(0), NBF = L / R;
	constexpr int NB = (NBF + C::T - 1) / C::T;
	constexpr bool FULL = (NBF % C::T) == 0;
#pragma unroll 2
	for (int b = 0; b < NB; b++) {
		const int j = tid + b * C::T;
		if (FULL || j < NBF) {
			float2 v[R];
#pragma unroll
			for (int p = 0; p < R; p++)
				v[p] = make_float2(first.ld(j + p * NBF), -first.ld(L + j + p * NBF));
			mod_steps<R>(v, mods[j]);
			Radix<R>::run(v);
#pragma unroll
			for (int q = 0; q < R; q++)
				st(j * R + q, v[q]);
		}
	}
}

template <class C, int R, int NS>
__device__ __forceinline__ void pp_last_modc(int tid, const float2 *tws, const Ex<C> &src, float *y,
                                             const float2 *mods)
{
	constexpr int L = C::L, NBF = L / R;
	static_assert(NS == NBF, "the last stage's ns is L/R");
	constexpr int NB = (NBF + C::T - 1) / C::T;
	constexpr bool FULL = (NBF % C::T) == 0;
#pragma unroll 2
	for (int b = 0; b < NB; b++) {
		const int j = tid + b * C::T;
		if (FULL || j < NBF) {
			float2 v[R];
#pragma unroll
			for (int p = 0; p < R; p++)
				v[p] = src(j + p * NBF);
			twiddle_in<C, R, NS>(v, tws, j);
			Radix<R>::run(v);
			mod_steps<R>(v, mods[j]);
#pragma unroll
			for (int q = 0; q < R; q++) {
				stcs(y + j + q * NBF, v[q].x);
				stcs(y + L + j + q * NBF, v[q].y);
			}
		}
	}
}

/* forward stages S..E-1 between the two buffers; returns via the template
 * the buffer parity after the last one (buffers alternate every stage) */
template <class C, int S, int E>
__device__ __forceinline__ void pp_fwd(int tid, int g, float2 *buf0, float2 *buf1, const float2 *tws)
{
	if constexpr (S < E) {
		constexpr int R = C::fr(S), NS = C::fns(S);
		/* stage S reads buffer (S-1)&1 ... stage 0 wrote buffer 0 */
		const Ex<C> src{((S - 1) & 1) ? buf1 : buf0}, dst{((S - 1) & 1) ? buf0 : buf1};
		pp_stage<C, R, NS>(tid, tws + C::ftw_off(S), src, [&](int i, float2 v) { dst.put(i, v); });
		gsync<C>(g);
		pp_fwd<C, S + 1, E>(tid, g, buf0, buf1, tws);
	}
}

/* reversed-chain stages S..E-1; the fused stage (global index N-1) wrote
 * buffer (N-1)&1, so reversed stage s (global index N-1+s) reads (N-2+s)&1 */
template <class C, int S, int E>
__device__ __forceinline__ void pp_inv(int tid, int g, float2 *buf0, float2 *buf1, const float2 *tws)
{
	if constexpr (S < E) {
		constexpr int R = C::ir(S), NS = C::ins(S);
		constexpr int RD = (C::N - 2 + S) & 1;
		const Ex<C> src{RD ? buf1 : buf0}, dst{RD ? buf0 : buf1};
		pp_stage<C, R, NS>(tid, tws + C::itw_off(S), src, [&](int i, float2 v) { dst.put(i, v); });
		gsync<C>(g);
		pp_inv<C, S + 1, E>(tid, g, buf0, buf1, tws);
	}
}

template <class C, int OP>
__device__ __forceinline__ void pp_transform(int tid, int g, float2 *buf0, float2 *buf1,
                                             const FirstLoad<C, OP, false> &first, float *y, const float2 *tws,
                                             const float2 *mods, const float2 *ks)
{
	constexpr int L = C::L, N = C::N;
	constexpr bool FREQ = C::MOD == FGK_MOD_FREQOFF;
	constexpr bool CONV = OP == FGK_OP_CONV || OP == FGK_OP_CORR;
	static_assert(N >= 2, "ping-pong kernels need two or more stages");
	auto out_final = [&](int i, float2 u) {
		if constexpr (FREQ) {
			const float2 r = cmul(u, mods[i]);
			stcs(y + i, r.x);
			stcs(y + L + i, r.y);
		} else {
			stcs2(reinterpret_cast<float2 *>(y) + i, conjf2(u));
		}
	};
	const Ex<C> b0{buf0};
	/* stage 0: HBM -> buffer 0 */
	if constexpr (C::MODC && FREQ && OP != FGK_OP_INVERSE)
		pp_first_modc<C, OP>(tid, first, mods, [&](int i, float2 v) { b0.put(i, v); });
	else
		pp_stage<C, C::fr(0), 1>(tid, tws, first, [&](int i, float2 v) { b0.put(i, v); });
	gsync<C>(g);
	pp_fwd<C, 1, N - 1>(tid, g, buf0, buf1, tws);
	/* stage N-1 reads buffer (N-2)&1 */
	const Ex<C> src{((N - 2) & 1) ? buf1 : buf0}, dst{((N - 2) & 1) ? buf0 : buf1};
	if constexpr (CONV) {
		constexpr int R = C::fr(N - 1), NS = C::fns(N - 1), NBF = L / R;
		constexpr int NB = (NBF + C::T - 1) / C::T;
		constexpr bool FULL = (NBF % C::T) == 0;
#pragma unroll 2
		for (int b = 0; b < NB; b++) {
			const int j = tid + b * C::T;
			if (FULL || j < NBF) {
				float2 v[R];
#pragma unroll
				for (int p = 0; p < R; p++)
					v[p] = src(j + p * NBF);
				if constexpr (NS > 1)
					twiddle_in<C, R, NS>(v, tws + C::ftw_off(N - 1), j);
				Radix<R>::run(v);
#pragma unroll
				for (int q = 0; q < R; q++)
					v[q] = conjf2(cmul(v[q], ks[j + q * NBF]));
				Radix<R>::run(v);
#pragma unroll
				for (int q = 0; q < R; q++)
					dst.put(j * R + q, v[q]);
			}
		}
		gsync<C>(g);
		pp_inv<C, 1, N - 1>(tid, g, buf0, buf1, tws);
		constexpr int RL = C::ir(N - 1), NSL = C::ins(N - 1);
		constexpr int RD = (2 * N - 3) & 1; /* reversed stage N-1 is global stage 2N-2 */
		const Ex<C> last{RD ? buf1 : buf0};
		if constexpr (C::MODC && FREQ)
			pp_last_modc<C, RL, NSL>(tid, tws + C::itw_off(N - 1), last, y, mods);
		else
			pp_stage<C, RL, NSL>(tid, tws + C::itw_off(N - 1), last, out_final);
		/* the next transform's stage 0 writes buffer 0: if this stage read
		 * it, every thread must be done first */
		if constexpr (RD == 0)
			gsync<C>(g);
	} else {
		constexpr int R = C::fr(N - 1), NS = C::fns(N - 1);
		if constexpr (OP == FGK_OP_INVERSE && C::MODC && FREQ) {
			pp_last_modc<C, R, NS>(tid, tws + C::ftw_off(N - 1), src, y, mods);
		} else if constexpr (OP == FGK_OP_INVERSE) {
			pp_stage<C, R, NS>(tid, tws + C::ftw_off(N - 1), src, out_final);
		} else if constexpr (!FREQ) {
			pp_stage<C, R, NS>(tid, tws + C::ftw_off(N - 1), src,
			                   [&](int i, float2 v) { stcs2(reinterpret_cast<float2 *>(y) + i, v); });
		} else {
			pp_stage<C, R, NS>(tid, tws + C::ftw_off(N - 1), src, [&](int i, float2 v) { dst.put(i, v); });
			gsync<C>(g);
			/* X[2m] = W[m], X[2m+1] = conj W[L-1-m] */
			float2 *y2 = reinterpret_cast<float2 *>(y);
			for (int m = tid; m < L / 2; m += C::T) {
				const float2 w0 = dst(m), w1 = dst(L - 1 - m);
				stcs2(y2 + 2 * m, w0);
				stcs2(y2 + 2 * m + 1, conjf2(w1));
			}
		}
		gsync<C>(g);
	}
}

/* ---- overlap-add, fused into the convolution ---------------------------
 * Block b of a real signal (FREQ_OFFSET_REAL): its first stage reads the
 * signal at b B directly, zero past B samples (or past the signal's end), so
 * the zero-padded blocks are never written out; its last stage writes the
 * first span = B + K - 1 samples of the block's result into the output at
 * b B. The host launches this only when span <= 2 B, so output t has one
 * contributor unless t mod B < K - 1, where block t/B and the block before
 * it meet: there (the block's first K - 1 and its last span - B samples) the
 * result is added with atomicAdd into an output the host has zeroed, and
 * elsewhere stored. Zero plus one term, or two terms in either order, are
 * exact and order-free, so the result is deterministic and equals the
 * unfused split / convolution / gather bit for bit. The compiled ping-pong
 * configurations with constant modulation (MODC) provide the stages. */
struct OlaArgs {
	const float *in;      /* the signal, n samples */
	uint64_t     n;
	uint32_t     B, span; /* block length; result samples added per block */
	uint32_t     nblocks;
	uint64_t     nout;    /* n + K - 1 */
	const float *kern;
	float       *out;     /* zero in the overlap zones (t mod B < K - 1) when the launch starts */
};

/* the zero-padded block as the first stage reads it */
struct OlaLoad {
	const float *x;
	uint32_t     valid; /* samples of the signal in this block */
	__device__ __forceinline__ float ld(int i) const { return (uint32_t)i < valid ? __ldcs(x + i) : 0.f; }
};

template <class C>
__global__ void __launch_bounds__(C::T *C::G, 1) static_kernel_ola(const fgk_plan p, OlaArgs a)
{
	static_assert(C::PP && C::MODC && C::MOD == FGK_MOD_FREQOFF, "the fused overlap-add uses the MODC ping-pong forms");
	extern __shared__ float2 smem[];
	using Lay = Layout<C, FGK_OP_CONV>;
	constexpr int L = C::L, N = C::N;
	const float2 *tws = C::TWG ? (const float2 *)p.tw : smem;
	float2 *mods = smem + Lay::TW;
	float2 *ks = mods + Lay::MODS;
	float2 *exb = ks + Lay::KS;
	StaticArgs sa{};
	sa.kern = a.kern;
	stage_tables<C, FGK_OP_CONV>(p, sa, smem, mods, ks);
	__syncthreads();

	const int g = threadIdx.x / C::T;
	const int tid = C::wt((int)threadIdx.x - g * C::T, g);
	float2 *buf0 = exb + (size_t)(2 * g) * C::SLOTS;
	float2 *buf1 = buf0 + C::SLOTS;
	for (uint64_t t = (uint64_t)blockIdx.x * C::G + g; t < a.nblocks; t += (uint64_t)gridDim.x * C::G) {
		const uint64_t base = t * a.B;
		const OlaLoad first{a.in + base, base + a.B <= a.n ? a.B : (uint32_t)(a.n - base)};
		const uint32_t lim = base + a.span <= a.nout ? a.span : (uint32_t)(a.nout - base);
		const uint32_t ovl = a.span - a.B; /* K - 1 */
		float *y = a.out + base;
		const Ex<C> b0{buf0};
		pp_first_modc<C, FGK_OP_CONV>(tid, first, mods, [&](int i, float2 v) { b0.put(i, v); });
		gsync<C>(g);
		pp_fwd<C, 1, N - 1>(tid, g, buf0, buf1, tws);
		const Ex<C> src{((N - 2) & 1) ? buf1 : buf0}, dst{((N - 2) & 1) ? buf0 : buf1};
		{
			constexpr int R = C::fr(N - 1), NS = C::fns(N - 1), NBF = L / R;
			constexpr int NB = (NBF + C::T - 1) / C::T;
			constexpr bool FULL = (NBF % C::T) == 0;
#pragma unroll 2
			for (int b = 0; b < NB; b++) {
				const int j = tid + b * C::T;
				if (FULL || j < NBF) {
					float2 v[R];
#pragma unroll
					for (int q = 0; q < R; q++)
						v[q] = src(j + q * NBF);
					if constexpr (NS > 1)
						twiddle_in<C, R, NS>(v, tws + C::ftw_off(N - 1), j);
					Radix<R>::run(v);
#pragma unroll
					for (int q = 0; q < R; q++)
						v[q] = conjf2(cmul(v[q], ks[j + q * NBF]));
					Radix<R>::run(v);
#pragma unroll
					for (int q = 0; q < R; q++)
						dst.put(j * R + q, v[q]);
				}
			}
			gsync<C>(g);
		}
		pp_inv<C, 1, N - 1>(tid, g, buf0, buf1, tws);
		{
			constexpr int RL = C::ir(N - 1), NSL = C::ins(N - 1), NBFL = L / RL;
			static_assert(NSL == NBFL, "the last stage's ns is L/R");
			constexpr int RD = (2 * N - 3) & 1;
			constexpr int NB = (NBFL + C::T - 1) / C::T;
			constexpr bool FULL = (NBFL % C::T) == 0;
			const Ex<C> last{RD ? buf1 : buf0};
#pragma unroll 2
			for (int b = 0; b < NB; b++) {
				const int j = tid + b * C::T;
				if (FULL || j < NBFL) {
					float2 v[RL];
#pragma unroll
					for (int q = 0; q < RL; q++)
						v[q] = last(j + q * NBFL);
					twiddle_in<C, RL, NSL>(v, tws + C::itw_off(N - 1), j);
					Radix<RL>::run(v);
					mod_steps<RL>(v, mods[j]);
#pragma unroll
					for (int q = 0; q < RL; q++) {
						const uint32_t i0 = (uint32_t)(j + q * NBFL), i1 = i0 + (uint32_t)L;
						/* an overlap zone: the first K - 1 samples and those from B on */
						if (i0 < lim) {
							if (i0 < ovl || i0 >= a.B)
								atomicAdd(y + i0, v[q].x);
							else
								stcs(y + i0, v[q].x);
						}
						if (i1 < lim) {
							if (i1 < ovl || i1 >= a.B)
								atomicAdd(y + i1, v[q].y);
							else
								stcs(y + i1, v[q].y);
						}
					}
				}
			}
			if constexpr (RD == 0)
				gsync<C>(g);
		}
	}
}

template <class C, int OP>
__global__ void __launch_bounds__(C::T *C::G, 1) static_kernel_pp(const fgk_plan p, StaticArgs a)
{
	extern __shared__ float2 smem[];
	using Lay = Layout<C, OP>;
	const float2 *tws = C::TWG ? (const float2 *)p.tw : smem;
	float2 *mods = smem + Lay::TW;
	float2 *ks = mods + Lay::MODS;
	float2 *exb = ks + Lay::KS;
	stage_tables<C, OP>(p, a, smem, mods, ks);
	__syncthreads();

	const int g = threadIdx.x / C::T;
	const int tid = C::wt((int)threadIdx.x - g * C::T, g);
	float2 *buf0 = exb + (size_t)(2 * g) * C::SLOTS;
	float2 *buf1 = buf0 + C::SLOTS;
	for (uint64_t t = (uint64_t)blockIdx.x * C::G + g; t < a.count; t += (uint64_t)gridDim.x * C::G) {
		const FirstLoad<C, OP, false> first{a.in + t * a.in_stride, mods};
		pp_transform<C, OP>(tid, g, buf0, buf1, first, a.out + t * a.out_stride, tws, mods, ks);
	}
}

/* ---- gradient with respect to the taps --------------------------------- */
/* For pairs (g_b, x_b) of blocks: P[m] = sum_b W_g,b[m] conj(W_x,b[m]), the
 * forward transforms' natural-order spectra before the FREQ_OFFSET_REAL
 * split, accumulated per CTA. Each group transforms g_b, parks the last
 * stage's outputs in its own buffer (the thread that writes a bin is the
 * one that reads it back, so no barrier guards it), transforms x_b and
 * accumulates the products in registers; at the end the groups' sums are
 * added and the CTA writes one row of `partials`. Every block pair crosses
 * HBM once (one read of g_b and of x_b); the partial rows are what is left
 * to reduce (fgk_adjoint.cu, kg_reduce). */
struct KgradArgs {
	const float *g, *x;
	size_t       g_stride, x_stride;
	uint32_t     count;
	float2      *partials; /* gridDim.x rows of L */
};

/* the forward chain of one block up to the last stage's butterflies, whose
 * outputs (bin j + q L/R of butterfly j) stay in t; ends with `ex` free */
template <class C, class First>
__device__ __forceinline__ void forward_to_tile(int tid, int g, const Ex<C> &ex, const First &first,
                                                const float2 *tws, Tile<C, C::fr(C::N - 1)> &t)
{
	constexpr int N = C::N;
	static_assert(N >= 2, "the gradient kernel needs two or more stages");
	{
		constexpr int R = C::fr(0);
		Tile<C, R> t0;
		t0.load(tid, first);
		t0.template butterfly<1>(tid, tws);
		t0.template store<1>(tid, [&](int i, float2 v) { ex.put(i, v); });
		gsync<C>(g);
	}
	fwd_mid<C, 1, N - 1>(tid, g, ex, tws);
	t.load(tid, ex);
	gsync<C>(g);
	t.template butterfly<C::fns(N - 1)>(tid, tws + C::ftw_off(N - 1));
}

template <class C>
__global__ void __launch_bounds__(C::T *C::G, 1) static_kernel_kgrad(const fgk_plan p, KgradArgs a)
{
	extern __shared__ float2 smem[];
	using Lay = Layout<C, FGK_OP_FORWARD>;
	constexpr int L = C::L, R = C::fr(C::N - 1), NBF = L / R;
	using TL = Tile<C, R>;
	const float2 *tws = C::TWG ? (const float2 *)p.tw : smem;
	float2 *mods = smem + Lay::TW;
	float2 *exb = mods + Lay::MODS;
	float2 *park = exb + (size_t)C::G * C::SLOTS; /* G x L */
	stage_tables<C, FGK_OP_FORWARD>(p, StaticArgs{}, smem, mods, nullptr);
	__syncthreads();

	const int g = threadIdx.x / C::T;
	const int tid = C::wt((int)threadIdx.x - g * C::T, g);
	const Ex<C> ex{exb + (size_t)g * C::SLOTS};
	float2 *pk = park + (size_t)g * L;
	float2 acc[TL::NB][R];
#pragma unroll
	for (int b = 0; b < TL::NB; b++)
#pragma unroll
		for (int q = 0; q < R; q++)
			acc[b][q] = make_float2(0.f, 0.f);
	for (uint64_t t = (uint64_t)blockIdx.x * C::G + g; t < a.count; t += (uint64_t)gridDim.x * C::G) {
		{
			TL tg;
			forward_to_tile<C>(tid, g, ex, FirstLoad<C, FGK_OP_FORWARD, false>{a.g + t * a.g_stride, mods}, tws, tg);
#pragma unroll
			for (int b = 0; b < TL::NB; b++)
				if (TL::live(tid, b))
#pragma unroll
					for (int q = 0; q < R; q++)
						pk[tid + b * C::T + q * NBF] = tg.v[b][q];
		}
		TL tx;
		forward_to_tile<C>(tid, g, ex, FirstLoad<C, FGK_OP_FORWARD, false>{a.x + t * a.x_stride, mods}, tws, tx);
#pragma unroll
		for (int b = 0; b < TL::NB; b++)
			if (TL::live(tid, b))
#pragma unroll
				for (int q = 0; q < R; q++) {
					const int i = tid + b * C::T + q * NBF;
					acc[b][q] = cadd(acc[b][q], cmulc(pk[i], tx.v[b][q]));
				}
	}
	/* the groups' sums, then one row per CTA */
#pragma unroll
	for (int b = 0; b < TL::NB; b++)
		if (TL::live(tid, b))
#pragma unroll
			for (int q = 0; q < R; q++)
				pk[tid + b * C::T + q * NBF] = acc[b][q];
	__syncthreads();
	float2 *row = a.partials + (size_t)blockIdx.x * L;
	for (int i = threadIdx.x; i < L; i += blockDim.x) {
		float2 sum = park[i];
#pragma unroll
		for (int gg = 1; gg < C::G; gg++)
			sum = cadd(sum, park[(size_t)gg * L + i]);
		row[i] = sum;
	}
}

template <class C> constexpr size_t kgrad_smem_bytes()
{
	return Layout<C, FGK_OP_FORWARD>::DIRECT_BYTES + sizeof(float2) * (size_t)C::G * C::L;
}

/* ---- the adjoint in one pass ---------------------------------------------
 * For block pairs (g_b, x_b): dx_b, the correlation of g_b with the taps
 * (the convolution of g_b with the conjugated kernel spectrum, what
 * FGK_OP_CORR computes), and the CTA's sum of W_g conj(W_x) for the taps
 * gradient. g_b is transformed once for both: its spectrum is parked on its
 * way through the correlation, then x_b is transformed and the product
 * accumulated. Per block pair HBM sees one read of g_b and x_b and one write
 * of dx_b. The FREQ_OFFSET_REAL modulation of the first and last stages is
 * mods[j] e^{-j pi p/(2R)} (mod_steps) for the points j + p L/R of butterfly
 * j, so only L/R table entries are staged, which leaves shared memory for
 * the park buffers. */
struct AdjArgs {
	const float *g, *x, *kern;
	float       *dx;
	size_t       g_stride, x_stride, dx_stride;
	uint32_t     count;
	float2      *partials; /* gridDim.x rows of L */
};

template <class C> struct AdjLayout {
	static constexpr int MODS = C::MOD == FGK_MOD_FREQOFF ? C::L / C::fr(0) : 0; /* float2 */
	static constexpr size_t TW = C::TWG ? 0 : (size_t)C::TW_TOTAL;
	static constexpr size_t BYTES =
	    sizeof(float2) * (TW + MODS + (size_t)C::L + (size_t)C::G * C::SLOTS + (size_t)C::G * C::L);
};

/* stage 0 of a forward chain from HBM into the exchange buffer */
template <class C>
__device__ __forceinline__ void adj_first(int tid, int g, const Ex<C> &ex, const float *x, const float2 *mods,
                                          const float2 *tws)
{
	constexpr int L = C::L, R = C::fr(0), NBF = L / R;
	using T0 = Tile<C, R>;
	T0 t0;
	if constexpr (C::MOD == FGK_MOD_FREQOFF) {
#pragma unroll
		for (int b = 0; b < T0::NB; b++) {
			const int j = tid + b * C::T;
			if (T0::live(tid, b)) {
#pragma unroll
				for (int p = 0; p < R; p++)
					t0.v[b][p] = make_float2(ldcs(x + j + p * NBF), -ldcs(x + L + j + p * NBF));
				mod_steps<R>(t0.v[b], mods[j]);
			}
		}
	} else {
		t0.load(tid, [&](int i) { return ldcs2(reinterpret_cast<const float2 *>(x) + i); });
	}
	t0.template butterfly<1>(tid, tws);
	t0.template store<1>(tid, [&](int i, float2 v) { ex.put(i, v); });
	gsync<C>(g);
}

template <class C>
__global__ void __launch_bounds__(C::T *C::G, 1) static_kernel_adj(const fgk_plan p, AdjArgs a)
{
	extern __shared__ float2 smem[];
	using Lay = AdjLayout<C>;
	constexpr int L = C::L, N = C::N;
	constexpr int R = C::fr(N - 1), NS = C::fns(N - 1), NBF = L / R;       /* last forward stage */
	constexpr int RL = C::ir(N - 1), NSL = C::ins(N - 1), NBFL = L / RL; /* last reversed stage */
	constexpr bool FREQ = C::MOD == FGK_MOD_FREQOFF;
	static_assert(N >= 2, "the adjoint kernel needs two or more stages");
	using TL = Tile<C, R>;
	using TR = Tile<C, RL>;
	const float2 *tws = C::TWG ? (const float2 *)p.tw : smem;
	float2 *mods = smem + Lay::TW;
	float2 *ks = mods + Lay::MODS;
	float2 *exb = ks + L;
	float2 *park = exb + (size_t)C::G * C::SLOTS;
	/* a programmatic dependent, as stage_tables describes: the plan's
	 * tables before the wait, the kernel buffer and the blocks after */
	asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
	if constexpr (!C::TWG)
		stage_twiddles<C, 1>(smem, (const float2 *)p.tw);
	if constexpr (FREQ)
		for (int i = threadIdx.x; i < Lay::MODS; i += blockDim.x)
			mods[i] = __ldg((const float2 *)p.modtw + i);
	asm volatile("griddepcontrol.wait;" ::: "memory");
	for (int i = threadIdx.x; i < L; i += blockDim.x) {
		const int o = __ldg(p.kidx + i);
		ks[i] = make_float2(__ldg(a.kern + o), -__ldg(a.kern + o + (int)p.kvw)); /* conj K: correlation */
	}
	__syncthreads();

	const int g = threadIdx.x / C::T;
	const int tid = C::wt((int)threadIdx.x - g * C::T, g);
	const Ex<C> ex{exb + (size_t)g * C::SLOTS};
	auto exput = [&](int i, float2 v) { ex.put(i, v); };
	float2 *pk = park + (size_t)g * L;
	float2 acc[TL::NB][R];
#pragma unroll
	for (int b = 0; b < TL::NB; b++)
#pragma unroll
		for (int q = 0; q < R; q++)
			acc[b][q] = make_float2(0.f, 0.f);
	for (uint64_t t = (uint64_t)blockIdx.x * C::G + g; t < a.count; t += (uint64_t)gridDim.x * C::G) {
		/* g_b: forward chain, park W_g, product with conj K, reversed chain */
		adj_first<C>(tid, g, ex, a.g + t * a.g_stride, mods, tws);
		fwd_mid<C, 1, N - 1>(tid, g, ex, tws);
		{
			TL tt;
			tt.load(tid, ex);
			gsync<C>(g);
			tt.template butterfly<NS>(tid, tws + C::ftw_off(N - 1));
#pragma unroll
			for (int b = 0; b < TL::NB; b++) {
				const int j = tid + b * C::T;
				if (TL::live(tid, b)) {
#pragma unroll
					for (int q = 0; q < R; q++) {
						pk[j + q * NBF] = tt.v[b][q];
						tt.v[b][q] = conjf2(cmul(tt.v[b][q], ks[j + q * NBF]));
					}
					Radix<R>::run(tt.v[b]);
				}
			}
			tt.template store<1>(tid, exput);
			gsync<C>(g);
		}
		inv_mid<C, 1, N - 1>(tid, g, ex, tws);
		{
			float *y = a.dx + t * a.dx_stride;
			TR tt;
			tt.load(tid, ex);
			tt.template butterfly<NSL>(tid, tws + C::itw_off(N - 1));
#pragma unroll
			for (int b = 0; b < TR::NB; b++) {
				const int j = tid + b * C::T;
				if (TR::live(tid, b)) {
					if constexpr (FREQ) {
						mod_steps<RL>(tt.v[b], mods[j]);
#pragma unroll
						for (int q = 0; q < RL; q++) {
							stcs(y + j + q * NBFL, tt.v[b][q].x);
							stcs(y + L + j + q * NBFL, tt.v[b][q].y);
						}
					} else {
#pragma unroll
						for (int q = 0; q < RL; q++)
							stcs2(reinterpret_cast<float2 *>(y) + j + q * NBFL, conjf2(tt.v[b][q]));
					}
				}
			}
			gsync<C>(g);
		}
		/* x_b: forward chain, product with the parked W_g */
		adj_first<C>(tid, g, ex, a.x + t * a.x_stride, mods, tws);
		fwd_mid<C, 1, N - 1>(tid, g, ex, tws);
		{
			TL tx;
			tx.load(tid, ex);
			gsync<C>(g);
			tx.template butterfly<NS>(tid, tws + C::ftw_off(N - 1));
#pragma unroll
			for (int b = 0; b < TL::NB; b++)
				if (TL::live(tid, b))
#pragma unroll
					for (int q = 0; q < R; q++) {
						const int i = tid + b * C::T + q * NBF;
						acc[b][q] = cadd(acc[b][q], cmulc(pk[i], tx.v[b][q]));
					}
		}
	}
#pragma unroll
	for (int b = 0; b < TL::NB; b++)
		if (TL::live(tid, b))
#pragma unroll
			for (int q = 0; q < R; q++)
				pk[tid + b * C::T + q * NBF] = acc[b][q];
	__syncthreads();
	float2 *row = a.partials + (size_t)blockIdx.x * L;
	for (int i = threadIdx.x; i < L; i += blockDim.x) {
		float2 sum = park[i];
#pragma unroll
		for (int gg = 1; gg < C::G; gg++)
			sum = cadd(sum, park[(size_t)gg * L + i]);
		row[i] = sum;
	}
}

/* ---- call service --------------------------------------------------------
 * One CTA of one group (T threads) serving single transforms of this
 * configuration on request (fgk.h, fgk_serve_words; the doorbell protocol
 * is fgk_serve.cuh's): the tables are staged once, then each request runs
 * the same stages as the batched kernel of the op (so the same bits), and
 * no request costs a launch. */
template <class C, int OP>
__device__ __forceinline__ void serve_one(int tid, float2 *exb, const float *in, float *out, const float2 *tws,
                                          const float2 *mods, const float2 *ks)
{
	const FirstLoad<C, OP, false> first{in, mods};
	if constexpr (C::PP)
		pp_transform<C, OP>(tid, 0, exb, exb + C::SLOTS, first, out, tws, mods, ks);
	else
		transform<C, OP, false>(tid, 0, Ex<C>{exb}, first, out, tws, mods, ks);
}

template <class C, int OPS>
__global__ void __launch_bounds__(C::T, 1)
    static_kernel_serve(const fgk_plan p, fgk_serve_words w, uint64_t seen, uint64_t id, uint32_t idle_polls)
{
	static_assert(!C::TMA, "the call service runs the direct or ping-pong stages");
	extern __shared__ float2 smem[];
	using Lay = Layout<C, FGK_OP_CONV>; /* the tables with room for the kernel spectrum */
	const float2 *tws = C::TWG ? (const float2 *)p.tw : smem;
	float2 *mods = smem + Lay::TW;
	float2 *ks = mods + Lay::MODS;
	float2 *exb = ks + Lay::KS;
	__shared__ ServeSlot slot;
	stage_tables<C, FGK_OP_FORWARD>(p, StaticArgs{}, smem, mods, nullptr);
	const int tid = C::wt((int)threadIdx.x, 0);
	for (;;) {
		if (threadIdx.x == 0)
			serve_next(w, seen, id, idle_polls, slot);
		__syncthreads();
		const int op = slot.op;
		if (op < 0)
			break;
		const float *in = reinterpret_cast<const float *>(slot.in);
		float *out = reinterpret_cast<float *>(slot.out);
		if (op == FGK_OP_CONV || op == FGK_OP_CORR) {
			/* the request's kernel spectrum, as the batched kernel stages it */
			const float *kern = reinterpret_cast<const float *>(slot.kern);
			const int32_t *kidx = p.kidx;
			const int kvw = (int)p.kvw;
			for (int i = threadIdx.x; i < C::L; i += blockDim.x) {
				const int o = __ldg(kidx + i);
				float2 k = make_float2(__ldg(kern + o), __ldg(kern + o + kvw));
				if (op == FGK_OP_CORR)
					k.y = -k.y;
				ks[i] = k;
			}
			__syncthreads();
		}
		if constexpr ((OPS >> FGK_OP_FORWARD) & 1)
			if (op == FGK_OP_FORWARD)
				serve_one<C, FGK_OP_FORWARD>(tid, exb, in, out, tws, mods, ks);
		if constexpr ((OPS >> FGK_OP_INVERSE) & 1)
			if (op == FGK_OP_INVERSE)
				serve_one<C, FGK_OP_INVERSE>(tid, exb, in, out, tws, mods, ks);
		if constexpr ((OPS >> FGK_OP_CONV) & 1)
			if (op == FGK_OP_CONV)
				serve_one<C, FGK_OP_CONV>(tid, exb, in, out, tws, mods, ks);
		if constexpr ((OPS >> FGK_OP_CORR) & 1)
			if (op == FGK_OP_CORR)
				serve_one<C, FGK_OP_CORR>(tid, exb, in, out, tws, mods, ks);
		__syncthreads();
		if (threadIdx.x == 0)
			serve_reply(w, slot);
	}
}

template <class C> constexpr size_t serve_smem_bytes()
{
	return sizeof(float2) * (Layout<C, FGK_OP_CONV>::TABLES + (C::PP ? 2 : 1) * (size_t)C::SLOTS);
}

/* ------------------------------------------------------------------------
 * Registry entries */
typedef void (*static_fn)(const fgk_plan, StaticArgs);
typedef void (*kgrad_fn)(const fgk_plan, KgradArgs);
typedef void (*adj_fn)(const fgk_plan, AdjArgs);
typedef void (*ola_fn)(const fgk_plan, OlaArgs);
typedef void (*serve_fn)(const fgk_plan, fgk_serve_words, uint64_t, uint64_t, uint32_t);

struct StaticEntry {
	uint32_t  mod, L, T, G, n, tma;
	uint32_t  radices[FGK_MAX_STAGES];
	size_t    smem[FGK_OP_COUNT];
	static_fn fn[FGK_OP_COUNT];
	kgrad_fn  kgrad; /* the taps-gradient kernel of this configuration, or null */
	size_t    kgrad_smem;
	adj_fn    adj; /* the one-pass adjoint (input and taps gradients), or null */
	size_t    adj_smem;
	ola_fn    ola; /* the fused overlap-add, or null */
	size_t    ola_smem;
	serve_fn  serve; /* the call service, or null */
	size_t    serve_smem;
	uint32_t  serve_ops;
};

template <class C, int OP> constexpr size_t smem_bytes()
{
	return C::TMA ? Layout<C, OP>::TMA_BYTES : C::PP ? Layout<C, OP>::PP_BYTES : Layout<C, OP>::DIRECT_BYTES;
}

template <class C, int OP> constexpr static_fn kernel_of()
{
	if constexpr (C::TMA)
		return static_kernel_tma<C, OP>;
	else if constexpr (C::PP)
		return static_kernel_pp<C, OP>;
	else
		return static_kernel<C, OP>;
}

/* OPS: bit mask of the ops compiled for this configuration */
/* dynamic shared memory of one CTA must fit the 227 KB opt-in limit, with
 * room for the few bytes of static shared memory the TMA mode declares */
constexpr size_t FGK_SMEM_LIMIT = 232448 - 1024;

template <class C, int OPS> StaticEntry make_entry()
{
	static_assert(smem_bytes<C, FGK_OP_CONV>() <= FGK_SMEM_LIMIT, "variant exceeds shared memory");
	static_assert(smem_bytes<C, FGK_OP_FORWARD>() <= FGK_SMEM_LIMIT, "variant exceeds shared memory");
	StaticEntry e{};
	e.mod = C::MOD;
	e.L = C::L;
	e.T = C::T;
	e.G = C::G;
	e.n = C::N;
	e.tma = C::TMA ? 1u : 0u;
	for (int i = 0; i < C::N; i++)
		e.radices[i] = C::R[i];
	if constexpr ((OPS >> FGK_OP_FORWARD) & 1) {
		e.fn[FGK_OP_FORWARD] = kernel_of<C, FGK_OP_FORWARD>();
		e.smem[FGK_OP_FORWARD] = smem_bytes<C, FGK_OP_FORWARD>();
	}
	if constexpr ((OPS >> FGK_OP_INVERSE) & 1) {
		e.fn[FGK_OP_INVERSE] = kernel_of<C, FGK_OP_INVERSE>();
		e.smem[FGK_OP_INVERSE] = smem_bytes<C, FGK_OP_INVERSE>();
	}
	if constexpr ((OPS >> FGK_OP_CONV) & 1) {
		e.fn[FGK_OP_CONV] = kernel_of<C, FGK_OP_CONV>();
		e.smem[FGK_OP_CONV] = smem_bytes<C, FGK_OP_CONV>();
	}
	if constexpr ((OPS >> FGK_OP_CORR) & 1) {
		e.fn[FGK_OP_CORR] = kernel_of<C, FGK_OP_CORR>();
		e.smem[FGK_OP_CORR] = smem_bytes<C, FGK_OP_CORR>();
	}
	return e;
}

/* adds the taps-gradient and one-pass adjoint kernels to an entry
 * (direct-load, in-place configurations: the kernels are built from their
 * transform stages) */
template <class C> StaticEntry with_kgrad(StaticEntry e)
{
	static_assert(C::MODE == 0, "the gradient kernel uses the in-place stages");
	static_assert(kgrad_smem_bytes<C>() <= FGK_SMEM_LIMIT, "gradient kernel exceeds shared memory");
	static_assert(AdjLayout<C>::BYTES <= FGK_SMEM_LIMIT, "adjoint kernel exceeds shared memory");
	e.kgrad = static_kernel_kgrad<C>;
	e.kgrad_smem = kgrad_smem_bytes<C>();
	e.adj = static_kernel_adj<C>;
	e.adj_smem = AdjLayout<C>::BYTES;
	return e;
}

/* adds the fused overlap-add kernel to an entry (MODC ping-pong
 * FREQ_OFFSET_REAL configurations) */
template <class C> StaticEntry with_ola(StaticEntry e)
{
	static_assert(smem_bytes<C, FGK_OP_CONV>() <= FGK_SMEM_LIMIT, "overlap-add kernel exceeds shared memory");
	e.ola = static_kernel_ola<C>;
	e.ola_smem = smem_bytes<C, FGK_OP_CONV>();
	return e;
}

/* adds the call service to an entry (configurations without bulk-copy
 * input), for the ops the entry compiles */
template <class C, int OPS> StaticEntry with_serve(StaticEntry e)
{
	static_assert(serve_smem_bytes<C>() <= FGK_SMEM_LIMIT, "call service exceeds shared memory");
	e.serve = static_kernel_serve<C, OPS>;
	e.serve_smem = serve_smem_bytes<C>();
	e.serve_ops = (uint32_t)OPS;
	return e;
}

constexpr int OPS_FWD_INV = (1 << FGK_OP_FORWARD) | (1 << FGK_OP_INVERSE);
constexpr int OPS_CONV = (1 << FGK_OP_CONV);
constexpr int OPS_CONV_CORR = (1 << FGK_OP_CONV) | (1 << FGK_OP_CORR);
constexpr int OPS_ALL = OPS_FWD_INV | OPS_CONV_CORR;

} /* namespace fgk */

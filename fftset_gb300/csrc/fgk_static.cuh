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

namespace fgk {

template <int MOD_, int L_, int T_, int G_, int TWG_, int... Rs> struct SCfg {
	static constexpr int MOD = MOD_;
	static constexpr bool TWG = TWG_ != 0; /* twiddles read from global memory (L1) instead of shared */
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
	static __host__ __device__ constexpr int itw_off(int s) { return s == 0 ? ftw_off(N) : itw_off(s - 1) + itw_size(s - 1); }
	static constexpr int TW_TOTAL = itw_off(N);
	static constexpr int SLOTS = L + L / 16 + 1; /* padded exchange buffer */
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
				if constexpr (NS > 1) {
					const int k = j % NS;
#pragma unroll
					for (int p = 1; p < R; p++)
						v[b][p] = cmul(v[b][p], C::TWG ? __ldg(tws + k * (R - 1) + (p - 1)) : tws[(p - 1) * NS + k]);
				}
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
	if constexpr (S < 2 * C::N) {
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
};

template <class C, int OP>
__global__ void __launch_bounds__(C::T *C::G, 1) static_kernel(const fgk_plan p, StaticArgs a)
{
	extern __shared__ float2 smem[];
	constexpr int L = C::L, N = C::N;
	constexpr bool FREQ = C::MOD == FGK_MOD_FREQOFF;
	constexpr bool CONV = OP == FGK_OP_CONV || OP == FGK_OP_CORR;
	/* twiddles: staged in shared memory ([p-1][k] per stage), or read from
	 * the plan's global table ([k][p-1] per stage) through L1 */
	const float2 *tws = C::TWG ? (const float2 *)p.tw : smem;
	float2 *mods = smem + (C::TWG ? 0 : C::TW_TOTAL);     /* L (FREQ) */
	float2 *ks = mods + (FREQ ? L : 0);                   /* L (CONV) */
	float2 *exb = ks + (CONV ? L : 0);                    /* G * SLOTS */

	/* ---- stage the tables once per CTA ---- */
	{
		if constexpr (!C::TWG)
			stage_twiddles<C, 1>(smem, (const float2 *)p.tw);
		if constexpr (FREQ) {
			const float2 *gm = (const float2 *)p.modtw;
			for (int i = threadIdx.x; i < L; i += blockDim.x)
				mods[i] = __ldg(gm + i);
		}
		if constexpr (CONV) {
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
		__syncthreads();
	}

	const int g = threadIdx.x / C::T;
	const int tid = threadIdx.x - g * C::T;
	const Ex<C> ex{exb + (size_t)g * C::SLOTS};

	for (uint64_t t = (uint64_t)blockIdx.x * C::G + g; t < a.count; t += (uint64_t)gridDim.x * C::G) {
		const float *x = a.in + t * a.in_stride;
		float *y = a.out + t * a.out_stride;

		/* first stage input */
		auto in_fwd = [&](int i) -> float2 {
			if constexpr (FREQ)
				return cmul(make_float2(ldcs(x + i), -ldcs(x + L + i)), mods[i]);
			else
				return ldcs2(reinterpret_cast<const float2 *>(x) + i);
		};
		auto in_inv = [&](int i) -> float2 {
			const float2 *X = reinterpret_cast<const float2 *>(x);
			if constexpr (FREQ)
				return i < ((L + 1) >> 1) ? conjf2(ldcs2(X + 2 * i)) : ldcs2(X + 2 * (L - 1 - i) + 1);
			else
				return conjf2(ldcs2(X + i));
		};
		/* final output from u = DFT(conj(.)) */
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

		if constexpr (CONV) {
			static_assert(N >= 2, "static conv needs two or more stages");
			{
				constexpr int R = C::fr(0);
				Tile<C, R> t0;
				t0.load(tid, in_fwd);
				t0.template butterfly<1>(tid, tws);
				t0.template store<1>(tid, exput);
				gsync<C>(g);
			}
			fwd_mid<C, 1, N - 1>(tid, g, ex, tws);
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
			/* forward chain on the modulated input (FORWARD) or on conj(W) (INVERSE) */
			{
				constexpr int R = C::fr(0);
				Tile<C, R> t0;
				if constexpr (OP == FGK_OP_INVERSE)
					t0.load(tid, in_inv);
				else
					t0.load(tid, in_fwd);
				t0.template butterfly<1>(tid, tws);
				t0.template store<1>(tid, exput);
				gsync<C>(g);
			}
			fwd_mid<C, 1, N - 1>(tid, g, ex, tws);
			{
				constexpr int R = C::fr(N - 1), NS = C::fns(N - 1);
				Tile<C, R> t;
				t.load(tid, ex);
				if constexpr (OP == FGK_OP_FORWARD && FREQ)
					gsync<C>(g); /* results go back to shared memory */
				t.template butterfly<NS>(tid, tws + C::ftw_off(N - 1));
				if constexpr (OP == FGK_OP_INVERSE) {
					t.template store<NS>(tid, out_final);
				} else if constexpr (!FREQ) {
					t.template store<NS>(tid, [&](int i, float2 v) {
						stcs2(reinterpret_cast<float2 *>(y) + i, v);
					});
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
		}
		gsync<C>(g); /* the exchange buffer is reused by the next transform */
	}
}

/* ------------------------------------------------------------------------
 * Registry entries */
typedef void (*static_fn)(const fgk_plan, StaticArgs);

struct StaticEntry {
	uint32_t  mod, L, T, G, n;
	uint32_t  radices[FGK_MAX_STAGES];
	size_t    smem[FGK_OP_COUNT];
	static_fn fn[FGK_OP_COUNT];
};

template <class C, int OP> constexpr size_t smem_bytes()
{
	constexpr bool FREQ = C::MOD == FGK_MOD_FREQOFF;
	constexpr bool CONV = OP == FGK_OP_CONV || OP == FGK_OP_CORR;
	return sizeof(float2) * ((C::TWG ? 0 : (size_t)C::TW_TOTAL) + (FREQ ? C::L : 0) + (CONV ? C::L : 0) +
	                         (size_t)C::G * C::SLOTS);
}

/* OPS: bit mask of the ops compiled for this configuration */
template <class C, int OPS> StaticEntry make_entry()
{
	StaticEntry e{};
	e.mod = C::MOD;
	e.L = C::L;
	e.T = C::T;
	e.G = C::G;
	e.n = C::N;
	for (int i = 0; i < C::N; i++)
		e.radices[i] = C::R[i];
	if constexpr ((OPS >> FGK_OP_FORWARD) & 1) {
		e.fn[FGK_OP_FORWARD] = static_kernel<C, FGK_OP_FORWARD>;
		e.smem[FGK_OP_FORWARD] = smem_bytes<C, FGK_OP_FORWARD>();
	}
	if constexpr ((OPS >> FGK_OP_INVERSE) & 1) {
		e.fn[FGK_OP_INVERSE] = static_kernel<C, FGK_OP_INVERSE>;
		e.smem[FGK_OP_INVERSE] = smem_bytes<C, FGK_OP_INVERSE>();
	}
	if constexpr ((OPS >> FGK_OP_CONV) & 1) {
		e.fn[FGK_OP_CONV] = static_kernel<C, FGK_OP_CONV>;
		e.smem[FGK_OP_CONV] = smem_bytes<C, FGK_OP_CONV>();
	}
	if constexpr ((OPS >> FGK_OP_CORR) & 1) {
		e.fn[FGK_OP_CORR] = static_kernel<C, FGK_OP_CORR>;
		e.smem[FGK_OP_CORR] = smem_bytes<C, FGK_OP_CORR>();
	}
	return e;
}

constexpr int OPS_FWD_INV = (1 << FGK_OP_FORWARD) | (1 << FGK_OP_INVERSE);
constexpr int OPS_CONV = (1 << FGK_OP_CONV);
constexpr int OPS_CONV_CORR = (1 << FGK_OP_CONV) | (1 << FGK_OP_CORR);
constexpr int OPS_ALL = OPS_FWD_INV | OPS_CONV_CORR;

} /* namespace fgk */

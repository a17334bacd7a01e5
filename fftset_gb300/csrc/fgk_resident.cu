/* Resident (shared-memory) transforms for sm_103a.
 *
 * One group of `threads` threads owns one transform of length L (several
 * groups share a CTA for small L). The transform is a Stockham chain
 * (fgk.h: fgk_stage): every stage's butterflies run in registers through the
 * codelets of fgk_codelets.cuh and exchange through one padded shared-memory
 * buffer; the first stage reads HBM directly and the last writes HBM
 * directly, so each signal crosses HBM once in and once out.
 *
 * The modulation edges of the reference are fused into those first and last
 * stages:
 *   FREQ_OFFSET_REAL pack   c[i] = conj(x[i] + j x[L+i]) e^{-j pi i/(2L)}
 *                           (src/fftset_mod_freqoffsetreal.c:947-956, :572-676)
 *   FREQ_OFFSET_REAL split  X[2m] = W[m], X[2m+1] = conj W[L-1-m]
 *                           (:958-971, :832-843)
 *   unnormalised inverse    u = DFT(conj W), y from conj(u) (:974-1010,
 *                           src/fftset_mod_cplx.c:212-239)
 *   convolution             DFT -> conj(W K) -> DFT, no reordering in
 *                           between (src/fftset_vec.c:1161-1220): here the
 *                           forward chain's last stage and the reversed
 *                           chain's first stage share one register tile.
 *   kernel spectrum         scattered into the reference's kernel-buffer
 *                           layout through a per-plan index table
 *                           (src/fftset_vec.c:1199-1207 leaves it in the
 *                           plan's digit-reversed SIMD-lane order). */
#include <cuda_runtime.h>
#include <stdint.h>
#include "fgk.h"
#include "fgk_codelets.cuh"
#include "fgk_serve.cuh"

namespace fgk {

/* Run CALL with the compile-time radix R_ equal to r. A macro rather than a
 * generic lambda: every case must inline into the kernel, otherwise the
 * register tiles travel through an ABI call frame in local memory. */
#define FGK_RADIX_SWITCH(r, CALL)                                   \
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

struct Group {
	int     L, T, ltid, pad;
	bool    active;
	float2 *sm;
	__device__ __forceinline__ int slot(int i) const { return pad ? i + (i >> 4) : i; }
	__device__ __forceinline__ float2 ld(int i) const { return sm[slot(i)]; }
	__device__ __forceinline__ void st(int i, float2 v) const { sm[slot(i)] = v; }
};

/* One Stockham stage in shared memory: load this thread's butterflies,
 * barrier, twiddle + transform, store, barrier. */
template <int R, int EMAX>
__device__ __forceinline__ void stage_sm(const Group &g, const fgk_stage &st, const float2 *__restrict__ tw)
{
	constexpr int BM = (EMAX / R) > 0 ? EMAX / R : 1;
	const int nbf = g.L / R;
	const int nb = (int)st.nb;
	const int ns = (int)st.ns;
	float2 v[BM][R];
#pragma unroll
	for (int b = 0; b < BM; b++) {
		const int j = g.ltid + b * g.T;
		if (g.active && b < nb && j < nbf) {
#pragma unroll
			for (int p = 0; p < R; p++)
				v[b][p] = g.ld(j + p * nbf);
		}
	}
	__syncthreads();
#pragma unroll
	for (int b = 0; b < BM; b++) {
		const int j = g.ltid + b * g.T;
		if (g.active && b < nb && j < nbf) {
			const int k = j % ns;
			if (ns > 1) {
				const float2 *t = tw + st.tw_off + k * (R - 1);
#pragma unroll
				for (int p = 1; p < R; p++)
					v[b][p] = cmul(v[b][p], __ldg(t + p - 1));
			}
			Radix<R>::run(v[b]);
			const int base = (j - k) * R + k;
#pragma unroll
			for (int q = 0; q < R; q++)
				g.st(base + q * ns, v[b][q]);
		}
	}
	__syncthreads();
}

/* Last forward stage + spectrum product + first stage of the reversed chain.
 * The forward last stage produces bins j + q L/R of butterfly j; the reversed
 * chain's first stage (ns = 1) consumes exactly those, so they stay in
 * registers. Product: conj(W K) (conv) or conj(W conj K) (correlation). */
template <int R, int EMAX>
__device__ __forceinline__ void fused_sm(const Group &g, const fgk_stage &stf, const float2 *__restrict__ tw,
                                         const float *__restrict__ kern, const int32_t *__restrict__ kidx, int kvw,
                                         bool corr)
{
	constexpr int BM = (EMAX / R) > 0 ? EMAX / R : 1;
	const int nbf = g.L / R;
	const int nb = (int)stf.nb;
	const int ns = (int)stf.ns; /* == nbf */
	float2 v[BM][R];
#pragma unroll
	for (int b = 0; b < BM; b++) {
		const int j = g.ltid + b * g.T;
		if (g.active && b < nb && j < nbf) {
#pragma unroll
			for (int p = 0; p < R; p++)
				v[b][p] = g.ld(j + p * nbf);
		}
	}
	__syncthreads();
#pragma unroll
	for (int b = 0; b < BM; b++) {
		const int j = g.ltid + b * g.T;
		if (g.active && b < nb && j < nbf) {
			if (ns > 1) {
				const float2 *t = tw + stf.tw_off + j * (R - 1);
#pragma unroll
				for (int p = 1; p < R; p++)
					v[b][p] = cmul(v[b][p], __ldg(t + p - 1));
			}
			Radix<R>::run(v[b]);
#pragma unroll
			for (int q = 0; q < R; q++) {
				const int o = __ldg(kidx + j + q * nbf);
				const float2 k = make_float2(__ldg(kern + o), __ldg(kern + o + kvw));
				v[b][q] = conjf2(corr ? cmulc(v[b][q], k) : cmul(v[b][q], k));
			}
			Radix<R>::run(v[b]);
#pragma unroll
			for (int q = 0; q < R; q++)
				g.st(j * R + q, v[b][q]);
		}
	}
	__syncthreads();
}

/* One transform by one group (every thread of the CTA calls it: the stages
 * end in CTA barriers): x the block's input, y its output. The modulation
 * edges run as a prologue (HBM -> shared memory) and an epilogue (shared
 * memory -> HBM); the chain between them is shared by all ops. */
template <int EMAX>
__device__ __forceinline__ void generic_one(const fgk_plan &p, Group &g, int op, float *y, const float *x,
                                            const float *__restrict__ kern)
{
	const int L = g.L;
	const bool freqoff = p.modulation == FGK_MOD_FREQOFF;
	const float2 *tw = (const float2 *)p.tw;
	const float2 *mod = (const float2 *)p.modtw;
	const bool inverse = op == FGK_OP_INVERSE;
	const bool conv = op == FGK_OP_CONV || op == FGK_OP_CORR;

	/* prologue: the sequence to transform, natural order, into shared memory */
	if (g.active) {
		if (!inverse) {
			if (freqoff) {
				for (int i = g.ltid; i < L; i += g.T)
					g.st(i, cmul(make_float2(x[i], -x[L + i]), __ldg(mod + i)));
			} else {
				const float2 *x2 = reinterpret_cast<const float2 *>(x);
				for (int i = g.ltid; i < L; i += g.T)
					g.st(i, x2[i]);
			}
		} else {
			/* conj(W): W[m] = X[2m], W[L-1-m] = conj X[2m+1] (FREQ_OFFSET_REAL) */
			const float2 *X = reinterpret_cast<const float2 *>(x);
			if (freqoff) {
				const int half = L >> 1;
				for (int m = g.ltid; m < half; m += g.T) {
					g.st(m, conjf2(X[2 * m]));
					g.st(L - 1 - m, X[2 * m + 1]);
				}
				if ((L & 1) && g.ltid == 0)
					g.st(half, conjf2(X[L - 1]));
			} else {
				for (int i = g.ltid; i < L; i += g.T)
					g.st(i, conjf2(X[i]));
			}
		}
	}
	__syncthreads();

	/* stage descriptors come from the device copy of the plan: indexing the
	 * kernel-parameter copy at run time would spill it to local memory */
	const fgk_stage *fst = p.dev->fwd.st;
	const fgk_stage *ist = p.dev->inv.st;
	const int n = (int)p.fwd.nstages;
	const int nf = conv ? n - 1 : n;
	for (int s = 0; s < nf; s++) {
		const fgk_stage st = fst[s];
		FGK_RADIX_SWITCH(st.radix, (stage_sm<R_, EMAX>(g, st, tw)));
	}
	if (conv) {
		const fgk_stage st = fst[n - 1];
		FGK_RADIX_SWITCH(st.radix, (fused_sm<R_, EMAX>(g, st, tw, kern, p.kidx, (int)p.kvw, op == FGK_OP_CORR)));
		for (int s = 1; s < n; s++) {
			const fgk_stage sti = ist[s];
			FGK_RADIX_SWITCH(sti.radix, (stage_sm<R_, EMAX>(g, sti, tw)));
		}
	}

	/* epilogue */
	if (!g.active)
		return;
	if (inverse || conv) {
		/* u = DFT(conj(.)): FREQ_OFFSET_REAL y[i] + j y[L+i] = u_i e^{-j pi i/(2L)};
		 * COMPLEX y = conj(u) */
		if (freqoff) {
			for (int i = g.ltid; i < L; i += g.T) {
				const float2 r = cmul(g.ld(i), __ldg(mod + i));
				y[i] = r.x;
				y[L + i] = r.y;
			}
		} else {
			float2 *y2 = reinterpret_cast<float2 *>(y);
			for (int i = g.ltid; i < L; i += g.T)
				y2[i] = conjf2(g.ld(i));
		}
	} else if (op == FGK_OP_KERNEL) {
		const int32_t *__restrict__ kidx = p.kidx;
		const int kvw = (int)p.kvw;
		for (int i = g.ltid; i < L; i += g.T) {
			const float2 v = g.ld(i);
			const int o = __ldg(kidx + i);
			y[o] = v.x;
			y[o + kvw] = v.y;
		}
	} else if (freqoff) {
		const int half = L >> 1;
		float2 *y2 = reinterpret_cast<float2 *>(y);
		for (int m = g.ltid; m < half; m += g.T) {
			const float2 a = g.ld(m), b = g.ld(L - 1 - m);
			y2[2 * m] = a;
			y2[2 * m + 1] = conjf2(b);
		}
		if ((L & 1) && g.ltid == 0)
			y2[L - 1] = g.ld(half);
	} else {
		float2 *y2 = reinterpret_cast<float2 *>(y);
		for (int i = g.ltid; i < L; i += g.T)
			y2[i] = g.ld(i);
	}
}

/* Generic resident kernel: any plan, any op, per_cta groups per CTA. */
template <int EMAX>
__global__ void __launch_bounds__(1024, 1) resident_generic(const fgk_plan p, int op, float *out, const float *in,
                                                         const float *__restrict__ kern, uint32_t count,
                                                         size_t in_stride, size_t out_stride)
{
	extern __shared__ float2 smem[];
	Group g;
	g.L = (int)p.L;
	g.T = (int)p.threads;
	g.pad = (int)p.pad;
	const int grp = (int)(threadIdx.x / p.threads);
	g.ltid = (int)threadIdx.x - grp * g.T;
	const uint64_t t = (uint64_t)blockIdx.x * p.per_cta + (uint64_t)grp;
	g.active = grp < (int)p.per_cta && t < count;
	g.sm = smem + (size_t)(grp < (int)p.per_cta ? grp : 0) * p.smem_stride;
	const uint64_t tt = g.active ? t : 0;
	generic_one<EMAX>(p, g, op, out + tt * out_stride, in + tt * in_stride, kern);
}

/* The call service of the generic kernel (fgk.h, fgk_serve_words; the
 * doorbell protocol is fgk_serve.cuh's): one CTA, one group, one transform
 * per request through the same stages as resident_generic, so the same
 * bits, without a launch per request. */
template <int EMAX>
__global__ void __launch_bounds__(1024, 1) resident_serve(const fgk_plan p, fgk_serve_words w, uint64_t seen,
                                                       uint64_t id, uint32_t idle_polls)
{
	extern __shared__ float2 smem[];
	__shared__ ServeSlot slot;
	Group g;
	g.L = (int)p.L;
	g.T = (int)p.threads;
	g.pad = (int)p.pad;
	g.ltid = (int)threadIdx.x;
	g.active = (int)threadIdx.x < g.T;
	g.sm = smem;
	for (;;) {
		if (threadIdx.x == 0)
			serve_next(w, seen, id, idle_polls, slot);
		__syncthreads();
		if (slot.op < 0)
			break;
		generic_one<EMAX>(p, g, slot.op, reinterpret_cast<float *>(slot.out),
		                  reinterpret_cast<const float *>(slot.in), reinterpret_cast<const float *>(slot.kern));
		__syncthreads();
		if (threadIdx.x == 0)
			serve_reply(w, slot);
	}
}

typedef void (*resident_fn)(const fgk_plan, int, float *, const float *, const float *, uint32_t, size_t, size_t);
typedef void (*resident_serve_fn)(const fgk_plan, fgk_serve_words, uint64_t, uint64_t, uint32_t);

} /* namespace fgk */

static unsigned long long fgk_launches;

extern "C" void fgk_count_launch(void)
{
	__atomic_fetch_add(&fgk_launches, 1ull, __ATOMIC_RELAXED);
}

extern "C" unsigned long long fftset__launch_count(void)
{
	return __atomic_load_n(&fgk_launches, __ATOMIC_RELAXED);
}

extern "C" int fgk_launch_resident_serve(const fgk_plan *p, fgk_serve_words w, uint64_t seen, uint64_t id,
                                         uint32_t idle_polls, void *stream)
{
	using namespace fgk;
	if (id == 0 || idle_polls == 0 || p->threads == 0 || p->threads > 1024)
		return -1;
	resident_serve_fn fn = p->emax > 16 ? resident_serve<32> : resident_serve<16>;
	const uint32_t threads = (p->threads + 31u) & ~31u;
	const size_t smem = (size_t)p->smem_stride * sizeof(float2);
	if (smem > 48 * 1024) {
		cudaError_t e = cudaFuncSetAttribute((const void *)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		if (e != cudaSuccess)
			return (int)e;
	}
	fn<<<1, threads, smem, (cudaStream_t)stream>>>(*p, w, seen, id, idle_polls);
	fgk_count_launch();
	return (int)cudaGetLastError();
}

extern "C" uint32_t fgk_max_resident_L(void)
{
	return 26244u; /* largest 2^a 3^b 5^c whose padded buffer fits 227 KB */
}

extern "C" int fgk_launch_resident(const fgk_plan *p, int op, float *out, const float *in, const float *kern,
                                   uint32_t count, size_t in_stride, size_t out_stride, void *stream)
{
	using namespace fgk;
	if (count == 0)
		return 0;
	if (op < 0 || op >= FGK_OP_COUNT)
		return (int)cudaErrorInvalidValue;
	resident_fn fn = p->emax > 16 ? resident_generic<32> : resident_generic<16>;
	const uint32_t threads = ((p->per_cta * p->threads) + 31u) & ~31u;
	const size_t smem = (size_t)p->per_cta * p->smem_stride * sizeof(float2);
	if (smem > 48 * 1024) {
		cudaError_t e = cudaFuncSetAttribute((const void *)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		if (e != cudaSuccess)
			return (int)e;
	}
	const uint64_t blocks = ((uint64_t)count + p->per_cta - 1) / p->per_cta;
	if (blocks > 0x7fffffffull)
		return (int)cudaErrorInvalidValue;
	fn<<<(unsigned)blocks, threads, smem, (cudaStream_t)stream>>>(*p, op, out, in, kern, count, in_stride, out_stride);
	fgk_count_launch();
	return (int)cudaGetLastError();
}

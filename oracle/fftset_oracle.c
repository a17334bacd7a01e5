/* ORACLE TEST INFRASTRUCTURE -- not part of the product.
 *
 * CPU restatement of fftset's transform and fast-convolution path
 * (templeblock/fftset), used only by tests/, by __graft_entry__.smoke() to
 * check its results, and by bench.py as the timed CPU baseline ("port"). It follows the
 * reference algorithm step by step:
 *
 *   planner          src/fftset_vec.c:945-971 (radix table), :1004-1062
 *                    (build_float_graph cost model and tie-breaking)
 *   pass twiddles    src/fftset_vec.c:1103-1109
 *   in-place DIF     src/fftset_vec.c:65-77 (BUILD_STANDARD_PASSES _dif),
 *                    :1161-1186 (fftset_vec_dif_passes)
 *   mulconj + DIT    src/fftset_vec.c:847-867, :1188-1196
 *   outer passes     src/fftset_mod_cplx.c:33-152 (COMPLEX, width 4),
 *                    :242-318 (width 1); src/fftset_mod_freqoffsetreal.c:
 *                    572-782 (width 4), :36-470 (width 8), :884-1010 (width 1)
 *   modulation init  src/fftset_mod_freqoffsetreal.c:1012-1131,
 *                    src/fftset_mod_cplx.c:320-347
 *
 * Data layout ("lane layout") is the reference's: a buffer of 2*L floats is
 * M = L/V slots; slot s holds V real parts then V imaginary parts
 * (src/fftset_vec.c:112-115). Lane l of slot s is element s of sub-sequence l.
 * V is 1, 4 or 8 and is picked per (modulation, L) exactly as the reference's
 * init functions pick their v1f / v4f / v8f branch for a given SIMD build
 * (build_vw = 1, 4 or 8).
 *
 * Forward and inverse are restated through the same DIF machinery followed by
 * a digit-reversal gather, instead of the reference's Stockham passes
 * (src/fftset_vec.c:1222-1249); both compute the same DFT with the same
 * twiddle values, so results agree to rounding. The inverse restates the
 * reference's conj -> forward -> conj structure (src/fftset_mod_cplx.c:212-239,
 * src/fftset_mod_freqoffsetreal.c:974-1010).
 *
 * Everything is FP32 like the reference, with its twiddle formulas. */
#define _GNU_SOURCE
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#define OR_MAX_CHAIN 40
#define OR_MOD_COMPLEX 0
#define OR_MOD_FREQOFF 1

/* ------------------------------------------------------------------------
 * Planner (src/fftset_vec.c:945-971, :1004-1062).
 * Table order per width: 2,3,4 usable at any stage; 5,6,8,16 last only.
 * cost = 100 + ((r+2)*(w+3)*10000)/(r*w), integer arithmetic (:1023).
 * The reference searches exhaustively and keeps the first candidate (in table
 * order) with a strictly lower total; the optimum for a sub-length does not
 * depend on the prefix, so a memo per length gives the same chain. */
static const unsigned OR_RADIX[7] = {2, 3, 4, 5, 6, 8, 16};

static unsigned or_pass_cost(unsigned r, unsigned w)
{
	return 100u + ((r + 2u) * (w + 3u) * 10000u) / (r * w);
}

/* Returns total cost (0 = impossible); fills chain[0..*n). */
static unsigned or_best_chain(unsigned length, unsigned w, unsigned *chain, unsigned *n)
{
	unsigned best_cost = 0, best_n = 0, i;
	unsigned best_chain[OR_MAX_CHAIN];
	for (i = 0; i < 7; i++) {
		unsigned r = OR_RADIX[i];
		unsigned c = or_pass_cost(r, w);
		if (length == r) {
			if (best_cost == 0 || best_cost > c) {
				best_cost = c;
				best_chain[0] = r;
				best_n = 1;
			}
			continue;
		}
		if (r > 4 || (length % r) != 0)
			continue;
		{
			unsigned sub[OR_MAX_CHAIN], sn = 0, sc;
			sc = or_best_chain(length / r, w, sub, &sn);
			if (sc == 0 || sn + 1 > OR_MAX_CHAIN)
				continue;
			if (best_cost == 0 || best_cost > sc + c) {
				best_cost = sc + c;
				best_chain[0] = r;
				memcpy(best_chain + 1, sub, sn * sizeof(unsigned));
				best_n = sn + 1;
			}
		}
	}
	if (best_cost) {
		memcpy(chain, best_chain, best_n * sizeof(unsigned));
		*n = best_n;
	}
	return best_cost;
}

/* Exported: radix chain for an inner transform of `length` at width `w`.
 * Returns the number of passes, 0 when the length has no chain. */
unsigned oracle_plan_chain(unsigned length, unsigned w, unsigned *chain)
{
	unsigned n = 0;
	if (length < 2)
		return 0;
	if (!or_best_chain(length, w, chain, &n))
		return 0;
	return n;
}

/* Lane width used for (modulation, L) by a reference built with SIMD width
 * build_vw: src/fftset_mod_cplx.c:322 (COMPLEX uses 4 when L>4 and L%4==0),
 * src/fftset_mod_freqoffsetreal.c:1016,1073 (8 when L%32==0, 4 when L%16==0). */
unsigned oracle_lane_width(int modulation, unsigned L, unsigned build_vw)
{
	if (modulation == OR_MOD_COMPLEX) {
		if (build_vw >= 4 && L > 4 && (L % 4) == 0)
			return 4;
		return 1;
	}
	if (build_vw >= 8 && L >= 32 && (L % 32) == 0)
		return 8;
	if (build_vw >= 4 && L >= 16 && (L % 16) == 0)
		return 4;
	return 1;
}

/* Digit reversal of an in-place DIF chain: slot s = q*(len/r) + s' holds bin
 * q + r*rev(s') of the length-len DFT (src/fftset_vec.c:65-77 write output q
 * of column j to j + q*lfft, then recurse on each block). */
static unsigned or_dif_bin(const unsigned *chain, unsigned n, unsigned len, unsigned s)
{
	unsigned bin = 0, mul = 1, i;
	for (i = 0; i < n; i++) {
		unsigned r = chain[i];
		unsigned m = len / r;
		unsigned q = s / m;
		s -= q * m;
		bin += mul * q;
		mul *= r;
		len = m;
	}
	return bin;
}

/* Exported: float offset of the real part of every DFT bin inside the
 * kernel buffer written by fftset_fft_conv_get_kernel; the imaginary part
 * is at re_off[bin] + V. Returns V, or 0 if the size has no plan. */
unsigned oracle_kernel_offsets(int modulation, unsigned L, unsigned build_vw, unsigned *re_off)
{
	unsigned V = oracle_lane_width(modulation, L, build_vw);
	unsigned M = L / V, chain[OR_MAX_CHAIN], n, s, l;
	n = oracle_plan_chain(M, V, chain);
	if (n == 0)
		return 0;
	for (s = 0; s < M; s++) {
		unsigned b = or_dif_bin(chain, n, M, s);
		for (l = 0; l < V; l++)
			re_off[l + V * b] = 2 * V * s + l;
	}
	return V;
}

/* ------------------------------------------------------------------------
 * Plans */
struct or_pass {
	unsigned radix;
	unsigned len;      /* transform length this pass splits */
	unsigned m;        /* len / radix (columns) */
	float   *tw;       /* m * (radix-1) complex, column-major per column */
};

struct oracle_plan {
	int           modulation;
	unsigned      L, V, M;
	unsigned      npass;
	struct or_pass pass[OR_MAX_CHAIN];
	unsigned     *bin_of_slot;   /* M entries */
	float        *outer_tw;      /* width 4/8 outer twiddles, see or_make_outer */
	float        *mod_tw;        /* width 1 FREQOFF modulation cos/sin per i */
};

/* src/fftset_vec.c:1103-1109 */
static int or_make_pass_tw(struct or_pass *p)
{
	unsigned j, k;
	float *t;
	if (p->m == 1) {
		p->tw = NULL;
		return 0;
	}
	t = (float *)malloc(sizeof(float) * 2 * (p->radix - 1) * p->m);
	if (!t)
		return -1;
	p->tw = t;
	for (j = 0; j < p->m; j++)
		for (k = 1; k < p->radix; k++) {
			*t++ = cosf(j * k * (-(float)M_PI * 2) / p->len);
			*t++ = sinf(j * k * (-(float)M_PI * 2) / p->len);
		}
	return 0;
}

/* Outer twiddles for width 4 / 8. Index n < L/4 (position inside a quarter):
 *   FREQOFF: modulation e^{j(fi + q*off)} for the four quarters q (4 complex)
 *            and radix-4 twiddles e^{j fi*4*k}, k=1..3 (3 complex), with
 *            off = -pi/8, fi = n*off/(L/4)  (src/fftset_mod_freqoffsetreal.c:
 *            1036-1061 and :1093-1108);
 *   COMPLEX: radix-4 twiddles e^{-j2pi n k / L}, k=1..3, evaluated as the
 *            reference does inline (src/fftset_mod_cplx.c:69-83).
 * Stored as 14 floats per n. For width 8 a second table of L/8 complex
 * radix-2 twiddles e^{-j2pi n/(L/4)} follows (:1057-1061). */
static int or_make_outer(struct oracle_plan *p)
{
	unsigned L = p->L, n;
	unsigned Q = L / 4;
	size_t sz = 14 * (size_t)Q + (p->V == 8 ? 2 * (size_t)(L / 8) : 0);
	float *t = (float *)malloc(sizeof(float) * sz);
	if (!t)
		return -1;
	p->outer_tw = t;
	if (p->modulation == OR_MOD_FREQOFF) {
		const float off = (float)(-M_PI * 0.125);
		const float scale = off / (float)(L / 4);
		for (n = 0; n < Q; n++) {
			float fi = n * scale;
			float *tp = t + 14 * n;
			unsigned q;
			for (q = 0; q < 4; q++) {
				tp[2 * q + 0] = cosf(fi + (float)q * off);
				tp[2 * q + 1] = sinf(fi + (float)q * off);
			}
			for (q = 1; q < 4; q++) {
				tp[8 + 2 * (q - 1) + 0] = cosf(fi * 4.0f * (float)q);
				tp[8 + 2 * (q - 1) + 1] = sinf(fi * 4.0f * (float)q);
			}
		}
	} else {
		for (n = 0; n < Q; n++) {
			float *tp = t + 14 * n;
			unsigned q;
			for (q = 0; q < 4; q++) {
				tp[2 * q + 0] = 1.0f;
				tp[2 * q + 1] = 0.0f;
			}
			for (q = 1; q < 4; q++) {
				tp[8 + 2 * (q - 1) + 0] = cosf(n * (float)(-2.0 * q * M_PI) / (L / 1));
				tp[8 + 2 * (q - 1) + 1] = sinf(n * (float)(-2.0 * q * M_PI) / (L / 1));
			}
		}
	}
	if (p->V == 8) {
		float *t2 = t + 14 * (size_t)Q;
		for (n = 0; n < L / 8; n++) {
			t2[2 * n + 0] = cosf(-2.0 * n * M_PI / (L / 4));
			t2[2 * n + 1] = sinf(-2.0 * n * M_PI / (L / 4));
		}
	}
	return 0;
}

void oracle_plan_destroy(struct oracle_plan *p)
{
	unsigned i;
	if (!p)
		return;
	for (i = 0; i < p->npass; i++)
		free(p->pass[i].tw);
	free(p->bin_of_slot);
	free(p->outer_tw);
	free(p->mod_tw);
	free(p);
}

/* The composite codelets' internal twiddles w_r^m = e^{-j 2 pi m / r}
 * (r = 6, 8, 16, m < r), each computed once in FP64 and rounded to FP32:
 * the values a per-butterfly cos/sin would give, without calling them for
 * every butterfly. Filled by oracle_plan_create. */
static float or_cw[17][16][2];
static pthread_once_t or_cw_once = PTHREAD_ONCE_INIT;

static void or_cw_init(void)
{
	static const unsigned rs[3] = {6, 8, 16};
	unsigned i, m;
	for (i = 0; i < 3; i++)
		for (m = 0; m < rs[i]; m++) {
			double ang = -2.0 * M_PI * (double)m / (double)rs[i];
			or_cw[rs[i]][m][0] = (float)cos(ang);
			or_cw[rs[i]][m][1] = (float)sin(ang);
		}
}

struct oracle_plan *oracle_plan_create(int modulation, unsigned L, unsigned build_vw)
{
	struct oracle_plan *p;
	unsigned chain[OR_MAX_CHAIN], n, i, len, s;
	if (L < 2)
		return NULL;
	pthread_once(&or_cw_once, or_cw_init);
	p = (struct oracle_plan *)calloc(1, sizeof(*p));
	if (!p)
		return NULL;
	p->modulation = modulation;
	p->L = L;
	p->V = oracle_lane_width(modulation, L, build_vw);
	p->M = L / p->V;
	n = oracle_plan_chain(p->M, p->V, chain);
	if (n == 0) {
		free(p);
		return NULL;
	}
	p->npass = n;
	len = p->M;
	for (i = 0; i < n; i++) {
		p->pass[i].radix = chain[i];
		p->pass[i].len = len;
		p->pass[i].m = len / chain[i];
		if (or_make_pass_tw(&p->pass[i]))
			goto fail;
		len /= chain[i];
	}
	p->bin_of_slot = (unsigned *)malloc(sizeof(unsigned) * p->M);
	if (!p->bin_of_slot)
		goto fail;
	for (s = 0; s < p->M; s++)
		p->bin_of_slot[s] = or_dif_bin(chain, n, p->M, s);
	if (p->V > 1 && or_make_outer(p))
		goto fail;
	if (p->V == 1 && modulation == OR_MOD_FREQOFF) {
		/* src/fftset_mod_freqoffsetreal.c:890-892 */
		p->mod_tw = (float *)malloc(sizeof(float) * 2 * L);
		if (!p->mod_tw)
			goto fail;
		for (i = 0; i < L; i++) {
			p->mod_tw[2 * i + 0] = cosf(-2.0f * (float)M_PI * i / (L * 4.0f));
			p->mod_tw[2 * i + 1] = sinf(-2.0f * (float)M_PI * i / (L * 4.0f));
		}
	}
	return p;
fail:
	oracle_plan_destroy(p);
	return NULL;
}

unsigned oracle_plan_lanes(const struct oracle_plan *p) { return p->V; }

/* ------------------------------------------------------------------------
 * Small DFT codelets on one lane (natural-order outputs, forward sign).
 * Constants are the exact values of cos/sin of the angles named. */
#define OR_C3 0.86602540378443864676f  /* sin(pi/3) */
#define OR_C5A 0.30901699437494742410f /* cos(2pi/5) */
#define OR_C5B 0.95105651629515357212f /* sin(2pi/5) */
#define OR_C5C 0.80901699437494742410f /* cos(pi/5) */
#define OR_C5D 0.58778525229247312917f /* sin(pi/5) */
#define OR_R2  0.70710678118654752440f

typedef float or_v4 __attribute__((vector_size(16)));

#define OR_T float
#define OR_SFX
#include "fftset_oracle_codelets.h"
#undef OR_T
#undef OR_SFX
#define OR_T or_v4
#define OR_SFX _v4
#include "fftset_oracle_codelets.h"
#undef OR_T
#undef OR_SFX

/* ------------------------------------------------------------------------
 * Passes over the lane layout. x points at slot 0; slot s real lane l is
 * x[2V s + l], imaginary x[2V s + V + l]. */
static inline or_v4 or_ld4(const float *p)
{
	or_v4 v;
	memcpy(&v, p, sizeof v);
	return v;
}

static inline void or_st4(float *p, or_v4 v) { memcpy(p, &v, sizeof v); }

/* Four lanes at a time (V a multiple of 4): the same operations per lane as
 * the one-lane loops below. */
static void or_pass_dif_v4(const struct or_pass *ps, unsigned V, unsigned nblk, float *x)
{
	unsigned r = ps->radix, m = ps->m, b, j, p, l;
	or_v4 re[16], im[16];
	for (b = 0; b < nblk; b++) {
		float *blk = x + (size_t)b * r * m * 2 * V;
		for (j = 0; j < m; j++) {
			const float *tw = ps->tw ? ps->tw + 2 * (r - 1) * j : NULL;
			for (l = 0; l < V; l += 4) {
				for (p = 0; p < r; p++) {
					re[p] = or_ld4(blk + 2 * V * (j + p * m) + l);
					im[p] = or_ld4(blk + 2 * V * (j + p * m) + V + l);
				}
				or_dft_small_v4(r, re, im);
				for (p = 0; p < r; p++) {
					or_v4 orr = re[p], oi = im[p];
					if (tw && p) {
						float wr = tw[2 * (p - 1)], wi = tw[2 * (p - 1) + 1];
						orr = re[p] * wr - im[p] * wi;
						oi = re[p] * wi + im[p] * wr;
					}
					or_st4(blk + 2 * V * (j + p * m) + l, orr);
					or_st4(blk + 2 * V * (j + p * m) + V + l, oi);
				}
			}
		}
	}
}

static void or_pass_dit_v4(const struct or_pass *ps, unsigned V, unsigned nblk, float *x)
{
	unsigned r = ps->radix, m = ps->m, b, j, p, l;
	or_v4 re[16], im[16];
	for (b = 0; b < nblk; b++) {
		float *blk = x + (size_t)b * r * m * 2 * V;
		for (j = 0; j < m; j++) {
			const float *tw = ps->tw ? ps->tw + 2 * (r - 1) * j : NULL;
			for (l = 0; l < V; l += 4) {
				for (p = 0; p < r; p++) {
					or_v4 ir = or_ld4(blk + 2 * V * (j + p * m) + l);
					or_v4 ii = or_ld4(blk + 2 * V * (j + p * m) + V + l);
					if (tw && p) {
						float wr = tw[2 * (p - 1)], wi = tw[2 * (p - 1) + 1];
						re[p] = ir * wr - ii * wi;
						im[p] = ir * wi + ii * wr;
					} else {
						re[p] = ir;
						im[p] = ii;
					}
				}
				or_dft_small_v4(r, re, im);
				for (p = 0; p < r; p++) {
					or_st4(blk + 2 * V * (j + p * m) + l, re[p]);
					or_st4(blk + 2 * V * (j + p * m) + V + l, im[p]);
				}
			}
		}
	}
}

static void or_pass_dif(const struct or_pass *ps, unsigned V, unsigned nblk, float *x)
{
	unsigned r = ps->radix, m = ps->m, b, j, p, l;
	float re[16], im[16];
	if (V % 4 == 0) {
		or_pass_dif_v4(ps, V, nblk, x);
		return;
	}
	for (b = 0; b < nblk; b++) {
		float *blk = x + (size_t)b * r * m * 2 * V;
		for (j = 0; j < m; j++) {
			const float *tw = ps->tw ? ps->tw + 2 * (r - 1) * j : NULL;
			for (l = 0; l < V; l++) {
				for (p = 0; p < r; p++) {
					re[p] = blk[2 * V * (j + p * m) + l];
					im[p] = blk[2 * V * (j + p * m) + V + l];
				}
				or_dft_small(r, re, im);
				for (p = 0; p < r; p++) {
					float orr = re[p], oi = im[p];
					if (tw && p) {
						float wr = tw[2 * (p - 1)], wi = tw[2 * (p - 1) + 1];
						orr = re[p] * wr - im[p] * wi;
						oi = re[p] * wi + im[p] * wr;
					}
					blk[2 * V * (j + p * m) + l] = orr;
					blk[2 * V * (j + p * m) + V + l] = oi;
				}
			}
		}
	}
}

static void or_pass_dit(const struct or_pass *ps, unsigned V, unsigned nblk, float *x)
{
	unsigned r = ps->radix, m = ps->m, b, j, p, l;
	float re[16], im[16];
	if (V % 4 == 0) {
		or_pass_dit_v4(ps, V, nblk, x);
		return;
	}
	for (b = 0; b < nblk; b++) {
		float *blk = x + (size_t)b * r * m * 2 * V;
		for (j = 0; j < m; j++) {
			const float *tw = ps->tw ? ps->tw + 2 * (r - 1) * j : NULL;
			for (l = 0; l < V; l++) {
				for (p = 0; p < r; p++) {
					float ir = blk[2 * V * (j + p * m) + l];
					float ii = blk[2 * V * (j + p * m) + V + l];
					if (tw && p) {
						float wr = tw[2 * (p - 1)], wi = tw[2 * (p - 1) + 1];
						re[p] = ir * wr - ii * wi;
						im[p] = ir * wi + ii * wr;
					} else {
						re[p] = ir;
						im[p] = ii;
					}
				}
				or_dft_small(r, re, im);
				for (p = 0; p < r; p++) {
					blk[2 * V * (j + p * m) + l] = re[p];
					blk[2 * V * (j + p * m) + V + l] = im[p];
				}
			}
		}
	}
}

static void or_dif_chain(const struct oracle_plan *p, float *x)
{
	unsigned i, nblk = 1;
	for (i = 0; i < p->npass; i++) {
		or_pass_dif(&p->pass[i], p->V, nblk, x);
		nblk *= p->pass[i].radix;
	}
}

static void or_dit_chain(const struct oracle_plan *p, float *x)
{
	unsigned i, nblk = 1;
	for (i = 0; i < p->npass; i++)
		nblk *= p->pass[i].radix;
	for (i = p->npass; i-- > 0;) {
		nblk /= p->pass[i].radix;
		or_pass_dit(&p->pass[i], p->V, nblk, x);
	}
}

/* Outer pass into the lane layout.
 * in: FREQOFF = 2L reals; COMPLEX = L interleaved complex.
 * Produces the modulated sequence c (FREQOFF: c[i] = conj(x[i] + j x[L+i]) *
 * e^{-j pi i/(2L)}; COMPLEX: c = x), then (V>1) one radix-4 DIF step over the
 * four quarters with twiddles w_L^{n k} (lane k), and (V=8) one radix-2 DIF
 * step inside each lane with twiddle w_{L/4}^{n} (lane k + 4 q2). */
static void or_outer_forward(const struct oracle_plan *p, float *w, const float *in)
{
	unsigned L = p->L, V = p->V, i;
	if (V == 1) {
		if (p->modulation == OR_MOD_FREQOFF) {
			for (i = 0; i < L; i++) {
				float re = in[i], im = in[L + i];
				float twr = p->mod_tw[2 * i], twi = p->mod_tw[2 * i + 1];
				w[2 * i + 0] = re * twr + im * twi;
				w[2 * i + 1] = re * twi - im * twr;
			}
		} else {
			memcpy(w, in, sizeof(float) * 2 * L);
		}
		return;
	}
	{
		unsigned Q = L / 4, n, q;
		/* quarter-lane sequences a_k[n], k<4, n<Q, written to slot n lane k of
		 * a width-4 scratch view when V == 4, or to slot (n mod Q/2),
		 * lane k + 4*(n >= Q/2) before the radix-2 step when V == 8. */
		for (n = 0; n < Q; n++) {
			const float *tp = p->outer_tw + 14 * (size_t)n;
			float re[4], im[4];
			for (q = 0; q < 4; q++) {
				float xr, xi;
				if (p->modulation == OR_MOD_FREQOFF) {
					float zr = in[q * Q + n], zi = in[L + q * Q + n];
					float twr = tp[2 * q], twi = tp[2 * q + 1];
					xr = twr * zr + twi * zi;
					xi = twi * zr - twr * zi;
				} else {
					xr = in[2 * (q * Q + n)];
					xi = in[2 * (q * Q + n) + 1];
				}
				re[q] = xr;
				im[q] = xi;
			}
			or_dft4(re, im);
			for (q = 1; q < 4; q++) {
				float wr = tp[8 + 2 * (q - 1)], wi = tp[8 + 2 * (q - 1) + 1];
				float tr = re[q] * wr - im[q] * wi;
				float ti = re[q] * wi + im[q] * wr;
				re[q] = tr;
				im[q] = ti;
			}
			if (V == 4) {
				for (q = 0; q < 4; q++) {
					w[8 * n + q] = re[q];
					w[8 * n + 4 + q] = im[q];
				}
			} else {
				unsigned h = Q / 2, s = n % h, half = n / h;
				for (q = 0; q < 4; q++) {
					w[16 * s + 4 * half + q] = re[q];
					w[16 * s + 8 + 4 * half + q] = im[q];
				}
			}
		}
		if (V == 8) {
			const float *t2 = p->outer_tw + 14 * (size_t)Q;
			unsigned s;
			for (s = 0; s < L / 8; s++) {
				float wr = t2[2 * s], wi = t2[2 * s + 1];
				for (q = 0; q < 4; q++) {
					float ar = w[16 * s + q], ai = w[16 * s + 8 + q];
					float br = w[16 * s + 4 + q], bi = w[16 * s + 12 + q];
					float dr = ar - br, di = ai - bi;
					w[16 * s + q] = ar + br;
					w[16 * s + 8 + q] = ai + bi;
					w[16 * s + 4 + q] = dr * wr - di * wi;
					w[16 * s + 12 + q] = dr * wi + di * wr;
				}
			}
		}
	}
}

/* Inverse of the outer structure for the convolution's last step. Input: the
 * lane layout holding, per lane, the natural-order DFT of the conjugated
 * product (the DIT chain's output). Recombines lanes (radix-2 then radix-4
 * with forward twiddles, the DIT mirror of or_outer_forward) into the
 * natural-order length-L sequence u, then writes
 *   FREQOFF: y[i] = Re(u_i * e^{-j pi i/(2L)}), y[L+i] = Im(...)
 *   COMPLEX: y[i] = conj(u_i)
 * (src/fftset_mod_freqoffsetreal.c:678-782, :941-954;
 *  src/fftset_mod_cplx.c:88-152, :264-271). */
static void or_outer_final(const struct oracle_plan *p, float *y, float *w)
{
	unsigned L = p->L, V = p->V, i;
	if (V == 1) {
		for (i = 0; i < L; i++) {
			float re = w[2 * i], im = w[2 * i + 1];
			if (p->modulation == OR_MOD_FREQOFF) {
				float twr = p->mod_tw[2 * i], twi = p->mod_tw[2 * i + 1];
				y[i] = re * twr - im * twi;
				y[L + i] = re * twi + im * twr;
			} else {
				y[2 * i] = re;
				y[2 * i + 1] = -im;
			}
		}
		return;
	}
	{
		unsigned Q = L / 4, n, q;
		if (V == 8) {
			const float *t2 = p->outer_tw + 14 * (size_t)Q;
			unsigned s;
			for (s = 0; s < L / 8; s++) {
				float wr = t2[2 * s], wi = t2[2 * s + 1];
				for (q = 0; q < 4; q++) {
					float ar = w[16 * s + q], ai = w[16 * s + 8 + q];
					float br0 = w[16 * s + 4 + q], bi0 = w[16 * s + 12 + q];
					float br = br0 * wr - bi0 * wi, bi = br0 * wi + bi0 * wr;
					w[16 * s + q] = ar + br;
					w[16 * s + 8 + q] = ai + bi;
					w[16 * s + 4 + q] = ar - br;
					w[16 * s + 12 + q] = ai - bi;
				}
			}
		}
		for (n = 0; n < Q; n++) {
			const float *tp = p->outer_tw + 14 * (size_t)n;
			float re[4], im[4];
			for (q = 0; q < 4; q++) {
				if (V == 4) {
					re[q] = w[8 * n + q];
					im[q] = w[8 * n + 4 + q];
				} else {
					unsigned h = Q / 2, s = n % h, half = n / h;
					re[q] = w[16 * s + 4 * half + q];
					im[q] = w[16 * s + 8 + 4 * half + q];
				}
			}
			for (q = 1; q < 4; q++) {
				float wr = tp[8 + 2 * (q - 1)], wi = tp[8 + 2 * (q - 1) + 1];
				float tr = re[q] * wr - im[q] * wi;
				float ti = re[q] * wi + im[q] * wr;
				re[q] = tr;
				im[q] = ti;
			}
			or_dft4(re, im);
			for (q = 0; q < 4; q++) {
				unsigned idx = q * Q + n;
				if (p->modulation == OR_MOD_FREQOFF) {
					float twr = tp[2 * q], twi = tp[2 * q + 1];
					y[idx] = twr * re[q] - twi * im[q];
					y[L + idx] = twi * re[q] + twr * im[q];
				} else {
					y[2 * idx] = re[q];
					y[2 * idx + 1] = -im[q];
				}
			}
		}
	}
}

/* Natural-order spectrum W[k] (interleaved complex, L bins) from the DIF
 * output in lane layout: slot s lane l holds W[l + V*bin_of_slot[s]]. */
static void or_gather_natural(const struct oracle_plan *p, float *W, const float *lanes)
{
	unsigned V = p->V, s, l;
	for (s = 0; s < p->M; s++) {
		unsigned b = p->bin_of_slot[s];
		for (l = 0; l < V; l++) {
			unsigned k = l + V * b;
			W[2 * k] = lanes[2 * V * s + l];
			W[2 * k + 1] = lanes[2 * V * s + V + l];
		}
	}
}

/* ------------------------------------------------------------------------
 * Public restated operations (buffers of 2L floats each). */
void oracle_get_kernel(const struct oracle_plan *p, float *out, const float *in)
{
	or_outer_forward(p, out, in);
	or_dif_chain(p, out);
}

/* src/fftset_vec.c:847-867: work = conj(work * kern), lane-wise. */
static void or_mulconj(const struct oracle_plan *p, float *w, const float *k)
{
	unsigned V = p->V, s, l;
	for (s = 0; s < p->M; s++)
		for (l = 0; l < V; l++) {
			float ar = w[2 * V * s + l], ai = w[2 * V * s + V + l];
			float br = k[2 * V * s + l], bi = k[2 * V * s + V + l];
			w[2 * V * s + l] = ar * br - ai * bi;
			w[2 * V * s + V + l] = -(ar * bi + ai * br);
		}
}

void oracle_conv(const struct oracle_plan *p, float *out, const float *in, const float *kern, float *work)
{
	or_outer_forward(p, work, in);
	or_dif_chain(p, work);
	or_mulconj(p, work, kern);
	or_dit_chain(p, work);
	or_outer_final(p, out, work);
}

/* Forward: DFT of c via the DIF machinery, gathered to natural order, then
 * (FREQOFF) X[2m] = W[m], X[2m+1] = conj W[L-1-m]
 * (src/fftset_mod_freqoffsetreal.c:958-971). */
void oracle_forward(const struct oracle_plan *p, float *out, const float *in, float *work)
{
	unsigned L = p->L, m;
	float *W = (float *)malloc(sizeof(float) * 2 * L);
	if (!W)
		return;
	or_outer_forward(p, work, in);
	or_dif_chain(p, work);
	or_gather_natural(p, W, work);
	if (p->modulation == OR_MOD_COMPLEX) {
		memcpy(out, W, sizeof(float) * 2 * L);
	} else {
		for (m = 0; m < L; m++) {
			unsigned k = (m & 1) ? (L - 1 - (m - 1) / 2) : m / 2;
			out[2 * m] = W[2 * k];
			out[2 * m + 1] = (m & 1) ? -W[2 * k + 1] : W[2 * k + 1];
		}
	}
	free(W);
}

/* Inverse (unnormalised, inverse(forward(x)) = L x): rebuild conj(W) in
 * natural order, take its forward DFT u = conj(IDFT(W)), then apply the final
 * step of or_outer_final to u. */
void oracle_inverse(const struct oracle_plan *p, float *out, const float *in, float *work)
{
	unsigned L = p->L, m, i;
	float *c = (float *)malloc(sizeof(float) * 2 * L);
	float *u = (float *)malloc(sizeof(float) * 2 * L);
	if (!c || !u) {
		free(c);
		free(u);
		return;
	}
	for (m = 0; m < L; m++) {
		unsigned k;
		float re = in[2 * m], im = in[2 * m + 1];
		if (p->modulation == OR_MOD_FREQOFF) {
			k = (m & 1) ? (L - 1 - (m - 1) / 2) : m / 2;
			if (m & 1)
				im = -im;
		} else {
			k = m;
		}
		c[2 * k] = re;
		c[2 * k + 1] = -im;
	}
	{
		/* forward DFT of c as a COMPLEX transform of the same lane width */
		struct oracle_plan q = *p;
		q.modulation = OR_MOD_COMPLEX;
		if (p->V > 1) {
			/* COMPLEX outer twiddles differ from FREQOFF ones: build them */
			q.outer_tw = NULL;
			if (or_make_outer(&q)) {
				free(c);
				free(u);
				return;
			}
		}
		or_outer_forward(&q, work, c);
		or_dif_chain(&q, work);
		or_gather_natural(&q, u, work);
		if (p->V > 1)
			free(q.outer_tw);
	}
	for (i = 0; i < L; i++) {
		float re = u[2 * i], im = u[2 * i + 1];
		if (p->modulation == OR_MOD_FREQOFF) {
			double ang = -M_PI * (double)i / (2.0 * L);
			float twr = (float)cos(ang), twi = (float)sin(ang);
			out[i] = re * twr - im * twi;
			out[L + i] = re * twi + im * twr;
		} else {
			out[2 * i] = re;
			out[2 * i + 1] = -im;
		}
	}
	free(c);
	free(u);
}

/* ------------------------------------------------------------------------
 * Multi-threaded batch driver for the CPU baseline: independent blocks split
 * across threads, one work buffer per thread (execution calls are
 * thread-safe given distinct outputs and work buffers, README.md:38).
 * Returns elapsed wall seconds. op: 0 conv, 1 forward, 2 inverse. */
struct or_job {
	const struct oracle_plan *p;
	int op;
	float *out;
	const float *in;
	const float *kern;
	size_t stride;
	unsigned b0, b1;
};

static void *or_worker(void *arg)
{
	struct or_job *j = (struct or_job *)arg;
	float *work = (float *)malloc(sizeof(float) * 2 * j->p->L);
	unsigned b;
	if (!work)
		return NULL;
	for (b = j->b0; b < j->b1; b++) {
		float *o = j->out + (size_t)b * j->stride;
		const float *i = j->in + (size_t)b * j->stride;
		if (j->op == 0)
			oracle_conv(j->p, o, i, j->kern, work);
		else if (j->op == 1)
			oracle_forward(j->p, o, i, work);
		else
			oracle_inverse(j->p, o, i, work);
	}
	free(work);
	return NULL;
}

double oracle_run_batch(const struct oracle_plan *p, int op, float *out, const float *in, const float *kern,
                        unsigned nblocks, size_t stride, unsigned nthreads)
{
	pthread_t th[512];
	struct or_job jobs[512];
	struct timespec t0, t1;
	unsigned t;
	if (nthreads < 1)
		nthreads = 1;
	if (nthreads > 512)
		nthreads = 512;
	if (nthreads > nblocks)
		nthreads = nblocks ? nblocks : 1;
	clock_gettime(CLOCK_MONOTONIC, &t0);
	for (t = 0; t < nthreads; t++) {
		jobs[t].p = p;
		jobs[t].op = op;
		jobs[t].out = out;
		jobs[t].in = in;
		jobs[t].kern = kern;
		jobs[t].stride = stride;
		jobs[t].b0 = (unsigned)(((unsigned long long)nblocks * t) / nthreads);
		jobs[t].b1 = (unsigned)(((unsigned long long)nblocks * (t + 1)) / nthreads);
		if (pthread_create(&th[t], NULL, or_worker, &jobs[t])) {
			or_worker(&jobs[t]);
			th[t] = 0;
		}
	}
	for (t = 0; t < nthreads; t++)
		if (th[t])
			pthread_join(th[t], NULL);
	clock_gettime(CLOCK_MONOTONIC, &t1);
	return (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
}

/* Planner for the GPU resident transform: picks the radix chain, the thread
 * mapping and the shared-memory layout of one transform of length L, and
 * generates its twiddles in FP64, rounded once to FP32.
 *
 * This is the GPU counterpart of the reference's planner
 * (src/fftset_vec.c:1004-1152) but it optimises a different machine: a chain
 * stage is one shared-memory round trip, so it prefers few, large radices
 * (16, 12, 10, 8, 6 ...) that a single thread computes in registers. The
 * reference's own chain only decides the kernel-buffer layout, which the host
 * layer reproduces separately (fftset_layout.c). */
#include <math.h>
#include <string.h>
#include "fgk.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* Radices with a register codelet, their exponents of 2, 3, 5 and a cost per
 * point per stage (x10): shared-memory store + load + twiddle load + index
 * arithmetic (~4 instructions) plus the codelet's flops per point. */
static const struct {
	uint32_t r, e2, e3, e5, cost;
} FGK_RADIX[] = {
	{16, 4, 0, 0, 195}, {15, 0, 1, 1, 217}, {12, 2, 1, 0, 188}, {10, 1, 0, 1, 182},
	{8, 3, 0, 0, 162},  {6, 1, 1, 0, 163},  {5, 0, 0, 1, 160},  {4, 2, 0, 0, 125},
	{3, 0, 1, 0, 133},  {2, 1, 0, 0, 90},   {9, 0, 2, 0, 218},
};
#define FGK_NRADIX (sizeof(FGK_RADIX) / sizeof(FGK_RADIX[0]))

/* Best chain for 2^a 3^b 5^c: dynamic programme over the exponents (the
 * cost is additive and the order of stages does not change it), ties broken
 * towards fewer stages, then towards the radix listed first. */
#define FGK_MAXE2 32
#define FGK_MAXE3 21
#define FGK_MAXE5 2
static uint32_t best_chain(uint32_t a, uint32_t b, uint32_t c, uint32_t allowed, uint32_t *chain, uint32_t *n)
{
	static uint32_t cost[FGK_MAXE2][FGK_MAXE3][FGK_MAXE5];
	static uint8_t  first[FGK_MAXE2][FGK_MAXE3][FGK_MAXE5];
	static uint8_t  len[FGK_MAXE2][FGK_MAXE3][FGK_MAXE5];
	uint32_t i2, i3, i5, i, k;
	if (a >= FGK_MAXE2 || b >= FGK_MAXE3 || c >= FGK_MAXE5)
		return 0;
	for (i5 = 0; i5 <= c; i5++)
		for (i3 = 0; i3 <= b; i3++)
			for (i2 = 0; i2 <= a; i2++) {
				uint32_t best = 0, bl = 0, bf = 0;
				if (i2 == 0 && i3 == 0 && i5 == 0) {
					cost[0][0][0] = 1; /* possible, empty */
					len[0][0][0] = 0;
					continue;
				}
				for (i = 0; i < FGK_NRADIX; i++) {
					uint32_t sc, tot;
					if (!(allowed & (1u << i)))
						continue;
					if (FGK_RADIX[i].e2 > i2 || FGK_RADIX[i].e3 > i3 || FGK_RADIX[i].e5 > i5)
						continue;
					sc = cost[i2 - FGK_RADIX[i].e2][i3 - FGK_RADIX[i].e3][i5 - FGK_RADIX[i].e5];
					if (sc == 0)
						continue;
					tot = sc + FGK_RADIX[i].cost;
					k = len[i2 - FGK_RADIX[i].e2][i3 - FGK_RADIX[i].e3][i5 - FGK_RADIX[i].e5] + 1u;
					if (best == 0 || tot < best || (tot == best && k < bl)) {
						best = tot;
						bl = k;
						bf = i;
					}
				}
				cost[i2][i3][i5] = best;
				len[i2][i3][i5] = (uint8_t)bl;
				first[i2][i3][i5] = (uint8_t)bf;
			}
	if (cost[a][b][c] == 0 || len[a][b][c] > FGK_MAX_STAGES)
		return 0;
	*n = 0;
	while (a || b || c) {
		uint32_t r = first[a][b][c];
		chain[(*n)++] = FGK_RADIX[r].r;
		a -= FGK_RADIX[r].e2;
		b -= FGK_RADIX[r].e3;
		c -= FGK_RADIX[r].e5;
	}
	return 1;
}

static int factor235(uint32_t L, uint32_t *a, uint32_t *b, uint32_t *c)
{
	*a = *b = *c = 0;
	if (L < 2)
		return -1;
	while (L % 2 == 0) { L /= 2; (*a)++; }
	while (L % 3 == 0) { L /= 3; (*b)++; }
	while (L % 5 == 0) { L /= 5; (*c)++; }
	return L == 1 ? 0 : -1;
}

/* Chain of radices, largest first: then every stage after the first sees
 * ns >= 16 when the first radix is 16, which keeps the Stockham scatter free of
 * shared-memory bank conflicts under the i + i/16 padding. */
/* radix sets: all codelets, or only those whose register tile divides a
 * 16/32-element budget well (used when the full set needs > 1024 threads) */
#define FGK_ALL_RADICES 0x7ffu
#define FGK_SMALL_RADICES ((1u << 0) | (1u << 4) | (1u << 6) | (1u << 7) | (1u << 8) | (1u << 9))

static int plan_chain_set(uint32_t L, uint32_t allowed, uint32_t *radices, uint32_t *nstages)
{
	uint32_t a, b, c, i, j;
	if (factor235(L, &a, &b, &c))
		return -1;
	if (!best_chain(a, b, c, allowed, radices, nstages))
		return -1;
	for (i = 0; i < *nstages; i++)
		for (j = i + 1; j < *nstages; j++)
			if (radices[j] > radices[i]) {
				uint32_t t = radices[i];
				radices[i] = radices[j];
				radices[j] = t;
			}
	return 0;
}

int fgk_plan_chain(uint32_t L, uint32_t *radices, uint32_t *nstages)
{
	return plan_chain_set(L, FGK_ALL_RADICES, radices, nstages);
}

/* Register budget: complex elements one thread holds per stage. Must match
 * the kernels' FGK_EMAX_SMALL / FGK_EMAX_LARGE. */
static uint32_t bmax(uint32_t r, uint32_t emax)
{
	uint32_t b = emax / r;
	return b ? b : 1;
}

static void fill_chain(fgk_chain *ch, const uint32_t *rad, uint32_t n, uint32_t L, uint32_t T)
{
	uint32_t s, ns = 1;
	ch->nstages = n;
	ch->reserved = 0;
	ch->code = n <= 15 ? n : 0;
	for (s = 0; s < n && n <= 15; s++)
		ch->code |= (uint64_t)(rad[s] - 1) << (4 * s + 4);
	for (s = 0; s < n; s++) {
		ch->st[s].radix = rad[s];
		ch->st[s].ns = ns;
		ch->st[s].nb = (L / rad[s] + T - 1) / T;
		ch->st[s].tw_off = 0;
		ns *= rad[s];
	}
}

/* Fills everything but the device pointers. Returns 0, or -1 when L has no
 * chain or does not fit in max_smem_bytes of shared memory. */
int fgk_plan_resident(fgk_plan *p, uint32_t L, uint32_t modulation, uint32_t max_smem_bytes,
                      const uint32_t *forced_radices, uint32_t forced_n)
{
	uint32_t rad[FGK_MAX_STAGES], rev[FGK_MAX_STAGES], n, s, T = 0, emax = 16, slots, pad, set;
	static const uint32_t sets[2] = {FGK_ALL_RADICES, FGK_SMALL_RADICES};
	memset(p, 0, sizeof(*p));
	for (set = 0; set < 2; set++) {
		if (forced_radices) {
			uint32_t prod = 1;
			if (forced_n == 0 || forced_n > FGK_MAX_STAGES)
				return -1;
			for (n = 0; n < forced_n; n++) {
				rad[n] = forced_radices[n];
				prod *= rad[n];
			}
			if (prod != L)
				return -1;
		} else if (plan_chain_set(L, sets[set], rad, &n)) {
			return -1;
		}
		for (emax = 16;; emax = 32) {
			T = 1;
			for (s = 0; s < n; s++) {
				uint32_t need = (L / rad[s] + bmax(rad[s], emax) - 1) / bmax(rad[s], emax);
				if (need > T)
					T = need;
			}
			if (T <= 1024 || emax == 32)
				break;
		}
		if (T <= 1024)
			break;
	}
	if (T > 1024)
		return -1;
	/* padded slots: one float2 of padding after every 16 */
	pad = 1;
	slots = L + L / 16 + 1;
	if ((size_t)slots * 8 > max_smem_bytes) {
		pad = 0;
		slots = L;
	}
	if ((size_t)slots * 8 > max_smem_bytes)
		return -1;
	p->L = L;
	p->modulation = modulation;
	p->threads = T;
	p->smem_stride = slots;
	/* several transforms per CTA for small sizes: aim at 256 threads */
	p->per_cta = T >= 256 ? 1 : 256 / T;
	while (p->per_cta > 1 && (size_t)p->per_cta * slots * 8 > 48 * 1024)
		p->per_cta--;
	p->pad = pad;
	p->emax = emax;
	fill_chain(&p->fwd, rad, n, L, T);
	for (s = 0; s < n; s++)
		rev[s] = rad[n - 1 - s];
	fill_chain(&p->inv, rev, n, L, T);
	return 0;
}

static size_t chain_twiddles(fgk_chain *ch, float *tw, size_t off)
{
	uint32_t s, k, q;
	for (s = 0; s < ch->nstages; s++) {
		uint32_t r = ch->st[s].radix, ns = ch->st[s].ns;
		ch->st[s].tw_off = (uint32_t)off;
		if (ns == 1)
			continue;
		for (k = 0; k < ns; k++)
			for (q = 1; q < r; q++) {
				if (tw) {
					double ang = -2.0 * M_PI * (double)((uint64_t)q * k) / ((double)ns * r);
					tw[2 * off + 0] = (float)cos(ang);
					tw[2 * off + 1] = (float)sin(ang);
				}
				off++;
			}
	}
	return off;
}

size_t fgk_plan_twiddles(fgk_plan *p, void *tw_host_float2)
{
	float *tw = (float *)tw_host_float2;
	size_t off = chain_twiddles(&p->fwd, tw, 0);
	return chain_twiddles(&p->inv, tw, off);
}

size_t fgk_chain_twiddles(fgk_chain *c, void *tw_host_float2)
{
	return chain_twiddles(c, (float *)tw_host_float2, 0);
}

/* Threads a lane-interleaved pass needs: every stage's NL * Lp / R
 * butterflies over at most `cap` threads, emax / R of them per thread. */
static uint32_t pass_threads(const uint32_t *rad, uint32_t n, uint32_t Lp, uint32_t nl, uint32_t emax)
{
	uint32_t s, T = 32;
	for (s = 0; s < n; s++) {
		uint32_t items = Lp / rad[s] * nl, b = bmax(rad[s], emax);
		uint32_t need = (items + b - 1) / b;
		if (need > T)
			T = need;
	}
	return (T + 31) & ~31u;
}

static int plan_pass(uint32_t Lp, int mirror, uint32_t max_smem, fgk_chain *ch, uint32_t *lshift, uint32_t *threads,
                     uint32_t *slots, uint32_t *emax_out)
{
	uint32_t rad[FGK_MAX_STAGES], n, ls, emax;
	if (fgk_plan_chain(Lp, rad, &n))
		return -1;
	/* ping-pong tiles (two buffers, no register batches, so no spills): the
	 * widest lane count (<= 16) whose two buffers fit half the shared memory
	 * (two CTAs per SM), or at most 4 lanes in the whole of it; threads: the
	 * widest stage's butterflies, 128 to 512; chains of up to 15 stages */
	for (ls = 4; n <= 15; ls--) {
		const uint32_t nl = 1u << ls, sl = (Lp * nl + (Lp * nl) / 16 + 1 + 3) & ~3u;
		if ((size_t)2 * sl * 8 <= max_smem / 2 || (ls <= 2 && (size_t)2 * sl * 8 <= max_smem)) {
			uint32_t s, T = 128;
			for (s = 0; s < n; s++)
				if (Lp / rad[s] * nl > T)
					T = Lp / rad[s] * nl;
			T = T > 512 ? 512 : (T + 31) & ~31u;
			*threads = T;
			*emax_out = 0;
			*slots = sl;
			*lshift = ls;
			fill_chain(ch, rad, n, Lp, T);
			return 0;
		}
		if (ls == (mirror ? 1u : 0u))
			break;
	}
	/* otherwise in place: the widest lane count (<= 16) whose tile fits
	 * half the shared memory (two CTAs per SM) and whose stages fit 512
	 * threads; below 4 lanes the HBM segments get narrower than a 32-byte
	 * sector, so 4 lanes may take the whole shared memory */
	for (ls = 4;; ls--) {
		uint32_t nl = 1u << ls, sl = Lp * nl + (Lp * nl) / 16 + 1;
		int ok = 0;
		if ((size_t)sl * 8 <= max_smem / 2 || (ls <= 2 && (size_t)sl * 8 <= max_smem)) {
			for (emax = 16; emax <= 32; emax *= 2) {
				uint32_t T = pass_threads(rad, n, Lp, nl, emax);
				if (T <= 512) {
					*threads = T;
					*emax_out = emax;
					*slots = sl;
					*lshift = ls;
					ok = 1;
					break;
				}
			}
		}
		if (ok)
			break;
		if (ls == (mirror ? 1u : 0u))
			return -1;
	}
	fill_chain(ch, rad, n, Lp, *threads);
	return 0;
}

int fgk_plan_fourstep(fgk_plan4 *p, uint32_t L, uint32_t modulation, uint32_t max_smem_bytes)
{
	uint32_t a, b, c, L1, best1 = 0;
	double bestd = 1e30;
	memset(p, 0, sizeof(*p));
	if (factor235(L, &a, &b, &c))
		return -1;
	/* most balanced split L1 * L2 (both at least 2) */
	for (L1 = 2; (uint64_t)L1 * L1 <= (uint64_t)L * 4 && L1 < L; L1++) {
		double d;
		if (L % L1)
			continue;
		d = fabs(log((double)L1) - log((double)(L / L1)));
		if (d < bestd) {
			bestd = d;
			best1 = L1;
		}
	}
	if (!best1)
		return -1;
	p->L1 = best1;
	p->L2 = L / best1;
	p->modulation = modulation;
	/* FREQ_OFFSET_REAL pairs mirror columns (inverse pass 1) and mirror rows
	 * (forward pass 2) inside a CTA */
	if (plan_pass(p->L1, modulation == FGK_MOD_FREQOFF, max_smem_bytes, &p->c1, &p->lshift1, &p->threads1,
	              &p->slots1, &p->emax1) ||
	    plan_pass(p->L2, modulation == FGK_MOD_FREQOFF, max_smem_bytes, &p->c2, &p->lshift2, &p->threads2,
	              &p->slots2, &p->emax2))
		return -1;
	return 0;
}

/* Three-level split: L1 in [16, 256], L2, L3 <= 256, L1 L2 L3 = L, the
 * smallest largest factor, ties towards L1 a multiple of 16 (whole C tiles). */
int fgk_plan_threestep(fgk_plan3 *p, uint32_t L, uint32_t modulation)
{
	uint32_t a, b, c, L1, L2, best = 0, b1 = 0, b2 = 0, bmul = 0, rad[FGK_MAX_STAGES], n;
	memset(p, 0, sizeof(*p));
	if (factor235(L, &a, &b, &c))
		return -1;
	for (L1 = 16; L1 <= 256; L1++) {
		if (L % L1)
			continue;
		for (L2 = 2; L2 <= 256; L2++) {
			uint32_t L3, m;
			if ((L / L1) % L2)
				continue;
			L3 = L / L1 / L2;
			if (L3 < 2 || L3 > 256)
				continue;
			m = L1 > L2 ? L1 : L2;
			m = m > L3 ? m : L3;
			if (!best || m < best || (m == best && (L1 % 16 == 0) && !bmul)) {
				best = m;
				b1 = L1;
				b2 = L2;
				bmul = L1 % 16 == 0;
			}
		}
	}
	if (!best)
		return -1;
	p->L1 = b1;
	p->L2 = b2;
	p->L3 = L / b1 / b2;
	p->modulation = modulation;
	if (plan_chain_set(p->L1, FGK_ALL_RADICES, rad, &n))
		return -1;
	fill_chain(&p->c1, rad, n, p->L1, 256);
	if (plan_chain_set(p->L2, FGK_ALL_RADICES, rad, &n))
		return -1;
	fill_chain(&p->c2, rad, n, p->L2, 256);
	if (plan_chain_set(p->L3, FGK_ALL_RADICES, rad, &n))
		return -1;
	fill_chain(&p->c3, rad, n, p->L3, 256);
	p->nq1 = p->c1.st[p->c1.nstages - 1].radix * p->L2;
	p->nq2 = p->c2.st[p->c2.nstages - 1].radix * p->L3;
	return 0;
}

/* Kernel-buffer layout of fftset_fft_conv_get_kernel, reproduced exactly.
 *
 * The reference leaves the kernel spectrum where its in-place DIF chain put
 * it (src/fftset_vec.c:1199-1207): the buffer is M = L/V slots of V real parts
 * followed by V imaginary parts (src/fftset_vec.c:112-115), slot s lane l
 * holding DFT bin l + V*rev(s), where rev is the digit reversal of the radix
 * chain its planner picked for an inner transform of length M at vector width
 * V. V itself is chosen per modulation and size by the reference's init code
 * for the SIMD width it was built with:
 *   COMPLEX           V = 4 if L > 4 and L % 4 == 0, else 1
 *                     (src/fftset_mod_cplx.c:322-345)
 *   FREQ_OFFSET_REAL  V = 8 if L % 32 == 0 (width-8 builds),
 *                     V = 4 if L % 16 == 0, else 1
 *                     (src/fftset_mod_freqoffsetreal.c:1016, :1073, :1118)
 * The planner (src/fftset_vec.c:945-971, :1004-1062) scores a chain as the
 * sum of 100 + ((r+2)(w+3)10000)/(r w) over its passes; radices 2, 3, 4 may
 * appear anywhere, 5, 6, 8, 16 only last; among equal scores the first radix
 * in the order 2, 3, 4, 5, 6, 8, 16 wins at every level. The layout must be
 * reproduced bit-for-bit because kernel buffers are interchangeable between
 * this library and CPU builds of the reference. */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "fftset_layout.h"

static const unsigned REF_RADICES[7] = {2, 3, 4, 5, 6, 8, 16};

static unsigned ref_cost(unsigned r, unsigned w)
{
	return 100u + ((r + 2u) * (w + 3u) * 10000u) / (r * w);
}

/* Best reference chain for every divisor d of `length` (d > 1), bottom-up over
 * the divisors in increasing order. Returns the number of passes or 0. */
unsigned fsl_reference_chain(unsigned length, unsigned w, unsigned *chain)
{
	/* divisors of length = 2^a 3^b 5^c, increasing */
	unsigned *div = NULL, *cost = NULL, *firstr = NULL, nd = 0, i, j, n;
	unsigned a = 0, b = 0, c = 0, rest = length, result = 0;
	if (length < 2)
		return 0;
	while (rest % 2 == 0) { rest /= 2; a++; }
	while (rest % 3 == 0) { rest /= 3; b++; }
	while (rest % 5 == 0) { rest /= 5; c++; }
	if (rest != 1)
		return 0;
	nd = (a + 1) * (b + 1) * (c + 1);
	div = (unsigned *)malloc(sizeof(unsigned) * nd);
	cost = (unsigned *)calloc(nd, sizeof(unsigned));
	firstr = (unsigned *)calloc(nd, sizeof(unsigned));
	if (!div || !cost || !firstr)
		goto out;
	n = 0;
	{
		unsigned i2, i3, i5;
		unsigned long long p5 = 1;
		for (i5 = 0; i5 <= c; i5++, p5 *= 5) {
			unsigned long long p3 = p5;
			for (i3 = 0; i3 <= b; i3++, p3 *= 3) {
				unsigned long long p2 = p3;
				for (i2 = 0; i2 <= a; i2++, p2 *= 2)
					div[n++] = (unsigned)p2;
			}
		}
	}
	for (i = 1; i < nd; i++) /* insertion sort: nd is small */
		for (j = i; j > 0 && div[j - 1] > div[j]; j--) {
			unsigned t = div[j];
			div[j] = div[j - 1];
			div[j - 1] = t;
		}
	for (i = 1; i < nd; i++) { /* skip d = 1 */
		unsigned len = div[i], k, best = 0, bestr = 0;
		for (k = 0; k < 7; k++) {
			unsigned r = REF_RADICES[k], pc = ref_cost(r, w);
			if (len == r) {
				if (best == 0 || best > pc) {
					best = pc;
					bestr = r;
				}
				continue;
			}
			if (r > 4 || len % r)
				continue;
			{
				/* locate len / r among the divisors */
				unsigned sub = len / r, lo = 0, hi = i;
				while (lo < hi) {
					unsigned mid = (lo + hi) / 2;
					if (div[mid] < sub)
						lo = mid + 1;
					else
						hi = mid;
				}
				if (div[lo] != sub || sub < 2 || cost[lo] == 0)
					continue;
				if (best == 0 || best > cost[lo] + pc) {
					best = cost[lo] + pc;
					bestr = r;
				}
			}
		}
		cost[i] = best;
		firstr[i] = bestr;
	}
	if (cost[nd - 1] == 0)
		goto out;
	{
		unsigned len = length, np = 0;
		while (len > 1) {
			unsigned lo = 0, hi = nd - 1, r;
			while (lo < hi) {
				unsigned mid = (lo + hi) / 2;
				if (div[mid] < len)
					lo = mid + 1;
				else
					hi = mid;
			}
			r = firstr[lo];
			if (r == 0 || np >= FSL_MAX_CHAIN)
				goto out;
			chain[np++] = r;
			len /= r;
		}
		result = np;
	}
out:
	free(div);
	free(cost);
	free(firstr);
	return result;
}

unsigned fsl_lane_width(int freq_offset_real, unsigned L, unsigned simd_width)
{
	if (!freq_offset_real)
		return (simd_width >= 4 && L > 4 && L % 4 == 0) ? 4u : 1u;
	if (simd_width >= 8 && L >= 32 && L % 32 == 0)
		return 8;
	if (simd_width >= 4 && L >= 16 && L % 16 == 0)
		return 4;
	return 1;
}

int fsl_kernel_offsets(int freq_offset_real, unsigned L, unsigned simd_width, int32_t *re_off, unsigned *lanes)
{
	unsigned V = fsl_lane_width(freq_offset_real, L, simd_width);
	unsigned M = L / V, chain[FSL_MAX_CHAIN], n, s, l;
	n = fsl_reference_chain(M, V, chain);
	if (n == 0)
		return -1;
	for (s = 0; s < M; s++) {
		/* digit reversal: s = q*(len/r) + s', bin = q + r*bin(s') */
		unsigned len = M, rem = s, bin = 0, mul = 1, i;
		for (i = 0; i < n; i++) {
			unsigned m = len / chain[i];
			unsigned q = rem / m;
			rem -= q * m;
			bin += mul * q;
			mul *= chain[i];
			len = m;
		}
		for (l = 0; l < V; l++)
			re_off[l + V * bin] = (int32_t)(2 * V * s + l);
	}
	*lanes = V;
	return 0;
}

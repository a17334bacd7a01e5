/* ORACLE TEST INFRASTRUCTURE -- not part of the product.
 *
 * The small DFT codelets of the C restatement (fftset_oracle.c), written
 * once for an element type OR_T: included once with OR_T = float (one lane)
 * and once with OR_T a vector of four floats (four lanes of the reference's
 * vector-of-transforms layout at a time, the width of its 128-bit build).
 * The vector form runs the same operations in the same order on each lane.
 * The includer defines OR_T and OR_SFX (the suffix of the function names)
 * and provides or_cw, the composite codelets' internal twiddles. */
#define OR_CAT2(a, b) a##b
#define OR_CAT(a, b) OR_CAT2(a, b)
#define OR_FN(name) OR_CAT(name, OR_SFX)

static inline void OR_FN(or_dft2)(OR_T *re, OR_T *im)
{
	OR_T ar = re[0] + re[1], ai = im[0] + im[1];
	OR_T br = re[0] - re[1], bi = im[0] - im[1];
	re[0] = ar; im[0] = ai; re[1] = br; im[1] = bi;
}

static inline void OR_FN(or_dft3)(OR_T *re, OR_T *im)
{
	OR_T sr = re[1] + re[2], si = im[1] + im[2];
	OR_T dr = re[1] - re[2], di = im[1] - im[2];
	OR_T mr = re[0] - 0.5f * sr, mi = im[0] - 0.5f * si;
	re[0] += sr; im[0] += si;
	re[1] = mr + OR_C3 * di; im[1] = mi - OR_C3 * dr;
	re[2] = mr - OR_C3 * di; im[2] = mi + OR_C3 * dr;
}

static inline void OR_FN(or_dft4)(OR_T *re, OR_T *im)
{
	OR_T ar = re[0] + re[2], ai = im[0] + im[2];
	OR_T br = re[0] - re[2], bi = im[0] - im[2];
	OR_T cr = re[1] + re[3], ci = im[1] + im[3];
	OR_T dr = re[1] - re[3], di = im[1] - im[3];
	re[0] = ar + cr; im[0] = ai + ci;
	re[2] = ar - cr; im[2] = ai - ci;
	re[1] = br + di; im[1] = bi - dr;
	re[3] = br - di; im[3] = bi + dr;
}

static inline void OR_FN(or_dft5)(OR_T *re, OR_T *im)
{
	OR_T s1r = re[1] + re[4], s1i = im[1] + im[4];
	OR_T d1r = re[1] - re[4], d1i = im[1] - im[4];
	OR_T s2r = re[2] + re[3], s2i = im[2] + im[3];
	OR_T d2r = re[2] - re[3], d2i = im[2] - im[3];
	OR_T a1r = re[0] + OR_C5A * s1r - OR_C5C * s2r;
	OR_T a1i = im[0] + OR_C5A * s1i - OR_C5C * s2i;
	OR_T a2r = re[0] - OR_C5C * s1r + OR_C5A * s2r;
	OR_T a2i = im[0] - OR_C5C * s1i + OR_C5A * s2i;
	OR_T b1r = OR_C5B * d1i + OR_C5D * d2i;
	OR_T b1i = OR_C5B * d1r + OR_C5D * d2r;
	OR_T b2r = OR_C5D * d1i - OR_C5B * d2i;
	OR_T b2i = OR_C5D * d1r - OR_C5B * d2r;
	re[0] += s1r + s2r; im[0] += s1i + s2i;
	re[1] = a1r + b1r; im[1] = a1i - b1i;
	re[4] = a1r - b1r; im[4] = a1i + b1i;
	re[2] = a2r + b2r; im[2] = a2i - b2i;
	re[3] = a2r - b2r; im[3] = a2i + b2i;
}

static void OR_FN(or_dft_small)(unsigned r, OR_T *re, OR_T *im);

/* r = a*b: X[b*k1 + k2] = sum_p1 w_a^{p1 k1} w_r^{p1 k2} sum_p2 x[p1 + a p2] w_b^{p2 k2} */
static void OR_FN(or_dft_composite)(unsigned a, unsigned b, OR_T *re, OR_T *im)
{
	OR_T tr[16], ti[16], ur[16], ui[16];
	unsigned p1, p2, k1, k2, r = a * b;
	for (p1 = 0; p1 < a; p1++) {
		OR_T cr[16], ci[16];
		for (p2 = 0; p2 < b; p2++) {
			cr[p2] = re[p1 + a * p2];
			ci[p2] = im[p1 + a * p2];
		}
		OR_FN(or_dft_small)(b, cr, ci);
		for (k2 = 0; k2 < b; k2++) {
			const float wr = or_cw[r][p1 * k2][0], wi = or_cw[r][p1 * k2][1];
			tr[p1 * b + k2] = cr[k2] * wr - ci[k2] * wi;
			ti[p1 * b + k2] = cr[k2] * wi + ci[k2] * wr;
		}
	}
	for (k2 = 0; k2 < b; k2++) {
		for (p1 = 0; p1 < a; p1++) {
			ur[p1] = tr[p1 * b + k2];
			ui[p1] = ti[p1 * b + k2];
		}
		OR_FN(or_dft_small)(a, ur, ui);
		for (k1 = 0; k1 < a; k1++) {
			re[b * k1 + k2] = ur[k1];
			im[b * k1 + k2] = ui[k1];
		}
	}
}

static void OR_FN(or_dft_small)(unsigned r, OR_T *re, OR_T *im)
{
	switch (r) {
	case 2: OR_FN(or_dft2)(re, im); break;
	case 3: OR_FN(or_dft3)(re, im); break;
	case 4: OR_FN(or_dft4)(re, im); break;
	case 5: OR_FN(or_dft5)(re, im); break;
	case 6: OR_FN(or_dft_composite)(2, 3, re, im); break;
	case 8: OR_FN(or_dft_composite)(2, 4, re, im); break;
	case 16: OR_FN(or_dft_composite)(4, 4, re, im); break;
	default: break;
	}
}

#undef OR_FN
#undef OR_CAT
#undef OR_CAT2

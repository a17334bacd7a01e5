/* Register-resident DFT codelets (forward sign, natural order in and out).
 *
 * dft<R>(v) replaces v[0..R) by X[k] = sum_p v[p] e^{-j 2 pi p k / R}.
 * Radices 2, 3, 4, 5, 8 are written out; 9 and 16 are 3x3 and 4x4
 * Cooley-Tukey with their internal twiddles written as constants; 6, 10, 12 and 15 are Good-Thomas
 * prime-factor composites (coprime factors, no internal twiddles, the index
 * maps are compile-time register renamings). These play the role of the
 * reference's radix butterflies (src/fftset_vec.c:109-845) but are this
 * project's own GPU codelets: one thread holds a whole butterfly in registers.
 *
 * The header also compiles as plain host C++ so the codelets can be unit
 * tested without a GPU. */
#pragma once

#ifdef __CUDACC__
#define FGK_HD __host__ __device__ __forceinline__
#define FGK_CX __host__ __device__ constexpr
#else
#define FGK_HD inline
#define FGK_CX constexpr
#include <cmath>
struct float2 { float x, y; };
static inline float2 make_float2(float a, float b) { float2 r; r.x = a; r.y = b; return r; }
#endif

namespace fgk {

/* Complex add/sub: on sm_100+ one packed f32x2 instruction (same FP32
 * throughput as two scalar adds, half the issue slots). */
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
FGK_HD float2 cadd(float2 a, float2 b)
{
	unsigned long long ra, rb, rd;
	float2 r;
	asm("mov.b64 %0, {%1, %2};" : "=l"(ra) : "f"(a.x), "f"(a.y));
	asm("mov.b64 %0, {%1, %2};" : "=l"(rb) : "f"(b.x), "f"(b.y));
	asm("add.rn.f32x2 %0, %1, %2;" : "=l"(rd) : "l"(ra), "l"(rb));
	asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(rd));
	return r;
}
FGK_HD float2 csub(float2 a, float2 b)
{
	unsigned long long ra, rb, rd;
	float2 r;
	asm("mov.b64 %0, {%1, %2};" : "=l"(ra) : "f"(a.x), "f"(a.y));
	asm("mov.b64 %0, {%1, %2};" : "=l"(rb) : "f"(b.x), "f"(b.y));
	asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(rd) : "l"(ra), "l"(rb));
	asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(rd));
	return r;
}
#else
FGK_HD float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
FGK_HD float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
#endif
FGK_HD float2 cmul(float2 a, float2 w) { return make_float2(a.x * w.x - a.y * w.y, a.x * w.y + a.y * w.x); }
/* a * conj(w) */
FGK_HD float2 cmulc(float2 a, float2 w) { return make_float2(a.x * w.x + a.y * w.y, a.y * w.x - a.x * w.y); }
FGK_HD float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }
/* a * (-j) */
FGK_HD float2 mul_mj(float2 a) { return make_float2(a.y, -a.x); }
FGK_HD float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }

/* ---- lean tables --------------------------------------------------------
 * Helpers for kernels that read fewer table entries and multiply instead. */

/* highest power of two <= p, for 1 <= p < 32 */
FGK_CX int hipow2(int p) { return p >= 16 ? 16 : p >= 8 ? 8 : p >= 4 ? 4 : p >= 2 ? 2 : 1; }

/* w[p] = w^{p k} for p = 1..R-1, where entry(p) reads w^{p k} from a table:
 * only the entries of p = 1, 2, 4, 8 are read and the others formed as
 * w^{h k} w^{(p-h) k}, h = hipow2(p), at most three products deep. */
template <int R, class Entry> FGK_HD void twiddle_powers(float2 (&w)[R], Entry &&entry)
{
#pragma unroll
	for (int p = 1; p < R; p++)
		w[p] = p == hipow2(p) ? entry(p) : cmul(w[hipow2(p)], w[p - hipow2(p)]);
}

/* sin and cos by their Taylor series for |x| <= pi/2, for compile-time
 * constants */
FGK_CX double cx_sin(double x)
{
	double t = x, s = x;
	for (int n = 1; n < 14; n++) {
		t *= -x * x / ((2.0 * n) * (2.0 * n + 1.0));
		s += t;
	}
	return s;
}
FGK_CX double cx_cos(double x)
{
	double t = 1.0, s = 1.0;
	for (int n = 1; n < 14; n++) {
		t *= -x * x / ((2.0 * n - 1.0) * (2.0 * n));
		s += t;
	}
	return s;
}

/* e^{-j pi P / (2R)}: the ratio between the FREQ_OFFSET_REAL modulation
 * factors e^{-j pi i / (2L)} of points i + P L/R and i */
template <int R, int P> struct ModStep {
	static constexpr double a = 3.14159265358979323846 * P / (2.0 * R);
	static constexpr float re = (float)cx_cos(a);
	static constexpr float im = (float)-cx_sin(a);
};

/* v[P..R-1] *= m e^{-j pi P / (2R)} */
template <int R, int P = 0> FGK_HD void mod_steps(float2 (&v)[R], float2 m)
{
	if constexpr (P < R) {
		v[P] = cmul(v[P], P == 0 ? m : cmul(m, make_float2(ModStep<R, P>::re, ModStep<R, P>::im)));
		mod_steps<R, P + 1>(v, m);
	}
}

/* exact decimal expansions of the constants named */
#define FGK_SQRT1_2 0.70710678118654752440f  /* cos(pi/4) */
#define FGK_COS_PI8 0.92387953251128675613f  /* cos(pi/8) */
#define FGK_SIN_PI8 0.38268343236508977173f  /* sin(pi/8) */
#define FGK_SIN_PI3 0.86602540378443864676f  /* sin(pi/3) */
#define FGK_C1_5    0.30901699437494742410f  /* cos(2pi/5) */
#define FGK_C2_5    0.80901699437494742410f  /* -cos(4pi/5) */
#define FGK_S1_5    0.95105651629515357212f  /* sin(2pi/5) */
#define FGK_S2_5    0.58778525229247312917f  /* sin(4pi/5) */
#define FGK_C1_9    0.76604444311897803520f  /* cos(2pi/9) */
#define FGK_S1_9    0.64278760968653932632f  /* sin(2pi/9) */
#define FGK_C2_9    0.17364817766693034885f  /* cos(4pi/9) */
#define FGK_S2_9    0.98480775301220805936f  /* sin(4pi/9) */
#define FGK_C4_9    0.93969262078590838405f  /* -cos(8pi/9) */
#define FGK_S4_9    0.34202014332566873304f  /* sin(8pi/9) */

FGK_HD void dft2(float2 &a, float2 &b)
{
	float2 t = a;
	a = cadd(t, b);
	b = csub(t, b);
}

FGK_HD void dft3(float2 &a, float2 &b, float2 &c)
{
	float2 s = cadd(b, c);
	float2 d = csub(b, c);
	float2 m = make_float2(a.x - 0.5f * s.x, a.y - 0.5f * s.y);
	a = cadd(a, s);
	/* X1 = m - j sin(pi/3) d ; X2 = m + j sin(pi/3) d */
	b = make_float2(m.x + FGK_SIN_PI3 * d.y, m.y - FGK_SIN_PI3 * d.x);
	c = make_float2(m.x - FGK_SIN_PI3 * d.y, m.y + FGK_SIN_PI3 * d.x);
}

FGK_HD void dft4(float2 &a, float2 &b, float2 &c, float2 &d)
{
	float2 s0 = cadd(a, c), d0 = csub(a, c);
	float2 s1 = cadd(b, d), d1 = mul_mj(csub(b, d));
	a = cadd(s0, s1);
	c = csub(s0, s1);
	b = cadd(d0, d1);
	d = csub(d0, d1);
}

FGK_HD void dft5(float2 &x0, float2 &x1, float2 &x2, float2 &x3, float2 &x4)
{
	float2 s1 = cadd(x1, x4), d1 = csub(x1, x4);
	float2 s2 = cadd(x2, x3), d2 = csub(x2, x3);
	float2 a1 = make_float2(x0.x + FGK_C1_5 * s1.x - FGK_C2_5 * s2.x, x0.y + FGK_C1_5 * s1.y - FGK_C2_5 * s2.y);
	float2 a2 = make_float2(x0.x - FGK_C2_5 * s1.x + FGK_C1_5 * s2.x, x0.y - FGK_C2_5 * s1.y + FGK_C1_5 * s2.y);
	/* b1 = sin(2pi/5) d1 + sin(4pi/5) d2 ; b2 = sin(4pi/5) d1 - sin(2pi/5) d2 */
	float2 b1 = make_float2(FGK_S1_5 * d1.x + FGK_S2_5 * d2.x, FGK_S1_5 * d1.y + FGK_S2_5 * d2.y);
	float2 b2 = make_float2(FGK_S2_5 * d1.x - FGK_S1_5 * d2.x, FGK_S2_5 * d1.y - FGK_S1_5 * d2.y);
	x0 = cadd(x0, cadd(s1, s2));
	/* X1 = a1 - j b1, X4 = a1 + j b1, X2 = a2 - j b2, X3 = a2 + j b2 */
	x1 = make_float2(a1.x + b1.y, a1.y - b1.x);
	x4 = make_float2(a1.x - b1.y, a1.y + b1.x);
	x2 = make_float2(a2.x + b2.y, a2.y - b2.x);
	x3 = make_float2(a2.x - b2.y, a2.y + b2.x);
}

/* 8 = 2 x 4 decimation in frequency:
 * u_p = v_p + v_{p+4}, t_p = (v_p - v_{p+4}) w8^p, X[2k] = DFT4(u)[k],
 * X[2k+1] = DFT4(t)[k]. */
FGK_HD void dft8(float2 *v)
{
	float2 u0 = cadd(v[0], v[4]), t0 = csub(v[0], v[4]);
	float2 u1 = cadd(v[1], v[5]), t1 = csub(v[1], v[5]);
	float2 u2 = cadd(v[2], v[6]), t2 = csub(v[2], v[6]);
	float2 u3 = cadd(v[3], v[7]), t3 = csub(v[3], v[7]);
	/* w8^1 = (1-j)/sqrt2, w8^2 = -j, w8^3 = -(1+j)/sqrt2 */
	t1 = make_float2(FGK_SQRT1_2 * (t1.x + t1.y), FGK_SQRT1_2 * (t1.y - t1.x));
	t2 = mul_mj(t2);
	t3 = make_float2(FGK_SQRT1_2 * (t3.y - t3.x), -FGK_SQRT1_2 * (t3.x + t3.y));
	dft4(u0, u1, u2, u3);
	dft4(t0, t1, t2, t3);
	v[0] = u0; v[2] = u1; v[4] = u2; v[6] = u3;
	v[1] = t0; v[3] = t1; v[5] = t2; v[7] = t3;
}

/* 9 = 3 x 3: column DFT3 over n1 of v[3 n1 + n2], twiddle w9^{n2 k1}, row
 * DFT3 over n2, X[k1 + 3 k2]. */
FGK_HD void dft9(float2 *v)
{
	float2 a0 = v[0], a1 = v[3], a2 = v[6];
	float2 b0 = v[1], b1 = v[4], b2 = v[7];
	float2 c0 = v[2], c1 = v[5], c2 = v[8];
	dft3(a0, a1, a2);
	dft3(b0, b1, b2);
	dft3(c0, c1, c2);
	b1 = cmul(b1, make_float2(FGK_C1_9, -FGK_S1_9));  /* w9^1 */
	b2 = cmul(b2, make_float2(FGK_C2_9, -FGK_S2_9));  /* w9^2 */
	c1 = cmul(c1, make_float2(FGK_C2_9, -FGK_S2_9));  /* w9^2 */
	c2 = cmul(c2, make_float2(-FGK_C4_9, -FGK_S4_9)); /* w9^4 */
	dft3(a0, b0, c0);
	dft3(a1, b1, c1);
	dft3(a2, b2, c2);
	v[0] = a0; v[3] = b0; v[6] = c0;
	v[1] = a1; v[4] = b1; v[7] = c1;
	v[2] = a2; v[5] = b2; v[8] = c2;
}

/* 16 = 4 x 4: column DFT4 over p2 of v[p1 + 4 p2], twiddle w16^{p1 k2},
 * row DFT4 over p1, X[4 k1 + k2]. */
FGK_HD void dft16(float2 *v)
{
	float2 c[4][4];
#pragma unroll
	for (int p1 = 0; p1 < 4; p1++) {
		c[p1][0] = v[p1];
		c[p1][1] = v[p1 + 4];
		c[p1][2] = v[p1 + 8];
		c[p1][3] = v[p1 + 12];
		dft4(c[p1][0], c[p1][1], c[p1][2], c[p1][3]);
	}
	/* twiddles w16^{p1 k2}: p1 = 1: k2=1 w, 2 w^2, 3 w^3;
	 * p1 = 2: w^2, w^4 = -j, w^6; p1 = 3: w^3, w^6, w^9 */
	const float2 w1 = make_float2(FGK_COS_PI8, -FGK_SIN_PI8);
	const float2 w3 = make_float2(FGK_SIN_PI8, -FGK_COS_PI8);
	c[1][1] = cmul(c[1][1], w1);
	c[1][2] = make_float2(FGK_SQRT1_2 * (c[1][2].x + c[1][2].y), FGK_SQRT1_2 * (c[1][2].y - c[1][2].x));
	c[1][3] = cmul(c[1][3], w3);
	c[2][1] = make_float2(FGK_SQRT1_2 * (c[2][1].x + c[2][1].y), FGK_SQRT1_2 * (c[2][1].y - c[2][1].x));
	c[2][2] = mul_mj(c[2][2]);
	c[2][3] = make_float2(FGK_SQRT1_2 * (c[2][3].y - c[2][3].x), -FGK_SQRT1_2 * (c[2][3].x + c[2][3].y));
	c[3][1] = cmul(c[3][1], w3);
	c[3][2] = make_float2(FGK_SQRT1_2 * (c[3][2].y - c[3][2].x), -FGK_SQRT1_2 * (c[3][2].x + c[3][2].y));
	/* w16^9 = -w16^1 */
	c[3][3] = cmul(c[3][3], make_float2(-FGK_COS_PI8, FGK_SIN_PI8));
#pragma unroll
	for (int k2 = 0; k2 < 4; k2++) {
		dft4(c[0][k2], c[1][k2], c[2][k2], c[3][k2]);
		v[k2] = c[0][k2];
		v[k2 + 4] = c[1][k2];
		v[k2 + 8] = c[2][k2];
		v[k2 + 12] = c[3][k2];
	}
}

template <int R> struct Radix;
template <> struct Radix<2> { static FGK_HD void run(float2 *v) { dft2(v[0], v[1]); } };
template <> struct Radix<3> { static FGK_HD void run(float2 *v) { dft3(v[0], v[1], v[2]); } };
template <> struct Radix<4> { static FGK_HD void run(float2 *v) { dft4(v[0], v[1], v[2], v[3]); } };
template <> struct Radix<5> { static FGK_HD void run(float2 *v) { dft5(v[0], v[1], v[2], v[3], v[4]); } };
template <> struct Radix<8> { static FGK_HD void run(float2 *v) { dft8(v); } };
template <> struct Radix<9> { static FGK_HD void run(float2 *v) { dft9(v); } };
template <> struct Radix<16> { static FGK_HD void run(float2 *v) { dft16(v); } };

/* Good-Thomas prime-factor composite for N = A*B, gcd(A,B) = 1:
 * input  n = (B n1 + A n2) mod N,
 * output k = (B (B^-1 mod A) k1 + A (A^-1 mod B) k2) mod N. */
FGK_CX int fgk_inv_mod(int a, int m, int t = 1)
{
	return ((a * t) % m == 1) ? t : fgk_inv_mod(a, m, t + 1);
}

template <int A, int B> struct PFA {
	static FGK_HD void run(float2 *v)
	{
		constexpr int N = A * B;
		float2 y[A][B];
#pragma unroll
		for (int n2 = 0; n2 < B; n2++) {
			float2 col[A];
#pragma unroll
			for (int n1 = 0; n1 < A; n1++)
				col[n1] = v[(B * n1 + A * n2) % N];
			Radix<A>::run(col);
#pragma unroll
			for (int k1 = 0; k1 < A; k1++)
				y[k1][n2] = col[k1];
		}
		constexpr int eA = (B * fgk_inv_mod(B % A, A)) % N;
		constexpr int eB = (A * fgk_inv_mod(A % B, B)) % N;
#pragma unroll
		for (int k1 = 0; k1 < A; k1++) {
			float2 row[B];
#pragma unroll
			for (int k2 = 0; k2 < B; k2++)
				row[k2] = y[k1][k2];
			Radix<B>::run(row);
#pragma unroll
			for (int k2 = 0; k2 < B; k2++)
				v[(eA * k1 + eB * k2) % N] = row[k2];
		}
	}
};
template <> struct Radix<6> { static FGK_HD void run(float2 *v) { PFA<2, 3>::run(v); } };
template <> struct Radix<10> { static FGK_HD void run(float2 *v) { PFA<2, 5>::run(v); } };
template <> struct Radix<12> { static FGK_HD void run(float2 *v) { PFA<4, 3>::run(v); } };
template <> struct Radix<15> { static FGK_HD void run(float2 *v) { PFA<3, 5>::run(v); } };

} /* namespace fgk */

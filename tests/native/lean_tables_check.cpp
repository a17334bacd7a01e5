// Host check of the lean-table helpers of fgk_codelets.cuh (plain C++):
//  - twiddle_powers: w^{p k} formed from the FP32-rounded table entries of
//    p = 1, 2, 4, 8 against FP64 e^{-j 2 pi p k / (ns R)}, for the radices and
//    strides the kernels use;
//  - ModStep: the compile-time e^{-j pi P / (2R)} against FP64 cos/sin;
//  - mod_steps: mods[j] e^{-j pi p / (2R)} against the FP64 factor
//    e^{-j pi (j + p L/R) / (2L)} of the 1536- and 4096-bin kernels.
// Prints "name maxerr" lines; exits non-zero when one exceeds its bound.
#include <cmath>
#include <cstdio>
#include <initializer_list>
#include "fgk_codelets.cuh"

using namespace fgk;

static float2 unit(double a) { return make_float2((float)std::cos(a), (float)std::sin(a)); }

template <int R> static double check_powers()
{
	double worst = 0;
	for (int ns : {1, 6, 16, 96, 256, 4096}) {
		for (int k = 0; k < ns; k += (ns > 64 ? 7 : 1)) {
			const double base = -2.0 * M_PI / ((double)ns * R);
			float2 w[R];
			twiddle_powers<R>(w, [&](int p) { return unit(base * p * k); });
			for (int p = 1; p < R; p++) {
				const double e = std::hypot(w[p].x - std::cos(base * p * k), w[p].y - std::sin(base * p * k));
				if (e > worst)
					worst = e;
			}
		}
	}
	std::printf("powers%d %.3e\n", R, worst);
	return worst;
}

template <int R, int P = 1> static double check_steps()
{
	if constexpr (P < R) {
		const double a = M_PI * P / (2.0 * R);
		const double e = std::hypot(ModStep<R, P>::re - std::cos(a), ModStep<R, P>::im + std::sin(a));
		const double rest = check_steps<R, P + 1>();
		return e > rest ? e : rest;
	}
	return 0;
}

template <int R> static double check_modulation(int L)
{
	double worst = 0;
	const int nbf = L / R;
	for (int j = 0; j < nbf; j++) {
		float2 v[R];
		for (int p = 0; p < R; p++)
			v[p] = make_float2(1.f, 0.f);
		mod_steps<R>(v, unit(-M_PI * j / (2.0 * L)));
		for (int p = 0; p < R; p++) {
			const double a = -M_PI * (j + (double)p * nbf) / (2.0 * L);
			const double e = std::hypot(v[p].x - std::cos(a), v[p].y - std::sin(a));
			if (e > worst)
				worst = e;
		}
	}
	std::printf("modulation%d_%d %.3e\n", R, L, worst);
	return worst;
}

int main()
{
	int bad = 0;
	/* products of unit values rounded to FP32: a few units of 2^-24 */
	bad |= check_powers<8>() > 5e-7;
	bad |= check_powers<9>() > 5e-7;
	bad |= check_powers<12>() > 5e-7;
	bad |= check_powers<16>() > 5e-7;
	double s = 0;
	s = std::fmax(s, check_steps<2>());
	s = std::fmax(s, check_steps<3>());
	s = std::fmax(s, check_steps<4>());
	s = std::fmax(s, check_steps<6>());
	s = std::fmax(s, check_steps<8>());
	s = std::fmax(s, check_steps<16>());
	std::printf("modstep %.3e\n", s);
	bad |= s > 6e-8; /* one FP32 rounding of a value below 1 */
	bad |= check_modulation<16>(1536) > 3e-7;
	bad |= check_modulation<16>(4096) > 3e-7;
	return bad;
}

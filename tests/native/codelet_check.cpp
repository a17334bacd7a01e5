// Host check of the register codelets (fgk_codelets.cuh compiles as plain
// C++): every Radix<R> against a direct FP64 DFT on seeded inputs. Prints
// one line per radix "R maxrel" and exits non-zero when one exceeds 1e-6.
#include <cmath>
#include <cstdio>
#include <cstdint>
#include "fgk_codelets.cuh"

using namespace fgk;

static uint64_t rng_state = 0x9e3779b97f4a7c15ull;
static double urand()
{
	rng_state ^= rng_state << 13;
	rng_state ^= rng_state >> 7;
	rng_state ^= rng_state << 17;
	return (double)(rng_state >> 11) / 9007199254740992.0 * 2.0 - 1.0;
}

template <int R> static double check()
{
	double worst = 0;
	for (int trial = 0; trial < 64; trial++) {
		float2 v[R];
		double xr[R], xi[R];
		for (int p = 0; p < R; p++) {
			v[p] = make_float2((float)urand(), (float)urand());
			xr[p] = v[p].x;
			xi[p] = v[p].y;
		}
		Radix<R>::run(v);
		double num = 0, den = 0;
		for (int k = 0; k < R; k++) {
			double sr = 0, si = 0;
			for (int p = 0; p < R; p++) {
				const double a = -2.0 * M_PI * (double)((p * k) % R) / R;
				sr += xr[p] * std::cos(a) - xi[p] * std::sin(a);
				si += xr[p] * std::sin(a) + xi[p] * std::cos(a);
			}
			num += (v[k].x - sr) * (v[k].x - sr) + (v[k].y - si) * (v[k].y - si);
			den += sr * sr + si * si;
		}
		const double rel = std::sqrt(num / den);
		if (rel > worst)
			worst = rel;
	}
	std::printf("%d %.3e\n", R, worst);
	return worst;
}

int main()
{
	double w = 0;
	w = std::fmax(w, check<2>());
	w = std::fmax(w, check<3>());
	w = std::fmax(w, check<4>());
	w = std::fmax(w, check<5>());
	w = std::fmax(w, check<6>());
	w = std::fmax(w, check<8>());
	w = std::fmax(w, check<9>());
	w = std::fmax(w, check<10>());
	w = std::fmax(w, check<12>());
	w = std::fmax(w, check<15>());
	w = std::fmax(w, check<16>());
	return w < 1e-6 ? 0 : 1;
}

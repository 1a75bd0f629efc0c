// Host shim over shape_atrophy_gb300/csrc/sa_fixsum.cuh (the fixed-point summation the CG grid
// reductions use) for the CPU tests: sum a set of doubles or floats the way one reduction does.
#include "../shape_atrophy_gb300/csrc/sa_fixsum.cuh"

template <typename T>
static double fx_sum(const T *v, int n)
{
	int emax = 1;
	for (int i = 0; i < n; ++i) {
		const int e = sa::fx_exp(v[i]);
		if (e > emax) emax = e;
	}
	sa::Fx s = sa::fx_zero();
	for (int i = 0; i < n; ++i) s = sa::fx_add(s, sa::fx_from(v[i], emax));
	return sa::fx_to_double(s, emax);
}

extern "C" double fx_sum_f64(const double *v, int n) { return fx_sum(v, n); }
extern "C" double fx_sum_f32(const float *v, int n) { return fx_sum(v, n); }

// Exact, order-independent summation of FP64 (or FP32) values in 128-bit fixed point.
//
// GB300 issues FP64 adds at 2 per clock per SM, so a reduction tree of doubles
// (a dependent chain of adds on one warp) costs more than the grid barrier it
// sits behind.  Here every value is aligned to the largest exponent of its set
// (found with one integer max-reduction) and added as a 128-bit two's-
// complement integer on the integer pipes: integer addition is associative,
// so the sum is independent of the order and grouping of the values (still a
// deterministic function of the set), and it is exact down to 2^-112 of the
// largest value.  The final conversion rounds to nearest-even, once.
//
// Layout: value = F * 2^(emax - 1135), F = significand << (e - emax + 60),
// where e is the biased FP64 exponent field (1 for zeros and subnormals) and
// emax the largest e of the set.  |F| < 2^113, so up to 2^14 values sum
// without overflow.  emax == 2047 (an Inf or NaN in the set) gives NaN.
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define SA_FX_HD __host__ __device__ __forceinline__
#else
#define SA_FX_HD inline
#endif

namespace sa {

struct Fx {
	unsigned long long lo, hi;      // two's complement, hi holds bits 64..127
};

SA_FX_HD int fx_clz64(unsigned long long x)
{
#if defined(__CUDA_ARCH__)
	return __clzll((long long) x);
#else
	return x ? __builtin_clzll(x) : 64;
#endif
}

SA_FX_HD Fx fx_zero() { return Fx{0ull, 0ull}; }

SA_FX_HD Fx fx_add(Fx a, Fx b)
{
	Fx r;
	r.lo = a.lo + b.lo;
	r.hi = a.hi + b.hi + (r.lo < a.lo ? 1ull : 0ull);
	return r;
}

SA_FX_HD Fx fx_neg(Fx a)
{
	Fx r;
	r.lo = ~a.lo + 1ull;
	r.hi = ~a.hi + (r.lo == 0ull ? 1ull : 0ull);
	return r;
}

// FP64 view of a value: biased exponent (1 for zero and subnormals, 2047 for Inf and NaN), 53-bit significand
SA_FX_HD void fx_parts(double v, int &e, unsigned long long &m, bool &neg)
{
	unsigned long long b;
#if defined(__CUDA_ARCH__)
	b = (unsigned long long) __double_as_longlong(v);
#else
	__builtin_memcpy(&b, &v, 8);
#endif
	neg = (b >> 63) != 0ull;
	e = (int) ((b >> 52) & 0x7FFull);
	m = b & ((1ull << 52) - 1ull);
	if (e) m |= 1ull << 52;
	else e = 1;
}

// an FP32 value in the same FP64 frame: exponent field + 896, significand << 29 (exact)
SA_FX_HD void fx_parts(float v, int &e, unsigned long long &m, bool &neg)
{
	unsigned int b;
#if defined(__CUDA_ARCH__)
	b = (unsigned int) __float_as_uint(v);
#else
	__builtin_memcpy(&b, &v, 4);
#endif
	neg = (b >> 31) != 0u;
	int ef = (int) ((b >> 23) & 0xFFu);
	unsigned long long mm = b & 0x7FFFFFu;
	if (ef == 255) { e = 2047; m = 0ull; return; }
	if (ef) mm |= 1ull << 23;
	else ef = 1;
	e = ef + 896;
	m = mm << 29;
}

template <typename T>
SA_FX_HD int fx_exp(T v)
{
	int e; unsigned long long m; bool n;
	fx_parts(v, e, m, n);
	return e;
}

// v in the fixed-point frame of exponent emax (emax >= the value's exponent)
template <typename T>
SA_FX_HD Fx fx_from(T v, int emax)
{
	int e; unsigned long long m; bool neg;
	fx_parts(v, e, m, neg);
	if (emax >= 2047) return fx_zero();
	const int sh = e - emax + 60;           // <= 60
	Fx r;
	if (sh >= 12) { r.lo = m << sh; r.hi = m >> (64 - sh); }
	else if (sh > 0) { r.lo = m << sh; r.hi = 0ull; }      // m < 2^53, m << sh < 2^64
	else if (sh == 0) { r.lo = m; r.hi = 0ull; }
	else if (sh > -64) { r.lo = m >> (-sh); r.hi = 0ull; }
	else { r.lo = 0ull; r.hi = 0ull; }
	return neg ? fx_neg(r) : r;
}

// round-to-nearest-even of a sum in the frame of emax
SA_FX_HD double fx_to_double(Fx s, int emax)
{
	unsigned long long bits;
	if (emax >= 2047) {
		bits = 0x7FF8000000000000ull;       // a non-finite value was summed
	} else {
		const bool neg = (long long) s.hi < 0;
		if (neg) s = fx_neg(s);
		if (s.hi == 0ull && s.lo == 0ull) {
			bits = 0ull;
		} else {
			const int p = s.hi ? 127 - fx_clz64(s.hi) : 63 - fx_clz64(s.lo);   // leading bit
			int low = p - 52;                                                   // lowest kept bit
			if (61 - emax > low) low = 61 - emax;                               // subnormal result
			unsigned long long sig;
			if (low <= 0) {
				sig = s.lo << (-low);                                           // exact, < 2^53
			} else {
				// sig = s >> low; round bit = bit low-1; sticky = bits below it
				unsigned long long q, rb, st;
				if (low < 64) {
					q = (s.lo >> low) | (s.hi << (64 - low));
					rb = (s.lo >> (low - 1)) & 1ull;
					st = (low >= 2) ? (s.lo & ((1ull << (low - 1)) - 1ull)) : 0ull;
				} else if (low == 64) {
					q = s.hi;
					rb = s.lo >> 63;
					st = s.lo & ((1ull << 63) - 1ull);
				} else {
					const int l2 = low - 64;                                     // 1..63
					q = s.hi >> l2;
					rb = (s.hi >> (l2 - 1)) & 1ull;
					st = s.lo | ((l2 >= 2) ? (s.hi & ((1ull << (l2 - 1)) - 1ull)) : 0ull);
				}
				sig = q;
				if (rb && (st || (sig & 1ull))) sig += 1ull;
			}
			// value = sig * 2^(low + emax - 1135): exponent field - 1 = low + emax - 61 (0 for subnormals)
			// (a rounding carry to 2^53 moves into the exponent field; f1 <= 2060, so no wrap-around)
			const unsigned long long f1 = (unsigned long long) (low + emax - 61);
			bits = (f1 << 52) + sig;
			if (bits >= 0x7FF0000000000000ull) bits = 0x7FF0000000000000ull;   // overflow to infinity
		}
		if (neg) bits |= 1ull << 63;
	}
	double d;
#if defined(__CUDA_ARCH__)
	d = __longlong_as_double((long long) bits);
#else
	__builtin_memcpy(&d, &bits, 8);
#endif
	return d;
}

#if defined(__CUDACC__)
// b << sh in 128 bits, b < 2^32
__device__ __forceinline__ Fx fx_shl_small(unsigned long long b, int sh)
{
	Fx r;
	if (sh == 0) { r.lo = b; r.hi = 0ull; }
	else if (sh < 64) { r.lo = b << sh; r.hi = b >> (64 - sh); }
	else { r.lo = 0ull; r.hi = b << (sh - 64); }
	return r;
}

// Sum over the warp; every lane gets it.  The 128-bit two's-complement values are cut into six 24-bit
// limbs, each limb summed over the 32 lanes with one warp-reduce instruction (a sum of 32 limbs stays
// below 2^29), and the limb sums recombined modulo 2^128: the same exact sum as a shuffle tree of
// 128-bit adds (5 levels of 4 shuffles each), in 6 reduce instructions.
__device__ __forceinline__ Fx fx_warp_sum(Fx a)
{
	const unsigned long long m24 = 0xFFFFFFull;
	unsigned l[6];
	l[0] = (unsigned) (a.lo & m24);
	l[1] = (unsigned) ((a.lo >> 24) & m24);
	l[2] = (unsigned) (((a.lo >> 48) | (a.hi << 16)) & m24);
	l[3] = (unsigned) ((a.hi >> 8) & m24);
	l[4] = (unsigned) ((a.hi >> 32) & m24);
	l[5] = (unsigned) (a.hi >> 56);
	Fx r = fx_zero();
#pragma unroll
	for (int k = 0; k < 6; ++k) r = fx_add(r, fx_shl_small(__reduce_add_sync(0xffffffffu, l[k]), 24 * k));
	return r;
}

__device__ __forceinline__ int fx_warp_max(int e) { return (int) __reduce_max_sync(0xffffffffu, (unsigned) e); }
#endif

}  // namespace sa

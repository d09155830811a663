/*
 * jn_fixed.cuh — the exact 64-bit fixed-point accumulation shared by the
 * product kernels: contributions are rounded once to integers in units of
 * 2^-S and added as integers, so a sum does not depend on the order of its
 * terms.
 */
#ifndef JN_FIXED_CUH
#define JN_FIXED_CUH

/* exponent S of the fixed-point unit 2^-S: |y| <= abs_bound * max|x| <= 2^(62-S).
 * Integer arithmetic on the exponent field only, identical in every kernel. */
__device__ __forceinline__ int fixed_exponent(unsigned int xmax_bits, double abs_bound)
{
	const double yb = abs_bound * (double)__uint_as_float(xmax_bits);
	if (!(yb > 0.0)) return 0;
	const long long bits = __double_as_longlong(yb);
	int e = (int)((bits >> 52) & 0x7ff) - 1022;       /* yb < 2^e */
	int S = 62 - e;
	return S < -60 ? -60 : (S > 100 ? 100 : S);
}

template <typename T> __device__ __forceinline__ long long to_fixed(T v);
template <> __device__ __forceinline__ long long to_fixed<float>(float v) { return __float2ll_rn(v); }
template <> __device__ __forceinline__ long long to_fixed<double>(double v) { return __double2ll_rn(v); }

/* 64-bit two's-complement add into separate low / high 32-bit shared words
 * with two native 32-bit atomics: the carry of each addition is taken from
 * the value its own atomic saw, so (high, low) holds the exact sum modulo
 * 2^64 once every addition has landed, whatever their interleaving. */
__device__ __forceinline__ void add_fixed(unsigned int *lo, unsigned int *hi, int i, long long v)
{
	if (v == 0) return;
	const unsigned int l = (unsigned int)(unsigned long long)v;
	unsigned int h = (unsigned int)((unsigned long long)v >> 32);
	const unsigned int old = atomicAdd(lo + i, l);
	h += (unsigned int)(old + l < old);
	if (h) atomicAdd(hi + i, h);
}

/* the same for a 32-bit contribution: the high word takes the sign and the
 * carry, and is touched only when they do not cancel */
__device__ __forceinline__ void add_fixed32(unsigned int *lo, unsigned int *hi, int i, int v)
{
	const unsigned int u = (unsigned int)v;
	const unsigned int old = atomicAdd(lo + i, u);
	const int h = (v >> 31) + (int)(old + u < old);
	if (h) atomicAdd(hi + i, (unsigned int)h);
}

#endif

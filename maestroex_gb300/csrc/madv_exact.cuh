// Exact FP64 building blocks that cost fewer FP64 instructions than the literal
// expressions they replace.  GB300 issues two FP64 instructions per clock per SM against
// 128 integer/FP32 lanes, so moving exact work off the FP64 pipe pays directly.
//
// 1. Comparisons against zero or a non-negative threshold t on the IEEE bit pattern.
//    For finite (non-NaN) x and t >= +0:  x > t  <=>  int64(bits(x)) > int64(bits(t)),
//    since non-negative doubles order like their bit patterns and every negative double
//    (or -0) has a negative int64 pattern.  |x| and -x are exact bit operations.
//
// 2. Division by a constant y from a precomputed double-word reciprocal zh + zl
//    (zh = RN(1/y), zl = RN(1/y - zh)):
//        q0 = RN(a*zh + RN(a*zl))            faithful (error <= 1/2 ulp + 2^-104 rel.)
//        r  = RN(a - q0*y)                   exact (FMA; the remainder is representable)
//        q  = RN(q0 + r*zh)                  = RN(a/y)
//    The last step is Markstein's theorem (P. Markstein, IBM J. Res. Dev. 34(1), 1990;
//    see also N. Brisebarre, J.-M. Muller, S. K. Raina, IEEE Trans. Comput. 53(8),
//    2004): with zh the correctly rounded reciprocal and q0 faithful, the corrected
//    quotient is the correctly rounded one.  It holds while no intermediate underflows or
//    overflows; zeros and |a| outside [2^-959, 2^977) take the IEEE division instead.
//    Cost: 1 DMUL + 3 DFMA.
#pragma once
#include <cstdint>

namespace madv {

constexpr long long SIGN_BIT = (long long)0x8000000000000000ULL;
constexpr long long ABS_MASK = 0x7fffffffffffffffLL;

__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }
__host__ inline long long dbits_host(double x) {
    long long b;
    __builtin_memcpy(&b, &x, sizeof(b));
    return b;
}

// x > 0.0
__device__ __forceinline__ bool gt0(double x) { return dbits(x) > 0; }
// x < 0.0 (-0 is not below 0): the pattern of -x is positive
__device__ __forceinline__ bool lt0(double x) { return (dbits(x) ^ SIGN_BIT) > 0; }
// |x| > 0.0
__device__ __forceinline__ bool nz(double x) { return (dbits(x) & ABS_MASK) != 0; }
// x > t, with tb = bits(t), t >= +0
__device__ __forceinline__ bool gt_t(double x, long long tb) { return dbits(x) > tb; }
// x < -t, with tb = bits(t), t >= +0
__device__ __forceinline__ bool lt_negt(double x, long long tb) { return (dbits(x) ^ SIGN_BIT) > tb; }
// |x| > t, with tb = bits(t), t >= +0
__device__ __forceinline__ bool abs_gt_t(double x, long long tb) { return (dbits(x) & ABS_MASK) > tb; }


// 3. Scaling by 2 and by 1/2 on the bit pattern, equal to the FP multiply (round to nearest
//    even) for every input: a normal result is an exponent step; a zero or subnormal x has
//    |x| = a * 2^-1074 with a its magnitude bits (exponent field 1 included), so 2x is the
//    pattern 2a and x/2 the pattern RN(a/2); 2x past the largest finite double is infinity.
//    Infinities and NaNs pass through.  No FP64 instruction is issued.
__device__ __forceinline__ double twice(double x) {
    const long long b = dbits(x), a = b & ABS_MASK, sg = b & SIGN_BIT;
    long long r;
    if (a < (1LL << 52)) r = sg | (a << 1);                  // zero or subnormal
    else if (a < (0x7feLL << 52)) r = b + (1LL << 52);       // normal result
    else if (a < (0x7ffLL << 52)) r = sg | (0x7ffLL << 52);  // overflow
    else r = b;                                              // infinity, NaN
    return __longlong_as_double(r);
}
__device__ __forceinline__ double half(double x) {
    const long long b = dbits(x), a = b & ABS_MASK, sg = b & SIGN_BIT;
    long long r;
    if (a >= (0x7ffLL << 52)) r = b;                              // infinity, NaN
    else if (a >= (2LL << 52)) r = b - (1LL << 52);               // normal result
    else r = sg | ((a >> 1) + (a & (a >> 1) & 1));                // subnormal result, ties to even
    return __longlong_as_double(r);
}

// Riemann upwinding of the reference:  v = (u > 0) ? l : r;  v = (|u| > t) ? v : (l+r)/2
// (0.5 * x as half(x): the same bits, no FP64 multiply)
__device__ __forceinline__ double upwind(double u, double l, double r, long long tb) {
    const long long ub = dbits(u);
    if ((ub & ABS_MASK) > tb) return ub > 0 ? l : r;
    return half(l + r);
}

// 4. The sign of a product, x*y > 0, without the multiply: the operands are non-zero with
//    equal signs and the product does not round to zero.  With M the 53-bit significand (the
//    magnitude bits of a subnormal, exponent field taken as 1) and E the exponent field,
//    |x*y| = Mx*My * 2^(Ex+Ey-2150), which rounds to zero exactly when it is <= 2^-1075,
//    i.e. Mx*My <= 2^(1075-Ex-Ey).  Normal operands with Ex+Ey >= 972 never do (the common
//    case, decided by the signs alone); the rest compare the 106-bit significand product.
//    Operands are not NaN.
__device__ __forceinline__ bool prod_gt0(double x, double y) {
    const long long bx = dbits(x), by = dbits(y);
    const long long ax = bx & ABS_MASK, ay = by & ABS_MASK;
    if ((bx ^ by) < 0 || ax == 0 || ay == 0) return false;
    const int ex = (int)(ax >> 52), ey = (int)(ay >> 52);
    if (ex >= 1 && ey >= 1 && ex + ey >= 972) return true;
    if (ex == 0x7ff || ey == 0x7ff) return true;  // an infinity times a non-zero
    const unsigned long long mx = ex ? (unsigned long long)((ax & 0x000fffffffffffffLL) | (1LL << 52)) : ax;
    const unsigned long long my = ey ? (unsigned long long)((ay & 0x000fffffffffffffLL) | (1LL << 52)) : ay;
    const int k = 1075 - (ex ? ex : 1) - (ey ? ey : 1);
    if (k < 0) return true;
    if (k >= 106) return false;
    const unsigned long long lo = mx * my, hi = __umul64hi(mx, my);
    if (k >= 64) {
        const unsigned long long t = 1ULL << (k - 64);
        return hi > t || (hi == t && lo != 0);
    }
    return hi != 0 || lo > (1ULL << k);
}

struct RecipC {
    double y, zh, zl;
};

__host__ inline RecipC make_recip(double y) {
    RecipC r;
    r.y = y;
    r.zh = 1.0 / y;
    // 1/y - zh = (1 - zh*y)/y; the residual 1 - zh*y is exact with an FMA
    const double e = __builtin_fma(-r.zh, y, 1.0);
    r.zl = e / y;
    return r;
}

__device__ __forceinline__ double div_c(double a, const RecipC& r) {
    const int ex = (int)((dbits(a) & ABS_MASK) >> 52);
    if (ex < 64 || ex >= 2000) return a / r.y;
    const double q0 = __fma_rn(a, r.zh, a * r.zl);
    const double rem = __fma_rn(-q0, r.y, a);
    return __fma_rn(rem, r.zh, q0);
}

}  // namespace madv

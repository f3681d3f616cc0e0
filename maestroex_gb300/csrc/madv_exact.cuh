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
// |x| > 0.0
__device__ __forceinline__ bool nz(double x) { return (dbits(x) & ABS_MASK) != 0; }
// x > t, with tb = bits(t), t >= +0
__device__ __forceinline__ bool gt_t(double x, long long tb) { return dbits(x) > tb; }
// x < -t, with tb = bits(t), t >= +0
__device__ __forceinline__ bool lt_negt(double x, long long tb) { return (dbits(x) ^ SIGN_BIT) > tb; }
// |x| > t, with tb = bits(t), t >= +0
__device__ __forceinline__ bool abs_gt_t(double x, long long tb) { return (dbits(x) & ABS_MASK) > tb; }

// Riemann upwinding of the reference:  v = (u > 0) ? l : r;  v = (|u| > t) ? v : (l+r)/2
__device__ __forceinline__ double upwind(double u, double l, double r, long long tb) {
    const long long ub = dbits(u);
    if ((ub & ABS_MASK) > tb) return ub > 0 ? l : r;
    return 0.5 * (l + r);
}

// 3. Scaling by 2 and by 1/2 as a step of the exponent field: exact, and equal to the FP
//    multiply, whenever x and the result are normal numbers; zeros, subnormals, infinities
//    and results that would leave the normal range take the multiply.
__device__ __forceinline__ double twice(double x) {
    const long long b = dbits(x);
    const int e = (int)((b >> 52) & 0x7ff);
    return (e >= 1 && e <= 2045) ? __longlong_as_double(b + (1LL << 52)) : 2.0 * x;
}
__device__ __forceinline__ double half(double x) {
    const long long b = dbits(x);
    const int e = (int)((b >> 52) & 0x7ff);
    return (e >= 2 && e <= 2046) ? __longlong_as_double(b - (1LL << 52)) : 0.5 * x;
}

// 4. The sign of a product, x*y > 0, without the multiply: for normal x and y whose biased
//    exponents sum to more than 971, |x*y| >= 2^-1074 cannot round to zero, and the product
//    is positive exactly when the signs agree.  Zeros, subnormals and smaller exponent sums
//    take the multiply.
__device__ __forceinline__ bool prod_gt0(double x, double y) {
    const long long bx = dbits(x), by = dbits(y);
    const int ex = (int)((bx & ABS_MASK) >> 52), ey = (int)((by & ABS_MASK) >> 52);
    if (ex == 0 || ey == 0 || ex + ey <= 971) return x * y > 0.0;
    return (bx ^ by) >= 0;
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

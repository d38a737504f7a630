// bfp.cuh — block floating point for the pseudospectral FFTs: 64-bit integer
// arithmetic with one exponent per transform line.
//
// On GB300 the FP64 pipe issues at 1/64 of the FP32 rate, while 32-bit
// integer multiply-adds (IMAD, IMAD.WIDE) and 64-bit adds on the integer ALU
// run tens of times faster.  An FFT butterfly is additions and twiddle
// products, so the transforms run in fixed point:
//
//   * A line (one row or column being transformed) of FP64 values is scaled
//     by one power of two 2^sh, chosen from the largest exponent field in the
//     line, so that every value the transform can produce keeps its complex
//     magnitude below 2^61: a length-L DFT grows magnitudes by at most L, the
//     real-transform pre/post-processing by at most 4, and a complex value's
//     magnitude is at most sqrt(2) times its largest component.  The largest
//     input component therefore keeps 61 - G bits, G = log2 L + 1 (column
//     transforms) or log2 L + 3 (the real-row transforms), 48 to 50 bits for
//     the boxes of the benchmark.  Values convert with integer operations
//     only (round to nearest, ties away from zero, on the way in; round to
//     nearest even on the way out).
//   * Additions are exact.  A twiddle w is stored as W = round(w 2^61), split
//     into 31-bit limbs W = h 2^31 + l (0 <= l < 2^31); a product
//     round(X W / 2^61) is formed from 32 x 32 -> 64-bit partial products
//     (IMAD.WIDE) and one high product __umulhi, exactly except for the
//     dropped fraction of the low limbs' product (< 2^-30 of a unit), so each
//     real component of a complex product is rounded once: error at most
//     1/2 + 2^-29 units.
//   * A line holding a NaN or an infinity yields NaN for the whole line, as a
//     floating-point transform would.
//
// Bounds that keep every 64-bit intermediate in range, with |X| < 2^61 for
// every complex magnitude: |X >> 31| <= 2^30 and |h| <= 2^30, so the
// high-limb products are below 2^60 and the middle sum of one component (two
// h l cross terms of each factor, two high products of at most 2^31, the
// rounding constant) stays below 2^62.8.
#pragma once

#include <cuda_runtime.h>

namespace chgb {

// A complex value of a line in fixed point; same size and alignment as double2.
struct __align__(16) fx2 {
    long long x, y;
};

constexpr int FX_TOP = 61;   // every complex magnitude stays below 2^FX_TOP

__device__ __forceinline__ int fx_hi(long long v) { return (int) (v >> 31); }
__device__ __forceinline__ int fx_lo(long long v) { return (int) (v & 0x7FFFFFFFll); }
// floor(xl * wl / 2^31) for limbs xl, wl in [0, 2^31)
__device__ __forceinline__ long long fx_lohi(int xl, int wl) {
    return (long long) __umulhi((unsigned) xl << 1, (unsigned) wl);
}
__device__ __forceinline__ long long wide(int a, int b) { return (long long) a * (long long) b; }

// round(a w / 2^61) (CONJ = false) or round(a conj(w) / 2^61) (CONJ = true);
// w = {hx, lx, hy, ly}, the limbs of the twiddle's real and imaginary parts.
template <bool CONJ>
__device__ __forceinline__ fx2 fx_cmul(fx2 a, int4 w) {
    const int xh = fx_hi(a.x), xl = fx_lo(a.x), yh = fx_hi(a.y), yl = fx_lo(a.y);
    const long long r1 = (1ll << 29);
    // X Wx and Y Wy, X Wy and Y Wx, each as (high part A, middle part M)
    const long long a_xx = wide(xh, w.x), m_xx = wide(xh, w.y) + wide(xl, w.x) + fx_lohi(xl, w.y);
    const long long a_yy = wide(yh, w.z), m_yy = wide(yh, w.w) + wide(yl, w.z) + fx_lohi(yl, w.w);
    const long long a_xy = wide(xh, w.z), m_xy = wide(xh, w.w) + wide(xl, w.z) + fx_lohi(xl, w.w);
    const long long a_yx = wide(yh, w.x), m_yx = wide(yh, w.y) + wide(yl, w.x) + fx_lohi(yl, w.y);
    fx2 r;
    if(!CONJ) {   // re = X Wx - Y Wy, im = X Wy + Y Wx
        r.x = 2 * (a_xx - a_yy) + ((m_xx - m_yy + r1) >> 30);
        r.y = 2 * (a_xy + a_yx) + ((m_xy + m_yx + r1) >> 30);
    }
    else {        // re = X Wx + Y Wy, im = Y Wx - X Wy
        r.x = 2 * (a_xx + a_yy) + ((m_xx + m_yy + r1) >> 30);
        r.y = 2 * (a_yx - a_xy) + ((m_yx - m_xy + r1) >> 30);
    }
    return r;
}

__device__ __forceinline__ fx2 fx_add(fx2 a, fx2 b) { return fx2{a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ fx2 fx_sub(fx2 a, fx2 b) { return fx2{a.x - b.x, a.y - b.y}; }

// Biased exponent field of a double (0 for zeros and subnormals, 2047 for inf/NaN).
__device__ __forceinline__ int fx_expo(double v) { return (int) ((__double_as_longlong(v) >> 52) & 0x7FF); }

// The scale of a line whose largest exponent field is `emax`, for headroom G:
// the largest component below 2^(FX_TOP - G) after multiplying by 2^sh.  A
// value with exponent field e is below 2^(e - 1022).
__device__ __forceinline__ int fx_scale(int emax, int G) { return FX_TOP - G + 1022 - (emax < 1 ? 1 : emax); }

// round(v 2^sh) to nearest, ties away from zero, with integer operations.
__device__ __forceinline__ long long fx_from_double(double v, int sh) {
    const long long b = __double_as_longlong(v);
    int e = (int) ((b >> 52) & 0x7FF);
    long long m = b & 0xFFFFFFFFFFFFFll;
    if(e) m |= 1ll << 52;
    else e = 1;
    // |v| = m 2^(e - 1075)
    const int s = e - 1075 + sh;
    long long r;
    if(s >= 0) r = m << s;
    else {
        const int t = -s;
        r = t > 62 ? 0 : ((m >> (t - 1)) + 1) >> 1;
    }
    return b < 0 ? -r : r;
}

// X 2^-sh as the nearest double (ties to even), with integer operations only
// (an FP64 fallback would be if-converted by the compiler and run for every
// value): results below the normal range round to a subnormal, results above
// it become infinities.
__device__ __forceinline__ double fx_to_double(long long X, int sh) {
    if(X == 0) return 0.0;
    const unsigned long long a = X < 0 ? (unsigned long long) (-X) : (unsigned long long) X;
    const int len = 64 - __clzll((long long) a);
    // keep 53 bits (a normal result, exponent field E) or, below the normal
    // range, the bits a subnormal holds; one rounding either way
    int d = len - 53;
    int E = d - sh + 1075;
    const bool sub = E <= 0;
    if(sub) d += 1 - E;
    unsigned long long q;
    if(d > 62) q = 0;
    else if(d > 0) {
        q = a >> d;
        const unsigned long long rem = a & ((1ull << d) - 1), half = 1ull << (d - 1);
        if(rem > half || (rem == half && (q & 1))) q++;
    }
    else {
        q = a << (-d);
    }
    unsigned long long bits;
    if(sub) {
        bits = q;   // units of 2^-1074; a carry into 2^52 is the smallest normal number
    }
    else {
        if(q >> 53) {
            q >>= 1;
            E++;
        }
        bits = E >= 2047 ? 0x7FF0000000000000ull : (((unsigned long long) E << 52) | (q & 0xFFFFFFFFFFFFFull));
    }
    if(X < 0) bits |= 1ull << 63;
    return __longlong_as_double((long long) bits);
}

__device__ __forceinline__ fx2 fx_load(double2 v, int sh) { return fx2{fx_from_double(v.x, sh), fx_from_double(v.y, sh)}; }
__device__ __forceinline__ double2 fx_store(fx2 v, int sh) {
    return make_double2(fx_to_double(v.x, sh), fx_to_double(v.y, sh));
}

// Maximum of `e` over the tpl threads of each line (threads li * tpl + lane of
// the block, tpl a power of two); the result lands in sm_e[li].  tpl >= 32:
// one warp reduction and one shared atomic per warp, sm_e[li] zeroed by the
// caller before a barrier; tpl < 32: shuffles within the line's lanes.  The
// caller synchronises before reading sm_e.
__device__ __forceinline__ void fx_line_max(int e, int tpl, int li, int lane, bool active, int *sm_e) {
    const int nthr = blockDim.x;
    const int wbase = threadIdx.x & ~31;
    const unsigned mask = (nthr - wbase >= 32) ? 0xffffffffu : ((1u << (nthr - wbase)) - 1u);
    if(tpl >= 32) {
        e = __reduce_max_sync(mask, e);
        if((threadIdx.x & 31) == 0 && active) atomicMax(&sm_e[li], e);
    }
    else {
        for(int o = tpl / 2; o > 0; o >>= 1) e = max(e, __shfl_xor_sync(mask, e, o));
        if(lane == 0 && active) sm_e[li] = e;
    }
}

}  // namespace chgb

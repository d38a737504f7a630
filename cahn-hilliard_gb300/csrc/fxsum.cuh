// fxsum.cuh — neighbour sums of the explicit steps' Laplacians in 64-bit
// fixed-point integer arithmetic (device code shared by the euler and adjoint
// kernels).
#pragma once

#include <cuda_runtime.h>

namespace chgb {

// Neighbour sums of the 2D and 3D Laplacians in integer arithmetic.
//
// GB300 issues FP64 instructions at 1/64 of its FP32 rate, and the explicit
// steps are bound by them while the integer pipes idle.  A sum of K doubles is
// formed here in 64-bit fixed point:
//   - each term x becomes T = +-mantissa * 2^FX_GUARD (|T| < 2^58) with the
//     exponent ek = max(biased exponent, 1) (fx_term);
//   - the terms are aligned to the largest ek, emax, by arithmetic right shifts
//     (floor: bits more than FX_GUARD places below the largest term's last
//     mantissa bit are dropped) and added exactly;
//   - the total is rounded once, to nearest, by the int64 -> double conversion
//     and scaled by 2^(emax - 1075 - FX_GUARD) through the exponent field.
// The error is one rounding of the sum plus less than K / 32 ulp of the
// largest term (a sequential FP64 sum rounds K - 1 times); the result does not
// depend on the order of the terms, nor on whether the fixed-point forms were
// computed where the sum is taken or once, when the values were staged in
// shared memory -- every kernel variant gets the same bits.  The update's
// Laplacian numerator (fx_lap) carries the centre's -2 dims psi as one more
// term, exact as a multiple of its fixed-point form, rounded with the sum.
// Sums whose largest term lies outside [2^-959, 2^977] (all zeros, subnormals only,
// overflow, inf, NaN) take the sequential FP64 sum in the reference's
// neighbour order (-x, +x, -y, +y, -z, +z) instead.
constexpr int FX_GUARD = 5;

static __device__ __noinline__ double seq_sum(double a, double b, double c, double d, double e, double f, int n) {
    double sum = a + b;
    sum += c;
    sum += d;
    if(n > 4) {
        sum += e;
        sum += f;
    }
    return sum;
}

__device__ __forceinline__ void fx_term(double x, long long &T, int &ek) {
    const unsigned long long u = (unsigned long long) __double_as_longlong(x);
    const int e = (int) (u >> 52) & 0x7FF;
    const unsigned long long mag = (u & 0xFFFFFFFFFFFFFull) | (e ? 1ull << 52 : 0ull);
    T = (long long) (((u >> 63) ? 0ull - mag : mag) << FX_GUARD);
    ek = e ? e : 1;
}

template <int K>
__device__ __forceinline__ int fx_emax(const int (&ek)[K]) {
    int emax = ek[0];
#pragma unroll
    for(int i = 1; i < K; i++) emax = ek[i] > emax ? ek[i] : emax;
    return emax;
}

__device__ __forceinline__ bool fx_in_range(int emax) { return emax >= 64 && emax <= 2000; }

// x >> n, arithmetic, for n >= 0.  PTX clamps a shift amount above 63 to 64,
// which leaves the sign fill (0 or -1) -- what a shift by 63 leaves for the
// |x| < 2^62 here -- so no clamp is needed before the shift (C++ leaves
// n >= 64 undefined).
__device__ __forceinline__ long long fx_sar(long long x, int n) {
    long long r;
    asm("shr.s64 %0, %1, %2;" : "=l"(r) : "l"(x), "r"(n));
    return r;
}

// The fixed-point total of K terms whose largest exponent emax is in range,
// plus an optional centre term Tc (already multiplied: |Tc| < 6 * 2^58) of
// exponent ekc <= emax -- the Laplacian's -2 dims psi, rounded with the sum.
// The final rounding to nearest-even is done either by the int64 -> double
// conversion (one instruction on the FP64 pipe) or, with INT_ROUND, in integer
// arithmetic (about thirty integer instructions) -- the same bits; a kernel
// whose FP64 pipe is the busier one takes the second.
template <int K, bool INT_ROUND = false>
__device__ __forceinline__ double fx_total(const long long (&T)[K], const int (&ek)[K], int emax, long long Tc = 0,
                                           int ekc = 1) {
    // K <= 6 terms below 2^58 and a centre term below 6 * 2^58: |acc| < 2^62
    long long acc = 0;
#pragma unroll
    for(int i = 0; i < K; i++) acc += fx_sar(T[i], emax - ek[i]);
    acc += fx_sar(Tc, emax - ekc);
    if(acc == 0) return 0.0;
    // the value is acc * 2^(emax - 1075 - FX_GUARD); its exponent stays in
    // [emax - 57, emax + 4]: a normal number
    if constexpr(INT_ROUND) {
        const unsigned long long a = acc < 0 ? 0ull - (unsigned long long) acc : (unsigned long long) acc;
        const int top = 63 - __clzll((long long) a);   // leading bit, <= 61
        int E = emax - FX_GUARD + top - 52;
        unsigned long long M;
        if(top > 52) {
            const int r = top - 52;
            const unsigned long long rem = a & ((1ull << r) - 1), half = 1ull << (r - 1);
            M = a >> r;
            if(rem > half || (rem == half && (M & 1))) {
                M++;
                if(M >> 53) {
                    M >>= 1;
                    E++;
                }
            }
        }
        else {
            M = a << (52 - top);
        }
        return __longlong_as_double((long long) (((unsigned long long) (acc < 0) << 63) |
                                                 ((unsigned long long) E << 52) | (M & 0xFFFFFFFFFFFFFull)));
    }
    else {
        const double f = __ll2double_rn(acc);
        return __longlong_as_double(__double_as_longlong(f) + ((long long) (emax - 1075 - FX_GUARD) << 52));
    }
}

template <int K>
__device__ __forceinline__ double fx_sum(const double (&x)[K]) {
    static_assert(K == 4 || K == 6, "4 or 6 neighbours");
    long long T[K];
    int ek[K];
#pragma unroll
    for(int i = 0; i < K; i++) fx_term(x[i], T[i], ek[i]);
    const int emax = fx_emax<K>(ek);
    if(!fx_in_range(emax))
        return seq_sum(x[0], x[1], x[2], x[3], K > 4 ? x[K > 4 ? 4 : 0] : 0.0, K > 4 ? x[K > 4 ? 5 : 0] : 0.0, K);
    return fx_total<K>(T, ek, emax);
}

// The Laplacian's numerator, sum(x) - K v (K = 2 dims neighbours), in one
// rounding: the centre term is -K times v's fixed-point form, exact.
template <int K>
__device__ __forceinline__ double fx_lap(const double (&x)[K], double v) {
    static_assert(K == 4 || K == 6, "4 or 6 neighbours");
    long long T[K];
    int ek[K];
#pragma unroll
    for(int i = 0; i < K; i++) fx_term(x[i], T[i], ek[i]);
    long long Tv;
    int ekv;
    fx_term(v, Tv, ekv);
    int emax = fx_emax<K>(ek);
    emax = ekv > emax ? ekv : emax;
    if(!fx_in_range(emax))
        return fma(-(double) K, v,
                   seq_sum(x[0], x[1], x[2], x[3], K > 4 ? x[K > 4 ? 4 : 0] : 0.0, K > 4 ? x[K > 4 ? 5 : 0] : 0.0, K));
    return fx_total<K>(T, ek, emax, -(long long) K * Tv, ekv);
}

__device__ __forceinline__ double lap4(double a, double b, double c, double d, double v) {
    const double x[4] = {a, b, c, d};
    return fx_lap<4>(x, v);
}

__device__ __forceinline__ double lap6(double a, double b, double c, double d, double e, double f, double v) {
    const double x[6] = {a, b, c, d, e, f};
    return fx_lap<6>(x, v);
}

__device__ __forceinline__ double nb_sum4(double a, double b, double c, double d) {
    const double x[4] = {a, b, c, d};
    return fx_sum<4>(x);
}

__device__ __forceinline__ double nb_sum6(double a, double b, double c, double d, double e, double f) {
    const double x[6] = {a, b, c, d, e, f};
    return fx_sum<6>(x);
}

}  // namespace chgb

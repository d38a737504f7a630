// common.cuh — shared device-side definitions of the chgb CUDA library
// (sm_103a, FP64 throughout).
//
// Layout of every field in HBM: species-major, data[s * bins + idx] with
// idx = x + N*y + N*N*z (the reference's MultiField, src/utils/MultiField.h:59-63),
// periodic wrap by bit mask (src/CahnHilliard.cpp:50-56).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/chgb.h"

namespace chgb {

// Free-energy model constants, derived once on the host from chgb_model_params
// the way the model constructors derive them (src/models/SimpleWertheim.cpp:20-34,
// src/models/SalehWertheim.cpp:19-41).
struct ModelDev {
    int kind;
    int S;
    double epsilon;                 // landau
    double valence;                 // simple_wertheim valence as double
    double B2, B3;
    double two_valence_delta;       // 2 * valence * delta
    double four_valence_delta;      // 2 * two_valence_delta (exact: a power-of-two multiple)
    double two_B2;                  // 2 * B2 (exact)
    double reg_delta, log_delta;    // regularisation_delta and log(regularisation_delta)
    double sv0, sv1, half;          // saleh valences of A and B, linker half valence
    double dAA, dBB;
    double dcf;                     // density conversion factor
    int ivalence;
    // table of tab_log (LOGTAB_N entries (1/c_j, ln c_j), then (ln 2 high, low)),
    // in device memory; nullptr: f' takes the library's log instead
    const double2 *logtab;
};

constexpr int LOGTAB_N = 128;

// with_log_table = false never allocates (the table is used if an earlier
// call made it for the current device).
ModelDev make_model_dev(const chgb_model_params &m, bool with_log_table = true);

// Grid geometry and the step constants folded once per handle.
struct Geom {
    int dims, N, log2N, mask;
    int bins;                       // N^dims
    int S;
};

struct EulerConsts {
    double c2[CHGB_MAX_SPECIES];    // 2 k_s / dx^2  (surface term of mu)
    double c1;                      // dt * M / dx^2 (constant-mobility update)
    double dt;
    double half_inv_dx2;            // 0.5 / dx^2   (face flux and divergence folded)
    double M;                       // constant mobility / M0
    double lshift[3];               // Landau: 2 d c2 - eps for d = 1, 2, 3 (species 0)
    int mobility_type;
    const double *mobf;             // regularised / gel: the mobility field of this step
};

// Per-step mobility update of the `regularised` and `gel` types
// (src/mobility/RegularisedMobility.h:26-33, src/mobility/GelMobility.h:41-58).
struct MobilityDev {
    int type;                       // CHGB_MOBILITY_REGULARISED or CHGB_MOBILITY_GEL
    double M, rho_min;              // regularised
    double p_gel, phi_critical, c0, M_c, dt;   // gel
    double one_m_phic, inv_one_m_phic, inv_c0;  // 1 - phi_c and the reciprocals of the gel's two divisors
    const double2 *exptab;          // table of tab_exp (null: the library's exp)
};

constexpr int EXPTAB_N = 64;   // tab_exp: 2^(j/64) for j < 64, then two rows of constants

// (0 + i k) z, as std::complex<double> evaluates it: the wave-vector factor of
// a spectral derivative (src/integrators/PseudospectralMobilityCPU.cpp:258-263)
__device__ __forceinline__ double2 mul_ik(double k, double2 z) {
    return make_double2(0.0 * z.x - k * z.y, 0.0 * z.y + k * z.x);
}

// ---------------------------------------------------------------------------
// Models.  Each formula follows the reference's CPU code (the oracle); the
// reference's own CUDA kernels are single precision and are not followed.
// ---------------------------------------------------------------------------

// x^n for the model's integer valence n >= 0, by repeated squaring: the
// reference's std::pow(X, (double) valence) to within a few ulp at a fraction
// of a general pow's FP64 work.
__device__ __forceinline__ double ipow(double x, int n) {
    double r = 1.0;
    while(n > 0) {
        if(n & 1) r *= x;
        x *= x;
        n >>= 1;
    }
    return r;
}

// 1/x: the hardware's approximate reciprocal (relative error below 2^-20,
// measured on GB300) refined by two Newton steps y <- y + y (1 - x y), each
// squaring the error.  Within 2 ulp of 1/x, for four FMAs instead of the ten
// or so FP64 instructions of a correctly rounded division.  Subnormal x is
// flushed to zero (1/x = inf, then NaN), as for x = 0.
__device__ __forceinline__ double fast_rcp(double x) {
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    double e = fma(-x, y, 1.0);
    y = fma(y, e, y);
    e = fma(-x, y, 1.0);
    return fma(y, e, y);
}

// x / d for a divisor d known in advance, y = RN(1/d): q0 = RN(x y), the
// remainder x - q0 d exact by one FMA, then q = RN(q0 + r y) -- division by a
// constant with one correction step (P. Markstein, "IA-64 and Elementary
// Functions", 2000; N. Brisebarre, J.-M. Muller and S. K. Raina, IEEE Trans.
// Computers 53 (2004)).  The correctly rounded quotient for all but rare
// (x, d) pairs, and within 1 ulp of it always, for three FP64 instructions
// against about ten for a division.  x infinite gives NaN, not infinity.
__device__ __forceinline__ double div_known(double x, double d, double y) {
    const double q0 = x * y;
    const double r = fma(-q0, d, x);
    return fma(r, y, q0);
}

// ln x by table lookup and a short polynomial, after P. T. P. Tang,
// "Table-driven implementation of the logarithm function in IEEE
// floating-point arithmetic", ACM TOMS 16 (1990): x = 2^k y with y in [1, 2),
// c_j = 1 + (j + 1/2)/128 for the top seven mantissa bits j of y, and
//     ln x = k ln 2 + ln c_j + ln(1 + r),  r = (y - c_j) / c_j,  |r| <= 2^-8,
// y - c_j exact, ln(1 + r) by its Taylor polynomial to r^7 (truncation below
// 2^-67).  13 FP64 instructions against 29 for the library's log (measured
// with ncu on GB300).  The error stays below 2 ulp of the result, or of 1.0
// where |ln x| < 1 (near x = 1 k ln 2 and ln c_j cancel; the f' terms fed are of
// order 10).  Zero,
// negative, subnormal, infinite and NaN arguments -- and a missing table --
// take the library's log.
__device__ __noinline__ static double log_fallback(double x) { return log(x); }

__device__ __forceinline__ double tab_log(double x, const double2 *__restrict__ tab) {
    const unsigned long long u = (unsigned long long) __double_as_longlong(x);
    const unsigned se = (unsigned) (u >> 52);   // sign and biased exponent
    if(tab == nullptr || se - 1u >= 2046u) return log_fallback(x);
    const int j = (int) (u >> 45) & (LOGTAB_N - 1);
    const double y = __longlong_as_double((long long) ((u & 0xFFFFFFFFFFFFFull) | 0x3FF0000000000000ull));
    const double c = __longlong_as_double(
        (long long) (0x3FF0000000000000ull | ((unsigned long long) j << 45) | (1ull << 44)));
    const double2 t = __ldg(&tab[j]);
    const double2 ln2 = __ldg(&tab[LOGTAB_N]);
    const double r = (y - c) * t.x;
    double q = fma(r, 1.0 / 7.0, -1.0 / 6.0);
    q = fma(q, r, 1.0 / 5.0);
    q = fma(q, r, -0.25);
    q = fma(q, r, 1.0 / 3.0);
    q = fma(q, r, -0.5);
    const double p = fma(r * r, q, r);
    const double k = (double) ((int) se - 1023);
    return fma(k, ln2.x, t.y) + fma(k, ln2.y, p);
}

// e^x by table lookup and a short polynomial, after P. T. P. Tang,
// "Table-driven implementation of the exponential function in IEEE
// floating-point arithmetic", ACM TOMS 15 (1989), with 64 table entries:
//     x = (64 m + j) ln2/64 + r,  |r| <= ln2/128 (plus rounding),
//     e^x = 2^m 2^(j/64) (1 + p(r)),  p(r) = e^r - 1 by its Taylor polynomial
// to r^6 (truncation below 2^-64).  n = 64 m + j comes from adding 1.5 2^52 to
// x 64/ln2 (round to nearest); r = x - n L1 - n L2 with ln2/64 = L1 + L2, L1
// of 37 significant bits, so that x - n L1 is exact (Sterbenz).  2^(j/64) is
// a pair (lead, trail); e^x = 2^m (lead + (trail + lead p)), and 2^m enters
// through the exponent field.  12 FP64 instructions; the error stays below
// 0.52 ulp plus the table's rounding (checked against an exact model on the
// CPU).  |x| > 700 (the result near the ends of the normal range or beyond),
// NaN and a missing table take the library's exp.  Table: EXPTAB_N entries
// (lead, trail), then (L1, L2), then (64/ln2, 0).
__device__ __noinline__ static double exp_fallback(double x) { return exp(x); }

__device__ __forceinline__ double tab_exp(double x, const double2 *__restrict__ tab) {
    const unsigned long long a = (unsigned long long) __double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
    if(tab == nullptr || a > 0x4085E00000000000ull) return exp_fallback(x);   // |x| > 700 or NaN
    const double2 L = __ldg(&tab[EXPTAB_N]);
    const double2 K = __ldg(&tab[EXPTAB_N + 1]);
    constexpr double SHIFT = 6755399441055744.0;   // 1.5 2^52
    const double t = fma(x, K.x, SHIFT);
    const int n = (int) __double2loint(t);
    const double nd = t - SHIFT;
    const double r = fma(-nd, L.y, fma(-nd, L.x, x));
    double q = fma(r, 1.0 / 720.0, 1.0 / 120.0);
    q = fma(q, r, 1.0 / 24.0);
    q = fma(q, r, 1.0 / 6.0);
    q = fma(q, r, 0.5);
    const double p = fma(r * r, q, r);
    const double2 sj = __ldg(&tab[n & (EXPTAB_N - 1)]);
    const double v = sj.x + fma(sj.x, p, sj.y);
    return __longlong_as_double(__double_as_longlong(v) + ((long long) (n >> 6) << 52));
}

// X(rho) of src/models/SimpleWertheim.cpp:88-90 (the division by the fast
// reciprocal above).
__device__ __forceinline__ double sw_X(const ModelDev &m, double rho) {
    return (-1.0 + sqrt(1.0 + m.four_valence_delta * rho)) * fast_rcp(m.two_valence_delta * rho);
}

// X of one Saleh species pair, src/models/SalehWertheim.cpp:80-85; returns log X.
__device__ __forceinline__ double saleh_log_X(double delta, double v, double rho_s, double half, double rho_linker,
                                              const double2 *tab) {
    double rho_factor = delta * (v * rho_s + half * rho_linker);
    double X = (-1.0 + sqrt(1.0 + 4.0 * rho_factor)) * fast_rcp(2.0 * rho_factor);
    return (rho_factor >= 0) ? tab_log(X, tab) : 0.0;
}

// f'(rho) of all S species of one cell: r[s] in, d[s] out.
template <int KIND>
__device__ __forceinline__ void der_bulk(const ModelDev &m, const double *r, double *d);

// src/models/Landau.cpp:46-53: f' = -eps psi + psi^3
template <>
__device__ __forceinline__ void der_bulk<CHGB_MODEL_LANDAU>(const ModelDev &m, const double *r, double *d) {
    double op = r[0];
    d[0] = fma(-m.epsilon, op, (op * op) * op);
}

// f' of simple_wertheim for a given X(rho), src/models/SimpleWertheim.cpp:40-53
__device__ __forceinline__ double sw_der_given_X(const ModelDev &m, double rho, double X) {
    double der_f_ref = m.two_B2 * rho;
    if(rho < m.reg_delta) {
        der_f_ref += m.log_delta + (rho - m.reg_delta) / m.reg_delta;
        double der_f_bond = (rho > 0.) ? m.valence * log(X) : 0.0;
        return der_f_ref + der_f_bond;
    }
    // log(rho) + valence log(X) as one logarithm, log(rho X^valence): the
    // same value to round-off for one logarithm's FP64 work instead of two
    return der_f_ref + tab_log(rho * ipow(X, m.ivalence), m.logtab);
}

// src/models/SimpleWertheim.cpp:40-53
template <>
__device__ __forceinline__ void der_bulk<CHGB_MODEL_SIMPLE_WERTHEIM>(const ModelDev &m, const double *r, double *d) {
    d[0] = sw_der_given_X(m, r[0], sw_X(m, r[0]));
}

// src/models/SalehWertheim.cpp:87-109.  A species whose density is exactly
// zero gets f' = 0 (the reference leaves the previous scratch value there).
template <>
__device__ __forceinline__ void der_bulk<CHGB_MODEL_SALEH>(const ModelDev &m, const double *r, double *d) {
    double rho_tot = ((0. + r[0]) + r[1]) + r[2];
    double b2 = m.two_B2 * rho_tot;
    double b3 = 3.0 * m.B3 * (rho_tot * rho_tot);
    double lx0 = saleh_log_X(m.dAA, m.sv0, r[0], m.half, r[2], m.logtab);
    double lx1 = saleh_log_X(m.dBB, m.sv1, r[1], m.half, r[2], m.logtab);
    d[0] = (r[0] != 0.) ? ((tab_log(r[0], m.logtab) + b2) + b3) + m.sv0 * lx0 : 0.0;
    d[1] = (r[1] != 0.) ? ((tab_log(r[1], m.logtab) + b2) + b3) + m.sv1 * lx1 : 0.0;
    d[2] = (r[2] != 0.) ? ((tab_log(r[2], m.logtab) + b2) + b3) + m.half * (lx0 + lx1) : 0.0;
}

// Free-energy mobility M0 * rho * X^valence, src/models/SimpleWertheim.cpp:104-111.
__device__ __forceinline__ double sw_mobility_given_X(const ModelDev &m, double M0, double rho, double X) {
    double D = M0 * ipow(X, m.ivalence);
    return rho * D;
}

__device__ __forceinline__ double sw_mobility(const ModelDev &m, double M0, double rho) {
    return sw_mobility_given_X(m, M0, rho, sw_X(m, rho));
}

// Bulk free-energy density f(rho) of one cell (r[s] for all species).
template <int KIND>
__device__ __forceinline__ double bulk_fe(const ModelDev &m, const double *r);

// src/models/Landau.cpp:55-58
template <>
__device__ __forceinline__ double bulk_fe<CHGB_MODEL_LANDAU>(const ModelDev &m, const double *r) {
    double op = r[0];
    return -0.5 * m.epsilon * (op * op) + 0.25 * ((op * op) * (op * op));
}

// src/models/SimpleWertheim.cpp:71-86
template <>
__device__ __forceinline__ double bulk_fe<CHGB_MODEL_SIMPLE_WERTHEIM>(const ModelDev &m, const double *r) {
    double rho = r[0];
    double reg = m.reg_delta;
    double f_ref = m.B2 * (rho * rho);
    if(rho < reg) {
        double a = 1 / (2.0 * reg);
        double b = m.log_delta - 1.0;
        double c = reg * (m.log_delta - 1.0) - a * (reg * reg) - b * reg;
        f_ref += a * (rho * rho) + b * rho + c;
    }
    else {
        f_ref += rho * (log(rho * m.dcf) - 1.0);
    }
    double f_bond = 0.0;
    if(rho > 0.) {
        double X = sw_X(m, rho);
        f_bond = m.valence * rho * (log(X) + 0.5 * (1. - X));
    }
    return f_ref + f_bond;
}

// src/models/SalehWertheim.cpp:47-78
template <>
__device__ __forceinline__ double bulk_fe<CHGB_MODEL_SALEH>(const ModelDev &m, const double *r) {
    double rho = ((0. + r[0]) + r[1]) + r[2];
    double mixing_S = 0.;
    for(int i = 0; i < 3; i++) {
        double x_i = r[i] / rho;
        mixing_S += (x_i > 0) ? x_i * log(x_i) : 0;
    }
    double B2_contrib = m.B2 * rho;
    double B3_contrib = 0.5 * m.B3 * (rho * rho);
    double f_ref = rho * (log(rho * m.dcf) - 1.0 + mixing_S + B2_contrib + B3_contrib);

    double rf = m.dAA * (m.sv0 * r[0] + m.half * r[2]);
    double X_1A = (-1.0 + sqrt(1.0 + 4.0 * rf)) / (2.0 * rf);
    double fe1 = log(X_1A) - X_1A / 2.0 + 0.5;
    rf = m.dBB * (m.sv1 * r[1] + m.half * r[2]);
    double X_2B = (-1.0 + sqrt(1.0 + 4.0 * rf)) / (2.0 * rf);
    double fe2 = log(X_2B) - X_2B / 2.0 + 0.5;
    double bonding = r[0] * m.sv0 * fe1 + r[1] * m.sv1 * fe2 + r[2] * m.half * (fe1 + fe2);
    return f_ref + bonding;
}

struct KArr {
    double v[CHGB_MAX_SPECIES];
};

template <int KIND>
struct NSpecies {
    static constexpr int value = (KIND == CHGB_MODEL_SALEH) ? 3 : 1;
};

}  // namespace chgb

// nc_fold.h — the reference's `float += double` of charge_insynapses
// (src/NeuCor.cpp:695: potential += deltaT*AP_depolFac*0.9943*exp(0.3702*deltaT), a
// float accumulator and a double term) without FP64 instructions on the common path.
//
// The result of one add is RN24(RN53(p + T)) for the float accumulator p and the double
// term T.  Each term is stored split (NcSplitTerm): hi = RN24(T) and the exact tail
// T - hi as an integer count of 2^(e_hi - 53), where e_hi is hi's exponent.  The add is
// then
//
//   s = RN24(p + hi);  e = (p + hi) - s   (Dekker's Fast2Sum: exact when e_hi <= e_p)
//
// and the result is s except when p + hi falls exactly halfway between s and its
// neighbour s + 2e (|e| = ulp(s)/2): the tail decides that tie — it moves the sum past
// the midpoint, after the 53-bit rounding, iff |tail| > 2^(e_s - 53), towards the
// neighbour iff the tail has e's sign.
//
// Why s is right otherwise: with 1 <= e_s - e_hi (a) p + hi is a multiple of
// g = ulp(hi) <= ulp(s)/2, so it is a midpoint of s's grid or at least g away from
// one; the tail moves it by at most g/2, and with e_s - e_hi <= 27 (b) the 53-bit
// rounding moves it by less than the remaining g/2, so the sum rounds like p + hi.
// A power-of-two s with e != 0 (its lower neighbour is ulp(s)/2 away, not ulp(s)) and
// everything outside (a), (b) and e_hi <= e_p is reported as rare: the caller redoes its
// batch with the hardware double add on the exact terms (nc_term_value).
//
// Terms outside [2^-90, 2^90) in magnitude (subnormal weights and the like) are kept as
// the float x = deltaT*AP_depolFac they came from and recomputed exactly when folded;
// their marker hi is a NaN, which always takes the rare path.
//
// Plain float arithmetic throughout: device code is built with --fmad=false and host
// code with -ffp-contract=off, so every + and - is one IEEE round-to-nearest operation
// on both, and the host build of this header checks the device's arithmetic.
#pragma once
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define NC_FOLD_HD __host__ __device__ __forceinline__
#else
#define NC_FOLD_HD inline
#endif

struct
#if defined(__CUDACC__)
    __align__(8)
#endif
        NcSplitTerm {
    float hi;    // RN24(T); +-0 for T = +-0; NC_TERM_EXOTIC for a term kept as x
    int32_t lo;  // (T - hi) / 2^(e_hi - 53), |lo| <= 2^29; the bits of x for an exotic term
};

constexpr uint32_t NC_TERM_EXOTIC = 0x7FC0DEADu;  // a quiet NaN
constexpr uint32_t NC_FEXP = 0x7F800000u;

NC_FOLD_HD uint32_t nc_fbits(float f)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}

NC_FOLD_HD float nc_ffrom(uint32_t u)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}

NC_FOLD_HD uint64_t nc_dbits(double d)
{
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(d);
#else
    uint64_t u;
    memcpy(&u, &d, 8);
    return u;
#endif
}

NC_FOLD_HD double nc_dfrom(uint64_t u)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double d;
    memcpy(&d, &u, 8);
    return d;
#endif
}

// Splits the term T = fl(fl(x*0.9943)*exp(0.3702*dt)) (x = deltaT*AP_depolFac, float).
NC_FOLD_HD NcSplitTerm nc_split_term(double T, float x)
{
    const uint64_t u = nc_dbits(T);
    const uint32_t E = (uint32_t)(u >> 52) & 0x7FFu;
    NcSplitTerm r;
    if ((u << 1) == 0ull) {  // +-0
        r.hi = nc_ffrom((uint32_t)(u >> 32) & 0x80000000u);
        r.lo = 0;
        return r;
    }
    if (E < 1023u - 90u || E >= 1023u + 90u) {  // kept as x, recomputed when folded
        r.hi = nc_ffrom(NC_TERM_EXOTIC);
        r.lo = (int32_t)nc_fbits(x);
        return r;
    }
    // RN24: round the 52-bit fraction at bit 29, half to even (a carry may bump E)
    const uint64_t v = (u + 0x0FFFFFFFull + ((u >> 29) & 1ull)) & ~0x1FFFFFFFull;
    const uint32_t Ev = (uint32_t)(v >> 52) & 0x7FFu;
    const uint32_t hb =
        ((uint32_t)(v >> 32) & 0x80000000u) | ((Ev - 896u) << 23) | ((uint32_t)(v >> 29) & 0x7FFFFFu);
    const int32_t r29 = (int32_t)(u & 0x1FFFFFFFull);
    const int32_t up = (int32_t)((uint32_t)(v >> 29) - (uint32_t)(u >> 29));  // rounded up: 0 or 1
    // |T| - |hi| in units of 2^(e_T - 52); those are 2^(e_hi - 53) when the rounding
    // carried into the exponent (e_hi = e_T + 1), half of them otherwise
    int32_t tl = r29 - up * 0x20000000;
    if (Ev == E) tl *= 2;
    r.hi = nc_ffrom(hb);
    r.lo = (u >> 63) ? -tl : tl;
    return r;
}

// The exact term again (for the rare path).
NC_FOLD_HD double nc_term_value(NcSplitTerm t, double e_term)
{
    const uint32_t hb = nc_fbits(t.hi);
    if ((hb & NC_FEXP) == NC_FEXP) {
        const double x = (double)nc_ffrom((uint32_t)t.lo);
        return (x * 0.9943) * e_term;
    }
    if (t.lo == 0) return (double)t.hi;
    const int32_t eh = (int32_t)((hb >> 23) & 0xFFu) - 127;
    const double unit = nc_dfrom((uint64_t)(eh - 53 + 1023) << 52);
    return (double)t.hi + (double)t.lo * unit;  // both exact: the sum is T
}

// One `p += T` (see the top of this file).  xp: the exponent bits of p or less (the
// exponent of the previous sum); rare: set when this add is outside the proven range.
NC_FOLD_HD float nc_add_term(float p, uint32_t& xp, NcSplitTerm t, bool& rare)
{
    const float s = p + t.hi;
    const float z = s - p;
    const float e = t.hi - z;
    const uint32_t fs = nc_fbits(s), fe = nc_fbits(e), ft = nc_fbits(t.hi);
    const uint32_t xs = fs & NC_FEXP, xt = ft & NC_FEXP;
    const uint32_t d = xs - xt;  // (e_s - e_hi) << 23
    const uint32_t ae = fe & 0x7FFFFFFFu;
    // a zero term leaves p as it is (s = p, e = 0); otherwise e_hi <= e_p and (a), (b)
    const bool ok = xt == 0u || (xt <= xp && d - (1u << 23) <= (26u << 23));
    rare |= !ok || ((fs & 0x7FFFFFu) == 0u && ae != 0u);
    const bool tie = ae == xs - (24u << 23);
    const uint32_t k = d >> 23;
    const uint32_t mag = (uint32_t)(t.lo < 0 ? -t.lo : t.lo);
    const bool past = k < 30u && mag > (1u << k);
    const bool toward = (((uint32_t)t.lo ^ fe) >> 31) == 0u;
    xp = xs;
    return (tie && past && toward) ? s + (e + e) : s;
}

// The same add with the hardware's double arithmetic (the reference's expression).
NC_FOLD_HD float nc_add_term_exact(float p, NcSplitTerm t, double e_term)
{
    return (float)((double)p + nc_term_value(t, e_term));
}

// nc_device.cuh — device helpers shared by the step kernels: the reference's
// plasticity and trace arithmetic, the ordered `float += double` fold, the input draws
// and bit iteration.
#pragma once
#include "nc_engine.cuh"

namespace nc_dev {

constexpr unsigned kFull = 0xffffffffu;

static __device__ __forceinline__ float trace_at(const float* tab, int len, int32_t now, int32_t then)
{
    if (then == NC_NEVER) return 0.0f;  // lastSpikeArrival = -inf / lastFire = NaN
    const int32_t k = now - then;
    return k < len ? __ldg(tab + k) : 0.0f;
}

static __device__ __forceinline__ bool inh_bit(const NcPools& P, int64_t s)
{
    return (__ldg(P.inh + (s >> 5)) >> (s & 31)) & 1u;
}

// The 32 inhibitory bits of synapses s .. s+31 (s need not be word-aligned; the pool
// keeps one spare word at its end).
static __device__ __forceinline__ uint32_t inh_bits32(const NcPools& P, int64_t s)
{
    const int64_t w0 = s >> 5;
    return __funnelshift_r(__ldg(P.inh + w0), __ldg(P.inh + w0 + 1), (uint32_t)(s & 31));
}

// The learning constants a kernel holds in registers (read from the descriptor once:
// the descriptor lives in global memory, where every store could alias it).
struct Rates {
    float pre, post, lr;
};
static __device__ __forceinline__ Rates rates_of(const NcNetDesc& D) { return Rates{D.pre_factor, D.post_factor, D.lr}; }

// Synapse::synapticPlasticity weight update and clamp (src/NeuCor.cpp:757-761);
// fmin/fmax keep the C library's generic semantics.
static __device__ __forceinline__ float plasticity(float w, bool inh, float traceS, float traceT, const Rates& R)
{
    const float weightChange = R.pre * traceS - R.post * traceT;
    float v = w + weightChange * R.lr;
    if (!inh) {
        const float m = (v <= 1.0f) ? v : 1.0f;
        v = (m >= 0.0f) ? m : 0.0f;
    } else {
        const float m = (v <= 0.0f) ? v : 0.0f;
        v = (m >= -1.0f) ? m : -1.0f;
    }
    return v;
}

// The same update with the clamp bounds of the synapse's sign given: hi = 1, lo = 0 for an
// excitatory synapse, hi = 0, lo = -1 for an inhibitory one (the same compares and
// selects as above, with the bounds chosen once per synapse).
static __device__ __forceinline__ float plasticity_b(float w, float lo, float hi, float traceS, float traceT,
                                                     const Rates& R)
{
    const float weightChange = R.pre * traceS - R.post * traceT;
    const float v = w + weightChange * R.lr;
    const float m = (v <= hi) ? v : hi;
    return (m >= lo) ? m : lo;
}

// trace_at with one unsigned compare: a step counter `then` of NC_NEVER (INT32_MIN) puts
// now - then at 2^31 or above, past any table.
static __device__ __forceinline__ float trace_at_u(const float* tab, int len, int32_t now, int32_t then)
{
    const uint32_t k = (uint32_t)now - (uint32_t)then;
    return k < (uint32_t)len ? __ldg(tab + k) : 0.0f;
}

static __device__ __forceinline__ float plasticity(float w, bool inh, float traceS, float traceT, const NcNetDesc& D)
{
    return plasticity(w, inh, traceS, traceT, rates_of(D));
}

// The charge_insynapses term of a launch, deltaT*AP_depolFac*0.9943*exp(0.3702*deltaT)
// (src/NeuCor.cpp:695) for x = deltaT*AP_depolFac.
static __device__ __forceinline__ double make_term(float x, double e_term)
{
    return __dmul_rn(__dmul_rn((double)x, 0.9943), e_term);
}

// RN32 of a double, returned as the (exactly representable) double: the 52-bit
// fraction is rounded to 23 bits, half to even, with integer operations, so the one
// double add of `float += double` (src/NeuCor.cpp:695) stays the only FP64 instruction
// of a fold.  `rare` is set for the magnitudes the integer path does not cover —
// nonzero values below the float normal range, values from 2^127 up, infinities and
// NaN — and the caller then redoes its batch with the hardware conversion.
static __device__ __forceinline__ double rn32_int(double d, bool& rare)
{
    unsigned long long u = (unsigned long long)__double_as_longlong(d);
    const unsigned e = (unsigned)(u >> 52) & 0x7ffu;
    rare |= (e - 897u > 1149u - 897u) && (u << 1) != 0ull;
    u += 0x0FFFFFFFull + ((u >> 29) & 1ull);
    u &= ~0x1FFFFFFFull;
    return __longlong_as_double((long long)u);
}

// Exact `float += double` of the terms tp[b_k] (b_k >= 0, in k order) with the
// hardware conversion.  Kept out of line so that the rare redo below is a branch and
// its conversions are not issued with every batch.
static __device__ __noinline__ double fold_exact8(double pd, const double* tp, int b0, int b1, int b2, int b3, int b4,
                                                  int b5, int b6, int b7)
{
    const int b[8] = {b0, b1, b2, b3, b4, b5, b6, b7};
#pragma unroll
    for (int k = 0; k < 8; ++k)
        if (b[k] >= 0) pd = (double)__double2float_rn(__dadd_rn(pd, tp[b[k]]));
    return pd;
}

// Whether a neuron out of its AP with potential `pot` (its sum so far) fires:
// charge_passive and the threshold test of charge_thresholdCheck (src/NeuCor.cpp:677-686),
// with the step kernels' own operations.  When no term of the net can be negative the sum
// only grows (rounding keeps the order) and so does this result, so a fold may stop once
// it holds: the neuron fires whatever the remaining terms are, and its potential is then
// replaced by the AP table (src/NeuCor.cpp:706-714).
#ifndef NC_FOLD_EARLY_EXIT
#define NC_FOLD_EARLY_EXIT 1
#endif
static __device__ __forceinline__ bool fires_at(float pot, float leak)
{
    return -55.0f < (pot - -70.0f) * leak + -70.0f;
}

// Folds v[k] = tp[b[k]] for every k with b[k] >= 0 (ascending) into pd, the float
// accumulator held as a double: `potential += term`, one double add and an integer
// rounding to float per term.  (A fold on float arithmetic alone — the term split into
// its float rounding and an integer tail, Fast2Sum and a tie test — is exact too, but
// measured slower on this GPU: a warp's double add costs the issue of about 55 integer
// instructions here, and the float path's fallback near a potential's zero crossing
// costs more.)
static __device__ __forceinline__ double fold8(double pd, const double v[8], const int b[8], const double* tp)
{
    const double pd0 = pd;
    bool rare = false;
#pragma unroll
    for (int k = 0; k < 8; ++k)
        if (b[k] >= 0) pd = rn32_int(__dadd_rn(pd, v[k]), rare);
    if (__builtin_expect(rare, 0)) pd = fold_exact8(pd0, tp, b[0], b[1], b[2], b[3], b[4], b[5], b[6], b[7]);
    return pd;
}

static __device__ __forceinline__ void philox(uint32_t a, uint32_t b, uint32_t stream, uint32_t c, const NcNetDesc& D,
                                       uint32_t out[4])
{
    nc_philox(a, b, stream, c, D.key0, D.key1, out);
}

#ifndef NC_GROUP_RANGE
#define NC_GROUP_RANGE 1
#endif
// Whether input neuron j requests a fire at step t (Poisson groups).
static __device__ bool input_request(const NcPools& P, const NcNetDesc& D, int32_t j, int32_t t)
{
    // most neurons are in no group: one range test instead of a walk over the groups
    if (NC_GROUP_RANGE && (j < D.group_lo || j >= D.group_hi)) return false;
    uint32_t o[4];
    for (int g = 0; g < D.n_groups; ++g) {
        const NcGroupDev G = P.groups[D.group_base + g];
        if (j < G.first || j >= G.first + G.count) continue;
        const uint32_t m = (uint32_t)(j - G.first);
        if (!G.correlated) {
            philox((uint32_t)G.index, (uint32_t)t, NC_STREAM_INDEPENDENT, m, D, o);
            if (o[0] < G.thresh) return true;
            continue;
        }
        for (int32_t src = t - G.jitter; src <= t + G.jitter; ++src) {
            if (src < 0) continue;
            philox((uint32_t)G.index, (uint32_t)src, NC_STREAM_SOURCE, 0u, D, o);
            if (!(o[0] < G.thresh)) continue;
            philox((uint32_t)G.index, (uint32_t)src, NC_STREAM_JITTER, m, D, o);
            const int32_t off = (int32_t)(o[0] % (uint32_t)(2 * G.jitter + 1)) - G.jitter;
            if (src + off == t) return true;
        }
    }
    return false;
}

// Pops up to 8 set bits of *m in ascending order into b[] (-1 when exhausted).
static __device__ __forceinline__ void pop8(uint32_t* m, int b[8])
{
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        b[k] = *m ? __ffs(*m) - 1 : -1;
        *m &= *m - 1u;
    }
}

static __device__ __forceinline__ void pop8_64(unsigned long long* m, int b[8])
{
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        b[k] = *m ? __ffsll((long long)*m) - 1 : -1;
        *m &= *m - 1ull;
    }
}

}  // namespace nc_dev

// Checks the FP64-free `float += double` of nc_fold.h against the expression it replaces,
// (float)((double)p + T), on the host: the split terms must reconstruct exactly, and the
// fast add (with its rare cases redone exactly) must give the same bits on
//   - constructed ties: p + hi exactly halfway between two floats, tails around the
//     53-bit rounding threshold and at the split's own limits;
//   - fold sequences of real terms fl(fl(x*0.9943)*exp(0.3702*dt)), x = dt*(10.4f*w);
//   - random bit patterns for p and T, zeros, subnormal and huge terms.
// Prints "cases N mismatches M rare R" and exits 1 on any mismatch.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "nc_fold.h"

namespace {

uint64_t g_state = 0x9E3779B97F4A7C15ull;
uint64_t next_u64()
{
    g_state ^= g_state << 13;
    g_state ^= g_state >> 7;
    g_state ^= g_state << 17;
    return g_state;
}
double unit() { return (double)(next_u64() >> 11) * (1.0 / 9007199254740992.0); }

long g_cases = 0, g_bad = 0, g_rare = 0;

bool same_float(float a, float b)
{
    if (std::isnan(a) || std::isnan(b)) return std::isnan(a) && std::isnan(b);
    return nc_fbits(a) == nc_fbits(b);
}

// One add through the fast path and, when it reports rare, the exact one.
float add_checked(float p, uint32_t& xp, NcSplitTerm t, double e_term, bool* was_rare)
{
    bool rare = false;
    uint32_t x = xp;
    float r = nc_add_term(p, x, t, rare);
    if (rare) {
        r = nc_add_term_exact(p, t, e_term);
        x = nc_fbits(r) & NC_FEXP;
    }
    *was_rare = rare;
    xp = x;
    return r;
}

void check(float p, double T, float x, double e_term, const char* what)
{
    const NcSplitTerm t = nc_split_term(T, x);
    const double back = nc_term_value(t, e_term);
    ++g_cases;
    if (nc_dbits(back) != nc_dbits(T) && !(std::isnan(back) && std::isnan(T))) {
        if (++g_bad <= 10) std::printf("split %s: T %.17g back %.17g\n", what, T, back);
        return;
    }
    const float want = (float)((double)p + T);
    uint32_t xp = nc_fbits(p) & NC_FEXP;
    bool rare = false;
    const float got = add_checked(p, xp, t, e_term, &rare);
    g_rare += rare;
    if (!same_float(got, want)) {
        if (++g_bad <= 10)
            std::printf("add %s: p %.9g (%08x) T %.17g got %08x want %08x\n", what, p, nc_fbits(p), T, nc_fbits(got),
                        nc_fbits(want));
    }
}

float rand_float(float lo, float hi) { return (float)(lo + (hi - lo) * unit()); }

// p + hi exactly at a midpoint of the result's grid, tails around every threshold.
void ties(long n)
{
    for (long i = 0; i < n; ++i) {
        const float p = (next_u64() & 1) ? rand_float(-80.0f, -30.0f) : rand_float(-4.0f, 90.0f);
        const int ep = (int)((nc_fbits(p) >> 23) & 0xFF) - 127;
        const int j = (int)(next_u64() % 28);  // e_p - e_hi
        const double mag = std::ldexp(1.0 + unit(), ep - j);
        const float h0 = (float)((next_u64() & 1) ? mag : -mag);
        const float s0 = p + h0;
        const int es = (int)((nc_fbits(s0) >> 23) & 0xFF) - 127;
        const double half = std::ldexp(1.0, es - 24);
        const double M = (double)s0 + ((next_u64() & 1) ? half : -half);
        const double hd = M - (double)p;  // exact
        const float hi = (float)hd;
        if ((double)hi != hd || hi == 0.0f) continue;
        const int eh = (int)((nc_fbits(hi) >> 23) & 0xFF) - 127;
        if (eh > ep) continue;
        const int k = es - eh;
        const int64_t cand[] = {0,
                                1,
                                -1,
                                k >= 0 && k < 30 ? (int64_t)1 << k : 3,
                                k >= 0 && k < 30 ? -((int64_t)1 << k) : -3,
                                k >= 0 && k < 29 ? ((int64_t)1 << k) + 1 : 5,
                                k >= 0 && k < 29 ? -((int64_t)1 << k) - 1 : -5,
                                k >= 1 && k < 30 ? ((int64_t)1 << k) - 1 : 7,
                                (int64_t)1 << 29,
                                -((int64_t)1 << 29),
                                ((int64_t)1 << 29) - 1,
                                (int64_t)(next_u64() % (1u << 30)) - (1 << 29)};
        for (int64_t c : cand) {
            const double T = (double)hi + (double)c * std::ldexp(1.0, eh - 53);
            check(p, T, 1.0f, 1.0, "tie");
        }
    }
}

// Folds like charge_insynapses: a potential and a run of real terms.
void folds(long n)
{
    const float dts[] = {0.02f, 0.1f, 0.25f, 0.5f, 1.0f, 2.0f};
    for (long i = 0; i < n; ++i) {
        const float dt = dts[next_u64() % 6];
        const double e_term = std::exp(0.3702 * (double)dt);
        float p = rand_float(-85.0f, 45.0f);
        float q = p;
        uint32_t xp = nc_fbits(p) & NC_FEXP;
        const int len = 1 + (int)(next_u64() % 64);
        for (int k = 0; k < len; ++k) {
            float w = rand_float(-1.0f, 1.0f);
            const unsigned pick = (unsigned)(next_u64() % 16);
            if (pick == 0) w = 0.0f;
            if (pick == 1) w = std::ldexp(w, -(int)(next_u64() % 140));  // down to subnormal weights
            const float x = dt * (0.2f * 52.0f * w);
            const double T = ((double)x * 0.9943) * e_term;
            const NcSplitTerm t = nc_split_term(T, x);
            ++g_cases;
            const double back = nc_term_value(t, e_term);
            if (nc_dbits(back) != nc_dbits(T)) {
                if (++g_bad <= 10) std::printf("split fold: T %.17g back %.17g\n", T, back);
            }
            bool rare = false;
            p = add_checked(p, xp, t, e_term, &rare);
            g_rare += rare;
            q = (float)((double)q + T);
            if (!same_float(p, q)) {
                if (++g_bad <= 10) std::printf("fold: step %d got %08x want %08x\n", k, nc_fbits(p), nc_fbits(q));
                break;
            }
        }
    }
}

void patterns(long n)
{
    for (long i = 0; i < n; ++i) {
        uint32_t pb = (uint32_t)next_u64();
        if ((pb & NC_FEXP) == NC_FEXP) pb &= ~0x00800000u;  // finite p
        uint64_t tb = next_u64();
        // T within a few octaves of p most of the time, anywhere otherwise
        const unsigned pick = (unsigned)(next_u64() % 4);
        if (pick < 3) {
            const int ep = (int)((pb >> 23) & 0xFF) - 127;
            const int et = ep - (int)(next_u64() % 40) + 8;
            if (et > -1000 && et < 1000) tb = (tb & 0x800FFFFFFFFFFFFFull) | ((uint64_t)(et + 1023) << 52);
        }
        const double T = nc_dfrom(tb);
        if (std::isnan(T) || std::isinf(T)) continue;
        const uint32_t E = (uint32_t)(tb >> 52) & 0x7FF;
        if (E < 1023u - 90u || E >= 1023u + 90u) continue;  // exotic terms come from an x (folds above)
        check(nc_ffrom(pb), T, 1.0f, 1.0, "pattern");
    }
    const float ps[] = {0.0f, -0.0f, 1e-40f, -1e-42f, 3.4e38f, -70.0f, 1.0f, 65.5f};
    const double ts[] = {0.0, -0.0, 1e-25, -2.5e-27, 1e27, 0.5, -0.5, 70.0, -70.0, 65.5, -65.5, 3.0e-8};
    for (float p : ps)
        for (double T : ts) check(p, T, 1.0f, 1.0, "edge");
}

}  // namespace

int main(int argc, char** argv)
{
    const long scale = argc > 1 ? std::atol(argv[1]) : 1;
    ties(200000 * scale);
    const long r0 = g_rare, c0 = g_cases;
    folds(100000 * scale);
    const long r1 = g_rare - r0, c1 = g_cases - c0;
    patterns(2000000 * scale);
    std::printf("cases %ld mismatches %ld rare %ld (folds: %ld of %ld)\n", g_cases, g_bad, g_rare, r1, c1);
    return g_bad ? 1 : 0;
}

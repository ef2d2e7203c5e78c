// nc_host.cpp — host-side construction: synapse table layout, reference-arithmetic
// tables, and the network builders.  Compiled with -ffp-contract=off: every float
// expression here mirrors a reference expression and must round the same way.
#include "nc_host.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <thread>

namespace nc {

float step_ms(int64_t k, float dt) { return (float)k * dt; }

float get_dist(const float* a, const float* b)
{
    // sqrtf(powf(x-c.x,2)+powf(y-c.y,2)+powf(z-c.z,2)); GCC folds powf(v,2) to v*v
    const float dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    return sqrtf(dx * dx + dy * dy + dz * dz);
}

int32_t delay_steps(float length, float dt)
{
    // AP_fireTime = length*AP_speed (AP_speed = 2.0, src/NeuCor.cpp:485,733), in
    // whole steps rounded to nearest, at least one step
    const float ms = length * 2.0f;
    const float q = floorf(ms / dt + 0.5f);
    if (!(q >= 1.0f)) return 1;
    if (q > 32767.0f) return -1;
    return (int32_t)q;
}

uint32_t rate_threshold(float rate_hz, float dt)
{
    const double prob = (double)rate_hz * (double)dt / 1000.0;
    if (!(prob > 0.0)) return 0u;
    const double v = prob * 4294967296.0;
    if (v >= 4294967295.0) return 4294967295u;
    return (uint32_t)v;
}

float ap_value(float x)
{
    // Neuron::AP with x = (float)currentT - lastFire; member values from the Neuron
    // constructor (src/NeuCor.cpp:376-385)
    const float AP_h = 100.0f, AP_depolW = 0.3f, AP_polW = 0.6f, AP_deltaPol = 1.16f;
    const float AP_depolFac = 0.2f, AP_deltaStart = 1.0f, baselevel = -70.0f, threshold = -55.0f;
    const float a = x - AP_deltaStart;
    const float b = x - AP_deltaStart - AP_deltaPol;
    const double v = AP_h * (exp(-(a * a) / (2.0 * AP_depolW * AP_depolW)) -
                             exp(-(b * b) / (2.0 * AP_polW * AP_polW)) * AP_depolFac) +
                     baselevel + (threshold - baselevel) * fmax(1.0 - (double)x, 0.0);
    return (float)v;
}

// Morton code of a position quantised to 10 bits per axis over the bounding box.
static uint32_t morton3(uint32_t x, uint32_t y, uint32_t z)
{
    auto spread = [](uint32_t v) {
        v &= 0x3ffu;
        v = (v | (v << 16)) & 0x30000ffu;
        v = (v | (v << 8)) & 0x300f00fu;
        v = (v | (v << 4)) & 0x30c30c3u;
        v = (v | (v << 2)) & 0x9249249u;
        return v;
    };
    return spread(x) | (spread(y) << 1) | (spread(z) << 2);
}

static void storage_order(NetHost& h, const float* xyz, int32_t order_kind)
{
    const int32_t n = h.n;
    h.orig_id.resize((size_t)n);
    h.slot_of.resize((size_t)n);
    for (int32_t i = 0; i < n; ++i) h.orig_id[(size_t)i] = i;
    if (order_kind == NC_ORDER_SPATIAL && xyz && n > 1) {
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        for (int32_t i = 0; i < n; ++i)
            for (int a = 0; a < 3; ++a) {
                const double v = xyz[3 * (size_t)i + a];
                if (std::isfinite(v)) {
                    lo[a] = std::min(lo[a], v);
                    hi[a] = std::max(hi[a], v);
                }
            }
        std::vector<uint32_t> code((size_t)n);
        for (int32_t i = 0; i < n; ++i) {
            uint32_t q[3];
            for (int a = 0; a < 3; ++a) {
                const double v = xyz[3 * (size_t)i + a];
                const double span = hi[a] - lo[a];
                double f = (std::isfinite(v) && span > 0) ? (v - lo[a]) / span : 0.0;
                f = std::min(1.0, std::max(0.0, f));
                q[a] = (uint32_t)(f * 1023.0);
            }
            code[(size_t)i] = morton3(q[0], q[1], q[2]);
        }
        std::stable_sort(h.orig_id.begin(), h.orig_id.end(),
                         [&](int32_t a, int32_t b) { return code[(size_t)a] < code[(size_t)b]; });
    }
    h.permuted = false;
    for (int32_t s = 0; s < n; ++s) {
        h.slot_of[(size_t)h.orig_id[(size_t)s]] = s;
        if (h.orig_id[(size_t)s] != s) h.permuted = true;
    }
}

int64_t NetHost::device_bytes() const
{
    const int64_t per_neuron = 4 + 4 + 4 + 4 + 8 + 8 + 4;             // pot lf firings act_start in_ptr out_ptr ring_off
    const bool dense = p.step_mode != NC_STEP_EVENT, event = p.step_mode != NC_STEP_DENSE;
    // w t_arr term | csc_pre csc_post csc_dl la_c (dense) and/or out_post out_csc delay ringpos last_arr (event)
    const int64_t per_syn = 4 + 4 + 8 + (dense ? 4 + 4 + 2 + 4 : 0) + (event ? 4 + 4 + 2 + 4 + 4 : 0);
    const int64_t words = ((int64_t)n + 31) / 32;
    const int64_t ring_bytes = event ? 4 * (int64_t)ring_slots * ring_words : 0;
    return per_neuron * (n + 1) + per_syn * s + ring_bytes + 4 * 4 * words +
           8 * 2 * (int64_t)n + 4 * (int64_t)tables.size() + (int64_t)sizeof(NcGroupDev) * (int64_t)groups.size();
}

// Trace table powf(decay, k*dt) for k = 0.. until it underflows to zero, with the
// reference's "a trace of exactly 1 counts as 0" rule (src/NeuCor.cpp:744-745).
static bool trace_table(float decay, float dt, std::vector<float>& out, int32_t& len)
{
    const int64_t cap = 1 << 22;
    len = 0;
    for (int64_t k = 0; k < cap; ++k) {
        const float raw = powf(decay, step_ms(k, dt));
        if (raw == 0.0f) {
            len = (int32_t)k;
            return true;
        }
        out.push_back(raw == 1.0f ? 0.0f : raw);
    }
    return false;
}

bool inhibitory_flag(const NetHost& h, int64_t c) { return (h.inh_bits[(size_t)(c >> 5)] >> (c & 31)) & 1u; }

// Whether the m-th synapse appended to an outSynapses vector that ends with `size`
// elements was copied by a reallocation: reserve(5) (src/NeuCor.cpp:374), then
// libstdc++ doubles the capacity of a full vector.
static bool grown_copy(int64_t m, int64_t size)
{
    int64_t cap = 5;
    while (cap <= m) cap *= 2;
    return size > cap;
}

KnnGrid knn_grid(int32_t n, int32_t k, float density)
{
    KnnGrid G;
    G.side = (float)std::cbrt((double)n / (double)density);
    // uniform grid, cells of about k/8 points
    const double cell_target = std::cbrt(std::max(1.0, (double)k / 8.0) / (double)density);
    G.g = std::max(1, (int32_t)std::floor((double)G.side / cell_target));
    G.g = std::min(G.g, 1024);
    G.h = G.side / (float)G.g;
    return G;
}

int build_net(int32_t n, const float* xyz, int64_t n_syn, const int32_t* from, const int32_t* to,
              const float* weight, const float* length, const uint8_t* inhibitory, const nc_params& p,
              NetHost& h, std::string& err)
{
    if (p.inhibitory_rule != NC_INHIBITORY_COPY_LOSS && p.inhibitory_rule != NC_INHIBITORY_SIGN) {
        err = "unknown inhibitory rule";
        return NC_ERR_INVALID;
    }
    if (n < 0 || n_syn < 0) { err = "negative size"; return NC_ERR_INVALID; }
    if (n >= (1 << 30)) { err = "too many neurons"; return NC_ERR_INVALID; }
    if (n_syn > 0 && (!from || !to || !weight)) { err = "null synapse array"; return NC_ERR_INVALID; }
    if (n_syn > 0 && !length && !xyz) { err = "need synapse lengths or neuron positions"; return NC_ERR_INVALID; }
    if (!(p.run_speed > 0.0f) || !std::isfinite(p.run_speed)) { err = "run_speed must be > 0"; return NC_ERR_INVALID; }
    if (!(p.presynaptic_trace_decay > 0.0f && p.presynaptic_trace_decay < 1.0f) ||
        !(p.postsynaptic_trace_decay > 0.0f && p.postsynaptic_trace_decay < 1.0f)) {
        err = "trace decays must lie in (0, 1)";
        return NC_ERR_INVALID;
    }
    for (int64_t k = 0; k < n_syn; ++k) {
        if (from[k] < 0 || from[k] >= n || to[k] < 0 || to[k] >= n) { err = "synapse endpoint out of range"; return NC_ERR_INVALID; }
        if (std::isnan(weight[k])) { err = "NaN weight"; return NC_ERR_INVALID; }
    }

    h = NetHost();
    h.n = n;
    h.n_input = n_syn;
    h.p = p;
    h.dt = p.run_speed;
    h.kc = 1;
    while (!(2.0f < step_ms(h.kc, h.dt))) h.kc++;
    {
        const int period = (int)(600.0f / h.dt);  // std::max(1, static_cast<int>(600.0f / runSpeed))
        h.bg_period = p.background_firing ? std::max(1, period) : 0;
    }
    h.leak = powf(0.5f, h.dt);                          // powf(recharge, deltaT)
    h.c52 = (float)((double)0.2f * 52.0);               // AP_depolFac = 0.2f; AP_depolFac *= 52.0
    h.e_term = exp(0.3702 * (double)h.dt);              // exp(0.3702*deltaT)
    h.xyz.assign(3 * (size_t)n, 0.0f);
    if (xyz) std::memcpy(h.xyz.data(), xyz, sizeof(float) * 3 * (size_t)n);
    if (p.storage_order != NC_ORDER_SPATIAL && p.storage_order != NC_ORDER_ID) {
        err = "unknown storage order";
        return NC_ERR_INVALID;
    }
    if (p.step_mode != NC_STEP_DENSE && p.step_mode != NC_STEP_EVENT && p.step_mode != NC_STEP_AUTO) {
        err = "unknown step mode";
        return NC_ERR_INVALID;
    }
    storage_order(h, xyz, p.storage_order);

    // CSC: bucket by target slot in input order, sort each bucket by the caller's source
    // id (stable), keep the first of repeated (source, target) pairs (createSynapse,
    // src/NeuCor.cpp:189-191)
    std::vector<int64_t> bstart((size_t)n + 1, 0);
    for (int64_t k = 0; k < n_syn; ++k) bstart[(size_t)h.slot_of[(size_t)to[k]] + 1]++;
    for (int32_t j = 0; j < n; ++j) bstart[j + 1] += bstart[j];
    std::vector<int64_t> order((size_t)n_syn);
    {
        std::vector<int64_t> fill(bstart.begin(), bstart.end() - 1);
        for (int64_t k = 0; k < n_syn; ++k) order[(size_t)fill[h.slot_of[(size_t)to[k]]]++] = k;
    }
    h.input_to_csc.assign((size_t)n_syn, -1);
    h.in_ptr.assign((size_t)n + 1, 0);
    h.csc_pre.reserve((size_t)n_syn);
    h.csc_delay.reserve((size_t)n_syn);
    h.w.reserve((size_t)n_syn);
    std::vector<int64_t> csc_input;
    csc_input.reserve((size_t)n_syn);
    for (int32_t j = 0; j < n; ++j) {
        auto b = order.begin() + bstart[j], e = order.begin() + bstart[j + 1];
        std::stable_sort(b, e, [&](int64_t x, int64_t y) { return from[x] < from[y]; });
        int32_t last_pre = -1;
        for (auto it = b; it != e; ++it) {
            const int64_t k = *it;
            if (from[k] == last_pre) continue;
            last_pre = from[k];
            const int64_t c = (int64_t)h.csc_pre.size();
            h.input_to_csc[(size_t)k] = c;
            csc_input.push_back(k);
            h.csc_pre.push_back(h.slot_of[(size_t)from[k]]);
            const float len = length ? length[k] : get_dist(&h.xyz[3 * (size_t)from[k]], &h.xyz[3 * (size_t)to[k]]);
            const int32_t d = delay_steps(len, h.dt);
            if (d < 0 || d > kMaxDelay) { err = "synapse delay exceeds 16383 steps"; return NC_ERR_INVALID; }
            h.csc_delay.push_back(d);
            h.max_delay = std::max(h.max_delay, d);
            h.w.push_back(weight[k]);
        }
        h.in_ptr[j + 1] = (int64_t)h.csc_pre.size();
    }
    h.s = (int64_t)h.csc_pre.size();

    // ring words per target: one bit per in-synapse
    h.ring_off.assign((size_t)n + 1, 0);
    for (int32_t j = 0; j < n; ++j) {
        const int64_t fan = h.in_ptr[j + 1] - h.in_ptr[j];
        const int64_t words = (fan + 31) / 32;
        if ((int64_t)h.ring_off[j] + words >= (1ll << 27)) { err = "network too large for one ring slot"; return NC_ERR_INVALID; }
        h.ring_off[j + 1] = h.ring_off[j] + (int32_t)words;
    }
    h.ring_words = h.ring_off[n];
    h.ring_slots = 1;
    while (h.ring_slots < h.max_delay + h.kc + 1) h.ring_slots <<= 1;

    // CSR: each source's out-synapses in creation order (Neuron::outSynapses)
    h.out_ptr.assign((size_t)n + 1, 0);
    for (int64_t c = 0; c < h.s; ++c) h.out_ptr[(size_t)h.csc_pre[c] + 1]++;
    for (int32_t i = 0; i < n; ++i) h.out_ptr[i + 1] += h.out_ptr[i];
    h.out_post.assign((size_t)h.s, 0);
    h.out_csc.assign((size_t)h.s, 0);
    h.out_delay.assign((size_t)h.s, 0);
    h.out_ringpos.assign((size_t)h.s, 0);
    h.csc_dl.assign((size_t)h.s, 0);
    {
        std::vector<int64_t> fill(h.out_ptr.begin(), h.out_ptr.end() - 1);
        std::vector<int32_t>& csc_post = h.csc_post;
        csc_post.assign((size_t)h.s, 0);
        for (int32_t j = 0; j < n; ++j)
            for (int64_t c = h.in_ptr[j]; c < h.in_ptr[j + 1]; ++c) csc_post[(size_t)c] = j;
        for (int64_t k = 0; k < n_syn; ++k) {
            const int64_t c = h.input_to_csc[(size_t)k];
            if (c < 0) continue;
            const int32_t i = h.csc_pre[(size_t)c], j = csc_post[(size_t)c];
            const int64_t q = fill[i]++;
            const int64_t b = c - h.in_ptr[j];
            h.out_post[(size_t)q] = j;
            h.out_csc[(size_t)q] = (int32_t)c;
            // the same-step order rules compare the caller's ids of target and source
            const uint32_t flags = (to[k] > from[k] ? 1u << kAfterBit : 0u) | (to[k] < from[k] ? 1u << kBeforeBit : 0u);
            h.out_delay[(size_t)q] = (int16_t)(uint16_t)((uint32_t)h.csc_delay[(size_t)c] | flags);
            h.csc_dl[(size_t)c] = (uint16_t)((uint32_t)h.csc_delay[(size_t)c] | flags);
            h.out_ringpos[(size_t)q] = ((uint32_t)(h.ring_off[j] + (int32_t)(b >> 5)) << 5) | (uint32_t)(b & 31);
        }
    }
    if (h.s >= (1ll << 31)) { err = "too many synapses in one network"; return NC_ERR_INVALID; }

    // Synapse::inhibitory: setWeight's sign (src/NeuCor.cpp:576-579), lost by synapses
    // the vector growth copied (rule COPY_LOSS), or the caller's own flags
    h.inh_bits.assign((size_t)((h.s + 31) / 32), 0u);
    for (int32_t i = 0; i < n; ++i) {
        const int64_t size = h.out_ptr[i + 1] - h.out_ptr[i];
        for (int64_t m = 0; m < size; ++m) {
            const int64_t c = h.out_csc[(size_t)(h.out_ptr[i] + m)];
            bool inh = h.w[(size_t)c] < 0.0f;
            if (p.inhibitory_rule == NC_INHIBITORY_COPY_LOSS && grown_copy(m, size)) inh = false;
            if (inh) h.inh_bits[(size_t)(c >> 5)] |= 1u << (c & 31);
        }
    }
    if (inhibitory) {
        for (int64_t k = 0; k < n_syn; ++k) {
            const int64_t c = h.input_to_csc[(size_t)k];
            if (c < 0) continue;
            if (inhibitory[k]) h.inh_bits[(size_t)(c >> 5)] |= 1u << (c & 31);
            else h.inh_bits[(size_t)(c >> 5)] &= ~(1u << (c & 31));
        }
    }

    // Every term a launch can add is >= 0 when no synapse is inhibitory and no weight is
    // negative: plasticity keeps an excitatory weight in [0, 1] (src/NeuCor.cpp:757-761)
    // and no call changes a weight after creation.
    h.nonneg_terms = true;
    for (uint32_t b : h.inh_bits) h.nonneg_terms = h.nonneg_terms && b == 0u;
    for (float x : h.w) h.nonneg_terms = h.nonneg_terms && x >= 0.0f;

    // tables: presynaptic trace, postsynaptic trace, AP shape
    h.tables.clear();
    if (!trace_table(p.presynaptic_trace_decay, h.dt, h.tables, h.tab_pre_len) ||
        !trace_table(p.postsynaptic_trace_decay, h.dt, h.tables, h.tab_post_len)) {
        err = "trace table does not underflow";
        return NC_ERR_INVALID;
    }
    h.ap_len = h.kc;
    for (int32_t k = 0; k < h.kc; ++k) h.tables.push_back(ap_value(step_ms(k, h.dt)));
    return NC_OK;
}

int set_groups(NetHost& h, int32_t n_groups, const nc_group* groups, std::string& err)
{
    if (n_groups < 0 || (n_groups > 0 && !groups)) { err = "bad group array"; return NC_ERR_INVALID; }
    std::vector<NcGroupDev> out;
    for (int32_t g = 0; g < n_groups; ++g) {
        const nc_group& G = groups[g];
        if (G.first < 0 || G.count < 0 || G.jitter < 0 || G.jitter > 1000 || (int64_t)G.first + G.count > h.n ||
            !(G.rate_hz >= 0.0f)) {
            err = "input group out of range";
            return NC_ERR_INVALID;
        }
        out.push_back(NcGroupDev{G.first, G.count, rate_threshold(G.rate_hz, h.dt), G.correlated ? 1 : 0,
                                 G.jitter, g});
    }
    h.groups = out;
    return NC_OK;
}

}  // namespace nc

// ------------------------------------------------------------------ C ABI
namespace {
thread_local std::string g_build_err;
using nc::kStreamPosition;
using nc::kStreamWeight;
using nc::unit24;

struct Cand {
    float d;
    int32_t j;
    bool operator<(const Cand& o) const { return d < o.d || (d == o.d && j < o.j); }
};
}  // namespace

extern "C" int nc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    if (!ctr || !key || !out) return NC_ERR_INVALID;
    nc_philox(ctr[0], ctr[1], ctr[2], ctr[3], key[0], key[1], out);
    return NC_OK;
}

extern "C" int nc_build_knn(int32_t n, int32_t k, float density, uint64_t seed, float* xyz, int32_t* syn_from,
                            int32_t* syn_to, float* syn_weight)
{
    if (n < 0 || k < 0 || !(density > 0.0f) || !xyz || ((int64_t)n * k > 0 && (!syn_from || !syn_to || !syn_weight)))
        return NC_ERR_INVALID;
    if (n > 0 && k >= n) return NC_ERR_INVALID;
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    const nc::KnnGrid grid = nc::knn_grid(n, k, density);
    const float side = grid.side;
    for (int32_t i = 0; i < n; ++i) {
        uint32_t o[4];
        nc_philox((uint32_t)i, 0u, kStreamPosition, 0u, k0, k1, o);
        xyz[3 * (size_t)i + 0] = unit24(o[0]) * side;
        xyz[3 * (size_t)i + 1] = unit24(o[1]) * side;
        xyz[3 * (size_t)i + 2] = unit24(o[2]) * side;
    }
    if (k == 0 || n == 0) return NC_OK;
    const int32_t g = grid.g;
    const float h = grid.h;
    auto cell_of = [&](float v) { return std::min(g - 1, std::max(0, (int32_t)(v / h))); };
    std::vector<int32_t> cstart((size_t)g * g * g + 1, 0), cell((size_t)n);
    for (int32_t i = 0; i < n; ++i) {
        const int32_t c = (cell_of(xyz[3 * (size_t)i]) * g + cell_of(xyz[3 * (size_t)i + 1])) * g +
                          cell_of(xyz[3 * (size_t)i + 2]);
        cell[i] = c;
        cstart[(size_t)c + 1]++;
    }
    for (size_t c = 0; c + 1 < cstart.size(); ++c) cstart[c + 1] += cstart[c];
    std::vector<int32_t> members((size_t)n);
    {
        std::vector<int32_t> fill(cstart.begin(), cstart.end() - 1);
        for (int32_t i = 0; i < n; ++i) members[(size_t)fill[cell[i]]++] = i;
    }
    auto worker = [&](int32_t lo, int32_t hi) {
        std::vector<Cand> cand;
        for (int32_t i = lo; i < hi; ++i) {
            const float* pi = &xyz[3 * (size_t)i];
            const int32_t cx = cell_of(pi[0]), cy = cell_of(pi[1]), cz = cell_of(pi[2]);
            cand.clear();
            for (int32_t r = 0;; ++r) {
                for (int32_t x = cx - r; x <= cx + r; ++x) {
                    if (x < 0 || x >= g) continue;
                    for (int32_t y = cy - r; y <= cy + r; ++y) {
                        if (y < 0 || y >= g) continue;
                        for (int32_t z = cz - r; z <= cz + r; ++z) {
                            if (z < 0 || z >= g) continue;
                            if (std::max(std::abs(x - cx), std::max(std::abs(y - cy), std::abs(z - cz))) != r) continue;
                            const int32_t c = (x * g + y) * g + z;
                            for (int32_t q = cstart[c]; q < cstart[(size_t)c + 1]; ++q) {
                                const int32_t j = members[(size_t)q];
                                if (j == i) continue;
                                cand.push_back(Cand{nc::get_dist(pi, &xyz[3 * (size_t)j]), j});
                            }
                        }
                    }
                }
                const bool all = r >= g;
                if ((int32_t)cand.size() >= k) {
                    // every unvisited point is at least r*h away
                    std::nth_element(cand.begin(), cand.begin() + (k - 1), cand.end());
                    if (all || cand[(size_t)k - 1].d < (float)r * h) break;
                } else if (all) {
                    break;
                }
            }
            std::partial_sort(cand.begin(), cand.begin() + k, cand.end());
            for (int32_t m = 0; m < k; ++m) {
                const size_t q = (size_t)i * k + m;
                syn_from[q] = i;
                syn_to[q] = cand[(size_t)m].j;
                uint32_t o[4];
                nc_philox((uint32_t)i, (uint32_t)(m >> 2), kStreamWeight, 0u, k0, k1, o);
                syn_weight[q] = unit24(o[m & 3]);
            }
        }
    };
    const int32_t threads = (int32_t)std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    std::vector<std::thread> pool;
    const int32_t chunk = (n + threads - 1) / threads;
    for (int32_t tb = 0; tb < threads; ++tb) {
        const int32_t lo = tb * chunk, hi = std::min(n, lo + chunk);
        if (lo >= hi) break;
        pool.emplace_back(worker, lo, hi);
    }
    for (auto& th : pool) th.join();
    return NC_OK;
}

namespace {
float randomUnit() { return static_cast<float>(rand()) / static_cast<float>(RAND_MAX); }
}  // namespace

extern "C" int nc_reference_positions(int32_t n, float* xyz)
{
    if (n < 0 || (n > 0 && !xyz)) return NC_ERR_INVALID;
    // createNeuron with NaN positions while totalGenNeurons = n (src/NeuCor.cpp:154-170)
    float spawnSize = 2.0f;
    if (n != 0) spawnSize = powf((float)((unsigned)n / (1.3333 * 3.1459 * 8)), (float)0.33333) * 2.0;
    for (int32_t i = 0; i < n; ++i) {
        float x, y, z;
        do {
            x = (randomUnit() - 0.5f) * spawnSize;
            y = (randomUnit() - 0.5f) * spawnSize;
            z = (randomUnit() - 0.5f) * spawnSize;
        } while ((double)x * x + (double)y * y + (double)z * z > (spawnSize / 2.0) * (spawnSize / 2.0));
        xyz[3 * (size_t)i] = x;
        xyz[3 * (size_t)i + 1] = y;
        xyz[3 * (size_t)i + 2] = z;
    }
    return NC_OK;
}

extern "C" int nc_reference_connection_count(int32_t n, const float* xyz, int64_t* n_synapses)
{
    if (n < 0 || !n_synapses || (n > 0 && !xyz)) return NC_ERR_INVALID;
    int64_t s = 0;
    for (int32_t i = 0; i < n; ++i)
        for (int32_t j = 0; j < n; ++j)
            if (nc::get_dist(&xyz[3 * (size_t)i], &xyz[3 * (size_t)j]) < 1.0 && j != i) ++s;
    *n_synapses = s;
    return NC_OK;
}

extern "C" int nc_reference_connections(int32_t n, const float* xyz, int32_t* syn_from, int32_t* syn_to,
                                        float* syn_weight, int64_t capacity)
{
    if (n < 0 || (n > 0 && !xyz)) return NC_ERR_INVALID;
    int64_t s = 0;
    // Neuron::makeConnections for every neuron in order (src/NeuCor.cpp:418-444); each new
    // Synapse draws its weight (src/NeuCor.cpp:471-473)
    for (int32_t i = 0; i < n; ++i) {
        for (int32_t j = 0; j < n; ++j) {
            const float distance = nc::get_dist(&xyz[3 * (size_t)i], &xyz[3 * (size_t)j]);
            if (!(distance < 1.0 && j != i)) continue;
            if (s >= capacity || !syn_from || !syn_to || !syn_weight) return NC_ERR_INVALID;
            float weight = randomUnit() * 0.8f + 0.2f;
            if (randomUnit() < 0.2f) weight = -weight;
            syn_from[s] = i;
            syn_to[s] = j;
            syn_weight[s] = weight;
            ++s;
        }
    }
    return NC_OK;
}

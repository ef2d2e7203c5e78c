// Host-side facts the step kernels rely on, checked without a GPU:
//   NetHost::nonneg_terms  lets the neuron passes stop a fold once the neuron is certain
//                          to fire, so it must be false whenever any term can be negative;
//   nc_group_range         the id range an input request tests before walking the groups.
// Built from neurocorrelation_gb300/csrc/nc_host.cpp by tests/test_host_flags.py.
#include "nc_host.h"

#include <cstdio>
#include <string>
#include <vector>

static nc_params defaults()
{
    nc_params p = {};
    p.run_speed = 1.0f;
    p.learning_rate = 1.0f;
    p.presynaptic_trace_decay = 0.75f;
    p.postsynaptic_trace_decay = 0.65f;
    p.presynaptic_factor = 0.13f;
    p.postsynaptic_factor = 0.30f;
    p.background_firing = 1;
    p.inhibitory_rule = NC_INHIBITORY_COPY_LOSS;
    return p;
}

static int fails = 0;

static void check(bool ok, const char* what)
{
    std::printf("%s %s\n", ok ? "ok  " : "FAIL", what);
    fails += ok ? 0 : 1;
}

// Four neurons on a line; synapses 0->1, 1->2, 2->3, 3->0 plus any extra pairs.
static bool nonneg(std::vector<float> w, const uint8_t* inh = nullptr, int rule = NC_INHIBITORY_COPY_LOSS,
                   std::vector<int32_t> from = {0, 1, 2, 3}, std::vector<int32_t> to = {1, 2, 3, 0})
{
    const float xyz[12] = {0, 0, 0, 1, 0, 0, 2, 0, 0, 3, 0, 0};
    nc_params p = defaults();
    p.inhibitory_rule = rule;
    nc::NetHost h;
    std::string err;
    const int rc = nc::build_net(4, xyz, (int64_t)w.size(), from.data(), to.data(), w.data(), nullptr, inh, p, h,
                                 err);
    if (rc != NC_OK) {
        std::printf("build_net failed: %s\n", err.c_str());
        ++fails;
        return false;
    }
    return h.nonneg_terms;
}

int main()
{
    check(nonneg({0.5f, 0.25f, 1.0f, 0.0f}), "non-negative weights: terms are >= 0");
    check(nonneg({0.5f, -0.0f, 1.0f, 0.0f}), "a negative zero weight adds -0.0, which is >= 0");
    check(!nonneg({0.5f, -0.25f, 1.0f, 0.0f}), "a negative weight");
    check(!nonneg({0.5f, -0.25f, 1.0f, 0.0f}, nullptr, NC_INHIBITORY_SIGN), "a negative weight, sign rule");
    const uint8_t inh[4] = {0, 0, 1, 0};
    check(!nonneg({0.5f, 0.25f, 1.0f, 0.0f}, inh), "an inhibitory flag on a positive weight");
    // a repeated (source, target) pair keeps its first weight: the dropped one does not count
    check(nonneg({0.5f, 0.25f, 1.0f, 0.0f, -0.5f}, nullptr, NC_INHIBITORY_COPY_LOSS, {0, 1, 2, 3, 0},
                 {1, 2, 3, 0, 1}),
          "a negative weight on a dropped repeated pair");
    check(!nonneg({-0.5f, 0.25f, 1.0f, 0.0f, 0.5f}, nullptr, NC_INHIBITORY_COPY_LOSS, {0, 1, 2, 3, 0},
                  {1, 2, 3, 0, 1}),
          "a negative weight on the kept one of a repeated pair");

    const NcGroupDev g[3] = {{10, 5, 0u, 1, 2, 0}, {0, 3, 0u, 0, 0, 1}, {100, 0, 0u, 0, 0, 2}};
    int32_t lo = -1, hi = -1;
    nc_group_range(g, 0, lo, hi);
    check(lo == hi, "no groups: empty range");
    nc_group_range(g, 3, lo, hi);
    check(lo == 0 && hi == 15, "three groups, one empty: [0, 15)");
    nc_group_range(g + 2, 1, lo, hi);
    check(lo == hi, "an empty group alone: empty range");
    nc_group_range(g, 1, lo, hi);
    check(lo == 10 && hi == 15, "one group: [10, 15)");
    std::printf("%s\n", fails ? "FAILED" : "OK");
    return fails != 0;
}

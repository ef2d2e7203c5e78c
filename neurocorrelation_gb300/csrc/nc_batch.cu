// nc_batch.cu — many independent networks in one engine (nc_batch_* in neucor_gb300.h).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "nc_pool.h"

namespace {
int bfail(int code, const std::string& msg) { return nc::set_last_error(code, msg); }
}  // namespace

struct nc_batch {
    std::vector<nc::NetHost> hosts;
    std::vector<int32_t> horizon;
    nc::Engine eng;
    int64_t ticks = 0;  // launch pairs issued
};

#define B_NEED(b)                                                    \
    do {                                                             \
        if (!(b)) return bfail(NC_ERR_INVALID, "null batch");        \
        cudaError_t e_ = cudaSetDevice((b)->eng.device);             \
        if (e_ != cudaSuccess) return bfail(NC_ERR_CUDA, nc::cuda_msg("cudaSetDevice", e_)); \
    } while (0)
#define B_CALL0(obj, method)                                         \
    do {                                                             \
        std::string err_;                                            \
        int rc_ = (obj).method(err_);                                \
        if (rc_ != NC_OK) return bfail(rc_, err_);                   \
    } while (0)
#define B_CALL(obj, method, ...)                                     \
    do {                                                             \
        std::string err_;                                            \
        int rc_ = (obj).method(__VA_ARGS__, err_);                   \
        if (rc_ != NC_OK) return bfail(rc_, err_);                   \
    } while (0)

// per-net step reached: nets advance one step per tick until their horizon
static int64_t net_step(const nc_batch* b, int32_t net)
{
    return std::min<int64_t>(b->ticks, b->horizon[(size_t)net]);
}

extern "C" {

int nc_batch_create(int32_t n_nets, const nc_net_spec* specs, nc_batch** out)
{
    if (!out || n_nets <= 0 || !specs) return bfail(NC_ERR_INVALID, "bad arguments");
    *out = nullptr;
    for (int32_t q = 0; q < n_nets; ++q)
        if (specs[q].params.step_mode == NC_STEP_AUTO)
            return bfail(NC_ERR_UNSUPPORTED, "NC_STEP_AUTO is for single networks; a batch runs in one form");
    int devices = 0;
    if (cudaGetDeviceCount(&devices) != cudaSuccess || devices == 0)
        return bfail(NC_ERR_NODEVICE, "no CUDA device: the GB300 step has no CPU fallback");
    nc_batch* b = new (std::nothrow) nc_batch();
    if (!b) return bfail(NC_ERR_NOMEM, "host allocation failed");
    b->hosts.resize((size_t)n_nets);
    b->horizon.resize((size_t)n_nets);
    std::vector<int> rcs((size_t)n_nets, NC_OK);
    std::vector<std::string> errs((size_t)n_nets);
    std::atomic<int32_t> next{0};
    auto worker = [&]() {
        for (int32_t q = next++; q < n_nets; q = next++) {
            const nc_net_spec& sp = specs[q];
            int rc = nc::build_net(sp.n_neurons, sp.xyz, sp.n_synapses, sp.syn_from, sp.syn_to, sp.syn_weight,
                                   sp.syn_length, sp.syn_inhibitory, sp.params, b->hosts[(size_t)q], errs[(size_t)q]);
            if (rc == NC_OK) rc = nc::set_groups(b->hosts[(size_t)q], sp.n_groups, sp.groups, errs[(size_t)q]);
            if (rc == NC_OK && sp.horizon < 0) {
                rc = NC_ERR_INVALID;
                errs[(size_t)q] = "negative horizon";
            }
            rcs[(size_t)q] = rc;
        }
    };
    const unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    std::vector<std::thread> pool;
    for (unsigned k = 0; k < nt; ++k) pool.emplace_back(worker);
    for (auto& t : pool) t.join();
    int32_t max_groups = 1;
    for (int32_t q = 0; q < n_nets; ++q) {
        if (rcs[(size_t)q] != NC_OK) {
            const std::string m = "network " + std::to_string(q) + ": " + errs[(size_t)q];
            delete b;
            return bfail(rcs[(size_t)q], m);
        }
        b->horizon[(size_t)q] = specs[q].horizon;
        max_groups = std::max<int32_t>(max_groups, (int32_t)b->hosts[(size_t)q].groups.size());
    }
    std::vector<const nc::NetHost*> ptrs;
    for (auto& h : b->hosts) ptrs.push_back(&h);
    std::string err;
    const int rc = b->eng.build(ptrs, max_groups, err, &b->horizon);
    if (rc != NC_OK) {
        delete b;
        return bfail(rc, err);
    }
    for (auto& h : b->hosts) {  // keep what read-back needs
        std::vector<int32_t>().swap(h.out_post);
        std::vector<int32_t>().swap(h.out_csc);
        std::vector<int16_t>().swap(h.out_delay);
        std::vector<uint32_t>().swap(h.out_ringpos);
        std::vector<float>().swap(h.w);
        std::vector<int64_t>().swap(h.in_ptr);
        std::vector<int32_t>().swap(h.ring_off);
        std::vector<int32_t>().swap(h.csc_pre);
        std::vector<uint16_t>().swap(h.csc_dl);
    }
    *out = b;
    return NC_OK;
}

int nc_batch_destroy(nc_batch* b)
{
    if (!b) return NC_OK;
    cudaSetDevice(b->eng.device);
    delete b;
    return NC_OK;
}

int nc_batch_run(nc_batch* b, int32_t steps)
{
    B_NEED(b);
    if (steps < 0) return bfail(NC_ERR_INVALID, "negative steps");
    B_CALL(b->eng, step, (int64_t)steps);
    b->ticks += steps;
    return NC_OK;
}

int nc_batch_time(nc_batch* b, int32_t steps, float* ms)
{
    B_NEED(b);
    if (steps < 0 || !ms) return bfail(NC_ERR_INVALID, "bad arguments");
    B_CALL(b->eng, step_timed, (int64_t)steps, ms);
    b->ticks += steps;
    return NC_OK;
}

int nc_batch_run_to_end(nc_batch* b)
{
    B_NEED(b);
    const int64_t last = *std::max_element(b->horizon.begin(), b->horizon.end());
    if (last > b->ticks) {
        B_CALL(b->eng, step, last - b->ticks);
        b->ticks = last;
    }
    B_CALL0(b->eng, sync);
    return NC_OK;
}

int nc_batch_get_launch(nc_batch* b, nc_launch_config* out)
{
    if (!b || !out) return bfail(NC_ERR_INVALID, "null argument");
    out->neuron_block = b->eng.L.neuron_block;
    out->launch_blocks = b->eng.L.launch_blocks;
    out->launch_block = b->eng.L.launch_block;
    out->graph_steps = b->eng.graph_ticks;
    out->dense_blocks = b->eng.L.dense_blocks;
    out->steps_per_launch = b->eng.L.fused_ticks;
    return NC_OK;
}

int nc_batch_set_launch(nc_batch* b, const nc_launch_config* c)
{
    B_NEED(b);
    // the step kernels are compiled for at most 256 threads per block
    if (!c || c->neuron_block < 32 || c->neuron_block > 256 || c->neuron_block % 32 || c->launch_block < 32 ||
        c->launch_block > 256 || c->launch_block % 32 || c->launch_blocks < 1 || c->launch_blocks > (1 << 20) ||
        c->graph_steps < 0 || c->graph_steps > 4096 || c->dense_blocks < 0 || c->dense_blocks > (1 << 20) ||
        c->steps_per_launch < 0 || c->steps_per_launch > (1 << 20))
        return bfail(NC_ERR_INVALID, "bad launch configuration (blocks of 32..256 threads)");
    B_CALL0(b->eng, sync);
    nc::LaunchShape L{c->neuron_block, c->launch_blocks, c->launch_block, c->dense_blocks, c->steps_per_launch};
    b->eng.set_launch(L, c->graph_steps);
    return NC_OK;
}

int nc_batch_autotune(nc_batch* b, int32_t steps_per_trial, nc_launch_config* best)
{
    B_NEED(b);
    if (steps_per_trial < 1) return bfail(NC_ERR_INVALID, "steps_per_trial must be >= 1");
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->eng.device);
    std::vector<nc_launch_config> cands;
    const nc_launch_config cur = {b->eng.L.neuron_block, b->eng.L.launch_blocks, b->eng.L.launch_block,
                                  b->eng.graph_ticks, b->eng.L.dense_blocks, b->eng.L.fused_ticks};
    if (b->eng.dense) {
        for (int nb : {64, 128, 256})
            for (int dbm : {0, 2})
                for (int g : {16, 64})
                    cands.push_back(nc_launch_config{nb, cur.launch_blocks, cur.launch_block, g, sms * dbm, 0});
        if (b->eng.P.n_firers == 0)
            for (int k : {4, 16, 64})
                cands.push_back(nc_launch_config{128, cur.launch_blocks, cur.launch_block, 16, 0, k});
    } else {
        for (int nb : {64, 128, 256})
            for (int lbm : {2, 4, 8})
                for (int lb : {128, 256})
                    for (int g : {16, 64}) cands.push_back(nc_launch_config{nb, sms * lbm, lb, g, 0, 0});
    }
    float best_ms = 1e30f;
    nc_launch_config chosen = cands[0];
    for (const auto& c : cands) {
        int rc = nc_batch_set_launch(b, &c);
        if (rc != NC_OK) return rc;
        float ms[3] = {0.0f, 0.0f, 0.0f};
        // warm-up trial: captures the graph, sizes the grid
        rc = nc_batch_time(b, std::max<int32_t>(steps_per_trial, c.steps_per_launch), &ms[0]);
        if (rc != NC_OK) return rc;
        for (float& m : ms) {
            rc = nc_batch_time(b, steps_per_trial, &m);
            if (rc != NC_OK) return rc;
        }
        std::sort(ms, ms + 3);
        if (ms[1] < best_ms) {
            best_ms = ms[1];
            chosen = c;
        }
    }
    int rc = nc_batch_set_launch(b, &chosen);
    if (rc != NC_OK) return rc;
    if (best) *best = chosen;
    return NC_OK;
}

int nc_batch_get_stats(nc_batch* b, int32_t net, nc_stats* out)
{
    B_NEED(b);
    if (!out || net < 0 || net >= (int32_t)b->hosts.size()) return bfail(NC_ERR_INVALID, "bad net index");
    unsigned long long s[4];
    B_CALL0(b->eng, flush_plasticity);  // the dense form's last launches
    B_CALL(b->eng, read_stats, net, s);
    out->fires = (int64_t)s[0];
    out->launched = (int64_t)s[1];
    out->dropped = (int64_t)s[2];
    out->steps = (int64_t)s[3];
    return NC_OK;
}

int nc_batch_get_step(nc_batch* b, int32_t net, int64_t* step)
{
    if (!b || !step || net < 0 || net >= (int32_t)b->hosts.size()) return bfail(NC_ERR_INVALID, "bad net index");
    *step = net_step(b, net);
    return NC_OK;
}

int nc_batch_read_potentials(nc_batch* b, int32_t net, float* out)
{
    B_NEED(b);
    if (!out || net < 0 || net >= (int32_t)b->hosts.size()) return bfail(NC_ERR_INVALID, "bad net index");
    const auto& sl = b->eng.slots[(size_t)net];
    std::vector<float> pot((size_t)sl.n);
    B_CALL(b->eng, download, pot.data(), (const float*)b->eng.P.pot + sl.neuron_base, (size_t)sl.n);
    nc::to_caller_order(b->hosts[(size_t)net], pot.data(), out);
    return NC_OK;
}

int nc_batch_read_weights(nc_batch* b, int32_t net, float* out)
{
    B_NEED(b);
    if (net < 0 || net >= (int32_t)b->hosts.size()) return bfail(NC_ERR_INVALID, "bad net index");
    const nc::NetHost& h = b->hosts[(size_t)net];
    if (!out && h.n_input) return bfail(NC_ERR_INVALID, "null output");
    B_CALL0(b->eng, flush_plasticity);
    const auto& sl = b->eng.slots[(size_t)net];
    std::vector<float> w((size_t)h.s);
    B_CALL(b->eng, download, w.data(), (const float*)b->eng.P.w + sl.syn_base, (size_t)h.s);
    for (int64_t k = 0; k < h.n_input; ++k) {
        const int64_t c = h.input_to_csc[(size_t)k];
        out[k] = c < 0 ? NAN : w[(size_t)c];
    }
    return NC_OK;
}

int nc_batch_read_last_fire(nc_batch* b, int32_t net, float* out)
{
    B_NEED(b);
    if (!out || net < 0 || net >= (int32_t)b->hosts.size()) return bfail(NC_ERR_INVALID, "bad net index");
    const auto& sl = b->eng.slots[(size_t)net];
    std::vector<int32_t> lf_s((size_t)sl.n), lf((size_t)sl.n);
    B_CALL(b->eng, download, lf_s.data(), (const int32_t*)b->eng.P.lf + sl.neuron_base, (size_t)sl.n);
    nc::to_caller_order(b->hosts[(size_t)net], lf_s.data(), lf.data());
    for (int32_t j = 0; j < sl.n; ++j) out[j] = lf[(size_t)j] == NC_NEVER ? NAN : nc::step_ms(lf[(size_t)j], sl.dt);
    return NC_OK;
}

}  // extern "C"

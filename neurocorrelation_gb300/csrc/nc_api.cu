// nc_api.cu — the C ABI of include/neucor_gb300.h for a single network.
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "nc_net.h"

namespace {
thread_local std::string g_err;

int fail(int code, const std::string& msg)
{
    g_err = msg;
    return code;
}
}  // namespace

int nc::set_last_error(int code, const std::string& msg) { return fail(code, msg); }

namespace {

// AP_RENDER_BEHAVIOUR (src/NeuCor.cpp:547-550)
float render_behaviour(float val)
{
    val = (float)fmin(fmax((double)val, 0.0), 0.7);
    if (val < 0.5) val = (float)(8.0 * 1000.0 * powf((float)(val / 5.0), 3.0f));
    else {
        const float x = (float)(3.5 - 5 * val);
        val = (float)(8.0 * (x * x));
    }
    return val;
}
}  // namespace


#define NC_NEED(net)                                                  \
    do {                                                              \
        if (!(net)) return fail(NC_ERR_INVALID, "null handle");       \
        cudaError_t e_ = cudaSetDevice((net)->eng.device);            \
        if (e_ != cudaSuccess) return fail(NC_ERR_CUDA, nc::cuda_msg("cudaSetDevice", e_)); \
    } while (0)

// Host step and time from the device's step counter, for handles advanced by
// nc_run_noalloc (nc_net::counters_on_device).  Waits for the handle's stream.
static int refresh_counters(nc_net* net)
{
    if (!net->counters_on_device) return NC_OK;
    std::string err;
    NcNetDesc d{};
    int rc = net->eng.sync(err);
    if (rc == NC_OK) rc = net->eng.read_desc(0, &d, err);
    if (rc != NC_OK) return fail(rc, err);
    net->step = (int64_t)d.t - 1;
    net->time = d.tsum;
    return NC_OK;
}

// NC_NEED, then the host counters brought up to date.
#define NC_NEED_COUNTERS(net)                                         \
    do {                                                              \
        NC_NEED(net);                                                 \
        if (int rc_c_ = refresh_counters(net)) return rc_c_;         \
    } while (0)

#define NC_TRY(expr)                              \
    do {                                          \
        std::string err_;                         \
        int rc_ = (expr);                         \
        if (rc_ != NC_OK) return fail(rc_, err_); \
    } while (0)

// NC_TRY needs `err_` visible inside expr
#define NC_CALL(obj, method, ...)                                  \
    do {                                                           \
        std::string err_;                                          \
        int rc_ = (obj).method(__VA_ARGS__, err_);                 \
        if (rc_ != NC_OK) return fail(rc_, err_);                  \
    } while (0)
#define NC_CALL0(obj, method)                                      \
    do {                                                           \
        std::string err_;                                          \
        int rc_ = (obj).method(err_);                              \
        if (rc_ != NC_OK) return fail(rc_, err_);                  \
    } while (0)

extern "C" {

const char* nc_last_error(void) { return g_err.c_str(); }
const char* nc_version(void) { return "neurocorrelation_gb300 0.1 (sm_103a)"; }

int nc_device_count(int* count)
{
    if (!count) return fail(NC_ERR_INVALID, "null count");
    int c = 0;
    cudaError_t e = cudaGetDeviceCount(&c);
    *count = (e == cudaSuccess) ? c : 0;
    return NC_OK;
}

int nc_set_device(int device)
{
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return fail(NC_ERR_CUDA, nc::cuda_msg("cudaSetDevice", e));
    return NC_OK;
}

int nc_default_params(nc_params* out)
{
    if (!out) return fail(NC_ERR_INVALID, "null params");
    std::memset(out, 0, sizeof(*out));
    out->run_speed = 1.0f;               // src/NeuCor.cpp:18
    out->learning_rate = 1.0f;           // src/NeuCor.cpp:24
    out->presynaptic_trace_decay = 0.75f;
    out->postsynaptic_trace_decay = 0.65f;
    out->presynaptic_factor = 0.13f;
    out->postsynaptic_factor = 0.30f;
    out->background_firing = 1;
    out->inhibitory_rule = NC_INHIBITORY_COPY_LOSS;
    out->seed = 0;
    return NC_OK;
}

int nc_create(int32_t n_neurons, const float* xyz, int64_t n_synapses, const int32_t* syn_from,
              const int32_t* syn_to, const float* syn_weight, const float* syn_length,
              const uint8_t* syn_inhibitory, const nc_params* params, nc_net** out)
{
    if (!out || !params) return fail(NC_ERR_INVALID, "null argument");
    *out = nullptr;
    int devices = 0;
    if (cudaGetDeviceCount(&devices) != cudaSuccess || devices == 0)
        return fail(NC_ERR_NODEVICE, "no CUDA device: the GB300 step has no CPU fallback");
    nc_net* net = new (std::nothrow) nc_net();
    if (!net) return fail(NC_ERR_NOMEM, "host allocation failed");
    std::string err;
    int rc = nc::build_net(n_neurons, xyz, n_synapses, syn_from, syn_to, syn_weight, syn_length, syn_inhibitory,
                           *params, net->host, err);
    if (rc == NC_OK) {
        std::vector<const nc::NetHost*> nets{&net->host};
        rc = net->eng.build(nets, 64, err);
    }
    if (rc != NC_OK) {
        delete net;
        return fail(rc, err);
    }
    net->auto_form = params->step_mode == NC_STEP_AUTO;
    // keep on the host only what read-back needs (the out-synapse tables serve the
    // synapse snapshots)
    nc::NetHost& h = net->host;
    std::vector<uint32_t>().swap(h.out_ringpos);
    std::vector<int32_t>().swap(h.csc_pre);
    std::vector<int32_t>().swap(h.csc_post);
    std::vector<uint16_t>().swap(h.csc_dl);
    std::vector<float>().swap(h.w);
    std::vector<int64_t>().swap(h.in_ptr);
    std::vector<int32_t>().swap(h.ring_off);
    *out = net;
    return NC_OK;
}

int nc_create_knn(int32_t n, int32_t k, float density, uint64_t seed, const nc_params* params, float* xyz_out,
                  nc_net** out)
{
    if (!out || !params) return fail(NC_ERR_INVALID, "null argument");
    *out = nullptr;
    if (n < 0 || k < 0 || !(density > 0.0f) || (n > 0 && k >= n)) return fail(NC_ERR_INVALID, "bad kNN shape");
    int devices = 0;
    if (cudaGetDeviceCount(&devices) != cudaSuccess || devices == 0)
        return fail(NC_ERR_NODEVICE, "no CUDA device: the GB300 step has no CPU fallback");
    nc_net* net = new (std::nothrow) nc_net();
    if (!net) return fail(NC_ERR_NOMEM, "host allocation failed");
    std::string err;
    int rc = nc::build_knn_device(n, k, density, seed, *params, net, err);
    if (rc == NC_ERR_UNSUPPORTED) {
        // outside the device builder's capacities: the host builder, same network
        delete net;
        std::vector<float> xyz(3 * (size_t)n), w((size_t)n * k);
        std::vector<int32_t> from((size_t)n * k), to((size_t)n * k);
        rc = nc_build_knn(n, k, density, seed, xyz.data(), from.data(), to.data(), w.data());
        if (rc != NC_OK) return fail(rc, "kNN build");
        if (xyz_out) std::copy(xyz.begin(), xyz.end(), xyz_out);
        return nc_create(n, xyz.data(), (int64_t)n * k, from.data(), to.data(), w.data(), nullptr, nullptr, params,
                         out);
    }
    if (rc != NC_OK) {
        delete net;
        return fail(rc, err);
    }
    if (xyz_out) std::copy(net->host.xyz.begin(), net->host.xyz.end(), xyz_out);
    std::vector<int64_t>().swap(net->host.in_ptr);
    *out = net;
    return NC_OK;
}

}  // extern "C"

// The read-back tables of a network built on the device (creation order -> CSC
// position, delays, inhibitory bits, out-synapse tables), fetched on first use.
static int ensure_host_tables(nc_net* net)
{
    if (!net->dev_i2c) return NC_OK;
    nc::NetHost& h = net->host;
    const int64_t S = h.s;
    const int32_t k = net->knn_k;
    const auto& P = net->eng.P;
    std::vector<int64_t> i2c((size_t)S);
    std::vector<int32_t> to((size_t)S);
    std::vector<uint16_t> dl((size_t)S);
    NC_CALL(net->eng, download, i2c.data(), (const int64_t*)net->dev_i2c, (size_t)S);
    NC_CALL(net->eng, download, to.data(), (const int32_t*)net->dev_to, (size_t)S);
    NC_CALL(net->eng, download, (int16_t*)dl.data(), (const int16_t*)P.csc_dl, (size_t)S);
    h.csc_delay.resize((size_t)S);
    for (int64_t c = 0; c < S; ++c) h.csc_delay[(size_t)c] = dl[(size_t)c] & 0x3fff;
    h.inh_bits.assign((size_t)((S + 31) / 32), 0u);  // U[0,1) weights: none inhibitory
    // out-synapses of the source in slot s: its k in creation order
    h.out_ptr.resize((size_t)h.n + 1);
    for (int32_t s = 0; s <= h.n; ++s) h.out_ptr[(size_t)s] = (int64_t)s * k;
    h.out_csc.resize((size_t)S);
    h.out_post.resize((size_t)S);
    h.out_delay.resize((size_t)S);
    for (int32_t s = 0; s < h.n; ++s) {
        const int32_t i = h.orig_id[(size_t)s];
        for (int32_t m = 0; m < k; ++m) {
            const int64_t e = (int64_t)i * k + m, q = (int64_t)s * k + m;
            const int64_t c = i2c[(size_t)e];
            h.out_csc[(size_t)q] = (int32_t)c;
            h.out_post[(size_t)q] = h.slot_of[(size_t)to[(size_t)e]];
            h.out_delay[(size_t)q] = (int16_t)dl[(size_t)c];
        }
    }
    h.input_to_csc = std::move(i2c);
    cudaFree(net->dev_i2c);
    cudaFree(net->dev_to);
    net->dev_i2c = nullptr;
    net->dev_to = nullptr;
    return NC_OK;
}

extern "C" {

int nc_destroy(nc_net* net)
{
    if (!net) return NC_OK;
    cudaSetDevice(net->eng.device);
    delete net;
    return NC_OK;
}

int nc_set_input_groups(nc_net* net, int32_t n_groups, const nc_group* groups)
{
    NC_NEED(net);
    std::string err;
    int rc = nc::set_groups(net->host, n_groups, groups, err);
    if (rc != NC_OK) return fail(rc, err);
    NC_CALL(net->eng, set_groups, 0, net->host.groups);
    return NC_OK;
}

// randomUnit(), src/NeuCor.cpp:12-14 (the C library's rand(), as the reference)
static float random_unit() { return (float)rand() / (float)RAND_MAX; }

// Neurons closer than `radius` to `a` (InputFirer / VoltageDetector constructors,
// src/NeuCor.cpp:323-327, 353-357), as caller ids in ascending order.
static std::vector<int32_t> near_ids(const nc::NetHost& h, const float a[3], float radius)
{
    std::vector<int32_t> out;
    for (int32_t j = 0; j < h.n; ++j)
        if (nc::get_dist(&h.xyz[3 * (size_t)j], a) < radius) out.push_back(j);
    return out;
}

// Uploads the firer set: state (lastFire) of the first `keep` firers carried over.
static int upload_firers(nc_net* net, const std::vector<NcFirer>& old, const std::vector<float>& rates)
{
    std::vector<NcFirer> f(net->firer_near.size());
    std::vector<int32_t> near;
    for (size_t i = 0; i < f.size(); ++i) {
        f[i].net = 0;
        f[i].last = i < old.size() ? old[i].last : 0.0f;  // InputFirer: lastFire(0.0)
        // a firer made before the first step also meets the run call at time 0
        f[i].first = i < old.size() ? old[i].first : (net->step == 0 ? 1 : 0);
        f[i].rate = i < rates.size() ? rates[i] : 0.0f;
        f[i].near_begin = (int32_t)near.size();
        for (int32_t id : net->firer_near[i]) near.push_back(net->host.slot_of[(size_t)id]);
        f[i].near_end = (int32_t)near.size();
    }
    NC_CALL(net->eng, set_firers, f, near);
    return NC_OK;
}

int nc_set_input_rate_array(nc_net* net, const float* rates_hz, uint32_t count, const float* xyz,
                            const float* radius)
{
    NC_NEED_COUNTERS(net);
    if (xyz && !radius) return fail(NC_ERR_INVALID, "positions given without radii");
    if (count > (1u << 24)) return fail(NC_ERR_INVALID, "too many input firers");
    std::vector<NcFirer> old;
    NC_CALL(net->eng, read_firers, old);
    const size_t cur = net->firer_near.size();
    // NeuCor::setInputRateArray (src/NeuCor.cpp:46-64): firers are appended (the i-th new
    // one taking position and radius i) or removed from the end to match the count
    if (count > cur) {
        for (size_t i = 0; i < count - cur; ++i) {
            float a[3];
            float r = 1.0f;
            if (xyz) {
                a[0] = xyz[3 * i];
                a[1] = xyz[3 * i + 1];
                a[2] = xyz[3 * i + 2];
                r = radius[i];
            } else {  // InputFirer's random position (src/NeuCor.cpp:312-313)
                for (int d = 0; d < 3; ++d) a[d] = (random_unit() - 0.5f) * 5.f;
            }
            net->firer_xyz.insert(net->firer_xyz.end(), a, a + 3);
            net->firer_radius.push_back(r);
            net->firer_near.push_back(near_ids(net->host, a, r));
        }
    } else {
        net->firer_near.resize(count);
        net->firer_xyz.resize(3 * (size_t)count);
        net->firer_radius.resize(count);
    }
    std::vector<float> rates(count, 0.0f);
    if (rates_hz) std::copy(rates_hz, rates_hz + count, rates.begin());
    return upload_firers(net, old, rates);
}

int nc_set_input_rates(nc_net* net, int32_t count, const float* rates_hz)
{
    NC_NEED(net);
    if (count < 0 || (count > 0 && !rates_hz) || (size_t)count > net->firer_near.size())
        return fail(NC_ERR_INVALID, "more rates than input firers");
    std::vector<NcFirer> f;
    NC_CALL(net->eng, read_firers, f);
    for (int32_t i = 0; i < count; ++i) f[(size_t)i].rate = rates_hz[i];
    NC_CALL(net->eng, write_firers, f);
    return NC_OK;
}

int nc_add_input_offset(nc_net* net, int32_t id, float t_ms)
{
    NC_NEED(net);
    if (id < 0 || (size_t)id >= net->firer_near.size()) return fail(NC_ERR_INVALID, "no such input firer");
    std::vector<NcFirer> f;
    NC_CALL(net->eng, read_firers, f);
    f[(size_t)id].last += t_ms;  // NeuCor::addInputOffset (src/NeuCor.cpp:66-68)
    NC_CALL(net->eng, write_firers, f);
    return NC_OK;
}

int nc_set_detectors(nc_net* net, int32_t count, const float* xyz, const float* radius)
{
    NC_NEED(net);
    if (count < 0 || count > (1 << 24)) return fail(NC_ERR_INVALID, "bad detector count");
    if (xyz && !radius) return fail(NC_ERR_INVALID, "positions given without radii");
    // NeuCor::setDetectors (src/NeuCor.cpp:70-77) appends `count` detectors
    for (int32_t i = 0; i < count; ++i) {
        float a[3];
        float r = 1.0f;
        if (xyz) {
            a[0] = xyz[3 * (size_t)i];
            a[1] = xyz[3 * (size_t)i + 1];
            a[2] = xyz[3 * (size_t)i + 2];
            r = radius[i];
        } else {  // VoltageDetector's random position (src/NeuCor.cpp:349-350)
            for (int d = 0; d < 3; ++d) a[d] = (random_unit() - 0.5f) * 3.f;
        }
        const std::vector<int32_t> ids = near_ids(net->host, a, r);
        net->det_near.insert(net->det_near.end(), ids.begin(), ids.end());
        net->det_ptr.push_back((int32_t)net->det_near.size());
    }
    // device copies: near ids, then the pointer array; one voltage per detector
    if (net->d_det) cudaFree(net->d_det);
    if (net->d_volt) cudaFree(net->d_volt);
    net->d_det = nullptr;
    net->d_volt = nullptr;
    std::vector<int32_t> flat(net->det_near);
    flat.insert(flat.end(), net->det_ptr.begin(), net->det_ptr.end());
    const size_t n_det = net->det_ptr.size() - 1;
    cudaError_t e = cudaMalloc(&net->d_det, sizeof(int32_t) * flat.size());
    if (e == cudaSuccess) e = cudaMalloc(&net->d_volt, sizeof(float) * std::max<size_t>(n_det, 1));
    if (e == cudaSuccess)
        e = cudaMemcpy(net->d_det, flat.data(), sizeof(int32_t) * flat.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(NC_ERR_CUDA, nc::cuda_msg("detector tables", e));
    return NC_OK;
}

int nc_get_detector_voltages(nc_net* net, float* out, int32_t capacity, int32_t* count)
{
    NC_NEED(net);
    const int32_t n_det = (int32_t)net->det_ptr.size() - 1;
    if (count) *count = n_det;
    if (!out || n_det == 0) return NC_OK;
    if (capacity < n_det) return fail(NC_ERR_INVALID, "voltage buffer too small");
    const auto& sl = net->eng.slots[0];
    const int32_t* near = net->d_det;
    const int32_t* ptr = net->d_det + net->det_near.size();
    if (nc::launch_detector_voltages(net->eng.P, sl.neuron_base, near, ptr, n_det, net->d_volt, net->eng.stream))
        return fail(NC_ERR_CUDA, nc::cuda_msg("detector voltages", cudaGetLastError()));
    NC_CALL(net->eng, download, out, (const float*)net->d_volt, (size_t)n_det);
    return NC_OK;
}

int nc_get_detector_voltage(nc_net* net, int32_t id, float* out)
{
    NC_NEED(net);
    const int32_t n_det = (int32_t)net->det_ptr.size() - 1;
    if (!out || id < 0 || id >= n_det) return fail(NC_ERR_INVALID, "no such detector");  // .at(ID) throws
    std::vector<float> v((size_t)n_det);
    const int rc = nc_get_detector_voltages(net, v.data(), n_det, nullptr);
    if (rc != NC_OK) return rc;
    *out = v[(size_t)id];
    return NC_OK;
}

int nc_set_rates(nc_net* net, float learning_rate, float presynaptic_factor, float postsynaptic_factor)
{
    NC_NEED(net);
    NC_CALL(net->eng, set_rates, 0, learning_rate, presynaptic_factor, postsynaptic_factor);
    net->host.p.learning_rate = learning_rate;
    net->host.p.presynaptic_factor = presynaptic_factor;
    net->host.p.postsynaptic_factor = postsynaptic_factor;
    return NC_OK;
}

int nc_schedule_fire(nc_net* net, int32_t count, const int32_t* ids)
{
    NC_NEED(net);
    if (count < 0 || (count > 0 && !ids)) return fail(NC_ERR_INVALID, "bad id array");
    std::vector<int32_t> slots((size_t)count);
    for (int32_t k = 0; k < count; ++k) {
        if (ids[k] < 0 || ids[k] >= net->host.n) return fail(NC_ERR_INVALID, "neuron id out of range");
        slots[(size_t)k] = net->host.slot_of[(size_t)ids[k]];
    }
    NC_CALL(net->eng, force_fire, 0, slots.data(), count);
    return NC_OK;
}

// Steps the engine; a network in NC_STEP_AUTO runs window by window (a window may span
// run calls, so single-step calls synchronise once per window, not per call) and, at
// the end of each, moves to the form its fire share calls for (NC_AUTO_* in
// neucor_gb300.h).
static int advance(nc_net* net, int64_t n_steps)
{
    if (!net->auto_form) {
        NC_CALL(net->eng, step, n_steps);
        return NC_OK;
    }
    const int32_t n = std::max(net->host.n, 1);
    while (n_steps > 0) {
        const int64_t m = std::min<int64_t>(n_steps, NC_AUTO_WINDOW - net->auto_steps);
        NC_CALL(net->eng, step, m);
        net->auto_steps += m;
        n_steps -= m;
        if (net->auto_steps < NC_AUTO_WINDOW) continue;
        unsigned long long st[4];
        NC_CALL(net->eng, read_stats, 0, st);  // fires are counted by the neuron update itself
        const double permille =
            1000.0 * (double)(st[0] - net->auto_fires) / ((double)n * (double)net->auto_steps);
        net->auto_fires = st[0];
        net->auto_steps = 0;
        if (net->eng.dense && permille < NC_AUTO_TO_EVENT_PERMILLE) NC_CALL(net->eng, set_form, false);
        else if (!net->eng.dense && permille > NC_AUTO_TO_DENSE_PERMILLE) NC_CALL(net->eng, set_form, true);
    }
    return NC_OK;
}

int nc_run(nc_net* net, int32_t n_steps)
{
    NC_NEED_COUNTERS(net);
    if (n_steps < 0) return fail(NC_ERR_INVALID, "negative step count");
    if (net->step + n_steps >= (1ll << 30)) return fail(NC_ERR_INVALID, "step counter limit reached");
    if (int rc = advance(net, n_steps)) return rc;
    net->step += n_steps;
    for (int32_t k = 0; k < n_steps; ++k) net->time = net->time + net->host.dt;  // currentTime = targetTime
    return NC_OK;
}

int nc_get_step_form(nc_net* net, int32_t* form)
{
    if (!net || !form) return fail(NC_ERR_INVALID, "null argument");
    *form = net->eng.dense ? NC_STEP_DENSE : NC_STEP_EVENT;
    return NC_OK;
}

int nc_set_step_form(nc_net* net, int32_t form)
{
    NC_NEED(net);
    if (form != NC_STEP_DENSE && form != NC_STEP_EVENT && form != NC_STEP_AUTO)
        return fail(NC_ERR_INVALID, "unknown step form");
    if (form == NC_STEP_AUTO) {
        if (!net->eng.both) return fail(NC_ERR_UNSUPPORTED, "the network was not created with NC_STEP_AUTO");
        unsigned long long st[4];
        NC_CALL(net->eng, read_stats, 0, st);
        net->auto_fires = st[0];
        net->auto_steps = 0;
        net->auto_form = true;
        return NC_OK;
    }
    if (!net->eng.both && (form == NC_STEP_DENSE) != net->eng.dense)
        return fail(NC_ERR_UNSUPPORTED, "the network holds the tables of its own form only (create it with NC_STEP_AUTO)");
    NC_CALL(net->eng, set_form, form == NC_STEP_DENSE);
    net->auto_form = false;
    return NC_OK;
}

int nc_sync(nc_net* net)
{
    NC_NEED(net);
    NC_CALL0(net->eng, sync);
    if (int rc = refresh_counters(net)) return rc;
    return NC_OK;
}

int nc_get_time(nc_net* net, float* ms)
{
    if (!net || !ms) return fail(NC_ERR_INVALID, "null argument");
    if (net->counters_on_device) NC_NEED_COUNTERS(net);
    *ms = net->time;
    return NC_OK;
}

int nc_get_step(nc_net* net, int64_t* step)
{
    if (!net || !step) return fail(NC_ERR_INVALID, "null argument");
    if (net->counters_on_device) NC_NEED_COUNTERS(net);
    *step = net->step;
    return NC_OK;
}

int nc_get_counts(nc_net* net, int32_t* n_neurons, int64_t* n_synapses)
{
    if (!net) return fail(NC_ERR_INVALID, "null handle");
    if (n_neurons) *n_neurons = net->host.n;
    if (n_synapses) *n_synapses = net->host.s;
    return NC_OK;
}

int nc_record_raster(nc_net* net, int32_t max_steps)
{
    NC_NEED_COUNTERS(net);
    if (max_steps < 0) return fail(NC_ERR_INVALID, "negative step count");
    NC_CALL0(net->eng, sync);
    net->raster_t0 = (int32_t)net->step + 1;
    if (net->d_raster && max_steps != net->raster_cap) {
        cudaFree(net->d_raster);
        net->d_raster = nullptr;
        if (net->d_raster_ids) cudaFree(net->d_raster_ids);
        net->d_raster_ids = nullptr;
        net->raster_cap = 0;
    }
    if (max_steps > 0 && !net->d_raster) {
        const size_t words = (size_t)max_steps * net->eng.slots[0].n_words;
        cudaError_t e = cudaMalloc(&net->d_raster, std::max<size_t>(words, 1) * sizeof(uint32_t));
        if (e != cudaSuccess) return fail(NC_ERR_NOMEM, nc::cuda_msg("cudaMalloc raster", e));
        if (net->host.permuted) {
            e = cudaMalloc(&net->d_raster_ids, std::max<size_t>(words, 1) * sizeof(uint32_t));
            if (e != cudaSuccess) return fail(NC_ERR_NOMEM, nc::cuda_msg("cudaMalloc raster", e));
        }
        e = cudaMemset(net->d_raster, 0, std::max<size_t>(words, 1) * sizeof(uint32_t));
        if (e != cudaSuccess) return fail(NC_ERR_CUDA, nc::cuda_msg("cudaMemset raster", e));
        net->raster_cap = max_steps;
    }
    NC_CALL(net->eng, set_raster, 0, net->d_raster, net->raster_t0, net->raster_cap);
    return NC_OK;
}

int nc_read_raster(nc_net* net, uint8_t* out, int64_t capacity_bytes, int32_t* steps)
{
    NC_NEED_COUNTERS(net);
    if (!steps) return fail(NC_ERR_INVALID, "null steps");
    const int64_t done = net->step - net->raster_t0 + 1;
    const int32_t rows = (int32_t)std::max<int64_t>(0, std::min<int64_t>(done, net->raster_cap));
    const int32_t nw = net->eng.slots[0].n_words;
    const int64_t row_bytes = ((int64_t)net->host.n + 7) / 8;
    *steps = rows;
    if (!out) return NC_OK;
    if (capacity_bytes < rows * row_bytes) return fail(NC_ERR_INVALID, "raster buffer too small");
    const nc::NetHost& h = net->host;
    const uint32_t* src = net->d_raster;
    if (h.permuted && rows > 0) {
        const auto& sl = net->eng.slots[0];
        if (nc::launch_raster_to_ids(net->d_raster, net->d_raster_ids, net->eng.P.slot_of + sl.neuron_base, h.n, nw,
                                     rows, net->eng.stream))
            return fail(NC_ERR_CUDA, nc::cuda_msg("raster reorder", cudaGetLastError()));
        src = net->d_raster_ids;
    }
    std::vector<uint32_t> buf((size_t)rows * nw);
    NC_CALL(net->eng, download, buf.data(), src, buf.size());
    for (int32_t r = 0; r < rows; ++r)
        std::memcpy(out + (int64_t)r * row_bytes, buf.data() + (size_t)r * nw, (size_t)row_bytes);
    return NC_OK;
}

int nc_read_potentials(nc_net* net, float* out_n)
{
    NC_NEED(net);
    if (!out_n && net->host.n) return fail(NC_ERR_INVALID, "null output");
    const auto& sl = net->eng.slots[0];
    std::vector<float> pot((size_t)sl.n);
    NC_CALL(net->eng, download, pot.data(), (const float*)net->eng.P.pot + sl.neuron_base, (size_t)sl.n);
    nc::to_caller_order(net->host, pot.data(), out_n);
    return NC_OK;
}

int nc_read_potact(nc_net* net, float* out_2n)
{
    NC_NEED_COUNTERS(net);
    const int32_t n = net->host.n;
    if (!out_2n && n) return fail(NC_ERR_INVALID, "null output");
    std::vector<float> pot((size_t)n);
    std::vector<uint32_t> fir((size_t)n);
    std::vector<int32_t> start((size_t)n);
    const auto& sl = net->eng.slots[0];
    NC_CALL(net->eng, download, pot.data(), (const float*)net->eng.P.pot + sl.neuron_base, (size_t)n);
    NC_CALL(net->eng, download, fir.data(), (const uint32_t*)net->eng.P.firings + sl.neuron_base, (size_t)n);
    NC_CALL(net->eng, download, start.data(), (const int32_t*)net->eng.P.act_start + sl.neuron_base, (size_t)n);
    const float dt = net->host.dt;
    const int64_t t = net->step;
    std::vector<float> pot_c((size_t)n);
    std::vector<uint32_t> fir_c((size_t)n);
    std::vector<int32_t> start_c((size_t)n);
    nc::to_caller_order(net->host, pot.data(), pot_c.data());
    nc::to_caller_order(net->host, fir.data(), fir_c.data());
    nc::to_caller_order(net->host, start.data(), start_c.data());
    pot.swap(pot_c);
    fir.swap(fir_c);
    start.swap(start_c);
    for (int32_t j = 0; j < n; ++j) {
        out_2n[2 * (size_t)j] = pot[j];
        // setActivity(firings/(((float) currentT-activityStartTime)/10.0)) at the last update
        float act = 0.0f;
        if (t >= 1 && t > start[j])
            act = (float)(fir[j] / (((float)nc::step_ms(t, dt) - nc::step_ms(start[j], dt)) / 10.0));
        out_2n[2 * (size_t)j + 1] = act;
    }
    return NC_OK;
}

int nc_read_positions(nc_net* net, float* out_3n)
{
    if (!net || (!out_3n && net->host.n)) return fail(NC_ERR_INVALID, "null argument");
    std::memcpy(out_3n, net->host.xyz.data(), sizeof(float) * net->host.xyz.size());
    return NC_OK;
}

int nc_read_last_fire(nc_net* net, float* out_n)
{
    NC_NEED(net);
    const int32_t n = net->host.n;
    if (!out_n && n) return fail(NC_ERR_INVALID, "null output");
    std::vector<int32_t> lf_s((size_t)n), lf((size_t)n);
    NC_CALL(net->eng, download, lf_s.data(), (const int32_t*)net->eng.P.lf + net->eng.slots[0].neuron_base, (size_t)n);
    nc::to_caller_order(net->host, lf_s.data(), lf.data());
    for (int32_t j = 0; j < n; ++j) out_n[j] = lf[j] == NC_NEVER ? NAN : nc::step_ms(lf[j], net->host.dt);
    return NC_OK;
}

int nc_read_weights(nc_net* net, float* out_s)
{
    NC_NEED(net);
    if (int rc = ensure_host_tables(net)) return rc;
    const nc::NetHost& h = net->host;
    if (!out_s && h.n_input) return fail(NC_ERR_INVALID, "null output");
    NC_CALL0(net->eng, flush_plasticity);
    std::vector<float> w((size_t)h.s);
    NC_CALL(net->eng, download, w.data(), (const float*)net->eng.P.w + net->eng.slots[0].syn_base, (size_t)h.s);
    for (int64_t k = 0; k < h.n_input; ++k) {
        const int64_t c = h.input_to_csc[(size_t)k];
        out_s[k] = c < 0 ? NAN : w[(size_t)c];
    }
    return NC_OK;
}

int nc_read_delays(nc_net* net, int32_t* out_s)
{
    NC_NEED(net);
    if (!out_s && net->host.n_input) return fail(NC_ERR_INVALID, "null argument");
    if (int rc = ensure_host_tables(net)) return rc;
    const nc::NetHost& h = net->host;
    for (int64_t k = 0; k < h.n_input; ++k) {
        const int64_t c = h.input_to_csc[(size_t)k];
        out_s[k] = c < 0 ? -1 : h.csc_delay[(size_t)c];
    }
    return NC_OK;
}

int nc_read_inhibitory(nc_net* net, uint8_t* out_s)
{
    NC_NEED(net);
    if (!out_s && net->host.n_input) return fail(NC_ERR_INVALID, "null argument");
    if (int rc = ensure_host_tables(net)) return rc;
    const nc::NetHost& h = net->host;
    for (int64_t k = 0; k < h.n_input; ++k) {
        const int64_t c = h.input_to_csc[(size_t)k];
        out_s[k] = c < 0 ? 255 : (nc::inhibitory_flag(h, c) ? 1 : 0);
    }
    return NC_OK;
}

int nc_read_synapse_snapshots(nc_net* net, nc_synapse_snapshot* out, int64_t capacity, int64_t* count)
{
    NC_NEED_COUNTERS(net);
    if (!count) return fail(NC_ERR_INVALID, "null count");
    const nc::NetHost& h = net->host;
    *count = h.s;
    if (!out) return NC_OK;
    if (capacity < h.s) return fail(NC_ERR_INVALID, "snapshot buffer too small");
    if (int rc = ensure_host_tables(net)) return rc;
    NC_CALL0(net->eng, flush_plasticity);
    const auto& sl = net->eng.slots[0];
    const auto& P = net->eng.P;
    std::vector<float> w((size_t)h.s);
    std::vector<int32_t> la((size_t)h.s);  // CSC order (dense form) or out-synapse order (event form)
    NC_CALL(net->eng, download, w.data(), (const float*)P.w + sl.syn_base, (size_t)h.s);
    const bool dense = net->eng.dense;
    NC_CALL(net->eng, download, la.data(), (const int32_t*)(dense ? P.la_c : P.last_arr) + sl.syn_base, (size_t)h.s);
    const float T = net->time;
    const int64_t t = net->step;
    int64_t q = 0;
    for (int32_t i = 0; i < h.n; ++i) {
        const int32_t si = h.slot_of[(size_t)i];
        for (int64_t k = h.out_ptr[(size_t)si]; k < h.out_ptr[(size_t)si + 1]; ++k) {
            nc_synapse_snapshot& o = out[q++];
            const int32_t c = h.out_csc[(size_t)k];
            const float weight = w[(size_t)c];
            o.from_id = i;
            o.to_id = h.orig_id[(size_t)h.out_post[(size_t)k]];
            o.weight = weight;
            o.inhibitory = weight < 0.0f;
            o.pre_potential = 0.0f;
            o.post_potential = 0.0f;
            const int32_t a = la[(size_t)(dense ? c : k)];
            // in flight (AP_fireTime != 0) until its target's update KC steps after arrival
            if (a == NC_NEVER || t - a >= h.kc) continue;
            const int32_t d = (int32_t)((uint16_t)h.out_delay[(size_t)k] & 0x3fffu);
            const float length_speed = ((float)d * h.dt / 2.0f) * 2.0f;  // length*AP_speed
            const float fire_time = nc::step_ms(a, h.dt);                  // AP_fireTime
            const float start = nc::step_ms(a - d, h.dt);                  // lastSpikeStart
            o.pre_potential = render_behaviour((float)(T - start) / length_speed) * weight;
            if (T < fire_time) o.post_potential = render_behaviour((float)(fire_time - T) / length_speed) * weight;
        }
    }
    return NC_OK;
}

int nc_read_input_snapshots(nc_net* net, nc_input_snapshot* out, int32_t capacity, int32_t* count)
{
    NC_NEED(net);
    if (!count) return fail(NC_ERR_INVALID, "null count");
    const int32_t nf = (int32_t)net->firer_near.size();
    *count = nf;
    if (!out || nf == 0) return NC_OK;
    if (capacity < nf) return fail(NC_ERR_INVALID, "input snapshot buffer too small");
    std::vector<NcFirer> f;  // the rates as the next step's run call reads them
    NC_CALL(net->eng, read_firers, f);
    for (int32_t i = 0; i < nf; ++i) {
        nc_input_snapshot& o = out[i];
        o.id = i;
        o.x = net->firer_xyz[3 * (size_t)i];
        o.y = net->firer_xyz[3 * (size_t)i + 1];
        o.z = net->firer_xyz[3 * (size_t)i + 2];
        o.radius = net->firer_radius[(size_t)i];
        o.frequency = (size_t)i < f.size() ? f[(size_t)i].rate : 0.0f;
        o.enabled = 1;
    }
    return NC_OK;
}

int nc_reset_activities(nc_net* net)
{
    NC_NEED_COUNTERS(net);
    const auto& sl = net->eng.slots[0];
    std::vector<int32_t> start((size_t)sl.n, (int32_t)net->step);
    cudaError_t e = cudaMemcpyAsync(net->eng.P.act_start + sl.neuron_base, start.data(), sizeof(int32_t) * sl.n,
                                    cudaMemcpyHostToDevice, net->eng.stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(net->eng.P.firings + sl.neuron_base, 0, sizeof(uint32_t) * sl.n,
                                              net->eng.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(net->eng.stream);
    if (e != cudaSuccess) return fail(NC_ERR_CUDA, nc::cuda_msg("reset activities", e));
    return NC_OK;
}

int nc_get_stats(nc_net* net, nc_stats* out)
{
    NC_NEED(net);
    if (!out) return fail(NC_ERR_INVALID, "null output");
    unsigned long long s[4];
    // the dense form counts a step's launches when the next step (or a flush) makes them
    NC_CALL0(net->eng, flush_plasticity);
    NC_CALL(net->eng, read_stats, 0, s);
    out->fires = (int64_t)s[0];
    out->launched = (int64_t)s[1];
    out->dropped = (int64_t)s[2];
    out->steps = (int64_t)s[3];
    return NC_OK;
}

int nc_delete_synapse(nc_net* net, int32_t from_id, int32_t to_id)
{
    (void)net; (void)from_id; (void)to_id;
    return fail(NC_ERR_UNSUPPORTED, "topology mutation is outside the GPU step model");
}

int nc_delete_neuron(nc_net* net, int32_t id)
{
    (void)net; (void)id;
    return fail(NC_ERR_UNSUPPORTED, "topology mutation is outside the GPU step model");
}

int nc_time_steps(nc_net* net, int32_t n_steps, float* ms, float* kernel_ms)
{
    NC_NEED_COUNTERS(net);
    if (n_steps < 0 || !ms) return fail(NC_ERR_INVALID, "bad argument");
    if (net->auto_form) {
        // the window reads and any switch are part of the timed steps
        cudaEvent_t a, b;
        if (cudaEventCreate(&a) != cudaSuccess) return fail(NC_ERR_CUDA, "cudaEventCreate");
        if (cudaEventCreate(&b) != cudaSuccess) {
            cudaEventDestroy(a);
            return fail(NC_ERR_CUDA, "cudaEventCreate");
        }
        cudaEventRecord(a, net->eng.stream);
        int rc = advance(net, n_steps);
        cudaEventRecord(b, net->eng.stream);
        cudaError_t e = cudaEventSynchronize(b);
        if (rc == NC_OK && e == cudaSuccess) e = cudaEventElapsedTime(ms, a, b);
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        if (rc != NC_OK) return rc;
        if (e != cudaSuccess) return fail(NC_ERR_CUDA, nc::cuda_msg("step timing", e));
    } else {
        NC_CALL(net->eng, step_timed, (int64_t)n_steps, ms);
    }
    net->step += n_steps;
    for (int32_t k = 0; k < n_steps; ++k) net->time = net->time + net->host.dt;
    if (kernel_ms) {
        const int m = std::min(n_steps, 200);
        NC_CALL(net->eng, time_kernels, m, &kernel_ms[0], &kernel_ms[1]);
        net->step += m;
        for (int k = 0; k < m; ++k) net->time = net->time + net->host.dt;
    }
    return NC_OK;
}

}  // extern "C"

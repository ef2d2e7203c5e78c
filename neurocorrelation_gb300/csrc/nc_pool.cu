// nc_pool.cu — the device engine (see nc_pool.h).
#include "nc_pool.h"

#include <algorithm>
#include <cstddef>
#include <cstring>
#include <string>

namespace nc {

std::string cuda_msg(const char* what, cudaError_t e)
{
    return std::string(what) + ": " + cudaGetErrorString(e);
}

#define NC_CK(call)                                                  \
    do {                                                             \
        cudaError_t e_ = (call);                                     \
        if (e_ != cudaSuccess) {                                     \
            err = cuda_msg(#call, e_);                               \
            return e_ == cudaErrorMemoryAllocation ? NC_ERR_NOMEM : NC_ERR_CUDA; \
        }                                                            \
    } while (0)

Engine::~Engine()
{
    release_graph();
    if (stream) cudaStreamSynchronize(stream);
    if (firers_buf_) cudaFree(firers_buf_);
    if (near_buf_) cudaFree(near_buf_);
    for (void* p : allocs_) cudaFree(p);
    if (stream) cudaStreamDestroy(stream);
}

template <class T>
T* Engine::alloc(size_t count, std::string& err)
{
    void* p = nullptr;
    const size_t bytes = std::max<size_t>(1, count) * sizeof(T);
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
        err = cuda_msg("cudaMalloc", e);
        return nullptr;
    }
    allocs_.push_back(p);
    e = cudaMemsetAsync(p, 0, bytes, stream);
    if (e != cudaSuccess) {
        err = cuda_msg("cudaMemsetAsync", e);
        return nullptr;
    }
    return (T*)p;
}

template <class T>
int Engine::download(T* host, const T* dev, size_t count, std::string& err)
{
    if (count == 0) return NC_OK;
    NC_CK(cudaMemcpyAsync(host, dev, count * sizeof(T), cudaMemcpyDeviceToHost, stream));
    NC_CK(cudaStreamSynchronize(stream));
    return NC_OK;
}

template int Engine::download<float>(float*, const float*, size_t, std::string&);
template int Engine::download<int32_t>(int32_t*, const int32_t*, size_t, std::string&);
template int Engine::download<uint32_t>(uint32_t*, const uint32_t*, size_t, std::string&);
template int Engine::download<int16_t>(int16_t*, const int16_t*, size_t, std::string&);
template int Engine::download<int64_t>(int64_t*, const int64_t*, size_t, std::string&);
template int Engine::download<double>(double*, const double*, size_t, std::string&);

#define NC_ALLOC(ptr, T, count)                  \
    do {                                         \
        ptr = alloc<T>((count), err);            \
        if (!ptr) return NC_ERR_NOMEM;           \
    } while (0)

template <class T>
static cudaError_t upload(T* dev, const std::vector<T>& host, size_t offset, cudaStream_t s)
{
    if (host.empty()) return cudaSuccess;
    return cudaMemcpyAsync(dev + offset, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice, s);
}

void Engine::set_launch(const LaunchShape& shape, int ticks_per_graph)
{
    release_graph();
    L = shape;
    graph_ticks = ticks_per_graph;
}

int Engine::build(const std::vector<const NetHost*>& nets, int group_capacity, std::string& err,
                  const std::vector<int32_t>* horizons, bool device_synapses)
{
    NC_CK(cudaGetDevice(&device));
    NC_CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    int sms = 0;
    NC_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    dense = nets.empty() || nets[0]->p.step_mode != NC_STEP_EVENT;
    both = !nets.empty() && nets[0]->p.step_mode == NC_STEP_AUTO;
    const bool event_tables = !dense || both;
    // the dense neuron pass is one wave: 128-thread blocks spread it more evenly over the
    // SMs (measured 2% faster on the 100k x 100 network than 256)
    L.neuron_block = dense ? NC_DNEURON_BLOCK : 256;
    L.launch_block = 256;
    L.launch_blocks = std::max(1, sms * NC_LAUNCH_MIN_BLOCKS);

    // pool sizes
    int64_t neurons = 0, ptrs = 0, words = 0, syn = 0, ring = 0, tables = 0, tiles = 0, spans = 0;
    const int ngroups_each = std::max(group_capacity, 1);
    slots.clear();
    std::vector<NcNetDesc> desc;
    for (size_t q = 0; q < nets.size(); ++q) {
        const NetHost& h = *nets[q];
        NetSlot sl;
        sl.n = h.n;
        sl.s = h.s;
        sl.kc = h.kc;
        sl.dt = h.dt;
        sl.n_words = (h.n + 31) / 32;
        sl.neuron_base = (int32_t)neurons;
        sl.ptr_base = (int32_t)ptrs;
        sl.word_base = (int32_t)words;
        sl.syn_base = syn;
        sl.group_cap = ngroups_each;
        sl.group_base = (int32_t)(q * ngroups_each);
        NcNetDesc d;
        std::memset(&d, 0, sizeof(d));
        d.t = 1;
        d.t_end = horizons ? (*horizons)[q] : (1 << 30);
        d.stdp_done = 0;
        d.n = h.n;
        d.neuron_base = sl.neuron_base;
        d.ptr_base = sl.ptr_base;
        d.word_base = sl.word_base;
        d.n_words = sl.n_words;
        d.syn_base = syn;
        d.ring_base = ring;
        d.ring_words = h.ring_words;
        d.ring_mask = h.ring_slots - 1;
        d.kc = h.kc;
        d.bg_period = h.bg_period;
        d.key0 = (uint32_t)h.p.seed;
        d.key1 = (uint32_t)(h.p.seed >> 32);
        d.table_base = (int32_t)tables;
        d.tab_pre_len = h.tab_pre_len;
        d.tab_post_len = h.tab_post_len;
        d.ap_base = (int32_t)(tables + h.tab_pre_len + h.tab_post_len);
        d.group_base = sl.group_base;
        d.n_groups = (int32_t)std::min<size_t>(h.groups.size(), (size_t)ngroups_each);
        nc_group_range(h.groups.data(), d.n_groups, d.group_lo, d.group_hi);
        d.active = 1;
        d.permuted = h.permuted ? 1 : 0;
        d.nonneg_terms = h.nonneg_terms ? 1 : 0;
        d.dt = h.dt;
        d.leak = h.leak;
        d.c52 = h.c52;
        d.lr = h.p.learning_rate;
        d.pre_factor = h.p.presynaptic_factor;
        d.post_factor = h.p.postsynaptic_factor;
        d.e_term = h.e_term;
        d.n_syn = h.s;
        desc.push_back(d);
        slots.push_back(sl);
        neurons += h.n;
        ptrs += h.n + 1;
        words += sl.n_words;
        syn += (h.s + 31) / 32 * 32;  // keeps every net's inhibitory bits word-aligned
        if (event_tables) ring += (int64_t)h.ring_slots * h.ring_words;
        tables += (int64_t)h.tables.size();
        tiles += sl.n_words;
        spans += ((h.s + 31) / 32 + NC_SPAN_CHUNKS - 1) / NC_SPAN_CHUNKS;
        if (h.groups.size() > (size_t)ngroups_each) {
            err = "more input groups than reserved";
            return NC_ERR_INVALID;
        }
    }
    if (neurons >= (1ll << 31) || tables >= (1ll << 31) || words >= (1ll << 31)) {
        err = "pool too large";
        return NC_ERR_INVALID;
    }

    NC_ALLOC(P.pot, float, neurons);
    NC_ALLOC(P.lf, int32_t, neurons);
    NC_ALLOC(P.firings, uint32_t, neurons);
    NC_ALLOC(P.act_start, int32_t, neurons);
    NC_ALLOC(P.orig_id, int32_t, neurons);
    NC_ALLOC(P.slot_of, int32_t, neurons);
    NC_ALLOC(P.in_ptr, int64_t, ptrs);
    NC_ALLOC(P.w, float, syn);
    NC_ALLOC(P.inh, uint32_t, (syn + 31) / 32 + 1);  // one spare word for 32-bit windows
    NC_ALLOC(P.t_arr, int32_t, syn);
    NC_ALLOC(P.term, double, syn);
    if (dense) {
        NC_ALLOC(P.csc_pre, int32_t, syn);
        NC_ALLOC(P.csc_post, int32_t, syn);
        NC_ALLOC(P.csc_dl, uint16_t, syn);
        NC_ALLOC(P.la_c, int32_t, syn);
        NC_ALLOC(P.pst, float, neurons);
        NC_ALLOC(P.win, uint32_t, syn / 32 + 1);
        NC_ALLOC(P.spans, NcTile, spans);
    }
    if (event_tables) {
        NC_ALLOC(P.out_ptr, int64_t, ptrs);
        NC_ALLOC(P.ring_off, int32_t, ptrs);
        NC_ALLOC(P.out_post, int32_t, syn);
        NC_ALLOC(P.out_csc, int32_t, syn);
        NC_ALLOC(P.out_delay, int16_t, syn);
        NC_ALLOC(P.out_ringpos, uint32_t, syn);
        NC_ALLOC(P.last_arr, int32_t, syn);
        NC_ALLOC(P.ring, uint32_t, ring);
        ring_words_total_ = ring;
    }
    P.total_words = std::max<int64_t>(words, 1);
    NC_ALLOC(P.fired, uint32_t, 2 * P.total_words);
    NC_ALLOC(P.forced, uint32_t, 2 * P.total_words);
    NC_ALLOC(P.ufire, uint32_t, 2 * P.total_words);
    P.fired_cap = event_tables ? std::max<int64_t>(neurons, 1) : 0;
    if (event_tables) NC_ALLOC(P.fired_list, int2, 2 * P.fired_cap);
    NC_ALLOC(P.fired_count, int32_t, 2);
    NC_ALLOC(P.tables, float, tables);
    NC_ALLOC(P.groups, NcGroupDev, nets.size() * ngroups_each);
    NC_ALLOC(P.nets, NcNetDesc, nets.size());
    NC_ALLOC(P.tiles, NcTile, tiles);
    NC_ALLOC(P.tick, int32_t, 1);
    NC_ALLOC(P.done_ctr, uint32_t, 1);
    NC_ALLOC(P.dev_err, uint32_t, 1);
    NC_ALLOC(d_bar_, unsigned, 2);
    NC_ALLOC(d_stats_, unsigned long long, 4 * nets.size());
    P.n_nets = (int32_t)nets.size();
    P.n_tiles = (int32_t)tiles;
    P.n_spans = dense ? (int32_t)spans : 0;

    // contents
    std::vector<NcTile> tile_host, span_host;
    tile_host.reserve((size_t)tiles);
    for (size_t q = 0; q < nets.size(); ++q) {
        const NetHost& h = *nets[q];
        const NetSlot& sl = slots[q];
        NcNetDesc& d = desc[q];
        d.stats = d_stats_ + 4 * q;
        std::vector<float> pot((size_t)h.n, -70.0f);  // setPotential(baselevel)
        std::vector<int32_t> lf((size_t)h.n, NC_NEVER);
        NC_CK(upload(P.pot, pot, sl.neuron_base, stream));
        NC_CK(upload(P.lf, lf, sl.neuron_base, stream));
        NC_CK(upload(P.orig_id, h.orig_id, sl.neuron_base, stream));
        NC_CK(upload(P.slot_of, h.slot_of, sl.neuron_base, stream));
        std::vector<int64_t> inp(h.in_ptr), outp(h.out_ptr);
        for (auto& v : inp) v += sl.syn_base;
        for (auto& v : outp) v += sl.syn_base;
        NC_CK(upload(P.in_ptr, inp, sl.ptr_base, stream));
        if (dense && device_synapses) {
            const int32_t chunks = (int32_t)((h.s + 31) / 32);
            for (int32_t c = 0; c < chunks; c += NC_SPAN_CHUNKS) span_host.push_back(NcTile{(int32_t)q, c});
        } else {
        NC_CK(upload(P.w, h.w, sl.syn_base, stream));
        NC_CK(upload(P.inh, h.inh_bits, sl.syn_base / 32, stream));
        std::vector<int32_t> never((size_t)h.s, NC_NEVER);
        NC_CK(upload(P.t_arr, never, sl.syn_base, stream));
        if (dense) {
            NC_CK(upload(P.csc_pre, h.csc_pre, sl.syn_base, stream));
            NC_CK(upload(P.csc_post, h.csc_post, sl.syn_base, stream));
            NC_CK(upload(P.csc_dl, h.csc_dl, sl.syn_base, stream));
            NC_CK(upload(P.la_c, never, sl.syn_base, stream));
            const int32_t chunks = (int32_t)((h.s + 31) / 32);
            for (int32_t c = 0; c < chunks; c += NC_SPAN_CHUNKS) span_host.push_back(NcTile{(int32_t)q, c});
        }
        if (event_tables) {
            NC_CK(upload(P.out_ptr, outp, sl.ptr_base, stream));
            NC_CK(upload(P.ring_off, h.ring_off, sl.ptr_base, stream));
            NC_CK(upload(P.last_arr, never, sl.syn_base, stream));
            NC_CK(upload(P.out_post, h.out_post, sl.syn_base, stream));
            NC_CK(upload(P.out_csc, h.out_csc, sl.syn_base, stream));
            NC_CK(upload(P.out_delay, h.out_delay, sl.syn_base, stream));
            NC_CK(upload(P.out_ringpos, h.out_ringpos, sl.syn_base, stream));
        }
        }
        NC_CK(upload(P.tables, h.tables, d.table_base, stream));
        if (!h.groups.empty()) NC_CK(upload(P.groups, h.groups, sl.group_base, stream));
        for (int32_t f = 0; f < h.n; f += 32) tile_host.push_back(NcTile{(int32_t)q, f});
        // the vectors above must stay alive until the copies finish
        NC_CK(cudaStreamSynchronize(stream));
    }
    NC_CK(upload(P.nets, desc, 0, stream));
    NC_CK(upload(P.tiles, tile_host, 0, stream));
    if (dense) NC_CK(upload(P.spans, span_host, 0, stream));
    NC_CK(cudaStreamSynchronize(stream));
    for (size_t q = 0; q < nets.size(); ++q) {
        if (launch_background_prologue(P, (int)q, nets[q]->n, stream) != 0) {
            err = cuda_msg("background prologue", cudaGetLastError());
            return NC_ERR_CUDA;
        }
    }
    NC_CK(cudaStreamSynchronize(stream));
    return NC_OK;
}

void Engine::release_graph()
{
    if (graph_) cudaGraphExecDestroy(graph_);
    graph_ = nullptr;
}

int Engine::capture_graph(std::string& err)
{
    release_graph();
    cudaGraph_t g = nullptr;
    if (dense) prepare_dense_launch();
    NC_CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    int rc = 0;
    for (int k = 0; k < graph_ticks && rc == 0; ++k) rc |= launch_tick(stream);
    cudaError_t e = cudaStreamEndCapture(stream, &g);
    if (rc != 0 || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        err = cuda_msg("graph capture", e != cudaSuccess ? e : cudaGetLastError());
        return NC_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&graph_, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        graph_ = nullptr;
        err = cuda_msg("cudaGraphInstantiate", e);
        return NC_ERR_CUDA;
    }
    return NC_OK;
}

int Engine::step(int64_t ticks, std::string& err)
{
    if (ticks <= 0) return NC_OK;
    if (dense && L.fused_ticks > 0 && P.n_firers == 0) {
        // several whole steps per cooperative launch
        while (ticks > 0) {
            const int32_t m = (int32_t)std::min<int64_t>(ticks, L.fused_ticks);
            if (launch_fused_dense(P, m, d_bar_, stream)) {
                err = cuda_msg("fused step launch", cudaGetLastError());
                return NC_ERR_CUDA;
            }
            ticks -= m;
        }
        return NC_OK;
    }
    if (ticks >= graph_ticks && graph_ticks > 0) {
        if (!graph_) {
            const int rc = capture_graph(err);
            if (rc) return rc;
        }
        while (ticks >= graph_ticks) {
            NC_CK(cudaGraphLaunch(graph_, stream));
            ticks -= graph_ticks;
        }
    }
    for (int64_t k = 0; k < ticks; ++k) {
        if (launch_tick(stream)) {
            err = cuda_msg("step launch", cudaGetLastError());
            return NC_ERR_CUDA;
        }
    }
    return NC_OK;
}

int Engine::launch_tick(cudaStream_t s)
{
    int rc = P.n_firers > 0 ? launch_input_firers(P, s) : 0;  // the step's run-call schedule first
    rc |= dense ? launch_step_dense(P, L, s) : (launch_neuron_step(P, L, s) | launch_spike_launch(P, L, s));
    return rc;
}

int Engine::set_firers(const std::vector<NcFirer>& firers, const std::vector<int32_t>& near, std::string& err)
{
    release_graph();  // the captured ticks change
    NC_CK(cudaStreamSynchronize(stream));
    if (firers_buf_) cudaFree(firers_buf_);
    if (near_buf_) cudaFree(near_buf_);
    firers_buf_ = nullptr;
    near_buf_ = nullptr;
    P.firers = nullptr;
    P.firer_near = nullptr;
    P.n_firers = 0;
    if (firers.empty()) return NC_OK;
    NC_CK(cudaMalloc(&firers_buf_, sizeof(NcFirer) * firers.size()));
    NC_CK(cudaMalloc(&near_buf_, sizeof(int32_t) * std::max<size_t>(near.size(), 1)));
    NC_CK(cudaMemcpyAsync(firers_buf_, firers.data(), sizeof(NcFirer) * firers.size(), cudaMemcpyHostToDevice, stream));
    if (!near.empty())
        NC_CK(cudaMemcpyAsync(near_buf_, near.data(), sizeof(int32_t) * near.size(), cudaMemcpyHostToDevice, stream));
    P.firers = (NcFirer*)firers_buf_;
    P.firer_near = (int32_t*)near_buf_;
    P.n_firers = (int32_t)firers.size();
    NC_CK(cudaStreamSynchronize(stream));
    return NC_OK;
}

int Engine::read_firers(std::vector<NcFirer>& out, std::string& err)
{
    out.resize((size_t)P.n_firers);
    if (P.n_firers == 0) return NC_OK;
    NC_CK(cudaMemcpyAsync(out.data(), P.firers, sizeof(NcFirer) * out.size(), cudaMemcpyDeviceToHost, stream));
    NC_CK(cudaStreamSynchronize(stream));
    return NC_OK;
}

int Engine::write_firers(const std::vector<NcFirer>& in, std::string& err)
{
    if ((int32_t)in.size() != P.n_firers) {
        err = "firer count mismatch";
        return NC_ERR_INVALID;
    }
    if (P.n_firers == 0) return NC_OK;
    NC_CK(cudaMemcpyAsync(P.firers, in.data(), sizeof(NcFirer) * in.size(), cudaMemcpyHostToDevice, stream));
    NC_CK(cudaStreamSynchronize(stream));
    return NC_OK;
}

int Engine::step_timed(int64_t ticks, float* ms, std::string& err)
{
    cudaEvent_t a, b;
    NC_CK(cudaEventCreate(&a));
    NC_CK(cudaEventCreate(&b));
    NC_CK(cudaEventRecord(a, stream));
    int rc = step(ticks, err);
    if (rc == NC_OK) {
        NC_CK(cudaEventRecord(b, stream));
        NC_CK(cudaEventSynchronize(b));
        NC_CK(cudaEventElapsedTime(ms, a, b));
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return rc;
}

int Engine::time_kernels(int ticks, float* neuron_ms, float* launch_ms, std::string& err)
{
    std::vector<cudaEvent_t> ev(3 * (size_t)std::max(ticks, 0));
    for (auto& e : ev) NC_CK(cudaEventCreate(&e));
    for (int k = 0; k < ticks; ++k) {
        if (P.n_firers > 0 && launch_input_firers(P, stream)) {
            err = "launch";
            return NC_ERR_CUDA;
        }
        NC_CK(cudaEventRecord(ev[3 * k], stream));
        if (dense ? launch_dense_synapses(P, L, stream) : launch_neuron_step(P, L, stream)) {
            err = "launch";
            return NC_ERR_CUDA;
        }
        NC_CK(cudaEventRecord(ev[3 * k + 1], stream));
        if (dense ? launch_dense_neurons(P, L, stream) : launch_spike_launch(P, L, stream)) {
            err = "launch";
            return NC_ERR_CUDA;
        }
        NC_CK(cudaEventRecord(ev[3 * k + 2], stream));
    }
    NC_CK(cudaStreamSynchronize(stream));
    double sa = 0, sb = 0;
    for (int k = 0; k < ticks; ++k) {
        float x = 0, y = 0;
        NC_CK(cudaEventElapsedTime(&x, ev[3 * k], ev[3 * k + 1]));
        NC_CK(cudaEventElapsedTime(&y, ev[3 * k + 1], ev[3 * k + 2]));
        sa += x;
        sb += y;
    }
    for (auto& e : ev) cudaEventDestroy(e);
    *neuron_ms = ticks ? (float)(sa / ticks) : 0.0f;
    *launch_ms = ticks ? (float)(sb / ticks) : 0.0f;
    return NC_OK;
}

int Engine::flush_plasticity(std::string& err)
{
    if (dense ? launch_flush_dense(P, L, stream) : launch_stdp_flush(P, L, stream)) {
        err = cuda_msg("plasticity flush", cudaGetLastError());
        return NC_ERR_CUDA;
    }
    return NC_OK;
}

int Engine::set_form(bool to_dense, std::string& err)
{
    if (to_dense == dense) return NC_OK;
    if (!both || slots.size() != 1) {
        err = "this network holds the tables of one form only (create it with NC_STEP_AUTO)";
        return NC_ERR_UNSUPPORTED;
    }
    int rc = flush_plasticity(err);
    if (rc != NC_OK) return rc;
    rc = to_dense ? launch_form_to_dense(P, 0, slots[0].s, stream)
                  : launch_form_to_event(P, 0, slots[0].s, ring_words_total_, stream);
    if (rc) {
        err = cuda_msg("form switch", cudaGetLastError());
        return NC_ERR_CUDA;
    }
    release_graph();
    dense = to_dense;
    if (dense) prepare_dense_launch();
    return sync(err);
}

int Engine::sync(std::string& err)
{
    NC_CK(cudaStreamSynchronize(stream));
    uint32_t dev_err = 0;
    NC_CK(cudaMemcpy(&dev_err, P.dev_err, sizeof(dev_err), cudaMemcpyDeviceToHost));
    if (dev_err) {
        err = "a device wait gave up (code " + std::to_string(dev_err) + ")";
        return NC_ERR_TIMEOUT;
    }
    return NC_OK;
}

template <class F>
static cudaError_t put_field(NcNetDesc* d_nets, int net, size_t offset, const F& value, cudaStream_t s)
{
    return cudaMemcpyAsync((char*)(d_nets + net) + offset, &value, sizeof(F), cudaMemcpyHostToDevice, s);
}

int Engine::set_groups(int net, const std::vector<NcGroupDev>& groups, std::string& err)
{
    if ((int)groups.size() > slots[net].group_cap) {
        err = "too many input groups for this engine";
        return NC_ERR_INVALID;
    }
    if (!groups.empty())
        NC_CK(cudaMemcpyAsync(P.groups + slots[net].group_base, groups.data(), groups.size() * sizeof(NcGroupDev),
                              cudaMemcpyHostToDevice, stream));
    const int32_t ng = (int32_t)groups.size();
    int32_t range[2];
    nc_group_range(groups.data(), ng, range[0], range[1]);
    static_assert(offsetof(NcNetDesc, group_hi) == offsetof(NcNetDesc, group_lo) + sizeof(int32_t), "range");
    NC_CK(cudaMemcpyAsync((char*)(P.nets + net) + offsetof(NcNetDesc, group_lo), range, sizeof(range),
                          cudaMemcpyHostToDevice, stream));
    NC_CK(put_field(P.nets, net, offsetof(NcNetDesc, n_groups), ng, stream));
    NC_CK(cudaStreamSynchronize(stream));
    return NC_OK;
}

int Engine::set_rates(int net, float lr, float pre_factor, float post_factor, std::string& err)
{
    // plasticity still pending from the last step belongs to the old rates
    const int rc = flush_plasticity(err);
    if (rc != NC_OK) return rc;
    NC_CK(put_field(P.nets, net, offsetof(NcNetDesc, lr), lr, stream));
    NC_CK(put_field(P.nets, net, offsetof(NcNetDesc, pre_factor), pre_factor, stream));
    NC_CK(put_field(P.nets, net, offsetof(NcNetDesc, post_factor), post_factor, stream));
    NC_CK(cudaStreamSynchronize(stream));
    return NC_OK;
}

int Engine::force_fire(int net, const int32_t* ids, int count, std::string& err)
{
    if (count <= 0) return NC_OK;
    if (count > ids_cap_) {
        if (d_ids_) {
            NC_CK(cudaStreamSynchronize(stream));
            cudaFree(d_ids_);
            d_ids_ = nullptr;
        }
        const int cap = std::max(count, 1024);
        NC_CK(cudaMalloc(&d_ids_, sizeof(int32_t) * cap));
        ids_cap_ = cap;
    }
    NC_CK(cudaMemcpyAsync(d_ids_, ids, sizeof(int32_t) * count, cudaMemcpyHostToDevice, stream));
    if (launch_force_bits(P, net, d_ids_, count, stream)) {
        err = cuda_msg("force bits", cudaGetLastError());
        return NC_ERR_CUDA;
    }
    NC_CK(cudaStreamSynchronize(stream));
    return NC_OK;
}

int Engine::set_raster(int net, uint32_t* d_raster, int32_t t0, int32_t len, std::string& err)
{
    NC_CK(put_field(P.nets, net, offsetof(NcNetDesc, raster), d_raster, stream));
    NC_CK(put_field(P.nets, net, offsetof(NcNetDesc, raster_t0), t0, stream));
    NC_CK(put_field(P.nets, net, offsetof(NcNetDesc, raster_len), len, stream));
    NC_CK(cudaStreamSynchronize(stream));
    return NC_OK;
}

int Engine::read_stats(int net, unsigned long long out[4], std::string& err)
{
    NC_CK(cudaMemcpyAsync(out, d_stats_ + 4 * net, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream));
    NC_CK(cudaStreamSynchronize(stream));
    return NC_OK;
}

int Engine::read_desc(int net, NcNetDesc* out, std::string& err)
{
    NC_CK(cudaMemcpyAsync(out, P.nets + net, sizeof(NcNetDesc), cudaMemcpyDeviceToHost, stream));
    NC_CK(cudaStreamSynchronize(stream));
    return NC_OK;
}

}  // namespace nc

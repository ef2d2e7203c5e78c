// nc_serve.cu — the served form (nc_server_* in neucor_gb300.h).
//
// Device memory is one set of fixed-capacity pools (the layout of nc_engine.cuh) carved
// from the configured budget.  A submitted request is prepared on a builder thread
// (the same host layout as nc_create), then the scheduler thread admits it as soon as
// a network slot and room in every pool are free: its arrays are uploaded into free
// ranges, its descriptor is activated and its tiles join the tile table.  Between
// admissions the scheduler replays a captured CUDA graph of `steps_per_batch` launch
// pairs; every resident network advances one step per pair until its horizon, so
// networks admitted at different times share the same launches.  A network that
// reached its horizon has its plasticity flushed, its counters (and, if kept, weights
// and potentials) copied out, and its ranges and slot released.
//
// The kernels read the tile count from device memory, so the graph stays valid while
// the resident set changes; nothing is shared between networks, so each computes the
// bits it computes alone.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "nc_pool.h"

namespace {

int sfail(int code, const std::string& msg) { return nc::set_last_error(code, msg); }

// First-fit allocator over [0, capacity) with coalescing.
class RangeAlloc {
public:
    void reset(int64_t cap)
    {
        free_.clear();
        cap_ = cap;
        if (cap > 0) free_[0] = cap;
    }
    int64_t alloc(int64_t len, int64_t align = 1)
    {
        if (len <= 0) return 0;
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            const int64_t s0 = it->first, e0 = it->first + it->second;
            const int64_t start = (s0 + align - 1) / align * align;
            if (start + len > e0) continue;
            free_.erase(it);
            if (start > s0) free_[s0] = start - s0;
            if (start + len < e0) free_[start + len] = e0 - (start + len);
            return start;
        }
        return -1;
    }
    void release(int64_t start, int64_t len)
    {
        if (len <= 0) return;
        auto it = free_.emplace(start, len).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }

private:
    std::map<int64_t, int64_t> free_;
    int64_t cap_ = 0;
};

struct Request {
    int64_t id = 0;
    nc_net_spec spec{};
    // a kNN network described by its parameters (nc_server_submit_knn): built by the
    // builder thread, which holds its arrays only while it prepares the request
    bool knn = false;
    int32_t knn_k = 0;
    float knn_density = 0.0f;
    uint64_t knn_seed = 0;
    std::vector<float> xyz, weight, length;
    std::vector<int32_t> from, to;
    std::vector<uint8_t> inh;
    std::vector<nc_group> groups;
    double submit_s = 0;
};

struct Resident {
    int64_t id = 0;
    nc::NetHost host;
    int32_t horizon = 0;
    double submit_s = 0, admit_s = 0;
    int32_t slot = -1;
    int64_t neuron0 = -1, ptr0 = -1, word0 = -1, syn0 = -1, ring0 = -1, table0 = -1;
    int64_t syn_len = 0, ring_len = 0, table_len = 0, words = 0;
    int64_t bytes = 0;
    int64_t steps_done = 0;
    int status = NC_OK;
    std::string err;
};

struct Kept {
    std::vector<float> weights, potentials;
};

constexpr int kGroupsPerNet = 16;
constexpr int64_t kBuiltHostCap = 8ll << 30;
// host bytes of a prepared request's tables (CSC, CSR, weights, maps)
int64_t host_bytes(const nc::NetHost& h) { return h.s * 64 + (int64_t)h.n * 64; }
// per synapse: w t_arr term inh | out_* last_arr (event form) or csc_pre csc_dl la_c (dense)
constexpr double kSynBytesEvent = 4 + 4 + 8 + 4 + 4 + 2 + 4 + 4 + 0.125;
constexpr double kSynBytesDense = 4 + 4 + 8 + 4 + 4 + 2 + 4 + 0.125 + 0.125;  // + csc_post, window bit
constexpr double kNeuronBytes = 4 * 6 + 16 + 20 + 0.5 + 0.25;         // state, fired list, pointers, bitsets, tiles

}  // namespace

struct nc_server {
    nc_server_config cfg{};
    int device = 0;
    cudaStream_t stream = nullptr;
    NcPools P{};
    nc::LaunchShape L{};
    std::vector<void*> allocs;
    int64_t syn_cap = 0, neuron_cap = 0, ptr_cap = 0, word_cap = 0, ring_cap = 0, table_cap = 0, tile_cap = 0;
    bool dense = true;
    double syn_bytes = kSynBytesDense;
    RangeAlloc a_neuron, a_ptr, a_word, a_syn, a_ring, a_table;
    std::vector<int32_t> free_slots;
    unsigned long long* d_stats = nullptr;
    int32_t* d_ntiles = nullptr;
    int32_t* d_nspans = nullptr;
    int64_t span_cap = 0;
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;

    std::mutex mu;
    std::condition_variable cv, cv_done;
    bool stop = false;
    int64_t next_id = 1;
    std::deque<std::unique_ptr<Request>> todo;              // awaiting a builder
    std::map<int64_t, std::unique_ptr<Resident>> built;     // prepared, awaiting admission
    // host memory the prepared, unadmitted requests hold; builders pause above
    // kBuiltHostCap so that a burst of submissions cannot fill the host
    int64_t built_host_bytes = 0;
    std::vector<nc_request_done> finished;                  // not yet polled
    std::map<int64_t, Kept> kept;
    nc_server_stats st{};
    int64_t outstanding = 0;                                // submitted, not finished
    std::vector<std::thread> builders;
    std::thread scheduler;
    std::chrono::steady_clock::time_point t0;

    std::vector<std::unique_ptr<Resident>> active;  // scheduler thread only

    double now() const
    {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    ~nc_server();
    int init(std::string& err);
    void builder_loop();
    void scheduler_loop();
    int admit(Resident& r, std::string& err);
    int retire(Resident& r, std::string& err);
    int upload_tiles(std::string& err);
    int capture(std::string& err);
};

#define S_CK(call)                                                   \
    do {                                                             \
        cudaError_t e_ = (call);                                     \
        if (e_ != cudaSuccess) {                                     \
            err = nc::cuda_msg(#call, e_);                           \
            return e_ == cudaErrorMemoryAllocation ? NC_ERR_NOMEM : NC_ERR_CUDA; \
        }                                                            \
    } while (0)

template <class T>
static int dev_alloc(nc_server* s, T** p, int64_t count, std::string& err)
{
    void* q = nullptr;
    const size_t bytes = (size_t)std::max<int64_t>(1, count) * sizeof(T);
    S_CK(cudaMalloc(&q, bytes));
    s->allocs.push_back(q);
    S_CK(cudaMemsetAsync(q, 0, bytes, s->stream));
    *p = (T*)q;
    return NC_OK;
}

int nc_server::init(std::string& err)
{
    S_CK(cudaGetDevice(&device));
    S_CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    S_CK(cudaEventCreate(&ev0));
    S_CK(cudaEventCreate(&ev1));
    int sms = 0;
    S_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    // pool capacities carved from the budget: the trace/AP tables first (~600 floats per
    // network at dt = 1 ms), then ~80% (event form) or ~87% (dense form, which keeps no
    // ring buffers) of the rest for synapse arrays, then neurons (fan-out of at least 16
    // assumed) and the event form's ring buffers
    const double budget = (double)cfg.memory_budget_bytes;
    dense = cfg.step_mode == NC_STEP_DENSE;
    syn_bytes = dense ? kSynBytesDense : kSynBytesEvent;
    const int32_t nets = cfg.max_networks;
    table_cap = (int64_t)nets * 8192 + 65536;
    const double avail = budget - 4.0 * (double)table_cap;
    syn_cap = avail > 0 ? (int64_t)((dense ? 0.87 : 0.80) * avail / syn_bytes) / 32 * 32 : 0;
    neuron_cap = std::max<int64_t>(1024, syn_cap / 16);
    ptr_cap = neuron_cap + nets;
    word_cap = neuron_cap / 32 + nets;
    tile_cap = word_cap;
    ring_cap = dense ? 0 : (int64_t)(0.07 * budget / 4.0);
    const double used = syn_cap * syn_bytes + neuron_cap * kNeuronBytes + ring_cap * 4.0 + table_cap * 4.0;
    if (syn_cap < 32 || used > 1.05 * budget) {
        err = "memory budget too small";
        return NC_ERR_BUDGET;
    }
    int rc = NC_OK;
#define S_AL(ptr, T, n)                         \
    if ((rc = dev_alloc(this, &(ptr), (n), err))) return rc;
    S_AL(P.pot, float, neuron_cap);
    S_AL(P.lf, int32_t, neuron_cap);
    S_AL(P.firings, uint32_t, neuron_cap);
    S_AL(P.act_start, int32_t, neuron_cap);
    S_AL(P.orig_id, int32_t, neuron_cap);
    S_AL(P.slot_of, int32_t, neuron_cap);
    S_AL(P.in_ptr, int64_t, ptr_cap);
    S_AL(P.w, float, syn_cap);
    S_AL(P.inh, uint32_t, syn_cap / 32 + 1);
    S_AL(P.t_arr, int32_t, syn_cap);
    S_AL(P.term, double, syn_cap);
    if (dense) {
        span_cap = syn_cap / (32 * NC_SPAN_CHUNKS) + nets;
        S_AL(P.csc_pre, int32_t, syn_cap);
        S_AL(P.csc_post, int32_t, syn_cap);
        S_AL(P.csc_dl, uint16_t, syn_cap);
        S_AL(P.la_c, int32_t, syn_cap);
        S_AL(P.pst, float, neuron_cap);
        S_AL(P.win, uint32_t, syn_cap / 32 + 1);
        S_AL(P.spans, NcTile, span_cap);
        S_AL(d_nspans, int32_t, 1);
    } else {
        S_AL(P.out_ptr, int64_t, ptr_cap);
        S_AL(P.ring_off, int32_t, ptr_cap);
        S_AL(P.out_post, int32_t, syn_cap);
        S_AL(P.out_csc, int32_t, syn_cap);
        S_AL(P.out_delay, int16_t, syn_cap);
        S_AL(P.out_ringpos, uint32_t, syn_cap);
        S_AL(P.last_arr, int32_t, syn_cap);
        S_AL(P.ring, uint32_t, ring_cap);
    }
    P.total_words = word_cap;
    S_AL(P.fired, uint32_t, 2 * word_cap);
    S_AL(P.forced, uint32_t, 2 * word_cap);
    S_AL(P.ufire, uint32_t, 2 * word_cap);
    P.fired_cap = dense ? 0 : neuron_cap;
    if (!dense) S_AL(P.fired_list, int2, 2 * neuron_cap);
    S_AL(P.fired_count, int32_t, 2);
    S_AL(P.tables, float, table_cap);
    S_AL(P.groups, NcGroupDev, (int64_t)nets * kGroupsPerNet);
    S_AL(P.nets, NcNetDesc, nets);
    S_AL(P.tiles, NcTile, tile_cap);
    S_AL(P.tick, int32_t, 1);
    S_AL(P.done_ctr, uint32_t, 1);
    S_AL(P.dev_err, uint32_t, 1);
    S_AL(d_stats, unsigned long long, 4 * (int64_t)nets);
    S_AL(d_ntiles, int32_t, 1);
#undef S_AL
    P.n_nets = nets;
    P.n_tiles = 0;
    P.n_tiles_dev = d_ntiles;
    P.n_spans = 0;
    P.n_spans_dev = d_nspans;
    a_neuron.reset(neuron_cap);
    a_ptr.reset(ptr_cap);
    a_word.reset(word_cap);
    a_syn.reset(syn_cap);
    a_ring.reset(ring_cap);
    a_table.reset(table_cap);
    for (int32_t q = nets - 1; q >= 0; --q) free_slots.push_back(q);
    L.neuron_block = dense ? NC_DNEURON_BLOCK : 256;
    L.launch_block = 256;
    L.launch_blocks = std::max(1, sms * NC_LAUNCH_MIN_BLOCKS);
    L.dense_blocks = 0;  // the synapse pass's persistent grid (its warps stride the span table)
    S_CK(cudaStreamSynchronize(stream));
    return capture(err);
}

int nc_server::capture(std::string& err)
{
    // the neuron update strides over the tile table, so its grid need not follow it
    NcPools G = P;
    G.n_tiles = (int32_t)std::min<int64_t>(tile_cap, 1 << 30);
    // likewise the synapse pass strides over the span table (its kernels read the live
    // counts from the device): grids are sized from the capacities
    G.n_spans = (int32_t)std::min<int64_t>(span_cap, 1 << 30);
    nc::LaunchShape shape = L;
    cudaGraph_t g = nullptr;
    if (dense) nc::prepare_dense_launch();
    S_CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    int rc = 0;
    const int nb_tiles = 152 * 16 * (shape.neuron_block / 32);  // grid of the captured neuron update
    NcPools Gg = G;
    Gg.n_tiles = (int32_t)std::min<int64_t>(G.n_tiles, nb_tiles);
    for (int k = 0; k < cfg.steps_per_batch && rc == 0; ++k) {
        if (dense) {
            rc |= nc::launch_dense_synapses(G, shape, stream);
            rc |= nc::launch_dense_neurons(Gg, shape, stream);
        } else {
            rc |= nc::launch_neuron_step(Gg, shape, stream);
            rc |= nc::launch_spike_launch(G, shape, stream);
        }
    }
    cudaError_t e = cudaStreamEndCapture(stream, &g);
    if (rc != 0 || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        err = nc::cuda_msg("server graph capture", e != cudaSuccess ? e : cudaGetLastError());
        return NC_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        graph = nullptr;
        err = nc::cuda_msg("cudaGraphInstantiate", e);
        return NC_ERR_CUDA;
    }
    return NC_OK;
}

nc_server::~nc_server()
{
    {
        std::lock_guard<std::mutex> lk(mu);
        stop = true;
    }
    cv.notify_all();
    for (auto& t : builders)
        if (t.joinable()) t.join();
    if (scheduler.joinable()) scheduler.join();
    if (graph) cudaGraphExecDestroy(graph);
    if (stream) cudaStreamSynchronize(stream);
    for (void* p : allocs) cudaFree(p);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
}

void nc_server::builder_loop()
{
    for (;;) {
        std::unique_ptr<Request> rq;
        {
            std::unique_lock<std::mutex> lk(mu);
            cv.wait(lk, [&] { return stop || (!todo.empty() && built_host_bytes < kBuiltHostCap); });
            if (stop && todo.empty()) return;
            rq = std::move(todo.front());
            todo.pop_front();
        }
        auto r = std::make_unique<Resident>();
        r->id = rq->id;
        r->submit_s = rq->submit_s;
        r->horizon = rq->spec.horizon;
        nc_net_spec& sp = rq->spec;
        std::string err;
        int rc = NC_OK;
        if (rq->knn) {
            const size_t n = (size_t)sp.n_neurons, m = n * (size_t)rq->knn_k;
            rq->xyz.resize(3 * n);
            rq->from.resize(m);
            rq->to.resize(m);
            rq->weight.resize(m);
            rc = nc_build_knn(sp.n_neurons, rq->knn_k, rq->knn_density, rq->knn_seed, rq->xyz.data(), rq->from.data(),
                              rq->to.data(), rq->weight.data());
            if (rc != NC_OK) err = "bad kNN request";
            sp.n_synapses = (int64_t)m;
        }
        if (rc == NC_OK)
            rc = nc::build_net(sp.n_neurons, rq->xyz.empty() ? nullptr : rq->xyz.data(), sp.n_synapses,
                               rq->from.data(), rq->to.data(), rq->weight.data(),
                               rq->length.empty() ? nullptr : rq->length.data(), rq->inh.empty() ? nullptr : rq->inh.data(),
                               sp.params, r->host, err);
        if (rq->knn) {  // the arrays are not needed past the host layout
            std::vector<float>().swap(rq->xyz);
            std::vector<int32_t>().swap(rq->from);
            std::vector<int32_t>().swap(rq->to);
            std::vector<float>().swap(rq->weight);
        }
        if (rc == NC_OK) rc = nc::set_groups(r->host, (int32_t)rq->groups.size(), rq->groups.data(), err);
        if (rc == NC_OK && (int)r->host.groups.size() > kGroupsPerNet) {
            rc = NC_ERR_INVALID;
            err = "more than 16 input groups";
        }
        if (rc == NC_OK) {
            const nc::NetHost& h = r->host;
            r->syn_len = (h.s + 31) / 32 * 32;
            r->ring_len = dense ? 0 : (int64_t)h.ring_slots * h.ring_words;
            r->table_len = (int64_t)h.tables.size();
            r->words = (h.n + 31) / 32;
            if (h.n > neuron_cap || r->syn_len > syn_cap || r->ring_len > ring_cap || r->table_len > table_cap) {
                rc = NC_ERR_BUDGET;
                err = "network larger than the server's memory budget";
            }
            r->bytes = (int64_t)(r->syn_len * syn_bytes + h.n * kNeuronBytes + r->ring_len * 4.0 + r->table_len * 4.0);
        }
        r->status = rc;
        r->err = err;
        {
            std::lock_guard<std::mutex> lk(mu);
            built_host_bytes += host_bytes(r->host);
            built.emplace(r->id, std::move(r));
        }
        cv.notify_all();
    }
}

template <class T>
static cudaError_t put(T* dev, const std::vector<T>& v, int64_t off, cudaStream_t s)
{
    if (v.empty()) return cudaSuccess;
    return cudaMemcpyAsync(dev + off, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s);
}

int nc_server::admit(Resident& r, std::string& err)
{
    const nc::NetHost& h = r.host;
    const int64_t nb = a_neuron.alloc(h.n), pb = a_ptr.alloc(h.n + 1), wb = a_word.alloc(r.words),
                  sb = a_syn.alloc(r.syn_len, 32), rb = a_ring.alloc(r.ring_len), tb = a_table.alloc(r.table_len);
    if (free_slots.empty() || nb < 0 || pb < 0 || wb < 0 || sb < 0 || rb < 0 || tb < 0) {
        if (nb >= 0) a_neuron.release(nb, h.n);
        if (pb >= 0) a_ptr.release(pb, h.n + 1);
        if (wb >= 0) a_word.release(wb, r.words);
        if (sb >= 0) a_syn.release(sb, r.syn_len);
        if (rb >= 0) a_ring.release(rb, r.ring_len);
        if (tb >= 0) a_table.release(tb, r.table_len);
        return 1;  // does not fit now
    }
    r.slot = free_slots.back();
    free_slots.pop_back();
    r.neuron0 = nb;
    r.ptr0 = pb;
    r.word0 = wb;
    r.syn0 = sb;
    r.ring0 = rb;
    r.table0 = tb;
    // upload: the same per-network layout as the static engine, state reset
    std::vector<float> pot((size_t)h.n, -70.0f);
    std::vector<int32_t> never_n((size_t)h.n, NC_NEVER), never_s((size_t)h.s, NC_NEVER);
    std::vector<int64_t> inp(h.in_ptr), outp(h.out_ptr);
    for (auto& v : inp) v += sb;
    for (auto& v : outp) v += sb;
    S_CK(put(P.pot, pot, nb, stream));
    S_CK(put(P.lf, never_n, nb, stream));
    S_CK(cudaMemsetAsync(P.firings + nb, 0, sizeof(uint32_t) * h.n, stream));
    S_CK(cudaMemsetAsync(P.act_start + nb, 0, sizeof(int32_t) * h.n, stream));
    S_CK(put(P.orig_id, h.orig_id, nb, stream));
    S_CK(put(P.slot_of, h.slot_of, nb, stream));
    S_CK(put(P.in_ptr, inp, pb, stream));
    S_CK(put(P.w, h.w, sb, stream));
    S_CK(put(P.inh, h.inh_bits, sb / 32, stream));
    S_CK(put(P.t_arr, never_s, sb, stream));
    if (dense) {
        S_CK(put(P.csc_pre, h.csc_pre, sb, stream));
        S_CK(put(P.csc_post, h.csc_post, sb, stream));
        S_CK(put(P.csc_dl, h.csc_dl, sb, stream));
        S_CK(put(P.la_c, never_s, sb, stream));
        S_CK(cudaMemsetAsync(P.win + sb / 32, 0, sizeof(uint32_t) * (r.syn_len / 32), stream));
    } else {
        S_CK(put(P.out_ptr, outp, pb, stream));
        S_CK(put(P.ring_off, h.ring_off, pb, stream));
        S_CK(put(P.last_arr, never_s, sb, stream));
        S_CK(put(P.out_post, h.out_post, sb, stream));
        S_CK(put(P.out_csc, h.out_csc, sb, stream));
        S_CK(put(P.out_delay, h.out_delay, sb, stream));
        S_CK(put(P.out_ringpos, h.out_ringpos, sb, stream));
        S_CK(cudaMemsetAsync(P.ring + rb, 0, sizeof(uint32_t) * r.ring_len, stream));
    }
    for (int par = 0; par < 2; ++par) {
        S_CK(cudaMemsetAsync(P.fired + par * P.total_words + wb, 0, sizeof(uint32_t) * r.words, stream));
        S_CK(cudaMemsetAsync(P.forced + par * P.total_words + wb, 0, sizeof(uint32_t) * r.words, stream));
        S_CK(cudaMemsetAsync(P.ufire + par * P.total_words + wb, 0, sizeof(uint32_t) * r.words, stream));
    }
    S_CK(put(P.tables, h.tables, tb, stream));
    if (!h.groups.empty()) S_CK(put(P.groups, h.groups, (int64_t)r.slot * kGroupsPerNet, stream));
    S_CK(cudaMemsetAsync(d_stats + 4 * (int64_t)r.slot, 0, 4 * sizeof(unsigned long long), stream));
    NcNetDesc d;
    std::memset(&d, 0, sizeof(d));
    d.t = 1;
    d.t_end = r.horizon;
    d.stdp_done = 0;
    d.n = h.n;
    d.neuron_base = (int32_t)nb;
    d.ptr_base = (int32_t)pb;
    d.word_base = (int32_t)wb;
    d.n_words = (int32_t)r.words;
    d.syn_base = sb;
    d.ring_base = rb;
    d.ring_words = h.ring_words;
    d.ring_mask = h.ring_slots - 1;
    d.kc = h.kc;
    d.bg_period = h.bg_period;
    d.key0 = (uint32_t)h.p.seed;
    d.key1 = (uint32_t)(h.p.seed >> 32);
    d.table_base = (int32_t)tb;
    d.tab_pre_len = h.tab_pre_len;
    d.tab_post_len = h.tab_post_len;
    d.ap_base = (int32_t)(tb + h.tab_pre_len + h.tab_post_len);
    d.group_base = r.slot * kGroupsPerNet;
    d.n_groups = (int32_t)h.groups.size();
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
    d.stats = d_stats + 4 * (int64_t)r.slot;
    S_CK(cudaMemcpyAsync(P.nets + r.slot, &d, sizeof(d), cudaMemcpyHostToDevice, stream));
    if (nc::launch_background_prologue(P, r.slot, h.n, stream)) {
        err = nc::cuda_msg("background prologue", cudaGetLastError());
        return NC_ERR_CUDA;
    }
    S_CK(cudaStreamSynchronize(stream));  // the host vectors above must outlive the copies
    return NC_OK;
}

int nc_server::retire(Resident& r, std::string& err)
{
    const nc::NetHost& h = r.host;
    const int32_t inactive = 0;
    S_CK(cudaMemcpyAsync((char*)(P.nets + r.slot) + offsetof(NcNetDesc, active), &inactive, sizeof(inactive),
                         cudaMemcpyHostToDevice, stream));
    a_neuron.release(r.neuron0, h.n);
    a_ptr.release(r.ptr0, h.n + 1);
    a_word.release(r.word0, r.words);
    a_syn.release(r.syn0, r.syn_len);
    a_ring.release(r.ring0, r.ring_len);
    a_table.release(r.table0, r.table_len);
    free_slots.push_back(r.slot);
    r.slot = -1;
    return NC_OK;
}

int nc_server::upload_tiles(std::string& err)
{
    std::vector<NcTile> tiles;
    for (const auto& r : active)
        for (int32_t f = 0; f < r->host.n; f += 32) tiles.push_back(NcTile{r->slot, f});
    if ((int64_t)tiles.size() > tile_cap) {
        err = "tile table overflow";
        return NC_ERR_INVALID;
    }
    const int32_t n = (int32_t)tiles.size();
    if (n) S_CK(cudaMemcpyAsync(P.tiles, tiles.data(), tiles.size() * sizeof(NcTile), cudaMemcpyHostToDevice, stream));
    S_CK(cudaMemcpyAsync(d_ntiles, &n, sizeof(n), cudaMemcpyHostToDevice, stream));
    std::vector<NcTile> spans;
    if (dense) {
        for (const auto& r : active) {
            const int32_t chunks = (int32_t)((r->host.s + 31) / 32);
            for (int32_t c = 0; c < chunks; c += NC_SPAN_CHUNKS) spans.push_back(NcTile{r->slot, c});
        }
        if ((int64_t)spans.size() > span_cap) {
            err = "span table overflow";
            return NC_ERR_INVALID;
        }
        const int32_t ns = (int32_t)spans.size();
        if (ns)
            S_CK(cudaMemcpyAsync(P.spans, spans.data(), spans.size() * sizeof(NcTile), cudaMemcpyHostToDevice, stream));
        S_CK(cudaMemcpyAsync(d_nspans, &ns, sizeof(ns), cudaMemcpyHostToDevice, stream));
        P.n_spans = ns;
    }
    S_CK(cudaStreamSynchronize(stream));
    P.n_tiles = n;
    return NC_OK;
}

void nc_server::scheduler_loop()
{
    cudaSetDevice(device);
    const int G = cfg.steps_per_batch;
    for (;;) {
        std::string err;
        // admission: prepared requests in submission order, each as soon as it fits
        std::vector<std::unique_ptr<Resident>> rejected;
        bool changed = false;
        {
            std::unique_lock<std::mutex> lk(mu);
            if (active.empty())
                cv.wait(lk, [&] { return stop || !built.empty(); });
            if (stop) return;  // destroy abandons resident and queued work
            for (auto it = built.begin(); it != built.end();) {
                Resident& r = *it->second;
                if (r.status != NC_OK) {
                    built_host_bytes -= host_bytes(r.host);
                    rejected.push_back(std::move(it->second));
                    it = built.erase(it);
                    continue;
                }
                const int rc = admit(r, err);
                if (rc == 1) {
                    ++it;
                    continue;
                }
                built_host_bytes -= host_bytes(r.host);
                if (rc != NC_OK) {
                    r.status = rc;
                    r.err = err;
                    rejected.push_back(std::move(it->second));
                    it = built.erase(it);
                    continue;
                }
                r.admit_s = now();
                st.admitted++;
                st.resident_bytes += r.bytes;
                active.push_back(std::move(it->second));
                it = built.erase(it);
                changed = true;
            }
            st.peak_resident_bytes = std::max(st.peak_resident_bytes, st.resident_bytes);
            st.peak_resident_networks = std::max<int64_t>(st.peak_resident_networks, (int64_t)active.size());
            for (auto& r : rejected) {
                nc_request_done d{};
                d.request_id = r->id;
                d.status = r->status;
                d.n_neurons = r->host.n;
                d.horizon = r->horizon;
                d.submit_s = r->submit_s;
                d.admit_s = d.done_s = now();
                finished.push_back(d);
                st.rejected++;
                st.finished++;
                outstanding--;
            }
        }
        if (!rejected.empty()) cv_done.notify_all();
        if (changed || !rejected.empty()) cv.notify_all();  // builders paused on the host cap
        if (changed && upload_tiles(err) != NC_OK) return;
        if (active.empty()) continue;
        // one batch of G launch pairs over every resident network
        cudaEventRecord(ev0, stream);
        if (cudaGraphLaunch(graph, stream) != cudaSuccess) return;
        cudaEventRecord(ev1, stream);
        cudaEventSynchronize(ev1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, ev0, ev1);
        // retire networks that reached their horizon
        std::vector<std::unique_ptr<Resident>> done;
        for (auto it = active.begin(); it != active.end();) {
            (*it)->steps_done = std::min<int64_t>((*it)->steps_done + G, (*it)->horizon);
            if ((*it)->steps_done >= (*it)->horizon) {
                done.push_back(std::move(*it));
                it = active.erase(it);
            } else {
                ++it;
            }
        }
        if (!done.empty()) {
            NcPools F = P;  // flush launched directly with the current tile count
            F.n_tiles_dev = nullptr;
            F.n_spans_dev = nullptr;
            if (dense ? nc::launch_flush_dense(F, L, stream) : nc::launch_stdp_flush(F, L, stream)) return;
            cudaStreamSynchronize(stream);
        }
        std::vector<nc_request_done> out;
        for (auto& r : done) {
            nc_request_done d{};
            d.request_id = r->id;
            d.status = NC_OK;
            d.n_neurons = r->host.n;
            d.horizon = r->horizon;
            d.n_synapses = r->host.s;
            d.submit_s = r->submit_s;
            d.admit_s = r->admit_s;
            unsigned long long s4[4];
            cudaMemcpyAsync(s4, d_stats + 4 * (int64_t)r->slot, sizeof(s4), cudaMemcpyDeviceToHost, stream);
            Kept k;
            if (cfg.keep_results) {
                const nc::NetHost& h = r->host;
                std::vector<float> w((size_t)h.s), pot((size_t)h.n);
                cudaMemcpyAsync(w.data(), P.w + r->syn0, sizeof(float) * h.s, cudaMemcpyDeviceToHost, stream);
                cudaMemcpyAsync(pot.data(), P.pot + r->neuron0, sizeof(float) * h.n, cudaMemcpyDeviceToHost, stream);
                cudaStreamSynchronize(stream);
                k.weights.resize((size_t)h.n_input);
                for (int64_t q = 0; q < h.n_input; ++q) {
                    const int64_t c = h.input_to_csc[(size_t)q];
                    k.weights[(size_t)q] = c < 0 ? NAN : w[(size_t)c];
                }
                k.potentials.resize((size_t)h.n);
                nc::to_caller_order(h, pot.data(), k.potentials.data());
            }
            cudaStreamSynchronize(stream);
            d.stats.fires = (int64_t)s4[0];
            d.stats.launched = (int64_t)s4[1];
            d.stats.dropped = (int64_t)s4[2];
            d.stats.steps = (int64_t)s4[3];
            retire(*r, err);
            d.done_s = now();
            out.push_back(d);
            if (cfg.keep_results) {
                std::lock_guard<std::mutex> lk(mu);
                kept.emplace(r->id, std::move(k));
            }
        }
        if (!done.empty() && upload_tiles(err) != NC_OK) return;
        {
            std::lock_guard<std::mutex> lk(mu);
            st.steps_run += G;
            st.device_busy_s += ms / 1000.0;
            for (auto& d : out) {
                finished.push_back(d);
                st.finished++;
                outstanding--;
            }
            for (auto& r : done) st.resident_bytes -= r->bytes;
        }
        if (!out.empty()) cv_done.notify_all();
    }
}

extern "C" {

int nc_server_create(const nc_server_config* config, nc_server** out)
{
    if (!config || !out) return sfail(NC_ERR_INVALID, "null argument");
    *out = nullptr;
    if (config->memory_budget_bytes <= 0 || config->max_networks < 1 || config->max_networks > 65536 ||
        config->steps_per_batch < 1 || config->steps_per_batch > 4096 || config->build_threads < 1 ||
        config->build_threads > 256 || (config->step_mode != NC_STEP_DENSE && config->step_mode != NC_STEP_EVENT))
        return sfail(NC_ERR_INVALID, "bad server configuration");
    int devices = 0;
    if (cudaGetDeviceCount(&devices) != cudaSuccess || devices == 0)
        return sfail(NC_ERR_NODEVICE, "no CUDA device: the GB300 step has no CPU fallback");
    nc_server* s = new (std::nothrow) nc_server();
    if (!s) return sfail(NC_ERR_NOMEM, "host allocation failed");
    s->cfg = *config;
    s->t0 = std::chrono::steady_clock::now();
    std::string err;
    const int rc = s->init(err);
    if (rc != NC_OK) {
        delete s;
        return sfail(rc, err);
    }
    for (int k = 0; k < config->build_threads; ++k) s->builders.emplace_back([s] { s->builder_loop(); });
    s->scheduler = std::thread([s] { s->scheduler_loop(); });
    *out = s;
    return NC_OK;
}

int nc_server_submit(nc_server* s, const nc_net_spec* sp, int64_t* request_id)
{
    if (!s || !sp || !request_id) return sfail(NC_ERR_INVALID, "null argument");
    if (sp->n_neurons < 0 || sp->n_synapses < 0 || sp->horizon < 0 || sp->n_groups < 0 ||
        (sp->n_synapses > 0 && (!sp->syn_from || !sp->syn_to || !sp->syn_weight)) ||
        (sp->n_groups > 0 && !sp->groups))
        return sfail(NC_ERR_INVALID, "bad network spec");
    auto rq = std::make_unique<Request>();
    rq->spec = *sp;
    const size_t n = (size_t)sp->n_neurons, m = (size_t)sp->n_synapses;
    if (sp->xyz) rq->xyz.assign(sp->xyz, sp->xyz + 3 * n);
    rq->from.assign(sp->syn_from, sp->syn_from + m);
    rq->to.assign(sp->syn_to, sp->syn_to + m);
    rq->weight.assign(sp->syn_weight, sp->syn_weight + m);
    if (sp->syn_length) rq->length.assign(sp->syn_length, sp->syn_length + m);
    if (sp->syn_inhibitory) rq->inh.assign(sp->syn_inhibitory, sp->syn_inhibitory + m);
    if (sp->n_groups) rq->groups.assign(sp->groups, sp->groups + sp->n_groups);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        rq->id = s->next_id++;
        rq->submit_s = s->now();
        *request_id = rq->id;
        s->todo.push_back(std::move(rq));
        s->st.submitted++;
        s->outstanding++;
    }
    s->cv.notify_all();
    return NC_OK;
}

int nc_server_submit_knn(nc_server* s, int32_t n, int32_t k, float density, uint64_t knn_seed,
                         const nc_params* params, int32_t n_groups, const nc_group* groups, int32_t horizon,
                         int64_t* request_id)
{
    if (!s || !params || !request_id) return sfail(NC_ERR_INVALID, "null argument");
    if (n < 2 || k < 1 || k >= n || !(density > 0.0f) || horizon < 0 || n_groups < 0 || (n_groups > 0 && !groups))
        return sfail(NC_ERR_INVALID, "bad kNN request (need 1 <= k < n, density > 0)");
    auto rq = std::make_unique<Request>();
    rq->knn = true;
    rq->knn_k = k;
    rq->knn_density = density;
    rq->knn_seed = knn_seed;
    rq->spec.n_neurons = n;
    rq->spec.params = *params;
    rq->spec.horizon = horizon;
    rq->spec.n_groups = n_groups;
    if (n_groups) rq->groups.assign(groups, groups + n_groups);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        rq->id = s->next_id++;
        rq->submit_s = s->now();
        *request_id = rq->id;
        s->todo.push_back(std::move(rq));
        s->st.submitted++;
        s->outstanding++;
    }
    s->cv.notify_all();
    return NC_OK;
}

int nc_server_poll(nc_server* s, nc_request_done* out, int32_t capacity, int32_t* count)
{
    if (!s || !count || (capacity > 0 && !out)) return sfail(NC_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    const int32_t k = (int32_t)std::min<size_t>((size_t)std::max(capacity, 0), s->finished.size());
    for (int32_t q = 0; q < k; ++q) out[q] = s->finished[(size_t)q];
    s->finished.erase(s->finished.begin(), s->finished.begin() + k);
    *count = k;
    return NC_OK;
}

int nc_server_drain(nc_server* s)
{
    if (!s) return sfail(NC_ERR_INVALID, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv_done.wait(lk, [&] { return s->outstanding == 0; });
    return NC_OK;
}

int nc_server_fetch(nc_server* s, int64_t id, float* weights, float* potentials)
{
    if (!s) return sfail(NC_ERR_INVALID, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->kept.find(id);
    if (it == s->kept.end()) return sfail(NC_ERR_INVALID, "no kept result for this request");
    if (weights) std::copy(it->second.weights.begin(), it->second.weights.end(), weights);
    if (potentials) std::copy(it->second.potentials.begin(), it->second.potentials.end(), potentials);
    s->kept.erase(it);
    return NC_OK;
}

int nc_server_get_stats(nc_server* s, nc_server_stats* out)
{
    if (!s || !out) return sfail(NC_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->st;
    return NC_OK;
}

int nc_server_destroy(nc_server* s)
{
    if (!s) return NC_OK;
    cudaSetDevice(s->device);
    delete s;
    return NC_OK;
}

}  // extern "C"

// nc_pool.h — device engine: packs one or more networks into pooled HBM arrays and
// advances them with the step kernels, replaying captured CUDA graphs.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "nc_host.h"

namespace nc {

struct NetSlot {       // host view of one packed net
    int32_t n = 0;
    int64_t s = 0;
    int32_t kc = 3;
    float dt = 1.0f;
    int32_t n_words = 0;
    int64_t syn_base = 0;
    int32_t neuron_base = 0, ptr_base = 0, word_base = 0, group_cap = 0, group_base = 0;
};

class Engine {
public:
    Engine() = default;
    ~Engine();
    Engine(const Engine&) = delete;
    Engine& operator=(const Engine&) = delete;

    // Packs the nets (all starting at step 1) and uploads them.  group_capacity is
    // the number of input-group entries reserved per net.
    // device_synapses: the in-synapse streams (dense form) are written on the device by
    // the caller (nc_build.cu); only the row starts come from the host description.
    int build(const std::vector<const NetHost*>& nets, int group_capacity, std::string& err,
              const std::vector<int32_t>* horizons = nullptr, bool device_synapses = false);
    void set_launch(const LaunchShape& shape, int ticks_per_graph);
    // Runs `ticks` engine steps (every active net advances one step per tick).
    int step(int64_t ticks, std::string& err);
    // Same, timed with CUDA events on the engine stream.
    int step_timed(int64_t ticks, float* ms, std::string& err);
    // Mean device time of one neuron-update and one spike-launch launch over `ticks`
    // individually timed ticks (these ticks also advance the nets).
    // (dense form: the synapse pass and the neuron pass)
    int time_kernels(int ticks, float* neuron_ms, float* launch_ms, std::string& err);
    int flush_plasticity(std::string& err);
    int sync(std::string& err);

    int set_groups(int net, const std::vector<NcGroupDev>& groups, std::string& err);
    int set_rates(int net, float lr, float pre_factor, float post_factor, std::string& err);
    int force_fire(int net, const int32_t* ids, int count, std::string& err);
    int set_raster(int net, uint32_t* d_raster, int32_t t0, int32_t len, std::string& err);
    int read_stats(int net, unsigned long long out[4], std::string& err);
    int read_desc(int net, NcNetDesc* out, std::string& err);

    template <class T>
    int download(T* host, const T* dev, size_t count, std::string& err);

    NcPools P{};
    LaunchShape L{};
    std::vector<NetSlot> slots;
    cudaStream_t stream = nullptr;
    int device = 0;
    int graph_ticks = 32;
    bool dense = true;  // the form the next steps run in: NC_STEP_DENSE (nc_dense.cu) or event
    bool both = false;  // NC_STEP_AUTO: the tables of both forms are on the device
    // Switches a single-net engine built with both forms' tables to the other form
    // between steps (flushes the current form's deferred plasticity, converts the
    // per-synapse arrival state, drops the captured graph).
    int set_form(bool to_dense, std::string& err);
    // Launches one tick of the engine's form on `s` (no graph), the input firers' schedule
    // included.
    int launch_tick(cudaStream_t s);
    // Periodic input firers (replaces the set), their state read and written back; the
    // next step's run-call schedule sees every change.
    int set_firers(const std::vector<NcFirer>& firers, const std::vector<int32_t>& near, std::string& err);
    int read_firers(std::vector<NcFirer>& out, std::string& err);
    int write_firers(const std::vector<NcFirer>& in, std::string& err);

private:
    int capture_graph(std::string& err);
    void release_graph();
    template <class T>
    T* alloc(size_t count, std::string& err);
    std::vector<void*> allocs_;
    cudaGraphExec_t graph_ = nullptr;
    void* firers_buf_ = nullptr;
    void* near_buf_ = nullptr;
    int32_t* d_ids_ = nullptr;
    int ids_cap_ = 0;
    unsigned long long* d_stats_ = nullptr;
    unsigned* d_bar_ = nullptr;  // grid barrier of the fused launch (arrivals, generation)
    int64_t ring_words_total_ = 0;
};

std::string cuda_msg(const char* what, cudaError_t e);
// Records the calling thread's last error (nc_last_error) and returns `code`.
int set_last_error(int code, const std::string& msg);

}  // namespace nc

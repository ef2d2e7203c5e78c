// nc_host.h — host-side network description (built once, uploaded to the GPU).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/neucor_gb300.h"
#include "nc_engine.cuh"

namespace nc {

// One network laid out for the step kernels (see nc_engine.cuh), all indices
// relative to the network.
struct NetHost {
    int32_t n = 0;
    int64_t s = 0;        // synapses kept
    int64_t n_input = 0;  // synapses given
    nc_params p{};
    float dt = 1.0f;
    int32_t kc = 3;
    int32_t ring_slots = 1;
    int32_t ring_words = 0;
    int32_t bg_period = 0;
    int32_t max_delay = 1;
    float leak = 0.5f, c52 = 0.0f;
    double e_term = 0.0;
    std::vector<float> xyz;                 // caller's id order
    std::vector<int32_t> orig_id;           // device slot -> caller's id
    std::vector<int32_t> slot_of;           // caller's id -> device slot
    bool permuted = false;
    // Below, neurons are device slots.  The in-synapses of a target are sorted by the
    // caller's source id; out_delay packs the delay (bits 0-13) and whether the target's
    // caller id is above (bit 14) or below (bit 15) the source's.
    std::vector<int64_t> in_ptr, out_ptr;   // n+1
    std::vector<int32_t> ring_off;          // n+1
    std::vector<float> w;                   // CSC
    std::vector<uint32_t> inh_bits;         // CSC, bit per synapse: Synapse::inhibitory
    std::vector<int32_t> csc_pre, csc_delay;
    std::vector<uint16_t> csc_dl;           // CSC: delay | flags, as out_delay (dense form)
    std::vector<int32_t> csc_post;          // CSC: target slot (dense form)
    std::vector<int32_t> out_post, out_csc;
    std::vector<int16_t> out_delay;
    std::vector<uint32_t> out_ringpos;
    std::vector<int64_t> input_to_csc;      // -1 for ignored duplicates
    std::vector<float> tables;              // pre trace | post trace | AP shape
    int32_t tab_pre_len = 0, tab_post_len = 0, ap_len = 0;
    std::vector<NcGroupDev> groups;
    bool nonneg_terms = true;               // no inhibitory synapse and no negative weight

    int64_t device_bytes() const;
};

// Builds the layout; returns NC_OK or an NC_ERR_* code with `err` set.
int build_net(int32_t n, const float* xyz, int64_t n_syn, const int32_t* from, const int32_t* to,
              const float* weight, const float* length, const uint8_t* inhibitory, const nc_params& p,
              NetHost& out, std::string& err);
bool inhibitory_flag(const NetHost& h, int64_t csc);
int set_groups(NetHost& net, int32_t n_groups, const nc_group* groups, std::string& err);

// Reference arithmetic helpers shared by build and read-back.
float get_dist(const float* a, const float* b);      // coord3::getDist, src/NeuCor.h:16-18
int32_t delay_steps(float length, float dt);          // -1 when it does not fit int16
constexpr int32_t kMaxDelay = (1 << 14) - 1;          // delay bits of out_delay
constexpr int kAfterBit = 14, kBeforeBit = 15;
// Scatters a device-slot-ordered array into the caller's id order.
template <class T>
void to_caller_order(const NetHost& h, const T* slots, T* out)
{
    for (int32_t i = 0; i < h.n; ++i) out[i] = slots[h.slot_of[(size_t)i]];
}
uint32_t rate_threshold(float rate_hz, float dt);

// kNN networks (nc_build_knn, and its device counterpart in nc_build.cu): positions
// uniform in a cube of side (n/density)^(1/3) from Philox stream kStreamPosition,
// weights from kStreamWeight, neighbours searched over a uniform grid of g^3 cells.
constexpr uint32_t kStreamPosition = 10u;
constexpr uint32_t kStreamWeight = 11u;
NC_HD inline float unit24(uint32_t r) { return (float)(r >> 8) * 0x1p-24f; }
struct KnnGrid {
    float side;
    int32_t g;
    float h;
};
KnnGrid knn_grid(int32_t n, int32_t k, float density);
float ap_value(float x);                              // Neuron::AP, src/NeuCor.cpp:706-714
float step_ms(int64_t k, float dt);                   // k steps as a float time difference

}  // namespace nc

// nc_engine.cuh — data layout shared by the step kernels and the host engine.
//
// One engine advances one or more independent networks ("nets") packed into
// pooled device arrays.  A single network (nc_create) is an engine with one net;
// the batched and served forms pack many.  Every net keeps its own step counter,
// constants, input groups and draw key, and no array is shared between nets, so a
// net computes the same bits alone or packed with others.
//
// Per net, in HBM:
//   neurons   pot, lf (last fire step), firings, act_start     SoA, pool-indexed
//   in_ptr    CSC row starts (n+1): in-synapses of target j, ascending source id
//             — the order of the reference's std::map inSynapses (src/NeuCor.h:212)
//   w, t_arr, term          per in-synapse (CSC order): weight, last arrival step,
//                           contribution term captured at launch (double)
//   inh                     one bit per in-synapse: Synapse::inhibitory
//   out_ptr   CSR row starts (n+1) and per out-synapse (CSR order): target,
//             CSC index, delay (bits 0-13; bit 14/15: the target's caller id is
//             above/below the source's), ring bit position, last accepted arrival step
//   Neurons sit in device slots (Morton order of positions by default); every rule
//   that depends on ids uses the caller's ids (orig_id, the out_delay flags, the
//   in-synapse order).
//   ring      R slots x W words: bit b of target j's words in slot a mod R set when
//             the spike on j's b-th in-synapse arrives at step a
//   fired / forced   two parities of one bit per neuron
#pragma once
#include <cstdint>
#include <vector_types.h>

#ifdef __CUDACC__
#define NC_HD __host__ __device__
#else
#define NC_HD
#endif

#define NC_NEVER INT32_MIN

// Device error codes (NcPools::dev_err).
#define NC_DEV_ERR_STAGE_TIMEOUT 1u  // a bulk copy into shared memory did not complete in time
#define NC_DEV_ERR_FIRER_LOOP 2u     // an input firer's schedule did not advance (capped)
#define NC_DEV_ERR_BARRIER 4u        // a grid barrier of the fused multi-step launch gave up

// Draw streams (third Philox counter word).
#define NC_STREAM_BACKGROUND 1u
#define NC_STREAM_SOURCE 2u
#define NC_STREAM_JITTER 3u
#define NC_STREAM_INDEPENDENT 4u

struct NcGroupDev {
    int32_t first;
    int32_t count;
    uint32_t thresh;     // Bernoulli threshold of the per-step probability, on a 32-bit draw
    int32_t correlated;
    int32_t jitter;
    int32_t index;       // group index within its net (first Philox counter word)
};

struct NcNetDesc {
    int32_t t;            // step processed by the next launch pair (>= 1)
    int32_t t_end;        // last step to simulate (inclusive)
    int32_t stdp_done;    // last step whose deferred plasticity has been applied
    int32_t n;            // neurons
    int32_t neuron_base;  // pool index of neuron 0
    int32_t ptr_base;     // pool index of in_ptr/out_ptr/ring_off entry 0 (n+1 entries)
    int32_t word_base;    // pool index of this net's first bitset word
    int32_t n_words;      // ceil(n/32)
    int64_t syn_base;     // pool index of synapse 0 (CSC and CSR arrays)
    int64_t ring_base;    // pool word index of ring slot 0
    int32_t ring_words;   // words per slot
    int32_t ring_mask;    // slots - 1
    int32_t kc;           // smallest k >= 1 with 2.0f < k*dt (AP_cutoff, src/NeuCor.cpp:385)
    int32_t bg_period;    // max(1, int(600/dt)); 0 = background off
    uint32_t key0, key1;  // Philox key
    int32_t table_base;   // pool index of the trace tables
    int32_t tab_pre_len;  // presynaptic trace table length
    int32_t tab_post_len; // postsynaptic trace table length
    int32_t ap_base;      // pool index of the AP shape table (kc entries)
    int32_t group_base;
    int32_t n_groups;
    int32_t active;       // 0: skipped by the kernels
    int32_t raster_len;   // recorded steps capacity (0 = off)
    int32_t raster_t0;    // first recorded step
    int32_t permuted;     // neurons are stored in a different order than the caller's ids
    float dt;
    float leak;           // powf(0.5f, dt)  (src/NeuCor.cpp:678)
    float c52;            // float(0.2f * 52.0) (src/NeuCor.cpp:729-730)
    float lr, pre_factor, post_factor;
    double e_term;        // 0.9943 is applied separately; this is exp(0.3702*dt) (src/NeuCor.cpp:695)
    uint32_t* raster;     // device raster rows of n_words words
    unsigned long long* stats; // 4 counters: fires, launched, dropped, steps
    int64_t n_syn;        // synapses (the pool range is padded to a multiple of 32)
    float tsum;           // NeuCor::currentTime after t-1 steps: the float sum of t-1 runSpeeds
    int32_t nonneg_terms; // 1: no launch can add a negative term (no inhibitory synapse, no
                          // negative weight), so a neuron's sum only grows within a step
    int32_t group_lo;     // caller ids [group_lo, group_hi) hold every input group's members
    int32_t group_hi;
};

// The smallest id range holding the members of groups g[0..n) (empty when n is 0).
inline void nc_group_range(const NcGroupDev* g, int n, int32_t& lo, int32_t& hi)
{
    lo = 0;
    hi = 0;
    for (int k = 0; k < n; ++k) {
        if (g[k].count <= 0) continue;
        const int32_t a = g[k].first, b = g[k].first + g[k].count;
        if (lo == hi) {
            lo = a;
            hi = b;
        } else {
            lo = a < lo ? a : lo;
            hi = b > hi ? b : hi;
        }
    }
}

struct NcTile {          // 32 consecutive neurons of one net, or (span table) 8 chunks of
    int32_t net;         // 32 in-synapses
    int32_t first;       // local id of the first neuron (multiple of 32), or first chunk
};

constexpr int NC_SPAN_CHUNKS = 8;  // 32-synapse chunks per span of the dense synapse pass

struct NcFirer {         // periodic input firer (InputFirer, src/NeuCor.cpp:305-345)
    int32_t net;
    float last;          // InputFirer::lastFire, ms
    float rate;          // its entry of the rate array, Hz
    int32_t near_begin;  // neuron slots firer_near[near_begin .. near_end)
    int32_t near_end;
    int32_t first;       // set before the net's first step: the run call at time 0 evaluates it too
};

struct NcPools {
    // neurons
    float* pot;
    int32_t* lf;
    uint32_t* firings;
    int32_t* act_start;
    int32_t* orig_id;    // device slot -> caller's id (local to the net)
    int32_t* slot_of;    // caller's id -> device slot (local to the net)
    // per-neuron pointers (n+1 per net)
    int64_t* in_ptr;     // absolute CSC index
    int64_t* out_ptr;    // absolute CSR index
    int32_t* ring_off;   // word offset within a slot
    // in-synapses (CSC); every net's synapse base is a multiple of 32
    float* w;
    uint32_t* inh;       // Synapse::inhibitory, one bit per synapse
    int32_t* t_arr;
    double* term;        // last launch's charge_insynapses term (src/NeuCor.cpp:695)
    // out-synapses (CSR)
    int32_t* out_post;   // local target id
    int32_t* out_csc;    // CSC index relative to syn_base
    int16_t* out_delay;
    uint32_t* out_ringpos; // (word within slot) << 5 | bit
    int32_t* last_arr;
    // dense form: in-synapse (CSC) order
    int32_t* csc_pre;    // source's device slot (local to the net)
    int32_t* csc_post;   // target's device slot (local to the net)
    uint16_t* csc_dl;    // delay | target-above-source << 14 | target-below-source << 15
    int32_t* la_c;       // arrival step of the last accepted launch
    float* pst;          // per neuron, written by the neuron pass of step t for the synapse
                         // pass of t+1: the postsynaptic trace at t (getTrace), or -0.0
                         // when the neuron fired at t
    uint32_t* win;       // bit per synapse: arrived within the fold window of the net's step
    NcTile* spans;       // work items of the synapse pass
    int32_t n_spans;
    int32_t* n_spans_dev; // when set, the span count is read from device memory (served engine)
    // ring and bitsets
    uint32_t* ring;
    uint32_t* fired;     // 2 parities x total_words
    uint32_t* forced;    // 2 parities x total_words
    uint32_t* ufire;     // 2 parities x total_words: input-firer fires (no threshold, no refractory)
    NcFirer* firers;
    int32_t n_firers;
    int32_t* firer_near;
    int64_t total_words;
    // fired list (global, 2 parities)
    int2* fired_list;    // (net, local id)
    int32_t* fired_count;// [2]
    int64_t fired_cap;
    // constants
    float* tables;
    NcGroupDev* groups;
    NcNetDesc* nets;
    int32_t n_nets;
    NcTile* tiles;
    int32_t n_tiles;
    int32_t* n_tiles_dev; // when set, the tile count is read from device memory (served engine)
    // engine
    int32_t* tick;       // engine tick (parity of the fired list)
    uint32_t* done_ctr;  // last-block detection
    uint32_t* dev_err;   // nonzero: a bounded device wait gave up (NC_DEV_ERR_*)
};

// ------------------------------------------------------------------ Philox
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).
NC_HD inline void nc_philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                          uint32_t k1, uint32_t out[4])
{
#ifdef __CUDACC__
#pragma unroll
#endif
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
#ifdef __CUDA_ARCH__
        const uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
#else
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
        const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

// Kernel launchers (nc_kernels.cu).
namespace nc {
// Resident 256-thread blocks per SM the step kernels' register allocation is held to
// (3 keep every tile of a 100k-neuron net in one wave for the event form's neuron
// update); the spike-launch grid defaults to NC_LAUNCH_MIN_BLOCKS blocks per SM.
#ifndef NC_NEURON_MIN_BLOCKS
#define NC_NEURON_MIN_BLOCKS 3
#endif
#ifndef NC_DENSE_MIN_BLOCKS
#define NC_DENSE_MIN_BLOCKS 4
#endif
#ifndef NC_DNEURON_BLOCK
#define NC_DNEURON_BLOCK 128  // threads per block of the dense neuron pass
#endif
#ifndef NC_LAUNCH_MIN_BLOCKS
#define NC_LAUNCH_MIN_BLOCKS 4
#endif

struct LaunchShape {
    int neuron_block;    // threads per block of the neuron-update kernel (multiple of 32)
    int launch_blocks;   // blocks of the spike-launch kernel
    int launch_block;    // threads per block of the spike-launch kernel
    int dense_blocks = 0; // blocks of the dense synapse pass (0: one warp per span)
    int fused_ticks = 0;  // dense form: steps per fused cooperative launch (0: two launches
                          // per step, replayed through CUDA graphs)
};
int launch_neuron_step(const NcPools& P, const LaunchShape& L, void* stream);
int launch_spike_launch(const NcPools& P, const LaunchShape& L, void* stream);
int launch_stdp_flush(const NcPools& P, const LaunchShape& L, void* stream);
// Dense form (nc_dense.cu): the synapse pass and the neuron pass of one step, and the
// plasticity flush (the synapse pass of the last step's fires) before read-back.
int launch_dense_synapses(const NcPools& P, const LaunchShape& L, void* stream);
int launch_dense_neurons(const NcPools& P, const LaunchShape& L, void* stream);
// Sizes the dense synapse pass's persistent grid (and sets its shared-memory opt-in) on
// the current device; called before a stream capture, where neither may happen.
int prepare_dense_launch();
int launch_step_dense(const NcPools& P, const LaunchShape& L, void* stream);
// `ticks` whole dense steps of every net in one cooperative launch (no periodic input
// firers); bar: two zero-initialised words of device memory for its grid barrier.
int launch_fused_dense(const NcPools& P, int32_t ticks, unsigned* bar, void* stream);
// Conversion of net `net`'s per-synapse arrival state between the forms (nc_form.cu),
// after the current form's plasticity flush.  ring_words: the words of the whole ring
// pool (cleared first).
int launch_form_to_event(const NcPools& P, int net, int64_t n_syn, int64_t ring_words, void* stream);
int launch_form_to_dense(const NcPools& P, int net, int64_t n_syn, void* stream);
int launch_flush_dense(const NcPools& P, const LaunchShape& L, void* stream);
int launch_background_prologue(const NcPools& P, int net, int n_neurons, void* stream);
int launch_force_bits(const NcPools& P, int net, const int32_t* d_ids, int count, void* stream);
// Input firers (nc_inputs.cu), launched before a step's kernels: each firer's schedule
// for the run call that starts at its net's step t; fires land in the ufire bits of
// step t+1 (and, before the first step, those of the time-0 call in step 1's).
int launch_input_firers(const NcPools& P, void* stream);
// Mean potential of each detector's near neurons (caller ids; near_ptr has count+1 entries).
int launch_detector_voltages(const NcPools& P, int32_t neuron_base, const int32_t* near, const int32_t* near_ptr,
                             int32_t count, float* out, void* stream);
int launch_raster_to_ids(const uint32_t* in, uint32_t* out, const int32_t* slot_of, int32_t n, int32_t n_words,
                         int32_t rows, void* stream);
}  // namespace nc

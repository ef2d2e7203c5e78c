// nc_form.cu — switching a single network between the two forms of the step kernels
// (NC_STEP_AUTO).  Both forms keep the same neuron state, weights, arrival steps
// (t_arr), captured terms and fired bitsets; they differ in how a synapse's last
// accepted launch is kept:
//   dense form  la_c[c]      per in-synapse (CSC order), plus the window bitmap of the
//                            next fold;
//   event form  last_arr[k]  per out-synapse (CSR order), plus the ring bits of the
//                            spikes still needed by a fold (arrived t-KC .. t-1) or in
//                            flight.
// A switch happens between steps, after the current form's plasticity flush (every
// launch and every plasticity update of step t-1 done, stdp_done = t-1); the next step
// t then skips its deferred part in either form, so the conversion below is all that
// changes.
#include "nc_engine.cuh"

#include <cuda_runtime.h>

namespace {

constexpr unsigned kFull = 0xffffffffu;

// Dense -> event: last_arr of every out-synapse from its CSC entry, and the ring bits of
// the spikes that arrived t-KC .. t-1 or arrive later (the ring was cleared before).
__global__ void k_form_to_event(NcPools P, int net)
{
    const NcNetDesc& D = P.nets[net];
    const int32_t t = D.t, kc = D.kc;
    const int64_t sb = D.syn_base;
    uint32_t* ring = P.ring + D.ring_base;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < D.n_syn; k += (int64_t)gridDim.x * blockDim.x) {
        const int32_t a = P.la_c[sb + P.out_csc[sb + k]];
        P.last_arr[sb + k] = a;
        if (a != NC_NEVER && a >= t - kc) {
            const uint32_t pos = P.out_ringpos[sb + k];
            atomicOr(ring + (int64_t)(a & D.ring_mask) * D.ring_words + (pos >> 5), 1u << (pos & 31));
        }
    }
}

// Event -> dense: la_c of every in-synapse from its out-synapse.
__global__ void k_form_to_dense(NcPools P, int net)
{
    const NcNetDesc& D = P.nets[net];
    const int64_t sb = D.syn_base;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < D.n_syn; k += (int64_t)gridDim.x * blockDim.x)
        P.la_c[sb + P.out_csc[sb + k]] = P.last_arr[sb + k];
}

// The window bitmap of step t's fold (arrived t-KC .. t-1), which the dense synapse
// pass of step t would have written: warp per 32 in-synapses.
__global__ void k_form_window(NcPools P, int net)
{
    const NcNetDesc& D = P.nets[net];
    const int32_t t = D.t, kc = D.kc;
    const int64_t sb = D.syn_base;
    const int lane = threadIdx.x & 31;
    const int64_t chunks = (D.n_syn + 31) / 32;
    for (int64_t c = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; c < chunks;
         c += ((int64_t)gridDim.x * blockDim.x) >> 5) {
        const int64_t s = c * 32 + lane;
        const int32_t a = s < D.n_syn ? P.la_c[sb + s] : NC_NEVER;
        const uint32_t m = __ballot_sync(kFull, a != NC_NEVER && t - a >= 1 && t - a <= kc);
        if (lane == 0) P.win[(sb >> 5) + c] = m;
    }
}

int grid_for(int64_t items, int per_block)
{
    const int64_t b = (items + per_block - 1) / per_block;
    return (int)(b < 1 ? 1 : (b > 65536 ? 65536 : b));
}

}  // namespace

namespace nc {

int launch_form_to_event(const NcPools& P, int net, int64_t n_syn, int64_t ring_words, void* stream)
{
    const cudaStream_t s = (cudaStream_t)stream;
    if (cudaMemsetAsync(P.ring, 0, sizeof(uint32_t) * (size_t)ring_words, s) != cudaSuccess) return -1;
    k_form_to_event<<<grid_for(n_syn, 256), 256, 0, s>>>(P, net);
    // the next step's neuron update starts a new fired list
    if (cudaMemsetAsync(P.fired_count, 0, 2 * sizeof(int32_t), s) != cudaSuccess) return -1;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_form_to_dense(const NcPools& P, int net, int64_t n_syn, void* stream)
{
    const cudaStream_t s = (cudaStream_t)stream;
    k_form_to_dense<<<grid_for(n_syn, 256), 256, 0, s>>>(P, net);
    k_form_window<<<grid_for((n_syn + 31) / 32 * 32, 256), 256, 0, s>>>(P, net);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace nc

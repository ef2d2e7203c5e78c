// nc_noalloc.cu — nc_run_noalloc (neucor_gb300.h): the simulation step for callers
// that cannot let the library allocate device memory once their network is set up.
//
// Some callers own every byte of device memory themselves: a simulation service that
// reserves a fixed budget per GPU up front and admits work against it, or a host
// program (a renderer, a game or robotics engine embedding the simulator) whose own
// allocator has carved up the GPU.  A cudaMalloc made behind their back can fail when
// the memory is spoken for, or silently break their accounting.  nc_run keeps the
// compacted list of neurons that fired in a step — the scratch the neuron-update kernel
// writes and the spike-launch kernel reads — in memory the handle allocated, and
// instantiates CUDA graphs (which allocate) on first use.  nc_run_noalloc launches the
// same kernels directly.  The event form gets its scratch from this file's static
// device array instead; the dense form needs none.  Nothing is allocated: the
// network's own arrays are the inputs and outputs.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "nc_net.h"

namespace {

constexpr int64_t kMaxNeurons = NC_NOALLOC_MAX_NEURONS;

// The fired list of both parities and the step kernels' counters.  16 bytes of counters
// follow the list so one memset clears them.
struct NoallocScratch {
    int2 fired_list[2 * kMaxNeurons];
    int32_t fired_count[2];
    int32_t tick;
    uint32_t done_ctr;
};

// Held by every GPU that loads this library, until the process exits (4 MiB + 16 B).
__device__ __align__(256) NoallocScratch g_noalloc_scratch;

constexpr int kMaxDevices = 256;
std::mutex g_setup_mu;
NoallocScratch* g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on `device` (which is current).  The name
// g_noalloc_scratch in host code is only a stand-in for the symbol, never an address a
// kernel may use, so the address is looked up once per device and kept.
int scratch_for(int device, NoallocScratch** out)
{
    if (device < 0 || device >= kMaxDevices) return nc::set_last_error(NC_ERR_INVALID, "device index out of range");
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_addr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return nc::set_last_error(NC_ERR_CUDA, nc::cuda_msg("cudaGetSymbolAddress(noalloc scratch)", e));
        g_scratch_addr[device] = (NoallocScratch*)p;
    }
    *out = g_scratch_addr[device];
    return NC_OK;
}

}  // namespace

extern "C" int nc_run_noalloc(nc_net* net, int32_t n_steps, void* stream)
{
    if (!net) return nc::set_last_error(NC_ERR_INVALID, "null handle");
    if (n_steps < 0) return nc::set_last_error(NC_ERR_INVALID, "negative step count");
    if (net->step + n_steps >= (1ll << 30)) return nc::set_last_error(NC_ERR_INVALID, "step counter limit reached");
    cudaError_t e = cudaSetDevice(net->eng.device);
    if (e != cudaSuccess) return nc::set_last_error(NC_ERR_CUDA, nc::cuda_msg("cudaSetDevice", e));
    cudaStream_t s = stream ? (cudaStream_t)stream : net->eng.stream;
    if (net->eng.dense) {
        // the dense form keeps no scratch between its launches: the network's own arrays
        // are all it reads and writes
        for (int32_t k = 0; k < n_steps; ++k)
            if (nc::launch_input_firers(net->eng.P, s) || nc::launch_step_dense(net->eng.P, net->eng.L, s))
                return nc::set_last_error(NC_ERR_CUDA, nc::cuda_msg("nc_run_noalloc launch", cudaGetLastError()));
    } else {
        const int64_t neurons = net->eng.P.fired_cap;
        if (neurons > kMaxNeurons)
            return nc::set_last_error(NC_ERR_INVALID, "nc_run_noalloc serves event-form networks of at most " +
                                                          std::to_string(kMaxNeurons) + " neurons; this one has " +
                                                          std::to_string(neurons) + " (use nc_run)");
        NoallocScratch* scratch = nullptr;
        const int rc = scratch_for(net->eng.device, &scratch);
        if (rc != NC_OK) return rc;
        // the same kernels and network arrays as nc_run; only the scratch moves
        NcPools P = net->eng.P;
        P.fired_list = scratch->fired_list;
        P.fired_count = scratch->fired_count;
        P.tick = &scratch->tick;
        P.done_ctr = &scratch->done_ctr;
        P.fired_cap = kMaxNeurons;
        // the array keeps the previous call's contents: the counters must start at zero
        e = cudaMemsetAsync(scratch->fired_count, 0, sizeof(int32_t) * 2 + sizeof(int32_t) + sizeof(uint32_t), s);
        if (e != cudaSuccess)
            return nc::set_last_error(NC_ERR_CUDA, nc::cuda_msg("cudaMemsetAsync(noalloc counters)", e));
        for (int32_t k = 0; k < n_steps; ++k) {
            if (nc::launch_input_firers(P, s) || nc::launch_neuron_step(P, net->eng.L, s) ||
                nc::launch_spike_launch(P, net->eng.L, s))
                return nc::set_last_error(NC_ERR_CUDA, nc::cuda_msg("nc_run_noalloc launch", cudaGetLastError()));
        }
    }
    net->step += n_steps;
    for (int32_t k = 0; k < n_steps; ++k) net->time = net->time + net->host.dt;
    // the launches above are not tracked by the handle once issued: later calls on the
    // handle read the step counter and simulated time back from the device
    net->counters_on_device = true;
    return NC_OK;
}

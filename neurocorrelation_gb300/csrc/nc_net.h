// nc_net.h — the single-network handle behind nc_net* (internal).
#pragma once
#include <vector>

#include "nc_pool.h"

struct nc_net {
    nc::NetHost host;
    nc::Engine eng;
    int64_t step = 0;      // completed steps
    float time = 0.0f;     // NeuCor::currentTime, accumulated per step
    // Set by nc_run_noalloc: its launches may run again without this handle seeing
    // them, so from then on step and time are read back from the device's step
    // counter (NcNetDesc t, tsum) before any call that uses them.
    bool counters_on_device = false;
    // NC_STEP_AUTO: nc_run picks the form from the last window's fires (auto_form);
    // auto_fires is the fire count at the start of the current window and auto_steps the
    // steps run in it so far (windows span run calls)
    bool auto_form = false;
    uint64_t auto_fires = 0;
    int64_t auto_steps = 0;
    uint32_t* d_raster = nullptr;
    uint32_t* d_raster_ids = nullptr;  // the same rows in caller-id order (read-back staging)
    int32_t raster_cap = 0;
    int32_t raster_t0 = 0;
    // periodic input firers (InputFirer): positions, radii and near lists (device slots)
    std::vector<float> firer_xyz, firer_radius;
    std::vector<std::vector<int32_t>> firer_near;
    // voltage detectors (VoltageDetector): near lists of caller ids, ascending
    std::vector<int32_t> det_near, det_ptr{0};
    int32_t* d_det = nullptr;      // det_near then det_ptr on the device
    float* d_volt = nullptr;
    // built on the device (nc_create_knn): targets in creation order and the CSC position
    // of every synapse, kept there until a read-back needs the host tables
    int32_t* dev_to = nullptr;
    int64_t* dev_i2c = nullptr;
    int32_t knn_k = 0;
    ~nc_net()
    {
        if (dev_to) cudaFree(dev_to);
        if (dev_i2c) cudaFree(dev_i2c);
        if (d_raster) cudaFree(d_raster);
        if (d_raster_ids) cudaFree(d_raster_ids);
        if (d_det) cudaFree(d_det);
        if (d_volt) cudaFree(d_volt);
    }
};

namespace nc {
// The kNN network of nc_build_knn built on the device into `net` (nc_build.cu);
// NC_ERR_UNSUPPORTED when it exceeds the device builder's capacities.
int build_knn_device(int32_t n, int32_t k, float density, uint64_t seed, const nc_params& p, nc_net* net,
                     std::string& err);
}  // namespace nc

// nc_net.h — the single-network handle behind nc_net* (internal).
#pragma once
#include <vector>

#include "nc_pool.h"

struct nc_net {
    nc::NetHost host;
    nc::Engine eng;
    int64_t step = 0;      // completed steps
    float time = 0.0f;     // NeuCor::currentTime, accumulated per step
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
    ~nc_net()
    {
        if (d_raster) cudaFree(d_raster);
        if (d_raster_ids) cudaFree(d_raster_ids);
        if (d_det) cudaFree(d_det);
        if (d_volt) cudaFree(d_volt);
    }
};

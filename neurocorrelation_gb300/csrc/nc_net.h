// nc_net.h — the single-network handle behind nc_net* (internal).
#pragma once
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
    ~nc_net()
    {
        if (d_raster) cudaFree(d_raster);
        if (d_raster_ids) cudaFree(d_raster_ids);
    }
};

// mrg_launch.h -- per-device launch setup cache.
#pragma once
#include <cuda_runtime.h>

namespace mrg {

constexpr int kMaxDevices = 64;

// Index of the calling thread's current device (0 when it cannot be read or
// is out of range), for per-device caches of function attributes and
// occupancy queries: both belong to the device a kernel launches on.
inline int launch_device()
{
    int d = 0;
    if(cudaGetDevice(&d) != cudaSuccess || d < 0 || d >= kMaxDevices) d = 0;
    return d;
}

} // namespace mrg

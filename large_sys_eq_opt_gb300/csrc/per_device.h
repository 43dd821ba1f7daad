// per_device.h -- launch set-up cached per CUDA device.
//
// Kernel attributes (the dynamic shared-memory opt-in) and occupancy-derived
// launch sizes belong to a device, not to the process: a process that drives
// several GPUs must set the attribute on each of them.  These helpers key the
// cache on the calling thread's current device.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>

namespace eu {

constexpr int kMaxDevices = 64;

// The calling thread's current device, or -1 when it cannot be read.
inline int current_device() {
    int d = 0;
    if (cudaGetDevice(&d) != cudaSuccess) {
        (void)cudaGetLastError();
        return -1;
    }
    return d;
}

// f() run once per device; later calls on that device return the first
// result.  Devices beyond kMaxDevices (or an unreadable current device) run
// f() on every call.
template <class R> struct PerDevice {
    std::once_flag flag[kMaxDevices];
    R value[kMaxDevices];
    template <class F> R get(F&& f) {
        const int d = current_device();
        if (d < 0 || d >= kMaxDevices) return f();
        std::call_once(flag[d], [&] { value[d] = f(); });
        return value[d];
    }
};

// Streaming multiprocessors of the current device (cached per device).
inline int sm_count_current() {
    static PerDevice<int> cache;
    return cache.get([] {
        int dev = current_device(), n = 0;
        if (dev < 0 || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) {
            (void)cudaGetLastError();
            n = 1;
        }
        return n;
    });
}

}  // namespace eu

// per_device.h -- host-side values that depend on the current CUDA device
// (kernel attributes, occupancy) computed once per device and thread-safe.
//
// Kernel attributes such as cudaFuncAttributeMaxDynamicSharedMemorySize and
// occupancy queries belong to the device that is current when they are made,
// so a process that draws on several GPUs must configure each one. Launchers
// may run on several host threads at once (different contexts, or the
// static draw on one stream from several threads), hence std::call_once and
// atomics rather than plain statics.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <mutex>

namespace cr {

constexpr int kMaxDevices = 64;

// The current device, or -1 when it cannot be cached (no device, or an index
// beyond kMaxDevices: callers then compute the value every time).
inline int currentDeviceSlot() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return -1;
    return dev;
}

// Runs init() once per device (with that device current).
class OncePerDevice {
public:
    template <class Init>
    void run(Init init) {
        const int dev = currentDeviceSlot();
        if (dev < 0) {
            init();
            return;
        }
        std::call_once(once_[dev], init);
    }

private:
    std::once_flag once_[kMaxDevices];
};

// N integers per device, each computed on first use by init(i) (> 0). Two
// threads may both compute a value the first time; they store the same one.
template <int N>
class IntsPerDevice {
public:
    template <class Init>
    int get(int i, Init init) {
        const int dev = currentDeviceSlot();
        if (dev < 0 || i < 0 || i >= N) return init(i);
        int v = value_[dev][i].load(std::memory_order_relaxed);
        if (v > 0) return v;
        v = init(i);
        value_[dev][i].store(v, std::memory_order_relaxed);
        return v;
    }

private:
    std::atomic<int> value_[kMaxDevices][N] = {};
};

}  // namespace cr

// Every handle of the library belongs to the device that was current when it
// was created. A call on a handle runs on that device whatever device is
// current in the calling thread: the guard selects it for the call and gives
// the thread its previous device back afterwards (on a one-device system, and
// whenever the devices agree, it does nothing).
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "internal.h"

namespace cvx {

class DeviceGuard {
   public:
    explicit DeviceGuard(int dev) : dev_(dev) {
        if (cudaGetDevice(&prev_) != cudaSuccess) {
            cudaGetLastError();
            return;
        }
        if (prev_ == dev) {
            ok_ = true;
        } else if (cudaSetDevice(dev) == cudaSuccess) {
            ok_ = restore_ = true;
        } else {
            cudaGetLastError();
        }
    }
    ~DeviceGuard() {
        if (restore_) cudaSetDevice(prev_);
    }
    DeviceGuard(const DeviceGuard&) = delete;
    DeviceGuard& operator=(const DeviceGuard&) = delete;
    // The handle's device is current; otherwise the error status to return.
    bool ok() const { return ok_; }
    int32_t fail() const {
        return set_error(CVX_ERR_CUDA, "cannot select device " + std::to_string(dev_) + " of the handle");
    }

   private:
    int dev_ = 0, prev_ = 0;
    bool ok_ = false, restore_ = false;
};

// Waits, whichever way the enclosing call returns, for the work it queued on
// its streams. Copies into the caller's buffers (or into locals of the call)
// and kernels reading the caller's memory in place must not outlive the call,
// and an error return halfway through would otherwise leave them in flight.
// Declare it after the locals that copies write to, so that it runs first.
class StreamSync {
   public:
    StreamSync(cudaStream_t a, cudaStream_t b = nullptr, cudaStream_t c = nullptr) : s_{a, b, c} {}
    ~StreamSync() {
        for (cudaStream_t s : s_)
            if (s) cudaStreamSynchronize(s);
    }
    StreamSync(const StreamSync&) = delete;
    StreamSync& operator=(const StreamSync&) = delete;

   private:
    cudaStream_t s_[3];
};

// The device current in the calling thread (-1 when none can be had).
inline int current_device() {
    int d = -1;
    if (cudaGetDevice(&d) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    return d;
}

}  // namespace cvx

// Selects handle device `dev` for the rest of the enclosing entry point, or
// returns the error status from it.
#define CVX_ON_DEVICE(dev)                              \
    ::cvx::DeviceGuard cvx_device_guard_(dev);          \
    if (!cvx_device_guard_.ok()) return cvx_device_guard_.fail()

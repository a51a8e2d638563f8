/*
 * fdgpu_device.h — run a library call on the device it belongs to, and leave the calling thread's
 * own device selection as it was.
 *
 * A context, a serving session or a c2f plan is bound to one device; its entry points make that
 * device current for the duration of the call and give the caller's current device back on
 * return, so that a program driving several GPUs from one thread (or mixing this library with
 * another CUDA library) does not find its device switched by a call.  When the caller's device is
 * already the right one, nothing is switched.
 */
#ifndef FDGPU_DEVICE_H
#define FDGPU_DEVICE_H

#include <cuda_runtime.h>

struct FdDeviceScope {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit FdDeviceScope(int device)
    {
        int cur = -1;
        if (cudaGetDevice(&cur) != cudaSuccess) cur = -1;
        if (cur != device) {
            err = cudaSetDevice(device);
            if (err == cudaSuccess) prev = cur;
        }
    }
    ~FdDeviceScope()
    {
        if (prev >= 0) cudaSetDevice(prev);
    }
    FdDeviceScope(const FdDeviceScope &) = delete;
    FdDeviceScope &operator=(const FdDeviceScope &) = delete;
};

#endif

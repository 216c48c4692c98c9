// Host-or-device staging of user buffers for the drop-in entry points: a
// buffer the caller passed in host memory is mirrored in device memory for
// the duration of one call (and copied back when it is an output); a device
// buffer is used in place.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdlib>

#include "sgb_common.cuh"

namespace {

bool is_device_ptr(const void *p)
{
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// A user buffer mirrored in device memory for the duration of one call.
struct Stage {
    void *user = nullptr, *dev = nullptr;
    size_t bytes = 0;
    bool owned = false;
    cudaError_t err = cudaSuccess;
    Stage(const void *u, size_t b, bool copy_in) : user(const_cast<void *>(u)), bytes(b)
    {
        if (!u || b == 0) return;
        if (is_device_ptr(u)) { dev = user; return; }
        err = cudaMalloc(&dev, b);
        if (err != cudaSuccess) { dev = nullptr; return; }
        owned = true;
        if (copy_in) err = cudaMemcpy(dev, u, b, cudaMemcpyHostToDevice);
    }
    cudaError_t back()
    {
        if (owned && err == cudaSuccess) return cudaMemcpy(user, dev, bytes, cudaMemcpyDeviceToHost);
        return err;
    }
    ~Stage() { if (owned && dev) cudaFree(dev); }
    Stage(const Stage &) = delete;
    Stage &operator=(const Stage &) = delete;
};

size_t span_bytes(int n, int inc, size_t el) { return n <= 0 ? 0 : ((size_t) (n - 1) * std::abs(inc) + 1) * el; }

int err_of(cudaError_t e, const char *what)
{
    return e == cudaSuccess ? 0 : sgb_set_error(e, what, __FILE__, __LINE__);
}

}  // namespace

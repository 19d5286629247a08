// Device buffers for the apps that pass device arrays to the C ABI (the boundary estimator, the
// VPL pair and walk on spheres take device pointers, as the reference's kernels read device memory).
#ifndef WOBAPP_CUDA_HPP
#define WOBAPP_CUDA_HPP

#include <cuda_runtime.h>

#include <algorithm>
#include <stdexcept>
#include <string>
#include <vector>

namespace wobapp {

inline void cuda_check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

template <class T> struct DeviceArray {
    T *p = nullptr;
    size_t n = 0;
    explicit DeviceArray(size_t count) : n(count) {
        cuda_check(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)), "cudaMalloc");
    }
    explicit DeviceArray(const std::vector<T> &host) : DeviceArray(host.size()) { upload(host); }
    ~DeviceArray() {
        if (p) cudaFree(p);
    }
    DeviceArray(const DeviceArray &) = delete;
    DeviceArray &operator=(const DeviceArray &) = delete;
    void upload(const std::vector<T> &host) {
        cuda_check(cudaMemcpy(p, host.data(), std::min(n, host.size()) * sizeof(T), cudaMemcpyHostToDevice), "copy to device");
    }
    void download(std::vector<T> &host) const {
        host.resize(n);
        cuda_check(cudaMemcpy(host.data(), p, n * sizeof(T), cudaMemcpyDeviceToHost), "copy to host");
    }
    void zero() { cuda_check(cudaMemset(p, 0, n * sizeof(T)), "cudaMemset"); }
};

}  // namespace wobapp

#endif  // WOBAPP_CUDA_HPP

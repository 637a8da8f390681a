// DeviceBuffer<T>: move-only owner of stream-ordered device memory
// (cudaMallocAsync / cudaFreeAsync on one stream). Same interface as the
// reference's DeviceBuffer (core/include/water/core/device_buffer.h:21-89).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <utility>

#include "water/core/cuda_check.h"

namespace water {

template <typename T>
class DeviceBuffer {
public:
    DeviceBuffer() = default;

    explicit DeviceBuffer(std::size_t count, cudaStream_t stream = 0) : size_(count), stream_(stream) {
        if (count > 0)
            WATER_CUDA_CHECK(cudaMallocAsync(reinterpret_cast<void**>(&ptr_), count * sizeof(T), stream_));
    }

    ~DeviceBuffer() {
        if (ptr_) cudaFreeAsync(ptr_, stream_);
    }

    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;

    DeviceBuffer(DeviceBuffer&& o) noexcept : ptr_(o.ptr_), size_(o.size_), stream_(o.stream_) {
        o.ptr_ = nullptr;
        o.size_ = 0;
    }
    DeviceBuffer& operator=(DeviceBuffer&& o) noexcept {
        if (this != &o) {
            if (ptr_) cudaFreeAsync(ptr_, stream_);
            ptr_ = o.ptr_;
            size_ = o.size_;
            stream_ = o.stream_;
            o.ptr_ = nullptr;
            o.size_ = 0;
        }
        return *this;
    }

    T* data() noexcept { return ptr_; }
    const T* data() const noexcept { return ptr_; }
    std::size_t size() const noexcept { return size_; }
    bool empty() const noexcept { return size_ == 0; }
    cudaStream_t stream() const noexcept { return stream_; }

    void fill_zero() {
        if (ptr_ && size_) WATER_CUDA_CHECK(cudaMemsetAsync(ptr_, 0, size_ * sizeof(T), stream_));
    }
    void copy_from_host(const T* src, std::size_t count) {
        WATER_CUDA_CHECK(cudaMemcpyAsync(ptr_, src, count * sizeof(T), cudaMemcpyHostToDevice, stream_));
    }
    void copy_to_host(T* dst, std::size_t count) const {
        WATER_CUDA_CHECK(cudaMemcpyAsync(dst, ptr_, count * sizeof(T), cudaMemcpyDeviceToHost, stream_));
    }

private:
    T* ptr_ = nullptr;
    std::size_t size_ = 0;
    cudaStream_t stream_ = 0;
};

}  // namespace water

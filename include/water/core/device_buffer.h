// DeviceBuffer<T>: a typed, move-only handle to device memory allocated and
// released in stream order on one stream. The public interface is the
// reference's (core/include/water/core/device_buffer.h:21-89): construction
// from a count and a stream, data/size/empty/stream, fill_zero and the two
// host copies, all asynchronous on that stream.
//
// Ownership is a std::unique_ptr whose deleter remembers the stream and
// returns the memory with cudaFreeAsync there, so moves, move-assignment and
// destruction are the unique_ptr's own; the element count travels with it.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <memory>

#include "water/core/cuda_check.h"

namespace water {

namespace detail {

// Releases stream-ordered device memory on the stream it was allocated on.
struct StreamFree {
    cudaStream_t stream = 0;
    void operator()(void* p) const noexcept {
        if (p) cudaFreeAsync(p, stream);  // a destructor must not throw: status dropped
    }
};

inline void* stream_alloc(std::size_t bytes, cudaStream_t stream) {
    void* p = nullptr;
    if (bytes) WATER_CUDA_CHECK(cudaMallocAsync(&p, bytes, stream));
    return p;
}

}  // namespace detail

template <typename T>
class DeviceBuffer {
public:
    DeviceBuffer() = default;
    explicit DeviceBuffer(std::size_t count, cudaStream_t stream = 0)
        : mem_(static_cast<T*>(detail::stream_alloc(count * sizeof(T), stream)), detail::StreamFree{stream}),
          count_(count) {}

    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    // the moved-from buffer is left empty
    DeviceBuffer(DeviceBuffer&& o) noexcept : mem_(std::move(o.mem_)), count_(o.release_count()) {}
    DeviceBuffer& operator=(DeviceBuffer&& o) noexcept {
        mem_ = std::move(o.mem_);  // frees what this buffer held, on its own stream
        count_ = o.release_count();
        return *this;
    }

    T* data() noexcept { return mem_.get(); }
    const T* data() const noexcept { return mem_.get(); }
    std::size_t size() const noexcept { return count_; }
    bool empty() const noexcept { return count_ == 0; }
    cudaStream_t stream() const noexcept { return mem_.get_deleter().stream; }

    void fill_zero() {
        if (!empty()) WATER_CUDA_CHECK(cudaMemsetAsync(data(), 0, bytes(count_), stream()));
    }
    void copy_from_host(const T* src, std::size_t count) { copy(data(), src, count, cudaMemcpyHostToDevice); }
    void copy_to_host(T* dst, std::size_t count) const { copy(dst, data(), count, cudaMemcpyDeviceToHost); }

private:
    static constexpr std::size_t bytes(std::size_t count) noexcept { return count * sizeof(T); }
    std::size_t release_count() noexcept {
        const std::size_t c = count_;
        count_ = 0;
        return c;
    }
    void copy(void* dst, const void* src, std::size_t count, cudaMemcpyKind kind) const {
        WATER_CUDA_CHECK(cudaMemcpyAsync(dst, src, bytes(count), kind, stream()));
    }

    std::unique_ptr<T, detail::StreamFree> mem_{nullptr, detail::StreamFree{}};
    std::size_t count_ = 0;
};

}  // namespace water

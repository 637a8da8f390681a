// ParticleStore: particle arrays of a fixed capacity with named, typed
// attributes; position and velocity are AoS Vec3f. The public interface and
// error behaviour are the reference's (core/include/water/core/particle_store.h
// :15-127, core/src/particle_store.cu): resize beyond the capacity throws
// std::out_of_range, a handle that names no attribute throws
// std::out_of_range, registering a name twice throws std::runtime_error, and
// every attribute starts zero-filled.
//
// Storage is pooled: attributes are carved, 256-byte aligned, out of arena
// blocks of device memory (stream ordered on the store's stream), so the
// position, velocity and the solver's four scalar attributes of a store live
// in one allocation instead of six. An attribute that does not fit the free
// tail of the current block opens a new block (existing attributes never
// move: their pointers stay valid for the store's lifetime).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <stdexcept>
#include <string>
#include <string_view>
#include <vector>

#include "water/core/device_buffer.h"
#include "water/core/types.h"

namespace water {

enum class AttribType { F32, F32x3, U32 };

// Bytes per particle of an attribute type.
inline std::size_t attrib_element_size(AttribType t) {
    return t == AttribType::F32x3 ? 3 * sizeof(float) : sizeof(float);  // F32 and U32 are both 4 bytes
}

template <typename T>
class AttribHandle {
public:
    AttribHandle() = default;
    explicit AttribHandle(std::size_t index) : index_(index) {}
    std::size_t index() const noexcept { return index_; }
    bool valid() const noexcept { return index_ != npos; }

private:
    static constexpr std::size_t npos = ~std::size_t(0);
    std::size_t index_ = npos;
};

class ParticleStore {
public:
    // The first arena block is sized for position, velocity and four scalar
    // attributes per particle (the solver's density, alpha, kappa, rho*).
    explicit ParticleStore(std::size_t capacity, cudaStream_t stream = 0)
        : capacity_(capacity), stream_(stream) {
        reserve_block(2 * padded(capacity * sizeof(Vec3f)) + 4 * padded(capacity * sizeof(float)));
        position_ = register_attribute<Vec3f>("position", AttribType::F32x3);
        velocity_ = register_attribute<Vec3f>("velocity", AttribType::F32x3);
    }

    ParticleStore(const ParticleStore&) = delete;
    ParticleStore& operator=(const ParticleStore&) = delete;
    ParticleStore(ParticleStore&&) = default;
    ParticleStore& operator=(ParticleStore&&) = default;

    AttribHandle<Vec3f> position_handle() const noexcept { return position_; }
    AttribHandle<Vec3f> velocity_handle() const noexcept { return velocity_; }

    Vec3f* positions() { return attribute_data(position_); }
    Vec3f* velocities() { return attribute_data(velocity_); }
    const Vec3f* positions() const { return attribute_data(position_); }
    const Vec3f* velocities() const { return attribute_data(velocity_); }

    template <typename T>
    AttribHandle<T> register_attribute(std::string_view name, AttribType type) {
        if (find(name) != attribs_.size())
            throw std::runtime_error("ParticleStore: the attribute '" + std::string(name) + "' exists already");
        const std::size_t bytes = capacity_ * attrib_element_size(type);
        unsigned char* at = carve(bytes);
        if (bytes) WATER_CUDA_CHECK(cudaMemsetAsync(at, 0, bytes, stream_));
        attribs_.push_back(Attrib{std::string(name), type, at});
        return AttribHandle<T>(attribs_.size() - 1);
    }

    template <typename T>
    T* attribute_data(AttribHandle<T> h) {
        return reinterpret_cast<T*>(slot(h.index()).data);
    }
    template <typename T>
    const T* attribute_data(AttribHandle<T> h) const {
        return reinterpret_cast<const T*>(slot(h.index()).data);
    }

    bool has_attribute(std::string_view name) const { return find(name) != attribs_.size(); }

    void resize(std::size_t count) {
        if (count > capacity_)
            throw std::out_of_range("ParticleStore::resize: " + std::to_string(count) + " particles requested, " +
                                    std::to_string(capacity_) + " is the capacity");
        count_ = count;
    }
    std::size_t count() const noexcept { return count_; }
    std::size_t capacity() const noexcept { return capacity_; }
    cudaStream_t stream() const noexcept { return stream_; }

private:
    static constexpr std::size_t kAlign = 256;
    static constexpr std::size_t padded(std::size_t b) noexcept { return (b + kAlign - 1) / kAlign * kAlign; }

    struct Attrib {
        std::string name;
        AttribType type;
        unsigned char* data;  // inside one of blocks_
    };

    // index of the attribute called `name`, or attribs_.size()
    std::size_t find(std::string_view name) const {
        std::size_t k = 0;
        while (k < attribs_.size() && attribs_[k].name != name) ++k;
        return k;
    }
    const Attrib& slot(std::size_t index) const {
        if (index >= attribs_.size()) throw std::out_of_range("ParticleStore: no attribute behind this handle");
        return attribs_[index];
    }
    void reserve_block(std::size_t bytes) {
        blocks_.emplace_back(bytes, stream_);
        used_ = 0;
    }
    // `bytes` of the current block's free tail, or of a new block
    unsigned char* carve(std::size_t bytes) {
        const std::size_t need = padded(bytes);
        if (blocks_.empty() || used_ + need > blocks_.back().size()) reserve_block(need);
        unsigned char* p = blocks_.back().data() + used_;
        used_ += need;
        return p;
    }

    std::size_t capacity_;
    std::size_t count_ = 0;
    cudaStream_t stream_;
    std::vector<DeviceBuffer<unsigned char>> blocks_;
    std::size_t used_ = 0;  // bytes taken from blocks_.back()
    std::vector<Attrib> attribs_;
    AttribHandle<Vec3f> position_;
    AttribHandle<Vec3f> velocity_;
};

}  // namespace water

// WATER_CUDA_CHECK: run a CUDA runtime call and throw std::runtime_error with
// the call, file and line when it fails (the reference's error contract,
// core/include/water/core/cuda_check.h:10-36).
#pragma once

#include <cuda_runtime.h>

#include <stdexcept>
#include <string>

namespace water::detail {

[[noreturn]] inline void cuda_throw(cudaError_t err, const char* expr, const char* file, int line) {
    throw std::runtime_error(std::string("CUDA error at ") + file + ":" + std::to_string(line) + "\n  call: " +
                             expr + "\n  err:  " + cudaGetErrorString(err));
}

}  // namespace water::detail

#define WATER_CUDA_CHECK(expr)                                                     \
    do {                                                                           \
        cudaError_t _water_e = (expr);                                             \
        if (_water_e != cudaSuccess)                                               \
            ::water::detail::cuda_throw(_water_e, #expr, __FILE__, __LINE__);      \
    } while (0)

#define WATER_CUDA_CHECK_LAST()                                                    \
    do {                                                                           \
        cudaError_t _water_e = cudaGetLastError();                                 \
        if (_water_e != cudaSuccess)                                               \
            ::water::detail::cuda_throw(_water_e, "cudaGetLastError", __FILE__, __LINE__); \
    } while (0)

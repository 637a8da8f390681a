// The reciprocal that centres the reference's 27-cell stencil.
//
// Every reference neighbour kernel evaluates `1.0f / cell_length` on the device
// (solvers/dfsph/src/dfsph_kernels.cu:52,89,101,138,...) and the reference is
// built with -use_fast_math (CMakeLists.txt:56), while particles are binned with
// the host's IEEE reciprocal (core/src/cell_grid.cu:81). This translation unit
// is compiled with -use_fast_math so that the same expression yields the same
// value; the rest of the library is compiled without it. Near a cell face the
// two reciprocals can put a particle's stencil centre one cell away from the
// cell it is binned in, and reproducing that keeps neighbour sets identical to
// the reference's.
#include <cuda_runtime.h>

#include "common.cuh"

namespace dfsph {

namespace {
__global__ void stencil_reciprocal_kernel(float cell_length, float* out) { out[0] = 1.0f / cell_length; }
}  // namespace

float device_stencil_reciprocal(float cell_length, cudaStream_t stream) {
    float* d = nullptr;
    float h = 0.0f;
    DFSPH_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&d), sizeof(float), stream));
    stencil_reciprocal_kernel<<<1, 1, 0, stream>>>(cell_length, d);
    DFSPH_LAUNCHED();
    DFSPH_CUDA(cudaMemcpyAsync(&h, d, sizeof(float), cudaMemcpyDeviceToHost, stream));
    DFSPH_CUDA(cudaFreeAsync(d, stream));
    DFSPH_CUDA(cudaStreamSynchronize(stream));
    return h;
}

}  // namespace dfsph

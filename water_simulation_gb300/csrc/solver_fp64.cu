// FP64 instantiation of the same kernels: the GPU oracle build.
#include "solver.cuh"

namespace dfsph {

std::unique_ptr<SolverBase> make_solver_fp64(const dfsph_config& cfg, int device, cudaStream_t s) {
    return std::unique_ptr<SolverBase>(new Solver<double>(cfg, device, s));
}

}  // namespace dfsph

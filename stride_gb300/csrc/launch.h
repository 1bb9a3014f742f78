// Host-side launchers of the templated step kernels (one translation unit per operator kind).
#pragma once
#include "common.cuh"

namespace sa {
cudaError_t launch_step2d_k0(bool ot4, int nt_threads, dim3 grid, cudaStream_t s, const Step2D& a);
cudaError_t launch_step2d_k1(bool ot4, int nt_threads, dim3 grid, cudaStream_t s, const Step2D& a);
cudaError_t launch_step2d_k2(bool ot4, int nt_threads, dim3 grid, cudaStream_t s, const Step2D& a);

inline cudaError_t launch_step2d(int kind, bool ot4, int nt_threads, dim3 grid, cudaStream_t s, const Step2D& a) {
    switch (kind) {
        case 0: return launch_step2d_k0(ot4, nt_threads, grid, s, a);
        case 1: return launch_step2d_k1(ot4, nt_threads, grid, s, a);
        default: return launch_step2d_k2(ot4, nt_threads, grid, s, a);
    }
}
}  // namespace sa

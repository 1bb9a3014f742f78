// Launchers of the 2D step passes for operator kind 0: the Laplacian (density none). One
// translation unit per kind so the build compiles them in parallel.
#include "fdtd2d.cuh"
#include "launch.h"

namespace sa {

template <int MODE>
static cudaError_t pass(int nt, dim3 grid, cudaStream_t s, const Step2D& a) {
    static bool configured = false;
    if (!configured) {
        const int most = (int)PassCfg<0, MODE>::bytes(STEP_MAX_THREADS);
        cudaError_t e = cudaFuncSetAttribute(fdtd2d_pass<0, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
        if (e != cudaSuccess) return e;
        e = cudaFuncSetAttribute(fdtd2d_pass<0, MODE>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    fdtd2d_pass<0, MODE><<<grid, nt, PassCfg<0, MODE>::bytes(nt), s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_step2d_k0(bool ot4, int nt_threads, dim3 grid, cudaStream_t s, const Step2D& a) {
    if (nt_threads < STEP_MIN_THREADS || nt_threads > STEP_MAX_THREADS) return cudaErrorInvalidValue;
    if (!ot4) return pass<PASS_U2>(nt_threads, grid, s, a);
    const cudaError_t e = pass<PASS_L>(nt_threads, grid, s, a);
    return e != cudaSuccess ? e : pass<PASS_U4>(nt_threads, grid, s, a);
}

}  // namespace sa

// Instantiations of the 2D step kernel for operator kind 0 (0 laplace, 1 variable density,
// 2 constant density); split per kind so the build compiles them in parallel.
#include "fdtd2d.cuh"
#include "launch.h"

namespace sa {

#ifndef SA_RB
#define SA_RB 2
#endif
constexpr int RB = SA_RB;  // rows per iteration
#ifndef SA_PF
#define SA_PF 2
#endif
constexpr int PF = SA_PF;  // iterations prefetched ahead

template <bool OT4, int NT>
static cudaError_t go(dim3 grid, cudaStream_t s, const Step2D& a) {
    constexpr size_t bytes = Smem2D<0, OT4, NT, RB, PF>::bytes;
    static bool configured = false;
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(fdtd2d_step<0, OT4, NT, RB, PF>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
        if (e != cudaSuccess) return e;
        e = cudaFuncSetAttribute(fdtd2d_step<0, OT4, NT, RB, PF>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    fdtd2d_step<0, OT4, NT, RB, PF><<<grid, NT, bytes, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_step2d_k0(bool ot4, int nt_threads, dim3 grid, cudaStream_t s, const Step2D& a) {
    switch (nt_threads) {
        case 96: return ot4 ? go<true, 96>(grid, s, a) : go<false, 96>(grid, s, a);
        case 128: return ot4 ? go<true, 128>(grid, s, a) : go<false, 128>(grid, s, a);
        case 160: return ot4 ? go<true, 160>(grid, s, a) : go<false, 160>(grid, s, a);
        case 192: return ot4 ? go<true, 192>(grid, s, a) : go<false, 192>(grid, s, a);
        case 256: return ot4 ? go<true, 256>(grid, s, a) : go<false, 256>(grid, s, a);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace sa

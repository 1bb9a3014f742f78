// Instantiations of the 3D passes for operator kind 1 (0 laplace, 1 variable density,
// 2 constant density).
#include "fdtd3d.cuh"
#include "launch.h"

namespace sa {

namespace {
constexpr int RB = kRows3d, PF = kPrefetch3d;

template <int TY, int TZ, bool FINAL, bool OT4, int LANES>
cudaError_t go(dim3 grid, cudaStream_t s, const Step3D& a) {
    constexpr size_t bytes = Smem3D<1, TY, TZ, RB, PF, LANES>::bytes;
    static bool configured = false;
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(fdtd3d_pass<1, FINAL, OT4, TY, TZ, RB, PF, LANES>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    fdtd3d_pass<1, FINAL, OT4, TY, TZ, RB, PF, LANES><<<grid, TY * TZ, bytes, s>>>(a);
    return cudaGetLastError();
}

template <int TY, int TZ, int LANES>
cudaError_t go_lanes(bool final_pass, bool ot4, dim3 grid, cudaStream_t s, const Step3D& a) {
    if (!final_pass) return go<TY, TZ, false, true, LANES>(grid, s, a);
    return ot4 ? go<TY, TZ, true, true, LANES>(grid, s, a) : go<TY, TZ, true, false, LANES>(grid, s, a);
}

template <int TY, int TZ>
cudaError_t go_tile(int lanes, bool final_pass, bool ot4, dim3 grid, cudaStream_t s, const Step3D& a) {
    return lanes == 1 ? go_lanes<TY, TZ, 1>(final_pass, ot4, grid, s, a) : go_lanes<TY, TZ, 2>(final_pass, ot4, grid, s, a);
}
}  // namespace

cudaError_t launch_step3d_k1(int tile, int lanes, bool final_pass, bool ot4, dim3 grid, cudaStream_t s,
                             const Step3D& a) {
    static_assert(kTiles3dN == 2, "tile list");
    if (tile == 1) return go_tile<kTiles3d[1].ty, kTiles3d[1].tz>(lanes, final_pass, ot4, grid, s, a);
    return go_tile<kTiles3d[0].ty, kTiles3d[0].tz>(lanes, final_pass, ot4, grid, s, a);
}

}  // namespace sa

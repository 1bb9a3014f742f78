// Host-side launchers of the templated step kernels (one translation unit per operator kind).
#pragma once
#include "common.cuh"

namespace sa {
cudaError_t launch_step2d_k0(bool ot4, int nt_threads, dim3 grid, cudaStream_t s, const Step2D& a);
cudaError_t launch_step2d_k1(bool ot4, int nt_threads, dim3 grid, cudaStream_t s, const Step2D& a);
cudaError_t launch_step2d_k2(bool ot4, int nt_threads, dim3 grid, cudaStream_t s, const Step2D& a);

struct Step3D;
// (y, z) tiles of a 3D CTA (threads = their product), chosen per plan (sa_autotune measures them)
struct Tile3D {
    int ty, tz;
};
constexpr Tile3D kTiles3d[] = {{16, 32}, {8, 32}};
constexpr int kTiles3dN = 2;
cudaError_t launch_step3d_k0(int tile, int lanes, bool final_pass, bool ot4, dim3 grid, cudaStream_t s,
                             const Step3D& a);
cudaError_t launch_step3d_k1(int tile, int lanes, bool final_pass, bool ot4, dim3 grid, cudaStream_t s,
                             const Step3D& a);
cudaError_t launch_step3d_k2(int tile, int lanes, bool final_pass, bool ot4, dim3 grid, cudaStream_t s,
                             const Step3D& a);
#ifndef SA_RB3
#define SA_RB3 2
#endif
#ifndef SA_PF3
#define SA_PF3 1
#endif
constexpr int kRows3d = SA_RB3, kPrefetch3d = SA_PF3;  // x rows per iteration of a 3D pass, iterations prefetched

// lanes 2: a.npairs pairs from shot a.shot0; lanes 1: the lone shot a.shot0
inline cudaError_t launch_step3d(int kind, int tile, int lanes, bool final_pass, bool ot4, dim3 grid, cudaStream_t s,
                                 const Step3D& a) {
    switch (kind) {
        case 0: return launch_step3d_k0(tile, lanes, final_pass, ot4, grid, s, a);
        case 1: return launch_step3d_k1(tile, lanes, final_pass, ot4, grid, s, a);
        default: return launch_step3d_k2(tile, lanes, final_pass, ot4, grid, s, a);
    }
}

// One 2D time step of a batch: OT4 launches pass L then pass U, OT2 pass U (fdtd2d.cuh);
// nt_threads in [STEP_MIN_THREADS, STEP_MAX_THREADS], two grid columns per thread.
inline cudaError_t launch_step2d(int kind, bool ot4, int nt_threads, dim3 grid, cudaStream_t s, const Step2D& a) {
    switch (kind) {
        case 0: return launch_step2d_k0(ot4, nt_threads, grid, s, a);
        case 1: return launch_step2d_k1(ot4, nt_threads, grid, s, a);
        default: return launch_step2d_k2(ot4, nt_threads, grid, s, a);
    }
}
}  // namespace sa

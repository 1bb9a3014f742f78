// Host launchers of the plan's helper kernels (helpers.cu).
#pragma once
#include "common.cuh"

namespace sa {
// Sponge ramps of the two axes (1/m), per distance to the edge.
struct Sponge {
    int a[2];
    float s[2][MAX_ABS];
};
cudaError_t medium2d(const float* vp_in, const float* rho_in, const float* alpha_in, int nx, int ny, int pitch,
                     int pitch_b, int density, double db_to_np, const Sponge& sp, float dt, float* W, float* vp,
                     float* alpha, float* buoy, float* bxh, float* byh, float* C1, float* C2, float* C3,
                     cudaStream_t s);
void set_last_error(const char* msg);
cudaError_t transpose(const float* in, int rows, int cols, float* out, cudaStream_t s);
cudaError_t final_gather2d(const float* field, long long shot_stride, int pitch, const Gather* g, int n, float* out,
                           int ld, int trow, cudaStream_t s);
cudaError_t reduce_shots(const float* buf, long long shot_stride, int nshots, int nx, int ny, int pitch, float* out,
                         cudaStream_t s);
}  // namespace sa

// Shared definitions of the GB300 iso-acoustic FDTD kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace sa {

constexpr int MAX_ABS = 64;  // longest sponge (cells) the on-the-fly damping tables hold

// 10th-order centred 2nd-derivative weights (Fornberg) for Devito's `laplace` at space order 10
// (stride/physics/iso_acoustic/devito.py:1652).
__host__ __device__ constexpr float kW2(int k) {
    return k == 0 ? (float)(-5269.0 / 1800.0)
         : k == 1 ? (float)(5.0 / 3.0)
         : k == 2 ? (float)(-5.0 / 21.0)
         : k == 3 ? (float)(5.0 / 126.0)
         : k == 4 ? (float)(-5.0 / 1008.0)
                  : (float)(1.0 / 3150.0);
}

// 10th-order staggered 1st-derivative weights at offsets k+1/2 (antisymmetric), for Devito's
// grad(shift=+1/2) / div(shift=-1/2) (iso_acoustic/devito.py:1655-1663).
__host__ __device__ constexpr float kWS(int k) {
    return k == 0 ? (float)(19845.0 / 16384.0)
         : k == 1 ? (float)(-735.0 / 8192.0)
         : k == 2 ? (float)(567.0 / 40960.0)
         : k == 3 ? (float)(-405.0 / 229376.0)
                  : (float)(35.0 / 294912.0);
}

// 10th-order centred first-derivative weights c_1..c_5 (c_-k = -c_k): Devito's Derivative(f, (d, 1))
// at space order 10, the CFS-PML's u_di (stride/physics/boundaries/devito.py:131).
__host__ __device__ constexpr float kW1(int k) {
    return k == 1 ? (float)(5.0 / 6.0)
         : k == 2 ? (float)(-5.0 / 21.0)
         : k == 3 ? (float)(5.0 / 84.0)
         : k == 4 ? (float)(-5.0 / 504.0)
                  : (float)(1.0 / 1260.0);
}

constexpr int GUARD = 40;  // zero rows above and below every pitched medium array (>= 3R + RB + 5)

// A receiver with Hicks interpolation: 8 x 8 support from (row, col), weights wx[i] * wy[j].
struct HicksGather {
    int row, col, point, shot;
    float wx[8], wy[8];
};

// One point of a gather: rec[t][point] = sum of the four bilinear corner terms; `pad` is the
// point's shot (its pair is pad / 2, its lane pad % 2).
struct Gather {
    int row, col, point, pad;
    float w00, w01, w10, w11;
};

// Arguments of one 2D time step over a batch of shots.
struct Step2D {
    int nx, ny, pitch;        // extended grid, row pitch (columns)
    long long shot_stride;    // float2 elements per shot pair in a field buffer (nx * pitch)
    int chunk_rows;           // output rows per CTA
    int by;                   // output columns per CTA (even, <= Cols2D::BYMAX)
    int t;                    // time index of the current level (cur = p[t])
    const float* cur;         // p[t] of shot pairs, interleaved: [pairs][nx][pitch][2]
    float* prev;              // other level in, new level out (in place)
    // medium (shared by all shots); pointers address row 0, GUARD zero rows on both sides
    const float* W;           // node coefficient: vp^2 (density none/constant) or vp^2 rho
    const float* bxh;         // buoyancy at (x+1/2, y), half-rows -5..nx+3 valid
    const float* byh;         // buoyancy at (x, y+1/2): column y+6 holds y = -6..ny+3
    int pitch_b;
    const float* C1;          // update p_new = C1 Lt + C2 p - C3 p_other (damping, attenuation)
    const float* C2;
    const float* C3;
    float hx, hy;             // spacing
    float dt;
    // wavefield save (forward); sources, receivers and the imaging condition are separate kernels
    int f;                    // undersampling factor
    int save;                 // forward, on t % f == 0: 1 stores p.dt2, 2 stores p[t] itself
    float* snaps;             // [pairs][n_snap][nx][pitch][2]
    long long snap_shot_stride, snap_stride;  // in float2 elements: per pair, per snapshot
};

}  // namespace sa

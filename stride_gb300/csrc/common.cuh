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

// Points per axis of the widest sparse-point support (sinc of half-width 7).
constexpr int SUPPORT_MAX = 14;

// A point with a wide support (Hicks or sinc interpolation): width x width points from (row, col),
// weights wx[i] * wy[j].
struct SupportGather {
    int row, col, point, shot, width;
    float wx[SUPPORT_MAX], wy[SUPPORT_MAX];
};

// One point of a gather: rec[t][point] = sum of the four bilinear corner terms; `pad` is the
// point's shot (its pair is pad / 2, its lane pad % 2).
struct Gather {
    int row, col, point, pad;
    float w00, w01, w10, w11;
};

// Arguments of one 2D time step over a batch of shots (the passes of fdtd2d.cuh).
struct Step2D {
    int nx, ny, pitch;         // extended grid, field row pitch (columns)
    long long shot_stride;     // float2 elements per shot pair in a field buffer (nx * pitch)
    int chunk_rows;            // output rows per CTA
    int by;                    // output columns per CTA (even, at most twice the threads)
    int t;                     // time index of the current level (cur = p[t])
    const float* cur;          // p[t] of shot pairs, interleaved: [pairs][nx][pitch][2]
    float* prev;               // other level in, new level out (in place)
    float* lbuf;               // OT4: l = W G(p[t]) of the first pass (same layout; zero beyond ny)
    // medium: point (x, y) of array m at m[x * mpitch + y] (pointers at row 0, column 0; MED_GUARD
    // rows above and below, MED_MARGIN columns left and right); a thread loads columns (c, c + 1)
    // of a field as one float2 and uses each value for both shots of its pair
    const float* Wm;           // vp^2 (density none or constant) or vp^2 rho
    const float* bxm;          // buoyancy at (x + 1/2, y)
    const float* bym;          // buoyancy at (x, y + 1/2)
    const float* C1m;          // new = C1 Lt + C2 p + NC3 p_other, NC3 = -C3 (damping, attenuation)
    const float* C2m;
    const float* NC3m;
    int mpitch;                // floats per medium row
    int ymax;                  // largest (even) medium column a thread may address
    float2 wx[6], wy[6];       // FD weights over h (staggered: 5) or over h^2 (laplace: 6), {w, w}
    float k12;                 // dt^2 / 12
    int wg_only;               // 1: new level = W G(p[t]) (OT2; the exact adjoint's W G pass)
    int f;                     // undersampling factor
    int save;                  // forward, on t % f == 0: 1 stores p.dt2, 2 stores p[t] itself
    float inv_dt2;
    float* snaps;              // [pairs][n_snap][nx][pitch][2]
    long long snap_shot_stride, snap_stride;  // in float2 elements: per pair, per snapshot
};

constexpr int MED_GUARD = 40;   // rows of the step passes' medium beyond the grid, each side
constexpr int MED_MARGIN = 32;  // columns of the step passes' medium beyond the grid, each side
constexpr int STEP_MAX_THREADS = 128;  // threads per CTA of the 2D passes (two columns each), at most
constexpr int STEP_MIN_THREADS = 16;   // and at least

}  // namespace sa

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

// One corner contribution of an injected point (source in the forward, receiver in the
// adjoint). The injected value is coef * amp[t][point] * vp(row,col)^vp_power.
struct Inject {
    int row, col, point;
    float coef;
};

// One receiver of a gather: rec[t][point] = sum of the four bilinear corner terms.
struct Gather {
    int row, col, point, pad;
    float w00, w01, w10, w11;
};

// Arguments of one 2D time step over a batch of shots.
struct Step2D {
    int nx, ny, pitch;        // extended grid, row pitch (floats)
    long long shot_stride;    // floats between shots in a field buffer
    int chunk_rows;           // output rows per CTA
    int by;                   // output columns per CTA (<= NT - 2*halo)
    int t;                    // time index of the current level (cur = p[t])
    int adjoint;              // 0: p[t+1] from p[t], p[t-1];  1: p_a[t-1] from p_a[t], p_a[t+1]
    const float* cur;         // p[t]                      [shots][nx][pitch]
    float* prev;              // other level in, new level out (in place)
    // medium
    const float* W;           // node coefficient: vp^2 (density none/constant) or vp^2 rho
    const float* vp;
    const float* alpha;       // Np/m or nullptr
    const float* bxh;         // buoyancy at (x+1/2, y), x = -5..nx+3 stored at row x+5, pitch
    const float* byh;         // buoyancy at (x, y+1/2), y = -5..ny+3 stored at col y+5, pitch_b
    int pitch_b;
    float hx, hy;             // spacing
    float dt;
    float sx[MAX_ABS], sy[MAX_ABS];  // damping ramp per distance to the edge, in 1/m
    int ax, ay;               // absorbing widths
    // sparse points (CSR over CTAs in launch order: shot-major, then chunk, then strip)
    const Inject* inj;
    const int* inj_off;
    const float* inj_amp;     // [nt][n_inj_points] time-major amplitudes
    int inj_ld;               // leading dimension of inj_amp
    int inj_vp_power;         // 1: forward source (vp), 2: adjoint receiver (vp^2)
    const Gather* gat;
    const int* gat_off;
    float* gat_out;           // [nt][n_gather_points]
    int gat_ld;
    // wavefield save (forward) / imaging condition (adjoint)
    int f;                    // undersampling factor
    int save;                 // forward: store p.dt2 on t % f == 0
    int grad;                 // adjoint: accumulate grad/prec on t % f == 0
    float* snaps;             // [shots][n_snap][nx][pitch]
    long long snap_shot_stride, snap_stride;
    float* gradb;             // [shots][nx][pitch]
    float* precb;
    int ix0, ix1, iy0, iy1;   // interior (imaging condition) bounds
};

}  // namespace sa

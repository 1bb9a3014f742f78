// 2D iso-acoustic FDTD time step for sm_103a: one launch advances every shot of a batch by one
// time level. Restates the Devito operator that IsoAcousticDevito builds
// (stride/physics/iso_acoustic/devito.py:1466-1608) as a streaming kernel:
//
//  * a CTA owns a strip of `by` output columns (the contiguous y axis) and a chunk of rows of
//    one shot, and streams the rows of the current level p[t] through shared memory one row
//    per iteration (coalesced row loads, zero halo beyond the grid as Devito's p halo);
//  * derivatives along the streamed x axis come from per-thread register queues (2.5D
//    streaming), derivatives along y from the shared row;
//  * OT4 (L + dt^2/12 L(L p)) is fused: the first application's rows feed a second pipeline
//    stage `R` rows behind, so the intermediate never touches memory;
//  * the sponge damping (boundaries/devito.py:49-67) is evaluated on the fly from two 1D
//    ramps, attenuation (devito.py:1536-1548) from alpha, the update solves
//    p.dt2 - Lt + 2 a vp p.dt + vp^2 (2 d p.dtc + d^2 p) = 0 (devito.py:1575-1581);
//  * source injection (devito.py:357-363), receiver interpolation (:364), the undersampled
//    p.dt2 save (:398-418) and the adjoint receiver injection / vp imaging condition
//    (:748-753, :1000-1024) are fused epilogues with per-CTA point lists (no atomics).
//
// The new level is written in place of the older one (each point's p[t-1] is read only by
// the thread that writes p[t+1] there), so a shot needs two field buffers.
#pragma once
#include "common.cuh"

namespace sa {

__device__ __forceinline__ float sponge2d(const Step2D& a, int x, int y) {
    // Boundary.damping (stride/physics/boundaries/boundary.py:116-160): the x slab at layer e
    // covers y layers >= e and vice versa, so corner points take the outer slab (both on the
    // diagonal).
    const int ex = min(x, a.nx - 1 - x), ey = min(y, a.ny - 1 - y);
    float s = 0.f;
    if (ex < a.ax && ex <= ey) s += a.sx[ex];
    if (ey < a.ay && ey <= ex) s += a.sy[ey];
    return s;
}

template <int KIND, bool OT4, int NT>
__global__ void __launch_bounds__(NT) fdtd2d_step(const __grid_constant__ Step2D a) {
    constexpr bool STAG = KIND != 0;        // staggered div(b grad) operator
    constexpr bool VARB = KIND == 1;        // variable buoyancy
    constexpr int R = STAG ? 9 : 5;         // radius of one operator application
    constexpr int S = OT4 ? 2 : 1;          // pipeline stages
    constexpr int H1 = (S - 1) * R;         // halo of the stage-1 output columns
    constexpr int C0 = NT + 2 * R;          // stage-1 input columns in shared memory
    constexpr int P = STAG ? 10 : 11;       // register queue period
    constexpr int NF1 = NT + 9;             // stage-1 half-column fluxes

    __shared__ float su[2][C0];
    __shared__ float sF[2][STAG ? NF1 : 1];
    __shared__ float sl[2][OT4 ? NT : 1];
    __shared__ float sF2[2][(OT4 && STAG) ? NT : 1];

    const int tid = threadIdx.x;
    const int strip = blockIdx.x, chunk = blockIdx.y, shot = blockIdx.z;
    const int BY = a.by;
    const int y0 = strip * BY;
    const int L1 = y0 - H1;  // first stage-1 output column
    const int L0 = L1 - R;   // first stage-1 input column
    const int c = L1 + tid;  // this thread's column
    const bool c_in = (c >= 0) && (c < a.ny);
    const bool out_col = (tid >= H1) && (tid < H1 + BY) && c_in;
    const int cc = min(max(c, 0), a.ny - 1);
    const int xo0 = chunk * a.chunk_rows;
    const int xo1 = min(a.nx, xo0 + a.chunk_rows);
    const int i0 = xo0 - S * R, i1 = xo1 + S * R;
    const int pitch = a.pitch;

    const long long soff = (long long)shot * a.shot_stride;
    const float* __restrict__ cur = a.cur + soff;
    float* __restrict__ prev = a.prev + soff;
    const float* __restrict__ Wm = a.W;
    const float* __restrict__ bxh = a.bxh;
    const float* __restrict__ byh = a.byh;

    const int cta = (shot * gridDim.y + chunk) * gridDim.x + strip;
    const int inj_b = a.inj ? a.inj_off[cta] : 0, inj_e = a.inj ? a.inj_off[cta + 1] : 0;
    const int gat_b = a.gat ? a.gat_off[cta] : 0, gat_e = a.gat ? a.gat_off[cta + 1] : 0;

    const float ihx = 1.f / a.hx, ihy = 1.f / a.hy;
    const float ihx2 = 1.f / (a.hx * a.hx), ihy2 = 1.f / (a.hy * a.hy);
    const float dt = a.dt, dt2 = a.dt * a.dt;
    const float k12 = (float)((double)a.dt * (double)a.dt / 12.0);

    float uq[P], gq[P];
    float fq[STAG ? P : 1];
    float lq[OT4 ? P : 1], g2q[OT4 ? P : 1], f2q[(OT4 && STAG) ? P : 1];
#pragma unroll
    for (int k = 0; k < P; k++) {
        uq[k] = 0.f;
        gq[k] = 0.f;
        if constexpr (STAG) fq[k] = 0.f;
        if constexpr (OT4) {
            lq[k] = 0.f;
            g2q[k] = 0.f;
            if constexpr (STAG) f2q[k] = 0.f;
        }
    }
    int inj_ptr = inj_b;
    const bool do_save = a.save && (a.t % a.f == 0);
    const bool do_grad = a.grad && (a.t % a.f == 0);

#define SL(lag) ((((ph) - (lag)) % P + 2 * P) % P)

    for (int ib = i0; ib < i1; ib += P) {
#pragma unroll
        for (int ph = 0; ph < P; ph++) {
            const int i = ib + ph;
            if (i < i1) {
                const int buf = i & 1;
                // ---- load row i of p[t] (zero halo) -------------------------------------
                const bool row_in = (i >= 0) && (i < a.nx);
                for (int k = tid; k < C0; k += NT) {
                    const int col = L0 + k;
                    float v = 0.f;
                    if (row_in && col >= 0 && col < a.ny) v = cur[(long long)i * pitch + col];
                    su[buf][k] = v;
                }
                __syncthreads();

                // ---- receiver interpolation of p[t] -> rec[t-1] (rows i-1 and i) ----------
                for (int e = gat_b + tid; e < gat_e; e += NT) {
                    const Gather G = a.gat[e];
                    if (G.row + 1 == i) {
                        const int k0 = G.col - L0;
                        const float v = G.w00 * su[buf ^ 1][k0] + G.w01 * su[buf ^ 1][k0 + 1] +
                                        G.w10 * su[buf][k0] + G.w11 * su[buf][k0 + 1];
                        a.gat_out[(long long)(a.t - 1) * a.gat_ld + G.point] = v;
                    }
                }

                // ---- stage 1: l = W * G(u) at row j = i - R --------------------------------
                uq[SL(0)] = su[buf][tid + R];
                float gy;
                if constexpr (STAG) {
                    const int ir = min(max(i, 0), a.nx - 1);
                    for (int k = tid; k < NF1; k += NT) {
                        float v = 0.f;
#pragma unroll
                        for (int m = 0; m < 5; m++) v += kWS(m) * (su[buf][k + 5 + m] - su[buf][k + 4 - m]);
                        v = v * ihy;
                        if constexpr (VARB) {
                            const int jh = min(max(L1 - 5 + k, -5), a.ny + 3);
                            v = v * __ldg(&byh[(long long)ir * a.pitch_b + jh + 5]);
                        }
                        sF[buf][k] = v;
                    }
                    __syncthreads();
                    float v = 0.f;
#pragma unroll
                    for (int m = 0; m < 5; m++) v += kWS(m) * (sF[buf][tid + 5 + m] - sF[buf][tid + 4 - m]);
                    gy = v * ihy;
                } else {
                    float v = kW2(0) * su[buf][tid + R];
#pragma unroll
                    for (int k = 1; k <= 5; k++) v += kW2(k) * (su[buf][tid + R + k] + su[buf][tid + R - k]);
                    gy = v * ihy2;
                }
                gq[SL(0)] = gy;

                float gx;
                if constexpr (STAG) {
                    float v = 0.f;
#pragma unroll
                    for (int m = 0; m < 5; m++) v += kWS(m) * (uq[SL(4 - m)] - uq[SL(5 + m)]);
                    v = v * ihx;
                    if constexpr (VARB) {
                        const int xh = min(max(i - 5, -5), a.nx + 3);
                        v = v * __ldg(&bxh[(long long)(xh + 5) * pitch + cc]);
                    }
                    fq[SL(0)] = v;
                    float w = 0.f;
#pragma unroll
                    for (int k = 0; k < 5; k++) w += kWS(k) * (fq[SL(4 - k)] - fq[SL(5 + k)]);
                    gx = w * ihx;
                } else {
                    float v = kW2(0) * uq[SL(5)];
#pragma unroll
                    for (int k = 1; k <= 5; k++) v += kW2(k) * (uq[SL(5 - k)] + uq[SL(5 + k)]);
                    gx = v * ihx2;
                }
                const int j = i - R;
                float lj = 0.f;  // the intermediate has a zero halo (Devito `laplacian` Function)
                if (j >= 0 && j < a.nx && c_in) lj = __ldg(&Wm[(long long)j * pitch + c]) * (gx + gq[SL(R)]);

                // ---- stage 2 (OT4): Lt = l + dt^2/12 W G(l) at row o = j - R -------------
                float Lt;
                int o;
                if constexpr (OT4) {
                    sl[buf][tid] = lj;
                    lq[SL(0)] = lj;
                    __syncthreads();
                    float gy2 = 0.f;
                    const bool s2 = (tid >= H1) && (tid < H1 + BY);
                    if constexpr (STAG) {
                        const int jr = min(max(j, 0), a.nx - 1);
                        for (int k = tid; k < BY + 9; k += NT) {
                            float v = 0.f;
#pragma unroll
                            for (int m = 0; m < 5; m++) v += kWS(m) * (sl[buf][k + 5 + m] - sl[buf][k + 4 - m]);
                            v = v * ihy;
                            if constexpr (VARB) {
                                const int jh = min(max(y0 - 5 + k, -5), a.ny + 3);
                                v = v * __ldg(&byh[(long long)jr * a.pitch_b + jh + 5]);
                            }
                            sF2[buf][k] = v;
                        }
                        __syncthreads();
                        if (s2) {
                            const int q = tid - H1;
                            float v = 0.f;
#pragma unroll
                            for (int m = 0; m < 5; m++) v += kWS(m) * (sF2[buf][q + 5 + m] - sF2[buf][q + 4 - m]);
                            gy2 = v * ihy;
                        }
                    } else {
                        if (s2) {
                            float v = kW2(0) * sl[buf][tid];
#pragma unroll
                            for (int k = 1; k <= 5; k++) v += kW2(k) * (sl[buf][tid + k] + sl[buf][tid - k]);
                            gy2 = v * ihy2;
                        }
                    }
                    g2q[SL(0)] = gy2;
                    float gx2;
                    if constexpr (STAG) {
                        float v = 0.f;
#pragma unroll
                        for (int m = 0; m < 5; m++) v += kWS(m) * (lq[SL(4 - m)] - lq[SL(5 + m)]);
                        v = v * ihx;
                        if constexpr (VARB) {
                            const int xh = min(max(j - 5, -5), a.nx + 3);
                            v = v * __ldg(&bxh[(long long)(xh + 5) * pitch + cc]);
                        }
                        f2q[SL(0)] = v;
                        float w = 0.f;
#pragma unroll
                        for (int k = 0; k < 5; k++) w += kWS(k) * (f2q[SL(4 - k)] - f2q[SL(5 + k)]);
                        gx2 = w * ihx;
                    } else {
                        float v = kW2(0) * lq[SL(5)];
#pragma unroll
                        for (int k = 1; k <= 5; k++) v += kW2(k) * (lq[SL(5 - k)] + lq[SL(5 + k)]);
                        gx2 = v * ihx2;
                    }
                    o = j - R;
                    Lt = 0.f;
                    if (o >= 0 && o < a.nx && c_in)
                        Lt = lq[SL(R)] + k12 * (__ldg(&Wm[(long long)o * pitch + c]) * (gx2 + g2q[SL(R)]));
                } else {
                    o = j;
                    Lt = lj;
                }

                // ---- update of row o, fused epilogues -----------------------------------
                if (o >= xo0 && o < xo1 && out_col) {
                    const long long idx = (long long)o * pitch + c;
                    float u_o;
                    if constexpr (OT4) u_o = cur[idx];
                    else u_o = uq[SL(R)];
                    const float pm = prev[idx];
                    const float vpv = __ldg(&a.vp[idx]);
                    const float vp2 = vpv * vpv;
                    const float d = 7.f * (sponge2d(a, o, c) * vpv) * dt;
                    float beta = vp2 * d;
                    if (a.alpha) beta = beta + __ldg(&a.alpha[idx]) * vpv;
                    beta = dt * beta;
                    const float num = dt2 * Lt + (2.f - dt2 * vp2 * d * d) * u_o - (1.f - beta) * pm;
                    float pn = num / (1.f + beta);
                    // injection into the new level (sources forward, receivers adjoint)
                    while (inj_ptr < inj_e && a.inj[inj_ptr].row < o) inj_ptr++;
                    for (int q = inj_ptr; q < inj_e; q++) {
                        const Inject E = a.inj[q];
                        if (E.row != o) break;
                        if (E.col == c) {
                            const float vpow = a.inj_vp_power == 2 ? vp2 : vpv;
                            pn = pn + (E.coef * a.inj_amp[(long long)a.t * a.inj_ld + E.point]) * vpow;
                        }
                    }
                    if (do_save) {
                        const long long si = (long long)shot * a.snap_shot_stride +
                                             (long long)(a.t / a.f) * a.snap_stride + idx;
                        a.snaps[si] = (pn - 2.f * u_o + pm) / dt2;
                    }
                    if (do_grad && o >= a.ix0 && o < a.ix1 && c >= a.iy0 && c < a.iy1) {
                        const long long si = (long long)shot * a.snap_shot_stride +
                                             (long long)(a.t / a.f) * a.snap_stride + idx;
                        const float sv = a.snaps[si];
                        const long long gi = (long long)shot * a.shot_stride + idx;
                        a.gradb[gi] += sv * u_o;
                        a.precb[gi] += sv * sv;
                    }
                    prev[idx] = pn;
                }
                if constexpr (!STAG && !OT4) {
                    // the receiver gather reads the other row buffer, which the next iteration
                    // overwrites; OT2/laplace has no later barrier in this iteration
                    if (gat_e > gat_b) __syncthreads();
                }
            }
        }
    }
#undef SL
}

// rec[row][point] = interp(field) for every receiver (the last forward level).
__global__ void gather_final2d(const float* __restrict__ field, long long shot_stride, int pitch,
                               const Gather* __restrict__ g, int n, float* out, int ld, int trow);

// out[p] = sum over shots of buf[shot][x][pitch] for the unpadded extended grid.
__global__ void reduce_shots2d(const float* __restrict__ buf, long long shot_stride, int nshots, int nx,
                               int ny, int pitch, float* __restrict__ out);

}  // namespace sa

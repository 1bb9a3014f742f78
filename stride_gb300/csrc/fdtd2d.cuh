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

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, bool valid) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    const int sz = valid ? 16 : 0;  // 0: zero-fill, nothing is read
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(gmem), "r"(sz) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

__host__ __device__ constexpr int round4(int x) { return (x + 3) / 4 * 4; }

// Shared-memory layout of one CTA (floats).
template <int KIND, bool OT4, int NT, int RB, int PF>
struct Smem2D {
    static constexpr bool STAG = KIND != 0;
    static constexpr int R = STAG ? 9 : 5;
    static constexpr int S = OT4 ? 2 : 1;
    static constexpr int H1 = (S - 1) * R;
    static constexpr int C0 = NT + 2 * R;
    static constexpr int NF1 = NT + 9;
    static constexpr int WU = round4(C0 + 3);   // u row (columns from floor4(L0))
    static constexpr int QU = S * R + RB * (PF + 1);  // u rows kept: o .. i + RB*(PF+1) - 1
    static constexpr int QLR = R + RB;          // rows of the intermediate kept (OT4)
    static constexpr int oU = 0;
    static constexpr int oL = oU + QU * WU;
    static constexpr int oF = oL + (OT4 ? QLR * NT : 0);
    static constexpr int oF2 = oF + (STAG ? RB * NF1 : 0);
    static constexpr int total = oF2 + ((OT4 && STAG) ? RB * NT : 0);
    static constexpr size_t bytes = (size_t)total * sizeof(float);
};

// Register queue shift by RB (the oldest RB entries leave).
template <int QL, int RB>
__device__ __forceinline__ void qshift(float (&q)[QL]) {
#pragma unroll
    for (int k = 0; k + RB < QL; k++) q[k] = q[k + RB];
}

template <int KIND, bool OT4, int NT, int RB, int PF>
__global__ void __launch_bounds__(NT) fdtd2d_step(const __grid_constant__ Step2D a) {
    using L = Smem2D<KIND, OT4, NT, RB, PF>;
    constexpr bool STAG = L::STAG;            // staggered div(b grad) operator
    constexpr bool VARB = KIND == 1;          // variable buoyancy
    constexpr int R = L::R;                   // radius of one operator application
    constexpr int S = L::S;                   // pipeline stages
    constexpr int H1 = L::H1;                 // halo of the stage-1 output columns
    constexpr int C0 = L::C0;
    constexpr int NF1 = L::NF1;
    constexpr int QU = L::QU, QLR = L::QLR;
    // register queues along x: u rows i-QB..i+RB-1, fluxes at half-rows i-QB-5..i-6+RB (STAG)
    constexpr int QB = STAG ? 9 : 10;
    constexpr int QL = QB + RB;

    extern __shared__ __align__(16) float smem[];
    float* const sU = smem + L::oU;
    float* const sLr = smem + L::oL;
    float* const sF = smem + L::oF;
    float* const sF2 = smem + L::oF2;

    const int tid = threadIdx.x;
    const int strip = blockIdx.x, chunk = blockIdx.y, shot = blockIdx.z;
    const int BY = a.by;
    const int y0 = strip * BY;
    const int L1 = y0 - H1;  // first stage-1 output column
    const int L0 = L1 - R;   // first stage-1 input column
    const int QU0 = L0 & ~3, shU = L0 - QU0;  // u rows start at floor4(L0)
    const int c = L1 + tid;  // this thread's column
    const bool c_in = (c >= 0) && (c < a.ny);
    const bool out_col = (tid >= H1) && (tid < H1 + BY) && c_in;
    const int cc = min(max(c, 0), a.ny - 1);
    const int xo0 = chunk * a.chunk_rows;
    const int xo1 = min(a.nx, xo0 + a.chunk_rows);
    const int i0 = xo0 - S * R, i1 = xo1 + S * R;
    const int pitch = a.pitch, pitch_b = a.pitch_b;

    const long long soff = (long long)shot * a.shot_stride;
    const float* __restrict__ cur = a.cur;
    float* __restrict__ prev = a.prev + soff;

    const int cta = (shot * gridDim.y + chunk) * gridDim.x + strip;
    const int inj_b = a.inj ? a.inj_off[cta] : 0, inj_e = a.inj ? a.inj_off[cta + 1] : 0;
    const int gat_b = a.gat ? a.gat_off[cta] : 0, gat_e = a.gat ? a.gat_off[cta + 1] : 0;

    const float ihx = 1.f / a.hx, ihy = 1.f / a.hy;
    const float ihx2 = 1.f / (a.hx * a.hx), ihy2 = 1.f / (a.hy * a.hy);
    const float dt2 = a.dt * a.dt;
    const float k12 = (float)((double)a.dt * (double)a.dt / 12.0);

    // per-thread medium pointers at row 0 of this thread's column (rows beyond the grid are
    // GUARD zero rows, so no clamping in the loop)
    const float* __restrict__ pW = a.W + cc;
    const float* __restrict__ pBX = a.bxh + cc;
    const int kb1 = min(max(L1 + tid, 0), a.ny + 8);        // stage-1 flux k = tid
    const int kb1b = min(max(L1 + tid + NT, 0), a.ny + 8);  // stage-1 flux k = NT + tid (tid < 9)
    const int kb2 = min(max(y0 + tid, 0), a.ny + 8);        // stage-2 flux k = tid
    const float* __restrict__ pC1 = a.C1 + c;
    const float* __restrict__ pC2 = a.C2 + c;
    const float* __restrict__ pC3 = a.C3 + c;

    // u ring: row r in slot (r - i0) mod QU; ring indices advance incrementally
    constexpr int NQU = (C0 + 3 + 3) / 4;
    static_assert(4 * NQU == L::WU, "u row width");
    auto wrapU = [](int sl) { return sl < 0 ? sl + QU : (sl >= QU ? sl - QU : sl); };
    auto rowU = [&](int sl) { return sU + sl * L::WU + shU; };  // rowU(s)[k] = u(row, L0 + k)
    int sI = 0;  // slot of row i
    auto prefetch = [&](int ii, int slot) {
        for (int rr = 0; rr < RB; rr++) {
            const int r = ii + rr;
            if (r < i1) {
                float* dst = sU + wrapU(slot + rr) * L::WU;
                const bool row_ok = r >= 0 && r < a.nx;
                const float* rowp = cur + soff + (long long)r * pitch;
                for (int k = tid; k < NQU; k += NT) {
                    const int q = QU0 + 4 * k;
                    const bool ok = row_ok && q >= 0 && q + 4 <= pitch;
                    cp_async16(dst + 4 * k, ok ? rowp + q : cur, ok);
                }
            }
        }
        cp_async_commit();
    };

    float uq[QL], fq[STAG ? QL : 1], lq[OT4 ? QL : 1], f2q[(OT4 && STAG) ? QL : 1];
#pragma unroll
    for (int k = 0; k < QL; k++) {
        uq[k] = 0.f;
        if constexpr (STAG) fq[k] = 0.f;
        if constexpr (OT4) {
            lq[k] = 0.f;
            if constexpr (STAG) f2q[k] = 0.f;
        }
    }
    int inj_ptr = inj_b, gat_ptr = gat_b;
    const bool do_save = a.save && (a.t % a.f == 0);
    const bool do_grad = a.grad && (a.t % a.f == 0);

    for (int k = 0; k < PF; k++) prefetch(i0 + k * RB, wrapU(k * RB % QU));

    int sJ = 0;  // ring slot of intermediate row j (slot of row x is (x - (i0 - R)) mod QLR)
    for (int i = i0; i < i1; i += RB) {
        const int j = i - R;        // first stage-1 output row of this iteration
        const int o = i - S * R;    // first output row of this iteration
        // ---- per-thread medium values of this iteration, loaded before the barrier ----
        float Wj[RB], Wo[RB], bxi[RB], bxj[RB], by1[RB], by1b[RB], by2[RB], c1[RB], c2[RB], c3[RB], pmo[RB];
#pragma unroll
        for (int r = 0; r < RB; r++) {
            Wj[r] = __ldg(pW + (long long)(j + r) * pitch);
            if constexpr (OT4) Wo[r] = __ldg(pW + (long long)(o + r) * pitch);
            if constexpr (VARB) {
                bxi[r] = __ldg(pBX + (long long)(i - 5 + r) * pitch);
                if constexpr (OT4) bxj[r] = __ldg(pBX + (long long)(j - 5 + r) * pitch);
                const float* byr = a.byh + (long long)(j + r) * pitch_b;
                by1[r] = __ldg(byr + kb1);
                by1b[r] = tid < 9 ? __ldg(byr + kb1b) : 0.f;
                if constexpr (OT4) by2[r] = __ldg(a.byh + (long long)(o + r) * pitch_b + kb2);
            }
            const bool o_ok = (o + r >= xo0) && (o + r < xo1) && out_col;
            const long long orow = (long long)(o + r) * pitch;
            c1[r] = o_ok ? __ldg(pC1 + orow) : 0.f;
            c2[r] = o_ok ? __ldg(pC2 + orow) : 0.f;
            c3[r] = o_ok ? __ldg(pC3 + orow) : 0.f;
            pmo[r] = o_ok ? prev[orow + c] : 0.f;
        }
        (void)bxj; (void)by2; (void)Wo; (void)by1b; (void)bxi; (void)by1;

        cp_async_wait<PF - 1>();
        __syncthreads();  // rows i..i+RB-1 visible; every thread is done with the last iteration
        prefetch(i + PF * RB, wrapU(sI + PF * RB >= QU ? sI + PF * RB - QU : sI + PF * RB));

        // ---- receiver interpolation of p[t] -> rec[t-1]: base rows i-1 .. i+RB-2 ----------
        while (gat_ptr < gat_e && a.gat[gat_ptr].row + 1 < i) gat_ptr++;
        for (int e = gat_ptr + tid; e < gat_e; e += NT) {
            const Gather G = a.gat[e];
            if (G.row + 1 >= i + RB) break;
            const float* s0 = rowU(wrapU(sI + G.row - i));
            const float* s1 = rowU(wrapU(sI + G.row + 1 - i));
            const int k0 = G.col - L0;
            const float v = G.w00 * s0[k0] + G.w01 * s0[k0 + 1] + G.w10 * s1[k0] + G.w11 * s1[k0 + 1];
            a.gat_out[(long long)(a.t - 1) * a.gat_ld + G.point] = v;
        }

        // ---- stage 1: l = W * G(u) at rows j .. j+RB-1 ----------------------------------
#pragma unroll
        for (int r = 0; r < RB; r++) uq[QB + r] = rowU(wrapU(sI + r))[tid + R];
        float gy[RB];
        if constexpr (STAG) {
#pragma unroll
            for (int r = 0; r < RB; r++) {
                const float* su = rowU(wrapU(sI - R + r));  // u(j+r, L0 + k)
                float* F = sF + r * NF1;
                {
                    const int k = tid;
                    float v = 0.f;
#pragma unroll
                    for (int m = 0; m < 5; m++) v += kWS(m) * (su[k + 5 + m] - su[k + 4 - m]);
                    v = v * ihy;
                    if constexpr (VARB) v = v * by1[r];
                    F[k] = v;
                }
                if (tid < 9) {
                    const int k = NT + tid;
                    float v = 0.f;
#pragma unroll
                    for (int m = 0; m < 5; m++) v += kWS(m) * (su[k + 5 + m] - su[k + 4 - m]);
                    v = v * ihy;
                    if constexpr (VARB) v = v * by1b[r];
                    F[k] = v;
                }
            }
            __syncthreads();
#pragma unroll
            for (int r = 0; r < RB; r++) {
                const float* F = sF + r * NF1;
                float v = 0.f;
#pragma unroll
                for (int m = 0; m < 5; m++) v += kWS(m) * (F[tid + 5 + m] - F[tid + 4 - m]);
                gy[r] = v * ihy;
            }
        } else {
#pragma unroll
            for (int r = 0; r < RB; r++) {
                const float* su = rowU(wrapU(sI - R + r)) + tid + R;
                float v = kW2(0) * su[0];
#pragma unroll
                for (int k = 1; k <= 5; k++) v += kW2(k) * (su[k] + su[-k]);
                gy[r] = v * ihy2;
            }
        }
        float lj[RB];
#pragma unroll
        for (int r = 0; r < RB; r++) {
            float gx;
            if constexpr (STAG) {
                // flux at half-row (i-5+r)+1/2 from u rows i-9+r .. i+r (queue index r .. r+9)
                float v = 0.f;
#pragma unroll
                for (int m = 0; m < 5; m++) v += kWS(m) * (uq[r + 5 + m] - uq[r + 4 - m]);
                v = v * ihx;
                if constexpr (VARB) v = v * bxi[r];
                fq[QB + r] = v;
                // D- at row j+r from fluxes at half-rows j+r-5 .. j+r+4 (queue index r .. r+9)
                float w = 0.f;
#pragma unroll
                for (int k = 0; k < 5; k++) w += kWS(k) * (fq[r + 5 + k] - fq[r + 4 - k]);
                gx = w * ihx;
            } else {
                // row j+r = i+r-5: u rows i+r-10 .. i+r (queue index r .. r+10)
                float v = kW2(0) * uq[r + 5];
#pragma unroll
                for (int k = 1; k <= 5; k++) v += kW2(k) * (uq[r + 5 + k] + uq[r + 5 - k]);
                gx = v * ihx2;
            }
            lj[r] = (j + r >= 0 && j + r < a.nx && c_in) ? Wj[r] * (gx + gy[r]) : 0.f;
        }
        qshift<QL, RB>(uq);
        if constexpr (STAG) qshift<QL, RB>(fq);

        // ---- stage 2 (OT4): Lt = l + dt^2/12 W G(l) at rows o .. o+RB-1 ------------------
        float Lt[RB];
        if constexpr (OT4) {
            auto wrapL = [](int sl) { return sl < 0 ? sl + QLR : (sl >= QLR ? sl - QLR : sl); };
#pragma unroll
            for (int r = 0; r < RB; r++) {
                sLr[wrapL(sJ + r) * NT + tid] = lj[r];
                lq[QB + r] = lj[r];
            }
            __syncthreads();
            float gy2[RB];
            const bool s2 = (tid >= H1) && (tid < H1 + BY);
            if constexpr (STAG) {
#pragma unroll
                for (int r = 0; r < RB; r++) {
                    const float* sl = sLr + wrapL(sJ - R + r) * NT;  // l(o+r, L1 + k)
                    float* F2 = sF2 + r * NT;
                    if (tid < BY + 9) {
                        const int k = tid;
                        float v = 0.f;
#pragma unroll
                        for (int m = 0; m < 5; m++) v += kWS(m) * (sl[k + 5 + m] - sl[k + 4 - m]);
                        v = v * ihy;
                        if constexpr (VARB) v = v * by2[r];
                        F2[k] = v;
                    }
                }
                __syncthreads();
#pragma unroll
                for (int r = 0; r < RB; r++) {
                    const float* F2 = sF2 + r * NT;
                    float v = 0.f;
                    if (s2) {
                        const int q = tid - H1;
#pragma unroll
                        for (int m = 0; m < 5; m++) v += kWS(m) * (F2[q + 5 + m] - F2[q + 4 - m]);
                    }
                    gy2[r] = v * ihy;
                }
            } else {
#pragma unroll
                for (int r = 0; r < RB; r++) {
                    float v = 0.f;
                    if (s2) {
                        const float* sl = sLr + wrapL(sJ - R + r) * NT + tid;
                        v = kW2(0) * sl[0];
#pragma unroll
                        for (int k = 1; k <= 5; k++) v += kW2(k) * (sl[k] + sl[-k]);
                    }
                    gy2[r] = v * ihy2;
                }
            }
#pragma unroll
            for (int r = 0; r < RB; r++) {
                float gx2;
                if constexpr (STAG) {
                    float v = 0.f;
#pragma unroll
                    for (int m = 0; m < 5; m++) v += kWS(m) * (lq[r + 5 + m] - lq[r + 4 - m]);
                    v = v * ihx;
                    if constexpr (VARB) v = v * bxj[r];
                    f2q[QB + r] = v;
                    float w = 0.f;
#pragma unroll
                    for (int k = 0; k < 5; k++) w += kWS(k) * (f2q[r + 5 + k] - f2q[r + 4 - k]);
                    gx2 = w * ihx;
                } else {
                    float v = kW2(0) * lq[r + 5];
#pragma unroll
                    for (int k = 1; k <= 5; k++) v += kW2(k) * (lq[r + 5 + k] + lq[r + 5 - k]);
                    gx2 = v * ihx2;
                }
                // l(o+r): queue index r (STAG, rows j-9..) or r+5 (laplace, rows j-10..)
                const float lo = STAG ? lq[r] : lq[r + 5];
                Lt[r] = (o + r >= 0 && o + r < a.nx && c_in) ? lo + k12 * (Wo[r] * (gx2 + gy2[r])) : 0.f;
            }
            qshift<QL, RB>(lq);
            if constexpr (STAG) qshift<QL, RB>(f2q);
        } else {
#pragma unroll
            for (int r = 0; r < RB; r++) Lt[r] = lj[r];
        }

        // ---- update of rows o .. o+RB-1, fused epilogues ------------------------------
#pragma unroll
        for (int r = 0; r < RB; r++) {
            const int orow = o + r;
            if (orow >= xo0 && orow < xo1 && out_col) {
                const long long idx = (long long)orow * pitch + c;
                const float u_o = rowU(wrapU(sI - S * R + r))[tid + R];
                const float pm = pmo[r];
                float pn = c1[r] * Lt[r] + c2[r] * u_o - c3[r] * pm;
                // injection into the new level (sources forward, receivers adjoint)
                while (inj_ptr < inj_e && a.inj[inj_ptr].row < orow) inj_ptr++;
                for (int q = inj_ptr; q < inj_e; q++) {
                    const Inject E = a.inj[q];
                    if (E.row != orow) break;
                    if (E.col == c) pn = pn + E.coef * a.inj_amp[(long long)a.t * a.inj_ld + E.point];
                }
                if (do_save) {
                    const long long si = (long long)shot * a.snap_shot_stride + (long long)(a.t / a.f) * a.snap_stride + idx;
                    a.snaps[si] = (pn - 2.f * u_o + pm) / dt2;
                }
                if (do_grad && orow >= a.ix0 && orow < a.ix1 && c >= a.iy0 && c < a.iy1) {
                    const long long si = (long long)shot * a.snap_shot_stride + (long long)(a.t / a.f) * a.snap_stride + idx;
                    const float sv = a.snaps[si];
                    const long long gi = soff + idx;
                    a.gradb[gi] += sv * u_o;
                    a.precb[gi] += sv * sv;
                }
                prev[idx] = pn;
            }
        }
        sI = sI + RB >= QU ? sI + RB - QU : sI + RB;
        if constexpr (OT4) sJ = sJ + RB >= QLR ? sJ + RB - QLR : sJ + RB;
    }
    cp_async_wait<0>();
}

// rec[row][point] = interp(field) for every receiver (the last forward level).
__global__ void gather_final2d(const float* __restrict__ field, long long shot_stride, int pitch,
                               const Gather* __restrict__ g, int n, float* out, int ld, int trow);

// out[p] = sum over shots of buf[shot][x][pitch] for the unpadded extended grid.
__global__ void reduce_shots2d(const float* __restrict__ buf, long long shot_stride, int nshots, int nx,
                               int ny, int pitch, float* __restrict__ out);

}  // namespace sa

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

// ---- packed FP32 helpers (sm_100 family f32x2 instructions) ----------------------------------
__device__ __forceinline__ float2 f2(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, f2(-1.f), a); }

// Staggered first derivative between register-queue entries: sum_m w_m (q[hi+m] - q[lo-m]).
template <int QL>
__device__ __forceinline__ float2 dstag2(const float2 (&q)[QL], int hi, int lo) {
    float2 a = mul2(f2(kWS(0)), q[hi]);
    float2 b = mul2(f2(kWS(0)), q[lo]);
#pragma unroll
    for (int m = 1; m < 5; m++) {
        a = fma2(f2(kWS(m)), q[hi + m], a);
        b = fma2(f2(kWS(m)), q[lo - m], b);
    }
    return sub2(a, b);
}
// Centred second derivative sum_k w_k (q[c+k] + q[c-k]) + w_0 q[c].
template <int QL>
__device__ __forceinline__ float2 dcent2(const float2 (&q)[QL], int cidx) {
    float2 a = mul2(f2(kW2(0)), q[cidx]);
#pragma unroll
    for (int k = 1; k <= 5; k++) a = fma2(f2(kW2(k)), add2(q[cidx + k], q[cidx - k]), a);
    return a;
}
// Scalar versions over a local array (y derivatives from shared memory).
__device__ __forceinline__ float dstag1(const float* v, int hi, int lo) {
    float a = kWS(0) * v[hi], b = kWS(0) * v[lo];
#pragma unroll
    for (int m = 1; m < 5; m++) {
        a = fmaf(kWS(m), v[hi + m], a);
        b = fmaf(kWS(m), v[lo - m], b);
    }
    return a - b;
}
__device__ __forceinline__ float dcent1(const float* v, int cidx) {
    float a = kW2(0) * v[cidx];
#pragma unroll
    for (int k = 1; k <= 5; k++) a = fmaf(kW2(k), v[cidx + k] + v[cidx - k], a);
    return a;
}
// n consecutive floats from shared memory as float2 loads (8-byte aligned source).
template <int N>
__device__ __forceinline__ void lds_pairs(float (&v)[N], const float* src) {
#pragma unroll
    for (int k = 0; k < N / 2; k++) {
        const float2 p = *reinterpret_cast<const float2*>(src + 2 * k);
        v[2 * k] = p.x;
        v[2 * k + 1] = p.y;
    }
}
__device__ __forceinline__ float2 ldg2(const float* p) { return __ldg(reinterpret_cast<const float2*>(p)); }

// Column layout of one CTA. Each thread owns the column pair (c0, c0+1), c0 = Lc + 2t even.
template <int KIND, bool OT4, int NT>
struct Cols2D {
    static constexpr bool STAG = KIND != 0;
    static constexpr int R = STAG ? 9 : 5;            // radius of one operator application
    static constexpr int S = OT4 ? 2 : 1;             // pipeline stages
    static constexpr int H1 = (S - 1) * R;            // halo of the stage-1 output columns
    static constexpr int HL = H1 + (H1 & 1);          // left halo rounded to even: Lc = y0 - HL
    static constexpr int NC = 2 * NT;                 // stage-1 columns of the CTA
    static constexpr int BYMAX = (NC - HL - H1) & ~1; // output columns (even)
};

// Shared-memory layout of one CTA (floats).
template <int KIND, bool OT4, int NT, int RB, int PF>
struct Smem2D {
    using C = Cols2D<KIND, OT4, NT>;
    static constexpr bool STAG = C::STAG;
    static constexpr int R = C::R, S = C::S, NC = C::NC;
    static constexpr int WU = round4(NC + 2 * R + 3) + 8;  // u row from floor4(Lc - R), slack for pair reads
    static constexpr int QU = S * R + RB * (PF + 1);        // u rows kept: o .. i + RB*(PF+1) - 1
    static constexpr int QLR = R + RB;                      // rows of the intermediate kept (OT4)
    static constexpr int WL = NC + 8;
    static constexpr int WF = NC + 12;
    static constexpr int oU = 0;
    static constexpr int oL = oU + QU * WU;
    static constexpr int oF = oL + (OT4 ? QLR * WL : 0);
    static constexpr int oF2 = oF + (STAG ? RB * WF : 0);
    static constexpr int total = oF2 + ((OT4 && STAG) ? RB * WF : 0);
    static constexpr size_t bytes = (size_t)total * sizeof(float);
};

// Register queue shift by RB (the oldest RB entries leave).
template <int QL, int RB>
__device__ __forceinline__ void qshift(float2 (&q)[QL]) {
#pragma unroll
    for (int k = 0; k + RB < QL; k++) q[k] = q[k + RB];
}

template <int KIND, bool OT4, int NT, int RB, int PF>
__global__ void __launch_bounds__(NT) fdtd2d_step(const __grid_constant__ Step2D a) {
    using L = Smem2D<KIND, OT4, NT, RB, PF>;
    using CL = Cols2D<KIND, OT4, NT>;
    constexpr bool STAG = CL::STAG;           // staggered div(b grad) operator
    constexpr bool VARB = KIND == 1;          // variable buoyancy
    constexpr int R = CL::R, S = CL::S, H1 = CL::H1, HL = CL::HL, NC = CL::NC;
    constexpr int QU = L::QU, QLR = L::QLR;
    // register queues along x (float2 = the thread's column pair):
    // u rows i-QB..i+RB-1; fluxes at half-rows i-QB-5..i-6+RB (STAG)
    constexpr int QB = STAG ? 9 : 10;
    constexpr int QL = QB + RB;
    (void)H1;
    (void)NC;

    extern __shared__ __align__(16) float smem[];
    float* const sU = smem + L::oU;
    float* const sLr = smem + L::oL;
    float* const sF = smem + L::oF;
    float* const sF2 = smem + L::oF2;

    const int tid = threadIdx.x;
    const int strip = blockIdx.x, chunk = blockIdx.y, shot = blockIdx.z;
    const int BY = a.by;                      // even, <= BYMAX
    const int y0 = strip * BY;                // even
    const int Lc = y0 - HL;                   // first stage-1 column (even)
    const int QU0 = (Lc - R) & ~3;            // u rows start at floor4(Lc - R)
    const int c0 = Lc + 2 * tid;              // this thread's column pair (c0, c0+1)
    const bool in0 = c0 >= 0 && c0 < a.ny, in1 = c0 + 1 >= 0 && c0 + 1 < a.ny;
    const bool outp = (c0 >= y0) && (c0 < y0 + BY) && in0;  // output pair (c0+1 checked by in1)
    const int cg = min(max(c0, 0), a.pitch - 2);            // clamped pair column for medium rows
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

    // medium pointers at row 0 of this thread's pair (GUARD zero rows make rows beyond the
    // grid addressable; their values only reach discarded lanes)
    const float* __restrict__ pW = a.W + cg;
    const float* __restrict__ pBX = a.bxh + cg;
    // byh storage column of half-col h is h + 6; flux pairs start at even half-cols
    const int kb1 = min(max(Lc + 2 * tid, 0), pitch_b - 2);        // stage-1 flux pair f = 2t
    const int kb1b = min(max(Lc + 2 * (NT + tid), 0), pitch_b - 2); // extra pair f = 2(NT+t), t < 5
    const int kb2 = min(max(y0 + 2 * tid, 0), pitch_b - 2);        // stage-2 flux pair
    const float* __restrict__ pC1 = a.C1 + cg;
    const float* __restrict__ pC2 = a.C2 + cg;
    const float* __restrict__ pC3 = a.C3 + cg;

    // u ring: row r in slot (r - i0) mod QU
    constexpr int NQU = L::WU / 4;
    auto wrapU = [](int sl) { return sl < 0 ? sl + QU : (sl >= QU ? sl - QU : sl); };
    auto rowU = [&](int sl) { return sU + sl * L::WU - QU0; };  // rowU(s)[col] = u(row, col)
    int sI = 0;  // slot of row i
    auto prefetch = [&](int ii, int slot) {
#pragma unroll
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

    float2 uq[QL], fq[STAG ? QL : 1], lq[OT4 ? QL : 1], f2q[(OT4 && STAG) ? QL : 1];
#pragma unroll
    for (int k = 0; k < QL; k++) {
        uq[k] = f2(0.f);
        if constexpr (STAG) fq[k] = f2(0.f);
        if constexpr (OT4) {
            lq[k] = f2(0.f);
            if constexpr (STAG) f2q[k] = f2(0.f);
        }
    }
    int inj_ptr = inj_b, gat_ptr = gat_b;
    const bool do_save = a.save && (a.t % a.f == 0);
    const bool do_grad = a.grad && (a.t % a.f == 0);

#pragma unroll 1
    for (int k = 0; k < PF; k++) prefetch(i0 + k * RB, wrapU(k * RB % QU));

    int sJ = 0;  // ring slot of intermediate row j (slot of row x is (x - (i0 - R)) mod QLR)
#pragma unroll 1
    for (int i = i0; i < i1; i += RB) {
        const int j = i - R;        // first stage-1 output row of this iteration
        const int o = i - S * R;    // first output row of this iteration
        // ---- stage-1 medium of this iteration, loaded before the barrier --------------
        float2 Wj[RB], bxi[RB], by1[RB], by1b[RB];
#pragma unroll
        for (int r = 0; r < RB; r++) {
            Wj[r] = ldg2(pW + (long long)(j + r) * pitch);
            if constexpr (VARB) {
                bxi[r] = ldg2(pBX + (long long)(i - 5 + r) * pitch);
                const float* byr = a.byh + (long long)(j + r) * pitch_b;
                by1[r] = ldg2(byr + kb1);
                by1b[r] = tid < 5 ? ldg2(byr + kb1b) : f2(0.f);
            }
        }

        cp_async_wait<PF - 1>();
        __syncthreads();  // rows i..i+RB-1 visible; every thread is done with the last iteration
        prefetch(i + PF * RB, sI + PF * RB >= QU ? sI + PF * RB - QU : sI + PF * RB);

        // ---- receiver interpolation of p[t] -> rec[t-1]: base rows i-1 .. i+RB-2 ----------
        while (gat_ptr < gat_e && a.gat[gat_ptr].row + 1 < i) gat_ptr++;
        for (int e = gat_ptr + tid; e < gat_e; e += NT) {
            const Gather G = a.gat[e];
            if (G.row + 1 >= i + RB) break;
            const float* s0 = rowU(wrapU(sI + G.row - i));
            const float* s1 = rowU(wrapU(sI + G.row + 1 - i));
            const float v = G.w00 * s0[G.col] + G.w01 * s0[G.col + 1] + G.w10 * s1[G.col] + G.w11 * s1[G.col + 1];
            a.gat_out[(long long)(a.t - 1) * a.gat_ld + G.point] = v;
        }

        // stage-2 and update medium of this iteration (used after the next barrier)
        float2 Wo[RB], bxj[RB], by2[RB], c1[RB], c2[RB], c3[RB], pmo[RB];
#pragma unroll
        for (int r = 0; r < RB; r++) {
            if constexpr (OT4) {
                Wo[r] = ldg2(pW + (long long)(o + r) * pitch);
                if constexpr (VARB) {
                    bxj[r] = ldg2(pBX + (long long)(j - 5 + r) * pitch);
                    by2[r] = ldg2(a.byh + (long long)(o + r) * pitch_b + kb2);
                }
            }
            const bool o_ok = (o + r >= xo0) && (o + r < xo1) && outp;
            const long long orow = (long long)(o + r) * pitch;
            c1[r] = o_ok ? ldg2(pC1 + orow) : f2(0.f);
            c2[r] = o_ok ? ldg2(pC2 + orow) : f2(0.f);
            c3[r] = o_ok ? ldg2(pC3 + orow) : f2(0.f);
            pmo[r] = o_ok ? *reinterpret_cast<const float2*>(prev + orow + c0) : f2(0.f);
        }
        (void)Wo; (void)bxj; (void)by2; (void)bxi; (void)by1; (void)by1b;

        // ---- stage 1: l = W * G(u) at rows j .. j+RB-1 ----------------------------------
#pragma unroll
        for (int r = 0; r < RB; r++) uq[QB + r] = *reinterpret_cast<const float2*>(rowU(wrapU(sI + r)) + c0);
        float gy[RB][2];
        if constexpr (STAG) {
#pragma unroll
            for (int r = 0; r < RB; r++) {
                const float* su = rowU(wrapU(sI - R + r));  // u(j+r, col)
                float* F = sF + r * L::WF;                  // F[f] = flux at half-col Lc-6+f
#pragma unroll
                for (int pass = 0; pass < 2; pass++) {
                    if (pass == 1 && tid >= 5) break;
                    const int f = 2 * (pass == 0 ? tid : NT + tid);
                    const int jh = Lc - 6 + f;  // even half-col
                    float uv[12];
                    lds_pairs<12>(uv, su + jh - 4);
                    float2 fl = make_float2(dstag1(uv, 5, 4), dstag1(uv, 6, 5));
                    fl = mul2(fl, f2(ihy));
                    if constexpr (VARB) fl = mul2(fl, pass == 0 ? by1[r] : by1b[r]);
                    *reinterpret_cast<float2*>(F + f) = fl;
                }
            }
            __syncthreads();
#pragma unroll
            for (int r = 0; r < RB; r++) {
                float fv[12];
                lds_pairs<12>(fv, sF + r * L::WF + 2 * tid);
                gy[r][0] = dstag1(fv, 6, 5) * ihy;
                gy[r][1] = dstag1(fv, 7, 6) * ihy;
            }
        } else {
#pragma unroll
            for (int r = 0; r < RB; r++) {
                float uv[14];
                lds_pairs<14>(uv, rowU(wrapU(sI - R + r)) + c0 - 6);
                gy[r][0] = dcent1(uv, 6) * ihy2;
                gy[r][1] = dcent1(uv, 7) * ihy2;
            }
        }
        float2 lj[RB];
#pragma unroll
        for (int r = 0; r < RB; r++) {
            float2 gx;
            if constexpr (STAG) {
                // flux at half-row (i-5+r)+1/2 from u rows i-9+r .. i+r (queue index r .. r+9)
                float2 v = mul2(dstag2<QL>(uq, r + 5, r + 4), f2(ihx));
                if constexpr (VARB) v = mul2(v, bxi[r]);
                fq[QB + r] = v;
                // D- at row j+r from fluxes at half-rows j+r-5 .. j+r+4 (queue index r .. r+9)
                gx = mul2(dstag2<QL>(fq, r + 5, r + 4), f2(ihx));
            } else {
                gx = mul2(dcent2<QL>(uq, r + 5), f2(ihx2));  // rows i+r-10 .. i+r
            }
            const bool row_in = j + r >= 0 && j + r < a.nx;
            float2 v = mul2(Wj[r], add2(gx, make_float2(gy[r][0], gy[r][1])));
            lj[r] = make_float2(row_in && in0 ? v.x : 0.f, row_in && in1 ? v.y : 0.f);  // zero halo
        }
        qshift<QL, RB>(uq);
        if constexpr (STAG) qshift<QL, RB>(fq);

        // ---- stage 2 (OT4): Lt = l + dt^2/12 W G(l) at rows o .. o+RB-1 ------------------
        float2 Lt[RB];
        if constexpr (OT4) {
            auto wrapL = [](int sl) { return sl < 0 ? sl + QLR : (sl >= QLR ? sl - QLR : sl); };
#pragma unroll
            for (int r = 0; r < RB; r++) {
                *reinterpret_cast<float2*>(sLr + wrapL(sJ + r) * L::WL + 2 * tid) = lj[r];  // l(j+r, Lc+k)
                lq[QB + r] = lj[r];
            }
            __syncthreads();
            float gy2[RB][2];
            if constexpr (STAG) {
#pragma unroll
                for (int r = 0; r < RB; r++) {
                    const float* sl = sLr + wrapL(sJ - R + r) * L::WL;  // l(o+r, Lc + k)
                    if (2 * tid < BY + 10) {
                        const int f = 2 * tid;  // flux at half-col y0-6+f: l index f .. f+11
                        float lv[12];
                        lds_pairs<12>(lv, sl + f);
                        float2 fl = make_float2(dstag1(lv, 5, 4), dstag1(lv, 6, 5));
                        fl = mul2(fl, f2(ihy));
                        if constexpr (VARB) fl = mul2(fl, by2[r]);
                        *reinterpret_cast<float2*>(sF2 + r * L::WF + f) = fl;
                    }
                }
                __syncthreads();
#pragma unroll
                for (int r = 0; r < RB; r++) {
                    gy2[r][0] = gy2[r][1] = 0.f;
                    if (outp) {
                        float fv[12];
                        lds_pairs<12>(fv, sF2 + r * L::WF + (c0 - y0));
                        gy2[r][0] = dstag1(fv, 6, 5) * ihy;
                        gy2[r][1] = dstag1(fv, 7, 6) * ihy;
                    }
                }
            } else {
#pragma unroll
                for (int r = 0; r < RB; r++) {
                    gy2[r][0] = gy2[r][1] = 0.f;
                    if (outp) {
                        float lv[14];
                        lds_pairs<14>(lv, sLr + wrapL(sJ - R + r) * L::WL + 2 * tid - 6);
                        gy2[r][0] = dcent1(lv, 6) * ihy2;
                        gy2[r][1] = dcent1(lv, 7) * ihy2;
                    }
                }
            }
#pragma unroll
            for (int r = 0; r < RB; r++) {
                float2 gx2;
                if constexpr (STAG) {
                    float2 v = mul2(dstag2<QL>(lq, r + 5, r + 4), f2(ihx));
                    if constexpr (VARB) v = mul2(v, bxj[r]);
                    f2q[QB + r] = v;
                    gx2 = mul2(dstag2<QL>(f2q, r + 5, r + 4), f2(ihx));
                } else {
                    gx2 = mul2(dcent2<QL>(lq, r + 5), f2(ihx2));
                }
                // l(o+r): queue index r (STAG, rows j-9..) or r+5 (laplace, rows j-10..)
                const float2 lo = STAG ? lq[r] : lq[r + 5];
                Lt[r] = fma2(f2(k12), mul2(Wo[r], add2(gx2, make_float2(gy2[r][0], gy2[r][1]))), lo);
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
            if (orow >= xo0 && orow < xo1 && outp) {
                const long long idx = (long long)orow * pitch + c0;
                const float2 u_o = *reinterpret_cast<const float2*>(rowU(wrapU(sI - S * R + r)) + c0);
                const float2 pm = pmo[r];
                float2 pn = fma2(c1[r], Lt[r], fma2(c2[r], u_o, mul2(c3[r], make_float2(-pm.x, -pm.y))));
                // injection into the new level (sources forward, receivers adjoint)
                while (inj_ptr < inj_e && a.inj[inj_ptr].row < orow) inj_ptr++;
                for (int q = inj_ptr; q < inj_e; q++) {
                    const Inject E = a.inj[q];
                    if (E.row != orow) break;
                    const float amp = E.coef * a.inj_amp[(long long)a.t * a.inj_ld + E.point];
                    if (E.col == c0) pn.x = pn.x + amp;
                    if (E.col == c0 + 1) pn.y = pn.y + amp;
                }
                const long long sbase = (long long)shot * a.snap_shot_stride + (long long)(a.t / a.f) * a.snap_stride + idx;
                if (do_save) {
                    const float2 sv = make_float2((pn.x - 2.f * u_o.x + pm.x) / dt2, (pn.y - 2.f * u_o.y + pm.y) / dt2);
                    if (in1) *reinterpret_cast<float2*>(a.snaps + sbase) = sv;
                    else a.snaps[sbase] = sv.x;
                }
                if (do_grad && orow >= a.ix0 && orow < a.ix1) {
                    const long long gi = soff + idx;
                    if (c0 >= a.iy0 && c0 < a.iy1) {
                        const float sv = a.snaps[sbase];
                        a.gradb[gi] += sv * u_o.x;
                        a.precb[gi] += sv * sv;
                    }
                    if (c0 + 1 >= a.iy0 && c0 + 1 < a.iy1) {
                        const float sv = a.snaps[sbase + 1];
                        a.gradb[gi + 1] += sv * u_o.y;
                        a.precb[gi + 1] += sv * sv;
                    }
                }
                if (in1) *reinterpret_cast<float2*>(prev + idx) = pn;
                else prev[idx] = pn.x;
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

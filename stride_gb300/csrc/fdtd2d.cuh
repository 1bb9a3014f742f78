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
//  * the undersampled save of p.dt2 or of p itself (:398-418) is a fused epilogue; source injection (:357-363),
//    receiver interpolation (:364), the adjoint receiver injection (:748-753) and the vp imaging
//    condition (:1000-1024) run as their own kernels after the step (helpers.cu), which kept
//    their irregular loads out of the stencil's loop.
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

// ---- arithmetic on the two lanes of a shot pair ---------------------------------------------
// SA_PACKED=1 issues the sm_100-family f32x2 instructions (one instruction for both shots;
// 4 % faster on the 64-shot gradient); 0 issues two scalar FP32 instructions, which take
// immediate operands (the FD weights) without register pairs. Both round identically.
#ifndef SA_PACKED
#define SA_PACKED 1
#endif
__device__ __forceinline__ float2 f2(float v) { return make_float2(v, v); }
#if SA_PACKED
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, f2(-1.f), a); }
#else
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
    return make_float2(fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y));
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return make_float2(a.x * b.x, a.y * b.y); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
#endif

// Staggered first derivative sum_m w_m (v[hi+m] - v[lo-m]) over float2 values (queue or shared).
template <class A>
__device__ __forceinline__ float2 dstag2(const A& v, int hi, int lo) {
    float2 a = mul2(f2(kWS(0)), v[hi]);
    float2 b = mul2(f2(kWS(0)), v[lo]);
#pragma unroll
    for (int m = 1; m < 5; m++) {
        a = fma2(f2(kWS(m)), v[hi + m], a);
        b = fma2(f2(kWS(m)), v[lo - m], b);
    }
    return sub2(a, b);
}
// Centred second derivative sum_k w_k (v[c+k] + v[c-k]) + w_0 v[c].
template <class A>
__device__ __forceinline__ float2 dcent2(const A& v, int cidx) {
    float2 a = mul2(f2(kW2(0)), v[cidx]);
#pragma unroll
    for (int k = 1; k <= 5; k++) a = fma2(f2(kW2(k)), add2(v[cidx + k], v[cidx - k]), a);
    return a;
}

// Column layout of one CTA: thread t owns column c = L1 + t; every value is a float2 holding
// the same grid point of the two shots of a shot pair.
template <int KIND, bool OT4, int NT>
struct Cols2D {
    static constexpr bool STAG = KIND != 0;
    static constexpr int R = STAG ? 9 : 5;            // radius of one operator application
    static constexpr int S = OT4 ? 2 : 1;             // pipeline stages
    static constexpr int H1 = (S - 1) * R;            // halo of the stage-1 output columns
    static constexpr int BYMAX = NT - 2 * H1;         // output columns
};

// Shared-memory layout of one CTA, in float2 units.
template <int KIND, bool OT4, int NT, int RB, int PF>
struct Smem2D {
    using C = Cols2D<KIND, OT4, NT>;
    static constexpr bool STAG = C::STAG;
    static constexpr int R = C::R, S = C::S;
    static constexpr int C0 = NT + 2 * R;                 // u columns [L0, L0 + C0)
    static constexpr int WU = ((C0 + 1 + 1) & ~1) + 2;    // u row from floor2(L0), even
    static constexpr int QU = S * R + RB * (PF + 1);      // u rows kept: o .. i + RB*(PF+1) - 1
    static constexpr int QLR = R + RB;                    // rows of the intermediate kept (OT4)
    static constexpr int WL = NT + 2;
    static constexpr int WF = NT + 10;
    static constexpr int oU = 0;
    static constexpr int oL = oU + QU * WU;
    // y-flux rows of both stages, double-buffered by iteration parity (written before the
    // iteration's barrier, read after it)
    static constexpr int oF = oL + (OT4 ? QLR * WL : 0);
    static constexpr int oF2 = oF + (STAG ? 2 * RB * WF : 0);
    static constexpr int total = oF2 + ((OT4 && STAG) ? 2 * RB * WF : 0);
    static constexpr size_t bytes = (size_t)total * sizeof(float2);
};

// Register queue shift by RB (the oldest RB entries leave).
template <int QL, int RB>
__device__ __forceinline__ void qshift(float2 (&q)[QL]) {
#pragma unroll
    for (int k = 0; k + RB < QL; k++) q[k] = q[k + RB];
}

#ifndef SA_MINBLOCKS
#define SA_MINBLOCKS 3  // CTAs per SM the register allocation must allow (latency hiding)
#endif
// CTAs per SM the register budget is sized for: SA_MINBLOCKS up to 192 threads (the OT2 kernels
// fit three CTAs of 192), two for the 256-thread CTA (whose three would leave 85 registers)
__host__ __device__ constexpr int step_min_blocks(int nt) { return nt <= 192 ? SA_MINBLOCKS : 2; }

template <int KIND, bool OT4, int NT, int RB, int PF>
__global__ void __launch_bounds__(NT, step_min_blocks(NT)) fdtd2d_step(const __grid_constant__ Step2D a) {
    using L = Smem2D<KIND, OT4, NT, RB, PF>;
    using CL = Cols2D<KIND, OT4, NT>;
    constexpr bool STAG = CL::STAG;           // staggered div(b grad) operator
    constexpr bool VARB = KIND == 1;          // variable buoyancy
    constexpr int R = CL::R, S = CL::S, H1 = CL::H1;
    constexpr int QU = L::QU, QLR = L::QLR;
    // register queues along x: u rows i-QB..i+RB-1; fluxes at half-rows i-QB-5..i-6+RB (STAG)
    constexpr int QB = STAG ? 9 : 10;
    constexpr int QL = QB + RB;

    extern __shared__ __align__(16) float2 smem2[];
    float2* const sU = smem2 + L::oU;
    float2* const sLr = smem2 + L::oL;
    float2* const sF = smem2 + L::oF;
    float2* const sF2 = smem2 + L::oF2;

    const int tid = threadIdx.x;
    const int strip = blockIdx.x, chunk = blockIdx.y, pair = blockIdx.z;
    const int BY = a.by;
    const int y0 = strip * BY;
    const int L1 = y0 - H1;                   // first stage-1 output column
    const int L0 = L1 - R;                    // first stage-1 input column
    const int QU0 = L0 & ~1;                  // u rows start at an even column (16-byte copies)
    const int c = L1 + tid;                   // this thread's column
    const bool c_in = (c >= 0) && (c < a.ny);
    const bool out_col = (tid >= H1) && (tid < H1 + BY) && c_in;
    const int cc = min(max(c, 0), a.ny - 1);
    const int xo0 = chunk * a.chunk_rows;
    const int xo1 = min(a.nx, xo0 + a.chunk_rows);
    const int i0 = xo0 - S * R, i1 = xo1 + S * R;
    const int pitch = a.pitch, pitch_b = a.pitch_b;

    const long long poff = (long long)pair * a.shot_stride;  // float2 elements per pair: nx*pitch
    const float2* __restrict__ cur = reinterpret_cast<const float2*>(a.cur);
    float2* __restrict__ prev = reinterpret_cast<float2*>(a.prev) + poff;


    const float2 ihx = f2(1.f / a.hx), ihy = f2(1.f / a.hy);
    const float2 ihx2 = f2(1.f / (a.hx * a.hx)), ihy2 = f2(1.f / (a.hy * a.hy));
    const float dt2 = a.dt * a.dt;
    const float2 k12 = f2((float)((double)a.dt * (double)a.dt / 12.0));

    // per-thread medium pointers at row 0 of this thread's column (GUARD zero rows make rows
    // beyond the grid addressable; their values only reach discarded lanes)
    const float* __restrict__ pW = a.W + cc;
    const float* __restrict__ pBX = a.bxh + cc;
    // byh storage column of half-col h is h + 6
    const int kb1 = min(max(L1 + 1 + tid, 0), pitch_b - 1);        // stage-1 flux k = tid
    const int kb1b = min(max(L1 + 1 + NT + tid, 0), pitch_b - 1);  // stage-1 flux k = NT + tid
    const int kb2 = min(max(y0 + 1 + tid, 0), pitch_b - 1);        // stage-2 flux k = tid
    const float* __restrict__ pC1 = a.C1 + cc;
    const float* __restrict__ pC2 = a.C2 + cc;
    const float* __restrict__ pC3 = a.C3 + cc;

    // u ring: row r in slot (r - i0) mod QU
    constexpr int NQU = L::WU / 2;  // 16-byte copies (2 columns x 2 shots)
    auto wrapU = [](int sl) { return sl < 0 ? sl + QU : (sl >= QU ? sl - QU : sl); };
    auto rowU = [&](int sl) { return sU + sl * L::WU - QU0; };  // rowU(s)[col] = u(row, col)
    int sI = 0;  // slot of row i
    auto prefetch = [&](int ii, int slot) {
#pragma unroll
        for (int rr = 0; rr < RB; rr++) {
            const int r = ii + rr;
            if (r < i1) {
                float2* dst = sU + wrapU(slot + rr) * L::WU;
                const bool row_ok = r >= 0 && r < a.nx;
                const float2* rowp = cur + poff + (long long)r * pitch;
                for (int k = tid; k < NQU; k += NT) {
                    const int q = QU0 + 2 * k;
                    const bool ok = row_ok && q >= 0 && q + 2 <= pitch;
                    cp_async16(dst + 2 * k, ok ? rowp + q : cur, ok);
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
    const bool do_save = a.save && (a.t % a.f == 0);

#pragma unroll 1
    for (int k = 0; k < PF; k++) prefetch(i0 + k * RB, wrapU(k * RB % QU));

    int sJ = 0;  // ring slot of intermediate row j (slot of row x is (x - (i0 - R)) mod QLR)
    auto wrapL = [](int sl) { return sl < 0 ? sl + QLR : (sl >= QLR ? sl - QLR : sl); };
    int par = 0;  // flux buffer of this iteration
    // One barrier per iteration. Before it, the y-fluxes of both stages are computed from rows
    // that became visible in earlier iterations (u rows j.., intermediate rows o..) into this
    // iteration's flux buffers; after it, the rows that just landed (cp.async) and the fluxes
    // are read. Ring slots written after the barrier (new intermediate rows, prefetched u rows)
    // hold rows no thread reads before the next barrier.
#pragma unroll 1
    for (int i = i0; i < i1; i += RB) {
        const int j = i - R;        // first stage-1 output row of this iteration
        const int o = i - S * R;    // first output row of this iteration
        // ---- stage-1 medium, stage-2 y medium -----------------------------------------
        float Wj[RB], bxi[RB], by1[RB], by1b[RB], by2[RB];
#pragma unroll
        for (int r = 0; r < RB; r++) {
            Wj[r] = __ldg(pW + (long long)(j + r) * pitch);
            if constexpr (VARB) {
                bxi[r] = __ldg(pBX + (long long)(i - 5 + r) * pitch);
                const float* byr = a.byh + (long long)(j + r) * pitch_b;
                by1[r] = __ldg(byr + kb1);
                by1b[r] = tid < 9 ? __ldg(byr + kb1b) : 0.f;
                if constexpr (OT4) by2[r] = __ldg(a.byh + (long long)(o + r) * pitch_b + kb2);
            }
        }
        (void)bxi; (void)by1; (void)by1b; (void)by2;
        float2* const F = sF + par * RB * L::WF;
        float2* const F2 = sF2 + par * RB * L::WF;
        if constexpr (STAG) {
            // stage-1 y-fluxes at half-cols L1-5+k from u rows j+r (F[k])
#pragma unroll
            for (int r = 0; r < RB; r++) {
                const float2* su = rowU(wrapU(sI - R + r)) + L0;  // su[k] = u(j+r, L0 + k)
                {
                    const int k = tid;
                    float2 v = mul2(dstag2(su, k + 5, k + 4), ihy);
                    if constexpr (VARB) v = mul2(v, f2(by1[r]));
                    F[r * L::WF + k] = v;
                }
                if (tid < 9) {
                    const int k = NT + tid;
                    float2 v = mul2(dstag2(su, k + 5, k + 4), ihy);
                    if constexpr (VARB) v = mul2(v, f2(by1b[r]));
                    F[r * L::WF + k] = v;
                }
            }
            if constexpr (OT4) {
                // stage-2 y-fluxes at half-cols y0-5+k from intermediate rows o+r (F2[k])
#pragma unroll
                for (int r = 0; r < RB; r++) {
                    const float2* sl = sLr + wrapL(sJ - R + r) * L::WL;  // l(o+r, L1 + k)
                    if (tid < BY + 9) {
                        const int k = tid;
                        float2 v = mul2(dstag2(sl, k + 5, k + 4), ihy);
                        if constexpr (VARB) v = mul2(v, f2(by2[r]));
                        F2[r * L::WF + k] = v;
                    }
                }
            }
        }

        cp_async_wait<PF - 1>();
        __syncthreads();  // rows i..i+RB-1 and this iteration's fluxes visible; last iteration done
        prefetch(i + PF * RB, sI + PF * RB >= QU ? sI + PF * RB - QU : sI + PF * RB);

        // stage-2 and update medium of this iteration
        float Wo[RB], bxj[RB], c1[RB], c2[RB], c3[RB];
        float2 pmo[RB];
#pragma unroll
        for (int r = 0; r < RB; r++) {
            if constexpr (OT4) {
                Wo[r] = __ldg(pW + (long long)(o + r) * pitch);
                if constexpr (VARB) bxj[r] = __ldg(pBX + (long long)(j - 5 + r) * pitch);
            }
            const bool o_ok = (o + r >= xo0) && (o + r < xo1) && out_col;
            const long long orow = (long long)(o + r) * pitch;
            c1[r] = o_ok ? __ldg(pC1 + orow) : 0.f;
            c2[r] = o_ok ? __ldg(pC2 + orow) : 0.f;
            c3[r] = o_ok ? __ldg(pC3 + orow) : 0.f;
            pmo[r] = o_ok ? prev[orow + c] : f2(0.f);
        }
        (void)Wo; (void)bxj;

        // ---- stage 1: l = W * G(u) at rows j .. j+RB-1 ----------------------------------
#pragma unroll
        for (int r = 0; r < RB; r++) uq[QB + r] = rowU(wrapU(sI + r))[c];
        float2 gy[RB];
        if constexpr (STAG) {
#pragma unroll
            for (int r = 0; r < RB; r++) gy[r] = mul2(dstag2(F + r * L::WF, tid + 5, tid + 4), ihy);
        } else {
#pragma unroll
            for (int r = 0; r < RB; r++) gy[r] = mul2(dcent2(rowU(wrapU(sI - R + r)), c), ihy2);
        }
        float2 lj[RB];
#pragma unroll
        for (int r = 0; r < RB; r++) {
            float2 gx;
            if constexpr (STAG) {
                // flux at half-row (i-5+r)+1/2 from u rows i-9+r .. i+r (queue index r .. r+9)
                float2 v = mul2(dstag2(uq, r + 5, r + 4), ihx);
                if constexpr (VARB) v = mul2(v, f2(bxi[r]));
                fq[QB + r] = v;
                // D- at row j+r from fluxes at half-rows j+r-5 .. j+r+4 (queue index r .. r+9)
                gx = mul2(dstag2(fq, r + 5, r + 4), ihx);
            } else {
                gx = mul2(dcent2(uq, r + 5), ihx2);  // rows i+r-10 .. i+r
            }
            const bool keep = j + r >= 0 && j + r < a.nx && c_in;  // zero halo of the intermediate
            lj[r] = keep ? mul2(f2(Wj[r]), add2(gx, gy[r])) : f2(0.f);
        }
        qshift<QL, RB>(uq);
        if constexpr (STAG) qshift<QL, RB>(fq);

        // ---- stage 2 (OT4): Lt = l + dt^2/12 W G(l) at rows o .. o+RB-1 ------------------
        float2 Lt[RB];
        if constexpr (OT4) {
#pragma unroll
            for (int r = 0; r < RB; r++) {
                sLr[wrapL(sJ + r) * L::WL + tid] = lj[r];  // l(j+r, L1 + k), read R rows later
                lq[QB + r] = lj[r];
            }
            float2 gy2[RB];
            const bool s2 = (tid >= H1) && (tid < H1 + BY);
            if constexpr (STAG) {
#pragma unroll
                for (int r = 0; r < RB; r++)
                    gy2[r] = s2 ? mul2(dstag2(F2 + r * L::WF, tid - H1 + 5, tid - H1 + 4), ihy) : f2(0.f);
            } else {
#pragma unroll
                for (int r = 0; r < RB; r++)
                    gy2[r] = s2 ? mul2(dcent2(sLr + wrapL(sJ - R + r) * L::WL, tid), ihy2) : f2(0.f);
            }
#pragma unroll
            for (int r = 0; r < RB; r++) {
                float2 gx2;
                if constexpr (STAG) {
                    float2 v = mul2(dstag2(lq, r + 5, r + 4), ihx);
                    if constexpr (VARB) v = mul2(v, f2(bxj[r]));
                    f2q[QB + r] = v;
                    gx2 = mul2(dstag2(f2q, r + 5, r + 4), ihx);
                } else {
                    gx2 = mul2(dcent2(lq, r + 5), ihx2);
                }
                // l(o+r): queue index r (STAG, rows j-9..) or r+5 (laplace, rows j-10..)
                const float2 lo = STAG ? lq[r] : lq[r + 5];
                Lt[r] = fma2(k12, mul2(f2(Wo[r]), add2(gx2, gy2[r])), lo);
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
                const long long idx = (long long)orow * pitch + c;  // float2 index within the pair
                const float2 u_o = rowU(wrapU(sI - S * R + r))[c];
                const float2 pm = pmo[r];
                float2 pn = fma2(f2(c1[r]), Lt[r], fma2(f2(c2[r]), u_o, mul2(f2(-c3[r]), pm)));
                if (do_save) {
                    float2* snap = reinterpret_cast<float2*>(a.snaps) + (long long)pair * a.snap_shot_stride +
                                   (long long)(a.t / a.f) * a.snap_stride + idx;
                    *snap = a.save == 2 ? u_o  // raw p[t] (rho / wavelet gradients)
                                        : make_float2((pn.x - 2.f * u_o.x + pm.x) / dt2, (pn.y - 2.f * u_o.y + pm.y) / dt2);
                }
                prev[idx] = pn;
            }
        }
        sI = sI + RB >= QU ? sI + RB - QU : sI + RB;
        if constexpr (OT4) sJ = sJ + RB >= QLR ? sJ + RB - QLR : sJ + RB;
        par ^= 1;
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

// 2D iso-acoustic FDTD time step for sm_103a: two streaming passes advance every shot pair of a
// batch by one time level.
//
// Restates the Devito operator that IsoAcousticDevito builds (stride/physics/iso_acoustic/
// devito.py:1466-1608): p.dt2 - Lt + 2 a vp p.dt + vp^2 (2 d p.dtc + d^2 p) = 0 solved for the new
// level (:1575-1581), Lt = W G(p) (OT2) or l + dt^2/12 W G(l) with l = W G(p) (OT4, :1503-1534),
// G the 10th-order Laplacian (rho absent) or the staggered div(b grad) (:1655-1665), W = vp^2 or
// vp^2 rho. As Devito materialises its `laplacian` Function, OT4 runs two passes: pass L writes
// l (zero beyond the grid) and pass U applies G to l and updates the level; OT2 runs pass U on
// p itself. Sources, receivers and the imaging condition run as their own kernels after a step.
//
// Work assignment of a pass. A CTA owns a strip of output columns, a chunk of rows and one shot
// pair; each thread owns two adjacent columns (c, c + 1, c even), so every value it handles is a
// float4 {col c shot 0, col c shot 1, col c+1 shot 0, col c+1 shot 1} of the pair-interleaved
// field layout and all arithmetic is the packed FP32 pairs of the sm_100 family. Rows of the
// pass input stream through the CTA (2.5D):
//   * derivatives along the streamed x axis come from per-thread register queues whose slots
//     rotate by compile-time index: the row loop is unrolled over the queue period P, so a new
//     row costs no register moves;
//   * derivatives along y read 12-column windows of the shared input row as six 16-byte loads
//     (the windows of a thread's two columns overlap in 11 columns); the staggered operator's
//     y-fluxes are computed once per half-column and exchanged through a double-buffered shared
//     row, with one barrier per row;
//   * input rows arrive by cp.async (zero-fill beyond the grid: Devito's zero halo of p and of
//     `laplacian`) PF rows ahead; the update's p[t] / p[t-1] values by per-thread cp.async PF2
//     rows ahead;
//   * the medium (one float per point and field) is loaded as the thread's two columns in one
//     8-byte load, AHEAD rows before its use, each value serving both shots of the pair.
// The new level is written in place of p[t-1] (each point's old value is read only by the
// thread that writes its new value). The undersampled save of p.dt2 or of p (:398-418) is a
// fused epilogue of pass U.
#pragma once
#include <utility>

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

// ---- packed FP32 arithmetic on the two shots of a pair (one sm_100-family f32x2 instruction) --
__device__ __forceinline__ float2 f2(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, f2(-1.f), a); }  // exact a - b

// Two columns (c, c + 1) of a shot pair.
struct Col2 {
    float2 a, b;
};
__device__ __forceinline__ Col2 as_col2(float4 v) { return {make_float2(v.x, v.y), make_float2(v.z, v.w)}; }
__device__ __forceinline__ float4 as_f4(Col2 v) { return make_float4(v.a.x, v.a.y, v.b.x, v.b.y); }
__device__ __forceinline__ Col2 ld_c2(const float4* p) { return as_col2(*p); }
__device__ __forceinline__ Col2 zero_c2() { return {f2(0.f), f2(0.f)}; }
__device__ __forceinline__ Col2 add_c2(Col2 x, Col2 y) { return {add2(x.a, y.a), add2(x.b, y.b)}; }
__device__ __forceinline__ Col2 mul_c2(Col2 x, Col2 y) { return {mul2(x.a, y.a), mul2(x.b, y.b)}; }
__device__ __forceinline__ Col2 fma_c2(Col2 x, Col2 y, Col2 z) { return {fma2(x.a, y.a, z.a), fma2(x.b, y.b, z.b)}; }

// Staggered first derivative along a queue: sum_m w[m] (q[(K + HI + m) % P] - q[(K + LO - m) % P]).
template <int P, int K, int HI, int LO>
__device__ __forceinline__ Col2 qstag(const Col2 (&q)[P], const float2 (&w)[6]) {
    constexpr int h0 = ((K + HI) % P + P) % P, l0 = ((K + LO) % P + P) % P;
    Col2 acc;
    acc.a = mul2(w[0], sub2(q[h0].a, q[l0].a));
    acc.b = mul2(w[0], sub2(q[h0].b, q[l0].b));
#pragma unroll
    for (int m = 1; m < 5; m++) {
        const int h = ((K + HI + m) % P + P) % P, l = ((K + LO - m) % P + P) % P;
        acc.a = fma2(w[m], sub2(q[h].a, q[l].a), acc.a);
        acc.b = fma2(w[m], sub2(q[h].b, q[l].b), acc.b);
    }
    return acc;
}
// Centred second derivative along a queue about slot (K + C) % P.
template <int P, int K, int C>
__device__ __forceinline__ Col2 qcent(const Col2 (&q)[P], const float2 (&w)[6]) {
    constexpr int c0 = ((K + C) % P + P) % P;
    Col2 acc;
    acc.a = mul2(w[0], q[c0].a);
    acc.b = mul2(w[0], q[c0].b);
#pragma unroll
    for (int k = 1; k <= 5; k++) {
        const int h = ((K + C + k) % P + P) % P, l = ((K + C - k) % P + P) % P;
        acc.a = fma2(w[k], add2(q[h].a, q[l].a), acc.a);
        acc.b = fma2(w[k], add2(q[h].b, q[l].b), acc.b);
    }
    return acc;
}

// Staggered y-fluxes at half-columns 4 and 5 of a 12-column window of a shared row (float2 per
// column, window start at float4 index k): F(h) = sum_m w[m] (v[h + 1 + m] - v[h - m]).
__device__ __forceinline__ Col2 yflux_pair(const float4* row, int k, const float2 (&w)[6]) {
    float2 v[12];
#pragma unroll
    for (int e = 0; e < 6; e++) {
        const float4 q = row[k + e];
        v[2 * e] = make_float2(q.x, q.y);
        v[2 * e + 1] = make_float2(q.z, q.w);
    }
    Col2 acc;
    acc.a = mul2(w[0], sub2(v[5], v[4]));
    acc.b = mul2(w[0], sub2(v[6], v[5]));
#pragma unroll
    for (int m = 1; m < 5; m++) {
        acc.a = fma2(w[m], sub2(v[5 + m], v[4 - m]), acc.a);
        acc.b = fma2(w[m], sub2(v[6 + m], v[5 - m]), acc.b);
    }
    return acc;
}
// D- along y at window columns 6 and 7 from a 12-entry flux window f starting at float4 index k0:
// D = sum_m w[m] (f[6 + m] - f[5 - m]) (flux f[e] at the half-column after window column e).
__device__ __forceinline__ Col2 ydiv_pair(const float4* frow, int k0, const float2 (&w)[6]) {
    float2 v[12];
#pragma unroll
    for (int e = 0; e < 6; e++) {
        const float4 q = frow[k0 + e];
        v[2 * e] = make_float2(q.x, q.y);
        v[2 * e + 1] = make_float2(q.z, q.w);
    }
    Col2 acc;
    acc.a = mul2(w[0], sub2(v[6], v[5]));
    acc.b = mul2(w[0], sub2(v[7], v[6]));
#pragma unroll
    for (int m = 1; m < 5; m++) {
        acc.a = fma2(w[m], sub2(v[6 + m], v[5 - m]), acc.a);
        acc.b = fma2(w[m], sub2(v[7 + m], v[6 - m]), acc.b);
    }
    return acc;
}
// Centred second derivative along y at window columns 6 and 7 of a 14-column window starting at
// float4 index k0.
__device__ __forceinline__ Col2 ycent_pair(const float4* row, int k0, const float2 (&w)[6]) {
    float2 v[14];
#pragma unroll
    for (int e = 0; e < 7; e++) {
        const float4 q = row[k0 + e];
        v[2 * e] = make_float2(q.x, q.y);
        v[2 * e + 1] = make_float2(q.z, q.w);
    }
    Col2 acc;
    acc.a = mul2(w[0], v[6]);
    acc.b = mul2(w[0], v[7]);
#pragma unroll
    for (int k = 1; k <= 5; k++) {
        acc.a = fma2(w[k], add2(v[6 + k], v[6 - k]), acc.a);
        acc.b = fma2(w[k], add2(v[7 + k], v[7 - k]), acc.b);
    }
    return acc;
}

template <int... K, class F>
__device__ __forceinline__ void unroll_period(std::integer_sequence<int, K...>, F&& f) {
    (f(std::integral_constant<int, K>{}), ...);
}

// What a pass computes.
enum PassMode : int {
    PASS_L = 0,   // l = W G(p[t]) into Step2D::lbuf (OT4's first pass)
    PASS_U4 = 1,  // new = C1 (l + dt^2/12 W G(l)) + C2 p[t] - C3 p[t-1] (OT4's second pass)
    PASS_U2 = 2,  // new = C1 W G(p[t]) + C2 p[t] - C3 p[t-1], or W G(p[t]) with wg_only (OT2)
};

#ifndef SA_PASS_MINB
#define SA_PASS_MINB 3
#endif
#ifndef SA_PASS_PF
#define SA_PASS_PF 3
#endif
#ifndef SA_PASS_QC
#define SA_PASS_QC 4
#endif
#ifndef SA_PASS_AHEAD
#define SA_PASS_AHEAD 2
#endif

// Geometry of a pass CTA of nt threads (nt <= STEP_MAX_THREADS, runtime): operator kind fixes
// the reach, the mode which per-thread update rings exist. Shared memory in float4 units.
template <int KIND, int MODE>
struct PassCfg {
    static constexpr bool STAG = KIND != 0;    // staggered div(b grad) operator
    static constexpr bool VARB = KIND == 1;    // variable buoyancy
    static constexpr int R = STAG ? 9 : 5;     // rows / columns of one operator application
    static constexpr int P = STAG ? 10 : 11;   // rows per period of the register queues
    static constexpr int UL = STAG ? 10 : 6;   // input columns left of the thread columns
    static constexpr int UX = STAG ? 10 : 7;   // float4 of an input row beyond the threads'
    static constexpr int QU = 16;              // shared input rows (ring)
    static constexpr int PF = SA_PASS_PF;      // input rows prefetched ahead (QU >= R + PF + 1)
    static constexpr int QC = SA_PASS_QC;      // rows of the update's p[t] / p[t-1] ring
    static constexpr int PF2 = SA_PASS_PF;     // update rows prefetched ahead (PF <= PF2 < QC)
    static constexpr bool HAS_C = MODE == PASS_U4;  // p[t] ring (U2 takes p[t] from its input queue)
    static constexpr bool HAS_P = MODE != PASS_L;   // p[t-1] ring
    __host__ __device__ static constexpr int WU(int nt) { return nt + UX; }
    __host__ __device__ static constexpr int NF(int nt) { return STAG ? nt + 5 : 0; }
    __host__ __device__ static constexpr int oF(int nt) { return QU * WU(nt); }
    __host__ __device__ static constexpr int oC(int nt) { return oF(nt) + 2 * NF(nt); }
    __host__ __device__ static constexpr int oP(int nt) { return oC(nt) + (HAS_C ? QC * nt : 0); }
    __host__ __device__ static constexpr int total(int nt) { return oP(nt) + (HAS_P ? QC * nt : 0); }
    __host__ __device__ static constexpr size_t bytes(int nt) { return (size_t)total(nt) * sizeof(float4); }
    static_assert(QU >= R + PF + 1 && (QU & (QU - 1)) == 0, "input ring");
    static_assert(PF2 >= PF && PF2 < QC && (QC & (QC - 1)) == 0, "update ring");
    static_assert(P % 2 == 0 || !STAG, "flux buffers alternate by the parity of the period slot");
};

// The medium values one iteration of a pass uses, each as the two values of the thread's columns
// (c, c + 1) (used for both shots of the pair). Each is reloaded AHEAD iterations further right
// after its last use, so the loads are in flight for AHEAD rows.
struct PassMedium {
    float2 by, byb;     // buoyancy at the y-flux half-columns of the thread's pair (and its extra pair)
    float2 bx;          // buoyancy at the x-flux half-row
    float2 W;           // W at the output row
    float2 c1, c2, nc3; // update coefficients at the output row
};
__device__ __forceinline__ Col2 dup_c2(float2 v) { return {f2(v.x), f2(v.y)}; }

template <int KIND, int MODE>
__global__ void __launch_bounds__(STEP_MAX_THREADS, SA_PASS_MINB) fdtd2d_pass(const __grid_constant__ Step2D a) {
    using CF = PassCfg<KIND, MODE>;
    constexpr bool STAG = CF::STAG, VARB = CF::VARB;
    constexpr int R = CF::R, UL = CF::UL, P = CF::P, QU = CF::QU, PF = CF::PF, QC = CF::QC, PF2 = CF::PF2;

    const int NT = blockDim.x;
    const int WU = CF::WU(NT), NF = CF::NF(NT);
    extern __shared__ __align__(16) float4 smem4[];
    float4* const sU = smem4;
    float4* const sF = smem4 + CF::oF(NT);
    float4* const sC = smem4 + CF::oC(NT);
    float4* const sP = smem4 + CF::oP(NT);

    const int tid = threadIdx.x;
    const int strip = blockIdx.x, chunk = blockIdx.y, pair = blockIdx.z;
    const int y0 = strip * a.by;
    const int BY = min(a.by, a.ny - y0);       // output columns of this strip
    const int L0 = y0 - UL;                    // column of shared input index 0 (even)
    const int c = y0 + 2 * tid;                // this thread's columns c, c + 1
    const int xo0 = chunk * a.chunk_rows;
    const int xo1 = min(a.nx, xo0 + a.chunk_rows);
    const int i0 = xo0 - R;                    // first input row streamed
    const int niter = (xo1 - xo0) + 2 * R;     // rows streamed; row i0 + n - R is output from n = 2R
    const int pitch = a.pitch;

    const bool out_t = 2 * tid < BY;           // output columns of this thread
    const bool out1 = out_t && c + 1 < a.ny;
    const int cm = min(c, a.ymax);             // medium column (clamped beyond the grid)

    const long long poff = (long long)pair * a.shot_stride * 2;  // floats per pair
    const float* __restrict__ in = (MODE == PASS_U4 ? a.lbuf : a.cur) + poff;
    const float* __restrict__ cur = a.cur + poff;
    float* __restrict__ prev = a.prev + poff;
    float* __restrict__ outp = (MODE == PASS_L ? a.lbuf : a.prev) + poff;

    float2 wx[6], wy[6];
#pragma unroll
    for (int m = 0; m < 6; m++) {
        wx[m] = a.wx[m];
        wy[m] = a.wy[m];
    }
    const bool do_save = MODE != PASS_L && a.save && (a.t % a.f == 0);

    // ---- prefetch of input rows (whole CTA) and of the update's p[t] / p[t-1] (own columns) ---
    // input-row copies of this thread: float4 k = tid and k = tid + NT (< WU), columns L0 + 2k,
    // L0 + 2k + 1, zero-filled outside the row's pitch
    const bool has2 = tid + NT < WU;
    const int q1 = L0 + 2 * tid, q2 = L0 + 2 * (tid + NT);
    const bool ok1 = q1 >= 0 && q1 + 2 <= pitch, ok2 = has2 && q2 >= 0 && q2 + 2 <= pitch;
    const int so1 = ok1 ? 2 * q1 : 0, so2 = ok2 ? 2 * q2 : 0;
    auto prefetch_in = [&](int n) {  // input row i0 + n into ring slot n % QU
        const int r = i0 + n;
        float4* dst = sU + (n & (QU - 1)) * WU + tid;
        const bool row_ok = r >= 0 && r < a.nx;
        const float* rowp = row_ok ? in + (long long)r * pitch * 2 : in;
        cp_async16(dst, rowp + so1, row_ok && ok1);
        if (has2) cp_async16(dst + NT, rowp + so2, row_ok && ok2);
    };
    auto out_row = [&](int n) { return i0 + n - R; };  // output row of iteration n (stored from n = 2R)
    auto prefetch_upd = [&](int n) {                   // p[t], p[t-1] at the output row of iteration n
        if constexpr (MODE != PASS_L) {
            const int ro = out_row(n);
            if (ro < xo0 || ro >= xo1 || !out_t) return;
            const long long off = (long long)ro * pitch * 2 + 2 * c;
            if constexpr (CF::HAS_C) cp_async16(sC + (n & (QC - 1)) * NT + tid, cur + off, true);
            cp_async16(sP + (n & (QC - 1)) * NT + tid, prev + off, true);
        }
    };
    for (int n = 0; n < PF; n++) {
        prefetch_in(n);
        if (n == 0)
            for (int m = 0; m < PF2; m++) prefetch_upd(m);
        cp_async_commit();
    }

    // ---- medium: pointers at this thread's (clamped) columns, rows added per iteration --------
    // AHEAD sets of values rotate with the iteration (slot n % AHEAD; AHEAD divides P)
    constexpr int AHEAD = (P % SA_PASS_AHEAD == 0) ? SA_PASS_AHEAD : 1;
    const int mp = a.mpitch;
    const float* __restrict__ mW = a.Wm + cm;
    const float* __restrict__ mBX = a.bxm + cm;
    const float* __restrict__ mC1 = a.C1m + cm;
    const float* __restrict__ mC2 = a.C2m + cm;
    const float* __restrict__ mC3 = a.NC3m + cm;
    // y-flux pair k = tid at half-columns y0 - 6 + 2k (and k = tid + NT for tid < 5)
    const float* __restrict__ mBY = a.bym + min(max(y0 - 6 + 2 * tid, -MED_MARGIN), a.ymax);
    const float* __restrict__ mBYb = a.bym + min(max(y0 - 6 + 2 * (tid + NT), -MED_MARGIN), a.ymax);
    auto ldm = [](const float* p) { return __ldg(reinterpret_cast<const float2*>(p)); };
    PassMedium md[AHEAD];
    auto ld_by = [&](PassMedium& m, int n) {  // output row
        const long long r = (long long)out_row(n) * mp;
        m.by = ldm(mBY + r);
        if (tid < 5) m.byb = ldm(mBYb + r);
    };
    auto ld_bx = [&](PassMedium& m, int n) { m.bx = ldm(mBX + (long long)(i0 + n - 5) * mp); };  // x-flux half-row
    auto ld_W = [&](PassMedium& m, int n) { m.W = ldm(mW + (long long)out_row(n) * mp); };
    auto ld_upd = [&](PassMedium& m, int n) {
        if constexpr (MODE != PASS_L) {
            const int ro = out_row(n);
            if (ro < xo0 || ro >= xo1 || !out_t || a.wg_only) return;
            const long long r = (long long)ro * mp;
            m.c1 = ldm(mC1 + r);
            m.c2 = ldm(mC2 + r);
            m.nc3 = ldm(mC3 + r);
        }
    };
#pragma unroll
    for (int k = 0; k < AHEAD; k++) {
        md[k].byb = make_float2(0.f, 0.f);
        if constexpr (VARB) {
            ld_by(md[k], k);
            ld_bx(md[k], k);
        }
        ld_W(md[k], k);
        ld_upd(md[k], k);
    }

    // ---- register queues (slot = iteration number mod P): input rows, staggered x-fluxes -------
    Col2 uq[P], fq[STAG ? P : 1];
#pragma unroll
    for (int k = 0; k < P; k++) {
        uq[k] = zero_c2();
        if constexpr (STAG) fq[k] = zero_c2();
    }
    // Warm-up: iteration n feeds the x-fluxes from n >= R (staggered) and outputs from n >= 2R;
    // earlier work would only reach rows that are not stored.
#pragma unroll 1
    for (int base = 0; base < niter; base += P) {
        unroll_period(std::make_integer_sequence<int, P>{}, [&](auto KC) {
            constexpr int K = decltype(KC)::value;
            const int n = base + K;
            if (n >= niter) return;  // uniform: the barrier below is reached by all or none
            [[maybe_unused]] const int par = K & 1;
            const bool outn = n >= 2 * R;
            PassMedium& m = md[K % AHEAD];

            // ---- phase A: y-fluxes of the output row (its input row is visible since earlier
            // barriers) into this iteration's flux buffer ----------------------------------------
            if constexpr (STAG) {
                if (outn) {
                    // input row r = i - R: index e <-> column L0 + e; pair k at half-columns y0 - 6 + 2k
                    const float4* urow = sU + ((n - R) & (QU - 1)) * WU;
                    Col2 F = yflux_pair(urow, tid, wy);
                    if constexpr (VARB) F = mul_c2(F, dup_c2(m.by));
                    sF[par * NF + tid] = as_f4(F);
                    if (tid < 5) {
                        Col2 Fb = yflux_pair(urow, tid + NT, wy);
                        if constexpr (VARB) Fb = mul_c2(Fb, dup_c2(m.byb));
                        sF[par * NF + tid + NT] = as_f4(Fb);
                    }
                }
                if constexpr (VARB) ld_by(m, n + AHEAD);
            }
            cp_async_wait<PF - 1>();
            __syncthreads();  // input row i, this iteration's fluxes visible; the previous iteration done
            prefetch_in(n + PF);
            prefetch_upd(n + PF2);
            cp_async_commit();

            // ---- G(in) at the output row r = i - R ----------------------------------------------
            uq[K] = ld_c2(sU + (n & (QU - 1)) * WU + tid + UL / 2);  // input row i, own columns
            if constexpr (STAG) {
                if (n >= R) {  // x-flux at half-row i - 5 from input rows i - 9 .. i
                    Col2 fx = qstag<P, K, -4, -5>(uq, wx);
                    if constexpr (VARB) fx = mul_c2(fx, dup_c2(m.bx));
                    fq[K] = fx;
                }
                if constexpr (VARB) ld_bx(m, n + AHEAD);
            }
            if (outn) {
                Col2 g;
                if constexpr (STAG) {
                    // D- along x at row r from fluxes at half-rows r - 5 .. r + 4 (iterations K - 9 .. K)
                    const Col2 gx = qstag<P, K, -4, -5>(fq, wx);
                    // D- along y at (c, c + 1) from flux pairs tid .. tid + 5
                    const Col2 gy = ydiv_pair(sF + par * NF, tid, wy);
                    g = add_c2(gx, gy);
                } else {
                    const Col2 gx = qcent<P, K, -5>(uq, wx);  // input rows i - 10 .. i about r = i - 5
                    const Col2 gy = ycent_pair(sU + ((n - R) & (QU - 1)) * WU, tid, wy);
                    g = add_c2(gx, gy);
                }
                [[maybe_unused]] const Col2 in_r = uq[((K - R) % P + P) % P];  // the input at the output row
                const int r = out_row(n);
                const long long idx = (long long)r * pitch + c;  // float2 index within the pair
                Col2 res;
                if constexpr (MODE == PASS_L) {
                    res = mul_c2(dup_c2(m.W), g);  // l; rows and columns beyond the grid are never stored (zero)
                } else {
                    Col2 Lt;
                    if constexpr (MODE == PASS_U4) {
                        Lt = fma_c2(dup_c2(make_float2(m.W.x * a.k12, m.W.y * a.k12)), g, in_r);
                    } else {
                        Lt = mul_c2(dup_c2(m.W), g);
                    }
                    if (out_t) {
                        const Col2 u_o = CF::HAS_C ? ld_c2(sC + (n & (QC - 1)) * NT + tid) : in_r;
                        const Col2 pm = ld_c2(sP + (n & (QC - 1)) * NT + tid);
                        if (a.wg_only) {
                            res = Lt;
                        } else {
                            res.a = fma2(f2(m.c1.x), Lt.a, fma2(f2(m.c2.x), u_o.a, mul2(f2(m.nc3.x), pm.a)));
                            res.b = fma2(f2(m.c1.y), Lt.b, fma2(f2(m.c2.y), u_o.b, mul2(f2(m.nc3.y), pm.b)));
                        }
                        if (do_save) {
                            float2* snap = reinterpret_cast<float2*>(a.snaps) + (long long)pair * a.snap_shot_stride +
                                           (long long)(a.t / a.f) * a.snap_stride + idx;
                            Col2 sv;
                            if (a.save == 2) {
                                sv = u_o;  // raw p[t] (rho / wavelet gradients)
                            } else {
                                const float2 id = f2(a.inv_dt2);
                                sv.a = mul2(add2(sub2(res.a, add2(u_o.a, u_o.a)), pm.a), id);
                                sv.b = mul2(add2(sub2(res.b, add2(u_o.b, u_o.b)), pm.b), id);
                            }
                            if (out1) *reinterpret_cast<float4*>(snap) = as_f4(sv);
                            else *snap = sv.a;
                        }
                    }
                }
                if (out_t) {
                    float2* dst = reinterpret_cast<float2*>(outp) + idx;
                    if (out1) *reinterpret_cast<float4*>(dst) = as_f4(res);
                    else *dst = res.a;
                }
            }
            ld_W(m, n + AHEAD);
            ld_upd(m, n + AHEAD);
        });
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

// 3D iso-acoustic FDTD time step for sm_103a (stride/physics/iso_acoustic/devito.py:1466-1608 in
// 3D). The grid is [x][y][z], z contiguous, one array per shot. A CTA owns a TY x TZ tile of
// (y, z) columns of a PAIR of shots and computes both in packed FP32 (one f32x2 instruction for
// the two shots; a lone shot of an odd batch runs the same code with one lane): it streams the x
// planes of its input field through a shared-memory ring (the two shots interleaved by 4-byte
// cp.async, zero-filled beyond the grid: Devito's zero halo). The y and z derivatives of a row are
// taken from its plane as soon as it arrives and wait in a per-thread shared-memory ring until the
// x derivatives (per-thread register queues along x) reach that row, so the plane ring holds only
// the planes in flight.
//
// One application of the spatial operator per pass (a 3D halo of 9 cells around a small tile
// makes fusing OT4's two applications more expensive than a second pass):
//   pass INTERMEDIATE: l = W G(in) on the grid (zero outside), written to memory;
//   pass FINAL:        Lt = W G(u) (OT2, in = u) or l + dt^2/12 W G(l) (OT4, in = l), then the
//                      update p_new = C1 Lt + C2 p - C3 p_other, the p.dt2 save (forward) and
//                      the imaging condition (adjoint).
// Sparse operations (source/receiver injection, receiver interpolation) run in small kernels
// after the FINAL pass.
#pragma once
#include <type_traits>
#include "common.cuh"
#include "fdtd2d.cuh"

namespace sa {

struct Step3D {
    int nx, ny, nz, zp;       // extended grid and z pitch
    long long shot_stride;    // floats per shot in a field buffer (nx*ny*zp)
    int chunk_rows;           // output x rows per CTA
    int ty0n;                 // tiles along y
    int nshots;               // shots of the batch
    int shot0, npairs;        // this launch: two lanes, blockIdx.x = pair + npairs * (tile_y + ty0n * tile_z),
                              // pair p holding shots shot0 + 2p and shot0 + 2p + 1; one lane (a lone shot),
                              // blockIdx.x = tile, shot shot0
    int t;
    const float* in;          // streamed field: u (OT2 / INTERMEDIATE) or l (OT4 FINAL)
    const float* cur;         // p[t] (FINAL: the current level at the output)
    float* prev;              // other level in, new level out (FINAL)
    float* out_l;             // INTERMEDIATE output
    // medium, [x][y][zp] with GUARD zero x planes on both sides; pointers address x = 0
    const float* W;
    const float* bxh;         // b(x+1/2, y, z), half-planes -5..nx+3
    const float* byh;         // b(x, y+1/2, z): y row y+6 holds y = -6..ny+3 ([x][ny+12][zp])
    const float* bzh;         // b(x, y, z+1/2): column z+6 holds z = -6..nz+3 ([x][y][zpb])
    int zpb;
    const float* C1;
    const float* C2;
    const float* C3;
    float hx, hy, hz, dt;
    // wavefield save
    int f, save;
    float* snaps;             // [shots][n_snap][nx][ny][zp]
    long long snap_shot_stride, snap_stride;
};

__host__ __device__ constexpr int pow2_at_least(int x) { return x <= 1 ? 1 : 2 * pow2_at_least((x + 1) / 2); }

__device__ __forceinline__ void cp_async4(void* smem, const void* gmem, bool valid) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    const int sz = valid ? 4 : 0;  // 0: zero-fill, nothing is read
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(sa), "l"(gmem), "r"(sz) : "memory");
}

template <int KIND, int TY, int TZ, int RB, int PF, int LANES = 2>
struct Smem3D {
    static constexpr bool STAG = KIND != 0;
    static constexpr int R = STAG ? 9 : 5;
    static constexpr int PY = TY + 2 * R;     // plane rows (y) incl. halo
    static constexpr int PZ = TZ + 2 * R;     // plane row width (z) incl. halo, from z0 - R
    static constexpr int PLANE = PY * PZ;     // values of the lanes (float2: the two shots of a pair)
    // planes in the ring (this iteration's and the prefetched), a power of two: slots by mask
    static constexpr int QU = pow2_at_least(RB * (PF + 1));
    static constexpr int FY = (TY + 9) * TZ;  // y fluxes of one row
    // z fluxes of one row: TZ + 9 per y row, densely (every lane of a warp holds one)
    static constexpr int WZF = TZ + 9;
    static constexpr int FZ = TY * WZF;
    static constexpr int QG = pow2_at_least(R + RB);  // slots of the y and z parts waiting for their x part
    static constexpr int oFY = QU * PLANE;
    static constexpr int oFZ = oFY + (STAG ? RB * FY : 0);
    static constexpr int oG = oFZ + (STAG ? RB * FZ : 0);
    static constexpr int total = oG + QG * TY * TZ;
    static constexpr size_t bytes = (size_t)total * sizeof(float) * LANES;
};

// Lane arithmetic: V = float2 (a pair of shots, one f32x2 instruction) or float (a lone shot).
template <class V> __device__ __forceinline__ V vs(float v);
template <> __device__ __forceinline__ float vs<float>(float v) { return v; }
template <> __device__ __forceinline__ float2 vs<float2>(float v) { return f2(v); }
__device__ __forceinline__ float vfma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ float2 vfma(float2 a, float2 b, float2 c) { return fma2(a, b, c); }
__device__ __forceinline__ float vmul(float a, float b) { return a * b; }
__device__ __forceinline__ float2 vmul(float2 a, float2 b) { return mul2(a, b); }
__device__ __forceinline__ float vadd(float a, float b) { return a + b; }
__device__ __forceinline__ float2 vadd(float2 a, float2 b) { return add2(a, b); }
__device__ __forceinline__ float vsub(float a, float b) { return fmaf(b, -1.f, a); }
__device__ __forceinline__ float2 vsub(float2 a, float2 b) { return sub2(a, b); }

template <int QL, int RB, class V>
__device__ __forceinline__ void qshift(V (&q)[QL]) {
#pragma unroll
    for (int k = 0; k + RB < QL; k++) q[k] = q[k + RB];
}
template <class V, class A>
__device__ __forceinline__ V dstag(const A& v, int hi, int lo, int stride) {
    V a = vmul(vs<V>(kWS(0)), v[hi]), b = vmul(vs<V>(kWS(0)), v[lo]);
#pragma unroll
    for (int m = 1; m < 5; m++) {
        a = vfma(vs<V>(kWS(m)), v[hi + m * stride], a);
        b = vfma(vs<V>(kWS(m)), v[lo - m * stride], b);
    }
    return vsub(a, b);
}
template <class V, class A>
__device__ __forceinline__ V dcent(const A& v, int c, int stride) {
    V a = vmul(vs<V>(kW2(0)), v[c]);
#pragma unroll
    for (int k = 1; k <= 5; k++) a = vfma(vs<V>(kW2(k)), vadd(v[c + k * stride], v[c - k * stride]), a);
    return a;
}

template <int KIND, bool FINAL, bool OT4, int TY, int TZ, int RB, int PF, int LANES>
__global__ void __launch_bounds__(TY* TZ, TY* TZ <= 256 ? 2 : 1) fdtd3d_pass(const __grid_constant__ Step3D a) {
    using L = Smem3D<KIND, TY, TZ, RB, PF, LANES>;
    using V = typename std::conditional<LANES == 2, float2, float>::type;
    constexpr int NT = TY * TZ;
    constexpr bool STAG = L::STAG, VARB = KIND == 1;
    constexpr int R = L::R, QU = L::QU, PZ = L::PZ, WZF = L::WZF;
    constexpr int QB = STAG ? 9 : 10;  // x queue: rows i - QB .. i + RB - 1
    constexpr int QL = QB + RB;
    constexpr int QG = L::QG;          // y/z parts of rows i - R .. i + RB - 1, one slot per row

    extern __shared__ __align__(16) float smem_f[];
    V* const smem2 = reinterpret_cast<V*>(smem_f);
    V* const sU = smem2;
    V* const sFY = smem2 + L::oFY;
    V* const sFZ = smem2 + L::oFZ;
    V* const sG = smem2 + L::oG + threadIdx.x;  // this thread's y/z parts: slot s at sG[s NT]

    const int tid = threadIdx.x;
    const int tz = tid % TZ, ty = tid / TZ;
    const int npairs = LANES == 2 ? a.npairs : 1;
    const int pair = blockIdx.x % npairs, tile = blockIdx.x / npairs;
    constexpr bool hasB = LANES == 2;
    const int tile_y = tile % a.ty0n, tile_z = tile / a.ty0n;
    const int chunk = blockIdx.y;
    const int y0 = tile_y * TY, z0 = tile_z * TZ;
    const int y = y0 + ty, z = z0 + tz;
    const bool col_in = y < a.ny && z < a.nz;
    const int yc = min(y, a.ny - 1), zc = min(z, a.nz - 1);
    const int xo0 = chunk * a.chunk_rows, xo1 = min(a.nx, xo0 + a.chunk_rows);
    const int i0 = xo0 - R, i1 = xo1 + R;
    const long long plane = (long long)a.ny * a.zp;
    const int shotA = a.shot0 + (LANES == 2 ? 2 * pair : 0);
    const long long offA = (long long)shotA * a.shot_stride;
    const long long offB = offA + a.shot_stride;  // the pair's second shot (two lanes only)
    const long long col = (long long)yc * a.zp + zc;             // offset of this column in a plane
    const float ihx = 1.f / a.hx, ihy = 1.f / a.hy, ihz = 1.f / a.hz;
    const float ihx2 = ihx * ihx, ihy2 = ihy * ihy, ihz2 = ihz * ihz;
    const float dt2 = a.dt * a.dt;
    const float k12 = (float)((double)a.dt * (double)a.dt / 12.0);

    // plane ring: x row r in slot (r - i0) mod QU, kept as a running slot index (sI: row i);
    // element (yy, zz) at [(yy - y0 + R) PZ + zz - z0 + R]
    auto wrap = [](int s) { return s & (QU - 1); };
    auto slotp = [&](int s) { return sU + s * L::PLANE; };
    // the plane elements this thread stages (element tid + q NT): their offset within an x plane
    // of the field, -1 beyond the grid (the same for every row)
    constexpr int NS = (L::PLANE + NT - 1) / NT;
    int gofs[NS];
#pragma unroll
    for (int q = 0; q < NS; q++) {
        const int k = tid + q * NT, py = k / PZ, pz = k - py * PZ;
        const int yy = y0 - R + py, zz = z0 - R + pz;
        gofs[q] = k < L::PLANE && yy >= 0 && yy < a.ny && zz >= 0 && zz < a.nz ? yy * a.zp + zz : -1;
    }
    const float* const inA = a.in + offA;
    const float* const inB = a.in + offB;
    auto prefetch = [&](int ii, int si) {  // rows ii, ii+1, ... into slots si, si+1, ...
#pragma unroll
        for (int rr = 0; rr < RB; rr++) {
            const int r = ii + rr;
            if (r < i1) {
                V* dst = slotp(wrap(si + rr)) + tid;
                const bool row_ok = r >= 0 && r < a.nx;
                const float* ga = inA + (row_ok ? (long long)r * plane : 0);
                [[maybe_unused]] const float* gb = inB + (row_ok ? (long long)r * plane : 0);
#pragma unroll
                for (int q = 0; q < NS; q++) {
                    if (q * NT + tid >= L::PLANE) break;
                    const bool ok = row_ok && gofs[q] >= 0;
                    const int o = ok ? gofs[q] : 0;
                    float* d = reinterpret_cast<float*>(dst + q * NT);
                    cp_async4(d, ga + o, ok);
                    if constexpr (hasB) cp_async4(d + 1, gb + o, ok);
                }
            }
        }
        cp_async_commit();
    };
    const int me = (ty + R) * PZ + (tz + R);  // this column's index in a plane

    // offsets of this thread's y- and z-flux buoyancies within an x plane of byh / bzh
    constexpr int KY = ((TY + 9) * TZ + NT - 1) / NT, KZ = (TY * WZF + NT - 1) / NT;
    int byo[VARB ? KY : 1], bzo[VARB ? KZ : 1];
    if constexpr (VARB) {
#pragma unroll
        for (int q = 0; q < KY; q++) {
            const int k = tid + q * NT;
            const int ky = min(k / TZ, TY + 8), kz = k % TZ;
            byo[q] = min(max(y0 - 5 + ky + 6, 0), a.ny + 9) * a.zp + min(z0 + kz, a.nz - 1);
        }
#pragma unroll
        for (int q = 0; q < KZ; q++) {
            const int k = tid + q * NT;
            const int ky = min(k / WZF, TY - 1), kz = k % WZF;  // (k beyond the row's fluxes: clamped, unused)
            bzo[q] = min(y0 + ky, a.ny - 1) * a.zpb + min(max(z0 - 5 + kz + 6, 0), a.zpb - 1);
        }
    }
    const long long byplane = (long long)(a.ny + 12) * a.zp, bzplane = (long long)a.ny * a.zpb;
    const int cidx = y * a.zp + z;  // this column's offset within a field plane (when col_in)

    V uq[QL], fq[STAG ? QL : 1];
#pragma unroll
    for (int k = 0; k < QL; k++) {
        uq[k] = vs<V>(0.f);
        if constexpr (STAG) fq[k] = vs<V>(0.f);
    }
    auto gwrap = [](int s) { return s & (QG - 1); };
    const bool do_save = FINAL && a.save && (a.t % a.f == 0);

#pragma unroll 1
    for (int k = 0; k < PF; k++) prefetch(i0 + k * RB, k * RB);

    int sI = 0;  // ring slot of row i (taken mod QU)
    int gI = 0;  // y/z-part slot of row i (mod QG; rows i0 .. i0 + R - 1 are never output rows)
#pragma unroll 1
    for (int i = i0; i < i1; i += RB) {
        const int j = i - R;  // output row of this iteration's first input row
        float Wj[RB], bxi[RB], byv[RB][VARB ? KY : 1], bzv[RB][VARB ? KZ : 1];
        float c1v[RB], c2v[RB], c3v[RB];
        V uov[RB], pmv[RB];
#pragma unroll
        for (int r = 0; r < RB; r++) {
            Wj[r] = __ldg(a.W + (long long)(j + r) * plane + col);
            if constexpr (VARB) {
                bxi[r] = __ldg(a.bxh + (long long)(i - 5 + r) * plane + col);
                // buoyancies of the y and z fluxes of the arriving row i + r
                const int xx = min(max(i + r, -sa::GUARD), a.nx + sa::GUARD - 1);
                const float* byr = a.byh + xx * byplane;
                const float* bzr = a.bzh + xx * bzplane;
#pragma unroll
                for (int q = 0; q < KY; q++) byv[r][q] = __ldg(byr + byo[q]);
#pragma unroll
                for (int q = 0; q < KZ; q++) bzv[r][q] = __ldg(bzr + bzo[q]);
            }
            if constexpr (FINAL) {
                const int row = j + r;
                const bool ok = row >= xo0 && row < xo1 && col_in;
                const long long idx = ok ? (long long)row * plane + cidx : 0;
                c1v[r] = ok ? __ldg(a.C1 + idx) : 0.f;
                c2v[r] = ok ? __ldg(a.C2 + idx) : 0.f;
                c3v[r] = ok ? -__ldg(a.C3 + idx) : 0.f;
                if constexpr (LANES == 2) {
                    uov[r] = make_float2(ok ? a.cur[offA + idx] : 0.f, ok ? a.cur[offB + idx] : 0.f);
                    pmv[r] = make_float2(ok ? a.prev[offA + idx] : 0.f, ok ? a.prev[offB + idx] : 0.f);
                } else {
                    uov[r] = ok ? a.cur[offA + idx] : 0.f;
                    pmv[r] = ok ? a.prev[offA + idx] : 0.f;
                }
            }
        }
        (void)bxi; (void)byv; (void)bzv; (void)c1v; (void)c2v; (void)c3v; (void)uov; (void)pmv;
        cp_async_wait<PF - 1>();
        __syncthreads();
        prefetch(i + PF * RB, sI + PF * RB);
#pragma unroll
        for (int r = 0; r < RB; r++) uq[QB + r] = slotp(wrap(sI + r))[me];
        // the y and z parts of the arriving rows i .. i+RB-1 (only rows that are output rows)
        if constexpr (STAG) {
#pragma unroll
            for (int r = 0; r < RB; r++) {
                if (i + r < xo0 || i + r >= xo1) continue;
                const V* pl = slotp(wrap(sI + r));
#pragma unroll
                for (int q = 0; q < KY; q++) {
                    const int k = tid + q * NT;
                    if (k < (TY + 9) * TZ) {
                        const int ky = k / TZ, kz = k % TZ;
                        const int base = (ky - 5 + R) * PZ + (kz + R);  // half row y0 - 5 + ky (+1/2)
                        V v = vmul(dstag<V>(pl, base + PZ, base, PZ), vs<V>(ihy));
                        if constexpr (VARB) v = vmul(v, vs<V>(byv[r][q]));
                        sFY[r * L::FY + k] = v;
                    }
                }
#pragma unroll
                for (int q = 0; q < KZ; q++) {
                    const int k = tid + q * NT;
                    const int ky = k / WZF, kz = k % WZF;
                    if (k < L::FZ) {
                        const int base = (ky + R) * PZ + (kz - 5 + R);  // half column z0 - 5 + kz (+1/2)
                        V v = vmul(dstag<V>(pl, base + 1, base, 1), vs<V>(ihz));
                        if constexpr (VARB) v = vmul(v, vs<V>(bzv[r][q]));
                        sFZ[r * L::FZ + k] = v;
                    }
                }
            }
            __syncthreads();
#pragma unroll
            for (int r = 0; r < RB; r++) {
                if (i + r < xo0 || i + r >= xo1) continue;
                const V* Fy = sFY + r * L::FY;
                const V* Fz = sFZ + r * L::FZ;
                // D- along y at row ty: fluxes at half rows ty-5 .. ty+4 (index ky = half - y0 + 5)
                const V gy = vmul(dstag<V>(Fy, (ty + 5) * TZ + tz, (ty + 4) * TZ + tz, TZ), vs<V>(ihy));
                const V gz = vmul(dstag<V>(Fz, ty * WZF + tz + 5, ty * WZF + tz + 4, 1), vs<V>(ihz));
                sG[gwrap(gI + r) * NT] = vadd(gy, gz);
            }
        } else {
#pragma unroll
            for (int r = 0; r < RB; r++) {
                if (i + r < xo0 || i + r >= xo1) continue;
                const V* pl = slotp(wrap(sI + r));
                sG[gwrap(gI + r) * NT] = vfma(dcent<V>(pl, me, PZ), vs<V>(ihy2), vmul(dcent<V>(pl, me, 1), vs<V>(ihz2)));
            }
        }
        // the x parts of the output rows j .. j+RB-1, their y and z parts from the queue
        V res[RB];
#pragma unroll
        for (int r = 0; r < RB; r++) {
            V gx;
            if constexpr (STAG) {
                V v = vmul(dstag<V>(uq, r + 5, r + 4, 1), vs<V>(ihx));
                if constexpr (VARB) v = vmul(v, vs<V>(bxi[r]));
                fq[QB + r] = v;
                gx = vmul(dstag<V>(fq, r + 5, r + 4, 1), vs<V>(ihx));
            } else {
                gx = vmul(dcent<V>(uq, r + 5, 1), vs<V>(ihx2));
            }
            // the y/z part of row j + r (written by this thread R rows ago; zero-row reads unused)
            const V g = vadd(gx, j + r >= xo0 && j + r < xo1 ? sG[gwrap(gI - R + r) * NT] : vs<V>(0.f));
            if constexpr (FINAL && OT4) {
                // Lt = l + dt^2/12 W G(l): the streamed l at row j+r is queue entry r (STAG,
                // rows i-9..) or r+5 (laplace, rows i-10..)
                res[r] = vfma(vs<V>(k12), vmul(vs<V>(Wj[r]), g), STAG ? uq[r] : uq[r + 5]);
            } else {
                res[r] = vmul(vs<V>(Wj[r]), g);
            }
        }
        qshift<QL, RB>(uq);
        if constexpr (STAG) qshift<QL, RB>(fq);
#pragma unroll
        for (int r = 0; r < RB; r++) {
            const int row = j + r;
            if (row < xo0 || row >= xo1 || !col_in) continue;
            const long long idx = (long long)row * plane + cidx;
            // lane values: .x and .y of a pair, the value itself for a lone shot
            const float* rv = reinterpret_cast<const float*>(&res[r]);
            if constexpr (!FINAL) {
                a.out_l[offA + idx] = rv[0];
                if constexpr (hasB) a.out_l[offB + idx] = rv[1];
            } else {
                const V u_o = uov[r], pm = pmv[r];
                const V pn = vfma(vs<V>(c1v[r]), res[r], vfma(vs<V>(c2v[r]), u_o, vmul(vs<V>(c3v[r]), pm)));
                const float* pnv = reinterpret_cast<const float*>(&pn);
                if (do_save) {  // 2: raw p[t] (rho gradient), else p.dt2
                    const float* uv = reinterpret_cast<const float*>(&u_o);
                    const float* pv = reinterpret_cast<const float*>(&pm);
                    float* sa0 = a.snaps + (long long)shotA * a.snap_shot_stride +
                                 (long long)(a.t / a.f) * a.snap_stride + idx;
#pragma unroll
                    for (int l = 0; l < LANES; l++)
                        sa0[l * a.snap_shot_stride] = a.save == 2 ? uv[l] : (pnv[l] - 2.f * uv[l] + pv[l]) / dt2;
                }
                a.prev[offA + idx] = pnv[0];
                if constexpr (hasB) a.prev[offB + idx] = pnv[1];
            }
        }
        sI += RB;
        gI += RB;
    }
    cp_async_wait<0>();
}

// Sparse epilogues of a 3D step: injection into the new level (and, when the level's p.dt2 is
// saved this step, into the saved snapshot: inj / dt^2), then receiver interpolation of the new
// level (trilinear, 8 corners).
struct Sparse3D {
    const int* shot;          // [n] shot of each point
    const int* base;          // [n][3] base corner
    const float* w;           // [n][8] corner weights (forward interpolation)
    const float* coef;        // [n][8] injection coefficients (weight * scale * vp^k at the corner)
};

// Wide interpolation in 3D (Hicks, common/devito.py:640-648,843-885; sinc, :634-638): injection as a
// flat list of weighted support points (up to 14^3 per source), receivers gathered over the support.
struct Entries3D {
    const int* shot;          // [n] shot of each entry
    const int* point;         // [n] its sparse point (row of the amplitude table)
    const long long* idx;     // [n] grid offset within a shot's field
    const float* coef;        // [n] weight * scale * vp^k at the support point
};
struct SupportGather3D {
    int x, y, z, point, shot, width;  // support origin (base - lo per axis) and points per axis
    float wx[SUPPORT_MAX], wy[SUPPORT_MAX], wz[SUPPORT_MAX];
};

__global__ void inject3d(const Sparse3D s, int n, const float* amp, int ld, int t, float* field, long long shot_stride,
                         int ny, int zp, float* snap, long long snap_shot_stride, long long snap_off, float inv_dt2);
__global__ void gather3d(const Sparse3D s, int n, const float* field, long long shot_stride, int ny, int zp, float* out,
                         int ld, int trow, float scale);

}  // namespace sa

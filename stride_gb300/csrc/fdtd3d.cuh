// 3D iso-acoustic FDTD time step for sm_103a (stride/physics/iso_acoustic/devito.py:1466-1608 in
// 3D). The grid is [x][y][z], z contiguous. A CTA owns a TY x TZ tile of (y, z) columns of one
// shot and streams the x planes of its input field through a shared-memory ring (16-byte
// cp.async, zero-filled beyond the grid: Devito's zero halo); x-derivatives come from
// per-thread register queues, y and z derivatives from the shared plane.
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
#include "common.cuh"
#include "fdtd2d.cuh"

namespace sa {

struct Step3D {
    int nx, ny, nz, zp;       // extended grid and z pitch
    long long shot_stride;    // floats per shot in a field buffer (nx*ny*zp)
    int chunk_rows;           // output x rows per CTA
    int ty0n;                 // tiles along y
    int nshots;               // blockIdx.x = shot + nshots * (tile_y + ty0n * tile_z): the shots of a
                              // tile run together and share the tile's medium through L2
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

template <int KIND, int TY, int TZ, int RB, int PF>
struct Smem3D {
    static constexpr bool STAG = KIND != 0;
    static constexpr int R = STAG ? 9 : 5;
    static constexpr int PY = TY + 2 * R;                   // plane rows (y) incl. halo
    static constexpr int PZ = round4(TZ + 2 * R + 3);       // plane row width (z) from floor4
    static constexpr int PLANE = PY * PZ;
    static constexpr int QU = R + RB * (PF + 1);            // planes kept: o .. i + RB*(PF+1) - 1
    static constexpr int FY = (TY + 9) * TZ;                // y fluxes of one row
    // z fluxes of one row: TZ + 9 per y row, stored at a power-of-two stride so that a flat index
    // splits into (y, z) with a shift and a mask
    static constexpr int WZF = pow2_at_least(TZ + 9);
    static constexpr int FZ = TY * WZF;
    static constexpr int oU = 0;
    static constexpr int oFY = QU * PLANE;
    static constexpr int oFZ = oFY + (STAG ? RB * FY : 0);
    static constexpr int total = oFZ + (STAG ? RB * FZ : 0);
    static constexpr size_t bytes = (size_t)total * sizeof(float);
};

template <int QL, int RB>
__device__ __forceinline__ void qshift1(float (&q)[QL]) {
#pragma unroll
    for (int k = 0; k + RB < QL; k++) q[k] = q[k + RB];
}
template <class A>
__device__ __forceinline__ float dstag_1(const A& v, int hi, int lo, int stride) {
    float a = kWS(0) * v[hi], b = kWS(0) * v[lo];
#pragma unroll
    for (int m = 1; m < 5; m++) {
        a = fmaf(kWS(m), v[hi + m * stride], a);
        b = fmaf(kWS(m), v[lo - m * stride], b);
    }
    return a - b;
}
template <class A>
__device__ __forceinline__ float dcent_1(const A& v, int c, int stride) {
    float a = kW2(0) * v[c];
#pragma unroll
    for (int k = 1; k <= 5; k++) a = fmaf(kW2(k), v[c + k * stride] + v[c - k * stride], a);
    return a;
}

template <int KIND, bool FINAL, bool OT4, int TY, int TZ, int RB, int PF>
__global__ void __launch_bounds__(TY* TZ) fdtd3d_pass(const __grid_constant__ Step3D a) {
    using L = Smem3D<KIND, TY, TZ, RB, PF>;
    constexpr int NT = TY * TZ;
    constexpr bool STAG = L::STAG, VARB = KIND == 1;
    constexpr int R = L::R, QU = L::QU, PY = L::PY, PZ = L::PZ, WZF = L::WZF;
    constexpr int QB = STAG ? 9 : 10;
    constexpr int QL = QB + RB;

    extern __shared__ __align__(16) float smem[];
    float* const sU = smem + L::oU;
    float* const sFY = smem + L::oFY;
    float* const sFZ = smem + L::oFZ;

    const int tid = threadIdx.x;
    const int tz = tid % TZ, ty = tid / TZ;
    const int shot = blockIdx.x % a.nshots, tile = blockIdx.x / a.nshots;
    const int tile_y = tile % a.ty0n, tile_z = tile / a.ty0n;
    const int chunk = blockIdx.y;
    const int y0 = tile_y * TY, z0 = tile_z * TZ;
    const int y = y0 + ty, z = z0 + tz;
    const bool col_in = y < a.ny && z < a.nz;
    const int yc = min(y, a.ny - 1), zc = min(z, a.nz - 1);
    const int Z0 = (z0 - R) & ~3;  // plane rows start at floor4(z0 - R)
    const int xo0 = chunk * a.chunk_rows, xo1 = min(a.nx, xo0 + a.chunk_rows);
    const int i0 = xo0 - R, i1 = xo1 + R;
    const long long plane = (long long)a.ny * a.zp;
    const long long soff = (long long)shot * a.shot_stride;
    const long long col = (long long)yc * a.zp + zc;  // offset of this column in a plane
    const float ihx = 1.f / a.hx, ihy = 1.f / a.hy, ihz = 1.f / a.hz;
    const float ihx2 = ihx * ihx, ihy2 = ihy * ihy, ihz2 = ihz * ihz;
    const float dt2 = a.dt * a.dt;
    const float k12 = (float)((double)a.dt * (double)a.dt / 12.0);

    // plane ring: x row r in slot (r - i0) mod QU, kept as a running slot index (sI: row i);
    // element (yy, zz) at [(yy-y0+R)*PZ + zz - Z0]
    auto wrap = [](int s) { return s < 0 ? s + QU : (s >= QU ? s - QU : s); };
    auto slotp = [&](int s) { return sU + s * L::PLANE; };
    constexpr int NQ = PY * (PZ / 4);
    auto prefetch = [&](int ii, int si) {  // rows ii, ii+1, ... into slots si, si+1, ...
#pragma unroll
        for (int rr = 0; rr < RB; rr++) {
            const int r = ii + rr;
            if (r < i1) {
                float* dst = slotp(wrap(si + rr));
                const bool row_ok = r >= 0 && r < a.nx;
                for (int k = tid; k < NQ; k += NT) {
                    const int py = k / (PZ / 4), q = Z0 + 4 * (k % (PZ / 4));
                    const int yy = y0 - R + py;
                    const bool ok = row_ok && yy >= 0 && yy < a.ny && q >= 0 && q + 4 <= a.zp;
                    const float* g = ok ? a.in + soff + (long long)r * plane + (long long)yy * a.zp + q : a.in;
                    cp_async16(dst + py * PZ + 4 * (k % (PZ / 4)), g, ok);
                }
            }
        }
        cp_async_commit();
    };
    const int me = (ty + R) * PZ + (z - Z0);  // this column's index in a plane

    float uq[QL], fq[STAG ? QL : 1];
#pragma unroll
    for (int k = 0; k < QL; k++) {
        uq[k] = 0.f;
        if constexpr (STAG) fq[k] = 0.f;
    }
    const bool do_save = FINAL && a.save && (a.t % a.f == 0);

#pragma unroll 1
    for (int k = 0; k < PF; k++) prefetch(i0 + k * RB, k * RB);

    int sI = 0;  // ring slot of row i
#pragma unroll 1
    for (int i = i0; i < i1; i += RB) {
        const int j = i - R;  // output row of this iteration's first input row
        constexpr int KY = ((TY + 9) * TZ + NT - 1) / NT, KZ = (TY * WZF + NT - 1) / NT;
        float Wj[RB], bxi[RB], byv[RB][VARB ? KY : 1], bzv[RB][VARB ? KZ : 1];
        float c1v[RB], c2v[RB], c3v[RB], uov[RB], pmv[RB];
#pragma unroll
        for (int r = 0; r < RB; r++) {
            Wj[r] = __ldg(a.W + (long long)(j + r) * plane + col);
            if constexpr (VARB) {
                bxi[r] = __ldg(a.bxh + (long long)(i - 5 + r) * plane + col);
                const int xx = min(max(j + r, -sa::GUARD), a.nx + sa::GUARD - 1);
#pragma unroll
                for (int q = 0; q < KY; q++) {
                    const int k = tid + q * NT;
                    const int ky = min(k / TZ, TY + 8), kz = k % TZ;
                    const int zz = min(z0 + kz, a.nz - 1), yy = min(max(y0 - 5 + ky + 6, 0), a.ny + 9);
                    byv[r][q] = __ldg(a.byh + (long long)xx * (a.ny + 12) * a.zp + (long long)yy * a.zp + zz);
                }
#pragma unroll
                for (int q = 0; q < KZ; q++) {
                    const int k = tid + q * NT;
                    const int ky = min(k / WZF, TY - 1), kz = k % WZF;
                    const int yy = min(y0 + ky, a.ny - 1), zz = min(max(z0 - 5 + kz + 6, 0), a.zpb - 1);
                    bzv[r][q] = __ldg(a.bzh + (long long)xx * a.ny * a.zpb + (long long)yy * a.zpb + zz);
                }
            }
            if constexpr (FINAL) {
                const int row = j + r;
                const bool ok = row >= xo0 && row < xo1 && col_in;
                const long long idx = (long long)row * plane + (long long)y * a.zp + z;
                c1v[r] = ok ? __ldg(a.C1 + idx) : 0.f;
                c2v[r] = ok ? __ldg(a.C2 + idx) : 0.f;
                c3v[r] = ok ? __ldg(a.C3 + idx) : 0.f;
                uov[r] = ok ? a.cur[soff + idx] : 0.f;
                pmv[r] = ok ? a.prev[soff + idx] : 0.f;
            }
        }
        (void)byv; (void)bzv; (void)c1v; (void)c2v; (void)c3v; (void)uov; (void)pmv;
        cp_async_wait<PF - 1>();
        __syncthreads();
        prefetch(i + PF * RB, sI + PF * RB);
        // y/z fluxes of rows j..j+RB-1 (staggered): F_y at half-rows y0-5+k, F_z at z0-5+k
        if constexpr (STAG) {
#pragma unroll
            for (int r = 0; r < RB; r++) {
                const float* pl = slotp(wrap(sI - R + r));
#pragma unroll
                for (int q = 0; q < KY; q++) {
                    const int k = tid + q * NT;
                    if (k < (TY + 9) * TZ) {
                        const int ky = k / TZ, kz = k % TZ;
                        const int hy = y0 - 5 + ky;  // half row hy + 1/2
                        const int base = (hy - y0 + R) * PZ + (z0 + kz - Z0);
                        float v = dstag_1(pl, base + PZ, base, PZ) * ihy;
                        if constexpr (VARB) v *= byv[r][q];
                        sFY[r * ((TY + 9) * TZ) + k] = v;
                    }
                }
#pragma unroll
                for (int q = 0; q < KZ; q++) {
                    const int k = tid + q * NT;
                    const int ky = k / WZF, kz = k % WZF;
                    if (ky < TY && kz < TZ + 9) {
                        const int hz = z0 - 5 + kz;  // half column hz + 1/2
                        const int base = (ky + R) * PZ + (hz - Z0);
                        float v = dstag_1(pl, base + 1, base, 1) * ihz;
                        if constexpr (VARB) v *= bzv[r][q];
                        sFZ[r * L::FZ + k] = v;
                    }
                }
            }
            __syncthreads();
        }
#pragma unroll
        for (int r = 0; r < RB; r++) uq[QB + r] = slotp(wrap(sI + r))[me];
        float res[RB];
#pragma unroll
        for (int r = 0; r < RB; r++) {
            float gx, gyz;
            if constexpr (STAG) {
                float v = dstag_1(uq, r + 5, r + 4, 1) * ihx;
                if constexpr (VARB) v *= bxi[r];
                fq[QB + r] = v;
                gx = dstag_1(fq, r + 5, r + 4, 1) * ihx;
                const float* Fy = sFY + r * ((TY + 9) * TZ);
                const float* Fz = sFZ + r * L::FZ;
                // D- along y at row ty: fluxes at half rows ty-5 .. ty+4 (index ky = half - y0 + 5)
                const float gy = dstag_1(Fy, (ty + 5) * TZ + tz, (ty + 4) * TZ + tz, TZ) * ihy;
                const float gz = dstag_1(Fz, ty * WZF + tz + 5, ty * WZF + tz + 4, 1) * ihz;
                gyz = gy + gz;
            } else {
                gx = dcent_1(uq, r + 5, 1) * ihx2;
                const float* pl = slotp(wrap(sI - R + r));
                gyz = dcent_1(pl, me, PZ) * ihy2 + dcent_1(pl, me, 1) * ihz2;
            }
            const float g = gx + gyz;
            if constexpr (!FINAL) {
                res[r] = Wj[r] * g;
            } else if constexpr (OT4) {
                // Lt = l + dt^2/12 W G(l): the streamed l at row j+r is queue entry r (STAG,
                // rows i-9..) or r+5 (laplace, rows i-10..)
                res[r] = fmaf(k12, Wj[r] * g, STAG ? uq[r] : uq[r + 5]);
            } else {
                res[r] = Wj[r] * g;
            }
        }
        qshift1<QL, RB>(uq);
        if constexpr (STAG) qshift1<QL, RB>(fq);
#pragma unroll
        for (int r = 0; r < RB; r++) {
            const int row = j + r;
            if (row < xo0 || row >= xo1 || !col_in) continue;
            const long long idx = (long long)row * plane + (long long)y * a.zp + z;
            if constexpr (!FINAL) {
                a.out_l[soff + idx] = res[r];
            } else {
                const float u_o = uov[r];
                const float pm = pmv[r];
                const float pn = c1v[r] * res[r] + c2v[r] * u_o - c3v[r] * pm;
                if (do_save) {
                    a.snaps[(long long)shot * a.snap_shot_stride + (long long)(a.t / a.f) * a.snap_stride + idx] =
                        a.save == 2 ? u_o : (pn - 2.f * u_o + pm) / dt2;  // 2: raw p[t] (rho gradient)
                }
                a.prev[soff + idx] = pn;
            }
        }
        sI = sI + RB >= QU ? sI + RB - QU : sI + RB;
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

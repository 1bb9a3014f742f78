#include <algorithm>
// Device helpers of 3D plans: medium preparation, sparse injection / interpolation and the
// reduction of per-shot gradients. Layout [x][y][zp], z contiguous.
#include "fdtd3d.cuh"
#include "helpers.h"

namespace sa {

// W = vp^2 (or vp^2 rho), buoyancy 1/rho, vp and alpha (Np/m) scratch
// (iso_acoustic/devito.py:476-497). Inputs unpadded [nx][ny][nz].
__global__ void k_medium3d(const float* __restrict__ vp_in, const float* __restrict__ rho_in,
                           const float* __restrict__ alpha_in, int nx, int ny, int nz, int zp, int density,
                           double db_to_np, float* W, float* vp, float* alpha, float* buoy) {
    const long long n = (long long)nx * ny * nz;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const long long xy = q / nz;
        const int z = (int)(q % nz);
        const long long p = xy * zp + z;
        const float v = vp_in[q];
        vp[p] = v;
        float w = v * v;
        if (density >= 1) {  // 1: variable density (W = vp^2 rho), 2: constant (b kept for the rho gradient)
            const float r = rho_in[q];
            if (density == 1) w = w * r;
            buoy[p] = 1.f / r;
        }
        W[p] = w;
        alpha[p] = alpha_in ? (float)((double)alpha_in[q] * db_to_np) : 0.f;
    }
}

// Buoyancy at half points along x, y and z (arithmetic mean of the two nodes, edge values
// beyond the grid): bxh half-planes x = -5..nx+3 (pointer at x = 0, plane ny*zp);
// byh[x][y+6][z] (row length zp, ny+12 rows per plane); bzh[x][y][z+6] (pitch zpb).
__global__ void k_bhalf3d(const float* __restrict__ b, int nx, int ny, int nz, int zp, int zpb, float* bxh,
                          float* byh, float* bzh) {
    const long long nxa = (long long)(nx + 9) * ny * nz;
    const long long nya = (long long)nx * (ny + 10) * nz;
    const long long nza = (long long)nx * ny * (nz + 10);
    const long long plane = (long long)ny * zp;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nxa + nya + nza;
         q += (long long)gridDim.x * blockDim.x) {
        if (q < nxa) {
            const int z = (int)(q % nz), y = (int)((q / nz) % ny), x = (int)(q / ((long long)nz * ny)) - 5;
            const int x0 = min(max(x, 0), nx - 1), x1 = min(max(x + 1, 0), nx - 1);
            bxh[(long long)x * plane + (long long)y * zp + z] =
                0.5f * (b[x0 * plane + (long long)y * zp + z] + b[x1 * plane + (long long)y * zp + z]);
        } else if (q < nxa + nya) {
            const long long r = q - nxa;
            const int z = (int)(r % nz), yr = (int)((r / nz) % (ny + 10)), x = (int)(r / ((long long)nz * (ny + 10)));
            const int y = yr - 6;
            const int y0 = min(max(y, 0), ny - 1), y1 = min(max(y + 1, 0), ny - 1);
            byh[(long long)x * (ny + 12) * zp + (long long)yr * zp + z] =
                0.5f * (b[x * plane + (long long)y0 * zp + z] + b[x * plane + (long long)y1 * zp + z]);
        } else {
            const long long r = q - nxa - nya;
            const int zr = (int)(r % (nz + 10)), y = (int)((r / (nz + 10)) % ny), x = (int)(r / ((long long)(nz + 10) * ny));
            const int z = zr - 6;
            const int z0 = min(max(z, 0), nz - 1), z1 = min(max(z + 1, 0), nz - 1);
            bzh[(long long)x * ny * zpb + (long long)y * zpb + zr] =
                0.5f * (b[x * plane + (long long)y * zp + z0] + b[x * plane + (long long)y * zp + z1]);
        }
    }
}

// Update coefficients (iso_acoustic/devito.py:1575-1581) with the SpongeBoundary2 damping; the
// slab of axis a at layer e covers the points whose layers on the other axes are >= e
// (boundaries/boundary.py:116-160).
__global__ void k_coef3d(const float* __restrict__ vp, const float* __restrict__ alpha, int nx, int ny, int nz, int zp,
                         Sponge3 sp, float dt, float* C1, float* C2, float* C3) {
    const long long n = (long long)nx * ny * nz;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int z = (int)(q % nz), y = (int)((q / nz) % ny), x = (int)(q / ((long long)nz * ny));
        const long long p = ((long long)x * ny + y) * zp + z;
        const int e[3] = {min(x, nx - 1 - x), min(y, ny - 1 - y), min(z, nz - 1 - z)};
        float s = 0.f;
        for (int a = 0; a < 3; a++) {
            bool ok = e[a] < sp.a[a];
            for (int b2 = 0; b2 < 3; b2++)
                if (b2 != a && e[b2] < e[a]) ok = false;
            if (ok) s += sp.s[a][e[a]];
        }
        const float v = vp[p], v2 = v * v;
        const float d = 7.f * (s * v) * dt;
        float beta = v2 * d;
        beta = beta + alpha[p] * v;
        beta = dt * beta;
        const float den = 1.f + beta;
        C1[p] = (dt * dt) / den;
        C2[p] = (2.f - dt * dt * v2 * d * d) / den;
        C3[p] = (1.f - beta) / den;
    }
}

__global__ void inject3d(const Sparse3D s, int n, const float* amp, int ld, int t, float* field, long long shot_stride,
                         int ny, int zp, float* snap, long long snap_shot_stride, long long snap_off, float inv_dt2) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= 8 * n) return;
    const int pnt = k >> 3, c = k & 7;
    const int* b = s.base + 3 * pnt;
    const int x = b[0] + ((c >> 2) & 1), y = b[1] + ((c >> 1) & 1), z = b[2] + (c & 1);
    const long long idx = ((long long)x * ny + y) * zp + z;
    const float v = s.coef[8 * pnt + c] * amp[(long long)t * ld + pnt];
    const int sh = s.shot[pnt];
    atomicAdd(field + (long long)sh * shot_stride + idx, v);
    if (snap) atomicAdd(snap + (long long)sh * snap_shot_stride + snap_off + idx, v * inv_dt2);
}

__global__ void gather3d(const Sparse3D s, int n, const float* field, long long shot_stride, int ny, int zp, float* out,
                         int ld, int trow, float scale) {
    const int pnt = blockIdx.x * blockDim.x + threadIdx.x;
    if (pnt >= n) return;
    const int* b = s.base + 3 * pnt;
    const float* f = field + (long long)s.shot[pnt] * shot_stride;
    float acc = 0.f;
    for (int c = 0; c < 8; c++) {
        const int x = b[0] + ((c >> 2) & 1), y = b[1] + ((c >> 1) & 1), z = b[2] + (c & 1);
        acc += s.w[8 * pnt + c] * f[((long long)x * ny + y) * zp + z];
    }
    out[(long long)trow * ld + pnt] = scale * acc;
}

__global__ void k_reduce3d(const float* __restrict__ buf, long long shot_stride, int nshots, int nx, int ny, int nz,
                           int zp, float* __restrict__ out) {
    const long long n = (long long)nx * ny * nz;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const long long p = (q / nz) * zp + q % nz;
        float acc = 0.f;
        for (int b2 = 0; b2 < nshots; b2++) acc += buf[(long long)b2 * shot_stride + p];
        out[q] = acc;
    }
}

cudaError_t medium3d(const float* vp_in, const float* rho_in, const float* alpha_in, int nx, int ny, int nz, int zp,
                     int zpb, int density, double db_to_np, const Sponge3& sp, float dt, float* W, float* vp,
                     float* alpha, float* buoy, float* bxh, float* byh, float* bzh, float* C1, float* C2, float* C3,
                     cudaStream_t s) {
    k_medium3d<<<2048, 256, 0, s>>>(vp_in, rho_in, alpha_in, nx, ny, nz, zp, density, db_to_np, W, vp, alpha, buoy);
    if (density == 1) k_bhalf3d<<<2048, 256, 0, s>>>(buoy, nx, ny, nz, zp, zpb, bxh, byh, bzh);
    k_coef3d<<<2048, 256, 0, s>>>(vp, alpha, nx, ny, nz, zp, sp, dt, C1, C2, C3);
    return cudaGetLastError();
}

cudaError_t sparse3d_inject(const Sparse3D& sp, int n, const float* amp, int ld, int t, float* field,
                            long long shot_stride, int ny, int zp, float* snap, long long snap_shot_stride,
                            long long snap_off, float inv_dt2, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    inject3d<<<(8 * n + 127) / 128, 128, 0, s>>>(sp, n, amp, ld, t, field, shot_stride, ny, zp, snap, snap_shot_stride,
                                                 snap_off, inv_dt2);
    return cudaGetLastError();
}

cudaError_t sparse3d_gather(const Sparse3D& sp, int n, const float* field, long long shot_stride, int ny, int zp,
                            float* out, int ld, int trow, cudaStream_t s, float scale) {
    if (n == 0) return cudaSuccess;
    gather3d<<<(n + 127) / 128, 128, 0, s>>>(sp, n, field, shot_stride, ny, zp, out, ld, trow, scale);
    return cudaGetLastError();
}

// Imaging condition of one adjoint level (t % f == 0), interior only, per shot:
// grad += snap q, prec += snap^2, q = p_a[t].
__global__ void k_image3d(const float* __restrict__ q, const float* __restrict__ snap, float* gradb, float* precb,
                          int ix0, int ix1, int iy0, int iy1, int iz0, int iz1, int ny, int zp, int nshots,
                          long long field, long long snap_shot_stride) {
    const int wz = iz1 - iz0, wy = iy1 - iy0;
    const long long per = (long long)(ix1 - ix0) * wy * wz;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < per * nshots;
         e += (long long)gridDim.x * blockDim.x) {
        const int shot = (int)(e / per);
        long long r = e - (long long)shot * per;
        const int z = iz0 + (int)(r % wz);
        r /= wz;
        const int y = iy0 + (int)(r % wy);
        const int x = ix0 + (int)(r / wy);
        const long long idx = ((long long)x * ny + y) * zp + z;
        const float sv = snap[(long long)shot * snap_shot_stride + idx];
        const long long gi = (long long)shot * field + idx;
        gradb[gi] += sv * q[gi];
        precb[gi] += sv * sv;
    }
}

cudaError_t image3d(const float* q, const float* snap, float* gradb, float* precb, const int* lo, const int* hi,
                    int ny, int zp, int nshots, long long field, long long snap_shot_stride, cudaStream_t s) {
    const long long n = (long long)(hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2]) * nshots;
    if (n <= 0) return cudaSuccess;
    const int blocks = (int)std::min<long long>((n + 255) / 256, 152 * 16);
    k_image3d<<<blocks, 256, 0, s>>>(q, snap, gradb, precb, lo[0], hi[0], lo[1], hi[1], lo[2], hi[2], ny, zp, nshots,
                                     field, snap_shot_stride);
    return cudaGetLastError();
}

// D-_x b, D-_y b, D-_z b at every node (staggered first derivatives at i-1/2 of the edge-padded
// buoyancy), the grad(buoy, shift=-0.5) factor of the rho imaging term (iso_acoustic/devito.py:1137).
__global__ void k_rho_terms3d(const float* __restrict__ b, int nx, int ny, int nz, int zp, float ihx, float ihy,
                              float ihz, float* dbx, float* dby, float* dbz) {
    const long long n = (long long)nx * ny * nz;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int z = (int)(q % nz);
        const int y = (int)((q / nz) % ny);
        const int x = (int)(q / ((long long)nz * ny));
        auto at = [&](int xx, int yy, int zz) { return b[((long long)xx * ny + yy) * zp + zz]; };
        float ax = 0.f, ay = 0.f, az = 0.f;
#pragma unroll
        for (int m = 0; m < 5; m++) {
            ax += kWS(m) * (at(min(x + m, nx - 1), y, z) - at(max(x - 1 - m, 0), y, z));
            ay += kWS(m) * (at(x, min(y + m, ny - 1), z) - at(x, max(y - 1 - m, 0), z));
            az += kWS(m) * (at(x, y, min(z + m, nz - 1)) - at(x, y, max(z - 1 - m, 0)));
        }
        const long long i = ((long long)x * ny + y) * zp + z;
        dbx[i] = ax * ihx;
        dby[i] = ay * ihy;
        dbz[i] = az * ihz;
    }
}

cudaError_t rho_terms3d(const float* b, int nx, int ny, int nz, int zp, const double* h, float* dbx, float* dby,
                        float* dbz, cudaStream_t s) {
    k_rho_terms3d<<<2048, 256, 0, s>>>(b, nx, ny, nz, zp, (float)(1.0 / h[0]), (float)(1.0 / h[1]),
                                       (float)(1.0 / h[2]), dbx, dby, dbz);
    return cudaGetLastError();
}

// Imaging from the raw saved wavefield s[n] = p[n f] in 3D (the 2D k_image_raw2d per shot): on a
// refresh step the held vp term (s[n+1] - 2 s[n] + s[n-1]) inv_fdt2 and, with hold_rho, the rho
// term -(grad(b, -1/2) . grad(s[n], -1/2)) - b laplace(s[n]) (zero halo for s) are recomputed at
// every interior point; every step accumulates grad += held q, prec += held^2.
// snap addresses slot n of shot 0.
__global__ void k_image_raw3d(const float* __restrict__ q, const float* __restrict__ snap, long long snap_stride,
                              long long snap_shot_stride, int refresh, float inv_fdt2, float* hold_vp,
                              float* hold_rho, const float* __restrict__ buoy, const float* __restrict__ dbx,
                              const float* __restrict__ dby, const float* __restrict__ dbz, float ihx, float ihy,
                              float ihz, int nx, int ny, int nz, int zp, float* gradb, float* precb, float* gradrb,
                              float* precrb, int ix0, int ix1, int iy0, int iy1, int iz0, int iz1, int nshots,
                              long long field) {
    const int wz = iz1 - iz0, wy = iy1 - iy0;
    const long long per = (long long)(ix1 - ix0) * wy * wz;
    const long long sx = (long long)ny * zp, sy = zp;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < per * nshots;
         e += (long long)gridDim.x * blockDim.x) {
        const int shot = (int)(e / per);
        long long r = e - (long long)shot * per;
        const int z = iz0 + (int)(r % wz);
        r /= wz;
        const int y = iy0 + (int)(r % wy);
        const int x = ix0 + (int)(r / wy);
        const long long idx = ((long long)x * ny + y) * zp + z;
        const long long gi = (long long)shot * field + idx;
        float hv, hr = 0.f;
        if (refresh) {
            const float* sp = snap + (long long)shot * snap_shot_stride;
            const float s0 = sp[idx];
            hv = ((sp[idx + snap_stride] - 2.f * s0) + sp[idx - snap_stride]) * inv_fdt2;
            hold_vp[gi] = hv;
            if (hold_rho) {
                float g[3] = {0.f, 0.f, 0.f}, l[3] = {kW2(0) * s0, kW2(0) * s0, kW2(0) * s0};
                const int pos[3] = {x, y, z}, n[3] = {nx, ny, nz};
                const long long st[3] = {sx, sy, 1};
#pragma unroll
                for (int d = 0; d < 3; d++) {
#pragma unroll
                    for (int m = 0; m < 5; m++) {
                        const float hi = pos[d] + m < n[d] ? sp[idx + m * st[d]] : 0.f;
                        const float lo = pos[d] - 1 - m >= 0 ? sp[idx - (m + 1) * st[d]] : 0.f;
                        g[d] += kWS(m) * (hi - lo);
                        const int k = m + 1;
                        const float fp = pos[d] + k < n[d] ? sp[idx + k * st[d]] : 0.f;
                        const float fm = pos[d] - k >= 0 ? sp[idx - k * st[d]] : 0.f;
                        l[d] += kW2(k) * (fp + fm);
                    }
                }
                hr = -(dbx[idx] * (g[0] * ihx) + dby[idx] * (g[1] * ihy) + dbz[idx] * (g[2] * ihz)) -
                     buoy[idx] * (l[0] * (ihx * ihx) + l[1] * (ihy * ihy) + l[2] * (ihz * ihz));
                hold_rho[gi] = hr;
            }
        } else {
            hv = hold_vp[gi];
            if (hold_rho) hr = hold_rho[gi];
        }
        const float u = q[gi];
        gradb[gi] += hv * u;
        precb[gi] += hv * hv;
        if (hold_rho) {
            gradrb[gi] += hr * u;
            precrb[gi] += hr * hr;
        }
    }
}

cudaError_t image_raw3d(const float* q, const float* snap, long long snap_stride, long long snap_shot_stride,
                        int refresh, float inv_fdt2, float* hold_vp, float* hold_rho, const float* buoy,
                        const float* dbx, const float* dby, const float* dbz, const double* h, int nx, int ny, int nz,
                        int zp, float* gradb, float* precb, float* gradrb, float* precrb, const int* lo,
                        const int* hi, int nshots, long long field, cudaStream_t s) {
    const long long n = (long long)(hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2]) * nshots;
    if (n <= 0) return cudaSuccess;
    const int blocks = (int)std::min<long long>((n + 255) / 256, 152 * 16);
    k_image_raw3d<<<blocks, 256, 0, s>>>(q, snap, snap_stride, snap_shot_stride, refresh, inv_fdt2, hold_vp, hold_rho,
                                         buoy, dbx, dby, dbz, (float)(1.0 / h[0]), (float)(1.0 / h[1]),
                                         (float)(1.0 / h[2]), nx, ny, nz, zp, gradb, precb, gradrb, precrb, lo[0],
                                         hi[0], lo[1], hi[1], lo[2], hi[2], nshots, field);
    return cudaGetLastError();
}

// Exact-gradient helpers of 3D plans (SA_GRAD_EXACT), the 3D counterparts of exact2d.cu: the
// per-point coefficients of the vp derivative of the update (with the damping and coefficients
// exactly as k_coef3d forms them), the per-step accumulation and the source term.
__global__ void k_exact_coef3d(const float* __restrict__ vp, const float* __restrict__ alpha,
                               const float* __restrict__ W, int nx, int ny, int nz, int zp, Sponge3 sp, float dt,
                               float* EA, float* EB, float* EC, float* EG4, float* ES) {
    const long long n = (long long)nx * ny * nz;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int z = (int)(q % nz), y = (int)((q / nz) % ny), x = (int)(q / ((long long)nz * ny));
        const long long p = ((long long)x * ny + y) * zp + z;
        const int e[3] = {min(x, nx - 1 - x), min(y, ny - 1 - y), min(z, nz - 1 - z)};
        float s = 0.f;
        for (int a = 0; a < 3; a++) {
            bool ok = e[a] < sp.a[a];
            for (int b2 = 0; b2 < 3; b2++)
                if (b2 != a && e[b2] < e[a]) ok = false;
            if (ok) s += sp.s[a][e[a]];
        }
        const float v = vp[p], v2 = v * v;
        const float d = 7.f * (s * v) * dt;
        float beta = v2 * d;
        beta = beta + alpha[p] * v;
        beta = dt * beta;
        const float den = 1.f + beta;
        const float C1 = (dt * dt) / den;
        const float C2 = (2.f - dt * dt * v2 * d * d) / den;
        const float C3 = (1.f - beta) / den;
        const double Dt = dt, V = v, Dd = d, Q = 1.0 + (double)beta;
        const double dbeta = Dt * (3.0 * V * Dd + (double)alpha[p]);
        const double dC1 = -Dt * Dt * dbeta / (Q * Q);
        const double dC2 = (-Dt * Dt * 4.0 * V * Dd * Dd * Q - (2.0 - Dt * Dt * V * V * Dd * Dd) * dbeta) / (Q * Q);
        const double dC3 = -2.0 * dbeta / (Q * Q);
        const double w = W[p], c1 = C1, c1w = c1 * w;
        const double G1 = (dC1 + 2.0 * c1 / V) / (c1 * c1w);
        EA[p] = (float)G1;
        EB[p] = (float)(-G1 * (double)C2 + dC2 / c1w);
        EC[p] = (float)(G1 * (double)C3 - dC3 / c1w);
        EG4[p] = (float)(Dt * Dt / (6.0 * V * w));
        ES[p] = (float)(1.0 / c1w - G1 * V);
    }
}

// grad[shot] += z (a u0 + b u1 + c u2) [+ g4 Lu Lz]; prec[shot] += ((u0 - 2 u1 + u2) / dt^2)^2
__global__ void k_exact_grad3d(const float* __restrict__ z, const float* __restrict__ u0,
                               const float* __restrict__ u1, const float* __restrict__ u2,
                               const float* __restrict__ Lu, const float* __restrict__ Lz,
                               const float* __restrict__ EA, const float* __restrict__ EB,
                               const float* __restrict__ EC, const float* __restrict__ EG4, int nx, int ny, int nz,
                               int zp, int nshots, long long field, float inv_dt2, float* gradb, float* precb) {
    const long long n = (long long)nx * ny * nz;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n * nshots;
         q += (long long)gridDim.x * blockDim.x) {
        const int shot = (int)(q / n);
        const long long r = q - (long long)shot * n;
        const int zz = (int)(r % nz), y = (int)((r / nz) % ny), x = (int)(r / ((long long)nz * ny));
        const long long p = ((long long)x * ny + y) * zp + zz;
        const long long i = (long long)shot * field + p;
        const float a0 = u0[i], a1 = u1[i], a2 = u2[i];
        float g = z[i] * (EA[p] * a0 + EB[p] * a1 + EC[p] * a2);
        if (Lu) g += EG4[p] * (Lu[i] * Lz[i]);
        const float dd = (a0 - 2.f * a1 + a2) * inv_dt2;
        gradb[i] += g;
        precb[i] += dd * dd;
    }
}

// Source term at the 8 corners of each source point: z w src[trow] scale ES.
__global__ void k_exact_src3d(const float* __restrict__ z, const Sparse3D s, int n, const float* __restrict__ amp,
                              int ld, int trow, float scale, const float* __restrict__ ES, int ny, int zp,
                              long long field, float* gradb) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= 8 * n) return;
    const int pnt = k >> 3, c = k & 7;
    const int* b = s.base + 3 * pnt;
    const int x = b[0] + ((c >> 2) & 1), y = b[1] + ((c >> 1) & 1), zz = b[2] + (c & 1);
    const long long p = ((long long)x * ny + y) * zp + zz;
    const long long i = (long long)s.shot[pnt] * field + p;
    atomicAdd(gradb + i, z[i] * s.w[8 * pnt + c] * amp[(long long)trow * ld + pnt] * scale * ES[p]);
}

cudaError_t exact_coef3d(const float* vp, const float* alpha, const float* W, int nx, int ny, int nz, int zp,
                         const Sponge3& sp, float dt, float* EA, float* EB, float* EC, float* EG4, float* ES,
                         cudaStream_t s) {
    k_exact_coef3d<<<2048, 256, 0, s>>>(vp, alpha, W, nx, ny, nz, zp, sp, dt, EA, EB, EC, EG4, ES);
    return cudaGetLastError();
}

cudaError_t exact_grad3d(const float* z, const float* u0, const float* u1, const float* u2, const float* Lu,
                         const float* Lz, const float* EA, const float* EB, const float* EC, const float* EG4, int nx,
                         int ny, int nz, int zp, int nshots, long long field, float inv_dt2, float* gradb,
                         float* precb, cudaStream_t s) {
    const long long n = (long long)nx * ny * nz * nshots;
    const int blocks = (int)std::min<long long>((n + 255) / 256, 152 * 16);
    k_exact_grad3d<<<blocks, 256, 0, s>>>(z, u0, u1, u2, Lu, Lz, EA, EB, EC, EG4, nx, ny, nz, zp, nshots, field,
                                          inv_dt2, gradb, precb);
    return cudaGetLastError();
}

cudaError_t exact_src3d(const float* z, const Sparse3D& sp, int n, const float* amp, int ld, int trow, float scale,
                        const float* ES, int ny, int zp, long long field, float* gradb, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_exact_src3d<<<(8 * n + 127) / 128, 128, 0, s>>>(z, sp, n, amp, ld, trow, scale, ES, ny, zp, field, gradb);
    return cudaGetLastError();
}

// Receiver injection coefficients of the exact adjoint: w C1 W at each corner.
__global__ void k_xcoef3d(const Sparse3D s, int n, const float* __restrict__ C1, const float* __restrict__ W, int ny,
                          int zp, float* out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= 8 * n) return;
    const int pnt = k >> 3, c = k & 7;
    const int* b = s.base + 3 * pnt;
    const int x = b[0] + ((c >> 2) & 1), y = b[1] + ((c >> 1) & 1), z = b[2] + (c & 1);
    const long long p = ((long long)x * ny + y) * zp + z;
    out[k] = s.w[k] * (C1[p] * W[p]);
}

cudaError_t xcoef3d(const Sparse3D& sp, int n, const float* C1, const float* W, int ny, int zp, float* out,
                    cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_xcoef3d<<<(8 * n + 127) / 128, 128, 0, s>>>(sp, n, C1, W, ny, zp, out);
    return cudaGetLastError();
}

// Wide-support (Hicks, sinc) injection: field[shot][idx[e]] += coef[e] amp[t][point[e]] (and its snapshot / dt^2).
__global__ void k_inject_entries3d(const Entries3D e, int n, const float* __restrict__ amp, int ld, int t, float* field,
                                   long long shot_stride, float* snap, long long snap_shot_stride, long long snap_off,
                                   float inv_dt2) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float v = e.coef[k] * amp[(long long)t * ld + e.point[k]];
    const int sh = e.shot[k];
    atomicAdd(field + (long long)sh * shot_stride + e.idx[k], v);
    if (snap) atomicAdd(snap + (long long)sh * snap_shot_stride + snap_off + e.idx[k], v * inv_dt2);
}

// Wide-support gather: out[trow][point] = scale * sum over the width^3 support of wx wy wz field.
__global__ void k_support_gather3d(const SupportGather3D* __restrict__ g, int n, const float* __restrict__ field,
                                   long long shot_stride, int ny, int zp, float* out, int ld, int trow, float scale) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const SupportGather3D& G = g[k];
    const float* f = field + (long long)G.shot * shot_stride;
    float v = 0.f;
    for (int a = 0; a < G.width; a++) {
        float va = 0.f;
        for (int b = 0; b < G.width; b++) {
            const float* row = f + ((long long)(G.x + a) * ny + (G.y + b)) * zp + G.z;
            float vb = 0.f;
            for (int c = 0; c < G.width; c++) vb += G.wz[c] * row[c];
            va += G.wy[b] * vb;
        }
        v += G.wx[a] * va;
    }
    out[(long long)trow * ld + G.point] = scale * v;
}

cudaError_t inject_entries3d(const Entries3D& e, int n, const float* amp, int ld, int t, float* field,
                             long long shot_stride, float* snap, long long snap_shot_stride, long long snap_off,
                             float inv_dt2, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_inject_entries3d<<<(n + 255) / 256, 256, 0, s>>>(e, n, amp, ld, t, field, shot_stride, snap, snap_shot_stride,
                                                       snap_off, inv_dt2);
    return cudaGetLastError();
}

cudaError_t support_gather3d(const SupportGather3D* g, int n, const float* field, long long shot_stride, int ny, int zp,
                           float* out, int ld, int trow, float scale, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_support_gather3d<<<(n + 127) / 128, 128, 0, s>>>(g, n, field, shot_stride, ny, zp, out, ld, trow, scale);
    return cudaGetLastError();
}

// CFS-PML after a 3D OT2 step (the 3D form of k_pml2d): at every point of the absorbing frame, for
// each axis whose slab holds it, the auxiliary fields u3, u2, u1 advance with the 10th-order
// derivatives of p[t] along that axis (adjoint: -f_d), and the new level takes -C1 vp^2 sum u1
// (its p.dt2 snapshot too on a save step). Interior points exit at once.
// prof: sigma, alpha, sigma', alpha' per axis (n_a each, axes in order); aux: 9 fields (u3, u2, u1
// of x, y, z), each nshots * field floats.
__global__ void k_pml3d(const float* __restrict__ cur, float* nxt, float* aux, const float* __restrict__ prof,
                        const float* __restrict__ C1, const float* __restrict__ vp, int nx, int ny, int nz, int zp,
                        int nshots, long long field, int ax, int ay, int az, float ihx, float ihy, float ihz, float dt,
                        int adjoint, float* snap, long long snap_shot_stride, float inv_dt2) {
    const long long n = (long long)nx * ny * nz;
    const long long fs = (long long)nshots * field;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n * nshots;
         q += (long long)gridDim.x * blockDim.x) {
        const int shot = (int)(q / n);
        const long long r = q - (long long)shot * n;
        const int z = (int)(r % nz), y = (int)((r / nz) % ny), x = (int)(r / ((long long)nz * ny));
        const int pos[3] = {x, y, z}, len[3] = {nx, ny, nz}, thick[3] = {ax, ay, az};
        bool any = false;
#pragma unroll
        for (int d = 0; d < 3; d++) any |= pos[d] < thick[d] || pos[d] >= len[d] - thick[d];
        if (!any) continue;
        const long long idx = ((long long)x * ny + y) * zp + z;
        const long long base = (long long)shot * field;
        const float* f = cur + base;
        const long long st[3] = {(long long)ny * zp, zp, 1};
        const float ihs[3] = {ihx, ihy, ihz};
        const int poff[3] = {0, 4 * nx, 4 * (nx + ny)};
        float B = 0.f;
#pragma unroll
        for (int d = 0; d < 3; d++) {
            const int i = pos[d], nn = len[d], a = thick[d];
            if (!(i < a || i >= nn - a)) continue;
            const float f0 = f[idx];
            float g = 0.f, l = kW2(0) * f0;
#pragma unroll
            for (int k = 1; k <= 5; k++) {
                const float fp = i + k < nn ? f[idx + k * st[d]] : 0.f;
                const float fm = i - k >= 0 ? f[idx - k * st[d]] : 0.f;
                g += kW1(k) * (fp - fm);
                l += kW2(k) * (fp + fm);
            }
            g *= adjoint ? -ihs[d] : ihs[d];
            l *= ihs[d] * ihs[d];
            const float* pr = prof + poff[d];
            const float s = pr[i], al = pr[nn + i], ds = pr[2 * nn + i], da = pr[3 * nn + i];
            float* u3 = aux + (3 * d) * fs + base + idx;
            float* u2 = aux + (3 * d + 1) * fs + base + idx;
            float* u1 = aux + (3 * d + 2) * fs + base + idx;
            const float as = al + s;
            const float v3 = *u3 - dt * (as * *u3 - s * s * (ds + da) * g);
            const float v2 = *u2 - dt * (as * *u2 - s * (2.f * ds * g + da * g + s * l) + v3);
            const float v1 = *u1 - dt * (as * *u1 - (ds * g + 2.f * s * l) + v2);
            *u3 = v3;
            *u2 = v2;
            *u1 = v1;
            B += v1;
        }
        const float v = vp[idx];
        const float k = C1[idx] * (v * v) * B;
        nxt[base + idx] -= k;
        if (snap) snap[(long long)shot * snap_shot_stride + idx] -= k * inv_dt2;
    }
}

cudaError_t pml3d(const float* cur, float* nxt, float* aux, const float* prof, const float* C1, const float* vp,
                  int nx, int ny, int nz, int zp, int nshots, long long field, const int* a, const double* h, float dt,
                  int adjoint, float* snap, long long snap_shot_stride, float inv_dt2, cudaStream_t s) {
    const long long n = (long long)nx * ny * nz * nshots;
    const int blocks = (int)std::min<long long>((n + 255) / 256, 152 * 16);
    k_pml3d<<<blocks, 256, 0, s>>>(cur, nxt, aux, prof, C1, vp, nx, ny, nz, zp, nshots, field, a[0], a[1], a[2],
                                   (float)(1.0 / h[0]), (float)(1.0 / h[1]), (float)(1.0 / h[2]), dt, adjoint, snap,
                                   snap_shot_stride, inv_dt2);
    return cudaGetLastError();
}

// Wide-support (Hicks, sinc) forms of the 3D exact gradient's point terms: receiver coefficients w C1 W at each
// support entry, and the source term z w src[trow] scale ES at each source support entry.
__global__ void k_xcoef_entries3d(const long long* __restrict__ idx, const float* __restrict__ w, int n,
                                  const float* __restrict__ C1, const float* __restrict__ W, float* out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = w[k] * (C1[idx[k]] * W[idx[k]]);
}

__global__ void k_exact_src_entries3d(const float* __restrict__ z, const Entries3D e, const float* __restrict__ w,
                                      int n, const float* __restrict__ amp, int ld, int trow, float scale,
                                      const float* __restrict__ ES, long long field, float* gradb) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const long long p = e.idx[k], i = (long long)e.shot[k] * field + p;
    atomicAdd(gradb + i, z[i] * w[k] * amp[(long long)trow * ld + e.point[k]] * scale * ES[p]);
}

cudaError_t xcoef_entries3d(const long long* idx, const float* w, int n, const float* C1, const float* W, float* out,
                            cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_xcoef_entries3d<<<(n + 255) / 256, 256, 0, s>>>(idx, w, n, C1, W, out);
    return cudaGetLastError();
}

cudaError_t exact_src_entries3d(const float* z, const Entries3D& e, const float* w, int n, const float* amp, int ld,
                                int trow, float scale, const float* ES, long long field, float* gradb, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_exact_src_entries3d<<<(n + 255) / 256, 256, 0, s>>>(z, e, w, n, amp, ld, trow, scale, ES, field, gradb);
    return cudaGetLastError();
}

cudaError_t reduce3d(const float* buf, long long shot_stride, int nshots, int nx, int ny, int nz, int zp, float* out,
                     cudaStream_t s) {
    k_reduce3d<<<2048, 256, 0, s>>>(buf, shot_stride, nshots, nx, ny, nz, zp, out);
    return cudaGetLastError();
}

}  // namespace sa

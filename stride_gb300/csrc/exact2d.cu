// Exact-gradient helpers of the 2D plan (SA_GRAD_EXACT): per-point coefficients of the vp
// derivative of the discrete update, the per-step gradient accumulation and the source
// term. The reference's own gradient is the imaging condition of
// iso_acoustic/devito.py:985-1043; this mode instead differentiates the discrete forward map
// exactly (the transpose of its linearisation), which is what a finite-difference check of
// the misfit measures.
//
// Update (per point, as k_coef2d): u[n+1] = C1 Lt(u[n]) + C2 u[n] - C3 u[n-1] + s[n] with
// beta = dt (vp^2 d + a vp), d = 7 dt vp S, C1 = dt^2/(1+beta), C2 = (2 - dt^2 vp^2 d^2)/(1+beta),
// C3 = (1-beta)/(1+beta) and Lt = W G (+ dt^2/12 W G W G for OT4). With the adjoint state in the
// form z = C1 W mu (which obeys the forward recursion), step n contributes, per point,
//   mu[n+1] ((dC1 + 2 C1/vp) Lt(u[n]) + dC2 u[n] - dC3 u[n-1])  +  dt^2/(6 vp W) (W G u[n]) (W G z[n+1])
// where Lt(u[n]) = (u[n+1] - C2 u[n] + C3 u[n-1] - s[n]) / C1 comes from three stored levels.
#include <algorithm>

#include "helpers.h"

namespace sa {

namespace {

__global__ void k_exact_coef2d(const float* __restrict__ vp, const float* __restrict__ alpha,
                               const float* __restrict__ W, int nx, int ny, int pitch, Sponge sp, float dt,
                               float* EA, float* EB, float* EC, float* EG4, float* ES) {
    const long long n = (long long)nx * ny;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(q / ny), y = (int)(q % ny);
        const long long p = (long long)x * pitch + y;
        const int ex = min(x, nx - 1 - x), ey = min(y, ny - 1 - y);
        float s = 0.f;
        if (ex < sp.a[0] && ex <= ey) s += sp.s[0][ex];
        if (ey < sp.a[1] && ey <= ex) s += sp.s[1][ey];
        // the update coefficients exactly as the step kernel uses them
        const float v = vp[p], v2 = v * v;
        const float d = 7.f * (s * v) * dt;
        float beta = v2 * d;
        beta = beta + alpha[p] * v;
        beta = dt * beta;
        const float den = 1.f + beta;
        const float C1 = (dt * dt) / den;
        const float C2 = (2.f - dt * dt * v2 * d * d) / den;
        const float C3 = (1.f - beta) / den;
        // their vp derivatives (d is proportional to vp: d(vp^2 d) = 3 vp d, d(vp^2 d^2) = 4 vp d^2)
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

// grad[pair] += z . (a u0 + b u1 + c u2) [+ g4 Lu . Lz]; prec[pair] += |(u0 - 2 u1 + u2) / dt^2|^2
__global__ void k_exact_grad2d(const float2* __restrict__ z, const float2* __restrict__ u0,
                               const float2* __restrict__ u1, const float2* __restrict__ u2,
                               const float2* __restrict__ Lu, const float2* __restrict__ Lz,
                               const float* __restrict__ EA, const float* __restrict__ EB,
                               const float* __restrict__ EC, const float* __restrict__ EG4, int nx, int ny,
                               int pitch, int npairs, long long shot_stride, float inv_dt2, float* gradb,
                               float* precb) {
    const long long n = (long long)nx * ny;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n * npairs;
         q += (long long)gridDim.x * blockDim.x) {
        const int pair = (int)(q / n);
        const long long r = q - (long long)pair * n;
        const int x = (int)(r / ny), y = (int)(r % ny);
        const long long p = (long long)x * pitch + y;
        const long long i = (long long)pair * shot_stride + p;
        const float2 zz = z[i], a0 = u0[i], a1 = u1[i], a2 = u2[i];
        const float ca = EA[p], cb = EB[p], cc = EC[p];
        float g = zz.x * (ca * a0.x + cb * a1.x + cc * a2.x) + zz.y * (ca * a0.y + cb * a1.y + cc * a2.y);
        if (Lu) {
            const float2 lu = Lu[i], lz = Lz[i];
            g += EG4[p] * (lu.x * lz.x + lu.y * lz.y);
        }
        const float dx = (a0.x - 2.f * a1.x + a2.x) * inv_dt2, dy = (a0.y - 2.f * a1.y + a2.y) * inv_dt2;
        gradb[i] += g;
        precb[i] += dx * dx + dy * dy;
    }
}

// Source term at each support point of each source (linear corners or the wide Hicks / sinc
// support): z w src[trow] (2 dt / h) ES.
__global__ void k_exact_src2d(const float* __restrict__ z, const ExactSrc2D* __restrict__ e, int n,
                              const float* __restrict__ amp, int ld, int trow, float scale,
                              const float* __restrict__ ES, float* gradb) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const ExactSrc2D E = e[k];
    const float a = amp[(long long)trow * ld + E.point] * scale;
    atomicAdd(gradb + E.i, z[2 * E.i + E.lane] * E.w * a * ES[E.p]);
}

}  // namespace

cudaError_t exact_coef2d(const float* vp, const float* alpha, const float* W, int nx, int ny, int pitch,
                         const Sponge& sp, float dt, float* EA, float* EB, float* EC, float* EG4, float* ES,
                         cudaStream_t s) {
    k_exact_coef2d<<<1024, 256, 0, s>>>(vp, alpha, W, nx, ny, pitch, sp, dt, EA, EB, EC, EG4, ES);
    return cudaGetLastError();
}

cudaError_t exact_grad2d(const float* z, const float* u0, const float* u1, const float* u2, const float* Lu,
                         const float* Lz, const float* EA, const float* EB, const float* EC, const float* EG4, int nx,
                         int ny, int pitch, int npairs, long long shot_stride, float inv_dt2, float* gradb,
                         float* precb, cudaStream_t s) {
    const long long n = (long long)nx * ny * npairs;
    const int blocks = (int)std::min<long long>((n + 255) / 256, 152 * 16);
    k_exact_grad2d<<<blocks, 256, 0, s>>>(
        reinterpret_cast<const float2*>(z), reinterpret_cast<const float2*>(u0), reinterpret_cast<const float2*>(u1),
        reinterpret_cast<const float2*>(u2), reinterpret_cast<const float2*>(Lu), reinterpret_cast<const float2*>(Lz),
        EA, EB, EC, EG4, nx, ny, pitch, npairs, shot_stride, inv_dt2, gradb, precb);
    return cudaGetLastError();
}

cudaError_t exact_src2d(const float* z, const ExactSrc2D* e, int n, const float* amp, int ld, int trow, float scale,
                        const float* ES, float* gradb, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_exact_src2d<<<(n + 127) / 128, 128, 0, s>>>(z, e, n, amp, ld, trow, scale, ES, gradb);
    return cudaGetLastError();
}

}  // namespace sa

#include <algorithm>
#include <cmath>
#include <vector>
// Small device helpers of the plan: medium preparation, sparse-trace transposes, the final
// receiver gather and the reduction of per-shot gradients.
#include "fdtd2d.cuh"
#include "helpers.h"

namespace sa {

// Hicks coefficients of one axis (GridDevito._calculate_hicks, common/devito.py:843-885): Kaiser-
// windowed sinc at offsets -3..3 from the base point (index 3 + offset; index 7 is zero), with the
// reference's smoothing of the central coefficients for sources.
void hicks_coefs(double frac, bool smooth, double c[8]) {
    const double kb = 4.14, half = 3.0, ext = half / 0.99, den = std::cyl_bessel_i(0.0, kb);
    for (int k = 0; k < 8; k++) c[k] = 0.0;
    for (int gp = -3; gp <= 3; gp++) {
        const double x = frac - gp;
        double w = (x / ext) * (x / ext);
        if (w > 1) w = 1;
        const double sinc = x == 0.0 ? 1.0 : std::sin(M_PI * x) / (M_PI * x);
        c[3 + gp] = sinc * std::cyl_bessel_i(0.0, kb * std::sqrt(1 - w)) / den;
    }
    if (smooth) {
        const int m = 2;
        const double a = c[m], b = c[m + 1], cc = c[m + 2];
        c[m - 1] = c[m - 1] + a * 0.01;
        c[m] = a * 0.98 + b * 0.03;
        c[m + 1] = b * 0.94 + (a + cc) * 0.01;
        c[m + 2] = cc * 0.98 + b * 0.03;
        c[m + 3] = c[m + 3] + cc * 0.01;
    }
}

// Kaiser-windowed sinc of half-width r (Hicks 2002, "Arbitrary source and receiver positioning in
// finite-difference schemes using Kaiser windowed sinc functions"), the interpolation of Devito's
// SparseTimeFunction(interpolation='sinc', r) that stride/physics/common/devito.py:634-638 builds with
// r = 7: weights at grid offsets -r+1 .. r from the base point (index i: offset i - r + 1),
// w(x) = sinc(x) I0(b sqrt(1 - (x/r)^2)) / I0(b) at x = offset - frac, with b from the paper's table
// of window parameters by half-width.
void sinc_coefs(double frac, int r, double* c) {
    static const double b_of_r[11] = {0.0, 1.24, 2.94, 4.53, 4.14, 5.26, 6.40, 7.51, 8.56, 9.56, 10.64};
    const double b = b_of_r[r], den = std::cyl_bessel_i(0.0, b);
    for (int i = 0; i < 2 * r; i++) {
        const double x = (double)(i - r + 1) - frac, q = x / r;
        const double sinc = x == 0.0 ? 1.0 : std::sin(M_PI * x) / (M_PI * x);
        c[i] = q * q >= 1.0 ? 0.0 : sinc * std::cyl_bessel_i(0.0, b * std::sqrt(1.0 - q * q)) / den;
    }
}

int support_coefs(int interp, double frac, bool smooth, double c[SUPPORT_MAX]) {
    for (int i = 0; i < SUPPORT_MAX; i++) c[i] = 0.0;
    if (interp == SA_INTERP_SINC) {
        sinc_coefs(frac, 7, c);
        return 14;
    }
    hicks_coefs(frac, smooth, c);
    return 8;
}

// CFS-PML profiles per axis (ComplexFrequencyShiftPML2.apply, stride/physics/boundaries/devito.py:
// 96-127, with Boundary.damping, boundaries/boundary.py:59-170), FP32 as the reference stores them:
// sigma 'power' degree 3 with the coefficient 2 ln(1/R) / (absorbing h) (0.67 / h for layers of 15
// cells or fewer), times max(vp); alpha a 'power' degree 2 mask, 0.01 pi f_centre in the interior
// and -0.01 pi f_centre pos^2 in the layer; sigma' and alpha' 2nd-order centred differences over an
// edge-padded halo. Layout: sigma, alpha, sigma', alpha' of axis 0 (shape[0] each), then axis 1, ...
std::vector<float> pml_profile_tables(const sa_desc& d, float vmax) {
    int amax = 0;
    for (int a = 0; a < d.dim; a++) amax = std::max(amax, d.absorbing[a]);
    const double refl = std::pow(10.0, -(std::log10((double)std::max(amax, 2)) - 1) / std::log10(2.0) - 3);
    std::vector<float> out;
    for (int a = 0; a < d.dim; a++) {
        const int n = d.shape[a], A = d.absorbing[a];
        const double h = d.spacing[a];
        const double cs = A > 15 ? (3 + 1) / 2.0 * std::log(1.0 / refl) / (A * h) : 0.67 / h;
        const double ca = 0.01 * M_PI * d.f_centre;
        std::vector<float> sg(n, 0.f), al(n, (float)ca), dsg(n), dal(n);
        for (int index = 0; index < A; index++) {
            const double pos = std::fabs((A - index - 1) / (double)(A - 1));
            sg[index] = sg[n - index - 1] = (float)(cs * pos * pos * pos);
            al[index] = al[n - index - 1] = (float)(ca * -(pos * pos));
        }
        for (float& v : sg) v *= vmax;
        for (int i = 0; i < n; i++) {
            const int ip = std::min(i + 1, n - 1), im = std::max(i - 1, 0);
            dsg[i] = (sg[ip] - sg[im]) / (float)(2 * h);
            dal[i] = (al[ip] - al[im]) / (float)(2 * h);
        }
        for (auto* v : {&sg, &al, &dsg, &dal}) out.insert(out.end(), v->begin(), v->end());
    }
    return out;
}

// vp, rho, alpha (dB/cm) on the unpadded extended grid -> pitched W (guarded layout, pointer
// at row 0), vp, alpha (Np/m) and buoyancy b = 1/rho scratch (iso_acoustic/devito.py:476-497).
__global__ void k_medium2d(const float* __restrict__ vp_in, const float* __restrict__ rho_in,
                           const float* __restrict__ alpha_in, int nx, int ny, int pitch, int density,
                           double db_to_np, float* W, float* vp, float* alpha, float* buoy) {
    const long long n = (long long)nx * ny;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(q / ny), y = (int)(q % ny);
        const long long p = (long long)x * pitch + y;
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

// Buoyancy at half points: bxh[x*pitch + y] = b(x+1/2, y) for x = -5..nx+3 (pointer at x = 0)
// and byh[x*pitch_b + y + 6] = b(x, y+1/2) for y = -6..ny+3; nodes beyond the grid take the
// edge value as the reference's edge-padded halo (common/devito.py:805-841), the half point is
// the arithmetic mean of its two nodes.
__global__ void k_bhalf2d(const float* __restrict__ buoy, int nx, int ny, int pitch, int pitch_b, float* bxh,
                          float* byh) {
    const long long nxa = (long long)(nx + 9) * ny;
    const long long nya = (long long)nx * (ny + 10);
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nxa + nya;
         q += (long long)gridDim.x * blockDim.x) {
        if (q < nxa) {
            const int x = (int)(q / ny) - 5, y = (int)(q % ny);
            const int x0 = min(max(x, 0), nx - 1), x1 = min(max(x + 1, 0), nx - 1);
            bxh[(long long)x * pitch + y] = 0.5f * (buoy[(long long)x0 * pitch + y] + buoy[(long long)x1 * pitch + y]);
        } else {
            const long long r = q - nxa;
            const int x = (int)(r / (ny + 10)), yr = (int)(r % (ny + 10));
            const int y = yr - 6;
            const int y0 = min(max(y, 0), ny - 1), y1 = min(max(y + 1, 0), ny - 1);
            byh[(long long)x * pitch_b + yr] = 0.5f * (buoy[(long long)x * pitch + y0] + buoy[(long long)x * pitch + y1]);
        }
    }
}

// Update coefficients of p_new = C1 Lt + C2 p - C3 p_other, the solved form of
// p.dt2 - Lt + 2 alpha vp p.dt + vp^2 (2 d p.dtc + d^2 p) = 0 (iso_acoustic/devito.py:1575-1581)
// with the SpongeBoundary2 damping d = 7 dt vp S(x) (boundaries/devito.py:52-67). S follows
// Boundary.damping's slab rule (boundary.py:116-160): the x slab at layer e covers y layers
// >= e and vice versa, so corner points take the outer slab (both on the diagonal).
__global__ void k_coef2d(const float* __restrict__ vp, const float* __restrict__ alpha, int nx, int ny, int pitch,
                         Sponge sp, float dt, float* C1, float* C2, float* C3) {
    const long long n = (long long)nx * ny;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(q / ny), y = (int)(q % ny);
        const long long p = (long long)x * pitch + y;
        const int ex = min(x, nx - 1 - x), ey = min(y, ny - 1 - y);
        float s = 0.f;
        if (ex < sp.a[0] && ex <= ey) s += sp.s[0][ex];
        if (ey < sp.a[1] && ey <= ex) s += sp.s[1][ey];
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

cudaError_t medium2d(const float* vp_in, const float* rho_in, const float* alpha_in, int nx, int ny, int pitch,
                     int pitch_b, int density, double db_to_np, const Sponge& sp, float dt, float* W, float* vp,
                     float* alpha, float* buoy, float* bxh, float* byh, float* C1, float* C2, float* C3,
                     cudaStream_t s) {
    k_medium2d<<<1024, 256, 0, s>>>(vp_in, rho_in, alpha_in, nx, ny, pitch, density, db_to_np, W, vp, alpha, buoy);
    if (density == 1) k_bhalf2d<<<1024, 256, 0, s>>>(buoy, nx, ny, pitch, pitch_b, bxh, byh);
    k_coef2d<<<1024, 256, 0, s>>>(vp, alpha, nx, ny, pitch, sp, dt, C1, C2, C3);
    return cudaGetLastError();
}

// Medium of the 2D step passes: six arrays (W, bx, by, C1, C2, -C3), each
// [nx + 2 MED_GUARD][mpitch] floats, `astride` floats apart, column y at index y + MED_MARGIN
// (one array per field: a warp's loads of one field are contiguous). Beyond what the source
// arrays hold, a value is the nearest held one: the edge-padded halo of the materials
// (stride/physics/common/devito.py:805-841) for the half-point buoyancy, any finite value
// elsewhere (it only reaches lanes the kernel discards). W, C1..C3 address row 0 (columns
// 0..ny-1); bxh half-row 0 (half-rows -5..nx+3); byh row 0 with half-column y at column y + 6
// (y = -6..ny+3). bxh/byh may be null (no buoyancy).
__global__ void k_step_medium2d(const float* __restrict__ W, const float* __restrict__ bxh,
                                const float* __restrict__ byh, const float* __restrict__ C1,
                                const float* __restrict__ C2, const float* __restrict__ C3, int nx, int ny, int pitch,
                                int pitch_b, int mpitch, long long astride, float* __restrict__ out) {
    const int rows = nx + 2 * MED_GUARD;
    const long long n = (long long)rows * mpitch;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(q / mpitch) - MED_GUARD, y = (int)(q % mpitch) - MED_MARGIN;
        const int xn = min(max(x, 0), nx - 1), yn = min(max(y, 0), ny - 1);
        const long long node = (long long)xn * pitch + yn;
        out[q] = W[node];
        out[astride + q] = bxh ? bxh[(long long)min(max(x, -5), nx + 3) * pitch + yn] : 1.f;
        out[2 * astride + q] = byh ? byh[(long long)xn * pitch_b + min(max(y, -6), ny + 3) + 6] : 1.f;
        out[3 * astride + q] = C1[node];
        out[4 * astride + q] = C2[node];
        out[5 * astride + q] = -C3[node];
    }
}

cudaError_t step_medium2d(const float* W, const float* bxh, const float* byh, const float* C1, const float* C2,
                          const float* C3, int nx, int ny, int pitch, int pitch_b, float* out, cudaStream_t s) {
    const int mp = med_pitch(ny);
    k_step_medium2d<<<1024, 256, 0, s>>>(W, bxh, byh, C1, C2, C3, nx, ny, pitch, pitch_b, mp,
                                         (long long)(nx + 2 * MED_GUARD) * mp, out);
    return cudaGetLastError();
}

// out[c][r] = in[r][c] for an rows x cols matrix (both dense).
__global__ void k_transpose(const float* __restrict__ in, int rows, int cols, float* __restrict__ out) {
    __shared__ float tile[32][33];
    const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int r = by + k, c = bx + threadIdx.x;
        if (r < rows && c < cols) tile[k][threadIdx.x] = in[(long long)r * cols + c];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int c = bx + k, r = by + threadIdx.x;
        if (r < rows && c < cols) out[(long long)c * rows + r] = tile[threadIdx.x][k];
    }
}

__device__ __forceinline__ void gather_point(const float* __restrict__ field, long long shot_stride, int pitch,
                                             const Gather* __restrict__ g, int e, float* out, int ld, int trow) {
    const Gather G = g[e];  // pad = shot: pair pad / 2, lane pad % 2 of the interleaved field
    const float* f = field + (long long)(G.pad / 2) * shot_stride * 2 + (G.pad & 1);
    const long long i0 = 2 * ((long long)G.row * pitch + G.col), i1 = i0 + 2 * (long long)pitch;
    out[(long long)trow * ld + G.point] = G.w00 * f[i0] + G.w01 * f[i0 + 2] + G.w10 * f[i1] + G.w11 * f[i1 + 2];
}

__global__ void gather_final2d(const float* __restrict__ field, long long shot_stride, int pitch,
                               const Gather* __restrict__ g, int n, float* out, int ld, int trow) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n) gather_point(field, shot_stride, pitch, g, e, out, ld, trow);
}

// rec[trow][point] = sum over the width x width support of wx[i] wy[j] field(row + i, col + j).
__global__ void k_support_gather2d(const float* __restrict__ field, long long shot_stride, int pitch,
                                   const SupportGather* __restrict__ g, int n, float* out, int ld, int trow) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const SupportGather& G = g[e];
    const float* f = field + (long long)(G.shot / 2) * shot_stride * 2 + (G.shot & 1);
    float v = 0.f;
    for (int i = 0; i < G.width; i++) {
        const float* row = f + 2 * (long long)(G.row + i) * pitch;
        float r = 0.f;
        for (int j = 0; j < G.width; j++) r += G.wy[j] * row[2 * (G.col + j)];
        v += G.wx[i] * r;
    }
    out[(long long)trow * ld + G.point] = v;
}

cudaError_t support_gather2d(const float* field, long long shot_stride, int pitch, const SupportGather* g, int n,
                             float* out, int ld, int trow, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_support_gather2d<<<(n + 127) / 128, 128, 0, s>>>(field, shot_stride, pitch, g, n, out, ld, trow);
    return cudaGetLastError();
}

// Imaging condition of one adjoint level t (t % f == 0), interior only: grad[pair] += snap . q,
// prec[pair] += snap . snap (both shots of a pair summed), q = p_a[t] (pair-interleaved).
__global__ void k_image2d(const float2* __restrict__ q, const float2* __restrict__ snap, float* gradb, float* precb,
                          int ix0, int ix1, int iy0, int iy1, int pitch, int npairs, long long shot_stride,
                          long long snap_shot_stride) {
    const int w = iy1 - iy0;
    const long long per = (long long)(ix1 - ix0) * w;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < per * npairs;
         e += (long long)gridDim.x * blockDim.x) {
        const int pair = (int)(e / per);
        const long long r = e - (long long)pair * per;
        const int x = ix0 + (int)(r / w), y = iy0 + (int)(r % w);
        const long long idx = (long long)x * pitch + y;
        const float2 sv = snap[(long long)pair * snap_shot_stride + idx];
        const float2 u = q[(long long)pair * shot_stride + idx];
        const long long gi = (long long)pair * shot_stride + idx;
        gradb[gi] += sv.x * u.x + sv.y * u.y;
        precb[gi] += sv.x * sv.x + sv.y * sv.y;
    }
}

cudaError_t image2d(const float* q, const float* snap, float* gradb, float* precb, int ix0, int ix1, int iy0, int iy1,
                    int pitch, int npairs, long long shot_stride, long long snap_shot_stride, cudaStream_t s) {
    const long long n = (long long)(ix1 - ix0) * (iy1 - iy0) * npairs;
    if (n <= 0) return cudaSuccess;
    const int blocks = (int)std::min<long long>((n + 255) / 256, 152 * 8);
    k_image2d<<<blocks, 256, 0, s>>>(reinterpret_cast<const float2*>(q), reinterpret_cast<const float2*>(snap), gradb,
                                     precb, ix0, ix1, iy0, iy1, pitch, npairs, shot_stride, snap_shot_stride);
    return cudaGetLastError();
}

// D-_x b and D-_y b at every node: the staggered first derivatives at x-1/2 and y-1/2 of the
// buoyancy, nodes beyond the grid taking the edge value (the reference's edge-padded material
// halo). They are the grad(buoy, shift=-0.5) factor of the rho imaging term
// (iso_acoustic/devito.py:1137).
__global__ void k_rho_terms2d(const float* __restrict__ buoy, int nx, int ny, int pitch, float ihx, float ihy,
                              float* dbx, float* dby) {
    const long long n = (long long)nx * ny;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(e / ny), y = (int)(e % ny);
        float ax = 0.f, ay = 0.f;
#pragma unroll
        for (int m = 0; m < 5; m++) {
            const int xh = min(x + m, nx - 1), xl = max(x - 1 - m, 0);
            const int yh = min(y + m, ny - 1), yl = max(y - 1 - m, 0);
            ax += kWS(m) * (buoy[(long long)xh * pitch + y] - buoy[(long long)xl * pitch + y]);
            ay += kWS(m) * (buoy[(long long)x * pitch + yh] - buoy[(long long)x * pitch + yl]);
        }
        dbx[(long long)x * pitch + y] = ax * ihx;
        dby[(long long)x * pitch + y] = ay * ihy;
    }
}

cudaError_t rho_terms2d(const float* buoy, int nx, int ny, int pitch, float hx, float hy, float* dbx, float* dby,
                        cudaStream_t s) {
    k_rho_terms2d<<<1024, 256, 0, s>>>(buoy, nx, ny, pitch, 1.f / hx, 1.f / hy, dbx, dby);
    return cudaGetLastError();
}

// Imaging from the raw saved wavefield s[n] = p[n f] (the reference's gradients when rho or the
// wavelets need one, iso_acoustic/devito.py:1003-1024, 1133-1150). On a refresh step (t = n f)
// the held terms of every interior point are recomputed from the snapshots:
//   vp:  (s[n+1] - 2 s[n] + s[n-1]) * inv_fdt2,
//   rho: -(D-_x b D-_x s[n] + D-_y b D-_y s[n]) - b laplace(s[n])  (zero halo for s),
// and every step accumulates grad += held q, prec += held^2 over the pair's two lanes.
// snap addresses slot n of pair 0 (float2 units for the strides); hold_rho null: vp only.
__global__ void k_image_raw2d(const float2* __restrict__ q, const float2* __restrict__ snap, long long snap_stride,
                              long long snap_shot_stride, int refresh, float inv_fdt2, float2* hold_vp,
                              float2* hold_rho, const float* __restrict__ buoy, const float* __restrict__ dbx,
                              const float* __restrict__ dby, float ihx, float ihy, int nx, int ny, float* gradb,
                              float* precb, float* gradrb, float* precrb, int ix0, int ix1, int iy0, int iy1,
                              int pitch, int npairs, long long shot_stride) {
    const int w = iy1 - iy0;
    const long long per = (long long)(ix1 - ix0) * w;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < per * npairs;
         e += (long long)gridDim.x * blockDim.x) {
        const int pair = (int)(e / per);
        const long long r = e - (long long)pair * per;
        const int x = ix0 + (int)(r / w), y = iy0 + (int)(r % w);
        const long long idx = (long long)x * pitch + y;
        const long long gi = (long long)pair * shot_stride + idx;
        float2 hv, hr = make_float2(0.f, 0.f);
        if (refresh) {
            const float2* sp = snap + (long long)pair * snap_shot_stride;
            const float2 s0 = sp[idx], sn = sp[idx + snap_stride], so = sp[idx - snap_stride];
            hv = make_float2(((sn.x - 2.f * s0.x) + so.x) * inv_fdt2, ((sn.y - 2.f * s0.y) + so.y) * inv_fdt2);
            hold_vp[gi] = hv;
            if (hold_rho) {
                float2 gx = make_float2(0.f, 0.f), gy = gx;
                float2 lx = make_float2(kW2(0) * s0.x, kW2(0) * s0.y), ly = lx;
#pragma unroll
                for (int m = 0; m < 5; m++) {
                    const float2 xh = x + m < nx ? sp[idx + (long long)m * pitch] : make_float2(0.f, 0.f);
                    const float2 xl = x - 1 - m >= 0 ? sp[idx - (long long)(m + 1) * pitch] : make_float2(0.f, 0.f);
                    const float2 yh = y + m < ny ? sp[idx + m] : make_float2(0.f, 0.f);
                    const float2 yl = y - 1 - m >= 0 ? sp[idx - (m + 1)] : make_float2(0.f, 0.f);
                    gx.x += kWS(m) * (xh.x - xl.x);
                    gx.y += kWS(m) * (xh.y - xl.y);
                    gy.x += kWS(m) * (yh.x - yl.x);
                    gy.y += kWS(m) * (yh.y - yl.y);
                    const int k = m + 1;
                    const float2 xp = x + k < nx ? sp[idx + (long long)k * pitch] : make_float2(0.f, 0.f);
                    const float2 xm = x - k >= 0 ? sp[idx - (long long)k * pitch] : make_float2(0.f, 0.f);
                    const float2 yp = y + k < ny ? sp[idx + k] : make_float2(0.f, 0.f);
                    const float2 ym = y - k >= 0 ? sp[idx - k] : make_float2(0.f, 0.f);
                    lx.x += kW2(k) * (xp.x + xm.x);
                    lx.y += kW2(k) * (xp.y + xm.y);
                    ly.x += kW2(k) * (yp.x + ym.x);
                    ly.y += kW2(k) * (yp.y + ym.y);
                }
                const float bx = dbx[idx], by = dby[idx], b = buoy[idx];
                const float ihx2 = ihx * ihx, ihy2 = ihy * ihy;
                hr.x = -(bx * (gx.x * ihx) + by * (gy.x * ihy)) - b * (lx.x * ihx2 + ly.x * ihy2);
                hr.y = -(bx * (gx.y * ihx) + by * (gy.y * ihy)) - b * (lx.y * ihx2 + ly.y * ihy2);
                hold_rho[gi] = hr;
            }
        } else {
            hv = hold_vp[gi];
            if (hold_rho) hr = hold_rho[gi];
        }
        const float2 u = q[gi];
        gradb[gi] += hv.x * u.x + hv.y * u.y;
        precb[gi] += hv.x * hv.x + hv.y * hv.y;
        if (hold_rho) {
            gradrb[gi] += hr.x * u.x + hr.y * u.y;
            precrb[gi] += hr.x * hr.x + hr.y * hr.y;
        }
    }
}

cudaError_t image_raw2d(const float* q, const float* snap, long long snap_stride, long long snap_shot_stride,
                        int refresh, float inv_fdt2, float* hold_vp, float* hold_rho, const float* buoy,
                        const float* dbx, const float* dby, float hx, float hy, int nx, int ny, float* gradb,
                        float* precb, float* gradrb, float* precrb, int ix0, int ix1, int iy0, int iy1, int pitch,
                        int npairs, long long shot_stride, cudaStream_t s) {
    const long long n = (long long)(ix1 - ix0) * (iy1 - iy0) * npairs;
    if (n <= 0) return cudaSuccess;
    const int blocks = (int)std::min<long long>((n + 255) / 256, 152 * 8);
    k_image_raw2d<<<blocks, 256, 0, s>>>(
        reinterpret_cast<const float2*>(q), reinterpret_cast<const float2*>(snap), snap_stride, snap_shot_stride,
        refresh, inv_fdt2, reinterpret_cast<float2*>(hold_vp), reinterpret_cast<float2*>(hold_rho), buoy, dbx, dby,
        1.f / hx, 1.f / hy, nx, ny, gradb, precb, gradrb, precrb, ix0, ix1, iy0, iy1, pitch, npairs, shot_stride);
    return cudaGetLastError();
}


// CFS-PML (ComplexFrequencyShiftPML2, boundaries/devito.py:72-191) after a step of the OT2
// operator: on every point of the absorbing frame, for each axis d whose slab holds the point,
// the auxiliary fields advance with the derivatives of the current level f = p[t] along d
// (zero halo; the adjoint transposes the first derivative, -f_d):
//   u3' = u3 - dt ((a + s) u3 - s^2 (s' + a') f_d)
//   u2' = u2 - dt ((a + s) u2 - s (2 s' f_d + a' f_d + s f_dd) + u3')
//   u1' = u1 - dt ((a + s) u1 - (s' f_d + 2 s f_dd) + u2')
// and the new level, computed by the step kernel without the boundary term, takes it:
// p[t+1] -= C1 vp^2 sum_d u1' (the term vp^2 u_1 of the boundary equation, iso_acoustic/devito.py:
// 1575-1582). On a p.dt2 save step the snapshot takes the same correction / dt^2.
// prof: sigma, alpha, sigma', alpha' of the x axis (nx each), then of the y axis (ny each).
// aux: 6 fields (u3, u2, u1 of x, then of y), each npairs * shot_stride float2.
__global__ void k_pml2d(const float2* __restrict__ cur, float2* nxt, float2* aux, const float* __restrict__ prof,
                        const float* __restrict__ C1, const float* __restrict__ vp, int nx, int ny, int pitch,
                        long long shot_stride, int npairs, int ax, int ay, float ihx, float ihy, float dt, int adjoint,
                        float2* snap, long long snap_shot_stride, float inv_dt2) {
    const long long band = (long long)ax * ny;             // points of one x slab
    const long long side = (long long)(nx - 2 * ax) * ay;  // points of one y slab between the x slabs
    const long long per = 2 * band + 2 * side;
    const long long fs = (long long)npairs * shot_stride;  // float2 per auxiliary field
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < per * npairs;
         e += (long long)gridDim.x * blockDim.x) {
        const int pair = (int)(e / per);
        long long r = e - (long long)pair * per;
        int x, y;
        if (r < 2 * band) {
            const long long q = r < band ? r : r - band;
            x = (int)(q / ny) + (r < band ? 0 : nx - ax);
            y = (int)(q % ny);
        } else {
            r -= 2 * band;
            const long long q = r < side ? r : r - side;
            x = ax + (int)(q / ay);
            y = (int)(q % ay) + (r < side ? 0 : ny - ay);
        }
        const long long idx = (long long)x * pitch + y;
        const long long base = (long long)pair * shot_stride;
        const float2* f = cur + base;
        float bx = 0.f, by = 0.f;  // sum of u1' over the axes, per lane
#pragma unroll
        for (int d = 0; d < 2; d++) {
            const int i = d == 0 ? x : y, n = d == 0 ? nx : ny, a = d == 0 ? ax : ay;
            if (!(i < a || i >= n - a)) continue;
            const long long st = d == 0 ? pitch : 1;
            const float ih = d == 0 ? ihx : ihy;
            const float2 f0 = f[idx];
            float2 g = make_float2(0.f, 0.f), l = make_float2(kW2(0) * f0.x, kW2(0) * f0.y);
#pragma unroll
            for (int k = 1; k <= 5; k++) {
                const float2 fp = i + k < n ? f[idx + k * st] : make_float2(0.f, 0.f);
                const float2 fm = i - k >= 0 ? f[idx - k * st] : make_float2(0.f, 0.f);
                g.x += kW1(k) * (fp.x - fm.x);
                g.y += kW1(k) * (fp.y - fm.y);
                l.x += kW2(k) * (fp.x + fm.x);
                l.y += kW2(k) * (fp.y + fm.y);
            }
            const float sgn = adjoint ? -ih : ih;
            g.x *= sgn;
            g.y *= sgn;
            l.x *= ih * ih;
            l.y *= ih * ih;
            const float* pr = prof + (d == 0 ? 0 : 4 * nx);
            const float s = pr[i], al = pr[n + i], ds = pr[2 * n + i], da = pr[3 * n + i];
            float2* u3 = aux + (3 * d) * fs + base + idx;
            float2* u2 = aux + (3 * d + 1) * fs + base + idx;
            float2* u1 = aux + (3 * d + 2) * fs + base + idx;
            float2 v3 = *u3, v2 = *u2, v1 = *u1;
            const float as = al + s;
            v3.x = v3.x - dt * (as * v3.x - s * s * (ds + da) * g.x);
            v3.y = v3.y - dt * (as * v3.y - s * s * (ds + da) * g.y);
            v2.x = v2.x - dt * (as * v2.x - s * (2.f * ds * g.x + da * g.x + s * l.x) + v3.x);
            v2.y = v2.y - dt * (as * v2.y - s * (2.f * ds * g.y + da * g.y + s * l.y) + v3.y);
            v1.x = v1.x - dt * (as * v1.x - (ds * g.x + 2.f * s * l.x) + v2.x);
            v1.y = v1.y - dt * (as * v1.y - (ds * g.y + 2.f * s * l.y) + v2.y);
            *u3 = v3;
            *u2 = v2;
            *u1 = v1;
            bx += v1.x;
            by += v1.y;
        }
        const float v = vp[idx];
        const float k = C1[idx] * (v * v);
        float2* pn = nxt + base + idx;
        float2 o = *pn;
        o.x -= k * bx;
        o.y -= k * by;
        *pn = o;
        if (snap) {
            float2* sp = snap + (long long)pair * snap_shot_stride + idx;
            float2 w = *sp;
            w.x -= k * bx * inv_dt2;
            w.y -= k * by * inv_dt2;
            *sp = w;
        }
    }
}

cudaError_t pml2d(const float* cur, float* nxt, float* aux, const float* prof, const float* C1, const float* vp, int nx,
                  int ny, int pitch, long long shot_stride, int npairs, int ax, int ay, float hx, float hy, float dt,
                  int adjoint, float* snap, long long snap_shot_stride, float inv_dt2, cudaStream_t s) {
    const long long n = (2LL * ax * ny + 2LL * (nx - 2 * ax) * ay) * npairs;
    if (n <= 0) return cudaSuccess;
    const int blocks = (int)std::min<long long>((n + 255) / 256, 152 * 8);
    k_pml2d<<<blocks, 256, 0, s>>>(reinterpret_cast<const float2*>(cur), reinterpret_cast<float2*>(nxt),
                                   reinterpret_cast<float2*>(aux), prof, C1, vp, nx, ny, pitch, shot_stride, npairs,
                                   ax, ay, 1.f / hx, 1.f / hy, dt, adjoint, reinterpret_cast<float2*>(snap),
                                   snap_shot_stride, inv_dt2);
    return cudaGetLastError();
}

// field[idx[k]] += sum over the target's entries of coef[e] * amp[t][point[e]] (one thread per
// target point; entries in a fixed order). With snap, the same sum times inv_dt2 also enters the
// pair-interleaved snapshot level (shot-pair stride snap_shot_stride instead of shot_stride).
__device__ __forceinline__ void inject_target(float* field, const long long* __restrict__ idx,
                                              const int* __restrict__ off, const float* __restrict__ coef,
                                              const int* __restrict__ point, int k, const float* __restrict__ amp,
                                              int ld, int t, float* snap, long long shot_stride,
                                              long long snap_shot_stride, float inv_dt2) {
    float v = 0.f;
    const float* a = amp + (long long)t * ld;
    for (int e = off[k]; e < off[k + 1]; e++) v += coef[e] * a[point[e]];
    const long long i = idx[k];
    field[i] += v;
    if (snap) {
        const long long pair = i / (2 * shot_stride);
        snap[pair * 2 * snap_shot_stride + (i - pair * 2 * shot_stride)] += v * inv_dt2;
    }
}

__global__ void k_inject_targets2d(float* field, const long long* __restrict__ idx, const int* __restrict__ off,
                                   const float* __restrict__ coef, const int* __restrict__ point, int n,
                                   const float* __restrict__ amp, int ld, int t, float* snap, long long shot_stride,
                                   long long snap_shot_stride, float inv_dt2) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) inject_target(field, idx, off, coef, point, k, amp, ld, t, snap, shot_stride, snap_shot_stride, inv_dt2);
}

// The sparse work between two forward steps in one launch: blocks [0, nbi) inject the sources of
// step t into the new level (as k_inject_targets2d), the other blocks gather the receivers of the
// previous step, rec[trow] = interp(gfield), from the current level. The two touch different
// levels, so their order does not matter; one launch instead of two per step.
__global__ void k_inject_gather2d(float* field, const long long* __restrict__ idx, const int* __restrict__ off,
                                  const float* __restrict__ coef, const int* __restrict__ point, int n,
                                  const float* __restrict__ amp, int ld, int t, float* snap, long long shot_stride,
                                  long long snap_shot_stride, float inv_dt2, int nbi, const float* __restrict__ gfield,
                                  int pitch, const Gather* __restrict__ g, int ng, float* out, int gld, int trow) {
    if ((int)blockIdx.x < nbi) {
        const int k = blockIdx.x * blockDim.x + threadIdx.x;
        if (k < n) inject_target(field, idx, off, coef, point, k, amp, ld, t, snap, shot_stride, snap_shot_stride, inv_dt2);
    } else {
        const int e = (blockIdx.x - nbi) * blockDim.x + threadIdx.x;
        if (e < ng) gather_point(gfield, shot_stride, pitch, g, e, out, gld, trow);
    }
}

cudaError_t inject_gather2d(float* field, const long long* idx, const int* off, const float* coef, const int* point,
                            int n, const float* amp, int ld, int t, float* snap, long long shot_stride,
                            long long snap_shot_stride, float inv_dt2, const float* gfield, int pitch,
                            const Gather* g, int ng, float* out, int gld, int trow, cudaStream_t s) {
    const int nbi = (n + 255) / 256, nbg = (ng + 255) / 256;
    if (nbi + nbg == 0) return cudaSuccess;
    k_inject_gather2d<<<nbi + nbg, 256, 0, s>>>(field, idx, off, coef, point, n, amp, ld, t, snap, shot_stride,
                                                snap_shot_stride, inv_dt2, nbi, gfield, pitch, g, ng, out, gld, trow);
    return cudaGetLastError();
}

cudaError_t inject_targets2d(float* field, const long long* idx, const int* off, const float* coef, const int* point,
                             int n, const float* amp, int ld, int t, float* snap, long long shot_stride,
                             long long snap_shot_stride, int, float inv_dt2, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_inject_targets2d<<<(n + 255) / 256, 256, 0, s>>>(field, idx, off, coef, point, n, amp, ld, t, snap, shot_stride,
                                                       snap_shot_stride, inv_dt2);
    return cudaGetLastError();
}

__global__ void reduce_shots2d(const float* __restrict__ buf, long long shot_stride, int nshots, int nx, int ny,
                               int pitch, float* __restrict__ out) {
    const long long n = (long long)nx * ny;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(q / ny), y = (int)(q % ny);
        const long long p = (long long)x * pitch + y;
        float s = 0.f;
        for (int b = 0; b < nshots; b++) s += buf[(long long)b * shot_stride + p];
        out[q] = s;
    }
}

cudaError_t transpose(const float* in, int rows, int cols, float* out, cudaStream_t s) {
    if (rows == 0 || cols == 0) return cudaSuccess;
    dim3 grid((cols + 31) / 32, (rows + 31) / 32);
    k_transpose<<<grid, dim3(32, 8), 0, s>>>(in, rows, cols, out);
    return cudaGetLastError();
}

cudaError_t final_gather2d(const float* field, long long shot_stride, int pitch, const Gather* g, int n, float* out,
                           int ld, int trow, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    gather_final2d<<<(n + 127) / 128, 128, 0, s>>>(field, shot_stride, pitch, g, n, out, ld, trow);
    return cudaGetLastError();
}

cudaError_t reduce_shots(const float* buf, long long shot_stride, int nshots, int nx, int ny, int pitch, float* out,
                         cudaStream_t s) {
    reduce_shots2d<<<1024, 256, 0, s>>>(buf, shot_stride, nshots, nx, ny, pitch, out);
    return cudaGetLastError();
}

}  // namespace sa

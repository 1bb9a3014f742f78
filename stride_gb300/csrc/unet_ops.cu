// Layer kernels of the learned preconditioner's U-Net around the tcgen05 GEMM (umma_gemm.cu):
// activations are NHWC fp32 ([pixels][channels], pixels = batch * H * W, channel stride ld),
// GEMM operands bf16. A 3x3 convolution is im2col (bf16 [pixels][Kp], column (ky*3+kx)*Cin+ci,
// zero padding of the image and of the columns Kp > 9*Cin) times the packed weights; its input
// gradient is the GEMM with the transposed weights followed by the col2im gather, its weight
// gradient the GEMM of the transposed output gradient with the transposed im2col.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "../../include/strideacc.h"
#include "helpers.h"

namespace {

int fail_n(int code, const char* msg) {
    sa::set_last_error(msg);
    return code;
}

#define CKN(x)                                                                    \
    do {                                                                          \
        cudaError_t e_ = (x);                                                     \
        if (e_ != cudaSuccess) return fail_n(SA_E_CUDA, cudaGetErrorString(e_)); \
    } while (0)

int nblocks(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152 * 32)); }

#define GRID_LOOP(q, n) \
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < (n); q += (long long)gridDim.x * blockDim.x)

__global__ void k_im2col(const float* __restrict__ x, int ldx, int B, int H, int W, int Cin, __nv_bfloat16* col,
                         int Kp) {
    const long long P = (long long)B * H * W;
    GRID_LOOP(q, P * Kp) {
        const long long p = q / Kp;
        const int k = (int)(q - p * Kp);
        float v = 0.f;
        if (k < 9 * Cin) {
            const int tap = k / Cin, ci = k - tap * Cin;
            const int ky = tap / 3, kx = tap - ky * 3;
            const int b = (int)(p / ((long long)H * W));
            const int r = (int)(p - (long long)b * H * W);
            const int y = r / W + ky - 1, xx = r % W + kx - 1;
            if (y >= 0 && y < H && xx >= 0 && xx < W) v = x[((long long)b * H * W + (long long)y * W + xx) * ldx + ci];
        }
        col[q] = __float2bfloat16_rn(v);
    }
}

// dx[p][ci] (= or +=) sum over taps of dcol[p'][tap*Cin+ci], p' the pixel whose tap reads p.
__global__ void k_col2im(const float* __restrict__ dcol, int Kp, int B, int H, int W, int Cin, float* dx, int ldx,
                         int accumulate) {
    const long long P = (long long)B * H * W;
    GRID_LOOP(q, P * Cin) {
        const long long p = q / Cin;
        const int ci = (int)(q - p * Cin);
        const int b = (int)(p / ((long long)H * W));
        const int r = (int)(p - (long long)b * H * W);
        const int y = r / W, xx = r % W;
        float s = 0.f;
        for (int ky = 0; ky < 3; ky++)
            for (int kx = 0; kx < 3; kx++) {
                const int yo = y - ky + 1, xo = xx - kx + 1;  // output pixel whose tap (ky,kx) reads (y,xx)
                if (yo >= 0 && yo < H && xo >= 0 && xo < W)
                    s += dcol[((long long)b * H * W + (long long)yo * W + xo) * Kp + (ky * 3 + kx) * Cin + ci];
            }
        float* d = dx + p * ldx + ci;
        *d = accumulate ? *d + s : s;
    }
}

// out[c][r] = in[r][c] for r < R, c < C (bf16), rows R..Rp-1 of the output zero.
__global__ void k_transpose_bf16(const __nv_bfloat16* __restrict__ in, int ldi, int R, int C,
                                 __nv_bfloat16* __restrict__ out, int ldo, int Cp) {
    __shared__ __nv_bfloat16 tile[32][34];
    const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int r = r0 + k, c = c0 + threadIdx.x;
        tile[k][threadIdx.x] = (r < R && c < C) ? in[(long long)r * ldi + c] : __float2bfloat16_rn(0.f);
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int c = c0 + k, r = r0 + threadIdx.x;
        if (c < Cp && r < R) out[(long long)c * ldo + r] = tile[threadIdx.x][k];
    }
}

__global__ void k_to_bf16(const float* __restrict__ x, int ldx, long long rows, int C, __nv_bfloat16* y, int ldy) {
    GRID_LOOP(q, rows * C) {
        const long long r = q / C;
        const int c = (int)(q - r * C);
        y[r * ldy + c] = __float2bfloat16_rn(x[r * ldx + c]);
    }
}

__global__ void k_relu_bwd(float* dy, int ldd, const float* __restrict__ y, int ldy, long long rows, int C) {
    GRID_LOOP(q, rows * C) {
        const long long r = q / C;
        const int c = (int)(q - r * C);
        if (!(y[r * ldy + c] > 0.f)) dy[r * ldd + c] = 0.f;
    }
}

// db[c] = sum over rows of dy[r][c] (FP64 partials, one atomic per block and channel block).
// Bias gradient in two fixed-order stages (a reproducible sum): block b of the first sums rows
// b*8 + y, advancing by gridDim.x * 8, into part[b][c]; the second sums the parts in block order.
constexpr int kBiasBlocks = 128;
__global__ void k_bias_grad(const float* __restrict__ dy, int ldd, long long rows, int C, double* part) {
    const int c = blockIdx.y * 32 + threadIdx.x;
    double s = 0.0;
    if (c < C)
        for (long long r = blockIdx.x * (long long)blockDim.y + threadIdx.y; r < rows; r += (long long)gridDim.x * blockDim.y)
            s += dy[r * ldd + c];
    __shared__ double sh[8][33];
    sh[threadIdx.y][threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.y == 0 && c < C) {
        double t = 0.0;
        for (int k = 0; k < (int)blockDim.y; k++) t += sh[k][threadIdx.x];
        part[(long long)blockIdx.x * C + c] = t;
    }
}
__global__ void k_bias_sum(const double* __restrict__ part, int nparts, int C, float* db) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    double t = 0.0;
    for (int b = 0; b < nparts; b++) t += part[(long long)b * C + c];
    db[c] = (float)t;
}
__global__ void k_sum_slabs(const float* __restrict__ in, long long slab, int nz, float* out, long long n,
                            int accumulate) {
    GRID_LOOP(i, n) {
        float t = in[i];
        for (int z = 1; z < nz; z++) t += in[z * slab + i];
        out[i] = accumulate ? out[i] + t : t;
    }
}

__global__ void k_maxpool(const float* __restrict__ x, int ldx, int B, int H, int W, int C, float* y, int ldy) {
    const int Ho = H / 2, Wo = W / 2;
    GRID_LOOP(q, (long long)B * Ho * Wo * C) {
        const long long p = q / C;
        const int c = (int)(q - p * C);
        const int b = (int)(p / ((long long)Ho * Wo));
        const int r = (int)(p - (long long)b * Ho * Wo);
        const int yo = r / Wo, xo = r % Wo;
        const long long base = (long long)b * H * W + (long long)(2 * yo) * W + 2 * xo;
        const float a = x[base * ldx + c], bb = x[(base + 1) * ldx + c], cc = x[(base + W) * ldx + c],
                    d = x[(base + W + 1) * ldx + c];
        y[p * ldy + c] = fmaxf(fmaxf(a, bb), fmaxf(cc, d));
    }
}

// the gradient of each 2x2 window goes to its first maximal element (row-major order)
__global__ void k_maxpool_bwd(const float* __restrict__ x, int ldx, const float* __restrict__ dy, int ldd, int B,
                              int H, int W, int C, float* dx, int lddx, int accumulate) {
    const int Ho = H / 2, Wo = W / 2;
    GRID_LOOP(q, (long long)B * Ho * Wo * C) {
        const long long p = q / C;
        const int c = (int)(q - p * C);
        const int b = (int)(p / ((long long)Ho * Wo));
        const int r = (int)(p - (long long)b * Ho * Wo);
        const int yo = r / Wo, xo = r % Wo;
        const long long base = (long long)b * H * W + (long long)(2 * yo) * W + 2 * xo;
        const long long idx[4] = {base, base + 1, base + W, base + W + 1};
        int best = 0;
        float bv = x[idx[0] * ldx + c];
        for (int k = 1; k < 4; k++) {
            const float v = x[idx[k] * ldx + c];
            if (v > bv) {
                bv = v;
                best = k;
            }
        }
        const float g = dy[p * ldd + c];
        for (int k = 0; k < 4; k++) {
            float* d = dx + idx[k] * lddx + c;
            const float v = k == best ? g : 0.f;
            *d = accumulate ? *d + v : v;
        }
    }
}

// nearest upsampling x2: y[b][y][x] = x[b][y/2][x/2] (H, W of the output)
__global__ void k_upsample(const float* __restrict__ x, int ldx, int B, int H, int W, int C, float* y, int ldy) {
    GRID_LOOP(q, (long long)B * H * W * C) {
        const long long p = q / C;
        const int c = (int)(q - p * C);
        const int b = (int)(p / ((long long)H * W));
        const int r = (int)(p - (long long)b * H * W);
        const int yy = r / W, xx = r % W;
        y[p * ldy + c] = x[((long long)b * (H / 2) * (W / 2) + (long long)(yy / 2) * (W / 2) + xx / 2) * ldx + c];
    }
}

__global__ void k_upsample_bwd(const float* __restrict__ dy, int ldd, int B, int H, int W, int C, float* dx,
                               int lddx) {
    const int Hi = H / 2, Wi = W / 2;
    GRID_LOOP(q, (long long)B * Hi * Wi * C) {
        const long long p = q / C;
        const int c = (int)(q - p * C);
        const int b = (int)(p / ((long long)Hi * Wi));
        const int r = (int)(p - (long long)b * Hi * Wi);
        const int yi = r / Wi, xi = r % Wi;
        const long long base = (long long)b * H * W + (long long)(2 * yi) * W + 2 * xi;
        dx[p * lddx + c] = dy[base * ldd + c] + dy[(base + 1) * ldd + c] + dy[(base + W) * ldd + c] +
                           dy[(base + W + 1) * ldd + c];
    }
}

// dst[r][c] (= or +=) src[r][c] for c < C (channel slices of NHWC tensors)
__global__ void k_copy_ch(const float* __restrict__ src, int lds, long long rows, int C, float* dst, int ldd,
                          int accumulate) {
    GRID_LOOP(q, rows * C) {
        const long long r = q / C;
        const int c = (int)(q - r * C);
        const float v = src[r * lds + c];
        float* d = dst + r * ldd + c;
        *d = accumulate ? *d + v : v;
    }
}

// W fp32 [Cout][Kr] -> Wb bf16 [Coutp][Kp] and Wt bf16 [Kp][Coutp] (zero padded)
__global__ void k_pack_w(const float* __restrict__ w, int Cout, int Kr, __nv_bfloat16* wb, __nv_bfloat16* wt, int Coutp,
                         int Kp) {
    GRID_LOOP(q, (long long)Coutp * Kp) {
        const int o = (int)(q / Kp), k = (int)(q - (long long)o * Kp);
        const float v = (o < Cout && k < Kr) ? w[(long long)o * Kr + k] : 0.f;
        const __nv_bfloat16 b = __float2bfloat16_rn(v);
        wb[(long long)o * Kp + k] = b;
        wt[(long long)k * Coutp + o] = b;
    }
}

__global__ void k_adam(float* w, const float* __restrict__ g, float* m, float* v, long long n, float lr, float b1,
                       float b2, float eps, float c1, float c2) {
    GRID_LOOP(q, n) {
        const float gg = g[q];
        const float mm = b1 * m[q] + (1.f - b1) * gg;
        const float vv = b2 * v[q] + (1.f - b2) * gg * gg;
        m[q] = mm;
        v[q] = vv;
        w[q] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
    }
}

// The same update with the step read on the device (a captured training step): bias corrections
// c12[2 (step - 1)], c12[2 (step - 1) + 1], the step clamped to the table.
__global__ void k_adam_dev(float* w, const float* __restrict__ g, float* m, float* v, long long n, float lr, float b1,
                           float b2, float eps, const float* __restrict__ c12, int nsteps, const int* step) {
    const int k = min(max(*step, 1), nsteps) - 1;
    const float c1 = c12[2 * k], c2 = c12[2 * k + 1];
    GRID_LOOP(q, n) {
        const float gg = g[q];
        const float mm = b1 * m[q] + (1.f - b1) * gg;
        const float vv = b2 * v[q] + (1.f - b2) * gg * gg;
        m[q] = mm;
        v[q] = vv;
        w[q] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
    }
}

// loss += sum (out - t)^2 / n (FP64), dout = 2 (out - t) / n; out has channel stride ldo
__global__ void k_mse(const float* __restrict__ out, int ldo, const float* __restrict__ t, long long n, float* dout,
                      int ldd, double* loss) {
    double s = 0.0;
    GRID_LOOP(q, n) {
        const float d = out[q * ldo] - t[q];
        s += (double)d * d;
        dout[q * ldd] = 2.f * d / (float)n;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, s / (double)n);
}

}  // namespace

extern "C" {

int sa_nn_im2col(const float* x, int ldx, int B, int H, int W, int Cin, void* col, int Kp, void* stream) {
    if (!x || !col || B < 1 || H < 1 || W < 1 || Cin < 1 || Kp < 9 * Cin || ldx < Cin)
        return fail_n(SA_E_INVALID, "sa_nn_im2col: bad arguments");
    const long long n = (long long)B * H * W * Kp;
    k_im2col<<<nblocks(n), 256, 0, (cudaStream_t)stream>>>(x, ldx, B, H, W, Cin, (__nv_bfloat16*)col, Kp);
    CKN(cudaGetLastError());
    return SA_OK;
}

int sa_nn_col2im(const float* dcol, int Kp, int B, int H, int W, int Cin, float* dx, int ldx, int accumulate,
                 void* stream) {
    if (!dcol || !dx || B < 1 || H < 1 || W < 1 || Cin < 1 || Kp < 9 * Cin || ldx < Cin)
        return fail_n(SA_E_INVALID, "sa_nn_col2im: bad arguments");
    const long long n = (long long)B * H * W * Cin;
    k_col2im<<<nblocks(n), 256, 0, (cudaStream_t)stream>>>(dcol, Kp, B, H, W, Cin, dx, ldx, accumulate);
    CKN(cudaGetLastError());
    return SA_OK;
}

int sa_nn_transpose_bf16(const void* in, int ldi, int R, int C, void* out, int ldo, int Cp, void* stream) {
    if (!in || !out || R < 1 || C < 1 || Cp < C || ldi < C || ldo < R)
        return fail_n(SA_E_INVALID, "sa_nn_transpose_bf16: bad arguments");
    const dim3 grid((R + 31) / 32, (Cp + 31) / 32);
    k_transpose_bf16<<<grid, dim3(32, 8), 0, (cudaStream_t)stream>>>((const __nv_bfloat16*)in, ldi, R, C,
                                                                     (__nv_bfloat16*)out, ldo, Cp);
    CKN(cudaGetLastError());
    return SA_OK;
}

int sa_nn_to_bf16(const float* x, int ldx, long long rows, int C, void* y, int ldy, void* stream) {
    if (!x || !y || rows < 0 || C < 1) return fail_n(SA_E_INVALID, "sa_nn_to_bf16: bad arguments");
    if (rows == 0) return SA_OK;
    k_to_bf16<<<nblocks(rows * C), 256, 0, (cudaStream_t)stream>>>(x, ldx, rows, C, (__nv_bfloat16*)y, ldy);
    CKN(cudaGetLastError());
    return SA_OK;
}

int sa_nn_relu_bwd(float* dy, int ldd, const float* y, int ldy, long long rows, int C, void* stream) {
    if (!dy || !y || rows < 0 || C < 1) return fail_n(SA_E_INVALID, "sa_nn_relu_bwd: bad arguments");
    if (rows == 0) return SA_OK;
    k_relu_bwd<<<nblocks(rows * C), 256, 0, (cudaStream_t)stream>>>(dy, ldd, y, ldy, rows, C);
    CKN(cudaGetLastError());
    return SA_OK;
}

int sa_nn_bias_grad(const float* dy, int ldd, long long rows, int C, float* db, double* scratch, void* stream) {
    if (!dy || !db || !scratch || rows < 1 || C < 1) return fail_n(SA_E_INVALID, "sa_nn_bias_grad: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    const int nb = (int)std::min<long long>((rows + 7) / 8, kBiasBlocks);
    k_bias_grad<<<dim3(nb, (C + 31) / 32), dim3(32, 8), 0, s>>>(dy, ldd, rows, C, scratch);
    k_bias_sum<<<(C + 127) / 128, 128, 0, s>>>(scratch, nb, C, db);
    CKN(cudaGetLastError());
    return SA_OK;
}

int sa_nn_sum_slabs(const float* in, long long slab, int n_slabs, float* out, long long n, int accumulate,
                    void* stream) {
    if (!in || !out || n_slabs < 1 || n < 0 || slab < n) return fail_n(SA_E_INVALID, "sa_nn_sum_slabs: bad arguments");
    if (n == 0) return SA_OK;
    k_sum_slabs<<<nblocks(n), 256, 0, (cudaStream_t)stream>>>(in, slab, n_slabs, out, n, accumulate);
    CKN(cudaGetLastError());
    return SA_OK;
}

int sa_nn_maxpool(const float* x, int ldx, int B, int H, int W, int C, float* y, int ldy, void* stream) {
    if (!x || !y || (H & 1) || (W & 1) || C < 1) return fail_n(SA_E_INVALID, "sa_nn_maxpool: bad arguments");
    k_maxpool<<<nblocks((long long)B * H * W * C / 4), 256, 0, (cudaStream_t)stream>>>(x, ldx, B, H, W, C, y, ldy);
    CKN(cudaGetLastError());
    return SA_OK;
}

int sa_nn_maxpool_bwd(const float* x, int ldx, const float* dy, int ldd, int B, int H, int W, int C, float* dx,
                      int lddx, int accumulate, void* stream) {
    if (!x || !dy || !dx || (H & 1) || (W & 1) || C < 1) return fail_n(SA_E_INVALID, "sa_nn_maxpool_bwd: bad arguments");
    k_maxpool_bwd<<<nblocks((long long)B * H * W * C / 4), 256, 0, (cudaStream_t)stream>>>(x, ldx, dy, ldd, B, H, W, C,
                                                                                          dx, lddx, accumulate);
    CKN(cudaGetLastError());
    return SA_OK;
}

int sa_nn_upsample(const float* x, int ldx, int B, int H, int W, int C, float* y, int ldy, void* stream) {
    if (!x || !y || (H & 1) || (W & 1) || C < 1) return fail_n(SA_E_INVALID, "sa_nn_upsample: bad arguments");
    k_upsample<<<nblocks((long long)B * H * W * C), 256, 0, (cudaStream_t)stream>>>(x, ldx, B, H, W, C, y, ldy);
    CKN(cudaGetLastError());
    return SA_OK;
}

int sa_nn_upsample_bwd(const float* dy, int ldd, int B, int H, int W, int C, float* dx, int lddx, void* stream) {
    if (!dy || !dx || (H & 1) || (W & 1) || C < 1) return fail_n(SA_E_INVALID, "sa_nn_upsample_bwd: bad arguments");
    k_upsample_bwd<<<nblocks((long long)B * H * W * C / 4), 256, 0, (cudaStream_t)stream>>>(dy, ldd, B, H, W, C, dx,
                                                                                            lddx);
    CKN(cudaGetLastError());
    return SA_OK;
}

int sa_nn_copy_channels(const float* src, int lds, long long rows, int C, float* dst, int ldd, int accumulate,
                        void* stream) {
    if (!src || !dst || rows < 0 || C < 1) return fail_n(SA_E_INVALID, "sa_nn_copy_channels: bad arguments");
    if (rows == 0) return SA_OK;
    k_copy_ch<<<nblocks(rows * C), 256, 0, (cudaStream_t)stream>>>(src, lds, rows, C, dst, ldd, accumulate);
    CKN(cudaGetLastError());
    return SA_OK;
}

int sa_nn_pack_weights(const float* w, int Cout, int Kr, void* wb, void* wt, int Coutp, int Kp, void* stream) {
    if (!w || !wb || !wt || Coutp < Cout || Kp < Kr) return fail_n(SA_E_INVALID, "sa_nn_pack_weights: bad arguments");
    k_pack_w<<<nblocks((long long)Coutp * Kp), 256, 0, (cudaStream_t)stream>>>(w, Cout, Kr, (__nv_bfloat16*)wb,
                                                                              (__nv_bfloat16*)wt, Coutp, Kp);
    CKN(cudaGetLastError());
    return SA_OK;
}

int sa_nn_adam(float* w, const float* g, float* m, float* v, long long n, float lr, float b1, float b2, float eps,
               int step, void* stream) {
    if (!w || !g || !m || !v || n < 0 || step < 1) return fail_n(SA_E_INVALID, "sa_nn_adam: bad arguments");
    if (n == 0) return SA_OK;
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    k_adam<<<nblocks(n), 256, 0, (cudaStream_t)stream>>>(w, g, m, v, n, lr, b1, b2, eps, c1, c2);
    CKN(cudaGetLastError());
    return SA_OK;
}

int sa_nn_adam_corrections(float b1, float b2, int nsteps, float* c12) {
    if (!c12 || nsteps < 1) return fail_n(SA_E_INVALID, "sa_nn_adam_corrections: bad arguments");
    std::vector<float> h(2 * (size_t)nsteps);
    for (int k = 0; k < nsteps; k++) {  // as sa_nn_adam forms them
        h[2 * k] = 1.f - powf(b1, (float)(k + 1));
        h[2 * k + 1] = 1.f - powf(b2, (float)(k + 1));
    }
    CKN(cudaMemcpy(c12, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
    return SA_OK;
}

int sa_nn_adam_dev(float* w, const float* g, float* m, float* v, long long n, float lr, float b1, float b2, float eps,
                   const float* c12, int nsteps, const int* step, void* stream) {
    if (!w || !g || !m || !v || !c12 || !step || n < 0 || nsteps < 1)
        return fail_n(SA_E_INVALID, "sa_nn_adam_dev: bad arguments");
    if (n == 0) return SA_OK;
    k_adam_dev<<<nblocks(n), 256, 0, (cudaStream_t)stream>>>(w, g, m, v, n, lr, b1, b2, eps, c12, nsteps, step);
    CKN(cudaGetLastError());
    return SA_OK;
}

int sa_nn_mse(const float* out, int ldo, const float* target, long long n, float* dout, int ldd, double* loss,
              void* stream) {
    if (!out || !target || !dout || !loss || n < 1) return fail_n(SA_E_INVALID, "sa_nn_mse: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    CKN(cudaMemsetAsync(loss, 0, sizeof(double), s));
    k_mse<<<nblocks(n), 256, 0, s>>>(out, ldo, target, n, dout, ldd, loss);
    CKN(cudaGetLastError());
    return SA_OK;
}

}  // extern "C"

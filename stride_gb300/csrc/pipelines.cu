// Trace and field processing on the GPU: the steps of Stride's optimisation pipelines that sit on
// either side of every gradient (stride/optimisation/pipelines/default_pipelines.py).
//
//  traces (rows = traces, [n][nt] row-major as Stride's Traces.extended_data):
//   * check_traces: per-trace NaN/inf flags, optional zeroing (steps/check_traces.py:44-78)
//   * filter_traces: cascaded second-order sections, direct form II transposed, FP64 state as
//     scipy.signal.sosfilt (utils/filters.py:14-170), and the cosine FIR lowpass
//     (utils/filters.py:400-465); the adjoint runs the filter on the time-reversed trace
//   * norm_per_shot: divide each shot's traces by sqrt(sum x^2 / n_traces) + 1e-31
//     (steps/norm_traces.py:43-69)
//   * mute_traces: modelled *= cosine-lowpassed (observed != 0) (steps/mute_traces.py:25-57)
//  fields ([nx][ny] or [nx][ny][nz], row-major):
//   * mask_field / clip / gradient step: elementwise (steps/mask_field.py, steps/clip.py,
//     optimisers/optimiser.py:273-298)
//   * smooth_field / preconditioner smoothing: separable Gaussian, 'nearest' or 'reflect'
//     borders as scipy.ndimage.gaussian_filter (steps/smooth_field.py:27-47, problem/data.py:411-446)
//   * norm_field: min / max / max |x| reduction and scaling (steps/norm_field.py:24-52)
//   * apply_prec: sum |prec| reduction, grad /= prec * factor + 1 (problem/data.py:411-446)
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/strideacc.h"
#include "helpers.h"

namespace {

int fail_p(int code, const char* msg) {
    sa::set_last_error(msg);
    return code;
}

#define CKP(x)                                                              \
    do {                                                                    \
        cudaError_t e_ = (x);                                               \
        if (e_ != cudaSuccess) return fail_p(SA_E_CUDA, cudaGetErrorString(e_)); \
    } while (0)

constexpr int kMaxSections = 32;
constexpr int kMaxTaps = 1025;

struct Sos {
    double c[kMaxSections][5];  // b0 b1 b2 a1 a2 (a0 = 1)
    int n;
};

// One thread per trace; the time loop carries two FP64 state values per section.
__global__ void k_sosfilt(const float* __restrict__ in, float* __restrict__ out, int n, int nt, Sos sos,
                          int reverse) {
    const int tr = blockIdx.x * blockDim.x + threadIdx.x;
    if (tr >= n) return;
    double z0[kMaxSections], z1[kMaxSections];
    for (int s = 0; s < sos.n; s++) z0[s] = z1[s] = 0.0;
    const float* x = in + (long long)tr * nt;
    float* y = out + (long long)tr * nt;
    for (int k = 0; k < nt; k++) {
        const int t = reverse ? nt - 1 - k : k;
        double v = x[t];
        for (int s = 0; s < sos.n; s++) {
            const double* c = sos.c[s];
            const double w = c[0] * v + z0[s];
            z0[s] = c[1] * v - c[3] * w + z1[s];
            z1[s] = c[2] * v - c[4] * w;
            v = w;
        }
        y[t] = (float)v;
    }
}

// out[t] = sum_k taps[k] x[t + k - c] (zero outside [0, nt)); reverse: the same on the
// time-reversed trace, i.e. out[t] = sum_k taps[k] x[t - k + c].
__global__ void k_fir(const float* __restrict__ in, float* __restrict__ out, int n, int nt,
                      const double* __restrict__ taps, int ntaps, int c, int reverse) {
    const long long total = (long long)n * nt;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const long long tr = q / nt;
        const int t = (int)(q - tr * nt);
        const float* x = in + tr * nt;
        double acc = 0.0;
        for (int k = 0; k < ntaps; k++) {
            const int u = reverse ? t - k + c : t + k - c;
            if (u >= 0 && u < nt) acc += taps[k] * (double)x[u];
        }
        out[q] = (float)acc;
    }
}

__global__ void k_flags(const float* __restrict__ x, int n, int nt, int* flags) {
    const long long total = (long long)n * nt;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x)
        if (!isfinite(x[q])) flags[q / nt] = 1;
}

__global__ void k_zero_rows(float* x, int n, int nt, const int* flags) {
    const long long total = (long long)n * nt;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x)
        if (flags[q / nt]) x[q] = 0.f;
}

// Sum of squares per shot (CSR trace offsets): FP64 partial sums, one atomic per block and shot.
__global__ void k_shot_sumsq(const float* __restrict__ x, const int* __restrict__ off, int n_shots, int nt,
                             double* sums) {
    const int shot = blockIdx.y;
    const long long b = (long long)off[shot] * nt, e = (long long)off[shot + 1] * nt;
    double acc = 0.0;
    for (long long q = b + blockIdx.x * (long long)blockDim.x + threadIdx.x; q < e;
         q += (long long)gridDim.x * blockDim.x) {
        const double v = x[q];
        acc += v * v;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    __shared__ double part[32];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += part[w];
        atomicAdd(sums + shot, s);
    }
}

__global__ void k_shot_scale(const float* __restrict__ in, float* __restrict__ out, const int* __restrict__ off,
                             int n_shots, int nt, const double* __restrict__ sums) {
    const int shot = blockIdx.y;
    const int nr = off[shot + 1] - off[shot];
    const long long b = (long long)off[shot] * nt, e = (long long)off[shot + 1] * nt;
    const float norm = (float)((nr > 0 ? sqrt(sums[shot] / nr) : 0.0) + 1e-31);
    for (long long q = b + blockIdx.x * (long long)blockDim.x + threadIdx.x; q < e;
         q += (long long)gridDim.x * blockDim.x)
        out[q] = __fdiv_rn(in[q], norm);
}

// modelled * lowpass(observed != 0), the lowpass centred (zero phase) with FP32 mask values.
__global__ void k_mute(const float* __restrict__ mod, const float* __restrict__ obs, float* __restrict__ out, int n,
                       int nt, const double* __restrict__ taps, int ntaps) {
    const long long total = (long long)n * nt;
    const int c = ntaps / 2;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const long long tr = q / nt;
        const int t = (int)(q - tr * nt);
        const float* o = obs + tr * nt;
        double m = 0.0;
        for (int k = 0; k < ntaps; k++) {
            const int u = t + k - c;
            if (u >= 0 && u < nt && o[u] != 0.f) m += taps[k];
        }
        out[q] = (float)(m * (double)mod[q]);
    }
}

// ---- fields ----------------------------------------------------------------------------------

__global__ void k_mul(float* x, const float* __restrict__ m, long long n) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        x[q] *= m[q];
}

__global__ void k_clip(float* x, long long n, float lo, float hi, int has_lo, int has_hi) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        float v = x[q];
        if (has_lo) v = fmaxf(v, lo);
        if (has_hi) v = fminf(v, hi);
        x[q] = v;
    }
}

__global__ void k_axpy(float* x, const float* __restrict__ d, long long n, float a) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        x[q] = x[q] + a * d[q];
}

__global__ void k_scale(float* x, long long n, double a) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        x[q] = (float)((double)x[q] * a);
}

// Order-preserving map of a float to an unsigned int (for atomic min/max).
__device__ __host__ inline unsigned fkey(float v) {
    unsigned b;
    memcpy(&b, &v, 4);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __host__ inline float funkey(unsigned k) {
    const unsigned b = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    float v;
    memcpy(&v, &b, 4);
    return v;
}

struct Stats {
    unsigned mn, mx, amx, pad;
    double sum_abs;
};

// min, max, max |x| and sum |x| (FP64) of an array.
__global__ void k_stats(const float* __restrict__ x, long long n, Stats* st) {
    float mn = INFINITY, mx = -INFINITY, amx = 0.f;
    double s = 0.0;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        const float v = x[q];
        mn = fminf(mn, v);
        mx = fmaxf(mx, v);
        amx = fmaxf(amx, fabsf(v));
        s += fabsf(v);
    }
    for (int o = 16; o > 0; o >>= 1) {
        mn = fminf(mn, __shfl_down_sync(0xffffffffu, mn, o));
        mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
        amx = fmaxf(amx, __shfl_down_sync(0xffffffffu, amx, o));
        s += __shfl_down_sync(0xffffffffu, s, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&st->mn, fkey(mn));
        atomicMax(&st->mx, fkey(mx));
        atomicMax(&st->amx, fkey(amx));
        atomicAdd(&st->sum_abs, s);
    }
}

// vp <- 1 / (1 / vp - step * direction): a gradient step in slowness (optimisers/optimiser.py:273-298
// with the slowness transform of the vp variable).
__global__ void k_slowness_step(float* vp, const float* __restrict__ d, long long n, float step) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        const float s = __fsub_rn(__fdiv_rn(1.f, vp[q]), __fmul_rn(step, d[q]));
        vp[q] = __fdiv_rn(1.f, s);
    }
}

// One axis of a separable correlation with an odd FP64 kernel (radius r) along `axis` of a
// [n0][n1][n2] array; border 0: 'nearest' (edge value), 1: 'reflect' (d c b a | a b c d).
__global__ void k_sep(const float* __restrict__ in, float* __restrict__ out, int n0, int n1, int n2, int axis,
                      const double* __restrict__ w, int r, int border) {
    const long long total = (long long)n0 * n1 * n2;
    const int len = axis == 0 ? n0 : (axis == 1 ? n1 : n2);
    const long long stride = axis == 0 ? (long long)n1 * n2 : (axis == 1 ? n2 : 1);
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const int i = (int)((q / stride) % len);
        const long long base = q - (long long)i * stride;
        double acc = 0.0;
        for (int k = -r; k <= r; k++) {
            int u = i + k;
            if (border == 0) {
                u = u < 0 ? 0 : (u >= len ? len - 1 : u);
            } else {
                const int period = 2 * len;
                u = ((u % period) + period) % period;
                if (u >= len) u = period - 1 - u;
            }
            acc += w[k + r] * (double)in[base + (long long)u * stride];
        }
        out[q] = (float)acc;
    }
}

// prec <- prec * factor + 1 (FP64 operations rounded once, as numpy's float32 array times a
// float64 scalar) and grad *= 1 / prec (FP32) where prec is non-zero (problem/data.py:437-444).
__global__ void k_prec(float* grad, float* prec, long long n, double factor) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        const float p = (float)__dadd_rn(__dmul_rn((double)prec[q], factor), 1.0);
        prec[q] = p;
        if (fabsf(p) > 0.f) grad[q] = __fmul_rn(grad[q], __fdiv_rn(1.f, p));
    }
}

int blocks_for(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152 * 32)); }

// Gaussian kernel of scipy.ndimage.gaussian_filter1d (truncate 4): radius int(4 sigma + 0.5).
int gaussian_taps(double sigma, double* w) {
    const int r = (int)(4.0 * sigma + 0.5);
    if (2 * r + 1 > kMaxTaps) return -1;
    double s = 0.0;
    for (int k = -r; k <= r; k++) {
        w[k + r] = std::exp(-0.5 * k * k / (sigma * sigma));
        s += w[k + r];
    }
    for (int k = 0; k <= 2 * r; k++) w[k] /= s;
    return r;
}

}  // namespace

extern "C" {

int sa_traces_sosfilt(const float* in, float* out, int n, int nt, const double* sos, int n_sections, int adjoint,
                      void* stream) {
    if (!in || !out || n < 0 || nt < 0 || !sos || n_sections < 1 || n_sections > kMaxSections)
        return fail_p(SA_E_INVALID, "sa_traces_sosfilt: bad arguments (at most 32 sections)");
    if (n == 0 || nt == 0) return SA_OK;
    Sos s{};
    s.n = n_sections;
    for (int k = 0; k < n_sections; k++) {
        const double a0 = sos[6 * k + 3];
        if (a0 == 0.0) return fail_p(SA_E_INVALID, "sa_traces_sosfilt: a0 of a section is zero");
        s.c[k][0] = sos[6 * k + 0] / a0;
        s.c[k][1] = sos[6 * k + 1] / a0;
        s.c[k][2] = sos[6 * k + 2] / a0;
        s.c[k][3] = sos[6 * k + 4] / a0;
        s.c[k][4] = sos[6 * k + 5] / a0;
    }
    k_sosfilt<<<(n + 63) / 64, 64, 0, (cudaStream_t)stream>>>(in, out, n, nt, s, adjoint ? 1 : 0);
    CKP(cudaGetLastError());
    return SA_OK;
}

int sa_traces_fir(const float* in, float* out, int n, int nt, const double* taps_dev, int ntaps, int center,
                  int adjoint, void* stream) {
    if (!in || !out || in == out || !taps_dev || ntaps < 1 || ntaps > kMaxTaps)
        return fail_p(SA_E_INVALID, "sa_traces_fir: bad arguments (out-of-place, 1..1025 taps)");
    if (n == 0 || nt == 0) return SA_OK;
    k_fir<<<blocks_for((long long)n * nt), 256, 0, (cudaStream_t)stream>>>(in, out, n, nt, taps_dev, ntaps, center,
                                                                          adjoint ? 1 : 0);
    CKP(cudaGetLastError());
    return SA_OK;
}

int sa_traces_check(float* x, int n, int nt, int* flags_dev, int zero_bad, void* stream) {
    if (!x || !flags_dev || n < 0 || nt < 0) return fail_p(SA_E_INVALID, "sa_traces_check: bad arguments");
    if (n == 0) return SA_OK;
    cudaStream_t s = (cudaStream_t)stream;
    CKP(cudaMemsetAsync(flags_dev, 0, n * sizeof(int), s));
    if (nt == 0) return SA_OK;
    k_flags<<<blocks_for((long long)n * nt), 256, 0, s>>>(x, n, nt, flags_dev);
    if (zero_bad) k_zero_rows<<<blocks_for((long long)n * nt), 256, 0, s>>>(x, n, nt, flags_dev);
    CKP(cudaGetLastError());
    return SA_OK;
}

int sa_traces_norm_per_shot(const float* in, float* out, const int* offsets_dev, int n_shots, int nt,
                            double* scratch_dev, void* stream) {
    if (!in || !out || !offsets_dev || !scratch_dev || n_shots < 0 || nt < 0)
        return fail_p(SA_E_INVALID, "sa_traces_norm_per_shot: bad arguments");
    if (n_shots == 0 || nt == 0) return SA_OK;
    cudaStream_t s = (cudaStream_t)stream;
    CKP(cudaMemsetAsync(scratch_dev, 0, n_shots * sizeof(double), s));
    const dim3 grid(64, n_shots);
    k_shot_sumsq<<<grid, 256, 0, s>>>(in, offsets_dev, n_shots, nt, scratch_dev);
    k_shot_scale<<<grid, 256, 0, s>>>(in, out, offsets_dev, n_shots, nt, scratch_dev);
    CKP(cudaGetLastError());
    return SA_OK;
}

int sa_traces_mute(const float* modelled, const float* observed, float* out, int n, int nt, const double* taps_dev,
                   int ntaps, void* stream) {
    if (!modelled || !observed || !out || !taps_dev || ntaps < 1 || ntaps > kMaxTaps || (ntaps & 1) == 0)
        return fail_p(SA_E_INVALID, "sa_traces_mute: bad arguments (odd tap count)");
    if (n == 0 || nt == 0) return SA_OK;
    k_mute<<<blocks_for((long long)n * nt), 256, 0, (cudaStream_t)stream>>>(modelled, observed, out, n, nt, taps_dev,
                                                                           ntaps);
    CKP(cudaGetLastError());
    return SA_OK;
}

int sa_field_mul(float* x, const float* m, long long n, void* stream) {
    if (!x || !m || n < 0) return fail_p(SA_E_INVALID, "sa_field_mul: bad arguments");
    if (n == 0) return SA_OK;
    k_mul<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(x, m, n);
    CKP(cudaGetLastError());
    return SA_OK;
}

int sa_field_clip(float* x, long long n, const float* lo, const float* hi, void* stream) {
    if (!x || n < 0) return fail_p(SA_E_INVALID, "sa_field_clip: bad arguments");
    if (n == 0 || (!lo && !hi)) return SA_OK;
    k_clip<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(x, n, lo ? *lo : 0.f, hi ? *hi : 0.f, lo != nullptr,
                                                           hi != nullptr);
    CKP(cudaGetLastError());
    return SA_OK;
}

int sa_field_axpy(float* x, const float* d, long long n, float a, void* stream) {
    if (!x || !d || n < 0) return fail_p(SA_E_INVALID, "sa_field_axpy: bad arguments");
    if (n == 0) return SA_OK;
    k_axpy<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(x, d, n, a);
    CKP(cudaGetLastError());
    return SA_OK;
}

int sa_field_stats(const float* x, long long n, float* out4, double* sum_abs, void* stream) {
    if (!x || n < 1 || !out4 || !sum_abs) return fail_p(SA_E_INVALID, "sa_field_stats: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    Stats* d = nullptr;
    CKP(cudaMallocAsync((void**)&d, sizeof(Stats), s));
    Stats init{fkey(INFINITY), fkey(-INFINITY), fkey(0.f), 0u, 0.0};
    cudaError_t e = cudaMemcpyAsync(d, &init, sizeof(Stats), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        k_stats<<<blocks_for(n), 256, 0, s>>>(x, n, d);
        e = cudaGetLastError();
    }
    Stats h{};
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, sizeof(Stats), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFreeAsync(d, s);
    CKP(e);
    out4[0] = funkey(h.mn);
    out4[1] = funkey(h.mx);
    out4[2] = funkey(h.amx);
    out4[3] = 0.f;
    *sum_abs = h.sum_abs;
    return SA_OK;
}

int sa_field_slowness_step(float* vp, const float* direction, long long n, float step, void* stream) {
    if (!vp || !direction || n < 0) return fail_p(SA_E_INVALID, "sa_field_slowness_step: bad arguments");
    if (n == 0) return SA_OK;
    k_slowness_step<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(vp, direction, n, step);
    CKP(cudaGetLastError());
    return SA_OK;
}

int sa_field_scale(float* x, long long n, double a, void* stream) {
    if (!x || n < 0) return fail_p(SA_E_INVALID, "sa_field_scale: bad arguments");
    if (n == 0) return SA_OK;
    k_scale<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(x, n, a);
    CKP(cudaGetLastError());
    return SA_OK;
}

int sa_field_gaussian(float* x, int dim, const int* shape, const double* sigma, int border, float* scratch,
                      void* stream) {
    if (!x || !shape || !sigma || !scratch || dim < 1 || dim > 3 || (border != 0 && border != 1))
        return fail_p(SA_E_INVALID, "sa_field_gaussian: bad arguments");
    int n[3] = {1, 1, 1};
    for (int a = 0; a < dim; a++) {
        if (shape[a] < 1) return fail_p(SA_E_INVALID, "sa_field_gaussian: empty axis");
        n[3 - dim + a] = shape[a];
    }
    const long long total = (long long)n[0] * n[1] * n[2];
    cudaStream_t s = (cudaStream_t)stream;
    double* wd = nullptr;
    CKP(cudaMallocAsync((void**)&wd, kMaxTaps * sizeof(double), s));
    std::vector<double> wv(kMaxTaps);
    double* w = wv.data();
    for (int a = 0; a < dim; a++) {
        if (!(sigma[a] > 0)) continue;
        const int r = gaussian_taps(sigma[a], w);
        if (r < 0) {
            cudaFreeAsync(wd, s);
            return fail_p(SA_E_INVALID, "sa_field_gaussian: sigma too large");
        }
        // the taps are staged through pageable memory: the copy completes before the call returns
        const cudaError_t e = cudaMemcpyAsync(wd, w, (2 * r + 1) * sizeof(double), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) {
            cudaFreeAsync(wd, s);
            return fail_p(SA_E_CUDA, cudaGetErrorString(e));
        }
        k_sep<<<blocks_for(total), 256, 0, s>>>(x, scratch, n[0], n[1], n[2], 3 - dim + a, wd, r, border);
        CKP(cudaMemcpyAsync(x, scratch, total * sizeof(float), cudaMemcpyDeviceToDevice, s));
        CKP(cudaStreamSynchronize(s));
    }
    cudaFreeAsync(wd, s);
    CKP(cudaGetLastError());
    return SA_OK;
}

int sa_field_apply_prec(float* grad, float* prec, long long n, double factor, void* stream) {
    if (!grad || !prec || n < 0) return fail_p(SA_E_INVALID, "sa_field_apply_prec: bad arguments");
    if (n == 0) return SA_OK;
    k_prec<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(grad, prec, n, factor);
    CKP(cudaGetLastError());
    return SA_OK;
}

}  // extern "C"

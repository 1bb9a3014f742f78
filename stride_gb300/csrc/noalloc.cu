// sa_forward_2d_noalloc: single-shot 2D forward modelling that allocates no device memory.
//
// Some callers cannot let a library allocate GPU memory: a host application that hands the
// whole device to a memory pool it manages and forbids allocations outside it, or a loop that
// must not pay for cudaMalloc/cudaFree (cudaFree synchronises the device). For them this entry
// point runs the same time-step kernels as sa_forward, but keeps every scratch buffer (the two
// wavefield levels, the intermediate level of OT4, the medium copies and the step passes' form
// of them, the point lists and the time-major traces) in one file-scope __device__ array of
// kScratchBytes. The caller passes the inputs and the output.
//
// Limits and behaviour:
//  * one shot, 2D, extended grid at most kMaxSide x kMaxSide, at most kMaxSrc sources and
//    kMaxRec receivers, and everything must fit in the array; larger requests fail with
//    SA_E_INVALID and a message naming the limit;
//  * every GPU that loads the library holds the array until the process exits;
//  * the array's device address is looked up once per device, with that device current, on
//    the first call made on it: make that first call before any stream capture;
//  * every call shares the array and it keeps the last call's contents (each call clears what
//    must start at zero), so calls that overlap on the GPU (different streams or threads)
//    race: issue them one after another.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/strideacc.h"
#include "common.cuh"
#include "helpers.h"
#include "launch.h"

namespace {

constexpr size_t kScratchBytes = 64u << 20;  // 64 MiB per device
constexpr int kMaxSide = 640;                // extended grid side
constexpr int kMaxSrc = 16;
constexpr int kMaxRec = 1024;
constexpr int kMaxDevices = 64;
constexpr int kMaxCta = 256;                 // strips x row chunks of the launch

__device__ __align__(256) unsigned char g_scratch[kScratchBytes];

std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {};

int err(int code, const char* msg) {
    char buf[256];
    snprintf(buf, sizeof(buf), "sa_forward_2d_noalloc: %s", msg);
    sa::set_last_error(buf);  // read back with sa_last_error
    return code;
}

// Device address of the scratch array for the current device (looked up once per device).
int scratch_address(void** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return err(SA_E_CUDA, "no current CUDA device");
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return err(SA_E_CUDA, "cudaGetSymbolAddress of the scratch array failed");
        }
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return SA_OK;
}

bool on_device(const void* p) {
    cudaPointerAttributes at;
    if (!p || cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// Bump allocator over the scratch array (256-byte aligned pieces).
struct Carve {
    unsigned char* base;
    size_t used = 0;
    template <class T>
    T* take(size_t n) {
        used = (used + 255) & ~size_t(255);
        T* p = reinterpret_cast<T*>(base + used);
        used += n * sizeof(T);
        return p;
    }
};

void damping_ramp(int A, double h, double refl, float* out) {
    for (int e = 0; e < sa::MAX_ABS; e++) out[e] = 0.f;
    if (A <= 0) return;
    double coef = 1.5 * std::log(1.0 / refl);
    coef = A > 15 ? coef / (A * h) : 0.67 / h;
    for (int e = 0; e < A; e++) {
        double pos = std::fabs((A - e - 1) / (double)(A - 1));
        pos = pos - std::sin(2 * M_PI * pos) / (2 * M_PI);
        out[e] = (float)(coef * pos);
    }
}

}  // namespace

extern "C" int sa_forward_2d_noalloc(const sa_desc* desc, const float* vp, const float* rho, const float* alpha,
                                     int n_src, const float* src_xyz, const float* wavelets, int n_rec,
                                     const float* rec_xyz, float* traces, void* stream) {
    if (!desc) return err(SA_E_INVALID, "null description");
    const sa_desc& d = *desc;
    if (d.dim != 2) return err(SA_E_UNSUPPORTED, "only 2D grids");
    const int nx = d.shape[0], ny = d.shape[1], nt = d.nt;
    if (nx < 24 || ny < 24 || nx > kMaxSide || ny > kMaxSide) return err(SA_E_INVALID, "grid side must be 24..640");
    if (nt < 3) return err(SA_E_INVALID, "nt must be at least 3");
    if (n_src < 0 || n_src > kMaxSrc || n_rec < 0 || n_rec > kMaxRec)
        return err(SA_E_INVALID, "at most 16 sources and 1024 receivers");
    if (d.kernel != SA_KERNEL_OT2 && d.kernel != SA_KERNEL_OT4) return err(SA_E_INVALID, "kernel must be OT2 or OT4");
    if (d.density < 0 || d.density > 2) return err(SA_E_INVALID, "density mode");
    if (d.interpolation != SA_INTERP_LINEAR) return err(SA_E_UNSUPPORTED, "linear interpolation only");
    if (d.boundary != SA_BOUNDARY_SPONGE) return err(SA_E_UNSUPPORTED, "sponge boundary only");
    if (!(d.dt > 0) || !(d.spacing[0] > 0) || !(d.spacing[1] > 0)) return err(SA_E_INVALID, "dt and spacing");
    for (int a = 0; a < 2; a++)
        if (d.absorbing[a] < 0 || d.absorbing[a] > sa::MAX_ABS || d.absorbing[a] == 1 || d.absorbing[a] > d.extra[a] ||
            2 * d.absorbing[a] > d.shape[a])
            return err(SA_E_INVALID, "absorbing width");
    if (!vp || (d.density != SA_DENSITY_NONE && !rho) || (d.attenuation && !alpha) || (n_src && !wavelets) ||
        (n_rec && !traces) || (n_src && !src_xyz) || (n_rec && !rec_xyz))
        return err(SA_E_INVALID, "missing input or output pointer");
    const float* dev_in[] = {vp, d.density == SA_DENSITY_VARIABLE ? rho : nullptr, d.attenuation ? alpha : nullptr,
                             n_src ? wavelets : nullptr, n_rec ? traces : nullptr};
    for (const float* q : dev_in)
        if (q && !on_device(q)) return err(SA_E_INVALID, "medium, wavelets and traces must be device pointers");
    if ((n_src && on_device(src_xyz)) || (n_rec && on_device(rec_xyz)))
        return err(SA_E_INVALID, "src_xyz and rec_xyz must be host pointers (they are read on the host)");

    void* sbase = nullptr;
    int rc = scratch_address(&sbase);
    if (rc != SA_OK) return rc;
    cudaStream_t s = (cudaStream_t)stream;

    // ---- layout (one shot = one shot pair with an empty second lane) --------------------
    const int kind = d.density == SA_DENSITY_NONE ? 0 : (d.density == SA_DENSITY_VARIABLE ? 1 : 2);
    const bool ot4 = d.kernel == SA_KERNEL_OT4;
    const int R = kind == 0 ? 5 : 9;
    const int pitch = (ny + 2 + 31) / 32 * 32, pitch_b = (ny + 12 + 31) / 32 * 32;
    int by = 0, NT = 0;  // the fewest column strips (two columns a thread)
    sa::step_strips(ny, (ny + 2 * sa::STEP_MAX_THREADS - 1) / (2 * sa::STEP_MAX_THREADS), &by, &NT);
    const int nstrips = (ny + by - 1) / by;
    const int warps = (NT + 31) / 32;
    int nchunks = std::max(1, std::min((152 * 12 / warps + nstrips - 1) / nstrips, nx / (4 * R)));
    const int chunk_rows = (nx + nchunks - 1) / nchunks;
    nchunks = (nx + chunk_rows - 1) / chunk_rows;
    const int ncta = nchunks * nstrips;
    if (ncta > kMaxCta) return err(SA_E_INVALID, "launch layout exceeds 256 CTAs");

    // ---- carve the scratch array --------------------------------------------------------
    const long long pe = (long long)nx * pitch;  // float2 per level
    const long long guarded = (long long)(nx + 2 * sa::GUARD) * pitch;
    Carve cv{static_cast<unsigned char*>(sbase)};
    float* field[2] = {cv.take<float>(2 * pe), cv.take<float>(2 * pe)};
    float* med_begin = reinterpret_cast<float*>(static_cast<unsigned char*>(sbase) + ((cv.used + 255) & ~size_t(255)));
    float* W = cv.take<float>(guarded);
    float* C1 = cv.take<float>(guarded);
    float* C2 = cv.take<float>(guarded);
    float* C3 = cv.take<float>(guarded);
    float* bxh = kind == 1 ? cv.take<float>((long long)(nx + 9 + 2 * sa::GUARD) * pitch) : nullptr;
    float* byh = kind == 1 ? cv.take<float>((long long)(nx + 2 * sa::GUARD) * pitch_b) : nullptr;
    float* vps = cv.take<float>(pe);
    float* als = cv.take<float>(pe);
    float* buoy = kind == 1 ? cv.take<float>(pe) : nullptr;
    const size_t med_bytes = (size_t)(reinterpret_cast<unsigned char*>(als + pe) - reinterpret_cast<unsigned char*>(med_begin));
    float* src_amp = cv.take<float>((size_t)nt * (n_src ? n_src : 1));
    float* rec_amp = cv.take<float>((size_t)nt * (n_rec ? n_rec : 1));
    long long* tidx = cv.take<long long>((size_t)4 * kMaxSrc);  // source corners grouped by target point
    int* toff = cv.take<int>((size_t)4 * kMaxSrc + 1);
    float* tcoef = cv.take<float>((size_t)4 * kMaxSrc);
    int* tpoint = cv.take<int>((size_t)4 * kMaxSrc);
    sa::Gather* gat = cv.take<sa::Gather>(kMaxRec);
    float* smed = cv.take<float>(sa::step_medium_size(nx, ny));  // the step passes' medium
    float* lbuf = ot4 ? cv.take<float>(2 * pe) : nullptr;          // OT4's intermediate level
    if (cv.used > kScratchBytes) return err(SA_E_INVALID, "grid, traces and lists exceed the 64 MiB scratch array");

    // ---- zero what must start at zero, then the medium ---------------------------------
    if (cudaMemsetAsync(field[0], 0, 2 * pe * sizeof(float), s) != cudaSuccess ||
        cudaMemsetAsync(field[1], 0, 2 * pe * sizeof(float), s) != cudaSuccess ||
        cudaMemsetAsync(med_begin, 0, med_bytes, s) != cudaSuccess ||
        (n_rec && cudaMemsetAsync(rec_amp, 0, (size_t)nt * n_rec * sizeof(float), s) != cudaSuccess) ||
        (lbuf && cudaMemsetAsync(lbuf, 0, 2 * pe * sizeof(float), s) != cudaSuccess))
        return err(SA_E_CUDA, "cudaMemsetAsync on the scratch array failed");
    sa::Sponge sp{};
    sp.a[0] = d.absorbing[0];
    sp.a[1] = d.absorbing[1];
    const int amax = std::max(d.absorbing[0], d.absorbing[1]);
    if (amax > 1) {
        const double refl = std::pow(10.0, -(std::log10((double)amax) - 1) / std::log10(2.0) - 3);
        damping_ramp(d.absorbing[0], d.spacing[0], refl, sp.s[0]);
        damping_ramp(d.absorbing[1], d.spacing[1], refl, sp.s[1]);
    }
    const double db_to_np = 100.0 / (20.0 * 0.43429448190325176);
    const long long g0 = (long long)sa::GUARD * pitch;
    if (sa::medium2d(vp, dev_in[1], dev_in[2], nx, ny, pitch, pitch_b, kind == 1 ? 1 : 0, db_to_np, sp, (float)d.dt,
                     W + g0, vps, als, buoy, bxh ? bxh + (long long)(sa::GUARD + 5) * pitch : nullptr,
                     byh ? byh + (long long)sa::GUARD * pitch_b : nullptr, C1 + g0, C2 + g0, C3 + g0, s) != cudaSuccess)
        return err(SA_E_CUDA, "medium preparation kernel failed");
    if (sa::step_medium2d(W + g0, bxh ? bxh + (long long)(sa::GUARD + 5) * pitch : nullptr,
                          byh ? byh + (long long)sa::GUARD * pitch_b : nullptr, C1 + g0, C2 + g0, C3 + g0, nx, ny, pitch,
                          pitch_b, smed, s) != cudaSuccess)
        return err(SA_E_CUDA, "step medium kernel failed");

    // ---- point lists (host arrays on the stack, copied into the scratch array) -----------
    const double h = std::max(d.spacing[0], d.spacing[1]);
    int sbx[kMaxSrc], sby[kMaxSrc];
    double sfx[kMaxSrc], sfy[kMaxSrc];
    auto locate = [&](const float* xyz, int i, int* bx, int* byy, double* fx, double* fy) -> bool {
        double rel[2];
        int base[2];
        for (int a = 0; a < 2; a++) {
            rel[a] = ((double)xyz[2 * i + a] + d.extra[a] * d.spacing[a]) / d.spacing[a];
            base[a] = (int)std::floor(rel[a]);
            if (!(base[a] >= 0 && base[a] + 1 <= d.shape[a] - 1)) return false;
        }
        *bx = base[0];
        *byy = base[1];
        *fx = rel[0] - base[0];
        *fy = rel[1] - base[1];
        return true;
    };
    for (int i = 0; i < n_src; i++)
        if (!locate(src_xyz, i, &sbx[i], &sby[i], &sfx[i], &sfy[i])) return err(SA_E_INVALID, "source outside the grid");
    // vp at the source corners (the injection scale 2 dt vp / h uses vp at each corner)
    float vpc[4 * kMaxSrc];
    for (int i = 0; i < n_src; i++)
        for (int k = 0; k < 4; k++) {
            const int x = sbx[i] + (k >> 1), y = sby[i] + (k & 1);
            if (cudaMemcpyAsync(&vpc[4 * i + k], vp + (long long)x * ny + y, sizeof(float), cudaMemcpyDeviceToHost, s) !=
                cudaSuccess)
                return err(SA_E_CUDA, "reading vp at the source corners failed");
        }
    if (cudaStreamSynchronize(s) != cudaSuccess) return err(SA_E_CUDA, "stream synchronisation failed");
    // source corners ordered by target point (insertion sort of at most 64 entries), grouped so
    // one thread sums each point's entries in a fixed order
    struct E {
        long long key;
        float coef;
        int point;
    } tmp[4 * kMaxSrc];
    int ninj = 0;
    for (int i = 0; i < n_src; i++)
        for (int k = 0; k < 4; k++) {
            const int cx = k >> 1, cy = k & 1, x = sbx[i] + cx, y = sby[i] + cy;
            const double w = (cx ? sfx[i] : 1 - sfx[i]) * (cy ? sfy[i] : 1 - sfy[i]);
            E v{2 * ((long long)x * pitch + y), (float)(w * 2.0 * d.dt / h * (double)vpc[4 * i + k]), i};
            int b = ninj - 1;
            while (b >= 0 && tmp[b].key > v.key) {
                tmp[b + 1] = tmp[b];
                b--;
            }
            tmp[b + 1] = v;
            ninj++;
        }
    long long htidx[4 * kMaxSrc];
    int htoff[4 * kMaxSrc + 1], htpoint[4 * kMaxSrc];
    float htcoef[4 * kMaxSrc];
    int ntgt = 0;
    for (int e = 0; e < ninj; e++) {
        if (e == 0 || tmp[e].key != tmp[e - 1].key) {
            htidx[ntgt] = tmp[e].key;
            htoff[ntgt++] = e;
        }
        htcoef[e] = tmp[e].coef;
        htpoint[e] = tmp[e].point;
    }
    htoff[ntgt] = ninj;
    static thread_local sa::Gather hg[kMaxRec];
    for (int r = 0; r < n_rec; r++) {
        int bx, byy;
        double fx, fy;
        if (!locate(rec_xyz, r, &bx, &byy, &fx, &fy)) return err(SA_E_INVALID, "receiver outside the grid");
        hg[r] = {bx, byy, r, 0, (float)((1 - fx) * (1 - fy)), (float)((1 - fx) * fy), (float)(fx * (1 - fy)),
                 (float)(fx * fy)};
    }
    if ((ntgt && (cudaMemcpyAsync(tidx, htidx, ntgt * sizeof(long long), cudaMemcpyHostToDevice, s) != cudaSuccess ||
                  cudaMemcpyAsync(toff, htoff, (ntgt + 1) * sizeof(int), cudaMemcpyHostToDevice, s) != cudaSuccess ||
                  cudaMemcpyAsync(tcoef, htcoef, ninj * sizeof(float), cudaMemcpyHostToDevice, s) != cudaSuccess ||
                  cudaMemcpyAsync(tpoint, htpoint, ninj * sizeof(int), cudaMemcpyHostToDevice, s) != cudaSuccess)) ||
        (n_rec && cudaMemcpyAsync(gat, hg, n_rec * sizeof(sa::Gather), cudaMemcpyHostToDevice, s) != cudaSuccess) ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return err(SA_E_CUDA, "copying the point lists failed");

    // ---- time loop ----------------------------------------------------------------------
    if (n_src && sa::transpose(wavelets, n_src, nt, src_amp, s) != cudaSuccess)
        return err(SA_E_CUDA, "wavelet transpose failed");
    sa::Step2D a{};
    a.nx = nx;
    a.ny = ny;
    a.pitch = pitch;
    a.shot_stride = pe;
    a.chunk_rows = chunk_rows;
    a.by = by;
    a.lbuf = lbuf;
    sa::step_medium(a, smed, nx, ny);
    sa::step_weights(a, kind, d.spacing[0], d.spacing[1], d.dt);
    a.f = d.undersampling > 0 ? d.undersampling : 4;
    const dim3 grid(nstrips, nchunks, 1);
    for (int t = 1; t <= nt - 2; t++) {
        a.t = t;
        a.cur = (t & 1) ? field[1] : field[0];
        a.prev = (t & 1) ? field[0] : field[1];
        if (sa::launch_step2d(kind, ot4, NT, grid, s, a) != cudaSuccess) return err(SA_E_CUDA, "step kernel launch failed");
        // p[t+1] += sources at t; rec[t] = interp(p[t+1])
        if (sa::inject_targets2d(a.prev, tidx, toff, tcoef, tpoint, ntgt, src_amp, n_src, t, nullptr, 0, 0, 0, 0.f, s) !=
                cudaSuccess ||
            (n_rec && sa::final_gather2d(a.prev, pe, pitch, gat, n_rec, rec_amp, n_rec, t, s) != cudaSuccess))
            return err(SA_E_CUDA, "source or receiver kernel launch failed");
    }
    if (n_rec && sa::transpose(rec_amp, nt, n_rec, traces, s) != cudaSuccess) return err(SA_E_CUDA, "trace transpose failed");
    return SA_OK;
}

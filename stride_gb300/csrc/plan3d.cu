// 3D plans behind the same C ABI (include/strideacc.h): wavefields of every shot, the medium,
// trilinear source/receiver lists, the undersampled wavefield and per-shot gradient
// accumulators, and the time loops of the forward (iso_acoustic/devito.py:515-581) and of the
// reverse-time adjoint with the vp imaging condition (devito.py:875-920, 985-1043).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/strideacc.h"
#include "fdtd3d.cuh"
#include "helpers.h"
#include "launch.h"
#include "plan3d.h"

namespace sa {

namespace {

int fail3(int code, const char* msg) {
    set_last_error(msg);
    return code;
}

#define CK3(x)                                                                                 \
    do {                                                                                       \
        cudaError_t e_ = (x);                                                                  \
        if (e_ != cudaSuccess) {                                                               \
            char b_[512];                                                                      \
            snprintf(b_, sizeof(b_), "%s: %s", #x, cudaGetErrorString(e_));                    \
            return fail3(SA_E_CUDA, b_);                                                       \
        }                                                                                      \
    } while (0)

template <class T>
int alloc3(T** p, size_t n) {
    if (*p) cudaFree(*p);
    *p = nullptr;
    if (cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return fail3(SA_E_NOMEM, "device allocation failed (3D plan)");
    }
    if (cudaMemset(*p, 0, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return fail3(SA_E_CUDA, "cudaMemset failed");
    return SA_OK;
}

bool dev_ptr(const void* p) {
    cudaPointerAttributes at;
    if (!p || cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

void ramp(int A, double h, double refl, float* out) {
    for (int e = 0; e < MAX_ABS; e++) out[e] = 0.f;
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

// The requested interval (50 by default), unless the checkpoints (ck_levels levels each) and one
// segment's snapshots exceed the byte budget; then the multiple of f nearest to it that fits. When
// no one-level interval fits, two levels (*K2_out > 0): the forward keeps coarse checkpoints every
// K steps, and the adjoint re-runs each coarse segment once to place fine checkpoints every K2
// steps in it (K a multiple of K2), then each fine segment once more for its snapshots. Every
// step is then recomputed at most twice; memory is (nt-2)/K + K/K2 - 1 checkpoints and K2/f
// snapshots. Of the pairs that fit, the largest K2 (fewest restores), then the least memory.
int choose_checkpoints(const sa_desc& d, double level, int* K_out, int* n_out, double ck_levels, int* K2_out) {
    const int f = d.undersampling;
    const int T0 = d.nt - 1 - f;
    int K = d.checkpoint_interval > 0 ? d.checkpoint_interval : 50;
    K = (K + f - 1) / f * f;
    int K2 = 0;
    // checkpoints after steps K, 2K, .. <= nt-2 (the exact adjoint's segments reach that far) and
    // one segment's K/f snapshots
    auto bytes = [&](int k) { return ((d.nt - 2) / k) * ck_levels * level + (k / f) * level; };
    if (d.checkpoint_budget > 0 && bytes(K) > d.checkpoint_budget) {
        int best = -1;
        double least = 1e300;
        for (int k = f; k <= std::max(f, T0); k += f) {
            least = std::min(least, bytes(k));
            if (bytes(k) <= d.checkpoint_budget && (best < 0 || std::abs(k - K) < std::abs(best - K))) best = k;
        }
        if (best < 0) {
            auto bytes2 = [&](int k1, int k2) {
                return ((d.nt - 2) / k1) * ck_levels * level + (k1 / k2 - 1) * ck_levels * level + (k2 / f) * level;
            };
            int b1 = -1, b2 = -1;
            for (int k2 = f; k2 <= std::max(f, T0); k2 += f)
                for (int k1 = 2 * k2; k1 <= std::max(2 * k2, T0 + k2 - 1); k1 += k2) {
                    const double b = bytes2(k1, k2);
                    least = std::min(least, b);
                    if (b <= d.checkpoint_budget && (k2 > b2 || (k2 == b2 && b < bytes2(b1, b2)))) {
                        b1 = k1;
                        b2 = k2;
                    }
                }
            if (b1 < 0) {
                char b[256];
                snprintf(b, sizeof(b), "no checkpoint schedule fits %.0f bytes (at least %.0f needed)",
                         d.checkpoint_budget, least);
                return fail3(SA_E_NOMEM, b);
            }
            best = b1;
            K2 = b2;
        }
        K = best;
    }
    *K_out = K;
    *n_out = (d.nt - 2) / K;
    if (K2_out) *K2_out = K2;
    return SA_OK;
}

struct Plan3D {
    sa_desc d{};
    int nx = 0, ny = 0, nz = 0, zp = 0, zpb = 0, kind = 0;
    bool ot4 = true;
    long long plane = 0, field = 0;  // floats per x plane and per shot
    float *F[2] = {nullptr, nullptr}, *Lbuf = nullptr;
    float *W = nullptr, *C1 = nullptr, *C2 = nullptr, *C3 = nullptr, *bxh = nullptr, *byh = nullptr, *bzh = nullptr;
    float *vp = nullptr, *alpha = nullptr, *buoy = nullptr, *stage = nullptr;
    std::vector<float> vp_host;
    Sponge3 sponge{};
    int n_shots = 0, n_src = 0, n_rec = 0;
    std::vector<int> so, ro;
    std::vector<float> sx, rx;
    // lists (device): shot, base, weights, injection coefficients
    int *s_shot = nullptr, *s_base = nullptr, *r_shot = nullptr, *r_base = nullptr;
    float *s_w = nullptr, *s_coef = nullptr, *r_w = nullptr, *r_coef = nullptr;
    float *src_amp = nullptr, *rec_amp = nullptr, *tstage = nullptr;
    size_t cap_tstage = 0;
    float* snaps = nullptr;
    size_t cap_snaps = 0;
    int n_snap = 0;
    long long snap_stride = 0;
    bool snaps_valid = false, medium_set = false, geometry_set = false;
    // checkpoints (SA_SAVE_CHECKPOINTS): both levels after every ck_K-th step, one segment's
    // recomputed snapshots, the adjoint's own two levels
    float *ckpt = nullptr, *segsnaps = nullptr, *A[2] = {nullptr, nullptr};
    size_t cap_ckpt = 0, cap_segsnaps = 0;
    int ck_K = 0, ck_n = 0;
    // two-level schedule (ck_K2 > 0): fine checkpoints every ck_K2 steps of one coarse segment
    int ck_K2 = 0;
    float *ckpt2 = nullptr, *pml_ck2 = nullptr;
    size_t cap_ckpt2 = 0, cap_pml_ck2 = 0;
    bool ckpt_valid = false;
    float *gradb = nullptr, *precb = nullptr;
    // raw snapshots (SA_SAVE_RAW): held vp/rho terms per shot, rho accumulators, D-b per axis
    bool snaps_raw = false, rho_valid = false;
    float *hold_vp = nullptr, *hold_rho = nullptr, *gradrb = nullptr, *precrb = nullptr, *db[3] = {};
    // wavelet gradient, time-major [nt][n_src]
    float* wgrad = nullptr;
    size_t cap_wgrad = 0;
    // exact gradient (SA_GRAD_EXACT): vp-derivative coefficients of the update, every level of a
    // segment, the W G(.) of a forward and an adjoint level, unit / zero update coefficients
    // (guarded), receiver injection coefficients w C1 W
    float *EA = nullptr, *EB = nullptr, *EC = nullptr, *EG4 = nullptr, *ES = nullptr, *levels = nullptr;
    float *Lu = nullptr, *Lz = nullptr, *ones = nullptr, *zeros = nullptr, *r_xcoef = nullptr;
    size_t cap_levels = 0;
    bool exact_valid = false;
    // wide interpolation (Hicks or sinc): injection entries of the sources [0] and receivers [1], receiver gathers
    bool wide = false;  // a wide sparse-point support (Hicks or sinc)
    int *e_shot[2] = {}, *e_point[2] = {};
    long long* e_idx[2] = {};
    float* e_coef[2] = {};
    float* e_w[2] = {};  // raw support weights (the exact gradient's point terms)
    float* e_xcoef = nullptr;  // receivers' w C1 W (exact gradient)
    int n_ent[2] = {0, 0};
    SupportGather3D* hgat = nullptr;
    SupportGather3D* hgat_src = nullptr;  // sources (Hicks: smoothed): the wavelet gradient's gathers
    // CFS-PML (SA_BOUNDARY_CFS_PML, OT2): profiles per axis and nine auxiliary fields per shot
    bool pml = false;
    float *pml_prof = nullptr, *pml_aux = nullptr;
    // with checkpoints: the forward's auxiliary fields at every checkpoint, and the set the forward
    // recompute advances (the adjoint keeps its own in pml_aux)
    float *pml_ck = nullptr, *pml_aux_f = nullptr;
    size_t cap_pml_ck = 0;
    long long launches = 0;
    int chunk_rows = 0, nchunks = 1, ty0n = 1, tz0n = 1;
    int tile = 0;               // kTiles3d entry of the passes
    bool layout_fixed = false;  // tile and chunks chosen by sa_autotune (kept across geometries)
};

long long plan3d_launches(const Plan3D* p) { return p->launches; }

static void set_tile(Plan3D* p, int tile) {
    p->tile = tile;
    p->ty0n = (p->ny + kTiles3d[tile].ty - 1) / kTiles3d[tile].ty;
    p->tz0n = (p->nz + kTiles3d[tile].tz - 1) / kTiles3d[tile].tz;
}

// x chunks of the passes: enough CTAs for four per SM, each chunk at least 4 R rows deep
static void set_chunks(Plan3D* p, int nchunks) {
    p->chunk_rows = (p->nx + nchunks - 1) / nchunks;
    p->nchunks = (p->nx + p->chunk_rows - 1) / p->chunk_rows;
}
static int default_chunks(const Plan3D* p, int n_shots) {
    const int R = p->kind == 0 ? 5 : 9;
    const int ctas = p->ty0n * p->tz0n * ((n_shots + 1) / 2);
    return std::max(1, std::min((152 * 4 + ctas - 1) / ctas, p->nx / (4 * R)));
}

int plan3d_create(const sa_desc& d, Plan3D** out) {
    *out = nullptr;
    Plan3D* p = new Plan3D();
    p->d = d;
    p->nx = d.shape[0];
    p->ny = d.shape[1];
    p->nz = d.shape[2];
    p->zp = (p->nz + 2 + 31) / 32 * 32;
    p->zpb = (p->nz + 12 + 31) / 32 * 32;
    p->kind = d.density == SA_DENSITY_NONE ? 0 : (d.density == SA_DENSITY_VARIABLE ? 1 : 2);
    p->ot4 = d.kernel == SA_KERNEL_OT4;
    p->wide = d.interpolation != SA_INTERP_LINEAR;
    p->pml = d.boundary == SA_BOUNDARY_CFS_PML;
    p->plane = (long long)p->ny * p->zp;
    p->field = (long long)p->nx * p->plane;
    p->n_snap = (d.nt + d.undersampling) / d.undersampling + 1;
    p->snap_stride = p->field;
    int amax = 0;
    for (int a = 0; a < 3; a++) {
        p->sponge.a[a] = d.absorbing[a];
        amax = std::max(amax, d.absorbing[a]);
    }
    if (amax > 1 && !p->pml) {  // the CFS-PML replaces the sponge: no damping in the update
        const double refl = std::pow(10.0, -(std::log10((double)amax) - 1) / std::log10(2.0) - 3);
        for (int a = 0; a < 3; a++) ramp(d.absorbing[a], d.spacing[a], refl, p->sponge.s[a]);
    }
    const long long G = GUARD;
    const size_t shots = std::max(1, d.max_shots);
    int rc = SA_OK;
    for (int k = 0; k < 2 && rc == SA_OK; k++) rc = alloc3(&p->F[k], shots * p->field);
    if (rc == SA_OK && p->ot4) rc = alloc3(&p->Lbuf, shots * p->field);
    if (rc == SA_OK && p->pml) rc = alloc3(&p->pml_prof, 4 * (size_t)(p->nx + p->ny + p->nz));
    if (rc == SA_OK && p->pml) rc = alloc3(&p->pml_aux, 9 * shots * p->field);
    const size_t guarded = (size_t)(p->nx + 2 * G) * p->plane;
    if (rc == SA_OK) rc = alloc3(&p->W, guarded);
    if (rc == SA_OK) rc = alloc3(&p->C1, guarded);
    if (rc == SA_OK) rc = alloc3(&p->C2, guarded);
    if (rc == SA_OK) rc = alloc3(&p->C3, guarded);
    if (rc == SA_OK) rc = alloc3(&p->vp, (size_t)p->field);
    if (rc == SA_OK) rc = alloc3(&p->alpha, (size_t)p->field);
    if (rc == SA_OK && p->kind >= 1) rc = alloc3(&p->buoy, (size_t)p->field);  // b = 1/rho (rho gradient)
    if (rc == SA_OK && p->kind == 1) {
        if (rc == SA_OK) rc = alloc3(&p->bxh, (size_t)(p->nx + 9 + 2 * G) * p->plane);
        if (rc == SA_OK) rc = alloc3(&p->byh, (size_t)(p->nx + 2 * G) * (p->ny + 12) * p->zp);
        if (rc == SA_OK) rc = alloc3(&p->bzh, (size_t)(p->nx + 2 * G) * p->ny * p->zpb);
    }
    if (rc != SA_OK) {
        plan3d_destroy(p);
        return rc;
    }
    set_tile(p, 0);
    *out = p;
    return SA_OK;
}

void plan3d_destroy(Plan3D* p) {
    if (!p) return;
    float* fb[] = {p->F[0], p->F[1], p->Lbuf, p->W, p->C1, p->C2, p->C3, p->bxh, p->byh, p->bzh, p->vp, p->alpha,
                   p->buoy, p->stage, p->s_w, p->s_coef, p->r_w, p->r_coef, p->src_amp, p->rec_amp, p->tstage,
                   p->snaps, p->gradb, p->precb, p->ckpt, p->segsnaps, p->A[0], p->A[1], p->hold_vp, p->hold_rho,
                   p->gradrb, p->precrb, p->db[0], p->db[1], p->db[2], p->wgrad, p->EA, p->EB, p->EC, p->EG4,
                   p->ES, p->levels, p->Lu, p->Lz, p->ones, p->zeros, p->r_xcoef, p->e_coef[0], p->e_coef[1],
                   p->pml_prof, p->pml_aux, p->pml_ck, p->pml_aux_f, p->ckpt2, p->pml_ck2, p->e_w[0], p->e_w[1], p->e_xcoef};
    for (float* b : fb)
        if (b) cudaFree(b);
    void* vb[] = {p->e_shot[0], p->e_shot[1], p->e_point[0], p->e_point[1], p->e_idx[0], p->e_idx[1], p->hgat,
                  p->hgat_src};
    for (void* b : vb)
        if (b) cudaFree(b);
    int* ib[] = {p->s_shot, p->s_base, p->r_shot, p->r_base};
    for (int* b : ib)
        if (b) cudaFree(b);
    delete p;
}

int plan3d_set_medium(Plan3D* p, const float* vp, const float* rho, const float* alpha) {
    const size_t N = (size_t)p->nx * p->ny * p->nz;
    const float* in[3] = {vp, p->kind >= 1 ? rho : nullptr, p->d.attenuation ? alpha : nullptr};
    const float* dv[3] = {nullptr, nullptr, nullptr};
    for (int k = 0; k < 3; k++) {
        if (!in[k]) continue;
        if (dev_ptr(in[k])) {
            dv[k] = in[k];
        } else {
            if (!p->stage) {
                int rc = alloc3(&p->stage, 3 * N);
                if (rc != SA_OK) return rc;
            }
            CK3(cudaMemcpy(p->stage + k * N, in[k], N * sizeof(float), cudaMemcpyHostToDevice));
            dv[k] = p->stage + k * N;
        }
    }
    const long long g0 = (long long)GUARD * p->plane;
    CK3(medium3d(dv[0], dv[1], dv[2], p->nx, p->ny, p->nz, p->zp, p->zpb, p->kind,
                 100.0 / (20.0 * 0.43429448190325176), p->sponge, (float)p->d.dt, p->W + g0, p->vp, p->alpha, p->buoy,
                 p->bxh ? p->bxh + (long long)(GUARD + 5) * p->plane : nullptr,
                 p->byh ? p->byh + (long long)GUARD * (p->ny + 12) * p->zp : nullptr,
                 p->bzh ? p->bzh + (long long)GUARD * p->ny * p->zpb : nullptr, p->C1 + g0, p->C2 + g0, p->C3 + g0, 0));
    CK3(cudaDeviceSynchronize());
    p->vp_host.resize(N);
    CK3(cudaMemcpy(p->vp_host.data(), dv[0], N * sizeof(float), cudaMemcpyDeviceToHost));
    if (p->pml) {
        float vmax = 0.f;
        for (float v : p->vp_host) vmax = std::max(vmax, v);
        const std::vector<float> prof = pml_profile_tables(p->d, vmax);
        CK3(cudaMemcpy(p->pml_prof, prof.data(), prof.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    p->medium_set = true;
    p->snaps_valid = false;
    p->ckpt_valid = false;
    p->rho_valid = false;
    p->exact_valid = false;
    if (p->geometry_set) return plan3d_set_geometry(p, p->n_shots, p->so.data(), p->sx.data(), p->ro.data(), p->rx.data());
    return SA_OK;
}

// Trilinear corner weights of Devito's linear SparseTimeFunction (common/devito.py:580-653);
// the injection coefficient at a corner carries the reference's scale and vp^k there.
static int build_points(Plan3D* p, int n_shots, const int* off, const float* xyz, double scale, int vp_power,
                        int** d_shot, int** d_base, float** d_w, float** d_coef) {
    const int n = off[n_shots];
    std::vector<int> shot(n), base(3 * n);
    std::vector<float> w(8 * n), coef(8 * n);
    for (int s = 0; s < n_shots; s++)
        for (int i = off[s]; i < off[s + 1]; i++) {
            double fr[3];
            for (int a = 0; a < 3; a++) {
                const double rel = ((double)xyz[3 * i + a] + p->d.extra[a] * p->d.spacing[a]) / p->d.spacing[a];
                const int b = (int)std::floor(rel);
                if (!(b >= 0 && b + 1 <= p->d.shape[a] - 1)) return fail3(SA_E_INVALID, "point outside the 3D grid");
                base[3 * i + a] = b;
                fr[a] = rel - b;
            }
            shot[i] = s;
            for (int c = 0; c < 8; c++) {
                const int cx = (c >> 2) & 1, cy = (c >> 1) & 1, cz = c & 1;
                const double ww = (cx ? fr[0] : 1 - fr[0]) * (cy ? fr[1] : 1 - fr[1]) * (cz ? fr[2] : 1 - fr[2]);
                w[8 * i + c] = (float)ww;
                const int x = base[3 * i] + cx, y = base[3 * i + 1] + cy, z = base[3 * i + 2] + cz;
                const float v = p->vp_host.empty() ? 0.f : p->vp_host[((size_t)x * p->ny + y) * p->nz + z];
                const double vpow = vp_power == 2 ? (double)(v * v) : (double)v;
                coef[8 * i + c] = (float)(ww * scale * vpow);
            }
        }
    int rc = alloc3(d_shot, n);
    if (rc == SA_OK) rc = alloc3(d_base, 3 * (size_t)n);
    if (rc == SA_OK) rc = alloc3(d_w, 8 * (size_t)n);
    if (rc == SA_OK) rc = alloc3(d_coef, 8 * (size_t)n);
    if (rc != SA_OK) return rc;
    if (n) {
        CK3(cudaMemcpy(*d_shot, shot.data(), n * sizeof(int), cudaMemcpyHostToDevice));
        CK3(cudaMemcpy(*d_base, base.data(), 3 * n * sizeof(int), cudaMemcpyHostToDevice));
        CK3(cudaMemcpy(*d_w, w.data(), 8 * n * sizeof(float), cudaMemcpyHostToDevice));
        CK3(cudaMemcpy(*d_coef, coef.data(), 8 * n * sizeof(float), cudaMemcpyHostToDevice));
    }
    return SA_OK;
}

// Wide support of every point (Hicks: 8 per axis from base - 3; sinc: 14 from base - 6; within the
// grid): injection entries (weight * scale * vp^k at the support point; Hicks sources smoothed as the
// reference's src) and the gathers of the width^3 support (receivers: the traces; sources: the
// wavelet gradient).
static int build_support(Plan3D* p, int n_shots, const int* off, const float* xyz, bool smooth, double scale,
                       int vp_power, int which) {
    const int n = off[n_shots];
    std::vector<int> shot, point;
    std::vector<long long> idx;
    std::vector<float> coef, wraw;
    std::vector<SupportGather3D> hg;
    const int interp = p->d.interpolation, lo = support_lo(interp);
    for (int s = 0; s < n_shots; s++)
        for (int i = off[s]; i < off[s + 1]; i++) {
            int base[3], width = 0;
            double c[3][SUPPORT_MAX];
            for (int a = 0; a < 3; a++) {
                const double rel = ((double)xyz[3 * i + a] + p->d.extra[a] * p->d.spacing[a]) / p->d.spacing[a];
                base[a] = (int)std::floor(rel);
                if (!(base[a] - lo >= 0 && base[a] - lo + support_width(interp) - 1 <= p->d.shape[a] - 1))
                    return fail3(SA_E_INVALID, "point's interpolation support lies outside the 3D grid");
                width = support_coefs(interp, rel - base[a], smooth, c[a]);
            }
            for (int u = 0; u < width; u++)
                for (int v = 0; v < width; v++)
                    for (int w = 0; w < width; w++) {
                        const double ww = c[0][u] * c[1][v] * c[2][w];
                        if (ww == 0.0) continue;
                        const int x = base[0] - lo + u, y = base[1] - lo + v, z = base[2] - lo + w;
                        const float vv = p->vp_host.empty() ? 0.f : p->vp_host[((size_t)x * p->ny + y) * p->nz + z];
                        const double vpow = vp_power == 2 ? (double)(vv * vv) : (double)vv;
                        shot.push_back(s);
                        point.push_back(i);
                        idx.push_back(((long long)x * p->ny + y) * p->zp + z);
                        coef.push_back((float)(ww * scale * vpow));
                        wraw.push_back((float)ww);
                    }
            {
                SupportGather3D G{};
                G.x = base[0] - lo;
                G.y = base[1] - lo;
                G.z = base[2] - lo;
                G.point = i;
                G.shot = s;
                G.width = width;
                for (int k = 0; k < SUPPORT_MAX; k++) {
                    G.wx[k] = (float)c[0][k];
                    G.wy[k] = (float)c[1][k];
                    G.wz[k] = (float)c[2][k];
                }
                hg.push_back(G);
            }
        }
    const size_t m = coef.size();
    int rc = SA_OK;
    if ((rc = alloc3(&p->e_shot[which], m)) != SA_OK || (rc = alloc3(&p->e_point[which], m)) != SA_OK ||
        (rc = alloc3(&p->e_idx[which], m)) != SA_OK || (rc = alloc3(&p->e_coef[which], m)) != SA_OK ||
        (rc = alloc3(&p->e_w[which], m)) != SA_OK)
        return rc;
    if (m) {
        CK3(cudaMemcpy(p->e_shot[which], shot.data(), m * sizeof(int), cudaMemcpyHostToDevice));
        CK3(cudaMemcpy(p->e_point[which], point.data(), m * sizeof(int), cudaMemcpyHostToDevice));
        CK3(cudaMemcpy(p->e_idx[which], idx.data(), m * sizeof(long long), cudaMemcpyHostToDevice));
        CK3(cudaMemcpy(p->e_coef[which], coef.data(), m * sizeof(float), cudaMemcpyHostToDevice));
        CK3(cudaMemcpy(p->e_w[which], wraw.data(), m * sizeof(float), cudaMemcpyHostToDevice));
    }
    p->n_ent[which] = (int)m;
    SupportGather3D** dst = which == 1 ? &p->hgat : &p->hgat_src;
    if ((rc = alloc3(dst, std::max<size_t>(1, hg.size()))) != SA_OK) return rc;
    if (!hg.empty()) CK3(cudaMemcpy(*dst, hg.data(), hg.size() * sizeof(SupportGather3D), cudaMemcpyHostToDevice));
    (void)n;
    return SA_OK;
}

int plan3d_set_geometry(Plan3D* p, int n_shots, const int* so, const float* sx, const int* ro, const float* rx) {
    p->exact_valid = false;  // the receivers' C1 W coefficients follow the geometry
    std::vector<int> so_(so, so + n_shots + 1), ro_(ro, ro + n_shots + 1);
    std::vector<float> sx_(sx ? sx : nullptr, sx ? sx + 3 * (size_t)so[n_shots] : nullptr);
    std::vector<float> rx_(rx ? rx : nullptr, rx ? rx + 3 * (size_t)ro[n_shots] : nullptr);
    const double h = std::max(p->d.spacing[0], std::max(p->d.spacing[1], p->d.spacing[2]));
    int rc = build_points(p, n_shots, so_.data(), sx_.data(), 2.0 * p->d.dt / h, 1, &p->s_shot, &p->s_base, &p->s_w,
                          &p->s_coef);
    if (rc == SA_OK)
        rc = build_points(p, n_shots, ro_.data(), rx_.data(), -p->d.dt * p->d.dt, 2, &p->r_shot, &p->r_base, &p->r_w,
                          &p->r_coef);
    if (rc == SA_OK && p->wide)
        rc = build_support(p, n_shots, so_.data(), sx_.data(), true, 2.0 * p->d.dt / h, 1, 0);
    if (rc == SA_OK && p->wide)
        rc = build_support(p, n_shots, ro_.data(), rx_.data(), false, -p->d.dt * p->d.dt, 2, 1);
    if (rc != SA_OK) return rc;
    p->so = so_;
    p->ro = ro_;
    p->sx = sx_;
    p->rx = rx_;
    p->n_shots = n_shots;
    p->n_src = so_[n_shots];
    p->n_rec = ro_[n_shots];
    if ((rc = alloc3(&p->src_amp, (size_t)p->d.nt * std::max(1, p->n_src))) != SA_OK) return rc;
    if ((rc = alloc3(&p->rec_amp, (size_t)p->d.nt * std::max(1, p->n_rec))) != SA_OK) return rc;
    if (!p->layout_fixed) set_chunks(p, default_chunks(p, n_shots));
    p->geometry_set = true;
    p->snaps_valid = false;
    p->ckpt_valid = false;
    return SA_OK;
}

static int load_tm(Plan3D* p, const float* user, int rows, int cols, float* dst, cudaStream_t s) {
    const size_t n = (size_t)rows * cols;
    if (!n) return SA_OK;
    const float* src = user;
    if (!dev_ptr(user)) {
        if (n > p->cap_tstage) {
            int rc = alloc3(&p->tstage, n);
            if (rc != SA_OK) return rc;
            p->cap_tstage = n;
        }
        CK3(cudaMemcpyAsync(p->tstage, user, n * sizeof(float), cudaMemcpyHostToDevice, s));
        src = p->tstage;
    }
    CK3(transpose(src, rows, cols, dst, s));
    return SA_OK;
}

static Step3D args3(const Plan3D* p) {
    Step3D a{};
    a.nx = p->nx;
    a.ny = p->ny;
    a.nz = p->nz;
    a.zp = p->zp;
    a.shot_stride = p->field;
    a.chunk_rows = p->chunk_rows;
    a.ty0n = p->ty0n;
    a.nshots = p->n_shots;
    const long long G = GUARD;
    a.W = p->W + G * p->plane;
    a.bxh = p->bxh ? p->bxh + (G + 5) * p->plane : nullptr;
    a.byh = p->byh ? p->byh + G * (p->ny + 12) * p->zp : nullptr;
    a.bzh = p->bzh ? p->bzh + G * p->ny * p->zpb : nullptr;
    a.zpb = p->zpb;
    a.C1 = p->C1 + G * p->plane;
    a.C2 = p->C2 + G * p->plane;
    a.C3 = p->C3 + G * p->plane;
    a.hx = (float)p->d.spacing[0];
    a.hy = (float)p->d.spacing[1];
    a.hz = (float)p->d.spacing[2];
    a.dt = (float)p->d.dt;
    a.f = p->d.undersampling;
    a.snaps = p->snaps;
    a.snap_stride = p->snap_stride;
    a.snap_shot_stride = (long long)p->n_snap * p->snap_stride;
    return a;
}

// Imaging condition of adjoint level t (t % f == 0) as its own streaming kernel, q = p_a[t].
static int image_level(Plan3D* p, const Step3D& a, const float* q, cudaStream_t s, long long& n) {
    if (a.t % a.f) return SA_OK;
    const int lo[3] = {p->d.absorbing[0], p->d.absorbing[1], p->d.absorbing[2]};
    const int hi[3] = {p->nx - p->d.absorbing[0], p->ny - p->d.absorbing[1], p->nz - p->d.absorbing[2]};
    CK3(image3d(q, a.snaps + (long long)(a.t / a.f) * a.snap_stride, p->gradb, p->precb, lo, hi, p->ny, p->zp,
                p->n_shots, p->field, a.snap_shot_stride, s));
    n++;
    return SA_OK;
}

// Imaging from raw snapshots of adjoint level t, q = p_a[t]: held terms refreshed on t % f == 0,
// accumulated every step (the 2D image_raw_step).
static int image_raw_level(Plan3D* p, const Step3D& a, const float* q, bool rho, cudaStream_t s, long long& n) {
    const bool refresh = a.t % a.f == 0;
    const int lo[3] = {p->d.absorbing[0], p->d.absorbing[1], p->d.absorbing[2]};
    const int hi[3] = {p->nx - p->d.absorbing[0], p->ny - p->d.absorbing[1], p->nz - p->d.absorbing[2]};
    const double fdt = (double)a.f * p->d.dt;
    CK3(image_raw3d(q, a.snaps + (long long)(refresh ? a.t / a.f : 0) * a.snap_stride, a.snap_stride,
                    a.snap_shot_stride, refresh ? 1 : 0, (float)(1.0 / (fdt * fdt)), p->hold_vp,
                    rho ? p->hold_rho : nullptr, p->buoy, p->db[0], p->db[1], p->db[2], p->d.spacing, p->nx, p->ny,
                    p->nz, p->zp, p->gradb, p->precb, p->gradrb, p->precrb, lo, hi, p->n_shots, p->field, s));
    n++;
    return SA_OK;
}

// One pass over every shot of the plan: the shot pairs in one launch (two lanes), a lone last shot
// of an odd batch in a one-lane launch. Returns the launches made (or a negative error).
static int pass3(Plan3D* p, bool final_pass, bool ot4, Step3D a, cudaStream_t s) {
    const int np = p->n_shots / 2, tiles = p->ty0n * p->tz0n;
    int made = 0;
    if (np > 0) {
        a.shot0 = 0;
        a.npairs = np;
        const cudaError_t e = launch_step3d(p->kind, p->tile, 2, final_pass, ot4, dim3(tiles * np, p->nchunks, 1), s, a);
        if (e != cudaSuccess) return fail3(SA_E_CUDA, cudaGetErrorString(e));
        made++;
    }
    if (p->n_shots & 1) {
        a.shot0 = p->n_shots - 1;
        a.npairs = 1;
        const cudaError_t e = launch_step3d(p->kind, p->tile, 1, final_pass, ot4, dim3(tiles, p->nchunks, 1), s, a);
        if (e != cudaSuccess) return fail3(SA_E_CUDA, cudaGetErrorString(e));
        made++;
    }
    return made;
}
#define PASS3(final_pass, ot4, a)                                \
    do {                                                         \
        const int m_ = pass3(p, (final_pass), (ot4), (a), s);    \
        if (m_ < 0) return m_;                                   \
        n += m_;                                                 \
    } while (0)

// One time level: [pass A] + pass B, then injection into the new level (and its snapshot).
// which: 0 injects the sources (amp = their samples), 1 the receivers, -1 nothing; linear or wide (Hicks, sinc)
// as the plan's interpolation. aux: the CFS-PML auxiliary fields advanced (default: the plan's).
static int step3(Plan3D* p, Step3D& a, const float* cur, float* prev, int which, const float* amp, bool save_now,
                 cudaStream_t s, long long& n, float* aux = nullptr) {
    a.cur = cur;
    a.prev = prev;
    if (p->ot4) {
        a.in = cur;
        a.out_l = p->Lbuf;
        PASS3(false, true, a);
        a.in = p->Lbuf;
    } else {
        a.in = cur;
    }
    PASS3(true, p->ot4, a);
    const float inv_dt2 = (float)(1.0 / ((double)a.dt * (double)a.dt));
    if (p->pml) {  // auxiliary fields and the boundary term of the new level (which 1: the adjoint)
        CK3(pml3d(cur, prev, aux ? aux : p->pml_aux, p->pml_prof, p->C1 + (long long)GUARD * p->plane, p->vp, p->nx, p->ny, p->nz,
                  p->zp, p->n_shots, p->field, p->d.absorbing, p->d.spacing, a.dt, which == 1 ? 1 : 0,
                  save_now ? a.snaps + (long long)(a.t / a.f) * a.snap_stride : nullptr, a.snap_shot_stride, inv_dt2,
                  s));
        n++;
    }
    if (which < 0) return SA_OK;
    const int npts = which == 0 ? p->n_src : p->n_rec;
    float* snap = save_now ? a.snaps : nullptr;
    const long long soff = (long long)(a.t / a.f) * a.snap_stride;
    if (p->wide) {
        const Entries3D e{p->e_shot[which], p->e_point[which], p->e_idx[which], p->e_coef[which]};
        CK3(inject_entries3d(e, p->n_ent[which], amp, npts, a.t, prev, p->field, snap, a.snap_shot_stride, soff,
                             inv_dt2, s));
    } else {
        const Sparse3D inj = which == 0 ? Sparse3D{p->s_shot, p->s_base, p->s_w, p->s_coef}
                                        : Sparse3D{p->r_shot, p->r_base, p->r_w, p->r_coef};
        CK3(sparse3d_inject(inj, npts, amp, npts, a.t, prev, p->field, p->ny, p->zp, snap, a.snap_shot_stride, soff,
                            inv_dt2, s));
    }
    if (npts) n++;
    return SA_OK;
}

int plan3d_forward(Plan3D* p, const float* wavelets, float* traces, int save_mode, cudaStream_t s) {
    if (!p->medium_set || !p->geometry_set) return fail3(SA_E_INVALID, "medium and geometry must be set first");
    const bool raw = save_mode == SA_SAVE_RAW;
    const bool save = save_mode == SA_SAVE_SNAPSHOTS || raw;
    const bool ckpt = save_mode == SA_SAVE_CHECKPOINTS;
    p->ckpt_valid = false;  // the wavelets the checkpointed adjoint re-injects are replaced
    if (save && (size_t)p->n_shots * p->n_snap * p->snap_stride > p->cap_snaps) {
        p->cap_snaps = (size_t)p->n_shots * p->n_snap * p->snap_stride;
        int rc = alloc3(&p->snaps, p->cap_snaps);
        if (rc != SA_OK) return rc;
    }
    const size_t level = (size_t)p->n_shots * p->field;  // floats of one level of every shot
    if (ckpt) {
        // a checkpoint holds both levels and, with the CFS-PML, its nine auxiliary fields
        int rc = choose_checkpoints(p->d, (double)level * sizeof(float), &p->ck_K, &p->ck_n, p->pml ? 11 : 2,
                                    &p->ck_K2);
        if (rc != SA_OK) return rc;
        const size_t need = std::max<size_t>(1, (size_t)p->ck_n * 2 * level);
        if (need > p->cap_ckpt) {
            if ((rc = alloc3(&p->ckpt, need)) != SA_OK) return rc;
            p->cap_ckpt = need;
        }
        const size_t need_pml = std::max<size_t>(1, (size_t)p->ck_n * 9 * level);
        if (p->pml && need_pml > p->cap_pml_ck) {
            if ((rc = alloc3(&p->pml_ck, need_pml)) != SA_OK) return rc;
            p->cap_pml_ck = need_pml;
        }
        if (p->pml && !p->pml_aux_f && (rc = alloc3(&p->pml_aux_f, 9 * std::max(1, p->d.max_shots) * (size_t)p->field)))
            return rc;
        p->snaps_valid = false;
    }
    int rc = load_tm(p, wavelets, p->n_src, p->d.nt, p->src_amp, s);
    if (rc != SA_OK) return rc;
    const size_t fb = (size_t)p->n_shots * p->field * sizeof(float);
    CK3(cudaMemsetAsync(p->F[0], 0, fb, s));
    CK3(cudaMemsetAsync(p->F[1], 0, fb, s));
    CK3(cudaMemsetAsync(p->rec_amp, 0, (size_t)p->d.nt * std::max(1, p->n_rec) * sizeof(float), s));
    if (p->pml) CK3(cudaMemsetAsync(p->pml_aux, 0, 9 * (size_t)p->n_shots * p->field * sizeof(float), s));
    Step3D a = args3(p);
    a.save = raw ? 2 : (save ? 1 : 0);
    if (raw) {  // slots the loop does not write (n = 0, n f > nt-2) read as zero, the reference's fresh buffer
        const int last = (p->d.nt - 2) / a.f;
        const size_t slot = (size_t)p->snap_stride * sizeof(float), pitch = (size_t)a.snap_shot_stride * sizeof(float);
        CK3(cudaMemset2DAsync(p->snaps, pitch, 0, slot, p->n_shots, s));
        if (last + 1 < p->n_snap)
            CK3(cudaMemset2DAsync(p->snaps + (size_t)(last + 1) * p->snap_stride, pitch, 0,
                                  (size_t)(p->n_snap - last - 1) * slot, p->n_shots, s));
    }
    const Sparse3D rec{p->r_shot, p->r_base, p->r_w, p->r_coef};
    long long n = p->n_src ? 1 : 0;
    for (int t = 1; t <= p->d.nt - 2; t++) {
        a.t = t;
        float* cur = (t & 1) ? p->F[1] : p->F[0];
        float* prev = (t & 1) ? p->F[0] : p->F[1];
        rc = step3(p, a, cur, prev, 0, p->src_amp, save && !raw && t % a.f == 0, s, n);
        if (rc != SA_OK) return rc;
        if (p->n_rec) {  // rec[t] = interp(p[t+1])
            if (p->wide)
                CK3(support_gather3d(p->hgat, p->n_rec, prev, p->field, p->ny, p->zp, p->rec_amp, p->n_rec, t, 1.f, s));
            else
                CK3(sparse3d_gather(rec, p->n_rec, prev, p->field, p->ny, p->zp, p->rec_amp, p->n_rec, t, s));
            n++;
        }
        if (ckpt && t % p->ck_K == 0 && t / p->ck_K <= p->ck_n) {  // (p[t+1], p[t]) into slot t/K - 1
            float* slot = p->ckpt + (size_t)(t / p->ck_K - 1) * 2 * level;
            CK3(cudaMemcpyAsync(slot, p->F[0], level * sizeof(float), cudaMemcpyDeviceToDevice, s));
            CK3(cudaMemcpyAsync(slot + level, p->F[1], level * sizeof(float), cudaMemcpyDeviceToDevice, s));
            if (p->pml)  // the CFS-PML's auxiliary fields after step t
                CK3(cudaMemcpyAsync(p->pml_ck + (size_t)(t / p->ck_K - 1) * 9 * level, p->pml_aux,
                                    9 * level * sizeof(float), cudaMemcpyDeviceToDevice, s));
        }
    }
    if (p->n_rec) {
        if (dev_ptr(traces)) {
            CK3(transpose(p->rec_amp, p->d.nt, p->n_rec, traces, s));
        } else {
            const size_t m = (size_t)p->d.nt * p->n_rec;
            if (m > p->cap_tstage) {
                if ((rc = alloc3(&p->tstage, m)) != SA_OK) return rc;
                p->cap_tstage = m;
            }
            CK3(transpose(p->rec_amp, p->d.nt, p->n_rec, p->tstage, s));
            CK3(cudaMemcpyAsync(traces, p->tstage, m * sizeof(float), cudaMemcpyDeviceToHost, s));
            CK3(cudaStreamSynchronize(s));
        }
        n++;
    }
    p->launches = n;
    if (save) {
        p->snaps_valid = true;
        p->snaps_raw = raw;
    }
    if (ckpt) p->ckpt_valid = true;
    return SA_OK;
}

// Reverse-time adjoint from checkpoints: segment k covers t = kK+1 .. min((k+1)K, T0); from
// last to first its start state is restored (zero for k = 0), its forward steps are re-run
// with p.dt2 saved into a K/f-slot segment buffer, and the adjoint steps run back through it
// on their own two levels. The recomputed snapshots are bitwise the stored ones.
// The wavelet gradient of adjoint level t: -interp(p_a[t]) at the sources into row t
// (src.interpolate(expr=-p_a), iso_acoustic/devito.py:755-756).
static int wavelet_level(Plan3D* p, const float* q, int t, bool wav, cudaStream_t s, long long& n) {
    if (!wav || !p->n_src) return SA_OK;
    const Sparse3D src{p->s_shot, p->s_base, p->s_w, p->s_coef};
    if (p->wide)
        CK3(support_gather3d(p->hgat_src, p->n_src, q, p->field, p->ny, p->zp, p->wgrad, p->n_src, t, -1.f, s));
    else
        CK3(sparse3d_gather(src, p->n_src, q, p->field, p->ny, p->zp, p->wgrad, p->n_src, t, s, -1.f));
    n++;
    return SA_OK;
}

// Checkpointed imaging condition: coarse segments from last to first; with two levels (ck_K2 > 0)
// each coarse segment is first re-run without snapshots to place fine checkpoints, then each fine
// segment restores its start, re-runs its forward steps with p.dt2 saved, and runs the adjoint
// back through it (the 2D plan's issue_adjoint_ckpt does the same).
static int adjoint_segments(Plan3D* p, Step3D& aa, const Sparse3D& rec, bool wav, cudaStream_t s, long long& n) {
    const size_t level = (size_t)p->n_shots * p->field;
    const size_t lb = level * sizeof(float);
    const int f = p->d.undersampling, K = p->ck_K;
    const int K2 = p->ck_K2 > 0 ? p->ck_K2 : K;  // fine interval (one level: the coarse one)
    const int T0 = p->d.nt - 1 - f;
    CK3(cudaMemsetAsync(p->A[0], 0, lb, s));
    CK3(cudaMemsetAsync(p->A[1], 0, lb, s));
    Step3D fa = args3(p);
    fa.save = 1;
    fa.snap_shot_stride = aa.snap_shot_stride = (long long)(K2 / f) * p->snap_stride;
    Step3D fr = args3(p);  // the recompute that places fine checkpoints saves nothing
    fr.save = 0;
    // forward state <- coarse checkpoint k (fine < 0) or fine checkpoint `fine`; zero for coarse 0
    auto restore = [&](int k, int fine) -> int {
        if (fine < 0 && k == 0) {
            CK3(cudaMemsetAsync(p->F[0], 0, lb, s));
            CK3(cudaMemsetAsync(p->F[1], 0, lb, s));
            if (p->pml) CK3(cudaMemsetAsync(p->pml_aux_f, 0, 9 * lb, s));
            return SA_OK;
        }
        const float* lv = fine < 0 ? p->ckpt + (size_t)(k - 1) * 2 * level : p->ckpt2 + (size_t)fine * 2 * level;
        CK3(cudaMemcpyAsync(p->F[0], lv, lb, cudaMemcpyDeviceToDevice, s));
        CK3(cudaMemcpyAsync(p->F[1], lv + level, lb, cudaMemcpyDeviceToDevice, s));
        if (p->pml) {
            const float* ax = fine < 0 ? p->pml_ck + (size_t)(k - 1) * 9 * level : p->pml_ck2 + (size_t)fine * 9 * level;
            CK3(cudaMemcpyAsync(p->pml_aux_f, ax, 9 * lb, cudaMemcpyDeviceToDevice, s));
        }
        return SA_OK;
    };
    for (int k = T0 >= 1 ? (T0 - 1) / K : -1; k >= 0; k--) {
        const int c0 = k * K, c_hi = std::min((k + 1) * K, T0);
        const int nf = (c_hi - c0 + K2 - 1) / K2;  // fine segments
        int rc = SA_OK;
        if (nf > 1) {  // fine checkpoints j = 1 .. nf-1 into slots j-1
            if ((rc = restore(k, -1)) != SA_OK) return rc;
            for (int t = c0 + 1; t <= c0 + (nf - 1) * K2; t++) {
                fr.t = t;
                rc = step3(p, fr, (t & 1) ? p->F[1] : p->F[0], (t & 1) ? p->F[0] : p->F[1], 0, p->src_amp, false, s,
                           n, p->pml_aux_f);
                if (rc != SA_OK) return rc;
                if ((t - c0) % K2 == 0) {
                    const size_t j = (size_t)((t - c0) / K2 - 1);
                    CK3(cudaMemcpyAsync(p->ckpt2 + j * 2 * level, p->F[0], lb, cudaMemcpyDeviceToDevice, s));
                    CK3(cudaMemcpyAsync(p->ckpt2 + j * 2 * level + level, p->F[1], lb, cudaMemcpyDeviceToDevice, s));
                    if (p->pml)
                        CK3(cudaMemcpyAsync(p->pml_ck2 + j * 9 * level, p->pml_aux_f, 9 * lb, cudaMemcpyDeviceToDevice,
                                            s));
                }
            }
        }
        for (int j = nf - 1; j >= 0; j--) {
            const int t_lo = c0 + j * K2 + 1, t_hi = std::min(c0 + (j + 1) * K2, c_hi);
            if ((rc = restore(k, j - 1)) != SA_OK) return rc;
            // the kernels address snapshot t/f; slot t/f - ((c0 + jK2)/f + 1) of the segment buffer is meant
            const long long first = (long long)(c0 + j * K2) / f + 1;
            float* base = reinterpret_cast<float*>(reinterpret_cast<uintptr_t>(p->segsnaps) -
                                                   (uintptr_t)(first * p->snap_stride * (long long)sizeof(float)));
            fa.snaps = aa.snaps = base;
            for (int t = t_lo; t <= t_hi; t++) {
                fa.t = t;
                rc = step3(p, fa, (t & 1) ? p->F[1] : p->F[0], (t & 1) ? p->F[0] : p->F[1], 0, p->src_amp, t % f == 0,
                           s, n, p->pml_aux_f);
                if (rc != SA_OK) return rc;
            }
            for (int t = t_hi; t >= t_lo; t--) {
                aa.t = t;
                const bool even = ((T0 - t) & 1) == 0;
                rc = step3(p, aa, even ? p->A[1] : p->A[0], even ? p->A[0] : p->A[1], 1, p->rec_amp, false, s, n);
                if (rc != SA_OK) return rc;
                if ((rc = image_level(p, aa, even ? p->A[1] : p->A[0], s, n)) != SA_OK) return rc;
                if ((rc = wavelet_level(p, even ? p->A[1] : p->A[0], t, wav, s, n)) != SA_OK) return rc;
            }
        }
    }
    return SA_OK;
}

int plan3d_adjoint(Plan3D* p, const float* residuals, float* grad, float* prec, cudaStream_t s, float* grad_rho,
                   float* prec_rho, float* grad_wavelets) {
    const bool wav = grad_wavelets != nullptr;
    const bool ck = p->ckpt_valid;
    if (!p->snaps_valid && !ck)
        return fail3(SA_E_INVALID, "sa_adjoint needs a prior sa_forward with SA_SAVE_SNAPSHOTS or SA_SAVE_CHECKPOINTS");
    const bool raw = !ck && p->snaps_raw;
    const bool rho = grad_rho != nullptr;
    if ((grad_rho == nullptr) != (prec_rho == nullptr)) return fail3(SA_E_INVALID, "grad_rho and prec_rho go together");
    if (rho && !raw) return fail3(SA_E_INVALID, "the rho gradient needs a prior sa_forward with SA_SAVE_RAW");
    if (rho && p->kind == 0) return fail3(SA_E_INVALID, "the rho gradient needs a plan with rho");
    int rc = SA_OK;
    const size_t fl = (size_t)std::max(1, p->d.max_shots) * p->field;
    if (raw) {
        if (!p->hold_vp && (rc = alloc3(&p->hold_vp, fl)) != SA_OK) return rc;
        if (rho) {
            float** bufs[] = {&p->hold_rho, &p->gradrb, &p->precrb};
            for (float** b : bufs)
                if (!*b && (rc = alloc3(b, fl)) != SA_OK) return rc;
            for (int k = 0; k < 3; k++)
                if (!p->db[k] && (rc = alloc3(&p->db[k], (size_t)p->field)) != SA_OK) return rc;
            if (!p->rho_valid) {
                CK3(rho_terms3d(p->buoy, p->nx, p->ny, p->nz, p->zp, p->d.spacing, p->db[0], p->db[1], p->db[2], 0));
                CK3(cudaDeviceSynchronize());
                p->rho_valid = true;
            }
        }
    }
    if (ck) {
        const size_t level = (size_t)std::max(1, p->d.max_shots) * p->field;
        for (int k = 0; k < 2; k++)
            if (!p->A[k] && (rc = alloc3(&p->A[k], level)) != SA_OK) return rc;
        const int K2 = p->ck_K2 > 0 ? p->ck_K2 : p->ck_K;
        const size_t need = (size_t)(K2 / p->d.undersampling) * p->n_shots * p->field;
        if (need > p->cap_segsnaps) {
            if ((rc = alloc3(&p->segsnaps, need)) != SA_OK) return rc;
            p->cap_segsnaps = need;
        }
        if (p->ck_K2 > 0) {  // fine checkpoints of one coarse segment
            const size_t nf = (size_t)std::max(1, p->ck_K / p->ck_K2 - 1);
            const size_t need2 = nf * 2 * (size_t)p->n_shots * p->field;
            if (need2 > p->cap_ckpt2) {
                if ((rc = alloc3(&p->ckpt2, need2)) != SA_OK) return rc;
                p->cap_ckpt2 = need2;
            }
            const size_t need_pml = nf * 9 * (size_t)p->n_shots * p->field;
            if (p->pml && need_pml > p->cap_pml_ck2) {
                if ((rc = alloc3(&p->pml_ck2, need_pml)) != SA_OK) return rc;
                p->cap_pml_ck2 = need_pml;
            }
        }
    }
    if (!p->gradb && (rc = alloc3(&p->gradb, fl)) != SA_OK) return rc;
    if (!p->precb && (rc = alloc3(&p->precb, fl)) != SA_OK) return rc;
    if ((rc = load_tm(p, residuals, p->n_rec, p->d.nt, p->rec_amp, s)) != SA_OK) return rc;
    const size_t wn = (size_t)p->d.nt * std::max(1, p->n_src);
    if (wav && wn > p->cap_wgrad) {
        if ((rc = alloc3(&p->wgrad, wn)) != SA_OK) return rc;
        p->cap_wgrad = wn;
    }
    if (wav) CK3(cudaMemsetAsync(p->wgrad, 0, wn * sizeof(float), s));
    const size_t fb = (size_t)p->n_shots * p->field * sizeof(float);
    CK3(cudaMemsetAsync(p->F[0], 0, fb, s));
    CK3(cudaMemsetAsync(p->F[1], 0, fb, s));
    CK3(cudaMemsetAsync(p->gradb, 0, fb, s));
    CK3(cudaMemsetAsync(p->precb, 0, fb, s));
    if (raw) CK3(cudaMemsetAsync(p->hold_vp, 0, fb, s));  // held terms start at zero
    if (p->pml) CK3(cudaMemsetAsync(p->pml_aux, 0, 9 * fb, s));
    if (rho) {
        CK3(cudaMemsetAsync(p->hold_rho, 0, fb, s));
        CK3(cudaMemsetAsync(p->gradrb, 0, fb, s));
        CK3(cudaMemsetAsync(p->precrb, 0, fb, s));
    }
    Step3D a = args3(p);
    a.save = 0;
    const Sparse3D rec{p->r_shot, p->r_base, p->r_w, p->r_coef};
    const int T0 = p->d.nt - 1 - p->d.undersampling;
    long long n = p->n_rec ? 1 : 0;
    if (ck && (rc = adjoint_segments(p, a, rec, wav, s, n)) != SA_OK) return rc;
    for (int t = ck ? 0 : T0; t >= 1; t--) {
        a.t = t;
        const bool even = ((T0 - t) & 1) == 0;
        float* cur = even ? p->F[1] : p->F[0];
        float* prev = even ? p->F[0] : p->F[1];
        rc = step3(p, a, cur, prev, 1, p->rec_amp, false, s, n);
        if (rc != SA_OK) return rc;
        rc = raw ? image_raw_level(p, a, cur, rho, s, n) : image_level(p, a, cur, s, n);
        if (rc != SA_OK) return rc;
        if ((rc = wavelet_level(p, cur, t, wav, s, n)) != SA_OK) return rc;
    }
    if (wav && p->n_src) {  // time-major -> [n_src, nt]
        if (dev_ptr(grad_wavelets)) {
            CK3(transpose(p->wgrad, p->d.nt, p->n_src, grad_wavelets, s));
        } else {
            if (wn > p->cap_tstage) {
                if ((rc = alloc3(&p->tstage, wn)) != SA_OK) return rc;
                p->cap_tstage = wn;
            }
            CK3(transpose(p->wgrad, p->d.nt, p->n_src, p->tstage, s));
            CK3(cudaMemcpyAsync(grad_wavelets, p->tstage, wn * sizeof(float), cudaMemcpyDeviceToHost, s));
            CK3(cudaStreamSynchronize(s));
        }
        n++;
    }
    const size_t N = (size_t)p->nx * p->ny * p->nz;
    for (int k = 0; k < (rho ? 4 : 2); k++) {
        float* user = k == 0 ? grad : (k == 1 ? prec : (k == 2 ? grad_rho : prec_rho));
        const float* buf = k == 0 ? p->gradb : (k == 1 ? p->precb : (k == 2 ? p->gradrb : p->precrb));
        if (dev_ptr(user)) {
            CK3(reduce3d(buf, p->field, p->n_shots, p->nx, p->ny, p->nz, p->zp, user, s));
        } else {
            if (N > p->cap_tstage) {
                if ((rc = alloc3(&p->tstage, N)) != SA_OK) return rc;
                p->cap_tstage = N;
            }
            CK3(reduce3d(buf, p->field, p->n_shots, p->nx, p->ny, p->nz, p->zp, p->tstage, s));
            CK3(cudaMemcpyAsync(user, p->tstage, N * sizeof(float), cudaMemcpyDeviceToHost, s));
            CK3(cudaStreamSynchronize(s));
        }
        n++;
    }
    p->launches = n;
    return SA_OK;
}

}  // namespace sa

namespace sa {

// Exact adjoint of the discrete 3D forward map (SA_GRAD_EXACT), the 3D form of the 2D plan's
// issue_adjoint_exact: with z = C1 W mu obeying the forward recursion, segment k of K steps is
// recomputed from checkpoint k with every level kept (K + 2 levels), then the adjoint steps run
// back through it: z[t-1] from z[t], z[t+1] (no receiver term inside the step), plus
// w C1 W dL/drec[t-2] at the receivers; the vp gradient of step t-1 from three stored levels,
// W G(u[t-1]) and W G(z[t]) (OT4, unit-coefficient OT2 passes) and the source term.
int plan3d_adjoint_exact(Plan3D* p, const float* residuals, float* grad, float* prec, cudaStream_t s) {
    if (!p->ckpt_valid)
        return fail3(SA_E_INVALID, "SA_GRAD_EXACT needs a prior sa_forward with SA_SAVE_CHECKPOINTS");
    if (p->ck_K2 > 0)
        return fail3(SA_E_NOMEM, "SA_GRAD_EXACT needs a one-level checkpoint schedule: checkpoint_budget is too small");
    const int nt = p->d.nt, K = p->ck_K;
    const size_t fl = (size_t)std::max(1, p->d.max_shots) * p->field;  // floats of one level (capacity)
    const size_t level = (size_t)p->n_shots * p->field;                  // floats of one level (in use)
    const size_t lb = level * sizeof(float);
    const long long G = GUARD;
    const size_t guarded = (size_t)(p->nx + 2 * G) * p->plane;
    int rc = SA_OK;
    for (int k = 0; k < 2; k++)
        if (!p->A[k] && (rc = alloc3(&p->A[k], fl)) != SA_OK) return rc;
    if (!p->gradb && (rc = alloc3(&p->gradb, fl)) != SA_OK) return rc;
    if (!p->precb && (rc = alloc3(&p->precb, fl)) != SA_OK) return rc;
    const size_t need = (size_t)(K + 2) * level;
    if (need > p->cap_levels) {
        if ((rc = alloc3(&p->levels, need)) != SA_OK) return rc;
        p->cap_levels = need;
    }
    if (!p->EA) {
        float** per_point[] = {&p->EA, &p->EB, &p->EC, &p->EG4, &p->ES};
        for (float** b : per_point)
            if ((rc = alloc3(b, (size_t)p->field)) != SA_OK) return rc;
        if ((rc = alloc3(&p->Lu, fl)) != SA_OK || (rc = alloc3(&p->Lz, fl)) != SA_OK) return rc;  // zeroed: finite
        if ((rc = alloc3(&p->zeros, guarded)) != SA_OK || (rc = alloc3(&p->ones, guarded)) != SA_OK) return rc;
        std::vector<float> one(guarded, 1.f);
        CK3(cudaMemcpy(p->ones, one.data(), guarded * sizeof(float), cudaMemcpyHostToDevice));
    }
    if (!p->exact_valid) {
        CK3(exact_coef3d(p->vp, p->alpha, p->W + G * p->plane, p->nx, p->ny, p->nz, p->zp, p->sponge, (float)p->d.dt,
                         p->EA, p->EB, p->EC, p->EG4, p->ES, 0));
        if ((rc = alloc3(&p->r_xcoef, 8 * (size_t)std::max(1, p->n_rec))) != SA_OK) return rc;
        const Sparse3D rec{p->r_shot, p->r_base, p->r_w, p->r_coef};
        CK3(xcoef3d(rec, p->n_rec, p->C1 + G * p->plane, p->W + G * p->plane, p->ny, p->zp, p->r_xcoef, 0));
        if (p->wide) {
            if ((rc = alloc3(&p->e_xcoef, std::max<size_t>(1, p->n_ent[1]))) != SA_OK) return rc;
            CK3(xcoef_entries3d(p->e_idx[1], p->e_w[1], p->n_ent[1], p->C1 + G * p->plane, p->W + G * p->plane,
                                p->e_xcoef, 0));
        }
        CK3(cudaDeviceSynchronize());
        p->exact_valid = true;
    }
    if ((rc = load_tm(p, residuals, p->n_rec, nt, p->rec_amp, s)) != SA_OK) return rc;
    CK3(cudaMemsetAsync(p->A[0], 0, lb, s));
    CK3(cudaMemsetAsync(p->A[1], 0, lb, s));
    CK3(cudaMemsetAsync(p->gradb, 0, lb, s));
    CK3(cudaMemsetAsync(p->precb, 0, lb, s));
    Step3D fa = args3(p);  // forward recompute, sources injected after each step
    fa.save = 0;
    Step3D aa = fa;        // adjoint steps, the receiver term injected separately
    Step3D la = fa;        // W G(.) with unit / zero update coefficients
    la.C1 = p->ones + G * p->plane;
    la.C2 = la.C3 = p->zeros + G * p->plane;
    const Sparse3D src{p->s_shot, p->s_base, p->s_w, p->s_coef};
    const Sparse3D recx{p->r_shot, p->r_base, p->r_w, p->r_xcoef};
    const float inv_dt2 = (float)(1.0 / (p->d.dt * p->d.dt));
    const double h = std::max(p->d.spacing[0], std::max(p->d.spacing[1], p->d.spacing[2]));
    const float src_scale = (float)(2.0 * p->d.dt / h);
    auto lvl = [&](int k, int m) { return p->levels + (size_t)(m - k * K) * level; };
    long long n = p->n_rec ? 1 : 0;
    for (int k = (nt - 2) / K; k >= 0; k--) {
        const int t_lo = std::max(2, k * K + 2), t_hi = std::min((k + 1) * K + 1, nt);
        if (t_lo > t_hi) continue;
        if (k == 0) {
            CK3(cudaMemsetAsync(p->F[0], 0, lb, s));
            CK3(cudaMemsetAsync(p->F[1], 0, lb, s));
        } else {
            const float* slot = p->ckpt + (size_t)(k - 1) * 2 * level;
            CK3(cudaMemcpyAsync(p->F[0], slot, lb, cudaMemcpyDeviceToDevice, s));
            CK3(cudaMemcpyAsync(p->F[1], slot + level, lb, cudaMemcpyDeviceToDevice, s));
        }
        // u[kK] lives in F[kK & 1], u[kK+1] in the other
        CK3(cudaMemcpyAsync(lvl(k, k * K), p->F[(k * K) & 1], lb, cudaMemcpyDeviceToDevice, s));
        CK3(cudaMemcpyAsync(lvl(k, k * K + 1), p->F[(k * K + 1) & 1], lb, cudaMemcpyDeviceToDevice, s));
        for (int m = k * K + 1; m <= std::min((k + 1) * K, nt - 2); m++) {  // forward step m -> u[m+1]
            fa.t = m;
            if ((rc = step3(p, fa, p->F[m & 1], p->F[(m + 1) & 1], 0, p->src_amp, false, s, n)) != SA_OK)
                return rc;
            CK3(cudaMemcpyAsync(lvl(k, m + 1), p->F[(m + 1) & 1], lb, cudaMemcpyDeviceToDevice, s));
        }
        for (int t = t_hi; t >= t_lo; t--) {
            float* zt = p->A[t & 1];
            float* znext = p->A[(t + 1) & 1];
            aa.t = t;
            if ((rc = step3(p, aa, zt, znext, -1, p->rec_amp, false, s, n)) != SA_OK) return rc;
            if (p->n_rec) {  // z[t-1] += w C1 W dL/drec[t-2]
                if (p->wide) {
                    const Entries3D e{p->e_shot[1], p->e_point[1], p->e_idx[1], p->e_xcoef};
                    CK3(inject_entries3d(e, p->n_ent[1], p->rec_amp, p->n_rec, t - 2, znext, p->field, nullptr, 0, 0,
                                         0.f, s));
                } else {
                    CK3(sparse3d_inject(recx, p->n_rec, p->rec_amp, p->n_rec, t - 2, znext, p->field, p->ny, p->zp,
                                        nullptr, 0, 0, 0.f, s));
                }
                n++;
            }
            if (t > nt - 1) continue;  // z[nt] = 0
            const float *Lu = nullptr, *Lz = nullptr;
            if (p->ot4) {
                la.t = t - 1;
                la.cur = la.in = lvl(k, t - 1);
                la.prev = p->Lu;
                PASS3(true, false, la);
                la.t = t;
                la.cur = la.in = zt;
                la.prev = p->Lz;
                PASS3(true, false, la);
                Lu = p->Lu;
                Lz = p->Lz;
            }
            CK3(exact_grad3d(zt, lvl(k, t), lvl(k, t - 1), lvl(k, t - 2), Lu, Lz, p->EA, p->EB, p->EC, p->EG4, p->nx,
                             p->ny, p->nz, p->zp, p->n_shots, p->field, inv_dt2, p->gradb, p->precb, s));
            n++;
            if (p->n_src) {
                if (p->wide) {
                    const Entries3D e{p->e_shot[0], p->e_point[0], p->e_idx[0], p->e_coef[0]};
                    CK3(exact_src_entries3d(zt, e, p->e_w[0], p->n_ent[0], p->src_amp, p->n_src, t - 1, src_scale,
                                            p->ES, p->field, p->gradb, s));
                } else {
                    CK3(exact_src3d(zt, src, p->n_src, p->src_amp, p->n_src, t - 1, src_scale, p->ES, p->ny, p->zp,
                                    p->field, p->gradb, s));
                }
                n++;
            }
        }
    }
    const size_t N = (size_t)p->nx * p->ny * p->nz;
    for (int k = 0; k < 2; k++) {
        float* user = k == 0 ? grad : prec;
        const float* buf = k == 0 ? p->gradb : p->precb;
        if (dev_ptr(user)) {
            CK3(reduce3d(buf, p->field, p->n_shots, p->nx, p->ny, p->nz, p->zp, user, s));
        } else {
            if (N > p->cap_tstage) {
                if ((rc = alloc3(&p->tstage, N)) != SA_OK) return rc;
                p->cap_tstage = N;
            }
            CK3(reduce3d(buf, p->field, p->n_shots, p->nx, p->ny, p->nz, p->zp, p->tstage, s));
            CK3(cudaMemcpyAsync(user, p->tstage, N * sizeof(float), cudaMemcpyDeviceToHost, s));
            CK3(cudaStreamSynchronize(s));
        }
        n++;
    }
    p->launches = n;
    return SA_OK;
}

// Layout search of a 3D plan: every tile of kTiles3d with the x chunkings that keep chunks at least
// 4 R rows deep, each timed over a few steps of the two passes on the plan's own wavefield buffers
// (their contents are overwritten); the fastest is kept. Results are remembered per (grid, operator,
// shots, device) for the life of the process.
int plan3d_autotune(Plan3D* p, const char* device_key, int* tile_out, int* chunks_out, bool* cached, cudaStream_t s) {
    if (!p->medium_set || !p->geometry_set) return fail3(SA_E_INVALID, "autotune needs medium and geometry");
    if (p->snaps_valid || p->ckpt_valid)
        return fail3(SA_E_INVALID, "autotune would overwrite the saved wavefield: run it before the saving forward");
    char key[256];
    snprintf(key, sizeof(key), "3d:%d,%d,%d:k%d:%s:s%d:%s", p->nx, p->ny, p->nz, p->kind, p->ot4 ? "ot4" : "ot2",
             p->n_shots, device_key);
    static std::map<std::string, std::pair<int, int>> cache;
    static std::mutex mu;
    {
        std::lock_guard<std::mutex> g(mu);
        auto it = cache.find(key);
        if (it != cache.end()) {
            set_tile(p, it->second.first);
            set_chunks(p, it->second.second);
            p->layout_fixed = true;
            *tile_out = p->tile;
            *chunks_out = p->nchunks;
            *cached = true;
            return SA_OK;
        }
    }
    const int R = p->kind == 0 ? 5 : 9;
    const int steps = std::min(6, p->d.nt - 2);
    cudaEvent_t e0, e1;
    CK3(cudaEventCreate(&e0));
    CK3(cudaEventCreate(&e1));
    float best = 1e30f;
    int bt = p->tile, bc = p->nchunks;
    for (int tile = 0; tile < kTiles3dN; tile++) {
        set_tile(p, tile);
        for (int nc : {1, 2, 3, 4, 6, 8}) {
            if (p->nx / nc < 4 * R) continue;
            set_chunks(p, nc);
            Step3D a = args3(p);
            a.save = 0;
            long long n = 0;
            for (int t = 0; t < 2 + steps; t++) {
                if (t == 2) CK3(cudaEventRecord(e0, s));
                a.t = 1 + t;
                a.cur = p->F[t & 1];
                a.prev = p->F[(t + 1) & 1];
                if (p->ot4) {
                    a.in = a.cur;
                    a.out_l = p->Lbuf;
                    PASS3(false, true, a);
                    a.in = p->Lbuf;
                } else {
                    a.in = a.cur;
                }
                PASS3(true, p->ot4, a);
            }
            CK3(cudaEventRecord(e1, s));
            CK3(cudaEventSynchronize(e1));
            float ms = 0.f;
            CK3(cudaEventElapsedTime(&ms, e0, e1));
            if (ms < best) {
                best = ms;
                bt = tile;
                bc = p->nchunks;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    set_tile(p, bt);
    set_chunks(p, bc);
    p->layout_fixed = true;
    {
        std::lock_guard<std::mutex> g(mu);
        cache[key] = {bt, bc};
    }
    *tile_out = bt;
    *chunks_out = p->nchunks;
    *cached = false;
    return SA_OK;
}

int plan3d_layout(const Plan3D* p, int* threads, int* tiles, int* chunks) {
    *threads = kTiles3d[p->tile].ty * kTiles3d[p->tile].tz;
    *tiles = p->ty0n * p->tz0n;
    *chunks = p->nchunks;
    return SA_OK;
}

}  // namespace sa

// libstrideacc: C ABI of the GB300 iso-acoustic FDTD path (declarations and reference
// citations in include/strideacc.h). A plan owns the device state of a batch of shots: two
// wavefield levels per shot, the medium, per-CTA source/receiver lists, the undersampled
// wavefield of the reference's gradient algorithm and per-shot gradient accumulators. The
// time loop is captured once into a CUDA graph per mode and replayed.
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/strideacc.h"
#include "common.cuh"
#include "helpers.h"
#include "launch.h"
#include "persist2d.h"
#include "plan3d.h"

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CK(x)                                                                                    \
    do {                                                                                         \
        cudaError_t e_ = (x);                                                                    \
        if (e_ != cudaSuccess) return fail(SA_E_CUDA, "%s: %s", #x, cudaGetErrorString(e_));     \
    } while (0)

#define CKR(x)                                                                                   \
    do {                                                                                         \
        int r_ = (x);                                                                            \
        if (r_ != SA_OK) return r_;                                                              \
    } while (0)

bool is_device(const void* p) {
    if (!p) return false;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

template <class T>
int ensure(T** ptr, size_t* cap, size_t n) {
    if (n <= *cap && *ptr) return SA_OK;
    if (*ptr) cudaFree(*ptr);
    *ptr = nullptr;
    *cap = 0;
    if (n == 0) n = 1;
    if (cudaMalloc((void**)ptr, n * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        *ptr = nullptr;
        return fail(SA_E_NOMEM, "device allocation of %zu bytes failed", n * sizeof(T));
    }
    *cap = n;
    return SA_OK;
}

constexpr double kDbToNeper = 100.0 / (20.0 * 0.43429448190325176);  // 100 / (20 log10 e)

}  // namespace

namespace sa {
// Message returned by sa_last_error for entry points defined in other translation units.
void set_last_error(const char* msg) { g_err = msg; }
}  // namespace sa

// Injection entries grouped by target point: field[idx[k]] += sum of coef[e] * amp[t][point[e]]
// over e in [off[k], off[k+1]).
struct Targets {
    long long* idx = nullptr;
    int *off = nullptr, *point = nullptr;
    float* coef = nullptr;
    size_t cap_idx = 0, cap_off = 0, cap_point = 0, cap_coef = 0;
    int n = 0;
    std::vector<long long> hidx;  // host copy of idx (the persistent forward's owner of each target)
};

struct sa_plan {
    sa_desc d{};
    sa::Plan3D* p3 = nullptr;  // dim == 3: the 3D plan (plan3d.cu) serves every entry point
    int nx = 0, ny = 0, pitch = 0, pitch_b = 0;
    long long shot_stride = 0;  // nx * pitch: float2 elements per shot pair (wavefields are pair-interleaved)
    int kind = 0;
    bool ot4 = true;
    float* field[2] = {nullptr, nullptr};
    size_t field_cap[2] = {0, 0};
    float* lbuf = nullptr;  // OT4: l = W G(p[t]) between the step's two passes (zero beyond the grid)
    size_t lbuf_cap = 0;
    // medium: W, bxh, byh, C1..C3 have GUARD zero rows on both sides (the *_0 pointers address
    // row 0 / half-row 0); vp, alpha, buoy are unguarded scratch of the preparation kernels
    float *W = nullptr, *vp = nullptr, *alpha = nullptr, *buoy = nullptr, *bxh = nullptr, *byh = nullptr;
    float *C1 = nullptr, *C2 = nullptr, *C3 = nullptr;
    // the step passes' copies of W, bxh, byh, C1, C2, -C3 (step_medium2d)
    float* smed = nullptr;
    size_t cap_smed = 0;
    size_t cap_W = 0, cap_vp = 0, cap_alpha = 0, cap_buoy = 0, cap_bxh = 0, cap_byh = 0, cap_C1 = 0, cap_C2 = 0,
           cap_C3 = 0;
    std::vector<float> vp_host;  // for the injection coefficients (vp at the corners)
    float* medium_stage = nullptr;
    size_t cap_medium_stage = 0;
    bool medium_set = false;
    // geometry (host copy)
    int n_shots = 0, n_src = 0, n_rec = 0;
    std::vector<int> src_off, rec_off;
    std::vector<int> src_bx, src_by, rec_bx, rec_by;
    std::vector<double> src_fx, src_fy, rec_fx, rec_fy;
    bool geometry_set = false;
    // receiver gathers (one per receiver, applied by their own kernel after each step)
    sa::Gather* gat_flat = nullptr;
    size_t cap_gat_flat = 0;
    // sparse traces, time-major
    float *src_amp = nullptr, *rec_amp = nullptr, *stage = nullptr;
    size_t cap_src_amp = 0, cap_rec_amp = 0, cap_stage = 0;
    // saved wavefield and gradient accumulators
    float* snaps = nullptr;
    size_t cap_snaps = 0;
    int n_snap = 0;
    long long snap_stride = 0, snap_shot_stride = 0;
    bool snaps_valid = false;
    bool adjoint_pending = false;  // a forward with save ran and no adjoint has used it yet
    bool snaps_raw = false;  // the snapshots hold p[t] (SA_SAVE_RAW), not p.dt2
    float *gradb = nullptr, *precb = nullptr;
    size_t cap_gradb = 0, cap_precb = 0;
    // raw-snapshot gradients: held vp/rho terms per shot pair, rho accumulators, D-b per node
    float *hold_vp = nullptr, *hold_rho = nullptr, *gradrb = nullptr, *precrb = nullptr, *dbx = nullptr,
          *dby = nullptr;
    size_t cap_hold_vp = 0, cap_hold_rho = 0, cap_gradrb = 0, cap_precrb = 0, cap_dbx = 0, cap_dby = 0;
    bool rho_terms_valid = false;
    // CFS-PML (SA_BOUNDARY_CFS_PML): sigma/alpha profiles and their derivatives per axis, and the
    // six auxiliary fields (u3, u2, u1 of each axis) per shot pair
    bool pml = false;
    float *pml_prof = nullptr, *pml_aux = nullptr;
    size_t cap_pml_prof = 0, cap_pml_aux = 0;
    // with checkpoints: the forward's auxiliary fields at every checkpoint, and a second set for the
    // forward recompute (the adjoint keeps its own in pml_aux)
    float *pml_ck = nullptr, *pml_aux_f = nullptr;
    size_t cap_pml_ck = 0, cap_pml_aux_f = 0;
    // checkpoints (SA_SAVE_CHECKPOINTS): both levels after every ck_K-th forward step, the
    // recomputed snapshots of one segment, and the adjoint's own two levels
    float *ckpt = nullptr, *segsnaps = nullptr, *afield[2] = {nullptr, nullptr};
    size_t cap_ckpt = 0, cap_segsnaps = 0, afield_cap[2] = {0, 0};
    int ck_K = 0, ck_n = 0;
    // two-level schedule (ck_K2 > 0): fine checkpoints every ck_K2 steps of one coarse segment,
    // placed by the adjoint's recompute (levels, and the CFS-PML's auxiliary fields)
    int ck_K2 = 0;
    float *ckpt2 = nullptr, *pml_ck2 = nullptr;
    size_t cap_ckpt2 = 0, cap_pml_ck2 = 0;
    bool ckpt_valid = false;
    // exact-gradient mode: per-point derivative coefficients, every level of a segment, the
    // W G(.) of a forward and an adjoint level (the step pass's wg_only mode), the receiver
    // injection with coefficient C1 W, flat source list
    float *EA = nullptr, *EB = nullptr, *EC = nullptr, *EG4 = nullptr, *ES = nullptr, *levels = nullptr;
    float *Lu = nullptr, *Lz = nullptr;
    size_t cap_EA = 0, cap_EB = 0, cap_EC = 0, cap_EG4 = 0, cap_ES = 0, cap_levels = 0, cap_Lu = 0, cap_Lz = 0;
    bool exact_coef_valid = false;
    std::vector<float> c1w_host;
    sa::ExactSrc2D* src_flat = nullptr;  // support points of the sources (exact gradient's source term)
    size_t cap_src_flat = 0;
    int n_src_flat = 0;
    // wavelet gradient: source gathers with negated weights and its time-major buffer
    sa::Gather* gat_src = nullptr;
    float* wgrad = nullptr;
    size_t cap_gat_src = 0, cap_wgrad = 0;
    // wide interpolation (Hicks, sinc): receiver gathers run as their own kernel after each step
    sa::SupportGather* hgat = nullptr;
    size_t cap_hgat = 0;
    sa::SupportGather* hgat_src = nullptr;  // sources (Hicks: smoothed), negated: the wavelet gradient
    size_t cap_hgat_src = 0;
    // source (forward), receiver (adjoint) and exact-gradient receiver injection grouped by target
    // point, each applied by its own kernel after the step
    Targets stgt, rtgt, xtgt;
    // layout
    int NT = 128, by = 110, chunk_rows = 1, nstrips = 1, nchunks = 1;
    bool layout_fixed = false;
    sa::Sponge sponge{};
    // graphs
    cudaStream_t cap = nullptr;
    cudaGraphExec_t g_fwd[4] = {nullptr, nullptr, nullptr, nullptr};  // by save mode
    // [from snapshots, from checkpoints, exact, raw vp, raw vp + rho][wavelet gradient]
    cudaGraphExec_t g_adj[5][2] = {};
    long long fwd_launches[4] = {0, 0, 0, 0};  // kernels in each forward loop (by save mode)
    long long adj_launches[5] = {0, 0, 0, 0, 0};  // kernels in each adjoint loop
    bool use_graphs = true;
    // persistent forward of small batches (persist2d.cu): mode (-1 never, 0 automatic, 1 whenever
    // eligible), the tests' barrier knobs, its tile layout and device state
    int persist_mode = 0;
    int persist_tuned = -1;  // the autotuner's choice for automatic mode: -1 none, 0 streaming, 1 persistent
    int persist_extra = 0;
    long long persist_spin = 10000000;
    int ptx = 0, pty = 0, ptiles_x = 0, ptiles_y = 0, pblocks = 0;
    size_t psmem = 0;
    int* pbar = nullptr;  // error flag of the persistent launch
    uint4* pxch = nullptr;  // its exchange lines
    size_t cap_pxch = 0;
    size_t cap_pbar = 0;
    int *pcta_off = nullptr, *pcta_tgt = nullptr, *prec_off = nullptr, *prec_idx = nullptr;
    size_t cap_pcta_off = 0, cap_pcta_tgt = 0, cap_prec_off = 0, cap_prec_idx = 0;
    float* psrcv = nullptr;  // the sources' values at every step
    size_t cap_psrcv = 0;
    // L2 residency of the duplicated medium: every shot pair's CTAs read each of its rows once per
    // pass, just after the previous pass streamed the wavefields through L2; the captured step
    // kernels carry this persisting window
    cudaAccessPolicyWindow l2win{};
    long long launches = 0;                   // kernels launched by the last sa_forward / sa_adjoint
};

namespace {

int npairs(const sa_plan* p) { return (p->n_shots + 1) / 2; }
int radius(const sa_plan* p) { return p->kind == 0 ? 5 : 9; }
// fewest column strips of the step passes (a CTA thread owns two columns)
int min_strips(const sa_plan* p) { return (p->ny + 2 * sa::STEP_MAX_THREADS - 1) / (2 * sa::STEP_MAX_THREADS); }
void set_strips(sa_plan* p, int strips) {
    int by = 0, nt = 0;
    sa::step_strips(p->ny, strips, &by, &nt);
    p->by = by;
    p->NT = nt;
    p->nstrips = (p->ny + by - 1) / by;
}

void drop_graphs(sa_plan* p) {
    for (auto& g : p->g_fwd)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    for (auto& row : p->g_adj)
        for (auto& g : row)
            if (g) {
                cudaGraphExecDestroy(g);
                g = nullptr;
            }
}

// Sponge ramp of Boundary.damping for one axis (stride/physics/boundaries/boundary.py:98-151),
// before the multiplication by vp and 7 dt (done per point in the kernel).
void damping_table(int A, double h, double refl, float* out) {  // out: MAX_ABS entries
    for (int e = 0; e < sa::MAX_ABS; e++) out[e] = 0.f;
    if (A <= 0) return;
    double coef = (2 + 1) / 2.0 * std::log(1.0 / refl);
    coef = A > 15 ? coef / (A * h) : 0.67 / h;
    for (int e = 0; e < A; e++) {
        double pos = std::fabs((A - e - 1) / (double)(A - 1));
        pos = pos - std::sin(2 * M_PI * pos) / (2 * M_PI);
        out[e] = (float)(coef * pos);
    }
}

void default_layout(sa_plan* p) {
    if (p->layout_fixed) return;
    set_strips(p, min_strips(p));
    // about one wave of 12 warps on each of the 152 SMs; each chunk keeps >= 2 pipeline depths of rows
    const int minrows = 4 * radius(p);
    const int shots = std::max(1, npairs(p));
    const int warps_per_chunk = p->nstrips * shots * ((p->NT + 31) / 32);
    const int target = 152 * 12;
    int nchunks = (target + warps_per_chunk - 1) / warps_per_chunk;
    nchunks = std::max(1, std::min(nchunks, p->nx / minrows));
    p->chunk_rows = (p->nx + nchunks - 1) / nchunks;
    p->nchunks = (p->nx + p->chunk_rows - 1) / p->chunk_rows;
}

struct HostInject {
    int cta, row, col, point;
    float coef;
    int lane;
};

// Builds the per-CTA source/receiver lists for the current layout. The captured graphs hold the
// list pointers (not their contents): they are dropped only when a list moves.
int build_lists_impl(sa_plan* p);
int build_lists(sa_plan* p) {
    const void* before[] = {p->gat_flat, p->src_flat, p->gat_src, p->hgat, p->hgat_src, p->rtgt.idx, p->rtgt.off, p->rtgt.point,
                            p->rtgt.coef, p->stgt.idx, p->stgt.off, p->stgt.point, p->stgt.coef, p->xtgt.idx,
                            p->xtgt.off, p->xtgt.point, p->xtgt.coef};
    const int counts_before[3] = {p->stgt.n, p->rtgt.n, p->xtgt.n};
    const int rc = build_lists_impl(p);
    const void* after[] = {p->gat_flat, p->src_flat, p->gat_src, p->hgat, p->hgat_src, p->rtgt.idx, p->rtgt.off, p->rtgt.point,
                           p->rtgt.coef, p->stgt.idx, p->stgt.off, p->stgt.point, p->stgt.coef, p->xtgt.idx,
                           p->xtgt.off, p->xtgt.point, p->xtgt.coef};
    if (counts_before[0] != p->stgt.n || counts_before[1] != p->rtgt.n || counts_before[2] != p->xtgt.n)
        drop_graphs(p);  // the injection kernels' launch sizes are captured
    for (size_t k = 0; k < sizeof(before) / sizeof(before[0]); k++)
        if (before[k] != after[k]) {
            drop_graphs(p);
            break;
        }
    return rc;
}

int build_lists_impl(sa_plan* p) {
    const int nc = p->nchunks, ns = p->nstrips;
    const double h = std::max(p->d.spacing[0], p->d.spacing[1]);
    const double dt = p->d.dt;
    // shots advance in pairs (the two lanes of a float2); CTA index of (pair, chunk, strip)
    auto cta_of = [&](int shot, int x, int y) { return ((shot / 2) * nc + x / p->chunk_rows) * ns + y / p->by; };
    // corner(x, y): the per-corner factor of the coefficient (vp, vp^2 or C1 W there)
    // linear: the 4 corners; Hicks / sinc: the width x width support from base - lo (smooth: the
    // Hicks sources' smoothing)
    const int interp = p->d.interpolation;
    const bool wide = interp != SA_INTERP_LINEAR;
    const int lo = sa::support_lo(interp);
    auto make_inj = [&](const std::vector<int>& off, const std::vector<int>& bx, const std::vector<int>& by,
                        const std::vector<double>& fx, const std::vector<double>& fy, double scale, auto corner,
                        std::vector<HostInject>& out, bool smooth) {
        out.clear();
        for (int s = 0; s < p->n_shots; s++)
            for (int i = off[s]; i < off[s + 1]; i++) {
                if (wide) {
                    double cxs[sa::SUPPORT_MAX], cys[sa::SUPPORT_MAX];
                    const int width = sa::support_coefs(interp, fx[i], smooth, cxs);
                    sa::support_coefs(interp, fy[i], smooth, cys);
                    for (int a = 0; a < width; a++)
                        for (int b = 0; b < width; b++) {
                            const double w = cxs[a] * cys[b];
                            if (w == 0.0) continue;
                            const int x = bx[i] - lo + a, y = by[i] - lo + b;
                            out.push_back({cta_of(s, x, y), x, y, i, (float)(w * scale * corner(x, y)), s & 1});
                        }
                    continue;
                }
                for (int cx = 0; cx < 2; cx++)
                    for (int cy = 0; cy < 2; cy++) {
                        const int x = bx[i] + cx, y = by[i] + cy;
                        const double w = (cx ? fx[i] : 1.0 - fx[i]) * (cy ? fy[i] : 1.0 - fy[i]);
                        out.push_back({cta_of(s, x, y), x, y, i, (float)(w * scale * corner(x, y)), s & 1});
                    }
            }
        std::stable_sort(out.begin(), out.end(), [](const HostInject& a, const HostInject& b) {
            return a.cta != b.cta ? a.cta < b.cta : a.row < b.row;
        });
    };
    // the entries grouped by target point for the injection kernels (one thread per target, entries
    // summed in a fixed order: deterministic without atomics)
    auto make_targets = [&](const std::vector<HostInject>& in, Targets& T) -> int {
        std::vector<std::pair<long long, size_t>> keyed(in.size());
        for (size_t k = 0; k < in.size(); k++) {
            const long long pair = in[k].cta / (nc * ns);
            keyed[k] = {2 * (pair * p->shot_stride + (long long)in[k].row * p->pitch + in[k].col) + in[k].lane, k};
        }
        std::stable_sort(keyed.begin(), keyed.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
        std::vector<long long> tidx;
        std::vector<int> toff, tpoint;
        std::vector<float> tcoef;
        for (size_t k = 0; k < keyed.size(); k++) {
            if (k == 0 || keyed[k].first != keyed[k - 1].first) {
                tidx.push_back(keyed[k].first);
                toff.push_back((int)k);
            }
            tcoef.push_back(in[keyed[k].second].coef);
            tpoint.push_back(in[keyed[k].second].point);
        }
        toff.push_back((int)keyed.size());
        T.n = (int)tidx.size();
        T.hidx = tidx;
        CKR(ensure(&T.idx, &T.cap_idx, tidx.size()));
        CKR(ensure(&T.off, &T.cap_off, toff.size()));
        CKR(ensure(&T.coef, &T.cap_coef, tcoef.size()));
        CKR(ensure(&T.point, &T.cap_point, tpoint.size()));
        if (!tidx.empty()) {
            CK(cudaMemcpy(T.idx, tidx.data(), tidx.size() * sizeof(long long), cudaMemcpyHostToDevice));
            CK(cudaMemcpy(T.coef, tcoef.data(), tcoef.size() * sizeof(float), cudaMemcpyHostToDevice));
            CK(cudaMemcpy(T.point, tpoint.data(), tpoint.size() * sizeof(int), cudaMemcpyHostToDevice));
        }
        CK(cudaMemcpy(T.off, toff.data(), toff.size() * sizeof(int), cudaMemcpyHostToDevice));
        return SA_OK;
    };
    std::vector<HostInject> tmp;
    // forward source: src * 2 dt^2 vp / h / dt (iso_acoustic/devito.py:349-363), vp at the corner
    auto vp_at = [&](int x, int y) { return p->vp_host.empty() ? 0.0 : (double)p->vp_host[(size_t)x * p->ny + y]; };
    auto vp2_at = [&](int x, int y) {
        const float v = p->vp_host.empty() ? 0.f : p->vp_host[(size_t)x * p->ny + y];
        return (double)(v * v);
    };
    auto c1w_at = [&](int x, int y) { return p->c1w_host.empty() ? 0.0 : (double)p->c1w_host[(size_t)x * p->ny + y]; };
    make_inj(p->src_off, p->src_bx, p->src_by, p->src_fx, p->src_fy, 2.0 * dt / h, vp_at, tmp, true);
    CKR(make_targets(tmp, p->stgt));
    // adjoint receiver: -rec * dt^2 * vp^2 (devito.py:748-753), vp^2 at the corner
    make_inj(p->rec_off, p->rec_bx, p->rec_by, p->rec_fx, p->rec_fy, -dt * dt, vp2_at, tmp, false);
    CKR(make_targets(tmp, p->rtgt));
    // exact-gradient adjoint: dL/drec injected with the update's own C1 W at the corner
    make_inj(p->rec_off, p->rec_bx, p->rec_by, p->rec_fx, p->rec_fy, 1.0, c1w_at, tmp, false);
    CKR(make_targets(tmp, p->xtgt));
    {  // the sources' support points with their raw weights, for the exact gradient's source term
        make_inj(p->src_off, p->src_bx, p->src_by, p->src_fx, p->src_fy, 1.0, [](int, int) { return 1.0; }, tmp, true);
        std::vector<sa::ExactSrc2D> sf;
        for (const HostInject& e : tmp) {
            const long long pair = e.cta / (nc * ns), pl = (long long)e.row * p->pitch + e.col;
            sf.push_back({pair * p->shot_stride + pl, (int)pl, e.lane, e.point, e.coef});
        }
        CKR(ensure(&p->src_flat, &p->cap_src_flat, std::max<size_t>(1, sf.size())));
        if (!sf.empty())
            CK(cudaMemcpy(p->src_flat, sf.data(), sf.size() * sizeof(sa::ExactSrc2D), cudaMemcpyHostToDevice));
        p->n_src_flat = (int)sf.size();
    }
    // gathers, one per point, owned by the CTA of its base corner: receivers (the forward's traces)
    // and sources with negated weights (the adjoint's wavelet gradient, -interp(p_a))
    auto make_gathers = [&](const std::vector<int>& off, const std::vector<int>& bx, const std::vector<int>& by,
                            const std::vector<double>& fx, const std::vector<double>& fy, float sign,
                            sa::Gather** dflat, size_t* capf) -> int {
        std::vector<sa::Gather> flat;
        for (int s = 0; s < p->n_shots; s++)
            for (int r = off[s]; r < off[s + 1]; r++) {
                sa::Gather G;
                G.row = bx[r];
                G.col = by[r];
                G.point = r;
                G.pad = s;
                G.w00 = sign * (float)((1 - fx[r]) * (1 - fy[r]));
                G.w01 = sign * (float)((1 - fx[r]) * fy[r]);
                G.w10 = sign * (float)(fx[r] * (1 - fy[r]));
                G.w11 = sign * (float)(fx[r] * fy[r]);
                flat.push_back(G);
            }
        CKR(ensure(dflat, capf, flat.size()));
        if (!flat.empty())
            CK(cudaMemcpy(*dflat, flat.data(), flat.size() * sizeof(sa::Gather), cudaMemcpyHostToDevice));
        return SA_OK;
    };
    CKR(make_gathers(p->rec_off, p->rec_bx, p->rec_by, p->rec_fx, p->rec_fy, 1.f, &p->gat_flat, &p->cap_gat_flat));
    CKR(make_gathers(p->src_off, p->src_bx, p->src_by, p->src_fx, p->src_fy, -1.f, &p->gat_src, &p->cap_gat_src));
    // gathers over the width x width support: receivers (the forward's traces) and, negated (and for
    // Hicks smoothed as the sources are), the sources (the adjoint's wavelet gradient, -interp(p_a))
    auto make_support = [&](const std::vector<int>& off, const std::vector<int>& bx, const std::vector<int>& by,
                          const std::vector<double>& fx, const std::vector<double>& fy, bool smooth, float sign,
                          sa::SupportGather** dst, size_t* cap) -> int {
        std::vector<sa::SupportGather> hg;
        for (int s = 0; s < p->n_shots; s++)
            for (int r = off[s]; r < off[s + 1]; r++) {
                sa::SupportGather G{};
                G.row = bx[r] - lo;
                G.col = by[r] - lo;
                G.point = r;
                G.shot = s;
                double cx[sa::SUPPORT_MAX], cy[sa::SUPPORT_MAX];
                G.width = sa::support_coefs(interp, fx[r], smooth, cx);
                sa::support_coefs(interp, fy[r], smooth, cy);
                for (int k = 0; k < sa::SUPPORT_MAX; k++) {
                    G.wx[k] = sign * (float)cx[k];
                    G.wy[k] = (float)cy[k];
                }
                hg.push_back(G);
            }
        CKR(ensure(dst, cap, hg.size()));
        if (!hg.empty())
            CK(cudaMemcpy(*dst, hg.data(), hg.size() * sizeof(sa::SupportGather), cudaMemcpyHostToDevice));
        return SA_OK;
    };
    if (wide) {
        CKR(make_support(p->rec_off, p->rec_bx, p->rec_by, p->rec_fx, p->rec_fy, false, 1.f, &p->hgat, &p->cap_hgat));
        CKR(make_support(p->src_off, p->src_bx, p->src_by, p->src_fx, p->src_fy, true, -1.f, &p->hgat_src,
                       &p->cap_hgat_src));
    }
    return SA_OK;
}

const float* row0(const sa_plan* p, const float* alloc, int pitch, int extra_rows = 0) {
    return alloc + (long long)(sa::GUARD + extra_rows) * pitch;
}

sa::Step2D base_args(const sa_plan* p) {
    sa::Step2D a{};
    a.nx = p->nx;
    a.ny = p->ny;
    a.pitch = p->pitch;
    a.shot_stride = p->shot_stride;
    a.chunk_rows = p->chunk_rows;
    a.by = p->by;
    a.lbuf = p->lbuf;
    sa::step_medium(a, p->smed, p->nx, p->ny);
    sa::step_weights(a, p->kind, p->d.spacing[0], p->d.spacing[1], p->d.dt);
    a.f = p->d.undersampling;
    a.snaps = p->snaps;
    a.snap_stride = p->snap_stride;
    a.snap_shot_stride = p->snap_shot_stride;
    return a;
}

// Adjoint receiver injection into the new level q[t-1] (devito.py:748-753): res[t] at every
// target point, its entries summed in a fixed order.
int inject_receivers(const sa_plan* p, float* level, int t, cudaStream_t s, long long& n) {
    if (!p->rtgt.n) return SA_OK;
    CK(sa::inject_targets2d(level, p->rtgt.idx, p->rtgt.off, p->rtgt.coef, p->rtgt.point, p->rtgt.n, p->rec_amp,
                            p->n_rec, t, nullptr, 0, 0, 0, 0.f, s));
    n++;
    return SA_OK;
}

// Forward source injection into the new level p[t+1] (devito.py:357-363); on a save step the
// injected amount / dt^2 also enters that level's p.dt2 snapshot (snaps_base: the snapshot
// array as the step kernel addresses it, slot t/f).
int inject_sources(const sa_plan* p, float* level, int t, const float* snaps_base, long long snap_shot_stride,
                   bool save_now, cudaStream_t s, long long& n) {
    if (!p->stgt.n) return SA_OK;
    float* snap = save_now ? const_cast<float*>(snaps_base) + 2 * (long long)(t / p->d.undersampling) * p->snap_stride
                           : nullptr;
    CK(sa::inject_targets2d(level, p->stgt.idx, p->stgt.off, p->stgt.coef, p->stgt.point, p->stgt.n, p->src_amp,
                            p->n_src, t, snap, p->shot_stride, snap_shot_stride, 0,
                            (float)(1.0 / (p->d.dt * p->d.dt)), s));
    n++;
    return SA_OK;
}

int image_step(const sa_plan* p, const float* q, const float* snaps_base, long long snap_shot_stride, int t,
               cudaStream_t s, long long& n) {
    const int f = p->d.undersampling;
    if (t % f) return SA_OK;
    const float* snap = snaps_base + (long long)(t / f) * p->snap_stride * 2;
    CK(sa::image2d(q, snap, p->gradb, p->precb, p->d.absorbing[0], p->nx - p->d.absorbing[0], p->d.absorbing[1],
                   p->ny - p->d.absorbing[1], p->pitch, npairs(p), p->shot_stride, snap_shot_stride, s));
    n++;
    return SA_OK;
}

// The CFS-PML after the step of level cur (new level nxt, its p.dt2 snapshot slot snap or null):
// auxiliary fields of the absorbing slabs and the boundary term of the new level.
// aux: the auxiliary fields advanced (default: the plan's), snap_pair: snapshot stride per pair.
int pml_step(const sa_plan* p, const float* cur, float* nxt, bool adjoint, float* snap, cudaStream_t s,
             long long& n, float* aux = nullptr, long long snap_pair = -1) {
    if (!p->pml) return SA_OK;
    CK(sa::pml2d(cur, nxt, aux ? aux : p->pml_aux, p->pml_prof, row0(p, p->C1, p->pitch), p->vp, p->nx, p->ny,
                 p->pitch, p->shot_stride, npairs(p), p->d.absorbing[0], p->d.absorbing[1], (float)p->d.spacing[0],
                 (float)p->d.spacing[1], (float)p->d.dt, adjoint ? 1 : 0, snap,
                 snap_pair >= 0 ? snap_pair : p->snap_shot_stride, (float)(1.0 / (p->d.dt * p->d.dt)), s));
    n++;
    return SA_OK;
}

size_t pml_aux_bytes(const sa_plan* p) { return 6 * 2 * (size_t)npairs(p) * p->shot_stride * sizeof(float); }

int pml_clear(const sa_plan* p, cudaStream_t s, float* aux = nullptr) {
    if (p->pml) CK(cudaMemsetAsync(aux ? aux : p->pml_aux, 0, pml_aux_bytes(p), s));
    return SA_OK;
}

// Imaging from raw snapshots (SA_SAVE_RAW): on t % f == 0 the held vp (and rho) terms are
// recomputed from slots t/f - 1 .. t/f + 1, and every step accumulates them against q = p_a[t]
// (the reference's unconditioned Inc of a Function written under the undersampling condition,
// iso_acoustic/devito.py:1007-1024, 1133-1150).
int image_raw_step(const sa_plan* p, const float* q, int t, bool rho, cudaStream_t s, long long& n) {
    const int f = p->d.undersampling;
    const bool refresh = t % f == 0;
    const float* snap = p->snaps + (long long)(refresh ? t / f : 0) * p->snap_stride * 2;
    const double fdt = (double)f * p->d.dt;
    CK(sa::image_raw2d(q, snap, p->snap_stride, p->snap_shot_stride, refresh ? 1 : 0, (float)(1.0 / (fdt * fdt)),
                       p->hold_vp, rho ? p->hold_rho : nullptr, p->buoy, p->dbx, p->dby, (float)p->d.spacing[0],
                       (float)p->d.spacing[1], p->nx, p->ny, p->gradb, p->precb, p->gradrb, p->precrb,
                       p->d.absorbing[0], p->nx - p->d.absorbing[0], p->d.absorbing[1], p->ny - p->d.absorbing[1],
                       p->pitch, npairs(p), p->shot_stride, s));
    n++;
    return SA_OK;
}

// Issues the forward time loop t = 1..nt-2 (iso_acoustic/devito.py:575-581) on stream s.
// SA_SAVE_SNAPSHOTS saves p.dt2 every f steps, SA_SAVE_RAW p[t] itself (its slots the loop does
// not write, n = 0 and n f > nt-2, are zeroed as the reference's fresh buffer);
// SA_SAVE_CHECKPOINTS copies both levels (p[t+1], p[t]) after every step t = kK, k = 1..ck_n,
// into checkpoint slot k-1.
int issue_forward(sa_plan* p, int mode, cudaStream_t s) {
    const bool save = mode == SA_SAVE_SNAPSHOTS;
    const bool raw = mode == SA_SAVE_RAW;
    const bool wide = p->d.interpolation != SA_INTERP_LINEAR;  // a wide support (Hicks or sinc)
    const size_t fbytes = (size_t)npairs(p) * p->shot_stride * sizeof(float2);
    CK(cudaMemsetAsync(p->field[0], 0, fbytes, s));
    CK(cudaMemsetAsync(p->field[1], 0, fbytes, s));
    CK(cudaMemsetAsync(p->rec_amp, 0, (size_t)p->d.nt * p->n_rec * sizeof(float), s));
    sa::Step2D a = base_args(p);  // sources and receivers are handled by their own kernels after the step
    a.save = save ? 1 : (raw ? 2 : 0);
    const dim3 grid(p->nstrips, p->nchunks, npairs(p));
    long long n = 0;
    CKR(pml_clear(p, s));
    if (raw) {
        const int f = p->d.undersampling, last = (p->d.nt - 2) / f;  // slots 1..last are written
        const size_t slot = (size_t)p->snap_stride * 2 * sizeof(float);
        const size_t pitchb = (size_t)p->snap_shot_stride * 2 * sizeof(float);
        CK(cudaMemset2DAsync(p->snaps, pitchb, 0, slot, npairs(p), s));
        if (last + 1 < p->n_snap)
            CK(cudaMemset2DAsync(p->snaps + (size_t)(last + 1) * p->snap_stride * 2, pitchb, 0,
                                 (size_t)(p->n_snap - last - 1) * slot, npairs(p), s));
    }
    for (int t = 1; t <= p->d.nt - 2; t++) {
        a.t = t;
        a.cur = (t & 1) ? p->field[1] : p->field[0];
        a.prev = (t & 1) ? p->field[0] : p->field[1];
        CK(sa::launch_step2d(p->kind, p->ot4, p->NT, grid, s, a));
        n++;
        const bool save_now = save && t % p->d.undersampling == 0;
        float* snap_now = save_now ? p->snaps + 2 * (long long)(t / p->d.undersampling) * p->snap_stride : nullptr;
        CKR(pml_step(p, a.cur, a.prev, false, snap_now, s, n));
        if (wide || !p->n_rec || t == 1) {
            CKR(inject_sources(p, a.prev, t, p->snaps, p->snap_shot_stride, save_now, s, n));
        } else {  // this step's sources into p[t+1] and the previous step's rec[t-1] = interp(p[t]), one launch
            CK(sa::inject_gather2d(a.prev, p->stgt.idx, p->stgt.off, p->stgt.coef, p->stgt.point, p->stgt.n,
                                   p->src_amp, p->n_src, t, snap_now, p->shot_stride, p->snap_shot_stride,
                                   (float)(1.0 / (p->d.dt * p->d.dt)), a.cur, p->pitch, p->gat_flat, p->n_rec,
                                   p->rec_amp, p->n_rec, t - 1, s));
            n++;
        }
        if (p->n_rec && wide) {  // rec[t] = interp(p[t+1]) over the wide support
            CK(sa::support_gather2d(a.prev, p->shot_stride, p->pitch, p->hgat, p->n_rec, p->rec_amp, p->n_rec, t, s));
            n++;
        }
        if (p->n_rec && !wide && t == p->d.nt - 2) {  // the last step's receivers
            CK(sa::final_gather2d(a.prev, p->shot_stride, p->pitch, p->gat_flat, p->n_rec, p->rec_amp, p->n_rec, t,
                                  s));
            n++;
        }
        if (mode == SA_SAVE_CHECKPOINTS && t % p->ck_K == 0 && t / p->ck_K <= p->ck_n) {
            float* slot = p->ckpt + (size_t)(t / p->ck_K - 1) * 2 * (fbytes / sizeof(float));
            CK(cudaMemcpyAsync(slot, p->field[0], fbytes, cudaMemcpyDeviceToDevice, s));
            CK(cudaMemcpyAsync(slot + fbytes / sizeof(float), p->field[1], fbytes, cudaMemcpyDeviceToDevice, s));
            if (p->pml)  // the CFS-PML's auxiliary fields after step t
                CK(cudaMemcpyAsync(p->pml_ck + (size_t)(t / p->ck_K - 1) * (pml_aux_bytes(p) / sizeof(float)),
                                   p->pml_aux, pml_aux_bytes(p), cudaMemcpyDeviceToDevice, s));
        }
    }
    p->fwd_launches[mode] = n;
    return SA_OK;
}

// Issues the reverse-time adjoint loop t = nt-1-f .. 1 (devito.py:915-920).
// The wavelet gradient: -interp(p_a[t]) at the sources into wgrad row t (negated gather weights).
int wavelet_gather(const sa_plan* p, const float* q, int t, bool wav, cudaStream_t s, long long& n) {
    if (!wav || !p->n_src) return SA_OK;
    if (p->d.interpolation != SA_INTERP_LINEAR)
        CK(sa::support_gather2d(q, p->shot_stride, p->pitch, p->hgat_src, p->n_src, p->wgrad, p->n_src, t, s));
    else
        CK(sa::final_gather2d(q, p->shot_stride, p->pitch, p->gat_src, p->n_src, p->wgrad, p->n_src, t, s));
    n++;
    return SA_OK;
}

// The imaging condition (grad += snap q, prec += snap^2, interior, t % f == 0) runs as its own
// streaming kernel after the step of level t: in the step kernel's epilogue its dependent loads
// stalled the adjoint (6 % slower overall).
int issue_adjoint(sa_plan* p, bool wav, bool raw, bool rho, cudaStream_t s) {
    const size_t fbytes = (size_t)npairs(p) * p->shot_stride * sizeof(float2);
    const size_t gbytes = (size_t)npairs(p) * p->shot_stride * sizeof(float);
    CK(cudaMemsetAsync(p->field[0], 0, fbytes, s));
    CK(cudaMemsetAsync(p->field[1], 0, fbytes, s));
    CK(cudaMemsetAsync(p->gradb, 0, gbytes, s));
    CK(cudaMemsetAsync(p->precb, 0, gbytes, s));
    if (raw) {  // held terms start at zero (a fresh Function)
        CK(cudaMemsetAsync(p->hold_vp, 0, fbytes, s));
        if (rho) {
            CK(cudaMemsetAsync(p->hold_rho, 0, fbytes, s));
            CK(cudaMemsetAsync(p->gradrb, 0, gbytes, s));
            CK(cudaMemsetAsync(p->precrb, 0, gbytes, s));
        }
    }
    sa::Step2D a = base_args(p);  // receivers are injected by inject_targets2d after the step
    a.save = 0;
    if (wav) CK(cudaMemsetAsync(p->wgrad, 0, (size_t)p->d.nt * p->n_src * sizeof(float), s));
    const dim3 grid(p->nstrips, p->nchunks, npairs(p));
    const int T0 = p->d.nt - 1 - p->d.undersampling;
    long long n = 0;
    CKR(pml_clear(p, s));
    for (int t = T0; t >= 1; t--) {
        a.t = t;
        const bool even = ((T0 - t) & 1) == 0;
        a.cur = even ? p->field[1] : p->field[0];
        a.prev = even ? p->field[0] : p->field[1];
        CK(sa::launch_step2d(p->kind, p->ot4, p->NT, grid, s, a));
        n++;
        CKR(pml_step(p, a.cur, a.prev, true, nullptr, s, n));
        CKR(inject_receivers(p, a.prev, t, s, n));
        if (raw)
            CKR(image_raw_step(p, a.cur, t, rho, s, n));
        else
            CKR(image_step(p, a.cur, p->snaps, p->snap_shot_stride, t, s, n));
        CKR(wavelet_gather(p, a.cur, t, wav, s, n));
    }
    p->adj_launches[raw ? (rho ? 4 : 3) : 0] = n;
    return SA_OK;
}

// Reverse-time adjoint from checkpoints: the same steps and gradient as issue_adjoint, with
// the snapshots recomputed per segment. Coarse segment k covers t = kK+1 .. min((k+1)K, T0);
// from last to first, its start state (checkpoint k, zero for k = 0) is restored. With two
// levels (ck_K2 > 0) the coarse segment's forward steps are first re-run without snapshots to
// place fine checkpoints after steps kK + jK2. Each fine segment (the whole coarse one with one
// level), last to first, then restores its start state, re-runs its forward steps with p.dt2
// saved into a segment buffer of K2/f slots, and runs the adjoint steps back through it on
// their own two levels. The recomputed steps are the forward's own launches (no receiver
// gather), so the snapshots are bitwise the ones SA_SAVE_SNAPSHOTS stores.
int issue_adjoint_ckpt(sa_plan* p, bool wav, cudaStream_t s) {
    const size_t fbytes = (size_t)npairs(p) * p->shot_stride * sizeof(float2);
    const size_t ffloats = fbytes / sizeof(float);
    const size_t gbytes = (size_t)npairs(p) * p->shot_stride * sizeof(float);
    const size_t abytes = p->pml ? pml_aux_bytes(p) : 0, afloats = abytes / sizeof(float);
    CK(cudaMemsetAsync(p->afield[0], 0, fbytes, s));
    CK(cudaMemsetAsync(p->afield[1], 0, fbytes, s));
    CK(cudaMemsetAsync(p->gradb, 0, gbytes, s));
    CK(cudaMemsetAsync(p->precb, 0, gbytes, s));
    const int f = p->d.undersampling, K = p->ck_K;
    const int K2 = p->ck_K2 > 0 ? p->ck_K2 : K;  // fine interval (one level: the coarse one)
    const int T0 = p->d.nt - 1 - f;
    sa::Step2D fa = base_args(p);  // sources are injected by inject_targets2d after the step
    fa.save = 1;
    fa.snap_shot_stride = (long long)(K2 / f) * p->shot_stride;
    sa::Step2D fr = base_args(p);  // the recompute that places fine checkpoints saves nothing
    fr.save = 0;
    sa::Step2D aa = base_args(p);  // receivers are injected by inject_targets2d after the step
    aa.save = 0;
    aa.snap_shot_stride = fa.snap_shot_stride;
    if (wav) CK(cudaMemsetAsync(p->wgrad, 0, (size_t)p->d.nt * p->n_src * sizeof(float), s));
    const dim3 grid(p->nstrips, p->nchunks, npairs(p));
    long long n = 0;
    CKR(pml_clear(p, s));  // the adjoint's own auxiliary fields
    // forward state <- coarse checkpoint k (fine < 0) or fine checkpoint `fine`; zero for coarse 0
    auto restore = [&](int k, int fine) -> int {
        if (fine < 0 && k == 0) {
            CK(cudaMemsetAsync(p->field[0], 0, fbytes, s));
            CK(cudaMemsetAsync(p->field[1], 0, fbytes, s));
            return pml_clear(p, s, p->pml_aux_f);
        }
        const float* lv = fine < 0 ? p->ckpt + (size_t)(k - 1) * 2 * ffloats : p->ckpt2 + (size_t)fine * 2 * ffloats;
        CK(cudaMemcpyAsync(p->field[0], lv, fbytes, cudaMemcpyDeviceToDevice, s));
        CK(cudaMemcpyAsync(p->field[1], lv + ffloats, fbytes, cudaMemcpyDeviceToDevice, s));
        if (p->pml) {
            const float* ax = fine < 0 ? p->pml_ck + (size_t)(k - 1) * afloats : p->pml_ck2 + (size_t)fine * afloats;
            CK(cudaMemcpyAsync(p->pml_aux_f, ax, abytes, cudaMemcpyDeviceToDevice, s));
        }
        return SA_OK;
    };
    auto forward_step = [&](sa::Step2D& a, int t, float* base) -> int {
        const bool save_now = base != nullptr && t % f == 0;
        a.t = t;
        a.cur = (t & 1) ? p->field[1] : p->field[0];
        a.prev = (t & 1) ? p->field[0] : p->field[1];
        CK(sa::launch_step2d(p->kind, p->ot4, p->NT, grid, s, a));
        n++;
        CKR(pml_step(p, a.cur, a.prev, false, save_now ? base + 2 * (long long)(t / f) * p->snap_stride : nullptr, s,
                     n, p->pml_aux_f, fa.snap_shot_stride));
        return inject_sources(p, a.prev, t, base, fa.snap_shot_stride, save_now, s, n);
    };
    for (int k = T0 >= 1 ? (T0 - 1) / K : -1; k >= 0; k--) {
        const int c0 = k * K, c_hi = std::min((k + 1) * K, T0);
        const int nf = (c_hi - c0 + K2 - 1) / K2;  // fine segments
        if (nf > 1) {  // fine checkpoints j = 1 .. nf-1 into slots j-1
            CKR(restore(k, -1));
            for (int t = c0 + 1; t <= c0 + (nf - 1) * K2; t++) {
                CKR(forward_step(fr, t, nullptr));
                if ((t - c0) % K2 == 0) {
                    const size_t j = (size_t)((t - c0) / K2 - 1);
                    CK(cudaMemcpyAsync(p->ckpt2 + j * 2 * ffloats, p->field[0], fbytes, cudaMemcpyDeviceToDevice, s));
                    CK(cudaMemcpyAsync(p->ckpt2 + j * 2 * ffloats + ffloats, p->field[1], fbytes,
                                       cudaMemcpyDeviceToDevice, s));
                    if (p->pml)
                        CK(cudaMemcpyAsync(p->pml_ck2 + j * afloats, p->pml_aux_f, abytes, cudaMemcpyDeviceToDevice,
                                           s));
                }
            }
        }
        for (int j = nf - 1; j >= 0; j--) {
            const int t_lo = c0 + j * K2 + 1, t_hi = std::min(c0 + (j + 1) * K2, c_hi);
            CKR(restore(k, j - 1));
            // the kernels address snapshot t/f; slot t/f - ((c0 + jK2)/f + 1) of the segment buffer is meant
            const long long first = (long long)(c0 + j * K2) / f + 1;
            float* base = reinterpret_cast<float*>(reinterpret_cast<uintptr_t>(p->segsnaps) -
                                                   (uintptr_t)(first * p->shot_stride * (long long)sizeof(float2)));
            fa.snaps = aa.snaps = base;
            for (int t = t_lo; t <= t_hi; t++) CKR(forward_step(fa, t, base));
            for (int t = t_hi; t >= t_lo; t--) {
                aa.t = t;
                const bool even = ((T0 - t) & 1) == 0;
                aa.cur = even ? p->afield[1] : p->afield[0];
                aa.prev = even ? p->afield[0] : p->afield[1];
                CK(sa::launch_step2d(p->kind, p->ot4, p->NT, grid, s, aa));
                n++;
                CKR(pml_step(p, aa.cur, aa.prev, true, nullptr, s, n));
                CKR(inject_receivers(p, aa.prev, t, s, n));
                CKR(image_step(p, aa.cur, base, aa.snap_shot_stride, t, s, n));
                CKR(wavelet_gather(p, aa.cur, t, wav, s, n));
            }
        }
    }
    p->adj_launches[1] = n;
    return SA_OK;
}

int plan_checkpoints(sa_plan* p) {
    // a checkpoint holds both levels and, with the CFS-PML, its six auxiliary fields (six more levels)
    return sa::choose_checkpoints(p->d, (double)npairs(p) * p->shot_stride * sizeof(float2), &p->ck_K, &p->ck_n,
                                  p->pml ? 8 : 2, &p->ck_K2);
}

// Exact gradient of the discrete forward map (SA_GRAD_EXACT) from checkpoints. With z = C1 W mu
// the adjoint obeys the forward recursion: adjoint step t (t = nt .. 2) computes z[t-1] from
// z[t], z[t+1] with dL/drec[t-2] injected with coefficient C1 W, and for t <= nt-1 adds the
// contribution of forward step t-1 (exact2d.cu), which needs the levels u[t], u[t-1], u[t-2]
// and, for OT4, W G u[t-1] and W G z[t]. Segment k covers t = kK+2 .. min((k+1)K+1, nt): its
// levels u[kK] .. are rebuilt from checkpoint k into `levels` (slot = level - kK); W G(.) is the
// OT2 step kernel with C1 = 1, C2 = C3 = 0.
int issue_adjoint_exact(sa_plan* p, cudaStream_t s) {
    const size_t fbytes = (size_t)npairs(p) * p->shot_stride * sizeof(float2);
    const size_t ffl = fbytes / sizeof(float);
    const size_t gbytes = (size_t)npairs(p) * p->shot_stride * sizeof(float);
    const int nt = p->d.nt, K = p->ck_K;
    CK(cudaMemsetAsync(p->afield[0], 0, fbytes, s));
    CK(cudaMemsetAsync(p->afield[1], 0, fbytes, s));
    CK(cudaMemsetAsync(p->gradb, 0, gbytes, s));
    CK(cudaMemsetAsync(p->precb, 0, gbytes, s));
    sa::Step2D fa = base_args(p);  // forward recompute (sources injected after each step)
    fa.save = 0;
    sa::Step2D aa = fa;  // adjoint (dL/drec[t-2] injected after step t)
    sa::Step2D la = fa;  // W G(cur) into prev
    la.wg_only = 1;
    const dim3 grid(p->nstrips, p->nchunks, npairs(p));
    const float inv_dt2 = (float)(1.0 / (p->d.dt * p->d.dt));
    const float src_scale = (float)(2.0 * p->d.dt / std::max(p->d.spacing[0], p->d.spacing[1]));
    auto level = [&](int k, int m) { return p->levels + (size_t)(m - k * K) * ffl; };
    long long n = 0;
    for (int k = (nt - 2) / K; k >= 0; k--) {
        const int t_lo = std::max(2, k * K + 2), t_hi = std::min((k + 1) * K + 1, nt);
        if (t_lo > t_hi) continue;
        if (k == 0) {
            CK(cudaMemsetAsync(p->field[0], 0, fbytes, s));
            CK(cudaMemsetAsync(p->field[1], 0, fbytes, s));
        } else {
            const float* slot = p->ckpt + (size_t)(k - 1) * 2 * ffl;
            CK(cudaMemcpyAsync(p->field[0], slot, fbytes, cudaMemcpyDeviceToDevice, s));
            CK(cudaMemcpyAsync(p->field[1], slot + ffl, fbytes, cudaMemcpyDeviceToDevice, s));
        }
        // u[kK] lives in field[kK & 1], u[kK+1] in the other
        CK(cudaMemcpyAsync(level(k, k * K), p->field[(k * K) & 1], fbytes, cudaMemcpyDeviceToDevice, s));
        CK(cudaMemcpyAsync(level(k, k * K + 1), p->field[(k * K + 1) & 1], fbytes, cudaMemcpyDeviceToDevice, s));
        for (int m = k * K + 1; m <= std::min((k + 1) * K, nt - 2); m++) {  // forward step m -> u[m+1]
            fa.t = m;
            fa.cur = p->field[m & 1];
            fa.prev = p->field[(m + 1) & 1];
            CK(sa::launch_step2d(p->kind, p->ot4, p->NT, grid, s, fa));
            CKR(inject_sources(p, fa.prev, m, nullptr, 0, false, s, n));
            CK(cudaMemcpyAsync(level(k, m + 1), p->field[(m + 1) & 1], fbytes, cudaMemcpyDeviceToDevice, s));
            n++;
        }
        for (int t = t_hi; t >= t_lo; t--) {
            float* zt = p->afield[t & 1];
            aa.t = t;
            aa.cur = zt;
            aa.prev = p->afield[(t + 1) & 1];
            CK(sa::launch_step2d(p->kind, p->ot4, p->NT, grid, s, aa));
            n++;
            if (p->xtgt.n) {  // z[t-1] += C1 W dL/drec[t-2] (rows read only for t >= 2)
                CK(sa::inject_targets2d(aa.prev, p->xtgt.idx, p->xtgt.off, p->xtgt.coef, p->xtgt.point, p->xtgt.n,
                                        p->rec_amp, p->n_rec, t - 2, nullptr, 0, 0, 0, 0.f, s));
                n++;
            }
            if (t > nt - 1) continue;  // z[nt] = 0
            const float *Lu = nullptr, *Lz = nullptr;
            if (p->ot4) {
                la.t = t - 1;
                la.cur = level(k, t - 1);
                la.prev = p->Lu;
                CK(sa::launch_step2d(p->kind, false, p->NT, grid, s, la));
                la.t = t;
                la.cur = zt;
                la.prev = p->Lz;
                CK(sa::launch_step2d(p->kind, false, p->NT, grid, s, la));
                Lu = p->Lu;
                Lz = p->Lz;
                n += 2;
            }
            CK(sa::exact_grad2d(zt, level(k, t), level(k, t - 1), level(k, t - 2), Lu, Lz, p->EA, p->EB, p->EC, p->EG4,
                                p->nx, p->ny, p->pitch, npairs(p), p->shot_stride, inv_dt2, p->gradb, p->precb, s));
            n++;
            if (p->n_src) {
                CK(sa::exact_src2d(zt, p->src_flat, p->n_src_flat, p->src_amp, p->n_src, t - 1, src_scale, p->ES,
                                   p->gradb, s));
                n++;
            }
        }
    }
    p->adj_launches[2] = n;
    return SA_OK;
}

// Runs `issue` through a cached CUDA graph (captured on the plan's own stream) or directly.
int medium_l2_window(sa_plan* p) {
    int dev = 0;
    CK(cudaGetDevice(&dev));
    int max_persist = 0, max_window = 0;
    CK(cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, dev));
    CK(cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, dev));
    const size_t bytes = std::min(sa::step_medium_size(p->nx, p->ny) * sizeof(float), (size_t)std::max(0, max_window));
    p->l2win = cudaAccessPolicyWindow{};
    if (max_persist <= 0 || bytes == 0) return SA_OK;  // no persisting L2 on this device
    size_t limit = 0;
    CK(cudaDeviceGetLimit(&limit, cudaLimitPersistingL2CacheSize));
    const size_t want = std::min(bytes, (size_t)max_persist);
    if (limit < want) {  // a limit of this process's context: raised, never lowered
        CK(cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, want));
        limit = want;
    }
    p->l2win.base_ptr = p->smed;
    p->l2win.num_bytes = bytes;
    p->l2win.hitRatio = (float)std::min(1.0, (double)limit / (double)bytes);
    p->l2win.hitProp = cudaAccessPropertyPersisting;
    p->l2win.missProp = cudaAccessPropertyStreaming;
    return SA_OK;
}

// Gives every kernel node of a captured loop the medium's persisting L2 window.
int apply_l2_window(const sa_plan* p, cudaGraph_t graph) {
    if (!p->l2win.num_bytes) return SA_OK;
    size_t n = 0;
    CK(cudaGraphGetNodes(graph, nullptr, &n));
    std::vector<cudaGraphNode_t> nodes(n);
    CK(cudaGraphGetNodes(graph, nodes.data(), &n));
    cudaKernelNodeAttrValue v{};
    v.accessPolicyWindow = p->l2win;
    for (cudaGraphNode_t nd : nodes) {
        cudaGraphNodeType t;
        CK(cudaGraphNodeGetType(nd, &t));
        if (t == cudaGraphNodeTypeKernel) CK(cudaGraphKernelNodeSetAttribute(nd, cudaKernelNodeAttributeAccessPolicyWindow, &v));
    }
    return SA_OK;
}

template <class F>
int run_loop(sa_plan* p, cudaGraphExec_t* slot, cudaStream_t s, F issue) {
    if (!p->use_graphs) return issue(s);
    if (!*slot) {
        if (!p->cap) CK(cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking));
        CK(cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal));
        const int rc = issue(p->cap);
        cudaGraph_t graph = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(p->cap, &graph);
        if (rc != SA_OK) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (ce != cudaSuccess) return fail(SA_E_CUDA, "graph capture: %s", cudaGetErrorString(ce));
        const int wr = apply_l2_window(p, graph);
        if (wr != SA_OK) {
            cudaGraphDestroy(graph);
            return wr;
        }
        const cudaError_t ie = cudaGraphInstantiate(slot, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) {
            *slot = nullptr;
            return fail(SA_E_CUDA, "graph instantiate: %s", cudaGetErrorString(ie));
        }
    }
    CK(cudaGraphLaunch(*slot, s));
    return SA_OK;
}

// Copies an [rows, cols] user matrix (host or device) into the time-major [cols, rows] buffer.
int load_transposed(sa_plan* p, const float* user, int rows, int cols, float* dst, cudaStream_t s) {
    const size_t n = (size_t)rows * cols;
    if (n == 0) return SA_OK;
    const float* src = user;
    if (!is_device(user)) {
        CKR(ensure(&p->stage, &p->cap_stage, n));
        CK(cudaMemcpyAsync(p->stage, user, n * sizeof(float), cudaMemcpyHostToDevice, s));
        src = p->stage;
    }
    CK(sa::transpose(src, rows, cols, dst, s));
    return SA_OK;
}

int store_transposed(sa_plan* p, const float* tm, int rows, int cols, float* user, cudaStream_t s) {
    // tm is [rows(time), cols(points)] -> user [cols, rows]
    const size_t n = (size_t)rows * cols;
    if (n == 0) return SA_OK;
    if (is_device(user)) {
        CK(sa::transpose(tm, rows, cols, user, s));
        return SA_OK;
    }
    CKR(ensure(&p->stage, &p->cap_stage, n));
    CK(sa::transpose(tm, rows, cols, p->stage, s));
    CK(cudaMemcpyAsync(user, p->stage, n * sizeof(float), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return SA_OK;
}

// The persistent forward: eligible for a plan with linear interpolation, the sponge and no saved
// wavefield; automatic when the whole batch is small (the streaming passes could not fill the
// GPU); its tiles are the smallest whose CTAs (one per tile and shot pair) are co-resident.
bool persist_layout(sa_plan* p) {
    const int kind = p->kind;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    const int pairs = npairs(p);
    long long best = -1;
    for (int ty = 16; ty <= 96; ty += 8)
        for (int tx = 8; tx <= 96; tx += 4) {
            const int tiles_x = (p->nx + tx - 1) / tx, tiles_y = (p->ny + ty - 1) / ty;
            const long long blocks = (long long)tiles_x * tiles_y * pairs;
            const size_t smem = sa::persist2d_smem(kind, p->ot4, tx, ty);
            const int per_sm = sa::persist2d_blocks_per_sm(kind, p->ot4, smem);
            if (per_sm < 1 || blocks > (long long)per_sm * sms) continue;
            const int H = (kind == 0 ? 5 : 9) * (p->ot4 ? 2 : 1);
            // points an SM loads per step: its CTAs share it
            const long long cost = (blocks + sms - 1) / sms * (long long)(tx + 2 * H) * (ty + 2 * H);
            if (best < 0 || cost < best) {
                best = cost;
                p->ptx = tx;
                p->pty = ty;
                p->ptiles_x = tiles_x;
                p->ptiles_y = tiles_y;
                p->pblocks = (int)blocks;
                p->psmem = smem;
            }
        }
    return best >= 0;
}

bool persist_eligible(const sa_plan* p) {
    return p->d.interpolation == SA_INTERP_LINEAR && p->d.boundary == SA_BOUNDARY_SPONGE;
}

// Automatic mode: the autotuner's measurement when it took one, else small batches only.
bool use_persistent(sa_plan* p, int save_mode) {
    if (p->persist_mode < 0 || save_mode != SA_SAVE_NONE || !persist_eligible(p)) return false;
    if (p->persist_mode == 0) {
        if (p->persist_tuned == 0) return false;
        if (p->persist_tuned < 0 && (long long)npairs(p) * p->nx * p->ny > 152LL * 4096) return false;
    }
    return persist_layout(p);
}

// nt_run: steps 1 .. nt_run-2 (the autotuner's short runs); 0 for the plan's nt.
int forward_persistent(sa_plan* p, cudaStream_t s, int nt_run = 0) {
    // the sources' targets by owning CTA (tile and shot pair of the target point), in target order
    const int ntile = p->ptiles_x * p->ptiles_y;
    std::vector<int> cnt(p->pblocks + 1, 0), tgt(p->stgt.n);
    std::vector<int> owner(p->stgt.n);
    for (int k = 0; k < p->stgt.n; k++) {
        const long long i = p->stgt.hidx[k];
        const long long pair = i / (2 * p->shot_stride), rem = (i % (2 * p->shot_stride)) / 2;
        const int x = (int)(rem / p->pitch), y = (int)(rem % p->pitch);
        owner[k] = (int)pair * ntile + (x / p->ptx) * p->ptiles_y + y / p->pty;
        cnt[owner[k] + 1]++;
    }
    for (int b = 0; b < p->pblocks; b++) cnt[b + 1] += cnt[b];
    std::vector<int> fill(cnt.begin(), cnt.end() - 1);
    for (int k = 0; k < p->stgt.n; k++) tgt[fill[owner[k]]++] = k;
    // the receivers by owning CTA (tile and shot pair of the base corner), in receiver order
    std::vector<int> rcnt(p->pblocks + 1, 0), ridx(p->n_rec), rown(p->n_rec);
    for (int sh = 0; sh < p->n_shots; sh++)
        for (int r = p->rec_off[sh]; r < p->rec_off[sh + 1]; r++) {
            rown[r] = (sh / 2) * ntile + (p->rec_bx[r] / p->ptx) * p->ptiles_y + p->rec_by[r] / p->pty;
            rcnt[rown[r] + 1]++;
        }
    for (int b = 0; b < p->pblocks; b++) rcnt[b + 1] += rcnt[b];
    std::vector<int> rfill(rcnt.begin(), rcnt.end() - 1);
    for (int r = 0; r < p->n_rec; r++) ridx[rfill[rown[r]]++] = r;
    CKR(ensure(&p->pcta_off, &p->cap_pcta_off, cnt.size()));
    CKR(ensure(&p->pcta_tgt, &p->cap_pcta_tgt, std::max<size_t>(1, tgt.size())));
    CKR(ensure(&p->prec_off, &p->cap_prec_off, rcnt.size()));
    CKR(ensure(&p->prec_idx, &p->cap_prec_idx, std::max<size_t>(1, ridx.size())));
    CKR(ensure(&p->psrcv, &p->cap_psrcv, std::max<size_t>(1, (size_t)p->stgt.n * p->d.nt)));
    CK(cudaMemcpyAsync(p->prec_off, rcnt.data(), rcnt.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    if (!ridx.empty())
        CK(cudaMemcpyAsync(p->prec_idx, ridx.data(), ridx.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    const size_t slot = (size_t)npairs(p) * p->shot_stride;
    CKR(ensure(&p->pbar, &p->cap_pbar, 1));
    CKR(ensure(&p->pxch, &p->cap_pxch, 2 * slot));
    CK(cudaMemcpyAsync(p->pcta_off, cnt.data(), cnt.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    if (!tgt.empty()) CK(cudaMemcpyAsync(p->pcta_tgt, tgt.data(), tgt.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(p->pbar, 0, sizeof(int), s));
    CK(cudaMemsetAsync(p->pxch, 0, 2 * slot * sizeof(uint4), s));  // no line holds a level of this run
    CK(cudaMemsetAsync(p->rec_amp, 0, (size_t)p->d.nt * p->n_rec * sizeof(float), s));
    sa::Persist2D a{};
    a.s = base_args(p);
    a.xch = p->pxch;
    a.xch_slot = (long long)slot;
    a.nt = nt_run > 0 ? std::min(nt_run, p->d.nt) : p->d.nt;
    a.tx = p->ptx;
    a.ty = p->pty;
    a.tiles_x = p->ptiles_x;
    a.tiles_y = p->ptiles_y;
    a.cta_off = p->pcta_off;
    a.cta_tgt = p->pcta_tgt;
    a.tidx = p->stgt.idx;
    a.toff = p->stgt.off;
    a.tcoef = p->stgt.coef;
    a.tpoint = p->stgt.point;
    a.src_amp = p->src_amp;
    a.n_src = p->n_src;
    a.srcv = p->psrcv;
    a.rec_off = p->prec_off;
    a.rec_idx = p->prec_idx;
    a.gat = p->gat_flat;
    a.n_rec = p->n_rec;
    a.rec_amp = p->rec_amp;
    a.err = p->pbar;
    a.extra = p->persist_extra;
    a.spin_limit = p->persist_spin;
    CK(sa::launch_persist2d(p->kind, p->ot4, p->pblocks, p->psmem, s, a));
    int err = 0;
    CK(cudaMemcpyAsync(&err, p->pbar, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (err)
        return fail(SA_E_TIMEOUT, "persistent forward: a halo wait gave up (%d CTAs, %d levels asked beyond the need)",
                    p->pblocks, a.extra);
    p->launches = 1;
    return SA_OK;
}

// Results of sa_autotune per (grid, operator, batch, device), for the life of the process:
// {strips, row chunks, time-blocking choice}.
std::map<std::string, std::array<int, 3>> g_tune;
std::mutex g_tune_mu;

// The current device's name and SM count (the autotuner caches' device component).
std::string device_key() {
    int dev = 0;
    cudaDeviceProp pr{};
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&pr, dev) != cudaSuccess) {
        cudaGetLastError();
        return "unknown";
    }
    char b[320];
    snprintf(b, sizeof(b), "%s/%d", pr.name, pr.multiProcessorCount);
    return b;
}

int ensure_fields(sa_plan* p) {
    const size_t n = (size_t)((std::max(1, p->d.max_shots) + 1) / 2) * p->shot_stride * 2;
    CKR(ensure(&p->field[0], &p->field_cap[0], n));
    CKR(ensure(&p->field[1], &p->field_cap[1], n));
    if (p->ot4) {  // pass L writes grid columns only: the pitch columns beyond ny stay zero (the halo)
        CKR(ensure(&p->lbuf, &p->lbuf_cap, n));
        CK(cudaMemset(p->lbuf, 0, n * sizeof(float)));
    }
    return SA_OK;
}

}  // namespace

extern "C" {

int sa_last_error(char* buf, int len) {
    if (!buf || len <= 0) return SA_E_INVALID;
    snprintf(buf, (size_t)len, "%s", g_err.c_str());
    return SA_OK;
}

long long sa_launch_count(const sa_plan* p) {
    if (!p) return -1;
    return p->p3 ? sa::plan3d_launches(p->p3) : p->launches;
}

int sa_plan_option(sa_plan* p, int option, long long value) {
    if (!p) return fail(SA_E_INVALID, "null plan");
    switch (option) {
        case SA_OPT_PERSISTENT:
            if (value < -1 || value > 1) return fail(SA_E_INVALID, "SA_OPT_PERSISTENT takes -1, 0 or 1");
            p->persist_mode = (int)value;
            return SA_OK;
        case SA_OPT_BARRIER_EXTRA:
            if (value < 0 || value > 1024) return fail(SA_E_INVALID, "SA_OPT_BARRIER_EXTRA takes 0..1024");
            p->persist_extra = (int)value;
            return SA_OK;
        case SA_OPT_BARRIER_SPIN:
            if (value < 1) return fail(SA_E_INVALID, "SA_OPT_BARRIER_SPIN takes a positive poll count");
            p->persist_spin = value;
            return SA_OK;
        default: return fail(SA_E_INVALID, "unknown option %d", option);
    }
}

int sa_plan_layout(const sa_plan* p, int* threads, int* strips, int* chunks) {
    if (!p || !threads || !strips || !chunks) return fail(SA_E_INVALID, "null argument");
    if (p->p3) return sa::plan3d_layout(p->p3, threads, strips, chunks);
    *threads = p->NT;
    *strips = p->nstrips;
    *chunks = p->nchunks;
    return SA_OK;
}

int sa_checkpoint_schedule(const sa_desc* d, int n_shots, int* K, int* n_ckpt, int* K2) {
    if (!d || !K || !n_ckpt || !K2 || n_shots < 1) return fail(SA_E_INVALID, "null argument or n_shots < 1");
    if (d->dim != 2 && d->dim != 3) return fail(SA_E_INVALID, "dim %d", d->dim);
    for (int a = 0; a < d->dim; a++)
        if (d->shape[a] < 1) return fail(SA_E_INVALID, "shape");
    if (d->nt < 3 || d->undersampling < 1) return fail(SA_E_INVALID, "nt or undersampling");
    const bool pml = d->boundary == SA_BOUNDARY_CFS_PML;
    double level;  // bytes of one wavefield level of every shot, as the plans lay it out
    if (d->dim == 2) {
        const long long pitch = (d->shape[1] + 2 + 31) / 32 * 32;
        level = (double)((n_shots + 1) / 2) * d->shape[0] * pitch * 2 * sizeof(float);
    } else {
        const long long zp = (d->shape[2] + 2 + 31) / 32 * 32;
        level = (double)n_shots * d->shape[0] * d->shape[1] * zp * sizeof(float);
    }
    // a checkpoint: both levels, plus the CFS-PML's auxiliary fields (six levels in 2D, nine in 3D)
    const double ck_levels = d->dim == 2 ? (pml ? 8 : 2) : (pml ? 11 : 2);
    return sa::choose_checkpoints(*d, level, K, n_ckpt, ck_levels, K2);
}

namespace {
int pml_profiles(sa_plan* p) {
    float vmax = 0.f;
    for (float v : p->vp_host) vmax = std::max(vmax, v);
    const std::vector<float> out = sa::pml_profile_tables(p->d, vmax);
    CK(cudaMemcpy(p->pml_prof, out.data(), out.size() * sizeof(float), cudaMemcpyHostToDevice));
    return SA_OK;
}
}  // namespace

int sa_plan_create(const sa_desc* desc, sa_plan** out) {
    if (!desc || !out) return fail(SA_E_INVALID, "null argument");
    *out = nullptr;
    const sa_desc& d = *desc;
    if (d.dim != 2 && d.dim != 3) return fail(SA_E_UNSUPPORTED, "dim %d: the operator is 2D or 3D", d.dim);
    if (d.kernel != SA_KERNEL_OT2 && d.kernel != SA_KERNEL_OT4)
        return fail(SA_E_INVALID, "Unrecognized kernel %d", d.kernel);
    if (d.density < 0 || d.density > 2) return fail(SA_E_INVALID, "density mode %d", d.density);
    if (d.interpolation != SA_INTERP_LINEAR && d.interpolation != SA_INTERP_HICKS && d.interpolation != SA_INTERP_SINC)
        return fail(SA_E_INVALID, "interpolation %d", d.interpolation);
    if (d.boundary != SA_BOUNDARY_SPONGE && d.boundary != SA_BOUNDARY_CFS_PML)
        return fail(SA_E_INVALID, "boundary %d", d.boundary);
    // With OT4 the reference's PML reads vp^2 laplace(p) where OT2 reads p (iso_acoustic/devito.py:1551):
    // its auxiliary fields gain two derivatives and a factor vp^2, and the update diverges
    if (d.boundary == SA_BOUNDARY_CFS_PML && d.kernel != SA_KERNEL_OT2)
        return fail(SA_E_UNSUPPORTED, "the CFS-PML runs with OT2 only: with OT4 the reference's boundary field is "
                                      "vp^2 laplace(p) and its literal update diverges");
    if (d.boundary == SA_BOUNDARY_CFS_PML && !(d.f_centre > 0)) return fail(SA_E_INVALID, "f_centre");
    if (d.nt < 3 || d.undersampling < 1 || d.max_shots < 1) return fail(SA_E_INVALID, "nt/undersampling/max_shots");
    for (int a = 0; a < d.dim; a++) {
        if (d.shape[a] < 24) return fail(SA_E_INVALID, "shape[%d] = %d is below 24 cells", a, d.shape[a]);
        if (!(d.spacing[a] > 0)) return fail(SA_E_INVALID, "spacing[%d]", a);
        if (d.absorbing[a] < 0 || d.absorbing[a] > d.extra[a] || d.absorbing[a] > sa::MAX_ABS ||
            d.absorbing[a] == 1 || 2 * d.absorbing[a] > d.shape[a])
            return fail(SA_E_INVALID, "absorbing[%d] = %d (extra %d)", a, d.absorbing[a], d.extra[a]);
    }
    if (!(d.dt > 0)) return fail(SA_E_INVALID, "dt");
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (d.dim == 3) {
        if (d.shape[2] < 24 || !(d.spacing[2] > 0) || d.absorbing[2] < 0 || d.absorbing[2] > d.extra[2] ||
            d.absorbing[2] > sa::MAX_ABS || d.absorbing[2] == 1 || 2 * d.absorbing[2] > d.shape[2])
            return fail(SA_E_INVALID, "third axis of the description");
        sa::Plan3D* p3 = nullptr;
        const int rc = sa::plan3d_create(d, &p3);
        if (rc != SA_OK) return rc;
        sa_plan* p = new sa_plan();
        p->d = d;
        p->p3 = p3;
        *out = p;
        return SA_OK;
    }
    sa_plan* p = new sa_plan();
    p->d = d;
    p->nx = d.shape[0];
    p->ny = d.shape[1];
    p->pitch = (p->ny + 2 + 31) / 32 * 32;     // a column pair starting at ny-1 stays in the row
    p->pitch_b = (p->ny + 12 + 31) / 32 * 32;  // half-cols -6..ny+3 at storage column y+6
    p->shot_stride = (long long)p->nx * p->pitch;
    p->kind = d.density == SA_DENSITY_NONE ? 0 : (d.density == SA_DENSITY_VARIABLE ? 1 : 2);
    p->ot4 = d.kernel == SA_KERNEL_OT4;
    p->n_snap = (d.nt + d.undersampling) / d.undersampling + 1;
    p->snap_stride = p->shot_stride;
    p->snap_shot_stride = (long long)p->n_snap * p->shot_stride;
    const char* env = getenv("STRIDEACC_NO_GRAPHS");
    p->use_graphs = !(env && env[0] == '1');
    p->sponge.a[0] = d.absorbing[0];
    p->sponge.a[1] = d.absorbing[1];
    int amax = 0;
    for (int a = 0; a < d.dim; a++) amax = std::max(amax, d.absorbing[a]);
    p->pml = d.boundary == SA_BOUNDARY_CFS_PML;
    if (amax > 1 && !p->pml) {  // the CFS-PML replaces the sponge: no damping in the update
        const double refl = std::pow(10.0, -(std::log10((double)amax) - 1) / std::log10(2.0) - 3);
        damping_table(d.absorbing[0], d.spacing[0], refl, p->sponge.s[0]);
        damping_table(d.absorbing[1], d.spacing[1], refl, p->sponge.s[1]);
    }
    int rc = ensure_fields(p);
    const size_t N = (size_t)p->shot_stride;
    const size_t NG = (size_t)(p->nx + 2 * sa::GUARD) * p->pitch;
    if (rc == SA_OK) rc = ensure(&p->W, &p->cap_W, NG);
    if (rc == SA_OK) rc = ensure(&p->C1, &p->cap_C1, NG);
    if (rc == SA_OK) rc = ensure(&p->C2, &p->cap_C2, NG);
    if (rc == SA_OK) rc = ensure(&p->C3, &p->cap_C3, NG);
    if (rc == SA_OK) rc = ensure(&p->vp, &p->cap_vp, N);
    if (rc == SA_OK) rc = ensure(&p->alpha, &p->cap_alpha, N);
    if (rc == SA_OK && p->kind >= 1) rc = ensure(&p->buoy, &p->cap_buoy, N);  // b = 1/rho (rho gradient)
    if (rc == SA_OK && p->pml) rc = ensure(&p->pml_prof, &p->cap_pml_prof, 4 * (size_t)(p->nx + p->ny));
    if (rc == SA_OK && p->pml)  // six auxiliary fields for every shot pair the plan can hold
        rc = ensure(&p->pml_aux, &p->cap_pml_aux, 6 * 2 * (size_t)((std::max(1, d.max_shots) + 1) / 2) * N);
    if (rc == SA_OK && p->kind == 1) {
        if (rc == SA_OK) rc = ensure(&p->bxh, &p->cap_bxh, (size_t)(p->nx + 9 + 2 * sa::GUARD) * p->pitch);
        if (rc == SA_OK) rc = ensure(&p->byh, &p->cap_byh, (size_t)(p->nx + 2 * sa::GUARD) * p->pitch_b);
    }
    if (rc != SA_OK) {
        sa_plan_destroy(p);
        return rc;
    }
    // pitch padding of every pitched array is read by the kernels' 16-byte row copies: zero
    const std::pair<float*, size_t> zero_bufs[] = {
        {p->field[0], p->field_cap[0]}, {p->field[1], p->field_cap[1]}, {p->W, p->cap_W}, {p->vp, p->cap_vp},
        {p->alpha, p->cap_alpha}, {p->buoy, p->cap_buoy}, {p->bxh, p->cap_bxh}, {p->byh, p->cap_byh},
        {p->C1, p->cap_C1}, {p->C2, p->cap_C2}, {p->C3, p->cap_C3}};
    for (const auto& zb : zero_bufs) {
        if (zb.first && cudaMemset(zb.first, 0, zb.second * sizeof(float)) != cudaSuccess) {
            sa_plan_destroy(p);
            return fail(SA_E_CUDA, "cudaMemset of plan buffers failed");
        }
    }
    *out = p;
    return SA_OK;
}

int sa_plan_destroy(sa_plan* p) {
    if (!p) return SA_OK;
    if (p->p3) {
        sa::plan3d_destroy(p->p3);
        delete p;
        return SA_OK;
    }
    drop_graphs(p);
    if (p->l2win.num_bytes) cudaCtxResetPersistingL2Cache();  // its lines go back to normal eviction
    void* bufs[] = {p->field[0], p->field[1], p->W, p->vp, p->alpha, p->buoy, p->bxh, p->byh, p->C1, p->C2, p->C3,
                    p->medium_stage,
                    p->gat_flat,
                    p->src_amp, p->rec_amp, p->stage, p->snaps, p->gradb, p->precb, p->ckpt, p->segsnaps,
                    p->afield[0], p->afield[1], p->EA, p->EB, p->EC, p->EG4, p->ES, p->levels, p->Lu, p->Lz,
                    p->smed, p->lbuf, p->pbar, p->pxch, p->prec_off, p->prec_idx, p->psrcv, p->pcta_off, p->pcta_tgt, p->src_flat, p->gat_src, p->hold_vp, p->hold_rho, p->gradrb, p->precrb,
                    p->dbx, p->dby, p->pml_prof, p->pml_aux, p->pml_ck, p->pml_aux_f, p->ckpt2, p->pml_ck2,
                    p->wgrad, p->hgat, p->hgat_src, p->rtgt.idx, p->rtgt.off, p->rtgt.point, p->rtgt.coef, p->stgt.idx,
                    p->stgt.off, p->stgt.point, p->stgt.coef, p->xtgt.idx, p->xtgt.off, p->xtgt.point, p->xtgt.coef};
    for (void* b : bufs)
        if (b) cudaFree(b);
    if (p->cap) cudaStreamDestroy(p->cap);
    delete p;
    return SA_OK;
}

int sa_set_medium(sa_plan* p, const float* vp, const float* rho, const float* alpha) {
    if (!p || !vp) return fail(SA_E_INVALID, "null plan or vp");
    if (p->d.density != SA_DENSITY_NONE && !rho) return fail(SA_E_INVALID, "rho required by the plan's density mode");
    if (p->d.attenuation && !alpha) return fail(SA_E_INVALID, "alpha required by the plan");
    // work still queued on the caller's streams reads the medium being replaced; the upload below runs on
    // the legacy default stream, which does not wait for non-blocking streams
    CK(cudaDeviceSynchronize());
    if (p->p3) return sa::plan3d_set_medium(p->p3, vp, rho, alpha);
    const size_t N = (size_t)p->nx * p->ny;
    const float* in[3] = {vp, p->d.density != SA_DENSITY_NONE ? rho : nullptr, p->d.attenuation ? alpha : nullptr};
    const float* dev[3] = {nullptr, nullptr, nullptr};
    const bool any_host = (in[0] && !is_device(in[0])) || (in[1] && !is_device(in[1])) || (in[2] && !is_device(in[2]));
    if (any_host) CKR(ensure(&p->medium_stage, &p->cap_medium_stage, 3 * N));
    for (int k = 0; k < 3; k++) {
        if (!in[k]) continue;
        if (is_device(in[k])) {
            dev[k] = in[k];
        } else {
            CK(cudaMemcpy(p->medium_stage + k * N, in[k], N * sizeof(float), cudaMemcpyHostToDevice));
            dev[k] = p->medium_stage + k * N;
        }
    }
    CK(sa::medium2d(dev[0], dev[1], dev[2], p->nx, p->ny, p->pitch, p->pitch_b, p->kind, kDbToNeper,
                    p->sponge, (float)p->d.dt, const_cast<float*>(row0(p, p->W, p->pitch)), p->vp, p->alpha, p->buoy,
                    p->bxh ? const_cast<float*>(row0(p, p->bxh, p->pitch, 5)) : nullptr,
                    p->byh ? const_cast<float*>(row0(p, p->byh, p->pitch_b)) : nullptr,
                    const_cast<float*>(row0(p, p->C1, p->pitch)), const_cast<float*>(row0(p, p->C2, p->pitch)),
                    const_cast<float*>(row0(p, p->C3, p->pitch)), 0));
    {
        float* old = p->smed;
        CKR(ensure(&p->smed, &p->cap_smed, sa::step_medium_size(p->nx, p->ny)));
        if (old != p->smed) drop_graphs(p);  // the captured step launches hold the medium pointers
        CK(sa::step_medium2d(row0(p, p->W, p->pitch), p->bxh ? row0(p, p->bxh, p->pitch, 5) : nullptr,
                             p->byh ? row0(p, p->byh, p->pitch_b) : nullptr, row0(p, p->C1, p->pitch),
                             row0(p, p->C2, p->pitch), row0(p, p->C3, p->pitch), p->nx, p->ny, p->pitch, p->pitch_b,
                             p->smed, 0));
        CKR(medium_l2_window(p));
    }
    CK(cudaDeviceSynchronize());
    p->vp_host.resize(N);
    CK(cudaMemcpy(p->vp_host.data(), dev[0], N * sizeof(float), cudaMemcpyDeviceToHost));
    {  // C1 W per point: the exact-gradient adjoint's receiver injection coefficient
        std::vector<float> c1((size_t)p->nx * p->pitch), w((size_t)p->nx * p->pitch);
        CK(cudaMemcpy(c1.data(), row0(p, p->C1, p->pitch), c1.size() * sizeof(float), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(w.data(), row0(p, p->W, p->pitch), w.size() * sizeof(float), cudaMemcpyDeviceToHost));
        p->c1w_host.resize(N);
        for (int x = 0; x < p->nx; x++)
            for (int y = 0; y < p->ny; y++)
                p->c1w_host[(size_t)x * p->ny + y] = c1[(size_t)x * p->pitch + y] * w[(size_t)x * p->pitch + y];
    }
    if (p->pml) CKR(pml_profiles(p));
    p->exact_coef_valid = false;
    p->rho_terms_valid = false;
    p->medium_set = true;
    if (p->geometry_set) CKR(build_lists(p));
    p->snaps_valid = false;
    p->ckpt_valid = false;
    return SA_OK;
}

int sa_set_geometry(sa_plan* p, int n_shots, const int* src_offsets, const float* src_xyz, const int* rec_offsets,
                    const float* rec_xyz) {
    if (!p || n_shots < 1 || !src_offsets || !rec_offsets) return fail(SA_E_INVALID, "bad geometry arguments");
    if (n_shots > p->d.max_shots) return fail(SA_E_INVALID, "%d shots exceed max_shots %d", n_shots, p->d.max_shots);
    for (int s = 0; s < n_shots; s++)
        if (src_offsets[s + 1] < src_offsets[s] || rec_offsets[s + 1] < rec_offsets[s])
            return fail(SA_E_INVALID, "offsets must be non-decreasing");
    if (src_offsets[0] != 0 || rec_offsets[0] != 0) return fail(SA_E_INVALID, "offsets must start at 0");
    CK(cudaDeviceSynchronize());  // queued work on any stream reads the point lists being replaced
    const int ns = src_offsets[n_shots], nr = rec_offsets[n_shots];
    if ((ns && !src_xyz) || (nr && !rec_xyz)) return fail(SA_E_INVALID, "missing coordinates");
    if (p->p3) return sa::plan3d_set_geometry(p->p3, n_shots, src_offsets, src_xyz, rec_offsets, rec_xyz);
    const int dim = p->d.dim;
    const bool wide = p->d.interpolation != SA_INTERP_LINEAR;  // a wide support (Hicks or sinc)
    auto convert = [&](const float* xyz, int n, std::vector<int>& bx, std::vector<int>& by, std::vector<double>& fx,
                       std::vector<double>& fy) -> int {
        bx.resize(n);
        by.resize(n);
        fx.resize(n);
        fy.resize(n);
        for (int i = 0; i < n; i++) {
            double rel[2];
            int base[2];
            for (int a = 0; a < 2; a++) {
                const double origin = -p->d.extra[a] * p->d.spacing[a];
                rel[a] = ((double)xyz[i * dim + a] - origin) / p->d.spacing[a];
                base[a] = (int)std::floor(rel[a]);
                const int n_a = a == 0 ? p->nx : p->ny;
                const int lo = wide ? sa::support_lo(p->d.interpolation) : 0;  // support base-lo .. base+hi
                const int hi = wide ? sa::support_width(p->d.interpolation) - 1 - lo : 1;
                if (!(base[a] - lo >= 0 && base[a] + hi <= n_a - 1))
                    return fail(SA_E_INVALID, "point %d lies outside the grid along axis %d", i, a);
            }
            bx[i] = base[0];
            by[i] = base[1];
            fx[i] = rel[0] - base[0];
            fy[i] = rel[1] - base[1];
        }
        return SA_OK;
    };
    CKR(convert(src_xyz, ns, p->src_bx, p->src_by, p->src_fx, p->src_fy));
    CKR(convert(rec_xyz, nr, p->rec_bx, p->rec_by, p->rec_fx, p->rec_fy));
    p->n_shots = n_shots;
    p->n_src = ns;
    p->n_rec = nr;
    p->src_off.assign(src_offsets, src_offsets + n_shots + 1);
    p->rec_off.assign(rec_offsets, rec_offsets + n_shots + 1);
    drop_graphs(p);  // shot count, point counts and layout are baked into the captured loops
    default_layout(p);
    CKR(build_lists(p));
    CKR(ensure(&p->src_amp, &p->cap_src_amp, (size_t)p->d.nt * ns));
    CKR(ensure(&p->rec_amp, &p->cap_rec_amp, (size_t)p->d.nt * nr));
    p->geometry_set = true;
    p->snaps_valid = false;
    p->ckpt_valid = false;
    return SA_OK;
}

int sa_forward(sa_plan* p, const float* wavelets, float* traces, int save_mode, void* stream) {
    if (!p) return fail(SA_E_INVALID, "null plan");
    if (save_mode != SA_SAVE_NONE && save_mode != SA_SAVE_SNAPSHOTS && save_mode != SA_SAVE_CHECKPOINTS &&
        save_mode != SA_SAVE_RAW)
        return fail(SA_E_INVALID, "save_mode %d", save_mode);
    if (p->p3) return sa::plan3d_forward(p->p3, wavelets, traces, save_mode, (cudaStream_t)stream);
    if (!p->medium_set || !p->geometry_set) return fail(SA_E_INVALID, "medium and geometry must be set first");
    if ((p->n_src && !wavelets) || (p->n_rec && !traces)) return fail(SA_E_INVALID, "null wavelets or traces");
    cudaStream_t s = (cudaStream_t)stream;
    // a forward replaces the plan's wavelets, which the checkpointed adjoint re-injects
    p->ckpt_valid = false;
    if (save_mode == SA_SAVE_SNAPSHOTS || save_mode == SA_SAVE_RAW) {
        const size_t n = (size_t)npairs(p) * p->snap_shot_stride * 2;
        float* old = p->snaps;
        CKR(ensure(&p->snaps, &p->cap_snaps, n));
        if (old != p->snaps) drop_graphs(p);
        // every slot the adjoint reads (t % f == 0, f <= t <= nt-1-f) is written by this forward
    } else if (save_mode == SA_SAVE_CHECKPOINTS) {
        const int oldK = p->ck_K, oldK2 = p->ck_K2;
        CKR(plan_checkpoints(p));
        const size_t n = std::max<size_t>(1, (size_t)p->ck_n * 2 * npairs(p) * p->shot_stride * 2);
        float *old = p->ckpt, *old_ck = p->pml_ck, *old_f = p->pml_aux_f;
        CKR(ensure(&p->ckpt, &p->cap_ckpt, n));
        if (p->pml) {
            const size_t na = pml_aux_bytes(p) / sizeof(float);
            CKR(ensure(&p->pml_ck, &p->cap_pml_ck, std::max<size_t>(1, (size_t)p->ck_n * na)));
            CKR(ensure(&p->pml_aux_f, &p->cap_pml_aux_f, na));
        }
        if (old != p->ckpt || old_ck != p->pml_ck || old_f != p->pml_aux_f || oldK != p->ck_K || oldK2 != p->ck_K2)
            drop_graphs(p);
        p->snaps_valid = false;
    }
    CKR(load_transposed(p, wavelets, p->n_src, p->d.nt, p->src_amp, s));
    if (use_persistent(p, save_mode)) {  // one cooperative launch runs every step
        CKR(forward_persistent(p, s));
        CKR(store_transposed(p, p->rec_amp, p->d.nt, p->n_rec, traces, s));
        p->launches = (p->n_src ? 1 : 0) + 1 + (p->n_rec ? 1 : 0);
        p->adjoint_pending = false;
        return SA_OK;
    }
    CKR(run_loop(p, &p->g_fwd[save_mode], s, [&](cudaStream_t cs) { return issue_forward(p, save_mode, cs); }));
    CKR(store_transposed(p, p->rec_amp, p->d.nt, p->n_rec, traces, s));
    p->launches = (p->n_src ? 1 : 0) + p->fwd_launches[save_mode] + (p->n_rec ? 1 : 0);
    if (save_mode == SA_SAVE_SNAPSHOTS || save_mode == SA_SAVE_RAW) {
        p->snaps_valid = true;
        p->snaps_raw = save_mode == SA_SAVE_RAW;
    }
    if (save_mode == SA_SAVE_CHECKPOINTS) p->ckpt_valid = true;
    p->adjoint_pending = save_mode != SA_SAVE_NONE;
    return SA_OK;
}

int sa_adjoint(sa_plan* p, const float* residuals, float* grad_vp, float* prec_vp, int grad_mode, void* stream) {
    return sa_adjoint_wavelets(p, residuals, grad_vp, prec_vp, nullptr, grad_mode, stream);
}

namespace {
int adjoint_impl(sa_plan* p, const float* residuals, float* grad_vp, float* prec_vp, float* grad_rho,
                 float* prec_rho, float* grad_wavelets, int grad_mode, void* stream);
}

int sa_adjoint_wavelets(sa_plan* p, const float* residuals, float* grad_vp, float* prec_vp, float* grad_wavelets,
                        int grad_mode, void* stream) {
    return adjoint_impl(p, residuals, grad_vp, prec_vp, nullptr, nullptr, grad_wavelets, grad_mode, stream);
}

int sa_adjoint_grads(sa_plan* p, const float* residuals, float* grad_vp, float* prec_vp, float* grad_rho,
                     float* prec_rho, float* grad_wavelets, void* stream) {
    if (!p) return fail(SA_E_INVALID, "null plan");
    if (p->p3) {
        if (!grad_vp || !prec_vp) return fail(SA_E_INVALID, "null outputs");
        return sa::plan3d_adjoint(p->p3, residuals, grad_vp, prec_vp, (cudaStream_t)stream, grad_rho, prec_rho,
                                  grad_wavelets);
    }
    if (!p->snaps_valid || !p->snaps_raw)
        return fail(SA_E_INVALID, "sa_adjoint_grads needs a prior sa_forward with SA_SAVE_RAW");
    if ((grad_rho == nullptr) != (prec_rho == nullptr)) return fail(SA_E_INVALID, "grad_rho and prec_rho go together");
    if (grad_rho && p->kind == 0) return fail(SA_E_INVALID, "the rho gradient needs a plan with rho");
    return adjoint_impl(p, residuals, grad_vp, prec_vp, grad_rho, prec_rho, grad_wavelets, SA_GRAD_PARITY, stream);
}

namespace {
int adjoint_impl(sa_plan* p, const float* residuals, float* grad_vp, float* prec_vp, float* grad_rho,
                 float* prec_rho, float* grad_wavelets, int grad_mode, void* stream) {
    if (!p) return fail(SA_E_INVALID, "null plan");
    if (grad_mode != SA_GRAD_PARITY && grad_mode != SA_GRAD_EXACT) return fail(SA_E_INVALID, "grad_mode %d", grad_mode);
    const bool exact = grad_mode == SA_GRAD_EXACT;
    const bool wav = grad_wavelets != nullptr;
    if (wav && exact) return fail(SA_E_UNSUPPORTED, "the wavelet gradient is the parity mode's (src.interpolate(-p_a))");
    if (exact && p->d.boundary != SA_BOUNDARY_SPONGE)
        return fail(SA_E_UNSUPPORTED, "the exact gradient is implemented for the sponge boundary");
    if (p->p3) {
        if (!grad_vp || !prec_vp) return fail(SA_E_INVALID, "null outputs");
        if (exact) return sa::plan3d_adjoint_exact(p->p3, residuals, grad_vp, prec_vp, (cudaStream_t)stream);
        return sa::plan3d_adjoint(p->p3, residuals, grad_vp, prec_vp, (cudaStream_t)stream, grad_rho, prec_rho,
                                  grad_wavelets);
    }
    const bool ck = p->ckpt_valid;
    const bool raw = !ck && p->snaps_valid && p->snaps_raw;  // imaging from raw snapshots
    const bool rho = grad_rho != nullptr;
    if (exact && !ck) return fail(SA_E_INVALID, "SA_GRAD_EXACT needs a prior sa_forward with SA_SAVE_CHECKPOINTS");
    if (exact && p->ck_K2 > 0)
        return fail(SA_E_NOMEM, "SA_GRAD_EXACT needs a one-level checkpoint schedule: checkpoint_budget is too small");
    if (!p->snaps_valid && !ck)
        return fail(SA_E_INVALID, "sa_adjoint needs a prior sa_forward with SA_SAVE_SNAPSHOTS or SA_SAVE_CHECKPOINTS");
    if ((p->n_rec && !residuals) || !grad_vp || !prec_vp) return fail(SA_E_INVALID, "null residuals or outputs");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t fe = (size_t)npairs(p) * p->shot_stride;
    float *og = p->gradb, *op = p->precb;
    CKR(ensure(&p->gradb, &p->cap_gradb, fe));
    CKR(ensure(&p->precb, &p->cap_precb, fe));
    if (og != p->gradb || op != p->precb) drop_graphs(p);
    if (ck) {
        float *o0 = p->afield[0], *o1 = p->afield[1], *os = p->segsnaps;
        CKR(ensure(&p->afield[0], &p->afield_cap[0], 2 * fe));
        CKR(ensure(&p->afield[1], &p->afield_cap[1], 2 * fe));
        float *oc2 = p->ckpt2, *oa2 = p->pml_ck2;
        const int K2 = p->ck_K2 > 0 ? p->ck_K2 : p->ck_K;
        if (!exact) CKR(ensure(&p->segsnaps, &p->cap_segsnaps, (size_t)(K2 / p->d.undersampling) * 2 * fe));
        if (!exact && p->ck_K2 > 0) {  // fine checkpoints of one coarse segment
            const size_t nf = (size_t)std::max(1, p->ck_K / p->ck_K2 - 1);
            CKR(ensure(&p->ckpt2, &p->cap_ckpt2, nf * 2 * 2 * fe));
            if (p->pml) CKR(ensure(&p->pml_ck2, &p->cap_pml_ck2, nf * (pml_aux_bytes(p) / sizeof(float))));
        }
        if (o0 != p->afield[0] || o1 != p->afield[1] || os != p->segsnaps || oc2 != p->ckpt2 || oa2 != p->pml_ck2)
            drop_graphs(p);
    }
    if (exact) {
        float* old[] = {p->EA, p->EB, p->EC, p->EG4, p->ES, p->levels, p->Lu, p->Lz};
        CKR(ensure(&p->EA, &p->cap_EA, (size_t)p->shot_stride));
        CKR(ensure(&p->EB, &p->cap_EB, (size_t)p->shot_stride));
        CKR(ensure(&p->EC, &p->cap_EC, (size_t)p->shot_stride));
        CKR(ensure(&p->EG4, &p->cap_EG4, (size_t)p->shot_stride));
        CKR(ensure(&p->ES, &p->cap_ES, (size_t)p->shot_stride));
        CKR(ensure(&p->levels, &p->cap_levels, (size_t)(p->ck_K + 2) * 2 * fe));
        CKR(ensure(&p->Lu, &p->cap_Lu, 2 * fe));
        CKR(ensure(&p->Lz, &p->cap_Lz, 2 * fe));
        float* now[] = {p->EA, p->EB, p->EC, p->EG4, p->ES, p->levels, p->Lu, p->Lz};
        if (!std::equal(std::begin(old), std::end(old), std::begin(now)) || !p->exact_coef_valid) {
            drop_graphs(p);
            CK(cudaMemset(p->Lu, 0, 2 * fe * sizeof(float)));
            CK(cudaMemset(p->Lz, 0, 2 * fe * sizeof(float)));
            CK(sa::exact_coef2d(p->vp, p->alpha, row0(p, p->W, p->pitch), p->nx, p->ny, p->pitch, p->sponge,
                                (float)p->d.dt, p->EA, p->EB, p->EC, p->EG4, p->ES, 0));
            CK(cudaDeviceSynchronize());
            p->exact_coef_valid = true;
        }
    }
    if (wav) {
        float* ow = p->wgrad;
        CKR(ensure(&p->wgrad, &p->cap_wgrad, (size_t)p->d.nt * std::max(1, p->n_src)));
        if (ow != p->wgrad) drop_graphs(p);
    }
    if (raw) {
        float* old[] = {p->hold_vp, p->hold_rho, p->gradrb, p->precrb, p->dbx, p->dby};
        CKR(ensure(&p->hold_vp, &p->cap_hold_vp, 2 * fe));
        if (rho) {
            CKR(ensure(&p->hold_rho, &p->cap_hold_rho, 2 * fe));
            CKR(ensure(&p->gradrb, &p->cap_gradrb, fe));
            CKR(ensure(&p->precrb, &p->cap_precrb, fe));
            CKR(ensure(&p->dbx, &p->cap_dbx, (size_t)p->shot_stride));
            CKR(ensure(&p->dby, &p->cap_dby, (size_t)p->shot_stride));
        }
        float* now[] = {p->hold_vp, p->hold_rho, p->gradrb, p->precrb, p->dbx, p->dby};
        if (!std::equal(std::begin(old), std::end(old), std::begin(now))) {
            drop_graphs(p);
            p->rho_terms_valid = false;
        }
        if (rho && !p->rho_terms_valid) {
            CK(sa::rho_terms2d(p->buoy, p->nx, p->ny, p->pitch, (float)p->d.spacing[0], (float)p->d.spacing[1],
                               p->dbx, p->dby, 0));
            CK(cudaDeviceSynchronize());
            p->rho_terms_valid = true;
        }
    }
    CKR(load_transposed(p, residuals, p->n_rec, p->d.nt, p->rec_amp, s));
    const int am = exact ? 2 : (ck ? 1 : (raw ? (rho ? 4 : 3) : 0));
    CKR(run_loop(p, &p->g_adj[am][wav ? 1 : 0], s, [&](cudaStream_t cs) {
        return exact ? issue_adjoint_exact(p, cs)
                     : (ck ? issue_adjoint_ckpt(p, wav, cs) : issue_adjoint(p, wav, raw, rho, cs));
    }));
    if (wav) CKR(store_transposed(p, p->wgrad, p->d.nt, p->n_src, grad_wavelets, s));
    const size_t N = (size_t)p->nx * p->ny;
    for (int k = 0; k < (rho ? 4 : 2); k++) {
        float* user = k == 0 ? grad_vp : (k == 1 ? prec_vp : (k == 2 ? grad_rho : prec_rho));
        const float* buf = k == 0 ? p->gradb : (k == 1 ? p->precb : (k == 2 ? p->gradrb : p->precrb));
        if (is_device(user)) {
            CK(sa::reduce_shots(buf, p->shot_stride, npairs(p), p->nx, p->ny, p->pitch, user, s));
        } else {
            CKR(ensure(&p->stage, &p->cap_stage, N));
            CK(sa::reduce_shots(buf, p->shot_stride, npairs(p), p->nx, p->ny, p->pitch, p->stage, s));
            CK(cudaMemcpyAsync(user, p->stage, N * sizeof(float), cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
        }
    }
    p->launches = (p->n_rec ? 1 : 0) + p->adj_launches[am] + (rho ? 4 : 2);
    p->adjoint_pending = false;
    return SA_OK;
}
}  // namespace

int sa_autotune(sa_plan* p, void* stream) {
    if (!p) return fail(SA_E_INVALID, "null plan");
    const std::string dev = device_key();
    if (p->p3) {
        int tile = 0, chunks = 0;
        bool cached = false;
        return sa::plan3d_autotune(p->p3, dev.c_str(), &tile, &chunks, &cached, (cudaStream_t)stream);
    }
    if (!p->geometry_set || !p->medium_set) return fail(SA_E_INVALID, "autotune needs medium and geometry");
    if (p->adjoint_pending && (p->snaps_valid || p->ckpt_valid))
        return fail(SA_E_INVALID, "autotune between a saving forward and its adjoint would discard the saved "
                                  "wavefield: run the adjoint first");
    cudaStream_t s = (cudaStream_t)stream;
    char key[256];
    snprintf(key, sizeof(key), "2d:%d,%d:k%d:%s:p%d:%s", p->nx, p->ny, p->kind, p->ot4 ? "ot4" : "ot2", npairs(p),
             dev.c_str());
    {
        std::lock_guard<std::mutex> g(g_tune_mu);
        auto it = g_tune.find(key);
        if (it != g_tune.end()) {
            p->layout_fixed = true;
            drop_graphs(p);
            set_strips(p, it->second[0]);
            p->chunk_rows = (p->nx + it->second[1] - 1) / it->second[1];
            p->nchunks = (p->nx + p->chunk_rows - 1) / p->chunk_rows;
            p->persist_tuned = it->second[2];
            CKR(build_lists(p));
            p->snaps_valid = false;
            p->ckpt_valid = false;
            return SA_OK;
        }
    }
    struct Cand {
        int strips, nchunks;
    };
    std::vector<Cand> cands;
    // column strips from the fewest (widest CTAs) to four more; row chunks: short chunks (more
    // CTAs, more pipeline warm-up rows) only pay off when the batch alone cannot fill the GPU
    const int s0 = min_strips(p);
    const int ctas1 = npairs(p) * s0;
    for (int st = s0; st <= s0 + 4; st++) {
        int by = 0, nt = 0;
        if (!sa::step_strips(p->ny, st, &by, &nt) || (st > s0 && by < 16)) continue;
        for (int nc : {1, 2, 3, 4, 6, 8, 12, 16, 24, 32, 48}) {
            const int min_rows = ctas1 >= 456 ? 4 * radius(p) : 8;
            if (p->nx / nc < min_rows) continue;
            cands.push_back({st, nc});
        }
    }
    const int steps = std::min(24, p->d.nt - 2);
    float best = 1e30f;
    Cand bc = {p->nstrips, p->nchunks};
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    p->layout_fixed = true;
    drop_graphs(p);  // the launch shape is baked into the captured loops
    for (const Cand& c : cands) {
        set_strips(p, c.strips);
        p->chunk_rows = (p->nx + c.nchunks - 1) / c.nchunks;
        p->nchunks = (p->nx + p->chunk_rows - 1) / p->chunk_rows;
        CKR(build_lists(p));
        sa::Step2D a = base_args(p);
        a.cur = p->field[0];
        a.prev = p->field[1];
        const dim3 grid(p->nstrips, p->nchunks, npairs(p));
        for (int w = 0; w < 3; w++) {
            a.t = 1 + w;
            CK(sa::launch_step2d(p->kind, p->ot4, p->NT, grid, s, a));
        }
        CK(cudaEventRecord(e0, s));
        for (int t = 0; t < steps; t++) {
            a.t = 1 + t;
            float* nc = const_cast<float*>(a.cur);
            a.cur = a.prev;
            a.prev = nc;
            CK(sa::launch_step2d(p->kind, p->ot4, p->NT, grid, s, a));
        }
        CK(cudaEventRecord(e1, s));
        CK(cudaEventSynchronize(e1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) {
            best = ms;
            bc = c;
        }
    }
    set_strips(p, bc.strips);
    p->chunk_rows = (p->nx + bc.nchunks - 1) / bc.nchunks;
    p->nchunks = (p->nx + p->chunk_rows - 1) / p->chunk_rows;
    CKR(build_lists(p));
    // time-blocking depth of a forward without a saved wavefield: one step per launch (the passes
    // above) or every step in one launch (the persistent kernel), per step over a short run
    p->persist_tuned = -1;
    if (persist_eligible(p) && persist_layout(p)) {
        const int nrun = std::min(p->d.nt, steps + 2);
        CKR(forward_persistent(p, s, nrun));  // warm-up: kernel configuration, tables
        CK(cudaEventRecord(e0, s));
        CKR(forward_persistent(p, s, nrun));
        CK(cudaEventRecord(e1, s));
        CK(cudaEventSynchronize(e1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        p->persist_tuned = ms < best ? 1 : 0;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    {
        std::lock_guard<std::mutex> g(g_tune_mu);
        g_tune[key] = {bc.strips, bc.nchunks, p->persist_tuned};
    }
    p->snaps_valid = false;
    p->ckpt_valid = false;
    return SA_OK;
}

}  // extern "C"

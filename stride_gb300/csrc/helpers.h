// Host launchers of the plan's helper kernels (helpers.cu).
#pragma once
#include <algorithm>
#include <vector>

#include "../../include/strideacc.h"
#include "common.cuh"

namespace sa {
// Sponge ramps of the two axes (1/m), per distance to the edge.
struct Sponge {
    int a[2];
    float s[2][MAX_ABS];
};
cudaError_t medium2d(const float* vp_in, const float* rho_in, const float* alpha_in, int nx, int ny, int pitch,
                     int pitch_b, int density, double db_to_np, const Sponge& sp, float dt, float* W, float* vp,
                     float* alpha, float* buoy, float* bxh, float* byh, float* C1, float* C2, float* C3,
                     cudaStream_t s);
// Row pitch (floats, even) of the step passes' medium for an ny-column grid, and the largest even
// column a step thread may address in it.
inline int med_pitch(int ny) { return (ny + 2 * MED_MARGIN + 15) / 16 * 16; }
inline int med_ymax(int ny) { return (ny + MED_MARGIN - 2) & ~1; }
// Floats of the six medium arrays of an nx x ny grid.
inline size_t step_medium_size(int nx, int ny) { return (size_t)6 * (nx + 2 * MED_GUARD) * med_pitch(ny); }
// The step passes' medium (helpers.cu k_step_medium2d), step_medium_size(nx, ny) floats.
cudaError_t step_medium2d(const float* W, const float* bxh, const float* byh, const float* C1, const float* C2,
                          const float* C3, int nx, int ny, int pitch, int pitch_b, float* out, cudaStream_t s);
// Points a step's medium fields at a step-medium allocation of an nx x ny grid.
inline void step_medium(Step2D& a, const float* med, int nx, int ny) {
    const int mp = med_pitch(ny);
    const long long astride = (long long)(nx + 2 * MED_GUARD) * mp;
    const float* at0 = med + (long long)MED_GUARD * mp + MED_MARGIN;
    a.Wm = at0;
    a.bxm = at0 + astride;
    a.bym = at0 + 2 * astride;
    a.C1m = at0 + 3 * astride;
    a.C2m = at0 + 4 * astride;
    a.NC3m = at0 + 5 * astride;
    a.mpitch = mp;
    a.ymax = med_ymax(ny);
}
// The step's FD weights over the spacing (kind 0: the 10th-order Laplacian's over h^2; else the
// staggered first derivative's over h), dt^2 / 12 and 1 / dt^2.
inline void step_weights(Step2D& a, int kind, double hx, double hy, double dt) {
    for (int m = 0; m < 6; m++) {
        float wx, wy;
        if (kind == 0) {
            wx = (float)((double)kW2(m) / (hx * hx));
            wy = (float)((double)kW2(m) / (hy * hy));
        } else {
            wx = m < 5 ? (float)((double)kWS(m) / hx) : 0.f;
            wy = m < 5 ? (float)((double)kWS(m) / hy) : 0.f;
        }
        a.wx[m] = make_float2(wx, wx);
        a.wy[m] = make_float2(wy, wy);
    }
    a.k12 = (float)(dt * dt / 12.0);
    a.inv_dt2 = (float)(1.0 / (dt * dt));
}
// Launch layout of the step passes for a ny-column grid split into `strips` column strips: output
// columns per strip (even) and threads per CTA (two columns each, at least STEP_MIN_THREADS);
// false when a strip needs more than STEP_MAX_THREADS threads.
inline bool step_strips(int ny, int strips, int* by, int* threads) {
    const int b = ((ny + strips - 1) / strips + 1) & ~1;
    const int t = std::max(STEP_MIN_THREADS, b / 2);
    *by = b;
    *threads = t;
    return t <= STEP_MAX_THREADS && strips >= 1;
}
void set_last_error(const char* msg);
// exact-gradient mode (exact2d.cu)
cudaError_t exact_coef2d(const float* vp, const float* alpha, const float* W, int nx, int ny, int pitch,
                         const Sponge& sp, float dt, float* EA, float* EB, float* EC, float* EG4, float* ES,
                         cudaStream_t s);
cudaError_t exact_grad2d(const float* z, const float* u0, const float* u1, const float* u2, const float* Lu,
                         const float* Lz, const float* EA, const float* EB, const float* EC, const float* EG4, int nx,
                         int ny, int pitch, int npairs, long long shot_stride, float inv_dt2, float* gradb,
                         float* precb, cudaStream_t s);
// One support point of a source for the exact gradient's source term: plane index within the
// pair's gradient buffer (i) and within a plane (p), lane of the pair, source row, raw weight.
struct ExactSrc2D {
    long long i;
    int p, lane, point;
    float w;
};
cudaError_t exact_src2d(const float* z, const ExactSrc2D* e, int n, const float* amp, int ld, int trow, float scale,
                        const float* ES, float* gradb, cudaStream_t s);

// 3D plans
// Hicks coefficients of one axis at the fractional offset frac (index 3 + grid offset, -3..4).
void hicks_coefs(double frac, bool smooth, double c[8]);
// Coefficients of one axis of a wide support (SA_INTERP_HICKS or SA_INTERP_SINC) at the fractional
// offset frac: returns the points per axis; c[i] weighs grid offset i - support_lo(interp).
int support_coefs(int interp, double frac, bool smooth, double c[SUPPORT_MAX]);
inline int support_lo(int interp) { return interp == SA_INTERP_SINC ? 6 : 3; }
inline int support_width(int interp) { return interp == SA_INTERP_SINC ? 14 : 8; }
// CFS-PML profile tables (sigma, alpha, sigma', alpha' per axis) of a plan description.
std::vector<float> pml_profile_tables(const sa_desc& d, float vmax);

struct Sponge3 {
    int a[3];
    float s[3][MAX_ABS];
};
struct Sparse3D;
struct Entries3D;
struct SupportGather3D;
// CFS-PML auxiliary update and boundary term after a 3D OT2 step.
cudaError_t pml3d(const float* cur, float* nxt, float* aux, const float* prof, const float* C1, const float* vp,
                  int nx, int ny, int nz, int zp, int nshots, long long field, const int* a, const double* h, float dt,
                  int adjoint, float* snap, long long snap_shot_stride, float inv_dt2, cudaStream_t s);
// Wide-support (Hicks, sinc) forms of the 3D exact gradient's receiver coefficients and source term.
cudaError_t xcoef_entries3d(const long long* idx, const float* w, int n, const float* C1, const float* W, float* out,
                            cudaStream_t s);
cudaError_t exact_src_entries3d(const float* z, const Entries3D& e, const float* w, int n, const float* amp, int ld,
                                int trow, float scale, const float* ES, long long field, float* gradb, cudaStream_t s);
// Wide-support injection (flat support entries) and gather (width^3 support) of 3D plans.
cudaError_t inject_entries3d(const Entries3D& e, int n, const float* amp, int ld, int t, float* field,
                             long long shot_stride, float* snap, long long snap_shot_stride, long long snap_off,
                             float inv_dt2, cudaStream_t s);
cudaError_t support_gather3d(const SupportGather3D* g, int n, const float* field, long long shot_stride, int ny, int zp,
                           float* out, int ld, int trow, float scale, cudaStream_t s);
cudaError_t medium3d(const float* vp_in, const float* rho_in, const float* alpha_in, int nx, int ny, int nz, int zp,
                     int zpb, int density, double db_to_np, const Sponge3& sp, float dt, float* W, float* vp,
                     float* alpha, float* buoy, float* bxh, float* byh, float* bzh, float* C1, float* C2, float* C3,
                     cudaStream_t s);
cudaError_t sparse3d_inject(const Sparse3D& sp, int n, const float* amp, int ld, int t, float* field,
                            long long shot_stride, int ny, int zp, float* snap, long long snap_shot_stride,
                            long long snap_off, float inv_dt2, cudaStream_t s);
// out[trow][k] = scale * trilinear interpolation of the field at point k
cudaError_t sparse3d_gather(const Sparse3D& sp, int n, const float* field, long long shot_stride, int ny, int zp,
                            float* out, int ld, int trow, cudaStream_t s, float scale = 1.f);
cudaError_t image3d(const float* q, const float* snap, float* gradb, float* precb, const int* lo, const int* hi,
                    int ny, int zp, int nshots, long long field, long long snap_shot_stride, cudaStream_t s);
// 3D rho-gradient medium terms (D-b per axis) and raw-snapshot imaging (held terms, every step).
cudaError_t rho_terms3d(const float* b, int nx, int ny, int nz, int zp, const double* h, float* dbx, float* dby,
                        float* dbz, cudaStream_t s);
cudaError_t image_raw3d(const float* q, const float* snap, long long snap_stride, long long snap_shot_stride,
                        int refresh, float inv_fdt2, float* hold_vp, float* hold_rho, const float* buoy,
                        const float* dbx, const float* dby, const float* dbz, const double* h, int nx, int ny, int nz,
                        int zp, float* gradb, float* precb, float* gradrb, float* precrb, const int* lo,
                        const int* hi, int nshots, long long field, cudaStream_t s);
// Exact-gradient helpers of 3D plans (the 3D counterparts of exact2d.cu).
cudaError_t exact_coef3d(const float* vp, const float* alpha, const float* W, int nx, int ny, int nz, int zp,
                         const Sponge3& sp, float dt, float* EA, float* EB, float* EC, float* EG4, float* ES,
                         cudaStream_t s);
cudaError_t exact_grad3d(const float* z, const float* u0, const float* u1, const float* u2, const float* Lu,
                         const float* Lz, const float* EA, const float* EB, const float* EC, const float* EG4, int nx,
                         int ny, int nz, int zp, int nshots, long long field, float inv_dt2, float* gradb,
                         float* precb, cudaStream_t s);
cudaError_t exact_src3d(const float* z, const Sparse3D& sp, int n, const float* amp, int ld, int trow, float scale,
                        const float* ES, int ny, int zp, long long field, float* gradb, cudaStream_t s);
cudaError_t xcoef3d(const Sparse3D& sp, int n, const float* C1, const float* W, int ny, int zp, float* out,
                    cudaStream_t s);
cudaError_t reduce3d(const float* buf, long long shot_stride, int nshots, int nx, int ny, int nz, int zp, float* out,
                     cudaStream_t s);
cudaError_t transpose(const float* in, int rows, int cols, float* out, cudaStream_t s);
cudaError_t inject_targets2d(float* field, const long long* idx, const int* off, const float* coef, const int* point,
                             int n, const float* amp, int ld, int t, float* snap, long long shot_stride,
                             long long snap_shot_stride, int unused, float inv_dt2, cudaStream_t s);
// Source injection of step t into `field` and the receiver gather rec[trow] = interp(gfield) in one
// launch (the two levels differ).
cudaError_t inject_gather2d(float* field, const long long* idx, const int* off, const float* coef, const int* point,
                            int n, const float* amp, int ld, int t, float* snap, long long shot_stride,
                            long long snap_shot_stride, float inv_dt2, const float* gfield, int pitch,
                            const Gather* g, int ng, float* out, int gld, int trow, cudaStream_t s);
cudaError_t image2d(const float* q, const float* snap, float* gradb, float* precb, int ix0, int ix1, int iy0, int iy1,
                    int pitch, int npairs, long long shot_stride, long long snap_shot_stride, cudaStream_t s);
// D-_x b and D-_y b at every node (edge-padded b), for the rho imaging term.
cudaError_t rho_terms2d(const float* buoy, int nx, int ny, int pitch, float hx, float hy, float* dbx, float* dby,
                        cudaStream_t s);
// Raw-snapshot imaging: held vp (and rho) terms refreshed on t = n f, accumulated every step.
cudaError_t image_raw2d(const float* q, const float* snap, long long snap_stride, long long snap_shot_stride,
                        int refresh, float inv_fdt2, float* hold_vp, float* hold_rho, const float* buoy,
                        const float* dbx, const float* dby, float hx, float hy, int nx, int ny, float* gradb,
                        float* precb, float* gradrb, float* precrb, int ix0, int ix1, int iy0, int iy1, int pitch,
                        int npairs, long long shot_stride, cudaStream_t s);
// CFS-PML auxiliary update on the absorbing frame and the boundary term of the new level (OT2).
cudaError_t pml2d(const float* cur, float* nxt, float* aux, const float* prof, const float* C1, const float* vp, int nx,
                  int ny, int pitch, long long shot_stride, int npairs, int ax, int ay, float hx, float hy, float dt,
                  int adjoint, float* snap, long long snap_shot_stride, float inv_dt2, cudaStream_t s);
cudaError_t support_gather2d(const float* field, long long shot_stride, int pitch, const SupportGather* g, int n, float* out,
                           int ld, int trow, cudaStream_t s);
cudaError_t final_gather2d(const float* field, long long shot_stride, int pitch, const Gather* g, int n, float* out,
                           int ld, int trow, cudaStream_t s);
cudaError_t reduce_shots(const float* buf, long long shot_stride, int nshots, int nx, int ny, int pitch, float* out,
                         cudaStream_t s);
}  // namespace sa

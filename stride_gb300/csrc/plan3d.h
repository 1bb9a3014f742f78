// 3D plans (plan3d.cu), used by the C ABI entry points when sa_desc.dim == 3.
#pragma once
#include <cuda_runtime.h>

#include "../../include/strideacc.h"

namespace sa {
struct Plan3D;
int plan3d_create(const sa_desc& d, Plan3D** out);
void plan3d_destroy(Plan3D* p);
int plan3d_set_medium(Plan3D* p, const float* vp, const float* rho, const float* alpha);
int plan3d_set_geometry(Plan3D* p, int n_shots, const int* so, const float* sx, const int* ro, const float* rx);
int plan3d_forward(Plan3D* p, const float* wavelets, float* traces, int save_mode, cudaStream_t s);
// grad_rho/prec_rho (both or neither) need a prior forward with SA_SAVE_RAW; after such a forward
// the vp gradient follows the raw-wavefield path too.
// grad_wavelets [n_src, nt] (host or device, optional): -interp(p_a[t]) at the sources.
int plan3d_adjoint(Plan3D* p, const float* residuals, float* grad, float* prec, cudaStream_t s,
                   float* grad_rho = nullptr, float* prec_rho = nullptr, float* grad_wavelets = nullptr);
// SA_GRAD_EXACT after a forward with SA_SAVE_CHECKPOINTS: residuals are dL/dtraces, grad receives
// dL/dvp of the discrete forward map at every point, prec the sum over all steps of p.dt2^2.
int plan3d_adjoint_exact(Plan3D* p, const float* residuals, float* grad, float* prec, cudaStream_t s);
long long plan3d_launches(const Plan3D* p);
// Layout search (tile of kTiles3d and x chunks) of a 3D plan; device_key names the GPU for the
// process-wide cache of results.
int plan3d_autotune(Plan3D* p, const char* device_key, int* tile, int* chunks, bool* cached, cudaStream_t s);
// The passes' layout: threads per CTA (the tile's columns), (y, z) tiles, x chunks.
int plan3d_layout(const Plan3D* p, int* threads, int* tiles, int* chunks);
// Checkpoint interval K (a multiple of f) and the number of stored checkpoints for a plan whose
// two state levels take `level_bytes` (SA_SAVE_CHECKPOINTS, both dimensions).
int choose_checkpoints(const sa_desc& d, double level_bytes, int* K, int* n_ckpt, double ck_levels = 2,
                       int* K2 = nullptr);
}  // namespace sa

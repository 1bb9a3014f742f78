/*
 * strideacc.h -- C ABI of the GB300 iso-acoustic FDTD library (libstrideacc.so).
 *
 * The library replaces the Devito-generated time loop that Stride's
 * IsoAcousticDevito builds and runs per shot. Each entry point names the
 * reference interface it stands in for (paths relative to the Stride
 * repository root). Every call returns an int status: SA_OK (0) or a negative
 * SA_E* code; sa_last_error() gives the message of the last failure on the
 * calling thread. No exception crosses the ABI. A plan is not thread-safe:
 * use one plan per host thread / stream.
 *
 * Pointers marked "host or device" are classified with cudaPointerGetAttributes:
 * device (or managed) pointers are used in place, host pointers are copied on
 * the call's stream (pageable or pinned).
 */
#ifndef STRIDEACC_H
#define STRIDEACC_H

#ifdef __cplusplus
extern "C" {
#endif

#define SA_OK 0
#define SA_E_INVALID (-1)     /* bad argument, shape or state (reference: ValueError) */
#define SA_E_UNSUPPORTED (-2) /* option the reference rejects or this build lacks (NotImplementedError) */
#define SA_E_CUDA (-3)        /* CUDA runtime error */
#define SA_E_NOMEM (-4)       /* device allocation failed */
#define SA_E_TIMEOUT (-5)     /* a bounded device wait gave up (error flag set by a kernel) */

#define SA_KERNEL_OT2 2
#define SA_KERNEL_OT4 4

#define SA_DENSITY_NONE 0     /* rho not given: vp^2 * laplace(p) */
#define SA_DENSITY_VARIABLE 1 /* vp^2 rho div(b grad p), staggered, b = 1/rho */
#define SA_DENSITY_CONSTANT 2 /* rho given but constant: vp^2 div(grad p), staggered */

#define SA_SAVE_NONE 0        /* forward only */
#define SA_SAVE_SNAPSHOTS 1   /* store p.dt2 every f steps (reference algorithm) */
#define SA_SAVE_CHECKPOINTS 2 /* store the state every checkpoint interval; the adjoint recomputes each
                                 segment's p.dt2 from its checkpoint (same gradient, less memory) */
#define SA_SAVE_RAW 3         /* store p[t] itself every f steps, as the reference does when the rho or
                                 wavelet gradient is needed (iso_acoustic/devito.py:410-413) */

#define SA_INTERP_LINEAR 0    /* bilinear / trilinear SparseTimeFunction (common/devito.py:580-653) */
#define SA_INTERP_HICKS 1     /* Kaiser-windowed sinc, 8 points per axis (common/devito.py:640-648,843-885);
                                 sources smoothed as the reference's src, receivers not */
#define SA_INTERP_SINC 2      /* Devito's SparseTimeFunction(interpolation='sinc', r=7) (common/devito.py:
                                 634-638): Kaiser-windowed sinc of half-width 7, 14 points per axis, no
                                 smoothing */

#define SA_BOUNDARY_SPONGE 0  /* SpongeBoundary2 (boundaries/devito.py:37-69), the reference's default */
#define SA_BOUNDARY_CFS_PML 1 /* ComplexFrequencyShiftPML2 (boundaries/devito.py:72-191): auxiliary fields on
                                 the absorbing slabs instead of the sponge; with OT2 (the combination the
                                 reference's own example runs), snapshot and raw saves */

#define SA_GRAD_PARITY 0      /* reference imaging condition: sum_{t%f==0} p_tt * p_a, interior only */
#define SA_GRAD_EXACT 1       /* gradient of the discrete forward map (its exact transpose), every grid
                                 point; needs SA_SAVE_CHECKPOINTS; 2D and 3D plans. No counterpart in the
                                 reference (whose gradient is SA_GRAD_PARITY) */

/* Options of sa_plan_option (no counterpart in the reference). */
#define SA_OPT_PERSISTENT 1     /* 2D forward without a saved wavefield as one persistent cooperative launch
                                   (linear interpolation, sponge): -1 never, 0 when the batch is small
                                   (default), 1 whenever eligible; the traces equal the step passes' bit for
                                   bit, and the call synchronises its stream to check the barrier status */
#define SA_OPT_BARRIER_EXTRA 2  /* for tests of the timeout path: each wait of the persistent launch for its
                                   neighbour tiles asks for this many steps more than it needs, so that no
                                   wait can complete and sa_forward returns SA_E_TIMEOUT (default 0) */
#define SA_OPT_BARRIER_SPIN 3   /* polls (each a global-memory load and a 32 ns sleep) before a persistent
                                   wait gives up and sets the kernel's error flag (default 10^7) */

/* Plan description (stride/physics/iso_acoustic/devito.py:119-183 defaults; shapes are the
 * extended grid of stride/problem/domain.py:48-74). */
typedef struct sa_desc {
    int dim;               /* 2 or 3 */
    int shape[3];          /* extended grid shape (x, y, z), z unused in 2D; last axis contiguous */
    double spacing[3];     /* metres */
    int extra[3];          /* padding cells per side: pml origin = -extra * spacing */
    int absorbing[3];      /* sponge cells per side (<= extra) */
    double dt;             /* seconds */
    int nt;                /* time samples (time.extended_num) */
    int kernel;            /* SA_KERNEL_OT2 or SA_KERNEL_OT4 */
    int density;           /* SA_DENSITY_* */
    int attenuation;       /* 0 none, 1 alpha given with attenuation power 0 */
    int undersampling;     /* f of the saved wavefield, >= 1 */
    int max_shots;         /* shots advanced together per launch */
    int checkpoint_interval;   /* steps between checkpoints for SA_SAVE_CHECKPOINTS (0: 50) */
    double checkpoint_budget;  /* bytes the checkpoints may use (0: no limit); widens the interval */
    int interpolation;         /* SA_INTERP_LINEAR, SA_INTERP_HICKS or SA_INTERP_SINC: sparse-point interpolation */
    int boundary;              /* SA_BOUNDARY_SPONGE or SA_BOUNDARY_CFS_PML */
    double f_centre;           /* Hz, centre of the propagated band (IsoAcousticDevito._bandwidth[1]): the
                                  CFS-PML's alpha = 0.01 pi f_centre; unused by the sponge */
} sa_desc;

typedef struct sa_plan sa_plan;

/* Creates a plan: validates the description and allocates the per-shot wavefields.
 * Replaces OperatorDevito.set_operator/compile (stride/physics/common/devito.py:909-1023). */
int sa_plan_create(const sa_desc* desc, sa_plan** out);

/* Frees every device buffer the plan owns (GridDevito.deallocate, common/devito.py:700-741). */
int sa_plan_destroy(sa_plan* plan);

/* Medium on the extended grid, C order, host or device float32: vp [m/s], rho [kg/m^3]
 * (NULL when desc.density == NONE), alpha [dB/cm] (NULL when desc.attenuation == 0).
 * Mirrors the vp/rho/buoy/alpha fills of before_forward (iso_acoustic/devito.py:476-497):
 * buoyancy is 1/rho and alpha is converted to Np/m with 100/(20 log10 e). */
int sa_set_medium(sa_plan* plan, const float* vp, const float* rho, const float* alpha);

/* Geometry of n_shots shots in CSR form (uneven counts allowed). src_offsets/rec_offsets have
 * n_shots+1 entries; src_xyz/rec_xyz are [total, dim] float32 coordinates in the inner-domain
 * frame (metres), already shifted by +1e-3*h as before_forward does (devito.py:307-309).
 * Host pointers. Replaces the src/rec SparseTimeFunction set-up (common/devito.py:580-653). */
int sa_set_geometry(sa_plan* plan, int n_shots, const int* src_offsets, const float* src_xyz,
                    const int* rec_offsets, const float* rec_xyz);

/* Forward modelling of every shot of the geometry. wavelets [n_src_total, nt] float32 are
 * the source samples as the reference stores them in src.data (Tukey-windowed; for
 * diff_source the caller passes dt * d/dt of the wavelet). traces [n_rec_total, nt] float32
 * receive rec.data.T (rows 0 and nt-1 of each trace are zero as in the reference's
 * time_m=1, time_M=nt-2 loop). save_mode SA_SAVE_SNAPSHOTS keeps p.dt2 every f steps for
 * sa_adjoint; SA_SAVE_CHECKPOINTS keeps the two state levels every checkpoint interval instead and
 * sa_adjoint recomputes each segment (the reference's layered/compressed wavefield storage,
 * devito.py:325-403, is the memory-saving counterpart). Host or device pointers; stream is a cudaStream_t (NULL = legacy default).
 * Replaces run_forward/after_forward (iso_acoustic/devito.py:515-685). */
int sa_forward(sa_plan* plan, const float* wavelets, float* traces, int save_mode, void* stream);

/* Adjoint of every shot: residuals [n_rec_total, nt] float32, the adjoint source as the
 * reference stores it in rec.data.T (Tukey-windowed as before_adjoint does, devito.py:863-869).
 * grad_vp/prec_vp [N] float32 on the extended grid receive the raw imaging condition summed
 * over the shots (Devito grad_vp/prec_vp data, zero outside the interior) before the
 * get_grad_vp chain rule. grad_mode SA_GRAD_PARITY. Requires a prior sa_forward with
 * SA_SAVE_SNAPSHOTS or SA_SAVE_CHECKPOINTS (then each segment is recomputed from its
 * checkpoint). Replaces run_adjoint/after_adjoint (devito.py:875-981).
 * grad_mode SA_GRAD_EXACT (2D, after SA_SAVE_CHECKPOINTS): residuals are dL/dtraces and grad_vp
 * receives dL/dvp of the discrete forward map at every point (no window, no interior cut, no
 * chain rule); prec_vp receives sum over all steps of p.dt2^2. */
int sa_adjoint(sa_plan* plan, const float* residuals, float* grad_vp, float* prec_vp, int grad_mode,
               void* stream);

/* sa_adjoint plus the gradient with respect to the wavelets: grad_wavelets [n_src_total, nt]
 * (host or device) receives -interp(p_a[t]) at the sources for t = 1 .. nt-1-f and zero
 * elsewhere, the reference's src.interpolate(expr=-p_a) (iso_acoustic/devito.py:755-756) read back
 * by get_grad_wavelets (:1226-1262). grad_mode SA_GRAD_PARITY; linear or Hicks interpolation (the
 * sources' smoothed support). */
int sa_adjoint_wavelets(sa_plan* plan, const float* residuals, float* grad_vp, float* prec_vp, float* grad_wavelets,
                        int grad_mode, void* stream);

/* The adjoint after a forward with SA_SAVE_RAW (2D and 3D), with the gradients the reference forms from
 * the raw saved wavefield p_s[n] = p[n f] (iso_acoustic/devito.py:985-1024, 1115-1150):
 *   vp:  p_dt = (p_s[n+1] - 2 p_s[n] + p_s[n-1]) / (f dt)^2,
 *   rho: g = -grad(b, shift=-1/2) . grad(p_s[n], shift=-1/2) - b laplace(p_s[n]), b = 1/rho,
 * each computed on the steps t = n f into a held buffer (the reference's p_dt_fun / grad_rho_fun,
 * written under the undersampling condition) and accumulated against p_a[t] on every adjoint
 * step: grad += held * p_a, prec += held^2, interior points, summed over the shots.
 * grad_vp/prec_vp [N] are required; grad_rho/prec_rho [N] (both or neither; the plan needs
 * rho, SA_DENSITY_VARIABLE or SA_DENSITY_CONSTANT) and grad_wavelets [n_src_total, nt]
 * (as sa_adjoint_wavelets) are optional. Host or device pointers. Replaces run_adjoint with
 * rho.needs_grad and/or wavelets.needs_grad, and get_grad_rho (:1171-1208). */
int sa_adjoint_grads(sa_plan* plan, const float* residuals, float* grad_vp, float* prec_vp, float* grad_rho,
                     float* prec_rho, float* grad_wavelets, void* stream);

/* Picks the launch layout for the current geometry by timing the candidates (no counterpart in
 * the reference, whose Devito autotuner is optional: common/devito.py:1043). 2D: the CTA width
 * and row chunking of the passes, and the time-blocking depth of forwards without a saved
 * wavefield (one step per launch, or every step in the persistent launch when SA_OPT_PERSISTENT
 * is automatic). 3D: the (y, z) tile and x chunking. Results are cached per grid, operator,
 * batch and device for the life of the process, so a second plan of the same shape takes them
 * without timing. It steps the plan's wavefield buffers, so it returns SA_E_INVALID while a
 * saved wavefield (snapshots or checkpoints of a forward with save) waits for its adjoint; a 3D
 * plan refuses while its saved wavefield is held. */
int sa_autotune(sa_plan* plan, void* stream);

/* Single-shot 2D forward modelling that allocates no device memory (no counterpart in the
 * reference). For callers that cannot let a library allocate GPU memory, e.g. an application
 * whose memory pool owns the whole device, or a loop that must not pay the device-wide
 * synchronisation of cudaFree. It runs the same time-step kernels as sa_forward with every
 * scratch buffer in one 64 MiB __device__ array of the library (held by each GPU that loads the
 * library until exit). Limits: extended grid at most 640 x 640, 16 sources, 1024 receivers,
 * and everything must fit the array (else SA_E_INVALID). desc gives the grid, dt, nt, kernel,
 * density and attenuation modes (max_shots and undersampling are not used). vp/rho/alpha
 * (unpadded extended grid), wavelets [n_src, nt] (as src.data) and traces [n_rec, nt] are
 * device pointers; src_xyz/rec_xyz are host [n, 2] coordinates, already shifted by +1e-3*h.
 * The first call on a device looks up the array's address with that device current: make it
 * before any stream capture. Calls share the array, so calls that overlap on the GPU race.
 * Every call synchronises `stream` twice while it prepares the point lists (it reads vp at the
 * source corners back to the host), so it blocks the calling host thread; host src_xyz/rec_xyz
 * are required (device pointers there return SA_E_INVALID). */
int sa_forward_2d_noalloc(const sa_desc* desc, const float* vp, const float* rho, const float* alpha, int n_src,
                          const float* src_xyz, const float* wavelets, int n_rec, const float* rec_xyz, float* traces,
                          void* stream);

/* ---- Trace and field processing of the optimisation pipelines (device pointers, stream-ordered) ----
 * Traces are [n, nt] float32 row-major (Traces.extended_data); fields are float32 row-major. */

/* Cascaded second-order sections (scipy.signal.sosfilt, FP64 state), n_sections rows of
 * (b0 b1 b2 a0 a1 a2) in host memory; adjoint runs on the time-reversed traces.
 * Replaces the butterworth filters of stride/utils/filters.py:14-170 (zero_phase=False) as
 * FilterTraces calls them (optimisation/pipelines/steps/filter_traces.py:57-96). in may equal out. */
int sa_traces_sosfilt(const float* in, float* out, int n, int nt, const double* sos, int n_sections, int adjoint,
                      void* stream);

/* FIR filter out[t] = sum_k taps[k] in[t + k - center] (zero outside the trace), taps FP64 on the
 * device; adjoint: the same on the time-reversed traces. With the cosine table of
 * utils/filters.py:400-410 and center = 2 * period it is lowpass_filter_cos(zero_phase=False)
 * (:413-465); with reversed firwin taps and center = ntaps - 1 it is the causal FIR filters
 * (:213-397). out must not alias in. */
int sa_traces_fir(const float* in, float* out, int n, int nt, const double* taps, int ntaps, int center,
                  int adjoint, void* stream);

/* Per-trace NaN/inf flags (flags [n] int on the device) and, with zero_bad, the flagged traces
 * zeroed (CheckTraces, optimisation/pipelines/steps/check_traces.py:44-78). */
int sa_traces_check(float* traces, int n, int nt, int* flags, int zero_bad, void* stream);

/* out = in / (sqrt(sum of squares of the shot's traces / its trace count) + 1e-31) per shot, the
 * shots given by device CSR trace offsets [n_shots + 1]; scratch: n_shots doubles on the device
 * (NormPerShot, optimisation/pipelines/steps/norm_traces.py:43-69). in may equal out. */
int sa_traces_norm_per_shot(const float* in, float* out, const int* offsets, int n_shots, int nt, double* scratch,
                            void* stream);

/* out = modelled * lowpass(observed != 0), the cosine lowpass centred (MuteTraces,
 * optimisation/pipelines/steps/mute_traces.py:25-57); taps FP64 on the device, odd count. */
int sa_traces_mute(const float* modelled, const float* observed, float* out, int n, int nt, const double* taps,
                   int ntaps, void* stream);

/* x *= m elementwise (MaskField's mask, optimisation/pipelines/steps/mask_field.py:52-70). */
int sa_field_mul(float* x, const float* m, long long n, void* stream);

/* Clip to [*lo, *hi] (either pointer NULL: no bound; Clip, steps/clip.py:25-36). */
int sa_field_clip(float* x, long long n, const float* lo, const float* hi, void* stream);

/* x += a * d elementwise (the update of optimisers/optimiser.py:273-298 without a transform). */
int sa_field_axpy(float* x, const float* d, long long n, float a, void* stream);

/* vp = 1 / (1 / vp - step * direction): the update in slowness, as the vp variable's transform
 * makes it. */
int sa_field_slowness_step(float* vp, const float* direction, long long n, float step, void* stream);

/* out4[0..2] = min, max, max |x|; *sum_abs = sum |x| (FP64). Synchronises the stream. n >= 1.
 * (NormField, steps/norm_field.py:24-52; apply_prec's sum, problem/data.py:437.) */
int sa_field_stats(const float* x, long long n, float* out4, double* sum_abs, void* stream);

/* x *= a (in FP64, rounded once). */
int sa_field_scale(float* x, long long n, double a, void* stream);

/* In-place Gaussian smoothing as scipy.ndimage.gaussian_filter (truncate 4, one pass per axis,
 * FP32 between passes); shape[dim], sigma[dim] on the host; border 0 'nearest' (SmoothField,
 * steps/smooth_field.py:27-47), 1 'reflect' (apply_prec, problem/data.py:432); scratch: a device
 * array of the field's size. Synchronises the stream. */
int sa_field_gaussian(float* x, int dim, const int* shape, const double* sigma, int border, float* scratch,
                      void* stream);

/* prec = prec * factor + 1 (FP64, rounded once) and grad *= 1 / prec (FP32) where prec != 0
 * (Data.apply_prec, stride/problem/data.py:411-446, after its smoothing and factor). */
int sa_field_apply_prec(float* grad, float* prec, long long n, double factor, void* stream);

/* ---- Learned preconditioner (no counterpart in the reference) ----
 * BF16 GEMM on the tcgen05 tensor cores: C[M][N] = (accumulate ? C : 0) + A[M][K] * B[N][K]^T
 * (+ bias[N], then ReLU if relu), A and B bf16 with K contiguous (lda, ldb elements, multiples of
 * 8, 16-byte aligned bases), C fp32 (ldc); Cb (optional, ldcb) receives C as bf16. M multiple of
 * 128, K of 16, N of 32. ksplit > 1 splits K over that many CTAs per tile, which add their partial
 * products into C atomically (accumulate 1, no bias/ReLU/Cb), or, with accumulate 2, store them to
 * slabs C + z M ldc, z < the number of splits (at most ksplit; the caller sums them in a fixed order
 * with sa_nn_sum_slabs, a reproducible result). *err (device int) is set to 1 if an internal wait
 * timed out. */
int sa_gemm_bf16(const void* A, int lda, const void* B, int ldb, float* C, int ldc, void* Cb, int ldcb, int M, int N,
                 int K, const float* bias, int relu, int accumulate, int ksplit, int* err, void* stream);

/* 3x3 convolution (padding 1) as an implicit GEMM on the tcgen05 tensor cores: C[P][N] = A W^T
 * (+ bias, ReLU; Cb optional bf16 copy), P = B*H*W pixels (a multiple of 128), where A[P][Kp] is the
 * im2col of x built in shared memory, never in HBM: column (ky*3+kx)*Cin+ci of pixel p is channel ci
 * of its neighbour (ky-1, kx-1) in x, bf16 NHWC [P][ldx] (zero outside the image and for columns
 * >= 9*Cin). Wt bf16 [N][ldw] with the same column order; Cin and ldx multiples of 8, Kp >= 9*Cin a
 * multiple of 16, N of 32, H <= 32767, W <= 65535. *err as for sa_gemm_bf16. */
int sa_conv3x3_bf16(const void* x, int ldx, int B, int H, int W, int Cin, const void* Wt, int ldw, float* C, int ldc,
                    void* Cb, int ldcb, int N, int Kp, const float* bias, int relu, int* err, void* stream);

/* U-Net layer kernels (NHWC fp32 activations [pixels][channels] with channel stride ld; bf16 GEMM
 * operands; B images of H x W). No counterpart in the reference. */
/* col bf16 [B*H*W][Kp]: column (ky*3+kx)*Cin+ci of pixel p = x at the 3x3 neighbour (zero outside
 * the image and for columns >= 9*Cin). */
int sa_nn_im2col(const float* x, int ldx, int B, int H, int W, int Cin, void* col, int Kp, void* stream);
/* dx (= or +=) the gather of dcol fp32 [B*H*W][Kp] back to the pixels its columns read. */
int sa_nn_col2im(const float* dcol, int Kp, int B, int H, int W, int Cin, float* dx, int ldx, int accumulate,
                 void* stream);
/* out[i] (= or += with accumulate) sum over z < n_slabs, in order, of in[z slab + i], i < n: the
 * fixed-order reduction of sa_gemm_bf16's split-K slabs. */
int sa_nn_sum_slabs(const float* in, long long slab, int n_slabs, float* out, long long n, int accumulate,
                    void* stream);
/* out[c][r] = in[r][c] (bf16), r < R, c < C; output rows C..Cp-1 are zero. */
int sa_nn_transpose_bf16(const void* in, int ldi, int R, int C, void* out, int ldo, int Cp, void* stream);
int sa_nn_to_bf16(const float* x, int ldx, long long rows, int C, void* y, int ldy, void* stream);
/* dy = 0 where y <= 0 (ReLU backward from the activation output). */
int sa_nn_relu_bwd(float* dy, int ldd, const float* y, int ldy, long long rows, int C, void* stream);
/* db[c] = sum over rows of dy[r][c], summed in a fixed order (reproducible); scratch: device
 * doubles, 128 * C of them. */
int sa_nn_bias_grad(const float* dy, int ldd, long long rows, int C, float* db, double* scratch, void* stream);
/* 2x2 max pooling (H, W of the input, even) and its backward (gradient to the first maximum). */
int sa_nn_maxpool(const float* x, int ldx, int B, int H, int W, int C, float* y, int ldy, void* stream);
int sa_nn_maxpool_bwd(const float* x, int ldx, const float* dy, int ldd, int B, int H, int W, int C, float* dx,
                      int lddx, int accumulate, void* stream);
/* Nearest x2 upsampling (H, W of the output, even) and its backward (sum of the 4 children). */
int sa_nn_upsample(const float* x, int ldx, int B, int H, int W, int C, float* y, int ldy, void* stream);
int sa_nn_upsample_bwd(const float* dy, int ldd, int B, int H, int W, int C, float* dx, int lddx, void* stream);
/* dst[r][c] (= or +=) src[r][c], c < C (channel concatenation and split). */
int sa_nn_copy_channels(const float* src, int lds, long long rows, int C, float* dst, int ldd, int accumulate,
                        void* stream);
/* fp32 weights [Cout][Kr] -> bf16 [Coutp][Kp] (GEMM B operand) and its transpose [Kp][Coutp]. */
int sa_nn_pack_weights(const float* w, int Cout, int Kr, void* wb, void* wt, int Coutp, int Kp, void* stream);
/* Adam step (bias-corrected, step >= 1) on fp32 master weights. */
int sa_nn_adam(float* w, const float* g, float* m, float* v, long long n, float lr, float b1, float b2, float eps,
               int step, void* stream);
/* Adam's bias corrections for steps 1..nsteps, c12[2k] = 1 - b1^(k+1), c12[2k+1] = 1 - b2^(k+1)
 * (the values sa_nn_adam forms), into device memory (synchronous). */
int sa_nn_adam_corrections(float b1, float b2, int nsteps, float* c12);
/* sa_nn_adam with the step read from device memory (*step, clamped to 1..nsteps) and its bias
 * corrections from c12: the form a captured training step (CUDA graph) replays. */
int sa_nn_adam_dev(float* w, const float* g, float* m, float* v, long long n, float lr, float b1, float b2, float eps,
                   const float* c12, int nsteps, const int* step, void* stream);
/* *loss = mean (out - target)^2 (FP64, device), dout = 2 (out - target) / n. */
int sa_nn_mse(const float* out, int ldo, const float* target, long long n, float* dout, int ldd, double* loss,
              void* stream);

/* Copies the message of the last failed call on this thread (NUL-terminated, truncated to len). */
int sa_last_error(char* buf, int len);

/* Kernel launches the last sa_forward/sa_adjoint issued (for throughput accounting). */
long long sa_launch_count(const sa_plan* plan);

/* Sets a plan option (SA_OPT_*). No counterpart in the reference. */
int sa_plan_option(sa_plan* plan, int option, long long value);

/* The launch layout of a plan's time-step passes (after sa_autotune, the tuned one). 2D: threads
 * per CTA (two grid columns each), column strips and row chunks of the grid. 3D: threads per CTA
 * (one (y, z) column each, two shots per thread), (y, z) tiles and x chunks. No counterpart in the
 * reference. */
int sa_plan_layout(const sa_plan* plan, int* threads, int* strips, int* chunks);

/* The checkpoint schedule sa_forward(SA_SAVE_CHECKPOINTS) takes for n_shots shots of a plan with
   description d (its checkpoint_interval, checkpoint_budget, grid, nt, undersampling, boundary):
   coarse interval *K and *n_ckpt checkpoints, and *K2 the fine interval of a two-level schedule (0:
   one level). SA_E_NOMEM when no schedule fits the budget. Host only: no device work. Replaces the
   memory planning the reference leaves to Devito's save options (iso_acoustic/devito.py:325-403). */
int sa_checkpoint_schedule(const sa_desc* d, int n_shots, int* K, int* n_ckpt, int* K2);

#ifdef __cplusplus
}
#endif
#endif

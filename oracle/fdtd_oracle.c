/*
 * C/OpenMP oracle for the iso-acoustic FDTD hot path (test infrastructure only).
 *
 * Restates the time loop of the reference's IsoAcousticDevito operator
 * (stride/physics/iso_acoustic/devito.py:1466-1608 stencil, :357-364 source
 * injection / receiver interpolation, :398-418 undersampled p.dt2 save,
 * :741-753 adjoint stencil and receiver injection, :1000-1024 vp imaging
 * condition) for 2D and 3D grids. The host-side preparation (damping profile,
 * interpolation weights, Tukey windows, attenuation units) is done by the
 * Python wrapper oracle/c_oracle.py with the same functions as the NumPy
 * restatement, so this file and oracle/numpy_oracle.py are independent
 * restatements of the time loop only.
 *
 * Used by the tests as the checker at full configuration sizes and by bench.py
 * as the timed CPU baseline; never by the product path. Parity against Devito
 * itself is unpinned (Devito is a third-party JIT compiler that is not vendored).
 *
 * Build: oracle/Makefile (gcc -O3 -fopenmp -ffp-contract=off, so that x86_64
 * and aarch64 round identically).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PAD 10 /* zero halo for fields, edge halo for materials: covers radius 9 */

typedef struct {
    int dim;
    int n[3];          /* extended grid shape; n[2] = 1 in 2D */
    double h[3];
    double dt;
    int nt;
    int kernel;        /* 2 = OT2, 4 = OT4 */
    int rho_mode;      /* 0 laplace, 1 variable density, 2 constant density (staggered, b = 1) */
    int has_alpha;
    int f;             /* undersampling factor */
    int absorbing[3];
    int nthreads;
} ora_desc;

typedef struct {
    int dim;
    int n[3], np[3];
    long long sx, sy, sz, total;
    double h[3];
} grid_t;

static const double W2[6] = {-5269.0 / 1800.0, 5.0 / 3.0, -5.0 / 21.0, 5.0 / 126.0, -5.0 / 1008.0, 1.0 / 3150.0};
static const double WS[5] = {19845.0 / 16384.0, -735.0 / 8192.0, 567.0 / 40960.0, -405.0 / 229376.0,
                             35.0 / 294912.0};

static void grid_init(grid_t* g, const ora_desc* d) {
    g->dim = d->dim;
    for (int i = 0; i < 3; i++) {
        g->n[i] = (i < d->dim) ? d->n[i] : 1;
        g->np[i] = (i < d->dim) ? d->n[i] + 2 * PAD : 1;
        g->h[i] = d->h[i];
    }
    g->sz = 1;
    g->sy = g->np[2];
    g->sx = (long long)g->np[1] * g->np[2];
    g->total = (long long)g->np[0] * g->sx;
}

static inline long long gidx(const grid_t* g, int x, int y, int z) {
    int oz = g->dim == 3 ? PAD : 0;
    return (long long)(x + PAD) * g->sx + (long long)(y + PAD) * g->sy + (z + oz);
}

static long long stride_of(const grid_t* g, int a) { return a == 0 ? g->sx : (a == 1 ? g->sy : g->sz); }

/* copy an unpadded array into a padded one; edge-extend if edge != 0 else zero halo */
static void pad_in(const grid_t* g, const float* src, float* dst, int edge) {
    memset(dst, 0, sizeof(float) * g->total);
    int nz = g->n[2], ny = g->n[1], nx = g->n[0];
    int lo = -PAD, hx = nx + PAD, hy = ny + PAD;
    int loz = g->dim == 3 ? -PAD : 0, hz = g->dim == 3 ? nz + PAD : 1;
    for (int x = lo; x < hx; x++)
        for (int y = lo; y < hy; y++)
            for (int z = loz; z < hz; z++) {
                int inside = x >= 0 && x < nx && y >= 0 && y < ny && z >= 0 && z < nz;
                if (!inside && !edge) continue;
                int cx = x < 0 ? 0 : (x >= nx ? nx - 1 : x);
                int cy = y < 0 ? 0 : (y >= ny ? ny - 1 : y);
                int cz = z < 0 ? 0 : (z >= nz ? nz - 1 : z);
                dst[gidx(g, x, y, z)] = src[((long long)cx * ny + cy) * nz + cz];
            }
}

typedef struct {
    grid_t g;
    const ora_desc* d;
    float *vp2, *w;       /* node coefficient of the operator: vp^2 or vp^2 rho */
    float* bh[3];         /* buoyancy at half points i+1/2 along each axis (padded grid) */
    float *F, *tmp, *lap; /* scratch */
    float *vp, *alpha, *damp;
} op_t;

/* out = W * G(u) on the grid nodes; u has a zero halo. */
static void apply_op(op_t* o, const float* u, float* out) {
    const grid_t* g = &o->g;
    int nx = g->n[0], ny = g->n[1], nz = g->n[2];
    int dim = g->dim;
    if (o->d->rho_mode == 0) {
#pragma omp parallel for schedule(static)
        for (int x = 0; x < nx; x++)
            for (int y = 0; y < ny; y++)
                for (int z = 0; z < nz; z++) {
                    long long i = gidx(g, x, y, z);
                    float acc = 0.f;
                    for (int a = 0; a < dim; a++) {
                        long long s = stride_of(g, a);
                        float v = (float)W2[0] * u[i];
                        for (int k = 1; k <= 5; k++) v += (float)W2[k] * (u[i + k * s] + u[i - k * s]);
                        acc += v / (float)(g->h[a] * g->h[a]);
                    }
                    out[i] = o->vp2[i] * acc;
                }
        return;
    }
    /* staggered: per axis F at half points j+1/2 (stored at j) then D- */
    memset(o->tmp, 0, sizeof(float) * g->total);
    for (int a = 0; a < dim; a++) {
        long long s = stride_of(g, a);
        float ih = (float)g->h[a];
        /* F for j in [-5, n_a+3] along axis a, all nodes along the other axes */
        int lo[3] = {0, 0, 0}, hi[3] = {nx, ny, nz};
        lo[a] = -5;
        hi[a] = g->n[a] + 4;
#pragma omp parallel for schedule(static)
        for (int x = lo[0]; x < hi[0]; x++)
            for (int y = lo[1]; y < hi[1]; y++)
                for (int z = lo[2]; z < hi[2]; z++) {
                    long long j = gidx(g, x, y, z);
                    float v = 0.f;
                    for (int k = 0; k < 5; k++) v += (float)WS[k] * (u[j + (k + 1) * s] - u[j - k * s]);
                    v = v / ih;
                    if (o->d->rho_mode == 1) v = v * o->bh[a][j];
                    o->F[j] = v;
                }
#pragma omp parallel for schedule(static)
        for (int x = 0; x < nx; x++)
            for (int y = 0; y < ny; y++)
                for (int z = 0; z < nz; z++) {
                    long long i = gidx(g, x, y, z);
                    float v = 0.f;
                    for (int k = 0; k < 5; k++) v += (float)WS[k] * (o->F[i + k * s] - o->F[i - (k + 1) * s]);
                    o->tmp[i] += v / ih;
                }
    }
#pragma omp parallel for schedule(static)
    for (int x = 0; x < nx; x++)
        for (int y = 0; y < ny; y++)
            for (int z = 0; z < nz; z++) {
                long long i = gidx(g, x, y, z);
                out[i] = o->w[i] * o->tmp[i];
            }
}

/* one time update: next = solve(...) from cur (p[t]) and other (p[t-1] forward, p[t+1]
 * backward). p.dt2 - Lt + 2 alpha vp p.dt + vp^2 (2 d p.dtc + d^2 p) = 0 with centred first
 * derivatives; the backward operator uses the transposed (negated) ones, which is the same
 * formula with the two neighbouring levels exchanged (iso_acoustic/devito.py:1536-1581,
 * boundaries/devito.py:62-67). OT4: Lt = l + dt^2/12 L(l), l = L p (devito.py:1503-1534). */
static void step(op_t* o, const float* cur, const float* other, float* next, float* lap4) {
    const grid_t* g = &o->g;
    int nx = g->n[0], ny = g->n[1], nz = g->n[2];
    float dt = (float)o->d->dt;
    apply_op(o, cur, o->lap);
    if (o->d->kernel == 4) apply_op(o, o->lap, lap4);
    float k12 = (float)(o->d->dt * o->d->dt / 12.0);
#pragma omp parallel for schedule(static)
    for (int x = 0; x < nx; x++)
        for (int y = 0; y < ny; y++)
            for (int z = 0; z < nz; z++) {
                long long i = gidx(g, x, y, z);
                float Lt = o->lap[i];
                if (o->d->kernel == 4) Lt = Lt + k12 * lap4[i];
                float vp = o->vp[i], vp2 = vp * vp, d = o->damp[i];
                float beta = vp2 * d;
                if (o->d->has_alpha) beta = beta + o->alpha[i] * vp;
                beta = dt * beta;
                float num = dt * dt * Lt + (2.f - dt * dt * vp2 * d * d) * cur[i] - (1.f - beta) * other[i];
                next[i] = num / (1.f + beta);
            }
}

typedef struct {
    op_t o;
    float *p0, *p1, *p2, *lap4;
} state_t;

static int state_init(state_t* s, const ora_desc* d, const float* vp, const float* rho, const float* alpha,
                      const float* damp) {
    memset(s, 0, sizeof(*s));
    op_t* o = &s->o;
    o->d = d;
    grid_init(&o->g, d);
    long long T = o->g.total;
    float** bufs[] = {&o->vp2, &o->w, &o->F, &o->tmp, &o->lap, &o->vp, &o->alpha, &o->damp,
                      &s->p0, &s->p1, &s->p2, &s->lap4, &o->bh[0], &o->bh[1], &o->bh[2]};
    for (unsigned i = 0; i < sizeof(bufs) / sizeof(bufs[0]); i++) {
        *bufs[i] = (float*)calloc((size_t)T, sizeof(float));
        if (!*bufs[i]) return -1;
    }
    pad_in(&o->g, vp, o->vp, 1);
    pad_in(&o->g, damp, o->damp, 0);
    if (alpha) pad_in(&o->g, alpha, o->alpha, 1);
    for (long long i = 0; i < T; i++) o->vp2[i] = o->vp[i] * o->vp[i];
    if (d->rho_mode == 1) {
        float* r = o->F; /* temporary: padded rho, edge halo */
        pad_in(&o->g, rho, r, 1);
        for (long long i = 0; i < T; i++) o->w[i] = o->vp2[i] * r[i];
        /* buoyancy = 1/rho on the padded grid, half points along each axis */
        for (long long i = 0; i < T; i++) o->tmp[i] = r[i] != 0.f ? 1.f / r[i] : 0.f;
        for (int a = 0; a < d->dim; a++) {
            long long st = stride_of(&o->g, a);
            for (long long i = 0; i + st < T; i++) o->bh[a][i] = 0.5f * (o->tmp[i] + o->tmp[i + st]);
        }
        /* half points at the top edge: both nodes edge copies */
        for (int a = 0; a < d->dim; a++) {
            long long st = stride_of(&o->g, a);
            for (long long i = T - st; i < T; i++) o->bh[a][i] = o->tmp[i];
        }
    } else {
        for (long long i = 0; i < T; i++) o->w[i] = o->vp2[i];
    }
    return 0;
}

static void state_free(state_t* s) {
    op_t* o = &s->o;
    float* bufs[] = {o->vp2, o->w, o->F, o->tmp, o->lap, o->vp, o->alpha, o->damp,
                     s->p0, s->p1, s->p2, s->lap4, o->bh[0], o->bh[1], o->bh[2]};
    for (unsigned i = 0; i < sizeof(bufs) / sizeof(bufs[0]); i++) free(bufs[i]);
}

static long long unpadded_to_padded(const grid_t* g, long long flat) {
    int nz = g->n[2], ny = g->n[1];
    int z = (int)(flat % nz);
    int y = (int)((flat / nz) % ny);
    int x = (int)(flat / ((long long)nz * ny));
    return gidx(g, x, y, z);
}

/*
 * Forward modelling of one shot. Sparse points are given per corner: flat unpadded indices
 * [n_pts * ncorner] and weights (double). src [nt * n_src] is already Tukey-windowed; the
 * injected amount at a corner is w * src[t] * src_scale * vp[corner]
 * (iso_acoustic/devito.py:349-363). rec [nt * n_rec] receives sum w * p[t+1][corner] for
 * t = 1..nt-2 (rows 0 and nt-1 stay zero). snaps [(nt+f)/f + 1, N] gets
 * (p[t+1] - 2 p[t] + p[t-1]) / dt^2 on t % f == 0 when save != 0.
 */
int ora_forward(const ora_desc* d, const float* vp, const float* rho, const float* alpha, const float* damp,
                int n_src, const long long* src_idx, const double* src_w, const float* src, double src_scale,
                int n_rec, const long long* rec_idx, const double* rec_w, float* rec, int save, float* snaps) {
#ifdef _OPENMP
    if (d->nthreads > 0) omp_set_num_threads(d->nthreads);
#endif
    state_t s;
    if (state_init(&s, d, vp, rho, alpha, damp)) {
        state_free(&s);
        return -1;
    }
    const grid_t* g = &s.o.g;
    int nc = 1 << d->dim;
    long long N = (long long)g->n[0] * g->n[1] * g->n[2];
    memset(rec, 0, sizeof(float) * (size_t)d->nt * n_rec);
    float *pm = s.p0, *p = s.p1, *pn = s.p2;
    float idt2 = (float)(d->dt * d->dt);
    for (int t = 1; t <= d->nt - 2; t++) {
        step(&s.o, p, pm, pn, s.lap4);
        for (int i = 0; i < n_src; i++)
            for (int c = 0; c < nc; c++) {
                long long pi = unpadded_to_padded(g, src_idx[i * nc + c]);
                double amp = (double)src[(long long)t * n_src + i] * src_scale * (double)s.o.vp[pi];
                pn[pi] += (float)(src_w[i * nc + c] * amp);
            }
        for (int r = 0; r < n_rec; r++) {
            double acc = 0.0;
            for (int c = 0; c < nc; c++)
                acc += rec_w[r * nc + c] * (double)pn[unpadded_to_padded(g, rec_idx[r * nc + c])];
            rec[(long long)t * n_rec + r] = (float)acc;
        }
        if (save && t % d->f == 0) {
            float* out = snaps + (long long)(t / d->f) * N;
#pragma omp parallel for schedule(static)
            for (long long q = 0; q < N; q++) {
                long long i = unpadded_to_padded(g, q);
                out[q] = (pn[i] - 2.f * p[i] + pm[i]) / idt2;
            }
        }
        float* tmp = pm;
        pm = p;
        p = pn;
        pn = tmp;
    }
    state_free(&s);
    return 0;
}

/*
 * Reverse-time adjoint of the reference (iso_acoustic/devito.py:689-920): for
 * t = nt-1-f .. 1, q[t-1] from q[t], q[t+1]; q[t-1][corner] += w * (-res[t] * dt^2 * vp^2[corner]);
 * on t % f == 0 inside the interior (absorbing cells excluded): grad += snap[t/f] * q[t],
 * prec += snap[t/f]^2 (devito.py:985-1024). grad/prec are unpadded [N] and accumulated.
 */
int ora_adjoint(const ora_desc* d, const float* vp, const float* rho, const float* alpha, const float* damp,
                int n_rec, const long long* rec_idx, const double* rec_w, const float* res, const float* snaps,
                float* grad, float* prec) {
#ifdef _OPENMP
    if (d->nthreads > 0) omp_set_num_threads(d->nthreads);
#endif
    state_t s;
    if (state_init(&s, d, vp, rho, alpha, damp)) {
        state_free(&s);
        return -1;
    }
    const grid_t* g = &s.o.g;
    int nc = 1 << d->dim;
    long long N = (long long)g->n[0] * g->n[1] * g->n[2];
    float *qp = s.p0, *q = s.p1, *qn = s.p2;
    double dt2 = d->dt * d->dt;
    int nx = g->n[0], ny = g->n[1], nz = g->n[2];
    int A0 = d->absorbing[0], A1 = d->absorbing[1], A2 = d->dim == 3 ? d->absorbing[2] : 0;
    for (int t = d->nt - 1 - d->f; t >= 1; t--) {
        step(&s.o, q, qp, qn, s.lap4);
        for (int r = 0; r < n_rec; r++)
            for (int c = 0; c < nc; c++) {
                long long pi = unpadded_to_padded(g, rec_idx[r * nc + c]);
                double v = (double)s.o.vp[pi];
                double amp = -(double)res[(long long)t * n_rec + r] * dt2 * (double)(float)(v * v);
                qn[pi] += (float)(rec_w[r * nc + c] * amp);
            }
        if (t % d->f == 0) {
            const float* sn = snaps + (long long)(t / d->f) * N;
#pragma omp parallel for schedule(static)
            for (int x = A0; x < nx - A0; x++)
                for (int y = A1; y < ny - A1; y++)
                    for (int z = A2; z < nz - A2; z++) {
                        long long qi = ((long long)x * ny + y) * nz + z;
                        float sv = sn[qi];
                        grad[qi] += sv * q[gidx(g, x, y, z)];
                        prec[qi] += sv * sv;
                    }
        }
        float* tmp = qp;
        qp = q;
        q = qn;
        qn = tmp;
    }
    state_free(&s);
    return 0;
}

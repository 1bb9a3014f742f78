// Persistent 2D forward for batches too small to fill the GPU with the streaming step passes.
//
// One cooperative launch runs every time step of the forward (the loop OperatorDevito.run drives,
// stride/physics/common/devito.py:1025-1070). Each CTA owns a tile of one shot pair and keeps in
// shared memory, for the whole run, the medium of its region, p[t-1] and p[t] of its tile and the
// halo of p[t]. CTAs exchange the tiles through global memory as self-validating lines (the value
// of a point with its level number in one 16-byte store), so that no fence, flag or barrier is
// needed: a CTA polls the lines of its halo until they hold the level it needs. A step of a CTA:
//   1. (t > 1) the halo of p[t], a ring of 2R (OT4) or R (OT2) points (zero beyond the grid,
//      Devito's halo of p); the receivers of the step before, rec[t-1] = interp(p[t])
//      (iso_acoustic/devito.py:364), by the CTA that holds each receiver's base corner;
//   2. OT4: l = W G(p[t]) over the tile and R more (zero beyond the grid, as Devito's `laplacian`),
//      recomputed by each CTA for its halo so that no second exchange is needed;
//   3. the update of the tile, p[t+1] = C1 Lt + C2 p[t] - C3 p[t-1];
//   4. the sources of step t at the tile's points (iso_acoustic/devito.py:357-363), each target
//      point's entries summed in a fixed order;
//   5. p[t+1] of the tile to its exchange lines (two slots, by the parity of the level).
// A slot is rewritten two levels later, by which time every neighbour has read it: a CTA that
// writes level t+1 has read level t of each neighbour, which that neighbour wrote after reading
// its halo of level t-1. Every point's arithmetic is the step passes' (fdtd2d.cuh) operation for
// operation, so the traces equal the streaming forward's bit for bit.
//
// The polls are bounded: a wait that gives up sets an error flag, every CTA leaves the time loop
// at its next wait, and the host reports SA_E_TIMEOUT. The cooperative launch guarantees that every
// CTA is resident, so that no wait depends on a CTA that cannot start.
#include <cooperative_groups.h>

#include "fdtd2d.cuh"
#include "persist2d.h"

namespace sa {

namespace {

// Exchange lines: p at one point of a shot pair with the level it belongs to, {p0, level, p1, level}
// as 32-bit words, stored and loaded as one 16-byte access of two 64-bit elements, each a value in
// its low word and the level in its high word. The memory model treats the elements of a vector
// access as separate accesses, each naturally aligned 64-bit element as one single-copy atomic
// access: a reader takes a line when both level words match, and each element then holds that
// level's value.
__device__ __forceinline__ void st_line(uint4* q, float2 v, unsigned level) {
    const unsigned long long hi = (unsigned long long)level << 32;
    asm volatile("st." PERSIST_LINE_SEM ".global.v2.u64 [%0], {%1, %2};" ::"l"(q),
                 "l"(hi | __float_as_uint(v.x)), "l"(hi | __float_as_uint(v.y))
                 : "memory");
}

__device__ __forceinline__ uint4 ld_line(const uint4* q) {
    unsigned long long e0, e1;
    asm volatile("ld." PERSIST_LINE_SEM ".global.v2.u64 {%0, %1}, [%2];" : "=l"(e0), "=l"(e1) : "l"(q) : "memory");
    return make_uint4((unsigned)e0, (unsigned)(e0 >> 32), (unsigned)e1, (unsigned)(e1 >> 32));
}

// Buoyancy tables of a CTA in shared memory: bx at half-rows [fx0, fx0 + fh) x columns
// [fy0, fy0 + fw), by at rows [gx0, gx0 + gh) x half-columns [gy0, gy0 + gw).
struct BTables {
    const float* bx;
    const float* by;
    int fx0, fy0, fw, gx0, gy0, gw;
};

// Rows of padding below the shared arrays that stencil_region reads: a block of NR output rows
// may run past the region's last row by up to NR - 1 rows, whose loads land in the padding.
constexpr int PERSIST_NR_MAX = 4;

// G(in) over the output region [ox0, ox1) x [oy0, oy1) of shared array `in` (origin (ix0, iy0),
// row stride iw; it covers the region and R more on every side, and PERSIST_NR_MAX - 1 rows of
// padding); epi(x, y, g) per output point. A thread computes a block of NR rows of one column,
// the x-direction loads shared between the rows. Staggered kinds stage the x- and y-fluxes in sFX
// / sFY first. Operation for operation the arithmetic of the step passes' queues and windows.
template <int KIND, int NR, class Epi>
__device__ __forceinline__ void stencil_region(const Step2D& a, const float2* in, int ix0, int iy0, int iw, int ox0,
                                               int ox1, int oy0, int oy1, float2* sFX, float2* sFY, const BTables& B,
                                               Epi epi) {
    static_assert(NR >= 1 && NR <= PERSIST_NR_MAX, "row block");
    constexpr bool STAG = KIND != 0, VARB = KIND == 1;
    const int NTH = blockDim.x, tid = threadIdx.x;
    const int ow = oy1 - oy0, oh = ox1 - ox0;
    if constexpr (STAG) {
        // x-fluxes at half-rows ox0 - 5 .. ox1 + 3 (flux h at h + 1/2), columns of the region
        const int fh = oh + 9, nbf = (fh + NR - 1) / NR;
        for (int e = tid; e < nbf * ow; e += NTH) {
            const int rb = e / ow, yc = e - rb * ow, h0 = ox0 - 5 + rb * NR, y = oy0 + yc;
            const float2* col = in + (h0 - 4 - ix0) * iw + (y - iy0);  // rows h0 - 4 ..
            float2 w[NR + 9];
#pragma unroll
            for (int i = 0; i < NR + 9; i++) w[i] = col[i * iw];
#pragma unroll
            for (int r = 0; r < NR; r++) {
                const int h = h0 + r;
                if (h - (ox0 - 5) >= fh) break;
                float2 acc = mul2(a.wx[0], sub2(w[r + 5], w[r + 4]));
#pragma unroll
                for (int m = 1; m < 5; m++) acc = fma2(a.wx[m], sub2(w[r + 5 + m], w[r + 4 - m]), acc);
                if constexpr (VARB) acc = mul2(acc, f2(B.bx[(h - B.fx0) * B.fw + (y - B.fy0)]));
                sFX[(h - (ox0 - 5)) * ow + yc] = acc;
            }
        }
        // y-fluxes at half-columns oy0 - 5 .. oy1 + 3, rows of the region
        for (int e = tid; e < oh * (ow + 9); e += NTH) {
            const int xr = e / (ow + 9), x = ox0 + xr, hc = oy0 - 5 + (e - xr * (ow + 9));
            const float2* row = in + (x - ix0) * iw + (hc - iy0);
            float2 acc = mul2(a.wy[0], sub2(row[1], row[0]));
#pragma unroll
            for (int m = 1; m < 5; m++) acc = fma2(a.wy[m], sub2(row[1 + m], row[-m]), acc);
            if constexpr (VARB) acc = mul2(acc, f2(B.by[(x - B.gx0) * B.gw + (hc - B.gy0)]));
            sFY[e] = acc;
        }
        __syncthreads();
        const int nb = (oh + NR - 1) / NR;
        for (int e = tid; e < nb * ow; e += NTH) {
            const int rb = e / ow, yc = e - rb * ow, xr0 = rb * NR;
            const float2* fxc = sFX + xr0 * ow + yc;  // half-rows x - 5 .. of output row x = ox0 + xr0
            float2 w[NR + 9];
#pragma unroll
            for (int i = 0; i < NR + 9; i++) w[i] = fxc[i * ow];
#pragma unroll
            for (int r = 0; r < NR; r++) {
                const int xr = xr0 + r;
                if (xr >= oh) break;
                const float2* fy = sFY + xr * (ow + 9) + yc + 5;  // flux at half-column y
                float2 gx = mul2(a.wx[0], sub2(w[r + 5], w[r + 4]));
                float2 gy = mul2(a.wy[0], sub2(fy[0], fy[-1]));
#pragma unroll
                for (int m = 1; m < 5; m++) {
                    gx = fma2(a.wx[m], sub2(w[r + 5 + m], w[r + 4 - m]), gx);
                    gy = fma2(a.wy[m], sub2(fy[m], fy[-1 - m]), gy);
                }
                epi(ox0 + xr, oy0 + yc, add2(gx, gy));
            }
        }
        __syncthreads();  // the flux rows are reused
    } else {
        const int nb = (oh + NR - 1) / NR;
        for (int e = tid; e < nb * ow; e += NTH) {
            const int rb = e / ow, yc = e - rb * ow, xs = ox0 + rb * NR, y = oy0 + yc;
            const float2* col = in + (xs - ix0) * iw + (y - iy0);  // (xs, y)
            float2 w[NR + 10];
#pragma unroll
            for (int i = 0; i < NR + 10; i++) w[i] = col[(i - 5) * iw];
#pragma unroll
            for (int r = 0; r < NR; r++) {
                if (xs + r >= ox1) break;
                const float2* row = col + r * iw;
                float2 gx = mul2(a.wx[0], w[r + 5]);
                float2 gy = mul2(a.wy[0], w[r + 5]);
#pragma unroll
                for (int k = 1; k <= 5; k++) {
                    gx = fma2(a.wx[k], add2(w[r + 5 + k], w[r + 5 - k]), gx);
                    gy = fma2(a.wy[k], add2(row[k], row[-k]), gy);
                }
                epi(xs + r, y, add2(gx, gy));
            }
        }
    }
}

template <int KIND, bool OT4>
struct PersistCfg {
    static constexpr int R = KIND != 0 ? 9 : 5;
    static constexpr int HU = OT4 ? 2 * R : R;  // p[t] halo
    static constexpr int HL = OT4 ? R : 0;      // stage-1 region beyond the tile
    // shared memory: float4 coefficients of the tile's points {C1, C2, -C3, W k12 (OT4) or W};
    // float2 arrays of p[t] over the tile and halo, l (OT4), the flux rows of the larger stage
    // (staggered), p[t-1] and p[t+1] over the tile; float tables of the medium: W over the
    // stage-1 region, bx and by over the stage-1 flux regions;
    // int arrays: the source slots of the tile's points and the CTA's halo points; the float values
    // of the CTA's sources at the step
    static constexpr int PADR = PERSIST_NR_MAX - 1;  // rows of padding of the arrays stencil_region reads
    __host__ __device__ static constexpr size_t nU(int tx, int ty) {
        return (size_t)(tx + 2 * HU + PADR) * (ty + 2 * HU);
    }
    __host__ __device__ static constexpr size_t nL(int tx, int ty) {
        return OT4 ? (size_t)(tx + 2 * HL + PADR) * (ty + 2 * HL) : 0;
    }
    __host__ __device__ static constexpr size_t nF(int tx, int ty) {
        return KIND != 0 ? (size_t)(tx + 2 * HL + 9 + PADR) * (ty + 2 * HL) : 0;
    }
    __host__ __device__ static constexpr size_t nG(int tx, int ty) {
        return KIND != 0 ? (size_t)(tx + 2 * HL) * (ty + 2 * HL + 9) : 0;
    }
    __host__ __device__ static constexpr size_t nT(int tx, int ty) { return (size_t)tx * ty; }
    __host__ __device__ static constexpr size_t nW(int tx, int ty) { return (size_t)(tx + 2 * HL) * (ty + 2 * HL); }
    __host__ __device__ static constexpr size_t floats2(int tx, int ty) {
        return nU(tx, ty) + nL(tx, ty) + nF(tx, ty) + nG(tx, ty) + 2 * nT(tx, ty);
    }
    // halo points of a tile (at most; fewer beyond the grid)
    __host__ __device__ static constexpr size_t nH(int tx, int ty) {
        return (size_t)2 * HU * (tx + ty) + (size_t)4 * HU * HU;
    }
    __host__ __device__ static constexpr size_t floats1(int tx, int ty) {
        return nW(tx, ty) + (KIND == 1 ? nF(tx, ty) + nG(tx, ty) : 0) + nT(tx, ty) + nH(tx, ty) + PERSIST_SRC_SLOTS;
    }
    __host__ __device__ static constexpr size_t bytes(int tx, int ty) {
        return nT(tx, ty) * sizeof(float4) + floats2(tx, ty) * sizeof(float2) + floats1(tx, ty) * sizeof(float);
    }
};

template <int KIND, bool OT4>
__global__ void __launch_bounds__(PERSIST_THREADS) fdtd2d_persist(const __grid_constant__ Persist2D P) {
    using CF = PersistCfg<KIND, OT4>;
    constexpr bool VARB = KIND == 1;
    constexpr int HU = CF::HU, HL = CF::HL;
    const Step2D& a = P.s;
    const int tx = P.tx, ty = P.ty;
    extern __shared__ __align__(16) float4 psm[];
    float4* const sC = psm;                                     // coefficients of the tile's points
    float2* const sU = reinterpret_cast<float2*>(sC + CF::nT(tx, ty));  // p[t], tile and halo
    float2* const sL = sU + CF::nU(tx, ty);  // l (OT4)
    float2* const sFX = sL + CF::nL(tx, ty);
    float2* const sFY = sFX + CF::nF(tx, ty);
    float2* const sPm = sFY + CF::nG(tx, ty);  // p[t-1] over the tile
    float2* const sN = sPm + CF::nT(tx, ty);   // p[t+1] over the tile (OT2, or a CTA with more sources than slots)
    float* const sW = reinterpret_cast<float*>(sN + CF::nT(tx, ty));
    float* const sBX = sW + CF::nW(tx, ty);
    float* const sBY = sBX + (VARB ? CF::nF(tx, ty) : 0);
    int* const sMap = reinterpret_cast<int*>(sBY + (VARB ? CF::nG(tx, ty) : 0));  // source slots + 1, lane 0 | lane 1 << 16
    int* const sHal = sMap + CF::nT(tx, ty);  // halo points: row | column << 8 relative to (ux0, uy0)
    float* const sSrc = reinterpret_cast<float*>(sHal + CF::nH(tx, ty));  // this step's source values

    const int tid = threadIdx.x, NTH = blockDim.x, b = blockIdx.x;
    const int ntile = P.tiles_x * P.tiles_y;
    const int pair = b / ntile, tile = b % ntile;
    const int x0 = (tile / P.tiles_y) * tx, y0 = (tile % P.tiles_y) * ty;
    const int x1 = min(x0 + tx, a.nx), y1 = min(y0 + ty, a.ny);
    const int th = x1 - x0, tw = y1 - y0;
    const int uw = ty + 2 * HU, lw = ty + 2 * HL;
    const int mp = a.mpitch, pitch = a.pitch;
    const int ux0 = x0 - HU, uy0 = y0 - HU, uh = th + 2 * HU, uwr = tw + 2 * HU;
    const int lx0 = x0 - HL, ly0 = y0 - HL, lh = th + 2 * HL, lwr = tw + 2 * HL;
    const bool inner = lx0 >= 0 && lx0 + lh <= a.nx && ly0 >= 0 && ly0 + lwr <= a.ny;  // stage-1 region in the grid
    const int sb = P.cta_off[b], ns = P.cta_off[b + 1] - sb;  // this CTA's source targets
    const int rb = P.rec_off[b], nr = P.rec_off[b + 1] - rb;  // and receivers
    const bool slots = ns <= PERSIST_SRC_SLOTS;  // sources added in the update (else through sN)
    const long long pair_floats = (long long)pair * a.shot_stride * 2;

    // ---- once: the medium of the CTA's region, p[1] = p[0] = 0, the halo points, the sources ----
    for (int e = tid; e < lh * lwr; e += NTH) {
        const int x = lx0 + e / lwr, y = ly0 + e % lwr;
        sW[(x - lx0) * lw + (y - ly0)] = __ldg(a.Wm + (long long)x * mp + y);
    }
    for (int e = tid; e < th * tw; e += NTH) {
        const int x = x0 + e / tw, y = y0 + e % tw;
        const long long q = (long long)x * mp + y;
        const int k = (x - x0) * ty + (y - y0);
        const float W = __ldg(a.Wm + q);
        sC[k] = make_float4(__ldg(a.C1m + q), __ldg(a.C2m + q), __ldg(a.NC3m + q), OT4 ? W * a.k12 : W);
        sPm[k] = f2(0.f);
        sMap[k] = 0;
    }
    BTables B{sBX, sBY, lx0 - 5, ly0, lw, lx0, ly0 - 5, lw + 9};
    if constexpr (VARB) {
        for (int e = tid; e < (lh + 9) * lwr; e += NTH) {
            const int h = lx0 - 5 + e / lwr, y = ly0 + e % lwr;
            sBX[(h - B.fx0) * B.fw + (y - B.fy0)] = __ldg(a.bxm + (long long)h * mp + y);
        }
        for (int e = tid; e < lh * (lwr + 9); e += NTH) {
            const int x = lx0 + e / (lwr + 9), hc = ly0 - 5 + e % (lwr + 9);
            sBY[(x - B.gx0) * B.gw + (hc - B.gy0)] = __ldg(a.bym + (long long)x * mp + hc);
        }
    }
    for (int e = tid; e < uh * uwr; e += NTH) sU[(e / uwr) * uw + e % uwr] = f2(0.f);
    __shared__ int nhal_s;
    if (tid < 32) {  // the in-grid points of the halo in row-major order (warp 0, by ballot)
        int cnt = 0;
        for (int e0 = 0; e0 < uh * uwr; e0 += 32) {
            const int e = e0 + tid, xr = e / uwr, yr = e % uwr, x = ux0 + xr, y = uy0 + yr;
            const bool tile = x >= x0 && x < x1 && y >= y0 && y < y1;
            const bool v = e < uh * uwr && !tile && x >= 0 && x < a.nx && y >= 0 && y < a.ny;
            const unsigned m = __ballot_sync(0xffffffffu, v);
            if (v) sHal[cnt + __popc(m & ((1u << tid) - 1u))] = xr | yr << 8;
            cnt += __popc(m);
        }
        if (tid == 0) nhal_s = cnt;
    }
    if (slots)
        for (int j = tid; j < ns; j += NTH) {  // the slot of each target at its point and lane
            const long long i = P.tidx[P.cta_tgt[sb + j]] - pair_floats, c2 = i / 2;
            const int x = (int)(c2 / pitch), y = (int)(c2 % pitch);
            atomicOr(sMap + (x - x0) * ty + (y - y0), (j + 1) << (16 * (int)(i & 1)));
        }
    // each target's value at every step, srcv[(sb + j) nt + t], summed in the targets' entry order
    for (int e = tid; e < ns * P.nt; e += NTH) {
        const int j = e / P.nt, t = e % P.nt, tg = P.cta_tgt[sb + j];
        const float* amp = P.src_amp + (long long)t * P.n_src;
        float v = 0.f;
        for (int k = P.toff[tg]; k < P.toff[tg + 1]; k++) v += P.tcoef[k] * amp[P.tpoint[k]];
        P.srcv[(long long)(sb + j) * P.nt + t] = v;
    }
    // this thread's receiver, kept in registers (a CTA with more receivers than threads reads the rest)
    Gather G{};
    if (tid < nr) G = P.gat[P.rec_idx[rb + tid]];
    __syncthreads();
    const int nhal = nhal_s;

    // p[level] beyond the tile, from the neighbour tiles' exchange lines: a thread loads its lines in
    // batches of PERSIST_BATCH and reloads the ones that do not hold the level yet, all together,
    // until they do (a bounded wait)
    auto load_halo = [&](int level) -> bool {
        const uint4* src = P.xch + (level & 1) * P.xch_slot + (long long)pair * a.shot_stride;
        const unsigned want = (unsigned)(level + P.extra);
        const volatile int* verr = P.err;
        bool ok = true;
        for (int e0 = tid; e0 < nhal && ok; e0 += PERSIST_BATCH * NTH) {
            uint4 v[PERSIST_BATCH];
            int at[PERSIST_BATCH], gi[PERSIST_BATCH];
            unsigned pending = 0;
#pragma unroll
            for (int k = 0; k < PERSIST_BATCH; k++) {
                const int e = e0 + k * NTH;
                const int hp = e < nhal ? sHal[e] : 0, xr = hp & 255, yr = hp >> 8;
                at[k] = xr * uw + yr;
                gi[k] = (ux0 + xr) * pitch + uy0 + yr;
                if (e < nhal) {
                    v[k] = ld_line(src + gi[k]);
                    pending |= 1u << k;
                }
            }
            for (long long n = 0;; n++) {
#pragma unroll
                for (int k = 0; k < PERSIST_BATCH; k++)
                    if ((pending >> k & 1) && v[k].y == want && v[k].w == want) {
                        sU[at[k]] = make_float2(__uint_as_float(v[k].x), __uint_as_float(v[k].z));
                        pending &= ~(1u << k);
                    }
                if (!pending) break;
                if (n >= P.spin_limit || *verr) {
                    atomicExch(P.err, 1);
                    ok = false;
                    break;
                }
                PERSIST_POLL_PAUSE;
#pragma unroll
                for (int k = 0; k < PERSIST_BATCH; k++)
                    if (pending >> k & 1) v[k] = ld_line(src + gi[k]);
            }
        }
        return __syncthreads_and(ok) != 0;
    };

    // the receivers whose base corner this CTA holds, from p[level] in sU
    auto gather_one = [&](const Gather& R, int trow) {
        const float2* f0 = sU + (R.row - ux0) * uw + (R.col - uy0);
        const float2* f1 = f0 + uw;
        const float v00 = (R.pad & 1) ? f0[0].y : f0[0].x, v01 = (R.pad & 1) ? f0[1].y : f0[1].x;
        const float v10 = (R.pad & 1) ? f1[0].y : f1[0].x, v11 = (R.pad & 1) ? f1[1].y : f1[1].x;
        P.rec_amp[(long long)trow * P.n_rec + R.point] = R.w00 * v00 + R.w01 * v01 + R.w10 * v10 + R.w11 * v11;
    };
    auto gather = [&](int trow) {
        if (tid < nr) gather_one(G, trow);
        for (int j = tid + NTH; j < nr; j += NTH) gather_one(P.gat[P.rec_idx[rb + j]], trow);
    };

    for (int t = 1; t <= P.nt - 2; t++) {
        uint4* out = P.xch + ((t + 1) & 1) * P.xch_slot + (long long)pair * a.shot_stride;  // p[t+1]
        const float sv = slots && tid < ns ? __ldcg(P.srcv + (long long)(sb + tid) * P.nt + t) : 0.f;
        // 1. p[t]: the halo (the tile's own points are in sU since last step)
        if (t > 1) {
            if (!load_halo(t)) return;
            gather(t - 1);  // rec[t-1] = interp(p[t])
        }
        if (slots) {
            if (tid < ns) sSrc[tid] = sv;
            for (int j = tid + NTH; j < ns; j += NTH) sSrc[j] = __ldcg(P.srcv + (long long)(sb + j) * P.nt + t);
        }
        // 2-3. the update of the tile: p[t+1] = C1 Lt + C2 p[t] - C3 p[t-1], plus the step's sources
        auto update = [&](int k, const float4& c, int x, int y, float2 Lt) -> float2 {
            const float2 u = sU[(x - ux0) * uw + (y - uy0)];
            return fma2(f2(c.x), Lt, fma2(f2(c.y), u, mul2(f2(c.z), sPm[k])));
        };
        // p[t+1] at (x, y) out: to the exchange line, p[t] to p[t-1], p[t+1] into the tile of sU
        auto emit = [&](int x, int y, float2 v) {
            const int k = (x - x0) * ty + (y - y0);
            if (ns) {
                const int m = sMap[k];
                if (m & 0xffff) v.x = v.x + sSrc[(m & 0xffff) - 1];
                if (m >> 16) v.y = v.y + sSrc[(m >> 16) - 1];
            }
            float2* u = sU + (x - ux0) * uw + (y - uy0);
            sPm[k] = *u;
            *u = v;
            st_line(out + (long long)x * pitch + y, v, (unsigned)(t + 1));
        };
        // OT4 with the sources in slots emits each point as it is updated (stage 2 reads only l);
        // otherwise the new level waits in sN for the sources and the stencil's last reads of p[t]
        const bool direct = OT4 && slots;
        if constexpr (OT4) {
            stencil_region<KIND, PERSIST_NR1>(a, sU, ux0, uy0, uw, lx0, x1 + HL, ly0, y1 + HL, sFX, sFY, B,
                                    [&](int x, int y, float2 g) {
                                        const bool in = inner || (x >= 0 && x < a.nx && y >= 0 && y < a.ny);
                                        const float W = sW[(x - lx0) * lw + (y - ly0)];
                                        sL[(x - lx0) * lw + (y - ly0)] = in ? mul2(f2(W), g) : f2(0.f);
                                    });
            __syncthreads();
            stencil_region<KIND, PERSIST_NR2>(a, sL, lx0, ly0, lw, x0, x1, y0, y1, sFX, sFY, B, [&](int x, int y, float2 g) {
                const int k = (x - x0) * ty + (y - y0);
                const float4 c = sC[k];
                const float2 v = update(k, c, x, y, fma2(f2(c.w), g, sL[(x - lx0) * lw + (y - ly0)]));
                if (direct)
                    emit(x, y, v);
                else
                    sN[(x - x0) * ty + (y - y0)] = v;
            });
        } else {
            stencil_region<KIND, 2>(a, sU, ux0, uy0, uw, x0, x1, y0, y1, sFX, sFY, B, [&](int x, int y, float2 g) {
                const int k = (x - x0) * ty + (y - y0);
                const float4 c = sC[k];
                sN[k] = update(k, c, x, y, mul2(f2(c.w), g));
            });
        }
        if (!direct) {
            __syncthreads();
            if (!slots) {  // 4. sources beyond the slots, straight into sN
                for (int j = tid; j < ns; j += NTH) {
                    const long long i = P.tidx[P.cta_tgt[sb + j]] - pair_floats, c2 = i / 2;
                    const int x = (int)(c2 / pitch), y = (int)(c2 % pitch);
                    float* q = reinterpret_cast<float*>(sN + (x - x0) * ty + (y - y0)) + (i & 1);
                    *q = *q + __ldcg(P.srcv + (long long)(sb + j) * P.nt + t);
                }
                __syncthreads();
            }
            // 5. p[t+1] out (the slots are empty here when there are none)
            for (int e = tid; e < th * tw; e += NTH) {
                const int x = x0 + e / tw, y = y0 + e % tw;
                emit(x, y, sN[(x - x0) * ty + (y - y0)]);
            }
        }
    }
    // the last step's receivers, rec[nt-2] = interp(p[nt-1]), with the halo of p[nt-1]
    if (P.nt < 3) return;
    if (!load_halo(P.nt - 1)) return;
    gather(P.nt - 2);
}

// Largest dynamic shared memory of a CTA of the kernel: the device's opt-in limit less the
// kernel's static shared memory. Configures the kernel for it once.
template <int KIND, bool OT4>
int dyn_limit() {
    static int limit = -1;
    if (limit < 0) {
        int dev = 0, optin = 0;
        cudaFuncAttributes fa{};
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
            cudaFuncGetAttributes(&fa, fdtd2d_persist<KIND, OT4>) != cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        const int l = optin - (int)fa.sharedSizeBytes;
        if (cudaFuncSetAttribute(fdtd2d_persist<KIND, OT4>, cudaFuncAttributeMaxDynamicSharedMemorySize, l) !=
            cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        limit = l;
    }
    return limit;
}

template <int KIND, bool OT4>
cudaError_t launch_one(int nblocks, size_t smem, cudaStream_t s, const Persist2D& a) {
    if ((int)smem > dyn_limit<KIND, OT4>()) return cudaErrorInvalidValue;
    void* args[] = {const_cast<Persist2D*>(&a)};
    return cudaLaunchCooperativeKernel((const void*)fdtd2d_persist<KIND, OT4>, dim3(nblocks), dim3(PERSIST_THREADS),
                                       args, smem, s);
}

template <int KIND, bool OT4>
int blocks_one(size_t smem) {
    if ((int)smem > dyn_limit<KIND, OT4>()) return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fdtd2d_persist<KIND, OT4>, PERSIST_THREADS, smem) !=
        cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

}  // namespace

size_t persist2d_smem(int kind, bool ot4, int tx, int ty) {
    switch (kind) {
        case 0: return ot4 ? PersistCfg<0, true>::bytes(tx, ty) : PersistCfg<0, false>::bytes(tx, ty);
        case 1: return ot4 ? PersistCfg<1, true>::bytes(tx, ty) : PersistCfg<1, false>::bytes(tx, ty);
        default: return ot4 ? PersistCfg<2, true>::bytes(tx, ty) : PersistCfg<2, false>::bytes(tx, ty);
    }
}

int persist2d_blocks_per_sm(int kind, bool ot4, size_t smem) {
    switch (kind) {
        case 0: return ot4 ? blocks_one<0, true>(smem) : blocks_one<0, false>(smem);
        case 1: return ot4 ? blocks_one<1, true>(smem) : blocks_one<1, false>(smem);
        default: return ot4 ? blocks_one<2, true>(smem) : blocks_one<2, false>(smem);
    }
}

cudaError_t launch_persist2d(int kind, bool ot4, int nblocks, size_t smem, cudaStream_t s, const Persist2D& a) {
    switch (kind) {
        case 0: return ot4 ? launch_one<0, true>(nblocks, smem, s, a) : launch_one<0, false>(nblocks, smem, s, a);
        case 1: return ot4 ? launch_one<1, true>(nblocks, smem, s, a) : launch_one<1, false>(nblocks, smem, s, a);
        default: return ot4 ? launch_one<2, true>(nblocks, smem, s, a) : launch_one<2, false>(nblocks, smem, s, a);
    }
}

}  // namespace sa

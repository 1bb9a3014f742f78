// BF16 GEMM on the 5th-generation tensor cores (tcgen05, accumulator in tensor memory) for the
// learned preconditioner's convolutions:  C[M][N] (+)= A[M][K] * B[N][K]^T  (+ bias[N], ReLU),
// A and B bf16 with K contiguous, C fp32 (optionally also written as bf16).
//
// One CTA of 128 threads computes a 128 x BN tile. K advances in 64-wide chunks staged in shared
// memory (3-4 stages, 16-byte cp.async) in the no-swizzle K-major canonical layout: 8-row x
// 16-byte core matrices, the core matrices of one 8-wide k group stacked along M (stride 128 B),
// k groups one after another (stride rows * 16 B). Thread 0 issues four kind::f16 MMAs (K = 16
// each) per chunk into a TMEM accumulator of BN fp32 columns and commits them to the stage's
// mbarrier, which releases the stage for the next load. The epilogue reads the accumulator with
// tcgen05.ld (warp w owns TMEM lanes / tile rows 32w .. 32w+31).
//
// Every mbarrier wait is bounded: on timeout the kernel records it in *err, skips the remaining
// MMAs and still waits (bounded) for the ones in flight before freeing its TMEM.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/strideacc.h"
#include "helpers.h"

namespace {

constexpr int kBM = 128;
constexpr int kBK = 64;  // k columns per staged chunk
constexpr long long kSpinLimit = 20000000;  // try_wait polls before giving up (far beyond any MMA chunk)

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async16z(uint32_t dst, const void* src, bool valid) {  // zero-fill if !valid
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(valid ? 16 : 0)
                 : "memory");
}

// Implicit-GEMM A operand of a 3x3 convolution (padding 1): row m of A is pixel m of B images of
// H x W, column k = (ky 3 + kx) Cin + ci the input channel ci of its (ky - 1, kx - 1) neighbour,
// read from the bf16 NHWC activations (row stride ldx) and zero outside the image or for
// k >= 9 Cin. Cin is a multiple of 8, so a 16-byte group of 8 columns never straddles two taps.
struct ConvA {
    int H, W, Cin, ldx;  // Cin 0: A is a plain matrix (lda)
};

// tcgen05 shared-memory matrix descriptor: start >> 4 (bits 0-13), leading byte offset >> 4
// (16-29), stride byte offset >> 4 (32-45), fixed 0b001 (46-48), no swizzle (61-63 = 0).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

// kind::f16 instruction descriptor: D f32 (bits 4-5 = 1), A and B bf16 (7-9 = 1, 10-12 = 1),
// both K-major (15, 16 = 0), N >> 3 (17-22), M >> 4 (24-28).
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (long long i = 0; i < kSpinLimit; i++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

template <int BN, int NS>
__global__ void __launch_bounds__(128) k_umma_gemm(const __nv_bfloat16* __restrict__ A, int lda,
                                                   const __nv_bfloat16* __restrict__ B, int ldb, float* C, int ldc,
                                                   __nv_bfloat16* Cb, int ldcb, int K, const float* __restrict__ bias,
                                                   int relu, int accumulate, int chunks_per_split, long long slab,
                                                   const ConvA conv, int* err) {
    constexpr int A_BYTES = kBM * kBK * 2;  // 16 KB
    constexpr int B_BYTES = BN * kBK * 2;
    constexpr int STAGE = A_BYTES + B_BYTES;
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t bars[NS];  // one per stage: its MMAs have finished reading it
    __shared__ uint32_t tmem_base_sh;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * BN;
    const uint32_t sbase = smem_u32(smem);
    auto bar = [&](int st) { return smem_u32(&bars[st]); };

    if (tid == 0) {
        for (int st = 0; st < NS; st++) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar(st)));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_base_sh)),
                     "r"(BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = tmem_base_sh;

    // implicit GEMM: the (y, x) of this thread's A rows (tid >> 3) + 16 i, packed y << 16 | x
    int rowyx[8];
    if (conv.Cin) {
        const int HW = conv.H * conv.W;
#pragma unroll
        for (int i = 0; i < 8; i++) {
            const int p = m0 + (tid >> 3) + 16 * i, q = p % HW, y = q / conv.W;
            rowyx[i] = y << 16 | (q - y * conv.W);
        }
    }
    // stage loader: A rows m (128) and B rows n (BN), k group g (8 per chunk), 16 bytes each
    // (the last chunk may be shorter: K is a multiple of 16, a chunk holds K - k0 <= 64 columns)
    auto load = [&](int kb, int stage) {
        const uint32_t sa = sbase + stage * STAGE, sb = sa + A_BYTES;
        const int k0 = kb * kBK;
        const int ng = min(kBK, K - k0) >> 3;  // k groups of 8 in this chunk
        if (conv.Cin == 0) {
            for (int c = tid; c < kBM * 8; c += 128) {
                const int m = c >> 3, g = c & 7;
                if (g < ng)
                    cp_async16(sa + g * (kBM * 16) + (m >> 3) * 128 + (m & 7) * 16,
                               A + (long long)(m0 + m) * lda + k0 + g * 8);
            }
        } else {
            // this thread's group g = tid & 7 of every chunk, rows (tid >> 3) + 16 i: the tap and channel of
            // its columns once per chunk, the rows' pixels precomputed
            const int g = tid & 7;
            const int k = k0 + g * 8, tap = k / conv.Cin, ci = k - tap * conv.Cin;
            const int dy = tap / 3 - 1, dx = tap % 3 - 1;
            const bool col_ok = g < ng && tap < 9;
            const long long toff = (long long)(dy * conv.W + dx) * conv.ldx + ci;
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const int m = (tid >> 3) + 16 * i;
                const int yy = (rowyx[i] >> 16) + dy, xx = (rowyx[i] & 0xffff) + dx;
                const bool ok = col_ok && yy >= 0 && yy < conv.H && xx >= 0 && xx < conv.W;
                const __nv_bfloat16* src = ok ? A + (long long)(m0 + m) * conv.ldx + toff : A;
                cp_async16z(sa + g * (kBM * 16) + (m >> 3) * 128 + (m & 7) * 16, src, ok);
            }
        }
        for (int c = tid; c < BN * 8; c += 128) {
            const int n = c >> 3, g = c & 7;
            if (g < ng)
                cp_async16(sb + g * (BN * 16) + (n >> 3) * 128 + (n & 7) * 16,
                           B + (long long)(n0 + n) * ldb + k0 + g * 8);
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    };

    // split K (gridDim.z > 1): this CTA takes chunks [kb0, kb1) and adds its partial tile to C, or
    // (slab > 0) stores it to its own slab C + z slab, for a reduction in a fixed order
    const int nk_all = (K + kBK - 1) / kBK;
    const int kb0 = blockIdx.z * chunks_per_split, kb1 = min(nk_all, kb0 + chunks_per_split);
    const int nk = max(0, kb1 - kb0);
    const bool split = gridDim.z > 1;
    constexpr uint32_t idesc = idesc_bf16(kBM, BN);
    bool ok = true;
    int issued = 0;  // MMA chunks committed (thread 0); chunk i commits to bar(i % NS)
    // prologue: chunks 0 .. NS-2 in flight (one commit group each, empty past the end)
    for (int i = 0; i < NS - 1; i++) {
        if (i < nk) load(kb0 + i, i);
        else asm volatile("cp.async.commit_group;\n" ::: "memory");
    }
    for (int i = 0; i < nk && ok; i++) {
        const int kb = kb0 + i;
        const int st = i % NS;
        // refill the stage chunk i-1 used with chunk i+NS-1, once chunk i-1's MMAs are done
        if (i + NS - 1 < nk) {
            const int s1 = (i + NS - 1) % NS;
            if (i >= 1 && !mbar_wait(bar(s1), (uint32_t)(((i - 1) / NS) & 1))) ok = false;
            if (ok) load(kb + NS - 1, s1);
            else asm volatile("cp.async.commit_group;\n" ::: "memory");
        } else {
            asm volatile("cp.async.commit_group;\n" ::: "memory");
        }
        asm volatile("cp.async.wait_group %0;\n" ::"n"(NS - 1) : "memory");  // chunk i has landed
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncthreads();
        ok = __syncthreads_and(ok ? 1 : 0) != 0;
        if (!ok) break;
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t sa = sbase + st * STAGE, sb = sa + A_BYTES;
            const int nmma = min(kBK, K - kb * kBK) >> 4;
#pragma unroll
            for (int j = 0; j < kBK / 16; j++) {  // two k groups per MMA
                if (j >= nmma) break;
                const uint64_t ad = smem_desc(sa + 2 * j * (kBM * 16), kBM * 16, 128);
                const uint64_t bd = smem_desc(sb + 2 * j * (BN * 16), BN * 16, 128);
                const uint32_t acc = (i > 0 || j > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             bar(st))
                         : "memory");
            issued++;
        }
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    // wait for every committed MMA: the last commit of each stage's barrier, bounded (a commit
    // tracks all earlier tcgen05 operations of the thread, so the last chunk's suffices)
    bool done = true;
    if (tid == 0 && issued > 0) {
        const int last = issued - 1;
        if (!mbar_wait(bar(last % NS), (uint32_t)((last / NS) & 1))) done = false;
    }
    ok = __syncthreads_and((ok && (tid != 0 || done)) ? 1 : 0) != 0;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (ok && nk > 0) {
        // epilogue: warp w reads lanes 32w..32w+31 (tile rows), 16 columns per load
        const int m = m0 + warp * 32 + lane;
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 16) {
            uint32_t r[16];
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                "[%16];\n"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            float* crow = C + (long long)m * ldc + n0 + c0;
            if (split) {
                if (slab) {
                    float* srow = crow + blockIdx.z * slab;
#pragma unroll
                    for (int q = 0; q < 16; q++) srow[q] = __uint_as_float(r[q]);
                } else {
#pragma unroll
                    for (int q = 0; q < 16; q++) atomicAdd(crow + q, __uint_as_float(r[q]));
                }
                continue;
            }
#pragma unroll
            for (int q = 0; q < 16; q++) {
                float v = __uint_as_float(r[q]);
                if (accumulate) v += crow[q];
                if (bias) v += bias[n0 + c0 + q];
                if (relu) v = fmaxf(v, 0.f);
                crow[q] = v;
                if (Cb) Cb[(long long)m * ldcb + n0 + c0 + q] = __float2bfloat16_rn(v);
            }
        }
    } else if (!ok && tid == 0) {
        atomicExch(err, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(BN));
}

template <int BN>
cudaError_t launch(const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, float* C, int ldc,
                   __nv_bfloat16* Cb, int ldcb, int M, int N, int K, const float* bias, int relu, int accumulate,
                   int ksplit, int* err, cudaStream_t s, ConvA conv = ConvA{0, 0, 0, 0}) {
    constexpr int NS = BN >= 128 ? 3 : 4;  // stages: 96 KB (BN 128) or <= 96 KB (BN <= 64) of shared memory
    const size_t bytes = NS * (size_t)(kBM * kBK * 2 + BN * kBK * 2);
    static bool configured = false;
    if (!configured) {
        cudaError_t e =
            cudaFuncSetAttribute(k_umma_gemm<BN, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    const int nk = (K + kBK - 1) / kBK;
    const int per = (nk + ksplit - 1) / ksplit;
    const dim3 grid(M / kBM, N / BN, (nk + per - 1) / per);
    const long long slab = accumulate == 2 && grid.z > 1 ? (long long)M * ldc : 0;
    k_umma_gemm<BN, NS><<<grid, 128, bytes, s>>>(A, lda, B, ldb, C, ldc, Cb, ldcb, K, bias, relu, accumulate, per,
                                                 slab, conv, err);
    return cudaGetLastError();
}

}  // namespace

extern "C" int sa_gemm_bf16(const void* A, int lda, const void* B, int ldb, float* C, int ldc, void* Cb, int ldcb,
                            int M, int N, int K, const float* bias, int relu, int accumulate, int ksplit, int* err,
                            void* stream) {
    if (ksplit < 1 || (ksplit > 1 && (bias || relu || Cb || !accumulate)) || accumulate < 0 || accumulate > 2 ||
        (accumulate == 2 && ksplit < 2))
        return (sa::set_last_error("sa_gemm_bf16: split K adds plain partial products into C (accumulate 1) or "
                                   "stores them to slabs (accumulate 2)"),
                SA_E_INVALID);
    if (!A || !B || !C || !err || M <= 0 || N <= 0 || K <= 0 || M % kBM || K % 16 || (N % 32))
        return (sa::set_last_error("sa_gemm_bf16: M must be a multiple of 128, K of 16, N of 32"), SA_E_INVALID);
    if (lda % 8 || ldb % 8 || lda < K || ldb < K || ldc < N || (Cb && ldcb < N) ||
        ((uintptr_t)A & 15) || ((uintptr_t)B & 15))
        return (sa::set_last_error("sa_gemm_bf16: leading dimensions and bases must allow 16-byte rows"),
                SA_E_INVALID);
    const auto* a = static_cast<const __nv_bfloat16*>(A);
    const auto* b = static_cast<const __nv_bfloat16*>(B);
    auto* cb = static_cast<__nv_bfloat16*>(Cb);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e;
    if (N % 128 == 0)
        e = launch<128>(a, lda, b, ldb, C, ldc, cb, ldcb, M, N, K, bias, relu, accumulate, ksplit, err, s);
    else if (N % 64 == 0)
        e = launch<64>(a, lda, b, ldb, C, ldc, cb, ldcb, M, N, K, bias, relu, accumulate, ksplit, err, s);
    else
        e = launch<32>(a, lda, b, ldb, C, ldc, cb, ldcb, M, N, K, bias, relu, accumulate, ksplit, err, s);
    if (e != cudaSuccess) return (sa::set_last_error(cudaGetErrorString(e)), SA_E_CUDA);
    return SA_OK;
}

extern "C" int sa_conv3x3_bf16(const void* x, int ldx, int B, int H, int W, int Cin, const void* Wt, int ldw, float* C,
                               int ldc, void* Cb, int ldcb, int N, int Kp, const float* bias, int relu, int* err,
                               void* stream) {
    const long long P = (long long)B * H * W;
    if (!x || !Wt || !C || !err || B < 1 || H < 1 || W < 1 || H > 32767 || W > 65535 || Cin < 8 || Cin % 8 ||
        P % kBM || P > INT32_MAX ||
        Kp < 9 * Cin || Kp % 16 || N % 32 || ldx < Cin || ldx % 8 || ldw < Kp || ldw % 8 || ldc < N ||
        (Cb && ldcb < N) || ((uintptr_t)x & 15) || ((uintptr_t)Wt & 15))
        return (sa::set_last_error("sa_conv3x3_bf16: pixels a multiple of 128, H <= 32767 and W <= 65535, Cin and "
                                   "ldx multiples of 8, Kp >= 9 Cin a multiple of 16, N of 32, 16-byte aligned operands"),
                SA_E_INVALID);
    const auto* a = static_cast<const __nv_bfloat16*>(x);
    const auto* b = static_cast<const __nv_bfloat16*>(Wt);
    auto* cb = static_cast<__nv_bfloat16*>(Cb);
    const ConvA conv{H, W, Cin, ldx};
    cudaStream_t s = (cudaStream_t)stream;
    const int M = (int)P;
    cudaError_t e;
    if (N % 128 == 0)
        e = launch<128>(a, 0, b, ldw, C, ldc, cb, ldcb, M, N, Kp, bias, relu, 0, 1, err, s, conv);
    else if (N % 64 == 0)
        e = launch<64>(a, 0, b, ldw, C, ldc, cb, ldcb, M, N, Kp, bias, relu, 0, 1, err, s, conv);
    else
        e = launch<32>(a, 0, b, ldw, C, ldc, cb, ldcb, M, N, Kp, bias, relu, 0, 1, err, s, conv);
    if (e != cudaSuccess) return (sa::set_last_error(cudaGetErrorString(e)), SA_E_CUDA);
    return SA_OK;
}

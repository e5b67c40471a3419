// tb_mlp_tc.cu -- inference of the charge MLP on the 5th-generation tensor
// cores (tcgen05).  No counterpart in the reference (its SCC loop starts from
// the neutral charges, withSP2_deltaH.cpp:1725-1740).
//
// One CTA of 128 threads takes 128 atoms.  The two dense layers are
// D[128 x 64] = A[128 x K] . B[K x 64] with K = 32 and 64: A (the normalised
// features, then the layer-1 activations) and B (the weights, stored [out][in]
// = K-major) sit in shared memory as BF16 in the canonical no-swizzle K-major
// layout -- core matrices of 8 rows x 16 bytes, 128 bytes apart along K (LBO)
// and (K/8) x 128 bytes apart along M/N (SBO).  Thread 0 issues
// tcgen05.mma.cta_group::1.kind::f16 (K = 16 per instruction) with FP32
// accumulators in tensor memory (128 lanes x 64 columns per layer, one
// allocation of 128 columns), commits to an mbarrier, and every warp reads its
// 32 lanes (= its 32 atoms) back with tcgen05.ld for bias + SiLU in registers.
// The 64 -> 1 output layer runs on the CUDA cores in FP32.
//
// Numerics: BF16 weights (the network's own parameters), BF16 inputs to each
// layer, FP32 accumulation and activations -- the same as the CUDA-core path
// except that the layer inputs are rounded to BF16 as well.
//
// The mbarrier waits are bounded; on a timeout the kernel raises the error
// flag, skips the rest, and still frees its tensor memory.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "tb_internal.h"

namespace tb {

namespace {

constexpr int kF = TB_MLP_NFEAT;  // 32
constexpr int kH = 64;
constexpr int kW1 = 0, kB1 = kW1 + kH * kF, kW2 = kB1 + kH, kB2 = kW2 + kH * kH, kW3 = kB2 + kH, kB3 = kW3 + kH;
constexpr int kRows = 128;  // atoms per CTA = MMA M
constexpr uint32_t kTmemCols = 128;
constexpr uint32_t kSpin = 1u << 22;

__device__ __forceinline__ uint32_t sm_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// element offset of (row, k) in a K-major no-swizzle operand with K columns
__device__ __forceinline__ int core_off(int row, int k, int K)
{
    return (row >> 3) * (K / 8) * 64 + (k >> 3) * 64 + (row & 7) * 8 + (k & 7);
}

// shared-memory matrix descriptor: start, LBO = 128 B (K direction), SBO
// (M/N direction), fixed version field 1 (bits 46-47), no swizzle
__device__ __forceinline__ uint64_t smem_desc(const void *p, uint32_t sbo_bytes)
{
    const uint64_t a = (sm_addr(p) & 0x3FFFFu) >> 4;
    return a | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)(sbo_bytes >> 4) << 32) | (1ull << 46);
}

// instruction descriptor, kind::f16: D FP32, A and B BF16, both K-major,
// N >> 3 at bit 17, M >> 4 at bit 24
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n"
        " .reg .pred p;\n"
        " setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
        "}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(sm_addr(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int j = 0; j < 16; j++) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

__device__ __forceinline__ bool bar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n"
        " .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(sm_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ float silu(float z) { return z / (1.f + __expf(-z)); }

__global__ void __launch_bounds__(kRows, 1)
    k_mlp_fwd_tc(int n, const float *__restrict__ X, const float *__restrict__ mean, const float *__restrict__ istd,
                 const float *__restrict__ Wq, float *__restrict__ out, int32_t *err)
{
    __shared__ __align__(1024) __nv_bfloat16 A1[kRows * kF];  // 8 KB
    __shared__ __align__(1024) __nv_bfloat16 B1[kH * kF];     // 4 KB
    __shared__ __align__(1024) __nv_bfloat16 A2[kRows * kH];  // 16 KB
    __shared__ __align__(1024) __nv_bfloat16 B2[kH * kH];     // 8 KB
    __shared__ float b1[kH], b2[kH], w3[kH];
    __shared__ uint64_t bar;
    __shared__ uint32_t tbase;
    __shared__ int s_fail;
    const int tid = threadIdx.x, warp = tid >> 5;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(sm_addr(&tbase)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(sm_addr(&bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        s_fail = 0;
    }
    // weights (exact in BF16: the parameters are BF16-rounded) and biases
    for (int e = tid; e < kH * kF; e += kRows) B1[core_off(e / kF, e % kF, kF)] = __float2bfloat16_rn(Wq[kW1 + e]);
    for (int e = tid; e < kH * kH; e += kRows) B2[core_off(e / kH, e % kH, kH)] = __float2bfloat16_rn(Wq[kW2 + e]);
    if (tid < kH) {
        b1[tid] = Wq[kB1 + tid];
        b2[tid] = Wq[kB2 + tid];
        w3[tid] = Wq[kW3 + tid];
    }
    // this thread's atom: normalised features as BF16 row `tid` of A1
    const int atom = blockIdx.x * kRows + tid;
#pragma unroll 4
    for (int i = 0; i < kF; i++) {
        const float x = atom < n ? (X[(int64_t)atom * kF + i] - mean[i]) * istd[i] : 0.f;
        A1[core_off(tid, i, kF)] = __float2bfloat16_rn(x);
    }
    fence_async_smem();  // generic-proxy operand writes -> tensor core (async proxy)
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tbase;
    const uint32_t lane_base = (uint32_t)(32 * warp) << 16;  // this warp's 32 TMEM lanes
    constexpr uint32_t kId = idesc_bf16(kRows, kH);

    // ---- layer 1: D[:, 0:64] = A1 . B1^T (K = 32: two K = 16 steps) ----
    if (tid == 0) {
#pragma unroll
        for (int ks = 0; ks < kF / 16; ks++)
            mma_bf16(tmem, smem_desc(A1 + ks * 16 * 8, (kF / 8) * 128), smem_desc(B1 + ks * 16 * 8, (kF / 8) * 128),
                     kId, ks > 0);
        mma_commit(&bar);
    }
    bool ok = true;
    {
        uint32_t it = 0;
        while (!bar_try_wait(&bar, 0u))
            if (++it >= kSpin) {
                ok = false;
                break;
            }
    }
    ok = __all_sync(0xffffffffu, ok);  // tcgen05.ld below needs the whole warp
    if (!ok) s_fail = 1;
    tc_fence_after();
    float h[16];
    if (ok) {
        for (int c = 0; c < kH; c += 16) {
            tmem_ld16(tmem + lane_base + (uint32_t)c, h);
            tmem_wait_ld();
#pragma unroll
            for (int j = 0; j < 16; j++) A2[core_off(tid, c + j, kH)] = __float2bfloat16_rn(silu(h[j] + b1[c + j]));
        }
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    // ---- layer 2: D[:, 64:128] = A2 . B2^T (K = 64: four K = 16 steps) ----
    const bool run2 = !s_fail;
    if (tid == 0 && run2) {
#pragma unroll
        for (int ks = 0; ks < kH / 16; ks++)
            mma_bf16(tmem + kH, smem_desc(A2 + ks * 16 * 8, (kH / 8) * 128), smem_desc(B2 + ks * 16 * 8, (kH / 8) * 128),
                     kId, ks > 0);
        mma_commit(&bar);
    }
    if (run2) {
        uint32_t it = 0;
        while (!bar_try_wait(&bar, 1u))
            if (++it >= kSpin) {
                ok = false;
                break;
            }
    } else {
        ok = false;
    }
    ok = __all_sync(0xffffffffu, ok);
    tc_fence_after();
    if (ok) {
        float y = Wq[kB3];
        for (int c = 0; c < kH; c += 16) {
            tmem_ld16(tmem + lane_base + (uint32_t)(kH + c), h);
            tmem_wait_ld();
#pragma unroll
            for (int j = 0; j < 16; j++) y = fmaf(w3[c + j], silu(h[j] + b2[c + j]), y);
        }
        if (atom < n) out[atom] = y;
    } else if (tid == 0) {
        atomicExch(err, 1);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

}  // namespace

void launch_mlp_forward_tc(cudaStream_t st, int n, const float *X, const float *mean, const float *istd,
                           const float *Wq, float *out, int32_t *err)
{
    k_mlp_fwd_tc<<<(n + kRows - 1) / kRows, kRows, 0, st>>>(n, X, mean, istd, Wq, out, err);
}

}  // namespace tb

// tb_pipe.cu -- FP32 Chebyshev step, pipelined form (K2 of the density-matrix
// path: the recurrence of getKPE, withSP2_deltaH.cpp:1134-1168, over identity
// columns, with the moments taken from column dot products as in
// k_cheb_f32_staged).
//
// Slab layout: chunk-major, [B/64][n][64] floats, so that a block row of one
// 64-column chunk is 1 KB contiguous and consecutive block rows are
// contiguous too.
//
// One CTA per SM loops over tiles (row group g of R block rows x one
// 64-column chunk).  A producer warp gathers each tile into a ring of
// shared-memory stages with bulk asynchronous copies (cp.async.bulk,
// completion counted in bytes on the stage's "full" mbarrier): the group's
// distinct referenced block rows of T_k as runs of consecutive rows (one copy
// per run), its own rows of T_{k-1} (one copy), its X blocks (one copy) and a
// packed index record (one copy).  Eight consumer warps compute the tile from
// shared memory while the producer fills the next stages.  Tile headers are
// read one tile ahead, so the producer never waits on its own index loads.
//
// Column dot products <T_k,T_k> and <T_k,T_{k+1}> accumulate in FP32 over one
// block row and then as unevaluated FP32 pairs (hi, lo) across rows and warps:
// every addition is Knuth's TwoSum (s = a + b, e = (a - (s - b')) + (b - b'),
// b' = s - a), its exact rounding error collected in lo.  GB300 issues FP64 at
// about 2 operations per clock per SM, so per-row FP64 accumulation would cost
// as much as the rest of the step; the pairs keep ~44 significant bits with
// FP32 arithmetic only.  The consumer warps' pairs are summed in a fixed order
// through a double-buffered shared array (one named barrier per tile), giving
// partial[g][col][2] as float2 (hi, lo); k_f32_finalize_pairs converts to FP64.
//
// Every mbarrier wait is bounded: after kPipeSpin unsuccessful polls the
// thread raises a block-wide abort flag and the device error flag; all
// consumer warps still run the same tile sequence (so the named barriers stay
// matched) but skip the work, and the producer, before it returns, waits (again
// bounded) for the copies it has issued.
#include <cuda_runtime.h>

#include <algorithm>

#include "tb_internal.h"

namespace tb {

namespace {

constexpr int kPipeCols = 64;
constexpr int kPipeCW = 8;  // consumer warps
constexpr int kPipeThreads = 32 * (kPipeCW + 1);
constexpr uint32_t kPipeSpin = 1u << 22;

struct PipeArgs {
    int n, nb, R, G, nchunk, stages, stage_bytes, maxU, maxBlk, B, first;
    const int4 *hdr;   // per group: {nu, tb0, nbk, rec_off}, {rec_len, run_off, nruns, nr}
    const int4 *runs;  // {first block row, rows, first slot, 0}
    const int32_t *rec;
    const float *x32, *Tin;
    float *Tout;
    float2 *partial;
    int32_t *err;
};

__device__ __forceinline__ uint32_t sm_addr(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(sm_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(sm_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(sm_addr(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
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

// global -> shared bulk copy; both addresses 16-byte aligned, bytes % 16 == 0
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
            sm_addr(dst)),
        "l"(src), "r"(bytes), "r"(sm_addr(bar))
        : "memory");
}

// (s, c) += x with the rounding error of s + x kept exactly in c (TwoSum)
__device__ __forceinline__ void pair_add(float &s, float &c, float x)
{
    const float t = s + x;
    const float bp = t - s;
    const float e = (s - (t - bp)) + (x - bp);
    s = t;
    c += e;
}

__device__ __forceinline__ void consumer_sync()
{
    asm volatile("bar.sync 1, %0;\n" ::"r"(32 * kPipeCW) : "memory");
}

// Poll until the phase of the given parity completes; false on abort or
// after kPipeSpin polls (then the abort and device error flags are raised).
__device__ __forceinline__ bool wait_phase(uint64_t *bar, uint32_t parity, volatile int *s_abort,
                                           int32_t *err)
{
    uint32_t n = 0;
    while (!mbar_try_wait(bar, parity)) {
        if (*s_abort) return false;
        if (++n >= kPipeSpin) {
            *s_abort = 1;
            atomicExch(err, 1);
            return false;
        }
    }
    return true;
}

__global__ void __launch_bounds__(kPipeThreads, 1) k_cheb_f32_pipe(const PipeArgs a)
{
    extern __shared__ __align__(128) unsigned char smem[];
    float *red = reinterpret_cast<float *>(smem + (size_t)a.stages * a.stage_bytes);  // [2][CW][64][2][2]
    uint64_t *full = reinterpret_cast<uint64_t *>(red + 2 * kPipeCW * kPipeCols * 4);
    uint64_t *empty = full + a.stages;
    volatile int *s_abort = reinterpret_cast<volatile int *>(empty + a.stages);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int s = 0; s < a.stages; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kPipeCW);
        }
        *s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    const int ntiles = a.G * a.nchunk;
    const int oT = 0, oP = a.maxU * 4 * kPipeCols, oX = oP + a.R * 4 * kPipeCols,
              oRec = oX + a.maxBlk * 16;  // float offsets inside a stage
    const int64_t chunk_floats = (int64_t)a.n * kPipeCols;

    if (warp == kPipeCW) {
        // ---------------- producer ----------------
        int i = 0;
        int t = blockIdx.x;
        int4 ha = make_int4(0, 0, 0, 0), hb = ha;
        if (t < ntiles) {
            const int g = t % a.G;
            ha = __ldg(a.hdr + 2 * g);
            hb = __ldg(a.hdr + 2 * g + 1);
        }
        for (; t < ntiles; t += gridDim.x, ++i) {
            const int chunk = t / a.G, g = t - chunk * a.G;
            const int nu = ha.x, tb0 = ha.y, nbk = ha.z, r0 = ha.w;
            const int rl = hb.x, roff = hb.y, nruns = hb.z, nr = hb.w;
            const int tn = t + gridDim.x;  // read the next tile's header now
            if (tn < ntiles) {
                const int gn = tn % a.G;
                ha = __ldg(a.hdr + 2 * gn);
                hb = __ldg(a.hdr + 2 * gn + 1);
            }
            const int4 run = lane < nruns ? __ldg(a.runs + roff + lane) : make_int4(0, 0, 0, 0);
            const int s = i % a.stages;
            if (i >= a.stages && !wait_phase(&empty[s], (uint32_t)((i / a.stages) - 1) & 1u, s_abort, a.err))
                break;
            float *stg = reinterpret_cast<float *>(smem + (size_t)s * a.stage_bytes);
            if (lane == 0)
                mbar_arrive_expect_tx(&full[s], (uint32_t)nu * 1024u + (a.first ? 0u : (uint32_t)nr * 1024u) +
                                                    (uint32_t)nbk * 64u + (uint32_t)rl * 4u);
            __syncwarp();
            const float *srcT = a.Tin + (int64_t)chunk * chunk_floats;
            if (lane < nruns)
                bulk_g2s(stg + oT + run.z * 4 * kPipeCols, srcT + (int64_t)run.x * 4 * kPipeCols,
                         (uint32_t)run.y * 1024u, &full[s]);
            for (int q = lane + 32; q < nruns; q += 32) {
                const int4 rr = __ldg(a.runs + roff + q);
                bulk_g2s(stg + oT + rr.z * 4 * kPipeCols, srcT + (int64_t)rr.x * 4 * kPipeCols,
                         (uint32_t)rr.y * 1024u, &full[s]);
            }
            if (lane == 0) {
                bulk_g2s(stg + oX, a.x32 + (int64_t)tb0 * 16, (uint32_t)nbk * 64u, &full[s]);
                bulk_g2s(stg + oRec, a.rec + r0, (uint32_t)rl * 4u, &full[s]);
                if (!a.first)
                    bulk_g2s(stg + oP, a.Tout + (int64_t)chunk * chunk_floats + (int64_t)g * a.R * 4 * kPipeCols,
                             (uint32_t)nr * 1024u, &full[s]);
            }
        }
        if (*s_abort) {
            // let the copies already issued land before the CTA exits
            for (int j = max(0, i - a.stages); j < i; j++) {
                uint32_t n = 0;
                while (!mbar_try_wait(&full[j % a.stages], (uint32_t)(j / a.stages) & 1u) && ++n < kPipeSpin) {
                }
            }
        }
        return;
    }

    // ---------------- consumers ----------------
    const int c = 2 * lane;
    int i = 0, buf = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++i, buf ^= 1) {
        const int s = i % a.stages;
        const int chunk = t / a.G, g = t - chunk * a.G;
        const int I0 = g * a.R, nr = min(a.nb, I0 + a.R) - I0;
        // pairs (hi, lo): [0] <T_k,T_k> col c, [1] <T_k,T_{k+1}> col c, [2], [3] the same for col c+1
        float hs[4] = {0.f, 0.f, 0.f, 0.f}, ls[4] = {0.f, 0.f, 0.f, 0.f};
        if (wait_phase(&full[s], (uint32_t)(i / a.stages) & 1u, s_abort, a.err)) {
            const float *stg = reinterpret_cast<const float *>(smem + (size_t)s * a.stage_bytes);
            const float *sT = stg + oT, *sP = stg + oP, *sX = stg + oX;
            const int32_t *sRp = reinterpret_cast<const int32_t *>(stg + oRec);
            const int32_t *sLc = sRp + nr + 1;
            const int32_t *sLs = sLc + sRp[nr];
            float *out = a.Tout + (int64_t)chunk * chunk_floats + (int64_t)I0 * 4 * kPipeCols + c;
            for (int r = warp; r < nr; r += kPipeCW) {
                float acc[4][2];
#pragma unroll
                for (int q = 0; q < 4; q++) acc[q][0] = acc[q][1] = 0.f;
                const int ta = sRp[r], te = sRp[r + 1];
                for (int tt = ta; tt < te; tt++) {
                    const float *tv = sT + sLc[tt] * 4 * kPipeCols + c;
                    const float4 *xb = reinterpret_cast<const float4 *>(sX + tt * 16);
                    float2 v[4];
#pragma unroll
                    for (int m = 0; m < 4; m++) v[m] = *reinterpret_cast<const float2 *>(tv + m * kPipeCols);
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        const float4 xr = xb[q];
                        const float xm[4] = {xr.x, xr.y, xr.z, xr.w};
#pragma unroll
                        for (int m = 0; m < 4; m++) {
                            acc[q][0] = fmaf(xm[m], v[m].x, acc[q][0]);
                            acc[q][1] = fmaf(xm[m], v[m].y, acc[q][1]);
                        }
                    }
                }
                const float *own = sT + sLs[r] * 4 * kPipeCols + c;
                float ee0 = 0.f, ee1 = 0.f, eo0 = 0.f, eo1 = 0.f;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const float2 ov = *reinterpret_cast<const float2 *>(own + q * kPipeCols);
                    float2 o;
                    if (a.first) {
                        o = make_float2(acc[q][0], acc[q][1]);
                    } else {
                        const float2 p = *reinterpret_cast<const float2 *>(sP + (r * 4 + q) * kPipeCols + c);
                        o.x = 2.f * acc[q][0] - p.x;
                        o.y = 2.f * acc[q][1] - p.y;
                    }
                    *reinterpret_cast<float2 *>(out + (r * 4 + q) * kPipeCols) = o;
                    ee0 = fmaf(ov.x, ov.x, ee0);
                    ee1 = fmaf(ov.y, ov.y, ee1);
                    eo0 = fmaf(ov.x, o.x, eo0);
                    eo1 = fmaf(ov.y, o.y, eo1);
                }
                pair_add(hs[0], ls[0], ee0);
                pair_add(hs[1], ls[1], eo0);
                pair_add(hs[2], ls[2], ee1);
                pair_add(hs[3], ls[3], eo1);
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);  // stage s may be refilled
        float4 *rb = reinterpret_cast<float4 *>(red + ((size_t)(buf * kPipeCW + warp) * kPipeCols + c) * 4);
        rb[0] = make_float4(hs[0], ls[0], hs[1], ls[1]);
        rb[1] = make_float4(hs[2], ls[2], hs[3], ls[3]);
        consumer_sync();
        if (tid < 2 * kPipeCols && !*s_abort) {
            const int j = tid >> 1, which = tid & 1;
            float hsum = 0.f, lsum = 0.f;
#pragma unroll
            for (int w = 0; w < kPipeCW; w++) {
                const float2 v =
                    *reinterpret_cast<const float2 *>(red + ((size_t)(buf * kPipeCW + w) * kPipeCols + j) * 4 + which * 2);
                pair_add(hsum, lsum, v.x);
                lsum += v.y;
            }
            a.partial[((int64_t)g * a.B + chunk * kPipeCols + j) * 2 + which] = make_float2(hsum, lsum);
        }
    }
}

// Identity columns c0 .. c0+B-1 in the chunk-major layout [B/64][n][64].
__global__ void k_slab_identity_cm(float *__restrict__ T0, int n, int B, int c0)
{
    const int64_t tot = (int64_t)n * B, per = (int64_t)n * kPipeCols;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
        const int chunk = (int)(e / per);
        const int64_t rem = e - (int64_t)chunk * per;
        const int row = (int)(rem / kPipeCols), j = (int)(rem % kPipeCols);
        T0[e] = (row == c0 + chunk * kPipeCols + j) ? 1.f : 0.f;
    }
}

}  // namespace

size_t cheb_f32_pipe_stage_bytes(int R, int maxU, int maxBlk, int rec_cap)
{
    const size_t b = (size_t)(maxU + R) * 4 * kPipeCols * sizeof(float) + (size_t)maxBlk * 16 * sizeof(float) +
                     (size_t)rec_cap * sizeof(int32_t);
    return (b + 127) / 128 * 128;
}

size_t cheb_f32_pipe_smem(size_t stage_bytes, int stages)
{
    return (size_t)stages * stage_bytes + (size_t)2 * kPipeCW * kPipeCols * 4 * sizeof(float) +
           (size_t)2 * stages * sizeof(uint64_t) + 16;
}

int cheb_f32_pipe_configure(size_t smem)
{
    return (int)cudaFuncSetAttribute(k_cheb_f32_pipe, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

// Sum the per-group (hi, lo) pairs of a slab in FP32 pairs, convert once to
// FP64 and form the moments d[2k][j] = 2 <T_k,T_k>_j - 1,
// d[2k+1][j] = 2 <T_k,T_{k+1}>_j - X_jj.
__global__ void k_f32_finalize_pairs(const float2 *__restrict__ partial, int K, int rowgroups, int B, int c0,
                                     int n, const float *__restrict__ xdiag32, double *__restrict__ d, int M)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    if (j >= B || k >= K) return;
    const int i = c0 + j;
    if (i >= n) return;
    float eh = 0.f, el = 0.f, oh = 0.f, ol = 0.f;
    const float2 *p = partial + (int64_t)k * rowgroups * B * 2;
    for (int g = 0; g < rowgroups; g++) {
        const float2 e = p[((int64_t)g * B + j) * 2 + 0], o = p[((int64_t)g * B + j) * 2 + 1];
        pair_add(eh, el, e.x);
        el += e.y;
        pair_add(oh, ol, o.x);
        ol += o.y;
    }
    const double se = (double)eh + (double)el, so = (double)oh + (double)ol;
    if (2 * k <= M) d[(int64_t)(2 * k) * n + i] = 2.0 * se - 1.0;
    if (2 * k + 1 <= M) d[(int64_t)(2 * k + 1) * n + i] = 2.0 * so - (double)xdiag32[i];
}

void launch_slab_identity_cm(cudaStream_t st, float *T0, int n, int B, int c0)
{
    const int64_t tot = (int64_t)n * B;
    const int blocks = (int)std::min<int64_t>((tot + 255) / 256, 152 * 16);
    k_slab_identity_cm<<<blocks, 256, 0, st>>>(T0, n, B, c0);
}

void launch_f32_finalize_pairs(cudaStream_t st, const DevMatrix &m, const float2 *partial, int K, int rowgroups,
                               int B, int c0, double *d, int M)
{
    dim3 grid((B + 127) / 128, K);
    k_f32_finalize_pairs<<<grid, 128, 0, st>>>(partial, K, rowgroups, B, c0, m.n, m.xdiag32, d, M);
}

int launch_cheb_step_f32_pipe(cudaStream_t st, const DevMatrix &m, const PipePlan &sp, const float *Tin,
                              float *Tout, int B, int first, float2 *partial_k)
{
    PipeArgs a;
    a.n = m.n;
    a.nb = m.nb;
    a.R = sp.R;
    a.G = sp.G;
    a.nchunk = B / kPipeCols;
    a.stages = sp.stages;
    a.stage_bytes = (int)sp.stage_bytes;
    a.maxU = sp.maxU;
    a.maxBlk = sp.maxBlk;
    a.B = B;
    a.first = first;
    a.hdr = reinterpret_cast<const int4 *>(sp.hdr);
    a.runs = reinterpret_cast<const int4 *>(sp.runs);
    a.rec = sp.rec;
    a.x32 = m.x32;
    a.Tin = Tin;
    a.Tout = Tout;
    a.partial = partial_k;
    a.err = sp.err;
    const int ntiles = sp.G * a.nchunk;
    const int grid = std::min(ntiles, sp.nsm);
    k_cheb_f32_pipe<<<grid, kPipeThreads, cheb_f32_pipe_smem(sp.stage_bytes, sp.stages), st>>>(a);
    return 1;
}

}  // namespace tb

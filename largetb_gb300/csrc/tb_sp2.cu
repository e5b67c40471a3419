// tb_sp2.cu -- SP2 purification as a thresholded 4x4-block SpGEMM (K6).
//
// Restates the matrix form of the reference's SP2 recursion (getSP2,
// withSP2.cpp:956-984; branch rule of computeAlphas, withSP2.cpp:1027-1030):
// X_0 = (lmax I - H)/(lmax - lmin) from the Gershgorin bounds, then per step
// X <- X^2 if 2 tr X > N_e, else 2X - X^2, dropping 4x4 blocks whose Frobenius
// norm falls below the drop tolerance.  Blocks are FP32 (FP64 for the plain
// form); traces and ||X^2 - X||_F are accumulated in FP64.
//
// Storage: "ragged BSR" -- per block row a start and a length into colidx /
// blocks, each row's columns sorted; rows need not be stored in order, so a
// step can append rows as CTAs finish them.
//
// k_sp2_step: one CTA per block row (grid-stride).  Phase A accumulates the
// row of X^2 = sum_K X_IK X_K* into a dense per-column accumulator (shared
// memory when nb * 16 values fit, else a per-CTA global slice) with a bitmap
// of touched columns; 16 lanes compute one 4x4 product (lane = one output
// element, 4 FMAs).  Phase B scans the bitmap in column order, forms the new
// block (the old X_IJ located through a bitmap of row I's columns and prefix
// counts), drops small blocks, and appends the compacted row to the output.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "tb_f32x2.cuh"
#include "tb_internal.h"

namespace tb {

struct Sp2Scalars {
    double trX2, idem2, trNew, trX;
    unsigned long long count;
    unsigned long long bound;
    unsigned long long products;  // 4x4 block products of the step (64 FMA each)
    int overflow;
    int pad;
};

namespace {

constexpr int kSp2Threads = 1024;  // 32 warps: the dense-row accumulator allows 2 CTAs per SM
static_assert(kSp2Threads % 32 == 0 && kSp2Threads <= 1024, "SP2 block size");
constexpr int kSp2ScanInts = 32;  // one int per warp for block_excl_scan
constexpr int kSp2MiscInts = 8;   // [0] total, [1] overflow, [2] output base

// Dynamic shared memory of k_sp2_step before its dense row accumulator:
// bitmap of the product's columns, bitmap of row I's own columns and its
// per-word prefix counts, touched-column list, keep flags, scan and misc words.
__host__ __device__ inline size_t sp2_base_smem(int nb)
{
    const size_t nw = ((size_t)nb + 31) / 32;
    return ((3 * nw + 2 * (size_t)nb + kSp2ScanInts + kSp2MiscInts) * 4 + 15) & ~(size_t)15;
}

__device__ __forceinline__ int block_excl_scan(int v, int *sh, int *total)
{
    // exclusive scan over the kSp2Threads threads; sh holds one int per warp
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        int t = lane < (kSp2Threads / 32) ? sh[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < (kSp2Threads / 32)) sh[lane] = t;
    }
    __syncthreads();
    const int before = (w > 0 ? sh[w - 1] : 0) + x - v;
    *total = sh[kSp2Threads / 32 - 1];
    __syncthreads();
    return before;
}

__device__ __forceinline__ double warp_sum_d(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Element (m, s) of the 4x4 block whose element (r, s) this lane holds, from
// lane 4 m + s of the same half warp.
template <typename T>
__device__ __forceinline__ T col_of(T e, int s, int m)
{
    return __shfl_sync(0xffffffffu, e, 4 * m + s, 16);
}

template <typename T>
__device__ int find_col(const int32_t *col, int start, int len, int J)
{
    int lo = 0, hi = len - 1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const int c = col[start + mid];
        if (c == J) return start + mid;
        if (c < J)
            lo = mid + 1;
        else
            hi = mid - 1;
    }
    return -1;
}

}  // namespace

// X_0 = (lmax I - H) / (lmax - lmin) on the pattern of H; tr X_0 in FP64.
template <typename T>
__global__ void k_sp2_init(int nb, const int32_t *__restrict__ rowptr,
                           const int32_t *__restrict__ colidx, const int32_t *__restrict__ blkrow,
                           const double *__restrict__ h0, const DevState *__restrict__ gs,
                           int32_t *__restrict__ rs, int32_t *__restrict__ rl,
                           int32_t *__restrict__ col, T *__restrict__ blk, Sp2Scalars *sc)
{
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nnzb = rowptr[nb];
    double tr = 0.0;
    if (e < nnzb * 16) {
        const int64_t t = e >> 4;
        const int rc = (int)(e & 15), r = rc >> 2, c = rc & 3;
        const int I = blkrow[t];
        const double width = gs->lmax - gs->lmin;
        double v = -h0[e];
        if (colidx[t] == I && r == c) v += gs->lmax;
        v /= width;
        blk[e] = (T)v;
        if (rc == 0) col[t] = colidx[t];
        if (colidx[t] == I && r == c) tr = (double)(T)v;
    }
    if (e < nb) {
        rs[e] = rowptr[e];
        rl[e] = rowptr[e + 1] - rowptr[e];
    }
    tr = warp_sum_d(tr);
    if ((threadIdx.x & 31) == 0 && tr != 0.0) atomicAdd(&sc->trX, tr);
}

// Upper bound of the blocks of X^2: sum_I min(nb, sum_{K in row I} len(K));
// the uncapped sum is the number of block products of the step.
__global__ void k_sp2_bound(int nb, const int32_t *__restrict__ rs, const int32_t *__restrict__ rl,
                            const int32_t *__restrict__ col, Sp2Scalars *sc)
{
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long b = 0, p = 0;
    if (I < nb) {
        long long s = 0;
        for (int t = 0; t < rl[I]; t++) s += rl[col[rs[I] + t]];
        b = (unsigned long long)(s < nb ? s : nb);
        p = (unsigned long long)s;
    }
    for (int o = 16; o > 0; o >>= 1) {
        b += __shfl_xor_sync(0xffffffffu, b, o);
        p += __shfl_xor_sync(0xffffffffu, p, o);
    }
    if ((threadIdx.x & 31) == 0 && b) {
        atomicAdd(&sc->bound, b);
        atomicAdd(&sc->products, p);
    }
}

template <typename T>
__global__ void __launch_bounds__(kSp2Threads)
    k_sp2_step(int nb, const int32_t *__restrict__ rs, const int32_t *__restrict__ rl,
               const int32_t *__restrict__ col, const T *__restrict__ blk, int branch,
               double drop2, int32_t *__restrict__ ors, int32_t *__restrict__ orl,
               int32_t *__restrict__ ocol, T *__restrict__ oblk, long long out_cap,
               Sp2Scalars *sc, T *__restrict__ gacc, int acc_in_smem)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    const int nw = (nb + 31) >> 5;
    uint32_t *bm = reinterpret_cast<uint32_t *>(smraw);       // nw words
    uint32_t *bmI = bm + nw;                                  // nw words: columns of row I of X
    int32_t *prefI = reinterpret_cast<int32_t *>(bmI + nw);   // nw: row-I columns in earlier words
    int32_t *list = prefI + nw;                               // nb entries
    int32_t *keep = list + nb;                                // nb entries
    int *scan = keep + nb;                                    // kSp2ScanInts
    int *misc = scan + kSp2ScanInts;                          // [0]=total, [1]=kept, [2]=base
    T *acc = acc_in_smem ? reinterpret_cast<T *>(smraw + sp2_base_smem(nb)) : gacc + (size_t)blockIdx.x * nb * 16;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int l16 = lane & 15, half = lane >> 4, r = l16 >> 2, s = l16 & 3;
    for (int i = tid; i < nw; i += kSp2Threads) bm[i] = bmI[i] = 0u;
    for (size_t i = tid; i < (size_t)nb * 16; i += kSp2Threads) acc[i] = T(0);
    __syncthreads();
    double trX2 = 0.0, idem2 = 0.0, trNew = 0.0;
    float ih = 0.f, il = 0.f;  // FP32 blocks: sum of (X^2 - X)^2 as a TwoSum pair
    for (int I = blockIdx.x; I < nb; I += gridDim.x) {
        const int ri = rs[I], li = rl[I];
        // row I's own columns as a bitmap: with per-word prefix counts it gives
        // the position of X_IJ in the (sorted) row without a search
        for (int t = tid; t < li; t += kSp2Threads) {
            const int J = col[ri + t];
            atomicOr(bmI + (J >> 5), 1u << (J & 31));
        }
        // ---- phase A: row I of X^2 ----
        // a half warp forms one 4x4 block product: lane (r, s) loads element
        // (r, s) of B (one coalesced 64-byte load per block), gathers column s
        // by shuffles and accumulates its entry of A B into the dense row;
        // four products per half warp have their loads in flight together.
        for (int t = w; t < li; t += kSp2Threads / 32) {
            const int K = col[ri + t];
            const T *A = blk + (size_t)(ri + t) * 16;
            const T a0 = A[4 * r + 0], a1 = A[4 * r + 1], a2 = A[4 * r + 2], a3 = A[4 * r + 3];
            const int rk = rs[K], lk = rl[K];
            // warp-uniform trip counts (base is the same in both half warps),
            // so the 16-lane shuffles always run converged
            int base = 0;
            for (; base + 7 < lk; base += 8) {
                const int u = base + half;
                int J[4];
                T e[4];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    J[j] = col[rk + u + 2 * j];
                    e[j] = blk[(size_t)(rk + u + 2 * j) * 16 + l16];
                }
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const T v = a0 * col_of(e[j], s, 0) + a1 * col_of(e[j], s, 1) + a2 * col_of(e[j], s, 2) +
                                a3 * col_of(e[j], s, 3);
                    atomicAdd(acc + (size_t)J[j] * 16 + l16, v);
                    if (l16 == 0) atomicOr(bm + (J[j] >> 5), 1u << (J[j] & 31));
                }
            }
            // remainder: the missing products of the last pair are masked
            for (; base < lk; base += 2) {
                const int uu = base + half;
                const bool ok = uu < lk;
                const int J = ok ? col[rk + uu] : 0;
                const T e = ok ? blk[(size_t)(rk + uu) * 16 + l16] : T(0);
                const T v = a0 * col_of(e, s, 0) + a1 * col_of(e, s, 1) + a2 * col_of(e, s, 2) + a3 * col_of(e, s, 3);
                if (ok) {
                    atomicAdd(acc + (size_t)J * 16 + l16, v);
                    if (l16 == 0) atomicOr(bm + (J >> 5), 1u << (J & 31));
                }
            }
        }
        __syncthreads();
        // ---- phase B1: touched columns in increasing order ----
        const int wpt = (nw + kSp2Threads - 1) / kSp2Threads;
        int cnt = 0;
        for (int q = 0; q < wpt; q++) {
            const int wi = tid * wpt + q;
            if (wi < nw) cnt += __popc(bm[wi]);
        }
        if (w == 0) {  // exclusive prefix of the row-I bitmap's word counts
            int carry = 0;
            for (int b0 = 0; b0 < nw; b0 += 32) {
                const int c = b0 + lane < nw ? __popc(bmI[b0 + lane]) : 0;
                int x = c;
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, x, o);
                    if (lane >= o) x += y;
                }
                if (b0 + lane < nw) prefI[b0 + lane] = carry + x - c;
                carry += __shfl_sync(0xffffffffu, x, 31);
            }
        }
        int total;
        int pos = block_excl_scan(cnt, scan, &total);  // its barriers also publish prefI
        for (int q = 0; q < wpt; q++) {
            const int wi = tid * wpt + q;
            if (wi >= nw) break;
            uint32_t bits = bm[wi];
            while (bits) {
                const int b = __ffs(bits) - 1;
                bits &= bits - 1;
                list[pos++] = wi * 32 + b;
            }
            bm[wi] = 0u;
        }
        __syncthreads();
        // ---- phase B2: new block, norms, traces, keep flag (16 lanes per entry) ----
        // warp-uniform trip count: both half-warps iterate, entries past
        // `total` are predicated off, so the 16-lane shuffles stay converged
        for (int i0 = w * 2; i0 < total; i0 += (kSp2Threads / 32) * 2) {
            const int i = i0 + half;
            const bool valid = i < total;
            const int J = valid ? list[i] : 0;
            T *a = acc + (size_t)J * 16;
            const T x2 = valid ? a[l16] : T(0);
            const uint32_t wI = bmI[J >> 5], bI = 1u << (J & 31);  // J = 0 when !valid: in range
            const int xi = valid && (wI & bI) ? ri + prefI[J >> 5] + __popc(wI & (bI - 1u)) : -1;
            const T xo = xi >= 0 ? blk[(size_t)xi * 16 + l16] : T(0);
            const T nv = branch < 0 ? x2 : T(2) * xo - x2;
            float nrm;
            if constexpr (sizeof(T) == 4) {
                // FP32 blocks: FP32 norms (GB300 issues FP64 at ~1/64 the rate);
                // the idempotency sum is a TwoSum pair
                const float dl = x2 - xo;
                pair_add(ih, il, dl * dl);
                nrm = nv * nv;
            } else {
                const double dl = (double)x2 - (double)xo;
                idem2 += dl * dl;
                nrm = (float)((double)nv * (double)nv);
            }
            for (int o = 8; o > 0; o >>= 1) nrm += __shfl_xor_sync(0xffffffffu, nrm, o);
            const int kp = (double)nrm >= drop2;
            if (valid) {
                if (J == I && r == s) {
                    trX2 += (double)x2;
                    if (kp) trNew += (double)nv;
                }
                a[l16] = nv;
                if (l16 == 0) keep[i] = kp;
            }
        }
        __syncthreads();
        // ---- phase B3: compaction ----
        int kc = 0;
        const int ept = (total + kSp2Threads - 1) / kSp2Threads;
        for (int q = 0; q < ept; q++) {
            const int i = tid * ept + q;
            if (i < total) kc += keep[i];
        }
        int kept;
        int kpos = block_excl_scan(kc, scan, &kept);
        if (tid == 0) {
            const unsigned long long base = atomicAdd(&sc->count, (unsigned long long)kept);
            misc[2] = (int)base;
            const bool over = (long long)(base + kept) > out_cap;
            misc[1] = over ? 1 : 0;
            if (over) sc->overflow = 1;
            ors[I] = over ? 0 : (int)base;
            orl[I] = over ? 0 : kept;
        }
        for (int q = 0; q < ept; q++) {
            const int i = tid * ept + q;
            if (i < total && keep[i]) {
                keep[i] = kpos++ + 1;  // 1-based output slot
            } else if (i < total) {
                keep[i] = 0;
            }
        }
        __syncthreads();
        const int base = misc[2], over = misc[1];
        for (int i = w * 2 + half; i < total; i += (kSp2Threads / 32) * 2) {
            const int J = list[i];
            T *a = acc + (size_t)J * 16;
            const int slot = keep[i];
            if (!over && slot > 0) {
                const size_t o = (size_t)base + slot - 1;
                oblk[o * 16 + l16] = a[l16];
                if (l16 == 0) ocol[o] = J;
            }
            a[l16] = T(0);
        }
        for (int i = tid; i < nw; i += kSp2Threads) bmI[i] = 0u;  // read last in phase B2
        __syncthreads();
    }
    idem2 += (double)ih + (double)il;
    trX2 = warp_sum_d(trX2);
    idem2 = warp_sum_d(idem2);
    trNew = warp_sum_d(trNew);
    if (lane == 0) {
        if (trX2 != 0.0) atomicAdd(&sc->trX2, trX2);
        if (idem2 != 0.0) atomicAdd(&sc->idem2, idem2);
        if (trNew != 0.0) atomicAdd(&sc->trNew, trNew);
    }
}

// diag P, q_a = 2 sum P_ii, and sum_{blocks} X_IJ . H_IJ (= tr(X H) for symmetric H).
template <typename T>
__global__ void k_sp2_outputs(int nb, const int32_t *__restrict__ rowptr,
                              const int32_t *__restrict__ colidx, const int32_t *__restrict__ blkrow,
                              const double *__restrict__ h0, const int32_t *__restrict__ rs,
                              const int32_t *__restrict__ rl, const int32_t *__restrict__ col,
                              const T *__restrict__ blk, double *__restrict__ diagP,
                              double *__restrict__ q, Sp2Scalars *sc)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nnzb = rowptr[nb];
    double xh = 0.0;
    if (t < nnzb) {
        const int I = blkrow[t], J = colidx[t];
        const int xi = find_col<T>(col, rs[I], rl[I], J);
        if (xi >= 0)
            for (int e = 0; e < 16; e++) xh += (double)blk[(size_t)xi * 16 + e] * h0[t * 16 + e];
    }
    if (t < nb) {
        const int I = (int)t;
        const int xi = find_col<T>(col, rs[I], rl[I], I);
        double s = 0.0;
        for (int r = 0; r < 4; r++) {
            const double v = xi >= 0 ? (double)blk[(size_t)xi * 16 + 5 * r] : 0.0;
            if (diagP) diagP[4 * I + r] = v;
            s += v;
        }
        if (q) q[I] = 2.0 * s;
    }
    xh = warp_sum_d(xh);
    if ((threadIdx.x & 31) == 0 && xh != 0.0) atomicAdd(&sc->trX, xh);
}

// ---------------------------------------------------------------------------
// host driver
// ---------------------------------------------------------------------------
namespace {

struct Sp2Buf {
    int32_t *rs = nullptr, *rl = nullptr, *col = nullptr;
    void *blk = nullptr;
    long long cap = 0;
};

void sp2_free(Sp2Buf &b)
{
    if (b.rs) cudaFree(b.rs);
    if (b.rl) cudaFree(b.rl);
    if (b.col) cudaFree(b.col);
    if (b.blk) cudaFree(b.blk);
    b = Sp2Buf{};
}

cudaError_t sp2_reserve(Sp2Buf &b, int nb, long long cap, size_t es)
{
    cudaError_t e = cudaSuccess;
    if (!b.rs) {
        if ((e = cudaMalloc(&b.rs, sizeof(int32_t) * nb))) return e;
        if ((e = cudaMalloc(&b.rl, sizeof(int32_t) * nb))) return e;
    }
    if (cap > b.cap) {
        if (b.col) cudaFree(b.col);
        if (b.blk) cudaFree(b.blk);
        b.col = nullptr;
        b.blk = nullptr;
        if ((e = cudaMalloc(&b.col, sizeof(int32_t) * cap))) return e;
        if ((e = cudaMalloc(&b.blk, es * 16 * cap))) return e;
        b.cap = cap;
    }
    return cudaSuccess;
}

template <typename T>
int sp2_run(tb_ctx *ctx, double *diagP_h, double *q_h, double *e_band, tb_report *rep,
            std::vector<int> &branches)
{
    DevMatrix &m = ctx->m;
    cudaStream_t st = ctx->stream;
    const int nb = m.nb;
    const double ne = ctx->p.n_electrons;
    const double drop2 = ctx->p.sp2_drop_tol * ctx->p.sp2_drop_tol;
    Sp2Buf A, B;
    Sp2Scalars *sc = nullptr;
    DevState *gs = nullptr;
    double *d_diag = nullptr, *d_q = nullptr;
    T *gacc = nullptr;
    int rc = TB_OK;
    auto cuda_fail = [&](cudaError_t e, const char *what) {
        ctx->err = std::string(what) + ": " + cudaGetErrorString(e);
        rc = e == cudaErrorMemoryAllocation ? TB_ERR_OUT_OF_MEMORY : TB_ERR_CUDA;
    };
    cudaError_t e;
    Sp2Scalars hs;
    int64_t launches = 0;
    double products = 0.0, moved = 0.0;  // block products and algorithmic bytes over all steps
    int64_t cur_nnzb = 0;
    int it = 0;
    double idem = INFINITY, prev1 = INFINITY, prev2 = INFINITY, trX = 0.0;
    // shared-memory budget of k_sp2_step
    const size_t base_smem = sp2_base_smem(nb);
    size_t acc_bytes = (size_t)nb * 16 * sizeof(T);
    int dev_smem = 0;
    cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
    const bool acc_smem = base_smem + acc_bytes <= (size_t)dev_smem;
    const size_t smem = acc_smem ? base_smem + acc_bytes : base_smem;
    int nsm = 152;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device);
    int grid = std::min(nb, nsm * (acc_smem ? std::max(1, (int)(227 * 1024 / (smem + 1024))) : 4));
    if ((e = cudaFuncSetAttribute(k_sp2_step<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  smem_optin_max((const void *)k_sp2_step<T>)))) {
        cuda_fail(e, "cudaFuncSetAttribute(k_sp2_step)");
        return rc;
    }
    if ((e = cudaMalloc(&sc, sizeof(Sp2Scalars))) || (e = cudaMalloc(&gs, sizeof(DevState))) ||
        (e = cudaMalloc(&d_diag, sizeof(double) * m.n)) || (e = cudaMalloc(&d_q, sizeof(double) * nb))) {
        cuda_fail(e, "cudaMalloc(sp2 scalars)");
        goto done;
    }
    if (!acc_smem && (e = cudaMalloc(&gacc, sizeof(T) * 16 * (size_t)nb * grid))) {
        cuda_fail(e, "cudaMalloc(sp2 accumulators)");
        goto done;
    }
    // Gershgorin bounds of H (no shift) and X_0
    launch_gershgorin(st, m, nullptr, 0.0, 0.0, 2, 1 << 22, gs);
    if ((e = sp2_reserve(A, nb, m.nnzb, sizeof(T)))) {
        cuda_fail(e, "cudaMalloc(sp2 X)");
        goto done;
    }
    cudaMemsetAsync(sc, 0, sizeof(Sp2Scalars), st);
    {
        const int64_t tot = std::max<int64_t>(m.nnzb * 16, nb);
        k_sp2_init<T><<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(nb, m.rowptr, m.colidx, m.blkrow, m.h0,
                                                                      gs, A.rs, A.rl, A.col, (T *)A.blk, sc);
        launches += 2;
    }
    cudaMemcpyAsync(&hs, sc, sizeof(hs), cudaMemcpyDeviceToHost, st);
    if ((e = cudaStreamSynchronize(st))) {
        cuda_fail(e, "sp2 init");
        goto done;
    }
    {
        DevState g;
        cudaMemcpy(&g, gs, sizeof(g), cudaMemcpyDeviceToHost);
        if (!(g.lmax > g.lmin)) {
            ctx->err = "Gershgorin interval collapsed";
            rc = TB_ERR_SPECTRUM;
            goto done;
        }
        if (rep) {
            rep->lmin = g.lmin;
            rep->lmax = g.lmax;
        }
    }
    trX = hs.trX;
    cur_nnzb = m.nnzb;
    for (it = 0;; it++) {
        // capacity of X^2
        cudaMemsetAsync(sc, 0, sizeof(Sp2Scalars), st);
        k_sp2_bound<<<(nb + 255) / 256, 256, 0, st>>>(nb, A.rs, A.rl, A.col, sc);
        cudaMemcpyAsync(&hs, sc, sizeof(hs), cudaMemcpyDeviceToHost, st);
        if ((e = cudaStreamSynchronize(st))) {
            cuda_fail(e, "sp2 bound");
            goto done;
        }
        if ((e = sp2_reserve(B, nb, (long long)hs.bound, sizeof(T)))) {
            cuda_fail(e, "cudaMalloc(sp2 X^2)");
            goto done;
        }
        products += (double)hs.products;
        const int branch = (2.0 * trX > ne) ? -1 : 1;  // withSP2.cpp:1029-1030
        k_sp2_step<T><<<grid, kSp2Threads, smem, st>>>(nb, A.rs, A.rl, A.col, (const T *)A.blk, branch, drop2,
                                                       B.rs, B.rl, B.col, (T *)B.blk, B.cap, sc, gacc,
                                                       acc_smem ? 1 : 0);
        launches += 2;
        cudaMemcpyAsync(&hs, sc, sizeof(hs), cudaMemcpyDeviceToHost, st);
        if ((e = cudaStreamSynchronize(st))) {
            cuda_fail(e, "sp2 step");
            goto done;
        }
        if (hs.overflow) {
            ctx->err = "SP2 output exceeded its bound";
            rc = TB_ERR_CUDA;
            goto done;
        }
        idem = std::sqrt(hs.idem2);
        // algorithmic bytes of the step: X_k blocks + columns read once, X_{k+1} written once
        moved += (double)(cur_nnzb + (int64_t)hs.count) * (16.0 * sizeof(T) + 4.0) + 16.0 * nb;
        bool stop = false;
        if (idem < ctx->p.sp2_idem_tol) stop = true;
        // stagnation once in the quadratic regime (the oracle's rule)
        if (it >= 2 && prev2 < 0.1 && idem >= prev2) stop = true;
        if (it >= ctx->p.sp2_max_iter) stop = true;
        if (stop) break;
        branches.push_back(branch);
        std::swap(A, B);
        cur_nnzb = (int64_t)hs.count;
        trX = hs.trNew;
        prev2 = prev1;
        prev1 = idem;
    }
    // outputs from X_it (buffer A)
    cudaMemsetAsync(sc, 0, sizeof(Sp2Scalars), st);
    {
        const int64_t tot = std::max<int64_t>(m.nnzb, nb);
        k_sp2_outputs<T><<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(nb, m.rowptr, m.colidx, m.blkrow, m.h0,
                                                                         A.rs, A.rl, A.col, (const T *)A.blk,
                                                                         d_diag, d_q, sc);
        launches++;
    }
    {
        std::vector<int32_t> rl(nb);
        cudaMemcpyAsync(&hs, sc, sizeof(hs), cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(rl.data(), A.rl, sizeof(int32_t) * nb, cudaMemcpyDeviceToHost, st);
        if (diagP_h) cudaMemcpyAsync(diagP_h, d_diag, sizeof(double) * m.n, cudaMemcpyDeviceToHost, st);
        if (q_h) cudaMemcpyAsync(q_h, d_q, sizeof(double) * nb, cudaMemcpyDeviceToHost, st);
        if ((e = cudaStreamSynchronize(st))) {
            cuda_fail(e, "sp2 outputs");
            goto done;
        }
        int64_t nnzb = 0;
        for (int v : rl) nnzb += v;
        if (e_band) *e_band = 2.0 * hs.trX;
        if (rep) {
            rep->e_band = 2.0 * hs.trX;
            rep->idem_err = idem;
            rep->sp2_iters = it;
            rep->sp2_nnzb = nnzb;
            rep->sp2_flops = 128.0 * products;
            rep->sp2_bytes = moved;
            rep->kernel_launches = launches;
            rep->precision = ctx->p.precision;
        }
    }
    if (it >= ctx->p.sp2_max_iter && !(idem < ctx->p.sp2_idem_tol)) {
        // the cap was the stopping reason only if the error was still falling
        if (!(prev2 <= idem)) {
            ctx->err = "SP2 reached sp2_max_iter";
            rc = TB_ERR_NOT_CONVERGED;
        }
    }
done:
    sp2_free(A);
    sp2_free(B);
    if (sc) cudaFree(sc);
    if (gs) cudaFree(gs);
    if (d_diag) cudaFree(d_diag);
    if (d_q) cudaFree(d_q);
    if (gacc) cudaFree(gacc);
    return rc;
}

}  // namespace

int run_sp2(tb_ctx *ctx, double *diagP, double *q, double *e_band, tb_report *rep,
            int32_t *branches_out, int32_t branches_cap)
{
    std::vector<int> br;
    int rc = ctx->p.precision == TB_PREC_FP32 ? sp2_run<float>(ctx, diagP, q, e_band, rep, br)
                                              : sp2_run<double>(ctx, diagP, q, e_band, rep, br);
    if (branches_out)
        for (int i = 0; i < (int)br.size() && i < branches_cap; i++) branches_out[i] = br[i];
    return rc;
}

}  // namespace tb

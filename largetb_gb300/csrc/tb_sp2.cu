// tb_sp2.cu -- SP2 purification as a thresholded 4x4-block SpGEMM (K6).
//
// Restates the matrix form of the reference's SP2 recursion (getSP2,
// withSP2.cpp:956-984; branch rule of computeAlphas, withSP2.cpp:1027-1030):
// X_0 = (lmax I - H)/(lmax - lmin) from the Gershgorin bounds, then per step
// X <- X^2 if 2 tr X > N_e, else 2X - X^2, dropping 4x4 blocks whose Frobenius
// norm falls below the drop tolerance.  Blocks are FP32 (FP64 for the plain
// form); traces and ||X^2 - X||_F are accumulated in FP64.
//
// X is block CSR with sorted columns.  Every X_k is symmetric (X_0 is, the
// product of a symmetric matrix with itself is, and the drop test is the same
// for a block and its transpose), so a step forms only the output blocks
// (I, J >= I) and writes each one twice, as itself and transposed at (J, I):
// half the block products, and X stays exactly symmetric.
//
// One step, per output block row I:
//   - row bitmaps: RB[I] has bit K set for every stored block (I, K), RP[I]
//     the per-word prefix counts, so the position of (I, K) in the row is
//     RP[I][K/32] + popc(RB[I][K/32] below bit K) -- no search;
//   - symbolic: the pattern of row I of X^2 (with X's own pattern, which
//     2X - X^2 needs) is the OR of the bitmaps of the rows K of row I;
//     its popcounts and a scan give the output's row pointers;
//   - numeric: (X^2)_IJ = sum_K X_IK X_KJ = sum_K X_IK (X_JK)^T over the K in
//     both rows I and J -- the AND of two bitmaps.  One warp owns one output
//     block: its lanes take the intersection's K round-robin and each forms
//     a whole 4x4 x 4x4 product into 16 register accumulators (FP32: 32
//     packed fma.rn.f32x2, even/odd m in the two halves), then 16 shuffles
//     reduce the 16 sums across the warp.  No shared-memory atomics, no
//     CTA-wide barrier per block; row I's blocks sit in shared memory;
//   - compaction of the kept blocks into the next X.
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
    unsigned long long count;          // kept blocks of X_{k+1}
    unsigned long long bound;          // blocks of the pattern of X_k^2 (uncompacted output)
    unsigned long long products;       // 4x4 block products performed (J >= I only)
    unsigned long long full_products;  // block products of the whole X_k^2 (sum_I sum_{K in I} len K)
    int overflow;                      // 1: output capacity, 2: asymmetric pattern
    int maxlen;                        // longest row of X_k
};

namespace {

constexpr int kNumWarps = 8;         // warps per CTA of the numeric kernel
constexpr int kJCap = 1024 / kNumWarps; // J items per warp and 32-word chunk (<= 1024 bits, round-robin)

__device__ __forceinline__ double warp_sum_d(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ int warp_incl_scan(int x, int lane)
{
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    return x;
}

template <typename T>
__device__ int find_col(const int32_t *col, int start, int end, int J)
{
    int lo = start, hi = end - 1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const int c = col[mid];
        if (c == J) return mid;
        if (c < J)
            lo = mid + 1;
        else
            hi = mid - 1;
    }
    return -1;
}

// Sum of 16 per-lane values over the warp by recursive halving: at each of
// the exchanges xor 16, 8, 4, 2 a lane keeps half of its values and adds its
// partner's copy of that half (8 + 4 + 2 + 1 shuffles), then xor 1 adds the
// last pair.  Lanes 2e and 2e + 1 end with element e = (lane >> 1) & 15.
template <typename T>
__device__ __forceinline__ T warp_reduce16(T (&v)[16], int lane)
{
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const bool up = lane & 16;
        const T send = up ? v[k] : v[k + 8];
        const T keep = up ? v[k + 8] : v[k];
        v[k] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const bool up = lane & 8;
        const T send = up ? v[k] : v[k + 4];
        const T keep = up ? v[k + 4] : v[k];
        v[k] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const bool up = lane & 4;
        const T send = up ? v[k] : v[k + 2];
        const T keep = up ? v[k + 2] : v[k];
        v[k] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    }
    {
        const bool up = lane & 2;
        const T send = up ? v[0] : v[1];
        const T keep = up ? v[1] : v[0];
        v[0] = keep + __shfl_xor_sync(0xffffffffu, send, 2);
    }
    return v[0] + __shfl_xor_sync(0xffffffffu, v[0], 1);
}

// Block storage of X: block row J (first block s = ptr[J], L blocks) keeps
// the 16 elements of its blocks as 8 planes of element pairs: pair p = 2r + h
// (elements (r, 2h), (r, 2h + 1)) of block pos sits at pair index
// 8 s + p L + pos.  Lanes working on neighbouring blocks of a row then load
// neighbouring 8-byte (16-byte in FP64) pairs: coalesced global loads and
// conflict-free shared-memory loads.
__device__ __forceinline__ size_t plane_elem(int s, int L, int pos, int e)
{
    return (size_t)s * 16 + 2 * ((size_t)(e >> 1) * L + pos) + (e & 1);
}

// acc[4r + c] += sum_m A[r][m] B[c][m] for blocks A (pairs a[p * la]) and
// B (pairs b[p * lb]).  FP32: the even and odd m in the two halves of a
// packed accumulator, 32 fma.rn.f32x2.
__device__ __forceinline__ void block_abt(float2 (&acc)[16], const float2 *a, int la, const float2 *b, int lb)
{
    float2 A[8], B[8];
#pragma unroll
    for (int p = 0; p < 8; p++) {
        A[p] = a[(size_t)p * la];
        B[p] = __ldg(b + (size_t)p * lb);
    }
#pragma unroll
    for (int r = 0; r < 4; r++)
#pragma unroll
        for (int c = 0; c < 4; c++) {
            acc[4 * r + c] = __ffma2_rn(A[2 * r], B[2 * c], acc[4 * r + c]);
            acc[4 * r + c] = __ffma2_rn(A[2 * r + 1], B[2 * c + 1], acc[4 * r + c]);
        }
}

// 8- or 16-byte asynchronous copy global -> shared (LDGSTS), and its group fences.
template <int N>
__device__ __forceinline__ void cp_async(void *smem_dst, const void *gmem_src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    if constexpr (N == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(gmem_src) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// acc += A B^T with A's pairs at a[p * la] and B's pairs at b[p * lb] (B in
// shared memory, stride lb = 32 entries).
__device__ __forceinline__ void block_abt_s(float2 (&acc)[16], const float2 *a, int la, const float2 *b)
{
    float2 A[8], B[8];
#pragma unroll
    for (int p = 0; p < 8; p++) {
        A[p] = a[(size_t)p * la];
        B[p] = b[32 * p];
    }
#pragma unroll
    for (int r = 0; r < 4; r++)
#pragma unroll
        for (int c = 0; c < 4; c++) {
            acc[4 * r + c] = __ffma2_rn(A[2 * r], B[2 * c], acc[4 * r + c]);
            acc[4 * r + c] = __ffma2_rn(A[2 * r + 1], B[2 * c + 1], acc[4 * r + c]);
        }
}
__device__ __forceinline__ void block_abt_s(double (&acc)[16], const double2 *a, int la, const double2 *b)
{
    double2 A[8], B[8];
#pragma unroll
    for (int p = 0; p < 8; p++) {
        A[p] = a[(size_t)p * la];
        B[p] = b[32 * p];
    }
#pragma unroll
    for (int r = 0; r < 4; r++)
#pragma unroll
        for (int c = 0; c < 4; c++) {
            double v = acc[4 * r + c];
            v = fma(A[2 * r].x, B[2 * c].x, v);
            v = fma(A[2 * r].y, B[2 * c].y, v);
            v = fma(A[2 * r + 1].x, B[2 * c + 1].x, v);
            v = fma(A[2 * r + 1].y, B[2 * c + 1].y, v);
            acc[4 * r + c] = v;
        }
}

// Two block products with all their loads issued before the arithmetic.
template <typename Acc, typename P2>
__device__ __forceinline__ void block_abt2(Acc (&acc)[16], const P2 *a0, const P2 *b0, const P2 *a1,
                                           const P2 *b1, int la, int lb);

__device__ __forceinline__ void block_abt(double (&acc)[16], const double2 *a, int la, const double2 *b, int lb)
{
    double2 A[8], B[8];
#pragma unroll
    for (int p = 0; p < 8; p++) {
        A[p] = a[(size_t)p * la];
        B[p] = __ldg(b + (size_t)p * lb);
    }
#pragma unroll
    for (int r = 0; r < 4; r++)
#pragma unroll
        for (int c = 0; c < 4; c++) {
            double v = acc[4 * r + c];
            v = fma(A[2 * r].x, B[2 * c].x, v);
            v = fma(A[2 * r].y, B[2 * c].y, v);
            v = fma(A[2 * r + 1].x, B[2 * c + 1].x, v);
            v = fma(A[2 * r + 1].y, B[2 * c + 1].y, v);
            acc[4 * r + c] = v;
        }
}

template <>
__device__ __forceinline__ void block_abt2(float2 (&acc)[16], const float2 *a0, const float2 *b0, const float2 *a1,
                                           const float2 *b1, int la, int lb)
{
    float2 A[8], B[8], C[8], D[8];
#pragma unroll
    for (int p = 0; p < 8; p++) {
        A[p] = a0[(size_t)p * la];
        B[p] = __ldg(b0 + (size_t)p * lb);
        C[p] = a1[(size_t)p * la];
        D[p] = __ldg(b1 + (size_t)p * lb);
    }
#pragma unroll
    for (int r = 0; r < 4; r++)
#pragma unroll
        for (int c = 0; c < 4; c++) {
            acc[4 * r + c] = __ffma2_rn(A[2 * r], B[2 * c], acc[4 * r + c]);
            acc[4 * r + c] = __ffma2_rn(A[2 * r + 1], B[2 * c + 1], acc[4 * r + c]);
            acc[4 * r + c] = __ffma2_rn(C[2 * r], D[2 * c], acc[4 * r + c]);
            acc[4 * r + c] = __ffma2_rn(C[2 * r + 1], D[2 * c + 1], acc[4 * r + c]);
        }
}

template <>
__device__ __forceinline__ void block_abt2(double (&acc)[16], const double2 *a0, const double2 *b0,
                                           const double2 *a1, const double2 *b1, int la, int lb)
{
    block_abt(acc, a0, la, b0, lb);
    block_abt(acc, a1, la, b1, lb);
}

__device__ __forceinline__ void acc_zero(float2 (&acc)[16])
{
#pragma unroll
    for (int e = 0; e < 16; e++) acc[e] = make_float2(0.f, 0.f);
}
__device__ __forceinline__ void acc_zero(double (&acc)[16])
{
#pragma unroll
    for (int e = 0; e < 16; e++) acc[e] = 0.0;
}
__device__ __forceinline__ void acc_fold(const float2 (&acc)[16], float (&v)[16])
{
#pragma unroll
    for (int e = 0; e < 16; e++) v[e] = acc[e].x + acc[e].y;
}
__device__ __forceinline__ void acc_fold(const double (&acc)[16], double (&v)[16])
{
#pragma unroll
    for (int e = 0; e < 16; e++) v[e] = acc[e];
}

template <typename T>
struct AccOf;
template <>
struct AccOf<float> {
    using type = float2;  // packed accumulator
    using pair = float2;  // element pair of a block plane
};
template <>
struct AccOf<double> {
    using type = double;
    using pair = double2;
};

}  // namespace

// X_0 = (lmax I - H) / (lmax - lmin) on the pattern of H; tr X_0 in FP64.
template <typename T>
__global__ void k_sp2_init(int nb, const int32_t *__restrict__ rowptr,
                           const int32_t *__restrict__ colidx, const int32_t *__restrict__ blkrow,
                           const double *__restrict__ h0, const DevState *__restrict__ gs,
                           int32_t *__restrict__ xptr, int32_t *__restrict__ col, T *__restrict__ blk,
                           Sp2Scalars *sc)
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
        blk[plane_elem(rowptr[I], rowptr[I + 1] - rowptr[I], (int)(t - rowptr[I]), rc)] = (T)v;
        if (rc == 0) col[t] = colidx[t];
        if (colidx[t] == I && r == c) tr = (double)(T)v;
    }
    if (e <= nb) xptr[e] = rowptr[e];
    tr = warp_sum_d(tr);
    if ((threadIdx.x & 31) == 0 && tr != 0.0) atomicAdd(&sc->trX, tr);
}

// Row bitmaps of X (bit K of RB[I] <=> block (I, K) stored) and their
// per-word exclusive prefix counts RP.  One warp per row, the row's bitmap
// assembled in shared memory.
__global__ void k_sp2_rowbits(int nb, int nw, const int32_t *__restrict__ xptr,
                              const int32_t *__restrict__ xcol, uint32_t *__restrict__ RB,
                              int32_t *__restrict__ RP)
{
    extern __shared__ uint32_t sbits[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int I = blockIdx.x * (blockDim.x >> 5) + w;
    if (I >= nb) return;
    uint32_t *b = sbits + (size_t)w * nw;
    for (int i = lane; i < nw; i += 32) b[i] = 0u;
    __syncwarp();
    for (int t = xptr[I] + lane; t < xptr[I + 1]; t += 32) {
        const int J = xcol[t];
        atomicOr(b + (J >> 5), 1u << (J & 31));
    }
    __syncwarp();
    int carry = 0;
    for (int b0 = 0; b0 < nw; b0 += 32) {
        const int i = b0 + lane;
        const uint32_t v = i < nw ? b[i] : 0u;
        const int c = __popc(v);
        const int x = warp_incl_scan(c, lane);
        if (i < nw) {
            RB[(size_t)I * nw + i] = v;
            RP[(size_t)I * nw + i] = carry + x - c;
        }
        carry += __shfl_sync(0xffffffffu, x, 31);
    }
}

// Pattern of row I of X^2 together with X's own row: OB[I] = RB[I] | OR_{K in
// row I} RB[K]; OP its per-word prefix counts, outlen[I] its popcount.  Also
// counts the block products of the full X^2 and the longest row of X.
__global__ void k_sp2_symbolic(int nb, int nw, const int32_t *__restrict__ xptr,
                               const int32_t *__restrict__ xcol, const uint32_t *__restrict__ RB,
                               uint32_t *__restrict__ OB, int32_t *__restrict__ OP,
                               int32_t *__restrict__ outlen, Sp2Scalars *sc)
{
    constexpr int R = 4;  // words per lane and chunk
    const int lane = threadIdx.x & 31;
    const int I = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (I >= nb) return;
    const int s = xptr[I], e = xptr[I + 1];
    int carry = 0;
    for (int c0 = 0; c0 < nw; c0 += 32 * R) {
        uint32_t acc[R];
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int i = c0 + lane + 32 * r;
            acc[r] = i < nw ? RB[(size_t)I * nw + i] : 0u;
        }
        for (int t0 = s; t0 < e; t0 += 32) {
            const int myK = t0 + lane < e ? xcol[t0 + lane] : 0;
            const int nt = min(32, e - t0);
            for (int j = 0; j < nt; j++) {
                const uint32_t *rk = RB + (size_t)__shfl_sync(0xffffffffu, myK, j) * nw;
#pragma unroll
                for (int r = 0; r < R; r++) {
                    const int i = c0 + lane + 32 * r;
                    if (i < nw) acc[r] |= __ldg(rk + i);
                }
            }
        }
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int i = c0 + lane + 32 * r;
            const int c = __popc(acc[r]);
            const int x = warp_incl_scan(c, lane);
            if (i < nw) {
                OB[(size_t)I * nw + i] = acc[r];
                OP[(size_t)I * nw + i] = carry + x - c;
            }
            carry += __shfl_sync(0xffffffffu, x, 31);
        }
    }
    if (lane == 0) {
        outlen[I] = carry;
        long long full = 0;
        for (int t = s; t < e; t++) {
            const int K = xcol[t];
            full += xptr[K + 1] - xptr[K];
        }
        atomicAdd(&sc->full_products, (unsigned long long)full);
        atomicMax(&sc->maxlen, e - s);
    }
}

// Exclusive scan of n counts into ptr[0..n] (one CTA); the total goes to
// *total as a 64-bit count (checked on the host before use as int32).
__global__ void __launch_bounds__(1024) k_sp2_scan(int n, const int32_t *__restrict__ in,
                                                   int32_t *__restrict__ ptr,
                                                   unsigned long long *total)
{
    __shared__ long long wsum[32];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int per = (n + 1023) / 1024;
    const int b0 = tid * per;
    long long loc = 0;
    for (int i = b0; i < min(n, b0 + per); i++) loc += in[i];
    long long x = loc;
    for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {
        long long t = wsum[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        wsum[lane] = t;
    }
    __syncthreads();
    long long run = (w > 0 ? wsum[w - 1] : 0) + x - loc;
    for (int i = b0; i < min(n, b0 + per); i++) {
        ptr[i] = (int32_t)run;
        run += in[i];
    }
    if (tid == 1023) {
        ptr[n] = (int32_t)wsum[31];
        *total = (unsigned long long)wsum[31];
    }
}

// The numeric step: one CTA per output block row I (grid-stride, heavy rows
// first), one warp per output block (I, J), J >= I.  The warp ANDs the
// bitmap words of rows I and J, 32 words at a time (one per lane), and each
// lane expands its word's common bits into list entries (positions of K in
// rows I and J, from the prefix counts) at its scanned offset; every 32
// entries each lane forms one block product.  Writes the new block
// (X^2 or 2X - X^2) at (I, J) and its transpose at (J, I) of the uncompacted
// output (row pointers optr over the pattern OB), the keep flag of both, and
// counts kept blocks per row.
template <typename T>
__global__ void __launch_bounds__(32 * kNumWarps)
    k_sp2_numeric(int nb, int nw, const int32_t *__restrict__ xptr, const int32_t *__restrict__ xcol,
                  const T *__restrict__ xblk, const uint32_t *__restrict__ RB,
                  const int32_t *__restrict__ RP, const uint32_t *__restrict__ OB,
                  const int32_t *__restrict__ OP, const int32_t *__restrict__ optr, int branch,
                  double drop2, int a_cap, int l_cap, int32_t *__restrict__ ocol, T *__restrict__ oblk,
                  uint8_t *__restrict__ okeep, long long out_cap, int32_t *__restrict__ kept,
                  Sp2Scalars *sc)
{
    using Acc = typename AccOf<T>::type;
    using P2 = typename AccOf<T>::pair;
    extern __shared__ __align__(16) unsigned char smraw[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    T *sA = reinterpret_cast<T *>(smraw);                                   // a_cap x 16 (planes)
    uint32_t *sRB = reinterpret_cast<uint32_t *>(sA + (size_t)a_cap * 16); // nw
    int32_t *sRP = reinterpret_cast<int32_t *>(sRB + nw);                  // nw
    uint32_t *sOB = reinterpret_cast<uint32_t *>(sRP + nw);                // nw
    int32_t *sOP = reinterpret_cast<int32_t *>(sOB + nw);                  // nw
    // per warp: row J's blocks of two product rounds (2 x 32 entries x 8
    // pairs, [pair][entry]), the intersection list (l_cap), its J items
    // (kJCap)
    const size_t wbase = ((size_t)a_cap * 16 * sizeof(T) + 16 * (size_t)nw + 15) & ~(size_t)15;
    const size_t wstride = (512 * sizeof(P2) + 4 * ((size_t)l_cap + kJCap) + 15) & ~(size_t)15;
    P2 *wB = reinterpret_cast<P2 *>(smraw + wbase + (size_t)w * wstride);
    uint32_t *list = reinterpret_cast<uint32_t *>(wB + 512);
    int32_t *jl = reinterpret_cast<int32_t *>(list + l_cap);               // kJCap
    const int e = (lane >> 1) & 15, er = e >> 2, ec = e & 3;  // the element this lane ends with
    const float drop2f = (float)drop2;
    double trX2 = 0.0, idem2 = 0.0, trNew = 0.0;
    float ih = 0.f, il = 0.f;
    unsigned long long prods = 0;
    for (int I = blockIdx.x; I < nb; I += gridDim.x) {
        const int ri = xptr[I], li = xptr[I + 1] - ri;
        const bool staged = li <= a_cap;
        __syncthreads();  // the previous row's readers are done
        if (staged) {
            const int4 *src = reinterpret_cast<const int4 *>(xblk + (size_t)ri * 16);
            int4 *dst = reinterpret_cast<int4 *>(sA);
            const int n16 = li * (int)sizeof(T);  // li blocks x 16 elements / 16 bytes
            for (int i = threadIdx.x; i < n16; i += blockDim.x) dst[i] = __ldg(src + i);
        }
        for (int i = threadIdx.x; i < nw; i += blockDim.x) {
            sRB[i] = RB[(size_t)I * nw + i];
            sRP[i] = RP[(size_t)I * nw + i];
            sOB[i] = OB[(size_t)I * nw + i];
            sOP[i] = OP[(size_t)I * nw + i];
        }
        __syncthreads();
        const P2 *Ab = reinterpret_cast<const P2 *>(staged ? sA : xblk + (size_t)ri * 16);
        const T *At = reinterpret_cast<const T *>(Ab);
        const int obase = optr[I];
        // the output columns J >= I of row I, item k to warp k % kNumWarps
        int item0 = 0;
        for (int c0 = I >> 5; c0 < nw; c0 += 32) {
            const int wi = c0 + lane;
            uint32_t bits = wi < nw ? sOB[wi] : 0u;
            if (wi == (I >> 5)) bits &= ~((1u << (I & 31)) - 1u);
            const int cnt = __popc(bits);
            const int incl = warp_incl_scan(cnt, lane);
            const int tot = __shfl_sync(0xffffffffu, incl, 31);
            int k = item0 + incl - cnt;  // global index of this lane's first item
            auto owned_below = [&](int idx) {  // items i < idx with i % kNumWarps == w
                return idx <= w ? 0 : (idx - w + kNumWarps - 1) / kNumWarps;
            };
            int pos = owned_below(k) - owned_below(item0);
            while (bits) {
                const int b = __ffs(bits) - 1;
                bits &= bits - 1u;
                if (k % kNumWarps == w) jl[pos++] = wi * 32 + b;
                k++;
            }
            const int mine = owned_below(item0 + tot) - owned_below(item0);
            item0 += tot;
            __syncwarp();
            for (int jj = 0; jj < mine; jj++) {
                const int J = jl[jj];
                const int rj = xptr[J], lj = xptr[J + 1] - rj;
                const P2 *Bb = reinterpret_cast<const P2 *>(xblk + (size_t)rj * 16);
                const uint32_t *RBJ = RB + (size_t)J * nw;
                const int32_t *RPJ = RP + (size_t)J * nw;
                Acc acc[16];
                acc_zero(acc);
                unsigned long long nprod = 0;
                // segments of whole bitmap words whose intersection fits the list:
                // all of them when row I is staged (the intersection is at most
                // li <= l_cap entries), else l_cap / 32 words (<= l_cap entries)
                const int W = staged ? nw : max(1, l_cap >> 5);
                for (int w0 = 0; w0 < nw; w0 += W) {
                    // the K held by both rows: AND of their bitmap words; each
                    // lane expands its word's bits into (position in row I,
                    // position in row J) entries at its prefix offset, so the
                    // list runs in increasing K as row I's columns do
                    int cnt_l = 0;
                    const int wend = min(nw, w0 + W);
                    for (int c0 = w0; c0 < wend; c0 += 32) {
                        const int wi = c0 + lane;
                        const uint32_t bI = wi < wend ? sRB[wi] : 0u;
                        const uint32_t bJ = wi < wend ? __ldg(RBJ + wi) : 0u;
                        uint32_t both = bI & bJ;
                        const int pI = both ? sRP[wi] : 0, pJ = both ? __ldg(RPJ + wi) : 0;
                        const int c = __popc(both);
                        const int incl = warp_incl_scan(c, lane);
                        int o = cnt_l + incl - c;
                        while (both) {
                            const uint32_t below = (both & (0u - both)) - 1u;  // bits under the lowest set bit
                            both &= both - 1u;
                            list[o++] = ((uint32_t)(pI + __popc(bI & below)) << 16) |
                                        (uint32_t)(pJ + __popc(bJ & below));
                        }
                        cnt_l += __shfl_sync(0xffffffffu, incl, 31);
                    }
                    __syncwarp();
                    // the block products: 32 entries per round, each lane's B block
                    // copied into this warp's double buffer one round ahead
                    const int rounds = (cnt_l + 31) >> 5;
                    auto stage = [&](int rd) {
                        const int q = rd * 32 + lane;
                        if (q < cnt_l) {
                            const P2 *src = Bb + (list[q] & 0xffffu);
                            P2 *dst = wB + (rd & 1) * 256 + lane;
#pragma unroll
                            for (int pp = 0; pp < 8; pp++) cp_async<sizeof(P2)>(dst + 32 * pp, src + (size_t)pp * lj);
                        }
                        cp_async_commit();
                    };
                    if (rounds > 0) stage(0);
                    for (int rd = 0; rd < rounds; rd++) {
                        if (rd + 1 < rounds) {
                            stage(rd + 1);
                            cp_async_wait<1>();
                        } else {
                            cp_async_wait<0>();
                        }
                        __syncwarp();
                        const int q = rd * 32 + lane;
                        if (q < cnt_l) block_abt_s(acc, Ab + (list[q] >> 16), li, wB + (rd & 1) * 256 + lane);
                        __syncwarp();
                    }
                    nprod += (unsigned long long)cnt_l;
                    __syncwarp();
                }
                T v[16];
                acc_fold(acc, v);
                const T x2 = warp_reduce16(v, lane);
                // old block X_IJ
                const uint32_t wI = sRB[J >> 5], bitJ = 1u << (J & 31);
                const T xo = (wI & bitJ)
                                 ? At[2 * ((size_t)(e >> 1) * li + sRP[J >> 5] + __popc(wI & (bitJ - 1u))) + (e & 1)]
                                 : T(0);
                const T nv = branch < 0 ? x2 : T(2) * xo - x2;
                // Frobenius norm of the new block: even lanes hold the 16 elements
                float nrm;
                if constexpr (sizeof(T) == 4)
                    nrm = (lane & 1) ? 0.f : nv * nv;
                else
                    nrm = (lane & 1) ? 0.f : (float)((double)nv * (double)nv);
                for (int o = 16; o > 0; o >>= 1) nrm += __shfl_xor_sync(0xffffffffu, nrm, o);
                const bool kp = nrm >= drop2f;
                if (!(lane & 1)) {
                    const T dl = x2 - xo;
                    if constexpr (sizeof(T) == 4) {
                        pair_add(ih, il, (J == I ? 1.f : 2.f) * dl * dl);
                    } else {
                        idem2 += (J == I ? 1.0 : 2.0) * (double)dl * (double)dl;
                    }
                    if (J == I && er == ec) {
                        trX2 += (double)x2;
                        if (kp) trNew += (double)nv;
                    }
                }
                // (I, J): its slot in row I of the output
                const uint32_t wo = sOB[J >> 5];
                const long long sIJ = (long long)obase + sOP[J >> 5] + __popc(wo & (bitJ - 1u));
                // (J, I): its slot in row J (the pattern is symmetric; checked)
                long long sJI = -1;
                if (J != I) {
                    const uint32_t woJ = __ldg(OB + (size_t)J * nw + (I >> 5)), bitI = 1u << (I & 31);
                    if (woJ & bitI)
                        sJI = (long long)optr[J] + __ldg(OP + (size_t)J * nw + (I >> 5)) + __popc(woJ & (bitI - 1u));
                    else if (lane == 0)
                        sc->overflow = 2;
                }
                if (sIJ < out_cap && sJI < out_cap) {
                    if (!(lane & 1)) oblk[(size_t)sIJ * 16 + e] = nv;
                    if (lane == 0) {
                        ocol[sIJ] = J;
                        okeep[sIJ] = kp;
                    }
                    if (sJI >= 0) {
                        if (lane & 1) oblk[(size_t)sJI * 16 + ec * 4 + er] = nv;
                        if (lane == 1) {
                            ocol[sJI] = I;
                            okeep[sJI] = kp;
                        }
                    }
                } else if (lane == 0) {
                    sc->overflow = 1;
                }
                if (kp && lane == 0) {
                    atomicAdd(kept + I, 1);
                    if (sJI >= 0) atomicAdd(kept + J, 1);
                }
                prods += (lane == 0) ? nprod : 0ull;
            }
            __syncwarp();
        }
    }
    idem2 += (double)ih + (double)il;
    trX2 = warp_sum_d(trX2);
    idem2 = warp_sum_d(idem2);
    trNew = warp_sum_d(trNew);
    prods = warp_sum_u64(prods);
    if (lane == 0) {
        if (trX2 != 0.0) atomicAdd(&sc->trX2, trX2);
        if (idem2 != 0.0) atomicAdd(&sc->idem2, idem2);
        if (trNew != 0.0) atomicAdd(&sc->trNew, trNew);
        if (prods) atomicAdd(&sc->products, prods);
    }
}

// The kept blocks of the uncompacted output (block-major), in column order,
// into the next X in its pair planes (row pointers nptr from a scan of the
// kept counts).  One warp per row.
template <typename T>
__global__ void k_sp2_compact(int nb, const int32_t *__restrict__ optr, const int32_t *__restrict__ ocol,
                              const T *__restrict__ oblk, const uint8_t *__restrict__ okeep,
                              const int32_t *__restrict__ nptr, int32_t *__restrict__ ncol,
                              T *__restrict__ nblk)
{
    using P2 = typename AccOf<T>::pair;
    const int lane = threadIdx.x & 31;
    const int I = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (I >= nb) return;
    const int s = nptr[I], L = nptr[I + 1] - s;
    const P2 *ob2 = reinterpret_cast<const P2 *>(oblk);
    P2 *nb2 = reinterpret_cast<P2 *>(nblk) + (size_t)s * 8;
    int dst = 0;
    for (int t0 = optr[I]; t0 < optr[I + 1]; t0 += 32) {
        const int t = t0 + lane;
        const bool k = t < optr[I + 1] && okeep[t];
        const uint32_t bal = __ballot_sync(0xffffffffu, k);
        if (k) {
            const int o = dst + __popc(bal & ((1u << lane) - 1u));
            ncol[s + o] = ocol[t];
#pragma unroll
            for (int p = 0; p < 8; p++) nb2[(size_t)p * L + o] = ob2[(size_t)t * 8 + p];
        }
        dst += __popc(bal);
    }
}

// diag P, q_a = 2 sum P_ii, and sum_{blocks} X_IJ . H_IJ (= tr(X H) for symmetric H).
template <typename T>
__global__ void k_sp2_outputs(int nb, const int32_t *__restrict__ rowptr,
                              const int32_t *__restrict__ colidx, const int32_t *__restrict__ blkrow,
                              const double *__restrict__ h0, const int32_t *__restrict__ xptr,
                              const int32_t *__restrict__ col, const T *__restrict__ blk,
                              double *__restrict__ diagP, double *__restrict__ q, Sp2Scalars *sc)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nnzb = rowptr[nb];
    double xh = 0.0;
    if (t < nnzb) {
        const int I = blkrow[t], J = colidx[t];
        const int xi = find_col<T>(col, xptr[I], xptr[I + 1], J);
        const int L = xptr[I + 1] - xptr[I];
        if (xi >= 0)
            for (int e = 0; e < 16; e++)
                xh += (double)blk[plane_elem(xptr[I], L, xi - xptr[I], e)] * h0[t * 16 + e];
    }
    if (t < nb) {
        const int I = (int)t;
        const int xi = find_col<T>(col, xptr[I], xptr[I + 1], I);
        const int L = xptr[I + 1] - xptr[I];
        double s = 0.0;
        for (int r = 0; r < 4; r++) {
            const double v = xi >= 0 ? (double)blk[plane_elem(xptr[I], L, xi - xptr[I], 5 * r)] : 0.0;
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

struct Sp2Csr {
    int32_t *ptr = nullptr, *col = nullptr;
    void *blk = nullptr;
    long long cap = 0;
};

void csr_free(Sp2Csr &b)
{
    if (b.ptr) cudaFree(b.ptr);
    if (b.col) cudaFree(b.col);
    if (b.blk) cudaFree(b.blk);
    b = Sp2Csr{};
}

cudaError_t csr_reserve(Sp2Csr &b, int nb, long long cap, size_t es)
{
    cudaError_t e = cudaSuccess;
    if (!b.ptr && (e = cudaMalloc(&b.ptr, sizeof(int32_t) * (nb + 1)))) return e;
    if (cap > b.cap) {
        if (b.col) cudaFree(b.col);
        if (b.blk) cudaFree(b.blk);
        b.col = nullptr;
        b.blk = nullptr;
        cap = std::max<long long>(cap, 1);
        if ((e = cudaMalloc(&b.col, sizeof(int32_t) * cap))) return e;
        if ((e = cudaMalloc(&b.blk, es * 16 * cap))) return e;
        b.cap = cap;
    }
    return cudaSuccess;
}

// Shared memory of k_sp2_numeric for a staging capacity of a_cap blocks of
// row I and per-warp intersection lists of l_cap entries.
size_t numeric_smem(int a_cap, int l_cap, int nw, size_t es)
{
    // the kernel's own layout: staged row, four bitmaps, then per-warp areas
    const size_t base = ((size_t)a_cap * 16 * es + 16 * (size_t)nw + 15) & ~(size_t)15;
    const size_t stride = (512 * 2 * es + 4 * ((size_t)l_cap + kJCap) + 15) & ~(size_t)15;
    return base + (size_t)kNumWarps * stride;
}

template <typename T>
int sp2_run(tb_ctx *ctx, double *diagP_h, double *q_h, double *e_band, tb_report *rep,
            std::vector<int> &branches)
{
    DevMatrix &m = ctx->m;
    cudaStream_t st = ctx->stream;
    const int nb = m.nb;
    const int nw = (nb + 31) / 32;
    const double ne = ctx->p.n_electrons;
    const double drop2 = ctx->p.sp2_drop_tol * ctx->p.sp2_drop_tol;
    Sp2Csr X, N;  // current and next X
    int32_t *optr = nullptr, *ocol = nullptr, *outlen = nullptr, *kept = nullptr, *RP = nullptr, *OP = nullptr;
    uint32_t *RB = nullptr, *OB = nullptr;
    T *oblk = nullptr;
    uint8_t *okeep = nullptr;
    long long ocap = 0;
    Sp2Scalars *sc = nullptr;
    DevState *gs = nullptr;
    double *d_diag = nullptr, *d_q = nullptr;
    int rc = TB_OK;
    auto cuda_fail = [&](cudaError_t e, const char *what) {
        ctx->err = std::string(what) + ": " + cudaGetErrorString(e);
        rc = e == cudaErrorMemoryAllocation ? TB_ERR_OUT_OF_MEMORY : TB_ERR_CUDA;
    };
    cudaError_t e;
    Sp2Scalars hs;
    int64_t launches = 0;
    double full_products = 0.0, done_products = 0.0, moved = 0.0;
    int64_t cur_nnzb = 0;
    int it = 0;
    double idem = INFINITY, prev1 = INFINITY, prev2 = INFINITY, trX = 0.0;
    int nsm = 152;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device);
    int dev_smem = 0;
    cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
    const int rb_warps = 8;
    const size_t rb_smem = (size_t)rb_warps * nw * 4;
    if (nb > 65535) {  // the intersection list packs two 16-bit row positions
        ctx->err = "SP2 supports at most 65535 block rows";
        return TB_ERR_UNSUPPORTED;
    }
    if (rb_smem > (size_t)dev_smem || numeric_smem(0, 64, nw, sizeof(T)) > (size_t)dev_smem) {
        ctx->err = "SP2 row bitmaps exceed shared memory";
        return TB_ERR_UNSUPPORTED;
    }
    if ((e = cudaFuncSetAttribute(k_sp2_numeric<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  smem_optin_max((const void *)k_sp2_numeric<T>))) ||
        (e = cudaFuncSetAttribute(k_sp2_rowbits, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  smem_optin_max((const void *)k_sp2_rowbits)))) {
        cuda_fail(e, "cudaFuncSetAttribute(sp2)");
        return rc;
    }
    if ((e = cudaMalloc(&sc, sizeof(Sp2Scalars))) || (e = cudaMalloc(&gs, sizeof(DevState))) ||
        (e = cudaMalloc(&d_diag, sizeof(double) * m.n)) || (e = cudaMalloc(&d_q, sizeof(double) * nb)) ||
        (e = cudaMalloc(&optr, sizeof(int32_t) * (nb + 1))) || (e = cudaMalloc(&outlen, sizeof(int32_t) * nb)) ||
        (e = cudaMalloc(&kept, sizeof(int32_t) * nb)) ||
        (e = cudaMalloc(&RB, sizeof(uint32_t) * (size_t)nb * nw)) ||
        (e = cudaMalloc(&RP, sizeof(int32_t) * (size_t)nb * nw)) ||
        (e = cudaMalloc(&OB, sizeof(uint32_t) * (size_t)nb * nw)) ||
        (e = cudaMalloc(&OP, sizeof(int32_t) * (size_t)nb * nw))) {
        cuda_fail(e, "cudaMalloc(sp2 scratch)");
        goto done;
    }
    // Gershgorin bounds of H (no shift) and X_0
    launch_gershgorin(st, m, nullptr, 0.0, 0.0, 2, 1 << 22, gs);
    if ((e = csr_reserve(X, nb, m.nnzb, sizeof(T))) || (e = csr_reserve(N, nb, 1, sizeof(T)))) {
        cuda_fail(e, "cudaMalloc(sp2 X)");
        goto done;
    }
    cudaMemsetAsync(sc, 0, sizeof(Sp2Scalars), st);
    {
        const int64_t tot = std::max<int64_t>(m.nnzb * 16, nb + 1);
        k_sp2_init<T><<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(nb, m.rowptr, m.colidx, m.blkrow, m.h0,
                                                                      gs, X.ptr, X.col, (T *)X.blk, sc);
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
        // pattern of X^2 and the output's row pointers
        cudaMemsetAsync(sc, 0, sizeof(Sp2Scalars), st);
        k_sp2_rowbits<<<(nb + rb_warps - 1) / rb_warps, 32 * rb_warps, rb_smem, st>>>(nb, nw, X.ptr, X.col, RB, RP);
        k_sp2_symbolic<<<(nb + 7) / 8, 256, 0, st>>>(nb, nw, X.ptr, X.col, RB, OB, OP, outlen, sc);
        k_sp2_scan<<<1, 1024, 0, st>>>(nb, outlen, optr, &sc->bound);
        launches += 3;
        cudaMemcpyAsync(&hs, sc, sizeof(hs), cudaMemcpyDeviceToHost, st);
        if ((e = cudaStreamSynchronize(st))) {
            cuda_fail(e, "sp2 symbolic");
            goto done;
        }
        if (hs.bound > 0x7fffffffull) {
            ctx->err = "SP2 product pattern exceeds 2^31 blocks";
            rc = TB_ERR_UNSUPPORTED;
            goto done;
        }
        if ((long long)hs.bound > ocap) {
            if (ocol) cudaFree(ocol);
            if (oblk) cudaFree(oblk);
            if (okeep) cudaFree(okeep);
            ocol = nullptr;
            oblk = nullptr;
            okeep = nullptr;
            ocap = (long long)hs.bound;
            if ((e = cudaMalloc(&ocol, sizeof(int32_t) * ocap)) || (e = cudaMalloc(&oblk, sizeof(T) * 16 * ocap)) ||
                (e = cudaMalloc(&okeep, ocap))) {
                cuda_fail(e, "cudaMalloc(sp2 X^2)");
                goto done;
            }
        }
        full_products += (double)hs.full_products;
        const int branch = (2.0 * trX > ne) ? -1 : 1;  // withSP2.cpp:1029-1030
        {
            // stage row I in shared memory and keep whole intersection lists
            // (l_cap = a_cap entries) when both fit: two CTAs per SM if possible
            const size_t per_blk = 16 * sizeof(T) + 4 * kNumWarps;
            const size_t fixed = numeric_smem(0, 0, nw, sizeof(T));
            const size_t half = (size_t)dev_smem / 2 > fixed + 1024 ? (size_t)dev_smem / 2 - fixed - 1024 : 0;
            int a_cap = (int)std::min<size_t>((size_t)hs.maxlen, ((size_t)dev_smem - fixed - 1024) / per_blk);
            if ((size_t)hs.maxlen <= half / per_blk) a_cap = hs.maxlen;
            a_cap = std::max(a_cap, 64);
            const int l_cap = (a_cap + 31) / 32 * 32;
            const size_t smem = numeric_smem(a_cap, l_cap, nw, sizeof(T));
            int per_sm = 1;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sp2_numeric<T>, 32 * kNumWarps, smem);
            const int grid = std::min(nb, nsm * std::max(1, per_sm));
            cudaMemsetAsync(kept, 0, sizeof(int32_t) * nb, st);
            k_sp2_numeric<T><<<grid, 32 * kNumWarps, smem, st>>>(nb, nw, X.ptr, X.col, (const T *)X.blk, RB, RP, OB, OP,
                                                                 optr, branch, drop2, a_cap, l_cap, ocol, oblk, okeep, ocap,
                                                                 kept, sc);
            k_sp2_scan<<<1, 1024, 0, st>>>(nb, kept, N.ptr, &sc->count);  // next X's row pointers
            launches += 3;
        }
        cudaMemcpyAsync(&hs, sc, sizeof(hs), cudaMemcpyDeviceToHost, st);
        if ((e = cudaStreamSynchronize(st))) {
            cuda_fail(e, "sp2 step");
            goto done;
        }
        if (hs.overflow) {
            ctx->err = hs.overflow == 2 ? "SP2: X lost its symmetric pattern" : "SP2 output exceeded its bound";
            rc = TB_ERR_CUDA;
            goto done;
        }
        done_products += (double)hs.products;
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
        if ((e = csr_reserve(N, nb, (long long)hs.count, sizeof(T)))) {
            cuda_fail(e, "cudaMalloc(sp2 X_next)");
            goto done;
        }
        k_sp2_compact<T><<<(nb + 7) / 8, 256, 0, st>>>(nb, optr, ocol, oblk, okeep, N.ptr, N.col, (T *)N.blk);
        launches++;
        std::swap(X, N);
        cur_nnzb = (int64_t)hs.count;
        trX = hs.trNew;
        prev2 = prev1;
        prev1 = idem;
    }
    // outputs from X_it
    cudaMemsetAsync(sc, 0, sizeof(Sp2Scalars), st);
    {
        const int64_t tot = std::max<int64_t>(m.nnzb, nb);
        k_sp2_outputs<T><<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(nb, m.rowptr, m.colidx, m.blkrow, m.h0,
                                                                         X.ptr, X.col, (const T *)X.blk, d_diag,
                                                                         d_q, sc);
        launches++;
    }
    {
        cudaMemcpyAsync(&hs, sc, sizeof(hs), cudaMemcpyDeviceToHost, st);
        if (diagP_h) cudaMemcpyAsync(diagP_h, d_diag, sizeof(double) * m.n, cudaMemcpyDeviceToHost, st);
        if (q_h) cudaMemcpyAsync(q_h, d_q, sizeof(double) * nb, cudaMemcpyDeviceToHost, st);
        if ((e = cudaStreamSynchronize(st))) {
            cuda_fail(e, "sp2 outputs");
            goto done;
        }
        if (e_band) *e_band = 2.0 * hs.trX;
        if (rep) {
            rep->e_band = 2.0 * hs.trX;
            rep->idem_err = idem;
            rep->sp2_iters = it;
            rep->sp2_nnzb = cur_nnzb;
            rep->sp2_flops = 128.0 * full_products;
            rep->sp2_flops_done = 128.0 * done_products;
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
    csr_free(X);
    csr_free(N);
    for (void *p : {(void *)optr, (void *)ocol, (void *)outlen, (void *)kept, (void *)RP, (void *)OP, (void *)RB,
                    (void *)OB, (void *)oblk, (void *)okeep, (void *)sc, (void *)gs, (void *)d_diag, (void *)d_q})
        if (p) cudaFree(p);
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

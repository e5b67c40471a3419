// tb_kpe.cu -- sm_103a kernels of the exact-trace KPE density-matrix path.
//
// Layout in HBM (n orbitals, nb = n/4 block rows, nnzb stored 4x4 blocks):
//   BSR: rowptr[nb+1], colidx[nnzb], blocks [nnzb][4][4] row-major (FP64 H0,
//   FP32 or FP64 scaled X).  Slab vectors T_k: [n][B] row-major, the B
//   identity columns of one slab contiguous per row, so a warp reads a
//   4-row x 128-column tile of T_k as 4 coalesced 512-byte rows (FP32:
//   one float4 per lane per row; FP64: one double2 per lane per row over 64
//   columns).  Diagonal moments d[k][i] = [T_k(X)]_ii, FP64, moment-major.
//
// Kernel map to the reference (withSP2_deltaH.cpp):
//   k_gershgorin        GershGorinParallel 144-209 + the a/b of runKPM 1548-1560
//   k_build_x           MatShift(-b)/MatScale(1/a) of runKPM 1559-1560, with the
//                       SCC diagonal shift of constructdeltaH 1443-1459
//   k_cheb_f64          getKPE recurrence 1134-1168 on identity column slabs with
//                       the unit-vector diagonal extraction of 1361-1379
//   k_cheb_f32*         same recurrence in FP32 to order M/2; moments from
//                       T_{2k} = 2 T_k^2 - I and T_{2k+1} = 2 T_k T_{k+1} - X
//                       (column dot products as FP32 TwoSum pairs; the
//                       pipelined form is in tb_pipe.cu)
//   k_moment_sums ..    tr T_k, damped DOS, mu bisection: runKPM 1579-1712
//   k_fermi_coeffs      getKPE coefficients 1100-1103 (Fermi instead of step)
//   k_charges           computeDiagonalElements 1375-1385 (diagP, orbital2Atom)
//   k_scc_update        constructdeltaH 1424-1429 + the SCC loop 1820-1840
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include "tb_f32x2.cuh"
#include "tb_internal.h"

namespace tb {

namespace {

constexpr double kPi = 3.141592653589793238463;

__device__ __forceinline__ double warp_sum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_min(double v)
{
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double warp_max(double v)
{
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Sum over a block of up to 1024 threads; result valid in every thread.
__device__ double block_sum(double v, double *sh)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double t = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
    if (w == 0) t = warp_sum(t);
    if (threadIdx.x == 0) sh[0] = t;
    __syncthreads();
    double r = sh[0];
    __syncthreads();
    return r;
}

// Above this beta_x the multisection evaluates the Fermi function node by node;
// below it e^{beta x} e^{-beta mu} stays far inside the FP64 range (|t| <= 600).
constexpr double kEtabBeta = 300.0;

__device__ __forceinline__ double fermi(double x, double mu_x, double beta_x)
{
    const double t = beta_x * (x - mu_x);
    if (t > 0) {
        const double e = exp(-t);
        return e / (1.0 + e);
    }
    return 1.0 / (1.0 + exp(t));
}

}  // namespace

// ---------------------------------------------------------------------------
// Coulomb shift V = Gamma (q - q0), orbital shift = V of the owning atom.
// ---------------------------------------------------------------------------
__global__ void k_coulomb_shift(int natoms, const int32_t *__restrict__ rp,
                                const int32_t *__restrict__ ci, const double *__restrict__ gv,
                                const double *__restrict__ q, const double *__restrict__ q0,
                                double *__restrict__ V, double *__restrict__ shift)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= natoms) return;
    double s = 0.0;
    for (int k = rp[a]; k < rp[a + 1]; k++) {
        const int b = ci[k];
        s += gv[k] * (q[b] - q0[b]);
    }
    if (V) V[a] = s;
    if (shift) {
        shift[4 * a + 0] = s;
        shift[4 * a + 1] = s;
        shift[4 * a + 2] = s;
        shift[4 * a + 3] = s;
    }
}

void launch_coulomb_shift(cudaStream_t st, const DevScc &s, const double *q, double *V,
                          double *shift)
{
    const int T = 256;
    k_coulomb_shift<<<(s.natoms + T - 1) / T, T, 0, st>>>(s.natoms, s.rowptr, s.colidx, s.val, q,
                                                         s.q0, V, shift);
}

// ---------------------------------------------------------------------------
// Gershgorin bounds of H0 + diag(shift) and the scaling X = (H - b)/a; with
// fix_hi > fix_lo the caller's interval [fix_lo, fix_hi] sets a and b instead
// (runKPM's refined a, b of withSP2_deltaH.cpp:1696-1703), unpadded.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_gershgorin(int n, const double *__restrict__ h0diag,
                                                     const double *__restrict__ radius,
                                                     const double *__restrict__ shift,
                                                     double pad, double kT, int M, int nq_cap,
                                                     double fix_lo, double fix_hi, DevState *st)
{
    __shared__ double smin[32], smax[32];
    double mn = INFINITY, mx = -INFINITY;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double c = h0diag[i] + (shift ? shift[i] : 0.0);
        mn = fmin(mn, c - radius[i]);
        mx = fmax(mx, c + radius[i]);
    }
    mn = warp_min(mn);
    mx = warp_max(mx);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        smin[w] = mn;
        smax[w] = mx;
    }
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        mn = lane < nw ? smin[lane] : INFINITY;
        mx = lane < nw ? smax[lane] : -INFINITY;
        mn = warp_min(mn);
        mx = warp_max(mx);
        if (lane == 0) {
            st->lmin = mn;
            st->lmax = mx;
            const bool fixed = fix_hi > fix_lo;
            const double half = fixed ? 0.5 * (fix_hi - fix_lo) : 0.5 * (mx - mn);
            const double a = fixed ? half : half * (1.0 + pad);
            st->a = a;
            st->b = fixed ? 0.5 * (fix_hi + fix_lo) : 0.5 * (mx + mn);
            st->status = (a > 0 && isfinite(a)) ? 0 : TB_ERR_SPECTRUM;
            st->beta_x = kT > 0 ? a / kT : 0.0;
            // quadrature size rule shared with the oracle: next power of two
            // >= max(4M, 13 beta_x, 256)
            double need = 4.0 * M;
            if (st->beta_x > 0 && 13.0 * st->beta_x > need) need = 13.0 * st->beta_x;
            if (need < 256) need = 256;
            int nq = 256;
            while (nq < need && nq < (1 << 22)) nq *= 2;
            if (nq > nq_cap) st->status = TB_ERR_SPECTRUM;
            st->nq = nq > nq_cap ? nq_cap : nq;
            st->bisect_done = 0;
            st->bisect_rounds = 0;
            st->lo = -1.0;
            st->hi = 1.0;
            st->converged = 0;
            st->ticket = 0u;
        }
    }
}

void launch_gershgorin(cudaStream_t st, const DevMatrix &m, const double *shift, double pad,
                            double kT, int M, int nq_cap, DevState *state, double fix_lo, double fix_hi)
{
    k_gershgorin<<<1, 1024, 0, st>>>(m.n, m.h0diag, m.radius, shift, pad, kT, M, nq_cap, fix_lo, fix_hi,
                                     state);
}

// ---------------------------------------------------------------------------
// X = (H0 + diag(shift) - b I) / a on the stored blocks.
// ---------------------------------------------------------------------------
__global__ void k_build_x(int64_t nnzb, const int32_t *__restrict__ blkrow,
                          const int32_t *__restrict__ colidx, const double *__restrict__ h0,
                          const double *__restrict__ shift, const DevState *__restrict__ st,
                          float *__restrict__ x32, double *__restrict__ x64,
                          float *__restrict__ xdiag32)
{
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nnzb * 16) return;
    const int64_t t = e >> 4;
    const int rc = (int)(e & 15), r = rc >> 2, c = rc & 3;
    const double a = st->a, b = st->b;
    double v = h0[e];
    const int I = blkrow[t];
    const bool diag = (colidx[t] == I) && (r == c);
    if (diag) v = v + (shift ? shift[4 * I + r] : 0.0) - b;
    v = v / a;
    if (x64) x64[e] = v;
    if (x32) {
        x32[e] = (float)v;
        if (diag && xdiag32) xdiag32[4 * I + r] = (float)v;
    }
}

// ---------------------------------------------------------------------------
// Identity slab T_0 = E[:, c0:c0+B] (and d[0][i] = 1 for the plain form).
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_slab_identity(T *__restrict__ T0, int n, int B, int c0)
{
    const int64_t tot = (int64_t)n * B;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(e / B), j = (int)(e % B);
        T0[e] = (i == c0 + j) ? T(1) : T(0);
    }
}

// ---------------------------------------------------------------------------
// Plain FP64 Chebyshev step.  Warp = one block row x 64 columns; lane = 2
// columns (double2).  Tout = X Tin (first) or 2 X Tin - Tout (in place over
// T_{k-1}).  The diagonal entry of each slab column is written to d[kout].
// ---------------------------------------------------------------------------
constexpr int kF64Warps = 4;

__global__ void __launch_bounds__(32 * kF64Warps)
    k_cheb_f64(int nb, int n, const int32_t *__restrict__ rowptr,
               const int32_t *__restrict__ colidx, const double *__restrict__ x64,
               const double *__restrict__ Tin, double *__restrict__ Tout, int B, int c0,
               int first, double *__restrict__ d, int kout)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int I = blockIdx.x * kF64Warps + w;
    if (I >= nb) return;
    const int col = blockIdx.y * 64 + lane * 2;
    double acc[4][2];
#pragma unroll
    for (int r = 0; r < 4; r++) acc[r][0] = acc[r][1] = 0.0;
    const int t0 = rowptr[I], t1 = rowptr[I + 1];
    for (int t = t0; t < t1; t++) {
        const int J = __ldg(colidx + t);
        const double2 *xb = reinterpret_cast<const double2 *>(x64 + (int64_t)t * 16);
        double x[16];
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const double2 v = __ldg(xb + q);
            x[2 * q] = v.x;
            x[2 * q + 1] = v.y;
        }
        double2 tv[4];
#pragma unroll
        for (int m = 0; m < 4; m++)
            tv[m] = __ldg(reinterpret_cast<const double2 *>(Tin + (int64_t)(4 * J + m) * B + col));
#pragma unroll
        for (int r = 0; r < 4; r++)
#pragma unroll
            for (int m = 0; m < 4; m++) {
                acc[r][0] = fma(x[4 * r + m], tv[m].x, acc[r][0]);
                acc[r][1] = fma(x[4 * r + m], tv[m].y, acc[r][1]);
            }
    }
#pragma unroll
    for (int r = 0; r < 4; r++) {
        double2 *dst = reinterpret_cast<double2 *>(Tout + (int64_t)(4 * I + r) * B + col);
        double2 o;
        if (first) {
            o.x = acc[r][0];
            o.y = acc[r][1];
        } else {
            const double2 p = *dst;
            o.x = 2.0 * acc[r][0] - p.x;
            o.y = 2.0 * acc[r][1] - p.y;
        }
        *dst = o;
        const int i = 4 * I + r;
        const int j = i - c0 - col;  // column offset inside this lane's pair
        if (j == 0) d[(int64_t)kout * n + i] = o.x;
        if (j == 1) d[(int64_t)kout * n + i] = o.y;
    }
}

void launch_slab_identity(cudaStream_t st, void *T0, int n, int B, int c0, int precision)
{
    const int T = 256;
    int64_t tot = (int64_t)n * B;
    int blocks = (int)((tot + T - 1) / T);
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (precision == TB_PREC_FP64)
        k_slab_identity<double><<<blocks, T, 0, st>>>((double *)T0, n, B, c0);
    else
        k_slab_identity<float><<<blocks, T, 0, st>>>((float *)T0, n, B, c0);
}

__global__ void k_diag_one(double *d, int n, int c0, int B)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < B && c0 + j < n) d[c0 + j] = 1.0;
}

void launch_cheb_step_f64(cudaStream_t st, const DevMatrix &m, const double *Tin, double *Tout,
                          int B, int c0, int first, double *d, int kout)
{
    if (first) k_diag_one<<<(B + 127) / 128, 128, 0, st>>>(d, m.n, c0, B);
    dim3 grid((m.nb + kF64Warps - 1) / kF64Warps, B / 64);
    k_cheb_f64<<<grid, 32 * kF64Warps, 0, st>>>(m.nb, m.n, m.rowptr, m.colidx, m.x64, Tin, Tout,
                                                B, c0, first, d, kout);
}

// The FP32 step kernels accumulate their column dot products as FP32 TwoSum
// pairs (pair_add, tb_f32x2.cuh) across block rows and warps and write
// (hi, lo) pairs.

// ---------------------------------------------------------------------------
// FP32 Chebyshev step with fused column dot products.
// CTA = 8 warps sharing one 128-column chunk; warp w handles kRowsPerWarp
// consecutive block rows; lane = 4 columns (float4).  For every column j the
// CTA accumulates  <T_k, T_k>  and  <T_k, T_{k+1}>  over its rows (FP32 per
// block row, FP32 pairs across block rows and warps) and writes one (hi, lo)
// pair per sum and column to partial_k[rowgroup][B][2].
// ---------------------------------------------------------------------------
constexpr int kF32Warps = 8;
constexpr int kRowsPerWarp = 2;

__global__ void __launch_bounds__(32 * kF32Warps)
    k_cheb_f32(int nb, const int32_t *__restrict__ rowptr, const int32_t *__restrict__ colidx,
               const float *__restrict__ x32, const float *__restrict__ Tin,
               float *__restrict__ Tout, int B, int first, float2 *__restrict__ partial_k)
{
    __shared__ __align__(16) float red[kF32Warps][128][4];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int chunk = blockIdx.y;
    const int col = chunk * 128 + lane * 4;
    const int Ibase = (blockIdx.x * kF32Warps + w) * kRowsPerWarp;
    float hee[4] = {0, 0, 0, 0}, lee[4] = {0, 0, 0, 0}, heo[4] = {0, 0, 0, 0}, leo[4] = {0, 0, 0, 0};
#pragma unroll 1
    for (int rr = 0; rr < kRowsPerWarp; rr++) {
        const int I = Ibase + rr;
        if (I >= nb) break;
        float acc[4][4];
        float own[4][4];
#pragma unroll
        for (int r = 0; r < 4; r++)
#pragma unroll
            for (int c = 0; c < 4; c++) acc[r][c] = 0.f, own[r][c] = 0.f;
        const int t0 = rowptr[I], t1 = rowptr[I + 1];
#pragma unroll 1
        for (int t = t0; t < t1; t++) {
            const int J = __ldg(colidx + t);
            const float4 *xb = reinterpret_cast<const float4 *>(x32 + (int64_t)t * 16);
            float4 xr[4];
#pragma unroll
            for (int q = 0; q < 4; q++) xr[q] = __ldg(xb + q);
            float4 tv[4];
#pragma unroll
            for (int m = 0; m < 4; m++)
                tv[m] = __ldg(reinterpret_cast<const float4 *>(Tin + (int64_t)(4 * J + m) * B + col));
            if (J == I) {
#pragma unroll
                for (int m = 0; m < 4; m++) {
                    own[m][0] = tv[m].x;
                    own[m][1] = tv[m].y;
                    own[m][2] = tv[m].z;
                    own[m][3] = tv[m].w;
                }
            }
#pragma unroll
            for (int r = 0; r < 4; r++) {
                const float xm[4] = {xr[r].x, xr[r].y, xr[r].z, xr[r].w};
#pragma unroll
                for (int m = 0; m < 4; m++) {
                    acc[r][0] = fmaf(xm[m], tv[m].x, acc[r][0]);
                    acc[r][1] = fmaf(xm[m], tv[m].y, acc[r][1]);
                    acc[r][2] = fmaf(xm[m], tv[m].z, acc[r][2]);
                    acc[r][3] = fmaf(xm[m], tv[m].w, acc[r][3]);
                }
            }
        }
        float ee[4] = {0.f, 0.f, 0.f, 0.f}, eo[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int r = 0; r < 4; r++) {
            float4 *dst = reinterpret_cast<float4 *>(Tout + (int64_t)(4 * I + r) * B + col);
            float4 o;
            if (first) {
                o = make_float4(acc[r][0], acc[r][1], acc[r][2], acc[r][3]);
            } else {
                const float4 p = *dst;
                o.x = 2.f * acc[r][0] - p.x;
                o.y = 2.f * acc[r][1] - p.y;
                o.z = 2.f * acc[r][2] - p.z;
                o.w = 2.f * acc[r][3] - p.w;
            }
            *dst = o;
            const float ov[4] = {o.x, o.y, o.z, o.w};
#pragma unroll
            for (int c = 0; c < 4; c++) {
                ee[c] = fmaf(own[r][c], own[r][c], ee[c]);
                eo[c] = fmaf(own[r][c], ov[c], eo[c]);
            }
        }
#pragma unroll
        for (int c = 0; c < 4; c++) {
            pair_add(hee[c], lee[c], ee[c]);
            pair_add(heo[c], leo[c], eo[c]);
        }
    }
#pragma unroll
    for (int c = 0; c < 4; c++)
        *reinterpret_cast<float4 *>(red[w][lane * 4 + c]) = make_float4(hee[c], lee[c], heo[c], leo[c]);
    __syncthreads();
    {
        const int j = threadIdx.x >> 1, which = threadIdx.x & 1;  // 256 threads = 128 cols x 2
        float hs = 0.f, ls = 0.f;
#pragma unroll
        for (int q = 0; q < kF32Warps; q++) {
            pair_add(hs, ls, red[q][j][2 * which]);
            ls += red[q][j][2 * which + 1];
        }
        partial_k[((int64_t)blockIdx.x * B + chunk * 128 + j) * 2 + which] = make_float2(hs, ls);
    }
}

int cheb_f32_rowgroups(int nb)
{
    const int per = kF32Warps * kRowsPerWarp;
    return (nb + per - 1) / per;
}

void launch_cheb_step_f32(cudaStream_t st, const DevMatrix &m, const float *Tin, float *Tout,
                          int B, int first, float2 *partial_k, int rowgroups)
{
    dim3 grid(rowgroups, B / 128);
    k_cheb_f32<<<grid, 32 * kF32Warps, 0, st>>>(m.nb, m.rowptr, m.colidx, m.x32, Tin, Tout, B,
                                                first, partial_k);
}

// ---------------------------------------------------------------------------
// FP32 Chebyshev step, staged form.  Block rows are cut into groups of R
// consecutive rows; for each group the host lists U_g, the distinct block
// rows its blocks reference (for beta-cristobalite in cell order, |U_g| is
// about 1.6 R against 3.67 R block reads without staging).  A CTA takes one
// group x 64 columns and copies, with 16-byte cp.async (LDGSTS), the U_g rows
// of T_k, its own rows of T_{k-1} and its X blocks into shared memory, then
// every warp computes its block rows from shared memory: lane = 2 columns.
// Column dot products as in k_cheb_f32, one FP64 pair per column per CTA.
// ---------------------------------------------------------------------------
constexpr int kV2Cols = 64;
constexpr int kV2Warps = 8;

__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gmem_src)
{
    // no memory clobber: the copies are ordered by cp_async_wait_all below
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem_src));
}
__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

__global__ void __launch_bounds__(32 * kV2Warps)
    k_cheb_f32_staged(int nb, int R, const int32_t *__restrict__ rowptr,
                      const int32_t *__restrict__ lcol, const int32_t *__restrict__ lself,
                      const int32_t *__restrict__ grp_ptr, const int32_t *__restrict__ grp_rows,
                      const float *__restrict__ x32, const float *__restrict__ Tin,
                      float *__restrict__ Tout, int B, int first, float2 *__restrict__ partial_k,
                      int maxU, int maxBlk)
{
    extern __shared__ float4 smem4[];
    float *sT = reinterpret_cast<float *>(smem4);  // maxU*4 rows x 64
    float *sP = sT + maxU * 4 * kV2Cols;            // R*4 rows x 64 (T_{k-1})
    float *sX = sP + R * 4 * kV2Cols;               // maxBlk*16
    int *sU = reinterpret_cast<int *>(sX + maxBlk * 16);  // maxU block rows
    int *sL = sU + maxU;                                  // maxBlk local columns
    int *sR = sL + maxBlk;                                // R+1 row offsets
    const int g = blockIdx.x, chunk = blockIdx.y, tid = threadIdx.x;
    const int I0 = g * R;
    const int I1 = min(nb, I0 + R);
    const int nr = I1 - I0;
    const int u0 = grp_ptr[g], nu = grp_ptr[g + 1] - u0;
    const int tb0 = rowptr[I0], nbk = rowptr[I1] - tb0;
    const int col0 = chunk * kV2Cols;
    // ---- indices first, so every copy address below comes from shared memory ----
    for (int i = tid; i < nu; i += blockDim.x) sU[i] = grp_rows[u0 + i];
    for (int i = tid; i < nbk; i += blockDim.x) sL[i] = lcol[tb0 + i];
    for (int i = tid; i <= nr; i += blockDim.x) sR[i] = rowptr[I0 + i] - tb0;
    for (int idx = tid; idx < nbk * 4; idx += blockDim.x)
        cp_async16(sX + idx * 4, x32 + (int64_t)tb0 * 16 + idx * 4);
    if (!first)
        for (int idx = tid; idx < nr * 64; idx += blockDim.x) {
            const int r = idx >> 6, m = (idx >> 4) & 3, sg = idx & 15;
            cp_async16(sP + (r * 4 + m) * kV2Cols + sg * 4,
                       Tout + (int64_t)(4 * (I0 + r) + m) * B + col0 + sg * 4);
        }
    __syncthreads();
    // ---- stage T_k rows: 16 segments of 16 bytes per 64-column row ----
    for (int idx = tid; idx < nu * 64; idx += blockDim.x) {
        const int u = idx >> 6, m = (idx >> 4) & 3, sg = idx & 15;
        cp_async16(sT + (u * 4 + m) * kV2Cols + sg * 4,
                   Tin + (int64_t)(4 * sU[u] + m) * B + col0 + sg * 4);
    }
    cp_async_wait_all();
    __syncthreads();
    // ---- compute ----
    const int lane = tid & 31, w = tid >> 5, c = 2 * lane;
    // pairs (hi, lo) packed over columns (c, c+1): <T_k,T_k> in (eh, el), <T_k,T_{k+1}> in (oh, ol)
    float2 eh = make_float2(0.f, 0.f), el = eh, oh = eh, ol = eh;
    for (int r = w; r < nr; r += kV2Warps) {
        const int I = I0 + r;
        const int ta = sR[r], te = sR[r + 1];
        float2 acc[4];  // row q of the block row, columns (c, c+1)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[q] = make_float2(0.f, 0.f);
        for (int t = ta; t < te; t++) {
            const float *tv = sT + sL[t] * 4 * kV2Cols + c;
            float2 v[4];
#pragma unroll
            for (int m = 0; m < 4; m++) v[m] = *reinterpret_cast<const float2 *>(tv + m * kV2Cols);
            block_fma2(acc, reinterpret_cast<const float4 *>(sX + t * 16), v);
        }
        const float *own = sT + lself[I] * 4 * kV2Cols + c;
        float2 ee = make_float2(0.f, 0.f), eo = ee;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const float2 ov = *reinterpret_cast<const float2 *>(own + q * kV2Cols);
            float2 o = acc[q];
            if (!first) o = cheb_next2(acc[q], *reinterpret_cast<const float2 *>(sP + (r * 4 + q) * kV2Cols + c));
            *reinterpret_cast<float2 *>(Tout + (int64_t)(4 * I + q) * B + col0 + c) = o;
            ee = __ffma2_rn(ov, ov, ee);
            eo = __ffma2_rn(ov, o, eo);
        }
        pair_add2(eh, el, ee);
        pair_add2(oh, ol, eo);
    }
    __syncthreads();  // shared T no longer needed: reuse for the reduction
    float *red = reinterpret_cast<float *>(smem4);  // [8][64][2 sums][hi, lo]
    float4 *rb = reinterpret_cast<float4 *>(red + ((size_t)w * kV2Cols + c) * 4);
    rb[0] = make_float4(eh.x, el.x, oh.x, ol.x);
    rb[1] = make_float4(eh.y, el.y, oh.y, ol.y);
    __syncthreads();
    if (tid < 2 * kV2Cols) {
        const int j = tid >> 1, which = tid & 1;
        float hsum = 0.f, lsum = 0.f;
#pragma unroll
        for (int q = 0; q < kV2Warps; q++) {
            const float2 v = *reinterpret_cast<const float2 *>(red + ((size_t)q * kV2Cols + j) * 4 + which * 2);
            pair_add(hsum, lsum, v.x);
            lsum += v.y;
        }
        partial_k[((int64_t)g * B + col0 + j) * 2 + which] = make_float2(hsum, lsum);
    }
}

int cheb_f32_staged_configure(size_t smem)
{
    const int lim = smem_optin_max((const void *)k_cheb_f32_staged);
    if ((int)smem > lim) return (int)cudaErrorInvalidValue;
    return (int)cudaFuncSetAttribute(k_cheb_f32_staged, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
}

size_t cheb_f32_staged_smem(int R, int maxU, int maxBlk)
{
    size_t b = (size_t)(maxU * 4 * kV2Cols + R * 4 * kV2Cols + maxBlk * 16) * sizeof(float) +
               (size_t)(maxU + maxBlk + R + 1) * sizeof(int);
    const size_t red = (size_t)kV2Warps * kV2Cols * 4 * sizeof(float);
    return b > red ? b : red;
}

int launch_cheb_step_f32_staged(cudaStream_t st, const DevMatrix &m, const StagePlan &sp,
                                const float *Tin, float *Tout, int B, int first,
                                float2 *partial_k)
{
    const size_t smem = cheb_f32_staged_smem(sp.R, sp.maxU, sp.maxBlk);
    dim3 grid(sp.G, B / kV2Cols);
    k_cheb_f32_staged<<<grid, 32 * kV2Warps, smem, st>>>(m.nb, sp.R, m.rowptr, sp.lcol, sp.lself,
                                                         sp.grp_ptr, sp.grp_rows, m.x32, Tin,
                                                         Tout, B, first, partial_k, sp.maxU,
                                                         sp.maxBlk);
    return 1;
}

// ---------------------------------------------------------------------------
// FP32 Chebyshev recurrence, persistent form: one cooperative launch runs all
// K steps of a slab.  CTA = one task (row group g of R block rows x one
// 64-column chunk), resident for the whole launch; its own rows of T_k and
// T_{k-1} stay in shared memory, so a step stages only the group's halo rows
// (the referenced rows owned by other groups) from global memory.  A task
// publishes its T_{k+1} rows to global buffer (k+1)%2 and then its step
// count in flags[task] (release); before step k it waits until every
// neighbouring task of the same chunk has published step k (acquire).  The
// block pattern is symmetric, so that one wait also guarantees that no
// neighbour still reads the buffer about to be overwritten.  Waits are
// bounded: past kSpinLimit polls the kernel raises *err and every CTA leaves
// at its next wait.  Co-residency of all tasks comes from the cooperative
// launch, which the host only uses when the tasks fit the device.
// ---------------------------------------------------------------------------
constexpr int kPCols = 64;
constexpr int kPWarps = 8;
constexpr long long kSpinLimit = 1ll << 24;

__device__ __forceinline__ int ld_acquire_gpu(const int *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_gpu(int *p, int v)
{
    asm volatile("st.release.gpu.global.s32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}

template <int kRPW>  // block rows per warp kept in registers: R <= 8 kRPW
__global__ void __launch_bounds__(32 * kPWarps, (kRPW <= 4 ? 3 : 2))
    k_cheb_f32_persistent(int nb, int R, int nc, int K, int B, int c0, const int32_t *__restrict__ rowptr,
                          const int32_t *__restrict__ lcode, const int32_t *__restrict__ hptr,
                          const int32_t *__restrict__ hrows, const int32_t *__restrict__ nptr,
                          const int32_t *__restrict__ ngrp, const float *__restrict__ x32,
                          float *__restrict__ G0, float *__restrict__ G1, float2 *__restrict__ partial,
                          int G, int *__restrict__ flags, int *__restrict__ err, int maxH, int maxBlk,
                          int maxNG)
{
    extern __shared__ float4 psm4[];
    const int rowf = 4 * kPCols;  // floats per staged block row
    float *own0 = reinterpret_cast<float *>(psm4);
    float *own1 = own0 + R * rowf;
    float *halo = own1 + R * rowf;  // also the dot-product reduction buffer
    const int halo_f = max(maxH * rowf, kPWarps * kPCols * 4);
    float *sX = halo + halo_f;
    int *sL = reinterpret_cast<int *>(sX + maxBlk * 16);
    int *sR = sL + maxBlk;
    int *sH = sR + R + 1;
    int *sN = sH + max(maxH, 1);
    const int task = blockIdx.x, g = task / nc, c = task % nc, col0 = c * kPCols;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, cl = 2 * lane;
    const int I0 = g * R, nr = min(R, nb - I0);
    const int tb0 = rowptr[I0], nbk = rowptr[I0 + nr] - tb0;
    const int h0 = hptr[g], nh = hptr[g + 1] - h0;
    const int n0 = nptr[g], nn = nptr[g + 1] - n0;
    for (int i = tid; i < nbk; i += blockDim.x) sL[i] = lcode[tb0 + i];
    for (int i = tid; i <= nr; i += blockDim.x) sR[i] = rowptr[I0 + i] - tb0;
    for (int i = tid; i < nh; i += blockDim.x) sH[i] = hrows[h0 + i];
    for (int i = tid; i < nn; i += blockDim.x) sN[i] = ngrp[n0 + i];
    for (int idx = tid; idx < nbk * 4; idx += blockDim.x)
        cp_async16(sX + idx * 4, x32 + (int64_t)tb0 * 16 + idx * 4);
    // own rows of T_0: the identity columns c0 + col0 .. c0 + col0 + 63
    for (int e = tid; e < nr * rowf; e += blockDim.x) {
        const int r = e / rowf, m = (e / kPCols) & 3, j = e % kPCols;
        own0[e] = (4 * (I0 + r) + m == c0 + col0 + j) ? 1.f : 0.f;
    }
    cp_async_wait_all();
    __syncthreads();
    const volatile int *verr = err;
    __shared__ int s_stop;
    for (int k = 0; k < K; k++) {
        float *cur = (k & 1) ? own1 : own0;
        float *prev = (k & 1) ? own0 : own1;
        const float *Gk = (k & 1) ? G1 : G0;
        float *Gn = (k & 1) ? G0 : G1;
        // ---- 1. contributions of the own rows (in shared memory already),
        // computed before waiting so the wait overlaps with work ----
        float2 acc[kRPW][4];  // row q of the warp's j-th block row, columns (cl, cl+1)
#pragma unroll
        for (int j = 0; j < kRPW; j++)
#pragma unroll
            for (int q = 0; q < 4; q++) acc[j][q] = make_float2(0.f, 0.f);
#pragma unroll
        for (int j = 0; j < kRPW; j++) {
            const int r = w + j * kPWarps;
            if (r >= nr) break;
            for (int t = sR[r]; t < sR[r + 1]; t++) {
                const int code = sL[t];
                if (code >= R) continue;
                const float *tv = cur + code * rowf + cl;
                float2 v[4];
#pragma unroll
                for (int m = 0; m < 4; m++) v[m] = *reinterpret_cast<const float2 *>(tv + m * kPCols);
                block_fma2(acc[j], reinterpret_cast<const float4 *>(sX + t * 16), v);
            }
        }
        // ---- 2. wait for the neighbours' step k: warp 0, one lane per
        // neighbour; the stop decision is broadcast through shared memory so
        // the CTA leaves as one ----
        if (w == 0) {
            bool give_up = false;
            if (k > 0) {
                for (int i0 = 0; i0 < nn; i0 += 32) {
                    const int i = i0 + lane;
                    const int *f = i < nn ? flags + sN[i] * nc + c : nullptr;
                    long long spins = 0;
                    bool ready = (f == nullptr);
                    while (!__all_sync(0xffffffffu, ready)) {
                        if (!ready) ready = ld_acquire_gpu(f) >= k;
                        if (__any_sync(0xffffffffu, *verr != 0)) {
                            give_up = true;
                            break;
                        }
                        if (++spins > kSpinLimit) {
                            if (lane == 0) atomicExch(err, 1);
                            give_up = true;
                            break;
                        }
                        __nanosleep(20);
                    }
                    if (give_up) break;
                }
                __threadfence();
            }
            if (lane == 0) s_stop = give_up ? 1 : *verr;
        }
        __syncthreads();
        if (s_stop) return;  // no copies are in flight here
        // ---- 3. halo rows of T_k ----
        if (k == 0) {
            for (int e = tid; e < nh * rowf; e += blockDim.x) {
                const int h = e / rowf, m = (e / kPCols) & 3, j = e % kPCols;
                halo[e] = (4 * sH[h] + m == c0 + col0 + j) ? 1.f : 0.f;
            }
        } else {
            for (int idx = tid; idx < nh * 64; idx += blockDim.x) {
                const int h = idx >> 6, m = (idx >> 4) & 3, sg = idx & 15;
                cp_async16(halo + (h * 4 + m) * kPCols + sg * 4,
                           Gk + (int64_t)(4 * sH[h] + m) * B + col0 + sg * 4);
            }
        }
        cp_async_wait_all();
        __syncthreads();
        // ---- 4. halo contributions, T_{k+1} for the own rows, dot products ----
        // pairs (hi, lo) over columns (cl, cl+1): <T_k,T_k> in (eh, el), <T_k,T_{k+1}> in (oh, ol)
        float2 eh = make_float2(0.f, 0.f), el = eh, oh = eh, ol = eh;
#pragma unroll
        for (int j = 0; j < kRPW; j++) {
            const int r = w + j * kPWarps;
            if (r >= nr) break;
            for (int t = sR[r]; t < sR[r + 1]; t++) {
                const int code = sL[t];
                if (code < R) continue;
                const float *tv = halo + (code - R) * rowf + cl;
                float2 v[4];
#pragma unroll
                for (int m = 0; m < 4; m++) v[m] = *reinterpret_cast<const float2 *>(tv + m * kPCols);
                block_fma2(acc[j], reinterpret_cast<const float4 *>(sX + t * 16), v);
            }
            float2 ee = make_float2(0.f, 0.f), eo = ee;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const float2 ov = *reinterpret_cast<const float2 *>(cur + r * rowf + q * kPCols + cl);
                float2 *pv = reinterpret_cast<float2 *>(prev + r * rowf + q * kPCols + cl);
                const float2 o = k == 0 ? acc[j][q] : cheb_next2(acc[j][q], *pv);
                *pv = o;
                *reinterpret_cast<float2 *>(Gn + (int64_t)(4 * (I0 + r) + q) * B + col0 + cl) = o;
                ee = __ffma2_rn(ov, ov, ee);
                eo = __ffma2_rn(ov, o, eo);
            }
            pair_add2(eh, el, ee);
            pair_add2(oh, ol, eo);
        }
        // ---- publish T_{k+1} ----
        __threadfence();
        __syncthreads();
        if (tid == 0) st_release_gpu(flags + task, k + 1);
        // ---- per-column partial sums (the halo buffer is free now) ----
        float *red = halo;  // [warps][64][2 sums][hi, lo]
        float4 *rb = reinterpret_cast<float4 *>(red + ((size_t)w * kPCols + cl) * 4);
        rb[0] = make_float4(eh.x, el.x, oh.x, ol.x);
        rb[1] = make_float4(eh.y, el.y, oh.y, ol.y);
        __syncthreads();
        if (tid < 2 * kPCols) {
            const int j = tid >> 1, which = tid & 1;
            float hsum = 0.f, lsum = 0.f;
#pragma unroll
            for (int q = 0; q < kPWarps; q++) {
                const float2 v = *reinterpret_cast<const float2 *>(red + ((size_t)q * kPCols + j) * 4 + which * 2);
                pair_add(hsum, lsum, v.x);
                lsum += v.y;
            }
            partial[(((int64_t)k * G + g) * B + col0 + j) * 2 + which] = make_float2(hsum, lsum);
        }
        __syncthreads();
    }
}

size_t cheb_f32_persistent_smem(int R, int maxH, int maxBlk, int maxNG)
{
    const size_t rowf = 4 * kPCols;
    const size_t halo_f = std::max((size_t)maxH * rowf, (size_t)kPWarps * kPCols * 4);
    return (2 * (size_t)R * rowf + halo_f + (size_t)maxBlk * 16) * sizeof(float) +
           ((size_t)maxBlk + R + 1 + std::max(maxH, 1) + maxNG) * sizeof(int);
}

static int persistent_rpw(int R) { return (R + kPWarps - 1) / kPWarps; }

template <int kRPW>
static int persistent_setup_t(size_t smem, int *ctas_per_sm)
{
    const int lim = smem_optin_max((const void *)k_cheb_f32_persistent<kRPW>);
    if ((int)smem > lim) return (int)cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(k_cheb_f32_persistent<kRPW>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    if (e != cudaSuccess) return (int)e;
    return (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, k_cheb_f32_persistent<kRPW>,
                                                              32 * kPWarps, smem);
}

int cheb_f32_persistent_setup(int R, size_t smem, int *ctas_per_sm)
{
    switch (persistent_rpw(R)) {
    case 2: return persistent_setup_t<2>(smem, ctas_per_sm);
    case 3: return persistent_setup_t<3>(smem, ctas_per_sm);
    case 4: return persistent_setup_t<4>(smem, ctas_per_sm);
    case 6: return persistent_setup_t<6>(smem, ctas_per_sm);
    case 8: return persistent_setup_t<8>(smem, ctas_per_sm);
    default: return (int)cudaErrorInvalidValue;
    }
}

int launch_cheb_f32_persistent(cudaStream_t st, const DevMatrix &m, const PersistPlan &pp, int K,
                               int B, int c0, float *G0, float *G1, float2 *partial, int *flags,
                               int *err)
{
    const size_t smem = cheb_f32_persistent_smem(pp.R, pp.maxH, pp.maxBlk, pp.maxNG);
    int nb = m.nb, R = pp.R, nc = pp.nc, G = pp.G, maxH = pp.maxH, maxBlk = pp.maxBlk,
        maxNG = pp.maxNG;
    const int32_t *rowptr = m.rowptr, *lcode = pp.lcode, *hptr = pp.hptr, *hrows = pp.hrows,
                  *nptr = pp.nptr, *ngrp = pp.ngrp;
    const float *x32 = m.x32;
    void *args[] = {&nb, &R, &nc, &K, &B, &c0, &rowptr, &lcode, &hptr, &hrows, &nptr, &ngrp,
                    &x32, &G0, &G1, &partial, &G, &flags, &err, &maxH, &maxBlk, &maxNG};
    const void *fn = nullptr;
    switch (persistent_rpw(pp.R)) {
    case 2: fn = (const void *)k_cheb_f32_persistent<2>; break;
    case 3: fn = (const void *)k_cheb_f32_persistent<3>; break;
    case 4: fn = (const void *)k_cheb_f32_persistent<4>; break;
    case 6: fn = (const void *)k_cheb_f32_persistent<6>; break;
    case 8: fn = (const void *)k_cheb_f32_persistent<8>; break;
    default: return (int)cudaErrorInvalidValue;
    }
    return (int)cudaLaunchCooperativeKernel(fn, dim3(G * nc), dim3(32 * kPWarps), args, smem, st);
}

// ---------------------------------------------------------------------------
// mu_k = sum_i d[k][i]  (deterministic block tree).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_moment_sums(const double *__restrict__ d, int n,
                                                     double *__restrict__ mom)
{
    __shared__ double sh[32];
    const int k = blockIdx.x;
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += d[(int64_t)k * n + i];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) mom[k] = s;
}

void launch_moment_sums(cudaStream_t st, const double *d, int n, int nmom, double *mom)
{
    k_moment_sums<<<nmom, 256, 0, st>>>(d, n, mom);
}

// tab[j] = cos(pi j / (2 nq_cap)), j < 4 nq_cap, built once per workspace.
// For a quadrature of nq nodes (nq and nq_cap powers of two, r = nq > 0 ? nq_cap / nq : 1)
// the nodes are theta_q = pi (2q+1) / (2 nq): cos(theta_q) is entry (2q+1) r
// (the same double as cos(pi (q + 1/2) / nq): the arguments differ by exact
// power-of-two scalings) and cos(k theta_q) is entry (k (2q+1) mod 4 nq) r;
// the residue is a mask, also after 32-bit wrap-around.  The node kernels
// below then evaluate no cosine per (k, q).
__global__ void k_cos_table(int nq_cap, double *__restrict__ tab)
{
    const double h = kPi / (2.0 * nq_cap);
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < 4 * nq_cap; j += gridDim.x * blockDim.x)
        tab[j] = cos(h * j);
}

void launch_cos_table(cudaStream_t st, int nq_cap, double *tab)
{
    const int T = 256;
    const int blocks = (int)std::min<int64_t>((4 * (int64_t)nq_cap + T - 1) / T, 1024);
    k_cos_table<<<blocks, T, 0, st>>>(nq_cap, tab);
}

// rho_q = g_0 mu_0 + 2 sum_{k>=1} g_k mu_k cos(k theta_q): the damped DOS at
// the Chebyshev-Gauss nodes (times pi sin theta), nq read from the state.
__global__ void k_dos_nodes(const double *__restrict__ g, const double *__restrict__ mom, int M,
                            const DevState *__restrict__ st, int nq_cap, const double *__restrict__ tab,
                            double *__restrict__ rho, double *__restrict__ ebx)
{
    extern __shared__ double wk[];  // (2 - delta_k0) g_k mu_k
    for (int k = threadIdx.x; k < M; k += blockDim.x) wk[k] = k == 0 ? g[0] * mom[0] : 2.0 * g[k] * mom[k];
    __syncthreads();
    const int nq = min(st->nq, nq_cap), r = nq > 0 ? nq_cap / nq : 1;
    const size_t cmask = 4 * (size_t)nq_cap - 1;  // keeps every table index in range
    const unsigned mask = 4u * (unsigned)nq - 1u;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x) {
        const unsigned step = 2u * (unsigned)q + 1u;
        unsigned j = 0;
        double s = wk[0];
        for (int k = 1; k < M; k++) {
            j = (j + step) & mask;
            s += wk[k] * tab[((size_t)j * r) & cmask];
        }
        rho[q] = s;
        // e^{beta_x x_q} for the multisection; unused above kEtabBeta
        const double bx = st->beta_x;
        ebx[q] = bx <= kEtabBeta ? exp(bx * tab[((size_t)step * r) & cmask]) : 0.0;
    }
}

void launch_dos_nodes(cudaStream_t st, const double *g, const double *mom, int M,
                      const DevState *state, int nq_cap, const double *tab, double *rho)
{
    const int T = 256;
    int blocks = (nq_cap + T - 1) / T;
    if (blocks > 1024) blocks = 1024;
    k_dos_nodes<<<blocks, T, sizeof(double) * M, st>>>(g, mom, M, state, nq_cap, tab, rho, rho + nq_cap);
}

// ---------------------------------------------------------------------------
// Multisection for mu_x: each CTA evaluates the electron count at one of
// kBisectCand equispaced points of [lo, hi]; the last CTA to finish narrows
// the bracket (or records a solution / a bracketing failure).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
    k_bisect_round(const double *__restrict__ rho, const double *__restrict__ g,
                   const double *__restrict__ mom, const double *__restrict__ tab, int nq_cap, int M,
                   double n_elec, double tol_n, int round, int last_round, double *__restrict__ cand,
                   DevState *st)
{
    __shared__ double sh[32];
    __shared__ int s_last;
    if (st->bisect_done) return;
    const int P = gridDim.x, p = blockIdx.x;
    const double lo = st->lo, hi = st->hi;
    const double mu = lo + (hi - lo) * (double)p / (double)(P - 1);
    const double beta_x = st->beta_x;
    double s = 0.0;
    if (beta_x > 0) {
        const int nq = st->nq;
        const int r = nq > 0 ? nq_cap / nq : 1;
        const size_t cmask = 4 * (size_t)nq_cap - 1;  // keeps every table index in range
        if (beta_x <= kEtabBeta) {
            // f(x_q) = 1 / (1 + e^{beta x_q} e^{-beta mu}): one exp per candidate,
            // the node factors from k_dos_nodes (no overflow below kEtabBeta)
            const double C = exp(-beta_x * mu), *ebx = rho + nq_cap;
            for (int q = threadIdx.x; q < nq; q += blockDim.x) s += rho[q] / (1.0 + ebx[q] * C);
        } else {
            for (int q = threadIdx.x; q < nq; q += blockDim.x)
                s += fermi(tab[((size_t)(2 * q + 1) * r) & cmask], mu, beta_x) * rho[q];
        }
        s = block_sum(s, sh);
        s = 2.0 * s / nq;
    } else {
        const double th = acos(mu);
        for (int k = threadIdx.x; k < M; k += blockDim.x) {
            const double c = (k == 0) ? 1.0 - th / kPi : -2.0 * sin(k * th) / (k * kPi);
            s += c * g[k] * mom[k];
        }
        s = block_sum(s, sh);
        s = 2.0 * s;
    }
    if (threadIdx.x == 0) {
        cand[p] = s;
        __threadfence();
        const unsigned int t = atomicAdd(&st->ticket, 1u);
        s_last = (t == (unsigned)(P - 1));
    }
    __syncthreads();
    if (!s_last || threadIdx.x != 0) return;
    __threadfence();
    st->ticket = 0u;
    volatile double *vc = cand;
    st->bisect_rounds = round + 1;
    if (round == 0 && !(vc[0] <= n_elec && n_elec <= vc[P - 1])) {
        st->status = TB_ERR_BISECTION;
        st->bisect_done = 1;
        st->mu_x = 0.0;
        return;
    }
    int best = 0;
    double bd = fabs(vc[0] - n_elec);
    int first_ge = P - 1;
    for (int i = 0; i < P; i++) {
        const double dv = fabs(vc[i] - n_elec);
        if (dv < bd) {
            bd = dv;
            best = i;
        }
        if (vc[i] >= n_elec && i < first_ge) first_ge = i;
    }
    for (int i = 0; i < P; i++)
        if (vc[i] >= n_elec) {
            first_ge = i;
            break;
        }
    const double h = (hi - lo) / (double)(P - 1);
    if (bd <= tol_n) {
        st->mu_x = lo + h * best;
        st->bisect_done = 1;
        return;
    }
    const double nlo = (first_ge > 0) ? lo + h * (first_ge - 1) : lo;
    const double nhi = lo + h * first_ge;
    st->lo = nlo;
    st->hi = nhi;
    if (round == last_round) {
        st->mu_x = 0.5 * (nlo + nhi);
        st->bisect_done = 1;
    }
}

void launch_bisect_round(cudaStream_t st, const double *rho, const double *g, const double *mom,
                         const double *tab, int nq_cap, int M, double n_elec, double tol_n, int round,
                         double *cand, DevState *state)
{
    k_bisect_round<<<kBisectCand, 256, 0, st>>>(rho, g, mom, tab, nq_cap, M, n_elec, tol_n, round,
                                                kBisectRounds - 1, cand, state);
}

// f_q = Fermi function at the quadrature nodes for the final mu_x
__global__ void k_fermi_nodes(const DevState *__restrict__ st, int nq_cap, const double *__restrict__ tab,
                              double *__restrict__ fq)
{
    const double beta_x = st->beta_x;
    if (!(beta_x > 0)) return;
    const int nq = min(st->nq, nq_cap), r = nq > 0 ? nq_cap / nq : 1;
    const size_t cmask = 4 * (size_t)nq_cap - 1;  // keeps every table index in range
    const double mu_x = st->mu_x;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x)
        fq[q] = fermi(tab[((size_t)(2 * q + 1) * r) & cmask], mu_x, beta_x);
}

// c_k(mu*) by Chebyshev-Gauss quadrature (FP64), or the step coefficients.
__global__ void __launch_bounds__(256) k_fermi_coeffs(int M, DevState *st, const double *__restrict__ tab,
                                                      int nq_cap, const double *__restrict__ fq,
                                                      double *__restrict__ c)
{
    __shared__ double sh[32];
    const int k = blockIdx.x;
    const double mu_x = st->mu_x, beta_x = st->beta_x;
    if (threadIdx.x == 0 && k == 0) st->mu = st->a * mu_x + st->b;
    if (beta_x > 0) {
        const int nq = st->nq, r = nq > 0 ? nq_cap / nq : 1;
        const size_t cmask = 4 * (size_t)nq_cap - 1;  // keeps every table index in range
        const unsigned mask = 4u * (unsigned)nq - 1u;
        double s = 0.0;
        for (int q = threadIdx.x; q < nq; q += blockDim.x)
            s += fq[q] * tab[((size_t)(((unsigned)k * (2u * (unsigned)q + 1u)) & mask) * r) & cmask];
        s = block_sum(s, sh);
        if (threadIdx.x == 0) c[k] = (k == 0 ? 1.0 : 2.0) * s / nq;
    } else if (threadIdx.x == 0) {
        const double th = acos(mu_x);
        c[k] = (k == 0) ? 1.0 - th / kPi : -2.0 * sin(k * th) / (k * kPi);
    }
}

void launch_fermi_coeffs(cudaStream_t st, int M, DevState *state, int nq_cap, const double *tab, double *fq,
                         double *c)
{
    const int T = 256;
    const int blocks = std::min((nq_cap + T - 1) / T, 1024);
    k_fermi_nodes<<<blocks, T, 0, st>>>(state, nq_cap, tab, fq);
    k_fermi_coeffs<<<M, T, 0, st>>>(M, state, tab, nq_cap, fq, c);
}

// diagP_i = sum_k c_k g_k d[k][i] (one thread per orbital, coalesced rows of
// d);  q_a = 2 sum_{i in a} diagP_i over the atom's four consecutive orbitals
// (lanes 4a' .. 4a'+3 of a warp, n = 4 natoms).
__global__ void __launch_bounds__(256)
    k_charges(const double *__restrict__ d, const double *__restrict__ c,
              const double *__restrict__ g, int M, int n, int natoms, double *__restrict__ diagP,
              double *__restrict__ q)
{
    extern __shared__ double wsh[];
    for (int k = threadIdx.x; k < M; k += blockDim.x) wsh[k] = c[k] * g[k];
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double p = 0.0;
    if (i < n) {
#pragma unroll 8
        for (int k = 0; k < M; k++) p += wsh[k] * d[(int64_t)k * n + i];
        if (diagP) diagP[i] = p;
    }
    // n is a multiple of 4 and blockDim.x of 32: an atom's orbitals share a warp
    double s = p + __shfl_xor_sync(0xffffffffu, p, 1);
    s += __shfl_xor_sync(0xffffffffu, s, 2);
    if (i < n && (i & 3) == 0) q[i >> 2] = 2.0 * s;
}

// n_found = 2 sum_k c_k g_k mu_k;  E_band = 2 sum_k c_k g_k (a tr(T_k X) + b mu_k).
__global__ void __launch_bounds__(256) k_eband(const double *__restrict__ c,
                                               const double *__restrict__ g,
                                               const double *__restrict__ mom, int M, DevState *st)
{
    __shared__ double sh[32];
    const double a = st->a, b = st->b;
    double ne = 0.0, eb = 0.0;
    for (int k = threadIdx.x; k < M; k += blockDim.x) {
        const double w = c[k] * g[k];
        const double tx = (k == 0) ? mom[1] : 0.5 * (mom[k + 1] + mom[k - 1]);
        ne += w * mom[k];
        eb += w * (a * tx + b * mom[k]);
    }
    ne = block_sum(ne, sh);
    eb = block_sum(eb, sh);
    if (threadIdx.x == 0) {
        st->n_found = 2.0 * ne;
        st->e_band = 2.0 * eb;
    }
}

void launch_charges(cudaStream_t st, const double *d, const double *c, const double *g,
                    const double *mom, int M, int n, int natoms, double *diagP, double *q,
                    DevState *state)
{
    const int T = 256;
    k_charges<<<(n + T - 1) / T, T, sizeof(double) * M, st>>>(d, c, g, M, n, natoms, diagP, q);
    k_eband<<<1, 256, 0, st>>>(c, g, mom, M, state);
}

// ---------------------------------------------------------------------------
// SCC update (one CTA): residual r = q_out - q_in, convergence test, Anderson
// mixing (D. G. Anderson, J. ACM 12, 547 (1965)) over the stored history,
// then the new Coulomb shift V = Gamma (q_in - q0).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024)
    k_scc_update(int natoms, const double *__restrict__ qout, double *__restrict__ qin,
                 const double *__restrict__ q0, double *__restrict__ hq, double *__restrict__ hr,
                 int32_t *__restrict__ meta, double beta, int history, double tol,
                 const int32_t *__restrict__ g_rp, const int32_t *__restrict__ g_ci,
                 const double *__restrict__ g_v, double *__restrict__ V, double *__restrict__ shift,
                 DevState *st)
{
    __shared__ double sh[32];
    __shared__ double A[kMaxHistory * kMaxHistory], rhs[kMaxHistory], gam[kMaxHistory];
    __shared__ int s_use, s_stop;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, nw = blockDim.x >> 5;
    // 1. residual norm
    double mx = 0.0;
    for (int a = tid; a < natoms; a += blockDim.x) mx = fmax(mx, fabs(qout[a] - qin[a]));
    mx = warp_max(mx);
    if (lane == 0) sh[w] = mx;
    __syncthreads();
    if (tid == 0) {
        double m = 0.0;
        for (int i = 0; i < nw; i++) m = fmax(m, sh[i]);
        st->dq_max = m;
        s_stop = 0;
        if (!(m < 1e3)) {
            st->status = TB_ERR_DIVERGED;
            s_stop = 1;
        } else if (m < tol) {
            st->converged = 1;
            s_stop = 1;
        }
    }
    __syncthreads();
    if (s_stop) return;
    const int m = meta[0], head = meta[1];
    // 2. normal equations of the Anderson least-squares problem
    const int npair = m * (m + 1) / 2;
    for (int pr = w; pr < npair + m; pr += nw) {
        int i, j;
        const bool is_rhs = pr >= npair;
        if (is_rhs) {
            i = pr - npair;
            j = -1;
        } else {
            i = 0;
            int rem = pr;
            while (rem > i) {
                rem -= i + 1;
                i++;
            }
            j = rem;
        }
        double s = 0.0;
        for (int a = lane; a < natoms; a += 32) {
            const double r = qout[a] - qin[a];
            const double di = r - hr[(int64_t)i * natoms + a];
            const double dj = is_rhs ? r : r - hr[(int64_t)j * natoms + a];
            s += di * dj;
        }
        s = warp_sum(s);
        if (lane == 0) {
            if (is_rhs)
                rhs[i] = s;
            else {
                A[i * m + j] = s;
                A[j * m + i] = s;
            }
        }
    }
    __syncthreads();
    if (tid == 0) {
        int use = m > 0;
        for (int i = 0; i < m; i++) A[i * m + i] *= (1.0 + 1e-10);
        for (int k = 0; k < m && use; k++) {
            int piv = k;
            for (int i = k + 1; i < m; i++)
                if (fabs(A[i * m + k]) > fabs(A[piv * m + k])) piv = i;
            if (!(fabs(A[piv * m + k]) > 1e-300)) {
                use = 0;
                break;
            }
            if (piv != k) {
                for (int jj = 0; jj < m; jj++) {
                    const double t = A[k * m + jj];
                    A[k * m + jj] = A[piv * m + jj];
                    A[piv * m + jj] = t;
                }
                const double t = rhs[k];
                rhs[k] = rhs[piv];
                rhs[piv] = t;
            }
            for (int i = k + 1; i < m; i++) {
                const double f = A[i * m + k] / A[k * m + k];
                for (int jj = k; jj < m; jj++) A[i * m + jj] -= f * A[k * m + jj];
                rhs[i] -= f * rhs[k];
            }
        }
        if (use)
            for (int k = m - 1; k >= 0; k--) {
                double s = rhs[k];
                for (int jj = k + 1; jj < m; jj++) s -= A[k * m + jj] * gam[jj];
                gam[k] = s / A[k * m + k];
            }
        s_use = use;
    }
    __syncthreads();
    // 3. mixed input charges; the history slot `head` takes (q_in, r)
    const int use = s_use;
    for (int a = tid; a < natoms; a += blockDim.x) {
        const double qi = qin[a], r = qout[a] - qi;
        double qb = qi, rb = r;
        if (use)
            for (int i = 0; i < m; i++) {
                qb -= gam[i] * (qi - hq[(int64_t)i * natoms + a]);
                rb -= gam[i] * (r - hr[(int64_t)i * natoms + a]);
            }
        if (history > 0) {
            hq[(int64_t)head * natoms + a] = qi;
            hr[(int64_t)head * natoms + a] = r;
        }
        qin[a] = qb + beta * rb;
    }
    __syncthreads();
    // 4. Coulomb shift of the new input charges
    for (int a = tid; a < natoms; a += blockDim.x) {
        double s = 0.0;
        for (int k = g_rp[a]; k < g_rp[a + 1]; k++) s += g_v[k] * (qin[g_ci[k]] - q0[g_ci[k]]);
        V[a] = s;
        shift[4 * a + 0] = s;
        shift[4 * a + 1] = s;
        shift[4 * a + 2] = s;
        shift[4 * a + 3] = s;
    }
    if (tid == 0 && history > 0) {
        meta[1] = (head + 1) % history;
        meta[0] = m < history ? m + 1 : history;
    }
}

void launch_scc_update(cudaStream_t st, DevScc &s, const double *qout, double beta, int history,
                       double tol, double *shift, DevState *state)
{
    k_scc_update<<<1, 1024, 0, st>>>(s.natoms, qout, s.qin, s.q0, s.hist_q, s.hist_r, s.hist_meta,
                                     beta, history, tol, s.rowptr, s.colidx, s.val, s.V, shift,
                                     state);
}

void launch_build_x(cudaStream_t st, const DevMatrix &m, const double *shift, int precision,
                    const DevState *state)
{
    const int64_t tot = m.nnzb * 16;
    const int T = 256;
    k_build_x<<<(unsigned)((tot + T - 1) / T), T, 0, st>>>(
        m.nnzb, m.blkrow, m.colidx, m.h0, shift, state, precision == TB_PREC_FP32 ? m.x32 : nullptr,
        precision == TB_PREC_FP64 ? m.x64 : nullptr, m.xdiag32);
}

}  // namespace tb

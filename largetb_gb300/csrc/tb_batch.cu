// tb_batch.cu -- many structures of uneven size solved together (K8).
//
// The structures are concatenated block-diagonally: structure s owns block
// rows [ao_s, ao_{s+1}) and orbitals [4 ao_s, 4 ao_{s+1}).  Each structure is
// one identity slab (all of its columns, B_s = n_s rounded up to 64, stored
// chunk-major [B_s/64][n_s][64]), so every Chebyshev step of every
// still-active structure is ONE launch over a list of (structure, row group,
// 64-column chunk) tiles; row groups never cross a structure boundary.  The
// step is the pipelined kernel (k_cheb_f32_pipe over a tile list: one
// persistent CTA per SM, bulk copies of each tile's halo rows into a
// shared-memory ring); when its stage does not fit, or fp32_kernel asks for
// TB_FP32_STAGED, k_bt_cheb_f32 stages each unit through shared memory as the
// single-structure staged kernel does.  After each step a
// reduction turns the per-group column dot products into moments, so the
// scratch holds one step of partials.  Gershgorin scaling, the damped DOS,
// the mu multisection, the Fermi coefficients, charges, band energy and the
// Anderson SCC update all run per structure (grid dimension = structure), with
// per-structure device state; a structure that converges drops out of the
// unit list and keeps its charges.
//
// Reference counterparts are those of the single-structure path
// (withSP2_deltaH.cpp: GershGorinParallel 144-209, getKPE 1068-1185, runKPM
// 1528-1723, computeDiagonalElements 1296-1399, constructdeltaH 1414-1487, the
// SCC loop 1820-1840); the reference itself handles one structure per run.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "tb_f32x2.cuh"
#include "tb_internal.h"

namespace tb {
namespace {

constexpr double kPi = 3.141592653589793238463;
constexpr int kBtCols = 64;
constexpr int kBtWarps = 8;
constexpr int kBtR = 24;  // block rows per group (one beta-cristobalite cell)
// Below this beta_x the multisection uses e^{beta x_q} e^{-beta mu} (|t| <= 600,
// inside the FP64 range) instead of one exp per node and candidate.
constexpr double kBtEtabBeta = 300.0;

__device__ __forceinline__ double wsum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ double bsum(double v, double *sh)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    v = wsum(v);
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double t = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
    if (w == 0) t = wsum(t);
    if (threadIdx.x == 0) sh[0] = t;
    __syncthreads();
    const double r = sh[0];
    __syncthreads();
    return r;
}

__device__ __forceinline__ double fermi_d(double x, double mu, double beta)
{
    const double t = beta * (x - mu);
    if (t > 0) {
        const double e = exp(-t);
        return e / (1.0 + e);
    }
    return 1.0 / (1.0 + exp(t));
}

__device__ __forceinline__ void cpa16(void *smem_dst, const void *gmem_src)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem_src));
}
__device__ __forceinline__ void cpa_wait()
{
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

struct Unit {
    int32_t s, g, chunk, pad;
};

// ---- per-structure scaling ----
__global__ void __launch_bounds__(1024)
    k_bt_gershgorin(const int32_t *__restrict__ s_ao, const double *__restrict__ h0diag,
                    const double *__restrict__ radius, const double *__restrict__ shift,
                    const int32_t *__restrict__ active, double kT, int M, int nq_cap,
                    DevState *__restrict__ st)
{
    __shared__ double smin[32], smax[32];
    const int s = blockIdx.x;
    if (!active[s]) return;
    const int i0 = 4 * s_ao[s], i1 = 4 * s_ao[s + 1];
    double mn = INFINITY, mx = -INFINITY;
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        const double c = h0diag[i] + shift[i];
        mn = fmin(mn, c - radius[i]);
        mx = fmax(mx, c + radius[i]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        smin[w] = mn;
        smax[w] = mx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) {
            mn = fmin(mn, smin[i]);
            mx = fmax(mx, smax[i]);
        }
        DevState &S = st[s];
        S.lmin = mn;
        S.lmax = mx;
        S.a = 0.5 * (mx - mn);
        S.b = 0.5 * (mx + mn);
        S.status = (S.a > 0 && isfinite(S.a)) ? 0 : TB_ERR_SPECTRUM;
        S.beta_x = kT > 0 ? S.a / kT : 0.0;
        double need = 4.0 * M;
        if (S.beta_x > 0 && 13.0 * S.beta_x > need) need = 13.0 * S.beta_x;
        if (need < 256) need = 256;
        int nq = 256;
        while (nq < need && nq < (1 << 22)) nq *= 2;
        if (nq > nq_cap) S.status = TB_ERR_SPECTRUM;
        S.nq = nq > nq_cap ? nq_cap : nq;
        S.bisect_done = 0;
        S.bisect_rounds = 0;
        S.lo = -1.0;
        S.hi = 1.0;
        S.ticket = 0u;
    }
}

__global__ void k_bt_build_x(int64_t nnzb, const int32_t *__restrict__ blkrow,
                             const int32_t *__restrict__ colidx, const int32_t *__restrict__ s_of_atom,
                             const int32_t *__restrict__ active, const double *__restrict__ h0,
                             const double *__restrict__ shift, const DevState *__restrict__ st,
                             float *__restrict__ x32, float *__restrict__ xdiag32)
{
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nnzb * 16) return;
    const int64_t t = e >> 4;
    const int rc = (int)(e & 15), r = rc >> 2, c = rc & 3;
    const int I = blkrow[t];
    const int s = s_of_atom[I];
    if (!active[s]) return;
    const bool diag = colidx[t] == I && r == c;
    double v = h0[e];
    if (diag) v = v + shift[4 * I + r] - st[s].b;
    v = v / st[s].a;
    x32[e] = (float)v;
    if (diag) xdiag32[4 * I + r] = (float)v;
}

__global__ void k_bt_identity(const Unit *__restrict__ units, int nunits, const int32_t *__restrict__ s_ao,
                              const int32_t *__restrict__ s_B, const int64_t *__restrict__ s_toff,
                              const int32_t *__restrict__ grp_I0, float *__restrict__ T0)
{
    // one unit: its group's rows x its 64 columns of the identity
    const int u = blockIdx.x;
    if (u >= nunits) return;
    const Unit un = units[u];
    const int ao = s_ao[un.s], ns = 4 * (s_ao[un.s + 1] - ao);
    const int I0 = grp_I0[un.g], I1 = grp_I0[un.g + 1];
    float *T = T0 + s_toff[un.s] + (int64_t)un.chunk * ns * kBtCols;  // chunk-major [B/64][n_s][64]
    const int col0 = un.chunk * kBtCols;
    for (int e = threadIdx.x; e < (I1 - I0) * 4 * kBtCols; e += blockDim.x) {
        const int rr = e / kBtCols, j = e % kBtCols;
        const int row = 4 * (I0 - ao) + rr;
        T[(int64_t)row * kBtCols + j] = (row == col0 + j) ? 1.f : 0.f;
    }
}

// ---- one FP32 Chebyshev step for every unit (staged as k_cheb_f32_staged) ----
__global__ void __launch_bounds__(32 * kBtWarps)
    k_bt_cheb_f32(const Unit *__restrict__ units, const int32_t *__restrict__ s_ao,
                  const int32_t *__restrict__ s_B, const int64_t *__restrict__ s_toff,
                  const int64_t *__restrict__ s_poff, const int32_t *__restrict__ s_g0,
                  const int32_t *__restrict__ grp_I0, const int32_t *__restrict__ rowptr,
                  const int32_t *__restrict__ lcol, const int32_t *__restrict__ lself,
                  const int32_t *__restrict__ grp_ptr, const int32_t *__restrict__ grp_rows,
                  const float *__restrict__ x32, const float *__restrict__ Tin_base,
                  float *__restrict__ Tout_base, int first, float2 *__restrict__ partial, int maxU,
                  int maxBlk)
{
    extern __shared__ float4 bsm4[];
    float *sT = reinterpret_cast<float *>(bsm4);
    float *sP = sT + maxU * 4 * kBtCols;
    float *sX = sP + kBtR * 4 * kBtCols;
    int *sU = reinterpret_cast<int *>(sX + maxBlk * 16);
    int *sL = sU + maxU;
    int *sR = sL + maxBlk;
    const Unit un = units[blockIdx.x];
    const int s = un.s, g = un.g, tid = threadIdx.x;
    const int ao = s_ao[s], B = s_B[s], ns = 4 * (s_ao[s + 1] - ao);
    // this unit's 64-column chunk of the structure's chunk-major slabs
    const int64_t coff = s_toff[s] + (int64_t)un.chunk * ns * kBtCols;
    const float *Tin = Tin_base + coff;
    float *Tout = Tout_base + coff;
    const int I0 = grp_I0[g], I1 = grp_I0[g + 1], nr = I1 - I0;
    const int u0 = grp_ptr[g], nu = grp_ptr[g + 1] - u0;
    const int tb0 = rowptr[I0], nbk = rowptr[I1] - tb0;
    const int col0 = un.chunk * kBtCols;
    for (int i = tid; i < nu; i += blockDim.x) sU[i] = grp_rows[u0 + i] - ao;
    for (int i = tid; i < nbk; i += blockDim.x) sL[i] = lcol[tb0 + i];
    for (int i = tid; i <= nr; i += blockDim.x) sR[i] = rowptr[I0 + i] - tb0;
    for (int idx = tid; idx < nbk * 4; idx += blockDim.x) cpa16(sX + idx * 4, x32 + (int64_t)tb0 * 16 + idx * 4);
    if (!first)
        for (int idx = tid; idx < nr * 64; idx += blockDim.x) {
            const int r = idx >> 6, m = (idx >> 4) & 3, sg = idx & 15;
            cpa16(sP + (r * 4 + m) * kBtCols + sg * 4,
                  Tout + (int64_t)(4 * (I0 - ao + r) + m) * kBtCols + sg * 4);
        }
    __syncthreads();
    for (int idx = tid; idx < nu * 64; idx += blockDim.x) {
        const int u = idx >> 6, m = (idx >> 4) & 3, sg = idx & 15;
        cpa16(sT + (u * 4 + m) * kBtCols + sg * 4, Tin + (int64_t)(4 * sU[u] + m) * kBtCols + sg * 4);
    }
    cpa_wait();
    __syncthreads();
    const int lane = tid & 31, w = tid >> 5, c = 2 * lane;
    // pairs (hi, lo) packed over columns (c, c+1): <T_k,T_k> in (eh, el), <T_k,T_{k+1}> in (oh, ol)
    float2 eh = make_float2(0.f, 0.f), el = eh, oh = eh, ol = eh;
    for (int r = w; r < nr; r += kBtWarps) {
        const int I = I0 + r;
        float2 acc[4];  // row q of the block row, columns (c, c+1)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[q] = make_float2(0.f, 0.f);
        for (int t = sR[r]; t < sR[r + 1]; t++) {
            const float *tv = sT + sL[t] * 4 * kBtCols + c;
            float2 v[4];
#pragma unroll
            for (int m = 0; m < 4; m++) v[m] = *reinterpret_cast<const float2 *>(tv + m * kBtCols);
            block_fma2(acc, reinterpret_cast<const float4 *>(sX + t * 16), v);
        }
        const float *own = sT + lself[I] * 4 * kBtCols + c;
        float2 ee = make_float2(0.f, 0.f), eo = ee;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const float2 ov = *reinterpret_cast<const float2 *>(own + q * kBtCols);
            float2 o = acc[q];
            if (!first) o = cheb_next2(acc[q], *reinterpret_cast<const float2 *>(sP + (r * 4 + q) * kBtCols + c));
            *reinterpret_cast<float2 *>(Tout + (int64_t)(4 * (I - ao) + q) * kBtCols + c) = o;
            ee = __ffma2_rn(ov, ov, ee);
            eo = __ffma2_rn(ov, o, eo);
        }
        pair_add2(eh, el, ee);
        pair_add2(oh, ol, eo);
    }
    __syncthreads();
    float *red = reinterpret_cast<float *>(bsm4);  // [warp][col][which][hi, lo]
    float4 *rb = reinterpret_cast<float4 *>(red + ((size_t)w * kBtCols + c) * 4);
    rb[0] = make_float4(eh.x, el.x, oh.x, ol.x);
    rb[1] = make_float4(eh.y, el.y, oh.y, ol.y);
    __syncthreads();
    if (tid < 2 * kBtCols) {
        const int j = tid >> 1, which = tid & 1;
        float hsum = 0.f, lsum = 0.f;
#pragma unroll
        for (int q = 0; q < kBtWarps; q++) {
            const float2 v = *reinterpret_cast<const float2 *>(red + ((size_t)q * kBtCols + j) * 4 + which * 2);
            pair_add(hsum, lsum, v.x);
            lsum += v.y;
        }
        partial[s_poff[s] + ((int64_t)(g - s_g0[s]) * B + col0 + j) * 2 + which] = make_float2(hsum, lsum);
    }
}

// moments 2k and 2k+1 of every orbital of the active structures
__global__ void k_bt_finalize(int n_total, int k, int M, const int32_t *__restrict__ s_of_atom,
                              const int32_t *__restrict__ active, const int32_t *__restrict__ s_ao,
                              const int32_t *__restrict__ s_B, const int64_t *__restrict__ s_poff,
                              const int32_t *__restrict__ s_g0, const float2 *__restrict__ partial,
                              const float *__restrict__ xdiag32, double *__restrict__ d)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_total) return;
    const int s = s_of_atom[i >> 2];
    if (!active[s]) return;
    const int j = i - 4 * s_ao[s], B = s_B[s], G = s_g0[s + 1] - s_g0[s];
    // (e, o) of column j in group g: one 16-byte load at [g][B][2] float2
    // (s_poff is even, so the base stays 16-byte aligned)
    const float4 *p = reinterpret_cast<const float4 *>(partial + s_poff[s]) + j;
    float eh = 0.f, el = 0.f, oh = 0.f, ol = 0.f;
    int g = 0;
    for (; g + 8 <= G; g += 8) {
        float4 v[8];
#pragma unroll
        for (int u = 0; u < 8; u++) v[u] = __ldg(p + (int64_t)(g + u) * B);
#pragma unroll
        for (int u = 0; u < 8; u++) {
            pair_add(eh, el, v[u].x);
            el += v[u].y;
            pair_add(oh, ol, v[u].z);
            ol += v[u].w;
        }
    }
    for (; g < G; g++) {
        const float4 v = __ldg(p + (int64_t)g * B);
        pair_add(eh, el, v.x);
        el += v.y;
        pair_add(oh, ol, v.z);
        ol += v.w;
    }
    const double se = (double)eh + (double)el, so = (double)oh + (double)ol;
    if (2 * k <= M) d[(int64_t)(2 * k) * n_total + i] = 2.0 * se - 1.0;
    if (2 * k + 1 <= M) d[(int64_t)(2 * k + 1) * n_total + i] = 2.0 * so - (double)xdiag32[i];
}

__global__ void __launch_bounds__(256)
    k_bt_moment_sums(const double *__restrict__ d, int n_total, int M, const int32_t *__restrict__ s_ao,
                     const int32_t *__restrict__ active, double *__restrict__ mom)
{
    __shared__ double sh[32];
    const int k = blockIdx.x, s = blockIdx.y;
    if (!active[s]) return;
    double v = 0.0;
    for (int i = 4 * s_ao[s] + threadIdx.x; i < 4 * s_ao[s + 1]; i += blockDim.x) v += d[(int64_t)k * n_total + i];
    v = bsum(v, sh);
    if (threadIdx.x == 0) mom[(int64_t)s * (M + 1) + k] = v;
}

// Node kernels index the cosine table of k_cos_table (tab[j] = cos(pi j /
// (2 nq_cap))): cos(theta_q) = tab[(2q+1) r], cos(k theta_q) = tab[(k (2q+1)
// mod 4 nq) r], r = nq > 0 ? nq_cap / nq : 1, as in the single-structure kernels.
__global__ void k_bt_dos_nodes(const double *__restrict__ g, const double *__restrict__ mom, int M,
                               const DevState *__restrict__ st, const int32_t *__restrict__ active,
                               int nq_cap, const double *__restrict__ tab, double *__restrict__ rho,
                               double *__restrict__ ebx)
{
    extern __shared__ double wk[];  // (2 - delta_k0) g_k mu_k of this structure
    const int s = blockIdx.y;
    if (!active[s]) return;
    const double *ms = mom + (int64_t)s * (M + 1);
    for (int kk = threadIdx.x; kk < M; kk += blockDim.x) wk[kk] = kk == 0 ? g[0] * ms[0] : 2.0 * g[kk] * ms[kk];
    __syncthreads();
    const int nq = min(st[s].nq, nq_cap), r = nq > 0 ? nq_cap / nq : 1;
    const size_t cmask = 4 * (size_t)nq_cap - 1;  // keeps every table index in range
    const unsigned mask = 4u * (unsigned)nq - 1u;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x) {
        const unsigned step = 2u * (unsigned)q + 1u;
        unsigned j = 0;
        double v = wk[0];
        for (int kk = 1; kk < M; kk++) {
            j = (j + step) & mask;
            v += wk[kk] * tab[((size_t)j * r) & cmask];
        }
        rho[(int64_t)s * nq_cap + q] = v;
        // e^{beta_x x_q} for the multisection; unused above kBtEtabBeta
        const double bx = st[s].beta_x;
        ebx[(int64_t)s * nq_cap + q] = bx <= kBtEtabBeta ? exp(bx * tab[((size_t)step * r) & cmask]) : 0.0;
    }
}

__global__ void k_bt_fermi_nodes(const DevState *__restrict__ st_all, const int32_t *__restrict__ active,
                                 int nq_cap, const double *__restrict__ tab, double *__restrict__ fq)
{
    const int s = blockIdx.y;
    if (!active[s]) return;
    const DevState *st = st_all + s;
    const double beta = st->beta_x, mu = st->mu_x;
    if (!(beta > 0)) return;
    const int nq = min(st->nq, nq_cap), r = nq > 0 ? nq_cap / nq : 1;
    const size_t cmask = 4 * (size_t)nq_cap - 1;  // keeps every table index in range
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x)
        fq[(int64_t)s * nq_cap + q] = fermi_d(tab[((size_t)(2 * q + 1) * r) & cmask], mu, beta);
}

__global__ void __launch_bounds__(256)
    k_bt_bisect(const double *__restrict__ rho, const double *__restrict__ ebx, int nq_cap,
                const double *__restrict__ tab,
                const double *__restrict__ g,
                const double *__restrict__ mom, int M, const double *__restrict__ n_elec, double tol_n,
                int round, int last_round, const int32_t *__restrict__ active, double *__restrict__ cand,
                DevState *__restrict__ st_all)
{
    __shared__ double sh[32];
    __shared__ int s_last;
    const int s = blockIdx.y, P = gridDim.x, p = blockIdx.x;
    DevState *st = st_all + s;
    if (!active[s] || st->bisect_done) return;
    const double lo = st->lo, hi = st->hi, beta = st->beta_x, ne = n_elec[s];
    const double mu = lo + (hi - lo) * (double)p / (double)(P - 1);
    const double *ms = mom + (int64_t)s * (M + 1);
    double v = 0.0;
    if (beta > 0) {
        const int nq = st->nq, r = nq > 0 ? nq_cap / nq : 1;
        const size_t cmask = 4 * (size_t)nq_cap - 1;  // keeps every table index in range
        const double *rs = rho + (int64_t)s * nq_cap;
        if (beta <= kBtEtabBeta) {
            // f(x_q) = 1 / (1 + e^{beta x_q} e^{-beta mu}): one exp per candidate
            const double C = exp(-beta * mu), *eb = ebx + (int64_t)s * nq_cap;
            for (int q = threadIdx.x; q < nq; q += blockDim.x) v += rs[q] / (1.0 + eb[q] * C);
        } else {
            for (int q = threadIdx.x; q < nq; q += blockDim.x)
                v += fermi_d(tab[((size_t)(2 * q + 1) * r) & cmask], mu, beta) * rs[q];
        }
        v = 2.0 * bsum(v, sh) / nq;
    } else {
        const double th = acos(mu);
        for (int kk = threadIdx.x; kk < M; kk += blockDim.x)
            v += ((kk == 0) ? 1.0 - th / kPi : -2.0 * sin(kk * th) / (kk * kPi)) * g[kk] * ms[kk];
        v = 2.0 * bsum(v, sh);
    }
    double *cs = cand + (int64_t)s * P;
    if (threadIdx.x == 0) {
        cs[p] = v;
        __threadfence();
        s_last = atomicAdd(&st->ticket, 1u) == (unsigned)(P - 1);
    }
    __syncthreads();
    if (!s_last || threadIdx.x != 0) return;
    __threadfence();
    st->ticket = 0u;
    volatile double *vc = cs;
    st->bisect_rounds = round + 1;
    if (round == 0 && !(vc[0] <= ne && ne <= vc[P - 1])) {
        st->status = TB_ERR_BISECTION;
        st->bisect_done = 1;
        st->mu_x = 0.0;
        return;
    }
    int best = 0, first_ge = P - 1;
    double bd = fabs(vc[0] - ne);
    for (int i = 0; i < P; i++) {
        const double dv = fabs(vc[i] - ne);
        if (dv < bd) {
            bd = dv;
            best = i;
        }
    }
    for (int i = 0; i < P; i++)
        if (vc[i] >= ne) {
            first_ge = i;
            break;
        }
    const double h = (hi - lo) / (double)(P - 1);
    if (bd <= tol_n) {
        st->mu_x = lo + h * best;
        st->bisect_done = 1;
        return;
    }
    st->lo = (first_ge > 0) ? lo + h * (first_ge - 1) : lo;
    st->hi = lo + h * first_ge;
    if (round == last_round) {
        st->mu_x = 0.5 * (st->lo + st->hi);
        st->bisect_done = 1;
    }
}

__global__ void __launch_bounds__(256)
    k_bt_coeffs(int M, DevState *__restrict__ st_all, const int32_t *__restrict__ active, int nq_cap,
                const double *__restrict__ tab, const double *__restrict__ fq, double *__restrict__ c)
{
    __shared__ double sh[32];
    const int k = blockIdx.x, s = blockIdx.y;
    if (!active[s]) return;
    DevState *st = st_all + s;
    const double mu = st->mu_x, beta = st->beta_x;
    if (threadIdx.x == 0 && k == 0) st->mu = st->a * mu + st->b;
    double *cs = c + (int64_t)s * M;
    if (beta > 0) {
        const int nq = st->nq, r = nq > 0 ? nq_cap / nq : 1;
        const size_t cmask = 4 * (size_t)nq_cap - 1;  // keeps every table index in range
        const unsigned mask = 4u * (unsigned)nq - 1u;
        const double *fs = fq + (int64_t)s * nq_cap;
        double v = 0.0;
        for (int q = threadIdx.x; q < nq; q += blockDim.x)
            v += fs[q] * tab[((size_t)(((unsigned)k * (2u * (unsigned)q + 1u)) & mask) * r) & cmask];
        v = bsum(v, sh);
        if (threadIdx.x == 0) cs[k] = (k == 0 ? 1.0 : 2.0) * v / nq;
    } else if (threadIdx.x == 0) {
        const double th = acos(mu);
        cs[k] = (k == 0) ? 1.0 - th / kPi : -2.0 * sin(k * th) / (k * kPi);
    }
}

__global__ void k_bt_charges(const double *__restrict__ d, const double *__restrict__ c,
                             const double *__restrict__ g, int M, int n_total, int na_total,
                             const int32_t *__restrict__ s_of_atom, const int32_t *__restrict__ active,
                             double *__restrict__ diagP, double *__restrict__ q)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= na_total) return;
    const int s = s_of_atom[a];
    if (!active[s]) return;
    const double *cs = c + (int64_t)s * M;
    double p[4] = {0, 0, 0, 0};
    for (int k = 0; k < M; k++) {
        const double w = cs[k] * g[k];
#pragma unroll
        for (int r = 0; r < 4; r++) p[r] += w * d[(int64_t)k * n_total + 4 * a + r];
    }
    for (int r = 0; r < 4; r++) diagP[4 * a + r] = p[r];
    q[a] = 2.0 * (p[0] + p[1] + p[2] + p[3]);
}

__global__ void __launch_bounds__(256)
    k_bt_eband(const double *__restrict__ c, const double *__restrict__ g, const double *__restrict__ mom,
               int M, const int32_t *__restrict__ active, DevState *__restrict__ st_all)
{
    __shared__ double sh[32];
    const int s = blockIdx.x;
    if (!active[s]) return;
    DevState *st = st_all + s;
    const double *cs = c + (int64_t)s * M, *ms = mom + (int64_t)s * (M + 1);
    double ne = 0.0, eb = 0.0;
    for (int k = threadIdx.x; k < M; k += blockDim.x) {
        const double w = cs[k] * g[k];
        const double tx = (k == 0) ? ms[1] : 0.5 * (ms[k + 1] + ms[k - 1]);
        ne += w * ms[k];
        eb += w * (st->a * tx + st->b * ms[k]);
    }
    ne = bsum(ne, sh);
    eb = bsum(eb, sh);
    if (threadIdx.x == 0) {
        st->n_found = 2.0 * ne;
        st->e_band = 2.0 * eb;
    }
}

// Per-structure SCC update (one CTA per structure): residual, convergence,
// Anderson mixing over the structure's atoms, new Coulomb shift.
__global__ void __launch_bounds__(1024)
    k_bt_scc_update(const int32_t *__restrict__ s_ao, const double *__restrict__ qout,
                    double *__restrict__ qin, const double *__restrict__ q0, double *__restrict__ hq,
                    double *__restrict__ hr, int na_total, int32_t *__restrict__ meta, double beta,
                    int history, double tol, const int32_t *__restrict__ g_rp,
                    const int32_t *__restrict__ g_ci, const double *__restrict__ g_v,
                    double *__restrict__ shift, int32_t *__restrict__ active, DevState *__restrict__ st_all)
{
    __shared__ double sh[32];
    __shared__ double A[kMaxHistory * kMaxHistory], rhs[kMaxHistory], gam[kMaxHistory];
    __shared__ int s_use, s_stop;
    const int s = blockIdx.x;
    if (!active[s]) return;
    DevState *st = st_all + s;
    const int a0 = s_ao[s], a1 = s_ao[s + 1];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, nw = blockDim.x >> 5;
    double mx = 0.0;
    for (int a = a0 + tid; a < a1; a += blockDim.x) mx = fmax(mx, fabs(qout[a] - qin[a]));
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) sh[w] = mx;
    __syncthreads();
    if (tid == 0) {
        double m = 0.0;
        for (int i = 0; i < nw; i++) m = fmax(m, sh[i]);
        st->dq_max = m;
        s_stop = 0;
        if (st->status) {
            active[s] = 0;
            s_stop = 1;
        } else if (!(m < 1e3)) {
            st->status = TB_ERR_DIVERGED;
            active[s] = 0;
            s_stop = 1;
        } else if (m < tol) {
            st->converged = 1;
            active[s] = 0;
            s_stop = 1;
        }
    }
    __syncthreads();
    if (s_stop) return;
    int32_t *mt = meta + 2 * s;
    const int m = mt[0], head = mt[1];
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
        double v = 0.0;
        for (int a = a0 + lane; a < a1; a += 32) {
            const double r = qout[a] - qin[a];
            const double di = r - hr[(int64_t)i * na_total + a];
            const double dj = is_rhs ? r : r - hr[(int64_t)j * na_total + a];
            v += di * dj;
        }
        v = wsum(v);
        if (lane == 0) {
            if (is_rhs)
                rhs[i] = v;
            else {
                A[i * m + j] = v;
                A[j * m + i] = v;
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
                double v = rhs[k];
                for (int jj = k + 1; jj < m; jj++) v -= A[k * m + jj] * gam[jj];
                gam[k] = v / A[k * m + k];
            }
        s_use = use;
    }
    __syncthreads();
    const int use = s_use;
    for (int a = a0 + tid; a < a1; a += blockDim.x) {
        const double qi = qin[a], r = qout[a] - qi;
        double qb = qi, rb = r;
        if (use)
            for (int i = 0; i < m; i++) {
                qb -= gam[i] * (qi - hq[(int64_t)i * na_total + a]);
                rb -= gam[i] * (r - hr[(int64_t)i * na_total + a]);
            }
        if (history > 0) {
            hq[(int64_t)head * na_total + a] = qi;
            hr[(int64_t)head * na_total + a] = r;
        }
        qin[a] = qb + beta * rb;
    }
    __syncthreads();
    for (int a = a0 + tid; a < a1; a += blockDim.x) {
        double v = 0.0;
        for (int k = g_rp[a]; k < g_rp[a + 1]; k++) v += g_v[k] * (qin[g_ci[k]] - q0[g_ci[k]]);
        shift[4 * a + 0] = v;
        shift[4 * a + 1] = v;
        shift[4 * a + 2] = v;
        shift[4 * a + 3] = v;
    }
    if (tid == 0 && history > 0) {
        mt[1] = (head + 1) % history;
        mt[0] = m < history ? m + 1 : history;
    }
}

__global__ void k_bt_coulomb(int na_total, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci,
                             const double *__restrict__ gv, const double *__restrict__ q,
                             const double *__restrict__ q0, double *__restrict__ shift)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= na_total) return;
    double v = 0.0;
    for (int k = rp[a]; k < rp[a + 1]; k++) v += gv[k] * (q[ci[k]] - q0[ci[k]]);
    for (int r = 0; r < 4; r++) shift[4 * a + r] = v;
}

size_t bt_smem(int maxU, int maxBlk)
{
    const size_t b = (size_t)(maxU * 4 * kBtCols + kBtR * 4 * kBtCols + maxBlk * 16) * sizeof(float) +
                     (size_t)(maxU + maxBlk + kBtR + 1) * sizeof(int);
    const size_t red = (size_t)kBtWarps * kBtCols * 4 * sizeof(float);  // FP32 pairs of 2 sums per column
    return std::max(b, red);
}

}  // namespace
}  // namespace tb

using namespace tb;

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct tb_batch {
    tb_params p{};
    int S = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    // host inputs, per structure
    std::vector<HostBsr> hb;
    std::vector<std::vector<int32_t>> grp, gci;
    std::vector<std::vector<double>> gv, q0;
    std::vector<int> natoms;
    std::vector<char> have;
    bool built = false;
    // device
    int n_total = 0, na_total = 0, M = 0, K = 0, nq_cap = 0, maxU = 0, maxBlk = 0, G = 0;
    int64_t nnzb = 0, t_floats = 0, p_doubles = 0;
    std::vector<void *> allocs;
    int32_t *rowptr = nullptr, *colidx = nullptr, *blkrow = nullptr, *s_ao = nullptr, *s_of_atom = nullptr;
    int32_t *s_B = nullptr, *s_g0 = nullptr, *grp_I0 = nullptr, *grp_ptr = nullptr, *grp_rows = nullptr;
    int32_t *lcol = nullptr, *lself = nullptr, *g_rp = nullptr, *g_ci = nullptr, *meta = nullptr, *active = nullptr;
    int64_t *s_toff = nullptr, *s_poff = nullptr;
    double *h0 = nullptr, *h0diag = nullptr, *radius = nullptr, *d = nullptr, *mom = nullptr, *c = nullptr;
    double *g = nullptr, *rho = nullptr, *cand = nullptr, *diagP = nullptr, *q = nullptr, *partial = nullptr;
    double *fq = nullptr, *costab = nullptr;  // Fermi function at the nodes [S][nq_cap]; cosine table 4 nq_cap
    double *ebx = nullptr;                      // e^{beta_x x_q} at the nodes [S][nq_cap]
    double *g_v = nullptr, *q0d = nullptr, *qin = nullptr, *shift = nullptr, *hq = nullptr, *hr = nullptr;
    double *ne = nullptr;
    float *x32 = nullptr, *xdiag32 = nullptr, *T0 = nullptr, *T1 = nullptr;
    Unit *units = nullptr;
    int units_cap = 0;
    // pipelined step (k_cheb_f32_pipe over a tile list): its plan (stages ==
    // 0: unavailable, the staged step k_bt_cheb_f32 runs) and tile list
    PipePlan pl;
    PipeBatchTile *ptiles = nullptr;
    int ptiles_cap = 0;
    DevState *st = nullptr;
    std::vector<int32_t> h_ao, h_B, h_g0, h_grpI0;
    std::vector<int64_t> h_toff, h_poff;
    // the SCC iteration as a CUDA graph, captured per active set (its grid
    // sizes and unit list change only when a structure converges)
    cudaGraphExec_t graph = nullptr;
    std::vector<int32_t> graph_act;
};

namespace {

int bfail(tb_batch *b, int code, const std::string &m)
{
    b->err = m;
    return code;
}

template <typename T>
int balloc(tb_batch *b, T *&p, size_t n)
{
    cudaError_t e = cudaMalloc((void **)&p, std::max<size_t>(n, 1) * sizeof(T));
    if (e != cudaSuccess) {
        p = nullptr;
        return bfail(b, TB_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    b->allocs.push_back((void *)p);
    return TB_OK;
}

template <typename T>
int bupload(tb_batch *b, T *&p, const std::vector<T> &v)
{
    int rc = balloc(b, p, v.size());
    if (rc) return rc;
    if (!v.empty()) cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, b->stream);
    return TB_OK;
}

void bfree(tb_batch *b)
{
    for (void *p : b->allocs) cudaFree(p);
    b->allocs.clear();
    b->built = false;
}

// Plan of the pipelined step over the batch's row groups (the groups of
// k_bt_cheb_f32: kBtR block rows inside each structure, numbered across the
// batch); rowptr: the concatenated block-row pointers.  Leaves b->pl.stages
// at 0 when a stage does not fit in shared memory.
int batch_pipe_plan(tb_batch *b, const std::vector<int32_t> &rowptr)
{
    b->pl = PipePlan{};
    std::vector<int32_t> hdr, rec, U, runs;
    std::vector<std::vector<int32_t>> grun;
    int maxU = 0, maxBlk = 0, rec_cap = 0, maxRuns = 0;
    for (int s = 0; s < b->S; s++) {
        const HostBsr &hb = b->hb[s];
        const int nb = b->natoms[s];
        for (int I0 = 0; I0 < nb; I0 += kBtR) {
            hdr.resize(hdr.size() + 8);
            pipe_group_records(hb.brow.data(), hb.bcol.data(), I0, std::min(nb, I0 + kBtR), rowptr[b->h_ao[s]],
                               &hdr[hdr.size() - 8], rec, runs, U);
            grun.push_back(runs);
            const int32_t *h = &hdr[hdr.size() - 8];
            maxU = std::max(maxU, h[0]);
            maxBlk = std::max(maxBlk, h[2]);
            rec_cap = std::max(rec_cap, h[4]);
            maxRuns = std::max(maxRuns, h[6]);
        }
    }
    const size_t stage_bytes = cheb_f32_pipe_stage_bytes(kBtR, maxU, maxBlk, rec_cap);
    int stages = 3;
    while (stages >= 2 && cheb_f32_pipe_smem(stage_bytes, stages) > 227 * 1024) stages--;
    int per_sm = 0;
    if (stages < 2 || cheb_f32_pipe_configure(cheb_f32_pipe_smem(stage_bytes, stages), &per_sm, true) != 0 ||
        per_sm < 1) {
        cudaGetLastError();
        return TB_OK;  // the staged step stays
    }
    const int G = (int)grun.size();
    const int run_stride = (maxRuns + 31) / 32 * 32;
    std::vector<int32_t> runs_all((size_t)G * run_stride * 4, 0);
    for (int g = 0; g < G; g++)
        std::copy(grun[g].begin(), grun[g].end(), runs_all.begin() + (size_t)g * run_stride * 4);
    int rc;
    if ((rc = bupload(b, b->pl.hdr, hdr)) || (rc = bupload(b, b->pl.runs, runs_all)) ||
        (rc = bupload(b, b->pl.rec, rec)) || (rc = balloc(b, b->pl.err, 1)))
        return rc;
    cudaMemsetAsync(b->pl.err, 0, sizeof(int32_t), b->stream);
    int nsm = 152;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, b->p.device);
    b->pl.R = kBtR;
    b->pl.G = G;
    b->pl.maxU = maxU;
    b->pl.maxBlk = maxBlk;
    b->pl.stages = stages;
    b->pl.stage_bytes = stage_bytes;
    b->pl.nsm = nsm * per_sm;
    b->pl.run_stride = run_stride;
    return TB_OK;
}

// Concatenate the structures and lay out groups, slabs and scratch.
int batch_build(tb_batch *b)
{
    bfree(b);
    if (b->graph) {  // captured against the buffers being replaced
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    const int S = b->S;
    const int M = b->p.M;
    b->M = M;
    b->K = (M + 2) / 2;
    std::vector<int32_t> rowptr{0}, colidx, blkrow, s_ao{0}, s_of_atom, s_B, s_g0{0}, grp_I0{0}, grp_ptr{0},
        grp_rows, lcol, lself, g_rp{0}, g_ci;
    std::vector<int64_t> s_toff, s_poff;
    std::vector<double> h0, h0diag, radius, g_v, q0, ne;
    int64_t toff = 0, poff = 0;
    int ao = 0, maxU = 0, maxBlk = 0;
    double lmin = 1e300, lmax = -1e300;
    for (int s = 0; s < S; s++) {
        const HostBsr &hb = b->hb[s];
        const int nb = b->natoms[s];
        for (int I = 0; I < nb; I++) {
            for (int t = hb.brow[I]; t < hb.brow[I + 1]; t++) {
                colidx.push_back(hb.bcol[t] + ao);
                blkrow.push_back(I + ao);
            }
            rowptr.push_back((int32_t)colidx.size());
            s_of_atom.push_back(s);
        }
        h0.insert(h0.end(), hb.blk.begin(), hb.blk.end());
        h0diag.insert(h0diag.end(), hb.h0diag.begin(), hb.h0diag.end());
        radius.insert(radius.end(), hb.radius.begin(), hb.radius.end());
        lmin = std::min(lmin, hb.lmin);
        lmax = std::max(lmax, hb.lmax);
        const int Bs = ((4 * nb + kBtCols - 1) / kBtCols) * kBtCols;
        s_B.push_back(Bs);
        s_toff.push_back(toff);
        toff += (int64_t)4 * nb * Bs;
        // groups of kBtR block rows inside the structure
        const int G = (nb + kBtR - 1) / kBtR;
        s_poff.push_back(poff);
        poff += (int64_t)G * Bs * 2;
        for (int gg = 0; gg < G; gg++) {
            const int I0 = gg * kBtR, I1 = std::min(nb, I0 + kBtR);
            std::vector<int32_t> U;
            for (int t = hb.brow[I0]; t < hb.brow[I1]; t++) U.push_back(hb.bcol[t]);
            std::sort(U.begin(), U.end());
            U.erase(std::unique(U.begin(), U.end()), U.end());
            for (int t = hb.brow[I0]; t < hb.brow[I1]; t++)
                lcol.push_back((int32_t)(std::lower_bound(U.begin(), U.end(), hb.bcol[t]) - U.begin()));
            for (int I = I0; I < I1; I++)
                lself.push_back((int32_t)(std::lower_bound(U.begin(), U.end(), I) - U.begin()));
            for (int J : U) grp_rows.push_back(J + ao);
            grp_ptr.push_back((int32_t)grp_rows.size());
            grp_I0.push_back(I1 + ao);
            maxU = std::max(maxU, (int)U.size());
            maxBlk = std::max(maxBlk, hb.brow[I1] - hb.brow[I0]);
        }
        s_g0.push_back(s_g0.back() + G);
        // Gamma with global atom columns
        for (int a = 0; a < nb; a++) {
            for (int k = b->grp[s][a]; k < b->grp[s][a + 1]; k++) {
                g_ci.push_back(b->gci[s][k] + ao);
                g_v.push_back(b->gv[s][k]);
            }
            g_rp.push_back((int32_t)g_ci.size());
        }
        q0.insert(q0.end(), b->q0[s].begin(), b->q0[s].end());
        double n_e = 0.0;
        for (double v : b->q0[s]) n_e += v;
        ne.push_back(b->p.n_electrons > 0 ? b->p.n_electrons : n_e);
        ao += nb;
        s_ao.push_back(ao);
    }
    b->na_total = ao;
    b->n_total = 4 * ao;
    b->nnzb = (int64_t)colidx.size();
    b->maxU = maxU;
    b->maxBlk = maxBlk;
    b->G = s_g0.back();
    b->t_floats = toff;
    b->p_doubles = poff;
    b->h_ao = s_ao;
    b->h_B = s_B;
    b->h_toff = s_toff;
    b->h_poff = s_poff;
    b->h_g0 = s_g0;
    b->h_grpI0 = grp_I0;
    int nq_cap = 1 << 14;
    if (b->p.kT > 0) {
        double need = 13.0 * 2.0 * (lmax - lmin) / b->p.kT;
        while (nq_cap < need && nq_cap < (1 << 22)) nq_cap *= 2;
    }
    b->nq_cap = nq_cap;
    const int na = b->na_total, n = b->n_total;
    int rc = TB_OK;
#define BT(x) \
    if ((rc = (x))) return rc
    BT(bupload(b, b->rowptr, rowptr));
    BT(bupload(b, b->colidx, colidx));
    BT(bupload(b, b->blkrow, blkrow));
    BT(bupload(b, b->s_ao, s_ao));
    BT(bupload(b, b->s_of_atom, s_of_atom));
    BT(bupload(b, b->s_B, s_B));
    BT(bupload(b, b->s_g0, s_g0));
    BT(bupload(b, b->grp_I0, grp_I0));
    BT(bupload(b, b->grp_ptr, grp_ptr));
    BT(bupload(b, b->grp_rows, grp_rows));
    BT(bupload(b, b->lcol, lcol));
    BT(bupload(b, b->lself, lself));
    BT(bupload(b, b->g_rp, g_rp));
    BT(bupload(b, b->g_ci, g_ci));
    BT(bupload(b, b->s_toff, s_toff));
    BT(bupload(b, b->s_poff, s_poff));
    BT(bupload(b, b->h0, h0));
    BT(bupload(b, b->h0diag, h0diag));
    BT(bupload(b, b->radius, radius));
    BT(bupload(b, b->g_v, g_v));
    BT(bupload(b, b->q0d, q0));
    BT(bupload(b, b->ne, ne));
    BT(balloc(b, b->x32, (size_t)b->nnzb * 16));
    BT(balloc(b, b->xdiag32, (size_t)n));
    BT(balloc(b, b->T0, (size_t)b->t_floats));
    BT(balloc(b, b->T1, (size_t)b->t_floats));
    BT(balloc(b, b->partial, (size_t)b->p_doubles));
    BT(balloc(b, b->d, (size_t)(M + 1) * n));
    BT(balloc(b, b->mom, (size_t)S * (M + 1)));
    BT(balloc(b, b->c, (size_t)S * M));
    BT(balloc(b, b->rho, (size_t)S * nq_cap));
    BT(balloc(b, b->fq, (size_t)S * nq_cap));
    BT(balloc(b, b->ebx, (size_t)S * nq_cap));
    BT(balloc(b, b->costab, 4 * (size_t)nq_cap));
    launch_cos_table(b->stream, nq_cap, b->costab);
    BT(balloc(b, b->cand, (size_t)S * kBisectCand));
    BT(balloc(b, b->diagP, (size_t)n));
    BT(balloc(b, b->q, (size_t)na));
    BT(balloc(b, b->qin, (size_t)na));
    BT(balloc(b, b->shift, (size_t)n));
    BT(balloc(b, b->hq, (size_t)kMaxHistory * na));
    BT(balloc(b, b->hr, (size_t)kMaxHistory * na));
    BT(balloc(b, b->meta, (size_t)2 * S));
    BT(balloc(b, b->active, (size_t)S));
    BT(balloc(b, b->st, (size_t)S));
    {
        std::vector<double> gh(M, 1.0);
        if (b->p.kernel == TB_KERNEL_JACKSON) {
            const double N = M, cotv = std::cos(kPi / (N + 1)) / std::sin(kPi / (N + 1));
            for (int k = 0; k < M; k++)
                gh[k] = ((N - k + 1) * std::cos(kPi * k / (N + 1)) + std::sin(kPi * k / (N + 1)) * cotv) / (N + 1);
        }
        gh[0] = 1.0;
        BT(bupload(b, b->g, gh));
    }
    // the staged step needs all of its shared memory opted in
    const size_t smem = bt_smem(maxU, maxBlk);
    if (smem > 227 * 1024) return bfail(b, TB_ERR_UNSUPPORTED, "row-group halo too large for shared memory");
    cudaError_t e = cudaFuncSetAttribute(k_bt_cheb_f32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         smem_optin_max((const void *)k_bt_cheb_f32));
    if (e != cudaSuccess) return bfail(b, TB_ERR_CUDA, cudaGetErrorString(e));
    BT(batch_pipe_plan(b, rowptr));
    e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return bfail(b, TB_ERR_CUDA, cudaGetErrorString(e));
#undef BT
    b->built = true;
    return TB_OK;
}

}  // namespace

extern "C" {

int tb_batch_create(const tb_params *p, int32_t count, tb_batch **out)
{
    TB_ABI_TRY
    if (!out || !p || count < 1) return TB_ERR_INVALID_ARG;
    *out = nullptr;
    if (p->struct_size != sizeof(tb_params) || p->M < 2 || p->M > 6000 || p->mix_history < 0 ||
        p->mix_history > kMaxHistory || !(p->scc_tol > 0) || p->scc_max_iter < 1)
        return TB_ERR_INVALID_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || p->device < 0 || p->device >= ndev) {
        cudaGetLastError();
        return TB_ERR_NO_DEVICE;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, p->device) != cudaSuccess || !(prop.major == 10 && prop.minor == 3))
        return TB_ERR_NO_DEVICE;
    tb_batch *b = new (std::nothrow) tb_batch();
    if (!b) return TB_ERR_OUT_OF_MEMORY;
    b->p = *p;
    b->S = count;
    b->hb.resize(count);
    b->grp.resize(count);
    b->gci.resize(count);
    b->gv.resize(count);
    b->q0.resize(count);
    b->natoms.assign(count, 0);
    b->have.assign(count, 0);
    if (cudaSetDevice(p->device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete b;
        return TB_ERR_CUDA;
    }
    *out = b;
    return TB_OK;
    TB_ABI_CATCH
}

int tb_batch_destroy(tb_batch *b)
{
    TB_ABI_TRY
    if (!b) return TB_OK;
    cudaSetDevice(b->p.device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    bfree(b);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->units) cudaFree(b->units);
    if (b->ptiles) cudaFree(b->ptiles);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return TB_OK;
    TB_ABI_CATCH
}

const char *tb_batch_last_error(const tb_batch *b) { return b ? b->err.c_str() : "no batch"; }

int tb_batch_set(tb_batch *b, int32_t index, int32_t n, const int32_t *rowptr, const int32_t *colidx,
                 const double *vals, int32_t natoms, const int32_t *g_rowptr, const int32_t *g_colidx,
                 const double *g_vals, const double *q0)
{
    TB_ABI_TRY
    if (!b) return TB_ERR_INVALID_ARG;
    if (index < 0 || index >= b->S) return bfail(b, TB_ERR_INVALID_ARG, "index out of range");
    std::vector<int32_t> o2a(n > 0 ? n : 0);
    for (int i = 0; i < n; i++) o2a[i] = i / 4;
    int rc = host_csr_to_bsr(n, rowptr, colidx, vals, o2a.data(), natoms, b->hb[index], b->err);
    if (rc) return rc;
    rc = host_check_gamma(natoms, g_rowptr, g_colidx, g_vals, q0, b->err);
    if (rc) return rc;
    b->grp[index].assign(g_rowptr, g_rowptr + natoms + 1);
    b->gci[index].assign(g_colidx, g_colidx + g_rowptr[natoms]);
    b->gv[index].assign(g_vals, g_vals + g_rowptr[natoms]);
    b->q0[index].assign(q0, q0 + natoms);
    b->natoms[index] = natoms;
    b->have[index] = 1;
    b->built = false;
    return TB_OK;
    TB_ABI_CATCH
}

int tb_batch_scc_solve(tb_batch *b, const double *q_init, double *q, int32_t *iters, double *e_band,
                       double *mu, tb_report *rep)
{
    TB_ABI_TRY
    if (!b) return TB_ERR_INVALID_ARG;
    for (int s = 0; s < b->S; s++)
        if (!b->have[s]) return bfail(b, TB_ERR_NOT_READY, "structure " + std::to_string(s) + " not set");
    if (cudaSetDevice(b->p.device) != cudaSuccess) return bfail(b, TB_ERR_CUDA, "cudaSetDevice");
    if (!b->built) {
        int rc = batch_build(b);
        if (rc) return rc;
    }
    const int S = b->S, M = b->M, K = b->K, na = b->na_total, n = b->n_total;
    cudaStream_t st = b->stream;
    cudaEvent_t e0, e1, m0, m1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventCreate(&m0);
    cudaEventCreate(&m1);
    cudaEventRecord(e0, st);
    int64_t launches = 0, spmm = 0;
    double spmm_bytes = 0.0, t_mom = 0.0;
    std::vector<int32_t> act(S, 1), conv_iter(S, 0);
    cudaMemcpyAsync(b->active, act.data(), sizeof(int32_t) * S, cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(b->meta, 0, sizeof(int32_t) * 2 * S, st);
    cudaMemsetAsync(b->st, 0, sizeof(DevState) * S, st);
    if (q_init)
        cudaMemcpyAsync(b->qin, q_init, sizeof(double) * na, cudaMemcpyHostToDevice, st);
    else
        cudaMemcpyAsync(b->qin, b->q0d, sizeof(double) * na, cudaMemcpyDeviceToDevice, st);
    k_bt_coulomb<<<(na + 255) / 256, 256, 0, st>>>(na, b->g_rp, b->g_ci, b->g_v, b->qin, b->q0d, b->shift);
    launches++;
    const size_t smem = bt_smem(b->maxU, b->maxBlk);
    int it = 0, rc = TB_OK;
    std::vector<Unit> units;
    std::vector<PipeBatchTile> ptiles;
    // the pipelined step unless its plan does not fit or fp32_kernel asks for the staged one
    const bool pipe = b->pl.stages > 0 && b->p.fp32_kernel != TB_FP32_STAGED;
    std::vector<DevState> hs(S);
    // tb_params.fp64_small: small members leave the batch and are solved on
    // their own with the plain FP64 recurrence (launch-bound either way)
    const int small_n = b->p.fp64_small == 0 ? kSmallFp64N : b->p.fp64_small;
    std::vector<char> small_done(S, 0);
    std::vector<int> small_rc(S, TB_OK);
    std::vector<DevState> small_hs(S);
    std::vector<std::vector<double>> small_q(S);
    std::vector<std::string> small_err(S);
    int64_t small_evals = 0;
    for (int s = 0; s < S && small_n > 0; s++) {
        const int na_s = b->h_ao[s + 1] - b->h_ao[s];
        if (4 * na_s > small_n) continue;
        tb_params pp = b->p;
        pp.precision = TB_PREC_FP64;
        pp.column_block = 256;  // a multiple of 128; ensure_work trims it to the structure
        pp.n_electrons = 0.0;   // sum(q0) of this structure
        tb_ctx *c = nullptr;
        int prc = tb_ctx_create(&pp, &c);
        if (prc != TB_OK) small_err[s] = std::string("context: ") + tb_status_string(prc);
        if (prc == TB_OK) prc = set_hamiltonian_bsr(c, 4 * na_s, na_s, b->hb[s]);
        if (prc == TB_OK)
            prc = tb_set_scc(c, na_s, b->grp[s].data(), b->gci[s].data(), b->gv[s].data(), b->q0[s].data());
        small_q[s].assign(na_s, 0.0);
        int32_t its = 0;
        if (prc == TB_OK)
            prc = tb_scc_solve(c, q_init ? q_init + b->h_ao[s] : nullptr, small_q[s].data(), nullptr,
                               &small_hs[s].e_band, &small_hs[s].mu, &its, nullptr);
        if (prc != TB_OK && c) small_err[s] = tb_last_error(c);
        if (c) tb_ctx_destroy(c);
        small_hs[s].converged = prc == TB_OK;
        small_rc[s] = prc == TB_ERR_NOT_CONVERGED ? TB_OK : prc;  // the cap is reported below
        small_done[s] = 1;
        small_evals += its;
        conv_iter[s] = its;
        act[s] = 0;
    }
    cudaMemcpyAsync(b->active, act.data(), sizeof(int32_t) * S, cudaMemcpyHostToDevice, st);
    const bool any_left = std::count(act.begin(), act.end(), 1) > 0;
    for (it = 1; any_left && it <= b->p.scc_max_iter; it++) {
        units.clear();
        int64_t act_cols = 0;
        for (int s = 0; s < S; s++) {
            if (!act[s]) continue;
            const int chunks = b->h_B[s] / kBtCols;
            for (int gg = b->h_g0[s]; gg < b->h_g0[s + 1]; gg++)
                for (int ch = 0; ch < chunks; ch++) units.push_back(Unit{s, gg, ch, 0});
            act_cols += 4 * (b->h_ao[s + 1] - b->h_ao[s]);
        }
        // the pipelined step's tiles: by structure, chunk, then group (the
        // groups that share halo rows run close together)
        ptiles.clear();
        for (int s = 0; pipe && s < S; s++) {
            if (!act[s]) continue;
            const int64_t ns = 4 * (int64_t)(b->h_ao[s + 1] - b->h_ao[s]);
            for (int ch = 0; ch < b->h_B[s] / kBtCols; ch++)
                for (int gg = b->h_g0[s]; gg < b->h_g0[s + 1]; gg++)
                    ptiles.push_back(PipeBatchTile{b->h_toff[s] + ch * ns * kBtCols,
                                                   b->h_poff[s] + ((int64_t)(gg - b->h_g0[s]) * b->h_B[s] +
                                                                   ch * kBtCols) * 2,
                                                   gg, {0, 0, 0}});
        }
        if ((int)ptiles.size() > b->ptiles_cap) {
            if (b->graph) {  // holds the old tile-list pointer
                cudaGraphExecDestroy(b->graph);
                b->graph = nullptr;
            }
            if (b->ptiles) cudaFree(b->ptiles);
            b->ptiles_cap = (int)ptiles.size();
            if (cudaMalloc(&b->ptiles, sizeof(PipeBatchTile) * b->ptiles_cap) != cudaSuccess) {
                b->ptiles = nullptr;
                b->ptiles_cap = 0;
                rc = bfail(b, TB_ERR_OUT_OF_MEMORY, "cudaMalloc(tiles)");
                break;
            }
        }
        const int npt = (int)ptiles.size();
        if ((int)units.size() > b->units_cap) {
            if (b->graph) {  // holds the old unit-list pointer
                cudaGraphExecDestroy(b->graph);
                b->graph = nullptr;
            }
            if (b->units) cudaFree(b->units);
            b->units_cap = (int)units.size();
            if (cudaMalloc(&b->units, sizeof(Unit) * b->units_cap) != cudaSuccess) {
                b->units = nullptr;
                b->units_cap = 0;
                rc = bfail(b, TB_ERR_OUT_OF_MEMORY, "cudaMalloc(units)");
                break;
            }
        }
        const int nu = (int)units.size();
        // The iteration's kernels: captured as a CUDA graph once per active
        // set (grid sizes and the unit list change only when a structure
        // converges) and replayed after that, or issued directly (no_graphs).
        const bool use_graph = !b->p.no_graphs;
        const bool fresh = !b->graph || b->graph_act != act;
        if (fresh || !use_graph) {
            cudaMemcpyAsync(b->units, units.data(), sizeof(Unit) * units.size(), cudaMemcpyHostToDevice, st);
            if (npt)
                cudaMemcpyAsync(b->ptiles, ptiles.data(), sizeof(PipeBatchTile) * npt, cudaMemcpyHostToDevice, st);
        }
        const bool capture = use_graph && fresh;
        auto record = [&](cudaEvent_t e) {
            if (capture)
                cudaEventRecordWithFlags(e, st, cudaEventRecordExternal);
            else
                cudaEventRecord(e, st);
        };
        auto issue = [&]() {
            k_bt_gershgorin<<<S, 1024, 0, st>>>(b->s_ao, b->h0diag, b->radius, b->shift, b->active, b->p.kT, M,
                                                b->nq_cap, b->st);
            k_bt_build_x<<<(unsigned)((b->nnzb * 16 + 255) / 256), 256, 0, st>>>(
                b->nnzb, b->blkrow, b->colidx, b->s_of_atom, b->active, b->h0, b->shift, b->st, b->x32, b->xdiag32);
            record(m0);
            k_bt_identity<<<nu, 256, 0, st>>>(b->units, nu, b->s_ao, b->s_B, b->s_toff, b->grp_I0, b->T0);
            for (int k = 0; k < K; k++) {
                const bool odd = (k + 1) & 1;
                const float *Tin = odd ? b->T0 : b->T1;
                float *Tout = odd ? b->T1 : b->T0;
                if (pipe)
                    launch_cheb_f32_pipe_batch(st, b->pl, b->ptiles, npt, b->x32, b->T0, b->T1, k,
                                               reinterpret_cast<float2 *>(b->partial));
                else
                    k_bt_cheb_f32<<<nu, 32 * kBtWarps, smem, st>>>(
                        b->units, b->s_ao, b->s_B, b->s_toff, b->s_poff, b->s_g0, b->grp_I0, b->rowptr, b->lcol,
                        b->lself, b->grp_ptr, b->grp_rows, b->x32, Tin, Tout, k == 0,
                        reinterpret_cast<float2 *>(b->partial), b->maxU, b->maxBlk);
                k_bt_finalize<<<(n + 255) / 256, 256, 0, st>>>(n, k, M, b->s_of_atom, b->active, b->s_ao, b->s_B,
                                                               b->s_poff, b->s_g0,
                                                               reinterpret_cast<const float2 *>(b->partial),
                                                               b->xdiag32, b->d);
            }
            record(m1);
            k_bt_moment_sums<<<dim3(M + 1, S), 256, 0, st>>>(b->d, n, M, b->s_ao, b->active, b->mom);
            if (b->p.kT > 0)
                k_bt_dos_nodes<<<dim3(64, S), 256, sizeof(double) * M, st>>>(b->g, b->mom, M, b->st, b->active,
                                                                             b->nq_cap, b->costab, b->rho, b->ebx);
            for (int r = 0; r < kBisectRounds; r++)
                k_bt_bisect<<<dim3(kBisectCand, S), 256, 0, st>>>(b->rho, b->ebx, b->nq_cap, b->costab, b->g, b->mom, M,
                                                                  b->ne, b->p.mu_tol, r, kBisectRounds - 1,
                                                                  b->active, b->cand, b->st);
            k_bt_fermi_nodes<<<dim3(16, S), 256, 0, st>>>(b->st, b->active, b->nq_cap, b->costab, b->fq);
            k_bt_coeffs<<<dim3(M, S), 256, 0, st>>>(M, b->st, b->active, b->nq_cap, b->costab, b->fq, b->c);
            k_bt_charges<<<(na + 255) / 256, 256, 0, st>>>(b->d, b->c, b->g, M, n, na, b->s_of_atom, b->active,
                                                           b->diagP, b->q);
            k_bt_eband<<<S, 256, 0, st>>>(b->c, b->g, b->mom, M, b->active, b->st);
            k_bt_scc_update<<<S, 1024, 0, st>>>(b->s_ao, b->q, b->qin, b->q0d, b->hq, b->hr, na, b->meta,
                                                b->p.mix_beta, b->p.mix_history, b->p.scc_tol, b->g_rp, b->g_ci,
                                                b->g_v, b->shift, b->active, b->st);
        };
        if (capture) {
            if (b->graph) {
                cudaGraphExecDestroy(b->graph);
                b->graph = nullptr;
            }
            cudaError_t ec = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
            if (ec == cudaSuccess) {
                issue();
                cudaGraph_t gr = nullptr;
                ec = cudaStreamEndCapture(st, &gr);
                if (ec == cudaSuccess) ec = cudaGraphInstantiate(&b->graph, gr, 0);
                if (gr) cudaGraphDestroy(gr);
            }
            if (ec != cudaSuccess) {
                b->graph = nullptr;
                rc = bfail(b, TB_ERR_CUDA, std::string("batch graph: ") + cudaGetErrorString(ec));
                break;
            }
            b->graph_act = act;
        }
        if (use_graph) {
            if (cudaGraphLaunch(b->graph, st) != cudaSuccess) {
                rc = bfail(b, TB_ERR_CUDA, "cudaGraphLaunch (batch)");
                break;
            }
        } else {
            issue();
        }
        launches += 3 + 2 * (int64_t)K + 7 + kBisectRounds - (b->p.kT > 0 ? 0 : 1);
        spmm += K;
        // algorithmic bytes of a batched step: the sum over active structures
        // of nnzb_s (16 s + 4) + (nb_s + 1) 4 + 3 n_s B_s s, s = 4
        for (int s = 0; s < S; s++)
            if (act[s]) {
                const int nb_s = b->h_ao[s + 1] - b->h_ao[s];
                const double nnzb_s = (double)b->hb[s].bcol.size();
                spmm_bytes += K * (nnzb_s * 68.0 + (nb_s + 1) * 4.0 + 3.0 * 4 * nb_s * (double)b->h_B[s] * 4.0);
            }
        cudaMemcpyAsync(act.data(), b->active, sizeof(int32_t) * S, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(hs.data(), b->st, sizeof(DevState) * S, cudaMemcpyDeviceToHost, st);
        cudaError_t e = cudaStreamSynchronize(st);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e != cudaSuccess) {
            rc = bfail(b, TB_ERR_CUDA, cudaGetErrorString(e));
            break;
        }
        float x = 0.f;
        cudaEventElapsedTime(&x, m0, m1);
        t_mom += x;
        int left = 0;
        for (int s = 0; s < S; s++) {
            if (!act[s] && conv_iter[s] == 0) conv_iter[s] = it;
            left += act[s];
        }
        if (!left) break;
    }
    if (it > b->p.scc_max_iter) it = b->p.scc_max_iter;
    if (q) cudaMemcpyAsync(q, b->q, sizeof(double) * na, cudaMemcpyDeviceToHost, st);
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    if (q)
        for (int s = 0; s < S; s++)
            if (small_done[s] && small_rc[s] == TB_OK)
                std::copy(small_q[s].begin(), small_q[s].end(), q + b->h_ao[s]);
    float tot = 0.f;
    cudaEventElapsedTime(&tot, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(m0);
    cudaEventDestroy(m1);
    if (rc == TB_OK && pipe) {  // bounded waits of the pipelined step that gave up
        int32_t perr = 0;
        cudaMemcpy(&perr, b->pl.err, sizeof(int32_t), cudaMemcpyDeviceToHost);
        if (perr) {
            cudaMemset(b->pl.err, 0, sizeof(int32_t));
            rc = bfail(b, TB_ERR_CUDA, "pipelined batch step: a bounded wait timed out");
        }
    }
    for (int s = 0; s < S; s++)
        if (small_done[s]) hs[s] = small_hs[s];
    if (rc == TB_OK) {
        for (int s = 0; s < S; s++) {
            if (small_done[s] && small_rc[s] != TB_OK) {
                rc = small_rc[s];
                b->err = "structure " + std::to_string(s) + " (solved alone in FP64): " + small_err[s];
                break;
            }
            if (hs[s].status) {
                rc = hs[s].status;
                b->err = "structure " + std::to_string(s) + ": " + tb_status_string(hs[s].status);
                break;
            }
            if (!hs[s].converged) {
                rc = TB_ERR_NOT_CONVERGED;
                b->err = "structure " + std::to_string(s) + " reached scc_max_iter";
            }
        }
    }
    for (int s = 0; s < S; s++) {
        if (iters) iters[s] = conv_iter[s] ? conv_iter[s] : it;
        if (e_band) e_band[s] = hs[s].e_band;
        if (mu) mu[s] = hs[s].mu;
    }
    if (rep) {
        std::memset(rep, 0, sizeof(*rep));
        rep->scc_iters = it;
        rep->t_total_ms = tot;
        rep->t_moments_ms = t_mom;
        rep->spmm_launches = spmm;
        rep->spmm_bytes = spmm_bytes;
        rep->kernel_launches = launches;
        rep->precision = TB_PREC_FP32;
        rep->column_block = -1;
        rep->fp64_evals = (int32_t)small_evals;
    }
    return rc;
    TB_ABI_CATCH
}

}  // extern "C"

// tb_noalloc.cu -- exact-trace Chebyshev moments with no device allocation.
//
// For callers that cannot call cudaMalloc: a host code whose device memory is
// owned by its own pool or allocator (a PETSc/Kokkos-style memory manager, a
// code running under a hard per-process memory budget), or one that must not
// change device-memory state at all in this phase of its run.  Such a caller
// hands in a CSR matrix and an output array that already live in device
// memory; the two slab vectors of the recurrence live in the file-scope array
// below, which every GPU that loads the library holds until the process exits
// (2 x 8192 x 64 doubles = 8 MiB).
//
// Computes mu_k = tr T_k(X), k = 0..M, of X = (H - b I)/a with the plain FP64
// recurrence T_{k+1} = 2 X T_k - T_{k-1} over 64-column slabs of the
// identity -- the same quantity tb_density returns in `moments`.
#include <cuda_runtime.h>

#include <mutex>

#include "tb_internal.h"

namespace {

constexpr int kNoAllocCols = 64;
constexpr int kNoAllocWarps = 8;

// The shared scratch: two n x 64 slabs (T_{k-1}/T_{k+1} and T_k).
static __device__ __align__(256) double g_noalloc_slabs[2 * TB_NOALLOC_MAX_N * kNoAllocCols];

std::mutex g_setup_mu;
// Device address of the array, per device ordinal, with the context it was
// looked up in: after a cudaDeviceReset (or under another driver context) the
// cached address would be stale, so a different current context repeats the
// lookup.
double *g_slab_ptr[64] = {nullptr};
void *g_slab_ctx[64] = {nullptr};

// The current driver context (the runtime API has no query of its own);
// nullptr when the entry point cannot be resolved.
void *current_context()
{
    using get_fn = int (*)(void **);
    static get_fn fn = [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        return reinterpret_cast<get_fn>(f);
    }();
    void *ctx = nullptr;
    if (fn && fn(&ctx) != 0) ctx = nullptr;
    return ctx;
}

// T0 = E[:, c0:c0+64] and mu_0 += (columns in range).
__global__ void k_noalloc_identity(double *__restrict__ T0, int n, int c0, double *__restrict__ mom)
{
    const int64_t tot = (int64_t)n * kNoAllocCols;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(e / kNoAllocCols), j = (int)(e % kNoAllocCols);
        T0[e] = (i == c0 + j) ? 1.0 : 0.0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const int w = min(kNoAllocCols, n - c0);
        atomicAdd(mom, (double)w);
    }
}

// One CSR step on a 64-column slab: warp = one row, lane = 2 columns.
// Tout = X Tin (first) or 2 X Tin - Tout; the slab's diagonal entries are
// summed per CTA and added to mom[kout].
__global__ void __launch_bounds__(32 * kNoAllocWarps)
    k_noalloc_step(int n, const int32_t *__restrict__ rowptr, const int32_t *__restrict__ colidx,
                   const double *__restrict__ vals, double inv_a, double b,
                   const double *__restrict__ Tin, double *__restrict__ Tout, int c0, int first,
                   double *__restrict__ mom, int kout)
{
    __shared__ double diag_sum[kNoAllocWarps];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int i = blockIdx.x * kNoAllocWarps + w;
    double dsum = 0.0;
    if (i < n) {
        const int col = 2 * lane;
        double2 acc = make_double2(0.0, 0.0);
        for (int k = rowptr[i]; k < rowptr[i + 1]; k++) {
            const double h = __ldg(vals + k);
            const double2 t = *reinterpret_cast<const double2 *>(Tin + (int64_t)__ldg(colidx + k) * kNoAllocCols + col);
            acc.x = fma(h, t.x, acc.x);
            acc.y = fma(h, t.y, acc.y);
        }
        const double2 ti = *reinterpret_cast<const double2 *>(Tin + (int64_t)i * kNoAllocCols + col);
        acc.x = (acc.x - b * ti.x) * inv_a;  // X = (H - b I) / a
        acc.y = (acc.y - b * ti.y) * inv_a;
        double2 *dst = reinterpret_cast<double2 *>(Tout + (int64_t)i * kNoAllocCols + col);
        double2 o;
        if (first) {
            o = acc;
        } else {
            const double2 p = *dst;
            o.x = 2.0 * acc.x - p.x;
            o.y = 2.0 * acc.y - p.y;
        }
        *dst = o;
        const int j = i - c0 - col;  // this row's diagonal column, if it is one of this lane's two
        if (j == 0) dsum = o.x;
        if (j == 1) dsum = o.y;
    }
    for (int o = 16; o > 0; o >>= 1) dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
    if (lane == 0) diag_sum[w] = dsum;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int q = 0; q < kNoAllocWarps; q++) s += diag_sum[q];
        if (s != 0.0) atomicAdd(mom + kout, s);
    }
}

}  // namespace

extern "C" int tb_moments_noalloc(int32_t n, const int32_t *d_rowptr, const int32_t *d_colidx,
                                  const double *d_vals, double a, double b, int32_t M,
                                  double *d_moments, void *stream)
{
    TB_ABI_TRY
    if (n <= 0 || M < 1 || !(a > 0) || !d_rowptr || !d_colidx || !d_vals || !d_moments)
        return TB_ERR_INVALID_ARG;
    if (n > TB_NOALLOC_MAX_N) return TB_ERR_UNSUPPORTED;  // beyond the static scratch
    // An error the caller left pending is theirs: report it before queueing
    // anything, and leave it in place.
    if (cudaPeekAtLastError() != cudaSuccess) return TB_ERR_CUDA;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return TB_ERR_NO_DEVICE;
    double *slabs = nullptr;
    {
        // set-up, once per device (again if its context changed), with that
        // device current: the device address of the file-scope array, whose
        // host-side name is only a stand-in
        std::lock_guard<std::mutex> lk(g_setup_mu);
        void *ctx = current_context();
        if (!g_slab_ptr[dev] || ctx != g_slab_ctx[dev]) {
            void *p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_slabs) != cudaSuccess || !p) {
                cudaGetLastError();
                g_slab_ptr[dev] = nullptr;
                return TB_ERR_CUDA;
            }
            g_slab_ptr[dev] = static_cast<double *>(p);
            g_slab_ctx[dev] = ctx;
        }
        slabs = g_slab_ptr[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    double *A = slabs, *Bf = slabs + (size_t)TB_NOALLOC_MAX_N * kNoAllocCols;
    if (cudaMemsetAsync(d_moments, 0, sizeof(double) * (M + 1), st) != cudaSuccess) return TB_ERR_CUDA;
    const double inv_a = 1.0 / a;
    const int grid = (n + kNoAllocWarps - 1) / kNoAllocWarps;
    for (int c0 = 0; c0 < n; c0 += kNoAllocCols) {
        k_noalloc_identity<<<(n * kNoAllocCols + 255) / 256, 256, 0, st>>>(A, n, c0, d_moments);
        for (int kout = 1; kout <= M; kout++) {
            const bool odd = kout & 1;  // T_{kout} goes where T_{kout-2} was
            k_noalloc_step<<<grid, 32 * kNoAllocWarps, 0, st>>>(n, d_rowptr, d_colidx, d_vals, inv_a, b,
                                                                odd ? A : Bf, odd ? Bf : A, c0,
                                                                kout == 1, d_moments, kout);
        }
        // a failed launch stops the loop at the end of its slab
        if (cudaGetLastError() != cudaSuccess) {
            cudaStreamSynchronize(st);
            return TB_ERR_CUDA;
        }
    }
    if (cudaStreamSynchronize(st) != cudaSuccess) return TB_ERR_CUDA;
    return TB_OK;
    TB_ABI_CATCH
}

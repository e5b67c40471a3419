// tb_dos.cu -- stochastic KPM density of states (runKPM's DOS,
// withSP2_deltaH.cpp:1579-1648) on the GPU.
//
// n_random Gaussian probe vectors r (counter-based splitmix64 + Box-Muller:
// entry i of vector t is deviate t*n + i of the stream seeded with `seed`)
// form the columns of one slab; the plain FP64 Chebyshev step advances them
// and k_probe_dot accumulates mu_k = sum_t r_t^T T_k(X) r_t after every step.
// The DOS at the Chebyshev nodes x_q = cos(pi (q+1/2)/npts) is
//   rho(x_q) = [g_0 mu_0 + 2 sum_{k>=1} g_k mu_k cos(k acos x_q)] / (pi sqrt(1 - x_q^2))
// with the closed-form Jackson g_k (N = n_moments), at energies a x_q + b.
#include <cuda_runtime.h>
#include <math.h>

#include <vector>

#include "tb_internal.h"

namespace tb {

namespace {

constexpr double kPi = 3.141592653589793238463;

__device__ __forceinline__ uint64_t splitmix_at(uint64_t seed, uint64_t k)
{
    uint64_t z = seed + (k + 1ull) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ double gauss_at(uint64_t seed, uint64_t idx)
{
    const double two53 = 1.0 / 9007199254740992.0;
    const double u1 = ((double)(splitmix_at(seed, 2ull * idx) >> 11) + 1.0) * two53;
    const double u2 = (double)(splitmix_at(seed, 2ull * idx + 1ull) >> 11) * two53;
    return sqrt(-2.0 * log(u1)) * cos(2.0 * kPi * u2);
}

__global__ void k_probe_init(double *__restrict__ T0, double *__restrict__ R, int n, int B, int nr,
                             uint64_t seed)
{
    const int64_t tot = (int64_t)n * B;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(e / B), t = (int)(e % B);
        const double v = t < nr ? gauss_at(seed, (uint64_t)t * n + i) : 0.0;
        T0[e] = v;
        R[e] = v;
    }
}

// mom_k += sum_{i,t} R[i][t] T_k[i][t]
__global__ void __launch_bounds__(256) k_probe_dot(const double *__restrict__ R,
                                                   const double *__restrict__ Tk, int64_t tot,
                                                   double *__restrict__ mom_k)
{
    __shared__ double sh[8];
    double s = 0.0;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot;
         e += (int64_t)gridDim.x * blockDim.x)
        s = fma(R[e], Tk[e], s);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < 8; w++) t += sh[w];
        atomicAdd(mom_k, t);
    }
}

__global__ void k_dos_eval(const double *__restrict__ g, const double *__restrict__ mom, int nmom,
                           int npts, const DevState *__restrict__ st, double *__restrict__ E,
                           double *__restrict__ dos)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= npts) return;
    const double x = cos(kPi * (q + 0.5) / npts);
    const double th = acos(x);
    double s = g[0] * mom[0];
    for (int k = 1; k < nmom; k++) s += 2.0 * g[k] * mom[k] * cos(k * th);
    dos[q] = s / (kPi * sqrt(1.0 - x * x));
    E[q] = x * st->a + st->b;
}

}  // namespace

int run_kpm_dos(tb_ctx *ctx, int nmom, int nr, uint64_t seed, int npts, double *mom_h, double *E_h,
                double *dos_h, double *a_out, double *b_out, int64_t *launches)
{
    DevMatrix &m = ctx->m;
    cudaStream_t st = ctx->stream;
    const int B = ((nr + 63) / 64) * 64;
    const int64_t tot = (int64_t)m.n * B;
    double *T0 = nullptr, *T1 = nullptr, *R = nullptr, *mom = nullptr, *g = nullptr, *E = nullptr,
           *dos = nullptr;
    DevState *state = nullptr;
    int rc = TB_OK;
    cudaError_t e = cudaSuccess;
    int64_t nl = 0;
    if ((e = cudaMalloc(&T0, sizeof(double) * tot)) || (e = cudaMalloc(&T1, sizeof(double) * tot)) ||
        (e = cudaMalloc(&R, sizeof(double) * tot)) || (e = cudaMalloc(&mom, sizeof(double) * nmom)) ||
        (e = cudaMalloc(&g, sizeof(double) * nmom)) || (e = cudaMalloc(&E, sizeof(double) * npts)) ||
        (e = cudaMalloc(&dos, sizeof(double) * npts)) || (e = cudaMalloc(&state, sizeof(DevState)))) {
        ctx->err = std::string("cudaMalloc(kpm dos): ") + cudaGetErrorString(e);
        rc = e == cudaErrorMemoryAllocation ? TB_ERR_OUT_OF_MEMORY : TB_ERR_CUDA;
    }
    if (rc == TB_OK && !m.x64 && (e = cudaMalloc(&m.x64, sizeof(double) * 16 * m.nnzb))) {
        ctx->err = std::string("cudaMalloc(x64): ") + cudaGetErrorString(e);
        rc = TB_ERR_OUT_OF_MEMORY;
    }
    if (rc == TB_OK) {
        // closed-form Jackson damping with N = nmom (runKPM, withSP2_deltaH.cpp:1593-1595)
        std::vector<double> gh(nmom);
        const double N = nmom, cotv = std::cos(kPi / (N + 1)) / std::sin(kPi / (N + 1));
        for (int k = 0; k < nmom; k++)
            gh[k] = ((N - k + 1) * std::cos(kPi * k / (N + 1)) + std::sin(kPi * k / (N + 1)) * cotv) / (N + 1);
        cudaMemcpyAsync(g, gh.data(), sizeof(double) * nmom, cudaMemcpyHostToDevice, st);
        cudaMemsetAsync(mom, 0, sizeof(double) * nmom, st);
        launch_gershgorin(st, m, nullptr, 0.0, 0.0, 2, 1 << 22, state, ctx->p.bounds_lo, ctx->p.bounds_hi);
        launch_build_x(st, m, nullptr, TB_PREC_FP64, state);
        int blocks = (int)std::min<int64_t>((tot + 255) / 256, 152 * 8);
        k_probe_init<<<blocks, 256, 0, st>>>(T0, R, m.n, B, nr, seed);
        k_probe_dot<<<blocks, 256, 0, st>>>(R, T0, tot, mom);
        nl += 4;
        for (int kout = 1; kout < nmom; kout++) {
            const bool odd = kout & 1;
            double *in = odd ? T0 : T1, *out = odd ? T1 : T0;
            // c0 = n: no identity diagonal to gather for probe vectors
            launch_cheb_step_f64(st, m, in, out, B, m.n, kout == 1, nullptr, kout);
            k_probe_dot<<<blocks, 256, 0, st>>>(R, out, tot, mom + kout);
            nl += (kout == 1) ? 3 : 2;
        }
        k_dos_eval<<<(npts + 127) / 128, 128, 0, st>>>(g, mom, nmom, npts, state, E, dos);
        nl++;
        DevState hs;
        cudaMemcpyAsync(mom_h, mom, sizeof(double) * nmom, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(E_h, E, sizeof(double) * npts, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(dos_h, dos, sizeof(double) * npts, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(&hs, state, sizeof(hs), cudaMemcpyDeviceToHost, st);
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess || (e = cudaGetLastError()) != cudaSuccess) {
            ctx->err = std::string("kpm dos: ") + cudaGetErrorString(e);
            rc = TB_ERR_CUDA;
        } else {
            if (hs.status) {
                ctx->err = "Gershgorin interval collapsed";
                rc = TB_ERR_SPECTRUM;
            }
            if (a_out) *a_out = hs.a;
            if (b_out) *b_out = hs.b;
        }
    }
    cudaFree(T0);
    cudaFree(T1);
    cudaFree(R);
    cudaFree(mom);
    cudaFree(g);
    cudaFree(E);
    cudaFree(dos);
    cudaFree(state);
    if (launches) *launches = nl;
    return rc;
}

}  // namespace tb

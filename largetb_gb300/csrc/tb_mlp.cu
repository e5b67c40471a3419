// tb_mlp.cu -- learned SCC starting charges: per-atom radial features and a
// small MLP (32 -> 64 -> 64 -> 1, SiLU), trained and evaluated on the GPU by
// these kernels.  No counterpart in the reference, which always starts its
// SCC loop from the neutral charges (withSP2_deltaH.cpp:1725-1740, 1804-1812).
//
// Features of atom i: 16 Gaussians exp(-eta (r_ij - mu_k)^2) f_c(r_ij) summed
// over Si neighbours j, then 16 over O neighbours, mu_k = 0.8 + 0.28 k A,
// eta = 12.5 A^-2, f_c(r) = (cos(pi r / 5 A) + 1)/2 inside 5 A, minimum image
// in an orthorhombic box.
//
// Network: y = w3 . silu(W2 silu(W1 x~ + b1) + b2) + b3 with
// x~ = (x - mean) * istd (feature normalisation fixed from the first
// training set).  Weights are used in BF16 (a round-to-nearest-even copy of
// FP32 master weights), activations and accumulation in FP32; training is
// minibatch Adam on the mean squared error.  Each CTA takes tiles of 64 atoms
// with the weights (transposed where a warp reads along output units) in
// shared memory; weight gradients accumulate in registers across tiles and
// are added to global memory once per CTA.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include "tb_internal.h"

namespace tb {
namespace {

constexpr int kF = TB_MLP_NFEAT;  // 32
constexpr int kH = 64;
constexpr int kW1 = 0, kB1 = kW1 + kH * kF, kW2 = kB1 + kH, kB2 = kW2 + kH * kH, kW3 = kB2 + kH,
              kB3 = kW3 + kH, kNP = kB3 + 1;
static_assert(kNP == TB_MLP_NPARAM, "parameter layout");
constexpr int kTile = 64;
constexpr double kBohrPerAng = 1.88973;

__device__ __forceinline__ float sigm(float z) { return 1.f / (1.f + __expf(-z)); }

// ---- features --------------------------------------------------------------
__global__ void k_features(int natoms, const double *__restrict__ xyz, const int32_t *__restrict__ sp,
                           double bx, double by, double bz, float *__restrict__ feat)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= natoms) return;
    const double box[3] = {bx, by, bz};
    const double rc = 5.0 * kBohrPerAng, rc2 = rc * rc;
    // FP32 prefilter of the pair distance (minimum image by a multiply with
    // the inverse box), with a 1 % margin on rc^2 that covers its rounding;
    // pairs inside it are recomputed in FP64 below, so the features are the
    // same as with the FP64 test alone
    const float fbox[3] = {(float)bx, (float)by, (float)bz};
    const float finv[3] = {bx > 0 ? (float)(1.0 / bx) : 0.f, by > 0 ? (float)(1.0 / by) : 0.f,
                           bz > 0 ? (float)(1.0 / bz) : 0.f};
    const float fi[3] = {(float)xyz[3 * i], (float)xyz[3 * i + 1], (float)xyz[3 * i + 2]};
    const float rc2_loose = (float)(rc2 * 1.01);
    float f[2 * 16];
    for (int k = 0; k < 32; k++) f[k] = 0.f;
    for (int j = 0; j < natoms; j++) {
        if (j == i) continue;
        float r2f = 0.f;
#pragma unroll
        for (int q = 0; q < 3; q++) {
            float t = (float)xyz[3 * j + q] - fi[q];
            t -= fbox[q] * rintf(t * finv[q]);
            r2f = fmaf(t, t, r2f);
        }
        if (r2f >= rc2_loose) continue;
        double d[3];
        for (int q = 0; q < 3; q++) {
            double t = xyz[3 * j + q] - xyz[3 * i + q];
            if (box[q] > 0) t -= box[q] * nearbyint(t / box[q]);
            d[q] = t;
        }
        const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        if (r2 >= rc2) continue;
        const double r = sqrt(r2) / kBohrPerAng;  // angstrom
        const double fc = 0.5 * (cos(3.141592653589793 * r / 5.0) + 1.0);
        const int base = sp[j] == 14 ? 0 : 16;
        for (int k = 0; k < 16; k++) {
            const double dr = r - (0.8 + 0.28 * k);
            f[base + k] += (float)(exp(-12.5 * dr * dr) * fc);
        }
    }
    for (int k = 0; k < 32; k++) feat[(int64_t)i * kF + k] = f[k];
}

// ---- forward / backward over tiles of 64 atoms ---------------------------------
// Wq: BF16-rounded parameters (FP32 storage).  idx (optional) maps sample
// positions to rows of X / target.  With target == nullptr only the forward
// pass runs and y goes to out.
__global__ void __launch_bounds__(256)
    k_mlp_fb(int n, const int32_t *__restrict__ idx, const float *__restrict__ X,
             const float *__restrict__ mean, const float *__restrict__ istd, const float *__restrict__ Wq,
             const float *__restrict__ target, float inv_n, float *__restrict__ out,
             float *__restrict__ grad, float *__restrict__ loss)
{
    extern __shared__ float ms[];
    float *W1T = ms;                 // [i][u]   32 x 64
    float *W2T = W1T + kF * kH;      // [v][u]   64 x 64 (u = output unit)
    float *W2 = W2T + kH * kH;       // [u][v]
    float *b1 = W2 + kH * kH;
    float *b2 = b1 + kH;
    float *w3 = b2 + kH;
    float *Xs = w3 + kH;             // [a][33]
    float *Z1 = Xs + kTile * (kF + 1);
    float *H1 = Z1 + kTile * kH;
    float *Z2 = H1 + kTile * kH;
    float *dy = Z2 + kTile * kH;     // [64]
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    for (int e = tid; e < kH * kF; e += blockDim.x) {
        const int u = e / kF, i = e % kF;
        W1T[i * kH + u] = Wq[kW1 + e];
    }
    for (int e = tid; e < kH * kH; e += blockDim.x) {
        const int u = e / kH, v = e % kH;
        W2[e] = Wq[kW2 + e];
        W2T[v * kH + u] = Wq[kW2 + e];
    }
    for (int e = tid; e < kH; e += blockDim.x) {
        b1[e] = Wq[kB1 + e];
        b2[e] = Wq[kB2 + e];
        w3[e] = Wq[kW3 + e];
    }
    const float b3 = Wq[kB3];
    const bool bwd = target != nullptr;
    const int u = tid & (kH - 1), a0 = tid >> 6;  // 4 atom phases x 64 units
    float gW2[16], gW1[8], gb1 = 0.f, gb2 = 0.f, gw3 = 0.f, gb3 = 0.f, lsum = 0.f;
    for (int q = 0; q < 16; q++) gW2[q] = 0.f;
    for (int q = 0; q < 8; q++) gW1[q] = 0.f;
    __syncthreads();
    for (int tile = blockIdx.x; tile * kTile < n; tile += gridDim.x) {
        const int base = tile * kTile;
        for (int e = tid; e < kTile * kF; e += blockDim.x) {
            const int a = e / kF, i = e % kF, s = base + a;
            float v = 0.f;
            if (s < n) {
                const int row = idx ? idx[s] : s;
                v = (X[(int64_t)row * kF + i] - mean[i]) * istd[i];
            }
            Xs[a * (kF + 1) + i] = v;
        }
        __syncthreads();
        // layer 1
        for (int a = a0; a < kTile; a += 4) {
            float z = b1[u];
#pragma unroll 8
            for (int i = 0; i < kF; i++) z = fmaf(W1T[i * kH + u], Xs[a * (kF + 1) + i], z);
            Z1[a * kH + u] = z;
            H1[a * kH + u] = z * sigm(z);
        }
        __syncthreads();
        // layer 2
        for (int a = a0; a < kTile; a += 4) {
            float z = b2[u];
#pragma unroll 8
            for (int v = 0; v < kH; v++) z = fmaf(W2T[v * kH + u], H1[a * kH + v], z);
            Z2[a * kH + u] = z;
        }
        __syncthreads();
        // output: warp w takes atoms w, w+8, ...
        for (int a = w; a < kTile; a += 8) {
            float p = 0.f;
            for (int v = lane; v < kH; v += 32) {
                const float z = Z2[a * kH + v];
                p = fmaf(w3[v], z * sigm(z), p);
            }
            for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
            const int s = base + a;
            if (lane == 0) {
                const float y = p + b3;
                if (out && s < n) out[s] = y;
                float g = 0.f;
                if (bwd && s < n) {
                    const int row = idx ? idx[s] : s;
                    const float err = y - target[row];
                    g = 2.f * err * inv_n;
                    lsum += err * err * inv_n;
                }
                dy[a] = g;
            }
        }
        __syncthreads();
        if (!bwd) continue;
        // output layer gradients and dZ2 (in place over Z2)
        if (tid < kH) {
            float s3 = 0.f;
            for (int a = 0; a < kTile; a++) {
                const float z = Z2[a * kH + tid];
                s3 = fmaf(dy[a], z * sigm(z), s3);
            }
            gw3 += s3;
        }
        if (tid == 0)
            for (int a = 0; a < kTile; a++) gb3 += dy[a];
        __syncthreads();
        for (int a = a0; a < kTile; a += 4) {
            const float z = Z2[a * kH + u], sg = sigm(z);
            Z2[a * kH + u] = dy[a] * w3[u] * sg * (1.f + z * (1.f - sg));
        }
        __syncthreads();
        // dW2[u][v] for v = a0 + 4q, db2
        for (int a = 0; a < kTile; a++) {
            const float dz = Z2[a * kH + u];
            if (a0 == 0) gb2 += dz;
#pragma unroll
            for (int q = 0; q < 16; q++) gW2[q] = fmaf(dz, H1[a * kH + a0 + 4 * q], gW2[q]);
        }
        __syncthreads();
        // dH1 -> dZ1 (in place over Z1): thread owns unit v = u of layer 1
        for (int a = a0; a < kTile; a += 4) {
            float dh = 0.f;
#pragma unroll 8
            for (int k = 0; k < kH; k++) dh = fmaf(W2[k * kH + u], Z2[a * kH + k], dh);
            const float z = Z1[a * kH + u], sg = sigm(z);
            Z1[a * kH + u] = dh * sg * (1.f + z * (1.f - sg));
        }
        __syncthreads();
        // dW1[u][i] for i = a0 + 4q, db1
        for (int a = 0; a < kTile; a++) {
            const float dz = Z1[a * kH + u];
            if (a0 == 0) gb1 += dz;
#pragma unroll
            for (int q = 0; q < 8; q++) gW1[q] = fmaf(dz, Xs[a * (kF + 1) + a0 + 4 * q], gW1[q]);
        }
        __syncthreads();
    }
    if (!bwd) return;
#pragma unroll
    for (int q = 0; q < 16; q++) atomicAdd(grad + kW2 + u * kH + a0 + 4 * q, gW2[q]);
#pragma unroll
    for (int q = 0; q < 8; q++) atomicAdd(grad + kW1 + u * kF + a0 + 4 * q, gW1[q]);
    if (a0 == 0) {
        atomicAdd(grad + kB1 + u, gb1);
        atomicAdd(grad + kB2 + u, gb2);
    }
    if (tid < kH) atomicAdd(grad + kW3 + tid, gw3);
    if (tid == 0) atomicAdd(grad + kB3, gb3);
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if (lane == 0 && lsum != 0.f) atomicAdd(loss, lsum);
}

constexpr size_t kFbSmem =
    sizeof(float) * (kF * kH + 2 * kH * kH + 3 * kH + kTile * (kF + 1) + 3 * kTile * kH + kTile);

// Adam on the FP32 master weights, then the BF16 working copy.
__global__ void k_adam(int np, float *__restrict__ W, float *__restrict__ Wq, float *__restrict__ m1,
                       float *__restrict__ m2, const float *__restrict__ g, float lr, float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const float gi = g[i];
    const float a = 0.9f * m1[i] + 0.1f * gi, b = 0.999f * m2[i] + 0.001f * gi * gi;
    m1[i] = a;
    m2[i] = b;
    const float w = W[i] - lr * (a * c1) / (sqrtf(b * c2) + 1e-8f);
    W[i] = w;
    Wq[i] = __bfloat162float(__float2bfloat16_rn(w));
}

__global__ void k_round_bf16(int np, const float *__restrict__ W, float *__restrict__ Wq)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < np) Wq[i] = __bfloat162float(__float2bfloat16_rn(W[i]));
}

uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

}  // namespace
}  // namespace tb

using namespace tb;

struct tb_mlp {
    int device = 0;
    cudaStream_t stream = nullptr;
    float *W = nullptr, *Wq = nullptr, *m1 = nullptr, *m2 = nullptr, *g = nullptr, *loss = nullptr;
    float *mean = nullptr, *istd = nullptr;
    int32_t *err = nullptr;  // bounded-wait flag of the tensor-core forward
    bool have_norm = false;
    int64_t step = 0;
};

namespace {

int mlp_alloc(tb_mlp *m)
{
    if (cudaMalloc(&m->W, sizeof(float) * kNP) || cudaMalloc(&m->Wq, sizeof(float) * kNP) ||
        cudaMalloc(&m->m1, sizeof(float) * kNP) || cudaMalloc(&m->m2, sizeof(float) * kNP) ||
        cudaMalloc(&m->g, sizeof(float) * kNP) || cudaMalloc(&m->loss, sizeof(float)) ||
        cudaMalloc(&m->mean, sizeof(float) * kF) || cudaMalloc(&m->istd, sizeof(float) * kF) ||
        cudaMalloc(&m->err, sizeof(int32_t)) || cudaMemset(m->err, 0, sizeof(int32_t)))
        return TB_ERR_OUT_OF_MEMORY;
    return TB_OK;
}

// Upload host features (and targets); returns device pointers owned by the caller.
int upload_set(cudaStream_t st, int n, const float *feat, const float *target, float **dX, float **dT)
{
    *dX = nullptr;
    if (dT) *dT = nullptr;
    if (cudaMalloc(dX, sizeof(float) * (size_t)n * kF)) return TB_ERR_OUT_OF_MEMORY;
    cudaMemcpyAsync(*dX, feat, sizeof(float) * (size_t)n * kF, cudaMemcpyHostToDevice, st);
    if (dT && target) {
        if (cudaMalloc(dT, sizeof(float) * n)) return TB_ERR_OUT_OF_MEMORY;
        cudaMemcpyAsync(*dT, target, sizeof(float) * n, cudaMemcpyHostToDevice, st);
    }
    return TB_OK;
}

int fb_grid(int n)
{
    const int tiles = (n + kTile - 1) / kTile;
    return std::max(1, std::min(tiles, 152 * 2));
}

}  // namespace

extern "C" {

int tb_mlp_features(int32_t natoms, const double *xyz, const int32_t *species, const double *box, float *feat)
{
    TB_ABI_TRY
    if (natoms <= 0 || !xyz || !species || !box || !feat) return TB_ERR_INVALID_ARG;
    double *dx = nullptr;
    int32_t *ds = nullptr;
    float *df = nullptr;
    int rc = TB_OK;
    if (cudaMalloc(&dx, sizeof(double) * 3 * natoms) || cudaMalloc(&ds, sizeof(int32_t) * natoms) ||
        cudaMalloc(&df, sizeof(float) * (size_t)natoms * kF)) {
        rc = TB_ERR_OUT_OF_MEMORY;
    } else {
        cudaMemcpy(dx, xyz, sizeof(double) * 3 * natoms, cudaMemcpyHostToDevice);
        cudaMemcpy(ds, species, sizeof(int32_t) * natoms, cudaMemcpyHostToDevice);
        k_features<<<(natoms + 127) / 128, 128>>>(natoms, dx, ds, box[0], box[1], box[2], df);
        if (cudaMemcpy(feat, df, sizeof(float) * (size_t)natoms * kF, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = TB_ERR_CUDA;
    }
    cudaFree(dx);
    cudaFree(ds);
    cudaFree(df);
    return rc;
    TB_ABI_CATCH
}

int tb_mlp_create(int32_t device, uint64_t seed, tb_mlp **out)
{
    TB_ABI_TRY
    if (!out) return TB_ERR_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return TB_ERR_NO_DEVICE;
    }
    tb_mlp *m = new (std::nothrow) tb_mlp();
    if (!m) return TB_ERR_OUT_OF_MEMORY;
    m->device = device;
    cudaSetDevice(device);
    if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess || mlp_alloc(m)) {
        tb_mlp_destroy(m);
        return TB_ERR_CUDA;
    }
    // He-style uniform initialisation from splitmix64, zero biases
    std::vector<float> w(kNP, 0.f);
    uint64_t k = 0;
    auto uni = [&](double lim) {
        const double u = (double)(mix64(seed + (++k) * 0x9E3779B97F4A7C15ull) >> 11) / 9007199254740992.0;
        return (float)((2.0 * u - 1.0) * lim);
    };
    for (int i = 0; i < kH * kF; i++) w[kW1 + i] = uni(std::sqrt(6.0 / kF));
    for (int i = 0; i < kH * kH; i++) w[kW2 + i] = uni(std::sqrt(6.0 / kH));
    for (int i = 0; i < kH; i++) w[kW3 + i] = uni(std::sqrt(3.0 / kH));
    std::vector<float> zero(kNP, 0.f), mean(kF, 0.f), one(kF, 1.f);
    cudaMemcpy(m->W, w.data(), sizeof(float) * kNP, cudaMemcpyHostToDevice);
    cudaMemcpy(m->m1, zero.data(), sizeof(float) * kNP, cudaMemcpyHostToDevice);
    cudaMemcpy(m->m2, zero.data(), sizeof(float) * kNP, cudaMemcpyHostToDevice);
    cudaMemcpy(m->mean, mean.data(), sizeof(float) * kF, cudaMemcpyHostToDevice);
    cudaMemcpy(m->istd, one.data(), sizeof(float) * kF, cudaMemcpyHostToDevice);
    k_round_bf16<<<(kNP + 255) / 256, 256, 0, m->stream>>>(kNP, m->W, m->Wq);
    if (cudaFuncSetAttribute(k_mlp_fb, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFbSmem) != cudaSuccess ||
        cudaStreamSynchronize(m->stream) != cudaSuccess) {
        tb_mlp_destroy(m);
        return TB_ERR_CUDA;
    }
    *out = m;
    return TB_OK;
    TB_ABI_CATCH
}

int tb_mlp_destroy(tb_mlp *m)
{
    TB_ABI_TRY
    if (!m) return TB_OK;
    cudaSetDevice(m->device);
    if (m->stream) cudaStreamSynchronize(m->stream);
    cudaFree(m->W);
    cudaFree(m->Wq);
    cudaFree(m->m1);
    cudaFree(m->m2);
    cudaFree(m->g);
    cudaFree(m->loss);
    cudaFree(m->mean);
    cudaFree(m->istd);
    cudaFree(m->err);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return TB_OK;
    TB_ABI_CATCH
}

int tb_mlp_get(const tb_mlp *m, float *params, float *norm)
{
    TB_ABI_TRY
    if (!m) return TB_ERR_INVALID_ARG;
    cudaSetDevice(m->device);
    if (params && cudaMemcpy(params, m->W, sizeof(float) * kNP, cudaMemcpyDeviceToHost)) return TB_ERR_CUDA;
    if (norm && (cudaMemcpy(norm, m->mean, sizeof(float) * kF, cudaMemcpyDeviceToHost) ||
                 cudaMemcpy(norm + kF, m->istd, sizeof(float) * kF, cudaMemcpyDeviceToHost)))
        return TB_ERR_CUDA;
    return TB_OK;
    TB_ABI_CATCH
}

int tb_mlp_set(tb_mlp *m, const float *params, const float *norm)
{
    TB_ABI_TRY
    if (!m) return TB_ERR_INVALID_ARG;
    cudaSetDevice(m->device);
    if (params) {
        for (int i = 0; i < kNP; i++)
            if (!std::isfinite(params[i])) return TB_ERR_NONFINITE;
        cudaMemcpy(m->W, params, sizeof(float) * kNP, cudaMemcpyHostToDevice);
        k_round_bf16<<<(kNP + 255) / 256, 256, 0, m->stream>>>(kNP, m->W, m->Wq);
    }
    if (norm) {
        cudaMemcpy(m->mean, norm, sizeof(float) * kF, cudaMemcpyHostToDevice);
        cudaMemcpy(m->istd, norm + kF, sizeof(float) * kF, cudaMemcpyHostToDevice);
        m->have_norm = true;
    }
    return cudaStreamSynchronize(m->stream) == cudaSuccess ? TB_OK : TB_ERR_CUDA;
    TB_ABI_CATCH
}

int tb_mlp_grad(tb_mlp *m, int32_t n, const float *feat, const float *target, float *grad, float *loss)
{
    TB_ABI_TRY
    if (!m || n <= 0 || !feat || !target || !grad) return TB_ERR_INVALID_ARG;
    cudaSetDevice(m->device);
    float *dX, *dT;
    int rc = upload_set(m->stream, n, feat, target, &dX, &dT);
    if (rc == TB_OK) {
        cudaMemsetAsync(m->g, 0, sizeof(float) * kNP, m->stream);
        cudaMemsetAsync(m->loss, 0, sizeof(float), m->stream);
        k_mlp_fb<<<fb_grid(n), 256, kFbSmem, m->stream>>>(n, nullptr, dX, m->mean, m->istd, m->Wq, dT, 1.f / n,
                                                         nullptr, m->g, m->loss);
        cudaMemcpyAsync(grad, m->g, sizeof(float) * kNP, cudaMemcpyDeviceToHost, m->stream);
        if (loss) cudaMemcpyAsync(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream);
        if (cudaStreamSynchronize(m->stream) != cudaSuccess || cudaGetLastError() != cudaSuccess) rc = TB_ERR_CUDA;
    }
    cudaFree(dX);
    cudaFree(dT);
    return rc;
    TB_ABI_CATCH
}

int tb_mlp_predict(tb_mlp *m, int32_t n, const float *feat, float *out)
{
    TB_ABI_TRY
    if (!m || n <= 0 || !feat || !out) return TB_ERR_INVALID_ARG;
    cudaSetDevice(m->device);
    float *dX = nullptr, *dY = nullptr;
    int rc = upload_set(m->stream, n, feat, nullptr, &dX, nullptr);
    if (rc == TB_OK && cudaMalloc(&dY, sizeof(float) * n)) rc = TB_ERR_OUT_OF_MEMORY;
    if (rc == TB_OK) {
        launch_mlp_forward_tc(m->stream, n, dX, m->mean, m->istd, m->Wq, dY, m->err);
        int32_t e = 0;
        cudaMemcpyAsync(out, dY, sizeof(float) * n, cudaMemcpyDeviceToHost, m->stream);
        cudaMemcpyAsync(&e, m->err, sizeof(int32_t), cudaMemcpyDeviceToHost, m->stream);
        if (cudaStreamSynchronize(m->stream) != cudaSuccess || cudaGetLastError() != cudaSuccess) rc = TB_ERR_CUDA;
        if (rc == TB_OK && e) {
            cudaMemsetAsync(m->err, 0, sizeof(int32_t), m->stream);
            rc = TB_ERR_CUDA;
        }
    }
    cudaFree(dX);
    cudaFree(dY);
    return rc;
    TB_ABI_CATCH
}

int tb_mlp_predict_fp32(tb_mlp *m, int32_t n, const float *feat, float *out)
{
    TB_ABI_TRY
    if (!m || n <= 0 || !feat || !out) return TB_ERR_INVALID_ARG;
    cudaSetDevice(m->device);
    float *dX = nullptr, *dY = nullptr;
    int rc = upload_set(m->stream, n, feat, nullptr, &dX, nullptr);
    if (rc == TB_OK && cudaMalloc(&dY, sizeof(float) * n)) rc = TB_ERR_OUT_OF_MEMORY;
    if (rc == TB_OK) {
        k_mlp_fb<<<fb_grid(n), 256, kFbSmem, m->stream>>>(n, nullptr, dX, m->mean, m->istd, m->Wq, nullptr, 0.f,
                                                         dY, nullptr, nullptr);
        cudaMemcpyAsync(out, dY, sizeof(float) * n, cudaMemcpyDeviceToHost, m->stream);
        if (cudaStreamSynchronize(m->stream) != cudaSuccess || cudaGetLastError() != cudaSuccess) rc = TB_ERR_CUDA;
    }
    cudaFree(dX);
    cudaFree(dY);
    return rc;
    TB_ABI_CATCH
}

int tb_mlp_train(tb_mlp *m, int32_t n, const float *feat, const float *target, int32_t epochs, int32_t batch,
                 float lr, uint64_t seed, float *loss_per_epoch)
{
    TB_ABI_TRY
    if (!m || n <= 0 || !feat || !target || epochs < 1 || batch < 1 || !(lr > 0)) return TB_ERR_INVALID_ARG;
    cudaSetDevice(m->device);
    cudaStream_t st = m->stream;
    if (!m->have_norm) {
        // fix the feature normalisation from this training set
        std::vector<double> mu(kF, 0.0), var(kF, 0.0);
        for (int64_t s = 0; s < n; s++)
            for (int i = 0; i < kF; i++) mu[i] += feat[s * kF + i];
        for (int i = 0; i < kF; i++) mu[i] /= n;
        for (int64_t s = 0; s < n; s++)
            for (int i = 0; i < kF; i++) {
                const double d = feat[s * kF + i] - mu[i];
                var[i] += d * d;
            }
        std::vector<float> norm(2 * kF);
        for (int i = 0; i < kF; i++) {
            norm[i] = (float)mu[i];
            const double sd = std::sqrt(var[i] / n);
            norm[kF + i] = (float)(sd > 1e-6 ? 1.0 / sd : 1.0);
        }
        tb_mlp_set(m, nullptr, norm.data());
    }
    float *dX, *dT;
    int32_t *dI = nullptr;
    int rc = upload_set(st, n, feat, target, &dX, &dT);
    if (rc == TB_OK && cudaMalloc(&dI, sizeof(int32_t) * n)) rc = TB_ERR_OUT_OF_MEMORY;
    std::vector<int32_t> perm(n);
    std::iota(perm.begin(), perm.end(), 0);
    uint64_t rs = seed;
    for (int ep = 0; ep < epochs && rc == TB_OK; ep++) {
        for (int i = n - 1; i > 0; i--) {  // Fisher-Yates with splitmix64
            rs += 0x9E3779B97F4A7C15ull;
            const int j = (int)(mix64(rs) % (uint64_t)(i + 1));
            std::swap(perm[i], perm[j]);
        }
        cudaMemcpyAsync(dI, perm.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, st);
        cudaMemsetAsync(m->loss, 0, sizeof(float), st);
        for (int b0 = 0; b0 < n; b0 += batch) {
            const int nb = std::min(batch, n - b0);
            cudaMemsetAsync(m->g, 0, sizeof(float) * kNP, st);
            k_mlp_fb<<<fb_grid(nb), 256, kFbSmem, st>>>(nb, dI + b0, dX, m->mean, m->istd, m->Wq, dT,
                                                        1.f / nb, nullptr, m->g, m->loss);
            m->step++;
            const float c1 = 1.f / (1.f - std::pow(0.9f, (float)m->step));
            const float c2 = 1.f / (1.f - std::pow(0.999f, (float)m->step));
            k_adam<<<(kNP + 255) / 256, 256, 0, st>>>(kNP, m->W, m->Wq, m->m1, m->m2, m->g, lr, c1, c2);
        }
        float l = 0.f;
        cudaMemcpyAsync(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess) rc = TB_ERR_CUDA;
        // the per-batch losses are batch means: average over the batches
        if (loss_per_epoch) loss_per_epoch[ep] = l * (float)batch / (float)n;
    }
    cudaFree(dX);
    cudaFree(dT);
    cudaFree(dI);
    return rc;
    TB_ABI_CATCH
}

}  // extern "C"

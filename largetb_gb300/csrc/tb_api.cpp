// tb_api.cpp -- host side of the C-ABI in include/largetb.h: context,
// validation and CSR -> BSR conversion of the caller's PETSc-style AIJ
// arrays, and the orchestration of one density evaluation / SCC solve on the
// context stream.  No compute happens on the host: every numeric stage is a
// kernel in tb_kpe.cu / tb_sp2.cu, and there is no CPU fallback.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "tb_internal.h"

using namespace tb;

namespace {

constexpr double kPi = 3.141592653589793238463;

int fail(tb_ctx *ctx, int code, const std::string &msg)
{
    if (ctx) ctx->err = msg;
    return code;
}

#define TB_CUDA(call)                                                                   \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? TB_ERR_OUT_OF_MEMORY     \
                                                             : TB_ERR_CUDA,             \
                        std::string(#call) + ": " + cudaGetErrorString(e_));            \
        }                                                                               \
    } while (0)

#define TB_TRY(expr)            \
    do {                        \
        int rc_ = (expr);       \
        if (rc_ != TB_OK) return rc_; \
    } while (0)

template <typename T>
void dfree(T *&p)
{
    if (p) cudaFree((void *)p);
    p = nullptr;
}

template <typename T>
int dalloc(tb_ctx *ctx, T *&p, size_t count)
{
    dfree(p);
    if (count == 0) count = 1;
    TB_CUDA(cudaMalloc((void **)&p, count * sizeof(T)));
    return TB_OK;
}

template <typename T>
int upload(tb_ctx *ctx, T *&p, const T *src, size_t count)
{
    TB_TRY(dalloc(ctx, p, count));
    if (count) TB_CUDA(cudaMemcpyAsync(p, src, count * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    return TB_OK;
}

int quad_nodes(int M, double beta_x)
{
    double need = 4.0 * M;
    if (beta_x > 0 && 13.0 * beta_x > need) need = 13.0 * beta_x;
    if (need < 256) need = 256;
    int nq = 256;
    while (nq < need && nq < (1 << 22)) nq *= 2;
    return nq;
}

void damping(int kind, int M, std::vector<double> &g)
{
    g.assign(M, 1.0);
    if (kind == TB_KERNEL_JACKSON) {
        // closed form of runKPM (withSP2_deltaH.cpp:1593-1595) with N = M terms
        const double N = M;
        const double cotv = std::cos(kPi / (N + 1)) / std::sin(kPi / (N + 1));
        for (int k = 0; k < M; k++)
            g[k] = ((N - k + 1) * std::cos(kPi * k / (N + 1)) + std::sin(kPi * k / (N + 1)) * cotv) /
                   (N + 1);
    } else if (kind == TB_KERNEL_AUTOCORR) {
        // getKPE's autocorrelation of normalised U_i(cos(pi/(M+2)))
        // (withSP2_deltaH.cpp:1104-1132, including its i < M-m-1 bound)
        std::vector<double> u(M);
        const double al = std::acos(std::cos(kPi / (M + 2)));
        double nrm = 0.0;
        for (int m = 0; m < M; m++) {
            u[m] = std::sin((m + 1) * al) / std::sin(al);
            nrm += u[m] * u[m];
        }
        nrm = std::sqrt(nrm);
        for (int m = 0; m < M; m++) u[m] /= nrm;
        for (int m = 0; m < M; m++) {
            double s = 0.0;
            for (int i = 0; i < M - m - 1; i++) s += u[i] * u[m + i];
            g[m] = s;
        }
    }
    g[0] = 1.0;  // the n = 0 term carries no damping factor (getKPE, line 1136)
}

int check_params(tb_ctx *ctx, const tb_params *p)
{
    if (!p) return fail(ctx, TB_ERR_INVALID_ARG, "params is NULL");
    if (p->struct_size != sizeof(tb_params))
        return fail(ctx, TB_ERR_INVALID_ARG, "tb_params.struct_size mismatch (call tb_params_init)");
    if (p->M < 2 || p->M > 6000) return fail(ctx, TB_ERR_INVALID_ARG, "M must be in [2, 6000]");
    if (p->kernel < 0 || p->kernel > 2) return fail(ctx, TB_ERR_INVALID_ARG, "unknown kernel kind");
    if (p->precision != TB_PREC_FP64 && p->precision != TB_PREC_FP32)
        return fail(ctx, TB_ERR_INVALID_ARG, "unknown precision");
    if (!std::isfinite(p->kT)) return fail(ctx, TB_ERR_INVALID_ARG, "kT not finite");
    if (p->column_block < 0 || p->column_block % 128 != 0)
        return fail(ctx, TB_ERR_INVALID_ARG, "column_block must be 0 or a multiple of 128");
    if (!(p->spectral_pad >= 0) || !(p->mu_tol > 0) || !(p->scc_tol > 0) || p->scc_max_iter < 1)
        return fail(ctx, TB_ERR_INVALID_ARG, "bad pad / tolerance / iteration cap");
    if (p->mix_history < 0 || p->mix_history > kMaxHistory || !(p->mix_beta > 0))
        return fail(ctx, TB_ERR_INVALID_ARG, "mix_history must be in [0,16], mix_beta > 0");
    if (p->mode != TB_MODE_KPE && p->mode != TB_MODE_SP2) return fail(ctx, TB_ERR_INVALID_ARG, "unknown mode");
    if (!std::isfinite(p->bounds_lo) || !std::isfinite(p->bounds_hi))
        return fail(ctx, TB_ERR_INVALID_ARG, "spectral bounds not finite");
    if (p->fp32_kernel < TB_FP32_AUTO || p->fp32_kernel > TB_FP32_PIPELINED_STEP)
        return fail(ctx, TB_ERR_INVALID_ARG, "unknown fp32_kernel");
    if (!(p->sp2_drop_tol >= 0) || p->sp2_max_iter < 1 || !(p->sp2_idem_tol >= 0))
        return fail(ctx, TB_ERR_INVALID_ARG, "bad SP2 parameters");
    return TB_OK;
}

int set_device(tb_ctx *ctx)
{
    TB_CUDA(cudaSetDevice(ctx->device));
    return TB_OK;
}

double step_bytes(const DevMatrix &m, int B, int s);

void reset_tuning(tb_ctx *ctx)
{
    for (int a = 0; a < 2; a++)
        for (int b = 0; b < kNumKinds; b++) ctx->tuned_kind[a][b] = ctx->tuned_B[a][b] = 0;
}

// Error flags raised by the bounded waits of the persistent and pipelined
// step kernels; synchronises the stream.
int check_kernel_flags(tb_ctx *ctx)
{
    int32_t perr = 0, serr = 0;
    if (ctx->pp.err)
        TB_CUDA(cudaMemcpyAsync(&perr, ctx->pp.err, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    if (ctx->pl.err)
        TB_CUDA(cudaMemcpyAsync(&serr, ctx->pl.err, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    TB_CUDA(cudaStreamSynchronize(ctx->stream));
    if (perr) {
        cudaMemsetAsync(ctx->pp.err, 0, sizeof(int32_t), ctx->stream);
        return fail(ctx, TB_ERR_TIMEOUT, "persistent Chebyshev kernel: a neighbour-flag wait ran out");
    }
    if (serr) {
        cudaMemsetAsync(ctx->pl.err, 0, sizeof(int32_t), ctx->stream);
        return fail(ctx, TB_ERR_TIMEOUT, serr == 2 ? "pipelined Chebyshev kernel: a neighbour-flag wait ran out"
                                                   : "pipelined Chebyshev kernel: a stage mbarrier wait ran out");
    }
    return TB_OK;
}

// Step-flag array of the one-launch-per-slab pipelined mode: one int per
// tile (row group x 64-column chunk) of a B-column slab.
int ensure_pipe_flags(tb_ctx *ctx, int B)
{
    PipePlan &pl = ctx->pl;
    const int64_t need = (int64_t)pl.G * ((B + 63) / 64);
    if (pl.flags && pl.flags_cap >= need) return TB_OK;
    dfree(pl.flags);
    pl.flags_cap = 0;
    TB_TRY(dalloc(ctx, pl.flags, (size_t)need));
    pl.flags_cap = need;
    return TB_OK;
}

// Slab-width autotuner (column_block = 0): time kTuneSteps Chebyshev steps of
// one slab for every candidate kernel/width on this matrix and keep the one
// with the least estimated time per density evaluation (slab time x slabs, so
// that a last, mostly padded slab counts).  Runs once per matrix, precision
// and requested FP32 kernel (req, a StepKind; kKindAuto tries them all); the
// X used is the unshifted one.
int autotune(tb_ctx *ctx, int req)
{
    constexpr int kTuneSteps = 12;
    DevMatrix &m = ctx->m;
    cudaStream_t st = ctx->stream;
    const int prec = ctx->p.precision;
    const int n64 = ((m.n + 63) / 64) * 64, n128 = ((m.n + 127) / 128) * 128;
    struct Cand {
        int kind;
        int B;
    };
    std::vector<Cand> cands;
    auto widths = [&](int kind, std::initializer_list<int> Bs, int q) {
        const int nr = q == 128 ? n128 : n64;
        for (int B : Bs) {
            const int Bc = std::min(B, nr);
            bool dup = false;
            for (const Cand &c : cands) dup |= (c.kind == kind && c.B == Bc);
            if (!dup) cands.push_back({kind, Bc});
        }
    };
    // widths in [lo, hi] (multiples of 64) that split n into equal slabs with
    // the least padding: B = 64 ceil(ceil(n / s) / 64) over slab counts s
    auto even_widths = [&](int lo, int hi) {
        std::vector<std::pair<int64_t, int>> w;  // (padding, -B)
        for (int ns = std::max(1, (m.n + hi - 1) / hi); ns <= (m.n + lo - 1) / lo; ns++) {
            const int B = ((m.n + ns - 1) / ns + 63) / 64 * 64;
            if (B < lo || B > hi) continue;
            w.push_back({(int64_t)ns * B - m.n, -B});
        }
        std::sort(w.begin(), w.end());
        std::vector<int> out;
        for (auto &e : w)
            if ((int)out.size() < 3 && std::find(out.begin(), out.end(), -e.second) == out.end()) out.push_back(-e.second);
        return out;
    };
    // the FP32 partial array holds K * rowgroups * B pairs of 16 bytes: keep it
    // under a quarter of the free device memory (at least 4 GiB)
    const int Kp = (ctx->p.M + 2) / 2;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        free_b = 0;
    }
    const double part_cap = std::max(4.0 * 1073741824.0, 0.25 * (double)free_b);
    auto fits = [&](int B, int groups) { return (double)Kp * groups * B * 16.0 <= part_cap; };
    if (prec == TB_PREC_FP32) {
        if ((req == kKindAuto || req == kKindPersistent) && ctx->pp.R > 0) cands.push_back({kKindPersistent, ctx->pp.B});
        if ((req == kKindAuto || req == kKindPipelined) && ctx->pl.stages > 0 && ctx->pl.coop)
            widths(kKindPipelined, {256, 512, 1024}, 64);
        if ((req == kKindAuto || req == kKindPipelinedStep) && ctx->pl.stages > 0) {
            widths(kKindPipelinedStep, {512, 1024}, 64);
            // wider slabs amortise each launch's pipeline fill and drain over
            // more tiles (6x6x6, M = 400: 171.5 ms per density at B = 3456,
            // 165.6 ms at B = 20736, one slab)
            for (int B : even_widths(768, n64))
                if (fits(B, ctx->pl.G)) widths(kKindPipelinedStep, {B}, 64);
        }
        if (req == kKindAuto || req == kKindStaged) widths(kKindStaged, {256, 384, 512}, ctx->sp.R > 0 ? 64 : 128);
    } else {
        widths(kKindStaged, {64, 128, 256}, 64);
    }
    if (cands.empty()) return fail(ctx, TB_ERR_UNSUPPORTED, "requested FP32 step kernel has no plan for this matrix");
    DevState *state = nullptr;
    TB_TRY(dalloc(ctx, state, 1));
    if (prec == TB_PREC_FP32 && !m.x32) TB_TRY(dalloc(ctx, m.x32, (size_t)m.nnzb * 16));
    if (prec == TB_PREC_FP64 && !m.x64) TB_TRY(dalloc(ctx, m.x64, (size_t)m.nnzb * 16));
    launch_gershgorin(st, m, nullptr, 0.0, 0.0, 2, 1 << 22, state);
    launch_build_x(st, m, nullptr, prec, state);
    double best = 1e300;
    Cand pick = cands.front();
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    for (const Cand &cd : cands) {
        const int B = cd.B;
        const size_t es = prec == TB_PREC_FP32 ? 4 : 8;
        const bool pipe = cd.kind == kKindPipelined || cd.kind == kKindPipelinedStep;
        const int rowgroups = cd.kind == kKindPersistent ? ctx->pp.G
                              : pipe                     ? ctx->pl.G
                                                         : (ctx->sp.R > 0 ? ctx->sp.G : cheb_f32_rowgroups(m.nb));
        if (cd.kind == kKindPipelined) TB_TRY(ensure_pipe_flags(ctx, B));
        char *T0 = nullptr, *T1 = nullptr;
        double *part = nullptr, *dd = nullptr;
        TB_TRY(dalloc(ctx, T0, (size_t)m.n * B * es));
        TB_TRY(dalloc(ctx, T1, (size_t)m.n * B * es));
        if (prec == TB_PREC_FP32)
            TB_TRY(dalloc(ctx, part, (size_t)(kTuneSteps + 1) * rowgroups * B * 2));
        else
            TB_TRY(dalloc(ctx, dd, (size_t)(kTuneSteps + 2) * m.n));
        float ms = 0.f;
        for (int rep = 0; rep < 2; rep++) {  // the first pass warms up
            cudaEventRecord(a, st);
            if (cd.kind == kKindPersistent) {
                cudaMemsetAsync(ctx->pp.flags, 0, sizeof(int32_t) * ctx->pp.G * ctx->pp.nc, st);
                launch_cheb_f32_persistent(st, m, ctx->pp, kTuneSteps, B, 0, (float *)T0, (float *)T1,
                                           reinterpret_cast<float2 *>(part), ctx->pp.flags, ctx->pp.err);
            } else if (cd.kind == kKindPipelined) {
                launch_slab_identity_cm(st, (float *)T0, m.n, B, 0);
                const int e = launch_cheb_f32_pipe(st, m, ctx->pl, (float *)T0, (float *)T1, B, 0, kTuneSteps,
                                                   reinterpret_cast<float2 *>(part), true);
                if (e != (int)cudaSuccess)
                    return fail(ctx, TB_ERR_CUDA,
                                std::string("cooperative launch: ") + cudaGetErrorString((cudaError_t)e));
            } else {
                if (cd.kind == kKindPipelinedStep)
                    launch_slab_identity_cm(st, (float *)T0, m.n, B, 0);
                else
                    launch_slab_identity(st, T0, m.n, B, 0, prec);
                for (int k = 0; k < kTuneSteps; k++) {
                    const bool odd = (k + 1) & 1;
                    char *in = odd ? T0 : T1, *out = odd ? T1 : T0;
                    double *pk = part ? part + (int64_t)k * rowgroups * B * 2 : nullptr;
                    if (prec == TB_PREC_FP64)
                        launch_cheb_step_f64(st, m, (double *)in, (double *)out, B, 0, k == 0, dd, k + 1);
                    else if (cd.kind == kKindPipelinedStep)
                        launch_cheb_f32_pipe(st, m, ctx->pl, (float *)T0, (float *)T1, B, k, 1,
                                             reinterpret_cast<float2 *>(pk), false);
                    else if (ctx->sp.R > 0)
                        launch_cheb_step_f32_staged(st, m, ctx->sp, (float *)in, (float *)out, B, k == 0,
                                                    reinterpret_cast<float2 *>(pk));
                    else
                        launch_cheb_step_f32(st, m, (float *)in, (float *)out, B, k == 0,
                                             reinterpret_cast<float2 *>(pk), rowgroups);
                }
            }
            cudaEventRecord(b, st);
            TB_CUDA(cudaEventSynchronize(b));
            cudaEventElapsedTime(&ms, a, b);
        }
        TB_CUDA(cudaGetLastError());
        // estimated moment time of a density evaluation: per-slab time x slabs
        const double per_density = ms * (double)((m.n + B - 1) / B);
        if (per_density < best) {
            best = per_density;
            pick = cd;
        }
        dfree(T0);
        dfree(T1);
        dfree(part);
        dfree(dd);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    dfree(state);
    TB_TRY(check_kernel_flags(ctx));
    ctx->tuned_kind[prec][req] = pick.kind;
    ctx->tuned_B[prec][req] = pick.B;
    return TB_OK;
}

// Work buffers sized for the current parameters and matrix.
int ensure_work(tb_ctx *ctx)
{
    DevWork &w = ctx->w;
    const DevMatrix &m = ctx->m;
    const tb_params &p = ctx->p;
    const int M = p.M;
    const int prec = p.precision;
    const int req = prec == TB_PREC_FP32 ? p.fp32_kernel : kKindAuto;
    int kind = kKindStaged, B = p.column_block;
    if (B == 0) {
        if (ctx->tuned_B[prec][req] == 0) TB_TRY(autotune(ctx, req));
        kind = ctx->tuned_kind[prec][req];
        B = ctx->tuned_B[prec][req];
    } else if (prec == TB_PREC_FP32) {
        kind = req != kKindAuto ? req
                                : (ctx->pl.stages > 0 ? (ctx->pl.coop ? kKindPipelined : kKindPipelinedStep) : kKindStaged);
    }
    if (kind == kKindPersistent && ctx->pp.R == 0)
        return fail(ctx, TB_ERR_UNSUPPORTED, "persistent FP32 kernel: no task plan fits this matrix");
    if ((kind == kKindPipelined || kind == kKindPipelinedStep) && ctx->pl.stages == 0)
        return fail(ctx, TB_ERR_UNSUPPORTED, "pipelined FP32 kernel: no stage plan fits this matrix");
    if (kind == kKindPipelined && !ctx->pl.coop)
        return fail(ctx, TB_ERR_UNSUPPORTED, "pipelined FP32 kernel: cooperative launch not available");
    if (kind == kKindPersistent) {
        B = ctx->pp.B;
    } else {
        // the unstaged FP32 kernel works in 128-column chunks, the others in 64
        const int q = (prec == TB_PREC_FP32 && ctx->sp.R == 0) ? 128 : 64;
        const int nround = ((m.n + q - 1) / q) * q;
        if (B > nround) B = nround;
    }
    const bool persist = kind == kKindPersistent;
    const bool pipe = kind == kKindPipelined || kind == kKindPipelinedStep;
    if (kind == kKindPipelined) TB_TRY(ensure_pipe_flags(ctx, B));
    const int K = (prec == TB_PREC_FP32) ? (M + 2) / 2 : 0;
    const int rowgroups = (prec != TB_PREC_FP32)       ? 0
                          : persist                      ? ctx->pp.G
                          : pipe                         ? ctx->pl.G
                          : ctx->sp.R > 0                ? ctx->sp.G
                                                         : cheb_f32_rowgroups(m.nb);
    w.kind = kind;
    // quadrature capacity from the Gershgorin width of H0 with a 2x margin
    // for SCC shifts; the device flags TB_ERR_SPECTRUM if it is exceeded.
    int nq_cap = 1 << 14;
    if (p.kT > 0)
        nq_cap = std::max(nq_cap, quad_nodes(M, 2.0 * (ctx->h0_lmax - ctx->h0_lmin) / p.kT));
    const bool same = w.M == M && w.B == B && w.K == K && w.precision == p.precision &&
                      w.kind == kind &&
                      w.rowgroups == rowgroups && w.nq_cap >= nq_cap && w.d && w.mom && w.T0 &&
                      w.kernel == p.kernel;
    if (same) return TB_OK;
    ctx->gen++;  // buffers change: captured graphs are stale
    w.kernel = p.kernel;
    w.M = M;
    w.B = B;
    w.K = K;
    w.rowgroups = rowgroups;
    w.precision = p.precision;
    w.nq_cap = nq_cap;
    const size_t es = (p.precision == TB_PREC_FP32) ? 4 : 8;
    w.slab_bytes = (size_t)m.n * B * es;
    {
        char *t0 = (char *)w.T0, *t1 = (char *)w.T1;
        dfree(t0);
        dfree(t1);
        w.T0 = w.T1 = nullptr;
        TB_TRY(dalloc(ctx, t0, w.slab_bytes));
        TB_TRY(dalloc(ctx, t1, w.slab_bytes));
        w.T0 = t0;
        w.T1 = t1;
    }
    TB_TRY(dalloc(ctx, w.d, (size_t)(M + 1) * m.n));
    TB_TRY(dalloc(ctx, w.mom, (size_t)M + 1));
    TB_TRY(dalloc(ctx, w.c, (size_t)M));
    TB_TRY(dalloc(ctx, w.rho, 2 * (size_t)w.nq_cap));  // DOS at the nodes, then e^{beta x_q}
    TB_TRY(dalloc(ctx, w.fq, (size_t)w.nq_cap));
    TB_TRY(dalloc(ctx, w.costab, 4 * (size_t)w.nq_cap));
    launch_cos_table(ctx->stream, w.nq_cap, w.costab);
    TB_TRY(dalloc(ctx, w.cand, (size_t)kBisectCand));
    TB_TRY(dalloc(ctx, w.diagP, (size_t)m.n));
    TB_TRY(dalloc(ctx, w.q, (size_t)m.natoms));
    TB_TRY(dalloc(ctx, w.shift, (size_t)m.n));
    if (!w.state) {
        TB_TRY(dalloc(ctx, w.state, 1));
        TB_CUDA(cudaMemsetAsync(w.state, 0, sizeof(DevState), ctx->stream));
    }
    if (p.precision == TB_PREC_FP32) {
        w.partial_elems = (int64_t)K * rowgroups * B * 2;
        TB_TRY(dalloc(ctx, w.partial, (size_t)w.partial_elems));
    } else {
        dfree(w.partial);
        w.partial_elems = 0;
    }
    std::vector<double> g;
    damping(p.kernel, M, g);
    TB_TRY(upload(ctx, w.g, g.data(), g.size()));
    if (p.precision == TB_PREC_FP32) {
        if (!ctx->m.x32) TB_TRY(dalloc(ctx, ctx->m.x32, (size_t)m.nnzb * 16));
    } else {
        if (!ctx->m.x64) TB_TRY(dalloc(ctx, ctx->m.x64, (size_t)m.nnzb * 16));
    }
    return TB_OK;
}

// Algorithmic bytes of one Chebyshev step over one slab:
// nnzb (16 s + 4) + (nb + 1) 4 + 3 n B s.
double step_bytes(const DevMatrix &m, int B, int s)
{
    return (double)m.nnzb * (16.0 * s + 4.0) + (double)(m.nb + 1) * 4.0 + 3.0 * m.n * (double)B * s;
}

// Row-group staging plan for k_cheb_f32_staged: the group size R is the
// candidate with the least estimated step traffic (distinct referenced block
// rows, weighted by wave efficiency at 256 columns) whose staging buffers
// fit three CTAs per SM; without one the unstaged kernel is used.
int build_stage_plan(tb_ctx *ctx, const std::vector<int32_t> &brow, const std::vector<int32_t> &bcol)
{
    StagePlan &sp = ctx->sp;
    dfree(sp.grp_ptr);
    dfree(sp.grp_rows);
    dfree(sp.lcol);
    dfree(sp.lself);
    sp = StagePlan{};
    const int nb = (int)brow.size() - 1;
    int nsm = 152;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device);
    const size_t smem_cap = 74 * 1024;  // 3 CTAs per SM
    double best = 1e300;
    int bestR = 0;
    std::vector<int32_t> mark(nb, -1);
    for (int R : {16, 24, 32, 48, 64}) {
        const int G = (nb + R - 1) / R;
        int64_t tot = 0;
        int maxU = 0, maxBlk = 0;
        for (int g = 0; g < G; g++) {
            const int I0 = g * R, I1 = std::min(nb, I0 + R);
            int u = 0;
            for (int t = brow[I0]; t < brow[I1]; t++)
                if (mark[bcol[t]] != g) {
                    mark[bcol[t]] = g;
                    u++;
                }
            tot += u;
            maxU = std::max(maxU, u);
            maxBlk = std::max(maxBlk, brow[I1] - brow[I0]);
        }
        std::fill(mark.begin(), mark.end(), -1);
        if (cheb_f32_staged_smem(R, maxU, maxBlk) > smem_cap) continue;
        const int64_t ctas = (int64_t)G * 4, slots = (int64_t)nsm * 3;
        const double eff = (double)ctas / (double)(((ctas + slots - 1) / slots) * slots);
        const double cost = (double)(tot + 2 * nb) / eff;
        if (cost < best) {
            best = cost;
            bestR = R;
        }
    }
    if (bestR == 0) return TB_OK;  // unstaged fallback
    const int R = bestR, G = (nb + R - 1) / R;
    std::vector<int32_t> gptr(G + 1, 0), grows, lcol(bcol.size()), lself(nb);
    int maxU = 0, maxBlk = 0;
    for (int g = 0; g < G; g++) {
        const int I0 = g * R, I1 = std::min(nb, I0 + R);
        std::vector<int32_t> U;
        for (int t = brow[I0]; t < brow[I1]; t++) U.push_back(bcol[t]);
        std::sort(U.begin(), U.end());
        U.erase(std::unique(U.begin(), U.end()), U.end());
        for (int t = brow[I0]; t < brow[I1]; t++)
            lcol[t] = (int32_t)(std::lower_bound(U.begin(), U.end(), bcol[t]) - U.begin());
        for (int I = I0; I < I1; I++)
            lself[I] = (int32_t)(std::lower_bound(U.begin(), U.end(), I) - U.begin());
        grows.insert(grows.end(), U.begin(), U.end());
        gptr[g + 1] = (int32_t)grows.size();
        maxU = std::max(maxU, (int)U.size());
        maxBlk = std::max(maxBlk, brow[I1] - brow[I0]);
    }
    TB_TRY(upload(ctx, sp.grp_ptr, gptr.data(), gptr.size()));
    TB_TRY(upload(ctx, sp.grp_rows, grows.data(), grows.size()));
    TB_TRY(upload(ctx, sp.lcol, lcol.data(), lcol.size()));
    TB_TRY(upload(ctx, sp.lself, lself.data(), lself.size()));
    const size_t smem = cheb_f32_staged_smem(R, maxU, maxBlk);
    if (cheb_f32_staged_configure(smem) != (int)cudaSuccess) {
        cudaGetLastError();
        return TB_OK;  // sp.R stays 0: unstaged fallback
    }
    sp.R = R;
    sp.G = G;
    sp.maxU = maxU;
    sp.maxBlk = maxBlk;
    sp.totalU = (int64_t)grows.size();
    return TB_OK;
}

// Plan of the pipelined FP32 kernel: R is the candidate with the least
// estimated step traffic (distinct referenced rows plus own T_{k-1} rows,
// divided by the wave efficiency of 512-column slabs on one CTA per SM) among
// those whose stage fits a ring of three (else two) stages in 227 KB.
int build_pipe_plan(tb_ctx *ctx, const std::vector<int32_t> &brow, const std::vector<int32_t> &bcol)
{
    PipePlan &pl = ctx->pl;
    dfree(pl.hdr);
    dfree(pl.runs);
    dfree(pl.rec);
    dfree(pl.nbr_ptr);
    dfree(pl.nbr);
    dfree(pl.flags);
    dfree(pl.err);
    pl = PipePlan{};
    const int nb = (int)brow.size() - 1;
    int nsm = 152;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device);
    std::vector<int32_t> mark(nb, -1);
    struct Pick {
        int R = 0, stages = 0;
        double cost = 1e300;
    } best;
    for (int R : {12, 16, 20, 24, 28, 32}) {
        const int G = (nb + R - 1) / R;
        int64_t tot = 0;
        int maxU = 0, maxBlk = 0;
        for (int g = 0; g < G; g++) {
            const int I0 = g * R, I1 = std::min(nb, I0 + R);
            int u = 0;
            for (int t = brow[I0]; t < brow[I1]; t++)
                if (mark[bcol[t]] != g) {
                    mark[bcol[t]] = g;
                    u++;
                }
            tot += u;
            maxU = std::max(maxU, u);
            maxBlk = std::max(maxBlk, brow[I1] - brow[I0]);
        }
        std::fill(mark.begin(), mark.end(), -1);
        const int rec_cap = ((2 * R + 1 + maxBlk) + 3) / 4 * 4;
        const size_t stage = cheb_f32_pipe_stage_bytes(R, maxU, maxBlk, rec_cap);
        int stages = 3;
        while (stages >= 2 && cheb_f32_pipe_smem(stage, stages) > 227 * 1024) stages--;
        if (stages < 2) continue;
        const int64_t tiles = (int64_t)G * 8;
        const double eff = (double)tiles / (double)(((tiles + nsm - 1) / nsm) * nsm);
        const double cost = (double)(tot + nb) / eff * (stages >= 3 ? 1.0 : 1.25);
        if (cost < best.cost) best = {R, stages, cost};
    }
    if (best.R == 0) return TB_OK;  // pipelined kernel unavailable for this matrix
    const int R = best.R, G = (nb + R - 1) / R;
    std::vector<int32_t> hdr((size_t)G * 8, 0), rec, nptr(G + 1, 0), nbr;
    std::vector<std::vector<int32_t>> grun(G);
    int maxU = 0, maxBlk = 0, rec_cap = 0, maxRuns = 0;
    std::vector<int32_t> U;
    for (int g = 0; g < G; g++) {
        const int I0 = g * R, I1 = std::min(nb, I0 + R);
        int32_t *h = &hdr[(size_t)g * 8];
        pipe_group_records(brow.data(), bcol.data(), I0, I1, 0, h, rec, grun[g], U);
        for (int J : U)  // U is sorted, so the owner groups come in order
            if (nbr.size() == (size_t)nptr[g] || nbr.back() != J / R) nbr.push_back(J / R);
        nptr[g + 1] = (int32_t)nbr.size();
        maxRuns = std::max(maxRuns, h[6]);
        maxU = std::max(maxU, h[0]);
        maxBlk = std::max(maxBlk, h[2]);
        rec_cap = std::max(rec_cap, h[4]);
    }
    const size_t stage_bytes = cheb_f32_pipe_stage_bytes(R, maxU, maxBlk, rec_cap);
    const size_t smem = cheb_f32_pipe_smem(stage_bytes, best.stages);
    int per_sm = 0;
    if (smem > 227 * 1024 || cheb_f32_pipe_configure(smem, &per_sm) != (int)cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        return TB_OK;
    }
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device);
    const int run_stride = (maxRuns + 31) / 32 * 32;
    std::vector<int32_t> runs((size_t)G * run_stride * 4, 0);
    for (int g = 0; g < G; g++) std::copy(grun[g].begin(), grun[g].end(), runs.begin() + (size_t)g * run_stride * 4);
    TB_TRY(upload(ctx, pl.hdr, hdr.data(), hdr.size()));
    TB_TRY(upload(ctx, pl.nbr_ptr, nptr.data(), nptr.size()));
    TB_TRY(upload(ctx, pl.nbr, nbr.data(), nbr.size()));
    TB_TRY(upload(ctx, pl.runs, runs.data(), runs.size()));
    TB_TRY(upload(ctx, pl.rec, rec.data(), rec.size()));
    TB_TRY(dalloc(ctx, pl.err, 1));
    TB_CUDA(cudaMemsetAsync(pl.err, 0, sizeof(int32_t), ctx->stream));
    pl.R = R;
    pl.G = G;
    pl.maxU = maxU;
    pl.maxBlk = maxBlk;
    pl.stages = best.stages;
    pl.stage_bytes = stage_bytes;
    pl.nsm = nsm;
    pl.run_stride = run_stride;
    pl.coop = coop != 0;
    return TB_OK;
}

// Task plan of the persistent FP32 kernel: row groups of R block rows, each
// with its halo (referenced rows owned by other groups) and its neighbouring
// groups; nc 64-column chunks per slab so that all G * nc tasks are resident
// together (a requirement of the cooperative launch).  R minimises
// slabs x tasks per SM x (R + mean halo); without a fitting R the per-step
// kernels are used.
int build_persist_plan(tb_ctx *ctx, const std::vector<int32_t> &brow, const std::vector<int32_t> &bcol)
{
    PersistPlan &pp = ctx->pp;
    dfree(pp.lcode);
    dfree(pp.hptr);
    dfree(pp.hrows);
    dfree(pp.nptr);
    dfree(pp.ngrp);
    dfree(pp.flags);
    dfree(pp.err);
    pp = PersistPlan{};
    const int nb = (int)brow.size() - 1, n = 4 * nb;
    int nsm = 152, coop = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device);
    if (!coop) return TB_OK;
    struct Cand {
        int R, G, nc, B, maxH, maxBlk, maxNG;
        double cost;
    };
    Cand best{0, 0, 0, 0, 0, 0, 0, 1e300};
    for (int R : {16, 24, 32, 48, 64}) {  // kernel instances for 2, 3, 4, 6, 8 rows per warp
        const int G = (nb + R - 1) / R;
        int maxH = 0, maxBlk = 0, maxNG = 0;
        int64_t totH = 0;
        for (int g = 0; g < G; g++) {
            const int I0 = g * R, I1 = std::min(nb, I0 + R);
            std::vector<int32_t> halo, ng;
            for (int t = brow[I0]; t < brow[I1]; t++)
                if (bcol[t] < I0 || bcol[t] >= I1) halo.push_back(bcol[t]);
            std::sort(halo.begin(), halo.end());
            halo.erase(std::unique(halo.begin(), halo.end()), halo.end());
            for (int J : halo) ng.push_back(J / R);
            ng.erase(std::unique(ng.begin(), ng.end()), ng.end());
            maxH = std::max(maxH, (int)halo.size());
            maxNG = std::max(maxNG, (int)ng.size());
            maxBlk = std::max(maxBlk, brow[I1] - brow[I0]);
            totH += (int64_t)halo.size();
        }
        const size_t smem = cheb_f32_persistent_smem(R, maxH, maxBlk, maxNG);
        if (smem > 227 * 1024) continue;
        int per_sm = 0;
        if (cheb_f32_persistent_setup(R, smem, &per_sm) != (int)cudaSuccess || per_sm < 1) {
            cudaGetLastError();
            continue;
        }
        const int64_t slots = (int64_t)nsm * per_sm;
        int nc = (int)std::min<int64_t>(slots / G, (n + 63) / 64);
        if (nc < 1) continue;
        const int B = 64 * nc, nslab = (n + B - 1) / B;
        const double tasks_per_sm = std::ceil((double)G * nc / nsm);
        const double cost = (double)nslab * tasks_per_sm * (R + (double)totH / G);
        if (cost < best.cost) best = Cand{R, G, nc, B, maxH, maxBlk, maxNG, cost};
    }
    if (best.R == 0) return TB_OK;
    const int R = best.R, G = best.G;
    std::vector<int32_t> lcode(bcol.size()), hptr(G + 1, 0), hrows, nptr(G + 1, 0), ngrp;
    for (int g = 0; g < G; g++) {
        const int I0 = g * R, I1 = std::min(nb, I0 + R);
        std::vector<int32_t> halo;
        for (int t = brow[I0]; t < brow[I1]; t++)
            if (bcol[t] < I0 || bcol[t] >= I1) halo.push_back(bcol[t]);
        std::sort(halo.begin(), halo.end());
        halo.erase(std::unique(halo.begin(), halo.end()), halo.end());
        for (int t = brow[I0]; t < brow[I1]; t++) {
            const int J = bcol[t];
            lcode[t] = (J >= I0 && J < I1)
                           ? J - I0
                           : R + (int32_t)(std::lower_bound(halo.begin(), halo.end(), J) - halo.begin());
        }
        std::vector<int32_t> ng;
        for (int J : halo) ng.push_back(J / R);
        ng.erase(std::unique(ng.begin(), ng.end()), ng.end());
        hrows.insert(hrows.end(), halo.begin(), halo.end());
        ngrp.insert(ngrp.end(), ng.begin(), ng.end());
        hptr[g + 1] = (int32_t)hrows.size();
        nptr[g + 1] = (int32_t)ngrp.size();
    }
    if (hrows.empty()) hrows.push_back(0);
    if (ngrp.empty()) ngrp.push_back(0);
    TB_TRY(upload(ctx, pp.lcode, lcode.data(), lcode.size()));
    TB_TRY(upload(ctx, pp.hptr, hptr.data(), hptr.size()));
    TB_TRY(upload(ctx, pp.hrows, hrows.data(), hrows.size()));
    TB_TRY(upload(ctx, pp.nptr, nptr.data(), nptr.size()));
    TB_TRY(upload(ctx, pp.ngrp, ngrp.data(), ngrp.size()));
    TB_TRY(dalloc(ctx, pp.flags, (size_t)G * best.nc));
    TB_TRY(dalloc(ctx, pp.err, 1));
    TB_CUDA(cudaMemsetAsync(pp.err, 0, sizeof(int32_t), ctx->stream));
    // re-apply the chosen shared-memory size (setup ran for several candidates)
    int per_sm = 0;
    cheb_f32_persistent_setup(R, cheb_f32_persistent_smem(R, best.maxH, best.maxBlk, best.maxNG), &per_sm);
    pp.R = R;
    pp.G = G;
    pp.nc = best.nc;
    pp.B = best.B;
    pp.maxH = best.maxH;
    pp.maxBlk = best.maxBlk;
    pp.maxNG = best.maxNG;
    return TB_OK;
}

std::pair<cudaEvent_t, cudaEvent_t> next_events(tb_ctx *ctx)
{
    if (ctx->capturing) return {ctx->graph_ev[0], ctx->graph_ev[1]};
    if (ctx->ev_used == ctx->moment_events.size()) {
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        ctx->moment_events.push_back({a, b});
    }
    return ctx->moment_events[ctx->ev_used++];
}

// One density evaluation of H0 + diag(w.shift); leaves diagP / q / state on
// the device.  Kernels only; no host synchronisation.
int density_eval(tb_ctx *ctx, bool have_shift)
{
    DevWork &w = ctx->w;
    DevMatrix &m = ctx->m;
    const tb_params &p = ctx->p;
    cudaStream_t st = ctx->stream;
    const int M = p.M, B = w.B;
    const double *shift = have_shift ? w.shift : nullptr;
    launch_gershgorin(st, m, shift, p.spectral_pad, p.kT, M, w.nq_cap, w.state, p.bounds_lo, p.bounds_hi);
    launch_build_x(st, m, shift, p.precision, w.state);
    ctx->launches += 2;

    auto ev = next_events(ctx);
    // under stream capture an event record joins the graph only as an external node
    auto record = [&](cudaEvent_t e) {
        if (ctx->capturing)
            cudaEventRecordWithFlags(e, st, cudaEventRecordExternal);
        else
            cudaEventRecord(e, st);
    };
    record(ev.first);
    const int nslab = (m.n + B - 1) / B;
    for (int s = 0; s < nslab; s++) {
        const int c0 = s * B;
        if (w.kind == kKindPipelined || w.kind == kKindPipelinedStep) {
            launch_slab_identity_cm(st, (float *)w.T0, m.n, B, c0);
            ctx->launches++;
        } else if (w.kind != kKindPersistent) {
            launch_slab_identity(st, w.T0, m.n, B, c0, p.precision);
            ctx->launches++;
        }
        if (p.precision == TB_PREC_FP64) {
            double *A = (double *)w.T0, *Bf = (double *)w.T1;
            for (int kout = 1; kout <= M; kout++) {
                const bool odd = kout & 1;
                launch_cheb_step_f64(st, m, odd ? A : Bf, odd ? Bf : A, B, c0, kout == 1, w.d, kout);
                ctx->launches += (kout == 1) ? 2 : 1;
            }
            ctx->spmm_launches += M;
            ctx->spmm_bytes += M * step_bytes(m, B, 8);
        } else if (w.kind == kKindPipelined) {
            const int e = launch_cheb_f32_pipe(st, m, ctx->pl, (float *)w.T0, (float *)w.T1, B, 0, w.K,
                                               reinterpret_cast<float2 *>(w.partial), true);
            if (e != (int)cudaSuccess)
                return fail(ctx, TB_ERR_CUDA,
                            std::string("cooperative launch: ") + cudaGetErrorString((cudaError_t)e));
            launch_f32_finalize_pairs(st, m, reinterpret_cast<const float2 *>(w.partial), w.K, w.rowgroups, B, c0,
                                      w.d, M);
            ctx->launches += 3;  // flag reset, slab kernel, finalize
            ctx->spmm_launches += w.K;  // one launch carries all K slab steps
            ctx->spmm_bytes += w.K * step_bytes(m, B, 4);
        } else if (w.kind == kKindPersistent) {
            TB_CUDA(cudaMemsetAsync(ctx->pp.flags, 0, sizeof(int32_t) * ctx->pp.G * ctx->pp.nc, st));
            const int e = launch_cheb_f32_persistent(st, m, ctx->pp, w.K, B, c0, (float *)w.T0,
                                                     (float *)w.T1, reinterpret_cast<float2 *>(w.partial),
                                                     ctx->pp.flags, ctx->pp.err);
            if (e != (int)cudaSuccess)
                return fail(ctx, TB_ERR_CUDA,
                            std::string("cooperative launch: ") + cudaGetErrorString((cudaError_t)e));
            launch_f32_finalize_pairs(st, m, reinterpret_cast<const float2 *>(w.partial), w.K, w.rowgroups, B, c0,
                                      w.d, M);
            ctx->launches += 2;
            ctx->spmm_launches += w.K;  // one launch carries all K slab steps
            ctx->spmm_bytes += w.K * step_bytes(m, B, 4);
        } else {
            float *A = (float *)w.T0, *Bf = (float *)w.T1;
            for (int k = 0; k < w.K; k++) {
                const int kout = k + 1;
                const bool odd = kout & 1;
                double *pk = w.partial + (int64_t)k * w.rowgroups * B * 2;
                if (w.kind == kKindPipelinedStep)
                    launch_cheb_f32_pipe(st, m, ctx->pl, A, Bf, B, k, 1, reinterpret_cast<float2 *>(pk), false);
                else if (ctx->sp.R > 0)
                    launch_cheb_step_f32_staged(st, m, ctx->sp, odd ? A : Bf, odd ? Bf : A, B, k == 0,
                                                reinterpret_cast<float2 *>(pk));
                else
                    launch_cheb_step_f32(st, m, odd ? A : Bf, odd ? Bf : A, B, k == 0,
                                         reinterpret_cast<float2 *>(pk), w.rowgroups);
                ctx->launches++;
            }
            launch_f32_finalize_pairs(st, m, reinterpret_cast<const float2 *>(w.partial), w.K, w.rowgroups, B, c0,
                                      w.d, M);
            ctx->launches++;
            ctx->spmm_launches += w.K;
            ctx->spmm_bytes += w.K * step_bytes(m, B, 4);
        }
    }
    record(ev.second);

    launch_moment_sums(st, w.d, m.n, M + 1, w.mom);
    ctx->launches++;
    if (p.kT > 0) {
        launch_dos_nodes(st, w.g, w.mom, M, w.state, w.nq_cap, w.costab, w.rho);
        ctx->launches++;
    }
    for (int r = 0; r < kBisectRounds; r++) {
        launch_bisect_round(st, w.rho, w.g, w.mom, w.costab, w.nq_cap, M, ctx->p.n_electrons, p.mu_tol, r,
                            w.cand, w.state);
        ctx->launches++;
    }
    launch_fermi_coeffs(st, M, w.state, w.nq_cap, w.costab, w.fq, w.c);
    launch_charges(st, w.d, w.c, w.g, w.mom, M, m.n, m.natoms, w.diagP, w.q, w.state);
    ctx->launches += 4;
    TB_CUDA(cudaGetLastError());
    return TB_OK;
}

// One SCC iteration (density evaluation + mixing update) on the stream.  The
// iteration is captured once as a CUDA graph per configuration (ctx->gen) and
// replayed after that: a density evaluation is ~10^3 small launches, which
// bound the iteration for small systems.  The cooperative-launch kernels are
// not captured; their iterations are launched directly.
int scc_iteration(tb_ctx *ctx, bool *graphed)
{
    cudaStream_t st = ctx->stream;
    DevScc &s = ctx->s;
    DevWork &w = ctx->w;
    *graphed = false;
    const bool coop = w.precision == TB_PREC_FP32 && (w.kind == kKindPersistent || w.kind == kKindPipelined);
    if (coop || ctx->p.no_graphs) {
        TB_TRY(density_eval(ctx, true));
        launch_scc_update(st, s, w.q, ctx->p.mix_beta, ctx->p.mix_history, ctx->p.scc_tol, w.shift, w.state);
        ctx->launches++;
        return TB_OK;
    }
    if (!ctx->scc_graph || ctx->scc_graph_gen != ctx->gen) {
        if (ctx->scc_graph) {
            cudaGraphExecDestroy(ctx->scc_graph);
            ctx->scc_graph = nullptr;
        }
        for (cudaEvent_t &e : ctx->graph_ev)
            if (!e) TB_CUDA(cudaEventCreate(&e));
        const int64_t l0 = ctx->launches, s0 = ctx->spmm_launches;
        const double b0 = ctx->spmm_bytes;
        TB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        ctx->capturing = true;
        int rc = density_eval(ctx, true);
        if (rc == TB_OK) {
            launch_scc_update(st, s, w.q, ctx->p.mix_beta, ctx->p.mix_history, ctx->p.scc_tol, w.shift, w.state);
            ctx->launches++;
        }
        ctx->capturing = false;
        cudaGraph_t g = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(st, &g);
        if (rc == TB_OK && ec == cudaSuccess) {
            const cudaError_t ei = cudaGraphInstantiate(&ctx->scc_graph, g, 0);
            if (ei != cudaSuccess) {
                ctx->scc_graph = nullptr;
                rc = fail(ctx, TB_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ei));
            }
        } else if (rc == TB_OK) {
            rc = fail(ctx, TB_ERR_CUDA, std::string("stream capture: ") + cudaGetErrorString(ec));
        }
        if (g) cudaGraphDestroy(g);
        // nothing ran yet: the counts of the captured iteration are added per replay
        ctx->g_launches = ctx->launches - l0;
        ctx->g_spmm_launches = ctx->spmm_launches - s0;
        ctx->g_spmm_bytes = ctx->spmm_bytes - b0;
        ctx->launches = l0;
        ctx->spmm_launches = s0;
        ctx->spmm_bytes = b0;
        if (rc != TB_OK) return rc;
        ctx->scc_graph_gen = ctx->gen;
    }
    TB_CUDA(cudaGraphLaunch(ctx->scc_graph, st));
    ctx->launches += ctx->g_launches;
    ctx->spmm_launches += ctx->g_spmm_launches;
    ctx->spmm_bytes += ctx->g_spmm_bytes;
    *graphed = true;
    return TB_OK;
}

// FP32-form check: the plain FP64 recurrence on the first min(64, n) identity
// columns with the a, b of the evaluation just run (the FP64 X is rebuilt from
// the same device state); moments into chk_d[(M+1)][n].
int fp32_check_slab(tb_ctx *ctx, bool have_shift, float *ms)
{
    DevMatrix &m = ctx->m;
    const int M = ctx->p.M;
    cudaStream_t st = ctx->stream;
    if (ctx->chk_M != M || !ctx->chk_d) {
        dfree(ctx->chk_T0);
        dfree(ctx->chk_T1);
        dfree(ctx->chk_d);
        ctx->chk_M = 0;
        TB_TRY(dalloc(ctx, ctx->chk_T0, (size_t)m.n * 64));
        TB_TRY(dalloc(ctx, ctx->chk_T1, (size_t)m.n * 64));
        TB_TRY(dalloc(ctx, ctx->chk_d, (size_t)(M + 1) * m.n));
        ctx->chk_M = M;
    }
    if (!m.x64) TB_TRY(dalloc(ctx, m.x64, (size_t)m.nnzb * 16));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    launch_build_x(st, m, have_shift ? ctx->w.shift : nullptr, TB_PREC_FP64, ctx->w.state);
    launch_slab_identity(st, ctx->chk_T0, m.n, 64, 0, TB_PREC_FP64);
    for (int kout = 1; kout <= M; kout++) {
        const bool odd = kout & 1;
        launch_cheb_step_f64(st, m, odd ? ctx->chk_T0 : ctx->chk_T1, odd ? ctx->chk_T1 : ctx->chk_T0, 64, 0,
                             kout == 1, ctx->chk_d, kout);
    }
    cudaEventRecord(e1, st);
    const cudaError_t e = cudaEventSynchronize(e1);
    cudaEventElapsedTime(ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    TB_CUDA(e);
    ctx->launches += 2 + M + 1;
    return TB_OK;
}

// max over the checked orbitals of |sum_k c_k g_k (d32[k][i] - d64[k][i])|
int fp32_check_compare(tb_ctx *ctx, double *err)
{
    const int M = ctx->p.M, n = ctx->m.n, cols = std::min(64, n);
    std::vector<double> d32((size_t)M * cols), d64((size_t)M * cols), c(M), g(M);
    TB_CUDA(cudaMemcpy2DAsync(d32.data(), cols * 8, ctx->w.d, (size_t)n * 8, cols * 8, M, cudaMemcpyDeviceToHost,
                              ctx->stream));
    TB_CUDA(cudaMemcpy2DAsync(d64.data(), cols * 8, ctx->chk_d, (size_t)n * 8, cols * 8, M, cudaMemcpyDeviceToHost,
                              ctx->stream));
    TB_CUDA(cudaMemcpyAsync(c.data(), ctx->w.c, M * 8, cudaMemcpyDeviceToHost, ctx->stream));
    TB_CUDA(cudaMemcpyAsync(g.data(), ctx->w.g, M * 8, cudaMemcpyDeviceToHost, ctx->stream));
    TB_CUDA(cudaStreamSynchronize(ctx->stream));
    double e = 0.0;
    for (int i = 0; i < cols; i++) {
        double s = 0.0;
        for (int k = 0; k < M; k++) s += c[k] * g[k] * (d32[(size_t)k * cols + i] - d64[(size_t)k * cols + i]);
        e = std::max(e, std::fabs(s));
    }
    *err = e;
    return TB_OK;
}

int read_state(tb_ctx *ctx, DevState &hs)
{
    TB_CUDA(cudaMemcpyAsync(&hs, ctx->w.state, sizeof(DevState), cudaMemcpyDeviceToHost, ctx->stream));
    return check_kernel_flags(ctx);
}

int state_status(tb_ctx *ctx, const DevState &hs)
{
    if (hs.status == TB_ERR_SPECTRUM)
        return fail(ctx, TB_ERR_SPECTRUM, "Gershgorin interval collapsed or too wide for the quadrature");
    if (hs.status == TB_ERR_BISECTION)
        return fail(ctx, TB_ERR_BISECTION, "electron count not bracketed by mu in the spectrum");
    if (hs.status == TB_ERR_DIVERGED) return fail(ctx, TB_ERR_DIVERGED, "SCC charges diverged");
    if (hs.status != 0) return fail(ctx, hs.status, "device reported an error");
    return TB_OK;
}

void begin_call(tb_ctx *ctx, cudaEvent_t *e0)
{
    ctx->launches = 0;
    ctx->spmm_launches = 0;
    ctx->spmm_bytes = 0.0;
    ctx->ev_used = 0;
    ctx->extra_moment_ms = 0.0;
    cudaEventCreate(e0);
    cudaEventRecord(*e0, ctx->stream);
}

void fill_report(tb_ctx *ctx, cudaEvent_t e0, const DevState &hs, int iters, tb_report *rep)
{
    cudaEvent_t e1;
    cudaEventCreate(&e1);
    cudaEventRecord(e1, ctx->stream);
    cudaEventSynchronize(e1);
    float tot = 0.f;
    cudaEventElapsedTime(&tot, e0, e1);
    double tm = 0.0;
    for (size_t i = 0; i < ctx->ev_used; i++) {
        float x = 0.f;
        cudaEventElapsedTime(&x, ctx->moment_events[i].first, ctx->moment_events[i].second);
        tm += x;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!rep) return;
    std::memset(rep, 0, sizeof(*rep));
    rep->lmin = hs.lmin;
    rep->lmax = hs.lmax;
    rep->a = hs.a;
    rep->b = hs.b;
    rep->mu = hs.mu;
    rep->n_electrons_found = hs.n_found;
    rep->e_band = hs.e_band;
    rep->dq_max = hs.dq_max;
    rep->scc_iters = iters;
    rep->bisect_rounds = hs.bisect_rounds;
    rep->column_block = ctx->w.B;
    rep->step_kernel = ctx->w.precision == TB_PREC_FP32 ? ctx->w.kind : 0;
    rep->precision = ctx->p.precision;
    rep->t_total_ms = tot;
    rep->t_moments_ms = tm + ctx->extra_moment_ms;
    rep->spmm_launches = ctx->spmm_launches;
    rep->spmm_bytes = ctx->spmm_bytes;
    rep->kernel_launches = ctx->launches;
    rep->asym_max = ctx->asym_max;
}

void free_all(tb_ctx *ctx)
{
    DevMatrix &m = ctx->m;
    dfree(m.rowptr);
    dfree(m.colidx);
    dfree(m.diagblk);
    dfree(m.blkrow);
    dfree(m.h0);
    dfree(m.h0diag);
    dfree(m.radius);
    dfree(m.x32);
    dfree(m.x64);
    dfree(m.xdiag32);
    DevScc &s = ctx->s;
    dfree(s.rowptr);
    dfree(s.colidx);
    dfree(s.val);
    dfree(s.q0);
    dfree(s.qin);
    dfree(s.qout);
    dfree(s.V);
    dfree(s.hist_q);
    dfree(s.hist_r);
    dfree(s.hist_meta);
    DevWork &w = ctx->w;
    dfree(w.shift);
    dfree(w.d);
    dfree(w.mom);
    dfree(w.g);
    dfree(w.c);
    dfree(w.rho);
    dfree(w.fq);
    dfree(w.costab);
    dfree(w.cand);
    dfree(w.diagP);
    dfree(w.q);
    dfree(w.partial);
    dfree(w.state);
    dfree(ctx->chk_T0);
    dfree(ctx->chk_T1);
    dfree(ctx->chk_d);
    ctx->chk_M = 0;
    {
        char *t0 = (char *)w.T0, *t1 = (char *)w.T1;
        dfree(t0);
        dfree(t1);
        w.T0 = w.T1 = nullptr;
    }
    w = DevWork{};
    dfree(ctx->sp.grp_ptr);
    dfree(ctx->sp.grp_rows);
    dfree(ctx->sp.lcol);
    dfree(ctx->sp.lself);
    ctx->sp = StagePlan{};
    dfree(ctx->pl.hdr);
    dfree(ctx->pl.runs);
    dfree(ctx->pl.rec);
    dfree(ctx->pl.nbr_ptr);
    dfree(ctx->pl.nbr);
    dfree(ctx->pl.flags);
    dfree(ctx->pl.err);
    ctx->pl = PipePlan{};
    dfree(ctx->pp.lcode);
    dfree(ctx->pp.hptr);
    dfree(ctx->pp.hrows);
    dfree(ctx->pp.nptr);
    dfree(ctx->pp.ngrp);
    dfree(ctx->pp.flags);
    dfree(ctx->pp.err);
    ctx->pp = PersistPlan{};
    if (ctx->sp2_scratch) cudaFree(ctx->sp2_scratch);
    ctx->sp2_scratch = nullptr;
}

}  // namespace

namespace tb {

void pipe_group_records(const int32_t *brow, const int32_t *bcol, int I0, int I1, int64_t blk0, int32_t *h,
                        std::vector<int32_t> &rec, std::vector<int32_t> &runs, std::vector<int32_t> &U)
{
    const int tb0 = brow[I0];
    U.assign(bcol + tb0, bcol + brow[I1]);
    std::sort(U.begin(), U.end());
    U.erase(std::unique(U.begin(), U.end()), U.end());
    const int nu = (int)U.size();
    const size_t rstart = rec.size();
    for (int I = I0; I <= I1; I++) rec.push_back(brow[I] - tb0);
    for (int t = tb0; t < brow[I1]; t++)
        rec.push_back((int32_t)(std::lower_bound(U.begin(), U.end(), bcol[t]) - U.begin()));
    for (int I = I0; I < I1; I++) rec.push_back((int32_t)(std::lower_bound(U.begin(), U.end(), I) - U.begin()));
    while ((rec.size() - rstart) % 4) rec.push_back(0);
    runs.clear();
    for (int k = 0; k < nu;) {
        int e = k + 1;
        while (e < nu && U[e] == U[e - 1] + 1) e++;
        runs.insert(runs.end(), {U[k], e - k, k, 0});
        k = e;
    }
    h[0] = nu;
    h[1] = (int32_t)(blk0 + tb0);
    h[2] = brow[I1] - tb0;
    h[3] = (int32_t)rstart;
    h[4] = (int32_t)(rec.size() - rstart);
    h[5] = I0;
    h[6] = (int32_t)(runs.size() / 4);
    h[7] = I1 - I0;
}

// Validation and conversion of a PETSc-style CSR (4 orbitals per atom) to
// symmetrised 4x4 BSR on the host: the pattern of H + H^T with every diagonal
// block present, values (H + H^T)/2 (runKPM, withSP2_deltaH.cpp:1536-1538),
// Gershgorin centres and radii.
int host_csr_to_bsr(int32_t n, const int32_t *rowptr, const int32_t *colidx, const double *vals,
                    const int32_t *orb2atom, int32_t natoms, HostBsr &hb, std::string &err)
{
    auto bad = [&](int code, const char *msg) {
        err = msg;
        return code;
    };
    if (n <= 0 || natoms <= 0 || !rowptr || !colidx || !vals || !orb2atom)
        return bad(TB_ERR_INVALID_ARG, "null array or non-positive size");
    if ((int64_t)natoms * 4 != n)
        return bad(TB_ERR_STRUCTURE, "n must be 4 * natoms (sp3: 4 orbitals per atom)");
    for (int i = 0; i < n; i++)
        if (orb2atom[i] != i / 4)
            return bad(TB_ERR_STRUCTURE,
                       "orb2atom must map orbitals 4a..4a+3 to atom a (contiguous sp3 blocks)");
    if (rowptr[0] != 0) return bad(TB_ERR_STRUCTURE, "rowptr[0] != 0");
    for (int i = 0; i < n; i++) {
        if (rowptr[i + 1] < rowptr[i]) return bad(TB_ERR_STRUCTURE, "rowptr not monotone");
        for (int k = rowptr[i]; k < rowptr[i + 1]; k++) {
            if (colidx[k] < 0 || colidx[k] >= n) return bad(TB_ERR_STRUCTURE, "column index out of range");
            if (k > rowptr[i] && colidx[k] <= colidx[k - 1])
                return bad(TB_ERR_STRUCTURE, "column indices not strictly increasing");
            if (!std::isfinite(vals[k])) return bad(TB_ERR_NONFINITE, "NaN/Inf in Hamiltonian");
        }
    }
    const int nb = natoms;
    std::vector<std::vector<int32_t>> pat(nb);
    for (int I = 0; I < nb; I++) pat[I].push_back(I);
    for (int i = 0; i < n; i++)
        for (int k = rowptr[i]; k < rowptr[i + 1]; k++) {
            const int I = i / 4, J = colidx[k] / 4;
            pat[I].push_back(J);
            pat[J].push_back(I);
        }
    hb.brow.assign(nb + 1, 0);
    for (int I = 0; I < nb; I++) {
        auto &v = pat[I];
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
        hb.brow[I + 1] = hb.brow[I] + (int32_t)v.size();
    }
    const int64_t nnzb = hb.brow[nb];
    hb.bcol.assign(nnzb, 0);
    hb.blkrow.assign(nnzb, 0);
    hb.diagblk.assign(nb, 0);
    for (int I = 0; I < nb; I++)
        for (size_t t = 0; t < pat[I].size(); t++) {
            hb.bcol[hb.brow[I] + t] = pat[I][t];
            hb.blkrow[hb.brow[I] + t] = I;
            if (pat[I][t] == I) hb.diagblk[I] = hb.brow[I] + (int32_t)t;
        }
    pat.clear();
    auto find_blk = [&](int I, int J) -> int64_t {
        const int32_t *b = hb.bcol.data() + hb.brow[I], *e = hb.bcol.data() + hb.brow[I + 1];
        return (int64_t)(std::lower_bound(b, e, J) - hb.bcol.data());
    };
    hb.blk.assign((size_t)nnzb * 16, 0.0);
    hb.asym = 0.0;
    for (int i = 0; i < n; i++)
        for (int k = rowptr[i]; k < rowptr[i + 1]; k++) {
            const int j = colidx[k];
            const double v = vals[k];
            const int64_t t1 = find_blk(i / 4, j / 4), t2 = find_blk(j / 4, i / 4);
            hb.blk[t1 * 16 + (i % 4) * 4 + (j % 4)] += 0.5 * v;
            hb.blk[t2 * 16 + (j % 4) * 4 + (i % 4)] += 0.5 * v;
            const int32_t *b = colidx + rowptr[j], *e = colidx + rowptr[j + 1];
            const int32_t *it = std::lower_bound(b, e, i);
            const double vt = (it != e && *it == i) ? vals[rowptr[j] + (it - b)] : 0.0;
            hb.asym = std::max(hb.asym, std::fabs(v - vt));
        }
    hb.h0diag.assign(n, 0.0);
    hb.radius.assign(n, 0.0);
    hb.lmin = 1e300;
    hb.lmax = -1e300;
    for (int I = 0; I < nb; I++)
        for (int r = 0; r < 4; r++) {
            double rad = 0.0, dg = 0.0;
            for (int t = hb.brow[I]; t < hb.brow[I + 1]; t++)
                for (int c = 0; c < 4; c++) {
                    const double v = hb.blk[(size_t)t * 16 + r * 4 + c];
                    if (hb.bcol[t] == I && c == r)
                        dg = v;
                    else
                        rad += std::fabs(v);
                }
            hb.h0diag[4 * I + r] = dg;
            hb.radius[4 * I + r] = rad;
            hb.lmin = std::min(hb.lmin, dg - rad);
            hb.lmax = std::max(hb.lmax, dg + rad);
        }
    return TB_OK;
}

int host_check_gamma(int32_t natoms, const int32_t *g_rowptr, const int32_t *g_colidx,
                     const double *g_vals, const double *q0, std::string &err)
{
    if (!g_rowptr || !g_colidx || !g_vals || !q0) {
        err = "null Gamma or q0 array";
        return TB_ERR_INVALID_ARG;
    }
    if (g_rowptr[0] != 0) {
        err = "Gamma rowptr[0] != 0";
        return TB_ERR_STRUCTURE;
    }
    for (int a = 0; a < natoms; a++) {
        if (g_rowptr[a + 1] < g_rowptr[a]) {
            err = "Gamma rowptr not monotone";
            return TB_ERR_STRUCTURE;
        }
        for (int k = g_rowptr[a]; k < g_rowptr[a + 1]; k++) {
            if (g_colidx[k] < 0 || g_colidx[k] >= natoms) {
                err = "Gamma column out of range";
                return TB_ERR_STRUCTURE;
            }
            if (!std::isfinite(g_vals[k])) {
                err = "NaN/Inf in Gamma";
                return TB_ERR_NONFINITE;
            }
        }
        if (!std::isfinite(q0[a])) {
            err = "NaN/Inf in q0";
            return TB_ERR_NONFINITE;
        }
    }
    return TB_OK;
}

}  // namespace tb

// ===========================================================================
// C-ABI
// ===========================================================================
// The SCC iterations from the state already on the device (ctx->s.qin, the
// Anderson ring and its meta): the Coulomb shift of the input charges, then
// one density evaluation and mixing update per iteration until the residual
// is below scc_tol.  Returns TB_OK, TB_ERR_NOT_CONVERGED at the cap, a state
// error, or a failure of the launches; *it_out is the last iteration run.
static int scc_loop(tb_ctx *ctx, int *it_out, DevState &hs)
{
    cudaStream_t st = ctx->stream;
    DevScc &s = ctx->s;
    DevWork &w = ctx->w;
    TB_CUDA(cudaMemsetAsync(w.state, 0, sizeof(DevState), st));
    launch_coulomb_shift(st, s, s.qin, s.V, w.shift);
    ctx->launches++;
    std::memset(&hs, 0, sizeof(hs));
    int it = 0, rc = TB_ERR_NOT_CONVERGED;
    for (it = 1; it <= ctx->p.scc_max_iter; it++) {
        bool graphed = false;
        TB_TRY(scc_iteration(ctx, &graphed));
        TB_CUDA(cudaGetLastError());
        TB_TRY(read_state(ctx, hs));
        if (graphed) {  // the replay's moment phase, timed by the graph's own events
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, ctx->graph_ev[0], ctx->graph_ev[1]) == cudaSuccess)
                ctx->extra_moment_ms += ms;
            else
                cudaGetLastError();  // a timing gap is not an error of the solve
        }
        if (hs.status) {
            rc = state_status(ctx, hs);
            break;
        }
        if (hs.converged) {
            rc = TB_OK;
            break;
        }
    }
    if (it > ctx->p.scc_max_iter) {
        it = ctx->p.scc_max_iter;
        fail(ctx, TB_ERR_NOT_CONVERGED, "SCC reached scc_max_iter");
    }
    *it_out = it;
    return rc;
}

// tb_params.fp64_small: while alive, a small structure of an FP32 context
// runs the plain FP64 recurrence (the context's own parameters are restored
// on destruction).
struct SmallFp64 {
    tb_ctx *ctx;
    bool on = false;
    int prec = 0, B = 0;
    explicit SmallFp64(tb_ctx *c) : ctx(c)
    {
        const int lim = c->p.fp64_small == 0 ? kSmallFp64N : c->p.fp64_small;
        if (c->p.precision == TB_PREC_FP32 && lim > 0 && c->m.n <= lim) {
            on = true;
            prec = c->p.precision;
            B = c->p.column_block;
            c->p.precision = TB_PREC_FP64;
            c->p.column_block = 256;  // ensure_work trims it to the matrix
        }
    }
    ~SmallFp64()
    {
        if (on) {
            ctx->p.precision = prec;
            ctx->p.column_block = B;
        }
    }
};

namespace tb {

// The Hamiltonian of a context from an already validated host BSR.
int set_hamiltonian_bsr(tb_ctx *ctx, int32_t n, int32_t natoms, const HostBsr &hb)
{
    ctx->gen++;
    TB_TRY(set_device(ctx));
    free_all(ctx);
    ctx->have_h = ctx->have_scc = false;
    // the autotuner's choice depends on the block pattern only: a new matrix
    // with the previous pattern (the next geometry of a relaxation, the same
    // cell again) keeps it
    if (hb.brow != ctx->tuned_brow || hb.bcol != ctx->tuned_bcol) {
        reset_tuning(ctx);
        ctx->tuned_brow = hb.brow;
        ctx->tuned_bcol = hb.bcol;
    }
    DevMatrix &m = ctx->m;
    m.n = n;
    m.natoms = natoms;
    m.nb = natoms;
    m.nnzb = (int64_t)hb.bcol.size();
    TB_TRY(upload(ctx, m.rowptr, hb.brow.data(), hb.brow.size()));
    TB_TRY(upload(ctx, m.colidx, hb.bcol.data(), hb.bcol.size()));
    TB_TRY(upload(ctx, m.blkrow, hb.blkrow.data(), hb.blkrow.size()));
    TB_TRY(upload(ctx, m.diagblk, hb.diagblk.data(), hb.diagblk.size()));
    TB_TRY(upload(ctx, m.h0, hb.blk.data(), hb.blk.size()));
    TB_TRY(upload(ctx, m.h0diag, hb.h0diag.data(), hb.h0diag.size()));
    TB_TRY(upload(ctx, m.radius, hb.radius.data(), hb.radius.size()));
    TB_TRY(dalloc(ctx, m.xdiag32, (size_t)n));
    TB_TRY(build_stage_plan(ctx, hb.brow, hb.bcol));
    TB_TRY(build_persist_plan(ctx, hb.brow, hb.bcol));
    TB_TRY(build_pipe_plan(ctx, hb.brow, hb.bcol));
    ctx->h0_lmin = hb.lmin;
    ctx->h0_lmax = hb.lmax;
    TB_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->asym_max = hb.asym;
    ctx->have_h = true;
    return TB_OK;
}

}  // namespace tb

extern "C" {

int tb_abi_version(void) { return TB_ABI_VERSION; }

const char *tb_status_string(int s)
{
    switch (s) {
    case TB_OK: return "ok";
    case TB_ERR_INVALID_ARG: return "invalid argument";
    case TB_ERR_STRUCTURE: return "bad matrix structure";
    case TB_ERR_NONFINITE: return "non-finite input";
    case TB_ERR_NOT_READY: return "input not set";
    case TB_ERR_SPECTRUM: return "spectral bounds unusable";
    case TB_ERR_BISECTION: return "chemical potential not bracketed";
    case TB_ERR_NOT_CONVERGED: return "iteration cap reached";
    case TB_ERR_DIVERGED: return "SCC diverged";
    case TB_ERR_CUDA: return "CUDA error";
    case TB_ERR_NO_DEVICE: return "no sm_103 CUDA device";
    case TB_ERR_OUT_OF_MEMORY: return "out of device memory";
    case TB_ERR_UNSUPPORTED: return "unsupported";
    case TB_ERR_TIMEOUT: return "a bounded device wait ran out";
    default: return "unknown status";
    }
}

int tb_params_init(tb_params *p)
{
    TB_ABI_TRY
    if (!p) return TB_ERR_INVALID_ARG;
    std::memset(p, 0, sizeof(*p));
    p->struct_size = sizeof(tb_params);
    p->M = 200;
    p->kernel = TB_KERNEL_JACKSON;
    p->precision = TB_PREC_FP64;
    p->kT = 0.01;
    p->n_electrons = 0.0;
    p->column_block = 0;
    p->device = 0;
    p->spectral_pad = 0.0;
    p->mu_tol = 1e-9;
    p->scc_tol = 1e-6;
    p->scc_max_iter = 100;
    p->mix_history = 16;
    p->mix_beta = 0.2;
    p->sp2_drop_tol = 1e-5;
    p->sp2_max_iter = 40;
    p->sp2_idem_tol = 1e-10;
    return TB_OK;
    TB_ABI_CATCH
}

int tb_ctx_create(const tb_params *p, tb_ctx **out)
{
    TB_ABI_TRY
    if (!out) return TB_ERR_INVALID_ARG;
    *out = nullptr;
    int rc = check_params(nullptr, p);
    if (rc) return rc;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= p->device || p->device < 0) {
        cudaGetLastError();
        return TB_ERR_NO_DEVICE;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, p->device) != cudaSuccess) return TB_ERR_NO_DEVICE;
    if (!(prop.major == 10 && prop.minor == 3)) return TB_ERR_NO_DEVICE;
    tb_ctx *ctx = new (std::nothrow) tb_ctx();
    if (!ctx) return TB_ERR_OUT_OF_MEMORY;
    ctx->p = *p;
    ctx->device = p->device;
    if (cudaSetDevice(ctx->device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete ctx;
        return TB_ERR_CUDA;
    }
    *out = ctx;
    return TB_OK;
    TB_ABI_CATCH
}

int tb_ctx_destroy(tb_ctx *ctx)
{
    TB_ABI_TRY
    if (!ctx) return TB_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    free_all(ctx);
    for (auto &e : ctx->moment_events) {
        cudaEventDestroy(e.first);
        cudaEventDestroy(e.second);
    }
    if (ctx->scc_graph) cudaGraphExecDestroy(ctx->scc_graph);
    for (cudaEvent_t e : ctx->graph_ev)
        if (e) cudaEventDestroy(e);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return TB_OK;
    TB_ABI_CATCH
}

int tb_set_params(tb_ctx *ctx, const tb_params *p)
{
    TB_ABI_TRY
    if (!ctx) return TB_ERR_INVALID_ARG;
    ctx->gen++;
    TB_TRY(check_params(ctx, p));
    if (p->device != ctx->device) return fail(ctx, TB_ERR_INVALID_ARG, "device cannot change");
    // the tuned slab width was admitted for this M's column-sum array (K x G x B)
    if (p->M != ctx->p.M) reset_tuning(ctx);
    const double ne = ctx->p.n_electrons;
    ctx->p = *p;
    if (!(p->n_electrons > 0) && ctx->have_scc) ctx->p.n_electrons = ne;
    return TB_OK;
    TB_ABI_CATCH
}

int tb_get_params(const tb_ctx *ctx, tb_params *p)
{
    TB_ABI_TRY
    if (!ctx || !p) return TB_ERR_INVALID_ARG;
    *p = ctx->p;
    return TB_OK;
    TB_ABI_CATCH
}

const char *tb_last_error(const tb_ctx *ctx)
{
    if (!ctx) return "no context";
    return ctx->err.c_str();
}

int tb_set_hamiltonian(tb_ctx *ctx, int32_t n, const int32_t *rowptr, const int32_t *colidx,
                       const double *vals, const int32_t *orb2atom, int32_t natoms)
{
    TB_ABI_TRY
    if (!ctx) return TB_ERR_INVALID_ARG;
    ctx->gen++;
    HostBsr hb;
    const int vrc = host_csr_to_bsr(n, rowptr, colidx, vals, orb2atom, natoms, hb, ctx->err);
    if (vrc) return vrc;
    return set_hamiltonian_bsr(ctx, n, natoms, hb);
    TB_ABI_CATCH
}

int tb_set_geometry(tb_ctx *ctx, int32_t natoms, const double *xyz, const int32_t *species,
                    const double *box, double rcut_bohr, double gamma_diag)
{
    TB_ABI_TRY
    if (!ctx) return TB_ERR_INVALID_ARG;
    ctx->gen++;
    if (natoms <= 0 || !xyz || !species || !box || !(rcut_bohr > 0) || !std::isfinite(gamma_diag))
        return fail(ctx, TB_ERR_INVALID_ARG, "bad geometry arguments");
    for (int d = 0; d < 3; d++) {
        if (!(box[d] >= 0) || !std::isfinite(box[d])) return fail(ctx, TB_ERR_INVALID_ARG, "bad box");
        if (box[d] > 0 && box[d] <= 2.0 * rcut_bohr)
            return fail(ctx, TB_ERR_INVALID_ARG, "periodic box edges must exceed 2 * rcut (one image per pair)");
    }
    for (int i = 0; i < natoms; i++) {
        if (species[i] != 14 && species[i] != 8)
            return fail(ctx, TB_ERR_STRUCTURE, "species must be 14 (Si) or 8 (O)");
        for (int d = 0; d < 3; d++)
            if (!std::isfinite(xyz[3 * i + d])) return fail(ctx, TB_ERR_NONFINITE, "NaN/Inf in positions");
    }
    TB_TRY(set_device(ctx));
    free_all(ctx);
    ctx->have_h = ctx->have_scc = false;
    reset_tuning(ctx);
    ctx->tuned_brow.clear();  // a pattern built on the device: no host copy to compare
    ctx->tuned_bcol.clear();
    GeomDevice g;
    const int rc = geom_build_device(ctx->stream, natoms, xyz, species, box, rcut_bohr, gamma_diag, g, ctx->err);
    DevMatrix &m = ctx->m;
    m.rowptr = g.rowptr;
    m.colidx = g.colidx;
    m.blkrow = g.blkrow;
    m.diagblk = g.diagblk;
    m.h0 = g.h0;
    m.h0diag = g.h0diag;
    m.radius = g.radius;
    DevScc &sc = ctx->s;
    sc.val = g.gval;
    sc.q0 = g.q0;
    if (rc) return rc;
    m.n = 4 * natoms;
    m.natoms = m.nb = natoms;
    m.nnzb = g.nnzb;
    TB_TRY(dalloc(ctx, m.xdiag32, (size_t)m.n));
    sc.natoms = natoms;
    sc.nnz = g.nnzb;
    TB_TRY(upload(ctx, sc.rowptr, g.brow.data(), g.brow.size()));
    TB_TRY(upload(ctx, sc.colidx, g.bcol.data(), g.bcol.size()));
    TB_TRY(dalloc(ctx, sc.qin, (size_t)natoms));
    TB_TRY(dalloc(ctx, sc.qout, (size_t)natoms));
    TB_TRY(dalloc(ctx, sc.V, (size_t)natoms));
    TB_TRY(dalloc(ctx, sc.hist_q, (size_t)kMaxHistory * natoms));
    TB_TRY(dalloc(ctx, sc.hist_r, (size_t)kMaxHistory * natoms));
    TB_TRY(dalloc(ctx, sc.hist_meta, 2));
    TB_TRY(build_stage_plan(ctx, g.brow, g.bcol));
    TB_TRY(build_persist_plan(ctx, g.brow, g.bcol));
    TB_TRY(build_pipe_plan(ctx, g.brow, g.bcol));
    double mn = 1e300, mx = -1e300, ne = 0.0;
    for (int i = 0; i < m.n; i++) {
        mn = std::min(mn, g.h0diag_h[i] - g.radius_h[i]);
        mx = std::max(mx, g.h0diag_h[i] + g.radius_h[i]);
    }
    for (int i = 0; i < natoms; i++) ne += species[i] == 14 ? 4.0 : 6.0;
    ctx->h0_lmin = mn;
    ctx->h0_lmax = mx;
    if (!(ctx->p.n_electrons > 0)) ctx->p.n_electrons = ne;
    ctx->asym_max = 0.0;
    TB_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->have_h = ctx->have_scc = true;
    return TB_OK;
    TB_ABI_CATCH
}

int tb_set_scc(tb_ctx *ctx, int32_t natoms, const int32_t *g_rowptr, const int32_t *g_colidx,
               const double *g_vals, const double *q0)
{
    TB_ABI_TRY
    if (!ctx) return TB_ERR_INVALID_ARG;
    ctx->gen++;
    if (!ctx->have_h) return fail(ctx, TB_ERR_NOT_READY, "tb_set_hamiltonian must come first");
    if (natoms != ctx->m.natoms) return fail(ctx, TB_ERR_INVALID_ARG, "natoms mismatch");
    {
        const int grc = host_check_gamma(natoms, g_rowptr, g_colidx, g_vals, q0, ctx->err);
        if (grc) return grc;
    }
    TB_TRY(set_device(ctx));
    DevScc &s = ctx->s;
    s.natoms = natoms;
    s.nnz = g_rowptr[natoms];
    TB_TRY(upload(ctx, s.rowptr, g_rowptr, (size_t)natoms + 1));
    TB_TRY(upload(ctx, s.colidx, g_colidx, (size_t)s.nnz));
    TB_TRY(upload(ctx, s.val, g_vals, (size_t)s.nnz));
    TB_TRY(upload(ctx, s.q0, q0, (size_t)natoms));
    TB_TRY(dalloc(ctx, s.qin, (size_t)natoms));
    TB_TRY(dalloc(ctx, s.qout, (size_t)natoms));
    TB_TRY(dalloc(ctx, s.V, (size_t)natoms));
    TB_TRY(dalloc(ctx, s.hist_q, (size_t)kMaxHistory * natoms));
    TB_TRY(dalloc(ctx, s.hist_r, (size_t)kMaxHistory * natoms));
    TB_TRY(dalloc(ctx, s.hist_meta, 2));
    double ne = 0.0;
    for (int a = 0; a < natoms; a++) ne += q0[a];
    if (!(ctx->p.n_electrons > 0)) ctx->p.n_electrons = ne;
    TB_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->have_scc = true;
    return TB_OK;
    TB_ABI_CATCH
}

int tb_gershgorin(tb_ctx *ctx, const double *shift, double *lmin, double *lmax)
{
    TB_ABI_TRY
    if (!ctx || !lmin || !lmax) return TB_ERR_INVALID_ARG;
    if (!ctx->have_h) return fail(ctx, TB_ERR_NOT_READY, "Hamiltonian not set");
    TB_TRY(set_device(ctx));
    TB_TRY(ensure_work(ctx));
    if (shift) TB_CUDA(cudaMemcpyAsync(ctx->w.shift, shift, sizeof(double) * ctx->m.n,
                                       cudaMemcpyHostToDevice, ctx->stream));
    launch_gershgorin(ctx->stream, ctx->m, shift ? ctx->w.shift : nullptr, 0.0, ctx->p.kT, ctx->p.M,
                      ctx->w.nq_cap, ctx->w.state);
    TB_CUDA(cudaGetLastError());
    DevState hs;
    TB_TRY(read_state(ctx, hs));
    *lmin = hs.lmin;
    *lmax = hs.lmax;
    return TB_OK;
    TB_ABI_CATCH
}

int tb_density(tb_ctx *ctx, const double *shift, double *diagP, double *q, double *e_band,
               double *mu, double *moments, tb_report *rep)
{
    TB_ABI_TRY
    if (!ctx) return TB_ERR_INVALID_ARG;
    if (!ctx->have_h) return fail(ctx, TB_ERR_NOT_READY, "Hamiltonian not set");
    if (!(ctx->p.n_electrons > 0))
        return fail(ctx, TB_ERR_NOT_READY, "n_electrons unset (give it in tb_params or tb_set_scc)");
    if (shift)
        for (int i = 0; i < ctx->m.n; i++)
            if (!std::isfinite(shift[i])) return fail(ctx, TB_ERR_NONFINITE, "NaN/Inf in shift");
    if (ctx->p.mode == TB_MODE_SP2) {
        if (shift) return fail(ctx, TB_ERR_UNSUPPORTED, "SP2 mode takes no diagonal shift");
        return tb_sp2(ctx, diagP, q, e_band, rep);
    }
    TB_TRY(set_device(ctx));
    SmallFp64 small(ctx);
    TB_TRY(ensure_work(ctx));
    cudaEvent_t e0;
    begin_call(ctx, &e0);
    if (shift)
        TB_CUDA(cudaMemcpyAsync(ctx->w.shift, shift, sizeof(double) * ctx->m.n,
                                cudaMemcpyHostToDevice, ctx->stream));
    TB_TRY(density_eval(ctx, shift != nullptr));
    DevState hs;
    TB_TRY(read_state(ctx, hs));
    int rc = state_status(ctx, hs);
    const bool check = ctx->p.check_fp32 && ctx->p.precision == TB_PREC_FP32 && rc == TB_OK;
    double chk_err = 0.0;
    float chk_ms = 0.f;
    if (check) {
        TB_TRY(fp32_check_slab(ctx, shift != nullptr, &chk_ms));
        TB_TRY(fp32_check_compare(ctx, &chk_err));
    }
    const size_t n = ctx->m.n, na = ctx->m.natoms;
    if (diagP) TB_CUDA(cudaMemcpyAsync(diagP, ctx->w.diagP, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (q) TB_CUDA(cudaMemcpyAsync(q, ctx->w.q, na * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (moments)
        TB_CUDA(cudaMemcpyAsync(moments, ctx->w.mom, (ctx->p.M + 1) * 8, cudaMemcpyDeviceToHost,
                                ctx->stream));
    TB_CUDA(cudaStreamSynchronize(ctx->stream));
    if (e_band) *e_band = hs.e_band;
    if (mu) *mu = hs.mu;
    fill_report(ctx, e0, hs, 1, rep);
    if (rep) {
        rep->fp32_diag_err = chk_err;
        rep->fp32_check_ms = chk_ms;
        if (small.on) {
            rep->fp64_evals = 1;
            rep->precision = TB_PREC_FP64;
        }
    }
    return rc;
    TB_ABI_CATCH
}

int tb_coulomb_shift(tb_ctx *ctx, const double *q, double *V)
{
    TB_ABI_TRY
    if (!ctx || !q || !V) return TB_ERR_INVALID_ARG;
    if (!ctx->have_scc) return fail(ctx, TB_ERR_NOT_READY, "SCC data not set");
    TB_TRY(set_device(ctx));
    const size_t na = ctx->s.natoms;
    TB_CUDA(cudaMemcpyAsync(ctx->s.qout, q, na * 8, cudaMemcpyHostToDevice, ctx->stream));
    launch_coulomb_shift(ctx->stream, ctx->s, ctx->s.qout, ctx->s.V, nullptr);
    TB_CUDA(cudaGetLastError());
    TB_CUDA(cudaMemcpyAsync(V, ctx->s.V, na * 8, cudaMemcpyDeviceToHost, ctx->stream));
    TB_CUDA(cudaStreamSynchronize(ctx->stream));
    return TB_OK;
    TB_ABI_CATCH
}

int tb_scc_solve(tb_ctx *ctx, const double *q_init, double *q, double *diagP, double *e_band,
                 double *mu, int32_t *iters, tb_report *rep)
{
    TB_ABI_TRY
    if (!ctx) return TB_ERR_INVALID_ARG;
    if (!ctx->have_h || !ctx->have_scc)
        return fail(ctx, TB_ERR_NOT_READY, "Hamiltonian and SCC data must be set");
    if (ctx->p.mode != TB_MODE_KPE)
        return fail(ctx, TB_ERR_UNSUPPORTED, "the SCC loop runs on the KPE solver only (as the reference's)");
    const size_t n = ctx->m.n, na = ctx->m.natoms;
    if (q_init)
        for (size_t a = 0; a < na; a++)
            if (!std::isfinite(q_init[a])) return fail(ctx, TB_ERR_NONFINITE, "NaN/Inf in q_init");
    TB_TRY(set_device(ctx));
    SmallFp64 small(ctx);
    TB_TRY(ensure_work(ctx));
    cudaEvent_t e0;
    begin_call(ctx, &e0);
    cudaStream_t st = ctx->stream;
    DevScc &s = ctx->s;
    DevWork &w = ctx->w;
    if (q_init)
        TB_CUDA(cudaMemcpyAsync(s.qin, q_init, na * 8, cudaMemcpyHostToDevice, st));
    else
        TB_CUDA(cudaMemcpyAsync(s.qin, s.q0, na * 8, cudaMemcpyDeviceToDevice, st));
    TB_CUDA(cudaMemsetAsync(s.hist_meta, 0, 2 * sizeof(int32_t), st));
    DevState hs;
    int it = 0;
    const int rc = scc_loop(ctx, &it, hs);
    if (rc != TB_OK && rc != TB_ERR_NOT_CONVERGED && !(rc >= TB_ERR_SPECTRUM && rc <= TB_ERR_DIVERGED)) return rc;
    if (q) TB_CUDA(cudaMemcpyAsync(q, w.q, na * 8, cudaMemcpyDeviceToHost, st));
    if (diagP) TB_CUDA(cudaMemcpyAsync(diagP, w.diagP, n * 8, cudaMemcpyDeviceToHost, st));
    TB_CUDA(cudaStreamSynchronize(st));
    if (e_band) *e_band = hs.e_band;
    if (mu) *mu = hs.mu;
    if (iters) *iters = it;
    fill_report(ctx, e0, hs, it, rep);
    if (rep && small.on) {
        rep->fp64_evals = it;
        rep->precision = TB_PREC_FP64;
    }
    return rc;
    TB_ABI_CATCH
}

int tb_sp2(tb_ctx *ctx, double *diagP, double *q, double *e_band, tb_report *rep)
{
    TB_ABI_TRY
    if (!ctx) return TB_ERR_INVALID_ARG;
    if (!ctx->have_h) return fail(ctx, TB_ERR_NOT_READY, "Hamiltonian not set");
    if (!(ctx->p.n_electrons > 0))
        return fail(ctx, TB_ERR_NOT_READY, "n_electrons unset (give it in tb_params or tb_set_scc)");
    TB_TRY(set_device(ctx));
    cudaEvent_t e0;
    begin_call(ctx, &e0);
    tb_report r;
    std::memset(&r, 0, sizeof(r));
    const int rc = run_sp2(ctx, diagP, q, e_band, &r, nullptr, 0);
    cudaEvent_t e1;
    cudaEventCreate(&e1);
    cudaEventRecord(e1, ctx->stream);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    r.t_total_ms = ms;
    r.asym_max = ctx->asym_max;
    if (rep) *rep = r;
    return rc;
    TB_ABI_CATCH
}

int tb_density_stochastic(tb_ctx *ctx, const double *shift, int32_t n_probes, uint64_t seed,
                          int32_t dos_moments, int32_t dos_points, double *diagP, double *q, double *mu,
                          tb_report *rep)
{
    TB_ABI_TRY
    if (!ctx) return TB_ERR_INVALID_ARG;
    if (!ctx->have_h) return fail(ctx, TB_ERR_NOT_READY, "Hamiltonian not set");
    if (!(ctx->p.n_electrons > 0))
        return fail(ctx, TB_ERR_NOT_READY, "n_electrons unset (give it in tb_params or tb_set_scc)");
    if (n_probes < 1 || n_probes > 65536 || dos_moments < 2 || dos_moments > 100000 || dos_points < 2 ||
        dos_points > 1000000)
        return fail(ctx, TB_ERR_INVALID_ARG,
                    "need 1 <= n_probes <= 65536, 2 <= dos_moments <= 100000, 2 <= dos_points <= 1e6");
    if (shift)
        for (int i = 0; i < ctx->m.n; i++)
            if (!std::isfinite(shift[i])) return fail(ctx, TB_ERR_NONFINITE, "NaN/Inf in shift");
    TB_TRY(set_device(ctx));
    TB_TRY(ensure_work(ctx));
    cudaEvent_t e0;
    begin_call(ctx, &e0);
    if (shift)
        TB_CUDA(cudaMemcpyAsync(ctx->w.shift, shift, sizeof(double) * ctx->m.n, cudaMemcpyHostToDevice,
                                ctx->stream));
    int64_t nl = 0;
    TB_TRY(run_density_stochastic(ctx, shift ? ctx->w.shift : nullptr, n_probes, seed, dos_moments, dos_points,
                                  &nl));
    DevState hs;
    TB_CUDA(cudaMemcpyAsync(&hs, ctx->w.state, sizeof(DevState), cudaMemcpyDeviceToHost, ctx->stream));
    if (diagP) TB_CUDA(cudaMemcpyAsync(diagP, ctx->w.diagP, ctx->m.n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (q) TB_CUDA(cudaMemcpyAsync(q, ctx->w.q, ctx->m.natoms * 8, cudaMemcpyDeviceToHost, ctx->stream));
    TB_CUDA(cudaStreamSynchronize(ctx->stream));
    if (hs.status == TB_ERR_SPECTRUM)
        return fail(ctx, TB_ERR_SPECTRUM, "DOS support collapsed or too wide for the quadrature");
    if (mu) *mu = hs.mu;
    cudaEvent_t e1;
    cudaEventCreate(&e1);
    cudaEventRecord(e1, ctx->stream);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rep) {
        std::memset(rep, 0, sizeof(*rep));
        rep->lmin = hs.lmin;
        rep->lmax = hs.lmax;
        rep->a = hs.a;
        rep->b = hs.b;
        rep->mu = hs.mu;
        rep->t_total_ms = ms;
        rep->kernel_launches = nl;
        rep->precision = TB_PREC_FP64;
    }
    return TB_OK;
    TB_ABI_CATCH
}

int tb_kpm_dos(tb_ctx *ctx, int32_t n_moments, int32_t n_random, uint64_t seed, int32_t npts,
               double *moments, double *energies, double *dos, tb_report *rep)
{
    TB_ABI_TRY
    if (!ctx) return TB_ERR_INVALID_ARG;
    if (!ctx->have_h) return fail(ctx, TB_ERR_NOT_READY, "Hamiltonian not set");
    if (n_moments < 2 || n_moments > 100000 || n_random < 1 || n_random > 4096 || npts < 1 ||
        !moments || !energies || !dos)
        return fail(ctx, TB_ERR_INVALID_ARG,
                    "need 2 <= n_moments <= 100000, 1 <= n_random <= 4096, npts >= 1, outputs");
    TB_TRY(set_device(ctx));
    cudaEvent_t e0;
    begin_call(ctx, &e0);
    double a = 0.0, b = 0.0;
    int64_t nl = 0;
    const int rc = run_kpm_dos(ctx, n_moments, n_random, seed, npts, moments, energies, dos, &a, &b, &nl);
    cudaEvent_t e1;
    cudaEventCreate(&e1);
    cudaEventRecord(e1, ctx->stream);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rep) {
        std::memset(rep, 0, sizeof(*rep));
        rep->a = a;
        rep->b = b;
        rep->lmin = b - a;
        rep->lmax = b + a;
        rep->t_total_ms = ms;
        rep->kernel_launches = nl;
        rep->precision = TB_PREC_FP64;
    }
    return rc;
    TB_ABI_CATCH
}

}  // extern "C"

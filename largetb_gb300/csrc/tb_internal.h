// tb_internal.h -- shared declarations of the largeTB GB300 hot path
// (context layout, device scratch, kernel launchers).  Not part of the ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <new>
#include <string>
#include <vector>

#include "../../include/largetb.h"
#include "tb_abi_guard.h"

namespace tb {

// Scalars of one density evaluation, resident in device memory so that a
// whole SCC iteration runs without a host round trip.
struct DevState {
    double lmin, lmax, a, b;  // Gershgorin bounds, X = (H - b)/a
    double lo, hi;            // bisection bracket (scaled units)
    double mu_x, mu;          // chemical potential, scaled and Hartree
    double n_found, e_band;
    double dq_max;
    double beta_x;            // a / kT (0: step function)
    int32_t nq;               // quadrature nodes
    int32_t bisect_done;
    int32_t bisect_rounds;
    int32_t status;           // enum tb_status raised on the device
    int32_t converged;
    uint32_t ticket;          // last-block counter of the multisection round
};

// Candidates evaluated per multisection round.
constexpr int kBisectCand = 128;
constexpr int kBisectRounds = 8;
constexpr int kMaxHistory = 16;

// Device buffers owned by a context.  All sizes in elements.
struct DevMatrix {
    int32_t n = 0, natoms = 0, nb = 0;
    int64_t nnzb = 0;
    int32_t *rowptr = nullptr;   // nb+1
    int32_t *colidx = nullptr;   // nnzb
    int32_t *diagblk = nullptr;  // nb: index of block (I,I)
    int32_t *blkrow = nullptr;   // nnzb: block row of each stored block
    double *h0 = nullptr;        // nnzb*16, symmetrised H blocks (row-major 4x4)
    double *h0diag = nullptr;    // n
    double *radius = nullptr;    // n, Gershgorin radius sum_{j!=i} |H_ij|
    float *x32 = nullptr;        // nnzb*16 scaled blocks (FP32 form)
    double *x64 = nullptr;       // nnzb*16 scaled blocks (FP64 form)
    float *xdiag32 = nullptr;    // n, diagonal of the FP32 X actually used
};

// Row-group staging plan of the FP32 step kernel (see k_cheb_f32_staged).
struct StagePlan {
    int32_t R = 0, G = 0, maxU = 0, maxBlk = 0;
    int64_t totalU = 0;
    int32_t *grp_ptr = nullptr;   // G+1
    int32_t *grp_rows = nullptr;  // totalU distinct block rows per group
    int32_t *lcol = nullptr;      // nnzb: local index of colidx[t] in its group's list
    int32_t *lself = nullptr;     // nb: local index of block row I in its own group's list
};

// Plan of the pipelined FP32 kernel (k_cheb_f32_pipe): row groups of R block
// rows; per group a header {nu, tb0, nbk, rec_off, rec_len, 0, nruns, nr},
// the runs of consecutive distinct referenced rows {J0, rows, slot0, 0} at a
// fixed stride of run_stride per group, and a packed index record [local row offsets (nr+1) | local column per
// block (nbk) | own-row slot (nr)] padded to 4 ints (16-byte aligned).
struct PipePlan {
    int32_t R = 0, G = 0, maxU = 0, maxBlk = 0, stages = 0, nsm = 0;
    int32_t run_stride = 0;  // runs per group slot (a multiple of 32)
    bool coop = false;       // one CTA per SM fits: the one-launch-per-slab mode is available
    size_t stage_bytes = 0;
    int32_t *hdr = nullptr;
    int32_t *runs = nullptr;
    int32_t *rec = nullptr;
    int32_t *nbr_ptr = nullptr;  // G+1
    int32_t *nbr = nullptr;      // groups owning rows that group g references (g included)
    int32_t *flags = nullptr;    // completed steps per tile of the one-launch-per-slab mode
    int64_t flags_cap = 0;
    int32_t *err = nullptr;  // device error flag (bounded waits)
};

// One tile of the batched pipelined step: a row group of one structure x one
// 64-column chunk of that structure's chunk-major slabs.
struct PipeBatchTile {
    int64_t coff;   // float offset of the chunk in the slab buffers ([B_s/64][n_s][64] per structure)
    int64_t pbase;  // float2 offset of the tile's column sums (hi, lo) in the partial array
    int32_t g;      // row group: index into the plan's headers and copy runs
    int32_t pad[3];
};

// Chebyshev step kernels of the FP32 form (values of tb_params.fp32_kernel).
enum StepKind {
    kKindAuto = 0,
    kKindStaged = 1,
    kKindPersistent = 2,
    kKindPipelined = 3,     // k_cheb_f32_pipe, one cooperative launch per slab
    kKindPipelinedStep = 4  // k_cheb_f32_pipe, one launch per step
};
constexpr int kNumKinds = 5;

// Task plan of the persistent FP32 kernel (see k_cheb_f32_persistent).
struct PersistPlan {
    int32_t R = 0, G = 0, nc = 0, B = 0, maxH = 0, maxBlk = 0, maxNG = 0;
    int32_t *lcode = nullptr;  // nnzb: own row r (< R) or R + halo index
    int32_t *hptr = nullptr;   // G+1
    int32_t *hrows = nullptr;  // halo block rows per group
    int32_t *nptr = nullptr;   // G+1
    int32_t *ngrp = nullptr;   // neighbouring groups per group
    int32_t *flags = nullptr;  // G * nc step counters
    int32_t *err = nullptr;    // device wait-timeout flag
};

struct DevScc {
    int32_t natoms = 0;
    int64_t nnz = 0;
    int32_t *rowptr = nullptr, *colidx = nullptr;
    double *val = nullptr;
    double *q0 = nullptr;
    double *qin = nullptr, *qout = nullptr;
    double *V = nullptr;
    double *hist_q = nullptr, *hist_r = nullptr;  // kMaxHistory * natoms
    int32_t *hist_meta = nullptr;                 // {count, head}
};

struct DevWork {
    int32_t M = 0, nq_cap = 0, B = 0, K = 0, rowgroups = 0;
    int32_t precision = -1;
    int32_t kernel = -1;
    int32_t kind = 0;           // StepKind of the FP32 form (kKindStaged for FP64)
    double *shift = nullptr;   // n
    double *d = nullptr;       // (M+1) * n diagonal moments [k][i]
    double *mom = nullptr;     // M+1
    double *g = nullptr;       // M damping factors
    double *c = nullptr;       // M expansion coefficients
    double *rho = nullptr;     // [2 nq_cap]: damped DOS at the nodes, then e^{beta_x x_q}
    double *fq = nullptr;      // nq Fermi function at the quadrature nodes
    double *costab = nullptr;  // 4 nq_cap: cos(pi j / (2 nq_cap)), see k_cos_table
    double *cand = nullptr;    // kBisectCand electron counts
    double *diagP = nullptr;   // n
    double *q = nullptr;       // natoms
    double *partial = nullptr; // FP32 form: K * rowgroups * B * 2 dot-product slots, each a float2 (hi, lo)
    void *T0 = nullptr, *T1 = nullptr;  // slab buffers, n x B
    size_t slab_bytes = 0;
    int64_t partial_elems = 0;
    DevState *state = nullptr;
};

}  // namespace tb

struct tb_ctx {
    tb_params p{};
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    bool have_h = false, have_scc = false;
    double asym_max = 0.0;
    double h0_lmin = 0.0, h0_lmax = 0.0;  // Gershgorin bounds of the unshifted H
    tb::DevMatrix m;
    tb::DevScc s;
    tb::DevWork w;
    tb::StagePlan sp;
    tb::PersistPlan pp;
    tb::PipePlan pl;
    int64_t launches = 0;
    int64_t spmm_launches = 0;
    double spmm_bytes = 0.0;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> moment_events;
    size_t ev_used = 0;
    // autotuner result per precision and requested fp32_kernel: kind and slab
    // width (0 = not tuned yet)
    int tuned_kind[2][tb::kNumKinds] = {};
    int tuned_B[2][tb::kNumKinds] = {};
    std::vector<int32_t> tuned_brow, tuned_bcol;  // block pattern the tuned choices belong to
    // SP2 device scratch (lazily sized)
    // SCC iteration as a CUDA graph: captured once per configuration (gen) and
    // replayed; its moment-phase events are its own, its counts added per replay
    uint64_t gen = 1;
    cudaGraphExec_t scc_graph = nullptr;
    uint64_t scc_graph_gen = 0;
    cudaEvent_t graph_ev[2] = {nullptr, nullptr};
    bool capturing = false;
    int64_t g_launches = 0, g_spmm_launches = 0;
    double g_spmm_bytes = 0.0;
    double extra_moment_ms = 0.0;
    // FP32-vs-FP64 check of tb_density (tb_params.check_fp32): a 64-column FP64 slab
    double *chk_T0 = nullptr, *chk_T1 = nullptr, *chk_d = nullptr;
    int chk_M = 0;
    void *sp2_scratch = nullptr;
    size_t sp2_scratch_bytes = 0;
};

namespace tb {

// The most dynamic shared memory kernel `func` can opt in to on the current
// device: the per-block opt-in limit less the kernel's static shared memory.
// Kernels opt in to all of it: the attribute is per process, so a smaller
// value set for one context's plan must not cap another context's launches
// (the launch's own size still decides occupancy).
inline int smem_optin_max(const void *func)
{
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (v <= 0) v = 227 * 1024;
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, func) == cudaSuccess) v -= (int)fa.sharedSizeBytes;
    return v;
}

// ---- launchers implemented in tb_kpe.cu ----------------------------------
void launch_coulomb_shift(cudaStream_t st, const DevScc &s, const double *q, double *V,
                          double *shift);
void launch_gershgorin(cudaStream_t st, const DevMatrix &m, const double *shift, double pad,
                       double kT, int M, int nq_cap, DevState *state, double fix_lo = 0.0,
                       double fix_hi = 0.0);
void launch_build_x(cudaStream_t st, const DevMatrix &m, const double *shift, int precision,
                    const DevState *state);
void launch_slab_identity(cudaStream_t st, void *T0, int n, int B, int c0, int precision);
// One plain FP64 Chebyshev step on a slab: first != 0: Tout = X Tin, else
// Tout = 2 X Tin - Tout; the slab's diagonal entries go to d[kout].
void launch_cheb_step_f64(cudaStream_t st, const DevMatrix &m, const double *Tin, double *Tout,
                          int B, int c0, int first, double *d, int kout);
// One FP32 step with the fused column dot products of T_k.
void launch_cheb_step_f32(cudaStream_t st, const DevMatrix &m, const float *Tin, float *Tout,
                          int B, int first, float2 *partial_k, int rowgroups);
int cheb_f32_rowgroups(int nb);
size_t cheb_f32_staged_smem(int R, int maxU, int maxBlk);
int cheb_f32_staged_configure(size_t smem);  // returns a cudaError_t
size_t cheb_f32_persistent_smem(int R, int maxH, int maxBlk, int maxNG);
int cheb_f32_persistent_setup(int R, size_t smem, int *ctas_per_sm);  // returns a cudaError_t
int launch_cheb_f32_persistent(cudaStream_t st, const DevMatrix &m, const PersistPlan &pp, int K,
                               int B, int c0, float *G0, float *G1, float2 *partial, int *flags,
                               int *err);  // returns a cudaError_t
// ---- tb_mlp_tc.cu ----
void launch_mlp_forward_tc(cudaStream_t st, int n, const float *X, const float *mean, const float *istd,
                           const float *Wq, float *out, int32_t *err);

// ---- tb_pipe.cu ----
size_t cheb_f32_pipe_stage_bytes(int R, int maxU, int maxBlk, int rec_cap);
// identity columns in the chunk-major slab layout [B/64][n][64] of the pipelined kernel
void launch_slab_identity_cm(cudaStream_t st, float *T0, int n, int B, int c0);
size_t cheb_f32_pipe_smem(size_t stage_bytes, int stages);
// batch: the instance of launch_cheb_f32_pipe_batch.  Returns a cudaError_t.
int cheb_f32_pipe_configure(size_t smem, int *ctas_per_sm, bool batch = false);
// Steps k0 .. k0+steps-1 of a slab held in T0/T1 (chunk-major; step k reads
// T_k from T0 when k is even); partial: float2 (hi, lo) pairs in the slots of
// the double partial array, block k - k0 per step.  multi: one cooperative
// launch synchronised by per-tile flags; else a plain launch (steps = 1).
// Returns a cudaError_t.
int launch_cheb_f32_pipe(cudaStream_t st, const DevMatrix &m, const PipePlan &pl, float *T0, float *T1, int B,
                         int k0, int steps, float2 *partial, bool multi);
// Step k of every tile of a batch of structures (one plain launch): tiles
// ordered by structure, chunk and group; x32: the concatenated FP32 blocks.
void launch_cheb_f32_pipe_batch(cudaStream_t st, const PipePlan &pl, const PipeBatchTile *tiles, int ntiles,
                                const float *x32, float *T0, float *T1, int k, float2 *partial);
void launch_f32_finalize_pairs(cudaStream_t st, const DevMatrix &m, const float2 *partial, int K, int rowgroups,
                               int B, int c0, double *d, int M);
int launch_cheb_step_f32_staged(cudaStream_t st, const DevMatrix &m, const StagePlan &sp,
                                const float *Tin, float *Tout, int B, int first,
                                float2 *partial_k);
void launch_moment_sums(cudaStream_t st, const double *d, int n, int nmom, double *mom);
void launch_cos_table(cudaStream_t st, int nq_cap, double *tab);

// Records of the pipelined step kernel for the row group [I0, I1) of a block
// pattern (brow / bcol over one structure, rows local to it): the 8-int header
// at h (distinct referenced block rows nu, first block blk0 + brow[I0], blocks,
// record offset, record length, I0, copy runs, rows), the index record
// appended to rec (row pointers, slot of each block's column among the
// distinct rows, slot of each own row; padded to a multiple of 4) and the copy
// runs of consecutive rows (first row, rows, first slot, 0).  U returns the
// sorted distinct referenced rows.
void pipe_group_records(const int32_t *brow, const int32_t *bcol, int I0, int I1, int64_t blk0, int32_t *h,
                        std::vector<int32_t> &rec, std::vector<int32_t> &runs, std::vector<int32_t> &U);
void launch_dos_nodes(cudaStream_t st, const double *g, const double *mom, int M,
                      const DevState *state, int nq_cap, const double *tab, double *rho);
void launch_bisect_round(cudaStream_t st, const double *rho, const double *g, const double *mom,
                         const double *tab, int nq_cap, int M, double n_elec, double tol_n, int round,
                         double *cand, DevState *state);
void launch_fermi_coeffs(cudaStream_t st, int M, DevState *state, int nq_cap, const double *tab, double *fq,
                         double *c);
void launch_charges(cudaStream_t st, const double *d, const double *c, const double *g,
                    const double *mom, int M, int n, int natoms, double *diagP, double *q,
                    DevState *state);
void launch_scc_update(cudaStream_t st, DevScc &s, const double *qout, double beta, int history,
                       double tol, double *shift, DevState *state);

// ---- tb_api.cpp: host-side conversion shared by the context and the batch ----
struct HostBsr {
    std::vector<int32_t> brow, bcol, blkrow, diagblk;
    std::vector<double> blk, h0diag, radius;
    double asym = 0.0, lmin = 0.0, lmax = 0.0;
};
int host_csr_to_bsr(int32_t n, const int32_t *rowptr, const int32_t *colidx, const double *vals,
                    const int32_t *orb2atom, int32_t natoms, HostBsr &hb, std::string &err);
int host_check_gamma(int32_t natoms, const int32_t *g_rowptr, const int32_t *g_colidx,
                     const double *g_vals, const double *q0, std::string &err);
// tb_api.cpp: the Hamiltonian of a context from a validated host BSR (a
// batch member solved on its own in FP64, tb_params.fp64_small)
int set_hamiltonian_bsr(tb_ctx *ctx, int32_t n, int32_t natoms, const HostBsr &hb);
constexpr int kSmallFp64N = 512;  // default orbital limit of tb_params.fp64_small

// ---- tb_geom.cu ----------------------------------------------------------
struct GeomDevice {
    int64_t nnzb = 0;
    int32_t *rowptr = nullptr, *colidx = nullptr, *blkrow = nullptr, *diagblk = nullptr;
    double *h0 = nullptr, *h0diag = nullptr, *radius = nullptr, *gval = nullptr, *q0 = nullptr;
    std::vector<int32_t> brow, bcol;
    std::vector<double> h0diag_h, radius_h;
};
int geom_build_device(cudaStream_t st, int natoms, const double *xyz_h, const int32_t *sp_h,
                      const double box[3], double rcut, double gamma_diag, GeomDevice &out,
                      std::string &err);

// ---- tb_sp2.cu ----------------------------------------------------------
// SP2 purification of the context's H; branches_out (optional) receives the
// applied branch sequence (-1: X^2, +1: 2X - X^2).
int run_sp2(tb_ctx *ctx, double *diagP, double *q, double *e_band, tb_report *rep,
            int32_t *branches_out, int32_t branches_cap);

// ---- tb_dos.cu ----------------------------------------------------------
int run_density_stochastic(tb_ctx *ctx, const double *d_shift, int nr, uint64_t seed, int nmom_dos, int npts,
                           int64_t *launches);
int run_kpm_dos(tb_ctx *ctx, int nmom, int nr, uint64_t seed, int npts, double *mom, double *E,
                double *dos, double *a_out, double *b_out, int64_t *launches);

}  // namespace tb

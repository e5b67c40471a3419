/*
 * largetb.h -- C-ABI of the GB300 (sm_103a) density-matrix hot path for the
 * largeTB self-consistent-charge tight-binding code.
 *
 * The reference (pghale/largeTB, withSP2_deltaH.cpp / withSP2.cpp) runs this
 * path as PETSc CPU code on file-scope globals: runKPM() and
 * computeDensityMatrix() read the assembled AIJ matrix Htotal, the
 * orbital2Atom map and Nelectrons, and write muval, diagP and chargeOnAtom;
 * constructdeltaH()/updateHtotal() close the SCC loop.  This header replaces
 * those entry points with explicit, re-entrant calls on a context that owns
 * one CUDA device stream.  Conventions:
 *
 *   - Every function returns an int status: TB_OK (0) or a positive error
 *     code, like PetscErrorCode.  No C++ exception crosses this boundary.
 *     tb_last_error() gives the message of the last failure on a context.
 *   - Inputs are plain host arrays, copied during the call; the caller keeps
 *     ownership.  Outputs are caller-owned host arrays.  Every call is
 *     synchronous at return (like the reference's collective PETSc calls).
 *   - One context per host thread; a context is not thread-safe.
 *   - Units: bohr, Hartree, electrons.  Orbitals are 4 per atom (s, px, py,
 *     pz), contiguous: orbital i belongs to atom i/4, as the reference's
 *     localBeginIndex/localEndIndex layout (withSP2_deltaH.cpp:525-664).
 *   - Charges are electron counts over both spins: q_a = 2 sum_{i in a} P_ii;
 *     diagP is per spin (the reference's diagP, withSP2_deltaH.cpp:1375).
 *   - There is no CPU fallback: without a usable CUDA device every compute
 *     call returns TB_ERR_NO_DEVICE.
 */
#ifndef LARGETB_H
#define LARGETB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TB_ABI_VERSION 1

enum tb_status {
    TB_OK = 0,
    TB_ERR_INVALID_ARG = 1,   /* null pointer, bad size, bad parameter */
    TB_ERR_STRUCTURE = 2,     /* CSR not sorted/in range, or orb2atom not 4-per-atom contiguous */
    TB_ERR_NONFINITE = 3,     /* NaN or Inf in an input */
    TB_ERR_NOT_READY = 4,     /* Hamiltonian or SCC data not set */
    TB_ERR_SPECTRUM = 5,      /* Gershgorin interval collapsed (lmax <= lmin) */
    TB_ERR_BISECTION = 6,     /* electron count not bracketed by mu in [lmin, lmax] */
    TB_ERR_NOT_CONVERGED = 7, /* SCC or SP2 stopped at its iteration cap */
    TB_ERR_DIVERGED = 8,      /* SCC charges left any physical range */
    TB_ERR_CUDA = 9,          /* CUDA runtime error; message in tb_last_error */
    TB_ERR_NO_DEVICE = 10,    /* no CUDA device of compute capability 10.3 */
    TB_ERR_OUT_OF_MEMORY = 11,
    TB_ERR_UNSUPPORTED = 12,
    TB_ERR_TIMEOUT = 13       /* a bounded device wait ran out: the kernel stopped early and
                                 returned; results of the call are void, the context stays usable */
};

enum tb_precision {
    TB_PREC_FP64 = 0, /* plain form: FP64 recurrence, T_{k+1} = 2 X T_k - T_{k-1} */
    TB_PREC_FP32 = 1  /* FP32 recurrence to order M/2; moments from T_{2k} = 2 T_k^2 - 1,
                         T_{2k+1} = 2 T_k T_{k+1} - X, the column dot products summed as
                         FP32 TwoSum pairs (~44 bits) and returned in FP64 */
};

/* Chebyshev step kernel of the FP32 form (tb_params.fp32_kernel).  No
 * counterpart in the reference, whose recurrence is PETSc's MatMult. */
enum tb_fp32_kernel {
    TB_FP32_AUTO = 0,       /* autotuner picks kernel and slab width (column_block = 0);
                               with column_block set: pipelined where it fits, else staged */
    TB_FP32_STAGED = 1,     /* one launch per step, row-group staging in shared memory */
    TB_FP32_PERSISTENT = 2, /* one cooperative launch per slab, neighbour-synchronised */
    TB_FP32_PIPELINED = 3,     /* SM-resident CTAs with a bulk-copy stage ring; one cooperative
                                  launch per slab, tiles synchronised with their neighbours */
    TB_FP32_PIPELINED_STEP = 4 /* the same kernel, one launch per step */
};

/* Density-matrix solver of tb_density (tb_params.mode): the reference's two
 * programs, withSP2_deltaH.cpp (KPE) and withSP2.cpp (SP2). */
enum tb_mode {
    TB_MODE_KPE = 0, /* kernel polynomial expansion (runKPM + computeDensityMatrix) */
    TB_MODE_SP2 = 1  /* SP2 purification (getSP2 / computeAlphas); tb_density then
                        leaves mu and moments untouched, and tb_scc_solve answers
                        TB_ERR_UNSUPPORTED: the reference's SCC program is KPE only */
};

enum tb_kernel_kind {
    TB_KERNEL_JACKSON = 0,  /* closed form of runKPM, withSP2_deltaH.cpp:1593-1595 */
    TB_KERNEL_AUTOCORR = 1, /* getKPE's autocorrelation form, withSP2_deltaH.cpp:1104-1132 */
    TB_KERNEL_NONE = 2
};

typedef struct tb_params {
    uint32_t struct_size;  /* sizeof(tb_params); set by tb_params_init */
    int32_t M;             /* expansion terms n = 0..M-1 (getKPE's M, withSP2_deltaH.cpp:1094);
                              2 <= M <= 6000 */
    int32_t kernel;        /* enum tb_kernel_kind */
    int32_t precision;     /* enum tb_precision */
    double kT;             /* electronic temperature, Hartree; <= 0 selects the step
                              function of getKPE (withSP2_deltaH.cpp:1100-1103) */
    double n_electrons;    /* electrons, both spins; <= 0 takes sum(q0) from tb_set_scc */
    int32_t column_block;  /* identity columns per slab (multiple of 128), or 0: on the
                              first density evaluation of a matrix, time a few
                              Chebyshev steps of every kernel/width candidate and
                              keep the cheapest per column */
    int32_t device;        /* CUDA device ordinal */
    double spectral_pad;   /* relative widening of the Gershgorin interval */
    double mu_tol;         /* bisection tolerance on the electron count */
    double scc_tol;        /* convergence: max_a |q_out - q_in| < scc_tol (electrons) */
    int32_t scc_max_iter;
    int32_t mix_history;   /* Anderson mixing depth, 0 = linear mixing (max 16) */
    double mix_beta;       /* mixing parameter */
    double sp2_drop_tol;   /* SP2: drop 4x4 blocks with Frobenius norm below this */
    int32_t sp2_max_iter;
    int32_t fp32_kernel;   /* enum tb_fp32_kernel */
    double sp2_idem_tol;   /* SP2: stop when ||X^2 - X||_F < sp2_idem_tol */
    double bounds_lo;      /* if bounds_hi > bounds_lo: the spectral interval that sets   */
    double bounds_hi;      /* X = (H - b)/a for tb_density / tb_scc_solve / tb_kpm_dos
                              instead of Gershgorin, unpadded -- runKPM's refined a, b
                              (withSP2_deltaH.cpp:1696-1703); the caller vouches that it
                              holds the spectrum.  Default 0, 0: Gershgorin. */
    int32_t mode;          /* enum tb_mode */
    int32_t check_fp32;    /* FP32 form: tb_density also runs the plain FP64 recurrence on
                              the first 64 identity columns (same a, b) and reports the
                              largest diagP difference there (tb_report.fp32_diag_err) */
    int32_t no_graphs;     /* 1: launch every kernel of an SCC iteration directly instead of
                              replaying the iteration's captured CUDA graph (debugging,
                              profiling) */
    int32_t fp64_small;    /* FP32 form: structures of at most this many orbitals run the plain
                              FP64 recurrence instead (tb_density, tb_scc_solve, and batch
                              members, which then leave the batch).  Small structures are
                              launch-bound, so FP64 costs about what FP32 does there, and it
                              removes the FP32 recurrence's ~2e-7 e charge noise, which the
                              SCC response of surface slabs amplifies to ~1e-6 e at the fixed
                              point.  0: 512 orbitals; -1: never; k > 0: n <= k.
                              tb_report.fp64_evals counts the evaluations run so. */
    double reserved[2];
} tb_params;

typedef struct tb_report {
    double lmin, lmax;        /* Gershgorin bounds of the last density evaluation */
    double a, b;              /* X = (H - b)/a */
    double mu;                /* chemical potential, Hartree */
    double n_electrons_found; /* 2 sum_n c_n g_n mu_n at the returned mu */
    double e_band;            /* 2 tr(P H) */
    double dq_max;            /* last SCC residual max_a |q_out - q_in| */
    int32_t scc_iters;        /* density evaluations performed */
    int32_t bisect_rounds;
    int32_t column_block;     /* slab width used */
    int32_t precision;
    double t_total_ms;        /* CUDA-event time of the call on the context stream */
    double t_moments_ms;      /* CUDA-event time of the Chebyshev moment passes */
    int64_t spmm_launches;    /* Chebyshev step kernel launches */
    double spmm_bytes;        /* algorithmic bytes moved by those launches */
    int64_t kernel_launches;  /* all kernels this call launched */
    double asym_max;          /* max |H_ij - H_ji| seen by tb_set_hamiltonian */
    double idem_err;          /* SP2: ||X^2 - X||_F of the returned X */
    int32_t sp2_iters;
    int32_t step_kernel;      /* FP32 form: enum tb_fp32_kernel actually used */
    int64_t sp2_nnzb;         /* SP2: stored blocks of the returned X */
    double sp2_flops;         /* SP2: 128 x (4x4 block products) over all steps */
    double sp2_bytes;         /* SP2: algorithmic bytes, every X_k read once and X_{k+1} written once */
    double fp32_diag_err;     /* with check_fp32: max |diagP(FP32) - diagP(FP64)| over the
                                 checked orbitals, else 0 */
    double fp32_check_ms;     /* CUDA-event time of that check */
    double sp2_flops_done;    /* SP2: 128 x block products actually formed (the symmetric
                                 product forms the blocks J >= I only) */
    int32_t fp64_evals;       /* FP32 form: density evaluations run in FP64 by tb_params.fp64_small */
    int32_t reserved_i;
    double reserved[2];
} tb_report;

typedef struct tb_ctx tb_ctx;

/* Fill *p with defaults (M = 200, Jackson, kT = 0.01, FP64, Anderson 16 / 0.2,
 * scc_tol = 1e-6, SP2 drop 1e-5 / 40 iterations). */
int tb_params_init(tb_params *p);

/* Create a context on p->device.  Replaces PetscInitialize + the global state
 * of withSP2_deltaH.cpp:26-66.  Returns TB_ERR_NO_DEVICE without an sm_103
 * device. */
int tb_ctx_create(const tb_params *p, tb_ctx **out);
int tb_ctx_destroy(tb_ctx *ctx);

/* Replace the parameters of an existing context (precision, M, kT, ...). */
int tb_set_params(tb_ctx *ctx, const tb_params *p);
int tb_get_params(const tb_ctx *ctx, tb_params *p);

/* The assembled Hamiltonian Htotal as PETSc seqaij i/j/a arrays (what
 * MatGetRowIJ + MatSeqAIJGetArrayRead return) plus the orbital -> atom map
 * (row i of orbital2Atom, withSP2_deltaH.cpp:905-922).  Replaces the
 * MatSetValues(H/Htotal) assembly of constructH (withSP2_deltaH.cpp:969-1066)
 * as the input of runKPM.  n = 4 * natoms; column indices within a row must
 * be strictly increasing.  Missing transposed entries are filled and the
 * matrix is symmetrised as (H + H^T)/2 (runKPM, withSP2_deltaH.cpp:1536-1538);
 * the largest asymmetry is reported in tb_report.asym_max. */
int tb_set_hamiltonian(tb_ctx *ctx, int32_t n, const int32_t *rowptr, const int32_t *colidx,
                       const double *vals, const int32_t *orb2atom, int32_t natoms);

/* Gamma_ab as CSR (natoms x natoms) and the neutral electron counts q0 of
 * each atom.  Replaces initializeForSCF (withSP2_deltaH.cpp:854-967) and the
 * neutralCharges vector (withSP2_deltaH.cpp:713-720). */
int tb_set_scc(tb_ctx *ctx, int32_t natoms, const int32_t *g_rowptr, const int32_t *g_colidx,
               const double *g_vals, const double *q0);

/* Build H, Gamma and q0 on the GPU from atom positions (bohr, 3*natoms) and
 * species (14 Si, 8 O) in an orthorhombic box (box[d] > 0: periodic edge
 * along d, 0: open), neighbours with 0.1 < d^2 < rcut^2 under the minimum
 * image, the reference's sp3 block model, Gamma_aa = gamma_diag and 1/r off
 * the diagonal, q0 = 4 (Si) / 6 (O) electrons.  Replaces getHaloAtoms +
 * constructH + initializeForSCF (withSP2_deltaH.cpp:372-501, 969-1066,
 * 854-899) and stands in for tb_set_hamiltonian + tb_set_scc.  Periodic
 * edges must exceed 2 * rcut. */
int tb_set_geometry(tb_ctx *ctx, int32_t natoms, const double *xyz, const int32_t *species,
                    const double *box, double rcut_bohr, double gamma_diag);

/* Gershgorin bounds of H + diag(shift) (shift may be NULL).
 * Replaces GershGorinParallel, withSP2_deltaH.cpp:144-209. */
int tb_gershgorin(tb_ctx *ctx, const double *shift, double *lmin, double *lmax);

/* One density evaluation of H + diag(shift) (shift: n values or NULL):
 * Gershgorin scaling, exact-trace Chebyshev moments over identity column
 * slabs, Jackson damping, mu bisection on the electron count, then diagP (n),
 * q (natoms), e_band, mu and the moments mu_k = tr T_k(X), k = 0..M
 * (moments may be NULL).  Replaces runKPM + computeDensityMatrix
 * (withSP2_deltaH.cpp:1401-1411, 1528-1723) with the exact trace the
 * reference leaves commented out (lines 1361-1379). */
int tb_density(tb_ctx *ctx, const double *shift, double *diagP, double *q, double *e_band,
               double *mu, double *moments, tb_report *rep);

/* Coulomb shift V = Gamma (q - q0) per atom (natoms).  Replaces the
 * netCharges/gammaq steps of constructdeltaH, withSP2_deltaH.cpp:1424-1429;
 * the orbital shift of atom a is V_a on its four diagonal entries
 * (withSP2_deltaH.cpp:1443-1459). */
int tb_coulomb_shift(tb_ctx *ctx, const double *q, double *V);

/* Self-consistent charges: H = H0 + diag(V(q_in)), density, Anderson mixing,
 * until max_a |q_out - q_in| < scc_tol.  q_init may be NULL (start from q0).
 * Replaces the SCC loop of main, withSP2_deltaH.cpp:1820-1840 (which never
 * adds delta H: mixRatio = 0 at line 56).  Outputs: q and diagP of the last
 * evaluation, e_band, mu, iteration count.  Returns TB_ERR_NOT_CONVERGED at
 * scc_max_iter (outputs still written). */
int tb_scc_solve(tb_ctx *ctx, const double *q_init, double *q, double *diagP, double *e_band,
                 double *mu, int32_t *iters, tb_report *rep);

/* SP2 purification of H as a thresholded 4x4 block SpGEMM (FP32 blocks with
 * FP64 traces when precision is TB_PREC_FP32, FP64 otherwise).  X0 from the
 * Gershgorin bounds; per step X <- X^2 if 2 tr X > N_e else 2X - X^2
 * (computeAlphas branch rule, withSP2.cpp:1027-1030; getSP2 recursion,
 * withSP2.cpp:956-984).  Outputs diagP, q, e_band = 2 tr(X H); the report
 * carries iterations, ||X^2 - X||_F and the stored block count. */
int tb_sp2(tb_ctx *ctx, double *diagP, double *q, double *e_band, tb_report *rep);

/* The reference's default, stochastic density path (runKPM +
 * computeDensityMatrix with random vectors): replaces the DOS, chemical
 * potential and interval refinement of runKPM (withSP2_deltaH.cpp:1579-1703,
 * random vectors 1236-1264) and computeDiagonalElements' random-vector
 * estimator (1296-1399).  On H (+ diag(shift) if given, n doubles):
 *   1. the stochastic KPM DOS of tb_kpm_dos with n_probes Gaussian probes
 *      (counter-based stream `seed`), dos_moments Jackson-damped moments and
 *      dos_points nodes on the Gershgorin interval;
 *   2. mu where the DOS area from the bottom reaches N_e/(2n) of the total,
 *      and the interval [E_min, E_max] where DOS/n >= 0.001 first holds
 *      from either end (X = (H - b)/a with a, b of that interval);
 *   3. diagP_i = sum_r x_i (P x)_i / sum_r x_i^2 over n_probes fresh probes
 *      (stream seed + 1), P x = sum_{k<M} c_k g_k T_k(X) x with the Fermi
 *      (kT > 0) or step (kT <= 0) coefficients at mu and tb_params.kernel.
 * FP64 throughout.  diagP (n, per spin), q (natoms, both spins), mu
 * (Hartree); the report gives a, b, mu and timings. */
int tb_density_stochastic(tb_ctx *ctx, const double *shift, int32_t n_probes, uint64_t seed,
                          int32_t dos_moments, int32_t dos_points, double *diagP, double *q, double *mu,
                          tb_report *rep);

/* Stochastic KPM density of states of H (runKPM's DOS, withSP2_deltaH.cpp:1579-1648):
 * n_random Gaussian vectors (counter-based splitmix64/Box-Muller with `seed`),
 * n_moments Jackson-damped moments, the DOS at npts Chebyshev nodes.  Writes
 * moments (n_moments), energies and dos (npts each). */
int tb_kpm_dos(tb_ctx *ctx, int32_t n_moments, int32_t n_random, uint64_t seed, int32_t npts,
               double *moments, double *energies, double *dos, tb_report *rep);

/* ------------------------------------------------------------------------ */
/* Batches: many structures of uneven size in one solve                      */
/* ------------------------------------------------------------------------ */
/* The reference solves one structure per run (main, withSP2_deltaH.cpp:
 * 1742-1849).  A batch solves `count` independent structures together: each
 * structure keeps its own Gershgorin scaling, chemical potential, Anderson
 * history and convergence test on the device, while every Chebyshev step of
 * all still-unconverged structures runs as one launch (FP32 recurrence, FP64
 * moments; the precision field is ignored): the pipelined step kernel over
 * a tile list of every structure's row groups and column chunks, or, with
 * fp32_kernel = TB_FP32_STAGED (or when a pipeline stage does not fit in
 * shared memory), the staged one.  M, kT, kernel, the SCC tolerance, mixer
 * and iteration cap come from p; n_electrons <= 0 takes sum(q0) per
 * structure. */
typedef struct tb_batch tb_batch;

int tb_batch_create(const tb_params *p, int32_t count, tb_batch **out);
int tb_batch_destroy(tb_batch *b);

/* Structure `index`: its Hamiltonian (the tb_set_hamiltonian input, orbitals
 * 4 per atom, contiguous), Gamma and neutral charges (the tb_set_scc input). */
int tb_batch_set(tb_batch *b, int32_t index, int32_t n, const int32_t *rowptr,
                 const int32_t *colidx, const double *vals, int32_t natoms,
                 const int32_t *g_rowptr, const int32_t *g_colidx, const double *g_vals,
                 const double *q0);

/* SCC solve of every structure.  q_init (may be NULL) and q are the
 * structures' atoms concatenated in index order; iters, e_band and mu have
 * `count` entries.  Returns TB_ERR_NOT_CONVERGED if any structure reached
 * scc_max_iter (all outputs still written). */
int tb_batch_scc_solve(tb_batch *b, const double *q_init, double *q, int32_t *iters,
                       double *e_band, double *mu, tb_report *rep);

const char *tb_batch_last_error(const tb_batch *b);

/* ------------------------------------------------------------------------ */
/* Learned SCC starting charges (no counterpart in the reference, which      */
/* starts every SCC loop from the neutral charges, withSP2_deltaH.cpp:1725)  */
/* ------------------------------------------------------------------------ */
#define TB_MLP_NFEAT 32
#define TB_MLP_NPARAM 6337 /* W1[64][32] b1[64] W2[64][64] b2[64] w3[64] b3 */

/* Per-atom radial features on the current device: for each atom, 16
 * Gaussians exp(-12.5 (r - mu_k)^2) (r in angstrom, mu_k = 0.8 + 0.28 k) times
 * the cosine cutoff (cos(pi r / 5) + 1)/2, summed over Si neighbours within
 * 5 A, then 16 over O neighbours; minimum image in an orthorhombic box
 * (edges in bohr, 0 = open).  feat is natoms x 32, row-major. */
int tb_mlp_features(int32_t natoms, const double *xyz, const int32_t *species, const double *box,
                    float *feat);

/* A 32 -> 64 -> 64 -> 1 SiLU network predicting each atom's net charge
 * q - q0 from its features; BF16 weights (rounded from FP32 masters), FP32
 * activations and accumulation, trained by minibatch Adam on the mean
 * squared error -- all on the GPU. */
typedef struct tb_mlp tb_mlp;
int tb_mlp_create(int32_t device, uint64_t seed, tb_mlp **out);
int tb_mlp_destroy(tb_mlp *m);
/* FP32 master parameters (TB_MLP_NPARAM) and the feature normalisation
 * (mean[32], 1/std[32]); either pointer may be NULL. */
int tb_mlp_get(const tb_mlp *m, float *params, float *norm);
int tb_mlp_set(tb_mlp *m, const float *params, const float *norm);
/* Train for `epochs` over n samples (the normalisation is fixed from the
 * first training set unless set before); loss_per_epoch (may be NULL). */
int tb_mlp_train(tb_mlp *m, int32_t n, const float *feat, const float *target, int32_t epochs,
                 int32_t batch, float lr, uint64_t seed, float *loss_per_epoch);
/* Predicted q - q0 for n atoms, on the tensor cores (tcgen05: BF16 weights
 * and layer inputs, FP32 accumulation in tensor memory). */
int tb_mlp_predict(tb_mlp *m, int32_t n, const float *feat, float *out);
/* The same network on the CUDA cores with FP32 layer inputs (the training
 * kernels' forward pass). */
int tb_mlp_predict_fp32(tb_mlp *m, int32_t n, const float *feat, float *out);
/* Gradient of the mean squared error w.r.t. the (BF16-rounded) parameters. */
int tb_mlp_grad(tb_mlp *m, int32_t n, const float *feat, const float *target, float *grad,
                float *loss);

/* Message of the last failure on ctx (never NULL). */
const char *tb_last_error(const tb_ctx *ctx);
const char *tb_status_string(int status);
int tb_abi_version(void);

/* ------------------------------------------------------------------------ */
/* Allocation-free variant                                                   */
/* ------------------------------------------------------------------------ */
/* No counterpart in the reference: an entry point for callers that cannot
 * allocate device memory -- codes whose device memory belongs to their own
 * pool or allocator, or that run under a fixed memory budget.  It computes
 * the exact-trace moments mu_k = tr T_k(X), k = 0..M (the `moments` output
 * of tb_density) of X = (H - b I)/a for a CSR matrix H (n x n, any pattern,
 * FP64) that is already in device memory, and allocates nothing: the
 * recurrence's scratch is a static device array of 2 x TB_NOALLOC_MAX_N x 64
 * doubles (8 MiB) that every GPU loading this library holds until the
 * process exits.  d_rowptr (n+1), d_colidx and d_vals (nnz) and d_moments
 * (M+1) are device pointers owned by the caller; d_moments is cleared and
 * overwritten.  `stream` is a cudaStream_t (NULL: the legacy default stream);
 * the call ends with a cudaStreamSynchronize of `stream`, so it returns after
 * the stream has finished the work.
 *   - The first call on a device looks up the scratch array's device address
 *     (cudaGetSymbolAddress) with that device current, and looks it up again
 *     when the device's context has changed (after a cudaDeviceReset); make
 *     that first call before any stream capture.
 *   - A CUDA error already pending on entry returns TB_ERR_CUDA before any
 *     work is queued and is left pending for the caller.
 *   - Every call shares the one scratch array: calls that overlap on the GPU
 *     (from several host threads or streams) race and give wrong results.
 *   - n > TB_NOALLOC_MAX_N returns TB_ERR_UNSUPPORTED without touching the
 *     GPU; bad arguments return TB_ERR_INVALID_ARG. */
#define TB_NOALLOC_MAX_N 8192
int tb_moments_noalloc(int32_t n, const int32_t *d_rowptr, const int32_t *d_colidx,
                       const double *d_vals, double a, double b, int32_t M, double *d_moments,
                       void *stream);

/* ------------------------------------------------------------------------ */
/* Model builder: upstream of the boundary.  Builds what the reference's     */
/* arrangeCoordinates/constructH/initializeForSCF produce, for synthetic     */
/* inputs: the reference's alpha-quartz cell, or beta-cristobalite.          */
/* ------------------------------------------------------------------------ */
typedef struct tb_model tb_model;

/* alpha-quartz L x M x N exactly as the reference builds it (x/y periodic,
 * 0.1 < d^2 < 16 bohr^2, Gamma diagonal -1): withSP2_deltaH.cpp:372-740, 854-1066. */
int tb_model_quartz(int32_t L, int32_t M, int32_t N, tb_model **out);

/* beta-cristobalite nx x ny x nz conventional cells (24 atoms each), edge
 * a_ang, Gaussian displacements sigma_ang per Cartesian component from a
 * counter-based splitmix64/Box-Muller stream with `seed`, 3-D periodic,
 * neighbours within rcut_bohr, reference block model, Gamma diagonal
 * gamma_diag (+1: Hubbard U = 1 Ha with the physical sign). */
int tb_model_cristobalite(int32_t nx, int32_t ny, int32_t nz, double a_ang, double sigma_ang,
                          uint64_t seed, double rcut_bohr, double gamma_diag, tb_model **out);

int tb_model_sizes(const tb_model *m, int32_t *natoms, int32_t *n, int64_t *nnz,
                   int64_t *g_nnz);

/* Copy the model out (any pointer may be NULL): H CSR (n+1, nnz, nnz),
 * orb2atom (n), Gamma CSR (natoms+1, g_nnz, g_nnz), q0 (natoms),
 * xyz (3*natoms, bohr), species (natoms, atomic numbers). */
int tb_model_export(const tb_model *m, int32_t *rowptr, int32_t *colidx, double *vals,
                    int32_t *orb2atom, int32_t *g_rowptr, int32_t *g_colidx, double *g_vals,
                    double *q0, double *xyz, int32_t *species);
int tb_model_destroy(tb_model *m);

#ifdef __cplusplus
}
#endif
#endif

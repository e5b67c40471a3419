/*
 * tb_oracle.h -- CPU FP64 restatement of the largeTB density-matrix hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path in
 * largetb_gb300/: only tests/, __graft_entry__.smoke() and the cpu_baseline leg
 * of bench.py may load it.  The product never links, loads or falls back to it.
 *
 * Every routine restates a function of the reference programs
 * (withSP2_deltaH.cpp / withSP2.cpp of pghale/largeTB) in plain C; the citation
 * is on each declaration.  The reference itself needs PETSc and MPI, which are
 * external libraries, so it is not built here.
 *
 * What pins this restatement (checked by tests/test_oracle_golden.py):
 *   - the sp3 block model, neighbour rules and quartz geometry against the
 *     reference's own matrix dumps Amat.m (1x1x1 quartz) and H.m (4x4x4);
 *   - the Gamma builder against GAMMA_AB.m, the orbital->atom map against
 *     orbit2Atom.m;
 *   - the Coulomb shift against the netCharge.m -> GammaQ_vector.m -> deltaH.m
 *     triple of one reference run;
 *   - the closed-form Jackson damping against column 1 of gnsfile.txt;
 *   - statistically, the Chebyshev moment recurrence: the exact traces
 *     tr T_k((H - b)/a) of the reference's Htotal_scc.m (symmetrised as
 *     runKPM does) at the reference's own a, b match the moments behind its
 *     20-vector DOS dosfile.txt to sampling noise (|z| < 2 over 400 moments;
 *     a different matrix scores mean z^2 ~ 2700).
 * What no reference output pins exactly (every reference run seeds its random
 * vectors from std::random_device): the exact-trace moments beyond that
 * statistical agreement, mu, diagP, charges, the SCC loop and SP2 results.
 * Those are checked against dense eigendecomposition (numpy) and the kT -> 0
 * limit of the reference's step coefficients.
 *
 * Units: bohr, Hartree, electrons.  Orbital order per atom: s, px, py, pz.
 */
#ifndef TB_ORACLE_H
#define TB_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    ORC_OK = 0,
    ORC_ERR_ARG = 1,
    ORC_ERR_TOO_MANY_NEIGHBOURS = 2, /* ModifyNList throws past maxN_A, withSP2_deltaH.cpp:355-360 */
    ORC_ERR_DUP_NEIGHBOUR = 3,       /* two images of one atom inside the cutoff */
    ORC_ERR_BAD_PAIR = 4,            /* unknown species or r < 0.01 between distinct atoms */
    ORC_ERR_BISECTION = 5,           /* N_e not bracketed */
    ORC_ERR_NOT_CONVERGED = 6,
    ORC_ERR_CAPACITY = 7
};

/* Atomic numbers used by the reference block model (withSP2_deltaH.cpp:217,254,287). */
#define ORC_SI 14
#define ORC_O 8

/* Hexagonal alpha-quartz supercell, 9 atoms per cell, positions in bohr.
 * Restates initializeCoordinates, withSP2_deltaH.cpp:504-667. */
int orc_quartz_positions(int L, int M, int N, double *xyz, int32_t *species);

/* Supercell lattice vectors (rows) of the quartz cell: L*R1, M*R2, N*R3,
 * withSP2_deltaH.cpp:378-388. */
void orc_quartz_cell(int L, int M, int N, double cell[9]);

/* Ideal Fd-3m beta-cristobalite, conventional cubic cell with 8 Si on diamond
 * sites and 16 O at the Si-Si bond midpoints; atoms ordered cell by cell
 * (x outer, z inner, as the reference's i/j/k loops) and within a cell Si
 * first, then O.  Each Cartesian component is displaced by N(0, sigma^2)
 * drawn from splitmix64 + Box-Muller with the given seed.  Lengths in
 * angstrom on input, bohr on output (1.88973 bohr/A, withSP2_deltaH.cpp:377). */
int orc_cristobalite_positions(int nx, int ny, int nz, double a_ang, double sigma_ang,
                               uint64_t seed, double *xyz, int32_t *species);
void orc_cristobalite_cell(int nx, int ny, int nz, double a_ang, double cell[9]);

/* Neighbour list by brute force over periodic images -1..1 along each
 * periodic axis; pairs with rmin2 < d^2 < rcut2 (reference: 0.1 < d^2 < 16,
 * withSP2_deltaH.cpp:392,422).  Restates getHaloAtoms + ModifyNList,
 * withSP2_deltaH.cpp:355-501.  nbvec holds r_j(image) - r_i. */
int orc_neighbours(int natoms, const double *xyz, const double cell[9], const int periodic[3],
                   double rcut2, double rmin2, int maxnb, int32_t *nnb, int32_t *nbidx,
                   double *nbvec);

/* One 4x4 sp3 block.  Restates get4by4HmatrixElements, withSP2_deltaH.cpp:211-349. */
int orc_hblock(int zi, int zj, double x, double y, double z, double out[16]);

/* Orbital Hamiltonian in CSR (4 orbitals per atom, contiguous; rows sorted by
 * column; explicit zeros of each stored 4x4 block kept, as MatSetValues
 * stores them).  Restates constructH, withSP2_deltaH.cpp:969-1066.
 * rowptr has 4*natoms+1 entries, col/val capacity 16*(natoms+sum nnb). */
int orc_build_h(int natoms, const int32_t *species, const int32_t *nnb, const int32_t *nbidx,
                const double *nbvec, int maxnb, int32_t *rowptr, int32_t *col, double *val);

/* Gamma (natoms x natoms): Gamma_aa = diag_value (reference: -Us with Us=1),
 * Gamma_ab = 1/r_ab for neighbours.  Restates initializeForSCF,
 * withSP2_deltaH.cpp:876-899. */
int orc_build_gamma(int natoms, const int32_t *nnb, const int32_t *nbidx, const double *nbvec,
                    int maxnb, double diag_value, int32_t *rowptr, int32_t *col, double *val);

/* Gershgorin bounds min/max_i (h_ii -/+ sum_{j!=i} |h_ij|), with an optional
 * per-row diagonal shift (the SCC shift; NULL for none).  Restates
 * GershGorinParallel, withSP2_deltaH.cpp:144-209. */
void orc_gershgorin(int n, const int32_t *rowptr, const int32_t *col, const double *val,
                    const double *diag_shift, double *lmin, double *lmax);

/* Closed-form Jackson damping for M terms (n = 0..M-1, N = M in the formula).
 * Restates the gns[] loop of runKPM, withSP2_deltaH.cpp:1593-1595. */
void orc_jackson(int M, double *g);

/* The damping getKPE actually uses: autocorrelation of the normalised
 * U_i(cos(pi/(M+2))) sequence with the reference's i < M-m-1 bound.
 * Restates withSP2_deltaH.cpp:1104-1132. */
void orc_kernel_autocorr(int M, double *g);

/* Chebyshev coefficients of the zero-temperature step theta(mu - x),
 * c_0 = 1 - acos(mu)/pi, c_m = -2 sin(m acos mu)/(m pi).
 * Restates mu_mvals of getKPE, withSP2_deltaH.cpp:1100-1103,1136. */
void orc_step_coeffs(int M, double mu_x, double *c);

/* Chebyshev coefficients of the Fermi function f(x) = 1/(1+exp(beta_x (x-mu_x)))
 * on [-1,1] by nq-point Chebyshev-Gauss quadrature:
 * c_0 = (1/nq) sum_k f(x_k), c_n = (2/nq) sum_k f(x_k) cos(n theta_k),
 * theta_k = pi (k+1/2)/nq.  Reduces to orc_step_coeffs as beta_x -> inf. */
void orc_fermi_coeffs(int M, double mu_x, double beta_x, int nq, double *c);

/* Quadrature size rule shared by the oracle and the CUDA path. */
int orc_quadrature_nodes(int M, double beta_x);

/* Exact-trace moments: d[k*n + i] = [T_k(X)]_ii for k = 0..nmom-1, with
 * X = (H + diag(shift) - b I)/a, from the plain recurrence
 * T_{k+1} = 2 X T_k - T_{k-1} applied to column blocks of the identity.
 * Restates the vector recurrence of getKPE (withSP2_deltaH.cpp:1134-1168) with
 * the unit-vector trace of computeDiagonalElements (withSP2_deltaH.cpp:1361-1379). */
int orc_exact_moments(int n, const int32_t *rowptr, const int32_t *col, const double *val,
                      const double *diag_shift, double a, double b, int nmom, double *d,
                      int nthreads);

/* Same, for identity columns c_begin..c_end-1 only (entries of d outside
 * that range are left untouched); used to time a bounded sample. */
int orc_exact_moments_cols(int n, const int32_t *rowptr, const int32_t *col, const double *val,
                           const double *diag_shift, double a, double b, int nmom, int c_begin,
                           int c_end, double *d, int nthreads);

/* Electron count N(mu_x) = 2 sum_{n<M} c_n(mu_x) g_n mu_n, evaluated through the
 * damped DOS at the quadrature nodes (the same finite sums reordered);
 * beta_x <= 0 selects the step coefficients. */
double orc_electron_count(int M, const double *g, const double *mom, double mu_x,
                          double beta_x, int nq);

/* Bisection for mu_x in [-1,1] with N(mu_x) = n_elec.  Replaces the
 * integrated-DOS chemical potential of runKPM (withSP2_deltaH.cpp:1663-1712). */
int orc_bisect_mu(int M, const double *g, const double *mom, double n_elec, double beta_x,
                  int nq, double tol_n, int max_iter, double *mu_x, int *iters);

typedef struct {
    int32_t M;           /* expansion terms n = 0..M-1 (getKPE's M, withSP2_deltaH.cpp:1094);
                            moments 0..M are computed, the last one feeds the band energy */
    int32_t kernel;      /* 0 closed-form Jackson, 1 getKPE autocorrelation, 2 none */
    double kT;           /* Hartree; <= 0 selects the step function */
    double n_elec;       /* electrons, both spins */
    double pad;          /* relative widening of the Gershgorin interval */
    double tol_n;        /* bisection tolerance on the electron count */
    int32_t nthreads;
} orc_kpe_params;

typedef struct {
    double lmin, lmax, a, b; /* Gershgorin bounds and the scaling X = (H-b)/a */
    double mu_x, mu;         /* chemical potential, scaled and in Hartree */
    double e_band;           /* 2 tr(P H) */
    double n_elec_found;
    int32_t bisect_iters;
} orc_kpe_result;

/* One density evaluation: Gershgorin, exact-trace moments, mu bisection,
 * per-spin diagP and per-atom electron counts q_a = 2 sum_{i in a} P_ii.
 * Stands in for runKPM + computeDensityMatrix, withSP2_deltaH.cpp:1401-1411,1528-1723.
 * orb2atom maps orbital -> atom.  moments (length M+1) and d ((M+1)*n) optional. */
int orc_density(int n, const int32_t *rowptr, const int32_t *col, const double *val,
                const double *diag_shift, const int32_t *orb2atom, int natoms,
                const orc_kpe_params *p, double *diagP, double *q, double *moments, double *d,
                orc_kpe_result *res);

/* Gamma * dq (natoms).  Restates MatMult(Gamma_ab, netCharges, gammaq),
 * withSP2_deltaH.cpp:1424-1429. */
void orc_gamma_mult(int natoms, const int32_t *rowptr, const int32_t *col, const double *val,
                    const double *dq, double *out);

typedef struct {
    double tol;        /* convergence: max_a |q_out - q_in| < tol (electrons) */
    int32_t max_iter;
    double beta;       /* Anderson mixing parameter */
    int32_t history;   /* Anderson history depth (0 = linear mixing) */
} orc_scc_params;

/* Anderson mixing step (shared restatement for oracle and CUDA path):
 * given q_in, r = q_out - q_in and a history of previous (q_in, r), return the
 * next q_in.  hist_q / hist_r are [history][natoms] ring buffers managed by the
 * caller through *hcount and *hhead. */
int orc_anderson(int natoms, const double *q_in, const double *r, double beta, int history,
                 double *hist_q, double *hist_r, int *hcount, int *hhead, double *q_next);

/* Full SCC loop: H = H0 + diag(Gamma (q_in - q0)) per atom, density, Anderson
 * mixing, until max|q_out - q_in| < tol.  The reference's loop
 * (withSP2_deltaH.cpp:1820-1840) never adds delta H (mixRatio = 0, line 56);
 * this is the working loop it sketches.  q_init NULL starts from q0. */
int orc_scc(int n, const int32_t *rowptr, const int32_t *col, const double *val,
            const int32_t *orb2atom, int natoms, const int32_t *g_rowptr, const int32_t *g_col,
            const double *g_val, const double *q0, const double *q_init,
            const orc_kpe_params *p, const orc_scc_params *s, double *q_out, double *diagP,
            double *dq_hist, int *iters, orc_kpe_result *res);

typedef struct {
    double n_elec;
    double drop_tol;   /* blocks with Frobenius norm below this are dropped */
    int32_t max_iter;
    double idem_tol;   /* stop when ||X^2-X||_F < idem_tol */
    double trace_tol;  /* the reference's |2 tr X - N_e| < trace_tol test, withSP2.cpp:1027 */
    int32_t nthreads;
} orc_sp2_params;

typedef struct {
    int32_t iters;
    double idem_err;       /* ||X^2 - X||_F of the returned X */
    double trace;          /* tr X (per spin) */
    double e_band;         /* 2 tr(X H) */
    int64_t nnzb;          /* stored blocks of the returned X */
    double lmin, lmax;
} orc_sp2_result;

/* SP2 purification on 4x4 blocks with thresholding, in FP64.
 * X0 = (lmax I - H)/(lmax - lmin) from Gershgorin; per iteration X <- X^2 if
 * 2 tr X > N_e else 2X - X^2 (branch rule of computeAlphas,
 * withSP2.cpp:1027-1030; recursion getSP2, withSP2.cpp:956-984).
 * branches (length max_iter, may be NULL) receives -1 for X^2, +1 for 2X-X^2;
 * idem_hist receives ||X^2-X||_F before each step.  Stops when the error is
 * below idem_tol, when (after the oscillating start, errors < 0.1) it fails
 * to fall over two steps, or at max_iter; returns the last X whose error
 * was measured. */
int orc_sp2(int n, const int32_t *rowptr, const int32_t *col, const double *val,
            const int32_t *orb2atom, int natoms, const orc_sp2_params *p, double *diagP,
            double *q, int32_t *branches, double *idem_hist, double *trace_hist,
            orc_sp2_result *res);

/* Stochastic KPM density of states, restating runKPM, withSP2_deltaH.cpp:1579-1648:
 * moments mu_n = sum_r r^T T_n(X) r over n_random Gaussian vectors (seeded
 * splitmix64/Box-Muller instead of std::random_device), closed-form Jackson
 * damping, DOS on npts Chebyshev nodes x_k = cos(pi (k+1/2)/npts), energies
 * E_k = a x_k + b.  mom has nmom entries, energies/dos npts entries. */
int orc_kpm_dos(int n, const int32_t *rowptr, const int32_t *col, const double *val, double a,
                double b, int nmom, int n_random, uint64_t seed, int npts, double *mom,
                double *energies, double *dos);

/* Chemical potential and refined spectral interval from a DOS on the npts
 * Chebyshev nodes x_k = cos(pi (k+1/2)/npts) (energies E_k = a0 x_k + b0):
 * restates runKPM, withSP2_deltaH.cpp:1663-1703.  The trapezoid area from
 * the bottom of the spectrum reaches N_e/(2n) of the total at node mu_index,
 * mu = E[mu_index]; the interval [E_min, E_max] is where DOS/n >= 0.001 first
 * holds from either end (-10, 10 when it never does); a = (E_max - E_min)/2,
 * b = (E_max + E_min)/2. */
void orc_dos_mu(int npts, const double *energies, const double *dos, double n_elec, int n,
                double *mu, int *mu_index, double *a, double *b);

/* Stochastic-trace density, the reference's default path: runKPM's DOS from
 * n_random Gaussian probes (seed) with dos_moments Jackson-damped moments on
 * dos_points nodes, mu and the refined interval from it (orc_dos_mu), then
 * computeDiagonalElements' ratio estimator (withSP2_deltaH.cpp:1296-1399)
 *   diagP_i = sum_r x_i^r (P x^r)_i / sum_r (x_i^r)^2,
 *   P x = sum_{k<M} c_k g_k T_k(X) x  (getKPE, withSP2_deltaH.cpp:1134-1168)
 * on X = (H - b)/a with n_random fresh probes (stream seed + 1), c_k the
 * Fermi (kT > 0) or step (kT <= 0) coefficients at mu_x = (mu - b)/a and g_k
 * p->kernel's damping.  q_a = 2 sum_{i in a} diagP_i.  res receives a, b,
 * mu, mu_x and the Gershgorin bounds. */
int orc_density_stochastic(int n, const int32_t *rowptr, const int32_t *col, const double *val,
                           const int32_t *orb2atom, int natoms, const orc_kpe_params *p,
                           int n_random, uint64_t seed, int dos_moments, int dos_points,
                           double *diagP, double *q, orc_kpe_result *res);

/* Counter-based N(0,1) deviate: Box-Muller (cosine branch) on outputs 2*index
 * and 2*index+1 of the splitmix64 stream seeded with `seed`.  The CUDA path
 * and the product's model builder use the same definition. */
double orc_gauss(uint64_t seed, uint64_t index);

#ifdef __cplusplus
}
#endif
#endif

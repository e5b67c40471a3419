/*
 * tb_oracle.c -- CPU FP64 restatement of the largeTB density-matrix hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see tb_oracle.h): the checker for the CUDA path,
 * never part of the product.  Plain C99 + optional OpenMP, built with
 * -ffp-contract=off so that x86-64 and aarch64 hosts round identically.
 */
#include "tb_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* Constants as the reference writes them (withSP2_deltaH.cpp:28,377). */
static const double ORC_PI = 3.141592653589793238463;
static const double BOHR_PER_ANG = 1.88973;

/* ------------------------------------------------------------------------- */
/* Slater-Koster-like polynomial tables, 20 x {cp2, cp3, cp5, cp6}:           */
/* withSP2_deltaH.cpp:75-142 (Si_Si_e, O_O_e, Si_O_e).  These are the         */
/* reference's model parameters; the model is defined by them, so they are   */
/* restated value for value.                                                 */
/* ------------------------------------------------------------------------- */
static const double T_SISI[20][4] = {
    {17.865, -5.7398, 17.262, -13.794},   {87.114, 5.8664, 39.685, -7.1328},
    {-722.33, -52.111, -283.25, 27.816},  {66.059, -3.2651, 34.498, -27.631},
    {-613.94, -6.6631, -41.298, 12.075},  {-727.27, 1.3757, -112.62, 5.9498},
    {246.1, -84.273, 241.71, -164.58},    {-1564.3, 4.1541, -179.83, 22.449},
    {-589.53, -7.9678, 215.3, -36.682},   {-1020.8, 33.73, 7.8809, -87.911},
    {-812.85, -33.408, 13.727, 158.22},   {1189.7, 49.751, 54.842, -56.155},
    {-96.931, 8.9531, 102.98, -91.347},   {860.35, 1.2204, -44.669, 12.487},
    {3551.6, 9.5425, -32.771, 10.438},    {468.97, 1.6056, -128.73, -1.5888},
    {-317.44, 6.9669, 133.21, 82.532},    {517.74, 47.052, -56.922, 1.1376},
    {210.8, -18.241, -18.441, 80.163},    {-443.57, 36.135, 52.835, -13.413}};

static const double T_OO[20][4] = {
    {5.5526, -0.82118, 3.813, -1.2323},   {-31.886, 10.518, -41.071, 52.454},
    {233.96, -39.064, 272.9, -407.19},    {-60.015, 61.253, -128.95, -294.22},
    {213.73, -204.34, 410.72, 1263.6},    {49.054, 32.239, -78.906, -1060},
    {-73.081, 132.93, -81.269, 1956.2},   {33.537, -13.278, -137.34, -384.47},
    {78.858, 165.14, -273.61, -873.53},   {-167.41, 68.088, -277.49, 642.65},
    {75.731, 7.9468, -767.04, -615.24},   {-63.795, -44.453, -288.57, 988.73},
    {-78.765, 32.997, -76.092, -811.61},  {124.63, -144.7, -189.3, 554.51},
    {40.615, -149.44, 780.52, 379.23},    {82.116, -29.881, 410.4, -93.407},
    {-80.656, -54.736, 203.1, -131.08},   {-74.163, 16.814, 710.57, -213.88},
    {7.3441, 20.02, -100.83, 128.52},     {-93.219, 6.9584, 267.84, -242.74}};

static const double T_SIO[20][4] = {
    {13.778, -2.7061, 8.6477, -7.6931},   {9.0798, 19.494, -22.43, 52.885},
    {-15.173, -145.38, 262.06, -468.23},  {9.4007, -23.026, 223.86, -100.16},
    {40.783, 126.17, -785.64, 228.63},    {23.249, -34.501, 334.88, -253.56},
    {-17.829, -75.476, 156.18, -638.68},  {18.37, -22.003, 10.705, -312.46},
    {1.7289, 75.972, 572.55, -1010.6},    {-30.424, 17.518, -55.884, -478.46},
    {-31.663, -36.928, -349.49, -688.24}, {-82.425, -26.609, -390.25, -296.52},
    {35.07, 77.948, -143.41, 157.81},     {-27.066, -22.899, -390.79, 580.81},
    {-20.555, -140.91, -152.48, 401.59},  {49.585, -5.9967, 502.82, 768.76},
    {-8.7806, 109.97, -113.52, 980.42},   {37.13, -18.019, -148.42, 243.34},
    {-20.674, 15.652, 904.76, 317.15},    {16.513, 39.501, -630.1, 84.78}};

/* On-site energies (withSP2_deltaH.cpp:255-261 for Si, 288-294 for O). */
static const double ES_SI = -0.39572506, EP_SI = -0.15031380;
static const double ES_O = -0.87883246, EP_O = -0.33213167;

/* ------------------------------------------------------------------------- */
/* Random numbers                                                            */
/* ------------------------------------------------------------------------- */
static uint64_t sm64_at(uint64_t seed, uint64_t k)
{
    /* Output k (0-based) of the splitmix64 stream seeded with `seed`. */
    uint64_t z = seed + (k + 1u) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

double orc_gauss(uint64_t seed, uint64_t index)
{
    const double two53 = 1.0 / 9007199254740992.0;
    double u1 = ((double)(sm64_at(seed, 2u * index) >> 11) + 1.0) * two53; /* (0,1] */
    double u2 = (double)(sm64_at(seed, 2u * index + 1u) >> 11) * two53;    /* [0,1) */
    return sqrt(-2.0 * log(u1)) * cos(2.0 * ORC_PI * u2);
}

/* ------------------------------------------------------------------------- */
/* Geometry                                                                  */
/* ------------------------------------------------------------------------- */
static void quartz_vectors(double R1[3], double R2[3], double R3[3])
{
    const double a = 9.725, b = a, c = 10.7; /* bohr, withSP2_deltaH.cpp:378 */
    R1[0] = a;
    R1[1] = 0.0;
    R1[2] = 0.0;
    R2[0] = b * (-sin(ORC_PI / 6));
    R2[1] = b * cos(ORC_PI / 6);
    R2[2] = 0.0;
    R3[0] = 0.0;
    R3[1] = 0.0;
    R3[2] = c;
}

/* Fractional sites of the quartz cell and their species,
 * withSP2_deltaH.cpp:525-664 (3 Si then 6 O). */
static const double QZ_FRAC[9][3] = {
    {0.4697, 0.0000, 0.0000}, {0.0000, 0.4697, 0.6777}, {0.5303, 0.5303, 0.3333},
    {0.4133, 0.2672, 0.1188}, {0.2672, 0.4133, 0.5479}, {0.7328, 0.1461, 0.7855},
    {0.5867, 0.8539, 0.2145}, {0.8539, 0.5867, 0.4521}, {0.1461, 0.7328, 0.8812}};
static const int QZ_SPECIES[9] = {ORC_SI, ORC_SI, ORC_SI, ORC_O, ORC_O, ORC_O, ORC_O, ORC_O, ORC_O};

int orc_quartz_positions(int L, int M, int N, double *xyz, int32_t *species)
{
    if (L < 1 || M < 1 || N < 1 || !xyz || !species) return ORC_ERR_ARG;
    double R1[3], R2[3], R3[3];
    quartz_vectors(R1, R2, R3);
    int atom = 0;
    for (int i = 0; i < L; i++)
        for (int j = 0; j < M; j++)
            for (int k = 0; k < N; k++) {
                double x0 = i * R1[0] + j * R2[0] + k * R3[0];
                double y0 = i * R1[1] + j * R2[1] + k * R3[1];
                double z0 = i * R1[2] + j * R2[2] + k * R3[2];
                for (int s = 0; s < 9; s++) {
                    const double *f = QZ_FRAC[s];
                    double xi = f[0] * R1[0] + f[1] * R2[0] + f[2] * R3[0];
                    double yi = f[0] * R1[1] + f[1] * R2[1] + f[2] * R3[1];
                    double zi = f[0] * R1[2] + f[1] * R2[2] + f[2] * R3[2];
                    xyz[3 * atom + 0] = x0 + xi;
                    xyz[3 * atom + 1] = y0 + yi;
                    xyz[3 * atom + 2] = z0 + zi;
                    species[atom] = QZ_SPECIES[s];
                    atom++;
                }
            }
    return ORC_OK;
}

void orc_quartz_cell(int L, int M, int N, double cell[9])
{
    double R1[3], R2[3], R3[3];
    quartz_vectors(R1, R2, R3);
    for (int c = 0; c < 3; c++) {
        cell[0 + c] = L * R1[c];
        cell[3 + c] = M * R2[c];
        cell[6 + c] = N * R3[c];
    }
}

/* beta-cristobalite sites (fractions of the cubic cell edge): fcc Si, fcc Si
 * shifted by (1/4,1/4,1/4), then the four bond midpoints around each shifted
 * Si.  Public crystallography of the ideal Fd-3m structure. */
static void cristobalite_site(int s, double f[3], int *z)
{
    static const double fcc[4][3] = {{0, 0, 0}, {0, 0.5, 0.5}, {0.5, 0, 0.5}, {0.5, 0.5, 0}};
    static const double mid[4][3] = {
        {0.125, 0.125, 0.125}, {0.375, 0.375, 0.125}, {0.375, 0.125, 0.375}, {0.125, 0.375, 0.375}};
    if (s < 4) {
        f[0] = fcc[s][0];
        f[1] = fcc[s][1];
        f[2] = fcc[s][2];
        *z = ORC_SI;
    } else if (s < 8) {
        f[0] = fcc[s - 4][0] + 0.25;
        f[1] = fcc[s - 4][1] + 0.25;
        f[2] = fcc[s - 4][2] + 0.25;
        *z = ORC_SI;
    } else {
        int t = s - 8, c = t / 4, m = t % 4;
        f[0] = fcc[c][0] + mid[m][0];
        f[1] = fcc[c][1] + mid[m][1];
        f[2] = fcc[c][2] + mid[m][2];
        *z = ORC_O;
    }
}

int orc_cristobalite_positions(int nx, int ny, int nz, double a_ang, double sigma_ang,
                               uint64_t seed, double *xyz, int32_t *species)
{
    if (nx < 1 || ny < 1 || nz < 1 || !(a_ang > 0) || !(sigma_ang >= 0) || !xyz || !species)
        return ORC_ERR_ARG;
    const double a = a_ang * BOHR_PER_ANG, sigma = sigma_ang * BOHR_PER_ANG;
    int atom = 0;
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++)
                for (int s = 0; s < 24; s++) {
                    double f[3];
                    int z;
                    cristobalite_site(s, f, &z);
                    xyz[3 * atom + 0] = (i + f[0]) * a + sigma * orc_gauss(seed, 3u * atom + 0u);
                    xyz[3 * atom + 1] = (j + f[1]) * a + sigma * orc_gauss(seed, 3u * atom + 1u);
                    xyz[3 * atom + 2] = (k + f[2]) * a + sigma * orc_gauss(seed, 3u * atom + 2u);
                    species[atom] = z;
                    atom++;
                }
    return ORC_OK;
}

void orc_cristobalite_cell(int nx, int ny, int nz, double a_ang, double cell[9])
{
    const double a = a_ang * BOHR_PER_ANG;
    memset(cell, 0, 9 * sizeof(double));
    cell[0] = nx * a;
    cell[4] = ny * a;
    cell[8] = nz * a;
}

int orc_neighbours(int natoms, const double *xyz, const double cell[9], const int periodic[3],
                   double rcut2, double rmin2, int maxnb, int32_t *nnb, int32_t *nbidx,
                   double *nbvec)
{
    if (natoms < 1 || maxnb < 1) return ORC_ERR_ARG;
    const double rcut = sqrt(rcut2);
    int lo[3], hi[3];
    for (int d = 0; d < 3; d++) {
        lo[d] = periodic[d] ? -1 : 0;
        hi[d] = periodic[d] ? 1 : 0;
    }
    int err = ORC_OK;
    for (int i = 0; i < natoms; i++) nnb[i] = 0;
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < natoms; i++) {
        const double xi = xyz[3 * i], yi = xyz[3 * i + 1], zi = xyz[3 * i + 2];
        int cnt = 0;
        for (int l = lo[0]; l <= hi[0]; l++)
            for (int m = lo[1]; m <= hi[1]; m++)
                for (int q = lo[2]; q <= hi[2]; q++) {
                    const double sx = l * cell[0] + m * cell[3] + q * cell[6];
                    const double sy = l * cell[1] + m * cell[4] + q * cell[7];
                    const double sz = l * cell[2] + m * cell[5] + q * cell[8];
                    for (int j = 0; j < natoms; j++) {
                        double dx = (xyz[3 * j] + sx) - xi;
                        if (dx > rcut || dx < -rcut) continue;
                        double dy = (xyz[3 * j + 1] + sy) - yi;
                        if (dy > rcut || dy < -rcut) continue;
                        double dz = (xyz[3 * j + 2] + sz) - zi;
                        double d2 = dx * dx + dy * dy + dz * dz;
                        if (d2 < rcut2 && d2 > rmin2) {
                            for (int t = 0; t < cnt; t++)
                                if (nbidx[(size_t)i * maxnb + t] == j) {
#pragma omp critical
                                    err = ORC_ERR_DUP_NEIGHBOUR;
                                }
                            if (cnt >= maxnb) {
#pragma omp critical
                                err = ORC_ERR_TOO_MANY_NEIGHBOURS;
                                continue;
                            }
                            size_t o = (size_t)i * maxnb + cnt;
                            nbidx[o] = j;
                            nbvec[3 * o + 0] = dx;
                            nbvec[3 * o + 1] = dy;
                            nbvec[3 * o + 2] = dz;
                            cnt++;
                        }
                    }
                }
        nnb[i] = cnt;
    }
    return err;
}

/* ------------------------------------------------------------------------- */
/* sp3 block model, withSP2_deltaH.cpp:211-349                               */
/* ------------------------------------------------------------------------- */
int orc_hblock(int zi, int zj, double x, double y, double z, double out[16])
{
    double H[4][4] = {{0}};
    const double rSq = x * x + y * y + z * z;
    const double r = sqrt(rSq);
    const double(*tab)[4] = NULL;
    if ((zi == ORC_SI && zj == ORC_O) || (zi == ORC_O && zj == ORC_SI)) {
        if (r < 0.01) return ORC_ERR_BAD_PAIR;
        tab = T_SIO;
    } else if (zi == ORC_SI && zj == ORC_SI) {
        if (r < 0.01) {
            H[0][0] = ES_SI;
            H[1][1] = H[2][2] = H[3][3] = EP_SI;
        } else
            tab = T_SISI;
    } else if (zi == ORC_O && zj == ORC_O) {
        if (r < 0.01) {
            H[0][0] = ES_O;
            H[1][1] = H[2][2] = H[3][3] = EP_O;
        } else
            tab = T_OO;
    } else
        return ORC_ERR_BAD_PAIR;

    if (tab) {
        const double l[3] = {x, y, z};
        for (int p = 1; p <= 20; p++) {
            const double cp2 = tab[p - 1][0], cp3 = tab[p - 1][1];
            const double cp5 = tab[p - 1][2], cp6 = tab[p - 1][3];
            const double C = cos(p * acos(r / 10)); /* T_p(r/10) */
            const double E = exp(-p * r);
            H[0][0] = H[0][0] + cp6 * C * E;
            for (int k = 0; k < 3; k++) {
                H[0][k + 1] = H[0][k + 1] + (cp5 * l[k] * C * E) / r;
                H[k + 1][0] = H[k + 1][0] + -(cp5 * l[k] * C * E) / r;
            }
            for (int k = 0; k < 3; k++)
                for (int m = 0; m < 3; m++) {
                    if (k == m)
                        H[k + 1][k + 1] = H[k + 1][k + 1] + (cp2 * (l[k] * l[k]) * C * E) / rSq -
                                          cp3 * C * E * ((l[k] * l[k]) / rSq - 1);
                    else
                        H[k + 1][m + 1] = H[k + 1][m + 1] + (cp2 * l[k] * l[m] * C * E) / rSq -
                                          (cp3 * l[k] * l[m] * C * E) / rSq;
                }
        }
    }
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) out[4 * i + j] = H[i][j];
    return ORC_OK;
}

/* Sorted column-block list of atom i: itself plus its neighbours. */
static int row_blocks(int i, const int32_t *nnb, const int32_t *nbidx, int maxnb, int32_t *cols,
                      int32_t *slot)
{
    int cnt = nnb[i] + 1;
    cols[0] = i;
    slot[0] = -1;
    for (int t = 0; t < nnb[i]; t++) {
        cols[t + 1] = nbidx[(size_t)i * maxnb + t];
        slot[t + 1] = t;
    }
    for (int a = 1; a < cnt; a++) { /* insertion sort, lists are short */
        int32_t c = cols[a], s = slot[a];
        int b = a - 1;
        while (b >= 0 && cols[b] > c) {
            cols[b + 1] = cols[b];
            slot[b + 1] = slot[b];
            b--;
        }
        cols[b + 1] = c;
        slot[b + 1] = s;
    }
    return cnt;
}

int orc_build_h(int natoms, const int32_t *species, const int32_t *nnb, const int32_t *nbidx,
                const double *nbvec, int maxnb, int32_t *rowptr, int32_t *col, double *val)
{
    int32_t *cols = (int32_t *)malloc(sizeof(int32_t) * (maxnb + 1));
    int32_t *slot = (int32_t *)malloc(sizeof(int32_t) * (maxnb + 1));
    double *blk = (double *)malloc(sizeof(double) * 16 * (maxnb + 1));
    int err = ORC_OK;
    int64_t nz = 0;
    rowptr[0] = 0;
    for (int i = 0; i < natoms && err == ORC_OK; i++) {
        int cnt = row_blocks(i, nnb, nbidx, maxnb, cols, slot);
        for (int b = 0; b < cnt; b++) {
            if (slot[b] < 0)
                err = orc_hblock(species[i], species[i], 0.0, 0.0, 0.0, blk + 16 * b);
            else {
                const double *v = nbvec + 3 * ((size_t)i * maxnb + slot[b]);
                err = orc_hblock(species[i], species[cols[b]], v[0], v[1], v[2], blk + 16 * b);
            }
            if (err) break;
        }
        for (int r = 0; r < 4; r++) {
            for (int b = 0; b < cnt; b++)
                for (int c = 0; c < 4; c++) {
                    col[nz] = 4 * cols[b] + c;
                    val[nz] = blk[16 * b + 4 * r + c];
                    nz++;
                }
            rowptr[4 * i + r + 1] = (int32_t)nz;
        }
    }
    free(cols);
    free(slot);
    free(blk);
    return err;
}

int orc_build_gamma(int natoms, const int32_t *nnb, const int32_t *nbidx, const double *nbvec,
                    int maxnb, double diag_value, int32_t *rowptr, int32_t *col, double *val)
{
    int32_t *cols = (int32_t *)malloc(sizeof(int32_t) * (maxnb + 1));
    int32_t *slot = (int32_t *)malloc(sizeof(int32_t) * (maxnb + 1));
    int64_t nz = 0;
    rowptr[0] = 0;
    for (int i = 0; i < natoms; i++) {
        int cnt = row_blocks(i, nnb, nbidx, maxnb, cols, slot);
        for (int b = 0; b < cnt; b++) {
            col[nz] = cols[b];
            if (slot[b] < 0)
                val[nz] = diag_value;
            else {
                const double *v = nbvec + 3 * ((size_t)i * maxnb + slot[b]);
                /* r = pow(dx^2+dy^2+dz^2, 0.5), withSP2_deltaH.cpp:896 */
                double r = pow(pow(v[0], 2) + pow(v[1], 2) + pow(v[2], 2), 0.5);
                val[nz] = 1 / r;
            }
            nz++;
        }
        rowptr[i + 1] = (int32_t)nz;
    }
    free(cols);
    free(slot);
    return ORC_OK;
}

void orc_gershgorin(int n, const int32_t *rowptr, const int32_t *col, const double *val,
                    const double *diag_shift, double *lmin, double *lmax)
{
    double mn = INFINITY, mx = -INFINITY;
    for (int i = 0; i < n; i++) {
        double dg = 0.0, off = 0.0;
        for (int k = rowptr[i]; k < rowptr[i + 1]; k++) {
            if (col[k] == i)
                dg = val[k];
            else
                off = off + fabs(val[k]);
        }
        if (diag_shift) dg += diag_shift[i];
        if (dg - off < mn) mn = dg - off;
        if (dg + off > mx) mx = dg + off;
    }
    *lmin = mn;
    *lmax = mx;
}

/* ------------------------------------------------------------------------- */
/* Expansion coefficients and damping                                        */
/* ------------------------------------------------------------------------- */
void orc_jackson(int M, double *g)
{
    const double N = (double)M;
    const double cotv = cos(ORC_PI / (N + 1)) / sin(ORC_PI / (N + 1));
    for (int n = 0; n < M; n++)
        g[n] = ((N - n + 1) * cos(ORC_PI * (double)n / (N + 1)) +
                sin(ORC_PI * (double)n / (N + 1)) * cotv) /
               (N + 1);
}

void orc_kernel_autocorr(int M, double *g)
{
    double *U = (double *)malloc(sizeof(double) * M);
    const double alpha = ORC_PI / (M + 2);
    const double lam = cos(alpha);
    double nrm = 0.0;
    for (int m = 0; m < M; m++) {
        U[m] = sin((m + 1) * acos(lam)) / sin(acos(lam));
        nrm = nrm + U[m] * U[m];
    }
    nrm = sqrt(nrm);
    for (int m = 0; m < M; m++) U[m] = U[m] / nrm;
    for (int m = 0; m < M; m++) {
        double s = 0.0;
        for (int i = 0; i < (M - m - 1); i++) s = s + U[i] * U[m + i];
        g[m] = s;
    }
    free(U);
}

void orc_step_coeffs(int M, double mu_x, double *c)
{
    const double th = acos(mu_x);
    c[0] = 1 - th / ORC_PI;
    for (int m = 1; m < M; m++) c[m] = -2 * sin(m * th) / (m * ORC_PI);
}

static double fermi(double x, double mu_x, double beta_x)
{
    double t = beta_x * (x - mu_x);
    if (t > 0) {
        double e = exp(-t);
        return e / (1.0 + e);
    }
    return 1.0 / (1.0 + exp(t));
}

void orc_fermi_coeffs(int M, double mu_x, double beta_x, int nq, double *c)
{
    for (int n = 0; n < M; n++) c[n] = 0.0;
    for (int k = 0; k < nq; k++) {
        const double th = ORC_PI * (k + 0.5) / nq;
        const double f = fermi(cos(th), mu_x, beta_x);
        for (int n = 0; n < M; n++) c[n] += f * cos(n * th);
    }
    c[0] = c[0] / nq;
    for (int n = 1; n < M; n++) c[n] = 2.0 * c[n] / nq;
}

int orc_quadrature_nodes(int M, double beta_x)
{
    /* Nodes must resolve the Fermi width 1/beta_x (the trapezoid rule in theta
     * converges like exp(-nq * pi / beta_x)) and alias no retained cos(n theta). */
    double need = 4.0 * M;
    if (beta_x > 0 && 13.0 * beta_x > need) need = 13.0 * beta_x;
    if (need < 256) need = 256;
    if (need > (double)(1 << 22)) need = (double)(1 << 22); /* spectra this wide are rejected upstream */
    int nq = 256;
    while (nq < need) nq *= 2;
    return nq;
}

/* ------------------------------------------------------------------------- */
/* Exact-trace moments                                                       */
/* ------------------------------------------------------------------------- */
#define ORC_COLBLK 32

int orc_exact_moments(int n, const int32_t *rowptr, const int32_t *col, const double *val,
                      const double *diag_shift, double a, double b, int nmom, double *d,
                      int nthreads)
{
    return orc_exact_moments_cols(n, rowptr, col, val, diag_shift, a, b, nmom, 0, n, d, nthreads);
}

int orc_exact_moments_cols(int n, const int32_t *rowptr, const int32_t *col, const double *val,
                           const double *diag_shift, double a, double b, int nmom, int c_begin,
                           int c_end, double *d, int nthreads)
{
    if (n < 1 || nmom < 1 || !(a > 0) || c_begin < 0 || c_end > n || c_begin >= c_end)
        return ORC_ERR_ARG;
    const int B = ORC_COLBLK;
    const int nblk = (c_end - c_begin + B - 1) / B;
    const int64_t nnz = rowptr[n];
    /* X = (H + diag(shift) - b I) / a, folded into a scaled copy of the values
     * plus a diagonal term for rows whose diagonal entry is not stored. */
    double *xv = (double *)malloc(sizeof(double) * (nnz > 0 ? nnz : 1));
    double *xd = (double *)malloc(sizeof(double) * n);
    for (int i = 0; i < n; i++) {
        double extra = (diag_shift ? diag_shift[i] : 0.0) - b;
        int found = 0;
        for (int k = rowptr[i]; k < rowptr[i + 1]; k++) {
            if (col[k] == i) {
                xv[k] = (val[k] + extra) / a;
                found = 1;
            } else
                xv[k] = val[k] / a;
        }
        xd[i] = found ? 0.0 : extra / a;
    }
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel
    {
        double *V0 = (double *)malloc(sizeof(double) * (size_t)n * B);
        double *V1 = (double *)malloc(sizeof(double) * (size_t)n * B);
#pragma omp for schedule(dynamic, 1)
        for (int blk = 0; blk < nblk; blk++) {
            const int c0 = c_begin + blk * B;
            const int w = (c_end - c0) < B ? (c_end - c0) : B;
            memset(V0, 0, sizeof(double) * (size_t)n * B);
            for (int j = 0; j < w; j++) V0[(size_t)(c0 + j) * B + j] = 1.0;
            for (int j = 0; j < w; j++) d[(size_t)0 * n + c0 + j] = 1.0;
            if (nmom < 2) continue;
            /* V1 = X V0 */
            for (int i = 0; i < n; i++) {
                double acc[ORC_COLBLK];
                for (int j = 0; j < B; j++) acc[j] = xd[i] * V0[(size_t)i * B + j];
                for (int k = rowptr[i]; k < rowptr[i + 1]; k++) {
                    const double x = xv[k];
                    const double *src = V0 + (size_t)col[k] * B;
                    for (int j = 0; j < B; j++) acc[j] += x * src[j];
                }
                memcpy(V1 + (size_t)i * B, acc, sizeof(acc));
            }
            for (int j = 0; j < w; j++) d[(size_t)1 * n + c0 + j] = V1[(size_t)(c0 + j) * B + j];
            /* T_{k+1} = 2 X T_k - T_{k-1}, written over T_{k-1} */
            for (int kk = 2; kk < nmom; kk++) {
                for (int i = 0; i < n; i++) {
                    double acc[ORC_COLBLK];
                    for (int j = 0; j < B; j++) acc[j] = xd[i] * V1[(size_t)i * B + j];
                    for (int k = rowptr[i]; k < rowptr[i + 1]; k++) {
                        const double x = xv[k];
                        const double *src = V1 + (size_t)col[k] * B;
                        for (int j = 0; j < B; j++) acc[j] += x * src[j];
                    }
                    double *dst = V0 + (size_t)i * B;
                    for (int j = 0; j < B; j++) dst[j] = 2.0 * acc[j] - dst[j];
                }
                for (int j = 0; j < w; j++)
                    d[(size_t)kk * n + c0 + j] = V0[(size_t)(c0 + j) * B + j];
                double *t = V0;
                V0 = V1;
                V1 = t;
            }
        }
        free(V0);
        free(V1);
    }
    free(xv);
    free(xd);
    return ORC_OK;
}

/* ------------------------------------------------------------------------- */
/* Chemical potential                                                        */
/* ------------------------------------------------------------------------- */
/* Damped DOS at the quadrature nodes: rho_k = sum_n (2-delta_n0) g_n mu_n cos(n th_k). */
static void dos_at_nodes(int M, const double *g, const double *mom, int nq, double *xk,
                         double *rho)
{
    for (int k = 0; k < nq; k++) {
        const double th = ORC_PI * (k + 0.5) / nq;
        double s = g[0] * mom[0];
        for (int n = 1; n < M; n++) s += 2.0 * g[n] * mom[n] * cos(n * th);
        rho[k] = s;
        xk[k] = cos(th);
    }
}

static double count_from_nodes(int nq, const double *xk, const double *rho, double mu_x,
                               double beta_x)
{
    double s = 0.0;
    for (int k = 0; k < nq; k++) s += fermi(xk[k], mu_x, beta_x) * rho[k];
    return 2.0 * s / nq;
}

static double count_step(int M, const double *g, const double *mom, double mu_x, double *c)
{
    orc_step_coeffs(M, mu_x, c);
    double s = 0.0;
    for (int n = 0; n < M; n++) s += c[n] * g[n] * mom[n];
    return 2.0 * s;
}

double orc_electron_count(int M, const double *g, const double *mom, double mu_x,
                          double beta_x, int nq)
{
    double v;
    if (beta_x > 0) {
        double *xk = (double *)malloc(sizeof(double) * nq);
        double *rho = (double *)malloc(sizeof(double) * nq);
        dos_at_nodes(M, g, mom, nq, xk, rho);
        v = count_from_nodes(nq, xk, rho, mu_x, beta_x);
        free(xk);
        free(rho);
    } else {
        double *c = (double *)malloc(sizeof(double) * M);
        v = count_step(M, g, mom, mu_x, c);
        free(c);
    }
    return v;
}

int orc_bisect_mu(int M, const double *g, const double *mom, double n_elec, double beta_x,
                  int nq, double tol_n, int max_iter, double *mu_x, int *iters)
{
    double *xk = NULL, *rho = NULL, *c = NULL;
    if (beta_x > 0) {
        xk = (double *)malloc(sizeof(double) * nq);
        rho = (double *)malloc(sizeof(double) * nq);
        dos_at_nodes(M, g, mom, nq, xk, rho);
    } else
        c = (double *)malloc(sizeof(double) * M);
#define COUNT(m) (beta_x > 0 ? count_from_nodes(nq, xk, rho, (m), beta_x) : count_step(M, g, mom, (m), c))
    double lo = -1.0, hi = 1.0;
    int err = ORC_OK, it = 0;
    double nlo = COUNT(lo), nhi = COUNT(hi);
    double mid = 0.0;
    if (!(nlo <= n_elec && n_elec <= nhi)) {
        err = ORC_ERR_BISECTION;
    } else {
        for (it = 1; it <= max_iter; it++) {
            mid = 0.5 * (lo + hi);
            double nm = COUNT(mid);
            if (fabs(nm - n_elec) <= tol_n) break;
            if (nm < n_elec)
                lo = mid;
            else
                hi = mid;
        }
        if (it > max_iter) it = max_iter;
    }
#undef COUNT
    free(xk);
    free(rho);
    free(c);
    *mu_x = mid;
    if (iters) *iters = it;
    return err;
}

/* ------------------------------------------------------------------------- */
/* Density evaluation                                                        */
/* ------------------------------------------------------------------------- */
int orc_density(int n, const int32_t *rowptr, const int32_t *col, const double *val,
                const double *diag_shift, const int32_t *orb2atom, int natoms,
                const orc_kpe_params *p, double *diagP, double *q, double *moments, double *dout,
                orc_kpe_result *res)
{
    const int M = p->M;
    if (M < 2 || n < 1) return ORC_ERR_ARG;
    orc_kpe_result r;
    memset(&r, 0, sizeof(r));
    orc_gershgorin(n, rowptr, col, val, diag_shift, &r.lmin, &r.lmax);
    double half = 0.5 * (r.lmax - r.lmin);
    r.b = 0.5 * (r.lmax + r.lmin);
    r.a = half * (1.0 + p->pad);
    if (!(r.a > 0)) return ORC_ERR_ARG;

    double *d = dout ? dout : (double *)malloc(sizeof(double) * (size_t)(M + 1) * n);
    int err = orc_exact_moments(n, rowptr, col, val, diag_shift, r.a, r.b, M + 1, d, p->nthreads);
    if (err) {
        if (!dout) free(d);
        return err;
    }
    double *mom = (double *)malloc(sizeof(double) * (M + 1));
    for (int k = 0; k <= M; k++) {
        double s = 0.0;
        for (int i = 0; i < n; i++) s += d[(size_t)k * n + i];
        mom[k] = s;
    }
    double *g = (double *)malloc(sizeof(double) * M);
    if (p->kernel == 0)
        orc_jackson(M, g);
    else if (p->kernel == 1)
        orc_kernel_autocorr(M, g);
    else
        for (int k = 0; k < M; k++) g[k] = 1.0;
    g[0] = 1.0; /* the n = 0 term carries no damping factor (getKPE line 1136) */

    const double beta_x = p->kT > 0 ? r.a / p->kT : 0.0;
    const int nq = orc_quadrature_nodes(M, beta_x);
    int it = 0;
    err = orc_bisect_mu(M, g, mom, p->n_elec, beta_x, nq, p->tol_n, 200, &r.mu_x, &it);
    r.bisect_iters = it;
    r.mu = r.a * r.mu_x + r.b;
    double *c = (double *)malloc(sizeof(double) * M);
    if (beta_x > 0)
        orc_fermi_coeffs(M, r.mu_x, beta_x, nq, c);
    else
        orc_step_coeffs(M, r.mu_x, c);
    double *w = (double *)malloc(sizeof(double) * M);
    for (int k = 0; k < M; k++) w[k] = c[k] * g[k];

    /* P_ii = sum_k c_k g_k [T_k(X)]_ii ; q_a = 2 sum_{i in a} P_ii */
    if (q)
        for (int a = 0; a < natoms; a++) q[a] = 0.0;
    for (int i = 0; i < n; i++) {
        double s = 0.0;
        for (int k = 0; k < M; k++) s += w[k] * d[(size_t)k * n + i];
        if (diagP) diagP[i] = s;
        if (q) q[orb2atom[i]] += 2.0 * s;
    }
    double ne = 0.0, eb = 0.0;
    for (int k = 0; k < M; k++) {
        ne += w[k] * mom[k];
        const double tx = (k == 0) ? mom[1] : 0.5 * (mom[k + 1] + mom[k - 1]);
        eb += w[k] * (r.a * tx + r.b * mom[k]);
    }
    r.n_elec_found = 2.0 * ne;
    r.e_band = 2.0 * eb;
    if (moments)
        for (int k = 0; k <= M; k++) moments[k] = mom[k];
    if (res) *res = r;
    free(mom);
    free(g);
    free(c);
    free(w);
    if (!dout) free(d);
    return err;
}

void orc_gamma_mult(int natoms, const int32_t *rowptr, const int32_t *col, const double *val,
                    const double *dq, double *out)
{
    for (int a = 0; a < natoms; a++) {
        double s = 0.0;
        for (int k = rowptr[a]; k < rowptr[a + 1]; k++) s += val[k] * dq[col[k]];
        out[a] = s;
    }
}

/* ------------------------------------------------------------------------- */
/* SCC loop with Anderson mixing                                             */
/* ------------------------------------------------------------------------- */
static int solve_small(int m, double *A, double *rhs)
{
    /* Gaussian elimination with partial pivoting, in place (A row-major m x m). */
    for (int k = 0; k < m; k++) {
        int piv = k;
        for (int i = k + 1; i < m; i++)
            if (fabs(A[i * m + k]) > fabs(A[piv * m + k])) piv = i;
        if (!(fabs(A[piv * m + k]) > 1e-300)) return 1;
        if (piv != k) {
            for (int j = 0; j < m; j++) {
                double t = A[k * m + j];
                A[k * m + j] = A[piv * m + j];
                A[piv * m + j] = t;
            }
            double t = rhs[k];
            rhs[k] = rhs[piv];
            rhs[piv] = t;
        }
        for (int i = k + 1; i < m; i++) {
            double f = A[i * m + k] / A[k * m + k];
            for (int j = k; j < m; j++) A[i * m + j] -= f * A[k * m + j];
            rhs[i] -= f * rhs[k];
        }
    }
    for (int k = m - 1; k >= 0; k--) {
        double s = rhs[k];
        for (int j = k + 1; j < m; j++) s -= A[k * m + j] * rhs[j];
        rhs[k] = s / A[k * m + k];
    }
    return 0;
}

int orc_anderson(int natoms, const double *q_in, const double *r, double beta, int history,
                 double *hist_q, double *hist_r, int *hcount, int *hhead, double *q_next)
{
    /* Anderson mixing (D. G. Anderson, J. ACM 12, 547 (1965)): minimise
     * || r - sum_j gamma_j (r - r_j) || over the stored residuals r_j, then
     * q_next = qbar + beta * rbar with qbar = q - sum_j gamma_j (q - q_j) and
     * rbar likewise.  A relative 1e-10 Tikhonov term keeps the normal
     * equations regular. */
    const int m = *hcount;
    double gam[16];
    int use = 0;
    if (m > 0) {
        double A[16 * 16], rhs[16];
        for (int i = 0; i < m; i++) {
            const double *ri = hist_r + (size_t)i * natoms;
            double bi = 0.0;
            for (int a = 0; a < natoms; a++) bi += (r[a] - ri[a]) * r[a];
            rhs[i] = bi;
            for (int j = 0; j <= i; j++) {
                const double *rj = hist_r + (size_t)j * natoms;
                double s = 0.0;
                for (int a = 0; a < natoms; a++) s += (r[a] - ri[a]) * (r[a] - rj[a]);
                A[i * m + j] = s;
                A[j * m + i] = s;
            }
        }
        for (int i = 0; i < m; i++) A[i * m + i] *= (1.0 + 1e-10);
        if (solve_small(m, A, rhs) == 0) {
            use = 1;
            for (int i = 0; i < m; i++) gam[i] = rhs[i];
        }
    }
    /* q_next may alias q_in: the update of entry a reads only entry a of
     * q_in, and the history slot is written afterwards from a saved copy. */
    double *save = (double *)malloc(sizeof(double) * natoms);
    memcpy(save, q_in, sizeof(double) * natoms);
    for (int a = 0; a < natoms; a++) {
        double qb = save[a], rb = r[a];
        if (use)
            for (int i = 0; i < m; i++) {
                qb -= gam[i] * (save[a] - hist_q[(size_t)i * natoms + a]);
                rb -= gam[i] * (r[a] - hist_r[(size_t)i * natoms + a]);
            }
        q_next[a] = qb + beta * rb;
    }
    if (history > 0) {
        int slot = *hhead;
        memcpy(hist_q + (size_t)slot * natoms, save, sizeof(double) * natoms);
        memcpy(hist_r + (size_t)slot * natoms, r, sizeof(double) * natoms);
        *hhead = (slot + 1) % history;
        if (*hcount < history) *hcount = *hcount + 1;
    }
    free(save);
    return ORC_OK;
}

int orc_scc(int n, const int32_t *rowptr, const int32_t *col, const double *val,
            const int32_t *orb2atom, int natoms, const int32_t *g_rowptr, const int32_t *g_col,
            const double *g_val, const double *q0, const double *q_init,
            const orc_kpe_params *p, const orc_scc_params *s, double *q_out, double *diagP,
            double *dq_hist, int *iters, orc_kpe_result *res)
{
    if (s->history > 16) return ORC_ERR_ARG;
    double *q_in = (double *)malloc(sizeof(double) * natoms);
    double *qo = (double *)malloc(sizeof(double) * natoms);
    double *dq = (double *)malloc(sizeof(double) * natoms);
    double *V = (double *)malloc(sizeof(double) * natoms);
    double *shift = (double *)malloc(sizeof(double) * n);
    double *r = (double *)malloc(sizeof(double) * natoms);
    int hist = s->history > 0 ? s->history : 1;
    double *hq = (double *)malloc(sizeof(double) * (size_t)hist * natoms);
    double *hr = (double *)malloc(sizeof(double) * (size_t)hist * natoms);
    int hcount = 0, hhead = 0;
    for (int a = 0; a < natoms; a++) q_in[a] = q_init ? q_init[a] : q0[a];
    int err = ORC_ERR_NOT_CONVERGED, it;
    for (it = 1; it <= s->max_iter; it++) {
        for (int a = 0; a < natoms; a++) dq[a] = q_in[a] - q0[a];
        orc_gamma_mult(natoms, g_rowptr, g_col, g_val, dq, V);
        for (int i = 0; i < n; i++) shift[i] = V[orb2atom[i]];
        int e = orc_density(n, rowptr, col, val, shift, orb2atom, natoms, p, diagP, qo, NULL,
                            NULL, res);
        if (e) {
            err = e;
            break;
        }
        double mx = 0.0;
        for (int a = 0; a < natoms; a++) {
            r[a] = qo[a] - q_in[a];
            if (fabs(r[a]) > mx) mx = fabs(r[a]);
        }
        if (dq_hist) dq_hist[it - 1] = mx;
        if (mx < s->tol) {
            err = ORC_OK;
            break;
        }
        if (!(mx < 1e3)) { /* diverged: charges beyond any physical range */
            err = ORC_ERR_NOT_CONVERGED;
            break;
        }
        orc_anderson(natoms, q_in, r, s->beta, s->history, hq, hr, &hcount, &hhead, q_in);
    }
    if (it > s->max_iter) it = s->max_iter;
    memcpy(q_out, qo, sizeof(double) * natoms);
    if (iters) *iters = it;
    free(q_in);
    free(qo);
    free(dq);
    free(V);
    free(shift);
    free(r);
    free(hq);
    free(hr);
    return err;
}

/* ------------------------------------------------------------------------- */
/* SP2 on thresholded 4x4 blocks                                             */
/* ------------------------------------------------------------------------- */
typedef struct {
    int nb;          /* block rows */
    int32_t *rowptr; /* nb+1 */
    int32_t *col;    /* nnzb */
    double *blk;     /* nnzb*16, row-major 4x4 */
} bsr_t;

static void bsr_free(bsr_t *m)
{
    free(m->rowptr);
    free(m->col);
    free(m->blk);
    memset(m, 0, sizeof(*m));
}

static double bnorm2(const double *b)
{
    double s = 0.0;
    for (int t = 0; t < 16; t++) s += b[t] * b[t];
    return s;
}

/* Per-row dense accumulator over block columns (used by the SpGEMM). */
typedef struct {
    int32_t *pos;  /* nb, -1 when absent */
    int32_t *list; /* touched columns */
    double *acc;   /* capacity*16 */
    int cnt, cap;
} accum_t;

static void acc_init(accum_t *A, int nb)
{
    A->pos = (int32_t *)malloc(sizeof(int32_t) * nb);
    for (int i = 0; i < nb; i++) A->pos[i] = -1;
    A->cap = 256;
    A->list = (int32_t *)malloc(sizeof(int32_t) * A->cap);
    A->acc = (double *)malloc(sizeof(double) * 16 * A->cap);
    A->cnt = 0;
}

static double *acc_slot(accum_t *A, int c)
{
    if (A->pos[c] < 0) {
        if (A->cnt == A->cap) {
            A->cap *= 2;
            A->list = (int32_t *)realloc(A->list, sizeof(int32_t) * A->cap);
            A->acc = (double *)realloc(A->acc, sizeof(double) * 16 * A->cap);
        }
        A->pos[c] = A->cnt;
        A->list[A->cnt] = c;
        memset(A->acc + 16 * A->cnt, 0, 16 * sizeof(double));
        A->cnt++;
    }
    return A->acc + 16 * A->pos[c];
}

static int cmp_i32(const void *a, const void *b)
{
    int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

/* One SP2 step on block row I: computes (X^2)_I exactly, accumulates
 * ||X^2 - X||_F^2 and tr(X^2) contributions, and emits the thresholded new
 * row (X^2 or 2X - X^2).  Returns the number of kept blocks written to
 * out_col/out_blk (caller-provided growable buffers). */
typedef struct {
    int32_t *col;
    double *blk;
    int cnt, cap;
} rowbuf_t;

static void rowbuf_push(rowbuf_t *R, int c, const double *b)
{
    if (R->cnt == R->cap) {
        R->cap = R->cap ? 2 * R->cap : 256;
        R->col = (int32_t *)realloc(R->col, sizeof(int32_t) * R->cap);
        R->blk = (double *)realloc(R->blk, sizeof(double) * 16 * R->cap);
    }
    R->col[R->cnt] = c;
    memcpy(R->blk + 16 * R->cnt, b, 16 * sizeof(double));
    R->cnt++;
}

int orc_sp2(int n, const int32_t *rowptr, const int32_t *col, const double *val,
            const int32_t *orb2atom, int natoms, const orc_sp2_params *p, double *diagP,
            double *q, int32_t *branches, double *idem_hist, double *trace_hist,
            orc_sp2_result *res)
{
    if (n % 4 != 0 || n < 4) return ORC_ERR_ARG;
    const int nb = n / 4;
    orc_sp2_result R;
    memset(&R, 0, sizeof(R));
    orc_gershgorin(n, rowptr, col, val, NULL, &R.lmin, &R.lmax);
    const double width = R.lmax - R.lmin;
    const double drop2 = p->drop_tol * p->drop_tol;

    /* H as BSR (for the band energy) and X0 = (lmax I - H)/(lmax - lmin). */
    bsr_t H = {nb, NULL, NULL, NULL}, X = {nb, NULL, NULL, NULL};
    {
        accum_t A;
        acc_init(&A, nb);
        rowbuf_t rb = {NULL, NULL, 0, 0};
        H.rowptr = (int32_t *)malloc(sizeof(int32_t) * (nb + 1));
        H.rowptr[0] = 0;
        for (int I = 0; I < nb; I++) {
            A.cnt = 0;
            for (int r = 0; r < 4; r++) {
                const int i = 4 * I + r;
                for (int k = rowptr[i]; k < rowptr[i + 1]; k++) {
                    double *s = acc_slot(&A, col[k] / 4);
                    s[4 * r + col[k] % 4] = val[k];
                }
            }
            qsort(A.list, A.cnt, sizeof(int32_t), cmp_i32);
            for (int t = 0; t < A.cnt; t++) {
                rowbuf_push(&rb, A.list[t], A.acc + 16 * A.pos[A.list[t]]);
                A.pos[A.list[t]] = -1;
            }
            H.rowptr[I + 1] = rb.cnt;
        }
        H.col = rb.col;
        H.blk = rb.blk;
        free(A.pos);
        free(A.list);
        free(A.acc);
        X.rowptr = (int32_t *)malloc(sizeof(int32_t) * (nb + 1));
        const int64_t nz = H.rowptr[nb];
        X.col = (int32_t *)malloc(sizeof(int32_t) * (nz > 0 ? nz : 1));
        X.blk = (double *)malloc(sizeof(double) * 16 * (nz > 0 ? nz : 1));
        memcpy(X.rowptr, H.rowptr, sizeof(int32_t) * (nb + 1));
        memcpy(X.col, H.col, sizeof(int32_t) * nz);
        for (int64_t t = 0; t < nz; t++)
            for (int e = 0; e < 16; e++) X.blk[16 * t + e] = -H.blk[16 * t + e] / width;
        for (int Ib = 0; Ib < nb; Ib++)
            for (int t = X.rowptr[Ib]; t < X.rowptr[Ib + 1]; t++)
                if (X.col[t] == Ib)
                    for (int r = 0; r < 4; r++) X.blk[16 * t + 5 * r] += R.lmax / width;
    }

    int it;
    double prev1 = INFINITY, prev2 = INFINITY;
#ifdef _OPENMP
    if (p->nthreads > 0) omp_set_num_threads(p->nthreads);
#endif
    for (it = 0;; it++) {
        /* X^2 row by row (exact), idempotency error and traces. */
        double trX = 0.0, trX2 = 0.0, idem2 = 0.0;
        for (int I = 0; I < nb; I++)
            for (int t = X.rowptr[I]; t < X.rowptr[I + 1]; t++)
                if (X.col[t] == I)
                    for (int r = 0; r < 4; r++) trX += X.blk[16 * t + 5 * r];
        const int branch = (2.0 * trX > p->n_elec) ? -1 : 1; /* withSP2.cpp:1029-1030 */
        rowbuf_t *rows = (rowbuf_t *)calloc(nb, sizeof(rowbuf_t));
#pragma omp parallel reduction(+ : trX2, idem2)
        {
            accum_t A;
            acc_init(&A, nb);
#pragma omp for schedule(dynamic, 8)
            for (int I = 0; I < nb; I++) {
                A.cnt = 0;
                for (int t = X.rowptr[I]; t < X.rowptr[I + 1]; t++) {
                    const int K = X.col[t];
                    const double *a = X.blk + 16 * t;
                    for (int u = X.rowptr[K]; u < X.rowptr[K + 1]; u++) {
                        double *c = acc_slot(&A, X.col[u]);
                        const double *bb = X.blk + 16 * u;
                        for (int r = 0; r < 4; r++)
                            for (int s = 0; s < 4; s++) {
                                double v = 0.0;
                                for (int m = 0; m < 4; m++) v += a[4 * r + m] * bb[4 * m + s];
                                c[4 * r + s] += v;
                            }
                    }
                }
                /* X itself into a second view: mark its blocks */
                for (int t = X.rowptr[I]; t < X.rowptr[I + 1]; t++) (void)acc_slot(&A, X.col[t]);
                qsort(A.list, A.cnt, sizeof(int32_t), cmp_i32);
                int xt = X.rowptr[I];
                for (int t = 0; t < A.cnt; t++) {
                    const int J = A.list[t];
                    const double *x2 = A.acc + 16 * A.pos[J];
                    const double *xb = NULL;
                    while (xt < X.rowptr[I + 1] && X.col[xt] < J) xt++;
                    if (xt < X.rowptr[I + 1] && X.col[xt] == J) xb = X.blk + 16 * xt;
                    double nb2[16];
                    for (int e = 0; e < 16; e++) {
                        const double xv = xb ? xb[e] : 0.0;
                        const double dlt = x2[e] - xv;
                        idem2 += dlt * dlt;
                        nb2[e] = (branch < 0) ? x2[e] : 2.0 * xv - x2[e];
                    }
                    if (J == I)
                        for (int r = 0; r < 4; r++) trX2 += x2[5 * r];
                    if (bnorm2(nb2) >= drop2) rowbuf_push(&rows[I], J, nb2);
                    A.pos[J] = -1;
                }
            }
            free(A.pos);
            free(A.list);
            free(A.acc);
        }
        const double idem = sqrt(idem2);
        if (idem_hist && it < p->max_iter + 1) idem_hist[it] = idem;
        if (trace_hist && it < p->max_iter + 1) trace_hist[it] = trX;
        int stop = 0;
        if (idem < p->idem_tol) stop = 1;
        if (p->trace_tol > 0 && fabs(2.0 * trX - p->n_elec) < p->trace_tol && idem < 1.0) stop = 1;
        /* stagnation: past the oscillating start (errors below 0.1, where the
         * expansion converges quadratically) an error that no longer falls
         * over two steps has reached the drop-tolerance / round-off floor */
        if (it >= 2 && prev2 < 0.1 && idem >= prev2) stop = 1;
        if (it >= p->max_iter) stop = 1;
        if (stop) {
            R.idem_err = idem;
            R.trace = trX;
            for (int I = 0; I < nb; I++) free(rows[I].col), free(rows[I].blk);
            free(rows);
            break;
        }
        if (branches) branches[it] = branch;
        /* assemble X_{k+1} */
        int64_t tot = 0;
        for (int I = 0; I < nb; I++) tot += rows[I].cnt;
        bsr_t Y;
        Y.nb = nb;
        Y.rowptr = (int32_t *)malloc(sizeof(int32_t) * (nb + 1));
        Y.col = (int32_t *)malloc(sizeof(int32_t) * (tot > 0 ? tot : 1));
        Y.blk = (double *)malloc(sizeof(double) * 16 * (tot > 0 ? tot : 1));
        Y.rowptr[0] = 0;
        int64_t o = 0;
        for (int I = 0; I < nb; I++) {
            memcpy(Y.col + o, rows[I].col, sizeof(int32_t) * rows[I].cnt);
            memcpy(Y.blk + 16 * o, rows[I].blk, sizeof(double) * 16 * rows[I].cnt);
            o += rows[I].cnt;
            Y.rowptr[I + 1] = (int32_t)o;
            free(rows[I].col);
            free(rows[I].blk);
        }
        free(rows);
        bsr_free(&X);
        X = Y;
        prev2 = prev1;
        prev1 = idem;
    }
    R.iters = it;
    R.nnzb = X.rowptr[nb];
    /* outputs: diag P, charges, band energy 2 tr(X H) */
    double eb = 0.0;
    for (int I = 0; I < nb; I++) {
        for (int t = X.rowptr[I]; t < X.rowptr[I + 1]; t++) {
            const int J = X.col[t];
            if (J == I && diagP)
                for (int r = 0; r < 4; r++) diagP[4 * I + r] = X.blk[16 * t + 5 * r];
            /* tr(X H) = sum_{I,J} sum_{r,s} X_IJ[r][s] H_JI[s][r] */
            for (int u = H.rowptr[J]; u < H.rowptr[J + 1]; u++)
                if (H.col[u] == I) {
                    const double *xb = X.blk + 16 * t, *hb = H.blk + 16 * u;
                    for (int r = 0; r < 4; r++)
                        for (int s = 0; s < 4; s++) eb += xb[4 * r + s] * hb[4 * s + r];
                }
        }
    }
    R.e_band = 2.0 * eb;
    if (q && diagP) {
        for (int a = 0; a < natoms; a++) q[a] = 0.0;
        for (int i = 0; i < n; i++) q[orb2atom[i]] += 2.0 * diagP[i];
    }
    if (res) *res = R;
    bsr_free(&X);
    bsr_free(&H);
    return ORC_OK;
}

/* ------------------------------------------------------------------------- */
/* Stochastic KPM density of states                                          */
/* ------------------------------------------------------------------------- */
int orc_kpm_dos(int n, const int32_t *rowptr, const int32_t *col, const double *val, double a,
                double b, int nmom, int n_random, uint64_t seed, int npts, double *mom,
                double *energies, double *dos)
{
    if (nmom < 2 || n_random < 1 || !(a > 0)) return ORC_ERR_ARG;
    double *xv = (double *)malloc(sizeof(double) * rowptr[n]);
    double *xd = (double *)malloc(sizeof(double) * n);
    for (int i = 0; i < n; i++) {
        int found = 0;
        for (int k = rowptr[i]; k < rowptr[i + 1]; k++) {
            if (col[k] == i) {
                xv[k] = (val[k] - b) / a;
                found = 1;
            } else
                xv[k] = val[k] / a;
        }
        xd[i] = found ? 0.0 : -b / a;
    }
    double *r = (double *)malloc(sizeof(double) * n);
    double *v0 = (double *)malloc(sizeof(double) * n);
    double *v1 = (double *)malloc(sizeof(double) * n);
    for (int k = 0; k < nmom; k++) mom[k] = 0.0;
    for (int t = 0; t < n_random; t++) {
        for (int i = 0; i < n; i++) r[i] = orc_gauss(seed, (uint64_t)t * n + i);
        double s0 = 0.0, s1 = 0.0;
        for (int i = 0; i < n; i++) {
            v0[i] = r[i];
            s0 += r[i] * v0[i];
        }
        for (int i = 0; i < n; i++) {
            double acc = xd[i] * v0[i];
            for (int k = rowptr[i]; k < rowptr[i + 1]; k++) acc += xv[k] * v0[col[k]];
            v1[i] = acc;
            s1 += r[i] * acc;
        }
        mom[0] += s0;
        mom[1] += s1;
        for (int kk = 2; kk < nmom; kk++) {
            double s = 0.0;
            for (int i = 0; i < n; i++) {
                double acc = xd[i] * v1[i];
                for (int k = rowptr[i]; k < rowptr[i + 1]; k++) acc += xv[k] * v1[col[k]];
                double nv = 2.0 * acc - v0[i];
                v0[i] = nv;
            }
            for (int i = 0; i < n; i++) s += r[i] * v0[i];
            mom[kk] += s;
            double *tmp = v0;
            v0 = v1;
            v1 = tmp;
        }
    }
    double *g = (double *)malloc(sizeof(double) * nmom);
    orc_jackson(nmom, g);
    for (int k = 0; k < npts; k++) {
        const double x = cos(ORC_PI * (k + 1.0 / 2.0) / npts);
        double s = g[0] * mom[0];
        for (int j = 1; j < nmom; j++) s = s + 2 * g[j] * mom[j] * cos(j * acos(x));
        dos[k] = s / (ORC_PI * sqrt(1.0 - x * x));
        energies[k] = x * a + b;
    }
    free(g);
    free(xv);
    free(xd);
    free(r);
    free(v0);
    free(v1);
    return ORC_OK;
}

/* ------------------------------------------------------------------------- */
/* Stochastic-trace density                                                  */
/* ------------------------------------------------------------------------- */
void orc_dos_mu(int npts, const double *energies, const double *dos, double n_elec, int n,
                double *mu, int *mu_index, double *a, double *b)
{
    /* node abscissae as runKPM has them: x_k = cos(pi (k+1/2)/npts), falling in k */
    double dosall = 0.0;
    for (int i = npts - 1; i > 0; i--) {
        const double xi = cos(ORC_PI * (i + 0.5) / npts), xm = cos(ORC_PI * (i - 0.5) / npts);
        dosall += (xm - xi) * (dos[i] + dos[i - 1]) / 2;
    }
    const double area = n_elec * dosall / (2.0 * n);
    double cum = 0.0;
    int mi = 0;
    for (int i = npts - 1; i > 0; i--) {
        const double xi = cos(ORC_PI * (i + 0.5) / npts), xm = cos(ORC_PI * (i - 0.5) / npts);
        cum += (xm - xi) * (dos[i] + dos[i - 1]) / 2;
        if (cum >= area) {
            mi = i;
            break;
        }
    }
    double emin = -10.0, emax = 10.0;
    for (int i = npts - 1; i > 0; i--)
        if (dos[i] / n >= 0.001) {
            emin = energies[i];
            break;
        }
    for (int i = 0; i < npts; i++)
        if (dos[i] / n >= 0.001) {
            emax = energies[i];
            break;
        }
    *mu = energies[mi];
    *mu_index = mi;
    *a = (emax - emin) / 2;
    *b = (emax + emin) / 2;
}

int orc_density_stochastic(int n, const int32_t *rowptr, const int32_t *col, const double *val,
                           const int32_t *orb2atom, int natoms, const orc_kpe_params *p,
                           int n_random, uint64_t seed, int dos_moments, int dos_points,
                           double *diagP, double *q, orc_kpe_result *res)
{
    const int M = p->M;
    if (M < 2 || n < 1 || n_random < 1 || dos_moments < 2 || dos_points < 2) return ORC_ERR_ARG;
    orc_kpe_result r;
    memset(&r, 0, sizeof(r));
    orc_gershgorin(n, rowptr, col, val, NULL, &r.lmin, &r.lmax);
    const double a0 = 0.5 * (r.lmax - r.lmin) * (1.0 + p->pad), b0 = 0.5 * (r.lmax + r.lmin);
    if (!(a0 > 0)) return ORC_ERR_ARG;
    double *mom = (double *)malloc(sizeof(double) * dos_moments);
    double *E = (double *)malloc(sizeof(double) * dos_points);
    double *dos = (double *)malloc(sizeof(double) * dos_points);
    int err = orc_kpm_dos(n, rowptr, col, val, a0, b0, dos_moments, n_random, seed, dos_points, mom, E, dos);
    if (err) {
        free(mom);
        free(E);
        free(dos);
        return err;
    }
    int mi = 0;
    orc_dos_mu(dos_points, E, dos, p->n_elec, n, &r.mu, &mi, &r.a, &r.b);
    free(mom);
    free(E);
    free(dos);
    if (!(r.a > 0)) return ORC_ERR_ARG;
    r.mu_x = (r.mu - r.b) / r.a;
    double *g = (double *)malloc(sizeof(double) * M);
    if (p->kernel == 0)
        orc_jackson(M, g);
    else if (p->kernel == 1)
        orc_kernel_autocorr(M, g);
    else
        for (int k = 0; k < M; k++) g[k] = 1.0;
    g[0] = 1.0;
    double *c = (double *)malloc(sizeof(double) * M);
    const double beta_x = p->kT > 0 ? r.a / p->kT : 0.0;
    if (beta_x > 0)
        orc_fermi_coeffs(M, r.mu_x, beta_x, orc_quadrature_nodes(M, beta_x), c);
    else
        orc_step_coeffs(M, r.mu_x, c);
    /* X = (H - b)/a */
    double *xv = (double *)malloc(sizeof(double) * (rowptr[n] > 0 ? rowptr[n] : 1));
    double *xd = (double *)malloc(sizeof(double) * n);
    for (int i = 0; i < n; i++) {
        int found = 0;
        for (int k = rowptr[i]; k < rowptr[i + 1]; k++) {
            if (col[k] == i) {
                xv[k] = (val[k] - r.b) / r.a;
                found = 1;
            } else
                xv[k] = val[k] / r.a;
        }
        xd[i] = found ? 0.0 : -r.b / r.a;
    }
    double *x = (double *)malloc(sizeof(double) * n);
    double *v0 = (double *)malloc(sizeof(double) * n);
    double *v1 = (double *)malloc(sizeof(double) * n);
    double *num = (double *)calloc(n, sizeof(double));
    double *den = (double *)calloc(n, sizeof(double));
    for (int t = 0; t < n_random; t++) {
        for (int i = 0; i < n; i++) {
            x[i] = orc_gauss(seed + 1, (uint64_t)t * n + i);
            v0[i] = x[i];
            den[i] += x[i] * x[i];
            num[i] += c[0] * g[0] * x[i] * x[i];
        }
        for (int i = 0; i < n; i++) {
            double acc = xd[i] * v0[i];
            for (int k = rowptr[i]; k < rowptr[i + 1]; k++) acc += xv[k] * v0[col[k]];
            v1[i] = acc;
            num[i] += c[1] * g[1] * x[i] * acc;
        }
        for (int kk = 2; kk < M; kk++) {
            for (int i = 0; i < n; i++) {
                double acc = xd[i] * v1[i];
                for (int k = rowptr[i]; k < rowptr[i + 1]; k++) acc += xv[k] * v1[col[k]];
                v0[i] = 2.0 * acc - v0[i];
            }
            for (int i = 0; i < n; i++) num[i] += c[kk] * g[kk] * x[i] * v0[i];
            double *tmp = v0;
            v0 = v1;
            v1 = tmp;
        }
    }
    if (q)
        for (int at = 0; at < natoms; at++) q[at] = 0.0;
    for (int i = 0; i < n; i++) {
        const double d = num[i] / den[i];
        if (diagP) diagP[i] = d;
        if (q) q[orb2atom[i]] += 2.0 * d;
    }
    if (res) *res = r;
    free(g);
    free(c);
    free(xv);
    free(xd);
    free(x);
    free(v0);
    free(v1);
    free(num);
    free(den);
    return ORC_OK;
}

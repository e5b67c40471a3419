// tb_model.cpp -- synthetic-input builder upstream of the C-ABI boundary:
// geometry, neighbour lists, the reference's sp3 block model, Gamma and q0.
// Produces what arrangeCoordinates + constructH + initializeForSCF of the
// reference build (withSP2_deltaH.cpp:372-740, 854-1066) as plain CSR arrays.
//
// The block model is written through its four radial functions
//   R_i(r) = sum_{p=1..20} cp_i T_p(r/10) e^{-p r},  i in {2,3,5,6},
// from the 20-term tables of withSP2_deltaH.cpp:75-142, so that with
// l = (x,y,z)/r:  H_ss = R6,  H_s,pk = R5 l_k = -H_pk,s,
//                 H_pk,pm = (R2 - R3) l_k l_m + R3 delta_km
// -- the same block get4by4HmatrixElements (withSP2_deltaH.cpp:211-349)
// accumulates term by term.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/largetb.h"
#include "tb_abi_guard.h"

namespace {

constexpr double kPi = 3.141592653589793238463;
constexpr double kBohrPerAng = 1.88973;  // withSP2_deltaH.cpp:377

// cp2, cp3, cp5, cp6 per power p (withSP2_deltaH.cpp:75-142).
const double kSiSi[20][4] = {
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
const double kOO[20][4] = {
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
const double kSiO[20][4] = {
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

struct Onsite {
    double es, ep;
};
// withSP2_deltaH.cpp:255-261 (Si) and 288-294 (O)
Onsite onsite(int z) { return z == 14 ? Onsite{-0.39572506, -0.15031380} : Onsite{-0.87883246, -0.33213167}; }

const double (*pair_table(int zi, int zj))[4]
{
    if (zi == 14 && zj == 14) return kSiSi;
    if (zi == 8 && zj == 8) return kOO;
    if ((zi == 14 && zj == 8) || (zi == 8 && zj == 14)) return kSiO;
    return nullptr;
}

// 4x4 block for the displacement (x,y,z) = r_j - r_i.
int hopping_block(int zi, int zj, double x, double y, double z, double out[16])
{
    const double (*tab)[4] = pair_table(zi, zj);
    if (!tab) return TB_ERR_INVALID_ARG;
    const double r2 = x * x + y * y + z * z, r = std::sqrt(r2);
    if (r < 0.01) return TB_ERR_INVALID_ARG;
    double R2 = 0, R3 = 0, R5 = 0, R6 = 0;
    const double th = std::acos(r / 10);
    for (int p = 1; p <= 20; p++) {
        const double f = std::cos(p * th) * std::exp(-p * r);
        R2 += tab[p - 1][0] * f;
        R3 += tab[p - 1][1] * f;
        R5 += tab[p - 1][2] * f;
        R6 += tab[p - 1][3] * f;
    }
    const double l[3] = {x / r, y / r, z / r};
    out[0] = R6;
    for (int k = 0; k < 3; k++) {
        out[1 + k] = R5 * l[k];
        out[4 * (1 + k)] = -R5 * l[k];
        for (int m = 0; m < 3; m++)
            out[4 * (1 + k) + 1 + m] = (R2 - R3) * l[k] * l[m] + (k == m ? R3 : 0.0);
    }
    return TB_OK;
}

uint64_t splitmix_at(uint64_t seed, uint64_t k)
{
    uint64_t z = seed + (k + 1u) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Box-Muller (cosine branch) on splitmix64 outputs 2 idx and 2 idx + 1.
double gauss_at(uint64_t seed, uint64_t idx)
{
    const double two53 = 1.0 / 9007199254740992.0;
    const double u1 = ((double)(splitmix_at(seed, 2u * idx) >> 11) + 1.0) * two53;
    const double u2 = (double)(splitmix_at(seed, 2u * idx + 1u) >> 11) * two53;
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * kPi * u2);
}

struct Neighbour {
    int32_t j;
    double dx, dy, dz;
};

}  // namespace

struct tb_model {
    int32_t natoms = 0;
    std::vector<double> xyz;
    std::vector<int32_t> species;
    std::vector<int32_t> rowptr, colidx;
    std::vector<double> vals;
    std::vector<int32_t> g_rowptr, g_colidx;
    std::vector<double> g_vals;
    std::vector<double> q0;
};

namespace {

// Assemble H and Gamma from per-atom neighbour lists (sorted by j).
int assemble(tb_model *m, std::vector<std::vector<Neighbour>> &nb, double gamma_diag)
{
    const int na = m->natoms, n = 4 * na;
    m->rowptr.assign(n + 1, 0);
    m->g_rowptr.assign(na + 1, 0);
    m->colidx.clear();
    m->vals.clear();
    m->g_colidx.clear();
    m->g_vals.clear();
    std::vector<double> blocks;
    std::vector<int32_t> cols;
    for (int i = 0; i < na; i++) {
        auto &L = nb[i];
        std::sort(L.begin(), L.end(), [](const Neighbour &a, const Neighbour &b) { return a.j < b.j; });
        for (size_t t = 1; t < L.size(); t++)
            if (L[t].j == L[t - 1].j) return TB_ERR_STRUCTURE;  // two images of one atom
        cols.clear();
        blocks.clear();
        bool self_done = false;
        auto push_self = [&]() {
            const Onsite o = onsite(m->species[i]);
            double b[16] = {0};
            b[0] = o.es;
            b[5] = b[10] = b[15] = o.ep;
            cols.push_back(i);
            blocks.insert(blocks.end(), b, b + 16);
            m->g_colidx.push_back(i);
            m->g_vals.push_back(gamma_diag);
            self_done = true;
        };
        for (const Neighbour &e : L) {
            if (!self_done && e.j > i) push_self();
            double b[16];
            if (hopping_block(m->species[i], m->species[e.j], e.dx, e.dy, e.dz, b)) return TB_ERR_STRUCTURE;
            cols.push_back(e.j);
            blocks.insert(blocks.end(), b, b + 16);
            m->g_colidx.push_back(e.j);
            m->g_vals.push_back(1.0 / std::sqrt(e.dx * e.dx + e.dy * e.dy + e.dz * e.dz));
        }
        if (!self_done) push_self();
        m->g_rowptr[i + 1] = (int32_t)m->g_colidx.size();
        for (int r = 0; r < 4; r++) {
            for (size_t t = 0; t < cols.size(); t++)
                for (int c = 0; c < 4; c++) {
                    m->colidx.push_back(4 * cols[t] + c);
                    m->vals.push_back(blocks[16 * t + 4 * r + c]);
                }
            m->rowptr[4 * i + r + 1] = (int32_t)m->colidx.size();
        }
    }
    m->q0.resize(na);
    for (int i = 0; i < na; i++) m->q0[i] = m->species[i] == 14 ? 4.0 : 6.0;
    return TB_OK;
}

}  // namespace

extern "C" {

int tb_model_quartz(int32_t L, int32_t M, int32_t N, tb_model **out)
{
    TB_ABI_TRY
    if (!out || L < 1 || M < 1 || N < 1) return TB_ERR_INVALID_ARG;
    *out = nullptr;
    tb_model *m = new (std::nothrow) tb_model();
    if (!m) return TB_ERR_OUT_OF_MEMORY;
    // hexagonal cell and the nine sites of withSP2_deltaH.cpp:511-664
    const double a = 9.725, c = 10.7;
    const double R[3][3] = {{a, 0, 0}, {a * (-std::sin(kPi / 6)), a * std::cos(kPi / 6), 0}, {0, 0, c}};
    static const double frac[9][3] = {
        {0.4697, 0.0000, 0.0000}, {0.0000, 0.4697, 0.6777}, {0.5303, 0.5303, 0.3333},
        {0.4133, 0.2672, 0.1188}, {0.2672, 0.4133, 0.5479}, {0.7328, 0.1461, 0.7855},
        {0.5867, 0.8539, 0.2145}, {0.8539, 0.5867, 0.4521}, {0.1461, 0.7328, 0.8812}};
    m->natoms = 9 * L * M * N;
    m->xyz.resize(3 * (size_t)m->natoms);
    m->species.resize(m->natoms);
    int at = 0;
    for (int i = 0; i < L; i++)
        for (int j = 0; j < M; j++)
            for (int k = 0; k < N; k++)
                for (int s = 0; s < 9; s++, at++) {
                    for (int d = 0; d < 3; d++)
                        m->xyz[3 * at + d] = (i * R[0][d] + j * R[1][d] + k * R[2][d]) +
                                             (frac[s][0] * R[0][d] + frac[s][1] * R[1][d] + frac[s][2] * R[2][d]);
                    m->species[at] = s < 3 ? 14 : 8;
                }
    // x/y periodic halo (the z image loop is commented out in the reference,
    // withSP2_deltaH.cpp:401-403), window 0.1 < d^2 < 16
    std::vector<std::vector<Neighbour>> nb(m->natoms);
    for (int p = 0; p < m->natoms; p++)
        for (int lp = -1; lp <= 1; lp++)
            for (int mp = -1; mp <= 1; mp++) {
                double sh[3];
                for (int d = 0; d < 3; d++) sh[d] = lp * L * R[0][d] + mp * M * R[1][d];
                for (int q = 0; q < m->natoms; q++) {
                    const double dx = m->xyz[3 * q] + sh[0] - m->xyz[3 * p];
                    const double dy = m->xyz[3 * q + 1] + sh[1] - m->xyz[3 * p + 1];
                    const double dz = m->xyz[3 * q + 2] + sh[2] - m->xyz[3 * p + 2];
                    const double d2 = dx * dx + dy * dy + dz * dz;
                    if (d2 < 16.0 && d2 > 0.1) {
                        if (nb[p].size() >= 20) {  // maxN_A, withSP2_deltaH.cpp:27,357-359
                            delete m;
                            return TB_ERR_STRUCTURE;
                        }
                        nb[p].push_back({q, dx, dy, dz});
                    }
                }
            }
    int rc = assemble(m, nb, -1.0);
    if (rc) {
        delete m;
        return rc;
    }
    *out = m;
    return TB_OK;
    TB_ABI_CATCH
}

int tb_model_cristobalite(int32_t nx, int32_t ny, int32_t nz, double a_ang, double sigma_ang,
                          uint64_t seed, double rcut_bohr, double gamma_diag, tb_model **out)
{
    TB_ABI_TRY
    if (!out || nx < 1 || ny < 1 || nz < 1 || !(a_ang > 0) || !(sigma_ang >= 0) || !(rcut_bohr > 0) ||
        !std::isfinite(gamma_diag))
        return TB_ERR_INVALID_ARG;
    *out = nullptr;
    const double a = a_ang * kBohrPerAng, sig = sigma_ang * kBohrPerAng;
    const double box[3] = {nx * a, ny * a, nz * a};
    for (int d = 0; d < 3; d++)
        if (box[d] <= 2.0 * rcut_bohr) return TB_ERR_INVALID_ARG;  // one image per pair
    tb_model *m = new (std::nothrow) tb_model();
    if (!m) return TB_ERR_OUT_OF_MEMORY;
    // Fd-3m sites: fcc Si, fcc Si + (1/4,1/4,1/4), and the four Si-Si bond
    // midpoints (1/8,1/8,1/8) (3/8,3/8,1/8) (3/8,1/8,3/8) (1/8,3/8,3/8)
    // around each shifted Si.
    static const double fcc[4][3] = {{0, 0, 0}, {0, 0.5, 0.5}, {0.5, 0, 0.5}, {0.5, 0.5, 0}};
    static const double mid[4][3] = {
        {0.125, 0.125, 0.125}, {0.375, 0.375, 0.125}, {0.375, 0.125, 0.375}, {0.125, 0.375, 0.375}};
    double site[24][3];
    int sp[24];
    for (int s = 0; s < 24; s++) {
        for (int d = 0; d < 3; d++) {
            if (s < 4)
                site[s][d] = fcc[s][d];
            else if (s < 8)
                site[s][d] = fcc[s - 4][d] + 0.25;
            else
                site[s][d] = fcc[(s - 8) / 4][d] + mid[(s - 8) % 4][d];
        }
        sp[s] = s < 8 ? 14 : 8;
    }
    m->natoms = 24 * nx * ny * nz;
    m->xyz.resize(3 * (size_t)m->natoms);
    m->species.resize(m->natoms);
    int at = 0;
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++)
                for (int s = 0; s < 24; s++, at++) {
                    const int cidx[3] = {i, j, k};
                    for (int d = 0; d < 3; d++)
                        m->xyz[3 * at + d] = (cidx[d] + site[s][d]) * a + sig * gauss_at(seed, 3u * at + d);
                    m->species[at] = sp[s];
                }
    // cell-list search in the periodic box (bins >= rcut wide)
    int nbin[3];
    for (int d = 0; d < 3; d++) nbin[d] = std::max(1, (int)std::floor(box[d] / rcut_bohr));
    const int ncell = nbin[0] * nbin[1] * nbin[2];
    std::vector<std::vector<int32_t>> bins(ncell);
    auto bin_of = [&](int at_, int d) {
        double f = m->xyz[3 * at_ + d] / box[d];
        f -= std::floor(f);
        int b = (int)(f * nbin[d]);
        return b >= nbin[d] ? nbin[d] - 1 : b;
    };
    for (int p = 0; p < m->natoms; p++)
        bins[(bin_of(p, 0) * nbin[1] + bin_of(p, 1)) * nbin[2] + bin_of(p, 2)].push_back(p);
    const double rc2 = rcut_bohr * rcut_bohr;
    std::vector<std::vector<Neighbour>> nb(m->natoms);
    for (int p = 0; p < m->natoms; p++) {
        const int bp[3] = {bin_of(p, 0), bin_of(p, 1), bin_of(p, 2)};
        // neighbouring bins, each visited once even when nbin < 3
        std::vector<int> seen;
        for (int ox = -1; ox <= 1; ox++)
            for (int oy = -1; oy <= 1; oy++)
                for (int oz = -1; oz <= 1; oz++) {
                    const int bx = (bp[0] + ox + nbin[0]) % nbin[0];
                    const int by = (bp[1] + oy + nbin[1]) % nbin[1];
                    const int bz = (bp[2] + oz + nbin[2]) % nbin[2];
                    const int b = (bx * nbin[1] + by) * nbin[2] + bz;
                    if (std::find(seen.begin(), seen.end(), b) != seen.end()) continue;
                    seen.push_back(b);
                    for (int q : bins[b]) {
                        double dv[3];
                        for (int d = 0; d < 3; d++) {
                            double t = m->xyz[3 * q + d] - m->xyz[3 * p + d];
                            t -= box[d] * std::nearbyint(t / box[d]);  // minimum image
                            dv[d] = t;
                        }
                        const double d2 = dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2];
                        if (d2 < rc2 && d2 > 0.1) nb[p].push_back({q, dv[0], dv[1], dv[2]});
                    }
                }
    }
    int rc = assemble(m, nb, gamma_diag);
    if (rc) {
        delete m;
        return rc;
    }
    *out = m;
    return TB_OK;
    TB_ABI_CATCH
}

int tb_model_sizes(const tb_model *m, int32_t *natoms, int32_t *n, int64_t *nnz, int64_t *g_nnz)
{
    TB_ABI_TRY
    if (!m) return TB_ERR_INVALID_ARG;
    if (natoms) *natoms = m->natoms;
    if (n) *n = 4 * m->natoms;
    if (nnz) *nnz = (int64_t)m->vals.size();
    if (g_nnz) *g_nnz = (int64_t)m->g_vals.size();
    return TB_OK;
    TB_ABI_CATCH
}

int tb_model_export(const tb_model *m, int32_t *rowptr, int32_t *colidx, double *vals,
                    int32_t *orb2atom, int32_t *g_rowptr, int32_t *g_colidx, double *g_vals,
                    double *q0, double *xyz, int32_t *species)
{
    TB_ABI_TRY
    if (!m) return TB_ERR_INVALID_ARG;
    const size_t n = 4 * (size_t)m->natoms;
    if (rowptr) std::memcpy(rowptr, m->rowptr.data(), (n + 1) * sizeof(int32_t));
    if (colidx) std::memcpy(colidx, m->colidx.data(), m->colidx.size() * sizeof(int32_t));
    if (vals) std::memcpy(vals, m->vals.data(), m->vals.size() * sizeof(double));
    if (orb2atom)
        for (size_t i = 0; i < n; i++) orb2atom[i] = (int32_t)(i / 4);
    if (g_rowptr) std::memcpy(g_rowptr, m->g_rowptr.data(), m->g_rowptr.size() * sizeof(int32_t));
    if (g_colidx) std::memcpy(g_colidx, m->g_colidx.data(), m->g_colidx.size() * sizeof(int32_t));
    if (g_vals) std::memcpy(g_vals, m->g_vals.data(), m->g_vals.size() * sizeof(double));
    if (q0) std::memcpy(q0, m->q0.data(), m->q0.size() * sizeof(double));
    if (xyz) std::memcpy(xyz, m->xyz.data(), m->xyz.size() * sizeof(double));
    if (species) std::memcpy(species, m->species.data(), m->species.size() * sizeof(int32_t));
    return TB_OK;
    TB_ABI_CATCH
}

int tb_model_destroy(tb_model *m)
{
    TB_ABI_TRY
    delete m;
    return TB_OK;
    TB_ABI_CATCH
}

}  // extern "C"

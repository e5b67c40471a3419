// tb_geom.cu -- Hamiltonian, Gamma and q0 built on the GPU from atom
// positions: the device form of the reference's getHaloAtoms + constructH +
// initializeForSCF (withSP2_deltaH.cpp:372-501, 969-1066, 854-899) for an
// orthorhombic periodic box.
//
//   k_geo_count   one thread per atom: neighbours j with 0.1 < d^2 < rc^2
//                 under the minimum image (plus the atom itself)
//   k_geo_fill    block columns of each row, ascending (self included)
//   k_geo_blocks  one thread per stored block: the on-site block, or the sp3
//                 hopping block from the radial functions
//                 R_i(r) = sum_p cp_i T_p(r/10) e^{-p r} of the 20-term tables
//                 (withSP2_deltaH.cpp:75-142, 211-349); Gamma = diag_value on
//                 the diagonal, 1/r off it
//   k_geo_rowstats per orbital: diagonal and Gershgorin radius
#include <cuda_runtime.h>
#include <math.h>

#include <string>
#include <vector>

#include "tb_internal.h"

namespace tb {
namespace {

__constant__ double c_tab[3][20][4];  // Si-Si, O-O, Si-O: cp2 cp3 cp5 cp6

const double h_tab[3][20][4] = {
    {{17.865, -5.7398, 17.262, -13.794},   {87.114, 5.8664, 39.685, -7.1328},
     {-722.33, -52.111, -283.25, 27.816},  {66.059, -3.2651, 34.498, -27.631},
     {-613.94, -6.6631, -41.298, 12.075},  {-727.27, 1.3757, -112.62, 5.9498},
     {246.1, -84.273, 241.71, -164.58},    {-1564.3, 4.1541, -179.83, 22.449},
     {-589.53, -7.9678, 215.3, -36.682},   {-1020.8, 33.73, 7.8809, -87.911},
     {-812.85, -33.408, 13.727, 158.22},   {1189.7, 49.751, 54.842, -56.155},
     {-96.931, 8.9531, 102.98, -91.347},   {860.35, 1.2204, -44.669, 12.487},
     {3551.6, 9.5425, -32.771, 10.438},    {468.97, 1.6056, -128.73, -1.5888},
     {-317.44, 6.9669, 133.21, 82.532},    {517.74, 47.052, -56.922, 1.1376},
     {210.8, -18.241, -18.441, 80.163},    {-443.57, 36.135, 52.835, -13.413}},
    {{5.5526, -0.82118, 3.813, -1.2323},   {-31.886, 10.518, -41.071, 52.454},
     {233.96, -39.064, 272.9, -407.19},    {-60.015, 61.253, -128.95, -294.22},
     {213.73, -204.34, 410.72, 1263.6},    {49.054, 32.239, -78.906, -1060},
     {-73.081, 132.93, -81.269, 1956.2},   {33.537, -13.278, -137.34, -384.47},
     {78.858, 165.14, -273.61, -873.53},   {-167.41, 68.088, -277.49, 642.65},
     {75.731, 7.9468, -767.04, -615.24},   {-63.795, -44.453, -288.57, 988.73},
     {-78.765, 32.997, -76.092, -811.61},  {124.63, -144.7, -189.3, 554.51},
     {40.615, -149.44, 780.52, 379.23},    {82.116, -29.881, 410.4, -93.407},
     {-80.656, -54.736, 203.1, -131.08},   {-74.163, 16.814, 710.57, -213.88},
     {7.3441, 20.02, -100.83, 128.52},     {-93.219, 6.9584, 267.84, -242.74}},
    {{13.778, -2.7061, 8.6477, -7.6931},   {9.0798, 19.494, -22.43, 52.885},
     {-15.173, -145.38, 262.06, -468.23},  {9.4007, -23.026, 223.86, -100.16},
     {40.783, 126.17, -785.64, 228.63},    {23.249, -34.501, 334.88, -253.56},
     {-17.829, -75.476, 156.18, -638.68},  {18.37, -22.003, 10.705, -312.46},
     {1.7289, 75.972, 572.55, -1010.6},    {-30.424, 17.518, -55.884, -478.46},
     {-31.663, -36.928, -349.49, -688.24}, {-82.425, -26.609, -390.25, -296.52},
     {35.07, 77.948, -143.41, 157.81},     {-27.066, -22.899, -390.79, 580.81},
     {-20.555, -140.91, -152.48, 401.59},  {49.585, -5.9967, 502.82, 768.76},
     {-8.7806, 109.97, -113.52, 980.42},   {37.13, -18.019, -148.42, 243.34},
     {-20.674, 15.652, 904.76, 317.15},    {16.513, 39.501, -630.1, 84.78}}};

__device__ __forceinline__ void min_image(const double *xyz, int i, int j, const double *box,
                                          double dv[3])
{
    for (int d = 0; d < 3; d++) {
        double t = xyz[3 * j + d] - xyz[3 * i + d];
        if (box[d] > 0) t -= box[d] * nearbyint(t / box[d]);
        dv[d] = t;
    }
}

__global__ void k_geo_count(int natoms, const double *__restrict__ xyz, double bx, double by,
                            double bz, double rc2, int32_t *__restrict__ cnt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= natoms) return;
    const double box[3] = {bx, by, bz};
    int c = 1;  // the on-site block
    for (int j = 0; j < natoms; j++) {
        double dv[3];
        min_image(xyz, i, j, box, dv);
        const double d2 = dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2];
        if (d2 < rc2 && d2 > 0.1) c++;
    }
    cnt[i] = c;
}

__global__ void k_geo_fill(int natoms, const double *__restrict__ xyz, double bx, double by, double bz,
                           double rc2, const int32_t *__restrict__ rowptr, int32_t *__restrict__ colidx,
                           int32_t *__restrict__ blkrow)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= natoms) return;
    const double box[3] = {bx, by, bz};
    int o = rowptr[i];
    for (int j = 0; j < natoms; j++) {
        if (j == i) {
            colidx[o] = i;
            blkrow[o++] = i;
            continue;
        }
        double dv[3];
        min_image(xyz, i, j, box, dv);
        const double d2 = dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2];
        if (d2 < rc2 && d2 > 0.1) {
            colidx[o] = j;
            blkrow[o++] = i;
        }
    }
}

__global__ void k_geo_blocks(int64_t nnzb, const double *__restrict__ xyz, const int32_t *__restrict__ sp,
                             double bx, double by, double bz, const int32_t *__restrict__ colidx,
                             const int32_t *__restrict__ blkrow, double gamma_diag,
                             double *__restrict__ h0, double *__restrict__ gval, int32_t *__restrict__ err)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nnzb) return;
    const int i = blkrow[t], j = colidx[t];
    double b[16];
    for (int e = 0; e < 16; e++) b[e] = 0.0;
    if (i == j) {
        // on-site energies, withSP2_deltaH.cpp:255-261 (Si) and 288-294 (O)
        const bool si = sp[i] == 14;
        b[0] = si ? -0.39572506 : -0.87883246;
        b[5] = b[10] = b[15] = si ? -0.15031380 : -0.33213167;
        gval[t] = gamma_diag;
    } else {
        const double box[3] = {bx, by, bz};
        double dv[3];
        min_image(xyz, i, j, box, dv);
        const double r = sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
        const int zi = sp[i], zj = sp[j];
        int tab = -1;
        if (zi == 14 && zj == 14) tab = 0;
        if (zi == 8 && zj == 8) tab = 1;
        if ((zi == 14 && zj == 8) || (zi == 8 && zj == 14)) tab = 2;
        if (tab < 0 || r < 0.01) {
            atomicExch(err, 1);
            return;
        }
        double R2 = 0, R3 = 0, R5 = 0, R6 = 0;
        const double th = acos(r / 10);
        for (int p = 1; p <= 20; p++) {
            const double f = cos(p * th) * exp(-p * r);
            R2 += c_tab[tab][p - 1][0] * f;
            R3 += c_tab[tab][p - 1][1] * f;
            R5 += c_tab[tab][p - 1][2] * f;
            R6 += c_tab[tab][p - 1][3] * f;
        }
        const double l[3] = {dv[0] / r, dv[1] / r, dv[2] / r};
        b[0] = R6;
        for (int k = 0; k < 3; k++) {
            b[1 + k] = R5 * l[k];
            b[4 * (1 + k)] = -R5 * l[k];
            for (int m = 0; m < 3; m++) b[4 * (1 + k) + 1 + m] = (R2 - R3) * l[k] * l[m] + (k == m ? R3 : 0.0);
        }
        gval[t] = 1.0 / r;
    }
    for (int e = 0; e < 16; e++) h0[t * 16 + e] = b[e];
}

__global__ void k_geo_rowstats(int nb, const int32_t *__restrict__ rowptr, const int32_t *__restrict__ colidx,
                               const double *__restrict__ h0, double *__restrict__ h0diag,
                               double *__restrict__ radius, int32_t *__restrict__ diagblk)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 4 * nb) return;
    const int I = i >> 2, r = i & 3;
    double dg = 0.0, rad = 0.0;
    for (int t = rowptr[I]; t < rowptr[I + 1]; t++) {
        if (r == 0 && colidx[t] == I) diagblk[I] = t;
        for (int c = 0; c < 4; c++) {
            const double v = h0[(int64_t)t * 16 + r * 4 + c];
            if (colidx[t] == I && c == r)
                dg = v;
            else
                rad += fabs(v);
        }
    }
    h0diag[i] = dg;
    radius[i] = rad;
}

}  // namespace

// Builds everything tb_set_hamiltonian + tb_set_scc would install, on the
// device.  Outputs are device buffers the caller adopts (freed with cudaFree);
// brow/bcol are also returned on the host for the staging plans.
int geom_build_device(cudaStream_t st, int natoms, const double *xyz_h, const int32_t *sp_h,
                      const double box[3], double rcut, double gamma_diag, GeomDevice &out,
                      std::string &err)
{
    static bool tab_ready[64] = {false};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && !tab_ready[dev]) {
        if (cudaMemcpyToSymbol(c_tab, h_tab, sizeof(h_tab)) != cudaSuccess) {
            err = "cudaMemcpyToSymbol(c_tab)";
            return TB_ERR_CUDA;
        }
        tab_ready[dev] = true;
    }
    const double rc2 = rcut * rcut;
    double *xyz = nullptr;
    int32_t *sp = nullptr, *cnt = nullptr, *derr = nullptr;
    auto cleanup = [&]() {
        cudaFree(xyz);
        cudaFree(sp);
        cudaFree(cnt);
        cudaFree(derr);
    };
    if (cudaMalloc(&xyz, sizeof(double) * 3 * natoms) || cudaMalloc(&sp, sizeof(int32_t) * natoms) ||
        cudaMalloc(&cnt, sizeof(int32_t) * natoms) || cudaMalloc(&derr, sizeof(int32_t))) {
        cleanup();
        err = "cudaMalloc(geometry)";
        return TB_ERR_OUT_OF_MEMORY;
    }
    cudaMemcpyAsync(xyz, xyz_h, sizeof(double) * 3 * natoms, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(sp, sp_h, sizeof(int32_t) * natoms, cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(derr, 0, sizeof(int32_t), st);
    const int T = 128, grid = (natoms + T - 1) / T;
    k_geo_count<<<grid, T, 0, st>>>(natoms, xyz, box[0], box[1], box[2], rc2, cnt);
    std::vector<int32_t> c(natoms);
    cudaMemcpyAsync(c.data(), cnt, sizeof(int32_t) * natoms, cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) {
        cleanup();
        err = "geometry count kernel failed";
        return TB_ERR_CUDA;
    }
    out.brow.assign(natoms + 1, 0);
    for (int i = 0; i < natoms; i++) out.brow[i + 1] = out.brow[i] + c[i];
    const int64_t nnzb = out.brow[natoms];
    out.nnzb = nnzb;
    if (cudaMalloc(&out.rowptr, sizeof(int32_t) * (natoms + 1)) ||
        cudaMalloc(&out.colidx, sizeof(int32_t) * nnzb) || cudaMalloc(&out.blkrow, sizeof(int32_t) * nnzb) ||
        cudaMalloc(&out.diagblk, sizeof(int32_t) * natoms) || cudaMalloc(&out.h0, sizeof(double) * 16 * nnzb) ||
        cudaMalloc(&out.h0diag, sizeof(double) * 4 * natoms) ||
        cudaMalloc(&out.radius, sizeof(double) * 4 * natoms) || cudaMalloc(&out.gval, sizeof(double) * nnzb) ||
        cudaMalloc(&out.q0, sizeof(double) * natoms)) {
        cleanup();
        err = "cudaMalloc(geometry outputs)";
        return TB_ERR_OUT_OF_MEMORY;
    }
    cudaMemcpyAsync(out.rowptr, out.brow.data(), sizeof(int32_t) * (natoms + 1), cudaMemcpyHostToDevice, st);
    k_geo_fill<<<grid, T, 0, st>>>(natoms, xyz, box[0], box[1], box[2], rc2, out.rowptr, out.colidx, out.blkrow);
    k_geo_blocks<<<(unsigned)((nnzb + T - 1) / T), T, 0, st>>>(nnzb, xyz, sp, box[0], box[1], box[2], out.colidx,
                                                               out.blkrow, gamma_diag, out.h0, out.gval, derr);
    k_geo_rowstats<<<(4 * natoms + T - 1) / T, T, 0, st>>>(natoms, out.rowptr, out.colidx, out.h0, out.h0diag,
                                                           out.radius, out.diagblk);
    std::vector<double> q0(natoms);
    for (int i = 0; i < natoms; i++) q0[i] = sp_h[i] == 14 ? 4.0 : 6.0;
    cudaMemcpyAsync(out.q0, q0.data(), sizeof(double) * natoms, cudaMemcpyHostToDevice, st);
    out.bcol.assign(nnzb, 0);
    out.h0diag_h.assign(4 * natoms, 0.0);
    out.radius_h.assign(4 * natoms, 0.0);
    int32_t herr = 0;
    cudaMemcpyAsync(out.bcol.data(), out.colidx, sizeof(int32_t) * nnzb, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(out.h0diag_h.data(), out.h0diag, sizeof(double) * 4 * natoms, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(out.radius_h.data(), out.radius, sizeof(double) * 4 * natoms, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&herr, derr, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    cleanup();
    if (e != cudaSuccess) {
        err = std::string("geometry kernels: ") + cudaGetErrorString(e);
        return TB_ERR_CUDA;
    }
    if (herr) {
        err = "unknown species or coincident atoms in the geometry";
        return TB_ERR_STRUCTURE;
    }
    return TB_OK;
}

}  // namespace tb

// Stabilized incompressible fluid MPM: one Newton system of
// StabilizedMPM::SolveNS (module/fluid/MPM/solve_ns_mpm.cpp:28-62) on the GPU.
//
//   MakNSStabCoeff (VMS)       solve_ns_mpm.cpp:64-135           -> k_ns_assemble (per particle, first part)
//   PredictNewmarkBetaVelAndAccel  nonlinear_time_integration.cpp:58-70 -> folded into the gathers
//   ImplicitDsfCorr            material_point.cpp:127-172        -> k_ns_assemble
//   AssembleNSSystem           solve_ns_mpm.cpp:137-320          -> k_ns_assemble (64 ordered node pairs)
//   AddInertialForceToRHS      material_point.h:74-85            -> k_ns_inertia
//
// Layout: the 4x4 (u, v, w, p) blocks of the 27-point stencil are stored as
// [27 slots][16 entries][nodec] FP64, entry k = row_var * 4 + col_var (the
// block_id order of CrsMat, module/solver/crsmat.cpp:73-75); slot
// s = (dx+1) + 3(dy+1) + 9(dz+1) of the column node's offset from the row
// node.  The right-hand side is component-major [4][nodec].  Linear shape
// functions only (idimc = 1, the order every fluid deck of the reference uses).
#include <cuda_runtime.h>

#include <cstdio>

#include "mpm_device.cuh"

using namespace mpm;

namespace {

struct NsArgs {
    KGeom<double> g;
    double rho, rmu, dti, nb[6], f[3], mtol, he0;
    int64_t n;
};

// Linear weights and gradients of the 8 nodes of cell (cx, cy, cz) at x,
// node q = i + 2j + 4k at (cx + i, cy + j, cz + k) (module/shape_function.cpp:28-110).
__device__ __forceinline__ void shape8(const KGeom<double> &g, const double *x, int cx, int cy, int cz, double *N,
                                       double (*dN)[3], int *nid) {
    Axis<double, 1> ax, ay, az;
    axis_linear<double>(x[0], g.xmin[0], g.dx[0], g.inv_dx[0], cx, ax);
    axis_linear<double>(x[1], g.xmin[1], g.dx[1], g.inv_dx[1], cy, ay);
    axis_linear<double>(x[2], g.xmin[2], g.dx[2], g.inv_dx[2], cz, az);
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const int i = q & 1, j = (q >> 1) & 1, k = q >> 2;
        N[q] = ax.w[i] * ay.w[j] * az.w[k];
        dN[q][0] = ax.dw[i] * ay.w[j] * az.w[k];
        dN[q][1] = ax.w[i] * ay.dw[j] * az.w[k];
        dN[q][2] = ax.w[i] * ay.w[j] * az.dw[k];
        nid[q] = (cx + i) + g.nnc[0] * ((cy + j) + g.nnc[1] * (cz + k));
    }
}

// One thread per particle: VMS coefficients from the element-centre velocity,
// then the particle's 8 x 8 node-pair blocks and its RHS rows, added into the
// stencil and b with FP64 atomics.  Points outside the grid set *bad.
__global__ void __launch_bounds__(128) k_ns_assemble(NsArgs a, const double *__restrict__ xs,
                                                     const double *__restrict__ mass, const double *__restrict__ vol,
                                                     const double *__restrict__ nvel, const double *__restrict__ naccel,
                                                     const double *__restrict__ ndispl,
                                                     const double *__restrict__ npres, double *__restrict__ tau1o,
                                                     double *__restrict__ tau2o, double *A, double *b, int *bad) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n) return;
    const size_t N = (size_t)a.g.nodec;
    const double x[3] = {xs[p], xs[a.n + p], xs[2 * a.n + p]};
    bool oob = false;
    const int cx = cell_of(x[0], a.g, 0, oob), cy = cell_of(x[1], a.g, 1, oob), cz = cell_of(x[2], a.g, 2, oob);
    if (oob) {
        atomicExch(bad, 1);
        return;
    }
    double Nw[8], dN[8][3];
    int nid[8];
    // ---- MakNSStabCoeff: velocity at the element centre (solve_ns_mpm.cpp:79-104)
    {
        const double xc[3] = {a.g.xmin[0] + a.g.dx[0] * ((double)cx + 0.5), a.g.xmin[1] + a.g.dx[1] * ((double)cy + 0.5),
                              a.g.xmin[2] + a.g.dx[2] * ((double)cz + 0.5)};
        shape8(a.g, xc, cx, cy, cz, Nw, dN, nid);
    }
    double uc[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int q = 0; q < 8; q++)
#pragma unroll
        for (int r = 0; r < 3; r++) uc[r] += Nw[q] * nvel[r * N + nid[q]];
    const double uvw = uc[0] * uc[0] + uc[1] * uc[1] + uc[2] * uc[2];
    double udsf = 0.0;
#pragma unroll
    for (int q = 0; q < 8; q++) udsf += fabs(uc[0] * dN[q][0] + uc[1] * dN[q][1] + uc[2] * dN[q][2]);
    const double he = udsf < a.mtol ? a.he0 : 2.0 * sqrt(uvw) / udsf;
    const double t1 = 1.0 / (a.rho * a.dti + 2.0 * a.rho * sqrt(uvw) / he + 4.0 * a.rmu / (he * he));
    const double t2 = (he * he) / (4.0 * t1);
    tau1o[p] = t1;
    tau2o[p] = t2;
    // ---- AssembleNSSystem (solve_ns_mpm.cpp:159-318)
    shape8(a.g, x, cx, cy, cz, Nw, dN, nid);
    double d[3][3] = {{1.0, 0.0, 0.0}, {0.0, 1.0, 0.0}, {0.0, 0.0, 1.0}};
#pragma unroll
    for (int q = 0; q < 8; q++)
#pragma unroll
        for (int r = 0; r < 3; r++) {
            const double u = ndispl[r * N + nid[q]];
#pragma unroll
            for (int c = 0; c < 3; c++) d[r][c] += dN[q][c] * u;
        }
    {   // ImplicitDsfCorr: dN <- dN (I + grad u)^-1
        const double id = 1.0 / det3(d);
        double di[3][3];
        di[0][0] = (d[1][1] * d[2][2] - d[1][2] * d[2][1]) * id;
        di[0][1] = (d[0][2] * d[2][1] - d[0][1] * d[2][2]) * id;
        di[0][2] = (d[0][1] * d[1][2] - d[0][2] * d[1][1]) * id;
        di[1][0] = (d[1][2] * d[2][0] - d[1][0] * d[2][2]) * id;
        di[1][1] = (d[0][0] * d[2][2] - d[0][2] * d[2][0]) * id;
        di[1][2] = (d[0][2] * d[1][0] - d[0][0] * d[1][2]) * id;
        di[2][0] = (d[1][0] * d[2][1] - d[1][1] * d[2][0]) * id;
        di[2][1] = (d[0][1] * d[2][0] - d[0][0] * d[2][1]) * id;
        di[2][2] = (d[0][0] * d[1][1] - d[0][1] * d[1][0]) * id;
#pragma unroll
        for (int q = 0; q < 8; q++) {
            double t[3];
#pragma unroll
            for (int c = 0; c < 3; c++) t[c] = dN[q][0] * di[0][c] + dN[q][1] * di[1][c] + dN[q][2] * di[2][c];
#pragma unroll
            for (int c = 0; c < 3; c++) dN[q][c] = t[c];
        }
    }
    // Newton-state gathers; nvel_k / naccel_k of the Newmark predictor are formed per node
    double pres = 0.0, acc[3] = {0.0, 0.0, 0.0}, gp[3] = {0.0, 0.0, 0.0};
    double gv[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const int n = nid[q];
        const double pn = npres[n];
        pres += Nw[q] * pn;
#pragma unroll
        for (int c = 0; c < 3; c++) gp[c] += dN[q][c] * pn;
#pragma unroll
        for (int r = 0; r < 3; r++) {
            const double u = ndispl[r * N + n], v = nvel[r * N + n], w = naccel[r * N + n];
            const double vk = a.nb[0] * u - a.nb[1] * v - a.nb[2] * w;
            const double ak = a.nb[3] * u - a.nb[4] * v - a.nb[5] * w;
            acc[r] += Nw[q] * ak;
#pragma unroll
            for (int c = 0; c < 3; c++) gv[r][c] += dN[q][c] * vk;
        }
    }
    const double V = vol[p], m = mass[p];
    const double divv = gv[0][0] + gv[1][1] + gv[2][2];
    const double vmu = V * a.rmu, vt2 = V * t2, mt1 = a.nb[3] * m * t1;
#pragma unroll 1
    for (int qa = 0; qa < 8; qa++) {
        const int na = nid[qa];
        const double ai[3] = {dN[qa][0], dN[qa][1], dN[qa][2]};
        const double Ni = Nw[qa];
        const double emd = a.nb[3] * Ni * m;   // ComputeNRLumpedMat
#pragma unroll 1
        for (int qb = 0; qb < 8; qb++) {
            const double bj[3] = {dN[qb][0], dN[qb][1], dN[qb][2]};
            const double Nj = Nw[qb];
            const int s = ((qb & 1) - (qa & 1) + 1) + 3 * (((qb >> 1) & 1) - ((qa >> 1) & 1) + 1) +
                          9 * ((qb >> 2) - (qa >> 2) + 1);
            const double ab = ai[0] * bj[0] + ai[1] * bj[1] + ai[2] * bj[2];
            double K[16];
#pragma unroll
            for (int r = 0; r < 3; r++) {
#pragma unroll
                for (int c = 0; c < 3; c++)
                    K[4 * r + c] = a.nb[0] * (vmu * (ai[c] * bj[r] + (r == c ? ab : 0.0)) + vt2 * ai[r] * bj[c]);
                K[4 * r + 3] = -V * ai[r] * Nj;
                K[12 + r] = a.nb[0] * V * Ni * bj[r] + mt1 * ai[r] * Nj;
            }
            K[15] = V * t1 * ab;
            if (qa == qb) {
                K[0] += emd;
                K[5] += emd;
                K[10] += emd;
            }
            double *row = A + (size_t)s * 16 * N + na;
#pragma unroll
            for (int k = 0; k < 16; k++) atomicAdd(row + (size_t)k * N, K[k]);
        }
        double rg[4];
#pragma unroll
        for (int r = 0; r < 3; r++) {
            const double dev = a.rmu * (ai[0] * (gv[r][0] + gv[0][r]) + ai[1] * (gv[r][1] + gv[1][r]) +
                                        ai[2] * (gv[r][2] + gv[2][r]));
            rg[r] = V * dev - Ni * m * a.f[r] - V * ai[r] * pres + vt2 * ai[r] * divv;
        }
        rg[3] = V * Ni * divv +
                t1 * m * (ai[0] * (acc[0] - a.f[0]) + ai[1] * (acc[1] - a.f[1]) + ai[2] * (acc[2] - a.f[2])) +
                t1 * V * (ai[0] * gp[0] + ai[1] * gp[1] + ai[2] * gp[2]);
#pragma unroll
        for (int r = 0; r < 4; r++) atomicAdd(b + r * N + na, -rg[r]);
    }
}

// AddInertialForceToRHS with the predicted acceleration (material_point.h:74-85)
__global__ void k_ns_inertia(NsArgs a, const double *__restrict__ nvel, const double *__restrict__ naccel,
                             const double *__restrict__ ndispl, const double *__restrict__ nmass, double *b) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= a.g.nodec) return;
    const size_t N = (size_t)a.g.nodec;
#pragma unroll
    for (int r = 0; r < 3; r++) {
        const double ak = a.nb[3] * ndispl[r * N + n] - a.nb[4] * nvel[r * N + n] - a.nb[5] * naccel[r * N + n];
        b[r * N + n] -= nmass[n] * ak;
    }
}

}  // namespace

extern "C" mpm_status mpm_gpu_ns_assemble(const mpm_grid_desc *grid, const mpm_ns_params *prm, int64_t n,
                                          const double *x, const double *mass, const double *vol, const double *nvel,
                                          const double *naccel, const double *ndispl, const double *npres,
                                          const double *nmass, double *tau1, double *tau2, double *stencil,
                                          double *b_rhs, int *status, void *stream) {
    if (!grid || !prm || n < 0 || !status || !stencil || !b_rhs || !nvel || !naccel || !ndispl || !npres || !nmass)
        return MPM_ERR_BAD_ARG;
    if (n > 0 && (!x || !mass || !vol || !tau1 || !tau2)) return MPM_ERR_BAD_ARG;
    NsArgs a;
    memset(&a, 0, sizeof(a));
    int64_t nodec = 1;
    for (int d = 0; d < 3; d++) {
        if (grid->idimc[d] != 1 || grid->xyelem[d] < 1 || !(grid->dxy[d] > 0.0)) return MPM_ERR_BAD_ARG;
        a.g.xmin[d] = grid->xymin[d];
        a.g.dx[d] = grid->dxy[d];
        a.g.inv_dx[d] = 1.0 / grid->dxy[d];
        a.g.nel[d] = grid->xyelem[d];
        a.g.nnc[d] = grid->xyelem[d] + 1;
        nodec *= a.g.nnc[d];
    }
    if (nodec > (int64_t)INT32_MAX / 27 || !(prm->dt > 0.0) || !(prm->beta_nb > 0.0)) return MPM_ERR_BAD_ARG;
    a.g.nodec = (int)nodec;
    a.rho = prm->rho;
    a.rmu = prm->rmu;
    a.dti = 1.0 / prm->dt;
    const double dt = prm->dt, be = prm->beta_nb, ga = prm->gamma_nb;
    a.nb[0] = ga / (be * dt);   // NewmarkBetaParaSet (nonlinear_time_integration.cpp:42-56)
    a.nb[1] = ga / be - 1.0;
    a.nb[2] = dt / 2.0 * (ga / be - 2.0);
    a.nb[3] = 1.0 / (be * dt * dt);
    a.nb[4] = 1.0 / (be * dt);
    a.nb[5] = 1.0 / (2.0 * be) - 1.0;
    for (int d = 0; d < 3; d++) a.f[d] = prm->gravity[d] * prm->facl;
    a.mtol = prm->mtol;
    a.he0 = grid->dxy[0] * cbrt(6.0 / M_PI);
    a.n = n;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(stencil, 0, sizeof(double) * 27 * 16 * (size_t)nodec, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b_rhs, 0, sizeof(double) * 4 * (size_t)nodec, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(status, 0, sizeof(int), st);
    if (e != cudaSuccess) return MPM_ERR_CUDA;
    if (n > 0)
        k_ns_assemble<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(a, x, mass, vol, nvel, naccel, ndispl, npres, tau1,
                                                                    tau2, stencil, b_rhs, status);
    k_ns_inertia<<<(unsigned)((nodec + 255) / 256), 256, 0, st>>>(a, nvel, naccel, ndispl, nmass, b_rhs);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        fprintf(stderr, "mpm_gpu_ns_assemble: %s\n", cudaGetErrorString(e));
        return MPM_ERR_CUDA;
    }
    return MPM_OK;
}

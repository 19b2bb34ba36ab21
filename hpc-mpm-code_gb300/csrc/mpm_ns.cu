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

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

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
    // the velocity block of the pair (a, b) is the transpose of that of (b, a)
    // and K_33 is symmetric, so each unordered pair is formed once:
    //   K_rc = nb0 vmu (a_c b_r + (a.b) d_rc) + nb0 vt2 a_r b_c,  K_r3 = -V a_r N_j,
    //   K_3c = nb0 V N_i b_c + mt1 a_c N_j,  K_33 = V t1 (a.b)
    // (a the row node's corrected gradient, b the column node's)
    const double kv = a.nb[0] * vmu, kt = a.nb[0] * vt2, kc = a.nb[0] * V, vt1 = V * t1;
#pragma unroll 1
    for (int qa = 0; qa < 8; qa++) {
        const int na = nid[qa];
        const double ai[3] = {dN[qa][0], dN[qa][1], dN[qa][2]};
        const double Ni = Nw[qa];
        const double emd = a.nb[3] * Ni * m;   // ComputeNRLumpedMat
        double A1[3], A2[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            A1[c] = kv * ai[c];
            A2[c] = kt * ai[c];
        }
        const double c1a = kc * Ni, mNi = mt1 * Ni, vNi = -V * Ni;
#pragma unroll 1
        for (int qb = qa; qb < 8; qb++) {
            const double bj[3] = {dN[qb][0], dN[qb][1], dN[qb][2]};
            const double Nj = Nw[qb];
            const int s = ((qb & 1) - (qa & 1) + 1) + 3 * (((qb >> 1) & 1) - ((qa >> 1) & 1) + 1) +
                          9 * ((qb >> 2) - (qa >> 2) + 1);
            const double ab = fma(ai[0], bj[0], fma(ai[1], bj[1], ai[2] * bj[2]));
            const double ab1 = kv * ab, k33 = vt1 * ab;
            double Vb[3][3];   // velocity block of row a, column b
#pragma unroll
            for (int r = 0; r < 3; r++)
#pragma unroll
                for (int c = 0; c < 3; c++) Vb[r][c] = fma(A1[c], bj[r], A2[r] * bj[c]) + (r == c ? ab1 : 0.0);
            const double Pj = -V * Nj, mNj = mt1 * Nj;
            {   // row a, column b
                double *row = A + (size_t)s * 16 * N + na;
#pragma unroll
                for (int r = 0; r < 3; r++) {
#pragma unroll
                    for (int c = 0; c < 3; c++)
                        atomicAdd(row + (size_t)(4 * r + c) * N, Vb[r][c] + (qa == qb && r == c ? emd : 0.0));
                    atomicAdd(row + (size_t)(4 * r + 3) * N, Pj * ai[r]);
                    atomicAdd(row + (size_t)(12 + r) * N, fma(c1a, bj[r], mNj * ai[r]));
                }
                atomicAdd(row + (size_t)15 * N, k33);
            }
            if (qb != qa) {   // row b, column a: the transposed velocity block
                double *row = A + (size_t)(26 - s) * 16 * N + nid[qb];
                const double c1b = kc * Nj;
#pragma unroll
                for (int r = 0; r < 3; r++) {
#pragma unroll
                    for (int c = 0; c < 3; c++) atomicAdd(row + (size_t)(4 * r + c) * N, Vb[c][r]);
                    atomicAdd(row + (size_t)(4 * r + 3) * N, vNi * bj[r]);
                    atomicAdd(row + (size_t)(12 + r) * N, fma(c1b, ai[r], mNi * bj[r]));
                }
                atomicAdd(row + (size_t)15 * N, k33);
            }
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

// NsArgs of a grid and the fluid constants; false for an unusable grid
static bool ns_args(const mpm_grid_desc *grid, const mpm_ns_params *prm, int64_t n, NsArgs &a) {
    memset(&a, 0, sizeof(a));
    int64_t nodec = 1;
    for (int d = 0; d < 3; d++) {
        if (grid->idimc[d] != 1 || grid->xyelem[d] < 1 || !(grid->dxy[d] > 0.0)) return false;
        a.g.xmin[d] = grid->xymin[d];
        a.g.dx[d] = grid->dxy[d];
        a.g.inv_dx[d] = 1.0 / grid->dxy[d];
        a.g.nel[d] = grid->xyelem[d];
        a.g.nnc[d] = grid->xyelem[d] + 1;
        nodec *= a.g.nnc[d];
    }
    if (nodec > (int64_t)INT32_MAX / 27 || !(prm->dt > 0.0) || !(prm->beta_nb > 0.0)) return false;
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
    return true;
}

// The system of one Newton iteration into stencil / b_rhs (cleared first) on `st`.
static cudaError_t ns_assemble_launch(const NsArgs &a, const double *x, const double *mass, const double *vol,
                                      const double *nvel, const double *naccel, const double *ndispl,
                                      const double *npres, const double *nmass, double *tau1, double *tau2,
                                      double *stencil, double *b_rhs, int *status, cudaStream_t st) {
    const size_t nodec = (size_t)a.g.nodec;
    cudaError_t e = cudaMemsetAsync(stencil, 0, sizeof(double) * 27 * 16 * nodec, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b_rhs, 0, sizeof(double) * 4 * nodec, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(status, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    if (a.n > 0)
        k_ns_assemble<<<(unsigned)((a.n + 127) / 128), 128, 0, st>>>(a, x, mass, vol, nvel, naccel, ndispl, npres,
                                                                      tau1, tau2, stencil, b_rhs, status);
    k_ns_inertia<<<(unsigned)((nodec + 255) / 256), 256, 0, st>>>(a, nvel, naccel, ndispl, nmass, b_rhs);
    return cudaGetLastError();
}

extern "C" mpm_status mpm_gpu_ns_assemble(const mpm_grid_desc *grid, const mpm_ns_params *prm, int64_t n,
                                          const double *x, const double *mass, const double *vol, const double *nvel,
                                          const double *naccel, const double *ndispl, const double *npres,
                                          const double *nmass, double *tau1, double *tau2, double *stencil,
                                          double *b_rhs, int *status, void *stream) {
    if (!grid || !prm || n < 0 || !status || !stencil || !b_rhs || !nvel || !naccel || !ndispl || !npres || !nmass)
        return MPM_ERR_BAD_ARG;
    if (n > 0 && (!x || !mass || !vol || !tau1 || !tau2)) return MPM_ERR_BAD_ARG;
    NsArgs a;
    if (!ns_args(grid, prm, n, a)) return MPM_ERR_BAD_ARG;
    const cudaError_t e = ns_assemble_launch(a, x, mass, vol, nvel, naccel, ndispl, npres, nmass, tau1, tau2, stencil,
                                             b_rhs, status, (cudaStream_t)stream);
    if (e != cudaSuccess) {
        fprintf(stderr, "mpm_gpu_ns_assemble: %s\n", cudaGetErrorString(e));
        return MPM_ERR_CUDA;
    }
    return MPM_OK;
}

// ===================================================================== SolveNS
// The Newton loop of StabilizedMPM::SolveNS (solve_ns_mpm.cpp:28-62) with the
// reference's native solver path (use_petsc off): per Newton iteration
// BCNRSet, the system (k_ns_assemble / k_ns_inertia), BuildDiagonalPreconditioner
// for 4 degrees of freedom (crsmat.cpp:87-184), GPBiCGSafe on the scaled system
// (solver.cpp:19-141) restated with device-side reductions, UpdateNRIncrement
// and CheckNRConvergence (solver.cpp:484-593).  Vectors are component-major
// [u | v | w | p] of nodec each.
namespace {

enum NsScal {
    NS_RTR = 0, NS_RSR, NS_RSR0, NS_BTB, NS_BETA, NS_ALPH, NS_ZETA, NS_ETA, NS_DONE, NS_ITER, NS_RES, NS_IDOF,
    NS_EU, NS_GD, NS_NSCAL
};

struct NsVec {
    double *rr, *rs, *pp, *Ap, *Ar, *Az, *Au, *uu, *zz, *xs, *Ax;
};

// Sums of V per-thread values over the grid: block partials in part[v * gridDim.x + b];
// the last block to finish adds them in block order (run-to-run identical) and returns true.
template <int V>
__device__ bool ns_reduce(double (&v)[V], double *part, unsigned *cnt, double (&tot)[V]) {
    __shared__ double sh[V][8];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < V; j++) {
        double t = v[j];
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (lane == 0) sh[j][wid] = t;
    }
    __syncthreads();
    if ((int)threadIdx.x < V) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[threadIdx.x][w];
        part[threadIdx.x * gridDim.x + blockIdx.x] = t;
        __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(cnt, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return false;
    __threadfence();
    if ((int)threadIdx.x < V) {
        double t = 0.0;
        for (unsigned b = 0; b < gridDim.x; b++) t += __ldcg(part + threadIdx.x * gridDim.x + b);
        sh[threadIdx.x][0] = t;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < V; j++) tot[j] = sh[j][0];
    if (threadIdx.x == 0) *cnt = 0u;
    return true;
}

// D^-1/2 of the four diagonal entries of every node (ExtractDiagonal + ComputeDiagonalInverseSqrt)
__global__ void k_nsv_diag(int nodec, double mtol, const double *A, double *adiag) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nodec) return;
    const size_t N = (size_t)nodec;
    for (int m = 0; m < 4; m++) {
        const double d = fabs(A[(size_t)(13 * 16 + 5 * m) * N + n]);
        adiag[m * N + n] = d < mtol ? 0.0 : 1.0 / sqrt(d);
    }
}

// ApplyDiagonalScaling: A_ij <- D_i A_ij D_j
__global__ void k_nsv_scale_mat(KGeom<double> g, double *A, const double *adiag) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.nodec) return;
    const size_t N = (size_t)g.nodec;
    const int i = n % g.nnc[0], j = (n / g.nnc[0]) % g.nnc[1], k = n / (g.nnc[0] * g.nnc[1]);
    for (int s = 0; s < 27; s++) {
        const int ii = i + s % 3 - 1, jj = j + (s / 3) % 3 - 1, kk = k + s / 9 - 1;
        if (ii < 0 || jj < 0 || kk < 0 || ii >= g.nnc[0] || jj >= g.nnc[1] || kk >= g.nnc[2]) continue;
        const size_t col = ii + (size_t)g.nnc[0] * (jj + (size_t)g.nnc[1] * kk);
        for (int r = 0; r < 4; r++)
            for (int c = 0; c < 4; c++) A[(size_t)(s * 16 + 4 * r + c) * N + n] *= adiag[r * N + n] * adiag[c * N + col];
    }
}

// y = A x with the BC rows zeroed (MatVecMult + BCResidualSet)
__global__ void __launch_bounds__(256) k_nsv_matvec(KGeom<double> g, const double *__restrict__ A,
                                                    const unsigned char *__restrict__ bcf, const double *x, double *y,
                                                    const double *done) {
    if (done && *done != 0.0) return;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.nodec) return;
    const size_t N = (size_t)g.nodec;
    const int i = n % g.nnc[0], j = (n / g.nnc[0]) % g.nnc[1], k = n / (g.nnc[0] * g.nnc[1]);
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int s = 0; s < 27; s++) {
        const int ii = i + s % 3 - 1, jj = j + (s / 3) % 3 - 1, kk = k + s / 9 - 1;
        if (ii < 0 || jj < 0 || kk < 0 || ii >= g.nnc[0] || jj >= g.nnc[1] || kk >= g.nnc[2]) continue;
        const size_t col = ii + (size_t)g.nnc[0] * (jj + (size_t)g.nnc[1] * kk);
        const double xc[4] = {x[col], x[N + col], x[2 * N + col], x[3 * N + col]};
#pragma unroll
        for (int r = 0; r < 4; r++)
#pragma unroll
            for (int c = 0; c < 4; c++) acc[r] = fma(__ldg(A + (size_t)(s * 16 + 4 * r + c) * N + n), xc[c], acc[r]);
    }
    const unsigned char f = bcf[n];
#pragma unroll
    for (int r = 0; r < 4; r++) y[r * N + n] = (f >> r) & 1 ? 0.0 : acc[r];
}

// ScaleSolution + BCResidualSet: xs = x / D, rr = b D (zero where D < mtol and on BC rows)
__global__ void k_nsv_scale_in(int nodec, double mtol, const unsigned char *bcf, const double *x, const double *b,
                               const double *adiag, double *xs, double *rr) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nodec) return;
    const size_t N = (size_t)nodec;
    const unsigned char f = bcf[n];
    for (int m = 0; m < 4; m++) {
        const size_t i = m * N + n;
        const double d = adiag[i];
        xs[i] = d < mtol ? 0.0 : x[i] / d;
        rr[i] = (d < mtol || ((f >> m) & 1)) ? 0.0 : b[i] * d;
    }
}

// rr = rr - Ax, rs = rr, the other GPBiCGSafe vectors zero; rtr (= rsr = btb), beta = 0
__global__ void __launch_bounds__(256) k_nsv_init(int nodec, NsVec v, double *part, unsigned *cnt, double *scal) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    double d[1] = {0.0};
    if (n < nodec) {
        const size_t N = (size_t)nodec;
        for (int m = 0; m < 4; m++) {
            const size_t i = m * N + n;
            const double r = v.rr[i] - v.Ax[i];
            v.rr[i] = r;
            v.rs[i] = r;
            v.pp[i] = v.Ap[i] = v.Au[i] = v.Az[i] = v.uu[i] = v.zz[i] = 0.0;
            d[0] += r * r;
        }
    }
    double t[1];
    if (!ns_reduce<1>(d, part, cnt, t)) return;
    if (threadIdx.x == 0) {
        scal[NS_RTR] = scal[NS_RSR] = scal[NS_BTB] = t[0];
        scal[NS_BETA] = 0.0;
        scal[NS_ITER] = 0.0;
        scal[NS_DONE] = 0.0;
    }
}

// pp = rr + beta (pp - uu), Ap = Ar + beta (Ap - Au); the six dots; then alpha, zeta, eta
__global__ void __launch_bounds__(256) k_gpb_1(int nodec, NsVec v, double *part, unsigned *cnt, double *scal) {
    if (scal[NS_DONE] != 0.0) return;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const double beta = scal[NS_BETA];
    double d[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    if (n < nodec) {
        const size_t N = (size_t)nodec;
        for (int m = 0; m < 4; m++) {
            const size_t i = m * N + n;
            const double p = v.rr[i] + beta * (v.pp[i] - v.uu[i]);
            const double ap = v.Ar[i] + beta * (v.Ap[i] - v.Au[i]);
            v.pp[i] = p;
            v.Ap[i] = ap;
            const double az = v.Az[i], ar = v.Ar[i], r = v.rr[i];
            d[0] += v.rs[i] * ap;
            d[1] += az * az;
            d[2] += ar * r;
            d[3] += az * r;
            d[4] += ar * az;
            d[5] += ar * ar;
        }
    }
    double t[6];
    if (!ns_reduce<6>(d, part, cnt, t)) return;
    if (threadIdx.x == 0) {
        const double rAp = t[0], AzAz = t[1], Arrr = t[2], Azrr = t[3], ArAz = t[4], ArAr = t[5];
        scal[NS_RSR0] = scal[NS_RSR];
        scal[NS_ALPH] = scal[NS_RSR] / rAp;
        if (scal[NS_ITER] == 0.0) {
            scal[NS_ZETA] = Arrr / ArAr;
            scal[NS_ETA] = 0.0;
        } else {
            const double den = ArAr * AzAz - ArAz * ArAz;
            scal[NS_ZETA] = (AzAz * Arrr - Azrr * ArAz) / den;
            scal[NS_ETA] = (ArAr * Azrr - ArAz * Arrr) / den;
        }
    }
}

// uu = zeta Ap + eta (Az + beta uu)
__global__ void k_gpb_2(int nodec, NsVec v, const double *scal) {
    if (scal[NS_DONE] != 0.0) return;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nodec) return;
    const double zeta = scal[NS_ZETA], eta = scal[NS_ETA], beta = scal[NS_BETA];
    const size_t N = (size_t)nodec;
    for (int m = 0; m < 4; m++) {
        const size_t i = m * N + n;
        v.uu[i] = zeta * v.Ap[i] + eta * (v.Az[i] + beta * v.uu[i]);
    }
}

// tt = rr - alpha Ap; zz = zeta rr + eta zz - alpha uu; Az = zeta Ar + eta Az - alpha Au;
// x += alpha pp + zz; rr = tt - Az; then rsr, rtr, the stopping test rtr < eps btb and beta
__global__ void __launch_bounds__(256) k_gpb_3(int nodec, NsVec v, double eps, double *part, unsigned *cnt,
                                               double *scal) {
    if (scal[NS_DONE] != 0.0) return;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const double alph = scal[NS_ALPH], zeta = scal[NS_ZETA], eta = scal[NS_ETA];
    double d[2] = {0.0, 0.0};
    if (n < nodec) {
        const size_t N = (size_t)nodec;
        for (int m = 0; m < 4; m++) {
            const size_t i = m * N + n;
            const double r = v.rr[i];
            const double tt = r - alph * v.Ap[i];
            const double zz = zeta * r + eta * v.zz[i] - alph * v.uu[i];
            const double az = zeta * v.Ar[i] + eta * v.Az[i] - alph * v.Au[i];
            v.zz[i] = zz;
            v.Az[i] = az;
            v.xs[i] += alph * v.pp[i] + zz;
            const double rn = tt - az;
            v.rr[i] = rn;
            d[0] += v.rs[i] * rn;
            d[1] += rn * rn;
        }
    }
    double t[2];
    if (!ns_reduce<2>(d, part, cnt, t)) return;
    if (threadIdx.x == 0) {
        scal[NS_RSR] = t[0];
        scal[NS_RTR] = t[1];
        scal[NS_ITER] += 1.0;
        if (t[1] < eps * scal[NS_BTB]) scal[NS_DONE] = 1.0;
        else scal[NS_BETA] = (alph / zeta) * (t[0] / scal[NS_RSR0]);
    }
}

// RestorSolution: x = xs D (zero where D <= mtol)
__global__ void k_nsv_restore(int nodec, double mtol, const double *xs, const double *adiag, double *x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 4 * nodec) return;
    x[i] = adiag[i] > mtol ? xs[i] * adiag[i] : 0.0;
}

// x_pre = x / D for the physical residual (ComputeRefResidual)
__global__ void k_nsv_prep(int nodec, double mtol, const double *x, const double *adiag, double *xp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 4 * nodec) return;
    xp[i] = adiag[i] > mtol ? x[i] / adiag[i] : 0.0;
}

// r = b - (A x_pre) / D with b's BC rows zeroed: r.r and the active row count
__global__ void __launch_bounds__(256) k_nsv_resid(int nodec, double mtol, const unsigned char *bcf, const double *b,
                                                   const double *Ax, const double *adiag, double *part, unsigned *cnt,
                                                   double *scal) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    double d[2] = {0.0, 0.0};
    if (n < nodec) {
        const size_t N = (size_t)nodec;
        const unsigned char f = bcf[n];
        for (int m = 0; m < 4; m++) {
            const size_t i = m * N + n;
            const double bi = ((f >> m) & 1) ? 0.0 : b[i];
            const double ax = adiag[i] > mtol ? Ax[i] / adiag[i] : 0.0;
            const double r = bi - ax;
            d[0] += r * r;
            d[1] += adiag[i] > mtol ? 1.0 : 0.0;
        }
    }
    double t[2];
    if (!ns_reduce<2>(d, part, cnt, t)) return;
    if (threadIdx.x == 0) {
        scal[NS_RES] = t[0];
        scal[NS_IDOF] = t[1];
    }
}

// BCNRSet: ndispl = fbc dt facl on the u/v/w lists, npres = fbc facl on the p list
__global__ void k_nsv_bcnr(int nodec, const unsigned char *bcf, const double *bcv, double dt_facl, double facl,
                           double *ndispl, double *npres) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nodec) return;
    const size_t N = (size_t)nodec;
    const unsigned char f = bcf[n];
    for (int m = 0; m < 3; m++)
        if ((f >> m) & 1) ndispl[m * N + n] = bcv[m * N + n] * dt_facl;
    if ((f >> 3) & 1) npres[n] = bcv[3 * N + n] * facl;
}

// UpdateNRIncrement: ndispl += x[0..3N), npres += x[3N..4N)
__global__ void k_nsv_update(int nodec, const double *x, double *ndispl, double *npres) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 4 * nodec) return;
    if (i < 3 * nodec) ndispl[i] += x[i];
    else npres[i - 3 * nodec] += x[i];
}

// ================================================================ time step
// Particle2Node and Node2Particle of StabilizedMPM
// (module/fluid/MPM/var_trans_fluid.cpp:17-135) around the Newton loop, one
// thread per particle or node.  The P2G sums are int64 fixed point (scales
// 2^e from the step's bounds: exact, order-independent sums), the shifting
// sums reduce in block order: a step is run-to-run identical.
enum NsBound { NB_M = 0, NB_VOL, NB_MV, NB_MA, NB_N };
enum NsStatusBit { NS_OUTSIDE = 1, NS_NONFINITE = 2 };

struct NsStepArgs {
    KGeom<double> g;
    int64_t n;
    double mtol, facl, dt, gamma, nb[6];
    int flip;
};

__device__ __forceinline__ void ns_max(unsigned *slot, double v) {
    float f = (float)v * 1.000001f;   // bounds only: rounded up to a float
    if (!(f >= 0.0f)) f = INFINITY;
    atomicMax(slot, __float_as_uint(f));
}

// bounds of the P2G contributions (max m, vol, m |v|, m |a|); particles outside
// the grid or with non-finite inputs are reported and skipped by the scatter
__global__ void k_nsp_bounds(NsStepArgs a, const double *__restrict__ x, const double *__restrict__ vel,
                             const double *__restrict__ acc, const double *__restrict__ mass,
                             const double *__restrict__ vol, unsigned *bnd, int *status) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n) return;
    const int64_t n = a.n;
    const double m = mass[p], V = vol[p];
    double vm = 0.0, am = 0.0, sum = m + V;
    bool oob = false;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        vm = fmax(vm, fabs(vel[c * n + p]));
        am = fmax(am, fabs(acc[c * n + p]));
        sum += x[c * n + p] + vel[c * n + p] + acc[c * n + p];
        (void)cell_of(x[c * n + p], a.g, c, oob);
    }
    if (!isfinite(sum)) {
        atomicOr(status, NS_NONFINITE);
        return;
    }
    if (oob) {
        atomicOr(status, NS_OUTSIDE);
        return;
    }
    ns_max(bnd + NB_M, fabs(m));
    ns_max(bnd + NB_VOL, fabs(V));
    ns_max(bnd + NB_MV, fabs(m) * vm);
    ns_max(bnd + NB_MA, fabs(m) * am);
}

__device__ __forceinline__ void ns_scales(const NsStepArgs &a, const unsigned *bnd, Fix *F) {
    const double nump = (double)a.n;
#pragma unroll
    for (int k = 0; k < NB_N; k++) F[k] = make_fix(nump * (double)__uint_as_float(bnd[k]));
}

// StandardVarP2G (mass, vol), VelP2G, AccelP2G (material_point.h:223-247,
// module/map_and_interpolate.cpp:12-49) for PIC / FLIP: 8 int64 sums per node
__global__ void __launch_bounds__(128) k_nsp_scatter(NsStepArgs a, const double *__restrict__ x,
                                                     const double *__restrict__ vel, const double *__restrict__ acc,
                                                     const double *__restrict__ mass, const double *__restrict__ vol,
                                                     const unsigned *bnd, unsigned long long *sums) {
    __shared__ Fix F[NB_N];
    if (threadIdx.x == 0) ns_scales(a, bnd, F);
    __syncthreads();
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n) return;
    const int64_t n = a.n;
    const size_t N = (size_t)a.g.nodec;
    const double xp[3] = {x[p], x[n + p], x[2 * n + p]};
    const double m = mass[p], V = vol[p];
    const double v[3] = {vel[p], vel[n + p], vel[2 * n + p]}, ac[3] = {acc[p], acc[n + p], acc[2 * n + p]};
    bool oob = false;
    double sum = m + V;
    for (int c = 0; c < 3; c++) sum += xp[c] + v[c] + ac[c];
    const int cx = cell_of(xp[0], a.g, 0, oob), cy = cell_of(xp[1], a.g, 1, oob), cz = cell_of(xp[2], a.g, 2, oob);
    if (oob || !isfinite(sum)) return;   // reported by k_nsp_bounds
    double Nw[8], dN[8][3];
    int nid[8];
    shape8(a.g, xp, cx, cy, cz, Nw, dN, nid);
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const double nm = Nw[q] * m;
        long long o[8];
        o[0] = fx(nm, F[NB_M]);
        o[1] = fx(Nw[q] * V, F[NB_VOL]);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            o[2 + c] = fx(nm * v[c], F[NB_MV]);
            o[5 + c] = fx(nm * ac[c], F[NB_MA]);
        }
#pragma unroll
        for (int f = 0; f < 8; f++)
            if (o[f]) atomic_add_i64(sums + (size_t)f * N + nid[q], o[f]);
    }
}

// nmass, nvof, nvel = nmome / nmass, naccel = nforce / nmass (nmass > mtol), then
// BCSetVal (value facl) on nvel and BCSetZero on naccel for the u, v, w lists
// (var_trans_fluid.cpp:52-78)
__global__ void k_nsp_grid(NsStepArgs a, const unsigned long long *__restrict__ sums, const unsigned *bnd,
                           const unsigned char *__restrict__ bcf, const double *__restrict__ bcv, double *nmass,
                           double *nvof, double *nvel, double *naccel) {
    __shared__ Fix F[NB_N];
    if (threadIdx.x == 0) ns_scales(a, bnd, F);
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.g.nodec) return;
    const size_t N = (size_t)a.g.nodec;
    const double m = unfx((long long)sums[i], F[NB_M], 0.0);
    nmass[i] = m;
    nvof[i] = unfx((long long)sums[N + i], F[NB_VOL], 0.0);
    const unsigned char f = bcf[i];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        double v = 0.0, ac = 0.0;
        if (m > a.mtol) {
            v = unfx((long long)sums[(2 + c) * N + i], F[NB_MV], 0.0) / m;
            ac = unfx((long long)sums[(5 + c) * N + i], F[NB_MA], 0.0) / m;
        }
        if ((f >> c) & 1) {
            v = bcv[c * N + i] * a.facl;
            ac = 0.0;
        }
        nvel[c * N + i] = v;
        naccel[c * N + i] = ac;
    }
}

// PredictNewmarkBetaVelAndAccel + CommitNodalKinematics
// (nonlinear_time_integration.cpp:58-77) and the shifting's nei = max(0, nvof -
// nvol) with sum nei^2 (material_point.cpp:175-185) into scal[slot]
__global__ void __launch_bounds__(256) k_nsn_commit(NsStepArgs a, const double *__restrict__ ndispl,
                                                    const double *__restrict__ nvof, const double *__restrict__ nvol,
                                                    double *nvel, double *naccel, double *nei, double *part,
                                                    unsigned *cnt, double *scal, int slot) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double d[1] = {0.0};
    if (i < a.g.nodec) {
        const size_t N = (size_t)a.g.nodec;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const size_t k = c * N + i;
            const double u = ndispl[k], v = nvel[k], w = naccel[k];
            nvel[k] = a.nb[0] * u - a.nb[1] * v - a.nb[2] * w;
            naccel[k] = a.nb[3] * u - a.nb[4] * v - a.nb[5] * w;
        }
        const double e = fmax(0.0, -nvol[i] + nvof[i]);
        nei[i] = e;
        d[0] = e * e;
    }
    double t[1];
    if (ns_reduce<1>(d, part, cnt, t) && threadIdx.x == 0) scal[slot] = t[0];
}

// Node2Particle's gathers (var_trans_fluid.cpp:104-124): pressure, displacement,
// acceleration and (PIC) velocity; FLIP's velocity update and the
// displacement of CommitParticleKinematics (nonlinear_time_integration.cpp:79-96);
// the shifting gradient geup = 2 vol sum dN nei at the step's start position
// (material_point.cpp:187-213) and sum |geup|^2 into scal[slot]
__global__ void __launch_bounds__(256) k_nsp_g2p(NsStepArgs a, double *x, double *vel, double *acc, double *pres,
                                                 const double *__restrict__ vol, const double *__restrict__ nvel,
                                                 const double *__restrict__ naccel, const double *__restrict__ ndispl,
                                                 const double *__restrict__ npres, const double *__restrict__ nei,
                                                 double *geup, double *part, unsigned *cnt, double *scal, int slot) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double d[1] = {0.0};
    if (p < a.n) {
        const int64_t n = a.n;
        const size_t N = (size_t)a.g.nodec;
        const double xp[3] = {x[p], x[n + p], x[2 * n + p]};
        bool oob = false;
        const int cx = cell_of(xp[0], a.g, 0, oob), cy = cell_of(xp[1], a.g, 1, oob),
                  cz = cell_of(xp[2], a.g, 2, oob);
        double Nw[8], dN[8][3];
        int nid[8];
        shape8(a.g, xp, cx, cy, cz, Nw, dN, nid);
        double pr = 0.0, du[3] = {0.0, 0.0, 0.0}, an[3] = {0.0, 0.0, 0.0}, vn[3] = {0.0, 0.0, 0.0};
        double gu[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const int k = nid[q];
            const double w = Nw[q], e = nei[k];
            pr += w * npres[k];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                du[c] += w * ndispl[c * N + k];
                an[c] += w * naccel[c * N + k];
                vn[c] += w * nvel[c * N + k];
                gu[c] += dN[q][c] * e;
            }
        }
        const double tv = 2.0 * vol[p];
        pres[p] = pr;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const double aold = acc[c * n + p];
            vel[c * n + p] = a.flip ? vel[c * n + p] + a.dt * ((1.0 - a.gamma) * aold + a.gamma * an[c]) : vn[c];
            acc[c * n + p] = an[c];
            x[c * n + p] = xp[c] + du[c];
            const double g = gu[c] * tv;
            geup[c * n + p] = g;
            d[0] += g * g;
        }
    }
    double t[1];
    if (ns_reduce<1>(d, part, cnt, t) && threadIdx.x == 0) scal[slot] = t[0];
}

// x += -b0 geup, b0 = eu / gd unless gd < mtol (material_point.cpp:215-225)
__global__ void k_nsp_shift(NsStepArgs a, const double *__restrict__ geup, const double *__restrict__ scal, int eu,
                            int gd, double *x) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n) return;
    const double g = scal[gd];
    const double b0 = g < a.mtol ? 0.0 : scal[eu] / g;
    if (b0 == 0.0) return;
#pragma unroll
    for (int c = 0; c < 3; c++) x[c * a.n + p] += -b0 * geup[c * a.n + p];
}

}  // namespace

struct mpm_ns {
    mpm_grid_desc grid;
    mpm_ns_params prm;
    NsArgs a;
    cudaStream_t stream = nullptr;
    int nodec = 0;
    double *A = nullptr, *b = nullptr, *adiag = nullptr, *x = nullptr, *bcv = nullptr, *part = nullptr;
    double *scal = nullptr, *h_scal = nullptr;
    unsigned char *bcf = nullptr;
    unsigned *cnt = nullptr;
    int *status = nullptr;
    NsVec v{};
    std::vector<int> bc_nodes[4];
    std::vector<double> bc_vals[4];
    // time step (mpm_ns_step): nodal state, P2G sums and bounds, particle scratch
    double *nmass = nullptr, *nvof = nullptr, *nvel = nullptr, *naccel = nullptr, *ndispl = nullptr;
    double *npres = nullptr, *nvol = nullptr, *nei = nullptr;
    unsigned long long *sums = nullptr;
    unsigned *bnd = nullptr;
    double *tau1 = nullptr, *tau2 = nullptr, *geup = nullptr, *ppart = nullptr;
    int64_t pcap = 0;
    bool nvol_ready = false;   // MakNodalVol has run into nvol
    // particles held by the context (mpm_ns_load_particles): 12 SoA arrays of np
    double *pbuf = nullptr;
    int64_t np = 0;
    bool p2g_done = false;     // Particle2Node ran since the last Node2Particle
    int p2g_scheme = MPM_PIC;
};

#define CKN(call)                                                                                                      \
    do {                                                                                                               \
        cudaError_t _e = (call);                                                                                       \
        if (_e != cudaSuccess) {                                                                                       \
            fprintf(stderr, "mpm_gb300: %s failed: %s\n", #call, cudaGetErrorString(_e));                              \
            return _e == cudaErrorMemoryAllocation ? MPM_ERR_OOM : MPM_ERR_CUDA;                                       \
        }                                                                                                              \
    } while (0)

extern "C" void mpm_ns_destroy(mpm_ns *s) {
    if (!s) return;
    void *bufs[] = {s->A,     s->b,      s->adiag,  s->x,      s->bcv,    s->part, s->scal,  s->bcf,
                    s->cnt,   s->status, s->v.rr,   s->v.rs,   s->v.pp,   s->v.Ap, s->v.Ar,  s->v.Az,
                    s->v.Au,  s->v.uu,   s->v.zz,   s->v.xs,   s->v.Ax,   s->nmass, s->nvof, s->nvel,
                    s->naccel, s->ndispl, s->npres, s->nvol,   s->nei,    s->sums, s->bnd,   s->tau1,
                    s->tau2,  s->geup,   s->ppart,  s->pbuf};
    for (void *p : bufs)
        if (p) cudaFree(p);
    if (s->h_scal) cudaFreeHost(s->h_scal);
    delete s;
}

extern "C" mpm_status mpm_ns_create(const mpm_grid_desc *grid, const mpm_ns_params *prm, mpm_ns **out) {
    if (!grid || !prm || !out) return MPM_ERR_BAD_ARG;
    *out = nullptr;
    NsArgs a;
    if (!ns_args(grid, prm, 0, a)) return MPM_ERR_BAD_ARG;
    mpm_ns *s = new (std::nothrow) mpm_ns();
    if (!s) return MPM_ERR_OOM;
    s->grid = *grid;
    s->prm = *prm;
    s->a = a;
    s->nodec = a.g.nodec;
    const size_t N = (size_t)a.g.nodec;
    const int nb = (int)((N + 255) / 256);
    cudaError_t e = cudaSuccess;
    auto alloc = [&](void **p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes);
    };
    alloc((void **)&s->A, sizeof(double) * 27 * 16 * N);
    alloc((void **)&s->b, sizeof(double) * 4 * N);
    alloc((void **)&s->adiag, sizeof(double) * 4 * N);
    alloc((void **)&s->x, sizeof(double) * 4 * N);
    alloc((void **)&s->bcv, sizeof(double) * 4 * N);
    alloc((void **)&s->part, sizeof(double) * 8 * (size_t)nb);
    alloc((void **)&s->scal, sizeof(double) * NS_NSCAL);
    alloc((void **)&s->bcf, N);
    alloc((void **)&s->cnt, sizeof(unsigned) * 4);
    alloc((void **)&s->status, sizeof(int));
    double **vecs[] = {&s->v.rr, &s->v.rs, &s->v.pp, &s->v.Ap, &s->v.Ar, &s->v.Az,
                       &s->v.Au, &s->v.uu, &s->v.zz, &s->v.xs, &s->v.Ax};
    for (double **p : vecs) alloc((void **)p, sizeof(double) * 4 * N);
    if (e == cudaSuccess) e = cudaMallocHost((void **)&s->h_scal, sizeof(double) * NS_NSCAL);
    if (e == cudaSuccess) e = cudaMemset(s->cnt, 0, sizeof(unsigned) * 4);
    if (e == cudaSuccess) e = cudaMemset(s->bcf, 0, N);
    if (e == cudaSuccess) e = cudaMemset(s->bcv, 0, sizeof(double) * 4 * N);
    if (e == cudaSuccess) e = cudaMemset(s->scal, 0, sizeof(double) * NS_NSCAL);
    if (e != cudaSuccess) {
        mpm_ns_destroy(s);
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? MPM_ERR_OOM : MPM_ERR_CUDA;
    }
    *out = s;
    return MPM_OK;
}

extern "C" mpm_status mpm_ns_set_stream(mpm_ns *s, void *stream) {
    if (!s) return MPM_ERR_BAD_ARG;
    s->stream = (cudaStream_t)stream;
    return MPM_OK;
}

extern "C" mpm_status mpm_ns_set_bc(mpm_ns *s, int comp, int n, const int *nodes, const double *vals) {
    if (!s || comp < 0 || comp > 3 || n < 0 || (n > 0 && (!nodes || !vals))) return MPM_ERR_BAD_ARG;
    for (int i = 0; i < n; i++)
        if (nodes[i] < 0 || nodes[i] >= s->nodec) return MPM_ERR_BAD_ARG;
    s->bc_nodes[comp].assign(nodes, nodes + n);
    s->bc_vals[comp].assign(vals, vals + n);
    const size_t N = (size_t)s->nodec;
    std::vector<unsigned char> flag(N, 0);
    std::vector<double> val(4 * N, 0.0);
    for (int k = 0; k < 4; k++)
        for (size_t i = 0; i < s->bc_nodes[k].size(); i++) {   // later entries win, as the BC loops
            const int nd = s->bc_nodes[k][i];
            flag[nd] |= (unsigned char)(1 << k);
            val[k * N + nd] = s->bc_vals[k][i];
        }
    CKN(cudaStreamSynchronize(s->stream));
    CKN(cudaMemcpy(s->bcf, flag.data(), N, cudaMemcpyHostToDevice));
    CKN(cudaMemcpy(s->bcv, val.data(), sizeof(double) * 4 * N, cudaMemcpyHostToDevice));
    return MPM_OK;
}

// ||b - A x|| and sqrt(rtr / idof) of the scaled system in s (ComputeRefResidual /
// ComputeAbsResidual); x is physical.  Synchronises the stream.
static mpm_status ns_residual(mpm_ns *s, const double *x, double *ref, double *absr) {
    const int nodec = s->nodec, nb = (nodec + 255) / 256, nb4 = (4 * nodec + 255) / 256;
    k_nsv_prep<<<nb4, 256, 0, s->stream>>>(nodec, s->a.mtol, x, s->adiag, s->v.Ax);
    k_nsv_matvec<<<nb, 256, 0, s->stream>>>(s->a.g, s->A, s->bcf, s->v.Ax, s->v.Ar, nullptr);
    k_nsv_resid<<<nb, 256, 0, s->stream>>>(nodec, s->a.mtol, s->bcf, s->b, s->v.Ar, s->adiag, s->part, s->cnt,
                                           s->scal);
    CKN(cudaMemcpyAsync(s->h_scal, s->scal, sizeof(double) * NS_NSCAL, cudaMemcpyDeviceToHost, s->stream));
    CKN(cudaStreamSynchronize(s->stream));
    const double rtr = s->h_scal[NS_RES], idof = s->h_scal[NS_IDOF];
    *ref = sqrt(rtr);
    if (absr) *absr = idof <= 1.0e-30 ? 0.0 : sqrt(rtr / idof);
    return MPM_OK;
}

// One GPBiCGSafe call (solver.cpp:19-141) on the scaled system from the current
// physical s->x, stopped at rtr < eps btb as the reference does, or at kmax
// iterations.  Iterations are launched in blocks of 8; once the device-side
// test has stopped the solve the remaining launches of a block return at once.
static mpm_status ns_gpbicgsafe(mpm_ns *s, double eps, int kmax, int *iters) {
    const int nodec = s->nodec, nb = (nodec + 255) / 256, nb4 = (4 * nodec + 255) / 256;
    cudaStream_t st = s->stream;
    const double *done = s->scal + NS_DONE;
    k_nsv_scale_in<<<nb, 256, 0, st>>>(nodec, s->a.mtol, s->bcf, s->x, s->b, s->adiag, s->v.xs, s->v.rr);
    k_nsv_matvec<<<nb, 256, 0, st>>>(s->a.g, s->A, s->bcf, s->v.xs, s->v.Ax, nullptr);
    k_nsv_init<<<nb, 256, 0, st>>>(nodec, s->v, s->part, s->cnt, s->scal);
    int it = 0;
    bool finished = false;
    while (!finished && it < kmax) {
        const int blk = kmax - it < 8 ? kmax - it : 8;
        for (int k = 0; k < blk; k++) {
            k_nsv_matvec<<<nb, 256, 0, st>>>(s->a.g, s->A, s->bcf, s->v.rr, s->v.Ar, done);
            k_gpb_1<<<nb, 256, 0, st>>>(nodec, s->v, s->part, s->cnt + 1, s->scal);
            k_gpb_2<<<nb, 256, 0, st>>>(nodec, s->v, s->scal);
            k_nsv_matvec<<<nb, 256, 0, st>>>(s->a.g, s->A, s->bcf, s->v.uu, s->v.Au, done);
            k_gpb_3<<<nb, 256, 0, st>>>(nodec, s->v, eps, s->part, s->cnt + 2, s->scal);
        }
        CKN(cudaGetLastError());
        CKN(cudaMemcpyAsync(s->h_scal, s->scal, sizeof(double) * NS_NSCAL, cudaMemcpyDeviceToHost, st));
        CKN(cudaStreamSynchronize(st));
        it = (int)s->h_scal[NS_ITER];
        if (s->h_scal[NS_RTR] != s->h_scal[NS_RTR]) return MPM_ERR_NONFINITE;
        finished = s->h_scal[NS_DONE] != 0.0;
    }
    k_nsv_restore<<<nb4, 256, 0, st>>>(nodec, s->a.mtol, s->v.xs, s->adiag, s->x);
    CKN(cudaGetLastError());
    *iters = it;
    return finished ? MPM_OK : MPM_ERR_KRYLOV_MAXIT;
}

extern "C" mpm_status mpm_ns_solve(mpm_ns *s, int64_t n, const double *x, const double *mass, const double *vol,
                                   const double *nvel, const double *naccel, const double *nmass, double *ndispl,
                                   double *npres, double *tau1, double *tau2, double rtol, int kmax,
                                   mpm_ns_stats *stats) {
    if (!s || n < 0 || !nvel || !naccel || !nmass || !ndispl || !npres || !(rtol > 0.0) || kmax < 1)
        return MPM_ERR_BAD_ARG;
    if (n > 0 && (!x || !mass || !vol || !tau1 || !tau2)) return MPM_ERR_BAD_ARG;
    const int nodec = s->nodec, nb = (nodec + 255) / 256, nb4 = (4 * nodec + 255) / 256;
    const size_t N = (size_t)nodec;
    cudaStream_t st = s->stream;
    NsArgs a = s->a;
    a.n = n;
    // SolveNS: ndispl, npres and the solver's iterate start at zero
    CKN(cudaMemsetAsync(ndispl, 0, sizeof(double) * 3 * N, st));
    CKN(cudaMemsetAsync(npres, 0, sizeof(double) * N, st));
    CKN(cudaMemsetAsync(s->x, 0, sizeof(double) * 4 * N, st));
    const int iter_max = 100;
    double r0r = 0.0, rkr = 0.0, rabs = 0.0;
    int NR_it, ktot = 0;
    mpm_status rc = MPM_OK;
    for (NR_it = 0; NR_it <= iter_max; NR_it++) {
        k_nsv_bcnr<<<nb, 256, 0, st>>>(nodec, s->bcf, s->bcv, s->prm.dt * s->prm.facl, s->prm.facl, ndispl, npres);
        CKN(cudaGetLastError());
        CKN(ns_assemble_launch(a, x, mass, vol, nvel, naccel, ndispl, npres, nmass, tau1, tau2, s->A, s->b,
                               s->status, st));
        k_nsv_diag<<<nb, 256, 0, st>>>(nodec, a.mtol, s->A, s->adiag);
        k_nsv_scale_mat<<<nb, 256, 0, st>>>(a.g, s->A, s->adiag);
        CKN(cudaGetLastError());
        int bad = 0;
        CKN(cudaMemcpyAsync(&bad, s->status, sizeof(int), cudaMemcpyDeviceToHost, st));
        CKN(cudaStreamSynchronize(st));
        if (bad) {
            rc = MPM_ERR_PARTICLE_OUT_OF_BOX;
            break;
        }
        // the linear solve: GPBiCGSafe at the reference's own test (eps 1e-8 on
        // squared norms), called again from where it stopped until the physical
        // residual is below rtol ||b|| (||b|| with the BC rows zeroed: the
        // residual of x = 0)
        CKN(cudaMemsetAsync(s->v.xs, 0, sizeof(double) * 4 * N, st));
        double bnorm;
        mpm_status q = ns_residual(s, s->v.xs, &bnorm, nullptr);
        if (q != MPM_OK) return q;
        for (int call = 0; call < 20; call++) {
            double r;
            q = ns_residual(s, s->x, &r, nullptr);
            if (q != MPM_OK) return q;
            if (r <= rtol * bnorm) break;
            int k = 0;
            rc = ns_gpbicgsafe(s, 1.0e-8, kmax, &k);
            ktot += k;
            if (rc != MPM_OK) break;
        }
        if (rc != MPM_OK) break;
        k_nsv_update<<<nb4, 256, 0, st>>>(nodec, s->x, ndispl, npres);
        CKN(cudaGetLastError());
        // CheckNRConvergence: the residual of the solved linear system
        q = ns_residual(s, s->x, &rkr, &rabs);
        if (q != MPM_OK) return q;
        if (NR_it == 0) r0r = rkr;
        const double rref = r0r > 1.0e-30 ? rkr / r0r : 0.0;
        if (rref < 1.0e-6 || r0r < 1.0e-6 || rabs < 1.0e-8) break;
    }
    if (rc == MPM_OK && NR_it > iter_max) rc = MPM_ERR_NEWTON_MAXIT;
    if (stats) {
        stats->newton_iters = NR_it > iter_max ? iter_max + 1 : NR_it + 1;
        stats->krylov_iters = ktot;
        stats->r0r = r0r;
        stats->last_residual = rkr;
        stats->last_abs_residual = rabs;
    }
    return rc;
}

// =============================================================== time step
// The nodal state, P2G sums and nodal volume of mpm_ns_step, allocated on the
// first step; the particle scratch (tau1, tau2, geup, reduction partials)
// grows with the particle count.
static mpm_status ns_step_buffers(mpm_ns *s, int64_t n) {
    const size_t N = (size_t)s->nodec;
    cudaError_t e = cudaSuccess;
    auto alloc = [&](void **p, size_t bytes) {
        if (e == cudaSuccess && !*p) e = cudaMalloc(p, bytes);
    };
    alloc((void **)&s->nmass, sizeof(double) * N);
    alloc((void **)&s->nvof, sizeof(double) * N);
    alloc((void **)&s->nvel, sizeof(double) * 3 * N);
    alloc((void **)&s->naccel, sizeof(double) * 3 * N);
    alloc((void **)&s->ndispl, sizeof(double) * 3 * N);
    alloc((void **)&s->npres, sizeof(double) * N);
    alloc((void **)&s->nei, sizeof(double) * N);
    alloc((void **)&s->sums, sizeof(unsigned long long) * 8 * N);
    alloc((void **)&s->bnd, sizeof(unsigned) * NB_N);
    alloc((void **)&s->nvol, sizeof(double) * N);
    if (e == cudaSuccess && !s->nvol_ready) {
        Geom g{};
        for (int d = 0; d < 3; d++) {
            g.nel[d] = s->grid.xyelem[d];
            g.nnc[d] = s->grid.xyelem[d] + 1;
            g.order[d] = 1;
            g.xmin[d] = s->grid.xymin[d];
            g.dx[d] = s->grid.dxy[d];
        }
        g.nodec = s->nodec;
        g.nelem = s->grid.xyelem[0] * s->grid.xyelem[1] * s->grid.xyelem[2];
        launch_nodal_volume(g, s->grid.npxye, s->nvol, s->stream);
        e = cudaGetLastError();
        s->nvol_ready = e == cudaSuccess;
    }
    if (e == cudaSuccess && n > s->pcap) {
        for (double **p : {&s->tau1, &s->tau2, &s->geup, &s->ppart}) {
            if (*p) cudaFree(*p);
            *p = nullptr;
        }
        const int64_t cap = n + n / 4 + 256;
        alloc((void **)&s->tau1, sizeof(double) * cap);
        alloc((void **)&s->tau2, sizeof(double) * cap);
        alloc((void **)&s->geup, sizeof(double) * 3 * cap);
        alloc((void **)&s->ppart, sizeof(double) * ((cap + 255) / 256 + 1));
        s->pcap = e == cudaSuccess ? cap : 0;
    }
    if (e != cudaSuccess) {
        fprintf(stderr, "mpm_ns_step: %s\n", cudaGetErrorString(e));
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? MPM_ERR_OOM : MPM_ERR_CUDA;
    }
    return MPM_OK;
}

static NsStepArgs ns_step_args(const mpm_ns *s, int64_t n, int scheme, double facl) {
    NsStepArgs a;
    memset(&a, 0, sizeof(a));
    a.g = s->a.g;
    a.n = n;
    a.mtol = s->prm.mtol;
    a.facl = facl;
    a.dt = s->prm.dt;
    a.gamma = s->prm.gamma_nb;
    for (int k = 0; k < 6; k++) a.nb[k] = s->a.nb[k];
    a.flip = scheme == MPM_FLIP;
    return a;
}

static mpm_status ns_step_check(mpm_ns *s, int64_t n, const double *x, const double *vel, const double *accel,
                                const double *mass, const double *vol, int scheme, double facl) {
    if (!s || n < 0 || n > ((int64_t)1 << 31) - 256 || !(facl == facl)) return MPM_ERR_BAD_ARG;
    if (scheme != MPM_PIC && scheme != MPM_FLIP) return MPM_ERR_UNSUPPORTED;
    if (n > 0 && (!x || !vel || !accel || !mass || !vol)) return MPM_ERR_BAD_ARG;
    mpm_status rc = ns_step_buffers(s, n);
    if (rc != MPM_OK) return rc;
    // the step's load factor: BCSetVal, BCNRSet and the body force read it
    s->prm.facl = facl;
    for (int d = 0; d < 3; d++) s->a.f[d] = s->prm.gravity[d] * facl;
    return MPM_OK;
}

// Particle2Node (var_trans_fluid.cpp:17-80) into the context's nodal state.
// Synchronises the stream.
static mpm_status ns_p2g(mpm_ns *s, const NsStepArgs &a, const double *x, const double *vel, const double *accel,
                         const double *mass, const double *vol) {
    const size_t N = (size_t)s->nodec;
    cudaStream_t st = s->stream;
    CKN(cudaMemsetAsync(s->sums, 0, sizeof(unsigned long long) * 8 * N, st));
    CKN(cudaMemsetAsync(s->bnd, 0, sizeof(unsigned) * NB_N, st));
    CKN(cudaMemsetAsync(s->status, 0, sizeof(int), st));
    const unsigned npb = (unsigned)((a.n + 127) / 128);
    if (a.n > 0) {
        k_nsp_bounds<<<npb, 128, 0, st>>>(a, x, vel, accel, mass, vol, s->bnd, s->status);
        k_nsp_scatter<<<npb, 128, 0, st>>>(a, x, vel, accel, mass, vol, s->bnd, s->sums);
    }
    k_nsp_grid<<<(s->nodec + 255) / 256, 256, 0, st>>>(a, s->sums, s->bnd, s->bcf, s->bcv, s->nmass, s->nvof,
                                                       s->nvel, s->naccel);
    CKN(cudaGetLastError());
    int bad = 0;
    CKN(cudaMemcpyAsync(&bad, s->status, sizeof(int), cudaMemcpyDeviceToHost, st));
    CKN(cudaStreamSynchronize(st));
    if (bad & NS_NONFINITE) return MPM_ERR_NONFINITE;
    if (bad & NS_OUTSIDE) return MPM_ERR_PARTICLE_OUT_OF_BOX;
    return MPM_OK;
}

extern "C" mpm_status mpm_ns_p2g(mpm_ns *s, int64_t n, const double *x, const double *vel, const double *accel,
                                 const double *mass, const double *vol, int scheme, double facl) {
    mpm_status rc = ns_step_check(s, n, x, vel, accel, mass, vol, scheme, facl);
    if (rc != MPM_OK) return rc;
    return ns_p2g(s, ns_step_args(s, n, scheme, facl), x, vel, accel, mass, vol);
}

// Node2Particle (var_trans_fluid.cpp:82-135) from the context's nodal state
// after the solve.  Synchronises the stream.
static mpm_status ns_g2p(mpm_ns *s, const NsStepArgs &a, double *x, double *vel, double *accel, double *pres,
                         const double *vol) {
    cudaStream_t st = s->stream;
    k_nsn_commit<<<(s->nodec + 255) / 256, 256, 0, st>>>(a, s->ndispl, s->nvof, s->nvol, s->nvel, s->naccel, s->nei,
                                                         s->part, s->cnt + 3, s->scal, NS_EU);
    if (a.n > 0) {
        const unsigned npb = (unsigned)((a.n + 255) / 256);
        k_nsp_g2p<<<npb, 256, 0, st>>>(a, x, vel, accel, pres, vol, s->nvel, s->naccel, s->ndispl, s->npres, s->nei,
                                       s->geup, s->ppart, s->cnt + 3, s->scal, NS_GD);
        k_nsp_shift<<<npb, 256, 0, st>>>(a, s->geup, s->scal, NS_EU, NS_GD, x);
    }
    CKN(cudaGetLastError());
    CKN(cudaStreamSynchronize(st));
    return MPM_OK;
}

extern "C" mpm_status mpm_ns_step(mpm_ns *s, int64_t n, double *x, double *vel, double *accel, double *pres,
                                  const double *mass, const double *vol, int scheme, double facl, double rtol,
                                  int kmax, mpm_ns_stats *stats) {
    if (!(rtol > 0.0) || kmax < 1 || (n > 0 && !pres)) return MPM_ERR_BAD_ARG;
    mpm_status rc = ns_step_check(s, n, x, vel, accel, mass, vol, scheme, facl);
    if (rc != MPM_OK) return rc;
    const NsStepArgs a = ns_step_args(s, n, scheme, facl);
    rc = ns_p2g(s, a, x, vel, accel, mass, vol);
    if (rc != MPM_OK) return rc;
    // ---- SolveNS (solve_ns_mpm.cpp:28-62)
    rc = mpm_ns_solve(s, n, x, mass, vol, s->nvel, s->naccel, s->nmass, s->ndispl, s->npres, s->tau1, s->tau2, rtol,
                      kmax, stats);
    if (rc != MPM_OK) return rc;
    return ns_g2p(s, a, x, vel, accel, pres, vol);
}

// ------------------------------------------------- particles held by the context
// The three member calls of a StabilizedMPM time step on particles the
// context holds (uploaded once from the reference's AoS host vectors).
extern "C" mpm_status mpm_ns_load_particles(mpm_ns *s, int64_t n, const double *coord, const double *vel,
                                            const double *accel, const double *mass, const double *vol) {
    if (!s || n < 0 || n > ((int64_t)1 << 31) - 256) return MPM_ERR_BAD_ARG;
    if (n > 0 && (!coord || !mass || !vol)) return MPM_ERR_BAD_ARG;
    CKN(cudaStreamSynchronize(s->stream));
    if (s->pbuf) cudaFree(s->pbuf);
    s->pbuf = nullptr;
    s->np = 0;
    s->p2g_done = false;
    const size_t N = (size_t)(n > 0 ? n : 1);
    // SoA: x 3, vel 3, accel 3, pres, mass, vol
    CKN(cudaMalloc((void **)&s->pbuf, sizeof(double) * 12 * N));
    std::vector<double> h(12 * N, 0.0);
    for (int64_t p = 0; p < n; p++) {
        for (int d = 0; d < 3; d++) {
            h[d * N + p] = coord[3 * p + d];
            h[(3 + d) * N + p] = vel ? vel[3 * p + d] : 0.0;
            h[(6 + d) * N + p] = accel ? accel[3 * p + d] : 0.0;
        }
        h[10 * N + p] = mass[p];
        h[11 * N + p] = vol[p];
    }
    CKN(cudaMemcpy(s->pbuf, h.data(), sizeof(double) * 12 * N, cudaMemcpyHostToDevice));
    s->np = n;
    return MPM_OK;
}

extern "C" mpm_status mpm_ns_download_particles(mpm_ns *s, double *coord, double *vel, double *accel, double *pres) {
    if (!s || (s->np > 0 && !s->pbuf)) return MPM_ERR_BAD_ARG;
    const int64_t n = s->np;
    if (n == 0) return MPM_OK;
    const size_t N = (size_t)n;
    std::vector<double> h(12 * N);
    CKN(cudaStreamSynchronize(s->stream));
    CKN(cudaMemcpy(h.data(), s->pbuf, sizeof(double) * 12 * N, cudaMemcpyDeviceToHost));
    for (int64_t p = 0; p < n; p++) {
        for (int d = 0; d < 3; d++) {
            if (coord) coord[3 * p + d] = h[d * N + p];
            if (vel) vel[3 * p + d] = h[(3 + d) * N + p];
            if (accel) accel[3 * p + d] = h[(6 + d) * N + p];
        }
        if (pres) pres[p] = h[9 * N + p];
    }
    return MPM_OK;
}

// the resident arrays: x, vel, accel (3 blocks each), pres, mass, vol
static void ns_resident(mpm_ns *s, double *&x, double *&vel, double *&accel, double *&pres, double *&mass,
                        double *&vol) {
    const size_t N = (size_t)(s->np > 0 ? s->np : 1);
    x = s->pbuf;
    vel = s->pbuf + 3 * N;
    accel = s->pbuf + 6 * N;
    pres = s->pbuf + 9 * N;
    mass = s->pbuf + 10 * N;
    vol = s->pbuf + 11 * N;
}

extern "C" mpm_status mpm_ns_particle2node(mpm_ns *s, int scheme, double facl) {
    if (!s || !s->pbuf) return MPM_ERR_STATE;
    double *x, *vel, *accel, *pres, *mass, *vol;
    ns_resident(s, x, vel, accel, pres, mass, vol);
    mpm_status rc = ns_step_check(s, s->np, x, vel, accel, mass, vol, scheme, facl);
    if (rc != MPM_OK) return rc;
    rc = ns_p2g(s, ns_step_args(s, s->np, scheme, facl), x, vel, accel, mass, vol);
    s->p2g_done = rc == MPM_OK;
    s->p2g_scheme = scheme;
    return rc;
}

extern "C" mpm_status mpm_ns_solve_ns(mpm_ns *s, double rtol, int kmax, mpm_ns_stats *stats) {
    if (!s || !s->pbuf || !s->p2g_done) return MPM_ERR_STATE;
    double *x, *vel, *accel, *pres, *mass, *vol;
    ns_resident(s, x, vel, accel, pres, mass, vol);
    return mpm_ns_solve(s, s->np, x, mass, vol, s->nvel, s->naccel, s->nmass, s->ndispl, s->npres, s->tau1, s->tau2,
                        rtol, kmax, stats);
}

extern "C" mpm_status mpm_ns_node2particle(mpm_ns *s) {
    if (!s || !s->pbuf || !s->p2g_done) return MPM_ERR_STATE;
    double *x, *vel, *accel, *pres, *mass, *vol;
    ns_resident(s, x, vel, accel, pres, mass, vol);
    s->p2g_done = false;   // the next time step starts with Particle2Node
    return ns_g2p(s, ns_step_args(s, s->np, s->p2g_scheme, s->prm.facl), x, vel, accel, pres, vol);
}

extern "C" mpm_status mpm_ns_get_nodal(mpm_ns *s, int field, double *host) {
    if (!s || !host || field < 0 || field > 6) return MPM_ERR_BAD_ARG;
    if (!s->nvol) return MPM_ERR_BAD_ARG;   // no time step yet
    const size_t N = (size_t)s->nodec;
    const double *src[7] = {s->nmass, s->nvof, s->nvel, s->naccel, s->ndispl, s->npres, s->nvol};
    const size_t len[7] = {N, N, 3 * N, 3 * N, 3 * N, N, N};
    CKN(cudaStreamSynchronize(s->stream));
    CKN(cudaMemcpy(host, src[field], sizeof(double) * len[field], cudaMemcpyDeviceToHost));
    return MPM_OK;
}

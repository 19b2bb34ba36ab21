// Implicit solid MPM on the GPU (FP64): generalized-alpha / Newmark time
// integration, Newton iteration, assembly of the stiffness operator into a
// 27-point block stencil, symmetric diagonal scaling, and a preconditioned
// conjugate-gradient solve with FP64 reductions.
//
// Reference (module/solid/implicit/, module/solver/, module/nonlinear_time_integration.cpp):
//   Particle2Node            var_trans_solid_implicit.cpp:20-80      -> run_p2g (AccelP2G mode) + k_imp_grid
//   SolveSolid (Newton)      solve_solid_implicit.cpp:65-103         -> implicit_newton
//   BCNRSet / Predict        implicit_mpm_solid.h:55-64,
//                            nonlinear_time_integration.cpp:59-71    -> k_imp_bcnr, k_imp_predict
//   AssembleSystem           solve_solid_implicit.cpp:105-204        -> k_imp_assemble, k_imp_rhs_diag
//   ComputeTangentModulus    solve_solid_implicit.cpp:34-63          -> pair loop of k_imp_assemble
//   BuildDiagonalPreconditioner crsmat.cpp:87-184                     -> k_imp_rhs_diag, k_imp_scale
//   MatVecMult               solver.cpp:405-433                      -> k_imp_matvec
//   GPBiCGSafe               solver.cpp:19-141                       -> conjugate gradients (the scaled
//                            system is symmetric), stopped on the same squared-norm ratio
//   CheckNRConvergence       solver.cpp:484-593                      -> newton_residuals
//   Node2Particle            var_trans_solid_implicit.cpp:106-167,
//                            nonlinear_time_integration.cpp:73-96    -> k_imp_g2p, k_imp_shift
//
// Matrix storage: for control point n and stencil slot s (the neighbours
// n + (dx, dy, dz) with |dx| <= rx, |dy| <= ry, |dz| <= rz, where the radius
// of an axis is its shape order: 1 for linear shape functions, 2 for the
// quadratic B-spline, so 27, 75 or 125 slots; s = (dx+rx) + sx ((dy+ry) +
// sy (dz+rz)), sx = 2 rx + 1), the 3x3 block entry q = s * 9 + 3 a + b lives
// at A[aidx(q, n, qp)], tiled by 32 control points and by pairs of entries:
// ((n / 32) * qp + q / 2) * 64 + (n % 32) * 2 + q % 2, qp = ceil(9 ns / 2).
// A thread reads entry pairs as one vector load and a warp reading its 32
// nodes' values walks one contiguous range (coalesced and DRAM-page
// friendly); no column indices (the grid is structured).
//
// Precision: a context of precision 64 computes and stores everything in
// FP64 (the parity mode).  Precision 32 keeps the particles (F as H = F - I),
// the assembly arithmetic and the matrix in FP32 and the matvec of the
// Krylov iterations in FP32 arithmetic; the Krylov vectors, their inner
// products and norms, the true residual b - A x (the FP32-stored matrix
// applied in FP64 arithmetic), the Newton check and the nodal kinematics
// stay FP64.
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <vector>

#include "mpm_device.cuh"
#include "mpm_nn.cuh"

namespace mpm {
mpm_status run_p2g(mpm_ctx *c, double facl);
}

struct ImpState {
    int nr_flag = 0;
    double alpha_f = 1, alpha_m = 1, gamma = 0.5, beta = 0.25, nb[6] = {0};
    int prec = 64;                         // 64: FP64 operator; 32: FP32 particles, assembly and matrix
    int qp = 122;                          // entry pairs per node of the stencil matrix (aidx)
    void *A = nullptr;                     // 9 ns values per node (FP64 or FP32), tiled by 32 nodes (aidx)
    double *adiag = nullptr, *b = nullptr;  // 3 * nodec
    double *x = nullptr, *r = nullptr, *p = nullptr, *Ap = nullptr, *xs = nullptr;
    double *ndispl = nullptr, *nvel = nullptr, *naccel = nullptr, *naccel_k = nullptr;
    double *nmass = nullptr, *nvof = nullptr, *nei = nullptr;
    double *bcval64 = nullptr;             // 3 * nodec prescribed BC values in FP64 (implicit_bc_changed)
    void *stress_k = nullptr;              // 6 * num, Newton stress of the step (particle precision)
    void *geup = nullptr;                  // 3 * num (particle precision)
    double *part = nullptr;                // reduction partials
    double *scal = nullptr;                // device scalars
    double *h_scal = nullptr;              // pinned mirror
    int nblk = 0;
    int64_t num_alloc = 0;
    int64_t krylov_total = 0, newton_total = 0;
    double last_rel = 0.0;
    // flexible CG with the learned preconditioner
    mpm_nn *net = nullptr;
    double *z = nullptr, *bs = nullptr;    // preconditioned residual, scaled RHS (3 * nodec)
    double *xstar = nullptr, *ev = nullptr; // training-pair harvest: converged solution, error
    double *gp = nullptr, *gq = nullptr;    // flexible GCR: GM directions and their images (GM * 3 * nodec)
    double *gqq = nullptr, *gbeta = nullptr;  // |A p|^2 of each kept direction, projection coefficients
    float *gqf = nullptr;                   // FP32 copies of the kept images (GM * 3 * nodec), for the dots
    float *gp32 = nullptr, *gq32 = nullptr;  // FP32 operator: the directions and images in FP32 (GM * 3 * nodec)
    float *dfx = nullptr;                   // FP32 operator: x split into high and low FP32 parts (2 * 3 * nodec)
    unsigned *cnt = nullptr;                // block counters of the single-launch reductions (zero between launches)
    int fallbacks = 0;                      // solves that switched from the network to Jacobi
    int nn_applications = 0;
    // CUDA graphs of 8 Krylov iterations (CG; FCG with the network; FCG with Jacobi)
    cudaGraphExec_t g_cg = nullptr, g_fcg_nn = nullptr, g_fcg_jac = nullptr, g_gcr = nullptr;
    mpm_nn *g_net = nullptr;
    bool no_graph = false;
    bool gcr = true;      // learned preconditioner: flexible GCR first (else flexible CG only)
    int gm = 4;           // GCR window in use (1, 2, 4 or 8 <= GM directions; 4 measured fastest on the cantilever)
    bool debug = false;   // MPM_GB300_KRYLOV_TRACE set: residual history to stderr
};

namespace mpm {

constexpr int GM = 8;   // directions kept by the flexible GCR solver

enum Scal { S_RR0 = 0, S_RR1, S_PAP, S_RR_INIT, S_RES, S_IDOF, S_EU, S_GD, S_ZQ, S_PR, S_RRC, S_DZZ, S_DZR, S_QR, S_QQ, S_NSCAL };

struct ImpArgs {
    int nnc[3];
    int nel[3];
    int nodec;
    double xmin[3], dx[3], inv_dx[3];
    double dt, facl, mtol, grav[3];
    double af, am, gamma, nb[6];
    int nr_flag;
    int shifting;
    int scheme;
    int rad[3];   // stencil radius per axis (the shape order)
    int ns;       // stencil slots (2 rad + 1 per axis)
    int qp;       // entry pairs per node (aidx)
    int64_t num;
    const unsigned char *bcflag;
    const double *bcval;
    const double *nvol;
    const int *iprop;
    const double *matprop;
};

__host__ __device__ __forceinline__ size_t aidx(int q, int n, int qp) {
    return (((size_t)(n >> 5) * qp + (size_t)(q >> 1)) << 6) + (size_t)((n & 31) << 1) + (size_t)(q & 1);
}
static size_t a_size(int nodec, int qp) { return (size_t)((nodec + 31) / 32) * 64 * (size_t)qp; }

static ImpArgs imp_args(mpm_ctx *c) {
    ImpArgs a;
    memset(&a, 0, sizeof(a));
    for (int d = 0; d < 3; d++) {
        a.nnc[d] = c->g.nnc[d];
        a.nel[d] = c->g.nel[d];
        a.xmin[d] = c->g.xmin[d];
        a.dx[d] = c->g.dx[d];
        a.inv_dx[d] = 1.0 / c->g.dx[d];
        a.grav[d] = c->gravity[d];
    }
    a.nodec = c->g.nodec;
    a.dt = c->dt;
    a.facl = c->facl;
    a.mtol = c->mtol;
    ImpState *s = c->imp;
    a.af = s->alpha_f;
    a.am = s->alpha_m;
    a.gamma = s->gamma;
    for (int k = 0; k < 6; k++) a.nb[k] = s->nb[k];
    a.nr_flag = s->nr_flag;
    a.shifting = c->shifting;
    a.scheme = c->scheme;
    a.ns = 1;
    for (int d = 0; d < 3; d++) {
        a.rad[d] = c->g.order[d];
        a.ns *= 2 * a.rad[d] + 1;
    }
    a.qp = (9 * a.ns + 1) / 2;
    a.num = c->num;
    a.bcflag = c->d_bcflag;
    // prescribed values in FP64 whatever the context's precision (an FP32
    // context keeps its own copy in FP32, d_bcval)
    a.bcval = s->bcval64;
    a.nvol = c->d_nvol;
    a.iprop = c->d_iprop;
    a.matprop = c->d_matprop;
    return a;
}

// Particle fields of an implicit context (precision R; FP32 stores H = F - I in F)
template <typename R>
struct PView {
    R *x[3], *v[3], *F[9], *s[6], *m, *vol0, *vol, *acc[3];
    int *matid;
};

template <typename R>
static PView<R> pview(mpm_ctx *c) {
    PView<R> v;
    size_t n = c->pstride;
    R *f = (R *)c->pbuf[c->cur];
    for (int k = 0; k < 3; k++) v.x[k] = f + k * n;
    for (int k = 0; k < 3; k++) v.v[k] = f + (3 + k) * n;
    for (int k = 0; k < 9; k++) v.F[k] = f + (6 + k) * n;
    for (int k = 0; k < 6; k++) v.s[k] = f + (15 + k) * n;
    v.m = f + 21 * n;
    v.vol0 = f + 22 * n;
    v.vol = f + 23 * n;
    for (int k = 0; k < 3; k++) v.acc[k] = f + (24 + k) * n;
    v.matid = (int *)(f + 27 * n);
    return v;
}

__device__ __forceinline__ void node_ijk(int n, const int *nnc, int &i, int &j, int &k) {
    i = n % nnc[0];
    j = (n / nnc[0]) % nnc[1];
    k = n / (nnc[0] * nnc[1]);
}

template <typename R>
__device__ __forceinline__ KGeom<R> kgeom(const ImpArgs &a) {
    KGeom<R> g;
    for (int d = 0; d < 3; d++) {
        g.xmin[d] = (R)a.xmin[d];
        g.dx[d] = (R)a.dx[d];
        g.inv_dx[d] = (R)a.inv_dx[d];
        g.nel[d] = a.nel[d];
        g.nnc[d] = a.nnc[d];
        g.ntile[d] = 0;
    }
    g.nodec = a.nodec;
    return g;
}

// Shape functions at x (MakSf, module/shape_function.cpp:8-119) for shape
// orders OX, OY, OZ: weights, gradients and control-point ids of the
// (OX+1)(OY+1)(OZ+1) nodes in MakSf order (x fastest), and each node's
// offset inside the element's node box (for the stencil slot).
template <typename R, int OX, int OY, int OZ>
__device__ __forceinline__ void shape_nodes(const ImpArgs &a, const KGeom<R> &g, const R *x, R *N, R (*dN)[3],
                                            int *nid, bool &oob) {
    const int cx = cell_of(x[0], g, 0, oob), cy = cell_of(x[1], g, 1, oob), cz = cell_of(x[2], g, 2, oob);
    Axis<R, OX> ax;
    Axis<R, OY> ay;
    Axis<R, OZ> az;
    axis_eval<R, OX>(x[0], g, 0, cx, ax);
    axis_eval<R, OY>(x[1], g, 1, cy, ay);
    axis_eval<R, OZ>(x[2], g, 2, cz, az);
    int id = 0;
#pragma unroll
    for (int k = 0; k <= OZ; k++)
#pragma unroll
        for (int j = 0; j <= OY; j++)
#pragma unroll
            for (int i = 0; i <= OX; i++) {
                N[id] = ax.w[i] * ay.w[j] * az.w[k];
                dN[id][0] = ax.dw[i] * ay.w[j] * az.w[k];
                dN[id][1] = ax.w[i] * ay.dw[j] * az.w[k];
                dN[id][2] = ax.w[i] * ay.w[j] * az.dw[k];
                nid[id] = (cx + i) + a.nnc[0] * ((cy + j) + a.nnc[1] * (cz + k));
                id++;
            }
}

// ------------------------------------------------------------ node kernels
// Particle2Node's grid part: nvel = p/m, naccel = f/m, BCs (var_trans_solid_implicit.cpp:47-75)
__global__ void k_imp_grid(ImpArgs a, const unsigned long long *acc, const double *inv, double *nmass, double *nvof,
                           double *nvel, double *naccel) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= a.nodec) return;
    const size_t N = (size_t)a.nodec;
    const double m = (double)(long long)acc[n] * inv[0];
    nmass[n] = m;
    nvof[n] = (double)(long long)acc[N + n] * inv[1];
    const unsigned char bf = a.bcflag[n];
    for (int c = 0; c < 3; c++) {
        double v = 0.0, ac = 0.0;
        if (m > a.mtol) {
            v = (double)(long long)acc[(2 + c) * N + n] * inv[2] / m;
            ac = (double)(long long)acc[(5 + c) * N + n] * inv[3] / m;
        }
        if (bf & (1 << c)) {
            v = a.bcval[c * N + n] * a.facl;
            ac = 0.0;
        }
        nvel[c * N + n] = v;
        naccel[c * N + n] = ac;
    }
}

// BCNRSet (BCSetDt on ndispl) then PredictNewmarkBetaVelAndAccel's acceleration
__global__ void k_imp_predict(ImpArgs a, double *ndispl, const double *nvel, const double *naccel, double *naccel_k,
                              double *nvel_k, int set_bc) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= a.nodec) return;
    const size_t N = (size_t)a.nodec;
    const unsigned char bf = a.bcflag[n];
    for (int c = 0; c < 3; c++) {
        const size_t i = c * N + n;
        if (set_bc && (bf & (1 << c))) ndispl[i] = a.bcval[i] * a.dt * a.facl;
        const double d = ndispl[i];
        naccel_k[i] = a.nb[3] * d - a.nb[4] * nvel[i] - a.nb[5] * naccel[i];
        if (nvel_k) nvel_k[i] = a.nb[0] * d - a.nb[1] * nvel[i] - a.nb[2] * naccel[i];
    }
}

// ------------------------------------------------------------- assembly
// Material tangent of one particle in a factored form that the pair loop
// contracts with the scaled gradient a of the row node and the gradient b of
// the column node (K_ij = sum_kl a_k C_ikjl b_l of ComputeTangentModulus,
// solve_solid_implicit.cpp:34-63, written out for each model's C):
//   isotropic (models -1, 0, 1; C = lambda' I(x)I + 2 mu' I4sym):
//       K = lambda' a b^T + mu' b a^T + mu' (a.b) I
//   general (models 2, 3):
//       K = (G a) b^T + a (G' b)^T + alpha (a.b) I + gam b a^T
//           + eps (B a)(B b)^T + beta (a.B b) B + delta (B b)(B a)^T
// plus, with NR_flag, the geometric term ((sigma a).b) I.
template <typename R>
struct Tangent {
    bool general;
    R lam, mu;                    // isotropic
    R B[3][3], G[3][3], Gp[3][3];  // general
    R alpha, gam, eps, beta, delta;
};

// St.Venant-Kirchhoff (MatStVk's stif_mat, constitutive_model.cpp:160-183):
// C = lambda' b(x)b + mu' (b_ik b_jl + b_il b_jk), lambda' = lambda / J, mu' = mu / J, b = F F^T.
template <typename R>
__device__ __forceinline__ void tangent_stvk(Tangent<R> &t, const R F[3][3], R J, R E, R nu) {
    const R rd = (R)1 / (((R)1 + nu) * ((R)1 - (R)2 * nu));
    const R ij = (R)1 / J;
    t.general = true;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            t.B[i][j] = F[i][0] * F[j][0] + F[i][1] * F[j][1] + F[i][2] * F[j][2];
            t.G[i][j] = (R)0;
            t.Gp[i][j] = (R)0;
        }
    t.alpha = t.gam = (R)0;
    t.eps = nu * E * rd * ij;
    t.beta = t.delta = (R)0.5 * E * ((R)1 - (R)2 * nu) * rd * ij;
}

// Mooney-Rivlin (MatMooneyRivlin's stif_mat, constitutive_model.cpp:235-283)
// with B the isochoric b, I1, I2 its invariants, hp = bulk ln J / J, s the
// Cauchy stress, A = I1 B - B^2:
//   G  = (bulk / J - t1 / 3 + c4) I - 2/3 dev(s) - c3 A,  G' = -2/3 dev(s) - c3 A,
//   alpha = gam = t1 / 2 - hp,  eps = c2',  beta = delta = -c2' / 2,
// t1 = 4 (c1 I1 + 2 c2 I2) / (3 J), c2' = 4 c2 / J, c3 = 4 c2 / (3 J), c4 = 8 c2 I2 / (9 J).
template <typename R>
__device__ __forceinline__ void tangent_mooney_rivlin(Tangent<R> &t, const R F[3][3], R J, R lnJ, const R *s, R c1,
                                                      R c2, R bulk) {
    const R ij = (R)1 / J;
    const R k2 = exp((R)(-2.0 / 3.0) * lnJ);   // J^(-2/3)
    R B2[3][3];
    t.general = true;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) t.B[i][j] = k2 * (F[i][0] * F[j][0] + F[i][1] * F[j][1] + F[i][2] * F[j][2]);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) B2[i][j] = t.B[i][0] * t.B[0][j] + t.B[i][1] * t.B[1][j] + t.B[i][2] * t.B[2][j];
    const R i1 = t.B[0][0] + t.B[1][1] + t.B[2][2];
    const R i2 = (R)0.5 * (i1 * i1 - (B2[0][0] + B2[1][1] + B2[2][2]));
    const R hp = bulk * lnJ * ij;
    const R t1 = (R)4 * (c1 * i1 + (R)2 * c2 * i2) * ij / (R)3;
    const R c2p = (R)4 * c2 * ij, c3 = c2p / (R)3, c4 = (R)8 * c2 * i2 * ij / (R)9;
    const R sg[3][3] = {{s[0], s[5], s[4]}, {s[5], s[1], s[3]}, {s[4], s[3], s[2]}};
    const R tr3 = (s[0] + s[1] + s[2]) / (R)3;
    const R g0 = bulk * ij - t1 / (R)3 + c4;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const R dev = sg[i][j] - (i == j ? tr3 : (R)0);
            const R Aij = i1 * t.B[i][j] - B2[i][j];
            t.Gp[i][j] = (R)(-2.0 / 3.0) * dev - c3 * Aij;
            t.G[i][j] = t.Gp[i][j] + (i == j ? g0 : (R)0);
        }
    t.alpha = t.gam = (R)0.5 * t1 - hp;
    t.eps = c2p;
    t.beta = t.delta = (R)(-0.5) * c2p;
}

// One thread per particle (AssembleSystem, solve_solid_implicit.cpp:123-189):
// UpdateDefGrad with alpha_f, the stress of the Newton iterate, the gradient
// correction dN <- dN dF^-1, then the tangent blocks of each unordered node
// pair once (K_ba = K_ab^T: every C here has the major symmetry) + lumped
// mass, and the internal/external force into the RHS, with atomics.  R is
// the particle precision and the precision of the arithmetic and of A; the
// RHS is summed in FP64.
template <typename R, int OX, int OY, int OZ>
__global__ void __launch_bounds__(128) k_imp_assemble(ImpArgs a, PView<R> P, const double *ndispl, R *stress_k,
                                                      R *A, double *b) {
    constexpr int NX = OX + 1, NY = OY + 1, NZ = OZ + 1, NE = NX * NY * NZ;
    constexpr int SX = 2 * OX + 1, SY = 2 * OY + 1, NS = SX * SY * (2 * OZ + 1);
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.num) return;
    const size_t N = (size_t)a.nodec, NP = (size_t)a.num;
    const KGeom<R> g = kgeom<R>(a);
    const R x[3] = {P.x[0][p], P.x[1][p], P.x[2][p]};
    int nid[NE];
    R Nw[NE], dN[NE][3];
    bool oob = false;
    shape_nodes<R, OX, OY, OZ>(a, g, x, Nw, dN, nid, oob);
    // ComputeDeltaDefGrad with alpha_f (material_point.cpp:127-151): d = I + Dm
    R Dm[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int q = 0; q < NE; q++)
        for (int r = 0; r < 3; r++) {
            const R u = (R)ndispl[r * N + nid[q]];
            for (int c = 0; c < 3; c++) Dm[r][c] += dN[q][c] * u;
        }
    const R af = (R)a.af;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) Dm[r][c] *= af;
    R d[3][3];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) d[r][c] = Dm[r][c] + (r == c ? (R)1 : (R)0);
    // UpdateDefGrad: Fn = d F.  FP32 stores H = F - I and forms
    // Hn = Dm + H + Dm H, J - 1 = det(I + Hn) - 1 without the rounding of numbers near 1.
    R Fn[3][3], Hn[3][3], J, jm1;
    if constexpr (sizeof(R) == 8) {
        R F[3][3];
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) F[r][c] = P.F[3 * r + c][p];
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) {
                R sum = 0.0;
                for (int k = 0; k < 3; k++) sum += d[r][k] * F[k][c];
                Fn[r][c] = sum;
            }
        J = det3(Fn);
        jm1 = J - (R)1;
    } else {
        R H[3][3];
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) H[r][c] = P.F[3 * r + c][p];
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) {
                R sum = Dm[r][c] + H[r][c];
                for (int k = 0; k < 3; k++) sum += Dm[r][k] * H[k][c];
                Hn[r][c] = sum;
            }
        jm1 = det_ipm1(Hn);
        J = (R)1 + jm1;
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) Fn[r][c] = Hn[r][c] + (r == c ? (R)1 : (R)0);
    }
    const R vol = J * P.vol0[p];
    // UpdateConstitutiveModel on the Newton stress (constitutive_model.cpp:16-305)
    R sk[6];
    for (int k = 0; k < 6; k++) sk[k] = stress_k[k * NP + p];
    const int mid = P.matid[p];
    const int model = a.iprop[mid];
    const R E = (R)a.matprop[3 * mid], nu = (R)a.matprop[3 * mid + 1], m3 = (R)a.matprop[3 * mid + 2];
    Tangent<R> t;
    t.general = false;
    t.lam = t.mu = (R)0;
    if (model == 0) {
        // the strain increment: FP64 takes d - I as the reference does, FP32 the exact Dm
        R De[3][3];
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++)
                De[r][c] = sizeof(R) == 8 ? (r == c ? d[r][c] - (R)1 : d[r][c]) : Dm[r][c];
        lin_elast_update(sk, De, E, nu);
        t.lam = E * nu / (((R)1 - (R)2 * nu) * ((R)1 + nu));
        t.mu = E / ((R)2 * ((R)1 + nu));
    } else if (model == 1) {
        R lnj;
        if constexpr (sizeof(R) == 8) {
            lnj = neo_hookean_stress(sk, Fn, J, E, nu);
        } else {
            neo_hookean_stress_h(sk, Hn, jm1, E, nu);
            lnj = log1pf(jm1);
        }
        const R rd = (R)1 / (((R)1 + nu) * ((R)1 - (R)2 * nu));
        const R lmd = nu * E * rd;
        const R mu0 = (R)0.5 * E * ((R)1 - (R)2 * nu) * rd;
        const R ij = (R)1 / J;
        t.lam = lmd * ij;
        t.mu = (mu0 - lmd * lnj) * ij;
    } else if (model == 2) {
        if constexpr (sizeof(R) == 8) {
            stvk_stress(sk, Fn, J, E, nu);
        } else {
            stvk_stress_h(sk, Hn, jm1, E, nu);
        }
        tangent_stvk(t, Fn, J, E, nu);
    } else if (model == 3) {   // mat_prop = {c1, c2, bulk}
        R lnj;
        if constexpr (sizeof(R) == 8) {
            mooney_rivlin_stress(sk, Fn, J, E, nu, m3);
            lnj = log(J);
        } else {
            mooney_rivlin_stress_h(sk, Hn, jm1, E, nu, m3);
            lnj = log1pf(jm1);
        }
        tangent_mooney_rivlin(t, Fn, J, lnj, sk, E, nu, m3);
    } else {
        for (int k = 0; k < 6; k++) sk[k] = (R)0;
    }
    for (int k = 0; k < 6; k++) stress_k[k * NP + p] = sk[k];
    // ImplicitDsfCorr: dN <- dN d^-1 (material_point.cpp:153-172)
    R di[3][3];
    {
        const R det = (R)1 / det3(d);
        di[0][0] = (d[1][1] * d[2][2] - d[1][2] * d[2][1]) * det;
        di[0][1] = (d[0][2] * d[2][1] - d[0][1] * d[2][2]) * det;
        di[0][2] = (d[0][1] * d[1][2] - d[0][2] * d[1][1]) * det;
        di[1][0] = (d[1][2] * d[2][0] - d[1][0] * d[2][2]) * det;
        di[1][1] = (d[0][0] * d[2][2] - d[0][2] * d[2][0]) * det;
        di[1][2] = (d[0][2] * d[1][0] - d[0][0] * d[1][2]) * det;
        di[2][0] = (d[1][0] * d[2][1] - d[1][1] * d[2][0]) * det;
        di[2][1] = (d[0][1] * d[2][0] - d[0][0] * d[2][1]) * det;
        di[2][2] = (d[0][0] * d[1][1] - d[0][1] * d[1][0]) * det;
    }
    for (int q = 0; q < NE; q++) {
        R tq[3];
        for (int c = 0; c < 3; c++) tq[c] = dN[q][0] * di[0][c] + dN[q][1] * di[1][c] + dN[q][2] * di[2][c];
        for (int c = 0; c < 3; c++) dN[q][c] = tq[c];
    }
    const R sg[3][3] = {{sk[0], sk[5], sk[4]}, {sk[5], sk[1], sk[3]}, {sk[4], sk[3], sk[2]}};
    const R m = P.m[p];
    const R fx = (R)(a.grav[0] * a.facl), fy = (R)(a.grav[1] * a.facl), fz = (R)(a.grav[2] * a.facl);
    const R afv = af * vol;
    const R am = (R)a.am, nb3 = (R)a.nb[3];
    for (int qa = 0; qa < NE; qa++) {
        const int na = nid[qa];
        const int ia = qa % NX, ja = (qa / NX) % NY, ka = qa / (NX * NY);
        const R emd = nb3 * Nw[qa] * m;   // ComputeNRLumpedMat (material_point.h:144)
        R ah[3], Sa[3];
#pragma unroll
        for (int k = 0; k < 3; k++) ah[k] = afv * dN[qa][k];
#pragma unroll
        for (int k = 0; k < 3; k++)
            Sa[k] = a.nr_flag ? sg[k][0] * ah[0] + sg[k][1] * ah[1] + sg[k][2] * ah[2] : (R)0;
        // isotropic: L = lambda' a, M = mu' a, T = M + sigma a;  general: G a, B a
        R L[3], M[3], T[3], Ga[3], Ba[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            L[k] = t.lam * ah[k];
            M[k] = t.mu * ah[k];
            T[k] = M[k] + Sa[k];
        }
        if (t.general) {
#pragma unroll
            for (int k = 0; k < 3; k++) {
                Ga[k] = t.G[k][0] * ah[0] + t.G[k][1] * ah[1] + t.G[k][2] * ah[2];
                Ba[k] = t.B[k][0] * ah[0] + t.B[k][1] * ah[1] + t.B[k][2] * ah[2];
            }
        }
#pragma unroll 1
        for (int qb = qa; qb < NE; qb++) {
            const int nbn = nid[qb];
            const int dxo = qb % NX - ia, dyo = (qb / NX) % NY - ja, dzo = qb / (NX * NY) - ka;
            const int sl = (dxo + OX) + SX * ((dyo + OY) + SY * (dzo + OZ));
            const R db[3] = {dN[qb][0], dN[qb][1], dN[qb][2]};
            R K[3][3];
            if (!t.general) {
                const R dg = T[0] * db[0] + T[1] * db[1] + T[2] * db[2];
#pragma unroll
                for (int i = 0; i < 3; i++)
#pragma unroll
                    for (int j = 0; j < 3; j++) K[i][j] = L[i] * db[j] + M[j] * db[i] + (i == j ? dg : (R)0);
            } else {
                R Bb[3], Gb[3];
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    Bb[k] = t.B[k][0] * db[0] + t.B[k][1] * db[1] + t.B[k][2] * db[2];
                    Gb[k] = t.Gp[k][0] * db[0] + t.Gp[k][1] * db[1] + t.Gp[k][2] * db[2];
                }
                const R ab = ah[0] * db[0] + ah[1] * db[1] + ah[2] * db[2];
                const R aBb = ah[0] * Bb[0] + ah[1] * Bb[1] + ah[2] * Bb[2];
                const R sab = Sa[0] * db[0] + Sa[1] * db[1] + Sa[2] * db[2];
                const R dg = t.alpha * ab + sab;
                const R bsc = t.beta * aBb;
#pragma unroll
                for (int i = 0; i < 3; i++)
#pragma unroll
                    for (int j = 0; j < 3; j++)
                        K[i][j] = Ga[i] * db[j] + ah[i] * Gb[j] + t.gam * db[i] * ah[j] + t.eps * Ba[i] * Bb[j] +
                                  t.delta * Bb[i] * Ba[j] + bsc * t.B[i][j] + (i == j ? dg : (R)0);
            }
            if (qa == qb) {
#pragma unroll
                for (int i = 0; i < 3; i++) K[i][i] += am * emd;
            }
#pragma unroll
            for (int i = 0; i < 3; i++)
#pragma unroll
                for (int j = 0; j < 3; j++) {
                    atomicAdd(&A[aidx(sl * 9 + 3 * i + j, na, a.qp)], K[i][j]);
                    if (qb != qa) atomicAdd(&A[aidx((NS - 1 - sl) * 9 + 3 * j + i, nbn, a.qp)], K[i][j]);
                }
        }
        const R f0 = -vol * (sk[0] * dN[qa][0] + sk[5] * dN[qa][1] + sk[4] * dN[qa][2]) + Nw[qa] * (m * fx);
        const R f1 = -vol * (sk[5] * dN[qa][0] + sk[1] * dN[qa][1] + sk[3] * dN[qa][2]) + Nw[qa] * (m * fy);
        const R f2 = -vol * (sk[4] * dN[qa][0] + sk[3] * dN[qa][1] + sk[2] * dN[qa][2]) + Nw[qa] * (m * fz);
        atomicAdd(&b[na], (double)f0);
        atomicAdd(&b[N + na], (double)f1);
        atomicAdd(&b[2 * N + na], (double)f2);
    }
}

// AddInertialForceToRHS (material_point.h:151-161) and the diagonal of the
// scaling D^-1/2 (crsmat.cpp:87-146, FEM_flag false)
template <typename R>
__global__ void k_imp_rhs_diag(ImpArgs a, const R *A, const double *nmass, const double *naccel_k,
                               const double *naccel, double *b, double *adiag) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= a.nodec) return;
    const size_t N = (size_t)a.nodec;
    const int dslot = (a.ns - 1) / 2;
    for (int c = 0; c < 3; c++) {
        const double aam = a.am * naccel_k[c * N + n] + (1.0 - a.am) * naccel[c * N + n];
        b[c * N + n] -= nmass[n] * aam;
        const double dg = fabs((double)A[aidx(dslot * 9 + 4 * c, n, a.qp)]);
        adiag[c * N + n] = dg < a.mtol ? 0.0 : 1.0 / sqrt(dg);
    }
}

// ApplyDiagonalScaling (crsmat.cpp:152-172)
template <typename R>
__global__ void k_imp_scale(ImpArgs a, R *A, const double *adiag) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= a.nodec) return;
    const size_t N = (size_t)a.nodec;
    int i, j, k;
    node_ijk(n, a.nnc, i, j, k);
    const int sx = 2 * a.rad[0] + 1, sy = 2 * a.rad[1] + 1;
    for (int s = 0; s < a.ns; s++) {
        const int ii = i + s % sx - a.rad[0], jj = j + (s / sx) % sy - a.rad[1], kk = k + s / (sx * sy) - a.rad[2];
        if (ii < 0 || jj < 0 || kk < 0 || ii >= a.nnc[0] || jj >= a.nnc[1] || kk >= a.nnc[2]) continue;
        const size_t col = ii + (size_t)a.nnc[0] * (jj + (size_t)a.nnc[1] * kk);
        if constexpr (sizeof(R) == 8) {
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) A[aidx(s * 9 + 3 * r + c, n, a.qp)] *= adiag[r * N + n] * adiag[c * N + col];
        } else {
            // the FP32 matrix is scaled in FP32 (one FP64 operation per entry
            // would make this pass FP64-pipe bound)
            const float dr[3] = {(float)adiag[n], (float)adiag[N + n], (float)adiag[2 * N + n]};
            const float dc[3] = {(float)adiag[col], (float)adiag[N + col], (float)adiag[2 * N + col]};
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) A[aidx(s * 9 + 3 * r + c, n, a.qp)] *= dr[r] * dc[c];
        }
    }
}

// ----------------------------------------------------------- reductions
// Per-block partial sums in fixed order; k_finish adds the partials in index order.
__device__ __forceinline__ double block_sum(double v, double *sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) r += sh[w];
    return r;
}

// Warp sums of V values (V a power of two <= 32) with the values spread over
// the lanes as the butterfly goes: at each of the first log2(V) steps a lane
// keeps half of its values and adds its partner's copy of that half, so a
// lane adds 2V - 1 + log2(32 / V) numbers instead of 5 V.  FP64 adds are the
// scarce resource on this part.  Returns the value index whose warp total the
// lane holds in v[0] (every lane of a group of 32 / V lanes holds it).
template <int V, typename T>
__device__ __forceinline__ int warp_sums(T (&v)[V]) {
    const int lane = threadIdx.x & 31;
    int j = 0, o = 16;
#pragma unroll
    for (int h = V / 2; h >= 1; h /= 2, o >>= 1) {
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int i = 0; i < h; i++) {
            const T send = up ? v[i] : v[i + h];
            const T keep = up ? v[i + h] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
        if (up) j += h;
    }
    for (; o >= 1; o >>= 1) v[0] += __shfl_xor_sync(0xffffffffu, v[0], o);
    return j;
}

template <int V>
__device__ __forceinline__ bool partials_last(const double (&vin)[V], int nv, double *part, unsigned *cnt) {
    __shared__ double sh[V][8];
    __shared__ bool s_last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    double v[V];
#pragma unroll
    for (int j = 0; j < V; j++) v[j] = vin[j];
    const int j = warp_sums<V>(v);
    if ((lane & (32 / V - 1)) == 0) sh[j][wid] = v[0];
    __syncthreads();
    if ((int)threadIdx.x < nv) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[threadIdx.x][w];
        part[threadIdx.x * gridDim.x + blockIdx.x] = t;
        __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(cnt, 1u) == gridDim.x - 1;
    __syncthreads();
    if (s_last) __threadfence();
    return s_last;
}

// in the last block: the total of value j over all blocks (thread 0)
__device__ __forceinline__ double last_sum(const double *part, int j, double *sh32) {
    double acc = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) acc += __ldcg(part + (size_t)j * gridDim.x + i);
    return block_sum(acc, sh32);
}

__global__ void k_finish(const double *part, int nblk, double *out, int slot) {
    __shared__ double sh[32];
    double acc = 0.0;
    for (int i = threadIdx.x; i < nblk; i += blockDim.x) acc += part[i];
    const double t = block_sum(acc, sh);
    if (threadIdx.x == 0) out[slot] = t;
}

// y = A x with BC rows zeroed (MatVecMult + BCResidualSet), optional dot(x, y).
// TA: storage of A; TC: arithmetic (FP32 in the Krylov iterations of the
// FP32 operator, FP64 for its true residual and in the FP64 mode); TV: the
// vectors x and y (FP64, or FP32 for the flexible GCR directions of the FP32
// operator).  RX, RY, RZ: the stencil radius per axis.
template <typename TA, typename TC, int RX, int RY, int RZ, typename TV = double>
__global__ void __launch_bounds__(256) k_imp_matvec(ImpArgs a, const TA *A, const TV *x, TV *y,
                                                    double *part, unsigned *cnt = nullptr, double *scal = nullptr,
                                                    int slot = 0) {
    using TA2 = typename std::conditional<sizeof(TA) == 8, double2, float2>::type;
    constexpr int SX = 2 * RX + 1, SY = 2 * RY + 1, NS = SX * SY * (2 * RZ + 1);
    __shared__ double sh[32];
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    double dot = 0.0;
    if (n < a.nodec) {
        const size_t N = (size_t)a.nodec;
        int i, j, k;
        node_ijk(n, a.nnc, i, j, k);
        TC acc[3] = {(TC)0, (TC)0, (TC)0};
#pragma unroll
        for (int s = 0; s < NS; s++) {
            const int ii = i + s % SX - RX, jj = j + (s / SX) % SY - RY, kk = k + s / (SX * SY) - RZ;
            if (ii < 0 || jj < 0 || kk < 0 || ii >= a.nnc[0] || jj >= a.nnc[1] || kk >= a.nnc[2]) continue;
            const size_t col = ii + (size_t)a.nnc[0] * (jj + (size_t)a.nnc[1] * kk);
            const TC x0 = (TC)x[col], x1 = (TC)x[N + col], x2 = (TC)x[2 * N + col];
            // the block's 9 entries: 4 aligned pairs and 1 single (which end depends on the parity of 9 s)
            TC e[9];
            if ((s & 1) == 0) {
#pragma unroll
                for (int t = 0; t < 4; t++) {
                    const TA2 v = __ldg(reinterpret_cast<const TA2 *>(A + aidx(s * 9 + 2 * t, n, a.qp)));
                    e[2 * t] = (TC)v.x;
                    e[2 * t + 1] = (TC)v.y;
                }
                e[8] = (TC)__ldg(A + aidx(s * 9 + 8, n, a.qp));
            } else {
                e[0] = (TC)__ldg(A + aidx(s * 9, n, a.qp));
#pragma unroll
                for (int t = 0; t < 4; t++) {
                    const TA2 v = __ldg(reinterpret_cast<const TA2 *>(A + aidx(s * 9 + 1 + 2 * t, n, a.qp)));
                    e[1 + 2 * t] = (TC)v.x;
                    e[2 + 2 * t] = (TC)v.y;
                }
            }
            // chained FMAs: in FP64 the FP64 pipe is this kernel's limit, and a
            // separate product and add per entry would cost a third more
#pragma unroll
            for (int r = 0; r < 3; r++) acc[r] = fma(e[3 * r + 2], x2, fma(e[3 * r + 1], x1, fma(e[3 * r], x0, acc[r])));
        }
        const unsigned char bf = a.bcflag[n];
        for (int c = 0; c < 3; c++) {
            const double v = (bf & (1 << c)) ? 0.0 : (double)acc[c];
            y[c * N + n] = (TV)v;
            dot += (double)x[c * N + n] * v;
        }
    }
    if (part && cnt) {   // dot(x, y) reduced by the last block into scal[slot]
        const double v[1] = {dot};
        if (!partials_last<1>(v, 1, part, cnt)) return;
        const double t = last_sum(part, 0, sh);
        if (threadIdx.x == 0) {
            scal[slot] = t;
            *cnt = 0u;
        }
    } else if (part) {
        const double t = block_sum(dot, sh);
        if (threadIdx.x == 0) part[blockIdx.x] = t;
    }
}

// x = xh + xl with FP32 parts (xl the rounding error of xh): 48 bits of x
__global__ void k_split_df(const double *__restrict__ x, float *__restrict__ xh, float *__restrict__ xl, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = x[i];
    const float h = (float)v;
    xh[i] = h;
    xl[i] = (float)(v - (double)h);
}

// y = A x for the FP32-stored stencil of the FP32 operator, in double-float
// arithmetic instead of FP64 (the true residual and the Newton check): each
// product e x = e (xh + xl) is e xh exactly (an FMA gives its rounding error)
// plus e xl, and the row sums are carried as an unevaluated FP32 pair
// (Knuth's two-sum for the high part).  About 44 bits of the sum, on the FP32
// pipe (GB300 executes 2 FP64 FMAs per SM and clock, against 128 FP32 lanes).
template <int RX, int RY, int RZ>
__global__ void __launch_bounds__(256) k_imp_matvec_df(ImpArgs a, const float *A, const float *__restrict__ xh,
                                                       const float *__restrict__ xl, double *y) {
    constexpr int SX = 2 * RX + 1, SY = 2 * RY + 1, NS = SX * SY * (2 * RZ + 1);
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= a.nodec) return;
    const size_t N = (size_t)a.nodec;
    int i, j, k;
    node_ijk(n, a.nnc, i, j, k);
    float sh[3] = {0.0f, 0.0f, 0.0f}, sl[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int s = 0; s < NS; s++) {
        const int ii = i + s % SX - RX, jj = j + (s / SX) % SY - RY, kk = k + s / (SX * SY) - RZ;
        if (ii < 0 || jj < 0 || kk < 0 || ii >= a.nnc[0] || jj >= a.nnc[1] || kk >= a.nnc[2]) continue;
        const size_t col = ii + (size_t)a.nnc[0] * (jj + (size_t)a.nnc[1] * kk);
        const float h[3] = {__ldg(xh + col), __ldg(xh + N + col), __ldg(xh + 2 * N + col)};
        const float l[3] = {__ldg(xl + col), __ldg(xl + N + col), __ldg(xl + 2 * N + col)};
        float e[9];
        if ((s & 1) == 0) {
#pragma unroll
            for (int t = 0; t < 4; t++) {
                const float2 v = __ldg(reinterpret_cast<const float2 *>(A + aidx(s * 9 + 2 * t, n, a.qp)));
                e[2 * t] = v.x;
                e[2 * t + 1] = v.y;
            }
            e[8] = __ldg(A + aidx(s * 9 + 8, n, a.qp));
        } else {
            e[0] = __ldg(A + aidx(s * 9, n, a.qp));
#pragma unroll
            for (int t = 0; t < 4; t++) {
                const float2 v = __ldg(reinterpret_cast<const float2 *>(A + aidx(s * 9 + 1 + 2 * t, n, a.qp)));
                e[1 + 2 * t] = v.x;
                e[2 + 2 * t] = v.y;
            }
        }
#pragma unroll
        for (int r = 0; r < 3; r++)
#pragma unroll
            for (int c = 0; c < 3; c++) {
                // round-to-nearest intrinsics: the compiler may not fuse or
                // reorder them, which the error-free transformations rely on
                const float ev = e[3 * r + c];
                const float p = __fmul_rn(ev, h[c]);
                const float pe = fmaf(ev, h[c], -p);   // e xh - p, exactly
                const float sum = __fadd_rn(sh[r], p);   // two-sum of sh and p
                const float bp = __fsub_rn(sum, sh[r]);
                const float err = __fadd_rn(__fsub_rn(sh[r], __fsub_rn(sum, bp)), __fsub_rn(p, bp));
                sh[r] = sum;
                sl[r] += err + fmaf(ev, l[c], pe);
            }
    }
    const unsigned char bf = a.bcflag[n];
#pragma unroll
    for (int c = 0; c < 3; c++) y[c * N + n] = (bf & (1 << c)) ? 0.0 : (double)sh[c] + (double)sl[c];
}

// ScaleSolution + BCResidualSet: xs = x / D, r = b D (crsmat.cpp:190-209)
__global__ void k_cg_scale_in(ImpArgs a, const double *x, const double *b, const double *adiag, double *xs,
                              double *rr) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= a.nodec) return;
    const size_t N = (size_t)a.nodec;
    const unsigned char bf = a.bcflag[n];
    for (int c = 0; c < 3; c++) {
        const size_t i = c * N + n;
        const double dg = adiag[i];
        if (dg < a.mtol) {
            xs[i] = 0.0;
            rr[i] = 0.0;
        } else {
            xs[i] = x[i] / dg;
            rr[i] = b[i] * dg;
        }
        if (bf & (1 << c)) rr[i] = 0.0;
    }
}

// r = rr - Ax, p = r, partial r.r
__global__ void k_cg_init(ImpArgs a, const double *Ax, double *r, double *p, double *part) {
    __shared__ double sh[32];
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    double dot = 0.0;
    if (n < a.nodec) {
        const size_t N = (size_t)a.nodec;
        for (int c = 0; c < 3; c++) {
            const size_t i = c * N + n;
            const double v = r[i] - Ax[i];
            r[i] = v;
            p[i] = v;
            dot += v * v;
        }
    }
    const double t = block_sum(dot, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// num / den (0 when den is 0 or `zero`) evaluated by one thread of the block
// and shared: an FP64 division costs tens of FP64-pipe operations on this
// part, too many to repeat in every thread.  Every thread of the block must
// call it (it synchronises the block), at most once per kernel.
__device__ __forceinline__ double block_div(double num, double den, bool zero = false) {
    __shared__ double s_q;
    if (threadIdx.x == 0) s_q = (zero || den == 0.0) ? 0.0 : num / den;
    __syncthreads();
    return s_q;
}

// x += alpha p, r -= alpha Ap, then (last block) r.r;  alpha = rr_cur / pAp
__global__ void k_cg_update(ImpArgs a, double *scal, int cur, double *x, double *r, const double *p,
                            const double *Ap, double *part, unsigned *cnt) {
    __shared__ double sh[32];
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const double alpha = block_div(scal[cur], scal[S_PAP]);
    double dot = 0.0;
    if (n < a.nodec) {
        const size_t N = (size_t)a.nodec;
        for (int c = 0; c < 3; c++) {
            const size_t i = c * N + n;
            x[i] += alpha * p[i];
            const double v = r[i] - alpha * Ap[i];
            r[i] = v;
            dot += v * v;
        }
    }
    const double v[1] = {dot};
    if (!partials_last<1>(v, 1, part, cnt)) return;
    const double t = last_sum(part, 0, sh);
    if (threadIdx.x == 0) {
        scal[cur ^ 1] = t;
        *cnt = 0u;
    }
}

// p = r + beta p;  beta = rr_new / rr_cur
__global__ void k_cg_dir(ImpArgs a, const double *scal, int cur, const double *r, double *p) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const double beta = block_div(scal[cur ^ 1], scal[cur]);
    if (n >= a.nodec) return;
    const size_t N = (size_t)a.nodec;
    for (int c = 0; c < 3; c++) {
        const size_t i = c * N + n;
        p[i] = r[i] + beta * p[i];
    }
}

// RestorSolution: x = xs D (crsmat.cpp:214-230)
__global__ void k_cg_scale_out(ImpArgs a, const double *xs, const double *adiag, double *x) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= 3 * a.nodec) return;
    x[n] = adiag[n] > a.mtol ? xs[n] * adiag[n] : 0.0;
}

// Newton residual of the linear system (ComputeRefResidual / ComputeAbsResidual,
// solver.cpp:484-555): b with BC rows zeroed, r = b - (A (x / D)) / D
__global__ void k_imp_prepare_residual(ImpArgs a, const double *x, const double *adiag, double *b, double *xs) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= a.nodec) return;
    const size_t N = (size_t)a.nodec;
    const unsigned char bf = a.bcflag[n];
    for (int c = 0; c < 3; c++) {
        const size_t i = c * N + n;
        if (bf & (1 << c)) b[i] = 0.0;
        xs[i] = adiag[i] > a.mtol ? x[i] / adiag[i] : 0.0;
    }
}

__global__ void k_imp_residual(ImpArgs a, const double *Ax, const double *adiag, const double *b, double *part) {
    __shared__ double sh[32];
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    double rr = 0.0, cnt = 0.0;
    if (n < a.nodec) {
        const size_t N = (size_t)a.nodec;
        for (int c = 0; c < 3; c++) {
            const size_t i = c * N + n;
            const double axp = adiag[i] > a.mtol ? Ax[i] / adiag[i] : 0.0;
            const double r = b[i] - axp;
            rr += r * r;
            if (adiag[i] > a.mtol) cnt += 1.0;
        }
    }
    const double t = block_sum(rr, sh);
    const double u = block_sum(cnt, sh);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = t;
        part[gridDim.x + blockIdx.x] = u;
    }
}

// ---------------------------------------------------------------- G2P
// nei = max(0, nvof - nvol) and sum nei^2 (material_point.cpp:175-185)
__global__ void k_imp_nei(ImpArgs a, const double *nvof, double *nei, double *part) {
    __shared__ double sh[32];
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    double e2 = 0.0;
    if (n < a.nodec) {
        const double e = fmax(0.0, -a.nvol[n] + nvof[n]);
        nei[n] = e;
        e2 = e * e;
    }
    const double t = block_sum(e2, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// Node2Particle (var_trans_solid_implicit.cpp:202-255) with the nodal kinematics
// already committed: F, J, vol, stress, displacement/acceleration/velocity
// gathers and the shifting gradient; CommitParticleKinematics without the shift.
template <typename R, int OX, int OY, int OZ>
__global__ void __launch_bounds__(128) k_imp_g2p(ImpArgs a, PView<R> P, const double *ndispl, const double *nvel,
                                                 const double *naccel, const double *nei, R *geup, double *part,
                                                 DevCtl *ctl, int parity) {
    constexpr int NE = (OX + 1) * (OY + 1) * (OZ + 1);
    __shared__ double sh[32];
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    double gd = 0.0;
    if (p < a.num) {
        const size_t N = (size_t)a.nodec, NP = (size_t)a.num;
        const KGeom<R> g = kgeom<R>(a);
        const R x[3] = {P.x[0][p], P.x[1][p], P.x[2][p]};
        int nid[NE];
        R Nw[NE], dN[NE][3];
        bool oob = false;
        shape_nodes<R, OX, OY, OZ>(a, g, x, Nw, dN, nid, oob);
        R Dm[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (int q = 0; q < NE; q++)
            for (int r = 0; r < 3; r++) {
                const R u = (R)ndispl[r * N + nid[q]];
                for (int c = 0; c < 3; c++) Dm[r][c] += dN[q][c] * (R)1 * u;
            }
        R d[3][3];
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) d[r][c] = Dm[r][c] + (r == c ? (R)1 : (R)0);
        R Fn[3][3], Hn[3][3], J, jm1;
        if constexpr (sizeof(R) == 8) {
            R F[3][3];
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) F[r][c] = P.F[3 * r + c][p];
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) {
                    R sum = 0.0;
                    for (int k = 0; k < 3; k++) sum += d[r][k] * F[k][c];
                    Fn[r][c] = sum;
                }
            J = det3(Fn);
            jm1 = J - (R)1;
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) P.F[3 * r + c][p] = Fn[r][c];
        } else {
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) {
                    R sum = Dm[r][c] + P.F[3 * r + c][p];
                    for (int k = 0; k < 3; k++) sum += Dm[r][k] * P.F[3 * k + c][p];
                    Hn[r][c] = sum;
                }
            jm1 = det_ipm1(Hn);
            J = (R)1 + jm1;
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) {
                    Fn[r][c] = Hn[r][c] + (r == c ? (R)1 : (R)0);
                    P.F[3 * r + c][p] = Hn[r][c];
                }
        }
        const R vol = J * P.vol0[p];
        P.vol[p] = vol;
        R sk[6];
        for (int k = 0; k < 6; k++) sk[k] = P.s[k][p];
        const int mid = P.matid[p];
        const int model = a.iprop[mid];
        const R E = (R)a.matprop[3 * mid], nu = (R)a.matprop[3 * mid + 1], m3 = (R)a.matprop[3 * mid + 2];
        if (model == 0) {
            R De[3][3];
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++)
                    De[r][c] = sizeof(R) == 8 ? (r == c ? d[r][c] - (R)1 : d[r][c]) : Dm[r][c];
            lin_elast_update(sk, De, E, nu);
        } else if (model == 1) {
            if constexpr (sizeof(R) == 8) neo_hookean_stress(sk, Fn, J, E, nu);
            else neo_hookean_stress_h(sk, Hn, jm1, E, nu);
        } else if (model == 2) {
            if constexpr (sizeof(R) == 8) stvk_stress(sk, Fn, J, E, nu);
            else stvk_stress_h(sk, Hn, jm1, E, nu);
        } else if (model == 3) {
            if constexpr (sizeof(R) == 8) mooney_rivlin_stress(sk, Fn, J, E, nu, m3);
            else mooney_rivlin_stress_h(sk, Hn, jm1, E, nu, m3);
        } else {
            for (int k = 0; k < 6; k++) sk[k] = (R)0;
        }
        for (int k = 0; k < 6; k++) P.s[k][p] = sk[k];
        const bool flip = (a.scheme == MPM_FLIP);
        // gathers in the particle precision (FP64 arithmetic for FP32
        // particles would make this pass FP64-pipe bound)
        R disp[3] = {0, 0, 0}, acc[3] = {0, 0, 0}, vel[3] = {0, 0, 0};
        const R aold[3] = {P.acc[0][p], P.acc[1][p], P.acc[2][p]};
        if (model != -1) {
            for (int q = 0; q < NE; q++)
                for (int c = 0; c < 3; c++) {
                    disp[c] += Nw[q] * (R)ndispl[c * N + nid[q]];
                    acc[c] += Nw[q] * (R)naccel[c * N + nid[q]];
                    vel[c] += Nw[q] * (R)nvel[c * N + nid[q]];
                }
        }
        // shifting gradient at the old position with the new volume (material_point.cpp:192-216)
        R gv[3] = {0, 0, 0};
        for (int q = 0; q < NE; q++)
            for (int c = 0; c < 3; c++) gv[c] += dN[q][c] * (R)nei[nid[q]];
        for (int c = 0; c < 3; c++) {
            gv[c] *= (R)2 * vol;
            geup[c * NP + p] = gv[c];
            gd += (double)gv[c] * (double)gv[c];
        }
        // CommitParticleKinematics (nonlinear_time_integration.cpp:83-96), shift added by k_imp_shift
        float amax = 0.0f, vmax = 0.0f;
        const R dtr = (R)a.dt, gam = (R)a.gamma;
        for (int c = 0; c < 3; c++) {
            const R vc = flip ? P.v[c][p] + dtr * (((R)1 - gam) * aold[c] + gam * acc[c]) : vel[c];
            P.v[c][p] = vc;
            P.acc[c][p] = acc[c];
            P.x[c][p] = x[c] + disp[c];
            amax = fmaxf(amax, (float)fabs(acc[c]));
            vmax = fmaxf(vmax, (float)fabs(vc));
        }
        const float rs = (float)fmax(fabs((double)sk[0]) + fabs((double)sk[5]) + fabs((double)sk[4]),
                                     fmax(fabs((double)sk[5]) + fabs((double)sk[1]) + fabs((double)sk[3]),
                                          fabs((double)sk[4]) + fabs((double)sk[3]) + fabs((double)sk[2])));
        atomic_max_pos(&ctl->nxt[parity ^ 1][B_AMAX], amax * 1.000001f);
        atomic_max_pos(&ctl->nxt[parity ^ 1][B_VMAX], vmax * 1.000001f);
        atomic_max_pos(&ctl->nxt[parity ^ 1][B_VOLMAX], (float)fabs((double)vol) * 1.000001f);
        atomic_max_pos(&ctl->nxt[parity ^ 1][B_VOLSMAX], (float)fabs((double)vol) * rs * 1.000001f);
    }
    const double t = block_sum(gd, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// x += -b0 geup, b0 = eu / gd unless gd < mtol (material_point.cpp:219-225)
template <typename R>
__global__ void k_imp_shift(ImpArgs a, PView<R> P, const R *geup, const double *scal) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const double gd = scal[S_GD];
    const double b0 = block_div(scal[S_EU], gd, gd < a.mtol);
    if (p >= a.num || !a.shifting || b0 == 0.0) return;
    const size_t NP = (size_t)a.num;
    for (int c = 0; c < 3; c++) P.x[c][p] = (R)((double)P.x[c][p] + -b0 * (double)geup[c * NP + p]);
}

// ------------------------------------------------ flexible CG (Notay's FCG(1))
// partial dot u.w over the 3 * nodec vector (node-blocked like the matvec)
__global__ void k_dot3(ImpArgs a, const double *u, const double *w, double *part) {
    __shared__ double sh[32];
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    double d = 0.0;
    if (n < a.nodec) {
        const size_t N = (size_t)a.nodec;
        for (int c = 0; c < 3; c++) d += u[c * N + n] * w[c * N + n];
    }
    const double t = block_sum(d, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// p = z - (z.q_prev / p_prev.q_prev) p_prev (p = z on a restart); partial p.r
__global__ void k_fcg_dir(ImpArgs a, const double *scal, int restart, const double *z, const double *r, double *p,
                          double *part) {
    __shared__ double sh[32];
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const double beta = block_div(-scal[S_ZQ], scal[S_PAP], restart != 0);
    double d = 0.0;
    if (n < a.nodec) {
        const size_t N = (size_t)a.nodec;
        for (int c = 0; c < 3; c++) {
            const size_t i = c * N + n;
            const double v = z[i] + beta * p[i];
            p[i] = v;
            d += v * r[i];
        }
    }
    const double t = block_sum(d, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// alpha = p.r / p.q; x += alpha p; r -= alpha q; partial r.r
__global__ void k_fcg_update(ImpArgs a, const double *scal, double *x, double *r, const double *p, const double *q,
                             double *part) {
    __shared__ double sh[32];
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const double alpha = block_div(scal[S_PR], scal[S_PAP]);
    double d = 0.0;
    if (n < a.nodec) {
        const size_t N = (size_t)a.nodec;
        for (int c = 0; c < 3; c++) {
            const size_t i = c * N + n;
            x[i] += alpha * p[i];
            const double v = r[i] - alpha * q[i];
            r[i] = v;
            d += v * v;
        }
    }
    const double t = block_sum(d, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// true residual r = bs - Ax (scaled system, BC rows already zero in Ax and bs); partial r.r
__global__ void k_true_residual(ImpArgs a, const double *bs, const double *Ax, double *r, double *part) {
    __shared__ double sh[32];
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    double d = 0.0;
    if (n < a.nodec) {
        const size_t N = (size_t)a.nodec;
        for (int c = 0; c < 3; c++) {
            const size_t i = c * N + n;
            const double v = bs[i] - Ax[i];
            r[i] = v;
            d += v * v;
        }
    }
    const double t = block_sum(d, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// network feature channels: the mass term's share of each diagonal entry,
// phi = alpha_m nb3 nmass / diag (diag = 1 / adiag^2), clamped to [0, 1]
__global__ void k_phi(ImpArgs a, const double *nmass, const double *adiag, double *phi) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= a.nodec) return;
    const size_t N = (size_t)a.nodec;
    for (int c = 0; c < 3; c++) {
        const double d = adiag[c * N + n];
        const double v = a.am * a.nb[3] * nmass[n] * d * d;
        phi[c * N + n] = v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v);
    }
}

// e = xstar - x
__global__ void k_sub3(const double *xstar, const double *x, double *e, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) e[i] = xstar[i] - x[i];
}

// seeded random right-hand side of the scaled system for training-pair
// harvesting: a few random low-wavenumber cosine modes per component
// (wavenumber 0, a uniform load, included) plus white noise, zero on
// inactive and boundary rows
__device__ __forceinline__ uint64_t hash64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ double hash_unit(uint64_t k) { return ((hash64(k) >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

__global__ void k_random_rhs(ImpArgs a, const double *adiag, uint64_t seed, double smooth_amp, double noise_amp,
                             double *bs) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= a.nodec) return;
    int i, j, k;
    node_ijk(n, a.nnc, i, j, k);
    const size_t N = (size_t)a.nodec;
    const unsigned char bf = a.bcflag[n];
    for (int c = 0; c < 3; c++) {
        double v = 0.0;
        for (int m = 0; m < 4; m++) {
            const uint64_t key = seed * 1315423911ull + (uint64_t)(c * 4 + m) * 97;
            const double kx = floor(4.0 * hash_unit(key + 1)), ky = floor(4.0 * hash_unit(key + 2));
            const double kz = floor(4.0 * hash_unit(key + 3));
            const double ph = 6.283185307179586 * hash_unit(key + 4);
            const double amp = 2.0 * hash_unit(key + 5) - 1.0;
            v += amp * cos(3.141592653589793 * (kx * i / a.nnc[0] + ky * j / a.nnc[1] + kz * k / a.nnc[2]) + ph);
        }
        const uint64_t nk = seed * 2654435761ull + (uint64_t)n * 3 + c;
        const double u1 = hash_unit(nk * 2 + 11), u2 = hash_unit(nk * 2 + 12);
        const double g = sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
        const size_t idx = c * N + n;
        const bool off = (bf & (1 << c)) || !(adiag[idx] >= a.mtol);
        bs[idx] = off ? 0.0 : smooth_amp * v + noise_amp * g;
    }
}

__global__ void k_set_modulus(double *matprop, int nmat, double E) {
    const int m = threadIdx.x;
    if (m < nmat) matprop[3 * m] = E;
}

// ------------------------------------------------ flexible GCR(GM)
// slot of the direction kept j + 1 iterations before the one in `slot` (ring of w)
__device__ __forceinline__ int gcr_prev(int slot, int j, int w) { return (slot - 1 - j + 2 * w) % w; }

// partial dots q . Q_j with the `used` previous images (j = 0 the newest)
// Per-block partial sums of nv (<= V) values into part[j * gridDim.x + b];
// true in the last block to finish (the blocks count themselves on *cnt),
// which then reduces the partials in block order (last_sum), so the sums
// are reproducible without a separate reduction launch.
// flexible GCR: the dots q . Q_j of the new image with the kept ones, then
// (last block) beta_j = (q . Q_j) / (Q_j . Q_j).  beta only has to be close:
// the same beta_j update both the direction and its image (k_gcr_axpy, in
// FP64), so A p = q holds whatever their accuracy and only the
// orthogonality of the kept images is at FP32 level.  So the dots run in
// FP32 on FP32 copies of the kept images (the FP64 pipe is this part's
// scarce resource), and the block partials are summed in FP64.
template <typename T>
__global__ void __launch_bounds__(256) k_gcr_dots(ImpArgs a, const T *Q, const float *Qf, int slot, int used,
                                                  int w, double *part, unsigned *cnt, const double *qq,
                                                  double *beta) {
    __shared__ double sh[32];
    __shared__ double shw[GM][8];
    __shared__ bool s_last;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const size_t N = (size_t)a.nodec, st = 3 * N;
    float d[GM];
#pragma unroll
    for (int j = 0; j < GM; j++) d[j] = 0.0f;
    if (n < a.nodec) {
        const T *q = Q + (size_t)slot * st;
        const float q0 = (float)q[n], q1 = (float)q[N + n], q2 = (float)q[2 * N + n];
#pragma unroll
        for (int j = 0; j < GM; j++)
            if (j < used) {
                const float *qj = Qf + (size_t)gcr_prev(slot, j, w) * st;
                d[j] = q0 * qj[n] + q1 * qj[N + n] + q2 * qj[2 * N + n];
            }
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int jv = warp_sums<GM>(d);
    if ((lane & (32 / GM - 1)) == 0) shw[jv][wid] = (double)d[0];
    __syncthreads();
    if ((int)threadIdx.x < used) {
        double t = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) t += shw[threadIdx.x][q];
        part[threadIdx.x * gridDim.x + blockIdx.x] = t;
        __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(cnt, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    for (int j = 0; j < used; j++) {
        const double t = last_sum(part, j, sh);
        if (threadIdx.x == 0) {
            const double dq = qq[gcr_prev(slot, j, w)];
            beta[j] = dq > 0.0 ? t / dq : 0.0;
        }
    }
    if (threadIdx.x == 0) *cnt = 0u;
}

// p -= sum beta_j P_j, q -= sum beta_j Q_j in the precision T of the
// directions (FP64: an FP32 copy of q is kept for the dots; FP32: the images
// themselves are what the dots read, Qf is null); then (last block) q.r and
// q.q in FP64
template <typename T>
__global__ void __launch_bounds__(256) k_gcr_axpy(ImpArgs a, T *P, T *Q, float *Qf, int slot, int used,
                                                  int w, const double *beta, const double *r, double *part,
                                                  unsigned *cnt, double *scal) {
    __shared__ double sh[32];
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const size_t N = (size_t)a.nodec, st = 3 * N;
    double v[2] = {0.0, 0.0};
    if (n < a.nodec) {
        T *p = P + (size_t)slot * st, *q = Q + (size_t)slot * st;
        T bj[GM];
#pragma unroll
        for (int j = 0; j < GM; j++) bj[j] = j < used ? (T)beta[j] : (T)0;
        for (int c = 0; c < 3; c++) {
            const size_t i = c * N + n;
            T pv = p[i], qv = q[i];
#pragma unroll
            for (int j = 0; j < GM; j++)
                if (j < used) {
                    const size_t o = (size_t)gcr_prev(slot, j, w) * st + i;
                    pv -= bj[j] * P[o];
                    qv -= bj[j] * Q[o];
                }
            p[i] = pv;
            q[i] = qv;
            if (Qf) Qf[(size_t)slot * st + i] = (float)qv;   // the copy k_gcr_dots reads
            v[0] += (double)qv * r[i];
            v[1] += (double)qv * (double)qv;
        }
    }
    if (!partials_last<2>(v, 2, part, cnt)) return;
    const double qr = last_sum(part, 0, sh);
    const double qq = last_sum(part, 1, sh);
    if (threadIdx.x == 0) {
        scal[S_QR] = qr;
        scal[S_QQ] = qq;
        *cnt = 0u;
    }
}

// alpha = q.r / q.q; x += alpha p; r -= alpha q; keeps q.q of the slot; then
// (last block) r.r
template <typename T>
__global__ void __launch_bounds__(256) k_gcr_update(ImpArgs a, double *scal, double *x, double *r, const T *P,
                                                    const T *Q, int slot, double *qq, double *part,
                                                    unsigned *cnt) {
    __shared__ double sh[32];
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const size_t N = (size_t)a.nodec, st = 3 * N;
    const double dqq = scal[S_QQ];
    const double alpha = block_div(scal[S_QR], dqq, !(dqq > 0.0));
    if (blockIdx.x == 0 && threadIdx.x == 0) qq[slot] = dqq;
    double v[1] = {0.0};
    if (n < a.nodec) {
        const T *p = P + (size_t)slot * st, *q = Q + (size_t)slot * st;
        for (int c = 0; c < 3; c++) {
            const size_t i = c * N + n;
            x[i] += alpha * (double)p[i];
            const double w = r[i] - alpha * (double)q[i];
            r[i] = w;
            v[0] += w * w;
        }
    }
    if (!partials_last<1>(v, 1, part, cnt)) return;
    const double rr = last_sum(part, 0, sh);
    if (threadIdx.x == 0) {
        scal[S_RRC] = rr;
        *cnt = 0u;
    }
}

__global__ void k_imp_reset_next(DevCtl *ctl, int parity) {
    for (int k = 0; k < B_NB; k++) ctl->nxt[parity ^ 1][k] = 0u;
}

}  // namespace mpm

using namespace mpm;

#define CKI(call)                                                                                                      \
    do {                                                                                                               \
        cudaError_t _e = (call);                                                                                       \
        if (_e != cudaSuccess) {                                                                                       \
            fprintf(stderr, "mpm_gb300: %s failed: %s\n", #call, cudaGetErrorString(_e));                              \
            return _e == cudaErrorMemoryAllocation ? MPM_ERR_OOM : MPM_ERR_CUDA;                                       \
        }                                                                                                              \
    } while (0)

namespace mpm {
void implicit_free(mpm_ctx *c) {
    ImpState *s = c->imp;
    if (!s) return;
    void *bufs[] = {s->A, s->bcval64, s->adiag, s->b, s->x, s->r, s->p, s->Ap, s->xs, s->ndispl, s->nvel, s->naccel,
                      s->naccel_k, s->nmass, s->nvof, s->nei, s->stress_k, s->geup, s->part, s->scal,
                      s->z, s->bs, s->xstar, s->ev, s->gp, s->gq, s->gqq, s->gbeta};
    for (void *b : bufs)
        if (b) cudaFree(b);
    if (s->cnt) cudaFree(s->cnt);
    if (s->gqf) cudaFree(s->gqf);
    if (s->gp32) cudaFree(s->gp32);
    if (s->dfx) cudaFree(s->dfx);
    if (s->gq32) cudaFree(s->gq32);
    if (s->h_scal) cudaFreeHost(s->h_scal);
    for (cudaGraphExec_t g : {s->g_cg, s->g_fcg_nn, s->g_fcg_jac, s->g_gcr})
        if (g) cudaGraphExecDestroy(g);
    delete s;
    c->imp = nullptr;
}
}  // namespace mpm

namespace mpm {
// The FP64 copy of the BC values the implicit kernels read, from the host
// lists of mpm_gpu_set_bc (later entries win, as there).
mpm_status implicit_bc_changed(mpm_ctx *c) {
    ImpState *s = c->imp;
    if (!s || !s->bcval64) return MPM_OK;
    const size_t N = (size_t)c->g.nodec;
    std::vector<double> val(3 * N, 0.0);
    for (int k = 0; k < 3; k++)
        for (size_t i = 0; i < c->bc_nodes[k].size(); i++) val[k * N + c->bc_nodes[k][i]] = c->bc_vals[k][i];
    CKI(cudaStreamSynchronize(c->stream));
    CKI(cudaMemcpy(s->bcval64, val.data(), sizeof(double) * 3 * N, cudaMemcpyHostToDevice));
    return MPM_OK;
}
}  // namespace mpm

static mpm_status ensure_particle_scratch(mpm_ctx *c) {
    ImpState *s = c->imp;
    if (s->num_alloc == c->num && s->stress_k) return MPM_OK;
    if (s->stress_k) cudaFree(s->stress_k);
    if (s->geup) cudaFree(s->geup);
    s->stress_k = s->geup = nullptr;
    size_t n = (size_t)(c->num > 0 ? c->num : 1);
    CKI(cudaMalloc((void **)&s->stress_k, c->rsize * 6 * n));
    CKI(cudaMalloc((void **)&s->geup, c->rsize * 3 * n));
    s->num_alloc = c->num;
    return MPM_OK;
}

mpm_status mpm_gpu_implicit_setup(mpm_ctx *c, int nr_flag, double spec_rad) {
    if (!c) return MPM_ERR_BAD_ARG;
    if (c->nreal != 27) return MPM_ERR_UNSUPPORTED;
    {
        // the shape orders mpm_gpu_create takes: linear, quadratic, or quadratic in x and z
        const int *o = c->g.order;
        const bool ok = (o[0] == 1 && o[1] == 1 && o[2] == 1) || (o[0] == 2 && o[1] == 2 && o[2] == 2) ||
                        (o[0] == 2 && o[1] == 1 && o[2] == 2);
        if (!ok) return MPM_ERR_UNSUPPORTED;
    }
    {
        std::vector<int> ip(c->nmat);
        CKI(cudaMemcpy(ip.data(), c->d_iprop, sizeof(int) * c->nmat, cudaMemcpyDeviceToHost));
        for (int m : ip)
            if (m > 3) return MPM_ERR_UNSUPPORTED;   // no tangent for the fluid model
    }
    implicit_free(c);
    ImpState *s = new ImpState();
    c->imp = s;
    s->debug = getenv("MPM_GB300_KRYLOV_TRACE") != nullptr;
    s->gcr = getenv("MPM_GB300_FCG_ONLY") == nullptr;
    if (const char *w = getenv("MPM_GB300_GCR_WINDOW")) {
        const int v = atoi(w);
        if (v == 1 || v == 2 || v == 4 || v == 8) s->gm = v;   // divides the 8 iterations of a graph launch
    }
    s->nr_flag = nr_flag ? 1 : 0;
    s->prec = c->precision;
    s->qp = imp_args(c).qp;
    // GeneralizedAlphaParaSet + NewmarkBetaParaSet (nonlinear_time_integration.cpp:10-56), second order
    double t = 1.0 + spec_rad;
    s->alpha_f = 1.0 / t;
    s->alpha_m = (2.0 - spec_rad) / t;
    t = 1.0 - s->alpha_f + s->alpha_m;
    s->gamma = t - 0.5;
    s->beta = 0.25 * t * t;
    const double g = s->gamma, b = s->beta, dt = c->dt;
    s->nb[0] = g / (b * dt);
    s->nb[1] = g / b - 1.0;
    s->nb[2] = dt / 2.0 * (g / b - 2.0);
    s->nb[3] = 1.0 / (b * dt * dt);
    s->nb[4] = 1.0 / (b * dt);
    s->nb[5] = 1.0 / (2.0 * b) - 1.0;
    const size_t N = (size_t)c->g.nodec;
    CKI(cudaMalloc((void **)&s->A, (s->prec == 64 ? sizeof(double) : sizeof(float)) * a_size((int)N, s->qp)));
    CKI(cudaMalloc((void **)&s->bcval64, sizeof(double) * 3 * N));
    {
        const mpm_status q = implicit_bc_changed(c);
        if (q != MPM_OK) return q;
    }
    double **vec3[] = {&s->adiag, &s->b,    &s->x,       &s->r, &s->p,  &s->Ap,    &s->xs, &s->ndispl,
                       &s->nvel,  &s->naccel, &s->naccel_k, &s->z, &s->bs, &s->xstar, &s->ev};
    for (double **v : vec3) CKI(cudaMalloc((void **)v, sizeof(double) * 3 * N));
    CKI(cudaMalloc((void **)&s->gp, sizeof(double) * GM * 3 * N));
    CKI(cudaMalloc((void **)&s->gq, sizeof(double) * GM * 3 * N));
    CKI(cudaMalloc((void **)&s->gqq, sizeof(double) * GM));
    CKI(cudaMalloc((void **)&s->gbeta, sizeof(double) * GM));
    CKI(cudaMalloc((void **)&s->gqf, sizeof(float) * GM * 3 * N));
    if (s->prec == 32) {
        CKI(cudaMalloc((void **)&s->gp32, sizeof(float) * GM * 3 * N));
        CKI(cudaMalloc((void **)&s->gq32, sizeof(float) * GM * 3 * N));
        if (!getenv("MPM_GB300_TRUE_RESIDUAL_FP64")) CKI(cudaMalloc((void **)&s->dfx, sizeof(float) * 2 * 3 * N));
    }
    CKI(cudaMalloc((void **)&s->cnt, sizeof(unsigned) * 8));
    CKI(cudaMemset(s->cnt, 0, sizeof(unsigned) * 8));
    CKI(cudaMalloc((void **)&s->nmass, sizeof(double) * N));
    CKI(cudaMalloc((void **)&s->nvof, sizeof(double) * N));
    CKI(cudaMalloc((void **)&s->nei, sizeof(double) * N));
    s->nblk = (int)((N + 255) / 256);
    int pblk = (int)((c->num + 127) / 128);
    int nparts = 2 * (s->nblk > pblk ? s->nblk : pblk) + 2 * ((3 * (int)N + 255) / 256) + (GM + 2) * s->nblk + 64;
    CKI(cudaMalloc((void **)&s->part, sizeof(double) * (size_t)nparts));
    CKI(cudaMalloc((void **)&s->scal, sizeof(double) * S_NSCAL));
    CKI(cudaMallocHost((void **)&s->h_scal, sizeof(double) * S_NSCAL));
    CKI(cudaMemset(s->ndispl, 0, sizeof(double) * 3 * N));
    CKI(cudaMemset(s->x, 0, sizeof(double) * 3 * N));
    CKI(cudaMemset(s->scal, 0, sizeof(double) * S_NSCAL));
    return ensure_particle_scratch(c);
}

static int nb_nodes(mpm_ctx *c) { return (c->g.nodec + 255) / 256; }

// y = A x on the context's stream (k_imp_matvec for the context's matrix
// precision and stencil); hi: FP64 arithmetic whatever the storage (the
// true residual and the Newton check of the FP32 operator).
static void launch_matvec(mpm_ctx *c, const ImpArgs &a, int nb, const double *x, double *y, double *part,
                          unsigned *cnt = nullptr, double *scal = nullptr, int slot = 0, bool hi = false) {
    ImpState *s = c->imp;
    const int *o = c->g.order;
    auto go = [&](auto ta, auto tc) {
        using TA = decltype(ta);
        using TC = decltype(tc);
        const TA *A = (const TA *)s->A;
        if (o[0] == 1 && o[1] == 1 && o[2] == 1)
            k_imp_matvec<TA, TC, 1, 1, 1><<<nb, 256, 0, c->stream>>>(a, A, x, y, part, cnt, scal, slot);
        else if (o[1] == 2)
            k_imp_matvec<TA, TC, 2, 2, 2><<<nb, 256, 0, c->stream>>>(a, A, x, y, part, cnt, scal, slot);
        else
            k_imp_matvec<TA, TC, 2, 1, 2><<<nb, 256, 0, c->stream>>>(a, A, x, y, part, cnt, scal, slot);
    };
    if (s->prec == 64) {
        go(double(), double());
    } else if (hi && !part && s->dfx) {
        // FP32 operator, true residual / Newton check: double-float arithmetic
        const int n3 = 3 * c->g.nodec;
        k_split_df<<<(n3 + 255) / 256, 256, 0, c->stream>>>(x, s->dfx, s->dfx + n3, n3);
        const float *A = (const float *)s->A;
        if (o[0] == 1 && o[1] == 1 && o[2] == 1)
            k_imp_matvec_df<1, 1, 1><<<nb, 256, 0, c->stream>>>(a, A, s->dfx, s->dfx + n3, y);
        else if (o[1] == 2)
            k_imp_matvec_df<2, 2, 2><<<nb, 256, 0, c->stream>>>(a, A, s->dfx, s->dfx + n3, y);
        else
            k_imp_matvec_df<2, 1, 2><<<nb, 256, 0, c->stream>>>(a, A, s->dfx, s->dfx + n3, y);
    } else if (hi) {
        go(float(), double());
    } else {
        go(float(), float());
    }
}

// y = A x with FP32 vectors and FP32 arithmetic (FP32 operator only): the
// matvec of the flexible GCR directions.
static void launch_matvec_f32(mpm_ctx *c, const ImpArgs &a, int nb, const float *x, float *y) {
    const int *o = c->g.order;
    const float *A = (const float *)c->imp->A;
    if (o[0] == 1 && o[1] == 1 && o[2] == 1)
        k_imp_matvec<float, float, 1, 1, 1, float><<<nb, 256, 0, c->stream>>>(a, A, x, y, nullptr);
    else if (o[1] == 2)
        k_imp_matvec<float, float, 2, 2, 2, float><<<nb, 256, 0, c->stream>>>(a, A, x, y, nullptr);
    else
        k_imp_matvec<float, float, 2, 1, 2, float><<<nb, 256, 0, c->stream>>>(a, A, x, y, nullptr);
}

// AssembleSystem: k_imp_assemble (per particle), k_imp_rhs_diag, k_imp_scale
template <typename R>
static void launch_assemble(mpm_ctx *c, const ImpArgs &a) {
    ImpState *s = c->imp;
    const PView<R> P = pview<R>(c);
    R *A = (R *)s->A, *sk = (R *)s->stress_k;
    const int pb = (int)((c->num + 127) / 128);
    const int *o = c->g.order;
    if (o[0] == 1 && o[1] == 1 && o[2] == 1)
        k_imp_assemble<R, 1, 1, 1><<<pb, 128, 0, c->stream>>>(a, P, s->ndispl, sk, A, s->b);
    else if (o[1] == 2)
        k_imp_assemble<R, 2, 2, 2><<<pb, 128, 0, c->stream>>>(a, P, s->ndispl, sk, A, s->b);
    else
        k_imp_assemble<R, 2, 1, 2><<<pb, 128, 0, c->stream>>>(a, P, s->ndispl, sk, A, s->b);
    k_imp_rhs_diag<R><<<nb_nodes(c), 256, 0, c->stream>>>(a, A, s->nmass, s->naccel_k, s->naccel, s->b, s->adiag);
    k_imp_scale<R><<<nb_nodes(c), 256, 0, c->stream>>>(a, A, s->adiag);
}

// Node2Particle's particle pass (k_imp_g2p) and the shift (k_imp_shift)
template <typename R>
static void launch_g2p(mpm_ctx *c, const ImpArgs &a, int parity, int pb) {
    ImpState *s = c->imp;
    const PView<R> P = pview<R>(c);
    R *geup = (R *)s->geup;
    const int *o = c->g.order;
    if (o[0] == 1 && o[1] == 1 && o[2] == 1)
        k_imp_g2p<R, 1, 1, 1><<<pb, 128, 0, c->stream>>>(a, P, s->ndispl, s->nvel, s->naccel, s->nei, geup, s->part,
                                                          c->d_ctl, parity);
    else if (o[1] == 2)
        k_imp_g2p<R, 2, 2, 2><<<pb, 128, 0, c->stream>>>(a, P, s->ndispl, s->nvel, s->naccel, s->nei, geup, s->part,
                                                          c->d_ctl, parity);
    else
        k_imp_g2p<R, 2, 1, 2><<<pb, 128, 0, c->stream>>>(a, P, s->ndispl, s->nvel, s->naccel, s->nei, geup, s->part,
                                                          c->d_ctl, parity);
    k_finish<<<1, 256, 0, c->stream>>>(s->part, pb, s->scal, S_GD);
    k_imp_shift<R><<<pb, 128, 0, c->stream>>>(a, P, geup, s->scal);
}

// stress_k <- the particles' stress (InitializeNRStress)
static mpm_status copy_stress_k(mpm_ctx *c) {
    ImpState *s = c->imp;
    const size_t rs = c->rsize, n = (size_t)c->num;
    const char *f = (const char *)c->pbuf[c->cur];
    for (int k = 0; k < 6; k++)
        CKI(cudaMemcpyAsync((char *)s->stress_k + k * n * rs, f + (15 + k) * c->pstride * rs, rs * n,
                            cudaMemcpyDeviceToDevice, c->stream));
    return MPM_OK;
}

// P2G of the implicit solid: AccelP2G mode of the scatter + k_imp_grid
static mpm_status imp_p2g(mpm_ctx *c, double facl) {
    ImpState *s = c->imp;
    c->facl = facl;
    const size_t N = (size_t)c->g.nodec;
    if (c->steps_since_sort >= c->resort_period) {
        mpm_status st = sort_particles(c);
        if (st != MPM_OK) return st;
    }
    CKI(cudaMemsetAsync(c->d_acc, 0, sizeof(unsigned long long) * NACC * N, c->stream));
    c->write_nodal_dl = false;
    mpm_status st = run_p2g(c, facl);
    if (st != MPM_OK) return st;
    ImpArgs a = imp_args(c);
    k_imp_grid<<<nb_nodes(c), 256, 0, c->stream>>>(a, c->d_acc, c->d_ctl->p2g_inv, s->nmass, s->nvof, s->nvel,
                                                   s->naccel);
    c->launches++;
    return check_launch(c);
}

// one linear solve of the assembled, scaled system; s->x holds the initial
// guess (physical) and receives the physical solution.  Returns iterations.
static constexpr int KCHECK = 8;   // Krylov iterations between residual checks (and per graph)
// Within this factor of the tolerance (squared norms, 100x in the norm) the
// solvers leave the 8-iteration graphs and check after every iteration, so
// that a solve stops at the iteration that reaches the tolerance instead of
// at the end of the next block of 8.
static constexpr double FINE_FACTOR = 1.0e4;

static bool graphs_on(mpm_ctx *c) { return c->use_graph && c->stream != nullptr && !c->timer.on && !c->imp->no_graph; }

template <typename F>
static mpm_status capture_iters(mpm_ctx *c, cudaGraphExec_t *exec, F body) {
    CKI(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    body();
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return MPM_ERR_CUDA;
    }
    e = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        *exec = nullptr;
        cudaGetLastError();
        return MPM_ERR_CUDA;
    }
    return MPM_OK;
}

// one CG iteration on the scaled system; `it` fixes the residual-norm slot parity
static void cg_iteration(mpm_ctx *c, const ImpArgs &a, int nb, int it) {
    ImpState *s = c->imp;
    const int cur = (it & 1) ? S_RR1 : S_RR0;
    timer_begin(c, K_MATVEC);
    launch_matvec(c, a, nb, s->p, s->Ap, s->part, s->cnt + 3, s->scal, S_PAP);
    timer_end(c, K_MATVEC);
    timer_begin(c, K_KRYLOV);
    k_cg_update<<<nb, 256, 0, c->stream>>>(a, s->scal, cur, s->xs, s->r, s->p, s->Ap, s->part, s->cnt + 4);
    k_cg_dir<<<nb, 256, 0, c->stream>>>(a, s->scal, cur, s->r, s->p);
    timer_end(c, K_KRYLOV);
    c->launches += 3;
}

static mpm_status imp_cg(mpm_ctx *c, double eps, int kmax, int *iters) {
    ImpState *s = c->imp;
    ImpArgs a = imp_args(c);
    const int nb = nb_nodes(c);
    k_cg_scale_in<<<nb, 256, 0, c->stream>>>(a, s->x, s->b, s->adiag, s->xs, s->r);
    if (s->prec == 32)   // the scaled RHS, for the true residual of the FP32 operator
        CKI(cudaMemcpyAsync(s->bs, s->r, sizeof(double) * 3 * c->g.nodec, cudaMemcpyDeviceToDevice, c->stream));
    launch_matvec(c, a, nb, s->xs, s->Ap, nullptr, nullptr, nullptr, 0, true);
    k_cg_init<<<nb, 256, 0, c->stream>>>(a, s->Ap, s->r, s->p, s->part);
    k_finish<<<1, 256, 0, c->stream>>>(s->part, nb, s->scal, S_RR0);
    c->launches += 4;
    CKI(cudaMemcpyAsync(s->h_scal, s->scal, sizeof(double) * S_NSCAL, cudaMemcpyDeviceToHost, c->stream));
    CKI(cudaStreamSynchronize(c->stream));
    const double rr0 = s->h_scal[S_RR0];
    int it = 0;
    bool done = !(rr0 > 1.0e-300);
    bool fine = false;   // close to the tolerance: one iteration at a time, checked after each
    while (!done && it < kmax) {
        if (graphs_on(c) && !fine && it % KCHECK == 0 && it + KCHECK <= kmax) {
            if (!s->g_cg && capture_iters(c, &s->g_cg, [&] {
                    for (int k = 0; k < KCHECK; k++) cg_iteration(c, a, nb, k);
                }) != MPM_OK)
                s->no_graph = true;
            if (s->g_cg) {
                CKI(cudaGraphLaunch(s->g_cg, c->stream));
                it += KCHECK;
                if (it > KCHECK) c->launches += 5 * KCHECK;   // the capture counted the first block
            } else {
                continue;
            }
        } else {
            cg_iteration(c, a, nb, it);
            it++;
        }
        if (it % KCHECK == 0 || it == kmax || fine) {
            CKI(cudaMemcpyAsync(s->h_scal, s->scal, sizeof(double) * 2, cudaMemcpyDeviceToHost, c->stream));
            CKI(cudaStreamSynchronize(c->stream));
            const double rr = s->h_scal[(it & 1) ? S_RR1 : S_RR0];
            if (rr != rr) {
                *iters = it;
                return MPM_ERR_NONFINITE;
            }
            if (s->debug) fprintf(stderr, "mpm_gb300 cg: it %d |r|/|r0| %.3e\n", it, sqrt(rr / rr0));
            if (rr < eps * rr0 && s->prec == 32) {
                // FP32 operator: the recursive residual carries the rounding of
                // the FP32 matvecs, so convergence is judged on the true
                // residual bs - A x (FP64 arithmetic); if it is not below the
                // tolerance, CG restarts from it (r, and p = r).  Keeping the
                // old direction instead diverged: at this point the recursive
                // residual, and with it p, has fallen far below the true
                // residual, so alpha = r.r / p.Ap overshoots.
                const int cur = (it & 1) ? S_RR1 : S_RR0;
                launch_matvec(c, a, nb, s->xs, s->z, nullptr, nullptr, nullptr, 0, true);
                k_true_residual<<<nb, 256, 0, c->stream>>>(a, s->bs, s->z, s->r, s->part);
                k_finish<<<1, 256, 0, c->stream>>>(s->part, nb, s->scal, cur);
                CKI(cudaMemcpyAsync(s->p, s->r, sizeof(double) * 3 * c->g.nodec, cudaMemcpyDeviceToDevice,
                                    c->stream));
                c->launches += 3;
                CKI(cudaMemcpyAsync(s->h_scal, s->scal, sizeof(double) * 2, cudaMemcpyDeviceToHost, c->stream));
                CKI(cudaStreamSynchronize(c->stream));
                const double rrt = s->h_scal[cur];
                if (s->debug) fprintf(stderr, "mpm_gb300 cg: it %d true |r|/|r0| %.3e\n", it, sqrt(rrt / rr0));
                if (rrt < eps * rr0) done = true;
                s->last_rel = sqrt(rrt / rr0);
            } else {
                if (rr < eps * rr0) done = true;
                else if (rr < FINE_FACTOR * eps * rr0) fine = true;
                s->last_rel = sqrt(rr / rr0);
            }
        }
    }
    k_cg_scale_out<<<(3 * c->g.nodec + 255) / 256, 256, 0, c->stream>>>(a, s->xs, s->adiag, s->x);
    c->launches++;
    *iters = it;
    if (!done) return MPM_ERR_KRYLOV_MAXIT;
    return check_launch(c);
}

// One flexible GCR iteration on the scaled system: z = M(r) into direction
// slot `sl`, q = A z, orthogonalised against the `u` previous images, then
// x += alpha z, r -= alpha q with alpha = q.r / q.q.
static mpm_status gcr_iter(mpm_ctx *c, const ImpArgs &a, int nb, int u, int sl) {
    ImpState *s = c->imp;
    const size_t st3 = 3 * (size_t)c->g.nodec;
    if (s->gp32 && mpm_nn_fp32_output(s->net)) {
        // FP32 operator: directions and images in FP32 (the FP32 matvec computes
        // them in FP32 anyway; x, r and the true residual stay FP64)
        float *p = s->gp32 + (size_t)sl * st3, *q = s->gq32 + (size_t)sl * st3;
        timer_begin(c, K_PRECOND);
        mpm_status st = mpm_nn_apply_precond_f32(s->net, c->stream, s->r, s->scal + S_RRC, s->adiag, a.bcflag, a.mtol,
                                                 p);
        timer_end(c, K_PRECOND);
        if (st != MPM_OK) return st;
        timer_begin(c, K_MATVEC);
        launch_matvec_f32(c, a, nb, p, q);
        timer_end(c, K_MATVEC);
        timer_begin(c, K_KRYLOV);
        if (u > 0)
            k_gcr_dots<float><<<nb, 256, 0, c->stream>>>(a, s->gq32, s->gq32, sl, u, s->gm, s->part, s->cnt, s->gqq,
                                                         s->gbeta);
        k_gcr_axpy<float><<<nb, 256, 0, c->stream>>>(a, s->gp32, s->gq32, nullptr, sl, u, s->gm, s->gbeta, s->r,
                                                     s->part, s->cnt + 1, s->scal);
        k_gcr_update<float><<<nb, 256, 0, c->stream>>>(a, s->scal, s->xs, s->r, s->gp32, s->gq32, sl, s->gqq,
                                                       s->part, s->cnt + 2);
        timer_end(c, K_KRYLOV);
        c->launches += 9 + 3 + (u > 0 ? 1 : 0);
        return MPM_OK;
    }
    timer_begin(c, K_PRECOND);
    mpm_status st = mpm_nn_apply_precond(s->net, c->stream, s->r, s->scal + S_RRC, s->adiag, a.bcflag, a.mtol,
                                         s->gp + (size_t)sl * st3);
    timer_end(c, K_PRECOND);
    if (st != MPM_OK) return st;
    timer_begin(c, K_MATVEC);
    launch_matvec(c, a, nb, s->gp + (size_t)sl * st3, s->gq + (size_t)sl * st3, nullptr);
    timer_end(c, K_MATVEC);
    timer_begin(c, K_KRYLOV);
    if (u > 0)
        k_gcr_dots<double><<<nb, 256, 0, c->stream>>>(a, s->gq, s->gqf, sl, u, s->gm, s->part, s->cnt, s->gqq,
                                                      s->gbeta);
    k_gcr_axpy<double><<<nb, 256, 0, c->stream>>>(a, s->gp, s->gq, s->gqf, sl, u, s->gm, s->gbeta, s->r, s->part,
                                                  s->cnt + 1, s->scal);
    k_gcr_update<double><<<nb, 256, 0, c->stream>>>(a, s->scal, s->xs, s->r, s->gp, s->gq, sl, s->gqq, s->part,
                                                    s->cnt + 2);
    timer_end(c, K_KRYLOV);
    c->launches += 9 + 3 + (u > 0 ? 1 : 0);
    return MPM_OK;
}

// One solve of the assembled, scaled system by flexible CG with the learned
// preconditioner z = net(r) (Notay's FCG(1): p = z - (z.q'/p'.q') p',
// alpha = p.r / p.q).  The residual is checked every 8 iterations; when two
// checks in a row find no new minimum the solve continues with the Jacobi
// preconditioner (z = r in the scaled system).  Convergence is accepted only
// on the true residual bs - A x, recomputed in FP64.
static mpm_status imp_fcg(mpm_ctx *c, double eps, int kmax, int *iters) {
    ImpState *s = c->imp;
    ImpArgs a = imp_args(c);
    const int nb = nb_nodes(c);
    const size_t N = (size_t)c->g.nodec;
    k_cg_scale_in<<<nb, 256, 0, c->stream>>>(a, s->x, s->b, s->adiag, s->xs, s->r);
    CKI(cudaMemcpyAsync(s->bs, s->r, sizeof(double) * 3 * N, cudaMemcpyDeviceToDevice, c->stream));
    launch_matvec(c, a, nb, s->xs, s->Ap, nullptr, nullptr, nullptr, 0, true);
    k_true_residual<<<nb, 256, 0, c->stream>>>(a, s->bs, s->Ap, s->r, s->part);
    k_finish<<<1, 256, 0, c->stream>>>(s->part, nb, s->scal, S_RR0);
    k_finish<<<1, 256, 0, c->stream>>>(s->part, nb, s->scal, S_RRC);
    c->launches += 5;
    CKI(cudaMemcpyAsync(s->h_scal, s->scal, sizeof(double) * S_NSCAL, cudaMemcpyDeviceToHost, c->stream));
    CKI(cudaStreamSynchronize(c->stream));
    const double rr0 = s->h_scal[S_RR0];
    int it = 0;
    bool done = !(rr0 > 1.0e-300);
    bool use_nn = s->net != nullptr;
    if (use_nn) {
        k_phi<<<nb, 256, 0, c->stream>>>(a, s->nmass, s->adiag, s->ev);
        mpm_status st = mpm_nn_set_feature(s->net, c->stream, s->ev);
        if (st != MPM_OK) return st;
    }
    int restart = 1;
    double rr_window = rr0;   // smallest residual norm seen at a check
    int stall = 0;
    const int check = KCHECK;
    // one FCG iteration: z = M(r), p = z - (z.q'/p'.q') p', q = A p, x, r update
    auto iteration = [&](bool nn, int rs) -> mpm_status {
        if (nn) {
            timer_begin(c, K_PRECOND);
            mpm_status st = mpm_nn_apply_precond(s->net, c->stream, s->r, s->scal + S_RRC, s->adiag, a.bcflag, a.mtol,
                                                 s->z);
            timer_end(c, K_PRECOND);
            if (st != MPM_OK) return st;
            c->launches += 9;
        } else {
            CKI(cudaMemcpyAsync(s->z, s->r, sizeof(double) * 3 * N, cudaMemcpyDeviceToDevice, c->stream));
        }
        if (!rs) {
            k_dot3<<<nb, 256, 0, c->stream>>>(a, s->z, s->Ap, s->part);
            k_finish<<<1, 256, 0, c->stream>>>(s->part, nb, s->scal, S_ZQ);
            c->launches += 2;
        }
        timer_begin(c, K_KRYLOV);
        k_fcg_dir<<<nb, 256, 0, c->stream>>>(a, s->scal, rs, s->z, s->r, s->p, s->part);
        k_finish<<<1, 256, 0, c->stream>>>(s->part, nb, s->scal, S_PR);
        timer_end(c, K_KRYLOV);
        timer_begin(c, K_MATVEC);
        launch_matvec(c, a, nb, s->p, s->Ap, s->part);
        timer_end(c, K_MATVEC);
        timer_begin(c, K_KRYLOV);
        k_finish<<<1, 256, 0, c->stream>>>(s->part, nb, s->scal, S_PAP);
        k_fcg_update<<<nb, 256, 0, c->stream>>>(a, s->scal, s->xs, s->r, s->p, s->Ap, s->part);
        k_finish<<<1, 256, 0, c->stream>>>(s->part, nb, s->scal, S_RRC);
        timer_end(c, K_KRYLOV);
        c->launches += 6;
        return MPM_OK;
    };
    if (s->g_fcg_nn && s->g_net != s->net) {
        cudaGraphExecDestroy(s->g_fcg_nn);
        s->g_fcg_nn = nullptr;
    }
    if (s->g_gcr && s->g_net != s->net) {
        cudaGraphExecDestroy(s->g_gcr);
        s->g_gcr = nullptr;
    }
    // Phase 1: flexible GCR(GM) with the network as right preconditioner.  It
    // minimises the residual over the kept directions, so it needs no
    // symmetry of the (learned, non-symmetric) preconditioner.  It runs while
    // every window of `check` iterations at least halves the residual norm.
    if (use_nn && s->gcr) {
        int used = 0, slot = 0;
        double rr_win = rr0;
        bool fine = false;   // close to the tolerance: one iteration at a time, checked after each
        auto gcr_iteration = [&](int u, int sl) -> mpm_status { return gcr_iter(c, a, nb, u, sl); };
        while (!done && use_nn && it < kmax) {
            if (graphs_on(c) && !fine && used == s->gm && slot == 0 && it % check == 0 && it + check <= kmax) {
                const int64_t l0 = c->launches;
                if (!s->g_gcr && capture_iters(c, &s->g_gcr, [&] {
                        for (int k = 0; k < check; k++) gcr_iteration(s->gm, k % s->gm);
                    }) != MPM_OK)
                    s->no_graph = true;
                if (!s->g_gcr) continue;
                s->g_net = s->net;
                CKI(cudaGraphLaunch(s->g_gcr, c->stream));
                if (c->launches == l0) c->launches += 18 * check;
                s->nn_applications += check;
                it += check;
            } else {
                mpm_status st = gcr_iteration(used, slot);
                if (st != MPM_OK) return st;
                s->nn_applications++;
                used = used < s->gm ? used + 1 : s->gm;
                slot = (slot + 1) % s->gm;
                it++;
            }
            if (it % check == 0 || it == kmax || fine) {
                if (s->prec == 32) {
                    // FP32 operator: the recursive residual drifts from the true one
                    // by the rounding of the FP32 matvecs, so at every check it is
                    // replaced by the true residual bs - A x (FP64 arithmetic); the
                    // kept directions and their images stay valid
                    launch_matvec(c, a, nb, s->xs, s->z, nullptr, nullptr, nullptr, 0, true);
                    k_true_residual<<<nb, 256, 0, c->stream>>>(a, s->bs, s->z, s->r, s->part);
                    k_finish<<<1, 256, 0, c->stream>>>(s->part, nb, s->scal, S_RRC);
                    c->launches += 3;
                }
                CKI(cudaMemcpyAsync(s->h_scal, s->scal, sizeof(double) * S_NSCAL, cudaMemcpyDeviceToHost, c->stream));
                CKI(cudaStreamSynchronize(c->stream));
                double rr = s->h_scal[S_RRC];
                if (rr != rr) {
                    *iters = it;
                    return MPM_ERR_NONFINITE;
                }
                if (s->debug) fprintf(stderr, "mpm_gb300 gcr: it %d |r|/|r0| %.3e\n", it, sqrt(rr / rr0));
                if (rr < eps * rr0 && s->prec == 32) {
                    done = true;   // rr is the true residual
                } else if (rr < eps * rr0) {
                    launch_matvec(c, a, nb, s->xs, s->z, nullptr, nullptr, nullptr, 0, true);
                    k_true_residual<<<nb, 256, 0, c->stream>>>(a, s->bs, s->z, s->r, s->part);
                    k_finish<<<1, 256, 0, c->stream>>>(s->part, nb, s->scal, S_RRC);
                    c->launches += 3;
                    CKI(cudaMemcpyAsync(s->h_scal, s->scal, sizeof(double) * S_NSCAL, cudaMemcpyDeviceToHost,
                                        c->stream));
                    CKI(cudaStreamSynchronize(c->stream));
                    rr = s->h_scal[S_RRC];
                    if (rr < eps * rr0) done = true;
                    used = 0;   // the residual was replaced: the kept directions no longer apply
                    slot = 0;
                }
                if (!done && rr < FINE_FACTOR * eps * rr0) fine = true;
                if (it % check == 0 || it == kmax) {   // the window test, at window ends only
                    if (!done && !(rr < 0.25 * rr_win)) {
                        use_nn = false;   // less than a halving of |r| per window: Jacobi does better
                        s->fallbacks++;
                    }
                    rr_win = rr;
                }
                s->last_rel = sqrt(rr / rr0);
            }
        }
        restart = 1;
    }
    while (!done && it < kmax) {
        cudaGraphExec_t *gx = use_nn ? &s->g_fcg_nn : &s->g_fcg_jac;
        if (s->debug && use_nn) {
            // diagnostics: |z| / |r| and cos(z, r) of the preconditioned residual
            mpm_nn_apply_precond(s->net, c->stream, s->r, s->scal + S_RRC, s->adiag, a.bcflag, a.mtol, s->z);
            k_dot3<<<nb, 256, 0, c->stream>>>(a, s->z, s->z, s->part);
            k_finish<<<1, 256, 0, c->stream>>>(s->part, nb, s->scal, S_DZZ);
            k_dot3<<<nb, 256, 0, c->stream>>>(a, s->z, s->r, s->part);
            k_finish<<<1, 256, 0, c->stream>>>(s->part, nb, s->scal, S_DZR);
            CKI(cudaMemcpyAsync(s->h_scal, s->scal, sizeof(double) * S_NSCAL, cudaMemcpyDeviceToHost, c->stream));
            CKI(cudaStreamSynchronize(c->stream));
            const double zz = s->h_scal[S_DZZ], zr = s->h_scal[S_DZR], rr = s->h_scal[S_RRC];
            fprintf(stderr, "mpm_gb300 fcg: it %d |z|/|r| %.3e cos(z,r) %.3e\n", it, sqrt(zz / rr),
                    zr / sqrt(zz * rr + 1e-300));
        }
        if (graphs_on(c) && !restart && it % check == 0 && it + check <= kmax) {
            const int64_t l0 = c->launches;
            if (!*gx && capture_iters(c, gx, [&] {
                    for (int k = 0; k < check; k++) iteration(use_nn, 0);
                }) != MPM_OK)
                s->no_graph = true;
            if (*gx) {
                if (use_nn) s->g_net = s->net;
                CKI(cudaGraphLaunch(*gx, c->stream));
                if (c->launches == l0) c->launches += (use_nn ? 17 : 8) * check;
                if (use_nn) s->nn_applications += check;
                it += check;
            } else {
                continue;
            }
        } else {
            mpm_status st = iteration(use_nn, restart);
            if (st != MPM_OK) return st;
            if (use_nn) s->nn_applications++;
            restart = 0;
            it++;
        }
        if (it % check == 0 || it == kmax) {
            CKI(cudaMemcpyAsync(s->h_scal, s->scal, sizeof(double) * S_NSCAL, cudaMemcpyDeviceToHost, c->stream));
            CKI(cudaStreamSynchronize(c->stream));
            double rr = s->h_scal[S_RRC];
            if (rr != rr) {
                *iters = it;
                return MPM_ERR_NONFINITE;
            }
            if (s->debug)
                fprintf(stderr, "mpm_gb300 fcg: it %d |r|/|r0| %.3e (%s)\n", it, sqrt(rr / rr0),
                        use_nn ? "network" : "jacobi");
            if (rr < eps * rr0) {
                // confirm on the true residual
                launch_matvec(c, a, nb, s->xs, s->z, nullptr, nullptr, nullptr, 0, true);
                k_true_residual<<<nb, 256, 0, c->stream>>>(a, s->bs, s->z, s->r, s->part);
                k_finish<<<1, 256, 0, c->stream>>>(s->part, nb, s->scal, S_RRC);
                c->launches += 3;
                CKI(cudaMemcpyAsync(s->h_scal, s->scal, sizeof(double) * S_NSCAL, cudaMemcpyDeviceToHost, c->stream));
                CKI(cudaStreamSynchronize(c->stream));
                rr = s->h_scal[S_RRC];
                if (rr < eps * rr0) done = true;
                else restart = 1;
            }
            // the residual norm of a preconditioned solve need not fall at every
            // check: fall back only after two windows without a new minimum
            if (rr < rr_window) {
                rr_window = rr;
                stall = 0;
            } else {
                stall++;
            }
            if (!done && use_nn && stall >= 2) {
                use_nn = false;   // the network stopped reducing the residual
                restart = 1;
                s->fallbacks++;
            }
            s->last_rel = sqrt(rr / rr0);
        }
    }
    k_cg_scale_out<<<(3 * c->g.nodec + 255) / 256, 256, 0, c->stream>>>(a, s->xs, s->adiag, s->x);
    c->launches++;
    *iters = it;
    if (!done) return MPM_ERR_KRYLOV_MAXIT;
    return check_launch(c);
}

static mpm_status imp_assemble(mpm_ctx *c) {
    ImpState *s = c->imp;
    ImpArgs a = imp_args(c);
    const size_t N = (size_t)c->g.nodec;
    CKI(cudaMemsetAsync(s->A, 0, (s->prec == 64 ? sizeof(double) : sizeof(float)) * a_size((int)N, s->qp),
                        c->stream));
    CKI(cudaMemsetAsync(s->b, 0, sizeof(double) * 3 * N, c->stream));
    timer_begin(c, K_ASSEMBLE);
    if (s->prec == 64) launch_assemble<double>(c, a);
    else launch_assemble<float>(c, a);
    timer_end(c, K_ASSEMBLE);
    c->launches += 3;
    return check_launch(c);
}

// CheckNRConvergence's two residual measures of the last linear solve
static mpm_status imp_residuals(mpm_ctx *c, double *ref, double *absr) {
    ImpState *s = c->imp;
    ImpArgs a = imp_args(c);
    const int nb = nb_nodes(c);
    k_imp_prepare_residual<<<nb, 256, 0, c->stream>>>(a, s->x, s->adiag, s->b, s->xs);
    launch_matvec(c, a, nb, s->xs, s->Ap, nullptr, nullptr, nullptr, 0, true);
    k_imp_residual<<<nb, 256, 0, c->stream>>>(a, s->Ap, s->adiag, s->b, s->part);
    k_finish<<<1, 256, 0, c->stream>>>(s->part, nb, s->scal, S_RES);
    k_finish<<<1, 256, 0, c->stream>>>(s->part + nb, nb, s->scal, S_IDOF);
    c->launches += 5;
    CKI(cudaMemcpyAsync(s->h_scal, s->scal, sizeof(double) * S_NSCAL, cudaMemcpyDeviceToHost, c->stream));
    CKI(cudaStreamSynchronize(c->stream));
    const double rtr = s->h_scal[S_RES], idof = s->h_scal[S_IDOF];
    *ref = sqrt(rtr);
    *absr = idof <= 1.0e-30 ? 0.0 : sqrt(rtr / idof);
    return MPM_OK;
}

__global__ void k_add(double *y, const double *x, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] += x[i];
}

// SolidMaterialPoint::SolveSolid (solve_solid_implicit.cpp:65-103)
static mpm_status imp_newton(mpm_ctx *c, double eps, int kmax, int *krylov, int *newton) {
    ImpState *s = c->imp;
    ImpArgs a = imp_args(c);
    const size_t N = (size_t)c->g.nodec;
    if (copy_stress_k(c) != MPM_OK) return MPM_ERR_CUDA;
    CKI(cudaMemsetAsync(s->ndispl, 0, sizeof(double) * 3 * N, c->stream));
    CKI(cudaMemsetAsync(s->x, 0, sizeof(double) * 3 * N, c->stream));
    const int iter_max = s->nr_flag ? 1000 : 0;
    double r0r = 0.0;
    int ktot = 0, it;
    mpm_status st = MPM_OK;
    for (it = 0; it <= iter_max; it++) {
        k_imp_predict<<<nb_nodes(c), 256, 0, c->stream>>>(a, s->ndispl, s->nvel, s->naccel, s->naccel_k, nullptr, 1);
        c->launches++;
        st = imp_assemble(c);
        if (st != MPM_OK) return st;
        int k = 0;
        st = s->net ? imp_fcg(c, eps, kmax, &k) : imp_cg(c, eps, kmax, &k);
        ktot += k;
        if (st != MPM_OK) break;
        k_add<<<(3 * c->g.nodec + 255) / 256, 256, 0, c->stream>>>(s->ndispl, s->x, 3 * c->g.nodec);
        c->launches++;
        if (s->nr_flag) {
            double rkr, ra;
            st = imp_residuals(c, &rkr, &ra);
            if (st != MPM_OK) break;
            if (it == 0) r0r = rkr;
            const double rref = r0r > 1.0e-30 ? rkr / r0r : 0.0;
            if (rref < 1.0e-6 || r0r < 1.0e-6 || ra < 1.0e-8) break;
        }
    }
    *krylov = ktot;
    *newton = (it > iter_max ? iter_max : it) + 1;
    if (st == MPM_OK && s->nr_flag && it > iter_max) st = MPM_ERR_NEWTON_MAXIT;
    return st;
}

// Node2Particle (var_trans_solid_implicit.cpp:106-167)
static mpm_status imp_g2p(mpm_ctx *c) {
    ImpState *s = c->imp;
    ImpArgs a = imp_args(c);
    const int nb = nb_nodes(c);
    const int parity = (int)(c->step & 1);
    // PredictNewmarkBetaVelAndAccel + CommitNodalKinematics: nvel, naccel <- predicted
    k_imp_predict<<<nb, 256, 0, c->stream>>>(a, s->ndispl, s->nvel, s->naccel, s->naccel_k, s->Ap, 0);
    CKI(cudaMemcpyAsync(s->nvel, s->Ap, sizeof(double) * 3 * c->g.nodec, cudaMemcpyDeviceToDevice, c->stream));
    CKI(cudaMemcpyAsync(s->naccel, s->naccel_k, sizeof(double) * 3 * c->g.nodec, cudaMemcpyDeviceToDevice,
                        c->stream));
    k_imp_nei<<<nb, 256, 0, c->stream>>>(a, s->nvof, s->nei, s->part);
    k_finish<<<1, 256, 0, c->stream>>>(s->part, nb, s->scal, S_EU);
    k_imp_reset_next<<<1, 1, 0, c->stream>>>(c->d_ctl, parity);
    const int pb = (int)((c->num + 127) / 128);
    if (s->prec == 64) launch_g2p<double>(c, a, parity, pb);
    else launch_g2p<float>(c, a, parity, pb);
    c->launches += 7;
    return check_launch(c);
}

mpm_status mpm_gpu_implicit_step(mpm_ctx *c, int nsteps, double facl, double eps, int kmax, mpm_solve_stats *stats) {
    if (!c || !c->imp || nsteps < 0 || !(eps > 0.0) || kmax <= 0) return MPM_ERR_BAD_ARG;
    if (c->num == 0) return MPM_ERR_STATE;
    mpm_status st = ensure_particle_scratch(c);
    if (st != MPM_OK) return st;
    int kt = 0, nt = 0;
    const int fb0 = c->imp->fallbacks, na0 = c->imp->nn_applications;
    for (int i = 0; i < nsteps; i++) {
        st = imp_p2g(c, facl);
        if (st != MPM_OK) break;
        int k = 0, n = 0;
        st = imp_newton(c, eps, kmax, &k, &n);
        kt += k;
        nt += n;
        if (st != MPM_OK) break;
        st = imp_g2p(c);
        if (st != MPM_OK) break;
        c->step++;
        c->steps_since_sort++;
    }
    c->imp->krylov_total += kt;
    c->imp->newton_total += nt;
    if (stats) {
        stats->krylov_iters = kt;
        stats->newton_iters = nt;
        stats->last_rel_residual = c->imp->last_rel;
        stats->precond_fallbacks = c->imp->fallbacks - fb0;
        stats->nn_applications = c->imp->nn_applications - na0;
    }
    if (st != MPM_OK) return st;
    CKI(cudaStreamSynchronize(c->stream));
    return check_launch(c);
}

// ------------------------------------------------------------- test hooks
mpm_status mpm_gpu_implicit_assemble(mpm_ctx *c, double facl) {
    if (!c || !c->imp) return MPM_ERR_BAD_ARG;
    if (c->num == 0) return MPM_ERR_STATE;
    mpm_status st = ensure_particle_scratch(c);
    if (st != MPM_OK) return st;
    st = imp_p2g(c, facl);
    if (st != MPM_OK) return st;
    ImpState *s = c->imp;
    ImpArgs a = imp_args(c);
    if (copy_stress_k(c) != MPM_OK) return MPM_ERR_CUDA;
    CKI(cudaMemsetAsync(s->ndispl, 0, sizeof(double) * 3 * c->g.nodec, c->stream));
    CKI(cudaMemsetAsync(s->x, 0, sizeof(double) * 3 * c->g.nodec, c->stream));
    k_imp_predict<<<nb_nodes(c), 256, 0, c->stream>>>(a, s->ndispl, s->nvel, s->naccel, s->naccel_k, nullptr, 1);
    c->launches++;
    st = imp_assemble(c);
    if (st != MPM_OK) return st;
    CKI(cudaStreamSynchronize(c->stream));
    return MPM_OK;
}

mpm_status mpm_gpu_implicit_get_system(mpm_ctx *c, double *stencil, double *adiag, double *b_rhs) {
    if (!c || !c->imp) return MPM_ERR_BAD_ARG;
    ImpState *s = c->imp;
    const size_t N = (size_t)c->g.nodec;
    CKI(cudaStreamSynchronize(c->stream));
    if (stencil) {
        const int nq = 9 * imp_args(c).ns;
        if (s->prec == 64) {
            std::vector<double> t(a_size((int)N, s->qp));
            CKI(cudaMemcpy(t.data(), s->A, sizeof(double) * t.size(), cudaMemcpyDeviceToHost));
            for (int q = 0; q < nq; q++)
                for (size_t n = 0; n < N; n++) stencil[(size_t)q * N + n] = t[aidx(q, (int)n, s->qp)];
        } else {
            std::vector<float> t(a_size((int)N, s->qp));
            CKI(cudaMemcpy(t.data(), s->A, sizeof(float) * t.size(), cudaMemcpyDeviceToHost));
            for (int q = 0; q < nq; q++)
                for (size_t n = 0; n < N; n++) stencil[(size_t)q * N + n] = (double)t[aidx(q, (int)n, s->qp)];
        }
    }
    if (adiag) CKI(cudaMemcpy(adiag, s->adiag, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost));
    if (b_rhs) CKI(cudaMemcpy(b_rhs, s->b, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost));
    return MPM_OK;
}

mpm_status mpm_gpu_implicit_matvec(mpm_ctx *c, const double *x, double *y) {
    if (!c || !c->imp || !x || !y) return MPM_ERR_BAD_ARG;
    ImpState *s = c->imp;
    const size_t N = (size_t)c->g.nodec;
    CKI(cudaMemcpyAsync(s->xs, x, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, c->stream));
    ImpArgs a = imp_args(c);
    timer_begin(c, K_MATVEC);
    launch_matvec(c, a, nb_nodes(c), s->xs, s->Ap, nullptr, nullptr, nullptr, 0, true);
    timer_end(c, K_MATVEC);
    c->launches++;
    CKI(cudaMemcpyAsync(y, s->Ap, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, c->stream));
    CKI(cudaStreamSynchronize(c->stream));
    return check_launch(c);
}

mpm_status mpm_gpu_implicit_solve(mpm_ctx *c, double eps, int kmax, double *x, int *iters) {
    if (!c || !c->imp || !(eps > 0.0) || kmax <= 0) return MPM_ERR_BAD_ARG;
    ImpState *s = c->imp;
    const size_t N = (size_t)c->g.nodec;
    CKI(cudaMemsetAsync(s->x, 0, sizeof(double) * 3 * N, c->stream));
    int it = 0;
    mpm_status st = s->net ? imp_fcg(c, eps, kmax, &it) : imp_cg(c, eps, kmax, &it);
    if (iters) *iters = it;
    if (x) CKI(cudaMemcpy(x, s->x, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost));
    return st;
}

// ------------------------------------------------ learned preconditioner hooks
mpm_status mpm_gpu_implicit_set_precond(mpm_ctx *c, mpm_nn *net) {
    if (!c || !c->imp) return MPM_ERR_BAD_ARG;
    if (net && !mpm_nn_grid_matches(net, c->g.nnc)) return MPM_ERR_BAD_ARG;
    c->imp->net = net;
    return MPM_OK;
}

// CG on the scaled system from x = 0 with right-hand side s->bs.  With a
// network, every `stride`-th iterate appends the pair (r_k, xstar - x_k).
static mpm_status cg_scaled(mpm_ctx *c, double eps, int kmax, mpm_nn *net, int stride, int max_pairs, int *iters) {
    ImpState *s = c->imp;
    ImpArgs a = imp_args(c);
    const int nb = nb_nodes(c);
    const size_t N = (size_t)c->g.nodec;
    CKI(cudaMemsetAsync(s->xs, 0, sizeof(double) * 3 * N, c->stream));
    CKI(cudaMemsetAsync(s->Ap, 0, sizeof(double) * 3 * N, c->stream));
    CKI(cudaMemcpyAsync(s->r, s->bs, sizeof(double) * 3 * N, cudaMemcpyDeviceToDevice, c->stream));
    k_cg_init<<<nb, 256, 0, c->stream>>>(a, s->Ap, s->r, s->p, s->part);
    k_finish<<<1, 256, 0, c->stream>>>(s->part, nb, s->scal, S_RR0);
    CKI(cudaMemcpyAsync(s->h_scal, s->scal, sizeof(double) * S_NSCAL, cudaMemcpyDeviceToHost, c->stream));
    CKI(cudaStreamSynchronize(c->stream));
    const double rr0 = s->h_scal[S_RR0];
    int it = 0, pairs = 0;
    bool done = !(rr0 > 1.0e-300);
    while (!done && it < kmax) {
        const int cur = (it & 1) ? S_RR1 : S_RR0;
        if (net && it % stride == 0 && pairs < max_pairs) {
            k_sub3<<<(3 * c->g.nodec + 255) / 256, 256, 0, c->stream>>>(s->xstar, s->xs, s->ev, 3 * c->g.nodec);
            mpm_status st = mpm_nn_append_pair(net, c->stream, s->r, s->scal + cur, s->ev);
            if (st != MPM_OK) return st;
            pairs++;
        }
        launch_matvec(c, a, nb, s->p, s->Ap, s->part, s->cnt + 3, s->scal, S_PAP);
        k_cg_update<<<nb, 256, 0, c->stream>>>(a, s->scal, cur, s->xs, s->r, s->p, s->Ap, s->part, s->cnt + 4);
        k_cg_dir<<<nb, 256, 0, c->stream>>>(a, s->scal, cur, s->r, s->p);
        it++;
        if (it % 8 == 0 || it == kmax) {
            CKI(cudaMemcpyAsync(s->h_scal, s->scal, sizeof(double) * 2, cudaMemcpyDeviceToHost, c->stream));
            CKI(cudaStreamSynchronize(c->stream));
            const double rr = s->h_scal[(it & 1) ? S_RR1 : S_RR0];
            if (rr != rr) return MPM_ERR_NONFINITE;
            if (rr < eps * rr0) done = true;
        }
    }
    *iters = it;
    return check_launch(c);
}

// Flexible GCR with the context's preconditioner from x = 0 for the RHS s->bs,
// storing (r_k, xstar - x_k) before each of its first `npairs` iterations.
static mpm_status gcr_record(mpm_ctx *c, mpm_nn *rec, int npairs) {
    ImpState *s = c->imp;
    ImpArgs a = imp_args(c);
    const int nb = nb_nodes(c);
    const size_t N = (size_t)c->g.nodec;
    CKI(cudaMemsetAsync(s->xs, 0, sizeof(double) * 3 * N, c->stream));
    CKI(cudaMemcpyAsync(s->r, s->bs, sizeof(double) * 3 * N, cudaMemcpyDeviceToDevice, c->stream));
    k_dot3<<<nb, 256, 0, c->stream>>>(a, s->r, s->r, s->part);
    k_finish<<<1, 256, 0, c->stream>>>(s->part, nb, s->scal, S_RRC);
    int used = 0, slot = 0;
    for (int k = 0; k < npairs; k++) {
        k_sub3<<<(3 * c->g.nodec + 255) / 256, 256, 0, c->stream>>>(s->xstar, s->xs, s->ev, 3 * c->g.nodec);
        mpm_status st = mpm_nn_append_pair(rec, c->stream, s->r, s->scal + S_RRC, s->ev);
        if (st != MPM_OK) return st;
        st = gcr_iter(c, a, nb, used, slot);
        if (st != MPM_OK) return st;
        used = used < s->gm ? used + 1 : s->gm;
        slot = (slot + 1) % s->gm;
    }
    return check_launch(c);
}

mpm_status mpm_gpu_implicit_harvest(mpm_ctx *c, mpm_nn *net, int nsystems, int loads_per_system, int pairs_per_load,
                                    double e_min, double e_max, uint64_t seed, double eps, int kmax) {
    if (!c || !c->imp || !net || nsystems < 1 || loads_per_system < 1 || pairs_per_load < 1 || !(e_min > 0.0) ||
        !(e_max >= e_min) || !(eps > 0.0) || kmax < 1)
        return MPM_ERR_BAD_ARG;
    if (!mpm_nn_grid_matches(net, c->g.nnc)) return MPM_ERR_BAD_ARG;
    if (c->num == 0) return MPM_ERR_STATE;
    ImpState *s = c->imp;
    ImpArgs a = imp_args(c);
    const int nb = nb_nodes(c);
    const size_t N = (size_t)c->g.nodec;
    std::vector<double> saved(3 * (size_t)c->nmat);
    CKI(cudaMemcpy(saved.data(), c->d_matprop, sizeof(double) * saved.size(), cudaMemcpyDeviceToHost));
    mpm_status st = MPM_OK;
    uint64_t z = seed;
    auto next_unit = [&z]() {
        z += 0x9E3779B97F4A7C15ull;
        uint64_t t = z;
        t = (t ^ (t >> 30)) * 0xBF58476D1CE4E5B9ull;
        t = (t ^ (t >> 27)) * 0x94D049BB133111EBull;
        t ^= t >> 31;
        return ((t >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    };
    for (int sys = 0; sys < nsystems && st == MPM_OK; sys++) {
        const double E = exp(log(e_min) + next_unit() * (log(e_max) - log(e_min)));
        k_set_modulus<<<1, 32, 0, c->stream>>>(c->d_matprop, c->nmat, E);
        st = mpm_gpu_implicit_assemble(c, 1.0);
        if (st == MPM_OK) {
            k_phi<<<nb, 256, 0, c->stream>>>(a, s->nmass, s->adiag, s->ev);
            st = mpm_nn_begin_system(net, c->stream, s->ev);
            if (st == MPM_OK && s->net) st = mpm_nn_set_feature(s->net, c->stream, s->ev);
        }
        for (int ld = 0; ld < loads_per_system && st == MPM_OK; ld++) {
            const uint64_t key = seed * 1000003ull + (uint64_t)sys * 1009ull + (uint64_t)ld;
            if (ld == 0) {
                // the assembled system's own right-hand side (body force and inertia)
                k_cg_scale_in<<<nb, 256, 0, c->stream>>>(a, s->x, s->b, s->adiag, s->xs, s->bs);
            } else {
                // alternate smooth-dominated and noise-dominated loads
                const double smooth = (ld & 1) ? 0.2 : 1.0, noise = (ld & 1) ? 1.0 : 0.2;
                k_random_rhs<<<nb, 256, 0, c->stream>>>(a, s->adiag, key, smooth, noise, s->bs);
            }
            int K = 0;
            st = cg_scaled(c, eps, kmax, nullptr, 1, 0, &K);
            if (st != MPM_OK) break;
            CKI(cudaMemcpyAsync(s->xstar, s->xs, sizeof(double) * 3 * N, cudaMemcpyDeviceToDevice, c->stream));
            if (s->net) {
                // pairs along the learned solve itself: the residuals the
                // preconditioner meets once it has removed what it can
                st = gcr_record(c, net, pairs_per_load);
            } else {
                const int stride = K / pairs_per_load > 1 ? K / pairs_per_load : 1;
                int K2 = 0;
                st = cg_scaled(c, eps, K, net, stride, pairs_per_load, &K2);
            }
        }
    }
    cudaMemcpy(c->d_matprop, saved.data(), sizeof(double) * saved.size(), cudaMemcpyHostToDevice);
    if (st != MPM_OK) return st;
    CKI(cudaStreamSynchronize(c->stream));
    return check_launch(c);
}

// Test hook: z = M(r) for host arrays r, z (3 * nodec, scaled system) with the
// preconditioner set on ctx and the features of the assembled system.
mpm_status mpm_gpu_implicit_apply_precond(mpm_ctx *c, const double *r, double *z) {
    if (!c || !c->imp || !c->imp->net || !r || !z) return MPM_ERR_BAD_ARG;
    ImpState *s = c->imp;
    ImpArgs a = imp_args(c);
    const int nb = nb_nodes(c);
    const size_t N = (size_t)c->g.nodec;
    CKI(cudaMemcpyAsync(s->r, r, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, c->stream));
    k_phi<<<nb, 256, 0, c->stream>>>(a, s->nmass, s->adiag, s->ev);
    mpm_status st = mpm_nn_set_feature(s->net, c->stream, s->ev);
    if (st != MPM_OK) return st;
    k_dot3<<<nb, 256, 0, c->stream>>>(a, s->r, s->r, s->part);
    k_finish<<<1, 256, 0, c->stream>>>(s->part, nb, s->scal, S_RRC);
    st = mpm_nn_apply_precond(s->net, c->stream, s->r, s->scal + S_RRC, s->adiag, a.bcflag, a.mtol, s->z);
    if (st != MPM_OK) return st;
    CKI(cudaMemcpyAsync(z, s->z, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, c->stream));
    CKI(cudaStreamSynchronize(c->stream));
    return check_launch(c);
}

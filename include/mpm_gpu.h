/*
 * mpm_gpu.h -- C ABI of the GB300 MPM transfer path (libmpm_gb300.so).
 *
 * The reference (HPC-MPM-Code) has no FFI layer: its operator surface is the
 * C++ member functions of MaterialPoint / SolidMaterialPointBase and the
 * module globals.  Each entry point below replaces one of those calls; the
 * C++ shim in hpc-mpm-code_gb300/host/ re-exposes them with the reference's
 * own names (Particle2Node / SolveSolid / Node2Particle).
 *
 * Conventions
 *   - Plain pointers and sizes only.  Host arrays are FP64 and laid out like
 *     the reference: particle vectors AoS (coord[3*p+i]), F row-major
 *     (F[9*p+3*i+j]), Voigt stress [xx,yy,zz,yz,xz,xy] (stress[6*p+k]),
 *     nodal vectors component-major with the u/v/w blocks at offsets
 *     0, nodec, 2*nodec (module/data_io.cpp:53-56).
 *   - Every call returns an mpm_status; nothing aborts the process or traps
 *     the GPU.  Device-side problems (non-finite values, particles leaving
 *     the grid, solver limits) are latched in the context and returned by the
 *     next synchronising call.
 *   - One context per host thread; calls are ordered on the context's CUDA
 *     stream (mpm_gpu_set_stream).  The caller owns host memory; the context
 *     owns all device memory.
 */
#ifndef MPM_GPU_H
#define MPM_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    MPM_OK = 0,
    MPM_ERR_BAD_ARG = 1,
    MPM_ERR_OOM = 2,
    MPM_ERR_NONFINITE = 3,
    MPM_ERR_PARTICLE_OUT_OF_BOX = 4,
    MPM_ERR_KRYLOV_MAXIT = 5,
    MPM_ERR_DEVICE_TIMEOUT = 6,
    MPM_ERR_CUDA = 7,
    MPM_ERR_STATE = 8,
    MPM_ERR_UNSUPPORTED = 9,
    MPM_ERR_NEWTON_MAXIT = 10
} mpm_status;

/* MapScheme, module/dataset.h:19.  TPIC and APIC (module/map_and_interpolate.h:57-175)
 * carry a 3x3 affine velocity matrix per particle (TPIC vel_grad; APIC
 * vel_Bmat . inv_Dmat); their P2G reads the control-point coordinate as
 * xyc[nid][j], where the reference's VarP2G reads xyc[j][nid] (past the end
 * of xyc).  Explicit contexts only. */
typedef enum { MPM_PIC = 0, MPM_FLIP = 1, MPM_TPIC = 2, MPM_APIC = 3 } mpm_scheme;

typedef struct mpm_ctx mpm_ctx;

/* Grid header of one rank: InputParaGriddata (module/data_io.cpp:31-125) and
 * datain_para (work/src_solid/explicit/datain_para.cpp:43-90). */
typedef struct {
    int xyelem[3];    /* cells per direction (xyelem) */
    double xymin[3];  /* grid origin (xymin) */
    double dxy[3];    /* cell size (dxy) */
    int idimc[3];     /* shape order per direction: 1 linear, 2 quadratic B-spline (idimc) */
    int npxye[3];     /* particles per cell per direction, for the nodal volume (npxye) */
} mpm_grid_desc;

/* Material table: iprop[nmat] and mat_prop[3*nmat] (module/dataset.h:13-14),
 * the model numbers of ConstitutiveModel::UpdateStress
 * (module/solid/constitutive_model.cpp:287-305): -1 rigid, 0 linear elastic,
 * 1 Neo-Hookean, 2 St.Venant-Kirchhoff ({E, nu, -}), 3 Mooney-Rivlin
 * ({c1, c2, bulk modulus}).  Implicit contexts take -1 to 3 (each with its
 * tangent of ComputeTangentModulus); explicit contexts all of them and
 * iprop 4 (no counterpart in the reference): a weakly compressible Newtonian
 * fluid with the Tait equation of state, mat_prop = {c0 (speed of sound),
 * gamma, mu (dynamic viscosity)}; the rest density is each particle's
 * mass / vol0. */
typedef struct {
    int nmat;
    const int *iprop;
    const double *mat_prop;
} mpm_material_desc;

typedef struct {
    double dt;          /* time step (dt) */
    double mtol;        /* mass tolerance (mtol) */
    double gravity[3];  /* body force per unit mass (bb) */
    int scheme;         /* mpm_scheme (solswitch) */
    int precision;      /* 32: FP32 particle/grid arithmetic; 64: FP64 */
    int shifting;       /* 1: DeltaCorrectionParticleShifting as the reference; 0: off */
    int resort_period;  /* physical re-sort of particles by brick every N steps (>= 1); 0 = default (8) */
    int scatter;        /* 0: per-cell register scatter for FP32 linear grids (default); 1: staging-box atomics */
    int implicit;       /* 1: implicit solid context (particles carry acceleration; mpm_gpu_implicit_*) */
    int fbar;           /* 1: F-bar projection (Fbar_flag, module/solid/explicit/fbar_projection.cpp:18-93);
                           explicit contexts only */
    int reserved[5];
} mpm_config;

/* ---- lifetime ------------------------------------------------------------
 * Replaces the grid set-up of the drivers: BuildMesh / BuildControlPoint /
 * MakNodalVol (module/mesh.cpp:56,105,160) and the globals in dataset.h /
 * mesh.h. */
mpm_status mpm_gpu_create(const mpm_grid_desc *grid, const mpm_material_desc *mat, const mpm_config *cfg,
                          mpm_ctx **out);
void mpm_gpu_destroy(mpm_ctx *ctx);
/* stream: a cudaStream_t (as void*); NULL selects the legacy default stream. */
mpm_status mpm_gpu_set_stream(mpm_ctx *ctx, void *stream);
const char *mpm_gpu_status_string(mpm_status s);

/* ---- particles and boundary conditions ------------------------------------
 * Replaces SolidMaterialPointBase::InputPointData (module/solid/solid_data_io.cpp:13-36):
 * vel, F, stress and matid may be NULL (zero, identity, zero, material 0).
 * A non-finite input value refuses the load with MPM_ERR_NONFINITE (the
 * context is then left without particles); mpm_gpu_upload_particles and
 * mpm_gpu_steps_host report one through the next synchronising call. */
mpm_status mpm_gpu_load_particles(mpm_ctx *ctx, int64_t n, const double *coord, const double *vel,
                                  const double *mass, const double *vol0, const double *F, const double *stress,
                                  const int *matid);
/* Replaces BoundaryCondition::BCInput for ubc/vbc/wbc (module/bc.cpp:9-27):
 * comp 0/1/2 = u/v/w, node ids and prescribed values (applied x facl). */
mpm_status mpm_gpu_set_bc(mpm_ctx *ctx, int comp, int n, const int *nodes, const double *vals);

/* ---- the explicit transfer path -------------------------------------------
 * mpm_gpu_p2g          MeshPointLinklist + Particle2NodeS
 *                      (module/material_point.cpp:52, module/solid/explicit/var_trans_solid_explicit.cpp:20-99)
 * mpm_gpu_grid_update  SolveSolid (module/solid/explicit/solve_solid_explicit.cpp:8-31)
 * mpm_gpu_g2p          Node2ParticleS + MUSL + update_point_coord_and_stress
 *                      (module/solid/explicit/var_trans_solid_explicit.cpp:101-311)
 * mpm_gpu_step_explicit  nsteps x (p2g, grid_update, g2p), fused: the hot path
 *                      (work/src_solid/explicit/main.cpp:39-73). */
mpm_status mpm_gpu_p2g(mpm_ctx *ctx, double facl);
mpm_status mpm_gpu_grid_update(mpm_ctx *ctx);
mpm_status mpm_gpu_g2p(mpm_ctx *ctx);
mpm_status mpm_gpu_step_explicit(mpm_ctx *ctx, int nsteps, double facl);
/* No counterpart in the reference.  on (default): mpm_gpu_step_explicit on a
 * non-default stream with at least 6 x resort_period steps replays blocks of
 * 2 x resort_period steps from one captured CUDA graph (results are identical
 * to launching the steps one by one); off: always launches kernel by kernel. */
mpm_status mpm_gpu_set_graph(mpm_ctx *ctx, int on);

/* ---- results ----------------------------------------------------------------
 * field: 0 nmass, 1 nvof, 2 nmome, 3 nforce, 4 nvel, 5 naccel, 6 nvol
 * (MaterialPoint members, module/material_point.h:151-153; nvol from mesh.h).
 * Vectors are written component-major (3*nodec). Synchronises the stream. */
mpm_status mpm_gpu_download_nodal(mpm_ctx *ctx, int field, double *host);
/* Particles in the order they were loaded; any pointer may be NULL.  The
 * state of the particle vectors (coord, vel, def_grad, stress, vol) that the
 * reference's drivers read after Node2Particle (module/material_point.h:186-198).
 * Host buffers in pinned memory transfer at full link speed.  A precision-32
 * context whose materials are all Tait fluids (iprop 4) keeps only J = det F
 * of the deformation gradient: F comes back as J^(1/3) I, and an uploaded F
 * contributes its determinant. */
mpm_status mpm_gpu_download_particles(mpm_ctx *ctx, double *coord, double *vel, double *F, double *stress,
                                      double *vol);
/* TPIC / APIC contexts: the affine velocity matrix of each particle, 9
 * row-major values per particle in load order (TPIC vel_grad, APIC
 * vel_Bmat . inv_Dmat, module/map_and_interpolate.h:59,105); zeros for PIC
 * and FLIP.  Synchronises the stream. */
mpm_status mpm_gpu_download_affine(mpm_ctx *ctx, double *affine);
/* F-bar contexts: def_grad_bar (9 row-major values per particle) and
 * det_def_grad_bar in load order (module/material_point.h:116,121); either
 * pointer may be NULL.  Synchronises the stream. */
mpm_status mpm_gpu_download_fbar(mpm_ctx *ctx, double *Fbar, double *Jbar);
/* Overwrites the affine matrices of a TPIC / APIC context (same layout; a
 * restart, SolidMaterialPointBase::RestartInput, module/solid/solid_data_io.cpp:61-96)
 * and raises the next P2G's fixed-point bound to cover them. */
mpm_status mpm_gpu_upload_affine(mpm_ctx *ctx, const double *affine);
/* Overwrites the state of the loaded particles (same count, load order) from
 * host arrays; NULL leaves a field unchanged.  Replaces writing the particle
 * vectors between steps (e.g. SolidMaterialPointBase::RestartInput,
 * module/solid/solid_data_io.cpp:61-100). */
mpm_status mpm_gpu_upload_particles(mpm_ctx *ctx, const double *coord, const double *vel, const double *F,
                                    const double *stress, const double *vol);
/* nsteps explicit steps, each with the particle state uploaded from the host
 * arrays before it and downloaded into them after it (the reference's time
 * loop with the particle vectors on the host between steps); any pointer may
 * be NULL (that field stays on the device).  Uploads and downloads run on
 * two internal copy streams in pieces (four per field by default, environment
 * MPM_GB300_IO_CHUNKS = 1..16), pipelined across steps: the upload of a piece
 * waits only for the download of the same piece from the step before, so both
 * directions of the host link are busy at once.  Synchronises before
 * returning.  Explicit contexts only. */
mpm_status mpm_gpu_steps_host(mpm_ctx *ctx, int nsteps, double facl, double *coord, double *vel, double *F,
                              double *stress, double *vol);
/* Wait for the stream and return (and clear) any latched device error. */
mpm_status mpm_gpu_sync(mpm_ctx *ctx);
/* Test hook with no counterpart in the reference (whose waits are blocking
 * MPI calls): launches one CTA on the context's stream that waits, through
 * the bounded mbarrier wait of the bulk-copy staged kernels, on a barrier
 * that nothing completes, giving up after `seconds` (0 < seconds <= 1).  The
 * kernel records the timeout and returns, so the next mpm_gpu_sync returns
 * MPM_ERR_DEVICE_TIMEOUT and the context stays usable afterwards. */
mpm_status mpm_gpu_selftest_wait(mpm_ctx *ctx, double seconds);

typedef struct {
    int64_t num;            /* particles */
    int64_t nodec;          /* control points */
    int64_t steps;          /* explicit steps taken */
    int64_t resorts;        /* physical re-sorts done */
    int64_t kernel_launches;/* kernels launched by this context */
    int64_t out_of_box;     /* particles found outside the grid (clamped) */
    int64_t tile_misses;    /* particles scattered outside their tile's staging box, last step */
    int32_t ntiles;
    int32_t nwork;
} mpm_stats;
mpm_status mpm_gpu_get_stats(mpm_ctx *ctx, mpm_stats *out);

/* Per-kernel device time, accumulated between calls of this function with
 * CUDA events recorded on the context's stream around each kernel class
 * (enabled by mpm_gpu_enable_kernel_timing).  names[i] / ms[i] / launches[i]
 * for i < *count (count in: capacity).  Synchronises the stream. */
mpm_status mpm_gpu_enable_kernel_timing(mpm_ctx *ctx, int on);
/* No counterpart in the reference (which has no tuning): picks, per kernel,
 * the launch variant with the lowest measured time (shared-memory staged or
 * direct per-cell P2G and the resident CTAs per SM of the per-cell scatter and
 * gather kernels, persistent CTAs per SM of the staged particle update) by
 * running 3 x steps_per_trial explicit steps.
 * The variants it switches between compute bitwise the same results, so the
 * trial steps are ordinary steps of the simulation; with the moment-form
 * P2G and gather (the defaults) selected, only the update variant changes.
 * Neither the form (moment or corner) nor the re-sort period is tuned: both
 * change FP32 rounding. */
mpm_status mpm_gpu_autotune(mpm_ctx *ctx, int steps_per_trial, double facl);
/* p2g_minb / musl_minb: 0 = the shared-memory staged kernel, 2 or 3 = the
 * direct per-cell kernel compiled for that many resident CTAs per SM;
 * p2g_minb 4 (default) / 5 / 7 = the moment-form P2G over the active-brick
 * list for 2 / 1 / 3 resident CTAs per SM, 6 = chunked bricks, 8 / 9 = the
 * moment-form P2G loading each particle one iteration ahead, for 2 / 1
 * resident CTAs per SM; musl_minb 4 = one CTA per brick, 5 = the corner-form
 * gather over the brick list for 4 resident CTAs per SM, 7 (default) / 6 =
 * the moment-form gather for 2 / 3 resident CTAs per SM.  The moment forms
 * differ from the corner forms by FP32 rounding; the corner-form variants
 * (p2g_minb 0, 2, 3; musl_minb 0, 2, 3, 5) are bitwise identical to one
 * another, as are the update variants; update_ctas_per_sm: 1..8 persistent CTAs per SM
 * of the bulk-copy staged particle update (3, the default, is what its 80
 * registers let reside), 0 = the update with one CTA per brick and the
 * brick's nodal values in shared memory. */
mpm_status mpm_gpu_get_tuning(mpm_ctx *ctx, int *p2g_minb, int *musl_minb, int *update_ctas_per_sm);
mpm_status mpm_gpu_set_tuning(mpm_ctx *ctx, int p2g_minb, int musl_minb, int update_ctas_per_sm);
mpm_status mpm_gpu_kernel_times(mpm_ctx *ctx, int *count, const char **names, double *ms, int64_t *launches);

/* ---- the implicit solid (module/solid/implicit/, module/solver/) ----------------
 * A context created with cfg->implicit = 1, linear or quadratic B-spline
 * shape functions (idimc 1 1 1, 2 2 2 or 2 1 2) and precision 64 (the FP64
 * operator, the parity mode) or 32 (the FP32 operator: FP32 particles,
 * assembly, matrix and Krylov matvecs; FP64 Krylov inner products and norms,
 * true residual b - A x with the FP32 matrix applied in FP64 arithmetic, and
 * Newton check; the FP32 solves replace their recursive residual by the true
 * one at their checks).  mpm_gpu_implicit_setup replaces the solid set-up of
 * the FSI driver: GeneralizedAlphaParaSet + NewmarkBetaParaSet
 * (module/nonlinear_time_integration.cpp:10-56, spec_rad = 1 gives
 * alpha_f = alpha_m = 0.5, Newmark beta = 1/4, gamma = 1/2) and
 * CrsMat::BuildCrsMat (module/solver/crsmat.cpp:21-81; here a block stencil of
 * 27 slots for linear shapes, 125 for quadratic ones, 75 for idimc 2 1 2).
 * nr_flag as MaterialPoint::NR_flag (module/material_point.h:134). */
typedef struct {
    int newton_iters;          /* linear solves (Newton iterations) over the call */
    int krylov_iters;          /* CG iterations over the call */
    double last_rel_residual;  /* ||r|| / ||r0|| of the last solve (scaled system) */
    int precond_fallbacks;     /* solves that left the learned preconditioner for Jacobi */
    int nn_applications;       /* learned-preconditioner applications over the call */
} mpm_solve_stats;
mpm_status mpm_gpu_implicit_setup(mpm_ctx *ctx, int nr_flag, double spec_rad);
/* nsteps x (MeshPointLinklist, Particle2Node, SolveSolid, Node2Particle) of the
 * implicit solid (module/solid/implicit/var_trans_solid_implicit.cpp:20-167,
 * solve_solid_implicit.cpp:65-204).  Each linear system is solved by
 * diagonally scaled conjugate gradients until ||r||^2 < eps ||r0||^2 (the
 * reference's GPBiCGSafe stops at eps = 1e-8, module/solver/solver.cpp:64,128),
 * at most kmax iterations per solve. */
mpm_status mpm_gpu_implicit_step(mpm_ctx *ctx, int nsteps, double facl, double eps, int kmax,
                                 mpm_solve_stats *stats);
/* Test hooks.  assemble: Particle2Node + the first Newton system of a step
 * (ndispl = 0), scaled as BuildDiagonalPreconditioner leaves it.
 * get_system: stencil values [ns][9][nodec] (ns slots, slot s = (dx+r0) +
 * (2 r0 + 1)((dy+r1) + (2 r1 + 1)(dz+r2)) for the radius r = idimc per axis,
 * entry 3a+b), D^-1/2 and the RHS (3*nodec each).  matvec: y = A x with BC
 * rows zeroed, CrsMat::MatVecMult (module/solver/solver.cpp:405-433), host
 * arrays of 3*nodec.  solve: the assembled system from x = 0, physical x
 * (x may be NULL: the solution then stays on the device, no copy back). */
mpm_status mpm_gpu_implicit_assemble(mpm_ctx *ctx, double facl);
mpm_status mpm_gpu_implicit_get_system(mpm_ctx *ctx, double *stencil, double *adiag, double *b_rhs);
mpm_status mpm_gpu_implicit_matvec(mpm_ctx *ctx, const double *x, double *y);
mpm_status mpm_gpu_implicit_solve(mpm_ctx *ctx, double eps, int kmax, double *x, int *iters);

/* ---- learned preconditioner ------------------------------------------------
 * No counterpart in the reference, whose solid solves use GPBiCGSafe with
 * diagonal scaling or PETSc (module/solver/solver.cpp:19-141,
 * module/solver/crsmat.cpp:338-686).  A 3-level convolutional
 * encoder-decoder over the control-point grid (3 input and 3 output
 * channels, 16/32/64 hidden channels, BF16 weights and activations, FP32
 * accumulation on tcgen05 tensor cores) serves as the right preconditioner
 * of a flexible Krylov solver (GCR over the last 4 directions; flexible CG
 * when MPM_GB300_FCG_ONLY is set).  Convergence is always judged on
 * the true FP64 residual, and a solve falls back to the Jacobi preconditioner
 * when the network stops reducing the residual, so the accuracy of the
 * solution does not depend on the network.
 *
 * Input channels: the residual (3) and, per degree of freedom, the share of
 * the diagonal entry that comes from the mass term (3; 1 for a mass-dominated
 * row, small for a stiffness-dominated one), so that one network serves
 * systems of different stiffness.  Output: 3 channels.
 * Parameters (FP32, mpm_nn_num_params() values): for the five 3x3x3
 * convolutions l = 0..4 with (cin, cout) = (6,16), (16,32), (32,64),
 * (64,32), (32,16): W_l[27][cin][cout] (tap t = (dx+1) + 3(dy+1) + 9(dz+1))
 * then b_l[cout]; then the 1x1 output layer W5[16][3], b5[3].
 * Host tensors of forward/backward are FP32, input [batch][nodes][6],
 * output and its gradient [batch][nodes][3], nodes in control-point order
 * i + nx (j + ny k). */
typedef struct mpm_nn mpm_nn;
int64_t mpm_nn_num_params(void);
/* nodes: control points per direction of the grid the network runs on;
 * max_pairs: capacity of the on-device training set (0: none). */
mpm_status mpm_nn_create(const int nodes[3], int max_batch, int64_t max_pairs, mpm_nn **out);
mpm_status mpm_nn_destroy(mpm_nn *net);
mpm_status mpm_nn_set_stream(mpm_nn *net, void *stream);
/* linear = 1 (default): no activations and no biases, and the stiffness
 * channels enter as residual x mass share, so the network is a linear
 * operator of the residual (a preconditioner must not change with the
 * residual's scale or sign); 0: ReLU activations with biases. */
mpm_status mpm_nn_set_linear(mpm_nn *net, int linear);
/* additive = 1 (default): the preconditioner is z = r + net(r) (Jacobi in the
 * scaled system plus a learned correction) and training fits net(r) to
 * e - r; 0: z = net(r), trained on e. */
mpm_status mpm_nn_set_additive(mpm_nn *net, int additive);
/* symmetric = 1 (linear additive networks): the solver applies the
 * symmetric part z = r + (N r + N^T r) / 2, N^T by the network's transposed
 * (data-gradient) convolutions, so that conjugate gradients see a symmetric
 * preconditioner; 0 (default): z = r + N r, for the residual-minimising
 * flexible GCR phase of the solve. */
mpm_status mpm_nn_set_symmetric(mpm_nn *net, int symmetric);
mpm_status mpm_nn_init_params(mpm_nn *net, uint64_t seed);
mpm_status mpm_nn_set_params(mpm_nn *net, const float *params);
mpm_status mpm_nn_get_params(mpm_nn *net, float *params);
mpm_status mpm_nn_forward(mpm_nn *net, int batch, const float *in, float *out);
/* gradient of sum(out * gout) with respect to the parameters */
mpm_status mpm_nn_backward(mpm_nn *net, int batch, const float *in, const float *gout, float *grad);
mpm_status mpm_nn_num_pairs(mpm_nn *net, int64_t *n);
/* Adam on the stored (residual, error) pairs, loss = mean |net(r) - e|^2 / |e|^2,
 * step size lr with a cosine decay to 0 over the call;
 * epoch_loss[epochs] receives the mean loss of each epoch (may be NULL). */
mpm_status mpm_nn_train(mpm_nn *net, int epochs, int batch, double lr, uint64_t seed, float *epoch_loss);
/* Use `net` (NULL: none) as the preconditioner of the implicit solves of ctx. */
mpm_status mpm_gpu_implicit_set_precond(mpm_ctx *ctx, mpm_nn *net);
/* Test hook: z = M(r) for host arrays (3 * nodec, diagonally scaled system)
 * with the preconditioner set on ctx, after mpm_gpu_implicit_assemble. */
mpm_status mpm_gpu_implicit_apply_precond(mpm_ctx *ctx, const double *r, double *z);
/* Training pairs from the solver's own solves: for each of nsystems moduli
 * E drawn log-uniformly from [e_min, e_max] the system of the current state
 * is assembled; for its own right-hand side and loads_per_system - 1 seeded
 * random ones it is solved twice by Jacobi-PCG to ||r||^2 < eps ||r0||^2, the
 * second time storing pairs_per_load (residual, error) pairs spread over the
 * iterations.  When ctx already has a preconditioner (set_precond), the pairs
 * come instead from the first pairs_per_load iterations of the learned
 * flexible GCR solve: the residuals that preconditioner leaves behind.
 * The materials' moduli are restored afterwards. */
mpm_status mpm_gpu_implicit_harvest(mpm_ctx *ctx, mpm_nn *net, int nsystems, int loads_per_system, int pairs_per_load,
                                    double e_min, double e_max, uint64_t seed, double eps, int kmax);

/* ---- stabilized incompressible fluid: one Newton system ----------------
 * Constants of StabilizedMPM (module/fluid/MPM/stabilized_mpm.h:14-100,
 * module/material_point.h:41-112): density rho, dynamic viscosity rmu, the
 * time step, the Newmark coefficients (beta_nb, gamma_nb), the body force bb
 * with its load factor facl, and the mass tolerance mtol. */
typedef struct {
    double rho, rmu;
    double dt;
    double beta_nb, gamma_nb;
    double gravity[3];
    double facl;
    double mtol;
} mpm_ns_params;

/* Replaces the system set-up of StabilizedMPM::SolveNS
 * (module/fluid/MPM/solve_ns_mpm.cpp:28-62): MakNSStabCoeff (VMS, :64-135),
 * PredictNewmarkBetaVelAndAccel (module/nonlinear_time_integration.cpp:58-70),
 * AssembleNSSystem (:137-320, with ImplicitDsfCorr and AddInertialForceToRHS)
 * for linear shape functions (idimc = 1 in every direction).  All pointers
 * are caller-owned device arrays: particles x (three blocks of n), mass, vol;
 * the Newton state nvel, naccel, ndispl (component-major, 3*nodec, after
 * BCNRSet), npres and nmass (nodec).  Writes tau1 and tau2 (n), the unscaled
 * matrix as 4x4 blocks of the 27-point stencil, stencil[(s*16 + k)*nodec + i]
 * with k = row_var*4 + col_var over (u, v, w, p) and s = (dx+1) + 3(dy+1) +
 * 9(dz+1) of column node minus row node i, and b_rhs (component-major
 * 4*nodec); both are cleared first.  As in the reference, where SolveNS calls
 * MakNSStabCoeff once before its Newton loop, tau1 / tau2 are computed from
 * nvel, which must be the nodal velocity from before the Newton loop (not
 * the current iterate); the gradient correction uses alpha_f = 1 (the
 * Newmark scheme StabilizedMPM sets up, no generalized-alpha weighting).  *status (device int) is set to 1 when a
 * particle lies outside the grid (that particle is skipped), else 0.  Runs on
 * `stream` (a cudaStream_t, NULL = default stream) without waiting. */
mpm_status mpm_gpu_ns_assemble(const mpm_grid_desc *grid, const mpm_ns_params *prm, int64_t n, const double *x,
                               const double *mass, const double *vol, const double *nvel, const double *naccel,
                               const double *ndispl, const double *npres, const double *nmass, double *tau1,
                               double *tau2, double *stencil, double *b_rhs, int *status, void *stream);

/* ---- stabilized incompressible fluid: the Newton loop of one time step ------
 * Replaces StabilizedMPM::SolveNS (module/fluid/MPM/solve_ns_mpm.cpp:28-62)
 * on the reference's native solver path: MakNSStabCoeff once, then per Newton
 * iteration BCNRSet (module/fluid/MPM/stabilized_mpm.h:56-63), the system of
 * mpm_gpu_ns_assemble, BuildDiagonalPreconditioner for 4 degrees of freedom
 * (module/solver/crsmat.cpp:87-184), GPBiCGSafe on the scaled system
 * (module/solver/solver.cpp:19-141, the same method in FP64 with its stopping
 * test ||r||^2 < 1e-8 ||r0||^2), UpdateNRIncrement (solve_ns_mpm.cpp:21-26)
 * and CheckNRConvergence (module/solver/solver.cpp:565-593).  The one
 * difference: the linear solve is GPBiCGSafe called again from where it
 * stopped until the physical residual ||b - A x|| is below rtol ||b||, so that
 * the result does not depend on where a Krylov method happens to stop (with a
 * tight solve the reference's Newton test, which measures the residual of the
 * solved linear system, ends the loop after the first iteration).
 * A context holds the 27-point stencil of 4x4 blocks, the solver's vectors
 * and the boundary conditions (comp 0..3 = u, v, w, p: ubc, vbc, wbc with
 * BCSetDt on the displacement, pbc with BCSetVal on the pressure; BC rows are
 * zeroed in the matvec and the right-hand side, BCResidualSet). */
typedef struct mpm_ns mpm_ns;
typedef struct {
    int newton_iters;          /* Newton iterations of the call */
    int krylov_iters;          /* GPBiCGSafe iterations over all linear solves */
    double r0r;                /* CheckNRConvergence's reference residual (first iteration) */
    double last_residual;      /* ||b - A x|| of the last linear system */
    double last_abs_residual;  /* its sqrt(r.r / active rows) */
} mpm_ns_stats;
mpm_status mpm_ns_create(const mpm_grid_desc *grid, const mpm_ns_params *prm, mpm_ns **out);
void mpm_ns_destroy(mpm_ns *ns);
mpm_status mpm_ns_set_stream(mpm_ns *ns, void *stream);
mpm_status mpm_ns_set_bc(mpm_ns *ns, int comp, int n, const int *nodes, const double *vals);
/* Caller-owned device arrays as mpm_gpu_ns_assemble: particles x (three blocks
 * of n), mass, vol; the nodal state of the time step nvel, naccel (3*nodec,
 * component-major) and nmass (nodec).  Writes ndispl (3*nodec) and npres
 * (nodec), both starting from zero as SolveNS sets them, and tau1 / tau2.
 * kmax bounds each GPBiCGSafe call (MPM_ERR_KRYLOV_MAXIT); at most 100 Newton
 * iterations (MPM_ERR_NEWTON_MAXIT); a particle outside the grid returns
 * MPM_ERR_PARTICLE_OUT_OF_BOX.  Synchronises the context's stream. */
mpm_status mpm_ns_solve(mpm_ns *ns, int64_t n, const double *x, const double *mass, const double *vol,
                        const double *nvel, const double *naccel, const double *nmass, double *ndispl,
                        double *npres, double *tau1, double *tau2, double rtol, int kmax, mpm_ns_stats *stats);

/* ---- stabilized incompressible fluid: whole time steps --------------------
 * The particle side of the fluid loop of work/src_fluid/MPM/main.cpp:45-68 on
 * caller-owned device arrays (FP64, structure of arrays): x, vel, accel as
 * three blocks of n, pres, mass, vol (n); linear shape functions; scheme
 * MPM_PIC or MPM_FLIP (TPIC / APIC: MPM_ERR_UNSUPPORTED).  facl is the load
 * factor of the step (the reference's global facl: BCSetVal, BCNRSet and the
 * body force read it) and stays the context's load factor afterwards.
 * mpm_ns_p2g replaces StabilizedMPM::Particle2Node
 * (module/fluid/MPM/var_trans_fluid.cpp:17-80): nmass, nvof, nvel = sum N m v /
 * nmass, naccel = sum N m a / nmass (where nmass > mtol), BCSetVal (value
 * facl) on nvel and BCSetZero on naccel for the u, v, w lists; the sums are
 * int64 fixed point, so they do not depend on the particle order.  It writes
 * the context's own nodal state (mpm_ns_get_nodal reads it).
 * mpm_ns_step is one time step: Particle2Node as above, SolveNS as
 * mpm_ns_solve (linear systems to ||b - A x|| <= rtol ||b||), then
 * Node2Particle (var_trans_fluid.cpp:82-135): the Newmark predictor committed
 * to the nodes (module/nonlinear_time_integration.cpp:58-77), the pressure,
 * displacement, acceleration and (PIC) velocity gathers, FLIP's velocity
 * update and the displacement of CommitParticleKinematics
 * (nonlinear_time_integration.cpp:79-96), and DeltaCorrectionParticleShifting
 * (module/material_point.cpp:174-228) with the nodal volume of MakNodalVol
 * (module/mesh.cpp:160-202, the grid's npxye).  Updates x, vel, accel, pres in
 * place.  MeshPointLinklist has no counterpart: each particle finds its cell.
 * A particle outside the grid returns MPM_ERR_PARTICLE_OUT_OF_BOX, a
 * non-finite input MPM_ERR_NONFINITE (both before anything is written).
 * Synchronises the context's stream. */
mpm_status mpm_ns_p2g(mpm_ns *ns, int64_t n, const double *x, const double *vel, const double *accel,
                      const double *mass, const double *vol, int scheme, double facl);
mpm_status mpm_ns_step(mpm_ns *ns, int64_t n, double *x, double *vel, double *accel, double *pres,
                       const double *mass, const double *vol, int scheme, double facl, double rtol, int kmax,
                       mpm_ns_stats *stats);
/* The same time step as the reference's three member calls, on particles the
 * context holds: mpm_ns_load_particles copies the reference's host vectors
 * (coord, vel, accel as n x 3, mass and vol of n; vel and accel may be NULL
 * for zero) to the device once; then per time step
 *   mpm_ns_particle2node  replaces StabilizedMPM::Particle2Node
 *                         (module/fluid/MPM/var_trans_fluid.cpp:17-80),
 *   mpm_ns_solve_ns       replaces StabilizedMPM::SolveNS
 *                         (module/fluid/MPM/solve_ns_mpm.cpp:28-62) on the
 *                         nodal state Particle2Node left (as mpm_ns_solve),
 *   mpm_ns_node2particle  replaces StabilizedMPM::Node2Particle
 *                         (var_trans_fluid.cpp:82-135),
 * each with the semantics of mpm_ns_step (scheme and facl are those of the
 * step's Particle2Node).  mpm_ns_download_particles copies coord, vel, accel
 * (n x 3) and pres (n) back (any pointer may be NULL), where the reference
 * writes output or restarts.  solve_ns and node2particle before a
 * particle2node return MPM_ERR_STATE.  All synchronise the context's stream. */
mpm_status mpm_ns_load_particles(mpm_ns *ns, int64_t n, const double *coord, const double *vel,
                                 const double *accel, const double *mass, const double *vol);
mpm_status mpm_ns_particle2node(mpm_ns *ns, int scheme, double facl);
mpm_status mpm_ns_solve_ns(mpm_ns *ns, double rtol, int kmax, mpm_ns_stats *stats);
mpm_status mpm_ns_node2particle(mpm_ns *ns);
mpm_status mpm_ns_download_particles(mpm_ns *ns, double *coord, double *vel, double *accel, double *pres);
/* The context's nodal state after mpm_ns_p2g / mpm_ns_step, to a host array:
 * field 0 nmass, 1 nvof, 2 nvel, 3 naccel, 4 ndispl, 5 npres, 6 nvol
 * (3*nodec component-major for 2-4, nodec otherwise).  After a step, nvel and
 * naccel hold the committed Newmark values of Node2Particle. */
mpm_status mpm_ns_get_nodal(mpm_ns *ns, int field, double *host);

/* ---- allocation-free P2G -----------------------------------------------------
 * No counterpart in the reference: an extra entry point for callers that
 * cannot let a library allocate device memory (a host program that owns
 * every allocation through its own pool, or a time loop that must not hit
 * the device-wide synchronisation of cudaMalloc/cudaFree).  It runs the P2G
 * scatter of Particle2NodeS for linear shape functions and writes nmass,
 * nvof (zeroed below mtol), nmome and nforce (component-major, 3*nodec) into
 * caller-owned device arrays.  Inputs are caller-owned device arrays in
 * structure-of-arrays FP32 layout: x and v as three blocks of n, stress as
 * six Voigt blocks of n, mass and vol of n.  Launches on `stream`
 * (a cudaStream_t, NULL = default stream) and returns without waiting.
 * status: a caller-owned device int, set to 0 by the call; a particle outside
 * the grid sets bit 0 (1) and a particle with a non-finite coordinate,
 * velocity, stress, mass or volume sets bit 1 (2), and such a particle is
 * skipped (it adds nothing to the nodal fields), as the regular P2G counts
 * particles out of the box instead of scattering them.
 * Scratch: one static device array sized for at most 262,144 control points
 * (64^3); larger grids return MPM_ERR_BAD_ARG.  Every call shares that array
 * and clears it first, so calls that overlap on the GPU race.  The first call
 * on a device looks up the array's address (cudaGetSymbolAddress) and should
 * come before any stream capture; that address is kept for the life of the
 * process, so the library must not be used across a cudaDeviceReset.
 * Nothing is allocated or freed. */
mpm_status mpm_gpu_p2g_noalloc(const mpm_grid_desc *grid, const double *gravity, double facl, double mtol, int64_t n,
                               const float *x, const float *v, const float *stress, const float *mass,
                               const float *vol, float *nmass, float *nvof, float *nmome, float *nforce,
                               int *status, void *stream);

#ifdef __cplusplus
}
#endif
#endif

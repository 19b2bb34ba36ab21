/*
 * ORACLE -- test infrastructure only.  A plain-C, FP64 restatement of the
 * reference's (HPC-MPM-Code) solid MPM transfer path, used to check the CUDA
 * path on the same inputs.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py may load it; the product never does.
 *
 * It is pinned against the reference's own compiled code: the fixtures in
 * tests/golden/ are produced by oracle/_ref (the reference translation units
 * built unchanged) and tests/test_oracle_golden.py checks this restatement
 * against them.
 */
#ifndef MPM_ORACLE_H
#define MPM_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct mo_ctx mo_ctx;

/* grid: cells per direction, origin, cell size, shape order (1 or 2), particles
 * per cell per direction (for the nodal reference volume, module/mesh.cpp:160). */
mo_ctx *mo_create(const int *xyelem, const double *xymin, const double *dxy, const int *idimc, const int *npxye,
                  double dt, double mtol, const double *gravity, int nmat, const int *iprop, const double *mat_prop);
void mo_destroy(mo_ctx *c);
int mo_nodec(const mo_ctx *c);
int mo_load(mo_ctx *c, int num, const double *coord, const double *vel, const double *mass, const double *vol0,
            const int *matid, int scheme, int shifting);
int mo_set_state(mo_ctx *c, const double *F, const double *stress, const double *vol);
int mo_set_bc(mo_ctx *c, int comp, int n, const int *nodes, const double *vals);
int mo_explicit_p2g(mo_ctx *c, double facl);
int mo_explicit_steps(mo_ctx *c, int nsteps, double facl);
/* field: 0 nmass, 1 nvof, 2 nmome, 3 nforce, 4 nvel, 5 naccel, 6 nvol, 7 ndispl */
int mo_get_nodal(const mo_ctx *c, int field, double *out);
int mo_get_particles(const mo_ctx *c, double *coord, double *vel, double *F, double *stress, double *vol);
/* scheme 2 (TPIC) / 3 (APIC): the affine velocity matrix per particle, 9
 * row-major values (TPIC vel_grad; APIC vel_Bmat . inv_Dmat); zeros otherwise */
int mo_get_affine(const mo_ctx *c, double *out);
/* F-bar projection (Fbar_flag; module/solid/explicit/fbar_projection.cpp): on / off
 * after mo_load; def_grad_bar (9 per particle) and det_def_grad_bar */
int mo_set_fbar(mo_ctx *c, int on);
int mo_get_fbar(const mo_ctx *c, double *Fbar, double *Jbar);
/* shape functions at one point in element m: returns nenode */
int mo_shape(const mo_ctx *c, int m, const double *x, int *nc, double *sf, double *dsf);

/* ---- implicit solid ---- */
int mo_implicit_setup(mo_ctx *c, int nr_flag, double spec_rad);
int mo_implicit_nnzb(const mo_ctx *c);
int mo_implicit_assemble(mo_ctx *c, double facl);
int mo_implicit_get_matrix(const mo_ctx *c, int *matrow, int *matcolid, double *amat, double *adiag, double *b_rhs);
int mo_implicit_matvec(mo_ctx *c, const double *x, double *y);
int mo_implicit_solve(mo_ctx *c, double eps, int kmax, double *x_out);
int mo_implicit_steps(mo_ctx *c, int nsteps, double facl, double eps, int *krylov_total, int *newton_total);

#ifdef __cplusplus
}
#endif
#endif

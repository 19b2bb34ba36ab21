/*
 * ORACLE -- test infrastructure only (see mpm_oracle.h).  Plain C, FP64.
 *
 * Restates, function by function, the reference's solid MPM path:
 *   shape functions            module/shape_function.cpp:8-119 (MakSf)
 *   nodal reference volume     module/mesh.cpp:160-202 (MakNodalVol)
 *   cell linked list           module/material_point.cpp:52-78 (MeshPointLinklist)
 *   explicit P2G               module/solid/explicit/var_trans_solid_explicit.cpp:20-99
 *   explicit grid update       module/solid/explicit/solve_solid_explicit.cpp:8-31
 *   explicit G2P + MUSL        module/solid/explicit/var_trans_solid_explicit.cpp:101-148,187-311
 *   position/stress update     module/solid/explicit/var_trans_solid_explicit.cpp:150-185
 *   particle shifting          module/material_point.cpp:174-228
 *   constitutive models        module/solid/constitutive_model.cpp:7-285,287-305
 *   implicit P2G/G2P           module/solid/implicit/var_trans_solid_implicit.cpp:20-167
 *   implicit Newton + assembly module/solid/implicit/solve_solid_implicit.cpp:26-204
 *   Newmark / gen.-alpha       module/nonlinear_time_integration.cpp:10-96
 *   CSR graph + diag scaling   module/solver/crsmat.cpp:21-233
 *   matvec + GPBiCGSafe        module/solver/solver.cpp:19-141,405-433
 *   Newton convergence check   module/solver/solver.cpp:484-593
 * Traversal orders (element-major, then particle order within an element)
 * follow the reference so that FP64 sums agree to rounding.
 */
#include "mpm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define MAXN 27

struct mo_ctx {
    int nel[3], idimc[3], npxye[3], nnc[3];
    double xmin[3], dx[3];
    int nelem, nodec;
    double dt, mtol, bb[3], facl;
    int nmat;
    int *iprop;
    double *mat_prop; /* nmat x 3 */
    int scheme, shifting;
    /* particles (AoS like the reference: coord[3p+i], F[9p+3i+j], stress[6p+k]) */
    int num;
    double *coord, *vel, *accel, *mass, *vol0, *vol, *F, *stress, *jac;
    /* TPIC: vel_grad; APIC: vel_Bmat and inv_Dmat (module/map_and_interpolate.h:59,105), row major */
    double *aff, *aff_dinv;
    /* F-bar (Fbar_flag, module/solid/solid_material_point.h:16): def_grad_bar, det_def_grad_bar */
    int fbar;
    double *fbarF, *jbar;
    int *matid;
    /* nodal, component-major: comp c of node n at c*nodec + n */
    double *nmass, *nvof, *nmome, *nforce, *nvel, *naccel, *nvol, *ndispl;
    int nbc[3];
    int *bc_nodes[3];
    double *bc_vals[3];
    int *idepf, *idp2p, *numep;
    /* implicit */
    int nr_flag;
    double alpha_f, alpha_m, gamma_nb, beta_nb, nb[6];
    int nmat_csr;
    int *matrow, *matcolid;
    double *amat, *adiag, *b_rhs, *x_lhs;
    double stif[6][6];
};

static const int IDM[3][3] = {{0, 5, 4}, {5, 1, 3}, {4, 3, 2}}; /* module/dataset.h:15 */

static void *zalloc(size_t n) { return calloc(n ? n : 1, 1); }

/* ---------------------------------------------------------------- set-up */
static void make_nodal_vol(mo_ctx *c);

mo_ctx *mo_create(const int *xyelem, const double *xymin, const double *dxy, const int *idimc, const int *npxye,
                  double dt, double mtol, const double *gravity, int nmat, const int *iprop, const double *mat_prop) {
    mo_ctx *c = (mo_ctx *)zalloc(sizeof(mo_ctx));
    for (int i = 0; i < 3; i++) {
        c->nel[i] = xyelem[i];
        c->xmin[i] = xymin[i];
        c->dx[i] = dxy[i];
        c->idimc[i] = idimc[i];
        c->npxye[i] = npxye[i];
        c->nnc[i] = xyelem[i] + idimc[i];
        c->bb[i] = gravity[i];
    }
    c->nelem = c->nel[0] * c->nel[1] * c->nel[2];
    c->nodec = c->nnc[0] * c->nnc[1] * c->nnc[2];
    c->dt = dt;
    c->mtol = mtol;
    c->facl = 1.0;
    c->nmat = nmat;
    c->iprop = (int *)zalloc(sizeof(int) * nmat);
    c->mat_prop = (double *)zalloc(sizeof(double) * 3 * nmat);
    memcpy(c->iprop, iprop, sizeof(int) * nmat);
    memcpy(c->mat_prop, mat_prop, sizeof(double) * 3 * nmat);
    size_t N = (size_t)c->nodec;
    c->nmass = (double *)zalloc(sizeof(double) * N);
    c->nvof = (double *)zalloc(sizeof(double) * N);
    c->nvol = (double *)zalloc(sizeof(double) * N);
    c->nmome = (double *)zalloc(sizeof(double) * 3 * N);
    c->nforce = (double *)zalloc(sizeof(double) * 3 * N);
    c->nvel = (double *)zalloc(sizeof(double) * 3 * N);
    c->naccel = (double *)zalloc(sizeof(double) * 3 * N);
    c->ndispl = (double *)zalloc(sizeof(double) * 3 * N);
    c->idepf = (int *)zalloc(sizeof(int) * c->nelem);
    c->numep = (int *)zalloc(sizeof(int) * c->nelem);
    make_nodal_vol(c);
    return c;
}

static void free_particles(mo_ctx *c) {
    free(c->coord); free(c->vel); free(c->accel); free(c->mass); free(c->vol0); free(c->vol);
    free(c->F); free(c->stress); free(c->jac); free(c->matid); free(c->idp2p);
    free(c->aff); free(c->aff_dinv); free(c->fbarF); free(c->jbar);
}

void mo_destroy(mo_ctx *c) {
    if (!c) return;
    free_particles(c);
    free(c->iprop); free(c->mat_prop);
    free(c->nmass); free(c->nvof); free(c->nvol); free(c->nmome); free(c->nforce); free(c->nvel);
    free(c->naccel); free(c->ndispl); free(c->idepf); free(c->numep);
    for (int k = 0; k < 3; k++) { free(c->bc_nodes[k]); free(c->bc_vals[k]); }
    free(c->matrow); free(c->matcolid); free(c->amat); free(c->adiag); free(c->b_rhs); free(c->x_lhs);
    free(c);
}

int mo_nodec(const mo_ctx *c) { return c->nodec; }

int mo_load(mo_ctx *c, int num, const double *coord, const double *vel, const double *mass, const double *vol0,
            const int *matid, int scheme, int shifting) {
    free_particles(c);
    size_t n = (size_t)num;
    c->num = num;
    c->scheme = scheme;
    c->shifting = shifting;
    c->coord = (double *)zalloc(sizeof(double) * 3 * n);
    c->vel = (double *)zalloc(sizeof(double) * 3 * n);
    c->accel = (double *)zalloc(sizeof(double) * 3 * n);
    c->mass = (double *)zalloc(sizeof(double) * n);
    c->vol0 = (double *)zalloc(sizeof(double) * n);
    c->vol = (double *)zalloc(sizeof(double) * n);
    c->jac = (double *)zalloc(sizeof(double) * n);
    c->F = (double *)zalloc(sizeof(double) * 9 * n);
    c->stress = (double *)zalloc(sizeof(double) * 6 * n);
    c->matid = (int *)zalloc(sizeof(int) * n);
    c->idp2p = (int *)zalloc(sizeof(int) * n);
    c->aff = (double *)zalloc(sizeof(double) * 9 * n);       /* VectorAssign: zero, solid_material_point.cpp:36-42 */
    c->aff_dinv = (double *)zalloc(sizeof(double) * 9 * n);
    c->fbarF = (double *)zalloc(sizeof(double) * 9 * n);     /* def_grad_bar = I, det_def_grad_bar = 1 */
    c->jbar = (double *)zalloc(sizeof(double) * n);
    memcpy(c->coord, coord, sizeof(double) * 3 * n);
    if (vel) memcpy(c->vel, vel, sizeof(double) * 3 * n);
    memcpy(c->mass, mass, sizeof(double) * n);
    memcpy(c->vol0, vol0, sizeof(double) * n);
    memcpy(c->vol, vol0, sizeof(double) * n); /* module/solid/solid_data_io.cpp:32 */
    for (size_t p = 0; p < n; p++) {
        c->matid[p] = matid ? matid[p] : 0;
        c->jac[p] = 1.0; /* det_def_grad initialised to 1, solid_material_point.cpp:10 */
        c->F[9 * p + 0] = c->F[9 * p + 4] = c->F[9 * p + 8] = 1.0; /* solid_data_io.cpp:28 */
        c->fbarF[9 * p + 0] = c->fbarF[9 * p + 4] = c->fbarF[9 * p + 8] = 1.0;
        c->jbar[p] = 1.0;
    }
    return 0;
}

/* A loaded state other than the undeformed one (as the GPU path's load +
 * upload): F (9 per particle), stress (6) and vol, any may be NULL; jac
 * follows F. */
int mo_set_state(mo_ctx *c, const double *F, const double *stress, const double *vol) {
    for (size_t p = 0; p < (size_t)c->num; p++) {
        if (F) {
            memcpy(c->F + 9 * p, F + 9 * p, sizeof(double) * 9);
            const double *f = F + 9 * p;
            c->jac[p] = f[0] * (f[4] * f[8] - f[5] * f[7]) + f[1] * (f[5] * f[6] - f[3] * f[8]) +
                        f[2] * (f[3] * f[7] - f[4] * f[6]);
        }
        if (stress) memcpy(c->stress + 6 * p, stress + 6 * p, sizeof(double) * 6);
        if (vol) c->vol[p] = vol[p];
    }
    return 0;
}

int mo_set_bc(mo_ctx *c, int comp, int n, const int *nodes, const double *vals) {
    if (comp < 0 || comp > 2) return -1;
    free(c->bc_nodes[comp]);
    free(c->bc_vals[comp]);
    c->nbc[comp] = n;
    c->bc_nodes[comp] = (int *)zalloc(sizeof(int) * n);
    c->bc_vals[comp] = (double *)zalloc(sizeof(double) * n);
    memcpy(c->bc_nodes[comp], nodes, sizeof(int) * n);
    memcpy(c->bc_vals[comp], vals, sizeof(double) * n);
    return 0;
}

/* BoundaryCondition::BCSetVal / BCSetZero / BCSetDt, module/bc.cpp:45-79 */
static void bc_set_val(const mo_ctx *c, double *v3) {
    for (int k = 0; k < 3; k++)
        for (int i = 0; i < c->nbc[k]; i++) v3[(size_t)k * c->nodec + c->bc_nodes[k][i]] = c->bc_vals[k][i] * c->facl;
}
static void bc_set_zero(const mo_ctx *c, double *v3) {
    for (int k = 0; k < 3; k++)
        for (int i = 0; i < c->nbc[k]; i++) v3[(size_t)k * c->nodec + c->bc_nodes[k][i]] = 0.0;
}
static void bc_set_dt(const mo_ctx *c, double *v3) {
    for (int k = 0; k < 3; k++)
        for (int i = 0; i < c->nbc[k]; i++)
            v3[(size_t)k * c->nodec + c->bc_nodes[k][i]] = c->bc_vals[k][i] * c->dt * c->facl;
}

/* ------------------------------------------------------- shape functions */
/* MakSf, module/shape_function.cpp:8-119 (single rank: aelemmin = 0). */
static int maksf(const mo_ctx *c, int m, const double *x, int *nc, double *sf, double *dsf) {
    int nex = c->nel[0], ney = c->nel[1];
    int ize = m / (nex * ney);
    int iye = (m - ize * nex * ney) / nex;
    int ixe = m - ize * nex * ney - iye * nex;
    int id = 0, ixyn[3];
    for (int k = 0; k <= c->idimc[2]; k++) {
        ixyn[2] = ize + k;
        for (int j = 0; j <= c->idimc[1]; j++) {
            ixyn[1] = iye + j;
            for (int i = 0; i <= c->idimc[0]; i++) {
                ixyn[0] = ixe + i;
                nc[id] = ixyn[0] + c->nnc[0] * ixyn[1] + c->nnc[0] * c->nnc[1] * ixyn[2];
                double s[3], d[3];
                for (int ii = 0; ii < 3; ii++) {
                    double dxi = c->dx[ii];
                    if (c->idimc[ii] == 1) {
                        double xy = c->xmin[ii] + dxi * (double)ixyn[ii];
                        double r = x[ii] - xy;
                        s[ii] = 1.0 - fabs(r) / dxi;
                        d[ii] = (r < 0.0) ? 1.0 / dxi : -1.0 / dxi;
                    } else {
                        int ncxy = ixyn[ii];
                        double xy = c->xmin[ii] + dxi * (double)(ixyn[ii] - 2);
                        double h = (x[ii] - xy) / dxi;
                        double s1, s2, s3, d1, d2;
                        if (ncxy == 0) {
                            h -= 2.0;
                            s1 = 1.0; s2 = -2.0; s3 = 1.0; d1 = 2.0; d2 = -2.0;
                        } else if (ncxy == 1) {
                            h -= 1.0;
                            if (h <= 1.0) { s1 = -1.5; s2 = 2.0; s3 = 0.0; d1 = -3.0; d2 = 2.0; }
                            else { s1 = 0.5; s2 = -2.0; s3 = 2.0; d1 = 1.0; d2 = -2.0; }
                        } else if (ncxy == c->nnc[ii] - 1) {
                            s1 = 1.0; s2 = 0.0; s3 = 0.0; d1 = 2.0; d2 = 0.0;
                        } else if (ncxy == c->nnc[ii] - 2) {
                            if (h <= 1.0) { s1 = 0.5; s2 = 0.0; s3 = 0.0; d1 = 1.0; d2 = 0.0; }
                            else { s1 = -1.5; s2 = 4.0; s3 = -2.0; d1 = -3.0; d2 = 4.0; }
                        } else {
                            if (h <= 1.0) { s1 = 0.5; s2 = 0.0; s3 = 0.0; d1 = 1.0; d2 = 0.0; }
                            else if (h <= 2.0) { s1 = -1.0; s2 = 3.0; s3 = -1.5; d1 = -2.0; d2 = 3.0; }
                            else { s1 = 0.5; s2 = -3.0; s3 = 4.5; d1 = 1.0; d2 = -3.0; }
                        }
                        s[ii] = (s1 * h + s2) * h + s3;
                        d[ii] = (d1 * h + d2) / dxi;
                    }
                }
                sf[id] = s[0] * s[1] * s[2];
                dsf[3 * id + 0] = d[0] * s[1] * s[2];
                dsf[3 * id + 1] = s[0] * d[1] * s[2];
                dsf[3 * id + 2] = s[0] * s[1] * d[2];
                id++;
            }
        }
    }
    return id;
}

int mo_shape(const mo_ctx *c, int m, const double *x, int *nc, double *sf, double *dsf) {
    return maksf(c, m, x, nc, sf, dsf);
}

/* GaussianDistribution offsets, module/mesh.cpp:12-54 */
static double gauss_off(int npc, int i, double d) {
    switch (npc) {
    case 1: return 0.0;
    case 2: return (i == 0 ? -0.25 : 0.25) * d;
    case 3: return (i == 0 ? -1.0 / 3.0 : i == 1 ? 0.0 : 1.0 / 3.0) * d;
    case 4: { static const double t[4] = {-0.375, -0.125, 0.125, 0.375}; return t[i] * d; }
    case 5: { static const double t[5] = {-0.4, -0.2, 0.0, 0.2, 0.4}; return t[i] * d; }
    case 6: { static const double t[6] = {-5.0 / 12.0, -3.0 / 12.0, -1.0 / 12.0, 1.0 / 12.0, 3.0 / 12.0, 5.0 / 12.0};
              return t[i] * d; }
    }
    return 0.0;
}

/* MakNodalVol, module/mesh.cpp:160-202 */
static void make_nodal_vol(mo_ctx *c) {
    double volp = c->dx[0] * c->dx[1] * c->dx[2] / (double)(c->npxye[0] * c->npxye[1] * c->npxye[2]);
    int nc[MAXN];
    double sf[MAXN], dsf[3 * MAXN];
    memset(c->nvol, 0, sizeof(double) * c->nodec);
    for (int m = 0; m < c->nelem; m++) {
        int ize = m / (c->nel[0] * c->nel[1]);
        int iye = (m - ize * c->nel[0] * c->nel[1]) / c->nel[0];
        int ixe = m - ize * c->nel[0] * c->nel[1] - iye * c->nel[0];
        double xe[3] = {c->xmin[0] + c->dx[0] * (ixe + 0.5), c->xmin[1] + c->dx[1] * (iye + 0.5),
                        c->xmin[2] + c->dx[2] * (ize + 0.5)};
        double xp[3];
        for (int iz = 0; iz < c->npxye[2]; iz++) {
            xp[2] = xe[2] + gauss_off(c->npxye[2], iz, c->dx[2]);
            for (int iy = 0; iy < c->npxye[1]; iy++) {
                xp[1] = xe[1] + gauss_off(c->npxye[1], iy, c->dx[1]);
                for (int ix = 0; ix < c->npxye[0]; ix++) {
                    xp[0] = xe[0] + gauss_off(c->npxye[0], ix, c->dx[0]);
                    int ne = maksf(c, m, xp, nc, sf, dsf);
                    for (int i = 0; i < ne; i++) c->nvol[nc[i]] += sf[i] * volp;
                }
            }
        }
    }
}

/* MeshPointLinklist, module/material_point.cpp:52-78 */
static void linklist(mo_ctx *c) {
    int *last = (int *)malloc(sizeof(int) * c->nelem);
    for (int m = 0; m < c->nelem; m++) { c->numep[m] = 0; c->idepf[m] = -1; last[m] = -1; }
    for (int p = 0; p < c->num; p++) c->idp2p[p] = -1;
    for (int p = 0; p < c->num; p++) {
        int ie[3];
        for (int i = 0; i < 3; i++) ie[i] = (int)floor((c->coord[3 * p + i] - c->xmin[i]) / c->dx[i]);
        int ne = ie[0] + ie[1] * c->nel[0] + ie[2] * c->nel[0] * c->nel[1];
        c->numep[ne]++;
        if (c->numep[ne] == 1) c->idepf[ne] = p;
        else c->idp2p[last[ne]] = p;
        last[ne] = p;
    }
    free(last);
}

#define FOR_PARTICLES(c, m, p)                                                                                         \
    for (int m = 0; m < (c)->nelem; m++)                                                                               \
        for (int p = (c)->idepf[m]; p != -1; p = (c)->idp2p[p])

/* ------------------------------------------------------ constitutive models */
/* MatLinElast, module/solid/constitutive_model.cpp:16-60 (incremental; fills
 * the 6x6 tangent when implicit). */
static void mat_lin_elast(mo_ctx *c, double *sts, const double d[3][3], const double *mp, int implicit) {
    double E = mp[0], nu = mp[1];
    double C0 = E * (1.0 - nu) / ((1.0 - 2.0 * nu) * (1.0 + nu));
    double C1 = E * nu / ((1.0 - 2.0 * nu) * (1.0 + nu));
    double C2 = E / (2.0 * (1.0 + nu));
    double e[6] = {d[0][0] - 1.0, d[1][1] - 1.0, d[2][2] - 1.0, d[1][2] + d[2][1], d[2][0] + d[0][2], d[0][1] + d[1][0]};
    double ds[6];
    ds[0] = C0 * e[0] + C1 * e[1] + C1 * e[2];
    ds[1] = C1 * e[0] + C0 * e[1] + C1 * e[2];
    ds[2] = C1 * e[0] + C1 * e[1] + C0 * e[2];
    ds[3] = C2 * e[3];
    ds[4] = C2 * e[4];
    ds[5] = C2 * e[5];
    for (int k = 0; k < 6; k++) sts[k] += ds[k];
    if (implicit) {
        memset(c->stif, 0, sizeof(c->stif));
        for (int i = 0; i < 3; i++) {
            for (int j = 0; j < 3; j++)
                if (i != j) c->stif[i][j] = C1;
            c->stif[i][i] = C0;
        }
        c->stif[3][3] = c->stif[4][4] = c->stif[5][5] = C2;
    }
}

/* MatNeoHookean, module/solid/constitutive_model.cpp:62-120 */
static void mat_neo_hookean(mo_ctx *c, double *sts, const double FF[3][3], const double *mp, double jac,
                            double jac_bar, int implicit) {
    double yng = mp[0], nu = mp[1];
    double lmd = nu * yng / ((1.0 + nu) * (1.0 - 2.0 * nu));
    double mu = yng / (2.0 * (1.0 + nu));
    double lnj = log(jac_bar);
    double be[3][3], sig[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) be[i][j] = FF[i][0] * FF[j][0] + FF[i][1] * FF[j][1] + FF[i][2] * FF[j][2];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) sig[i][j] = (mu * (be[i][j] - (i == j)) + lmd * lnj * (i == j)) / jac;
    sts[0] = sig[0][0]; sts[1] = sig[1][1]; sts[2] = sig[2][2];
    sts[3] = sig[1][2]; sts[4] = sig[0][2]; sts[5] = sig[0][1];
    if (implicit) {
        double c0 = lmd / jac, c1 = (mu - lmd * lnj) / jac;
        memset(c->stif, 0, sizeof(c->stif));
        for (int l = 0; l < 3; l++)
            for (int k = 0; k < 3; k++)
                for (int j = 0; j < 3; j++)
                    for (int i = 0; i < 3; i++)
                        c->stif[IDM[i][j]][IDM[k][l]] =
                            c0 * ((i == j) * (k == l)) + c1 * ((i == k) * (j == l) + (i == l) * (j == k));
    }
}

/* MatStVk, module/solid/constitutive_model.cpp:122-185; with `implicit` also
 * the 6x6 tangent lambda' be(x)be + mu' (be_ik be_jl + be_il be_jk), lambda' =
 * lambda / J, mu' = mu / J, in the Voigt slots IDM (:160-183) */
static void mat_stvk(mo_ctx *c, double *sts, const double FF[3][3], const double *mp, double jac, int implicit) {
    double yng = mp[0], nu = mp[1];
    double lmd = nu * yng / ((1.0 + nu) * (1.0 - 2.0 * nu));
    double mu = yng / (2.0 * (1.0 + nu));
    double be[3][3], be2[3][3], sig[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) be[i][j] = FF[i][0] * FF[j][0] + FF[i][1] * FF[j][1] + FF[i][2] * FF[j][2];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) be2[i][j] = be[i][0] * be[0][j] + be[i][1] * be[1][j] + be[i][2] * be[2][j];
    double tr_gls = 0.5 * (be[0][0] + be[1][1] + be[2][2] - 3.0);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) sig[i][j] = (mu * be2[i][j] + (lmd * tr_gls - mu) * be[i][j]) / jac;
    sts[0] = sig[0][0]; sts[1] = sig[1][1]; sts[2] = sig[2][2];
    sts[3] = sig[1][2]; sts[4] = sig[0][2]; sts[5] = sig[0][1];
    if (implicit) {
        double c0 = lmd / jac, c1 = mu / jac;
        memset(c->stif, 0, sizeof(c->stif));
        for (int l = 0; l < 3; l++)
            for (int k = 0; k < 3; k++)
                for (int j = 0; j < 3; j++)
                    for (int i = 0; i < 3; i++)
                        c->stif[IDM[i][j]][IDM[k][l]] =
                            c0 * (be[i][j] * be[k][l]) + c1 * (be[i][k] * be[j][l] + be[i][l] * be[j][k]);
    }
}

/* MatMooneyRivlin, module/solid/constitutive_model.cpp:187-285; mat_prop =
 * {c1, c2, bulk}.  With `implicit` also the 6x6 tangent of :235-283: the
 * volumetric part (bulk / J) I(x)I - 2 hp I4sym, the deviatoric-stress part
 * -2/3 (dev(s) (x) I + I (x) dev(s)) and the isochoric part (four terms). */
static void mat_mooney_rivlin(mo_ctx *c, double *sts, const double FF[3][3], const double *mp, double jac,
                              int implicit) {
    double c1 = mp[0], c2 = mp[1], bulk = mp[2];
    double fi[3][3], be[3][3], be2[3][3], sig[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) fi[i][j] = 1.0 / cbrt(jac) * FF[i][j];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) be[i][j] = fi[i][0] * fi[j][0] + fi[i][1] * fi[j][1] + fi[i][2] * fi[j][2];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) be2[i][j] = be[i][0] * be[0][j] + be[i][1] * be[1][j] + be[i][2] * be[2][j];
    double i1 = be[0][0] + be[1][1] + be[2][2];
    double i2 = 0.5 * (i1 * i1 - (be2[0][0] + be2[1][1] + be2[2][2]));
    double hp = bulk * log(jac) / jac;
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 3; j++) sig[i][j] = 2.0 * ((c1 + c2 * i1) * be[i][j] - c2 * be2[i][j]) / jac;
        sig[i][i] += hp - 2.0 / (3.0 * jac) * (c1 * i1 + 2.0 * c2 * i2);
    }
    sts[0] = sig[0][0]; sts[1] = sig[1][1]; sts[2] = sig[2][2];
    sts[3] = sig[1][2]; sts[4] = sig[0][2]; sts[5] = sig[0][1];
    if (implicit) {
        double trs = sig[0][0] + sig[1][1] + sig[2][2];
        double dev[3][3];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) dev[i][j] = sig[i][j] - trs / 3.0 * (i == j);
        memset(c->stif, 0, sizeof(c->stif));
        for (int l = 0; l < 3; l++)
            for (int k = 0; k < 3; k++)
                for (int j = 0; j < 3; j++)
                    for (int i = 0; i < 3; i++) {
                        double dij = (i == j), dkl = (k == l), dik = (i == k), djl = (j == l), dil = (i == l),
                               djk = (j == k);
                        double i4 = 0.5 * (dik * djl + dil * djk);
                        double aij = i1 * be[i][j] - be2[i][j], akl = i1 * be[k][l] - be2[k][l];
                        double c_hp = bulk / jac * (dij * dkl) - 2.0 * hp * i4;
                        double c_dev = -2.0 / 3.0 * (dev[i][j] * dkl + dij * dev[k][l]);
                        double t1 = 4.0 / (3.0 * jac) * (c1 * i1 + 2.0 * c2 * i2) * (i4 - (1.0 / 3.0) * dij * dkl);
                        double t2 = 4.0 * c2 / jac * (be[i][j] * be[k][l] - 0.5 * (be[i][k] * be[j][l] + be[i][l] * be[j][k]));
                        double t3 = -4.0 * c2 / (3.0 * jac) * (aij * dkl + dij * akl);
                        double t4 = 8.0 * c2 * i2 / (9.0 * jac) * dij * dkl;
                        c->stif[IDM[i][j]][IDM[k][l]] = c_hp + c_dev + (t1 + t2 + t3 + t4);
                    }
    }
}

/* Weakly compressible Newtonian fluid (material model 4, no counterpart in
 * the reference): Tait equation of state p = (rho0 c0^2 / gamma)((rho/rho0)^gamma - 1),
 * rho = rho0 / J, rho0 = m / V0, and sigma = -p I + 2 mu dev(D) with
 * D = sym(dF - I) / dt; mat_prop = {c0, gamma, mu}.  (rho/rho0)^gamma - 1 is
 * evaluated as expm1(-gamma log1p(J - 1)). */
static void mat_tait(mo_ctx *c, int p, double *sts, const double d[3][3], const double *mp) {
    double c0 = mp[0], gam = mp[1], mu = mp[2];
    double rho0 = c->mass[p] / c->vol0[p];
    double pr = rho0 * c0 * c0 / gam * expm1(-gam * log1p(c->jac[p] - 1.0));
    double inv_dt = 1.0 / c->dt;
    double d0 = (d[0][0] - 1.0) * inv_dt, d1 = (d[1][1] - 1.0) * inv_dt, d2 = (d[2][2] - 1.0) * inv_dt;
    double tr3 = (d0 + d1 + d2) / 3.0;
    sts[0] = -pr + 2.0 * mu * (d0 - tr3);
    sts[1] = -pr + 2.0 * mu * (d1 - tr3);
    sts[2] = -pr + 2.0 * mu * (d2 - tr3);
    sts[3] = mu * (d[1][2] + d[2][1]) * inv_dt;
    sts[4] = mu * (d[0][2] + d[2][0]) * inv_dt;
    sts[5] = mu * (d[0][1] + d[1][0]) * inv_dt;
}

/* ConstitutiveModel::UpdateStress dispatch, module/solid/constitutive_model.cpp:287-305 */
static void update_stress(mo_ctx *c, int p, double *sts, const double FF[3][3], const double d[3][3], int implicit) {
    int mid = c->matid[p];
    int model = c->iprop[mid];
    const double *mp = c->mat_prop + 3 * mid;
    if (model == -1) {
        for (int k = 0; k < 6; k++) sts[k] = 0.0;
        if (implicit) memset(c->stif, 0, sizeof(c->stif));
    } else if (model == 0) {
        mat_lin_elast(c, sts, d, mp, implicit);
    } else if (model == 1) {
        /* UpdateStress passes det_def_grad and det_def_grad_bar (constitutive_model.cpp:287-297) */
        mat_neo_hookean(c, sts, FF, mp, c->jac[p], c->fbar ? c->jbar[p] : c->jac[p], implicit);
    } else if (model == 2) {
        mat_stvk(c, sts, FF, mp, c->jac[p], implicit);
    } else if (model == 3) {
        mat_mooney_rivlin(c, sts, FF, mp, c->jac[p], implicit);
    } else if (model == 4 && !implicit) {
        mat_tait(c, p, sts, d, mp);
    }
}

static double det3(const double a[3][3]) {
    return a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) + a[0][1] * (a[1][2] * a[2][0] - a[1][0] * a[2][2]) +
           a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
}

/* InvMat3, module/cal_mat.h:38-66 */
static void inv3(const double a[3][3], double r[3][3]) {
    double det = 1.0 / det3(a);
    r[0][0] = (a[1][1] * a[2][2] - a[1][2] * a[2][1]) * det;
    r[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) * det;
    r[0][2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) * det;
    r[1][0] = (a[1][2] * a[2][0] - a[1][0] * a[2][2]) * det;
    r[1][1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) * det;
    r[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) * det;
    r[2][0] = (a[1][0] * a[2][1] - a[1][1] * a[2][0]) * det;
    r[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) * det;
    r[2][2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) * det;
}

/* --------------------------------------------------------------- explicit */
/* Control-point coordinate xyc[nid][dir] (DefineCpPos, module/mesh.h:32-47)
 * on one rank: xyminw = xymin, xymaxw = xymin + nel dx. */
static double cp_coord(const mo_ctx *c, int dir, int idx) {
    if (c->idimc[dir] == 1) return c->xmin[dir] + c->dx[dir] * (double)idx;
    if (idx == 0) return c->xmin[dir];
    if (idx == c->nnc[dir] - 1) return c->xmin[dir] + c->dx[dir] * (double)c->nel[dir];
    return c->xmin[dir] + c->dx[dir] * ((double)idx - 0.5);
}

/* The particle's affine velocity matrix A of TPIC (vel_grad) or APIC
 * (vel_Bmat . inv_Dmat, APIC::VarP2G, module/map_and_interpolate.h:108-118). */
static void affine_matrix(const mo_ctx *c, int p, double A[3][3]) {
    const double *B = c->aff + 9 * p, *Di = c->aff_dinv + 9 * p;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            if (c->scheme == 2) {
                A[i][j] = B[3 * i + j];
            } else {
                double t = 0.0;
                for (int k = 0; k < 3; k++) t += B[3 * i + k] * Di[3 * k + j];
                A[i][j] = t;
            }
        }
}

/* Momentum of one particle at one node: TPIC::VarP2G / APIC::VarP2G
 * (module/map_and_interpolate.h:62-77,104-130) with the node coordinate read
 * as xyc[nid][j] (the reference writes xyc[j][nid], past the end of xyc),
 * StandardVarP2G for PIC / FLIP. */
static void momentum_terms(const mo_ctx *c, int p, int n, double A[3][3], double out[3]) {
    const double *v = c->vel + 3 * p;
    if (c->scheme < 2) {
        out[0] = v[0]; out[1] = v[1]; out[2] = v[2];
        return;
    }
    int nx = c->nnc[0], ny = c->nnc[1];
    int idx[3] = {n % nx, (n / nx) % ny, n / (nx * ny)};
    double d[3];
    for (int j = 0; j < 3; j++) d[j] = cp_coord(c, j, idx[j]) - c->coord[3 * p + j];
    for (int i = 0; i < 3; i++) {
        double t = 0.0;
        for (int j = 0; j < 3; j++) t += A[i][j] * d[j];
        out[i] = v[i] + t;
    }
}

static void p2g(mo_ctx *c) {
    size_t N = (size_t)c->nodec;
    int nc[MAXN];
    double sf[MAXN], dsf[3 * MAXN];
    memset(c->nmass, 0, sizeof(double) * N);
    memset(c->nvof, 0, sizeof(double) * N);
    memset(c->nmome, 0, sizeof(double) * 3 * N);
    memset(c->nforce, 0, sizeof(double) * 3 * N);
    double fx = c->bb[0] * c->facl, fy = c->bb[1] * c->facl, fz = c->bb[2] * c->facl;
    FOR_PARTICLES(c, m, p) {
        const double *s = c->stress + 6 * p;
        int ne = maksf(c, m, c->coord + 3 * p, nc, sf, dsf);
        double mp = c->mass[p], vp = c->vol[p];
        double A[3][3];
        if (c->scheme >= 2) affine_matrix(c, p, A);
        for (int i = 0; i < ne; i++) {
            int n = nc[i];
            double N_ = sf[i], d1 = dsf[3 * i], d2 = dsf[3 * i + 1], d3 = dsf[3 * i + 2];
            double vm[3];
            momentum_terms(c, p, n, A, vm);
            c->nmass[n] += N_ * mp;
            c->nvof[n] += N_ * vp;
            c->nmome[n] += N_ * mp * vm[0];
            c->nmome[N + n] += N_ * mp * vm[1];
            c->nmome[2 * N + n] += N_ * mp * vm[2];
            /* ComputeInternalForce / ComputeExternalForce, solid_material_point.h:48-73 */
            double fi0 = -vp * (s[0] * d1 + s[5] * d2 + s[4] * d3);
            double fi1 = -vp * (s[5] * d1 + s[1] * d2 + s[3] * d3);
            double fi2 = -vp * (s[4] * d1 + s[3] * d2 + s[2] * d3);
            double fe0 = N_ * (mp * fx), fe1 = N_ * (mp * fy), fe2 = N_ * (mp * fz);
            c->nforce[n] += fi0 + fe0;
            c->nforce[N + n] += fi1 + fe1;
            c->nforce[2 * N + n] += fi2 + fe2;
        }
    }
    for (size_t n = 0; n < N; n++) {
        if (c->nmass[n] > c->mtol) {
            for (int k = 0; k < 3; k++) c->nvel[k * N + n] = c->nmome[k * N + n] / c->nmass[n];
        } else {
            for (int k = 0; k < 3; k++) c->nvel[k * N + n] = 0.0;
        }
        if (c->nvof[n] < c->mtol) c->nvof[n] = 0.0;
    }
    bc_set_val(c, c->nvel);
}

static void grid_update(mo_ctx *c) {
    size_t N = (size_t)c->nodec;
    for (size_t n = 0; n < N; n++) {
        for (int k = 0; k < 3; k++)
            c->naccel[k * N + n] = (c->nmass[n] > c->mtol) ? c->nforce[k * N + n] / c->nmass[n] : 0.0;
    }
    bc_set_zero(c, c->naccel);
}

/* DeltaCorrectionParticleShifting, module/material_point.cpp:174-228 */
static void shifting(mo_ctx *c, double *delta) {
    size_t N = (size_t)c->nodec;
    int nc[MAXN];
    double sf[MAXN], dsf[3 * MAXN];
    double *nei = (double *)malloc(sizeof(double) * N);
    double eu = 0.0;
    for (size_t i = 0; i < N; i++) {
        double e = c->nvof[i] - c->nvol[i];
        nei[i] = e > 0.0 ? e : 0.0;
        eu += nei[i] * nei[i]; /* dbc = 1 on one rank */
    }
    double *geup = (double *)zalloc(sizeof(double) * 3 * (size_t)c->num);
    FOR_PARTICLES(c, m, p) {
        int ne = maksf(c, m, c->coord + 3 * p, nc, sf, dsf);
        for (int i = 0; i < ne; i++)
            for (int k = 0; k < 3; k++) geup[3 * p + k] += dsf[3 * i + k] * nei[nc[i]];
    }
    double gd = 0.0;
    for (int p = 0; p < c->num; p++)
        for (int k = 0; k < 3; k++) {
            geup[3 * p + k] *= 2.0 * c->vol[p];
            gd += geup[3 * p + k] * geup[3 * p + k];
        }
    double b0 = (gd < c->mtol) ? 0.0 : eu / gd;
    for (int p = 0; p < c->num; p++)
        for (int k = 0; k < 3; k++) delta[3 * p + k] = -b0 * geup[3 * p + k];
    free(nei);
    free(geup);
}

static void g2p_explicit(mo_ctx *c) {
    size_t N = (size_t)c->nodec;
    int nc[MAXN];
    double sf[MAXN], dsf[3 * MAXN];
    int flip = (c->scheme == 1);
    if (!flip) {
        for (size_t i = 0; i < 3 * N; i++) c->nvel[i] += c->dt * c->naccel[i];
        memset(c->vel, 0, sizeof(double) * 3 * c->num);
    }
    if (c->scheme >= 2) {
        memset(c->aff, 0, sizeof(double) * 9 * (size_t)c->num);
        memset(c->aff_dinv, 0, sizeof(double) * 9 * (size_t)c->num);
    }
    FOR_PARTICLES(c, m, p) {
        int ne = maksf(c, m, c->coord + 3 * p, nc, sf, dsf);
        double D[3][3] = {{0}};
        double *B = c->aff + 9 * p;
        for (int i = 0; i < ne; i++) {
            for (int k = 0; k < 3; k++) {
                if (!flip) c->vel[3 * p + k] += sf[i] * c->nvel[k * N + nc[i]];           /* PIC::VarG2P */
                else c->vel[3 * p + k] += sf[i] * c->dt * c->naccel[k * N + nc[i]];       /* FLIP::VarG2P */
            }
            if (c->scheme == 2) {
                /* TPIC::VarGradG2P (map_and_interpolate.h:79-98): vel_grad[a][j] += dsf_j nvel_a */
                for (int a = 0; a < 3; a++)
                    for (int j = 0; j < 3; j++) B[3 * a + j] += dsf[3 * i + j] * c->nvel[a * N + nc[i]];
            } else if (c->scheme == 3) {
                /* APIC::VarBmatG2P and DmatG2P (map_and_interpolate.h:132-162) */
                int n = nc[i], nx = c->nnc[0], ny = c->nnc[1];
                int idx[3] = {n % nx, (n / nx) % ny, n / (nx * ny)};
                double d[3];
                for (int j = 0; j < 3; j++) d[j] = cp_coord(c, j, idx[j]) - c->coord[3 * p + j];
                for (int a = 0; a < 3; a++)
                    for (int j = 0; j < 3; j++) {
                        B[3 * a + j] += sf[i] * c->nvel[a * N + n] * d[j];
                        D[a][j] += sf[i] * d[a] * d[j];
                    }
            }
        }
        if (c->scheme == 3) {
            /* APIC::InvDmatG2P (map_and_interpolate.h:164-172) */
            double Di[3][3];
            inv3(D, Di);
            for (int a = 0; a < 3; a++)
                for (int j = 0; j < 3; j++) c->aff_dinv[9 * p + 3 * a + j] = Di[a][j];
        }
    }
    /* MUSL, var_trans_solid_explicit.cpp:101-148 */
    memset(c->nmome, 0, sizeof(double) * 3 * N);
    FOR_PARTICLES(c, m, p) {
        int ne = maksf(c, m, c->coord + 3 * p, nc, sf, dsf);
        double A[3][3];
        if (c->scheme >= 2) affine_matrix(c, p, A);
        for (int i = 0; i < ne; i++) {
            double vm[3];
            momentum_terms(c, p, nc[i], A, vm);
            for (int k = 0; k < 3; k++) c->nmome[k * N + nc[i]] += sf[i] * c->mass[p] * vm[k];
        }
    }
    for (size_t n = 0; n < N; n++)
        for (int k = 0; k < 3; k++)
            c->nvel[k * N + n] = (c->nmass[n] > c->mtol) ? c->nmome[k * N + n] / c->nmass[n] : 0.0;
    bc_set_val(c, c->nvel);
    /* deformation gradient, var_trans_solid_explicit.cpp:247-296 */
    double *dF = (double *)malloc(sizeof(double) * 9 * (size_t)c->num);
    FOR_PARTICLES(c, m, p) {
        int ne = maksf(c, m, c->coord + 3 * p, nc, sf, dsf);
        double d[3][3] = {{0}};
        for (int i = 0; i < ne; i++)
            for (int a = 0; a < 3; a++)
                for (int j = 0; j < 3; j++) d[a][j] += dsf[3 * i + j] * c->nvel[a * N + nc[i]] * c->dt;
        for (int a = 0; a < 3; a++) d[a][a] += 1.0;
        double Fn[3][3] = {{0}};
        double *Fp = c->F + 9 * p;
        for (int a = 0; a < 3; a++)
            for (int j = 0; j < 3; j++)
                for (int k = 0; k < 3; k++) Fn[a][j] += d[a][k] * Fp[3 * k + j];
        for (int a = 0; a < 3; a++)
            for (int j = 0; j < 3; j++) { Fp[3 * a + j] = Fn[a][j]; dF[9 * p + 3 * a + j] = d[a][j]; }
        c->jac[p] = det3(Fn);
    }
    /* cal_def_grad_bar (module/solid/explicit/fbar_projection.cpp:18-93): the trial
     * J = det_def_grad_bar det(dF) projected to the nodes by volume (sum N J vol / nvof),
     * gathered back as Jbar; dF scaled by cbrt(Jbar / J); def_grad_bar <- dF def_grad_bar,
     * det_def_grad_bar <- Jbar */
    if (c->fbar) {
        double *nJ = (double *)zalloc(sizeof(double) * N);
        FOR_PARTICLES(c, m, p) {
            int ne = maksf(c, m, c->coord + 3 * p, nc, sf, dsf);
            double d[3][3];
            for (int a = 0; a < 3; a++)
                for (int j = 0; j < 3; j++) d[a][j] = dF[9 * p + 3 * a + j];
            double jt = c->jbar[p] * det3(d);
            for (int i = 0; i < ne; i++) nJ[nc[i]] += sf[i] * jt * c->vol[p];
        }
        for (size_t n = 0; n < N; n++) nJ[n] = (c->nvof[n] > c->mtol) ? nJ[n] / c->nvof[n] : 0.0;
        FOR_PARTICLES(c, m, p) {
            int ne = maksf(c, m, c->coord + 3 * p, nc, sf, dsf);
            double Jb = 0.0;
            for (int i = 0; i < ne; i++) Jb += sf[i] * nJ[nc[i]];
            double d[3][3];
            for (int a = 0; a < 3; a++)
                for (int j = 0; j < 3; j++) d[a][j] = dF[9 * p + 3 * a + j];
            double J = c->jbar[p] * det3(d);
            double sc = cbrt(Jb / J);
            for (int a = 0; a < 9; a++) dF[9 * p + a] *= sc;
            double Fb[3][3] = {{0}};
            for (int a = 0; a < 3; a++)
                for (int j = 0; j < 3; j++)
                    for (int k = 0; k < 3; k++) Fb[a][j] += dF[9 * p + 3 * a + k] * c->fbarF[9 * p + 3 * k + j];
            for (int a = 0; a < 3; a++)
                for (int j = 0; j < 3; j++) c->fbarF[9 * p + 3 * a + j] = Fb[a][j];
            c->jbar[p] = Jb;
        }
        free(nJ);
    }
    /* update_point_coord_and_stress, var_trans_solid_explicit.cpp:150-185 */
    double *delta = (double *)zalloc(sizeof(double) * 3 * (size_t)c->num);
    shifting(c, delta);
    FOR_PARTICLES(c, m, p) {
        double xp[3] = {c->coord[3 * p], c->coord[3 * p + 1], c->coord[3 * p + 2]};
        int ne = maksf(c, m, xp, nc, sf, dsf);
        for (int i = 0; i < ne; i++)
            for (int k = 0; k < 3; k++) c->coord[3 * p + k] += sf[i] * c->dt * c->nvel[k * N + nc[i]];
        if (c->shifting)
            for (int k = 0; k < 3; k++) c->coord[3 * p + k] += delta[3 * p + k];
        c->vol[p] = c->jac[p] * c->vol0[p];
        double Fm[3][3], dm[3][3];
        const double *Fsrc = c->fbar ? c->fbarF : c->F;   /* F-bar: the stress sees def_grad_bar */
        for (int a = 0; a < 3; a++)
            for (int j = 0; j < 3; j++) { Fm[a][j] = Fsrc[9 * p + 3 * a + j]; dm[a][j] = dF[9 * p + 3 * a + j]; }
        update_stress(c, p, c->stress + 6 * p, Fm, dm, 0);
    }
    free(dF);
    free(delta);
}

int mo_explicit_p2g(mo_ctx *c, double facl) {
    c->facl = facl;
    linklist(c);
    p2g(c);
    grid_update(c);
    return 0;
}

int mo_explicit_steps(mo_ctx *c, int nsteps, double facl) {
    c->facl = facl;
    for (int s = 0; s < nsteps; s++) {
        linklist(c);
        p2g(c);
        grid_update(c);
        g2p_explicit(c);
    }
    return 0;
}

int mo_get_nodal(const mo_ctx *c, int field, double *out) {
    size_t N = (size_t)c->nodec;
    const double *src = NULL;
    size_t n = N;
    switch (field) {
    case 0: src = c->nmass; break;
    case 1: src = c->nvof; break;
    case 2: src = c->nmome; n = 3 * N; break;
    case 3: src = c->nforce; n = 3 * N; break;
    case 4: src = c->nvel; n = 3 * N; break;
    case 5: src = c->naccel; n = 3 * N; break;
    case 6: src = c->nvol; break;
    case 7: src = c->ndispl; n = 3 * N; break;
    default: return -1;
    }
    memcpy(out, src, sizeof(double) * n);
    return (int)n;
}

int mo_set_fbar(mo_ctx *c, int on) {
    c->fbar = on != 0;
    return 0;
}

int mo_get_fbar(const mo_ctx *c, double *Fbar, double *Jbar) {
    if (Fbar) memcpy(Fbar, c->fbarF, sizeof(double) * 9 * (size_t)c->num);
    if (Jbar) memcpy(Jbar, c->jbar, sizeof(double) * (size_t)c->num);
    return c->num;
}

int mo_get_affine(const mo_ctx *c, double *out) {
    if (c->scheme < 2) {
        memset(out, 0, sizeof(double) * 9 * (size_t)c->num);
        return c->num;
    }
    for (int p = 0; p < c->num; p++) {
        double A[3][3];
        affine_matrix(c, p, A);
        for (int a = 0; a < 3; a++)
            for (int j = 0; j < 3; j++) out[9 * p + 3 * a + j] = A[a][j];
    }
    return c->num;
}

int mo_get_particles(const mo_ctx *c, double *coord, double *vel, double *F, double *stress, double *vol) {
    size_t n = (size_t)c->num;
    if (coord) memcpy(coord, c->coord, sizeof(double) * 3 * n);
    if (vel) memcpy(vel, c->vel, sizeof(double) * 3 * n);
    if (F) memcpy(F, c->F, sizeof(double) * 9 * n);
    if (stress) memcpy(stress, c->stress, sizeof(double) * 6 * n);
    if (vol) memcpy(vol, c->vol, sizeof(double) * n);
    return c->num;
}

/* =============================================================== implicit */
/* CrsMat::BuildCrsMat, module/solver/crsmat.cpp:21-81 */
static void build_crs(mo_ctx *c) {
    int nx = c->nnc[0], ny = c->nnc[1], nz = c->nnc[2];
    int w = 0;
    for (int i = 0; i < 3; i++) w = c->idimc[i] > w ? c->idimc[i] : w;
    size_t cap = (size_t)c->nodec * (size_t)((2 * w + 1) * (2 * w + 1) * (2 * w + 1));
    free(c->matrow); free(c->matcolid);
    c->matrow = (int *)malloc(sizeof(int) * ((size_t)c->nodec + 1));
    int *col = (int *)malloc(sizeof(int) * cap);
    int nmat = 0;
    for (int kz = 0; kz < nz; kz++) {
        int zs = kz - c->idimc[2] < 0 ? 0 : kz - c->idimc[2], ze = kz + c->idimc[2] >= nz ? nz - 1 : kz + c->idimc[2];
        for (int jy = 0; jy < ny; jy++) {
            int ys = jy - c->idimc[1] < 0 ? 0 : jy - c->idimc[1], ye = jy + c->idimc[1] >= ny ? ny - 1 : jy + c->idimc[1];
            for (int ix = 0; ix < nx; ix++) {
                int xs = ix - c->idimc[0] < 0 ? 0 : ix - c->idimc[0];
                int xe = ix + c->idimc[0] >= nx ? nx - 1 : ix + c->idimc[0];
                c->matrow[ix + nx * jy + nx * ny * kz] = nmat;
                for (int z = zs; z <= ze; z++)
                    for (int y = ys; y <= ye; y++)
                        for (int x = xs; x <= xe; x++) col[nmat++] = x + nx * y + nx * ny * z;
            }
        }
    }
    c->matrow[c->nodec] = nmat;
    c->nmat_csr = nmat;
    c->matcolid = (int *)realloc(col, sizeof(int) * (size_t)nmat);
    free(c->amat); free(c->adiag); free(c->b_rhs); free(c->x_lhs);
    c->amat = (double *)zalloc(sizeof(double) * 9 * (size_t)nmat);
    c->adiag = (double *)zalloc(sizeof(double) * 3 * (size_t)c->nodec);
    c->b_rhs = (double *)zalloc(sizeof(double) * 3 * (size_t)c->nodec);
    c->x_lhs = (double *)zalloc(sizeof(double) * 3 * (size_t)c->nodec);
}

/* GeneralizedAlphaParaSet + NewmarkBetaParaSet, nonlinear_time_integration.cpp:10-56 (ode_order 2) */
int mo_implicit_setup(mo_ctx *c, int nr_flag, double spec_rad) {
    c->nr_flag = nr_flag;
    double t = 1.0 + spec_rad;
    c->alpha_f = 1.0 / t;
    c->alpha_m = (2.0 - spec_rad) / t;
    t = 1.0 - c->alpha_f + c->alpha_m;
    c->gamma_nb = t - 0.5;
    c->beta_nb = 0.25 * t * t;
    double g = c->gamma_nb, b = c->beta_nb, dt = c->dt;
    c->nb[0] = g / (b * dt);
    c->nb[1] = g / b - 1.0;
    c->nb[2] = dt / 2.0 * (g / b - 2.0);
    c->nb[3] = 1.0 / (b * dt * dt);
    c->nb[4] = 1.0 / (b * dt);
    c->nb[5] = 1.0 / (2.0 * b) - 1.0;
    build_crs(c);
    memset(c->ndispl, 0, sizeof(double) * 3 * (size_t)c->nodec);
    return c->nmat_csr;
}

int mo_implicit_nnzb(const mo_ctx *c) { return c->nmat_csr; }

/* SolidMaterialPoint::Particle2Node, var_trans_solid_implicit.cpp:20-80 */
static void p2g_implicit(mo_ctx *c) {
    size_t N = (size_t)c->nodec;
    int nc[MAXN];
    double sf[MAXN], dsf[3 * MAXN];
    memset(c->nmass, 0, sizeof(double) * N);
    memset(c->nvof, 0, sizeof(double) * N);
    memset(c->nmome, 0, sizeof(double) * 3 * N);
    memset(c->nforce, 0, sizeof(double) * 3 * N);
    FOR_PARTICLES(c, m, p) {
        int ne = maksf(c, m, c->coord + 3 * p, nc, sf, dsf);
        for (int i = 0; i < ne; i++) {
            int n = nc[i];
            c->nmass[n] += sf[i] * c->mass[p];
            c->nvof[n] += sf[i] * c->vol[p];
            for (int k = 0; k < 3; k++) c->nmome[k * N + n] += sf[i] * c->mass[p] * c->vel[3 * p + k];
            for (int k = 0; k < 3; k++) c->nforce[k * N + n] += sf[i] * c->mass[p] * c->accel[3 * p + k];
        }
    }
    memset(c->nvel, 0, sizeof(double) * 3 * N);
    memset(c->naccel, 0, sizeof(double) * 3 * N);
    for (size_t n = 0; n < N; n++)
        if (c->nmass[n] > c->mtol)
            for (int k = 0; k < 3; k++) {
                c->nvel[k * N + n] = c->nmome[k * N + n] / c->nmass[n];
                c->naccel[k * N + n] = c->nforce[k * N + n] / c->nmass[n];
            }
    bc_set_val(c, c->nvel);
    bc_set_zero(c, c->naccel);
}

/* PredictNewmarkBetaVelAndAccel, nonlinear_time_integration.cpp:59-71 */
static void predict(const mo_ctx *c, double *nvel_k, double *naccel_k) {
    for (size_t n = 0; n < 3 * (size_t)c->nodec; n++) {
        nvel_k[n] = c->nb[0] * c->ndispl[n] - c->nb[1] * c->nvel[n] - c->nb[2] * c->naccel[n];
        naccel_k[n] = c->nb[3] * c->ndispl[n] - c->nb[4] * c->nvel[n] - c->nb[5] * c->naccel[n];
    }
}

/* ComputeDeltaDefGrad, material_point.cpp:127-151 */
static void delta_def_grad(const mo_ctx *c, const int *nc, int ne, double af, const double *dsf, double d[3][3]) {
    size_t N = (size_t)c->nodec;
    memset(d, 0, sizeof(double) * 9);
    for (int i = 0; i < ne; i++)
        for (int a = 0; a < 3; a++)
            for (int j = 0; j < 3; j++) d[a][j] += dsf[3 * i + j] * af * c->ndispl[a * N + nc[i]];
    d[0][0] += 1.0; d[1][1] += 1.0; d[2][2] += 1.0;
}

/* UpdateDefGrad, var_trans_solid_implicit.cpp:82-104: returns F_new, updates jac & vol */
static void update_def_grad(mo_ctx *c, int p, const int *nc, int ne, double af, const double *dsf, double d[3][3],
                            double Fn[3][3]) {
    delta_def_grad(c, nc, ne, af, dsf, d);
    const double *Fp = c->F + 9 * p;
    for (int a = 0; a < 3; a++)
        for (int j = 0; j < 3; j++) {
            Fn[a][j] = 0.0;
            for (int k = 0; k < 3; k++) Fn[a][j] += d[a][k] * Fp[3 * k + j];
        }
    c->jac[p] = det3(Fn);
    c->vol[p] = c->jac[p] * c->vol0[p];
}

/* CrsMat::FindIndex, crsmat.h:42-51 (same result: the CSR slot of column njd in row nid) */
static int find_index(const mo_ctx *c, int nid, int njd) {
    for (int j = c->matrow[nid]; j < c->matrow[nid + 1]; j++)
        if (c->matcolid[j] == njd) return j;
    return -1;
}

/* SolidMaterialPoint::AssembleSystem, solve_solid_implicit.cpp:105-204, followed by
 * CrsMat::BuildDiagonalPreconditioner, crsmat.cpp:87-184 */
static void assemble(mo_ctx *c, const double *naccel_k, double *stress_k) {
    size_t N = (size_t)c->nodec;
    size_t nm = (size_t)c->nmat_csr;
    double af = c->alpha_f, am = c->alpha_m;
    int nc[MAXN];
    double sf[MAXN], dsf[3 * MAXN];
    memset(c->amat, 0, sizeof(double) * 9 * nm);
    memset(c->adiag, 0, sizeof(double) * 3 * N);
    memset(c->b_rhs, 0, sizeof(double) * 3 * N);
    double fx = c->bb[0] * c->facl, fy = c->bb[1] * c->facl, fz = c->bb[2] * c->facl;
    FOR_PARTICLES(c, m, p) {
        int ne = maksf(c, m, c->coord + 3 * p, nc, sf, dsf);
        double d[3][3], Fn[3][3];
        update_def_grad(c, p, nc, ne, af, dsf, d, Fn);
        update_stress(c, p, stress_k + 6 * p, Fn, d, 1);
        /* ImplicitDsfCorr, material_point.cpp:153-172 */
        double d2[3][3], di[3][3];
        delta_def_grad(c, nc, ne, af, dsf, d2);
        inv3(d2, di);
        for (int i = 0; i < ne; i++) {
            double t[3];
            for (int j = 0; j < 3; j++) t[j] = dsf[3 * i] * di[0][j] + dsf[3 * i + 1] * di[1][j] + dsf[3 * i + 2] * di[2][j];
            for (int j = 0; j < 3; j++) dsf[3 * i + j] = t[j];
        }
        const double *s = stress_k + 6 * p;
        double sm[3][3];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) sm[i][j] = s[IDM[i][j]];
        /* ComputeTangentModulus, solve_solid_implicit.cpp:34-63 */
        double ce[3][3][3][3];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
                for (int k = 0; k < 3; k++)
                    for (int l = 0; l < 3; l++) {
                        ce[i][j][k][l] = c->stif[IDM[i][j]][IDM[k][l]];
                        if (c->nr_flag) ce[i][j][k][l] += sm[j][l] * (i == k);
                    }
        double vp = c->vol[p], mp = c->mass[p];
        for (int a = 0; a < ne; a++) {
            int nid = nc[a];
            double emd = c->nb[3] * sf[a] * mp; /* ComputeNRLumpedMat, material_point.h:144 */
            for (int b = 0; b < ne; b++) {
                int njd = nc[b];
                int ida = find_index(c, nid, njd);
                double K[3][3] = {{0}};
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++)
                        for (int k = 0; k < 3; k++)
                            for (int l = 0; l < 3; l++) K[i][j] += dsf[3 * a + k] * ce[i][k][j][l] * dsf[3 * b + l];
                if (nid == njd) {
                    c->amat[ida + 0 * nm] += am * emd;
                    c->amat[ida + 4 * nm] += am * emd;
                    c->amat[ida + 8 * nm] += am * emd;
                }
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++) c->amat[ida + (3 * i + j) * nm] += af * K[i][j] * vp;
            }
            double d1 = dsf[3 * a], d2_ = dsf[3 * a + 1], d3 = dsf[3 * a + 2];
            double fi0 = -vp * (s[0] * d1 + s[5] * d2_ + s[4] * d3);
            double fi1 = -vp * (s[5] * d1 + s[1] * d2_ + s[3] * d3);
            double fi2 = -vp * (s[4] * d1 + s[3] * d2_ + s[2] * d3);
            c->b_rhs[nid] += fi0 + sf[a] * (mp * fx);
            c->b_rhs[N + nid] += fi1 + sf[a] * (mp * fy);
            c->b_rhs[2 * N + nid] += fi2 + sf[a] * (mp * fz);
        }
    }
    /* AddInertialForceToRHS, material_point.h:151-161 */
    for (size_t n = 0; n < N; n++)
        for (int k = 0; k < 3; k++) {
            double aam = am * naccel_k[k * N + n] + (1.0 - am) * c->naccel[k * N + n];
            c->b_rhs[k * N + n] -= c->nmass[n] * aam;
        }
    /* ExtractDiagonal + ComputeDiagonalInverseSqrt + ApplyDiagonalScaling (FEM_flag false) */
    for (size_t i = 0; i < N; i++) {
        int jd = find_index(c, (int)i, (int)i);
        for (int k = 0; k < 3; k++) c->adiag[k * N + i] = c->amat[jd + (size_t)(4 * k) * nm];
    }
    for (size_t n = 0; n < 3 * N; n++) {
        double a = fabs(c->adiag[n]);
        c->adiag[n] = (a < c->mtol) ? 0.0 : 1.0 / sqrt(a);
    }
    for (size_t i = 0; i < N; i++)
        for (int j = c->matrow[i]; j < c->matrow[i + 1]; j++) {
            int col = c->matcolid[j];
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) c->amat[j + (size_t)(3 * a + b) * nm] *= c->adiag[a * N + i] * c->adiag[b * N + col];
        }
}

/* CrsMat::MatVecMult + BCResidualSet, solver.cpp:405-433 */
static void matvec(const mo_ctx *c, const double *x, double *y) {
    size_t N = (size_t)c->nodec, nm = (size_t)c->nmat_csr;
    memset(y, 0, sizeof(double) * 3 * N);
    for (size_t i = 0; i < N; i++)
        for (int j = c->matrow[i]; j < c->matrow[i + 1]; j++) {
            int col = c->matcolid[j];
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) y[i + a * N] += c->amat[j + (size_t)(3 * a + b) * nm] * x[col + b * N];
        }
    bc_set_zero(c, y);
}

int mo_implicit_matvec(mo_ctx *c, const double *x, double *y) {
    matvec(c, x, y);
    return 0;
}

/* GPBiCGSafe, solver.cpp:19-141.  eps is the stopping threshold on the squared
 * norm ratio (the reference uses 1e-8); kmax bounds the iterations (10000 there).
 * Starts from c->x_lhs; returns iterations, or -1 if kmax is reached. */
static int gpbicgsafe(mo_ctx *c, double eps, int kmax) {
    size_t n3 = 3 * (size_t)c->nodec;
    double *rr = zalloc(sizeof(double) * n3), *pp = zalloc(sizeof(double) * n3), *tt = zalloc(sizeof(double) * n3);
    double *Ap = zalloc(sizeof(double) * n3), *Ar = zalloc(sizeof(double) * n3), *Az = zalloc(sizeof(double) * n3);
    double *Au = zalloc(sizeof(double) * n3), *Ax = zalloc(sizeof(double) * n3), *rs = zalloc(sizeof(double) * n3);
    double *uu = zalloc(sizeof(double) * n3), *zz = zalloc(sizeof(double) * n3);
    /* ScaleSolution, crsmat.cpp:190-209 */
    for (size_t n = 0; n < n3; n++) {
        if (c->adiag[n] < c->mtol) { c->x_lhs[n] = 0.0; rr[n] = 0.0; }
        else { c->x_lhs[n] /= c->adiag[n]; rr[n] = c->b_rhs[n] * c->adiag[n]; }
    }
    bc_set_zero(c, rr);
    matvec(c, c->x_lhs, Ax);
    double rtr = 0.0;
    for (size_t n = 0; n < n3; n++) {
        double r = rr[n] - Ax[n];
        rr[n] = r;
        rs[n] = r;
        rtr += r * r;
    }
    double rsr = rtr, btb = rtr;
    double epsbtb = eps * btb;
    double beta = 0.0;
    int iter;
    for (iter = 0; iter < kmax; iter++) {
        if (btb < 1.0e-300) break;
        matvec(c, rr, Ar);
        double rAp = 0.0;
        for (size_t n = 0; n < n3; n++) {
            pp[n] = rr[n] + beta * (pp[n] - uu[n]);
            Ap[n] = Ar[n] + beta * (Ap[n] - Au[n]);
            rAp += rs[n] * Ap[n];
        }
        double rsr0 = rsr, alph = rsr0 / rAp;
        double AzAz = 0, Arrr = 0, Azrr = 0, ArAz = 0, ArAr = 0;
        for (size_t n = 0; n < n3; n++) {
            AzAz += Az[n] * Az[n]; Arrr += Ar[n] * rr[n]; Azrr += Az[n] * rr[n];
            ArAz += Ar[n] * Az[n]; ArAr += Ar[n] * Ar[n];
        }
        double zeta, eta;
        if (iter == 0) { zeta = Arrr / ArAr; eta = 0.0; }
        else {
            double den = ArAr * AzAz - ArAz * ArAz;
            zeta = (AzAz * Arrr - Azrr * ArAz) / den;
            eta = (ArAr * Azrr - ArAz * Arrr) / den;
        }
        for (size_t n = 0; n < n3; n++) uu[n] = zeta * Ap[n] + eta * (Az[n] + beta * uu[n]);
        matvec(c, uu, Au);
        rsr = 0.0; rtr = 0.0;
        for (size_t n = 0; n < n3; n++) {
            tt[n] = rr[n] - alph * Ap[n];
            zz[n] = zeta * rr[n] + eta * zz[n] - alph * uu[n];
            Az[n] = zeta * Ar[n] + eta * Az[n] - alph * Au[n];
            c->x_lhs[n] += alph * pp[n] + zz[n];
            rr[n] = tt[n] - Az[n];
            rsr += rs[n] * rr[n];
            rtr += rr[n] * rr[n];
        }
        if (rtr < epsbtb) break;
        beta = (alph / zeta) * (rsr / rsr0);
    }
    /* RestorSolution, crsmat.cpp:214-230 */
    for (size_t n = 0; n < n3; n++) c->x_lhs[n] = (c->adiag[n] > c->mtol) ? c->x_lhs[n] * c->adiag[n] : 0.0;
    free(rr); free(pp); free(tt); free(Ap); free(Ar); free(Az); free(Au); free(Ax); free(rs); free(uu); free(zz);
    return iter >= kmax ? -1 : iter;
}

int mo_implicit_assemble(mo_ctx *c, double facl) {
    c->facl = facl;
    linklist(c);
    p2g_implicit(c);
    size_t n3 = 3 * (size_t)c->nodec;
    double *nvel_k = zalloc(sizeof(double) * n3), *naccel_k = zalloc(sizeof(double) * n3);
    double *stress_k = malloc(sizeof(double) * 6 * (size_t)c->num);
    memcpy(stress_k, c->stress, sizeof(double) * 6 * (size_t)c->num);
    memset(c->ndispl, 0, sizeof(double) * n3);
    memset(c->x_lhs, 0, sizeof(double) * n3);
    bc_set_dt(c, c->ndispl);
    predict(c, nvel_k, naccel_k);
    assemble(c, naccel_k, stress_k);
    free(nvel_k); free(naccel_k); free(stress_k);
    return c->nmat_csr;
}

int mo_implicit_get_matrix(const mo_ctx *c, int *matrow, int *matcolid, double *amat, double *adiag, double *b_rhs) {
    size_t N = (size_t)c->nodec, nm = (size_t)c->nmat_csr;
    if (matrow) memcpy(matrow, c->matrow, sizeof(int) * (N + 1));
    if (matcolid) memcpy(matcolid, c->matcolid, sizeof(int) * nm);
    if (amat) memcpy(amat, c->amat, sizeof(double) * 9 * nm);
    if (adiag) memcpy(adiag, c->adiag, sizeof(double) * 3 * N);
    if (b_rhs) memcpy(b_rhs, c->b_rhs, sizeof(double) * 3 * N);
    return (int)nm;
}

int mo_implicit_solve(mo_ctx *c, double eps, int kmax, double *x_out) {
    memset(c->x_lhs, 0, sizeof(double) * 3 * (size_t)c->nodec);
    int it = gpbicgsafe(c, eps, kmax);
    if (x_out) memcpy(x_out, c->x_lhs, sizeof(double) * 3 * (size_t)c->nodec);
    return it;
}

/* CrsMat::ComputeRefResidual / ComputeAbsResidual, solver.cpp:484-555 (native path) */
static void nr_residuals(mo_ctx *c, double *ref, double *absr) {
    size_t n3 = 3 * (size_t)c->nodec;
    double *xp = zalloc(sizeof(double) * n3), *Ax = zalloc(sizeof(double) * n3);
    bc_set_zero(c, c->b_rhs);
    for (size_t n = 0; n < n3; n++) xp[n] = (c->adiag[n] > c->mtol) ? c->x_lhs[n] / c->adiag[n] : 0.0;
    matvec(c, xp, Ax);
    double rtr = 0.0, idof = 0.0;
    for (size_t n = 0; n < n3; n++) {
        double axp = (c->adiag[n] > c->mtol) ? Ax[n] / c->adiag[n] : 0.0;
        double r = c->b_rhs[n] - axp;
        rtr += r * r;
        if (c->adiag[n] > c->mtol) idof += 1.0;
    }
    *ref = sqrt(rtr);
    *absr = idof <= 1.0e-30 ? 0.0 : sqrt(rtr / idof);
    free(xp); free(Ax);
}

/* Node2Particle, var_trans_solid_implicit.cpp:106-167, with CommitNodalKinematics and
 * CommitParticleKinematics, nonlinear_time_integration.cpp:73-96 */
static void g2p_implicit(mo_ctx *c) {
    size_t N = (size_t)c->nodec;
    size_t n3 = 3 * N;
    double *nvel_k = zalloc(sizeof(double) * n3), *naccel_k = zalloc(sizeof(double) * n3);
    predict(c, nvel_k, naccel_k);
    memcpy(c->nvel, nvel_k, sizeof(double) * n3);
    memcpy(c->naccel, naccel_k, sizeof(double) * n3);
    int flip = (c->scheme == 1);
    size_t np = (size_t)c->num;
    double *accel_old = zalloc(sizeof(double) * 3 * np), *disp = zalloc(sizeof(double) * 3 * np);
    if (flip) memcpy(accel_old, c->accel, sizeof(double) * 3 * np);
    memset(c->accel, 0, sizeof(double) * 3 * np);
    if (!flip) memset(c->vel, 0, sizeof(double) * 3 * np);
    int nc[MAXN];
    double sf[MAXN], dsf[3 * MAXN];
    FOR_PARTICLES(c, m, p) {
        int ne = maksf(c, m, c->coord + 3 * p, nc, sf, dsf);
        double d[3][3], Fn[3][3];
        update_def_grad(c, p, nc, ne, 1.0, dsf, d, Fn);
        for (int a = 0; a < 3; a++)
            for (int j = 0; j < 3; j++) c->F[9 * p + 3 * a + j] = Fn[a][j];
        update_stress(c, p, c->stress + 6 * p, Fn, d, 1);
        if (c->iprop[c->matid[p]] != -1) {
            for (int i = 0; i < ne; i++)
                for (int k = 0; k < 3; k++) {
                    disp[3 * p + k] += sf[i] * c->ndispl[k * N + nc[i]];
                    c->accel[3 * p + k] += sf[i] * c->naccel[k * N + nc[i]];
                    if (!flip) c->vel[3 * p + k] += sf[i] * c->nvel[k * N + nc[i]];
                }
        }
    }
    double *delta = zalloc(sizeof(double) * 3 * np);
    shifting(c, delta);
    for (size_t p = 0; p < np; p++)
        for (int k = 0; k < 3; k++) {
            if (flip) c->vel[3 * p + k] += c->dt * ((1.0 - c->gamma_nb) * accel_old[3 * p + k] + c->gamma_nb * c->accel[3 * p + k]);
            c->coord[3 * p + k] += disp[3 * p + k];
            if (c->shifting) c->coord[3 * p + k] += delta[3 * p + k];
        }
    free(nvel_k); free(naccel_k); free(accel_old); free(disp); free(delta);
}

/* SolidMaterialPoint::SolveSolid, solve_solid_implicit.cpp:65-103; returns Krylov iterations */
static int solve_solid(mo_ctx *c, double eps, int *newton) {
    size_t n3 = 3 * (size_t)c->nodec;
    int iter_max = c->nr_flag ? 1000 : 0;
    double *stress_k = malloc(sizeof(double) * 6 * (size_t)c->num);
    memcpy(stress_k, c->stress, sizeof(double) * 6 * (size_t)c->num);
    double *nvel_k = zalloc(sizeof(double) * n3), *naccel_k = zalloc(sizeof(double) * n3);
    memset(c->ndispl, 0, sizeof(double) * n3);
    memset(c->x_lhs, 0, sizeof(double) * n3);
    double r0r = 0.0;
    int ktot = 0, it;
    for (it = 0; it <= iter_max; it++) {
        bc_set_dt(c, c->ndispl);
        predict(c, nvel_k, naccel_k);
        assemble(c, naccel_k, stress_k);
        int k = gpbicgsafe(c, eps, 10000);
        ktot += k < 0 ? 10000 : k;
        for (size_t n = 0; n < n3; n++) c->ndispl[n] += c->x_lhs[n];
        if (c->nr_flag) {
            double rkr, ra;
            nr_residuals(c, &rkr, &ra);
            if (it == 0) r0r = rkr;
            double rref = (r0r > 1.0e-30) ? rkr / r0r : 0.0;
            if (rref < 1.0e-6 || r0r < 1.0e-6 || ra < 1.0e-8) break;
        }
    }
    if (newton) *newton = (it > iter_max ? iter_max : it) + 1;
    free(stress_k); free(nvel_k); free(naccel_k);
    return ktot;
}

int mo_implicit_steps(mo_ctx *c, int nsteps, double facl, double eps, int *krylov_total, int *newton_total) {
    c->facl = facl;
    int kt = 0, nt = 0;
    for (int s = 0; s < nsteps; s++) {
        linklist(c);
        p2g_implicit(c);
        int nw = 0;
        kt += solve_solid(c, eps, &nw);
        nt += nw;
        g2p_implicit(c);
    }
    if (krylov_total) *krylov_total = kt;
    if (newton_total) *newton_total = nt;
    return 0;
}

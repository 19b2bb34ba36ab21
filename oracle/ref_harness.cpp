/*
 * ORACLE (test infrastructure only) -- drives the reference's own compiled
 * translation units (module/*.cpp of HPC-MPM-Code, built unchanged by
 * oracle/build_ref.sh against the single-rank stubs in oracle/ref_stubs/).
 *
 * Only tests/golden/make_golden.py and the CPU-baseline leg of bench.py may
 * load the resulting oracle/_ref/libmpmref.so.  The product never does.
 *
 * What is reference code and what is restated here:
 *   - Grid set-up, MakSf, the particle container, StandardVarP2G, VelP2G,
 *     ComputeInternalForce/ComputeExternalForce, PIC/FLIP VarG2P,
 *     UpdateConstitutiveModel, DeltaCorrectionParticleShifting, DetMat3,
 *     BoundaryCondition::BCSet*, and the whole implicit solid
 *     (implicitmpm::SolidMaterialPoint, CrsMat, GPBiCGSafe) are the
 *     reference's compiled code, called as-is.
 *   - The explicit solid driver functions in module/solid/explicit/ and
 *     work/src_solid/ do not compile (they include a missing header and use
 *     undeclared globals), so ExplicitSolid below restates
 *       Particle2NodeS          module/solid/explicit/var_trans_solid_explicit.cpp:20-99
 *       SolveSolid              module/solid/explicit/solve_solid_explicit.cpp:8-31
 *       Node2ParticleS + MUSL   module/solid/explicit/var_trans_solid_explicit.cpp:101-148,187-311
 *       update_point_coord_and_stress  ...var_trans_solid_explicit.cpp:150-185
 *     on top of the compiled primitives, replacing the dead names
 *     (sp -> this object, usbc/vsbc/wsbc -> ubc/vbc/wbc, the
 *     vector-of-vector delta_def_grad -> one 3x3 per particle).
 *   - The grid globals are set the way datain_para + InputParaGriddata set
 *     them for one rank (work/src_fsi/datain_para.cpp:90-110,
 *     module/data_io.cpp:31-125 with isb == 0).
 */
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <vector>

#include "bc.h"
#include "cal_mat.h"
#include "data_io.h"
#include "dataset.h"
#include "material_point.h"
#include "mesh.h"
#include "mpi_data.h"
#include "shape_function.h"
#include "solid/implicit/implicit_mpm_solid.h"
#include "fluid/MPM/stabilized_mpm.h"
#include "solid/solid_material_point.h"

namespace {

// ---------------------------------------------------------------------------
// Explicit solid: restated driver functions on the compiled primitives.
// ---------------------------------------------------------------------------
class ExplicitSolid : public SolidMaterialPointBase {
  public:
    // Particle2NodeS, var_trans_solid_explicit.cpp:20-99
    void Particle2Node() override {
        int nenode;
        std::vector<int> ncm;
        std::vector<double> sf;
        std::vector<std::array<double, 3>> dsf;
        VectorAssign(nodec, this->nmass);
        VectorAssign(nodec, this->nvof);
        VectorAssign(nodec * 3, this->nmome);
        VectorAssign(nodec * 3, this->nforce);
        for (int m = 0; m < nelem; m++) {
            int pid = this->idepf[m];
            while (pid != -1) {
                std::array<double, 3> xyp = this->coord[pid];
                std::array<double, 6> sts = this->stress[pid];
                MakSf(m, xyp, idimc, xynodec, ncm, nenode, sf, dsf);
                for (int ni = 0; ni < nenode; ni++) {
                    int nid = ncm[ni];
                    double sfi = sf[ni];
                    this->StandardVarP2G(pid, nid, sfi, this->mass, this->nmass);
                    this->StandardVarP2G(pid, nid, sfi, this->vol, this->nvof);
                    MomentumP2G(pid, nid, sfi);
                    std::array<double, 3> fi = this->ComputeInternalForce(ni, pid, dsf, sts);
                    std::array<double, 3> fe = this->ComputeExternalForce(pid, sfi);
                    this->nforce[nid + nuc] += fi[0] + fe[0];
                    this->nforce[nid + nvc] += fi[1] + fe[1];
                    this->nforce[nid + nwc] += fi[2] + fe[2];
                }
                pid = this->idp2p[pid];
            }
        }
        NodeVarComm(this->nmass, 0);
        NodeVarComm(this->nvof, 0);
        NodeVarComm(this->nmome, {nuc, nvc, nwc});
        NodeVarComm(this->nforce, {nuc, nvc, nwc});
        VectorAssign(nodec * 3, this->nvel);
        for (int n = 0; n < nodec; n++) {
            if (this->nmass[n] > mtol) {
                this->nvel[n + nuc] = this->nmome[n + nuc] / this->nmass[n];
                this->nvel[n + nvc] = this->nmome[n + nvc] / this->nmass[n];
                this->nvel[n + nwc] = this->nmome[n + nwc] / this->nmass[n];
            }
            if (this->nvof[n] < mtol) this->nvof[n] = 0.0e0;
        }
        SetVelBC();
    }

    // SolveSolid, solve_solid_explicit.cpp:8-31
    void SolveSolid() override {
        VectorAssign(nodec * 3, this->naccel);
        for (int n = 0; n < nodec; n++) {
            if (this->nmass[n] > mtol) {
                this->naccel[n + nuc] = this->nforce[n + nuc] / this->nmass[n];
                this->naccel[n + nvc] = this->nforce[n + nvc] / this->nmass[n];
                this->naccel[n + nwc] = this->nforce[n + nwc] / this->nmass[n];
            }
        }
        this->ubc.BCSetZero(nuc, this->naccel);
        this->vbc.BCSetZero(nvc, this->naccel);
        this->wbc.BCSetZero(nwc, this->naccel);
        this->rigid_bc.BCSetZero(nuc, this->naccel);
        this->rigid_bc.BCSetZero(nvc, this->naccel);
        this->rigid_bc.BCSetZero(nwc, this->naccel);
    }

    // MaterialPoint::VelP2G (module/map_and_interpolate.cpp:12-23).  For TPIC
    // and APIC it is restated here: TPIC::VarP2G / APIC::VarP2G
    // (module/map_and_interpolate.h:62-77,104-130) read the node coordinate
    // as xyc[j][nid], past the end of xyc (a vector of nodec 3-arrays); the
    // restatement reads xyc[nid][j] and is otherwise the same arithmetic.
    void MomentumP2G(int pid, int nid, double sfi) {
        if (this->solswitch == MapScheme::PIC || this->solswitch == MapScheme::FLIP) {
            this->VelP2G(pid, nid, sfi);
            return;
        }
        std::array<std::array<double, 3>, 3> A{};
        if (this->solswitch == MapScheme::TPIC) {
            A = this->tpic.vel_grad[pid];
        } else {
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++)
                    for (int k = 0; k < 3; k++) A[i][j] += this->apic.vel_Bmat[pid][i][k] * this->apic.inv_Dmat[pid][k][j];
        }
        std::array<double, 3> t{};
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) t[i] += A[i][j] * (xyc[nid][j] - this->coord[pid][j]);
        this->nmome[nid + nuc] += sfi * this->mass[pid] * (this->vel[pid][0] + t[0]);
        this->nmome[nid + nvc] += sfi * this->mass[pid] * (this->vel[pid][1] + t[1]);
        this->nmome[nid + nwc] += sfi * this->mass[pid] * (this->vel[pid][2] + t[2]);
    }

    // Node2ParticleS, var_trans_solid_explicit.cpp:187-311 (PIC / FLIP / TPIC / APIC, no F-bar)
    void Node2Particle() override {
        int nenode;
        std::vector<int> ncm;
        std::vector<double> sf;
        std::vector<std::array<double, 3>> dsf;
        const bool flip = (this->solswitch == MapScheme::FLIP);
        if (!flip) {
            for (int n = 0; n < nodec; n++) {
                this->nvel[n + nuc] += dt * this->naccel[n + nuc];
                this->nvel[n + nvc] += dt * this->naccel[n + nvc];
                this->nvel[n + nwc] += dt * this->naccel[n + nwc];
            }
            VectorAssign(this->num, this->vel);
        }
        const bool tpic = (this->solswitch == MapScheme::TPIC), apic = (this->solswitch == MapScheme::APIC);
        if (tpic) VectorAssign(this->num, this->tpic.vel_grad);
        if (apic) {
            VectorAssign(this->num, this->apic.vel_Bmat);
            VectorAssign(this->num, this->apic.inv_Dmat);
        }
        for (int m = 0; m < nelem; m++) {
            int pid = this->idepf[m];
            while (pid != -1) {
                std::array<double, 3> xyp = this->coord[pid];
                MakSf(m, xyp, idimc, xynodec, ncm, nenode, sf, dsf);
                std::array<std::array<double, 3>, 3> ADp{};
                for (int ni = 0; ni < nenode; ni++) {
                    if (!flip)
                        this->pic.VarG2P(pid, ncm[ni], sf[ni], this->vel, this->nvel);
                    else
                        this->flip.VarG2P(pid, ncm[ni], sf[ni], this->vel, this->naccel);
                    if (tpic) this->tpic.VarGradG2P(pid, ncm[ni], ni, dsf, this->tpic.vel_grad, this->nvel);
                    if (apic) {
                        this->apic.VarBmatG2P(pid, ncm[ni], sf[ni], this->apic.vel_Bmat, this->nvel, this->coord);
                        this->apic.DmatG2P(pid, ncm[ni], sf[ni], this->coord, ADp);
                    }
                }
                if (apic) this->apic.InvDmatG2P(pid, ADp);
                pid = this->idp2p[pid];
            }
        }

        MUSL();

        std::vector<std::array<std::array<double, 3>, 3>> ddg(this->num);
        for (int m = 0; m < nelem; m++) {
            int pid = this->idepf[m];
            while (pid != -1) {
                std::array<double, 3> xyp = this->coord[pid];
                MakSf(m, xyp, idimc, xynodec, ncm, nenode, sf, dsf);
                std::array<std::array<double, 3>, 3> d{};
                for (int ni = 0; ni < nenode; ni++) {
                    int nid = ncm[ni];
                    for (int j = 0; j < 3; j++) {
                        d[0][j] += dsf[ni][j] * this->nvel[nid + nuc] * dt;
                        d[1][j] += dsf[ni][j] * this->nvel[nid + nvc] * dt;
                        d[2][j] += dsf[ni][j] * this->nvel[nid + nwc] * dt;
                    }
                }
                for (int i = 0; i < 3; i++) d[i][i] += 1.0e0;
                std::array<std::array<double, 3>, 3> F{};
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++)
                        for (int k = 0; k < 3; k++) F[i][j] += d[i][k] * this->def_grad[pid][k][j];
                this->def_grad[pid] = F;
                this->det_def_grad[pid] = DetMat3(F);
                ddg[pid] = d;
                pid = this->idp2p[pid];
            }
        }

        if (this->Fbar_flag) DefGradBar(ddg);

        // update_point_coord_and_stress, var_trans_solid_explicit.cpp:150-185
        std::vector<std::array<double, 3>> delta_corr = this->DeltaCorrectionParticleShifting();
        for (int m = 0; m < nelem; m++) {
            int pid = this->idepf[m];
            while (pid != -1) {
                std::array<double, 3> xyp = this->coord[pid];
                MakSf(m, xyp, idimc, xynodec, ncm, nenode, sf, dsf);
                for (int ni = 0; ni < nenode; ni++) this->flip.VarG2P(pid, ncm[ni], sf[ni], this->coord, this->nvel);
                if (shifting_)
                    for (int i = 0; i < 3; i++) this->coord[pid][i] += delta_corr[pid][i];
                this->vol[pid] = this->det_def_grad[pid] * this->vol0[pid];
                if (this->Fbar_flag)   // var_trans_solid_explicit.cpp:298-304
                    this->UpdateConstitutiveModel(pid, this->stress, this->det_def_grad_bar, this->def_grad_bar, ddg);
                else
                    this->UpdateConstitutiveModel(pid, this->stress, this->det_def_grad, this->def_grad, ddg);
                pid = this->idp2p[pid];
            }
        }
    }

    // cal_def_grad_bar (module/solid/explicit/fbar_projection.cpp:18-93) restated
    // on the members: that file does not compile here (it reads a global `sp`
    // and includes the implicit solver's header).
    void DefGradBar(std::vector<std::array<std::array<double, 3>, 3>> &ddg) {
        int nenode;
        std::vector<int> ncm;
        std::vector<double> sf;
        std::vector<std::array<double, 3>> dsf;
        std::vector<double> det_ddg(this->num), nJbar(nodec, 0.0e0);
        for (int p = 0; p < this->num; p++) det_ddg[p] = DetMat3(ddg[p]);
        for (int m = 0; m < nelem; m++) {
            int pid = this->idepf[m];
            while (pid != -1) {
                std::array<double, 3> xyp = this->coord[pid];
                MakSf(m, xyp, idimc, xynodec, ncm, nenode, sf, dsf);
                for (int ni = 0; ni < nenode; ni++)
                    nJbar[ncm[ni]] += sf[ni] * (this->det_def_grad_bar[pid] * det_ddg[pid]) * this->vol[pid];
                pid = this->idp2p[pid];
            }
        }
        for (int n = 0; n < nodec; n++) nJbar[n] = (this->nvof[n] > mtol) ? nJbar[n] / this->nvof[n] : 0.0e0;
        for (int m = 0; m < nelem; m++) {
            int pid = this->idepf[m];
            while (pid != -1) {
                std::array<double, 3> xyp = this->coord[pid];
                MakSf(m, xyp, idimc, xynodec, ncm, nenode, sf, dsf);
                double Jbar = 0.0e0;
                for (int ni = 0; ni < nenode; ni++) Jbar += sf[ni] * nJbar[ncm[ni]];
                double J = this->det_def_grad_bar[pid] * det_ddg[pid];
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++) ddg[pid][i][j] *= cbrt((Jbar / J));
                std::array<std::array<double, 3>, 3> Fb{};
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++)
                        for (int k = 0; k < 3; k++) Fb[i][j] += ddg[pid][i][k] * this->def_grad_bar[pid][k][j];
                this->def_grad_bar[pid] = Fb;
                this->det_def_grad_bar[pid] = Jbar;
                pid = this->idp2p[pid];
            }
        }
    }

    // MUSL, var_trans_solid_explicit.cpp:101-148
    void MUSL() {
        int nenode;
        std::vector<int> ncm;
        std::vector<double> sf;
        std::vector<std::array<double, 3>> dsf;
        VectorAssign(nodec * 3, this->nmome);
        for (int m = 0; m < nelem; m++) {
            int pid = this->idepf[m];
            while (pid != -1) {
                std::array<double, 3> xyp = this->coord[pid];
                MakSf(m, xyp, idimc, xynodec, ncm, nenode, sf, dsf);
                for (int ni = 0; ni < nenode; ni++) MomentumP2G(pid, ncm[ni], sf[ni]);
                pid = this->idp2p[pid];
            }
        }
        NodeVarComm(this->nmome, {nuc, nvc, nwc});
        VectorAssign(nodec * 3, this->nvel);
        for (int n = 0; n < nodec; n++) {
            if (this->nmass[n] > mtol) {
                this->nvel[n + nuc] = this->nmome[n + nuc] / this->nmass[n];
                this->nvel[n + nvc] = this->nmome[n + nvc] / this->nmass[n];
                this->nvel[n + nwc] = this->nmome[n + nwc] / this->nmass[n];
            }
        }
        SetVelBC();
    }

    void SetVelBC() {
        this->ubc.BCSetVal(nuc, this->nvel);
        this->vbc.BCSetVal(nvc, this->nvel);
        this->wbc.BCSetVal(nwc, this->nvel);
        this->rigid_bc.BCSetVal(nuc, this->nvel);
        this->rigid_bc.BCSetVal(nvc, this->nvel);
        this->rigid_bc.BCSetVal(nwc, this->nvel);
    }

    bool shifting_ = true;
};

std::unique_ptr<ExplicitSolid> g_exp;
int g_fbar = 0;   // Fbar_flag of the next explicit solid
std::unique_ptr<implicitmpm::SolidMaterialPoint> g_imp;
std::unique_ptr<stabilizedmpm::StabilizedMPM> g_ns;
int g_last_krylov = 0;

MaterialPoint *active() {
    if (g_exp) return g_exp.get();
    if (g_imp) return g_imp.get();
    return nullptr;
}

void load_particles(SolidMaterialPointBase &sp, int num, const double *coord, const double *vel, const double *mass,
                    const double *vol0, const int *matid, int scheme) {
    sp.num = num;
    const MapScheme schemes[4] = {MapScheme::PIC, MapScheme::FLIP, MapScheme::TPIC, MapScheme::APIC};
    sp.solswitch = schemes[(scheme >= 0 && scheme < 4) ? scheme : 0];
    sp.Fbar_flag = g_fbar != 0;
    sp.InitializePointData();
    for (int p = 0; p < num; p++) {
        sp.id[p] = p;
        sp.matid[p] = matid ? matid[p] : 0;
        sp.mass[p] = mass[p];
        sp.vol0[p] = vol0[p];
        sp.vol[p] = vol0[p];  // solid_data_io.cpp:32
        for (int i = 0; i < 3; i++) {
            sp.coord[p][i] = coord[3 * p + i];
            sp.vel[p][i] = vel ? vel[3 * p + i] : 0.0;
            for (int j = 0; j < 3; j++) {
                sp.def_grad[p][i][j] = eye_mat[i][j];  // solid_data_io.cpp:28
                if (sp.Fbar_flag) sp.def_grad_bar[p][i][j] = eye_mat[i][j];
            }
        }
    }
}

}  // namespace

extern "C" {

/* Grid + material globals for one rank. mat_prop is nmat x 3 (E, nu, spare). */
int ref_setup(const int *xyelem_in, const double *xymin_in, const double *dxy_in, const int *idimc_in,
              const int *npxye_in, double dt_in, double mtol_in, const double *bb_in, int nmat_in, const int *iprop_in,
              const double *mat_prop_in) {
    g_exp.reset();
    g_ns.reset();
    g_imp.reset();
    nprocs = 1;
    myrank = 0;
    dt = dt_in;
    dti = 1.0 / dt_in;
    mtol = mtol_in;
    facl = 1.0;
    for (int i = 0; i < 3; i++) {
        xyelem[i] = xyelem_in[i];
        xyelemw[i] = xyelem_in[i];
        dxy[i] = dxy_in[i];
        xymin[i] = xymin_in[i];
        xyminw[i] = xymin_in[i];
        xymax[i] = xymin_in[i] + dxy_in[i] * xyelem_in[i];
        xymaxw[i] = xymax[i];
        idimc[i] = idimc_in[i];
        npxye[i] = npxye_in[i];
        bb[i] = bb_in[i];
        xynode[i] = xyelem[i] + 1;
        xynodew[i] = xynode[i];
        xynodec[i] = xyelem[i] + idimc[i];
        xynodecw[i] = xynodec[i];
        aelemmin[i] = 0;
        aelemmax[i] = xyelem[i] - 1;
        nxyr[i] = 1;
    }
    nelem = xyelem[0] * xyelem[1] * xyelem[2];
    node = xynode[0] * xynode[1] * xynode[2];
    nodec = xynodec[0] * xynodec[1] * xynodec[2];
    // module/data_io.cpp:48-56
    nu = 0; nv = nu + node; nw = nv + node; np = nw + node;
    nuc = 0; nvc = nuc + nodec; nwc = nvc + nodec; npc = nwc + nodec;
    // module/data_io.cpp:114-123 (isb == 0)
    isb = 0;
    naid.resize(0); nsbc.resize(0); nsubc.resize(0); nsbl.resize(0); nsubl.resize(0);
    dbc.assign(nodec * 4, 1.0);
    dbl.assign(node * 4, 1.0);
    nmat = nmat_in;
    npropmax = 3;
    iprop.assign(nmat, 0.0);
    nprop.assign(nmat, 2.0);
    mat_prop.assign(nmat, std::vector<double>(3, 0.0));
    for (int n = 0; n < nmat; n++) {
        iprop[n] = iprop_in[n];
        for (int k = 0; k < 3; k++) mat_prop[n][k] = mat_prop_in[3 * n + k];
    }
    BuildMesh();
    BuildControlPoint();
    MakNodalVol();
    return nodec;
}

int ref_explicit_init(int num, const double *coord, const double *vel, const double *mass, const double *vol0,
                      const int *matid, int scheme, int shifting) {
    g_imp.reset();
    g_exp = std::make_unique<ExplicitSolid>();
    g_exp->shifting_ = shifting != 0;
    load_particles(*g_exp, num, coord, vel, mass, vol0, matid, scheme);
    g_exp->MeshPointLinklist();
    g_exp->DetermineRigidBC();
    return 0;
}

/* which: 0 u, 1 v, 2 w (BoundaryCondition ubc/vbc/wbc) */
int ref_set_bc(int which, int n, const int *nodes, const double *vals) {
    MaterialPoint *mp = active();
    if (!mp) return -1;
    BoundaryCondition *bc = which == 0 ? &mp->ubc : which == 1 ? &mp->vbc : &mp->wbc;
    bc->ibc = n;
    bc->nbc.assign(nodes, nodes + n);
    bc->fbc.assign(vals, vals + n);
    return 0;
}

/* One explicit step = MeshPointLinklist, Particle2NodeS, SolveSolid, Node2ParticleS
 * (work/src_solid/explicit/main.cpp:39-73). */
int ref_explicit_steps(int nsteps, double facl_in) {
    if (!g_exp) return -1;
    facl = facl_in;
    for (int s = 0; s < nsteps; s++) {
        g_exp->MeshPointLinklist();
        g_exp->Particle2Node();
        g_exp->SolveSolid();
        g_exp->Node2Particle();
    }
    return 0;
}

/* P2G only (binning + Particle2NodeS + SolveSolid): the first-kernel parity point. */
int ref_explicit_p2g(double facl_in) {
    if (!g_exp) return -1;
    facl = facl_in;
    g_exp->MeshPointLinklist();
    g_exp->Particle2Node();
    g_exp->SolveSolid();
    return 0;
}

/* field: 0 nmass, 1 nvof, 2 nmome, 3 nforce, 4 nvel, 5 naccel, 6 nvol, 7 ndispl */
int ref_get_nodal(int field, double *out) {
    MaterialPoint *mp = active();
    const std::vector<double> *v = nullptr;
    switch (field) {
    case 0: v = &mp->nmass; break;
    case 1: v = &mp->nvof; break;
    case 2: v = &mp->nmome; break;
    case 3: v = &mp->nforce; break;
    case 4: v = &mp->nvel; break;
    case 5: v = &mp->naccel; break;
    case 6: v = &nvol; break;
    case 7: v = &mp->ndispl; break;
    default: return -1;
    }
    std::memcpy(out, v->data(), v->size() * sizeof(double));
    return (int)v->size();
}

// TPIC: vel_grad; APIC: vel_Bmat . inv_Dmat; 9 row-major values per particle
int ref_get_affine(double *out) {
    if (!g_exp) return -1;
    ExplicitSolid &sp = *g_exp;
    for (int p = 0; p < sp.num; p++)
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double a = 0.0;
                if (sp.solswitch == MapScheme::TPIC) {
                    a = sp.tpic.vel_grad[p][i][j];
                } else if (sp.solswitch == MapScheme::APIC) {
                    for (int k = 0; k < 3; k++) a += sp.apic.vel_Bmat[p][i][k] * sp.apic.inv_Dmat[p][k][j];
                }
                out[9 * p + 3 * i + j] = a;
            }
    return sp.num;
}

/* ---- on-disk formats, through the reference's own readers and writers ----
 * Reads a grid deck (InputParaGriddata, module/data_io.cpp:31-125, followed by
 * the u / v / w BoundaryCondition lists, BCInput, module/bc.cpp:9-28) and a
 * particle deck (SolidMaterialPointBase::InputPointData,
 * module/solid/solid_data_io.cpp:13-36) into a fresh explicit solid.
 * ints: nelem, xyelem[3], node, xynode[3], nodec, xynodec[3], nxyr[3], isb,
 * then ibc u, v, w, then num.  dbl: xymin[3], xymax[3], aelemmin[3],
 * aelemmax[3].  Particle arrays are returned by ref_io_particles. */
int ref_io_read(const char *grid_path, const char *point_path, int *ints, double *dbl) {
    g_imp.reset();
    g_exp = std::make_unique<ExplicitSolid>();
    std::ifstream gin(grid_path);
    if (!gin.is_open()) return -1;
    InputParaGriddata(gin);
    g_exp->ubc.BCInput(gin, true);
    g_exp->vbc.BCInput(gin, true);
    g_exp->wbc.BCInput(gin, true);
    std::ifstream pin(point_path);
    if (!pin.is_open()) return -2;
    g_exp->InputPointData(pin);
    int k = 0;
    ints[k++] = nelem;
    for (int i = 0; i < 3; i++) ints[k++] = xyelem[i];
    ints[k++] = node;
    for (int i = 0; i < 3; i++) ints[k++] = xynode[i];
    ints[k++] = nodec;
    for (int i = 0; i < 3; i++) ints[k++] = xynodec[i];
    for (int i = 0; i < 3; i++) ints[k++] = nxyr[i];
    ints[k++] = isb;
    ints[k++] = g_exp->ubc.ibc;
    ints[k++] = g_exp->vbc.ibc;
    ints[k++] = g_exp->wbc.ibc;
    ints[k++] = g_exp->num;
    for (int i = 0; i < 3; i++) {
        dbl[i] = xymin[i];
        dbl[3 + i] = xymax[i];
        dbl[6 + i] = aelemmin[i];
        dbl[9 + i] = aelemmax[i];
    }
    return 0;
}

/* BC lists (node, value) of the last ref_io_read, which 0 u, 1 v, 2 w */
int ref_io_bc(int which, int *nodes, double *vals) {
    BoundaryCondition &b = which == 0 ? g_exp->ubc : which == 1 ? g_exp->vbc : g_exp->wbc;
    for (int i = 0; i < b.ibc; i++) {
        nodes[i] = b.nbc[i];
        vals[i] = b.fbc[i];
    }
    return b.ibc;
}

/* id, matid, surf_point, mass, vol0 of the last ref_io_read (coord via ref_get_particles) */
int ref_io_particles(int *id, int *matid, int *surf, double *mass, double *vol0) {
    for (int p = 0; p < g_exp->num; p++) {
        id[p] = g_exp->id[p];
        matid[p] = g_exp->matid[p];
        surf[p] = g_exp->surf_point[p];
        mass[p] = g_exp->mass[p];
        vol0[p] = g_exp->vol0[p];
    }
    return g_exp->num;
}

/* SolidMaterialPointBase::RestartOutput / RestartInput (solid_data_io.cpp:61-142)
 * of the explicit solid: file = prefix + "0_re.txt" (pointfile, rank 0). */
int ref_restart_output(const char *prefix) {
    if (!g_exp) return -1;
    pointfile = prefix;
    myrank = 0;
    g_exp->RestartOutput();
    return 0;
}

int ref_restart_input(const char *prefix) {
    if (!g_exp) return -1;
    pointfile = prefix;
    myrank = 0;
    g_exp->RestartInput();
    g_exp->MeshPointLinklist();
    return g_exp->num;
}

/* Fbar_flag of the explicit solids created after this call */
int ref_set_fbar(int on) {
    g_fbar = on;
    return 0;
}

/* def_grad_bar (9 per particle) and det_def_grad_bar of an F-bar run */
int ref_get_fbar(double *Fbar, double *Jbar) {
    if (!g_exp || !g_exp->Fbar_flag) return -1;
    for (int p = 0; p < g_exp->num; p++) {
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) Fbar[9 * p + 3 * i + j] = g_exp->def_grad_bar[p][i][j];
        Jbar[p] = g_exp->det_def_grad_bar[p];
    }
    return g_exp->num;
}

int ref_get_particles(double *coord, double *vel, double *F, double *stress, double *vol) {
    MaterialPoint *mp = active();
    for (int p = 0; p < mp->num; p++) {
        for (int i = 0; i < 3; i++) {
            coord[3 * p + i] = mp->coord[p][i];
            vel[3 * p + i] = mp->vel[p][i];
            for (int j = 0; j < 3; j++) F[9 * p + 3 * i + j] = mp->def_grad[p][i][j];
        }
        for (int k = 0; k < 6; k++) stress[6 * p + k] = mp->stress[p][k];
        vol[p] = mp->vol[p];
    }
    return mp->num;
}

/* ------------------------------------------------------------------------- */
/* Implicit solid: the reference's implicitmpm::SolidMaterialPoint as-is.      */
/* ------------------------------------------------------------------------- */
int ref_implicit_init(int num, const double *coord, const double *vel, const double *mass, const double *vol0,
                      const int *matid, int scheme, int nr_flag, double spec_rad) {
    g_exp.reset();
    g_imp = std::make_unique<implicitmpm::SolidMaterialPoint>();
    auto &sp = *g_imp;
    sp.SM_.use_petsc = false;  // native GPBiCGSafe + diagonal scaling
    sp.NR_flag = nr_flag != 0;
    sp.spec_rad = spec_rad;
    load_particles(sp, num, coord, vel, mass, vol0, matid, scheme);
    sp.GeneralizedAlphaParaSet();  // work/src_fsi/datain_para.cpp:103-105
    sp.NewmarkBetaParaSet();
    sp.SM_.BuildCrsMat(9);  // work/src_fsi/main.cpp:47
    sp.MeshPointLinklist();
    sp.DetermineRigidBC();
    VectorAssign(nodec * 3, sp.ndispl);
    return sp.SM_.nmat;
}

/* Steps of work/src_fsi/main.cpp:80-88 without the fluid. */
int ref_implicit_steps(int nsteps, double facl_in) {
    if (!g_imp) return -1;
    facl = facl_in;
    for (int s = 0; s < nsteps; s++) {
        g_imp->MeshPointLinklist();
        g_imp->Particle2Node();
        g_imp->SolveSolid();
        g_imp->Node2Particle();
    }
    return 0;
}

/* Assemble the first Newton system of a step (ndispl = 0) exactly as
 * SolveSolid does before its first linear solve, and leave it in SM_:
 * amat/adiag are the diagonally scaled matrix and its D^{-1/2}. */
int ref_implicit_assemble(double facl_in) {
    if (!g_imp) return -1;
    auto &sp = *g_imp;
    facl = facl_in;
    sp.MeshPointLinklist();
    sp.Particle2Node();
    std::vector<double> nvel_k(nodec * 3), naccel_k(nodec * 3);
    std::vector<std::array<double, 6>> stress_k = sp.InitializeNRStress();
    VectorAssign(nodec * 3, sp.ndispl);
    VectorAssign(nodec * 3, sp.SM_.x_lhs);
    sp.BCNRSet();
    sp.PredictNewmarkBetaVelAndAccel(nvel_k, naccel_k);
    sp.AssembleSystem(naccel_k, nvel_k, stress_k);
    return sp.SM_.nmat;
}

/* CSR graph + block-major values of the assembled (scaled) matrix. */
int ref_implicit_get_matrix(int *matrow, int *matcolid, double *amat, double *adiag, double *b_rhs) {
    auto &M = g_imp->SM_;
    std::memcpy(matrow, M.matrow.data(), M.matrow.size() * sizeof(int));
    std::memcpy(matcolid, M.matcolid.data(), M.matcolid.size() * sizeof(int));
    std::memcpy(amat, M.amat.data(), M.amat.size() * sizeof(double));
    std::memcpy(adiag, M.adiag.data(), M.adiag.size() * sizeof(double));
    std::memcpy(b_rhs, M.b_rhs.data(), M.b_rhs.size() * sizeof(double));
    return M.nmat;
}

/* y = CrsMat::MatVecMult(x) on the assembled, scaled matrix (solver.cpp:405-433). */
int ref_implicit_matvec(const double *x, double *y) {
    auto &M = g_imp->SM_;
    std::vector<double> xx(x, x + (size_t)nodec * 3);
    M.x_lhs.assign((size_t)nodec * 3, 0.0);
    std::vector<double> yy = M.MatVecMult(xx);
    std::memcpy(y, yy.data(), yy.size() * sizeof(double));
    return 0;
}

/* GPBiCGSafe (solver.cpp:19-141) on the assembled system from x = 0;
 * returns the iteration count and leaves the physical solution in x_out. */
int ref_implicit_solve(double *x_out) {
    auto &M = g_imp->SM_;
    M.x_lhs.assign((size_t)nodec * 3, 0.0);
    int it = GPBiCGSafe(M);
    std::memcpy(x_out, M.x_lhs.data(), M.x_lhs.size() * sizeof(double));
    g_last_krylov = it;
    return it;
}

/* ------------------------------------------------------------------------- */
/* Stabilized fluid MPM: the reference's stabilizedmpm::StabilizedMPM as-is.  */
/* ------------------------------------------------------------------------- */
/* Particles (coord as num x 3, mass, vol), fluid constants and Newmark
 * coefficients; builds the 4-DOF CSR graph (work/src_fluid/MPM/main.cpp:29)
 * and the element link list.  Returns the number of CSR entries. */
int ref_ns_init(int num, const double *coord, const double *mass, const double *vol, double rho, double rmu,
                double beta_nb, double gamma_nb) {
    g_exp.reset();
    g_imp.reset();
    g_ns = std::make_unique<stabilizedmpm::StabilizedMPM>();
    auto &w = *g_ns;
    w.num = num;
    w.InitializePointData();
    for (int p = 0; p < num; p++) {
        w.id[p] = p;
        w.mass[p] = mass[p];
        w.vol[p] = vol[p];
        for (int i = 0; i < 3; i++) w.coord[p][i] = coord[3 * p + i];
    }
    w.rho = rho;
    w.rmu = rmu;
    w.beta_nb = beta_nb;
    w.gamma_nb = gamma_nb;
    w.NewmarkBetaParaSet();  // work/src_fluid/MPM/datain_para.cpp:80
    w.NS_.use_petsc = false;  // graph only: no PETSc objects behind the single-rank stubs
    w.NS_.BuildCrsMat(16);
    w.NS_.use_petsc = true;   // AssembleNSSystem then leaves the matrix unscaled
    w.MeshPointLinklist();
    return w.NS_.nmat;
}

/* One Newton system of SolveNS (solve_ns_mpm.cpp:28-62) on the given nodal
 * state (component-major nvel/naccel/ndispl of 3*nodec, npres/nmass of
 * nodec): MakNSStabCoeff, PredictNewmarkBetaVelAndAccel, AssembleNSSystem.
 * The matrix stays unscaled (use_petsc is left true, so no diagonal scaling). */
int ref_ns_assemble(const double *nvel, const double *naccel, const double *ndispl, const double *npres,
                    const double *nmass, double facl_in, double *tau1, double *tau2) {
    if (!g_ns) return -1;
    auto &w = *g_ns;
    facl = facl_in;
    w.nvel.assign(nvel, nvel + (size_t)nodec * 3);
    w.naccel.assign(naccel, naccel + (size_t)nodec * 3);
    w.ndispl.assign(ndispl, ndispl + (size_t)nodec * 3);
    w.npres.assign(npres, npres + (size_t)nodec);
    w.nmass.assign(nmass, nmass + (size_t)nodec);
    w.MakNSStabCoeff();
    std::vector<double> nvel_k(nodec * 3), naccel_k(nodec * 3);
    w.PredictNewmarkBetaVelAndAccel(nvel_k, naccel_k);
    w.AssembleNSSystem(nvel_k, naccel_k);
    std::memcpy(tau1, w.tau1.data(), (size_t)w.num * sizeof(double));
    std::memcpy(tau2, w.tau2.data(), (size_t)w.num * sizeof(double));
    return 0;
}

/* CSR graph, the 16 block-major value arrays amat[b * nmat + e]
 * (b = row_var * 4 + col_var) and b_rhs (4 * nodec). */
int ref_ns_get_matrix(int *matrow, int *matcolid, double *amat, double *b_rhs) {
    if (!g_ns) return -1;
    auto &M = g_ns->NS_;
    std::memcpy(matrow, M.matrow.data(), M.matrow.size() * sizeof(int));
    std::memcpy(matcolid, M.matcolid.data(), M.matcolid.size() * sizeof(int));
    std::memcpy(amat, M.amat.data(), M.amat.size() * sizeof(double));
    std::memcpy(b_rhs, M.b_rhs.data(), M.b_rhs.size() * sizeof(double));
    return M.nmat;
}

}  // extern "C"

namespace {

void ns_set_bcs(stabilizedmpm::StabilizedMPM &w, const int *nbc_n, const int *nbc_u, const double *fbc_u,
                const int *nbc_v, const double *fbc_v, const int *nbc_w, const double *fbc_w, const int *nbc_p,
                const double *fbc_p) {
    BoundaryCondition *bcs[4] = {&w.ubc, &w.vbc, &w.wbc, &w.pbc};
    const int *nb[4] = {nbc_u, nbc_v, nbc_w, nbc_p};
    const double *fb[4] = {fbc_u, fbc_v, fbc_w, fbc_p};
    for (int k = 0; k < 4; k++) {
        bcs[k]->ibc = nbc_n[k];
        bcs[k]->nbc.assign(nb[k], nb[k] + nbc_n[k]);
        bcs[k]->fbc.assign(fb[k], fb[k] + nbc_n[k]);
    }
}

/* The Newton loop of SolveNS on w's nodal state (nvel, naccel, nmass and the
 * BC lists already set); see ref_ns_solve.  Returns the Newton iterations. */
int ns_newton(stabilizedmpm::StabilizedMPM &w, double rtol, int max_newton, int *ktot, double *rkr_hist) {
    w.NS_.use_petsc = false;
    std::vector<double> nvel_k(nodec * 3), naccel_k(nodec * 3);
    constexpr int iter_max = 10000;
    w.MakNSStabCoeff();
    VectorAssign(nodec * 3, w.ndispl);
    VectorAssign(nodec, w.npres);
    VectorAssign(nodec * 4, w.NS_.x_lhs);
    double r0r = 0.0;
    int NR_it;
    for (NR_it = 0; NR_it <= iter_max && NR_it < max_newton; NR_it++) {
        w.BCNRSet();
        w.PredictNewmarkBetaVelAndAccel(nvel_k, naccel_k);
        w.AssembleNSSystem(nvel_k, naccel_k);
        double bb = 0.0;
        w.BCResidualSet(w.NS_.b_rhs);
        for (double v : w.NS_.b_rhs) bb += v * v;
        const double bnorm = std::sqrt(bb);
        for (int call = 0; call < 20; call++) {
            if (w.NS_.ComputeRefResidual() <= rtol * bnorm) break;
            *ktot += GPBiCGSafe(w.NS_);
        }
        w.UpdateNRIncrement();
        if (rkr_hist) rkr_hist[NR_it] = w.NS_.ComputeRefResidual();
        if (w.NS_.CheckNRConvergence(NR_it, iter_max, 0, r0r)) break;
    }
    w.NS_.use_petsc = true;
    return NR_it + 1;
}

}  // namespace

extern "C" {

/* SolveNS (solve_ns_mpm.cpp:28-62) on the given nodal state, restated as a
 * loop over the reference's own members: MakNSStabCoeff once, then per
 * Newton iteration BCNRSet, PredictNewmarkBetaVelAndAccel, AssembleNSSystem
 * (with BuildDiagonalPreconditioner: use_petsc off), the native GPBiCGSafe,
 * UpdateNRIncrement and CheckNRConvergence.  The one change is the linear
 * solve's stopping point: GPBiCGSafe stops at a relative residual of 1e-4
 * (squared 1e-8, solver.cpp:64) and is called again from where it stopped
 * until the physical residual ||b - A x|| (ComputeRefResidual) is below
 * rtol ||b||, so that the result does not depend on the Krylov method.
 * BC lists: n_c nodes and values per component u, v, w, p.  At most
 * max_newton iterations; rkr_hist (may be NULL) receives the residual of
 * each iteration's linear system after the update (as CheckNRConvergence
 * measures it).  Returns the Newton iterations; ndispl (3 nodec) and npres
 * (nodec) receive the state. */
int ref_ns_solve(const double *nvel, const double *naccel, const double *nmass, double facl_in, const int *nbc_n,
                 const int *nbc_u, const double *fbc_u, const int *nbc_v, const double *fbc_v, const int *nbc_w,
                 const double *fbc_w, const int *nbc_p, const double *fbc_p, double rtol, int max_newton,
                 double *ndispl, double *npres, int *krylov_out, double *rkr_hist) {
    if (!g_ns) return -1;
    auto &w = *g_ns;
    facl = facl_in;
    w.nvel.assign(nvel, nvel + (size_t)nodec * 3);
    w.naccel.assign(naccel, naccel + (size_t)nodec * 3);
    w.nmass.assign(nmass, nmass + (size_t)nodec);
    ns_set_bcs(w, nbc_n, nbc_u, fbc_u, nbc_v, fbc_v, nbc_w, fbc_w, nbc_p, fbc_p);
    int ktot = 0;
    const int it = ns_newton(w, rtol, max_newton, &ktot, rkr_hist);
    std::memcpy(ndispl, w.ndispl.data(), sizeof(double) * 3 * (size_t)nodec);
    std::memcpy(npres, w.npres.data(), sizeof(double) * (size_t)nodec);
    if (krylov_out) *krylov_out = ktot;
    return it;
}

/* nsteps time steps of work/src_fluid/MPM/main.cpp:45-68 on the particles
 * given to ref_ns_init: MeshPointLinklist, the reference's own
 * Particle2Node (module/fluid/MPM/var_trans_fluid.cpp:17-80), SolveNS as in
 * ref_ns_solve (ns_newton) and the reference's own Node2Particle
 * (var_trans_fluid.cpp:82-135: Newmark predictor, CommitNodalKinematics,
 * pressure / displacement / acceleration / velocity gathers,
 * DeltaCorrectionParticleShifting, CommitParticleKinematics).  vel and accel
 * are num x 3; scheme 0 PIC, 1 FLIP.  nodal1 (may be NULL) receives
 * Particle2Node's nmass, nvof, nvel (3), naccel (3) of the first step (8
 * nodec, component-major); the particle state after the last step goes to
 * coord_out, vel_out, accel_out (num x 3) and pres_out (num).  Returns the
 * Newton iterations of all steps. */
int ref_ns_run(const double *vel, const double *accel, int scheme, double facl_in, const int *nbc_n,
               const int *nbc_u, const double *fbc_u, const int *nbc_v, const double *fbc_v, const int *nbc_w,
               const double *fbc_w, const int *nbc_p, const double *fbc_p, double rtol, int nsteps,
               double *nodal1, double *coord_out, double *vel_out, double *accel_out, double *pres_out,
               int *krylov_out) {
    if (!g_ns) return -1;
    auto &w = *g_ns;
    facl = facl_in;
    w.solswitch = scheme == 1 ? MapScheme::FLIP : MapScheme::PIC;
    for (int p = 0; p < w.num; p++)
        for (int i = 0; i < 3; i++) {
            w.vel[p][i] = vel[3 * p + i];
            w.accel[p][i] = accel[3 * p + i];
        }
    ns_set_bcs(w, nbc_n, nbc_u, fbc_u, nbc_v, fbc_v, nbc_w, fbc_w, nbc_p, fbc_p);
    int ntot = 0, ktot = 0;
    for (int st = 0; st < nsteps; st++) {
        w.MeshPointLinklist();
        w.Particle2Node();
        if (st == 0 && nodal1) {
            const size_t N = (size_t)nodec;
            std::memcpy(nodal1, w.nmass.data(), sizeof(double) * N);
            std::memcpy(nodal1 + N, w.nvof.data(), sizeof(double) * N);
            std::memcpy(nodal1 + 2 * N, w.nvel.data(), sizeof(double) * 3 * N);
            std::memcpy(nodal1 + 5 * N, w.naccel.data(), sizeof(double) * 3 * N);
        }
        ntot += ns_newton(w, rtol, 100, &ktot, nullptr);
        w.Node2Particle();
    }
    for (int p = 0; p < w.num; p++) {
        for (int i = 0; i < 3; i++) {
            coord_out[3 * p + i] = w.coord[p][i];
            vel_out[3 * p + i] = w.vel[p][i];
            accel_out[3 * p + i] = w.accel[p][i];
        }
        pres_out[p] = w.pres[p];
    }
    if (krylov_out) *krylov_out = ktot;
    return ntot;
}

int ref_nodec(void) { return nodec; }
int ref_num(void) {
    MaterialPoint *mp = active();
    return mp ? mp->num : 0;
}

}  // extern "C"

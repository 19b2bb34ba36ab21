// GpuStabilizedMPM: the binding a maintainer adds to HPC-MPM-Code so that the
// stabilized fluid MPM driver (work/src_fluid/MPM/main.cpp) runs its time
// steps on the GPU through the C ABI (include/mpm_gpu.h, libmpm_gb300.so)
// without changing its calls.
//
// It derives from the reference's own stabilizedmpm::StabilizedMPM
// (module/fluid/MPM/stabilized_mpm.h:14-100), overrides the virtual
// Particle2Node and Node2Particle (module/material_point.h:161,207) and hides
// SolveNS (a non-virtual member, called on the derived object by the
// driver), so the driver loop of MeshPointLinklist / Particle2Node / SolveNS /
// Node2Particle (work/src_fluid/MPM/main.cpp:45-68) is unchanged.  It reads
// the grid globals of module/dataset.h and module/mesh.h, the fluid constants
// (rho, rmu) and Newmark coefficients (beta_nb, gamma_nb) of the object, the
// BC lists ubc / vbc / wbc / pbc and the particle vectors of MaterialPoint
// (module/material_point.h:110-121) as they are.  PIC and FLIP only.
//
// Build inside the reference tree: -I<reference>/module -I<this repository>/include,
// link -lmpm_gb300.  Compiled against the reference's headers by the
// repository's test suite (tests/test_reference_binding.py).
#pragma once

#include <vector>

#include "fluid/MPM/stabilized_mpm.h"
#include "gpu_reference_common.h"
#include "mpm_gpu.h"

class GpuStabilizedMPM : public stabilizedmpm::StabilizedMPM {
  public:
    double rtol = 1.0e-10;   // each linear system to ||b - A x|| <= rtol ||b||
    int kmax = 10000;        // GPBiCGSafe iterations per call
    mpm_ns_stats last{};     // the last SolveNS's Newton / Krylov counts

    // The constants the C ABI takes, from the object's members and the globals.
    mpm_ns_params Params() const {
        mpm_ns_params p{};
        p.rho = this->rho;
        p.rmu = this->rmu;
        p.dt = dt;
        p.beta_nb = this->beta_nb;
        p.gamma_nb = this->gamma_nb;
        for (int d = 0; d < 3; ++d) p.gravity[d] = bb[d];
        p.facl = facl;
        p.mtol = mtol;
        return p;
    }

    // After DataInput and the mesh set-up: creates the context, hands over the
    // four BC lists and uploads the particles.
    void Setup() {
        const mpm_grid_desc g = mpmgpu_ref::GridDesc();
        const mpm_ns_params p = Params();
        mpmgpu_ref::Check(mpm_ns_create(&g, &p, &ns_), "mpm_ns_create");
        const BoundaryCondition *bcs[4] = {&this->ubc, &this->vbc, &this->wbc, &this->pbc};
        for (int k = 0; k < 4; ++k)
            mpmgpu_ref::Check(mpm_ns_set_bc(ns_, k, bcs[k]->ibc, bcs[k]->nbc.data(), bcs[k]->fbc.data()),
                              "mpm_ns_set_bc");
        mpmgpu_ref::Check(mpm_ns_load_particles(ns_, this->num, &this->coord[0][0], &this->vel[0][0],
                                                &this->accel[0][0], this->mass.data(), this->vol.data()),
                          "mpm_ns_load_particles");
    }

    void Particle2Node() override {
        mpmgpu_ref::Check(mpm_ns_particle2node(ns_, static_cast<int>(this->solswitch), facl), "mpm_ns_particle2node");
    }
    void SolveNS() { mpmgpu_ref::Check(mpm_ns_solve_ns(ns_, rtol, kmax, &last), "mpm_ns_solve_ns"); }
    void Node2Particle() override { mpmgpu_ref::Check(mpm_ns_node2particle(ns_), "mpm_ns_node2particle"); }

    // Only where the driver reads particle state (output and restart steps).
    void Download() {
        mpmgpu_ref::Check(mpm_ns_download_particles(ns_, &this->coord[0][0], &this->vel[0][0], &this->accel[0][0],
                                                    this->pres.data()),
                          "mpm_ns_download_particles");
    }

    ~GpuStabilizedMPM() override {
        if (ns_) mpm_ns_destroy(ns_);
    }

  private:
    mpm_ns *ns_ = nullptr;
};

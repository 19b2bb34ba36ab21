// GpuSolidMaterialPoint: the binding a maintainer adds to HPC-MPM-Code so that
// its drivers run the explicit solid transfers on the GPU through the C ABI
// (include/mpm_gpu.h, libmpm_gb300.so) without changing their calls.
//
// It derives from the reference's own SolidMaterialPointBase
// (module/solid/solid_material_point.h:14-87) and overrides the virtual
// operator calls the drivers make -- Particle2Node and Node2Particle
// (module/material_point.h:161,207) and SolveSolid
// (module/solid/solid_material_point.h:75) -- so a driver loop of
// MeshPointLinklist / Particle2Node / SolveSolid / Node2Particle
// (work/src_solid/explicit/main.cpp:39-73) is unchanged.  It reads the grid
// and material globals of module/dataset.h and module/mesh.h and the particle
// vectors of MaterialPoint (module/material_point.h:110-121) as they are.
//
// Build inside the reference tree: -I<reference>/module -I<this repository>/include,
// link -lmpm_gb300.  Compiled against the reference's headers by the
// repository's test suite (tests/test_reference_binding.py).
#pragma once

#include <algorithm>
#include <stdexcept>
#include <string>
#include <vector>

#include "gpu_reference_common.h"
#include "mpm_gpu.h"
#include "solid/solid_material_point.h"

namespace mpmgpu_ref {

// The material table of dataset.h (iprop is a vector of doubles there,
// mat_prop holds npropmax values per material) as the C ABI takes it: the
// model number as an int and the first three properties of every material
// ({E, nu, -}, or Mooney-Rivlin's {c1, c2, bulk modulus}: all three matter),
// zero-padded when npropmax < 3.
inline void MaterialTable(std::vector<int> &ip, std::vector<double> &mp) {
    ip.assign(nmat, 0);
    mp.assign(3 * (size_t)nmat, 0.0);
    for (int k = 0; k < nmat; ++k) {
        ip[k] = static_cast<int>(iprop[k]);
        const size_t np = std::min<size_t>(3, mat_prop[k].size());
        for (size_t j = 0; j < np; ++j) mp[3 * k + j] = mat_prop[k][j];
    }
}

inline mpm_config Config(MapScheme scheme, int precision) {
    mpm_config c{};
    c.dt = dt;
    c.mtol = mtol;
    for (int d = 0; d < 3; ++d) c.gravity[d] = bb[d];
    c.scheme = static_cast<int>(scheme);   // MapScheme order: PIC, FLIP, TPIC, APIC
    c.precision = precision;
    c.shifting = 1;                        // DeltaCorrectionParticleShifting, as the reference
    c.fbar = 0;
    return c;
}

}  // namespace mpmgpu_ref

class GpuSolidMaterialPoint : public SolidMaterialPointBase {
  public:
    int precision = 32;   // 32: FP32 particle and grid arithmetic; 64: FP64 (parity mode)

    // After InputParaGriddata / datain_para and InputPointData: creates the
    // context and uploads the particles and the three BC lists.
    void Setup() {
        std::vector<int> ip;
        std::vector<double> mp;
        mpmgpu_ref::MaterialTable(ip, mp);
        const mpm_grid_desc g = mpmgpu_ref::GridDesc();
        const mpm_material_desc m{nmat, ip.data(), mp.data()};
        const mpm_config c = mpmgpu_ref::Config(solswitch, precision);
        mpmgpu_ref::Check(mpm_gpu_create(&g, &m, &c, &ctx_), "mpm_gpu_create");
        std::vector<double> F(9 * (size_t)num), s(6 * (size_t)num);
        for (int p = 0; p < num; ++p) {
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) F[9 * p + 3 * i + j] = def_grad[p][i][j];
            for (int k = 0; k < 6; ++k) s[6 * p + k] = stress[p][k];
        }
        mpmgpu_ref::Check(mpm_gpu_load_particles(ctx_, num, &coord[0][0], &vel[0][0], mass.data(), vol0.data(),
                                                 F.data(), s.data(), matid.data()),
                          "mpm_gpu_load_particles");
        const BoundaryCondition *bcs[3] = {&ubc, &vbc, &wbc};
        for (int k = 0; k < 3; ++k)
            mpmgpu_ref::Check(mpm_gpu_set_bc(ctx_, k, bcs[k]->ibc, bcs[k]->nbc.data(), bcs[k]->fbc.data()),
                              "mpm_gpu_set_bc");
    }

    void Particle2Node() override { mpmgpu_ref::Check(mpm_gpu_p2g(ctx_, facl), "mpm_gpu_p2g"); }
    void SolveSolid() override { mpmgpu_ref::Check(mpm_gpu_grid_update(ctx_), "mpm_gpu_grid_update"); }
    void Node2Particle() override { mpmgpu_ref::Check(mpm_gpu_g2p(ctx_), "mpm_gpu_g2p"); }

    // Only where the driver reads particle state (output and restart steps):
    // the device state into coord, vel, def_grad, stress and vol.
    void Download() {
        std::vector<double> F(9 * (size_t)num), s(6 * (size_t)num);
        mpmgpu_ref::Check(mpm_gpu_download_particles(ctx_, &coord[0][0], &vel[0][0], F.data(), s.data(), vol.data()),
                          "mpm_gpu_download_particles");
        for (int p = 0; p < num; ++p) {
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) def_grad[p][i][j] = F[9 * p + 3 * i + j];
            for (int k = 0; k < 6; ++k) stress[p][k] = s[6 * p + k];
        }
    }

    ~GpuSolidMaterialPoint() override {
        if (ctx_) mpm_gpu_destroy(ctx_);
    }

  private:
    mpm_ctx *ctx_ = nullptr;
};

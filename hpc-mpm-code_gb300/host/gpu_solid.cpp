// Host layer over the C ABI: see gpu_solid.h.
#include "gpu_solid.h"

#include <cstring>

namespace mpmgpu {

GpuSolidMaterialPoint::GpuSolidMaterialPoint(const GridState &g, int precision) : g_(g), precision_(precision) {}

GpuSolidMaterialPoint::~GpuSolidMaterialPoint() {
    if (ctx_) mpm_gpu_destroy(ctx_);
}

void GpuSolidMaterialPoint::InitializePointData(int n) {
    num = n;
    matid.assign(n, 0);
    mass.assign(n, 0.0);
    vol0.assign(n, 0.0);
    vol.assign(n, 0.0);
    coord.assign(n, {});
    vel.assign(n, {});
    stress.assign(n, {});
    def_grad.assign(n, {});
    for (auto &F : def_grad)
        for (int i = 0; i < 3; i++) F[i][i] = 1.0;   // solid_data_io.cpp:28
    id.resize(n);
    for (int p = 0; p < n; p++) id[p] = p;
    surf_point.assign(n, 0);
    accel.assign(n, {});
    affine.assign(n, {});
}

void GpuSolidMaterialPoint::Upload() {
    if (!ctx_) {
        mpm_grid_desc gd{};
        for (int d = 0; d < 3; d++) {
            gd.xyelem[d] = g_.xyelem[d];
            gd.xymin[d] = g_.xymin[d];
            gd.dxy[d] = g_.dxy[d];
            gd.idimc[d] = g_.idimc[d];
            gd.npxye[d] = g_.npxye[d];
        }
        std::vector<double> mp(3 * g_.mat_prop.size());
        for (size_t k = 0; k < g_.mat_prop.size(); k++)
            for (int j = 0; j < 3; j++) mp[3 * k + j] = g_.mat_prop[k][j];
        mpm_material_desc md{(int)g_.iprop.size(), g_.iprop.data(), mp.data()};
        mpm_config cfg{};
        cfg.dt = g_.dt;
        cfg.mtol = g_.mtol;
        for (int d = 0; d < 3; d++) cfg.gravity[d] = g_.bb[d];
        cfg.scheme = static_cast<int>(solswitch);   // MPM_PIC .. MPM_APIC
        cfg.precision = precision_;
        cfg.shifting = 1;
        check(mpm_gpu_create(&gd, &md, &cfg, &ctx_), "mpm_gpu_create");
    }
    check(mpm_gpu_load_particles(ctx_, num, &coord[0][0], &vel[0][0], mass.data(), vol0.data(), &def_grad[0][0][0],
                                 &stress[0][0], matid.data()),
          "mpm_gpu_load_particles");
    // a restart carries vol (vol0 otherwise) and the affine matrix (zero otherwise)
    if (from_restart_ && num > 0) {
        check(mpm_gpu_upload_particles(ctx_, nullptr, nullptr, nullptr, nullptr, vol.data()), "mpm_gpu_upload_particles");
        if (solswitch == MapScheme::TPIC || solswitch == MapScheme::APIC)
            check(mpm_gpu_upload_affine(ctx_, &affine[0][0][0]), "mpm_gpu_upload_affine");
    }
    const BoundaryCondition *bcs[3] = {&ubc, &vbc, &wbc};
    for (int k = 0; k < 3; k++)
        check(mpm_gpu_set_bc(ctx_, k, bcs[k]->ibc, bcs[k]->nbc.data(), bcs[k]->fbc.data()), "mpm_gpu_set_bc");
}

void GpuSolidMaterialPoint::Download() {
    check(mpm_gpu_download_particles(ctx_, &coord[0][0], &vel[0][0], &def_grad[0][0][0], &stress[0][0], vol.data()),
          "mpm_gpu_download_particles");
    if (solswitch == MapScheme::TPIC || solswitch == MapScheme::APIC) {
        affine.resize(num);
        check(mpm_gpu_download_affine(ctx_, &affine[0][0][0]), "mpm_gpu_download_affine");
    }
}

void GpuSolidMaterialPoint::Particle2Node() { check(mpm_gpu_p2g(ctx_, g_.facl), "mpm_gpu_p2g"); }
void GpuSolidMaterialPoint::SolveSolid() { check(mpm_gpu_grid_update(ctx_), "mpm_gpu_grid_update"); }
void GpuSolidMaterialPoint::Node2Particle() { check(mpm_gpu_g2p(ctx_), "mpm_gpu_g2p"); }
void GpuSolidMaterialPoint::Steps(int nsteps) {
    check(mpm_gpu_step_explicit(ctx_, nsteps, g_.facl), "mpm_gpu_step_explicit");
    check(mpm_gpu_sync(ctx_), "mpm_gpu_sync");
}

std::vector<double> GpuSolidMaterialPoint::Nodal(int field) const {
    const int n = (field >= 2 && field <= 5) ? 3 * g_.nodec() : g_.nodec();
    std::vector<double> out(n);
    check(mpm_gpu_download_nodal(ctx_, field, out.data()), "mpm_gpu_download_nodal");
    return out;
}

}  // namespace mpmgpu

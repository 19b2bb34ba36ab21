// Test program (test infrastructure): compiles the reference-side binding
// hpc-mpm-code_gb300/host/reference/gpu_solid_material_point.h against the
// reference's own headers, instantiates the subclass (every pure virtual of
// SolidMaterialPointBase is overridden) and prints what the binding hands to
// the C ABI for a set of module globals: the material table (a Mooney-Rivlin
// material with three properties and a Neo-Hookean one), the grid
// descriptor and the configuration.  No GPU call is made.
#include <cstdio>

#include "reference/gpu_solid_material_point.h"

int main() {
    nmat = 2;
    npropmax = 3;
    iprop = {3.0, 1.0};
    mat_prop = {{2.5e5, 6.25e4, 1.75e7}, {1.0e6, 0.3, 0.0}};
    xyelem = {12, 10, 8};
    xymin = {0.5, -0.25, 0.125};
    dxy = {1.0e-2, 2.0e-2, 4.0e-2};
    idimc = {1, 2, 1};
    npxye = {2, 3, 2};
    dt = 1.0e-5;
    mtol = 1.0e-12;
    bb = {0.0, -1.0, -9.81};

    std::vector<int> ip;
    std::vector<double> mp;
    mpmgpu_ref::MaterialTable(ip, mp);
    const mpm_grid_desc g = mpmgpu_ref::GridDesc();
    const mpm_config c = mpmgpu_ref::Config(MapScheme::APIC, 32);
    GpuSolidMaterialPoint sp;   // concrete: SolveSolid, Particle2Node, Node2Particle overridden
    sp.solswitch = MapScheme::FLIP;

    std::printf("nmat %zu\n", ip.size());
    for (size_t k = 0; k < ip.size(); ++k)
        std::printf("mat %zu %d %.17g %.17g %.17g\n", k, ip[k], mp[3 * k], mp[3 * k + 1], mp[3 * k + 2]);
    std::printf("grid");
    for (int d = 0; d < 3; ++d)
        std::printf(" %d %.17g %.17g %d %d", g.xyelem[d], g.xymin[d], g.dxy[d], g.idimc[d], g.npxye[d]);
    std::printf("\nconfig %.17g %.17g %.17g %.17g %.17g %d %d %d\n", c.dt, c.mtol, c.gravity[0], c.gravity[1],
                c.gravity[2], c.scheme, c.precision, c.shifting);
    std::printf("scheme %d\n", static_cast<int>(sp.solswitch));
    return 0;
}

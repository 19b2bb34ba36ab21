// Test program (test infrastructure): compiles the reference-side binding
// hpc-mpm-code_gb300/host/reference/gpu_stabilized_mpm.h against the
// reference's own headers, instantiates the subclass of StabilizedMPM and
// prints what it hands to the C ABI for a set of module globals and members:
// the grid descriptor and the fluid constants.  No GPU call is made.
#include <cstdio>

#include "reference/gpu_stabilized_mpm.h"

int main() {
    xyelem = {6, 5, 4};
    xymin = {0.0, 0.5, -1.0};
    dxy = {1.0e-2, 2.0e-2, 1.0e-2};
    idimc = {1, 1, 1};
    npxye = {2, 2, 2};
    dt = 2.0e-3;
    mtol = 1.0e-12;
    facl = 0.75;
    bb = {0.0, 0.0, -9.8};

    GpuStabilizedMPM wp;   // concrete: Particle2Node and Node2Particle overridden, SolveNS hidden
    wp.rho = 1000.0;
    wp.rmu = 1.0e-3;
    wp.beta_nb = 0.25;
    wp.gamma_nb = 0.5;
    wp.solswitch = MapScheme::FLIP;
    const mpm_grid_desc g = mpmgpu_ref::GridDesc();
    const mpm_ns_params p = wp.Params();
    std::printf("grid");
    for (int d = 0; d < 3; ++d)
        std::printf(" %d %.17g %.17g %d %d", g.xyelem[d], g.xymin[d], g.dxy[d], g.idimc[d], g.npxye[d]);
    std::printf("\nparams %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n", p.rho, p.rmu, p.dt,
                p.beta_nb, p.gamma_nb, p.gravity[0], p.gravity[1], p.gravity[2], p.facl, p.mtol);
    std::printf("scheme %d\n", static_cast<int>(wp.solswitch));
    return 0;
}

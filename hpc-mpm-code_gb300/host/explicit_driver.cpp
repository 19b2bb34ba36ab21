// Explicit solid driver on the GPU path, following the time loop of the
// reference's explicit solid driver (work/src_solid/explicit/main.cpp:39-73):
// per step MeshPointLinklist, Particle2Node, SolveSolid, Node2Particle.
// The scene is the 64,000-particle elastic block (32^3 cells, dx = 1e-2 m,
// a 20^3-cell block at 2x2x2 particles per cell, gravity, fixed bottom face,
// E = 1e6 Pa, nu = 0.3, rho = 1000 kg/m^3, dt = 1e-5 s) without jitter.
//
//   explicit_driver [nsteps] [precision 32|64]
// prints the particle count, the steps and the mean particle velocity and
// position after the run.
#include <cstdio>
#include <cstdlib>

#include "gpu_solid.h"

int main(int argc, char **argv) {
    const int nsteps = argc > 1 ? std::atoi(argv[1]) : 100;
    const int precision = argc > 2 ? std::atoi(argv[2]) : 32;
    mpmgpu::GridState g;
    g.xyelem = {32, 32, 32};
    g.dxy = {1.0e-2, 1.0e-2, 1.0e-2};
    g.dt = 1.0e-5;
    g.bb = {0.0, 0.0, -9.81};
    g.iprop = {0};
    g.mat_prop = {{1.0e6, 0.3, 0.0}};
    try {
        mpmgpu::GpuSolidMaterialPoint sp(g, precision);
        const int npc = 2, lo[3] = {6, 6, 0}, hi[3] = {26, 26, 20};
        const int n = (hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2]) * npc * npc * npc;
        sp.InitializePointData(n);
        const double vp = g.dxy[0] * g.dxy[1] * g.dxy[2] / (npc * npc * npc);
        int p = 0;
        for (int k = lo[2]; k < hi[2]; k++)
            for (int j = lo[1]; j < hi[1]; j++)
                for (int i = lo[0]; i < hi[0]; i++)
                    for (int c = 0; c < npc * npc * npc; c++) {   // GaussianDistribution offsets +-dx/4
                        const double off[2] = {-0.25, 0.25};
                        sp.coord[p] = {(i + 0.5 + off[c & 1]) * g.dxy[0], (j + 0.5 + off[(c >> 1) & 1]) * g.dxy[1],
                                       (k + 0.5 + off[(c >> 2) & 1]) * g.dxy[2]};
                        sp.mass[p] = 1000.0 * vp;
                        sp.vol0[p] = vp;
                        p++;
                    }
        const int nx = g.xyelem[0] + 1, ny = g.xyelem[1] + 1;
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {   // bottom face k = 0, all components fixed
                for (mpmgpu::BoundaryCondition *bc : {&sp.ubc, &sp.vbc, &sp.wbc}) {
                    bc->nbc.push_back(i + nx * j);
                    bc->fbc.push_back(0.0);
                    bc->ibc++;
                }
            }
        sp.Upload();
        for (int s = 0; s < nsteps; s++) {
            sp.MeshPointLinklist();
            sp.Particle2Node();
            sp.SolveSolid();
            sp.Node2Particle();
        }
        sp.Download();
        double vz = 0.0, z = 0.0;
        for (int q = 0; q < n; q++) {
            vz += sp.vel[q][2];
            z += sp.coord[q][2];
        }
        std::printf("particles %d steps %d mean_vz %.17e mean_z %.17e\n", n, nsteps, vz / n, z / n);
    } catch (const mpmgpu::Error &e) {
        std::fprintf(stderr, "explicit_driver: %s\n", e.what());
        return 2;
    }
    return 0;
}

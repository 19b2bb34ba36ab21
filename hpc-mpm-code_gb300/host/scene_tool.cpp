// Reads and writes the reference's decks and restarts through the host layer
// (scene_io.h), and runs a deck on the GPU path.
//
//   scene_tool parse <grid deck> <particle deck>
//       prints what InputParaGriddata, the boundary lists and InputPointData
//       read (one "name values..." line per field); no GPU call
//   scene_tool copy-restart <PIC|FLIP|TPIC|APIC> <restart in> <restart out>
//       RestartInput then RestartOutput; no GPU call
//   scene_tool run <parameter deck> <grid deck> <particle deck or restart> <nsteps> <32|64> <out prefix>
//       the explicit time loop (work/src_solid/explicit/main.cpp:39-73) for
//       nsteps steps from a particle deck, or from a restart when the
//       parameter deck's rstflag is 1; writes the restart <out prefix>0_re.txt
//       and the raw state <out prefix>.bin (float64: x 3n, v 3n, F 9n,
//       stress 6n, vol n, affine 9n, in load order)
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>

#include "scene_io.h"

using namespace mpmgpu;

namespace {

std::ifstream open_in(const char *path) {
    std::ifstream f(path);
    if (!f.is_open()) throw Error(MPM_ERR_BAD_ARG, std::string("cannot open ") + path);
    return f;
}

void print_row(const char *name, const double *v, size_t n) {
    std::printf("%s", name);
    for (size_t i = 0; i < n; i++) std::printf(" %.17g", v[i]);
    std::printf("\n");
}

int parse(const char *grid_path, const char *point_path) {
    std::ifstream gin = open_in(grid_path), pin = open_in(point_path);
    GridDeck g = InputParaGriddata(gin);
    GridState gs;
    GpuSolidMaterialPoint sp(gs);
    for (BoundaryCondition *b : {&sp.ubc, &sp.vbc, &sp.wbc}) BCInput(gin, *b);
    sp.InputPointData(pin);
    std::printf("ints %d %d %d %d %d %d %d %d %d %d %d %d %d %d %d %d %d %d %d %d\n", g.nelem, g.xyelem[0],
                g.xyelem[1], g.xyelem[2], g.node, g.xynode[0], g.xynode[1], g.xynode[2], g.nodec, g.xynodec[0],
                g.xynodec[1], g.xynodec[2], g.nxyr[0], g.nxyr[1], g.nxyr[2], g.isb, sp.ubc.ibc, sp.vbc.ibc,
                sp.wbc.ibc, sp.num);
    double d[12];
    for (int i = 0; i < 3; i++) {
        d[i] = g.xymin[i];
        d[3 + i] = g.xymax[i];
        d[6 + i] = g.aelemmin[i];
        d[9 + i] = g.aelemmax[i];
    }
    print_row("dbl", d, 12);
    const BoundaryCondition *bcs[3] = {&sp.ubc, &sp.vbc, &sp.wbc};
    for (int k = 0; k < 3; k++) {
        std::vector<double> nodes(bcs[k]->nbc.begin(), bcs[k]->nbc.end());
        print_row(k == 0 ? "bc0_nodes" : k == 1 ? "bc1_nodes" : "bc2_nodes", nodes.data(), nodes.size());
        print_row(k == 0 ? "bc0_vals" : k == 1 ? "bc1_vals" : "bc2_vals", bcs[k]->fbc.data(), bcs[k]->fbc.size());
    }
    print_row("coord", sp.num ? &sp.coord[0][0] : nullptr, 3 * (size_t)sp.num);
    std::vector<double> id(sp.id.begin(), sp.id.end()), matid(sp.matid.begin(), sp.matid.end()),
        surf(sp.surf_point.begin(), sp.surf_point.end());
    print_row("id", id.data(), id.size());
    print_row("matid", matid.data(), matid.size());
    print_row("surf", surf.data(), surf.size());
    print_row("mass", sp.mass.data(), sp.mass.size());
    print_row("vol0", sp.vol0.data(), sp.vol0.size());
    return 0;
}

int copy_restart(const char *scheme, const char *in_path, const char *out_path) {
    GridState gs;
    GpuSolidMaterialPoint sp(gs);
    sp.solswitch = ParseMapScheme(scheme);
    std::ifstream in = open_in(in_path);
    sp.RestartInput(in);
    std::ofstream out(out_path);
    sp.RestartOutput(out);
    return out.good() ? 0 : 1;
}

int run(const char *para_path, const char *grid_path, const char *point_path, int nsteps, int precision,
        const std::string &prefix) {
    std::ifstream pin = open_in(para_path), gin = open_in(grid_path), sin = open_in(point_path);
    ParaDeck p;
    GridDeck g;
    BoundaryCondition bcs[3];
    ReadDecks(pin, gin, p, g, bcs);
    GpuSolidMaterialPoint sp(p.grid, precision);
    sp.solswitch = p.scheme;
    sp.ubc = bcs[0];
    sp.vbc = bcs[1];
    sp.wbc = bcs[2];
    if (p.rstflag == 1) sp.RestartInput(sin);
    else sp.InputPointData(sin);
    sp.Upload();
    for (int s = 0; s < nsteps; s++) {
        sp.MeshPointLinklist();
        sp.Particle2Node();
        sp.SolveSolid();
        sp.Node2Particle();
    }
    sp.Download();
    std::ofstream rout(RestartFileName(prefix, 0));
    sp.RestartOutput(rout);
    std::FILE *f = std::fopen((prefix + ".bin").c_str(), "wb");
    if (!f) throw Error(MPM_ERR_BAD_ARG, "cannot write " + prefix + ".bin");
    const size_t n = (size_t)sp.num;
    std::vector<std::array<std::array<double, 3>, 3>> aff = sp.affine;
    aff.resize(n);
    if (n) {
        std::fwrite(&sp.coord[0][0], sizeof(double), 3 * n, f);
        std::fwrite(&sp.vel[0][0], sizeof(double), 3 * n, f);
        std::fwrite(&sp.def_grad[0][0][0], sizeof(double), 9 * n, f);
        std::fwrite(&sp.stress[0][0], sizeof(double), 6 * n, f);
        std::fwrite(sp.vol.data(), sizeof(double), n, f);
        std::fwrite(&aff[0][0][0], sizeof(double), 9 * n, f);
    }
    std::fclose(f);
    std::printf("particles %d steps %d scheme %s\n", sp.num, nsteps, MapSchemeName(p.scheme));
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    try {
        if (argc == 4 && !std::strcmp(argv[1], "parse")) return parse(argv[2], argv[3]);
        if (argc == 5 && !std::strcmp(argv[1], "copy-restart")) return copy_restart(argv[2], argv[3], argv[4]);
        if (argc == 8 && !std::strcmp(argv[1], "run"))
            return run(argv[2], argv[3], argv[4], std::atoi(argv[5]), std::atoi(argv[6]), argv[7]);
    } catch (const Error &e) {
        std::fprintf(stderr, "scene_tool: %s\n", e.what());
        return 2;
    }
    std::fprintf(stderr, "usage: scene_tool parse | copy-restart | run (see scene_tool.cpp)\n");
    return 1;
}

// The reference's on-disk formats on either side of the transfer path, read
// and written by the host layer:
//   parameter deck   datain_para (work/src_solid/explicit/datain_para.cpp:28-84)
//   grid deck        InputParaGriddata (module/data_io.cpp:31-125) followed by
//                    the u / v / w boundary lists (BoundaryCondition::BCInput,
//                    module/bc.cpp:9-28)
//   particle deck    SolidMaterialPointBase::InputPointData
//                    (module/solid/solid_data_io.cpp:13-36)
//   restart          SolidMaterialPointBase::RestartInput / RestartOutput
//                    (module/solid/solid_data_io.cpp:61-142)
// All are whitespace-separated text with one record per line; whatever
// follows the values on a line is a comment (the readers skip to the end of
// the line, as the reference's infile.ignore(1000, '\n') does).  Only
// single-rank grid decks (isb == 0) are accepted: the GPU path has no halo.
#pragma once

#include <array>
#include <istream>
#include <ostream>
#include <string>

#include "gpu_solid.h"

namespace mpmgpu {

// What InputParaGriddata reads (the grid globals of mesh.h and mpi_data.h).
struct GridDeck {
    int myrank = 0, nelem = 0, node = 0, nodec = 0, isb = 0;
    std::array<int, 3> xyelem{}, xynode{}, xynodec{}, nxyr{};
    std::array<double, 3> xymin{}, xymax{}, aelemmin{}, aelemmax{};
};

// What datain_para reads besides the file names.
struct ParaDeck {
    MapScheme scheme = MapScheme::PIC;
    int rstflag = 0, nlstep = 1, ista = 0, iend = 0, iout = 1;
    double rho = 0.0;
    std::array<double, 3> xyminw{}, xymaxw{};
    GridState grid;   // dt, mtol, xyelem (xyelemw), xymin, dxy, idimc, npxye, iprop, mat_prop, bb
};

MapScheme ParseMapScheme(const std::string &s);   // module/dataset.h:21-27
const char *MapSchemeName(MapScheme s);

ParaDeck InputParameters(std::istream &in);
GridDeck InputParaGriddata(std::istream &in);
void BCInput(std::istream &in, BoundaryCondition &bc);

// Reads the parameter deck, then the grid deck with its u / v / w boundary
// lists, and checks that the two describe the same grid.
void ReadDecks(std::istream &para, std::istream &grid, ParaDeck &p, GridDeck &g, BoundaryCondition bcs[3]);

// file name of a rank's restart (solid_data_io.cpp:62)
inline std::string RestartFileName(const std::string &pointfile, int myrank) {
    return pointfile + std::to_string(myrank) + "_re.txt";
}

}  // namespace mpmgpu

// The reference's text formats: see scene_io.h.
#include "scene_io.h"

#include <cmath>
#include <iomanip>
#include <limits>

namespace mpmgpu {

namespace {

void skip_line(std::istream &in) { in.ignore(std::numeric_limits<std::streamsize>::max(), '\n'); }

void need(std::istream &in, const char *what) {
    if (!in) throw Error(MPM_ERR_BAD_ARG, std::string("reading ") + what);
}

template <typename T, size_t N>
void read3(std::istream &in, std::array<T, N> &a) {
    for (auto &v : a) in >> v;
    skip_line(in);
}

// one particle record of an array-of-arrays field (InputVector, module/data_io.h)
template <size_t N>
void read_rows(std::istream &in, int n, std::vector<std::array<double, N>> &v, const char *what) {
    v.resize(n);
    for (int p = 0; p < n; p++) {
        for (size_t k = 0; k < N; k++) in >> v[p][k];
        skip_line(in);
    }
    need(in, what);
}

void read_mats(std::istream &in, int n, std::vector<std::array<std::array<double, 3>, 3>> &v, const char *what) {
    v.resize(n);
    for (int p = 0; p < n; p++) {
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) in >> v[p][i][j];
        skip_line(in);
    }
    need(in, what);
}

// OutputVector (module/data_io.h): every value std::setw(15), scientific,
// the stream's default precision (6)
template <size_t N>
void write_rows(std::ostream &out, const std::vector<std::array<double, N>> &v) {
    for (const auto &r : v) {
        for (size_t k = 0; k < N; k++) out << std::setw(15) << r[k];
        out << "\n";
    }
}

void write_mats(std::ostream &out, const std::vector<std::array<std::array<double, 3>, 3>> &v) {
    for (const auto &m : v) {
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) out << std::setw(15) << m[i][j];
        out << "\n";
    }
}

}  // namespace

MapScheme ParseMapScheme(const std::string &s) {
    if (s == "FLIP") return MapScheme::FLIP;
    if (s == "PIC") return MapScheme::PIC;
    if (s == "TPIC") return MapScheme::TPIC;
    if (s == "APIC") return MapScheme::APIC;
    throw Error(MPM_ERR_BAD_ARG, "ParseMapScheme: unknown mapping scheme '" + s + "'");
}

const char *MapSchemeName(MapScheme s) {
    switch (s) {
    case MapScheme::PIC: return "PIC";
    case MapScheme::FLIP: return "FLIP";
    case MapScheme::TPIC: return "TPIC";
    case MapScheme::APIC: return "APIC";
    }
    return "PIC";
}

// datain_para (work/src_solid/explicit/datain_para.cpp:28-84): a comment line
// before every record.
ParaDeck InputParameters(std::istream &in) {
    ParaDeck p;
    std::string scheme;
    skip_line(in);
    in >> scheme >> p.rstflag >> p.nlstep;
    skip_line(in);
    need(in, "parameter deck: scheme, rstflag, nlstep");
    p.scheme = ParseMapScheme(scheme);
    skip_line(in);
    in >> p.ista >> p.iend >> p.iout;
    skip_line(in);
    skip_line(in);
    in >> p.grid.dt >> p.grid.mtol;
    skip_line(in);
    skip_line(in);
    read3(in, p.xyminw);
    skip_line(in);
    read3(in, p.xymaxw);
    skip_line(in);
    read3(in, p.grid.xyelem);
    skip_line(in);
    read3(in, p.grid.idimc);
    skip_line(in);
    read3(in, p.grid.npxye);
    skip_line(in);
    int nmat = 0, npropmax = 0;
    in >> p.rho >> nmat >> npropmax;
    skip_line(in);
    need(in, "parameter deck: grid and rho / nmat / npropmax");
    if (nmat <= 0 || npropmax < 0) throw Error(MPM_ERR_BAD_ARG, "parameter deck: nmat / npropmax");
    p.grid.iprop.assign(nmat, 0);
    p.grid.mat_prop.assign(nmat, {});
    for (int n = 0; n < nmat; n++) {
        int nprop = 0;
        skip_line(in);
        in >> p.grid.iprop[n] >> nprop;
        skip_line(in);
        if (nprop < 0 || nprop > 3) throw Error(MPM_ERR_UNSUPPORTED, "parameter deck: more than 3 material properties");
        for (int i = 0; i < nprop; i++) in >> p.grid.mat_prop[n][i];
        skip_line(in);
    }
    skip_line(in);
    read3(in, p.grid.bb);
    need(in, "parameter deck: materials and gravity");
    for (int i = 0; i < 3; i++) {
        if (p.grid.xyelem[i] <= 0) throw Error(MPM_ERR_BAD_ARG, "parameter deck: xyelemw");
        p.grid.xymin[i] = p.xyminw[i];
        p.grid.dxy[i] = (p.xymaxw[i] - p.xyminw[i]) / double(p.grid.xyelem[i]);   // datain_para.cpp:87
    }
    return p;
}

// InputParaGriddata (module/data_io.cpp:31-125); the overlap lists of a
// multi-rank deck (isb != 0) are refused.
GridDeck InputParaGriddata(std::istream &in) {
    GridDeck g;
    in >> g.myrank;
    skip_line(in);
    in >> g.nelem;
    read3(in, g.xyelem);
    in >> g.node;
    read3(in, g.xynode);
    in >> g.nodec;
    read3(in, g.xynodec);
    read3(in, g.nxyr);
    read3(in, g.xymin);
    read3(in, g.xymax);
    read3(in, g.aelemmin);
    read3(in, g.aelemmax);
    in >> g.isb;
    skip_line(in);
    need(in, "grid deck");
    if (g.isb != 0) throw Error(MPM_ERR_UNSUPPORTED, "grid deck of a rank with overlap neighbours (isb != 0)");
    return g;
}

// BoundaryCondition::BCInput with values (module/bc.cpp:9-28)
void BCInput(std::istream &in, BoundaryCondition &bc) {
    in >> bc.ibc;
    skip_line(in);
    need(in, "boundary list length");
    if (bc.ibc < 0) throw Error(MPM_ERR_BAD_ARG, "boundary list length");
    bc.nbc.resize(bc.ibc);
    bc.fbc.resize(bc.ibc);
    for (int i = 0; i < bc.ibc; i++) {
        in >> bc.nbc[i] >> bc.fbc[i];
        skip_line(in);
    }
    need(in, "boundary list");
}

void ReadDecks(std::istream &para, std::istream &grid, ParaDeck &p, GridDeck &g, BoundaryCondition bcs[3]) {
    p = InputParameters(para);
    g = InputParaGriddata(grid);
    for (int i = 0; i < 3; i++) {
        if (g.xyelem[i] != p.grid.xyelem[i] || g.xynodec[i] != p.grid.xyelem[i] + p.grid.idimc[i])
            throw Error(MPM_ERR_BAD_ARG, "grid deck and parameter deck describe different grids");
        if (std::fabs(g.xymin[i] - p.xyminw[i]) > 1e-12 * (1.0 + std::fabs(p.xyminw[i])))
            throw Error(MPM_ERR_BAD_ARG, "grid deck origin differs from the parameter deck's");
    }
    for (int k = 0; k < 3; k++) BCInput(grid, bcs[k]);
}

// ---------------------------------------------------------------- particles
void GpuSolidMaterialPoint::InputPointData(std::istream &in) {
    int n = 0;
    in >> n;
    skip_line(in);
    need(in, "particle count");
    if (n < 0) throw Error(MPM_ERR_BAD_ARG, "particle count");
    InitializePointData(n);
    read_rows(in, n, coord, "particle coordinates");
    for (int p = 0; p < n; p++) {
        in >> id[p] >> matid[p] >> surf_point[p] >> mass[p] >> vol0[p];
        skip_line(in);
        vol[p] = vol0[p];   // solid_data_io.cpp:32
    }
    need(in, "particle records");
    from_restart_ = false;
}

void GpuSolidMaterialPoint::RestartInput(std::istream &in) {
    int n = 0;
    in >> n;
    skip_line(in);
    need(in, "restart particle count");
    if (n < 0) throw Error(MPM_ERR_BAD_ARG, "restart particle count");
    InitializePointData(n);
    if (n > 0) {
        read_rows(in, n, coord, "restart coordinates");
        for (int p = 0; p < n; p++) {
            in >> id[p] >> matid[p] >> surf_point[p] >> mass[p] >> vol0[p] >> vol[p];
            skip_line(in);
        }
        need(in, "restart records");
        read_rows(in, n, vel, "restart velocities");
        read_rows(in, n, accel, "restart accelerations");
        read_rows(in, n, stress, "restart stresses");
        read_mats(in, n, def_grad, "restart deformation gradients");
        if (solswitch == MapScheme::TPIC) {
            std::vector<std::array<std::array<double, 3>, 3>> accel_grad;
            read_mats(in, n, affine, "restart vel_grad");
            read_mats(in, n, accel_grad, "restart accel_grad");
        } else if (solswitch == MapScheme::APIC) {
            std::vector<std::array<std::array<double, 3>, 3>> bmat, accel_bmat, dinv;
            read_mats(in, n, bmat, "restart vel_Bmat");
            read_mats(in, n, accel_bmat, "restart accel_Bmat");
            read_mats(in, n, dinv, "restart inv_Dmat");
            for (int p = 0; p < n; p++)   // the product APIC::VarP2G forms (map_and_interpolate.h:113-118)
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++) {
                        double t = 0.0;
                        for (int k = 0; k < 3; k++) t += bmat[p][i][k] * dinv[p][k][j];
                        affine[p][i][j] = t;
                    }
        }
    }
    from_restart_ = true;
}

// RestartOutput: APIC's vel_Bmat is written as the affine matrix with
// inv_Dmat the identity (their product is all the transfers use) and
// accel_Bmat / accel_grad as zero (no explicit kernel reads them).
void GpuSolidMaterialPoint::RestartOutput(std::ostream &out) const {
    const auto flags = out.flags();
    out.flags(std::ios::right | std::ios::scientific);
    out << num << "     --- Number of solid material point --- " << "\n";
    if (num != 0) {
        write_rows(out, coord);
        for (int i = 0; i < num; i++)
            out << id[i] << std::setw(15) << matid[i] << std::setw(15) << surf_point[i] << std::setw(15) << mass[i]
                << std::setw(15) << vol0[i] << std::setw(15) << vol[i] << "\n";
        write_rows(out, vel);
        write_rows(out, accel);
        write_rows(out, stress);
        write_mats(out, def_grad);
        const std::vector<std::array<std::array<double, 3>, 3>> zero(num);
        if (solswitch == MapScheme::TPIC) {
            write_mats(out, affine);
            write_mats(out, zero);
        } else if (solswitch == MapScheme::APIC) {
            std::vector<std::array<std::array<double, 3>, 3>> eye(num);
            for (auto &m : eye)
                for (int i = 0; i < 3; i++) m[i][i] = 1.0;
            write_mats(out, affine);
            write_mats(out, zero);
            write_mats(out, eye);
        }
    }
    out.flags(flags);
}

}  // namespace mpmgpu

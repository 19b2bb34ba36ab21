// C++ host layer over the C ABI (include/mpm_gpu.h) that mirrors the
// reference's solid operator surface, so a driver written against
// SolidMaterialPointBase (module/solid/solid_material_point.h) calls the GPU
// path with the same names and the same data: the particle vectors of
// MaterialPoint (module/material_point.h:186-198), the BoundaryCondition
// lists (module/bc.h:7-21) and the grid / material globals of dataset.h and
// mesh.h, gathered here in GridState.
#pragma once

#include <array>
#include <istream>
#include <ostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "mpm_gpu.h"

namespace mpmgpu {

// The module globals the transfer path reads (module/dataset.h:8-17, module/mesh.h:6-21).
struct GridState {
    std::array<int, 3> xyelem{};
    std::array<double, 3> xymin{}, dxy{};
    std::array<int, 3> idimc{{1, 1, 1}}, npxye{{2, 2, 2}};
    double dt = 0.0, mtol = 1.0e-12, facl = 1.0;
    std::array<double, 3> bb{};                 // gravity
    std::vector<int> iprop;                     // per material: -1 rigid, 0 linear elastic, 1 Neo-Hookean
    std::vector<std::array<double, 3>> mat_prop;  // E, nu, spare
    int nodec() const { return (xyelem[0] + idimc[0]) * (xyelem[1] + idimc[1]) * (xyelem[2] + idimc[2]); }
};

// BoundaryCondition (module/bc.h:7-21)
struct BoundaryCondition {
    int ibc = 0;
    std::vector<int> nbc;
    std::vector<double> fbc;
};

// MapScheme (module/dataset.h:19), in the reference's order
enum class MapScheme { PIC, FLIP, TPIC, APIC };

class Error : public std::runtime_error {
  public:
    Error(mpm_status s, const std::string &where)
        : std::runtime_error(where + ": " + mpm_gpu_status_string(s)), status(s) {}
    mpm_status status;
};

// Explicit solid on the GPU with the reference's call names.
class GpuSolidMaterialPoint {
  public:
    // particle vectors in the reference's AoS layout (MaterialPoint members)
    int num = 0;
    MapScheme solswitch = MapScheme::PIC;
    std::vector<int> matid;
    std::vector<double> mass, vol0, vol;
    std::vector<std::array<double, 3>> coord, vel;
    std::vector<std::array<double, 6>> stress;
    std::vector<std::array<std::array<double, 3>, 3>> def_grad;
    std::vector<int> id, surf_point;              // carried through the decks, not used by the transfers
    std::vector<std::array<double, 3>> accel;     // restart field; zero on the explicit path
    // TPIC: tpic.vel_grad; APIC: apic.vel_Bmat . apic.inv_Dmat (module/map_and_interpolate.h:59,105)
    std::vector<std::array<std::array<double, 3>, 3>> affine;
    BoundaryCondition ubc, vbc, wbc;

    explicit GpuSolidMaterialPoint(const GridState &g, int precision = 32);
    ~GpuSolidMaterialPoint();
    GpuSolidMaterialPoint(const GpuSolidMaterialPoint &) = delete;
    GpuSolidMaterialPoint &operator=(const GpuSolidMaterialPoint &) = delete;

    // InputPointData (module/solid/solid_data_io.cpp:13-36) then upload
    void InitializePointData(int n);
    void Upload();          // particles (with vol and the affine matrix) + boundary conditions to the device
    void Download();        // device particle state into the vectors above

    // the reference's text formats (scene_io.cpp): InputPointData
    // (module/solid/solid_data_io.cpp:13-36), RestartInput / RestartOutput (:61-142)
    void InputPointData(std::istream &in);
    void RestartInput(std::istream &in);
    void RestartOutput(std::ostream &out) const;

    void MeshPointLinklist() {}           // the GPU bins every step inside Particle2Node
    void Particle2Node();                 // Particle2NodeS
    void SolveSolid();                    // SolveSolid (explicit)
    void Node2Particle();                 // Node2ParticleS + MUSL + update_point_coord_and_stress
    void Steps(int nsteps);               // the three above, fused, nsteps times

    std::vector<double> Nodal(int field) const;   // nmass .. nvol, component-major
    mpm_ctx *context() const { return ctx_; }

  private:
    GridState g_;
    int precision_;
    bool from_restart_ = false;   // set by RestartInput: Upload also sends vol and the affine matrix
    mpm_ctx *ctx_ = nullptr;
    void check(mpm_status s, const char *where) const {
        if (s != MPM_OK) throw Error(s, where);
    }
};

}  // namespace mpmgpu

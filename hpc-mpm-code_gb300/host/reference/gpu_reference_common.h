// Helpers shared by the reference-side bindings (gpu_solid_material_point.h,
// gpu_stabilized_mpm.h): the status check and the grid descriptor of the
// module globals of module/dataset.h and module/mesh.h.
#pragma once

#include <stdexcept>
#include <string>

#include "dataset.h"
#include "mesh.h"
#include "mpm_gpu.h"

namespace mpmgpu_ref {

inline void Check(mpm_status s, const char *where) {
    if (s != MPM_OK) throw std::runtime_error(std::string(where) + ": " + mpm_gpu_status_string(s));
}

// The grid globals of mesh.h / dataset.h (set by InputParaGriddata and datain_para).
inline mpm_grid_desc GridDesc() {
    mpm_grid_desc g{};
    for (int d = 0; d < 3; ++d) {
        g.xyelem[d] = xyelem[d];
        g.xymin[d] = xymin[d];
        g.dxy[d] = dxy[d];
        g.idimc[d] = idimc[d];
        g.npxye[d] = npxye[d];
    }
    return g;
}

}  // namespace mpmgpu_ref

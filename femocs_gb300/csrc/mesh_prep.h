// Device preparation of a tetrahedral mesh (tet -> hex split, grouping, interpolation
// tables): the same PreparedMesh as prepare_mesh, built by kernels on the current device.
#pragma once

#include <cuda_runtime.h>

#include "prepared.h"

namespace fgb {

struct MeshPrepTiming {
    double kernel_ms = 0;  // device time of the preparation kernels (CUDA events)
    double total_ms = 0;   // wall time including the upload of the tets and the download of the tables
};

// Tables equal bit for bit to prepare_mesh(tm) (mesh.cpp / prepared.cpp); throws the same
// errors for degenerate tets and non-manifold faces. Meshes up to 2^21 tet vertices.
PreparedMesh prepare_mesh_device(TetMesh&& tm, cudaStream_t stream, MeshPrepTiming* timing = nullptr);

}  // namespace fgb

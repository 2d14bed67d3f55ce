// Device output stage (output.cu).
#pragma once
#include <cuda_runtime.h>

#include "../../include/mmcgb.h"
#include "engine.h"
#include "mesh.h"

namespace mmcgb {

struct DeviceOutputArgs {
    const HostMesh* host;
    const mmcgb_config* cfg;
    int maxgate;
    double energytot, energyesc;
    // raw element deposits: f64, or the two float32 halves
    const double* f64;
    const float* f32a;
    const float* f32b;
    // mesh / simulation tables on the device
    const int4* elem;
    const int* label;
    const float* evol;
    const float* nvol;      // nodal volumes after the surface fix (basisorder 1)
    const float4* media;
    double* out;            // maxgate * datalen
    size_t gridlen;         // dual-grid output (cfg->method 1): voxels per gate, else 0
};

cudaError_t device_output(const DeviceOutputArgs& args, cudaStream_t stream, double* normalizer);

// Nodal volumes with the surface correction of src/mmc_mesh.c:1344-1386
// applied when cfg.isnormalized == 1 and basisorder == 1.
std::vector<float> surface_fixed_nvol(const HostMesh& m, const mmcgb_config& cfg);

}  // namespace mmcgb

// Definition of the opaque mmcgb_mesh handle (include/mmcgb.h): the host
// copy of the prepared mesh plus its device-resident arrays.
#pragma once
#include <mutex>
#include "engine.h"
#include "mesh.h"

struct mmcgb_mesh {
    mmcgb::HostMesh host;
    int device = 0;
    mmcgb::TetRec* rec = nullptr;
    int4* elem = nullptr;
    float4* node = nullptr;
    int* label = nullptr;
    float* evol = nullptr;
    unsigned* loc_start = nullptr;  // bounding-box grid (HostMesh::grid) on the device, uploaded
    unsigned* loc_items = nullptr;  // by the first simulation whose photons are located there
    std::mutex loc_mu;
    float lo[3] = {0.f, 0.f, 0.f};  // bounding box of the nodes
    float hi[3] = {0.f, 0.f, 0.f};
};

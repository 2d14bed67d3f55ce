// Host mesh representation and preparation routines (see mesh.cpp).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/mmcgb.h"
#include "engine.h"

namespace mmcgb {

extern const int kOut[4][3];
extern const int kFaceMap[4];
extern const int kIFaceOrder[4];
extern const int kFaceList[4][3];

struct LocGrid {
    int res = 0;
    float lo[3] = {0, 0, 0};
    float inv[3] = {0, 0, 0};
    std::vector<uint32_t> start;  // CSR offsets, res^3 + 1
    std::vector<uint32_t> items;  // element ids (0-based)
};

struct HostMesh {
    int nn = 0, ne = 0, nf = 0, maxlabel = 0;
    std::vector<float> node;     // nn*3
    std::vector<int> elem;       // ne*4, 1-based, orientation-fixed
    std::vector<int> label;      // ne
    std::vector<int> facenb;     // ne*4, exterior faces numbered -1,-2,...
    std::vector<float> normals;  // ne*16: nx[4] ny[4] nz[4] d[4]
    std::vector<float> evol;     // ne
    std::vector<float> nvol;     // nn (before the surface fix)
    LocGrid grid;
};

int prepare_mesh(const mmcgb_mesh_desc& d, HostMesh& m, std::string& err);
void pack_records(const HostMesh& m, std::vector<TetRec>& rec);
void build_locator(HostMesh& m);
int locate(const HostMesh& m, const float p[3]);

// Output stage (elem->node scatter, surface nodal-volume fix, normalization);
// returns the normalization factor.  `raw` holds maxgate*ne element deposits.
double normalize_output(const HostMesh& m, const mmcgb_config& cfg, int maxgate, const double* raw,
                        double energytot, double energyesc, double* field);

}  // namespace mmcgb

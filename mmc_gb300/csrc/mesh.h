// Host mesh representation and preparation routines (see mesh.cpp).
#pragma once
#include <atomic>
#include <cstdint>
#include <mutex>
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
    int lbits = 1;               // label bits of the packed face words (label_bits(maxlabel))
    std::vector<float> node;     // nn*3
    std::vector<int> elem;       // ne*4, 1-based, orientation-fixed
    std::vector<int> label;      // ne
    std::vector<int> facenb;     // ne*4, exterior faces numbered -1,-2,...
    std::vector<float> evol;     // ne
    std::vector<float> nvol;     // nn (before the surface fix)
    // the bounding-box grid of the source locator, built on first need (ensure_locator)
    LocGrid grid;
    std::atomic<bool> grid_built{false};
    std::mutex grid_mu;
};

int prepare_mesh(const mmcgb_mesh_desc& d, HostMesh& m, std::string& err);
void pack_records(const HostMesh& m, std::vector<TetRec>& rec);
// Face normals and plane offsets of every element, ne*16 floats: nx[4] ny[4] nz[4] d[4].
void element_normals_all(const HostMesh& m, float* out);
// Builds the locator grid once (thread-safe); false when its 32-bit offsets would overflow.
bool ensure_locator(HostMesh& m);
// First element (1-based, by index) enclosing p, 0 if none: through the grid when it is built,
// else by a scan of every element on all host threads (what one query costs less than the grid).
int locate(const HostMesh& m, const float p[3]);

// The configuration checks every simulation entry makes before it allocates
// (api.cpp); MMCGB_E_* status, message in `err`.
int validate_config(const HostMesh& m, const mmcgb_config& c, std::string& err);
// Initial element of a simulation: a given e0 if it encloses srcpos, else the
// located element; 0 when no element encloses the source.
int initial_element(const HostMesh& m, const mmcgb_config& c);

// Output stage (elem->node scatter, surface nodal-volume fix, normalization);
// returns the normalization factor.  `raw` holds maxgate*ne element deposits.
double normalize_output(const HostMesh& m, const mmcgb_config& cfg, int maxgate, const double* raw,
                        double energytot, double energyesc, double* field);
// Its two halves: the elem->node scatter (a copy for element output) of `raw`
// into `field`, and the normalization of a scattered field in place (returns
// the factor; 1 when cfg.isnormalized is 0).
void scatter_output(const HostMesh& m, const mmcgb_config& cfg, int maxgate, const double* raw, double* field);
double normalize_in_place(const HostMesh& m, const mmcgb_config& cfg, int maxgate, double energytot,
                          double energyesc, double* field);
// The single scale factor of the dual-grid output.
double grid_normalizer(const mmcgb_config& cfg, double energytot);

}  // namespace mmcgb

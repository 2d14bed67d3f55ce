// Internal types shared by the host runtime (api.cpp, mesh.cpp) and the CUDA
// photon engine (engine.cu).  Not part of the public C ABI (include/mmcgb.h).
#pragma once
#include <cstdint>
#include <string>
#include <cuda_runtime.h>

namespace mmcgb {

// Output/physics enums follow the reference numbering (src/mmc_utils.h:92-110).
enum OutputType { OT_FLUX = 0, OT_FLUENCE = 1, OT_ENERGY = 2, OT_JACOBIAN = 3, OT_WL = 4, OT_WP = 5,
                  // replay only, no reference counterpart: replay weight deposited once per
                  // scattering event in the element where it happens (the scatter-count term of
                  // the mus derivative of a detected photon's likelihood)
                  OT_WN = 16 };
enum Boundary { BC_NOREFLECT = 0, BC_REFLECT = 1, BC_ABSORBEXT = 2, BC_MIRROR = 3 };

constexpr int kMaxMedia = 64;        // media rows (incl. background) staged in shared memory
constexpr int kMaxSimsShared = 256;  // simulations whose media tables fit in one block's shared memory
constexpr int kMaxLabel = 63;        // medium labels a mesh may use (kMaxMedia - 1)
// A packed face word holds the neighbour's medium label in its low lbits bits and the
// neighbour id, signed, in the 32 - lbits bits above, lbits being the fewest bits (1..6) that
// hold the mesh's largest label: labels 0-1 leave 31 bits for signed element ids
// (1,073,741,823 elements), labels up to 63 leave 26 (33,554,431).
inline int label_bits(int maxlabel) {
    int b = 1;
    while (b < 6 && (1 << b) <= maxlabel) b++;
    return b;
}
inline int max_elem(int lbits) { return (int)((1u << (31 - lbits)) - 1u); }
// Fluence cells (gates x elements or voxels) one simulation may hold: deposit indices are
// 32-bit and 0x7FFFFFFF marks "no pending deposit", so every index stays below it.
constexpr unsigned kMaxFluenceCells = 0x7FFFFFFFu;
// Slots of per-pattern energy tallies (photon sharing): a block adds into slot blockIdx % 64.
constexpr int kEnergySlots = 64;
// Replicated accumulators of the cells next to a point source.  Every photon deposits into the
// few elements around its launch point first, so their reductions queue on the L2 slices that
// hold those cells.  The gate-0 deposits of a photon's first kHotSteps ray-tet tests go instead
// to one of kHotReps copies of the gate-0 plane, chosen by block; the copies are added into the
// fluence after each launch.
constexpr int kHotReps = 4;
constexpr unsigned kHotSteps = 16;

// One tetrahedron as the step kernel reads it: 80 bytes, 16-byte aligned.
//   nx/ny/nz/nd : outward unit normals and plane offsets of the 4 faces
//                 (face k of the reference normal table, src/mmc_mesh.c:1572-1601)
//   nb          : for each face in neighbour order (src/mmc_highorder.cpp:50),
//                 word = neighbour element << lbits | its medium label (element
//                 1-based, signed: <=0 is an exterior face numbered -1,-2,...,
//                 whose label is 0).
struct __align__(16) TetRec {
    float4 nx, ny, nz, nd;
    int4 nb;
};
static_assert(sizeof(TetRec) == 80, "TetRec must be 80 bytes");

// Per-simulation parameter block.  Plain launches pass it by value as a
// __grid_constant__ kernel parameter; batched launches read an array of them
// from global memory.
struct SimDev {
    // mesh
    const TetRec* rec;
    const int4* elem;      // 1-based node ids (after orientation fix)
    const float4* node;    // xyz + pad
    const int* label;      // medium label per element
    int ne;
    int lbits;             // label bits of the packed face words (label_bits of the mesh)
    int lmask;             // (1 << lbits) - 1
    int e0;                // initial element (1-based)
    int nmedia;
    int detnum;
    const float4* media;   // nmedia rows: mua mus g n
    const float* nodemua;  // per-node mua (nn), or null: an element's mua is the mean of its nodes'
    const float* nodemusp; // per-node mus (nn), read only with nodemua
    const float4* det;     // detnum rows: x y z r
    // photons
    unsigned long long nphoton;
    unsigned long long photon_offset;
    unsigned long long seed;
    unsigned long long step_budget;
    // source (the reference's TSrcType codes, src/mmc_utils.h:101-105)
    float srcpos[3];
    float srcdir[3];
    int srctype;
    float4 srcp1, srcp2;   // srcparam1, srcparam2
    float focus;
    const float* srcpattern;  // pixel-major: the srcnum patterns' values of a pixel adjacent
    int srcnum;               // patterns sharing each photon (pattern sources), 1 otherwise
    double* energy_src;       // srcnum > 1: 64 slots of [launched, escaped] weight per pattern
    // bounding-box grid of the mesh (per-photon source element search):
    // cell (x,y,z) lists the elements whose bounding boxes overlap it
    const unsigned* loc_start;  // res^3 + 1 offsets
    const unsigned* loc_items;  // 0-based element ids
    int loc_res;
    float loc_lo[3], loc_inv[3];
    // time gates
    float tstart, tend, Rtstep;
    int maxgate;
    int roulette_on;       // minenergy > 0 and (tend-tstart)*Rtstep <= 1, as the reference tests it
    float minenergy, roulettesize, nout;
    // switches
    int isreflect, isspecular, voidtime;
    int issavedet, issaveexit, ismomentum, issaveseed;
    int outputtype;
    int replay;            // replay mode (seeds from a previous run)
    int accum_f64;
    int fast_math;         // 1: hardware-approximate math, 0: bit-exact with the CPU oracle
    int reclen;            // detected-photon columns excluding the detector id
    int nmed_ppath;        // M = nmedia-1
    // replay inputs
    const unsigned long long* replayseed;  // 2 words per photon
    const float* replayweight;
    const float* replaytime;
    // outputs
    float* f32a;           // ne*maxgate (accum_f64 == 0)
    float* f32b;           // overflow half
    double* f64;           // ne*maxgate (accum_f64 == 1)
    float* detp;           // maxdet * (reclen+1)
    unsigned long long* seeds;  // maxdet * 2
    unsigned int* detcount;
    unsigned int maxdet;
    double* energy;        // [0] launched weight, [1] escaped weight
    unsigned long long* counters;  // [0] ray-tet tests, [1] aborted photons, [2] photons launched outside
    int ncounters;         // entries of `counters` (2 for callers that give two)
    // DMMC grid output (method 1): voxel (x,y,z) of gate g at g*framelen + (z*dim.y + y)*dim.x + x
    int grid;
    float gstep_inv;       // 1 / voxel edge
    float gmin[3];         // grid origin (node minimum - EPS)
    unsigned gdim[3];
    unsigned framelen;     // fluence entries per gate: ne, or dim.x*dim.y*dim.z
    float* traj;           // trajectory records (6 words) at launch, scattering and photon end
    unsigned* trajcount;
    unsigned maxtraj;
    double* dref;          // issaveref: exiting weight per exterior face and gate, [gate][face]
    int nf;                // exterior faces
    // optional per-photon trace (parity tests)
    float* photon_weight;
    unsigned int* photon_steps;
    int* photon_det;
    // replicated near-source accumulators (kHot*), or hot_steps = 0 when off
    double* hot;              // kHotReps copies of the gate-0 plane, copy r at hot + r * ne
    unsigned hot_steps;
};

struct LaunchShape {
    int blocks;
    int threads;
};

// Gate-phased tracing.  Launch g of a phased run traces every live photon
// while its time lies in gate g; a photon whose time reaches gate g+1 is parked
// as a PState record (plus its partial-path columns and saved seed) in the
// queue that launch g+1 resumes from.  Only one or two gate planes of the
// fluence then receive deposits at a time.  A parked photon keeps exactly
// the state the step loop carries from one trip to the next, so its sequence
// of operations (and random numbers) is the same as in one unbroken launch.
struct __align__(16) PState {
    float4 pos;   // px py pz ptime
    float4 dir;   // vx vy vz weight
    float4 len;   // slen slen0 oldw, oldidx bits
    int4 elem;    // eid label mode fixcount
    uint4 meta;   // steps, pid (low, high), unused
    uint4 rng;    // xorshift128+ state t0 (low, high), t1 (low, high)
};
static_assert(sizeof(PState) == 96, "PState must be 96 bytes");

struct PhaseQueue {
    PState* rec;                // capacity records
    float* ppath;               // reclen floats per record (saved detections only)
    unsigned long long* seed0;  // 2 words per record (saved seeds only)
    unsigned long long* count;  // records written
};

// Parked photons are resumed in spatial order: each is keyed by the cell of a
// 16x16x16 grid over the mesh's bounding box that holds it (Morton order of
// the cells), and between launches the queue is bucketed by key.  At any
// moment the SMs then work on photons of a few neighbouring cells, whose
// records and gate-plane entries stay in L2 together.
constexpr int kSortBits = 4;                            // per axis
constexpr int kBuckets = 1 << (3 * kSortBits);          // 4096

struct PhaseArgs {
    int phase;   // first gate g traced by this launch
    int span;    // gates per launch: photons are parked when their time reaches gate g + span
    int last;    // 1: the last launch, photons run to their end
    PhaseQueue in, out;
    unsigned long long cap;
    const unsigned* order;   // resume order of `in` (nullptr: queue order)
    unsigned* bcount;        // kBuckets photon counts of `out` by spatial key
    float lo[3];             // bounding box origin of the mesh
    float scale[3];          // grid cells per mm along each axis
    float tpark;             // photons whose time reaches this (s) are parked for the next launch
};

// Bytes of queue storage per photon of a phased launch (both queues).
size_t phase_bytes_per_photon(const SimDev& sim);
// Enqueues a phased run of `sim` on `stream`: one launch per `span` gates,
// queues q[0], q[1] (capacity sim.nphoton each) used alternately.  No host
// synchronization between the launches.
// `order` (sim.nphoton entries) and `bscratch` (2*kBuckets entries) hold the
// spatial resume order between launches; `lo`/`hi` bound the mesh.
cudaError_t launch_phased(const SimDev& sim, unsigned long long* work_counter, LaunchShape shape,
                          cudaStream_t stream, const PhaseQueue q[2], int span, unsigned* order,
                          unsigned* bscratch, const float lo[3], const float hi[3]);

// Launches the photon engine for one simulation on `stream`.
cudaError_t launch_plain(const SimDev& sim, unsigned long long* work_counter, LaunchShape shape,
                         cudaStream_t stream);
// Launches the batched engine over `nsims` simulations (`sims` in device memory,
// `cum` = inclusive prefix sums of photon counts, length nsims).  `general_src`:
// some simulation needs the general kernels (general_source); `replay`: some
// simulation is a replay.
cudaError_t launch_batched(const SimDev* sims, const unsigned long long* cum, int nsims,
                           unsigned long long total, int nmed_stride, int reclen_max, int want_seed,
                           unsigned long long* work_counter, LaunchShape shape, cudaStream_t stream,
                           int fast_math, int general_src, int replay);
LaunchShape default_shape(int device, bool batched);
// Whether `s` needs the general kernels (a non-pencil source, a pencil without
// a known initial element, dual-grid output, trajectory records, per-photon
// trace outputs or momentum transfer).  Russian roulette (SimDev::roulette_on)
// runs in a pencil kernel of its own for forward single-simulation launches and
// in the general kernels otherwise.
bool general_source(const SimDev& s);
// Adds the replicated near-source cells of `s` into its fluence and clears them
// (nothing when s.hot_steps == 0).
cudaError_t fold_hot(const SimDev& s, cudaStream_t stream);

// The launchers of each arithmetic policy: engine.cu is compiled once per
// policy, and the entry points above dispatch on SimDev::fast_math.
namespace exact {
cudaError_t launch_plain(const SimDev& sim, unsigned long long* work_counter, LaunchShape shape,
                         cudaStream_t stream);
cudaError_t launch_phased(const SimDev& sim, unsigned long long* work_counter, LaunchShape shape,
                          cudaStream_t stream, const PhaseQueue q[2], int span, unsigned* order,
                          unsigned* bscratch, const float lo[3], const float hi[3]);
cudaError_t launch_batched(const SimDev* sims, const unsigned long long* cum, int nsims,
                           unsigned long long total, int nmed_stride, int reclen_max, int want_seed,
                           unsigned long long* work_counter, LaunchShape shape, cudaStream_t stream,
                           int general_src, int replay);
}  // namespace exact
namespace fast {
cudaError_t launch_plain(const SimDev& sim, unsigned long long* work_counter, LaunchShape shape,
                         cudaStream_t stream);
cudaError_t launch_phased(const SimDev& sim, unsigned long long* work_counter, LaunchShape shape,
                          cudaStream_t stream, const PhaseQueue q[2], int span, unsigned* order,
                          unsigned* bscratch, const float lo[3], const float hi[3]);
cudaError_t launch_batched(const SimDev* sims, const unsigned long long* cum, int nsims,
                           unsigned long long total, int nmed_stride, int reclen_max, int want_seed,
                           unsigned long long* work_counter, LaunchShape shape, cudaStream_t stream,
                           int general_src, int replay);
}  // namespace fast

// Records the message returned by mmcgb_last_error() on this thread.
void set_last_error(const std::string& msg);

}  // namespace mmcgb

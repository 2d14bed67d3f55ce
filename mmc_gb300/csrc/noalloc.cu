// mmcgb_simulate_noalloc: the photon engine for callers that cannot allocate
// device memory.
//
// Who needs it: a host program that owns every byte of the GPU through its
// own pool (a framework whose caching allocator already holds the free HBM, so
// a library cudaMalloc can fail although the pool has room), and serving loops
// that must not call cudaMalloc/cudaFree because those calls synchronize the
// whole device and would stall the simulations already in flight.  Such a
// caller passes its own device buffers for every output; the only other
// global memory the engine needs -- the work counter that hands photons to
// lanes, and the staged media and detector tables -- lives in the file-scope
// array below, which every GPU that loads the library holds until the process
// exits (8 KiB per device).
//
// Rules of use:
//  * The first call on a device resolves the array's device address with
//    cudaGetSymbolAddress (host code cannot use the array's name as a device
//    pointer).  Make that first call before any stream capture.
//  * Every call shares the one array and leaves its contents behind; the call
//    clears what must start at zero (the work counter) itself.  Calls whose
//    work overlaps on the GPU -- on different streams, or on one stream from
//    several host threads without ordering -- race on the array.
//  * Limits: at most kNoAllocMaxMedia media rows and kNoAllocMaxDet detectors;
//    point sources, element output, float64 accumulation only; no replay, no
//    per-photon trace, exiting weight or trajectories.  Anything else is
//    rejected with MMCGB_E_ARG, after the checks mmcgb_simulate makes.
//  * Nothing here calls cudaMalloc, cudaFree or an allocating library routine.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/mmcgb.h"
#include "engine.h"
#include "mesh.h"
#include "mesh_handle.h"

namespace {

constexpr int kNoAllocMaxMedia = MMCGB_NOALLOC_MAX_MEDIA;
constexpr int kNoAllocMaxDet = MMCGB_NOALLOC_MAX_DET;
constexpr size_t kCounterOff = 0;      // unsigned long long work counter
constexpr size_t kMediaOff = 256;      // float4[kNoAllocMaxMedia]
constexpr size_t kDetOff = kMediaOff + sizeof(float4) * kNoAllocMaxMedia;
constexpr size_t kScratchBytes = kDetOff + sizeof(float4) * kNoAllocMaxDet;
static_assert(kScratchBytes <= 8192, "no-alloc scratch must stay within 8 KiB");

static __device__ __align__(256) unsigned char g_noalloc_scratch[8192];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_scratch_ptr[kMaxDevices] = {nullptr};

int fail(int code, const std::string& msg) {
    mmcgb::set_last_error(msg);
    return code;
}

// Source types whose photons all start at srcpos in the initial element.
bool point_source(int t) { return t == 0 || t == 1 || t == 2 || t == 7; }

// Device address of the scratch array on `device` (which must be current).
int scratch_address(int device, unsigned char** out) {
    if (device < 0 || device >= kMaxDevices) return fail(MMCGB_E_ARG, "device index out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_ptr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return fail(MMCGB_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_scratch_ptr[device] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_ptr[device];
    return MMCGB_OK;
}

}  // namespace

extern "C" int32_t mmcgb_simulate_noalloc(mmcgb_mesh* mesh, const mmcgb_config* c, const mmcgb_device_out* out,
                                          void* stream_handle) {
    using namespace mmcgb;
    if (!mesh || !c || !out) return fail(MMCGB_E_ARG, "null argument");
    if (!out->field_raw || !out->energy || !out->counters) return fail(MMCGB_E_ARG, "field_raw, energy and counters are required");
    const HostMesh& m = mesh->host;
    // the checks of the allocating entries first (time gates, media values, unit direction,
    // fluence cell count), then the limits of this entry
    std::string err;
    int rc = validate_config(m, *c, err);
    if (rc) return fail(rc, err);
    if (!point_source(c->srctype))
        return fail(MMCGB_E_ARG, "no-alloc entry: point sources only (pencil, isotropic, cone, arcsine)");
    if (c->nmedia > kNoAllocMaxMedia)
        return fail(MMCGB_E_ARG, "no-alloc entry: nmedia " + std::to_string(c->nmedia) + " exceeds the maximum " +
                                     std::to_string(kNoAllocMaxMedia));
    if (c->detnum > kNoAllocMaxDet)
        return fail(MMCGB_E_ARG, "no-alloc entry: detnum " + std::to_string(c->detnum) + " exceeds the maximum " +
                                     std::to_string(kNoAllocMaxDet));
    if (!c->accum_f64) return fail(MMCGB_E_ARG, "no-alloc entry accumulates in float64 only");
    if (c->replayseed) return fail(MMCGB_E_ARG, "no-alloc entry does not replay");
    if (c->method != 0) return fail(MMCGB_E_ARG, "no-alloc entry deposits on the elements (method 0)");
    if (c->issaveref || c->maxjumpdebug) return fail(MMCGB_E_ARG, "no-alloc entry has no exiting-weight or trajectory output");
    if (c->nodemua) return fail(MMCGB_E_ARG, "no-alloc entry reads no per-node properties");
    if (c->issavedet && (!out->detp || !out->detcount))
        return fail(MMCGB_E_ARG, "issavedet needs detp and detcount");
    if (c->issavedet && c->issaveseed && !out->seeds) return fail(MMCGB_E_ARG, "issaveseed needs seeds");
    // a given e0 is used only when it encloses the source, as in mmcgb_simulate
    const int e0 = initial_element(m, *c);
    if (e0 <= 0) return fail(MMCGB_E_SOURCE, "no element encloses the source");

    cudaError_t e = cudaSetDevice(mesh->device);
    if (e != cudaSuccess) return fail(MMCGB_E_CUDA, cudaGetErrorString(e));
    unsigned char* scratch = nullptr;
    rc = scratch_address(mesh->device, &scratch);
    if (rc) return rc;
    cudaStream_t stream = static_cast<cudaStream_t>(stream_handle);

    const int maxgate = (int)((c->tend - c->tstart) / c->tstep + 0.5f);
    const int M = c->nmedia - 1;
    const int reclen = (2 + (c->ismomentum > 0)) * M + (c->issaveexit > 0) * 6 + 1;
    const size_t flen = (size_t)m.ne * maxgate;
    float4* dmed = reinterpret_cast<float4*>(scratch + kMediaOff);
    float4* ddet = reinterpret_cast<float4*>(scratch + kDetOff);
    unsigned long long* work = reinterpret_cast<unsigned long long*>(scratch + kCounterOff);

    // stage inputs into the scratch array and clear the caller's outputs
    if ((e = cudaMemcpyAsync(dmed, c->media, sizeof(float4) * c->nmedia, cudaMemcpyHostToDevice, stream)) != cudaSuccess ||
        (c->detnum && (e = cudaMemcpyAsync(ddet, c->detpos, sizeof(float4) * c->detnum, cudaMemcpyHostToDevice, stream)) != cudaSuccess) ||
        (e = cudaMemsetAsync(out->field_raw, 0, sizeof(double) * flen, stream)) != cudaSuccess ||
        (e = cudaMemsetAsync(out->energy, 0, sizeof(double) * 2, stream)) != cudaSuccess ||
        (e = cudaMemsetAsync(out->counters, 0, sizeof(unsigned long long) * 2, stream)) != cudaSuccess ||
        (c->issavedet && (e = cudaMemsetAsync(out->detcount, 0, sizeof(unsigned), stream)) != cudaSuccess))
        return fail(MMCGB_E_CUDA, std::string("staging: ") + cudaGetErrorString(e));

    SimDev S;
    std::memset(&S, 0, sizeof(S));
    S.rec = mesh->rec;
    S.elem = mesh->elem;
    S.node = mesh->node;
    S.label = mesh->label;
    S.ne = m.ne;
    S.lbits = m.lbits;
    S.lmask = (1 << m.lbits) - 1;
    S.e0 = e0;
    S.nmedia = c->nmedia;
    S.detnum = c->detnum;
    S.media = dmed;
    S.det = ddet;
    S.nphoton = c->nphoton;
    S.photon_offset = c->photon_offset;
    S.seed = c->seed;
    S.step_budget = c->step_budget ? c->step_budget : 100000000ull;
    for (int k = 0; k < 3; k++) {
        S.srcpos[k] = c->srcpos[k];
        S.srcdir[k] = c->srcdir[k];
    }
    S.srctype = c->srctype;
    S.srcp1 = make_float4(c->srcparam1[0], c->srcparam1[1], c->srcparam1[2], c->srcparam1[3]);
    S.srcp2 = make_float4(c->srcparam2[0], c->srcparam2[1], c->srcparam2[2], c->srcparam2[3]);
    S.focus = c->focus;
    S.tstart = c->tstart;
    S.tend = c->tstart + c->tstep * (float)maxgate;
    S.Rtstep = 1.f / c->tstep;
    S.maxgate = maxgate;
    S.roulette_on = ((S.tend - S.tstart) * S.Rtstep <= 1.f && c->minenergy > 0.f) ? 1 : 0;
    S.minenergy = c->minenergy;
    S.roulettesize = c->roulettesize;
    S.nout = c->nout;
    S.isreflect = c->isreflect;
    S.isspecular = c->isspecular;
    S.voidtime = c->voidtime;
    S.issavedet = c->issavedet ? 1 : 0;
    S.issaveexit = c->issaveexit ? 1 : 0;
    S.ismomentum = c->ismomentum ? 1 : 0;
    S.issaveseed = (c->issavedet && c->issaveseed) ? 1 : 0;
    S.outputtype = c->outputtype;
    S.accum_f64 = 1;
    S.fast_math = c->fast_math ? 1 : 0;
    S.reclen = reclen;
    S.nmed_ppath = M;
    S.f64 = out->field_raw;
    S.detp = c->issavedet ? out->detp : nullptr;
    S.seeds = S.issaveseed ? reinterpret_cast<unsigned long long*>(out->seeds) : nullptr;
    S.detcount = c->issavedet ? out->detcount : nullptr;
    S.maxdet = c->issavedet ? c->maxdetphoton : 0;
    S.energy = out->energy;
    S.counters = reinterpret_cast<unsigned long long*>(out->counters);
    S.ncounters = 2;

    LaunchShape shape = default_shape(mesh->device, false);
    if (c->threads > 0) shape.threads = std::max(32, std::min(c->threads, 128) / 32 * 32);
    if (c->blocks > 0) shape.blocks = c->blocks;
    e = launch_plain(S, work, shape, stream);  // zeroes the work counter on `stream` first
    if (e != cudaSuccess) return fail(MMCGB_E_CUDA, std::string("photon engine launch: ") + cudaGetErrorString(e));
    return MMCGB_OK;
}

// C ABI of libmmcgb (include/mmcgb.h): resident meshes, single and batched
// simulations.  Every failure returns a status and records a message; nothing
// here exits the process (the reference's mcx_error path,
// src/mmc_utils.c:1426-1443, terminates instead).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/mmcgb.h"
#include "engine.h"
#include "mesh.h"
#include "mesh_handle.h"
#include "output_dev.h"

using namespace mmcgb;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

}  // namespace

void mmcgb::set_last_error(const std::string& msg) { g_err = msg; }

namespace {

int cuda_fail(cudaError_t e, const char* what) {
    return fail(MMCGB_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                         \
    do {                                                 \
        cudaError_t _e = (call);                         \
        if (_e != cudaSuccess) return cuda_fail(_e, #call); \
    } while (0)

int gates_of(const mmcgb_config& c) { return (int)((c.tend - c.tstart) / c.tstep + 0.5f); }

// Patterns sharing each photon (mmcgb_config.srcnum; 0 means 1).
int src_count(const mmcgb_config& c) { return c.srcnum > 1 ? c.srcnum : 1; }

// Free device memory for new stream-ordered allocations: what the driver
// reports plus what the default pool holds without using.
size_t free_device_memory(int device) {
    size_t freeb = 0, totalb = 0;
    if (cudaMemGetInfo(&freeb, &totalb) != cudaSuccess) {
        (void)cudaGetLastError();
        return 0;
    }
    cudaMemPool_t pool;
    uint64_t reserved = 0, used = 0;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess &&
        cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved) == cudaSuccess &&
        cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used) == cudaSuccess && reserved > used)
        freeb += (size_t)(reserved - used);
    (void)cudaGetLastError();
    return freeb;
}

// Dual-grid geometry (mesh_createdualmesh, src/mmc_mesh.c:349-381): float
// arithmetic, bounding box padded by EPS, dim = (int)(span / step) + 1.
void grid_geometry(const HostMesh& m, float step, unsigned dim[3], float nmin[3]) {
    float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
    for (int i = 0; i < m.nn; i++)
        for (int k = 0; k < 3; k++) {
            lo[k] = std::min(m.node[3 * (size_t)i + k], lo[k]);
            hi[k] = std::max(m.node[3 * (size_t)i + k], hi[k]);
        }
    for (int k = 0; k < 3; k++) {
        lo[k] -= 1e-6f;
        hi[k] += 1e-6f;
        nmin[k] = lo[k];
        dim[k] = (unsigned)(int)((hi[k] - lo[k]) / step) + 1u;
    }
}

float grid_step(const mmcgb_config& c) { return c.gridstep > 0.f ? c.gridstep : 1.f; }

// Fluence entries per gate: elements, or grid voxels for the dual-grid output.
size_t frame_len(const HostMesh& m, const mmcgb_config& c) {
    if (c.method != 1) return (size_t)m.ne;
    unsigned dim[3];
    float nmin[3];
    grid_geometry(m, grid_step(c), dim, nmin);
    return (size_t)dim[0] * dim[1] * dim[2];
}

// Source types whose photons all start at srcpos in the initial element (the
// reference returns early from the launch for them, src/mmc_raytrace.c:2353-2357,
// :2483-2485); the others are located per photon.
bool point_source(int t) { return t == 0 || t == 1 || t == 2 || t == 7; }

size_t pattern_len(const mmcgb_config& c) {
    if (c.srctype == 5)
        return (size_t)std::max(0, (int)c.srcparam1[3]) * (size_t)std::max(0, (int)c.srcparam2[3]) *
               (size_t)src_count(c);
    if (c.srctype == 15)
        return (size_t)std::max(0, (int)c.srcparam1[0]) * (size_t)std::max(0, (int)c.srcparam1[1]) *
               (size_t)std::max(0, (int)c.srcparam1[2]);
    return 0;
}

}  // namespace

// The checks every simulation entry makes before it allocates anything
// (declared in mesh.h; mmcgb_simulate_noalloc runs them too).
int mmcgb::validate_config(const HostMesh& m, const mmcgb_config& c, std::string& err) {
    if (c.srctype < 0 || c.srctype > 17) { err = "srctype must be 0..17"; return MMCGB_E_ARG; }
    if (c.method != 0 && c.method != 1) { err = "method must be 0 (element output) or 1 (dual grid)"; return MMCGB_E_ARG; }
    if (c.method == 1 && c.replayseed) { err = "replay runs deposit on the elements (method 0)"; return MMCGB_E_ARG; }
    if (c.method == 1 && !(c.gridstep >= 0.f && std::isfinite(c.gridstep))) { err = "gridstep must be >= 0"; return MMCGB_E_ARG; }
    if ((c.srctype == 5 || c.srctype == 15) && (!c.srcpattern || pattern_len(c) == 0)) {
        err = "pattern sources need srcpattern and a positive pattern size in srcparam1/srcparam2";
        return MMCGB_E_ARG;
    }
    if (c.srctype == 14 && (!(c.srcparam1[3] > 1.f) || !(c.srcparam2[3] > 1.f))) {
        err = "pencil-array sources need at least 2 beams along each edge (srcparam1.w, srcparam2.w)";
        return MMCGB_E_ARG;
    }
    for (int k = 0; k < 4; k++)
        if (!std::isfinite(c.srcparam1[k]) || !std::isfinite(c.srcparam2[k])) { err = "source parameters must be finite"; return MMCGB_E_ARG; }
    if (c.srcnum < 0) { err = "srcnum must be >= 0"; return MMCGB_E_ARG; }
    if (c.srcnum > 1 && c.srctype != 5) { err = "srcnum > 1 needs a pattern source (srctype 5)"; return MMCGB_E_ARG; }
    // the reference refuses the same (src/mmc_utils.c:3534-3536)
    if (c.srcnum > 1 && c.replayseed) { err = "photon sharing (srcnum > 1) does not replay"; return MMCGB_E_ARG; }
    if (!(c.tstep > 0.f) || !(c.tend > c.tstart)) { err = "time gates need tstep > 0 and tend > tstart"; return MMCGB_E_ARG; }
    if (gates_of(c) < 1) { err = "time window holds no gate"; return MMCGB_E_ARG; }
    // The engine addresses a fluence cell (gate, element or voxel) with a 32-bit index and keeps
    // 0x7FFFFFFF as its "no pending deposit" mark, so every cell index must stay below it.
    if (frame_len(m, c) * (size_t)gates_of(c) * (size_t)src_count(c) >= (size_t)kMaxFluenceCells) {
        err = "fluence of " + std::to_string(frame_len(m, c)) + " cells x " + std::to_string(gates_of(c)) +
              " gates" + (src_count(c) > 1 ? " x " + std::to_string(src_count(c)) + " patterns" : std::string()) +
              " exceeds the engine's 2^31-1 cells: use fewer gates" + (c.method == 1 ? " or a larger gridstep" : "");
        return MMCGB_E_ARG;
    }
    if (c.nmedia < 2 || c.nmedia > kMaxMedia || !c.media) { err = "media table needs 2..64 rows (row 0 = background)"; return MMCGB_E_ARG; }
    if (m.maxlabel > c.nmedia - 1) { err = "mesh label exceeds the number of media"; return MMCGB_E_ARG; }
    if (c.detnum < 0 || (c.detnum > 0 && !c.detpos)) { err = "detnum > 0 needs detpos"; return MMCGB_E_ARG; }
    if (c.issavedet && c.maxdetphoton == 0) { err = "issavedet needs maxdetphoton > 0"; return MMCGB_E_ARG; }
    if (c.replayseed && (!c.replayweight || !c.replaytime)) { err = "replay needs replayseed, replayweight and replaytime"; return MMCGB_E_ARG; }
    if (c.nphoton > 0xFFFFFFFFull && (c.replayseed)) { err = "replay photon count must fit 32 bits"; return MMCGB_E_ARG; }
    for (int i = 0; i < c.nmedia; i++)
        for (int k = 0; k < 4; k++)
            if (!std::isfinite(c.media[4 * i + k])) { err = "media values must be finite"; return MMCGB_E_ARG; }
    const float vn = c.srcdir[0] * c.srcdir[0] + c.srcdir[1] * c.srcdir[1] + c.srcdir[2] * c.srcdir[2];
    if (!(std::fabs(vn - 1.f) < 1e-3f)) { err = "srcdir must be a unit vector"; return MMCGB_E_ARG; }
    for (const float* v : {c.nodemua, c.nodemua ? c.nodemusp : nullptr})
        if (v)
            for (int i = 0; i < m.nn; i++)
                if (!std::isfinite(v[i])) { err = "per-node mua/musp values must be finite"; return MMCGB_E_ARG; }
    return MMCGB_OK;
}

// Initial element: a given e0 is kept only if it encloses the source
// (src/mmc_mesh.c:1325-1329), otherwise the source is located; 0 when no
// element encloses it.
int mmcgb::initial_element(const HostMesh& m, const mmcgb_config& c) {
    int e0 = c.e0;
    if (e0 > 0 && e0 <= m.ne) {
        const float* p = c.srcpos;
        const int* el = &m.elem[4 * (size_t)(e0 - 1)];
        bool inside = true;
        for (int i = 0; i < 4; i++) {
            const float* a = &m.node[3 * (size_t)(el[kOut[i][0]] - 1)];
            const float* b = &m.node[3 * (size_t)(el[kOut[i][1]] - 1)];
            const float* cc = &m.node[3 * (size_t)(el[kOut[i][2]] - 1)];
            const float ab[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
            const float ac[3] = {cc[0] - a[0], cc[1] - a[1], cc[2] - a[2]};
            const float s[3] = {p[0] - a[0], p[1] - a[1], p[2] - a[2]};
            const float n[3] = {ab[1] * ac[2] - ab[2] * ac[1], ab[2] * ac[0] - ab[0] * ac[2], ab[0] * ac[1] - ab[1] * ac[0]};
            if (-(s[0] * n[0] + s[1] * n[1] + s[2] * n[2]) < 0.f) inside = false;
        }
        if (inside) return e0;
    }
    const int e = locate(m, c.srcpos);
    return e > 0 ? e : 0;
}

namespace {

// Device buffers of one simulation (stream-ordered allocations).
struct SimBuffers {
    float4* media = nullptr;
    float4* det = nullptr;
    double* f64 = nullptr;
    float* f32 = nullptr;
    float* detp = nullptr;
    unsigned long long* seeds = nullptr;
    unsigned int* detcount = nullptr;
    double* energy = nullptr;
    double* energy_src = nullptr;  // photon sharing: 64 slots x 2 x srcnum
    unsigned long long* counters = nullptr;
    float* pattern = nullptr;
    double* hot = nullptr;        // replicated near-source cells (SimDev::hot), allocated at first launch
    float* nodemua = nullptr;   // per-node mua / mus (nn each), when given
    float* nodemusp = nullptr;
    double* dref = nullptr;
    float* traj = nullptr;
    unsigned* trajcount = nullptr;
    unsigned long long* rseed = nullptr;
    float* rweight = nullptr;
    float* rtime = nullptr;
    float* pw = nullptr;
    unsigned int* ps = nullptr;
    int* pd = nullptr;
    std::vector<void*> owned;
    cudaStream_t stream = nullptr;

    template <class T>
    cudaError_t alloc(T** p, size_t count) {
        if (count == 0) { *p = nullptr; return cudaSuccess; }
        cudaError_t e = cudaMallocAsync((void**)p, sizeof(T) * count, stream);
        if (e == cudaSuccess) owned.push_back(*p);
        return e;
    }
    void release() {
        for (void* p : owned) cudaFreeAsync(p, stream);
        owned.clear();
    }
};

struct Prepared {
    SimDev sim;
    SimBuffers buf;
    int maxgate = 0;
    int reclen = 0;   // columns per record incl. detector id
    size_t flen = 0;
    bool hot_ok = false;  // the simulation may use replicated near-source cells (SimDev::hot)
};

// The source locator on the device, for simulations whose launch positions are located per
// photon (every source but the pencil beam): built and uploaded once per mesh.
int ensure_device_locator(mmcgb_mesh* m) {
    std::lock_guard<std::mutex> lock(m->loc_mu);
    if (m->loc_start) return MMCGB_OK;
    if (!ensure_locator(m->host))
        return fail(MMCGB_E_MESH, "mesh too large for the source locator (more than 2^32 element-bin pairs)");
    const LocGrid& g = m->host.grid;
    unsigned *start = nullptr, *items = nullptr;
    cudaError_t e;
    if ((e = cudaMalloc((void**)&start, sizeof(unsigned) * g.start.size())) != cudaSuccess ||
        (e = cudaMalloc((void**)&items, sizeof(unsigned) * std::max<size_t>(1, g.items.size()))) != cudaSuccess ||
        (e = cudaMemcpy(start, g.start.data(), sizeof(unsigned) * g.start.size(), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(items, g.items.data(), sizeof(unsigned) * g.items.size(), cudaMemcpyHostToDevice)) != cudaSuccess) {
        if (start) cudaFree(start);
        if (items) cudaFree(items);
        return cuda_fail(e, "source locator upload");
    }
    m->loc_start = start;
    m->loc_items = items;
    return MMCGB_OK;
}

int prepare_sim(mmcgb_mesh* mesh, const mmcgb_config& c, const mmcgb_result* res, cudaStream_t stream, Prepared& P) {
    const HostMesh& m = mesh->host;
    std::string err;
    int rc = validate_config(m, c, err);
    if (rc) return fail(rc, err);
    int e0 = initial_element(m, c);
    // point sources start in e0; the others are located per photon and may lie outside the mesh
    if (e0 <= 0 && point_source(c.srctype)) return fail(MMCGB_E_SOURCE, "initial element does not enclose the source");

    if (c.srctype != 0) {  // launch positions located on the device
        rc = ensure_device_locator(mesh);
        if (rc) return rc;
    }
    P.maxgate = gates_of(c);
    const int M = c.nmedia - 1;
    const int reclen_dev = (2 + (c.ismomentum > 0)) * M + (c.issaveexit > 0) * 6 + 1;
    P.reclen = reclen_dev + 1;
    P.flen = frame_len(m, c) * P.maxgate * (size_t)src_count(c);
    SimBuffers& B = P.buf;
    B.stream = stream;
    const bool f64 = c.accum_f64 != 0;
    const size_t maxdet = c.issavedet ? c.maxdetphoton : 0;
    size_t need = P.flen * (f64 ? 8 : 8) + maxdet * (P.reclen * 4 + (c.issaveseed ? 16 : 0));
    const size_t freeb = free_device_memory(mesh->device);
    if (need + (64ull << 20) > freeb) return fail(MMCGB_E_NOMEM, "not enough free device memory for fluence and detector buffers");
    CK(B.alloc(&B.media, c.nmedia));
    CK(B.alloc(&B.det, c.detnum));
    if (f64) CK(B.alloc(&B.f64, P.flen)); else CK(B.alloc(&B.f32, 2 * P.flen));
    CK(B.alloc(&B.detp, maxdet * P.reclen));
    if (c.issaveseed) CK(B.alloc(&B.seeds, maxdet * 2));
    CK(B.alloc(&B.detcount, 1));
    CK(B.alloc(&B.energy, 2));
    if (src_count(c) > 1) {
        CK(B.alloc(&B.energy_src, (size_t)kEnergySlots * 2 * src_count(c)));
        CK(cudaMemsetAsync(B.energy_src, 0, sizeof(double) * kEnergySlots * 2 * src_count(c), stream));
    }
    CK(B.alloc(&B.counters, 3));
    if (c.maxjumpdebug) {
        CK(B.alloc(&B.traj, (size_t)c.maxjumpdebug * 6));
        CK(B.alloc(&B.trajcount, 1));
        CK(cudaMemsetAsync(B.trajcount, 0, sizeof(unsigned), stream));
    }
    if (c.issaveref) {
        CK(B.alloc(&B.dref, (size_t)m.nf * P.maxgate));
        CK(cudaMemsetAsync(B.dref, 0, sizeof(double) * (size_t)m.nf * P.maxgate, stream));
    }
    const size_t plen = pattern_len(c);
    if (plen) {
        CK(B.alloc(&B.pattern, plen));
        CK(cudaMemcpyAsync(B.pattern, c.srcpattern, sizeof(float) * plen, cudaMemcpyHostToDevice, stream));
    }
    // replicated near-source cells (allocated by the first unbatched launch, ensure_hot):
    // forward element-output runs of a point source with float64 sums
    P.hot_ok = f64 && c.method == 0 && !c.replayseed && point_source(c.srctype) && src_count(c) == 1;
    if (c.nodemua) {
        CK(B.alloc(&B.nodemua, (size_t)m.nn));
        CK(cudaMemcpyAsync(B.nodemua, c.nodemua, sizeof(float) * m.nn, cudaMemcpyHostToDevice, stream));
        if (c.nodemusp) {
            CK(B.alloc(&B.nodemusp, (size_t)m.nn));
            CK(cudaMemcpyAsync(B.nodemusp, c.nodemusp, sizeof(float) * m.nn, cudaMemcpyHostToDevice, stream));
        }
    }
    if (c.replayseed) {
        CK(B.alloc(&B.rseed, 2 * c.nphoton));
        CK(B.alloc(&B.rweight, c.nphoton));
        CK(B.alloc(&B.rtime, c.nphoton));
        CK(cudaMemcpyAsync(B.rseed, c.replayseed, 16 * c.nphoton, cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(B.rweight, c.replayweight, 4 * c.nphoton, cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(B.rtime, c.replaytime, 4 * c.nphoton, cudaMemcpyHostToDevice, stream));
    }
    if (res && res->photon_weight) CK(B.alloc(&B.pw, c.nphoton));
    if (res && res->photon_steps) CK(B.alloc(&B.ps, c.nphoton));
    if (res && res->photon_det) CK(B.alloc(&B.pd, c.nphoton));
    CK(cudaMemcpyAsync(B.media, c.media, sizeof(float4) * c.nmedia, cudaMemcpyHostToDevice, stream));
    if (c.detnum) CK(cudaMemcpyAsync(B.det, c.detpos, sizeof(float4) * c.detnum, cudaMemcpyHostToDevice, stream));
    if (f64) CK(cudaMemsetAsync(B.f64, 0, sizeof(double) * P.flen, stream));
    else CK(cudaMemsetAsync(B.f32, 0, sizeof(float) * 2 * P.flen, stream));
    CK(cudaMemsetAsync(B.detcount, 0, sizeof(unsigned), stream));
    CK(cudaMemsetAsync(B.energy, 0, sizeof(double) * 2, stream));
    CK(cudaMemsetAsync(B.counters, 0, sizeof(unsigned long long) * 3, stream));

    SimDev& S = P.sim;
    std::memset(&S, 0, sizeof(S));
    S.rec = mesh->rec;
    S.elem = mesh->elem;
    S.node = mesh->node;
    S.label = mesh->label;
    S.ne = m.ne;
    S.lbits = m.lbits;
    S.lmask = (1 << m.lbits) - 1;
    S.e0 = e0;
    S.nmedia = c.nmedia;
    S.detnum = c.detnum;
    S.media = B.media;
    S.nodemua = B.nodemua;
    S.nodemusp = B.nodemusp;
    S.det = B.det;
    S.nphoton = c.nphoton;
    S.photon_offset = c.photon_offset;
    S.seed = c.seed;
    S.step_budget = c.step_budget ? c.step_budget : 100000000ull;
    for (int k = 0; k < 3; k++) {
        S.srcpos[k] = c.srcpos[k];
        S.srcdir[k] = c.srcdir[k];
    }
    S.srctype = c.srctype;
    S.srcp1 = make_float4(c.srcparam1[0], c.srcparam1[1], c.srcparam1[2], c.srcparam1[3]);
    S.srcp2 = make_float4(c.srcparam2[0], c.srcparam2[1], c.srcparam2[2], c.srcparam2[3]);
    S.focus = c.focus;
    S.srcpattern = B.pattern;
    S.srcnum = src_count(c);
    S.energy_src = B.energy_src;
    S.loc_start = mesh->loc_start;
    S.loc_items = mesh->loc_items;
    S.loc_res = m.grid.res;
    for (int k = 0; k < 3; k++) {
        S.loc_lo[k] = m.grid.lo[k];
        S.loc_inv[k] = m.grid.inv[k];
    }
    // per-launch time window (src/mmc_cu_host.cu:642-662): all gates in one launch
    S.tstart = c.tstart;
    S.tend = c.tstart + c.tstep * (float)P.maxgate;
    S.Rtstep = 1.f / c.tstep;
    S.maxgate = P.maxgate;
    S.roulette_on = ((S.tend - S.tstart) * S.Rtstep <= 1.f && c.minenergy > 0.f) ? 1 : 0;
    S.minenergy = c.minenergy;
    S.roulettesize = c.roulettesize;
    S.nout = c.nout;
    S.isreflect = c.isreflect;
    S.isspecular = c.isspecular;
    S.voidtime = c.voidtime;
    S.issavedet = c.issavedet ? 1 : 0;
    S.issaveexit = c.issaveexit ? 1 : 0;
    S.ismomentum = c.ismomentum ? 1 : 0;
    S.issaveseed = c.issaveseed ? 1 : 0;
    S.outputtype = c.outputtype;
    S.replay = c.replayseed ? 1 : 0;
    S.accum_f64 = f64 ? 1 : 0;
    S.fast_math = c.fast_math ? 1 : 0;
    S.reclen = reclen_dev;
    S.nmed_ppath = M;
    S.replayseed = B.rseed;
    S.replayweight = B.rweight;
    S.replaytime = B.rtime;
    S.f64 = B.f64;
    S.f32a = B.f32;
    S.f32b = B.f32 ? B.f32 + P.flen : nullptr;
    S.detp = B.detp;
    S.seeds = B.seeds;
    S.detcount = B.detcount;
    S.maxdet = (unsigned)maxdet;
    S.energy = B.energy;
    S.counters = B.counters;
    S.ncounters = 3;
    S.photon_weight = B.pw;
    S.photon_steps = B.ps;
    S.photon_det = B.pd;
    S.dref = B.dref;
    S.nf = m.nf;
    S.traj = B.traj;
    S.trajcount = B.trajcount;
    S.maxtraj = c.maxjumpdebug;
    S.grid = (c.method == 1) ? 1 : 0;
    S.framelen = (unsigned)frame_len(m, c);
    if (S.grid) {
        grid_geometry(m, grid_step(c), S.gdim, S.gmin);
        S.gstep_inv = 1.f / grid_step(c);
    }
    return MMCGB_OK;
}

// Reads back one simulation and runs the output stage.
int finish_sim(mmcgb_mesh* mesh, const mmcgb_config& c, Prepared& P, mmcgb_result* res, cudaStream_t stream,
               unsigned long long launched) {
    SimBuffers& B = P.buf;
    unsigned detected = 0;
    double energy[2] = {0, 0};
    unsigned long long counters[3] = {0, 0, 0};
    CK(cudaMemcpyAsync(&detected, B.detcount, sizeof(unsigned), cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(energy, B.energy, sizeof(energy), cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(counters, B.counters, sizeof(counters), cudaMemcpyDeviceToHost, stream));
    const size_t saved = std::min<size_t>(detected, c.issavedet ? c.maxdetphoton : 0);
    const int K = src_count(c);
    std::vector<double> esrc;  // photon sharing: launched weight per pattern, then escaped weight
    if (K > 1) {
        std::vector<double> slots((size_t)kEnergySlots * 2 * K);
        CK(cudaMemcpyAsync(slots.data(), B.energy_src, sizeof(double) * slots.size(), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        esrc.assign(2 * (size_t)K, 0.0);
        for (int sl = 0; sl < kEnergySlots; sl++)
            for (size_t i = 0; i < 2 * (size_t)K; i++) esrc[i] += slots[(size_t)sl * 2 * K + i];
    }
    double normalizer = 1.0;
    if (res->field && K > 1) {
        // Photon sharing: each pattern's deposits (cells of one gate and element adjacent,
        // src/mmc_cu_host.cu:961-971) scattered, accumulated and normalized with that pattern's
        // energies (src/mmc_cu_host.cu:984-995); the normalizer reported is their mean.
        // Host output stage.
        const int G = P.maxgate;
        std::vector<double> raw(P.flen);
        if (B.f64) {
            CK(cudaMemcpyAsync(raw.data(), B.f64, sizeof(double) * P.flen, cudaMemcpyDeviceToHost, stream));
            CK(cudaStreamSynchronize(stream));
        } else {
            std::vector<float> ab(2 * P.flen);
            CK(cudaMemcpyAsync(ab.data(), B.f32, sizeof(float) * 2 * P.flen, cudaMemcpyDeviceToHost, stream));
            CK(cudaStreamSynchronize(stream));
            for (size_t i = 0; i < P.flen; i++) raw[i] = (double)ab[i] + (double)ab[P.flen + i];
        }
        const size_t frame = P.flen / ((size_t)G * K);
        const size_t datalen = (c.method == 1) ? frame : (c.basisorder ? (size_t)mesh->host.nn : (size_t)mesh->host.ne);
        const size_t nout = datalen * G;
        std::vector<double> raw_p(frame * G), add(nout), field_p(nout);
        double sum_norm = 0.0;
        for (int p = 0; p < K; p++) {
            for (size_t i = 0; i < frame * G; i++) raw_p[i] = raw[i * K + p];
            for (size_t i = 0; i < nout; i++) field_p[i] = c.accumulate ? res->field[i * K + p] : 0.0;
            double norm;
            if (c.method == 1) {
                norm = grid_normalizer(c, esrc[p]);
                for (size_t i = 0; i < nout; i++) field_p[i] = (field_p[i] + raw_p[i]) * norm;
            } else {
                scatter_output(mesh->host, c, G, raw_p.data(), add.data());
                for (size_t i = 0; i < nout; i++) field_p[i] += add[i];
                norm = normalize_in_place(mesh->host, c, G, esrc[p], esrc[K + p], field_p.data());
            }
            sum_norm += norm;
            for (size_t i = 0; i < nout; i++) res->field[i * K + p] = field_p[i];
        }
        normalizer = sum_norm / K;
    } else if (res->field && c.accumulate) {
        // mmc_run_cu's semantics (src/mmc_cu_host.cu:916-976, :984-1061): this run's deposits
        // (scattered to the nodes) are added to what the caller's field holds, then the sum is
        // normalized in place with this run's energies.  Host output stage.
        const int G = P.maxgate;
        std::vector<double> raw(P.flen);
        if (B.f64) {
            CK(cudaMemcpyAsync(raw.data(), B.f64, sizeof(double) * P.flen, cudaMemcpyDeviceToHost, stream));
            CK(cudaStreamSynchronize(stream));
        } else {
            std::vector<float> ab(2 * P.flen);
            CK(cudaMemcpyAsync(ab.data(), B.f32, sizeof(float) * 2 * P.flen, cudaMemcpyDeviceToHost, stream));
            CK(cudaStreamSynchronize(stream));
            for (size_t i = 0; i < P.flen; i++) raw[i] = (double)ab[i] + (double)ab[P.flen + i];
        }
        if (c.method == 1) {
            normalizer = grid_normalizer(c, energy[0]);
            for (size_t i = 0; i < P.flen; i++) res->field[i] = (res->field[i] + raw[i]) * normalizer;
        } else {
            const size_t nout = (size_t)(c.basisorder ? mesh->host.nn : mesh->host.ne) * G;
            std::vector<double> add(nout);
            scatter_output(mesh->host, c, G, raw.data(), add.data());
            for (size_t i = 0; i < nout; i++) res->field[i] += add[i];
            normalizer = normalize_in_place(mesh->host, c, G, energy[0], energy[1], res->field);
        }
    } else if (res->field) {
        // output stage on the device, then one copy of the final field
        const size_t datalen = c.method == 1 ? frame_len(mesh->host, c)
                                             : (c.basisorder ? (size_t)mesh->host.nn : (size_t)mesh->host.ne);
        const size_t nout = datalen * P.maxgate;
        double* dout = nullptr;
        float* dnvol = nullptr;
        CK(cudaStreamSynchronize(stream));  // energies are needed by the normalization
        CK(cudaMallocAsync((void**)&dout, sizeof(double) * nout, stream));
        if (c.basisorder && c.method != 1) {
            const std::vector<float> nv = surface_fixed_nvol(mesh->host, c);
            CK(cudaMallocAsync((void**)&dnvol, sizeof(float) * nv.size(), stream));
            CK(cudaMemcpyAsync(dnvol, nv.data(), sizeof(float) * nv.size(), cudaMemcpyHostToDevice, stream));
            CK(cudaStreamSynchronize(stream));  // nv is a host temporary
        }
        DeviceOutputArgs A;
        A.host = &mesh->host;
        A.cfg = &c;
        A.maxgate = P.maxgate;
        A.energytot = energy[0];
        A.energyesc = energy[1];
        A.f64 = B.f64;
        A.f32a = B.f32;
        A.f32b = B.f32 ? B.f32 + P.flen : nullptr;
        A.elem = mesh->elem;
        A.label = mesh->label;
        A.evol = mesh->evol;
        A.nvol = dnvol;
        A.media = B.media;
        A.out = dout;
        A.gridlen = c.method == 1 ? datalen : 0;
        CK(device_output(A, stream, &normalizer));
        CK(cudaMemcpyAsync(res->field, dout, sizeof(double) * nout, cudaMemcpyDeviceToHost, stream));
        CK(cudaFreeAsync(dout, stream));
        if (dnvol) CK(cudaFreeAsync(dnvol, stream));
    }
    if (res->detp && saved) CK(cudaMemcpyAsync(res->detp, B.detp, sizeof(float) * P.reclen * saved, cudaMemcpyDeviceToHost, stream));
    if (res->seeds && saved && B.seeds) CK(cudaMemcpyAsync(res->seeds, B.seeds, 16 * saved, cudaMemcpyDeviceToHost, stream));
    if (res->photon_weight) CK(cudaMemcpyAsync(res->photon_weight, B.pw, sizeof(float) * c.nphoton, cudaMemcpyDeviceToHost, stream));
    if (res->photon_steps) CK(cudaMemcpyAsync(res->photon_steps, B.ps, sizeof(unsigned) * c.nphoton, cudaMemcpyDeviceToHost, stream));
    if (res->photon_det) CK(cudaMemcpyAsync(res->photon_det, B.pd, sizeof(int) * c.nphoton, cudaMemcpyDeviceToHost, stream));
    unsigned ntraj = 0;
    if (B.trajcount) {
        CK(cudaMemcpyAsync(&ntraj, B.trajcount, sizeof(unsigned), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        if (res->traj && ntraj)
            CK(cudaMemcpyAsync(res->traj, B.traj, sizeof(float) * 6 * std::min(ntraj, c.maxjumpdebug),
                               cudaMemcpyDeviceToHost, stream));
    }
    res->ntraj = ntraj;
    const size_t nref = (size_t)mesh->host.nf * P.maxgate;
    std::vector<double> dref_run;
    if (res->dref && B.dref) {
        double* dst = res->dref;
        if (c.accumulate) {
            dref_run.resize(nref);
            dst = dref_run.data();
        }
        CK(cudaMemcpyAsync(dst, B.dref, sizeof(double) * nref, cudaMemcpyDeviceToHost, stream));
    }
    B.release();
    CK(cudaStreamSynchronize(stream));
    res->detected = detected;
    res->saved = (uint32_t)saved;
    res->reclen = P.reclen;
    res->maxgate = P.maxgate;
    (void)launched;
    res->energytot = energy[0];  // launched weight, summed on the device (source weights may be < 1)
    res->energyesc = energy[1];
    const double launched_w = energy[0];
    if (K > 1) {  // the patterns' sums, as the reference reports them (src/mmc_cu_host.cu:776-781)
        res->energytot = res->energyesc = 0.0;
        for (int p = 0; p < K; p++) {
            res->energytot += esrc[p];
            res->energyesc += esrc[K + p];
        }
        if (res->energy_src) std::memcpy(res->energy_src, esrc.data(), sizeof(double) * 2 * K);
    }
    res->raytet = counters[0];
    res->aborted = counters[1];
    res->outside = counters[2];
    res->normalizer = normalizer;
    if (!dref_run.empty())  // mesh->dref += dref (src/mmc_cu_host.cu:978-982)
        for (size_t i = 0; i < nref; i++) res->dref[i] += dref_run[i];
    if (res->dref && B.dref == nullptr && nref && !c.accumulate) std::memset(res->dref, 0, sizeof(double) * nref);
    if (res->dref && c.isnormalized && launched_w > 0) {  // src/mmc_mesh.c:2160-2167
        // (a shared photon's exit weight is not scaled by the patterns: the launched photon
        // weight normalizes it)
        const float normalizor = 1.f / (float)launched_w;
        for (size_t i = 0; i < nref; i++) res->dref[i] *= normalizor;
    }
    if (res->outside)
        return fail(MMCGB_E_SOURCE, std::to_string(res->outside) + " photons were launched at positions no element encloses");
    if (res->aborted) return fail(MMCGB_E_BUDGET, "some photons exceeded the per-photon step budget");
    return MMCGB_OK;
}

}  // namespace

struct mmcgb_session {
    mmcgb_mesh* mesh = nullptr;
    mmcgb_config cfg;
    Prepared P;
    cudaStream_t stream = nullptr;
    unsigned long long* work = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t ready = nullptr;  // recorded after the session's buffers are set up
    unsigned long long launched = 0;
    int launches = 0;
    bool timed = false;  // ev0/ev1 bracket this session's last launch
    LaunchShape shape{0, 0};
    cudaGraphExec_t gexec = nullptr;  // respin graph (mmcgb_session_launch_repeat) and its shape
    uint64_t g_nphoton = 0;
    int g_repeats = 0;
    PhaseQueue pq[2] = {};            // gate-phased tracing queues, capacity pq_cap photons each
    unsigned* pq_order = nullptr;     // spatial resume order (pq_cap entries), null beyond 2^32 photons
    unsigned* pq_bucket = nullptr;    // 2 * kBuckets counters
    void* pq_mem = nullptr;
    uint64_t pq_cap = 0;
    int pq_span = 0;                  // gates per phased launch
};

namespace {

void free_mesh_device(mmcgb_mesh* m) {
    if (m->rec) cudaFree(m->rec);
    if (m->elem) cudaFree(m->elem);
    if (m->node) cudaFree(m->node);
    if (m->label) cudaFree(m->label);
    if (m->evol) cudaFree(m->evol);
    if (m->loc_start) cudaFree(m->loc_start);
    if (m->loc_items) cudaFree(m->loc_items);
    m->evol = nullptr;
    m->loc_start = nullptr;
    m->loc_items = nullptr;
    m->rec = nullptr;
    m->elem = nullptr;
    m->node = nullptr;
    m->label = nullptr;
}

}  // namespace

extern "C" {

int32_t mmcgb_abi_version(void) { return MMCGB_ABI_VERSION; }

const char* mmcgb_last_error(void) { return g_err.c_str(); }

void mmcgb_config_defaults(mmcgb_config* c) {
    std::memset(c, 0, sizeof(*c));
    c->seed = 0x623F9A9E;
    c->srcdir[2] = 1.f;
    c->tstart = 0.f;
    c->tend = 5e-9f;
    c->tstep = 5e-9f;
    c->isreflect = 1;
    c->isnormalized = 1;
    c->basisorder = 1;
    c->minenergy = 1e-6f;
    c->roulettesize = 10.f;
    c->nout = 1.f;
    c->unitinmm = 1.f;
    c->outputtype = MMCGB_OUT_FLUX;
    c->maxdetphoton = 1000000;
    c->accum_f64 = 1;
    c->fast_math = 1;
    c->srcnum = 1;
}

int32_t mmcgb_mesh_create(const mmcgb_mesh_desc* desc, int32_t device, mmcgb_mesh** out) {
    if (!desc || !out) return fail(MMCGB_E_ARG, "null argument");
    *out = nullptr;
    std::unique_ptr<mmcgb_mesh> m(new mmcgb_mesh());
    std::string err;
    int rc = prepare_mesh(*desc, m->host, err);
    if (rc) return fail(rc, err);
    m->device = device;
    CK(cudaSetDevice(device));
    {
        // Simulations allocate their buffers stream-ordered from the device's default pool
        // (fluence, records, gate-phase queues of tens of GB); keep up to 32 GB of freed blocks
        // in the pool instead of returning them at every synchronization, so repeated
        // simulate() calls reuse them.  A setting of this process's pool only.
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
            uint64_t keep = 32ull << 30;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        (void)cudaGetLastError();
    }
    std::vector<TetRec> rec;
    pack_records(m->host, rec);
    std::vector<float4> node(m->host.nn);
    for (int a = 0; a < 3; a++) {
        m->lo[a] = m->host.nn ? m->host.node[a] : 0.f;
        m->hi[a] = m->lo[a];
    }
    for (int i = 0; i < m->host.nn; i++) {
        node[i] = make_float4(m->host.node[3 * (size_t)i], m->host.node[3 * (size_t)i + 1], m->host.node[3 * (size_t)i + 2], 0.f);
        for (int a = 0; a < 3; a++) {
            m->lo[a] = std::min(m->lo[a], m->host.node[3 * (size_t)i + a]);
            m->hi[a] = std::max(m->hi[a], m->host.node[3 * (size_t)i + a]);
        }
    }
    cudaError_t e;
    if ((e = cudaMalloc((void**)&m->rec, sizeof(TetRec) * rec.size())) != cudaSuccess ||
        (e = cudaMalloc((void**)&m->elem, sizeof(int4) * m->host.ne)) != cudaSuccess ||
        (e = cudaMalloc((void**)&m->node, sizeof(float4) * m->host.nn)) != cudaSuccess ||
        (e = cudaMalloc((void**)&m->label, sizeof(int) * m->host.ne)) != cudaSuccess ||
        (e = cudaMalloc((void**)&m->evol, sizeof(float) * m->host.ne)) != cudaSuccess ||
        (e = cudaMemcpy(m->evol, m->host.evol.data(), sizeof(float) * m->host.ne, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(m->rec, rec.data(), sizeof(TetRec) * rec.size(), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(m->elem, m->host.elem.data(), sizeof(int4) * m->host.ne, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(m->node, node.data(), sizeof(float4) * m->host.nn, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(m->label, m->host.label.data(), sizeof(int) * m->host.ne, cudaMemcpyHostToDevice)) != cudaSuccess) {
        free_mesh_device(m.get());
        return cuda_fail(e, "mesh upload");
    }
    *out = m.release();
    return MMCGB_OK;
}

int32_t mmcgb_mesh_destroy(mmcgb_mesh* m) {
    if (!m) return MMCGB_OK;
    cudaSetDevice(m->device);
    cudaDeviceSynchronize();  // no launch still reading the records outlives them
    free_mesh_device(m);
    delete m;
    return MMCGB_OK;
}

int32_t mmcgb_mesh_info(const mmcgb_mesh* m, int32_t* nn, int32_t* ne, int32_t* nf) {
    if (!m) return fail(MMCGB_E_ARG, "null mesh");
    if (nn) *nn = m->host.nn;
    if (ne) *ne = m->host.ne;
    if (nf) *nf = m->host.nf;
    return MMCGB_OK;
}

int32_t mmcgb_mesh_export(const mmcgb_mesh* m, int32_t* elem, int32_t* facenb, float* evol, float* nvol) {
    if (!m) return fail(MMCGB_E_ARG, "null mesh");
    const HostMesh& h = m->host;
    if (elem) std::memcpy(elem, h.elem.data(), sizeof(int) * h.elem.size());
    if (facenb) std::memcpy(facenb, h.facenb.data(), sizeof(int) * h.facenb.size());
    if (evol) std::memcpy(evol, h.evol.data(), sizeof(float) * h.evol.size());
    if (nvol) std::memcpy(nvol, h.nvol.data(), sizeof(float) * h.nvol.size());
    return MMCGB_OK;
}

int32_t mmcgb_mesh_locate(const mmcgb_mesh* m, const float p[3]) {
    if (!m || !p) return 0;
    return locate(m->host, p);
}

int32_t mmcgb_session_begin(mmcgb_mesh* mesh, const mmcgb_config* cfg, mmcgb_result* trace, mmcgb_session** out) {
    if (!mesh || !cfg || !out) return fail(MMCGB_E_ARG, "null argument");
    *out = nullptr;
    CK(cudaSetDevice(mesh->device));
    std::unique_ptr<mmcgb_session> s(new mmcgb_session());
    s->mesh = mesh;
    s->cfg = *cfg;
    CK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    int rc = prepare_sim(mesh, *cfg, trace, s->stream, s->P);
    if (rc == MMCGB_OK) {
        cudaError_t e = cudaMallocAsync((void**)&s->work, sizeof(unsigned long long), s->stream);
        if (e == cudaSuccess) e = cudaEventCreate(&s->ev0);
        if (e == cudaSuccess) e = cudaEventCreate(&s->ev1);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ready, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(s->ready, s->stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "session setup");
    }
    if (rc) {
        s->P.buf.release();
        if (s->work) cudaFreeAsync(s->work, s->stream);
        cudaStreamSynchronize(s->stream);
        for (cudaEvent_t ev : {s->ev0, s->ev1, s->ready})
            if (ev) cudaEventDestroy(ev);
        cudaStreamDestroy(s->stream);
        return rc;
    }
    s->shape = default_shape(mesh->device, false);
    if (cfg->threads > 0) s->shape.threads = std::max(32, std::min(cfg->threads, 128) / 32 * 32);
    if (cfg->blocks > 0) s->shape.blocks = cfg->blocks;
    *out = s.release();
    return MMCGB_OK;
}

}  // extern "C"

namespace {

// The window of automatic gate phasing: the live gate planes (window + 1 of
// them) fill about 70% of the L2, leaving the rest to the tet records.
// Measured on the 1.296M-tet, 50-gate benchmark (10.4 MB planes, photons
// resumed in spatial order, 1e8 photons): windows of 5, 6, 7, 8, 9, 10 and 12
// gates ran at 103.0k, 103.8k, 104.2k, 104.4k, 104.4k, 103.4k and 95.9k
// photons/ms (one launch: 59.4k).
int auto_window(int device, size_t plane_bytes) {
    int l2 = 0;
    cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, device);
    return std::max(1, (int)(0.75 * (double)l2 / (double)plane_bytes) - 1);
}

// How a launch of `nphoton` photons of this session is traced: `span` gates
// per phased launch (0 = one unphased launch) and `chunk` photons per phased
// launch.  Automatic phasing engages for >= 8 gates, >= 64 MB of fluence and
// >= 4e6 photons.  The parked states of a phased launch's photons are
// double-buffered queues (phase_bytes_per_photon each, plus a resume-order
// index); when those for all the photons would not fit in half of the free
// device memory the launch is split into phased launches of as many photons
// as fit (mmcgb_config.phase_chunk caps them further).  Automatic phasing
// needs >= 4e6 photons per such launch, else the launch runs unphased.
struct PhasePlan {
    int span = 0;
    uint64_t chunk = 0;
};

PhasePlan phase_plan(const mmcgb_session* s, uint64_t nphoton) {
    PhasePlan plan;
    const mmcgb_config& c = s->cfg;
    if (nphoton == 0 || c.phased < 0 || c.replayseed || s->P.maxgate < 2) return plan;
    int span = c.phased;
    if (span == 0) {
        const size_t plane = s->P.flen / (size_t)s->P.maxgate * (c.accum_f64 ? 8 : 4);
        span = auto_window(s->mesh->device, plane);
        const size_t fluence = s->P.flen * 8;
        if (s->P.maxgate < 8 || fluence < ((size_t)64 << 20) || nphoton < 4000000ull || span >= s->P.maxgate)
            return plan;
    }
    uint64_t chunk = std::min<uint64_t>(nphoton, 0xFFFFFFFFull);  // the resume order holds 32-bit indices
    // per-photon trace outputs are indexed by the photon's place in its kernel launch: one launch
    const bool traced = s->P.buf.pw || s->P.buf.ps || s->P.buf.pd;
    if (c.phase_chunk > 0 && !traced) chunk = std::min<uint64_t>(chunk, c.phase_chunk);
    if (chunk > s->pq_cap && !traced) {
        const size_t per = phase_bytes_per_photon(s->P.sim) + sizeof(unsigned);
        const size_t fixed = sizeof(unsigned) * 2 * kBuckets + 16 * 256;
        const size_t avail = free_device_memory(s->mesh->device) / 2;
        const uint64_t fit = avail > fixed ? (uint64_t)((avail - fixed) / per) : 0;
        if (fit < chunk) {
            // a forced window still tries a modest queue (and reports E_NOMEM if even that fails)
            chunk = std::max<uint64_t>({fit, s->pq_cap, c.phased > 0 ? std::min<uint64_t>(nphoton, 1u << 20) : 0});
        }
    }
    if (chunk == 0 || (c.phased == 0 && chunk < 4000000ull)) return plan;
    const uint64_t parts = (nphoton + chunk - 1) / chunk;
    plan.chunk = (nphoton + parts - 1) / parts;  // equal parts
    plan.span = span;
    return plan;
}

// Allocates the gate-phased queues for `chunk` photons per launch (kept for
// later launches that need no more).  Returns a status.
int phased_setup(mmcgb_session* s, const PhasePlan& plan) {
    s->pq_span = plan.span;
    const uint64_t n = plan.chunk;
    if (n <= s->pq_cap) return MMCGB_OK;
    const size_t per = phase_bytes_per_photon(s->P.sim) + sizeof(unsigned);
    const size_t need = per * n + sizeof(unsigned) * 2 * kBuckets + 16 * 256;
    if (s->pq_mem) CK(cudaFreeAsync(s->pq_mem, s->stream));
    s->pq_mem = nullptr;
    s->pq_cap = 0;
    cudaError_t e = cudaMallocAsync(&s->pq_mem, need, s->stream);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return fail(MMCGB_E_NOMEM, "no device memory for the gate-phased queues");
    }
    s->pq_cap = n;
    const SimDev& sim = s->P.sim;
    const bool want_seed = sim.issavedet && sim.seeds;
    char* p = static_cast<char*>(s->pq_mem);
    auto take = [&](size_t bytes) {
        char* r = p;
        p += (bytes + 255) & ~(size_t)255;
        return r;
    };
    for (int i = 0; i < 2; i++) {
        s->pq[i].rec = reinterpret_cast<PState*>(take(sizeof(PState) * n));
        s->pq[i].ppath = sim.issavedet ? reinterpret_cast<float*>(take(sizeof(float) * sim.reclen * n)) : nullptr;
        s->pq[i].seed0 = want_seed ? reinterpret_cast<unsigned long long*>(take(16 * n)) : nullptr;
        s->pq[i].count = reinterpret_cast<unsigned long long*>(take(sizeof(unsigned long long)));
    }
    s->pq_order = reinterpret_cast<unsigned*>(take(sizeof(unsigned) * n));
    s->pq_bucket = reinterpret_cast<unsigned*>(take(sizeof(unsigned) * 2 * kBuckets));
    return MMCGB_OK;
}

}  // namespace

extern "C" {

namespace {

// The replicated near-source cells of an unbatched session, allocated at its first launch:
// kHotReps copies of the gate-0 plane, when they take at most 2 GiB and fit in free memory.
// A session without them deposits into the cells themselves (same sums, other order).
int ensure_hot(mmcgb_session* s) {
    Prepared& P = s->P;
    if (!P.hot_ok || P.buf.hot) return MMCGB_OK;
    P.hot_ok = false;  // one attempt
    const size_t n = (size_t)kHotReps * (size_t)P.sim.ne;
    if (n * sizeof(double) > (2ull << 30) ||
        n * sizeof(double) + (256ull << 20) > free_device_memory(s->mesh->device))
        return MMCGB_OK;
    if (P.buf.alloc(&P.buf.hot, n) != cudaSuccess) {
        (void)cudaGetLastError();
        P.buf.hot = nullptr;
        return MMCGB_OK;
    }
    CK(cudaMemsetAsync(P.buf.hot, 0, sizeof(double) * n, s->stream));
    P.sim.hot = P.buf.hot;
    P.sim.hot_steps = kHotSteps;
    return MMCGB_OK;
}

}  // namespace

int32_t mmcgb_session_launch(mmcgb_session* s, uint64_t photon_offset, uint64_t nphoton) {
    if (!s) return fail(MMCGB_E_ARG, "null session");
    if (s->cfg.replayseed && (photon_offset != 0 || nphoton != s->cfg.nphoton))
        return fail(MMCGB_E_ARG, "replay sessions run all replayed photons in one launch");
    if ((s->P.buf.pw || s->P.buf.ps || s->P.buf.pd) && nphoton > s->cfg.nphoton)
        return fail(MMCGB_E_ARG, "per-photon trace buffers hold cfg.nphoton photons");
    CK(cudaSetDevice(s->mesh->device));
    if (const int rc = ensure_hot(s)) return rc;
    SimDev sim = s->P.sim;
    sim.nphoton = nphoton;
    sim.photon_offset = s->cfg.photon_offset + photon_offset;
    const PhasePlan plan = phase_plan(s, nphoton);
    if (plan.span > 0) {
        const int rc = phased_setup(s, plan);
        if (rc) return rc;
    }
    CK(cudaEventRecord(s->ev0, s->stream));
    if (plan.span > 0) {
        for (uint64_t off = 0; off < nphoton; off += plan.chunk) {  // photon ranges whose queues fit
            SimDev part = sim;
            part.photon_offset = sim.photon_offset + off;
            part.nphoton = std::min<uint64_t>(plan.chunk, nphoton - off);
            CK(launch_phased(part, s->work, s->shape, s->stream, s->pq, s->pq_span, s->pq_order, s->pq_bucket,
                             s->mesh->lo, s->mesh->hi));
        }
    } else {
        CK(launch_plain(sim, s->work, s->shape, s->stream));
    }
    CK(fold_hot(sim, s->stream));
    CK(cudaEventRecord(s->ev1, s->stream));
    s->launched += nphoton;
    s->launches++;
    s->timed = true;
    return MMCGB_OK;
}

}  // extern "C"

namespace {

// The parameter blocks and photon-count prefix sums of one batched launch over
// sessions ss[0..n) (session i simulating photons [offsets[i], offsets[i]+counts[i])
// of its run), with what the kernel needs to know about them.
struct BatchPlan {
    std::vector<SimDev> sims;
    std::vector<unsigned long long> cum;
    unsigned long long total = 0;
    int nmed_stride = 0, reclen_max = 0, want_seed = 0, want_io = 0, want_replay = 0, fast = 0;
};

int plan_batch(int32_t n, mmcgb_session* const* ss, const uint64_t* offsets, const uint64_t* counts, BatchPlan& B) {
    if (n <= 0 || !ss || !offsets || !counts || !ss[0]) return fail(MMCGB_E_ARG, "null or empty batch");
    const int device = ss[0]->mesh->device;
    B.fast = ss[0]->cfg.fast_math ? 1 : 0;
    B.sims.resize(n);
    B.cum.resize(n);
    for (int i = 0; i < n; i++) {
        mmcgb_session* s = ss[i];
        if (!s || s->mesh->device != device) return fail(MMCGB_E_ARG, "batched sessions must live on one device");
        if ((s->cfg.fast_math ? 1 : 0) != B.fast) return fail(MMCGB_E_ARG, "batched sessions must share fast_math");
        if (s->cfg.replayseed && (offsets[i] != 0 || counts[i] != s->cfg.nphoton))
            return fail(MMCGB_E_ARG, "replay sessions run all replayed photons in one launch");
        if ((s->P.buf.pw || s->P.buf.ps || s->P.buf.pd) && counts[i] > s->cfg.nphoton)
            return fail(MMCGB_E_ARG, "per-photon trace buffers hold cfg.nphoton photons");
        B.sims[i] = s->P.sim;
        B.sims[i].hot_steps = 0;  // batched launches deposit into the cells themselves
        B.sims[i].nphoton = counts[i];
        B.sims[i].photon_offset = s->cfg.photon_offset + offsets[i];
        B.nmed_stride = std::max(B.nmed_stride, s->cfg.nmedia);
        if (s->cfg.issavedet) B.reclen_max = std::max(B.reclen_max, s->P.sim.reclen);
        if (s->cfg.issavedet && s->P.sim.seeds) B.want_seed = 1;
        if (general_source(s->P.sim) || s->P.sim.roulette_on) B.want_io = 1;  // batched kernels: lean or general
        if (s->P.sim.replay) B.want_replay = 1;
        B.total += counts[i];
        B.cum[i] = B.total;
    }
    if ((size_t)n * B.nmed_stride * sizeof(float4) > 40 * 1024)
        return fail(MMCGB_E_ARG, "batch media tables exceed shared memory; split the batch");
    return MMCGB_OK;
}

// Instantiated graphs of mmcgb_session_launch_batches, one per device: a new
// capture of the same shape (the same number of launches of the same kernels)
// updates the instantiated graph in place instead of instantiating again.
// The executable graphs live until the process exits.
std::mutex g_graph_mu;
std::map<int, cudaGraphExec_t> g_graph_exec;

cudaError_t launch_cached_graph(int device, cudaGraph_t graph, cudaStream_t st) {
    std::lock_guard<std::mutex> lk(g_graph_mu);
    cudaGraphExec_t& ex = g_graph_exec[device];
    if (ex) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(ex, graph, &info) != cudaSuccess) {
            (void)cudaGetLastError();
            cudaGraphExecDestroy(ex);
            ex = nullptr;
        }
    }
    if (!ex) {
        const cudaError_t e = cudaGraphInstantiate(&ex, graph, 0);
        if (e != cudaSuccess) {
            ex = nullptr;
            return e;
        }
    }
    return cudaGraphLaunch(ex, st);
}

// One persistent launch over several sessions.  `ordered`: on the first
// session's stream, after every session's earlier work and before its later
// work, timed with the first session's events.  Otherwise on `st` with its own
// work counter and no ordering against the sessions' streams.
int batch_launch(int32_t n, mmcgb_session* const* ss, const uint64_t* offsets, const uint64_t* counts,
                 cudaStream_t st, bool ordered) {
    if (n <= 0 || !ss || !offsets || !counts) return fail(MMCGB_E_ARG, "null or empty batch");
    mmcgb_session* s0 = ss[0];
    if (!s0) return fail(MMCGB_E_ARG, "null session");
    const int device = s0->mesh->device;
    BatchPlan B;
    int rc = plan_batch(n, ss, offsets, counts, B);
    if (rc) return rc;
    std::vector<SimDev>& sims = B.sims;
    std::vector<unsigned long long>& cum = B.cum;
    const unsigned long long total = B.total;
    const int nmed_stride = B.nmed_stride, reclen_max = B.reclen_max, want_seed = B.want_seed,
              want_io = B.want_io, want_replay = B.want_replay, fast = B.fast;
    CK(cudaSetDevice(device));
    if (ordered) st = s0->stream;
    // order the batch after every session's earlier work, and every session's later work after it
    std::vector<cudaEvent_t> evs;
    // unordered: only after each session's setup (buffer allocation and zeroing, table uploads)
    for (int i = 0; !ordered && i < n; i++) CK(cudaStreamWaitEvent(st, ss[i]->ready, 0));
    for (int i = 1; ordered && i < n; i++) {
        if (ss[i]->stream == st) continue;
        cudaEvent_t e;
        CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        evs.push_back(e);
        CK(cudaEventRecord(e, ss[i]->stream));
        CK(cudaStreamWaitEvent(st, e, 0));
    }
    SimDev* dsims = nullptr;
    unsigned long long* dcum = nullptr;
    unsigned long long* work = ordered ? s0->work : nullptr;
    CK(cudaMallocAsync((void**)&dsims, sizeof(SimDev) * n, st));
    CK(cudaMallocAsync((void**)&dcum, sizeof(unsigned long long) * n, st));
    if (!ordered) CK(cudaMallocAsync((void**)&work, sizeof(unsigned long long), st));
    CK(cudaMemcpyAsync(dsims, sims.data(), sizeof(SimDev) * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dcum, cum.data(), sizeof(unsigned long long) * n, cudaMemcpyHostToDevice, st));
    LaunchShape shape = default_shape(device, true);
    if (s0->cfg.threads > 0) shape.threads = std::max(32, std::min(s0->cfg.threads, 128) / 32 * 32);
    if (s0->cfg.blocks > 0) shape.blocks = s0->cfg.blocks;
    if (ordered) CK(cudaEventRecord(s0->ev0, st));
    if (n == 1)  // a single simulation takes the plain kernel (its parameter block in constant memory)
        CK(launch_plain(sims[0], work, s0->shape, st));
    else
        CK(launch_batched(dsims, dcum, n, total, nmed_stride, reclen_max, want_seed, work, shape, st, fast, want_io,
                          want_replay));
    if (ordered) CK(cudaEventRecord(s0->ev1, st));
    CK(cudaFreeAsync(dsims, st));
    CK(cudaFreeAsync(dcum, st));
    if (!ordered) CK(cudaFreeAsync(work, st));
    // every session's later work (sync, output stage, freeing its buffers) waits for this launch;
    // unordered launches never wait on the session streams, so they still overlap one another
    cudaEvent_t done = nullptr;
    CK(cudaEventCreateWithFlags(&done, cudaEventDisableTiming));
    CK(cudaEventRecord(done, st));
    for (int i = 0; i < n; i++) {
        ss[i]->launched += counts[i];
        ss[i]->launches++;
        ss[i]->timed = ordered && (i == 0);  // the batch is timed on the first session's events
        if (ss[i]->stream != st) CK(cudaStreamWaitEvent(ss[i]->stream, done, 0));
    }
    for (cudaEvent_t e : evs) cudaEventDestroy(e);
    if (done) cudaEventDestroy(done);
    return MMCGB_OK;
}

}  // namespace

extern "C" {

int32_t mmcgb_session_launch_batch(int32_t n, mmcgb_session* const* ss, const uint64_t* offsets,
                                   const uint64_t* counts) {
    return batch_launch(n, ss, offsets, counts, nullptr, true);
}

int32_t mmcgb_session_launch_batch_on(int32_t n, mmcgb_session* const* ss, const uint64_t* offsets,
                                      const uint64_t* counts, void* stream) {
    if (!stream) return fail(MMCGB_E_ARG, "null stream");
    return batch_launch(n, ss, offsets, counts, (cudaStream_t)stream, false);
}

int32_t mmcgb_session_launch_batches(int32_t ngroups, const int32_t* group_sizes, mmcgb_session* const* ss,
                                     const uint64_t* offsets, const uint64_t* counts, void* stream_handle) {
    if (ngroups <= 0 || !group_sizes || !ss || !offsets || !counts || !stream_handle)
        return fail(MMCGB_E_ARG, "null or empty group list");
    cudaStream_t st = static_cast<cudaStream_t>(stream_handle);
    // plan every group before anything is enqueued
    std::vector<BatchPlan> plans(ngroups);
    std::vector<int> first(ngroups);
    int nsess = 0;
    for (int g = 0; g < ngroups; g++) {
        if (group_sizes[g] <= 0) return fail(MMCGB_E_ARG, "every group needs a session");
        first[g] = nsess;
        const int rc = plan_batch(group_sizes[g], ss + nsess, offsets + nsess, counts + nsess, plans[g]);
        if (rc) return rc;
        nsess += group_sizes[g];
    }
    const int device = ss[0]->mesh->device;
    for (int i = 0; i < nsess; i++)
        if (ss[i]->mesh->device != device) return fail(MMCGB_E_ARG, "batched sessions must live on one device");
    CK(cudaSetDevice(device));
    // one device buffer holds every group's parameter blocks, prefix sums and work counter
    size_t bytes = 0;
    std::vector<size_t> off_sims(ngroups), off_cum(ngroups), off_work(ngroups);
    for (int g = 0; g < ngroups; g++) {
        off_sims[g] = bytes;
        bytes += (sizeof(SimDev) * group_sizes[g] + 255) & ~(size_t)255;
        off_cum[g] = bytes;
        bytes += (sizeof(unsigned long long) * group_sizes[g] + 255) & ~(size_t)255;
        off_work[g] = bytes;
        bytes += 256;
    }
    std::vector<unsigned char> host(bytes, 0);
    for (int g = 0; g < ngroups; g++) {
        std::memcpy(host.data() + off_sims[g], plans[g].sims.data(), sizeof(SimDev) * group_sizes[g]);
        std::memcpy(host.data() + off_cum[g], plans[g].cum.data(), sizeof(unsigned long long) * group_sizes[g]);
    }
    const LaunchShape bshape = default_shape(device, true);
    // the groups run after every session's setup
    for (int i = 0; i < nsess; i++) CK(cudaStreamWaitEvent(st, ss[i]->ready, 0));
    unsigned char* dev = nullptr;
    CK(cudaMallocAsync((void**)&dev, bytes, st));
    cudaError_t e = cudaMemcpyAsync(dev, host.data(), bytes, cudaMemcpyHostToDevice, st);
    // the launches, captured as one graph (each zeroes its own work counter first)
    if (e == cudaSuccess) e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaFreeAsync(dev, st);
        return cuda_fail(e, "batched graph capture");
    }
    for (int g = 0; g < ngroups && e == cudaSuccess; g++) {
        const BatchPlan& B = plans[g];
        mmcgb_session* s0 = ss[first[g]];
        auto* work = reinterpret_cast<unsigned long long*>(dev + off_work[g]);
        if (group_sizes[g] == 1) {
            e = launch_plain(B.sims[0], work, s0->shape, st);
        } else {
            LaunchShape shape = bshape;
            if (s0->cfg.threads > 0) shape.threads = std::max(32, std::min(s0->cfg.threads, 128) / 32 * 32);
            if (s0->cfg.blocks > 0) shape.blocks = s0->cfg.blocks;
            e = launch_batched(reinterpret_cast<const SimDev*>(dev + off_sims[g]),
                               reinterpret_cast<const unsigned long long*>(dev + off_cum[g]), group_sizes[g], B.total,
                               B.nmed_stride, B.reclen_max, B.want_seed, work, shape, st, B.fast, B.want_io,
                               B.want_replay);
        }
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(st, &graph);
    if (e == cudaSuccess) e = ec;
    if (e == cudaSuccess) e = launch_cached_graph(device, graph, st);
    if (graph) cudaGraphDestroy(graph);
    cudaFreeAsync(dev, st);
    if (e != cudaSuccess) return cuda_fail(e, "batched graph");
    // every session's later work (sync, output stage, freeing its buffers) waits for the groups
    cudaEvent_t done = nullptr;
    CK(cudaEventCreateWithFlags(&done, cudaEventDisableTiming));
    CK(cudaEventRecord(done, st));
    for (int i = 0; i < nsess; i++) {
        ss[i]->launched += counts[i];
        ss[i]->launches++;
        ss[i]->timed = false;
        if (ss[i]->stream != st) CK(cudaStreamWaitEvent(ss[i]->stream, done, 0));
    }
    cudaEventDestroy(done);
    return MMCGB_OK;
}

int32_t mmcgb_session_launch_repeat(mmcgb_session* s, uint64_t photon_offset, uint64_t nphoton, int32_t repeats) {
    if (!s) return fail(MMCGB_E_ARG, "null session");
    if (repeats < 1 || nphoton == 0) return fail(MMCGB_E_ARG, "repeats and nphoton must be positive");
    if (s->cfg.replayseed) return fail(MMCGB_E_ARG, "replay sessions run all replayed photons in one launch");
    if ((s->P.buf.pw || s->P.buf.ps || s->P.buf.pd) && nphoton * (uint64_t)repeats > s->cfg.nphoton)
        return fail(MMCGB_E_ARG, "per-photon trace buffers hold cfg.nphoton photons");
    CK(cudaSetDevice(s->mesh->device));
    if (const int rc = ensure_hot(s)) return rc;  // allocates outside the capture
    CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < repeats && e == cudaSuccess; k++) {
        SimDev sim = s->P.sim;
        sim.nphoton = nphoton;
        sim.photon_offset = s->cfg.photon_offset + photon_offset + (uint64_t)k * nphoton;
        e = launch_plain(sim, s->work, s->shape, s->stream);
    }
    if (e == cudaSuccess) e = fold_hot(s->P.sim, s->stream);
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(s->stream, &g);
    if (e == cudaSuccess) e = ec;
    if (e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return cuda_fail(e, "respin graph capture");
    }
    if (s->gexec && (s->g_nphoton != nphoton || s->g_repeats != repeats)) {
        cudaGraphExecDestroy(s->gexec);
        s->gexec = nullptr;
    }
    if (s->gexec) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(s->gexec, g, &info) != cudaSuccess) {
            (void)cudaGetLastError();
            cudaGraphExecDestroy(s->gexec);
            s->gexec = nullptr;
        }
    }
    if (!s->gexec) {
        e = cudaGraphInstantiate(&s->gexec, g, 0);
        if (e != cudaSuccess) {
            cudaGraphDestroy(g);
            s->gexec = nullptr;
            return cuda_fail(e, "respin graph instantiation");
        }
        s->g_nphoton = nphoton;
        s->g_repeats = repeats;
    }
    cudaGraphDestroy(g);
    CK(cudaEventRecord(s->ev0, s->stream));
    CK(cudaGraphLaunch(s->gexec, s->stream));
    CK(cudaEventRecord(s->ev1, s->stream));
    s->launched += nphoton * (uint64_t)repeats;
    s->launches += repeats;
    s->timed = true;
    return MMCGB_OK;
}

void* mmcgb_session_stream(mmcgb_session* s) { return s ? (void*)s->stream : nullptr; }

int32_t mmcgb_session_phase_window(mmcgb_session* s, uint64_t nphoton, int32_t* window, uint64_t* chunk) {
    if (!s || !window) return fail(MMCGB_E_ARG, "null argument");
    CK(cudaSetDevice(s->mesh->device));
    const PhasePlan plan = phase_plan(s, nphoton);
    *window = plan.span;
    if (chunk) *chunk = plan.chunk;
    return MMCGB_OK;
}

int32_t mmcgb_session_device_buffers(mmcgb_session* s, mmcgb_device_out* out) {
    if (!s || !out) return fail(MMCGB_E_ARG, "null argument");
    const SimBuffers& B = s->P.buf;
    out->field_raw = B.f64;
    out->detp = B.detp;
    out->seeds = reinterpret_cast<uint8_t*>(B.seeds);
    out->detcount = B.detcount;
    out->energy = B.energy;
    out->counters = reinterpret_cast<uint64_t*>(B.counters);
    out->energy_src = B.energy_src;
    return MMCGB_OK;
}

int32_t mmcgb_session_sync(mmcgb_session* s, float* last_kernel_ms) {
    if (!s) return fail(MMCGB_E_ARG, "null session");
    CK(cudaSetDevice(s->mesh->device));
    CK(cudaStreamSynchronize(s->stream));
    if (last_kernel_ms) {
        *last_kernel_ms = 0.f;
        if (s->timed) CK(cudaEventElapsedTime(last_kernel_ms, s->ev0, s->ev1));
    }
    return MMCGB_OK;
}

int32_t mmcgb_session_end(mmcgb_session* s, mmcgb_result* res) {
    if (!s) return fail(MMCGB_E_ARG, "null session");
    cudaSetDevice(s->mesh->device);
    int rc = MMCGB_OK;
    if (res) {
        rc = finish_sim(s->mesh, s->cfg, s->P, res, s->stream, s->launched);
        float ms = 0.f;
        if (s->timed && cudaEventElapsedTime(&ms, s->ev0, s->ev1) == cudaSuccess) res->kernel_ms = ms;
    } else {
        s->P.buf.release();
    }
    if (s->work) cudaFreeAsync(s->work, s->stream);
    if (s->pq_mem) cudaFreeAsync(s->pq_mem, s->stream);
    cudaStreamSynchronize(s->stream);
    if (s->gexec) cudaGraphExecDestroy(s->gexec);
    cudaEventDestroy(s->ev0);
    cudaEventDestroy(s->ev1);
    if (s->ready) cudaEventDestroy(s->ready);
    cudaStreamDestroy(s->stream);
    delete s;
    return rc;
}

int32_t mmcgb_simulate(mmcgb_mesh* mesh, const mmcgb_config* cfg, mmcgb_result* res) {
    if (!mesh || !cfg || !res) return fail(MMCGB_E_ARG, "null argument");
    mmcgb_session* s = nullptr;
    int rc = mmcgb_session_begin(mesh, cfg, res, &s);
    if (rc) return rc;
    rc = mmcgb_session_launch(s, 0, cfg->nphoton);
    if (rc) {
        std::string msg = g_err;
        mmcgb_session_end(s, nullptr);
        return fail(rc, msg);
    }
    return mmcgb_session_end(s, res);
}

int32_t mmcgb_simulate_batch(int32_t n, mmcgb_mesh* const* meshes, const mmcgb_config* cfgs, mmcgb_result* res) {
    if (n <= 0 || !meshes || !cfgs || !res) return fail(MMCGB_E_ARG, "null or empty batch");
    const int device = meshes[0]->device;
    for (int i = 0; i < n; i++)
        if (!meshes[i] || meshes[i]->device != device) return fail(MMCGB_E_ARG, "batched meshes must live on one device");
    CK(cudaSetDevice(device));
    cudaStream_t stream;
    CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    std::vector<Prepared> P(n);
    int rc = MMCGB_OK;
    int nmed_stride = 0, reclen_max = 0, want_seed = 0, want_io = 0, want_replay = 0;
    std::vector<unsigned long long> cum(n);
    unsigned long long total = 0;
    for (int i = 0; i < n && rc == MMCGB_OK; i++) {
        rc = prepare_sim(meshes[i], cfgs[i], &res[i], stream, P[i]);
        if (rc) break;
        nmed_stride = std::max(nmed_stride, cfgs[i].nmedia);
        if (cfgs[i].issavedet) reclen_max = std::max(reclen_max, P[i].sim.reclen);
        if (cfgs[i].issavedet && cfgs[i].issaveseed) want_seed = 1;
        if (general_source(P[i].sim) || P[i].sim.roulette_on) want_io = 1;
        if (P[i].sim.replay) want_replay = 1;
        if ((cfgs[i].fast_math != 0) != (cfgs[0].fast_math != 0)) {
            rc = fail(MMCGB_E_ARG, "batched simulations must share fast_math");
            break;
        }
        total += cfgs[i].nphoton;
        cum[i] = total;
    }
    if (rc == MMCGB_OK && (size_t)n * nmed_stride * 16 > 40 * 1024) rc = fail(MMCGB_E_ARG, "batch media tables exceed shared memory; split the batch");
    SimDev* dsims = nullptr;
    unsigned long long* dcum = nullptr;
    unsigned long long* work = nullptr;
    cudaEvent_t ev0, ev1;
    cudaEventCreate(&ev0);
    cudaEventCreate(&ev1);
    if (rc == MMCGB_OK) {
        std::vector<SimDev> sims(n);
        for (int i = 0; i < n; i++) {
            sims[i] = P[i].sim;
            sims[i].hot_steps = 0;  // batched launches deposit into the cells themselves
        }
        cudaError_t e = cudaMallocAsync((void**)&dsims, sizeof(SimDev) * n, stream);
        if (e == cudaSuccess) e = cudaMallocAsync((void**)&dcum, sizeof(unsigned long long) * n, stream);
        if (e == cudaSuccess) e = cudaMallocAsync((void**)&work, sizeof(unsigned long long), stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dsims, sims.data(), sizeof(SimDev) * n, cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dcum, cum.data(), sizeof(unsigned long long) * n, cudaMemcpyHostToDevice, stream);
        LaunchShape shape = default_shape(device, true);
        if (cfgs[0].threads > 0) shape.threads = std::max(32, std::min(cfgs[0].threads, 128) / 32 * 32);
        if (cfgs[0].blocks > 0) shape.blocks = cfgs[0].blocks;
        if (e == cudaSuccess) e = cudaEventRecord(ev0, stream);
        if (e == cudaSuccess)
            e = launch_batched(dsims, dcum, n, total, nmed_stride, reclen_max, want_seed, work, shape, stream,
                               cfgs[0].fast_math ? 1 : 0, want_io, want_replay);
        if (e == cudaSuccess) e = cudaEventRecord(ev1, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "batched photon engine");
    }
    float ms = 0.f;
    if (rc == MMCGB_OK) cudaEventElapsedTime(&ms, ev0, ev1);
    for (int i = 0; i < n; i++) {
        if (rc == MMCGB_OK) {
            int r = finish_sim(meshes[i], cfgs[i], P[i], &res[i], stream, cfgs[i].nphoton);
            res[i].kernel_ms = ms;
            if (r) rc = r;
        } else {
            P[i].buf.release();
        }
    }
    if (dsims) cudaFreeAsync(dsims, stream);
    if (dcum) cudaFreeAsync(dcum, stream);
    if (work) cudaFreeAsync(work, stream);
    cudaStreamSynchronize(stream);
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    cudaStreamDestroy(stream);
    return rc;
}

int32_t mmcgb_prepare_host(const mmcgb_mesh_desc* desc, int32_t* elem, int32_t* facenb, float* normals, float* evol,
                           float* nvol, int32_t* nf) {
    if (!desc) return fail(MMCGB_E_ARG, "null argument");
    HostMesh h;
    std::string err;
    int rc = prepare_mesh(*desc, h, err);
    if (rc) return fail(rc, err);
    if (elem) std::memcpy(elem, h.elem.data(), sizeof(int) * h.elem.size());
    if (facenb) std::memcpy(facenb, h.facenb.data(), sizeof(int) * h.facenb.size());
    if (normals) element_normals_all(h, normals);
    if (evol) std::memcpy(evol, h.evol.data(), sizeof(float) * h.evol.size());
    if (nvol) std::memcpy(nvol, h.nvol.data(), sizeof(float) * h.nvol.size());
    if (nf) *nf = h.nf;
    return MMCGB_OK;
}

int32_t mmcgb_check_config(const mmcgb_mesh_desc* desc, const mmcgb_config* cfg, int32_t* e0) {
    if (!desc || !cfg) return fail(MMCGB_E_ARG, "null argument");
    HostMesh h;
    std::string err;
    int rc = prepare_mesh(*desc, h, err);
    if (rc) return fail(rc, err);
    rc = validate_config(h, *cfg, err);
    if (rc) return fail(rc, err);
    const int e = initial_element(h, *cfg);
    if (e <= 0 && point_source(cfg->srctype)) return fail(MMCGB_E_SOURCE, "initial element does not enclose the source");
    if (e0) *e0 = e;
    return MMCGB_OK;
}

int32_t mmcgb_normalize_host(const mmcgb_mesh_desc* desc, const mmcgb_config* cfg, const double* raw,
                             double energytot, double energyesc, double* field, double* normalizer) {
    if (!desc || !cfg || !raw || !field) return fail(MMCGB_E_ARG, "null argument");
    HostMesh h;
    std::string err;
    int rc = prepare_mesh(*desc, h, err);
    if (rc) return fail(rc, err);
    if (cfg->nmedia < 2 || !cfg->media || h.maxlabel > cfg->nmedia - 1) return fail(MMCGB_E_ARG, "media table does not cover the mesh labels");
    if (!(cfg->tstep > 0.f)) return fail(MMCGB_E_ARG, "tstep must be positive");
    if (cfg->method == 1) {  // dual-grid output: one scale factor, src/mmc_mesh.c:2204-2206
        const size_t n = frame_len(h, *cfg) * gates_of(*cfg);
        const double norm = grid_normalizer(*cfg, energytot);
        for (size_t i = 0; i < n; i++) field[i] = raw[i] * norm;
        if (normalizer) *normalizer = norm;
        return MMCGB_OK;
    }
    const double n = normalize_output(h, *cfg, gates_of(*cfg), raw, energytot, energyesc, field);
    if (normalizer) *normalizer = n;
    return MMCGB_OK;
}

int32_t mmcgb_grid_info(const mmcgb_mesh* m, float step, int32_t dim[3], float origin[3]) {
    if (!m || !dim) return fail(MMCGB_E_ARG, "null argument");
    if (!(step > 0.f)) return fail(MMCGB_E_ARG, "step must be positive");
    unsigned d[3];
    float o[3];
    grid_geometry(m->host, step, d, o);
    for (int k = 0; k < 3; k++) {
        dim[k] = (int32_t)d[k];
        if (origin) origin[k] = o[k];
    }
    return MMCGB_OK;
}

int32_t mmcgb_run(const mmcgb_mesh_desc* desc, const mmcgb_config* cfg, int32_t device, mmcgb_result* res) {
    mmcgb_mesh* m = nullptr;
    int rc = mmcgb_mesh_create(desc, device, &m);
    if (rc) return rc;
    rc = mmcgb_simulate(m, cfg, res);
    mmcgb_mesh_destroy(m);
    return rc;
}

}  // extern "C"

/*
 * mmcgb -- GB300-native per-photon tetrahedral tracing for Mesh-based Monte
 * Carlo (fangq/mmc).  C ABI of libmmcgb.so.
 *
 * The library replaces the reference's CUDA photon path, whose single entry is
 *     void mmc_run_cu(mcconfig* cfg, tetmesh* mesh, raytracer* tracer);
 * (src/mmc_cu_host.h:56, implemented as mmc_run_simulation in
 * src/mmc_cu_host.cu:204-1528).  That entry takes the whole reference config
 * and mesh structs, accumulates into cfg->exportfield and exits the process on
 * error.  Here the same work is split into plain-pointer calls:
 *
 *   mmcgb_mesh_create   mesh upload + ray-tracer precompute, kept resident on
 *                       the GPU (replaces the per-call uploads of
 *                       src/mmc_cu_host.cu:447-487 and tracer_build/tracer_prep,
 *                       src/mmc_mesh.c:1241-1602)
 *   mmcgb_simulate      one simulation on a resident mesh: launch, readback,
 *                       elem->node scatter and normalization
 *                       (src/mmc_cu_host.cu:642-995, src/mmc_mesh.c:2154-2279)
 *   mmcgb_simulate_batch  many simulations in one persistent launch
 *   mmcgb_run           one-shot create + simulate + destroy, the direct
 *                       counterpart of mmc_run_cu
 *
 * Every call returns an mmcgb_status; none exits the process.  The message of
 * the last failure on the calling thread is available from mmcgb_last_error().
 * All arrays are host memory owned by the caller unless stated otherwise.
 * Indices in node/elem/facenb follow the reference: 1-based, 0 = no neighbour.
 */
#ifndef MMCGB_H
#define MMCGB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MMCGB_ABI_VERSION 6

typedef enum mmcgb_status {
    MMCGB_OK = 0,
    MMCGB_E_ARG = 1,      /* invalid argument or configuration */
    MMCGB_E_CUDA = 2,     /* CUDA runtime error */
    MMCGB_E_MESH = 3,     /* malformed mesh (bad node id, too many elements) */
    MMCGB_E_SOURCE = 4,   /* no element encloses the source */
    MMCGB_E_BUDGET = 5,   /* photons stopped by the per-photon step budget */
    MMCGB_E_NOMEM = 6     /* not enough device memory for the requested outputs */
} mmcgb_status;

/* output quantity, same numbering as the reference's -O option */
typedef enum mmcgb_output {
    MMCGB_OUT_FLUX = 0, MMCGB_OUT_FLUENCE = 1, MMCGB_OUT_ENERGY = 2,
    MMCGB_OUT_JACOBIAN = 3, MMCGB_OUT_WL = 4, MMCGB_OUT_WP = 5
} mmcgb_output;

typedef struct mmcgb_mesh mmcgb_mesh; /* opaque, device-resident mesh */
typedef struct mmcgb_device_out mmcgb_device_out; /* device buffers, defined below */

/* Mesh input (tetmesh subset, src/mmc_mesh.h:87-122). */
typedef struct mmcgb_mesh_desc {
    int32_t nn;              /* nodes */
    int32_t ne;              /* tetrahedra */
    const float* node;       /* nn*3 coordinates (mm) */
    const int32_t* elem;     /* ne*4 node ids, 1-based */
    const int32_t* label;    /* ne medium labels, 0 = background/void */
    const int32_t* facenb;   /* ne*4 face neighbours, or NULL to compute */
} mmcgb_mesh_desc;

/* Simulation settings (the mcconfig fields the photon path reads,
 * src/mmc_utils.h:210-345). */
typedef struct mmcgb_config {
    uint64_t nphoton;        /* photons to launch (replay: replayed photons) */
    uint64_t photon_offset;  /* index of the first photon (sharded runs) */
    uint64_t seed;           /* RNG seed */
    float srcpos[3];         /* source position (mm) */
    float srcdir[3];         /* unit launch direction */
    int32_t srctype;         /* the reference's source types (src/mmc_utils.h:101-105): 0 pencil,
                                1 isotropic, 2 cone, 3 gaussian, 4 planar, 5 pattern, 6 fourier,
                                7 arcsine, 8 disk, 9 fourierx, 10 fourierx2d, 11 zgaussian, 12 line,
                                13 slit, 14 pencilarray, 15 pattern3d, 16 hyperboloid, 17 ring;
                                parameters in srcparam1/srcparam2/focus/srcpattern below */
    int32_t e0;              /* initial element, 1-based; 0 = locate it */
    float tstart, tend, tstep;  /* time gates (s) */
    int32_t isreflect;       /* 0 no mismatch, 1 Fresnel, 2 absorbing exterior, 3 mirror */
    int32_t isspecular;
    int32_t voidtime;
    int32_t issavedet;       /* save detected photons */
    int32_t issaveseed;      /* save 16-byte RNG seeds of detected photons */
    int32_t issaveexit;      /* save exit position/direction */
    int32_t ismomentum;      /* save momentum transfer */
    float minenergy;         /* roulette threshold */
    float roulettesize;
    float nout;              /* refractive index outside the mesh */
    float unitinmm;
    int32_t outputtype;      /* mmcgb_output */
    int32_t basisorder;      /* 0 element output, 1 node output */
    int32_t isnormalized;    /* 0 raw, 1 normalized (2 = skip surface nvol fix) */
    uint32_t maxdetphoton;
    int32_t nmedia;          /* rows in media, including background row 0 */
    const float* media;      /* nmedia*4: mua mus g n (1/mm) */
    int32_t detnum;
    const float* detpos;     /* detnum*4: x y z radius (mm) */
    const uint64_t* replayseed;   /* replay: nphoton*2 words (16-byte seeds), else NULL */
    const float* replayweight;    /* replay: nphoton */
    const float* replaytime;      /* replay: nphoton (s) */
    int32_t accum_f64;       /* 1: double atomics (default), 0: float + overflow buffer */
    uint64_t step_budget;    /* max ray-tet tests per photon, 0 = 100,000,000 */
    int32_t threads;         /* threads per block, 0 = auto */
    int32_t blocks;          /* persistent blocks, 0 = auto */
    int32_t fast_math;       /* 1: hardware-approximate division/exp/log/sincos and fused
                                multiply-adds (as the reference's -use_fast_math build);
                                0: IEEE arithmetic, photon-for-photon reproducible on the CPU */
    int32_t phased;          /* gate-phased tracing of a launch (one launch per window of k time
                                gates, photons parked between windows, so only k+1 gate planes of
                                the fluence take deposits at a time; same results photon for
                                photon): 0 = auto (when >= 8 gates, fluence >= 64 MB, >= 4e6
                                photons per launch and queue memory available; k sized so the
                                k+1 live planes fill ~70% of the L2), k >= 1 = window of k gates
                                whenever possible (not for replay), -1 = never */
    float srcparam1[4];      /* source parameters 1 and 2, as the reference's cfg->srcparam1/2
                                (src/mmc_utils.h:219-220), e.g. disk radius, area-source edge
                                vectors with the pattern size in w, Fourier wave numbers */
    float srcparam2[4];
    float focus;             /* focal length (the reference's srcdir.w): 0 none, > 0 converging,
                                < 0 diverging; NaN random direction, -inf Lambertian */
    const float* srcpattern; /* pattern source weights: srcparam1.w x srcparam2.w values (type 5)
                                or srcparam1.x x .y x .z (type 15), row-major, else NULL; with
                                srcnum > 1 patterns, srcnum values per pixel, adjacent */
    int32_t issaveref;       /* 1: accumulate the weight of photons leaving through each exterior
                                face per gate (diffuse reflectance/transmittance, -X) into
                                mmcgb_result.dref */
    int32_t method;          /* 0: element output (branchless Badouel, -M S); 1: dual-grid output
                                (DMMC, -M G): fluence on a voxel grid over the mesh's bounding
                                box, datalen = dim.x*dim.y*dim.z (mmcgb_grid_info), x fastest */
    float gridstep;          /* voxel edge of the grid output in mm (the reference's Domain.Step);
                                0 = 1 mm */
    uint32_t maxjumpdebug;   /* > 0: save photon trajectories (the reference's -D M): a record at
                                each launch, scattering event and photon end, at most this many,
                                into mmcgb_result.traj */
    uint64_t phase_chunk;    /* at most this many photons per gate-phased launch (their parked
                                states are queued on the device); 0 = as many as half of the free
                                device memory holds.  A launch of more photons is traced as several
                                phased launches, with the same results */
    int32_t accumulate;      /* 0: mmcgb_result.field and .dref are overwritten; 1: this run's
                                deposits (scattered to the nodes for basisorder 1) are added to
                                what the caller's arrays hold, and with isnormalized the sum is
                                then normalized in place with this run's energies -- what
                                mmc_run_cu does to cfg->exportfield / mesh->dref
                                (src/mmc_cu_host.cu:916-976, normalization :984-1061) */
    int32_t srcnum;          /* pattern sources (type 5): number of patterns sharing each photon
                                (the reference's cfg->srcnum, photon sharing: a photon starts with
                                weight 1 and every deposit is scaled by each pattern's value at its
                                launch pixel, src/mmc_core.cl:929-942, :1907-1911); the field then
                                holds srcnum values per (gate, element|node|voxel), adjacent, each
                                pattern normalized with its own energies; the last column of a
                                detected record holds the launch pixel (uint32 bits) instead of
                                the initial weight.  0 or 1: one pattern */
    const float* nodemua;    /* nn per-node absorption coefficients (1/mm), or NULL: each step then
                                takes its element's mua as the mean of the element's four nodal
                                values instead of the media row of its label -- the reference's
                                DOT-reconstruction mode (cfg->nodemua with isnodalmua,
                                src/mmc_core.cl:785-793, src/mmc_utils.h:314-322); the deposit
                                divides by that mua, the output stage still normalizes with the
                                media table */
    const float* nodemusp;   /* nn per-node scattering coefficients (1/mm) taking the element's mus
                                the same way (isnodalmusp); read only with nodemua, as the
                                reference reads it; g and n stay those of the label's media row */
} mmcgb_config;

/* Outputs.  Pointers may be NULL to skip an output; counts are always set. */
typedef struct mmcgb_result {
    double* field;           /* maxgate*datalen(*srcnum), datalen = ne (basisorder 0) or nn */
    float* detp;             /* maxdetphoton*reclen detected-photon records */
    uint8_t* seeds;          /* maxdetphoton*16 */
    float* photon_weight;    /* nphoton final weights (parity tracing), or NULL; any of the three
                                per-photon outputs selects the general kernels (same results) */
    uint32_t* photon_steps;  /* nphoton ray-tet tests per photon, or NULL */
    int32_t* photon_det;     /* nphoton detector ids (0 = none), or NULL */
    uint32_t detected;       /* detected photons (may exceed maxdetphoton) */
    uint32_t saved;          /* records written */
    int32_t reclen;          /* columns per record: 1 + (2+mom)*M + 6*exit + 1 */
    int32_t maxgate;
    double energytot;        /* launched weight */
    double energyesc;        /* escaped weight */
    double normalizer;
    uint64_t raytet;         /* ray-tetrahedron tests */
    uint64_t aborted;        /* photons stopped by the step budget */
    uint64_t outside;        /* photons whose launch position lies in no element (an error) */
    float* traj;             /* maxjumpdebug*6 trajectory records: photon id (uint32 bits), x, y, z,
                                weight, element id (int32 bits); src/mmc_core.cl:692-704 */
    uint32_t ntraj;          /* trajectory records produced (may exceed maxjumpdebug) */
    double* dref;            /* issaveref: maxgate*nf exiting weight per exterior face (faces
                                numbered as mmcgb_mesh_info's nf), divided by the launched weight
                                when isnormalized, else NULL */
    float kernel_ms;         /* device time of the photon kernel */
    double* energy_src;      /* srcnum > 1: 2*srcnum values, the launched weight of each pattern,
                                then the escaped weight of each (energytot/energyesc are their
                                sums, as the reference reports them), or NULL */
} mmcgb_result;

int32_t mmcgb_abi_version(void);
const char* mmcgb_last_error(void);

/* Builds the ray-tracer records for `desc` on `device` and keeps them resident.
 * Replaces mesh_getvolume/mesh_getfacenb/tracer_build/tracer_prep
 * (src/mmc_mesh.c:910-974, src/mmc_highorder.cpp:128-159,
 * src/mmc_mesh.c:1496-1602, :1241-1483) and the uploads of
 * src/mmc_cu_host.cu:447-487.  Labels must lie in -1..63 (-1 = void); a mesh
 * whose largest label needs b bits may hold up to 2^(31-b) - 1 elements
 * (1,073,741,823 with labels 0-1, 33,554,431 with labels up to 63), else
 * MMCGB_E_MESH. */
int32_t mmcgb_mesh_create(const mmcgb_mesh_desc* desc, int32_t device, mmcgb_mesh** out);
int32_t mmcgb_mesh_destroy(mmcgb_mesh* mesh);
/* Sizes of a resident mesh: nodes, elements, exterior faces. */
int32_t mmcgb_mesh_info(const mmcgb_mesh* mesh, int32_t* nn, int32_t* ne, int32_t* nf);
/* Host copies of the prepared mesh (any pointer may be NULL): elem after the
 * orientation fix (ne*4), facenb with exterior faces numbered -1,-2,...
 * (ne*4), element volumes (ne), nodal volumes before the surface fix (nn). */
int32_t mmcgb_mesh_export(const mmcgb_mesh* mesh, int32_t* elem, int32_t* facenb,
                          float* evol, float* nvol);
/* Dimensions and origin of the dual-grid output of `m` for voxel edge `step`
 * (mesh_createdualmesh, src/mmc_mesh.c:349-381): origin = node minimum - 1e-6,
 * dim = (int)((max - min + 2e-6) / step) + 1 per axis. */
int32_t mmcgb_grid_info(const mmcgb_mesh* m, float step, int32_t dim[3], float origin[3]);
/* First element (1-based, by index) enclosing p, 0 if none
 * (src/mmc_mesh.c:1060-1090). */
int32_t mmcgb_mesh_locate(const mmcgb_mesh* mesh, const float p[3]);

/* One simulation on a resident mesh (src/mmc_cu_host.cu:204-1528). */
int32_t mmcgb_simulate(mmcgb_mesh* mesh, const mmcgb_config* cfg, mmcgb_result* res);

/* A simulation run as a sequence of launches that accumulate into the same
 * device buffers (the reference's respin loop, src/mmc_cu_host.cu:656-906).
 * begin allocates and zeroes the outputs; each launch simulates photons
 * [photon_offset, photon_offset+nphoton) of the run asynchronously on the
 * session's stream; sync waits and reports the last launch's device time;
 * end reads back, normalizes into `res` (may be NULL to discard) and frees.
 * `trace` may carry per-photon trace buffers (single-launch sessions only). */
typedef struct mmcgb_session mmcgb_session;
int32_t mmcgb_session_begin(mmcgb_mesh* mesh, const mmcgb_config* cfg, mmcgb_result* trace,
                            mmcgb_session** out);
int32_t mmcgb_session_launch(mmcgb_session* s, uint64_t photon_offset, uint64_t nphoton);
/* One persistent launch over several sessions (same device, same fast_math):
 * session i simulates photons [offsets[i], offsets[i]+counts[i]) of its run.
 * Photons are handed out from one pool, so sessions of very different sizes
 * keep every SM busy to the end.  Used for batched runs and for the waves of
 * the continuous-batching server. */
int32_t mmcgb_session_launch_batch(int32_t n, mmcgb_session* const* sessions, const uint64_t* offsets,
                                   const uint64_t* counts);
/* As mmcgb_session_launch_batch, but enqueued on the caller's CUDA stream
 * `stream` (a cudaStream_t), ordered after each session's setup but not
 * against the sessions' launches: several such launches may be in flight at once and
 * accumulate into the same sessions concurrently (every accumulation is
 * atomic).  Each session's later work (mmcgb_session_sync/_end, freeing its
 * buffers) is ordered after the launch, so ending a session early is safe.
 * Pipelined serving waves use it: the next wave's blocks take over the SMs
 * while the current wave's last photons drain.  No counterpart in the
 * reference. */
int32_t mmcgb_session_launch_batch_on(int32_t n, mmcgb_session* const* sessions, const uint64_t* offsets,
                                      const uint64_t* counts, void* stream);
/* A sequence of batched launches, captured as one CUDA graph and enqueued on
 * `stream` (a cudaStream_t): group g runs one persistent launch over the next
 * group_sizes[g] sessions of `sessions` (session i simulating photons
 * [offsets[i], offsets[i]+counts[i]) of its run), the groups one after
 * another.  The graph is instantiated once per device and updated in place by
 * later calls of the same shape (the same number of launches of the same
 * kernels).  The groups wait for every session's setup, and every session's
 * later work waits for the groups.  No counterpart in the reference (one
 * simulation per device, src/mmc_core.cl:464-467); batching.simulate_many
 * runs its size-sorted groups through it. */
int32_t mmcgb_session_launch_batches(int32_t ngroups, const int32_t* group_sizes, mmcgb_session* const* sessions,
                                     const uint64_t* offsets, const uint64_t* counts, void* stream);
/* The reference's respin loop (src/mmc_cu_host.cu:656-906: `repeats` launches
 * accumulating into one set of buffers) as one CUDA graph: launch k traces
 * photons [photon_offset + k*nphoton, photon_offset + (k+1)*nphoton).  The
 * graph is captured on the session's stream; later calls of the same shape
 * update the instantiated graph in place instead of instantiating again. */
int32_t mmcgb_session_launch_repeat(mmcgb_session* s, uint64_t photon_offset, uint64_t nphoton, int32_t repeats);
int32_t mmcgb_session_sync(mmcgb_session* s, float* last_kernel_ms);
/* The session's CUDA stream (a cudaStream_t): callers may record events on it
 * to pipeline work, e.g. to know when a batched launch led by this session
 * has finished.  Valid until mmcgb_session_end. */
void* mmcgb_session_stream(mmcgb_session* s);
int32_t mmcgb_session_end(mmcgb_session* s, mmcgb_result* res);
/* How a launch of `nphoton` photons of this session would be traced:
 * *window = 0 for one launch, k for one launch per window of k gates (the
 * value of mmcgb_config.phased, or the automatic choice: the live gate planes
 * fill about 70% of the L2); *chunk (may be NULL) = photons per phased launch
 * (fewer than nphoton when the queues for all of them do not fit in half of
 * the free device memory, or mmcgb_config.phase_chunk caps them).  No
 * counterpart in the reference. */
int32_t mmcgb_session_phase_window(mmcgb_session* s, uint64_t nphoton, int32_t* window, uint64_t* chunk);
/* Device addresses of a session's raw buffers (valid until
 * mmcgb_session_end), for a caller that combines sessions on several GPUs
 * before the output stage -- the reference's multi-device sum of fields,
 * energies and counters and concatenation of detected records
 * (src/mmc_cu_host.cu:772-783, :916-921), done here with device collectives:
 *   field_raw  maxgate*datalen doubles (NULL for float32 accumulation)
 *   energy     2 doubles: launched, escaped weight
 *   counters   3 uint64: ray-tet tests, photons stopped by the step budget,
 *              photons launched outside the mesh
 *   detcount   1 uint32; detp maxdetphoton*reclen floats; seeds 16 bytes each
 * Synchronize the session (mmcgb_session_sync) before touching them; what a
 * caller leaves in them is what mmcgb_session_end reads back and normalizes. */
int32_t mmcgb_session_device_buffers(mmcgb_session* s, mmcgb_device_out* out);

/* `n` simulations sharing one persistent launch; meshes may differ.  Each
 * simulation's results land in its own mmcgb_result. */
int32_t mmcgb_simulate_batch(int32_t n, mmcgb_mesh* const* meshes, const mmcgb_config* cfgs,
                             mmcgb_result* res);

/* One-shot drop-in for mmc_run_cu (src/mmc_cu_host.h:56). */
int32_t mmcgb_run(const mmcgb_mesh_desc* desc, const mmcgb_config* cfg, int32_t device,
                  mmcgb_result* res);

/* ---- for callers that cannot allocate device memory ----------------------
 * No counterpart in the reference (its CUDA host allocates every buffer per
 * run, src/mmc_cu_host.cu:447-610).  Some callers cannot let a library call
 * cudaMalloc: programs whose own pool already owns the free GPU memory (a
 * framework's caching allocator), and serving loops where the device-wide
 * synchronization of cudaMalloc/cudaFree would stall work in flight.  This
 * entry runs one simulation of the photon engine on `stream` (a cudaStream_t,
 * NULL = legacy default stream) into device buffers the caller owns, and
 * allocates nothing: the work counter and the staged media/detector tables
 * live in a fixed 8 KiB device array inside the library, held by every GPU
 * that loads the library until the process exits.
 *   - outputs are overwritten (zeroed first): field_raw holds the raw element
 *     deposits, maxgate*ne doubles, gate-major (the layout of mmcgb_result.field
 *     for basisorder 0, isnormalized 0); energy[0] = launched weight, energy[1] =
 *     escaped weight; counters[0] = ray-tet tests,
 *     counters[1] = photons stopped by the step budget
 *   - issavedet: detp holds maxdetphoton records of
 *     reclen = (2 + ismomentum)*(nmedia - 1) + 6*issaveexit + 2 floats each
 *     (detector id, scatter counts, partial paths, exit position/direction,
 *     launch weight), seeds maxdetphoton*16 bytes when issaveseed.  *detcount
 *     counts every detected photon and can exceed maxdetphoton; only the first
 *     min(*detcount, maxdetphoton) records are written, so clamp before reading
 *   - the configuration passes the checks of mmcgb_simulate first (a given e0
 *     is used only if it encloses srcpos, otherwise the source is located);
 *     then limits: point sources, element output, nmedia <=
 *     MMCGB_NOALLOC_MAX_MEDIA, detnum <= MMCGB_NOALLOC_MAX_DET, accum_f64 = 1,
 *     no replay, exiting weight, trajectories or per-node properties; anything else returns
 *     MMCGB_E_ARG
 *   - the first call on a device looks up the array's device address; make it
 *     before any stream capture
 *   - all calls share the array and keep its last contents; the call clears the
 *     work counter itself.  Calls that overlap on the GPU race on the array.
 * The call returns after enqueueing; synchronize `stream` before reading. */
#define MMCGB_NOALLOC_MAX_MEDIA 64
#define MMCGB_NOALLOC_MAX_DET 256
struct mmcgb_device_out {
    double* field_raw;       /* device, maxgate*ne(*srcnum) */
    float* detp;             /* device, maxdetphoton*reclen (issavedet) */
    uint8_t* seeds;          /* device, maxdetphoton*16 (issaveseed) */
    uint32_t* detcount;      /* device, 1 (issavedet) */
    double* energy;          /* device, 2 */
    uint64_t* counters;      /* device, 2 */
    double* energy_src;      /* device, 64*2*srcnum (srcnum > 1, else NULL): launched and escaped
                                weight per pattern in 64 slots [slot][launched|escaped][pattern],
                                summed over the slots at the end (mmcgb_simulate_noalloc: unused) */
};
int32_t mmcgb_simulate_noalloc(mmcgb_mesh* mesh, const mmcgb_config* cfg, const mmcgb_device_out* out,
                               void* stream);

/* ---- host-only stages (no GPU needed) ---------------------------------- */
/* Mesh preparation alone: orientation fix and volumes (src/mmc_mesh.c:910-974),
 * face neighbours (src/mmc_highorder.cpp:128-159), face normals and plane
 * offsets (src/mmc_mesh.c:1572-1601), exterior-face numbering
 * (src/mmc_mesh.c:1466-1474).  Outputs (any may be NULL): elem ne*4,
 * facenb ne*4, normals ne*16 (nx[4] ny[4] nz[4] d[4]), evol ne, nvol nn, nf. */
int32_t mmcgb_prepare_host(const mmcgb_mesh_desc* desc, int32_t* elem, int32_t* facenb, float* normals,
                           float* evol, float* nvol, int32_t* nf);
/* Output stage alone: elem->node scatter of raw element deposits
 * (src/mmc_cu_host.cu:916-976), surface nodal-volume fix
 * (src/mmc_mesh.c:1344-1386) and normalization (src/mmc_mesh.c:2154-2279).
 * raw: maxgate*ne; field: maxgate*datalen (datalen = nn if basisorder). */
int32_t mmcgb_normalize_host(const mmcgb_mesh_desc* desc, const mmcgb_config* cfg, const double* raw,
                             double energytot, double energyesc, double* field, double* normalizer);

/* Checks a configuration against a mesh on the host, with no GPU: the tests
 * mmcgb_simulate makes before it allocates (the reference's mcx_validatecfg,
 * src/mmc_utils.c:3500, plus the engine's own limits such as at most 2^31-1
 * fluence cells of gates x elements, or voxels).  Writes the initial element
 * the run would start in to *e0 when e0 is not NULL. */
int32_t mmcgb_check_config(const mmcgb_mesh_desc* desc, const mmcgb_config* cfg, int32_t* e0);

/* Diagnostic, no counterpart in the reference: the L2 read bandwidth of
 * `device` in GB/s -- a buffer of `bytes` (at most half of the L2) read once
 * to make it resident, then `reps` sweeps with L1-bypassing 16-byte loads from
 * every SM.  The engine's gathers are served from L2; this is the ceiling its
 * L2 traffic is compared with.  Allocates and frees the buffer itself. */
int32_t mmcgb_l2_read_bandwidth(int32_t device, uint64_t bytes, int32_t reps, double* gbs);

/* Fills `cfg` with the reference defaults (src/mmc_utils.c:207-363). */
void mmcgb_config_defaults(mmcgb_config* cfg);

#ifdef __cplusplus
}
#endif
#endif

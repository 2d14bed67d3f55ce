/*
 * CPU oracle for the per-photon tetrahedral tracing path of Mesh-based Monte
 * Carlo (fangq/mmc).  TEST INFRASTRUCTURE ONLY: tests, the smoke check and the
 * CPU-baseline leg of bench.py use it as the checker.  It is never linked into,
 * or called by, the product library.
 *
 * It restates the reference GPU path (src/mmc_core.cl, run through
 * src/mmc_cu_host.cu) in plain C, photon by photon, with the same RNG recipe
 * (xorshift128+) and the same control flow.  Two deliberate differences from
 * the reference, shared with the CUDA engine so that both agree photon by
 * photon:
 *   - each photon's xorshift128+ state comes from (seed, photon index) through
 *     a splitmix64 hash instead of per-thread srand()/rand() streams;
 *   - exp/log/sincos are evaluated with the project's own polynomial routines
 *     (Cody-Waite reduction + Taylor/atanh series), so host and device produce
 *     identical bits.
 * Parity against the reference itself is statistical (golden fixtures made by
 * running the reference CPU binary, tests/golden/make_golden.py).
 */
#ifndef MMC_ORACLE_H
#define MMC_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_cfg {
    uint64_t nphoton;       /* photons to launch (or replayed photons) */
    uint64_t photon_offset; /* index of the first photon (sharding) */
    uint64_t seed;
    float srcpos[3];
    float srcdir[3];
    int e0;                 /* initial element, 1-based; 0 = locate */
    float tstart, tend, tstep;
    int maxgate;
    int isreflect;          /* 0 none, 1 Fresnel, 2 absorb at exterior, 3 mirror */
    int isspecular;
    int voidtime;
    int issavedet, issaveexit, ismomentum;
    float minenergy, roulettesize, nout;
    int outputtype;         /* 0 flux 1 fluence 2 energy 3 jacobian 4 wl 5 wp */
    int basisorder;
    int isnormalized;
    uint32_t maxdetphoton;
    int nmedia;             /* rows in media incl. background row 0 */
    const float* media;     /* nmedia*4: mua mus g n */
    int detnum;
    const float* detpos;    /* detnum*4: x y z r */
    const uint64_t* replayseed;  /* nphoton*2 or NULL */
    const float* replayweight;
    const float* replaytime;
    int accum_f64;          /* 1: double fluence sums; 0: float + 1000 overflow split */
    uint64_t step_budget;   /* max ray-tet tests per photon */
    int srctype;            /* the reference's source types, src/mmc_utils.h:101-105 */
    float srcparam1[4], srcparam2[4];
    float focus;            /* srcdir.w of the reference */
    const float* srcpattern;
    int issaveref;          /* exiting weight per exterior face and gate into oracle_out.dref */
    int method;             /* 0 element output, 1 dual-grid (DMMC) output */
    float gridstep;         /* voxel edge of the grid output (mm), 0 = 1 */
    int srcnum;             /* patterns sharing each photon (pattern source, src/mmc_core.cl:1907-1911);
                               field_raw then holds srcnum values per cell, adjacent; 0 or 1 = one */
    const float* nodemua;   /* nn per-node absorption, or NULL: an element's mua is then the mean of
                               its four nodes' values (src/mmc_core.cl:785-793) */
    const float* nodemusp;  /* nn per-node scattering coefficients, read only with nodemua */
} oracle_cfg;

typedef struct oracle_out {
    double* field_raw;      /* maxgate*ne(*srcnum) raw element deposits (required) */
    float* detp;            /* maxdetphoton*reclen, may be NULL */
    uint8_t* seeds;         /* maxdetphoton*16, may be NULL */
    float* photon_weight;   /* per photon final weight, may be NULL */
    uint32_t* photon_steps; /* per photon ray-tet tests, may be NULL */
    int32_t* photon_det;    /* per photon detector id (0 none), may be NULL */
    uint32_t detected;
    int reclen;
    double energytot, energyesc;
    uint64_t raytet;
    uint64_t aborted;
    uint64_t outside;       /* photons launched at a position no element encloses */
    double* dref;           /* issaveref: maxgate*nf (raw, unnormalized), may be NULL */
    int nf;                 /* exterior faces of the prepared mesh */
    float* traj;            /* maxtraj*6 trajectory records (id, x, y, z, w, eid), may be NULL */
    uint32_t maxtraj;
    uint32_t ntraj;         /* records written or attempted (may exceed maxtraj) */
    double sim_seconds;     /* wall time of the photon loop (mesh preparation excluded) */
    double* energy_src;     /* srcnum > 1: launched weight per pattern, then escaped weight per
                               pattern (2*srcnum); energytot/energyesc are then their sums */
} oracle_out;

/* Mesh preparation (volumes with orientation fix, face neighbours, normals,
 * surface numbering).  Outputs are caller-allocated:
 *   elem_out ne*4, facenb_out ne*4, normals ne*16, evol ne, nvol nn. */
int oracle_prep_mesh(int nn, const float* node, int ne, const int* elem, const int* label,
                     const int* facenb_in, int* elem_out, int* facenb_out, float* normals,
                     float* evol, float* nvol, int* nf);

/* Dual-grid dimensions for voxel edge `step`: mesh_createdualmesh,
 * src/mmc_mesh.c:349-381 (bounding box padded by 1e-6, dim = (int)(span/step)+1). */
void oracle_grid_dims(int nn, const float* node, float step, int dim[3], float nmin[3]);

/* First element (by index) whose bounding box and barycentric test enclose p. */
int oracle_initelem(int nn, const float* node, int ne, const int* elem, const float* p);

int oracle_run(int nn, const float* node, int ne, const int* elem, const int* label,
               const oracle_cfg* cfg, oracle_out* out, int nthreads);

/* Host-side output stage: elem->node scatter (basisorder 1), surface nvol fix
 * and normalization, written into field (maxgate*datalen doubles). */
double oracle_normalize(int nn, const float* node, int ne, const int* elem, const int* label,
                        const oracle_cfg* cfg, const double* field_raw, double energytot,
                        double energyesc, double* field);

/* math kernels, exposed for accuracy tests */
float oracle_expf(float x);
float oracle_logf(float x);
void oracle_sincos2pi(float u, float* s, float* c);
void oracle_rng_seed(uint64_t seed, uint64_t pid, uint64_t st[2]);
float oracle_rng_next(uint64_t st[2]);

#ifdef __cplusplus
}
#endif
#endif

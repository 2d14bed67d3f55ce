/*
 * CPU oracle: plain-C restatement of MMC's per-photon tetrahedral tracing
 * (GPU path, branchless Badouel tracer, element-based deposit).
 * TEST INFRASTRUCTURE ONLY -- see mmc_oracle.h.  Each routine cites the
 * reference file:line it restates (paths inside the fangq/mmc tree).
 *
 * Build: gcc -O2 -ffp-contract=off -fopenmp -fPIC -shared (no -ffast-math): the
 * float operation sequence below is the contract the CUDA engine follows, so
 * contraction into FMAs must stay off; explicit fmaf() appears only inside the
 * polynomial math routines, where the CUDA engine uses the same fmaf().
 */
#include "mmc_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- constants (src/mmc_core.cl:330-360, src/mmc_mesh.h:66-74) ---- */
#define O_EPS        1e-6f              /* EPS seen by the CUDA build: src/mmc_mesh.h:70 */
#define O_PI         3.14159265358979323846f
#define O_R_C0       3.335640951981520e-12f
#define O_MAX_ACCUM  1000.f
#define O_R_MIN_MUS  1e9f
#define O_FIX_PHOTON 1e-3f
#define O_MAX_TRIAL  3
#define O_UNDEF      3.40282347e+38F    /* MMC_UNDEFINED */
#define O_ID_UNDEF   0x7FFFFFFF
#define O_DELTA_MUA  1e-4f

enum { OT_FLUX = 0, OT_FLUENCE, OT_ENERGY, OT_JACOBIAN, OT_WL, OT_WP, OT_WN = 16 };
enum { BC_NOREFLECT = 0, BC_REFLECT, BC_ABSORBEXT, BC_MIRROR };

/* face tables: src/mmc_mesh.c:59 (out), :71 (facemap), :95 (faceorder),
 * :107 (ifaceorder); face list of the neighbour search src/mmc_highorder.cpp:50 */
static const int OUTF[4][3] = {{0, 3, 1}, {3, 2, 1}, {0, 2, 3}, {0, 1, 2}};
static const int FACEMAP[4] = {2, 0, 1, 3};
static const int FACEORDER[5] = {1, 3, 2, 0, -1};
static const int IFACEORDER[4] = {3, 0, 2, 1};
static const int FACELIST[4][3] = {{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}};

/* ======================================================================
 * math: Cody-Waite argument reduction + truncated series (Cody & Waite,
 * "Software Manual for the Elementary Functions", 1980).  Coefficients are
 * the Taylor / atanh series terms 1/n!, 1/(2k+1).
 * ====================================================================== */
#define LN2_HI 0.693145751953125f          /* ln2 with its low 9 mantissa bits cleared */
#define LN2_LO 1.42860682030941723212e-6f  /* ln2 - LN2_HI */
#define LOG2E  1.44269504088896340736f

static float bits2f(uint32_t b) { float f; memcpy(&f, &b, 4); return f; }
static uint32_t f2bits(float f) { uint32_t b; memcpy(&b, &f, 4); return b; }

float oracle_expf(float x) {
    if (x < -104.f) return 0.f;
    if (x > 88.7f) return INFINITY;
    float k = rintf(x * LOG2E);
    float r = fmaf(k, -LN2_HI, x);
    r = fmaf(k, -LN2_LO, r);
    /* e^r, |r| <= 0.347: Taylor to r^7 */
    float p = 1.f / 5040.f;
    p = fmaf(p, r, 1.f / 720.f);
    p = fmaf(p, r, 1.f / 120.f);
    p = fmaf(p, r, 1.f / 24.f);
    p = fmaf(p, r, 1.f / 6.f);
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.f);
    p = fmaf(p, r, 1.f);
    int ki = (int)k;
    if (ki < -125) { p *= 5.42101086242752217e-20f; ki += 64; } /* 2^-64 */
    return p * bits2f((uint32_t)(ki + 127) << 23);
}

float oracle_logf(float x) {
    /* x > 0, finite: x = m 2^e, m in [sqrt(1/2), sqrt(2)); log m = 2 atanh(s), s=(m-1)/(m+1) */
    uint32_t b = f2bits(x);
    int e = (int)((b >> 23) & 0xFF) - 127;
    float m = bits2f((b & 0x007FFFFFu) | 0x3F800000u);
    if (m > 1.41421356f) { m *= 0.5f; e += 1; }
    float s = (m - 1.f) / (m + 1.f);
    float z = s * s;
    float p = 1.f / 11.f;
    p = fmaf(p, z, 1.f / 9.f);
    p = fmaf(p, z, 1.f / 7.f);
    p = fmaf(p, z, 1.f / 5.f);
    p = fmaf(p, z, 1.f / 3.f);
    p = fmaf(p, z, 1.f);
    float lm = 2.f * s * p;
    float fe = (float)e;
    return fmaf(fe, LN2_HI, fmaf(fe, LN2_LO, lm));
}

void oracle_sincos2pi(float u, float* s, float* c) {
    /* sin/cos(2 pi u): quadrant from u, |x| <= pi/4 after reduction */
    float q = rintf(u * 4.f);
    float f = u - q * 0.25f;
    float x = f * 6.28318530717958647692f;
    float z = x * x;
    float ps = 1.f / 362880.f;
    ps = fmaf(ps, z, -1.f / 5040.f);
    ps = fmaf(ps, z, 1.f / 120.f);
    ps = fmaf(ps, z, -1.f / 6.f);
    ps = fmaf(ps * z, x, x);
    float pc = -1.f / 3628800.f;
    pc = fmaf(pc, z, 1.f / 40320.f);
    pc = fmaf(pc, z, -1.f / 720.f);
    pc = fmaf(pc, z, 1.f / 24.f);
    pc = fmaf(pc, z, -0.5f);
    pc = fmaf(pc, z, 1.f);
    int qi = ((int)q) & 3;
    float sv, cv;
    switch (qi) {
        case 0: sv = ps; cv = pc; break;
        case 1: sv = pc; cv = -ps; break;
        case 2: sv = -ps; cv = -pc; break;
        default: sv = -pc; cv = ps; break;
    }
    *s = sv;
    *c = cv;
}

/* ======================================================================
 * RNG: xorshift128+ exactly as src/mmc_core.cl:517-531 (float from the top
 * 23 bits of the low word of s0+s1).  Per-photon initial state: splitmix64
 * (Vigna) of (seed, photon index).
 * ====================================================================== */
static uint64_t splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

void oracle_rng_seed(uint64_t seed, uint64_t pid, uint64_t st[2]) {
    uint64_t base = splitmix64(seed ^ 0x6D6D63676233ull) + 2ull * pid * 0x9E3779B97F4A7C15ull;
    st[0] = splitmix64(base);
    st[1] = splitmix64(base + 0x9E3779B97F4A7C15ull);
    if ((st[0] | st[1]) == 0) st[1] = 1;
}

float oracle_rng_next(uint64_t t[2]) {
    uint64_t s1 = t[0];
    const uint64_t s0 = t[1];
    t[0] = s0;
    s1 ^= s1 << 23;
    t[1] = s1 ^ s0 ^ (s1 >> 18) ^ (s0 >> 5);
    uint64_t r = t[1] + s0;
    uint32_t lo = (uint32_t)r;
    return bits2f(0x3F800000u | (lo >> 9)) - 1.0f;
}

/* ======================================================================
 * mesh preparation
 * ====================================================================== */
typedef struct { float x, y, z; } f3;

static f3 nodeat(const float* node, int i) { f3 r = {node[3 * i], node[3 * i + 1], node[3 * i + 2]}; return r; }

typedef struct { int a, b, c; int slot; } facekey;

static int cmp_face(const void* p, const void* q) {
    const facekey* x = (const facekey*)p;
    const facekey* y = (const facekey*)q;
    if (x->a != y->a) return x->a < y->a ? -1 : 1;
    if (x->b != y->b) return x->b < y->b ? -1 : 1;
    if (x->c != y->c) return x->c < y->c ? -1 : 1;
    return x->slot < y->slot ? -1 : (x->slot > y->slot);
}

static void sort3(int* v) {
    int t;
    if (v[0] > v[1]) { t = v[0]; v[0] = v[1]; v[1] = t; }
    if (v[1] > v[2]) { t = v[1]; v[1] = v[2]; v[2] = t; }
    if (v[0] > v[1]) { t = v[0]; v[0] = v[1]; v[1] = t; }
}

/* neighbour across face j (FACELIST order); src/mmc_highorder.cpp:128-159 */
static void get_facenb(int ne, const int* elem, int* facenb) {
    facekey* keys = (facekey*)malloc(sizeof(facekey) * (size_t)ne * 4);
    for (int i = 0; i < ne; i++)
        for (int j = 0; j < 4; j++) {
            int v[3] = {elem[i * 4 + FACELIST[j][0]], elem[i * 4 + FACELIST[j][1]], elem[i * 4 + FACELIST[j][2]]};
            sort3(v);
            facekey* k = keys + i * 4 + j;
            k->a = v[0]; k->b = v[1]; k->c = v[2]; k->slot = i * 4 + j;
        }
    qsort(keys, (size_t)ne * 4, sizeof(facekey), cmp_face);
    memset(facenb, 0, sizeof(int) * (size_t)ne * 4);
    for (size_t n = 0; n + 1 < (size_t)ne * 4; n++) {
        facekey* x = keys + n;
        facekey* y = keys + n + 1;
        if (x->a == y->a && x->b == y->b && x->c == y->c) {
            facenb[x->slot] = (y->slot >> 2) + 1;
            facenb[y->slot] = (x->slot >> 2) + 1;
            n++;
        }
    }
    free(keys);
}

int oracle_prep_mesh(int nn, const float* node, int ne, const int* elem, const int* label,
                     const int* facenb_in, int* ee, int* facenb, float* nrm,
                     float* evol, float* nvol, int* nf) {
    memcpy(ee, elem, sizeof(int) * (size_t)ne * 4);
    memset(nvol, 0, sizeof(float) * (size_t)nn);
    /* volumes + orientation: src/mmc_mesh.c:910-974 */
    for (int i = 0; i < ne; i++) {
        int* e = ee + 4 * i;
        for (int j = 0; j < 4; j++)
            if (e[j] < 1 || e[j] > nn) return -1;
        f3 n0 = nodeat(node, e[0] - 1), n1 = nodeat(node, e[1] - 1), n2 = nodeat(node, e[2] - 1), n3 = nodeat(node, e[3] - 1);
        float dx = n2.x - n3.x, dy = n2.y - n3.y, dz = n2.z - n3.z;
        float v = n1.x * (n2.y * n3.z - n2.z * n3.y) - n1.y * (n2.x * n3.z - n2.z * n3.x) + n1.z * (n2.x * n3.y - n2.y * n3.x);
        v += -n0.x * ((n2.y * n3.z - n2.z * n3.y) + n1.y * dz - n1.z * dy);
        v += +n0.y * ((n2.x * n3.z - n2.z * n3.x) + n1.x * dz - n1.z * dx);
        v += -n0.z * ((n2.x * n3.y - n2.y * n3.x) + n1.x * dy - n1.y * dx);
        v = -v;
        if (v < 0.f) {
            int t = e[3]; e[3] = e[2]; e[2] = t;
            v = -v;
        }
        v *= (1.f / 6.f);
        evol[i] = v;
        if (label[i] == 0) continue;
        for (int j = 0; j < 4; j++) nvol[e[j] - 1] += v * 0.25f;
    }
    if (facenb_in) memcpy(facenb, facenb_in, sizeof(int) * (size_t)ne * 4);
    else get_facenb(ne, ee, facenb);
    /* outward unit normals + plane offsets: src/mmc_mesh.c:1572-1601 */
    for (int i = 0; i < ne; i++) {
        float* vn = nrm + 16 * i;
        for (int j = 0; j < 4; j++) {
            f3 a = nodeat(node, ee[4 * i + OUTF[j][0]] - 1);
            f3 b = nodeat(node, ee[4 * i + OUTF[j][1]] - 1);
            f3 c = nodeat(node, ee[4 * i + OUTF[j][2]] - 1);
            f3 ab = {b.x - a.x, b.y - a.y, b.z - a.z};
            f3 ac = {c.x - a.x, c.y - a.y, c.z - a.z};
            f3 n = {ab.y * ac.z - ab.z * ac.y, ab.z * ac.x - ab.x * ac.z, ab.x * ac.y - ab.y * ac.x};
            float rn = (float)(1.f / sqrt((double)(n.x * n.x + n.y * n.y + n.z * n.z)));
            n.x *= rn; n.y *= rn; n.z *= rn;
            vn[j] = n.x;
            vn[j + 4] = n.y;
            vn[j + 8] = n.z;
            vn[j + 12] = n.x * a.x + n.y * a.y + n.z * a.z;
        }
    }
    /* surface faces numbered -1,-2,...: src/mmc_mesh.c:1466-1474 */
    int cnt = 0;
    for (int i = 0; i < ne * 4; i++)
        if (facenb[i] == 0) facenb[i] = -(++cnt);
    *nf = cnt;
    return 0;
}

/* barycentric enclosure test: src/mmc_mesh.c:1170-1205 */
static int barycentric_inside(const float* node, const int* e, const float* p) {
    float bary[4];
    for (int i = 0; i < 4; i++) {
        f3 a = nodeat(node, e[OUTF[i][0]] - 1);
        f3 b = nodeat(node, e[OUTF[i][1]] - 1);
        f3 c = nodeat(node, e[OUTF[i][2]] - 1);
        f3 ab = {b.x - a.x, b.y - a.y, b.z - a.z};
        f3 ac = {c.x - a.x, c.y - a.y, c.z - a.z};
        f3 s = {p[0] - a.x, p[1] - a.y, p[2] - a.z};
        f3 n = {ab.y * ac.z - ab.z * ac.y, ab.z * ac.x - ab.x * ac.z, ab.x * ac.y - ab.y * ac.x};
        bary[FACEMAP[i]] = -(s.x * n.x + s.y * n.y + s.z * n.z);
    }
    for (int i = 0; i < 4; i++)
        if (bary[i] < 0.f) return 0;
    return 1;
}

/* linear scan, first enclosing element: src/mmc_mesh.c:1060-1090 */
int oracle_initelem(int nn, const float* node, int ne, const int* elem, const float* p) {
    (void)nn;
    for (int i = 0; i < ne; i++) {
        const int* e = elem + 4 * i;
        double lo[3] = {1e30, 1e30, 1e30}, hi[3] = {-1e30, -1e30, -1e30};
        for (int j = 0; j < 4; j++)
            for (int d = 0; d < 3; d++) {
                double v = node[3 * (e[j] - 1) + d];
                if (v < lo[d]) lo[d] = v;
                if (v > hi[d]) hi[d] = v;
            }
        if (p[0] <= hi[0] && p[0] >= lo[0] && p[1] <= hi[1] && p[1] >= lo[1] && p[2] <= hi[2] && p[2] >= lo[2])
            if (barycentric_inside(node, e, p)) return i + 1;
    }
    return 0;
}

/* ======================================================================
 * photon engine
 * ====================================================================== */
/* bounding-box grid over the mesh: cell (x,y,z) lists the elements whose
 * bounding boxes overlap it, in index order (the CUDA library builds the same
 * grid in its mesh preparation; the per-photon source search reads it) */
typedef struct {
    int res;
    float lo[3], inv[3];
    uint32_t* start;
    uint32_t* items;
} locgrid;

typedef struct {
    int ne, nn, M;
    const float* node;
    const int* elem;
    const int* type;
    const locgrid* grid;
    int dgrid;         /* dual-grid output (method 1) */
    float gstep_inv;
    float gmin[3];
    uint32_t gdim[3];
    uint32_t framelen; /* fluence entries per gate */
    const int* facenb;
    const float* nrm;
    const oracle_cfg* cfg;
    float Rtstep;
    int maxgate;
    float* f32a;     /* float fluence + overflow half (accum_f64 == 0) */
    float* f32b;
    double* f64;     /* double fluence (accum_f64 == 1) */
    int reclen;      /* detreclen (without the det id column) */
    int K;           /* patterns sharing each photon */
} engine;

typedef struct {
    float px, py, pz, vx, vy, vz, ox, oy, oz; /* p0, vec, pout */
    int eid, faceid, isend;
    float weight, photontimer, slen, Lmove, slen0, oldweight;
    uint32_t oldidx;
    uint32_t photonid;
    int posidx;      /* launch pixel of a pattern source */
} ray;

static void deposit(engine* g, uint32_t idx, float val) {
    if (g->cfg->accum_f64) {
#pragma omp atomic
        g->f64[idx] += (double)val;
        return;
    }
    /* float sums with a second buffer for running sums above MAX_ACCUM
     * (src/mmc_core.cl:880-912); the content is moved by exchange, as the
     * CUDA engine does */
    float old, moved;
#pragma omp atomic capture
    { old = g->f32a[idx]; g->f32a[idx] += val; }
    if (old > O_MAX_ACCUM) {
#pragma omp atomic capture
        { moved = g->f32a[idx]; g->f32a[idx] = 0.f; }
        if (moved != 0.f) {
#pragma omp atomic
            g->f32b[idx] += moved;
        }
    }
}

/* photon sharing (src/mmc_core.cl:929-942, :989-1002): a deposit of w adds w times each
 * pattern's value at the photon's launch pixel to that pattern's cell */
static void deposit_src(engine* g, const ray* r, uint32_t idx, float val) {
    if (g->K > 1) {
        const float* pat = g->cfg->srcpattern + (size_t)r->posidx * g->K;
        for (int p = 0; p < g->K; p++) deposit(g, idx * (uint32_t)g->K + (uint32_t)p, val * pat[p]);
        return;
    }
    deposit(g, idx, val);
}

static float medium(const engine* g, int t, int k) { return g->cfg->media[4 * t + k]; }

/* one branchless Badouel step: src/mmc_core.cl:721-1226 (rtBLBadouel branch) */
static float raytet_step(engine* g, ray* r) {
    const oracle_cfg* cfg = g->cfg;
    if (r->eid <= 0) return -1.f;
    const float* N = g->nrm + 16 * (size_t)(r->eid - 1);
    r->ox = O_UNDEF;
    r->faceid = -1;
    r->isend = 0;
    float T[4], S[4];
    for (int k = 0; k < 4; k++) {
        S[k] = ((r->vx * N[k]) + (r->vy * N[k + 4])) + (r->vz * N[k + 8]);
        T[k] = N[k + 12] - (((r->px * N[k]) + (r->py * N[k + 4])) + (r->pz * N[k + 8]));
        T[k] = T[k] / S[k];
        T[k] = (S[k] > 0.f) ? T[k] : 1e10f;
    }
    float Lmin = fminf(fminf(fminf(T[0], T[1]), T[2]), T[3]);
    int faceidx = (Lmin == 1e10f) ? 4 : (Lmin == T[0] ? 0 : (Lmin == T[1] ? 1 : (Lmin == T[2] ? 2 : 3)));
    r->faceid = FACEORDER[faceidx];
    if (r->faceid >= 0 && Lmin >= 0.f) {
        int type = g->type[r->eid - 1];
        float mua = medium(g, type, 0), mus = medium(g, type, 1), nmed = medium(g, type, 3);
        if (g->cfg->nodemua) {
            /* src/mmc_core.cl:785-793: the mean of the element's four nodal values, summed in
               node order */
            const int* e = g->elem + 4 * (size_t)(r->eid - 1);
            const float* nm = g->cfg->nodemua;
            mua = 0.25f * (((nm[e[0] - 1] + nm[e[1] - 1]) + nm[e[2] - 1]) + nm[e[3] - 1]);
            if (g->cfg->nodemusp) {
                const float* ns = g->cfg->nodemusp;
                mus = 0.25f * (((ns[e[0] - 1] + ns[e[1] - 1]) + ns[e[2] - 1]) + ns[e[3] - 1]);
            }
        }
        float currweight = r->weight;
        r->Lmove = (mus <= O_EPS) ? O_R_MIN_MUS : r->slen / mus;
        r->isend = (Lmin > r->Lmove);
        r->Lmove = r->isend ? r->Lmove : Lmin;
        r->ox = r->px + Lmin * r->vx;
        r->oy = r->py + Lmin * r->vy;
        r->oz = r->pz + Lmin * r->vz;
        float rc = nmed * O_R_C0;
        /* (int)x > maxgate-1 (src/mmc_core.cl:803), without the float->int conversion */
        if ((r->photontimer + r->Lmove * rc - cfg->tstart) * g->Rtstep >= (float)g->maxgate) {
            r->faceid = -2;
            r->ox = O_UNDEF;
            r->Lmove = (cfg->tend - r->photontimer) / rc - 1e-4f;
        }
        float totalloss = oracle_expf(-mua * r->Lmove);
        r->weight *= totalloss;
        int replay = (cfg->replayseed != NULL);
        if (replay) {
            float rw = cfg->replayweight[r->photonid];
            if (cfg->outputtype == OT_WL || cfg->outputtype == OT_JACOBIAN) {
                currweight = r->Lmove;
                currweight *= rw;
                currweight += r->weight;
            } else if (cfg->outputtype == OT_WP) {
                currweight = (r->slen0 < O_EPS) ? 1.f : r->Lmove * mus / r->slen0;
                currweight *= rw;
                currweight += r->weight;
            }
        }
        r->slen -= r->Lmove * mus;
        float ww = currweight - r->weight;
        r->photontimer += r->Lmove * rc;
        if (cfg->outputtype == OT_WN) { /* deposits happen at scattering events only */
            r->px = r->px + r->Lmove * r->vx;
            r->py = r->py + r->Lmove * r->vy;
            r->pz = r->pz + r->Lmove * r->vz;
            return (r->faceid == -2) ? 0.f : r->slen;
        }
        float gf;
        if (replay && (cfg->outputtype == OT_WL || cfg->outputtype == OT_WP))
            gf = cfg->replaytime[r->photonid] * g->Rtstep;
        else
            gf = (r->photontimer - cfg->tstart) * g->Rtstep;
        /* MIN((int)gf, maxgate-1) of src/mmc_core.cl:835-838, kept inside the buffer */
        int gate = (gf < (float)(g->maxgate - 1)) ? (int)gf : g->maxgate - 1;
        if (gate < 0) gate = 0;
        uint32_t tshift = (uint32_t)(gate * g->ne);
        if (cfg->outputtype != OT_ENERGY && cfg->outputtype != OT_WP && cfg->outputtype != OT_WL)
            ww = (mua < O_EPS) ? (currweight * r->Lmove) : (ww / mua);
        if (g->dgrid) {
            /* dual-grid (DMMC) deposit: src/mmc_core.cl:1019-1218, src/mmc_raytrace.c:1614-1666;
             * voxel indices clamped to the grid */
            int nseg = ((int)(r->Lmove * g->gstep_inv) + 1) << 1;
            float seg = r->Lmove / (float)nseg;
            float segloss = oracle_expf(-mua * seg);
            float tx = r->vx * seg, ty = r->vy * seg, tz = r->vz * seg;
            float sx = (r->px - g->gmin[0]) + tx * 0.5f;
            float sy = (r->py - g->gmin[1]) + ty * 0.5f;
            float sz = (r->pz - g->gmin[2]) + tz * 0.5f;
            float loss = 1.f - totalloss;
            float frac = (loss == 0.f) ? 0.f : (1.f - segloss) / loss;
            uint32_t gshift = (uint32_t)gate * g->framelen;
            float w0 = ww;
            int flush = (r->faceid == -2 || !r->isend);
            for (int k = 0; k < nseg; k++) {
                uint32_t ix = (sx > 0.f) ? (uint32_t)floorf(sx * g->gstep_inv) : 0u;
                uint32_t iy = (sy > 0.f) ? (uint32_t)floorf(sy * g->gstep_inv) : 0u;
                uint32_t iz = (sz > 0.f) ? (uint32_t)floorf(sz * g->gstep_inv) : 0u;
                if (ix > g->gdim[0] - 1) ix = g->gdim[0] - 1;
                if (iy > g->gdim[1] - 1) iy = g->gdim[1] - 1;
                if (iz > g->gdim[2] - 1) iz = g->gdim[2] - 1;
                uint32_t nidx = iz * (g->gdim[0] * g->gdim[1]) + iy * g->gdim[0] + ix + gshift;
                float dw = w0 * frac;
                if (r->oldidx == (uint32_t)O_ID_UNDEF) r->oldidx = nidx;
                if (nidx != r->oldidx) {
                    if (r->oldweight > 0.f) deposit_src(g, r, r->oldidx, r->oldweight);
                    r->oldidx = nidx;
                    r->oldweight = dw;
                } else {
                    r->oldweight += dw;
                }
                if (flush) {
                    deposit_src(g, r, nidx, r->oldweight);
                    r->oldweight = 0.f;
                }
                w0 *= segloss;
                sx += tx; sy += ty; sz += tz;
            }
            r->px = r->px + r->Lmove * r->vx;
            r->py = r->py + r->Lmove * r->vy;
            r->pz = r->pz + r->Lmove * r->vz;
            return (r->faceid == -2) ? 0.f : r->slen;
        }
        uint32_t newidx = (uint32_t)(r->eid - 1) + tshift;
        if (r->oldidx == (uint32_t)O_ID_UNDEF) r->oldidx = newidx;
        if (newidx != r->oldidx) {
            if (r->oldweight > 0.f) deposit_src(g, r, r->oldidx, r->oldweight);
            r->oldidx = newidx;
            r->oldweight = ww;
        } else {
            r->oldweight += ww;
        }
        if (r->faceid == -2 || !r->isend) {
            deposit_src(g, r, newidx, r->oldweight);
            r->oldweight = 0.f;
        }
        r->px = r->px + r->Lmove * r->vx;
        r->py = r->py + r->Lmove * r->vy;
        r->pz = r->pz + r->Lmove * r->vz;
    }
    return (r->faceid == -2) ? 0.f : r->slen;
}

/* Fresnel / TIR at a face: src/mmc_core.cl:1247-1303 */
static void reflectray(engine* g, ray* r, int oldeid, int* eid, int faceid, uint64_t* ran) {
    const oracle_cfg* cfg = g->cfg;
    const float* N = g->nrm + 16 * (size_t)(oldeid - 1);
    int fi = IFACEORDER[faceid];
    float pnx = N[fi], pny = N[fi + 4], pnz = N[fi + 8];
    float Icos = fabsf(((r->vx * pnx) + (r->vy * pny)) + (r->vz * pnz));
    float n1 = (oldeid != *eid) ? medium(g, g->type[oldeid - 1], 3) : cfg->nout;
    float n2 = (*eid > 0) ? medium(g, g->type[*eid - 1], 3) : cfg->nout;
    float tmp0 = n1 * n1;
    float tmp1 = n2 * n2;
    float tmp2 = 1.f - tmp0 / tmp1 * (1.f - Icos * Icos);
    if (tmp2 > 0.f && !((*eid <= 0) && (cfg->isreflect == BC_MIRROR))) {
        float Re = tmp0 * Icos * Icos + tmp1 * tmp2;
        tmp2 = sqrtf(tmp2);
        float Im = 2.f * n1 * n2 * Icos * tmp2;
        float Rtotal = (Re - Im) / (Re + Im);
        Re = tmp1 * Icos * Icos + tmp0 * tmp2 * tmp2;
        Rtotal = (Rtotal + (Re - Im) / (Re + Im)) * 0.5f;
        if (oracle_rng_next(ran) <= Rtotal) {
            float k = -2.f * Icos;
            r->vx += k * pnx; r->vy += k * pny; r->vz += k * pnz;
            *eid = oldeid;
        } else if ((cfg->isspecular == 2) && (*eid == 0)) {
        } else {
            float k = -Icos;
            r->vx += k * pnx; r->vy += k * pny; r->vz += k * pnz;
            float q = n1 / n2;
            r->vx = tmp2 * pnx + q * r->vx;
            r->vy = tmp2 * pny + q * r->vy;
            r->vz = tmp2 * pnz + q * r->vz;
        }
    } else {
        float k = -2.f * Icos;
        r->vx += k * pnx; r->vy += k * pny; r->vz += k * pnz;
        *eid = oldeid;
    }
    float inv = 1.f / sqrtf(r->vx * r->vx + r->vy * r->vy + r->vz * r->vz);
    r->vx *= inv; r->vy *= inv; r->vz *= inv;
}

/* direction update: src/mmc_core.cl:1345-1377 */
static void rotatevector(ray* r, float stheta, float ctheta, float sphi, float cphi) {
    float px, py, pz;
    if (r->vz > -1.f + O_EPS && r->vz < 1.f - O_EPS) {
        float tmp0 = 1.f - r->vz * r->vz;
        float tmp1 = 1.f / sqrtf(tmp0);
        tmp1 = stheta * tmp1;
        px = tmp1 * (r->vx * r->vz * cphi - r->vy * sphi) + r->vx * ctheta;
        py = tmp1 * (r->vy * r->vz * cphi + r->vx * sphi) + r->vy * ctheta;
        pz = -tmp1 * tmp0 * cphi + r->vz * ctheta;
    } else {
        px = stheta * cphi;
        py = stheta * sphi;
        pz = (r->vz > 0.f) ? ctheta : -ctheta;
    }
    float inv = 1.f / sqrtf(px * px + py * py + pz * pz);
    r->vx = px * inv; r->vy = py * inv; r->vz = pz * inv;
}

/* Henyey-Greenstein scatter: src/mmc_core.cl:1348-1377 */
static float next_scatter(float gg, ray* r, uint64_t* ran, float* mom) {
    float nextslen = -oracle_logf(oracle_rng_next(ran) + O_EPS);
    float sphi, cphi, stheta, ctheta;
    oracle_sincos2pi(oracle_rng_next(ran), &sphi, &cphi);
    if (gg > O_EPS) {
        float tmp0 = (1.f - gg * gg) / (1.f - gg + 2.f * gg * oracle_rng_next(ran));
        tmp0 *= tmp0;
        tmp0 = (1.f + gg * gg - tmp0) / (2.f * gg);
        tmp0 = fmaxf(-1.f, fminf(tmp0, 1.f));
        stheta = sqrtf(1.f - tmp0 * tmp0);
        ctheta = tmp0;
    } else {
        /* cos(acos(x)) = x, sin(acos(x)) = sqrt(1-x^2) */
        ctheta = 2.f * oracle_rng_next(ran) - 1.f;
        stheta = sqrtf(1.f - ctheta * ctheta);
    }
    rotatevector(r, stheta, ctheta, sphi, cphi);
    *mom += (1.f - ctheta);
    return nextslen;
}

/* centroid nudge at edge/vertex hits: src/mmc_core.cl:1390-1402 */
static void fixphoton(engine* g, ray* r) {
    const int* e = g->elem + 4 * (size_t)(r->eid - 1);
    float cx = 0.f, cy = 0.f, cz = 0.f;
    for (int i = 0; i < 4; i++) {
        const float* p = g->node + 3 * (size_t)(e[i] - 1);
        cx += p[0]; cy += p[1]; cz += p[2];
    }
    r->px += (cx * 0.25f - r->px) * O_FIX_PHOTON;
    r->py += (cy * 0.25f - r->py) * O_FIX_PHOTON;
    r->pz += (cz * 0.25f - r->pz) * O_FIX_PHOTON;
}

static int valid_eid(const engine* g, int eid) { return eid > 0 && eid <= g->ne; }

/* detector search: src/mmc_core.cl:608-621 */
static int finddetector(const engine* g, const ray* r) {
    const oracle_cfg* cfg = g->cfg;
    for (int i = 0; i < cfg->detnum; i++) {
        const float* d = cfg->detpos + 4 * i;
        if ((d[0] - r->px) * (d[0] - r->px) + (d[1] - r->py) * (d[1] - r->py) + (d[2] - r->pz) * (d[2] - r->pz) < d[3] * d[3])
            return i + 1;
    }
    return 0;
}

void oracle_grid_dims(int nn, const float* node, float step, int dim[3], float nmin[3]) {
    float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
    for (int i = 0; i < nn; i++)
        for (int k = 0; k < 3; k++) {
            if (node[3 * (size_t)i + k] < lo[k]) lo[k] = node[3 * (size_t)i + k];
            if (node[3 * (size_t)i + k] > hi[k]) hi[k] = node[3 * (size_t)i + k];
        }
    for (int k = 0; k < 3; k++) {
        lo[k] -= O_EPS;
        hi[k] += O_EPS;
        nmin[k] = lo[k];
        dim[k] = (int)((hi[k] - lo[k]) / step) + 1;
    }
}

static void grid_range(const float* node, const int* e, const locgrid* g, int b0[3], int b1[3]) {
    float mn[3] = {1e30f, 1e30f, 1e30f}, mx[3] = {-1e30f, -1e30f, -1e30f};
    for (int j = 0; j < 4; j++)
        for (int d = 0; d < 3; d++) {
            float v = node[3 * (size_t)(e[j] - 1) + d];
            if (v < mn[d]) mn[d] = v;
            if (v > mx[d]) mx[d] = v;
        }
    for (int d = 0; d < 3; d++) {
        int a = (int)floorf((mn[d] - g->lo[d]) * g->inv[d]);
        int b = (int)floorf((mx[d] - g->lo[d]) * g->inv[d]);
        b0[d] = a < 0 ? 0 : (a > g->res - 1 ? g->res - 1 : a);
        b1[d] = b < 0 ? 0 : (b > g->res - 1 ? g->res - 1 : b);
    }
}

static void grid_build(int nn, const float* node, int ne, const int* elem, locgrid* g) {
    float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
    for (int i = 0; i < nn; i++)
        for (int d = 0; d < 3; d++) {
            if (node[3 * (size_t)i + d] < lo[d]) lo[d] = node[3 * (size_t)i + d];
            if (node[3 * (size_t)i + d] > hi[d]) hi[d] = node[3 * (size_t)i + d];
        }
    int res = (int)cbrt((double)ne / 4.0);
    if (res < 1) res = 1;
    if (res > 256) res = 256;
    g->res = res;
    for (int d = 0; d < 3; d++) {
        float span = hi[d] - lo[d];
        g->lo[d] = lo[d];
        g->inv[d] = span > 0 ? res / span : 0.f;
    }
    size_t nbin = (size_t)res * res * res;
    g->start = (uint32_t*)calloc(nbin + 1, sizeof(uint32_t));
    int b0[3], b1[3];
    for (int e = 0; e < ne; e++) {
        grid_range(node, elem + 4 * (size_t)e, g, b0, b1);
        for (int z = b0[2]; z <= b1[2]; z++)
            for (int y = b0[1]; y <= b1[1]; y++)
                for (int x = b0[0]; x <= b1[0]; x++) g->start[((size_t)z * res + y) * res + x + 1]++;
    }
    for (size_t i = 0; i < nbin; i++) g->start[i + 1] += g->start[i];
    g->items = (uint32_t*)malloc(sizeof(uint32_t) * (g->start[nbin] ? g->start[nbin] : 1));
    uint32_t* fill = (uint32_t*)malloc(sizeof(uint32_t) * nbin);
    memcpy(fill, g->start, sizeof(uint32_t) * nbin);
    for (int e = 0; e < ne; e++) {
        grid_range(node, elem + 4 * (size_t)e, g, b0, b1);
        for (int z = b0[2]; z <= b1[2]; z++)
            for (int y = b0[1]; y <= b1[1]; y++)
                for (int x = b0[0]; x <= b1[0]; x++) g->items[fill[((size_t)z * res + y) * res + x]++] = (uint32_t)e;
    }
    free(fill);
}

/* barycentric test of the reference's source-element search
 * (src/mmc_raytrace.c:2599-2652): unnormalized face normals, tolerance -1e-4 */
static float face_bary(const float* a, const float* b, const float* c, float px, float py, float pz) {
    float abx = b[0] - a[0], aby = b[1] - a[1], abz = b[2] - a[2];
    float acx = c[0] - a[0], acy = c[1] - a[1], acz = c[2] - a[2];
    float sx = px - a[0], sy = py - a[1], sz = pz - a[2];
    float nx = aby * acz - abz * acy, ny = abz * acx - abx * acz, nz = abx * acy - aby * acx;
    return -((sx * nx + sy * ny) + sz * nz);
}

static int src_encloses(const engine* g, int e, float px, float py, float pz) {
    const int* el = g->elem + 4 * (size_t)e;
    const float* n0 = g->node + 3 * (size_t)(el[0] - 1);
    const float* n1 = g->node + 3 * (size_t)(el[1] - 1);
    const float* n2 = g->node + 3 * (size_t)(el[2] - 1);
    const float* n3 = g->node + 3 * (size_t)(el[3] - 1);
    float b2 = face_bary(n0, n3, n1, px, py, pz);
    float b0 = face_bary(n3, n2, n1, px, py, pz);
    float b1 = face_bary(n0, n2, n3, px, py, pz);
    float b3 = face_bary(n0, n1, n2, px, py, pz);
    return !(b0 < -1e-4f || b1 < -1e-4f || b2 < -1e-4f || b3 < -1e-4f);
}

/* lowest-index enclosing element in p's grid cell, else in the 26 neighbours */
static int src_locate(const engine* g, float px, float py, float pz) {
    const locgrid* G = g->grid;
    int res = G->res;
    float fx = (px - G->lo[0]) * G->inv[0], fy = (py - G->lo[1]) * G->inv[1], fz = (pz - G->lo[2]) * G->inv[2];
    float lo = -1e-3f * res, hi = res * (1.f + 1e-3f);
    if (!(fx >= lo) || !(fx <= hi) || !(fy >= lo) || !(fy <= hi) || !(fz >= lo) || !(fz <= hi)) return 0;
    int b[3] = {(int)floorf(fx), (int)floorf(fy), (int)floorf(fz)};
    for (int d = 0; d < 3; d++) b[d] = b[d] < 0 ? 0 : (b[d] > res - 1 ? res - 1 : b[d]);
    for (int pass = 0; pass < 2; pass++) {
        int best = 0x7FFFFFFF;
        for (int z = b[2] - pass; z <= b[2] + pass; z++)
            for (int y = b[1] - pass; y <= b[1] + pass; y++)
                for (int x = b[0] - pass; x <= b[0] + pass; x++) {
                    if (x < 0 || y < 0 || z < 0 || x >= res || y >= res || z >= res) continue;
                    size_t cell = ((size_t)z * res + y) * res + x;
                    for (uint32_t k = G->start[cell]; k < G->start[cell + 1]; k++) {
                        int e = (int)G->items[k];
                        if (e < best && src_encloses(g, e, px, py, pz)) best = e;
                    }
                }
        if (best != 0x7FFFFFFF) return best + 1;
    }
    return 0;
}

/* photon launch for every source type, src/mmc_raytrace.c:2346-2671 (the CPU
 * launch; the GPU version src/mmc_core.cl:1416-1834 differs in leaving
 * cone/arcsine/zgaussian directions unrotated and the disk radius without an
 * inner bound).  Restated with these changes, which the CUDA engine shares:
 * the cone's polar angle is sampled by inversion instead of rejection; acos
 * is replaced by the identities cos(acos x) = x, sin(acos x) = sqrt(1-x^2);
 * the Gaussian radius and angle add EPS inside the log; a photon is located
 * in the initial element first, then through the bounding-box grid (the
 * reference searches a user-labelled candidate list).  Returns 0 when no
 * element encloses the launch position. */
static int launch_photon(const engine* g, ray* r, uint64_t* ran) {
    const oracle_cfg* cfg = g->cfg;
    const float* p1 = cfg->srcparam1;
    const float* p2 = cfg->srcparam2;
    const int st = cfg->srctype;
    float ox = r->px, oy = r->py, oz = r->pz;
    int canfocus = 1;
    r->slen = -oracle_logf(oracle_rng_next(ran) + O_EPS);
    if (st == 0) {
        if (r->eid > 0) return 1;
    } else if (st == 4 || st == 5 || st == 15 || st == 6 || st == 14) {
        float rx = oracle_rng_next(ran);
        float ry = oracle_rng_next(ran);
        if (st == 15) {
            float rz = oracle_rng_next(ran);
            r->px = cfg->srcpos[0] + rx * p1[0];
            r->py = cfg->srcpos[1] + ry * p1[1];
            r->pz = cfg->srcpos[2] + rz * p1[2];
            int nx = (int)p1[0], ny = (int)p1[1], nz = (int)p1[2];
            int ix = (int)(rx * nx), iy = (int)(ry * ny), iz = (int)(rz * nz);
            if (ix > nx - 1) ix = nx - 1;
            if (iy > ny - 1) iy = ny - 1;
            if (iz > nz - 1) iz = nz - 1;
            r->weight = cfg->srcpattern[((size_t)iz * ny + iy) * nx + ix];
            ox += p1[0] * 0.5f; oy += p1[1] * 0.5f; oz += p1[2] * 0.5f;
        } else if (st == 14) {
            float fx = floorf(rx * p1[3]), fy = floorf(ry * p2[3]);
            r->px = cfg->srcpos[0] + fx * p1[0] / (p1[3] - 1.f) + fy * p2[0] / (p2[3] - 1.f);
            r->py = cfg->srcpos[1] + fx * p1[1] / (p1[3] - 1.f) + fy * p2[1] / (p2[3] - 1.f);
            r->pz = cfg->srcpos[2] + fx * p1[2] / (p1[3] - 1.f) + fy * p2[2] / (p2[3] - 1.f);
            ox += (p1[0] + p2[0]) * 0.5f; oy += (p1[1] + p2[1]) * 0.5f; oz += (p1[2] + p2[2]) * 0.5f;
        } else {
            r->px = cfg->srcpos[0] + rx * p1[0] + ry * p2[0];
            r->py = cfg->srcpos[1] + rx * p1[1] + ry * p2[1];
            r->pz = cfg->srcpos[2] + rx * p1[2] + ry * p2[2];
            if (st == 5) {
                int nx = (int)p1[3], ny = (int)p2[3];
                int iy = (int)(ry * ny), ix = (int)(rx * nx);
                if (iy > ny - 1) iy = ny - 1;
                if (ix > nx - 1) ix = nx - 1;
                /* with several patterns the photon starts with weight 1 (src/mmc_raytrace.c:2394) */
                r->posidx = iy * nx + ix;
                r->weight = (g->K > 1) ? 1.f : cfg->srcpattern[iy * nx + ix];
            } else if (st == 6) {
                float sv, cv;
                oracle_sincos2pi(floorf(p1[3]) * rx + floorf(p2[3]) * ry + p1[3] - floorf(p1[3]), &sv, &cv);
                r->weight = (cv * (1.f - p2[3] + floorf(p2[3])) + 1.f) * 0.5f;
            }
            ox += (p1[0] + p2[0]) * 0.5f; oy += (p1[1] + p2[1]) * 0.5f; oz += (p1[2] + p2[2]) * 0.5f;
        }
    } else if (st == 9 || st == 10) {
        float rx = oracle_rng_next(ran);
        float ry = oracle_rng_next(ran);
        float w = p1[3] * (1.f / sqrtf(p1[0] * p1[0] + p1[1] * p1[1] + p1[2] * p1[2]));
        float v2x = w * (cfg->srcdir[1] * p1[2] - cfg->srcdir[2] * p1[1]);
        float v2y = w * (cfg->srcdir[2] * p1[0] - cfg->srcdir[0] * p1[2]);
        float v2z = w * (cfg->srcdir[0] * p1[1] - cfg->srcdir[1] * p1[0]);
        r->px = cfg->srcpos[0] + rx * p1[0] + ry * v2x;
        r->py = cfg->srcpos[1] + rx * p1[1] + ry * v2y;
        r->pz = cfg->srcpos[2] + rx * p1[2] + ry * v2z;
        float s1, c1, s2, c2;
        if (st == 10) {
            oracle_sincos2pi(p2[0] * rx + p2[2], &s1, &c1);
            oracle_sincos2pi(p2[1] * ry + p2[3], &s2, &c2);
            r->weight = (s1 * s2 + 1.f) * 0.5f;
        } else {
            oracle_sincos2pi(p2[0] * rx + p2[1] * ry + p2[2], &s1, &c1);
            r->weight = (c1 * (1.f - p2[3]) + 1.f) * 0.5f;
        }
        ox += (p1[0] + v2x) * 0.5f; oy += (p1[1] + v2y) * 0.5f; oz += (p1[2] + v2z) * 0.5f;
    } else if (st == 8 || st == 17 || st == 3) {
        float sphi, cphi, r0;
        if (st == 17 && (p1[2] > 0.f || p1[3] > 0.f)) {
            float phi = fabsf(p1[2] - p1[3]) * oracle_rng_next(ran) + fminf(p1[2], p1[3]);
            oracle_sincos2pi(phi * (0.5f / O_PI), &sphi, &cphi);
        } else {
            oracle_sincos2pi(oracle_rng_next(ran), &sphi, &cphi);
        }
        if (st == 8 || st == 17) {
            r0 = sqrtf(oracle_rng_next(ran) * fabsf(p1[0] * p1[0] - p1[1] * p1[1]) + p1[1] * p1[1]);
        } else if (fabsf(cfg->focus) < 1e-5f || fabsf(p1[1]) < 1e-5f) {
            r0 = sqrtf(-oracle_logf(oracle_rng_next(ran) + O_EPS)) * p1[0];
        } else {
            float z0 = p1[0] * p1[0] * O_PI / p1[1];
            r0 = sqrtf(-oracle_logf(oracle_rng_next(ran) + O_EPS) * (1.f + (cfg->focus * cfg->focus / (z0 * z0)))) * p1[0];
        }
        float dx = cfg->srcdir[0], dy = cfg->srcdir[1], dz = cfg->srcdir[2];
        if (dz > -1.f + O_EPS && dz < 1.f - O_EPS) {
            float tmp0 = 1.f - dz * dz;
            float tmp1 = r0 / sqrtf(tmp0);
            r->px = cfg->srcpos[0] + tmp1 * (dx * dz * cphi - dy * sphi);
            r->py = cfg->srcpos[1] + tmp1 * (dy * dz * cphi + dx * sphi);
            r->pz = cfg->srcpos[2] - tmp1 * tmp0 * cphi;
        } else {
            r->px += r0 * cphi;
            r->py += r0 * sphi;
        }
    } else if (st == 2 || st == 1 || st == 7) {
        float sphi, cphi, stheta, ctheta;
        oracle_sincos2pi(oracle_rng_next(ran), &sphi, &cphi);
        if (st == 2) {
            float u = oracle_rng_next(ran);
            if (p1[1] > 0.f) {
                oracle_sincos2pi(u * p1[0] * (0.5f / O_PI), &stheta, &ctheta);
            } else {
                float sa, ca;
                oracle_sincos2pi(p1[0] * (0.5f / O_PI), &sa, &ca);
                ctheta = 1.f - u * (1.f - ca);
                stheta = sqrtf(fmaxf(0.f, 1.f - ctheta * ctheta));
            }
        } else if (st == 1) {
            ctheta = 2.f * oracle_rng_next(ran) - 1.f;
            stheta = sqrtf(fmaxf(0.f, 1.f - ctheta * ctheta));
        } else {
            oracle_sincos2pi(0.5f * oracle_rng_next(ran), &stheta, &ctheta);
        }
        rotatevector(r, stheta, ctheta, sphi, cphi);
        canfocus = 0;
        if (r->eid > 0) return 1;
    } else if (st == 11) {
        float sphi, cphi, stheta, ctheta;
        oracle_sincos2pi(oracle_rng_next(ran), &sphi, &cphi);
        float u1 = oracle_rng_next(ran);
        float u2 = oracle_rng_next(ran);
        float ang = sqrtf(-2.f * oracle_logf(u1 + O_EPS)) * (1.f - 2.f * u2) * p1[0];
        oracle_sincos2pi(ang * (0.5f / O_PI), &stheta, &ctheta);
        rotatevector(r, stheta, ctheta, sphi, cphi);
        canfocus = 0;
    } else if (st == 16) {
        float sphi, cphi;
        oracle_sincos2pi(oracle_rng_next(ran), &sphi, &cphi);
        float r0 = sqrtf(0.5f * -oracle_logf(oracle_rng_next(ran) + O_EPS)) * p1[0];
        float tilt = (p1[2] > 0.f) ? (-p1[1] / p1[2]) : 0.f;
        float bx = -r0 * sphi, by = r0 * cphi, bz = p1[2];
        float nb = 1.f / sqrtf(bx * bx + by * by + bz * bz);
        bx *= nb; by *= nb; bz *= nb;
        float qx = r0 * (cphi - tilt * sphi), qy = r0 * (sphi + tilt * cphi);
        float dx = cfg->srcdir[0], dy = cfg->srcdir[1], dz = cfg->srcdir[2];
        if (dz > -1.f + O_EPS && dz < 1.f - O_EPS) {
            float sint = sqrtf(1.f - dz * dz);
            float isint = 1.f / sint;
            float cb = dx * isint, sb = dy * isint;
            r->px = cfg->srcpos[0] + qx * cb * dz - qy * sb;
            r->py = cfg->srcpos[1] + qx * sb * dz + qy * cb;
            r->pz = cfg->srcpos[2] - qx * sint;
            r->vx = bx * cb * dz - by * sb + bz * cb * sint;
            r->vy = bx * sb * dz + by * cb + bz * sb * sint;
            r->vz = -bx * sint + bz * dz;
        } else {
            r->px = cfg->srcpos[0] + qx;
            r->py = cfg->srcpos[1] + qy;
            r->pz = cfg->srcpos[2];
            r->vx = bx; r->vy = by;
            r->vz = (dz > 0.f) ? bz : -bz;
        }
        float nv = 1.f / sqrtf(r->vx * r->vx + r->vy * r->vy + r->vz * r->vz);
        r->vx *= nv; r->vy *= nv; r->vz *= nv;
        canfocus = 0;
    } else if (st == 12 || st == 13) {
        float t = oracle_rng_next(ran);
        r->px += t * p1[0]; r->py += t * p1[1]; r->pz += t * p1[2];
        if (st == 12) {
            t = 1.f - 2.f * oracle_rng_next(ran);
            float s = 1.f - 2.f * oracle_rng_next(ran);
            float sign = (oracle_rng_next(ran) > 0.5f) ? 1.f : -1.f;
            float p = sqrtf(1.f - r->vx * r->vx - r->vy * r->vy) * sign;
            float vx = r->vy * p - r->vz * s, vy = r->vz * t - r->vx * p, vz = r->vx * s - r->vy * t;
            r->vx = vx; r->vy = vy; r->vz = vz;
        }
        ox += p1[0] * 0.5f; oy += p1[1] * 0.5f; oz += p1[2] * 0.5f;
        canfocus = (st == 13);
    }
    if (canfocus) {
        float f = cfg->focus;
        if (f != f) {
            float sphi, cphi;
            oracle_sincos2pi(oracle_rng_next(ran), &sphi, &cphi);
            float ctheta = 2.f * oracle_rng_next(ran) - 1.f;
            rotatevector(r, sqrtf(fmaxf(0.f, 1.f - ctheta * ctheta)), ctheta, sphi, cphi);
        } else if (f < 0.f && isinf(f)) {
            float sphi, cphi;
            oracle_sincos2pi(oracle_rng_next(ran), &sphi, &cphi);
            float stheta = sqrtf(oracle_rng_next(ran));
            rotatevector(r, stheta, sqrtf(1.f - stheta * stheta), sphi, cphi);
        } else if (f != 0.f) {
            ox += f * r->vx; oy += f * r->vy; oz += f * r->vz;
            float vx, vy, vz;
            if (f < 0.f) { vx = r->px - ox; vy = r->py - oy; vz = r->pz - oz; }
            else { vx = ox - r->px; vy = oy - r->py; vz = oz - r->pz; }
            float rn = 1.f / sqrtf(vx * vx + vy * vy + vz * vz);
            r->vx = vx * rn; r->vy = vy * rn; r->vz = vz * rn;
        }
    }
    r->px = r->px + r->vx * O_EPS;
    r->py = r->py + r->vy * O_EPS;
    r->pz = r->pz + r->vz * O_EPS;
    int e = 0;
    if (r->eid > 0 && src_encloses(g, r->eid - 1, r->px, r->py, r->pz)) e = r->eid;
    else if (g->grid) e = src_locate(g, r->px, r->py, r->pz);
    if (e <= 0) return 0;
    r->eid = e;
    return 1;
}

typedef struct {
    double etot, eesc;
    uint64_t raytet;
    uint64_t aborted;
    uint64_t outside;
    double* esrc;    /* srcnum > 1: launched weight per pattern, then escaped (2*srcnum) */
} tallies;

/* a shared photon's launched (which 0) or escaped (1) weight per pattern (src/mmc_core.cl:
 * 1907-1911, :2154-2159) */
static void tally_src(const engine* g, const ray* r, tallies* tl, int which) {
    const float* pat = g->cfg->srcpattern + (size_t)r->posidx * g->K;
    for (int p = 0; p < g->K; p++) tl->esrc[which * g->K + p] += (double)(r->weight * pat[p]);
}

/* the photon life: src/mmc_core.cl:1851-2161 */
/* One trajectory record, savedebugdata in src/mmc_raytrace.c:1739-1756:
 * photon id, position, weight and element (the ids as raw 32-bit words). */
static void save_traj(const engine* g, const ray* r, uint64_t pidx, oracle_out* out) {
    uint32_t pos;
#pragma omp atomic capture
    pos = out->ntraj++;
    if (pos < out->maxtraj) {
        float* rec = out->traj + (size_t)pos * 6;
        uint32_t id = (uint32_t)(g->cfg->photon_offset + pidx);
        int32_t eid = r->eid;
        memcpy(rec, &id, 4);
        rec[1] = r->px; rec[2] = r->py; rec[3] = r->pz;
        rec[4] = r->weight;
        memcpy(rec + 5, &eid, 4);
    }
}

static void onephoton(engine* g, uint64_t pidx, float* ppath, oracle_out* out, tallies* tl) {
    const oracle_cfg* cfg = g->cfg;
    const int M = g->M;
    const int reclen = g->reclen;
    uint64_t ran[2], seed0[2];
    uint32_t photonid = (uint32_t)pidx;
    if (cfg->replayseed) {
        ran[0] = cfg->replayseed[2 * pidx];
        ran[1] = cfg->replayseed[2 * pidx + 1];
    } else {
        oracle_rng_seed(cfg->seed, cfg->photon_offset + pidx, ran);
    }
    seed0[0] = ran[0]; seed0[1] = ran[1];
    ray rr;
    ray* r = &rr;
    memset(r, 0, sizeof(ray));
    r->px = cfg->srcpos[0]; r->py = cfg->srcpos[1]; r->pz = cfg->srcpos[2];
    r->vx = cfg->srcdir[0]; r->vy = cfg->srcdir[1]; r->vz = cfg->srcdir[2];
    r->ox = O_UNDEF;
    r->eid = cfg->e0;
    r->weight = 1.f;
    r->oldidx = (uint32_t)O_ID_UNDEF;
    r->photonid = photonid;
    memset(ppath, 0, sizeof(float) * (size_t)reclen);
    int fixcount = 0, oldeid = 0, detid = 0;
    uint64_t steps = 0;
    int aborted = 0;
    /* launch: src/mmc_raytrace.c:2346-2671 */
    const int placed = launch_photon(g, r, ran);
    /* the last record column: the initial weight, or a shared photon's launch pixel */
    if (cfg->issavedet) ppath[reclen - 1] = (g->K > 1) ? bits2f((uint32_t)r->posidx) : r->weight;
    tl->etot += r->weight;
    if (g->K > 1) tally_src(g, r, tl, 0);
    if (!placed) {
        tl->outside++;
        tl->eesc += r->weight;
        if (g->K > 1) tally_src(g, r, tl, 1);
        if (out->photon_weight) out->photon_weight[pidx] = r->weight;
        if (out->photon_steps) out->photon_steps[pidx] = 0;
        if (out->photon_det) out->photon_det[pidx] = 0;
        return;
    }
    if (out->traj) save_traj(g, r, pidx, out);   /* src/mmc_raytrace.c:1804-1806 */

#define STEP()                                                         \
    do {                                                               \
        r->slen = raytet_step(g, r);                                   \
        steps++;                                                       \
        if (steps > cfg->step_budget) { aborted = 1; goto done; }      \
    } while (0)
#define PPATH()                                                                       \
    do {                                                                              \
        if (cfg->issavedet && r->Lmove > 0.f && valid_eid(g, r->eid)) {               \
            int tp = g->type[r->eid - 1];                                             \
            if (tp > 0) ppath[M + tp - 1] += r->Lmove;                                \
        }                                                                             \
    } while (0)

    while (1) {
        STEP();
        if (r->ox == O_UNDEF) {
            if (r->faceid == -2) break;
            if (fixcount++ < O_MAX_TRIAL) {
                fixphoton(g, r);
                continue;
            }
            r->eid = O_ID_UNDEF;
            r->faceid = -1;
        }
        PPATH();
        while (r->faceid >= 0 && !r->isend) {
            r->px = r->ox; r->py = r->oy; r->pz = r->oz;
            oldeid = r->eid;
            r->eid = g->facenb[4 * (size_t)(r->eid - 1) + r->faceid];
            if (cfg->isreflect) {
                float nold = medium(g, g->type[oldeid - 1], 3);
                if (r->eid <= 0 || medium(g, g->type[r->eid - 1], 3) != nold) {
                    if (!(r->eid <= 0 && (((nold == cfg->nout) && (cfg->isreflect != BC_MIRROR)) || (cfg->isreflect == BC_ABSORBEXT))))
                        reflectray(g, r, oldeid, &r->eid, r->faceid, ran);
                }
            }
            if (r->eid <= 0) break;
            if (g->type[oldeid - 1] == 0 && g->type[r->eid - 1]) {
                if (!cfg->voidtime) r->photontimer = 0.f;
            }
            if (g->type[oldeid - 1] && g->type[r->eid - 1] == 0) {
                r->eid = 0;
                break;
            }
            STEP();
            PPATH();
            if (r->faceid == -2) break;
            fixcount = 0;
            while (r->ox == O_UNDEF && fixcount++ < O_MAX_TRIAL) {
                fixphoton(g, r);
                STEP();
                PPATH();
            }
            if (r->ox == O_UNDEF) {
                r->eid = O_ID_UNDEF;
                break;
            }
        }
        if (r->eid <= 0 || r->ox == O_UNDEF) {
            if (r->eid != O_ID_UNDEF && cfg->issavedet && cfg->issaveexit) {
                ppath[reclen - 7] = r->px; ppath[reclen - 6] = r->py; ppath[reclen - 5] = r->pz;
                ppath[reclen - 4] = r->vx; ppath[reclen - 3] = r->vy; ppath[reclen - 2] = r->vz;
            }
            /* diffuse reflectance per exterior face: src/mmc_raytrace.c:2000-2003 */
            if (cfg->issaveref && out->dref && r->eid < 0 && -r->eid <= out->nf) {
                float gf = (r->photontimer - cfg->tstart) * g->Rtstep;
                int gate = (gf < (float)(g->maxgate - 1)) ? (int)gf : g->maxgate - 1;
                if (gate < 0) gate = 0;
#pragma omp atomic
                out->dref[((-r->eid) - 1) + (size_t)gate * out->nf] += (double)r->weight;
            }
            if (cfg->issavedet && r->eid <= 0) {
                /* savedetphoton: src/mmc_core.cl:624-682 */
                detid = finddetector(g, r);
                if (detid) {
                    uint32_t slot;
#pragma omp atomic capture
                    slot = out->detected++;
                    if (slot < cfg->maxdetphoton) {
                        if (out->seeds) memcpy(out->seeds + 16 * (size_t)slot, seed0, 16);
                        if (out->detp) {
                            float* rec = out->detp + (size_t)slot * (reclen + 1);
                            rec[0] = (float)detid;
                            for (int i = 0; i < reclen; i++) rec[1 + i] = ppath[i];
                        }
                    }
                }
            }
            break;
        }
        /* Russian roulette: src/mmc_core.cl:2101-2114 */
        if ((cfg->minenergy > 0.f) && (r->weight < cfg->minenergy) && ((cfg->tend - cfg->tstart) * g->Rtstep <= 1.f)) {
            if (oracle_rng_next(ran) * cfg->roulettesize <= 1.f) {
                r->weight *= cfg->roulettesize;
            } else {
                break;
            }
        }
        if (cfg->replayseed && cfg->outputtype == OT_WN) {
            /* replay weight once per scattering event, in the element where it happens */
            float gf = cfg->replaytime[r->photonid] * g->Rtstep;
            int gate = (gf < (float)(g->maxgate - 1)) ? (int)gf : g->maxgate - 1;
            if (gate < 0) gate = 0;
            deposit(g, (uint32_t)(r->eid - 1) + (uint32_t)(gate * g->ne), cfg->replayweight[r->photonid]);
        }
        float mom = 0.f;
        int tp = g->type[r->eid - 1];
        r->slen0 = next_scatter(medium(g, tp, 2), r, ran, &mom);
        r->slen = r->slen0;
        if (out->traj) save_traj(g, r, pidx, out);   /* src/mmc_raytrace.c:2065-2067 */
        if (cfg->issavedet) {
            if (cfg->ismomentum && tp > 0) ppath[2 * M + tp - 1] += mom;
            if (tp > 0) ppath[tp - 1] += 1.f;
        }
    }
done:
#undef STEP
#undef PPATH
    if (out->traj) save_traj(g, r, pidx, out);   /* src/mmc_raytrace.c:2109-2111 */
    tl->eesc += r->weight;
    if (g->K > 1) tally_src(g, r, tl, 1);
    tl->raytet += steps;
    tl->aborted += aborted;
    if (out->photon_weight) out->photon_weight[pidx] = r->weight;
    if (out->photon_steps) out->photon_steps[pidx] = (uint32_t)steps;
    if (out->photon_det) out->photon_det[pidx] = detid;
}

int oracle_run(int nn, const float* node, int ne, const int* elem, const int* label,
               const oracle_cfg* cfg, oracle_out* out, int nthreads) {
    int* ee = (int*)malloc(sizeof(int) * (size_t)ne * 4);
    int* fnb = (int*)malloc(sizeof(int) * (size_t)ne * 4);
    float* nrm = (float*)malloc(sizeof(float) * (size_t)ne * 16);
    float* evol = (float*)malloc(sizeof(float) * (size_t)ne);
    float* nvol = (float*)malloc(sizeof(float) * (size_t)nn);
    int nf = 0, rc = 0;
    if (oracle_prep_mesh(nn, node, ne, elem, label, NULL, ee, fnb, nrm, evol, nvol, &nf) != 0) {
        rc = -1;
        goto cleanup;
    }
    engine g;
    memset(&g, 0, sizeof(g));
    g.ne = ne; g.nn = nn; g.M = cfg->nmedia - 1;
    g.node = node; g.elem = ee; g.type = label; g.facenb = fnb; g.nrm = nrm; g.cfg = cfg;
    locgrid grid;
    memset(&grid, 0, sizeof(grid));
    if (!(cfg->srctype == 0 && cfg->e0 > 0)) {
        grid_build(nn, node, ne, ee, &grid);
        g.grid = &grid;
    }
    g.Rtstep = 1.f / cfg->tstep;
    g.maxgate = cfg->maxgate;
    g.reclen = (2 + (cfg->ismomentum > 0)) * g.M + (cfg->issaveexit > 0) * 6 + 1;
    g.K = (cfg->srcnum > 1 && cfg->srctype == 5) ? cfg->srcnum : 1;
    out->reclen = g.reclen + 1;
    out->nf = nf;
    if (out->dref) memset(out->dref, 0, sizeof(double) * (size_t)nf * cfg->maxgate);
    g.framelen = (uint32_t)ne;
    if (cfg->method == 1) {
        int d[3];
        float step = cfg->gridstep > 0.f ? cfg->gridstep : 1.f;
        oracle_grid_dims(nn, node, step, d, g.gmin);
        g.dgrid = 1;
        g.gstep_inv = 1.f / step;
        for (int k = 0; k < 3; k++) g.gdim[k] = (uint32_t)d[k];
        g.framelen = (uint32_t)d[0] * (uint32_t)d[1] * (uint32_t)d[2];
    }
    size_t flen = (size_t)g.framelen * cfg->maxgate * g.K;
    if (out->energy_src && g.K > 1) memset(out->energy_src, 0, sizeof(double) * 2 * g.K);
    if (cfg->accum_f64) {
        g.f64 = out->field_raw;
        memset(g.f64, 0, sizeof(double) * flen);
    } else {
        g.f32a = (float*)calloc(flen, sizeof(float));
        g.f32b = (float*)calloc(flen, sizeof(float));
    }
    out->detected = 0;
    double etot = 0, eesc = 0;
    uint64_t raytet = 0, aborted = 0, outside = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    /* the photon loop alone is timed, as the reference times its speed report (src/mmc_host.c:194, :359-362) */
    struct timespec t_start, t_end;
    clock_gettime(CLOCK_MONOTONIC, &t_start);
#pragma omp parallel reduction(+:etot, eesc, raytet, aborted, outside)
    {
        float* ppath = (float*)calloc((size_t)g.reclen + 1, sizeof(float));
        tallies tl = {0, 0, 0, 0, 0, NULL};
        if (g.K > 1) tl.esrc = (double*)calloc(2 * (size_t)g.K, sizeof(double));
#pragma omp for schedule(dynamic, 64)
        for (long long i = 0; i < (long long)cfg->nphoton; i++) onephoton(&g, (uint64_t)i, ppath, out, &tl);
        etot += tl.etot; eesc += tl.eesc; raytet += tl.raytet; aborted += tl.aborted; outside += tl.outside;
        if (tl.esrc) {
#pragma omp critical
            for (int k = 0; k < 2 * g.K; k++)
                if (out->energy_src) out->energy_src[k] += tl.esrc[k];
            free(tl.esrc);
        }
        free(ppath);
    }
    clock_gettime(CLOCK_MONOTONIC, &t_end);
    out->sim_seconds = (double)(t_end.tv_sec - t_start.tv_sec) + 1e-9 * (double)(t_end.tv_nsec - t_start.tv_nsec);
    out->energytot = etot;
    out->energyesc = eesc;
    if (g.K > 1 && out->energy_src) {  /* the patterns' sums, as the reference reports them */
        out->energytot = out->energyesc = 0.0;
        for (int k = 0; k < g.K; k++) {
            out->energytot += out->energy_src[k];
            out->energyesc += out->energy_src[g.K + k];
        }
    }
    out->raytet = raytet;
    out->aborted = aborted;
    out->outside = outside;
    free(grid.start);
    free(grid.items);
    if (!cfg->accum_f64) {
        for (size_t i = 0; i < flen; i++) out->field_raw[i] = (double)g.f32a[i] + (double)g.f32b[i];
        free(g.f32a);
        free(g.f32b);
    }
cleanup:
    free(ee); free(fnb); free(nrm); free(evol); free(nvol);
    return rc;
}

/* ======================================================================
 * output stage
 * ====================================================================== */
/* effective reflection coefficient: src/mmc_mesh.c:2305-2334 */
static double getreff(double n_in, double n_out) {
    double oc = asin(1.0 / n_in);
    const double count = 1000.0;
    const double ostep = (3.14159265358979323846 / (2.0 * count));
    double r_phi = 0.0, r_j = 0.0;
    for (int i = 0; i < count; i++) {
        double o = i * ostep, coso = cos(o), r_fres, cosop, tmp;
        if (o < oc) {
            cosop = n_in * sin(o);
            cosop = sqrt(1. - cosop * cosop);
            tmp = (n_in * cosop - n_out * coso) / (n_in * cosop + n_out * coso);
            r_fres = 0.5 * tmp * tmp;
            tmp = (n_in * coso - n_out * cosop) / (n_in * coso + n_out * cosop);
            r_fres += 0.5 * tmp * tmp;
        } else {
            r_fres = 1.f;
        }
        r_phi += 2.0 * sin(o) * coso * r_fres;
        r_j += 3.0 * sin(o) * coso * coso * r_fres;
    }
    r_phi *= ostep;
    r_j *= ostep;
    return (r_phi + r_j) / (2.0 - r_phi + r_j);
}

double oracle_normalize(int nn, const float* node, int ne, const int* elem, const int* label,
                        const oracle_cfg* cfg, const double* raw, double energytot,
                        double energyesc, double* field) {
    int* ee = (int*)malloc(sizeof(int) * (size_t)ne * 4);
    int* fnb = (int*)malloc(sizeof(int) * (size_t)ne * 4);
    float* nrm = (float*)malloc(sizeof(float) * (size_t)ne * 16);
    float* evol = (float*)malloc(sizeof(float) * (size_t)ne);
    float* nvol = (float*)malloc(sizeof(float) * (size_t)nn);
    int nf = 0, prop = cfg->nmedia - 1, G = cfg->maxgate;
    const float* med = cfg->media;
    double normalizor = 1.0;
    oracle_prep_mesh(nn, node, ne, elem, label, NULL, ee, fnb, nrm, evol, nvol, &nf);
    int datalen = cfg->basisorder ? nn : ne;
    /* surface nodal volume fix: src/mmc_mesh.c:1344-1386 (faces with no
     * neighbour are the ones prep numbered negative) */
    if (cfg->isnormalized == 1 && cfg->basisorder) {
        float* Reff = (float*)calloc((size_t)prop + 1, sizeof(float));
        if (cfg->isreflect) {
            for (int i = 1; i <= prop; i++) {
                for (int j = 1; j < i; j++)
                    if (med[4 * j + 3] == med[4 * i + 3]) { Reff[i] = Reff[j]; break; }
                if (Reff[i] == 0.f) Reff[i] = (float)getreff(med[4 * i + 3], med[3]);
            }
        }
        for (int i = 0; i < ne; i++)
            for (int j = 0; j < 4; j++)
                if (fnb[4 * i + j] < 0) {
                    for (int k = 0; k < 3; k++) {
                        int nid = ee[4 * i + OUTF[IFACEORDER[j]][k]] - 1;
                        if (nvol[nid] > 0.f && label[i] >= 0)
                            nvol[nid] *= -(2.f / (1.0 + Reff[label[i]]));
                    }
                }
        for (int i = 0; i < nn; i++)
            if (nvol[i] < 0.f) nvol[i] = -nvol[i];
        free(Reff);
    }
    /* elem -> node scatter: src/mmc_cu_host.cu:916-976 */
    memset(field, 0, sizeof(double) * (size_t)datalen * G);
    if (!cfg->basisorder) {
        for (size_t i = 0; i < (size_t)ne * G; i++) field[i] = raw[i];
    } else {
        for (int i = 0; i < G; i++)
            for (int j = 0; j < ne; j++) {
                double ww = raw[(size_t)i * ne + j] * 0.25;
                for (int k = 0; k < 4; k++) field[(size_t)i * nn + ee[4 * j + k] - 1] += ww;
            }
    }
    if (cfg->isnormalized) {
        /* src/mmc_mesh.c:2154-2279 (single source) */
        float Etotal = (float)energytot;
        float Eabsorb = (float)(energytot - energyesc);
        int replay = (cfg->replayseed != NULL);
        if (replay && (cfg->outputtype == OT_JACOBIAN || cfg->outputtype == OT_WL || cfg->outputtype == OT_WP ||
                       cfg->outputtype == OT_WN)) {
            normalizor = 1.f / (O_DELTA_MUA * cfg->nphoton);
            if (cfg->outputtype != OT_JACOBIAN) normalizor = 1.f / Etotal;
        } else if (cfg->outputtype == OT_ENERGY) {
            normalizor = 1.f / Etotal;
        } else {
            double energydeposit = 0.0;
            if (cfg->basisorder) {
                for (int i = 0; i < G; i++)
                    for (int j = 0; j < datalen; j++)
                        if (nvol[j] > 0.f) field[(size_t)i * datalen + j] /= nvol[j];
                for (int i = 0; i < ne; i++) {
                    double energyelem = 0.0;
                    for (int j = 0; j < G; j++)
                        for (int k = 0; k < 4; k++) energyelem += field[(size_t)j * nn + ee[4 * i + k] - 1];
                    energydeposit += energyelem * evol[i] * med[4 * label[i]];
                }
                normalizor = Eabsorb / (Etotal * energydeposit * 0.25f);
            } else {
                for (int i = 0; i < datalen; i++)
                    for (int j = 0; j < G; j++) energydeposit += field[(size_t)j * datalen + i];
                for (int i = 0; i < datalen; i++) {
                    double energyelem = evol[i] * med[4 * label[i]];
                    for (int j = 0; j < G; j++) field[(size_t)j * datalen + i] /= energyelem;
                }
                normalizor = Eabsorb / (Etotal * energydeposit);
            }
            if (cfg->outputtype == OT_FLUX) normalizor /= cfg->tstep;
        }
        for (size_t i = 0; i < (size_t)datalen * G; i++) field[i] *= normalizor;
    }
    free(ee); free(fnb); free(nrm); free(evol); free(nvol);
    return normalizor;
}

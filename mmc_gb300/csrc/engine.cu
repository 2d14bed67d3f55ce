// GB300 photon engine: persistent, flat per-lane state machine over the
// reference's per-photon algorithm (src/mmc_core.cl:1851-2161, one ray-tet step
// per loop trip instead of the reference's nested scatter/crossing loops, so
// every lane of a warp does one step per trip whatever phase its photon is in).
//
// Each trip:  (1) lanes whose photon ended draw new photon ids from a global
//             counter (one atomic per warp), (2) every live lane performs one
//             branchless Badouel ray-tet step (src/mmc_core.cl:721-1226) with
//             the deposit fused in, (3) the lane applies the reference's
//             post-step control flow (fix/cross/reflect/exit/detect/roulette/
//             scatter) as a state transition.
// The file is compiled twice, with -fmad=false: MMCGB_ENGINE_FAST=0 builds the
// ExactMath kernels, whose float sequence is the contract shared with the CPU
// oracle (no contraction; the polynomial exp/log/sincos of devmath.cuh), and
// MMCGB_ENGINE_FAST=1 the FastMath kernels, which fuse multiply-adds only where
// the policy says so (MP::mad, MP::msub, MP::plane), so every kernel of a policy
// computes the same floats (a simulation gives the same result alone, batched
// or phased).  The fast unit also holds the dispatchers that pick a policy per
// simulation.
#if !defined(MMCGB_ENGINE_FAST) || (MMCGB_ENGINE_FAST != 0 && MMCGB_ENGINE_FAST != 1)
#error "compile engine.cu with -DMMCGB_ENGINE_FAST=0 (exact kernels) or =1 (fast kernels)"
#endif
#include <cooperative_groups.h>
#include <algorithm>
#include <cstdio>
#include "devmath.cuh"
#include "engine.h"

namespace cg = cooperative_groups;

namespace mmcgb {

namespace {

constexpr float kEps = 1e-6f;                     // src/mmc_mesh.h:70 (EPS in the CUDA build)
constexpr float kRC0 = 3.335640951981520e-12f;    // 1/c0 in s/mm
constexpr float kMaxAccum = 1000.f;               // src/mmc_core.cl:352
constexpr float kRMinMus = 1e9f;
constexpr float kFixPhoton = 1e-3f;
constexpr int kMaxTrial = 3;
constexpr int kIdUndef = 0x7FFFFFFF;
constexpr unsigned kFull = 0xFFFFFFFFu;

enum Mode : int { M_NEED = 0, M_OUTER = 1, M_INNER = 2, M_FIXIN = 3, M_DONE = 4, M_SCAT = 5 };
// modes of a photon in flight (it can be parked between gate windows)
constexpr unsigned kLiveModes = (1u << M_OUTER) | (1u << M_INNER) | (1u << M_FIXIN) | (1u << M_SCAT);
// modes that take no ray-tet step in the current trip
constexpr unsigned kIdleModes = (1u << M_NEED) | (1u << M_DONE) | (1u << M_SCAT);

// Kernel kinds: the lean pencil kernels, the pencil kernel with Russian roulette
// (single-window runs with minenergy > 0), and the general kernels (every
// source type, dual-grid output, trajectories, trace outputs, momentum).
enum KernelKind : int { KIND_LEAN = 0, KIND_ROULETTE = 1, KIND_GENERAL = 2 };

// Scattering runs at the top of the trip after the step that ends inside an
// element (roulette, then the scatter), ahead of that lane's next step.
// Batching it across lanes (a lane waiting until 8 lanes of its warp need a
// scatter, or for 4 trips) measured 4% slower on GB300 than scattering at once.

struct Lane {
    float px, py, pz, vx, vy, vz;
    float weight, ptime, slen, Lmove, slen0, oldw;
    unsigned oldidx;
    int eid, faceid, isend, hit, label, nbword;
    int fixcount, mode;
    unsigned steps;
    unsigned long long t0, t1;
    unsigned long long pid;  // photon index inside its simulation
    int sim;
    int posidx;  // launch pixel of a photon shared by several patterns (general kernels only)
};

// Arithmetic policies.  Exact: IEEE division and square root, the project's
// polynomial exp/log/sincos, no contraction -- bit-identical to the CPU
// oracle.  Fast: hardware approximations (__fdividef, __expf, __logf,
// __sincosf, rsqrtf), fused multiply-adds and float denormals flushed to zero
// (its translation unit is built with -ftz=true), as the reference's CUDA
// build gets from -use_fast_math; validated statistically.
struct ExactMath {
    static __device__ __forceinline__ float div(float a, float b) { return a / b; }
    static __device__ __forceinline__ float exp(float x) { return mmc_expf(x); }
    static __device__ __forceinline__ float log(float x) { return mmc_logf(x); }
    static __device__ __forceinline__ void sincos2pi(float u, float& s, float& c) { mmc_sincos2pi(u, s, c); }
    static __device__ __forceinline__ float rsqrt(float x) { return 1.f / sqrtf(x); }
    static __device__ __forceinline__ float mad(float a, float b, float c) { return a * b + c; }
    static __device__ __forceinline__ float msub(float a, float b, float c) { return c - a * b; }
    // d - p.n of a face plane, summed as the oracle does
    static __device__ __forceinline__ float plane(float d, float px, float py, float pz, float nx, float ny,
                                                  float nz) {
        return d - ((px * nx + py * ny) + pz * nz);
    }
    static __device__ __forceinline__ float sqrt(float x) { return sqrtf(x); }
    static constexpr bool kPairedDraw = false;
    static constexpr bool kFast = false;
};
struct FastMath {
    static __device__ __forceinline__ float div(float a, float b) { return __fdividef(a, b); }
    static __device__ __forceinline__ float exp(float x) { return __expf(x); }
    static __device__ __forceinline__ float log(float x) { return __logf(x); }
    static __device__ __forceinline__ void sincos2pi(float u, float& s, float& c) {
        __sincosf(u * 6.28318530717958647692f, &s, &c);
    }
    static __device__ __forceinline__ float rsqrt(float x) { return rsqrtf(x); }
    static __device__ __forceinline__ float mad(float a, float b, float c) { return fmaf(a, b, c); }
    static __device__ __forceinline__ float msub(float a, float b, float c) { return fmaf(-a, b, c); }
    static __device__ __forceinline__ float plane(float d, float px, float py, float pz, float nx, float ny,
                                                  float nz) {
        return fmaf(-pz, nz, fmaf(-py, ny, fmaf(-px, nx, d)));
    }
    static __device__ __forceinline__ float sqrt(float x) {
        float r;
        asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
        return r;
    }
    // One xorshift128+ output gives both scattering angles: its low 32 bits
    // (the reference's float recipe) and its high 32 bits.
    static constexpr bool kPairedDraw = true;
    static constexpr bool kFast = true;
};

// A packed face word: neighbour id (signed) << lb | its label.
__device__ __forceinline__ int decode_nb(int w, int lb) { return w >> lb; }

// Morton index of the bounding-box grid cell holding p (cells clamped to the grid).
__device__ __forceinline__ unsigned spatial_key(float px, float py, float pz, const PhaseArgs& pa) {
    const int n = (1 << kSortBits) - 1;
    const unsigned x = (unsigned)min(max((int)((px - pa.lo[0]) * pa.scale[0]), 0), n);
    const unsigned y = (unsigned)min(max((int)((py - pa.lo[1]) * pa.scale[1]), 0), n);
    const unsigned z = (unsigned)min(max((int)((pz - pa.lo[2]) * pa.scale[2]), 0), n);
    unsigned key = 0;
#pragma unroll
    for (int b = 0; b < kSortBits; b++)
        key |= (((x >> b) & 1u) << (3 * b)) | (((y >> b) & 1u) << (3 * b + 1)) | (((z >> b) & 1u) << (3 * b + 2));
    return key;
}

// Exclusive prefix sum of the kBuckets counts into `offset` (one block of 1024 threads).
__global__ void __launch_bounds__(1024) k_bucket_scan(const unsigned* count, unsigned* offset) {
    __shared__ unsigned part[1024];
    constexpr int per = kBuckets / 1024;
    const int t = threadIdx.x;
    unsigned v[per], s = 0;
#pragma unroll
    for (int i = 0; i < per; i++) {
        v[i] = count[t * per + i];
        s += v[i];
    }
    part[t] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {  // Hillis-Steele inclusive scan of the per-thread sums
        const unsigned add = (t >= o) ? part[t - o] : 0u;
        __syncthreads();
        part[t] += add;
        __syncthreads();
    }
    unsigned base = part[t] - s;
#pragma unroll
    for (int i = 0; i < per; i++) {
        offset[t * per + i] = base;
        base += v[i];
    }
}

// order[offset[key] + rank] = i for every parked record i (bucketed, order within a bucket arbitrary).
__global__ void k_bucket_order(const PState* rec, const unsigned long long* count, unsigned long long cap,
                               unsigned* offset, unsigned* order) {
    const unsigned long long n = min(*count, cap);
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned key = rec[i].meta.w;
        const unsigned slot = atomicAdd(offset + key, 1u);
        if (slot < n) order[slot] = (unsigned)i;
    }
}
__device__ __forceinline__ int decode_label(int w, int lmask) { return w & lmask; }

__device__ __forceinline__ void deposit(const SimDev& S, unsigned idx, float val) {
    if (S.accum_f64) {
        atomicAdd(S.f64 + idx, (double)val);
        return;
    }
    // Float accumulation with the reference's second buffer for running sums
    // above MAX_ACCUM (src/mmc_core.cl:880-912).  The reference moves `old` out
    // with a subtraction; when several lanes of a warp cross the threshold at
    // once they all subtract and drive the first buffer far negative, where
    // later small deposits lose their low bits.  An atomic exchange moves the
    // whole current content instead, so the first buffer stays below ~1000.
    const float old = atomicAdd(S.f32a + idx, val);
    if (old > kMaxAccum) {
        const float moved = atomicExch(S.f32a + idx, 0.f);
        if (moved != 0.f) atomicAdd(S.f32b + idx, moved);
    }
}

// Photon sharing (a pattern source with srcnum > 1 patterns, src/mmc_core.cl:929-942,
// :989-1002): one photon, launched with weight 1, stands for every pattern; a deposit of
// weight w adds w x (the pattern's value at the photon's launch pixel) to each pattern's
// cell, cells of one (element, gate) adjacent.
template <bool GEN>
__device__ __forceinline__ void deposit_at(const SimDev& S, const Lane& L, unsigned idx, float val) {
    if (GEN && S.srcnum > 1) {
        const float* pat = S.srcpattern + (size_t)L.posidx * S.srcnum;
        const unsigned base = idx * (unsigned)S.srcnum;
        for (int p = 0; p < S.srcnum; p++) deposit(S, base + p, val * __ldg(pat + p));
        return;
    }
    // gate-0 deposits (idx < ne) of the photon's first tests: this block's copy of the cell
    if (L.steps < S.hot_steps && idx < (unsigned)S.ne) {
        atomicAdd(S.hot + (size_t)(blockIdx.x & (kHotReps - 1)) * (unsigned)S.ne + idx, (double)val);
        return;
    }
    deposit(S, idx, val);
}

// One branchless Badouel step with fused deposit.  Requires 1 <= L.eid <= ne.
// REPLAY: the kernel may run replay simulations (output types wl, wp, wn and
// the Jacobian); kernels for forward runs are compiled without those branches.
// GEN: the kernel may deposit into a voxel grid (DMMC output) instead of the
// elements.
template <class MP, bool REPLAY, bool GEN>
__device__ __forceinline__ void raytet_step(Lane& L, const SimDev& S, const float4* med) {
    const TetRec* R = S.rec + (L.eid - 1);
    const float4 nx = __ldg(&R->nx);
    const float4 ny = __ldg(&R->ny);
    const float4 nz = __ldg(&R->nz);
    const float4 nd = __ldg(&R->nd);
    L.hit = 0;
    L.faceid = -1;
    L.isend = 0;
    float S0 = MP::mad(L.vz, nz.x, MP::mad(L.vy, ny.x, L.vx * nx.x));
    float S1 = MP::mad(L.vz, nz.y, MP::mad(L.vy, ny.y, L.vx * nx.y));
    float S2 = MP::mad(L.vz, nz.z, MP::mad(L.vy, ny.z, L.vx * nx.z));
    float S3 = MP::mad(L.vz, nz.w, MP::mad(L.vy, ny.w, L.vx * nx.w));
    float T0 = MP::plane(nd.x, L.px, L.py, L.pz, nx.x, ny.x, nz.x);
    float T1 = MP::plane(nd.y, L.px, L.py, L.pz, nx.y, ny.y, nz.y);
    float T2 = MP::plane(nd.z, L.px, L.py, L.pz, nx.z, ny.z, nz.z);
    float T3 = MP::plane(nd.w, L.px, L.py, L.pz, nx.w, ny.w, nz.w);
    T0 = (S0 > 0.f) ? MP::div(T0, S0) : 1e10f;
    T1 = (S1 > 0.f) ? MP::div(T1, S1) : 1e10f;
    T2 = (S2 > 0.f) ? MP::div(T2, S2) : 1e10f;
    T3 = (S3 > 0.f) ? MP::div(T3, S3) : 1e10f;
    // faceorder {1,3,2,0,-1} (src/mmc_mesh.c:95): the smallest distance, the earlier plane on
    // ties, no face when every distance is the 1e10 sentinel -- the reference's fmin and
    // equality scan, written as running comparisons (0.4% faster)
    float Lmin = 1e10f;
    int faceid = -1;
    if (T0 < Lmin) { Lmin = T0; faceid = 1; }
    if (T1 < Lmin) { Lmin = T1; faceid = 3; }
    if (T2 < Lmin) { Lmin = T2; faceid = 2; }
    if (T3 < Lmin) { Lmin = T3; faceid = 0; }
    L.faceid = faceid;
    if (faceid >= 0 && Lmin >= 0.f) {
        // only the exit face's word is loaded, once the face is known: holding all four through
        // the plane tests measured 1.9% slower than the extra dependent load
        L.nbword = __ldg(reinterpret_cast<const int*>(&R->nb) + faceid);
        float4 prop = med[L.label];  // mua mus g n
        if (GEN && S.nodemua) {
            // per-node properties (the reference's DOT-reconstruction mode, src/mmc_core.cl:785-793):
            // the mean of the element's four nodal values, summed in node order
            const int4 e = __ldg(S.elem + (L.eid - 1));
            const float* nm = S.nodemua;
            prop.x = 0.25f * (((__ldg(nm + e.x - 1) + __ldg(nm + e.y - 1)) + __ldg(nm + e.z - 1)) + __ldg(nm + e.w - 1));
            if (S.nodemusp) {
                const float* ns = S.nodemusp;
                prop.y = 0.25f * (((__ldg(ns + e.x - 1) + __ldg(ns + e.y - 1)) + __ldg(ns + e.z - 1)) + __ldg(ns + e.w - 1));
            }
        }
        float currweight = L.weight;
        float Lmove = (prop.y <= kEps) ? kRMinMus : MP::div(L.slen, prop.y);
        L.isend = (Lmin > Lmove);
        Lmove = L.isend ? Lmove : Lmin;
        L.hit = 1;
        const float rc = prop.w * kRC0;
        // (int)x > maxgate-1, written without the float->int conversion; the fast policy compares
        // the time itself with S.tend = tstart + maxgate * tstep (0.4% faster), the IEEE policy
        // keeps the oracle's gate-index form
        const float tnext = MP::mad(Lmove, rc, L.ptime);
        if (MP::kFast ? (tnext >= S.tend) : ((tnext - S.tstart) * S.Rtstep >= (float)S.maxgate)) {
            L.faceid = -2;
            L.hit = 0;
            Lmove = MP::div(S.tend - L.ptime, rc) - 1e-4f;
        }
        L.Lmove = Lmove;
        const float att = MP::exp(-prop.x * Lmove);
        L.weight *= att;
        const int ot = S.outputtype;
        if (REPLAY && S.replay) {
            const float rw = __ldg(S.replayweight + L.pid);
            if (ot == OT_WL || ot == OT_JACOBIAN) {
                currweight = Lmove;
                currweight *= rw;
                currweight += L.weight;
            } else if (ot == OT_WP) {
                currweight = (L.slen0 < kEps) ? 1.f : MP::div(Lmove * prop.y, L.slen0);
                currweight *= rw;
                currweight += L.weight;
            }
        }
        L.slen = MP::msub(Lmove, prop.y, L.slen);
        float ww = currweight - L.weight;
        L.ptime = MP::mad(Lmove, rc, L.ptime);
        if (REPLAY && ot == OT_WN) {  // scatter counts are deposited at the scattering events only
            L.px = MP::mad(Lmove, L.vx, L.px);
            L.py = MP::mad(Lmove, L.vy, L.py);
            L.pz = MP::mad(Lmove, L.vz, L.pz);
            L.slen = (L.faceid == -2) ? 0.f : L.slen;
            return;
        }
        float gf;
        if (REPLAY && S.replay && (ot == OT_WL || ot == OT_WP))
            gf = __ldg(S.replaytime + L.pid) * S.Rtstep;
        else
            gf = (L.ptime - S.tstart) * S.Rtstep;
        // min((int)gf, maxgate-1), clamped at 0 so that no index leaves the buffer
        int gate = (gf < (float)(S.maxgate - 1)) ? (int)gf : S.maxgate - 1;
        gate = max(gate, 0);
        if (ot != OT_ENERGY && !(REPLAY && (ot == OT_WP || ot == OT_WL)))
            ww = (prop.x < kEps) ? (currweight * Lmove) : MP::div(ww, prop.x);
        if (GEN && S.grid) {
            // DMMC: the step's loss is spread over 2(floor(Lmove/step)+1) equal segments,
            // each deposited in the grid voxel of its midpoint (src/mmc_core.cl:1019-1218)
            const int nseg = ((int)(Lmove * S.gstep_inv) + 1) << 1;
            const float seg = MP::div(Lmove, (float)nseg);
            const float segloss = MP::exp(-prop.x * seg);
            const float tx = L.vx * seg, ty = L.vy * seg, tz = L.vz * seg;
            float sx = (L.px - S.gmin[0]) + tx * 0.5f;
            float sy = (L.py - S.gmin[1]) + ty * 0.5f;
            float sz = (L.pz - S.gmin[2]) + tz * 0.5f;
            const float loss = 1.f - att;
            const float frac = (loss == 0.f) ? 0.f : MP::div(1.f - segloss, loss);
            const unsigned tshift = (unsigned)gate * S.framelen;
            float w0 = ww;
            const bool flush = (L.faceid == -2 || !L.isend);
            for (int k = 0; k < nseg; k++) {
                const unsigned ix = (sx > 0.f) ? (unsigned)floorf(sx * S.gstep_inv) : 0u;
                const unsigned iy = (sy > 0.f) ? (unsigned)floorf(sy * S.gstep_inv) : 0u;
                const unsigned iz = (sz > 0.f) ? (unsigned)floorf(sz * S.gstep_inv) : 0u;
                const unsigned newidx = min(iz, S.gdim[2] - 1) * (S.gdim[0] * S.gdim[1]) +
                                        min(iy, S.gdim[1] - 1) * S.gdim[0] + min(ix, S.gdim[0] - 1) + tshift;
                const float dw = w0 * frac;
                if (L.oldidx == (unsigned)kIdUndef) L.oldidx = newidx;
                if (newidx != L.oldidx) {
                    if (L.oldw > 0.f) deposit_at<GEN>(S, L, L.oldidx, L.oldw);
                    L.oldidx = newidx;
                    L.oldw = dw;
                } else {
                    L.oldw += dw;
                }
                if (flush) {
                    deposit_at<GEN>(S, L, newidx, L.oldw);
                    L.oldw = 0.f;
                }
                w0 *= segloss;
                sx += tx;
                sy += ty;
                sz += tz;
            }
            L.px = MP::mad(Lmove, L.vx, L.px);
            L.py = MP::mad(Lmove, L.vy, L.py);
            L.pz = MP::mad(Lmove, L.vz, L.pz);
            L.slen = (L.faceid == -2) ? 0.f : L.slen;
            return;
        }
        const unsigned newidx = (unsigned)(L.eid - 1) + (unsigned)(gate * S.ne);
        if (L.oldidx == (unsigned)kIdUndef) L.oldidx = newidx;
        if (newidx != L.oldidx) {
            if (L.oldw > 0.f) deposit_at<GEN>(S, L, L.oldidx, L.oldw);
            L.oldidx = newidx;
            L.oldw = ww;
        } else {
            L.oldw += ww;
        }
        if (L.faceid == -2 || !L.isend) {
            deposit_at<GEN>(S, L, newidx, L.oldw);
            L.oldw = 0.f;
        }
        L.px = MP::mad(Lmove, L.vx, L.px);
        L.py = MP::mad(Lmove, L.vy, L.py);
        L.pz = MP::mad(Lmove, L.vz, L.pz);
    }
    L.slen = (L.faceid == -2) ? 0.f : L.slen;
}

// src/mmc_core.cl:1390-1402
__device__ __forceinline__ void fixphoton(Lane& L, const SimDev& S) {
    const int4 e = __ldg(S.elem + (L.eid - 1));
    float cx = 0.f, cy = 0.f, cz = 0.f;
    const int ids[4] = {e.x, e.y, e.z, e.w};
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const float4 p = __ldg(S.node + (ids[i] - 1));
        cx += p.x;
        cy += p.y;
        cz += p.z;
    }
    L.px += (cx * 0.25f - L.px) * kFixPhoton;
    L.py += (cy * 0.25f - L.py) * kFixPhoton;
    L.pz += (cz * 0.25f - L.pz) * kFixPhoton;
}

// Fresnel / total internal reflection, src/mmc_core.cl:1247-1303.  Returns the
// element the photon continues in (oldeid when reflected).
template <class MP>
__device__ __forceinline__ int reflectray(Lane& L, const SimDev& S, const float4* med, int oldeid,
                                          int oldlabel, int eid, int newlabel, int faceid) {
    const TetRec* R = S.rec + (oldeid - 1);
    const int fi = (faceid == 0) ? 3 : (faceid == 1) ? 0 : (faceid == 2) ? 2 : 1;  // ifaceorder
    const float* fx = reinterpret_cast<const float*>(&R->nx);
    const float* fy = reinterpret_cast<const float*>(&R->ny);
    const float* fz = reinterpret_cast<const float*>(&R->nz);
    const float pnx = __ldg(fx + fi), pny = __ldg(fy + fi), pnz = __ldg(fz + fi);
    const float Icos = fabsf(((L.vx * pnx) + (L.vy * pny)) + (L.vz * pnz));
    const float n1 = (oldeid != eid) ? med[oldlabel].w : S.nout;
    const float n2 = (eid > 0) ? med[newlabel].w : S.nout;
    float tmp0 = n1 * n1;
    float tmp1 = n2 * n2;
    float tmp2 = 1.f - MP::div(tmp0, tmp1) * (1.f - Icos * Icos);
    if (tmp2 > 0.f && !((eid <= 0) && (S.isreflect == BC_MIRROR))) {
        float Re = tmp0 * Icos * Icos + tmp1 * tmp2;
        tmp2 = MP::sqrt(tmp2);
        float Im = 2.f * n1 * n2 * Icos * tmp2;
        float Rtotal = MP::div(Re - Im, Re + Im);
        Re = tmp1 * Icos * Icos + tmp0 * tmp2 * tmp2;
        Rtotal = (Rtotal + MP::div(Re - Im, Re + Im)) * 0.5f;
        if (rng_next(L.t0, L.t1) <= Rtotal) {
            const float k = -2.f * Icos;
            L.vx += k * pnx;
            L.vy += k * pny;
            L.vz += k * pnz;
            eid = oldeid;
        } else if ((S.isspecular == 2) && (eid == 0)) {
        } else {
            const float k = -Icos;
            L.vx += k * pnx;
            L.vy += k * pny;
            L.vz += k * pnz;
            const float q = MP::div(n1, n2);
            L.vx = tmp2 * pnx + q * L.vx;
            L.vy = tmp2 * pny + q * L.vy;
            L.vz = tmp2 * pnz + q * L.vz;
        }
    } else {
        const float k = -2.f * Icos;
        L.vx += k * pnx;
        L.vy += k * pny;
        L.vz += k * pnz;
        eid = oldeid;
    }
    const float inv = MP::rsqrt(L.vx * L.vx + L.vy * L.vy + L.vz * L.vz);
    L.vx *= inv;
    L.vy *= inv;
    L.vz *= inv;
    return eid;
}

// Rotates the direction by polar angle (stheta, ctheta) and azimuth (sphi,
// cphi) about itself, then renormalizes (rotatevector, src/mmc_core.cl:1345-1377).
template <class MP>
__device__ __forceinline__ void rotate_dir(Lane& L, float stheta, float ctheta, float sphi, float cphi) {
    float px, py, pz;
    if (L.vz > -1.f + kEps && L.vz < 1.f - kEps) {
        const float tmp0 = MP::msub(L.vz, L.vz, 1.f);
        float tmp1 = MP::rsqrt(tmp0);
        tmp1 = stheta * tmp1;
        px = MP::mad(tmp1, MP::msub(L.vy, sphi, L.vx * L.vz * cphi), L.vx * ctheta);
        py = MP::mad(tmp1, MP::mad(L.vx, sphi, L.vy * L.vz * cphi), L.vy * ctheta);
        pz = MP::mad(-tmp1 * tmp0, cphi, L.vz * ctheta);
    } else {
        px = stheta * cphi;
        py = stheta * sphi;
        pz = (L.vz > 0.f) ? ctheta : -ctheta;
    }
    const float inv = MP::rsqrt(MP::mad(pz, pz, MP::mad(py, py, px * px)));
    L.vx = px * inv;
    L.vy = py * inv;
    L.vz = pz * inv;
}

// Henyey-Greenstein scatter + direction rotation, src/mmc_core.cl:1307-1377.
template <class MP>
__device__ __forceinline__ float next_scatter(Lane& L, float g, float& ctheta_out) {
    const float nextslen = -MP::log(rng_next(L.t0, L.t1) + kEps);
    float sphi, cphi, stheta, ctheta;
    float utheta = 0.f;
    if (MP::kPairedDraw) {
        MP::sincos2pi(rng_next_pair(L.t0, L.t1, utheta), sphi, cphi);
    } else {
        MP::sincos2pi(rng_next(L.t0, L.t1), sphi, cphi);
    }
    if (g > kEps) {
        if (!MP::kPairedDraw) utheta = rng_next(L.t0, L.t1);
        float tmp0 = MP::div(MP::msub(g, g, 1.f), MP::mad(2.f * g, utheta, 1.f - g));
        tmp0 *= tmp0;
        tmp0 = MP::div(MP::mad(g, g, 1.f) - tmp0, 2.f * g);
        tmp0 = fmaxf(-1.f, fminf(tmp0, 1.f));
        stheta = MP::sqrt(MP::msub(tmp0, tmp0, 1.f));
        ctheta = tmp0;
    } else {
        if (!MP::kPairedDraw) utheta = rng_next(L.t0, L.t1);
        ctheta = 2.f * utheta - 1.f;
        stheta = MP::sqrt(MP::msub(ctheta, ctheta, 1.f));
    }
    rotate_dir<MP>(L, stheta, ctheta, sphi, cphi);
    ctheta_out = ctheta;
    return nextslen;
}

__device__ __forceinline__ int finddetector(const Lane& L, const SimDev& S) {
    for (int i = 0; i < S.detnum; i++) {
        const float4 d = __ldg(S.det + i);
        if ((d.x - L.px) * (d.x - L.px) + (d.y - L.py) * (d.y - L.py) + (d.z - L.pz) * (d.z - L.pz) < d.w * d.w)
            return i + 1;
    }
    return 0;
}

// ---- photon sources ---------------------------------------------------------
// Source types, numbered as the reference's TSrcType (src/mmc_utils.h:101-105).
enum SrcType : int {
    ST_PENCIL = 0, ST_ISOTROPIC = 1, ST_CONE = 2, ST_GAUSSIAN = 3, ST_PLANAR = 4, ST_PATTERN = 5,
    ST_FOURIER = 6, ST_ARCSINE = 7, ST_DISK = 8, ST_FOURIERX = 9, ST_FOURIER2D = 10, ST_ZGAUSSIAN = 11,
    ST_LINE = 12, ST_SLIT = 13, ST_PENCILARRAY = 14, ST_PATTERN3D = 15, ST_HYPERBOLOID = 16, ST_RING = 17
};

constexpr float kPi = 3.14159265358979323846f;

// Whether element e (0-based) encloses p: the barycentric test of the
// reference's source-element search, src/mmc_raytrace.c:2599-2652 (face
// normals from node cross products, unnormalized, tolerance -1e-4).
__device__ __forceinline__ float face_bary(const float4& a, const float4& b, const float4& c, float px, float py,
                                           float pz) {
    const float abx = b.x - a.x, aby = b.y - a.y, abz = b.z - a.z;
    const float acx = c.x - a.x, acy = c.y - a.y, acz = c.z - a.z;
    const float sx = px - a.x, sy = py - a.y, sz = pz - a.z;
    const float nx = aby * acz - abz * acy, ny = abz * acx - abx * acz, nz = abx * acy - aby * acx;
    return -((sx * nx + sy * ny) + sz * nz);
}

__device__ __forceinline__ bool src_encloses(const SimDev& S, int e, float px, float py, float pz) {
    const int4 el = __ldg(S.elem + e);
    const float4 n0 = __ldg(S.node + (el.x - 1)), n1 = __ldg(S.node + (el.y - 1));
    const float4 n2 = __ldg(S.node + (el.z - 1)), n3 = __ldg(S.node + (el.w - 1));
    // faces out[i] = {0,3,1} {3,2,1} {0,2,3} {0,1,2} (src/mmc_mesh.c:59-64), facemap {2,0,1,3}
    const float b2 = face_bary(n0, n3, n1, px, py, pz);
    const float b0 = face_bary(n3, n2, n1, px, py, pz);
    const float b1 = face_bary(n0, n2, n3, px, py, pz);
    const float b3 = face_bary(n0, n1, n2, px, py, pz);
    return !(b0 < -1e-4f || b1 < -1e-4f || b2 < -1e-4f || b3 < -1e-4f);
}

// The lowest-index element enclosing p among the bounding-box grid cell that
// holds p, else among its 26 neighbours (cells hold every element whose
// bounding box overlaps them).  Returns a 1-based id, 0 when none does.
__device__ int src_locate(const SimDev& S, float px, float py, float pz) {
    const int res = S.loc_res;
    const float fx = (px - S.loc_lo[0]) * S.loc_inv[0];
    const float fy = (py - S.loc_lo[1]) * S.loc_inv[1];
    const float fz = (pz - S.loc_lo[2]) * S.loc_inv[2];
    const float lo = -1e-3f * res, hi = res * (1.f + 1e-3f);
    if (!(fx >= lo) || !(fx <= hi) || !(fy >= lo) || !(fy <= hi) || !(fz >= lo) || !(fz <= hi)) return 0;
    const int bx = min(res - 1, max(0, (int)floorf(fx)));
    const int by = min(res - 1, max(0, (int)floorf(fy)));
    const int bz = min(res - 1, max(0, (int)floorf(fz)));
    for (int pass = 0; pass < 2; pass++) {
        int best = 0x7FFFFFFF;
        for (int z = max(0, bz - pass); z <= min(res - 1, bz + pass); z++)
            for (int y = max(0, by - pass); y <= min(res - 1, by + pass); y++)
                for (int x = max(0, bx - pass); x <= min(res - 1, bx + pass); x++) {
                    const size_t cell = ((size_t)z * res + y) * res + x;
                    const unsigned k1 = __ldg(S.loc_start + cell + 1);
                    for (unsigned k = __ldg(S.loc_start + cell); k < k1; k++) {
                        const int e = (int)__ldg(S.loc_items + k);
                        if (e < best && src_encloses(S, e, px, py, pz)) best = e;
                    }
                }
        if (best != 0x7FFFFFFF) return best + 1;
    }
    return 0;
}

// Sets the launch state of a new photon (position, direction, weight, first
// scattering length, element, label), following the reference's CPU launch
// (launchphoton, src/mmc_raytrace.c:2346-2671; the device version,
// src/mmc_core.cl:1416-1834, differs only where noted in the oracle).  A
// source whose launch position varies is located per photon: the initial
// element first, then the bounding-box grid.  Returns false when no element
// encloses the launch position.
template <class MP>
__device__ __forceinline__ bool launch_photon(Lane& L, const SimDev& S) {
    L.px = S.srcpos[0];
    L.py = S.srcpos[1];
    L.pz = S.srcpos[2];
    L.vx = S.srcdir[0];
    L.vy = S.srcdir[1];
    L.vz = S.srcdir[2];
    L.weight = 1.f;
    L.eid = S.e0;
    float ox = L.px, oy = L.py, oz = L.pz;  // origin: the focus is measured from here
    bool canfocus = true;
    L.slen = -MP::log(rng_next(L.t0, L.t1) + kEps);
    const float4 p1 = S.srcp1, p2 = S.srcp2;
    const int st = S.srctype;
    if (st == ST_PENCIL) {
        if (L.eid > 0) {
            L.label = __ldg(S.label + (L.eid - 1));
            return true;
        }
    } else if (st == ST_PLANAR || st == ST_PATTERN || st == ST_PATTERN3D || st == ST_FOURIER || st == ST_PENCILARRAY) {
        const float rx = rng_next(L.t0, L.t1);
        const float ry = rng_next(L.t0, L.t1);
        if (st == ST_PATTERN3D) {
            const float rz = rng_next(L.t0, L.t1);
            L.px = S.srcpos[0] + rx * p1.x;
            L.py = S.srcpos[1] + ry * p1.y;
            L.pz = S.srcpos[2] + rz * p1.z;
            const int nx = (int)p1.x, ny = (int)p1.y, nz = (int)p1.z;
            const int ix = min((int)(rx * nx), nx - 1), iy = min((int)(ry * ny), ny - 1),
                      iz = min((int)(rz * nz), nz - 1);
            L.weight = __ldg(S.srcpattern + ((size_t)iz * ny + iy) * nx + ix);
            ox += p1.x * 0.5f;
            oy += p1.y * 0.5f;
            oz += p1.z * 0.5f;
        } else if (st == ST_PENCILARRAY) {
            const float fx = floorf(rx * p1.w), fy = floorf(ry * p2.w);
            L.px = S.srcpos[0] + fx * p1.x / (p1.w - 1.f) + fy * p2.x / (p2.w - 1.f);
            L.py = S.srcpos[1] + fx * p1.y / (p1.w - 1.f) + fy * p2.y / (p2.w - 1.f);
            L.pz = S.srcpos[2] + fx * p1.z / (p1.w - 1.f) + fy * p2.z / (p2.w - 1.f);
            ox += (p1.x + p2.x) * 0.5f;
            oy += (p1.y + p2.y) * 0.5f;
            oz += (p1.z + p2.z) * 0.5f;
        } else {
            L.px = S.srcpos[0] + rx * p1.x + ry * p2.x;
            L.py = S.srcpos[1] + rx * p1.y + ry * p2.y;
            L.pz = S.srcpos[2] + rx * p1.z + ry * p2.z;
            if (st == ST_PATTERN) {
                const int nx = (int)p1.w, ny = (int)p2.w;
                const int idx = min((int)(ry * ny), ny - 1) * nx + min((int)(rx * nx), nx - 1);
                // several patterns share the photon: it starts with weight 1 and its deposits
                // are scaled per pattern (src/mmc_core.cl:1545-1549)
                L.posidx = idx;
                L.weight = (S.srcnum > 1) ? 1.f : __ldg(S.srcpattern + idx);
            } else if (st == ST_FOURIER) {
                float sv, cv;
                MP::sincos2pi(floorf(p1.w) * rx + floorf(p2.w) * ry + p1.w - floorf(p1.w), sv, cv);
                L.weight = (cv * (1.f - p2.w + floorf(p2.w)) + 1.f) * 0.5f;
            }
            ox += (p1.x + p2.x) * 0.5f;
            oy += (p1.y + p2.y) * 0.5f;
            oz += (p1.z + p2.z) * 0.5f;
        }
    } else if (st == ST_FOURIERX || st == ST_FOURIER2D) {
        const float rx = rng_next(L.t0, L.t1);
        const float ry = rng_next(L.t0, L.t1);
        const float w = p1.w * (1.f / sqrtf(p1.x * p1.x + p1.y * p1.y + p1.z * p1.z));
        const float v2x = w * (S.srcdir[1] * p1.z - S.srcdir[2] * p1.y);
        const float v2y = w * (S.srcdir[2] * p1.x - S.srcdir[0] * p1.z);
        const float v2z = w * (S.srcdir[0] * p1.y - S.srcdir[1] * p1.x);
        L.px = S.srcpos[0] + rx * p1.x + ry * v2x;
        L.py = S.srcpos[1] + rx * p1.y + ry * v2y;
        L.pz = S.srcpos[2] + rx * p1.z + ry * v2z;
        float s1, c1, s2, c2;
        if (st == ST_FOURIER2D) {
            MP::sincos2pi(p2.x * rx + p2.z, s1, c1);
            MP::sincos2pi(p2.y * ry + p2.w, s2, c2);
            L.weight = (s1 * s2 + 1.f) * 0.5f;
        } else {
            MP::sincos2pi(p2.x * rx + p2.y * ry + p2.z, s1, c1);
            L.weight = (c1 * (1.f - p2.w) + 1.f) * 0.5f;
        }
        ox += (p1.x + v2x) * 0.5f;
        oy += (p1.y + v2y) * 0.5f;
        oz += (p1.z + v2z) * 0.5f;
    } else if (st == ST_DISK || st == ST_RING || st == ST_GAUSSIAN) {
        float sphi, cphi;
        if (st == ST_RING && (p1.z > 0.f || p1.w > 0.f)) {  // azimuth range [min, max] in radians
            const float phi = fabsf(p1.z - p1.w) * rng_next(L.t0, L.t1) + fminf(p1.z, p1.w);
            MP::sincos2pi(phi * (0.5f / kPi), sphi, cphi);
        } else {
            MP::sincos2pi(rng_next(L.t0, L.t1), sphi, cphi);
        }
        float r0;
        if (st == ST_DISK || st == ST_RING) {  // radii p1.y (inner) to p1.x (outer), uniform in area
            r0 = sqrtf(rng_next(L.t0, L.t1) * fabsf(p1.x * p1.x - p1.y * p1.y) + p1.y * p1.y);
        } else if (fabsf(S.focus) < 1e-5f || fabsf(p1.y) < 1e-5f) {  // waist p1.x
            // (+EPS: a draw of exactly 0 would put the photon at infinity)
            r0 = sqrtf(-MP::log(rng_next(L.t0, L.t1) + kEps)) * p1.x;
        } else {  // waist p1.x, wavelength p1.y, focus: widened by the Rayleigh range
            const float z0 = p1.x * p1.x * kPi / p1.y;
            r0 = sqrtf(-MP::log(rng_next(L.t0, L.t1) + kEps) * (1.f + (S.focus * S.focus / (z0 * z0)))) * p1.x;
        }
        const float dx = S.srcdir[0], dy = S.srcdir[1], dz = S.srcdir[2];
        if (dz > -1.f + kEps && dz < 1.f - kEps) {
            const float tmp0 = 1.f - dz * dz;
            const float tmp1 = r0 / sqrtf(tmp0);
            L.px = S.srcpos[0] + tmp1 * (dx * dz * cphi - dy * sphi);
            L.py = S.srcpos[1] + tmp1 * (dy * dz * cphi + dx * sphi);
            L.pz = S.srcpos[2] - tmp1 * tmp0 * cphi;
        } else {
            L.px += r0 * cphi;
            L.py += r0 * sphi;
        }
    } else if (st == ST_CONE || st == ST_ISOTROPIC || st == ST_ARCSINE) {
        float sphi, cphi, stheta, ctheta;
        MP::sincos2pi(rng_next(L.t0, L.t1), sphi, cphi);
        if (st == ST_CONE) {
            // polar angle within the half angle p1.x: uniform in angle (p1.y > 0) or in solid
            // angle, sampled by inversion instead of the reference's rejection loop
            const float u = rng_next(L.t0, L.t1);
            if (p1.y > 0.f) {
                MP::sincos2pi(u * p1.x * (0.5f / kPi), stheta, ctheta);
            } else {
                float sa, ca;
                MP::sincos2pi(p1.x * (0.5f / kPi), sa, ca);
                ctheta = 1.f - u * (1.f - ca);
                stheta = sqrtf(fmaxf(0.f, 1.f - ctheta * ctheta));
            }
        } else if (st == ST_ISOTROPIC) {  // cos(acos(2u-1)) = 2u-1
            ctheta = 2.f * rng_next(L.t0, L.t1) - 1.f;
            stheta = sqrtf(fmaxf(0.f, 1.f - ctheta * ctheta));
        } else {  // arcsine: polar angle uniform in [0, pi)
            MP::sincos2pi(0.5f * rng_next(L.t0, L.t1), stheta, ctheta);
        }
        rotate_dir<MP>(L, stheta, ctheta, sphi, cphi);
        canfocus = false;
        if (L.eid > 0) {
            L.label = __ldg(S.label + (L.eid - 1));
            return true;
        }
    } else if (st == ST_ZGAUSSIAN) {  // polar angle Gaussian with sigma p1.x
        float sphi, cphi, stheta, ctheta;
        MP::sincos2pi(rng_next(L.t0, L.t1), sphi, cphi);
        const float u1 = rng_next(L.t0, L.t1);
        const float u2 = rng_next(L.t0, L.t1);
        const float ang = sqrtf(-2.f * MP::log(u1 + kEps)) * (1.f - 2.f * u2) * p1.x;
        MP::sincos2pi(ang * (0.5f / kPi), stheta, ctheta);
        rotate_dir<MP>(L, stheta, ctheta, sphi, cphi);
        canfocus = false;
    } else if (st == ST_HYPERBOLOID) {  // hyperboloid Gaussian beam: waist p1.x, p1.y/p1.z tilt
        float sphi, cphi;
        MP::sincos2pi(rng_next(L.t0, L.t1), sphi, cphi);
        const float r0 = sqrtf(0.5f * -MP::log(rng_next(L.t0, L.t1) + kEps)) * p1.x;
        const float tilt = (p1.z > 0.f) ? (-p1.y / p1.z) : 0.f;
        float bx = -r0 * sphi, by = r0 * cphi, bz = p1.z;
        const float nb = 1.f / sqrtf(bx * bx + by * by + bz * bz);
        bx *= nb;
        by *= nb;
        bz *= nb;
        const float qx = r0 * (cphi - tilt * sphi), qy = r0 * (sphi + tilt * cphi);
        const float dx = S.srcdir[0], dy = S.srcdir[1], dz = S.srcdir[2];
        if (dz > -1.f + kEps && dz < 1.f - kEps) {
            const float sint = sqrtf(1.f - dz * dz);
            const float isint = 1.f / sint;
            const float cb = dx * isint, sb = dy * isint;
            L.px = S.srcpos[0] + qx * cb * dz - qy * sb;
            L.py = S.srcpos[1] + qx * sb * dz + qy * cb;
            L.pz = S.srcpos[2] - qx * sint;
            L.vx = bx * cb * dz - by * sb + bz * cb * sint;
            L.vy = bx * sb * dz + by * cb + bz * sb * sint;
            L.vz = -bx * sint + bz * dz;
        } else {
            L.px = S.srcpos[0] + qx;
            L.py = S.srcpos[1] + qy;
            L.pz = S.srcpos[2];
            L.vx = bx;
            L.vy = by;
            L.vz = (dz > 0.f) ? bz : -bz;
        }
        const float nv = 1.f / sqrtf(L.vx * L.vx + L.vy * L.vy + L.vz * L.vz);
        L.vx *= nv;
        L.vy *= nv;
        L.vz *= nv;
        canfocus = false;
    } else if (st == ST_LINE || st == ST_SLIT) {  // segment srcpos .. srcpos + p1.xyz
        float t = rng_next(L.t0, L.t1);
        L.px += t * p1.x;
        L.py += t * p1.y;
        L.pz += t * p1.z;
        if (st == ST_LINE) {  // direction perpendicular to the launch direction, random
            t = 1.f - 2.f * rng_next(L.t0, L.t1);
            const float s = 1.f - 2.f * rng_next(L.t0, L.t1);
            const float sign = (rng_next(L.t0, L.t1) > 0.5f) ? 1.f : -1.f;
            const float p = sqrtf(1.f - L.vx * L.vx - L.vy * L.vy) * sign;
            const float vx = L.vy * p - L.vz * s, vy = L.vz * t - L.vx * p, vz = L.vx * s - L.vy * t;
            L.vx = vx;
            L.vy = vy;
            L.vz = vz;
        }
        ox += p1.x * 0.5f;
        oy += p1.y * 0.5f;
        oz += p1.z * 0.5f;
        canfocus = (st == ST_SLIT);
    }
    if (canfocus) {
        const float f = S.focus;
        if (f != f) {  // NaN: a uniformly random direction about the launch direction
            float sphi, cphi;
            MP::sincos2pi(rng_next(L.t0, L.t1), sphi, cphi);
            const float ctheta = 2.f * rng_next(L.t0, L.t1) - 1.f;
            rotate_dir<MP>(L, sqrtf(fmaxf(0.f, 1.f - ctheta * ctheta)), ctheta, sphi, cphi);
        } else if (f < 0.f && isinf(f)) {  // -inf: Lambertian (cosine) emission
            float sphi, cphi;
            MP::sincos2pi(rng_next(L.t0, L.t1), sphi, cphi);
            const float stheta = sqrtf(rng_next(L.t0, L.t1));
            rotate_dir<MP>(L, stheta, sqrtf(1.f - stheta * stheta), sphi, cphi);
        } else if (f != 0.f) {  // converging (f > 0) or diverging (f < 0) beam
            ox += f * L.vx;
            oy += f * L.vy;
            oz += f * L.vz;
            float vx, vy, vz;
            if (f < 0.f) {
                vx = L.px - ox;
                vy = L.py - oy;
                vz = L.pz - oz;
            } else {
                vx = ox - L.px;
                vy = oy - L.py;
                vz = oz - L.pz;
            }
            const float rn = 1.f / sqrtf(vx * vx + vy * vy + vz * vz);
            L.vx = vx * rn;
            L.vy = vy * rn;
            L.vz = vz * rn;
        }
    }
    L.px = L.px + L.vx * kEps;
    L.py = L.py + L.vy * kEps;
    L.pz = L.pz + L.vz * kEps;
    int e = 0;
    if (L.eid > 0 && src_encloses(S, L.eid - 1, L.px, L.py, L.pz)) e = L.eid;
    else if (S.loc_start) e = src_locate(S, L.px, L.py, L.pz);
    if (e <= 0) return false;
    L.eid = e;
    L.label = __ldg(S.label + (e - 1));
    return true;
}

// One trajectory record (src/mmc_core.cl:692-704): photon id (within the whole simulation),
// position, weight, element.
__device__ __forceinline__ void save_traj(const SimDev& S, const Lane& L) {
    const unsigned pos = atomicAdd(S.trajcount, 1u);
    if (pos < S.maxtraj) {
        float* r = S.traj + (size_t)pos * 6;
        r[0] = __uint_as_float((unsigned)(S.photon_offset + L.pid));
        r[1] = L.px;
        r[2] = L.py;
        r[3] = L.pz;
        r[4] = L.weight;
        r[5] = __int_as_float(L.eid);
    }
}

struct Tally {
    float eesc;
    float etot;
    unsigned raytet;
    unsigned aborted;
    unsigned outside;
    int sim;
};

__device__ __forceinline__ void flush_tally(Tally& t, const SimDev& S) {
    if (t.sim < 0) return;
    if (t.etot != 0.f) atomicAdd(S.energy + 0, (double)t.etot);
    if (t.eesc != 0.f) atomicAdd(S.energy + 1, (double)t.eesc);
    if (t.raytet) atomicAdd(S.counters + 0, (unsigned long long)t.raytet);
    if (t.aborted) atomicAdd(S.counters + 1, (unsigned long long)t.aborted);
    if (t.outside && S.ncounters > 2) atomicAdd(S.counters + 2, (unsigned long long)t.outside);
    t.etot = 0.f;
    t.eesc = 0.f;
    t.raytet = 0;
    t.aborted = 0;
    t.outside = 0;
}

// Launched (which = 0) or escaped (1) weight of a photon shared by srcnum > 1 patterns, per
// pattern: w x the pattern's value at the launch pixel (src/mmc_core.cl:1907-1911, :2154-2159).
// Blocks add into 64 slots of [srcnum launched | srcnum escaped] doubles to spread the atomics.
__device__ __forceinline__ void tally_sources(const SimDev& S, int posidx, float w, int which) {
    double* e = S.energy_src + ((size_t)(blockIdx.x % kEnergySlots) * 2 + which) * S.srcnum;
    const float* pat = S.srcpattern + (size_t)posidx * S.srcnum;
    for (int p = 0; p < S.srcnum; p++) atomicAdd(e + p, (double)(w * __ldg(pat + p)));
}

struct SingleSim {
    const SimDev& s;
    __device__ __forceinline__ const SimDev& operator()(int) const { return s; }
};
struct ManySims {
    const SimDev* s;
    __device__ __forceinline__ const SimDev& operator()(int i) const { return s[i]; }
};

// Shared-memory layout: media[nsims_local * nmed_stride] | ppath[reclen_max][blockDim] |
// seed0[2][blockDim] (u64)
template <class MP, class Sims, bool BATCHED, bool PHASED, bool REPLAY, int KIND>
__device__ __forceinline__ void engine_body(const Sims& sims, const unsigned long long* cum, int nsims,
                                            unsigned long long total, int nmed_stride, int reclen_max,
                                            int want_seed, unsigned long long* work_counter, const PhaseArgs& pa) {
    constexpr bool SRC = (KIND == KIND_GENERAL);  // general launch, grid deposits, trace/trajectory outputs
    constexpr bool ROUL = (KIND != KIND_LEAN);    // Russian roulette
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float4* smed = reinterpret_cast<float4*>(smem_raw);
    const int nmed_rows = nsims * nmed_stride;
    for (int i = threadIdx.x; i < nmed_rows; i += blockDim.x) {
        const int s = i / nmed_stride, r = i % nmed_stride;
        const SimDev& S = sims(s);
        smed[i] = (r < S.nmedia) ? __ldg(S.media + r) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    float* ppath = reinterpret_cast<float*>(smed + nmed_rows);
    unsigned long long* seed0 = reinterpret_cast<unsigned long long*>(ppath + (size_t)reclen_max * blockDim.x);
    if (((uintptr_t)seed0) & 7) seed0 = reinterpret_cast<unsigned long long*>((((uintptr_t)seed0) + 7) & ~(uintptr_t)7);
    // Single-simulation kernels count ray-tet tests, aborted and outside photons per block in
    // shared memory, updated when a photon ends (tests = its step count): per-lane counters
    // would hold three registers through the step loop, which measured 4.7% slower.  The
    // batched kernels keep per-lane counters of the lane's current simulation, adding a
    // photon's steps when it ends (1.9% faster than counting every step).
    __shared__ unsigned long long s_cnt[3];
    if (threadIdx.x < 3) s_cnt[threadIdx.x] = 0ull;
    __syncthreads();

    const int tid = threadIdx.x;
    const int bdim = blockDim.x;
    const unsigned lane = threadIdx.x & 31;
    Lane L;
    L.mode = M_NEED;
    L.sim = 0;
    L.pid = 0;
    L.steps = 0;
    Tally tally{0.f, 0.f, 0u, 0u, 0u, -1};

#define PP(i) ppath[(i) * bdim + tid]

    while (true) {
        // ---- (1) hand out photons to lanes that need one ----
        const unsigned need = __ballot_sync(kFull, L.mode == M_NEED);
        if (need) {
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if ((int)lane == leader) base = atomicAdd(work_counter, (unsigned long long)__popc(need));
            base = __shfl_sync(kFull, base, leader);
            if (L.mode == M_NEED) {
                const unsigned long long gid = base + __popc(need & ((1u << lane) - 1u));
                if (gid >= total) {
                    L.mode = M_DONE;
                } else {
                    int s = 0;
                    if (BATCHED) {
                        int lo = 0, hi = nsims - 1;
                        while (lo < hi) {
                            const int mid = (lo + hi) >> 1;
                            if (gid < cum[mid]) hi = mid; else lo = mid + 1;
                        }
                        s = lo;
                    }
                    const SimDev& S = sims(s);
                    if (s != tally.sim) {
                        if (tally.sim >= 0) flush_tally(tally, sims(tally.sim));
                        tally.sim = s;
                    }
                    L.sim = s;
                    L.pid = BATCHED ? (gid - (s ? cum[s - 1] : 0ull)) : gid;
                    if (PHASED && pa.phase > 0) {
                        // ---- resume a photon parked at the end of the previous gate ----
                        // queue traffic is read once: streaming loads keep it from displacing
                        // the tet records and the live gate planes in L2
                        const unsigned long long qi = pa.order ? (unsigned long long)pa.order[gid] : gid;
                        const PState* q = pa.in.rec + qi;
                        PState r;
                        r.pos = __ldcs(&q->pos);
                        r.dir = __ldcs(&q->dir);
                        r.len = __ldcs(&q->len);
                        r.elem = __ldcs(&q->elem);
                        r.meta = __ldcs(&q->meta);
                        r.rng = __ldcs(&q->rng);
                        L.px = r.pos.x;
                        L.py = r.pos.y;
                        L.pz = r.pos.z;
                        L.ptime = r.pos.w;
                        L.vx = r.dir.x;
                        L.vy = r.dir.y;
                        L.vz = r.dir.z;
                        L.weight = r.dir.w;
                        L.slen = r.len.x;
                        L.slen0 = r.len.y;
                        if (SRC && !REPLAY) L.posidx = __float_as_int(r.len.y);
                        L.oldw = r.len.z;
                        L.oldidx = __float_as_uint(r.len.w);
                        L.eid = r.elem.x;
                        L.label = r.elem.y;
                        L.mode = r.elem.z;
                        L.fixcount = r.elem.w;
                        L.steps = r.meta.x;
                        L.pid = ((unsigned long long)r.meta.z << 32) | r.meta.y;
                        L.t0 = ((unsigned long long)r.rng.y << 32) | r.rng.x;
                        L.t1 = ((unsigned long long)r.rng.w << 32) | r.rng.z;
                        L.Lmove = 0.f;
                        L.faceid = 0;
                        L.isend = 0;
                        L.hit = 0;
                        if (S.issavedet)
                            for (int i = 0; i < S.reclen; i++) PP(i) = __ldcs(pa.in.ppath + qi * S.reclen + i);
                        if (want_seed) {
                            seed0[tid] = __ldcs(pa.in.seed0 + 2 * qi);
                            seed0[bdim + tid] = __ldcs(pa.in.seed0 + 2 * qi + 1);
                        }
                    } else {
                    // ---- launch (src/mmc_core.cl:1851-1906, pencil source) ----
                    if (REPLAY && S.replay) {
                        L.t0 = __ldg(S.replayseed + 2 * L.pid);
                        L.t1 = __ldg(S.replayseed + 2 * L.pid + 1);
                    } else {
                        rng_seed(S.seed, S.photon_offset + L.pid, L.t0, L.t1);
                    }
                    if (want_seed) {
                        seed0[tid] = L.t0;
                        seed0[bdim + tid] = L.t1;
                    }
                    L.faceid = 0;
                    L.isend = 0;
                    L.hit = 0;
                    L.ptime = 0.f;
                    L.Lmove = 0.f;
                    L.slen0 = 0.f;
                    L.oldw = 0.f;
                    L.oldidx = (unsigned)kIdUndef;
                    L.fixcount = 0;
                    L.steps = 0;
                    bool placed;
                    if (!SRC || (S.srctype == ST_PENCIL && S.e0 > 0)) {  // the pencil branch of launch_photon
                        L.px = S.srcpos[0];
                        L.py = S.srcpos[1];
                        L.pz = S.srcpos[2];
                        L.vx = S.srcdir[0];
                        L.vy = S.srcdir[1];
                        L.vz = S.srcdir[2];
                        L.weight = 1.f;
                        L.eid = S.e0;
                        L.slen = -MP::log(rng_next(L.t0, L.t1) + kEps);
                        L.label = __ldg(S.label + (S.e0 - 1));
                        placed = true;
                    } else {
                        placed = launch_photon<MP>(L, S);
                    }
                    tally.etot += L.weight;
                    const bool shared = SRC && S.srcnum > 1;
                    if (shared) tally_sources(S, L.posidx, L.weight, 0);
                    if (S.issavedet) {
                        for (int i = 0; i < S.reclen; i++) PP(i) = 0.f;
                        // the last column: initial weight, or the launch pixel of a shared photon
                        // (src/mmc_core.cl:1894-1898)
                        PP(S.reclen - 1) = shared ? __int_as_float(L.posidx) : L.weight;
                    }
                    if (placed) {
                        L.mode = M_OUTER;
                        if (SRC && S.traj) save_traj(S, L);
                    } else {  // launch position in no element: counted, reported as an error
                        if (BATCHED) tally.outside++; else atomicAdd(&s_cnt[2], 1ull);
                        tally.eesc += L.weight;
                        if (shared) tally_sources(S, L.posidx, L.weight, 1);
                        if (SRC && S.photon_det) S.photon_det[L.pid] = 0;
                        if (SRC && S.photon_weight) S.photon_weight[L.pid] = L.weight;
                        if (SRC && S.photon_steps) S.photon_steps[L.pid] = 0;
                        L.mode = M_NEED;
                    }
                    }
                }
            }
            // a lane becomes M_DONE only here, so the warp can only have finished in a trip that
            // handed out photons: testing here instead of every trip is 0.3% faster
            if (__all_sync(kFull, L.mode == M_DONE)) break;
        }

        // ---- (1a) gate-phased runs: park photons whose time reached the next gate ----
        if (PHASED && !pa.last) {
            const SimDev& S = sims(0);
            // modes M_OUTER, M_INNER, M_FIXIN and M_SCAT as one bit test (0.9% faster than four compares)
            const bool live = ((kLiveModes >> L.mode) & 1u) != 0u;
            // the window's end as a time, precomputed on the host: where a photon is parked
            // changes only which launch continues it, not what it computes
            if (live && L.ptime >= pa.tpark) {
                cg::coalesced_group grp = cg::coalesced_threads();
                unsigned long long base = 0;
                if (grp.thread_rank() == 0) base = atomicAdd(pa.out.count, (unsigned long long)grp.size());
                base = grp.shfl(base, 0);
                const unsigned long long slot = base + grp.thread_rank();
                // each photon is parked at most once per gate, so slot < cap; checked all the same
                if (slot < pa.cap) {
                    const unsigned key = spatial_key(L.px, L.py, L.pz, pa);
                    atomicAdd(pa.bcount + key, 1u);
                    PState* q = pa.out.rec + slot;  // streaming stores: written once, read once
                    __stcs(&q->pos, make_float4(L.px, L.py, L.pz, L.ptime));
                    __stcs(&q->dir, make_float4(L.vx, L.vy, L.vz, L.weight));
                    // slen0 is read only by replay kernels; the others leave it out so it holds no register
                    // (forward kernels carry a shared photon's launch pixel there instead)
                    __stcs(&q->len, make_float4(L.slen, REPLAY ? L.slen0 : (SRC ? __int_as_float(L.posidx) : 0.f),
                                               L.oldw, __uint_as_float(L.oldidx)));
                    __stcs(&q->elem, make_int4(L.eid, L.label, L.mode, L.fixcount));
                    __stcs(&q->meta, make_uint4(L.steps, (unsigned)L.pid, (unsigned)(L.pid >> 32), key));
                    __stcs(&q->rng, make_uint4((unsigned)L.t0, (unsigned)(L.t0 >> 32), (unsigned)L.t1,
                                               (unsigned)(L.t1 >> 32)));
                    if (S.issavedet)
                        for (int i = 0; i < S.reclen; i++) __stcs(pa.out.ppath + slot * S.reclen + i, PP(i));
                    if (want_seed) {
                        __stcs(pa.out.seed0 + 2 * slot, seed0[tid]);
                        __stcs(pa.out.seed0 + 2 * slot + 1, seed0[bdim + tid]);
                    }
                } else {  // queue full (never expected): the photon is dropped and counted as aborted
                    atomicAdd(&s_cnt[1], 1ull);
                    atomicAdd(&s_cnt[0], (unsigned long long)L.steps);
                }
                L.mode = M_NEED;
            }
        }

        // ---- (1b) deferred roulette + scatter, src/mmc_core.cl:2101-2134 ----
        if (__any_sync(kFull, L.mode == M_SCAT)) {
            if (L.mode == M_SCAT) {
                const SimDev& S = sims(L.sim);
                const float4* med = smed + (BATCHED ? L.sim * nmed_stride : 0);
                bool killed = false;
                if (ROUL && S.roulette_on && (L.weight < S.minenergy)) {
                    if (rng_next(L.t0, L.t1) * S.roulettesize <= 1.f)
                        L.weight *= S.roulettesize;
                    else
                        killed = true;
                }
                if (killed) {
                    if (SRC && S.traj) save_traj(S, L);
                    if (SRC && S.photon_det) S.photon_det[L.pid] = 0;
                    tally.eesc += L.weight;
                    if (SRC && S.srcnum > 1) tally_sources(S, L.posidx, L.weight, 1);
                    if (BATCHED) tally.raytet += L.steps; else atomicAdd(&s_cnt[0], (unsigned long long)L.steps);
                    if (SRC && S.photon_weight) S.photon_weight[L.pid] = L.weight;
                    if (SRC && S.photon_steps) S.photon_steps[L.pid] = L.steps;
                    L.mode = M_NEED;
                } else {
                    if (REPLAY && S.replay && S.outputtype == OT_WN) {
                        const float gf = __ldg(S.replaytime + L.pid) * S.Rtstep;
                        int gate = (gf < (float)(S.maxgate - 1)) ? (int)gf : S.maxgate - 1;
                        gate = max(gate, 0);
                        deposit(S, (unsigned)(L.eid - 1) + (unsigned)(gate * S.ne), __ldg(S.replayweight + L.pid));
                    }
                    float ctheta;
                    const int tp = L.label;
                    L.slen0 = next_scatter<MP>(L, med[tp].z, ctheta);
                    L.slen = L.slen0;
                    if (SRC && S.traj) save_traj(S, L);
                    if (S.issavedet && tp > 0) {
                        const int M = S.nmedia - 1;
                        if (SRC && S.ismomentum) PP(2 * M + tp - 1) += (1.f - ctheta);
                        PP(tp - 1) += 1.f;
                    }
                    L.mode = M_OUTER;
                }
            }
        }
        if (((kIdleModes >> L.mode) & 1u) != 0u) continue;  // as one bit test: 1.0% faster

        const SimDev& S = sims(L.sim);
        const float4* med = smed + (BATCHED ? L.sim * nmed_stride : 0);
        const int M = S.nmedia - 1;

        // ---- (2) one ray-tet step ----
        const bool bad_elem = (L.eid < 1 || L.eid > S.ne);  // defensive: never expected
        if (!bad_elem) raytet_step<MP, REPLAY, SRC>(L, S, med);
        L.steps++;
        bool ended = false;
        const bool aborted = bad_elem || (L.steps > S.step_budget);
        // after_inner: 0 = continue stepping, 1 = go to exit/scatter decision
        int decide = 0;
        bool cross = false;

        // ---- (3) post-step control flow ----
        if (!aborted) {
            const int mode = L.mode;
            // partial path of a step that reached a face (outer mode) or ran to its end (inner
            // modes), as one site before the mode branches: 1.1% faster than one per branch
            if (S.issavedet && (mode != M_OUTER || L.hit) && L.Lmove > 0.f && L.label > 0) PP(M + L.label - 1) += L.Lmove;
            // a step that reached a face and did not use up its length crosses, whatever the mode
            // (a hit implies faceid >= 0); deciding it before the mode branches lets the warp run
            // one crossing block instead of one per branch (+0.5%)
            cross = L.hit && L.faceid >= 0 && !L.isend;
            if (cross) {
                if (mode == M_INNER) L.fixcount = 0;
            } else if (mode == M_OUTER) {
                if (!L.hit) {
                    if (L.faceid == -2) {
                        ended = true;
                    } else if (L.fixcount++ < kMaxTrial) {
                        fixphoton(L, S);
                    } else {
                        L.eid = kIdUndef;
                        L.faceid = -1;
                        decide = 1;
                    }
                } else {
                    decide = 1;
                }
            } else if (mode == M_INNER) {
                if (L.faceid == -2) {
                    decide = 1;
                } else {
                    L.fixcount = 0;
                    if (!L.hit) {
                        L.fixcount = 1;
                        fixphoton(L, S);
                        L.mode = M_FIXIN;
                    } else {
                        decide = 1;
                    }
                }
            } else {  // M_FIXIN
                if (!L.hit) {
                    if (L.fixcount++ < kMaxTrial) {
                        fixphoton(L, S);
                    } else {
                        L.eid = kIdUndef;
                        decide = 1;
                    }
                } else {
                    decide = 1;
                }
            }

            if (cross) {
                // face crossing, src/mmc_core.cl:1950-1993
                const int oldeid = L.eid, oldlabel = L.label;
                int eid = decode_nb(L.nbword, S.lbits);
                int nlabel = decode_label(L.nbword, S.lmask);
                // a crossing into the same medium cannot refract: its index loads are skipped (1.5% faster)
                if (S.isreflect && (eid <= 0 || nlabel != oldlabel)) {
                    const float nold = med[oldlabel].w;
                    if (eid <= 0 || med[nlabel].w != nold) {
                        if (!(eid <= 0 && (((nold == S.nout) && (S.isreflect != BC_MIRROR)) || (S.isreflect == BC_ABSORBEXT)))) {
                            eid = reflectray<MP>(L, S, med, oldeid, oldlabel, eid, nlabel, L.faceid);
                            if (eid == oldeid) nlabel = oldlabel;
                        }
                    }
                }
                L.eid = eid;
                if (eid <= 0) {
                    decide = 1;
                } else {
                    if (oldlabel == 0 && nlabel != 0 && !S.voidtime) L.ptime = 0.f;
                    if (oldlabel != 0 && nlabel == 0) {
                        L.eid = 0;
                        decide = 1;
                    } else {
                        L.label = nlabel;
                        L.mode = M_INNER;
                    }
                }
            }

            if (decide) {
                // exit / roulette / scatter, src/mmc_core.cl:2033-2138
                if (L.eid <= 0 || !L.hit) {
                    if (L.eid != kIdUndef && S.issavedet && S.issaveexit) {
                        PP(S.reclen - 7) = L.px;
                        PP(S.reclen - 6) = L.py;
                        PP(S.reclen - 5) = L.pz;
                        PP(S.reclen - 4) = L.vx;
                        PP(S.reclen - 3) = L.vy;
                        PP(S.reclen - 2) = L.vz;
                    }
                    // diffuse reflectance/transmittance per exterior face, src/mmc_raytrace.c:2000-2003
                    if (S.dref && L.eid < 0 && -L.eid <= S.nf) {
                        const float gf = (L.ptime - S.tstart) * S.Rtstep;
                        int gate = (gf < (float)(S.maxgate - 1)) ? (int)gf : S.maxgate - 1;
                        gate = max(gate, 0);
                        atomicAdd(S.dref + ((-L.eid) - 1) + (size_t)gate * S.nf, (double)L.weight);
                    }
                    int detid = 0;
                    if (S.issavedet && L.eid <= 0) {
                        detid = finddetector(L, S);
                        if (detid) {
                            // ballot-compacted slot reservation: one atomic per group of detecting
                            // lanes of the same simulation (a batched warp mixes simulations)
                            cg::coalesced_group grp = BATCHED ? cg::labeled_partition(cg::coalesced_threads(), L.sim)
                                                              : cg::coalesced_threads();
                            unsigned base = 0;
                            if (grp.thread_rank() == 0) base = atomicAdd(S.detcount, grp.size());
                            base = grp.shfl(base, 0);
                            const unsigned slot = base + grp.thread_rank();
                            if (slot < S.maxdet) {
                                if (S.seeds && want_seed) {
                                    S.seeds[2 * (size_t)slot] = seed0[tid];
                                    S.seeds[2 * (size_t)slot + 1] = seed0[bdim + tid];
                                }
                                float* rec = S.detp + (size_t)slot * (S.reclen + 1);
                                rec[0] = (float)detid;
                                for (int i = 0; i < S.reclen; i++) rec[1 + i] = PP(i);
                            }
                        }
                    }
                    if (SRC && S.photon_det) S.photon_det[L.pid] = detid;
                    ended = true;
                } else {
                    L.mode = M_SCAT;  // roulette + scatter run batched at the top of a later trip
                }
            } else if (ended) {
                if (SRC && S.photon_det) S.photon_det[L.pid] = 0;
            }
        } else {
            ended = true;
            if (BATCHED) tally.aborted++; else atomicAdd(&s_cnt[1], 1ull);
            if (SRC && S.photon_det) S.photon_det[L.pid] = 0;
        }
        if (ended) {
            if (SRC && S.traj) save_traj(S, L);
            tally.eesc += L.weight;
            if (SRC && S.srcnum > 1) tally_sources(S, L.posidx, L.weight, 1);
            if (BATCHED) tally.raytet += L.steps; else atomicAdd(&s_cnt[0], (unsigned long long)L.steps);
            if (SRC && S.photon_weight) S.photon_weight[L.pid] = L.weight;
            if (SRC && S.photon_steps) S.photon_steps[L.pid] = L.steps;
            L.mode = M_NEED;
        }
    }
#undef PP
    if (tally.sim >= 0) flush_tally(tally, sims(tally.sim));
    if (!BATCHED) {
        __syncthreads();
        if (threadIdx.x == 0) {
            const SimDev& S = sims(0);
            if (s_cnt[0]) atomicAdd(S.counters + 0, s_cnt[0]);
            if (s_cnt[1]) atomicAdd(S.counters + 1, s_cnt[1]);
            if (s_cnt[2] && S.ncounters > 2) atomicAdd(S.counters + 2, s_cnt[2]);
        }
    }
}

template <class MP, bool REPLAY, int KIND>
__global__ void __launch_bounds__(128, 8) photon_engine_plain(const __grid_constant__ SimDev sim,
                                                              unsigned long long* work_counter, int reclen_max,
                                                              int want_seed) {
    SingleSim acc{sim};
    const PhaseArgs none{};
    engine_body<MP, SingleSim, false, false, REPLAY, KIND>(acc, nullptr, 1, sim.nphoton, sim.nmedia, reclen_max,
                                                          want_seed, work_counter, none);
}

template <class MP, int KIND>
__global__ void __launch_bounds__(128, 8) photon_engine_phased(const __grid_constant__ SimDev sim,
                                                               const __grid_constant__ PhaseArgs pa,
                                                               unsigned long long* work_counter, int reclen_max,
                                                               int want_seed) {
    SingleSim acc{sim};
    // gate 0 launches the run's photons; later gates resume the ones parked by the previous launch
    unsigned long long total = sim.nphoton;
    if (pa.phase > 0) total = min(*pa.in.count, pa.cap);
    engine_body<MP, SingleSim, false, true, false, KIND>(acc, nullptr, 1, total, sim.nmedia, reclen_max, want_seed,
                                                        work_counter, pa);
}

template <class MP, bool REPLAY, int KIND>
__global__ void __launch_bounds__(128, 8) photon_engine_batched(const SimDev* __restrict__ sims,
                                                                const unsigned long long* __restrict__ cum,
                                                                int nsims, unsigned long long total,
                                                                int nmed_stride, unsigned long long* work_counter,
                                                                int reclen_max, int want_seed) {
    ManySims acc{sims};
    const PhaseArgs none{};
    engine_body<MP, ManySims, true, false, REPLAY, KIND>(acc, cum, nsims, total, nmed_stride, reclen_max, want_seed,
                                                      work_counter, none);
}

size_t smem_bytes(int nmed_rows, int reclen_max, int threads, int want_seed) {
    size_t b = (size_t)nmed_rows * sizeof(float4) + (size_t)reclen_max * threads * sizeof(float);
    b = (b + 7) & ~(size_t)7;
    if (want_seed) b += (size_t)2 * threads * sizeof(unsigned long long);
    return b;
}

}  // namespace

#if MMCGB_ENGINE_FAST
namespace {
// Per gate-0 cell: the sum of its copies, in copy order, is added to the cell and the copies
// are cleared for the next launch (only the ones that took deposits are written).
__global__ void fold_hot_kernel(double* __restrict__ hot, double* __restrict__ f64, unsigned ne) {
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < ne; i += gridDim.x * blockDim.x) {
        double sum = 0.0;
        for (int r = 0; r < kHotReps; r++) {
            double* p = hot + (size_t)r * ne + i;
            const double v = *p;
            if (v != 0.0) {
                sum += v;
                *p = 0.0;
            }
        }
        if (sum != 0.0) f64[i] += sum;
    }
}
}  // namespace

cudaError_t fold_hot(const SimDev& s, cudaStream_t stream) {
    if (!s.hot_steps) return cudaSuccess;
    const unsigned blocks = std::min<unsigned>(((unsigned)s.ne + 255) / 256, 152u * 8u);
    fold_hot_kernel<<<blocks, 256, 0, stream>>>(s.hot, s.f64, (unsigned)s.ne);
    return cudaGetLastError();
}

#endif

// Kernels compiled with the general launch and deposit (SRC) serve
// simulations whose source is not a pencil beam starting in a known element,
// that deposit into a voxel grid, record trajectories, write the per-photon
// trace outputs, save momentum transfer or read per-node properties; the others carry only the pencil
// launch and the element deposit, which keeps the step loop lean (the trace
// outputs' eleven null tests alone cost the pencil kernels 4.9%, the roulette
// and momentum tests 2%).  Forward single-simulation runs with Russian
// roulette have a pencil kernel of their own (KIND_ROULETTE).
#if MMCGB_ENGINE_FAST
bool general_source(const SimDev& s) {
    return s.srctype != ST_PENCIL || s.e0 <= 0 || s.grid || s.traj || s.photon_weight || s.photon_steps ||
           s.photon_det || s.ismomentum || s.nodemua;
}
#endif

#if MMCGB_ENGINE_FAST
#define MMCGB_POLICY_NS fast
using Policy = FastMath;
#else
#define MMCGB_POLICY_NS exact
using Policy = ExactMath;
#endif

template <class MP, bool REPLAY, int KIND>
static cudaError_t launch_plain_t(const SimDev& sim, unsigned long long* work_counter, LaunchShape shape,
                                  cudaStream_t stream) {
    const int want_seed = (sim.issavedet && sim.seeds) ? 1 : 0;
    const int reclen_max = sim.issavedet ? sim.reclen : 0;
    const size_t smem = smem_bytes(sim.nmedia, reclen_max, shape.threads, want_seed);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(photon_engine_plain<MP, REPLAY, KIND>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    cudaError_t e = cudaMemsetAsync(work_counter, 0, sizeof(unsigned long long), stream);
    if (e != cudaSuccess) return e;
    (void)cudaGetLastError();  // the launch check below must see this launch's status only
    photon_engine_plain<MP, REPLAY, KIND><<<shape.blocks, shape.threads, smem, stream>>>(sim, work_counter,
                                                                                       reclen_max, want_seed);
    return cudaGetLastError();
}

template <class MP, int KIND>
static cudaError_t launch_phased_t(const SimDev& sim, unsigned long long* work_counter, LaunchShape shape,
                                   cudaStream_t stream, const PhaseQueue q[2], int span, unsigned* order,
                                   unsigned* bscratch, const float lo[3], const float hi[3]) {
    const int want_seed = (sim.issavedet && sim.seeds) ? 1 : 0;
    const int reclen_max = sim.issavedet ? sim.reclen : 0;
    const size_t smem = smem_bytes(sim.nmedia, reclen_max, shape.threads, want_seed);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(photon_engine_phased<MP, KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
    }
    span = std::max(1, span);
    for (int g = 0, k = 0; g < sim.maxgate; g += span, k++) {
        PhaseArgs pa;
        pa.phase = g;
        pa.span = span;
        pa.tpark = sim.tstart + (float)(g + span) / sim.Rtstep;
        pa.last = (g + span >= sim.maxgate) ? 1 : 0;
        pa.in = q[(k + 1) & 1];  // written by the previous launch
        pa.out = q[k & 1];
        pa.cap = sim.nphoton;
        pa.order = (k > 0 && order) ? order : nullptr;
        pa.bcount = bscratch;
        for (int a = 0; a < 3; a++) {
            pa.lo[a] = lo[a];
            pa.scale[a] = (hi[a] > lo[a]) ? (float)(1 << kSortBits) / (hi[a] - lo[a]) : 0.f;
        }
        cudaError_t e = cudaMemsetAsync(work_counter, 0, sizeof(unsigned long long), stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(pa.out.count, 0, sizeof(unsigned long long), stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(bscratch, 0, sizeof(unsigned) * kBuckets, stream);
        if (e != cudaSuccess) return e;
        (void)cudaGetLastError();
        photon_engine_phased<MP, KIND><<<shape.blocks, shape.threads, smem, stream>>>(sim, pa, work_counter,
                                                                                    reclen_max, want_seed);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        if (!pa.last && order) {  // resume order of the photons just parked
            k_bucket_scan<<<1, 1024, 0, stream>>>(bscratch, bscratch + kBuckets);
            k_bucket_order<<<shape.blocks, 256, 0, stream>>>(pa.out.rec, pa.out.count, pa.cap, bscratch + kBuckets,
                                                            order);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
        }
    }
    return cudaSuccess;
}

template <class MP, bool REPLAY, int KIND>
static cudaError_t launch_batched_t(const SimDev* sims, const unsigned long long* cum, int nsims,
                                    unsigned long long total, int nmed_stride, int reclen_max, int want_seed,
                                    unsigned long long* work_counter, LaunchShape shape, cudaStream_t stream) {
    const size_t smem = smem_bytes(nsims * nmed_stride, reclen_max, shape.threads, want_seed);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(photon_engine_batched<MP, REPLAY, KIND>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    cudaError_t e = cudaMemsetAsync(work_counter, 0, sizeof(unsigned long long), stream);
    if (e != cudaSuccess) return e;
    (void)cudaGetLastError();  // the launch check below must see this launch's status only
    // a batch holding a replay simulation runs the kernel with the replay branches
    photon_engine_batched<MP, REPLAY, KIND><<<shape.blocks, shape.threads, smem, stream>>>(
        sims, cum, nsims, total, nmed_stride, work_counter, reclen_max, want_seed);
    return cudaGetLastError();
}

// The launchers of this unit's arithmetic policy.
namespace MMCGB_POLICY_NS {

cudaError_t launch_plain(const SimDev& sim, unsigned long long* work_counter, LaunchShape shape,
                         cudaStream_t stream) {
    // replays with roulette run in the general kernel (the roulette pencil kernel is forward-only)
    const bool src = general_source(sim) || (sim.replay && sim.roulette_on);
    if (sim.replay)
        return src ? launch_plain_t<Policy, true, KIND_GENERAL>(sim, work_counter, shape, stream)
                   : launch_plain_t<Policy, true, KIND_LEAN>(sim, work_counter, shape, stream);
    if (src) return launch_plain_t<Policy, false, KIND_GENERAL>(sim, work_counter, shape, stream);
    return sim.roulette_on ? launch_plain_t<Policy, false, KIND_ROULETTE>(sim, work_counter, shape, stream)
                           : launch_plain_t<Policy, false, KIND_LEAN>(sim, work_counter, shape, stream);
}

cudaError_t launch_phased(const SimDev& sim, unsigned long long* work_counter, LaunchShape shape,
                          cudaStream_t stream, const PhaseQueue q[2], int span, unsigned* order,
                          unsigned* bscratch, const float lo[3], const float hi[3]) {
    // roulette needs a single gate window, so phased runs never play it; checked all the same
    return (general_source(sim) || sim.roulette_on)
               ? launch_phased_t<Policy, KIND_GENERAL>(sim, work_counter, shape, stream, q, span, order, bscratch, lo, hi)
               : launch_phased_t<Policy, KIND_LEAN>(sim, work_counter, shape, stream, q, span, order, bscratch, lo, hi);
}

cudaError_t launch_batched(const SimDev* sims, const unsigned long long* cum, int nsims,
                           unsigned long long total, int nmed_stride, int reclen_max, int want_seed,
                           unsigned long long* work_counter, LaunchShape shape, cudaStream_t stream,
                           int general_src, int replay) {
#define MMCGB_BATCHED(R, G) \
    launch_batched_t<Policy, R, G>(sims, cum, nsims, total, nmed_stride, reclen_max, want_seed, work_counter, shape, stream)
    if (replay) return general_src ? MMCGB_BATCHED(true, KIND_GENERAL) : MMCGB_BATCHED(true, KIND_LEAN);
    return general_src ? MMCGB_BATCHED(false, KIND_GENERAL) : MMCGB_BATCHED(false, KIND_LEAN);
#undef MMCGB_BATCHED
}

}  // namespace MMCGB_POLICY_NS

#if MMCGB_ENGINE_FAST
// Entry points (engine.h): one definition, in the fast unit, dispatching on the policy.
LaunchShape default_shape(int device, bool batched) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    int per_sm = 0;
    const int threads = 128;
    if (batched)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, photon_engine_batched<FastMath, true, KIND_LEAN>, threads,
                                                      4096);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, photon_engine_plain<FastMath, false, KIND_LEAN>, threads,
                                                      1024);
    if (per_sm < 1) per_sm = 1;
    return LaunchShape{sms * per_sm, threads};
}

size_t phase_bytes_per_photon(const SimDev& sim) {
    const int want_seed = (sim.issavedet && sim.seeds) ? 1 : 0;
    return 2 * (sizeof(PState) + (sim.issavedet ? (size_t)sim.reclen * sizeof(float) : 0) +
                (want_seed ? 2 * sizeof(unsigned long long) : 0));
}

cudaError_t launch_plain(const SimDev& sim, unsigned long long* work_counter, LaunchShape shape,
                         cudaStream_t stream) {
    return sim.fast_math ? fast::launch_plain(sim, work_counter, shape, stream)
                         : exact::launch_plain(sim, work_counter, shape, stream);
}

cudaError_t launch_phased(const SimDev& sim, unsigned long long* work_counter, LaunchShape shape,
                          cudaStream_t stream, const PhaseQueue q[2], int span, unsigned* order,
                          unsigned* bscratch, const float lo[3], const float hi[3]) {
    return sim.fast_math ? fast::launch_phased(sim, work_counter, shape, stream, q, span, order, bscratch, lo, hi)
                         : exact::launch_phased(sim, work_counter, shape, stream, q, span, order, bscratch, lo, hi);
}

cudaError_t launch_batched(const SimDev* sims, const unsigned long long* cum, int nsims,
                           unsigned long long total, int nmed_stride, int reclen_max, int want_seed,
                           unsigned long long* work_counter, LaunchShape shape, cudaStream_t stream, int fast_math,
                           int general_src, int replay) {
    return fast_math ? fast::launch_batched(sims, cum, nsims, total, nmed_stride, reclen_max, want_seed,
                                            work_counter, shape, stream, general_src, replay)
                     : exact::launch_batched(sims, cum, nsims, total, nmed_stride, reclen_max, want_seed,
                                             work_counter, shape, stream, general_src, replay);
}
#endif

}  // namespace mmcgb

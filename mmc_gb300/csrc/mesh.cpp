// Host-side mesh preparation for the photon engine: orientation fix and
// volumes, face neighbours, face normals/plane offsets, exterior-face
// numbering, packed 80-byte records, and point location for the source.
// Compiled with -ffp-contract=off: the normals feed the bit-exact parity
// contract with the CPU oracle.
#include "mesh.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>

namespace mmcgb {

// face tables of the reference (src/mmc_mesh.c:59-107, src/mmc_highorder.cpp:50)
const int kOut[4][3] = {{0, 3, 1}, {3, 2, 1}, {0, 2, 3}, {0, 1, 2}};
const int kFaceMap[4] = {2, 0, 1, 3};
const int kIFaceOrder[4] = {3, 0, 2, 1};
const int kFaceList[4][3] = {{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}};

namespace {

struct F3 {
    float x, y, z;
};

inline F3 node_at(const std::vector<float>& node, int i) {
    return F3{node[3 * (size_t)i], node[3 * (size_t)i + 1], node[3 * (size_t)i + 2]};
}

// Runs body(begin, end) over [0, n) split into contiguous ranges, one per
// hardware thread (at most 16); small ranges run on the calling thread.
template <class F>
void parallel_ranges(size_t n, F body) {
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const size_t nt = std::min<size_t>(hw, std::max<size_t>(1, n / 65536));
    if (nt <= 1) {
        body((size_t)0, n);
        return;
    }
    std::vector<std::thread> pool;
    pool.reserve(nt - 1);
    for (size_t t = 1; t < nt; t++) pool.emplace_back(body, n * t / nt, n * (t + 1) / nt);
    body((size_t)0, n / nt);
    for (std::thread& th : pool) th.join();
}

// Face neighbours (src/mmc_highorder.cpp:128-159): element faces are matched by
// their sorted node triple; facenb[4e+j] is the element sharing face j.  The
// faces are ordered by (smallest node, middle node, largest node, face slot):
// a counting sort on the smallest node, then each node's short list sorted on
// its own; runs of equal triples pair up in that order (first with second,
// third with fourth, ...).
void compute_facenb(int nn, int ne, const std::vector<int>& elem, std::vector<int>& facenb) {
    const size_t nface = (size_t)ne * 4;
    facenb.assign(nface, 0);
    std::vector<int> tri(3 * nface);
    parallel_ranges((size_t)ne, [&](size_t b, size_t e) {
        for (size_t i = b; i < e; i++)
            for (int j = 0; j < 4; j++) {
                int* v = &tri[3 * (4 * i + j)];
                v[0] = elem[4 * i + kFaceList[j][0]];
                v[1] = elem[4 * i + kFaceList[j][1]];
                v[2] = elem[4 * i + kFaceList[j][2]];
                std::sort(v, v + 3);
            }
    });
    // bucket the faces by smallest node (counts and fill with relaxed atomics: the order inside a
    // bucket does not matter, the sort below breaks ties by face slot)
    std::vector<uint32_t> start((size_t)nn + 2, 0);
    parallel_ranges(nface, [&](size_t b, size_t e) {
        for (size_t f = b; f < e; f++) __atomic_fetch_add(&start[(size_t)tri[3 * f] + 1], 1u, __ATOMIC_RELAXED);
    });
    for (size_t i = 1; i < start.size(); i++) start[i] += start[i - 1];
    std::vector<uint32_t> order(nface);
    {
        std::vector<uint32_t> fill(start.begin(), start.end() - 1);
        parallel_ranges(nface, [&](size_t b, size_t e) {
            for (size_t f = b; f < e; f++)
                order[__atomic_fetch_add(&fill[(size_t)tri[3 * f]], 1u, __ATOMIC_RELAXED)] = (uint32_t)f;
        });
    }
    parallel_ranges((size_t)nn + 1, [&](size_t b, size_t e) {
        for (size_t v0 = b; v0 < e; v0++) {
            uint32_t* lo = order.data() + start[v0];
            uint32_t* hi = order.data() + start[v0 + 1];
            std::sort(lo, hi, [&](uint32_t a, uint32_t c) {
                const int* ta = &tri[3 * (size_t)a];
                const int* tc = &tri[3 * (size_t)c];
                if (ta[1] != tc[1]) return ta[1] < tc[1];
                if (ta[2] != tc[2]) return ta[2] < tc[2];
                return a < c;
            });
            for (uint32_t* q = lo; q + 1 < hi; q++) {
                const int* ta = &tri[3 * (size_t)q[0]];
                const int* tb = &tri[3 * (size_t)q[1]];
                if (ta[1] == tb[1] && ta[2] == tb[2]) {
                    facenb[q[0]] = (int)(q[1] >> 2) + 1;
                    facenb[q[1]] = (int)(q[0] >> 2) + 1;
                    q++;
                }
            }
        }
    });
}

}  // namespace

int prepare_mesh(const mmcgb_mesh_desc& d, HostMesh& m, std::string& err) {
    if (d.nn <= 0 || d.ne <= 0 || !d.node || !d.elem || !d.label) {
        err = "mesh needs nn > 0, ne > 0 and node/elem/label arrays";
        return MMCGB_E_ARG;
    }
    int maxlabel = 0;
    for (int i = 0; i < d.ne; i++) {
        // -1 marks the reference's source-element candidates, which it then treats as
        // void (mesh_srcdetelem, src/mmc_mesh.c:390-425); sources are located here by a
        // search over all elements, so such a tet is simply void
        const int lab = (d.label[i] == -1) ? 0 : d.label[i];
        if (lab < 0 || lab > kMaxLabel) {
            err = "medium labels must be in -1.." + std::to_string(kMaxLabel) +
                  " (-2, wide-field detector elements, is not supported)";
            return MMCGB_E_MESH;
        }
        maxlabel = std::max(maxlabel, lab);
    }
    // the packed face words share 32 bits between the neighbour id and its label
    const int lbits = label_bits(maxlabel);
    if (d.ne > max_elem(lbits)) {
        err = "mesh has more elements than the packed record format holds with labels up to " +
              std::to_string(maxlabel) + " (" + std::to_string(max_elem(lbits)) + ")";
        return MMCGB_E_MESH;
    }
    m.nn = d.nn;
    m.ne = d.ne;
    m.maxlabel = maxlabel;
    m.lbits = lbits;
    m.node.assign(d.node, d.node + 3 * (size_t)d.nn);
    m.elem.assign(d.elem, d.elem + 4 * (size_t)d.ne);
    m.label.assign(d.label, d.label + (size_t)d.ne);
    for (int& lab : m.label)
        if (lab == -1) lab = 0;
    m.evol.assign(d.ne, 0.f);
    m.nvol.assign(d.nn, 0.f);
    for (size_t i = 0; i < 4 * (size_t)d.ne; i++)
        if (m.elem[i] < 1 || m.elem[i] > d.nn) {
            err = "element " + std::to_string(i / 4 + 1) + " references a node outside 1..nn";
            return MMCGB_E_MESH;
        }
    // volumes and orientation (src/mmc_mesh.c:910-974): swap nodes 3,4 of a
    // negatively oriented tet so that the face tables give outward normals
    parallel_ranges((size_t)d.ne, [&](size_t b, size_t end) {
    for (size_t i = b; i < end; i++) {
        int* e = &m.elem[4 * i];
        F3 n0 = node_at(m.node, e[0] - 1), n1 = node_at(m.node, e[1] - 1), n2 = node_at(m.node, e[2] - 1),
           n3 = node_at(m.node, e[3] - 1);
        float dx = n2.x - n3.x, dy = n2.y - n3.y, dz = n2.z - n3.z;
        float v = n1.x * (n2.y * n3.z - n2.z * n3.y) - n1.y * (n2.x * n3.z - n2.z * n3.x) +
                  n1.z * (n2.x * n3.y - n2.y * n3.x);
        v += -n0.x * ((n2.y * n3.z - n2.z * n3.y) + n1.y * dz - n1.z * dy);
        v += +n0.y * ((n2.x * n3.z - n2.z * n3.x) + n1.x * dz - n1.z * dx);
        v += -n0.z * ((n2.x * n3.y - n2.y * n3.x) + n1.x * dy - n1.y * dx);
        v = -v;
        if (v < 0.f) {
            std::swap(e[2], e[3]);
            v = -v;
        }
        v *= (1.f / 6.f);
        m.evol[i] = v;
    }
    });
    // nodal volumes: float sums in element order, as the reference adds them
    for (size_t i = 0; i < (size_t)d.ne; i++) {
        if (m.label[i] == 0) continue;
        const int* e = &m.elem[4 * i];
        const float q = m.evol[i] * 0.25f;
        for (int j = 0; j < 4; j++) m.nvol[e[j] - 1] += q;
    }
    if (d.facenb) {
        m.facenb.assign(d.facenb, d.facenb + 4 * (size_t)d.ne);
        for (size_t i = 0; i < m.facenb.size(); i++)
            if (m.facenb[i] < 0 || m.facenb[i] > d.ne) {
                err = "facenb entries must be 0 (exterior) or a 1-based element id";
                return MMCGB_E_MESH;
            }
    } else {
        compute_facenb(d.nn, d.ne, m.elem, m.facenb);
    }
    // exterior faces numbered -1,-2,... (src/mmc_mesh.c:1466-1474)
    const long long nf_max = (long long)max_elem(m.lbits) + 1;
    long long nf = 0;
    for (size_t i = 0; i < m.facenb.size(); i++)
        if (m.facenb[i] == 0) {
            if (++nf > nf_max) {
                err = "too many exterior faces for the packed record format";
                return MMCGB_E_MESH;
            }
            m.facenb[i] = -(int)nf;
        }
    m.nf = (int)nf;
    return MMCGB_OK;
}

// Outward unit normals and plane offsets of element i (src/mmc_mesh.c:1572-1601):
// vn = nx[4] ny[4] nz[4] d[4].  Computed where they are used (the packed records,
// the host-stage export) rather than kept as a mesh array.
void element_normals(const HostMesh& m, size_t i, float vn[16]) {
    const int* e = &m.elem[4 * i];
    for (int j = 0; j < 4; j++) {
        F3 a = node_at(m.node, e[kOut[j][0]] - 1);
        F3 b = node_at(m.node, e[kOut[j][1]] - 1);
        F3 c = node_at(m.node, e[kOut[j][2]] - 1);
        F3 ab{b.x - a.x, b.y - a.y, b.z - a.z};
        F3 ac{c.x - a.x, c.y - a.y, c.z - a.z};
        F3 n{ab.y * ac.z - ab.z * ac.y, ab.z * ac.x - ab.x * ac.z, ab.x * ac.y - ab.y * ac.x};
        float rn = (float)(1.f / std::sqrt((double)(n.x * n.x + n.y * n.y + n.z * n.z)));
        n.x *= rn;
        n.y *= rn;
        n.z *= rn;
        vn[j] = n.x;
        vn[j + 4] = n.y;
        vn[j + 8] = n.z;
        vn[j + 12] = n.x * a.x + n.y * a.y + n.z * a.z;
    }
}

void element_normals_all(const HostMesh& m, float* out) {
    parallel_ranges((size_t)m.ne, [&](size_t b, size_t end) {
        for (size_t i = b; i < end; i++) element_normals(m, i, out + 16 * i);
    });
}

void pack_records(const HostMesh& m, std::vector<TetRec>& rec) {
    rec.resize(m.ne);
    const int lb = m.lbits;
    parallel_ranges((size_t)m.ne, [&](size_t b, size_t end) {
    for (size_t i = b; i < end; i++) {
        float vn[16];
        element_normals(m, i, vn);
        TetRec& r = rec[i];
        r.nx = make_float4(vn[0], vn[1], vn[2], vn[3]);
        r.ny = make_float4(vn[4], vn[5], vn[6], vn[7]);
        r.nz = make_float4(vn[8], vn[9], vn[10], vn[11]);
        r.nd = make_float4(vn[12], vn[13], vn[14], vn[15]);
        int w[4];
        for (int j = 0; j < 4; j++) {
            const int nbid = m.facenb[4 * i + j];
            const int lab = (nbid > 0) ? m.label[nbid - 1] : 0;
            w[j] = (int)(((uint32_t)nbid << lb) | (uint32_t)lab);
        }
        r.nb = make_int4(w[0], w[1], w[2], w[3]);
    }
    });
}

// ---------------------------------------------------------------------------
// point location: the reference scans all elements and takes the first whose
// bounding box and barycentric test enclose the point (src/mmc_mesh.c:1060-1090,
// :1170-1205).  A uniform grid of bounding boxes gives the same answer (the
// smallest qualifying index) without the O(ne) scan per request.
// ---------------------------------------------------------------------------
namespace {
bool build_locator(HostMesh& m) {
    float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
    for (int i = 0; i < m.nn; i++)
        for (int d = 0; d < 3; d++) {
            lo[d] = std::min(lo[d], m.node[3 * (size_t)i + d]);
            hi[d] = std::max(hi[d], m.node[3 * (size_t)i + d]);
        }
    int res = std::max(1, (int)std::cbrt((double)m.ne / 4.0));
    res = std::min(res, 256);
    LocGrid& g = m.grid;
    g.res = res;
    for (int d = 0; d < 3; d++) {
        g.lo[d] = lo[d];
        float span = hi[d] - lo[d];
        g.inv[d] = span > 0 ? res / span : 0.f;
    }
    const size_t nbin = (size_t)res * res * res;
    const size_t ne = (size_t)m.ne;
    // bins spanned by each element's bounding box: x, y, z low, then x, y, z high
    std::vector<int> br(6 * ne);
    parallel_ranges(ne, [&](size_t b, size_t e_end) {
        for (size_t e = b; e < e_end; e++) {
            float mn[3] = {1e30f, 1e30f, 1e30f}, mx[3] = {-1e30f, -1e30f, -1e30f};
            for (int j = 0; j < 4; j++)
                for (int d = 0; d < 3; d++) {
                    float v = m.node[3 * (size_t)(m.elem[4 * e + j] - 1) + d];
                    mn[d] = std::min(mn[d], v);
                    mx[d] = std::max(mx[d], v);
                }
            for (int d = 0; d < 3; d++) {
                br[6 * e + d] = std::max(0, std::min(res - 1, (int)std::floor((mn[d] - g.lo[d]) * g.inv[d])));
                br[6 * e + 3 + d] = std::max(0, std::min(res - 1, (int)std::floor((mx[d] - g.lo[d]) * g.inv[d])));
            }
        }
    });
    // Contiguous element chunks count and then fill their bins independently; chunk c's
    // entries of a bin follow those of chunks < c, so every bin lists its elements in
    // ascending order, as one pass over the elements would.  Per-chunk counts take at
    // most 64 MB.
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    size_t nchunk = std::min<size_t>(hw, ((size_t)64 << 20) / (4 * nbin));
    nchunk = std::max<size_t>(1, std::min<size_t>(nchunk, ne / 65536));
    std::vector<std::vector<uint32_t>> cnt(nchunk, std::vector<uint32_t>(nbin, 0));
    auto over_chunks = [&](auto body) {
        std::vector<std::thread> pool;
        for (size_t c = 1; c < nchunk; c++) pool.emplace_back(body, c);
        body((size_t)0);
        for (std::thread& th : pool) th.join();
    };
    auto for_bins = [&](size_t e, auto fn) {
        const int* r = &br[6 * e];
        for (int z = r[2]; z <= r[5]; z++)
            for (int y = r[1]; y <= r[4]; y++)
                for (int x = r[0]; x <= r[3]; x++) fn(((size_t)z * res + y) * res + x);
    };
    over_chunks([&](size_t c) {
        std::vector<uint32_t>& k = cnt[c];
        for (size_t e = ne * c / nchunk; e < ne * (c + 1) / nchunk; e++) for_bins(e, [&](size_t bin) { k[bin]++; });
    });
    // the CSR offsets are 32-bit (the device walks them as such)
    uint64_t pairs = 0;
    for (size_t c = 0; c < nchunk; c++)
        for (size_t bin = 0; bin < nbin; bin++) pairs += cnt[c][bin];
    if (pairs > 0xFFFFFFFFull) return false;
    g.start.assign(nbin + 1, 0);
    uint32_t run = 0;
    for (size_t bin = 0; bin < nbin; bin++) {
        g.start[bin] = run;
        for (size_t c = 0; c < nchunk; c++) {
            const uint32_t k = cnt[c][bin];
            cnt[c][bin] = run;  // this chunk's first slot in the bin
            run += k;
        }
    }
    g.start[nbin] = run;
    g.items.assign(run, 0);
    over_chunks([&](size_t c) {
        std::vector<uint32_t>& k = cnt[c];
        for (size_t e = ne * c / nchunk; e < ne * (c + 1) / nchunk; e++)
            for_bins(e, [&](size_t bin) { g.items[k[bin]++] = (uint32_t)e; });
    });
    return true;
}
}  // namespace

bool ensure_locator(HostMesh& m) {
    if (m.grid_built.load(std::memory_order_acquire)) return true;
    std::lock_guard<std::mutex> lock(m.grid_mu);
    if (m.grid_built.load(std::memory_order_relaxed)) return true;
    if (!build_locator(m)) return false;
    m.grid_built.store(true, std::memory_order_release);
    return true;
}

static bool encloses(const HostMesh& m, int e, const float* p) {
    const int* el = &m.elem[4 * (size_t)e];
    double lo[3] = {1e30, 1e30, 1e30}, hi[3] = {-1e30, -1e30, -1e30};
    for (int j = 0; j < 4; j++)
        for (int d = 0; d < 3; d++) {
            double v = m.node[3 * (size_t)(el[j] - 1) + d];
            lo[d] = std::min(lo[d], v);
            hi[d] = std::max(hi[d], v);
        }
    if (!(p[0] <= hi[0] && p[0] >= lo[0] && p[1] <= hi[1] && p[1] >= lo[1] && p[2] <= hi[2] && p[2] >= lo[2]))
        return false;
    float bary[4];
    for (int i = 0; i < 4; i++) {
        F3 a = node_at(m.node, el[kOut[i][0]] - 1);
        F3 b = node_at(m.node, el[kOut[i][1]] - 1);
        F3 c = node_at(m.node, el[kOut[i][2]] - 1);
        F3 ab{b.x - a.x, b.y - a.y, b.z - a.z};
        F3 ac{c.x - a.x, c.y - a.y, c.z - a.z};
        F3 s{p[0] - a.x, p[1] - a.y, p[2] - a.z};
        F3 n{ab.y * ac.z - ab.z * ac.y, ab.z * ac.x - ab.x * ac.z, ab.x * ac.y - ab.y * ac.x};
        bary[kFaceMap[i]] = -(s.x * n.x + s.y * n.y + s.z * n.z);
    }
    for (int i = 0; i < 4; i++)
        if (bary[i] < 0.f) return false;
    return true;
}

int locate(const HostMesh& m, const float p[3]) {
    if (!m.grid_built.load(std::memory_order_acquire)) {
        // no grid yet: every element, in parallel ranges, each range's lowest enclosing index
        std::vector<int> best_of(16, -1);
        std::atomic<int> slot{0};
        parallel_ranges((size_t)m.ne, [&](size_t b, size_t e) {
            int best = -1;
            for (size_t i = b; i < e && best < 0; i++)
                if (encloses(m, (int)i, p)) best = (int)i;
            best_of[slot.fetch_add(1)] = best;
        });
        int best = -1;
        for (int v : best_of)
            if (v >= 0 && (best < 0 || v < best)) best = v;
        return best >= 0 ? best + 1 : 0;
    }
    const LocGrid& g = m.grid;
    int b[3];
    for (int d = 0; d < 3; d++) {
        float f = (p[d] - g.lo[d]) * g.inv[d];
        if (!(f >= -1e-3f * g.res) || !(f <= g.res * (1.f + 1e-3f))) return 0;
        b[d] = std::max(0, std::min(g.res - 1, (int)std::floor(f)));
    }
    // a point on a bin boundary may belong to elements binned only in the
    // neighbouring bin: look at every bin within one cell and take the minimum
    int best = -1;
    for (int z = std::max(0, b[2] - 1); z <= std::min(g.res - 1, b[2] + 1); z++)
        for (int y = std::max(0, b[1] - 1); y <= std::min(g.res - 1, b[1] + 1); y++)
            for (int x = std::max(0, b[0] - 1); x <= std::min(g.res - 1, b[0] + 1); x++) {
                const size_t bin = ((size_t)z * g.res + y) * g.res + x;
                for (uint32_t k = g.start[bin]; k < g.start[bin + 1]; k++) {
                    const int e = (int)g.items[k];
                    if (best >= 0 && e >= best) continue;
                    if (encloses(m, e, p)) best = e;
                }
            }
    return best >= 0 ? best + 1 : 0;
}

}  // namespace mmcgb

// Output stage of a simulation: element -> node scatter of the raw element
// deposits (src/mmc_cu_host.cu:916-976), the surface nodal-volume correction
// (src/mmc_mesh.c:1344-1386) and the fluence normalization
// (src/mmc_mesh.c:2154-2279), for one pattern's deposits (patterns sharing
// photons run it once per pattern with that pattern's energies, api.cpp).
#include <cmath>
#include <cstring>
#include <vector>

#include "mesh.h"
#include "output_dev.h"

namespace mmcgb {

namespace {

// Effective reflection coefficient of a diffusive medium against n_out,
// integrated over 1000 angular steps (src/mmc_mesh.c:2305-2334).
double effective_reflection(double n_in, double n_out) {
    const double oc = std::asin(1.0 / n_in);
    const double count = 1000.0;
    const double ostep = M_PI / (2.0 * count);
    double r_phi = 0.0, r_j = 0.0;
    for (int i = 0; i < (int)count; i++) {
        const double o = i * ostep, coso = std::cos(o);
        double r_fres;
        if (o < oc) {
            double cosop = n_in * std::sin(o);
            cosop = std::sqrt(1. - cosop * cosop);
            double t = (n_in * cosop - n_out * coso) / (n_in * cosop + n_out * coso);
            r_fres = 0.5 * t * t;
            t = (n_in * coso - n_out * cosop) / (n_in * coso + n_out * cosop);
            r_fres += 0.5 * t * t;
        } else {
            r_fres = 1.f;
        }
        r_phi += 2.0 * std::sin(o) * coso * r_fres;
        r_j += 3.0 * std::sin(o) * coso * coso * r_fres;
    }
    r_phi *= ostep;
    r_j *= ostep;
    return (r_phi + r_j) / (2.0 - r_phi + r_j);
}

}  // namespace

std::vector<float> surface_fixed_nvol(const HostMesh& m, const mmcgb_config& cfg) {
    const int nn = m.nn, ne = m.ne;
    const int prop = cfg.nmedia - 1;
    const float* med = cfg.media;
    std::vector<float> nvol(m.nvol);
    if (cfg.isnormalized == 1 && cfg.basisorder) {
        std::vector<float> Reff(prop + 1, 0.f);
        if (cfg.isreflect) {
            for (int i = 1; i <= prop; i++) {
                for (int j = 1; j < i; j++)
                    if (med[4 * j + 3] == med[4 * i + 3]) {
                        Reff[i] = Reff[j];
                        break;
                    }
                if (Reff[i] == 0.f) Reff[i] = (float)effective_reflection(med[4 * i + 3], med[3]);
            }
        }
        for (int i = 0; i < ne; i++)
            for (int j = 0; j < 4; j++)
                if (m.facenb[4 * (size_t)i + j] < 0) {
                    for (int k = 0; k < 3; k++) {
                        const int nid = m.elem[4 * (size_t)i + kOut[kIFaceOrder[j]][k]] - 1;
                        if (nvol[nid] > 0.f && m.label[i] >= 0) nvol[nid] *= -(2.f / (1.0 + Reff[m.label[i]]));
                    }
                }
        for (int i = 0; i < nn; i++)
            if (nvol[i] < 0.f) nvol[i] = -nvol[i];
    }
    return nvol;
}

void scatter_output(const HostMesh& m, const mmcgb_config& cfg, int G, const double* raw, double* field) {
    const int nn = m.nn, ne = m.ne;
    const size_t total = (size_t)(cfg.basisorder ? nn : ne) * G;
    if (!cfg.basisorder) {
        if (field != raw) std::memcpy(field, raw, sizeof(double) * total);
        return;
    }
    std::memset(field, 0, sizeof(double) * total);
    for (int i = 0; i < G; i++) {
        const double* r = raw + (size_t)i * ne;
        double* f = field + (size_t)i * nn;
        for (int j = 0; j < ne; j++) {
            const double ww = r[j] * 0.25;
            const int* e = &m.elem[4 * (size_t)j];
            f[e[0] - 1] += ww;
            f[e[1] - 1] += ww;
            f[e[2] - 1] += ww;
            f[e[3] - 1] += ww;
        }
    }
}

double normalize_in_place(const HostMesh& m, const mmcgb_config& cfg, int G, double energytot, double energyesc,
                          double* field) {
    const int nn = m.nn, ne = m.ne;
    const float* med = cfg.media;
    const int datalen = cfg.basisorder ? nn : ne;
    const size_t total = (size_t)datalen * G;
    double normalizor = 1.0;
    if (!cfg.isnormalized) return normalizor;
    const std::vector<float> nvol = surface_fixed_nvol(m, cfg);
    const float Etotal = (float)energytot;
    const float Eabsorb = (float)(energytot - energyesc);
    const bool replay = cfg.replayseed != nullptr;
    if (replay && (cfg.outputtype == OT_JACOBIAN || cfg.outputtype == OT_WL || cfg.outputtype == OT_WP ||
                   cfg.outputtype == OT_WN)) {
        normalizor = 1.f / (1e-4f * (float)cfg.nphoton);
        if (cfg.outputtype != OT_JACOBIAN) normalizor = 1.f / Etotal;
    } else if (cfg.outputtype == OT_ENERGY) {
        normalizor = 1.f / Etotal;
    } else {
        double energydeposit = 0.0;
        if (cfg.basisorder) {
            for (int i = 0; i < G; i++)
                for (int j = 0; j < datalen; j++)
                    if (nvol[j] > 0.f) field[(size_t)i * datalen + j] /= nvol[j];
            for (int i = 0; i < ne; i++) {
                double energyelem = 0.0;
                const int* e = &m.elem[4 * (size_t)i];
                for (int j = 0; j < G; j++)
                    for (int k = 0; k < 4; k++) energyelem += field[(size_t)j * nn + e[k] - 1];
                energydeposit += energyelem * m.evol[i] * med[4 * m.label[i]];
            }
            normalizor = Eabsorb / (Etotal * energydeposit * 0.25f);
        } else {
            for (int i = 0; i < datalen; i++)
                for (int j = 0; j < G; j++) energydeposit += field[(size_t)j * datalen + i];
            for (int i = 0; i < datalen; i++) {
                const double energyelem = m.evol[i] * med[4 * m.label[i]];
                for (int j = 0; j < G; j++) field[(size_t)j * datalen + i] /= energyelem;
            }
            normalizor = Eabsorb / (Etotal * energydeposit);
        }
        if (cfg.outputtype == OT_FLUX) normalizor /= cfg.tstep;
    }
    for (size_t i = 0; i < total; i++) field[i] *= normalizor;
    return normalizor;
}

double normalize_output(const HostMesh& m, const mmcgb_config& cfg, int G, const double* raw,
                        double energytot, double energyesc, double* field) {
    scatter_output(m, cfg, G, raw, field);
    return normalize_in_place(m, cfg, G, energytot, energyesc, field);
}

double grid_normalizer(const mmcgb_config& cfg, double energytot) {
    if (!cfg.isnormalized) return 1.0;
    const float Et = (float)energytot;
    if (cfg.outputtype == OT_ENERGY) return 1.f / Et;  // src/mmc_mesh.c:2185-2192
    double norm = 1.0 / (Et * cfg.unitinmm * cfg.unitinmm * cfg.unitinmm);  // src/mmc_mesh.c:2204-2206
    if (cfg.outputtype == OT_FLUX) norm /= cfg.tstep;
    return norm;
}

}  // namespace mmcgb

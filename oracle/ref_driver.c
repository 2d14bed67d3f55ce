/* Test-infrastructure driver around the reference MMC CPU engine.  It runs the
 * reference's own lifecycle (mmc_init_from_cmd -> mmc_prep -> mmc_run_mp ->
 * mmc_cleanup, src/mmc_host.h:49-54) with the usual command line and exposes
 * intermediate results the reference binary keeps in memory:
 *
 *   MMCGB_MESH_OUT=f   after mmc_prep: int32 nn, ne, nf; int32 elem[ne*4]
 *                      (orientation-fixed); int32 facenb[ne*4] (exterior faces
 *                      numbered); float evol[ne]; float nvol[nn] (after the
 *                      surface fix); float normals[ne*16] (tracer->n)
 *   MMCGB_DETP_OUT=f   after the run: int32 count, int32 cols, float rows --
 *                      the detected-photon table in cfg.exportdetected (the
 *                      reference's standalone .mch/.jdt writers take the column
 *                      count from cfg.his, which the CPU path leaves at 0)
 *   MMCGB_SEED_OUT=f   after the run (with -q 1): int32 count, int32 seedbyte,
 *                      then count*seedbyte bytes -- the RNG states the detected
 *                      photons started from, cfg.exportseed (src/mmc_host.c:405-409),
 *                      which replay (-E file.mch) reads back
 *   MMCGB_NORM_IN=f    instead of simulating: read double Eabsorb, double
 *   MMCGB_NORM_OUT=g   Etotal, double raw[maxgate*ne] element deposits; scatter
 *                      them to the nodes when basisorder=1 as the CUDA host does
 *                      (src/mmc_cu_host.cu:916-976, restated below), normalize
 *                      with the reference's mesh_normalize and write
 *                      double weight[maxgate*datalen] and double normalizer.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "mmc_host.h"

static void dump_mesh(const char* path, tetmesh* mesh, raytracer* tracer) {
    FILE* f = fopen(path, "wb");
    if (!f) exit(3);
    fwrite(&mesh->nn, sizeof(int), 1, f);
    fwrite(&mesh->ne, sizeof(int), 1, f);
    fwrite(&mesh->nf, sizeof(int), 1, f);
    fwrite(mesh->elem, sizeof(int), (size_t)mesh->ne * 4, f);
    fwrite(mesh->facenb, sizeof(int), (size_t)mesh->ne * 4, f);
    fwrite(mesh->evol, sizeof(float), (size_t)mesh->ne, f);
    fwrite(mesh->nvol, sizeof(float), (size_t)mesh->nn, f);
    fwrite(tracer->n, sizeof(float), (size_t)mesh->ne * 16, f);
    fclose(f);
}

static int normalize_only(mcconfig* cfg, tetmesh* mesh, const char* in, const char* out) {
    FILE* f = fopen(in, "rb");
    if (!f) return 3;
    double eabs, etot;
    size_t flen = (size_t)mesh->ne * cfg->maxgate;
    double* raw = (double*)malloc(sizeof(double) * flen);
    if (fread(&eabs, sizeof(double), 1, f) != 1 || fread(&etot, sizeof(double), 1, f) != 1 ||
        fread(raw, sizeof(double), flen, f) != flen) {
        fclose(f);
        return 4;
    }
    fclose(f);
    int datalen = cfg->basisorder ? mesh->nn : mesh->ne;
    memset(mesh->weight, 0, sizeof(double) * (size_t)datalen * cfg->maxgate);
    for (int i = 0; i < cfg->maxgate; i++)
        for (int j = 0; j < mesh->ne; j++) {
            if (!cfg->basisorder) {
                mesh->weight[(size_t)i * mesh->ne + j] += (float)raw[(size_t)i * mesh->ne + j];
            } else {
                float ww = (float)raw[(size_t)i * mesh->ne + j] * 0.25f;
                for (int k = 0; k < 4; k++) mesh->weight[(size_t)i * mesh->nn + mesh->elem[j * 4 + k] - 1] += ww;
            }
        }
    double norm = mesh_normalize(mesh, cfg, (float)eabs, (float)etot, 0);
    f = fopen(out, "wb");
    if (!f) return 3;
    fwrite(mesh->weight, sizeof(double), (size_t)datalen * cfg->maxgate, f);
    fwrite(&norm, sizeof(double), 1, f);
    fclose(f);
    free(raw);
    return 0;
}

int main(int argc, char** argv) {
    mcconfig cfg;
    tetmesh mesh;
    raytracer tracer;
    const char* detp_out = getenv("MMCGB_DETP_OUT");
    const char* seed_out = getenv("MMCGB_SEED_OUT");
    const char* mesh_out = getenv("MMCGB_MESH_OUT");
    const char* norm_in = getenv("MMCGB_NORM_IN");
    const char* norm_out = getenv("MMCGB_NORM_OUT");
    mmc_init_from_cmd(&cfg, &mesh, &tracer, argc, argv);
    mmc_prep(&cfg, &mesh, &tracer);
    if (mesh_out) dump_mesh(mesh_out, &mesh, &tracer);
    if (norm_in && norm_out) {
        int rc = normalize_only(&cfg, &mesh, norm_in, norm_out);
        mmc_cleanup(&cfg, &mesh, &tracer);
        return rc;
    }
    mmc_run_mp(&cfg, &mesh, &tracer);
    if (detp_out && cfg.issavedet) {
        int cols = (2 + (cfg.ismomentum > 0)) * mesh.prop + (cfg.issaveexit > 0) * 6 + 2;
        int count = (int)cfg.detectedcount;
        FILE* f = fopen(detp_out, "wb");
        if (!f) return 3;
        fwrite(&count, sizeof(int), 1, f);
        fwrite(&cols, sizeof(int), 1, f);
        if (count > 0 && cfg.exportdetected) fwrite(cfg.exportdetected, sizeof(float), (size_t)count * cols, f);
        fclose(f);
    }
    if (seed_out && cfg.issavedet && cfg.issaveseed) {
        int count = (int)cfg.detectedcount;
        int seedbyte = (int)(sizeof(RandType) * RAND_BUF_LEN);
        FILE* f = fopen(seed_out, "wb");
        if (!f) return 3;
        fwrite(&count, sizeof(int), 1, f);
        fwrite(&seedbyte, sizeof(int), 1, f);
        if (count > 0 && cfg.exportseed) fwrite(cfg.exportseed, 1, (size_t)count * seedbyte, f);
        fclose(f);
    }
    mmc_cleanup(&cfg, &mesh, &tracer);
    return 0;
}

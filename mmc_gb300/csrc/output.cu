// Output stage on the GPU: the same arithmetic as normalize_output()
// (output.cpp) -- element->node scatter (src/mmc_cu_host.cu:916-976), surface
// nodal-volume fix applied on the host to the nodal volumes, normalization
// (src/mmc_mesh.c:2154-2279) -- run on the device buffers so that only the
// final field crosses to the host.  Sums are accumulated with float64
// atomics, so they agree with the host version to summation order.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "engine.h"
#include "mesh.h"
#include "output_dev.h"

namespace mmcgb {

namespace {

__device__ __forceinline__ double raw_at(const double* f64, const float* a, const float* b, size_t i) {
    return f64 ? f64[i] : (double)a[i] + (double)b[i];
}

__device__ __forceinline__ void block_add(double v, double* out) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
    if ((threadIdx.x & 31) == 0 && v != 0.0) atomicAdd(out, v);
}

__global__ void k_sum(const double* f64, const float* a, const float* b, size_t n, double* out) {
    double v = 0.0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        v += raw_at(f64, a, b, i);
    block_add(v, out);
}

// element output: out = raw / (evol * mua) * scale  (two roundings, as the host)
__global__ void k_elem(const double* f64, const float* a, const float* b, const float* evol, const int* label,
                       const float4* media, int ne, size_t n, int divide, double scale, double* out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int e = (int)(i % (size_t)ne);
        double v = raw_at(f64, a, b, i);
        if (divide) v /= (double)(evol[e] * media[label[e]].x);
        out[i] = v * scale;
    }
}

__global__ void k_node_scatter(const double* f64, const float* a, const float* b, const int4* elem, int ne, int nn,
                               size_t n, double* node) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const size_t g = i / (size_t)ne;
        const int e = (int)(i % (size_t)ne);
        const double ww = raw_at(f64, a, b, i) * 0.25;
        if (ww == 0.0) continue;
        const int4 el = elem[e];
        double* row = node + g * (size_t)nn;
        atomicAdd(row + el.x - 1, ww);
        atomicAdd(row + el.y - 1, ww);
        atomicAdd(row + el.z - 1, ww);
        atomicAdd(row + el.w - 1, ww);
    }
}

__global__ void k_node_div(double* node, const float* nvol, int nn, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float v = nvol[i % (size_t)nn];
        if (v > 0.f) node[i] /= v;
    }
}

__global__ void k_node_energy(const double* node, const int4* elem, const float* evol, const int* label,
                              const float4* media, int ne, int nn, int G, double* out) {
    double acc = 0.0;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x) {
        const int4 el = elem[e];
        double s = 0.0;
        for (int g = 0; g < G; g++) {
            const double* row = node + (size_t)g * nn;
            s += row[el.x - 1];
            s += row[el.y - 1];
            s += row[el.z - 1];
            s += row[el.w - 1];
        }
        acc += s * evol[e] * media[label[e]].x;
    }
    block_add(acc, out);
}

__global__ void k_scale(double* x, size_t n, double s) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        x[i] *= s;
}

int grid_for(size_t n) {
    size_t b = (n + 255) / 256;
    return (int)(b < 4096 ? (b ? b : 1) : 4096);
}

}  // namespace

cudaError_t device_output(const DeviceOutputArgs& A, cudaStream_t st, double* normalizer) {
    const HostMesh& m = *A.host;
    const mmcgb_config& cfg = *A.cfg;
    const int G = A.maxgate, ne = m.ne, nn = m.nn;
    const size_t nraw = (size_t)ne * G;
    const size_t nout = (size_t)(cfg.basisorder ? nn : ne) * G;
    cudaError_t e;
    if (A.gridlen) {
        // dual-grid output: one scale factor, src/mmc_mesh.c:2204-2206 (no volume division)
        const size_t n = A.gridlen * G;
        double norm = 1.0;
        const float Et = (float)A.energytot;
        if (cfg.isnormalized) {
            if (cfg.outputtype == OT_ENERGY) {
                norm = 1.f / Et;
            } else {
                norm = 1.0 / (Et * cfg.unitinmm * cfg.unitinmm * cfg.unitinmm);
                if (cfg.outputtype == OT_FLUX) norm /= cfg.tstep;
            }
        }
        k_elem<<<grid_for(n), 256, 0, st>>>(A.f64, A.f32a, A.f32b, A.evol, A.label, A.media, ne, n, 0, norm, A.out);
        *normalizer = norm;
        return cudaGetLastError();
    }
    double* scratch = nullptr;  // [0] sum
    if ((e = cudaMallocAsync((void**)&scratch, sizeof(double) * 2, st)) != cudaSuccess) return e;
    cudaMemsetAsync(scratch, 0, sizeof(double) * 2, st);
    double norm = 1.0;
    const bool replay = cfg.replayseed != nullptr;
    const int ot = cfg.outputtype;
    const bool fluence_norm = cfg.isnormalized && !(replay && (ot == OT_JACOBIAN || ot == OT_WL || ot == OT_WP || ot == OT_WN)) &&
                              ot != OT_ENERGY;
    const float Etotal = (float)A.energytot;
    const float Eabsorb = (float)(A.energytot - A.energyesc);
    if (cfg.isnormalized && !fluence_norm) {
        if (replay && ot == OT_JACOBIAN) norm = 1.f / (1e-4f * (float)cfg.nphoton);
        else norm = 1.f / Etotal;
    }
    if (!cfg.basisorder) {
        if (fluence_norm) {
            k_sum<<<grid_for(nraw), 256, 0, st>>>(A.f64, A.f32a, A.f32b, nraw, scratch);
            double dep = 0.0;
            if ((e = cudaMemcpyAsync(&dep, scratch, sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
            if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
            norm = Eabsorb / (Etotal * dep);
            if (ot == OT_FLUX) norm /= cfg.tstep;
        }
        k_elem<<<grid_for(nraw), 256, 0, st>>>(A.f64, A.f32a, A.f32b, A.evol, A.label, A.media, ne, nraw,
                                               fluence_norm ? 1 : 0, cfg.isnormalized ? norm : 1.0, A.out);
    } else {
        cudaMemsetAsync(A.out, 0, sizeof(double) * nout, st);
        k_node_scatter<<<grid_for(nraw), 256, 0, st>>>(A.f64, A.f32a, A.f32b, A.elem, ne, nn, nraw, A.out);
        if (fluence_norm) {
            k_node_div<<<grid_for(nout), 256, 0, st>>>(A.out, A.nvol, nn, nout);
            k_node_energy<<<grid_for((size_t)ne), 256, 0, st>>>(A.out, A.elem, A.evol, A.label, A.media, ne, nn, G,
                                                               scratch);
            double dep = 0.0;
            if ((e = cudaMemcpyAsync(&dep, scratch, sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
            if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
            norm = Eabsorb / (Etotal * dep * 0.25f);
            if (ot == OT_FLUX) norm /= cfg.tstep;
        }
        if (cfg.isnormalized) k_scale<<<grid_for(nout), 256, 0, st>>>(A.out, nout, norm);
    }
    cudaFreeAsync(scratch, st);
    *normalizer = cfg.isnormalized ? norm : 1.0;
    return cudaGetLastError();
}

}  // namespace mmcgb

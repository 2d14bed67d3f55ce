// Diagnostics of the GPU the engine runs on (no counterpart in the reference).
//
// mmcgb_l2_read_bandwidth: the rate at which this GPU's L2 serves 16-byte
// reads of data it already holds -- the level the engine's dependent record
// gathers and fluence reductions are served from, so the engine's L2 traffic
// can be stated as a fraction of it beside the HBM roofline.  A buffer well
// below the L2 capacity is read once to make it resident, then swept `reps`
// more times with L1-bypassing loads (ld.global.cg), four independent loads
// in flight per thread; every SM runs 8 blocks of 256 threads.
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/mmcgb.h"
#include "engine.h"

namespace {

__global__ void __launch_bounds__(256) k_l2_sweep(const uint4* __restrict__ buf, size_t n16, int reps,
                                                  unsigned* sink) {
    unsigned acc = 0u;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    for (int r = 0; r < reps; r++) {
        for (size_t i = t; i < n16; i += 4 * stride) {
            uint4 v0 = __ldcg(buf + i);
            uint4 v1 = (i + stride < n16) ? __ldcg(buf + i + stride) : make_uint4(0u, 0u, 0u, 0u);
            uint4 v2 = (i + 2 * stride < n16) ? __ldcg(buf + i + 2 * stride) : make_uint4(0u, 0u, 0u, 0u);
            uint4 v3 = (i + 3 * stride < n16) ? __ldcg(buf + i + 3 * stride) : make_uint4(0u, 0u, 0u, 0u);
            acc ^= (v0.x ^ v0.y ^ v0.z ^ v0.w) ^ (v1.x ^ v1.y ^ v1.z ^ v1.w) ^ (v2.x ^ v2.y ^ v2.z ^ v2.w) ^
                   (v3.x ^ v3.y ^ v3.z ^ v3.w);
        }
    }
    if (acc == 0x9e3779b9u) atomicAdd(sink, 1u);  // a data-dependent store keeps every load
}

int fail(int code, const std::string& msg) {
    mmcgb::set_last_error(msg);
    return code;
}

}  // namespace

extern "C" int32_t mmcgb_l2_read_bandwidth(int32_t device, uint64_t bytes, int32_t reps, double* gbs) {
    if (!gbs || reps < 1 || bytes < (1u << 20) || (bytes & 15u)) return fail(MMCGB_E_ARG, "need bytes >= 1 MiB, a multiple of 16, and reps >= 1");
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return fail(MMCGB_E_CUDA, cudaGetErrorString(e));
    int sms = 0, l2 = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, device);
    if ((uint64_t)l2 > 0 && bytes > (uint64_t)l2 / 2) return fail(MMCGB_E_ARG, "the buffer must fit in half of the L2");
    uint4* buf = nullptr;
    unsigned* sink = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    float ms = 0.f;
    const size_t n16 = bytes / 16;
    const int blocks = (sms > 0 ? sms : 1) * 8;
    if ((e = cudaMalloc(&buf, bytes)) != cudaSuccess || (e = cudaMalloc(&sink, sizeof(unsigned))) != cudaSuccess ||
        (e = cudaMemset(buf, 0x5a, bytes)) != cudaSuccess || (e = cudaMemset(sink, 0, sizeof(unsigned))) != cudaSuccess ||
        (e = cudaEventCreate(&a)) != cudaSuccess || (e = cudaEventCreate(&b)) != cudaSuccess) {
        cudaFree(buf);
        cudaFree(sink);
        return fail(MMCGB_E_CUDA, cudaGetErrorString(e));
    }
    k_l2_sweep<<<blocks, 256>>>(buf, n16, 1, sink);  // makes the buffer L2-resident
    cudaEventRecord(a);
    k_l2_sweep<<<blocks, 256>>>(buf, n16, reps, sink);
    cudaEventRecord(b);
    e = cudaEventSynchronize(b);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(buf);
    cudaFree(sink);
    if (e != cudaSuccess) return fail(MMCGB_E_CUDA, cudaGetErrorString(e));
    *gbs = (double)bytes * reps / (ms * 1e-3) / 1e9;
    return MMCGB_OK;
}

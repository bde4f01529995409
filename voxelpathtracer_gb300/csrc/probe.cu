// Roof measurement for the benchmark: the read bandwidth of a buffer that
// stays in L2. The trace kernels gather the distance field from an L2-resident
// volume, so their memory roof is this number, not the HBM copy bandwidth.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "vpt.h"

namespace {

// Every thread reads 128-bit words with a grid stride; the XOR of what it read
// is stored per block so the loads cannot be dropped.
__global__ void __launch_bounds__(512) k_l2_read(const uint4* __restrict__ p, size_t n, unsigned* sink) {
    unsigned acc = 0;
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        const uint4 v = __ldcg(p + k);   // cached in L2 only, as the gathers of other SMs' rays are
        acc ^= v.x ^ v.y ^ v.z ^ v.w;
    }
    acc = __reduce_xor_sync(0xffffffffu, acc);
    if ((threadIdx.x & 31) == 0 && acc == 0x9e3779b9u) atomicAdd(sink, 1u);
}

}  // namespace

extern "C" vpt_status vpt_measure_l2_read(int32_t device, uint64_t bytes, int32_t reps, float* gbs) {
    if (!gbs || bytes < (1u << 20) || bytes > ((uint64_t)1 << 32) || reps < 1 || reps > 1000)
        return VPT_ERR_INVALID_ARG;
    *gbs = 0.0f;
    if (cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        return VPT_ERR_NO_DEVICE;
    }
    const size_t n = (size_t)(bytes / 16);
    uint4* buf = nullptr;
    unsigned* sink = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    vpt_status st = VPT_OK;
    int sms = 0;
    std::vector<float> ms;
    if (cudaMalloc(&buf, n * 16) != cudaSuccess || cudaMalloc(&sink, 4) != cudaSuccess) {
        st = VPT_ERR_OOM;
        goto done;
    }
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaMemsetAsync(buf, 1, n * 16, s) != cudaSuccess) {
        st = VPT_ERR_CUDA;
        goto done;
    }
    for (int r = 0; r < reps + 2 && st == VPT_OK; r++) {   // two warm-up reads bring the buffer into L2
        cudaEventRecord(e0, s);
        k_l2_read<<<sms * 4, 512, 0, s>>>(buf, n, sink);
        cudaEventRecord(e1, s);
        if (cudaEventSynchronize(e1) != cudaSuccess) {
            st = VPT_ERR_CUDA;
            break;
        }
        float m = 0.0f;
        cudaEventElapsedTime(&m, e0, e1);
        if (r >= 2) ms.push_back(m);
    }
    if (st == VPT_OK) {
        std::sort(ms.begin(), ms.end());
        *gbs = (float)((double)n * 16.0 / (ms[ms.size() / 2] * 1e-3) / 1e9);
    }
done:
    cudaGetLastError();
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    if (buf) cudaFree(buf);
    if (sink) cudaFree(sink);
    return st;
}

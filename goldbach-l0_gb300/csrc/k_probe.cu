// k_probe.cu -- measurement only (libgbc_probe.so, include/gbc_probe.h): the
// shared-memory atomic roof the sieve stages are measured against,
// conflict-free 32-bit atomicAnd throughput of this GPU.
//
// One CTA of 1024 threads per SM, the tile sieve's shape; each thread clears
// bits of its own word column (warp w, lane l, round i: word
// (32 w + l + 1024 i) mod 16384 of a 64 KB tile), so every warp instruction
// touches 32 different banks. The result is atomics per second over the
// event-timed launch and atomics per SM clock (clock64 of CTA 0).
#include <cuda_runtime.h>

#include "../../include/gbc.h"
#include "../../include/gbc_probe.h"

namespace {

constexpr uint32_t kProbeWords = 32768;
constexpr int kProbeThreads = 1024;

__global__ void __launch_bounds__(kProbeThreads, 1) k_smem_atomic_probe(uint32_t iters, uint32_t *sink,
                                                                        long long *cycles)
{
    extern __shared__ uint32_t s[];
    for (uint32_t i = threadIdx.x; i < kProbeWords / 2; i += blockDim.x) s[i] = ~0u;
    __syncthreads();
    const long long t0 = clock64();
    uint32_t w = threadIdx.x;
    const uint32_t bit = ~(1u << (threadIdx.x & 31));
#pragma unroll 8
    for (uint32_t i = 0; i < iters; ++i) {
        atomicAnd(&s[w], bit);
        w = (w + kProbeThreads) & (kProbeWords / 2 - 1);
    }
    __syncthreads();
    const long long t1 = clock64();
    if (threadIdx.x == 0) {
        sink[blockIdx.x] = s[blockIdx.x & (kProbeWords / 2 - 1)];
        if (blockIdx.x == 0) *cycles = t1 - t0;
    }
}

// the probe on one device; the caller's current device is restored by
// gbc_smem_atomic_peak
int probe(int device, double *atomics_per_s, double *per_clock_per_sm)
{
    if (cudaSetDevice(device) != cudaSuccess) return GBC_E_CUDA;
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return GBC_E_CUDA;
    const int sms = prop.multiProcessorCount;
    const int smem = int(kProbeWords / 2 * 4);
    if (cudaFuncSetAttribute(k_smem_atomic_probe, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
        return GBC_E_CUDA;
    uint32_t *sink = nullptr;
    long long *cyc = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = GBC_OK;
    if (cudaMalloc(&sink, size_t(sms) * 4) != cudaSuccess || cudaMalloc(&cyc, sizeof(long long)) != cudaSuccess ||
        cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        rc = GBC_E_CUDA;
    const uint32_t iters = 1u << 14;
    float ms = 0;
    long long cycles = 0;
    if (!rc) {
        k_smem_atomic_probe<<<sms, kProbeThreads, smem>>>(64, sink, cyc);  // warm-up
        if (cudaEventRecord(e0) != cudaSuccess) rc = GBC_E_CUDA;
    }
    if (!rc) {
        k_smem_atomic_probe<<<sms, kProbeThreads, smem>>>(iters, sink, cyc);
        if (cudaEventRecord(e1) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
            cudaGetLastError() != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess ||
            cudaMemcpy(&cycles, cyc, sizeof cycles, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = GBC_E_CUDA;
    }
    const double total = double(iters) * kProbeThreads * sms;
    if (!rc && ms > 0 && cycles > 0) {
        if (atomics_per_s) *atomics_per_s = total / (ms * 1e-3);
        if (per_clock_per_sm) *per_clock_per_sm = double(iters) * kProbeThreads / double(cycles);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(sink);
    cudaFree(cyc);
    return rc;
}

}  // namespace

extern "C" int gbc_smem_atomic_peak(int device, double *atomics_per_s, double *per_clock_per_sm)
{
    int prev = 0;
    if (cudaGetDevice(&prev) != cudaSuccess) return GBC_E_CUDA;
    const int rc = probe(device, atomics_per_s, per_clock_per_sm);
    if (cudaSetDevice(prev) != cudaSuccess) return GBC_E_CUDA;
    return rc;
}

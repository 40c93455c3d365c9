// pq_peak.cu -- measured issue rates of the pipes the enumeration kernel uses.
//
// The enumeration's arithmetic is FP32 fused multiply-add work (the reference form of the same
// sum is integer logic / popcount work), for which no vendor peak is published per chip
// configuration; these kernels measure the rates on the device: eight independent dependency
// chains per thread of one instruction type (lop3.b32, popc.b32, fma.rn.f32) over a persistent
// grid, timed with CUDA events.  Every thread writes one word to
// `out` (grid * block words) so the chains are not removed.
#include <cuda_runtime.h>

#include <cstdint>

#include "polyq_gb300.h"

namespace pq {

__global__ void __launch_bounds__(256) peak_lop3(uint32_t *out, int iters) {
    uint32_t a0 = threadIdx.x, a1 = a0 * 3u + 1u, a2 = a0 * 5u + 2u, a3 = a0 * 7u + 3u;
    uint32_t a4 = a0 * 11u + 4u, a5 = a0 * 13u + 5u, a6 = a0 * 17u + 6u, a7 = a0 * 19u + 7u;
    const uint32_t b = blockIdx.x * 0x9E3779B9u, c = (blockIdx.x + 1u) * 0x85EBCA6Bu;
    for (int i = 0; i < iters; i++) {
#define PQ_LOP(x) asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(x) : "r"(b), "r"(c))
        PQ_LOP(a0); PQ_LOP(a1); PQ_LOP(a2); PQ_LOP(a3); PQ_LOP(a4); PQ_LOP(a5); PQ_LOP(a6); PQ_LOP(a7);
#undef PQ_LOP
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = a0 ^ a1 ^ a2 ^ a3 ^ a4 ^ a5 ^ a6 ^ a7;
}

__global__ void __launch_bounds__(256) peak_popc(uint32_t *out, int iters) {
    uint32_t a0 = threadIdx.x, a1 = a0 * 3u + 1u, a2 = a0 * 5u + 2u, a3 = a0 * 7u + 3u;
    uint32_t a4 = a0 * 11u + 4u, a5 = a0 * 13u + 5u, a6 = a0 * 17u + 6u, a7 = a0 * 19u + 7u;
    const uint32_t c = blockIdx.x * 0x9E3779B9u;
    for (int i = 0; i < iters; i++) {
#define PQ_POPC(x) asm volatile("{ .reg .b32 t; popc.b32 t, %0; add.u32 %0, t, %1; }" : "+r"(x) : "r"(c))
        PQ_POPC(a0); PQ_POPC(a1); PQ_POPC(a2); PQ_POPC(a3); PQ_POPC(a4); PQ_POPC(a5); PQ_POPC(a6); PQ_POPC(a7);
#undef PQ_POPC
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = a0 ^ a1 ^ a2 ^ a3 ^ a4 ^ a5 ^ a6 ^ a7;
}

__global__ void __launch_bounds__(256) peak_ffma(uint32_t *out, int iters) {
    float a0 = threadIdx.x * 1e-3f, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f;
    float a4 = a0 + 4.f, a5 = a0 + 5.f, a6 = a0 + 6.f, a7 = a0 + 7.f;
    const float c = 1e-7f * (float)(blockIdx.x + 1), s = 0.999f;
    for (int i = 0; i < iters; i++) {
#define PQ_FADD(x) asm volatile("fma.rn.f32 %0, %0, %1, %2;" : "+f"(x) : "f"(s), "f"(c))
        PQ_FADD(a0); PQ_FADD(a1); PQ_FADD(a2); PQ_FADD(a3); PQ_FADD(a4); PQ_FADD(a5); PQ_FADD(a6); PQ_FADD(a7);
#undef PQ_FADD
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = __float_as_uint(a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7);
}

// Paired FP32 FMA (fma.rn.f32x2 on a 64-bit register pair: two FP32 FMA per instruction), the
// form the enumeration's even quarter-turn steps issue.
__global__ void __launch_bounds__(256) peak_ffma2(uint32_t *out, int iters) {
    uint64_t a[8];
    for (int k = 0; k < 8; k++) {
        const float lo = threadIdx.x * 1e-3f + (float)k, hi = lo + 0.5f;
        asm("mov.b64 %0, {%1, %2};" : "=l"(a[k]) : "f"(lo), "f"(hi));
    }
    uint64_t s2, c2;
    {
        const float s = 0.999f, c = 1e-7f * (float)(blockIdx.x + 1);
        asm("mov.b64 %0, {%1, %1};" : "=l"(s2) : "f"(s));
        asm("mov.b64 %0, {%1, %1};" : "=l"(c2) : "f"(c));
    }
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) asm volatile("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(a[k]) : "l"(s2), "l"(c2));
    }
    uint64_t x = 0;
    for (int k = 0; k < 8; k++) x ^= a[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = (uint32_t)x ^ (uint32_t)(x >> 32);
}

}  // namespace pq

using namespace pq;

extern "C" PQ_API pq_status pq_measure_fma2_rate(double *out) {
    // FP32 FMA operations per second issued as fma.rn.f32x2 (two per instruction)
    if (!out) return PQ_ERR_INVALID_ARG;
    int dev = 0;
    cudaDeviceProp p;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&p, dev) != cudaSuccess) return PQ_ERR_NO_DEVICE;
    const int block = 256, blocks_per_sm = 8, iters = 4096;
    const int grid = p.multiProcessorCount * blocks_per_sm;
    uint32_t *buf = nullptr;
    if (cudaMalloc(&buf, (size_t)grid * block * sizeof(uint32_t)) != cudaSuccess) return PQ_ERR_OUT_OF_MEMORY;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    pq_status st = PQ_OK;
    peak_ffma2<<<grid, block>>>(buf, iters);  // warm-up
    cudaEventRecord(e0);
    for (int r = 0; r < 5; r++) peak_ffma2<<<grid, block>>>(buf, iters);
    cudaEventRecord(e1);
    if (cudaEventSynchronize(e1) != cudaSuccess) st = PQ_ERR_DEVICE;
    float ms = 0.f;
    if (st == PQ_OK) cudaEventElapsedTime(&ms, e0, e1);
    *out = ms > 0.f ? 5.0 * (double)grid * block * iters * 8.0 * 2.0 / (ms * 1e-3) : 0.0;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    return st;
}

extern "C" PQ_API pq_status pq_measure_peaks(double out[4]) {
    // out: lop3.b32 ops/s, popc.b32 ops/s, fma.f32 ops/s, SM count
    if (!out) return PQ_ERR_INVALID_ARG;
    int dev = 0;
    cudaDeviceProp p;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&p, dev) != cudaSuccess) return PQ_ERR_NO_DEVICE;
    const int block = 256, blocks_per_sm = 8, iters = 4096;
    const int grid = p.multiProcessorCount * blocks_per_sm;
    uint32_t *buf = nullptr;
    if (cudaMalloc(&buf, (size_t)grid * block * sizeof(uint32_t)) != cudaSuccess) return PQ_ERR_OUT_OF_MEMORY;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    void (*kern[3])(uint32_t *, int) = {peak_lop3, peak_popc, peak_ffma};
    pq_status st = PQ_OK;
    for (int k = 0; k < 3 && st == PQ_OK; k++) {
        kern[k]<<<grid, block>>>(buf, iters);  // warm-up
        cudaEventRecord(e0);
        for (int r = 0; r < 5; r++) kern[k]<<<grid, block>>>(buf, iters);
        cudaEventRecord(e1);
        if (cudaEventSynchronize(e1) != cudaSuccess) { st = PQ_ERR_DEVICE; break; }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double ops = 5.0 * (double)grid * block * iters * 8.0;
        out[k] = ms > 0.f ? ops / (ms * 1e-3) : 0.0;
    }
    out[3] = (double)p.multiProcessorCount;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    return st;
}

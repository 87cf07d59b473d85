// lp.cu -- learned target function (learned p-hat): a small MLP on the fifth-generation
// tensor cores.  This file holds the tcgen05 building blocks and their self test.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/vrestir.h"
#include "umma.cuh"

namespace {

// One CTA of 128 threads: D[128x64] = A[128x64] * B[64x64]^T with BF16 operands staged in
// shared memory in the canonical K-major layout and an FP32 accumulator in TMEM.
// `variant` selects which descriptor field carries the K-direction core-matrix stride.
__global__ void __launch_bounds__(128) k_selftest_umma(const uint16_t* __restrict__ A, const uint16_t* __restrict__ B,
                                                       float* __restrict__ D, int variant, int* status) {
    __shared__ __align__(1024) uint16_t sA[128 * 64];
    __shared__ __align__(1024) uint16_t sB[64 * 64];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int i = tid; i < 128 * 64; i += 128) sA[umma::canon_offset(i >> 6, i & 63, 64) >> 1] = A[i];
    for (int i = tid; i < 64 * 64; i += 128) sB[umma::canon_offset(i >> 6, i & 63, 64) >> 1] = B[i];
    if (warp == 0) umma::tmem_alloc(&tmem_base, 64);
    if (tid == 0) umma::mbar_init(&mbar, 1);
    umma::fence_async_shared();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tb = tmem_base;
    const uint32_t lbo = variant == 0 ? 128u : 1024u, sbo = variant == 0 ? 1024u : 128u;
    if (tid == 0) {
        const uint32_t idesc = umma::idesc_bf16_f32(128, 64);
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            uint64_t a = umma::make_desc(umma::smem_addr(sA) + 256u * s, lbo, sbo);
            uint64_t b = umma::make_desc(umma::smem_addr(sB) + 256u * s, lbo, sbo);
            umma::mma_bf16(tb, a, b, idesc, s > 0 ? 1u : 0u);
        }
        umma::commit_to(&mbar);
    }
    bool ok = umma::mbar_wait_bounded(&mbar, 0, status, 1);
    umma::fence_after_sync();
    if (ok) {
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            float v[16];
            umma::tmem_ld16(tb + ((uint32_t)(32 * warp) << 16) + 16u * c, v);
#pragma unroll
            for (int i = 0; i < 16; ++i) D[(32 * warp + lane) * 64 + 16 * c + i] = v[i];
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tb, 64);
}

}  // namespace

extern "C" int vr_selftest_umma(const uint16_t* A, const uint16_t* B, float* D, int32_t variant) {
    if (!A || !B || !D || variant < 0 || variant > 1) return VR_ERR_INVALID_ARG;
    uint16_t *dA = nullptr, *dB = nullptr;
    float* dD = nullptr;
    int* dS = nullptr;
    if (cudaMalloc(&dA, 128 * 64 * 2) != cudaSuccess || cudaMalloc(&dB, 64 * 64 * 2) != cudaSuccess ||
        cudaMalloc(&dD, 128 * 64 * 4) != cudaSuccess || cudaMalloc(&dS, 4) != cudaSuccess) {
        cudaFree(dA); cudaFree(dB); cudaFree(dD); cudaFree(dS);
        return VR_ERR_OOM;
    }
    cudaMemcpy(dA, A, 128 * 64 * 2, cudaMemcpyHostToDevice);
    cudaMemcpy(dB, B, 64 * 64 * 2, cudaMemcpyHostToDevice);
    cudaMemset(dD, 0, 128 * 64 * 4);
    cudaMemset(dS, 0, 4);
    k_selftest_umma<<<1, 128>>>(dA, dB, dD, variant, dS);
    int st = 0;
    cudaError_t e = cudaMemcpy(&st, dS, 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(D, dD, 128 * 64 * 4, cudaMemcpyDeviceToHost);
    cudaFree(dA); cudaFree(dB); cudaFree(dD); cudaFree(dS);
    if (e != cudaSuccess) return VR_ERR_CUDA;
    return st ? VR_ERR_LOOP_LIMIT : VR_OK;
}

// lp.cu -- learned target function (learned p-hat): a small MLP whose inference runs on the
// fifth-generation tensor cores (tcgen05, TMEM accumulators), trained online with Adam.  Also
// holds the tcgen05 GEMM self test that pins the descriptor layout.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

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

// ---------------------------------------------------------------------------------------
// the learned target's network: tensor-core inference, training step, Adam
// ---------------------------------------------------------------------------------------
#include "lp_net.h"
#include "vr_lp.h"

namespace lpk {

using lpn::kHid;
using lpn::kInPad;
using vrd::NetView;

__device__ __forceinline__ void load_query(const float4* q, size_t i, float f[kInPad], const NetView& net) {
    const float4 a = q[2 * i], b = q[2 * i + 1];
    float x[3] = {a.x, a.y, a.z}, w[3] = {a.w, b.x, b.y}, s[5];
    lpn::query_scalars(x, w, net.bmin, net.binv, s);
    lpn::encode(s, f);
}

// Inference: persistent CTAs of 128 threads, one query per thread and tile of 128 queries.
// Each hidden layer is one 128x64x64 BF16 product on the tensor cores (four K=16 steps) into a
// TMEM accumulator, read back with tcgen05.ld for the bias + ReLU + BF16 epilogue that writes the
// next layer's A operand; the output layer (64 -> 1) is a per-thread dot product.
constexpr int kInferSmem = 4 * 8192 + 16384 + (256 + 64 + 4) * 4 + 64;

__global__ void __launch_bounds__(128) k_net_infer(NetView net, const float4* __restrict__ q, int n, const int* __restrict__ nptr,
                                                   float* __restrict__ out, int scatter, int* status) {
    extern __shared__ __align__(1024) unsigned char smem[];
    uint16_t* sW = (uint16_t*)smem;                                     // 4 x (64x64) canonical K-major
    uint16_t* sH = (uint16_t*)(smem + 4 * 8192);                        // 128x64 canonical K-major
    float* sBias = (float*)(smem + 4 * 8192 + 16384);                   // 4 x 64
    float* sW4 = sBias + 256;                                           // 64
    float* sB4 = sW4 + 64;
    uint64_t* mbar = (uint64_t*)(smem + kInferSmem - 64);
    uint32_t* tmem_slot = (uint32_t*)(smem + kInferSmem - 48);
    const int tid = threadIdx.x, warp = tid >> 5;
    if (nptr) n = min(n, *nptr);
    for (int i = tid; i < 4 * 4096; i += 128) {
        int l = i >> 12, r = (i >> 6) & 63, k = i & 63;
        sW[(l * 8192 + (int)umma::canon_offset(r, k, 64)) >> 1] = net.wbf[i];
    }
    for (int i = tid; i < 256; i += 128) sBias[i] = net.bias[i];
    if (tid < 64) sW4[tid] = lpn::bf2f(net.wbf[4 * 4096 + tid]);
    if (tid == 0) *sB4 = net.bias[256];
    if (warp == 0) umma::tmem_alloc(tmem_slot, 64);
    if (tid == 0) umma::mbar_init(mbar, 1);
    umma::fence_async_shared();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tb = *tmem_slot;
    const uint32_t idesc = umma::idesc_bf16_f32(128, 64);
    const uint32_t taddr = tb + ((uint32_t)(32 * warp) << 16);
    uint32_t phase = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile * 128 < n && ok; tile += gridDim.x) {
        const int qi = tile * 128 + tid;
        {
            float f[kInPad];
            if (qi < n) load_query(q, (size_t)qi, f, net);
            else {
#pragma unroll
                for (int k = 0; k < kInPad; ++k) f[k] = 0.f;
            }
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                uint4 v;
                v.x = (uint32_t)lpn::f2bf(f[8 * c + 0]) | ((uint32_t)lpn::f2bf(f[8 * c + 1]) << 16);
                v.y = (uint32_t)lpn::f2bf(f[8 * c + 2]) | ((uint32_t)lpn::f2bf(f[8 * c + 3]) << 16);
                v.z = (uint32_t)lpn::f2bf(f[8 * c + 4]) | ((uint32_t)lpn::f2bf(f[8 * c + 5]) << 16);
                v.w = (uint32_t)lpn::f2bf(f[8 * c + 6]) | ((uint32_t)lpn::f2bf(f[8 * c + 7]) << 16);
                *(uint4*)((unsigned char*)sH + umma::canon_offset(tid, 8 * c, 64)) = v;
            }
        }
        float o = 0.f;
        for (int l = 0; l < 4; ++l) {
            umma::fence_async_shared();
            umma::fence_before_sync();
            __syncthreads();
            umma::fence_after_sync();
            if (tid == 0) {
#pragma unroll
                for (int s = 0; s < 4; ++s) {
                    uint64_t a = umma::make_desc(umma::smem_addr(sH) + 256u * s, 128u, 1024u);
                    uint64_t b = umma::make_desc(umma::smem_addr(sW + l * 4096) + 256u * s, 128u, 1024u);
                    umma::mma_bf16(tb, a, b, idesc, s > 0 ? 1u : 0u);
                }
                umma::commit_to(mbar);
            }
            const bool got = umma::mbar_wait_bounded(mbar, phase, status, 4);
            phase ^= 1u;
            ok = __syncthreads_and(got ? 1 : 0) != 0;
            if (!ok) break;
            umma::fence_after_sync();
            float z[kHid];
#pragma unroll
            for (int c = 0; c < 4; ++c) umma::tmem_ld16(taddr + 16u * c, z + 16 * c);
            if (l < 3) {
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    uint32_t hb[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        float a = z[8 * c + j] + sBias[l * 64 + 8 * c + j];
                        hb[j] = lpn::f2bf(a > 0.f ? a : 0.f);
                    }
                    uint4 v;
                    v.x = hb[0] | (hb[1] << 16);
                    v.y = hb[2] | (hb[3] << 16);
                    v.z = hb[4] | (hb[5] << 16);
                    v.w = hb[6] | (hb[7] << 16);
                    *(uint4*)((unsigned char*)sH + umma::canon_offset(tid, 8 * c, 64)) = v;
                }
            } else {
                float acc = 0.f;
#pragma unroll
                for (int j = 0; j < kHid; ++j) {
                    float a = z[j] + sBias[192 + j];
                    acc += lpn::round_bf(a > 0.f ? a : 0.f) * sW4[j];
                }
                o = acc + *sB4;
            }
        }
        if (ok && qi < n) {
            const float t = lpn::predict_from_logit(o, net.floor_);
            if (scatter) out[__float_as_int(q[2 * (size_t)qi + 1].w)] = t;
            else out[qi] = t;
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tb, 64);
}

// Training step on the CUDA cores: each thread owns one sample (forward, loss, backward); the
// CTA's gradient over its 128 samples is written to its own row of `partials` (no atomics, so a
// step is deterministic).  Loss: (T(x, w) - target)^2 averaged over the batch, T = exp(o).
constexpr int kTrainSmem = 4 * 4096 * 4 + 5 * 64 * 128 * 2 + 128 * 65 * 4 + 320 * 4 + 2 * 128 * 4;

__global__ void __launch_bounds__(128) k_net_train(NetView net, const float4* __restrict__ samples, int n, float invB,
                                                   float* __restrict__ partials, float* __restrict__ lossParts) {
    extern __shared__ __align__(1024) unsigned char smem[];
    float* sW = (float*)smem;                                       // 4 x [64 out][64 in]
    uint16_t* sH = (uint16_t*)(smem + 4 * 4096 * 4);                // 5 x [64][128] activations (bf16)
    float* sDZ = (float*)(smem + 4 * 4096 * 4 + 5 * 64 * 128 * 2);  // [128][65]
    float* sMisc = sDZ + 128 * 65;                                  // biases 256, output weights 64
    float* sG = sMisc + 320;                                        // per-sample dL/do
    float* sL = sG + 128;                                           // per-sample loss
    const int tid = threadIdx.x;
    for (int i = tid; i < 4 * 4096; i += 128) sW[i] = lpn::bf2f(net.wbf[i]);
    for (int i = tid; i < 256; i += 128) sMisc[i] = net.bias[i];
    if (tid < 64) sMisc[256 + tid] = lpn::bf2f(net.wbf[4 * 4096 + tid]);
    __syncthreads();
    const int si = blockIdx.x * 128 + tid;
    bool valid = si < n;
    float h[kHid];
    {
        float f[kInPad];
        if (valid) {
            load_query(samples, (size_t)si, f, net);
            valid = samples[2 * (size_t)si + 1].z >= 0.f;
        } else {
            for (int k = 0; k < kInPad; ++k) f[k] = 0.f;
        }
        for (int k = 0; k < kInPad; ++k) {
            uint16_t b = lpn::f2bf(f[k]);
            sH[k * 128 + tid] = b;
            h[k] = lpn::bf2f(b);
        }
    }
    for (int l = 0; l < 4; ++l) {
        const float* W = sW + l * 4096;
        float hn[kHid];
        for (int nn = 0; nn < kHid; ++nn) {
            float acc = 0.f;
#pragma unroll 16
            for (int k = 0; k < kInPad; ++k) acc += W[nn * 64 + k] * h[k];
            float a = acc + sMisc[l * 64 + nn];
            uint16_t b = lpn::f2bf(a > 0.f ? a : 0.f);
            sH[((l + 1) * 64 + nn) * 128 + tid] = b;
            hn[nn] = lpn::bf2f(b);
        }
        for (int k = 0; k < kHid; ++k) h[k] = hn[k];
    }
    float o = 0.f;
    for (int k = 0; k < kHid; ++k) o += h[k] * sMisc[256 + k];
    o += net.bias[256];
    float g = 0.f, lv = 0.f;
    if (valid) {
        const float p = vr::exp_(o);
        const float d = p - samples[2 * (size_t)si + 1].w;
        g = 2.f * d * p * invB;
        lv = d * d * invB;
    }
    sG[tid] = g;
    sL[tid] = lv;
    float* part = partials + (size_t)blockIdx.x * lpn::kParamsPad;
    // output layer
    float dh[kHid];
    for (int k = 0; k < kHid; ++k) dh[k] = g * sMisc[256 + k];
    for (int k = 0; k < kHid; ++k) sDZ[tid * 65 + k] = h[k];
    __syncthreads();
    if (tid < 64) {
        float acc = 0.f;
        for (int t = 0; t < 128; ++t) acc += sG[t] * sDZ[t * 65 + tid];
        part[lpn::kOutW + tid] = acc;
    } else if (tid == 64) {
        float acc = 0.f, ls = 0.f;
        for (int t = 0; t < 128; ++t) { acc += sG[t]; ls += sL[t]; }
        part[lpn::kOutB] = acc;
        lossParts[blockIdx.x] = ls;
    }
    __syncthreads();
    for (int l = 3; l >= 0; --l) {
        const float* W = sW + l * 4096;
        float dz[kHid];
        for (int nn = 0; nn < kHid; ++nn) {
            float hv = lpn::bf2f(sH[((l + 1) * 64 + nn) * 128 + tid]);
            dz[nn] = hv > 0.f ? dh[nn] : 0.f;
            sDZ[tid * 65 + nn] = dz[nn];
        }
        if (l > 0) {
            for (int k = 0; k < kHid; ++k) {
                float acc = 0.f;
#pragma unroll 16
                for (int nn = 0; nn < kHid; ++nn) acc += W[nn * 64 + k] * dz[nn];
                dh[k] = acc;
            }
        }
        __syncthreads();
        // dW[nn][k] = sum_t dz[t][nn] * h_l[t][k]: thread -> row nn = tid / 2, half of the k range
        {
            const int nn = tid >> 1, k0 = (tid & 1) * 32;
            float acc[32], accb = 0.f;
#pragma unroll
            for (int j = 0; j < 32; ++j) acc[j] = 0.f;
            for (int t = 0; t < 128; ++t) {
                const float d = sDZ[t * 65 + nn];
                accb += d;
#pragma unroll
                for (int j = 0; j < 32; ++j) acc[j] += d * lpn::bf2f(sH[(l * 64 + k0 + j) * 128 + t]);
            }
            float* gw = part + lpn::w_off(l) + nn * 64 + k0;
#pragma unroll
            for (int j = 0; j < 32; ++j) gw[j] = acc[j];
            if ((tid & 1) == 0) part[lpn::b_off(l) + nn] = accb;
        }
        __syncthreads();
    }
}

__device__ __forceinline__ void scatter_param(int i, float wi, uint16_t* wbf, float* bias) {
    const int l = i / lpn::kLayerStride, r = i % lpn::kLayerStride;
    if (i < lpn::kOutW) {
        if (r < 4096) wbf[l * 4096 + r] = lpn::f2bf(wi);
        else bias[l * 64 + (r - 4096)] = wi;
    } else if (i < lpn::kOutB) {
        wbf[4 * 4096 + (i - lpn::kOutW)] = lpn::f2bf(wi);
    } else {
        bias[256] = wi;
    }
}

// sums the CTAs' partial gradients in a fixed order, then (update != 0) one Adam step
// (beta1 0.9, beta2 0.999, eps 1e-8) on the FP32 master weights, refreshing the BF16 copy
__global__ void k_net_reduce_adam(const float* __restrict__ partials, int parts, const float* __restrict__ lossParts, float* __restrict__ w,
                                  float* __restrict__ m, float* __restrict__ v, float* __restrict__ grads, float* __restrict__ loss,
                                  uint16_t* __restrict__ wbf, float* __restrict__ bias, float lr, float c1, float c2, int update) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        float ls = 0.f;
        for (int p = 0; p < parts; ++p) ls += lossParts[p];
        *loss = ls;
    }
    if (i >= lpn::kParams) return;
    float gi = 0.f;
    for (int p = 0; p < parts; ++p) gi += partials[(size_t)p * lpn::kParamsPad + i];
    grads[i] = gi;
    if (!update) return;
    const float mi = 0.9f * m[i] + 0.1f * gi;
    const float vi = 0.999f * v[i] + 0.001f * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (vr::sqrt_(vi / c2) + 1e-8f);
    w[i] = wi;
    scatter_param(i, wi, wbf, bias);
}

__global__ void k_net_pack(const float* __restrict__ w, uint16_t* __restrict__ wbf, float* __restrict__ bias) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < lpn::kParams) scatter_param(i, w[i], wbf, bias);
}

}  // namespace lpk

namespace vrk {

int net_infer_smem() { return lpk::kInferSmem; }
int net_train_smem() { return lpk::kTrainSmem; }

cudaError_t net_setup() {
    cudaError_t e = cudaFuncSetAttribute(lpk::k_net_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, lpk::kInferSmem);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(lpk::k_net_train, cudaFuncAttributeMaxDynamicSharedMemorySize, lpk::kTrainSmem);
}

// grid: persistent, 4 CTAs per SM (TMEM: 4 x 64 columns)
void launch_net_infer(const vrd::NetView& net, const float4* q, int n, const int* nptr, float* out, int scatter, int* status, int numSMs,
                      cudaStream_t st) {
    int tiles = (n + 127) / 128;
    int grid = std::max(1, std::min(tiles, numSMs * 4));
    lpk::k_net_infer<<<grid, 128, lpk::kInferSmem, st>>>(net, q, n, nptr, out, scatter, status);
}

void launch_net_train(const vrd::NetView& net, const float4* samples, int n, float* partials, float* lossParts, cudaStream_t st) {
    int grid = (n + 127) / 128;
    lpk::k_net_train<<<grid, 128, lpk::kTrainSmem, st>>>(net, samples, n, 1.f / (float)n, partials, lossParts);
}

void launch_net_reduce_adam(const float* partials, int parts, const float* lossParts, float* w, float* m, float* v, float* grads, float* loss,
                            uint16_t* wbf, float* bias, float lr, float c1, float c2, int update, cudaStream_t st) {
    lpk::k_net_reduce_adam<<<(lpn::kParams + 255) / 256, 256, 0, st>>>(partials, parts, lossParts, w, m, v, grads, loss, wbf, bias, lr, c1, c2,
                                                                         update);
}

void launch_net_pack(const float* w, uint16_t* wbf, float* bias, cudaStream_t st) {
    lpk::k_net_pack<<<(lpn::kParams + 255) / 256, 256, 0, st>>>(w, wbf, bias);
}

}  // namespace vrk

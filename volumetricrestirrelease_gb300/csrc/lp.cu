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

// two floats -> packed BF16 pair (lo in the low half), round to nearest even in one instruction
__device__ __forceinline__ uint32_t bf16x2(float lo, float hi) {
    uint32_t r;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}
__device__ __forceinline__ float bfround(float f) { return __uint_as_float(bf16x2(f, 0.f) << 16); }

// the query's 64 input features; band 0 from the hardware sine/cosine (the higher bands follow by
// the double-angle recurrences as in lpn::encode)
__device__ __forceinline__ void load_query(const float4* q, size_t i, float f[kInPad], const NetView& net) {
    const float4 a = q[2 * i], b = q[2 * i + 1];
    float x[3] = {a.x, a.y, a.z}, w[3] = {a.w, b.x, b.y}, s[5];
    lpn::query_scalars(x, w, net.bmin, net.binv, s);
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        float sn, cs;
        __sincosf(s[k] * 3.14159265358979323846f, &sn, &cs);
#pragma unroll
        for (int band = 0; band < lpn::kBands; ++band) {
            f[12 * k + 2 * band] = sn;
            f[12 * k + 2 * band + 1] = cs;
            const float s2 = 2.f * sn * cs, c2 = cs * cs - sn * sn;
            sn = s2;
            cs = c2;
        }
    }
#pragma unroll
    for (int k = lpn::kIn; k < kInPad; ++k) f[k] = 0.f;
}

// Inference: persistent CTAs of 128 threads, one query per thread and tile of 128 queries.
// Each hidden layer is one 128x64x64 BF16 product on the tensor cores (four K=16 steps) into a
// TMEM accumulator, read back with tcgen05.ld for the bias + ReLU + BF16 epilogue that writes the
// next layer's A operand; the output layer (64 -> 1) is a per-thread dot product.
constexpr int kInferSmem = 4 * 8192 + 16384 + (256 + 64 + 4) * 4 + 64;

// idx == nullptr: query qi is record qi and its T goes to out[qi]; otherwise query qi is record
// idx[qi] (a slot of the frame's per-slot query array) and its T goes to out[idx[qi]]
__global__ void __launch_bounds__(128) k_net_infer(NetView net, const float4* __restrict__ q, int n, const int* __restrict__ nptr,
                                                   float* __restrict__ out, const int* __restrict__ idx, int* status) {
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
        const int rec = qi < n ? (idx ? idx[qi] : qi) : 0;
        {
            float f[kInPad];
            if (qi < n) load_query(q, (size_t)rec, f, net);
            else {
#pragma unroll
                for (int k = 0; k < kInPad; ++k) f[k] = 0.f;
            }
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                uint4 v;
                v.x = bf16x2(f[8 * c + 0], f[8 * c + 1]);
                v.y = bf16x2(f[8 * c + 2], f[8 * c + 3]);
                v.z = bf16x2(f[8 * c + 4], f[8 * c + 5]);
                v.w = bf16x2(f[8 * c + 6], f[8 * c + 7]);
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
                    float hf[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        float a = z[8 * c + j] + sBias[l * 64 + 8 * c + j];
                        hf[j] = a > 0.f ? a : 0.f;
                    }
                    uint4 v;
                    v.x = bf16x2(hf[0], hf[1]);
                    v.y = bf16x2(hf[2], hf[3]);
                    v.z = bf16x2(hf[4], hf[5]);
                    v.w = bf16x2(hf[6], hf[7]);
                    *(uint4*)((unsigned char*)sH + umma::canon_offset(tid, 8 * c, 64)) = v;
                }
            } else {
                float acc = 0.f;
#pragma unroll
                for (int j = 0; j < kHid; ++j) {
                    float a = z[j] + sBias[192 + j];
                    acc += bfround(a > 0.f ? a : 0.f) * sW4[j];
                }
                o = acc + *sB4;
            }
        }
        if (ok && qi < n) out[rec] = lpn::predict_from_logit(o, net.floor_);
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tb, 64);
}

// Training step on the tensor cores.  One CTA of 128 threads owns a tile of 128 samples, one
// sample per thread (TMEM lane).  Forward: four 128x64x64 BF16 products (as in inference),
// keeping every layer's BF16 input transposed in shared memory.  Backward, per hidden layer l
// from the top: dZ_l = dH ∘ [X_{l+1} > 0] is rounded to BF16 and stored twice, as the A operand
// of dH_l = dZ_l W_l (128x64x64) and, transposed and padded to 128 rows, as the A operand of
// dW_l = dZ_l^T X_l (128x64, K = 128 samples); both products accumulate in FP32 in TMEM.  The
// output layer and the biases are reduced on the CUDA cores.  The CTA writes its gradient to
// its own row of `partials` (no atomics: a step is deterministic).
// Loss: mean over the batch of (T - target)^2 with T = exp(o), or of (o - log max(target, floor))^2;
// samples with tmax < 0 add zero.
namespace ts {
constexpr int W = 0;               // 4 x 8192: W_l, [64 out][64 in] K-major (forward B operand)
constexpr int WT = 32768;          // 3 x 8192: W_l^T for l = 1..3, [64 in][64 out] K-major (dH B operand)
constexpr int X = 57344;           // 16384: layer input, [128 samples][64] K-major (forward A operand)
constexpr int XT = 73728;          // 4 x 16384: X_l^T, [64][128 samples] K-major (dW B operand)
constexpr int DZ = 139264;         // 16384: dZ, [128 samples][64] K-major (dH A operand)
constexpr int DZT = 155648;        // 32768: dZ^T padded, [128 rows, 64..127 zero][128 samples] (dW A operand)
constexpr int F = 188416;          // floats: biases 256, w4 64, b4 1 (+3), g 128, loss 128
constexpr int MB = F + (256 + 64 + 4 + 128 + 128) * 4;   // mbarrier, TMEM address
constexpr int Total = MB + 16;
}  // namespace ts
constexpr int kTrainSmem = ts::Total;
constexpr uint32_t kTmemZ = 0, kTmemH = 64, kTmemW = 128;   // column bases; 512 columns allocated

__device__ __forceinline__ void st_row_bf16(unsigned char* base, int row, const float* v, int K) {
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        uint4 u;
        u.x = bf16x2(v[8 * c + 0], v[8 * c + 1]);
        u.y = bf16x2(v[8 * c + 2], v[8 * c + 3]);
        u.z = bf16x2(v[8 * c + 4], v[8 * c + 5]);
        u.w = bf16x2(v[8 * c + 6], v[8 * c + 7]);
        *(uint4*)(base + umma::canon_offset(row, 8 * c, K)) = u;
    }
}
// column `col` of a [64 rows][128] K-major tile: v[r] -> element (r, col)
__device__ __forceinline__ void st_col_bf16(unsigned char* base, int col, const float* v) {
#pragma unroll
    for (int r = 0; r < 64; ++r) *(uint16_t*)(base + umma::canon_offset(r, col, 128)) = lpn::f2bf(v[r]);
}

__device__ __forceinline__ bool train_mma_wait(uint64_t* mbar, uint32_t& phase, int* status) {
    const bool got = umma::mbar_wait_bounded(mbar, phase, status, 8);
    phase ^= 1u;
    const bool ok = __syncthreads_and(got ? 1 : 0) != 0;
    umma::fence_after_sync();
    return ok;
}
__device__ __forceinline__ void train_issue_sync() {
    umma::fence_async_shared();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
}

__global__ void __launch_bounds__(128, 1) k_net_train(NetView net, const float4* __restrict__ samples, int n, float invB,
                                                      float* __restrict__ partials, float* __restrict__ lossParts, int* status) {
    extern __shared__ __align__(1024) unsigned char smem[];
    float* sBias = (float*)(smem + ts::F);
    float* sW4 = sBias + 256;
    float* sB4 = sW4 + 64;
    float* sG = sB4 + 4;
    float* sL = sG + 128;
    uint64_t* mbar = (uint64_t*)(smem + ts::MB);
    uint32_t* tmem_slot = (uint32_t*)(smem + ts::MB + 8);
    const int tid = threadIdx.x, warp = tid >> 5;
    // weights (and their transposes) in the canonical K-major layout, zero padding of dZ^T
    for (int i = tid; i < 4 * 4096; i += 128) {
        const int l = i >> 12, r = (i >> 6) & 63, k = i & 63;
        const uint16_t w = net.wbf[i];
        *(uint16_t*)(smem + ts::W + l * 8192 + umma::canon_offset(r, k, 64)) = w;
        if (l > 0) *(uint16_t*)(smem + ts::WT + (l - 1) * 8192 + umma::canon_offset(k, r, 64)) = w;
    }
    for (int i = tid; i < 16384 / 16; i += 128) *(uint4*)(smem + ts::DZT + 16384 + 16 * i) = make_uint4(0, 0, 0, 0);
    for (int i = tid; i < 256; i += 128) sBias[i] = net.bias[i];
    if (tid < 64) sW4[tid] = lpn::bf2f(net.wbf[4 * 4096 + tid]);
    if (tid == 0) *sB4 = net.bias[256];
    if (warp == 0) umma::tmem_alloc(tmem_slot, 512);
    if (tid == 0) umma::mbar_init(mbar, 1);
    train_issue_sync();
    const uint32_t tb = *tmem_slot;
    const uint32_t lane_off = (uint32_t)(32 * warp) << 16;
    const uint32_t id64 = umma::idesc_bf16_f32(128, 64);
    uint32_t phase = 0;
    bool ok = true;

    const int si = blockIdx.x * 128 + tid;
    bool valid = si < n;
    float h[64];
    {
        if (si < n) {
            load_query(samples, (size_t)si, h, net);
            valid = samples[2 * (size_t)si + 1].z >= 0.f;
        } else {
#pragma unroll
            for (int k = 0; k < 64; ++k) h[k] = 0.f;
        }
        st_row_bf16(smem + ts::X, tid, h, 64);
        st_col_bf16(smem + ts::XT, tid, h);
    }
    // forward
    for (int l = 0; l < 4 && ok; ++l) {
        train_issue_sync();
        if (tid == 0) {
#pragma unroll
            for (int s = 0; s < 4; ++s) {
                uint64_t a = umma::make_desc(umma::smem_addr(smem + ts::X) + 256u * s, 128u, 1024u);
                uint64_t b = umma::make_desc(umma::smem_addr(smem + ts::W + l * 8192) + 256u * s, 128u, 1024u);
                umma::mma_bf16(tb + kTmemZ, a, b, id64, s > 0 ? 1u : 0u);
            }
            umma::commit_to(mbar);
        }
        if (!(ok = train_mma_wait(mbar, phase, status))) break;
#pragma unroll
        for (int c = 0; c < 4; ++c) umma::tmem_ld16(tb + lane_off + kTmemZ + 16u * c, h + 16 * c);
#pragma unroll
        for (int k = 0; k < 64; ++k) {
            const float a = h[k] + sBias[l * 64 + k];
            h[k] = bfround(a > 0.f ? a : 0.f);
        }
        if (l < 3) {
            st_row_bf16(smem + ts::X, tid, h, 64);
            st_col_bf16(smem + ts::XT + (l + 1) * 16384, tid, h);
        }
    }
    // output layer, loss, dL/do
    float g = 0.f;
    if (ok) {
        float o = 0.f;
#pragma unroll
        for (int k = 0; k < 64; ++k) o += h[k] * sW4[k];
        o += *sB4;
        float lv = 0.f;
        if (valid) {
            const float y = samples[2 * (size_t)si + 1].w;
            if (net.lossLog) {
                const float d = o - vr::log_(vr::fmax_(y, net.floor_));
                g = 2.f * d * invB;
                lv = d * d * invB;
            } else {
                const float p = vr::exp_(o);
                const float d = p - y;
                g = 2.f * d * p * invB;
                lv = d * d * invB;
            }
        }
        sG[tid] = g;
        sL[tid] = lv;
        st_row_bf16(smem + ts::X, tid, h, 64);      // X_4 (exact: already BF16 values)
    }
    float* part = partials + (size_t)blockIdx.x * lpn::kParamsPad;
    __syncthreads();
    if (ok) {
        if (tid < 64) {
            float acc = 0.f;
            for (int t = 0; t < 128; ++t) acc += sG[t] * lpn::bf2f(*(const uint16_t*)(smem + ts::X + umma::canon_offset(t, tid, 64)));
            part[lpn::kOutW + tid] = acc;
        } else if (tid == 64) {
            float acc = 0.f, ls = 0.f;
            for (int t = 0; t < 128; ++t) { acc += sG[t]; ls += sL[t]; }
            part[lpn::kOutB] = acc;
            lossParts[blockIdx.x] = ls;
        }
    }
    // backward through the hidden layers; h holds X_{l+1} of this sample
    float dz[64];
#pragma unroll
    for (int k = 0; k < 64; ++k) dz[k] = h[k] > 0.f ? g * sW4[k] : 0.f;
    for (int l = 3; l >= 0 && ok; --l) {
        st_row_bf16(smem + ts::DZ, tid, dz, 64);
        // column tid of dZ^T (rows 0..63)
#pragma unroll
        for (int r = 0; r < 64; ++r) *(uint16_t*)(smem + ts::DZT + umma::canon_offset(r, tid, 128)) = lpn::f2bf(dz[r]);
        train_issue_sync();
        if (tid == 0) {
            if (l > 0) {
#pragma unroll
                for (int s = 0; s < 4; ++s) {
                    uint64_t a = umma::make_desc(umma::smem_addr(smem + ts::DZ) + 256u * s, 128u, 1024u);
                    uint64_t b = umma::make_desc(umma::smem_addr(smem + ts::WT + (l - 1) * 8192) + 256u * s, 128u, 1024u);
                    umma::mma_bf16(tb + kTmemH, a, b, id64, s > 0 ? 1u : 0u);
                }
            }
#pragma unroll
            for (int s = 0; s < 8; ++s) {
                uint64_t a = umma::make_desc(umma::smem_addr(smem + ts::DZT) + 256u * s, 128u, 2048u);
                uint64_t b = umma::make_desc(umma::smem_addr(smem + ts::XT + l * 16384) + 256u * s, 128u, 2048u);
                umma::mma_bf16(tb + kTmemW + 64u * l, a, b, id64, s > 0 ? 1u : 0u);
            }
            umma::commit_to(mbar);
        }
        // bias gradient of layer l from the BF16 dZ^T rows (read while the products run)
        if (tid < 64) {
            float acc = 0.f;
            for (int t0 = 0; t0 < 128; t0 += 8) {
                const uint4 u = *(const uint4*)(smem + ts::DZT + umma::canon_offset(tid, t0, 128));
                const uint32_t w4[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    acc += lpn::bf2f((uint16_t)(w4[j] & 0xFFFFu));
                    acc += lpn::bf2f((uint16_t)(w4[j] >> 16));
                }
            }
            part[lpn::b_off(l) + tid] = acc;
        }
        if (!(ok = train_mma_wait(mbar, phase, status))) break;
        if (l > 0) {
            float dh[64];
#pragma unroll
            for (int c = 0; c < 4; ++c) umma::tmem_ld16(tb + lane_off + kTmemH + 16u * c, dh + 16 * c);
            // ReLU mask from this sample's input of layer l (column tid of X_l^T)
#pragma unroll
            for (int k = 0; k < 64; ++k) {
                const float xv = lpn::bf2f(*(const uint16_t*)(smem + ts::XT + l * 16384 + umma::canon_offset(k, tid, 128)));
                dz[k] = xv > 0.f ? dh[k] : 0.f;
            }
        }
    }
    // weight gradients: TMEM lanes 0..63 (warps 0 and 1) hold the rows of dW_l
    if (ok && warp < 2) {
        const int r = tid;
        for (int l = 0; l < 4; ++l) {
            float v[64];
#pragma unroll
            for (int c = 0; c < 4; ++c) umma::tmem_ld16(tb + lane_off + kTmemW + 64u * l + 16u * c, v + 16 * c);
            float* gw = part + lpn::w_off(l) + r * 64;
#pragma unroll
            for (int k = 0; k < 64; k += 4) *(float4*)(gw + k) = make_float4(v[k], v[k + 1], v[k + 2], v[k + 3]);
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tb, 512);
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
// (beta1 0.9, beta2 0.999, eps 1e-8) on the FP32 master weights, refreshing the BF16 copy; the
// bias corrections c1 = 1 - 0.9^t, c2 = 1 - 0.999^t come as arguments or, when cc is not null,
// from device memory (cc[0], cc[1]) so that a captured graph can replay the step
__global__ void k_net_reduce_adam(const float* __restrict__ partials, int parts, const float* __restrict__ lossParts, float* __restrict__ w,
                                  float* __restrict__ m, float* __restrict__ v, float* __restrict__ grads, float* __restrict__ loss,
                                  uint16_t* __restrict__ wbf, float* __restrict__ bias, float lr, float c1, float c2, const float* cc,
                                  int update) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (cc) { c1 = cc[0]; c2 = cc[1]; }
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
void launch_net_infer(const vrd::NetView& net, const float4* q, int n, const int* nptr, float* out, const int* idx, int* status, int numSMs,
                      cudaStream_t st) {
    int tiles = (n + 127) / 128;
    int grid = std::max(1, std::min(tiles, numSMs * 4));
    lpk::k_net_infer<<<grid, 128, lpk::kInferSmem, st>>>(net, q, n, nptr, out, idx, status);
}

void launch_net_train(const vrd::NetView& net, const float4* samples, int n, float* partials, float* lossParts, int* status, cudaStream_t st) {
    int grid = (n + 127) / 128;
    lpk::k_net_train<<<grid, 128, lpk::kTrainSmem, st>>>(net, samples, n, 1.f / (float)n, partials, lossParts, status);
}

void launch_net_reduce_adam(const float* partials, int parts, const float* lossParts, float* w, float* m, float* v, float* grads, float* loss,
                            uint16_t* wbf, float* bias, float lr, float c1, float c2, const float* cc, int update, cudaStream_t st) {
    lpk::k_net_reduce_adam<<<(lpn::kParams + 255) / 256, 256, 0, st>>>(partials, parts, lossParts, w, m, v, grads, loss, wbf, bias, lr, c1, c2,
                                                                         cc, update);
}

void launch_net_pack(const float* w, uint16_t* wbf, float* bias, cudaStream_t st) {
    lpk::k_net_pack<<<(lpn::kParams + 255) / 256, 256, 0, st>>>(w, wbf, bias);
}

}  // namespace vrk

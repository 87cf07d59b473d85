// post.cu -- the post-process passes around the frame loop: frame accumulation
// (AccumulatePass: Accumulate.cs.slang:55-125, precision modes of AccumulatePass.h:66-71) and
// error measurement against a reference image (ErrorMeasurePass: ErrorMeasurer.cs.slang, the
// sum reduction and averages of ErrorMeasurePass.cpp:216-250), plus the relative MSE the
// benchmark reports.  Both are streaming kernels over float4 pixels: one thread per pixel,
// coalesced 16-byte loads, HBM-bound.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

#include "../../include/vrestir.h"

struct vr_accumulator {
    int W = 0, H = 0, precision = VR_ACCUM_DOUBLE;
    int64_t count = 0;
    void* sum = nullptr;            // double4 (double) or float4 (single modes) per pixel
    float4* corr = nullptr;         // compensation terms (single compensated)
};

namespace {

struct D4 { double v[4]; };

__global__ void k_accum_double(const float4* __restrict__ cur, D4* __restrict__ sum, float4* __restrict__ out, int64_t n, double denom,
                               int reset) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 c = cur[i];
    D4 s = reset ? D4{{0.0, 0.0, 0.0, 0.0}} : sum[i];
    s.v[0] += (double)c.x; s.v[1] += (double)c.y; s.v[2] += (double)c.z; s.v[3] += (double)c.w;
    sum[i] = s;
    if (out) out[i] = make_float4((float)(s.v[0] / denom), (float)(s.v[1] / denom), (float)(s.v[2] / denom), (float)(s.v[3] / denom));
}

__global__ void k_accum_single(const float4* __restrict__ cur, float4* __restrict__ sum, float4* __restrict__ out, int64_t n, float denom,
                               int reset) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 c = cur[i];
    float4 s = reset ? make_float4(0.f, 0.f, 0.f, 0.f) : sum[i];
    s.x = __fadd_rn(s.x, c.x); s.y = __fadd_rn(s.y, c.y); s.z = __fadd_rn(s.z, c.z); s.w = __fadd_rn(s.w, c.w);
    sum[i] = s;
    if (out) out[i] = make_float4(__fdiv_rn(s.x, denom), __fdiv_rn(s.y, denom), __fdiv_rn(s.z, denom), __fdiv_rn(s.w, denom));
}

// Kahan summation, one channel
__device__ __forceinline__ void kahan(float& s, float& c, float x) {
    const float y = __fsub_rn(x, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
}

__global__ void k_accum_kahan(const float4* __restrict__ cur, float4* __restrict__ sum, float4* __restrict__ corr, float4* __restrict__ out,
                              int64_t n, float denom, int reset) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 x = cur[i];
    float4 s = reset ? make_float4(0.f, 0.f, 0.f, 0.f) : sum[i];
    float4 c = reset ? make_float4(0.f, 0.f, 0.f, 0.f) : corr[i];
    kahan(s.x, c.x, x.x); kahan(s.y, c.y, x.y); kahan(s.z, c.z, x.z); kahan(s.w, c.w, x.w);
    sum[i] = s;
    corr[i] = c;
    if (out) out[i] = make_float4(__fdiv_rn(s.x, denom), __fdiv_rn(s.y, denom), __fdiv_rn(s.z, denom), __fdiv_rn(s.w, denom));
}

// per-pixel error terms, summed per block in FP64 (fixed tree order), block partials summed on
// the host in block order: the result does not depend on scheduling
constexpr int kErrThreads = 256;
__global__ void k_error(const float4* __restrict__ src, const float4* __restrict__ ref, const float4* __restrict__ wpos, int64_t n, int mode,
                        float eps, double* __restrict__ partial, float4* __restrict__ diffOut) {
    __shared__ double sh[3][kErrThreads];
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double e[3] = {0.0, 0.0, 0.0};
    if (i < n) {
        const float4 a = src[i], r = ref[i];
        const bool valid = !(mode & VR_ERRM_IGNORE_BACKGROUND) || !wpos || wpos[i].w != 0.f;
        float d[3] = {0.f, 0.f, 0.f};
        if (valid) {
            const float s3[3] = {a.x, a.y, a.z}, r3[3] = {r.x, r.y, r.z};
            for (int k = 0; k < 3; ++k) {
                float t = fabsf(__fsub_rn(s3[k], r3[k]));
                if (mode & VR_ERRM_RELATIVE) t = __fdiv_rn(__fmul_rn(t, t), __fadd_rn(__fmul_rn(r3[k], r3[k]), eps));
                else if (mode & VR_ERRM_SQUARED) t = __fmul_rn(t, t);
                d[k] = t;
            }
            if (mode & VR_ERRM_AVERAGE) {
                const float m = __fdiv_rn(__fadd_rn(__fadd_rn(d[0], d[1]), d[2]), 3.f);
                d[0] = d[1] = d[2] = m;
            }
        }
        if (diffOut) diffOut[i] = make_float4(d[0], d[1], d[2], 0.f);
        for (int k = 0; k < 3; ++k) e[k] = (double)d[k];
    }
    for (int k = 0; k < 3; ++k) sh[k][threadIdx.x] = e[k];
    __syncthreads();
    for (int w = kErrThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int k = 0; k < 3; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 3; ++k) partial[(size_t)blockIdx.x * 3 + k] = sh[k][0];
}

}  // namespace

extern "C" {

int vr_accumulator_create(int32_t width, int32_t height, int32_t precision, vr_accumulator** out) {
    if (!out || width <= 0 || height <= 0 || (int64_t)width * height > ((int64_t)1 << 31) ||
        (precision != VR_ACCUM_DOUBLE && precision != VR_ACCUM_SINGLE && precision != VR_ACCUM_SINGLE_COMPENSATED))
        return VR_ERR_INVALID_ARG;
    vr_accumulator* a = new vr_accumulator();
    a->W = width; a->H = height; a->precision = precision;
    const size_t n = (size_t)width * height;
    if (cudaMalloc(&a->sum, n * (precision == VR_ACCUM_DOUBLE ? sizeof(D4) : sizeof(float4))) != cudaSuccess ||
        (precision == VR_ACCUM_SINGLE_COMPENSATED && cudaMalloc(&a->corr, n * sizeof(float4)) != cudaSuccess)) {
        cudaFree(a->sum); cudaFree(a->corr);
        delete a;
        return VR_ERR_OOM;
    }
    *out = a;
    return VR_OK;
}

void vr_accumulator_destroy(vr_accumulator* a) {
    if (!a) return;
    cudaFree(a->sum);
    cudaFree(a->corr);
    delete a;
}

void vr_accumulator_reset(vr_accumulator* a) { if (a) a->count = 0; }
int64_t vr_accumulator_count(const vr_accumulator* a) { return a ? a->count : 0; }

int vr_accumulate(vr_accumulator* a, const float* frame_rgba, float* out_rgba, void* stream) {
    if (!a || !frame_rgba) return VR_ERR_INVALID_ARG;
    const int64_t n = (int64_t)a->W * a->H;
    const int threads = 256;
    const unsigned blocks = (unsigned)((n + threads - 1) / threads);
    cudaStream_t st = (cudaStream_t)stream;
    const int reset = a->count == 0;
    const auto* cur = reinterpret_cast<const float4*>(frame_rgba);
    auto* outp = reinterpret_cast<float4*>(out_rgba);
    if (a->precision == VR_ACCUM_DOUBLE)
        k_accum_double<<<blocks, threads, 0, st>>>(cur, (D4*)a->sum, outp, n, (double)(a->count + 1), reset);
    else if (a->precision == VR_ACCUM_SINGLE)
        k_accum_single<<<blocks, threads, 0, st>>>(cur, (float4*)a->sum, outp, n, (float)(a->count + 1), reset);
    else
        k_accum_kahan<<<blocks, threads, 0, st>>>(cur, (float4*)a->sum, a->corr, outp, n, (float)(a->count + 1), reset);
    if (cudaGetLastError() != cudaSuccess) return VR_ERR_CUDA;
    a->count++;
    return VR_OK;
}

int vr_error_measure(const float* src_rgba, const float* ref_rgba, const float* world_pos_or_null, int32_t width, int32_t height, int32_t mode,
                     float eps, double error_out[3], float* diff_out_or_null, void* stream) {
    if (!src_rgba || !ref_rgba || !error_out || width <= 0 || height <= 0 || !(eps >= 0.f) ||
        (mode & ~(VR_ERRM_IGNORE_BACKGROUND | VR_ERRM_SQUARED | VR_ERRM_AVERAGE | VR_ERRM_RELATIVE)))
        return VR_ERR_INVALID_ARG;
    const int64_t n = (int64_t)width * height;
    const unsigned blocks = (unsigned)((n + kErrThreads - 1) / kErrThreads);
    double* partial = nullptr;
    if (cudaMalloc(&partial, (size_t)blocks * 3 * sizeof(double)) != cudaSuccess) return VR_ERR_OOM;
    cudaStream_t st = (cudaStream_t)stream;
    k_error<<<blocks, kErrThreads, 0, st>>>(reinterpret_cast<const float4*>(src_rgba), reinterpret_cast<const float4*>(ref_rgba),
                                            reinterpret_cast<const float4*>(world_pos_or_null), n, mode, eps, partial,
                                            reinterpret_cast<float4*>(diff_out_or_null));
    double* host = new double[(size_t)blocks * 3];
    const bool ok = cudaGetLastError() == cudaSuccess &&
                    cudaMemcpyAsync(host, partial, (size_t)blocks * 3 * sizeof(double), cudaMemcpyDeviceToHost, st) == cudaSuccess &&
                    cudaStreamSynchronize(st) == cudaSuccess;
    cudaFree(partial);
    if (!ok) { delete[] host; return VR_ERR_CUDA; }
    double s[3] = {0.0, 0.0, 0.0};
    for (unsigned b = 0; b < blocks; ++b)
        for (int k = 0; k < 3; ++k) s[k] += host[(size_t)b * 3 + k];
    delete[] host;
    for (int k = 0; k < 3; ++k) error_out[k] = s[k] / (double)n;
    return VR_OK;
}

}  // extern "C"

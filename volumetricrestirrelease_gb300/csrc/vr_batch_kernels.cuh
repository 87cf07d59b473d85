// vr_batch_kernels.cuh -- the persistent batched frame kernels (see batch.cu).
#pragma once

#include "vr_batch.h"
#include "vr_lp_kernels.cuh"

namespace vrd {

enum BatchPass { kPassInitial = 0, kPassGenerate, kPassSelect, kPassSpatial, kPassFinal };

__device__ __forceinline__ int batchFind(const BatchLaunch& BL, int t) {
    int i = 0;
    while (i + 1 < BL.numInst && BL.inst[i + 1].tileStart <= t) ++i;
    return i;
}

template <class T>
__device__ __forceinline__ void blockCopy(T* dst, const T* src) {
    static_assert(sizeof(T) % 4 == 0, "word copy");
    int* d = reinterpret_cast<int*>(dst);
    const int* s = reinterpret_cast<const int*>(src);
#if defined(VR_HOST_EMULATION)
    for (int k = 0; k < (int)(sizeof(T) / 4); ++k) d[k] = s[k];
#else
    for (int k = threadIdx.x; k < (int)(sizeof(T) / 4); k += blockDim.x) d[k] = s[k];
#endif
}

template <int MB, int PASS>
__global__ void __launch_bounds__(128, VR_KINIT_MIN_BLOCKS) kb_pixels(const BatchLaunch BL) {
    __shared__ FrameParams sP;
    __shared__ FrameBuffers sB;
    __shared__ LpBuffers sL;
    __shared__ SpatialParams sS;
    int cur = -1;
    for (int t = blockIdx.x; t < BL.totalTiles; t += gridDim.x) {
        const int i = batchFind(BL, t);
        const BatchInstance& I = BL.inst[i];
        bool active;
        if (PASS == kPassInitial) active = !I.learned;
        else if (PASS == kPassGenerate || PASS == kPassSelect) active = I.learned != 0;
        else if (PASS == kPassSpatial) active = BL.round < I.spatialRounds;
        else active = I.spatialRounds == 0;
        if (!active) continue;
        if (i != cur) {
            __syncthreads();
            blockCopy(&c_scene, I.scene);
            blockCopy(&sP, &I.P);
            blockCopy(&sB, &I.B);
            if (PASS == kPassGenerate || PASS == kPassSelect) blockCopy(&sL, &I.L);
            if (PASS == kPassSpatial) blockCopy(&sS, &I.S[BL.round]);
            __syncthreads();
            cur = i;
        }
        const int lt = t - I.tileStart;
        const int tx = lt % I.tilesX, ty = lt / I.tilesX;
        const int px = tx * BL.tileW + (int)threadIdx.x % BL.tileW;
        const int py = ty * BL.tileH + (int)threadIdx.x / BL.tileW;
        if (px < sP.W && py < sP.H) {
            if (PASS == kPassInitial) initialPixel<MB>(sP, sB, px, py);
            else if (PASS == kPassGenerate) lpGeneratePixel<MB>(sP, sB, sL, px, py);
            else if (PASS == kPassSelect) lpSelectPixel<MB>(sP, sB, sL, px, py);
            else if (PASS == kPassSpatial) spatialPixel<MB>(sP, sB, sS, px, py);
            else finalPixel<MB>(sP, sB, 0, px, py);
        }
    }
}

// the bounce pass b of learned instance `inst` (its queue of continuing candidate paths)
template <int MB>
__global__ void __launch_bounds__(128, VR_KINIT_MIN_BLOCKS) kb_lp_bounce(const BatchLaunch BL, int inst, int b) {
    __shared__ FrameParams sP;
    __shared__ LpBuffers sL;
    const BatchInstance& I = BL.inst[inst];
    blockCopy(&c_scene, I.scene);
    blockCopy(&sP, &I.P);
    blockCopy(&sL, &I.L);
    __syncthreads();
    const int n = min(sL.pcount[b], sL.pcapacity);
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < (size_t)n; i += (size_t)gridDim.x * blockDim.x)
        lpBouncePath<MB>(sP, sL, b, sL.paths[b & 1], i);
}

// the bounce pass b of learned instance `inst` as resumable walks over its queue, then the
// vertices (point-sampled distances; see k_lp_walk)
template <int MB>
__global__ void __launch_bounds__(128, VR_KINIT_MIN_BLOCKS) kb_lp_walk(const BatchLaunch BL, int inst, int b) {
    __shared__ FrameParams sP;
    __shared__ LpBuffers sL;
    const BatchInstance& I = BL.inst[inst];
    blockCopy(&c_scene, I.scene);
    blockCopy(&sP, &I.P);
    blockCopy(&sL, &I.L);
    __syncthreads();
    lpWalkPass<MB>(sP, sL, b, sL.paths[b & 1]);
}
template <int MB>
__global__ void __launch_bounds__(128, VR_KINIT_MIN_BLOCKS) kb_lp_vertex(const BatchLaunch BL, int inst, int b) {
    __shared__ FrameParams sP;
    __shared__ LpBuffers sL;
    const BatchInstance& I = BL.inst[inst];
    blockCopy(&c_scene, I.scene);
    blockCopy(&sP, &I.P);
    blockCopy(&sL, &I.L);
    __syncthreads();
    lpVertexPass<MB>(sP, sL, b, sL.paths[b & 1]);
}

// training samples of every learned instance, in chunks of 128 that never straddle instances
template <int MB>
__global__ void __launch_bounds__(128) kb_train_gen(const BatchLaunch BL) {
    __shared__ FrameParams sP;
    __shared__ LpBuffers sL;
    int cur = -1;
    for (int ch = blockIdx.x; ch < BL.trainChunks; ch += gridDim.x) {
        int i = 0;
        while (i + 1 < BL.numInst && BL.inst[i + 1].trainChunkStart <= ch) ++i;
        const BatchInstance& I = BL.inst[i];
        if (!I.learned || I.L.trainCount <= 0) continue;
        if (i != cur) {
            __syncthreads();
            blockCopy(&c_scene, I.scene);
            blockCopy(&sP, &I.P);
            blockCopy(&sL, &I.L);
            __syncthreads();
            cur = i;
        }
        const int s = (ch - I.trainChunkStart) * 128 + (int)threadIdx.x;
        if (s < sL.trainCount) lpTrainSample<MB>(sP, sL, I.trainSeed, s);
    }
}

}  // namespace vrd

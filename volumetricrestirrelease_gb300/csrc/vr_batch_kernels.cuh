// vr_batch_kernels.cuh -- the persistent batched frame kernels (see batch.cu).
#pragma once

#include "vr_batch.h"
#include "vr_lp_kernels.cuh"

namespace vrd {

enum BatchPass { kPassInitial = 0, kPassGenerate, kPassSelect, kPassSpatial, kPassFinal, kPassSplitA, kPassSplitB, kPassSplitC };

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

// resident blocks per SM each pass is compiled for: the select pass and the spatial rounds'
// last kernels at 4 (128 registers; their per-pixel state spills at 96, more so than in the
// single-instance kernels, whose parameters are constant-bank operands rather than shared
// memory loads), the others at VR_KINIT_MIN_BLOCKS (96 registers)
__host__ __device__ constexpr int batchPassBlocks(int pass) {
    return (pass == kPassSelect || pass == kPassSpatial || pass == kPassSplitC) ? 4 : VR_KINIT_MIN_BLOCKS;
}

template <int MB, int PASS>
__global__ void __launch_bounds__(128, batchPassBlocks(PASS)) kb_pixels(const BatchLaunch BL) {
    __shared__ FrameParams sP;
    __shared__ FrameBuffers sB;
    __shared__ LpBuffers sL;
    __shared__ SpatialParams sS;
    __shared__ SpatialSplit sSS;
    constexpr bool kSplit = PASS == kPassSplitA || PASS == kPassSplitB || PASS == kPassSplitC;
    int cur = -1;
    for (int t = blockIdx.x; t < BL.totalTiles; t += gridDim.x) {
        const int i = batchFind(BL, t);
        const BatchInstance& I = BL.inst[i];
        bool active;
        if (PASS == kPassInitial) active = !I.learned;
        else if (PASS == kPassGenerate || PASS == kPassSelect) active = I.learned != 0;
        else if (PASS == kPassSpatial) active = BL.round < I.spatialRounds && !I.split;
        else if (kSplit) active = BL.round < I.spatialRounds && I.split;
        else active = I.spatialRounds == 0;
        if (!active) continue;
        if (i != cur) {
            __syncthreads();
            blockCopy(&c_scene, I.scene);
            blockCopy(&sP, &I.P);
            blockCopy(&sB, &I.B);
            if (PASS == kPassGenerate || PASS == kPassSelect) blockCopy(&sL, &I.L);
            if (PASS == kPassSpatial || kSplit) blockCopy(&sS, &I.S[BL.round]);
            if (kSplit) blockCopy(&sSS, &I.SS);
            __syncthreads();
            cur = i;
        }
        const int lt = t - I.tileStart;
        const int tx = lt % I.tilesX, ty = lt / I.tilesX;
        const int px = tx * BL.tileW + (int)threadIdx.x % BL.tileW;
        const int py = ty * BL.tileH + (int)threadIdx.x / BL.tileW;
        if (px < sP.W && py < sP.H) {
            if (PASS == kPassInitial) initialPixel<MB>(sP, sB, px, py);
            else if (PASS == kPassGenerate) lpRoundsPixel<MB>(sP, sB, sL, px, py);
            else if (PASS == kPassSelect) lpSelectPixel<MB>(sP, sB, sL, px, py);
            else if (PASS == kPassSpatial) spatialPixel<MB>(sP, sB, sS, px, py);
            else if (PASS == kPassSplitA) splitAPixel<MB>(sP, sB, sS, sSS, px, py);
            else if (PASS == kPassSplitB) splitBPixel<MB>(sP, sB, sS, sSS, px, py);
            else if (PASS == kPassSplitC) splitCPixel<MB>(sP, sB, sS, sSS, px, py);
            else finalPixel<MB>(sP, sB, 0, px, py);
        }
    }
}

// the recorded segments of the split spatial round of every instance in the round: the blocks
// take the instances' lists one after another (a block moves on when its warps have used up the
// list, loading the next instance's scene), so small instances share the grid
static __global__ void __launch_bounds__(128, VR_KINIT_MIN_BLOCKS) kb_split_march(const BatchLaunch BL) {
    __shared__ SpatialSplit sSS;
    for (int i = 0; i < BL.numInst; ++i) {
        const BatchInstance& I = BL.inst[i];
        if (!I.split || BL.round >= I.spatialRounds) continue;
        __syncthreads();
        blockCopy(&c_scene, I.scene);
        blockCopy(&sSS, &I.SS);
        __syncthreads();
        splitMarchList(sSS);
    }
}
// clears the list counters of every instance's split round
static __global__ void kb_split_reset(const BatchLaunch BL) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < BL.numInst && BL.inst[i].split) {
        BL.inst[i].SS.counts[0] = 0;
        BL.inst[i].SS.counts[1] = 0;
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

// the bounce pass b of every walking instance in one launch each for the walks and the vertices:
// the blocks take the instances' queues one after another (a block moves on when its warps have
// used up the queue, loading the next instance's scene), so the tail of one instance's walks
// overlaps the next instance's
template <int MB>
__global__ void __launch_bounds__(128, VR_KINIT_MIN_BLOCKS) kb_lp_walk_all(const BatchLaunch BL, int b) {
    __shared__ FrameParams sP;
    __shared__ LpBuffers sL;
    for (int i = 0; i < BL.numInst; ++i) {
        const BatchInstance& I = BL.inst[i];
        if (!I.walk) continue;
        __syncthreads();
        blockCopy(&c_scene, I.scene);
        blockCopy(&sP, &I.P);
        blockCopy(&sL, &I.L);
        __syncthreads();
        lpWalkPass<MB>(sP, sL, b, sL.paths[b & 1]);
    }
}
template <int MB>
__global__ void __launch_bounds__(128, VR_KINIT_MIN_BLOCKS) kb_lp_vertex_all(const BatchLaunch BL, int b) {
    __shared__ FrameParams sP;
    __shared__ LpBuffers sL;
    for (int i = 0; i < BL.numInst; ++i) {
        const BatchInstance& I = BL.inst[i];
        if (!I.walk) continue;
        __syncthreads();
        blockCopy(&c_scene, I.scene);
        blockCopy(&sP, &I.P);
        blockCopy(&sL, &I.L);
        __syncthreads();
        lpVertexPass<MB>(sP, sL, b, sL.paths[b & 1]);
    }
}

// the first vertices of every learned instance's candidates (after the generate pass's rounds),
// in chunks of 128 candidates that never straddle instances; candidate c of pixel pid is entry
// c * N + pid of its instance, as in k_lp_vertex0
template <int MB>
__global__ void __launch_bounds__(128, VR_KINIT_MIN_BLOCKS) kb_vertex0(const BatchLaunch BL) {
    __shared__ FrameParams sP;
    __shared__ LpBuffers sL;
    int cur = -1;
    for (int ch = blockIdx.x; ch < BL.candChunks; ch += gridDim.x) {
        int i = 0;
        while (i + 1 < BL.numInst && BL.inst[i + 1].candChunkStart <= ch) ++i;
        const BatchInstance& I = BL.inst[i];
        if (!I.learned) continue;
        if (i != cur) {
            __syncthreads();
            blockCopy(&c_scene, I.scene);
            blockCopy(&sP, &I.P);
            blockCopy(&sL, &I.L);
            __syncthreads();
            cur = i;
        }
        const size_t e = (size_t)(ch - I.candChunkStart) * 128 + threadIdx.x;
        if (e < (size_t)sP.initialM * (size_t)sP.N) {
            const int c = (int)(e / (size_t)sP.N), pid = (int)(e - (size_t)c * (size_t)sP.N);
            lpVertex0<MB>(sP, sL, c, pid % sP.W, pid / sP.W);
        }
    }
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

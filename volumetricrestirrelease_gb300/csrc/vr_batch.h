// vr_batch.h -- device view of a batch: many independent instances (volume, view, options,
// buffers) rendered by persistent kernels that walk one list of pixel tiles over all of them.
#pragma once

#include "vr_kernels.cuh"
#include "vr_lp.h"

namespace vrd {

constexpr int kBatchMaxRounds = 16;

struct BatchInstance {
    FrameParams P;
    FrameBuffers B;
    LpBuffers L;
    SpatialParams S[kBatchMaxRounds];   // one per spatial round of the frame
    const DevScene* scene;               // the instance's scene constants in global memory
    int tilesX, tileStart;               // tile grid of the instance and its first tile in the list
    int spatialRounds;
    int learned;                         // generate / select instead of the fused initial kernel
    uint32_t trainSeed;
    int trainChunkStart;                 // first 128-sample chunk of the instance's training samples
};

struct BatchLaunch {
    const BatchInstance* inst;           // device array
    int numInst, totalTiles;
    int tileW, tileH;                    // tileW * tileH = 128
    int round;                           // spatial round of this launch
    int trainChunks;                     // 128-sample chunks of training samples over all instances
};

}  // namespace vrd

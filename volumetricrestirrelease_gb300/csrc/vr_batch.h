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
    int split;                           // the spatial rounds with their marches split out (k_split_*)
    SpatialSplit SS;                     // the instance's buffers of the split rounds
    int learned;                         // generate / select instead of the fused initial kernel
    int walk;                            // learned, point-sampled distances: the bounce passes as walks
    uint32_t trainSeed;
    int trainChunkStart;                 // first 128-sample chunk of the instance's training samples
    int candChunkStart;                  // first 128-candidate chunk of the instance's first vertices
};

struct BatchLaunch {
    const BatchInstance* inst;           // device array
    int numInst, totalTiles;
    int tileW, tileH;                    // tileW * tileH = 128
    int round;                           // spatial round of this launch
    int trainChunks;                     // 128-sample chunks of training samples over all instances
    int candChunks;                      // 128-candidate chunks of first vertices over all instances
};

}  // namespace vrd
